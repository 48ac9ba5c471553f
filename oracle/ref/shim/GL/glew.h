/* Header stand-in so the reference's sources compile without OpenGL: GL types, the enum
   values they mention, and no-op calls. Rendering through OpenGL is not part of the oracle. */
#pragma once
#include <cstddef>
typedef unsigned int GLuint;
typedef int GLint;
typedef unsigned short GLushort;
typedef unsigned int GLenum;
typedef float GLfloat;
typedef double GLdouble;
typedef int GLsizei;
typedef unsigned char GLubyte;
enum {
    GL_COMPILE = 1, GL_TEXTURE_2D, GL_FRONT_AND_BACK, GL_AMBIENT, GL_DIFFUSE, GL_SPECULAR, GL_EMISSION, GL_SHININESS,
    GL_VERTEX_ARRAY, GL_NORMAL_ARRAY, GL_TEXTURE_COORD_ARRAY, GL_FLOAT, GL_RESCALE_NORMAL, GL_QUADS, GL_UNSIGNED_SHORT,
    GL_TEXTURE_WRAP_S, GL_TEXTURE_WRAP_T, GL_REPEAT, GL_TEXTURE_MAG_FILTER, GL_TEXTURE_MIN_FILTER, GL_NEAREST, GL_RGB,
    GL_BGR_EXT, GL_UNSIGNED_BYTE, GL_CLAMP, GL_LINEAR, GL_TRIANGLES, GL_LIGHT_MODEL_AMBIENT, GL_LIGHT0, GL_POSITION,
    GL_CONSTANT_ATTENUATION, GL_LINEAR_ATTENUATION, GL_QUADRATIC_ATTENUATION, GL_LINE, GL_FILL
};
template <class... A> inline void gl_noop(A...) {}
inline GLuint glGenLists(GLsizei) { return 0; }
#define glNewList gl_noop
#define glEndList gl_noop
#define glCallList gl_noop
#define glBindTexture gl_noop
#define glMaterialfv gl_noop
#define glMaterialf gl_noop
#define glEnableClientState gl_noop
#define glDisableClientState gl_noop
#define glVertexPointer gl_noop
#define glNormalPointer gl_noop
#define glTexCoordPointer gl_noop
#define glEnable gl_noop
#define glDisable gl_noop
#define glScalef gl_noop
#define glDrawElements gl_noop
#define glDrawArrays gl_noop
#define glTexParameteri gl_noop
#define glTexImage2D gl_noop
#define glBegin gl_noop
#define glEnd gl_noop
#define glNormal3fv gl_noop
#define glTexCoord2f gl_noop
#define glTexCoord2fv gl_noop
#define glVertex3fv gl_noop
#define glGenTextures gl_noop
#define glDeleteTextures gl_noop
#define glPushMatrix gl_noop
#define glPopMatrix gl_noop
#define glTranslatef gl_noop
#define glTranslated gl_noop
#define glLightModelfv gl_noop
#define glLightfv gl_noop
#define glLightf gl_noop
#define glPolygonMode gl_noop
#define gluLookAt gl_noop
