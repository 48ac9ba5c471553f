/* Windows.h stand-in for the reference's sources: the timer, Sleep, BMP headers and _wfopen */
#pragma once
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cwchar>
#include <functional>
#include <string>
#include <thread>
typedef union _LARGE_INTEGER {
    long long QuadPart;
} LARGE_INTEGER;
inline int QueryPerformanceFrequency(LARGE_INTEGER *f) { f->QuadPart = 1000000000LL; return 1; }
inline int QueryPerformanceCounter(LARGE_INTEGER *c)
{
    c->QuadPart = (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(
                      std::chrono::steady_clock::now().time_since_epoch()).count();
    return 1;
}
inline void Sleep(unsigned ms) { std::this_thread::sleep_for(std::chrono::milliseconds(ms)); }
#pragma pack(push, 2)
typedef struct tagBITMAPFILEHEADER {
    uint16_t bfType;
    uint32_t bfSize;
    uint16_t bfReserved1, bfReserved2;
    uint32_t bfOffBits;
} BITMAPFILEHEADER;
#pragma pack(pop)
typedef struct tagBITMAPINFOHEADER {
    uint32_t biSize;
    int32_t biWidth, biHeight;
    uint16_t biPlanes, biBitCount;
    uint32_t biCompression, biSizeImage;
    int32_t biXPelsPerMeter, biYPelsPerMeter;
    uint32_t biClrUsed, biClrImportant;
} BITMAPINFOHEADER;
inline FILE *_wfopen(const wchar_t *name, const wchar_t *mode)
{
    std::string n, m;
    for (const wchar_t *p = name; *p; ++p) n += (char)*p;
    for (const wchar_t *p = mode; *p; ++p) m += (char)*p;
    return std::fopen(n.c_str(), m.c_str());
}
