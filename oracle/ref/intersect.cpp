// intersect.cpp — runs the shared per-ray sequence (tests/cpp/intersect_sequence.inc) on the
// reference's own objects, compiled from the reference sources by oracle/ref/Makefile into
// oracle/_ref/rt_ref_intersect. TEST INFRASTRUCTURE ONLY: its output is the golden trace
// tests/golden/intersect/trace_ref.txt (tests/golden/make_intersect_golden.py).
// Usage: rt_ref_intersect [rays per object]   (run in tests/golden/obj)
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "Model.h"
#include "Scene.h"

static void emit(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
}

// a reference model's hit token is the address of an octant-list copy of the triangle
// (clTri, Model.cpp:402-480), which carries the triangle's part and index
static bool tri_index(const Model *m, intptr_t token, int *part, int *index)
{
    for (const auto &list : m->octclparts)
        if (!list.empty() && token >= (intptr_t)list.data() && token < (intptr_t)(list.data() + list.size())) {
            const clTri *t = (const clTri *)token;
            *part = t->numa;
            *index = t->numb;
            return true;
        }
    return false;
}

#include "../../tests/cpp/intersect_sequence.inc"

int main(int argc, char **argv)
{
    run_intersect_sequence(argc > 1 ? std::atoi(argv[1]) : 300);
    return 0;
}
