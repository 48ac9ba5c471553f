// intersect_trace.cpp — runs the shared per-ray sequence (intersect_sequence.inc) on the drop-in
// classes (raytrace_gb300/cpp) and prints its records to stdout. Built and run by
// tests/test_intersect.py with g++ from the drop-in's host sources; no GPU is involved.
// Usage: intersect_trace [rays per object]   (run in tests/golden/obj)
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../raytrace_gb300/cpp/Model.h"
#include "../../raytrace_gb300/cpp/Scene.h"

static void emit(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
}

// a drop-in model's hit token is the address of the Triangle it hit
static bool tri_index(const Model *m, intptr_t token, int *part, int *index)
{
    for (size_t a = 0; a < m->parts.size(); ++a) {
        const auto &p = m->parts[a];
        if (!p.empty() && token >= (intptr_t)p.data() && token < (intptr_t)(p.data() + p.size())) {
            *part = (int)a;
            *index = (int)(((const Triangle *)token) - p.data());
            return true;
        }
    }
    return false;
}

#include "intersect_sequence.inc"

int main(int argc, char **argv)
{
    run_intersect_sequence(argc > 1 ? std::atoi(argv[1]) : 300);
    return 0;
}
