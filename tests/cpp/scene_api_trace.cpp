// scene_api_trace.cpp — runs the shared Scene API sequence on the drop-in classes
// (raytrace_gb300/cpp) and prints its trace to stdout. Built and run by
// tests/test_scene_api.py with g++ from the drop-in's host sources; no GPU is involved.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "../../raytrace_gb300/cpp/Scene.h"

static void emit(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
}

#include "scene_api_sequence.inc"

int main()
{
    run_scene_api_sequence();
    return 0;
}
