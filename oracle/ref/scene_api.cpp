// scene_api.cpp — runs the shared Scene API sequence (tests/cpp/scene_api_sequence.inc) on the
// reference's own Scene / Light / Camera classes, compiled from the reference sources by
// oracle/ref/Makefile into oracle/_ref/rt_ref_scene_api. TEST INFRASTRUCTURE ONLY: its output
// is the golden trace tests/golden/scene_api/trace_ref.txt (tests/golden/make_scene_api_golden.py).
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "Scene.h"

static void emit(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vprintf(fmt, ap);
    va_end(ap);
}

#include "../../tests/cpp/scene_api_sequence.inc"

int main()
{
    run_scene_api_sequence();
    return 0;
}
