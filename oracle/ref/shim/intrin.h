/* MSVC intrinsics header stand-in: the same SSE/AVX intrinsics from GCC's immintrin.h */
#pragma once
#include <immintrin.h>
#define _VCRT_ALIGN(x) __attribute__((aligned(x)))
#ifndef _MM_ALIGN16
#define _MM_ALIGN16
#endif
