// Portable stand-in for the three x86 intrinsics the reference uses
// (src/core/sampler.hpp:3,104-106,124-126, src/core/RWR.cpp:95), so its
// sources also build on aarch64.  The prefetch keeps its meaning; the cache
// flushes become no-ops, which can only make the reference faster.  Test
// infrastructure for building the reference baseline.
#pragma once
#define _MM_HINT_T0 3
#define _MM_HINT_T1 2
#define _MM_HINT_T2 1
#define _MM_HINT_NTA 0
#define _mm_prefetch(p, hint) __builtin_prefetch((const void *)(p), 0, (hint))
#define _mm_clflushopt(p) ((void)(p))
#define _mm_clflush(p) ((void)(p))
