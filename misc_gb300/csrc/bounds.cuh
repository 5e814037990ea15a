// Index guards of the checked build (device code).
//
// Built with -DASTRO_BOUNDS_CHECK (misc_gb300/build.py with ASTRO_BOUNDS_CHECK=1 in the
// environment, into libastro_gpu_checked.so), every guarded access first tests its index against
// the size of the buffer it touches.  A failing test records the guard's site number in a status
// word (the first failure wins, by compare-and-swap) and skips the access: the device function
// returns.  There is no trap and no assert, so the context stays usable; the host reads the word
// after the launches and turns a non-zero site into an error return.  In the normal build the
// guards compile to nothing.
#pragma once

#ifdef ASTRO_BOUNDS_CHECK
#define ASTRO_CHECKED 1
#define ASTRO_GUARD(status, site, ok)                              \
    do {                                                           \
        if (!(ok)) {                                               \
            if (status) atomicCAS((status), 0, (site));            \
            return;                                                \
        }                                                          \
    } while (0)
// the same for kernels whose warps synchronise: the whole warp evaluates the test (each lane
// its own condition) and leaves together, so no lane waits at a warp barrier for one that left
#define ASTRO_GUARD_WARP(status, site, ok)                                       \
    do {                                                                         \
        if (!__all_sync(0xffffffffu, (ok))) {                                    \
            if ((threadIdx.x & 31) == 0 && (status)) atomicCAS((status), 0, (site)); \
            return;                                                              \
        }                                                                        \
    } while (0)
#else
#define ASTRO_CHECKED 0
#define ASTRO_GUARD(status, site, ok) \
    do {                              \
    } while (0)
#define ASTRO_GUARD_WARP(status, site, ok) \
    do {                                   \
    } while (0)
#endif

// 0 <= i < n
#define ASTRO_IN(i, n) ((long long)(i) >= 0 && (long long)(i) < (long long)(n))
