// cnv_sync.cuh -- device helpers shared by the persistent kernels (SOR, mixed, batched): acquire
// loads and release stores at GPU scope for progress flags, the global nanosecond timer that
// bounds every wait, the bounded wait itself, and the split-layout column helper.
#pragma once

#include "cnv_kernels.h"

namespace cnv {
namespace {

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ long long globaltimer_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int ld_volatile_int(const int* p) { return *(const volatile int*)p; }

// Wait until *p >= want (as sweep counters, modulo 2^32). Returns false when the abort flag is
// raised, or after timeout_ns (then records CNV_TIMEOUT and raises the abort flag).
__device__ bool wait_geq(const unsigned* p, unsigned want, Ctrl* ctl, long long timeout_ns) {
    long long t0 = 0;
    int polls = 0;
    while ((int)(ld_acquire(p) - want) < 0) {
        if (ld_volatile_int(&ctl->abort)) return false;
        if (++polls == 64) t0 = globaltimer_ns();
        if (polls > 64 && globaltimer_ns() - t0 > timeout_ns) {
            atomicExch(&ctl->status, CNV_TIMEOUT);
            atomicExch(&ctl->abort, 1);
            return false;
        }
    }
    return true;
}

// floor(j / 2) for any sign: the split-layout column of cell column j.
__host__ __device__ __forceinline__ int floor_half(int j) { return j >= 0 ? j / 2 : -((1 - j) / 2); }

}  // namespace
}  // namespace cnv
