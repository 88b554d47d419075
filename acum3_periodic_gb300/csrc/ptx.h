// ptx.h -- device helpers shared by the kernels: mbarrier operations (every wait
// bounded), the bulk (TMA) global -> shared copy, the device error word, packed FP32.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "acum_internal.h"

namespace acum {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Every wait on a barrier is bounded in time: it gives up after limit_ns of the global
// timer (2 s by default; kMaxSpin polls should the timer not advance), and the caller
// records ACUM_DEVERR_TIMEOUT and unwinds instead of hanging.  A wait whose first poll
// succeeds (the common case) reads no timer.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;
constexpr long kMaxSpin = 1L << 26;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  unsigned long long limit_ns = kWaitLimitNs)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (long it = 0; it < kMaxSpin; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255) == 255 && global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// bulk TMA copy global -> shared, completion signalled on `bar` (bytes % 16 == 0,
// both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void flag(DeviceErr* e, unsigned bit, unsigned* counter)
{
    atomicOr(&e->bits, bit);
    atomicAdd(counter, 1u);
}

// packed FP32: two values in an f32x2 register pair, one instruction (sm_100 and later)
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
// One MUFU operation each (approximate, ~1 ulp): the reciprocal and the reciprocal square
// root with denormal operands and results flushed to zero, which leaves out the range
// scaling of the non-flushing forms.  Every operand of these in the kernels is a normal
// number or a value whose result is rejected as invalid anyway.
__device__ __forceinline__ float rcp_ftz(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(rcp_ftz(a.x), rcp_ftz(a.y)); }

}  // namespace acum
