// po_device.cuh -- device helpers shared by the PO kernels: mbarrier waits,
// 1-D TMA bulk copies, error-free additions.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "po_kernels.cuh"

namespace po {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
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

// Bounded wait: gives up after kWaitLimit polls (each poll may itself block
// for a bounded hardware time slice) and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Error-free transformation: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Round-to-nearest integer of |x| < 2^22 without the conversion pipe.
__device__ __forceinline__ float rint_magic(float x)
{
    return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f);
}

// sin(pi f2) and cos(pi f2) for a phase given as f2 = twice its value in turns
// (|f2| <= about 1). A float pi (or 1/2pi) in the argument is a relative scale
// error of 3e-8 on every pair; on sums of millions of pairs with spread-out
// phases it adds up coherently to ~1e-5. Here no scaled argument is formed:
// f2 = q/2 + y with q = rint(2 f2) and |y| <= 1/4 (both exact), and
// sin(pi y) = y P(y^2), cos(pi y) = 1 + y^2 Q(y^2) with degree-3 P and Q
// (least-squares fits on |y| <= 1/4, |error| < 3e-9 before rounding) whose
// leading coefficients carry a second float for the part the first rounds
// off. The quadrant q mod 4 is read from the low bits of 1.5*2^23 + q.
__device__ __forceinline__ void sincos_pi(float f2, float *s, float *c)
{
    const float t = fmaf(f2, 2.0f, 12582912.0f);
    const float q = __fsub_rn(t, 12582912.0f);
    const float y = fmaf(q, -0.5f, f2);
    const float y2 = __fmul_rn(y, y);
    float p = fmaf(y2, -0.5893663167953491f, 2.5497970581054688f);
    p = fmaf(y2, p, -5.167708873748779f);
    p = fmaf(y2, p, 3.1415927410125732f);
    const float sn = fmaf(y, p, __fmul_rn(y, -9.207879969608257e-08f));
    float r = fmaf(y2, 0.23146405816078186f, -1.3350627422332764f);
    r = fmaf(y2, r, 4.058708190917969f);
    r = fmaf(y2, r, -4.934802055358887f);
    const float cn = fmaf(y2, -1.1989475012796902e-07f, fmaf(y2, r, 1.0f));
    const unsigned qi = __float_as_uint(t);
    const float a = (qi & 1u) ? cn : sn;
    const float b = (qi & 1u) ? sn : cn;
    *s = __uint_as_float(__float_as_uint(a) ^ ((qi & 2u) << 30));
    *c = __uint_as_float(__float_as_uint(b) ^ (((qi + 1u) & 2u) << 30));
}

}  // namespace po
