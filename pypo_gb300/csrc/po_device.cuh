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

// Bounded wait: gives up after `limit` polls (kWaitLimit in the kernels; each
// poll may itself block for a bounded hardware time slice) and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit = kWaitLimit)
{
    for (uint32_t i = 0; i < limit; ++i)
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

// ------------------------------------------------- packed FP32x2 arithmetic
//
// Blackwell's FFMA2/FADD2/FMUL2 do two FP32 operations per issued
// instruction (the FP32 pipe rate is unchanged, the issue slots are halved).
// Each lane rounds exactly like the scalar __f*_rn form, so error-free
// transformations written with these stay exact.
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// 1/sqrt(x), flush-to-zero form (x = R^2 in turns^2 is never subnormal for
// distinct points).
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Phases are reduced exactly to half turns before any sin/cos: the phase in
// half turns is f = q + y with q an integer and |y| <= 1/2, and sin(pi f),
// cos(pi f) = (-1)^q sin(pi y), (-1)^q cos(pi y). Why exactly: a rounded pi
// (or 1/2pi) in the argument is a relative scale error of ~3e-8 on every
// pair, which on sums of millions of pairs with spread-out phases adds up
// coherently (the sum grows like sqrt(N), the error like N), to ~1e-5. After
// the exact reduction any error of the reduced sin/cos flips sign with q, so
// over phases spread across many turns it averages out instead.
//
// sincos_poly2: sin(pi y) = y P(y^2) and cos(pi y) = 1 + y^2 Q(y^2) on both
// lanes for |y| <= 1/2, degree-4 P and Q (near-minimax fits, |error| < 4e-9
// before rounding) whose leading coefficients are carried as two floats, so
// that no rounded pi scales the argument either.
__device__ __forceinline__ void sincos_poly2(float2 y, float2 &sn, float2 &cs)
{
    const float2 y2 = mul2(y, y);
    float2 p = fma2(y2, dup2(0.07722020894289017f), dup2(-0.5980452299118042f));
    p = fma2(y2, p, dup2(2.5500314235687256f));
    p = fma2(y2, p, dup2(-5.1677069664001465f));
    p = fma2(y2, p, dup2(3.141592502593994f));
    sn = fma2(y, p, mul2(y, dup2(7.752134223437679e-08f)));
    float2 r = fma2(y2, dup2(-0.02442070282995701f), dup2(0.23495392501354218f));
    r = fma2(y2, r, dup2(-1.3352161645889282f));
    r = fma2(y2, r, dup2(4.058709621429443f));
    r = fma2(y2, r, dup2(-4.934802055358887f));
    cs = fma2(y2, dup2(-1.0072982092879101e-07f), fma2(y2, r, dup2(1.0f)));
}

// a * (-1)^q per lane, the parity of q being the low bit of t = 1.5*2^23 + q as
// the phase helpers below return it (integer pipe, two ops a lane).
__device__ __forceinline__ float2 flip_parity(float2 a, float2 t)
{
    return make_float2(__uint_as_float(__float_as_uint(a.x) ^ (__float_as_uint(t.x) << 31)),
                       __uint_as_float(__float_as_uint(a.y) ^ (__float_as_uint(t.y) << 31)));
}

// sin(pi y), cos(pi y) for the exactly reduced |y| <= 1/2 (plus a rounding).
__device__ __forceinline__ void sincos_reduced2(float2 y, float2 &sn, float2 &cs)
{
#if PO_MUFU_SINCOS
    // hardware sin/cos of the exactly reduced angle pi y (|pi y| <= pi/2)
    const float2 a = mul2(y, dup2(3.14159265358979324f));
    __sincosf(a.x, &sn.x, &cs.x);
    __sincosf(a.y, &sn.y, &cs.y);
#else
    sincos_poly2(y, sn, cs);
#endif
}

// Far-field phase 2 pi (P + p) in turns, P the exact hi projection (|P| below
// 2^21), p the lo projection. In half turns: q1 = rint(2P) from one fma
// against 1.5*2^23, x = 2P - q1 exact (Sterbenz, |x| <= 1/2); y1 = x + 2p
// rounded once; q2 = rint(y1), y = y1 - q2 exact, so |y| <= 1/2 for any
// size of p. sin/cos up to (-1)^(q1 + q2); the parity of q1 + q2 is the low
// bit of t (t1's bits with t2's low bit xor-ed in, one logic op a lane).
__device__ __forceinline__ void ff_phase_sincos2(float2 P, float2 p, float2 &sn, float2 &cs, float2 &t)
{
    const float2 two = dup2(2.0f), magic = dup2(12582912.0f);
    const float2 t1 = fma2(P, two, magic);
    const float2 y1 = fma2(p, two, fma2(P, two, neg2(sub2(t1, magic))));
    const float2 t2 = add2(y1, magic);
    sincos_reduced2(sub2(y1, sub2(t2, magic)), sn, cs);
    t = make_float2(__uint_as_float(__float_as_uint(t1.x) ^ (__float_as_uint(t2.x) & 1u)),
                    __uint_as_float(__float_as_uint(t1.y) ^ (__float_as_uint(t2.y) & 1u)));
}

// Phase of a pair from the split separation, and its sin/cos up to (-1)^q.
// R^2 = S0 + S1 (S0 exact, S1 small), Rh = R^2 rinv0 ~ R (turns). The
// residual res = (S0 - Rh^2) + S1 gives R = Rh + res / (2 Rh); the fma
// rounds S0 - Rh^2 once, an error of ~2^-47 R turns. In half turns,
// 2R = 2 Rh + res rinv0: q = rint(2 Rh) from one fma against 1.5*2^23,
// y = (2 Rh - q) + res rinv0 with 2 Rh - q exact (Sterbenz). |y| <= 1/2 +
// |res rinv0|, and |res rinv0| ~ 2 |R - Rh| <= 2^-22 R from the rsqrt
// estimate: below 0.03 for R up to 2e5 turns, where both the hardware
// sin/cos and the polynomials (error 3e-8 at |y| = 0.52) are still exact
// to FP32 level. R below 2^21 turns.
__device__ __forceinline__ void phase_sincos2(float2 S0, float2 S1, float2 Rh, float2 rinv0, float2 &sn, float2 &cs,
                                              float2 &t)
{
    const float2 two = dup2(2.0f), magic = dup2(12582912.0f);
    const float2 res = add2(fma2(neg2(Rh), Rh, S0), S1);
    t = fma2(Rh, two, magic);
    sincos_reduced2(fma2(res, rinv0, fma2(Rh, two, neg2(sub2(t, magic)))), sn, cs);
}

// Trapezoid weight of grid point i (row-major over x/u, y/v): 1/2 on the
// x/u end rows, and on the y/v end columns unless the grid is uv (periodic in
// v); 1 for a point cloud (gmode < 0). Reference src/CPU/Propagation.h:
// the x/u end rows always, the y/v end columns for gmode != 1.
__device__ __forceinline__ double trap_weight(long i, int gmode, int ncx, int ncy)
{
    if (gmode < 0) return 1.0;
    const long xu = i / ncy, yv = i - xu * ncy;
    double w = (xu == 0 || xu == ncx - 1) ? 0.5 : 1.0;
    if (gmode != 1 && (yv == 0 || yv == ncy - 1)) w *= 0.5;
    return w;
}

// A coordinate x (turns, relative to the frame origin) as hi + lo: hi on the
// frame's quantum q (at most 11 significant bits), lo the small rest.
__device__ __forceinline__ void split_hi_lo(double x, const Frame &fr, float &h, float &l)
{
    const double hd = rint(x * fr.inv_q) * fr.q;
    h = (float)hd;
    l = (float)(x - hd);
}

// ------------------------------------- the reference's illumination decision
//
// The reference skips a source when its FP64 n . R_hat < 0 (near field;
// far field n . r_hat < 0), with R_hat = d (1/R) and the dot product summed
// left to right (src/CPU/Propagation.h:977-1144, :1656-1781). The FP64
// kernels repeat that rounding exactly; the mixed kernels use it for the
// pairs their FP32 test cannot decide (kTangentBand), through the band list.
__device__ __forceinline__ bool lit_fp64(const double *n, double dx, double dy, double dz, double rinv)
{
    const double ndr = __dadd_rn(__dadd_rn(__dmul_rn(n[0], __dmul_rn(dx, rinv)), __dmul_rn(n[1], __dmul_rn(dy, rinv))),
                                 __dmul_rn(n[2], __dmul_rn(dz, rinv)));
    return !(ndr < 0.0);
}

// A pair inside the tangent band: listed for the FP64 fixup (one atomic; the
// rare branch of the pair loops). A full list drops the entry; the fixup
// then reports the overflow.
__device__ __forceinline__ void band_defer(const BandList &bl, long si, long ti)
{
    const unsigned i = atomicAdd(bl.count, 1u);
    if (i < bl.cap) bl.pairs[i] = make_int2((int)si, (int)ti);
}

// One source's FP64 record (kRecD doubles: x y z nx ny nz, J' (re, im) x y z,
// M' likewise; scalar: S' in the J'x slot): the currents times the trapezoid
// weight, the area and the complex factor (fac_re, fac_im).
__device__ __forceinline__ void src_record_d(long i, long ns, const double *src7, const double *cur, int gmode,
                                             int ncx, int ncy, double fac_re, double fac_im, int scalar, double *o)
{
    for (int c = 0; c < 6; ++c) o[c] = src7[c * ns + i];
    const double w = trap_weight(i, gmode, ncx, ncy) * src7[6 * ns + i];
    const double fr_ = fac_re * w, fi_ = fac_im * w;
    if (scalar) {
        const double re = cur[i], im = cur[ns + i];
        o[6] = fr_ * re - fi_ * im;
        o[7] = fr_ * im + fi_ * re;
        for (int q = 8; q < kRecD; ++q) o[q] = 0.0;
        return;
    }
    for (int q = 0; q < 6; ++q) {
        const int grp = q / 3, ax = q % 3;
        const double re = cur[(grp * 6 + ax) * ns + i];
        const double im = cur[(grp * 6 + 3 + ax) * ns + i];
        o[6 + 2 * q] = fr_ * re - fi_ * im;
        o[7 + 2 * q] = fr_ * im + fi_ * re;
    }
}

// The direction of far-field target i from its (polar, azimuth), as the FP64
// kernels form it.
__device__ __forceinline__ void ff_direction_d(const double *tgt7, long nt, long i, double *p)
{
    const double th = tgt7[i], ph = tgt7[nt + i];
    p[0] = cos(ph) * sin(th);
    p[1] = sin(ph) * sin(th);
    p[2] = cos(th);
}

// --------------------------------------------------- EHP reflection, generic
//
// The reflected field of mode EHP (reference src/CPU/Propagation.h:840-913,
// Snell's law Utils.h:421-432): the incident Poynting direction
// s_i = Re(E x conj H) / |.|, the reflected direction s_r = s_i - 2 (s_i.n) n,
// the incident and reflected polarisation bases, E_r = -(E.p_r) p_i -
// (E.a_r) a_i and H_r = zeta_inv s_r x E_r. Written for any real type F with
// the arithmetic operators (double in the epilogue; a dual number in the
// adjoint's cotangent mapping, which differentiates it forward mode).
// out: E_r re xyz, im xyz, H_r re xyz, im xyz, s_r xyz (15).
template <typename F>
__device__ __forceinline__ void ehp_cross(const F *a, const F *b, F *o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename F>
__device__ __forceinline__ void ehp_normalize(const F *v, F *o)
{
    F n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n <= 4.9406564584124654e-324) n = 4.9406564584124654e-324;
    for (int c = 0; c < 3; ++c) o[c] = v[c] / n;
}

template <typename F>
__device__ __forceinline__ void ehp_reflect(const F *er, const F *ei, const F *hr, const F *hi, const double *nd,
                                            double zeta_inv, F *out)
{
    F s[3], si[3], tmp[3], pip[3], pia[3], sr[3], prp[3], pra[3], n[3];
    for (int c = 0; c < 3; ++c) {
        n[c] = nd[c];
        // Re(E x conj(H))_c
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        s[c] = (er[a1] * hr[a2] + ei[a1] * hi[a2]) - (er[a2] * hr[a1] + ei[a2] * hi[a1]);
    }
    ehp_normalize(s, si);
    ehp_cross(si, n, tmp);
    ehp_normalize(tmp, pip);
    ehp_cross(pip, si, pia);
    const F f = 2.0 * (si[0] * n[0] + si[1] * n[1] + si[2] * n[2]);
    for (int c = 0; c < 3; ++c) sr[c] = si[c] - n[c] * f;
    ehp_cross(sr, n, tmp);
    ehp_normalize(tmp, prp);
    ehp_cross(sr, prp, pra);
    const F epr = er[0] * prp[0] + er[1] * prp[1] + er[2] * prp[2];
    const F epi = ei[0] * prp[0] + ei[1] * prp[1] + ei[2] * prp[2];
    const F ear = er[0] * pra[0] + er[1] * pra[1] + er[2] * pra[2];
    const F eai = ei[0] * pra[0] + ei[1] * pra[1] + ei[2] * pra[2];
    F rr[3], ri[3], xr[3], xi[3];
    for (int c = 0; c < 3; ++c) {
        rr[c] = -epr * pip[c] - ear * pia[c];
        ri[c] = -epi * pip[c] - eai * pia[c];
    }
    ehp_cross(sr, rr, xr);
    ehp_cross(sr, ri, xi);
    for (int c = 0; c < 3; ++c) {
        out[c] = rr[c];
        out[3 + c] = ri[c];
        out[6 + c] = xr[c] * zeta_inv;
        out[9 + c] = xi[c] * zeta_inv;
        out[12 + c] = sr[c];
    }
}

// Forward-mode dual number: value and derivative along one seed direction.
// (sqrt is a hidden friend, found by argument-dependent lookup only, so it
// does not hide ::sqrt for doubles in this namespace.)
struct Dual {
    double v, d;
    __device__ Dual() : v(0.0), d(0.0) {}
    __device__ Dual(double x) : v(x), d(0.0) {}
    __device__ Dual(double x, double dx) : v(x), d(dx) {}
    __device__ friend Dual sqrt(Dual a)
    {
        const double r = ::sqrt(a.v);
        return Dual(r, r > 0.0 ? a.d / (2.0 * r) : 0.0);
    }
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b)
{
    const double q = a.v / b.v;
    return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ bool operator<=(Dual a, double b) { return a.v <= b; }

}  // namespace po
