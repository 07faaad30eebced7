// po_adjoint_pk.cu -- pair-packed adjoint kernels (mixed precision).
//
// Near field: one fused kernel computes, for every (source, target) pair,
// both halves of the near-field adjoint of po_adjoint.cu:
//   source side  Jbar', Mbar' (12 accumulators) and n_s . grad_d phi (1);
//   target side  n_t . grad_d phi, summed over the sources.
// Both displacement terms share the pair's geometry, phase, coefficients and
// S = G (D1 alpha + D2 beta + D3 W.R_hat); only the normal differs
// (n . grad_d phi = (1/R) Re[(R_hat.n) S + C2 (grad(beta).n) + C3 (W.n)]).
//
// Layout: a thread owns one source (forward-packed record, registers) and
// streams PAIRS of targets through shared memory with TMA bulk copies; every
// packed FP32x2 operation works on the two targets of a pair (lane x: target
// 2p, lane y: target 2p + 1). Source-side sums stay per thread (float-float
// totals per tile). Target-side values are transposed through shared memory
// every kFlush target pairs, summed over the CTA's sources, and added into
// an FP64 accumulator per target with atomicAdd (the order of those adds
// varies from run to run: grad_dt is reproducible to ~1e-16, not bitwise).
//
// The three projections of W (on R_hat, n_s, n_t) come from one complex
// vector per pair, Z = b x J - a x M: W.v = -v.Z (scalar triple product).
//
// Far field: the same kernel with the far-field pair (currents and source
// displacement; far-field targets are directions and do not move). A CTA
// owns one tile of 128 sources in Hilbert order (the forward's tile records,
// po_farfield.cu): e^{-t j k r.s} = e^{-t j k r.c} e^{-t j k r.(s - c)}, so
// each stage's cotangents are multiplied once by conj(e^{-t j k r.c}) for
// the CTA's centre c (ff_rotate_cot), and the pair loop takes only the
// offset's phase: FP32 for a narrow tile, split for a wide one. With M = 0,
// a cotangent tile whose direction box proves every pair lit for the CTA's
// source normals skips the illumination mask.
#include <cuda_runtime.h>
#include <math_constants.h>
#include <cstdint>
#include <type_traits>

#include "po_device.cuh"
#include "po_kernels.cuh"

namespace po {

// Pair-packed cotangent record, float2 slots (target 2p, target 2p + 1):
//   0-2 hi position, 3-5 lo position (turns), 6-11 gE (re, im) x y z, 12-17 gH;
//   with the target displacement: 18-20 n_t, 21-22 a.n_t; with M as well:
//   23-24 b.n_t (a = conj(gE), b = conj(gH)). A padding target has zero
//   cotangent.
// Far field: 0-2 r_hat hi (on 2^-11), 3-5 r_hat lo, 6-11 gS_J, 12-17 gS_M,
//   18-20 r_hat = hi + lo (11 float4).
__host__ __device__ constexpr int adj2_rec(int kind, bool has_m, bool want_t)
{
    return kind == kKindFF ? 11 : (want_t ? (has_m ? 13 : 12) : 9);   // scalar: the near-field layout
}

constexpr int kPairsA2 = PO_PAIRS_A;   // target pairs per shared-memory stage
#ifndef PO_FLUSH_A
#define PO_FLUSH_A 16
#endif
constexpr int kFlush = PO_FLUSH_A;   // target pairs per transpose of the target-side values
constexpr int kSegs = kThreadsA / kFlush;   // threads summing one target pair
static_assert(kThreadsA == 128 && (kFlush == 16 || kFlush == 32),
              "the transpose maps 128 threads onto 16 pairs x 8 segments or 32 pairs x 4");

__global__ void po_adj_pack_tgt2_kernel(long nt, const double *__restrict__ tgt7, const double *__restrict__ gam,
                                        const Frame *__restrict__ frp, int far, int rec4, float *__restrict__ out)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long np = (nt + 1) / 2;
    if (i >= 2 * np) return;
    const long k = i < nt ? i : nt - 1;
    const bool real = i < nt;
    const Frame fr = *frp;
    float v[26];
    if (far) {
        const double th = tgt7[k], ph = tgt7[nt + k];
        const double rd[3] = {cos(ph) * sin(th), sin(ph) * sin(th), cos(th)};
        for (int c = 0; c < 3; ++c) {
            const double hd = rint(rd[c] * 2048.0) / 2048.0;
            v[c] = (float)hd;
            v[3 + c] = (float)(rd[c] - hd);
        }
    } else {
        for (int c = 0; c < 3; ++c) {
            const double x = (tgt7[c * nt + k] - fr.o[c]) * fr.kappa;
            const double hd = rint(x * fr.inv_q) * fr.q;
            v[c] = (float)hd;
            v[3 + c] = (float)(x - hd);
        }
    }
    double ge[6], gh[6], n[3];   // (re, im) x y z
    for (int c = 0; c < 3; ++c) {
        ge[2 * c] = real ? gam[c * nt + k] : 0.0;
        ge[2 * c + 1] = real ? gam[(3 + c) * nt + k] : 0.0;
        gh[2 * c] = real ? gam[(6 + c) * nt + k] : 0.0;
        gh[2 * c + 1] = real ? gam[(9 + c) * nt + k] : 0.0;
        n[c] = real && !far ? tgt7[(3 + c) * nt + k] : 0.0;
    }
    for (int q = 0; q < 6; ++q) {
        v[6 + q] = (float)ge[q];
        v[12 + q] = (float)gh[q];
    }
    // a = conj(gE), b = conj(gH): a.n and b.n
    for (int w = 0; w < 2; ++w) {
        const double *g = w == 0 ? ge : gh;
        const double dr = g[0] * n[0] + g[2] * n[1] + g[4] * n[2];
        const double di = -(g[1] * n[0] + g[3] * n[1] + g[5] * n[2]);
        const int dot_at = w == 0 ? 21 : 23;   // a.n | b.n
        v[dot_at] = (float)dr;
        v[dot_at + 1] = (float)di;
    }
    for (int c = 0; c < 3; ++c) v[18 + c] = far ? v[c] + v[3 + c] : (float)n[c];
    v[25] = 0.f;
    float *o = out + (i >> 1) * (long)(rec4 * 4) + (i & 1);
    for (int q = 0; q < 2 * rec4; ++q) o[2 * q] = v[q];
}

// Per-thread constants of the thread's source (forward-packed record).
struct SrcC {
    float sh[3], sl[3], n[3];
    float J[6], M[6];            // (re, im) x y z
    float Jn[2], Mn[2];          // J.n_s, M.n_s
};

// The geometry of a target pair record against the thread's source, in the
// split representation: S0 = |d_hi|^2 (exact), S1 the rest of |d|^2, 1/R
// (approximate), R, d = t - s, and n_s . d. adj_nf_pair2 and
// adj_nf_band_scan both use these, so the scan's band decision is the pair
// loop's, bit for bit.
struct AdjGeo2 {
    float2 S0, S1, rinv0, Rh, dx, dy, dz, ndd;
};

__device__ __forceinline__ AdjGeo2 adj_geo2(const float2 *r, const SrcC &s)
{
    AdjGeo2 g;
    const float2 dhx = sub2(r[0], dup2(s.sh[0])), dhy = sub2(r[1], dup2(s.sh[1])), dhz = sub2(r[2], dup2(s.sh[2]));
    const float2 dlx = sub2(r[3], dup2(s.sl[0])), dly = sub2(r[4], dup2(s.sl[1])), dlz = sub2(r[5], dup2(s.sl[2]));
    const float2 two = dup2(2.0f);
    g.S0 = fma2(dhz, dhz, fma2(dhy, dhy, mul2(dhx, dhx)));
    g.S1 = fma2(dlz, fma2(two, dhz, dlz), fma2(dly, fma2(two, dhy, dly), mul2(dlx, fma2(two, dhx, dlx))));
    const float2 R2 = add2(g.S0, g.S1);
    g.rinv0 = make_float2(rsqrt_ftz(R2.x), rsqrt_ftz(R2.y));
    g.Rh = mul2(R2, g.rinv0);
    g.dx = add2(dhx, dlx);
    g.dy = add2(dhy, dly);
    g.dz = add2(dhz, dlz);
    g.ndd = fma2(dup2(s.n[2]), g.dz, fma2(dup2(s.n[1]), g.dy, mul2(dup2(s.n[0]), g.dx)));
    return g;
}

// One pair of targets against the thread's source. acc: 12 current
// accumulators + the source displacement term; vt: the two targets' terms.
// band: set when a pair lies inside the tangent band (left out here; the
// kernel lists it afterwards with adj_band_scan).
template <int T, bool HAS_M, bool WANT_D, bool WANT_T>
__device__ __forceinline__ void adj_nf_pair2(float2 *acc, float2 &vt, const float2 *r, const SrcC &s, bool &band)
{
    const AdjGeo2 g = adj_geo2(r, s);
    const float2 S0 = g.S0, S1 = g.S1, rinv0 = g.rinv0, Rh = g.Rh, dx = g.dx, dy = g.dy, dz = g.dz, ndd = g.ndd;
    float2 sn, cs, tq;
    phase_sincos2(S0, S1, Rh, rinv0, sn, cs, tq);
    cs = flip_parity(cs, tq);   // cos, sin of k R
    sn = flip_parity(sn, tq);
    const float2 bw = mul2(dup2(kTangentBand), Rh);
    band = band || (fabsf(ndd.x) < bw.x) || (fabsf(ndd.y) < bw.y);
    const float2 rinv = make_float2(ndd.x >= bw.x ? rinv0.x : 0.0f, ndd.y >= bw.y ? rinv0.y : 0.0f);
    const float2 ex = mul2(dx, rinv), ey = mul2(dy, rinv), ez = mul2(dz, rinv);
    const float2 u = mul2(rinv, dup2(0.159154943091895336f));
    // c1 = Gu (t u + j(u^2 - 1)), C2 = -3 c1 - 2 j Gu, C3 = Gu (-u + j t)
    const float2 gur = mul2(cs, u);
    const float2 gui = mul2(T > 0 ? sn : neg2(sn), u);
    const float2 tu = T > 0 ? u : neg2(u);
    const float2 b = fma2(u, u, dup2(-1.0f));
    const float2 c1r = fma2(gur, tu, mul2(neg2(gui), b));
    const float2 c1i = fma2(gur, b, mul2(gui, tu));
    const float2 C2r = fma2(dup2(-3.0f), c1r, add2(gui, gui));
    const float2 C2i = fma2(dup2(-3.0f), c1i, mul2(dup2(-2.0f), gur));
    const float2 C3r = T > 0 ? fma2(neg2(gur), u, neg2(gui)) : fma2(neg2(gur), u, gui);
    const float2 C3i = T > 0 ? fma2(neg2(gui), u, gur) : fma2(neg2(gui), u, neg2(gur));

    const float2 Exr = r[6], Exi = r[7], Eyr = r[8], Eyi = r[9], Ezr = r[10], Ezi = r[11];
    const float2 Hxr = r[12], Hxi = r[13], Hyr = r[14], Hyi = r[15], Hzr = r[16], Hzi = r[17];
    // gE.R_hat, gH.R_hat
    const float2 ger = fma2(Ezr, ez, fma2(Eyr, ey, mul2(Exr, ex))), gei = fma2(Ezi, ez, fma2(Eyi, ey, mul2(Exi, ex)));
    const float2 ghr = fma2(Hzr, ez, fma2(Hyr, ey, mul2(Hxr, ex))), ghi = fma2(Hzi, ez, fma2(Hyi, ey, mul2(Hxi, ex)));
    // P = conj(C2) (gE.R_hat), Q = conj(C2) (gH.R_hat)
    const float2 Pr = fma2(C2r, ger, mul2(C2i, gei)), Pi = fma2(C2r, gei, mul2(neg2(C2i), ger));
    const float2 Qr = fma2(C2r, ghr, mul2(C2i, ghi)), Qi = fma2(C2r, ghi, mul2(neg2(C2i), ghr));
    // K = conj(C3) gH, L = conj(C3) gE
    const float2 Kxr = fma2(C3r, Hxr, mul2(C3i, Hxi)), Kxi = fma2(C3r, Hxi, mul2(neg2(C3i), Hxr));
    const float2 Kyr = fma2(C3r, Hyr, mul2(C3i, Hyi)), Kyi = fma2(C3r, Hyi, mul2(neg2(C3i), Hyr));
    const float2 Kzr = fma2(C3r, Hzr, mul2(C3i, Hzi)), Kzi = fma2(C3r, Hzi, mul2(neg2(C3i), Hzr));
    const float2 Lxr = fma2(C3r, Exr, mul2(C3i, Exi)), Lxi = fma2(C3r, Exi, mul2(neg2(C3i), Exr));
    const float2 Lyr = fma2(C3r, Eyr, mul2(C3i, Eyi)), Lyi = fma2(C3r, Eyi, mul2(neg2(C3i), Eyr));
    const float2 Lzr = fma2(C3r, Ezr, mul2(C3i, Ezi)), Lzi = fma2(C3r, Ezi, mul2(neg2(C3i), Ezr));
    // Jbar' += conj(c1) gE + P R_hat + K x R_hat
    acc[0] = fma2(c1r, Exr, fma2(c1i, Exi, fma2(Pr, ex, fma2(Kyr, ez, fma2(neg2(Kzr), ey, acc[0])))));
    acc[1] = fma2(c1r, Eyr, fma2(c1i, Eyi, fma2(Pr, ey, fma2(Kzr, ex, fma2(neg2(Kxr), ez, acc[1])))));
    acc[2] = fma2(c1r, Ezr, fma2(c1i, Ezi, fma2(Pr, ez, fma2(Kxr, ey, fma2(neg2(Kyr), ex, acc[2])))));
    acc[3] = fma2(c1r, Exi, fma2(neg2(c1i), Exr, fma2(Pi, ex, fma2(Kyi, ez, fma2(neg2(Kzi), ey, acc[3])))));
    acc[4] = fma2(c1r, Eyi, fma2(neg2(c1i), Eyr, fma2(Pi, ey, fma2(Kzi, ex, fma2(neg2(Kxi), ez, acc[4])))));
    acc[5] = fma2(c1r, Ezi, fma2(neg2(c1i), Ezr, fma2(Pi, ez, fma2(Kxi, ey, fma2(neg2(Kyi), ex, acc[5])))));
    // Mbar' += conj(c1) gH + Q R_hat - L x R_hat
    acc[6] = fma2(c1r, Hxr, fma2(c1i, Hxi, fma2(Qr, ex, fma2(neg2(Lyr), ez, fma2(Lzr, ey, acc[6])))));
    acc[7] = fma2(c1r, Hyr, fma2(c1i, Hyi, fma2(Qr, ey, fma2(neg2(Lzr), ex, fma2(Lxr, ez, acc[7])))));
    acc[8] = fma2(c1r, Hzr, fma2(c1i, Hzi, fma2(Qr, ez, fma2(neg2(Lxr), ey, fma2(Lyr, ex, acc[8])))));
    acc[9] = fma2(c1r, Hxi, fma2(neg2(c1i), Hxr, fma2(Qi, ex, fma2(neg2(Lyi), ez, fma2(Lzi, ey, acc[9])))));
    acc[10] = fma2(c1r, Hyi, fma2(neg2(c1i), Hyr, fma2(Qi, ey, fma2(neg2(Lzi), ex, fma2(Lxi, ez, acc[10])))));
    acc[11] = fma2(c1r, Hzi, fma2(neg2(c1i), Hzr, fma2(Qi, ez, fma2(neg2(Lxi), ey, fma2(Lyi, ex, acc[11])))));
    if (!WANT_D && !WANT_T) return;

    // a = conj(gE), b = conj(gH): alpha = a.J (+ b.M), beta = (J.R_hat)(a.R_hat) (+ (M.R_hat)(b.R_hat)),
    // w = W.R_hat = -b.(J x R_hat) (+ a.(M x R_hat))
    const float2 Jxr = dup2(s.J[0]), Jxi = dup2(s.J[1]), Jyr = dup2(s.J[2]), Jyi = dup2(s.J[3]);
    const float2 Jzr = dup2(s.J[4]), Jzi = dup2(s.J[5]);
    float2 alr = fma2(Ezr, Jzr, fma2(Ezi, Jzi, fma2(Eyr, Jyr, fma2(Eyi, Jyi, fma2(Exr, Jxr, mul2(Exi, Jxi))))));
    float2 ali = fma2(Ezr, Jzi, fma2(neg2(Ezi), Jzr, fma2(Eyr, Jyi, fma2(neg2(Eyi), Jyr, fma2(Exr, Jxi,
                      mul2(neg2(Exi), Jxr))))));
    const float2 jer = fma2(Jzr, ez, fma2(Jyr, ey, mul2(Jxr, ex))), jei = fma2(Jzi, ez, fma2(Jyi, ey, mul2(Jxi, ex)));
    float2 ber = fma2(jer, ger, mul2(jei, gei)), bei = fma2(jei, ger, mul2(neg2(jer), gei));
    // Z = b x J (- a x M): by the scalar triple product, W.v = -b.(J x v)
    // (+ a.(M x v)) = -v.Z for each of v = R_hat, n_s and n_t.
    float2 zxr = fma2(Hyr, Jzr, fma2(Hyi, Jzi, fma2(neg2(Hzr), Jyr, mul2(neg2(Hzi), Jyi))));
    float2 zxi = fma2(Hyr, Jzi, fma2(neg2(Hyi), Jzr, fma2(neg2(Hzr), Jyi, mul2(Hzi, Jyr))));
    float2 zyr = fma2(Hzr, Jxr, fma2(Hzi, Jxi, fma2(neg2(Hxr), Jzr, mul2(neg2(Hxi), Jzi))));
    float2 zyi = fma2(Hzr, Jxi, fma2(neg2(Hzi), Jxr, fma2(neg2(Hxr), Jzi, mul2(Hxi, Jzr))));
    float2 zzr = fma2(Hxr, Jyr, fma2(Hxi, Jyi, fma2(neg2(Hyr), Jxr, mul2(neg2(Hyi), Jxi))));
    float2 zzi = fma2(Hxr, Jyi, fma2(neg2(Hxi), Jyr, fma2(neg2(Hyr), Jxi, mul2(Hyi, Jxr))));
    float2 mer = dup2(0.f), mei = dup2(0.f);
    if (HAS_M) {
        const float2 Mxr = dup2(s.M[0]), Mxi = dup2(s.M[1]), Myr = dup2(s.M[2]), Myi = dup2(s.M[3]);
        const float2 Mzr = dup2(s.M[4]), Mzi = dup2(s.M[5]);
        alr = fma2(Hzr, Mzr, fma2(Hzi, Mzi, fma2(Hyr, Myr, fma2(Hyi, Myi, fma2(Hxr, Mxr, fma2(Hxi, Mxi, alr))))));
        ali = fma2(Hzr, Mzi, fma2(neg2(Hzi), Mzr, fma2(Hyr, Myi, fma2(neg2(Hyi), Myr, fma2(Hxr, Mxi,
                   fma2(neg2(Hxi), Mxr, ali))))));
        mer = fma2(Mzr, ez, fma2(Myr, ey, mul2(Mxr, ex)));
        mei = fma2(Mzi, ez, fma2(Myi, ey, mul2(Mxi, ex)));
        ber = fma2(mer, ghr, fma2(mei, ghi, ber));
        bei = fma2(mei, ghr, fma2(neg2(mer), ghi, bei));
        // Z -= a x M
        zxr = fma2(neg2(Eyr), Mzr, fma2(neg2(Eyi), Mzi, fma2(Ezr, Myr, fma2(Ezi, Myi, zxr))));
        zxi = fma2(neg2(Eyr), Mzi, fma2(Eyi, Mzr, fma2(Ezr, Myi, fma2(neg2(Ezi), Myr, zxi))));
        zyr = fma2(neg2(Ezr), Mxr, fma2(neg2(Ezi), Mxi, fma2(Exr, Mzr, fma2(Exi, Mzi, zyr))));
        zyi = fma2(neg2(Ezr), Mxi, fma2(Ezi, Mxr, fma2(Exr, Mzi, fma2(neg2(Exi), Mzr, zyi))));
        zzr = fma2(neg2(Exr), Myr, fma2(neg2(Exi), Myi, fma2(Eyr, Mxr, fma2(Eyi, Mxi, zzr))));
        zzi = fma2(neg2(Exr), Myi, fma2(Exi, Myr, fma2(Eyr, Mxi, fma2(neg2(Eyi), Mxr, zzi))));
    }
    const float2 wr = neg2(fma2(ez, zzr, fma2(ey, zyr, mul2(ex, zxr))));
    const float2 wi = neg2(fma2(ez, zzi, fma2(ey, zyi, mul2(ex, zxi))));
    // Re S, S = G (D1 alpha + D2 beta + D3 w), G = (cs, t sn)
    const float2 u2 = mul2(u, u);
    const float2 p1 = fma2(dup2(-3.0f), u2, dup2(1.0f));
    const float2 d1r = T > 0 ? p1 : neg2(p1), d1i = mul2(u, fma2(dup2(-3.0f), u2, dup2(2.0f)));
    const float2 p2 = fma2(dup2(-15.0f), u2, dup2(1.0f));
    const float2 d2r = T > 0 ? neg2(p2) : p2, d2i = mul2(u, fma2(dup2(15.0f), u2, dup2(-6.0f)));
    const float2 d3r = neg2(p1), d3i = mul2(u, dup2(T > 0 ? -3.0f : 3.0f));
    const float2 xr = fma2(d3r, wr, fma2(neg2(d3i), wi, fma2(d2r, ber, fma2(neg2(d2i), bei, fma2(d1r, alr,
                           mul2(neg2(d1i), ali))))));
    const float2 xi = fma2(d3r, wi, fma2(d3i, wr, fma2(d2r, bei, fma2(d2i, ber, fma2(d1r, ali, mul2(d1i, alr))))));
    const float2 gi = T > 0 ? sn : neg2(sn);
    const float2 Sr = fma2(cs, xr, mul2(neg2(gi), xi));

    if (WANT_D) {
        // W.n_s = -n_s.Z; grad(beta).n_s = (a.R_hat)(J.n_s) + (J.R_hat)(a.n_s) (+ M terms)
        const float2 nsx = dup2(s.n[0]), nsy = dup2(s.n[1]), nsz = dup2(s.n[2]);
        const float2 wnr = neg2(fma2(nsz, zzr, fma2(nsy, zyr, mul2(nsx, zxr))));
        const float2 wni = neg2(fma2(nsz, zzi, fma2(nsy, zyi, mul2(nsx, zxi))));
        const float2 anr = fma2(Ezr, nsz, fma2(Eyr, nsy, mul2(Exr, nsx)));
        const float2 ani = neg2(fma2(Ezi, nsz, fma2(Eyi, nsy, mul2(Exi, nsx))));
        float2 gbr = fma2(ger, dup2(s.Jn[0]), fma2(gei, dup2(s.Jn[1]), fma2(jer, anr, mul2(neg2(jei), ani))));
        float2 gbi = fma2(ger, dup2(s.Jn[1]), fma2(neg2(gei), dup2(s.Jn[0]), fma2(jer, ani, mul2(jei, anr))));
        if (HAS_M) {
            const float2 bnr = fma2(Hzr, nsz, fma2(Hyr, nsy, mul2(Hxr, nsx)));
            const float2 bni = neg2(fma2(Hzi, nsz, fma2(Hyi, nsy, mul2(Hxi, nsx))));
            gbr = fma2(ghr, dup2(s.Mn[0]), fma2(ghi, dup2(s.Mn[1]), fma2(mer, bnr, fma2(neg2(mei), bni, gbr))));
            gbi = fma2(ghr, dup2(s.Mn[1]), fma2(neg2(ghi), dup2(s.Mn[0]), fma2(mer, bni, fma2(mei, bnr, gbi))));
        }
        const float2 en = mul2(ndd, rinv);   // R_hat . n_s
        const float2 inner = fma2(en, Sr, fma2(C2r, gbr, fma2(neg2(C2i), gbi, fma2(C3r, wnr,
                                  mul2(neg2(C3i), wni)))));
        acc[12] = fma2(rinv, inner, acc[12]);
    }
    if (WANT_T) {
        // W.n_t = -n_t.Z; grad(beta).n_t = (a.R_hat)(J.n_t) + (J.R_hat)(a.n_t) (+ M terms)
        const float2 ntx = r[18], nty = r[19], ntz = r[20];
        const float2 ent = fma2(ez, ntz, fma2(ey, nty, mul2(ex, ntx)));
        const float2 jnr = fma2(Jzr, ntz, fma2(Jyr, nty, mul2(Jxr, ntx)));
        const float2 jni = fma2(Jzi, ntz, fma2(Jyi, nty, mul2(Jxi, ntx)));
        float2 gbr = fma2(ger, jnr, fma2(gei, jni, fma2(jer, r[21], mul2(neg2(jei), r[22]))));
        float2 gbi = fma2(ger, jni, fma2(neg2(gei), jnr, fma2(jer, r[22], mul2(jei, r[21]))));
        const float2 wnr = neg2(fma2(ntz, zzr, fma2(nty, zyr, mul2(ntx, zxr))));
        const float2 wni = neg2(fma2(ntz, zzi, fma2(nty, zyi, mul2(ntx, zxi))));
        if (HAS_M) {
            const float2 Mxr = dup2(s.M[0]), Mxi = dup2(s.M[1]), Myr = dup2(s.M[2]), Myi = dup2(s.M[3]);
            const float2 Mzr = dup2(s.M[4]), Mzi = dup2(s.M[5]);
            const float2 mnr = fma2(Mzr, ntz, fma2(Myr, nty, mul2(Mxr, ntx)));
            const float2 mni = fma2(Mzi, ntz, fma2(Myi, nty, mul2(Mxi, ntx)));
            gbr = fma2(ghr, mnr, fma2(ghi, mni, fma2(mer, r[23], fma2(neg2(mei), r[24], gbr))));
            gbi = fma2(ghr, mni, fma2(neg2(ghi), mnr, fma2(mer, r[24], fma2(mei, r[23], gbi))));
        }
        const float2 inner = fma2(ent, Sr, fma2(C2r, gbr, fma2(neg2(C2i), gbi, fma2(C3r, wnr,
                                  mul2(neg2(C3i), wni)))));
        vt = mul2(rinv, inner);
    }
}

// Scalar pair of targets against the thread's source (S' in the J.x slot,
// the cotangent g in the gE.x slot): the forward term is S' c with
// c = e^{-t j k R} / R, so
//   Sbar' += conj(c) g,
//   n . grad_d phi = (dphi/dR) (n . d) / R with phi = Re[conj(g) S' c] and
//   dc/dR = c (-t j k - 1 / R)   (k = 2 pi in turns);
// no illumination test (the reference's scalar sum has none).
template <int T, bool WANT_D, bool WANT_T>
__device__ __forceinline__ void adj_sc_pair2(float2 *acc, float2 &vt, const float2 *r, const SrcC &s)
{
    const float2 dhx = sub2(r[0], dup2(s.sh[0])), dhy = sub2(r[1], dup2(s.sh[1])), dhz = sub2(r[2], dup2(s.sh[2]));
    const float2 dlx = sub2(r[3], dup2(s.sl[0])), dly = sub2(r[4], dup2(s.sl[1])), dlz = sub2(r[5], dup2(s.sl[2]));
    const float2 two = dup2(2.0f);
    const float2 S0 = fma2(dhz, dhz, fma2(dhy, dhy, mul2(dhx, dhx)));
    const float2 S1 = fma2(dlz, fma2(two, dhz, dlz), fma2(dly, fma2(two, dhy, dly), mul2(dlx, fma2(two, dhx, dlx))));
    const float2 R2 = add2(S0, S1);
    const float2 rinv = make_float2(rsqrt_ftz(R2.x), rsqrt_ftz(R2.y));
    const float2 Rh = mul2(R2, rinv);
    float2 sn, cs, tq;
    phase_sincos2(S0, S1, Rh, rinv, sn, cs, tq);
    // c = G / R, G = e^{-t j 2 pi R} = cos - t j sin
    const float2 rs = flip_parity(rinv, tq);
    const float2 cr = mul2(cs, rs), ci = mul2(T > 0 ? neg2(sn) : sn, rs);
    const float2 gr = r[6], gi = r[7];
    acc[0] = fma2(cr, gr, fma2(ci, gi, acc[0]));
    acc[3] = fma2(cr, gi, fma2(neg2(ci), gr, acc[3]));
    if (!WANT_D && !WANT_T) return;
    // X = conj(g) S', Y = X c, dphi/dR = Re[Y (-1/R - t j 2 pi)] = -Y.re / R + t 2 pi Y.im
    const float2 Sr = dup2(s.J[0]), Si = dup2(s.J[1]);
    const float2 xr = fma2(gr, Sr, mul2(gi, Si)), xi = fma2(gr, Si, mul2(neg2(gi), Sr));
    const float2 yr = fma2(xr, cr, mul2(neg2(xi), ci)), yi = fma2(xr, ci, mul2(xi, cr));
    const float2 dphi = fma2(neg2(yr), rinv, mul2(yi, dup2(T > 0 ? 6.28318530717958647f : -6.28318530717958647f)));
    const float2 dx = add2(dhx, dlx), dy = add2(dhy, dly), dz = add2(dhz, dlz);
    const float2 g = mul2(dphi, rinv);
    if (WANT_D) {
        const float2 ndd = fma2(dup2(s.n[2]), dz, fma2(dup2(s.n[1]), dy, mul2(dup2(s.n[0]), dx)));
        acc[12] = fma2(g, ndd, acc[12]);
    }
    if (WANT_T) vt = mul2(g, fma2(r[20], dz, fma2(r[19], dy, mul2(r[18], dx))));
}

// Far-field pair of targets against the thread's source:
//   Jbar' += conj(G) gS_J, Mbar' += conj(G) gS_M (G = e^{-t j k r'.r_hat}),
//   source displacement: Re[-t j k G (conj(gS_J).J' + conj(gS_M).M')] (n_s . r_hat),
// k in turns is 2 pi.
// LIT: the tile is proven lit for the CTA's sources (every pair passes the
// illumination test), so the sign (-1)^q is set on the bits and the mask is
// left out; the result is the same bits.
__device__ __forceinline__ float2 adj_ff_ndr2(const float2 *r, const SrcC &s)
{
    return fma2(dup2(s.n[2]), r[20], fma2(dup2(s.n[1]), r[19], mul2(dup2(s.n[0]), r[18])));
}

template <int T, bool HAS_M, bool WANT_D, bool LIT, bool WIDE>
__device__ __forceinline__ void adj_ff_pair2(float2 *acc, const float2 *r, const SrcC &s, bool &band)
{
    // the phase of the source's offset w from its tile centre (the centre's
    // phase is already in the cotangents): narrow tiles p = r.w in FP32
    // (|w| <= kFFNarrow turns), reduced exactly to the nearest turn; wide
    // tiles from the split offset, reduced in half turns with a parity
    float2 sn, cs, tq = dup2(0.0f);
    if (WIDE) {
        const float2 Ph = fma2(dup2(s.sh[2]), r[2], fma2(dup2(s.sh[1]), r[1], mul2(dup2(s.sh[0]), r[0])));
        const float2 Pl = fma2(dup2(s.sl[2]), r[20], fma2(dup2(s.sl[1]), r[19], fma2(dup2(s.sl[0]), r[18],
                          fma2(dup2(s.sh[2]), r[5], fma2(dup2(s.sh[1]), r[4], mul2(dup2(s.sh[0]), r[3]))))));
        ff_phase_sincos2(Ph, Pl, sn, cs, tq);
    } else {
        const float2 magic = dup2(12582912.0f), twopi = dup2(6.28318530717958648f);
        const float2 P = fma2(dup2(s.sh[2]), r[20], fma2(dup2(s.sh[1]), r[19], mul2(dup2(s.sh[0]), r[18])));
        const float2 ang = mul2(sub2(P, sub2(add2(P, magic), magic)), twopi);
        __sincosf(ang.x, &sn.x, &cs.x);
        __sincosf(ang.y, &sn.y, &cs.y);
    }
    const float2 ndr = adj_ff_ndr2(r, s);
    float2 gc, gs;                                          // G = (gc, gs)
    if (LIT) {
        gc = WIDE ? flip_parity(cs, tq) : cs;
        gs = WIDE ? flip_parity(T > 0 ? neg2(sn) : sn, tq) : (T > 0 ? neg2(sn) : sn);
    } else {
        const float2 one = WIDE ? flip_parity(dup2(1.0f), tq) : dup2(1.0f);
        band = band || (fabsf(ndr.x) < kTangentBand) || (fabsf(ndr.y) < kTangentBand);
        const float2 m = make_float2(ndr.x >= kTangentBand ? one.x : 0.0f, ndr.y >= kTangentBand ? one.y : 0.0f);
        gc = mul2(cs, m);
        gs = mul2(T > 0 ? neg2(sn) : sn, m);
    }
    // conj(G) g = (gc g.re + gs g.im, gc g.im - gs g.re)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        acc[c] = fma2(gs, r[7 + 2 * c], fma2(gc, r[6 + 2 * c], acc[c]));
        acc[3 + c] = fma2(neg2(gs), r[6 + 2 * c], fma2(gc, r[7 + 2 * c], acc[3 + c]));
        acc[6 + c] = fma2(gs, r[13 + 2 * c], fma2(gc, r[12 + 2 * c], acc[6 + c]));
        acc[9 + c] = fma2(neg2(gs), r[12 + 2 * c], fma2(gc, r[13 + 2 * c], acc[9 + c]));
    }
    if (WANT_D) {
        // X = conj(gS_J).J' (+ conj(gS_M).M'); Z = G X, Im Z = gc X.im + gs X.re
        float2 xr = dup2(0.f), xi = dup2(0.f);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 jr = dup2(s.J[2 * c]), ji = dup2(s.J[2 * c + 1]);
            xr = fma2(r[6 + 2 * c], jr, fma2(r[7 + 2 * c], ji, xr));
            xi = fma2(r[6 + 2 * c], ji, fma2(neg2(r[7 + 2 * c]), jr, xi));
            if (HAS_M) {
                const float2 mr = dup2(s.M[2 * c]), mi = dup2(s.M[2 * c + 1]);
                xr = fma2(r[12 + 2 * c], mr, fma2(r[13 + 2 * c], mi, xr));
                xi = fma2(r[12 + 2 * c], mi, fma2(neg2(r[13 + 2 * c]), mr, xi));
            }
        }
        const float2 zi = fma2(gc, xi, mul2(gs, xr));
        acc[12] = fma2(mul2(zi, ndr), dup2(T > 0 ? 6.28318530717958647f : -6.28318530717958647f), acc[12]);
    }
}

// Direction box of each far-field cotangent tile (kPairsA2 pair records) for
// the lit-tile proof of the far-field adjoint: lowest and highest r_hat per
// axis, written into the unused slot 21 of the tile's first three pair
// records. One warp per tile; the padding target of an odd count repeats
// the last target, so it changes nothing.
__global__ void po_adj_tgt_box_kernel(float2 *__restrict__ rec, long nt)
{
    constexpr int R2 = 2 * adj2_rec(kKindFF, false, false);   // float2 slots per pair record
    float v[6] = {CUDART_INF_F, CUDART_INF_F, CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F};
    const long np = (nt + 1) / 2;
    for (int p = threadIdx.x; p < kPairsA2; p += 32) {
        const long pair = (long)blockIdx.x * kPairsA2 + p;
        if (pair >= np) break;
        const float2 *r = rec + pair * R2;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = fminf(v[c], fminf(r[18 + c].x, r[18 + c].y));
            v[3 + c] = fmaxf(v[3 + c], fmaxf(r[18 + c].x, r[18 + c].y));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float u = __shfl_xor_sync(0xffffffffu, v[q], o);
            v[q] = q < 3 ? fminf(v[q], u) : fmaxf(v[q], u);
        }
    if (threadIdx.x < 6) {
        const long pair = (long)blockIdx.x * kPairsA2 + (threadIdx.x >> 1);
        float *slot = reinterpret_cast<float *>(rec + pair * R2 + 21);
        if (pair < np) slot[threadIdx.x & 1] = v[threadIdx.x];
    }
}

// Far field: one stage's pair record of two directions (lanes), its
// cotangents gS_J, gS_M (slots 6-17, (re, im) per axis) multiplied in place by
// conj(e^{-t j k r.c}) for the CTA's tile centre c (hi xyz, lo xyz, turns).
// One thread per record: spreading a record over four threads (each forming
// the phase and rotating its share) measured 279.6 -> 297.0 ms on dish_ff.
// With s = c + w, conj(G) g = conj(G_w) (conj(G_c) g), so the pair loop needs
// only the offset's phase. r.c in split form: hi products exact (r hi on
// 2^-11, c hi on the frame's quantum), the rest in one FP32 sum, reduced
// exactly to half turns, as the forward's tile phase.
template <int T>
__device__ __forceinline__ void ff_rotate_cot(float4 *rec4, const float *c)
{
    float2 *r = reinterpret_cast<float2 *>(rec4);
    const float2 Ph = fma2(dup2(c[2]), r[2], fma2(dup2(c[1]), r[1], mul2(dup2(c[0]), r[0])));
    const float2 Pl = fma2(dup2(c[5]), r[20], fma2(dup2(c[4]), r[19], fma2(dup2(c[3]), r[18],
                      fma2(dup2(c[2]), r[5], fma2(dup2(c[1]), r[4], mul2(dup2(c[0]), r[3]))))));
    float2 sn, cs, tq;
    ff_phase_sincos2(Ph, Pl, sn, cs, tq);
    const float2 gc = flip_parity(cs, tq), gs = flip_parity(T > 0 ? neg2(sn) : sn, tq);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const float2 re = r[6 + 2 * q], im = r[7 + 2 * q];
        r[6 + 2 * q] = fma2(gc, re, mul2(gs, im));
        r[7 + 2 * q] = fma2(gc, im, mul2(neg2(gs), re));
    }
}

// The rare path of a tile in which some pair fell inside the tangent band:
// the thread's source is tested again against the tile's targets, with the
// pair loop's operations, and each pair inside the band is listed for the
// FP64 fixup (an idle source or padding target is only left out). tile:
// cnt target pair records (RT float4 each), the first with target index
// 2 * pfirst.
template <int KIND, int RT>
__device__ __forceinline__ void adj_band_scan(const float4 *tile, int cnt, long pfirst, const SrcC &s, long si,
                                              long ns, long nt, BandList bl)
{
    if (si >= ns) return;
#pragma unroll 1
    for (int p = 0; p < cnt; ++p) {
        float2 r[22];
        if (KIND == kKindFF) {
            const float4 v0 = tile[p * RT + 9], v1 = tile[p * RT + 10];   // float2 slots 18-21
            r[18] = make_float2(v0.x, v0.y);
            r[19] = make_float2(v0.z, v0.w);
            r[20] = make_float2(v1.x, v1.y);
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float4 v = tile[p * RT + c];
                r[2 * c] = make_float2(v.x, v.y);
                r[2 * c + 1] = make_float2(v.z, v.w);
            }
        }
        const float2 nd = KIND == kKindFF ? adj_ff_ndr2(r, s) : adj_geo2(r, s).ndd;
        const float2 bw = KIND == kKindFF ? dup2(kTangentBand) : mul2(dup2(kTangentBand), adj_geo2(r, s).Rh);
        const long t0 = 2 * (pfirst + p);
        if (fabsf(nd.x) < bw.x && t0 < nt) band_defer(bl, si, t0);
        if (fabsf(nd.y) < bw.y && t0 + 1 < nt) band_defer(bl, si, t0 + 1);
    }
}

template <int KIND, int T, bool HAS_M, bool WANT_D, bool WANT_T>
__global__ void __launch_bounds__(kThreadsA, KIND == kKindFF ? kMinBlocksFF : (HAS_M ? kMinBlocksA2M : kMinBlocksA2))
po_adj_pk_kernel(const float4 *__restrict__ srcpk, long ns, const float4 *__restrict__ trec, long nt, long chunk,
                 double *__restrict__ part, double *__restrict__ gt, int *__restrict__ err, int boxes, BandList bl,
                 const int *__restrict__ order)
{
    static_assert(KIND != kKindFF || !WANT_T, "far-field targets do not move");
    constexpr int RT = adj2_rec(KIND, HAS_M, WANT_T);
    constexpr int NL = 2 * RT;                    // float2 slots read per pair
    extern __shared__ __align__(128) float4 stage[];   // kStages * kPairsA2 * RT, lo, transpose buffer
    __shared__ __align__(8) uint64_t full[kStages];
    float *lo = reinterpret_cast<float *>(stage + (size_t)kStages * kPairsA2 * RT);
    float2 *vbuf = reinterpret_cast<float2 *>(lo + kAccAdj * kThreadsA);   // [kFlush][kThreadsA]

    SrcC s;
    long si;                 // the thread's source (its index in the caller's arrays)
    [[maybe_unused]] bool wide = false;     // far field: the CTA's tile stores split offsets
    [[maybe_unused]] float cen[6] = {};     // far field: the tile centre, hi xyz and lo xyz (turns)
    if constexpr (KIND == kKindFF) {
        // one CTA per far-field source tile (po_ff_pack_kernel's records, in
        // Hilbert order): the offset from the tile centre, J', the normal, M'
        constexpr int R4 = ff_rec4(HAS_M), T4 = ff_tile4(HAS_M);
        static_assert(kThreadsA == kTile, "one far-field source tile per adjoint CTA");
        const float *tf = reinterpret_cast<const float *>(srcpk + (size_t)blockIdx.x * T4);
#pragma unroll
        for (int c = 0; c < 6; ++c) cen[c] = tf[c];
        wide = tf[12] != 0.0f;
        const float *rec = tf + kFFHead * 4 + (threadIdx.x >> 1) * R4 * 4 + (threadIdx.x & 1);   // slot k: rec[2k]
        const long pos = (long)blockIdx.x * kThreadsA + threadIdx.x;
        si = pos < ns ? (long)order[pos] : ns;   // padding: past the end, never written
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            s.sh[c] = rec[2 * c];
            s.sl[c] = rec[2 * (12 + c)];
            s.n[c] = rec[2 * (9 + c)];
            s.J[2 * c] = rec[2 * (3 + c)];
            s.J[2 * c + 1] = rec[2 * (6 + c)];
            s.M[2 * c] = HAS_M ? rec[2 * (16 + c)] : 0.0f;
            s.M[2 * c + 1] = HAS_M ? rec[2 * (19 + c)] : 0.0f;
        }
    } else {
        si = (long)blockIdx.x * kThreadsA + threadIdx.x;
        float4 q[kRec];
#pragma unroll
        for (int c = 0; c < kRec; ++c) q[c] = si < ns ? srcpk[(size_t)kRec * si + c] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (si >= ns) q[0].z = 1e3f;   // idle lanes: keep R > 0 (zero currents)
        s.sh[0] = q[0].x; s.sh[1] = q[0].y; s.sh[2] = q[0].z;
        s.sl[0] = q[1].x; s.sl[1] = q[1].y; s.sl[2] = q[1].z;
        s.n[0] = q[0].w; s.n[1] = q[1].w; s.n[2] = q[5].x;
        const float jm[12] = {q[2].x, q[2].y, q[2].z, q[2].w, q[3].x, q[3].y, q[3].z, q[3].w, q[4].x, q[4].y, q[4].z,
                              q[4].w};
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            s.J[c] = jm[c];
            s.M[c] = jm[6 + c];
        }
    }
#pragma unroll
    for (int w = 0; w < 2; ++w) {
        const float *v = w == 0 ? s.J : s.M;
        float *dn = w == 0 ? s.Jn : s.Mn;
#pragma unroll
        for (int ri = 0; ri < 2; ++ri) dn[ri] = fmaf(v[4 + ri], s.n[2], fmaf(v[2 + ri], s.n[1], v[ri] * s.n[0]));
    }

    float hi[kAccAdj];
#pragma unroll
    for (int a = 0; a < kAccAdj; ++a) {
        hi[a] = 0.f;
        lo[a * kThreadsA + threadIdx.x] = 0.f;
    }

    // Far field, M = 0: the CTA's box of source normals for the lit-tile
    // proof (a tile's directions r_hat against it: min n.r_hat >= 1e-5, the
    // least of n.r over the two boxes being the sum of the least corner
    // products per axis; the per-pair test: lit when n.r_hat >= 1e-6). Only there: the
    // near-field adjoint needs n_s.R for its displacement gradient anyway,
    // and a second copy of the loop is not worth its cost with M.
    constexpr bool kLitA = KIND == kKindFF && !HAS_M;
    __shared__ float nbox_w[kThreadsA / 32][6];
    __shared__ float nbox[6];
    if (kLitA) {
        float v[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[c] = si < ns ? s.n[c] : CUDART_INF_F;
            v[3 + c] = si < ns ? s.n[c] : -CUDART_INF_F;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float u = __shfl_xor_sync(0xffffffffu, v[q], o);
                v[q] = q < 3 ? fminf(v[q], u) : fmaxf(v[q], u);
            }
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int q = 0; q < 6; ++q) nbox_w[threadIdx.x >> 5][q] = v[q];
        __syncthreads();
        if (threadIdx.x < 6) {
            const int q = threadIdx.x;
            float r = nbox_w[0][q];
            for (int w = 1; w < kThreadsA / 32; ++w) r = q < 3 ? fminf(r, nbox_w[w][q]) : fmaxf(r, nbox_w[w][q]);
            nbox[q] = r;
        }
    }

    const long t0 = (long)blockIdx.y * chunk;     // chunk: a multiple of 2 * kPairsA2 targets
    const long t1 = min(nt, t0 + chunk);
    const long p0 = t0 / 2, p1 = (t1 + 1) / 2;
    const int ntiles = p1 > p0 ? (int)((p1 - p0 + kPairsA2 - 1) / kPairsA2) : 0;
    if (threadIdx.x == 0) {
        for (int st = 0; st < kStages; ++st) mbar_init(&full[st], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int it) {
        const long first = p0 + (long)it * kPairsA2;
        const long cnt = min((long)kPairsA2, p1 - first);
        const uint32_t bytes = (uint32_t)(cnt * RT * sizeof(float4));
        uint64_t *bar = &full[it % kStages];
        fence_proxy_async();
        mbar_expect_tx(bar, bytes);
        tma_load_1d(stage + (size_t)(it % kStages) * kPairsA2 * RT, trec + first * RT, bytes, bar);
    };
    if (threadIdx.x == 0)
        for (int it = 0; it < ntiles && it < kStages; ++it) issue(it);

    for (int it = 0; it < ntiles; ++it) {
        const bool ok = mbar_wait_bounded(&full[it % kStages], (uint32_t)((it / kStages) & 1));
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicExch(err, kErrWaitTimeout);
                for (int st = 0; st < kStages; ++st) (void)mbar_wait_bounded(&full[st], 0);
            }
            return;
        }
        const float4 *tile = stage + (size_t)(it % kStages) * kPairsA2 * RT;
        const long pfirst = p0 + (long)it * kPairsA2;
        const int cnt = (int)min((long)kPairsA2, p1 - pfirst);
        if constexpr (KIND == kKindFF) {
            // the stage's cotangents times conj(e^{-t j k r.c}) for this CTA's tile centre c
            if (threadIdx.x < cnt)
                ff_rotate_cot<T>(stage + (size_t)(it % kStages) * kPairsA2 * RT + threadIdx.x * RT, cen);
            __syncthreads();
        }
        float2 acc[kAccAdj];
#pragma unroll
        for (int a = 0; a < kAccAdj; ++a) acc[a] = make_float2(0.f, 0.f);
        bool band = false;   // a pair of this tile fell inside the tangent band
        // block-uniform: the tile's direction box (in the first three pair
        // records, as po_adj_tgt_box_kernel wrote it) against the CTA's normals
        [[maybe_unused]] bool lit = false;
        if constexpr (kLitA) {
            if (boxes && cnt >= 3) {
                const float *f = reinterpret_cast<const float *>(tile);
                float L = 0.0f;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float tl = f[(c >> 1) * RT * 4 + 42 + (c & 1)];
                    const float th = f[((3 + c) >> 1) * RT * 4 + 42 + ((3 + c) & 1)];
                    L += fminf(fminf(nbox[c] * tl, nbox[c] * th), fminf(nbox[3 + c] * tl, nbox[3 + c] * th));
                }
                lit = L >= 1e-5f;
            }
        }
        for (int fb = 0; fb < cnt; fb += kFlush) {
            const int fend = min(cnt, fb + kFlush);
            if constexpr (KIND == kKindFF) {
                // far field: one copy of the pair loop per case, all block-uniform.
                // LIT: the tile is proven lit (M = 0), so the mask is left out.
                // WIDE: the CTA's offsets are split, so the phase is too.
                auto pairs = [&](auto lit_c, auto wide_c) {
                    constexpr bool LIT = decltype(lit_c)::value, WIDE = decltype(wide_c)::value;
#pragma unroll kUnrollA
                    for (int p = fb; p < fend; ++p) {
                        float2 rec[NL];
#pragma unroll
                        for (int c = 0; c < RT; ++c) {
                            const float4 v = tile[p * RT + c];
                            rec[2 * c] = make_float2(v.x, v.y);
                            rec[2 * c + 1] = make_float2(v.z, v.w);
                        }
                        adj_ff_pair2<T, HAS_M, WANT_D, LIT, WIDE>(acc, rec, s, band);
                    }
                };
                if (wide)
                    pairs(std::false_type{}, std::true_type{});
                else if (lit)
                    pairs(std::bool_constant<kLitA>{}, std::false_type{});
                else
                    pairs(std::false_type{}, std::false_type{});
            } else {
#pragma unroll kUnrollA
                for (int p = fb; p < fend; ++p) {
                    float2 rec[NL];
#pragma unroll
                    for (int c = 0; c < RT; ++c) {
                        const float4 v = tile[p * RT + c];
                        rec[2 * c] = make_float2(v.x, v.y);
                        rec[2 * c + 1] = make_float2(v.z, v.w);
                    }
                    float2 vt = make_float2(0.f, 0.f);
                    if (KIND == kKindNF)
                        adj_nf_pair2<T, HAS_M, WANT_D, WANT_T>(acc, vt, rec, s, band);
                    else adj_sc_pair2<T, WANT_D, WANT_T>(acc, vt, rec, s);
                    if (WANT_T) vbuf[(p - fb) * kThreadsA + threadIdx.x] = vt;
                }
            }
            if (WANT_T) {
                // Sum the CTA's sources for each target pair of this flush: thread
                // (pl, k) adds kThreadsA / kSegs sources of pair pl (rotated reads:
                // the 8 threads of a shared-memory phase hit distinct banks), then
                // the kSegs segments combine by shuffles.
                __syncthreads();
                constexpr int kPer = kThreadsA / kSegs / 2;   // float4 (two sources each) per thread
                const int pl = threadIdx.x / kSegs, k = threadIdx.x % kSegs;
                const int rot = kSegs == 8 ? k : 4 * (pl & 1) + k;
                float2 sum = make_float2(0.f, 0.f);
                if (pl < fend - fb) {
                    const float4 *row = reinterpret_cast<const float4 *>(vbuf + pl * kThreadsA);
#pragma unroll
                    for (int j = 0; j < kPer; ++j) {
                        const float4 v = row[kPer * k + ((j + rot) & (kPer - 1))];
                        sum = add2(sum, add2(make_float2(v.x, v.y), make_float2(v.z, v.w)));
                    }
                }
#pragma unroll
                for (int m = 1; m < kSegs; m <<= 1) {
                    sum.x += __shfl_xor_sync(0xffffffffu, sum.x, m);
                    sum.y += __shfl_xor_sync(0xffffffffu, sum.y, m);
                }
                if (k == 0 && pl < fend - fb) {
                    const long tg = 2 * (pfirst + fb + pl);
                    if (tg < nt) atomicAdd(&gt[tg], (double)sum.x);
                    if (tg + 1 < nt) atomicAdd(&gt[tg + 1], (double)sum.y);
                }
                __syncthreads();
            }
        }
#pragma unroll
        for (int a = 0; a < kAccAdj; ++a) {
            float sm, e;
            two_sum(hi[a], __fadd_rn(acc[a].x, acc[a].y), sm, e);
            hi[a] = sm;
            float &l = lo[a * kThreadsA + threadIdx.x];
            l = __fadd_rn(l, e);
        }
        if (KIND != kKindScalar && band) adj_band_scan<KIND, RT>(tile, cnt, pfirst, s, si, ns, nt, bl);
        __syncthreads();
        if (threadIdx.x == 0 && it + kStages < ntiles) issue(it + kStages);
    }
    if (si >= ns) return;
#pragma unroll
    for (int a = 0; a < kAccAdj; ++a)
        part[((long)blockIdx.y * kAccAdj + a) * ns + si] = (double)hi[a] + (double)lo[a * kThreadsA + threadIdx.x];
}

int adj_pk_smem_bytes(int kind, bool has_m, bool want_t)
{
    return kStages * kPairsA2 * adj2_rec(kind, has_m, want_t) * 16 + kAccAdj * kThreadsA * 4 +
           (want_t ? kFlush * kThreadsA * 8 : 0);
}

int adj_pk_pairs_per_tile() { return kPairsA2; }

int adj_pk_rec4(int kind, bool has_m, bool want_t) { return adj2_rec(kind, has_m, want_t); }

void *adj_tgt_box_kernel() { return reinterpret_cast<void *>(&po_adj_tgt_box_kernel); }

template <int KIND, int T, bool HAS_M, bool WANT_D, bool WANT_T>
static void *adj_pk_ptr()
{
    return reinterpret_cast<void *>(&po_adj_pk_kernel<KIND, T, HAS_M, WANT_D, WANT_T>);
}

template <int T, bool HAS_M>
static void *adj_pk_sel(int kind, bool want_d, bool want_t)
{
    if (kind == kKindFF) return want_d ? adj_pk_ptr<kKindFF, T, HAS_M, true, false>()
                                       : adj_pk_ptr<kKindFF, T, HAS_M, false, false>();
    if (kind == kKindScalar) {
        if (want_d) return want_t ? adj_pk_ptr<kKindScalar, T, false, true, true>()
                                  : adj_pk_ptr<kKindScalar, T, false, true, false>();
        return want_t ? adj_pk_ptr<kKindScalar, T, false, false, true>() : adj_pk_ptr<kKindScalar, T, false, false, false>();
    }
    if (want_d) return want_t ? adj_pk_ptr<kKindNF, T, HAS_M, true, true>() : adj_pk_ptr<kKindNF, T, HAS_M, true, false>();
    return want_t ? adj_pk_ptr<kKindNF, T, HAS_M, false, true>() : adj_pk_ptr<kKindNF, T, HAS_M, false, false>();
}

void *adj_pk_kernel(int kind, int t_sign, bool has_m, bool want_d, bool want_t)
{
    if (t_sign < 0) return has_m ? adj_pk_sel<-1, true>(kind, want_d, want_t) : adj_pk_sel<-1, false>(kind, want_d, want_t);
    return has_m ? adj_pk_sel<1, true>(kind, want_d, want_t) : adj_pk_sel<1, false>(kind, want_d, want_t);
}

void *adj_pack_tgt2_kernel() { return reinterpret_cast<void *>(&po_adj_pack_tgt2_kernel); }

}  // namespace po
