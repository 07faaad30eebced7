// po_farfield.cu -- far-field forward (mode FF) of the physical-optics
// integrator, with the phase of every source tile factored out.
//
// The far field in direction r is a sum over sources s of G J' with
// G = e^{-t j k r.s} (reference src/CPU/Propagation.h:1656-1781; the
// projection onto the transverse plane is linear and done once per direction
// in the FP64 epilogue). r.s reaches ~1e4 turns on the large dishes, so a
// direct FP32 phase is useless; computing it in split hi/lo form per pair
// costs as much as the physics. Here the sources are ordered along a 2-D
// Hilbert curve (po_ff_key_kernel, then a radix sort), so that every kTile
// consecutive sources form a compact tile with centre c, and
//   e^{-t j k r.s} = e^{-t j k r.c} e^{-t j k r.(s - c)}.
//   * per pair: p = r.(s - c) in FP32 (the offsets span only the tile, tens
//     of turns, so FP32 holds p to ~1e-6 turns), one exact reduction to the
//     nearest turn, sin/cos of the remainder on the SFU, and the complex
//     accumulation of G J' into the tile's FP32 sums;
//   * per (direction, tile): r.c in split hi/lo form, reduced exactly
//     (ff_phase_sincos2, the two directions of a thread in the two lanes),
//     the tile's sums rotated by e^{-t j k r.c} and folded into float-float
//     totals (two-sum).
// FP32 holds p to about 2^-24 of the tile's radius, so a tile wider than
// kFFNarrow turns (a sparsely sampled surface) splits its offsets instead:
// hi parts on a power-of-two quantum with at most 11 significant bits (their
// products with the directions' hi parts, on 2^-11, are exact) and small lo
// parts, and reduces p as the tile phase is reduced; the choice is per tile
// and block-uniform.
// Each tile is one record block: a 64-byte header (centre hi xyz, lo xyz on
// the frame's quantum; the tile's box of normals for the lit-tile proof; the
// wide-tile flag) followed by 64 pair records (float2 slots: offset (or its
// hi part) xyz, J' re xyz, J' im xyz, normal xyz, the offset's lo part xyz
// (wide tiles), a spare slot, then M' re xyz, im xyz). The main kernel
// streams tiles through shared memory with 1-D TMA bulk copies on
// mbarriers, 3 stages deep, with the bounded waits of the other kernels.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cstdint>
#include <type_traits>

#include <cub/device/device_radix_sort.cuh>

#include "po_device.cuh"
#include "po_kernels.cuh"

namespace po {

// ---------------------------------------------------------------- ordering

// Index of (x, y) along the Hilbert curve of a 2^21 x 2^21 grid (the usual
// quadrant recursion: at each level the quadrant's number, then the rotation
// or reflection that makes the sub-curve continue the parent's).
__device__ __forceinline__ unsigned long long hilbert_index(uint32_t x, uint32_t y)
{
    constexpr uint32_t n = 1u << 21;
    unsigned long long d = 0;
    for (uint32_t s = n >> 1; s > 0; s >>= 1) {
        const uint32_t rx = (x & s) ? 1u : 0u, ry = (y & s) ? 1u : 0u;
        d += (unsigned long long)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = n - 1 - x;
                y = n - 1 - y;
            }
            const uint32_t t = x;
            x = y;
            y = t;
        }
    }
    return d;
}

// Sort keys of the sources: the Hilbert index of their projection onto the
// two axes along which their box is widest, on one common scale.
__global__ void po_ff_key_kernel(long ns, const double *__restrict__ src7, const Frame *__restrict__ frp,
                                 unsigned long long *__restrict__ key, int *__restrict__ idx)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns) return;
    const Frame fr = *frp;
    double ext[3];
    for (int c = 0; c < 3; ++c) ext[c] = fr.hi[c] - fr.lo[c];
    int a0 = 0;
    for (int c = 1; c < 3; ++c)
        if (ext[c] > ext[a0]) a0 = c;
    int a1 = a0 == 0 ? 1 : 0;
    for (int c = 0; c < 3; ++c)
        if (c != a0 && ext[c] > ext[a1]) a1 = c;
    const double span = fmax(ext[a0], ext[a1]);
    const double top = (double)((1u << 21) - 1);
    const double sc = span > 0.0 ? top / span : 0.0;
    const double u = fmin(fmax((src7[a0 * ns + i] - fr.lo[a0]) * sc, 0.0), top);
    const double v = fmin(fmax((src7[a1 * ns + i] - fr.lo[a1]) * sc, 0.0), top);
    key[i] = hilbert_index((uint32_t)u, (uint32_t)v);
    idx[i] = (int)i;
}

// Bits of the sort key.
constexpr int kFFKeyBits = 42;

// ------------------------------------------------------------------ packing

// One warp per tile of kTile sources in curve order: the tile's box gives its
// centre c (FP64, turns) and its box of normals; every source's record holds
// its offset s - c (FP32) and its currents times the trapezoid weight, the
// area and the complex prefactor. The tile is assembled in shared memory and
// written out in coalesced float4. The last tile is padded with copies of the
// last source carrying zero currents.
template <bool HAS_M>
__global__ void __launch_bounds__(32)
po_ff_pack_kernel(long ns, const int *__restrict__ order, const double *__restrict__ src7,
                  const double *__restrict__ cur, int gmode, int ncx, int ncy, const Frame *__restrict__ frp,
                  double fac_re, double fac_im, float4 *__restrict__ out)
{
    constexpr int R4 = ff_rec4(HAS_M), T4 = ff_tile4(HAS_M);
    constexpr int PER = kTile / 32;   // sources per lane
    __shared__ __align__(16) float4 buf[T4];
    float *bf = reinterpret_cast<float *>(buf);
    const Frame fr = *frp;
    const long first = (long)blockIdx.x * kTile;
    const int lane = threadIdx.x;

    double p[PER][3];
    long src[PER];
    bool real[PER];
    double lo[3] = {CUDART_INF, CUDART_INF, CUDART_INF}, hi[3] = {-CUDART_INF, -CUDART_INF, -CUDART_INF};
    float nlo[3] = {CUDART_INF_F, CUDART_INF_F, CUDART_INF_F}, nhi[3] = {-CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F};
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const long j = first + lane + 32 * q;
        real[q] = j < ns;
        const long k = order[real[q] ? j : ns - 1];
        src[q] = k;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            p[q][c] = (src7[c * ns + k] - fr.o[c]) * fr.kappa;
            lo[c] = fmin(lo[c], p[q][c]);
            hi[c] = fmax(hi[c], p[q][c]);
            const float nv = (float)src7[(3 + c) * ns + k];
            nlo[c] = fminf(nlo[c], nv);
            nhi[c] = fmaxf(nhi[c], nv);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
            nlo[c] = fminf(nlo[c], __shfl_xor_sync(0xffffffffu, nlo[c], o));
            nhi[c] = fmaxf(nhi[c], __shfl_xor_sync(0xffffffffu, nhi[c], o));
        }
    double cen[3], half[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        cen[c] = 0.5 * (lo[c] + hi[c]);
        half[c] = 0.5 * (hi[c] - lo[c]);
    }
    // narrow: the box's half-diagonal within kFFNarrow turns; a wide tile's
    // offsets split on the smallest power of two q with max |offset| <= 1024 q
    const bool wide = !(sqrt(half[0] * half[0] + half[1] * half[1] + half[2] * half[2]) <= (double)kFFNarrow);
    const double hmax = fmax(half[0], fmax(half[1], half[2]));
    double qt = 0x1p-40;
    for (int g = 0; g < 1100 && wide && qt * 1024.0 < hmax; ++g) qt *= 2.0;
    if (lane < 3) {
        float h, l;
        split_hi_lo(cen[lane], fr, h, l);
        bf[lane] = h;
        bf[3 + lane] = l;
        bf[6 + lane] = nlo[lane];
        bf[9 + lane] = nhi[lane];
    } else if (lane < 7) {
        bf[9 + lane] = lane == 3 && wide ? 1.0f : 0.0f;   // float 12: the wide-tile flag; 13-15 spare
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int jt = lane + 32 * q;
        float *rec = bf + (kFFHead + (jt >> 1) * R4) * 4 + (jt & 1);
        const long k = src[q];
        const double w = real[q] ? trap_weight(k, gmode, ncx, ncy) * src7[6 * ns + k] : 0.0;
        const double fr_ = fac_re * w, fi_ = fac_im * w;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double off = p[q][c] - cen[c];
            const double oh = wide ? rint(off / qt) * qt : off;
            rec[2 * c] = (float)oh;
            rec[2 * (12 + c)] = (float)(off - oh);   // 0 in a narrow tile
            const double jr = cur[c * ns + k], ji = cur[(3 + c) * ns + k];
            rec[2 * (3 + c)] = (float)(fr_ * jr - fi_ * ji);
            rec[2 * (6 + c)] = (float)(fr_ * ji + fi_ * jr);
            rec[2 * (9 + c)] = (float)src7[(3 + c) * ns + k];
            if (HAS_M) {
                const double mr = cur[(6 + c) * ns + k], mi = cur[(9 + c) * ns + k];
                rec[2 * (16 + c)] = (float)(fr_ * mr - fi_ * mi);
                rec[2 * (19 + c)] = (float)(fr_ * mi + fi_ * mr);
            }
        }
        rec[2 * 15] = 0.0f;
    }
    __syncwarp();
    float4 *dst = out + (size_t)blockIdx.x * T4;
    for (int q = lane; q < T4; q += 32) dst[q] = buf[q];
}

// ---------------------------------------------------------------- main kernel

// n_s . r_hat for a pair record's two sources (normals in float2 slots 9-11)
// and one direction duplicated into both lanes; the pair loop and the band
// scan both use it, so the scan's decision is the loop's, bit for bit.
__device__ __forceinline__ float2 ff_ndr2(const float2 *r, const float2 *rf)
{
    return fma2(r[11], rf[2], fma2(r[10], rf[1], mul2(r[9], rf[0])));
}

// The rare path of a tile in which some pair fell inside the tangent band:
// the thread's pairs are tested again and each one inside the band is
// listed for the FP64 fixup under the source's original index (curve
// position -> order); padding sources and idle directions are only left
// out. recs: the tile's kTile / 2 pair records (R4 float4 each); pos0: the
// curve position of its first source.
template <int TP, int R4>
__device__ __forceinline__ void ff_band_scan(const float4 *recs, long pos0, const float2 (*rf)[3], long tbase, long ns,
                                             long nt, const int *__restrict__ order, BandList bl)
{
#pragma unroll 1
    for (int s = 0; s < kTile / 2; ++s) {
        float2 r[12];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float4 v = recs[s * R4 + q];
            r[2 * q] = make_float2(v.x, v.y);
            r[2 * q + 1] = make_float2(v.z, v.w);
        }
        const long pos = pos0 + 2 * s;
#pragma unroll
        for (int j = 0; j < TP; ++j) {
            const long ti = tbase + (long)j * kThreads;
            const float2 ndr = ff_ndr2(r, rf[j]);
            if (fabsf(ndr.x) < kTangentBand && ti < nt && pos < ns) band_defer(bl, order[pos], ti);
            if (fabsf(ndr.y) < kTangentBand && ti < nt && pos + 1 < ns) band_defer(bl, order[pos + 1], ti);
        }
    }
}

// Grid = (direction blocks of 2 * kThreads, tile chunks). Every thread owns
// two directions (lanes of the per-tile phase); each pair record's two
// sources are the two lanes of every packed operation of the pair loop.
// `boxes`: the tiles' normal boxes may prove a tile lit for the CTA's
// directions (M = 0 kernels), which skips the per-pair illumination test.
template <int T, bool HAS_M>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
po_ff_kernel(const float4 *__restrict__ src, long ntiles, long chunk, const float4 *__restrict__ tgt, long nt,
             double *__restrict__ part, int *__restrict__ err, int boxes, BandList bl, long ns,
             const int *__restrict__ order)
{
    constexpr int R4 = ff_rec4(HAS_M), T4 = ff_tile4(HAS_M), TP = 2;
    constexpr int NA = HAS_M ? 12 : 6;   // accumulators in use: S_J (re xyz, im xyz), then S_M
    constexpr bool kLitPath = !HAS_M;
    extern __shared__ __align__(128) float4 stage[];   // kStages tiles, then the compensation words
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ float tbox_w[kThreads / 32][6];
    __shared__ float tbox[6];

    const long tbase = (long)blockIdx.x * kThreads * TP + threadIdx.x;
    float2 rf[TP][3];          // direction in FP32, duplicated into both lanes
    float2 rh[3], rl[3], rw[3];   // hi, lo and FP32 direction; lane j = direction j
#pragma unroll
    for (int j = 0; j < TP; ++j) {
        const long ti = tbase + (long)j * kThreads;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), c = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ti < nt) {
            a = tgt[2 * ti];
            c = tgt[2 * ti + 1];
        }
        const float h[3] = {a.x, a.y, a.z}, l[3] = {a.w, c.x, c.y};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float f = h[q] + l[q];
            rf[j][q] = dup2(f);
            if (j == 0) {
                rh[q].x = h[q];
                rl[q].x = l[q];
                rw[q].x = f;
            } else {
                rh[q].y = h[q];
                rl[q].y = l[q];
                rw[q].y = f;
            }
        }
    }

    // The CTA's box of directions (the lit-tile proof, M = 0 kernels).
    if (kLitPath) {
        float v[6] = {CUDART_INF_F, CUDART_INF_F, CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F};
#pragma unroll
        for (int j = 0; j < TP; ++j) {
            if (tbase + (long)j * kThreads >= nt) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                v[c] = fminf(v[c], rf[j][c].x);
                v[3 + c] = fmaxf(v[3 + c], rf[j][c].x);
            }
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
            for (int q = 0; q < 6; ++q) tbox_w[threadIdx.x >> 5][q] = v[q];
        __syncthreads();
        if (threadIdx.x < 6) {
            const int q = threadIdx.x;
            float r = tbox_w[0][q];
            for (int w = 1; w < kThreads / 32; ++w) r = q < 3 ? fminf(r, tbox_w[w][q]) : fmaxf(r, tbox_w[w][q]);
            tbox[q] = r;
        }
    }

    float hi[TP][NA];
    float *lo = reinterpret_cast<float *>(stage + (size_t)kStages * T4);
#pragma unroll
    for (int j = 0; j < TP; ++j)
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            hi[j][a] = 0.f;
            lo[(a * TP + j) * kThreads + threadIdx.x] = 0.f;
        }

    const long t0 = (long)blockIdx.y * chunk;
    const int ntl = (int)max(0L, min(ntiles, t0 + chunk) - t0);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
        mbar_fence_init();
    }
    __syncthreads();

    auto issue = [&](int it) {
        constexpr uint32_t bytes = (uint32_t)(T4 * sizeof(float4));
        uint64_t *bar = &full[it % kStages];
        fence_proxy_async();
        mbar_expect_tx(bar, bytes);
        tma_load_1d(stage + (size_t)(it % kStages) * T4, src + (t0 + it) * T4, bytes, bar);
    };
    if (threadIdx.x == 0)
        for (int it = 0; it < ntl && it < kStages; ++it) issue(it);

    const float2 magic = dup2(12582912.0f), twopi = dup2(6.28318530717958648f);
    bool aborted = false;
    for (int it = 0; it < ntl; ++it) {
        const bool ok = mbar_wait_bounded(&full[it % kStages], (uint32_t)((it / kStages) & 1));
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicExch(err, kErrWaitTimeout);
            aborted = true;
            break;
        }
        const float4 *tile = stage + (size_t)(it % kStages) * T4;
        const float *hdr = reinterpret_cast<const float *>(tile);
        float2 acc[TP][NA];
#pragma unroll
        for (int j = 0; j < TP; ++j)
#pragma unroll
            for (int a = 0; a < NA; ++a) acc[j][a] = make_float2(0.f, 0.f);

        bool band = false;   // a pair of this tile fell inside the tangent band
        // VAR 0: narrow tile proven lit (M = 0); 1: narrow tile; 2: wide tile
        auto pairs = [&](auto var_c) {
            constexpr int VAR = decltype(var_c)::value;
            // float4 read per pair record: offsets and J' (and the normal
            // unless the tile is proven lit; the lo offsets in a wide tile;
            // M')
            constexpr int NLD = HAS_M ? R4 : (VAR == 0 ? 5 : (VAR == 1 ? 6 : 8));
            const float4 *recs = tile + kFFHead;
#pragma unroll 2
            for (int s = 0; s < kTile / 2; ++s) {
                float2 r[2 * NLD];
#pragma unroll
                for (int q = 0; q < NLD; ++q) {
                    const float4 v = recs[s * R4 + q];
                    r[2 * q] = make_float2(v.x, v.y);
                    r[2 * q + 1] = make_float2(v.z, v.w);
                }
#pragma unroll
                for (int j = 0; j < TP; ++j) {
                    float2 gc, gs;
                    if (VAR < 2) {
                        // p = r . (s - c) in turns; y = p - rint(p), exact, |y| <= 1/2
                        const float2 P = fma2(r[2], rf[j][2], fma2(r[1], rf[j][1], mul2(r[0], rf[j][0])));
                        const float2 y = sub2(P, sub2(add2(P, magic), magic));
                        const float2 ang = mul2(y, twopi);
                        float2 sn, cs;
                        __sincosf(ang.x, &sn.x, &cs.x);
                        __sincosf(ang.y, &sn.y, &cs.y);
                        // G = e^{-t j 2 pi p} = cos - t j sin
                        gc = cs;
                        gs = T > 0 ? neg2(sn) : sn;
                    } else {
                        // p = r_hi . s_hi (exact) + (r . s_lo + r_lo . s_hi), reduced in half turns
                        const float2 hx = dup2(j == 0 ? rh[0].x : rh[0].y), hy = dup2(j == 0 ? rh[1].x : rh[1].y),
                                     hz = dup2(j == 0 ? rh[2].x : rh[2].y);
                        const float2 lx = dup2(j == 0 ? rl[0].x : rl[0].y), ly = dup2(j == 0 ? rl[1].x : rl[1].y),
                                     lz = dup2(j == 0 ? rl[2].x : rl[2].y);
                        const float2 Ph = fma2(r[2], hz, fma2(r[1], hy, mul2(r[0], hx)));
                        const float2 Pl = fma2(r[14], rf[j][2], fma2(r[13], rf[j][1], fma2(r[12], rf[j][0],
                                          fma2(r[2], lz, fma2(r[1], ly, mul2(r[0], lx))))));
                        float2 sn, cs, tq;
                        ff_phase_sincos2(Ph, Pl, sn, cs, tq);
                        gc = flip_parity(cs, tq);
                        gs = flip_parity(T > 0 ? neg2(sn) : sn, tq);
                    }
                    if (VAR != 0) {
                        // lit when n . r >= the band, not when below minus it; a pair
                        // inside it is left out here and listed afterwards (ff_band_scan)
                        const float2 ndr = ff_ndr2(r, rf[j]);
                        band = band || (fabsf(ndr.x) < kTangentBand) || (fabsf(ndr.y) < kTangentBand);
                        const float2 m = make_float2(ndr.x >= kTangentBand ? 1.0f : 0.0f, ndr.y >= kTangentBand ? 1.0f : 0.0f);
                        gc = mul2(gc, m);
                        gs = mul2(gs, m);
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        acc[j][c] = fma2(neg2(gs), r[6 + c], fma2(gc, r[3 + c], acc[j][c]));
                        acc[j][3 + c] = fma2(gs, r[3 + c], fma2(gc, r[6 + c], acc[j][3 + c]));
                        if (HAS_M) {
                            acc[j][6 + c] = fma2(neg2(gs), r[19 + c], fma2(gc, r[16 + c], acc[j][6 + c]));
                            acc[j][9 + c] = fma2(gs, r[16 + c], fma2(gc, r[19 + c], acc[j][9 + c]));
                        }
                    }
                }
            }
        };
        bool lit = false;
        if (kLitPath && boxes) {
            // every pair lit when the least n . r over the tile's box of
            // normals and the CTA's box of directions is at least 1e-5 (the
            // per-pair test is lit when n . r >= 1e-6): the least of n r over n in
            // [a, b], r in [c, d] is the least of the four corner products
            float L = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float a = hdr[6 + c], b = hdr[9 + c];
                L += fminf(fminf(a * tbox[c], a * tbox[3 + c]), fminf(b * tbox[c], b * tbox[3 + c]));
            }
            lit = L >= 1e-5f;   // block-uniform: every thread reads the same boxes
        }
        // block-uniform as well
        if (hdr[12] != 0.0f)
            pairs(std::integral_constant<int, 2>{});
        else if (kLitPath && lit)
            pairs(std::integral_constant<int, 0>{});
        else
            pairs(std::integral_constant<int, 1>{});

        // The tile's phase r . c for both directions (lanes): hi products
        // exact, the rest in one FP32 sum; reduced exactly to half turns.
        const float ch[3] = {hdr[0], hdr[1], hdr[2]}, cl[3] = {hdr[3], hdr[4], hdr[5]};
        const float2 Ph = fma2(dup2(ch[2]), rh[2], fma2(dup2(ch[1]), rh[1], mul2(dup2(ch[0]), rh[0])));
        const float2 Pl = fma2(dup2(cl[2]), rw[2], fma2(dup2(cl[1]), rw[1], fma2(dup2(cl[0]), rw[0],
                          fma2(dup2(ch[2]), rl[2], fma2(dup2(ch[1]), rl[1], mul2(dup2(ch[0]), rl[0]))))));
        float2 sn, cs, tq;
        ff_phase_sincos2(Ph, Pl, sn, cs, tq);
        const float2 gc = flip_parity(cs, tq), gs = flip_parity(T > 0 ? neg2(sn) : sn, tq);
#pragma unroll
        for (int j = 0; j < TP; ++j) {
            const float c0 = j == 0 ? gc.x : gc.y, s0 = j == 0 ? gs.x : gs.y;
#pragma unroll
            for (int g = 0; g < NA / 6; ++g)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int ar = 6 * g + c, ai = 6 * g + 3 + c;
                    const float Sr = __fadd_rn(acc[j][ar].x, acc[j][ar].y);
                    const float Si = __fadd_rn(acc[j][ai].x, acc[j][ai].y);
                    const float vr = __fmaf_rn(c0, Sr, -s0 * Si);
                    const float vi = __fmaf_rn(c0, Si, s0 * Sr);
                    float sum, e;
                    two_sum(hi[j][ar], vr, sum, e);
                    hi[j][ar] = sum;
                    float &l0 = lo[(ar * TP + j) * kThreads + threadIdx.x];
                    l0 = __fadd_rn(l0, e);
                    two_sum(hi[j][ai], vi, sum, e);
                    hi[j][ai] = sum;
                    float &l1 = lo[(ai * TP + j) * kThreads + threadIdx.x];
                    l1 = __fadd_rn(l1, e);
                }
        }
        if (band) ff_band_scan<TP, R4>(tile + kFFHead, (t0 + it) * kTile, rf, tbase, ns, nt, order, bl);
        __syncthreads();
        if (threadIdx.x == 0 && it + kStages < ntl) issue(it + kStages);
    }

    if (aborted) {
        if (threadIdx.x == 0)
            for (int s = 0; s < kStages; ++s) (void)mbar_wait_bounded(&full[s], 0);
        return;
    }

#pragma unroll
    for (int j = 0; j < TP; ++j) {
        const long ti = tbase + (long)j * kThreads;
        if (ti >= nt) continue;
#pragma unroll
        for (int a = 0; a < kAcc; ++a)
            part[((long)blockIdx.y * kAcc + a) * nt + ti] =
                a < NA ? (double)hi[j][a] + (double)lo[(a * TP + j) * kThreads + threadIdx.x] : 0.0;
    }
}

// ------------------------------------------------------------------ host side

int ff_smem_bytes(bool has_m) { return kStages * ff_tile4(has_m) * 16 + (has_m ? 12 : 6) * 2 * kThreads * 4; }

void *ff_key_kernel() { return reinterpret_cast<void *>(&po_ff_key_kernel); }

void *ff_pack_kernel(bool has_m)
{
    return has_m ? reinterpret_cast<void *>(&po_ff_pack_kernel<true>)
                 : reinterpret_cast<void *>(&po_ff_pack_kernel<false>);
}

void *ff_kernel(int t_sign, bool has_m)
{
    if (t_sign < 0)
        return has_m ? reinterpret_cast<void *>(&po_ff_kernel<-1, true>)
                     : reinterpret_cast<void *>(&po_ff_kernel<-1, false>);
    return has_m ? reinterpret_cast<void *>(&po_ff_kernel<1, true>)
                 : reinterpret_cast<void *>(&po_ff_kernel<1, false>);
}

// Radix sort of (key, index) pairs on `s`; with temp == nullptr only sets
// *temp_bytes (a host computation, no device work).
cudaError_t ff_sort(void *temp, size_t *temp_bytes, const unsigned long long *key_in, unsigned long long *key_out,
                    const int *idx_in, int *idx_out, long n, cudaStream_t s)
{
    return cub::DeviceRadixSort::SortPairs(temp, *temp_bytes, key_in, key_out, idx_in, idx_out, (int)n, 0,
                                           kFFKeyBits, s);
}

}  // namespace po
