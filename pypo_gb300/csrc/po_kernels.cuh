// po_kernels.cuh -- constants and kernel handles shared by the PO kernels and
// their host launcher.
#pragma once
#include <cstdint>

namespace po {

// Propagation modes (numbering of the reference's GpropagateBeam_0..5).
enum Mode { kJM = 0, kEH = 1, kJMEH = 2, kEHP = 3, kFF = 4, kScalar = 5 };

// Kernel families.
constexpr int kKindNF = 0;      // near field (JM, EH, JMEH, EHP)
constexpr int kKindFF = 1;      // far field
constexpr int kKindScalar = 2;  // scalar Green's function

// Mixed-precision N-body kernel geometry (the PO_* macros exist for tuning
// sweeps; the defaults are the shipped configuration).
#ifndef PO_THREADS
#define PO_THREADS 128
#endif
#ifndef PO_TILE
#define PO_TILE 128
#endif
#ifndef PO_MINB
#define PO_MINB 1
#endif
#ifndef PO_THREADS_A
#define PO_THREADS_A 128
#endif
constexpr int kThreads = PO_THREADS;   // threads per CTA
constexpr int kTile = PO_TILE;         // sources per shared-memory stage
constexpr int kMinBlocks = PO_MINB;    // resident CTAs per SM asked of ptxas
#ifndef PO_MINB_M
// The near-field forward with magnetic currents: 5 CTAs/SM hold it at 90
// registers (feed -> dish JM forward 0.673 -> 0.624 ms); asking the M = 0
// kernel for 5 as well slows dish_eh's forward (68.4 -> 70.1 ms).
#define PO_MINB_M 5
#endif
constexpr int kMinBlocksM = PO_MINB_M;
#ifndef PO_STAGES
#define PO_STAGES 3
#endif
constexpr int kStages = PO_STAGES;     // TMA pipeline depth
constexpr int kRec = 6;         // float4 per packed source record (96 B)
constexpr int kRecScalar = 2;   // float4 per packed scalar record (32 B)
constexpr int kAcc = 12;        // accumulators per target (E, H re/im x y z)
constexpr int kRec2 = 11;       // float4 per pair-packed record (two sources), near and far field
constexpr int kRec2Scalar = 4;  // float4 per pair-packed scalar record
constexpr int kBoxF = 8;        // floats per source-tile box (lit-tile proof)
#ifndef PO_MUFU_SINCOS
#define PO_MUFU_SINCOS 1         // 0: the polynomial sin/cos (accuracy comparisons)
#endif
// Targets per thread of the pair-packed kernel (near field, scalar): one; a
// second costs the near field 0.9 % (162 registers). The far-field kernel
// (po_farfield.cu) takes two directions per thread.
__host__ __device__ constexpr int pk_tpt(int) { return 1; }
constexpr uint32_t kWaitLimit = 1u << 24;   // bounded mbarrier polls

// Adjoint kernels: one source (or target) per thread; 12 current
// accumulators + 1 displacement accumulator.
constexpr int kThreadsA = PO_THREADS_A;
#ifndef PO_UNROLL_F
#define PO_UNROLL_F 1            // pair records per iteration of the forward pair loop
#endif
#ifndef PO_UNROLL_A
#define PO_UNROLL_A 1            // target pairs per iteration of the adjoint pair loop
#endif
#ifndef PO_PAIRS_A
#define PO_PAIRS_A 32            // target pairs per stage of the pair-packed adjoint
#endif
#ifndef PO_MINB_A2
// Resident CTAs per SM asked of ptxas for the pair-packed adjoint: 3 holds the
// fused near-field kernel at 150-165 registers with no spills (182 at 2), and
// dish_eh's adjoint measured 208.6 -> 206.1 ms with it.
#define PO_MINB_A2 3
#endif
constexpr int kMinBlocksA2 = PO_MINB_A2;
#ifndef PO_MINB_A2M
// The same with magnetic source currents: 2 (feed -> dish JM adjoint
// 1.394 -> 1.348 ms against 3).
#define PO_MINB_A2M 2
#endif
constexpr int kMinBlocksA2M = PO_MINB_A2M;
#ifndef PO_MINB_FF
#define PO_MINB_FF 5             // the far-field adjoint: 5 CTAs/SM hold it under 96 registers
#endif
constexpr int kMinBlocksFF = PO_MINB_FF;
constexpr int kUnrollF = PO_UNROLL_F;
constexpr int kUnrollA = PO_UNROLL_A;   // target pairs per iteration of the adjoint pair loop
constexpr int kAccAdj = 13;

// FP64 comparison kernel.
constexpr int kThreadsD = 128;
constexpr int kTileD = 64;
constexpr int kRecD = 18;       // x y z nx ny nz, J' 6, M' 6 (doubles)

constexpr int kBboxThreads = 256;
constexpr int kBboxBlocks = 152;

// Illumination test of the mixed-precision kernels: a pair with
// n . R_hat >= kTangentBand is lit, one below -kTangentBand is not (the FP32
// test's own error is below 4.2e-7). A pair inside the band is left out of
// the FP32 sums and listed; a fixup kernel then decides it with the
// reference's FP64 rounding, as the FP64 kernels decide every pair, and adds
// its FP64 term if it is lit. The lit-tile proofs keep a margin of 1e-5.
constexpr float kTangentBand = 1e-6f;

// The list of pairs inside the band: (source, target) entries, their count
// (zeroed before the main kernel) and the capacity; a count above the
// capacity is reported as kErrBandOverflow by the fixup.
struct BandList {
    int2 *pairs;
    unsigned *count;
    unsigned cap;
};
constexpr unsigned kBandCap = 1u << 22;        // entries, calls on the library's pool: every pair up
                                               // to this many, else at least this many
constexpr unsigned kBandCapMax = 1u << 24;     // ... and at most (one entry per 2^16 pairs between)
constexpr unsigned kBandCapStatic = 1u << 14;  // entries, the allocation-free entry

// Band-list entries of a call on the library's pool with ns x nt pairs: a
// call of up to 2^22 pairs can list all of them (targets in the sources'
// own plane put every pair in the band); larger calls one per 2^16 pairs.
inline unsigned band_cap_for(long ns, long nt)
{
    const double pairs = (double)ns * (double)nt;
    if (pairs <= (double)kBandCap) return pairs < 1.0 ? 1u : (unsigned)pairs;
    const double want = pairs / 65536.0;
    return want <= kBandCap ? kBandCap : (want >= kBandCapMax ? kBandCapMax : (unsigned)want);
}
constexpr unsigned kFixupBlocks = 152;         // grid of the fixup kernels (grid-stride over the list)

// Device error codes (written to the call's error word).
constexpr int kErrWaitTimeout = 101;
constexpr int kErrRngBound = 102;   // the device normal generator ran past its bound (never expected)
constexpr int kErrBandOverflow = 103;   // more near-tangent pairs than the band list holds

// Frame of the split representation: positions in turns (mm * kappa),
// relative to origin o, hi parts on multiples of q.
struct Frame {
    double o[3];
    double kappa;
    double q;
    double inv_q;
    double m;   // half-extent in wavelengths (turns), which sets q and the precision
    double lo[3], hi[3];   // the points' box (mm), from which the far field orders its sources
};

// Far-field forward (po_farfield.cu): sources in tiles of kTile along a
// Hilbert curve, each tile a 64-byte header and kTile / 2 pair records of
// ff_rec4 float4 (offset from the tile centre, J', normal, the offset's lo
// part in a wide tile, M').
constexpr int kFFHead = 4;
__host__ __device__ constexpr int ff_rec4(bool has_m) { return has_m ? 11 : 8; }
// Tiles up to this radius (turns) take the per-pair phase in plain FP32;
// wider ones (sparse sampling) split their offsets into hi + lo. At 64 turns
// the FP32 phase leaves about 2e-6 relative L2 error on a sum of random
// (incoherent) currents, the worst case (FP32 emulation on a 501 x 501 dish
// of 2000 wavelengths), and 1.2 % of that dish's tiles are wide; the full
// 1001 x 1001 configuration has 0.1 %.
constexpr float kFFNarrow = 64.0f;
__host__ __device__ constexpr int ff_tile4(bool has_m) { return kFFHead + (kTile / 2) * ff_rec4(has_m); }
int ff_smem_bytes(bool has_m);
void *ff_key_kernel();
void *ff_pack_kernel(bool has_m);
void *ff_kernel(int t_sign, bool has_m);

// Pair-packed main kernel: stages plus the compensation words.
inline int pk_smem_bytes(int kind)
{
    const bool sc = kind == kKindScalar;
    return kStages * (kTile / 2) * (sc ? kRec2Scalar : kRec2) * 16 + (sc ? 2 : kAcc) * pk_tpt(kind) * kThreads * 4;
}

void *pk_kernel(int kind, int t_sign, bool has_m);
void *pack_src2_kernel();
void *src_box_kernel();
void *fp64_kernel(int kind);
void *bbox_kernel();
void *frame_kernel();
void *pack_src_kernel();
void *pack_tgt_kernel();
void *pack_src_d_kernel();
void *epilogue_kernel();
void *f2d_kernel();   // float -> double, grid-stride over n
void *d2f_kernel();   // double -> float
void *fp32_probe_kernel();
void *band_fixup_kernel(int kind);
void *adj_band_fixup_kernel(int kind, int t_sign, bool want_d, bool want_t);
void *wait_selftest_kernel();
void *adj_src_fp64_kernel(int kind, int t_sign);
void *adj_tgt_fp64_kernel(int kind, int t_sign);
void *adj_cot_kernel();
void *adj_ehp_cot_kernel();
void *adj_src_epilogue_kernel();
// Pair-packed adjoint: near field fused (currents, source and target
// displacement), far field (currents, source displacement).
void *adj_pk_kernel(int kind, int t_sign, bool has_m, bool want_d, bool want_t);
void *adj_pack_tgt2_kernel();
int adj_pk_smem_bytes(int kind, bool has_m, bool want_t);
int adj_pk_pairs_per_tile();
int adj_pk_rec4(int kind, bool has_m, bool want_t);   // float4 per pair-packed cotangent record
void *adj_tgt_box_kernel();   // far-field cotangent tiles: direction boxes for the lit-tile proof
void *adj_tgt_epilogue_kernel();

}  // namespace po
