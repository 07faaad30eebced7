// po_noalloc.cu -- the propagation entry point that allocates nothing.
//
// Some callers of this library cannot allocate device memory: a serving or
// simulation framework that reserves the GPU's memory for its own pool (a
// cudaMalloc from inside it fails or fragments that pool), or a
// latency-critical loop that cannot accept the device-wide synchronisation
// cudaFree implies. po_run_dev_static serves them. It runs the same
// mixed-precision kernels as po_run_dev, but its scratch (frame, packed
// sources and targets, source-chunk partials) lives in a fixed file-scope
// device array of kStaticScratchBytes. Every GPU that loads this library
// holds that array until the process exits.
//
// Rules of use:
//   * the first call on a device looks up the array's device address and the
//     kernels' occupancy (the set-up below); make that first call before any
//     stream capture;
//   * a kernel that gives up a bounded wait sets the caller's status word,
//     or (status == NULL) the array's own word, which po_device_error reads
//     and clears;
//   * every call shares the one array per device and leaves its contents for
//     the next; calls that overlap on the GPU (different streams, or threads)
//     race on it and must be serialised by the caller;
//   * sizes whose scratch exceeds kStaticScratchBytes are rejected with a
//     status and a message, before any device work.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "po_internal.h"
#include "po_kernels.cuh"

namespace {

using po::fail;

// 64 MiB: the dish_eh workload (251,001 sources, 90,601 targets) fits with
// four source chunks.
constexpr size_t kStaticScratchBytes = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr size_t kAlign = 256;
inline size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Offsets inside the array.
constexpr size_t kOffStatus = 0;                       // int: timeouts of calls with status == NULL
constexpr size_t kOffFrame = 256;                      // po::Frame
constexpr size_t kOffBbox = 512;                       // kBboxBlocks * 6 doubles
static_assert(sizeof(po::Frame) <= kOffBbox - kOffFrame, "the frame must fit its slot");
constexpr size_t kFixed = kOffBbox + ((po::kBboxBlocks * 6 * sizeof(double) + kAlign - 1) / kAlign) * kAlign;

struct StaticSetup {
    bool ready = false;
    unsigned char *base = nullptr;   // device address of g_static_scratch
    int sms = 0;
    int occ[3][2][2] = {};
};

std::mutex g_mu;
StaticSetup g_setup[64];

// Once per device, with that device current: the array's device address and
// the resident-CTA counts of the main kernels.
int setup(StaticSetup *&out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(2, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(2, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    StaticSetup &s = g_setup[dev];
    if (!s.ready) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess)
            return fail(2, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
        e = cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(2, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
        for (int kind = 0; kind < 3; ++kind)
            for (int ts = 0; ts < 2; ++ts)
                for (int hm = 0; hm < 2; ++hm) {
                    if (kind == po::kKindScalar && hm) continue;
                    void *fn = po::pk_kernel(kind, ts ? 1 : -1, hm != 0);
                    const int smem = po::pk_smem_bytes(kind);
                    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
                    if (e != cudaSuccess) return fail(2, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
                    int nb = 0;
                    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, po::kThreads, smem);
                    if (e != cudaSuccess) return fail(2, std::string("occupancy query: ") + cudaGetErrorString(e));
                    s.occ[kind][ts][hm] = std::max(nb, 1);
                }
        s.base = static_cast<unsigned char *>(ptr);
        s.ready = true;
    }
    out = &s;
    return 0;
}

// Scratch bytes for a given chunk count (rec2: float4 per pair-packed record).
size_t need_bytes(long ns, long nt, int rec2, int nacc, long chunks)
{
    return kFixed + up((size_t)((std::max(ns, 1L) + 1) / 2) * rec2 * 16) + up((size_t)nt * 32) +
           up((size_t)chunks * nacc * nt * sizeof(double));
}

int launch(void *fn, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t s)
{
    if (grid.x == 0 || grid.y == 0) return 0;
    cudaError_t e = cudaLaunchKernel(fn, grid, block, args, smem, s);
    if (e != cudaSuccess) return fail(2, std::string("kernel launch: ") + cudaGetErrorString(e));
    po::note_launches(1);
    return 0;
}

}  // namespace

// The internal status word of the current device, or null before the entry's
// first call there. Read and cleared by po::read_device_error.
int *po::static_status_word()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    return g_setup[dev].ready ? reinterpret_cast<int *>(g_setup[dev].base + kOffStatus) : nullptr;
}

extern "C" int po_run_dev_static(int mode, long ns, const double *src7, int gmode, int ncx, int ncy,
                                 const double *cur, long nt, const double *tgt7, double k, double epsilon,
                                 double t_direction, int flags, double *out, int *status, void *stream)
{
    po::clear_error();
    po::RunArgs a;
    a.mode = mode;
    a.ns = ns;
    a.src7 = src7;
    a.gmode = gmode;
    a.ncx = ncx;
    a.ncy = ncy;
    a.cur = cur;
    a.nt = nt;
    a.tgt7 = tgt7;
    a.k = k;
    a.epsilon = epsilon;
    a.t_dir = t_direction;
    a.precision = 0;
    a.out = out;
    if (int rc = po::validate(a)) return rc;
    const int kind = mode == po::kFF ? po::kKindFF : (mode == po::kScalar ? po::kKindScalar : po::kKindNF);
    const int scalar = kind == po::kKindScalar;
    const int nacc = scalar ? 2 : po::kAcc;
    const int rec2 = scalar ? po::kRec2Scalar : po::kRec2;
    const size_t minimum = need_bytes(ns, nt, rec2, nacc, 1);
    if (minimum > kStaticScratchBytes)
        return fail(5, "po_run_dev_static: this problem needs " + std::to_string(minimum) +
                           " bytes of scratch, more than the " + std::to_string(kStaticScratchBytes) +
                           "-byte static array (about 88*ns + 128*nt bytes are needed)");
    StaticSetup *st = nullptr;
    if (int rc = setup(st)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The caller's status word starts every call at zero. The internal word
    // (status == NULL) keeps a timeout until po_device_error reads and clears
    // it, so a later call cannot hide it.
    int *err = status ? status : reinterpret_cast<int *>(st->base + kOffStatus);
    if (status) {
        cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), s);
        if (e != cudaSuccess) return fail(2, std::string("clearing the status word: ") + cudaGetErrorString(e));
    }
    if (nt == 0) return 0;

    const int ts = t_direction > 0 ? 1 : -1;
    const bool has_m = kind != po::kKindScalar && !(flags & 1);
    const long ntb = (nt + (long)po::kThreads * po::pk_tpt(kind) - 1) / ((long)po::kThreads * po::pk_tpt(kind));
    const size_t part_room = kStaticScratchBytes - (need_bytes(ns, nt, rec2, nacc, 0));
    const long max_chunks = std::max(1L, (long)(part_room / ((size_t)nacc * nt * sizeof(double))));
    // the allocating path's chunk choice, capped so that the partials fit the array
    const long nsplit = po::choose_split(ntb, ns, (long)st->sms * st->occ[kind][ts > 0][has_m ? 1 : 0], max_chunks,
                                         po::kTile);
    const long tiles = std::max(1L, (ns + po::kTile - 1) / po::kTile);
    long chunk = ((tiles + nsplit - 1) / nsplit) * po::kTile;

    unsigned char *b = st->base;
    po::Frame *frame = reinterpret_cast<po::Frame *>(b + kOffFrame);
    double *bbox = reinterpret_cast<double *>(b + kOffBbox);
    size_t off = kFixed;
    float4 *srcpk = reinterpret_cast<float4 *>(b + off);
    off += up((size_t)((std::max(ns, 1L) + 1) / 2) * rec2 * 16);
    float4 *tgtpk = reinterpret_cast<float4 *>(b + off);
    off += up((size_t)nt * 32);
    double *part = reinterpret_cast<double *>(b + off);

    const double pif = (double)3.14159265359f;
    const double pref = k * k / (4.0 * pif);
    const double kappa = k / (2.0 * 3.14159265358979323846);
    const double c_l = (double)2.99792458e8f, mu0 = (double)1.2566370614e-6f;
    const double eps = epsilon * (1.0 / (mu0 * c_l * c_l));
    double zeta_inv = 1.0 / std::sqrt(mu0 / eps);
    double fac_re = pref, fac_im = 0.0;
    if (kind == po::kKindFF) { fac_re = 0.0; fac_im = -pref; }
    if (scalar) fac_re = -pref * kappa;
    const bool far = kind == po::kKindFF;
    long nb = far ? 0 : nt;
    const unsigned nblk_t = (unsigned)((nt + 255) / 256);
    int rc = 0;
    void *bargs[] = {&src7, &ns, &tgt7, &nb, &bbox};
    rc = launch(po::bbox_kernel(), dim3(po::kBboxBlocks), dim3(po::kBboxThreads), bargs, 0, s);
    int nbb = po::kBboxBlocks;
    double kap = kappa;
    int centred = far ? 0 : 1;
    void *frargs[] = {&bbox, &nbb, &kap, &centred, &frame};
    if (!rc) rc = launch(po::frame_kernel(), dim3(1), dim3(32), frargs, 0, s);
    float *srcf = reinterpret_cast<float *>(srcpk);
    void *psargs[] = {&ns, &src7, &cur, &gmode, &ncx, &ncy, &frame, &fac_re, &fac_im, (void *)&scalar, &srcf};
    const unsigned nblk_p = (unsigned)((2 * ((ns + 1) / 2) + 255) / 256);
    if (!rc && ns > 0) rc = launch(po::pack_src2_kernel(), dim3(nblk_p), dim3(256), psargs, 0, s);
    float2 *rec2p = reinterpret_cast<float2 *>(srcpk);
    void *sbargs[] = {&rec2p, &ns};
    int boxes = !scalar && !has_m && ns > 0;   // the lit-tile proof serves the M = 0 kernels
    if (!rc && boxes) rc = launch(po::src_box_kernel(), dim3((unsigned)tiles), dim3(32), sbargs, 0, s);
    int farflag = far ? 1 : 0;
    void *ptargs[] = {&nt, &tgt7, &frame, &farflag, &tgtpk};
    if (!rc) rc = launch(po::pack_tgt_kernel(), dim3(nblk_t), dim3(256), ptargs, 0, s);
    const float4 *srcc = srcpk, *tgtc = tgtpk;
    void *margs[] = {&srcc, &ns, &chunk, &tgtc, &nt, &part, &err, &boxes};
    if (!rc)
        rc = launch(po::pk_kernel(kind, ts, has_m), dim3((unsigned)ntb, (unsigned)nsplit), dim3(po::kThreads),
                    margs, po::pk_smem_bytes(kind), s);
    int nspl = (int)nsplit;
    double t = t_direction;
    void *eargs[] = {&mode, &nspl, &nt, &part, &tgt7, &t, &zeta_inv, &out};
    if (!rc) rc = launch(po::epilogue_kernel(), dim3(nblk_t), dim3(256), eargs, 0, s);
    return rc;
}
