// po_engine.cu -- host orchestration of one propagation on device buffers.
//
// Mixed precision (precision 0):
//   bbox -> frame -> pack sources / targets -> main N-body kernel over a
//   (target block, source chunk) grid -> FP64 epilogue summing the chunks.
// Plain FP64 (precision 1):
//   pack sources (double) -> one-thread-per-target FP64 direct sum -> epilogue.
// Scratch is stream-ordered on the caller's stream, from the library's own
// memory pool (scratch_alloc / scratch_free); nothing here synchronises the
// device.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "po_internal.h"
#include "po_kernels.cuh"

namespace po {

namespace {

thread_local std::string t_err;
thread_local int t_launches = 0;

struct DeviceInfo {
    bool ready = false;
    int sms = 0;
    cudaMemPool_t pool = nullptr;   // the library's own scratch pool
    int occ2[3][2][2] = {};  // pair-packed kernels, [kind][t>0][has_m]
    int occ_ff[2][2] = {};   // far-field tile kernels, [t>0][has_m]
    std::map<void *, int> occ_adj;   // adjoint kernels: resident CTAs, attribute set
};

std::mutex g_mu;
DeviceInfo g_dev[64];
constexpr uint64_t kPoolKeep = 16ull << 30;   // freed scratch a device's pool keeps (bytes)

// Timing ring: CUDA event pairs recorded around each main-kernel launch.
struct Timing {
    bool on = false;
    std::vector<cudaEvent_t> ev;   // 2 per slot
    int used = 0;
};
Timing g_timing;

const char *err_str(cudaError_t e) { return cudaGetErrorString(e); }

}  // namespace

int fail(int code, const std::string &msg)
{
    t_err = msg;
    return code;
}

void clear_error()
{
    t_err.clear();
    t_launches = 0;
}

void note_launches(int n) { t_launches += n; }

const char *last_error() { return t_err.c_str(); }
int last_launches() { return t_launches; }

int n_out(int mode)
{
    static const int n[6] = {12, 12, 24, 15, 12, 2};
    return (mode >= 0 && mode < 6) ? n[mode] : -1;
}

// Record a CUDA failure in rc (once) and carry on to the caller's cleanup.
#define PO_CK_RC(expr)                                                                      \
    do {                                                                                    \
        if (!rc) {                                                                          \
            cudaError_t e_ = (expr);                                                        \
            if (e_ != cudaSuccess) rc = fail(2, std::string(#expr) + ": " + err_str(e_));   \
        }                                                                                   \
    } while (0)

#define PO_CK(expr)                                                                         \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess) return fail(2, std::string(#expr) + ": " + err_str(e_));     \
    } while (0)

static int device_info(DeviceInfo *&out)
{
    int dev = 0;
    PO_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(2, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceInfo &di = g_dev[dev];
    if (!di.ready) {
        PO_CK(cudaDeviceGetAttribute(&di.sms, cudaDevAttrMultiProcessorCount, dev));
        for (int kind = 0; kind < 3; ++kind)
            for (int ts = 0; ts < 2; ++ts)
                for (int hm = 0; hm < 2; ++hm) {
                    if (kind == kKindFF || (kind == kKindScalar && hm)) continue;   // FF: occ_ff below
                    void *fn = pk_kernel(kind, ts ? 1 : -1, hm != 0);
                    const int smem = pk_smem_bytes(kind);
                    PO_CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
                    int nb = 0;
                    PO_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, smem));
                    di.occ2[kind][ts][hm] = std::max(nb, 1);
                }
        for (int ts = 0; ts < 2; ++ts)
            for (int hm = 0; hm < 2; ++hm) {
                void *fn = ff_kernel(ts ? 1 : -1, hm != 0);
                const int smem = ff_smem_bytes(hm != 0);
                PO_CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
                int nb = 0;
                PO_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, smem));
                di.occ_ff[ts][hm] = std::max(nb, 1);
            }
        di.ready = true;
    }
    out = &di;
    return 0;
}

long choose_split(long nb, long ns, long slots, long max_chunks, long tile)
{
    const long tiles = std::max(1L, (ns + tile - 1) / tile);
    long best = 1;
    double best_cost = 1e300;
    for (long s = 1; s <= std::min(tiles, std::min(std::max(1L, max_chunks), 1024L)); ++s) {
        const long chunk = (tiles + s - 1) / s;
        const long real = (tiles + chunk - 1) / chunk;
        if (real != s) continue;
        const long waves = (nb * real + slots - 1) / slots;
        const double cost = (double)waves * chunk + 0.05 * real;
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = real;
        }
    }
    return best;
}

// Partial buffers of the chunked kernels are capped near 1 GiB.
static long partial_cap(long n, int nacc) { return std::max(1L, (1L << 30) / std::max(1L, n * nacc * 8)); }

int scratch_alloc(void **p, size_t bytes, cudaStream_t s)
{
    DeviceInfo *di = nullptr;
    if (int rc = device_info(di)) return rc;
    cudaMemPool_t pool = nullptr;
    {
        // Scratch comes from a stream-ordered pool of the library's own, made
        // on first use, so the device's default pool (shared with every
        // other user in the process) keeps its settings. A pool hands freed
        // memory back to the driver at every synchronisation unless told
        // otherwise, so each host-buffer call (which synchronises) would map
        // its scratch afresh; this one keeps up to kPoolKeep bytes of freed
        // scratch.
        std::lock_guard<std::mutex> lk(g_mu);
        if (!di->pool) {
            int dev = 0;
            PO_CK(cudaGetDevice(&dev));
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t np = nullptr;
            PO_CK(cudaMemPoolCreate(&np, &props));
            uint64_t keep = kPoolKeep;
            PO_CK(cudaMemPoolSetAttribute(np, cudaMemPoolAttrReleaseThreshold, &keep));
            di->pool = np;
        }
        pool = di->pool;
    }
    cudaError_t e = cudaMallocFromPoolAsync(p, std::max<size_t>(bytes, 16), pool, s);
    if (e != cudaSuccess) return fail(3, std::string("device scratch allocation failed: ") + err_str(e));
    return 0;
}

void scratch_free(void *p, cudaStream_t s)
{
    if (p) cudaFreeAsync(p, s);
}

int scratch_used(unsigned long long *bytes)
{
    *bytes = 0;
    int dev = 0;
    PO_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(2, "device ordinal out of range");
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        pool = g_dev[dev].pool;
    }
    if (!pool) return 0;
    uint64_t used = 0;
    PO_CK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
    *bytes = used;
    return 0;
}

template <typename T>
static int salloc(T **p, size_t count, cudaStream_t s, std::vector<void *> &owned)
{
    void *q = nullptr;
    if (int rc = scratch_alloc(&q, count * sizeof(T), s)) return rc;
    owned.push_back(q);
    *p = static_cast<T *>(q);
    return 0;
}

static void sfree(std::vector<void *> &owned, cudaStream_t s)
{
    for (void *q : owned) scratch_free(q, s);
    owned.clear();
}

// Stream-ordered scratch from the library's pool, freed (in stream order)
// when the call's work is queued.
class PoolScratch : public Scratch {
public:
    explicit PoolScratch(cudaStream_t s) : s_(s) {}
    ~PoolScratch() override { sfree(owned_, s_); }
    int take(void **p, size_t bytes) override
    {
        const int rc = scratch_alloc(p, bytes, s_);
        if (!rc) owned_.push_back(*p);
        return rc;
    }
    size_t room() const override { return ~(size_t)0; }

private:
    cudaStream_t s_;
    std::vector<void *> owned_;
};

static int launch(void *fn, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t s)
{
    if (grid.x == 0 || grid.y == 0) return 0;
    PO_CK(cudaLaunchKernel(fn, grid, block, args, smem, s));
    note_launches(1);
    return 0;
}

static void timing_mark(cudaStream_t s, bool begin)
{
    if (!g_timing.on) return;
    std::lock_guard<std::mutex> lk(g_mu);
    const int slots = (int)g_timing.ev.size() / 2;
    if (slots == 0) return;
    if (begin) {
        if (g_timing.used >= slots) return;
        cudaEventRecord(g_timing.ev[2 * g_timing.used], s);
    } else {
        if (g_timing.used >= slots) return;
        cudaEventRecord(g_timing.ev[2 * g_timing.used + 1], s);
        ++g_timing.used;
    }
}

int timing_enable(int slots)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (cudaEvent_t e : g_timing.ev) cudaEventDestroy(e);
    g_timing.ev.clear();
    g_timing.used = 0;
    g_timing.on = slots > 0;
    for (int i = 0; i < 2 * std::max(slots, 0); ++i) {
        cudaEvent_t e;
        PO_CK(cudaEventCreate(&e));
        g_timing.ev.push_back(e);
    }
    return 0;
}

int timing_collect(float *ms, int max)
{
    std::lock_guard<std::mutex> lk(g_mu);
    int n = std::min(g_timing.used, max);
    for (int i = 0; i < n; ++i) {
        PO_CK(cudaEventSynchronize(g_timing.ev[2 * i + 1]));
        PO_CK(cudaEventElapsedTime(&ms[i], g_timing.ev[2 * i], g_timing.ev[2 * i + 1]));
    }
    g_timing.used = 0;
    return n;
}

// Persistent per-device error word, written by kernels that give up a wait.
static int *g_words[64] = {};

static int *error_word_impl(bool create)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_words[dev] && create) {
        if (cudaMalloc(&g_words[dev], sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemset(g_words[dev], 0, sizeof(int)) != cudaSuccess) return nullptr;
    }
    return g_words[dev];
}

int *error_word() { return error_word_impl(true); }

int read_device_error(cudaStream_t s, int *code)
{
    // Both words: the allocating paths' (if it exists yet) and the
    // allocation-free entry's (if it has set up on this device). Nothing is
    // allocated here, so callers of the allocation-free entry can use it.
    int *w[2] = {error_word_impl(false), static_status_word()};
    int got[2] = {0, 0};
    for (int i = 0; i < 2; ++i) {
        if (!w[i]) continue;
        PO_CK(cudaMemcpyAsync(&got[i], w[i], sizeof(int), cudaMemcpyDeviceToHost, s));
        PO_CK(cudaMemsetAsync(w[i], 0, sizeof(int), s));
    }
    PO_CK(cudaStreamSynchronize(s));
    *code = got[0] ? got[0] : got[1];
    return 0;
}

int validate(const RunArgs &a)
{
    if (a.mode < 0 || a.mode > 5) return fail(1, "mode must be 0..5 (JM EH JMEH EHP FF scalar)");
    if (a.ns < 0 || a.nt < 0) return fail(1, "negative size");
    if (a.ns > INT_MAX || a.nt > INT_MAX)
        return fail(1, "at most 2^31 - 1 sources and targets per call (indices are 32-bit on the device)");
    if (a.ns > 0 && a.gmode >= 0 && (a.ncx < 1 || a.ncy < 1)) return fail(1, "bad source grid shape");
    if (a.ns > 0 && a.gmode >= 0 && (long)a.ncx * a.ncy != a.ns)
        return fail(1, "ncx * ncy must equal the number of source points");
    if (!(a.t_dir == 1.0 || a.t_dir == -1.0)) return fail(1, "t_direction must be -1 (fwd) or +1 (bwd)");
    if (!(a.k > 0.0) || !std::isfinite(a.k)) return fail(1, "wavenumber k must be positive and finite");
    if (a.precision != 0 && a.precision != 1) return fail(1, "precision must be 0 (mixed) or 1 (fp64)");
    if (a.nt > 0 && ((a.ns > 0 && (!a.src7 || !a.cur)) || !a.tgt7 || !a.out)) return fail(1, "null buffer");
    return 0;
}

int run_device(const RunArgs &a)
{
    if (int rc = validate(a)) return rc;
    if (a.nt == 0) return 0;
    cudaStream_t s = a.stream;
    if (a.precision == 0) {
        int *err = error_word();
        if (!err) return fail(2, "could not allocate the device error word");
        PoolScratch pool(s);
        return run_mixed(a, pool, err);
    }

    // ---- plain FP64: one thread per target, the comparison path
    const int kind = a.mode == kFF ? kKindFF : (a.mode == kScalar ? kKindScalar : kKindNF);
    const int nacc = kind == kKindScalar ? 2 : kAcc;
    const double pif = (double)3.14159265359f;   // the reference's float-literal pi
    const double pref = a.k * a.k / (4.0 * pif);
    const double c_l = (double)2.99792458e8f, mu0 = (double)1.2566370614e-6f;
    const double eps = a.epsilon * (1.0 / (mu0 * c_l * c_l));
    double zeta_inv = 1.0 / std::sqrt(mu0 / eps);
    // complex factor folded into each source's weighted current
    double fac_re = pref, fac_im = 0.0;
    if (kind == kKindFF) { fac_re = 0.0; fac_im = -pref; }
    if (kind == kKindScalar) fac_re = -pref;
    std::vector<void *> owned;
    int rc = 0;
    const unsigned nblk_s = (unsigned)((a.ns + 255) / 256), nblk_t = (unsigned)((a.nt + 255) / 256);
    long nt = a.nt, ns = a.ns;
    int mode = a.mode, gmode = a.gmode, ncx = a.ncx, ncy = a.ncy;
    double t = a.t_dir, k = a.k;
    const int scalar = kind == kKindScalar;
    const double *src7 = a.src7, *cur = a.cur, *tgt7 = a.tgt7;
    double *out = a.out;
    double *srcd = nullptr, *part = nullptr;
    if ((rc = salloc(&srcd, (size_t)std::max(ns, 1L) * kRecD, s, owned)) ||
        (rc = salloc(&part, (size_t)nacc * nt, s, owned))) {
        sfree(owned, s);
        return rc;
    }
    void *pargs[] = {&ns, &src7, &cur, &gmode, &ncx, &ncy, &fac_re, &fac_im, (void *)&scalar, &srcd};
    if (ns > 0) rc = launch(pack_src_d_kernel(), dim3(nblk_s), dim3(256), pargs, 0, s);
    void *fargs[] = {&srcd, &ns, &tgt7, &nt, &k, &t, &part};
    timing_mark(s, true);
    if (!rc) rc = launch(fp64_kernel(kind), dim3((unsigned)((nt + kThreadsD - 1) / kThreadsD)), dim3(kThreadsD),
                         fargs, 0, s);
    timing_mark(s, false);
    int one = 1;
    void *eargs[] = {&mode, &one, &nt, &part, &tgt7, &t, &zeta_inv, &out};
    if (!rc) rc = launch(epilogue_kernel(), dim3(nblk_t), dim3(256), eargs, 0, s);
    sfree(owned, s);
    return rc;
}

int mixed_prepare(const RunArgs &a, Scratch &sc, MixedPlan &p)
{
    DeviceInfo *di = nullptr;
    if (int rc = device_info(di)) return rc;
    p.kind = a.mode == kFF ? kKindFF : (a.mode == kScalar ? kKindScalar : kKindNF);
    p.nacc = p.kind == kKindScalar ? 2 : kAcc;
    const double pif = (double)3.14159265359f;   // the reference's float-literal pi
    const double pref = a.k * a.k / (4.0 * pif);
    p.kappa = a.k / (2.0 * 3.14159265358979323846);
    const double c_l = (double)2.99792458e8f, mu0 = (double)1.2566370614e-6f;
    const double eps = a.epsilon * (1.0 / (mu0 * c_l * c_l));
    p.zeta_inv = 1.0 / std::sqrt(mu0 / eps);
    p.ts = a.t_dir > 0 ? 1 : -1;
    // complex factor folded into each source's weighted current
    p.fac_re = pref;
    p.fac_im = 0.0;
    if (p.kind == kKindFF) { p.fac_re = 0.0; p.fac_im = -pref; }
    if (p.kind == kKindScalar) p.fac_re = -pref * p.kappa;
    const bool scalar = p.kind == kKindScalar;
    p.far = p.kind == kKindFF;
    p.has_m = !scalar && !a.m_zero;
    const long ns = a.ns, nt = a.nt;
    p.tiles = std::max(1L, (ns + kTile - 1) / kTile);
    int rc = 0;
    if ((rc = sc.get(&p.bbox, (size_t)kBboxBlocks * 6)) || (rc = sc.get(&p.frame, 1)) ||
        (rc = sc.get(&p.tgtpk, (size_t)nt * 2)))
        return rc;
    if (!scalar) {
        p.band.cap = sc.band_cap(ns, nt);
        if ((rc = sc.get(&p.band.pairs, p.band.cap)) || (rc = sc.get(&p.band.count, 1))) return rc;
    }
    if (p.far) {
        // the far field's tiles along the sources' Hilbert order
        const long n1 = std::max(ns, 1L);
        cudaError_t e = ff_sort(nullptr, &p.sort_bytes, nullptr, nullptr, nullptr, nullptr, n1, a.stream);
        if (e != cudaSuccess) return fail(2, std::string("sort size query: ") + err_str(e));
        if ((rc = sc.get(&p.srcpk, (size_t)p.tiles * ff_tile4(p.has_m))) || (rc = sc.get(&p.keys, 2 * (size_t)n1)) ||
            (rc = sc.get(&p.order, 2 * (size_t)n1)) || (rc = sc.take(&p.sort_tmp, p.sort_bytes)))
            return rc;
    } else {
        const size_t src_f4 = (size_t)((std::max(ns, 1L) + 1) / 2) * (scalar ? kRec2Scalar : kRec2);
        if ((rc = sc.get(&p.srcpk, src_f4))) return rc;
    }
    // source chunks: balance waves over the SMs; the partials must fit the scratch left
    const int tpt = p.far ? 2 : pk_tpt(p.kind);   // targets per thread
    p.ntb = (nt + (long)kThreads * tpt - 1) / ((long)kThreads * tpt);
    const int occ = p.far ? di->occ_ff[p.ts > 0][p.has_m ? 1 : 0] : di->occ2[p.kind][p.ts > 0][p.has_m ? 1 : 0];
    const size_t room = std::min(sc.room(), (size_t)1 << 30);
    const long max_chunks = (long)(room / ((size_t)p.nacc * nt * sizeof(double)));
    if (max_chunks < 1) return sc.get(&p.part, (size_t)p.nacc * nt);   // fails with the source's message
    p.nsplit = choose_split(p.ntb, ns, (long)di->sms * occ, max_chunks, kTile);
    const long chunk_tiles = (p.tiles + p.nsplit - 1) / p.nsplit;
    p.chunk = chunk_tiles * (p.far ? 1 : kTile);   // tiles (far field) or sources per chunk
    return sc.get(&p.part, (size_t)p.nsplit * p.nacc * nt);
}

int mixed_launch(const RunArgs &a, MixedPlan &p, int *err)
{
    cudaStream_t s = a.stream;
    long nt = a.nt, ns = a.ns;
    int mode = a.mode, gmode = a.gmode, ncx = a.ncx, ncy = a.ncy;
    double t = a.t_dir;
    const int scalar = p.kind == kKindScalar;
    const double *src7 = a.src7, *cur = a.cur, *tgt7 = a.tgt7;
    double *out = a.out;
    const unsigned nblk_s = (unsigned)((ns + 255) / 256), nblk_t = (unsigned)((nt + 255) / 256);
    int rc = 0;
    // ---- frame: far field keeps the coordinate origin (its phase reference)
    long nb = p.far ? 0 : nt;   // the box covers the sources, plus the targets in the near field
    void *bargs[] = {&src7, &ns, &tgt7, &nb, &p.bbox};
    rc = launch(bbox_kernel(), dim3(kBboxBlocks), dim3(kBboxThreads), bargs, 0, s);
    int nbb = kBboxBlocks;
    int centred = p.far ? 0 : 1;
    void *frargs[] = {&p.bbox, &nbb, &p.kappa, &centred, &p.frame};
    if (!rc) rc = launch(frame_kernel(), dim3(1), dim3(32), frargs, 0, s);
    int boxes = !scalar && !p.has_m && ns > 0;   // the lit-tile proof serves the M = 0 kernels
    if (p.far) {
        // sources in Hilbert order, packed tile by tile with their centres
        const long n1 = std::max(ns, 1L);
        unsigned long long *k_in = p.keys, *k_out = p.keys + n1;
        int *i_in = p.order, *i_out = p.order + n1;
        void *kargs[] = {&ns, &src7, &p.frame, &k_in, &i_in};
        if (!rc && ns > 0) rc = launch(ff_key_kernel(), dim3(nblk_s), dim3(256), kargs, 0, s);
        if (!rc && ns > 0) {
            cudaError_t e = ff_sort(p.sort_tmp, &p.sort_bytes, k_in, k_out, i_in, i_out, ns, s);
            if (e != cudaSuccess) rc = fail(2, std::string("source sort: ") + err_str(e));
            else note_launches(1);
        }
        const int *ord = i_out;
        void *pargs[] = {&ns, &ord, &src7, &cur, &gmode, &ncx, &ncy, &p.frame, &p.fac_re, &p.fac_im, &p.srcpk};
        if (!rc && ns > 0) rc = launch(ff_pack_kernel(p.has_m), dim3((unsigned)p.tiles), dim3(32), pargs, 0, s);
    } else {
        float *srcf = reinterpret_cast<float *>(p.srcpk);
        void *psargs[] = {&ns, &src7, &cur, &gmode, &ncx, &ncy, &p.frame, &p.fac_re, &p.fac_im, (void *)&scalar, &srcf};
        const unsigned nblk_p = (unsigned)((2 * ((ns + 1) / 2) + 255) / 256);
        if (!rc && ns > 0) rc = launch(pack_src2_kernel(), dim3(nblk_p), dim3(256), psargs, 0, s);
        float2 *rec2 = reinterpret_cast<float2 *>(p.srcpk);
        void *sbargs[] = {&rec2, &ns};
        if (!rc && boxes) rc = launch(src_box_kernel(), dim3((unsigned)p.tiles), dim3(32), sbargs, 0, s);
    }
    int farflag = p.far ? 1 : 0;
    void *ptargs[] = {&nt, &tgt7, &p.frame, &farflag, &p.tgtpk};
    if (!rc) rc = launch(pack_tgt_kernel(), dim3(nblk_t), dim3(256), ptargs, 0, s);
    const float4 *srcc = p.srcpk, *tgtc = p.tgtpk;
    long ntiles = ns > 0 ? p.tiles : 0;
    const int *sorted = p.order ? p.order + std::max(ns, 1L) : nullptr;   // far field: curve position -> source
    if (!rc && p.band.count) PO_CK_RC(cudaMemsetAsync(p.band.count, 0, sizeof(unsigned), s));
    void *margs[] = {&srcc, p.far ? (void *)&ntiles : (void *)&ns, &p.chunk, &tgtc, &nt, &p.part, &err, &boxes,
                     &p.band, &ns, &sorted};
    timing_mark(s, true);
    if (!rc) {
        if (p.far)
            rc = launch(ff_kernel(p.ts, p.has_m), dim3((unsigned)p.ntb, (unsigned)p.nsplit), dim3(kThreads), margs,
                        ff_smem_bytes(p.has_m), s);
        else
            rc = launch(pk_kernel(p.kind, p.ts, p.has_m), dim3((unsigned)p.ntb, (unsigned)p.nsplit), dim3(kThreads),
                        margs, pk_smem_bytes(p.kind), s);
    }
    timing_mark(s, false);
    if (!rc && p.band.count && ns > 0) {
        // the near-tangent pairs, decided and summed in FP64 into chunk 0
        double k = a.k;
        void *xargs[] = {&p.band, &ns, &src7, &cur, &gmode, &ncx, &ncy, &p.fac_re, &p.fac_im, &nt, &tgt7, &k, &t,
                         &p.part, &err};
        rc = launch(band_fixup_kernel(p.kind), dim3(kFixupBlocks), dim3(256), xargs, 0, s);
    }
    int nspl = (int)p.nsplit;
    void *eargs[] = {&mode, &nspl, &nt, &p.part, &tgt7, &t, &p.zeta_inv, &out};
    if (!rc) rc = launch(epilogue_kernel(), dim3(nblk_t), dim3(256), eargs, 0, s);
    if (!rc && a.extent_host) PO_CK_RC(cudaMemcpyAsync(a.extent_host, &p.frame->m, sizeof(double),
                                                       cudaMemcpyDeviceToHost, s));
    if (!rc && a.band_host && p.band.count)
        PO_CK_RC(cudaMemcpyAsync(a.band_host, p.band.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    return rc;
}

int run_mixed(const RunArgs &a, Scratch &sc, int *err)
{
    if (a.nt == 0) return 0;
    MixedPlan p;
    if (int rc = mixed_prepare(a, sc, p)) return rc;
    return mixed_launch(a, p, err);
}


// ---------------------------------------------------------------- adjoint

int run_adjoint(const AdjArgs &a)
{
    if (int rc = validate(a)) return rc;
    if (a.mode == kFF && a.grad_dt) return fail(1, "far-field targets are directions: no target displacement");
    if (a.nt > 0 && !a.cot) return fail(1, "null cotangent buffer");
    if (a.ns == 0) {
        // no sources: the target gradient is zero (the source gradients are empty)
        if (a.grad_dt && a.nt > 0) PO_CK(cudaMemsetAsync(a.grad_dt, 0, sizeof(double) * a.nt, a.stream));
        return 0;
    }
    if (a.nt == 0) {
        // no targets: every gradient is zero
        if (a.grad_cur)
            PO_CK(cudaMemsetAsync(a.grad_cur, 0, sizeof(double) * (a.mode == kScalar ? 2 : 12) * a.ns, a.stream));
        if (a.grad_ds) PO_CK(cudaMemsetAsync(a.grad_ds, 0, sizeof(double) * a.ns, a.stream));
        return 0;
    }
    DeviceInfo *di = nullptr;
    if (int rc = device_info(di)) return rc;
    int *err = error_word();
    if (!err) return fail(2, "could not allocate the device error word");

    const int kind = a.mode == kFF ? kKindFF : (a.mode == kScalar ? kKindScalar : kKindNF);
    const double pif = (double)3.14159265359f;
    const double pref = a.k * a.k / (4.0 * pif);
    const double kappa = a.k / (2.0 * 3.14159265358979323846);
    double fac_re = pref, fac_im = 0.0;
    if (kind == kKindFF) { fac_re = 0.0; fac_im = -pref; }
    if (kind == kKindScalar) fac_re = -pref * (a.precision == 0 ? kappa : 1.0);
    const int ts = a.t_dir > 0 ? 1 : -1;
    const bool far = kind == kKindFF;
    const bool has_m = kind != kKindScalar && !a.m_zero;
    const bool want_d = a.grad_ds != nullptr;
    cudaStream_t s = a.stream;
    long ns = a.ns, nt = a.nt;
    int mode = a.mode, gmode = a.gmode, ncx = a.ncx, ncy = a.ncy;
    double t = a.t_dir, k = a.k;
    const double *src7 = a.src7, *cur = a.cur, *tgt7 = a.tgt7, *cot = a.cot;
    double *grad_cur = a.grad_cur, *grad_ds = a.grad_ds, *grad_dt = a.grad_dt;
    const unsigned nblk_s = (unsigned)((ns + 255) / 256), nblk_t = (unsigned)((nt + 255) / 256);
    std::vector<void *> owned;
    int rc = 0;
    double *gam = nullptr;
    if ((rc = salloc(&gam, (size_t)12 * nt, s, owned))) { sfree(owned, s); return rc; }
    if (a.mode == kEHP) {
        // EHP is nonlinear in the target's fields: the EH forward at the same
        // inputs and precision, then the EHP map's vector-Jacobian product
        // there (po_adj_ehp_cot_kernel) gives the EH adjoint's cotangents
        double *eh = nullptr;
        if ((rc = salloc(&eh, (size_t)12 * nt, s, owned))) { sfree(owned, s); return rc; }
        RunArgs fa = a;
        fa.mode = kEH;
        fa.out = eh;
        fa.extent_host = nullptr;
        fa.band_host = nullptr;
        rc = run_device(fa);
        const double c_l = (double)2.99792458e8f, mu0 = (double)1.2566370614e-6f;
        double zi = 1.0 / std::sqrt(mu0 / (a.epsilon * (1.0 / (mu0 * c_l * c_l))));
        void *eargs[] = {&nt, &cot, &eh, &tgt7, &zi, &gam};
        if (!rc) rc = launch(adj_ehp_cot_kernel(), dim3((unsigned)((nt + 127) / 128)), dim3(128), eargs, 0, s);
    } else {
        void *cargs[] = {&mode, &nt, &cot, &tgt7, &t, &gam};
        rc = launch(adj_cot_kernel(), dim3(nblk_t), dim3(256), cargs, 0, s);
    }
    // scalar sources: 2-row currents (FP64 record: S' in its J.x slot; mixed
    // one-source record: the same, the other currents zero)
    const int fp64_scalar = kind == kKindScalar ? 1 : 0, mixed_scalar = kind == kKindScalar ? 2 : 0;

    if (a.precision == 1) {
        double *srcd = nullptr, *part = nullptr, *partt = nullptr;
        if (!rc && ((rc = salloc(&srcd, (size_t)ns * kRecD, s, owned)) ||
                    (rc = salloc(&part, (size_t)kAccAdj * ns, s, owned)) ||
                    (rc = salloc(&partt, (size_t)std::max(nt, 1L), s, owned)))) {
            sfree(owned, s);
            return rc;
        }
        void *pargs[] = {&ns, &src7, &cur, &gmode, &ncx, &ncy, &fac_re, &fac_im, (void *)&fp64_scalar, &srcd};
        if (!rc) rc = launch(pack_src_d_kernel(), dim3(nblk_s), dim3(256), pargs, 0, s);
        void *sargs[] = {&srcd, &ns, &tgt7, &gam, &nt, &k, &part};
        timing_mark(s, true);
        if (!rc) rc = launch(adj_src_fp64_kernel(kind, ts), dim3((unsigned)((ns + kThreadsD - 1) / kThreadsD)),
                             dim3(kThreadsD), sargs, 0, s);
        timing_mark(s, false);
        int one = 1;
        double dsc = far ? 1.0 : -1.0;
        void *eargs[] = {(void *)&kind, &one, &ns, &part, &src7, &gmode, &ncx, &ncy, &fac_re, &fac_im, &dsc,
                         &grad_cur, &grad_ds};
        if (!rc) rc = launch(adj_src_epilogue_kernel(), dim3(nblk_s), dim3(256), eargs, 0, s);
        if (!rc && grad_dt) {
            void *targs[] = {&srcd, &ns, &tgt7, &gam, &nt, &k, &partt};
            timing_mark(s, true);
            rc = launch(adj_tgt_fp64_kernel(kind, ts), dim3((unsigned)((nt + kThreadsD - 1) / kThreadsD)), dim3(kThreadsD),
                        targs, 0, s);
            timing_mark(s, false);
            double one_d = 1.0;
            void *teargs[] = {&one, &nt, &partt, &one_d, &grad_dt};
            if (!rc) rc = launch(adj_tgt_epilogue_kernel(), dim3(nblk_t), dim3(256), teargs, 0, s);
        }
        sfree(owned, s);
        return rc;
    }

    // ---- mixed precision
    double *bbox = nullptr;
    Frame *frame = nullptr;
    float4 *srcpk = nullptr;
    if (!rc && ((rc = salloc(&bbox, (size_t)kBboxBlocks * 6, s, owned)) || (rc = salloc(&frame, 1, s, owned)) ||
                (!far && (rc = salloc(&srcpk, (size_t)ns * kRec, s, owned))))) {
        sfree(owned, s);
        return rc;
    }
    long nb = far ? 0 : nt;
    void *bargs[] = {&src7, &ns, &tgt7, &nb, &bbox};
    if (!rc) rc = launch(bbox_kernel(), dim3(kBboxBlocks), dim3(kBboxThreads), bargs, 0, s);
    int nbb = kBboxBlocks;
    double kap = kappa;
    int centred = far ? 0 : 1;
    void *frargs[] = {&bbox, &nbb, &kap, &centred, &frame};
    if (!rc) rc = launch(frame_kernel(), dim3(1), dim3(32), frargs, 0, s);
    const int *ff_order = nullptr;   // far field: curve position -> source
    if (far) {
        // sources in Hilbert order, in the forward's tile records: one adjoint
        // CTA per tile, whose centre's phase goes into the cotangents
        const long n1 = std::max(ns, 1L);
        const long ntile = (ns + kTile - 1) / kTile;
        size_t sort_bytes = 0;
        unsigned long long *keys = nullptr;
        int *ord = nullptr;
        unsigned char *sort_tmp = nullptr;
        float4 *tiles = nullptr;
        cudaError_t e = ff_sort(nullptr, &sort_bytes, nullptr, nullptr, nullptr, nullptr, n1, s);
        if (e != cudaSuccess) rc = fail(2, std::string("sort size query: ") + err_str(e));
        if (!rc && ((rc = salloc(&keys, 2 * (size_t)n1, s, owned)) || (rc = salloc(&ord, 2 * (size_t)n1, s, owned)) ||
                    (rc = salloc(&sort_tmp, std::max<size_t>(sort_bytes, 16), s, owned)) ||
                    (rc = salloc(&tiles, (size_t)ntile * ff_tile4(has_m), s, owned)))) {
            sfree(owned, s);
            return rc;
        }
        unsigned long long *k_in = keys, *k_out = keys + n1;
        int *i_in = ord, *i_out = ord + n1;
        void *kargs[] = {&ns, &src7, &frame, &k_in, &i_in};
        if (!rc) rc = launch(ff_key_kernel(), dim3(nblk_s), dim3(256), kargs, 0, s);
        if (!rc) {
            e = ff_sort(sort_tmp, &sort_bytes, k_in, k_out, i_in, i_out, ns, s);
            if (e != cudaSuccess) rc = fail(2, std::string("source sort: ") + err_str(e));
            else note_launches(1);
        }
        ff_order = i_out;
        void *fpargs[] = {&ns, &ff_order, &src7, &cur, &gmode, &ncx, &ncy, &frame, &fac_re, &fac_im, &tiles};
        if (!rc) rc = launch(ff_pack_kernel(has_m), dim3((unsigned)ntile), dim3(32), fpargs, 0, s);
        srcpk = tiles;
    } else {
        void *psargs[] = {&ns, &src7, &cur, &gmode, &ncx, &ncy, &frame, &fac_re, &fac_im, (void *)&mixed_scalar,
                          &srcpk};
        if (!rc) rc = launch(pack_src_kernel(), dim3(nblk_s), dim3(256), psargs, 0, s);
    }
    // Pair-packed adjoint: sources in registers, pairs of targets streamed.
    // Near field fused (currents, source and target displacement in one pass).
    const bool want_t = grad_dt != nullptr;
    const int rec4 = adj_pk_rec4(kind, has_m, want_t);
    const long npair = (nt + 1) / 2;
    float *trec2 = nullptr;
    double *gt = nullptr;
    if (!rc && ((rc = salloc(&trec2, (size_t)npair * rec4 * 4, s, owned)) ||
                (want_t && (rc = salloc(&gt, (size_t)nt, s, owned))))) {
        sfree(owned, s);
        return rc;
    }
    int farflag = far ? 1 : 0;
    void *p2args[] = {&nt, &tgt7, &gam, &frame, &farflag, (void *)&rec4, &trec2};
    const unsigned nblk_p = (unsigned)((2 * npair + 255) / 256);
    if (!rc) rc = launch(adj_pack_tgt2_kernel(), dim3(nblk_p), dim3(256), p2args, 0, s);
    // direction boxes of the far-field tiles for the lit-tile proof (M = 0 kernels)
    int boxes = far && !has_m && nt > 0;
    void *tbargs[] = {&trec2, &nt};
    const unsigned ntile_a = (unsigned)((npair + adj_pk_pairs_per_tile() - 1) / adj_pk_pairs_per_tile());
    if (!rc && boxes) rc = launch(adj_tgt_box_kernel(), dim3(ntile_a), dim3(32), tbargs, 0, s);
    if (want_t) PO_CK_RC(cudaMemsetAsync(gt, 0, sizeof(double) * nt, s));
    BandList band{nullptr, nullptr, 0};   // near-tangent pairs (not the scalar kind)
    if (!rc && kind != kKindScalar) {
        band.cap = band_cap_for(ns, nt);
        if ((rc = salloc(&band.pairs, band.cap, s, owned)) || (rc = salloc(&band.count, 1, s, owned))) {
            sfree(owned, s);
            return rc;
        }
        PO_CK_RC(cudaMemsetAsync(band.count, 0, sizeof(unsigned), s));
    }
    void *fk = adj_pk_kernel(kind, ts, has_m, want_d, want_t);
    const int smem2 = adj_pk_smem_bytes(kind, has_m, want_t);
    int occ2 = 1;
    {
        // once per device and kernel: the shared-memory attribute and the occupancy
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = di->occ_adj.find(fk);
        if (it != di->occ_adj.end()) {
            occ2 = it->second;
        } else {
            PO_CK_RC(cudaFuncSetAttribute(fk, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2));
            PO_CK_RC(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, fk, kThreadsA, smem2));
            occ2 = std::max(occ2, 1);
            if (!rc) di->occ_adj[fk] = occ2;
        }
    }
    const long tile_t = 2L * adj_pk_pairs_per_tile();
    const long nsb = (ns + kThreadsA - 1) / kThreadsA;
    const long split = choose_split(nsb, nt, (long)di->sms * occ2, partial_cap(ns, kAccAdj), tile_t);
    const long tiles = std::max(1L, (nt + tile_t - 1) / tile_t);
    long chunk = ((tiles + split - 1) / split) * tile_t;
    double *part = nullptr;
    if (!rc && (rc = salloc(&part, (size_t)split * kAccAdj * ns, s, owned))) { sfree(owned, s); return rc; }
    const float4 *srcc = srcpk, *trc2 = reinterpret_cast<const float4 *>(trec2);
    void *fargs[] = {&srcc, &ns, &trc2, &nt, &chunk, &part, &gt, &err, &boxes, &band, &ff_order};
    timing_mark(s, true);
    if (!rc) rc = launch(fk, dim3((unsigned)nsb, (unsigned)split), dim3(kThreadsA), fargs, smem2, s);
    timing_mark(s, false);
    if (!rc && band.count) {
        // the near-tangent pairs, decided and summed in FP64 into chunk 0 (and gt)
        double inv_kappa = 1.0 / kappa;
        void *xargs[] = {&band, &ns, &src7, &cur, &gmode, &ncx, &ncy, &fac_re, &fac_im, &nt, &tgt7, &gam, &k,
                         &inv_kappa, &part, &gt, &err};
        rc = launch(adj_band_fixup_kernel(kind, ts, want_d, want_t), dim3(kFixupBlocks), dim3(256), xargs, 0, s);
    }
    int nspl = (int)split;
    double dsc = far ? kappa : -kappa;
    void *eargs[] = {(void *)&kind, &nspl, &ns, &part, &src7, &gmode, &ncx, &ncy, &fac_re, &fac_im, &dsc,
                     &grad_cur, &grad_ds};
    if (!rc) rc = launch(adj_src_epilogue_kernel(), dim3(nblk_s), dim3(256), eargs, 0, s);
    if (!rc && want_t) {
        int one = 1;
        double dsct = kappa;
        void *teargs[] = {&one, &nt, &gt, &dsct, &grad_dt};
        rc = launch(adj_tgt_epilogue_kernel(), dim3(nblk_t), dim3(256), teargs, 0, s);
    }
    if (!rc && a.extent_host) PO_CK_RC(cudaMemcpyAsync(a.extent_host, &frame->m, sizeof(double),
                                                       cudaMemcpyDeviceToHost, s));
    if (!rc && a.band_host && band.count)
        PO_CK_RC(cudaMemcpyAsync(a.band_host, band.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    sfree(owned, s);
    return rc;
}

}  // namespace po
