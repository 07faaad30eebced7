// po_noalloc.cu -- the propagation entry point that allocates nothing.
//
// Some callers of this library cannot allocate device memory: a serving or
// simulation framework that reserves the GPU's memory for its own pool (a
// cudaMalloc from inside it fails or fragments that pool), or a
// latency-critical loop that cannot accept the device-wide synchronisation
// cudaFree implies. po_run_dev_static serves them. It runs the same
// mixed-precision path as po_run_dev (po::mixed_prepare / mixed_launch), but
// its scratch (frame, packed sources and targets, the far field's sort
// buffers, source-chunk partials) is carved out of a fixed file-scope device
// array of kStaticScratchBytes. Every GPU that loads this library holds that
// array until the process exits.
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
constexpr size_t kOffStatus = 0;       // int: timeouts of calls with status == NULL
constexpr size_t kOffScratch = 256;    // the calls' scratch, from here to the end

std::mutex g_mu;
unsigned char *g_base[64] = {};        // device address of g_static_scratch, per device

// Once per device, with that device current: the array's device address.
// (cudaGetSymbolAddress gives it; the array's name in host code is only a
// host-side stand-in, not a device address.)
int setup(unsigned char *&base)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(2, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(2, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess)
            return fail(2, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
        g_base[dev] = static_cast<unsigned char *>(ptr);
    }
    base = g_base[dev];
    return 0;
}

// Scratch carved from the static array in order; no device work, no
// allocation. Running out is status 5, before the first launch.
class StaticScratch : public po::Scratch {
public:
    explicit StaticScratch(unsigned char *base) : base_(base) {}
    int take(void **p, size_t bytes) override
    {
        const size_t need = (std::max<size_t>(bytes, 16) + kAlign - 1) / kAlign * kAlign;
        if (need > room())
            return fail(5, "po_run_dev_static: this problem needs more scratch than the " +
                               std::to_string(kStaticScratchBytes) + "-byte static array holds (" +
                               std::to_string(used_ + need) + " bytes by the time it ran out; roughly 88*ns + "
                               "128*nt near field, 90*ns + 128*nt far field)");
        *p = base_ + kOffScratch + used_;
        used_ += need;
        return 0;
    }
    size_t room() const override { return kStaticScratchBytes - kOffScratch - used_; }
    unsigned band_cap(long, long) const override { return po::kBandCapStatic; }

private:
    unsigned char *base_;
    size_t used_ = 0;
};

}  // namespace

// The internal status word of the current device, or null before the entry's
// first call there. Read and cleared by po::read_device_error.
int *po::static_status_word()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    return g_base[dev] ? reinterpret_cast<int *>(g_base[dev] + kOffStatus) : nullptr;
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
    a.m_zero = (flags & 1) != 0;
    a.out = out;
    a.stream = static_cast<cudaStream_t>(stream);
    if (int rc = po::validate(a)) return rc;
    unsigned char *base = nullptr;
    if (int rc = setup(base)) return rc;
    // every buffer is carved out before any device work
    StaticScratch sc(base);
    po::MixedPlan plan;
    if (nt > 0)
        if (int rc = po::mixed_prepare(a, sc, plan)) return rc;
    // The caller's status word starts every call at zero. The internal word
    // (status == NULL) keeps a timeout until po_device_error reads and clears
    // it, so a later call cannot hide it.
    int *err = status ? status : reinterpret_cast<int *>(base + kOffStatus);
    if (status) {
        cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), a.stream);
        if (e != cudaSuccess) return fail(2, std::string("clearing the status word: ") + cudaGetErrorString(e));
    }
    if (nt == 0) return 0;
    return po::mixed_launch(a, plan, err);
}
