// static_scan.cu -- level counting for one potential without any device
// allocation (epscu_count_levels_static).
//
// Some callers cannot allocate device memory: code that runs inside another
// framework's memory pool or under a strict allocation budget, a process whose
// allocations are made up front by someone else, or a plugin called from a
// context where cudaMalloc is not permitted.  For them this entry point runs
// the trial-energy scan (the same prepare and TMA scan kernels as
// epscu_solve) on scratch that lives in a file-scope __device__ array of fixed
// size, allocated by the CUDA runtime when the library is loaded on a device
// and held until the process exits.  The caller passes the potential and the
// output buffer (both device pointers) and a stream.
//
//  * Maximum grid: kStaticMaxPoints points; longer grids are rejected.
//  * Host code cannot use the array's name as a device address, so the first
//    call on each device looks the address up with cudaGetSymbolAddress (with
//    that device current) and caches it; make that first call before any
//    stream capture.
//  * Every call shares the array and leaves its contents behind; the queue
//    header is cleared on the device at the start of each call.  Calls that
//    overlap on the GPU (different streams, or several host threads) race on
//    the array and must be serialised by the caller.
//  * The call returns before the GPU has run it, so a failure found on the
//    device (bad input flagged by the prepare kernel, a bounded wait of the
//    scan that ran out) is reported in the output: a last one-CTA kernel
//    then sets every count to EPSCU_STATIC_FAILED (-1).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "epscu.h"
#include "launch.h"

namespace epscu {

constexpr int kStaticMaxPoints = 65536;  // multiple of the scan's largest tile (4096)

struct StaticScanScratch {
    double W64[kStaticMaxPoints];
    double Msuf[kStaticMaxPoints];
    float2 Wf2[kStaticMaxPoints];
    PotMeta meta;
    Header hdr;
    int32_t order[4];
};

// ~1.5 MiB per device, for the lifetime of the process
static __device__ __align__(256) StaticScanScratch g_static_scan;

namespace {

__global__ void static_init_kernel(StaticScanScratch* s, double r_min, double r_max, double mu, double e_cap, int32_t N,
                                   int32_t n_trial) {
    PotMeta m{};
    m.r_min = r_min;
    m.r_max = r_max;
    m.mu = mu;
    m.e_cap = e_cap;
    m.off = 0;
    m.offf = 0;
    m.N = N;
    m.n_trial = n_trial;
    s->meta = m;
    Header h{};
    s->hdr = h;  // the scan's work queue starts at zero on every call
    s->order[0] = 0;
}

// Runs after the scan on the same stream: a device-side failure of the call
// (the scan's error word, or a potential the prepare kernel rejected) turns
// every count into EPSCU_STATIC_FAILED, so the caller can tell a failed call
// from a potential with no bound levels.
__global__ void static_finish_kernel(const StaticScanScratch* s, int32_t n_trial, int32_t* counts) {
    const bool failed = s->hdr.error != 0 || (s->meta.status & EPSCU_STATUS_BAD) != 0;
    if (!failed) return;
    for (int j = threadIdx.x; j < n_trial; j += blockDim.x) counts[j] = EPSCU_STATIC_FAILED;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
StaticScanScratch* g_addr[kMaxDevices] = {};

epscu_status static_fail(epscu_status s, const std::string& m) {
    set_last_error(m);  // read back with epscu_last_error()
    return s;
}

}  // namespace

}  // namespace epscu

using namespace epscu;

extern "C" epscu_status epscu_count_levels_static(const double* V, int32_t N, double r_min, double r_max, double mu,
                                                  double e_cap, int32_t n_trial, int32_t* counts, void* stream) {
    if (!V || !counts) return static_fail(EPSCU_ERR_INVALID, "V and counts must be device pointers");
    if (N < 5) return static_fail(EPSCU_ERR_INVALID, "fewer than 5 grid points");
    if (N > kStaticMaxPoints)
        return static_fail(EPSCU_ERR_CAPACITY, "grid of " + std::to_string(N) + " points exceeds the static scratch (" +
                                                   std::to_string(kStaticMaxPoints) + " points)");
    if (n_trial < 1 || n_trial > (1 << 24)) return static_fail(EPSCU_ERR_INVALID, "n_trial out of range");
    if (!(r_max > r_min) || !(mu > 0.0)) return static_fail(EPSCU_ERR_INVALID, "bad grid or mass");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return static_fail(EPSCU_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return static_fail(EPSCU_ERR_INVALID, "device ordinal out of range");
    StaticScanScratch* S = nullptr;
    int sm_count = 0;
    {
        // once per device, with that device current: the scratch's device
        // address and the scan kernels' shared-memory attributes
        std::lock_guard<std::mutex> g(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_static_scan);
            if (e != cudaSuccess) return static_fail(EPSCU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            scan32_set_attributes();
            g_addr[dev] = static_cast<StaticScanScratch*>(p);
        }
        S = g_addr[dev];
    }
    e = cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return static_fail(EPSCU_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = (cudaStream_t)stream;

    DevBatch b{};
    b.n = 1;
    b.meta = &S->meta;
    b.V64 = V;
    b.W64 = S->W64;
    b.Msuf = S->Msuf;
    b.Wf2 = S->Wf2;
    b.counts = counts;
    b.hdr = &S->hdr;
    b.order = S->order;
    b.n_trial = n_trial;
    b.min_level = 0;
    b.max_level = -1;
    b.max_N = N;
    b.tol = 1e-12;
    static_init_kernel<<<1, 1, 0, s>>>(S, r_min, r_max, mu, e_cap, N, n_trial);
    launch_prepare(b, s);
    const ScanShape shape{256, 2048, 3, 0};
    launch_scan32(b, shape, sm_count, s);
    static_finish_kernel<<<1, 1024, 0, s>>>(S, n_trial, counts);
    e = cudaGetLastError();
    if (e != cudaSuccess) return static_fail(EPSCU_ERR_CUDA, cudaGetErrorString(e));
    return EPSCU_OK;
}
