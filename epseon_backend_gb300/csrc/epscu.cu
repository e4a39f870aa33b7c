// epscu.cu -- host orchestration and C ABI of libepseon_cuda.
//
// One context per device: a stream, a growable device arena (block size from
// HardwareConfig::allocation_block_size, hardware_config.hpp:18), pinned
// staging buffers, a host-mapped cancel flag polled by the persistent kernels,
// the autotune cache of the scan kernel and a CUDA graph of the last
// device-resident solve (replayed when the same buffers are solved again).
//
// Solve pipeline:
//   prepare -> scan (FP64 | FP32 TMA persistent; for batches of >= 512
//   potentials the FP32 scan on every 16th trial energy, then a count round
//   inside the cells where the counts change) -> level set-up + brackets
//   plain : bisect64 -> norm64 -> twist64 -> write64            (native FP64)
//   fast  : window, then two branches on two streams (graph fork/join):
//             lane levels: refine32 -> newton_df -> norm_df
//             long levels: refine_long -> norm_long, then (after newton_df)
//                          the fallback levels' refinement and norm -> zero_psi
//           -> twist_long -> scale_psi   (FP32, then compensated FP32 with
//           FP64 matching and norm integral; the norm passes store psi-hat)
//   -> gather into the caller's layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "epscu.h"
#include "dfpass.cuh"
#include "launch.h"

using namespace epscu;

namespace {

thread_local std::string g_err;

epscu_status fail(epscu_status s, const std::string& msg) {
    g_err = msg;
    return s;
}

#define EPSCU_CU(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? EPSCU_ERR_NOMEM : EPSCU_ERR_CUDA,         \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

// The caller's stream (NULL: the legacy default stream) orders the inputs and
// receives the outputs; the work itself runs on the context's stream.
inline cudaStream_t caller_stream(const epscu_opts& o) { return o.stream ? (cudaStream_t)o.stream : cudaStreamLegacy; }

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

constexpr int kStageEvents = 12;  // 0-6 stages, 6-7 autotune, 8-9 around refine_long, 10-11 around zero_psi

}  // namespace

void epscu::set_last_error(const std::string& msg) { g_err = msg; }

struct epscu_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // the long levels' branch of the fast pipeline
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_newton = nullptr;
    size_t block = size_t(64) << 20;
    std::map<std::string, DevBuf> bufs;
    std::map<std::string, std::pair<void*, size_t>> pinned;
    volatile int32_t* cancel_host = nullptr;
    int32_t* cancel_dev = nullptr;
    cudaEvent_t ev[kStageEvents] = {};
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;  // ordering with the caller's stream
    // last solve (kept for the adjoint)
    DevBatch last{};
    bool have_last = false;
    int last_method = 0;
    bool last_psi = false;
    int64_t* last_offsets_dev = nullptr;
    int32_t* last_tiles_dev = nullptr;  // the adjoint's tile prefix over the potentials
    int32_t last_n_tiles = 0;
    int64_t last_total_points = 0;
    int64_t last_psi_total = 0;
    epscu_stats stats{};
    std::map<std::string, ScanShape> tune_cache;
    // CUDA graph of the last device-resident solve
    cudaGraphExec_t graph = nullptr;
    std::string graph_key;
    std::mutex mu;

    ~epscu_ctx() {
        cudaSetDevice(device);
        if (graph) cudaGraphExecDestroy(graph);
        for (auto& kv : bufs)
            if (kv.second.p) cudaFree(kv.second.p);
        for (auto& kv : pinned)
            if (kv.second.first) cudaFreeHost(kv.second.first);
        if (cancel_host) cudaFreeHost((void*)cancel_host);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (ev_newton) cudaEventDestroy(ev_newton);
        if (stream2) cudaStreamDestroy(stream2);
        if (stream) cudaStreamDestroy(stream);
    }

    // device buffer `name` with at least `bytes` (grown in arena blocks)
    void* get(const std::string& name, size_t bytes, cudaError_t* err) {
        DevBuf& b = bufs[name];
        if (bytes == 0) bytes = 256;
        if (b.cap >= bytes) return b.p;
        if (b.p) {
            cudaStreamSynchronize(stream);
            cudaFree(b.p);
            b.p = nullptr;
            b.cap = 0;
            if (graph) {  // captured pointers are stale
                cudaGraphExecDestroy(graph);
                graph = nullptr;
                graph_key.clear();
            }
        }
        const size_t blk = block ? block : (size_t(64) << 20);
        size_t want = bytes < blk ? ((bytes + 4095) & ~size_t(4095)) : ((bytes + blk - 1) / blk) * blk;
        *err = cudaMalloc(&b.p, want);
        if (*err != cudaSuccess) {
            b.p = nullptr;
            return nullptr;
        }
        b.cap = want;
        return b.p;
    }

    void* host(const std::string& name, size_t bytes, cudaError_t* err) {
        auto& h = pinned[name];
        if (h.second >= bytes && h.first) return h.first;
        if (h.first) {
            cudaStreamSynchronize(stream);
            cudaFreeHost(h.first);
            if (graph) {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
                graph_key.clear();
            }
        }
        h.first = nullptr;
        h.second = 0;
        *err = cudaHostAlloc(&h.first, bytes ? bytes : 64, cudaHostAllocDefault);
        if (*err != cudaSuccess) {
            h.first = nullptr;
            return nullptr;
        }
        h.second = bytes;
        return h.first;
    }
};

extern "C" {

int32_t epscu_abi_version(void) { return EPSCU_ABI_VERSION; }

const char* epscu_last_error(void) { return g_err.c_str(); }

epscu_status epscu_device_count(int32_t* count) {
    if (!count) return fail(EPSCU_ERR_INVALID, "count is NULL");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        *count = 0;
        cudaGetLastError();
        return fail(EPSCU_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    }
    *count = c;
    return EPSCU_OK;
}

epscu_status epscu_get_device_info(int32_t ordinal, epscu_device_info* info) {
    if (!info) return fail(EPSCU_ERR_INVALID, "info is NULL");
    cudaDeviceProp p;
    EPSCU_CU(cudaGetDeviceProperties(&p, ordinal));
    std::memset(info, 0, sizeof(*info));
    std::strncpy(info->name, p.name, sizeof(info->name) - 1);
    info->ordinal = ordinal;
    info->pci_device_id = p.pciDeviceID;
    info->pci_bus_id = p.pciBusID;
    info->cc_major = p.major;
    info->cc_minor = p.minor;
    info->sm_count = p.multiProcessorCount;
    info->total_global_mem = (int64_t)p.totalGlobalMem;
    info->shared_mem_per_block_optin = (int32_t)p.sharedMemPerBlockOptin;
    info->max_threads_per_block = p.maxThreadsPerBlock;
    for (int i = 0; i < 3; ++i) {
        info->max_grid_dim[i] = p.maxGridSize[i];
        info->max_block_dim[i] = p.maxThreadsDim[i];
    }
    info->l2_cache_size = p.l2CacheSize;
    int dv = 0, rv = 0;
    cudaDriverGetVersion(&dv);
    cudaRuntimeGetVersion(&rv);
    info->driver_version = dv;
    info->runtime_version = rv;
    std::memcpy(info->uuid, p.uuid.bytes, 16);
    return EPSCU_OK;
}

epscu_status epscu_create(int32_t device_ordinal, epscu_ctx** out) {
    if (!out) return fail(EPSCU_ERR_INVALID, "ctx out pointer is NULL");
    *out = nullptr;
    int count = 0;
    EPSCU_CU(cudaGetDeviceCount(&count));
    if (device_ordinal < 0 || device_ordinal >= count)
        return fail(EPSCU_ERR_INVALID, "device ordinal " + std::to_string(device_ordinal) + " out of range");
    EPSCU_CU(cudaSetDevice(device_ordinal));
    auto* c = new epscu_ctx();
    c->device = device_ordinal;
    cudaDeviceProp p;
    cudaError_t e = cudaGetDeviceProperties(&p, device_ordinal);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking);
    void* hc = nullptr;
    if (e == cudaSuccess) e = cudaHostAlloc(&hc, 64, cudaHostAllocMapped);
    if (e == cudaSuccess) {
        c->cancel_host = (volatile int32_t*)hc;
        *c->cancel_host = 0;
        e = cudaHostGetDevicePointer((void**)&c->cancel_dev, hc, 0);
    }
    for (int i = 0; i < kStageEvents && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_newton, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete c;
        return fail(EPSCU_ERR_CUDA, std::string("context set-up: ") + cudaGetErrorString(e));
    }
    c->sm_count = p.multiProcessorCount;
    scan32_set_attributes();
    *out = c;
    return EPSCU_OK;
}

epscu_status epscu_destroy(epscu_ctx* ctx) {
    if (!ctx) return EPSCU_OK;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    delete ctx;
    return EPSCU_OK;
}

epscu_status epscu_set_arena_block(epscu_ctx* ctx, int64_t bytes) {
    if (!ctx || bytes < 0) return fail(EPSCU_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->block = bytes ? (size_t)bytes : (size_t(64) << 20);
    return EPSCU_OK;
}

epscu_status epscu_cancel(epscu_ctx* ctx) {
    if (!ctx) return fail(EPSCU_ERR_INVALID, "ctx is NULL");
    // no lock (a running solve holds it); the kernels read the mapped flag
    __atomic_store_n(const_cast<int32_t*>(ctx->cancel_host), 1, __ATOMIC_RELEASE);
    return EPSCU_OK;
}

epscu_status epscu_cancel_clear(epscu_ctx* ctx) {
    if (!ctx) return fail(EPSCU_ERR_INVALID, "ctx is NULL");
    __atomic_store_n(const_cast<int32_t*>(ctx->cancel_host), 0, __ATOMIC_RELEASE);
    return EPSCU_OK;
}

epscu_status epscu_last_stats(epscu_ctx* ctx, epscu_stats* stats) {
    if (!ctx || !stats) return fail(EPSCU_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> g(ctx->mu);
    *stats = ctx->stats;
    return EPSCU_OK;
}

epscu_status epscu_measure_fma_peaks(epscu_ctx* ctx, double* fp32, double* fp64) {
    if (!ctx) return fail(EPSCU_ERR_INVALID, "ctx is NULL");
    std::lock_guard<std::mutex> g(ctx->mu);
    cudaSetDevice(ctx->device);
    measure_fma_peaks(ctx->sm_count, fp32, fp64);
    EPSCU_CU(cudaGetLastError());
    return EPSCU_OK;
}

}  // extern "C"

namespace {

// Launch the solve stages of DevBatch b on stream s (capturable).  part 0:
// everything; 1: up to the level setup (the psi size is then known on the
// device); 2: the rest.
void enqueue_pipeline(epscu_ctx* ctx, const DevBatch& b, int method, bool want_psi, const ScanShape& shape,
                      bool stage_events, cudaStream_t s, int part = 0) {
    auto rec = [&](int i) {
        if (stage_events) cudaEventRecord(ctx->ev[i], s);
    };
    if (part != 2) {
        rec(0);
        launch_prepare(b, s);
        if (method == EPSCU_METHOD_FAST_FP32C) launch_scan_window(b, ctx->sm_count, s);  // timed with prepare
        rec(1);
        if (method == EPSCU_METHOD_PLAIN_FP64) launch_scan64(b, s);
        else if (b.bis_list) launch_bisect_scan(b, shape, ctx->sm_count, s);
        else launch_scan32(b, shape, ctx->sm_count, s);
        rec(2);
        launch_level_setup(b, s);
        if (part == 1) return;
    }
    if (method == EPSCU_METHOD_PLAIN_FP64) {
        launch_bisect64(b, ctx->sm_count, s);
        rec(3);
        launch_norm64(b, 0, ctx->sm_count, s);
        launch_twist64(b, ctx->sm_count, s);
        rec(4);
        if (want_psi) launch_write64(b, ctx->sm_count, s);
    } else {
        launch_window(b, ctx->sm_count, s);
        if (!stage_events) {
            // the long levels (one CTA each), the middle levels (FP32 on lanes,
            // then one warp each) and the lane levels are disjoint: the CTA
            // branch runs beside the other two, filling the SMs the per-level
            // kernels leave idle as they drain.  The psi rows are zeroed
            // outside the level windows at the end of that branch, an HBM
            // stream beside the compute-bound lane kernels (the norm passes
            // write only inside the windows, so they need not wait for it;
            // zeroing first held back the long levels' refinement: measured
            // 29.6 against 28.7 ms a step on the 2048-potential batch).  The
            // levels newton_df could not settle take their refinement and
            // norm pass on CTAs in that branch too, once newton_df is done,
            // so norm_df need not wait for them (28.7 -> 27.7 ms)
            cudaEventRecord(ctx->ev_fork, s);
            cudaStreamWaitEvent(ctx->stream2, ctx->ev_fork, 0);
            launch_refine32(b, ctx->sm_count, s);
            launch_refine_long(b, ctx->sm_count, ctx->stream2);
            launch_norm_long(b, ctx->sm_count, ctx->stream2);
            launch_refine_mid(b, ctx->sm_count, s);
            launch_newton_df(b, ctx->sm_count, s);
            cudaEventRecord(ctx->ev_newton, s);
            cudaStreamWaitEvent(ctx->stream2, ctx->ev_newton, 0);
            launch_fallback_long(b, ctx->sm_count, ctx->stream2);
            launch_norm_fallback(b, ctx->sm_count, ctx->stream2);
            if (want_psi) launch_zero_psi(b, ctx->sm_count, ctx->stream2);
            cudaEventRecord(ctx->ev_join, ctx->stream2);
            launch_norm_mid(b, ctx->sm_count, s);
            launch_norm_df(b, ctx->sm_count, s);
            cudaStreamWaitEvent(s, ctx->ev_join, 0);
            launch_twist_long(b, ctx->sm_count, s);
        } else {
            // stage timing: one stream, stages in sequence
            launch_refine32(b, ctx->sm_count, s);
            rec(8);
            launch_refine_long(b, ctx->sm_count, s);
            rec(9);
            rec(3);
            launch_refine_mid(b, ctx->sm_count, s);
            launch_newton_df(b, ctx->sm_count, s);
            launch_fallback_long(b, ctx->sm_count, s);
            launch_norm_fallback(b, ctx->sm_count, s);
            rec(10);
            if (want_psi) launch_zero_psi(b, ctx->sm_count, s);
            rec(11);
            launch_norm_mid(b, ctx->sm_count, s);
            launch_norm_df(b, ctx->sm_count, s);
            launch_norm_long(b, ctx->sm_count, s);
            launch_twist_long(b, ctx->sm_count, s);
        }
        rec(4);
        // rows written unnormalised by norm_df / norm_long / twist_long
        if (want_psi) launch_scale_psi(b, ctx->sm_count, s);
    }
    rec(5);
}

std::string shape_key(int n, int n_trial, int64_t total) {
    return std::to_string(n) + ":" + std::to_string(n_trial) + ":" + std::to_string(total >> 16);
}

}  // namespace

extern "C" epscu_status epscu_solve(epscu_ctx* ctx, const epscu_batch* batch, epscu_result* res,
                                    const epscu_opts* opts_in) {
    if (!ctx || !batch || !res) return fail(EPSCU_ERR_INVALID, "NULL argument");
    epscu_opts opts{};
    opts.method = EPSCU_METHOD_FAST_FP32C;
    opts.tol = 1e-12;
    if (opts_in) opts = *opts_in;
    if (opts.tol <= 0) opts.tol = 1e-12;
    std::lock_guard<std::mutex> guard(ctx->mu);
    cudaSetDevice(ctx->device);
    const int n = batch->n_potentials;
    const int cap = res->level_capacity;
    const int method = opts.method;
    const bool dev = (opts.flags & EPSCU_MEM_DEVICE) != 0;
    const bool want_psi = (opts.flags & EPSCU_WANT_PSI) && res->psi && res->psi_capacity > 0;
    // host buffers, no psi buffer, psi kept in device memory for the adjoint:
    // the psi size is read back after the level setup, then the rest runs
    const bool keep_psi = (opts.flags & EPSCU_KEEP_PSI) && !want_psi && !dev;
    // device buffers, no psi buffer, an allocator: psi sized exactly after the
    // level setup, in the caller's memory
    const bool alloc_psi = dev && (opts.flags & EPSCU_WANT_PSI) && !res->psi && opts.psi_alloc != nullptr;
    // per-stage events (one stream, stages in sequence) only when asked for;
    // otherwise the fast method's two branches run side by side, graph-replayed
    // for device-resident inputs and launched directly for host buffers
    const bool stage_events = (opts.flags & EPSCU_STAGE_TIMING) != 0;
    if (n <= 0) return fail(EPSCU_ERR_INVALID, "n_potentials must be positive");
    if (cap <= 0) return fail(EPSCU_ERR_INVALID, "level_capacity must be positive");
    if (method != EPSCU_METHOD_PLAIN_FP64 && method != EPSCU_METHOD_FAST_FP32C)
        return fail(EPSCU_ERR_INVALID, "unknown method " + std::to_string(method));
    if (batch->n_trial < 1 || batch->n_trial > (1 << 24)) return fail(EPSCU_ERR_INVALID, "n_trial out of range");
    if (batch->min_level < 0) return fail(EPSCU_ERR_INVALID, "min_level must be >= 0");
    if (batch->max_level >= 0 && batch->max_level < batch->min_level)
        return fail(EPSCU_ERR_INVALID, "max_level < min_level");
    if (!batch->V || !batch->offsets || !batch->N || !batch->r_min || !batch->r_max || !batch->mu || !batch->e_cap)
        return fail(EPSCU_ERR_INVALID, "batch array is NULL");
    if (!res->n_total || !res->n_out || !res->energy || !res->nodes || !res->status)
        return fail(EPSCU_ERR_INVALID, "result array is NULL");
    if ((int64_t)n * cap > (int64_t)1 << 30) return fail(EPSCU_ERR_INVALID, "n * level_capacity too large");

    // ---- host-side metadata
    const int64_t tile = scan32_max_tile();
    int64_t total_points = 0, total_padded = 0;
    int32_t max_N = 0;
    cudaError_t ce = cudaSuccess;
    auto* hm = (PotMeta*)ctx->host("meta", sizeof(PotMeta) * n, &ce);
    auto* ho = (int32_t*)ctx->host("order", sizeof(int32_t) * n, &ce);
    auto* hoff = (int64_t*)ctx->host("offsets", sizeof(int64_t) * n, &ce);
    // the adjoint's CTAs: tiles of kAdjointPoints points of each potential, in
    // potential order (htile[p] = the first tile of potential p)
    auto* htile = (int32_t*)ctx->host("adj_tiles", sizeof(int32_t) * (n + 1), &ce);
    if (!hm || !ho || !hoff || !htile) return fail(EPSCU_ERR_NOMEM, "pinned staging allocation failed");
    htile[0] = 0;
    for (int p = 0; p < n; ++p) {
        const int32_t N = batch->N[p];
        const int64_t off = batch->offsets[p];
        if (N < 5) return fail(EPSCU_ERR_INVALID, "potential " + std::to_string(p) + " has fewer than 5 points");
        if (off < 0) return fail(EPSCU_ERR_INVALID, "negative offset");
        if (!(batch->r_max[p] > batch->r_min[p]) || !(batch->mu[p] > 0.0) || !std::isfinite(batch->e_cap[p]))
            return fail(EPSCU_ERR_INVALID, "potential " + std::to_string(p) + " has a bad grid, mass or energy cap");
        PotMeta m{};
        m.r_min = batch->r_min[p];
        m.r_max = batch->r_max[p];
        m.mu = batch->mu[p];
        m.e_cap = batch->e_cap[p];
        m.off = off;
        m.offf = total_padded;
        m.N = N;
        m.n_trial = batch->n_trial;
        hm[p] = m;
        hoff[p] = off;
        htile[p + 1] = htile[p] + (N + kAdjointPoints - 1) / kAdjointPoints;
        total_points = std::max<int64_t>(total_points, off + N);
        total_padded += ((N + tile - 1) / tile) * tile;
        max_N = std::max(max_N, N);
    }
    std::vector<int32_t> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return batch->N[a] > batch->N[b]; });
    std::memcpy(ho, ord.data(), sizeof(int32_t) * n);

    // ---- device buffers
    cudaStream_t s = ctx->stream;
    const cudaStream_t caller = caller_stream(opts);
    EPSCU_CU(cudaEventRecord(ctx->ev_in, caller));
    EPSCU_CU(cudaStreamWaitEvent(s, ctx->ev_in, 0));
    const int64_t lv = (int64_t)n * cap;
    DevBatch b{};
    b.n = n;
    b.meta = (PotMeta*)ctx->get("meta", sizeof(PotMeta) * n, &ce);
    b.W64 = (double*)ctx->get("W64", sizeof(double) * total_points, &ce);
    b.Msuf = (double*)ctx->get("Msuf", sizeof(double) * total_points, &ce);
    b.Wf2 = method == EPSCU_METHOD_FAST_FP32C ? (float2*)ctx->get("Wf2", sizeof(float2) * total_padded, &ce) : nullptr;
    b.counts = (int32_t*)ctx->get("counts", sizeof(int32_t) * (size_t)n * batch->n_trial, &ce);
    b.gam = method == EPSCU_METHOD_FAST_FP32C ? (float*)ctx->get("gam", sizeof(float) * (size_t)n * batch->n_trial, &ce)
                                              : nullptr;
    b.levels = (LevelWork*)ctx->get("levels", sizeof(LevelWork) * lv, &ce);
    b.fallback_list = (int32_t*)ctx->get("fallback_list", sizeof(int32_t) * lv, &ce);
    b.max_units = (int32_t)(n + lv / 32 + 1);
    b.units = (int2*)ctx->get("units", sizeof(int2) * (size_t)b.max_units, &ce);
    b.max_twist = 4096;
    b.twist_list = (int32_t*)ctx->get("twist_list", sizeof(int32_t) * b.max_twist, &ce);
    b.hdr = (Header*)ctx->get("hdr", sizeof(Header), &ce);
    b.order = (int32_t*)ctx->get("order", sizeof(int32_t) * n, &ce);
    b.scan_win = nullptr;
    b.long_list = nullptr;
    b.mid_list = nullptr;
    b.bis_list = nullptr;
    b.bis_n = nullptr;
    b.bis_items = nullptr;
    b.max_bis_items = 0;
    b.Mpre = nullptr;
    b.Bmin = nullptr;
    if (method == EPSCU_METHOD_FAST_FP32C) {
        b.Mpre = (double*)ctx->get("Mpre", sizeof(double) * total_points, &ce);
        b.Bmin = (float*)ctx->get("Bmin", sizeof(float) * (size_t)(total_padded / 32 + 1), &ce);
        if (!b.Mpre || !b.Bmin) return fail(EPSCU_ERR_NOMEM, "device arena (window bounds)");
        b.long_list = (int32_t*)ctx->get("long_list", sizeof(int32_t) * lv, &ce);
        if (!b.long_list) return fail(EPSCU_ERR_NOMEM, "device arena (long list)");
        b.mid_list = (int32_t*)ctx->get("mid_list", sizeof(int32_t) * lv, &ce);
        if (!b.mid_list) return fail(EPSCU_ERR_NOMEM, "device arena (middle list)");
        const size_t nb = (size_t)(batch->n_trial + kScanWinBlock - 1) / kScanWinBlock;
        b.scan_win = (int2*)ctx->get("scan_win", sizeof(int2) * (size_t)n * nb, &ce);
        if (!b.scan_win) return fail(EPSCU_ERR_NOMEM, "device arena (scan windows)");
        if (n >= kBisectMinPotentials) {
            // batches: the bisection scan (counts where they change only)
            b.bis_list = (int32_t*)ctx->get("bis_list", sizeof(int32_t) * (size_t)n * batch->n_trial, &ce);
            b.bis_n = (int32_t*)ctx->get("bis_n", sizeof(int32_t) * (size_t)n, &ce);
            const int64_t items = bisect_max_items(n, batch->n_trial);
            b.bis_items = (int2*)ctx->get("bis_items", sizeof(int2) * (size_t)items, &ce);
            b.max_bis_items = (int32_t)std::min<int64_t>(items, 1 << 30);
            if (!b.bis_list || !b.bis_n || !b.bis_items) return fail(EPSCU_ERR_NOMEM, "device arena (bisection scan)");
        }
    }
    int64_t* d_off = (int64_t*)ctx->get("offsets", sizeof(int64_t) * n, &ce);
    int32_t* d_tiles = (int32_t*)ctx->get("adj_tiles", sizeof(int32_t) * (n + 1), &ce);
    if (ce != cudaSuccess || !b.meta || !b.W64 || !b.Msuf || !b.counts || !b.levels || !b.fallback_list || !b.units ||
        !b.hdr ||
        !b.order || !d_off || !d_tiles ||
        (method == EPSCU_METHOD_FAST_FP32C && !b.Wf2))
        return fail(EPSCU_ERR_NOMEM, std::string("device arena: ") + cudaGetErrorString(ce));
    if (dev) {
        b.V64 = batch->V;
    } else {
        double* v = (double*)ctx->get("V64", sizeof(double) * total_points, &ce);
        if (!v) return fail(EPSCU_ERR_NOMEM, "device arena (V)");
        b.V64 = v;
    }
    b.max_levels = (int32_t)lv;
    b.level_capacity = cap;
    b.cancel = ctx->cancel_dev;
    b.n_trial = batch->n_trial;
    b.min_level = batch->min_level;
    b.max_level = batch->max_level;
    b.max_N = max_N;
    b.twist_stride = max_N / kTwistSample + 4;
    b.twist_scratch = (double*)ctx->get("twist_scratch", sizeof(double) * (size_t)b.max_twist * b.twist_stride, &ce);
    if (!b.twist_scratch || !b.twist_list) return fail(EPSCU_ERR_NOMEM, "device arena (twist search)");
    b.tol = opts.tol;
    b.long_window = opts.long_window > 0 ? opts.long_window : 0;  // 0: chosen from the level count
    b.wait_polls = opts.wait_polls;  // 0: the default bound; < 0: the failure self-test
    b.mid_window = opts.mid_window;  // 0: the default middle-tier threshold; < 0: no middle tier
    b.max_iter = opts.max_iter > 0 ? opts.max_iter : 0;            // 0: the default caps
    b.psi = nullptr;
    b.psi_capacity = 0;
    if (want_psi) {
        if (dev) {
            b.psi = res->psi;
        } else {
            b.psi = (double*)ctx->get("psi", sizeof(double) * (size_t)res->psi_capacity, &ce);
            if (!b.psi) return fail(EPSCU_ERR_NOMEM, "device arena (psi)");
        }
        b.psi_capacity = res->psi_capacity;
    }
    int32_t *o_nt, *o_no, *o_nd, *o_st;
    double *o_e, *o_err;
    if (dev) {
        o_nt = res->n_total;
        o_no = res->n_out;
        o_e = res->energy;
        o_nd = res->nodes;
        o_st = res->status;
        o_err = res->err_est;
    } else {
        o_nt = (int32_t*)ctx->get("o_nt", sizeof(int32_t) * n, &ce);
        o_no = (int32_t*)ctx->get("o_no", sizeof(int32_t) * n, &ce);
        o_e = (double*)ctx->get("o_e", sizeof(double) * lv, &ce);
        o_nd = (int32_t*)ctx->get("o_nd", sizeof(int32_t) * lv, &ce);
        o_st = (int32_t*)ctx->get("o_st", sizeof(int32_t) * lv, &ce);
        o_err = (double*)ctx->get("o_err", sizeof(double) * lv, &ce);
        if (!o_nt || !o_no || !o_e || !o_nd || !o_st || !o_err) return fail(EPSCU_ERR_NOMEM, "device arena (outputs)");
    }
    auto* hh = (Header*)ctx->host("hdr", sizeof(Header), &ce);
    if (!hh) return fail(EPSCU_ERR_NOMEM, "pinned staging (hdr)");
    std::memset(hh, 0, sizeof(Header));
    // (the cancel flag is not cleared here: a request made before the solve
    // starts stops this solve, which consumes it below)

    // ---- launch shape of the FP32 scan (autotuned per batch shape)
    ScanShape shape{256, 2048, 3, 0};
    const std::string skey = shape_key(n, batch->n_trial, total_points);
    auto it = ctx->tune_cache.find(skey);
    if (it != ctx->tune_cache.end()) shape = it->second;

    // ---- inputs
    if (!dev) EPSCU_CU(cudaMemcpyAsync((void*)b.V64, batch->V, sizeof(double) * total_points, cudaMemcpyHostToDevice, s));

    if (method == EPSCU_METHOD_FAST_FP32C && opts.tune && it == ctx->tune_cache.end()) {
        // time each scan variant on this batch, keep the fastest
        EPSCU_CU(cudaMemcpyAsync(b.meta, hm, sizeof(PotMeta) * n, cudaMemcpyHostToDevice, s));
        EPSCU_CU(cudaMemcpyAsync(b.order, ho, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
        EPSCU_CU(cudaMemsetAsync(b.Wf2, 0, sizeof(float2) * total_padded, s));
        EPSCU_CU(cudaMemsetAsync(b.hdr, 0, sizeof(Header), s));
        launch_prepare(b, s);
        launch_scan_window(b, ctx->sm_count, s);
        // (fewer stages: less shared memory, more resident CTAs per SM)
        const ScanShape cands[] = {{128, 1024, 2, 0}, {128, 1024, 4, 0}, {128, 2048, 2, 0}, {128, 2048, 3, 0},
                                   {256, 1024, 2, 0}, {256, 1024, 4, 0}, {256, 2048, 3, 0}, {256, 4096, 2, 0},
                                   {512, 1024, 4, 0}, {512, 2048, 3, 0}};
        float best = 1e30f;
        for (const ScanShape& c : cands) {
            EPSCU_CU(cudaMemsetAsync(&b.hdr->queue_scan, 0, sizeof(int32_t), s));
            EPSCU_CU(cudaEventRecord(ctx->ev[6], s));
            launch_scan32(b, c, ctx->sm_count, s, b.bis_list ? kBisectCoarse : 1);
            EPSCU_CU(cudaEventRecord(ctx->ev[7], s));
            EPSCU_CU(cudaEventSynchronize(ctx->ev[7]));
            EPSCU_CU(cudaGetLastError());
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]);
            if (ms < best) {
                best = ms;
                shape = c;
            }
        }
        ctx->tune_cache[skey] = shape;
    }

    // ---- the pipeline (graph-replayed when the device-resident inputs repeat)
    const bool use_graph = dev && !stage_events && !alloc_psi;
    char keybuf[512];
    std::string keybuf_extra;
    std::snprintf(keybuf, sizeof(keybuf), "%d|%d|%d|%d|%p|%p|%p|%p|%p|%p|%p|%p|%lld|%d|%d|%d|%d|%d|%g|%p", n,
                  batch->n_trial, batch->min_level, batch->max_level, (const void*)b.V64, (void*)b.psi,
                  (void*)o_e, (void*)o_nt, (void*)o_no, (void*)o_nd, (void*)o_st, (void*)o_err,
                  (long long)b.psi_capacity, method, cap, shape.threads, shape.tile, shape.stages, opts.tol,
                  (void*)s);  // s is the context's own stream
    keybuf_extra = std::to_string(b.long_window) + "|" + std::to_string(b.mid_window) + "|" +
                   std::to_string(b.wait_polls) + "|" + std::to_string(b.max_iter);
    const std::string gkey = std::string(keybuf) + "|" + std::to_string(total_points) + "|" + keybuf_extra;

    auto enqueue_inputs = [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = cudaMemcpyAsync(b.meta, hm, sizeof(PotMeta) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(b.order, ho, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(d_off, hoff, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(d_tiles, htile, sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return e;
        if ((e = cudaMemsetAsync(b.hdr, 0, sizeof(Header), s)) != cudaSuccess) return e;
        if (b.Wf2 && (e = cudaMemsetAsync(b.Wf2, 0, sizeof(float2) * total_padded, s)) != cudaSuccess) return e;
        return cudaSuccess;
    };
    auto enqueue_all = [&]() -> cudaError_t {
        cudaError_t e = enqueue_inputs();
        if (e != cudaSuccess) return e;
        enqueue_pipeline(ctx, b, method, want_psi, shape, stage_events, s);
        launch_gather(b, o_nt, o_no, o_e, o_nd, o_st, o_err, method == EPSCU_METHOD_FAST_FP32C ? 1 : 0, s);
        if (stage_events) cudaEventRecord(ctx->ev[6], s);
        return cudaGetLastError();
    };

    if (use_graph) {
        if (!ctx->graph || ctx->graph_key != gkey) {
            if (ctx->graph) {
                cudaGraphExecDestroy(ctx->graph);
                ctx->graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            EPSCU_CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue_all();
            cudaError_t e2 = cudaStreamEndCapture(s, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return fail(EPSCU_ERR_CUDA, std::string("graph capture: ") +
                                                cudaGetErrorString(e != cudaSuccess ? e : e2));
            }
            e = cudaGraphInstantiate(&ctx->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                ctx->graph = nullptr;
                return fail(EPSCU_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            }
            ctx->graph_key = gkey;
        }
        EPSCU_CU(cudaEventRecord(ctx->ev[0], s));
        EPSCU_CU(cudaGraphLaunch(ctx->graph, s));
        EPSCU_CU(cudaEventRecord(ctx->ev[6], s));
    } else if (keep_psi || alloc_psi) {
        if (!stage_events) EPSCU_CU(cudaEventRecord(ctx->ev[0], s));
        EPSCU_CU(enqueue_inputs());
        enqueue_pipeline(ctx, b, method, true, shape, stage_events, s, 1);
        EPSCU_CU(cudaMemcpyAsync(hh, b.hdr, sizeof(Header), cudaMemcpyDeviceToHost, s));
        EPSCU_CU(cudaStreamSynchronize(s));
        const int64_t need = std::max<int64_t>(1, hh->psi_total);
        if (keep_psi) {
            b.psi = (double*)ctx->get("psi_keep", sizeof(double) * (size_t)need, &ce);
            if (!b.psi) return fail(EPSCU_ERR_NOMEM, "device arena (kept psi)");
            b.psi_capacity = need;
        } else {
            b.psi = static_cast<double*>(opts.psi_alloc(need * (int64_t)sizeof(double), opts.psi_alloc_user));
            b.psi_capacity = b.psi ? need : 0;
            res->psi = b.psi;
            res->psi_capacity = b.psi_capacity;
        }
        enqueue_pipeline(ctx, b, method, b.psi != nullptr, shape, stage_events, s, 2);
        launch_gather(b, o_nt, o_no, o_e, o_nd, o_st, o_err, method == EPSCU_METHOD_FAST_FP32C ? 1 : 0, s);
        EPSCU_CU(cudaEventRecord(ctx->ev[6], s));
        EPSCU_CU(cudaGetLastError());
    } else {
        if (!stage_events) EPSCU_CU(cudaEventRecord(ctx->ev[0], s));
        EPSCU_CU(enqueue_all());
        if (!stage_events) EPSCU_CU(cudaEventRecord(ctx->ev[6], s));
    }

    // ---- outputs back
    if (!dev) {
        EPSCU_CU(cudaMemcpyAsync(res->n_total, o_nt, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
        EPSCU_CU(cudaMemcpyAsync(res->n_out, o_no, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
        EPSCU_CU(cudaMemcpyAsync(res->energy, o_e, sizeof(double) * lv, cudaMemcpyDeviceToHost, s));
        EPSCU_CU(cudaMemcpyAsync(res->nodes, o_nd, sizeof(int32_t) * lv, cudaMemcpyDeviceToHost, s));
        EPSCU_CU(cudaMemcpyAsync(res->status, o_st, sizeof(int32_t) * lv, cudaMemcpyDeviceToHost, s));
        if (res->err_est)
            EPSCU_CU(cudaMemcpyAsync(res->err_est, o_err, sizeof(double) * lv, cudaMemcpyDeviceToHost, s));
    }
    EPSCU_CU(cudaMemcpyAsync(hm, b.meta, sizeof(PotMeta) * n, cudaMemcpyDeviceToHost, s));
    EPSCU_CU(cudaMemcpyAsync(hh, b.hdr, sizeof(Header), cudaMemcpyDeviceToHost, s));
    EPSCU_CU(cudaEventRecord(ctx->ev_out, s));
    EPSCU_CU(cudaStreamWaitEvent(caller, ctx->ev_out, 0));
    EPSCU_CU(cudaStreamSynchronize(s));
    EPSCU_CU(cudaGetLastError());

    // psi offsets / size
    int64_t psi_total = 0;
    for (int p = 0; p < n; ++p) {
        if (res->psi_offsets) res->psi_offsets[p] = hm[p].psi_off;
        psi_total = std::max<int64_t>(psi_total, hm[p].psi_off + (int64_t)hm[p].n_out * hm[p].N);
    }
    res->psi_required = psi_total;
    if (want_psi && !dev && hh->error == 0 && psi_total > 0)
        EPSCU_CU(cudaMemcpy(res->psi, b.psi, sizeof(double) * psi_total, cudaMemcpyDeviceToHost));

    // stats
    epscu_stats st{};
    float ms = 0.f;
    if (stage_events) {
        auto el = [&](int a, int c) {
            float x = 0.f;
            cudaEventElapsedTime(&x, ctx->ev[a], ctx->ev[c]);
            return x;
        };
        st.ms_prepare = el(0, 1);
        st.ms_scan = el(1, 2);
        if (method == EPSCU_METHOD_PLAIN_FP64) {
            st.ms_refine32 = 0.f;
            st.ms_polish64 = el(2, 3) + el(3, 4);
        } else {
            st.ms_refine32 = el(2, 3);
            st.ms_polish64 = el(3, 4);
        }
        st.ms_write = el(4, 5);
        st.ms_total = el(0, 6);
        if (method == EPSCU_METHOD_FAST_FP32C) {
            st.ms_refine_long = el(8, 9);
            st.ms_zero_psi = el(10, 11);
        }
    } else {
        cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[6]);
        st.ms_total = ms;
    }
    int64_t scan_pts = 0, lvl_pts = 0;
    int64_t nlev = 0;
    for (int p = 0; p < n; ++p) {
        const int64_t interior = std::max(0, hm[p].i1 - hm[p].i0);
        scan_pts += interior * batch->n_trial;
        lvl_pts += interior * hm[p].n_out;
        nlev += hm[p].n_out;
    }
    // the windowed FP32 scan counts what it did; the FP64 scan covers [i0, i1]
    st.scan_point_updates = hh->scan_updates > 0 ? (int64_t)hh->scan_updates : scan_pts;
    st.n_levels = nlev;
    st.fallbacks = hh->fallbacks;
    st.twist_searches = hh->n_twist;
    st.norm_redos = hh->n_redo;
    const bool psi_on = want_psi || keep_psi || (alloc_psi && b.psi);
    st.psi_bytes = psi_on ? psi_total * 8 : 0;
    // plain: prepare, scan64, level/unit setup, bracket, bisect64, norm64,
    // twist64, gather (+ write64); fast: prepare, scan window, scan32, level/unit
    // setup, bracket, window, refine32, refine_long, newton_df, fallback
    // (refine_long over the fallback list), its norm (norm_long over the
    // fallback list), norm_df, norm_long, twist_long, gather (+ refine_mid,
    // norm_mid with the middle tier; + zero_psi, scale_psi)
    const bool psi_kernels = psi_on;
    const bool mid_on = b.mid_list && (b.mid_window != 0 ? b.mid_window : kMidWindow) > 0;
    st.kernel_launches = method == EPSCU_METHOD_FAST_FP32C ? 16 + (mid_on ? 2 : 0) + (psi_kernels ? 2 : 0)
                                                           : 9 + (psi_kernels ? 1 : 0);
    if (b.bis_list) {  // the plan + count rounds after the coarse scan32
        for (int W = kBisectCoarse; W > 1; W /= (W < kBisectSplit ? W : kBisectSplit)) st.kernel_launches += 2;
    }
    if (method == EPSCU_METHOD_PLAIN_FP64) {
        st.refine_point_updates = 0;
        int64_t bis = 0;
        for (int p = 0; p < n; ++p) bis += (int64_t)std::max(0, hm[p].i1 - hm[p].i0) * hm[p].n_out * hm[p].n_bisect;
        st.fp64_point_updates = scan_pts + bis + lvl_pts * (psi_on ? 2 : 1);
    } else {
        // counted by the kernels over the level windows (algorithmic
        // point-updates: the long-window passes do ~3x this on 256 threads)
        st.refine_point_updates = (int64_t)hh->refine_updates;
        st.fp64_point_updates = (int64_t)hh->df_updates;
        st.refine_max_level_updates = (int64_t)hh->refine_max_updates;
        st.df_max_level_updates = (int64_t)hh->df_max_updates;
        st.refine_max_iters = hh->refine_max_iters;
        st.long_fp32_point_updates = (int64_t)hh->long32_updates;
        st.long_df_point_updates = (int64_t)hh->longdf_updates;
        st.psi_zero_points = (int64_t)hh->psi_zero_points;
        st.psi_window_points = (int64_t)hh->psi_window_points;
    }
    ctx->stats = st;

    // keep for the adjoint
    ctx->last = b;
    ctx->have_last = true;
    ctx->last_method = method;
    ctx->last_psi = psi_on && hh->error == 0;
    ctx->last_offsets_dev = d_off;
    ctx->last_tiles_dev = d_tiles;
    ctx->last_n_tiles = htile[n];
    ctx->last_total_points = total_points;
    ctx->last_psi_total = psi_total;

    // a cancel request is consumed by the solve it reached
    const bool cancelled = __atomic_exchange_n(const_cast<int32_t*>(ctx->cancel_host), 0, __ATOMIC_ACQ_REL) != 0;
    if (hh->error == EPSCU_ERR_CAPACITY || (want_psi && psi_total > res->psi_capacity))
        return fail(EPSCU_ERR_CAPACITY, "psi buffer too small: " + std::to_string(psi_total) + " doubles required");
    if (hh->error == EPSCU_ERR_TIMEOUT)
        return fail(EPSCU_ERR_TIMEOUT, "a bounded wait of the TMA scan ran out (results incomplete)");
    if (hh->error) return fail(hh->error, "device-side error " + std::to_string(hh->error));
    if (cancelled) return fail(EPSCU_ERR_CANCELLED, "solve cancelled");
    return EPSCU_OK;
}

extern "C" epscu_status epscu_adjoint(epscu_ctx* ctx, const double* dL_dE, double* dL_dV, int32_t recompute,
                                      const epscu_opts* opts_in) {
    if (!ctx || !dL_dE || !dL_dV) return fail(EPSCU_ERR_INVALID, "NULL argument");
    epscu_opts opts{};
    if (opts_in) opts = *opts_in;
    std::lock_guard<std::mutex> guard(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->have_last) return fail(EPSCU_ERR_INVALID, "no solve to differentiate on this context");
    DevBatch b = ctx->last;
    cudaStream_t s = ctx->stream;
    const cudaStream_t caller = caller_stream(opts);
    EPSCU_CU(cudaEventRecord(ctx->ev_in, caller));
    EPSCU_CU(cudaStreamWaitEvent(s, ctx->ev_in, 0));
    cudaError_t ce = cudaSuccess;
    if (!ctx->last_psi) {
        if (!recompute) return fail(EPSCU_ERR_INVALID, "last solve kept no wavefunctions; pass recompute=1");
        // recompute psi of the last solve into the arena
        double* psi = (double*)ctx->get("psi_adj", sizeof(double) * (size_t)std::max<int64_t>(1, ctx->last_psi_total), &ce);
        if (!psi) return fail(EPSCU_ERR_NOMEM, "device arena (recomputed psi)");
        b.psi = psi;
        b.psi_capacity = ctx->last_psi_total;
        // the writer of the solve's own method (its norm constants belong to it)
        const int qid = ctx->last_method == EPSCU_METHOD_FAST_FP32C ? kQWriteDF : kQWrite64;
        EPSCU_CU(cudaMemsetAsync(&b.hdr->queue[qid], 0, sizeof(int32_t), s));
        if (ctx->last_method == EPSCU_METHOD_FAST_FP32C) {
            launch_zero_psi(b, ctx->sm_count, s);  // write_long writes only the windows
            launch_write_df(b, ctx->sm_count, s);
            launch_write_long(b, ctx->sm_count, s);
        } else {
            launch_write64(b, ctx->sm_count, s);
        }
    }
    const bool dev = (opts.flags & EPSCU_MEM_DEVICE) != 0;
    const int64_t lv = (int64_t)b.n * b.level_capacity;
    const double* gE = dL_dE;
    double* gV = dL_dV;
    if (!dev) {
        double* d_gE = (double*)ctx->get("adj_gE", sizeof(double) * lv, &ce);
        double* d_gV = (double*)ctx->get("adj_gV", sizeof(double) * ctx->last_total_points, &ce);
        if (!d_gE || !d_gV) return fail(EPSCU_ERR_NOMEM, "device arena (adjoint)");
        EPSCU_CU(cudaMemcpyAsync(d_gE, dL_dE, sizeof(double) * lv, cudaMemcpyHostToDevice, s));
        EPSCU_CU(cudaMemsetAsync(d_gV, 0, sizeof(double) * ctx->last_total_points, s));
        gE = d_gE;
        gV = d_gV;
    }
    launch_adjoint(b, gE, gV, ctx->last_offsets_dev, ctx->last_tiles_dev, ctx->last_n_tiles, s);
    EPSCU_CU(cudaGetLastError());
    if (!dev) EPSCU_CU(cudaMemcpyAsync(dL_dV, gV, sizeof(double) * ctx->last_total_points, cudaMemcpyDeviceToHost, s));
    EPSCU_CU(cudaEventRecord(ctx->ev_out, s));
    EPSCU_CU(cudaStreamWaitEvent(caller, ctx->ev_out, 0));
    EPSCU_CU(cudaStreamSynchronize(s));
    return EPSCU_OK;
}

extern "C" epscu_status epscu_adjoint_psi(epscu_ctx* ctx, int32_t n, const int64_t* offsets, const int32_t* N,
                                          const double* r_min, const double* r_max, const int32_t* n_out,
                                          int32_t cap, const double* psi, const int64_t* psi_offsets,
                                          const double* dL_dE, double* dL_dV, const epscu_opts* opts_in) {
    if (!ctx || n <= 0 || cap <= 0 || !offsets || !N || !r_min || !r_max || !n_out || !psi || !psi_offsets ||
        !dL_dE || !dL_dV)
        return fail(EPSCU_ERR_INVALID, "bad arguments");
    epscu_opts opts{};
    if (opts_in) opts = *opts_in;
    std::lock_guard<std::mutex> guard(ctx->mu);
    cudaSetDevice(ctx->device);
    const bool dev = (opts.flags & EPSCU_MEM_DEVICE) != 0;
    std::vector<double> h(n);
    int64_t total = 0, psi_total = 0;
    int32_t max_N = 0;
    for (int p = 0; p < n; ++p) {
        if (N[p] < 2 || n_out[p] < 0 || n_out[p] > cap) return fail(EPSCU_ERR_INVALID, "bad N or n_out");
        h[p] = (r_max[p] - r_min[p]) / (double)(N[p] - 1);
        total = std::max<int64_t>(total, offsets[p] + N[p]);
        psi_total = std::max<int64_t>(psi_total, psi_offsets[p] + (int64_t)n_out[p] * N[p]);
        max_N = std::max(max_N, N[p]);
    }
    cudaError_t ce = cudaSuccess;
    auto* d_off = (int64_t*)ctx->get("adjx_off", sizeof(int64_t) * n, &ce);
    auto* d_N = (int32_t*)ctx->get("adjx_N", sizeof(int32_t) * n, &ce);
    auto* d_h = (double*)ctx->get("adjx_h", sizeof(double) * n, &ce);
    auto* d_no = (int32_t*)ctx->get("adjx_no", sizeof(int32_t) * n, &ce);
    auto* d_po = (int64_t*)ctx->get("adjx_po", sizeof(int64_t) * n, &ce);
    if (!d_off || !d_N || !d_h || !d_no || !d_po) return fail(EPSCU_ERR_NOMEM, "device arena (adjoint)");
    cudaStream_t s = ctx->stream;
    const cudaStream_t caller = caller_stream(opts);
    EPSCU_CU(cudaEventRecord(ctx->ev_in, caller));
    EPSCU_CU(cudaStreamWaitEvent(s, ctx->ev_in, 0));
    EPSCU_CU(cudaMemcpyAsync(d_off, offsets, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_N, N, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_h, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_no, n_out, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_po, psi_offsets, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    const double* g_psi = psi;
    const double* g_E = dL_dE;
    double* g_V = dL_dV;
    if (!dev) {
        auto* a = (double*)ctx->get("adjx_psi", sizeof(double) * std::max<int64_t>(psi_total, 1), &ce);
        auto* b = (double*)ctx->get("adjx_gE", sizeof(double) * (size_t)n * cap, &ce);
        auto* c = (double*)ctx->get("adjx_gV", sizeof(double) * std::max<int64_t>(total, 1), &ce);
        if (!a || !b || !c) return fail(EPSCU_ERR_NOMEM, "device arena (adjoint)");
        EPSCU_CU(cudaMemcpyAsync(a, psi, sizeof(double) * psi_total, cudaMemcpyHostToDevice, s));
        EPSCU_CU(cudaMemcpyAsync(b, dL_dE, sizeof(double) * (size_t)n * cap, cudaMemcpyHostToDevice, s));
        EPSCU_CU(cudaMemsetAsync(c, 0, sizeof(double) * total, s));
        g_psi = a;
        g_E = b;
        g_V = c;
    }
    launch_adjoint_explicit(n, cap, max_N, d_off, d_N, d_h, d_no, d_po, g_psi, g_E, g_V, s);
    EPSCU_CU(cudaGetLastError());
    if (!dev) EPSCU_CU(cudaMemcpyAsync(dL_dV, g_V, sizeof(double) * total, cudaMemcpyDeviceToHost, s));
    EPSCU_CU(cudaEventRecord(ctx->ev_out, s));
    EPSCU_CU(cudaStreamWaitEvent(caller, ctx->ev_out, 0));
    EPSCU_CU(cudaStreamSynchronize(s));
    return EPSCU_OK;
}

extern "C" epscu_status epscu_tabulate(epscu_ctx* ctx, int32_t n, const int32_t* kind, const double* params,
                                       const int64_t* offsets, const int32_t* N, const double* r_min,
                                       const double* r_max, int32_t n_knots, double* V, const epscu_opts* opts_in) {
    if (!ctx || n <= 0 || !kind || !params || !offsets || !N || !r_min || !r_max || !V)
        return fail(EPSCU_ERR_INVALID, "bad arguments");
    if (n_knots < 4) n_knots = 1024;
    epscu_opts opts{};
    if (opts_in) opts = *opts_in;
    std::lock_guard<std::mutex> guard(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    const cudaStream_t caller = caller_stream(opts);
    EPSCU_CU(cudaEventRecord(ctx->ev_in, caller));
    EPSCU_CU(cudaStreamWaitEvent(s, ctx->ev_in, 0));
    const bool dev = (opts.flags & EPSCU_MEM_DEVICE) != 0;
    int64_t total = 0;
    // host copies of the per-potential arrays (always host-side per the ABI)
    for (int p = 0; p < n; ++p) {
        if (N[p] < 2) return fail(EPSCU_ERR_INVALID, "grid with fewer than 2 points");
        total = std::max<int64_t>(total, offsets[p] + N[p]);
    }
    cudaError_t ce = cudaSuccess;
    auto* d_kind = (int32_t*)ctx->get("tab_kind", sizeof(int32_t) * n, &ce);
    auto* d_par = (double*)ctx->get("tab_par", sizeof(double) * 12 * n, &ce);
    auto* d_off = (int64_t*)ctx->get("tab_off", sizeof(int64_t) * n, &ce);
    auto* d_N = (int32_t*)ctx->get("tab_N", sizeof(int32_t) * n, &ce);
    auto* d_r0 = (double*)ctx->get("tab_r0", sizeof(double) * n, &ce);
    auto* d_r1 = (double*)ctx->get("tab_r1", sizeof(double) * n, &ce);
    auto* d_scr = (double*)ctx->get("tab_scratch", sizeof(double) * 3 * (size_t)n_knots * n, &ce);
    if (!d_kind || !d_par || !d_off || !d_N || !d_r0 || !d_r1 || !d_scr) return fail(EPSCU_ERR_NOMEM, "device arena");
    EPSCU_CU(cudaMemcpyAsync(d_kind, kind, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_par, params, sizeof(double) * 12 * n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_off, offsets, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_N, N, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_r0, r_min, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_r1, r_max, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    double* out = V;
    if (!dev) {
        out = (double*)ctx->get("tab_V", sizeof(double) * total, &ce);
        if (!out) return fail(EPSCU_ERR_NOMEM, "device arena (V)");
    }
    launch_tabulate(n, d_kind, d_par, d_off, d_N, d_r0, d_r1, n_knots, d_scr, out, s);
    EPSCU_CU(cudaGetLastError());
    if (!dev) EPSCU_CU(cudaMemcpyAsync(V, out, sizeof(double) * total, cudaMemcpyDeviceToHost, s));
    EPSCU_CU(cudaEventRecord(ctx->ev_out, s));
    EPSCU_CU(cudaStreamWaitEvent(caller, ctx->ev_out, 0));
    EPSCU_CU(cudaStreamSynchronize(s));
    return EPSCU_OK;
}

extern "C" epscu_status epscu_tabulate_adjoint(epscu_ctx* ctx, int32_t n, const int32_t* kind, const double* params,
                                               const int64_t* offsets, const int32_t* N, const double* r_min,
                                               const double* r_max, int32_t n_knots, const double* dL_dV,
                                               double* dL_dparams, const epscu_opts* opts_in) {
    if (!ctx || n <= 0 || !kind || !params || !offsets || !N || !r_min || !r_max || !dL_dV || !dL_dparams)
        return fail(EPSCU_ERR_INVALID, "bad arguments");
    if (n_knots < 4) n_knots = 1024;
    epscu_opts opts{};
    if (opts_in) opts = *opts_in;
    std::lock_guard<std::mutex> guard(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    const cudaStream_t caller = caller_stream(opts);
    EPSCU_CU(cudaEventRecord(ctx->ev_in, caller));
    EPSCU_CU(cudaStreamWaitEvent(s, ctx->ev_in, 0));
    const bool dev = (opts.flags & EPSCU_MEM_DEVICE) != 0;
    int64_t total = 0;
    for (int p = 0; p < n; ++p) {
        if (N[p] < 2) return fail(EPSCU_ERR_INVALID, "grid with fewer than 2 points");
        if (kind[p] < EPSCU_KIND_MORSE || kind[p] > EPSCU_KIND_SPLINE) return fail(EPSCU_ERR_INVALID, "unknown kind");
        total = std::max<int64_t>(total, offsets[p] + N[p]);
    }
    cudaError_t ce = cudaSuccess;
    auto* d_kind = (int32_t*)ctx->get("tab_kind", sizeof(int32_t) * n, &ce);
    auto* d_off = (int64_t*)ctx->get("tab_off", sizeof(int64_t) * n, &ce);
    auto* d_N = (int32_t*)ctx->get("tab_N", sizeof(int32_t) * n, &ce);
    auto* d_r0 = (double*)ctx->get("tab_r0", sizeof(double) * n, &ce);
    auto* d_r1 = (double*)ctx->get("tab_r1", sizeof(double) * n, &ce);
    auto* d_scr = (double*)ctx->get("tabadj_scratch", sizeof(double) * 6 * (size_t)n_knots * n, &ce);
    if (!d_kind || !d_off || !d_N || !d_r0 || !d_r1 || !d_scr) return fail(EPSCU_ERR_NOMEM, "device arena");
    EPSCU_CU(cudaMemcpyAsync(d_kind, kind, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_off, offsets, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_N, N, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_r0, r_min, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    EPSCU_CU(cudaMemcpyAsync(d_r1, r_max, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    const double* d_par = params;
    const double* d_gV = dL_dV;
    double* d_gP = dL_dparams;
    if (!dev) {
        auto* a = (double*)ctx->get("tabadj_par", sizeof(double) * 12 * n, &ce);
        auto* b = (double*)ctx->get("tabadj_gV", sizeof(double) * total, &ce);
        auto* c = (double*)ctx->get("tabadj_gP", sizeof(double) * 12 * n, &ce);
        if (!a || !b || !c) return fail(EPSCU_ERR_NOMEM, "device arena");
        EPSCU_CU(cudaMemcpyAsync(a, params, sizeof(double) * 12 * n, cudaMemcpyHostToDevice, s));
        EPSCU_CU(cudaMemcpyAsync(b, dL_dV, sizeof(double) * total, cudaMemcpyHostToDevice, s));
        d_par = a;
        d_gV = b;
        d_gP = c;
    }
    launch_tabulate_adjoint(n, d_kind, d_par, d_off, d_N, d_r0, d_r1, n_knots, d_scr, d_gV, d_gP, s);
    EPSCU_CU(cudaGetLastError());
    if (!dev) EPSCU_CU(cudaMemcpyAsync(dL_dparams, d_gP, sizeof(double) * 12 * n, cudaMemcpyDeviceToHost, s));
    EPSCU_CU(cudaEventRecord(ctx->ev_out, s));
    EPSCU_CU(cudaStreamWaitEvent(caller, ctx->ev_out, 0));
    EPSCU_CU(cudaStreamSynchronize(s));
    return EPSCU_OK;
}
