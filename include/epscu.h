/*
 * epscu.h -- C ABI of libepseon_cuda, the GB300 (sm_103a) vibrational-level
 * solver behind epseon_backend's device/task interface.
 *
 * The reference binds its gpu device through pybind11 over C++ templates; the
 * algorithm slot that this library fills is
 *     Algorithm<FP>::run(const std::stop_token&, TaskHandle<FP>*)
 *         cpp/gpu/include/epseon/gpu/algorithms/algorithm.hpp:34
 *     VibwaAlgorithm<FP>::run            .../algorithms/vibwa.hpp:605-637
 * and its inputs come from
 *     HardwareConfig          .../task_configurator/hardware_config.hpp:16-18
 *     MorsePotentialConfig    .../task_configurator/potential_source.hpp:103-183
 *     VibwaAlgorithmConfig    .../task_configurator/algorithm_config.hpp:76-199
 * Each entry point below names the reference interface it stands in for.
 *
 * Conventions: plain C types, caller-owned buffers, every call returns an
 * epscu_status (0 = success); epscu_last_error() describes the last failure
 * on the calling thread.  Units are atomic units (Hartree, bohr, electron
 * masses) unless stated otherwise.
 */
#ifndef EPSCU_H
#define EPSCU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EPSCU_ABI_VERSION 2

typedef int32_t epscu_status;
enum {
    EPSCU_OK = 0,
    EPSCU_ERR_INVALID = 1,     /* bad argument (message in epscu_last_error) */
    EPSCU_ERR_CUDA = 2,        /* CUDA runtime error */
    EPSCU_ERR_NOMEM = 3,       /* device allocation failed */
    EPSCU_ERR_CANCELLED = 4,   /* epscu_cancel() was called during the solve */
    EPSCU_ERR_CAPACITY = 5,    /* an output buffer is too small (size reported) */
    EPSCU_ERR_TIMEOUT = 6      /* a bounded device wait ran out */
};

/* per-level status bits (also used by the FP64 oracle) */
enum {
    EPSCU_LEVEL_OK = 0,
    EPSCU_LEVEL_MAXITER = 1,        /* refinement iteration cap reached */
    EPSCU_LEVEL_NONFINITE = 2,      /* NaN/Inf in the potential or the recurrence */
    EPSCU_LEVEL_UNDER_RESOLVED = 4, /* k_max h > 1 on this potential's grid */
    EPSCU_LEVEL_CANCELLED = 8,
    EPSCU_LEVEL_NOT_FOUND = 16,     /* the level could not be bracketed/verified */
    EPSCU_LEVEL_BAD_INPUT = 32
};

/* solver methods */
enum {
    EPSCU_METHOD_PLAIN_FP64 = 0, /* FP64 scan + FP64 bisection (the plain method) */
    EPSCU_METHOD_FAST_FP32C = 1  /* FP32 difference-form scan + FP32 Cooley refinement
                                    + FP64 Cooley polish, persistent work-queue kernels */
};

/* potential kinds for device-side tabulation (epscu_tabulate) */
enum { EPSCU_KIND_MORSE = 0, EPSCU_KIND_LJ = 1, EPSCU_KIND_SPLINE = 2 };

/* flags */
enum {
    EPSCU_MEM_DEVICE = 1,  /* V / params / outputs are device pointers (else host) */
    EPSCU_WANT_PSI = 2,    /* write normalised wavefunctions */
    EPSCU_STAGE_TIMING = 4, /* record per-stage CUDA events (disables graph replay) */
    EPSCU_KEEP_PSI = 8      /* host buffers without a psi buffer: keep the normalised
                               wavefunctions in device memory for epscu_adjoint (no
                               recompute, nothing copied back) */
};

typedef struct epscu_ctx epscu_ctx;

/* A ragged batch of tabulated potentials on uniform grids.  Potential p
 * occupies V[offsets[p] .. offsets[p] + N[p]) with r_i = r_min + i h,
 * h = (r_max - r_min)/(N-1).  Host arrays except V (device when
 * EPSCU_MEM_DEVICE is set).  Stands in for PotentialSource<FP>::
 * get_potential_data() (potential_source.hpp:38) and the per-slot staging
 * buffers of VibwaAlgorithm (vibwa.hpp:153-233). */
typedef struct epscu_batch {
    int32_t n_potentials;
    const double* V;        /* concatenated potentials */
    const int64_t* offsets; /* [n] first element of each potential in V */
    const int32_t* N;       /* [n] grid points */
    const double* r_min;    /* [n] */
    const double* r_max;    /* [n] */
    const double* mu;       /* [n] reduced masses */
    const double* e_cap;    /* [n] top of each energy window */
    int32_t n_trial;        /* trial energies per potential */
    int32_t min_level;      /* first level reported (VibwaAlgorithmConfig min_level) */
    int32_t max_level;      /* last level reported; < 0: every level below e_cap */
} epscu_batch;

/* Allocator callback: returns a device buffer of at least `bytes` bytes (16-byte
 * aligned), or NULL when the caller cannot provide one.  See epscu_opts.psi_alloc. */
typedef void* (*epscu_alloc_fn)(int64_t bytes, void* user);

typedef struct epscu_opts {
    int32_t method;      /* EPSCU_METHOD_* */
    int32_t flags;       /* EPSCU_MEM_DEVICE | EPSCU_WANT_PSI | EPSCU_STAGE_TIMING | EPSCU_KEEP_PSI */
    double tol;          /* bisection width of the plain method (default 1e-12) */
    void* stream;        /* cudaStream_t the inputs are ordered on and the outputs are
                            ordered back to (NULL: the legacy default stream); the work
                            itself runs on the context's stream */
    int32_t tune;        /* 0 = use cached/default launch shape, 1 = autotune */
    int32_t long_window; /* fast method: levels whose window exceeds this many points run
                            their passes one CTA per level (0: chosen from the number of
                            levels, 1024 - 8192) */
    int32_t wait_polls;  /* fast method: bound of each wait of the TMA scan on a staged
                            tile, in non-blocking polls; when it runs out the solve gives up
                            with EPSCU_ERR_TIMEOUT and reports no levels.  0: the default,
                            4194304 polls that may each suspend until the copy lands.  The
                            copies already in flight are still drained with the default
                            bound, so the context stays usable.  < 0: self-test of that
                            failure path: every scan item first waits -wait_polls polls on
                            a barrier that no copy completes, and gives up as above. */
    int32_t max_iter;    /* fast method: cap on the FP32 refinement passes of a level and
                            on its double-float fallback passes (0: 48 and 96); a level
                            that reaches it carries EPSCU_LEVEL_MAXITER */
    int32_t mid_window;  /* fast method: > 0: levels whose window exceeds this many points
                            (and not the long-window threshold) run their double-float passes
                            one warp per level after the lane FP32 refinement; 0 or < 0: off
                            (the default: on the 2048-potential batch it did not shorten
                            the solve) */
    epscu_alloc_fn psi_alloc;  /* EPSCU_MEM_DEVICE with EPSCU_WANT_PSI and result->psi NULL:
                                  the solve reads the wavefunctions' exact size back after
                                  its level set-up and asks psi_alloc for that buffer
                                  (called once, from the calling thread, inside the solve);
                                  result->psi and psi_capacity then name it.  NULL from the
                                  callback: the solve goes on without wavefunctions
                                  (psi_required still reports their size).  Such solves
                                  are launched directly, not from the replayed graph. */
    void* psi_alloc_user;      /* passed to psi_alloc */
} epscu_opts;

/* Caller-owned outputs.  Level slot s of potential p is p*level_capacity + s
 * and holds level min_level + s.  psi (optional) is written compactly: the
 * rows of potential p start at psi_offsets[p] and row s has N[p] points. */
typedef struct epscu_result {
    int32_t level_capacity;  /* slots per potential */
    int32_t* n_total;        /* [n] bound levels below e_cap */
    int32_t* n_out;          /* [n] slots written */
    double* energy;          /* [n*cap] */
    int32_t* nodes;          /* [n*cap] node count of the level's wavefunction */
    int32_t* status;         /* [n*cap] EPSCU_LEVEL_* bits */
    double* err_est;         /* [n*cap] |last FP64 correction| (NULL allowed) */
    double* psi;             /* compact wavefunctions (NULL allowed) */
    int64_t psi_capacity;    /* doubles available at psi */
    int64_t* psi_offsets;    /* [n] host: first element of each potential's rows */
    int64_t psi_required;    /* out: doubles the wavefunctions need */
} epscu_result;

typedef struct epscu_device_info {
    char name[256];
    int32_t ordinal;
    int32_t pci_device_id;
    int32_t pci_bus_id;
    int32_t cc_major, cc_minor;
    int32_t sm_count;
    int64_t total_global_mem;
    int32_t shared_mem_per_block_optin;
    int32_t max_threads_per_block;
    int32_t max_grid_dim[3];
    int32_t max_block_dim[3];
    int32_t l2_cache_size;
    int32_t driver_version;  /* e.g. 13000 */
    int32_t runtime_version;
    uint8_t uuid[16];
} epscu_device_info;

/* Library / device discovery: stands in for ComputeContext::create,
 * getPhysicalDevicesInfo and getVulkanAPIVersion
 * (cpp/gpu/source/epseon/gpu/compute_context.cpp:41-104). */
int32_t epscu_abi_version(void);
epscu_status epscu_device_count(int32_t* count);
epscu_status epscu_get_device_info(int32_t ordinal, epscu_device_info* info);
const char* epscu_last_error(void);

/* Context on one device (stands in for ComputeContext::getDeviceInterface,
 * compute_context.cpp:106-117, plus the logical device VibwaAlgorithm creates,
 * vibwa.hpp:654-674).  Owns a stream, a device arena and the autotune cache. */
epscu_status epscu_create(int32_t device_ordinal, epscu_ctx** ctx);
epscu_status epscu_destroy(epscu_ctx* ctx);

/* Device arena growth granularity in bytes (HardwareConfig
 * allocation_block_size, hardware_config.hpp:18). 0 = 64 MiB. */
epscu_status epscu_set_arena_block(epscu_ctx* ctx, int64_t bytes);

/* Solve every bound level in the window of every potential of the batch
 * (the body of VibwaAlgorithm<FP>::run, vibwa.hpp:605-637, which in the
 * reference allocates its buffers and computes nothing). */
epscu_status epscu_solve(epscu_ctx* ctx, const epscu_batch* batch, epscu_result* result,
                         const epscu_opts* opts);

/* Hellmann-Feynman adjoint of the last solve on this context:
 * dL_dV[offsets[p] + i] = sum_s dL_dE[p*cap + s] * psi_s(r_i)^2 h.
 * Uses the wavefunctions the last solve wrote (EPSCU_WANT_PSI) or kept in
 * device memory (EPSCU_KEEP_PSI), or recomputes them when recompute != 0.  Pointers follow opts->flags
 * (EPSCU_MEM_DEVICE).  No reference counterpart: the reference has no
 * gradients. */
epscu_status epscu_adjoint(epscu_ctx* ctx, const double* dL_dE, double* dL_dV, int32_t recompute,
                           const epscu_opts* opts);

/* Stateless form of the adjoint on explicit wavefunctions (as written by
 * epscu_solve with EPSCU_WANT_PSI):
 *   dL_dV[offsets[p] + i] = h_p sum_{s < n_out[p]} dL_dE[p*cap + s]
 *                           * psi[psi_offsets[p] + s N[p] + i]^2,
 * h_p = (r_max[p] - r_min[p]) / (N[p] - 1).  offsets, N, r_min, r_max, n_out
 * and psi_offsets are host arrays; psi, dL_dE and dL_dV follow opts->flags
 * (EPSCU_MEM_DEVICE).  Any number of solves may be differentiated in any
 * order.  No reference counterpart. */
epscu_status epscu_adjoint_psi(epscu_ctx* ctx, int32_t n, const int64_t* offsets, const int32_t* N,
                               const double* r_min, const double* r_max, const int32_t* n_out,
                               int32_t level_capacity, const double* psi, const int64_t* psi_offsets,
                               const double* dL_dE, double* dL_dV, const epscu_opts* opts);

/* Tabulate parametric potentials on their grids on the device (Morse, shifted
 * Lennard-Jones, Morse + Gaussian bumps through a natural cubic spline on
 * n_knots uniform knots spanning [r_min, r_max]).  params is [n, 12]: Morse
 * (De, a, re) or LJ (eps, sigma) at params[0..2], bumps (amp, width, centre)
 * x 3 at params[3..11], a bump being amp exp(-(r-centre)^2 / (2 width^2)).
 * kind, offsets, N, r_min, r_max are host arrays; params and V follow
 * opts->flags (EPSCU_MEM_DEVICE).  Writes V at the given offsets.  Replaces
 * the MorsePotentialGenerator stub get_potential_data()
 * (potential_source.hpp:223-225). */
epscu_status epscu_tabulate(epscu_ctx* ctx, int32_t n, const int32_t* kind, const double* params,
                            const int64_t* offsets, const int32_t* N, const double* r_min,
                            const double* r_max, int32_t n_knots, double* V, const epscu_opts* opts);

/* The adjoint of epscu_tabulate (same arguments and conventions): from
 * dL_dV (the gradient of a loss with respect to the tabulated values V) it
 * writes dL_dparams [n, 12] in the parameter layout of epscu_tabulate (zero
 * where a kind has no parameter).  Morse and LJ rows take the analytic
 * derivatives summed over the grid; Morse + bump rows go through the
 * transpose of the natural-spline map from knots to grid (one tridiagonal
 * sweep per potential) and then the knot values' derivatives.  One kernel,
 * FP64, deterministic.  kind, offsets, N, r_min, r_max are host arrays;
 * params, dL_dV and dL_dparams follow opts->flags (EPSCU_MEM_DEVICE).  No
 * reference counterpart: the reference has no gradients (the forward is the
 * MorsePotentialGenerator stub, potential_source.hpp:223-225). */
epscu_status epscu_tabulate_adjoint(epscu_ctx* ctx, int32_t n, const int32_t* kind, const double* params,
                                    const int64_t* offsets, const int32_t* N, const double* r_min,
                                    const double* r_max, int32_t n_knots, const double* dL_dV, double* dL_dparams,
                                    const epscu_opts* opts);

/* Cooperative cancellation (TaskHandle::cancel,
 * cpp/gpu/include/epseon/gpu/task_handle.hpp:136-144).  Sets a host-mapped
 * flag that the persistent kernels poll between work items.  The request
 * stops the solve running on ctx or, when none is running, the next solve
 * to start; the solve it stops consumes it (returns EPSCU_ERR_CANCELLED and
 * clears the flag).  A solve stopped before its level set-up reports no
 * levels; levels set up before the request carry EPSCU_LEVEL_CANCELLED. */
epscu_status epscu_cancel(epscu_ctx* ctx);

/* Withdraws a cancel request that no solve has consumed (the reference's
 * request_stop is per task, task_handle.hpp:136-144; a context shared by
 * several tasks needs this so that a request which arrived after its task's
 * last solve does not stop another task's solve). */
epscu_status epscu_cancel_clear(epscu_ctx* ctx);

/* Timing of the last solve: per-stage milliseconds (CUDA events on the solve
 * stream) and the counters the roofline uses.  Stages: prepare (set-up and,
 * for the fast method, the scan's decay windows), scan (the scan kernel
 * alone), refine32 (fast: level windows, FP32 refinement and the long-window
 * Newton), polish (Newton, fallback, norm and twist passes; plain: bisection,
 * norm, twist), write (psi write-back). */
typedef struct epscu_stats {
    float ms_prepare, ms_scan, ms_refine32, ms_polish64, ms_write, ms_total;
    int64_t scan_point_updates;    /* trial energies x points of the scan (its window for the fast method) */
    int64_t refine_point_updates;  /* FP32 refinement passes x points (fast method) */
    int64_t fp64_point_updates;    /* FP64 passes x points (plain); double-float passes x points (fast) */
    int64_t psi_bytes;             /* wavefunction bytes written */
    int64_t n_levels;              /* levels solved */
    int32_t kernel_launches;       /* kernels launched by the solve */
    int32_t fallbacks;             /* levels that needed the bisection fallback */
    int32_t twist_searches;        /* levels re-matched by the twist-index search */
    int32_t norm_redos;            /* norm passes redone at E + dE (fast method) */
    int64_t refine_max_level_updates; /* largest point-updates of one level's FP32
                                         refinement (fast method; the tail of the
                                         lane kernel) */
    int64_t df_max_level_updates;  /* largest point-updates of one level's double-float
                                      passes on the lane path (fast method) */
    int32_t refine_max_iters;      /* most FP32 refinement passes of one level */
    int32_t reserved;
    /* the long levels' refinement kernel (CTA per level; fast method): its time
       (EPSCU_STAGE_TIMING only) and its point-updates in FP32 and double-float
       passes (algorithmic: one grid point of one pass) */
    float ms_refine_long;
    int32_t reserved2;
    int64_t long_fp32_point_updates;
    int64_t long_df_point_updates;
    /* the psi write-back of the fast method: zero_psi writes zeros outside the
       level windows (its time with EPSCU_STAGE_TIMING only; ms_write is the
       time of scale_psi, which reads the window's stored pairs and writes the
       normalised doubles) */
    float ms_zero_psi;
    int32_t reserved3;
    int64_t psi_zero_points;   /* points zero_psi wrote (8 B each) */
    int64_t psi_window_points; /* window points scale_psi converted (8 B read + 8 B written each) */
} epscu_stats;
epscu_status epscu_last_stats(epscu_ctx* ctx, epscu_stats* stats);

/* FP32 / FP64 FMA throughput of the device measured by a short burst
 * kernel (TFLOP/s, 2 flops per FMA).  Used for the roofline denominators. */
epscu_status epscu_measure_fma_peaks(epscu_ctx* ctx, double* fp32_tflops, double* fp64_tflops);

/* Level counting for one potential that allocates nothing.  Some callers
 * cannot call cudaMalloc (a plugin inside another framework's memory pool or
 * allocation budget, a context where allocation is not permitted); this entry
 * point runs the trial-energy scan of epscu_solve on scratch held in a
 * file-scope __device__ array of the library (about 1.5 MiB per device, kept
 * until the process exits).  No counterpart in the reference.
 *   V      : device pointer, N grid values (Hartree) on [r_min, r_max]
 *   counts : device pointer, n_trial outputs: the number of bound levels below
 *            E_j = min V + (j+1) (e_cap - min V) / n_trial
 *   stream : cudaStream_t the work is queued on (NULL: legacy default stream);
 *            the call returns without synchronising.
 * The counts come from the fast method's FP32 difference-form scan: reliable
 * to about 1e-9 Hartree, so a trial energy within ~1e-9 Eh of a level may be
 * counted on either side of it (epscu_solve's plain FP64 method gives exact
 * counts).  Failures found on the device cannot change the return code of an
 * asynchronous call: the call then sets every one of the n_trial counts to
 * -1 (EPSCU_STATIC_FAILED).  That happens for a non-finite potential, a grid
 * with fewer than three points inside its cut-offs, e_cap <= min V, and a
 * bounded wait of the scan that ran out.
 * Grids longer than 65536 points return EPSCU_ERR_CAPACITY.  The first call
 * on each device looks up the scratch's device address (make it before any
 * stream capture).  All calls share the scratch: calls that overlap on the GPU
 * race and must be serialised by the caller. */
#define EPSCU_STATIC_FAILED (-1)
epscu_status epscu_count_levels_static(const double* V, int32_t N, double r_min, double r_max, double mu,
                                       double e_cap, int32_t n_trial, int32_t* counts, void* stream);

#ifdef __cplusplus
}
#endif
#endif
