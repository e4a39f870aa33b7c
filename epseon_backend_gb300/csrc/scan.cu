// scan.cu -- trial-energy scan: Sturm counts at the n_trial trial energies
// of every potential.
//
//  scan64 : the plain method.  One thread per trial energy, FP64 projective
//           Numerov outward to the twist index and inward to it, arithmetic
//           identical to the oracle's eo_count (bit-exact counts).
//  scan32 : the fast method.  Persistent CTAs pull (potential, energy block)
//           work items from a device queue, ordered longest grid first.  Each
//           potential's W = a V (a float pair per point) is staged into
//           shared memory tile by tile with 1-D bulk TMA copies
//           (cp.async.bulk + mbarrier, STAGES deep), converted once per tile
//           to one float per point relative to the item's reference energy,
//           and read as warp-wide broadcasts.  Each thread carries one trial
//           energy through the FP32 difference-form recurrence
//             D' = D + T (D - 12 A),  A' = A + (T A + D')
//           (A ~ u_i, D ~ u_i - u_{i-1}; Blatt 1967) with T = aE - W rounded
//           once relative to |T| and to the energy offset inside the item, so
//           the count is reliable to |E - E_v| of a few 1e-9 Hartree.  The
//           twist pivot is evaluated in FP64 in the cancellation-free form
//           -12 T_k A C + f_k (D_o C + D_i A).  With a stride it counts only
//           at every stride-th trial energy (the bisection scan's coarse grid).
//  bisect_plan + count_list : the bisection rounds (below).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "launch.h"

namespace epscu {

namespace {

constexpr int kScan64Threads = 128;

__global__ void __launch_bounds__(kScan64Threads) scan64_kernel(DevBatch b, int ipp) {
    const int item = blockIdx.x;
    const int p = b.order[item / ipp];
    const int blk = item % ipp;
    const PotMeta m = b.meta[p];
    const int j = blk * kScan64Threads + threadIdx.x;
    if (j >= b.n_trial) return;
    int32_t c = 0;
    if (!(m.status & EPSCU_STATUS_BAD)) c = count64(m, b.W64 + m.off, trial_energy(m, j), m.k_scan);
    b.counts[(int64_t)p * b.n_trial + j] = c;
}

// ------------------------------------------------------------------ TMA plumbing

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// non-blocking test of a phase
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on a phase of an mbarrier; false when the limit ran out.
// polls == 0: up to kWaitPolls try_waits, each of which may suspend the
// thread for a hardware-defined time until the phase completes; polls > 0
// (epscu_opts.wait_polls): that many non-blocking tests, a bound measured in
// instructions rather than in copy latency.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int polls = 0) {
    if (polls > 0) {
        for (int it = 0; it < polls; ++it)
            if (mbar_test_wait(bar, parity)) return true;
        return false;
    }
    for (int it = 0; it < kWaitPolls; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Tile t of the item's sequence: outward tiles ascending over [j0, k-1], then
// inward tiles descending over [k+1, j1] ([j0, j1] = the item's window).
struct TileSeq {
    int out_first, n_out, in_first, n_in;  // tile indices
    __device__ int tile(int t) const { return t < n_out ? out_first + t : in_first - (t - n_out); }
    __device__ int size() const { return n_out + n_in; }
};

__device__ __forceinline__ TileSeq make_seq(int j0, int j1, int k, int tile) {
    TileSeq s;
    if (k > j0) {
        s.out_first = j0 / tile;
        s.n_out = (k - 1) / tile - s.out_first + 1;
    } else {
        s.out_first = 0;
        s.n_out = 0;
    }
    if (k < j1) {
        s.in_first = j1 / tile;
        s.n_in = s.in_first - (k + 1) / tile + 1;
    } else {
        s.in_first = 0;
        s.n_in = 0;
    }
    return s;
}

__device__ __forceinline__ void renorm_f(float& A, float& D) {
    const float m = fmaxf(fabsf(A), fabsf(D));
    const int e = ((__float_as_int(m) >> 23) & 0xff) - 126;
    if (m > 0.0f && e > -100 && e < 100) {
        const float s = __int_as_float((127 - e) << 23);
        A *= s;
        D *= s;
    }
}

// Each landed tile of W = w.x + w.y (a float pair per point) is converted
// once into c_i = (H - w.x) - w.y, one float per point, for the item's
// reference energy H = a E_mid, and a thread's energy enters as l = a E - H, so
//     T = a E - W = c_i + l
// costs one FADD per point.  Rounding: near the turning point of H, H and w.x
// agree to a factor 2 and H - w.x is exact; c_i then carries one rounding of
// |H - W|, and T one of |T|.  At a thread's own turning point (T ~ 0,
// |H - W| ~ |l|) the error is ulp(l)/2 with l at most THREADS trial spacings,
// the same as keeping W's low part through a second FADD; elsewhere it is at
// most twice that scheme's ulp(T)/2.

// One FP32 difference-form step at a point with converted tile entry c.
__device__ __forceinline__ void step32(float l, float c, float& A, float& D, int& nodes) {
    const float T = c + l;
    const float X = fmaf(-12.0f, A, D);
    D = fmaf(T, X, D);
    const float inc = fmaf(T, A, D);
    const float An = A + inc;
    nodes += (__float_as_uint(An) ^ __float_as_uint(A)) >> 31;
    A = An;
}

// Step with the sign of A shifted into a bit history (one funnel shift per
// step; the sign changes are popcounted once per 16-step chunk).
__device__ __forceinline__ void step32b(float l, float c, float& A, float& D, uint32_t& bits) {
    const float T = c + l;
    const float X = fmaf(-12.0f, A, D);
    D = fmaf(T, X, D);
    A = A + fmaf(T, A, D);
    bits = __funnelshift_l(__float_as_uint(A), bits, 1);
}

__device__ __forceinline__ void flush_bits(uint32_t& bits, int& nodes) {
    nodes += __popc((bits ^ (bits >> 1)) & 0xffffu);
    bits &= 1u;
}

// 16 ascending points starting at a 16-aligned offset of the tile
__device__ __forceinline__ void chunk16_up(const float* __restrict__ c, float l, float& A, float& D,
                                           uint32_t& bits, int& nodes) {
    const float4* q4 = reinterpret_cast<const float4*>(c);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const float4 q = q4[u];
        step32b(l, q.x, A, D, bits);
        step32b(l, q.y, A, D, bits);
        step32b(l, q.z, A, D, bits);
        step32b(l, q.w, A, D, bits);
    }
    flush_bits(bits, nodes);
    renorm_f(A, D);
}

// the same 16 points descending
__device__ __forceinline__ void chunk16_down(const float* __restrict__ c, float l, float& A, float& D,
                                             uint32_t& bits, int& nodes) {
    const float4* q4 = reinterpret_cast<const float4*>(c);
#pragma unroll
    for (int u = 3; u >= 0; --u) {
        const float4 q = q4[u];
        step32b(l, q.w, A, D, bits);
        step32b(l, q.z, A, D, bits);
        step32b(l, q.y, A, D, bits);
        step32b(l, q.x, A, D, bits);
    }
    flush_bits(bits, nodes);
    renorm_f(A, D);
}

// points a0..a1 (a0 <= a1) of tile tb (first point T0), ascending
__device__ __forceinline__ void run_up(const float* __restrict__ tb, int T0, int a0, int a1, float l, float& A,
                                       float& D, int& nodes) {
    int i = a0;
    for (; i <= a1 && (i & 15); ++i) step32(l, tb[i - T0], A, D, nodes);
    renorm_f(A, D);
    uint32_t bits = __float_as_uint(A) >> 31;
    for (; i + 15 <= a1; i += 16) chunk16_up(tb + (i - T0), l, A, D, bits, nodes);
    for (; i <= a1; ++i) step32(l, tb[i - T0], A, D, nodes);
}

// points a0..a1 (a0 >= a1) of tile tb, descending
__device__ __forceinline__ void run_down(const float* __restrict__ tb, int T0, int a0, int a1, float l, float& A,
                                         float& D, int& nodes) {
    int i = a0;
    for (; i >= a1 && ((i & 15) != 15); --i) step32(l, tb[i - T0], A, D, nodes);
    renorm_f(A, D);
    uint32_t bits = __float_as_uint(A) >> 31;
    for (; i - 15 >= a1; i -= 16) chunk16_down(tb + (i - 15 - T0), l, A, D, bits, nodes);
    for (; i >= a1; --i) step32(l, tb[i - T0], A, D, nodes);
}

template <int THREADS, int TILE, int STAGES>
__global__ void __launch_bounds__(THREADS) scan32_kernel(DevBatch b, int ipp, int n_items, int stride) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);               // STAGES TMA tiles of (w.x, w.y)
    float* conv = reinterpret_cast<float*>(buf + (size_t)STAGES * TILE);  // the converted tile
    __shared__ __align__(8) uint64_t full[STAGES];
    __shared__ __align__(8) uint64_t never;  // the failure self-test's barrier: nothing arrives
    __shared__ int s_item;
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
        mbar_init(&never, 1);
        fence_barrier_init();
        s_abort = 0;
    }
    __syncthreads();

    const int wait_polls = b.wait_polls > 0 ? b.wait_polls : 0;
    uint32_t g_tile = 0;   // tiles consumed by this CTA so far (phase bookkeeping)
    uint32_t g_issue = 0;  // tiles issued by this CTA so far (thread 0)
    for (;;) {
        __syncthreads();  // everyone has read the previous s_item
        if (tid == 0) {
            int it = atomicAdd(&b.hdr->queue_scan, 1);
            if (b.cancel && *b.cancel) it = n_items;
            s_item = it;
        }
        __syncthreads();
        const int item = s_item;
        if (item >= n_items || s_abort) break;
        const int p = b.order[item / ipp];
        // energy blocks highest first: windows (and so the work) grow with
        // the energy, so the longest items of a potential start first
        const int blk = ipp - 1 - item % ipp;
        // trial energies stride - 1, 2 stride - 1, ... (and the last one):
        // every one for stride 1, the bisection scan's coarse grid otherwise
        const int last = b.n_trial - 1;
        const int n_sel = (b.n_trial + stride - 1) / stride;
        auto sel = [&](int q) { return min(q * stride + stride - 1, last); };
        const bool valid = blk * THREADS + tid < n_sel;
        const int j = sel(blk * THREADS + tid);
        const PotMeta m = b.meta[p];
        if (m.status & EPSCU_STATUS_BAD) {
            if (valid) b.counts[(int64_t)p * b.n_trial + j] = 0;
            continue;  // uniform across the CTA
        }
        // the item's window: union of the decay windows of its energy blocks
        // (they contain the twist index k_scan = argmin V), else [i0, i1]
        int j0 = m.i0, j1 = m.i1;
        if (b.scan_win) {
            const int nb = (b.n_trial + kScanWinBlock - 1) / kScanWinBlock;
            const int q0 = sel(blk * THREADS) / kScanWinBlock;
            const int q1 = min(nb - 1, sel(min(blk * THREADS + THREADS, n_sel) - 1) / kScanWinBlock);
            j0 = m.i1;
            j1 = m.i0;
            for (int q = q0; q <= q1; ++q) {
                const int2 wq = b.scan_win[(int64_t)p * nb + q];
                j0 = min(j0, wq.x);
                j1 = max(j1, wq.y);
            }
            j0 = min(j0, m.k_scan);
            j1 = max(j1, m.k_scan);
        }
        const TileSeq seq = make_seq(j0, j1, m.k_scan, TILE);
        if (tid == 0) {
            const int n_e = min(THREADS, n_sel - blk * THREADS);
            atomicAdd(&b.hdr->scan_updates, (unsigned long long)n_e * (unsigned long long)(j1 - j0));
        }
        const int L = seq.size();
        const float2* src = b.Wf2 + m.offf;

        // prologue: up to STAGES tiles in flight
        if (tid == 0) {
            fence_proxy_async();
            for (int t = 0; t < STAGES && t < L; ++t) {
                const int st = (g_tile + t) % STAGES;
                mbar_expect_tx(&full[st], TILE * sizeof(float2));
                bulk_load(buf + st * TILE, src + (int64_t)seq.tile(t) * TILE, TILE * sizeof(float2), &full[st]);
                ++g_issue;
            }
        }

        if (b.wait_polls < 0) {
            // self-test of the failure path (epscu_opts.wait_polls < 0): a wait
            // that runs out, on a barrier no copy completes, taken exactly as
            // a lost copy is (abort, drain the copies in flight, error word)
            if (!mbar_wait_bounded(&never, 0, -b.wait_polls)) {
                atomicExch(&s_abort, 1);
                atomicCAS(&b.hdr->error, 0, EPSCU_ERR_TIMEOUT);
            }
        }

        const double E = trial_energy(m, j);
        const double aE = __dmul_rn(m.a, E);
        // the item's reference energy (middle of its block) and this thread's
        // offset (at most THREADS / 2 strides of trial spacings)
        const float H = __double2float_rn(__dmul_rn(m.a, trial_energy(m, sel(blk * THREADS + THREADS / 2))));
        const float l = __double2float_rn(aE - (double)H);
        const int k = m.k_scan;
        float A = 1.0f, D = 1.0f;  // u_{j0} = 1, u_{j0-1} = 0
        float Ao = 1.0f, Do = 1.0f;
        int nodes = 0;
        bool inward = false;

        for (int t = 0; t < L; ++t) {
            const int st = (g_tile + t) % STAGES;
            const uint32_t par = ((g_tile + t) / STAGES) & 1u;
            const bool landed = mbar_wait_bounded(&full[st], par, wait_polls);
            if (!landed) {
                atomicExch(&s_abort, 1);
                atomicCAS(&b.hdr->error, 0, EPSCU_ERR_TIMEOUT);
            }
            const float2* tb = buf + st * TILE;
            // convert the tile: c_i = (H - w.x) - w.y
            if (landed)
                for (int x = tid; x < TILE; x += THREADS) {
                    const float2 v = tb[x];
                    conv[x] = __fsub_rn(__fsub_rn(H, v.x), v.y);
                }
            __syncthreads();  // conv is complete, stage st is free
            if (s_abort) {
                g_tile += t;  // tiles t.. were issued but not consumed
                break;
            }
            // refill stage st while the tile is marched
            if (tid == 0 && t + STAGES < L) {
                fence_proxy_async();
                mbar_expect_tx(&full[st], TILE * sizeof(float2));
                bulk_load(buf + st * TILE, src + (int64_t)seq.tile(t + STAGES) * TILE, TILE * sizeof(float2),
                          &full[st]);
                ++g_issue;
            }
            const int T0 = seq.tile(t) * TILE;
            if (t < seq.n_out) {
                const int a0 = max(j0, T0), a1 = min(k - 1, T0 + TILE - 1);
                run_up(conv, T0, a0, a1, l, A, D, nodes);
            } else {
                if (!inward) {
                    inward = true;
                    Ao = A;
                    Do = D;
                    A = 1.0f;  // v_{j1} = 1, v_{j1+1} = 0
                    D = 1.0f;
                }
                const int a0 = min(j1, T0 + TILE - 1), a1 = max(k + 1, T0);
                run_down(conv, T0, a0, a1, l, A, D, nodes);
            }
            __syncthreads();  // every thread is done with conv
        }
        if (s_abort) break;
        g_tile += L;
        if (!inward) {  // no inward tiles: k == j1
            Ao = A;
            Do = D;
            A = 1.0f;
            D = 1.0f;
        }
        // twist pivot sign in FP64: -12 T_k u_k v_k + f_k (D_o v_k + D_i u_k)
        const double Tk = aE - b.W64[m.off + k];
        const double fk = 1.0 + Tk;
        const double uA = (double)Ao, vC = (double)A;
        const double AC = uA * vC;
        const double num = -12.0 * Tk * AC + fk * ((double)Do * vC + (double)D * uA);
        nodes += (num < 0.0) != (AC < 0.0);
        if (valid) {
            b.counts[(int64_t)p * b.n_trial + j] = nodes;
            if (b.gam) b.gam[(int64_t)p * b.n_trial + j] = (float)(num / AC);
        }
    }
    __syncthreads();
    if (s_abort && tid == 0) {
        // drain: wait (bounded, always with the default limit so that no copy
        // is still landing in this CTA's shared memory when it exits) for the
        // copies issued but never consumed
        for (uint32_t q = g_tile; q < g_issue; ++q) (void)mbar_wait_bounded(&full[q % STAGES], (q / STAGES) & 1u);
    }
}

// ------------------------------------------------------------ bisection scan
// The levels' brackets need the count only where it changes: the counts at
// every kBisectCoarse-th trial energy (and the last), then counts inside the
// cells whose end counts differ.  A cell with two or more levels is cut to
// single trial spacings (the full scan's brackets there: the count is
// monotone in the energy); a cell with one level into kBisectSingle parts,
// whose bracket isolates the level.  counts[] holds -1 where no count was
// taken.

// The trial indices of the next round (W = 0: the coarse boundaries; else
// the split - 1 interior points that cut each cell of width W whose end counts
// differ into `split` equal cells, or kBisectSingle - 1 points for a coarse
// cell with one level), and the round's work items: the potential's list in
// chunks of kCountEnergies, so that the count kernel runs every chunk of
// every potential side by side.
// One CTA per potential, longest grids first (their items are listed first).
constexpr int kCountThreads = 128;
constexpr int kCountEnergies = kCountThreads / 2;

// Exclusive prefix sum of v over the CTA (blockDim.x a multiple of 32, at
// most 1024 threads); *total gets the sum.  Every thread must call it.
__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    __shared__ int s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int t = lane < nw ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) s_warp[lane] = t;  // inclusive over the warps
    }
    __syncthreads();
    const int before = (warp > 0 ? s_warp[warp - 1] : 0) + x - v;
    *total = s_warp[nw - 1];
    __syncthreads();  // s_warp is reused by the next call
    return before;
}

__global__ void __launch_bounds__(256) bisect_plan_kernel(DevBatch b, int W, int split) {
    __shared__ int s_n;
    const int p = b.order[blockIdx.x];
    const PotMeta m = b.meta[p];
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    int32_t* list = b.bis_list + (int64_t)p * b.n_trial;
    const int32_t* c = b.counts + (int64_t)p * b.n_trial;
    const int last = b.n_trial - 1;
    // the list is in ascending trial order, written at prefix-sum offsets: a
    // chunk of the count round (and so the window its energies march) is the
    // same from run to run, and with it the matching function stored beside
    // each count (atomic list positions made the refinement's first energies,
    // and the final energies' last bits, vary between runs)
    if (!(m.status & EPSCU_STATUS_BAD)) {
        if (W == 0) {
            const int K = (b.n_trial + kBisectCoarse - 1) / kBisectCoarse;
            for (int k = 1 + threadIdx.x; k <= K; k += blockDim.x) list[k - 1] = min(k * kBisectCoarse - 1, last);
            if (threadIdx.x == 0) s_n = K;
        } else {
            const int ncell = (b.n_trial + W - 1) / W;
            int base = 0;
            for (int t0 = 0; t0 < ncell; t0 += blockDim.x) {
                const int t = t0 + threadIdx.x;
                int a = 0, parts = 0, n_pts = 0;
                if (t < ncell) {
                    a = t * W - 1;  // cell (a, a + W], count(-1) = 0
                    const int ca = a < 0 ? 0 : c[a];
                    const int cb = c[min(a + W, last)];
                    // a coarse cell with one level is cut into kBisectSingle parts
                    parts = (cb - ca == 1 && W == kBisectCoarse) ? min(kBisectSingle, split) : split;
                    if (ca >= 0 && cb > ca)
                        for (int q = 1; q < parts; ++q) n_pts += (a + q * (W / parts) < last) ? 1 : 0;
                }
                int total = 0;
                int at = base + block_exclusive_scan(n_pts, &total);
                for (int q = 1; q < parts && n_pts > 0; ++q) {
                    const int pt = a + q * (W / parts);
                    if (pt < last) list[at++] = pt;
                }
                base += total;
            }
            if (threadIdx.x == 0) s_n = base;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        b.bis_n[p] = s_n;
        const int nch = (s_n + kCountEnergies - 1) / kCountEnergies;
        if (nch > 0) {
            const int base = atomicAdd(&b.hdr->bis_items_n, nch);
            for (int c = 0; c < nch && base + c < b.max_bis_items; ++c)
                b.bis_items[base + c] = make_int2(p, c * kCountEnergies);
        }
    }
}

// Counts at the listed trial energies: persistent CTAs take the round's
// (potential, chunk of kCountEnergies entries) items from a device queue, so
// a round lasts about one serial march of its longest window however many
// levels a potential has.  Each energy is carried through the FP32
// difference form with T = (aE_hi - W_hi) + (aE_lo - W_lo) (three FADDs: the
// energies of a round spread over the whole spectrum, so no shared reference
// energy), on tiles of the window of the chunk's highest energy staged in
// shared memory.
constexpr int kCountTile = 2048;

// the three-FADD step on a raw (w.x, w.y) tile: per point, with the node
// count; and with the sign history (16-step chunks, popcounted)
__device__ __forceinline__ void step32t(float aEh, float aEl, float2 w, float& A, float& D, int& nodes) {
    const float T = (aEh - w.x) + (aEl - w.y);
    const float X = fmaf(-12.0f, A, D);
    D = fmaf(T, X, D);
    const float An = A + fmaf(T, A, D);
    nodes += (__float_as_uint(An) ^ __float_as_uint(A)) >> 31;
    A = An;
}

__device__ __forceinline__ void step32tb(float aEh, float aEl, float wx, float wy, float& A, float& D, uint32_t& bits) {
    const float T = (aEh - wx) + (aEl - wy);
    const float X = fmaf(-12.0f, A, D);
    D = fmaf(T, X, D);
    A = A + fmaf(T, A, D);
    bits = __funnelshift_l(__float_as_uint(A), bits, 1);
}

// points a0..a1 ascending (a0 <= a1) of a raw tile tb whose first point is T0
__device__ __forceinline__ void run_up_raw(const float2* __restrict__ tb, int T0, int a0, int a1, float aEh, float aEl,
                                           float& A, float& D, int& nodes) {
    int i = a0;
    for (; i <= a1 && (i & 15); ++i) step32t(aEh, aEl, tb[i - T0], A, D, nodes);
    renorm_f(A, D);
    uint32_t bits = __float_as_uint(A) >> 31;
    for (; i + 15 <= a1; i += 16) {
        const float4* q4 = reinterpret_cast<const float4*>(tb + (i - T0));
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const float4 q = q4[u];
            step32tb(aEh, aEl, q.x, q.y, A, D, bits);
            step32tb(aEh, aEl, q.z, q.w, A, D, bits);
        }
        flush_bits(bits, nodes);
        renorm_f(A, D);
    }
    for (; i <= a1; ++i) step32t(aEh, aEl, tb[i - T0], A, D, nodes);
}

// points a0..a1 descending (a0 >= a1)
__device__ __forceinline__ void run_down_raw(const float2* __restrict__ tb, int T0, int a0, int a1, float aEh,
                                             float aEl, float& A, float& D, int& nodes) {
    int i = a0;
    for (; i >= a1 && ((i & 15) != 15); --i) step32t(aEh, aEl, tb[i - T0], A, D, nodes);
    renorm_f(A, D);
    uint32_t bits = __float_as_uint(A) >> 31;
    for (; i - 15 >= a1; i -= 16) {
        const float4* q4 = reinterpret_cast<const float4*>(tb + (i - 15 - T0));
#pragma unroll
        for (int u = 7; u >= 0; --u) {
            const float4 q = q4[u];
            step32tb(aEh, aEl, q.z, q.w, A, D, bits);
            step32tb(aEh, aEl, q.x, q.y, A, D, bits);
        }
        flush_bits(bits, nodes);
        renorm_f(A, D);
    }
    for (; i >= a1; --i) step32t(aEh, aEl, tb[i - T0], A, D, nodes);
}

// Two threads per listed energy: warps 0-1 march the outward side, warps 2-3
// the inward side of the same kCountEnergies energies, on their own tiles,
// so a chunk waits for half of its window's serial march; the inward half
// hands its state to the outward one for the twist pivot.
__global__ void __launch_bounds__(kCountThreads) count_list_kernel(DevBatch b) {
    __shared__ __align__(16) float2 tile_o[kCountTile];
    __shared__ __align__(16) float2 tile_i[kCountTile];
    __shared__ float s_A[kCountEnergies], s_D[kCountEnergies];
    __shared__ int s_nodes[kCountEnergies];
    __shared__ int s_jmax;
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int side = tid / kCountEnergies;  // 0: outward, 1: inward (warp-uniform)
    const int e = tid - side * kCountEnergies;
    const int n_items = min(b.hdr->bis_items_n, b.max_bis_items);
    for (;;) {
        __syncthreads();  // everyone has read the previous item
        if (tid == 0) s_item = atomicAdd(&b.hdr->bis_items_q, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= n_items) break;
        const int2 it = b.bis_items[item];
        const int p = it.x, c0 = it.y;
        const PotMeta m = b.meta[p];
        const int ne = b.bis_n[p];
        if (ne <= 0 || (m.status & EPSCU_STATUS_BAD)) continue;  // uniform over the CTA
        const int32_t* list = b.bis_list + (int64_t)p * b.n_trial;
        const float2* src = b.Wf2 + m.offf;  // padded to whole tiles
        const int k = m.k_scan;
        const int q = c0 + e;
        const int j = q < ne ? list[q] : -1;
        if (tid == 0) s_jmax = -1;
        __syncthreads();
        if (j >= 0) atomicMax(&s_jmax, j);
        __syncthreads();
        const int jmax = s_jmax;
        // the window of the chunk's highest energy holds the others'
        int j0 = m.i0, j1 = m.i1;
        if (b.scan_win) {
            const int nb = (b.n_trial + kScanWinBlock - 1) / kScanWinBlock;
            const int2 wq = b.scan_win[(int64_t)p * nb + jmax / kScanWinBlock];
            j0 = min(wq.x, k);
            j1 = max(wq.y, k);
        }
        if (tid == 0)
            atomicAdd(&b.hdr->scan_updates,
                      (unsigned long long)min(kCountEnergies, ne - c0) * (unsigned long long)(j1 - j0));
        const double aE = __dmul_rn(m.a, trial_energy(m, max(j, 0)));
        const float aEh = __double2float_rn(aE);
        const float aEl = __double2float_rn(aE - (double)aEh);
        // outward: u_{j0} = 1, u_{j0-1} = 0; inward: v_{j1} = 1, v_{j1+1} = 0
        float A = 1.0f, D = 1.0f;
        int nodes = 0;
        const TileSeq seq = make_seq(j0, j1, k, kCountTile);
        const int L = max(seq.n_out, seq.n_in);
        for (int t = 0; t < L; ++t) {
            const int To = t < seq.n_out ? seq.tile(t) * kCountTile : -1;
            const int Ti = t < seq.n_in ? seq.tile(seq.n_out + t) * kCountTile : -1;
            __syncthreads();  // the previous tiles are consumed
            for (int x = tid; x < kCountTile; x += kCountThreads) {
                if (To >= 0) tile_o[x] = src[To + x];
                if (Ti >= 0) tile_i[x] = src[Ti + x];
            }
            __syncthreads();
            if (side == 0) {
                if (To >= 0)
                    run_up_raw(tile_o, To, max(j0, To), min(k - 1, To + kCountTile - 1), aEh, aEl, A, D, nodes);
            } else if (Ti >= 0) {
                run_down_raw(tile_i, Ti, min(j1, Ti + kCountTile - 1), max(k + 1, Ti), aEh, aEl, A, D, nodes);
            }
        }
        if (side == 1) {
            s_A[e] = A;
            s_D[e] = D;
            s_nodes[e] = nodes;
        }
        __syncthreads();
        if (side == 0) {
            // twist pivot sign in FP64: -12 T_k u_k v_k + f_k (D_o v_k + D_i u_k)
            const double Tk = aE - b.W64[m.off + k];
            const double fk = 1.0 + Tk;
            const double uA = (double)A, vC = (double)s_A[e];
            const double AC = uA * vC;
            const double num = -12.0 * Tk * AC + fk * ((double)D * vC + (double)s_D[e] * uA);
            nodes += s_nodes[e] + ((num < 0.0) != (AC < 0.0));
            if (j >= 0) {
                b.counts[(int64_t)p * b.n_trial + j] = nodes;
                if (b.gam) b.gam[(int64_t)p * b.n_trial + j] = (float)(num / AC);
            }
        }
    }
}

// (the count kernel's persistent grid: CTAs per SM)
constexpr int kCountCtasPerSm = 8;

template <int THREADS, int TILE, int STAGES>
void launch_scan32_t(const DevBatch& b, int ctas_per_sm, int sm_count, cudaStream_t s, int stride) {
    const int ipp = ((b.n_trial + stride - 1) / stride + THREADS - 1) / THREADS;
    const int n_items = ipp * b.n;
    const size_t smem = (size_t)TILE * STAGES * sizeof(float2) + (size_t)TILE * sizeof(float);
    auto kern = scan32_kernel<THREADS, TILE, STAGES>;
    if (ctas_per_sm <= 0) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, THREADS, smem);
        ctas_per_sm = occ > 0 ? occ : 1;
    }
    int grid = sm_count * ctas_per_sm;
    if (grid > n_items) grid = n_items;
    if (grid < 1) grid = 1;
    kern<<<grid, THREADS, smem, s>>>(b, ipp, n_items, stride);
}

template <int THREADS, int TILE, int STAGES>
void set_attr_t() {
    cudaFuncSetAttribute(scan32_kernel<THREADS, TILE, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(TILE * STAGES * sizeof(float2) + TILE * sizeof(float)));
}

}  // namespace

void scan32_set_attributes() {
    set_attr_t<128, 1024, 2>();
    set_attr_t<128, 1024, 4>();
    set_attr_t<128, 2048, 2>();
    set_attr_t<128, 2048, 3>();
    set_attr_t<256, 1024, 2>();
    set_attr_t<256, 1024, 4>();
    set_attr_t<256, 2048, 3>();
    set_attr_t<256, 4096, 2>();
    set_attr_t<512, 1024, 4>();
    set_attr_t<512, 2048, 3>();
}

void launch_scan64(const DevBatch& b, cudaStream_t s) {
    const int ipp = (b.n_trial + kScan64Threads - 1) / kScan64Threads;
    scan64_kernel<<<ipp * b.n, kScan64Threads, 0, s>>>(b, ipp);
}

int scan32_max_tile() { return 4096; }

// a round lists fewer than n_trial entries per potential
int64_t bisect_max_items(int n, int n_trial) {
    return (int64_t)n * ((n_trial + kCountEnergies - 1) / kCountEnergies + 1);
}

void launch_bisect_scan(const DevBatch& b, const ScanShape& sh, int sm_count, cudaStream_t s) {
    cudaMemsetAsync(b.counts, 0xff, sizeof(int32_t) * (size_t)b.n * b.n_trial, s);  // -1: no count taken
    // the coarse grid with the throughput scan, then the bisection rounds
    launch_scan32(b, sh, sm_count, s, kBisectCoarse);
    // each round cuts the cells that hold two or more levels into
    // kBisectSplit parts (the last round into what is left), and a cell that
    // holds one level into kBisectSingle parts once: its bracket of
    // kBisectCoarse / kBisectSingle spacings isolates the level already, and
    // the refinement needs about one pass more than from one spacing.  Every
    // round lasts about one march of its longest window (the total work of a
    // round is a fraction of that), so fewer rounds with more counts each are
    // shorter.  Measured on the 2048-potential batch (scan stage / step):
    // cells of 8, three rounds of 2: 6.8 ms (scan); cells of 8, one round of
    // 8: 5.0 / 31.6 ms; one-level cells halved: 3.9 / 30.4 ms; cells of 16
    // (15 counts in a cell with several levels, 3 in a one-level cell):
    // 3.6 / 29.7 ms; cells of 32 (31 and 7): 4.9 / 30.8 ms.  The bracket
    // kernel descends while the midpoints it visits have a count.
    for (int W = kBisectCoarse; W > 1;) {
        const int split = W < kBisectSplit ? W : kBisectSplit;
        cudaMemsetAsync(&b.hdr->bis_items_n, 0, 2 * sizeof(int32_t), s);  // the round's items and queue
        bisect_plan_kernel<<<b.n, 256, 0, s>>>(b, W, split);
        count_list_kernel<<<sm_count * kCountCtasPerSm, kCountThreads, 0, s>>>(b);
        W /= split;
    }
}

void launch_scan32(const DevBatch& b, const ScanShape& sh, int sm_count, cudaStream_t s, int stride) {
#define EPSCU_SCAN32_CASE(TH, TI, ST)                                              \
    if (sh.threads == TH && sh.tile == TI && sh.stages == ST) {                    \
        launch_scan32_t<TH, TI, ST>(b, sh.ctas_per_sm, sm_count, s, stride);       \
        return;                                                                    \
    }
    EPSCU_SCAN32_CASE(128, 1024, 2)
    EPSCU_SCAN32_CASE(128, 1024, 4)
    EPSCU_SCAN32_CASE(128, 2048, 2)
    EPSCU_SCAN32_CASE(128, 2048, 3)
    EPSCU_SCAN32_CASE(256, 1024, 2)
    EPSCU_SCAN32_CASE(256, 1024, 4)
    EPSCU_SCAN32_CASE(256, 2048, 3)
    EPSCU_SCAN32_CASE(256, 4096, 2)
    EPSCU_SCAN32_CASE(512, 1024, 4)
    EPSCU_SCAN32_CASE(512, 2048, 3)
#undef EPSCU_SCAN32_CASE
    launch_scan32_t<256, 2048, 3>(b, sh.ctas_per_sm, sm_count, s, stride);
}

}  // namespace epscu
