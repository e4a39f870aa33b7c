// prepare.cu -- per-potential set-up of the discrete problem, level-slot
// bookkeeping and device-side tabulation of parametric potentials.
//
// The set-up gives the oracle's eo_prepare() results exactly: minimum of V,
// E-independent Dirichlet cut-offs (a (V_i - E_lo) <= 1/2 in FP64), scan
// twist index (first argmin of V), trial spacing and the bisection step count.
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "dfpass.cuh"
#include "launch.h"

namespace epscu {

namespace {

constexpr int kPrepThreads = 256;

template <typename T, typename Op>
__device__ T block_reduce(T v, Op op, T* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    v = threadIdx.x < nw ? sh[threadIdx.x] : sh[0];
    if (warp == 0)
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) sh[0] = v;
    __syncthreads();
    v = sh[0];
    __syncthreads();
    return v;
}

struct MinI {
    __device__ int operator()(int a, int b) const { return min(a, b); }
};
struct MaxI {
    __device__ int operator()(int a, int b) const { return max(a, b); }
};
struct OrI {
    __device__ int operator()(int a, int b) const { return a | b; }
};

// An unsigned integer image of a double that orders like the double (for
// non-NaN values): minima taken on it are exact and need no FP64 instruction.
constexpr unsigned long long kKeyMax = ~0ull;  // above every image (+inf's image is below it)
__device__ __forceinline__ unsigned long long dkey(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}
// the same with the two zeros on one key (they compare equal as doubles)
__device__ __forceinline__ unsigned long long dkey0(double x) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    if ((u << 1) == 0ull) u = 0ull;
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
struct MinU {
    __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return min(a, b); }
};

// (__double2float_rn(w), __double2float_rn(w - hi)) with integer operations
// for 2^-60 <= |w| < 2^101 (the conversions otherwise): hi rounds the 52-bit
// significand to 23 bits to nearest, ties to even; w - hi is the signed
// remainder of the 29 dropped bits times 2^(e-52), exact in a double, so one
// integer-to-float rounding of the remainder and two exact power-of-two
// scalings give the same float as converting w - hi.  No FP64 instruction.
__device__ __forceinline__ float2 split_double_rn(double w) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(w);
    const int e = (int)((u >> 52) & 0x7ffull) - 1023;
    if (e < -60 || e > 100) {
        const float hi = __double2float_rn(w);
        return make_float2(hi, __double2float_rn(__dsub_rn(w, (double)hi)));
    }
    const uint32_t sgn = (uint32_t)(u >> 32) & 0x80000000u;
    const unsigned long long mant = u & 0xfffffffffffffull;
    const uint32_t r = (uint32_t)(mant & 0x1fffffffull);
    uint32_t hb = ((uint32_t)(e + 127) << 23) | (uint32_t)(mant >> 29);
    const uint32_t up = (r > 0x10000000u || (r == 0x10000000u && (hb & 1u))) ? 1u : 0u;
    hb += up;  // a carry out of the significand raises the exponent
    const int rr = (int)r - (up ? 0x20000000 : 0);
    float lo = 0.0f;
    if (rr != 0) {
        lo = __fmul_rn(__fmul_rn(__int2float_rn(rr), 2.220446049250313e-16f), __int_as_float((127 + e) << 23));
        if (sgn) lo = -lo;
    }
    return make_float2(__uint_as_float(sgn | hb), lo);
}

__global__ void __launch_bounds__(kPrepThreads) prepare_kernel(DevBatch b) {
    __shared__ int shi[32];
    __shared__ unsigned long long shk[32];
    __shared__ unsigned long long s_kt;
    const int p = b.order[blockIdx.x];  // longest grids first (the tail is the last CTAs)
    PotMeta m = b.meta[p];
    const double* V = b.V64 + m.off;
    const int N = m.N;
    const int tid = threadIdx.x, nt = blockDim.x;

    // The per-point comparisons run on order-preserving integer images of the
    // doubles (dkey0), exact and on the integer pipes: min V and its finiteness,
    // the cut-off test a (V_i - V_min) <= 1/2 (monotone in V_i, so it holds
    // exactly up to a threshold image found once per potential by bisection
    // on the images with the FP64 test itself) and the first argmin; the only
    // FP64 instruction per point is W = a V.
    unsigned long long kmin = kKeyMax;
    int bad = 0;
    for (int i = tid; i < N; i += nt) {
        const double v = V[i];
        if ((((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ffull) == 0x7ffull) bad = 1;  // inf, NaN
        else kmin = min(kmin, dkey0(v));
    }
    kmin = block_reduce(kmin, MinU(), shk);
    bad = block_reduce(bad, OrI(), shi);
    const double vmin = dkey_inv(kmin);

    const double h = __ddiv_rn(__dsub_rn(m.r_max, m.r_min), (double)(N - 1));
    const double a = __ddiv_rn(__dmul_rn(__dmul_rn(m.mu, h), h), 6.0);
    if (tid == 0) {
        // the largest image whose double passes the cut-off test (the test
        // holds at V_min; the images above +inf are NaNs, which fail it)
        unsigned long long lo = kmin, hi = kKeyMax;
        while (hi - lo > 1ull) {
            const unsigned long long mid = lo + (hi - lo) / 2;
            if (__dmul_rn(a, __dsub_rn(dkey_inv(mid), vmin)) <= 0.5) lo = mid;
            else hi = mid;
        }
        s_kt = lo;
    }
    __syncthreads();
    const unsigned long long kt = s_kt;
    int first = N, last = -1;
    for (int i = tid; i < N; i += nt) {
        if (dkey0(V[i]) <= kt) {
            first = min(first, i);
            last = max(last, i);
        }
    }
    first = block_reduce(first, MinI(), shi);
    last = block_reduce(last, MaxI(), shi);
    const int i0 = first < 1 ? 1 : first;
    const int i1 = last > N - 2 ? N - 2 : last;

    // argmin on [i0, i1], first occurrence
    unsigned long long bk = kKeyMax;
    int bi = N;
    for (int i = i0 + tid; i <= i1; i += nt) {
        const unsigned long long k = dkey0(V[i]);
        if (k < bk) {
            bk = k;
            bi = i;
        }
    }
    const unsigned long long gk = block_reduce(bk, MinU(), shk);
    int cand = (bk == gk) ? bi : N;
    const int k_scan = block_reduce(cand, MinI(), shi);

    // W = a V in FP64 and as an unevaluated (hi, lo) float pair; zero padding
    double* W = b.W64 + m.off;
    float2* Wf = b.Wf2 ? b.Wf2 + m.offf : nullptr;
    for (int i = tid; i < N; i += nt) {
        const double w = __dmul_rn(a, V[i]);
        W[i] = w;
        if (Wf) Wf[i] = split_double_rn(w);
    }

    // Suffix minima of V on [i0, i1] (M), and for the fast method prefix
    // minima (P) and the minima of a V over 32-point blocks clipped to
    // [i0, i1], rounded down to float (the decay-window bounds).  Coalesced
    // warp scans over the absolute 32-point blocks B0..B1: each warp owns a
    // contiguous run of blocks and scans it with shuffles, seeded with the
    // minimum of the runs to its right (suffix) or left (prefix).  Minima are
    // taken on an order-preserving integer image of the doubles (exact, and
    // no FP64 instruction at GB300's 1/64 rate).
    {
        const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
        const int B0 = i0 >> 5, B1 = i1 >> 5, nblk = i1 >= i0 ? B1 - B0 + 1 : 0;
        const int per = (nblk + nw - 1) / nw;
        const int wb0 = B0 + min(warp * per, nblk), wb1 = B0 + min((warp + 1) * per, nblk);  // [wb0, wb1)
        __shared__ unsigned long long s_run[32];
        auto load_key = [&](int B) {
            const int idx = (B << 5) + lane;
            return (idx >= i0 && idx <= i1) ? dkey(V[idx]) : kKeyMax;
        };
        // this warp's run minimum
        unsigned long long rm = kKeyMax;
        for (int B = wb0; B < wb1; ++B) rm = min(rm, load_key(B));
        for (int o = 16; o > 0; o >>= 1) rm = min(rm, __shfl_xor_sync(0xffffffffu, rm, o));
        if (lane == 0) s_run[warp] = rm;
        __syncthreads();
        double* M = b.Msuf + m.off;
        unsigned long long carry = kKeyMax;  // the minimum right of this warp's run
        for (int w = warp + 1; w < nw; ++w) carry = min(carry, s_run[w]);
        float* Bm = b.Mpre ? b.Bmin + m.offf / 32 : nullptr;
        for (int B = wb1 - 1; B >= wb0; --B) {
            unsigned long long k = load_key(B);
            // inclusive suffix minimum over the lanes (lane l: lanes l..31)
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_down_sync(0xffffffffu, k, o);
                if (lane + o < 32) k = min(k, y);
            }
            const unsigned long long blk = __shfl_sync(0xffffffffu, k, 0);  // the block's minimum
            const int idx = (B << 5) + lane;
            if (idx >= i0 && idx <= i1) M[idx] = dkey_inv(min(k, carry));
            if (Bm && lane == 0) Bm[B] = __double2float_rd(__dmul_rn(a, dkey_inv(blk)));
            carry = min(carry, blk);
        }
        if (b.Mpre) {
            double* P = b.Mpre + m.off;
            carry = kKeyMax;  // the minimum left of this warp's run
            for (int w = 0; w < warp; ++w) carry = min(carry, s_run[w]);
            for (int B = wb0; B < wb1; ++B) {
                unsigned long long k = load_key(B);
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long y = __shfl_up_sync(0xffffffffu, k, o);
                    if (lane >= o) k = min(k, y);
                }
                const int idx = (B << 5) + lane;
                if (idx >= i0 && idx <= i1) P[idx] = dkey_inv(min(k, carry));
                carry = min(carry, __shfl_sync(0xffffffffu, k, 31));
            }
        }
    }

    if (tid == 0) {
        int status = 0;
        if (bad) status |= EPSCU_STATUS_BAD | EPSCU_STATUS_NONFINITE;
        if (i1 - i0 < 2) status |= EPSCU_STATUS_BAD;
        if (!(m.e_cap > vmin)) status |= EPSCU_STATUS_BAD;
        m.h = h;
        m.a = a;
        m.e_lo = vmin;
        m.i0 = i0;
        m.i1 = i1;
        m.k_scan = k_scan < N ? k_scan : i0;
        m.delta = __ddiv_rn(__dsub_rn(m.e_cap, vmin), (double)m.n_trial);
        const double tol = b.tol > 0.0 ? b.tol : 1e-12;
        int K = 0;
        for (double w = m.delta; w > tol && K < 200; w = __dmul_rn(w, 0.5)) ++K;
        m.n_bisect = K;
        const double kmax = sqrt(2.0 * m.mu * (m.e_cap - vmin));
        if (kmax * h > 1.0) status |= EPSCU_STATUS_UNDER;
        m.status = status;
        m.n_total = 0;
        m.n_out = 0;
        b.meta[p] = m;
    }
}

// Level counts per potential, exclusive prefix sums (level slots and psi
// offsets) and the total level count.  One CTA.
// A solve cancelled before this point, or whose scan gave up on a bounded wait
// (the error word is set), may have skipped scan work: its counts are
// incomplete and it gets no levels.  The cancel flag only goes from 0 to 1
// while a solve runs, so a scan that saw it is always followed by a set-up
// that does.
__global__ void __launch_bounds__(1024) level_setup_kernel(DevBatch b) {
    __shared__ int32_t s_lv[1024];
    __shared__ long long s_ps[1024];
    __shared__ int32_t carry_lv;
    __shared__ long long carry_ps;
    __shared__ int s_cancelled, s_failed;
    if (threadIdx.x == 0) {
        carry_lv = 0;
        carry_ps = 0;
        s_cancelled = b.cancel && *b.cancel;
        s_failed = b.hdr->error != 0;
    }
    __syncthreads();
    const bool cancelled = s_cancelled != 0, failed = s_failed != 0;
    for (int base = 0; base < b.n; base += blockDim.x) {
        const int p = base + threadIdx.x;
        int32_t n_out = 0;
        long long ps = 0;
        if (p < b.n) {
            PotMeta& m = b.meta[p];
            int32_t n_total = 0;
            if (cancelled) m.status |= EPSCU_STATUS_CANCELLED;
            else if (!failed && !(m.status & EPSCU_STATUS_BAD)) n_total = b.counts[(int64_t)p * b.n_trial + b.n_trial - 1];
            int32_t last = b.max_level < 0 ? n_total - 1 : min(b.max_level, n_total - 1);
            n_out = last - b.min_level + 1;
            n_out = max(0, min(n_out, b.level_capacity));
            m.n_total = n_total;
            m.n_out = n_out;
            ps = (long long)n_out * m.N;
        }
        s_lv[threadIdx.x] = n_out;
        s_ps[threadIdx.x] = ps;
        __syncthreads();
        // inclusive Hillis-Steele scan
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {
            int32_t x = threadIdx.x >= o ? s_lv[threadIdx.x - o] : 0;
            long long y = threadIdx.x >= o ? s_ps[threadIdx.x - o] : 0;
            __syncthreads();
            s_lv[threadIdx.x] += x;
            s_ps[threadIdx.x] += y;
            __syncthreads();
        }
        if (p < b.n) {
            b.meta[p].level_base = carry_lv + s_lv[threadIdx.x] - n_out;
            b.meta[p].psi_off = carry_ps + s_ps[threadIdx.x] - ps;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) {
            carry_lv += s_lv[threadIdx.x];
            carry_ps += s_ps[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        b.hdr->total_levels = carry_lv;
        b.hdr->psi_total = carry_ps;
        b.hdr->queue_refine = 0;
        b.hdr->queue_polish = 0;
        if (b.psi && carry_ps > b.psi_capacity) atomicCAS(&b.hdr->error, 0, 5);
    }
}

// Warp work units for the per-level kernels: each potential's level slots in
// chunks of 32, potentials in decreasing grid length (the `order` array), so
// the warp queue hands out the longest work first.  One CTA.
__global__ void __launch_bounds__(1024) unit_setup_kernel(DevBatch b) {
    __shared__ int32_t s_u[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < b.n; base += blockDim.x) {
        const int q = base + threadIdx.x;
        int32_t nu = 0;
        int p = 0;
        if (q < b.n) {
            p = b.order[q];
            nu = (b.meta[p].n_out + 31) / 32;
        }
        s_u[threadIdx.x] = nu;
        __syncthreads();
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {
            const int32_t x = threadIdx.x >= o ? s_u[threadIdx.x - o] : 0;
            __syncthreads();
            s_u[threadIdx.x] += x;
            __syncthreads();
        }
        if (q < b.n) {
            const int32_t first = carry + s_u[threadIdx.x] - nu;
            const PotMeta& m = b.meta[p];
            for (int u = 0; u < nu; ++u) {
                const int32_t at = first + u;
                if (at < b.max_units) b.units[at] = make_int2(m.level_base + 32 * u, min(32, m.n_out - 32 * u));
            }
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += s_u[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) b.hdr->n_units = min(carry, b.max_units);
}

// Bracket of every level slot from the scan counts: first trial j with
// count_j > v; bracket [E_{j-1}, E_j] (E_{-1} = E_lo).
__global__ void bracket_kernel(DevBatch b) {
    const int p = blockIdx.x;
    const PotMeta m = b.meta[p];
    const int32_t* c = b.counts + (int64_t)p * b.n_trial;
    for (int s = threadIdx.x; s < m.n_out; s += blockDim.x) {
        const int v = b.min_level + s;
        int lo = 0, hi = m.n_trial;
        int top = -1;  // trial index of the bracket's upper end (lo when -1)
        if (!b.bis_list) {
            while (lo < hi) {
                const int mid = lo + (hi - lo) / 2;
                if (c[mid] > v) hi = mid;
                else lo = mid + 1;
            }
        } else {
            // bisection scan: counts exist at the coarse boundaries and at the
            // midpoints of every cell that held a level; descend the same
            // cells to the first trial index with a count above v
            const int last = m.n_trial - 1;
            const int ctop = c[last];
            if (v >= ctop) {
                lo = m.n_trial;
            } else {
                const int K = (m.n_trial + kBisectCoarse - 1) / kBisectCoarse;
                int kl = 1, kh = K;  // first coarse boundary with a count above v
                while (kl < kh) {
                    const int km = (kl + kh) / 2;
                    if (c[min(km * kBisectCoarse - 1, last)] > v) kh = km;
                    else kl = km + 1;
                }
                // then down the cell's halves while their midpoints have a
                // count (a cell cut into fewer parts ends the descent early:
                // the bracket is the last cell (a, a + W])
                int a = (kl - 1) * kBisectCoarse - 1;
                int W = kBisectCoarse;
                for (; W > 1; W >>= 1) {
                    const int mid = a + W / 2;
                    const int cm = mid >= last ? ctop : c[mid];
                    if (cm < 0) break;  // no count taken there
                    if (cm <= v) a = mid;
                }
                lo = min(a + 1, last);
                top = min(a + W, last);
            }
        }
        LevelWork w;
        w.p = p;
        w.v = v;
        w.status = m.status & EPSCU_STATUS_UNDER;
        w.nodes = -1;
        w.iters = 0;
        w.k = m.k_scan;
        w.dE = 0.0;
        w.norm_k_out = w.norm_k_in = 0.0;
        w.ex_out = w.ex_in = 0;
        w.n_in_bracket = 0;
        if (lo >= m.n_trial) {
            w.status |= EPSCU_STATUS_NOTFOUND;
            w.lo = w.hi = w.E = m.e_cap;
        } else {
            if (top < lo) top = lo;
            w.lo = lo == 0 ? m.e_lo : trial_energy(m, lo - 1);
            w.hi = trial_energy(m, top);
            w.E = __dmul_rn(0.5, __dadd_rn(w.lo, w.hi));
            w.n_in_bracket = c[top] - (lo == 0 ? 0 : c[lo - 1]);
            if (b.gam && lo > 0 && w.n_in_bracket == 1) {
                // the first energy of the refinement: the zero of the scan's
                // matching function interpolated between the bracket's ends,
                // when it falls from positive to negative there (one level, no
                // pole between); the midpoint otherwise
                const float* g = b.gam + (int64_t)p * b.n_trial;
                const float gl = g[lo - 1], gr = g[top];
                if (gl > 0.0f && gr < 0.0f && gl < INFINITY && gr > -INFINITY) {
                    const double t = fmin(0.95, fmax(0.05, (double)gl / ((double)gl - (double)gr)));
                    w.E = w.lo + t * (w.hi - w.lo);
                }
            }
        }
        w.lo0 = w.lo;
        w.hi0 = w.hi;
        w.j0 = m.i0;
        w.j1 = m.i1;
        w.pad1 = 0;
        b.levels[m.level_base + s] = w;
    }
}

// Decay window at energy Eu (fast method; one call per warp, all lanes).
// Beyond the classical turning points of Eu (V > Eu there) the discrete
// solution decays at least by the constant-coefficient rate of the Numerov
// recurrence, acosh(1 + 6 t_i) per step with t_i = W_i - a Eu (for small t it
// is kappa h, the WKB exponent; for larger t it is below the true rate).  The
// window ends where that exponent, summed from the turning point, reaches
// `decay`: Dirichlet ends there change the solution by about e^-decay relative
// to its size at the turning point and an eigenvalue by a relative e^-2 decay,
// and every energy below Eu has a narrower window.  The classical choice of
// the start of the inward integration in Numerov-Cooley codes.
// Turning points come from binary searches on the suffix and prefix minima of
// V; the sums run over whole 32-point blocks beyond the turning point's block,
// a block of n points counting n acosh(1 + 6 (min W - a Eu)) (block minima
// rounded down, a Eu rounded up): a lower bound of the decay, so the window
// can only come out wider.  Returns [j0, j1] within [i0, i1].
__device__ int2 decay_window(const PotMeta& m, const DevBatch& b, double Eu, float decay) {
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const float aEu = __double2float_ru(m.a * Eu);
    const float* Bm = b.Bmin + m.offf / 32;
    const int t_out = match_index(m, b.Msuf, Eu);
    int t_in;
    {
        // first i with min(V_i0 .. V_i) <= Eu (the prefix minima do not increase)
        const double* P = b.Mpre + m.off;
        int lo = m.i0, hi = m.i1;
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (P[mid] <= Eu) hi = mid;
            else lo = mid + 1;
        }
        t_in = lo;
    }
    const int B_first = m.i0 >> 5, B_last = m.i1 >> 5;
    auto block_decay = [&](int B) {
        const int n = min((B << 5) + 31, m.i1) - max(B << 5, m.i0) + 1;
        return (float)n * acoshf(1.0f + 6.0f * fmaxf(Bm[B] - aEu, 0.0f));
    };
    int j1 = m.i1;
    float X = 0.0f;
    for (int B0 = (t_out >> 5) + 1; B0 <= B_last; B0 += 32) {
        const int B = B0 + lane;
        float s = B <= B_last ? block_decay(B) : 0.0f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(full, s, o);
            if (lane >= o) s += y;
        }
        const unsigned hit = __ballot_sync(full, B <= B_last && X + s >= decay);
        if (hit) {
            j1 = min(((B0 + __ffs(hit) - 1) << 5) + 31, m.i1);
            break;
        }
        X += __shfl_sync(full, s, 31);
    }
    int j0 = m.i0;
    X = 0.0f;
    for (int B0 = (t_in >> 5) - 1; B0 >= B_first; B0 -= 32) {
        const int B = B0 - lane;
        float s = B >= B_first ? block_decay(B) : 0.0f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(full, s, o);
            if (lane >= o) s += y;
        }
        const unsigned hit = __ballot_sync(full, B >= B_first && X + s >= decay);
        if (hit) {
            j0 = max((B0 - (__ffs(hit) - 1)) << 5, m.i0);
            break;
        }
        X += __shfl_sync(full, s, 31);
    }
    if (j1 - j0 < 4) return make_int2(m.i0, m.i1);
    return make_int2(j0, j1);
}

// Decay window of every level slot (fast method), at E_up = hi0 + 2 delta:
// an energy above every energy the level's passes use (bracket, Newton steps,
// the fallback's widened bracket), so one window serves all of them.  Levels
// whose window is longer than the long-window threshold (DevBatch::long_window,
// else default_long_window of the level count) go to the long list
// (CTA-per-level passes), those above the middle threshold to the middle list
// (lane FP32 refinement, then warp-per-level double-float passes); the rest
// stay on the lane kernels.  One warp per level.
// (Sharing one window per warp unit would keep the lanes' loads of W
// warp-wide broadcasts, but the unit's widest window costs more point-updates
// than the divergent loads: measured slower on the mixed batch.)
__global__ void __launch_bounds__(128) window_kernel(DevBatch b, int sm_count) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int total = b.hdr->total_levels;
    (void)sm_count;
    const int long_min = b.long_window > 0 ? b.long_window : default_long_window(total);
    const int mid_w = b.mid_window != 0 ? b.mid_window : kMidWindow;
    const int mid_min = mid_w <= 0 || !b.mid_list ? 0x7fffffff : mid_w;
    for (int slot = warp; slot < total; slot += n_warps) {
        const LevelWork w = b.levels[slot];
        if (w.status & EPSCU_STATUS_NOTFOUND) continue;
        const PotMeta m = b.meta[w.p];
        const int2 jw = decay_window(m, b, w.hi0 + 2.0 * m.delta, kWindowDecay);
        if ((threadIdx.x & 31) == 0) {
            b.levels[slot].j0 = jw.x;
            b.levels[slot].j1 = jw.y;
            if (jw.y - jw.x > long_min && b.long_list) {
                const int q = atomicAdd(&b.hdr->n_long, 1);
                if (q < b.max_levels) {
                    b.long_list[q] = slot;
                    b.levels[slot].status = w.status | EPSCU_STATUS_LONG;
                }
            } else if (jw.y - jw.x > mid_min) {
                const int q = atomicAdd(&b.hdr->n_mid, 1);
                if (q < b.max_levels) {
                    b.mid_list[q] = slot;
                    b.levels[slot].status = w.status | EPSCU_STATUS_MID;
                }
            }
        }
    }
}

// Decay windows of the scan: entry (p, q) is the window of the highest trial
// energy of block q (kScanWinBlock consecutive trial energies) of potential p,
// which contains the windows of every energy of the block.  One warp per entry.
__global__ void __launch_bounds__(128) scan_window_kernel(DevBatch b, int n_blk) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int total = b.n * n_blk;
    for (int e = warp; e < total; e += n_warps) {
        const int p = e / n_blk, q = e % n_blk;
        const PotMeta m = b.meta[p];
        int2 jw = make_int2(m.i0, m.i1);
        if (!(m.status & EPSCU_STATUS_BAD)) {
            const int j = min((q + 1) * kScanWinBlock, b.n_trial) - 1;
            jw = decay_window(m, b, trial_energy(m, j), kWindowDecay);
        }
        if ((threadIdx.x & 31) == 0) b.scan_win[e] = jw;
    }
}

// ------------------------------------------------------------- tabulation (K0)

__device__ double morse_v(double r, double De, double a, double re) {
    const double x = 1.0 - exp(-a * (r - re));
    return De * x * x;
}

__global__ void tabulate_kernel(int32_t n, const int32_t* kind, const double* params, const int64_t* offsets,
                                const int32_t* Ns, const double* r_min, const double* r_max, int32_t n_knots,
                                double* scratch, double* V) {
    const int p = blockIdx.x;
    const int N = Ns[p];
    const double r0 = r_min[p], r1 = r_max[p];
    const double h = (r1 - r0) / (double)(N - 1);
    const double* P = params + (int64_t)p * 12;
    double* out = V + offsets[p];
    const int k = kind[p];
    if (k == EPSCU_KIND_SPLINE) {
        // knot values (Morse + Gaussian bumps), natural spline second derivatives
        double* y = scratch + (int64_t)p * 3 * n_knots;
        double* M = y + n_knots;
        double* cp = M + n_knots;
        const double hk = (r1 - r0) / (double)(n_knots - 1);
        for (int j = threadIdx.x; j < n_knots; j += blockDim.x) {
            const double r = r0 + j * hk;
            double v = morse_v(r, P[0], P[1], P[2]);
            for (int q = 0; q < 3; ++q) {
                const double amp = P[3 + 3 * q], w = P[4 + 3 * q], c = P[5 + 3 * q];
                if (amp != 0.0) v += amp * exp(-((r - c) * (r - c)) / (2.0 * w * w));
            }
            y[j] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // Thomas algorithm for M_{k-1} + 4 M_k + M_{k+1} = 6 (y_{k+1} - 2 y_k + y_{k-1}) / hk^2
            const int nn = n_knots - 2;
            const double s6 = 6.0 / (hk * hk);
            M[0] = 0.0;
            M[n_knots - 1] = 0.0;
            // forward sweep: cp in cp[], dp in M[1..]
            cp[0] = 1.0 / 4.0;
            M[1] = s6 * (y[2] - 2.0 * y[1] + y[0]) / 4.0;
            for (int i = 1; i < nn; ++i) {
                const double den = 4.0 - cp[i - 1];
                cp[i] = 1.0 / den;
                const double rhs = s6 * (y[i + 2] - 2.0 * y[i + 1] + y[i]);
                M[i + 1] = (rhs - M[i]) / den;
            }
            for (int i = nn - 2; i >= 0; --i) M[i + 1] = M[i + 1] - cp[i] * M[i + 2];
        }
        __syncthreads();
        const double h2 = hk * hk / 6.0;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double r = r0 + i * h;
            const double t = (r - r0) / hk;
            int j = (int)floor(t);
            j = max(0, min(j, n_knots - 2));
            const double u = t - j, w = 1.0 - u;
            out[i] = w * y[j] + u * y[j + 1] + h2 * ((w * w * w - w) * M[j] + (u * u * u - u) * M[j + 1]);
        }
    } else if (k == EPSCU_KIND_LJ) {
        const double eps = P[0], sigma = P[1];
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double r = r0 + i * h;
            const double s = sigma / r;
            const double s2 = s * s;
            const double s6 = s2 * s2 * s2;
            out[i] = 4.0 * eps * (s6 * s6 - s6) + eps;
        }
    } else {
        for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = morse_v(r0 + i * h, P[0], P[1], P[2]);
    }
}

// The adjoint of tabulate_kernel: dL/dparams from dL/dV, one CTA per
// potential (kTabAdjThreads threads), in FP64.
//   Morse, LJ: sum_i g_i dV_i/dtheta over the grid.
//   Morse + bumps through the spline: V_i = w y_j + u y_{j+1}
//     + hk^2/6 ((w^3 - w) M_j + (u^3 - u) M_{j+1}) with M = A^-1 (6/hk^2) D2 y
//     (A = tridiag(1, 4, 1) on the interior knots, M_0 = M_{K-1} = 0), so
//     dL/dy = S^T g = P^T g + (6/hk^2) D2^T A^-1 Q^T g, with P^T g and Q^T g
//     the grid's pull-back onto the knots (the w/u and the cubic weights) and
//     A^-1 applied by the same Thomas sweep as the forward; then
//     sum_k dL/dy_k dy_k/dtheta over the knots (Morse and Gaussian terms).
// The pull-back is deterministic: each thread owns a contiguous range of knot
// intervals and the grid points that fall in them (the same interval rule as
// the forward), writing the interval's left and right sums; every sum then
// runs in a fixed order (no atomics), so repeated calls give identical bits.
constexpr int kTabAdjThreads = 256;

__device__ __forceinline__ int tab_interval(int i, double r0, double h, double hk, int n_knots) {
    const double r = r0 + i * h;
    const double t = (r - r0) / hk;
    int j = (int)floor(t);
    return max(0, min(j, n_knots - 2));
}

// deterministic sum of one value per thread over the CTA (fixed tree)
__device__ __forceinline__ double cta_sum(double v, double* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = kTabAdjThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kTabAdjThreads) tabulate_adjoint_kernel(
    int32_t n, const int32_t* kind, const double* params, const int64_t* offsets, const int32_t* Ns,
    const double* r_min, const double* r_max, int32_t n_knots, double* scratch, const double* gV, double* gP) {
    __shared__ double red[kTabAdjThreads];
    const int p = blockIdx.x;
    const int N = Ns[p];
    const double r0 = r_min[p], r1 = r_max[p];
    const double h = (r1 - r0) / (double)(N - 1);
    const double* P = params + (int64_t)p * 12;
    const double* g = gV + offsets[p];
    double acc[12];
    for (int q = 0; q < 12; ++q) acc[q] = 0.0;
    const int k = kind[p];
    if (k == EPSCU_KIND_SPLINE) {
        const int K = n_knots;
        const double hk = (r1 - r0) / (double)(K - 1);
        const double h2 = hk * hk / 6.0, s6 = 6.0 / (hk * hk);
        double* Ly = scratch + (int64_t)p * 6 * K;  // per interval: left and right sums of w, u weights
        double* Ry = Ly + K;
        double* LM = Ry + K;                          // and of the cubic weights
        double* RM = LM + K;
        double* z = RM + K;                           // A^-1 (Q^T g) on the interior knots
        double* cp = z + K;
        // ---- pull-back onto the knot intervals [jb, je) owned by this thread
        const int nint = K - 1;
        const int per = (nint + kTabAdjThreads - 1) / kTabAdjThreads;
        const int jb = min((int)threadIdx.x * per, nint), je = min(jb + per, nint);
        if (jb < je) {
            // first grid point of interval jb: an estimate, then the forward's rule
            int i = (int)fmax(0.0, floor(jb * hk / h) - 2.0);
            i = min(i, N - 1);
            while (i > 0 && tab_interval(i, r0, h, hk, K) >= jb) --i;
            while (i < N && tab_interval(i, r0, h, hk, K) < jb) ++i;
            for (int j = jb; j < je; ++j) {
                double ly = 0.0, ry = 0.0, lm = 0.0, rm = 0.0;
                for (; i < N; ++i) {
                    const double r = r0 + i * h;
                    const double t = (r - r0) / hk;
                    int jj = (int)floor(t);
                    jj = max(0, min(jj, K - 2));
                    if (jj != j) break;
                    const double u = t - jj, w = 1.0 - u;
                    const double gi = g[i];
                    ly += gi * w;
                    ry += gi * u;
                    lm += gi * h2 * (w * w * w - w);
                    rm += gi * h2 * (u * u * u - u);
                }
                Ly[j] = ly;
                Ry[j] = ry;
                LM[j] = lm;
                RM[j] = rm;
            }
        }
        __syncthreads();
        // ---- z = A^-1 (Q^T g)_interior (A symmetric): the forward's Thomas sweep
        if (threadIdx.x == 0) {
            const int nn = K - 2;
            auto gm = [&](int kk) { return LM[kk] + (kk > 0 ? RM[kk - 1] : 0.0); };  // (Q^T g) at knot kk
            cp[0] = 1.0 / 4.0;
            z[1] = gm(1) / 4.0;
            for (int q = 1; q < nn; ++q) {
                const double den = 4.0 - cp[q - 1];
                cp[q] = 1.0 / den;
                z[q + 1] = (gm(q + 1) - z[q]) / den;
            }
            for (int q = nn - 2; q >= 0; --q) z[q + 1] = z[q + 1] - cp[q] * z[q + 2];
            z[0] = 0.0;
            z[K - 1] = 0.0;
        }
        __syncthreads();
        // ---- dL/dy_k = (P^T g)_k + s6 (D2^T z)_k, then the knots' parameter derivatives
        for (int kk = threadIdx.x; kk < K; kk += kTabAdjThreads) {
            // (intervals are 0..K-2: the last knot has no interval of its own)
            double gy = (kk < K - 1 ? Ly[kk] : 0.0) + (kk > 0 ? Ry[kk - 1] : 0.0);
            const double zl = kk >= 1 ? z[kk - 1] : 0.0, zc = z[kk], zr = kk + 1 < K ? z[kk + 1] : 0.0;
            gy += s6 * (zl - 2.0 * zc + zr);
            const double r = r0 + kk * hk;
            const double De = P[0], a = P[1], re = P[2];
            const double e = exp(-a * (r - re));
            const double x = 1.0 - e;
            acc[0] += gy * x * x;
            acc[1] += gy * 2.0 * De * x * e * (r - re);
            acc[2] += gy * -2.0 * De * x * e * a;
            for (int q = 0; q < 3; ++q) {
                const double amp = P[3 + 3 * q], wd = P[4 + 3 * q], c = P[5 + 3 * q];
                if (amp == 0.0) continue;
                const double d = r - c;
                const double G = exp(-(d * d) / (2.0 * wd * wd));
                acc[3 + 3 * q] += gy * G;
                acc[4 + 3 * q] += gy * amp * G * d * d / (wd * wd * wd);
                acc[5 + 3 * q] += gy * amp * G * d / (wd * wd);
            }
        }
    } else if (k == EPSCU_KIND_LJ) {
        const double eps = P[0], sigma = P[1];
        for (int i = threadIdx.x; i < N; i += kTabAdjThreads) {
            const double r = r0 + i * h;
            const double s = sigma / r;
            const double s2 = s * s;
            const double s6 = s2 * s2 * s2;
            acc[0] += g[i] * (4.0 * (s6 * s6 - s6) + 1.0);
            acc[1] += g[i] * 4.0 * eps * (12.0 * s6 * s6 - 6.0 * s6) / sigma;
        }
    } else {
        const double De = P[0], a = P[1], re = P[2];
        for (int i = threadIdx.x; i < N; i += kTabAdjThreads) {
            const double r = r0 + i * h;
            const double e = exp(-a * (r - re));
            const double x = 1.0 - e;
            acc[0] += g[i] * x * x;
            acc[1] += g[i] * 2.0 * De * x * e * (r - re);
            acc[2] += g[i] * -2.0 * De * x * e * a;
        }
    }
    for (int q = 0; q < 12; ++q) {
        const double v = cta_sum(acc[q], red);
        if (threadIdx.x == 0) gP[(int64_t)p * 12 + q] = v;
    }
}

}  // namespace

void launch_tabulate_adjoint(int32_t n, const int32_t* kind, const double* params, const int64_t* offsets,
                             const int32_t* N, const double* r_min, const double* r_max, int32_t n_knots,
                             double* knot_scratch, const double* gV, double* gP, cudaStream_t s) {
    tabulate_adjoint_kernel<<<n, kTabAdjThreads, 0, s>>>(n, kind, params, offsets, N, r_min, r_max, n_knots,
                                                         knot_scratch, gV, gP);
}

void launch_prepare(const DevBatch& b, cudaStream_t s) {
    prepare_kernel<<<b.n, kPrepThreads, 0, s>>>(b);
}

void launch_level_setup(const DevBatch& b, cudaStream_t s) {
    level_setup_kernel<<<1, 1024, 0, s>>>(b);
    unit_setup_kernel<<<1, 1024, 0, s>>>(b);
    bracket_kernel<<<b.n, 128, 0, s>>>(b);
}

void launch_window(const DevBatch& b, int sm_count, cudaStream_t s) {
    window_kernel<<<sm_count * 8, 128, 0, s>>>(b, sm_count);
}

void launch_scan_window(const DevBatch& b, int sm_count, cudaStream_t s) {
    if (!b.scan_win) return;
    scan_window_kernel<<<sm_count * 8, 128, 0, s>>>(b, (b.n_trial + kScanWinBlock - 1) / kScanWinBlock);
}

void launch_tabulate(int32_t n, const int32_t* kind, const double* params, const int64_t* offsets, const int32_t* N,
                     const double* r_min, const double* r_max, int32_t n_knots, double* knot_scratch, double* V,
                     cudaStream_t s) {
    tabulate_kernel<<<n, 256, 0, s>>>(n, kind, params, offsets, N, r_min, r_max, n_knots, knot_scratch, V);
}

}  // namespace epscu
