// adjoint.cu -- Hellmann-Feynman adjoint of the discrete problem.
//
// For the symmetric discretisation H = diag(V) - B^{-1} D2 / (2 mu h^2) the
// derivative of a level with respect to the potential at a grid point is
// exactly dE_v / dV_i = psi_v(r_i)^2 h for the wavefunction normalised with
// sum psi^2 h = 1, so for L(E) the gradient is
//     dL/dV_i = sum_v dL/dE_v psi_v(r_i)^2 h.
// One thread per grid point, reading the potential's psi rows coalesced.  The
// sum runs in double-float on the FP32 pipes (each psi double split into a
// float pair by its bits, dL/dE_v psi^2 by two-product arithmetic, ~1e-14
// relative): with an FP64 multiply-add per level and point the kernel was
// bound by GB300's FP64 pipe (ncu: 82% busy), not by HBM.  psi is zero
// outside each level's window [j0, j1] (the written rows hold zeros there), so
// those reads are skipped: on the mixed batch the fast method's windows hold
// about a fifth of the row points.
#include <cuda_runtime.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "launch.h"

namespace epscu {

namespace {

// psi rows of the last solve in place (row s of potential p at psi_off + s N);
// accumulate = add into dL_dV instead of storing.  One CTA per (potential,
// 256 points); the CTA first narrows the level loop to the levels whose
// window meets its points (windows grow with the level, so near the ends of
// a grid only the highest levels remain), stages their windows and dL/dE in
// shared memory, and reads four rows per step (four loads in flight per
// thread: the kernel is bound by HBM latency otherwise).
constexpr int kAdjTile = 256;  // levels staged per round

__global__ void __launch_bounds__(kAdjointPoints) adjoint_kernel(DevBatch b, const double* __restrict__ gE,
                                                                 double* __restrict__ gV,
                                                                 const int64_t* __restrict__ offsets,
                                                                 const int32_t* __restrict__ tiles,
                                                                 const double* __restrict__ psi, int accumulate) {
    __shared__ int s_lo, s_hi, s_p;
    __shared__ int2 s_win[kAdjTile];
    __shared__ float s_gh[kAdjTile], s_gl[kAdjTile];  // dL/dE as double-float pairs
    if (threadIdx.x == 0) {
        // the potential of this tile: the last p with tiles[p] <= blockIdx.x
        int lo = 0, hi = b.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tiles[mid] <= (int)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        s_p = lo;
    }
    __syncthreads();
    const int p = s_p;
    const PotMeta m = b.meta[p];
    const int i_a = ((int)blockIdx.x - tiles[p]) * kAdjointPoints;
    const int i_b = min(i_a + (int)blockDim.x, m.N) - 1;
    const LevelWork* lw = b.levels + m.level_base;
    if (threadIdx.x == 0) {
        s_lo = m.n_out;
        s_hi = -1;
    }
    __syncthreads();
    for (int s = threadIdx.x; s < m.n_out; s += blockDim.x) {
        if (lw[s].j0 <= i_b && lw[s].j1 >= i_a) {
            atomicMin(&s_lo, s);
            atomicMax(&s_hi, s);
        }
    }
    __syncthreads();
    const int lo = s_lo, hi = s_hi;
    const int i = i_a + threadIdx.x;
    const double* rows = psi + m.psi_off + i;
    const double* g = gE + (int64_t)p * b.level_capacity;
    dfl acc = {0.0f, 0.0f};
    for (int t0 = lo; t0 <= hi; t0 += kAdjTile) {
        const int nt = min(kAdjTile, hi - t0 + 1);
        __syncthreads();  // the previous round's stage is consumed
        for (int q = threadIdx.x; q < nt; q += blockDim.x) {
            s_win[q] = make_int2(lw[t0 + q].j0, lw[t0 + q].j1);
            const dfl gq = df_from_double(g[t0 + q]);
            s_gh[q] = gq.h;
            s_gl[q] = gq.l;
        }
        __syncthreads();
        if (i > i_b) continue;
        // (a level's term is added only inside its window, as if the loop
        // skipped the others: a non-finite dL/dE stays out of their sums)
        auto inside = [&](int q) {
            const int2 wq = s_win[q];
            return i >= wq.x && i <= wq.y;
        };
        auto load = [&](int q) { return inside(q) ? __ldg(rows + (int64_t)(t0 + q) * m.N) : 0.0; };
        auto add = [&](int q, double v) {
            if (!inside(q)) return;
            const dfl x = df_split_double_bits(v);
            acc = df_add(acc, df_mul(df_mul(x, x), dfl{s_gh[q], s_gl[q]}));
        };
        int q = 0;
        for (; q + 3 < nt; q += 4) {
            const double v0 = load(q), v1 = load(q + 1), v2 = load(q + 2), v3 = load(q + 3);
            add(q, v0);
            add(q + 1, v1);
            add(q + 2, v2);
            add(q + 3, v3);
        }
        for (; q < nt; ++q) add(q, load(q));
    }
    if (i > i_b) return;
    const double r = (f2d(acc.h) + f2d(acc.l)) * m.h;
    if (accumulate) gV[offsets[p] + i] += r;
    else gV[offsets[p] + i] = r;
}

// Explicit layout (stateless adjoint): per-potential arrays on the device.
__global__ void adjoint_explicit_kernel(int32_t cap, const int64_t* __restrict__ offsets, const int32_t* __restrict__ Ns,
                                        const double* __restrict__ hs, const int32_t* __restrict__ n_outs,
                                        const int64_t* __restrict__ psi_offs, const double* __restrict__ psi,
                                        const double* __restrict__ gE, double* __restrict__ gV) {
    const int p = blockIdx.y;
    const int N = Ns[p];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int n_out = n_outs[p];
    const double* rows = psi + psi_offs[p] + i;
    const double* g = gE + (int64_t)p * cap;
    double acc = 0.0;
    for (int s = 0; s < n_out; ++s) {
        const double v = __ldg(rows + (int64_t)s * N);
        acc = fma(g[s] * v, v, acc);
    }
    gV[offsets[p] + i] = acc * hs[p];
}

}  // namespace

void launch_adjoint_explicit(int32_t n, int32_t cap, int32_t max_N, const int64_t* offsets, const int32_t* N,
                             const double* h, const int32_t* n_out, const int64_t* psi_off, const double* psi,
                             const double* gE, double* gV, cudaStream_t s) {
    dim3 grid((max_N + 255) / 256, n);
    adjoint_explicit_kernel<<<grid, 256, 0, s>>>(cap, offsets, N, h, n_out, psi_off, psi, gE, gV);
}

void launch_adjoint(const DevBatch& b, const double* dL_dE, double* dL_dV, const int64_t* offsets_dev,
                    const int32_t* tiles_dev, int32_t n_tiles, cudaStream_t s) {
    // one CTA per tile of kAdjointPoints points of a potential (a 2-D grid
    // over the longest grid left ~3/4 of its CTAs empty on the mixed batch)
    if (n_tiles <= 0) return;
    adjoint_kernel<<<n_tiles, kAdjointPoints, 0, s>>>(b, dL_dE, dL_dV, offsets_dev, tiles_dev, b.psi, 0);
}

}  // namespace epscu
