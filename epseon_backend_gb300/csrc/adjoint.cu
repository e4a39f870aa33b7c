// adjoint.cu -- Hellmann-Feynman adjoint of the discrete problem.
//
// For the symmetric discretisation H = diag(V) - B^{-1} D2 / (2 mu h^2) the
// derivative of a level with respect to the potential at a grid point is
// exactly dE_v / dV_i = psi_v(r_i)^2 h for the wavefunction normalised with
// sum psi^2 h = 1, so for L(E) the gradient is
//     dL/dV_i = sum_v dL/dE_v psi_v(r_i)^2 h.
// One thread per grid point, reading the potential's psi rows coalesced; the
// kernel is HBM-bound (8 bytes of psi per level and point).  psi is zero
// outside each level's window [j0, j1] (the written rows hold zeros there), so
// those reads are skipped: on the mixed batch the fast method's windows hold
// about a fifth of the row points.
#include <cuda_runtime.h>

#include "common.cuh"
#include "launch.h"

namespace epscu {

namespace {

// psi rows of the last solve in place (row s of potential p at psi_off + s N);
// accumulate = add into dL_dV instead of storing.  One CTA per (potential,
// 256 points); the CTA first narrows the level loop to the levels whose
// window meets its points (windows grow with the level, so near the ends of
// a grid only the highest levels remain).
__global__ void __launch_bounds__(256) adjoint_kernel(DevBatch b, const double* __restrict__ gE, double* __restrict__ gV,
                                                      const int64_t* __restrict__ offsets, const double* __restrict__ psi,
                                                      int accumulate) {
    __shared__ int s_lo, s_hi;
    const int p = blockIdx.y;
    const PotMeta m = b.meta[p];
    const int i_a = blockIdx.x * blockDim.x;
    if (i_a >= m.N) return;
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
    const int i = i_a + threadIdx.x;
    if (i > i_b) return;
    const double* rows = psi + m.psi_off + i;
    const double* g = gE + (int64_t)p * b.level_capacity;
    double acc = 0.0;
    for (int s = s_lo; s <= s_hi; ++s) {
        if (i < lw[s].j0 || i > lw[s].j1) continue;
        const double v = __ldg(rows + (int64_t)s * m.N);
        acc = fma(g[s] * v, v, acc);
    }
    acc *= m.h;
    if (accumulate) gV[offsets[p] + i] += acc;
    else gV[offsets[p] + i] = acc;
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

void launch_adjoint(const DevBatch& b, const double* dL_dE, double* dL_dV, int64_t total_points,
                    const int64_t* offsets_dev, int recompute, int sm_count, cudaStream_t s) {
    (void)total_points;
    (void)recompute;
    (void)sm_count;
    // grid.x covers the longest grid; threads past a shorter grid exit at once
    dim3 grid((b.max_N + 255) / 256, b.n);
    adjoint_kernel<<<grid, 256, 0, s>>>(b, dL_dE, dL_dV, offsets_dev, b.psi, 0);
}

}  // namespace epscu
