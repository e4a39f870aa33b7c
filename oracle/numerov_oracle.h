/*
 * numerov_oracle.h -- FP64 CPU oracle for the vibrational-level solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path is
 * compared against (tests, smoke check, and the CPU baseline leg of bench.py).
 * The product path never links, loads or calls it.
 *
 * PARITY UNPINNED with respect to the reference: epseon_backend contains no
 * solver arithmetic (VibwaAlgorithm<FP>::run, cpp/gpu/include/epseon/gpu/
 * algorithms/vibwa.hpp:605-637, allocates buffers and returns; both
 * get_potential_data() stubs return {} in cpp/gpu/include/epseon/gpu/
 * task_configurator/potential_source.hpp:89-91 and :223-225) and its tests hold
 * no golden vectors.  The oracle is a restatement of the published methods:
 *   - Numerov's three-term recurrence in divide-free projective form,
 *   - Sturm-sequence (twisted LDL^T) node counting, cf. Blatt, J. Comput.
 *     Phys. 1, 382 (1967) and Johnson, J. Chem. Phys. 67, 4086 (1977),
 *   - level bracketing from a trial-energy scan plus bisection,
 *   - Cooley's energy correction, Math. Comp. 15, 363 (1961),
 * and is pinned instead against (tests/test_oracle.py): the dense symmetric
 * eigen-decomposition of the same discretisation, the analytic Morse spectrum
 * to O(h^4), node count == level index, and Hellmann-Feynman vs central
 * finite differences.
 *
 * The discrete problem (identical in the oracle and the CUDA kernels):
 *   r_i = r_min + i h, h = (r_max - r_min)/(N-1),  a = mu h^2 / 6,
 *   T_i(E) = a E - a V_i,  f_i = 1 + T_i,  g_i = 2 - 10 T_i,
 *   f_{i+1} psi_{i+1} - g_i psi_i + f_{i-1} psi_{i-1} = 0 on i0..i1 with
 *   psi_{i0-1} = psi_{i1+1} = 0.  Points with a (V_i - E_lo) > 1/2 at either
 *   end (E_lo = min V) are cut off, so f_i > 0 on the whole window and the
 *   problem is exactly H psi = E psi with H = diag(V) - B^{-1} D2 / (2 mu h^2)
 *   symmetric (B = I + D2/12).
 */
#ifndef EPSEON_NUMEROV_ORACLE_H
#define EPSEON_NUMEROV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status bits (same values as the CUDA library's EPSCU_LEVEL_* codes) */
#define EO_OK 0
#define EO_MAXITER 1
#define EO_NONFINITE 2
#define EO_UNDER_RESOLVED 4
#define EO_NOT_FOUND 16
#define EO_BAD_INPUT 32

typedef struct eo_problem {
    const double* V;    /* [N] potential on the uniform grid (Hartree) */
    int32_t N;          /* grid points */
    double r_min;       /* first grid point (bohr) */
    double r_max;       /* last grid point (bohr) */
    double mu;          /* reduced mass (electron masses) */
    double e_cap;       /* top of the energy window (Hartree) */
    int32_t n_trial;    /* trial energies of the scan: E_j = E_lo + (j+1)(e_cap-E_lo)/n_trial */
    int32_t min_level;  /* first level reported */
    int32_t max_level;  /* last level reported; < 0 means every level below e_cap */
    double tol;         /* bisection width (Hartree), e.g. 1e-12 */
} eo_problem;

typedef struct eo_grid {
    double h;       /* grid step */
    double a;       /* mu h^2 / 6 */
    double e_lo;    /* min V over the grid */
    double delta;   /* trial-energy spacing */
    int32_t i0;     /* first interior point */
    int32_t i1;     /* last interior point */
    int32_t k_scan; /* twist index of the scan (argmin V on i0..i1) */
    int32_t n_bisect; /* bisection steps: smallest K with delta / 2^K <= tol */
    int32_t N;      /* grid points */
} eo_grid;

typedef struct eo_result {
    int32_t capacity;         /* entries available in the per-level arrays */
    int32_t n_total;          /* bound levels below e_cap (scan count at e_cap) */
    int32_t n_out;            /* levels written: min_level .. min(max_level, n_total-1) */
    int32_t status;           /* potential-wide status bits */
    double* energy;           /* [capacity] bisection result (plain method) */
    double* energy_polished;  /* [capacity] bisection continued to the last bit, or NULL */
    int32_t* nodes;           /* [capacity] nodes of the level's wavefunction, or NULL */
    int32_t* level_status;    /* [capacity] per-level status bits, or NULL */
    double* psi;              /* [capacity * N] normalised wavefunctions, or NULL */
    int32_t* counts;          /* [n_trial] scan counts, or NULL */
} eo_result;

/* Derive the discrete-problem constants.  Returns 0 or EO_BAD_INPUT. */
int eo_prepare(const eo_problem* p, eo_grid* g);

/* Number of eigenvalues of the discrete problem below E (twisted Sturm count
 * at index k, i0 <= k <= i1). */
int32_t eo_count(const double* V, const eo_grid* g, double E, int32_t k);

/* Outer classical turning point: largest i in [i0, i1] with V_i <= E, or
 * k_scan when there is none. */
int32_t eo_match_index(const double* V, const eo_grid* g, double E);

/* Match point used for wavefunctions and Cooley corrections: the peak of
 * |psi| of the solution stitched at the outer turning point (clamped to
 * i0+1..i1-1). */
int32_t eo_match_point(const double* V, const eo_grid* g, double E);

/* One Cooley pass at E (match point k, or eo_match_point): returns the Newton
 * correction dE (E + dE is the improved energy) and the node count of the
 * stitched solution. */
double eo_cooley_pass(const double* V, const eo_grid* g, double E, int32_t* nodes);
double eo_cooley_pass_k(const double* V, const eo_grid* g, double E, int32_t k, int32_t* nodes);

/* Normalised wavefunction at E (sum psi^2 h = 1, psi > 0 next to the inner
 * wall), written to psi[0..N-1] (zero outside i0..i1). */
void eo_wavefunction(const double* V, const eo_grid* g, double E, double* psi);

/* Scan counts at the n_trial trial energies. */
void eo_scan(const double* V, const eo_grid* g, int32_t n_trial, int32_t* counts);

/* Solve one potential (single thread). Returns the potential status. */
int eo_solve(const eo_problem* p, eo_result* r);

/* Solve a batch over n_threads threads (0: all online cores). Returns the OR
 * of the potential status words. */
int eo_solve_batch(const eo_problem* p, eo_result* r, int32_t n, int32_t n_threads);

#ifdef __cplusplus
}
#endif
#endif
