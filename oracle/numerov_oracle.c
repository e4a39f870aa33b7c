/*
 * numerov_oracle.c -- FP64 CPU oracle for the vibrational-level solver.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
 * product path never uses it.  Parity with the reference is UNPINNED: the
 * reference's algorithm slot (VibwaAlgorithm<FP>::run, cpp/gpu/include/epseon/
 * gpu/algorithms/vibwa.hpp:605-637) computes nothing.  See numerov_oracle.h for
 * the discrete problem and the published methods restated here.
 *
 * Build with -ffp-contract=off: every fused multiply-add below is written
 * explicitly with fma() so that the arithmetic is the same sequence of
 * correctly rounded operations as the CUDA FP64 kernels (which use the same
 * expressions with __fma_rn / __dmul_rn / __dadd_rn), on x86 and on Arm.
 */
#include "numerov_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* Renormalise the projective state every RENORM steps by a power of two.
 * Scaling by 2^e is exact, so where it happens does not change any result. */
#define RENORM 32

static inline void renorm2(double* x, double* y, double* s) {
    double m = fabs(*x) > fabs(*y) ? fabs(*x) : fabs(*y);
    if (m == 0.0 || !isfinite(m)) return;
    int e;
    (void)frexp(m, &e);
    *x = ldexp(*x, -e);
    *y = ldexp(*y, -e);
    if (s) *s = ldexp(*s, -2 * e);
}

/* Order of operations shared with the CUDA FP64 kernels (numerov_step64). */
static inline void numerov_step(double aE, double w, double* A, double* B) {
    double T = aE - w;
    double f = 1.0 + T;
    double g = fma(-10.0, T, 2.0);
    double An = fma(g, *A, -(f * *B));
    *B = f * *A;
    *A = An;
}

int eo_prepare(const eo_problem* p, eo_grid* g) {
    memset(g, 0, sizeof(*g));
    if (!p || !p->V || p->N < 5 || !(p->mu > 0.0) || !(p->r_max > p->r_min) || p->n_trial < 1)
        return EO_BAD_INPUT;
    const double* V = p->V;
    const int32_t N = p->N;
    double vmin = V[0];
    for (int32_t i = 0; i < N; ++i) {
        if (!isfinite(V[i])) return EO_BAD_INPUT | EO_NONFINITE;
        if (V[i] < vmin) vmin = V[i];
    }
    g->N = N;
    g->h = (p->r_max - p->r_min) / (double)(N - 1);
    g->a = p->mu * g->h * g->h / 6.0;
    g->e_lo = vmin;
    /* admissible: a (V_i - E_lo) <= 1/2, i.e. T_i(E_lo) >= -1/2 */
    int32_t first = -1, last = -1;
    for (int32_t i = 0; i < N; ++i) {
        if (g->a * (V[i] - vmin) <= 0.5) {
            if (first < 0) first = i;
            last = i;
        }
    }
    g->i0 = first < 1 ? 1 : first;
    g->i1 = last > N - 2 ? N - 2 : last;
    if (g->i1 - g->i0 < 2) return EO_BAD_INPUT;
    int32_t k = g->i0;
    for (int32_t i = g->i0; i <= g->i1; ++i)
        if (V[i] < V[k]) k = i;
    g->k_scan = k;
    if (!(p->e_cap > vmin)) return EO_BAD_INPUT;
    g->delta = (p->e_cap - vmin) / (double)p->n_trial;
    double tol = p->tol > 0.0 ? p->tol : 1e-12;
    int32_t K = 0;
    for (double w = g->delta; w > tol && K < 200; w *= 0.5) ++K;
    g->n_bisect = K;
    return EO_OK;
}

int32_t eo_count(const double* V, const eo_grid* g, double E, int32_t k) {
    const double a = g->a;
    const double aE = a * E;
    int32_t nodes = 0;
    double A = 1.0, B = 0.0;
    int32_t s = 0;
    for (int32_t i = g->i0; i < k; ++i) {
        double An_prev = A;
        numerov_step(aE, a * V[i], &A, &B);
        nodes += (A < 0.0) != (An_prev < 0.0);
        if (++s == RENORM) { s = 0; renorm2(&A, &B, NULL); }
    }
    double C = 1.0, D = 0.0;
    s = 0;
    for (int32_t i = g->i1; i > k; --i) {
        double Cp = C;
        numerov_step(aE, a * V[i], &C, &D);
        nodes += (C < 0.0) != (Cp < 0.0);
        if (++s == RENORM) { s = 0; renorm2(&C, &D, NULL); }
    }
    /* twisted pivot gamma_k = c_k - u_{k-1}/u_k - v_{k+1}/v_k; only its sign */
    double Tk = aE - a * V[k];
    double fk = 1.0 + Tk;
    double gk = fma(-10.0, Tk, 2.0);
    double AC = A * C;
    double num = fma(gk, AC, -(fk * fma(B, C, D * A)));
    nodes += (num < 0.0) != (AC < 0.0);
    return nodes;
}

int32_t eo_match_index(const double* V, const eo_grid* g, double E) {
    for (int32_t i = g->i1; i >= g->i0; --i)
        if (V[i] <= E) return i;
    return g->k_scan;
}

/* The projective state after step i is s_{i+1} (u_{i+1}, u_i) with the scale
 * s_{i+1} = f_{i0} ... f_i, so psi_i = u_i / f_i = A_i / (s_i f_i).  Sums of
 * psi^2 are carried in the current scale without any division:
 *   S_{i+1} = f_i^2 S_i + A_i^2   (S_i = s_i^2 sum_{j<i} psi_j^2),
 * and sum_{j<k} (psi_j / psi_k)^2 = S_k f_k^2 / A_k^2 at the end. */
double eo_cooley_pass(const double* V, const eo_grid* g, double E, int32_t* nodes_out) {
    return eo_cooley_pass_k(V, g, E, eo_match_point(V, g, E), nodes_out);
}

double eo_cooley_pass_k(const double* V, const eo_grid* g, double E, int32_t k, int32_t* nodes_out) {
    const double a = g->a;
    const double aE = a * E;
    int32_t nodes = 0, s = 0;
    double A = 1.0, B = 0.0, S1 = 0.0;
    for (int32_t i = g->i0; i < k; ++i) {
        double f = 1.0 + (aE - a * V[i]);
        S1 = fma(f * f, S1, A * A);
        double Ap = A;
        numerov_step(aE, a * V[i], &A, &B);
        nodes += (A < 0.0) != (Ap < 0.0);
        if (++s == RENORM) { s = 0; renorm2(&A, &B, &S1); }
    }
    double C = 1.0, D = 0.0, S2 = 0.0;
    s = 0;
    for (int32_t i = g->i1; i > k; --i) {
        double f = 1.0 + (aE - a * V[i]);
        S2 = fma(f * f, S2, C * C);
        double Cp = C;
        numerov_step(aE, a * V[i], &C, &D);
        nodes += (C < 0.0) != (Cp < 0.0);
        if (++s == RENORM) { s = 0; renorm2(&C, &D, &S2); }
    }
    double Tk = aE - a * V[k];
    double fk = 1.0 + Tk;
    double gk = fma(-10.0, Tk, 2.0);
    double fk2 = fk * fk;
    double norm = fk2 * (S1 / (A * A) + S2 / (C * C)) + 1.0;
    double gamma = gk / fk - B / A - D / C;
    if (nodes_out) *nodes_out = nodes;
    return gamma * fk2 / (12.0 * a * norm);
}

/* One side of the wavefunction: raw[i] * 2^ex[i] is proportional to psi_i. */
static void wf_side(const double* V, const eo_grid* g, double aE, int32_t from, int32_t to, int32_t dir,
                    double* raw, int32_t* ex, double* raw_k, int32_t* ex_k) {
    const double a = g->a;
    double A = 1.0, B = 0.0, sc = 1.0;
    int32_t eA = 0, eS = 0, s = 0;
    for (int32_t i = from; i != to; i += dir) {
        double f = 1.0 + (aE - a * V[i]);
        raw[i] = A / (sc * f);
        ex[i] = eA - eS;
        numerov_step(aE, a * V[i], &A, &B);
        sc *= f;
        if (++s == RENORM) {
            s = 0;
            double m = fabs(A) > fabs(B) ? fabs(A) : fabs(B);
            int e;
            (void)frexp(m, &e);
            A = ldexp(A, -e);
            B = ldexp(B, -e);
            eA += e;
            (void)frexp(sc, &e);
            sc = ldexp(sc, -e);
            eS += e;
        }
    }
    double fk = 1.0 + (aE - a * V[to]);
    *raw_k = A / (sc * fk);
    *ex_k = eA - eS;
}

/* Stitched wavefunction at E with match index k (sum psi^2 h = 1, positive
 * next to the inner wall); returns the index of max |psi|. */
static int32_t wavefunction_k(const double* V, const eo_grid* g, double E, int32_t k, double* psi,
                              double* peak_ratio) {
    const double aE = g->a * E;
    for (int32_t i = 0; i < g->N; ++i) psi[i] = 0.0;
    double* raw = (double*)malloc(sizeof(double) * (size_t)g->N);
    int32_t* ex = (int32_t*)malloc(sizeof(int32_t) * (size_t)g->N);
    double pko, pki;
    int32_t exo, exi;
    wf_side(V, g, aE, g->i0, k, +1, raw, ex, &pko, &exo);
    wf_side(V, g, aE, g->i1, k, -1, raw, ex, &pki, &exi);
    /* tilde-psi: 1 at k, continuous from both sides */
    double sum = 1.0, best = 1.0;
    int32_t arg = k;
    for (int32_t i = g->i0; i < k; ++i) {
        raw[i] = ldexp(raw[i] / pko, ex[i] - exo);
        sum += raw[i] * raw[i];
        if (fabs(raw[i]) > best) { best = fabs(raw[i]); arg = i; }
    }
    for (int32_t i = g->i1; i > k; --i) {
        raw[i] = ldexp(raw[i] / pki, ex[i] - exi);
        sum += raw[i] * raw[i];
        if (fabs(raw[i]) > best) { best = fabs(raw[i]); arg = i; }
    }
    raw[k] = 1.0;
    /* sum psi^2 h = 1; positive next to the inner wall, where the outward
     * solution (started at +1) has not changed sign yet */
    double ck = 1.0 / sqrt(g->h * sum);
    if (pko < 0.0) ck = -ck;
    for (int32_t i = g->i0; i <= g->i1; ++i) psi[i] = raw[i] * ck;
    free(raw);
    free(ex);
    if (peak_ratio) *peak_ratio = best;
    return arg;
}

static int32_t clamp_inner(const eo_grid* g, int32_t k) {
    if (k < g->i0 + 1) k = g->i0 + 1;
    if (k > g->i1 - 1) k = g->i1 - 1;
    return k;
}

/* Match point: the twist index k minimising |gamma_k(E)| over i0+1..i1-1,
 * gamma_k = c_k - u_{k-1}/u_k - v_{k+1}/v_k from one full outward and one full
 * inward sweep (the twisted-factorisation rule of Dhillon and Parlett's MRRR:
 * at an eigenvalue |gamma_k| is smallest where the eigenvector is largest).
 * Matching there keeps Cooley's correction quadratic and the stitched vector
 * accurate, also for levels separated from the turning point by a barrier. */
int32_t eo_match_point(const double* V, const eo_grid* g, double E) {
    const double a = g->a, aE = a * E;
    double* rho = (double*)malloc(sizeof(double) * (size_t)g->N);
    double A = 1.0, B = 0.0;
    int32_t s = 0;
    for (int32_t i = g->i0; i < g->i1; ++i) {
        rho[i] = B / A; /* u_{i-1} / u_i */
        numerov_step(aE, a * V[i], &A, &B);
        if (++s == RENORM) { s = 0; renorm2(&A, &B, NULL); }
    }
    rho[g->i1] = B / A;
    double C = 1.0, D = 0.0, best = INFINITY;
    int32_t kbest = clamp_inner(g, eo_match_index(V, g, E));
    s = 0;
    for (int32_t i = g->i1; i > g->i0; --i) {
        /* here (C, D) ~ (v_i, v_{i+1}) */
        if (i <= g->i1 - 1) {
            const double Ti = aE - a * V[i];
            const double gam = fabs((2.0 - 10.0 * Ti) / (1.0 + Ti) - rho[i] - D / C);
            if (gam < best) { best = gam; kbest = i; }
        }
        numerov_step(aE, a * V[i], &C, &D);
        if (++s == RENORM) { s = 0; renorm2(&C, &D, NULL); }
    }
    free(rho);
    return clamp_inner(g, kbest);
}

void eo_wavefunction(const double* V, const eo_grid* g, double E, double* psi) {
    (void)wavefunction_k(V, g, E, eo_match_point(V, g, E), psi, NULL);
}

static inline double trial_energy(const eo_grid* g, int32_t j) {
    /* E_j = E_lo + (j+1) delta, two roundings, no contraction */
    double t = (double)(j + 1) * g->delta;
    return g->e_lo + t;
}

void eo_scan(const double* V, const eo_grid* g, int32_t n_trial, int32_t* counts) {
    for (int32_t j = 0; j < n_trial; ++j) counts[j] = eo_count(V, g, trial_energy(g, j), g->k_scan);
}

/* first j with counts[j] > v (counts are non-decreasing); n_trial if none */
static int32_t bracket_of(const int32_t* counts, int32_t n_trial, int32_t v) {
    int32_t lo = 0, hi = n_trial;
    while (lo < hi) {
        int32_t mid = lo + (hi - lo) / 2;
        if (counts[mid] > v) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

static void solve_level(const eo_problem* p, const eo_grid* g, const int32_t* counts, eo_result* r,
                        int32_t v) {
    const int32_t slot = v - p->min_level;
    const int32_t j = bracket_of(counts, p->n_trial, v);
    int32_t st = EO_OK;
    double E;
    if (j >= p->n_trial) {
        st |= EO_NOT_FOUND;
        E = NAN;
    } else {
        double lo = j == 0 ? g->e_lo : trial_energy(g, j - 1);
        double hi = trial_energy(g, j);
        for (int32_t it = 0; it < g->n_bisect; ++it) {
            double mid = 0.5 * (lo + hi);
            if (eo_count(p->V, g, mid, eo_match_index(p->V, g, mid)) > v) hi = mid;
            else lo = mid;
        }
        E = 0.5 * (lo + hi);
        if (r->energy_polished) {
            /* the FP64 "truth": keep bisecting until the bracket stops shrinking */
            for (int32_t it = 0; it < 64; ++it) {
                double mid = 0.5 * (lo + hi);
                if (!(mid > lo && mid < hi)) break;
                if (eo_count(p->V, g, mid, eo_match_index(p->V, g, mid)) > v) hi = mid;
                else lo = mid;
            }
            r->energy_polished[slot] = 0.5 * (lo + hi);
        }
    }
    r->energy[slot] = E;
    int32_t nodes = -1;
    if (!(st & EO_NOT_FOUND)) {
        (void)eo_cooley_pass(p->V, g, E, &nodes);
        if (nodes != v) st |= EO_NOT_FOUND;
        if (r->psi) eo_wavefunction(p->V, g, E, r->psi + (size_t)slot * (size_t)p->N);
    } else if (r->energy_polished) {
        r->energy_polished[slot] = NAN;
    }
    if (r->nodes) r->nodes[slot] = nodes;
    if (r->level_status) r->level_status[slot] = st;
}

static int finish_prepare(const eo_problem* p, const eo_grid* g, eo_result* r, int32_t* counts) {
    r->n_total = counts[p->n_trial - 1];
    int32_t last = p->max_level < 0 ? r->n_total - 1 : p->max_level;
    if (last > r->n_total - 1) last = r->n_total - 1;
    int32_t n_out = last - p->min_level + 1;
    if (n_out < 0) n_out = 0;
    if (n_out > r->capacity) n_out = r->capacity;
    r->n_out = n_out;
    double kmax = sqrt(2.0 * p->mu * (p->e_cap - g->e_lo));
    if (kmax * g->h > 1.0) r->status |= EO_UNDER_RESOLVED;
    if (r->psi)
        memset(r->psi, 0, sizeof(double) * (size_t)r->capacity * (size_t)p->N);
    return r->status;
}

int eo_solve(const eo_problem* p, eo_result* r) {
    eo_grid g;
    r->n_total = r->n_out = 0;
    r->status = eo_prepare(p, &g);
    if (r->status) return r->status;
    int32_t* counts = r->counts ? r->counts : (int32_t*)malloc(sizeof(int32_t) * (size_t)p->n_trial);
    eo_scan(p->V, &g, p->n_trial, counts);
    finish_prepare(p, &g, r, counts);
    for (int32_t s = 0; s < r->n_out; ++s) solve_level(p, &g, counts, r, p->min_level + s);
    if (!r->counts) free(counts);
    return r->status;
}

/* ---------------- multi-threaded batch ---------------- */

#define SCAN_CHUNK 32

typedef struct {
    int32_t p;
    int32_t a, b; /* scan: trial range [a, b); level: v in a */
} task_t;

typedef struct {
    const eo_problem* probs;
    eo_result* res;
    eo_grid* grids;
    int32_t** counts;
    task_t* tasks;
    int32_t n_tasks;
    int phase; /* 0 scan, 1 levels */
    atomic_int next;
} batch_t;

static void* worker(void* arg) {
    batch_t* b = (batch_t*)arg;
    for (;;) {
        int t = atomic_fetch_add(&b->next, 1);
        if (t >= b->n_tasks) break;
        task_t tk = b->tasks[t];
        const eo_problem* p = &b->probs[tk.p];
        const eo_grid* g = &b->grids[tk.p];
        if (b->phase == 0) {
            for (int32_t j = tk.a; j < tk.b; ++j)
                b->counts[tk.p][j] = eo_count(p->V, g, trial_energy(g, j), g->k_scan);
        } else {
            solve_level(p, g, b->counts[tk.p], &b->res[tk.p], tk.a);
        }
    }
    return NULL;
}

static void run_phase(batch_t* b, int32_t n_threads) {
    atomic_store(&b->next, 0);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
    int32_t started = 0;
    for (int32_t t = 0; t < n_threads; ++t)
        if (pthread_create(&th[t], NULL, worker, b) == 0) ++started;
    if (started == 0) worker(b);
    for (int32_t t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
}

int eo_solve_batch(const eo_problem* probs, eo_result* res, int32_t n, int32_t n_threads) {
    if (n_threads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        n_threads = c > 0 ? (int32_t)c : 1;
    }
    batch_t b;
    memset(&b, 0, sizeof(b));
    b.probs = probs;
    b.res = res;
    b.grids = (eo_grid*)calloc((size_t)n, sizeof(eo_grid));
    b.counts = (int32_t**)calloc((size_t)n, sizeof(int32_t*));
    size_t n_scan = 0;
    for (int32_t i = 0; i < n; ++i) {
        res[i].n_total = res[i].n_out = 0;
        res[i].status = eo_prepare(&probs[i], &b.grids[i]);
        if (res[i].status) continue;
        b.counts[i] = res[i].counts ? res[i].counts
                                    : (int32_t*)malloc(sizeof(int32_t) * (size_t)probs[i].n_trial);
        n_scan += (size_t)(probs[i].n_trial + SCAN_CHUNK - 1) / SCAN_CHUNK;
    }
    b.tasks = (task_t*)malloc(sizeof(task_t) * (n_scan + 1));
    b.n_tasks = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (res[i].status) continue;
        for (int32_t j = 0; j < probs[i].n_trial; j += SCAN_CHUNK) {
            task_t t = {i, j, j + SCAN_CHUNK < probs[i].n_trial ? j + SCAN_CHUNK : probs[i].n_trial};
            b.tasks[b.n_tasks++] = t;
        }
    }
    b.phase = 0;
    run_phase(&b, n_threads);
    free(b.tasks);
    size_t n_lev = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (res[i].status) continue;
        finish_prepare(&probs[i], &b.grids[i], &res[i], b.counts[i]);
        n_lev += (size_t)res[i].n_out;
    }
    b.tasks = (task_t*)malloc(sizeof(task_t) * (n_lev + 1));
    b.n_tasks = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (res[i].status & EO_BAD_INPUT) continue;
        for (int32_t s = 0; s < res[i].n_out; ++s) {
            task_t t = {i, probs[i].min_level + s, 0};
            b.tasks[b.n_tasks++] = t;
        }
    }
    b.phase = 1;
    run_phase(&b, n_threads);
    free(b.tasks);
    int st = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (b.counts[i] && b.counts[i] != res[i].counts) free(b.counts[i]);
        st |= res[i].status;
    }
    free(b.counts);
    free(b.grids);
    return st;
}
