/* TEST INFRASTRUCTURE ONLY -- the CPU oracle (see ocsl_oracle.h).
 *
 * Restates OpenCSLSolver's cmatrix_solver.cpp in C.  Each function cites the
 * reference lines it follows.  OpenMP is used the way the reference uses it
 * (parallel loops over rows), so the same code serves as the timed CPU
 * baseline; every parallel loop writes disjoint outputs and every reduction
 * follows the fixed tile order, so results do not depend on the thread count.
 */
#include "ocsl_oracle.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define PHANTOM UINT64_MAX

void orc_set_threads(int threads)
{
    omp_set_dynamic(0);
    omp_set_num_threads(threads > 0 ? threads : 1);
}

/* ---------------------------------------------------------------- reductions */

/* The 32-lane xor butterfly used by the GPU's __shfl_xor_sync reduction. */
static double butterfly32(const double* v_in)
{
    double v[32], w[32];
    memcpy(v, v_in, sizeof v);
    for (int off = 16; off >= 1; off >>= 1) {
        for (int i = 0; i < 32; ++i) w[i] = v[i] + v[i ^ off];
        memcpy(v, w, sizeof v);
    }
    return v[0];
}

/* 256 lane values -> one sum: butterfly per 32-lane group, groups in order. */
static double lanes_to_sum(const double* lanes)
{
    double s = butterfly32(lanes);
    for (int g = 1; g < ORC_LANES / 32; ++g) s = s + butterfly32(lanes + 32 * g);
    return s;
}

static double tile_dot(size_t n, size_t tile, const double* x, const double* y)
{
    double lanes[ORC_LANES];
    const size_t base = tile * ORC_TILE;
    for (int t = 0; t < ORC_LANES; ++t) {
        double acc = 0.0;
        for (int j = 0; j < ORC_TILE / ORC_LANES; ++j) {
            size_t e = base + (size_t)j * ORC_LANES + (size_t)t;
            if (e < n) acc = fma(x[e], y[e], acc);
        }
        lanes[t] = acc;
    }
    return lanes_to_sum(lanes);
}

static double reduce_partials(size_t P, const double* part)
{
    double lanes[ORC_LANES];
    for (int t = 0; t < ORC_LANES; ++t) {
        double acc = 0.0;
        for (size_t k = (size_t)t; k < P; k += ORC_LANES) acc = acc + part[k];
        lanes[t] = acc;
    }
    return lanes_to_sum(lanes);
}

double orc_dot(size_t n, const double* x, const double* y)
{
    if (n == 0) return 0.0;
    const size_t P = (n + ORC_TILE - 1) / ORC_TILE;
    double* part = (double*)malloc(P * sizeof(double));
    long long p;
#pragma omp parallel for schedule(static)
    for (p = 0; p < (long long)P; ++p) part[p] = tile_dot(n, (size_t)p, x, y);
    double s = reduce_partials(P, part);
    free(part);
    return s;
}

static double tile_sum(size_t n, size_t tile, const double* x, int absolute)
{
    double lanes[ORC_LANES];
    const size_t base = tile * ORC_TILE;
    for (int t = 0; t < ORC_LANES; ++t) {
        double acc = 0.0;
        for (int j = 0; j < ORC_TILE / ORC_LANES; ++j) {
            size_t e = base + (size_t)j * ORC_LANES + (size_t)t;
            if (e < n) acc = acc + (absolute ? fabs(x[e]) : x[e]);
        }
        lanes[t] = acc;
    }
    return lanes_to_sum(lanes);
}

/* cmatrix_solver.cpp:244-252 sum and :255-263 ABSsum, in the tile order. */
double orc_sum(size_t n, const double* x, int absolute)
{
    if (n == 0) return 0.0;
    const size_t P = (n + ORC_TILE - 1) / ORC_TILE;
    double* part = (double*)malloc(P * sizeof(double));
    for (size_t p = 0; p < P; ++p) part[p] = tile_sum(n, p, x, absolute);
    double s = reduce_partials(P, part);
    free(part);
    return s;
}

/* :266-272 product */
void orc_product(size_t n, const double* x, const double* y, double* out)
{
    for (size_t i = 0; i < n; ++i) out[i] = x[i] * y[i];
}

/* :275-335 axpy; y == NULL is the one-vector overload out = a x.  The
 * reference's a*x + y forms are contracted under -ffast-math: fma here. */
void orc_axpy(size_t n, double a, const double* x, double b, const double* y, double* out)
{
    for (size_t i = 0; i < n; ++i) {
        if (!y) {
            out[i] = a * x[i];
        } else if (b == 1.0) {
            out[i] = a == 1.0 ? x[i] + y[i] : (a == -1.0 ? y[i] - x[i] : fma(a, x[i], y[i]));
        } else if (b == -1.0) {
            out[i] = a == 1.0 ? x[i] - y[i] : (a == -1.0 ? -y[i] - x[i] : fma(a, x[i], -y[i]));
        } else {
            out[i] = fma(a, x[i], b * y[i]);
        }
    }
}

double orc_dot_seq(size_t n, const double* x, const double* y)
{
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s = fma(x[i], y[i], s);
    return s;
}

/* ---------------------------------------------------------------- SpMV */

/* One CSR row in storage order: dum = fma(a_ij, x_j, dum) from 0.0
 * (cmatrix_solver.cpp:346-350).  The phantom column is skipped: the reference
 * multiplies its exact 0 by x[-1], which adds nothing for finite x[-1]. */
static inline double row_dot(const uint64_t* rp, const uint64_t* col, const double* val,
                             size_t n, size_t i, const double* x)
{
    double dum = 0.0;
    for (uint64_t q = rp[i]; q < rp[i + 1]; ++q) {
        uint64_t c = col[q];
        if (c < n) dum = fma(val[q], x[c], dum);
    }
    return dum;
}

void orc_gemv(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
              const double* x, int mode, double a, const double* z, double* y)
{
    long long i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < (long long)n; ++i) {
        double dum = row_dot(rp, col, val, n, (size_t)i, x);
        if (mode == 0) y[i] = dum;                      /* gemv(1, A, x, y)        */
        else if (mode == 1) y[i] = z[i] - dum;          /* gemv(-1, A, x, 1, z, y) */
        else y[i] = fma(a, dum, z[i]);                  /* gemv(a, A, x, 1, z, y)  */
    }
}

/* ---------------------------------------------------------------- ILU */

int orc_extract_diag(size_t n, const uint64_t* rp, const uint64_t* col, int32_t* diag)
{
    int ok = 0;
    for (size_t i = 0; i < n; ++i) {
        diag[i] = -1;
        for (uint64_t q = rp[i]; q < rp[i + 1]; ++q)
            if (col[q] == i) { diag[i] = (int32_t)q; break; }
        if (diag[i] < 0) ok = -1;
    }
    return ok;
}

/* CCSR::get_element (cmatrix_solver.cpp:47-55): linear search of row i. */
static inline double get_element(const uint64_t* rp, const uint64_t* col, const double* M,
                                 uint64_t i, uint64_t j, size_t n)
{
    if (i >= n) return 0.0;
    for (uint64_t q = rp[i]; q < rp[i + 1]; ++q)
        if (col[q] == j) return M[q];
    return 0.0;
}

/* One Jacobi sweep (cmatrix_solver.cpp:525-549): lower entries
 *   Mnew_ij = (A_ij - sum_{k before j} M_ik M_(k,j)) / M_(j,j)
 * and diagonal / upper / phantom entries
 *   Mnew_ij = A_ij - sum_{k before diag} M_ik M_(k,j),
 * every product reading the previous sweep's M. */
static void ilu_sweep(size_t n, const uint64_t* rp, const uint64_t* col, const double* A,
                      const int32_t* diag, const double* M, double* Mnew)
{
    long long ii;
#pragma omp parallel for schedule(static)
    for (ii = 0; ii < (long long)n; ++ii) {
        const uint64_t i = (uint64_t)ii;
        for (uint64_t j = rp[i]; j < rp[i + 1]; ++j) {
            const uint64_t cj = col[j];
            double dum = 0.0;
            if (i > cj) {
                for (uint64_t k = rp[i]; k < j; ++k)
                    dum = fma(M[k], get_element(rp, col, M, col[k], cj, n), dum);
                Mnew[j] = (A[j] - dum) / M[diag[cj]];
            } else {
                for (uint64_t k = rp[i]; k < (uint64_t)diag[i]; ++k)
                    dum = fma(M[k], get_element(rp, col, M, col[k], cj, n), dum);
                Mnew[j] = A[j] - dum;
            }
        }
    }
}

void orc_ilu_fixed_point(size_t n, const uint64_t* rp, const uint64_t* col, const double* A,
                         const int32_t* diag, int sweeps, double* M)
{
    const size_t nnz = n ? (size_t)rp[n] : 0;
    double* Mold = (double*)malloc((nnz ? nnz : 1) * sizeof(double));
    memcpy(M, A, nnz * sizeof(double)); /* M.copy_same_structure(matrix), :702 */
    for (int s = 0; s < sweeps; ++s) {
        memcpy(Mold, M, nnz * sizeof(double));
        ilu_sweep(n, rp, col, A, diag, Mold, M);
    }
    free(Mold);
}

void orc_forsub(size_t n, const uint64_t* rp, const uint64_t* col, const double* M,
                const int32_t* diag, const double* b, double* y)
{
    (void)n;
    for (size_t i = 0; i < n; ++i) {
        double sum = 0.0;
        for (uint64_t q = rp[i]; q < (uint64_t)diag[i]; ++q) sum = fma(M[q], y[col[q]], sum);
        y[i] = b[i] - sum;
    }
}

void orc_backsub(size_t n, const uint64_t* rp, const uint64_t* col, const double* M,
                 const int32_t* diag, const double* y, double* x)
{
    for (size_t ii = n; ii-- > 0;) {
        double sum = 0.0;
        for (uint64_t q = (uint64_t)diag[ii] + 1; q < rp[ii + 1]; ++q)
            if (col[q] < n) sum = fma(M[q], x[col[q]], sum);
        x[ii] = (y[ii] - sum) / M[diag[ii]];
    }
}

/* ---------------------------------------------------------------- helpers */

static double* dalloc(size_t n)
{
    double* p = (double*)calloc(n ? n : 1, sizeof(double));
    return p;
}

/* ---------------------------------------------------------------- CG_solve */

double orc_cg_ref(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                  const double* b, double* x, int* iters)
{
    const int n_iter = 4;            /* :637 */
    const double res_limit = 1.0e-6; /* :638 */
    double* r = dalloc(n);
    double* p = dalloc(n);
    double* Ap = dalloc(n);
    double* rn = dalloc(n);
    double res = 0.0;
    int it_done = 0;
    long long i;

    orc_gemv(n, rp, col, val, x, 1, 0.0, b, r); /* r = b - A x, :652 */
    memcpy(p, r, n * sizeof(double));           /* p = r,       :655 */
    double rr = orc_dot(n, r, r);
    for (int it = 0; it < n_iter; ++it) {
        orc_gemv(n, rp, col, val, p, 0, 0.0, NULL, Ap);       /* :659 */
        const double a = rr / (orc_dot(n, p, Ap) + 1.0e-40);  /* :660 */
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) {
            x[i] = fma(a, p[i], x[i]);     /* :662-663 */
            rn[i] = fma(-a, Ap[i], r[i]);  /* :665, A p recomputed identically */
        }
        res = orc_dot(n, rn, rn);          /* :667 */
        it_done = it + 1;
        if (res < res_limit) break;        /* :669-670 */
        const double beta = res / (rr + 1.0e-40); /* :672 */
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) p[i] = fma(beta, p[i], rn[i]); /* :674 */
        memcpy(r, rn, n * sizeof(double)); /* :676-677 */
        rr = res;
    }
    if (iters) *iters = it_done;
    free(r); free(p); free(Ap); free(rn);
    return res;
}

/* ---------------------------------------------------------------- ILU_BICGSTAB_solve */

double orc_bicgstab_ref(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                        const double* b, double* x, int* iters)
{
    const int n_iter = 3;              /* :684 */
    const double res_limit = 1.0e-20;  /* :685 */
    const size_t nnz = n ? (size_t)rp[n] : 0;
    double omega = 1.0, alpha = 1.0, rhon = 1.0, res = 0.0; /* :689 */
    double *r = dalloc(n), *p = dalloc(n), *v = dalloc(n), *r0 = dalloc(n), *s = dalloc(n);
    double *dum = dalloc(n), *h = dalloc(n), *t = dalloc(n), *y = dalloc(n), *z = dalloc(n);
    double *dum2 = dalloc(n), *M = dalloc(nnz);
    int32_t* diag = (int32_t*)malloc((n ? n : 1) * sizeof(int32_t));
    int it_done = 0;
    long long i;

    orc_extract_diag(n, rp, col, diag);
    orc_ilu_fixed_point(n, rp, col, val, diag, 3, M);  /* :702-704 */
    orc_gemv(n, rp, col, val, x, 1, 0.0, b, r);          /* :708 */
    memcpy(r0, r, n * sizeof(double));                   /* :710 */
    const double bb = orc_dot(n, b, b);
    for (int it = 0; it < n_iter; ++it) {
        rhon = orc_dot(n, r0, r);                        /* :714 */
        /* :718-720: dum = p - omega v; p = r + omega dum (the reference uses
         * omega where its comment says beta; beta is unused). */
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) {
            dum[i] = fma(-omega, v[i], p[i]);
            p[i] = fma(omega, dum[i], r[i]);
        }
        orc_forsub(n, rp, col, M, diag, p, dum);         /* :722 */
        orc_backsub(n, rp, col, M, diag, dum, y);        /* :723 */
        orc_gemv(n, rp, col, val, y, 0, 0.0, NULL, v);   /* :725 */
        alpha = rhon / (orc_dot(n, r0, v) + DBL_MIN);    /* :727-728 */
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) h[i] = fma(alpha, y[i], x[i]); /* :731 */
        res = orc_dot(n, r, r) / bb + DBL_MIN;           /* :733, r from the start of the iteration */
        if (res < res_limit) break;                      /* :734-735, x not updated */
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) s[i] = fma(-alpha, v[i], r[i]); /* :738 */
        orc_forsub(n, rp, col, M, diag, s, dum2);        /* :741 and :747 (identical) */
        orc_backsub(n, rp, col, M, diag, dum2, z);       /* :742 */
        orc_gemv(n, rp, col, val, z, 0, 0.0, NULL, t);   /* :744 */
        orc_forsub(n, rp, col, M, diag, t, dum);         /* :746 */
        omega = orc_dot(n, dum, dum2) / (orc_dot(n, dum, dum) + 1.0e-40); /* :750 */
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) {
            x[i] = fma(omega, z[i], h[i]);               /* :753 */
            r[i] = fma(-omega, t[i], s[i]);              /* :756 */
        }
        it_done = it + 1;
    }
    if (iters) *iters = it_done;
    free(r); free(p); free(v); free(r0); free(s); free(dum); free(h); free(t); free(y);
    free(z); free(dum2); free(M); free(diag);
    return res;
}

/* ---------------------------------------------------------------- tolerance mode */

double orc_true_relres(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                       const double* b, const double* x)
{
    long double rr = 0.0L, bb = 0.0L;
    for (size_t i = 0; i < n; ++i) {
        long double acc = b[i];
        for (uint64_t q = rp[i]; q < rp[i + 1]; ++q)
            if (col[q] < n) acc -= (long double)val[q] * (long double)x[col[q]];
        rr += acc * acc;
        bb += (long double)b[i] * (long double)b[i];
    }
    if (bb == 0.0L) return rr == 0.0L ? 0.0 : INFINITY;
    return (double)sqrtl(rr / bb);
}

/* Backward sweep with a precomputed reciprocal diagonal (tolerance mode). */
static void backsub_dinv(size_t n, const uint64_t* rp, const uint64_t* col, const double* M,
                         const int32_t* diag, const double* dinv, const double* y, double* x)
{
    for (size_t ii = n; ii-- > 0;) {
        double sum = 0.0;
        for (uint64_t q = (uint64_t)diag[ii] + 1; q < rp[ii + 1]; ++q)
            if (col[q] < n) sum = fma(M[q], x[col[q]], sum);
        x[ii] = (y[ii] - sum) * dinv[ii];
    }
}

/* Preconditioned BiCGSTAB (van der Vorst 1992; Barrett et al., "Templates",
 * 1994, fig. 2.10) with the reference's ILU factor, FP64, to a relative
 * residual tol.  Recursive-residual convergence is confirmed with a true
 * residual; on disagreement the iteration restarts from the current x. */
int orc_bicgstab_tol(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                     const double* b, double* x, double tol, int maxit, int ilu_sweeps,
                     int* iters, double* relres)
{
    const size_t nnz = n ? (size_t)rp[n] : 0;
    double *r = dalloc(n), *rh = dalloc(n), *p = dalloc(n), *ph = dalloc(n), *v = dalloc(n);
    double *s = dalloc(n), *sh = dalloc(n), *t = dalloc(n), *tmp = dalloc(n), *M = dalloc(nnz);
    double* dinv = dalloc(n);
    int32_t* diag = (int32_t*)malloc((n ? n : 1) * sizeof(int32_t));
    long long i;
    int it = 0, converged = 0;
    const double tol2 = tol * tol;

    orc_extract_diag(n, rp, col, diag);
    orc_ilu_fixed_point(n, rp, col, val, diag, ilu_sweeps, M);
    for (size_t k = 0; k < n; ++k) dinv[k] = 1.0 / M[diag[k]];
    const double bb = orc_dot(n, b, b);
    if (bb == 0.0) {
        memset(x, 0, n * sizeof(double));
        converged = 1;
    }
    while (!converged && it < maxit) {
        orc_gemv(n, rp, col, val, x, 1, 0.0, b, r);
        double rr = orc_dot(n, r, r);
        if (rr <= tol2 * bb) { converged = 1; break; }
        memcpy(rh, r, n * sizeof(double));
        memcpy(p, r, n * sizeof(double));
        double rho = rr;
        int recursive_done = 0;
        while (it < maxit) {
            ++it;
            orc_forsub(n, rp, col, M, diag, p, tmp);
            backsub_dinv(n, rp, col, M, diag, dinv, tmp, ph);
            orc_gemv(n, rp, col, val, ph, 0, 0.0, NULL, v);
            const double sigma = orc_dot(n, rh, v);
            if (sigma == 0.0) break; /* breakdown: restart */
            const double alpha = rho / sigma;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) s[i] = fma(-alpha, v[i], r[i]);
            const double ss = orc_dot(n, s, s);
            if (ss <= tol2 * bb) {
#pragma omp parallel for schedule(static)
                for (i = 0; i < (long long)n; ++i) x[i] = fma(alpha, ph[i], x[i]);
                recursive_done = 1;
                break;
            }
            orc_forsub(n, rp, col, M, diag, s, tmp);
            backsub_dinv(n, rp, col, M, diag, dinv, tmp, sh);
            orc_gemv(n, rp, col, val, sh, 0, 0.0, NULL, t);
            const double ts = orc_dot(n, t, s), tt = orc_dot(n, t, t);
            const double omega = tt != 0.0 ? ts / tt : 0.0;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) {
                x[i] = fma(omega, sh[i], fma(alpha, ph[i], x[i]));
                r[i] = fma(-omega, t[i], s[i]);
            }
            rr = orc_dot(n, r, r);
            const double rho_new = orc_dot(n, rh, r);
            if (rr <= tol2 * bb) { recursive_done = 1; break; }
            if (omega == 0.0 || rho == 0.0) break; /* breakdown: restart */
            const double beta = (rho_new / rho) * (alpha / omega);
            rho = rho_new;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) p[i] = fma(beta, fma(-omega, v[i], p[i]), r[i]);
        }
        (void)recursive_done; /* the outer loop re-checks the true residual */
    }
    if (!converged && n) {
        orc_gemv(n, rp, col, val, x, 1, 0.0, b, r);
        converged = orc_dot(n, r, r) <= tol2 * bb;
    }
    if (iters) *iters = it;
    if (relres) *relres = orc_true_relres(n, rp, col, val, b, x);
    free(r); free(rh); free(p); free(ph); free(v); free(s); free(sh); free(t); free(tmp);
    free(M); free(dinv); free(diag);
    return converged ? 0 : 1;
}

/* Jacobi-preconditioned CG (Hestenes-Stiefel), FP64, for symmetric systems. */
int orc_pcg_tol(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                const double* b, double* x, double tol, int maxit, int* iters, double* relres)
{
    double *r = dalloc(n), *z = dalloc(n), *p = dalloc(n), *q = dalloc(n), *dinv = dalloc(n);
    int32_t* diag = (int32_t*)malloc((n ? n : 1) * sizeof(int32_t));
    long long i;
    int it = 0, converged = 0;
    const double tol2 = tol * tol;
    orc_extract_diag(n, rp, col, diag);
    for (size_t k = 0; k < n; ++k) dinv[k] = 1.0 / val[diag[k]];
    const double bb = orc_dot(n, b, b);
    if (bb == 0.0) {
        memset(x, 0, n * sizeof(double));
        converged = 1;
    }
    while (!converged && it < maxit) {
        orc_gemv(n, rp, col, val, x, 1, 0.0, b, r);
        double rr = orc_dot(n, r, r);
        if (rr <= tol2 * bb) { converged = 1; break; }
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) { z[i] = r[i] * dinv[i]; p[i] = z[i]; }
        double rz = orc_dot(n, r, z);
        while (it < maxit) {
            ++it;
            orc_gemv(n, rp, col, val, p, 0, 0.0, NULL, q);
            const double pq = orc_dot(n, p, q);
            if (pq == 0.0) break;
            const double alpha = rz / pq;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) {
                x[i] = fma(alpha, p[i], x[i]);
                r[i] = fma(-alpha, q[i], r[i]);
                z[i] = r[i] * dinv[i];
            }
            rr = orc_dot(n, r, r);
            const double rz_new = orc_dot(n, r, z);
            if (rr <= tol2 * bb) break;
            const double beta = rz_new / rz;
            rz = rz_new;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) p[i] = fma(beta, p[i], z[i]);
        }
        orc_gemv(n, rp, col, val, x, 1, 0.0, b, r);
        converged = orc_dot(n, r, r) <= tol2 * bb;
    }
    if (iters) *iters = it;
    if (relres) *relres = orc_true_relres(n, rp, col, val, b, x);
    free(r); free(z); free(p); free(q); free(dinv); free(diag);
    return converged ? 0 : 1;
}

/* ---------------------------------------------------------------- mixed precision */

static double dot32(size_t n, const float* a, const float* b)
{
    /* FP64 accumulation of exact FP32 products, tile order. */
    if (n == 0) return 0.0;
    const size_t P = (n + ORC_TILE - 1) / ORC_TILE;
    double* part = (double*)malloc(P * sizeof(double));
    long long pp;
#pragma omp parallel for schedule(static)
    for (pp = 0; pp < (long long)P; ++pp) {
        double lanes[ORC_LANES];
        const size_t base = (size_t)pp * ORC_TILE;
        for (int t = 0; t < ORC_LANES; ++t) {
            double acc = 0.0;
            for (int j = 0; j < ORC_TILE / ORC_LANES; ++j) {
                size_t e = base + (size_t)j * ORC_LANES + (size_t)t;
                if (e < n) acc = fma((double)a[e], (double)b[e], acc);
            }
            lanes[t] = acc;
        }
        part[pp] = lanes_to_sum(lanes);
    }
    double s = reduce_partials(P, part);
    free(part);
    return s;
}

static void spmv32(size_t n, const uint64_t* rp, const uint64_t* col, const float* val,
                   const float* x, float* y)
{
    long long i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < (long long)n; ++i) {
        float dum = 0.0f;
        for (uint64_t q = rp[i]; q < rp[i + 1]; ++q)
            if (col[q] < n) dum = fmaf(val[q], x[col[q]], dum);
        y[i] = dum;
    }
}

static void precond32(size_t n, const uint64_t* rp, const uint64_t* col, const float* M,
                      const int32_t* diag, const float* dinv, const float* in, float* tmp,
                      float* out)
{
    for (size_t i = 0; i < n; ++i) {
        float sum = 0.0f;
        for (uint64_t q = rp[i]; q < (uint64_t)diag[i]; ++q) sum = fmaf(M[q], tmp[col[q]], sum);
        tmp[i] = in[i] - sum;
    }
    for (size_t ii = n; ii-- > 0;) {
        float sum = 0.0f;
        for (uint64_t q = (uint64_t)diag[ii] + 1; q < rp[ii + 1]; ++q)
            if (col[q] < n) sum = fmaf(M[q], out[col[q]], sum);
        out[ii] = (tmp[ii] - sum) * dinv[ii];
    }
}

int orc_bicgstab_ir32(size_t n, const uint64_t* rp, const uint64_t* col, const double* val,
                      const double* b, double* x, double tol, int maxit, double inner_tol,
                      int inner_maxit, int ilu_sweeps, int* iters, int* outer, double* relres)
{
    const size_t nnz = n ? (size_t)rp[n] : 0;
    double *r = dalloc(n), *M = dalloc(nnz);
    int32_t* diag = (int32_t*)malloc((n ? n : 1) * sizeof(int32_t));
    float *A32 = (float*)calloc(nnz ? nnz : 1, 4), *M32 = (float*)calloc(nnz ? nnz : 1, 4);
    float* dinv32 = (float*)calloc(n ? n : 1, 4);
    float *ri = (float*)calloc(n ? n : 1, 4), *rh = (float*)calloc(n ? n : 1, 4);
    float *p = (float*)calloc(n ? n : 1, 4), *ph = (float*)calloc(n ? n : 1, 4);
    float *v = (float*)calloc(n ? n : 1, 4), *s = (float*)calloc(n ? n : 1, 4);
    float *sh = (float*)calloc(n ? n : 1, 4), *t = (float*)calloc(n ? n : 1, 4);
    float *tmp = (float*)calloc(n ? n : 1, 4), *d = (float*)calloc(n ? n : 1, 4);
    long long i;
    int it = 0, nout = 0, converged = 0;
    const double tol2 = tol * tol;

    orc_extract_diag(n, rp, col, diag);
    orc_ilu_fixed_point(n, rp, col, val, diag, ilu_sweeps, M);
    for (size_t q = 0; q < nnz; ++q) { A32[q] = (float)val[q]; M32[q] = (float)M[q]; }
    for (size_t k = 0; k < n; ++k) dinv32[k] = (float)(1.0 / M[diag[k]]);
    const double bb = orc_dot(n, b, b);
    if (bb == 0.0) { memset(x, 0, n * sizeof(double)); converged = 1; }
    while (!converged) {
        orc_gemv(n, rp, col, val, x, 1, 0.0, b, r);     /* FP64 residual */
        const double rr = orc_dot(n, r, r);
        if (rr <= tol2 * bb) { converged = 1; break; }
        if (it >= maxit) break;
        const double rnorm = sqrt(rr), scale = 1.0 / rnorm;
        for (size_t k = 0; k < n; ++k) {
            ri[k] = (float)(r[k] * scale);
            rh[k] = ri[k];
            p[k] = ri[k];
            d[k] = 0.0f;
        }
        double rho = dot32(n, rh, ri);
        /* inner target: the reduction still missing (margin 2), at most inner_tol */
        const double itol = fmax(inner_tol, 0.5 * tol / sqrt(rr / bb));
        const double r0 = dot32(n, ri, ri), itol2 = itol * itol * r0;
        for (int k = 0; k < inner_maxit && it < maxit; ++k) {
            ++it;
            precond32(n, rp, col, M32, diag, dinv32, p, tmp, ph);
            spmv32(n, rp, col, A32, ph, v);
            const double sigma = dot32(n, rh, v);
            if (sigma == 0.0) break;
            const double alpha = rho / sigma;
            const float af = (float)alpha;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) s[i] = fmaf(-af, v[i], ri[i]);
            const double ss = dot32(n, s, s);
            if (ss <= itol2) {
#pragma omp parallel for schedule(static)
                for (i = 0; i < (long long)n; ++i) d[i] = fmaf(af, ph[i], d[i]);
                break;
            }
            precond32(n, rp, col, M32, diag, dinv32, s, tmp, sh);
            spmv32(n, rp, col, A32, sh, t);
            const double ts = dot32(n, t, s), tt = dot32(n, t, t);
            const double omega = tt != 0.0 ? ts / tt : 0.0;
            const float of = (float)omega;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) {
                d[i] = fmaf(of, sh[i], fmaf(af, ph[i], d[i]));
                ri[i] = fmaf(-of, t[i], s[i]);
            }
            const double rri = dot32(n, ri, ri), rho_new = dot32(n, rh, ri);
            if (rri <= itol2 || omega == 0.0 || rho == 0.0) break;
            const double beta = (rho_new / rho) * (alpha / omega);
            rho = rho_new;
            const float bf = (float)beta;
#pragma omp parallel for schedule(static)
            for (i = 0; i < (long long)n; ++i) p[i] = fmaf(bf, fmaf(-of, v[i], p[i]), ri[i]);
        }
#pragma omp parallel for schedule(static)
        for (i = 0; i < (long long)n; ++i) x[i] = fma((double)d[i], rnorm, x[i]);
        ++nout;
    }
    if (iters) *iters = it;
    if (outer) *outer = nout;
    if (relres) *relres = orc_true_relres(n, rp, col, val, b, x);
    free(r); free(M); free(diag); free(A32); free(M32); free(dinv32); free(ri); free(rh);
    free(p); free(ph); free(v); free(s); free(sh); free(t); free(tmp); free(d);
    return converged ? 0 : 1;
}
