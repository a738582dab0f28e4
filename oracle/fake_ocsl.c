/* TEST INFRASTRUCTURE ONLY -- a CPU stand-in for the handful of C-ABI entry
 * points (include/ocsl.h) that the C++ drop-in
 * opencslsolver_gb300/shim/cmatrix_solver_gpu.cpp calls, implemented on the
 * oracle.  oracle/Makefile links the shim against it, together with the
 * reference's own objects, so that a CPU test can run the reference's SIMPLE
 * loop through the shim and compare with the reference's own solver: it checks
 * the shim's routing (which member lands where, what it returns, when the
 * pattern is uploaded), not the GPU kernels.  Only the Mode R methods exist. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ocsl.h"
#include "ocsl_oracle.h"

struct ocsl_ctx {
    size_t n;
    uint64_t* rp;
    uint64_t* col;
    long pattern_uploads;
    long solves;
    char err[128];
};

void ocsl_default_opts(ocsl_opts* o)
{
    o->tol = 1e-10;
    o->maxit = 5000;
    o->ilu_sweeps = 3;
    o->inner_tol = 1e-5;
    o->inner_maxit = 500;
}

const char* ocsl_status_string(int s)
{
    return s == OCSL_OK ? "ok" : s == OCSL_BAD_ARGUMENT ? "bad argument" : "fake failure";
}

const char* ocsl_last_error(const ocsl_ctx* c) { return c ? c->err : "no context"; }

int ocsl_create(ocsl_ctx** out, int device)
{
    (void)device;
    *out = (ocsl_ctx*)calloc(1, sizeof(ocsl_ctx));
    return *out ? OCSL_OK : OCSL_BAD_ARGUMENT;
}

int ocsl_destroy(ocsl_ctx* c)
{
    if (c) {
        fprintf(stderr, "fake_ocsl: %ld pattern uploads, %ld solves\n", c->pattern_uploads,
                c->solves);
        free(c->rp);
        free(c->col);
        free(c);
    }
    return OCSL_OK;
}

/* The CPU restatement has no device loop to switch: accepted, nothing changes. */
int ocsl_set_device_loop(ocsl_ctx* c, int enable)
{
    (void)enable;
    return c ? OCSL_OK : OCSL_BAD_ARGUMENT;
}

int ocsl_set_pattern(ocsl_ctx* c, size_t n, const size_t* rp, const size_t* col)
{
    const size_t nnz = rp[n];
    free(c->rp);
    free(c->col);
    c->rp = (uint64_t*)malloc((n + 1) * sizeof(uint64_t));
    c->col = (uint64_t*)malloc((nnz ? nnz : 1) * sizeof(uint64_t));
    for (size_t i = 0; i <= n; ++i) c->rp[i] = rp[i];
    for (size_t k = 0; k < nnz; ++k) c->col[k] = col[k];
    c->n = n;
    ++c->pattern_uploads;
    return OCSL_OK;
}

int ocsl_solve(ocsl_ctx* c, int method, const double* value, const double* b, double* x,
               const ocsl_opts* opts, ocsl_result* res)
{
    (void)opts;
    int iters = 0;
    memset(res, 0, sizeof *res);
    if (!c->rp) {
        snprintf(c->err, sizeof c->err, "no pattern");
        return OCSL_NO_PATTERN;
    }
    if (method == OCSL_CG_REF)
        res->residual = orc_cg_ref(c->n, c->rp, c->col, value, b, x, &iters);
    else if (method == OCSL_BICGSTAB_REF)
        res->residual = orc_bicgstab_ref(c->n, c->rp, c->col, value, b, x, &iters);
    else {
        snprintf(c->err, sizeof c->err, "fake supports the reference methods only");
        return OCSL_BAD_ARGUMENT;
    }
    res->iterations = iters;
    ++c->solves;
    if (getenv("FAKE_OCSL_LOG"))
        fprintf(stderr, "fake_ocsl: solve %ld method %d n %zu iters %d res %.17g uploads %ld\n",
                c->solves, method, c->n, iters, res->residual, c->pattern_uploads);
    return OCSL_OK;
}
