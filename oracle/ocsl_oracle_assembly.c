/* TEST INFRASTRUCTURE ONLY -- oracle restatement of the flow solver's
 * face-loop coefficient assembly (cflow_solver_cell_face_loops.cpp:37-446,
 * solvers_common.h:32-151) and of the heat solver's (cheat_solver.cpp:32-65),
 * in the order the reference's loops run on one thread: clear, interior faces
 * ascending, boundary faces ascending, cells ascending (cflow_solver.cpp:258-290
 * momentum, 319-349 pressure correction, 431-460 enthalpy; cheat_solver.cpp:112-136).  Each entry of the matrix and of b is a running sum
 * from 0.0 in exactly that order.
 *
 * Rounding: the reference is compiled with -ffast-math, so a product that is
 * added in the same statement (or, after inlining, the next one) is
 * contracted; the restatement writes those as fma() and everything else as
 * separate operations.  Sutherland's law is C1 * (T * sqrt(T)) / (T + C2)
 * (the reference's pow(T, 1.5) differs by at most an ulp).  Pinned against
 * the reference's own assembled systems (tests/golden/assembly_*.npz,
 * recorded by oracle/ref_assembly.cpp). */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ocsl_oracle.h"

#define ALPHA 0.7 /* solvers_common.h:29 */

static double mu(const ocsl_assembly* q, double T)
{
    return q->sutherland[0] * (T * sqrt(T)) / (T + q->sutherland[1]); /* cfluid_properties.cpp:123-128 */
}

static double drho_dp(const ocsl_assembly* q, double T) /* cfluid_properties.cpp:79-86 */
{
    double r = q->R_specific * T;
    r = r * q->gamma;
    return 1.0 / r;
}

static double face_avg(double geo, double l, double r) /* solvers_common.h:32-39 */
{
    return fma(1.0 - geo, r, geo * l);
}

static double face_interp(int blended, double geo, double m, double l, double r)
{ /* solvers_common.h:70-92 */
    if (m >= 0.0) return blended ? fma(ALPHA, face_avg(geo, l, r), l * (1.0 - ALPHA)) : l;
    if (m < 0.0) return blended ? fma(ALPHA, face_avg(geo, l, r), r * (1.0 - ALPHA)) : r;
    return 0.0;
}

static int64_t slot(const uint64_t* rp, const uint64_t* col, int64_t i, int64_t j)
{
    for (uint64_t q = rp[i]; q < rp[i + 1]; ++q)
        if (col[q] == (uint64_t)j) return (int64_t)q;
    return -1;
}

typedef struct {
    const uint64_t* rp;
    const uint64_t* col;
    double* A;
    double* b;
} Sys;

static void addA(Sys* s, int64_t i, int64_t j, double v) { s->A[slot(s->rp, s->col, i, j)] += v; }

/* solvers_common.h:96-135 */
static void convective(Sys* s, int blended, double geo, int64_t L, int64_t R, double m, double l,
                       double r)
{
    if (m >= 0.0) {
        addA(s, L, L, m);
        addA(s, R, L, -m);
        if (blended) {
            const double val = ALPHA * (face_avg(geo, l, r) - l);
            s->b[L] += -m * val;
            s->b[R] += m * val;
        }
    } else if (m < 0.0) {
        addA(s, L, R, m);
        addA(s, R, R, -m);
        if (blended) {
            const double val = ALPHA * (face_avg(geo, l, r) - r);
            s->b[L] += -m * val;
            s->b[R] += m * val;
        }
    }
}

/* solvers_common.h:42-53 */
static void diffusive(Sys* s, int64_t L, int64_t R, double D)
{
    addA(s, L, L, D);
    addA(s, L, R, -D);
    addA(s, R, R, D);
    addA(s, R, L, -D);
}

/* solvers_common.h:138-151 */
static void neumann_zero(Sys* s, int64_t P, double m)
{
    if (m >= 0.0)
        addA(s, P, P, m);
    else if (m < 0.0)
        addA(s, P, P, m);
}

void orc_assemble(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                  const int32_t* left, const int32_t* right, int64_t nb, const int32_t* bc_left,
                  const ocsl_assembly* q, const ocsl_flow_state* st, double* value, double* b,
                  double* x0, double* ap, double* total_mdot)
{
    Sys s = {rp, col, value, b};
    const int d = q->dimension, eq = q->equation;
    memset(value, 0, rp[n] * sizeof(double));
    memset(b, 0, n * sizeof(double));
    if (total_mdot) memset(total_mdot, 0, n * sizeof(double));
    const double* u = st->velocity ? st->velocity + (size_t)d * n : NULL;
    /* interior faces */
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t L = left[f], R = right[f];
        if (eq == OCSL_EQ_HEAT) { /* cheat_solver.cpp:32-37 */
            const double D = q->thermal_diffusivity * st->ksi_A[f];
            diffusive(&s, L, R, D);
            continue;
        }
        const double g = st->geo_aver[f], m = st->mdot[f];
        if (eq == OCSL_EQ_MOMENTUM) { /* :37-57 */
            convective(&s, q->blended, g, L, R, m, u[L], u[R]);
            if (q->viscous) {
                const double Tf = face_avg(g, st->temperature[L], st->temperature[R]);
                double D = mu(q, Tf);
                D = D * st->ksi_A[f];
                diffusive(&s, L, R, D);
                const double sp = st->stress[(size_t)d * nf + f];
                b[L] += sp;
                b[R] += -sp;
            }
        } else if (eq == OCSL_EQ_PRESSURE) { /* :176-211 */
            b[L] += -m;
            b[R] += m;
            if (total_mdot) {
                total_mdot[L] += m;
                total_mdot[R] -= m;
            }
            const double Tf = face_interp(q->blended, g, m, st->temperature[L], st->temperature[R]);
            double dum = drho_dp(q, Tf);
            dum = dum / st->density[f];
            dum *= m;
            convective(&s, q->blended, g, L, R, dum, st->pressure_corr[L], st->pressure_corr[R]);
            const double D = st->qy[f] * st->density[f];
            diffusive(&s, L, R, D);
        } else { /* :334-345 */
            convective(&s, q->blended, g, L, R, m, st->enthalpy[L], st->enthalpy[R]);
            const double Tf = face_avg(g, st->temperature[L], st->temperature[R]);
            double D = mu(q, Tf);
            D = D / q->prandtl * st->ksi_A[f];
            diffusive(&s, L, R, D);
        }
    }
    /* boundary faces */
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t P = bc_left[k];
        if (eq == OCSL_EQ_HEAT) { /* cheat_solver.cpp:39-56: constant-temperature faces */
            if (st->bc_thermal[k] == OCSL_THERMAL_CONSTANT_TEMPERATURE) {
                const double D = q->thermal_diffusivity * st->bc_ksi_A[k];
                addA(&s, P, P, D);
                b[P] += D * st->bc_temperature[k];
            }
            continue;
        }
        const int type = st->bc_type[k];
        const double m = st->bc_mdot[k];
        const double bv = st->bc_value ? st->bc_value[k] : 0.0;
        if (eq == OCSL_EQ_MOMENTUM) { /* :75-131 */
            if (type == OCSL_BC_WALL && q->viscous && st->bc_wall[k] == OCSL_WALL_NO_SLIP) {
                const double inv = 1.0 / st->bc_area[k];
                double nv[3];
                for (int c = 0; c < 3; ++c) nv[c] = inv * st->bc_area_vector[(size_t)c * nb + k];
                double D = mu(q, st->temperature[P]);
                D *= st->bc_area[k] / st->bc_perp_dist[k];
                double dum = D * (1.0 - (nv[d] * nv[d]));
                addA(&s, P, P, dum);
                dum = 0.0;
                for (int i = d + 1; i < d + 3; ++i) {
                    const int i_ = i % 3;
                    dum = fma(st->velocity[(size_t)i_ * n + P] * nv[i_], nv[d], dum);
                }
                dum = D * dum;
                b[P] += dum;
            }
            if (type == OCSL_BC_VELOCITY_INLET || type == OCSL_BC_SUPERSONIC_INLET)
                b[P] += -(m * st->bc_velocity[(size_t)d * nb + k]);
            if (type == OCSL_BC_PRESSURE_OUTLET) addA(&s, P, P, m);
        } else if (eq == OCSL_EQ_PRESSURE) { /* :214-270 */
            if (type == OCSL_BC_VELOCITY_INLET) {
                b[P] += -m;
                if (total_mdot) total_mdot[P] += m;
                double dum = drho_dp(q, st->bc_temperature[k]) / st->density_c[P];
                dum *= m;
                neumann_zero(&s, P, dum);
            }
            if (type == OCSL_BC_SUPERSONIC_INLET) {
                b[P] += -m;
                if (total_mdot) total_mdot[P] += m;
                const double D = st->bc_qy[k] * st->bc_density[k];
                addA(&s, P, P, D);
                b[P] += D * bv;
            }
            if (type == OCSL_BC_PRESSURE_OUTLET) {
                b[P] += -m;
                if (total_mdot) total_mdot[P] += m;
                if (st->bc_supersonic[k]) {
                    double dum = drho_dp(q, st->temperature[P]) / st->density_c[P];
                    dum *= m;
                    neumann_zero(&s, P, dum);
                } else {
                    const double D = st->bc_qy[k] * st->density_c[P];
                    addA(&s, P, P, D);
                    b[P] += D * bv;
                }
            }
        } else { /* :350-410 */
            if (type == OCSL_BC_VELOCITY_INLET || type == OCSL_BC_SUPERSONIC_INLET) {
                b[P] += -(m * st->bc_enthalpy[k]);
                double D = mu(q, st->bc_temperature[k]);
                D *= q->prandtl * st->bc_ksi_A[k];
                addA(&s, P, P, D);
                b[P] += D * st->bc_enthalpy[k];
            }
            if (type == OCSL_BC_PRESSURE_OUTLET) neumann_zero(&s, P, m);
        }
    }
    /* cells */
    const double urf = q->implicit_underrelaxation;
    for (size_t i = 0; i < n; ++i) {
        const int64_t dg = slot(rp, col, (int64_t)i, (int64_t)i);
        const double vol = st->volume[i];
        if (eq == OCSL_EQ_MOMENTUM) { /* :143-172 */
            double dum = 0.0, dum2 = 0.0;
            if (q->transient) {
                dum = vol / st->delta_t[i];
                dum2 = dum * st->density_c[i];
                value[dg] += dum2;
                dum2 = dum * (st->velocity_last[(size_t)d * n + i] * st->density_last[i]);
            }
            dum2 = fma(-st->pressure_grad[(size_t)d * n + i], vol, dum2);
            b[i] += dum2;
            if (!q->transient) {
                dum = value[dg];
                value[dg] = dum / urf;
                dum = (1.0 - urf) / urf * dum * st->velocity_last[(size_t)d * n + i];
                b[i] += dum;
            }
            x0[i] = u[i];
        } else if (eq == OCSL_EQ_HEAT) { /* cheat_solver.cpp:58-66 (global dt per cell) */
            const double dum = vol / st->delta_t[i];
            value[dg] += dum;
            b[i] += st->temperature[i] * dum;
            x0[i] = st->temperature[i];
        } else if (eq == OCSL_EQ_PRESSURE) { /* :273-296 */
            if (q->transient) {
                const double dum = vol / st->delta_t[i];
                double dum2 = dum * (st->density_c[i] - st->density_last[i]);
                b[i] += -dum2;
                dum2 = dum * drho_dp(q, st->temperature[i]);
                value[dg] += dum2;
            } else {
                value[dg] = value[dg] / urf;
            }
            x0[i] = st->pressure_corr[i];
        } else { /* :413-436 */
            if (q->transient) {
                const double dum = vol / st->delta_t[i];
                double dum2 = dum * st->density_c[i];
                value[dg] += dum2;
                dum2 = dum * (st->enthalpy_last[i] * st->density_last[i]);
                dum2 = fma((st->pressure[i] - st->pressure_last[i]) / st->delta_t[i], vol, dum2);
                b[i] += dum2;
            } else {
                double dum = value[dg];
                value[dg] = dum / urf;
                dum = (1.0 - urf) / urf * dum * st->enthalpy_last[i];
                b[i] += dum;
            }
            x0[i] = st->enthalpy[i];
        }
        if (ap) ap[i] = value[dg];
    }
}

/* d_grad[k] = lambda[P] * D_k for the Dirichlet pressure-correction faces. */
void orc_bc_value_grad(size_t n, const uint64_t* rp, int64_t nb, const int32_t* bc_left,
                       const ocsl_assembly* q, const ocsl_flow_state* st, const double* lambda,
                       double* grad)
{
    (void)n;
    (void)rp;
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t P = bc_left[k];
        const int type = st->bc_type[k];
        double D = 0.0;
        if (q->equation == OCSL_EQ_PRESSURE) {
            if (type == OCSL_BC_SUPERSONIC_INLET) D = st->bc_qy[k] * st->bc_density[k];
            if (type == OCSL_BC_PRESSURE_OUTLET && !st->bc_supersonic[k])
                D = st->bc_qy[k] * st->density_c[P];
        }
        grad[k] = lambda[P] * D;
    }
}
