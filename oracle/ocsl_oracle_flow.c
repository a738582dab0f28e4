/* TEST INFRASTRUCTURE ONLY -- oracle restatement of the SIMPLE inner
 * iteration around the assembly and the solves: CFlow_solver::iterate
 * (cflow_solver.cpp:229-476), the routines of cflow_solver_supply.cpp it
 * calls, and update_timestep (:503-512), for every boundary kind, inviscid
 * or viscous, transient or steady.  Loops run in the reference's
 * single-thread order (faces ascending, boundary faces ascending, cells
 * ascending), so every gradient component is the running sum the reference
 * forms.
 *
 * Rounding: the reference is compiled with -ffast-math, so a product added in
 * the same expression is contracted; those are written fma() here, the rest
 * as separate operations.  The residual sums are the library's tile-order
 * sums (orc_sum), not the reference's serial ones.  The assembly is
 * orc_assemble; the solves are orc_cg_ref / orc_bicgstab_ref (the reference's
 * solvers), orc_pcg_tol / orc_bicgstab_tol (the library's tolerance mode), or
 * -- to check the stages between the solves against the reference's own
 * recorded solutions -- a given x per solve.
 *
 * Pinned against states the reference itself wrote before every solve and
 * after whole inner iterations of the 1000-cell shock tube and the 200-cell
 * viscous channel and steady cases (tests/golden/flow_*.npz, recorded by
 * oracle/ref_flow.cpp).  The 1D cases carry no transverse velocity, so the
 * summation order inside |u|^2 and the rounding of the viscous stress (about
 * 1e-10 of the momentum terms there) are not discriminated by them. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ocsl_oracle.h"

#define ALPHA 0.7 /* solvers_common.h:29 */

/* solvers_common.h:32-39 and :69-90 as compiled into cflow_solver_supply.cpp:
 * there the compiler contracts the FIRST product of each a*b + c*d (the
 * face-loop assembly's translation unit contracts the second one). */
static double face_avg(double geo, double l, double r)
{
    return fma(geo, l, (1.0 - geo) * r);
}

static double face_interp(int blended, double geo, double m, double l, double r)
{
    const double up = m >= 0.0 ? l : r;
    return blended ? fma(up, 1.0 - ALPHA, ALPHA * face_avg(geo, l, r)) : up;
}

static double dot3(const double a[3], const double b[3]) /* tensor.h:128-134 */
{
    double r = a[0] * b[0];
    r = fma(a[1], b[1], r);
    return fma(a[2], b[2], r);
}

#define W(p) ((double*)(uintptr_t)(p))

static double density(const ocsl_assembly* q, double p, double T) /* cfluid_properties.cpp:46-51 */
{
    return p / (q->R_specific * T); /* p / R / T under -ffast-math */
}

static double sound(const ocsl_assembly* q, double T) /* cfluid_properties.cpp:89-96 */
{
    return sqrt(q->R_specific * T * q->gamma);
}

static double usq(const double u[3]) /* |u|^2 in the order the compiled mag() sums it */
{
    return fma(u[2], u[2], fma(u[0], u[0], u[1] * u[1]));
}

static double enthalpy(const ocsl_flow_iteration* it, double T, const double u[3])
{ /* cfluid_properties.cpp:98-106: Hf + (T - Tref) cp + |u| |u| / 2 */
    return fma(usq(u), 0.5, fma(T - it->Tref, it->cp, it->H_formation));
}

static double mu(const ocsl_assembly* q, double T) /* cfluid_properties.cpp:123-128 */
{
    return q->sutherland[0] * (T * sqrt(T)) / (T + q->sutherland[1]);
}

static void vec3(const double* a, size_t stride, size_t k, double out[3])
{
    out[0] = a[k];
    out[1] = a[stride + k];
    out[2] = a[2 * stride + k];
}

/* CFlow_solver::set_boundary_conditions (cflow_solver.cpp:195-227), per
 * boundary face.  Outlets read their density from the boundary pressure of
 * the previous iteration and then mark themselves supersonic on both
 * branches, as the reference does. */
void orc_flow_set_bc(size_t n, int64_t nb, const int32_t* bc_left, const ocsl_assembly* q,
                     const ocsl_flow_state* st, const ocsl_flow_iteration* it)
{
    for (int64_t g = 0; g < nb; ++g) {
        const int32_t c = bc_left[g];
        double A[3], V[3], u[3];
        vec3(st->bc_area_vector, (size_t)nb, (size_t)g, A);
        switch (st->bc_type[g]) {
        case OCSL_BC_VELOCITY_INLET:
            vec3(st->bc_velocity, (size_t)nb, (size_t)g, V);
            it->bc_pressure[g] = st->pressure[c];
            W(st->bc_density)[g] = density(q, st->pressure[c], st->bc_temperature[g]);
            W(st->bc_mdot)[g] = st->bc_density[g] * dot3(V, A);
            W(st->bc_enthalpy)[g] = enthalpy(it, st->bc_temperature[g], V);
            break;
        case OCSL_BC_PRESSURE_OUTLET: {
            vec3(st->velocity, n, (size_t)c, u);
            W(st->bc_temperature)[g] = st->temperature[c];
            for (int d = 0; d < 3; ++d) W(st->bc_velocity)[d * nb + g] = u[d];
            W(st->bc_density)[g] = density(q, it->bc_pressure[g], st->temperature[c]);
            W(st->bc_enthalpy)[g] = enthalpy(it, st->temperature[c], u);
            const double speed = st->bc_mdot[g] / (st->density_c[c] * st->bc_area[g]);
            ((int32_t*)(uintptr_t)st->bc_supersonic)[g] = 1;
            it->bc_pressure[g] = speed >= sound(q, st->temperature[c]) ? st->pressure[c]
                                                                       : it->bc_out_pressure[g];
            break;
        }
        case OCSL_BC_WALL: {
            double gp[3], un[3];
            vec3(st->pressure_grad, n, (size_t)c, gp);
            vec3(it->bc_unit, (size_t)nb, (size_t)g, un);
            it->bc_pressure[g] = fma(dot3(gp, un), it->bc_distance[g], st->pressure[c]);
            break;
        }
        default: break; /* supersonic inlets, symmetry, empty faces: nothing */
        }
    }
}

/* The explicit part of the viscous stress on the interior faces
 * (cflow_solver_cell_face_loops.cpp:25-35, tensor.h:194-225): mu(T_f) times
 * (grad u^T - 2/3 div u I) applied to the area vector, with the gradients
 * taken along the cell-to-cell direction. */
void orc_flow_stress(size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                     const ocsl_assembly* q, const ocsl_flow_state* st,
                     const ocsl_flow_iteration* it)
{
    for (int64_t k = 0; k < nf; ++k) {
        const int32_t L = left[k], R = right[k];
        double dv[3], un[3], A[3];
        for (int d = 0; d < 3; ++d) dv[d] = st->velocity[d * n + R] - st->velocity[d * n + L];
        vec3(it->face_unit, (size_t)nf, (size_t)k, un);
        vec3(it->face_area_vector, (size_t)nf, (size_t)k, A);
        const double dist = it->face_distance[k];
        double div = dv[0] * un[0] / dist;
        div = div + dv[1] * un[1] / dist;
        div = div + dv[2] * un[2] / dist;
        const double geo = st->geo_aver[k];
        const double m = mu(q, fma(1.0 - geo, st->temperature[R], geo * st->temperature[L]));
        for (int i = 0; i < 3; ++i) {
            double t[3];
            for (int j = 0; j < 3; ++j) t[j] = dv[j] * un[i] / dist; /* transpose(grad u) */
            t[i] = fma(-(2.0 / 3.0), div, t[i]);
            for (int j = 0; j < 3; ++j) t[j] = m * t[j];
            W(st->stress)[i * nf + k] = dot3(t, A);
        }
    }
}

/* Green-Gauss gradients: the pressure with the ap-weighted face value
 * (cflow_solver_supply.cpp:132-177) or the pressure correction with the face
 * average (:179-220).  Boundary faces add the cell's own value, except that
 * outlets and supersonic inlets add their boundary pressure to the pressure
 * gradient, and add nothing to the correction's unless the outlet is
 * supersonic (supersonic inlets never). */
void orc_flow_grad(int corr, size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                   int64_t nb, const int32_t* bc_left, const ocsl_flow_state* st,
                   const ocsl_flow_iteration* it)
{
    const double* v = corr ? st->pressure_corr : st->pressure;
    double* g = corr ? it->pressure_corr_grad : W(st->pressure_grad);
    memset(g, 0, 3 * n * sizeof(double));
    for (int64_t k = 0; k < nf; ++k) {
        const int32_t L = left[k], R = right[k];
        double fp;
        if (corr) {
            fp = face_avg(st->geo_aver[k], v[L], v[R]);
        } else {
            const double den = it->ap[L] + it->ap[R];
            fp = fma(it->ap[L], v[L], it->ap[R] * v[R]) / den;
        }
        for (int d = 0; d < 3; ++d) {
            const double a = it->face_area_vector[d * nf + k];
            g[d * n + L] = fma(fp, a, g[d * n + L]);
            g[d * n + R] = fma(-fp, a, g[d * n + R]);
        }
    }
    for (int64_t q = 0; q < nb; ++q) {
        const int32_t c = bc_left[q];
        const int kind = st->bc_type[q];
        double fv = v[c];
        if (kind == OCSL_BC_PRESSURE_OUTLET || kind == OCSL_BC_SUPERSONIC_INLET) {
            if (!corr) fv = it->bc_pressure[q];
            else if (kind == OCSL_BC_SUPERSONIC_INLET || !st->bc_supersonic[q]) continue;
        }
        for (int d = 0; d < 3; ++d) g[d * n + c] = fma(fv, st->bc_area_vector[d * nb + q], g[d * n + c]);
    }
    for (size_t c = 0; c < n; ++c) {
        const double inv = 1.0 / st->volume[c];
        for (int d = 0; d < 3; ++d) g[d * n + c] = inv * g[d * n + c];
    }
}

/* After the solve of momentum component d (cflow_solver.cpp:292-301) and the
 * ap of its cell loop (cflow_solver_cell_face_loops.cpp:168): res = |u_d - x|,
 * u_d = x, ap += ap_vec_d / 3. */
void orc_flow_velocity_update(size_t n, int d, const double* x, const ocsl_flow_state* st,
                              const ocsl_flow_iteration* it, double* res)
{
    double* u = W(st->velocity) + (size_t)d * n;
    for (size_t c = 0; c < n; ++c) {
        res[c] = fabs(u[c] - x[c]);
        u[c] = x[c];
        /* -ffast-math turns the division by 3 into a product with 1/3, contracted */
        it->ap[c] = fma(it->ap_vec[(size_t)d * n + c], 1.0 / 3.0, it->ap[c]);
    }
}

/* Face mass fluxes with the pressure-gradient correction (cflow_solver_supply.cpp:25-44). */
void orc_flow_face_mdot(size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                        int blended, const ocsl_flow_state* st, const ocsl_flow_iteration* it)
{
    for (int64_t k = 0; k < nf; ++k) {
        const int32_t L = left[k], R = right[k];
        double al[3], av[3], pg[3], dv[3], vf[3];
        for (int d = 0; d < 3; ++d) {
            al[d] = it->face_alpha[d * nf + k];
            av[d] = it->face_area_vector[d * nf + k];
        }
        const double qy = (st->volume[L] / it->ap[L] + st->volume[R] / it->ap[R]) * dot3(al, av);
        const double geo = st->geo_aver[k];
        for (int d = 0; d < 3; ++d) {
            pg[d] = face_avg(geo, st->pressure_grad[d * n + L], st->pressure_grad[d * n + R]);
            dv[d] = it->face_distance[k] * it->face_unit[d * nf + k];
            vf[d] = face_avg(geo, st->velocity[d * n + L], st->velocity[d * n + R]);
        }
        const double t = st->pressure[R] - st->pressure[L] - dot3(pg, dv);
        double m = fma(-qy, t, dot3(vf, av)); /* dot(v_f, A) - Qy t */
        const double rho = face_interp(blended, geo, m, st->density_c[L], st->density_c[R]);
        m *= rho;
        W(st->qy)[k] = qy;
        W(st->density)[k] = rho;
        W(st->mdot)[k] = m;
    }
}

/* Boundary mass fluxes (cflow_solver_supply.cpp:51-93). */
void orc_flow_bc_mdot(size_t n, int64_t nb, const int32_t* bc_left, const ocsl_assembly* q,
                      const ocsl_flow_state* st, const ocsl_flow_iteration* it)
{
    for (int64_t g = 0; g < nb; ++g) {
        const int32_t c = bc_left[g];
        const int kind = st->bc_type[g];
        double A[3], al[3], u[3];
        vec3(st->bc_area_vector, (size_t)nb, (size_t)g, A);
        vec3(it->bc_alpha, (size_t)nb, (size_t)g, al);
        vec3(st->velocity, n, (size_t)c, u);
        if (kind == OCSL_BC_VELOCITY_INLET) {
            double V[3];
            vec3(st->bc_velocity, (size_t)nb, (size_t)g, V);
            W(st->bc_mdot)[g] = density(q, st->pressure[c], st->bc_temperature[g]) * dot3(V, A);
        } else if (kind == OCSL_BC_SUPERSONIC_INLET) {
            W(st->bc_qy)[g] = st->volume[c] / it->ap[c] * dot3(al, A);
        } else if (kind == OCSL_BC_PRESSURE_OUTLET) {
            if (st->bc_supersonic[g]) {
                W(st->bc_mdot)[g] = density(q, st->pressure[c], st->temperature[c]) * dot3(u, A);
                W(st->bc_qy)[g] = 1.0;
            } else {
                const double qy = st->volume[c] / it->ap[c] * dot3(al, A);
                double gp[3], dv[3];
                vec3(st->pressure_grad, n, (size_t)c, gp);
                for (int d = 0; d < 3; ++d) dv[d] = it->bc_distance[g] * it->bc_unit[d * nb + g];
                const double t = it->bc_pressure[g] - st->pressure[c] - 0.5 * dot3(gp, dv);
                W(st->bc_qy)[g] = qy;
                W(st->bc_mdot)[g] = fma(-qy, t, dot3(u, A)) * st->bc_density[g];
            }
        }
    }
}

/* p' = relax_p x, p += p' (cflow_solver.cpp:352-358). */
void orc_flow_pcorr(size_t n, const double* x, const ocsl_flow_state* st,
                    const ocsl_flow_iteration* it)
{
    for (size_t c = 0; c < n; ++c) {
        const double pc = it->relax_p * x[c];
        W(st->pressure_corr)[c] = pc;
        W(st->pressure)[c] = st->pressure[c] + pc;
    }
}

/* Boundary pressures that follow the corrected cell pressure (cflow_solver.cpp:361-372). */
void orc_flow_bc_pcorr(int64_t nb, const int32_t* bc_left, const ocsl_flow_state* st,
                       const ocsl_flow_iteration* it)
{
    for (int64_t g = 0; g < nb; ++g) {
        const int kind = st->bc_type[g];
        if (kind == OCSL_BC_VELOCITY_INLET ||
            (kind == OCSL_BC_PRESSURE_OUTLET && st->bc_supersonic[g]))
            it->bc_pressure[g] = st->pressure[bc_left[g]];
    }
}

/* Mass-flux correction (cflow_solver_supply.cpp:95-123), densities from the
 * corrected pressure, cells and boundary faces (cflow_solver.cpp:386-410,
 * cfluid_properties.cpp:46-51) and the velocity correction (:422-426,
 * tensor.h:136-146). */
void orc_flow_correct(size_t n, int64_t nf, const int32_t* left, const int32_t* right,
                      int64_t nb, const int32_t* bc_left, const ocsl_assembly* q,
                      const ocsl_flow_state* st, const ocsl_flow_iteration* it)
{
    for (int64_t k = 0; k < nf; ++k) {
        const int32_t L = left[k], R = right[k];
        const double geo = st->geo_aver[k];
        double m = st->mdot[k];
        const double tf = face_interp(q->blended, geo, m, st->temperature[L], st->temperature[R]);
        const double pcf = face_interp(q->blended, geo, m, st->pressure_corr[L], st->pressure_corr[R]);
        const double rho = st->density[k];
        double dp = q->R_specific * tf; /* cfluid_properties.cpp:79-86 */
        dp = dp * q->gamma;
        dp = 1.0 / dp;
        /* the two `Mdot +=` of the reference, reassociated by the compiler:
         * the Qy term is added first */
        const double t = fma(st->qy[k] * rho, st->pressure_corr[L] - st->pressure_corr[R], m);
        W(st->mdot)[k] = fma(m / rho * dp, pcf, t);
    }
    for (int64_t g = 0; g < nb; ++g) /* cflow_solver_supply.cpp:113-123 */
        if (st->bc_type[g] == OCSL_BC_PRESSURE_OUTLET && !st->bc_supersonic[g])
            W(st->bc_mdot)[g] = fma(st->bc_qy[g] * st->bc_density[g],
                                    st->pressure_corr[bc_left[g]], st->bc_mdot[g]);
    for (size_t c = 0; c < n; ++c) {
        W(st->density_c)[c] = density(q, st->pressure[c], st->temperature[c]);
        const double s = it->relax_u * st->volume[c];
        for (int d = 0; d < 3; ++d) {
            double a = it->ap_vec[d * n + c];
            if (a == 0.0) a = DBL_MIN;
            const double r = it->pressure_corr_grad[d * n + c] / a;
            W(st->velocity)[d * n + c] = fma(-s, r, st->velocity[d * n + c]);
        }
    }
    for (int64_t g = 0; g < nb; ++g) { /* cflow_solver.cpp:393-410 */
        const int32_t c = bc_left[g];
        if (st->bc_type[g] == OCSL_BC_VELOCITY_INLET)
            W(st->bc_density)[g] = density(q, st->pressure[c], st->bc_temperature[g]);
        else if (st->bc_type[g] == OCSL_BC_PRESSURE_OUTLET)
            W(st->bc_density)[g] = density(q, st->bc_supersonic[g] ? st->pressure[c] : it->bc_pressure[g],
                                           st->temperature[c]);
    }
}

/* After the enthalpy solve (cflow_solver.cpp:463-474, cfluid_properties.cpp:
 * 88-120): res = |h - x|, h = x, T from h and |u| clamped to [200, 6000],
 * Mach = |u| / sqrt(R T gamma). */
void orc_flow_enthalpy_update(size_t n, const double* x, const ocsl_assembly* q,
                              const ocsl_flow_state* st, const ocsl_flow_iteration* it,
                              double* res)
{
    for (size_t c = 0; c < n; ++c) {
        res[c] = fabs(st->enthalpy[c] - x[c]);
        const double h = x[c];
        W(st->enthalpy)[c] = h;
        double u[3];
        vec3(st->velocity, n, c, u);
        const double s = usq(u); /* |u| |u| folds to |u|^2 */
        double T = it->Tref + fma(-s, 0.5, h - it->H_formation) / it->cp;
        if (T <= 200.0) T = 200.0;
        if (T >= 6000.0) T = 6000.0;
        W(st->temperature)[c] = T;
        it->mach[c] = sqrt(s) / sound(q, T);
    }
}

void orc_flow_end_step(size_t n, const ocsl_flow_state* st)
{ /* cflow_solver.cpp:505-512 */
    memcpy(W(st->velocity_last), st->velocity, 3 * n * sizeof(double));
    memcpy(W(st->density_last), st->density_c, n * sizeof(double));
    memcpy(W(st->pressure_last), st->pressure, n * sizeof(double));
    memcpy(W(st->enthalpy_last), st->enthalpy, n * sizeof(double));
}

static int run_solve(size_t n, const uint64_t* rp, const uint64_t* col, int method,
                     const ocsl_opts* o, const double* val, const double* b, double* x,
                     const double* given, int* iters)
{
    double relres;
    *iters = 0;
    if (given) {
        memcpy(x, given, n * sizeof(double));
        return 0;
    }
    switch (method) {
    case OCSL_CG_REF: orc_cg_ref(n, rp, col, val, b, x, iters); return 0;
    case OCSL_BICGSTAB_REF: orc_bicgstab_ref(n, rp, col, val, b, x, iters); return 0;
    case OCSL_PCG:
        if (!o) return -1;
        orc_pcg_tol(n, rp, col, val, b, x, o->tol, o->maxit, iters, &relres);
        return 0;
    case OCSL_ILU_BICGSTAB:
        if (!o) return -1;
        orc_bicgstab_tol(n, rp, col, val, b, x, o->tol, o->maxit, o->ilu_sweeps, iters, &relres);
        return 0;
    default: return -1;
    }
}

static int flow_iterate(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                        const int32_t* left, const int32_t* right, int64_t nb,
                        const int32_t* bc_left, const ocsl_assembly* q,
                        const ocsl_flow_state* st, const ocsl_flow_iteration* it,
                        const int* methods, const ocsl_opts* opts,
                        const double* const* given_x, orc_solve_fn ext, void* user,
                        double* sys_value, double* sys_b, double* sys_x0, double* residual,
                        int* iterations)
{
    const size_t nnz = rp[n];
    double* val = (double*)malloc((nnz ? nnz : 1) * sizeof(double));
    double* b = (double*)malloc((n ? n : 1) * sizeof(double));
    double* x = (double*)malloc((n ? n : 1) * sizeof(double));
    double* res = (double*)malloc((n ? n : 1) * sizeof(double));
    int rc = 0;
    ocsl_assembly qe = *q;
    const int eq_method[5] = {methods[0], methods[0], methods[0], methods[1], methods[2]};
    int slot = 0;
#define SOLVE()                                                                            \
    do {                                                                                   \
        if (sys_value) memcpy(sys_value + (size_t)slot * nnz, val, nnz * sizeof(double));  \
        if (sys_b) memcpy(sys_b + (size_t)slot * n, b, n * sizeof(double));                \
        if (sys_x0) memcpy(sys_x0 + (size_t)slot * n, x, n * sizeof(double));              \
        if (ext) {                                                                         \
            iterations[slot] = 0;                                                          \
            if (ext(user, slot, eq_method[slot], n, val, b, x)) rc = -1;                   \
        } else if (run_solve(n, rp, col, eq_method[slot], opts, val, b, x,                 \
                             given_x ? given_x[slot] : NULL, &iterations[slot]))           \
            rc = -1;                                                                       \
    } while (0)

    orc_flow_set_bc(n, nb, bc_left, q, st, it);                 /* :234-237 */
    orc_flow_grad(0, n, nf, left, right, nb, bc_left, st, it);  /* :240 */
    memset(it->ap, 0, n * sizeof(double));                      /* :244-247 */
    if (q->viscous) orc_flow_stress(n, nf, left, right, q, st, it); /* :250-255 */
    for (int d = 0; d < 3; ++d, ++slot) {                       /* :257-302 */
        qe.equation = OCSL_EQ_MOMENTUM;
        qe.dimension = d;
        orc_assemble(n, rp, col, nf, left, right, nb, bc_left, &qe, st, val, b, x,
                     it->ap_vec + (size_t)d * n, it->total_mdot);
        SOLVE();
        orc_flow_velocity_update(n, d, x, st, it, res);
        residual[d] = orc_sum(n, res, 1);
    }
    orc_flow_face_mdot(n, nf, left, right, q->blended, st, it); /* :305-309 */
    orc_flow_bc_mdot(n, nb, bc_left, q, st, it);                /* :312-315 */
    qe.equation = OCSL_EQ_PRESSURE;                             /* :316-346 */
    qe.dimension = 0;
    orc_assemble(n, rp, col, nf, left, right, nb, bc_left, &qe, st, val, b, x, NULL,
                 it->total_mdot);
    residual[3] = orc_sum(n, b, 1);
    SOLVE();
    ++slot;
    orc_flow_pcorr(n, x, st, it);                               /* :352-358 */
    orc_flow_bc_pcorr(nb, bc_left, st, it);                     /* :361-372 */
    orc_flow_grad(1, n, nf, left, right, nb, bc_left, st, it);  /* :375 */
    orc_flow_correct(n, nf, left, right, nb, bc_left, q, st, it); /* :379-426 */
    qe.equation = OCSL_EQ_ENTHALPY;                             /* :428-474 */
    orc_assemble(n, rp, col, nf, left, right, nb, bc_left, &qe, st, val, b, x, NULL, NULL);
    SOLVE();
    orc_flow_enthalpy_update(n, x, q, st, it, res);
    residual[4] = orc_sum(n, res, 1);
#undef SOLVE
    free(val);
    free(b);
    free(x);
    free(res);
    return rc;
}

int orc_flow_iterate(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                     const int32_t* left, const int32_t* right, int64_t nb,
                     const int32_t* bc_left, const ocsl_assembly* q, const ocsl_flow_state* st,
                     const ocsl_flow_iteration* it, const int* methods, const ocsl_opts* opts,
                     const double* const* given_x, double* sys_value, double* sys_b,
                     double* sys_x0, double* residual, int* iterations)
{
    return flow_iterate(n, rp, col, nf, left, right, nb, bc_left, q, st, it, methods, opts,
                        given_x, NULL, NULL, sys_value, sys_b, sys_x0, residual, iterations);
}

int orc_flow_iterate_with(size_t n, const uint64_t* rp, const uint64_t* col, int64_t nf,
                          const int32_t* left, const int32_t* right, int64_t nb,
                          const int32_t* bc_left, const ocsl_assembly* q,
                          const ocsl_flow_state* st, const ocsl_flow_iteration* it,
                          const int* methods, orc_solve_fn solve, void* user,
                          double* residual)
{
    int iterations[5];
    if (!solve) return -1;
    return flow_iterate(n, rp, col, nf, left, right, nb, bc_left, q, st, it, methods, NULL,
                        NULL, solve, user, NULL, NULL, NULL, residual, iterations);
}
