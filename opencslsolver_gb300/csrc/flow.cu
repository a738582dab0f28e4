// The rest of the SIMPLE inner iteration on the device
// (CFlow_solver::iterate, cflow_solver.cpp:229-476, and the routines of
// cflow_solver_supply.cpp it calls), around the face-loop assembly and the
// linear solves: boundary pressures, Green-Gauss pressure and
// pressure-correction gradients, face mass fluxes and their correction, the
// field updates after each solve, and the end-of-step copy
// (update_timestep, :503-512).
//
// Every kernel is owner-computes, like the assembly: a per-cell gradient is
// one thread walking the cell's faces in ascending face order and then its
// boundary faces (the incidence lists of ocsl_set_faces), so each component
// is the running sum the reference's serial face loops produce, without
// atomics; per-face and per-cell updates are one thread each.  Rounding
// follows the reference as compiled (-ffast-math: contractions, a / 3 as
// a * (1/3), p / R / T as p / (R T), the two mass-flux corrections
// reassociated), and the CPU oracle (oracle/ocsl_oracle_flow.c) makes the
// same choices, so results are bit-identical to it.
//
// Boundary kinds: walls, symmetry and empty faces (the shock tube's); the
// host refuses states with inlets or outlets.  Inviscid flows only (the
// explicit viscous stress is not formed here).
#include <cfloat>

#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr double kAlpha = 0.7;  // solvers_common.h:29

// solvers_common.h:32-39 and :69-90 as compiled into cflow_solver_supply.cpp:
// the first product of each a*b + c*d is the contracted one there.
__device__ __forceinline__ double face_avg(double geo, double l, double r)
{
    return fma(geo, l, (1.0 - geo) * r);
}

__device__ __forceinline__ double face_interp(int blended, double geo, double m, double l, double r)
{
    const double up = m >= 0.0 ? l : r;
    return blended ? fma(up, 1.0 - kAlpha, kAlpha * face_avg(geo, l, r)) : up;
}

// tensor.h:128-134, summed from 0 in component order
__device__ __forceinline__ double dot3(double a0, double a1, double a2, double b0, double b1,
                                       double b2)
{
    double r = a0 * b0;
    r = fma(a1, b1, r);
    return fma(a2, b2, r);
}

__device__ __forceinline__ double drho_dp(double R, double gamma, double T)  // cfluid_properties.cpp:79-86
{
    double r = R * T;
    r = r * gamma;
    return 1.0 / r;
}

// Wall faces take the cell pressure extrapolated along the cell-to-face
// vector with the current gradient (cflow_solver.cpp:221-226).
__global__ void bc_pressure_kernel(int n, int nb, FlowDev f)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    if (f.bc_type[g] != OCSL_BC_WALL) return;
    const int c = f.bc_left[g];
    const double* gp = f.pressure_grad;
    const double d = dot3(gp[c], gp[n + c], gp[2 * n + c], f.bc_unit[g], f.bc_unit[nb + g],
                          f.bc_unit[2 * nb + g]);
    f.bc_pressure[g] = fma(d, f.bc_distance[g], f.pressure[c]);
}

// Green-Gauss gradient of the pressure (cflow_solver_supply.cpp:132-177,
// face value weighted by the cells' ap) or of the pressure correction
// (:179-220, face average), for the boundary kinds accepted here: the cell's
// own value on every boundary face.
template <bool CORR>
__global__ void grad_kernel(int n, int nf, int nb, FlowDev f, DevFaces F)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double* v = CORR ? f.pressure_corr : f.pressure;
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int e = F.cell_ptr[c]; e < F.cell_ptr[c + 1]; ++e) {
        const int ent = F.cell_ent[e];
        const int k = ent >> 1;
        const int L = F.left[k], R = F.right[k];
        double fp;
        if (CORR) {
            fp = face_avg(f.geo_aver[k], v[L], v[R]);
        } else {
            const double den = f.ap[L] + f.ap[R];
            fp = fma(f.ap[L], v[L], f.ap[R] * v[R]) / den;
        }
        const double s = (ent & 1) ? -fp : fp;  // the right cell subtracts
        g0 = fma(s, f.area_vector[k], g0);
        g1 = fma(s, f.area_vector[nf + k], g1);
        g2 = fma(s, f.area_vector[2 * nf + k], g2);
    }
    for (int e = F.bc_ptr[c]; e < F.bc_ptr[c + 1]; ++e) {
        const int k = F.bc_ent[e];
        const double pc = v[c];
        g0 = fma(pc, f.bc_area_vector[k], g0);
        g1 = fma(pc, f.bc_area_vector[nb + k], g1);
        g2 = fma(pc, f.bc_area_vector[2 * nb + k], g2);
    }
    const double inv = 1.0 / f.volume[c];
    double* out = CORR ? f.pressure_corr_grad : f.pressure_grad;
    out[c] = inv * g0;
    out[n + c] = inv * g1;
    out[2 * n + c] = inv * g2;
}

// After momentum component d's solve (cflow_solver.cpp:292-301) and its cell
// loop's ap (cflow_solver_cell_face_loops.cpp:168): the residual term
// |u_d - x|, u_d = x, ap += ap_vec_d / 3.
__global__ void velocity_update_kernel(int n, int d, const double* x, FlowDev f, double* res)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double* u = f.velocity + (size_t)d * n;
    res[c] = fabs(u[c] - x[c]);
    u[c] = x[c];
    f.ap[c] = fma(f.ap_vec[(size_t)d * n + c], 1.0 / 3.0, f.ap[c]);  // a / 3 as a * (1/3)
}

// Face mass flux with the pressure-gradient (Rhie-Chow-like) correction
// (cflow_solver_supply.cpp:25-44).
__global__ void face_mdot_kernel(int n, int nf, FlowDev f, int blended)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    const int L = f.left[k], R = f.right[k];
    const size_t n1 = n, n2 = 2 * (size_t)n, f1 = nf, f2 = 2 * (size_t)nf;
    const double qy = (f.volume[L] / f.ap[L] + f.volume[R] / f.ap[R]) *
                      dot3(f.alpha[k], f.alpha[f1 + k], f.alpha[f2 + k], f.area_vector[k],
                           f.area_vector[f1 + k], f.area_vector[f2 + k]);
    const double geo = f.geo_aver[k];
    const double* gp = f.pressure_grad;
    const double pg0 = face_avg(geo, gp[L], gp[R]);
    const double pg1 = face_avg(geo, gp[n1 + L], gp[n1 + R]);
    const double pg2 = face_avg(geo, gp[n2 + L], gp[n2 + R]);
    const double dist = f.distance[k];
    const double d0 = dist * f.unit[k], d1 = dist * f.unit[f1 + k], d2 = dist * f.unit[f2 + k];
    const double t = f.pressure[R] - f.pressure[L] - dot3(pg0, pg1, pg2, d0, d1, d2);
    const double* u = f.velocity;
    const double v0 = face_avg(geo, u[L], u[R]);
    const double v1 = face_avg(geo, u[n1 + L], u[n1 + R]);
    const double v2 = face_avg(geo, u[n2 + L], u[n2 + R]);
    // dot(v_f, A) - Qy t, contracted
    double m = fma(-qy, t, dot3(v0, v1, v2, f.area_vector[k], f.area_vector[f1 + k],
                                f.area_vector[f2 + k]));
    const double rho = face_interp(blended, geo, m, f.density_c[L], f.density_c[R]);
    m *= rho;
    f.qy[k] = qy;
    f.face_density[k] = rho;
    f.mdot[k] = m;
}

// p' = relax_p x, p += p' (cflow_solver.cpp:352-358).
__global__ void pcorr_kernel(int n, const double* x, FlowDev f)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double pc = f.relax_p * x[c];
    f.pressure_corr[c] = pc;
    f.pressure[c] = f.pressure[c] + pc;
}

// Mass-flux correction with the compressible term (cflow_solver_supply.cpp:95-123).
__global__ void correct_mdot_kernel(int nf, FlowDev f, int blended, double R_specific, double gamma)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    const int L = f.left[k], R = f.right[k];
    const double geo = f.geo_aver[k];
    double m = f.mdot[k];
    const double tf = face_interp(blended, geo, m, f.temperature[L], f.temperature[R]);
    const double pcf = face_interp(blended, geo, m, f.pressure_corr[L], f.pressure_corr[R]);
    const double rho = f.face_density[k];
    // the reference's two `Mdot +=`, reassociated: the Qy term goes in first
    const double t = fma(f.qy[k] * rho, f.pressure_corr[L] - f.pressure_corr[R], m);
    f.mdot[k] = fma(m / rho * drho_dp(R_specific, gamma, tf), pcf, t);
}

// Densities from the corrected pressure (cflow_solver.cpp:386-391) and the
// velocity correction u -= relax_u vol grad(p') / ap_vec (:422-426, tensor.h:136-146).
__global__ void correct_cells_kernel(int n, FlowDev f, double R_specific)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    f.density_c[c] = f.pressure[c] / (R_specific * f.temperature[c]);  // p / R / T
    const double s = f.relax_u * f.volume[c];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double a = f.ap_vec[(size_t)d * n + c];
        if (a == 0.0) a = DBL_MIN;
        const double q = f.pressure_corr_grad[(size_t)d * n + c] / a;
        f.velocity[(size_t)d * n + c] = fma(-s, q, f.velocity[(size_t)d * n + c]);
    }
}

// After the enthalpy solve (cflow_solver.cpp:463-474, cfluid_properties.cpp:
// 88-120): residual term |h - x|, h = x, T from h and |u|, Mach number.
__global__ void enthalpy_update_kernel(int n, const double* x, FlowDev f, double* res,
                                       double R_specific, double gamma)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    res[c] = fabs(f.enthalpy[c] - x[c]);
    const double h = x[c];
    f.enthalpy[c] = h;
    const double u0 = f.velocity[c], u1 = f.velocity[(size_t)n + c],
                 u2 = f.velocity[2 * (size_t)n + c];
    // |u|^2 in the order the compiled mag() sums it; |u| |u| folds to it
    const double s = fma(u2, u2, fma(u0, u0, u1 * u1));
    double T = f.Tref + fma(-s, 0.5, h - f.H_formation) / f.cp;
    if (T <= 200.0) T = 200.0;
    if (T >= 6000.0) T = 6000.0;
    f.temperature[c] = T;
    f.mach[c] = sqrt(s) / sqrt(R_specific * T * gamma);
}

// update_timestep (cflow_solver.cpp:505-512).
__global__ void end_step_kernel(int n, FlowDev f)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    for (int d = 0; d < 3; ++d)
        f.velocity_last[(size_t)d * n + c] = f.velocity[(size_t)d * n + c];
    f.density_last[c] = f.density_c[c];
    f.pressure_last[c] = f.pressure[c];
    f.enthalpy_last[c] = f.enthalpy[c];
}

__global__ void take_sum_kernel(const Scalars* sc, double* out) { *out = sc->sum[0]; }

inline int blocks(int count) { return (count + kThreads - 1) / kThreads; }

}  // namespace

void launch_flow_bc_pressure(cudaStream_t st, int n, int nb, const FlowDev& f)
{
    if (nb > 0) bc_pressure_kernel<<<blocks(nb), kThreads, 0, st>>>(n, nb, f);
}

void launch_flow_grad(cudaStream_t st, bool corr, int n, int nf, int nb, const FlowDev& f,
                      const DevFaces& F)
{
    if (n == 0) return;
    if (corr)
        grad_kernel<true><<<blocks(n), kThreads, 0, st>>>(n, nf, nb, f, F);
    else
        grad_kernel<false><<<blocks(n), kThreads, 0, st>>>(n, nf, nb, f, F);
}

void launch_flow_velocity_update(cudaStream_t st, int n, int d, const double* x, const FlowDev& f,
                                 double* res)
{
    if (n > 0) velocity_update_kernel<<<blocks(n), kThreads, 0, st>>>(n, d, x, f, res);
}

void launch_flow_face_mdot(cudaStream_t st, int n, int nf, const FlowDev& f, int blended)
{
    if (nf > 0) face_mdot_kernel<<<blocks(nf), kThreads, 0, st>>>(n, nf, f, blended);
}

void launch_flow_pcorr(cudaStream_t st, int n, const double* x, const FlowDev& f)
{
    if (n > 0) pcorr_kernel<<<blocks(n), kThreads, 0, st>>>(n, x, f);
}

void launch_flow_correct(cudaStream_t st, int n, int nf, const FlowDev& f, int blended,
                         double R_specific, double gamma)
{
    if (nf > 0)
        correct_mdot_kernel<<<blocks(nf), kThreads, 0, st>>>(nf, f, blended, R_specific, gamma);
    if (n > 0) correct_cells_kernel<<<blocks(n), kThreads, 0, st>>>(n, f, R_specific);
}

void launch_flow_enthalpy_update(cudaStream_t st, int n, const double* x, const FlowDev& f,
                                 double* res, double R_specific, double gamma)
{
    if (n > 0)
        enthalpy_update_kernel<<<blocks(n), kThreads, 0, st>>>(n, x, f, res, R_specific, gamma);
}

void launch_flow_end_step(cudaStream_t st, int n, const FlowDev& f)
{
    if (n > 0) end_step_kernel<<<blocks(n), kThreads, 0, st>>>(n, f);
}

void launch_take_sum(cudaStream_t st, const Scalars* sc, double* out)
{
    take_sum_kernel<<<1, 1, 0, st>>>(sc, out);
}

}  // namespace ocsl
