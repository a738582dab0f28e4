// The rest of the SIMPLE inner iteration on the device
// (CFlow_solver::iterate, cflow_solver.cpp:229-476, and the routines of
// cflow_solver_supply.cpp it calls), around the face-loop assembly and the
// linear solves: boundary conditions, Green-Gauss pressure and
// pressure-correction gradients, the explicit viscous stress, face and
// boundary mass fluxes and their correction, the field updates after each
// solve, and the end-of-step copy (update_timestep, :503-512).
//
// Every kernel is owner-computes, like the assembly: a per-cell gradient is
// one thread walking the cell's faces in ascending face order and then its
// boundary faces (the incidence lists of ocsl_set_faces), so each component
// is the running sum the reference's serial face loops produce, without
// atomics; per-face, per-boundary-face and per-cell updates are one thread
// each.  Rounding follows the reference as compiled (-ffast-math:
// contractions, a / 3 as a * (1/3), p / R / T as p / (R T), the two
// mass-flux corrections reassociated), and the CPU oracle
// (oracle/ocsl_oracle_flow.c) makes the same choices, so results are
// bit-identical to it.
#include <cfloat>

#include "division.cuh"
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

__device__ __forceinline__ double dot3(const double* a, size_t sa, size_t ka, const double* b,
                                       size_t sb, size_t kb)
{
    return dot3(a[ka], a[sa + ka], a[2 * sa + ka], b[kb], b[sb + kb], b[2 * sb + kb]);
}

// |u|^2 in the order the compiled mag() sums it
__device__ __forceinline__ double usq(double u0, double u1, double u2)
{
    return fma(u2, u2, fma(u0, u0, u1 * u1));
}

// cfluid_properties.cpp:46-51 (p / R / T under -ffast-math), :79-86, :89-96,
// :98-106, :123-128
__device__ __forceinline__ double density(const FlowDev& f, double p, double T)
{
    return p / (f.R * T);
}

__device__ __forceinline__ double drho_dp(const FlowDev& f, double T)
{
    double r = f.R * T;
    r = r * f.gamma;
    return 1.0 / r;
}

__device__ __forceinline__ double sound(const FlowDev& f, double T)
{
    return sqrt(f.R * T * f.gamma);
}

__device__ __forceinline__ double enthalpy(const FlowDev& f, double T, double u0, double u1,
                                           double u2)
{
    return fma(usq(u0, u1, u2), 0.5, fma(T - f.Tref, f.cp, f.H_formation));
}

__device__ __forceinline__ double viscosity(const FlowDev& f, double T)
{
    return f.suth0 * (T * sqrt(T)) / (T + f.suth1);
}

// The face-loop translation unit's forms (cflow_solver_cell_face_loops.cpp
// as compiled: the other product of a*b + c*d is the contracted one there),
// for the per-face values the assembly reads (assembly.cu uses the same).
__device__ __forceinline__ double loop_face_avg(double geo, double l, double r)
{
    return fma(1.0 - geo, r, geo * l);
}

__device__ __forceinline__ double loop_face_interp(int blended, double geo, double m, double l,
                                                   double r)
{
    if (m >= 0.0) return blended ? fma(kAlpha, loop_face_avg(geo, l, r), l * (1.0 - kAlpha)) : l;
    if (m < 0.0) return blended ? fma(kAlpha, loop_face_avg(geo, l, r), r * (1.0 - kAlpha)) : r;
    return 0.0;
}

// CFlow_solver::set_boundary_conditions (cflow_solver.cpp:195-227).  Outlets
// read their density from the boundary pressure of the previous iteration and
// then mark themselves supersonic on both branches, as the reference does.
__global__ void set_bc_kernel(int n, int nb, FlowDev f)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int c = f.bc_left[g];
    const size_t N = n, B = nb;
    switch (f.bc_type[g]) {
    case OCSL_BC_VELOCITY_INLET: {
        const double v0 = f.bc_velocity[g], v1 = f.bc_velocity[B + g], v2 = f.bc_velocity[2 * B + g];
        f.bc_pressure[g] = f.pressure[c];
        const double rho = density(f, f.pressure[c], f.bc_temperature[g]);
        f.bc_density[g] = rho;
        f.bc_mdot[g] = rho * dot3(v0, v1, v2, f.bc_area_vector[g], f.bc_area_vector[B + g],
                                  f.bc_area_vector[2 * B + g]);
        f.bc_enthalpy[g] = enthalpy(f, f.bc_temperature[g], v0, v1, v2);
        break;
    }
    case OCSL_BC_PRESSURE_OUTLET: {
        const double u0 = f.velocity[c], u1 = f.velocity[N + c], u2 = f.velocity[2 * N + c];
        const double T = f.temperature[c];
        f.bc_temperature[g] = T;
        f.bc_velocity[g] = u0;
        f.bc_velocity[B + g] = u1;
        f.bc_velocity[2 * B + g] = u2;
        f.bc_density[g] = density(f, f.bc_pressure[g], T);
        f.bc_enthalpy[g] = enthalpy(f, T, u0, u1, u2);
        const double speed = f.bc_mdot[g] / (f.density_c[c] * f.bc_area[g]);
        f.bc_supersonic[g] = 1;
        f.bc_pressure[g] = speed >= sound(f, T) ? f.pressure[c] : f.bc_out_pressure[g];
        break;
    }
    case OCSL_BC_WALL: {
        const double d = dot3(f.pressure_grad, N, c, f.bc_unit, B, g);
        f.bc_pressure[g] = fma(d, f.bc_distance[g], f.pressure[c]);
        break;
    }
    default: break;  // supersonic inlets, symmetry, empty faces: nothing
    }
}

// Green-Gauss gradient of the pressure (cflow_solver_supply.cpp:132-177, face
// value weighted by the cells' ap) or of the pressure correction (:179-220,
// face average).  Boundary faces add the cell's own value, except that
// outlets and supersonic inlets add their boundary pressure to the pressure
// gradient, and add nothing to the correction's unless the outlet is
// supersonic (supersonic inlets never).
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
        g1 = fma(s, f.area_vector[(size_t)nf + k], g1);
        g2 = fma(s, f.area_vector[2 * (size_t)nf + k], g2);
    }
    for (int e = F.bc_ptr[c]; e < F.bc_ptr[c + 1]; ++e) {
        const int k = F.bc_ent[e];
        const int kind = f.bc_type[k];
        double fv = v[c];
        if (kind == OCSL_BC_PRESSURE_OUTLET || kind == OCSL_BC_SUPERSONIC_INLET) {
            if (!CORR) fv = f.bc_pressure[k];
            else if (kind == OCSL_BC_SUPERSONIC_INLET || !f.bc_supersonic[k]) continue;
        }
        g0 = fma(fv, f.bc_area_vector[k], g0);
        g1 = fma(fv, f.bc_area_vector[(size_t)nb + k], g1);
        g2 = fma(fv, f.bc_area_vector[2 * (size_t)nb + k], g2);
    }
    const double inv = 1.0 / f.volume[c];
    double* out = CORR ? f.pressure_corr_grad : f.pressure_grad;
    out[c] = inv * g0;
    out[(size_t)n + c] = inv * g1;
    out[2 * (size_t)n + c] = inv * g2;
}

// The explicit part of the viscous stress (cflow_solver_cell_face_loops.cpp:
// 25-35, tensor.h:194-225): mu(T_f) (grad u^T - 2/3 div u I) A, the gradients
// taken along the cell-to-cell direction; T_f is the face-loop translation
// unit's face average.  mu(T_f) is kept per face (face_mu) for the momentum
// and enthalpy assemblies of the iteration, which evaluate the same
// expression on the same temperatures; without viscosity only face_mu.
template <bool VISCOUS>
__global__ void stress_kernel(int n, int nf, FlowDev f)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    const int L = f.left[k], R = f.right[k];
    const double geo = f.geo_aver[k];
    const double m = viscosity(f, loop_face_avg(geo, f.temperature[L], f.temperature[R]));
    f.face_mu[k] = m;
    if constexpr (!VISCOUS) return;
    const size_t N = n, NF = nf;
    double dv[3], un[3], A[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dv[d] = f.velocity[d * N + R] - f.velocity[d * N + L];
        un[d] = f.unit[d * NF + k];
        A[d] = f.area_vector[d * NF + k];
    }
    // the nine quotients (dv_j un_i) / dist over one distance: one IEEE
    // division (division.cuh); div u sums the three with i = j
    const Recip dist = recip(f.distance[k]);
    double g[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) g[i][j] = divide(dv[j] * un[i], dist);  // transpose(grad u)
    double div = g[0][0];
    div = div + g[1][1];
    div = div + g[2][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double t[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) t[j] = g[i][j];
        t[i] = fma(-(2.0 / 3.0), div, t[i]);
#pragma unroll
        for (int j = 0; j < 3; ++j) t[j] = m * t[j];
        f.stress[i * NF + k] = dot3(t[0], t[1], t[2], A[0], A[1], A[2]);
    }
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
    const double ap = fma(f.ap_vec[(size_t)d * n + c], 1.0 / 3.0, f.ap[c]);  // a / 3 as a * (1/3)
    f.ap[c] = ap;
    // ap is final after the last component: vol / ap once per cell for the
    // face and boundary mass fluxes (each face side divided again before)
    if (d == 2) f.vol_ap[c] = f.volume[c] / ap;
}

// Face mass flux with the pressure-gradient (Rhie-Chow-like) correction
// (cflow_solver_supply.cpp:25-44).
__global__ void face_mdot_kernel(int n, int nf, FlowDev f, int blended)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    const int L = f.left[k], R = f.right[k];
    const size_t n1 = n, n2 = 2 * (size_t)n, f1 = nf, f2 = 2 * (size_t)nf;
    const double qy = (f.vol_ap[L] + f.vol_ap[R]) *
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
    // the pressure equation's convective coefficient of this face
    // (cflow_solver_cell_face_loops.cpp:186-191), once per face
    const double tf = loop_face_interp(blended, geo, m, f.temperature[L], f.temperature[R]);
    double dum = drho_dp(f, tf);
    dum = dum / rho;
    dum *= m;
    f.face_pdum[k] = dum;
}

// Boundary mass fluxes (cflow_solver_supply.cpp:51-93).
__global__ void bc_mdot_kernel(int n, int nb, FlowDev f)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int c = f.bc_left[g];
    const int kind = f.bc_type[g];
    const size_t N = n, B = nb;
    if (kind == OCSL_BC_VELOCITY_INLET) {
        f.bc_mdot[g] = density(f, f.pressure[c], f.bc_temperature[g]) *
                       dot3(f.bc_velocity, B, g, f.bc_area_vector, B, g);
    } else if (kind == OCSL_BC_SUPERSONIC_INLET) {
        f.bc_qy[g] = f.vol_ap[c] * dot3(f.bc_alpha, B, g, f.bc_area_vector, B, g);
    } else if (kind == OCSL_BC_PRESSURE_OUTLET) {
        const double ua = dot3(f.velocity, N, c, f.bc_area_vector, B, g);
        if (f.bc_supersonic[g]) {
            f.bc_mdot[g] = density(f, f.pressure[c], f.temperature[c]) * ua;
            f.bc_qy[g] = 1.0;
        } else {
            const double qy = f.vol_ap[c] * dot3(f.bc_alpha, B, g, f.bc_area_vector, B, g);
            const double dist = f.bc_distance[g];
            const double t = f.bc_pressure[g] - f.pressure[c] -
                             0.5 * dot3(f.pressure_grad[c], f.pressure_grad[N + c],
                                        f.pressure_grad[2 * N + c], dist * f.bc_unit[g],
                                        dist * f.bc_unit[B + g], dist * f.bc_unit[2 * B + g]);
            f.bc_qy[g] = qy;
            f.bc_mdot[g] = fma(-qy, t, ua) * f.bc_density[g];
        }
    }
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

// Boundary pressures that follow the corrected cell pressure (cflow_solver.cpp:361-372).
__global__ void bc_pcorr_kernel(int nb, FlowDev f)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int kind = f.bc_type[g];
    if (kind == OCSL_BC_VELOCITY_INLET || (kind == OCSL_BC_PRESSURE_OUTLET && f.bc_supersonic[g]))
        f.bc_pressure[g] = f.pressure[f.bc_left[g]];
}

// Mass-flux correction with the compressible term (cflow_solver_supply.cpp:95-123).
__global__ void correct_mdot_kernel(int nf, FlowDev f, int blended)
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
    f.mdot[k] = fma(m / rho * drho_dp(f, tf), pcf, t);
}

// Densities from the corrected pressure (cflow_solver.cpp:386-391) and the
// velocity correction u -= relax_u vol grad(p') / ap_vec (:422-426, tensor.h:136-146).
__global__ void correct_cells_kernel(int n, FlowDev f)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    f.density_c[c] = density(f, f.pressure[c], f.temperature[c]);
    const double s = f.relax_u * f.volume[c];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double a = f.ap_vec[(size_t)d * n + c];
        if (a == 0.0) a = DBL_MIN;
        const double q = f.pressure_corr_grad[(size_t)d * n + c] / a;
        f.velocity[(size_t)d * n + c] = fma(-s, q, f.velocity[(size_t)d * n + c]);
    }
}

// Boundary faces after the correction: the subsonic outlets' mass flux
// (cflow_solver_supply.cpp:113-123, with the density before its update) and
// the boundary densities (cflow_solver.cpp:393-410).
__global__ void correct_bc_kernel(int nb, FlowDev f)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int c = f.bc_left[g];
    const int kind = f.bc_type[g];
    if (kind == OCSL_BC_PRESSURE_OUTLET && !f.bc_supersonic[g])
        f.bc_mdot[g] = fma(f.bc_qy[g] * f.bc_density[g], f.pressure_corr[c], f.bc_mdot[g]);
    if (kind == OCSL_BC_VELOCITY_INLET)
        f.bc_density[g] = density(f, f.pressure[c], f.bc_temperature[g]);
    else if (kind == OCSL_BC_PRESSURE_OUTLET)
        f.bc_density[g] =
            density(f, f.bc_supersonic[g] ? f.pressure[c] : f.bc_pressure[g], f.temperature[c]);
}

// After the enthalpy solve (cflow_solver.cpp:463-474, cfluid_properties.cpp:
// 88-120): residual term |h - x|, h = x, T from h and |u| clamped to
// [200, 6000], Mach = |u| / sqrt(R T gamma).
__global__ void enthalpy_update_kernel(int n, const double* x, FlowDev f, double* res)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    res[c] = fabs(f.enthalpy[c] - x[c]);
    const double h = x[c];
    f.enthalpy[c] = h;
    const double s = usq(f.velocity[c], f.velocity[(size_t)n + c], f.velocity[2 * (size_t)n + c]);
    double T = f.Tref + fma(-s, 0.5, h - f.H_formation) / f.cp;  // |u| |u| folds to |u|^2
    if (T <= 200.0) T = 200.0;
    if (T >= 6000.0) T = 6000.0;
    f.temperature[c] = T;
    f.mach[c] = sqrt(s) / sound(f, T);
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

void launch_flow_set_bc(cudaStream_t st, int n, int nb, const FlowDev& f)
{
    if (nb > 0) set_bc_kernel<<<blocks(nb), kThreads, 0, st>>>(n, nb, f);
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

void launch_flow_stress(cudaStream_t st, int n, int nf, const FlowDev& f, bool viscous)
{
    if (nf == 0) return;
    if (viscous)
        stress_kernel<true><<<blocks(nf), kThreads, 0, st>>>(n, nf, f);
    else
        stress_kernel<false><<<blocks(nf), kThreads, 0, st>>>(n, nf, f);
}

void launch_flow_velocity_update(cudaStream_t st, int n, int d, const double* x, const FlowDev& f,
                                 double* res)
{
    if (n > 0) velocity_update_kernel<<<blocks(n), kThreads, 0, st>>>(n, d, x, f, res);
}

void launch_flow_face_mdot(cudaStream_t st, int n, int nf, int nb, const FlowDev& f, int blended)
{
    if (nf > 0) face_mdot_kernel<<<blocks(nf), kThreads, 0, st>>>(n, nf, f, blended);
    if (nb > 0) bc_mdot_kernel<<<blocks(nb), kThreads, 0, st>>>(n, nb, f);
}

void launch_flow_pcorr(cudaStream_t st, int n, int nb, const double* x, const FlowDev& f)
{
    if (n > 0) pcorr_kernel<<<blocks(n), kThreads, 0, st>>>(n, x, f);
    if (nb > 0) bc_pcorr_kernel<<<blocks(nb), kThreads, 0, st>>>(nb, f);
}

void launch_flow_correct(cudaStream_t st, int n, int nf, int nb, const FlowDev& f, int blended)
{
    if (nf > 0) correct_mdot_kernel<<<blocks(nf), kThreads, 0, st>>>(nf, f, blended);
    if (n > 0) correct_cells_kernel<<<blocks(n), kThreads, 0, st>>>(n, f);
    if (nb > 0) correct_bc_kernel<<<blocks(nb), kThreads, 0, st>>>(nb, f);
}

void launch_flow_enthalpy_update(cudaStream_t st, int n, const double* x, const FlowDev& f,
                                 double* res)
{
    if (n > 0) enthalpy_update_kernel<<<blocks(n), kThreads, 0, st>>>(n, x, f, res);
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
