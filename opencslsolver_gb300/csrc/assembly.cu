// Face-loop coefficient assembly on the GPU: the flow solver's momentum,
// pressure-correction and enthalpy equations (cflow_solver_cell_face_loops.cpp:37-446,
// solvers_common.h:32-151) and the heat solver's conduction equation
// (cheat_solver.cpp:32-65).
//
// The reference scatters every face's contributions into the CSR with atomic
// adds from an OpenMP face loop, then a boundary-face loop, then a cell loop.
// Here one thread owns one cell (one CSR row and one entry of b): it walks
// the cell's faces in ascending face order (a per-cell incidence list built
// once per mesh, with the CSR slot of each off-diagonal entry), evaluates
// each face's contributions and keeps the ones that land in its row, then its
// boundary faces, then its cell terms.  No atomics, nothing written by two
// threads, and every entry is the running sum in the order the reference's
// loops produce on one thread -- so the result equals the single-thread
// reference up to its -ffast-math contractions, and the oracle restatement
// (oracle/ocsl_oracle_assembly.c, same contraction choices) bit for bit.
//
// Memory: per cell one pass over its incidence entries (face index, slot),
// the face arrays of those faces and the neighbour's cell fields; every face
// is evaluated by both of its cells (the evaluation is a few flops, the
// bytes dominate).  Bound: HBM / L2 gathers.
#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

constexpr double kAlpha = 0.7;  // solvers_common.h:29

enum Target { T_LL, T_LR, T_RR, T_RL, T_BL, T_BR, T_ML, T_MR };

// The running sums of one cell's row while it walks a face: a face
// contribution with target t lands in the diagonal, this face's off-diagonal
// slot, b or total_mdot when t names the cell's side of the face, else
// nowhere -- in call order, so every sum is the reference's sequence of
// additions.  (Targets are constants at every call site once inlined.)
struct Sink {
    bool left;
    double a, b, tm, off;
    __device__ __forceinline__ void add(int t, double x)
    {
        if (left) {
            if (t == T_LL) a += x;
            else if (t == T_LR) off += x;
            else if (t == T_BL) b += x;
            else if (t == T_ML) tm += x;
        } else {
            if (t == T_RR) a += x;
            else if (t == T_RL) off += x;
            else if (t == T_BR) b += x;
            else if (t == T_MR) tm += x;
        }
    }
};

__device__ __forceinline__ double mu(const ocsl_assembly& q, double T)
{
    return q.sutherland[0] * (T * sqrt(T)) / (T + q.sutherland[1]);  // cfluid_properties.cpp:123
}

__device__ __forceinline__ double drho_dp(const ocsl_assembly& q, double T)  // :79-86
{
    double r = q.R_specific * T;
    r = r * q.gamma;
    return 1.0 / r;
}

__device__ __forceinline__ double face_avg(double geo, double l, double r)  // solvers_common.h:32
{
    return fma(1.0 - geo, r, geo * l);
}

__device__ __forceinline__ double face_interp(int blended, double geo, double m, double l, double r)
{
    if (m >= 0.0) return blended ? fma(kAlpha, face_avg(geo, l, r), l * (1.0 - kAlpha)) : l;
    if (m < 0.0) return blended ? fma(kAlpha, face_avg(geo, l, r), r * (1.0 - kAlpha)) : r;
    return 0.0;
}

// solvers_common.h:96-135
__device__ __forceinline__ void convective(Sink& o, int blended, double geo, double m, double l,
                                           double r)
{
    if (m >= 0.0) {
        o.add(T_LL, m);
        o.add(T_RL, -m);
        if (blended) {
            const double val = kAlpha * (face_avg(geo, l, r) - l);
            o.add(T_BL, -m * val);
            o.add(T_BR, m * val);
        }
    } else if (m < 0.0) {
        o.add(T_LR, m);
        o.add(T_RR, -m);
        if (blended) {
            const double val = kAlpha * (face_avg(geo, l, r) - r);
            o.add(T_BL, -m * val);
            o.add(T_BR, m * val);
        }
    }
}

// solvers_common.h:42-53
__device__ __forceinline__ void diffusive(Sink& o, double D)
{
    o.add(T_LL, D);
    o.add(T_LR, -D);
    o.add(T_RR, D);
    o.add(T_RL, -D);
}

// One interior face's contributions, in the reference's call order.  mu_f
// and pdum_f: the face's viscosity and pressure coefficient computed once per
// face by the iteration (null: evaluated here, the same expressions).
__device__ __forceinline__ void face_ops(const ocsl_assembly& q, const ocsl_flow_state& st, int n,
                                         int nf, int f, int L, int R, const double* mu_f,
                                         const double* pdum_f, Sink& o)
{
    if (q.equation == OCSL_EQ_HEAT) {  // cheat_solver.cpp:32-37 (reads no flow state)
        diffusive(o, q.thermal_diffusivity * st.ksi_A[f]);
        return;
    }
    const double g = st.geo_aver[f], m = st.mdot[f];
    if (q.equation == OCSL_EQ_MOMENTUM) {  // :37-57
        const double* u = st.velocity + (size_t)q.dimension * n;
        convective(o, q.blended, g, m, u[L], u[R]);
        if (q.viscous) {
            double D = mu_f ? mu_f[f] : mu(q, face_avg(g, st.temperature[L], st.temperature[R]));
            D = D * st.ksi_A[f];
            diffusive(o, D);
            const double sp = st.stress[(size_t)q.dimension * nf + f];
            o.add(T_BL, sp);
            o.add(T_BR, -sp);
        }
    } else if (q.equation == OCSL_EQ_PRESSURE) {  // :176-211
        o.add(T_BL, -m);
        o.add(T_BR, m);
        o.add(T_ML, m);
        o.add(T_MR, -m);
        double dum;
        if (pdum_f) {
            dum = pdum_f[f];
        } else {
            const double Tf = face_interp(q.blended, g, m, st.temperature[L], st.temperature[R]);
            dum = drho_dp(q, Tf);
            dum = dum / st.density[f];
            dum *= m;
        }
        convective(o, q.blended, g, dum, st.pressure_corr[L], st.pressure_corr[R]);
        diffusive(o, st.qy[f] * st.density[f]);
    } else {  // :334-345
        convective(o, q.blended, g, m, st.enthalpy[L], st.enthalpy[R]);
        double D = mu_f ? mu_f[f] : mu(q, face_avg(g, st.temperature[L], st.temperature[R]));
        D = D / q.prandtl * st.ksi_A[f];
        diffusive(o, D);
    }
}

struct Acc {
    double a = 0.0;   // diagonal
    double b = 0.0;
    double tm = 0.0;  // total_mdot
};

__device__ __forceinline__ void neumann_zero(Acc& c, double m)  // solvers_common.h:138-151
{
    if (m >= 0.0)
        c.a += m;
    else if (m < 0.0)
        c.a += m;
}

// One boundary face of cell P, in the reference's call order.
__device__ void bc_apply(const ocsl_assembly& q, const ocsl_flow_state& st, int n, int nb, int k,
                         int P, Acc& c)
{
    if (q.equation == OCSL_EQ_HEAT) {  // cheat_solver.cpp:39-56
        if (st.bc_thermal[k] == OCSL_THERMAL_CONSTANT_TEMPERATURE) {
            const double D = q.thermal_diffusivity * st.bc_ksi_A[k];
            c.a += D;
            c.b += D * st.bc_temperature[k];
        }
        return;
    }
    const int type = st.bc_type[k];
    const double m = st.bc_mdot[k];
    const double bv = st.bc_value ? st.bc_value[k] : 0.0;
    const int d = q.dimension;
    if (q.equation == OCSL_EQ_MOMENTUM) {  // :75-131
        if (type == OCSL_BC_WALL && q.viscous && st.bc_wall[k] == OCSL_WALL_NO_SLIP) {
            const double inv = 1.0 / st.bc_area[k];
            double nv[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) nv[e] = inv * st.bc_area_vector[(size_t)e * nb + k];
            double D = mu(q, st.temperature[P]);
            D *= st.bc_area[k] / st.bc_perp_dist[k];
            c.a += D * (1.0 - (nv[d] * nv[d]));
            double dum = 0.0;
            for (int i = d + 1; i < d + 3; ++i) {
                const int i_ = i % 3;
                dum = fma(st.velocity[(size_t)i_ * n + P] * nv[i_], nv[d], dum);
            }
            c.b += D * dum;
        }
        if (type == OCSL_BC_VELOCITY_INLET || type == OCSL_BC_SUPERSONIC_INLET)
            c.b += -(m * st.bc_velocity[(size_t)d * nb + k]);
        if (type == OCSL_BC_PRESSURE_OUTLET) c.a += m;
    } else if (q.equation == OCSL_EQ_PRESSURE) {  // :214-270
        if (type == OCSL_BC_VELOCITY_INLET) {
            c.b += -m;
            c.tm += m;
            double dum = drho_dp(q, st.bc_temperature[k]) / st.density_c[P];
            dum *= m;
            neumann_zero(c, dum);
        }
        if (type == OCSL_BC_SUPERSONIC_INLET) {
            c.b += -m;
            c.tm += m;
            const double D = st.bc_qy[k] * st.bc_density[k];
            c.a += D;
            c.b += D * bv;
        }
        if (type == OCSL_BC_PRESSURE_OUTLET) {
            c.b += -m;
            c.tm += m;
            if (st.bc_supersonic[k]) {
                double dum = drho_dp(q, st.temperature[P]) / st.density_c[P];
                dum *= m;
                neumann_zero(c, dum);
            } else {
                const double D = st.bc_qy[k] * st.density_c[P];
                c.a += D;
                c.b += D * bv;
            }
        }
    } else {  // :350-410
        if (type == OCSL_BC_VELOCITY_INLET || type == OCSL_BC_SUPERSONIC_INLET) {
            c.b += -(m * st.bc_enthalpy[k]);
            double D = mu(q, st.bc_temperature[k]);
            D *= q.prandtl * st.bc_ksi_A[k];
            c.a += D;
            c.b += D * st.bc_enthalpy[k];
        }
        if (type == OCSL_BC_PRESSURE_OUTLET) neumann_zero(c, m);
    }
}

__global__ void __launch_bounds__(kThreads)
assemble_kernel(DevPattern P, DevFaces F, ocsl_assembly q, ocsl_flow_state st, double* value,
                double* bvec, double* x0, double* ap, double* total_mdot, const double* face_mu,
                const double* face_pdum)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = P.n;
    if (i >= n) return;
    const int r0 = P.rp[i], r1 = P.rp[i + 1];
    for (int k = r0; k < r1; ++k) value[k] = 0.0;  // clear (phantoms stay 0)
    Acc c;
    Sink o;
    o.a = 0.0;
    o.b = 0.0;
    o.tm = 0.0;
    // interior faces, ascending
    for (int e = F.cell_ptr[i]; e < F.cell_ptr[i + 1]; ++e) {
        const int ent = F.cell_ent[e];
        const int f = ent >> 1;
        const int k = F.cell_slot[e];
        o.left = (ent & 1) == 0;
        o.off = value[k];  // continues this slot's sum (0 unless an earlier face shares it)
        face_ops(q, st, n, F.nf, f, F.left[f], F.right[f], face_mu, face_pdum, o);
        value[k] = o.off;
    }
    c.a = o.a;
    c.b = o.b;
    c.tm = o.tm;
    // boundary faces, ascending
    for (int e = F.bc_ptr[i]; e < F.bc_ptr[i + 1]; ++e) bc_apply(q, st, n, F.nb, F.bc_ent[e], i, c);
    // cell terms (:143-172 momentum, :273-296 pressure, :413-436 enthalpy)
    const double vol = st.volume[i];
    const double urf = q.implicit_underrelaxation;
    double xi;
    if (q.equation == OCSL_EQ_MOMENTUM) {
        const int d = q.dimension;
        const double ul = st.velocity_last[(size_t)d * n + i];
        double dum = 0.0, dum2 = 0.0;
        if (q.transient) {
            dum = vol / st.delta_t[i];
            dum2 = dum * st.density_c[i];
            c.a += dum2;
            dum2 = dum * (ul * st.density_last[i]);
        }
        dum2 = fma(-st.pressure_grad[(size_t)d * n + i], vol, dum2);
        c.b += dum2;
        if (!q.transient) {
            dum = c.a;
            c.a = dum / urf;
            dum = (1.0 - urf) / urf * dum * ul;
            c.b += dum;
        }
        xi = st.velocity[(size_t)d * n + i];
        c.tm = 0.0;
    } else if (q.equation == OCSL_EQ_HEAT) {  // cheat_solver.cpp:58-66
        const double dum = vol / st.delta_t[i];
        c.a += dum;
        c.b += st.temperature[i] * dum;
        xi = st.temperature[i];
        c.tm = 0.0;
    } else if (q.equation == OCSL_EQ_PRESSURE) {
        if (q.transient) {
            const double dum = vol / st.delta_t[i];
            double dum2 = dum * (st.density_c[i] - st.density_last[i]);
            c.b += -dum2;
            dum2 = dum * drho_dp(q, st.temperature[i]);
            c.a += dum2;
        } else {
            c.a = c.a / urf;
        }
        xi = st.pressure_corr[i];
    } else {
        if (q.transient) {
            const double dum = vol / st.delta_t[i];
            double dum2 = dum * st.density_c[i];
            c.a += dum2;
            dum2 = dum * (st.enthalpy_last[i] * st.density_last[i]);
            dum2 = fma((st.pressure[i] - st.pressure_last[i]) / st.delta_t[i], vol, dum2);
            c.b += dum2;
        } else {
            double dum = c.a;
            c.a = dum / urf;
            dum = (1.0 - urf) / urf * dum * st.enthalpy_last[i];
            c.b += dum;
        }
        xi = st.enthalpy[i];
        c.tm = 0.0;
    }
    value[P.diag[i]] = c.a;
    bvec[i] = c.b;
    x0[i] = xi;
    if (ap) ap[i] = c.a;
    if (total_mdot) total_mdot[i] = c.tm;
}

__global__ void __launch_bounds__(kThreads)
bc_value_grad_kernel(DevFaces F, ocsl_assembly q, ocsl_flow_state st, const double* lambda,
                     double* grad)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= F.nb) return;
    const int P = F.bc_left[k];
    const int type = st.bc_type[k];
    double D = 0.0;
    if (q.equation == OCSL_EQ_PRESSURE) {
        if (type == OCSL_BC_SUPERSONIC_INLET) D = st.bc_qy[k] * st.bc_density[k];
        if (type == OCSL_BC_PRESSURE_OUTLET && !st.bc_supersonic[k])
            D = st.bc_qy[k] * st.density_c[P];
    }
    grad[k] = lambda[P] * D;
}

}  // namespace

void launch_assemble(cudaStream_t st, const DevPattern& P, const DevFaces& F,
                     const ocsl_assembly& q, const ocsl_flow_state& s, double* value, double* b,
                     double* x0, double* ap, double* total_mdot, const double* face_mu,
                     const double* face_pdum)
{
    if (P.n == 0) return;
    assemble_kernel<<<(P.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        P, F, q, s, value, b, x0, ap, total_mdot, face_mu, face_pdum);
}

void launch_bc_value_grad(cudaStream_t st, const DevFaces& F, const ocsl_assembly& q,
                          const ocsl_flow_state& s, const double* lambda, double* grad)
{
    if (F.nb == 0) return;
    bc_value_grad_kernel<<<(F.nb + kThreads - 1) / kThreads, kThreads, 0, st>>>(F, q, s, lambda,
                                                                              grad);
}

}  // namespace ocsl
