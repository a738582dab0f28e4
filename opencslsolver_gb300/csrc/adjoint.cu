// Kernels that move values between two layouts of one pattern, and the
// outer product on the pattern (no reference counterpart).
//
// Adjoint: for x = A^-1 b and a loss L(x) with gradient g = dL/dx,
//   A^T lambda = g,   dL/db = lambda,   dL/dA_ij = -lambda_i x_j on A's pattern;
// the transposed system reuses the forward machinery on the transposed CSR.
// Multicolour ordering: a tolerance-mode solve runs on the permuted system
// P A P^T, P b, P x and scatters x back.
#include "ocsl_internal.cuh"

namespace ocsl {

namespace {

// valT[k'] = val[perm[k']]: the values of A^T in its own CSR order.
__global__ void __launch_bounds__(kThreads)
gather_values_kernel(long long nnz, const int* __restrict__ perm, const double* __restrict__ val,
                     double* __restrict__ out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz; k += stride)
        out[k] = __ldg(val + __ldg(perm + k));
}

// out[perm[k]] = in[k]: a permuted vector back to the original order.
__global__ void __launch_bounds__(kThreads)
scatter_values_kernel(long long n, const int* __restrict__ perm, const double* __restrict__ in,
                      double* __restrict__ out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride)
        out[__ldg(perm + k)] = in[k];
}

// out[k] = (alpha * u[i]) * v[col[k]] for entry k of row i; 0 on phantom
// entries (col < 0), whose values the reference never reads.
__global__ void __launch_bounds__(kThreads)
pattern_outer_kernel(int n, const int* __restrict__ rp, const int* __restrict__ col, double alpha,
                     const double* __restrict__ u, const double* __restrict__ v,
                     double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double au = alpha * u[i];
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
        const int j = col[k];
        out[k] = j >= 0 ? au * __ldg(v + j) : 0.0;
    }
}

}  // namespace

void launch_gather_values(cudaStream_t st, long long nnz, const int* perm, const double* val,
                          double* out)
{
    if (nnz <= 0) return;
    long long blocks = (nnz + kThreads - 1) / kThreads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    gather_values_kernel<<<(int)blocks, kThreads, 0, st>>>(nnz, perm, val, out);
}

void launch_scatter_values(cudaStream_t st, long long n, const int* perm, const double* in,
                           double* out)
{
    if (n <= 0) return;
    long long blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    scatter_values_kernel<<<(int)blocks, kThreads, 0, st>>>(n, perm, in, out);
}

void launch_pattern_outer(cudaStream_t st, const DevPattern& P, double alpha, const double* u,
                          const double* v, double* out)
{
    if (P.n == 0) return;
    pattern_outer_kernel<<<(P.n + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        P.n, P.rp, P.col, alpha, u, v, out);
}

}  // namespace ocsl
