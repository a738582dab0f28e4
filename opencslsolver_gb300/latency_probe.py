"""Dependent-operation latency of the GPU's arithmetic pipes, the bound of
every serial chain on the solve path (triangular sweeps of narrow meshes).

    python -m opencslsolver_gb300.latency_probe

Compiles a small CUDA program for sm_103a (nvcc, a temporary directory) in
which one thread (or a full warp) runs a chain of 4096 dependent FP64 fma /
multiply / divide operations, or FP32 fma, timed with clock64(), and prints
the SM cycles per operation.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

from .build import ARCH, nvcc

SOURCE = r"""
#include <cstdio>
#include <cuda_runtime.h>
__global__ void chain64(int n, double* out, double a, double b, int op, int active)
{
    if ((int)threadIdx.x >= active) return;
    double x = a + threadIdx.x * 1e-3;
    const long long t0 = clock64();
    for (int i = 0; i < n; ++i) {
        if (op == 0) x = fma(x, b, 1e-300);
        else if (op == 1) x = x * b;
        else x = x / b;
    }
    const long long t1 = clock64();
    out[threadIdx.x] = x;
    if (threadIdx.x == 0) out[64] = (double)(t1 - t0) / n;
}
__global__ void chain32(int n, float* out, float a, float b, int active)
{
    if ((int)threadIdx.x >= active) return;
    float x = a;
    const long long t0 = clock64();
    for (int i = 0; i < n; ++i) x = fmaf(x, b, 1e-30f);
    const long long t1 = clock64();
    out[threadIdx.x] = x;
    if (threadIdx.x == 0) out[64] = (float)(t1 - t0) / n;
}
int main()
{
    double* d;
    float* f;
    if (cudaMalloc(&d, 128 * sizeof(double)) != cudaSuccess) return 1;
    if (cudaMalloc(&f, 128 * sizeof(float)) != cudaSuccess) return 1;
    const char* names[3] = {"fma", "mul", "div"};
    for (int op = 0; op < 3; ++op)
        for (int act : {1, 32}) {
            chain64<<<1, 32>>>(4096, d, 1.0000001, 0.9999999, op, act);
            double h[65];
            cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
            std::printf("fp64 %s, %2d active lanes: %.1f cycles per dependent op\n", names[op], act,
                        h[64]);
        }
    for (int act : {1, 32}) {
        chain32<<<1, 32>>>(4096, f, 1.0000001f, 0.9999999f, act);
        float h[65];
        cudaMemcpy(h, f, sizeof h, cudaMemcpyDeviceToHost);
        std::printf("fp32 fma, %2d active lanes: %.1f cycles per dependent op\n", act, h[64]);
    }
    const cudaError_t e = cudaGetLastError();
    std::printf("%s\n", cudaGetErrorString(e));
    return e == cudaSuccess ? 0 : 1;
}
"""


def main() -> int:
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "latency.cu")
        exe = os.path.join(d, "latency")
        with open(src, "w") as fh:
            fh.write(SOURCE)
        subprocess.run([nvcc(), *ARCH, "-O3", "-o", exe, src], check=True)
        return subprocess.run([exe]).returncode


if __name__ == "__main__":
    raise SystemExit(main())
