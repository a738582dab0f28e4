"""The allocation-free entry point, ocsl_dot_noalloc.

It serves callers that cannot call cudaMalloc (hosts whose device memory
another allocator has already reserved, or whose plugins may not allocate
because cudaMalloc and cudaFree can synchronise the device): its scratch is a
fixed device array inside the library.  This test calls it through the C ABI twice in a row on the same
inputs and checks each result against the context-based ocsl_dot_device.
Both use the same fixed reduction order, so the tolerance is 0 (bit-equal).
The file name makes pytest collect it last; it passes alone or after the
rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dot_noalloc_matches_dot_device(lib_built, torch_cuda):
    import opencslsolver_gb300 as ocsl

    torch = torch_cuda
    L = lib_built
    n = 3_000_001
    rng = np.random.default_rng(123)
    X = torch.from_numpy(rng.standard_normal(n)).cuda()
    Y = torch.from_numpy(rng.standard_normal(n)).cuda()
    with ocsl.Context(0) as ctx:
        want = ctx.dot_device(X, Y)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # the scratch keeps the previous call's contents
        out.fill_(float("nan"))
        st = L.ocsl_dot_noalloc(n, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert st == 0, L.ocsl_noalloc_last_error()
        torch.cuda.synchronize()
        got = out.item()
        assert abs(got - want) <= 0.0 * abs(want), (got, want)


def test_dot_noalloc_limits(lib_built, torch_cuda):
    torch = torch_cuda
    L = lib_built
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    X = torch.ones(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # n beyond the stated maximum is refused before any launch
    st = L.ocsl_dot_noalloc(8_388_609, C.c_void_p(X.data_ptr()), C.c_void_p(X.data_ptr()),
                            C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert st == 7 and b"exceeds the no-alloc limit" in L.ocsl_noalloc_last_error()
    # empty input gives 0
    st = L.ocsl_dot_noalloc(0, None, None, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert st == 0
    torch.cuda.synchronize()
    assert out.item() == 0.0


def test_dot_noalloc_at_the_limit(lib_built, torch_cuda):
    # n exactly at the maximum uses all 4,096 tile slots, the counter sits in
    # the slot right after them; bit-equal to the context-based dot
    import opencslsolver_gb300 as ocsl

    torch = torch_cuda
    L = lib_built
    n = 8_388_608
    g = torch.Generator(device="cuda").manual_seed(7)
    X = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    Y = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    with ocsl.Context(0) as ctx:
        want = ctx.dot_device(X, Y)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        st = L.ocsl_dot_noalloc(n, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert st == 0, L.ocsl_noalloc_last_error()
        torch.cuda.synchronize()
        assert out.item() == want
    # a misaligned device pointer is refused before any launch
    bad = C.c_void_p(X.data_ptr() + 4)
    st = L.ocsl_dot_noalloc(16, bad, C.c_void_p(Y.data_ptr()), C.c_void_p(out.data_ptr()),
                            C.c_void_p(stream))
    assert st == 7 and b"aligned" in L.ocsl_noalloc_last_error()
