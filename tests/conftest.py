import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc

    if not os.path.isfile(orc.ORACLE_SO):
        orc.build()
    return orc.Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import oracle as orc

    if not orc.reference_available():
        pytest.skip("reference not built here (oracle/_ref needs the reference's sources)")
    r = orc.Reference()
    r.set_threads(1)
    return r


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def golden_small():
    z = load_golden("small_systems.npz")
    cases = []
    for k in range(int(z["count"])):
        p = f"c{k}_"
        cases.append({key[len(p):]: z[key] for key in z.files if key.startswith(p)})
    return cases


@pytest.fixture(scope="session")
def golden_kat():
    return load_golden("kat_tridiag10.npz")


@pytest.fixture(scope="session")
def golden_shocktube():
    return load_golden("shocktube_calls.npz")


@pytest.fixture(scope="session")
def lib_built():
    from opencslsolver_gb300 import _abi

    if not os.path.isfile(_abi.LIB_PATH):
        from opencslsolver_gb300 import build

        build.build()
    return _abi.lib()


@pytest.fixture(scope="session")
def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    return torch


@pytest.fixture()
def ctx(lib_built, torch_cuda):
    import opencslsolver_gb300 as ocsl

    c = ocsl.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def hex128():
    """The 128^3 jittered hex p' system (2,097,152 cells), generated once."""
    from opencslsolver_gb300 import workloads as W

    return W.hex_pprime(128, peclet=10.0)
