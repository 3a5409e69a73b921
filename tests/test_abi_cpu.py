"""The C-ABI library loads here (no GPU) and exports every symbol include/cfd_gpu.h
declares; argument checks answer with a status before any device work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "cfd_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cfd_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from cfd_gb300 import abi, build
    build.build()
    return abi.load()


def test_exports_every_declared_symbol(lib):
    from cfd_gb300 import abi
    names = declared_symbols()
    assert len(names) >= 28
    for n in names:
        assert hasattr(lib, n), f"{n} declared but not exported"
        assert n in abi.SIGNATURES, f"{n} has no ctypes signature"


def test_status_strings(lib):
    for s in range(10):
        assert lib.cfd_strerror(s)
    assert lib.cfd_strerror(0) == b"ok"


def test_argument_checks_without_device(lib):
    from cfd_gb300 import abi
    one = C.c_int(1)
    assert lib.cfd_calcrhs(*([None] * 11), None, C.byref(one), C.byref(one), None, None) == abi.CFD_ERR_ARG
    assert lib.cfd_bicg(*([None] * 10), None) == abi.CFD_ERR_ARG
    assert lib.cfd_step(None, 1, None) == abi.CFD_ERR_ARG


def test_host_adjacency_matches_oracle(lib, oracle):
    """getEsup/getPsup/pattern are host code in the library: checked here on the CPU."""
    from conftest import small_case
    from cfd_gb300 import solver
    k = small_case(1, scale=10)
    e1, e2 = solver.getEsup(k.inpoel, k.npoin)
    o1, o2 = oracle.esup(k.inpoel, k.npoin)
    np.testing.assert_array_equal(e1, o1)
    np.testing.assert_array_equal(e2, o2)
    p1, p2 = solver.getPsup(k.inpoel, k.npoin)
    q1, q2 = oracle.psup(k.inpoel, k.npoin)
    np.testing.assert_array_equal(p1, q1)
    np.testing.assert_array_equal(p2, q2)
    rp, idx = solver.laplace_pattern(k.inpoel, k.npoin)
    orp, oidx = oracle.laplace_pattern(k.inpoel, k.npoin)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(idx, oidx)
    bad = k.inpoel.copy()
    bad[0, 0] = 0
    from cfd_gb300 import abi
    with pytest.raises(abi.CfdError) as e:
        solver.getPsup(bad, k.npoin)
    assert e.value.status == abi.CFD_ERR_MESH
