"""The golden fixtures of tests/golden/ (made by tests/golden/make_golden.py from the
oracle): the oracle and the FP64 CUDA form both reproduce them bit for bit (three steps of
each synthetic configuration: state, moved mesh, mesh-motion solution, forces, clock)."""
import os

import numpy as np
import pytest

from golden.make_golden import CASES, STEPS, input_digest, path

FIELDS = ("U", "T", "X", "Y", "xpos", "ypos")


def fixture_case(which, scale, seed):
    from cfd_gb300 import case as C
    g = dict(np.load(path(which, scale, seed)))
    k = C.config_case(which, scale=scale, seed=seed)
    assert input_digest(k) == str(g["digest"]), "the case generator's connectivity changed"
    k.x, k.y = g["x0"].copy(), g["y0"].copy()
    return k, g


def check(g, st, xp, yp, rep):
    got = dict(st, xpos=xp, ypos=yp)
    for f in FIELDS:
        assert np.array_equal(got[f], g[f]), f
    n = int(rep.nset_numb)
    assert np.array_equal(np.array(rep.fx[:n]), g["fx"])
    assert np.array_equal(np.array(rep.fy[:n]), g["fy"])
    assert np.array_equal(np.array(rep.rm[:n]), g["rm"])
    assert rep.dtmin == float(g["dtmin"]) and rep.time == float(g["time"])
    assert list(rep.bicg_iters[:2]) == list(g["bicg_iters"])


@pytest.mark.parametrize("which,scale,seed", CASES)
def test_oracle_reproduces_golden(oracle, which, scale, seed):
    k, g = fixture_case(which, scale, seed)
    o = oracle.OracleCase(k)
    rep = o.step(STEPS)
    st = o.state()
    xp, yp = o.motion()
    o.close()
    check(g, st, xp, yp, rep)


@pytest.mark.gpu
@pytest.mark.parametrize("which,scale,seed", CASES)
def test_fp64_cuda_reproduces_golden(gpu_lib, which, scale, seed):
    from cfd_gb300 import abi, solver
    k, g = fixture_case(which, scale, seed)
    s = solver.Solver(k, precision=abi.CFD_PREC_FP64)
    rep = s.step(STEPS)
    st = s.state()
    xp, yp = s.motion()
    s.close()
    check(g, st, xp, yp, rep)
