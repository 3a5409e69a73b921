"""The oracle's thread modes: calcRHS and FUENTE scatter with OpenMP atomics like the
reference (thread order), or in element order at any thread count."""
import numpy as np

from conftest import small_case


def _run(O, k, threads, ordered, steps=3):
    O.set_threads(threads)
    O.set_ordered_scatter(ordered)
    try:
        o = O.OracleCase(k)
        o.step(steps)
        st = o.state()
        o.close()
    finally:
        O.set_ordered_scatter(False)
        O.set_threads(1)
    return st


def test_ordered_scatter_is_the_one_thread_result(oracle):
    from cfd_gb300 import abi
    k = small_case(5, scale=48, seed=2, estab_mode=abi.CFD_ESTAB_REFERENCE)
    one = _run(oracle, k, 1, False)
    many = _run(oracle, k, 4, True)
    for q in ("U", "T", "X", "Y"):
        assert np.array_equal(one[q].view(np.uint64), many[q].view(np.uint64)), q
