"""The oracle's pow exposure: x**1.5d0, x**.5d0 and x**(-.5d0) as correctly rounded
compositions (x*sqrt(x), sqrt(x), 1/sqrt(x); the oracle's and the FP64 GPU path's form)
against the C library's pow (the form a Fortran build without unsafe math takes).

On a developed state about a quarter of the element temperature ratios give a pow that
differs from the composition in the last bit.  One step then changes the state by ~1e-17;
with the reference ESTAB (subrutinas.f90:374-393, whose unit vectors are round-off noise
where the gradients vanish) the difference grows to 1e-4..1e-2 within a few steps, while
under the regularized ESTAB it stays at round-off level.  So the bit-exact FP64 path is
pinned to the oracle, and a gfortran build of the reference would sit within 1e-16 of it for
the first steps and then drift by as much as its own threaded runs do.
"""
import numpy as np


def test_pow_census_known_values(oracle):
    # exact powers: the composition and pow agree on them
    x = np.array([1.0, 4.0, 0.25, 16.0, 9.0])
    assert oracle.pow_census(x) == (0, 0, 0)
    rng = np.random.default_rng(0)
    r = rng.uniform(0.8, 1.3, 20000)
    c15, cm05, c05 = oracle.pow_census(r)
    # a last-bit difference on a sizeable share of the ratios; sqrt(x) and pow(x, .5) are
    # both correctly rounded almost everywhere
    assert 0.05 * r.size < c15 < 0.6 * r.size
    assert 0.05 * r.size < cm05 < 0.6 * r.size
    assert c05 < 0.01 * r.size


def test_pow_mode_exposure(oracle):
    from oracle import pow_exposure as P
    d = P.measure(scale=48, checkpoints=(1, 3, 10))
    assert d["census_freestream"]["pow1.5_differs"] == 0
    assert d["census_perturbed"]["pow1.5_differs"] > 0.1 * d["census_perturbed"]["values"]
    for start in ("freestream", "perturbed"):
        ref = d[f"{start}_estab_reference"]["rel_l2_per_variable"]
        reg = d[f"{start}_estab_regularized"]["rel_l2_per_variable"]
        # one step: round-off level either way
        assert max(ref[0]) < 1e-15 and max(reg[0]) < 1e-15
        # ten steps: the regularized ESTAB keeps it there, the reference ESTAB does not
        assert max(reg[2]) < 1e-14
        assert max(ref[2]) > 1e-8
    oracle.set_pow_mode(0)
    assert oracle.get_pow_mode() == 0
