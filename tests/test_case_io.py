"""The reference's input formats round-trip, and the generator's meshes are valid."""
import numpy as np
import pytest

from cfd_gb300 import case as C


@pytest.mark.parametrize("which,scale", [(1, None), (2, 12), (3, 16), (5, 10)])
def test_roundtrip(tmp_path, which, scale):
    k = C.config_case(which, scale=scale, seed=4)
    C.write_case(k, str(tmp_path))
    k2 = C.read_case(str(tmp_path))
    for f in ("x", "y", "inpoel", "ifixrho_node", "rfixrho_value", "ifixv_node", "rfixv_valuex",
              "rfixv_valuey", "ifixt_node", "rfixt_value", "wall", "iset_entries", "i_m", "ifm"):
        np.testing.assert_array_equal(getattr(k, f), getattr(k2, f), err_msg=f)
    assert k2.params == k.params
    assert k2.meta == k.meta


def test_generator_sizes_and_orientation():
    k = C.config_case(1)
    assert (k.npoin, k.nelem) == (8192, 16128)
    n = k.inpoel - 1
    X, Y = k.x[n], k.y[n]
    a2 = (X[:, 1] - X[:, 0]) * (Y[:, 2] - Y[:, 0]) - (X[:, 2] - X[:, 0]) * (Y[:, 1] - Y[:, 0])
    assert np.all(a2 > 0)
    assert k.meta["ratio"] == 1.05
    # seeded: same seed, same mesh; other seed, other jitter
    assert np.array_equal(C.config_case(1).x, k.x)
    assert not np.array_equal(C.config_case(1, seed=1).x, k.x)
    for which, nn in [(2, 512 * 512), (3, 1024 * 1024)]:
        kk = C.config_case(which, scale=32)
        assert kk.npoin == 32 * 32 and kk.nelem == 2 * 31 * 32
    assert C.config_case(3, scale=16).meta["ratio"] > 1.0


def test_derived_parameters():
    p = C.flow_params(0.8, 5000.0, aoa_deg=2.0)
    assert p.u_inf ** 2 + p.v_inf ** 2 == pytest.approx((5000 * 0.017) ** 2)
    assert p.c_inf == pytest.approx(np.hypot(p.u_inf, p.v_inf) / 0.8)
    assert p.p_inf == pytest.approx(p.rho_inf * p.fr * p.t_inf)


def test_case_cli_writes_a_readable_case(tmp_path):
    """`python -m cfd_gb300.case DIR --config 3 --scale 16` writes the reference's three
    input files; reading them back gives the same mesh and parameters."""
    from cfd_gb300 import case as C
    d = str(tmp_path / "c3")
    C.main([d, "--config", "3", "--scale", "16", "--maxiter", "7"])
    k = C.read_case(d)
    ref = C.config_case(3, scale=16)
    assert k.npoin == ref.npoin and k.nelem == ref.nelem and k.params.maxiter == 7
    assert np.array_equal(k.inpoel, ref.inpoel)
    np.testing.assert_allclose(k.x, ref.x, rtol=0, atol=1e-12 * np.abs(ref.x).max())
