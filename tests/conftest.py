import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.set_threads(1)
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library with a device; GPU tests fail (not skip) without one."""
    from cfd_gb300 import build, abi
    build.build()
    return abi.lib()


def small_case(which=1, scale=8, seed=3, **over):
    from cfd_gb300 import case as C
    k = C.config_case(which, scale=scale, seed=seed)
    for key, v in over.items():
        setattr(k.params, key, v)
    return k


def perturbed_state(case, seed=0, amp=0.05):
    """A freestream state with smooth + random perturbations (rho, velocity, T)."""
    rng = np.random.default_rng(seed)
    p = case.params
    n = case.npoin
    x, y = case.x, case.y
    rho = p.rho_inf * (1.0 + amp * np.sin(0.7 * x) * np.cos(0.5 * y) + 0.2 * amp * rng.uniform(-1, 1, n))
    u = p.u_inf * (1.0 + amp * np.cos(0.3 * x + 0.2 * y)) + 0.1 * amp * p.u_inf * rng.uniform(-1, 1, n)
    v = p.u_inf * amp * np.sin(0.4 * y) + 0.1 * amp * p.u_inf * rng.uniform(-1, 1, n)
    T = p.t_inf * (1.0 + amp * np.sin(0.2 * x + 0.3 * y) + 0.1 * amp * rng.uniform(-1, 1, n))
    P = rho * p.fr * T
    E = P / ((p.gama - 1.0) * rho) + 0.5 * (u * u + v * v)
    U = np.stack([rho, rho * u, rho * v, rho * E], 1)
    return U, T, u, v
