"""cfd_bicg_device_noalloc: the BiCG solve for callers that cannot allocate device memory
where they solve (their arrays already live on the GPU; the library keeps its work
vectors in a fixed static device array).  Checked through the C-ABI against the existing
cfd_bicg_ex entry on the same system, on two calls in a row (the shared work array keeps
the previous call's contents, so the second call shows nothing stale leaks through); the
second call takes b = NULL and must not change the device's free memory.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_case

pytestmark = pytest.mark.gpu


def _system(oracle, scale=16, seed=3):
    k = small_case(1, scale=scale, seed=seed)
    g = oracle.deriv(k.x, k.y, k.inpoel)
    rp, idx = oracle.laplace_pattern(k.inpoel, k.npoin)
    vals, diag = oracle.laplace(k.inpoel, g["dNx"], g["dNy"], k.x, k.y, rp, idx)
    fix = k.ilaux()
    rng = np.random.default_rng(seed)
    data = 1e-3 * rng.normal(size=len(fix))
    x0 = 1e-4 * rng.normal(size=k.npoin)
    return vals, idx, rp, diag, fix, data, x0


def test_noalloc_bicg_matches_bicg_twice(gpu_lib, oracle):
    import torch
    from cfd_gb300 import abi, solver
    L = abi.lib()
    for seed, scale in ((3, 16), (7, 24)):
        vals, idx, rp, diag, fix, data, x0 = _system(oracle, scale=scale, seed=seed)
        n = len(diag)
        b = np.zeros(n)
        x_ref, info_ref = solver.biCG(vals, idx, rp, diag, x0, b, data, fix)
        # device copies owned by the caller; Dirichlet values applied to x as copy1 does
        xd0 = x0.copy()
        xd0[fix - 1] = data
        isfix = np.zeros(n, np.uint8)
        isfix[fix - 1] = 1
        dev = "cuda"
        t_val = torch.from_numpy(np.ascontiguousarray(vals)).to(dev)
        t_col = torch.from_numpy((idx - 1).astype(np.int32)).to(dev)
        t_rp = torch.from_numpy(rp.astype(np.int32)).to(dev)
        t_diag = torch.from_numpy(np.ascontiguousarray(diag)).to(dev)
        t_fix = torch.from_numpy(isfix).to(dev)
        t_b = torch.zeros(n, dtype=torch.float64, device=dev)
        # both calls' x buffers exist before the first call, so nothing in between allocates
        t_xs = [torch.from_numpy(xd0.copy()).to(dev) for _ in range(2)]
        torch.cuda.synchronize()
        for call, t_x in enumerate(t_xs):
            # the second call passes b = NULL (a zero right-hand side, like the zero b of the
            # first) and must leave the device's free memory exactly as it was
            b_ptr = t_b.data_ptr() if call == 0 else None
            free_before = torch.cuda.mem_get_info()[0]
            info = abi.CfdSolveInfo()
            st = L.cfd_bicg_device_noalloc(t_val.data_ptr(), t_col.data_ptr(), t_rp.data_ptr(),
                                           t_diag.data_ptr(), t_fix.data_ptr(), t_x.data_ptr(),
                                           b_ptr, n, 1.0e-10, 1000, None, C.byref(info))
            assert st == abi.CFD_OK, L.cfd_strerror(st)
            if call == 1:
                assert torch.cuda.mem_get_info()[0] == free_before, "the call allocated"
            x = t_x.cpu().numpy()
            assert (info.iters, info.converged) == (info_ref.iters, info_ref.converged), call
            assert info.rz == info_ref.rz
            np.testing.assert_array_equal(x, x_ref, err_msg=f"call {call + 1}")


def test_noalloc_rejects_sizes_above_cap(gpu_lib):
    from cfd_gb300 import abi
    L = abi.lib()
    big = 65536 + 1
    info = abi.CfdSolveInfo()
    st = L.cfd_bicg_device_noalloc(1, 1, 1, 1, 1, 1, None, big, 1e-10, 10, None, C.byref(info))
    assert st == abi.CFD_ERR_LIMIT
