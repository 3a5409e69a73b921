"""Writes the golden fixtures of tests/golden/: the oracle's state, motion and forces after
three steps of each synthetic configuration (cfd_gb300.case.config_case 1-3) at a small
size, with the generated node coordinates (so that a platform whose libm rounds the
generator's sin/cos differently still starts from the same mesh) and a checksum of the
generated connectivity.

    python tests/golden/make_golden.py

The reference ships no test vectors and cannot be built here, so these fixtures pin the
oracle (and the case generator) against later changes, and give the GPU tests a fixed
answer that does not need the oracle at run time."""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = [(1, 12, 7), (2, 12, 7), (3, 16, 7)]  # (configuration, scale, seed)
STEPS = 3


def input_digest(k):
    h = hashlib.sha256()
    for a in (k.inpoel, k.wall, k.iset_entries, k.ilaux()):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def path(which, scale, seed):
    return os.path.join(HERE, f"case{which}_s{scale}_seed{seed}.npz")


def generate(which, scale, seed):
    from cfd_gb300 import case as C
    from oracle import oracle as O
    O.set_threads(1)
    k = C.config_case(which, scale=scale, seed=seed)
    o = O.OracleCase(k)
    rep = o.step(STEPS)
    st = o.state()
    xp, yp = o.motion()
    out = dict(x0=k.x, y0=k.y, U=st["U"], T=st["T"], X=st["X"], Y=st["Y"], xpos=xp, ypos=yp,
               fx=np.array(rep.fx[:rep.nset_numb]), fy=np.array(rep.fy[:rep.nset_numb]),
               rm=np.array(rep.rm[:rep.nset_numb]), dtmin=np.float64(rep.dtmin),
               time=np.float64(rep.time), bicg_iters=np.array(rep.bicg_iters[:2]),
               steps=np.int64(STEPS), digest=np.array(input_digest(k)))
    o.close()
    return out


if __name__ == "__main__":
    for which, scale, seed in CASES:
        np.savez_compressed(path(which, scale, seed), **generate(which, scale, seed))
        print("wrote", path(which, scale, seed))
