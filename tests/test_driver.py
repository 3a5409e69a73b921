"""The host driver (ns2DComp.ALE.f90's run loop and files): Fortran edit descriptors, the
.RST record layout, a run of a case directory with the oracle as the engine (CPU), a
restart, and the same run on the FP64 CUDA form giving byte-identical files (GPU)."""
import os
import struct

import numpy as np
import pytest

from conftest import small_case

FILES = ("{name}.cnv", "DESPLAZAMIENTO", "FORCES", "SKIN.DAT", "{name}.RST", "FORCES_HISTORY")


def test_fortran_edit_descriptors():
    from cfd_gb300.driver import fortran_e, fortran_es, fortran_i
    assert fortran_e(1.5, 14, 6) == "  0.150000E+01"
    assert fortran_e(-0.00123456789, 14, 6) == " -0.123457E-02"
    assert fortran_e(0.0, 13, 5) == "  0.00000E+00"
    assert fortran_e(9.999996, 14, 6) == "  0.100000E+02"
    assert fortran_e(1.0e-120, 14, 6) == "  0.100000-119"
    assert fortran_i(12, 7) == "     12" and fortran_i(3, 2) == " 3"
    assert fortran_es(-0.25) == "-2.5000000000000000E-001".rjust(25)


def test_restart_record_layout(tmp_path):
    from cfd_gb300.driver import read_restart, write_restart
    U = np.arange(8, dtype=float).reshape(2, 4) + 0.5
    T, G = np.array([300.0, 301.0]), np.array([1.4, 1.4])
    path = tmp_path / "c.RST"
    write_restart(path, 7, 0.25, U, T, G)
    data = path.read_bytes()
    want = struct.pack("<iidi", 12, 7, 0.25, 12)
    for n in range(2):
        want += struct.pack("<i6di", 48, *U[n], T[n], G[n], 48)
    assert data == want
    it, tm, U2, T2, G2 = read_restart(path, 2)
    assert (it, tm) == (7, 0.25)
    assert np.array_equal(U2, U) and np.array_equal(T2, T) and np.array_equal(G2, G)


def write_small(tmp_path, maxiter=4, iprint=2, irestart=0):
    from cfd_gb300.case import write_case
    k = small_case(1, scale=8, seed=3, maxiter=maxiter, iprint=iprint, irestart=irestart)
    d = tmp_path / "case"
    write_case(k, str(d))
    return k, str(d)


def oracle_engine(directory):
    from cfd_gb300.case import read_case
    from oracle import oracle as O
    return O.OracleCase(read_case(directory))


def test_run_with_oracle_engine(tmp_path):
    from cfd_gb300 import driver
    from cfd_gb300.case import read_case
    k, d = write_small(tmp_path)
    eng = oracle_engine(d)
    out = tmp_path / "out"
    summary = driver.run_case(d, out_dir=str(out), engine=eng)
    name = read_case(d).name
    for f in FILES:
        assert (out / f.format(name=name)).exists(), f
    cnv = (out / f"{name}.cnv").read_text().splitlines()
    assert len(cnv) == 2 and cnv[1].startswith("      4")
    assert len(cnv[0]) == 7 + 5 * 14
    assert summary["iter"] == 4
    it, tm, U, T, G = driver.read_restart(out / f"{name}.RST", k.npoin)
    assert it == 4 and tm == summary["time"]
    assert np.array_equal(U, eng.state()["U"]) and np.array_equal(T, eng.state()["T"])
    assert len((out / "DESPLAZAMIENTO").read_text().splitlines()) == 2
    assert "FUERZA VISCOSA EN X:" in (out / "FORCES").read_text()
    skin = np.loadtxt(out / "SKIN.DAT")
    assert skin.shape == (int(k.iset_array()[1][0]), 3)


def test_restart_reads_state(tmp_path):
    from cfd_gb300 import driver
    from cfd_gb300.case import read_case, write_case
    k, d = write_small(tmp_path)
    driver.run_case(d, engine=oracle_engine(d))  # writes <name>.RST into the case dir
    name = read_case(d).name
    _, _, U, T, _ = driver.read_restart(os.path.join(d, name + ".RST"), k.npoin)
    k2 = read_case(d)
    k2.params.irestart = 1
    write_case(k2, d)
    eng = oracle_engine(d)
    driver.run_case(d, out_dir=str(tmp_path / "r"), engine=eng, maxiter=0)
    assert np.array_equal(eng.state()["U"], U) and np.array_equal(eng.state()["T"], T)


@pytest.mark.gpu
def test_fp64_run_files_identical_to_oracle(gpu_lib, tmp_path):
    from cfd_gb300 import driver
    from cfd_gb300.case import read_case
    k, d = write_small(tmp_path, maxiter=6, iprint=3)
    name = read_case(d).name
    driver.run_case(d, out_dir=str(tmp_path / "gpu"))
    driver.run_case(d, out_dir=str(tmp_path / "cpu"), engine=oracle_engine(d))
    for f in FILES:
        f = f.format(name=name)
        assert (tmp_path / "gpu" / f).read_bytes() == (tmp_path / "cpu" / f).read_bytes(), f


@pytest.mark.gpu
def test_command_lines_write_and_run_a_case(gpu_lib, tmp_path, capsys):
    """`python -m cfd_gb300.case DIR` then `python -m cfd_gb300.driver DIR`: the mixed form
    with per-step smoothing runs the written case and writes the reference's files."""
    import json
    import os
    from cfd_gb300 import case as C, driver
    d, out = str(tmp_path / "c3"), str(tmp_path / "out")
    C.main([d, "--config", "3", "--scale", "24", "--maxiter", "4"])
    driver.main([d, "--out", out, "--precision", "mixed", "--smooth-every", "2"])
    last = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert last["iter"] == 4 and all(np.isfinite(last["residuals"]))
    names = set(os.listdir(out))
    assert {"FORCES", "DESPLAZAMIENTO", "FORCES_HISTORY"} <= names
    assert any(n.endswith(".RST") for n in names) and any(n.endswith(".cnv") for n in names)
