"""cfd_gb300 — GB300-native (sm_103a) explicit SUPG compressible Navier–Stokes step on
linear triangles with ALE mesh motion, behind the reference's routine signatures.

Modules: abi (ctypes mirror of include/cfd_gpu.h), case (reference data model, file
formats and synthetic O-grids), solver (host mirror of the reference driver and
routines), build (nvcc recipe of the in-tree CUDA library), driver (the reference's time
loop and output files), learned (the learned initial guess).  `python -m cfd_gb300.case`
writes a synthetic workload as a case directory; `python -m cfd_gb300.driver` runs one."""
from . import abi  # noqa: F401
