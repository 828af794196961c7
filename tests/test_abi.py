"""The C-ABI library loads and exports every entry point include/mpsq.h declares (no GPU)."""
import re
import subprocess

import pytest
from pathlib import Path

from conftest import ROOT


def header_functions():
    text = (ROOT / "include" / "mpsq.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*([a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in {"if", "while"}))


def test_header_parses_expected_symbols():
    names = header_functions()
    assert "finufft2d1_" in names and "mpsq_job_create" in names
    from mp_tools_gb300 import _lib
    assert sorted(names) == sorted(_lib.EXPORTS)


def test_library_exports_all_declared(lib):
    from mp_tools_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in header_functions() if n not in exported]
    assert not missing, missing
    for n in header_functions():
        assert hasattr(lib, n)


def test_version_and_counters(lib):
    assert b"sm_103a" in lib.mpsq_version()
    assert lib.mpsq_launch_count() >= 0


def _c_struct_members():
    text = (ROOT / "include" / "mpsq.h").read_text()
    body = text[text.index("typedef struct mpsq_job_desc {"):text.index("} mpsq_job_desc;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    return re.findall(r"^\s*(?:int32_t|int64_t|double)\s+([a-z_0-9]+)", body, flags=re.M)


def test_job_descriptor_bindings_match_the_header():
    """The ctypes mirror and the Fortran bind(C) type list the C struct's members in order."""
    from mp_tools_gb300 import _lib
    members = _c_struct_members()
    assert members[0] == "ndim" and members[-1] == "q_slab"
    assert [f[0] for f in _lib.JobDesc._fields_] == members
    f90 = (ROOT / "include" / "mpsq_api.f90").read_text()
    typ = f90[f90.index("type, bind(C), public :: mpsq_job_desc_t"):f90.index("end type")]
    fnames = re.findall(r"::\s*([a-z_0-9]+)", typ)[1:]      # skip the type name itself
    assert fnames == members
    # every function the Fortran module binds is exported under that name
    bound = set(re.findall(r'bind\(C, name="([a-z_0-9]+)"\)', f90))
    assert bound and bound <= set(header_functions())


def test_injected_allocation_failure_reports_err_alloc(lib, monkeypatch):
    """Fault injection on the host: with MPSQ_FAIL_ALLOC=1 the job's first device allocation
    reports out-of-memory before the allocator is called, so job creation returns
    MPSQ_ERR_ALLOC (2) with its message and no handle, on any machine."""
    import ctypes as C
    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import QGrid, SqomJob
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=2.0, a_par=(10.0,) * 3, ndim=3)
    d = SqomJob.describe(grid, species_counts=[100], n_frames=2, n_atoms_frame=100)
    h = C.c_void_p()
    monkeypatch.setenv("MPSQ_FAIL_ALLOC", "1")
    assert lib.mpsq_job_create(C.byref(d), None, C.byref(h)) == 2
    assert not h.value
    msg = lib.mpsq_last_error()
    assert b"job_create" in (msg if isinstance(msg, bytes) else msg.encode())


def _run_harness(tmp_path):
    from mp_tools_gb300 import build as mbuild
    so = Path(mbuild.LIB)
    exe = tmp_path / "abi_harness"
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "abi_harness.c"), "-o", str(exe), "-L", str(so.parent),
                        "-lmpsq", f"-Wl,-rpath,{so.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    rows = {ln.split()[0]: ln.split()[1:] for ln in run.stdout.splitlines()}
    ier = {k: int(v[0].split("=")[1]) for k, v in rows.items()}
    return run, rows, ier


def _check_harness_modes(rows):
    import numpy as np
    import oracle
    x, y, z = [0.1, -1.2, 2.5], [-2.0, 0.7, 3.0], [1.5, -0.3, -3.1]
    c = np.array([1.0, 0.5 - 0.5j, -1.0 + 2.0j])
    got = np.array([float(v) for v in rows["2d"][1:]]).view(np.complex128)
    want = oracle.dirft2d1(x, y, c, -1, 4, 3).ravel()
    assert np.abs(got - want).max() < 1e-7 * np.abs(want).max()
    got3 = np.array([float(v) for v in rows["3d"][1:]]).view(np.complex128)
    want3 = oracle.dirft3d1(x, y, z, c, -1, 4, 3, 2).ravel()
    assert np.abs(got3 - want3).max() < 1e-7 * np.abs(want3).max()


def test_c_caller_of_the_fortran_entry_points(lib, tmp_path):
    """tests/abi_harness.c, compiled as C against include/mpsq.h and linked to libmpsq, calls
    finufft2d1_ / finufft3d1_ with gfortran's by-reference convention.  On a machine with a
    GPU the modes equal the FP64 direct sum (column-major, k1 fastest); without one every call
    reports MPSQ_ERR_CUDA in ier, a null scalar MPSQ_ERR_ARG, and the first failure is
    printed once to stderr (the reference never reads ier)."""
    run, rows, ier = _run_harness(tmp_path)
    assert ier["null"] == 1
    if ier["2d"] == 0:
        _check_harness_modes(rows)
    else:
        assert ier["2d"] == 3 and ier["3d"] == 3
        assert run.stderr.count("mpsq: finufft replacement failed") == 1


@pytest.mark.gpu
def test_c_caller_of_the_fortran_entry_points_on_gpu(lib, cuda, tmp_path):
    """The same C caller on a GPU: both calls succeed (ier = 0), the modes equal the FP64
    direct sum, the null-scalar call reports MPSQ_ERR_ARG and only that failure is printed."""
    run, rows, ier = _run_harness(tmp_path)
    assert ier["2d"] == 0 and ier["3d"] == 0, run.stderr
    _check_harness_modes(rows)
    assert ier["null"] == 1
    assert run.stderr.count("mpsq: finufft replacement failed") == 1


def test_job_memory_estimate_structure(lib):
    """mpsq_job_estimate_bytes (host arithmetic, used for admission): each extra frame adds its
    16-byte positions and its row of the complex amplitude store; keeping per-species
    amplitudes adds their store; FP64 doubles the amplitude bytes per frame."""
    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import QGrid, SqomJob
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=3.0, a_par=(20.0,) * 3, ndim=3)
    nq, na = grid.n_modes, 500

    def est(**kw):
        d = SqomJob.describe(grid, species_counts=[400, 100], n_atoms_frame=na, **kw)
        return SqomJob.estimate_bytes(d)

    f1, f2 = est(n_frames=4), est(n_frames=10)
    assert f2 - f1 == 6 * (na * 16 + nq * 8)
    assert est(n_frames=4, store_species=True) - f1 == 4 * 2 * nq * 8
    g1, g2 = est(n_frames=4, precision=_lib.FP64), est(n_frames=10, precision=_lib.FP64)
    assert g2 - g1 == 6 * (na * 16 + nq * 16)
