"""Host-side fault injection on a GPU: with MPSQ_FAIL_ALLOC=k the k-th device allocation of a
job reports out-of-memory without calling the allocator.  Sweeping k over every allocation a
job makes (FP32 pruned-transform job, FP64 cuFFT job) checks that each failure returns
MPSQ_ERR_ALLOC with a message and no handle, that the allocations made before it are released
(device free memory back to its level before the call), and that the job created once k is past
the last allocation works."""
import ctypes as C

import numpy as np
import pytest

from mp_tools_gb300 import _lib
from mp_tools_gb300.sqom import QGrid, SqomJob

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [_lib.FP32, _lib.FP64])
def test_every_failed_allocation_releases_the_others(lib, cuda, monkeypatch, precision):
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=3.0, a_par=(30.0,) * 3, ndim=3)
    d = SqomJob.describe(grid, species_counts=[300, 100], n_frames=3, n_atoms_frame=400,
                         precision=precision, eps=1e-6)
    h = C.c_void_p()
    # warm-up: context, library state and one complete job
    assert lib.mpsq_job_create(C.byref(d), None, C.byref(h)) == 0
    lib.mpsq_job_destroy(h)
    cuda.cuda.synchronize()
    free0 = cuda.cuda.mem_get_info()[0]
    created = False
    for k in range(1, 60):
        monkeypatch.setenv("MPSQ_FAIL_ALLOC", str(k))
        h = C.c_void_p()
        rc = lib.mpsq_job_create(C.byref(d), None, C.byref(h))
        if rc == 0:                       # k beyond the job's allocations: a working job
            created = True
            monkeypatch.delenv("MPSQ_FAIL_ALLOC")
            lib.mpsq_job_destroy(h)
            break
        assert rc == 2, (k, rc)
        assert not h.value
        cuda.cuda.synchronize()
        free = cuda.cuda.mem_get_info()[0]
        # allocations are released (2 MiB slack for the driver's bookkeeping)
        assert free >= free0 - (2 << 20), (k, free0 - free)
    assert created, "the sweep never got past the job's allocations"
    cuda.cuda.synchronize()
    assert cuda.cuda.mem_get_info()[0] >= free0 - (2 << 20)


def test_injected_failure_then_a_normal_job_gives_results(lib, cuda, monkeypatch):
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=3.0, a_par=(30.0,) * 3, ndim=3)
    rng = np.random.default_rng(5)
    fr = np.zeros((2, 400, 4), np.float32)
    fr[..., :3] = rng.uniform(-15, 15, (2, 400, 3))
    monkeypatch.setenv("MPSQ_FAIL_ALLOC", "3")
    with pytest.raises(_lib.MpsqError):
        SqomJob(grid, species_counts=[300, 100], n_frames=2, eps=1e-6)
    monkeypatch.delenv("MPSQ_FAIL_ALLOC")
    job = SqomJob(grid, species_counts=[300, 100], n_frames=2, eps=1e-6)
    try:
        job.set_frames(fr)
        job.transform()
        sq = job.sq_total()
    finally:
        job.close()
    assert np.isfinite(sq).all() and sq.max() > 0
