"""Jobs run slab by slab along kz (q_slab > 0: the amplitude store holds a few kz planes at a
time, for jobs whose whole store does not fit in device memory) give the amplitudes and maps of
the same job with the whole store: FP32 through the pruned three-pass transform and through
cuFFT, FP64; the last slab is shorter than the others."""
import numpy as np
import pytest

from helpers import rel_l2
from mp_tools_gb300 import _lib
from mp_tools_gb300.sqom import QGrid, SqomJob, TimeAxis

pytestmark = pytest.mark.gpu

XFF_AL = [6.4202, 3.0387, 1.9002, 0.7426, 1.5936, 31.5472, 1.9646, 85.0886, 1.1151]
XFF_U = [36.0228, 0.5293, 23.4128, 3.3253, 14.9491, 16.0927, 4.1880, 100.6130, 13.3966]


def _frames(F=16, n=3000, box=66.0, seed=4):
    rng = np.random.default_rng(seed)
    fr = np.zeros((F, n, 4), np.float32)
    p = rng.uniform(-box / 2, box / 2, (n, 3))
    for t in range(F):
        fr[t, :, :3] = p
        p = p + rng.normal(0, 0.1, p.shape)
    return fr, [2700, 300]


def _maps(job, taxis):
    return (job.amplitudes(), job.sq_total(), job.sqw_econst(taxis, 2),
            job.sqw_gauss(fwhm_frames=8, n_freq=9, t_step=0.01))


@pytest.mark.parametrize("precision,pruned,tol", [(_lib.FP32, True, 1e-5), (_lib.FP32, False, 1e-5),
                                                 (_lib.FP64, False, 1e-12)])
def test_slab_by_slab_equals_whole_store(cuda, precision, pruned, tol):
    fr, counts = _frames()
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=3.0, a_par=(66.0,) * 3, ndim=3)   # 32^3 modes
    taxis = TimeAxis(fr.shape[0], 0.01)
    kw = dict(species_counts=counts, n_frames=fr.shape[0], precision=precision, eps=1e-6,
              weight_mode=_lib.WEIGHT_XRAY, xff=[XFF_AL, XFF_U], no_pruned_fft=not pruned,
              n_atoms_frame=fr.shape[1])
    full = SqomJob(grid, **kw)
    try:
        assert full.uses_pruned_fft() == (pruned and precision == _lib.FP32)
        full.set_frames(fr)
        full.transform()
        want = _maps(full, taxis)
    finally:
        full.close()
    nz = grid.n_q[2]
    slab = SqomJob(grid, q_slab=5, **kw)
    try:
        assert nz % 5 != 0                       # a shorter last slab
        slab.set_frames(fr)
        parts = []
        for z0, planes, q0 in slab.slabs():
            slab.set_q_slab(z0)
            assert slab.store_modes == grid.n_q[0] * grid.n_q[1] * planes
            slab.transform()
            parts.append(_maps(slab, taxis))
        got = [np.concatenate([p[i] for p in parts], axis=-1) for i in range(4)]
    finally:
        slab.close()
    for g, w, what in zip(got, want, ("amplitudes", "S(Q)", "E=const", "Gaussian spectrum")):
        assert g.shape == w.shape, what
        assert rel_l2(g, w) < tol, (what, rel_l2(g, w))


def test_slab_errors(lib, cuda):
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=2.0, a_par=(10.0,) * 3, ndim=3)
    job = SqomJob(grid, species_counts=[100], n_frames=2, n_atoms_frame=100)
    try:
        with pytest.raises(_lib.MpsqError):
            job.set_q_slab(0)                   # created without q_slab
    finally:
        job.close()
    job = SqomJob(grid, species_counts=[100], n_frames=2, n_atoms_frame=100, q_slab=2)
    try:
        with pytest.raises(_lib.MpsqError):
            job.set_q_slab(grid.n_q[2])         # beyond the grid
    finally:
        job.close()
