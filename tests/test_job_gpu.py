"""Parity of the fused S(Q,omega) job pipeline (selection, phases, strengths, NUFFT, species
weights, time transforms) with the oracle: FP64 direct sums + the numpy restatement of the
mp_sqom loops.  Tolerance on relative l2 errors: 1e-8 for FP64 at eps 1e-10, 3e-5 for FP32 at
eps 1e-6 (|F|^2 quantities carry twice the amplitude error)."""
import numpy as np
import pytest

import oracle
from helpers import abo3_cell, rel_l2
from mp_tools_gb300 import _lib
from mp_tools_gb300.sqom import QGrid, SqomJob, TimeAxis
from oracle import sqom_ref

pytestmark = pytest.mark.gpu

XFF_AL = [6.4202, 3.0387, 1.9002, 0.7426, 1.5936, 31.5472, 1.9646, 85.0886, 1.1151]
XFF_U = [36.0228, 0.5293, 23.4128, 3.3253, 14.9491, 16.0927, 4.1880, 100.6130, 13.3966]


def oracle_cs(frames, counts, grid, *, weight_mode=1, b_coh=None, xff=None, kappa=1 / 16.0,
              mask=None, window=False, phase_rounding=False, tol=0.1):
    S = len(counts)
    off = np.concatenate([[0], np.cumsum(counts)])
    F = frames.shape[0]
    nq = grid.n_modes
    A = np.zeros((F, S, nq), np.complex128)
    for t in range(F):
        for s in range(S):
            coords, c = sqom_ref.prep_points(
                frames[t], off[s], off[s + 1], input_method=grid.input_method, ndim=grid.ndim,
                axis=grid.axis, tpe=grid.tpe, centre=grid.at_pos_centre, q_center=grid.q_center,
                window=window, phase_rounding=phase_rounding, pos_min=grid.at_pos_min,
                pos_max=grid.at_pos_max, tol=tol)
            if grid.ndim == 3:
                f = oracle.dirft3d1(coords[0], coords[1], coords[2], c, -1, *grid.n_q)
            else:
                f = oracle.dirft2d1(coords[0], coords[1], c, -1, grid.n_q[0], grid.n_q[1])
            A[t, s] = f.ravel()
    if weight_mode == 1:
        w = np.ones((S, nq))
    elif weight_mode == 2:
        w = np.repeat(np.asarray(b_coh, float)[:, None], nq, axis=1)
    else:
        origin, steps, extra = grid.qphys()
        k = [np.arange(n) - n // 2 for n in grid.n_q]
        kz, ky, kx = np.meshgrid(k[2], k[1], k[0], indexing="ij")
        Q = (origin[None, :] + kx.reshape(-1, 1) * steps[0] + ky.reshape(-1, 1) * steps[1]
             + kz.reshape(-1, 1) * steps[2])
        s2 = kappa * ((Q ** 2).sum(1) + extra)
        w = np.stack([sqom_ref.xray_ff(xff[s], s2) for s in range(S)])
    wnorm = (0.25 if grid.ndim == 2 else 0.125) if window else 1.0
    return sqom_ref.weighted_sum(A, w, mask, wnorm)


def run_job(grid, frames, counts, **kw):
    F = frames.shape[0]
    job = SqomJob(grid, species_counts=counts, n_frames=F, **kw)
    job.set_frames(frames)
    job.transform()
    job.sync()
    return job


def cell_system(n=4, F=8, seed=0):
    rng = np.random.default_rng(seed)
    base, ind, counts = abo3_cell(n, rng)
    frames = np.repeat(base[None], F, axis=0).copy()
    frames[:, :, :3] += rng.normal(0, 0.02, size=frames[:, :, :3].shape).astype(np.float32)
    return frames, ind, counts


@pytest.mark.parametrize("prec,eps,tol", [(_lib.FP64, 1e-10, 1e-8), (_lib.FP32, 1e-6, 3e-5)])
def test_cell_volume_all_maps(cuda, prec, eps, tol):
    frames, _, counts = cell_system()
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    job = run_job(grid, frames, counts, precision=prec, eps=eps, weight_mode=2,
                  b_coh=[0.507, 0.716, 0.5803, 0.5803, 0.5803])
    ref = oracle_cs(frames, counts, grid, weight_mode=2, b_coh=[0.507, 0.716, 0.5803, 0.5803, 0.5803])
    cs = job.amplitudes()
    assert rel_l2(cs, ref) < tol
    n2 = float(sum(counts)) ** 2
    assert rel_l2(job.sq_total(), sqom_ref.sq_total(ref, n2)) < 2 * tol
    ta = TimeAxis(nfile=8, t_step=0.01)
    q2 = grid.q2_norm()
    scale = ta.t_step / n2 / (0.5 * ta.n_frame * ta.n_int)
    for jf in (1, 2, 3):
        got = job.sqw_econst(ta, jf, q2_norm=q2)
        want = sqom_ref.econst(cs.astype(np.complex128), ta.n_int, ta.window(), jf, q2, scale)
        assert rel_l2(got, want) < 1e-5
    path = np.arange(0, grid.n_modes, 37)
    got = job.sqw_dispersion(ta, path)
    want = sqom_ref.dispersion(cs.astype(np.complex128), ta.n_int, ta.window(), path, ta.n_freq_max,
                               None, scale)
    assert rel_l2(got, want) < 1e-5
    g = job.sqw_gauss(fwhm_frames=4, t_step=ta.t_step)
    gw = sqom_ref.gauss_window(8, 4)
    want = sqom_ref.gauss_spectrum(cs.astype(np.complex128), 4, 5, None, ta.t_step / n2 / gw.sum())
    assert rel_l2(g, want) < 1e-5
    job.close()


def test_pairing_does_not_change_results(cuda):
    frames, _, counts = cell_system(seed=1)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    a = run_job(grid, frames, counts, precision=_lib.FP64, eps=1e-10).amplitudes()
    b = run_job(grid, frames, counts, precision=_lib.FP64, eps=1e-10, no_pack=True).amplitudes()
    assert rel_l2(a, b) < 1e-10


@pytest.mark.parametrize("prec,eps,tol", [(_lib.FP64, 1e-10, 1e-8), (_lib.FP32, 1e-6, 3e-5)])
def test_q_center_complex_strengths(cuda, prec, eps, tol):
    frames, _, counts = cell_system(seed=2)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, q_center=(1, 0, 0.5), a_par=(4.19,) * 3, ndim=3)
    job = run_job(grid, frames, counts, precision=prec, eps=eps)
    ref = oracle_cs(frames, counts, grid)
    assert rel_l2(job.amplitudes(), ref) < tol


def test_plane_hhl_with_spatial_window_and_mask(cuda):
    frames, _, counts = cell_system(n=6, F=4, seed=3)
    grid = QGrid(_lib.CELL, (6, 6, 6), e1=(1, 1, 0), e2=(0, 0, 1), n_bz=3, q_center=(2, 2, 1),
                 a_par=(4.19,) * 3)
    mask = [1, 0, 1, 1, 0]
    job = run_job(grid, frames, counts, precision=_lib.FP64, eps=1e-10, window=True, mask=mask)
    ref = oracle_cs(frames, counts, grid, window=True, mask=mask)
    assert rel_l2(job.amplitudes(), ref) < 1e-8


def test_reference_phase_rounding(cuda):
    frames, _, counts = cell_system(seed=4)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, q_center=(0, 1, 0), a_par=(4.19,) * 3)
    job = run_job(grid, frames, counts, precision=_lib.FP64, eps=1e-11, phase_rounding=True)
    ref = oracle_cs(frames, counts, grid, phase_rounding=True)
    assert rel_l2(job.amplitudes(), ref) < 1e-9


def test_vacancies_are_skipped(cuda):
    frames, _, counts = cell_system(F=2, seed=5)
    frames[:, 7, :3] = 0.0     # a vacancy (all three coordinates exactly zero)
    frames[:, 70, :3] = 0.0
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    job = run_job(grid, frames, counts, precision=_lib.FP64, eps=1e-10)
    ref = oracle_cs(frames, counts, grid)
    assert rel_l2(job.amplitudes(), ref) < 1e-8


@pytest.mark.parametrize("ffc,kappa", [(_lib.FF_MP_SQOM, 1 / 16.0), (_lib.FF_STANDARD, 1 / (16 * np.pi ** 2))])
@pytest.mark.parametrize("prec,eps,tol", [(_lib.FP64, 1e-10, 1e-8), (_lib.FP32, 1e-6, 3e-5)])
def test_bulk_xray_with_box_selection(cuda, ffc, kappa, prec, eps, tol):
    rng = np.random.default_rng(6)
    L = 24.0
    counts = [900, 100]
    F = 4
    frames = np.zeros((F, 1000, 4), np.float32)
    frames[..., :3] = rng.uniform(-L / 2, L / 2, (F, 1000, 3)).astype(np.float32)
    frames[:, :20, 0] = L / 2 + 0.05    # just outside, inside the eps_x tolerance: kept
    frames[:, 20:30, 1] = -L / 2 - 0.3  # outside the tolerance: dropped
    grid = QGrid(_lib.BULK, (1, 1, 1), n_bz=3.0, a_par=(L,) * 3, ndim=3)
    job = run_job(grid, frames, counts, precision=prec, eps=eps, weight_mode=3, xff=[XFF_AL, XFF_U],
                  ff_convention=ffc, eps_x=0.1)
    ref = oracle_cs(frames, counts, grid, weight_mode=3, xff=[XFF_AL, XFF_U], kappa=kappa, tol=0.1)
    assert rel_l2(job.amplitudes(), ref) < tol


def test_pruned_transform_matches_cufft_path(cuda):
    """FP32 volumes use the pruned three-pass transform fused with the deconvolution; it must
    agree with cuFFT + the separate deconvolution kernel (5 species: two packed pairs and a
    single grid)."""
    frames, _, counts = cell_system(seed=7)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    kw = dict(precision=_lib.FP32, eps=1e-6, weight_mode=2, b_coh=[0.507, 0.716, 0.5803, 0.5803, 0.5803])
    a = run_job(grid, frames, counts, **kw)
    d = run_job(grid, frames, counts, no_pruned_fft=True, **kw)
    assert rel_l2(a.amplitudes(), d.amplitudes()) < 3e-6


@pytest.mark.parametrize("n_q", [(31, 47, 29), (30, 45, 64)])
def test_pruned_transform_odd_and_mixed_mode_counts(cuda, n_q):
    frames, _, counts = cell_system(F=2, seed=8)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    grid.n_q = n_q
    job = run_job(grid, frames, counts, precision=_lib.FP32, eps=1e-6)
    ref = oracle_cs(frames, counts, grid)
    assert rel_l2(job.amplitudes(), ref) < 3e-5


@pytest.mark.parametrize("prec,eps,tol", [(_lib.FP64, 1e-10, 1e-8), (_lib.FP32, 1e-6, 3e-5)])
def test_intermediate_scattering_function(cuda, prec, eps, tol):
    """I(Q,t) map and path cut (mp_sqom's j_sq /= 1 branch) vs the oracle on the job's own
    amplitudes, with and without the 1/|Q| factor."""
    frames, _, counts = cell_system(F=12, seed=4)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    job = run_job(grid, frames, counts, precision=prec, eps=eps, weight_mode=2,
                  b_coh=[0.507, 0.716, 0.5803, 0.5803, 0.5803])
    cs = job.amplitudes().astype(np.complex128)
    q2 = grid.q2_norm()
    n_int = 6
    for lag in (0, 3, 6):
        for qn in (None, q2):
            got = job.iqt(n_int, lag, q2_norm=qn, normalize=False)
            want = sqom_ref.iqt_map(cs, n_int, lag, qn)
            assert rel_l2(got, want) < 1e-5
    path = np.arange(0, grid.n_modes, 29)
    got = job.iqt_dispersion(n_int, path, q2_norm=q2, normalize=False)
    want = sqom_ref.iqt_dispersion(cs, n_int, path, q2)
    assert got.shape == (len(path), 12 - n_int + 1)
    assert rel_l2(got, want) < 1e-5
    job.close()


@pytest.mark.parametrize("prec,eps,tol", [(_lib.FP64, 1e-10, 1e-8), (_lib.FP32, 1e-6, 3e-5)])
def test_atom_pair_maps(cuda, prec, eps, tol):
    """E=const map and E(Q) cut of species pair (B, O1) (mp_sqom's j_atc1/j_atc2 option) vs the
    oracle: raw amplitudes of the two species summed, no mean subtraction."""
    frames, _, counts = cell_system(F=8, seed=5)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
    job = run_job(grid, frames, counts, precision=prec, eps=eps, weight_mode=2,
                  b_coh=[0.507, 0.716, 0.5803, 0.5803, 0.5803], store_species=True)
    pair_sum = oracle_cs(frames, counts, grid, weight_mode=1, mask=[0, 1, 1, 0, 0])
    ta = TimeAxis(nfile=8, t_step=0.01)
    scale = 1.0 / (0.5 * ta.n_frame * ta.n_int)
    for jf in (1, 2):
        got = job.sqw_econst(ta, jf, normalize=False, atom_pair=(1, 2))
        want = sqom_ref.econst(pair_sum, ta.n_int, ta.window(), jf, None, scale, center=False)
        assert rel_l2(got, want) < 1e-5        # maps are written as float32
    path = np.arange(0, grid.n_modes, 31)
    got = job.sqw_dispersion(ta, path, normalize=False, atom_pair=(1, 2))
    want = sqom_ref.dispersion(pair_sum, ta.n_int, ta.window(), path, ta.n_freq_max, None, scale,
                               center=False)
    assert rel_l2(got, want) < 1e-5
    with pytest.raises(_lib.MpsqError):
        job.sqw_econst(ta, 1, atom_pair=(1, 7))
    job.close()
