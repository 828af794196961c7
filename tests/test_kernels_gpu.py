"""GPU parity of the FP32 fast paths that the small-system job tests do not reach:
the mixed-radix Gaussian-window spectrum (64..1024 frames, even and odd Q counts, with and
without the 1/|Q| factor) and the tensor-core spreading of packed species pairs (against the
CUDA-core spreading kernel, selected with MPSQ_SPREAD=fma in a child process, and against
the FP64 direct sum)."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import rel_l2
from mp_tools_gb300 import _lib, sql
from mp_tools_gb300.sqom import QGrid, SqomJob
from oracle import sqom_ref

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def random_walk(n_atoms, F, box, seed, sigma=0.05):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-box / 2, box / 2, (n_atoms, 3))
    fr = np.empty((F, n_atoms, 4), np.float32)
    for t in range(F):
        fr[t, :, :3] = p
        fr[t, :, 3] = 0.0
        p = p + rng.normal(0, sigma, p.shape)
    return fr


@pytest.mark.parametrize("F", [64, 128, 256, 512, 1024])
@pytest.mark.parametrize("grid_kind", ["even", "odd"])
def test_gauss_spectrum_long_runs(cuda, F, grid_kind):
    if grid_kind == "even":      # 8^3 = 512 modes: 16-byte rows, float4 loads
        grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3, ndim=3)
        box = 4.0
        frames = random_walk(60, F, box, seed=F, sigma=0.01)
    else:                        # 13^3 = 2197 modes: odd row length, float2 loads, ragged tile
        grid = sql.SqlGrid(4.0, (10.0,) * 3)
        frames = random_walk(60, F, 10.0, seed=F + 1)
    counts = [40, 20]
    job = SqomJob(grid, species_counts=counts, n_frames=F, precision=_lib.FP32, eps=1e-6,
                  n_atoms_frame=frames.shape[1])
    try:
        job.set_frames(frames)
        job.transform()
        job.sync()
        cs = job.amplitudes().astype(np.complex128)
        rng = np.random.default_rng(5)
        q2 = rng.uniform(0.5, 2.0, grid.n_modes).astype(np.float32)
        for fwhm, n_freq, qn in ((F / 2, F // 2 + 1, None), (F / 8, F // 4, q2)):
            got = job.sqw_gauss(fwhm_frames=fwhm, n_freq=n_freq, q2_norm=qn, normalize=False)
            g = sqom_ref.gauss_window(F, fwhm)
            want = sqom_ref.gauss_spectrum(cs, fwhm, n_freq, None if qn is None else qn.astype(np.float64),
                                           1.0 / g.sum())
            assert got.shape == want.shape
            assert rel_l2(got, want) < 2e-5, (F, grid_kind, fwhm)
    finally:
        job.close()


def _alloy(n_atoms=6000, F=2, box=30.0, seed=3):
    rng = np.random.default_rng(seed)
    fr = np.zeros((F, n_atoms, 4), np.float32)
    fr[:, :, :3] = rng.uniform(-box / 2, box / 2, (n_atoms, 3))
    fr[1:, :, :3] += rng.normal(0, 0.2, (F - 1, n_atoms, 3)).astype(np.float32)
    return fr, [int(n_atoms * 0.92), n_atoms - int(n_atoms * 0.92)]


_CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import test_kernels_gpu as T
from mp_tools_gb300 import _lib, sql
fr, counts = T._alloy()
grid = sql.SqlGrid(5.0, (30.0,) * 3)
job = T.SqomJob(grid, species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32,
                eps=float(sys.argv[3]), store_species=True, n_atoms_frame=fr.shape[1])
job.set_frames(fr); job.transform(); job.sync()
np.save(sys.argv[2], job.amplitudes())
job.close()
"""


# kernel widths 6, 7, 8 (eps 1e-5, 1e-6, 1e-7) and the FP32 error bound at each width
WIDTHS = [(1e-5, 6e-5), (1e-6, 1e-5), (1e-7, 2e-6)]


@pytest.mark.parametrize("eps", [w[0] for w in WIDTHS])
def test_tensor_core_spread_matches_cuda_core_spread(cuda, tmp_path, eps):
    """Packed Al/U pair job (both species in one grid) through the default (tensor-core)
    spread and, in a child process with MPSQ_SPREAD=fma, through the CUDA-core spread."""
    out = {}
    for mode in ("mma", "fma"):
        env = dict(os.environ)
        if mode == "fma":
            env["MPSQ_SPREAD"] = "fma"
        else:
            env.pop("MPSQ_SPREAD", None)
        path = tmp_path / f"cs_{mode}.npy"
        subprocess.run([sys.executable, "-c", _CHILD, str(ROOT), str(path), repr(eps)], check=True,
                       env=env, timeout=600)
        out[mode] = np.load(path)
    assert out["mma"].shape == out["fma"].shape
    assert rel_l2(out["mma"], out["fma"]) < 2e-6


@pytest.mark.parametrize("eps,tol", WIDTHS)
def test_tensor_core_spread_against_direct_sum(cuda, eps, tol):
    fr, counts = _alloy()
    grid = sql.SqlGrid(5.0, (30.0,) * 3)
    job = SqomJob(grid, species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32,
                  eps=eps, n_atoms_frame=fr.shape[1])
    try:
        job.set_frames(fr)
        job.transform()
        job.sync()
        cs = job.amplitudes()
    finally:
        job.close()
    n = grid.n_q[0]
    d = grid.d_q.astype(np.float64)
    for t in range(fr.shape[0]):
        r = fr[t, :, :3].astype(np.float64)
        want = oracle.dirft3d1(r[:, 0] * d[0], r[:, 1] * d[1], r[:, 2] * d[2], np.ones(len(r)),
                               -1, n, n, n)
        assert rel_l2(cs[t], want.reshape(-1)) < tol, (eps, t)


def test_transform_from_host_equals_device_upload(cuda):
    """Chunked upload on a second stream (pinned host tensor) gives the amplitudes of one upload
    followed by the transform, bit for bit with the reproducible order, also when the job is
    run twice back to back."""
    import torch
    fr, counts = _alloy(n_atoms=3000, F=40)
    grid = sql.SqlGrid(4.0, (30.0,) * 3)
    kw = dict(species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32, eps=1e-6,
              n_atoms_frame=fr.shape[1])
    a = SqomJob(grid, **kw)
    b = SqomJob(grid, **kw)
    try:
        for job in (a, b):
            job.set_option(_lib.OPT_REPRODUCIBLE, 1)
        a.set_frames(fr)
        a.transform()
        a.sync()
        pinned = torch.from_numpy(fr).pin_memory()
        for _ in range(2):
            b.transform_from_host(pinned, chunk=7)
        b.sync()
        assert np.array_equal(b.amplitudes(), a.amplitudes())
    finally:
        a.close()
        b.close()


_CHILD_LANES = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import test_kernels_gpu as T
from mp_tools_gb300 import _lib, sql
fr, counts = T._alloy(n_atoms=4000, F=9)
grid = sql.SqlGrid(4.0, (30.0,) * 3)
job = T.SqomJob(grid, species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32, eps=1e-6,
                n_atoms_frame=fr.shape[1], weight_mode=_lib.WEIGHT_XRAY, xff=[T.XFF_AL, T.XFF_U])
job.set_option(_lib.OPT_REPRODUCIBLE, 1)
job.set_frames(fr)
job.transform(0, 4)            # even count
job.transform(4, 5)            # odd count, second call
job.sync()
np.save(sys.argv[2], np.concatenate([job.amplitudes().ravel(), job.sq_total()]))
job.close()
"""
XFF_AL = [6.4202, 3.0387, 1.9002, 0.7426, 1.5936, 31.5472, 1.9646, 85.0886, 1.1151]
XFF_U = [36.0228, 0.5293, 23.4128, 3.3253, 14.9491, 16.0927, 4.1880, 100.6130, 13.3966]


def test_two_frame_lanes_match_one_lane(cuda, tmp_path):
    """Frames alternating between the job's stream and the second lane give the results of a
    single lane (MPSQ_LANES=1, child process) bit for bit (reproducible order), over two
    transform calls."""
    out = {}
    for lanes in ("2", "1"):
        env = dict(os.environ)
        if lanes == "1":
            env["MPSQ_LANES"] = "1"
        else:
            env.pop("MPSQ_LANES", None)
        path = tmp_path / f"lanes_{lanes}.npy"
        subprocess.run([sys.executable, "-c", _CHILD_LANES, str(ROOT), str(path)], check=True,
                       env=env, timeout=600)
        out[lanes] = np.load(path)
    assert np.array_equal(out["2"], out["1"])


def test_outputs_to_host_tensors_are_copied_asynchronously(cuda):
    """Maps written to host torch tensors go through a device staging buffer and a copy on a
    separate stream; after sync() they equal the device-resident results, also when the next
    transform is queued before the copies have finished."""
    import torch
    fr, counts = _alloy(n_atoms=3000, F=16)
    grid = sql.SqlGrid(4.0, (30.0,) * 3)
    job = SqomJob(grid, species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32,
                  eps=1e-6, n_atoms_frame=fr.shape[1])
    try:
        job.set_frames(fr)
        job.transform()
        dev_sqw = torch.empty((9, grid.n_modes), dtype=torch.float32, device="cuda")
        dev_sq = torch.empty(grid.n_modes, dtype=torch.float32, device="cuda")
        job.sqw_gauss(fwhm_frames=8, n_freq=9, out=dev_sqw)
        job.sq_total(out=dev_sq)
        host_sqw = torch.empty((9, grid.n_modes), dtype=torch.float32, pin_memory=True)
        host_sq = torch.empty(grid.n_modes, dtype=torch.float32, pin_memory=True)
        for _ in range(2):
            assert job.sqw_gauss(fwhm_frames=8, n_freq=9, out=host_sqw) is host_sqw
            assert job.sq_total(out=host_sq) is host_sq
            job.transform()                     # queued behind the copies' source reads
        job.sync()
        # (equal up to FP32 rounding: the re-transform sums the records in another order)
        assert rel_l2(host_sqw.numpy(), dev_sqw.cpu().numpy()) < 1e-5
        assert rel_l2(host_sq.numpy(), dev_sq.cpu().numpy()) < 1e-5
    finally:
        job.close()


@pytest.mark.parametrize("q_range,box", [(2.95, 100.0), (3.96, 100.0), (5.97, 100.0)])
def test_pruned_passes_match_cufft_path(cuda, q_range, box):
    """The pruned three-pass transform (two-stage radix plans, last stage finished in
    registers for the X pass) against cuFFT + the separate deconvolution, on fine grids of
    192, 256 and 384 points (95^3, 127^3, 191^3 modes; packed Al/U pair, X-ray weights)."""
    rng = np.random.default_rng(int(box))
    n = 20000
    fr = np.zeros((2, n, 4), np.float32)
    fr[:, :, :3] = rng.uniform(-box / 2, box / 2, (n, 3)).astype(np.float32)
    fr[1, :, :3] += rng.normal(0, 0.3, (n, 3)).astype(np.float32)
    counts = [18400, 1600]
    grid = sql.SqlGrid(q_range, (box,) * 3)
    kw = dict(species_counts=counts, n_frames=2, precision=_lib.FP32, eps=1e-6,
              n_atoms_frame=n, weight_mode=_lib.WEIGHT_XRAY, xff=[XFF_AL, XFF_U])
    out = {}
    for pruned in (True, False):
        job = SqomJob(grid, no_pruned_fft=not pruned, **kw)
        try:
            job.set_frames(fr)
            job.transform()
            out[pruned] = job.amplitudes()
        finally:
            job.close()
    assert rel_l2(out[True], out[False]) < 2e-6, grid.n_q
