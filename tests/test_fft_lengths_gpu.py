"""GPU parity of the pruned three-pass fine-grid transform at every compiled fine-grid length
(the ladder 160 ... 1600 that FP32 volumes snap their fine grids to) against the FP64 direct sum
(not against another GPU path).

Each case is a box whose three edges give odd mode counts m = 2 nint(q L / 2 pi) + 1 with fine
lengths (the smallest 2,3,5-smooth multiple of 16 >= 2m) chosen so that the X, the Y and the Z
pass each run the length under test while the other two stay short; packed Al/U pair, unit
weights, FP32 at eps 1e-6 (kernel width 7) and 1e-7 (width 8).  The sample is 3,000 random modes
of the full grid."""
import math

import numpy as np
import pytest

import oracle
from helpers import rel_l2
from mp_tools_gb300 import _lib, sql
from mp_tools_gb300.sqom import SqomJob

pytestmark = pytest.mark.gpu

Q_RANGE = 3.0
SHORT = 31           # nint(q L / 2 pi) of a short axis: m = 63, fine length 128
LENGTHS = (160, 192, 256, 320, 384, 512, 640, 768, 960, 1024, 1152, 1280, 1536, 1600)
HALF_M = {n: (n // 2 - 2) // 2 for n in LENGTHS}   # m = n/2 - 1 or - 2: 2m rounds up to n


def _box(half_m):
    return 2 * math.pi * half_m / Q_RANGE


@pytest.mark.parametrize("n", sorted(HALF_M))
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("eps,tol", [(1e-6, 1e-5), (1e-7, 2e-6)])
def test_pruned_length_against_direct_sum(cuda, n, axis, eps, tol):
    half = [SHORT] * 3
    half[axis] = HALF_M[n]
    box = tuple(_box(h) for h in half)
    grid = sql.SqlGrid(Q_RANGE, box)
    assert grid.n_q[axis] == 2 * HALF_M[n] + 1
    rng = np.random.default_rng(n + 10 * axis)
    n_pts = 20000
    fr = np.zeros((1, n_pts, 4), np.float32)
    fr[0, :, :3] = (rng.uniform(-0.5, 0.5, (n_pts, 3)) * np.array(box)).astype(np.float32)
    counts = [18400, 1600]
    job = SqomJob(grid, species_counts=counts, n_frames=1, precision=_lib.FP32, eps=eps,
                  n_atoms_frame=n_pts)
    try:
        assert job.uses_pruned_fft(), "fine length %d should take the pruned passes" % n
        assert job.info()["fine_grid"][axis] == n
        job.set_frames(fr)
        job.transform()
        job.sync()
        cs = job.amplitudes()[0]
    finally:
        job.close()
    m0, m1, m2 = grid.n_q
    q = rng.choice(grid.n_modes, 3000, replace=False)
    kq = np.stack([q % m0 - m0 // 2, (q // m0) % m1 - m1 // 2, q // (m0 * m1) - m2 // 2], 1)
    r = fr[0, :, :3].astype(np.float64)
    d = grid.d_q.astype(np.float64)
    want = oracle.dirft_modes(r[:, 0] * d[0], r[:, 1] * d[1], r[:, 2] * d[2], np.ones(n_pts), -1, kq)
    assert rel_l2(cs[q], want) < tol, (n, axis, eps)
