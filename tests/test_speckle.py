"""mp_sqom's speckle filter (code/src/mp_sqom56.f90:1531-1570).

CPU: the oracle's sequential walk on hand-worked cases (wrap-around at both ends, the filtered
left neighbour, the second walk over the transposed map, one-walk E(Q) cuts).
GPU: the speculative one-CTA kernel is bit-identical to the oracle's walk on random maps with
dense speckles (long chains of dependent replacements), ragged sizes (fewer values than
threads, not a multiple of the thread count, one and two values), both map kinds; the job's
maps with s_trig > 0 equal the oracle's filter applied to the same unnormalised map, times the
remaining normalisation."""
import numpy as np
import pytest

from oracle import sqom_ref

f32 = np.float32


def test_oracle_walk_hand_cases():
    # a lone spike is cut to the larger neighbour, a lone dip raised to the smaller one
    m = np.array([[1, 1, 50, 1, 1, 1]], f32)
    assert sqom_ref.speckle_filter(m, 2.0, dispersion=True).tolist() == [[1, 1, 1, 1, 1, 1]]
    m = np.array([[4, 4, 0.1, 4, 4, 4]], f32)
    assert sqom_ref.speckle_filter(m, 2.0, dispersion=True).tolist() == [[4, 4, 4, 4, 4, 4]]
    # within the trigger ratio nothing changes
    m = np.array([[1, 1.9, 1, 0.6, 1]], f32)
    assert np.array_equal(sqom_ref.speckle_filter(m, 2.0, dispersion=True), m)
    # the left neighbour is the filtered one: at 1 the dip 0.001 is raised to 6, so at 2 the
    # value 10 is compared with (6, 1) and kept (against the unfiltered (0.001, 1) it would be
    # cut to 1); at 3 the dip 1 is raised to min(10, 6)
    m = np.array([[6, 0.001, 10, 1, 6]], f32)
    assert sqom_ref.speckle_filter(m, 2.0, dispersion=True).tolist() == [[6, 6, 10, 6, 6]]
    # the last value's right neighbour is the filtered first value: the dip 0.001 at 0 is
    # raised to min(10, 6) = 6 first, so 10 at 4 is compared with (1, 6) and kept
    m = np.array([[0.001, 6, 1, 1, 10]], f32)
    assert sqom_ref.speckle_filter(m, 2.0, dispersion=True).tolist() == [[6, 6, 1, 1, 10]]


def test_oracle_walk_matches_plain_loop():
    """The oracle's walk against a literal transcription with 1-based indices."""
    rng = np.random.default_rng(0)
    for n in (2, 3, 7, 40):
        x = (10.0 ** rng.uniform(-3, 3, n)).astype(f32)
        want = x.copy()
        s = f32(2.0)
        for i2 in range(1, n + 1):
            i1 = i2 - 1
            if i1 < 1:
                i1 += n
            i3 = i2 + 1
            if i3 > n:
                i3 -= n
            a, b = want[i1 - 1], want[i3 - 1]
            if want[i2 - 1] < f32(min(a, b) / s):
                want[i2 - 1] = min(a, b)
            if want[i2 - 1] > f32(s * max(a, b)):
                want[i2 - 1] = max(a, b)
        got = sqom_ref.speckle_filter(x[None, :], 2.0, dispersion=True)[0]
        assert np.array_equal(got, want)


def test_oracle_plane_map_walks_both_directions():
    # a column-direction spike pair survives the row walk (neighbours along x are spikes too)
    # but not the walk over the transposed map
    m = np.ones((5, 4), f32)
    m[2, 1] = m[2, 2] = 40.0        # two neighbouring spikes along x
    one = sqom_ref.speckle_filter(m, 2.0, dispersion=True)      # first walk only
    assert one[2, 1] == 40.0 or one[2, 2] == 40.0
    both = sqom_ref.speckle_filter(m, 2.0)
    assert np.array_equal(both, np.ones((5, 4), f32))


def _speckled(shape, seed, density=0.3):
    rng = np.random.default_rng(seed)
    m = (10.0 ** rng.uniform(-1, 1, shape)).astype(f32)
    k = rng.random(shape) < density
    m[k] *= (10.0 ** rng.choice([-4, -3, 3, 4], size=int(k.sum()))).astype(f32)
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(1, 1), (1, 2), (3, 5), (17, 60), (40, 31), (1, 5000),
                                   (128, 128), (200, 333)])
@pytest.mark.parametrize("dispersion", [False, True])
def test_gpu_filter_bit_identical(cuda, shape, dispersion):
    from mp_tools_gb300.sqom import speckle_filter
    for seed, s_trig in ((1, 2.0), (2, 1.5), (3, 10.0)):
        m = _speckled(shape, seed + shape[0] * 7 + shape[1])
        want = sqom_ref.speckle_filter(m, s_trig, dispersion=dispersion)
        got = speckle_filter(m, s_trig, dispersion=dispersion)
        assert got.dtype == np.float32 and got.shape == m.shape
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (shape, seed)


@pytest.mark.gpu
def test_gpu_filter_long_dependent_chains(cuda):
    """Alternating dips 0.001, 0.3: every value's fate depends on its filtered predecessor, so
    a change entering a chunk runs through all of it and every chunk is refiltered once per
    chunk before it (about one pass per thread of the CTA)."""
    from mp_tools_gb300.sqom import speckle_filter
    n = 70_001
    m = np.tile(np.array([0.001, 0.3], f32), n // 2 + 1)[:n]
    want = sqom_ref.speckle_filter(m[None, :], 2.0, dispersion=True)
    got = speckle_filter(m[None, :], 2.0, dispersion=True)
    assert np.array_equal(got, want)
    post = speckle_filter(m[None, :], 2.0, dispersion=True, post_scale=0.125)
    assert np.array_equal(post, (want * f32(0.125)).astype(f32))
    m2 = m.reshape(1, n)[:, :70_000].reshape(280, 250)      # plane map, both walks
    assert np.array_equal(speckle_filter(m2, 2.0), sqom_ref.speckle_filter(m2, 2.0))


@pytest.mark.gpu
def test_job_maps_with_speckle_filter(cuda):
    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import QGrid, SqomJob, TimeAxis
    from helpers import abo3_cell
    rng = np.random.default_rng(11)
    base, ind, counts = abo3_cell(4, rng)
    F = 8
    frames = np.repeat(base[None], F, axis=0).copy()
    frames[:, :, :3] += rng.normal(0, 0.02, size=frames[:, :, :3].shape).astype(f32)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=3, a_par=(4.19,) * 3)
    assert grid.n_q[2] == 1
    job = SqomJob(grid, species_counts=counts, n_frames=F, precision=_lib.FP32, eps=1e-6,
                  weight_mode=2, b_coh=[0.507, 0.716, 0.5803, 0.5803, 0.5803])
    try:
        job.set_frames(frames)
        job.transform()
        job.sync()
        ta = TimeAxis(nfile=F, t_step=0.01)
        n2 = job.norm2()
        plane = (grid.n_q[1], grid.n_q[0])
        for jf in (1, 2):
            raw = job.sqw_econst(ta, jf, normalize=False).reshape(plane)
            want = sqom_ref.speckle_filter(raw, 2.0) * f32(ta.t_step / n2)
            got = job.sqw_econst(ta, jf, s_trig=2.0).reshape(plane)
            assert np.array_equal(got, want.astype(f32))
        path = np.arange(0, grid.n_modes, 5)
        raw = job.sqw_dispersion(ta, path, normalize=False)
        want = sqom_ref.speckle_filter(raw, 2.0, dispersion=True) * f32(ta.t_step / n2)
        assert np.array_equal(job.sqw_dispersion(ta, path, s_trig=2.0), want.astype(f32))
        raw = job.sq_total(normalize=False).reshape(plane)
        want = sqom_ref.speckle_filter(raw, 3.0) * f32(1.0 / n2)
        assert np.array_equal(job.sq_total(s_trig=3.0).reshape(plane), want.astype(f32))
        raw = job.iqt(ta.n_int, 2, normalize=False).reshape(plane)
        want = sqom_ref.speckle_filter(raw, 2.0) * f32(1.0 / n2)
        assert np.array_equal(job.iqt(ta.n_int, 2, s_trig=2.0).reshape(plane), want.astype(f32))
    finally:
        job.close()
