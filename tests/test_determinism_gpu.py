"""With the reproducible order (MPSQ_OPT_REPRODUCIBLE), FP32 volume jobs spread on the tensor
cores give bit-identical amplitudes however their work is scheduled: graph replay or launch by
launch, one or two frame lanes, whole-grid passes or the z-slab pipeline, separate job
instances.  The spreading kernel orders each tile's records by content before accumulating
them (the binning's atomics leave their order open), and for tiles with more records than one
staging chunk it partitions them into chunks by whole (component, start z) keys.  Tiles denser
than that (a single key over a chunk) take the records in binning order: correct to FP32
rounding, not bit-reproducible.  The default order is checked against the reproducible one."""
import numpy as np
import pytest

from helpers import rel_l2
from mp_tools_gb300 import _lib, sql
from mp_tools_gb300.sqom import SqomJob

pytestmark = pytest.mark.gpu


def _alloy(n, box, F=3, seed=11):
    rng = np.random.default_rng(seed)
    fr = np.zeros((F, n, 4), np.float32)
    p = rng.uniform(-box / 2, box / 2, (n, 3))
    for t in range(F):
        fr[t, :, :3] = p
        p = p + rng.normal(0, 0.2, p.shape)
    n_u = n // 12
    return fr, [n - n_u, n_u]


def _run(grid, fr, counts, options=(), repro=1):
    job = SqomJob(grid, species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32,
                  eps=1e-6, n_atoms_frame=fr.shape[1])
    try:
        job.set_option(_lib.OPT_REPRODUCIBLE, repro)
        for opt, val in options:
            job.set_option(opt, val)
        job.set_frames(fr)
        job.transform()
        job.sync()
        return job.amplitudes(), job.info()
    finally:
        job.close()


def test_scheduling_choices_give_identical_amplitudes(cuda):
    fr, counts = _alloy(20000, 30.0)
    grid = sql.SqlGrid(6.0, (30.0,) * 3)                  # 59^3 modes, fine grid 128^3
    ref, info = _run(grid, fr, counts)
    assert info["pruned"] and info["fine_grid"] == (128, 128, 128)
    for options in ([(_lib.OPT_GRAPH, 1)],
                    [(_lib.OPT_LANES, 1)],
                    [(_lib.OPT_ZSLAB, 32)],
                    [(_lib.OPT_GRAPH, 1), (_lib.OPT_LANES, 1), (_lib.OPT_ZSLAB, 48)],
                    [(_lib.OPT_GRAPH, 1), (_lib.OPT_ZSLAB, 96)],
                    []):
        got, _ = _run(grid, fr, counts, options)
        assert np.array_equal(got, ref), options
    fast, _ = _run(grid, fr, counts, repro=0)
    assert rel_l2(fast, ref) < 1e-6


def test_dense_tiles_chunked_by_key_are_identical_and_correct(cuda):
    """~1,400 records per 16^3 tile (six staging chunks, formed from whole keys)."""
    fr, counts = _alloy(100000, 30.0, F=2)
    grid = sql.SqlGrid(4.0, (30.0,) * 3)                  # 39^3 modes, fine grid 96^3
    ref, info = _run(grid, fr, counts)
    assert info["fine_grid"] == (96, 96, 96)
    got, _ = _run(grid, fr, counts, [(_lib.OPT_LANES, 1), (_lib.OPT_ZSLAB, 48)])
    assert np.array_equal(got, ref)
    fma, _ = _run(grid, fr, counts, [(_lib.OPT_SPREAD, 1)])   # CUDA-core spreading
    assert rel_l2(ref, fma) < 2e-6


def test_tiles_with_an_oversized_key_stay_correct(cuda):
    """A tile whose single (component, start z) key holds more records than a chunk: binning
    order, checked against the CUDA-core spreading."""
    fr, counts = _alloy(400000, 30.0, F=1)
    grid = sql.SqlGrid(4.0, (30.0,) * 3)
    ref, _ = _run(grid, fr, counts)
    fma, _ = _run(grid, fr, counts, [(_lib.OPT_SPREAD, 1)])
    assert rel_l2(ref, fma) < 5e-6      # ~5,500 records per tile: longer FP32 sums


def test_z_slab_option_values(cuda):
    fr, counts = _alloy(2000, 30.0, F=1)
    grid = sql.SqlGrid(4.0, (30.0,) * 3)
    job = SqomJob(grid, species_counts=counts, n_frames=1, precision=_lib.FP32, eps=1e-6,
                  n_atoms_frame=fr.shape[1])
    try:
        assert job.get_option(_lib.OPT_ZSLAB) == 0
        job.set_option(_lib.OPT_ZSLAB, 64)
        assert job.get_option(_lib.OPT_ZSLAB) == 64
        for bad in (-16, 10, 4112):
            with pytest.raises(RuntimeError):
                job.set_option(_lib.OPT_ZSLAB, bad)
        assert job.get_option(_lib.OPT_ZSLAB) == 64
        job.set_option(_lib.OPT_ZSLAB, 4096)   # larger than the grid: whole-grid passes
        job.set_frames(fr)
        job.transform()
        job.sync()
    finally:
        job.close()
