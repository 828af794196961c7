"""Autotuner: it times the applicable run-time choices, sets the fastest on the job, appends it
to a cache file under the job's shape, and a second job of the same shape takes the recorded
choice from the file; the tuned job's amplitudes equal those of the default settings."""
import numpy as np
import pytest

from mp_tools_gb300 import _lib, sql
from mp_tools_gb300.sqom import SqomJob

pytestmark = pytest.mark.gpu


def _job(fr, counts, grid):
    return SqomJob(grid, species_counts=counts, n_frames=fr.shape[0], precision=_lib.FP32,
                   eps=1e-6, n_atoms_frame=fr.shape[1])


def test_autotune_sets_records_and_reuses_a_choice(cuda, tmp_path):
    rng = np.random.default_rng(3)
    n, F = 20000, 6
    fr = np.zeros((F, n, 4), np.float32)
    fr[:, :, :3] = rng.uniform(-15.0, 15.0, (1, n, 3)) + rng.normal(0, 0.1, (F, n, 3))
    counts = [18400, 1600]
    grid = sql.SqlGrid(6.0, (30.0,) * 3)                  # fine grid 128^3, z-slabs apply
    cache = tmp_path / "tune.txt"
    a = _job(fr, counts, grid)
    b = _job(fr, counts, grid)
    try:
        a.set_option(_lib.OPT_REPRODUCIBLE, 1)   # the tuner keeps it; bit-exact comparison
        a.set_frames(fr)
        a.transform()
        a.sync()
        ref = a.amplitudes()
        ch = a.autotune(0, 4, cache=str(cache))
        assert ch["ms_per_call"] > 0
        assert ch["zslab"] in (0, 64) and ch["xrows"] in (4, 8) and ch["lanes"] in (1, 2)
        assert a.get_option(_lib.OPT_ZSLAB) == ch["zslab"]
        assert a.get_option(_lib.OPT_GRAPH) == ch["graph"]
        lines = cache.read_text().split("\n")
        assert len([ln for ln in lines if ln.strip()]) == 1
        fields = lines[0].split()
        assert fields[0].startswith("mpsq-tune-2:") and len(fields) == 7
        assert [int(v) for v in fields[1:6]] == [ch["graph"], ch["spread"] == "cuda-core",
                                                 ch["xrows"], ch["lanes"], ch["zslab"]]
        assert a.get_option(_lib.OPT_REPRODUCIBLE) == 1
        a.transform()
        a.sync()
        if ch["spread"] == "tensor-core":
            assert np.array_equal(a.amplitudes(), ref)
        # same shape: the recorded choice, without timing and without a new cache line
        b.set_frames(fr)
        chb = b.autotune(0, 4, cache=str(cache))
        assert {k: chb[k] for k in ("graph", "spread", "xrows", "lanes", "zslab")} == \
               {k: ch[k] for k in ("graph", "spread", "xrows", "lanes", "zslab")}
        assert chb["ms_per_call"] == pytest.approx(ch["ms_per_call"], rel=1e-3)
        assert len([ln for ln in cache.read_text().split("\n") if ln.strip()]) == 1
    finally:
        a.close()
        b.close()
