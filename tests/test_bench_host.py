"""Host-side helpers of bench.py (CPU): the e2e leg's host buffers and the accuracy figures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_e2e_host_buffer_falls_back_to_pageable():
    """Replicas on one node may pin more host memory than the node allows; the e2e leg then
    uses pageable buffers (here: no driver, so pinning is refused)."""
    import torch
    sys.path.insert(0, str(ROOT))
    import bench
    if torch.cuda.is_available():
        pytest.skip("pinning succeeds on a GPU host")
    t, pinned = bench.host_buffer((3, 5, 4))
    assert not pinned and tuple(t.shape) == (3, 5, 4) and t.dtype == torch.float32


def test_accuracy_metrics():
    """The bench's error figures: relative l2 of amplitudes and |F|^2, and the largest relative
    |F|^2 error over samples above 1e-3 of the maximum (weaker samples are left out)."""
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    ref = np.array([[10.0, 1.0 + 1.0j, 0.01], [3.0j, -2.0, 0.001]])
    got = ref.copy()
    got[0, 1] *= 1.001                  # |F|^2 off by 2.001e-3 relative
    got[1, 2] *= 2.0                    # below the 1e-3 cut: no effect on the maximum
    m = bench.error_metrics(got, ref)
    assert m["max_rel_S"] == pytest.approx(1.001 ** 2 - 1, rel=1e-9)
    d = (got - ref).ravel()
    assert m["rel_l2_amplitude"] == pytest.approx(np.linalg.norm(d) / np.linalg.norm(ref))
    s_g, s_r = np.abs(got) ** 2, np.abs(ref) ** 2
    assert m["rel_l2_S"] == pytest.approx(np.linalg.norm(s_g - s_r) / np.linalg.norm(s_r))
