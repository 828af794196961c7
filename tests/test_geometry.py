"""Q-grid geometry restated from mp_sqom56.f90:764-936 (CPU only)."""
import numpy as np

from mp_tools_gb300 import _lib
from mp_tools_gb300.sqom import QGrid, TimeAxis


def test_cell_hk0_pixels():
    # 20^3 cells, 8 zones, (hk0): 160 x 160 pixels, 1/20 r.l.u. steps
    g = QGrid(_lib.CELL, (20, 20, 20), n_bz=8, a_par=(4.19,) * 3)
    assert g.n_q[:2] == (160, 160)
    assert np.isclose(g.dq[0], 8 / 160)
    assert np.isclose(g.tpe[0], 2 * np.pi / 20, rtol=1e-6)
    g3 = QGrid(_lib.CELL, (20, 20, 20), n_bz=8, a_par=(4.19,) * 3, ndim=3)
    assert g3.n_q == (160, 160, 160)


def test_bzo_example_pixels():
    # the BZO example: 32^3 cells, 5 zones, (hk0) -> 160 x 160 (mp_sqom_cmd_log)
    g = QGrid(_lib.CELL, (32, 32, 32), n_bz=5, a_par=(4.19,) * 3)
    assert g.n_q[:2] == (160, 160)


def test_bulk_pixels_and_phase_scale():
    L = 255.4
    g = QGrid(_lib.BULK, (1, 1, 1), n_bz=4.72, a_par=(L,) * 3, ndim=3)
    assert g.n_q == (192, 192, 192)
    assert np.isclose(g.tpe[0], 2 * np.pi / L, rtol=1e-6)
    q2 = g.q2_norm()
    assert q2.shape == (192 ** 3,)
    origin, steps, extra = g.qphys()
    # mode k along x has physical Q = origin + k * dq (1/A, BULK units)
    assert np.isclose(steps[0][0], 4.72 / 192, rtol=1e-6)


def test_q_center_offsets_range():
    g = QGrid(_lib.CELL, (20, 20, 20), n_bz=4, q_center=(2, 2, 0), a_par=(4.0,) * 3)
    assert np.isclose(g.q_min[0], 0.0) and np.isclose(g.q_min[1], 0.0)
    qx = g.axis_values(0)
    assert np.isclose(qx[g.n_q[0] // 2], 2.0)


def test_time_axis_constants():
    t = TimeAxis(nfile=20, t_step=0.1)
    assert t.n_int == 11 and t.n_frame == 10 and t.n_freq_max == 6
    assert np.isclose(t.freq_step, 1.0 / (10 * 0.1))
    w = t.window()
    assert w[0] == 0 and np.isclose(w[5], 1.0)
    t2 = TimeAxis(nfile=256, t_step=0.01)
    assert t2.n_int == 129 and t2.n_freq_max == 65
