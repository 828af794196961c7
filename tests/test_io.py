"""Frame-file, parameter-file and text-map formats (CPU).

The .dat layout follows code/src/mp_latt56.f90:295-343 (4096-byte records, namelist header
records, at_ind int32 x 4 then at_pos float32 x 4, 256 atoms per record); the map body
follows code/src/mp_sqom56.f90:1995-2045 (format 200(1x,5e10.3)).
"""
from pathlib import Path

import numpy as np
import pytest

from mp_tools_gb300 import io

GOLDEN = Path(__file__).resolve().parent / "golden"
ALU_DAT = GOLDEN / "alu" / "Al_U_large_n0001.dat"


def test_read_reference_frame_file():
    f = io.read_dat(ALU_DAT)
    assert f.n_tot == 30000
    assert f.species_counts() == [27600, 2400]
    assert f.at_pos.dtype == np.float32 and f.at_pos.shape == (30000, 4)
    assert f.at_ind.dtype == np.int32 and f.at_ind.shape == (30000, 4)
    a_par = np.asarray(f.header["a_par"], np.float64)
    assert np.allclose(a_par, 79.815962, rtol=1e-6)
    # positions lie in the box centred on the origin, species-major: all Al (1) before U (2)
    half = 0.5 * a_par[0] + 1e-3
    assert f.at_pos[:, :3].min() >= -half and f.at_pos[:, :3].max() <= half
    assert np.all(np.diff(f.at_ind[:, 3]) >= 0)
    assert set(np.unique(f.at_ind[:, 3])) == {1, 2}


def test_dat_round_trip_is_bit_exact(tmp_path):
    f = io.read_dat(ALU_DAT)
    out = tmp_path / "copy_n0001.dat"
    io.write_dat(out, f)
    g = io.read_dat(out)
    assert out.stat().st_size % io.REC_BYTES == 0
    assert g.n_tot == f.n_tot and g.species_counts() == f.species_counts()
    assert np.array_equal(g.at_pos.view(np.uint32), f.at_pos.view(np.uint32))
    assert np.array_equal(g.at_ind, f.at_ind)
    for k in ("a_par", "n_tot", "nsuper_r", "input_method"):
        if k in f.header:
            assert g.header[k] == f.header[k], k


def test_dat_ragged_last_record(tmp_path):
    """n_tot not a multiple of 256: the last record is zero-padded and ignored on read."""
    rng = np.random.default_rng(7)
    n = 300
    pos = rng.random((n, 4), dtype=np.float32)
    ind = np.zeros((n, 4), np.int32)
    ind[:, 3] = np.repeat([1, 2], [200, 100])
    hdr = {"sim_type": "synthetic", "input_method": "BULK", "a_par": [1.0, 1.0, 1.0],
           "n_atom": 2, "nsuper_r": [200, 100], "at_name_out": ["Al", "U"]}
    f = io.DatFrame(header=hdr, at_ind=ind, at_pos=pos)
    p = tmp_path / "r_n0001.dat"
    io.write_dat(p, f)
    assert p.stat().st_size == (4 + 2 * 2) * io.REC_BYTES
    g = io.read_dat(p)
    assert np.array_equal(g.at_pos, pos) and np.array_equal(g.at_ind, ind)


def test_dat_rejects_corrupt_files(tmp_path):
    data = ALU_DAT.read_bytes()
    p = tmp_path / "bad.dat"
    p.write_bytes(data[:-io.REC_BYTES])          # truncated position block
    with pytest.raises(ValueError):
        io.read_dat(p)
    p.write_bytes(data[:1000])                   # not a whole record
    with pytest.raises(ValueError):
        io.read_dat(p)
    p.write_bytes(b"XX" + data[2:])              # wrong magic
    with pytest.raises(ValueError):
        io.read_dat(p)


def test_trajectory_naming_and_reading(tmp_path):
    f = io.read_dat(ALU_DAT)
    for i in (1, 2, 3):
        g = io.DatFrame(header=dict(f.header, sim_type="TIMESTEP", t_step=0.01, t_dump=0.01 * i),
                        at_ind=f.at_ind, at_pos=f.at_pos + np.float32(i))
        io.write_dat(io.frame_file(tmp_path, "traj", i), g)
    assert io.frame_file(tmp_path, "traj", 12).name == "traj_n0012.dat"
    frames, f0, t_step = io.read_trajectory(tmp_path, "traj", 1, 3)
    assert frames.shape == (3, 30000, 4)
    assert np.array_equal(frames[2], f.at_pos + np.float32(3))
    assert t_step == pytest.approx(0.01)
    # snapshots of another simulation type are unrelated in time: t_step 0
    g = io.DatFrame(header=dict(f.header, sim_type="STATIC", t_dump=0.5), at_ind=f.at_ind,
                    at_pos=f.at_pos)
    io.write_dat(io.frame_file(tmp_path, "stat", 1), g)
    io.write_dat(io.frame_file(tmp_path, "stat", 2), g)
    assert io.read_trajectory(tmp_path, "stat", 1, 2)[2] == 0.0


def test_t_step_mismatch_is_reported():
    """mp_sqom asks which value to take when the header's t_step and the t_dump difference
    differ by more than 1 %; here the caller answers or gets an error."""
    assert io.resolve_t_step("TIMESTEP", 0.01, 1.0, 1.01, 5) == pytest.approx(0.01)
    assert io.resolve_t_step("TIMESTEP", 0.01, 1.0, 1.01005, 5) == pytest.approx(0.01005)
    with pytest.raises(ValueError, match="t_dump difference"):
        io.resolve_t_step("TIMESTEP", 0.01, 1.0, 1.02, 5)
    assert io.resolve_t_step("TIMESTEP", 0.01, 1.0, 1.02, 5, prefer="header") == 0.01
    assert io.resolve_t_step("TIMESTEP", 0.01, 1.0, 1.02, 5, prefer="dump") == pytest.approx(0.02)
    assert io.resolve_t_step("TIMESTEP", 0.01, 1.0, None, 1) == 0.01
    assert io.resolve_t_step("timestep", 0.01, 1.0, 1.02, 1) == 0.01   # one frame: no check
    assert io.resolve_t_step("STATIC", 0.01, 1.0, 1.02, 5) == 0.0


def test_atom_names_par_against_dat():
    p = io.read_par(GOLDEN / "alu" / "Al_U_large.par")
    f = io.read_dat(ALU_DAT)
    par = [a[1] for a in p["atoms"]]
    assert io.resolve_atom_names(par, f.header["at_name_out"]) == ["Al", "U"]
    with pytest.raises(ValueError, match="species 2"):
        io.resolve_atom_names(["Al", "Zr"], ["Al", "U"])
    assert io.resolve_atom_names(["Al", "Zr"], ["Al", "U"], prefer="dat") == ["Al", "U"]
    assert io.resolve_atom_names(["Al", "Zr"], ["Al", "U"], prefer="par") == ["Al", "Zr"]
    with pytest.raises(ValueError, match="species in the .par"):
        io.resolve_atom_names(["Al"], ["Al", "U"], prefer="dat")


def test_read_par_namelist_and_atoms():
    p = io.read_par(GOLDEN / "alu" / "Al_U_large.par")
    flat = {}
    for grp in p.values():
        if isinstance(grp, dict):
            flat.update(grp)
    assert flat["j_weight"] == 3
    assert flat["q_step"] == pytest.approx(0.01)
    labels = [a[0] for a in p["atoms"]]
    assert labels[:2] == ["Al", "U"]


def test_namelist_parse_format_round_trip():
    items = {"a_par": [79.815962, 79.815962, 79.815962], "n_tot": 30000,
             "subst_name": "Al_U", "nsuper_r": [27600, 2400]}
    text = io.format_namelist("data_header_1", items)
    back = io.parse_namelist(text)["data_header_1"]
    assert back["n_tot"] == 30000 and back["nsuper_r"] == [27600, 2400]
    assert back["subst_name"] == "Al_U"
    assert np.allclose(back["a_par"], items["a_par"])


def test_fortran_e_edit_descriptor():
    assert io.fortran_e(0.000242) == " 0.242E-03"
    assert io.fortran_e(-1234.5) == "-0.123E+04"
    assert io.fortran_e(0.0) == " 0.000E+00"
    assert io.fortran_e(0.9996) == " 0.100E+01"      # rounding carries into a new digit
    assert io.fortran_e(1.5e-120) == " 0.150-119"    # three-digit exponent drops the E
    assert io.fortran_e(float("nan")) == "*" * 10


def test_map_rows_match_reference_output():
    """Three body lines of the reference's BZO map: parsed and re-emitted byte for byte."""
    lines = (GOLDEN / "bzo_map_rows.txt").read_text().splitlines()
    vals = np.array([[io._fix_exp(t) for t in ln.split()] for ln in lines])
    assert vals.shape[1] == 160
    assert io.format_map_rows(vals) == lines


def test_sq_table_write_read(tmp_path):
    rng = np.random.default_rng(3)
    m = rng.random((12, 7)) * 10.0 ** rng.integers(-5, 5, (12, 7))
    p = tmp_path / "map.txt"
    io.write_sq_table(p, m, substance="test", atoms=("Al", "U"), b_coh=(0.345, 0.842),
                      masks=(1, 1))
    back = io.read_sq_table(p)
    assert back.shape == m.shape
    # a 0.ddd mantissa keeps 3 digits: relative rounding error <= 0.0005/0.100
    assert np.allclose(back, m, rtol=5.01e-3, atol=0.0)


def test_sqom_settings_from_par(tmp_path):
    """&mp_sqom / &mp_out / &mp_gen of the example .par with the program's defaults for what it
    leaves out; a missing group is an error; non-periodic data switch the spatial window on."""
    st = io.read_sqom_settings(GOLDEN / "alu" / "Al_U_large.par")
    assert (st.n_int, st.s_trig, st.j_oneph, st.j_qsq) == (0, 0.0, 0, 1)
    assert (st.j_sq, st.j_wind, st.nfile_mem, st.nfile_step) == (1, 0, 200, 1)
    assert (st.j_weight, st.j_verb, st.j_proc) == (3, 0, 0)
    ta = st.time_axis(nfile=20, t_step=0.01)
    assert ta.n_int == 11                      # nfile/2, made odd for S(Q,w)
    st2 = io.read_sqom_settings(GOLDEN / "alu" / "Al_U_large.par", header={"n_cond": 0})
    assert st2.j_wind == 1
    text = (GOLDEN / "alu" / "Al_U_large.par").read_text()
    i = text.index("&mp_sqom")
    bad = tmp_path / "no_sqom.par"
    end = text.index("\n/", i) + 2            # the group's closing slash line
    bad.write_text(text[:i] + text[end:])
    with pytest.raises(ValueError, match="mp_sqom"):
        io.read_sqom_settings(bad)
    custom = tmp_path / "custom.par"
    custom.write_text(text.replace("n_int = 0", "n_int = 64\nj_sq = 0").replace("s_trig = 0", "s_trig = 2.5"))
    st3 = io.read_sqom_settings(custom)
    assert (st3.n_int, st3.j_sq, st3.s_trig) == (64, 0, 2.5)
    assert st3.time_axis(nfile=200, t_step=0.01).n_int == 64   # I(Q,t): not made odd
