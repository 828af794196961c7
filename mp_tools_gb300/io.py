"""MP_TOOLS file formats used on the S(Q,omega) path.

* ``.dat`` frame files (one frame per file, ``<master>_nNNNN.dat``): direct-access records of
  4096 bytes — record 1 ``MP_TOOLS <version> <n_head> <time stamp>``, records 2..n_head the
  namelists ``data_header_1/2/3`` as text, then ``n_rec`` records of ``at_ind`` (int32 x4 per
  atom) and ``n_rec`` records of ``at_pos`` (float32 x, y, z, charge), 256 atoms per record,
  the last record of each block zero-padded; velocities/forces/shells may follow.  Read as
  mp_sqom reads them (code/src/mp_sqom56.f90:247-301, :609-670, :967-1035), written as the
  MP_TOOLS converters write them (code/src/mp_latt56.f90:295-343).
* ``.par`` parameter files: an ``atoms`` section and Fortran namelists (``&mp_sqom``, ...).
* reference tables ``neutron_xs.txt`` / ``xray_ff.txt`` (name followed by values).
* the mp_sqom text map (code/src/mp_sqom56.f90:1995-2045): header lines, then one line per
  Q_x pixel with the Q_y pixels in the Fortran format ``200(1x,5e10.3)``.
"""
from __future__ import annotations

import math
import os
import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

REC_BYTES = 4096
ATOMS_PER_REC = 256  # 1024 32-bit words / 4 components


# ------------------------------------------------------------------------------ namelists
_TOKEN = re.compile(r"""'(?:[^']|'')*'|"(?:[^"]|"")*"|[^\s,]+""")


def _parse_value(tok: str):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"":
        return t[1:-1].replace(t[0] * 2, t[0]).rstrip()
    low = t.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    try:
        if re.fullmatch(r"[+-]?\d+", t):
            return int(t)
        return float(t.replace("d", "e").replace("D", "E"))
    except ValueError:
        return t


def _strip_comment(line: str) -> str:
    """Drops a trailing ``!`` comment that is not inside a quoted string."""
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i]
    return line


def parse_namelist(text: str) -> dict:
    """Parses Fortran namelist groups (``&name key=value ... /``) into
    {group_lower: {key_lower: value or list}}.  Supports repeat counts ``3*1.0``, quoted
    strings, logicals and ``!`` comments."""
    text = "\n".join(_strip_comment(line) for line in text.splitlines())
    groups = {}
    for m in re.finditer(r"&(\w+)(.*?)(?:/|&end)", text, flags=re.S | re.I):
        name = m.group(1).lower()
        body = m.group(2)
        items = {}
        parts = re.split(r"(\b[A-Za-z_]\w*(?:\(\s*[\d:, ]*\))?)\s*=", body)
        # parts: [pre, key1, vals1, key2, vals2, ...]
        for k in range(1, len(parts) - 1, 2):
            key = re.sub(r"\(.*\)", "", parts[k]).lower()
            vals = []
            for tok in _TOKEN.findall(parts[k + 1]):
                rep = re.fullmatch(r"(\d+)\*(.*)", tok)
                if rep and not tok.startswith(("'", '"')):
                    vals.extend([_parse_value(rep.group(2))] * int(rep.group(1)))
                else:
                    v = _parse_value(tok)
                    if v is not None:
                        vals.append(v)
            items[key] = vals[0] if len(vals) == 1 else vals
        groups[name] = items
    return groups


def _fmt_nml_value(v) -> str:
    if isinstance(v, str):
        return "'" + v.replace("'", "''") + "'"
    if isinstance(v, bool):
        return ".true." if v else ".false."
    if isinstance(v, (list, tuple, np.ndarray)):
        return ", ".join(_fmt_nml_value(x) for x in v)
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


def format_namelist(name: str, items: dict) -> str:
    body = ", ".join(f"{k.upper()}= {_fmt_nml_value(v)}" for k, v in items.items())
    return f"&{name.upper()}  {body},  /"


# ------------------------------------------------------------------------------ .dat files
@dataclass
class DatFrame:
    header: dict                      # data_header_1 (+ _2, _3) items, lower-case keys
    at_ind: np.ndarray                # (n_tot, 4) int32
    at_pos: np.ndarray                # (n_tot, 4) float32
    n_head: int = 4
    version: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n_tot(self) -> int:
        return int(self.at_pos.shape[0])

    def species_counts(self) -> list:
        v = self.header.get("nsuper_r")
        return [int(x) for x in (v if isinstance(v, list) else [v])]

    def a_cell_inv(self):
        v = self.header.get("a_cell_inv")
        if v is None:
            return None
        # the namelist writes a_cell_inv(3,3) column-major
        return np.asarray(v, np.float32).reshape(3, 3).T


def read_dat(path, read_index: bool = True) -> DatFrame:
    """Reads one frame file.  Raises ValueError on a truncated or corrupt file."""
    data = Path(path).read_bytes()
    if len(data) < REC_BYTES or len(data) % REC_BYTES:
        raise ValueError(f"{path}: size {len(data)} is not a positive multiple of {REC_BYTES}")
    rec1 = data[:REC_BYTES].decode("latin-1")
    if not rec1.startswith("MP_TOOLS"):
        raise ValueError(f"{path}: record 1 does not start with MP_TOOLS (old headers unsupported)")
    version = rec1[16:20].strip()
    try:
        n_head = int(rec1[20:36])
    except ValueError as exc:
        raise ValueError(f"{path}: bad n_head field {rec1[20:36]!r}") from exc
    if n_head < 3 or n_head * REC_BYTES > len(data):
        raise ValueError(f"{path}: n_head = {n_head} inconsistent with the file size")
    header = {}
    for r in range(1, n_head):
        txt = data[r * REC_BYTES:(r + 1) * REC_BYTES].decode("latin-1")
        for grp in parse_namelist(txt).values():
            header.update(grp)
    n_tot = int(header["n_tot"])
    n_rec = int(header.get("n_rec", math.ceil(n_tot / ATOMS_PER_REC)))
    if n_rec != math.ceil(n_tot / ATOMS_PER_REC):
        raise ValueError(f"{path}: n_rec {n_rec} does not match n_tot {n_tot}")
    need = (n_head + 2 * n_rec) * REC_BYTES
    if len(data) < need:
        raise ValueError(f"{path}: truncated ({len(data)} < {need} bytes)")
    o = n_head * REC_BYTES
    ind = np.frombuffer(data, dtype="<i4", count=4 * n_tot, offset=o).reshape(n_tot, 4)
    o += n_rec * REC_BYTES
    pos = np.frombuffer(data, dtype="<f4", count=4 * n_tot, offset=o).reshape(n_tot, 4)
    counts = header.get("nsuper_r")
    if counts is not None:
        counts = counts if isinstance(counts, list) else [counts]
        if sum(int(c) for c in counts) != n_tot:
            raise ValueError(f"{path}: species counts {counts} do not add up to n_tot {n_tot}")
    return DatFrame(header=header, at_ind=ind.copy() if read_index else ind, at_pos=pos.copy(),
                    n_head=n_head, version=version)


def write_dat(path, frame: DatFrame, version: str = "1.56", stamp: str = "") -> None:
    """Writes one frame in the MP_TOOLS layout (4 header records)."""
    h = dict(frame.header)
    n_tot = frame.n_tot
    n_rec = math.ceil(n_tot / ATOMS_PER_REC)
    h["n_tot"] = n_tot
    h["n_rec"] = n_rec
    keys1 = ["sim_type", "dat_type", "input_method", "file_par", "subst_name", "t_ms", "t_step",
             "t_dump", "temp", "temp_cs", "a_par", "angle", "n_row", "n_atom", "n_eq", "n_traj",
             "j_shell_out", "n_cond", "n_rec", "n_tot", "filter_name", "filter_fwhm"]
    keys2 = ["at_name_out", "at_base", "at_occup_r", "nsuper_r"]
    keys3 = ["a_cell", "a_cell_inv"]
    recs = [("MP_TOOLS".ljust(16) + version.ljust(4)[:4] + "4".rjust(16) + "   " + stamp)]
    recs.append(format_namelist("data_header_1", {k: h[k] for k in keys1 if k in h}))
    recs.append(format_namelist("data_header_2", {k: h[k] for k in keys2 if k in h}))
    recs.append(format_namelist("data_header_3", {k: h[k] for k in keys3 if k in h}))
    out = bytearray()
    for r in recs:
        b = r.encode("latin-1")
        if len(b) > REC_BYTES:
            raise ValueError("header record longer than 4096 bytes")
        out += b.ljust(REC_BYTES, b" ")
    for arr, dt in ((frame.at_ind, "<i4"), (frame.at_pos, "<f4")):
        blk = np.zeros(n_rec * ATOMS_PER_REC * 4, dt)
        blk[:4 * n_tot] = np.asarray(arr, dt).reshape(-1)
        out += blk.tobytes()
    Path(path).write_bytes(bytes(out))


def frame_file(data_dir, master: str, index: int | None) -> Path:
    """./data/<master>_nNNNN.dat naming (mp_sqom56.f90:236-244); index None = single file."""
    if index is None:
        return Path(data_dir) / f"{master}.dat"
    tag = f"{index:04d}" if index <= 9999 else str(index)
    return Path(data_dir) / f"{master}_n{tag}.dat"


def resolve_t_step(sim_type: str, t_step_header: float, t_dump0: float, t_dump1: float | None,
                   n_frames: int, prefer: str | None = None) -> float:
    """Time step between the frames used, as mp_sqom settles it (mp_sqom56.f90:304-342): 0
    for a simulation type other than TIMESTEP (unrelated snapshots); otherwise the t_dump
    difference of the first two frames used (the header's t_step for a single frame).  Where
    that difference and the header's t_step differ by more than 1 % of the latter and more
    than one frame is used, the reference asks which to take: prefer='header' or 'dump'
    answers, None raises ValueError naming both values."""
    if str(sim_type).strip().upper() != "TIMESTEP":
        return 0.0
    if t_dump1 is None or n_frames < 2:
        return float(t_step_header)
    dump = float(t_dump1) - float(t_dump0)
    if abs(dump - t_step_header) > 0.01 * abs(t_step_header):
        if prefer == "header":
            return float(t_step_header)
        if prefer == "dump":
            return dump
        raise ValueError(f"t_step {t_step_header} of the data header does not match the t_dump "
                         f"difference {dump}: pass t_step_prefer='header' or 'dump'")
    return dump


def resolve_atom_names(par_names, dat_names, prefer: str | None = None) -> list:
    """Species names of the .par atoms section checked against the .dat header's at_name_out
    (mp_sqom56.f90:435-443).  Equal lists pass.  At a mismatch the reference asks whether to
    take the .dat names: prefer='dat' returns them, 'par' keeps the .par names, None raises
    ValueError naming the first species that differs.  Lists of different lengths are an
    error."""
    par_names, dat_names = [str(x).strip() for x in par_names], [str(x).strip() for x in dat_names]
    if len(par_names) != len(dat_names):
        raise ValueError(f"{len(par_names)} species in the .par atoms section, "
                         f"{len(dat_names)} in the .dat header")
    for j, (a, b) in enumerate(zip(par_names, dat_names), start=1):
        if a != b:
            if prefer == "dat":
                return dat_names
            if prefer == "par":
                return par_names
            raise ValueError(f"species {j}: {a!r} in the .par file, {b!r} in the .dat header: "
                             "pass prefer='dat' or 'par'")
    return par_names


def read_trajectory(data_dir, master: str, first: int, last: int, step: int = 1,
                    t_step_prefer: str | None = None):
    """Reads frames first..last into (frames, n_tot, 4) float32 plus the first frame's header,
    cell indices and the time step between frames (``resolve_t_step`` on the first frame's
    header and the t_dump of the first two frames read, as mp_sqom derives it at :303-342)."""
    idx = list(range(first, last + 1, step))
    f0 = read_dat(frame_file(data_dir, master, idx[0]))
    frames = np.empty((len(idx), f0.n_tot, 4), np.float32)
    frames[0] = f0.at_pos
    t_dump = [float(f0.header.get("t_dump", 0.0))]
    for k, i in enumerate(idx[1:], start=1):
        f = read_dat(frame_file(data_dir, master, i), read_index=False)
        if f.n_tot != f0.n_tot:
            raise ValueError(f"frame {i}: {f.n_tot} atoms, frame {idx[0]}: {f0.n_tot}")
        frames[k] = f.at_pos
        t_dump.append(float(f.header.get("t_dump", 0.0)))
    t_step = resolve_t_step(f0.header.get("sim_type", ""), float(f0.header.get("t_step", 0.0)),
                            t_dump[0], t_dump[1] if len(idx) > 1 else None, len(idx),
                            prefer=t_step_prefer)
    return frames, f0, t_step


# --------------------------------------------------------------------------------- .par files
def read_par(path) -> dict:
    """Namelist groups of a .par file plus its ``atoms`` section as a list of
    (label, name, x, y, z, occupancy, extension) tuples (mp_sqom56.f90:357-443)."""
    text = Path(path).read_text(errors="replace")
    groups = parse_namelist(text)
    atoms = []
    lines = text.splitlines()
    for i, line in enumerate(lines):
        if line.strip().lower().startswith("atoms"):
            for ln in lines[i + 1:]:
                tok = re.split(r"[!#]", ln)[0].split()
                if len(tok) < 6:
                    break
                ext = tok[6] if len(tok) > 6 else ""
                if ext.lower() == "n":
                    ext = ""
                atoms.append((tok[0], tok[1], float(tok[2]), float(tok[3]), float(tok[4]),
                              float(tok[5]), ext))
            break
    groups["atoms"] = atoms
    return groups


@dataclass
class SqomSettings:
    """mp_sqom's run settings from a .par file: its namelist &mp_sqom, with the values the
    program assigns before reading it (mp_sqom56.f90:207-219; the documented defaults of the
    .par comments for n_int, j_oneph and j_qsq, which the program leaves unset), plus
    &mp_out's j_weight and &mp_gen's j_verb / j_proc (:153-160, :370-416)."""
    n_int: int = 0          # time window in frames, 0 = nfile/2 (odd for S(Q,w))
    nfile_mem: int = 200    # frames held in memory before the transform
    nfile_step: int = 1
    s_trig: float = 0.0     # speckle-filter trigger ratio, 0 = off
    j_oneph: int = 0        # 1 = one-phonon mode
    j_sq: int = 1           # 1 = S(Q,w), 0 = I(Q,t)
    j_qsq: int = 1          # 1 keeps the Q^2 scaling, 0 divides the maps by Q^2
    j_wind: int = 0         # spatial Hann window; forced on for non-periodic data (n_cond = 0)
    j_interp: int = 0
    j_test: int = 0
    j_weight: int = 1       # 1 unit, 2 neutron b_coh, 3 X-ray form factors
    j_verb: int = 1
    j_proc: int = 0

    def time_axis(self, nfile: int, t_step: float):
        """The TimeAxis these settings give for nfile frames t_step apart."""
        from .sqom import TimeAxis
        return TimeAxis(nfile=nfile, t_step=t_step, n_int=self.n_int, j_sq=self.j_sq)


def read_sqom_settings(path, header: dict | None = None) -> SqomSettings:
    """Reads mp_sqom's settings from a .par file.  The reference stops when &mp_gen, &mp_out or
    &mp_sqom is missing (mp_sqom56.f90:372-408): here that is a ValueError.  With a frame
    header whose n_cond is 0 (non-periodic boundaries) the spatial window is switched on, as
    the program does at :351-355."""
    groups = read_par(path)
    missing = [g for g in ("mp_gen", "mp_out", "mp_sqom") if not isinstance(groups.get(g), dict)]
    if missing:
        raise ValueError(f"{path}: namelist group(s) {', '.join(missing)} missing")
    st = SqomSettings()
    names = {f for f in st.__dataclass_fields__}
    for grp, keys in (("mp_sqom", None), ("mp_out", ("j_weight",)), ("mp_gen", ("j_verb", "j_proc"))):
        for k, v in groups[grp].items():
            if (keys is None and k in names) or (keys is not None and k in keys):
                setattr(st, k, type(getattr(st, k))(v))
    if header is not None and int(header.get("n_cond", 1)) == 0:
        st.j_wind = 1
    return st


def read_table(path) -> dict:
    """Reference tables (neutron_xs.txt: label b_coh[fm] ...; xray_ff.txt: label a1 b1 a2 b2 a3
    b3 a4 b4 c): {label: [values...]} of the numeric columns that follow each label."""
    out = {}
    for line in Path(path).read_text(errors="replace").splitlines():
        tok = line.split()
        if not tok or tok[0].startswith(("!", "#")):
            continue
        vals = []
        for t in tok[1:]:
            try:
                vals.append(float(t))
            except ValueError:
                break
        if vals:
            out.setdefault(tok[0], vals)
    return out


# ------------------------------------------------------------------------------- text maps
def fortran_e(v: float, w: int = 10, d: int = 3) -> str:
    """Fortran Ew.d edit descriptor (0.ddd E+ee mantissa form)."""
    v = float(v)
    if not math.isfinite(v):
        return ("*" * w)
    if v == 0.0:
        s = "0." + "0" * d + "E+00"
    else:
        e = math.floor(math.log10(abs(v))) + 1
        m = abs(v) / 10.0 ** e
        digits = round(m * 10 ** d)
        if digits >= 10 ** d:  # rounding carried into a new digit
            digits //= 10
            e += 1
        mant = "0." + str(digits).rjust(d, "0")
        s = (mant + ("E%+03d" % e)) if abs(e) <= 99 else (mant + ("%+04d" % e))
        if v < 0:
            s = "-" + s
    return s.rjust(w) if len(s) <= w else "*" * w


def format_map_rows(values: np.ndarray) -> list:
    """Lines of the mp_sqom map body: each row of `values` (n_qx x n_qy) in 200(1x,5e10.3)."""
    lines = []
    for row in np.asarray(values):
        parts = []
        for g in range(0, len(row), 5):
            parts.append(" " + "".join(fortran_e(x) for x in row[g:g + 5]))
        lines.append("".join(parts))
    return lines


def write_sq_table(path, values: np.ndarray, *, tool: str = "MP_SQOM 1.56 (GB300)",
                   substance: str = "", input_files: str = "", atoms=(), weights_label="",
                   b_coh=(), masks=(), e1=(1, 0, 0), e2=(0, 1, 0), q_center=(0, 0, 0),
                   energy=None, resolution=None, x_range=(0.0, 0.0), y_range=(0.0, 0.0)) -> None:
    """Writes an S(Q) / S(Q,omega) map in the layout of mp_sqom's text output."""
    n_qx, n_qy = np.asarray(values).shape
    hdr = [f" *****    {tool}: total scattering cross-section     *****", "",
           f" Substance:    {substance}", f" Input files:  {input_files}",
           " Atoms:        " + "".join(f"{a:<7s}" for a in atoms),
           f" {weights_label} b_coh:      " + "".join(f"{b:7.3f}" for b in b_coh),
           " Atom masks: " + "".join(f"{m:3d}    " for m in masks),
           " Q-plane: e1 = [" + "".join(f"{x:6.2f}" for x in e1) + "], e2 = ["
           + "".join(f"{x:6.2f}" for x in e2) + "]",
           " Q center:   " + "   ".join(f"{x:.8f}" for x in q_center)]
    if energy is None:
        hdr.append(" Total scattering (infinite energy width)   0.00000000       9999.00000")
    else:
        hdr.append(f" Energy transfer & resolution [THz]:   {energy:.8f}       {resolution:.8f}")
    hdr.append(f" Plot size X (lines):   {n_qx:10d} {x_range[0]:.9f}   {x_range[1]:.9f}")
    hdr.append(f" Plot size Y (columns): {n_qy:10d} {y_range[0]:.9f}   {y_range[1]:.9f}")
    hdr.append("")
    Path(path).write_text("\n".join(hdr + format_map_rows(values)) + "\n")


def read_sq_table(path) -> np.ndarray:
    """Reads the value block of an mp_sqom text map (any header length)."""
    lines = Path(path).read_text().splitlines()
    n_qx = n_qy = None
    for ln in lines:
        if "Plot size X" in ln:
            n_qx = int(ln.split(":")[1].split()[0])
        if "Plot size Y" in ln:
            n_qy = int(ln.split(":")[1].split()[0])
    if n_qx is None or n_qy is None:
        raise ValueError(f"{path}: no plot size lines")
    body = lines[-n_qx:]
    vals = [[float(x.replace("E", "e")) if "E" in x else _fix_exp(x) for x in ln.split()] for ln in body]
    arr = np.array(vals, dtype=np.float64)
    if arr.shape != (n_qx, n_qy):
        raise ValueError(f"{path}: body shape {arr.shape} != ({n_qx}, {n_qy})")
    return arr


def _fix_exp(tok: str) -> float:
    # 0.123-100 (three-digit exponent without the letter E)
    m = re.fullmatch(r"(-?\d*\.\d+)([+-]\d{3})", tok)
    if m:
        return float(m.group(1) + "e" + m.group(2))
    return float(tok)
