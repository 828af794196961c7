"""Builds the golden fixtures of the test suite from the MP_TOOLS reference tree.

Run once where the reference tree is mounted:
    python tests/golden/make_fixtures.py /path/to/MP_tools
It copies the Al-U example input (one frame file and its .par) and extracts the numbers of
mp_sql's Al-U output tables (Z(Q), I(Q), S(Q), unscaled I(Q): files _40.._43) and of mp_sqom's
BZO map body (three lines, for the text-format test) into small files beside this script.
"""
import json
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def table(path):
    lines = Path(path).read_text().splitlines()
    meta = {}
    for ln in lines:
        if ln.strip().startswith("Output:"):
            meta["output"] = ln.split(":", 1)[1].strip()
        if "Smoothing FWHM" in ln:
            meta["smooth_fwhm_A"] = float(ln.split()[-1])
        if ln.strip().startswith("Q [A-1]"):
            meta["columns"] = ln.split()[2:]
    rows = []
    for ln in lines:
        tok = ln.split()
        try:
            vals = [float(t) for t in tok]
        except ValueError:
            continue
        if len(vals) >= 4:
            rows.append(vals)
    return meta, np.array(rows)


def main(ref):
    ref = Path(ref)
    alu = ref / "examples" / "amorphous_Al92U08"
    (HERE / "alu").mkdir(exist_ok=True)
    shutil.copyfile(alu / "data" / "Al_U_large_n0001.dat", HERE / "alu" / "Al_U_large_n0001.dat")
    shutil.copyfile(alu / "Al_U_large.par", HERE / "alu" / "Al_U_large.par")
    arrays, metas = {}, {}
    for k, mode in ((40, 5), (41, 6), (42, 4), (43, 7)):
        meta, rows = table(alu / f"Al_U_large_sql_0001_{k}.txt")
        meta["mode"] = mode
        metas[str(k)] = meta
        arrays[f"t{k}"] = rows
    np.savez_compressed(HERE / "alu" / "sql_golden.npz", **arrays)
    (HERE / "alu" / "sql_golden.json").write_text(json.dumps(metas, indent=1))
    bzo = ref / "examples" / "single_crystal_BZO" / "bzo200d_sq_0001_0020_07.txt"
    lines = bzo.read_text().splitlines()
    (HERE / "bzo_map_rows.txt").write_text("\n".join(lines[-160:-157]) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of the MP_TOOLS source tree>")
    main(sys.argv[1])
