"""The C-ABI library loads and exports every entry point include/mpsq.h declares (no GPU)."""
import re
import subprocess

from conftest import ROOT


def header_functions():
    text = (ROOT / "include" / "mpsq.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*([a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in {"if", "while"}))


def test_header_parses_expected_symbols():
    names = header_functions()
    assert "finufft2d1_" in names and "mpsq_job_create" in names
    from mp_tools_gb300 import _lib
    assert sorted(names) == sorted(_lib.EXPORTS)


def test_library_exports_all_declared(lib):
    from mp_tools_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in header_functions() if n not in exported]
    assert not missing, missing
    for n in header_functions():
        assert hasattr(lib, n)


def test_version_and_counters(lib):
    assert b"sm_103a" in lib.mpsq_version()
    assert lib.mpsq_launch_count() >= 0
