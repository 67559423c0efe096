"""The reference program links against the engine through the frc_gb300.c shim.

mspms2_gb300/shim/build_md.sh compiles the reference's own sources (skipped when the
reference checkout is absent) without src/frclong.c and src/frcshort.c, adds the shim and
links libmspms2_gb300.so. Run on a machine without an sm_103 GPU, the program must read
its input, reach its first force call and stop there with the engine's no-device error,
which shows that frclong() resolves to the shim and the shim to the library.
"""
import os
import subprocess

import pytest

from mspms2_gb300 import build
from mspms2_gb300.system import load_system, write_reference_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCRIPT = os.path.join(ROOT, "mspms2_gb300", "shim", "build_md.sh")
BIN = os.path.join(ROOT, "mspms2_gb300", "shim", "_build", "mspms2_gb300_md")


@pytest.fixture(scope="module")
def md_binary():
    build.build()
    p = subprocess.run(["sh", SCRIPT], capture_output=True, text=True)
    if "skipping" in p.stderr:
        pytest.skip("reference checkout not available")
    assert p.returncode == 0, p.stderr[-2000:]
    assert os.path.exists(BIN)
    return BIN


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_program_reaches_engine_through_shim(md_binary, tmp_path):
    s, _ = load_system(os.path.join(ROOT, "tests", "golden", "water_wolf_216.npz"))
    s.nstep = 2
    write_reference_dir(s, str(tmp_path))
    p = subprocess.run([md_binary], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert p.returncode == 1
    assert "frc_gb300: mg_create (an sm_103 GPU is required) failed (status 3)" in p.stderr


def test_shim_exports_force_calls(md_binary):
    out = subprocess.run(["nm", md_binary], capture_output=True, text=True).stdout
    for sym in ("frclong", "frcshort", "initpotentialgrid_", "pass_grid_file_name_", "read_grids_", "cforce_atom_"):
        assert f" T {sym}\n" in out, sym
    dyn = subprocess.run(["nm", "-D", md_binary], capture_output=True, text=True).stdout
    assert " U mg_compute\n" in dyn
