import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103) device")


def golden_cases():
    """Force fixtures (frclong/frcshort outputs of the compiled reference)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and not f.startswith(("md_", "sfgrid_", "hmc_")))


def md_golden_cases():
    """Trajectory fixtures of the reference's NVT and NVE integrators."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and f.startswith("md_") and "_npt" not in f)


def npt_golden_cases():
    """Trajectory fixtures of the reference's npt_respa."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and f.startswith("md_") and "_npt" in f)


def load_npt_case(name):
    """(system at the start, npt params dict, start state dict (vts, vbs, rts), start box,
    start velocities [3, n], reference log [(nsteps+1), 12], reference end [6, n], nsteps)."""
    import numpy as np
    from mspms2_gb300.system import load_system
    s, d = load_system(os.path.join(GOLDEN, name + ".npz"))
    _, nstep_inner, nfree, nsteps, lj_lrc = (int(v) for v in d["md_int"])
    delt, treq, qts, qbs, preq = (float(v) for v in d["md_real"])
    npt = dict(nstep_inner=nstep_inner, delt=delt, treq=treq, preq=preq, qts=qts, qbs=qbs, nfree=nfree,
               lj_lrc=lj_lrc)
    vts, vbs, rts, boxlx, _ = (float(v) for v in d["md_state0"])
    return (s, npt, dict(vts=vts, vbs=vbs, rts=rts), np.array(s.box, dtype=float), np.array(d["md_v0"]),
            np.array(d["md_log"]), np.array(d["md_end"]), nsteps)


def load_md_case(name):
    """(system at the start, md params dict, start state dict, start velocities [3, n],
    reference log [(nsteps+1), 12], reference end [6, n], nsteps)."""
    import numpy as np
    from mspms2_gb300.system import load_system
    s, d = load_system(os.path.join(GOLDEN, name + ".npz"))
    scheme, nstep_inner, nfree, nsteps = (int(v) for v in d["md_int"])
    delt, treq, qq, qqs, gg, ggs = (float(v) for v in d["md_real"])
    md = dict(scheme=scheme, nstep_inner=nstep_inner, delt=delt, treq=treq, qq=qq, qqs=qqs, gg=gg, ggs=ggs,
              nfree=nfree)
    state = dict(zip(("ps", "ss", "pss", "sss"), (float(v) for v in d["md_state0"])))
    return s, md, state, np.array(d["md_v0"]), np.array(d["md_log"]), np.array(d["md_end"]), nsteps


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
