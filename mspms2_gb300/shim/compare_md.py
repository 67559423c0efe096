"""The reference program over the engine against the reference program over its own force
layer: a check of the drop-in boundary for maintainers who hold a reference checkout.

Both programs are built from the checkout (given as --ref or MSPMS2_REF):
  oracle/_ref/mspms2_ref                  the reference's own main and force layer
                                          (oracle/build_ref.sh: the src/frclong.c:86
                                          self-pair fix and raised array limits)
  mspms2_gb300/shim/_build/mspms2_gb300_md the same program with frclong()/frcshort() and the
                                          Tasos Fortran entry points from frc_gb300.c, i.e.
                                          the engine (mspms2_gb300/shim/build_md.sh)
Each case is written as an input directory (in.mspms, cfg.mspms, xyz.mspms and, for the Tasos
model, the text grids that read_grids_ reads), both programs run it for --steps steps of
the ensemble it names, writing a trajectory frame (trj.mspms) every step, and the frames
are compared. Start velocities come from the program's own seeded generator, so both runs
start from the same state; the integrator (vver_nh_3, npt_respa, vver) is the reference's
own in both. The shimmed program runs once per precision (MSPMS2_GB300_PRECISION).

  python -m mspms2_gb300.shim.compare_md --ref <checkout> [--steps 20] [--json out.json]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from mspms2_gb300 import build  # noqa: E402
from mspms2_gb300.files import read_trajectory  # noqa: E402
from mspms2_gb300.system import load_system, write_reference_dir  # noqa: E402

REF_PROG = os.path.join(ROOT, "oracle", "_ref", "mspms2_ref")
SHIM_PROG = os.path.join(HERE, "_build", "mspms2_gb300_md")

# (golden system, ensemble: 0 NVE / 1 NVT / 2 NPT, time step fs, inner steps, most steps)
CASES = {
    "water_wolf_216": ("water_wolf_216", 1, 0.5, 2, None),   # the 216-water Wolf system, NVT RESPA
    "water_ewald_512": ("water_ewald_512", 1, 0.5, 4, None),  # Ewald water, NVT RESPA
    # Tasos grids through read_grids_; after 10 steps a site of this small, hot system nears
    # the grid's edge (the reference then reuses the previous site's values, the engine
    # stops with MG_ERR_OUT_OF_GRID), so it runs at most 8 steps
    "sf_tasos": ("sf_tasos", 1, 1.0, 1, 8),
}


def build_programs(ref: str) -> None:
    build.build()
    for cmd in (["sh", os.path.join(ROOT, "oracle", "build_ref.sh"), ref],
                ["sh", os.path.join(HERE, "build_md.sh"), ref]):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0 or "skipping" in p.stderr:
            raise RuntimeError(f"{' '.join(cmd)} failed:\n{p.stderr[-3000:]}")


def run(prog: str, case_dir: str, env: dict) -> np.ndarray:
    p = subprocess.run([prog], cwd=case_dir, capture_output=True, text=True, env=env, timeout=1800)
    if p.returncode != 0:
        raise RuntimeError(f"{prog} in {case_dir} exited {p.returncode}:\n{p.stderr[-3000:]}")
    return read_trajectory(os.path.join(case_dir, "trj.mspms"))["frames"]


def compare_case(name: str, steps: int, work: str) -> dict:
    golden, ens, dt, inner, most = CASES[name]
    steps = min(steps, most) if most else steps
    s, _ = load_system(os.path.join(ROOT, "tests", "golden", golden + ".npz"))
    s.what_simulation, s.what_ensemble, s.delt_fs, s.nstep_inner, s.nstep = 0, ens, dt, inner, steps
    out = {"case": name, "ensemble": ["NVE", "NVT", "NPT"][ens], "steps": steps, "sites": s.natom}
    dirs = {}
    for key in ("ref", "fp64", "mixed"):
        d = os.path.join(work, f"{name}_{key}")
        write_reference_dir(s, d, nstep_trj=1)
        dirs[key] = d
    env = dict(os.environ)
    ref = run(REF_PROG, dirs["ref"], env)
    scale = float(np.abs(ref[-1]).max())
    for prec in ("fp64", "mixed"):
        e = dict(env, MSPMS2_GB300_PRECISION=prec)
        got = run(SHIM_PROG, dirs[prec], e)
        if got.shape != ref.shape:
            raise RuntimeError(f"{name}/{prec}: {got.shape} frames against {ref.shape}")
        diff = np.abs(got - ref).max(axis=(1, 2))
        out[prec] = {"frames": int(len(diff)), "max_abs_position_diff": float(diff.max()),
                     "final_rel_diff": float(diff[-1] / scale),
                     "per_frame_max_abs": [float(v) for v in diff]}
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MSPMS2_REF"), help="reference checkout")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--cases", default=",".join(CASES))
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    if not a.ref:
        sys.exit("give the reference checkout (--ref or MSPMS2_REF)")
    build_programs(a.ref)
    res = []
    with tempfile.TemporaryDirectory() as work:
        for name in a.cases.split(","):
            r = compare_case(name, a.steps, work)
            res.append(r)
            print(json.dumps({k: (v if k not in ("fp64", "mixed") else
                                  {kk: vv for kk, vv in v.items() if kk != "per_frame_max_abs"})
                              for k, v in r.items()}), flush=True)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(res, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
