"""NPT: the reference's npt_respa (src/nptnh.c:134-234) with npt_nh_operator
(src/nptnh.c:10-132): isotropic thermostat + barostat, positions and box scaled every
inner step, LJ long-range pressure correction, Ewald box constants refreshed.

Fixtures md_*_npt_*.npz are trajectories of the compiled reference's own npt_respa (see
tests/golden/gen_golden.py): Wolf water with the LJ correction and 2 inner steps, Ewald
water with 4 inner steps (the k-vector set stays, the box constants change).

CPU: the oracle's restatement (oracle/md_oracle.c) reproduces each trajectory.
GPU: mg_npt_run, through the C ABI, reproduces them: FP64 path 1e-9, mixed path 1e-5
(relative per logged quantity, displacement and velocities). Row 0's pinst is not
compared: the reference leaves pinst unset until its first step.
"""
import numpy as np
import pytest

from conftest import load_npt_case, npt_golden_cases
from mspms2_gb300.capi import NPT_LOG_NAMES


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def check(case, pos, vel, box, log, tol, start, ref_log, ref_end):
    escale = np.abs(ref_log[:, 1:4]).max()
    for k, name in enumerate(NPT_LOG_NAMES):
        rows = slice(1, None) if name == "pinst" else slice(None)
        ref = ref_log[rows, k]
        scale = escale if name in ("uinter", "uintra", "ushift") else max(np.abs(ref).max(), 1e-300)
        err = np.abs(log[rows, k] - ref).max() / scale
        assert err <= tol, (case, name, err)
    assert rel(pos - start, ref_end[:3] - start) <= tol, (case, "displacement")
    assert rel(vel, ref_end[3:]) <= tol, (case, "velocities")
    assert abs(box[0] - ref_log[-1, 10]) <= tol * ref_log[-1, 10]


@pytest.mark.parametrize("case", npt_golden_cases())
def test_oracle_npt_matches_reference(case):
    from oracle.pyoracle import Oracle
    s, npt, st0, box, v0, ref_log, ref_end, nsteps = load_npt_case(case)
    start = np.stack([s.x, s.y, s.z])
    pos, vel, bx, st, log = Oracle(s).npt_run(nsteps, npt, v0, box, st0)
    check(case, pos, vel, bx, log, 1e-12, start, ref_log, ref_end)


def test_npt_params_of_system():
    from mspms2_gb300.system import npt_params, npt_state0, pressure_base
    s, npt, st0, box, v0, ref_log, ref_end, nsteps = load_npt_case("md_water_npt_216")
    p = npt_params(s)
    for k in ("nstep_inner", "nfree", "lj_lrc"):
        assert p[k] == npt[k], k
    for k in ("delt", "treq", "preq", "qts", "qbs"):
        assert abs(p[k] - npt[k]) <= 1e-14 * abs(npt[k]), (k, p[k], npt[k])
    s0 = npt_state0(s)
    for k in ("vts", "vbs", "rts"):
        assert abs(s0[k] - st0[k]) <= 1e-14 * max(abs(st0[k]), 1e-300), k
    assert abs(pressure_base(s) * p["preq"] - s.preq_bar) <= 1e-12 * s.preq_bar


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("case", npt_golden_cases())
def test_engine_npt_matches_reference(case, prec):
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, npt, st0, box, v0, ref_log, ref_end, nsteps = load_npt_case(case)
    start = np.stack([s.x, s.y, s.z])
    with Engine(s, precision=prec) as eng:
        pos, vel, bx, st, log = eng.npt_run(nsteps, npt, v0, st0, box=box)
    check(case, pos, vel, bx, log, 1e-9 if prec == "fp64" else 1e-5, start, ref_log, ref_end)
