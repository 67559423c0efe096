"""Integrators: the reference's vver_nh_3 (src/nvtnh.c:11-271) and vver (src/md.c:22-85).

Fixtures md_*.npz are trajectories of the compiled reference's own integrators (see
tests/golden/gen_golden.py): NVT water with Wolf electrostatics and 2 inner steps, NVE
Lennard-Jones fluid, NVT water with Ewald and 4 inner RESPA steps.

CPU: the oracle's restatement (oracle/md_oracle.c) reproduces each trajectory.
GPU: mg_md_run, called through the C ABI, reproduces them. Tolerances: the FP64 path
1e-9 (relative, per logged quantity and for the end state); the mixed path 1e-5 for
energies, thermostat variables and velocities and 1e-5 of the displacement for positions,
the same force tolerance the parity tests use, carried through a few steps.
"""
import numpy as np
import pytest

from conftest import load_md_case, md_golden_cases

LOG_COLS = {"ukin": 0, "uinter": 1, "uintra": 2, "ushift": 3, "ps": 4, "ss": 5, "pss": 6, "sss": 7, "tinst": 8,
            "unhts": 9, "unhtss": 10}


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def check_run(case, pos, vel, log, tol, start, ref_log, ref_end, energy_scale):
    """Compares one run against the reference record."""
    for k, col in LOG_COLS.items():
        ref = ref_log[:, col]
        scale = max(np.abs(ref).max(), 1e-300)
        if k in ("uinter", "uintra", "ushift"):
            scale = max(scale, energy_scale)
        err = np.abs(log[:, col] - ref).max() / scale
        assert err <= tol, (case, k, err)
    disp_ref = ref_end[:3] - start
    assert rel(pos - start, disp_ref) <= tol, (case, "displacement", rel(pos - start, disp_ref))
    assert rel(vel, ref_end[3:]) <= tol, (case, "velocities", rel(vel, ref_end[3:]))


@pytest.mark.parametrize("case", md_golden_cases())
def test_oracle_integrator_matches_reference(case):
    from oracle.pyoracle import Oracle
    s, md, state, v0, ref_log, ref_end, nsteps = load_md_case(case)
    start = np.stack([s.x, s.y, s.z])
    pos, vel, st, log = Oracle(s).md_run(nsteps, md, v0, state)
    scale = np.abs(ref_log[:, 1:4]).max()
    check_run(case, pos, vel, log, 1e-12, start, ref_log, ref_end, scale)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("case", md_golden_cases())
def test_engine_integrator_matches_reference(case, prec):
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, md, state, v0, ref_log, ref_end, nsteps = load_md_case(case)
    start = np.stack([s.x, s.y, s.z])
    # the energy sums of the mixed path are judged against the largest term, as in the
    # force parity tests (uinter is a small difference of large components)
    scale = np.abs(ref_log[:, 1:4]).max() * (10.0 if prec == "mixed" else 1.0)
    with Engine(s, precision=prec) as eng:
        pos, vel, st, log = eng.md_run(nsteps, md, v0, state=state)
    tol = 1e-9 if prec == "fp64" else 1e-5
    check_run(case, pos, vel, log, tol, start, ref_log, ref_end, scale)
    assert st["ukin"] == pytest.approx(ref_log[-1, 0], rel=tol)


@pytest.mark.gpu
def test_engine_integrator_continues_like_one_run():
    """Two runs of k steps equal one run of 2k steps (state carried by the caller)."""
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, md, state, v0, _, _, nsteps = load_md_case("md_water_nvt_216")
    with Engine(s, precision="fp64") as eng:
        p1, v1, st1, _ = eng.md_run(4, md, v0, state=state)
        p2, v2, st2, _ = eng.md_run(4, md, v1, x=p1[0], y=p1[1], z=p1[2],
                                     state={k: st1[k] for k in ("ps", "ss", "pss", "sss", "unhts", "unhtss")})
        pa, va, sta, _ = eng.md_run(8, md, v0, state=state)
    assert np.array_equal(p2, pa) and np.array_equal(v2, va)
    assert st2["ps"] == sta["ps"] and st2["pss"] == sta["pss"]


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("case", md_golden_cases())
def test_graph_replay_matches_step_by_step(case, prec):
    """Steps replayed as one captured CUDA graph give exactly the results of the same
    steps launched one by one, and the replay path is the one that ran."""
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, md, state, v0, ref_log, ref_end, nsteps = load_md_case(case)
    out = {}
    for graphs in (True, False):
        with Engine(s, precision=prec) as eng:
            eng.set_md_graphs(graphs)
            out[graphs] = eng.md_run(nsteps, md, v0, state=state)
            assert eng.md_graph_steps() == (nsteps if graphs else 0), (case, prec, graphs)
    (p1, v1, s1, l1), (p2, v2, s2, l2) = out[True], out[False]
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2) and np.array_equal(l1, l2)
    assert s1 == s2
