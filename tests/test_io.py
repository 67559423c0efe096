"""The reference's trajectory file (trajectory(), src/dumpxyz.c:37-66) and checkpoint file
(saveit()/loadit(), src/loadsave.c:19-128).

Fixture md_ions_trj_64.npz: a run of the compiled reference (two species of LJ ions with
Ewald, NVT, 10 steps) with its trajectory file (a frame at the start and every 3 steps)
and its checkpoint after the last step, as bytes.

CPU: the reader parses the reference's trajectory; mg_checkpoint_load reads the reference's
checkpoint and mg_checkpoint_save writes it back byte for byte (no GPU needed).
GPU: a run of mg_md_run with mg_traj_open attached writes the same header bytes and the
reference's frames (FP64 path 1e-9, mixed 1e-5 of the displacement); a checkpoint of the
engine's end state matches the reference's; mg_checkpoint_apply drops the box-keyed caches.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, load_md_case
from mspms2_gb300 import capi
from mspms2_gb300.engine import TERMS_ALL, checkpoint_load, checkpoint_save
from mspms2_gb300.files import read_trajectory, write_snapshot
from mspms2_gb300.system import load_system

CASE = "md_ions_trj_64"


def fixture():
    d = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    return d, int(d["trj_every"]), d["ref_trj"].tobytes(), d["ref_sav"].tobytes()


def reference_trajectory(tmp):
    _, _, trj, _ = fixture()
    fn = os.path.join(tmp, "ref.trj")
    with open(fn, "wb") as f:
        f.write(trj)
    return read_trajectory(fn)


def test_reference_trajectory_parses():
    s, md, state, v0, ref_log, ref_end, nsteps = load_md_case(CASE)
    _, every, _, _ = fixture()
    with tempfile.TemporaryDirectory() as td:
        t = reference_trajectory(td)
    assert t["nmole"] == [sp.nmole for sp in s.species]
    assert t["names"] == [list(sp.atom_names) for sp in s.species]
    assert all(np.array_equal(a, sp.aw) for a, sp in zip(t["aw"], s.species))
    assert len(t["frames"]) == 1 + nsteps // every
    assert np.array_equal(t["frames"][0], np.stack([s.x, s.y, s.z]))


def test_checkpoint_reads_and_writes_the_reference_bytes():
    s, md, state, v0, ref_log, ref_end, nsteps = load_md_case(CASE)
    _, _, _, sav = fixture()
    with tempfile.TemporaryDirectory() as td:
        fn, out = os.path.join(td, "sav.mspms"), os.path.join(td, "ours.mspms")
        with open(fn, "wb") as f:
            f.write(sav)
        ck = checkpoint_load(fn, s.natom, with_counters=True)
        for k, row in zip(("x", "y", "z", "vx", "vy", "vz"), ref_end):
            assert np.array_equal(ck[k], row), k
        assert ck["qq"] == md["qq"] and ck["qqs"] == md["qqs"] and ck["gg"] == md["gg"]
        assert ck["ps"] == ref_log[-1, 4] and ck["ss"] == ref_log[-1, 5]
        assert ck["istep"] == nsteps and ck["nframe"] == 1 + nsteps // fixture()[1]
        assert np.isclose(ck["boxv"], np.prod(s.box), rtol=1e-15)
        checkpoint_save(out, ck)
        assert open(out, "rb").read() == sav
        # a new run (no counters) reads only the state
        ck0 = checkpoint_load(fn, s.natom, with_counters=False)
        assert ck0["istep"] == 0 and ck0["nframe"] == 0 and np.array_equal(ck0["x"], ck["x"])


def test_snapshot_layout():
    s, _, _, _, _, _, _ = load_md_case(CASE)
    with tempfile.TemporaryDirectory() as td:
        fn = os.path.join(td, "ss.mspms")
        write_snapshot(fn, s, 7, s.box, s.x, s.y, s.z)
        lines = open(fn).read().splitlines()
    assert lines[0] == str(s.natom)
    assert lines[1] == f"7 {s.box[0]:f} {s.box[1]:f} {s.box[2]:f}"
    assert len(lines) == 2 + s.natom
    assert lines[2].split()[0] == s.species[0].atom_names[0]
    assert float(lines[2].split()[1]) == round(float(s.x[0]), 6)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_engine_trajectory_and_checkpoint_match_reference(prec):
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, md, state, v0, ref_log, ref_end, nsteps = load_md_case(CASE)
    d, every, trj, sav = fixture()
    start = np.stack([s.x, s.y, s.z])
    tol = 1e-9 if prec == "fp64" else 1e-5
    with tempfile.TemporaryDirectory() as td:
        ref = reference_trajectory(td)
        fn = os.path.join(td, "trj.mspms")
        with Engine(s, precision=prec) as eng:
            eng.traj_open(fn, every)
            pos, vel, st, log = eng.md_run(nsteps, md, v0, state=state)
            assert eng.traj_close() == len(ref["frames"])
        ours = read_trajectory(fn)
        header = len(trj) - len(ref["frames"]) * (4 * len(s.species) + 24 * s.natom)
        assert open(fn, "rb").read()[:header] == trj[:header]
        assert np.array_equal(ours["frames"][0], ref["frames"][0])
        for f in range(1, len(ref["frames"])):
            dr, dd = ours["frames"][f] - start, ref["frames"][f] - start
            assert np.linalg.norm(dr - dd) <= tol * np.linalg.norm(dd), (prec, f)
        # the engine's end state in the reference's checkpoint (bookkeeping of the
        # reference's main loop taken from its file)
        fn_ref, fn_ours = os.path.join(td, "ref.sav"), os.path.join(td, "ours.sav")
        with open(fn_ref, "wb") as f:
            f.write(sav)
        rck = checkpoint_load(fn_ref, s.natom)
        ck = dict(rck)
        ck.update(x=pos[0], y=pos[1], z=pos[2], vx=vel[0], vy=vel[1], vz=vel[2], ps=st["ps"], ss=st["ss"],
                  pss=st["pss"], sss=st["sss"])
        checkpoint_save(fn_ours, ck)
        back = checkpoint_load(fn_ours, s.natom)
    for k in ("x", "y", "z"):
        i = "xyz".index(k)
        dr, dd = back[k] - start[i], rck[k] - start[i]
        assert np.linalg.norm(dr - dd) <= tol * max(np.linalg.norm(dd), 1e-300), (prec, k)
    for k in ("vx", "vy", "vz", "ps", "ss"):
        assert np.linalg.norm(np.asarray(back[k]) - rck[k]) <= tol * np.linalg.norm(rck[k]), (prec, k)
    for k in ("istep", "nframe", "equilibrium", "counts", "qq", "gg", "boxlx", "boxv"):
        assert back[k] == rck[k], k


@pytest.mark.gpu
def test_checkpoint_apply_drops_box_caches():
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    f = 1.02
    x, y, z = (np.asarray(a) * f for a in (s.x, s.y, s.z))
    with Engine(s, precision="fp64") as eng:
        eng.compute()  # list and k-vector tables for the old box
        box = np.asarray(s.box) * f
        ck = dict(x=x, y=y, z=z, vx=np.zeros(s.natom), vy=np.zeros(s.natom), vz=np.zeros(s.natom),
                  boxlx=box[0], boxly=box[1], boxlz=box[2], boxv=float(np.prod(box)))
        eng.checkpoint_apply(ck)
        # the Ewald box constants stay the caller's (loadit leaves them); give the new ones
        s2, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
        s2.box = box
        s2.x, s2.y, s2.z = x, y, z
        eng.set_params(capi.system_params(s2))
        fl, fs, e = eng.compute(x, y, z, TERMS_ALL)
    with Engine(s2, precision="fp64") as fresh:
        fl2, fs2, e2 = fresh.compute()
    assert np.array_equal(fl, fl2) and np.array_equal(fs, fs2)
