"""Simulated annealing (siman, src/siman.c:62-182): stages of velinit + Nose-Hoover RESPA
at decreasing temperatures.

CPU: the library's stage count (mg_siman_stage_count, callable without a GPU) matches the
oracle's restated loop, which ends after the first stage below t_min; velinit of the
oracle gives zero momentum and exactly the stage temperature.
GPU: mg_siman_run, through the C ABI, reproduces the oracle's run (same Philox streams)
stage by stage. Tolerances as for the integrators: FP64 path 1e-9, mixed path 1e-5.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mspms2_gb300.capi import SIMAN_LOG_NAMES
from mspms2_gb300.system import load_system, md_params


def water():
    s, _ = load_system(os.path.join(GOLDEN, "water_wolf_216.npz"))
    s.delt_fs, s.nstep_inner = 0.5, 2
    md = md_params(s)
    md["scheme"] = 1
    return s, md


def sched(s, **kw):
    d = dict(t_initial=600.0 / s.epsilon_base, t_min=300.0 / s.epsilon_base, mu_t=1.3, n_tries=3, max_stages=8,
             seed=20240611)
    d.update(kw)
    return d


def test_stage_count_matches_oracle_loop():
    from mspms2_gb300 import build
    from oracle.pyoracle import Oracle
    lib = C.CDLL(build.build())
    lib.mg_siman_stage_count.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
    lib.mg_siman_stage_count.restype = C.c_int
    for t0, tmin, mu in [(600.0, 300.0, 1.3), (500.0, 499.0, 1.001), (300.0, 300.0, 1.1), (300.0, 299.0, 2.0)]:
        T, k = t0, 0
        while True:
            k += 1
            if T < tmin:
                break
            T /= mu
        assert lib.mg_siman_stage_count(t0, tmin, mu, 10000) == k
    assert lib.mg_siman_stage_count(600.0, 300.0, 1.3, 3) == -1   # needs 4 stages
    assert lib.mg_siman_stage_count(600.0, 300.0, 1.0, 100) == -1  # no cooling
    # the oracle's restated loop runs the same number of stages, at these temperatures
    s, md = water()
    s.species[0].nmole = 8  # a small box keeps the CPU run short
    n = 3 * 8
    s.x, s.y, s.z = s.x[:n], s.y[:n], s.z[:n]
    pos, vel, st, log = Oracle(s).siman_run(md, sched(s, n_tries=1))
    assert len(log) == lib.mg_siman_stage_count(600.0, 300.0, 1.3, 8) == 4
    assert np.allclose(log[:, 0], 600.0 / 1.3 ** np.arange(4), rtol=1e-15)


def test_oracle_velinit_zero_momentum_and_temperature():
    from oracle.pyoracle import Oracle
    s, md = water()
    pos, vel, st, log = Oracle(s).siman_run(md, sched(s, n_tries=0, t_min=599.0, max_stages=2))
    m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
    assert np.abs((vel * m).sum(1)).max() <= 1e-12 * np.abs(vel * m).sum()
    T = (m * (vel ** 2).sum(0)).sum() / md["nfree"]
    assert abs(T - log[-1, 0]) <= 1e-12 * T
    assert abs(log[-1, 5] - log[-1, 0]) <= 1e-12 * log[-1, 0]  # tinst after 0 steps


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_engine_siman_matches_oracle(prec):
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    from oracle.pyoracle import Oracle
    build.build()
    s, md = water()
    sc = sched(s)
    start = np.stack([s.x, s.y, s.z]).copy()
    rpos, rvel, rst, rlog = Oracle(s).siman_run(md, sc)
    with Engine(s, precision=prec) as eng:
        pos, vel, st, log = eng.siman_run(md, sc)
    tol = 1e-9 if prec == "fp64" else 1e-5
    assert log.shape == rlog.shape
    escale = np.abs(rlog[:, 1:5]).max()
    for k, name in enumerate(SIMAN_LOG_NAMES):
        scale = escale if name in ("uinter", "uintra", "ushift") else max(np.abs(rlog[:, k]).max(), 1e-300)
        err = np.abs(log[:, k] - rlog[:, k]).max() / scale
        assert err <= tol, (prec, name, err)
    d = np.linalg.norm((pos - start) - (rpos - start)) / np.linalg.norm(rpos - start)
    assert d <= tol, (prec, "displacement", d)
    assert np.linalg.norm(vel - rvel) / np.linalg.norm(rvel) <= tol
    for k in ("ps", "pss"):
        assert abs(st[k] - rst[k]) <= tol * max(abs(rst[k]), 1e-12), (prec, k, st[k], rst[k])


BATCH = dict(eps=1.0, sigma=1.0, rcutoff=2.5, mass=1.0, delt=0.005, qq=50.0, qqs=50.0, t_initial=2.0, t_min=1.0,
             mu_t=1.3, n_tries=5, max_stages=8, seed=0x5EED1234ABCD, nconstraint=0)


def replica_seed(seed, r):
    return (seed ^ (r * 0x9E3779B97F4A7C15)) & 0xFFFFFFFFFFFFFFFF


@pytest.mark.gpu
def test_siman_batch_matches_oracle_per_replica():
    """mg_siman_batch anneals LJ replicas of uneven size (all-pairs and cell-list boxes)
    in one launch; each replica against the oracle's siman run of that replica alone with
    the replica's seed: stage log 1e-5 (energies against the stage's energy scale) and
    positions to 1e-5 of the displacement (FP32 pair forces against FP64)."""
    from mspms2_gb300 import build, configs
    from mspms2_gb300.engine import siman_batch
    from oracle.pyoracle import Oracle
    build.build()
    sizes = [200, 350, 500, 864]
    reps = [configs.lj_replica(n, seed=70 + i) for i, n in enumerate(sizes)]
    x, y, z = (np.concatenate([getattr(s, a) for s in reps]) for a in "xyz")
    bx, by, bz, log = siman_batch(BATCH, sizes, [s.box[0] for s in reps], x, y, z)
    assert log.shape == (4, 4, 5)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for r, s in enumerate(reps):
        n = sizes[r]
        md = dict(scheme=1, nstep_inner=1, delt=BATCH["delt"], treq=1.0, qq=BATCH["qq"], qqs=BATCH["qqs"],
                  gg=3.0 * n, ggs=3.0 * n, nfree=3 * n)
        sc = dict(t_initial=BATCH["t_initial"], t_min=BATCH["t_min"], mu_t=BATCH["mu_t"], n_tries=BATCH["n_tries"],
                  max_stages=BATCH["max_stages"], seed=replica_seed(BATCH["seed"], r))
        start = np.stack([s.x, s.y, s.z]).copy()
        rpos, _, _, rlog = Oracle(s).siman_run(md, sc)
        assert rlog.shape[0] == log.shape[1]
        escale = np.abs(rlog[:, [2, 4]]).max()
        for kk, ko in zip([0, 1, 2, 3, 4], [0, 1, 2, 4, 5]):
            scale = escale if kk in (2, 3) else np.abs(rlog[:, ko]).max()
            err = np.abs(log[r, :, kk] - rlog[:, ko]).max() / scale
            assert err <= 1e-5, (r, SIMAN_LOG_NAMES[ko], err)
        pos = np.stack([bx[off[r]:off[r + 1]], by[off[r]:off[r + 1]], bz[off[r]:off[r + 1]]])
        d = np.linalg.norm((pos - start) - (rpos - start)) / np.linalg.norm(rpos - start)
        assert d <= 1e-5, (r, d)


def tasos_replicas(nrep):
    """Replicas of the Tasos golden system (12 sites in a 12 A box over a 4.2 x 4.2 A grid),
    cooled briefly from a low temperature so that no site leaves the grid."""
    import os
    from conftest import GOLDEN
    from mspms2_gb300.system import load_system, md_params, time_base
    s, _ = load_system(os.path.join(GOLDEN, "sf_tasos.npz"))
    s.delt_fs, s.nstep_inner, s.treq_K = 0.5, 1, 30.0
    md = md_params(s)
    md["scheme"] = 1
    tau = 50.0 / time_base(s)
    md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
    scheds = [dict(t_initial=30.0 / s.epsilon_base, t_min=20.0 / s.epsilon_base, mu_t=1.2, n_tries=4, max_stages=4,
                   seed=1000 + r) for r in range(nrep)]
    return s, md, scheds


@pytest.mark.gpu
def test_shared_tasos_tables_and_concurrent_replicas():
    """Replicas that share one copy of the Tasos tables (mg_sf_tasos_share): the forces are
    the same bits as with tables of their own; the storage outlives the context that made
    it; and annealing runs of several replicas, each a context on its own stream driven from
    its own host thread, give each replica's result alone."""
    import threading
    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine
    build.build()
    s, md, scheds = tasos_replicas(3)
    own = Engine(s, precision="mixed")
    f_own = own.compute()
    own.close()
    alone = []
    for sc in scheds:  # a fresh context each, as the concurrent ones below
        with Engine(s, precision="mixed") as e:
            alone.append(e.siman_run(md, sc))
    src = Engine(s, precision="mixed")
    engs = [Engine(s, precision="mixed") for _ in scheds]
    for e in engs:
        e.sf_tasos_share(src)
    src.close()  # the tables stay with the contexts that share them
    f_sh = engs[0].compute()
    assert np.array_equal(f_own[0], f_sh[0]) and np.array_equal(f_own[1], f_sh[1]) and f_own[2] == f_sh[2]
    out = [None] * len(engs)

    def work(r):
        out[r] = engs[r].siman_run(md, scheds[r])

    th = [threading.Thread(target=work, args=(r,)) for r in range(len(engs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for r in range(len(engs)):
        for a, b in zip(out[r][:2] + (out[r][3],), alone[r][:2] + (alone[r][3],)):
            assert np.array_equal(a, b), r
    for e in engs:
        e.close()
