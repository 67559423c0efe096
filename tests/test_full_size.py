"""Parity at the benchmark sizes: the engine, called through its C ABI, against one full
call of the CPU oracle (orc_frclong_mt on all host threads, with orc_frcshort) and
against the CPU cluster-list builder.

  C2  32,768 SPC/Fw waters (98,304 sites), box 99.3 A, Ewald alpha 0.3/A, Rc 10 A,
      KMAX 24, KSQMAX 576 (src/frclong.c:56-218 and :988-1129 at that size)
  C4  4,096 waters (12,288 sites), box 49.66 A, Ewald alpha 0.3/A, Rc 10 A, KMAX 12
  C5  20,000 united-atom n-butane (80,000 sites), LJ Rc 14 A, inside 7 (11,11) nanotubes
      seen through two Tasos tables at 0.1 A (1271 x 1271 x 25 nodes each, computed on the
      GPU by mg_sfgrid_tasos and handed to the oracle and the engine alike)

Tolerances are those of test_gpu_parity: norm-wise relative force error 1e-5 (mixed) and
1e-10 (FP64); each energy relative to the terms it is made of. The benchmark molecules sit
at their template geometry, where the bonded (short) forces nearly vanish; that block's
error is judged against the system's force scale (the norm of the long forces). The oracle
call of each system runs once per session and is shared by both precisions.
"""
import os

import numpy as np
import pytest

from mspms2_gb300 import build, configs
from mspms2_gb300.engine import TERMS_LONG, Engine, sfgrid_tasos
from mspms2_gb300.system import SF_TASOS, TasosGrid
from test_gpu_parity import FLOOR, LONG_E, SHORT_E, TOL, component_scale, energy_scale, rel

pytestmark = pytest.mark.gpu

_ORACLE = {}


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def c5_system():
    """C5 with its two Tasos tables (CH3 type 1, CH2 type 2) computed on the GPU."""
    s, tubes = configs.butane_in_tube_bundle()
    nx, ny, nz, h = configs.C5_TASOS_NODES + (configs.c5_tasos_spacing(tubes),)
    s.tasos = []
    for sig, eps in configs.C5_TASOS_TYPES:
        v = sfgrid_tasos(configs.c5_tasos_spec(tubes, sig, eps), nx, ny, nz, h, precision="fp64")
        s.tasos.append(TasosGrid(nx, ny, nz, h[0], h[1], h[2], tubes["period"], v))
    s.sf_type = SF_TASOS
    return s


def system_and_reference(name):
    if name not in _ORACLE:
        from oracle.pyoracle import Oracle
        s = {"c2": configs.water_c2, "c4": configs.water_c4, "c5": c5_system}[name]()
        s.respa_split = 0.0
        o = Oracle(s)
        fl, el, flags = o.frclong_mt(host_threads())
        fs, es, err = o.frcshort()
        assert flags == 0 and err == 0
        _ORACLE[name] = (s, fl, fs, {**el, **es})
    return _ORACLE[name]


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("name", ["c4", "c5", "c2"])
def test_full_size_matches_oracle(name, prec):
    s, fl_ref, fs_ref, ref = system_and_reference(name)
    with Engine(s, precision=prec) as eng:
        fl, fs, e = eng.compute()
        st = eng.stats()
    tol = TOL[prec]
    assert rel(fl, fl_ref) <= tol, (name, prec, rel(fl, fl_ref))
    err_s = np.linalg.norm(fs - fs_ref) / max(np.linalg.norm(fs_ref), np.linalg.norm(fl_ref))
    assert err_s <= tol, (name, prec, err_s)
    scale = energy_scale(ref)
    for k in LONG_E + SHORT_E:
        assert abs(e[k] - ref[k]) <= tol * max(component_scale(ref, k), FLOOR[prec] * scale) + 1e-9, \
            (name, prec, k, e[k], ref[k])
    if name == "c2":
        # the pair count of the list pass against the oracle's count inside the cutoff
        from oracle.pyoracle import Oracle
        want = Oracle(s).count_pairs(max(s.rcutoff, s.rcutoffelec))
        assert abs(st["pairs_within_cutoff"] - want) <= 16, (st["pairs_within_cutoff"], want)


@pytest.mark.parametrize("name", ["c2", "c5"])
def test_full_size_list_bit_exact(name):
    """The device cluster-pair list of the whole system equals the CPU builder's, cluster by
    cluster and entry by entry (order and periodic image included)."""
    from oracle.pyoracle import nblist
    s = configs.water_c2() if name == "c2" else configs.butane_in_tube_bundle()[0]
    s.respa_split = 0.0
    s.sf_type = 0
    with Engine(s, precision="mixed") as eng:
        eng.compute(terms=TERMS_LONG)
        g = eng.debug_list()
    rlist = max(s.rcutoff, s.rcutoffelec)
    c = nblist(s.x, s.y, s.z, tuple(float(v) for v in s.box), rlist, g["grid"][0], g["grid"][1], g["grid"][2],
               g["zcap"])
    assert np.array_equal(g["clusters"], c["clusters"])
    assert np.array_equal(g["pairs"], c["pairs"])
    assert np.array_equal(g["shifts"], c["shifts"])
