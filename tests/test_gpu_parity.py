"""GPU parity: the engine, called through its C ABI, against the compiled reference's
golden vectors and the CPU oracle.

Tolerances (norm-wise relative error of each force block, relative error of each
energy): FP64 path 1e-10; mixed path (FP32 pair arithmetic, FP64 accumulation) 1e-5,
the force tolerance the benchmark contract states.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases
from mspms2_gb300 import build
from mspms2_gb300.capi import ENERGY_NAMES
from mspms2_gb300.engine import TERMS_ALL, TERMS_LONG, TERMS_SHORT, Engine
from mspms2_gb300.system import load_system

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-5}
LONG_E = ["uvdw", "ushift", "ureal", "uexcl", "ufourier", "uself", "uvacuum", "uelec", "usflj", "uinter",
          "virial_inter"]
SHORT_E = ["ubond", "uangle", "udih", "uimp", "uintra", "virial_intra"]


@pytest.fixture(scope="session", autouse=True)
def built():
    build.build()


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def energy_scale(ref):
    return max(abs(v) for v in ref.values())


def component_scale(ref, k):
    """Magnitude of the terms a derived energy is formed from: uelec, uinter and
    virial_inter are small differences of large components (ureal, uexcl, uself ...), so
    their error is judged against those components."""
    elec = abs(ref["ureal"]) + abs(ref["ufourier"]) + abs(ref["uself"]) + abs(ref["uexcl"]) + abs(ref["uvacuum"])
    elec = max(elec, abs(ref["uelec"]))
    if k == "uelec":
        return elec
    if k in ("uinter", "virial_inter"):
        return elec + abs(ref["uvdw"]) + abs(ref["usflj"]) + (abs(ref["virial_inter"]) if k == "virial_inter" else 0)
    return abs(ref[k])


# Floor of the energy tolerance, as a fraction of the largest energy of the system: an
# energy that is a near-zero sum of much larger terms (a torsion at its minimum, a bond
# virial at rest) carries the FP32 rounding of those terms in the mixed path.
FLOOR = {"fp64": 1e-6, "mixed": 1e-3}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("case", golden_cases())
def test_engine_matches_reference(case, prec):
    s, d = load_system(os.path.join(GOLDEN, case + ".npz"))
    ref = dict(zip(ENERGY_NAMES, d["ref_energies"]))
    with Engine(s, precision=prec) as eng:
        fl, fs, e = eng.compute()
    tol = TOL[prec]
    assert rel(fl, d["ref_fl"]) <= tol, (case, prec, rel(fl, d["ref_fl"]))
    assert rel(fs, d["ref_fs"]) <= tol, (case, prec, rel(fs, d["ref_fs"]))
    scale = energy_scale(ref)
    for k in LONG_E + SHORT_E:
        # each energy to tol relative to the terms it is made of (floor: 1e-6 of the
        # largest energy of the system)
        assert abs(e[k] - ref[k]) <= tol * max(component_scale(ref, k), FLOOR[prec] * scale) + 1e-9, \
            (case, prec, k, e[k], ref[k])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_deterministic(prec):
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    with Engine(s, precision=prec) as eng:
        a = eng.compute()
        b = eng.compute()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2] == b[2]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_respa_split_sums_to_full(prec):
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    with Engine(s, precision=prec) as full:
        fl, fs, e = full.compute()
    s.respa_split = 6.0
    with Engine(s, precision=prec) as sp:
        fl_o, _, e_o = sp.compute(terms=TERMS_LONG)
        _, fs_i, e_i = sp.compute(terms=TERMS_SHORT)
        fl_a, fs_a, e_a = sp.compute(terms=TERMS_ALL)
    tol = TOL[prec]
    assert rel(fl_o + fs_i, fl + fs) <= tol
    assert rel(fl_a + fs_a, fl + fs) <= tol
    for k in ("uvdw", "ureal", "uelec", "uinter", "virial_inter", "uintra"):
        assert abs(e_o[k] + e_i[k] - (e[k] + (0 if k != "uinter" else 0))) <= tol * max(1.0, abs(e[k])) * 10, k
        assert abs(e_a[k] - e[k]) <= tol * max(1.0, abs(e[k])) * 10, k


def test_skin_reuse_matches_rebuild():
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    rng = np.random.default_rng(5)
    x1, y1, z1 = (v + rng.uniform(-0.2, 0.2, size=v.shape) for v in (s.x, s.y, s.z))
    with Engine(s, precision="fp64", skin=1.0) as a, Engine(s, precision="fp64") as b:
        a.compute()
        assert a.stats()["list_rebuilt"] == 1
        fa = a.compute(x1, y1, z1)
        assert a.stats()["list_rebuilt"] == 0
        fb = b.compute(x1, y1, z1)
    assert rel(fa[0], fb[0]) <= 1e-12 and rel(fa[1], fb[1]) <= 1e-12


@pytest.mark.parametrize("case", ["water_ewald_512", "lj_fluid_500", "water_wolf_216"])
def test_neighbour_list_bit_exact(case):
    from oracle.pyoracle import nblist
    s, _ = load_system(os.path.join(GOLDEN, case + ".npz"))
    with Engine(s, precision="mixed") as eng:
        eng.compute(terms=TERMS_LONG)
        g = eng.debug_list()
    rlist = max(s.rcutoff, s.rcutoffelec)
    c = nblist(s.x, s.y, s.z, tuple(float(v) for v in s.box), rlist, g["grid"][0], g["grid"][1], g["grid"][2],
               g["zcap"])
    assert np.array_equal(g["clusters"], c["clusters"])
    assert np.array_equal(g["pairs"], c["pairs"])
    assert np.array_equal(g["shifts"], c["shifts"])


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("nside,rc", [(10, 1.5), (10, 4.0), (16, 4.0)])
def test_sparse_ions_match_oracle(prec, nside, rc):
    """One site per molecule: the first build asks for more clusters than the first
    capacity estimate holds, so the call is repeated with larger buffers. Repeated in
    one process, the later cases reuse device memory the earlier ones wrote."""
    from mspms2_gb300.configs import ion_box
    from oracle.pyoracle import Oracle
    s = ion_box(nside, seed=nside, kmax=8, ksqmax=64, rc=rc)
    f_ref, e_ref, _ = Oracle(s).frclong()
    with Engine(s, precision=prec) as eng:
        for _ in range(2):
            fl, _, e = eng.compute(terms=TERMS_LONG)
            assert rel(fl, f_ref) <= TOL[prec], rel(fl, f_ref)
            for k in ("ureal", "ufourier", "uself", "uelec"):
                assert abs(e[k] - e_ref[k]) <= TOL[prec] * component_scale(e_ref, k) + 1e-9, (k, e[k], e_ref[k])


def test_pair_count_matches_oracle():
    from oracle.pyoracle import Oracle
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    with Engine(s, precision="fp64") as eng:
        eng.compute(terms=TERMS_LONG)
        npair = eng.stats()["pairs_within_cutoff"]
    want = Oracle(s).count_pairs(max(s.rcutoff, s.rcutoffelec))
    assert abs(npair - want) <= 2


@pytest.mark.parametrize("geometry", [(0.8, 1.5, 2), (1.25, 0.75, 8)])
def test_tuned_geometry_keeps_parity(geometry):
    """Any launch geometry the autotuner may pick (cell size, cluster size, threads per
    site of the k-space force pass) keeps the list bit-exact against the CPU builder on that
    grid and the forces within the parity tolerances."""
    from oracle.pyoracle import nblist
    cell, zcap, fg = geometry
    s, d = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    for prec in ("mixed", "fp64"):
        with Engine(s, precision=prec) as eng:
            eng.set_tuning(cell, zcap, fg)
            fl, fs, e = eng.compute()
            g = eng.debug_list()
            assert eng.tuning()["kforce_threads"] == fg
        assert rel(fl, d["ref_fl"]) <= TOL[prec], (prec, rel(fl, d["ref_fl"]))
        assert rel(fs, d["ref_fs"]) <= TOL[prec]
    rlist = max(s.rcutoff, s.rcutoffelec)
    c = nblist(s.x, s.y, s.z, tuple(float(v) for v in s.box), rlist, g["grid"][0], g["grid"][1], g["grid"][2],
               g["zcap"])
    assert np.array_equal(g["clusters"], c["clusters"])
    assert np.array_equal(g["pairs"], c["pairs"])
    assert np.array_equal(g["shifts"], c["shifts"])


def test_autotune_picks_a_valid_faster_geometry():
    s, d = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    with Engine(s, precision="mixed") as eng:
        t = eng.autotune()
        assert t["kforce_threads"] in (2, 4, 8) and 0.5 <= t["cell_scale"] <= 2 and 0.5 <= t["zcap_scale"] <= 2
        # the FP32 table k-force pass has no threads-per-site choice: the 9 list geometries
        assert t["configs_tried"] == 9 and 0 < t["ms_tuned"] <= t["ms_default"]
        fl, fs, e = eng.compute()
        assert rel(fl, d["ref_fl"]) <= TOL["mixed"]
        from mspms2_gb300.engine import EngineError
        with pytest.raises(EngineError):
            eng.set_tuning(3.0, 1.0, 4)


def test_inner_sublist_under_skin_reuse():
    """The inner pass of the distance split walks a sub-list (cluster pairs within
    respa_split + skin at the build). After sites move by less than skin/2 the reused
    sub-list must still hold every inner pair: the short forces equal those of a fresh
    build at the new positions."""
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    s.respa_split = 6.0
    rng = np.random.default_rng(8)
    x1, y1, z1 = (v + rng.uniform(-0.28, 0.28, size=v.shape) for v in (s.x, s.y, s.z))
    with Engine(s, precision="fp64", skin=1.0) as a, Engine(s, precision="fp64") as b:
        a.compute(terms=TERMS_SHORT)
        _, fs_a, e_a = a.compute(x1, y1, z1, terms=TERMS_SHORT)
        assert a.stats()["list_rebuilt"] == 0
        _, fs_b, e_b = b.compute(x1, y1, z1, terms=TERMS_SHORT)
    assert rel(fs_a, fs_b) <= 1e-12, rel(fs_a, fs_b)
    assert abs(e_a["uinter"] - e_b["uinter"]) <= 1e-10 * abs(e_b["uinter"])


def test_long_kz_rows_take_the_horner_pass():
    """Rows of more than 64 |kz| values do not fit the FP32 table force pass's on-chip
    staging; their forces come from the packed Horner pass, which must agree with the FP64
    path like the table pass does (KMAXZ 70 against KMAX 3 in x and y)."""
    from mspms2_gb300 import configs
    from mspms2_gb300.system import ELEC_EWALD
    s = configs.water_box(4, 12.4, 11, ELEC_EWALD, 0.3, 6.0, kmax=3, ksqmax=4900)
    s.kmax = (3, 3, 70)
    out = {}
    for prec in ("fp64", "mixed"):
        with Engine(s, precision=prec) as eng:
            out[prec] = eng.compute(terms=TERMS_LONG)
    assert rel(out["mixed"][0], out["fp64"][0]) <= TOL["mixed"], rel(out["mixed"][0], out["fp64"][0])
    assert abs(out["mixed"][2]["ufourier"] - out["fp64"][2]["ufourier"]) <= 1e-5 * abs(out["fp64"][2]["ufourier"])


@pytest.mark.parametrize("case", ["water_ewald_512", "butane_ewald_switch"])
def test_kspace_overlap_is_bit_identical(case):
    """The reciprocal-space chain on its own stream (default) gives the same bits as the
    chain in line on the context's stream: forces, energies and the per-call statistics."""
    s, _ = load_system(os.path.join(GOLDEN, case + ".npz"))
    out = {}
    for overlap in (True, False):
        with Engine(s, precision="mixed") as eng:
            eng.set_kspace_overlap(overlap)
            out[overlap] = [eng.compute() for _ in range(2)]
    for a, b in zip(out[True], out[False]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert a[2] == b[2]


@pytest.mark.gpu
@pytest.mark.parametrize("kmax,ksqmax", [((12, 12, 12), 144), ((9, 7, 30), 400)])
def test_sk_tensor_pass_matches_cuda_core_pass(kmax, ksqmax):
    """Structure factors and k-space forces on the tensor cores (TF32 3-term split MMAs, FP32
    accumulation in tensor memory) against the CUDA-core FP32 passes and the FP64 path.
    11^3 waters = 3993 sites: four S(k) site blocks, the last one ragged within a 32-site
    chunk, and 32 force tiles of 128 sites, the last one ragged; 12^3 rows of KSQMAX 144 give
    S(k) tiles with kzmax above and below 16 (both MMA widths) and force row tiles with one
    and two K atoms; KMAXZ 30 is the largest the passes take."""
    from mspms2_gb300 import configs
    from mspms2_gb300.system import ELEC_EWALD
    s = configs.water_box(11, 34.0, 5, ELEC_EWALD, 0.3, 9.0, kmax=kmax[0], ksqmax=ksqmax)
    s.kmax = kmax
    out = {}
    for key, prec, tensor in (("tc", "mixed", True), ("cc", "mixed", False), ("fp64", "fp64", True)):
        with Engine(s, precision=prec) as eng:
            eng.set_kspace_tensor(tensor)
            out[key] = eng.compute(terms=TERMS_LONG)
    f64, e64 = out["fp64"][0], out["fp64"][2]
    for key in ("tc", "cc"):
        assert rel(out[key][0], f64) <= TOL["mixed"], (key, rel(out[key][0], f64))
        assert abs(out[key][2]["ufourier"] - e64["ufourier"]) <= 2e-6 * abs(e64["ufourier"]), key
    # the two FP32 passes differ by rounding only
    assert rel(out["tc"][0], out["cc"][0]) <= 2e-6, rel(out["tc"][0], out["cc"][0])


def test_sk_wait_give_up_fails_the_call_and_recovers():
    """With the pipeline-wait bound at 0 polls every CTA of the tensor-core S(k) pass gives
    up at its first wait: it stops issuing, waits (with the default bound) for the MMAs it
    issued, frees its tensor memory and returns. The call then fails with MG_ERR_CUDA; with
    the bound restored, the next call on the same context gives the same bits as before."""
    from mspms2_gb300.engine import EngineError, set_wait_limit
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    with Engine(s, precision="mixed") as eng:
        before = eng.compute()
        try:
            set_wait_limit(0)
            with pytest.raises(EngineError) as ei:
                eng.compute()
            assert ei.value.status == 2 and "wait ran out" in str(ei.value)
        finally:
            set_wait_limit(-1)
        after = eng.compute()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert before[2] == after[2]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("elec", ["wolf", "ewald"])
@pytest.mark.parametrize("nbp_index_quirk", [True, False])
def test_nbp_pairs_match_oracle(prec, elec, nbp_index_quirk):
    """Molecules with a non-bonded pair list (nbp, src/frclong.c:791-977): the engine
    against the oracle, with the reference's nbp_idx[ndih] index (MG_COMPAT_NBP_INDEX) and
    with the loop's own index. The compiled reference gives no finite output to compare
    here (its nbp indices are doubles read with %d), so the oracle is the check."""
    import sys
    from oracle.pyoracle import Oracle
    from mspms2_gb300.system import ELEC_EWALD
    sys.path.insert(0, GOLDEN)
    from golden_systems import custom_molecule_system
    s = custom_molecule_system(41, with_nbp=True)
    if elec == "ewald":
        s.charge_type, s.kappa, s.kmax, s.ksqmax = ELEC_EWALD, 0.3, (4, 4, 4), 24
    if not nbp_index_quirk:
        s.compat &= ~1
    o = Oracle(s)
    f_ref, e_ref, _ = o.frclong()
    with Engine(s, precision=prec) as eng:
        fl, _, e = eng.compute(terms=TERMS_LONG)
    assert rel(fl, f_ref) <= TOL[prec], rel(fl, f_ref)
    scale = energy_scale(e_ref)
    for k in LONG_E:
        assert abs(e[k] - e_ref[k]) <= TOL[prec] * max(component_scale(e_ref, k), FLOOR[prec] * scale) + 1e-9, \
            (k, e[k], e_ref[k])
