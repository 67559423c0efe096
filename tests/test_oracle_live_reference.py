"""The CPU oracle against the compiled reference itself, on seeded random systems.

Where the reference's force layer has been compiled (oracle/_ref/mspms_ref_force, built
by oracle/build_ref.sh from a reference checkout), each case builds a random system of one
family (water, water with molecules wrapped across the faces, charged butane, ions, a
six-site molecule with ghosts, 1-4 pairs and every bonded form, the four solid-fluid
models, and water split into two species with their own parameters), with random electrostatics (none, Wolf, Ewald with tin-foil or vacuum
boundaries, plain Coulomb), LJ switch, 1-4 scale, cutoffs, k-vector set and a non-cubic
box. It writes the system in the reference's input format, runs the reference's
frclong()/frcshort(), and compares the oracle's forces and all 18 energies (1e-12
relative; the restatement follows the reference expression by expression, so nearly all
cases agree bit for bit). The fixtures under tests/golden/ pin the same oracle on fixed
systems where the compiled reference is absent.

Molecules with non-bonded pair lists (nbp) are the one input the reference cannot
evaluate: its template stores the pair indices as doubles (src/molevars.h:72) and reads
them with %d (src/readins.c:238-241), so every pair resolves to site 0 with itself and the
forces come out non-finite. One test records that; the oracle and the engine read the
indices as the integers they are.

The integrators get the same treatment: random starts of four families run for four steps
through the reference's own vver (NVE), vver_nh_3 (NVT RESPA) or npt_respa (NPT) from the
velocities its velinit drew, and the oracle's restatement (oracle/md_oracle.c) continues
from those velocities; every logged quantity, the displacement and the end velocities
match to 1e-12. So do canonical HMC moves (the reference's md_move from the oracle's
Philox velocities; dH to 1e-9) and the reference's solid-fluid grid tool on random cells
(against the restatement the grid tests use; 1e-10).
"""
import sys
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN
from mspms2_gb300.capi import ENERGY_NAMES
from oracle.pyoracle import Oracle, reference_available, run_reference_md, run_reference_system

sys.path.insert(0, GOLDEN)
from golden_systems import FAMILIES, MD_FAMILIES, random_md_variant, random_variant  # noqa: E402

pytestmark = pytest.mark.skipif(not reference_available(), reason="compiled reference (oracle/_ref) not built")

SEEDS = range(8 * len(FAMILIES))


@pytest.mark.parametrize("seed", SEEDS)
def test_oracle_equals_reference_on_random_system(seed):
    s = random_variant(seed)
    ref_fl, ref_fs, ref_e, _ = run_reference_system(s)[0]
    o = Oracle(s)
    fl, el, flags = o.frclong()
    fs, es, err = o.frcshort()
    assert flags == 0 and err == 0, s.name
    for got, want, what in ((fl, ref_fl, "long"), (fs, ref_fs, "short")):
        scale = max(float(np.abs(want).max()), 1e-300)
        assert np.abs(got - want).max() <= 1e-12 * scale, (s.name, what)
    mine = {**el, **es}
    for k in ENERGY_NAMES:
        assert mine[k] == pytest.approx(ref_e[k], rel=1e-12, abs=1e-9), (s.name, k)


def test_variants_reach_every_switch():
    """The seeds above reach every family, electrostatics type, both Ewald boundary
    conditions, both LJ forms, an Ewald axis without k-vectors and the whole cube."""
    seen = set()
    for seed in SEEDS:
        s = random_variant(seed)
        seen.add(("family", seed % len(FAMILIES)))
        seen.add(("elec", s.charge_type, s.ewald_bc if s.charge_type == 1 else 0))
        seen.add(("switch", s.lj_switch))
        if s.charge_type == 1 and 0 in s.kmax:
            seen.add("zero kmax")
        if s.charge_type == 1 and s.ksqmax > sum(k * k for k in s.kmax):
            seen.add("cube")
    assert {"zero kmax", "cube"} <= seen
    assert {("family", f) for f in range(len(FAMILIES))} <= seen
    assert {("elec", 0, 0), ("elec", 1, 1), ("elec", 1, 2), ("elec", 2, 0), ("elec", 3, 0)} <= seen
    assert {("switch", 0), ("switch", 1)} <= seen


def test_reference_nbp_pairs_resolve_to_site_zero():
    """With nbp pairs in the template, the compiled reference returns non-finite long-range
    forces at exactly the first site of every molecule (the pair (0, 0) at r = 0), while the
    oracle's forces are finite. Without the nbp pairs both agree (the test above)."""
    sys.path.insert(0, GOLDEN)
    from golden_systems import custom_molecule_system
    s = custom_molecule_system(40, with_nbp=True)
    ref_fl = run_reference_system(s)[0][0]
    nat, nmole = s.species[0].natom, s.species[0].nmole
    bad = np.nonzero(~np.isfinite(ref_fl).all(0))[0]
    assert np.array_equal(bad, np.arange(nmole) * nat)
    fl, _, flags = Oracle(s).frclong()
    assert flags == 0 and np.isfinite(fl).all()


MD_SEEDS = range(6 * len(MD_FAMILIES))


@pytest.mark.parametrize("seed", MD_SEEDS)
def test_oracle_integrators_equal_reference_on_random_start(seed):
    from mspms2_gb300.system import read_reference_dir, write_reference_dir
    s = random_md_variant(seed)
    nsteps = 4
    with tempfile.TemporaryDirectory() as td:
        write_reference_dir(s, td)
        p = read_reference_dir(td)
        r = run_reference_md(td, nsteps)
    p.x, p.y, p.z = (r["start"][k].copy() for k in range(3))
    start, v0 = r["start"][:3], r["start"][3:]
    o = Oracle(p)
    if r.get("npt"):
        pos, vel, _, _, log = o.npt_run(nsteps, r["md"], v0, np.array(p.box, dtype=float), r["state"])
    else:
        pos, vel, _, log = o.md_run(nsteps, r["md"], v0, r["state"])
    assert np.isfinite(r["log"]).all(), s.name
    for k in range(log.shape[1]):
        rows = slice(1, None) if (r.get("npt") and k == 9) else slice(None)  # pinst unset before step 1
        ref = r["log"][rows, k]
        assert np.abs(log[rows, k] - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-300), (s.name, k)
    disp = r["end"][:3] - start
    assert np.linalg.norm((pos - start) - disp) <= 1e-12 * np.linalg.norm(disp), s.name
    assert np.linalg.norm(vel - r["end"][3:]) <= 1e-12 * np.linalg.norm(r["end"][3:]), s.name


def test_md_variants_reach_every_ensemble():
    seen = {(random_md_variant(seed).what_ensemble, seed % len(MD_FAMILIES)) for seed in MD_SEEDS}
    assert {e for e, _ in seen} == {0, 1, 2}
    assert {f for _, f in seen} == set(range(len(MD_FAMILIES)))


HMC_SEEDS = range(8)


@pytest.mark.parametrize("seed", HMC_SEEDS)
def test_oracle_hmc_move_equals_reference_md_move(seed):
    """One canonical HMC move of a random Lennard-Jones replica (size, temperature, time step
    and trajectory length drawn per seed) through the reference's own md_move over vver
    (src/dispmd.c:12-103), started from the velocities the oracle's Philox streams give:
    the oracle's dH equals the reference's to 1e-9."""
    from mspms2_gb300 import configs
    from mspms2_gb300.system import time_base, write_reference_dir
    from oracle.pyoracle import hmc_velocities, run_reference_hmc
    rng = np.random.default_rng(500 + seed)
    hp = dict(eps=1.0, sigma=1.0, rcutoff=2.5, mass=1.0, treq=float(rng.uniform(0.8, 1.5)),
              delt=float(rng.uniform(0.002, 0.008)), nstep_md=int(rng.integers(5, 16)),
              seed=int(rng.integers(1, 2 ** 40)), rescale=1, nconstraint=0)
    n = int(rng.integers(150, 600))
    s = configs.lj_replica(n, seed=700 + seed)
    s.treq_K, s.delt_fs, s.nstep_inner = hp["treq"], hp["delt"] * time_base(s), 1
    s.what_simulation, s.what_ensemble = 1, 0
    v = hmc_velocities(hp, seed, 0, n)
    with tempfile.TemporaryDirectory() as td:
        write_reference_dir(s, td)
        mv = run_reference_hmc(td, [v], hp["nstep_md"])["moves"][0]
    _, _, _, dh = Oracle(s).hmc_replica(hp, seed, 0, 1)
    assert abs(dh[0] - mv["dh"]) <= 1e-9 * max(1.0, abs(mv["dh"])), (seed, n, dh[0], mv["dh"])


@pytest.mark.parametrize("seed", range(8))
def test_grid_restatement_equals_reference_tool_on_random_cell(seed):
    """The reference's tools/sfgridgen.c on a random solid cell (atoms, cell, fluid and
    solid LJ parameters, cutoff, energy switch and spacing drawn per seed) against the
    numpy restatement the solid-fluid grid tests check the engine with: energy, gradient and
    (without the switch, where the tool assigns them all) the second derivatives at 40
    random nodes, to 1e-10."""
    from oracle.pyoracle import run_reference_sfgridgen
    from test_sfgrid import RGAS, node_terms
    rng = np.random.default_rng(300 + seed)
    ucl = (float(rng.uniform(8, 14)), float(rng.uniform(8, 14)), float(rng.uniform(2.0, 4.0)))
    atoms = rng.uniform(0, 1, size=(int(rng.integers(8, 30)), 3)) * np.array(ucl)
    sw = int(rng.integers(2))
    roff = float(rng.uniform(8, 14))
    spec = dict(f_sigma=float(rng.uniform(3.0, 4.0)), f_epsilon=float(rng.uniform(40, 120)), s_sigma=3.4,
                s_epsilon=float(rng.uniform(20, 40)), rcuton=roff - float(rng.uniform(1, 3)) if sw else roff,
                rcutoff=roff, lj_switch=sw, ucl=ucl, atoms=atoms)
    itvl = float(rng.choice([0.5, 0.8, 1.0]))
    dims, out, _ = run_reference_sfgridgen(spec, itvl)
    nn = dims[0] * dims[1] * dims[2]
    for idx in rng.choice(nn, size=min(40, nn), replace=False):
        i, rem = divmod(int(idx), dims[1] * dims[2])
        j, k = divmod(rem, dims[2])
        E, G, H, _ = node_terms(spec, np.array([i, j, k], dtype=float) * itvl, RGAS)
        assert abs(E - out[0, idx]) <= 1e-10 * max(abs(out[0, idx]), 1.0), (seed, idx)
        assert np.abs(G - out[1:4, idx]).max() <= 1e-10 * max(np.abs(out[1:4, idx]).max(), 1.0), (seed, idx)
        if not sw:
            assert np.abs(-H.reshape(9) - out[4:13, idx]).max() <= 1e-10 * max(np.abs(out[4:13, idx]).max(), 1.0)
