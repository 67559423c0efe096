"""The CPU oracle against the compiled reference itself, on seeded random systems.

Where the reference's force layer has been compiled (oracle/_ref/mspms_ref_force, built
by oracle/build_ref.sh from a reference checkout), each case builds a random system of one
family (water, water with molecules wrapped across the faces, charged butane, ions, a
six-site molecule with ghosts, 1-4 pairs and every bonded form, and the four solid-fluid
models), with random electrostatics (none, Wolf, Ewald with tin-foil or vacuum
boundaries, plain Coulomb), LJ switch, 1-4 scale, cutoffs, k-vector set and a non-cubic
box. It writes the system in the reference's input format, runs the reference's
frclong()/frcshort(), and compares the oracle's forces and all 18 energies (1e-12
relative; the restatement follows the reference expression by expression, so nearly all
cases agree bit for bit). The fixtures under tests/golden/ pin the same oracle on fixed
systems where the compiled reference is absent.

Molecules with non-bonded pair lists (nbp) are the one input the reference cannot
evaluate: its template stores the pair indices as doubles (src/molevars.h:72) and reads
them with %d (src/readins.c:238-241), so every pair resolves to site 0 with itself and the
forces come out non-finite. The last test records that; the oracle and the engine read the
indices as the integers they are.
"""
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from mspms2_gb300.capi import ENERGY_NAMES
from oracle.pyoracle import Oracle, reference_available, run_reference_system

sys.path.insert(0, GOLDEN)
from golden_systems import FAMILIES, random_variant  # noqa: E402

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
    conditions and both LJ forms."""
    seen = set()
    for seed in SEEDS:
        s = random_variant(seed)
        seen.add(("family", seed % len(FAMILIES)))
        seen.add(("elec", s.charge_type, s.ewald_bc if s.charge_type == 1 else 0))
        seen.add(("switch", s.lj_switch))
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
