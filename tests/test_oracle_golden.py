"""The CPU oracle (C restatement) against the compiled reference's golden vectors.

The restatement follows the reference expression by expression, so on the same
inputs it must reproduce the reference to rounding: forces and energies agree to
1e-12 relative (most cases are bit-identical).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases
from mspms2_gb300.capi import ENERGY_NAMES
from mspms2_gb300.system import derive_params, load_system
from oracle.pyoracle import Oracle

LONG = ENERGY_NAMES[:12]
SHORT = ENERGY_NAMES[12:]
DERIVED = ["rcutoffsq", "rcutonsq", "rcutoffelecsq", "roff2_minus_ron2_cube", "shift1", "shift4",
           "wolfvcon1", "wolfvcon2", "wolfvcon3", "wolffcon1", "wolffcon2", "bfactor_ewald",
           "vfactor_ewald", "twopi_lx", "twopi_ly", "twopi_lz", "twopi_over_3v", "kappa",
           "coulomb_prefactor"]


def _close(a, b, rtol=1e-12):
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) <= rtol * scale


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_matches_reference(case):
    s, d = load_system(os.path.join(GOLDEN, case + ".npz"))
    o = Oracle(s)
    fl, el, flags = o.frclong()
    fs, es, err = o.frcshort()
    assert flags == 0 and err == 0
    assert _close(fl, d["ref_fl"]), f"{case}: long forces differ"
    assert _close(fs, d["ref_fs"]), f"{case}: short forces differ"
    ref_e = dict(zip(ENERGY_NAMES, d["ref_energies"]))
    for k in LONG:
        assert el[k] == pytest.approx(ref_e[k], rel=1e-12, abs=1e-9), (case, k)
    for k in SHORT:
        assert es[k] == pytest.approx(ref_e[k], rel=1e-12, abs=1e-9), (case, k)


@pytest.mark.parametrize("case", golden_cases())
def test_derived_params_match_reference(case):
    s, d = load_system(os.path.join(GOLDEN, case + ".npz"))
    p = derive_params(s)
    ref = dict(zip(DERIVED, d["ref_derived"][:len(DERIVED)]))
    ref_box = d["ref_derived"][19:22]
    assert np.array_equal(ref_box, s.box)
    for k in DERIVED:
        if k in ("kappa",):
            want = s.kappa
        elif k == "coulomb_prefactor":
            want = s.coulomb_prefactor
        else:
            want = p[k]
        if (s.charge_type == 3 and k == "kappa") or (s.charge_type == 0 and k in ("kappa", "coulomb_prefactor")):
            continue  # the reference only sets these in init_charge (src/initvars.c:397-472)
        assert want == pytest.approx(ref[k], rel=1e-15, abs=0.0), (case, k)


def test_sampling_windows_partition_the_call():
    """The sampled windows the CPU baseline times in parallel cover the whole call: pair
    rows split at any point and k-vectors dealt round robin (k_offset) sum to the
    unwindowed forces and reciprocal energy. Every window with a huge k_stride still
    evaluates the first k-vector, which is taken out once per such window."""
    from oracle.pyoracle import OrcWindow
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    o = Oracle(s)
    M = s.nmole
    full, e_full, _ = o.frclong()
    k0 = o.frclong(window=OrcWindow(M, M + 1, 1 << 30, 1, 0))[0]
    intra = o.frclong(window=OrcWindow(M, M + 1, 1 << 30, 0, 0))[0] - k0
    pairs = sum(o.frclong(window=OrcWindow(a, b, 1 << 30, 1, 0))[0] - k0
                for a, b in ((0, 37), (37, 101), (101, M)))
    ks = [o.frclong(window=OrcWindow(M, M + 1, 3, 1, t)) for t in range(3)]
    kspace = sum(k[0] for k in ks)
    assert sum(k[1]["ufourier"] for k in ks) == pytest.approx(e_full["ufourier"], rel=1e-12)
    assert _close(pairs + kspace + intra, full, rtol=1e-11)


@pytest.mark.parametrize("case", ["water_ewald_512", "water_ewald_vacuum", "custom_wolf", "water_simple_coulomb",
                                  "sf_tasos", "butane_ewald_switch"])
def test_threaded_call_matches_serial(case):
    """orc_frclong_mt (pair rows and k-vectors over host threads, partial sums added in
    thread order) gives the serial call's forces and energies up to the order of the sums."""
    s, _ = load_system(os.path.join(GOLDEN, case + ".npz"))
    o = Oracle(s)
    f1, e1, fl1 = o.frclong()
    f5, e5, fl5 = o.frclong_mt(5)
    assert fl1 == fl5
    assert _close(f5, f1, rtol=1e-13)
    for k in LONG:
        assert e5[k] == pytest.approx(e1[k], rel=1e-11, abs=1e-9), (case, k)


def test_threaded_slices_partition_the_call():
    """Slices 0..n-1 of orc_frclong_mt together do the work of one call exactly once (the
    O(N) terms in slice 0): their forces and Fourier energies sum to the full call."""
    s, _ = load_system(os.path.join(GOLDEN, "water_ewald_512.npz"))
    o = Oracle(s)
    full, e_full, _ = o.frclong()
    parts = [o.frclong_mt(2, slice_=k, nslices=3) for k in range(3)]
    assert _close(sum(p[0] for p in parts), full, rtol=1e-11)
    assert sum(p[1]["ufourier"] for p in parts) == pytest.approx(e_full["ufourier"], rel=1e-12)
    assert sum(p[1]["uvdw"] for p in parts) == pytest.approx(e_full["uvdw"], rel=1e-12)
