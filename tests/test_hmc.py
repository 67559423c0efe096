"""Batched Hybrid Monte Carlo of Lennard-Jones replicas (mg_hmc_batch): the reference's
hmc() canonical move (src/hmc.c:23-40) with md_move over vver (src/dispmd.c:12-103,
src/md.c:22-85) for many boxes in one launch.

The random streams come from include/mg_philox.h (Philox4x32-10), checked against the
published known answers. The oracle restates one replica's moves (oracle/md_oracle.c:
velinit with the same streams, the restated frclong and vver, the reference's dH with
+dushift); the GPU batch is compared with it replica by replica: dH per move to
5e-4 + 1e-6 N (FP32 pair forces against FP64 over a 10-step trajectory), the same
accept/reject decisions and, when they agree, the final positions to 1e-5.
"""
import ctypes as C

import numpy as np
import pytest

from mspms2_gb300 import configs

HP = dict(eps=1.0, sigma=1.0, rcutoff=2.5, mass=1.0, treq=1.0, delt=0.005, nstep_md=10, seed=0x1234ABCD5678,
          rescale=1, nconstraint=0)
SIZES = [200, 337, 500, 864, 1500]  # all-pairs boxes (< 3 cells per axis) and cell-list boxes


def test_philox_known_answers():
    from oracle.pyoracle import lib
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in cases:
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        lib().orc_philox4x32_10(c, k, o)
        assert tuple(o) == want


def replicas(sizes, seed=40):
    return [configs.lj_replica(n, seed=seed + i) for i, n in enumerate(sizes)]


def test_oracle_hmc_conserves_energy_at_small_steps():
    """Steps so small that no pair crosses the cutoff: dH ~ 0 and every move accepted.
    (Each pair crossing the cutoff changes dH by twice its shift energy, about 0.016 at
    2.5 sigma: the reference adds the change of ushift to that of the truncated energy,
    src/dispmd.c:49-50.)"""
    from oracle.pyoracle import Oracle
    s = replicas([256])[0]
    hp = dict(HP, delt=1e-6)
    _, acc, _, dh = Oracle(s).hmc_replica(hp, 0, 0, 2)
    assert np.all(np.abs(dh) < 1e-6) and acc == 2


@pytest.mark.gpu
def test_gpu_batch_matches_oracle_per_replica():
    from mspms2_gb300 import build
    from mspms2_gb300.engine import hmc_batch
    from oracle.pyoracle import Oracle
    build.build()
    reps = replicas(SIZES)
    natom = [s.natom for s in reps]
    box = [float(s.box[0]) for s in reps]
    x = np.concatenate([s.x for s in reps])
    y = np.concatenate([s.y for s in reps])
    z = np.concatenate([s.z for s in reps])
    nmoves = 3
    gx, gy, gz, acc, energy, dh = hmc_batch(HP, natom, box, x, y, z, nmoves)
    off = 0
    for r, s in enumerate(reps):
        n = s.natom
        pos, oacc, oen, odh = Oracle(s).hmc_replica(HP, r, 0, nmoves)
        tol = 5e-4 + 1e-6 * n
        assert np.all(np.abs(dh[r] - odh) <= tol), (r, dh[r], odh)
        if acc[r] == oacc:
            gp = np.stack([gx[off:off + n], gy[off:off + n], gz[off:off + n]])
            assert np.abs(gp - pos).max() <= 1e-5 * max(1.0, np.abs(pos).max()), r
            assert abs(energy[r] - oen) <= 1e-5 * abs(oen) + 1e-3, (r, energy[r], oen)
        off += n
    assert acc.sum() > 0


@pytest.mark.gpu
def test_gpu_batch_is_reproducible_and_resumable():
    from mspms2_gb300 import build
    from mspms2_gb300.engine import hmc_batch
    build.build()
    reps = replicas([300, 700, 1200], seed=60)
    natom = [s.natom for s in reps]
    box = [float(s.box[0]) for s in reps]
    x, y, z = (np.concatenate([getattr(s, k) for s in reps]) for k in "xyz")
    a = hmc_batch(HP, natom, box, x, y, z, 4)
    b = hmc_batch(HP, natom, box, x, y, z, 4)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    h1 = hmc_batch(HP, natom, box, x, y, z, 2)
    h2 = hmc_batch(HP, natom, box, h1[0], h1[1], h1[2], 2, move0=2)
    assert np.array_equal(h2[0], a[0]) and np.array_equal(h2[1], a[1]) and np.array_equal(h2[2], a[2])
    assert np.array_equal(h1[3] + h2[3], a[3])


def ref_golden():
    """hmc_lj_ref (tests/golden/gen_golden.py): one canonical move of three LJ replicas through
    the compiled reference's own md_move() over vver() (src/dispmd.c:12-103, src/md.c:22-85),
    each started from the velocities mg_hmc_batch draws for move 0 of that replica."""
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "hmc_lj_ref.npz"))
    hp = dict(zip(("eps", "sigma", "rcutoff", "mass", "treq", "delt"), (float(v) for v in d["hp"])))
    hp.update(zip(("nstep_md", "seed", "rescale", "nconstraint"), (int(v) for v in d["hp_int"])))
    return d, hp


def test_oracle_move_matches_reference_md_move():
    """The oracle's restated move (velinit with the Philox streams, frclong, vver, dH with
    +d ushift) against the compiled reference's md_move from the same velocities: the
    velocities the golden file injected are those the streams give, and dH agrees to FP64
    rounding."""
    from oracle.pyoracle import Oracle, hmc_velocities
    d, hp = ref_golden()
    off = 0
    for r, n in enumerate(d["natom"]):
        n = int(n)
        assert np.array_equal(hmc_velocities(hp, r, 0, n), d["vel"][:, off:off + n])
        s = configs.lj_replica(n, seed=40 + r)
        assert np.array_equal(np.stack([s.x, s.y, s.z]), d["pos"][:, off:off + n])
        _, _, _, dh = Oracle(s).hmc_replica(hp, r, 0, 1)
        assert abs(dh[0] - d["dh"][r]) <= 1e-9 * max(1.0, abs(d["dh"][r])), (r, dh[0], d["dh"][r])
        off += n


@pytest.mark.gpu
def test_gpu_batch_matches_reference_md_move():
    """mg_hmc_batch, one move of the three replicas in one launch, against the compiled
    reference's md_move from the same velocities: dH to 5e-4 + 1e-6 N (FP32 pair forces over
    the 10-step trajectory against FP64); where the batch accepts, its positions are the
    reference's proposal to 1e-5 and its energy (potential plus shift) the proposal's; where
    it rejects (its own uniform draw), the positions are the start, unchanged."""
    from mspms2_gb300 import build
    from mspms2_gb300.engine import hmc_batch
    build.build()
    d, hp = ref_golden()
    natom = [int(v) for v in d["natom"]]
    gx, gy, gz, acc, energy, dh = hmc_batch(hp, natom, d["box"], d["pos"][0], d["pos"][1], d["pos"][2], 1)
    off = 0
    for r, n in enumerate(natom):
        assert abs(dh[r, 0] - d["dh"][r]) <= 5e-4 + 1e-6 * n, (r, dh[r, 0], d["dh"][r])
        gp = np.stack([gx[off:off + n], gy[off:off + n], gz[off:off + n]])
        if acc[r]:
            prop = d["prop"][:, off:off + n]
            assert np.abs(gp - prop).max() <= 1e-5 * max(1.0, np.abs(prop).max()), r
            want = d["prop_e"][r][1] + d["prop_e"][r][3]
            assert abs(energy[r] - want) <= 1e-5 * abs(want) + 1e-3, (r, energy[r], want)
        else:
            assert np.array_equal(gp, d["pos"][:, off:off + n]), r
        off += n
