"""Seeded synthetic systems with the shapes of the benchmark workloads.

No dataset is involved: every system is generated from a seed. Units: sigma_base = 1 A,
epsilon_base = 1 K, mass_base = 1e-27 kg, so the reduced units are A and K and the
reference-format files written by system.write_reference_dir round-trip exactly.

  water_box      flexible SPC water: O-O LJ eps 0.1553 kcal/mol, sigma 3.166 A, q(O)=-0.82,
                 q(H)=+0.41, harmonic O-H (r0 1.0 A, k 1059 kcal/mol/A^2), harmonic HOH
                 (109.47 deg, 75.9 kcal/mol/rad^2), U = k/2 (x-x0)^2 as src/bndfrc.c:143-145
                 and src/aglfrc.c:82-86 define it. Jittered cubic lattice (+-0.1 A) with
                 uniform random (Haar) orientations.
  water_c1       216 molecules, box 18.6 A, Wolf alpha 0.2/A, Rc 9 A.
  water_c2       32,768 molecules, box 99.3 A, Ewald alpha 0.3/A, Rc 10 A, kmax 24,
                 ksqmax 576 (spherical cut), RESPA split 7 A.
  water_c4       4,096 molecules, box 49.66 A, Ewald alpha 0.3/A, Rc 10 A, kmax 12,
                 ksqmax 144 (same reciprocal resolution as water_c2).
  lj_replica     LJ fluid, rho* 0.8, rc 2.5 sigma, jittered FCC (batched-HMC replicas).
  butane_box     united-atom n-butane (CH3 98 K/3.75 A, CH2 46 K/3.95 A), 1.54 A bonds,
                 114 deg angle, OPLS torsion with the reference's own constants
                 (cfg.mspms:18 of the reference checkout).
"""
from __future__ import annotations

import math

import numpy as np

from .system import (AVOGADRO, ELEC_EWALD, ELEC_NONE, ELEC_WOLF, GHOST_LJ, GHOST_NONE,
                     KCALMOL_TO_K, Species, System)


def _reduced_mass(kg_per_mol: float) -> float:
    return (kg_per_mol / AVOGADRO) / 1.0e-27


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from Haar-distributed unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def water_species(nmole: int) -> Species:
    theta0 = 109.47 * math.pi / 180.0
    tmpl = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [math.cos(theta0), math.sin(theta0), 0.0]])
    aw_in = np.array([0.0159994, 0.0010079, 0.0010079])
    sp = Species(
        name="water", nmole=nmole, atom_names=["O", "H", "H"],
        atom_type=np.array([0, 1, 1], np.int32), ghost=np.array([GHOST_NONE, GHOST_LJ, GHOST_LJ], np.int32),
        interp=np.array([1, 2, 2], np.int32),
        epsilon=np.array([0.1553 * KCALMOL_TO_K, 0.0, 0.0]), sigma=np.array([3.166, 0.0, 0.0]),
        charge=np.array([-0.82, 0.41, 0.41]), aw=np.array([_reduced_mass(v) for v in aw_in]),
        aw_input=aw_in, template_xyz=tmpl)
    sp.bond_idx = np.array([[0, 1], [0, 2]], np.int32)
    sp.bond_type = np.array([1, 1], np.int32)
    kb = 1059.0 * KCALMOL_TO_K
    sp.bond_param = np.array([[kb, 1.0, 0.0], [kb, 1.0, 0.0]])
    sp.angle_idx = np.array([[1, 0, 2]], np.int32)
    sp.angle_type = np.array([1], np.int32)
    sp.angle_param = np.array([[75.9 * KCALMOL_TO_K, theta0, 0.0, 0.0, 0.0]])
    return sp


def water_box(nside: int, box: float, seed: int, charge_type: int, kappa: float, rc: float,
              kmax: int = 0, ksqmax: int = 0, jitter: float = 0.1, name: str = "water",
              site_jitter: float = 0.0) -> System:
    rng = np.random.default_rng(seed)
    n = nside ** 3
    sp = water_species(n)
    a = box / nside
    g = np.arange(nside)
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    centres = (np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1) + 0.5) * a
    centres += rng.uniform(-jitter, jitter, size=centres.shape)
    rot = _random_rotations(rng, n)
    sites = centres[:, None, :] + np.einsum("mij,aj->mai", rot, sp.template_xyz)
    xyz = sites.reshape(-1, 3)
    if site_jitter > 0:  # distort the rigid template so bonded terms are not at rest
        xyz = xyz + rng.uniform(-site_jitter, site_jitter, size=xyz.shape)
    s = System(species=[sp], box=np.array([box, box, box]), x=xyz[:, 0].copy(), y=xyz[:, 1].copy(),
               z=xyz[:, 2].copy(), rcuton=rc, rcutoff=rc, rcutoffelec=rc, charge_type=charge_type,
               kappa=kappa, kmax=(kmax, kmax, kmax), ksqmax=ksqmax, name=name, delt_fs=0.5)
    return s


def water_c1(seed: int = 2024) -> System:
    return water_box(6, 18.6, seed, ELEC_WOLF, 0.2, 9.0, name="water_c1")


def water_c2(seed: int = 2024) -> System:
    s = water_box(32, 99.3, seed, ELEC_EWALD, 0.3, 10.0, kmax=24, ksqmax=576, name="water_c2")
    s.respa_split = 7.0
    s.nstep_inner = 4
    return s


def water_c4(seed: int = 2024) -> System:
    return water_box(16, 49.66, seed, ELEC_EWALD, 0.3, 10.0, kmax=12, ksqmax=144, name="water_c4")


def water_small(nside: int, box: float, seed: int, charge_type: int = ELEC_EWALD, kappa: float = 0.3,
                rc: float | None = None, kmax: int = 5, ksqmax: int = 27,
                site_jitter: float = 0.04) -> System:
    """Small water boxes for oracle-sized parity tests (templates distorted by
    +-site_jitter A so the bonded terms are exercised)."""
    rc = rc if rc is not None else min(9.0, 0.5 * box - 1e-9)
    return water_box(nside, box, seed, charge_type, kappa, rc, kmax=kmax, ksqmax=ksqmax,
                     name=f"water{nside}", site_jitter=site_jitter)


def lj_species(nmole: int) -> Species:
    return Species(name="lj", nmole=nmole, atom_names=["A"], atom_type=np.array([0], np.int32),
                   ghost=np.array([GHOST_NONE], np.int32), interp=np.array([1], np.int32),
                   epsilon=np.array([1.0]), sigma=np.array([1.0]), charge=np.array([0.0]),
                   aw=np.array([1.0]), aw_input=np.array([AVOGADRO * 1.0e-27]),
                   template_xyz=np.zeros((1, 3)))


def lj_replica(n: int, seed: int, rho: float = 0.8, rc: float = 2.5, jitter: float = 0.05) -> System:
    """One LJ-fluid replica: n atoms on a jittered FCC lattice at reduced density rho."""
    rng = np.random.default_rng(seed)
    box = (n / rho) ** (1.0 / 3.0)
    m = int(math.ceil((n / 4.0) ** (1.0 / 3.0)))
    a = box / m
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.arange(m)
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    cells = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1)
    pts = ((cells[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25) * a
    pts = pts[rng.permutation(len(pts))[:n]]
    pts = pts + rng.uniform(-jitter, jitter, size=pts.shape)
    return System(species=[lj_species(n)], box=np.array([box, box, box]), x=pts[:, 0].copy(),
                  y=pts[:, 1].copy(), z=pts[:, 2].copy(), rcuton=rc, rcutoff=rc, rcutoffelec=rc,
                  charge_type=ELEC_NONE, name=f"lj{n}")


def butane_species(nmole: int, charged: bool = False) -> Species:
    """United-atom n-butane, CH3-CH2-CH2-CH3."""
    th = 114.0 * math.pi / 180.0
    b = 1.54
    p0 = np.array([0.0, 0.0, 0.0])
    p1 = np.array([b, 0.0, 0.0])
    p2 = p1 + b * np.array([-math.cos(th), math.sin(th), 0.0])
    p3 = p2 + b * np.array([1.0, 0.0, 0.0])
    tmpl = np.array([p0, p1, p2, p3])
    q = np.array([-0.1, 0.1, -0.1, 0.1]) if charged else np.zeros(4)
    aw_in = np.array([0.015035, 0.014027, 0.014027, 0.015035])
    sp = Species(name="butane", nmole=nmole, atom_names=["CH3", "CH2", "CH2", "CH3"],
                 atom_type=np.array([0, 1, 1, 0], np.int32), ghost=np.zeros(4, np.int32),
                 interp=np.array([1, 2, 2, 1], np.int32), epsilon=np.array([98.0, 46.0, 46.0, 98.0]),
                 sigma=np.array([3.75, 3.95, 3.95, 3.75]), charge=q,
                 aw=np.array([_reduced_mass(v) for v in aw_in]), aw_input=aw_in, template_xyz=tmpl)
    sp.bond_idx = np.array([[0, 1], [1, 2], [2, 3]], np.int32)
    sp.bond_type = np.ones(3, np.int32)
    sp.bond_param = np.array([[130924.4893, b, 0.0]] * 3)
    sp.angle_idx = np.array([[0, 1, 2], [1, 2, 3]], np.int32)
    sp.angle_type = np.ones(2, np.int32)
    sp.angle_param = np.array([[62500.0, th, 0.0, 0.0, 0.0]] * 2)
    sp.dih_idx = np.array([[0, 1, 2, 3]], np.int32)
    sp.dih_type = np.array([1], np.int32)
    sp.dih_param = np.array([[0.0, 710.06, -136.38, 1582.64]])
    return sp


def butane_box(nside: int, box, seed: int, rc: float = 14.0, charged: bool = False,
               jitter: float = 0.05, name: str = "butane", site_jitter: float = 0.0) -> System:
    """Butane on a jittered cubic lattice of molecule centres, random orientations."""
    rng = np.random.default_rng(seed)
    box = np.broadcast_to(np.asarray(box, dtype=float), (3,)).copy()
    n = nside ** 3
    sp = butane_species(n, charged)
    a = box / nside
    g = np.arange(nside)
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    centres = (np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1) + 0.5) * a
    centres += rng.uniform(-jitter, jitter, size=centres.shape)
    rot = _random_rotations(rng, n)
    tm = sp.template_xyz - sp.template_xyz.mean(0)
    xyz = (centres[:, None, :] + np.einsum("mij,aj->mai", rot, tm)).reshape(-1, 3)
    if site_jitter > 0:
        xyz = xyz + rng.uniform(-site_jitter, site_jitter, size=xyz.shape)
    return System(species=[sp], box=box, x=xyz[:, 0].copy(), y=xyz[:, 1].copy(), z=xyz[:, 2].copy(),
                  rcuton=rc, rcutoff=rc, rcutoffelec=rc, f0=0.5, name=name, delt_fs=2.0,
                  charge_type=ELEC_NONE)


def ion_species(name: str, nmole: int, charge: float, epsilon: float = 0.0, sigma: float = 1.0) -> Species:
    """A single-site charged species (one ion per molecule)."""
    return Species(name=name, nmole=nmole, atom_names=[name], atom_type=np.array([0], np.int32),
                   ghost=np.array([GHOST_NONE], np.int32), interp=np.array([1], np.int32),
                   epsilon=np.array([epsilon]), sigma=np.array([sigma]), charge=np.array([charge]),
                   aw=np.array([1.0]), aw_input=np.array([AVOGADRO * 1.0e-27]), template_xyz=np.zeros((1, 3)))


def ion_box(nside: int, seed: int, kmax: int, ksqmax: int, rc: float = 1.5, spacing: float = 3.0,
            jitter: float = 0.4, kappa: float = 0.3) -> System:
    """nside^3 monovalent ions (half +1, half -1) on a jittered cubic lattice with Ewald
    electrostatics: one site per molecule, so the cluster count equals the site count,
    well above the list builder's first capacity estimate."""
    rng = np.random.default_rng(seed)
    g = np.arange(nside)
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    pts = (np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1) + 0.5) * spacing
    pts = pts[rng.permutation(len(pts))] + rng.uniform(-jitter, jitter, size=pts.shape)
    n = len(pts)
    species = [ion_species("Na", n // 2, 1.0), ion_species("Cl", n - n // 2, -1.0)]
    box = nside * spacing
    return System(species=species, box=np.array([box, box, box]), x=pts[:, 0].copy(), y=pts[:, 1].copy(),
                  z=pts[:, 2].copy(), rcuton=rc, rcutoff=rc, rcutoffelec=rc, charge_type=ELEC_EWALD,
                  kappa=kappa, kmax=(kmax, kmax, kmax), ksqmax=ksqmax, name=f"ions{n}")


def armchair_tube(n: int, cx: float, cy: float, acc: float = 1.42):
    """One axial period of an (n, n) armchair carbon nanotube centred at (cx, cy): 4n atoms
    on a cylinder of radius 3 n acc / (2 pi); the period along z is sqrt(3) acc. Returns
    (atoms [4n, 3], radius, period)."""
    circ = 3.0 * acc * n
    radius = circ / (2.0 * math.pi)
    period = math.sqrt(3.0) * acc
    pts = []
    for k in range(n):
        x0 = 3.0 * acc * k
        for dx, z in ((0.0, 0.0), (acc, 0.0), (1.5 * acc, period / 2), (2.5 * acc, period / 2)):
            th = 2.0 * math.pi * (x0 + dx) / circ
            pts.append((cx + radius * math.cos(th), cy + radius * math.sin(th), z))
    return np.array(pts), radius, period


def butane_in_tube_bundle(seed: int = 2024, nmole: int = 20000, cell_xy: float = 127.0, box_z: float = 200.0,
                          wall: float = 3.2, edge: float = 3.0, rc: float = 14.0):
    """United-atom n-butane around and inside a hexagonal bundle of 7 rigid (11,11) carbon
    nanotubes (diameter 14.9 A, 3.4 A wall-to-wall gaps), the bundle centred in a cell of
    cell_xy x cell_xy A; the fluid box is cell_xy x cell_xy x box_z. Molecules stand along
    the tube axis on a 4.2 x 4.2 x 6.45 A lattice, each turned about the axis by a seeded
    random angle and flipped or not (closest contact between molecules 2.7 A); molecules
    with a site within `wall` of a tube wall or within `edge` of the cell's x/y faces are
    left out, and nmole of the rest (seeded choice) are kept. Returns (system, tubes) with
    tubes = dict(atoms [n, 3] of one z period, period, radius, centres); the solid-fluid
    tables (Tasos model, types 1 = CH3, 2 = CH2) are made from them on the device."""
    rng = np.random.default_rng(seed)
    tube, radius, period = armchair_tube(11, 0.0, 0.0)
    spacing = 2.0 * radius + 3.4
    c0 = cell_xy / 2.0
    centres = [(c0, c0)] + [(c0 + spacing * math.cos(k * math.pi / 3), c0 + spacing * math.sin(k * math.pi / 3))
                            for k in range(6)]
    atoms = np.concatenate([tube + np.array([cx, cy, 0.0]) for cx, cy in centres])
    nxy, nz = int(cell_xy // 4.2), int(box_z // 6.45)
    g = np.stack(np.meshgrid(np.arange(nxy), np.arange(nxy), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    cen = (g + 0.5) * np.array([cell_xy / nxy, cell_xy / nxy, box_z / nz])
    tm = butane_species(1).template_xyz
    tm = tm - tm.mean(0)
    base = np.stack([tm[:, 1], tm[:, 2], tm[:, 0]], 1)  # long axis along z, zig-zag along x
    phi = rng.uniform(0.0, 2.0 * math.pi, len(cen))
    flip = rng.choice([-1.0, 1.0], len(cen))
    c, s_ = np.cos(phi)[:, None], np.sin(phi)[:, None]
    sites = cen[:, None, :] + np.stack([base[None, :, 0] * c - base[None, :, 1] * s_,
                                        base[None, :, 0] * s_ + base[None, :, 1] * c,
                                        base[None, :, 2] * flip[:, None]], -1)  # [m, 4, 3]
    keep = np.all((sites[..., 0] > edge) & (sites[..., 0] < cell_xy - edge) & (sites[..., 1] > edge) &
                  (sites[..., 1] < cell_xy - edge), axis=1)
    for cx, cy in centres:
        rho = np.hypot(sites[..., 0] - cx, sites[..., 1] - cy)
        keep &= np.all(np.abs(rho - radius) > wall, axis=1)
    idx = np.flatnonzero(keep)
    if len(idx) < nmole:
        raise ValueError(f"only {len(idx)} molecules fit; lower nmole")
    idx = np.sort(rng.permutation(idx)[:nmole])
    xyz = sites[idx].reshape(-1, 3)
    sp = butane_species(nmole)
    s = System(species=[sp], box=np.array([cell_xy, cell_xy, box_z]), x=xyz[:, 0].copy(), y=xyz[:, 1].copy(),
               z=xyz[:, 2].copy(), rcuton=rc, rcutoff=rc, rcutoffelec=rc, f0=0.5, name="butane_tube_bundle",
               delt_fs=2.0, charge_type=ELEC_NONE)
    s.sf_type = 3  # Tasos tables
    s.treq_K = 300.0
    return s, dict(atoms=atoms, period=period, radius=radius, centres=np.array(centres))


# Tasos tables of the butane / nanotube-bundle system: 0.1 A over the 127 x 127 A cell and
# 24 intervals of one tube period in z; type 1 = CH3 (sigma 3.75 A, eps/k 98 K), type 2 =
# CH2 (3.95 A, 46 K); tube carbon sigma 3.4 A, eps/k 28 K; LJ cut at 14 A, no switch.
C5_TASOS_NODES = (1271, 1271, 25)
C5_TASOS_TYPES = ((3.75, 98.0), (3.95, 46.0))


def c5_tasos_spacing(tubes: dict):
    return (0.1, 0.1, tubes["period"] / (C5_TASOS_NODES[2] - 1))


def c5_tasos_spec(tubes: dict, f_sigma: float, f_epsilon: float) -> dict:
    return dict(atoms=tubes["atoms"], ucl=(127.0, 127.0, tubes["period"]), f_sigma=f_sigma, f_epsilon=f_epsilon,
                s_sigma=3.4, s_epsilon=28.0, rcuton=14.0, rcutoff=14.0, lj_switch=0)
