"""System builders shared by the golden-fixture generator (gen_golden.py) and the live
comparison of the oracle with the compiled reference (tests/test_oracle_live_reference.py):
small LJ gases, an analytic Tasos test grid, a six-site molecule that reaches every bonded
and ghost switch, and seeded random variants of all of them. Nothing here needs the
reference checkout.
"""
from __future__ import annotations

import numpy as np

from mspms2_gb300 import configs
from mspms2_gb300.system import (ELEC_EWALD, ELEC_NONE, ELEC_SIMPLE_COULOMB, ELEC_WOLF, SF_ATOM_EXPLICIT,
                                 SF_HYPERGEO, SF_MY_INTERP, SF_TASOS, MyInterpGrid, Species, System,
                                 TasosGrid, tasos_dims)


def lj_gas(n, box, seed, sigma=3.5, eps=50.0, xy_range=None, rc=None, avoid=None):
    """n LJ sites on a jittered cubic lattice (spacing >= 1.05 sigma) inside the box, or
    inside xy_range in x and y; `avoid(p)` rejects lattice points (near solid walls)."""
    rng = np.random.default_rng(seed)
    lo, hi = (0.0, box) if xy_range is None else xy_range
    a = 1.05 * sigma
    gx = np.arange(lo + 0.5 * a, hi - 0.25 * a, a)
    gz = np.arange(0.5 * a, box - 0.25 * a, a)
    X, Y, Z = np.meshgrid(gx, gx, gz, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    if avoid is not None:
        pts = pts[[not avoid(p) for p in pts]]
    if len(pts) < n:
        raise ValueError(f"lattice holds {len(pts)} sites < {n}")
    pts = pts[rng.permutation(len(pts))[:n]] + rng.uniform(-0.05 * sigma, 0.05 * sigma, size=(n, 3))
    sp = configs.lj_species(n)
    sp.sigma = np.array([sigma])
    sp.epsilon = np.array([eps])
    rc = rc if rc is not None else 0.5 * box - 1e-6
    return System(species=[sp], box=np.array([box, box, box]), x=pts[:, 0].copy(), y=pts[:, 1].copy(),
                  z=pts[:, 2].copy(), rcuton=rc, rcutoff=rc, rcutoffelec=rc, name=f"ljgas{n}")


def tasos_test_grid(auc, buc, cuc, seed):
    """Smooth analytic field with exact derivatives, Dxyz perturbed so the reference's
    corner pairing of Dxyz is visible."""
    ngx, ngy, ngz, hx, hy, hz = tasos_dims(auc, buc, cuc)
    x = np.arange(ngx + 2) * hx
    y = np.arange(ngy + 2) * hy
    z = np.arange(ngz + 2) * hz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    a, b, c = 1.3, 0.9, 2 * np.pi / cuc
    A = 400.0
    sx, cx = np.sin(a * X), np.cos(a * X)
    sy, cy = np.sin(b * Y), np.cos(b * Y)
    sz, cz = np.sin(c * Z), np.cos(c * Z)
    F = A * sx * cy * cz - 900.0 + 30.0 * (X - auc / 2) ** 2
    v = np.zeros(F.shape + (8,))
    v[..., 0] = F
    v[..., 1] = A * a * cx * cy * cz + 60.0 * (X - auc / 2)
    v[..., 2] = -A * b * sx * sy * cz
    v[..., 3] = -A * c * sx * cy * sz
    v[..., 4] = -A * a * b * cx * sy * cz
    v[..., 5] = -A * a * c * cx * cy * sz
    v[..., 6] = A * b * c * sx * sy * sz
    rng = np.random.default_rng(seed)
    v[..., 7] = A * a * b * c * cx * sy * sz + rng.normal(scale=50.0, size=F.shape)
    return TasosGrid(ngx + 2, ngy + 2, ngz + 2, hx, hy, hz, cuc, v)


def custom_molecule_system(seed, with_nbp=False):
    """A 6-site molecule with ghosts (LJ and FULL), nbp pairs, CHARMM dihedral and
    improper, FENE/harmonic/Morse bonds, harmonic angles; Wolf electrostatics."""
    rng = np.random.default_rng(seed)
    tmpl = np.array([[0, 0, 0], [1.5, 0, 0], [2.1, 1.3, 0], [3.5, 1.4, 0.4], [1.4, -1.2, 0.5],
                     [4.2, 2.5, 0.3]], dtype=float)
    sp = Species(name="hexa", nmole=0, atom_names=["A", "B", "C", "D", "E", "F"],
                 atom_type=np.arange(6, dtype=np.int32),
                 ghost=np.array([0, 0, 1, 0, 2, 0], np.int32), interp=np.ones(6, np.int32),
                 epsilon=np.array([60.0, 45.0, 30.0, 80.0, 20.0, 55.0]),
                 sigma=np.array([3.4, 3.6, 2.5, 3.8, 2.0, 3.3]),
                 charge=np.array([-0.4, 0.3, 0.2, -0.3, 0.1, 0.1]),
                 aw=np.array([12.0, 14.0, 1.0, 16.0, 1.0, 12.0]) * 1.66054,
                 aw_input=np.array([12.0, 14.0, 1.0, 16.0, 1.0, 12.0]) * 1e-3, template_xyz=tmpl)
    sp.aw = (sp.aw_input / 6.0221415e23) / 1.0e-27
    sp.bond_idx = np.array([[0, 1], [1, 2], [2, 3], [1, 4], [3, 5]], np.int32)
    sp.bond_type = np.array([1, 2, 3, 1, 1], np.int32)
    sp.bond_param = np.array([[100000.0, 1.5, 0.0], [30000.0, 1.45, 2.0], [5000.0, 2.5, 0.0],
                              [90000.0, 1.3, 0.0], [80000.0, 1.4, 0.0]])
    sp.angle_idx = np.array([[0, 1, 2], [1, 2, 3], [0, 1, 4], [2, 3, 5]], np.int32)
    sp.angle_type = np.ones(4, np.int32)
    sp.angle_param = np.array([[40000.0, 1.9, 0, 0, 0], [35000.0, 2.0, 0, 0, 0], [30000.0, 1.95, 0, 0, 0],
                               [20000.0, 2.1, 0, 0, 0]])
    sp.dih_idx = np.array([[0, 1, 2, 3], [1, 2, 3, 5], [4, 1, 2, 3]], np.int32)
    sp.dih_type = np.array([1, 2, 1], np.int32)
    sp.dih_param = np.array([[0.0, 700.0, -130.0, 1500.0], [300.0, 3.0, 0.0, 0.0], [10.0, 200.0, 50.0, 300.0]])
    sp.imp_idx = np.array([[1, 0, 2, 4]], np.int32)
    sp.imp_type = np.array([1], np.int32)
    sp.imp_param = np.array([[150.0, 35.0]])
    if with_nbp:
        sp.nbp_idx = np.array([[0, 3], [0, 5], [4, 5], [2, 5]], np.int32)
    nside = 3
    box = 16.0
    sp.nmole = nside ** 3
    g = np.arange(nside)
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    cen = (np.stack([cx.ravel(), cy.ravel(), cz.ravel()], 1) + 0.5) * (box / nside)
    rot = configs._random_rotations(rng, sp.nmole)
    xyz = (cen[:, None, :] + np.einsum("mij,aj->mai", rot, tmpl - tmpl.mean(0))).reshape(-1, 3)
    return System(species=[sp], box=np.array([box] * 3), x=xyz[:, 0].copy(), y=xyz[:, 1].copy(),
                  z=xyz[:, 2].copy(), rcuton=6.0, rcutoff=7.9, rcutoffelec=7.9, lj_switch=1, f0=0.5,
                  charge_type=ELEC_WOLF, kappa=0.25, name="custom")


def _elec_and_cutoffs(s: System, rng, elec_choices=(ELEC_NONE, ELEC_WOLF, ELEC_EWALD, ELEC_EWALD,
                                                   ELEC_SIMPLE_COULOMB)):
    """Random electrostatics (with its kappa, k-vector set and boundary condition), LJ
    switch, 1-4 scale and cutoffs below half the shortest box edge; about one case in six
    each has the cutoff at 0.4999 of the shortest edge, an extreme kappa, no k-vectors along
    one axis, or the whole cube of k-vectors."""
    s.charge_type = int(elec_choices[rng.integers(len(elec_choices))])
    edge = int(rng.integers(6))  # 0-3: one edge case each (below), else none
    rc = (0.4999 if edge == 0 else float(rng.uniform(0.3, 0.48))) * float(np.min(s.box))
    s.rcutoff = s.rcutoffelec = rc
    s.kappa = float(rng.choice([0.05, 0.9])) if edge == 1 else float(rng.uniform(0.2, 0.4))
    s.kmax = tuple(int(v) for v in rng.integers(2, 6, size=3))
    if edge == 2:  # no k-vectors along one axis
        s.kmax = tuple(0 if a == int(rng.integers(3)) else k for a, k in enumerate(s.kmax))
    s.ksqmax = int(rng.integers(4, max(s.kmax) ** 2 + 2))
    if edge == 3:  # a bound above every corner of the box of k-vectors: the whole cube
        s.ksqmax = sum(k * k for k in s.kmax) + 1
    s.ewald_bc = int(rng.integers(1, 3)) if s.charge_type == ELEC_EWALD else 1
    s.lj_switch = int(rng.integers(2))
    s.rcuton = rc * float(rng.uniform(0.6, 0.9)) if s.lj_switch else rc
    s.f0 = float(rng.uniform(0.0, 1.0))


def _stretch(s: System, rng):
    """A non-cubic box: one axis and the positions along it stretched by up to 15%."""
    ax = int(rng.integers(3))
    f = float(rng.uniform(1.0, 1.15))
    s.box = np.array(s.box, dtype=float)
    s.box[ax] *= f
    v = (s.x, s.y, s.z)[ax]
    v *= f


FAMILIES = ("water", "water_wrapped", "butane", "ions", "custom", "hypergeo", "atom_explicit", "tasos",
            "myinterp", "two_species")


def _split_species(s: System, rng) -> System:
    """The water molecules as two species: the first k keep the template, the rest get
    their own LJ parameters and charges (scaled, still neutral), so that the pair loop's
    cross-species branch runs."""
    import copy
    sp = s.species[0]
    k = int(rng.integers(1, sp.nmole))
    b = copy.deepcopy(sp)
    b.name = sp.name + "_b"
    sp.nmole, b.nmole = k, sp.nmole - k
    b.epsilon = sp.epsilon * float(rng.uniform(0.7, 1.3))
    b.sigma = sp.sigma * float(rng.uniform(0.9, 1.1))
    b.charge = sp.charge * float(rng.uniform(0.8, 1.2))
    s.species = [sp, b]
    return s


def random_variant(seed: int) -> System:
    """Seeded random system of family FAMILIES[seed % len(FAMILIES)], with random model
    switches, cutoffs and box shape."""
    rng = np.random.default_rng(7000 + seed)
    fam = FAMILIES[seed % len(FAMILIES)]
    if fam in ("water", "water_wrapped"):
        nside = int(rng.integers(3, 5))
        box = float(rng.uniform(3.1, 3.6) * nside)
        s = configs.water_small(nside, box, seed=seed, charge_type=ELEC_EWALD, kappa=0.3, rc=0.45 * box, kmax=4,
                                ksqmax=20)
        _stretch(s, rng)
        _elec_and_cutoffs(s, rng)
        if fam == "water_wrapped":  # per-site wrap: molecules straddle the box faces
            for a, v in enumerate((s.x, s.y, s.z)):
                v -= s.box[a] * np.floor(v / s.box[a])
    elif fam == "two_species":
        nside = int(rng.integers(3, 5))
        box = float(rng.uniform(3.1, 3.6) * nside)
        s = configs.water_small(nside, box, seed=seed, charge_type=ELEC_EWALD, kappa=0.3, rc=0.45 * box, kmax=4,
                                ksqmax=20)
        _split_species(s, rng)
        _stretch(s, rng)
        _elec_and_cutoffs(s, rng)
    elif fam == "butane":
        s = configs.butane_box(3, float(rng.uniform(15.0, 17.0)), seed=seed, rc=7.0, charged=True,
                               site_jitter=0.05)
        _stretch(s, rng)
        _elec_and_cutoffs(s, rng)
    elif fam == "ions":
        s = configs.ion_box(4, seed=seed, kmax=4, ksqmax=20, rc=5.0, spacing=3.2)
        for sp in s.species:
            sp.epsilon = np.array([float(rng.uniform(20, 80))])
            sp.sigma = np.array([float(rng.uniform(2.4, 3.0))])
        _stretch(s, rng)
        _elec_and_cutoffs(s, rng)
    elif fam == "custom":
        # no nbp pairs: the reference's own nbp path gives non-finite forces (its pair indices
        # are doubles read with %d), which tests/test_oracle_live_reference.py records apart
        s = custom_molecule_system(seed)
        _stretch(s, rng)
        _elec_and_cutoffs(s, rng)
    elif fam == "hypergeo":
        tubes = np.column_stack([rng.uniform(3, 11, 3), rng.uniform(3, 11, 3), rng.uniform(1.6, 3.0, 3)])

        def near_wall(p, tubes=tubes):
            return any(abs(np.hypot(p[0] - t[0], p[1] - t[1]) - t[2]) < 2.2 for t in tubes)
        s = lj_gas(int(rng.integers(10, 25)), 14.0, seed=seed, avoid=near_wall, sigma=2.5)
        s.sf_type = SF_HYPERGEO
        s.tube_xy_r = tubes
        s.solid_sigma, s.solid_epsilon = float(rng.uniform(3.0, 3.6)), float(rng.uniform(20, 40))
    elif fam == "atom_explicit":
        solid = rng.uniform(0, 14.0, size=(int(rng.integers(10, 30)), 3))

        def near_solid(p, solid=solid):
            d = solid - p
            d -= 14.0 * np.rint(d / 14.0)
            return (d ** 2).sum(1).min() < 2.6 ** 2
        s = lj_gas(int(rng.integers(10, 20)), 14.0, seed=seed, avoid=near_solid, sigma=2.5)
        s.sf_type = SF_ATOM_EXPLICIT
        s.lj_switch = int(rng.integers(2))
        s.rcuton = float(rng.uniform(4.5, 6.0)) if s.lj_switch else s.rcutoff
        s.solid_xyz = solid
        s.solid_sigma, s.solid_epsilon = float(rng.uniform(3.0, 3.6)), float(rng.uniform(20, 40))
    elif fam == "tasos":
        s = lj_gas(int(rng.integers(6, 12)), 12.0, seed=seed, xy_range=(0.3, 3.7), sigma=1.0, eps=5.0)
        s.sf_type = SF_TASOS
        s.species[0].interp = np.array([1], np.int32)
        s.tasos_cell = (4.0, 4.0, 2.4595, 1.0)
        s.tasos = [tasos_test_grid(4.0, 4.0, 2.4595, seed)]
    else:
        s = lj_gas(int(rng.integers(6, 12)), 12.0, seed=seed, xy_range=(0.2, 3.8), sigma=1.0, eps=5.0)
        s.sf_type = SF_MY_INTERP
        s.species[0].interp = np.array([0], np.int32)
        ncx, ncy, ncz = 4, 4, 3
        scale = np.array([1, .1, .1, .1, .01, .01, .01, .01, .01, .01] + [.001] * 10 + [1e-4] * 12)
        coeff = rng.normal(size=(4, 32, ncx * ncy * ncz)) * (50.0 * scale)[None, :, None]
        s.myinterp = [MyInterpGrid(ncx, ncy, ncz, (1.0, 1.0, 1.0), 0.0, 0.0, 3.0, coeff)]
    s.name = f"live_{fam}_{seed}"
    return s


MD_FAMILIES = ("water", "lj", "butane", "ions")


def random_md_variant(seed: int) -> System:
    """Seeded random start for the reference's own integrators: family
    MD_FAMILIES[seed % 4], ensemble NVE (vver), NVT (vver_nh_3) or NPT (npt_respa), with
    random time step, inner steps, thermostat and barostat masses, pressure, LJ
    long-range correction and velocity seeds."""
    rng = np.random.default_rng(9000 + seed)
    fam = MD_FAMILIES[seed % len(MD_FAMILIES)]
    ens = int(rng.integers(0, 3))
    if fam == "water":
        nside = int(rng.integers(3, 5))
        box = float(rng.uniform(3.0, 3.3) * nside)
        elec = (ELEC_NONE, ELEC_WOLF, ELEC_EWALD)[rng.integers(3)]
        s = configs.water_small(nside, box, seed=seed, charge_type=elec, kappa=0.3, rc=0.45 * box, kmax=4, ksqmax=20)
        s.delt_fs = float(rng.uniform(0.2, 0.6))
    elif fam == "lj":
        s = configs.lj_replica(int(rng.integers(150, 300)), seed=seed)
        s.treq_K = float(rng.uniform(0.8, 1.5))
        s.delt_fs = float(rng.uniform(2.0, 5.0))
    elif fam == "butane":
        s = configs.butane_box(3, float(rng.uniform(17.0, 19.0)), seed=seed, rc=7.0, site_jitter=0.05)
        s.delt_fs = float(rng.uniform(0.5, 1.5))
    else:
        s = configs.ion_box(3, seed=seed, kmax=4, ksqmax=16, rc=4.0, spacing=3.5, jitter=0.2)
        for sp in s.species:
            sp.epsilon, sp.sigma = np.array([float(rng.uniform(30, 100))]), np.array([float(rng.uniform(2.6, 3.2))])
            sp.aw_input = sp.aw_input * 30.0
            sp.aw = sp.aw * 30.0
        s.delt_fs = float(rng.uniform(0.5, 2.0))
    s.what_ensemble = ens
    s.nstep_inner = int(rng.integers(1, 5)) if ens else 1
    s.nh_qq, s.nh_qqs = float(rng.uniform(200, 5000)), float(rng.uniform(200, 5000))
    s.seeds = (int(rng.integers(1, 30000)), int(rng.integers(1, 30000)))
    if ens == 2:
        s.preq_bar = float(rng.uniform(1, 1000))
        s.npt_qts, s.npt_qbs = float(rng.uniform(1e3, 5e4)), float(rng.uniform(1e3, 5e4))
        s.lj_lrc = int(rng.integers(2))
    s.name = f"md_live_{fam}_{seed}"
    return s
