"""System description on the host: the reference's molecule templates, globals and
input files, mirrored in Python.

`System` holds what the reference keeps in `sample_mole[]`, `nmole_per_specie[]`,
`xx/yy/zz` and its force-field globals (src/molevars.h:40-103, src/vars.h), already in
reduced units. `read_reference_dir` parses in.mspms / cfg.mspms / xyz.mspms exactly as
src/readins.c:21-263 and the section readers (src/initvars.c:397-472,
src/sffrc.c:16-222) do, including their unit reductions, and `write_reference_dir`
writes the same format so that the compiled reference can run any generated system.
`derive_params` restates the derived globals of src/initvars.c:591-599 and
:421-462.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# constants of src/defs.h:193-205
AVOGADRO = 6.0221415e23
BOLTZMAN_CONSTANT = 1.3806505e-23
COULOMB_PREFACTOR = 167100.80840
RGAS = 8.314472
R_RGAS = 0.120272219
PI = 3.141592653589793
C3_PI_SQ_THETA = 11.3105666436484
KCALMOL_TO_K = 4184.0 / RGAS  # 1 kcal/mol in K

GHOST_NONE, GHOST_LJ, GHOST_FULL = 0, 1, 2
ELEC_NONE, ELEC_EWALD, ELEC_WOLF, ELEC_SIMPLE_COULOMB = 0, 1, 2, 3
SF_NONE, SF_HYPERGEO, SF_ATOM_EXPLICIT, SF_TASOS, SF_MY_INTERP = 0, 1, 2, 3, 4
COMPAT_ALL = 0xF


@dataclass
class Species:
    """One molecule template (SAMPLE_MOLECULE, src/molevars.h:40-73), reduced units."""

    name: str
    nmole: int
    atom_names: list
    atom_type: np.ndarray
    ghost: np.ndarray
    interp: np.ndarray
    epsilon: np.ndarray
    sigma: np.ndarray
    charge: np.ndarray
    aw: np.ndarray  # reduced site mass
    aw_input: np.ndarray  # kg/mol as read (for writing files back)
    template_xyz: np.ndarray  # (natom, 3) reduced
    bond_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    bond_type: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    bond_param: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    angle_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    angle_type: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    angle_param: np.ndarray = field(default_factory=lambda: np.zeros((0, 5)))
    dih_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    dih_type: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    dih_param: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    imp_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    imp_type: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    imp_param: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    nbp_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))

    @property
    def natom(self) -> int:
        return len(self.atom_names)


@dataclass
class TasosGrid:
    """One Tasos grid (mylibtasos/grid.f90:54-129): values[nz, ny, nx, 8] in K, K/A..."""

    nx: int
    ny: int
    nz: int
    hx: float
    hy: float
    hz: float
    cuc: float
    values: np.ndarray  # float64 (nz, ny, nx, 8)


@dataclass
class MyInterpGrid:
    ncx: int
    ncy: int
    ncz: int
    itvl: tuple
    xmin: float
    ymin: float
    zmax: float
    coeff: np.ndarray  # (4, 32, ncube)


@dataclass
class System:
    species: list
    box: np.ndarray  # (3,) reduced
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    sigma_base: float = 1.0
    epsilon_base: float = 1.0
    mass_base: float = 1.0
    # force-field switches and parameters (reduced)
    rcuton: float = 0.0
    rcutoff: float = 0.0
    rcutoffelec: float = 0.0
    lj_switch: int = 0
    lj_lrc: int = 0
    f0: float = 0.0
    charge_type: int = ELEC_NONE
    kappa: float = 0.0
    kmax: tuple = (0, 0, 0)
    ksqmax: int = 0
    ewald_bc: int = 1
    ewald_dim: int = 3
    sf_type: int = SF_NONE
    compat: int = COMPAT_ALL
    respa_split: float = 0.0
    # integrator fields kept only to write the files back
    title: str = "mspms2_gb300 generated system"
    seeds: tuple = (1024, 768)
    treq_K: float = 298.0
    preq_bar: float = 1.0
    delt_fs: float = 1.0
    nstep_inner: int = 1
    what_simulation: int = 0
    what_ensemble: int = 1
    nconstraint: int = 0
    nh_qq: float = 1000.0  # Nose-Hoover masses of the MDNVT section (outer, inner)
    nh_qqs: float = 1000.0
    npt_qts: float = 1.0e3  # thermostat and barostat masses of the MDNPT section
    npt_qbs: float = 1.0e3
    nstep: int = 10
    # solid-fluid data
    tasos: list = field(default_factory=list)
    tasos_cell: tuple = (0.0, 0.0, 0.0, 0.0)  # auc, buc, cuc, radius (A)
    tube_xy_r: np.ndarray | None = None  # (ntube, 3) reduced
    solid_sigma: float = 0.0
    solid_epsilon: float = 0.0
    solid_xyz: np.ndarray | None = None  # (ns, 3) reduced
    myinterp: list = field(default_factory=list)
    name: str = "system"

    @property
    def natom(self) -> int:
        return sum(s.natom * s.nmole for s in self.species)

    @property
    def nmole(self) -> int:
        return sum(s.nmole for s in self.species)

    @property
    def coulomb_prefactor(self) -> float:
        return COULOMB_PREFACTOR / self.epsilon_base / self.sigma_base

    @property
    def const_3pisq_theta(self) -> float:
        return C3_PI_SQ_THETA * self.sigma_base * self.sigma_base

    def positions(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z])

    def site_arrays(self):
        """Per-site charge, ghost, molecule id in the reference's site order."""
        q, g, mol = [], [], []
        m = 0
        for s in self.species:
            q.append(np.tile(s.charge, s.nmole))
            g.append(np.tile(s.ghost, s.nmole))
            mol.append(np.repeat(np.arange(m, m + s.nmole), s.natom))
            m += s.nmole
        return np.concatenate(q), np.concatenate(g), np.concatenate(mol)


def derive_params(s: System) -> dict:
    """mg_params with its derived block, restating src/initvars.c:591-599, :433-462."""
    p = dict(
        rcutoff=s.rcutoff, rcuton=s.rcuton, rcutoffelec=s.rcutoffelec, lj_switch=s.lj_switch,
        f0=s.f0, charge_type=s.charge_type, kappa=s.kappa, kmax=tuple(s.kmax), ksqmax=s.ksqmax,
        ewald_bc=s.ewald_bc, coulomb_prefactor=s.coulomb_prefactor, sf_type=s.sf_type,
        sigma_base=s.sigma_base, epsilon_base=s.epsilon_base, compat=s.compat,
        respa_split=s.respa_split,
    )
    lx, ly, lz = (float(v) for v in s.box)
    p["rcutoffsq"] = s.rcutoff * s.rcutoff
    p["rcutonsq"] = s.rcuton * s.rcuton
    p["rcutoffelecsq"] = s.rcutoffelec * s.rcutoffelec
    d = p["rcutoffsq"] - p["rcutonsq"]
    p["roff2_minus_ron2_cube"] = d * d * d
    p["shift1"] = math.pow(1 / s.rcutoff, 6.0) if s.rcutoff > 0 else 0.0
    p["shift4"] = 4.0 * p["shift1"]
    for k in ("wolfvcon1", "wolfvcon2", "wolfvcon3", "wolffcon1", "wolffcon2", "bfactor_ewald",
              "vfactor_ewald", "twopi_lx", "twopi_ly", "twopi_lz", "twopi_over_3v"):
        p[k] = 0.0
    kap, rce = s.kappa, s.rcutoffelec
    if s.charge_type == ELEC_EWALD:
        p["bfactor_ewald"] = 1.0 / (4.0 * kap * kap)
        p["vfactor_ewald"] = 2.0 * PI / (lx * ly * lz)
        p["twopi_lx"] = 2.0 * PI / lx
        p["twopi_ly"] = 2.0 * PI / ly
        p["twopi_lz"] = 2.0 * PI / lz
        p["twopi_over_3v"] = 2.0 * PI / 3.0 / lx / ly / lz
    elif s.charge_type == ELEC_WOLF:
        p["wolfvcon1"] = -math.erfc(kap * rce) / rce
        p["wolfvcon2"] = math.erfc(kap * rce) / (rce * rce) + 2.0 * kap * math.exp(
            -(kap * rce) * (kap * rce)) / (math.sqrt(PI) * rce)
        p["wolfvcon3"] = kap / math.sqrt(PI) + math.erfc(kap * rce) / (2.0 * rce)
        p["wolffcon1"] = 2.0 * kap / math.sqrt(PI)
        p["wolffcon2"] = -p["wolfvcon2"]
    return p


# ---------------------------------------------------------------------------------
# reference file format
# ---------------------------------------------------------------------------------
BOLTZMANN = 1.3806505e-23  # J/K (src/defs.h:91)


def time_base(s: System) -> float:
    """Reduced time unit in fs (src/readins.c:37)."""
    return math.sqrt(s.mass_base * 1.0e-27 / (s.epsilon_base * BOLTZMANN)) * s.sigma_base * 1.0e5


def md_params(s: System) -> dict:
    """mg_md_params of the system's MD settings: delt and treq reduced as src/readins.c:44-45
    and :72-73 do, nfree = 3*natom - nconstraint (src/initvars.c:588), gg = ggs = nfree
    and the MDNVT masses (src/initvars.c:321-338)."""
    nfree = 3 * s.natom - s.nconstraint
    return dict(scheme=s.what_ensemble, nstep_inner=s.nstep_inner, delt=s.delt_fs / time_base(s),
                treq=s.treq_K / s.epsilon_base, qq=s.nh_qq, qqs=s.nh_qqs, gg=float(nfree), ggs=float(nfree),
                nfree=nfree)


def pressure_base(s: System) -> float:
    """Reduced pressure unit in bar (src/readins.c:39)."""
    return BOLTZMANN * s.epsilon_base * 1.0e25 / (s.sigma_base ** 3)


def npt_params(s: System) -> dict:
    """mg_npt_params of the system's MD settings: delt, treq and preq reduced as
    src/readins.c:44-47 and :72-73 do, nfree = 3*natom - nconstraint, the MDNPT masses
    (src/initvars.c:375) and the LJ long-range correction switch (isLJlrcOn)."""
    nfree = 3 * s.natom - s.nconstraint
    return dict(nstep_inner=s.nstep_inner, delt=s.delt_fs / time_base(s), treq=s.treq_K / s.epsilon_base,
                preq=s.preq_bar / pressure_base(s), qts=s.npt_qts, qbs=s.npt_qbs, nfree=nfree, lj_lrc=s.lj_lrc)


def npt_state0(s: System) -> dict:
    """The thermostat/barostat start of init_npt_respa (src/initvars.c:378-384)."""
    nfree = 3 * s.natom - s.nconstraint
    return dict(vts=math.sqrt((nfree + 1.0) / s.npt_qts), vbs=math.sqrt((nfree + 1.0) / s.npt_qbs), rts=0.0)


def _first(line: str) -> str:
    return line.split()[0]


def _find_section(lines, key):
    for i, ln in enumerate(lines):
        toks = ln.split()
        if toks and toks[0].upper() == key:
            return i + 1
    return None


def read_reference_dir(path: str) -> System:
    """Parse in.mspms, cfg.mspms and xyz.mspms as src/readins.c:21-263 does."""
    with open(os.path.join(path, "in.mspms")) as f:
        lines = f.read().split("\n")
    it = iter(lines)
    title = next(it)
    ij = int(_first(next(it)))
    jk = int(_first(next(it)))
    sigma_base = float(_first(next(it)))
    epsilon_base = float(_first(next(it)))
    mass_base = float(_first(next(it)))
    treq = float(_first(next(it)))
    preq = float(_first(next(it)))
    box = np.array([float(_first(next(it))) for _ in range(3)]) / sigma_base
    rcuton = float(_first(next(it))) / sigma_base
    rcutoff = float(_first(next(it))) / sigma_base
    rcutoffelec = float(_first(next(it))) / sigma_base
    lj_lrc = int(_first(next(it)))
    lj_switch = int(_first(next(it)))
    _start = int(_first(next(it)))
    nstep = int(_first(next(it)))
    for _ in range(6):
        next(it)
    delt = float(_first(next(it)))
    nstep_inner = int(_first(next(it)))
    f0 = float(_first(next(it)))
    what_sim = int(_first(next(it)))
    what_ens = int(_first(next(it)))
    ncons = int(_first(next(it)))
    _pot = int(_first(next(it)))
    charge_type = int(_first(next(it)))
    sf_type = int(_first(next(it)))
    ext_ff = int(_first(next(it)))
    if ext_ff != 0:
        raise ValueError("external force fields are not part of the nonbonded engine")

    with open(os.path.join(path, "cfg.mspms")) as f:
        toks_lines = [ln for ln in f.read().split("\n")]
    li = 0

    def nextline():
        nonlocal li
        while li < len(toks_lines) and not toks_lines[li].strip():
            li += 1
        ln = toks_lines[li]
        li += 1
        return ln

    _sysname = nextline().split()[0]
    nspecie = int(_first(nextline()))
    species = []
    for _ in range(nspecie):
        name = nextline().split()[0]
        nmole = int(_first(nextline()))
        natom = int(_first(nextline()))
        names, typ, ghost, interp, eps, sig, q, aw, awin, xyz = [], [], [], [], [], [], [], [], [], []
        for _a in range(natom):
            t = nextline().split()
            typ.append(int(t[0]))
            names.append(t[1])
            xyz.append([float(t[2]) / sigma_base, float(t[3]) / sigma_base, float(t[4]) / sigma_base])
            awin.append(float(t[8]))
            aw.append((float(t[8]) / AVOGADRO) / (mass_base * 1.0e-27))
            eps.append(float(t[9]) / epsilon_base)
            sig.append(float(t[10]) / sigma_base)
            q.append(float(t[11]))
            ghost.append(int(t[12]))
            interp.append(int(t[13]))
        sp = Species(name=name, nmole=nmole, atom_names=names, atom_type=np.array(typ, np.int32),
                     ghost=np.array(ghost, np.int32), interp=np.array(interp, np.int32),
                     epsilon=np.array(eps), sigma=np.array(sig), charge=np.array(q),
                     aw=np.array(aw), aw_input=np.array(awin), template_xyz=np.array(xyz))
        nb = int(_first(nextline()))
        bi, bt, bp = [], [], []
        for _b in range(nb):
            t = nextline().split()
            bi.append([int(t[0]), int(t[1])])
            bt.append(int(t[2]))
            kb, req, alp = float(t[3]), float(t[4]), float(t[5])
            if int(t[2]) == 2:
                kb /= epsilon_base
            else:
                kb = kb * sigma_base * sigma_base / epsilon_base
            bp.append([kb, req / sigma_base, alp / sigma_base])
        sp.bond_idx = np.array(bi, np.int32).reshape(-1, 2)
        sp.bond_type = np.array(bt, np.int32)
        sp.bond_param = np.array(bp).reshape(-1, 3)
        na = int(_first(nextline()))
        ai, at, ap = [], [], []
        for _g in range(na):
            t = nextline().split()
            ai.append([int(t[0]), int(t[1]), int(t[2])])
            at.append(int(t[3]))
            v = [float(x) for x in t[4:9]]
            if int(t[3]) == 2:
                v[0] = v[0] * sigma_base * sigma_base / epsilon_base
                v[1] = v[1] * sigma_base * sigma_base / epsilon_base
                v[2] = v[2] * sigma_base * sigma_base / epsilon_base
                v[3] /= sigma_base
                v[4] /= sigma_base
            else:
                v[0] /= epsilon_base
            ap.append(v)
        sp.angle_idx = np.array(ai, np.int32).reshape(-1, 3)
        sp.angle_type = np.array(at, np.int32)
        sp.angle_param = np.array(ap).reshape(-1, 5)
        nd = int(_first(nextline()))
        di, dt, dp = [], [], []
        for _d in range(nd):
            t = nextline().split()
            di.append([int(t[0]), int(t[1]), int(t[2]), int(t[3])])
            dt.append(int(t[4]))
            v = [float(x) for x in t[5:9]]
            if int(t[4]) == 1:
                v = [c / epsilon_base for c in v]
            elif int(t[4]) == 2:
                v[0] /= epsilon_base
            dp.append(v)
        sp.dih_idx = np.array(di, np.int32).reshape(-1, 4)
        sp.dih_type = np.array(dt, np.int32)
        sp.dih_param = np.array(dp).reshape(-1, 4)
        ni = int(_first(nextline()))
        ii, itp, ipar = [], [], []
        for _i in range(ni):
            t = nextline().split()
            ii.append([int(t[0]), int(t[1]), int(t[2]), int(t[3])])
            itp.append(int(t[4]))
            v = [float(t[5]), float(t[6])]
            if int(t[4]) == 1:
                v[0] /= epsilon_base
            ipar.append(v)
        sp.imp_idx = np.array(ii, np.int32).reshape(-1, 4)
        sp.imp_type = np.array(itp, np.int32)
        sp.imp_param = np.array(ipar).reshape(-1, 2)
        nn = int(_first(nextline()))
        nbp = []
        for _n in range(nn):
            t = nextline().split()
            nbp.append([int(float(t[0])), int(float(t[1]))])
        sp.nbp_idx = np.array(nbp, np.int32).reshape(-1, 2)
        species.append(sp)

    natom = sum(s.natom * s.nmole for s in species)
    with open(os.path.join(path, "xyz.mspms")) as f:
        xl = f.read().split("\n")
    coords = np.array([[float(v) for v in ln.split()[1:4]] for ln in xl[2:2 + natom]])
    coords = coords / sigma_base

    s = System(species=species, box=box, x=coords[:, 0].copy(), y=coords[:, 1].copy(),
               z=coords[:, 2].copy(), sigma_base=sigma_base, epsilon_base=epsilon_base,
               mass_base=mass_base, rcuton=rcuton, rcutoff=rcutoff, rcutoffelec=rcutoffelec,
               lj_switch=lj_switch, lj_lrc=lj_lrc, f0=f0, charge_type=charge_type, sf_type=sf_type,
               title=title, seeds=(ij, jk), treq_K=treq, preq_bar=preq, delt_fs=delt,
               nstep_inner=nstep_inner, what_simulation=what_sim, what_ensemble=what_ens,
               nconstraint=ncons, nstep=nstep, name=os.path.basename(os.path.normpath(path)))

    k = _find_section(lines, "MDNVT")
    if k is not None:
        s.nh_qq, s.nh_qqs = (float(v) for v in lines[k].split()[:2])
    k = _find_section(lines, "MDNPT")
    if k is not None:
        s.npt_qts, s.npt_qbs = (float(v) for v in lines[k].split()[:2])
    if charge_type in (ELEC_EWALD, ELEC_WOLF, ELEC_SIMPLE_COULOMB):
        k = _find_section(lines, "ELECTROSTATIC")
        if k is None:
            raise ValueError("ELECTROSTATIC section missing")
        if charge_type == ELEC_EWALD:
            s.kappa = float(_first(lines[k])) * sigma_base
            s.kmax = (int(_first(lines[k + 1])), int(_first(lines[k + 2])), int(_first(lines[k + 3])))
            s.ksqmax = int(_first(lines[k + 4]))
            s.ewald_bc = int(_first(lines[k + 5]))
            s.ewald_dim = int(_first(lines[k + 6]))
        elif charge_type == ELEC_WOLF:
            s.kappa = float(_first(lines[k])) * sigma_base
    if sf_type == SF_HYPERGEO:
        k = _find_section(lines, "HYPERGEO")
        ntube = int(_first(lines[k]))
        s.solid_sigma = float(_first(lines[k + 1])) / sigma_base
        s.solid_epsilon = float(_first(lines[k + 2])) / epsilon_base
        t = [[float(v) / sigma_base for v in lines[k + 3 + i].split()[:3]] for i in range(ntube)]
        s.tube_xy_r = np.array(t)
    elif sf_type == SF_ATOM_EXPLICIT:
        k = _find_section(lines, "ATOMEXPLICIT")
        ns = int(_first(lines[k]))
        t = lines[k + 1].split()
        s.solid_sigma = float(t[1]) / sigma_base
        s.solid_epsilon = float(t[2]) / epsilon_base
        s.solid_xyz = np.array([[float(v) / sigma_base for v in lines[k + 2 + i].split()[1:4]]
                                for i in range(ns)])
    elif sf_type == SF_TASOS:
        k = _find_section(lines, "TASOS")
        auc, buc, cuc, rad = (float(v) for v in lines[k].split()[:4])
        nuniq = int(_first(lines[k + 3]))
        files = [lines[k + 4 + i].split()[0] for i in range(nuniq)]
        s.tasos_cell = (auc, buc, cuc, rad)
        s.tasos = [read_tasos_grid(os.path.join(path, fn) if not os.path.isabs(fn) else fn,
                                   auc, buc, cuc) for fn in files]
    elif sf_type == SF_MY_INTERP:
        k = _find_section(lines, "MYINTERP")
        ucl = [float(v) for v in lines[k].split()[:3]]
        cen = [float(v) for v in lines[k + 1].split()[:3]]
        nuniq = int(_first(lines[k + 2]))
        for sp in species:  # init_my_interp turns Tasos-style ids into 0-based ones
            sp.interp = sp.interp - 1
        for i in range(nuniq):
            fn = lines[k + 3 + i].split()[0]
            fn = fn if os.path.isabs(fn) else os.path.join(path, fn)
            _u, itvl, dims, coeff = read_myinterp_grid(fn)
            s.myinterp.append(MyInterpGrid(int(dims[0]), int(dims[1]), int(dims[2]), itvl,
                                           cen[0] - ucl[0] / 2.0, cen[1] - ucl[1] / 2.0, ucl[2], coeff))
    return s


def tasos_dims(auc: float, buc: float, cuc: float, spacing: float = 0.2):
    """Grid size rule of mylibtasos/initialize.f90:97-104 (ANINT rounds half away)."""
    def anint(v):
        return int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)

    ngx, ngy, ngz = anint(auc / spacing), anint(buc / spacing), anint(cuc / spacing)
    return ngx, ngy, ngz, auc / ngx, buc / ngy, cuc / ngz


def read_tasos_grid(fn: str, auc: float, buc: float, cuc: float, spacing: float = 0.2) -> TasosGrid:
    ngx, ngy, ngz, hx, hy, hz = tasos_dims(auc, buc, cuc, spacing)
    v = np.loadtxt(fn).reshape(ngz + 2, ngy + 2, ngx + 2, 8)
    return TasosGrid(ngx + 2, ngy + 2, ngz + 2, hx, hy, hz, cuc, v)


def write_tasos_grid(fn: str, g: TasosGrid) -> None:
    """Text format of mylibtasos/grid.f90:81-93: K outer, J, I inner, 8 values a line."""
    with open(fn, "w") as f:
        np.savetxt(f, g.values.reshape(-1, 8), fmt="%.17g")


def _fmt(v: float) -> str:
    return repr(float(v))


def write_reference_dir(s: System, path: str, grid_names=None, nstep_trj: int = 0) -> None:
    """Write in.mspms / cfg.mspms / xyz.mspms that src/readins.c reads back to `s`
    (values written in input units: A, K, kg/mol); nstep_trj > 0 asks the program for a
    trajectory frame (trj.mspms) every nstep_trj steps."""
    os.makedirs(path, exist_ok=True)
    sb, eb = s.sigma_base, s.epsilon_base
    L = s.box * sb
    lines = [s.title, f"{s.seeds[0]}", f"{s.seeds[1]}", _fmt(sb), _fmt(eb), _fmt(s.mass_base),
             _fmt(s.treq_K), _fmt(s.preq_bar), _fmt(L[0]), _fmt(L[1]), _fmt(L[2]),
             _fmt(s.rcuton * sb), _fmt(s.rcutoff * sb), _fmt(s.rcutoffelec * sb), f"{s.lj_lrc}",
             f"{s.lj_switch}", "1", f"{s.nstep}", "0", "1", "1", "1000000", "1000000", f"{int(nstep_trj)}",
             _fmt(s.delt_fs), f"{s.nstep_inner}", _fmt(s.f0), f"{s.what_simulation}",
             f"{s.what_ensemble}", f"{s.nconstraint}", "0", f"{s.charge_type}", f"{s.sf_type}", "0",
             ""]
    lines.append("Electrostatic")
    if s.charge_type == ELEC_EWALD:
        lines += [_fmt(s.kappa / sb), f"{s.kmax[0]}", f"{s.kmax[1]}", f"{s.kmax[2]}",
                  f"{s.ksqmax}", f"{s.ewald_bc}", f"{s.ewald_dim}"]
    else:
        lines += [_fmt(s.kappa / sb)]
    lines += ["", "MDNVT", f"{_fmt(s.nh_qq)} {_fmt(s.nh_qqs)}", "", "MDNPT", f"{_fmt(s.npt_qts)} {_fmt(s.npt_qbs)}",
              ""]
    if s.sf_type == SF_HYPERGEO:
        lines += ["HyperGeo", f"{len(s.tube_xy_r)}", _fmt(s.solid_sigma * sb), _fmt(s.solid_epsilon * eb)]
        lines += [" ".join(_fmt(v * sb) for v in row) for row in s.tube_xy_r]
        lines.append("")
    if s.sf_type == SF_ATOM_EXPLICIT:
        lines += ["AtomExplicit", f"{len(s.solid_xyz)}",
                  f"1 {_fmt(s.solid_sigma * sb)} {_fmt(s.solid_epsilon * eb)} 0.0"]
        lines += ["C " + " ".join(_fmt(v * sb) for v in row) for row in s.solid_xyz]
        lines.append("")
    if s.sf_type == SF_TASOS:
        auc, buc, cuc, rad = s.tasos_cell
        names = grid_names or [f"grid{i + 1}.tasos" for i in range(len(s.tasos))]
        lines += ["Tasos", f"{_fmt(auc)} {_fmt(buc)} {_fmt(cuc)} {_fmt(rad)}", "1 1 1",
                  f"{len(s.tasos)}", f"{len(s.tasos)}"] + names + [""]
        for g, fn in zip(s.tasos, names):
            write_tasos_grid(os.path.join(path, fn), g)
    if s.sf_type == SF_MY_INTERP:
        g0 = s.myinterp[0]
        ucl = (g0.ncx * g0.itvl[0], g0.ncy * g0.itvl[1], g0.zmax)
        centre = (g0.xmin + ucl[0] / 2.0, g0.ymin + ucl[1] / 2.0, 0.0)
        names = grid_names or [f"grid{i + 1}.myinterp" for i in range(len(s.myinterp))]
        lines += ["MyInterp", " ".join(_fmt(v) for v in ucl), " ".join(_fmt(v) for v in centre),
                  f"{len(s.myinterp)}"] + names + [""]
        for g, fn in zip(s.myinterp, names):
            write_myinterp_grid(os.path.join(path, fn), g, ucl, centre)
    lines += ["HMC", "10", "1.0", "0.0", "0.0", "0.0", "0.5", "0.5", "100.0", "100", "100", "-10.0 1.0",
              "", "SimAn", "10 1", "1000.0 300.0 1.01", ""]
    with open(os.path.join(path, "in.mspms"), "w") as f:
        f.write("\n".join(lines))
    cl = [s.name.replace(" ", "_") or "system", f"{len(s.species)} species"]
    for sp in s.species:
        cl += [sp.name, f"{sp.nmole} molecules", f"{sp.natom} atoms"]
        for a in range(sp.natom):
            x, y, z = sp.template_xyz[a] * sb
            cl.append(" ".join([str(int(sp.atom_type[a])), sp.atom_names[a], _fmt(x), _fmt(y), _fmt(z),
                                _fmt(x), _fmt(y), _fmt(z), _fmt(sp.aw_input[a]), _fmt(sp.epsilon[a] * eb),
                                _fmt(sp.sigma[a] * sb), _fmt(sp.charge[a]), str(int(sp.ghost[a])),
                                str(int(sp.interp[a]) + (1 if s.sf_type == SF_MY_INTERP else 0))]))
        cl.append(f"{len(sp.bond_type)} bonds")
        for i in range(len(sp.bond_type)):
            kb, req, alp = sp.bond_param[i]
            kbin = kb * eb if sp.bond_type[i] == 2 else kb * eb / (sb * sb)
            cl.append(f"{sp.bond_idx[i, 0]} {sp.bond_idx[i, 1]} {sp.bond_type[i]} {_fmt(kbin)} "
                      f"{_fmt(req * sb)} {_fmt(alp * sb)}")
        cl.append(f"{len(sp.angle_type)} angles")
        for i in range(len(sp.angle_type)):
            v = list(sp.angle_param[i])
            if sp.angle_type[i] == 2:
                v[0] = v[0] * eb / (sb * sb)
                v[1] = v[1] * eb / (sb * sb)
                v[2] = v[2] * eb / (sb * sb)
                v[3] *= sb
                v[4] *= sb
            else:
                v[0] *= eb
            cl.append(" ".join(str(int(k)) for k in sp.angle_idx[i]) + f" {sp.angle_type[i]} " +
                      " ".join(_fmt(k) for k in v))
        cl.append(f"{len(sp.dih_type)} dihedrals")
        for i in range(len(sp.dih_type)):
            v = list(sp.dih_param[i])
            if sp.dih_type[i] == 1:
                v = [c * eb for c in v]
            elif sp.dih_type[i] == 2:
                v[0] *= eb
            cl.append(" ".join(str(int(k)) for k in sp.dih_idx[i]) + f" {sp.dih_type[i]} " +
                      " ".join(_fmt(k) for k in v))
        cl.append(f"{len(sp.imp_type)} impropers")
        for i in range(len(sp.imp_type)):
            v = list(sp.imp_param[i])
            if sp.imp_type[i] == 1:
                v[0] *= eb
            cl.append(" ".join(str(int(k)) for k in sp.imp_idx[i]) + f" {sp.imp_type[i]} " +
                      " ".join(_fmt(k) for k in v))
        cl.append(f"{len(sp.nbp_idx)} nonbonded")
        for i in range(len(sp.nbp_idx)):
            cl.append(f"{sp.nbp_idx[i, 0]} {sp.nbp_idx[i, 1]}")
    with open(os.path.join(path, "cfg.mspms"), "w") as f:
        f.write("\n".join(cl) + "\n")
    n = s.natom
    names = []
    for sp in s.species:
        names += sp.atom_names * sp.nmole
    xl = [str(n), ""] + [f"{names[i]} {_fmt(s.x[i] * sb)} {_fmt(s.y[i] * sb)} {_fmt(s.z[i] * sb)}"
                         for i in range(n)]
    with open(os.path.join(path, "xyz.mspms"), "w") as f:
        f.write("\n".join(xl) + "\n")


# ---------------------------------------------------------------------------------
# compact serialisation (npz) used for fixtures and benchmark inputs
# ---------------------------------------------------------------------------------
_SCALARS = ["sigma_base", "epsilon_base", "mass_base", "rcuton", "rcutoff", "rcutoffelec", "lj_switch",
            "lj_lrc", "f0", "charge_type", "kappa", "ksqmax", "ewald_bc", "ewald_dim", "sf_type",
            "compat", "respa_split", "solid_sigma", "solid_epsilon", "name"]
# MD settings, stored only when present in an archive (older archives lack them)
_MD_SCALARS = ["treq_K", "delt_fs", "nstep_inner", "what_ensemble", "nconstraint", "nh_qq", "nh_qqs", "preq_bar",
               "npt_qts", "npt_qbs"]
_SP_ARRAYS = ["atom_type", "ghost", "interp", "epsilon", "sigma", "charge", "aw", "aw_input",
              "template_xyz", "bond_idx", "bond_type", "bond_param", "angle_idx", "angle_type",
              "angle_param", "dih_idx", "dih_type", "dih_param", "imp_idx", "imp_type", "imp_param",
              "nbp_idx"]


def system_to_arrays(s: System, prefix: str = "") -> dict:
    d = {}
    for k in _SCALARS + _MD_SCALARS:
        d[prefix + k] = np.array(getattr(s, k))
    d[prefix + "kmax"] = np.array(s.kmax)
    d[prefix + "box"] = np.asarray(s.box)
    d[prefix + "xyz"] = np.stack([s.x, s.y, s.z])
    d[prefix + "nspecies"] = np.array(len(s.species))
    for i, sp in enumerate(s.species):
        p = f"{prefix}sp{i}_"
        d[p + "name"] = np.array(sp.name)
        d[p + "nmole"] = np.array(sp.nmole)
        d[p + "atom_names"] = np.array(sp.atom_names)
        for k in _SP_ARRAYS:
            d[p + k] = np.asarray(getattr(sp, k))
    if s.tube_xy_r is not None:
        d[prefix + "tube_xy_r"] = s.tube_xy_r
    if s.solid_xyz is not None:
        d[prefix + "solid_xyz"] = s.solid_xyz
    d[prefix + "ntasos"] = np.array(len(s.tasos))
    d[prefix + "tasos_cell"] = np.array(s.tasos_cell)
    for i, g in enumerate(s.tasos):
        p = f"{prefix}tasos{i}_"
        d[p + "dims"] = np.array([g.nx, g.ny, g.nz])
        d[p + "h"] = np.array([g.hx, g.hy, g.hz, g.cuc])
        d[p + "values"] = g.values
    d[prefix + "nmyinterp"] = np.array(len(s.myinterp))
    for i, g in enumerate(s.myinterp):
        p = f"{prefix}myi{i}_"
        d[p + "dims"] = np.array([g.ncx, g.ncy, g.ncz])
        d[p + "geom"] = np.array(list(g.itvl) + [g.xmin, g.ymin, g.zmax])
        d[p + "coeff"] = g.coeff
    return d


def system_from_arrays(d, prefix: str = "") -> System:
    def g(k):
        return d[prefix + k]

    species = []
    for i in range(int(g("nspecies"))):
        p = f"sp{i}_"
        kw = {k: np.array(g(p + k)) for k in _SP_ARRAYS}
        sp = Species(name=str(g(p + "name")), nmole=int(g(p + "nmole")),
                     atom_names=[str(v) for v in g(p + "atom_names")], **kw)
        species.append(sp)
    xyz = np.array(g("xyz"), dtype=np.float64)
    s = System(species=species, box=np.array(g("box"), dtype=np.float64), x=xyz[0].copy(),
               y=xyz[1].copy(), z=xyz[2].copy())
    for k in _SCALARS + [k for k in _MD_SCALARS if prefix + k in d]:
        v = g(k)
        cur = getattr(s, k)
        setattr(s, k, str(v) if isinstance(cur, str) else type(cur)(v.item()))
    s.kmax = tuple(int(v) for v in g("kmax"))
    if prefix + "tube_xy_r" in d:
        s.tube_xy_r = np.array(g("tube_xy_r"))
    if prefix + "solid_xyz" in d:
        s.solid_xyz = np.array(g("solid_xyz"))
    s.tasos_cell = tuple(float(v) for v in g("tasos_cell"))
    for i in range(int(g("ntasos"))):
        p = f"tasos{i}_"
        nx, ny, nz = (int(v) for v in g(p + "dims"))
        hx, hy, hz, cuc = (float(v) for v in g(p + "h"))
        s.tasos.append(TasosGrid(nx, ny, nz, hx, hy, hz, cuc, np.array(g(p + "values"))))
    for i in range(int(g("nmyinterp"))):
        p = f"myi{i}_"
        ncx, ncy, ncz = (int(v) for v in g(p + "dims"))
        geom = [float(v) for v in g(p + "geom")]
        s.myinterp.append(MyInterpGrid(ncx, ncy, ncz, tuple(geom[:3]), geom[3], geom[4], geom[5],
                                       np.array(g(p + "coeff"))))
    return s


def save_system(s: System, fn: str, **extra) -> None:
    d = system_to_arrays(s)
    d.update(extra)
    np.savez_compressed(fn, **d)


def load_system(fn: str):
    d = np.load(fn, allow_pickle=False)
    return system_from_arrays(d), d


def read_myinterp_grid(fn: str) -> tuple:
    """Binary grid of init_my_interp (src/sffrc.c:297-740): returns (ucl, itvl, dims, coeff)."""
    with open(fn, "rb") as f:
        raw = f.read()
    ucl = np.frombuffer(raw, np.float64, 3, 0)
    _centre = np.frombuffer(raw, np.float64, 3, 24)
    ints = np.frombuffer(raw, np.int32, 4, 48)
    itvl = np.frombuffer(raw, np.float64, 3, 64)
    ncube = (ints[1] - 1) * (ints[2] - 1) * (ints[3] - 1)
    coeff = np.frombuffer(raw, np.float64, 4 * 32 * ncube, 88).reshape(4, 32, ncube)
    return ucl.copy(), tuple(itvl), (ints[1] - 1, ints[2] - 1, ints[3] - 1), coeff.copy()


def write_myinterp_grid(fn: str, g: MyInterpGrid, ucl, centre) -> None:
    with open(fn, "wb") as f:
        f.write(np.asarray(ucl, np.float64).tobytes())
        f.write(np.asarray(centre, np.float64).tobytes())
        ng = [(g.ncx + 1) * (g.ncy + 1) * (g.ncz + 1), g.ncx + 1, g.ncy + 1, g.ncz + 1]
        f.write(np.asarray(ng, np.int32).tobytes())
        f.write(np.asarray(g.itvl, np.float64).tobytes())
        f.write(np.ascontiguousarray(g.coeff, np.float64).tobytes())
