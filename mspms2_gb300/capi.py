"""ctypes mirror of include/mspms2_gb300.h and marshalling of a `System` into it."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .system import System, derive_params

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class MgSpecies(C.Structure):
    _fields_ = [
        ("natom", C.c_int), ("nmole", C.c_int),
        ("ghost_type", _ip), ("interp_type", _ip),
        ("epsilon", _dp), ("sigma", _dp), ("charge", _dp), ("aw", _dp),
        ("nbond", C.c_int), ("bond_idx", _ip), ("bond_type", _ip), ("bond_param", _dp),
        ("nangle", C.c_int), ("angle_idx", _ip), ("angle_type", _ip), ("angle_param", _dp),
        ("ndih", C.c_int), ("dih_idx", _ip), ("dih_type", _ip), ("dih_param", _dp),
        ("nimp", C.c_int), ("imp_idx", _ip), ("imp_type", _ip), ("imp_param", _dp),
        ("nnbp", C.c_int), ("nbp_idx", _ip),
    ]


PARAM_FIELDS = [
    ("rcutoff", C.c_double), ("rcuton", C.c_double), ("rcutoffelec", C.c_double),
    ("lj_switch", C.c_int), ("f0", C.c_double), ("charge_type", C.c_int), ("kappa", C.c_double),
    ("kmax", C.c_int * 3), ("ksqmax", C.c_int), ("ewald_bc", C.c_int),
    ("coulomb_prefactor", C.c_double), ("sf_type", C.c_int),
    ("sigma_base", C.c_double), ("epsilon_base", C.c_double), ("compat", C.c_uint),
    ("respa_split", C.c_double),
    ("rcutoffsq", C.c_double), ("rcutonsq", C.c_double), ("rcutoffelecsq", C.c_double),
    ("roff2_minus_ron2_cube", C.c_double), ("shift1", C.c_double), ("shift4", C.c_double),
    ("wolfvcon1", C.c_double), ("wolfvcon2", C.c_double), ("wolfvcon3", C.c_double),
    ("wolffcon1", C.c_double), ("wolffcon2", C.c_double),
    ("bfactor_ewald", C.c_double), ("vfactor_ewald", C.c_double), ("twopi_lx", C.c_double),
    ("twopi_ly", C.c_double), ("twopi_lz", C.c_double), ("twopi_over_3v", C.c_double),
]


class MgParams(C.Structure):
    _fields_ = PARAM_FIELDS


ENERGY_NAMES = ["uvdw", "ushift", "ureal", "uexcl", "ufourier", "uself", "uvacuum", "uelec",
                "usflj", "uotherff", "uinter", "virial_inter",
                "ubond", "uangle", "udih", "uimp", "uintra", "virial_intra"]


class MgEnergies(C.Structure):
    _fields_ = [(n, C.c_double) for n in ENERGY_NAMES]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n in ENERGY_NAMES}


class MgOptions(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("skin", C.c_double),
                ("deterministic", C.c_int)]


class MgStats(C.Structure):
    _fields_ = [("pairs_within_cutoff", C.c_longlong), ("cluster_pairs", C.c_longlong),
                ("nclusters", C.c_longlong), ("kvectors", C.c_longlong),
                ("list_rebuilt", C.c_int), ("list_builds", C.c_int),
                ("kernel_ms", C.c_double * 8), ("kernel_launches", C.c_int)]


class MgMdParams(C.Structure):
    _fields_ = [("scheme", C.c_int), ("nstep_inner", C.c_int), ("delt", C.c_double), ("treq", C.c_double),
                ("qq", C.c_double), ("qqs", C.c_double), ("gg", C.c_double), ("ggs", C.c_double),
                ("nfree", C.c_int)]

    @classmethod
    def from_dict(cls, d: dict) -> "MgMdParams":
        return cls(**{k: d[k] for k, _ in cls._fields_})


class MgNptParams(C.Structure):
    _fields_ = [("nstep_inner", C.c_int), ("delt", C.c_double), ("treq", C.c_double), ("preq", C.c_double),
                ("qts", C.c_double), ("qbs", C.c_double), ("nfree", C.c_int), ("lj_lrc", C.c_int)]

    @classmethod
    def from_dict(cls, d: dict) -> "MgNptParams":
        return cls(**{k: d[k] for k, _ in cls._fields_})


class MgNptState(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("vts", "vbs", "rts", "utsbs", "ukin", "tinst", "pinst")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


NPT_LOG_NAMES = ["ukin", "uinter", "uintra", "ushift", "vts", "vbs", "rts", "utsbs", "tinst", "pinst", "boxlx",
                 "boxv"]


class MgTuning(C.Structure):
    _fields_ = [("cell_scale", C.c_double), ("zcap_scale", C.c_double), ("kforce_threads", C.c_int),
                ("ms_default", C.c_double), ("ms_tuned", C.c_double), ("configs_tried", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


NCOUNTS = 40


class MgCheckpoint(C.Structure):
    _fields_ = ([("natom", C.c_int)] + [(k, _dp) for k in ("x", "y", "z", "vx", "vy", "vz")] +
                [(k, C.c_double) for k in ("qq", "ps", "gg", "ss", "qqs", "pss", "ggs", "sss", "vts", "rts", "vbs",
                                           "boxlx", "boxly", "boxlz", "boxv")] +
                [("equilibrium", C.c_int), ("nframe", C.c_int), ("istep", C.c_int),
                 ("counts", C.c_int * NCOUNTS), ("accum", C.c_double * NCOUNTS)])


CHECKPOINT_SCALARS = ["qq", "ps", "gg", "ss", "qqs", "pss", "ggs", "sss", "vts", "rts", "vbs", "boxlx", "boxly",
                      "boxlz", "boxv"]


class MgSimanParams(C.Structure):
    _fields_ = [("md", MgMdParams), ("t_initial", C.c_double), ("t_min", C.c_double), ("mu_t", C.c_double),
                ("n_tries", C.c_int), ("max_stages", C.c_int), ("seed", C.c_ulonglong)]

    @classmethod
    def from_dict(cls, md: dict, sched: dict) -> "MgSimanParams":
        return cls(md=MgMdParams.from_dict(md), **sched)


SIMAN_LOG_NAMES = ["T", "ukin", "uinter", "uintra", "ushift", "tinst", "unhts", "unhtss"]
SIMAN_LOG = 8


class MgSfgridSpec(C.Structure):
    _fields_ = [("nsolid", C.c_int), ("sx", _dp), ("sy", _dp), ("sz", _dp), ("uclx", C.c_double),
                ("ucly", C.c_double), ("uclz", C.c_double), ("f_sigma", C.c_double), ("f_epsilon", C.c_double),
                ("s_sigma", C.c_double), ("s_epsilon", C.c_double), ("rcuton", C.c_double),
                ("rcutoff", C.c_double), ("lj_switch", C.c_int)]


class MgHmcParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("sigma", C.c_double), ("rcutoff", C.c_double), ("mass", C.c_double),
                ("treq", C.c_double), ("delt", C.c_double), ("nstep_md", C.c_int), ("seed", C.c_ulonglong),
                ("rescale", C.c_int), ("nconstraint", C.c_int)]


class MgSimanBatchParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("sigma", C.c_double), ("rcutoff", C.c_double), ("mass", C.c_double),
                ("delt", C.c_double), ("qq", C.c_double), ("qqs", C.c_double), ("t_initial", C.c_double),
                ("t_min", C.c_double), ("mu_t", C.c_double), ("n_tries", C.c_int), ("max_stages", C.c_int),
                ("seed", C.c_ulonglong), ("nconstraint", C.c_int)]


SIMAN_BATCH_LOG_NAMES = ["T", "ukin", "uinter", "ushift", "tinst"]
SIMAN_BATCH_LOG = 5


MD_STATE_NAMES = ["ps", "ss", "pss", "sss", "ukin", "tinst", "unhts", "unhtss"]
MD_LOG_NAMES = ["ukin", "uinter", "uintra", "ushift", "ps", "ss", "pss", "sss", "tinst", "unhts", "unhtss"]
MD_LOG = 12


class MgMdState(C.Structure):
    _fields_ = [(n, C.c_double) for n in MD_STATE_NAMES]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n in MD_STATE_NAMES}


def params_struct(p: dict) -> MgParams:
    m = MgParams()
    for name, ctype in PARAM_FIELDS:
        if name == "kmax":
            m.kmax[:] = list(p["kmax"])
        else:
            setattr(m, name, p[name])
    return m


def _arr(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel())


class SpeciesPack:
    """Owns the contiguous arrays behind an MgSpecies[] so the pointers stay valid."""

    def __init__(self, system: System):
        self.keep = []
        self.array = (MgSpecies * len(system.species))()
        for k, sp in enumerate(system.species):
            m = self.array[k]
            m.natom = sp.natom
            m.nmole = sp.nmole

            def ip(a):
                v = _arr(a, np.int32)
                self.keep.append(v)
                return v.ctypes.data_as(_ip)

            def dp(a):
                v = _arr(a, np.float64)
                self.keep.append(v)
                return v.ctypes.data_as(_dp)

            m.ghost_type = ip(sp.ghost)
            m.interp_type = ip(sp.interp)
            m.epsilon = dp(sp.epsilon)
            m.sigma = dp(sp.sigma)
            m.charge = dp(sp.charge)
            m.aw = dp(sp.aw)
            m.nbond = len(sp.bond_type)
            m.bond_idx, m.bond_type, m.bond_param = ip(sp.bond_idx), ip(sp.bond_type), dp(sp.bond_param)
            m.nangle = len(sp.angle_type)
            m.angle_idx, m.angle_type, m.angle_param = ip(sp.angle_idx), ip(sp.angle_type), dp(sp.angle_param)
            m.ndih = len(sp.dih_type)
            m.dih_idx, m.dih_type, m.dih_param = ip(sp.dih_idx), ip(sp.dih_type), dp(sp.dih_param)
            m.nimp = len(sp.imp_type)
            m.imp_idx, m.imp_type, m.imp_param = ip(sp.imp_idx), ip(sp.imp_type), dp(sp.imp_param)
            m.nnbp = len(sp.nbp_idx)
            m.nbp_idx = ip(sp.nbp_idx)

    @property
    def n(self) -> int:
        return len(self.array)


def system_params(system: System) -> MgParams:
    return params_struct(derive_params(system))
