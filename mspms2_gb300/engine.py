"""Host-side wrapper of the engine's C ABI (include/mspms2_gb300.h).

`Engine(system)` mirrors what the reference does around its force layer: it takes the
molecule templates and globals of a `System`, and `compute()` plays the role of one
frclong() + frcshort() pair (src/frclong.c:20, src/frcshort.c:20) on the GPU, returning
forces in the reference's layout (x/y/z arrays per site) and the reference's energy
names. There is no CPU path: without the compiled library or an sm_103 device the
constructor raises.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import capi
from .capi import MgEnergies, MgOptions, MgSpecies, MgStats, SpeciesPack
from .system import SF_ATOM_EXPLICIT, SF_HYPERGEO, SF_MY_INTERP, SF_TASOS, System, derive_params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmspms2_gb300.so")

MG_OK, MG_ERR_NONFINITE = 0, 6
TERMS_LONG, TERMS_SHORT, TERMS_ALL = 1, 2, 3
PREC = {"mixed": 0, "fp64": 1}
STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NO_DEVICE", 4: "STATE", 5: "OUT_OF_GRID", 6: "NONFINITE",
          7: "CAPACITY", 8: "UNSUPPORTED", 9: "ALLOC"}

_dp = C.POINTER(C.c_double)
_lib = None


class EngineError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mspms2_gb300 {STATUS.get(status, status)}: {msg}")
        self.status = status


def load_library(path: str = LIB_PATH):
    """Load the in-tree CUDA library (build it first with mspms2_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise EngineError(2, f"{path} is missing; run mspms2_gb300.build.build()")
    lib = C.CDLL(path)
    V, I, D = C.c_void_p, C.c_int, C.c_double
    lib.mg_create.argtypes = [C.POINTER(V), C.POINTER(MgOptions)]
    lib.mg_destroy.argtypes = [V]
    lib.mg_last_error.argtypes = [V]
    lib.mg_last_error.restype = C.c_char_p
    lib.mg_options_default.argtypes = [C.POINTER(MgOptions)]
    lib.mg_params_derive.argtypes = [C.POINTER(capi.MgParams), D, D, D]
    lib.mg_params_derive.restype = None
    lib.mg_set_topology.argtypes = [V, I, C.POINTER(MgSpecies)]
    lib.mg_set_params.argtypes = [V, C.POINTER(capi.MgParams)]
    lib.mg_set_box.argtypes = [V, D, D, D]
    lib.mg_set_stream.argtypes = [V, V]
    lib.mg_set_timing.argtypes = [V, I]
    lib.mg_sf_tasos_set_grid.argtypes = [V, I, I, I, I, D, D, D, D, _dp]
    lib.mg_sf_hypergeo_set.argtypes = [V, I, _dp, _dp, _dp, D, D, D]
    lib.mg_sf_atom_explicit_set.argtypes = [V, I, _dp, _dp, _dp, D, D]
    lib.mg_sf_myinterp_set.argtypes = [V, I, I, I, I, D, D, D, D, D, D, _dp]
    lib.mg_compute.argtypes = [V, _dp, _dp, _dp, I, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(MgEnergies)]
    lib.mg_compute_device.argtypes = [V, V, V, V, I, V, V, V, V, V, V, C.POINTER(MgEnergies)]
    lib.mg_get_stats.argtypes = [V, C.POINTER(MgStats)]
    lib.mg_get_device_flags.argtypes = [V, C.POINTER(C.c_uint)]
    lib.mg_debug_get_list.argtypes = [V, C.POINTER(I), C.POINTER(C.c_longlong), C.POINTER(I),
                                      C.POINTER(D), C.POINTER(I), C.POINTER(I), C.POINTER(I)]
    lib.mg_abi_version.restype = I
    lib.mg_md_run.argtypes = [V, C.POINTER(capi.MgMdParams), I, _dp, _dp, _dp, _dp, _dp, _dp,
                              C.POINTER(capi.MgMdState), _dp]
    lib.mg_hmc_batch.argtypes = [I, C.POINTER(capi.MgHmcParams), I, C.POINTER(I), _dp, _dp, _dp, _dp, I, I,
                                 C.POINTER(I), _dp, _dp]
    lib.mg_siman_batch.argtypes = [I, C.POINTER(capi.MgSimanBatchParams), I, C.POINTER(I), _dp, _dp, _dp, _dp,
                                   C.POINTER(I), _dp]
    lib.mg_sfgrid_sfgridgen.argtypes = [I, C.POINTER(capi.MgSfgridSpec), D, I, C.POINTER(I), _dp]
    lib.mg_sfgrid_tasos.argtypes = [I, C.POINTER(capi.MgSfgridSpec), I, I, I, D, D, D, I, _dp]
    lib.mg_adjoint_params.argtypes = [V, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(I)]
    lib.mg_adjoint_hvp.argtypes = [V, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.mg_sf_tasos_generate.argtypes = [V, I, C.POINTER(capi.MgSfgridSpec), I, I, I, D, D, D, D]
    lib.mg_sf_tasos_share.argtypes = [V, V]
    lib.mg_set_md_graphs.argtypes = [V, I]
    lib.mg_set_kspace_overlap.argtypes = [V, I]
    lib.mg_set_kspace_tensor.argtypes = [V, I]
    lib.mg_set_wait_limit.argtypes = [C.c_longlong]
    lib.mg_get_md_graphs.argtypes = [V, C.POINTER(I), C.POINTER(I)]
    lib.mg_autotune.argtypes = [V, _dp, _dp, _dp, I, C.POINTER(capi.MgTuning)]
    lib.mg_set_tuning.argtypes = [V, C.POINTER(capi.MgTuning)]
    lib.mg_get_tuning.argtypes = [V, C.POINTER(capi.MgTuning)]
    lib.mg_traj_open.argtypes = [V, C.c_char_p, I, C.c_char_p]
    lib.mg_traj_close.argtypes = [V, C.POINTER(C.c_longlong)]
    lib.mg_checkpoint_save.argtypes = [C.c_char_p, C.POINTER(capi.MgCheckpoint)]
    lib.mg_checkpoint_load.argtypes = [C.c_char_p, C.POINTER(capi.MgCheckpoint), I]
    lib.mg_checkpoint_apply.argtypes = [V, C.POINTER(capi.MgCheckpoint)]
    lib.mg_npt_run.argtypes = [V, C.POINTER(capi.MgNptParams), I, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                               C.POINTER(capi.MgNptState), _dp]
    lib.mg_siman_run.argtypes = [V, C.POINTER(capi.MgSimanParams), _dp, _dp, _dp, _dp, _dp, _dp,
                                 C.POINTER(capi.MgMdState), C.POINTER(I), _dp]
    lib.mg_siman_stage_count.argtypes = [D, D, D, I]
    lib.mg_siman_stage_count.restype = I
    lib.mg_force_match.argtypes = [V, _dp, _dp, _dp, _dp, _dp, _dp, D, _dp, _dp, _dp, _dp, C.POINTER(I)]
    _lib = lib
    return lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class Engine:
    """One system on one GPU."""

    def __init__(self, system: System, precision: str = "mixed", skin: float = 0.0, device: int = 0,
                 params: capi.MgParams | None = None):
        self.lib = load_library()
        self.system = system
        self.n = system.natom
        opt = MgOptions()
        self.lib.mg_options_default(C.byref(opt))
        opt.precision = PREC[precision]
        opt.skin = skin
        opt.device = device
        self.ctx = C.c_void_p()
        st = self.lib.mg_create(C.byref(self.ctx), C.byref(opt))
        if st != MG_OK:
            raise EngineError(st, "mg_create failed (an sm_103 GPU is required)")
        self.precision = precision
        self._pack = SpeciesPack(system)
        self.params = params if params is not None else capi.system_params(system)
        self._check(self.lib.mg_set_params(self.ctx, C.byref(self.params)))
        self._check(self.lib.mg_set_topology(self.ctx, self._pack.n, self._pack.array))
        self._check(self.lib.mg_set_box(self.ctx, *(float(v) for v in system.box)))
        self._load_solid(system)

    def _check(self, st: int) -> int:
        if st != MG_OK:
            raise EngineError(st, self.lib.mg_last_error(self.ctx).decode(errors="replace"))
        return st

    def _load_solid(self, s: System) -> None:
        if s.sf_type == SF_TASOS:
            for i, g in enumerate(s.tasos):
                v = np.ascontiguousarray(g.values, dtype=np.float64)
                self._check(self.lib.mg_sf_tasos_set_grid(self.ctx, i + 1, g.nx, g.ny, g.nz, g.hx, g.hy, g.hz,
                                                          g.cuc, _p(v)))
        elif s.sf_type == SF_HYPERGEO:
            t = np.ascontiguousarray(np.asarray(s.tube_xy_r, dtype=np.float64).T)
            self._check(self.lib.mg_sf_hypergeo_set(self.ctx, t.shape[1], _p(t[0]), _p(t[1]), _p(t[2]),
                                                    s.solid_sigma, s.solid_epsilon, s.const_3pisq_theta))
        elif s.sf_type == SF_ATOM_EXPLICIT:
            t = np.ascontiguousarray(np.asarray(s.solid_xyz, dtype=np.float64).T)
            self._check(self.lib.mg_sf_atom_explicit_set(self.ctx, t.shape[1], _p(t[0]), _p(t[1]), _p(t[2]),
                                                         s.solid_sigma, s.solid_epsilon))
        elif s.sf_type == SF_MY_INTERP:
            for i, g in enumerate(s.myinterp):
                c = np.ascontiguousarray(g.coeff, dtype=np.float64)
                self._check(self.lib.mg_sf_myinterp_set(self.ctx, i, g.ncx, g.ncy, g.ncz, *g.itvl, g.xmin, g.ymin,
                                                        g.zmax, _p(c)))

    def set_box(self, lx: float, ly: float, lz: float, params: capi.MgParams | None = None) -> None:
        if params is not None:
            self.params = params
            self._check(self.lib.mg_set_params(self.ctx, C.byref(params)))
        self._check(self.lib.mg_set_box(self.ctx, lx, ly, lz))

    def set_params(self, params: capi.MgParams) -> None:
        self.params = params
        self._check(self.lib.mg_set_params(self.ctx, C.byref(params)))

    def set_stream(self, stream_handle: int) -> None:
        self._check(self.lib.mg_set_stream(self.ctx, C.c_void_p(stream_handle)))

    def set_timing(self, on: bool) -> None:
        self._check(self.lib.mg_set_timing(self.ctx, 1 if on else 0))

    def compute(self, x=None, y=None, z=None, terms: int = TERMS_ALL, allow_nonfinite: bool = False):
        """Forces (long [3,n], short [3,n]) and energies for positions on the host."""
        s = self.system
        x = np.ascontiguousarray(s.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(s.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(s.z if z is None else z, dtype=np.float64)
        fl = np.zeros((3, self.n))
        fs = np.zeros((3, self.n))
        e = MgEnergies()
        st = self.lib.mg_compute(self.ctx, _p(x), _p(y), _p(z), terms, _p(fl[0]), _p(fl[1]), _p(fl[2]),
                                 _p(fs[0]), _p(fs[1]), _p(fs[2]), C.byref(e))
        if not (allow_nonfinite and st == MG_ERR_NONFINITE):
            self._check(st)
        return fl, fs, e.as_dict()

    def compute_into(self, x: np.ndarray, y: np.ndarray, z: np.ndarray, fl: np.ndarray, fs: np.ndarray,
                     terms: int = TERMS_ALL) -> dict:
        """Host-buffer call with caller-owned (e.g. pinned) arrays; fl, fs are [3, n]."""
        e = MgEnergies()
        self._check(self.lib.mg_compute(self.ctx, _p(x), _p(y), _p(z), terms, _p(fl[0]), _p(fl[1]), _p(fl[2]),
                                        _p(fs[0]), _p(fs[1]), _p(fs[2]), C.byref(e)))
        return e.as_dict()

    def compute_device(self, dx: int, dy: int, dz: int, dfl, dfs, terms: int = TERMS_ALL) -> dict:
        """Device pointers in (x, y, z) and out (each force block a [3][n] FP64 array)."""
        n = self.n
        e = MgEnergies()
        fl = [dfl, dfl + 8 * n, dfl + 16 * n] if dfl else [None] * 3
        fs = [dfs, dfs + 8 * n, dfs + 16 * n] if dfs else [None] * 3
        self._check(self.lib.mg_compute_device(self.ctx, dx, dy, dz, terms, *fl, *fs, C.byref(e)))
        return e.as_dict()

    def md_run(self, nsteps: int, md: dict, v, x=None, y=None, z=None, state: dict | None = None):
        """nsteps of the reference's integrator on the device (mg_md_run): md holds the
        mg_md_params fields (mspms2_gb300.system.md_params), v the [3, n] start velocities.
        Returns (positions [3, n], velocities [3, n], state dict, log [(nsteps+1), 12])."""
        s = self.system
        pos = np.ascontiguousarray(np.stack([s.x if x is None else x, s.y if y is None else y,
                                             s.z if z is None else z]), dtype=np.float64)
        vel = np.ascontiguousarray(v, dtype=np.float64).copy()
        st = capi.MgMdState(**(state or {}))
        log = np.zeros((nsteps + 1, capi.MD_LOG))
        mp = capi.MgMdParams.from_dict(md)
        self._check(self.lib.mg_md_run(self.ctx, C.byref(mp), nsteps, _p(pos[0]), _p(pos[1]), _p(pos[2]),
                                       _p(vel[0]), _p(vel[1]), _p(vel[2]), C.byref(st), _p(log)))
        return pos, vel, st.as_dict(), log

    def class_params(self):
        """(epsilon, sigma, charge) per site class: one class per site of each species
        template, numbered species by species (the order of mg_adjoint_params)."""
        sp = self.system.species
        return (np.concatenate([np.asarray(t.epsilon, float) for t in sp]),
                np.concatenate([np.asarray(t.sigma, float) for t in sp]),
                np.concatenate([np.asarray(t.charge, float) for t in sp]))

    def set_class_params(self, eps, sigma, charge) -> None:
        """Replaces the templates' epsilon, sigma and charge (arrays over the site classes)
        and uploads the topology again."""
        eps, sigma, charge = (np.asarray(a, dtype=np.float64).ravel() for a in (eps, sigma, charge))
        new, off = [], 0
        for t in self.system.species:
            k = t.natom
            new.append(dataclasses.replace(t, epsilon=eps[off:off + k].copy(), sigma=sigma[off:off + k].copy(),
                                           charge=charge[off:off + k].copy()))
            off += k
        if off != len(eps) or off != len(sigma) or off != len(charge):
            raise ValueError(f"expected {off} site classes")
        self.system = dataclasses.replace(self.system, species=new)
        self._pack = SpeciesPack(self.system)
        self._check(self.lib.mg_set_topology(self.ctx, self._pack.n, self._pack.array))

    def adjoint_params(self, g, x=None, y=None, z=None):
        """dL/d(epsilon, sigma, charge) per site class for g = dL/dF_long ([3, n]) at the
        given positions (mg_adjoint_params). Returns three arrays over the classes."""
        s = self.system
        x = np.ascontiguousarray(s.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(s.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(s.z if z is None else z, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64).reshape(3, self.n)
        nclass = sum(t.natom for t in s.species)
        ge, gs, gq = np.zeros(nclass), np.zeros(nclass), np.zeros(nclass)
        k = C.c_int(0)
        self._check(self.lib.mg_adjoint_params(self.ctx, _p(x), _p(y), _p(z), _p(g[0]), _p(g[1]), _p(g[2]),
                                               _p(ge), _p(gs), _p(gq), C.byref(k)))
        assert k.value == nclass
        return ge, gs, gq

    def force_match(self, target, scale=None, x=None, y=None, z=None):
        """(loss, (dL/d eps, dL/d sigma, dL/d q) per class) for L = scale * sum (F_long - target)^2
        (mg_force_match); scale defaults to 1 / (3 n), the mean squared force error."""
        s = self.system
        x = np.ascontiguousarray(s.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(s.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(s.z if z is None else z, dtype=np.float64)
        t = np.ascontiguousarray(target, dtype=np.float64).reshape(3, self.n)
        nclass = sum(sp.natom for sp in s.species)
        ge, gs, gq = np.zeros(nclass), np.zeros(nclass), np.zeros(nclass)
        loss = C.c_double(0.0)
        k = C.c_int(0)
        sc = 1.0 / (3 * self.n) if scale is None else float(scale)
        self._check(self.lib.mg_force_match(self.ctx, _p(x), _p(y), _p(z), _p(t[0]), _p(t[1]), _p(t[2]), sc,
                                            C.byref(loss), _p(ge), _p(gs), _p(gq), C.byref(k)))
        return loss.value, (ge, gs, gq)

    def hessian_vector(self, v, x=None, y=None, z=None):
        """H v = -(dF_long/dr) v ([3, n]) at the given positions (mg_adjoint_hvp)."""
        s = self.system
        x = np.ascontiguousarray(s.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(s.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(s.z if z is None else z, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(3, self.n)
        h = np.zeros((3, self.n))
        self._check(self.lib.mg_adjoint_hvp(self.ctx, _p(x), _p(y), _p(z), _p(v[0]), _p(v[1]), _p(v[2]),
                                            _p(h[0]), _p(h[1]), _p(h[2])))
        return h

    def sf_tasos_generate(self, type_id: int, spec: dict, nx: int, ny: int, nz: int, h, cuc: float) -> None:
        """Evaluates Tasos table type_id (1-based) on the device into the engine
        (mg_sf_tasos_generate); spec as for sfgrid_tasos."""
        c, _keep = _sfgrid_spec(spec)
        self._check(self.lib.mg_sf_tasos_generate(self.ctx, type_id, C.byref(c), nx, ny, nz, float(h[0]), float(h[1]),
                                                  float(h[2]), float(cuc)))

    def sf_tasos_share(self, other: "Engine") -> None:
        """Use the Tasos tables of another engine (same device and precision) without a copy
        (mg_sf_tasos_share)."""
        self._check(self.lib.mg_sf_tasos_share(self.ctx, other.ctx))

    def set_kspace_overlap(self, enable: bool) -> None:
        """Reciprocal space on a second stream beside the list and pairs (default) or in line."""
        self._check(self.lib.mg_set_kspace_overlap(self.ctx, 1 if enable else 0))

    def set_kspace_tensor(self, enable: bool) -> None:
        """Structure factors on the tensor cores (default) or on the CUDA cores (mixed path)."""
        self._check(self.lib.mg_set_kspace_tensor(self.ctx, 1 if enable else 0))

    def set_md_graphs(self, enable: bool) -> None:
        """Whole integrator steps as a replayed CUDA graph (default) or step by step."""
        self._check(self.lib.mg_set_md_graphs(self.ctx, 1 if enable else 0))

    def md_graph_steps(self) -> int:
        """Steps the last integrator run replayed as a graph (0: it ran step by step)."""
        en, last = C.c_int(), C.c_int()
        self._check(self.lib.mg_get_md_graphs(self.ctx, C.byref(en), C.byref(last)))
        return last.value

    def autotune(self, x=None, y=None, z=None, terms: int = TERMS_ALL) -> dict:
        """Picks the launch geometry (cell size, cluster size, threads per site of the
        k-space force pass) by timing evaluations at these positions (mg_autotune)."""
        s = self.system
        x = np.ascontiguousarray(s.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(s.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(s.z if z is None else z, dtype=np.float64)
        t = capi.MgTuning()
        self._check(self.lib.mg_autotune(self.ctx, _p(x), _p(y), _p(z), terms, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, cell_scale: float = 1.0, zcap_scale: float = 1.0, kforce_threads: int = 4) -> None:
        t = capi.MgTuning(cell_scale=cell_scale, zcap_scale=zcap_scale, kforce_threads=kforce_threads)
        self._check(self.lib.mg_set_tuning(self.ctx, C.byref(t)))

    def tuning(self) -> dict:
        t = capi.MgTuning()
        self._check(self.lib.mg_get_tuning(self.ctx, C.byref(t)))
        return t.as_dict()

    def traj_open(self, path: str, every: int, names=None) -> None:
        """Attaches the reference's trajectory file (mg_traj_open): the integrators then
        write a frame before their first step and every `every` steps."""
        names = names if names is not None else [nm for sp in self.system.species for nm in sp.atom_names]
        buf = b"".join(str(nm).encode()[:5].ljust(5, b"\0") for nm in names)
        self._check(self.lib.mg_traj_open(self.ctx, os.fsencode(path), every, buf))

    def traj_close(self) -> int:
        """Flushes and closes the trajectory file; returns the number of frames."""
        k = C.c_longlong(0)
        self._check(self.lib.mg_traj_close(self.ctx, C.byref(k)))
        return k.value

    def checkpoint_apply(self, ck: dict) -> None:
        """The box of a loaded checkpoint (mg_checkpoint_apply): caches keyed on the box
        are dropped."""
        c, _keep = checkpoint_struct(ck)
        self._check(self.lib.mg_checkpoint_apply(self.ctx, C.byref(c)))

    def npt_run(self, nsteps: int, npt: dict, v, state: dict, box=None, x=None, y=None, z=None):
        """nsteps of the reference's npt_respa on the device (mg_npt_run): npt holds the
        mg_npt_params fields (mspms2_gb300.system.npt_params), state vts, vbs, rts
        (system.npt_state0 for a new run). Returns (positions [3, n], velocities [3, n],
        box [3], state, log [(nsteps+1), 12])."""
        s = self.system
        pos = np.ascontiguousarray(np.stack([s.x if x is None else x, s.y if y is None else y,
                                             s.z if z is None else z]), dtype=np.float64)
        vel = np.ascontiguousarray(v, dtype=np.float64).copy()
        bx = np.ascontiguousarray(s.box if box is None else box, dtype=np.float64).copy()
        st = capi.MgNptState(**{k: state[k] for k in ("vts", "vbs", "rts")})
        log = np.zeros((nsteps + 1, capi.MD_LOG))
        self._check(self.lib.mg_npt_run(self.ctx, C.byref(capi.MgNptParams.from_dict(npt)), nsteps, _p(pos[0]),
                                        _p(pos[1]), _p(pos[2]), _p(vel[0]), _p(vel[1]), _p(vel[2]), _p(bx),
                                        C.byref(st), _p(log)))
        return pos, vel, bx, st.as_dict(), log

    def siman_run(self, md: dict, sched: dict, x=None, y=None, z=None, state: dict | None = None):
        """The reference's simulated annealing on the device (mg_siman_run): md holds the
        mg_md_params fields (scheme NVT), sched t_initial, t_min, mu_t, n_tries, max_stages
        and seed. Returns (positions [3, n], velocities [3, n], state, stage log [nstages, 8])."""
        s = self.system
        pos = np.ascontiguousarray(np.stack([s.x if x is None else x, s.y if y is None else y,
                                             s.z if z is None else z]), dtype=np.float64)
        vel = np.zeros((3, self.n))
        st = capi.MgMdState(**(state or {}))
        sp = capi.MgSimanParams.from_dict(md, sched)
        log = np.zeros((max(1, sched["max_stages"]), capi.SIMAN_LOG))
        k = C.c_int(0)
        self._check(self.lib.mg_siman_run(self.ctx, C.byref(sp), _p(pos[0]), _p(pos[1]), _p(pos[2]), _p(vel[0]),
                                          _p(vel[1]), _p(vel[2]), C.byref(st), C.byref(k), _p(log)))
        return pos, vel, st.as_dict(), log[:k.value]

    def stats(self) -> dict:
        st = MgStats()
        self._check(self.lib.mg_get_stats(self.ctx, C.byref(st)))
        return {"pairs_within_cutoff": st.pairs_within_cutoff, "cluster_pairs": st.cluster_pairs,
                "nclusters": st.nclusters, "kvectors": st.kvectors, "list_rebuilt": st.list_rebuilt,
                "list_builds": st.list_builds, "kernel_ms": list(st.kernel_ms),
                "kernel_launches": st.kernel_launches}

    def device_flags(self) -> int:
        f = C.c_uint()
        self._check(self.lib.mg_get_device_flags(self.ctx, C.byref(f)))
        return f.value

    def debug_list(self):
        ncl, npairs, zcap = C.c_int(), C.c_longlong(), C.c_double()
        grid = (C.c_int * 3)()
        self._check(self.lib.mg_debug_get_list(self.ctx, C.byref(ncl), C.byref(npairs), grid, C.byref(zcap),
                                               None, None, None))
        cl = np.zeros(ncl.value * 8, np.int32)
        pairs = np.zeros(2 * npairs.value, np.int32)
        shifts = np.zeros(3 * npairs.value, np.int32)
        ip = C.POINTER(C.c_int)
        self._check(self.lib.mg_debug_get_list(self.ctx, C.byref(ncl), C.byref(npairs), grid, C.byref(zcap),
                                               cl.ctypes.data_as(ip), pairs.ctypes.data_as(ip),
                                               shifts.ctypes.data_as(ip)))
        return {"grid": list(grid), "zcap": zcap.value, "clusters": cl.reshape(-1, 8),
                "pairs": pairs.reshape(-1, 2), "shifts": shifts.reshape(-1, 3)}

    def close(self) -> None:
        if getattr(self, "ctx", None) and self.ctx.value:
            self.lib.mg_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def set_wait_limit(polls: int) -> None:
    """Bound of each on-chip pipeline wait of the tensor-core S(k) pass, process-wide
    (mg_set_wait_limit); a negative value restores the default."""
    st = load_library().mg_set_wait_limit(int(polls))
    if st != MG_OK:
        raise EngineError(st, "mg_set_wait_limit")


def _sfgrid_spec(spec: dict):
    atoms = np.ascontiguousarray(np.asarray(spec["atoms"], dtype=np.float64).T)
    m = capi.MgSfgridSpec(nsolid=atoms.shape[1], sx=_p(atoms[0]), sy=_p(atoms[1]), sz=_p(atoms[2]),
                          uclx=spec["ucl"][0], ucly=spec["ucl"][1], uclz=spec["ucl"][2], f_sigma=spec["f_sigma"],
                          f_epsilon=spec["f_epsilon"], s_sigma=spec["s_sigma"], s_epsilon=spec["s_epsilon"],
                          rcuton=spec["rcuton"], rcutoff=spec["rcutoff"], lj_switch=int(spec["lj_switch"]))
    return m, atoms


def sfgrid_sfgridgen(spec: dict, itvl: float, precision: str = "fp64", device: int = 0):
    """The grids of the reference's tools/sfgridgen.c, computed on the GPU
    (mg_sfgrid_sfgridgen): returns (dims, out[13, N])."""
    lib = load_library()
    m, keep = _sfgrid_spec(spec)
    dims = (C.c_int * 3)()
    st = lib.mg_sfgrid_sfgridgen(device, C.byref(m), itvl, PREC[precision], dims, None)
    if st != MG_OK:
        raise EngineError(st, "mg_sfgrid_sfgridgen")
    out = np.zeros((13, dims[0] * dims[1] * dims[2]))
    st = lib.mg_sfgrid_sfgridgen(device, C.byref(m), itvl, PREC[precision], dims, _p(out))
    if st != MG_OK:
        raise EngineError(st, "mg_sfgrid_sfgridgen")
    return tuple(dims), out


def sfgrid_tasos(spec: dict, nx: int, ny: int, nz: int, h, precision: str = "fp64", device: int = 0):
    """A Tasos table (F, Dx, Dy, Dz, Dxy, Dxz, Dyz, Dxyz per node, K and A) computed on the
    GPU (mg_sfgrid_tasos): returns values[nz, ny, nx, 8]."""
    lib = load_library()
    m, keep = _sfgrid_spec(spec)
    out = np.zeros((nz, ny, nx, 8))
    st = lib.mg_sfgrid_tasos(device, C.byref(m), nx, ny, nz, h[0], h[1], h[2], PREC[precision], _p(out))
    if st != MG_OK:
        raise EngineError(st, "mg_sfgrid_tasos")
    return out


def hmc_batch(hp: dict, natom, box, x, y, z, nmoves: int, move0: int = 0, device: int = 0):
    """nmoves canonical HMC moves of every Lennard-Jones replica in one launch
    (mg_hmc_batch). natom[r], box[r] per replica; x/y/z hold all replicas one after
    another and are returned updated. Returns (x, y, z, accepted[r], energy[r],
    dh[r, nmoves])."""
    lib = load_library()
    natom = np.ascontiguousarray(natom, dtype=np.int32)
    box = np.ascontiguousarray(box, dtype=np.float64)
    x, y, z = (np.ascontiguousarray(v, dtype=np.float64).copy() for v in (x, y, z))
    nrep = len(natom)
    acc = np.zeros(nrep, np.int32)
    energy = np.zeros(nrep)
    dh = np.zeros((nrep, max(nmoves, 1)))
    p = capi.MgHmcParams(**hp)
    st = lib.mg_hmc_batch(device, C.byref(p), nrep, natom.ctypes.data_as(C.POINTER(C.c_int)), _p(box), _p(x), _p(y),
                          _p(z), nmoves, move0, acc.ctypes.data_as(C.POINTER(C.c_int)), _p(dh), _p(energy))
    if st != MG_OK:
        raise EngineError(st, "mg_hmc_batch")
    return x, y, z, acc, energy, dh[:, :nmoves]


def siman_batch(sp: dict, natom, box, x, y, z, device: int = 0):
    """Simulated annealing of every Lennard-Jones replica in one launch
    (mg_siman_batch). natom[r], box[r] per replica; x/y/z hold all replicas one after
    another and are returned annealed. Returns (x, y, z, log[r, stage, 5]) with the
    columns of capi.SIMAN_BATCH_LOG_NAMES at each stage end."""
    lib = load_library()
    natom = np.ascontiguousarray(natom, dtype=np.int32)
    box = np.ascontiguousarray(box, dtype=np.float64)
    x, y, z = (np.ascontiguousarray(v, dtype=np.float64).copy() for v in (x, y, z))
    nrep = len(natom)
    p = capi.MgSimanBatchParams(**sp)
    log = np.zeros((nrep, max(p.max_stages, 1), capi.SIMAN_BATCH_LOG))
    nst = C.c_int(0)
    st = lib.mg_siman_batch(device, C.byref(p), nrep, natom.ctypes.data_as(C.POINTER(C.c_int)), _p(box), _p(x),
                            _p(y), _p(z), C.byref(nst), _p(log))
    if st != MG_OK:
        raise EngineError(st, "mg_siman_batch")
    k = nst.value
    # the library writes [r][stage] with stage < k; rows are k long
    log = log.reshape(-1)[:nrep * k * capi.SIMAN_BATCH_LOG].reshape(nrep, k, capi.SIMAN_BATCH_LOG).copy()
    return x, y, z, log


def checkpoint_struct(ck: dict):
    """mg_checkpoint of a dict (positions/velocities [natom] arrays, the scalars, counters);
    returns the struct and the arrays that back its pointers."""
    arrs = {k: np.ascontiguousarray(ck[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
    c = capi.MgCheckpoint()
    c.natom = len(arrs["x"])
    for k, a in arrs.items():
        setattr(c, k, _p(a))
    for k in capi.CHECKPOINT_SCALARS:
        setattr(c, k, float(ck.get(k, 0.0)))
    c.equilibrium = int(ck.get("equilibrium", 0))
    c.nframe = int(ck.get("nframe", 0))
    c.istep = int(ck.get("istep", 0))
    for i, v in enumerate(ck.get("counts", [0] * capi.NCOUNTS)):
        c.counts[i] = int(v)
    for i, v in enumerate(ck.get("accum", [0.0] * capi.NCOUNTS)):
        c.accum[i] = float(v)
    return c, arrs


def checkpoint_save(path: str, ck: dict) -> None:
    """Writes the reference's checkpoint file (saveit layout) through mg_checkpoint_save."""
    c, _keep = checkpoint_struct(ck)
    st = load_library().mg_checkpoint_save(os.fsencode(path), C.byref(c))
    if st != MG_OK:
        raise EngineError(st, f"cannot write {path}")


def checkpoint_load(path: str, natom: int, with_counters: bool = True) -> dict:
    """Reads the reference's checkpoint file (loadit) through mg_checkpoint_load."""
    ck = {k: np.zeros(natom) for k in ("x", "y", "z", "vx", "vy", "vz")}
    c, arrs = checkpoint_struct(ck)
    st = load_library().mg_checkpoint_load(os.fsencode(path), C.byref(c), 1 if with_counters else 0)
    if st != MG_OK:
        raise EngineError(st, f"cannot read {path}")
    out = dict(arrs)
    for k in capi.CHECKPOINT_SCALARS:
        out[k] = getattr(c, k)
    out.update(equilibrium=c.equilibrium, nframe=c.nframe, istep=c.istep, counts=list(c.counts),
               accum=list(c.accum))
    return out


def derive(system: System) -> dict:
    return derive_params(system)
