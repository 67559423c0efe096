"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and the
`--impl reference` arm) import this module; it is the checker, never the product.
`run_reference_dir` runs the compiled reference (oracle/_ref/mspms_ref_force) when it
exists; `Oracle` runs the C restatement (oracle/liboracle.so).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from mspms2_gb300.capi import (ENERGY_NAMES, MD_LOG, SIMAN_LOG, MgEnergies, MgHmcParams, MgMdParams, MgMdState,
                               MgNptParams, MgNptState, MgParams, MgSimanParams, MgSpecies, SpeciesPack,
                               system_params)
from mspms2_gb300.system import System, write_reference_dir

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "mspms_ref_force")

_dp = C.POINTER(C.c_double)


class OrcTasos(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("hx", C.c_double),
                ("hy", C.c_double), ("hz", C.c_double), ("cuc", C.c_double), ("values", _dp),
                ("min_pe", C.c_double)]


class OrcMyInterp(C.Structure):
    _fields_ = [("ncx", C.c_int), ("ncy", C.c_int), ("ncz", C.c_int), ("itvl_x", C.c_double),
                ("itvl_y", C.c_double), ("itvl_z", C.c_double), ("xmin", C.c_double),
                ("ymin", C.c_double), ("zmax", C.c_double), ("coeff", _dp)]


class OrcSystem(C.Structure):
    _fields_ = [("nspecies", C.c_int), ("sp", C.POINTER(MgSpecies)), ("p", MgParams),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("ntasos", C.c_int), ("tasos", C.POINTER(OrcTasos)),
                ("ntube", C.c_int), ("tube_x", _dp), ("tube_y", _dp), ("tube_r", _dp),
                ("solid_sigma", C.c_double), ("solid_epsilon", C.c_double),
                ("const_3pisq_theta", C.c_double),
                ("nsolid", C.c_int), ("solid_x", _dp), ("solid_y", _dp), ("solid_z", _dp),
                ("nmyinterp", C.c_int), ("myinterp", C.POINTER(OrcMyInterp))]


class OrcWindow(C.Structure):
    _fields_ = [("imol_begin", C.c_int), ("imol_end", C.c_int), ("k_stride", C.c_int),
                ("skip_intra", C.c_int), ("k_offset", C.c_int)]


def build() -> str:
    src = [os.path.join(HERE, f) for f in ("mspms_oracle.c", "nblist_oracle.c", "md_oracle.c", "mspms_oracle.h",
                                           os.path.join("..", "include", "mspms2_gb300.h"))]
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_frclong.argtypes = [C.POINTER(OrcSystem), _dp, _dp, _dp, _dp, _dp, _dp,
                                     C.POINTER(MgEnergies), C.POINTER(OrcWindow)]
        _lib.orc_frclong_mt.argtypes = [C.POINTER(OrcSystem), _dp, _dp, _dp, _dp, _dp, _dp,
                                        C.POINTER(MgEnergies), C.c_int, C.c_int, C.c_int]
        _lib.orc_frcshort.argtypes = [C.POINTER(OrcSystem), _dp, _dp, _dp, _dp, _dp, _dp,
                                      C.POINTER(MgEnergies)]
        _lib.orc_count_pairs.argtypes = [C.POINTER(OrcSystem), _dp, _dp, _dp, C.c_double]
        _lib.orc_count_pairs.restype = C.c_longlong
        _lib.orc_tasos_force.argtypes = [C.POINTER(OrcTasos), C.c_uint, C.c_double, C.c_double,
                                         C.c_double, _dp, _dp]
        _lib.orc_md_run.argtypes = [C.POINTER(OrcSystem), C.POINTER(MgMdParams), C.c_int, _dp, _dp, _dp, _dp, _dp,
                                    _dp, C.POINTER(MgMdState), _dp]
        _lib.orc_hmc_replica.argtypes = [C.POINTER(OrcSystem), C.POINTER(MgHmcParams), C.c_int, C.c_int, C.c_int,
                                         _dp, _dp, _dp, C.POINTER(C.c_int), _dp, _dp]
        _lib.orc_npt_run.argtypes = [C.POINTER(OrcSystem), C.POINTER(MgNptParams), C.c_int, _dp, _dp, _dp, _dp, _dp,
                                     _dp, _dp, C.POINTER(MgNptState), _dp]
        _lib.orc_siman_run.argtypes = [C.POINTER(OrcSystem), C.POINTER(MgSimanParams), _dp, _dp, _dp, _dp, _dp, _dp,
                                       C.POINTER(MgMdState), C.POINTER(C.c_int), _dp]
        _lib.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        _lib.orc_philox4x32_10.restype = None
        _lib.orc_tasos_min_pe.argtypes = [C.POINTER(OrcTasos)]
        _lib.orc_tasos_min_pe.restype = C.c_double
        _lib.orc_nblist_build.argtypes = [_dp, _dp, _dp, C.c_int, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_longlong]
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Oracle:
    """The C restatement bound to one System."""

    def __init__(self, system: System, params: MgParams | None = None):
        self.system = system
        self.pack = SpeciesPack(system)
        self.keep = []
        s = OrcSystem()
        s.nspecies = self.pack.n
        s.sp = C.cast(self.pack.array, C.POINTER(MgSpecies))
        s.p = params if params is not None else system_params(system)
        s.lx, s.ly, s.lz = (float(v) for v in system.box)
        if system.tasos:
            arr = (OrcTasos * len(system.tasos))()
            for i, g in enumerate(system.tasos):
                v = np.ascontiguousarray(g.values, dtype=np.float64)
                self.keep.append(v)
                arr[i].nx, arr[i].ny, arr[i].nz = g.nx, g.ny, g.nz
                arr[i].hx, arr[i].hy, arr[i].hz, arr[i].cuc = g.hx, g.hy, g.hz, g.cuc
                arr[i].values = _ptr(v)
                arr[i].min_pe = float(v[..., 0].min())
            self.keep.append(arr)
            s.ntasos = len(system.tasos)
            s.tasos = C.cast(arr, C.POINTER(OrcTasos))
        if system.tube_xy_r is not None:
            t = np.ascontiguousarray(system.tube_xy_r.T, dtype=np.float64)
            self.keep.append(t)
            s.ntube = t.shape[1]
            s.tube_x, s.tube_y, s.tube_r = _ptr(t[0]), _ptr(t[1]), _ptr(t[2])
        s.solid_sigma, s.solid_epsilon = system.solid_sigma, system.solid_epsilon
        s.const_3pisq_theta = system.const_3pisq_theta
        if system.solid_xyz is not None:
            t = np.ascontiguousarray(system.solid_xyz.T, dtype=np.float64)
            self.keep.append(t)
            s.nsolid = t.shape[1]
            s.solid_x, s.solid_y, s.solid_z = _ptr(t[0]), _ptr(t[1]), _ptr(t[2])
        if system.myinterp:
            arr = (OrcMyInterp * len(system.myinterp))()
            for i, g in enumerate(system.myinterp):
                c = np.ascontiguousarray(g.coeff, dtype=np.float64)
                self.keep.append(c)
                arr[i].ncx, arr[i].ncy, arr[i].ncz = g.ncx, g.ncy, g.ncz
                arr[i].itvl_x, arr[i].itvl_y, arr[i].itvl_z = g.itvl
                arr[i].xmin, arr[i].ymin, arr[i].zmax = g.xmin, g.ymin, g.zmax
                arr[i].coeff = _ptr(c)
            self.keep.append(arr)
            s.nmyinterp = len(system.myinterp)
            s.myinterp = C.cast(arr, C.POINTER(OrcMyInterp))
        self.s = s

    def frclong(self, x=None, y=None, z=None, window: OrcWindow | None = None):
        sysm = self.system
        x = np.ascontiguousarray(sysm.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(sysm.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(sysm.z if z is None else z, dtype=np.float64)
        n = len(x)
        f = np.zeros((3, n))
        e = MgEnergies()
        flags = lib().orc_frclong(C.byref(self.s), _ptr(x), _ptr(y), _ptr(z), _ptr(f[0]), _ptr(f[1]),
                                  _ptr(f[2]), C.byref(e), C.byref(window) if window else None)
        return f, e.as_dict(), flags

    def frclong_mt(self, threads: int, x=None, y=None, z=None, slice_: int = 0, nslices: int = 1):
        """frclong on `threads` host threads (orc_frclong_mt): the same terms, with the pair
        rows and k-vectors shared out; only the order of the sums differs from frclong().
        slice_/nslices > 1 evaluate one of nslices equal shares of the pair and k-vector work."""
        sysm = self.system
        x = np.ascontiguousarray(sysm.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(sysm.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(sysm.z if z is None else z, dtype=np.float64)
        n = len(x)
        f = np.zeros((3, n))
        e = MgEnergies()
        flags = lib().orc_frclong_mt(C.byref(self.s), _ptr(x), _ptr(y), _ptr(z), _ptr(f[0]), _ptr(f[1]),
                                     _ptr(f[2]), C.byref(e), int(threads), int(slice_), int(nslices))
        return f, e.as_dict(), flags

    def frcshort(self, x=None, y=None, z=None):
        sysm = self.system
        x = np.ascontiguousarray(sysm.x if x is None else x, dtype=np.float64)
        y = np.ascontiguousarray(sysm.y if y is None else y, dtype=np.float64)
        z = np.ascontiguousarray(sysm.z if z is None else z, dtype=np.float64)
        n = len(x)
        f = np.zeros((3, n))
        e = MgEnergies()
        err = lib().orc_frcshort(C.byref(self.s), _ptr(x), _ptr(y), _ptr(z), _ptr(f[0]), _ptr(f[1]),
                                 _ptr(f[2]), C.byref(e))
        d = e.as_dict()
        return f, {k: d[k] for k in ("ubond", "uangle", "udih", "uimp", "uintra", "virial_intra")}, err

    def md_run(self, nsteps: int, md: dict, v, state: dict | None = None):
        """The restated vver()/vver_nh_3() (oracle/md_oracle.c), same contract as
        Engine.md_run: (positions, velocities, state, log)."""
        sysm = self.system
        pos = np.ascontiguousarray(np.stack([sysm.x, sysm.y, sysm.z]), dtype=np.float64)
        vel = np.ascontiguousarray(v, dtype=np.float64).copy()
        st = MgMdState(**(state or {}))
        log = np.zeros((nsteps + 1, MD_LOG))
        lib().orc_md_run(C.byref(self.s), C.byref(MgMdParams.from_dict(md)), nsteps, _ptr(pos[0]), _ptr(pos[1]),
                         _ptr(pos[2]), _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), C.byref(st), _ptr(log))
        return pos, vel, st.as_dict(), log

    def hmc_replica(self, hp: dict, replica: int, move0: int, nmoves: int):
        """The restated canonical HMC moves of one replica (oracle/md_oracle.c): returns
        (positions [3, n], accepted, energy, dh[nmoves])."""
        sysm = self.system
        pos = np.ascontiguousarray(np.stack([sysm.x, sysm.y, sysm.z]), dtype=np.float64)
        acc = C.c_int()
        energy = C.c_double()
        dh = np.zeros(max(nmoves, 1))
        lib().orc_hmc_replica(C.byref(self.s), C.byref(MgHmcParams(**hp)), replica, move0, nmoves, _ptr(pos[0]),
                              _ptr(pos[1]), _ptr(pos[2]), C.byref(acc), _ptr(dh), C.byref(energy))
        return pos, acc.value, energy.value, dh[:nmoves]

    def npt_run(self, nsteps: int, npt: dict, v, box, state: dict):
        """The restated npt_respa (oracle/md_oracle.c), same contract as Engine.npt_run:
        (positions, velocities, box, state, log)."""
        sysm = self.system
        pos = np.ascontiguousarray(np.stack([sysm.x, sysm.y, sysm.z]), dtype=np.float64)
        vel = np.ascontiguousarray(v, dtype=np.float64).copy()
        bx = np.ascontiguousarray(box, dtype=np.float64).copy()
        st = MgNptState(**state)
        log = np.zeros((nsteps + 1, MD_LOG))
        rc = lib().orc_npt_run(C.byref(self.s), C.byref(MgNptParams.from_dict(npt)), nsteps, _ptr(pos[0]),
                               _ptr(pos[1]), _ptr(pos[2]), _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), _ptr(bx),
                               C.byref(st), _ptr(log))
        if rc != 0:
            raise RuntimeError(f"orc_npt_run failed ({rc})")
        return pos, vel, bx, st.as_dict(), log

    def siman_run(self, md: dict, sched: dict, state: dict | None = None):
        """The restated simulated annealing (oracle/md_oracle.c), same contract as
        Engine.siman_run: (positions, velocities, state, stage log)."""
        sysm = self.system
        pos = np.ascontiguousarray(np.stack([sysm.x, sysm.y, sysm.z]), dtype=np.float64)
        vel = np.zeros((3, sysm.natom))
        st = MgMdState(**(state or {}))
        log = np.zeros((max(1, sched["max_stages"]), SIMAN_LOG))
        k = C.c_int(0)
        rc = lib().orc_siman_run(C.byref(self.s), C.byref(MgSimanParams.from_dict(md, sched)), _ptr(pos[0]),
                                 _ptr(pos[1]), _ptr(pos[2]), _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), C.byref(st),
                                 C.byref(k), _ptr(log))
        if rc != 0:
            raise RuntimeError(f"orc_siman_run failed ({rc})")
        return pos, vel, st.as_dict(), log[:k.value]

    def count_pairs(self, r: float) -> int:
        s = self.system
        x, y, z = (np.ascontiguousarray(v, dtype=np.float64) for v in (s.x, s.y, s.z))
        return int(lib().orc_count_pairs(C.byref(self.s), _ptr(x), _ptr(y), _ptr(z), r * r))


def read_ref_output(fn: str):
    raw = open(fn, "rb").read()
    n = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    a = np.frombuffer(raw[4:], dtype=np.float64)
    fl = a[0:3 * n].reshape(3, n).copy()
    fs = a[3 * n:6 * n].reshape(3, n).copy()
    e = dict(zip(ENERGY_NAMES, a[6 * n:6 * n + 18]))
    dnames = ["rcutoffsq", "rcutonsq", "rcutoffelecsq", "roff2_minus_ron2_cube", "shift1", "shift4",
              "wolfvcon1", "wolfvcon2", "wolfvcon3", "wolffcon1", "wolffcon2", "bfactor_ewald",
              "vfactor_ewald", "twopi_lx", "twopi_ly", "twopi_lz", "twopi_over_3v", "kappa",
              "coulomb_prefactor", "boxlx", "boxly", "boxlz", "sigma_base", "epsilon_base"]
    d = dict(zip(dnames, a[6 * n + 18:6 * n + 42]))
    return fl, fs, e, d


def run_reference_md(path: str, nsteps: int, trj_every: int = 0) -> dict:
    """Run the compiled reference's own integrator for the input's ensemble (harness md
    mode, oracle/ref_harness.c) and parse its record. With trj_every > 0 the result also
    holds the bytes of the reference's trajectory file and of its checkpoint after the
    run ("trj", "sav")."""
    files = {}
    with tempfile.TemporaryDirectory() as td:
        out, md = os.path.join(td, "out.bin"), os.path.join(td, "md.bin")
        args = [REF_BIN, path, out, "0", "md", str(nsteps), md] + ([str(trj_every)] if trj_every > 0 else [])
        p = subprocess.run(args, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"reference md run failed: {p.stderr[-2000:]}")
        b = open(md, "rb").read()
        if trj_every > 0:
            for k, fn in (("trj", "trj.mspms"), ("sav", "sav.mspms")):
                files[k] = open(os.path.join(path, fn), "rb").read()
    n, nstep_inner, ens, ns = (int(v) for v in np.frombuffer(b[:16], np.int32))
    sc = np.frombuffer(b[16:112])
    off = 112
    start = np.frombuffer(b[off:off + 48 * n]).reshape(6, n).copy()
    off += 48 * n
    log = np.frombuffer(b[off:off + 96 * (ns + 1)]).reshape(ns + 1, 12).copy()
    off += 96 * (ns + 1)
    end = np.frombuffer(b[off:off + 48 * n]).reshape(6, n).copy()
    if ens == 2:  # NPT: npt_respa (src/nptnh.c:134)
        md = dict(nstep_inner=nstep_inner, delt=sc[0], treq=sc[1], qts=sc[2], qbs=sc[3], preq=sc[4],
                  lj_lrc=int(sc[5]), nfree=int(sc[6]))
        state = dict(vts=sc[7], vbs=sc[8], rts=sc[9], boxlx=sc[10], pljlrc=sc[11])
        return {"md": md, "state": state, "start": start, "log": log, "end": end, "nsteps": ns, "npt": True}
    md = dict(scheme=ens, nstep_inner=nstep_inner, delt=sc[0], treq=sc[1], qq=sc[2], qqs=sc[3], gg=sc[4],
              ggs=sc[5], nfree=int(sc[6]))
    state = dict(ps=sc[7], ss=sc[8], pss=sc[9], sss=sc[10])
    return {"md": md, "state": state, "start": start, "log": log, "end": end, "nsteps": ns, **files}


def run_reference_hmc(path: str, velocities, nstep_md: int) -> dict:
    """Canonical HMC moves through the compiled reference's own md_move() over vver()
    (harness hmc mode, oracle/ref_harness.c), move m starting from velocities[m] ([3, n])
    in place of velinit()'s draw. Returns per move the energies before ({ukin, uinter,
    uintra, ushift}), dH, the accept decision, the energies after, the energies and the
    positions of the proposal (after the last vver step, kept even on rejection) and the
    final positions."""
    v = np.ascontiguousarray(np.asarray(velocities, dtype=np.float64))
    nm, _, n = v.shape
    with tempfile.TemporaryDirectory() as td:
        out, hb, vb = os.path.join(td, "out.bin"), os.path.join(td, "hmc.bin"), os.path.join(td, "vel.bin")
        v.tofile(vb)
        p = subprocess.run([REF_BIN, path, out, "0", "hmc", str(nm), str(nstep_md), hb, vb], capture_output=True,
                           text=True)
        if p.returncode != 0:
            raise RuntimeError(f"reference hmc run failed: {p.stderr[-2000:]}")
        b = open(hb, "rb").read()
    n2, nm2, ns = (int(x) for x in np.frombuffer(b[:12], np.int32))
    assert n2 == n and nm2 == nm and ns == nstep_md
    rec = 8 * (12 + 6 * n)
    res = []
    for m in range(nm):
        a = np.frombuffer(b, np.float64, 12 + 6 * n, 12 + m * rec)
        res.append({"pre": a[:4].copy(), "dh": float(a[4]), "accept": bool(a[5]), "post": a[6:8].copy(),
                    "proposal_energies": a[8:12].copy(), "proposal": a[12:12 + 3 * n].reshape(3, n).copy(),
                    "final": a[12 + 3 * n:].reshape(3, n).copy()})
    return {"moves": res}


def hmc_velocities(hp: dict, replica: int, move: int, n: int):
    """The velocities mg_hmc_batch draws for one move of one replica ([3, n])."""
    v = np.zeros((3, n))
    L = lib()
    L.orc_hmc_velocities.argtypes = [C.POINTER(MgHmcParams), C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
    L.orc_hmc_velocities(C.byref(MgHmcParams(**hp)), replica, move, n, _ptr(v[0]), _ptr(v[1]), _ptr(v[2]))
    return v


SFGRIDGEN_BIN = os.path.join(HERE, "_ref", "sfgridgen")


def run_reference_sfgridgen(spec: dict, itvl: float):
    """Run the reference's tools/sfgridgen.c (built into oracle/_ref by build_ref.sh) on a
    spec (fluid/solid sigma and epsilon, rcuton, rcutoff, lj_switch, cell, atoms [n, 3])
    and return (dims, out[13, N]) as the tool writes them."""
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "grid.in")
        def r(v):
            return repr(float(v))
        with open(inp, "w") as f:
            f.write(f"F {r(spec['f_sigma'])} {r(spec['f_epsilon'])}\n")
            f.write(f"{r(itvl)} {r(spec['rcuton'])} {r(spec['rcutoff'])} {int(spec['lj_switch'])}\n")
            ucl = spec["ucl"]
            f.write(f"{len(spec['atoms'])} {r(ucl[0])} {r(ucl[1])} {r(ucl[2])}\n")
            f.write(f"{r(spec['s_sigma'])} {r(spec['s_epsilon'])}\n")
            for a in spec["atoms"]:
                f.write(f"C {r(a[0])} {r(a[1])} {r(a[2])}\n")
        p = subprocess.run([SFGRIDGEN_BIN, inp], cwd=td, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"sfgridgen failed: {p.stderr[-2000:]}")
        b = open(os.path.join(td, "out.sfgridgen"), "rb").read()
    head = np.frombuffer(b[:48])
    ints = np.frombuffer(b[48:64], np.int32)
    ntot, dims = int(ints[0]), tuple(int(v) for v in ints[1:4])
    out = np.frombuffer(b[88:88 + 13 * 8 * ntot]).reshape(13, ntot).copy()
    return dims, out, head


def reference_available() -> bool:
    return os.path.exists(REF_BIN) and os.access(REF_BIN, os.X_OK)


def run_reference_dir(path: str, repeat: int = 0):
    """Run the compiled reference on a directory of reference-format inputs."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.bin")
        p = subprocess.run([REF_BIN, path, out, str(repeat)], capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"reference failed: {p.stderr[-2000:]}")
        res = read_ref_output(out)
    timing = {}
    for tok in p.stdout.split():
        if "=" in tok:
            k, v = tok.split("=", 1)
            timing[k] = float(v)
    return res, timing


def run_reference_system(system: System, repeat: int = 0):
    with tempfile.TemporaryDirectory() as td:
        write_reference_dir(system, td)
        return run_reference_dir(td, repeat)


def nblist(x, y, z, box, rlist, ncx, ncy, small, zcap):
    """CPU cluster-pair list (same algorithm and FP64 op order as the GPU build)."""
    L = lib()
    L.orc_nblist_build2.argtypes = [_dp, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                                    C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.c_longlong]
    x, y, z = (np.ascontiguousarray(v, dtype=np.float64) for v in (x, y, z))
    n = len(x)
    ncl, npairs = C.c_int(), C.c_longlong()
    ip = C.POINTER(C.c_int)
    L.orc_nblist_build2(_ptr(x), _ptr(y), _ptr(z), n, *box, rlist, ncx, ncy, small, zcap, C.byref(ncl), None, 0,
                        C.byref(npairs), None, None, 0)
    cl = np.zeros(ncl.value * 8, np.int32)
    pairs = np.zeros(2 * npairs.value, np.int32)
    shifts = np.zeros(3 * npairs.value, np.int32)
    L.orc_nblist_build2(_ptr(x), _ptr(y), _ptr(z), n, *box, rlist, ncx, ncy, small, zcap, C.byref(ncl),
                        cl.ctypes.data_as(ip), len(cl), C.byref(npairs), pairs.ctypes.data_as(ip),
                        shifts.ctypes.data_as(ip), npairs.value)
    return {"clusters": cl.reshape(-1, 8), "pairs": pairs.reshape(-1, 2), "shifts": shifts.reshape(-1, 3)}
