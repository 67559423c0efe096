"""Generate the golden fixtures under tests/golden/ from the compiled reference.

Each case is a system written in the reference's own input format, run through
oracle/_ref/mspms_ref_force (the reference force layer built by oracle/build_ref.sh
from the reference checkout), and stored as <case>.npz with:
  the parsed system (mspms2_gb300.system.system_to_arrays),
  ref_fl[3,n], ref_fs[3,n]  forces of frclong() / frcshort(),
  ref_energies[18]          in mspms2_gb300.capi.ENERGY_NAMES order,
  ref_derived[24]           derived globals after init_vars().
The md_* cases hold trajectories of the reference's own integrators instead (vver_nh_3,
vver or npt_respa, run by the harness's md mode): md_int (scheme, nstep_inner, nfree,
nsteps[, lj_lrc]), md_real (delt, treq, qq, qqs, gg, ggs; NPT: delt, treq, Qts, Qbs,
preq), md_state0 (ps, ss, pss, sss; NPT: vts, vbs, rts, boxlx, pljlrc), md_v0[3,n] start
velocities (drawn by the reference's velinit), md_log[nsteps+1, 12] and md_end[6, n] (x,
y, z, vx, vy, vz after the last step); the system's positions are the start. A case with
trj_every also holds the bytes of the reference's trajectory file (ref_trj) and of its
checkpoint after the last step (ref_sav). The sfgrid_* cases
hold grids of the reference's tools/sfgridgen.c (atoms, cell, LJ parameters, dims and its
13 output arrays).
Two cases use the reference's shipped inputs (Examples/Water and the root example);
the rest are seeded synthetic systems chosen to reach every model switch.

Run from the repository root:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mspms2_gb300 import configs  # noqa: E402
from mspms2_gb300.system import (ELEC_EWALD, ELEC_NONE, ELEC_SIMPLE_COULOMB, ELEC_WOLF,  # noqa: E402
                                 GHOST_FULL, SF_ATOM_EXPLICIT, SF_HYPERGEO, SF_MY_INTERP, SF_TASOS,
                                 MyInterpGrid, Species, System, TasosGrid, read_reference_dir,
                                 system_to_arrays, tasos_dims, write_reference_dir)
from golden_systems import custom_molecule_system, lj_gas, tasos_test_grid  # noqa: E402
from oracle.pyoracle import (reference_available, run_reference_dir, run_reference_md,  # noqa: E402
                             run_reference_sfgridgen)

def _checkout() -> str:
    """The reference checkout: MSPMS2_REF, else the one oracle/build_ref.sh recorded."""
    ref = os.environ.get("MSPMS2_REF")
    rec = os.path.join(ROOT, "oracle", "_ref", "checkout")
    if not ref and os.path.exists(rec):
        ref = open(rec).read().strip()
    if not ref:
        sys.exit("set MSPMS2_REF to the reference checkout (or run oracle/build_ref.sh <checkout> first)")
    return ref


REF = _checkout()
OUT = os.path.dirname(os.path.abspath(__file__))


def cases():
    out = {}
    out["water_example"] = ("dir", os.path.join(REF, "Examples", "Water"))
    out["butane_root"] = ("dir", REF)
    c1 = configs.water_box(6, 18.6, 11, ELEC_WOLF, 0.2, 9.0, name="water_c1", site_jitter=0.04)
    out["water_wolf_216"] = ("sys", c1)
    w = configs.water_small(4, 14.0, seed=12, charge_type=ELEC_EWALD, kappa=0.35, rc=6.5, kmax=5, ksqmax=27)
    w.ewald_bc = 2
    w.name = "water_vacuum"
    out["water_ewald_vacuum"] = ("sys", w)
    out["water_ewald_512"] = ("sys", configs.water_small(8, 24.8, seed=13, charge_type=ELEC_EWALD,
                                                         kappa=0.3, rc=10.0, kmax=7, ksqmax=49))
    sc = configs.water_small(4, 14.0, seed=14, charge_type=ELEC_SIMPLE_COULOMB, rc=6.5)
    sc.name = "water_coulomb"
    out["water_simple_coulomb"] = ("sys", sc)
    st = configs.water_small(4, 13.0, seed=15, charge_type=ELEC_EWALD, kappa=0.35, rc=6.4, kmax=4, ksqmax=20)
    st.x = st.x - st.box[0] * np.floor(st.x / st.box[0])  # per-site wrap breaks molecules apart
    st.y = st.y - st.box[1] * np.floor(st.y / st.box[1])
    st.z = st.z - st.box[2] * np.floor(st.z / st.box[2])
    st.name = "water_wrapped"
    out["water_wrapped_ewald"] = ("sys", st)
    stw = configs.water_small(4, 13.0, seed=16, charge_type=ELEC_WOLF, kappa=0.25, rc=6.4)
    stw.x = stw.x - stw.box[0] * np.floor(stw.x / stw.box[0])
    stw.name = "water_wrapped_wolf"
    out["water_wrapped_wolf"] = ("sys", stw)
    bt = configs.butane_box(3, 16.0, seed=17, rc=7.9, charged=True, site_jitter=0.05)
    bt.charge_type = ELEC_EWALD
    bt.kappa = 0.3
    bt.kmax = (4, 4, 4)
    bt.ksqmax = 24
    bt.lj_switch = 1
    bt.rcuton = 6.5
    bt.name = "butane_switch"
    out["butane_ewald_switch"] = ("sys", bt)
    out["custom_wolf"] = ("sys", custom_molecule_system(18))
    cu = custom_molecule_system(19)
    cu.charge_type = ELEC_EWALD
    cu.kappa, cu.kmax, cu.ksqmax = 0.3, (4, 4, 4), 24
    cu.name = "custom_ewald"
    out["custom_ewald"] = ("sys", cu)
    lj = configs.lj_replica(500, seed=20)
    out["lj_fluid_500"] = ("sys", lj)
    tubes = np.array([[4.0, 4.0, 3.0], [10.5, 9.0, 2.5], [7.0, 12.0, 1.8]])

    def near_wall(p, tubes=tubes):
        return any(abs(np.hypot(p[0] - t[0], p[1] - t[1]) - t[2]) < 2.2 for t in tubes)
    hg = lj_gas(30, 14.0, seed=21, avoid=near_wall, sigma=2.5)
    hg.sf_type = SF_HYPERGEO
    hg.tube_xy_r = tubes
    hg.solid_sigma, hg.solid_epsilon = 3.4, 28.0
    hg.name = "hypergeo"
    out["sf_hypergeo"] = ("sys", hg)
    hl = lj_gas(20, 12.0, seed=22, sigma=2.5, avoid=lambda p: abs(np.hypot(p[0] - 6, p[1] - 6) - 2.0) < 1.5)
    hl.sf_type = SF_HYPERGEO
    hl.tube_xy_r = np.array([[6.0, 6.0, 2.0]])
    hl.solid_sigma, hl.solid_epsilon = 3.4, 28.0
    hl.compat = 0x7
    hl.name = "hypergeo_sum"
    out["sf_hypergeo_sum"] = ("sys", hl)
    solid = np.random.default_rng(24).uniform(0, 14.0, size=(30, 3))

    def near_solid(p, solid=solid):
        d = solid - p
        d -= 14.0 * np.rint(d / 14.0)
        return (d ** 2).sum(1).min() < 2.6 ** 2
    ae = lj_gas(20, 14.0, seed=23, avoid=near_solid, sigma=2.5)
    ae.sf_type = SF_ATOM_EXPLICIT
    ae.lj_switch = 1
    ae.rcuton = 5.0
    ae.solid_xyz = solid
    ae.solid_sigma, ae.solid_epsilon = 3.4, 28.0
    ae.name = "atom_explicit"
    out["sf_atom_explicit"] = ("sys", ae)
    ta = lj_gas(12, 12.0, seed=25, xy_range=(0.3, 3.7), sigma=1.0, eps=5.0)
    ta.sf_type = SF_TASOS
    ta.species[0].interp = np.array([1], np.int32)
    ta.tasos_cell = (4.0, 4.0, 2.4595, 1.0)
    ta.tasos = [tasos_test_grid(4.0, 4.0, 2.4595, 26)]
    ta.name = "tasos"
    out["sf_tasos"] = ("sys", ta)
    mi = lj_gas(12, 12.0, seed=27, xy_range=(0.2, 3.8), sigma=1.0, eps=5.0)
    mi.sf_type = SF_MY_INTERP
    mi.species[0].interp = np.array([0], np.int32)
    rng = np.random.default_rng(28)
    ncx, ncy, ncz = 4, 4, 3
    scale = np.array([1, .1, .1, .1, .01, .01, .01, .01, .01, .01] + [.001] * 10 + [1e-4] * 12)
    coeff = rng.normal(size=(4, 32, ncx * ncy * ncz)) * (50.0 * scale)[None, :, None]
    mi.myinterp = [MyInterpGrid(ncx, ncy, ncz, (1.0, 1.0, 1.0), 0.0, 0.0, 3.0, coeff)]
    mi.name = "myinterp"
    out["sf_myinterp"] = ("sys", mi)
    return out


def md_cases():
    """Trajectories of the reference's own integrators (harness md mode): case -> (system, nsteps)."""
    out = {}
    w = configs.water_box(6, 18.6, 11, ELEC_WOLF, 0.2, 9.0, name="md_water_nvt", site_jitter=0.04)
    w.delt_fs, w.nstep_inner, w.what_ensemble = 0.5, 2, 1
    out["md_water_nvt_216"] = (w, 10)
    lj = configs.lj_replica(500, seed=30)
    lj.treq_K, lj.delt_fs, lj.nstep_inner, lj.what_ensemble = 1.0, 0.005 * 851.0, 1, 0
    lj.name = "md_lj_nve"
    out["md_lj_nve_500"] = (lj, 10)
    e = configs.water_small(8, 24.8, seed=13, charge_type=ELEC_EWALD, kappa=0.3, rc=10.0, kmax=7, ksqmax=49)
    e.delt_fs, e.nstep_inner, e.what_ensemble = 2.0, 4, 1
    e.nh_qq, e.nh_qqs = 5000.0, 2000.0
    e.name = "md_water_ewald_respa"
    out["md_water_ewald_respa_512"] = (e, 5)
    # NPT (npt_respa): Wolf water with the LJ long-range correction, 2 inner steps; Ewald
    # water with 4 inner RESPA steps (the box, the k-vectors and the Ewald constants change
    # every inner step)
    pw = configs.water_box(6, 18.6, 17, ELEC_WOLF, 0.2, 9.0, name="md_water_npt", site_jitter=0.04)
    pw.delt_fs, pw.nstep_inner, pw.what_ensemble, pw.lj_lrc = 0.5, 2, 2, 1
    pw.preq_bar, pw.npt_qts, pw.npt_qbs = 1000.0, 2.0e4, 5.0e3
    out["md_water_npt_216"] = (pw, 10)
    pe = configs.water_small(8, 24.8, seed=19, charge_type=ELEC_EWALD, kappa=0.3, rc=10.0, kmax=7, ksqmax=49)
    pe.delt_fs, pe.nstep_inner, pe.what_ensemble = 1.0, 4, 2
    pe.preq_bar, pe.npt_qts, pe.npt_qbs = 1.0, 5.0e4, 2.0e3
    pe.name = "md_water_ewald_npt"
    out["md_water_ewald_npt_512"] = (pe, 5)
    # trajectory and checkpoint files of the reference's own writers: two species (LJ ions
    # with Ewald), NVT, a frame every 3 steps and the checkpoint after the last step
    ions = configs.ion_box(4, seed=23, kmax=4, ksqmax=16, rc=7.5, spacing=4.0, jitter=0.3)
    for sp, (eps, sig, q) in zip(ions.species, ((50.0, 2.6, 0.3), (120.0, 3.4, -0.3))):
        sp.epsilon, sp.sigma, sp.charge = np.array([eps]), np.array([sig]), np.array([q])
        sp.aw_input = sp.aw_input * 30.0  # ~18 amu
        sp.aw = sp.aw * 30.0
    ions.delt_fs, ions.nstep_inner, ions.what_ensemble = 1.0, 1, 1
    ions.nh_qq = ions.nh_qqs = 500.0
    ions.name = "md_ions_trj"
    out["md_ions_trj_64"] = (ions, 10, 3)
    return out


def read_sfgridgen_input(fn):
    """The reference's sfgridgen input format (tools/sfgridgen.c:111-121)."""
    lines = [ln.split() for ln in open(fn) if ln.strip()]
    f_sigma, f_eps = float(lines[0][1]), float(lines[0][2])
    itvl, ron, roff, sw = float(lines[1][0]), float(lines[1][1]), float(lines[1][2]), int(lines[1][3])
    n, ux, uy, uz = int(lines[2][0]), float(lines[2][1]), float(lines[2][2]), float(lines[2][3])
    s_sigma, s_eps = float(lines[3][0]), float(lines[3][1])
    atoms = np.array([[float(v) for v in ln[1:4]] for ln in lines[4:4 + n]])
    return dict(f_sigma=f_sigma, f_epsilon=f_eps, rcuton=ron, rcutoff=roff, lj_switch=sw, ucl=(ux, uy, uz),
                s_sigma=s_sigma, s_epsilon=s_eps, atoms=atoms), itvl


def gen_sfgrid(only):
    """Grids of the reference's own generator on its shipped nanotube cells: the CH3 cell
    as given (no switch) and the CH2 cell with the energy switch on (12-14 A)."""
    cases = {}
    spec, _ = read_sfgridgen_input(os.path.join(REF, "tools", "CH3-SWNT11x11.in"))
    cases["sfgrid_ch3_swnt"] = (spec, 1.0)
    spec2, _ = read_sfgridgen_input(os.path.join(REF, "tools", "CH2-SWNT11x11.in"))
    spec2.update(rcuton=12.0, rcutoff=14.0, lj_switch=1)
    cases["sfgrid_ch2_switch"] = (spec2, 1.0)
    for name, (spec, itvl) in cases.items():
        if only and name not in only:
            continue
        dims, out, head = run_reference_sfgridgen(spec, itvl)
        fn = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(fn, atoms=spec["atoms"], ucl=np.array(spec["ucl"]),
                            lj=np.array([spec["f_sigma"], spec["f_epsilon"], spec["s_sigma"], spec["s_epsilon"],
                                         spec["rcuton"], spec["rcutoff"], spec["lj_switch"], itvl]),
                            dims=np.array(dims), out=out)
        print(f"{name}: dims={dims} -> {os.path.getsize(fn)} bytes")


def gen_md(only):
    for name, case in md_cases().items():
        system, nsteps = case[:2]
        trj_every = case[2] if len(case) > 2 else 0
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as td:
            write_reference_dir(system, td)
            parsed = read_reference_dir(td)
            r = run_reference_md(td, nsteps, trj_every)
        parsed.x, parsed.y, parsed.z = (r["start"][k].copy() for k in range(3))
        arrays = system_to_arrays(parsed)
        md = r["md"]
        if r.get("npt"):
            arrays["md_int"] = np.array([2, md["nstep_inner"], md["nfree"], r["nsteps"], md["lj_lrc"]])
            arrays["md_real"] = np.array([md["delt"], md["treq"], md["qts"], md["qbs"], md["preq"]])
            arrays["md_state0"] = np.array([r["state"][k] for k in ("vts", "vbs", "rts", "boxlx", "pljlrc")])
        else:
            arrays["md_int"] = np.array([md["scheme"], md["nstep_inner"], md["nfree"], r["nsteps"]])
            arrays["md_real"] = np.array([md["delt"], md["treq"], md["qq"], md["qqs"], md["gg"], md["ggs"]])
            arrays["md_state0"] = np.array([r["state"][k] for k in ("ps", "ss", "pss", "sss")])
        arrays["md_v0"] = r["start"][3:]
        if trj_every > 0:
            arrays["trj_every"] = np.array(trj_every)
            arrays["ref_trj"] = np.frombuffer(r["trj"], dtype=np.uint8)
            arrays["ref_sav"] = np.frombuffer(r["sav"], dtype=np.uint8)
        arrays["md_log"] = r["log"]
        arrays["md_end"] = r["end"]
        fn = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(fn, **arrays)
        print(f"{name}: natom={parsed.natom} steps={nsteps} tinst {r['log'][0, 8]:.6g} -> {r['log'][-1, 8]:.6g} "
              f"-> {os.path.getsize(fn)} bytes")


# the canonical HMC move of Lennard-Jones replicas (mg_hmc_batch's workload): parameters,
# replica sizes and Philox key shared with tests/test_hmc.py
HMC_HP = dict(eps=1.0, sigma=1.0, rcutoff=2.5, mass=1.0, treq=1.0, delt=0.001, nstep_md=10, seed=0x1234ABCD5678,
              rescale=1, nconstraint=0)
HMC_SIZES = (200, 500, 864)


def gen_hmc(only):
    """hmc_lj_ref: one canonical move of each of three LJ replicas through the compiled
    reference's own md_move() over vver(), started from the velocities mg_hmc_batch draws for
    move 0 of that replica (replica r of the batch: orc_hmc_velocities)."""
    name = "hmc_lj_ref"
    if only and name not in only:
        return
    from mspms2_gb300.system import time_base
    from oracle.pyoracle import hmc_velocities, run_reference_hmc
    rec = {k: [] for k in ("natom", "box", "pos", "vel", "dh", "accept", "pre", "prop_e", "prop", "final")}
    for r, n in enumerate(HMC_SIZES):
        s = configs.lj_replica(n, seed=40 + r)
        s.treq_K, s.delt_fs, s.nstep_inner = HMC_HP["treq"], HMC_HP["delt"] * time_base(s), 1
        s.what_simulation, s.what_ensemble = 1, 0  # HMC: the reference sets up md_move's state
        v = hmc_velocities(HMC_HP, r, 0, n)
        with tempfile.TemporaryDirectory() as td:
            write_reference_dir(s, td)
            mv = run_reference_hmc(td, [v], HMC_HP["nstep_md"])["moves"][0]
        rec["natom"].append(n)
        rec["box"].append(float(s.box[0]))
        rec["pos"].append(np.stack([s.x, s.y, s.z]))
        rec["vel"].append(v)
        rec["dh"].append(mv["dh"])
        rec["accept"].append(int(mv["accept"]))
        rec["pre"].append(mv["pre"])
        rec["prop_e"].append(mv["proposal_energies"])
        rec["prop"].append(mv["proposal"])
        rec["final"].append(mv["final"])
        print(f"{name}[{r}]: natom={n} dH={mv['dh']:.10g} accept={mv['accept']}")
    arrays = {"natom": np.array(rec["natom"], np.int32), "box": np.array(rec["box"]),
              "dh": np.array(rec["dh"]), "accept": np.array(rec["accept"], np.int32), "pre": np.array(rec["pre"]),
              "prop_e": np.array(rec["prop_e"]),
              "hp": np.array([HMC_HP[k] for k in ("eps", "sigma", "rcutoff", "mass", "treq", "delt")]),
              "hp_int": np.array([HMC_HP["nstep_md"], HMC_HP["seed"], HMC_HP["rescale"], HMC_HP["nconstraint"]],
                                 np.int64)}
    for k in ("pos", "vel", "prop", "final"):
        arrays[k] = np.concatenate(rec[k], axis=1)
    fn = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(fn, **arrays)
    print(f"{name} -> {os.path.getsize(fn)} bytes")


def main():
    if not reference_available():
        sys.exit("oracle/_ref/mspms_ref_force missing: run `sh oracle/build_ref.sh` first")
    only = set(sys.argv[1:])
    gen_hmc(only)
    gen_md(only)
    gen_sfgrid(only)
    for name, (kind, obj) in cases().items():
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as td:
            if kind == "dir":
                src = obj
            else:
                write_reference_dir(obj, td)
                src = td
            system = read_reference_dir(src)
            (fl, fs, e, d), _ = run_reference_dir(src)
        arrays = system_to_arrays(system)
        arrays["ref_fl"] = fl
        arrays["ref_fs"] = fs
        arrays["ref_energies"] = np.array(list(e.values()))
        arrays["ref_derived"] = np.array(list(d.values()))
        fn = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(fn, **arrays)
        print(f"{name}: natom={system.natom} uinter={e['uinter']:.10g} uintra={e['uintra']:.10g} "
              f"-> {os.path.getsize(fn)} bytes")


if __name__ == "__main__":
    main()
