"""Solid-fluid potential grids: mg_sfgrid_sfgridgen against the reference's own
tools/sfgridgen.c, and mg_sfgrid_tasos (the Tasos table generator the reference does not
ship) against analytic identities.

Fixtures sfgrid_*.npz hold the compiled reference tool's output on its shipped nanotube
cells (tools/CH3-SWNT11x11.in as given; CH2 with the energy switch on). The test's numpy
restatement below sums, per node, the same Lennard-Jones terms over the cell's atoms and
their z images; on CPU it is pinned to the fixtures, and it is then the checker of the
Tasos fields. Under the switch the reference leaves some second derivatives unassigned
(tools/sfgridgen.c:268-270), so for that case only energy and gradient are compared
with the tool; the generator returns the derivatives of the switched energy.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

RGAS = 8.314472


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    f_sigma, f_eps, s_sigma, s_eps, ron, roff, sw, itvl = (float(v) for v in d["lj"])
    spec = dict(atoms=np.array(d["atoms"]), ucl=tuple(float(v) for v in d["ucl"]), f_sigma=f_sigma,
                f_epsilon=f_eps, s_sigma=s_sigma, s_epsilon=s_eps, rcuton=ron, rcutoff=roff, lj_switch=int(sw))
    return spec, itvl, tuple(int(v) for v in d["dims"]), np.array(d["out"])


def node_terms(spec, p, eps_unit):
    """Energy, gradient [3], Hessian [3, 3] and d3U/dxdydz at point p (numpy, FP64)."""
    sig = (spec["f_sigma"] + spec["s_sigma"]) / 2.0
    eps4 = 4.0 * np.sqrt(spec["f_epsilon"] * spec["s_epsilon"]) * eps_unit
    uclz, rc = spec["ucl"][2], spec["rcutoff"]
    nimg = 1
    while nimg * uclz < rc:
        nimg += 1
    ron2, roff2 = spec["rcuton"] ** 2, rc * rc
    D = (roff2 - ron2) ** 3
    E, G, H, T = 0.0, np.zeros(3), np.zeros((3, 3)), 0.0
    for img in range(-nimg, nimg + 1):
        d = p[None, :] - spec["atoms"] + np.array([0.0, 0.0, img * uclz])
        s = (d * d).sum(1)
        keep = s < roff2
        d, s = d[keep], s[keep]
        a3 = (sig * sig / s) ** 3
        a6 = a3 * a3
        u = [eps4 * (a6 - a3), eps4 * (-6 * a6 + 3 * a3) / s, eps4 * (42 * a6 - 12 * a3) / s ** 2,
             eps4 * (-336 * a6 + 60 * a3) / s ** 3]
        g = u
        if spec["lj_switch"]:
            t, w = roff2 - s, roff2 + 2 * s - 3 * ron2
            S = [t * t * w / D, (-2 * t * w + 2 * t * t) / D, (2 * w - 8 * t) / D, np.full_like(s, 12.0 / D)]
            on = s >= ron2
            sw = [np.where(on, S[0], 1.0), np.where(on, S[1], 0.0), np.where(on, S[2], 0.0), np.where(on, S[3], 0.0)]
            g = [u[0] * sw[0], u[1] * sw[0] + u[0] * sw[1], u[2] * sw[0] + 2 * u[1] * sw[1] + u[0] * sw[2],
                 u[3] * sw[0] + 3 * u[2] * sw[1] + 3 * u[1] * sw[2] + u[0] * sw[3]]
        E += g[0].sum()
        G += (2 * g[1][:, None] * d).sum(0)
        H += (4 * g[2][:, None, None] * d[:, :, None] * d[:, None, :]).sum(0) + np.eye(3) * (2 * g[1]).sum()
        T += (8 * g[3] * d[:, 0] * d[:, 1] * d[:, 2]).sum()
    return E, G, H, T


def sample_nodes(dims, count=24, seed=0):
    rng = np.random.default_rng(seed)
    n = dims[0] * dims[1] * dims[2]
    return rng.choice(n, size=min(count, n), replace=False)


def node_point(idx, dims, itvl):
    i, rem = divmod(int(idx), dims[1] * dims[2])
    j, k = divmod(rem, dims[2])
    return np.array([i, j, k], dtype=float) * itvl


@pytest.mark.parametrize("name", ["sfgrid_ch3_swnt", "sfgrid_ch2_switch"])
def test_restatement_matches_reference_tool(name):
    spec, itvl, dims, out = load(name)
    for idx in sample_nodes(dims):
        E, G, H, _ = node_terms(spec, node_point(idx, dims, itvl), RGAS)
        scale = max(abs(out[0, idx]), 1.0)
        assert abs(E - out[0, idx]) <= 1e-10 * scale
        gs = max(np.abs(out[1:4, idx]).max(), 1.0)
        assert np.abs(G - out[1:4, idx]).max() <= 1e-10 * gs
        if spec["lj_switch"]:
            continue
        hs = max(np.abs(out[4:13, idx]).max(), 1.0)
        assert np.abs(-H.reshape(9) - out[4:13, idx]).max() <= 1e-10 * hs


def test_third_derivative_is_derivative_of_second():
    spec, _, _, _ = load("sfgrid_ch2_switch")
    rng = np.random.default_rng(3)
    h = 1e-4
    for p in rng.uniform([2.0, 2.0, 0.0], [12.0, 12.0, 2.4], size=(10, 3)):
        _, _, _, T = node_terms(spec, p, 1.0)
        hp = node_terms(spec, p + np.array([0, 0, h]), 1.0)[2][0, 1]
        hm = node_terms(spec, p - np.array([0, 0, h]), 1.0)[2][0, 1]
        fd = (hp - hm) / (2 * h)
        assert abs(T - fd) <= 1e-5 * max(abs(T), 1.0), (p, T, fd)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["sfgrid_ch3_swnt", "sfgrid_ch2_switch"])
def test_gpu_sfgridgen_matches_reference_tool(name, prec):
    from mspms2_gb300 import build
    from mspms2_gb300.engine import sfgrid_sfgridgen
    build.build()
    spec, itvl, dims, out = load(name)
    gdims, g = sfgrid_sfgridgen(spec, itvl, precision=prec)
    assert gdims == dims
    tol = 1e-10 if prec == "fp64" else 1e-5
    fields = range(4) if spec["lj_switch"] else range(13)
    for k in fields:
        scale = np.abs(out[k]).max()
        assert np.abs(g[k] - out[k]).max() <= tol * scale, (name, prec, k)
    if spec["lj_switch"]:  # second derivatives of the switched energy, from the restatement
        for idx in sample_nodes(dims, 12):
            _, _, H, _ = node_terms(spec, node_point(idx, dims, itvl), RGAS)
            assert np.abs(-H.reshape(9) - g[4:13, idx]).max() <= tol * max(np.abs(H).max(), 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_tasos_table(prec):
    from mspms2_gb300 import build
    from mspms2_gb300.engine import sfgrid_sfgridgen, sfgrid_tasos
    build.build()
    spec, itvl, dims, out = load("sfgrid_ch2_switch")
    nx, ny, nz = dims
    v = sfgrid_tasos(spec, nx, ny, nz, (itvl, itvl, itvl), precision=prec)
    tol = 1e-10 if prec == "fp64" else 1e-5
    # same nodes as the sfgridgen layout: F = E / Rgas, D = dE / Rgas
    e = out[0].reshape(nx, ny, nz).transpose(2, 1, 0) / RGAS
    assert np.abs(v[..., 0] - e).max() <= tol * np.abs(e).max()
    for q, k in ((1, 1), (2, 2), (3, 3)):
        ref = out[k].reshape(nx, ny, nz).transpose(2, 1, 0) / RGAS
        assert np.abs(v[..., q] - ref).max() <= tol * np.abs(ref).max()
    # mixed derivatives and Dxyz against the restatement
    rng = np.random.default_rng(1)
    for _ in range(12):
        i, j, k = rng.integers(0, nx), rng.integers(0, ny), rng.integers(0, nz)
        _, _, H, T = node_terms(spec, np.array([i, j, k], dtype=float) * itvl, 1.0)
        want = np.array([H[0, 1], H[0, 2], H[1, 2], T])
        got = v[k, j, i, 4:8]
        assert np.abs(got - want).max() <= tol * max(np.abs(want).max(), 1.0), (i, j, k, got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_device_generated_table_matches_host_route(prec):
    """mg_sf_tasos_generate (table evaluated into the engine on the device) gives the
    engine the same table, bit for bit, as mg_sfgrid_tasos + mg_sf_tasos_set_grid."""
    import ctypes as C

    from mspms2_gb300 import build
    from mspms2_gb300.engine import Engine, sfgrid_tasos
    from mspms2_gb300.system import load_system
    build.build()
    s, _ = load_system(os.path.join(GOLDEN, "sf_tasos.npz"))  # sites inside the first 3 A of the cell
    spec, _, _, _ = load("sfgrid_ch2_switch")
    cuc = spec["ucl"][2]
    nx = ny = 40
    nz = 13
    h = (0.2, 0.2, cuc / (nz - 1))
    with Engine(s, precision=prec) as ea:
        ea.sf_tasos_generate(1, spec, nx, ny, nz, h, cuc)
        fa, _, ea_e = ea.compute()
    v = np.ascontiguousarray(sfgrid_tasos(spec, nx, ny, nz, h, precision=prec), dtype=np.float64)
    with Engine(s, precision=prec) as eb:
        st = eb.lib.mg_sf_tasos_set_grid(eb.ctx, 1, nx, ny, nz, h[0], h[1], h[2], cuc,
                                         v.ctypes.data_as(C.POINTER(C.c_double)))
        assert st == 0
        fb, _, eb_e = eb.compute()
    assert np.array_equal(fa, fb)
    assert ea_e["usflj"] == eb_e["usflj"] and ea_e["usflj"] != 0.0
