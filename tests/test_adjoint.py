"""Derivatives of the long forces: the adjoint (mg_adjoint_params, dL/d(epsilon, sigma,
charge) per site class for a loss of the long forces) and the Hessian-vector product in
positions (mg_adjoint_hvp), checked against central finite differences of the FP64 engine
forces, the mixed path against the FP64 path, and the torch.autograd front end against
finite differences of a quadratic force-matching loss.

Tolerances, norm-wise relative: FP64 vs central differences 1e-6 (the differences' own
truncation and rounding error is far below); mixed vs FP64 1e-4 (FP32 pair arithmetic of
~1e5 terms summed in FP64).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mspms2_gb300 import build
from mspms2_gb300.engine import TERMS_LONG, Engine, EngineError
from mspms2_gb300.system import load_system

pytestmark = pytest.mark.gpu

CASES = ["lj_fluid_500", "water_wolf_216", "water_ewald_512"]


@pytest.fixture(scope="session", autouse=True)
def built():
    build.build()


def load(case):
    s, _ = load_system(os.path.join(GOLDEN, case + ".npz"))
    return s


def loss_lin(eng, g, p):
    eng.set_class_params(*p)
    fl, _, _ = eng.compute(terms=TERMS_LONG)
    return float(np.sum(g * fl))


def fd_grad(eng, g, base, kind, k, h):
    p = [a.copy() for a in base]
    p[kind][k] = base[kind][k] + h
    up = loss_lin(eng, g, p)
    p[kind][k] = base[kind][k] - h
    dn = loss_lin(eng, g, p)
    eng.set_class_params(*base)
    return (up - dn) / (2 * h)


def step(kind, v):
    return (1e-5 if kind < 2 else 1e-6) * max(abs(v), 1.0 if kind == 2 else 1e-3)


def nrel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("case", CASES)
def test_fp64_adjoint_matches_central_differences(case):
    s = load(case)
    rng = np.random.default_rng(7)
    g = rng.standard_normal((3, s.natom))
    with Engine(s, precision="fp64") as eng:
        base = list(eng.class_params())
        grads = eng.adjoint_params(g)
        for kind in range(3):
            fd = np.zeros(len(base[kind]))
            for k in range(len(fd)):
                if kind == 0 and base[0][k] == 0.0:
                    continue  # no derivative at eps = 0 (square root of the mixing rule)
                if kind == 2 and s.charge_type == 0:
                    continue
                fd[k] = fd_grad(eng, g, base, kind, k, step(kind, base[kind][k]))
            if not np.any(fd):
                assert not np.any(grads[kind]), (case, kind, grads[kind])
                continue
            assert nrel(grads[kind], fd) <= 1e-6, (case, kind, grads[kind], fd)


@pytest.mark.parametrize("case", CASES)
def test_mixed_adjoint_matches_fp64(case):
    s = load(case)
    g = np.random.default_rng(11).standard_normal((3, s.natom))
    with Engine(s, precision="fp64") as e64:
        ref = e64.adjoint_params(g)
    with Engine(s, precision="mixed") as emx:
        got = emx.adjoint_params(g)
        again = emx.adjoint_params(g)
    for kind in range(3):
        if np.any(ref[kind]):
            assert nrel(got[kind], ref[kind]) <= 1e-4, (case, kind, got[kind], ref[kind])
        # fixed-order sums: bit-reproducible
        assert np.array_equal(got[kind], again[kind])


def test_torch_force_matching_gradient():
    torch = pytest.importorskip("torch")
    from mspms2_gb300.adjoint import long_forces

    s = load("water_wolf_216")
    with Engine(s, precision="fp64") as eng:
        eps0, sig0, q0 = (torch.tensor(a) for a in eng.class_params())
        target = long_forces(eps0 * 1.05, sig0 * 0.98, q0 * 1.02, eng).detach()
        eps = eps0.clone().requires_grad_(True)
        sig = sig0.clone().requires_grad_(True)
        q = q0.clone().requires_grad_(True)
        loss = ((long_forces(eps, sig, q, eng) - target) ** 2).sum()
        loss.backward()

        def L(e, si, qq):
            with torch.no_grad():
                return float(((long_forces(e, si, qq, eng) - target) ** 2).sum())

        for kind, (t, grad) in enumerate([(eps0, eps.grad), (sig0, sig.grad), (q0, q.grad)]):
            fd = np.zeros(len(t))
            for k in range(len(t)):
                if kind == 0 and float(t[k]) == 0.0:
                    continue
                h = step(kind, float(t[k]))
                args_p = [eps0.clone(), sig0.clone(), q0.clone()]
                args_m = [eps0.clone(), sig0.clone(), q0.clone()]
                args_p[kind][k] += h
                args_m[kind][k] -= h
                fd[k] = (L(*args_p) - L(*args_m)) / (2 * h)
            assert nrel(grad.numpy(), fd) <= 1e-5, (kind, grad, fd)


def test_unsupported_options_are_refused():
    s = load("butane_ewald_switch")  # LJ energy switch
    with Engine(s, precision="fp64") as eng:
        with pytest.raises(EngineError) as ei:
            eng.adjoint_params(np.ones((3, s.natom)))
        assert ei.value.status == 8


def split_molecules(case):
    """The system shifted by 0.4 box lengths with its sites wrapped one by one, so that
    some molecules span the box edge."""
    s = load(case)
    x, y, z = (np.mod(np.asarray(a, float) + 0.4 * L, L) for a, L in zip((s.x, s.y, s.z), s.box))
    xyz = np.stack([x, y, z]).reshape(3, -1, s.species[0].natom)
    assert np.any(np.abs(xyz[:, :, :1] - xyz[:, :, 1:]) > np.asarray(s.box)[:, None, None] / 2)
    s.x, s.y, s.z = x, y, z
    return s


@pytest.mark.parametrize("case", ["water_wrapped_wolf", "water_wrapped_ewald"])
def test_adjoint_with_molecules_spanning_the_box(case):
    s = split_molecules(case)
    g = np.random.default_rng(5).standard_normal((3, s.natom))
    with Engine(s, precision="fp64") as eng:
        base = list(eng.class_params())
        grads = eng.adjoint_params(g)
        for kind in (1, 2):
            fd = np.array([fd_grad(eng, g, base, kind, k, step(kind, base[kind][k])) for k in range(len(base[kind]))])
            assert nrel(grads[kind], fd) <= 1e-6, (case, kind, grads[kind], fd)


def fd_hvp(eng, v, h=1e-6):
    s = eng.system
    x0 = np.stack([s.x, s.y, s.z]).astype(float)
    fp, _, _ = eng.compute(*(x0 + h * v), terms=TERMS_LONG)
    fm, _, _ = eng.compute(*(x0 - h * v), terms=TERMS_LONG)
    return -(fp - fm) / (2 * h)


@pytest.mark.parametrize("case", CASES + ["split:water_wrapped_ewald"])
def test_fp64_hessian_vector_matches_central_differences(case):
    s = split_molecules(case[6:]) if case.startswith("split:") else load(case)
    v = np.random.default_rng(3).standard_normal((3, s.natom))
    with Engine(s, precision="fp64") as eng:
        hv = eng.hessian_vector(v)
        fd = fd_hvp(eng, v)
    assert nrel(hv, fd) <= 1e-6, (case, nrel(hv, fd))


@pytest.mark.parametrize("case", CASES)
def test_mixed_hessian_vector_matches_fp64(case):
    s = load(case)
    v = np.random.default_rng(4).standard_normal((3, s.natom))
    with Engine(s, precision="fp64") as e64:
        ref = e64.hessian_vector(v)
    with Engine(s, precision="mixed") as emx:
        got = emx.hessian_vector(v)
        again = emx.hessian_vector(v)
    assert nrel(got, ref) <= 1e-4, (case, nrel(got, ref))
    assert np.array_equal(got, again)


def test_hessian_is_symmetric():
    # u . H v = v . H u for a conservative force field (Wolf: force-shifted, continuous)
    s = load("water_wolf_216")
    rng = np.random.default_rng(9)
    u, v = rng.standard_normal((2, 3, s.natom))
    with Engine(s, precision="fp64") as eng:
        hu, hv = eng.hessian_vector(u), eng.hessian_vector(v)
    a, b = float(np.sum(u * hv)), float(np.sum(v * hu))
    assert abs(a - b) <= 1e-9 * max(abs(a), np.linalg.norm(hu) * np.linalg.norm(v)), (a, b)


def test_force_match_matches_adjoint_and_differences():
    # fused loss + gradient against the separate calls, and the tied-charge gradient
    # (q_H = -q_O / 2) against central differences of the FP64 loss (h = 1e-4 relative)
    s = load("water_ewald_512")
    rng = np.random.default_rng(21)
    with Engine(s, precision="fp64") as eng:
        base = list(eng.class_params())
        pert = [a * (1 + 0.02 * rng.standard_normal(a.shape)) for a in base]
        pert[2] = np.array([pert[2][0], -pert[2][0] / 2, -pert[2][0] / 2])
        eng.set_class_params(*pert)
        target, _, _ = eng.compute(terms=TERMS_LONG)
        eng.set_class_params(*base)
        fl, _, _ = eng.compute(terms=TERMS_LONG)
        scale = 1.0 / (3 * s.natom)
        loss, grads = eng.force_match(target)
        assert abs(loss - scale * np.sum((fl - target) ** 2)) <= 1e-12 * loss
        sep = eng.adjoint_params(2 * scale * (fl - target))
        for a, b in zip(grads, sep):
            assert np.allclose(a, b, rtol=1e-12, atol=0)

        def tied(p):  # (eps_O, sigma_O, q_O) -> class parameters
            e, sg, q = (a.copy() for a in base)
            e[0], sg[0] = p[0], p[1]
            q[:] = [p[2], -p[2] / 2, -p[2] / 2]
            return e, sg, q

        p0 = np.array([base[0][0], base[1][0], base[2][0]])
        g_tied = np.array([grads[0][0], grads[1][0], grads[2][0] - 0.5 * (grads[2][1] + grads[2][2])])
        fd = np.zeros(3)
        for k in range(3):
            h = 1e-4 * abs(p0[k])
            pp, pm = p0.copy(), p0.copy()
            pp[k] += h
            pm[k] -= h
            eng.set_class_params(*tied(pp))
            lp, _ = eng.force_match(target)
            eng.set_class_params(*tied(pm))
            lm, _ = eng.force_match(target)
            fd[k] = (lp - lm) / (2 * h)
        eng.set_class_params(*base)
        assert nrel(g_tied, fd) <= 1e-4, (g_tied, fd)
    with Engine(s, precision="mixed") as emx:
        lmx, gmx = emx.force_match(target)
    # the residual is ~2% of the force, so the mixed path's ~1e-6 force error is ~5e-5 of it
    assert abs(lmx - loss) <= 1e-3 * loss, (lmx, loss)
    gmx_tied = np.array([gmx[0][0], gmx[1][0], gmx[2][0] - 0.5 * (gmx[2][1] + gmx[2][2])])
    assert nrel(gmx_tied, g_tied) <= 1e-4, (gmx_tied, g_tied)
