"""Known-answer tests of the oracle's Tasos tricubic-Hermite interpolation.

The reference evaluates the tabulated solid-fluid potential in Fortran
(mylibtasos/forces.f90:6-173, cubicinterpolation.f90:9-116, cubicauxiliary.f90:76-573),
which cannot be compiled here, so the oracle's restatement of it is pinned by what the
interpolation must satisfy by construction:
  1. at a grid node the interpolant equals the node value F and its gradient equals the
     node derivatives (Dx, Dy, Dz);
  2. a polynomial of degree <= 3 in each coordinate, tabulated with its exact
     derivatives (F, Dx, Dy, Dz, Dxy, Dxz, Dyz, Dxyz in physical units), is reproduced
     exactly inside every cell (value and gradient);
  3. the force is minus the gradient of the energy (central finite differences).
With the reference's Dxyz corner swap (MG_COMPAT_TASOS_DXYZ) property 2 holds when Dxyz
is the same at every node, which the tests use to cover that mode too.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.pyoracle import OrcTasos, lib

COMPAT_DXYZ, COMPAT_PE_FLIP = 2, 4
_dp = C.POINTER(C.c_double)


def poly_grid(coef, nx, ny, nz, h):
    """Node records (I fastest, then J, then K) of p(x,y,z) = sum coef[a,b,c] x^a y^b z^c."""
    x = np.arange(nx) * h[0]
    y = np.arange(ny) * h[1]
    z = np.arange(nz) * h[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    rec = np.zeros((nz, ny, nx, 8))
    for (dx, dy, dz), slot in (((0, 0, 0), 0), ((1, 0, 0), 1), ((0, 1, 0), 2), ((0, 0, 1), 3), ((1, 1, 0), 4),
                               ((1, 0, 1), 5), ((0, 1, 1), 6), ((1, 1, 1), 7)):
        rec[..., slot] = poly_eval(coef, X, Y, Z, dx, dy, dz)
    return rec.reshape(-1)


def poly_eval(coef, x, y, z, dx=0, dy=0, dz=0):
    out = np.zeros(np.broadcast(x, y, z).shape)
    for a in range(4):
        for b in range(4):
            for c in range(4):
                if a < dx or b < dy or c < dz or coef[a, b, c] == 0:
                    continue
                fa = np.prod(range(a - dx + 1, a + 1)) if dx else 1
                fb = np.prod(range(b - dy + 1, b + 1)) if dy else 1
                fc = np.prod(range(c - dz + 1, c + 1)) if dz else 1
                out = out + coef[a, b, c] * fa * fb * fc * x ** (a - dx) * y ** (b - dy) * z ** (c - dz)
    return out


class Grid:
    def __init__(self, values, nx, ny, nz, h):
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        self.g = OrcTasos(nx=nx, ny=ny, nz=nz, hx=h[0], hy=h[1], hz=h[2], cuc=(nz - 2) * h[2],
                          values=self.values.ctypes.data_as(_dp), min_pe=0.0)
        self.g.min_pe = lib().orc_tasos_min_pe(C.byref(self.g))

    def eval(self, x, y, z, compat):
        pe = C.c_double()
        f = (C.c_double * 3)()
        st = lib().orc_tasos_force(C.byref(self.g), compat, x, y, z, C.byref(pe), f)
        assert st == 0
        return pe.value, np.array(f[:])


NX, NY, NZ = 7, 6, 8
H = (0.2, 0.25, 0.3)


def random_coef(rng, keep_xyz_constant=False):
    coef = rng.uniform(-1.0, 1.0, size=(4, 4, 4))
    # p about -50 on the grid: every value lies above 1.5 x the table minimum (about -55),
    # so the reference's PE flip (PE = -F below 1.5 minPE) never applies
    coef[0, 0, 0] = -50.0
    if keep_xyz_constant:  # d3p/dxdydz constant: only the c[1,1,1] term mixes all three axes
        coef[1:, 1:, 1:] = 0.0
        coef[1, 1, 1] = 0.7
    return coef


@pytest.mark.parametrize("compat", [0, COMPAT_DXYZ | COMPAT_PE_FLIP])
def test_nodes_reproduce_value_and_gradient(compat):
    rng = np.random.default_rng(1)
    coef = random_coef(rng)
    grid = Grid(poly_grid(coef, NX, NY, NZ, H), NX, NY, NZ, H)
    rec = grid.values.reshape(NZ, NY, NX, 8)
    for i, j, k in [(1, 1, 1), (2, 3, 4), (4, 2, 5), (5, 4, 2)]:
        pe, f = grid.eval(i * H[0], j * H[1], k * H[2], compat)
        r = rec[k, j, i]
        assert abs(pe - r[0]) <= 1e-12 * abs(r[0])
        assert np.allclose(f, -r[1:4], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("compat,xyz_const", [(0, False), (COMPAT_DXYZ | COMPAT_PE_FLIP, True)])
def test_tricubic_polynomial_reproduced(compat, xyz_const):
    rng = np.random.default_rng(2)
    coef = random_coef(rng, keep_xyz_constant=xyz_const)
    grid = Grid(poly_grid(coef, NX, NY, NZ, H), NX, NY, NZ, H)
    pts = rng.uniform([0.01, 0.01, 0.01], [(NX - 2) * H[0] - 0.01, (NY - 2) * H[1] - 0.01, (NZ - 2) * H[2] - 0.01],
                      size=(200, 3))
    for x, y, z in pts:
        pe, f = grid.eval(x, y, z, compat)
        want = poly_eval(coef, x, y, z)
        grad = np.array([poly_eval(coef, x, y, z, 1, 0, 0), poly_eval(coef, x, y, z, 0, 1, 0),
                         poly_eval(coef, x, y, z, 0, 0, 1)])
        assert abs(pe - want) <= 1e-11 * abs(want), (x, y, z, pe, want)
        assert np.allclose(f, -grad, rtol=1e-9, atol=1e-9), (x, y, z, f, -grad)


def test_pe_flip_below_one_and_a_half_minimum():
    """forces.f90:167-171: PE = -F where F < 1.5 minPE (the force is not flipped)."""
    rng = np.random.default_rng(5)
    coef = random_coef(rng)
    coef[0, 0, 0] = 50.0  # values about 50 all lie below 1.5 x the minimum (about 75)
    grid = Grid(poly_grid(coef, NX, NY, NZ, H), NX, NY, NZ, H)
    p = (2.5 * H[0], 2.2 * H[1], 3.7 * H[2])
    pe_ref, f_ref = grid.eval(*p, 0)
    pe_flip, f_flip = grid.eval(*p, COMPAT_PE_FLIP)
    assert pe_ref > 0 and pe_flip == -pe_ref
    assert np.array_equal(f_ref, f_flip)


def test_dxyz_swap_breaks_reproduction_of_a_general_tricubic():
    """The compatibility mode is the reference's behaviour, not the exact interpolant:
    with a varying Dxyz it departs from the polynomial somewhere inside the cells."""
    rng = np.random.default_rng(3)
    coef = random_coef(rng)
    grid = Grid(poly_grid(coef, NX, NY, NZ, H), NX, NY, NZ, H)
    pts = rng.uniform(0.05, 0.9, size=(50, 3)) * np.array([(NX - 2) * H[0], (NY - 2) * H[1], (NZ - 2) * H[2]])
    err = max(abs(grid.eval(x, y, z, COMPAT_DXYZ)[0] - poly_eval(coef, x, y, z)) for x, y, z in pts)
    assert err > 1e-8


@pytest.mark.parametrize("compat", [0, COMPAT_DXYZ])
def test_force_is_minus_energy_gradient(compat):
    """Smooth non-polynomial data: F = exp(-r^2) style bump with its exact derivatives."""
    nx, ny, nz = 9, 9, 10
    h = (0.15, 0.15, 0.2)
    x = np.arange(nx) * h[0]
    y = np.arange(ny) * h[1]
    z = np.arange(nz) * h[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    a = np.array([0.5, 0.6, 0.7])
    e = np.exp(-((X - 0.6) ** 2 * a[0] + (Y - 0.55) ** 2 * a[1] + (Z - 0.8) ** 2 * a[2]))
    gx, gy, gz = -2 * a[0] * (X - 0.6), -2 * a[1] * (Y - 0.55), -2 * a[2] * (Z - 0.8)
    rec = np.stack([e, gx * e, gy * e, gz * e, gx * gy * e, gx * gz * e, gy * gz * e, gx * gy * gz * e], -1) + \
        np.array([10.0, 0, 0, 0, 0, 0, 0, 0])
    grid = Grid(rec.reshape(-1), nx, ny, nz, h)
    rng = np.random.default_rng(4)
    d = 1e-6
    for p in rng.uniform(0.1, 0.95, size=(40, 3)) * np.array([(nx - 2) * h[0], (ny - 2) * h[1], (nz - 2) * h[2]]):
        # stay inside one cell for the difference stencil
        cell = np.floor(p / h)
        if np.any(np.abs(p - cell * h) < 2 * d) or np.any(np.abs(p - (cell + 1) * h) < 2 * d):
            continue
        _, f = grid.eval(*p, compat)
        fd = []
        for ax in range(3):
            dp = np.zeros(3)
            dp[ax] = d
            fd.append(-(grid.eval(*(p + dp), compat)[0] - grid.eval(*(p - dp), compat)[0]) / (2 * d))
        assert np.allclose(f, fd, rtol=1e-6, atol=1e-6), (p, f, fd)
