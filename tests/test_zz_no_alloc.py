"""mg_ewald_recip_static (the reciprocal-space pass with no device allocation) against
mg_compute, both called through the C ABI on the same ion box.

The ions sit on a jittered cubic lattice (spacing 3 A, jitter 0.4 A per axis) and the
real-space cutoff is 1.5 A, so no pair lies inside it and mg_compute's long-range forces
are the reciprocal-space forces alone; its ufourier is the reciprocal energy. Both paths
run the same kernels on the same inputs, so forces and energy agree to 1e-12 (relative);
the energy differs only in the order of its final sum. Each case calls the static entry
point twice in a row: the second call reuses the k-vector tables the first one left in
the scratch array.
"""
import ctypes as C

import numpy as np
import pytest

from mspms2_gb300 import build
from mspms2_gb300.capi import MgParams
from mspms2_gb300.configs import ion_box
from mspms2_gb300.engine import PREC, TERMS_LONG, Engine

pytestmark = pytest.mark.gpu

MG_ERR_CAPACITY = 7
TOL = 1e-12


def bind(lib):
    V = C.c_void_p
    lib.mg_ewald_recip_static.argtypes = [C.c_int, V, C.c_int, C.c_int, V, V, V, V, C.POINTER(MgParams), V, V,
                                          C.c_char_p, C.c_size_t]
    lib.mg_ewald_recip_static.restype = C.c_int
    return lib.mg_ewald_recip_static


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("nside,kmax,ksqmax", [(10, 8, 64), (16, 10, 100)])
def test_static_matches_compute(prec, nside, kmax, ksqmax):
    torch = pytest.importorskip("torch")
    s = ion_box(nside, seed=nside, kmax=kmax, ksqmax=ksqmax)
    n = s.natom
    with Engine(s, precision=prec) as eng:
        fl, _, e = eng.compute(terms=TERMS_LONG)
        assert eng.stats()["pairs_within_cutoff"] == 0
        fn = bind(eng.lib)
        params = eng.params
        dev = torch.device("cuda:0")
        x, y, z = (torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in (s.x, s.y, s.z))
        q = torch.from_numpy(s.site_arrays()[0].astype(np.float64)).to(dev)
        for call in range(2):
            f = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=dev)  # overwritten by the call
            en = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
            err = C.create_string_buffer(256)
            torch.cuda.synchronize()
            st = fn(0, None, PREC[prec], n, x.data_ptr(), y.data_ptr(), z.data_ptr(), q.data_ptr(), C.byref(params),
                    f.data_ptr(), en.data_ptr(), err, len(err))
            assert st == 0, err.value.decode()
            torch.cuda.synchronize()
            fs = f.cpu().numpy().reshape(3, n)
            assert rel(fs, fl) <= TOL, (call, rel(fs, fl))
            assert abs(en.item() - e["ufourier"]) <= TOL * abs(e["ufourier"]), (call, en.item(), e["ufourier"])


def test_static_rejects_oversized_request():
    torch = pytest.importorskip("torch")
    s = ion_box(10, seed=3, kmax=8, ksqmax=64)
    n = s.natom
    with Engine(s, precision="mixed") as eng:
        fn = bind(eng.lib)
        params = MgParams.from_buffer_copy(eng.params)
        params.kmax[0] = params.kmax[1] = params.kmax[2] = 120
        params.ksqmax = 14400  # 3.6e6 S(k) slots: about 106 MiB of scratch, over three times the limit
        dev = torch.device("cuda:0")
        buf = torch.zeros(3 * n, dtype=torch.float64, device=dev)
        err = C.create_string_buffer(256)
        st = fn(0, None, PREC["mixed"], n, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                C.byref(params), buf.data_ptr(), None, err, len(err))
        assert st == MG_ERR_CAPACITY
        assert b"limit" in err.value
