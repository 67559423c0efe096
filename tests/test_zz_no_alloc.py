"""mg_ewald_recip_static (the reciprocal-space pass with no device allocation) against
mg_compute, both called through the C ABI on the same ion box.

The ions sit on a jittered cubic lattice (spacing 3 A, jitter 0.4 A per axis) and the
real-space cutoff is 1.5 A, so no pair lies inside it and mg_compute's long-range forces
are the reciprocal-space forces alone; its ufourier is the reciprocal energy. Both paths
run the same kernels on the same inputs, so forces and energy agree to 1e-12 (relative);
the energy differs only in the order of its final sum. Each case calls the static entry
point twice in a row: the second call reuses the k-vector tables the first one left in
the scratch array. Further cases: a caller's own stream; mixed precision with KMAXZ above
the tensor-core pass's 30 (the CUDA-core FP32 structure factors); a graph captured with
one KMAX and replayed after an eager call with another (the tables are re-keyed on the
device); and a bounded on-chip wait that gives up, which must show as NaN outputs.
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


def static_call(fn, params, prec, n, x, y, z, q, stream=0):
    """One call of the allocation-free entry point into fresh NaN-filled outputs; returns
    (status, message, forces [3, n] tensor, energy tensor), without synchronising."""
    import torch
    f = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=x.device)
    en = torch.full((1,), float("nan"), dtype=torch.float64, device=x.device)
    err = C.create_string_buffer(256)
    st = fn(0, C.c_void_p(stream) if stream else None, PREC[prec], n, x.data_ptr(), y.data_ptr(), z.data_ptr(),
            q.data_ptr(), C.byref(params), f.data_ptr(), en.data_ptr(), err, len(err))
    return st, err.value.decode(), f.view(3, n), en


def device_inputs(s):
    import torch
    dev = torch.device("cuda:0")
    x, y, z = (torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in (s.x, s.y, s.z))
    q = torch.from_numpy(s.site_arrays()[0].astype(np.float64)).to(dev)
    return x, y, z, q


@pytest.mark.parametrize("case", ["user_stream", "wide_kz"])
def test_static_stream_and_cuda_core_structure_factors(case):
    """On a torch stream of the caller (asynchronous on it), and on the mixed path with
    KMAXZ 34, where the structure factors come from the CUDA-core FP32 pass in both entry
    points. The k-space force pass splits its rows into ranges whose partial forces sit in
    the scratch left after the tables (checked through the split getter)."""
    torch = pytest.importorskip("torch")
    s = ion_box(10, seed=4, kmax=8, ksqmax=64)
    if case == "wide_kz":
        s.kmax = (4, 4, 34)
        s.ksqmax = 34 * 34
    n = s.natom
    with Engine(s, precision="mixed") as eng:
        fl, _, e = eng.compute(terms=TERMS_LONG)
        assert eng.stats()["pairs_within_cutoff"] == 0
        fn = bind(eng.lib)
        eng.lib.mg_ewald_recip_static_last_split.restype = C.c_int
        x, y, z, q = device_inputs(s)
        stream = torch.cuda.Stream() if case == "user_stream" else None
        torch.cuda.synchronize()
        for call in range(2):
            st, msg, f, en = static_call(fn, eng.params, "mixed", n, x, y, z, q,
                                         stream.cuda_stream if stream is not None else 0)
            assert st == 0, msg
            (stream or torch.cuda.current_stream()).synchronize()
            assert rel(f.cpu().numpy(), fl) <= TOL, (case, call, rel(f.cpu().numpy(), fl))
            assert abs(en.item() - e["ufourier"]) <= TOL * abs(e["ufourier"])
            assert eng.lib.mg_ewald_recip_static_last_split() > 1


def test_static_graph_replay_after_eager_key_change():
    """A call captured into a CUDA graph with KMAX 8 and replayed after an eager call with
    KMAX 6 gives the KMAX 8 result: the table kernel in the graph sees the other key in the
    scratch and rebuilds the tables before the pass reads them (and the eager call after the
    replay rebuilds its own)."""
    torch = pytest.importorskip("torch")
    s8 = ion_box(10, seed=6, kmax=8, ksqmax=64)
    s6 = ion_box(10, seed=6, kmax=6, ksqmax=36)
    n = s8.natom
    with Engine(s8, precision="mixed") as e8, Engine(s6, precision="mixed") as e6:
        f8 = e8.compute(terms=TERMS_LONG)[0]
        f6 = e6.compute(terms=TERMS_LONG)[0]
        fn = bind(e8.lib)
        p8, p6 = e8.params, e6.params
        x, y, z, q = device_inputs(s8)
        st, msg, _, _ = static_call(fn, p8, "mixed", n, x, y, z, q)  # set-up before any capture
        assert st == 0, msg
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        f = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=x.device)
        en = torch.full((1,), float("nan"), dtype=torch.float64, device=x.device)
        err = C.create_string_buffer(256)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
                st = fn(0, C.c_void_p(side.cuda_stream), PREC["mixed"], n, x.data_ptr(), y.data_ptr(), z.data_ptr(),
                        q.data_ptr(), C.byref(p8), f.data_ptr(), en.data_ptr(), err, len(err))
        assert st == 0, err.value.decode()
        torch.cuda.synchronize()
        st, msg, g6, _ = static_call(fn, p6, "mixed", n, x, y, z, q)
        assert st == 0, msg
        torch.cuda.synchronize()
        assert rel(g6.cpu().numpy(), f6) <= TOL
        f.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert rel(f.view(3, n).cpu().numpy(), f8) <= TOL
        st, msg, g6b, _ = static_call(fn, p6, "mixed", n, x, y, z, q)
        assert st == 0, msg
        torch.cuda.synchronize()
        assert rel(g6b.cpu().numpy(), f6) <= TOL


def test_static_wait_give_up_shows_as_nan():
    """With the pipeline-wait bound at 0 polls every CTA of the tensor-core structure-factor
    pass gives up (after waiting, with the default bound, for the MMAs it issued): the call
    still returns MG_OK, asynchronous as always, and every force and the energy are NaN.
    With the bound restored the next call is exact again."""
    torch = pytest.importorskip("torch")
    from mspms2_gb300.engine import set_wait_limit
    s = ion_box(16, seed=9, kmax=8, ksqmax=64)
    n = s.natom
    with Engine(s, precision="mixed") as eng:
        fl, _, e = eng.compute(terms=TERMS_LONG)
        fn = bind(eng.lib)
        x, y, z, q = device_inputs(s)
        torch.cuda.synchronize()
        try:
            set_wait_limit(0)
            st, msg, f, en = static_call(fn, eng.params, "mixed", n, x, y, z, q)
            assert st == 0, msg
            torch.cuda.synchronize()
        finally:
            set_wait_limit(-1)
        assert torch.isnan(f).all().item() and torch.isnan(en).all().item()
        st, msg, f, en = static_call(fn, eng.params, "mixed", n, x, y, z, q)
        assert st == 0, msg
        torch.cuda.synchronize()
        assert rel(f.cpu().numpy(), fl) <= TOL
        assert abs(en.item() - e["ufourier"]) <= TOL * abs(e["ufourier"])
