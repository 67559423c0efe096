"""CPU checks of the C ABI: the library builds for sm_103a, loads without a GPU, exports
every function include/*.h declares, refuses to run without a device, and its host
helper mg_params_derive reproduces the reference's derived globals."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_cases
from mspms2_gb300 import build
from mspms2_gb300.capi import MgOptions, MgParams, system_params
from mspms2_gb300.engine import load_library
from mspms2_gb300.system import derive_params, load_system


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            names |= set(re.findall(r"MG_API\s+[\w\s\*]*?\b(mg_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    build.build()
    return load_library()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_abi_version(lib):
    assert lib.mg_abi_version() == 1


def test_create_without_device_fails_loudly(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    ctx = C.c_void_p()
    opt = MgOptions()
    lib.mg_options_default(C.byref(opt))
    st = lib.mg_create(C.byref(ctx), C.byref(opt))
    assert st == 3  # MG_ERR_NO_DEVICE


@pytest.mark.parametrize("case", golden_cases())
def test_params_derive_matches_python_and_reference(lib, case):
    s, d = load_system(os.path.join(GOLDEN, case + ".npz"))
    py = derive_params(s)
    p = system_params(s)
    q = MgParams.from_buffer_copy(p)
    lib.mg_params_derive(C.byref(q), *(float(v) for v in s.box))
    for k in ("rcutoffsq", "rcutonsq", "rcutoffelecsq", "roff2_minus_ron2_cube", "shift1", "shift4",
              "wolfvcon1", "wolfvcon2", "wolfvcon3", "wolffcon1", "wolffcon2", "bfactor_ewald",
              "vfactor_ewald", "twopi_lx", "twopi_ly", "twopi_lz", "twopi_over_3v"):
        assert getattr(q, k) == pytest.approx(py[k], rel=1e-15, abs=0), (case, k)
    ref = d["ref_derived"]
    assert q.shift1 == ref[4] and q.twopi_lx == ref[13] and q.vfactor_ewald == ref[12]


NULL_OK = {"mg_destroy": 0, "mg_abi_version": None, "mg_set_wait_limit": 0, "mg_siman_stage_count": None,
           "mg_ewald_recip_static_last_split": None, "mg_last_error": None, "mg_options_default": None,
           "mg_params_derive": None}


def test_every_entry_point_survives_null_arguments():
    """Each function of the ABI, called with every argument NULL or zero, returns an error
    status (or, for the few that take no handle, its plain result) instead of crashing; run
    in a child process, so that a crash fails this test rather than the session."""
    import json
    import subprocess
    import sys
    src = open(os.path.join(ROOT, "include", "mspms2_gb300.h")).read()
    decls = re.findall(r"MG_API\s+[\w\s\*]+?\b(mg_\w+)\s*\(([^)]*)\)", src)
    calls = [(name, 0 if p.strip() in ("", "void") else p.count(",") + 1) for name, p in decls]
    child = f"""
import ctypes as C, json
lib = C.CDLL({build.LIB!r})
out = {{}}
for name, n in {calls!r}:
    f = getattr(lib, name)
    f.restype = C.c_int
    out[name] = f(*([None] * n))
print(json.dumps(out))
"""
    build.build()
    p = subprocess.run([sys.executable, "-c", child], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    got = json.loads(p.stdout.strip().splitlines()[-1])
    assert set(got) == {n for n, _ in calls}
    for name, status in got.items():
        if name in NULL_OK:
            if NULL_OK[name] is not None:
                assert status == NULL_OK[name], (name, status)
        else:
            assert status != 0, name


MINIMAL_C = r"""
#include <stdio.h>
#include <string.h>
#include "mspms2_gb300.h"

/* the minimal sequence of the integration guide: 27 LJ sites with Wolf electrostatics */
int main(void) {
    enum { N = 27 };
    double x[N], y[N], z[N], fxl[N], fyl[N], fzl[N], fxs[N], fys[N], fzs[N];
    for (int i = 0; i < N; i++) { x[i] = 2.0 * (i % 3); y[i] = 2.0 * ((i / 3) % 3); z[i] = 2.0 * (i / 9); }
    int ghost = MG_GHOST_NONE, interp = 0;
    double eps = 1.0, sig = 1.0, q = 0.0, aw = 1.0;
    mg_species sp;
    memset(&sp, 0, sizeof sp);
    sp.nmole = N;
    sp.natom = 1;
    sp.ghost_type = &ghost;
    sp.interp_type = &interp;
    sp.epsilon = &eps;
    sp.sigma = &sig;
    sp.charge = &q;
    sp.aw = &aw;
    mg_params p;
    memset(&p, 0, sizeof p);
    p.rcutoff = p.rcuton = p.rcutoffelec = 2.5;
    p.charge_type = MG_ELEC_WOLF;
    p.kappa = 0.2;
    p.coulomb_prefactor = 1.0;
    p.sigma_base = p.epsilon_base = 1.0;
    p.compat = MG_COMPAT_ALL;
    mg_params_derive(&p, 6.0, 6.0, 6.0);
    mg_options opt;
    mg_options_default(&opt);
    mg_ctx *ctx = NULL;
    mg_status st = mg_create(&ctx, &opt);
    if (st != MG_OK) {
        printf("create %d\n", (int)st);
        return (int)st;
    }
    mg_energies e;
    if ((st = mg_set_params(ctx, &p)) || (st = mg_set_topology(ctx, 1, &sp)) || (st = mg_set_box(ctx, 6.0, 6.0, 6.0)) ||
        (st = mg_compute(ctx, x, y, z, MG_TERMS_ALL, fxl, fyl, fzl, fxs, fys, fzs, &e)))
        printf("%s\n", mg_last_error(ctx));
    else
        printf("uinter %.17g\n", e.uinter);
    mg_destroy(ctx);
    return (int)st;
}
"""


def test_documented_minimal_sequence_compiles_and_links(tmp_path):
    """The integration guide's minimal C sequence, filled in for 27 Lennard-Jones sites,
    compiles as C99 against the header with every warning an error, links against the
    library, and on a machine without a GB300 stops at mg_create with MG_ERR_NO_DEVICE."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib_path = build.build()
    src = tmp_path / "minimal.c"
    src.write_text(MINIMAL_C)
    exe = tmp_path / "minimal"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe), lib_path, f"-Wl,-rpath,{os.path.dirname(lib_path)}"], check=True,
                   capture_output=True, text=True)
    p = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    if p.returncode == 0:  # a GB300 is present: the sequence ran through
        assert p.stdout.startswith("uinter ")
    else:
        assert p.stdout.strip() == "create 3"  # MG_ERR_NO_DEVICE
