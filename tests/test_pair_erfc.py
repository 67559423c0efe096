"""The FP32 pair kernel's erfc (mg_pair.cu, erfc_from_exp): erfc(x) = t P(t) e^{-x^2} with
t = 1 / (1 + 0.35 x), the form of Abramowitz & Stegun 7.1.26 with a degree-8 P fitted to
the relative error of e^{x^2} erfc(x) on [0, 6]. The coefficients are read from the CUDA
source and checked against scipy's erfc: the fit itself (FP64 evaluation) to 2e-7
relative on [0, 6], and the FP32 evaluation as the kernel does it (FMA steps rounded to
FP32, e^{-x^2} correctly rounded) to 1e-6 relative on [0, 5], the range of kappa r in the
real-space sums (kappa rc is 3 in the water workloads).
"""
import os
import re

import numpy as np
import pytest

scipy_special = pytest.importorskip("scipy.special")

SRC = os.path.join(os.path.dirname(__file__), "..", "mspms2_gb300", "csrc", "mg_pair.cu")


def coefficients():
    src = open(SRC).read()
    body = src[src.index("__device__ __forceinline__ float erfc_from_exp("):]
    body = body[:body.index("return t * p * ex;")]
    p_scale = float(re.search(r"fmaf\(([-0-9.e+]+)f, x, 1\.0f\)", body).group(1))
    first = float(re.search(r"float p = ([-0-9.e+]+)f;", body).group(1))
    rest = [float(v) for v in re.findall(r"p = fmaf\(p, t, ([-0-9.e+]+)f\);", body)]
    return p_scale, [first] + rest  # highest degree first


def f32(v):
    return np.asarray(v, dtype=np.float64).astype(np.float32).astype(np.float64)


def test_fit_relative_error_fp64():
    ps, c = coefficients()
    assert ps == 0.35 and len(c) == 9
    x = np.linspace(0.0, 6.0, 200001)
    t = 1.0 / (1.0 + ps * x)
    p = np.polyval(c, t)
    ec = t * p * np.exp(-x * x)
    ref = scipy_special.erfc(x)
    assert np.max(np.abs(ec - ref) / ref) <= 2e-7


def test_fp32_evaluation_relative_error():
    ps, c = coefficients()
    x = f32(np.linspace(0.0, 5.0, 200001))
    t = f32(1.0 / f32(f32(ps) * x + 1.0))  # the FMA, then a correctly rounded reciprocal
    p = np.full_like(x, f32(c[0]))
    for ck in c[1:]:
        p = f32(p * t + f32(ck))  # one rounding per FMA
    ex = f32(np.exp(-x * x))
    ec = f32(f32(t * p) * ex)
    ref = scipy_special.erfc(x)
    assert np.max(np.abs(ec - ref) / ref) <= 1e-6
