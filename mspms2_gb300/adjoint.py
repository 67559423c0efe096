"""torch.autograd front end of the engine's adjoint (mg_adjoint_params).

`long_forces(eps, sigma, charge, engine)` returns the long forces F ([3, n], those of
frclong(), src/frclong.c:20) for per-site-class Lennard-Jones epsilon, sigma and charges
as differentiable torch tensors: the forward pass is one engine evaluation, the backward
pass one adjoint call, which turns dL/dF into dL/d(epsilon, sigma, charge) on the GPU by
recomputing the pair terms. A class is one site of one species template, numbered species
by species (Engine.class_params gives the starting values). The tensors live on the host:
the engine takes host arrays and keeps its own device buffers.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import TERMS_LONG, Engine


def _np(t: torch.Tensor) -> np.ndarray:
    return t.detach().to("cpu", torch.float64).numpy()


class LongForces(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps, sigma, charge, engine: Engine, positions):
        engine.set_class_params(_np(eps), _np(sigma), _np(charge))
        x, y, z = positions
        fl, _, _ = engine.compute(x, y, z, terms=TERMS_LONG)
        ctx.engine = engine
        ctx.positions = positions
        ctx.save_for_backward(eps, sigma, charge)
        return torch.from_numpy(fl).to(eps.dtype)

    @staticmethod
    def backward(ctx, grad_f):
        eps, sigma, charge = ctx.saved_tensors
        eng = ctx.engine
        # the engine holds one parameter set: the one of this forward pass
        eng.set_class_params(_np(eps), _np(sigma), _np(charge))
        ge, gs, gq = eng.adjoint_params(_np(grad_f), *ctx.positions)
        out = [torch.from_numpy(v).to(eps.dtype) for v in (ge, gs, gq)]
        return out[0], out[1], out[2], None, None


def long_forces(eps: torch.Tensor, sigma: torch.Tensor, charge: torch.Tensor, engine: Engine,
                positions=None) -> torch.Tensor:
    """Long forces [3, n] as a differentiable function of the class parameters."""
    s = engine.system
    if positions is None:
        positions = (np.asarray(s.x, float), np.asarray(s.y, float), np.asarray(s.z, float))
    return LongForces.apply(eps, sigma, charge, engine, positions)
