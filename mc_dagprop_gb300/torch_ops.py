"""PyTorch autograd wrapper of the adjoint (torch is used only here).

``expected_tardiness(earliest, base, flat, gen, n, seed0)`` returns
J = mean over n samples of sum over events of (realized - earliest) as a 0-d
tensor whose backward gives dJ/d earliest (per event) and dJ/d base (per
activity of the flat DAG, i.e. per ``Activity.minimal_duration``), from the
hand-written adjoint kernel (``mcd_gradient_host``).  Each call compiles the DAG
with the given times, so the parameters can change between optimisation steps.
"""
from __future__ import annotations

import numpy as np
import torch

from . import batching


class ExpectedTardiness(torch.autograd.Function):
    @staticmethod
    def forward(ctx, earliest, base, flat, gen, n, seed0):
        f = dict(flat)
        f["earliest"] = earliest.detach().cpu().double().numpy()
        f["act_duration"] = base.detach().cpu().double().numpy()
        prop = batching.compile_dag(f, gen)
        out = prop.gradient(int(n), int(seed0))
        g_base_links = out["grad_base"]
        idx = np.asarray(flat["act_idx"], np.int64)
        g_base = np.where(idx < len(g_base_links), g_base_links[np.minimum(idx, max(len(g_base_links) - 1, 0))], 0.0)
        ctx.save_for_backward(torch.as_tensor(out["grad_earliest"], dtype=earliest.dtype, device=earliest.device),
                              torch.as_tensor(g_base, dtype=base.dtype, device=base.device))
        return torch.tensor(out["objective"], dtype=earliest.dtype, device=earliest.device)

    @staticmethod
    def backward(ctx, g):
        ge, gb = ctx.saved_tensors
        return g * ge, g * gb, None, None, None, None


def expected_tardiness(earliest: torch.Tensor, base: torch.Tensor, flat: dict, gen: list, n: int,
                       seed0: int = 0) -> torch.Tensor:
    return ExpectedTardiness.apply(earliest, base, flat, gen, n, seed0)
