"""torch.autograd.Function over the library's energy functional.

``RkEnergy.apply(pq, assembler, k, i1, i2, i3, i4, coef)`` returns
E = sum_e coef[e] R^k[e](i1,i2;i3,i4) (rk, dbsr_lib_dbs.f90:3981-4022) for
the orbital coefficients ``pq`` (ns x 2 x nbf, FP64) and, on backward, the
gradient dE/dpq computed on the GPU by ``dbsrg_backward``.  The orbitals are
uploaded into the assembler for each evaluation, so the pair potentials are
rebuilt from the cell moments every time.
"""
from __future__ import annotations

import numpy as np
import torch


class RkEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pq, assembler, k, i1, i2, i3, i4, coef):
        p = np.asfortranarray(pq.detach().cpu().numpy(), dtype=np.float64)
        assembler.set_orbitals(p, assembler_ipbs(assembler, p))
        e, g = assembler.backward(k, i1, i2, i3, i4, coef, grad=pq.requires_grad)
        if g is not None:
            ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(g)).to(pq.device))
        return pq.new_tensor(e)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return (gout * g,) + (None,) * 7


def assembler_ipbs(assembler, pq):
    """ipbs of the orbitals: the energy functional runs over bound orbitals."""
    ipbs = getattr(assembler, "_ipbs_bound", None)
    nbf = pq.shape[-1]
    if ipbs is None or len(ipbs) != nbf:
        ipbs = np.zeros(nbf, dtype=np.int32)
        assembler._ipbs_bound = ipbs
    return ipbs
