"""torch.autograd view of the energy (test harness only).

``XTBEnergy.apply(xyz)`` returns the GFN2-form energy of one structure; its
backward pass returns the analytic nuclear gradient computed by the CUDA
adjoint kernels (integral derivatives contracted with the density, the
energy-weighted density and the SCC potentials, plus the pair and
coordination-number terms). Tests compare it with central finite differences
(``torch.autograd.gradcheck``). The MD path never goes through torch.
"""
import numpy as np
import torch

from . import Batch


class XTBEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, batch):
        batch.set_state(xyz=xyz.detach().cpu().numpy())
        batch.egrad()
        r = batch.get()
        if r["status"][0] != 0:
            raise RuntimeError("SCC failed (status %d)" % r["status"][0])
        ctx.save_for_backward(torch.from_numpy(r["grad"]).to(xyz))
        return torch.tensor(r["energy"][0], dtype=xyz.dtype)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return gout * g, None


def energy_function(Z, charge=1, etemp=300.0, tight=True):
    """Return f(xyz) -> energy (torch, float64) for a fixed atom list."""
    b = Batch([{"Z": np.asarray(Z), "xyz": np.zeros((len(Z), 3)), "charge": charge}], etemp=etemp)
    if tight:
        b.set_scc(100, 1e-10, 1e-8, 0.25)
    return lambda xyz: XTBEnergy.apply(xyz, b)
