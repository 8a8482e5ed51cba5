"""Differentiable GB energy for parameter fitting: a torch.autograd.Function
over the device adjoint (``gbx_adjoint``).

One forward call runs the whole pipeline once in adjoint mode -- table,
integrals, Born radii, pair term, chain rule with dE/dR and dE/dq -- and
keeps the gradients with respect to positions, charges, input radii and the
two Born-radius coefficients (alpha0, alpha1) for the backward, which only
scales them by the incoming gradient.  Per-point volumes are recomputed
inside the chain rule rather than stored, so memory stays O(N + table).

The reference exposes the same gradients through its reference platform
(CharmmReferenceGBSW.cpp:597-674 for dB/dx, CharmmReferenceGBMV.cpp:349-443
for the chain rule and the parameter derivatives); here they come from the
GPU path.  Positions are in nm, energies in kJ/mol.
"""
from __future__ import annotations

import torch

from ._lib import EXEC_CHECK, Context
from .spec import GBModel


class GBEnergyFunction(torch.autograd.Function):
    """E = GB(positions [n,3], charges [n], radii [n], alpha [2]) on one context."""

    @staticmethod
    def forward(ctx, positions, charges, radii, alpha, gb: Context, check: bool = True):
        if not positions.is_cuda:
            raise ValueError("GBEnergyFunction: positions must be a CUDA tensor")
        n = gb.n
        if positions.shape != (n, 3) or charges.shape != (n,) or radii.shape != (n,) or alpha.shape != (2,):
            raise ValueError("GBEnergyFunction: expected positions [n,3], charges [n], radii [n], alpha [2]")
        gb.set_particle_parameters(charges.detach().double().cpu().numpy(), radii.detach().double().cpu().numpy())
        a = alpha.detach().double().cpu().numpy()
        gb.set_global_parameters(float(a[0]), float(a[1]))
        dev = positions.device
        posq = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        posq[:, :3] = positions.detach().to(torch.float32)
        f64 = dict(dtype=torch.float64, device=dev)
        energy = torch.zeros(1, **f64)
        forces = torch.zeros((n, 3), **f64)
        dq = torch.zeros(n, **f64)
        dR = torch.zeros(n, **f64)
        da = torch.zeros(2, **f64)
        stream = torch.cuda.current_stream(dev).cuda_stream
        gb.adjoint_device(posq.data_ptr(), energy.data_ptr(), forces.data_ptr(), dq.data_ptr(), dR.data_ptr(),
                          da.data_ptr(), EXEC_CHECK if check else 0, stream)
        ctx.save_for_backward(forces, dq, dR, da)
        ctx.dtypes = (positions.dtype, charges.dtype, radii.dtype, alpha.dtype)
        return energy[0].to(positions.dtype)

    @staticmethod
    def backward(ctx, grad):
        forces, dq, dR, da = ctx.saved_tensors
        g = grad.to(torch.float64)
        tp, tq, tr, ta = ctx.dtypes
        return (-forces * g).to(tp), (dq * g).to(tq), (dR * g).to(tr), (da * g).to(ta), None, None


class GBEnergy(torch.nn.Module):
    """Module form: owns the CUDA context; charges, radii and alpha may be
    nn.Parameters (the fitting use case)."""

    def __init__(self, model: GBModel, n_atoms: int):
        super().__init__()
        self.model = model
        self.gb = Context(model, n_atoms)

    def forward(self, positions, charges, radii, alpha=None):
        if alpha is None:
            alpha = torch.tensor([self.model.alpha0, self.model.alpha1], dtype=torch.float64,
                                 device=positions.device)
        return GBEnergyFunction.apply(positions, charges, radii, alpha, self.gb)


def gb_energy(positions, charges, radii, alpha, gb: Context):
    """Functional form of GBEnergyFunction."""
    return GBEnergyFunction.apply(positions, charges, radii, alpha, gb)


__all__ = ["GBEnergyFunction", "GBEnergy", "gb_energy"]
