"""torch.autograd wrapper of the lattice energy, for gradient checks.

``LatticeEnergy.apply(p, efield)`` uploads the dipoles ``p`` (N x 3) into one
replica of a ``Simulation``, sets its applied field, and returns the total
energy; its backward is the hand-written adjoint kernel (dE/dp_i = len_i h_i -
C nn_i + E - K sgn, and dE/dE = sum_i p_i).  The sweep never goes through
this class: it exists so that torch's machinery can be pointed at the adjoint
and checked against finite differences of the forward.  dE/dCageStrain and
dE/dDipole come from ``Simulation.adjoint`` directly.
"""
from __future__ import annotations

import numpy as np
import torch


class LatticeEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, efield, sim, replica=0, lengths=None, precision="fp64"):
        xyz = p.detach().to("cpu", torch.float32).contiguous().numpy()
        ln = None if lengths is None else np.asarray(lengths, np.float32)
        sim.set_field(replica, [float(v) for v in efield.detach().cpu().tolist()])
        sim.upload(replica, xyz, ln)
        g, dpar, E = sim.adjoint(replica)
        if precision == "fp64":
            E = sim.energy(replica, "fp64")
        ctx.save_for_backward(torch.from_numpy(g).to(p.device, p.dtype),
                              torch.tensor(dpar[2:5], dtype=efield.dtype, device=efield.device))
        return torch.tensor(E, dtype=torch.float64, device=p.device)

    @staticmethod
    def backward(ctx, gE):
        g, dEdE = ctx.saved_tensors
        return gE.to(g.dtype) * g, gE.to(dEdE.dtype) * dEdE, None, None, None, None


def lattice_energy(p, efield, sim, replica=0, lengths=None, precision="fp64"):
    return LatticeEnergy.apply(p, efield, sim, replica, lengths, precision)
