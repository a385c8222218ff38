"""torch.autograd.Function around the adjoint kernel: backward against
central finite differences of the forward (FP64 energy), for dipoles and
the applied field."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_autograd_backward_matches_finite_differences(native_lib):
    import torch
    from starrynight_gb300.autograd import lattice_energy
    sn = native_lib
    params = sn.ModelParams(cutoff=4, cage_strain=0.5, efield=(0.05, 0.0, 0.05), dipoles=(1.0, 0.0),
                            prevalence=(0.9, 0.1), seed=31)
    with sn.Simulation(params, [sn.Replica(12, 12, 12, T=300.0, seed=31)]) as sim:
        sim.init_lattice(0)
        sim.sweep(4)
        xyz, ln = sim.download(0)
        p = torch.tensor(xyz, dtype=torch.float64, requires_grad=True)
        ef = torch.tensor([0.05, 0.0, 0.05], dtype=torch.float64, requires_grad=True)
        E = lattice_energy(p, ef, sim, 0, ln)
        E.backward()
        gp, ge = p.grad.numpy(), ef.grad.numpy()

        def f(pp, ee):
            with torch.no_grad():
                return float(lattice_energy(pp, ee, sim, 0, ln))
        rng = np.random.default_rng(0)
        h = 1e-3
        for i in rng.choice(np.nonzero(ln)[0], 24, replace=False):
            for k in range(3):
                q = p.detach().clone()
                a = np.float32(xyz[i, k] + h)
                b = np.float32(xyz[i, k] - h)
                q[i, k] = float(a)
                ep = f(q, ef)
                q[i, k] = float(b)
                em = f(q, ef)
                fd = (ep - em) / (float(a) - float(b))
                assert abs(fd - gp[i, k]) <= 1e-4 * max(1.0, abs(fd)), (i, k, fd, gp[i, k])
        for k in range(3):
            up, dn = ef.detach().clone(), ef.detach().clone()
            a, b = float(np.float32(0.05 * (k != 1) + h)), float(np.float32(0.05 * (k != 1) - h))
            up[k], dn[k] = a, b
            fd = (f(p.detach(), up) - f(p.detach(), dn)) / (a - b)
            assert abs(fd - ge[k]) <= 1e-4 * max(1.0, abs(fd)), (k, fd, ge[k])
        assert np.all(gp[ln == 0] == 0)
