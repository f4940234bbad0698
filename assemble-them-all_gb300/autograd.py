"""Differentiable rollout of batched BDF1 scenes: torch.autograd over sdfc_sim.

The reference differentiates a rollout with Simulation::reset(backward_flag=True),
forward, and Simulation::backward (simulation/redmax/Simulation.cpp:1512-1634,
python_interface.cpp's `backward`).  Here the forward records the joint trajectory
on the device (sdfc_sim_record) and the backward runs sdfc_sim_backward, which
recomputes every step's BDF1 matrices from that trajectory in reverse.
"""
import numpy as np
import torch

__all__ = ["rollout"]


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sim, steps, energy, q0, qdot0, f_ext):
        sim.record_energy(bool(energy))
        sim.set_state(q0.detach().cpu().double().numpy(), qdot0.detach().cpu().double().numpy())
        sim.set_external_force(f_ext.detach().cpu().double().numpy())
        sim.record(steps)
        sim.step(steps)
        q = sim.history()[:, 1:]
        E = sim.energy()[1] if energy else np.zeros(sim.n)
        ctx.sim = sim
        ctx.energy = bool(energy)
        ctx.generation = sim.generation
        ctx.meta = (q0.device, q0.dtype, qdot0.dtype, f_ext.dtype)
        out_q = torch.from_numpy(np.ascontiguousarray(q)).to(device=q0.device, dtype=q0.dtype)
        out_E = torch.from_numpy(E).to(device=q0.device, dtype=q0.dtype)
        return out_q, out_E

    @staticmethod
    def backward(ctx, grad_q, grad_E):
        sim = ctx.sim
        if sim.generation != ctx.generation:
            raise RuntimeError("rollout: the simulation was stepped or reset after this rollout; "
                               "its recorded trajectory is gone")
        dev, dq0, dqd0, dfe = ctx.meta
        gq = np.zeros((sim.n, sim.history().shape[1] - 1, sim.ndof)) if grad_q is None else \
            grad_q.detach().cpu().double().numpy()
        gE = None
        if ctx.energy and grad_E is not None:
            gE = grad_E.detach().cpu().double().numpy()
        g0, gd0, gf = sim.backward(gq, gE)
        return (None, None, None, torch.from_numpy(g0).to(dev, dq0), torch.from_numpy(gd0).to(dev, dqd0),
                torch.from_numpy(gf).to(dev, dfe))


def rollout(sim, q0, qdot0, f_ext, steps, energy=False):
    """q_1..q_steps (n, steps, ndof) of every scene of `sim` (a sdfc.Sim) from joint state
    (q0, qdot0) (n, ndof) under external force f_ext (n, 6, world frame, torque then force),
    differentiable with respect to q0, qdot0 and f_ext.  Also returns the summed penetration
    energy of the steps (n,) (zeros unless `energy`), differentiable the same way."""
    return _Rollout.apply(sim, int(steps), bool(energy), q0, qdot0, f_ext)
