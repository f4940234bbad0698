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
    def forward(ctx, sim, steps, q0, qdot0, f_ext):
        sim.set_state(q0.detach().cpu().double().numpy(), qdot0.detach().cpu().double().numpy())
        sim.set_external_force(f_ext.detach().cpu().double().numpy())
        sim.record(steps)
        sim.step(steps)
        q = sim.history()[:, 1:]
        ctx.sim = sim
        ctx.generation = sim.generation
        ctx.meta = (q0.device, q0.dtype, qdot0.dtype, f_ext.dtype)
        return torch.from_numpy(np.ascontiguousarray(q)).to(device=q0.device, dtype=q0.dtype)

    @staticmethod
    def backward(ctx, grad_q):
        sim = ctx.sim
        if sim.generation != ctx.generation:
            raise RuntimeError("rollout: the simulation was stepped or reset after this rollout; "
                               "its recorded trajectory is gone")
        dev, dq0, dqd0, dfe = ctx.meta
        g0, gd0, gf = sim.backward(grad_q.detach().cpu().double().numpy())
        return (None, None, torch.from_numpy(g0).to(dev, dq0), torch.from_numpy(gd0).to(dev, dqd0),
                torch.from_numpy(gf).to(dev, dfe))


def rollout(sim, q0, qdot0, f_ext, steps):
    """q_1..q_steps (n, steps, 3) of every scene of `sim` (a sdfc.Sim) from joint state
    (q0, qdot0) (n, 3) under external force f_ext (n, 6, world frame, torque then
    force), differentiable with respect to q0, qdot0 and f_ext."""
    return _Rollout.apply(sim, int(steps), q0, qdot0, f_ext)
