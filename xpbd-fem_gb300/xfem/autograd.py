"""torch.autograd binding of the substep adjoint (xfem_adjoint_forward /
xfem_adjoint_backward in libxfem.so).

    traj, x1, v1 = xfem.autograd.substeps(body, mu, x0, v0, substeps, dt, tips)

runs `substeps` substeps of the handle from positions x0 and velocities v0
with per-tet shear modulus mu (all in the handle's concatenated caller order)
and returns the tip trajectory (substeps, len(tips), 3) and the final state.
Backpropagating through any of them calls the CUDA reverse pass and yields
dL/dmu, dL/dx0 and dL/dv0. The inverse masses are the handle's current ones
(a lock zeroes a vertex's inverse mass at the end of the first substep in
which it is applied, as the reference does). torch carries the tensors; the
forward and reverse passes both run in libxfem.so.
"""
import numpy as np
import torch


def _np(t):
    return None if t is None else t.detach().to("cpu", torch.float32).contiguous().numpy()


def _gather(body, fn):
    return np.concatenate([fn(b) for b in range(body.nbodies)], axis=0)


class Substeps(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mu, x0, v0, body, substeps, dt, tips, checkpoint_every):
        mu_h, x_h, v_h = _np(mu), _np(x0).reshape(-1, 3), _np(v0).reshape(-1, 3)
        vo = to = 0
        for b, (nv, nt) in enumerate(body.counts):
            body.set_tet_mu(mu_h[to:to + nt], b)
            body.set_positions(x_h[vo:vo + nv], b)
            body.set_velocities(v_h[vo:vo + nv], b)
            vo += nv
            to += nt
        traj = body.adjoint_forward(substeps, dt, tips, checkpoint_every)
        x1 = _gather(body, body.positions)
        v1 = _gather(body, body.velocities)
        ctx.body = body
        ctx.shape = (substeps, len(tips))
        dev = mu.device
        return torch.from_numpy(traj).to(dev), torch.from_numpy(x1).to(dev), torch.from_numpy(v1).to(dev)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, g_traj, g_x, g_v):
        g = _np(g_traj)
        if g is None:
            g = np.zeros(ctx.shape + (3,), np.float32)
        dmu, dx, dv = ctx.body.adjoint_backward(g, _np(g_x), _np(g_v))
        dev = g_traj.device if g_traj is not None else (g_x if g_x is not None else g_v).device
        return (torch.from_numpy(dmu).to(dev), torch.from_numpy(dx).to(dev), torch.from_numpy(dv).to(dev),
                None, None, None, None, None)


def substeps(body, mu, x0, v0, substeps, dt, tips, checkpoint_every=0):
    """Differentiable run of `substeps` substeps; see the module docstring."""
    return Substeps.apply(mu, x0, v0, body, int(substeps), float(dt), np.asarray(tips, np.uint32),
                          int(checkpoint_every))
