"""torch.autograd.Function around the C-ABI advection adjoint (test harness
only).  Inputs are compact periodic CUDA tensors indexed [i, j, k]; the
objective is J = sum (H(phi_T) - H(phi_target))^2 dV after `n_steps`
WENO5 / TVD-RK3 advection steps; backward returns dJ/dphi and dJ/dvel_*
scaled by the incoming gradient."""
import torch

import lsmlib_gb300 as L


def _ghosted(t):
    """[i, j, k] tensor -> C-ordered tensor of the Fortran ghost-box array
    (3 ghost cells of zeros), i.e. indexed [k, j, i]."""
    nx, ny, nz = t.shape
    out = torch.zeros((nz + 6, ny + 6, nx + 6), dtype=t.dtype, device=t.device)
    out[3:-3, 3:-3, 3:-3] = t.permute(2, 1, 0)
    return out


def _interior(t):
    return t[3:-3, 3:-3, 3:-3].permute(2, 1, 0).contiguous()


class AdvectObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phi, vx, vy, vz, target, spacing, dt, n_steps, eps, ckpt):
        precision = "f64" if phi.dtype == torch.float64 else "f32"
        nx, ny, nz = phi.shape
        gb = (-3, nx + 2, -3, ny + 2, -3, nz + 2)
        fb = (0, nx - 1, 0, ny - 1, 0, nz - 1)
        args = [_ghosted(x.detach()) for x in (phi, vx, vy, vz, target)]
        J, gp, gv = L.advect_adjoint_weno5_tvdrk3(args[0], gb, fb, args[1:4], gb, args[4], spacing[0], dt, n_steps,
                                                  eps, checkpoint_every=ckpt, precision=precision,
                                                  dy=spacing[1], dz=spacing[2])
        torch.cuda.synchronize()
        ctx.save_for_backward(_interior(gp), *[_interior(g) for g in gv])
        return torch.tensor(J, dtype=torch.float64, device=phi.device)

    @staticmethod
    def backward(ctx, gJ):
        gp, gx, gy, gz = ctx.saved_tensors
        s = gJ.to(gp.dtype)
        return gp * s, gx * s, gy * s, gz * s, None, None, None, None, None, None


class Reinit(torch.autograd.Function):
    """phi -> phi_T after `n_iter` periodic reinitialization iterations (phi0
    sign form); backward through the C-ABI vector-Jacobian product."""

    @staticmethod
    def forward(ctx, phi, spacing, dtau, n_iter, ckpt):
        precision = "f64" if phi.dtype == torch.float64 else "f32"
        nx, ny, nz = phi.shape
        gb = (-3, nx + 2, -3, ny + 2, -3, nz + 2)
        fb = (0, nx - 1, 0, ny - 1, 0, nz - 1)
        g = _ghosted(phi.detach())
        out, _ = L.reinit_vjp_weno5_tvdrk3(g, gb, fb, None, spacing[0], dtau, n_iter, checkpoint_every=ckpt,
                                           precision=precision, dy=spacing[1], dz=spacing[2])
        torch.cuda.synchronize()
        ctx.save_for_backward(phi.detach())
        ctx.args = (spacing, dtau, n_iter, ckpt, precision, gb, fb)
        return _interior(out)

    @staticmethod
    def backward(ctx, gout):
        (phi,) = ctx.saved_tensors
        spacing, dtau, n_iter, ckpt, precision, gb, fb = ctx.args
        _, gp = L.reinit_vjp_weno5_tvdrk3(_ghosted(phi), gb, fb, _ghosted(gout.contiguous()), spacing[0], dtau,
                                          n_iter, checkpoint_every=ckpt, precision=precision, dy=spacing[1],
                                          dz=spacing[2])
        torch.cuda.synchronize()
        return _interior(gp), None, None, None, None
