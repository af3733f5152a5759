"""Split-step operators with the reference's call surface, on the GPU.

``LinearOperator.half_linear`` and ``NonlinearOperator.split`` /
``update_plasma`` keep the signatures and semantics of the reference
(``deliverable (3)/sim/operators.py:22-183``): half_linear and split are pure
(return new tensors), update_plasma mutates rho and rho_s in place and accepts
(and ignores) the CUDA launch geometry arguments.  The arithmetic runs in the
sm_103a kernels of libnlse (FP32 fields, complex64 / float32 tensors).
"""
import torch

from ._lib import Context


class LinearOperator:
    """Diffraction + dispersion half step (operators.py:22-53)."""

    def __init__(self, cfg, g, ctx=None):
        self.ctx = ctx if ctx is not None else Context(cfg, g)
        self.komega = g["komega"]
        self.Y = g["Y"]
        self.j1last = g["j1last"]
        self.R = g["R"]
        self.Rk = self.R**2 / self.j1last
        self.iRk = self.j1last / self.R**2
        self.rhorho = g["rhorho"]
        self.delta_k = g["delta_k"]
        self.inv_U_op = g["inv_U_op"]
        self.spec_mask = g["spec_mask"]

    def half_linear(self, u, dz):
        out = u.clone(memory_format=torch.contiguous_format)
        self.ctx.half_linear(out, dz)
        return out


class NonlinearOperator:
    """Kerr / photo-ionisation / plasma terms and the carrier update (operators.py:58-183)."""

    def __init__(self, cfg, g, ctx=None):
        self.ctx = ctx if ctx is not None else Context(cfg, g)
        self.n0, self.Ui, self.f_R = cfg.n0, cfg.Ui, cfg.f_R
        self.invE2 = g["invE2"]
        self.rho_max = cfg.rho_max
        self.enable_ste = int(cfg.enable_ste)

    def split(self, u, rho, rho_s=None):
        """-> (rhs, alpha): RK right-hand side and absorption rate (operators.py:89-146)."""
        u = u.contiguous()
        rho = rho.contiguous()
        rho_s = rho_s.contiguous() if (rho_s is not None and self.enable_ste) else None
        rhs = torch.empty_like(u)
        alpha = torch.empty(u.shape, dtype=torch.float32, device=u.device)
        self.ctx.split(u, rho, rhs, alpha, rho_s)
        return rhs, alpha

    def update_plasma(self, u, rho, rho_s, dt=None, blocks=None, threads=None):
        """rho[:,0] = 0 then the carrier march along t (operators.py:165-183).
        Mutates rho and rho_s in place; dt/blocks/threads are accepted for
        signature compatibility (dt is fixed by the grid)."""
        self.ctx.update_plasma(u, rho, rho_s)

    def nonlinear_step(self, u, rho, dz, rho_s=None):
        """The alpha/2 + RK4 + alpha/2 block of Integrator.step, in place."""
        self.ctx.nonlinear_step(u, rho, dz, rho_s if self.enable_ste else None)
        return u
