"""Integrator: the z march with the reference's call surface.

Mirrors ``Integrator`` of the reference (``deliverable (3)/sim/integrator.py``):
``Integrator(cfg, envelope)`` with attributes ``u, rho, rho_s, lin, nl, dz,
dt, g``, ``step(dz)`` (integrator.py:138-149) and ``propagate()``
(integrator.py:151-177: nz+1 iterations of update_plasma then step).  The
state lives on the GPU as torch tensors (u complex64, rho/rho_s float32).
Per-save diagnostics are a subset of the reference's _record (fluence, peak
density and peak intensity per saved plane).
"""
import numpy as np
import torch

from ._lib import MODE_PLAIN_F32, MODE_SPLIT_BF16, Context
from .config import Config
from .grids import ENVELOPES, build_grids
from .operators import LinearOperator, NonlinearOperator

_MODES = {"plain": MODE_PLAIN_F32, "split_bf16": MODE_SPLIT_BF16}


class Integrator:
    def __init__(self, cfg: Config, envelope="gaussian_focused", device=None):
        self.cfg = cfg
        if device is not None:
            torch.cuda.set_device(device)
        g = build_grids(cfg)
        self.g = g
        self.dz, self.dt = cfg.dz, g["dt"]
        self.ctx = Context(cfg, g)
        self.lin = LinearOperator(cfg, g, self.ctx)
        self.nl = NonlinearOperator(cfg, g, self.ctx)
        self.mode = _MODES[cfg.linear_mode]
        fn = envelope if callable(envelope) else ENVELOPES[envelope]
        u0 = np.asarray(fn(g["rr"], g["tt"], cfg, g), dtype=np.complex128)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.u = torch.from_numpy(u0.astype(np.complex64)).to(dev).contiguous()
        self.Nr, self.Nt = self.u.shape
        self.rho = torch.zeros((self.Nr, self.Nt), dtype=torch.float32, device=dev)
        self.rho_s = torch.zeros((self.Nr, self.Nt), dtype=torch.float32, device=dev)
        self.mask_r = g["mask_r"]
        self.threads = 256
        self.blocks = (self.Nr + self.threads - 1) // self.threads
        r = g["rlist"]
        self._ring = torch.tensor(2.0 * np.pi * r * np.diff(r, prepend=0.0), dtype=torch.float64, device=dev)
        fl0 = np.sum(np.abs(u0) ** 2, axis=1) * self.dt * g["invE2"] * 1e4
        self.U0_uJ = float(np.sum(fl0 * 2.0 * np.pi * r * np.diff(r, prepend=0.0))) * 1e6
        if cfg.verbose:
            print(f"[init] U_beam(0) = {self.U0_uJ:.3f} uJ ", flush=True)

    def step(self, dz):
        """Integrator.step: half-linear, nonlinear block, half-linear, mask_r (rho frozen)."""
        self.ctx.step(self.u, self.rho, dz, self.mode)

    def advance(self, nsteps):
        """nsteps iterations of update_plasma + step, queued without host syncs."""
        self.ctx.propagate(self.u, self.rho, self.rho_s, self.dz, nsteps, self.mode)

    def _record(self, z_now, rec):
        I = self.u.real.double() ** 2 + self.u.imag.double() ** 2
        rec["fluence_rz"].append((I.sum(dim=1) * self.dt * self.g["invE2"]).float())
        rec["rho_rz"].append(self.rho.max(dim=1).values)
        rec["Imax_z"].append(I.max() * self.g["invE2"])
        rec["z"].append(z_now)

    def propagate(self):
        cfg = self.cfg
        rec = dict(fluence_rz=[], rho_rz=[], Imax_z=[], z=[])
        stride = max(1, int(cfg.save_stride))
        done = 0
        total = cfg.nz + 1
        while done < total:
            n = min(stride, total - done) if done > 0 else 1
            self.advance(n)
            done += n
            if (done - 1) % stride == 0:
                self._record(cfg.begin + (done - 1) * self.dz, rec)
        r = self.g["rlist"]
        flu = torch.stack(rec["fluence_rz"]).cpu().numpy()
        rho = torch.stack(rec["rho_rz"]).cpu().numpy()
        return dict(
            r=np.concatenate([-r[::-1], r]), rlist=r, z=np.asarray(rec["z"]),
            fluence_rz=np.hstack([flu[:, ::-1], flu]), rho_rz=np.hstack([rho[:, ::-1], rho]),
            Imax_z=torch.stack(rec["Imax_z"]).cpu().numpy(), t_full_fs=self.g["tlist"] * 1e15,
            u=self.u.cpu().numpy(), rho=self.rho.cpu().numpy(),
        )
