"""Integrator: the z march with the reference's call surface and outputs.

Mirrors ``Integrator`` of the reference (``deliverable (3)/sim/integrator.py``):
``Integrator(cfg, envelope)`` with attributes ``u, rho, rho_s, lin, nl, dz,
dt, g``, ``step(dz)`` (integrator.py:138-149) and ``propagate()``
(integrator.py:151-177: nz+1 iterations of update_plasma then step, a
``_record`` every ``save_stride`` iterations), returning the same result dict
and writing the same ``result.npz`` / ``params.json`` (integrator.py:238-340).
State lives on the GPU as torch tensors (u complex64, rho/rho_s float32); the
per-plane reductions run in one device kernel (nlse_record) with FP64
accumulation, and the z loop between two records is one nlse_propagate call.
"""
import hashlib
import json
import os

import numpy as np
import torch

from ._lib import MODE_PLAIN_F32, MODE_SPLIT_BF16, MODE_SPLIT_F16, Context
from .config import Config, resolved_linear_mode
from .grids import ENVELOPES, build_grids
from .operators import LinearOperator, NonlinearOperator

_MODES = {"plain": MODE_PLAIN_F32, "split_bf16": MODE_SPLIT_BF16, "split_f16": MODE_SPLIT_F16}


def code_fingerprint():
    """Short hash of this implementation's sources (config.py:31-45 of the
    reference hashes its solver files the same way): a cached result is stale
    once any of them changes."""
    here = os.path.dirname(os.path.abspath(__file__))
    h = hashlib.sha256()
    names = sorted(n for n in os.listdir(here) if n.endswith(".py"))
    names += sorted(os.path.join("csrc", n) for n in os.listdir(os.path.join(here, "csrc")))
    for n in names:
        with open(os.path.join(here, n), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:12]


class Integrator:
    def __init__(self, cfg: Config, envelope="gaussian_focused", device=None, ctx=None, g=None):
        """ctx / g: an existing context for this grid (e.g. a batch pulse's)
        and its build_grids() dict; built here when not given."""
        self.cfg = cfg
        if device is not None:
            torch.cuda.set_device(device)
        g = build_grids(cfg) if g is None else g
        self.g = g
        self.dz, self.dt = cfg.dz, g["dt"]
        self.ctx = Context(cfg, g) if ctx is None else ctx
        self.lin = LinearOperator(cfg, g, self.ctx)
        self.nl = NonlinearOperator(cfg, g, self.ctx)
        self.linear_mode = resolved_linear_mode(cfg)
        self.mode = _MODES[self.linear_mode]
        fn = envelope if callable(envelope) else ENVELOPES[envelope]
        u0 = np.asarray(fn(g["rr"], g["tt"], cfg, g), dtype=np.complex128)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.u = torch.from_numpy(u0.astype(np.complex64)).to(dev).contiguous()
        self.Nr, self.Nt = self.u.shape
        self.rho = torch.zeros((self.Nr, self.Nt), dtype=torch.float32, device=dev)
        self.rho_s = torch.zeros((self.Nr, self.Nt), dtype=torch.float32, device=dev)
        self.mask_r = g["mask_r"]
        self.threads = 256
        self.blocks = (self.Nr + self.threads - 1) // self.threads
        r = g["rlist"]
        self._ring = 2.0 * np.pi * r * np.diff(r, prepend=0.0)
        fl0 = np.sum(np.abs(u0) ** 2, axis=1) * self.dt * g["invE2"] * 1e4
        self.U0_uJ = float(np.sum(fl0 * self._ring)) * 1e6
        if cfg.verbose:
            print(f"[init] U_beam(0) = {self.U0_uJ:.3f} uJ ", flush=True)

        n_saves = cfg.nz // cfg.save_stride + 1
        self.n_saves = n_saves
        f32 = dict(dtype=torch.float32, device=dev)
        self.fluence_rz = torch.zeros((n_saves, self.Nr), **f32)
        self.rho_rz = torch.zeros((n_saves, self.Nr), **f32)
        self.rho_s_rz = torch.zeros((n_saves, self.Nr), **f32)
        self.absorbed_rz = torch.zeros((n_saves, self.Nr), **f32)
        self.Ipeak_rz = torch.zeros((n_saves, self.Nr), **f32)
        self.Imax_z = np.zeros(n_saves)
        self.z_saved = np.zeros(n_saves)
        self._dEdz_photo_uJm = np.zeros(n_saves)
        self._dEdz_plasma_uJm = np.zeros(n_saves)
        self.E_STE_z = np.zeros(n_saves)
        self.k_save = 0
        tl_fs = g["tlist"] * 1e15
        self.t_full_fs = tl_fs
        self._t_stride = max(1, cfg.rho_t_stride) if cfg.rho_t_stride > 0 else 0
        self._r_stride = max(1, cfg.rho_r_stride)
        if self._t_stride > 0:
            Nt_sub = (self.Nt - 1) // self._t_stride + 1
            Nr_sub = (self.Nr - 1) // self._r_stride + 1
            self.rho_rzt = np.zeros((n_saves, Nr_sub, Nt_sub), dtype=np.float32)
            self.rho_s_rzt = np.zeros((n_saves, Nr_sub, Nt_sub), dtype=np.float32)
            self.I_rzt = np.zeros((n_saves, Nr_sub, Nt_sub), dtype=np.float32)
            self.t_sub_fs = tl_fs[::self._t_stride]
            self.r_sub = r[::self._r_stride]
        else:
            self.rho_rzt = self.rho_s_rzt = self.I_rzt = self.t_sub_fs = self.r_sub = None
        if cfg.absorb_time_bins_fs:
            edges = np.asarray(cfg.absorb_time_bins_fs, dtype=np.float64)
            if len(edges) - 1 > 8:
                raise ValueError("at most 8 absorption time bins")
            b = np.full(self.Nt, -1, dtype=np.int32)
            for k, (lo, hi) in enumerate(zip(edges[:-1], edges[1:])):
                b[(tl_fs >= lo) & (tl_fs < hi)] = k
            self._bin_of_t = torch.from_numpy(b).to(dev)
            self._nbins = len(edges) - 1
            self.absorb_bin_edges_fs = edges
            self.absorbed_rz_bins = torch.zeros((n_saves, self._nbins, self.Nr), **f32)
        else:
            self._bin_of_t, self._nbins = None, 0
            self.absorb_bin_edges_fs = self.absorbed_rz_bins = None
        if cfg.rho_snapshot_t_fs is not None:
            self._it_snap = int(np.argmin(np.abs(tl_fs - cfg.rho_snapshot_t_fs)))
            self.rho_rz_at = torch.zeros((n_saves, self.Nr), **f32)
        else:
            self._it_snap, self.rho_rz_at = None, None
        self.rho_onaxis_t = np.zeros((n_saves, self.Nt), dtype=np.float32)
        self.rho_s_onaxis_t = np.zeros((n_saves, self.Nt), dtype=np.float32)
        self.I_onaxis_t = np.zeros((n_saves, self.Nt), dtype=np.float32)
        self._rec = torch.zeros((self.Nr, 6 + self._nbins), dtype=torch.float64, device=dev)

    # ------------------------------------------------------------------ stepping
    def step(self, dz):
        """Integrator.step: half-linear, nonlinear block, half-linear, mask_r (rho frozen)."""
        self.ctx.step(self.u, self.rho, dz, self.mode, self.rho_s)

    def advance(self, nsteps):
        """nsteps iterations of update_plasma + step, queued without host syncs."""
        self.ctx.propagate(self.u, self.rho, self.rho_s, self.dz, nsteps, self.mode)

    def chunks(self):
        """The z loop of Integrator.propagate (integrator.py:151-177) as
        (n, z_record, i) chunks: advance n iterations, then record the plane
        at z_record (None: no record); i = the last iteration's index.  The
        reference records after iterations 0, stride, 2 stride, ..."""
        cfg = self.cfg
        total, stride = cfg.nz + 1, max(1, int(cfg.save_stride))
        done = 0
        while done < total:
            n = 1 if done == 0 else min(stride, total - done)
            done += n
            i = done - 1
            yield n, (cfg.begin + i * self.dz if i % stride == 0 else None), i

    def after_chunk(self, z_record, i):
        """Record (and report) after a chunk of chunks()."""
        cfg = self.cfg
        if z_record is not None:
            self._record(z_record)
        if cfg.verbose and i > 0 and i % cfg.ckpt_every == 0 and self.k_save:
            k = self.k_save - 1
            flu = self.fluence_rz[k].double().cpu().numpy()
            pct = float(np.sum(flu * self._ring)) * 100.0 / self.U0_uJ * 100.0
            print(f"[z] {(cfg.begin + i * self.dz) * 1e6:+.0f} um  U {pct:.1f} %  "
                  f"I_peak {self.Imax_z[k]:.2e}", flush=True)

    def propagate(self):
        for n, z_rec, i in self.chunks():
            self.advance(n)
            self.after_chunk(z_rec, i)
        return self._results()

    # ------------------------------------------------------------------ recording
    def _record(self, z_now):
        k, g = self.k_save, self.g
        invE2, dt = g["invE2"], self.dt
        self.ctx.record(self.u, self.rho, self.rho_s, self._bin_of_t, self._nbins, self._rec)
        rec = self._rec
        self.fluence_rz[k] = (rec[:, 0] * dt * invE2).float()
        self.rho_rz[k] = rec[:, 1].float()
        self.rho_s_rz[k] = rec[:, 2].float()
        self.Ipeak_rz[k] = (rec[:, 3] * invE2).float()
        self.absorbed_rz[k] = ((rec[:, 4] + rec[:, 5]) * invE2 * dt * 100.0).float()
        if self._nbins:
            self.absorbed_rz_bins[k] = (rec[:, 6:].T * invE2 * dt * 100.0).float()
        if self._it_snap is not None:
            self.rho_rz_at[k] = self.rho[:, self._it_snap]
        host = rec.cpu().numpy()
        self.Imax_z[k] = float(host[:, 3].max() * invE2)
        self.z_saved[k] = float(z_now)
        self._dEdz_photo_uJm[k] = float(np.sum(host[:, 4] * invE2 * dt * self._ring)) * 1e4 * 1e6
        self._dEdz_plasma_uJm[k] = float(np.sum(host[:, 5] * invE2 * dt * self._ring)) * 1e4 * 1e6
        I0 = (self.u[0].real.float() ** 2 + self.u[0].imag.float() ** 2) * invE2
        self.rho_onaxis_t[k] = self.rho[0].cpu().numpy()
        self.rho_s_onaxis_t[k] = self.rho_s[0].cpu().numpy()
        self.I_onaxis_t[k] = I0.cpu().numpy()
        if self._t_stride > 0:
            rs, ts = self._r_stride, self._t_stride
            self.rho_rzt[k] = self.rho[::rs, ::ts].cpu().numpy()
            self.rho_s_rzt[k] = self.rho_s[::rs, ::ts].cpu().numpy()
            Is = self.u[::rs, ::ts]
            self.I_rzt[k] = ((Is.real.float() ** 2 + Is.imag.float() ** 2) * invE2).cpu().numpy()
        self.k_save += 1

    def _cumulative_energy_fraction(self, dEdz_uJm):
        """Trapezoidal cumulative integral of dE/dz over z_saved, / U0 (integrator.py:226-236)."""
        z = self.z_saved[:self.k_save]
        d = dEdz_uJm[:self.k_save]
        if len(z) < 2:
            return np.zeros_like(d)
        seg = 0.5 * (d[:-1] + d[1:]) * np.diff(z)
        return np.concatenate([[0.0], np.cumsum(seg)]) / self.U0_uJ

    def _results(self):
        cfg, g, k = self.cfg, self.g, self.k_save

        def mirror(a):
            return np.hstack([a[:, ::-1], a])

        r = g["rlist"]
        flu = self.fluence_rz[:k].cpu().numpy()
        rho = self.rho_rz[:k].cpu().numpy()
        rho_s = self.rho_s_rz[:k].cpu().numpy()
        E_MPI = self._cumulative_energy_fraction(self._dEdz_photo_uJm)
        E_pl = self._cumulative_energy_fraction(self._dEdz_plasma_uJm)
        out = dict(
            r=np.concatenate([-r[::-1], r]), rlist=r, z=self.z_saved[:k],
            fluence_rz=mirror(flu), rho_rz=mirror(rho), rho_s_rz=mirror(rho_s), Imax_z=self.Imax_z[:k],
            E_plasma_z=E_pl, E_MPI_z=E_MPI, E_STE_z=self.E_STE_z[:k], E_total_z=E_MPI + E_pl,
            rho_rzt=self.rho_rzt[:k] if self.rho_rzt is not None else None,
            rho_s_rzt=self.rho_s_rzt[:k] if self.rho_s_rzt is not None else None,
            I_rzt=self.I_rzt[:k] if self.I_rzt is not None else None,
            t_sub_fs=self.t_sub_fs, r_sub=self.r_sub,
            absorbed_rz=mirror(self.absorbed_rz[:k].cpu().numpy()),
            Ipeak_rz=mirror(self.Ipeak_rz[:k].cpu().numpy()),
            rho_rz_at=mirror(self.rho_rz_at[:k].cpu().numpy()) if self.rho_rz_at is not None else None,
            absorbed_rz_bins=(np.stack([mirror(self.absorbed_rz_bins[:k, b].cpu().numpy())
                                        for b in range(self._nbins)], axis=1) if self._nbins else None),
            absorb_bin_edges_fs=self.absorb_bin_edges_fs,
            rho_onaxis_t=self.rho_onaxis_t[:k], rho_s_onaxis_t=self.rho_s_onaxis_t[:k],
            I_onaxis_t=self.I_onaxis_t[:k], t_full_fs=self.t_full_fs,
        )
        if cfg.out_dir:
            os.makedirs(cfg.out_dir, exist_ok=True)
            final = os.path.join(cfg.out_dir, "result.npz")
            tmp = final + ".tmp.npz"
            try:
                np.savez_compressed(tmp, **out)
                os.replace(tmp, final)
            except BaseException:
                if os.path.exists(tmp):
                    os.remove(tmp)
                raise
            self._dump_params()
        return out

    def _dump_params(self):
        """params.json (integrator.py:300-340): probe optics, toggles, fingerprint."""
        cfg = self.cfg
        params = dict(
            n0=cfg.n0, n0_probe=cfg.n0_probe, nc_probe_cm3=cfg.nc_probe, lambda_probe_nm=cfg.lambda_probe * 1e9,
            wavelength_nm=cfg.wavelength * 1e9, n2=cfg.n2, U_g_eV=cfg.Ui_eV, Us_eV=cfg.Us_eV,
            energy_uJ=cfg.energy_uJ, w0_um=cfg.w0 * 1e6, delta_t_fs=cfg.delta_t * 1e15,
            code_fingerprint=code_fingerprint(), begin_um=cfg.begin * 1e6, end_um=cfg.end * 1e6,
            z_focus_air_um=cfg.z_focus_air_um,
            toggles=dict(
                enable_kerr_instantaneous=cfg.enable_kerr_instantaneous, enable_kerr_raman=cfg.enable_kerr_raman,
                enable_self_steepening=cfg.enable_self_steepening,
                enable_photoionization_loss=cfg.enable_photoionization_loss,
                enable_plasma_defocusing=cfg.enable_plasma_defocusing,
                enable_plasma_absorption=cfg.enable_plasma_absorption,
                enable_space_time_focusing=cfg.enable_space_time_focusing,
                enable_spectral_filter=cfg.enable_spectral_filter,
                tau_ste_fs=(cfg.tau_ste * 1e15 if cfg.tau_ste else None), enable_ste_index=cfg.enable_ste_index,
                E_tr_eV=cfg.E_tr_eV, f_ste_pump=float(self.g["f_ste"]), enable_avalanche=cfg.enable_avalanche,
                enable_recombination=cfg.enable_recombination, enable_ste=cfg.enable_ste,
            ),
            linear_mode=self.linear_mode, rate_model=cfg.rate_model,
        )
        with open(os.path.join(cfg.out_dir, "params.json"), "w") as f:
            json.dump(params, f, indent=2)
