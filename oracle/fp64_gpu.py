"""FP64 GPU restatement of the propagator, for long runs (1 cm = thousands of steps).

TEST INFRASTRUCTURE (part of the oracle).  The numpy oracle takes ~5 s per
z-step at 1024 x 2048; this restatement runs the same FP64 algorithm with
torch float64/complex128 on the GPU (cuBLAS DGEMM for the two real Hankel
products, cuFFT Z2Z for the t transforms) and the FP64 CUDA restatement of the
carrier march (oracle/rate_scan_gpu.cu).  It is pinned against the numpy
oracle by tests/test_gpu_accuracy.py before it is used as the long-run FP64
reference.  Only tests may use it; it never runs on the product path.

Follows (paths under ``deliverable (3)/sim``): half_linear operators.py:47-53,
split operators.py:89-146 with the measured toggles (Raman, self-steepening and
the exciton channel off) and optionally space-time focusing (the Omega-
dependent diffraction phase of half_linear, operators.py:50, and the U^-1
filter of split, operators.py:141-144), update_plasma operators.py:165-183 +
kernels.py:36-106, step integrator.py:138-149.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def _load():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle_scan_gpu.so")
        if not os.path.exists(path):
            import subprocess
            subprocess.check_call(["make", "-s", "-C", HERE, "liboracle_scan_gpu.so"])
        lib = ctypes.CDLL(path)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.oracle_rate_scan_gpu.argtypes = [P, P, I, I, D, D, D, D, D, P, I, D, D, D, D, P]
        lib.oracle_rate_scan_gpu.restype = I
        _lib = lib
    return _lib


class FP64GPU:
    """FP64 propagator on the GPU built from an oracle.nlse_oracle.OracleGrid."""

    def __init__(self, og, device="cuda"):
        import torch
        p = og.p
        for k in ("enable_kerr_raman", "enable_self_steepening", "enable_ste"):
            if p[k]:
                raise NotImplementedError(f"{k} is not restated here")
        self.t = torch
        self.og = og
        self.dev = torch.device(device)
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.Y = torch.tensor(og.Y, **f64)
        self.Rk, self.iRk = og.Rk, og.iRk
        self.delta_k = torch.tensor(og.delta_k, **f64)
        self.spec_mask = torch.tensor(og.spec_mask, **f64)
        self.rho2 = torch.tensor(og.rholist, **f64) ** 2
        self.mask_r = torch.tensor(og.mask_r, **f64)
        sp = og.f_spline
        self.knots = torch.tensor(og.I_tab, **f64)
        self.coef = torch.tensor(sp.c, **f64)  # (4, n-1), scipy PPoly order
        self.lut = torch.tensor(og.W_LUT, **f64)
        from scipy.constants import c, epsilon_0
        self.photo_k = 1e6 * og.Ui / (og.n0 * c * epsilon_0)
        self.kp = og.kerr_pref * ((1.0 - p["f_R"]) if p["enable_kerr_instantaneous"] else 0.0)
        self.pp = og.plasma_pref
        self.w0tc = og.omega0 * p["tau_c"]
        self.on_photo = bool(p["enable_photoionization_loss"])
        self.on_abs = bool(p["enable_plasma_absorption"])
        self.on_def = bool(p["enable_plasma_defocusing"])
        self.rho_max = p["rho_max"]
        self.stf = bool(p["enable_space_time_focusing"])
        self.inv_U_op = torch.tensor(og.inv_U_op, **f64)
        self.inv_U_nl = torch.tensor(og.inv_U_nl, **f64)
        self._phase_dz = None

    def _phase(self, dz):
        if self._phase_dz != dz:
            t = self.t
            # operators.py:50: the radial phase carries U^-1(Omega) with space-time focusing
            ph = (self.delta_k[None, :] - self.rho2[:, None] / (2 * self.og.komega) * self.inv_U_op[None, :]) * dz / 2
            self._P = t.exp(1j * ph) * self.spec_mask[None, :]
            self._phase_dz = dz
        return self._P

    def half_linear(self, u, dz):
        t = self.t
        Yu = t.complex(self.Y @ u.real.contiguous(), self.Y @ u.imag.contiguous()) * self.Rk
        f = t.fft.ifft(t.fft.fft(Yu, dim=1) * self._phase(dz), dim=1)
        return t.complex(self.Y @ f.real.contiguous(), self.Y @ f.imag.contiguous()) * self.iRk

    def _pchip(self, I):
        t = self.t
        x = t.clamp(I, self.og.Imin, self.og.Imax)
        i = t.clamp(t.searchsorted(self.knots, x, right=True) - 1, 0, self.knots.numel() - 2)
        s = x - self.knots[i]
        c = self.coef[:, i]
        v = ((c[0] * s + c[1]) * s + c[2]) * s + c[3]
        return t.nan_to_num(v.abs(), nan=0.0, posinf=0.0, neginf=0.0)

    def split(self, u, rho):
        t = self.t
        a2 = u.real**2 + u.imag**2
        if self.on_photo:
            W = self._pchip(a2 * self.og.invE2)
            dep = t.clamp(1.0 - rho / self.rho_max, 0.0, 1.0)
            photo = W * self.photo_k / (a2 + 1e-30) * dep
        else:
            photo = t.zeros_like(a2)
        araw = photo + (self.pp * rho if self.on_abs else 0.0)
        alpha = t.clamp(t.nan_to_num(araw, nan=0.0, posinf=0.0, neginf=0.0), min=0.0)
        coeff = complex((1.0 if self.on_abs else 0.0), (self.w0tc if self.on_def else 0.0))
        X = 1j * self.kp * a2 * u - photo * u - self.pp * coeff * rho * u
        if self.stf:
            # operators.py:141-144: the nonlinear polarisation through U^-1 (T-hat = 1)
            X = t.fft.ifft(t.fft.fft(X, dim=1) * self.inv_U_nl[None, :], dim=1)
        rhs = X + alpha * u
        rhs = t.where(a2 < 1e-30, t.zeros_like(rhs), rhs)
        return t.nan_to_num(rhs, nan=0.0, posinf=0.0, neginf=0.0), alpha

    def update_plasma(self, u, rho):
        og = self.og
        u = u.contiguous()
        st = self.t.cuda.current_stream().cuda_stream
        r = _load().oracle_rate_scan_gpu(
            ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(rho.data_ptr()), u.shape[0], u.shape[1], og.dt,
            og.invE2, og.avalanche_coef, self.rho_max, og.inv_taur_eff, ctypes.c_void_p(self.lut.data_ptr()),
            self.lut.numel(), og.logImin, og.inv_dlog, og.Imin, og.Imax, ctypes.c_void_p(st))
        if r != 0:
            raise RuntimeError(f"oracle scan launch failed ({r})")

    def step(self, u, rho, dz):
        t = self.t
        u = self.half_linear(u, dz)
        _, a = self.split(u, rho)
        u = u * t.exp(-0.5 * dz * a)
        k1, _ = self.split(u, rho)
        k2, _ = self.split(u + 0.5 * dz * k1, rho)
        k3, _ = self.split(u + 0.5 * dz * k2, rho)
        k4, _ = self.split(u + dz * k3, rho)
        u = u + dz / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        _, a = self.split(u, rho)
        u = u * t.exp(-0.5 * dz * a)
        return self.half_linear(u, dz) * self.mask_r[:, None]

    def propagate(self, u0, nsteps, dz):
        t = self.t
        u = t.tensor(u0, dtype=t.complex128, device=self.dev)
        rho = t.zeros(u.shape, dtype=t.float64, device=self.dev)
        for _ in range(nsteps):
            self.update_plasma(u, rho)
            u = self.step(u, rho, dz)
        return u, rho
