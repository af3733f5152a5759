"""FP64 CPU oracle for the axisymmetric split-step NLSE propagator.

TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import this module, and only as the checker
(or as the timed CPU stand-in for the reference).  It never runs on the
product path.

It restates, in numpy (complex128 / float64), the reference solver's hot path
(paths relative to ``.github/deliverable (3)/sim``):

* grid/operator construction   ``grids.py:29-175`` (``build_grids``)
* derived constants            ``config.py:202-241`` (``Config.__post_init__``)
* linear half step             ``operators.py:47-53`` (``LinearOperator.half_linear``)
* nonlinear right-hand side    ``operators.py:89-146`` (``NonlinearOperator.split``)
* carrier update               ``operators.py:165-183`` + ``kernels.py:36-106``
                               (C restatement in ``oracle/rate_scan.c``)
* Strang step                  ``integrator.py:138-149`` (``Integrator.step``)

Parity is pinned against golden fixtures generated from the reference itself
(``tests/golden/make_golden.py``), see ``tests/test_oracle_golden.py``.

The photo-ionisation rate source is a callable ``rate(I_Wcm2) -> cm^-3 s^-1``;
the measured workloads use the K-photon power law ``sigma_K I^K rho_nt``.
"""
import ctypes
import math
import os

import numpy as np
from scipy.constants import c, epsilon_0, m_e
from scipy.constants import elementary_charge as q_e
from scipy.interpolate import PchipInterpolator
from scipy.special import j0, j1, jn_zeros

HERE = os.path.dirname(os.path.abspath(__file__))

# Fused-silica Sellmeier coefficients (keldysh.py:22-23).
SELLMEIER_B = np.array([0.6961663, 0.4079426, 0.8974794])
SELLMEIER_L2 = np.array([0.0684043, 0.1162414, 9.896161]) ** 2


def n_sellmeier(lam_m):
    """keldysh.py:25-29."""
    lu2 = (lam_m * 1e6) ** 2
    return float(np.sqrt(1.0 + sum(b * lu2 / (lu2 - l2) for b, l2 in zip(SELLMEIER_B, SELLMEIER_L2))))


class MPIPowerLaw:
    """Photo-ionisation rate W = sigma_K I^K rho_nt in cm^-3 s^-1 (I in W/cm^2)."""

    def __init__(self, sigma_K=1e-71, K=6, rho_nt=2.1e22):
        self.sigma_K, self.K, self.rho_nt = sigma_K, K, rho_nt

    def __call__(self, I):
        return self.sigma_K * np.asarray(I, dtype=np.float64) ** self.K * self.rho_nt


_DEFAULTS = dict(
    Nt=4096, N=1025, R_factor=40.0, w0=10e-6, delta_t=263e-15, wavelength=1030e-9,
    n2=2.4e-20, Ui_eV=9.0, meff_drude_rel=1.0, tau_c=1.7e-15, tau_r=330e-15, f_R=0.18,
    tau_d=32e-15, tau_s=12e-15, rho_max=2.1e22, Us_eV=6.0, enable_ste=True, tau_ste=None,
    enable_kerr_instantaneous=True, enable_kerr_raman=True, enable_self_steepening=True,
    enable_photoionization_loss=True, enable_plasma_defocusing=True,
    enable_plasma_absorption=True, enable_space_time_focusing=True,
    enable_spectral_filter=True, enable_ste_index=True, E_tr_eV=4.2,
    enable_avalanche=True, enable_recombination=True,
)


class OracleGrid:
    """Everything ``build_grids`` + the operator constructors precompute (FP64).

    ``cfg`` is any object (or dict) carrying the reference ``Config`` field
    names; only primary fields are read and every derived constant is
    recomputed here (config.py:202-241, grids.py:29-175, operators.py:35-87).
    """

    def __init__(self, cfg, rate=None):
        get = (lambda k: cfg[k] if k in cfg else _DEFAULTS[k]) if isinstance(cfg, dict) else \
            (lambda k: getattr(cfg, k, _DEFAULTS.get(k)))
        self.p = {k: get(k) for k in _DEFAULTS}
        p = self.p
        lam = p["wavelength"]
        self.Nt, self.N = int(p["Nt"]), int(p["N"])
        self.Nr = self.N - 1
        # config.py:203-224
        self.omega0 = 2 * np.pi * c / lam
        self.frequency = c / lam
        self.n0 = n_sellmeier(lam)
        self.Ui = p["Ui_eV"] * q_e
        self.Us = p["Us_eV"] * q_e
        self.chi3 = 4 / 3 * epsilon_0 * self.n0**2 * c * p["n2"]
        self.komega = 2 * np.pi / lam * self.n0
        self.Omega_r2 = 1.0 / p["tau_s"] ** 2 + 1.0 / p["tau_d"] ** 2
        # time axis, grids.py:32-36
        tp = p["delta_t"] / np.sqrt(2 * np.log(2))
        tmax = 5 * tp
        self.dt = float(tmax * 2 / self.Nt)
        self.tlist = np.linspace(-tmax, tmax, self.Nt, endpoint=False)
        self.ff = np.fft.fftfreq(self.Nt, d=self.dt)
        # quasi-discrete Hankel transform, grids.py:38-44
        N = self.N
        jz = jn_zeros(0, N)
        self.jz = jz
        self.R = p["R_factor"] * p["w0"]
        jl = jz[:N - 1]
        # Y[i, k] = 2/j_N / J1(j_k)^2 * J0(j_i j_k / j_N)   (column-scaled kernel)
        self.Y = (2 / jz[N - 1]) / j1(jl)[None, :] ** 2 * j0(np.outer(jl, jl) / jz[N - 1])
        self.rlist = jl * self.R / jz[N - 1]
        self.rholist = jl / self.R
        self.Rk = self.R**2 / jz[N - 1]
        self.iRk = jz[N - 1] / self.R**2
        # Sellmeier dispersion, grids.py:46-60
        w_lo, w_hi = 2 * np.pi * c / 5.0e-6, 2 * np.pi * c / 0.18e-6
        omega_safe = np.clip(self.omega0 + 2 * np.pi * self.ff, w_lo, w_hi)
        lam_um = 2 * np.pi * c / omega_safe * 1e6
        n2m1 = sum(b * lam_um**2 / (lam_um**2 - l2) for b, l2 in zip(SELLMEIER_B, SELLMEIER_L2))

        def k_of(w):
            lu = 2 * np.pi * c / w * 1e6
            return (w / c) * np.sqrt(1.0 + sum(b * lu**2 / (lu**2 - l2)
                                               for b, l2 in zip(SELLMEIER_B, SELLMEIER_L2)))
        dw = self.omega0 / 1000.0
        self.k1 = (k_of(self.omega0 + dw) - k_of(self.omega0 - dw)) / (2 * dw)
        self.delta_k = (omega_safe / c) * np.sqrt(1.0 + n2m1) - self.komega - self.k1 * (2 * np.pi * self.ff)
        # spectral band mask, grids.py:65-73
        u_norm = (self.frequency + self.ff) / self.frequency
        if p["enable_spectral_filter"]:
            u_lo = (c / 5.0e-6) / self.frequency
            u_hi = (c / 0.18e-6) / self.frequency
            self.spec_mask = 0.25 * (1.0 + np.tanh((u_norm - u_lo) / 0.05)) * \
                (1.0 + np.tanh((u_hi - u_norm) / 0.05))
        else:
            self.spec_mask = np.ones_like(self.ff)
        # T-hat, U-hat, U^-1 (grids.py:79-111)
        self.T_op = (1.0 + self.ff / self.frequency) * self.spec_mask if p["enable_self_steepening"] \
            else np.ones_like(self.ff)
        U_op = 1.0 + self.k1 * (2 * np.pi * self.ff) / self.komega if p["enable_space_time_focusing"] \
            else np.ones_like(self.ff)
        self.inv_U_op = 1.0 / U_op
        self.inv_U_nl = self.spec_mask / np.maximum(U_op, 0.1) if p["enable_space_time_focusing"] \
            else np.ones_like(self.ff)
        # Raman response, grids.py:113-116
        t = self.tlist
        h = np.where(t > 0, self.Omega_r2 * p["tau_s"] * np.exp(-t / p["tau_d"]) * np.sin(t / p["tau_s"]), 0.0)
        self.R_f = np.fft.fft(np.fft.ifftshift(h)) * self.dt
        # Drude / carrier constants, grids.py:121-128
        meff_drude = p["meff_drude_rel"] * m_e
        self.sigmaomega = ((self.komega * q_e**2 * p["tau_c"]) /
                           (self.n0**2 * meff_drude * epsilon_0 * self.omega0 *
                            (1.0 + (self.omega0 * p["tau_c"]) ** 2))) * 1e4
        self.avalanche_coef = self.sigmaomega / self.Ui if p["enable_avalanche"] else 0.0
        self.avalanche_coef_s = self.sigmaomega / self.Us if (p["enable_ste"] and p["enable_avalanche"]) else 0.0
        self.inv_taur_eff = 1.0 / p["tau_r"] if p["enable_recombination"] else 0.0
        self.inv_tau_ste = 1.0 / p["tau_ste"] if (p["tau_ste"] and p["enable_ste"]) else 0.0
        self.invE2 = 0.5 * self.n0 * c * epsilon_0 * 1e-4
        # STE index prefactor, grids.py:133-137
        rho_c_pump = (epsilon_0 * m_e * self.omega0**2 / q_e**2) * 1e-6
        w_tr = p["E_tr_eV"] * q_e / 1.054571817e-34
        f_ste = self.omega0**2 / (w_tr**2 - self.omega0**2)
        self.ste_pref = ((self.omega0 / c) * f_ste / (2.0 * self.n0 * rho_c_pump)
                         if (p["enable_ste"] and p["enable_ste_index"]) else 0.0)
        self.mask_r = np.exp(-(self.rlist / (0.9 * self.R)) ** 20)
        # rate tables, grids.py:140-161
        self.rate = rate if rate is not None else MPIPowerLaw()
        self.I_tab = np.ravel(10 ** (np.arange(17) + 0.0)[:, None] * (0.01 * np.arange(900) + 1)[None, :])
        W = np.maximum(np.nan_to_num(self.rate(self.I_tab)), 0.0)
        self.W_tab = W
        self.f_spline = PchipInterpolator(self.I_tab, W)
        l0, l1 = float(np.log10(self.I_tab[0])), float(np.log10(self.I_tab[-1]))
        logI = np.linspace(l0, l1, 4096)
        self.W_LUT = np.nan_to_num(np.abs(self.f_spline(10.0 ** logI)), nan=0.0, posinf=0.0, neginf=0.0)
        # the power-law stand-in ignores the band gap, so the STE table (built at
        # Us in grids.py:147-156) equals the valence-band one
        self.W_LUT_s = self.W_LUT
        self.logImin, self.inv_dlog = l0, float(4095 / (l1 - l0))
        self.Imin, self.Imax = float(self.I_tab[0]), float(self.I_tab[-1])
        # operator constants, operators.py:60-68
        self.kerr_pref = 3 * self.chi3 * self.omega0**2 / (8 * self.komega * c**2)
        self.plasma_pref = (self.sigmaomega / 2.0) * 100.0
        self.plasma_phase = 1.0 + 1j * self.omega0 * p["tau_c"]

    # ------------------------------------------------------------------ ops
    def half_linear(self, u, dz):
        """operators.py:47-53 (the real Y is promoted to complex, as cp.dot does)."""
        psik = self.Rk * np.dot(self.Y, u)
        psik_f = np.fft.fft(psik, axis=1)
        phase = (self.delta_k[None, :] - self.rholist[:, None] ** 2 / (2 * self.komega)
                 * self.inv_U_op[None, :]) * dz / 2
        psik_f = psik_f * np.exp(1j * phase) * self.spec_mask[None, :]
        psik = np.fft.ifft(psik_f, axis=1)
        return self.iRk * np.dot(self.Y, psik)

    def pchip_rate(self, I):
        """|PCHIP(W)| on the clipped intensity, sanitised (operators.py:92-94)."""
        v = np.abs(self.f_spline(np.clip(I, self.Imin, self.Imax)))
        return np.nan_to_num(v, nan=0.0, posinf=0.0, neginf=0.0)

    def split(self, u, rho, rho_s=None):
        """operators.py:89-146 -> (rhs, alpha)."""
        p = self.p
        u = np.ascontiguousarray(u.astype(np.complex128, copy=False))
        absu2 = np.abs(u) ** 2
        W_PI = self.pchip_rate(absu2 * self.invE2)
        depl = np.clip(1.0 - rho / p["rho_max"], 0.0, 1.0)
        photo = (W_PI * 1e6) * self.Ui / (self.n0 * c * epsilon_0 * (absu2 + 1e-30)) * depl
        if not p["enable_photoionization_loss"]:
            photo = photo * 0.0
        alpha = photo
        if p["enable_plasma_absorption"]:
            alpha = alpha + self.plasma_pref * rho
        alpha = np.maximum(np.nan_to_num(alpha, nan=0.0, posinf=0.0, neginf=0.0), 0.0)
        kerr_I = np.zeros_like(absu2)
        if p["enable_kerr_instantaneous"]:
            kerr_I = kerr_I + (1.0 - p["f_R"]) * absu2
        if p["enable_kerr_raman"]:
            kerr_I = kerr_I + p["f_R"] * np.fft.ifft(np.fft.fft(absu2, axis=1) * self.R_f, axis=1).real
        plasma_coeff = ((1.0 if p["enable_plasma_absorption"] else 0.0)
                        + ((self.plasma_phase - 1.0) if p["enable_plasma_defocusing"] else 0.0))
        extra = -self.plasma_pref * plasma_coeff * rho * u
        if self.ste_pref and rho_s is not None:
            extra = extra + 1j * self.ste_pref * rho_s * u
        NL_freq = (np.fft.fft(1j * self.kerr_pref * kerr_I * u, axis=1) * self.T_op ** 2
                   - np.fft.fft(photo * u, axis=1) * self.T_op
                   + np.fft.fft(extra, axis=1))
        rhs = np.fft.ifft(NL_freq * self.inv_U_nl, axis=1) + alpha * u
        rhs = np.nan_to_num(np.where(absu2 < 1e-30, 0.0 + 0.0j, rhs), nan=0.0, posinf=0.0, neginf=0.0)
        return rhs, alpha

    def update_plasma(self, u, rho, rho_s):
        """operators.py:165-183: zero the t=0 column, then march (rate_scan.c)."""
        rho[:, 0] = 0.0
        rho_s[:, 0] = 0.0
        lut_s = self.W_LUT_s
        rate_scan(u, rho, rho_s, self.dt, self.invE2, self.avalanche_coef, self.avalanche_coef_s,
                  self.p["rho_max"], self.inv_taur_eff, self.inv_tau_ste, int(self.p["enable_ste"]),
                  self.W_LUT, lut_s, self.logImin, self.inv_dlog, self.Imin, self.Imax)

    def step(self, u, rho, rho_s, dz):
        """integrator.py:138-149 (Strang: half-linear, alpha/2, RK4, alpha/2, half-linear, mask)."""
        u = self.half_linear(u, dz)
        _, a = self.split(u, rho, rho_s)
        u = u * np.exp(-0.5 * dz * a)
        k1, _ = self.split(u, rho, rho_s)
        k2, _ = self.split(u + 0.5 * dz * k1, rho, rho_s)
        k3, _ = self.split(u + 0.5 * dz * k2, rho, rho_s)
        k4, _ = self.split(u + dz * k3, rho, rho_s)
        u = u + dz / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        _, a = self.split(u, rho, rho_s)
        u = u * np.exp(-0.5 * dz * a)
        u = self.half_linear(u, dz)
        return u * self.mask_r[:, None]

    def propagate(self, u, nsteps, dz, rho=None, rho_s=None):
        """``nsteps`` iterations of update_plasma + step (integrator.py:157-158)."""
        rho = np.zeros(u.shape) if rho is None else rho
        rho_s = np.zeros(u.shape) if rho_s is None else rho_s
        for _ in range(nsteps):
            self.update_plasma(u, rho, rho_s)
            u = self.step(u, rho, rho_s, dz)
        return u, rho, rho_s


def lens_gaussian(g, w0, fwhm, energy_uJ, f, seed, noise=0.01):
    """Seeded input pulse of the measured workloads:
    E0 exp(-r^2/w0^2) exp(-i k0 r^2 / 2f) exp(-t^2/tp^2) (1 + noise N(0,1)),
    E0 from the pulse energy as config.py:237-241 (tp = FWHM / sqrt(2 ln 2))."""
    tp = fwhm / np.sqrt(2 * np.log(2))
    P_in = energy_uJ * 1e-6 / (tp * np.sqrt(np.pi / 2))
    I0 = 2.0 * P_in / (np.pi * w0**2)
    E0 = np.sqrt(2.0 * I0 / (g.n0 * c * epsilon_0))
    rr = g.rlist[:, None]
    tt = g.tlist[None, :]
    z = np.random.default_rng(seed).standard_normal((g.Nr, g.Nt))
    return (E0 * np.exp(-rr**2 / w0**2) * np.exp(-1j * g.komega * rr**2 / (2 * f))
            * np.exp(-tt**2 / tp**2) * (1.0 + noise * z))


# ---------------------------------------------------------------- C scan
_lib = None


def _load():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle_scan.so")
        if not os.path.exists(path):
            import subprocess
            subprocess.check_call(["make", "-s", "-C", HERE])
        _lib = ctypes.CDLL(path)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        _lib.oracle_rate_scan.argtypes = [P, P, P, I, I, D, D, D, D, D, D, D, I, P, P, I, D, D, D, D]
        _lib.oracle_rate_scan.restype = None
    return _lib


def rate_scan(E, ne, ns, dt, field_to_I, beta_g, beta_s, na, inv_tau_r, inv_tau_ste,
              enable_ste, lut, lut_s, log_min, inv_dlog, Imin, Imax):
    """In-place FP64 carrier march over every row of E (kernels.py:36-106)."""
    lib = _load()
    E = np.ascontiguousarray(E, dtype=np.complex128)
    assert ne.dtype == np.float64 and ns.dtype == np.float64
    assert ne.flags.c_contiguous and ns.flags.c_contiguous and ne.shape == E.shape == ns.shape
    lut = np.ascontiguousarray(lut, dtype=np.float64)
    lut_s = np.ascontiguousarray(lut_s, dtype=np.float64)
    Nr, Nt = E.shape
    lib.oracle_rate_scan(E.ctypes.data, ne.ctypes.data, ns.ctypes.data, Nr, Nt, dt, field_to_I,
                         beta_g, beta_s, na, inv_tau_r, inv_tau_ste, int(enable_ste),
                         lut.ctypes.data, lut_s.ctypes.data, lut.size, log_min, inv_dlog,
                         Imin, Imax)


def workload_config(Nr, Nt, R_max, w0, T_half, **over):
    """Reference-Config field values for the measured workloads (800 nm fused
    silica, K=6 MPI, avalanche and recombination on, Raman / self-steepening /
    space-time focusing / STE off; the +-T_half window through delta_t)."""
    d = dict(Nt=Nt, N=Nr + 1, R_factor=R_max / w0, w0=w0, wavelength=800e-9,
             delta_t=T_half * math.sqrt(2 * math.log(2)) / 5.0, n2=3.2e-20, Ui_eV=9.0,
             rho_max=2.1e22, tau_r=150e-15, f_R=0.0, enable_kerr_raman=False,
             enable_self_steepening=False, enable_space_time_focusing=False, enable_ste=False)
    d.update(over)
    return d
