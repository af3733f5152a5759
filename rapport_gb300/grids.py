"""Host-side (FP64) grid and operator-table construction.

Restates ``build_grids`` of the reference (``deliverable (3)/sim/grids.py:29-175``)
on the host with numpy/scipy: time/frequency axes, the quasi-discrete Hankel
transform (QDHT) matrix, Sellmeier dispersion, spectral and radial masks, the
Drude/avalanche/recombination constants, and the photo-ionisation rate tables
(the PCHIP spline over I = 10^d (1 + 0.01 m) and the 4096-point log-uniform
table the carrier kernel reads).  Everything here runs once per Config; the
device only ever sees the FP32 tables the C library derives from it.

Returns a plain dict with the reference's keys (arrays are numpy, FP64).
"""
import numpy as np
from scipy.constants import c, epsilon_0, m_e
from scipy.constants import elementary_charge as q_e
from scipy.interpolate import PchipInterpolator
from scipy.special import dawsn, ellipe, ellipk, j0, j1, jn_zeros

from .config import SELLMEIER_B, SELLMEIER_L, Config

HBAR = 1.054571817e-34


def _n2m1(lam_um):
    x = lam_um**2
    return sum(b * x / (x - l * l) for b, l in zip(SELLMEIER_B, SELLMEIER_L))


def keldysh_rate(I_Wcm2, wavelength, Ui_eV, meff, n0, n_sum=60, beta_den=4.0):
    """Keldysh photo-ionisation rate in cm^-3 s^-1 (keldysh.py:94-130, the
    reference's default, non-monotone branch; Couairon 2005 Eqs. 7-8)."""
    U = Ui_eV * q_e
    w = 2 * np.pi * c / wavelength
    I = np.asarray(I_Wcm2, dtype=np.float64) * 1e4
    E = np.sqrt(2.0 * I / (n0 * c * epsilon_0))
    g = np.maximum(w * np.sqrt(meff * U) / (q_e * np.maximum(E, 1e-300)), 1e-12)
    Gam = g**2 / (1.0 + g**2)
    Xi = 1.0 / (1.0 + g**2)
    sG = np.sqrt(Gam)
    K1, E1 = ellipk(Gam), ellipe(Gam)
    K2, E2 = ellipk(Xi), ellipe(Xi)
    x = (2.0 * U * E2) / (np.pi * sG * HBAR * w)
    mx = np.floor(x + 1.0)
    nu = mx - x
    al = np.pi * (K1 - E1) / E2
    n = np.arange(n_sum).reshape((-1,) + (1,) * np.ndim(x))
    arg = np.pi * np.sqrt(np.maximum(n + 2.0 * nu, 0.0) / (beta_den * K2 * E2))
    Q = np.sqrt(np.pi / (2.0 * K2)) * np.sum(np.exp(-n * al) * dawsn(arg), axis=0)
    pref = (2.0 * w / (9.0 * np.pi)) * (w * meff / (HBAR * sG)) ** 1.5
    W = pref * Q * np.exp(-al * mx) * 1e-6
    return np.nan_to_num(W, nan=0.0, posinf=0.0, neginf=0.0)


def rate_function(cfg: Config, gap_eV):
    """I [W/cm^2] -> W [cm^-3 s^-1] for the configured rate model."""
    if cfg.rate_model == "mpi":
        return lambda I: cfg.sigma_K * np.asarray(I, dtype=np.float64) ** cfg.K_photons * cfg.rho_max
    return lambda I: keldysh_rate(I, cfg.wavelength, gap_eV, cfg.meff, cfg.n0)


def intensity_knots():
    """The reference's spline abscissae I = 10^d (1 + 0.01 m), d < 17, m < 900."""
    return (10.0 ** np.arange(17.0)[:, None] * (1.0 + 0.01 * np.arange(900.0))[None, :]).ravel()


def build_grids(cfg: Config) -> dict:
    k0, w0 = cfg.komega, cfg.omega0
    # time axis: +-5 t_p window, t_p = FWHM / sqrt(2 ln 2)
    tp = cfg.delta_t / np.sqrt(2 * np.log(2))
    tmax = 5 * tp
    dt = float(2 * tmax / cfg.Nt)
    tlist = np.linspace(-tmax, tmax, cfg.Nt, endpoint=False)
    ff = np.fft.fftfreq(cfg.Nt, d=dt)
    Om = 2 * np.pi * ff
    # QDHT on the first N zeros of J0 (the last one sets the radius scale)
    N = cfg.N
    jz = jn_zeros(0, N)
    jN = jz[N - 1]
    jr = jz[:N - 1]
    R = cfg.R_factor * cfg.w0
    Y = (2.0 / jN) * j0(np.outer(jr, jr) / jN) / j1(jr)[None, :] ** 2
    rlist = jr * R / jN
    rholist = jr / R
    # Sellmeier dispersion relative to k0 + k1 Omega, frequencies clipped to the fit window
    w_safe = np.clip(w0 + Om, 2 * np.pi * c / 5.0e-6, 2 * np.pi * c / 0.18e-6)

    def k_of(w):
        return (w / c) * np.sqrt(1.0 + _n2m1(2 * np.pi * c / w * 1e6))

    dw = w0 / 1000.0
    k1 = (k_of(w0 + dw) - k_of(w0 - dw)) / (2 * dw)
    delta_k = (w_safe / c) * np.sqrt(1.0 + _n2m1(2 * np.pi * c / w_safe * 1e6)) - k0 - k1 * Om
    # spectral band mask (tanh edges at 5 um and 0.18 um)
    un = (cfg.frequency + ff) / cfg.frequency
    if cfg.enable_spectral_filter:
        lo, hi = (c / 5.0e-6) / cfg.frequency, (c / 0.18e-6) / cfg.frequency
        spec_mask = 0.25 * (1.0 + np.tanh((un - lo) / 0.05)) * (1.0 + np.tanh((hi - un) / 0.05))
    else:
        spec_mask = np.ones_like(ff)
    T_op = (1.0 + ff / cfg.frequency) * spec_mask if cfg.enable_self_steepening else np.ones_like(ff)
    U_op = 1.0 + k1 * Om / k0 if cfg.enable_space_time_focusing else np.ones_like(ff)
    inv_U_op = 1.0 / U_op
    inv_U_nl = spec_mask / np.maximum(U_op, 0.1) if cfg.enable_space_time_focusing else np.ones_like(ff)
    resp = np.where(tlist > 0, cfg.Omega_r2 * cfg.tau_s * np.exp(-tlist / cfg.tau_d) * np.sin(tlist / cfg.tau_s), 0.0)
    R_f = np.fft.fft(np.fft.ifftshift(resp)) * dt
    tt, rr = np.meshgrid(tlist, rlist)
    _, rhorho = np.meshgrid(tlist, rholist)
    # Drude cross-section [cm^2] and carrier constants
    sigmaomega = ((k0 * q_e**2 * cfg.tau_c) /
                  (cfg.n0**2 * cfg.meff_drude * epsilon_0 * w0 * (1.0 + (w0 * cfg.tau_c) ** 2))) * 1e4
    avalanche_coef = sigmaomega / cfg.Ui if cfg.enable_avalanche else 0.0
    avalanche_coef_s = sigmaomega / cfg.Us if (cfg.enable_ste and cfg.enable_avalanche) else 0.0
    inv_taur_eff = 1.0 / cfg.tau_r if cfg.enable_recombination else 0.0
    inv_tau_ste = 1.0 / cfg.tau_ste if (cfg.tau_ste and cfg.enable_ste) else 0.0
    invE2 = 0.5 * cfg.n0 * c * epsilon_0 * 1e-4
    rho_c = (epsilon_0 * m_e * w0**2 / q_e**2) * 1e-6
    w_tr = cfg.E_tr_eV * q_e / HBAR
    f_ste = w0**2 / (w_tr**2 - w0**2)
    ste_pref = (w0 / c) * f_ste / (2.0 * cfg.n0 * rho_c) if (cfg.enable_ste and cfg.enable_ste_index) else 0.0
    mask_r = np.exp(-(rr / (0.9 * R)) ** 20)
    # rate tables: PCHIP on the structured intensity knots, then a 4096-point log-uniform table
    I_k = intensity_knots()
    W_g = np.maximum(np.nan_to_num(rate_function(cfg, cfg.Ui_eV)(I_k)), 0.0)
    W_s = np.maximum(np.nan_to_num(rate_function(cfg, cfg.Us_eV)(I_k)), 0.0)
    sp_g = PchipInterpolator(I_k, W_g)
    sp_s = PchipInterpolator(I_k, W_s)
    l0, l1 = float(np.log10(I_k[0])), float(np.log10(I_k[-1]))
    logI = np.linspace(l0, l1, 4096)
    keldysh = dict(
        f_spline=sp_g, f_spline_s=sp_s,
        W_LUT=np.nan_to_num(np.abs(sp_g(10.0 ** logI)), nan=0.0, posinf=0.0, neginf=0.0),
        W_LUT_s=np.nan_to_num(np.abs(sp_s(10.0 ** logI)), nan=0.0, posinf=0.0, neginf=0.0),
        NLUT=4096, logImin=l0, inv_dlog=float(4095 / (l1 - l0)),
        Imin=float(I_k[0]), Imax=float(I_k[-1]), I_knots=I_k,
    )
    return dict(
        komega=float(k0), tmax=tmax, dt=dt, tlist=tlist, ff=ff,
        Y=Y, R=R, j1last=jN, rlist=rlist, rholist=rholist,
        delta_k=delta_k, k1=k1, T_op=T_op, inv_U_op=inv_U_op, inv_U_nl=inv_U_nl, R_f=R_f,
        spec_mask=spec_mask, rr=rr, tt=tt, rhorho=rhorho,
        sigmaomega=sigmaomega, avalanche_coef=avalanche_coef, avalanche_coef_s=avalanche_coef_s,
        inv_taur_eff=inv_taur_eff, inv_tau_ste=inv_tau_ste, ste_pref=ste_pref, f_ste=f_ste,
        invE2=invE2, mask_r=mask_r, b=cfg.b, E0=cfg.E0, keldysh=keldysh,
    )


# ---------------------------------------------------------------- envelopes
def envelope_gaussian_focused(rr, tt, cfg, g):
    """Gaussian beam at distance cfg.begin from its focus (grids.py:180-183)."""
    tp = cfg.delta_t / np.sqrt(2 * np.log(2))
    q = 1 + 1j * 2 * cfg.begin / g["b"]
    return (g["E0"] / q) * np.exp(-rr**2 / cfg.w0**2 / q) * np.exp(-tt**2 / tp**2)


def envelope_lens(w0, fwhm, energy_uJ, f, seed, noise=0.01):
    """Seeded lens-focused Gaussian pulse of the measured workloads:
    E0 exp(-r^2/w0^2) exp(-i k0 r^2/(2 f)) exp(-t^2/tp^2) (1 + noise N(0,1)),
    with E0 from the pulse energy as in the reference Config (t_p = FWHM/sqrt(2 ln 2))
    and N(0,1) = numpy default_rng(seed).standard_normal((Nr, Nt))."""
    def fn(rr, tt, cfg, g):
        tp = fwhm / np.sqrt(2 * np.log(2))
        P = energy_uJ * 1e-6 / (tp * np.sqrt(np.pi / 2))
        I0 = 2.0 * P / (np.pi * w0**2)
        E0 = np.sqrt(2.0 * I0 / (cfg.n0 * c * epsilon_0))
        z = np.random.default_rng(seed).standard_normal(rr.shape)
        return (E0 * np.exp(-rr**2 / w0**2) * np.exp(-1j * cfg.komega * rr**2 / (2 * f))
                * np.exp(-tt**2 / tp**2) * (1.0 + noise * z))
    return fn


ENVELOPES = {"gaussian_focused": envelope_gaussian_focused}
