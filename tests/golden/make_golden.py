"""Generate the golden fixtures in tests/golden/*.npz from the REFERENCE itself.

Runs the reference solver package (``deliverable (3)/sim``) unmodified on the
CPU, with ``tests/golden/refshim`` standing in for cupy/cupyx and the
reference's carrier-rate CUDA-C kernel compiled as C++ (``oracle/ref_build.py``).
Only this container has the reference checkout; the fixtures it writes are
committed so that the tests run anywhere.

Workload adaptations (no reference code is edited; all through its own hooks):
  * MPI power law: ``grids.KeldyshSiO2`` is replaced by a class whose
    ``rate(I) = sigma_K * I**K * rho_nt`` (grids.py:142-150 then builds the
    PCHIP spline and the 4096-point LUT from it exactly as for Keldysh).
  * Window: ``cfg.delta_t = T_half * sqrt(2 ln 2) / 5`` gives a +-T_half window
    (grids.py:32-35); the real pulse duration goes through a callable envelope
    (integrator.py:39).
  * Radius: ``R_factor = R_max / w0`` (grids.py:40).
  * Lens: E0 exp(-r^2/w0^2) exp(-i k0 r^2/(2 f)) exp(-t^2/tp^2) (1 + 0.01 N(0,1)).
  * Steps: an explicit loop of ``nl.update_plasma`` + ``step`` (integrator.py:157-158).

Usage:  python tests/golden/make_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
REF_ROOT = os.environ.get("RAPPORT_REFERENCE", "/root/reference")
REF_SIM = os.path.join(REF_ROOT, ".github", "deliverable (3)", "sim")

sys.path.insert(0, os.path.join(HERE, "refshim"))
sys.path.insert(0, REF_SIM)

from scipy.constants import c, epsilon_0  # noqa: E402

import grids as ref_grids  # noqa: E402
import config as ref_config  # noqa: E402
import integrator as ref_integrator  # noqa: E402

SIGMA_K, K_PHOTONS, RHO_NT = 1e-71, 6, 2.1e22


class MPIPowerLaw:
    """Drop-in for keldysh.KeldyshSiO2: W = sigma_K I^K rho_nt (cm^-3 s^-1)."""

    def __init__(self, wavelength, Ui_eV, meff, n0):
        pass

    def rate(self, I):
        I = np.asarray(I, dtype=np.float64)
        return SIGMA_K * I**K_PHOTONS * RHO_NT


import keldysh as ref_keldysh  # noqa: E402

REF_KELDYSH = ref_keldysh.KeldyshSiO2  # the reference's own rate (its default table source)
ref_grids.KeldyshSiO2 = MPIPowerLaw


def make_config(Nr, Nt, R_max, w0, T_half, dz, nz, energy_uJ=1.0, **over):
    out = tempfile.mkdtemp(prefix="golden_")
    kw = dict(
        nz=nz, Nt=Nt, N=Nr + 1, begin=0.0, end=nz * dz,
        R_factor=R_max / w0, w0=w0, wavelength=800e-9,
        delta_t=T_half * np.sqrt(2 * np.log(2)) / 5.0, energy_uJ=energy_uJ,
        n2=3.2e-20, Ui_eV=9.0, rho_max=RHO_NT, tau_r=150e-15,
        f_R=0.0, enable_kerr_raman=False, enable_self_steepening=False,
        enable_space_time_focusing=False, enable_ste=False,
        verbose=False, out_dir=out, rho_t_stride=0)
    kw.update(over)
    return ref_config.Config(**kw)


def lens_envelope(fwhm, energy_uJ, w0, f, seed):
    def fn(rr, tt, cfg, g):
        tp = fwhm / np.sqrt(2 * np.log(2))
        P_in = energy_uJ * 1e-6 / (tp * np.sqrt(np.pi / 2))
        I0 = 2.0 * P_in / (np.pi * w0**2)
        E0 = np.sqrt(2.0 * I0 / (cfg.n0 * c * epsilon_0))
        noise = np.random.default_rng(seed).standard_normal(rr.shape)
        return (E0 * np.exp(-rr**2 / w0**2) * np.exp(-1j * cfg.komega * rr**2 / (2 * f))
                * np.exp(-tt**2 / tp**2) * (1.0 + 0.01 * noise))
    return fn


def grid_arrays(integ):
    g, nl = integ.g, integ.nl
    kel = g["keldysh"]
    I_probe = np.concatenate([np.geomspace(0.5, 2e17, 700),
                              [1.0, 1.005, 9.99e16, 1e13, 5e13, 1.01e13]])
    return dict(
        Y=g["Y"], rlist=g["rlist"], rholist=g["rholist"], tlist=g["tlist"], ff=g["ff"],
        dt=g["dt"], delta_k=g["delta_k"], spec_mask=g["spec_mask"],
        mask_r=g["mask_r"][:, 0], R=g["R"], j1last=g["j1last"], komega=g["komega"],
        W_LUT=kel["W_LUT"], logImin=kel["logImin"], inv_dlog=kel["inv_dlog"],
        Imin=kel["Imin"], Imax=kel["Imax"], invE2=g["invE2"],
        sigmaomega=g["sigmaomega"], avalanche_coef=g["avalanche_coef"],
        inv_taur_eff=g["inv_taur_eff"], kerr_pref=nl.kerr_pref,
        plasma_pref=nl.plasma_pref, n0=integ.cfg.n0, omega0=integ.cfg.omega0,
        I_probe=I_probe, W_probe=kel["f_spline"](I_probe),
    )


def run_case(Nr, Nt, R_max, w0, T_half, fwhm, energy_uJ, f, dz, nsteps, seed, rows,
             keep_steps, with_Y=True, keldysh=False, **over):
    cfg = make_config(Nr, Nt, R_max, w0, T_half, dz, nsteps, energy_uJ, **over)
    # keldysh=True: the reference's default rate model (KeldyshSiO2) fills the tables
    ref_grids.KeldyshSiO2 = REF_KELDYSH if keldysh else MPIPowerLaw
    try:
        integ = ref_integrator.Integrator(cfg, envelope=lens_envelope(fwhm, energy_uJ, w0, f, seed))
    finally:
        ref_grids.KeldyshSiO2 = MPIPowerLaw
    if keldysh:
        out_extra = dict(W_LUT_s=np.asarray(integ.g["keldysh"]["W_LUT_s"]))
    else:
        out_extra = {}
    out = grid_arrays(integ)
    out.update(out_extra)
    u0 = integ.u.copy()
    out["u0"] = u0[rows]
    # single-operator goldens on the initial field
    out["hl_u0"] = integ.lin.half_linear(u0, dz)[rows]
    rho0 = np.zeros(u0.shape)
    rs0 = np.zeros(u0.shape)
    integ.nl.update_plasma(u0, rho0, rs0, integ.dt, integ.blocks, integ.threads)
    out["rho_u0"] = rho0[rows]
    # split on a field with plasma present: the half-linear output + rho of u0
    rhs, alpha = integ.nl.split(out_hl := integ.lin.half_linear(u0, dz), rho0, rs0)
    out["split_rhs"], out["split_alpha"] = rhs[rows], alpha[rows]
    if over.get("enable_ste"):
        out["rho_s_u0"] = rs0[rows]
    del out_hl
    traj_u, traj_rho, traj_rs = [], [], []
    for i in range(nsteps):
        integ.nl.update_plasma(integ.u, integ.rho, integ.rho_s, integ.dt,
                               integ.blocks, integ.threads)
        integ.step(integ.dz)
        traj_u.append(integ.u[rows].copy())
        traj_rho.append(integ.rho[rows].copy())
        traj_rs.append(integ.rho_s[rows].copy())
    out["u_steps"] = np.stack([traj_u[i - 1] for i in keep_steps])
    out["rho_steps"] = np.stack([traj_rho[i - 1] for i in keep_steps])
    if over.get("enable_ste"):
        out["rho_s_steps"] = np.stack([traj_rs[i - 1] for i in keep_steps])
    out["steps_kept"] = np.asarray(keep_steps)
    if not with_Y:
        del out["Y"]
    out["rows"] = np.asarray(rows)
    out["meta"] = np.array([Nr, Nt, R_max, w0, T_half, fwhm, energy_uJ, f, dz, nsteps, seed],
                           dtype=np.float64)
    return out


def k1_edge_cases():
    """Known-answer vectors for the carrier-rate kernel, from the reference kernel."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ref_build
    k = ref_build.RefRateKernel()
    rng = np.random.default_rng(7)
    Nr, Nt = 12, 256
    t = np.linspace(-1, 1, Nt)
    amp = np.geomspace(1e6, 3e11, Nr)[:, None] * np.exp(-t**2 / 0.1)[None, :]
    E = amp * np.exp(1j * rng.uniform(0, 6.28, (Nr, Nt)))
    E[3, 40] = np.nan
    E[4, 41] = np.inf
    E[5, 10:20] = 0.0
    # intensity-saturation row: drives ne past na so the rescale clamp fires
    E[Nr - 1] = 4e11
    cfg = make_config(64, 128, 1e-4, 1e-5, 3e-13, 5e-6, 1)
    g = ref_grids.build_grids(cfg)
    kel = g["keldysh"]
    res = dict(E=E, dt=2.5e-15, invE2=g["invE2"], W_LUT=kel["W_LUT"],
               logImin=kel["logImin"], inv_dlog=kel["inv_dlog"], Imin=kel["Imin"],
               Imax=kel["Imax"])
    # ste=0 / ste=1 with assorted initial values, and ste=0 from zero (what
    # update_plasma feeds the kernel: operators.py:166-167 zero column 0)
    for ste, tag in ((0, "ste0"), (1, "ste1"), (0, "zero")):
        ne = np.zeros((Nr, Nt))
        ns = np.zeros((Nr, Nt))
        if tag != "zero":
            ne[:, 0] = np.where(np.arange(Nr) % 3 == 0, -1.0, 1e15)
            ns[:, 0] = 1e14 if ste else 0.0
        params = dict(beta_g=g["sigmaomega"] / cfg.Ui, beta_s=g["sigmaomega"] / cfg.Us,
                      na=2.1e22, inv_tau_r=1.0 / 150e-15, inv_tau_ste=1e12)
        res[f"ne0_{tag}"], res[f"ns0_{tag}"] = ne[:, 0].copy(), ns[:, 0].copy()
        k(E, ne, ns, res["dt"], g["invE2"], params["beta_g"], params["beta_s"], params["na"],
          params["inv_tau_r"], params["inv_tau_ste"], ste, kel["W_LUT"], kel["W_LUT"] * 0.3,
          kel["logImin"], kel["inv_dlog"], kel["Imin"], kel["Imax"])
        res[f"ne_{tag}"], res[f"ns_{tag}"] = ne, ns
        for kk, v in params.items():
            res[f"{kk}"] = v
    return res


def keldysh_tables():
    """The reference's KeldyshSiO2.rate (keldysh.py:94-148, default monotone=False)
    on the spline knots I = 10^d (1 + 0.01 m) that grids.py:140-150 evaluates it
    at: both band gaps (9 eV valence band, 6 eV exciton) at 800 nm and at the
    reference's default 1030 nm, with the Config-derived meff and n0."""
    out = {"I_knots": np.ravel(10 ** (np.arange(17) + 0.0)[:, None] * (0.01 * np.arange(900) + 1)[None, :])}
    for lam in (800e-9, 1030e-9):
        cfg = make_config(64, 128, 1e-4, 1e-5, 3e-13, 5e-6, 1, wavelength=lam)
        tag = f"{int(round(lam * 1e9))}"
        out[f"n0_{tag}"], out[f"meff_{tag}"] = cfg.n0, cfg.meff
        for gap, name in ((cfg.Ui_eV, "Ui"), (cfg.Us_eV, "Us")):
            out[f"W_{name}_{tag}"] = REF_KELDYSH(lam, gap, cfg.meff, cfg.n0).rate(out["I_knots"])
            out[f"gap_{name}_{tag}"] = gap
    return out


def record_case():
    """The reference's own Integrator.propagate() with every recording option on:
    save stride, (z, r, t) cube with r/t strides, absorption time bins, rho snapshot."""
    Nr, Nt, dz, nz = 64, 256, 5e-6, 8
    cfg = make_config(Nr, Nt, 100e-6, 10e-6, 300e-15, dz, nz, energy_uJ=2.0)
    cfg.save_stride, cfg.rho_t_stride, cfg.rho_r_stride = 2, 4, 2
    cfg.absorb_time_bins_fs = (-100.0, -50.0, 0.0, 50.0, 100.0)
    cfg.rho_snapshot_t_fs = 50.0
    integ = ref_integrator.Integrator(cfg, envelope=lens_envelope(100e-15, 2.0, 10e-6, 1e-2, 0))
    res = integ.propagate()
    keep = ("r", "rlist", "z", "fluence_rz", "rho_rz", "rho_s_rz", "Imax_z", "E_plasma_z", "E_MPI_z", "E_STE_z",
            "E_total_z", "rho_rzt", "rho_s_rzt", "I_rzt", "t_sub_fs", "r_sub", "absorbed_rz", "Ipeak_rz",
            "rho_rz_at", "absorbed_rz_bins", "absorb_bin_edges_fs", "rho_onaxis_t", "rho_s_onaxis_t",
            "I_onaxis_t", "t_full_fs")
    out = {k: res[k] for k in keep}
    out["U0_uJ"] = integ.U0_uJ
    out["meta"] = np.array([Nr, Nt, 100e-6, 10e-6, 300e-15, 100e-15, 2.0, 1e-2, dz, nz, 0], dtype=np.float64)
    return out


def main():
    # 2 uJ into a 10 um waist: Kerr phase ~0.2 rad and peak rho ~1e19 per step,
    # every term active, RK4 comfortably stable (used for propagation parity)
    tiny = run_case(Nr=64, Nt=128, R_max=100e-6, w0=10e-6, T_half=300e-15, fwhm=100e-15,
                    energy_uJ=2.0, f=1e-2, dz=5e-6, nsteps=10, seed=0, rows=list(range(64)),
                    keep_steps=[1, 3, 10])
    np.savez_compressed(os.path.join(HERE, "tiny.npz"), **tiny)
    # 5 uJ: 66 % of rho_nt ionised on axis -- deep depletion for the carrier
    # march and split(); the reference's RK4 is unstable there (plasma phase
    # ~100 rad per step), so only the single-operator outputs are kept
    hot = run_case(Nr=64, Nt=128, R_max=100e-6, w0=10e-6, T_half=300e-15, fwhm=100e-15,
                   energy_uJ=5.0, f=1e-2, dz=5e-6, nsteps=1, seed=0, rows=list(range(64)),
                   keep_steps=[1], with_Y=False)
    for k in ("u_steps", "rho_steps", "steps_kept"):
        del hot[k]
    np.savez_compressed(os.path.join(HERE, "tiny_hot.npz"), **hot)
    # the CPU-runnable case (256 x 512, 1 uJ, w0 100 um, R_max 1 mm, +-400 fs, f 10 cm),
    # first 3 of its 2000 steps; every 8th radial row is kept to bound the fixture size.
    c1 = run_case(Nr=256, Nt=512, R_max=1e-3, w0=100e-6, T_half=400e-15, fwhm=100e-15,
                  energy_uJ=1.0, f=0.1, dz=5e-6, nsteps=3, seed=0,
                  rows=list(range(0, 256, 8)), keep_steps=[1, 3], with_Y=False)
    np.savez_compressed(os.path.join(HERE, "config1_prefix.npz"), **c1)
    # every split() term of the reference on: Raman (f_R 0.18), self-steepening,
    # space-time focusing, the exciton channel (1 ps decay) -- the full-physics path
    full = run_case(Nr=64, Nt=128, R_max=100e-6, w0=10e-6, T_half=300e-15, fwhm=100e-15,
                    energy_uJ=2.0, f=1e-2, dz=5e-6, nsteps=4, seed=0, rows=list(range(64)),
                    keep_steps=[1, 4], f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True,
                    enable_space_time_focusing=True, enable_ste=True, tau_ste=1e-12)
    full["flags"] = np.array([0.18, 1, 1, 1, 1, 1e-12])
    np.savez_compressed(os.path.join(HERE, "tiny_full.npz"), **full)
    # the reference's default rate model: Keldysh tables (valence band and, with
    # the exciton channel on, the 6 eV exciton gap) -- no power-law substitution
    kel = run_case(Nr=64, Nt=256, R_max=100e-6, w0=10e-6, T_half=300e-15, fwhm=100e-15,
                   energy_uJ=2.0, f=1e-2, dz=5e-6, nsteps=4, seed=0, rows=list(range(64)),
                   keep_steps=[1, 4], with_Y=False, keldysh=True, enable_ste=True, tau_ste=1e-12)
    np.savez_compressed(os.path.join(HERE, "tiny_keldysh.npz"), **kel)
    np.savez_compressed(os.path.join(HERE, "keldysh_tables.npz"), **keldysh_tables())
    np.savez_compressed(os.path.join(HERE, "k1_edge.npz"), **k1_edge_cases())
    np.savez_compressed(os.path.join(HERE, "record_tiny.npz"), **record_case())
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
