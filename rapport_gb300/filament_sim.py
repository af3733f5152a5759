"""Facade: run() and the public surface (filament_sim.py:59-106 of the reference)."""
from .config import Config, n_sellmeier  # noqa: F401  (the reference's filament_sim exports both)
from .integrator import Integrator, code_fingerprint  # noqa: F401

FIELD_TOGGLES = [
    "enable_kerr_instantaneous",
    "enable_kerr_raman",
    "enable_self_steepening",
    "enable_photoionization_loss",
    "enable_plasma_defocusing",
    "enable_plasma_absorption",
]


def run_config(*, Nz, Nt, Nr, wavelength, energy_uJ=15.0, peak_power_W=None, w0=10e-6, delta_t=263e-15,
               begin=-600e-6, end=1800e-6, n2=3.54e-20, Ui_eV=9.0, R_factor=100.0, save_stride=1,
               ckpt_every=500, verbose=True, out_dir=None, **material):
    """The Config run() builds from its keywords (Nr is Config.N, i.e. radial points + 1)."""
    return Config(nz=Nz, Nt=Nt, N=Nr, wavelength=wavelength, energy_uJ=energy_uJ,
                  peak_power_W=peak_power_W, w0=w0, delta_t=delta_t, begin=begin, end=end, n2=n2,
                  Ui_eV=Ui_eV, R_factor=R_factor, save_stride=save_stride, ckpt_every=ckpt_every,
                  verbose=verbose, out_dir=out_dir, **material)


def run(*, Nz, Nt, Nr, wavelength, energy_uJ=15.0, peak_power_W=None, envelope="gaussian_focused",
        w0=10e-6, delta_t=263e-15, begin=-600e-6, end=1800e-6, n2=3.54e-20, Ui_eV=9.0, R_factor=100.0,
        save_stride=1, ckpt_every=500, verbose=True, out_dir=None, **material):
    """Build a Config (Nr is Config.N, i.e. radial points + 1) and propagate it."""
    cfg = run_config(Nz=Nz, Nt=Nt, Nr=Nr, wavelength=wavelength, energy_uJ=energy_uJ, peak_power_W=peak_power_W,
                     w0=w0, delta_t=delta_t, begin=begin, end=end, n2=n2, Ui_eV=Ui_eV, R_factor=R_factor,
                     save_stride=save_stride, ckpt_every=ckpt_every, verbose=verbose, out_dir=out_dir, **material)
    return Integrator(cfg, envelope=envelope).propagate()
