"""Host-side FP64 tables of the product (rapport_gb300.grids / config) against
the reference fixtures and the reference's published physics numbers."""
import numpy as np
import pytest

import rapport_gb300 as R
from conftest import meta_case, rel_l2


def _cfg(d):
    m = meta_case(d)
    return R.workload_config(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"], m["dz"], m["nsteps"]), m


def test_product_grids_match_reference(tiny):
    cfg, m = _cfg(tiny)
    g = R.build_grids(cfg)
    assert rel_l2(g["Y"], tiny["Y"]) < 1e-14
    assert rel_l2(g["delta_k"], tiny["delta_k"]) < 1e-11
    assert rel_l2(g["spec_mask"], tiny["spec_mask"]) < 1e-14
    assert rel_l2(g["mask_r"][:, 0], tiny["mask_r"]) < 1e-14
    assert rel_l2(g["rlist"], tiny["rlist"]) < 1e-15
    kel = g["keldysh"]
    assert rel_l2(kel["W_LUT"], tiny["W_LUT"]) < 1e-14
    assert rel_l2(kel["f_spline"](tiny["I_probe"]), tiny["W_probe"]) < 1e-14
    for k in ("invE2", "sigmaomega", "avalanche_coef", "inv_taur_eff", "dt", "komega"):
        assert g[k] == pytest.approx(float(tiny[k]), rel=1e-13), k
    assert kel["logImin"] == tiny["logImin"] and kel["inv_dlog"] == pytest.approx(float(tiny["inv_dlog"]))


def test_envelope_matches_reference(tiny):
    cfg, m = _cfg(tiny)
    g = R.build_grids(cfg)
    fn = R.envelope_lens(m["w0"], m["fwhm"], m["E"], m["f"], m["seed"])
    assert rel_l2(fn(g["rr"], g["tt"], cfg, g), tiny["u0"]) < 1e-14


def test_published_material_numbers():
    # n0(800 nm) = 1.4533 and k'' = 361.6 fs^2/cm (reference ANALYSE_CRITIQUE.md:58-59)
    cfg = R.Config(wavelength=800e-9, verbose=False, out_dir="")
    assert cfg.n0 == pytest.approx(1.4533, abs=5e-5)
    from scipy.constants import c
    n = R.n_sellmeier
    w0 = cfg.omega0
    k = lambda w: w / c * n(2 * np.pi * c / w)  # noqa: E731
    h = w0 * 1e-3
    k2 = (k(w0 + h) - 2 * k(w0) + k(w0 - h)) / h**2
    assert k2 * 1e30 * 1e-2 == pytest.approx(361.6, rel=2e-3)


def test_keldysh_multiphoton_limit():
    # Couairon 2005: for weak fields the Keldysh rate approaches sigma_6 I^6 rho_at
    # (sigma_6 = 9.6e-70, rho_at = 2.1e22); the reference asserts 0.8 < W/W_MPI < 1.25 at 1e12 W/cm^2
    from scipy.constants import m_e
    cfg = R.Config(wavelength=800e-9, verbose=False, out_dir="")
    W = R.keldysh_rate(1e12, 800e-9, 9.0, 0.64 * m_e, cfg.n0)
    ratio = W / (9.6e-70 * 1e12**6 * 2.1e22)
    assert 0.8 < ratio < 1.25


def test_config_validation():
    with pytest.raises(ValueError):
        R.Config(rate_model="tunnel", verbose=False, out_dir="")
    with pytest.raises(ValueError):
        R.Config(linear_mode="fp8", verbose=False, out_dir="")
    cfg = R.Config(verbose=False, out_dir="", begin=0.0, end=1e-2, nz=2000)
    assert cfg.dz == pytest.approx(5e-6)


def test_mpi_rate_table():
    cfg = R.workload_config(64, 128, 1e-4, 1e-5, 3e-13, 5e-6, 1)
    g = R.build_grids(cfg)
    I = np.array([1e10, 3e12, 5e13])
    assert np.allclose(g["keldysh"]["f_spline"](I), 1e-71 * I**6 * 2.1e22, rtol=2e-4)


def test_keldysh_rate_matches_reference():
    """grids.keldysh_rate against the reference's own KeldyshSiO2.rate
    (keldysh.py:94-148, keldysh_tables.npz) on every spline knot of
    grids.py:140-150: both band gaps, at 800 nm and the reference's 1030 nm."""
    from conftest import load_golden
    k = load_golden("keldysh_tables.npz")
    assert np.array_equal(k["I_knots"], R.grids.intensity_knots())
    for lam in (800, 1030):
        for gap in ("Ui", "Us"):
            W = R.keldysh_rate(k["I_knots"], lam * 1e-9, float(k[f"gap_{gap}_{lam}"]),
                               float(k[f"meff_{lam}"]), float(k[f"n0_{lam}"]))
            ref = k[f"W_{gap}_{lam}"]
            assert rel_l2(W, ref) < 1e-12, (lam, gap)
            big = ref > 1e-300
            assert np.max(np.abs(W[big] / ref[big] - 1)) < 1e-11, (lam, gap)


def test_keldysh_tables_match_reference(tiny_keldysh):
    """The reference's default rate model end to end on the host: build_grids'
    PCHIP spline and both 4096-point carrier tables (valence band and, with the
    exciton channel, the 6 eV gap) equal the reference's (grids.py:140-161)."""
    m = meta_case(tiny_keldysh)
    cfg = R.workload_config(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"], m["dz"], m["nsteps"],
                            rate_model="keldysh", enable_ste=True, tau_ste=1e-12)
    kel = R.build_grids(cfg)["keldysh"]
    assert rel_l2(kel["W_LUT"], tiny_keldysh["W_LUT"]) < 1e-12
    assert rel_l2(kel["W_LUT_s"], tiny_keldysh["W_LUT_s"]) < 1e-12
    # the raw Keldysh rate has cusps (channel closings) where PCHIP's slope
    # limiter turns last-bit differences of the knot values into ~1e-11
    assert rel_l2(kel["f_spline"](tiny_keldysh["I_probe"]), tiny_keldysh["W_probe"]) < 1e-10


def test_linear_mode_resolution():
    """auto = a tensor-core form wherever the library runs one (split-BF16, or
    split-FP16 with space-time focusing), else the plain FP32 form."""
    from rapport_gb300.config import resolved_linear_mode, split_supported
    mk = lambda **kw: R.Config(verbose=False, out_dir="", **kw)  # noqa: E731
    assert mk().linear_mode == "auto"
    assert resolved_linear_mode(mk(N=1025, Nt=2048, enable_space_time_focusing=False)) == "split_bf16"
    # space-time focusing: the sandwich Y P Y, whose arithmetic is the split-FP16 form's
    assert resolved_linear_mode(mk(N=1025, Nt=2048, enable_space_time_focusing=True)) == "split_f16"
    # N_r = 999 (the context pads it to 1024) and N_t = 128 (one partial tile) run split too
    assert resolved_linear_mode(mk(N=1000, Nt=2048, enable_space_time_focusing=False)) == "split_bf16"
    assert resolved_linear_mode(mk(N=65, Nt=128, enable_space_time_focusing=False)) == "split_bf16"
    assert resolved_linear_mode(mk(N=9000, Nt=128, enable_space_time_focusing=False)) == "plain"
    assert resolved_linear_mode(mk(linear_mode="split_f16")) == "split_f16"
    assert split_supported(mk(N=257, Nt=512, enable_space_time_focusing=False))
