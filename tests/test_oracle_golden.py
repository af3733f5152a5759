"""The FP64 oracle against golden fixtures generated from the reference itself.

The fixtures (tests/golden/make_golden.py) come from running the reference
solver package unmodified on the CPU; the oracle must reproduce them to
rounding (it restates the same FP64 arithmetic)."""
import numpy as np
import pytest

import nlse_oracle as O
from conftest import meta_case, rel_l2


def _grid(d):
    m = meta_case(d)
    return O.OracleGrid(O.workload_config(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"])), m


def test_grid_tables_match_reference(tiny):
    g, _ = _grid(tiny)
    assert rel_l2(g.Y, tiny["Y"]) < 1e-14
    assert rel_l2(g.delta_k, tiny["delta_k"]) < 1e-12
    assert rel_l2(g.spec_mask, tiny["spec_mask"]) < 1e-14
    assert rel_l2(g.mask_r, tiny["mask_r"]) < 1e-14
    assert rel_l2(g.W_LUT, tiny["W_LUT"]) < 1e-14
    assert rel_l2(g.f_spline(tiny["I_probe"]), tiny["W_probe"]) < 1e-14
    for k in ("invE2", "sigmaomega", "avalanche_coef", "inv_taur_eff", "kerr_pref", "plasma_pref",
              "logImin", "inv_dlog", "Imin", "Imax", "dt", "komega", "n0"):
        assert getattr(g, k) == pytest.approx(float(tiny[k]), rel=1e-13), k


@pytest.mark.parametrize("name", ["tiny", "hot", "cfg1"])
def test_envelope_and_operators(name, tiny, hot, cfg1):
    d = {"tiny": tiny, "hot": hot, "cfg1": cfg1}[name]
    g, m = _grid(d)
    rows = d["rows"]
    u0 = O.lens_gaussian(g, m["w0"], m["fwhm"], m["E"], m["f"], m["seed"])
    assert rel_l2(u0[rows], d["u0"]) < 1e-14
    assert rel_l2(g.half_linear(u0, m["dz"])[rows], d["hl_u0"]) < 1e-12
    rho = np.zeros(u0.shape)
    rs = np.zeros(u0.shape)
    g.update_plasma(u0, rho, rs)
    assert rel_l2(rho[rows], d["rho_u0"]) < 1e-12
    rhs, al = g.split(g.half_linear(u0, m["dz"]), rho, rs)
    assert rel_l2(rhs[rows], d["split_rhs"]) < 1e-12
    assert rel_l2(al[rows], d["split_alpha"]) < 1e-12


@pytest.mark.parametrize("name", ["tiny", "cfg1"])
def test_propagation_prefix(name, tiny, cfg1):
    d = tiny if name == "tiny" else cfg1
    g, m = _grid(d)
    rows = d["rows"]
    u = O.lens_gaussian(g, m["w0"], m["fwhm"], m["E"], m["f"], m["seed"])
    rho = np.zeros(u.shape)
    rs = np.zeros(u.shape)
    kept = list(d["steps_kept"])
    for i in range(1, max(kept) + 1):
        g.update_plasma(u, rho, rs)
        u = g.step(u, rho, rs, m["dz"])
        if i in kept:
            j = kept.index(i)
            assert rel_l2(u[rows], d["u_steps"][j]) < 1e-12, i
            assert rel_l2(rho[rows], d["rho_steps"][j]) < 1e-12, i


@pytest.mark.parametrize("tag,ste", [("ste0", 0), ("ste1", 1), ("zero", 0)])
def test_rate_scan_known_answers(k1edge, tag, ste):
    k = k1edge
    ne = np.zeros(k["E"].shape)
    ns = np.zeros(k["E"].shape)
    ne[:, 0] = k[f"ne0_{tag}"]
    ns[:, 0] = k[f"ns0_{tag}"]
    O.rate_scan(k["E"], ne, ns, float(k["dt"]), float(k["invE2"]), float(k["beta_g"]), float(k["beta_s"]),
                float(k["na"]), float(k["inv_tau_r"]), float(k["inv_tau_ste"]), ste, k["W_LUT"],
                k["W_LUT"] * 0.3, float(k["logImin"]), float(k["inv_dlog"]), float(k["Imin"]), float(k["Imax"]))
    np.testing.assert_array_equal(ne, k[f"ne_{tag}"])
    np.testing.assert_array_equal(ns, k[f"ns_{tag}"])
    if tag == "zero":
        assert ne[-1].max() == pytest.approx(2.1e22)       # saturation clamp fired
        assert ne[3, 40] == 0.0 and ne[3, 41] == 0.0         # NaN sample resets the march


def test_oracle_rate_scan_matches_compiled_reference_kernel():
    """oracle/rate_scan.c against the reference's own CUDA-C source compiled
    as C++ (oracle/ref_build.py); needs the reference checkout."""
    ref_build = pytest.importorskip("ref_build")
    if not ref_build.reference_available():
        pytest.skip("reference checkout not present")
    k = ref_build.RefRateKernel()
    rng = np.random.default_rng(3)
    Nr, Nt = 9, 200
    E = rng.standard_normal((Nr, Nt)) * np.geomspace(1e8, 4e11, Nr)[:, None] * (1 + 1j)
    E[2, 5] = np.nan
    lut = np.geomspace(1e-30, 1e40, 4096)
    args = (1.1e-15, 1.93e-7, 5.0, 7.0, 2.1e22, 1 / 150e-15, 1e12)
    for ste in (0, 1):
        ne_r, ns_r = np.zeros((Nr, Nt)), np.zeros((Nr, Nt))
        ne_o, ns_o = np.zeros((Nr, Nt)), np.zeros((Nr, Nt))
        ne_r[:, 0] = ne_o[:, 0] = 1e16
        ns_r[:, 0] = ns_o[:, 0] = 1e15 * ste
        k(E, ne_r, ns_r, *args, ste, lut, lut * 0.5, 0.0, 4095 / 17.0, 1.0, 9.99e16)
        O.rate_scan(E, ne_o, ns_o, *args, ste, lut, lut * 0.5, 0.0, 4095 / 17.0, 1.0, 9.99e16)
        np.testing.assert_array_equal(ne_o, ne_r)
        np.testing.assert_array_equal(ns_o, ns_r)


def test_full_physics_matches_reference(full):
    """Raman, self-steepening, space-time focusing and excitons all on: the
    oracle's half_linear (Omega-dependent diffraction), split and carrier march
    reproduce the reference's, and so do 4 whole z-steps."""
    from conftest import FULL_PHYSICS
    m = meta_case(full)
    g = O.OracleGrid(O.workload_config(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"], **FULL_PHYSICS))
    u0 = O.lens_gaussian(g, m["w0"], m["fwhm"], m["E"], m["f"], m["seed"])
    assert rel_l2(u0, full["u0"]) < 1e-14
    assert rel_l2(g.half_linear(u0, m["dz"]), full["hl_u0"]) < 1e-12
    rho, rs = np.zeros(u0.shape), np.zeros(u0.shape)
    g.update_plasma(u0, rho, rs)
    assert rel_l2(rho, full["rho_u0"]) < 1e-12
    assert rs.max() > 0 and rel_l2(rs, full["rho_s_u0"]) < 1e-12
    rhs, al = g.split(g.half_linear(u0, m["dz"]), rho, rs)
    assert rel_l2(rhs, full["split_rhs"]) < 1e-12
    assert rel_l2(al, full["split_alpha"]) < 1e-12
    u, rho, rs = u0, np.zeros(u0.shape), np.zeros(u0.shape)
    kept = list(full["steps_kept"])
    for i in range(1, max(kept) + 1):
        g.update_plasma(u, rho, rs)
        u = g.step(u, rho, rs, m["dz"])
        if i in kept:
            j = kept.index(i)
            assert rel_l2(u, full["u_steps"][j]) < 1e-12, i
            assert rel_l2(rho, full["rho_steps"][j]) < 1e-12, i
            assert rel_l2(rs, full["rho_s_steps"][j]) < 1e-12, i
