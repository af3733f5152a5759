"""Self-trapped-exciton channel (two carrier populations) through the C ABI.

The march of (rho, rho_s) (kernels.py:72-95) is checked against the
reference kernel's own outputs (k1_edge.npz, case 'ste1': assorted t = 0
values, decay time 1 ps, an exciton table 0.3 x the band table) and against
the FP64 oracle on a focused pulse; split()'s exciton index term
(operators.py:137-139) and whole z-steps in both forms against the oracle.

Tolerances, FP32 against FP64 as for one population: densities within
2e-4 of each row's peak (Newton-linearised scan); split rhs relative L2
2e-5; 10 z-steps: field relative L2 1e-4 (plain) / 5e-5 (split-BF16 vs
FP64 at the same step count), densities 1e-3 of the peak.
"""
import numpy as np
import pytest

from conftest import rel_l2
from gpu_util import Case, dev, host

pytestmark = pytest.mark.gpu

# 64 x 256 focused pulse (2 uJ into 10 um, f 1 cm), exciton channel with a 1 ps decay
STE = dict(Nr=64, Nt=256, R_max=1e-4, w0=1e-5, T_half=3e-13, fwhm=100e-15, E=2.0, f=1e-2, dz=5e-6,
           enable_ste=True, tau_ste=1e-12)


@pytest.fixture(scope="module")
def ste():
    return Case(**STE)


def _k1_ctx(k1edge, with_ste):
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    Nr, Nt = k1edge["E"].shape
    cfg = R.workload_config(Nr, Nt, 1e-4, 1e-5, 3e-13, 5e-6, 1)
    g = R.build_grids(cfg)
    desc, keep = _lib.make_desc(cfg, g)
    lut = np.ascontiguousarray(k1edge["W_LUT"], dtype=np.float64)
    lut_s = np.ascontiguousarray(k1edge["W_LUT"] * 0.3, dtype=np.float64)
    keep += [lut, lut_s]
    desc.lut = lut.ctypes.data
    desc.dt, desc.invE2 = float(k1edge["dt"]), float(k1edge["invE2"])
    desc.beta_g, desc.inv_tau_r, desc.rho_max = float(k1edge["beta_g"]), float(k1edge["inv_tau_r"]), float(k1edge["na"])
    desc.lut_log_min, desc.lut_inv_dlog = float(k1edge["logImin"]), float(k1edge["inv_dlog"])
    desc.lut_Imin, desc.lut_Imax = float(k1edge["Imin"]), float(k1edge["Imax"])
    if with_ste:
        desc.flags |= _lib.F_STE
        desc.lut_s = lut_s.ctypes.data
        desc.beta_s, desc.inv_tau_ste = float(k1edge["beta_s"]), float(k1edge["inv_tau_ste"])
    return _lib.Context(desc=desc)


def _peak_err(got, ref):
    return np.abs(got - ref) / np.maximum(np.abs(ref).max(axis=1, keepdims=True), 1e-30)


@pytest.mark.parametrize("tag", ["ste1", "ste0"])
def test_rate_equation_matches_reference_kernel(k1edge, tag):
    """The kernel alone from the fixture's t = 0 values (negative starts count as 0)."""
    ctx = _k1_ctx(k1edge, tag == "ste1")
    E = k1edge["E"]
    ne = np.zeros(E.shape)
    ns = np.full(E.shape, 7.0)   # t > 0 is overwritten (with 0 when the channel is off)
    ne[:, 0], ns[:, 0] = k1edge[f"ne0_{tag}"], k1edge[f"ns0_{tag}"]
    rho, rho_s = dev(ne), dev(ns)
    with np.errstate(invalid="ignore"):
        ctx.rate_equation(dev(E), rho, rho_s)
    r, s = host(rho), host(rho_s)
    ref_e, ref_s = k1edge[f"ne_{tag}"], k1edge[f"ns_{tag}"]
    assert np.array_equal(r[:, 0], np.float32(ne[:, 0]).astype(np.float64))
    err_e = _peak_err(r, ref_e)
    if tag == "ste1":
        # rows 9-11 saturate (row 11 at 3e16 W/cm^2 alternates between the
        # rescale and the decay with s / e ~ 1e-15): the FP32 march follows
        # them through the log-space form of e^{ze}
        err_s = _peak_err(s, ref_s)
        assert err_e.max() <= 2e-4, err_e.max(axis=1)
        assert err_s.max() <= 2e-4, err_s.max(axis=1)
        assert np.all(r[:, 1:] + s[:, 1:] <= float(k1edge["na"]) * (1 + 1e-6))
    else:
        # the saturating row (9) moves its clamp by a fraction of a sample in FP32
        assert np.all(np.delete(err_e, 9, axis=0) <= 2e-4), np.delete(err_e, 9, axis=0).max()
        assert err_e[9].max() <= 2e-3 and np.sum(err_e[9] > 2e-4) <= 4
        assert np.all(s[:, 1:] == 0)
    assert ctx.device_status() == 0


def test_update_plasma_matches_oracle(ste):
    c = ste
    rho, rs = dev(np.full(c.u0.shape, 3.0)), dev(np.full(c.u0.shape, 5.0))
    c.nl.update_plasma(dev(c.u0), rho, rs)
    ro, so = np.zeros(c.u0.shape), np.zeros(c.u0.shape)
    c.og.update_plasma(c.u0, ro, so)
    assert so.max() > 1e-3 * ro.max() > 0          # the channel is exercised
    assert np.all(_peak_err(host(rho), ro) <= 2e-4)
    assert np.all(_peak_err(host(rs), so) <= 2e-4)
    assert np.all(host(rho)[:, 0] == 0) and np.all(host(rs)[:, 0] == 0)


def test_split_index_term_matches_oracle(ste):
    c = ste
    ro, so = np.zeros(c.u0.shape), np.zeros(c.u0.shape)
    c.og.update_plasma(c.u0, ro, so)
    so = so * 50.0                                  # make the index term visible against Kerr
    rhs, alpha = c.nl.split(dev(c.u0), dev(ro), dev(so))
    ref, aref = c.og.split(c.u0, ro, so)
    ref0, _ = c.og.split(c.u0, ro, np.zeros_like(so))
    assert rel_l2(ref, ref0) > 1e-3                 # the term matters at this density
    assert rel_l2(host(rhs), ref) < 2e-5
    assert rel_l2(host(alpha), aref) < 2e-5


def test_ste_requires_rho_s(ste):
    from rapport_gb300._lib import NLSEError
    c = ste
    with pytest.raises(NLSEError, match="rho_s"):
        c.ctx.propagate(dev(c.u0), dev(np.zeros(c.u0.shape)), None, c.dz, 1)
    with pytest.raises(NLSEError, match="rho_s"):
        c.ctx.update_plasma(dev(c.u0), dev(np.zeros(c.u0.shape)), None)


@pytest.mark.parametrize("mode,tol", [(0, 1e-4), (1, 5e-5), (2, 5e-5)])
def test_propagate_matches_oracle(ste, mode, tol):
    c = ste
    u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
    c.ctx.propagate(u, rho, rs, c.dz, 10, mode)
    uo, ro, so = c.og.propagate(c.u0.copy(), 10, c.dz)
    assert rel_l2(host(u), uo) < tol
    assert np.abs(host(rho) - ro).max() <= 1e-3 * ro.max()
    assert np.abs(host(rs) - so).max() <= 1e-3 * so.max()
    assert c.ctx.device_status() == 0


def test_propagate_equals_update_plus_step(ste):
    c = ste
    for mode in (0, 1):
        u1, u2 = dev(c.u0), dev(c.u0)
        r1, r2 = dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        s1, s2 = dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u1, r1, s1, c.dz, 3, mode)
        for _ in range(3):
            c.nl.update_plasma(u2, r2, s2)
            c.ctx.step(u2, r2, c.dz, mode, s2)
        if mode == 0:
            assert np.array_equal(host(u1), host(u2))
        else:
            # the split form keeps the field in the spectral domain across steps
            assert rel_l2(host(u1), host(u2)) < 1e-6
        assert rel_l2(host(r1), host(r2)) < 1e-5
        assert rel_l2(host(s1), host(s2)) < 1e-5


def test_two_population_march_solves_every_row_at_nt_4096():
    """The reference's default physics on its default time grid (every term,
    N_t = 4096, 1024 radii: a 5 uJ pulse focused by a 10 cm lens): the Newton
    scan of the two-population march must solve every row.  At the rim of the
    ionised region the densities fall to ~1e-38 cm^-3, where the iterates settle
    into denormal rounding noise; a relative-only convergence test never met
    there sent ~0.7 rows a z-step to the sequential one-thread march (1.3 ms a
    row).  Densities stay finite and non-negative."""
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    over = dict(f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True, enable_space_time_focusing=True,
                enable_ste=True, enable_ste_index=True)
    cfg = R.workload_config(1024, 4096, 2e-3, 150e-6, 800e-15, 2.5e-6, 40, **over)
    g = R.build_grids(cfg)
    ctx = _lib.Context(cfg, g)
    u0 = R.envelope_lens(150e-6, 100e-15, 5.0, 0.1, 0)(g["rr"], g["tt"], cfg, g)
    u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
    ctx.propagate(u, rho, rs, 2.5e-6, 40, _lib.MODE_SPLIT_BF16)
    assert ctx.device_status() == 0
    assert ctx.scan_fallback_rows() == 0
    r, s = host(rho), host(rs)
    assert np.isfinite(r).all() and np.isfinite(s).all() and (r >= 0).all() and (s >= 0).all()
    assert r.max() > 0 and s.max() > 0
