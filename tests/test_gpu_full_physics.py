"""Full-physics split() through the C ABI: Raman (f_R 0.18), self-steepening,
space-time focusing and excitons, against the reference's own outputs
(tiny_full.npz) and the FP64 oracle (pinned to that fixture).

Each row's transforms run in shared memory inside the nonlinear block.
Tolerances, FP32 against FP64: half_linear / split / the nonlinear block
relative L2 2e-5; 4 z-steps 1e-4 (field) and 1e-3 of the peak (densities).
"""
import numpy as np
import pytest

from conftest import FULL_PHYSICS, meta_case, rel_l2
from gpu_util import Case, dev, host

pytestmark = pytest.mark.gpu

NO_STF = {k: v for k, v in FULL_PHYSICS.items() if k != "enable_space_time_focusing"}
# each term alone (the block takes a different transform path for each)
SINGLE = {
    "raman": dict(f_R=0.18, enable_kerr_raman=True),
    "steep": dict(enable_self_steepening=True),
    "stf": dict(enable_space_time_focusing=True),
    "steep+stf": dict(enable_self_steepening=True, enable_space_time_focusing=True),
}


def _case(full, **over):
    m = meta_case(full)
    return Case(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"], m["fwhm"], m["E"], m["f"], m["dz"],
                m["nsteps"], m["seed"], **over)


@pytest.fixture(scope="module")
def fc(full):
    return _case(full, **FULL_PHYSICS)


def _plasma(c, u):
    rho, rs = np.zeros(u.shape), np.zeros(u.shape)
    c.og.update_plasma(u, rho, rs)
    return rho, rs


def test_half_linear_space_time_focusing(fc, full):
    out = fc.lin.half_linear(dev(fc.u0), fc.dz)
    assert rel_l2(host(out), full["hl_u0"]) < 2e-5
    assert rel_l2(host(out), fc.og.half_linear(fc.u0, fc.dz)) < 2e-5


def test_split_matches_reference_fixture(fc, full):
    hl = fc.og.half_linear(fc.u0, fc.dz)
    rho, rs = _plasma(fc, fc.u0)
    rhs, alpha = fc.nl.split(dev(hl), dev(rho), dev(rs))
    assert rel_l2(host(rhs), full["split_rhs"]) < 2e-5
    assert rel_l2(host(alpha), full["split_alpha"]) < 2e-5


@pytest.mark.parametrize("term", sorted(SINGLE))
def test_split_each_term_vs_oracle(full, term):
    c = _case(full, **SINGLE[term])
    hl = c.og.half_linear(c.u0, c.dz)
    rho, rs = _plasma(c, c.u0)
    rhs, alpha = c.nl.split(dev(hl), dev(rho), dev(rs))
    ref, aref = c.og.split(hl, rho, rs)
    assert rel_l2(host(rhs), ref) < 2e-5
    assert rel_l2(host(alpha), aref) < 2e-5


def test_terms_change_the_rhs(full):
    """Each term moves split() well above the tolerance (the tests above see it)."""
    plain = _case(full)
    hl = plain.og.half_linear(plain.u0, plain.dz)
    rho, rs = _plasma(plain, plain.u0)
    r0, _ = plain.og.split(hl, rho, rs)
    for term, over in SINGLE.items():
        c = _case(full, **over)
        r1, _ = c.og.split(hl, rho, rs)
        assert rel_l2(r1, r0) > 1e-3, term


def test_nonlinear_block_vs_oracle(fc):
    hl = fc.og.half_linear(fc.u0, fc.dz)
    rho, rs = _plasma(fc, fc.u0)
    u = dev(hl)
    fc.nl.nonlinear_step(u, dev(rho), fc.dz, dev(rs))
    assert rel_l2(host(u), fc.oracle_nl_block(hl, rho, rs)) < 2e-5


def test_propagate_matches_reference_fixture(fc, full):
    u, rho, rs = dev(fc.u0), dev(np.zeros(fc.u0.shape)), dev(np.zeros(fc.u0.shape))
    done = 0
    for j, s in enumerate(full["steps_kept"]):
        fc.ctx.propagate(u, rho, rs, fc.dz, int(s) - done)
        done = int(s)
        assert rel_l2(host(u), full["u_steps"][j]) < 1e-4, s
        ro, so = full["rho_steps"][j], full["rho_s_steps"][j]
        assert np.abs(host(rho) - ro).max() <= 1e-3 * ro.max(), s
        assert np.abs(host(rs) - so).max() <= 1e-3 * so.max(), s


def test_row_with_a_nan_gets_no_nonlinear_term(fc):
    """One NaN sample makes the reference's whole row of split() non-finite
    (it passes through the row FFTs), and nan_to_num turns the row into 0."""
    hl = fc.og.half_linear(fc.u0, fc.dz)
    rho, rs = _plasma(fc, fc.u0)
    bad = hl.copy()
    bad[5, 40] = np.nan
    with np.errstate(invalid="ignore"):
        ref, _ = fc.og.split(bad, rho, rs)
    rhs, _ = fc.nl.split(dev(bad), dev(rho), dev(rs))
    got = host(rhs)
    assert np.all(ref[5] == 0) and np.all(got[5] == 0)
    keep = np.arange(got.shape[0]) != 5
    assert rel_l2(got[keep], ref[keep]) < 2e-5


def test_split_forms_without_space_time_focusing(full):
    """Raman + self-steepening + excitons in the tensor-core forms (row_nl runs
    the full block; the merged operator I + E)."""
    from rapport_gb300 import _lib
    m = meta_case(full)
    c = Case(64, 256, m["R_max"], m["w0"], m["T_half"], m["fwhm"], m["E"], m["f"], m["dz"], 4, 0, **NO_STF)
    uo, ro, so = c.og.propagate(c.u0.copy(), 4, c.dz)
    for mode in (_lib.MODE_SPLIT_BF16, _lib.MODE_SPLIT_F16):
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 4, mode)
        assert rel_l2(host(u), uo) < 5e-5, mode
        assert np.abs(host(rho) - ro).max() <= 1e-3 * ro.max(), mode
        assert np.abs(host(rs) - so).max() <= 1e-3 * so.max(), mode
        assert c.ctx.device_status() == 0


@pytest.mark.parametrize("mode", [1, 2])
def test_split_forms_every_term_match_reference_fixture(fc, full, mode):
    """The reference's default physics -- space-time focusing with Raman,
    self-steepening and excitons -- in the tensor-core forms: the half step is
    the sandwich Y P(rho, Omega) Y in scaled FP16 terms, against the
    reference's own z-steps (tiny_full.npz) at the plain form's tolerance."""
    u, rho, rs = dev(fc.u0), dev(np.zeros(fc.u0.shape)), dev(np.zeros(fc.u0.shape))
    done = 0
    for j, s in enumerate(full["steps_kept"]):
        fc.ctx.propagate(u, rho, rs, fc.dz, int(s) - done, mode)
        done = int(s)
        assert rel_l2(host(u), full["u_steps"][j]) < 1e-4, s
        ro, so = full["rho_steps"][j], full["rho_s_steps"][j]
        assert np.abs(host(rho) - ro).max() <= 1e-3 * ro.max(), s
        assert np.abs(host(rs) - so).max() <= 1e-3 * so.max(), s
    assert fc.ctx.device_status() == 0


@pytest.mark.parametrize("over,shape", [(FULL_PHYSICS, (64, 256)), (SINGLE["stf"], (256, 512)),
                                        (SINGLE["stf"], (100, 1024)), (FULL_PHYSICS, (32, 4096))])
def test_split_space_time_focusing_vs_oracle(full, over, shape):
    """Space-time focusing in the tensor-core forms against the FP64 oracle:
    with every term and alone, on a radial size that is padded (100 -> 128),
    and with every term at N_t = 4096 (the full-physics block and the exciton
    march at 512 threads a row)."""
    from rapport_gb300 import _lib
    m = meta_case(full)
    Nr, Nt = shape
    c = Case(Nr, Nt, m["R_max"] * Nr / 64, m["w0"], m["T_half"] * Nt / 128, m["fwhm"], m["E"], m["f"], m["dz"],
             4, 0, **over)
    uo, ro, so = c.og.propagate(c.u0.copy(), 4, c.dz)
    hl_o = c.og.half_linear(c.u0, c.dz)
    for mode in (_lib.MODE_SPLIT_BF16, _lib.MODE_SPLIT_F16):
        hl = dev(c.u0)
        c.ctx.half_linear(hl, c.dz, mode)
        assert rel_l2(host(hl), hl_o) < 2e-5, (shape, mode)
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 4, mode)
        assert rel_l2(host(u), uo) < 5e-5, (shape, mode)
        assert np.abs(host(rho) - ro).max() <= 1e-3 * max(ro.max(), 1e-30), (shape, mode)
        if so.max() > 0:
            assert np.abs(host(rs) - so).max() <= 1e-3 * so.max(), (shape, mode)
        assert c.ctx.device_status() == 0


def test_full_physics_limits():
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    cfg = R.workload_config(16, 8192, 1e-4, 1e-5, 3e-13, 5e-6, 1, enable_self_steepening=True)
    with pytest.raises(_lib.NLSEError, match="4096"):
        _lib.Context(cfg, R.build_grids(cfg))


def _raman_fit_error(Rf):
    """Relative error of the damped-sine model of the Raman kernel ifft(R_f)
    (the check the library makes before it takes the recurrence)."""
    n = len(Rf)
    k = np.fft.ifft(Rf).real
    k1, k2, k3 = k[1], k[2], k[3]
    p = k2 / k1
    q = (p * k2 - k3) / k1
    r = np.sqrt(q)
    th = np.arccos(p / (2 * r))
    a = k1 / (r * np.sin(th))
    m = np.arange(n)
    z = r * np.exp(1j * th)
    model = (a * z ** np.where(m == 0, n, m) / (1 - z ** n)).imag
    return np.abs(model - k).max() / np.abs(k).max()


@pytest.mark.parametrize("Nt", [1024, 2048])
def test_raman_recurrence_vs_oracle(Nt):
    """On a +-800 fs window the Raman response has decayed to ~e^-25 at the
    window's half width, so the library takes the Raman convolution as the
    periodic solution of a first-order recurrence (a block scan) instead of
    two row FFTs: split() and 6 z-steps with every term on, in the plain and
    split-BF16 forms, against the FP64 oracle (which convolves by FFTs as the
    reference does)."""
    from rapport_gb300 import _lib
    c = Case(64, Nt, 2e-4, 2e-5, 800e-15, 100e-15, 2.0, 1e-2, 5e-6, 6, 0, **FULL_PHYSICS)
    assert _raman_fit_error(c.g["R_f"]) <= 1e-9  # the library's acceptance test
    z0 = np.zeros(c.u0.shape)
    rhs_o, al_o = c.og.split(c.u0, z0, z0)
    rhs, al = c.nl.split(dev(c.u0), dev(z0), dev(z0))
    assert rel_l2(host(rhs), rhs_o) < 2e-5
    uo, ro, so = c.og.propagate(c.u0.copy(), 6, c.dz)
    for mode in (_lib.MODE_PLAIN_F32, _lib.MODE_SPLIT_BF16):
        u, rho, rs = dev(c.u0), dev(z0), dev(z0)
        c.ctx.propagate(u, rho, rs, c.dz, 6, mode)
        assert rel_l2(host(u), uo) < 5e-5, mode
        assert np.abs(host(rho) - ro).max() <= 1e-3 * max(ro.max(), 1e-30), mode
        if so.max() > 0:
            assert np.abs(host(rs) - so).max() <= 1e-3 * so.max(), mode
    assert c.ctx.device_status() == 0
