"""The tensor-core split forms (tcgen05 + TMA) against FP64: split-BF16
(3-term operator, hi/lo field, 4 MMAs) and split-FP16 (operator and field
each in 2 scaled FP16 terms, 3 MMAs).

Tolerances: the operator product E'w is exact to ~2^-17 of |E'||w| per
element (BF16 hi/lo field, 3-term operator); whole half steps and z-steps
must stay within 2e-5 relative L2 of the FP64 oracle (the FP32 plain path's
bar), and the device status word must stay clear (no bounded wait gave up,
no FP16 overflow).
"""
import numpy as np
import pytest

from conftest import rel_l2
from gpu_util import CONFIG2, Case, dev, host
from rapport_gb300._lib import MODE_PLAIN_F32, MODE_SPLIT_BF16, MODE_SPLIT_F16

SPLIT_MODES = [MODE_SPLIT_BF16, MODE_SPLIT_F16]

pytestmark = pytest.mark.gpu

SMALL = dict(Nr=64, Nt=256, R_max=1e-4, w0=1e-5, T_half=3e-13, fwhm=100e-15, E=2.0, f=1e-2, dz=5e-6)
CFG1 = dict(Nr=256, Nt=512, R_max=1e-3, w0=100e-6, T_half=400e-15, fwhm=100e-15, E=1.0, f=0.1, dz=5e-6)


@pytest.fixture(scope="module")
def small():
    return Case(**SMALL)


@pytest.fixture(scope="module")
def c1():
    return Case(**CFG1)


def _operator(c):
    og = c.og
    th = -og.rholist**2 * c.dz / (4 * og.komega)
    E = (og.Y * np.exp(1j * th)[None, :]) @ og.Y - np.eye(og.Nr)
    return np.block([[E.real, -E.imag], [E.imag, E.real]])


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("name", ["small", "c1"])
def test_operator_product(name, variant, small, c1):
    import torch
    c = small if name == "small" else c1
    c.ctx.set_gemm_variant(variant)
    rng = np.random.default_rng(11)
    w = rng.standard_normal((2 * c.og.Nr, c.og.Nt)) * np.geomspace(1e3, 1e-2, c.og.Nt)[None, :]
    wd = torch.from_numpy(w.astype(np.float32)).cuda()
    out = torch.empty_like(wd)
    c.ctx.debug_operator_product(wd, out, c.dz)
    A = _operator(c)
    ref = A @ w.astype(np.float32).astype(np.float64)
    o = out.cpu().numpy().astype(np.float64)
    scale = np.abs(A) @ np.abs(w)
    assert np.all(np.abs(o - ref) <= 2e-5 * scale + 1e-30)
    assert rel_l2(o, ref) < 2e-5
    assert c.ctx.device_status() == 0
    c.ctx.set_gemm_variant(-1)


def test_gemm_variants_agree_bitwise(c1):
    import torch
    rng = np.random.default_rng(12)
    w = torch.from_numpy(rng.standard_normal((2 * c1.og.Nr, c1.og.Nt)).astype(np.float32)).cuda()
    outs = []
    for v in (0, 1):
        c1.ctx.set_gemm_variant(v)
        o = torch.empty_like(w)
        c1.ctx.debug_operator_product(w, o, c1.dz)
        outs.append(o.cpu().numpy())
    c1.ctx.set_gemm_variant(-1)
    # same MMAs, same k order within the accumulator: identical results
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("mode", SPLIT_MODES)
@pytest.mark.parametrize("name", ["small", "c1"])
def test_half_linear_split(name, mode, small, c1):
    c = small if name == "small" else c1
    u = dev(c.u0)
    c.ctx.half_linear(u, c.dz, mode)
    assert rel_l2(host(u), c.og.half_linear(c.u0, c.dz)) < 2e-5
    assert c.ctx.device_status() == 0


@pytest.mark.parametrize("terms", [3, 2])
def test_propagate_split_vs_oracle(small, terms):
    c = small
    c.ctx.set_split_terms(terms)
    try:
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.ones(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 10, MODE_SPLIT_BF16)
        uo, rho_o, _ = c.og.propagate(c.u0.copy(), 10, c.dz)
        assert rel_l2(host(u), uo) < 5e-5
        assert np.abs(host(rho) - rho_o).max() <= 1e-3 * rho_o.max()
        assert np.all(host(rs) == 0)
        assert c.ctx.device_status() == 0
    finally:
        c.ctx.set_split_terms(3)


def test_propagate_split_f16_vs_oracle(small, c1):
    for c in (small, c1):
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.ones(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 10, MODE_SPLIT_F16)
        uo, rho_o, _ = c.og.propagate(c.u0.copy(), 10, c.dz)
        assert rel_l2(host(u), uo) < 5e-5
        assert np.abs(host(rho) - rho_o).max() <= 1e-3 * rho_o.max()
        assert np.all(host(rs) == 0)
        assert c.ctx.device_status() == 0


def test_split_forms_switch_on_one_context(small):
    """The operator is rebuilt when the form changes; results do not depend on the order."""
    c = small
    outs = {}
    for mode in (MODE_SPLIT_F16, MODE_SPLIT_BF16, MODE_SPLIT_F16):
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 3, mode)
        outs.setdefault(mode, []).append(host(u))
    assert np.array_equal(outs[MODE_SPLIT_F16][0], outs[MODE_SPLIT_F16][1])
    assert rel_l2(outs[MODE_SPLIT_F16][0], outs[MODE_SPLIT_BF16][0]) < 2e-5


@pytest.mark.parametrize("mode", SPLIT_MODES)
def test_step_split_equals_plain_within_fp32(small, mode):
    c = small
    rho = np.zeros(c.u0.shape)
    c.og.update_plasma(c.u0, rho, np.zeros(c.u0.shape))
    u1, u2 = dev(c.u0), dev(c.u0)
    c.ctx.step(u1, dev(rho), c.dz, MODE_PLAIN_F32)
    c.ctx.step(u2, dev(rho), c.dz, mode)
    ref = c.og.step(c.u0, rho, np.zeros(c.u0.shape), c.dz)
    assert rel_l2(host(u1), ref) < 2e-5
    assert rel_l2(host(u2), ref) < 2e-5


@pytest.mark.parametrize("mode", SPLIT_MODES)
def test_split_small_nt_matches_reference_fixture(tiny, mode):
    """N_t = 128 (below the 256-column tile: one partial tile column) in the
    tensor-core forms, against the reference's own z-steps (tiny.npz) at the
    plain form's tolerance."""
    c = Case.from_fixture(tiny)
    u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
    done = 0
    for j, s in enumerate(tiny["steps_kept"]):
        c.ctx.propagate(u, rho, rs, c.dz, int(s) - done, mode)
        done = int(s)
        assert rel_l2(host(u)[tiny["rows"]], tiny["u_steps"][j]) < 1e-4, s
        ro = tiny["rho_steps"][j]
        assert np.abs(host(rho)[tiny["rows"]] - ro).max() <= 1e-3 * max(ro.max(), 1e-30), s
    assert c.ctx.device_status() == 0


# radial sizes that are not multiples of 64: the context pads them (zero rows
# and columns of E', zero padding rows of the state).  1023 and 2999 are the
# grids run(Nr=1024) and run(Nr=3000) build (Config.N - 1 points).
PADDED = [dict(Nr=100, Nt=256, R_max=1.5e-4, w0=1e-5, T_half=3e-13, fwhm=100e-15, E=2.0, f=1e-2, dz=5e-6),
          dict(Nr=1023, Nt=2048, R_max=2e-3, w0=150e-6, T_half=800e-15, fwhm=100e-15, E=5.0, f=0.1, dz=2.5e-6),
          dict(Nr=2999, Nt=1024, R_max=3e-3, w0=150e-6, T_half=600e-15, fwhm=100e-15, E=5.0, f=0.1, dz=2.5e-6)]


@pytest.mark.parametrize("k", range(len(PADDED)))
def test_padded_radial_grid_vs_fp64(k):
    import fp64_gpu
    p = PADDED[k]
    c = Case(**p)
    ur, rr = fp64_gpu.FP64GPU(c.og).propagate(c.u0, 2, c.dz)
    ur, rr = ur.cpu().numpy(), rr.cpu().numpy()
    for mode in SPLIT_MODES:
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 2, mode)
        assert rel_l2(host(u), ur) < 2e-5, (p["Nr"], mode)
        assert np.abs(host(rho) - rr).max() <= 1e-3 * max(rr.max(), 1e-30), (p["Nr"], mode)
        hl = dev(c.u0)
        c.ctx.half_linear(hl, c.dz, mode)
        assert rel_l2(host(hl), c.og.half_linear(c.u0, c.dz)) < 2e-5, (p["Nr"], mode)
    assert c.ctx.device_status() == 0


def test_padded_operator_product():
    """The diagnostic product on a padded grid equals E'w on the unpadded E'."""
    import torch
    c = Case(**PADDED[0])
    rng = np.random.default_rng(13)
    w = rng.standard_normal((2 * c.og.Nr, c.og.Nt))
    wd = torch.from_numpy(w.astype(np.float32)).cuda()
    out = torch.empty_like(wd)
    c.ctx.debug_operator_product(wd, out, c.dz)
    A = _operator(c)
    ref = A @ w.astype(np.float32).astype(np.float64)
    o = out.cpu().numpy().astype(np.float64)
    assert np.all(np.abs(o - ref) <= 2e-5 * (np.abs(A) @ np.abs(w)) + 1e-30)


def test_config2_z_steps_split_vs_oracle():
    c = Case(**CONFIG2)
    uo, rho_o, _ = c.og.propagate(c.u0.copy(), 2, c.dz)
    for mode in SPLIT_MODES:
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 2, mode)
        assert rel_l2(host(u), uo) < 2e-5, mode
        assert np.abs(host(rho) - rho_o).max() <= 1e-3 * max(rho_o.max(), 1e-30), mode
        assert c.ctx.device_status() == 0
