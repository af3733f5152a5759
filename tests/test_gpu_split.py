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


def test_split_rejects_unsupported_grid(tiny):
    from rapport_gb300._lib import NLSEError
    c = Case.from_fixture(tiny)  # Nt = 128: not a multiple of the 256-column tile
    with pytest.raises(NLSEError, match="split-BF16"):
        c.ctx.half_linear(dev(c.u0), c.dz, MODE_SPLIT_BF16)


def test_config2_z_steps_split_vs_oracle():
    c = Case(**CONFIG2)
    uo, rho_o, _ = c.og.propagate(c.u0.copy(), 2, c.dz)
    for mode in SPLIT_MODES:
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 2, mode)
        assert rel_l2(host(u), uo) < 2e-5, mode
        assert np.abs(host(rho) - rho_o).max() <= 1e-3 * max(rho_o.max(), 1e-30), mode
        assert c.ctx.device_status() == 0
