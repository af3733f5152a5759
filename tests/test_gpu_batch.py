"""Batches of pulses with uneven grids (nlse_batch_*), split-BF16 / split-FP16 forms.

A batch runs the same per-pulse arithmetic as a single-pulse context (grouped
tensor-core launch over every pulse's tiles, one row launch per time-grid
class), so every pulse must come out bit-identical to its single-context
split-BF16 run, and within the parity tolerance of the FP64 oracle."""
import numpy as np
import pytest

import nlse_oracle as O
from conftest import rel_l2
from gpu_util import dev, host

pytestmark = pytest.mark.gpu

# (Nr, Nt, R_max, w0, T_half, fwhm, E_uJ, f) -- three grids, two time classes
PULSES = [(64, 256, 1e-4, 1e-5, 3e-13, 100e-15, 2.0, 1e-2),
          (128, 512, 2e-4, 2e-5, 4e-13, 80e-15, 6.0, 2e-2),
          (64, 512, 1.5e-4, 1.5e-5, 3e-13, 120e-15, 3.0, 1.5e-2)]
DZ, STEPS = 5e-6, 6


def _setup():
    import rapport_gb300 as R
    cfgs, grids, u0s, ogs = [], [], [], []
    for i, (Nr, Nt, Rm, w0, Th, fw, E, f) in enumerate(PULSES):
        cfg = R.workload_config(Nr, Nt, Rm, w0, Th, DZ, STEPS)
        g = R.build_grids(cfg)
        cfgs.append(cfg)
        grids.append(g)
        u0s.append(R.envelope_lens(w0, fw, E, f, i)(g["rr"], g["tt"], cfg, g))
        ogs.append(O.OracleGrid(O.workload_config(Nr, Nt, Rm, w0, Th)))
    return cfgs, grids, u0s, ogs


def test_batch_matches_single_contexts_and_oracle():
    from rapport_gb300 import _lib
    cfgs, grids, u0s, ogs = _setup()
    b = _lib.Batch(cfgs, grids)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    rss = [dev(np.ones(u.shape)) for u in u0s]
    b.propagate(us, rhos, rss, DZ, STEPS)
    assert b.device_status() == 0
    for i, (cfg, g, u0, og) in enumerate(zip(cfgs, grids, u0s, ogs)):
        ctx = _lib.Context(cfg, g)
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, STEPS, _lib.MODE_SPLIT_BF16)
        assert np.array_equal(host(us[i]), host(u)), i
        assert np.array_equal(host(rhos[i]), host(rho)), i
        assert np.all(host(rss[i]) == 0)
        uo, rho_o, _ = og.propagate(u0.copy(), STEPS, DZ)
        assert rel_l2(host(us[i]), uo) < 5e-5, i
        assert np.abs(host(rhos[i]) - rho_o).max() <= 1e-3 * max(rho_o.max(), 1e-30), i


def test_batch_two_calls_equal_one():
    from rapport_gb300 import _lib
    cfgs, grids, u0s, _ = _setup()
    b = _lib.Batch(cfgs, grids)
    a = [dev(u) for u in u0s]
    ra = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(a, ra, None, DZ, STEPS)
    c = [dev(u) for u in u0s]
    rc = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(c, rc, None, DZ, STEPS // 2)
    b.propagate(c, rc, None, DZ, STEPS - STEPS // 2)
    for i in range(len(a)):
        # a call boundary rounds the field through the physical domain once
        assert rel_l2(host(c[i]), host(a[i])) < 1e-6


def test_batch_takes_padded_grids():
    """N_r not a multiple of 64 (padded inside each context) and N_t = 128 (one
    partial tile column) in one grouped product: every pulse bit-identical to
    its single-context run and within the parity tolerance of the oracle."""
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    shapes = [(100, 128, 1.5e-4), (64, 256, 1e-4), (70, 128, 1.1e-4)]
    cfgs, grids, u0s = [], [], []
    for i, (Nr, Nt, Rm) in enumerate(shapes):
        cfg = R.workload_config(Nr, Nt, Rm, 1e-5, 3e-13 * Nt / 256, DZ, STEPS)
        g = R.build_grids(cfg)
        cfgs.append(cfg)
        grids.append(g)
        u0s.append(R.envelope_lens(1e-5, 100e-15, 1.5 + 0.3 * i, 1e-2, 40 + i)(g["rr"], g["tt"], cfg, g))
    b = _lib.Batch(cfgs, grids)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(us, rhos, None, DZ, STEPS)
    assert b.device_status() == 0
    for i, ((Nr, Nt, Rm), cfg, g, u0) in enumerate(zip(shapes, cfgs, grids, u0s)):
        ctx = _lib.Context(cfg, g)
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, STEPS, _lib.MODE_SPLIT_BF16)
        assert np.array_equal(host(us[i]), host(u)), i
        assert np.array_equal(host(rhos[i]), host(rho)), i
        og = O.OracleGrid(O.workload_config(Nr, Nt, Rm, 1e-5, 3e-13 * Nt / 256))
        uo, rho_o, _ = og.propagate(u0.copy(), STEPS, DZ)
        assert rel_l2(host(us[i]), uo) < 5e-5, i
        assert np.abs(host(rhos[i]) - rho_o).max() <= 1e-3 * max(rho_o.max(), 1e-30), i


def test_batch_shared_operator_pulses_match_single_contexts():
    """Pulses on one grid share the first pulse's operator copy inside the batch."""
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    cfg = R.workload_config(64, 256, 1e-4, 1e-5, 3e-13, DZ, STEPS)
    g = R.build_grids(cfg)
    u0s = [R.envelope_lens(1e-5, 100e-15, 1.5 + i, 1e-2, 10 + i)(g["rr"], g["tt"], cfg, g) for i in range(3)]
    b = _lib.Batch([cfg] * 3, [g] * 3)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(us, rhos, None, DZ, STEPS)
    ctx = _lib.Context(cfg, g)
    for i, u0 in enumerate(u0s):
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, STEPS, _lib.MODE_SPLIT_BF16)
        assert np.array_equal(host(us[i]), host(u)), i
        assert np.array_equal(host(rhos[i]), host(rho)), i


@pytest.mark.parametrize("mode", [0, 1])
def test_step_batched_equals_propagate_per_pulse(mode):
    """nlse_step_batched: pulses on one context's grid, each exactly as its own nlse_propagate."""
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    cfg = R.workload_config(64, 256, 1e-4, 1e-5, 3e-13, DZ, STEPS)
    g = R.build_grids(cfg)
    u0s = [R.envelope_lens(1e-5, 100e-15, 1.0 + i, 1e-2, i)(g["rr"], g["tt"], cfg, g) for i in range(3)]
    ctx = _lib.Context(cfg, g)
    bu = [dev(u) for u in u0s]
    br = [dev(np.zeros(u.shape)) for u in u0s]
    ctx.step_batched([(u, r, None) for u, r in zip(bu, br)], DZ, STEPS, mode)
    for i, u0 in enumerate(u0s):
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, STEPS, mode)
        assert np.array_equal(host(bu[i]), host(u)), i
        assert np.array_equal(host(br[i]), host(rho)), i
    with pytest.raises(_lib.NLSEError, match="pulse 0: dz"):
        ctx.step_batched([(bu[0], br[0], None), (bu[1], br[1], None)], -1.0, 1, mode)


def test_batch_f16_equals_single_contexts():
    """The split-FP16 form in a batch: every pulse bit-identical to its single-context run."""
    from rapport_gb300 import _lib
    cfgs, grids, u0s, ogs = _setup()
    b = _lib.Batch(cfgs, grids)
    b.set_mode(_lib.MODE_SPLIT_F16)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(us, rhos, None, DZ, STEPS)
    for i, (cfg, g, u0, og) in enumerate(zip(cfgs, grids, u0s, ogs)):
        ctx = _lib.Context(cfg, g)
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, STEPS, _lib.MODE_SPLIT_F16)
        assert np.array_equal(host(us[i]), host(u)), i
        assert np.array_equal(host(rhos[i]), host(rho)), i
        uo, _, _ = og.propagate(u0.copy(), STEPS, DZ)
        assert rel_l2(host(us[i]), uo) < 5e-5, i
        assert ctx.device_status() == 0


# (Nr, Nt, overrides): the measured toggles, Raman + self-steepening, the
# exciton channel, and both -- one batch, three row classes
MIXED = [(64, 256, {}),
         (64, 256, dict(f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True)),
         (128, 512, dict(enable_ste=True, tau_ste=1e-12)),
         (64, 512, dict(enable_ste=True, tau_ste=5e-13, f_R=0.18, enable_kerr_raman=True))]


def _mixed_setup():
    import rapport_gb300 as R
    cfgs, grids, u0s = [], [], []
    for i, (Nr, Nt, over) in enumerate(MIXED):
        # ~1 uJ at w0 15 um: at 5 uJ / 10 um self-steepening on this 256-point
        # window already diverges in the FP64 oracle within six steps
        cfg = R.workload_config(Nr, Nt, 1e-4 * Nr / 64, 1.5e-5, 3e-13 * Nt / 256, DZ, STEPS, **over)
        g = R.build_grids(cfg)
        cfgs.append(cfg)
        grids.append(g)
        u0s.append(R.envelope_lens(1.5e-5, 100e-15, 1.0 + 0.1 * i, 1e-2, 20 + i)(g["rr"], g["tt"], cfg, g))
    return cfgs, grids, u0s


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_full_physics_and_exciton_pulses_equal_single_contexts(mode):
    """Raman / self-steepening pulses (their own row class) and exciton-channel
    pulses (their two-population march launched per pulse, also inside the
    z-step graph) in one batch: each bit-identical to its single-context run,
    including after a second call on new buffers (the graph is re-captured)."""
    from rapport_gb300 import _lib
    cfgs, grids, u0s = _mixed_setup()
    b = _lib.Batch(cfgs, grids)
    b.set_mode(mode)
    runs = []
    for _ in range(2):  # the second call passes new tensors (new pointers)
        us = [dev(u) for u in u0s]
        rhos = [dev(np.zeros(u.shape)) for u in u0s]
        rss = [dev(np.ones(u.shape)) for u in u0s]
        b.propagate(us, rhos, rss, DZ, STEPS)
        assert b.device_status() == 0
        runs.append(([host(x) for x in us], [host(x) for x in rhos], [host(x) for x in rss]))
    for i, (cfg, g, u0) in enumerate(zip(cfgs, grids, u0s)):
        ctx = _lib.Context(cfg, g)
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, STEPS, mode)
        assert ctx.device_status() == 0
        for bu, brho, brs in runs:
            assert np.array_equal(bu[i], host(u)), i
            assert np.array_equal(brho[i], host(rho)), i
            assert np.array_equal(brs[i], host(rs)), i
        ste = bool(MIXED[i][2].get("enable_ste"))
        assert (host(rs).max() > 0) == ste, i  # exciton density only where the channel is on
        Nr, Nt, over = MIXED[i]
        og = O.OracleGrid(O.workload_config(Nr, Nt, 1e-4 * Nr / 64, 1.5e-5, 3e-13 * Nt / 256, **over))
        uo, rho_o, rs_o = og.propagate(O.lens_gaussian(og, 1.5e-5, 100e-15, 1.0 + 0.1 * i, 1e-2, 20 + i), STEPS, DZ)
        assert rel_l2(host(u), uo) < 5e-5, i
        assert np.abs(host(rho) - rho_o).max() <= 1e-3 * rho_o.max(), i
        if ste:
            assert np.abs(host(rs) - rs_o).max() <= 1e-3 * rs_o.max(), i


def test_batch_exciton_pulse_needs_rho_s():
    from rapport_gb300 import _lib
    cfgs, grids, u0s = _mixed_setup()
    b = _lib.Batch(cfgs, grids)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    with pytest.raises(_lib.NLSEError, match="rho_s is required"):
        b.propagate(us, rhos, None, DZ, STEPS)


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_with_space_time_focusing_pulses(mode):
    """Pulses with space-time focusing (their own grouped products of the
    sandwich Y P Y and a phase pass each) beside pulses in the batch's form:
    every pulse bit-identical to its single-context run, within the parity
    tolerance of the oracle, also over enough steps for the z-step graph."""
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    spec = [(64, 256, dict(enable_space_time_focusing=True)), (64, 256, {}),
            (100, 512, dict(enable_space_time_focusing=True, f_R=0.18, enable_kerr_raman=True)),
            (128, 512, {})]
    cfgs, grids, u0s = [], [], []
    for i, (Nr, Nt, over) in enumerate(spec):
        cfg = R.workload_config(Nr, Nt, 1e-4 * Nr / 64, 1.5e-5, 3e-13 * Nt / 256, DZ, 8, **over)
        g = R.build_grids(cfg)
        cfgs.append(cfg)
        grids.append(g)
        u0s.append(R.envelope_lens(1.5e-5, 100e-15, 1.0 + 0.2 * i, 1e-2, 30 + i)(g["rr"], g["tt"], cfg, g))
    b = _lib.Batch(cfgs, grids)
    b.set_mode(mode)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(us, rhos, None, DZ, 8)
    assert b.device_status() == 0
    for i, ((Nr, Nt, over), cfg, g, u0) in enumerate(zip(spec, cfgs, grids, u0s)):
        ctx = _lib.Context(cfg, g)
        u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
        ctx.propagate(u, rho, rs, DZ, 8, mode)
        assert np.array_equal(host(us[i]), host(u)), i
        assert np.array_equal(host(rhos[i]), host(rho)), i
        og = O.OracleGrid(O.workload_config(Nr, Nt, 1e-4 * Nr / 64, 1.5e-5, 3e-13 * Nt / 256, **over))
        uo, rho_o, _ = og.propagate(O.lens_gaussian(og, 1.5e-5, 100e-15, 1.0 + 0.2 * i, 1e-2, 30 + i), 8, DZ)
        assert rel_l2(host(us[i]), uo) < 5e-5, i
        assert np.abs(host(rhos[i]) - rho_o).max() <= 1e-3 * max(rho_o.max(), 1e-30), i


def test_batch_tunes_its_own_product_and_keeps_a_pinned_variant():
    """The batch times the product's pipeline variants on its own grouped
    launch (nlse_api.cu batch_tune) and takes the faster, in each form; the
    variants agree bit for bit, so every pulse still equals its single-context
    run.  A variant pinned on the first pulse's context is kept."""
    from rapport_gb300 import _lib
    cfgs, grids, u0s, _ = _setup()
    for mode in (_lib.MODE_SPLIT_BF16, _lib.MODE_SPLIT_F16):
        b = _lib.Batch(cfgs, grids)
        b.set_mode(mode)
        us = [dev(u) for u in u0s]
        rhos = [dev(np.zeros(u.shape)) for u in u0s]
        b.propagate(us, rhos, None, DZ, STEPS)
        assert b.device_status() == 0
        assert b.context(0).gemm_variant() in (0, 1)
        for i, (cfg, g, u0) in enumerate(zip(cfgs, grids, u0s)):
            ctx = _lib.Context(cfg, g)
            u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
            ctx.propagate(u, rho, rs, DZ, STEPS, mode)
            assert np.array_equal(host(us[i]), host(u)), (mode, i)
            assert np.array_equal(host(rhos[i]), host(rho)), (mode, i)
    b = _lib.Batch(cfgs, grids)
    b.context(0).set_gemm_variant(3)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(us, rhos, None, DZ, STEPS)
    assert b.device_status() == 0
    assert b.context(0).gemm_variant() == 3
