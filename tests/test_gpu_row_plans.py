"""Row-kernel plans of the split forms and their autotuner.

Each of the two z-step row kernels has two or three plans (shared-memory or
register-resident body, compile-time or compact run-time FFT passes; the same
butterflies, twiddles and point arithmetic); the first context of an N_t times
them on synthetic rows and keeps the fastest.  The pick
may differ between devices and runs, so every plan must give the same result
bit for bit: checked here for N_t = 512 .. 8192 (where a second plan exists) on
a single context and on a batch, in both tensor-core forms."""
import numpy as np
import pytest

from gpu_util import dev, host

pytestmark = pytest.mark.gpu

DZ, STEPS = 5e-6, 3


def _setup(Nr, Nt):
    import rapport_gb300 as R
    cfg = R.workload_config(Nr, Nt, 1e-4 * Nr / 64, 1e-5, 3e-13 * Nt / 256, DZ, STEPS)
    g = R.build_grids(cfg)
    u0 = R.envelope_lens(1e-5, 100e-15, 2.0, 1e-2, 3)(g["rr"], g["tt"], cfg, g)
    return cfg, g, u0


def _run(ctx, u0, mode):
    u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
    ctx.propagate(u, rho, rs, DZ, STEPS, mode)
    assert ctx.device_status() == 0
    return host(u), host(rho)


@pytest.mark.parametrize("Nt", [512, 1024, 2048, 4096, 8192])
def test_row_plans_agree_bitwise(Nt):
    from rapport_gb300 import _lib
    Nr = 64 if Nt < 8192 else 32
    cfg, g, u0 = _setup(Nr, Nt)
    ctx = _lib.Context(cfg, g)       # tunes the plans of this N_t
    nl, nx = _lib.row_plans(Nt)
    assert nl in (0, 1, 2) and nx in (0, 1)
    try:
        for mode in (_lib.MODE_SPLIT_BF16, _lib.MODE_SPLIT_F16):
            outs = []
            for plans in ((0, 0), (1, 1), (2, 0), (1, 0)):
                _lib.set_row_plans(Nt, *plans)
                outs.append(_run(ctx, u0, mode))
            for u, rho in outs[1:]:
                assert np.array_equal(u, outs[0][0]), (Nt, mode)
                assert np.array_equal(rho, outs[0][1]), (Nt, mode)
            assert np.isfinite(outs[0][0]).all()
    finally:
        _lib.set_row_plans(Nt, nl, nx)


def test_batch_row_plans_agree_bitwise():
    """A batch with three N_t classes: its captured z-step graph follows a
    change of plan (re-captured), and the results do not change."""
    from rapport_gb300 import _lib
    shapes = [(64, 1024), (64, 2048), (64, 4096)]
    setups = [_setup(*s) for s in shapes]
    b = _lib.Batch([c for c, _, _ in setups], [g for _, g, _ in setups])
    saved = {Nt: _lib.row_plans(Nt) for _, Nt in shapes}
    try:
        outs = []
        for plans in ((0, 0), (1, 1), (2, 1)):
            for _, Nt in shapes:
                _lib.set_row_plans(Nt, *plans)
            us = [dev(u0) for _, _, u0 in setups]
            rhos = [dev(np.zeros(u0.shape)) for _, _, u0 in setups]
            b.propagate(us, rhos, None, DZ, 8)   # 8 steps: the graph path runs
            assert b.device_status() == 0
            outs.append([(host(u), host(r)) for u, r in zip(us, rhos)])
        for other in outs[1:]:
            for (u0_, r0_), (u1_, r1_) in zip(outs[0], other):
                assert np.array_equal(u0_, u1_)
                assert np.array_equal(r0_, r1_)
    finally:
        for Nt, (a, c) in saved.items():
            _lib.set_row_plans(Nt, a, c)
