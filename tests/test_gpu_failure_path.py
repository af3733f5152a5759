"""The device-side failure path: a bounded wait that runs out is reported, and
nothing hangs or faults.

The tensor-core product bounds every mbarrier wait by %globaltimer (2 s) and,
when one gives up, raises a bit in the context's status word, drains what it
issued and returns; nlse_device_status turns the word into NLSE_ERR_TIMEOUT.
nlse_debug_wait_timeout runs the same bounded wait with a 1 ms limit on an
mbarrier that nothing arrives on, so the wait always runs out -- the only way
to make it run out without a broken kernel.  Checked: the status reads
NLSE_ERR_TIMEOUT with its message (for the context and for a batch holding
it), the context still runs a normal call, and a fresh context is clean.
"""
import numpy as np
import pytest

from gpu_util import dev

pytestmark = pytest.mark.gpu


def _cfg(Nr=64, Nt=256):
    import rapport_gb300 as R
    cfg = R.workload_config(Nr, Nt, 1e-4, 1e-5, 3e-13, 5e-6, 1)
    return cfg, R.build_grids(cfg)


def test_context_wait_timeout_is_reported():
    import torch
    from rapport_gb300 import _lib
    cfg, g = _cfg()
    ctx = _lib.Context(cfg, g)
    assert ctx.device_status() == 0
    ctx.debug_wait_timeout(1000)
    torch.cuda.synchronize()
    with pytest.raises(_lib.NLSEError, match="bounded device wait gave up") as ei:
        ctx.device_status()
    assert ei.value.status == _lib.NLSE_ERR_TIMEOUT
    # the context stays usable: a normal call runs and its results are finite
    u0 = _lib_env(cfg, g)
    u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
    ctx.propagate(u, rho, rs, 5e-6, 2, _lib.MODE_SPLIT_BF16)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(u).all())
    # a fresh context starts with a clear status word
    ctx2 = _lib.Context(cfg, g)
    ctx2.propagate(u, rho, rs, 5e-6, 1, _lib.MODE_SPLIT_BF16)
    assert ctx2.device_status() == 0


def test_batch_reports_a_pulse_wait_timeout():
    import torch
    from rapport_gb300 import _lib
    cfg, g = _cfg()
    b = _lib.Batch([cfg, cfg], [g, g])
    u0 = _lib_env(cfg, g)
    us = [dev(u0), dev(u0)]
    rhos = [dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))]
    b.propagate(us, rhos, None, 5e-6, 2)
    assert b.device_status() == 0
    b.context(1).debug_wait_timeout(1000)
    torch.cuda.synchronize()
    with pytest.raises(_lib.NLSEError, match="pulse 1: a bounded device wait gave up") as ei:
        b.device_status()
    assert ei.value.status == _lib.NLSE_ERR_TIMEOUT


def test_wait_limit_is_checked():
    from rapport_gb300 import _lib
    cfg, g = _cfg()
    ctx = _lib.Context(cfg, g)
    for bad in (0, -5, 2_000_000):
        with pytest.raises(_lib.NLSEError, match="limit_us"):
            ctx.debug_wait_timeout(bad)
    assert ctx.device_status() == 0


def _lib_env(cfg, g):
    import rapport_gb300 as R
    return R.envelope_lens(1e-5, 100e-15, 2.0, 1e-2, 0)(g["rr"], g["tt"], cfg, g)
