"""Batches at the measured sizes, the workloads the bench times.

* The bench's batch: 8 pulses of the 1024 x 2048 grid (5 uJ, w0 150 um,
  f 10 cm, noise seeds 0..7), 2 z-steps in the split-BF16 and split-FP16
  forms.  Every pulse must equal its own single-context run bit for bit, and
  the split-BF16 result must lie within 2e-5 (relative L2) of the FP64
  reference for the same input, densities within 1e-3 of the peak.
* Mixed grids of the 64-pulse batch workload (bench.mixed_pulses, seed 1):
  pulses 2, 3, 9 and 31 -- 1024 x 2048, 1024 x 4096, 512 x 1024 and
  768 x 4096, i.e. three N_t classes and three operator sizes in one grouped
  product -- with the same two checks.

The FP64 reference is oracle/fp64_gpu.py (pinned to the numpy oracle, which
is pinned to the reference, in test_gpu_accuracy.py)."""
import numpy as np
import pytest

import nlse_oracle as O
from conftest import rel_l2
from gpu_util import dev, host

pytestmark = pytest.mark.gpu

BENCH = dict(Nr=1024, Nt=2048, R_max=2e-3, w0=150e-6, T_half=800e-15, fwhm=100e-15, E=5.0, f=0.1, dz=2.5e-6)
STEPS = 2


def _fp64(Nr, Nt, R_max, w0, T_half, u0, dz):
    import fp64_gpu
    og = O.OracleGrid(O.workload_config(Nr, Nt, R_max, w0, T_half))
    u, rho = fp64_gpu.FP64GPU(og).propagate(u0, STEPS, dz)
    return u.cpu().numpy(), rho.cpu().numpy()


def _run_batch(cfgs, grids, u0s, dz, mode):
    from rapport_gb300 import _lib
    b = _lib.Batch(cfgs, grids)
    b.set_mode(mode)
    us = [dev(u) for u in u0s]
    rhos = [dev(np.zeros(u.shape)) for u in u0s]
    b.propagate(us, rhos, None, dz, STEPS)
    assert b.device_status() == 0
    out = [(host(u), host(r)) for u, r in zip(us, rhos)]
    del b, us, rhos
    return out


def _single(cfg, g, u0, dz, mode):
    from rapport_gb300 import _lib
    ctx = _lib.Context(cfg, g)
    u, rho, rs = dev(u0), dev(np.zeros(u0.shape)), dev(np.zeros(u0.shape))
    ctx.propagate(u, rho, rs, dz, STEPS, mode)
    assert ctx.device_status() == 0
    return host(u), host(rho)


@pytest.mark.parametrize("mode", [1, 2])
def test_bench_batch_8x1024x2048(mode):
    import rapport_gb300 as R
    w = BENCH
    cfg = R.workload_config(w["Nr"], w["Nt"], w["R_max"], w["w0"], w["T_half"], w["dz"], STEPS)
    g = R.build_grids(cfg)
    u0s = [R.envelope_lens(w["w0"], w["fwhm"], w["E"], w["f"], i)(g["rr"], g["tt"], cfg, g) for i in range(8)]
    got = _run_batch([cfg] * 8, [g] * 8, u0s, w["dz"], mode)
    for i, u0 in enumerate(u0s):
        su, sr = _single(cfg, g, u0, w["dz"], mode)
        assert np.array_equal(got[i][0], su), i
        assert np.array_equal(got[i][1], sr), i
    for i in (0, 7):   # the FP64 reference for the first and the last pulse
        uo, ro = _fp64(w["Nr"], w["Nt"], w["R_max"], w["w0"], w["T_half"], u0s[i], w["dz"])
        assert rel_l2(got[i][0], uo) < 2e-5, i
        assert np.abs(got[i][1] - ro).max() <= 1e-3 * max(ro.max(), 1e-30), i


@pytest.mark.parametrize("mode", [1, 2])
def test_mixed_64_pulse_grids(mode):
    import bench
    import rapport_gb300 as R
    P = bench.mixed_pulses()
    picks = [P[i] for i in (2, 3, 9, 31)]
    assert sorted((p["Nr"], p["Nt"]) for p in picks) == [(512, 1024), (768, 4096), (1024, 2048), (1024, 4096)]
    dz = picks[0]["dz"]
    cfgs, grids, u0s = [], [], []
    for p in picks:
        cfg = R.workload_config(p["Nr"], p["Nt"], p["R_max"], p["w0"], p["T_half"], dz, STEPS)
        g = R.build_grids(cfg)
        cfgs.append(cfg)
        grids.append(g)
        u0s.append(R.envelope_lens(p["w0"], p["fwhm"], p["E"], p["f"], p["noise_seed"])(g["rr"], g["tt"], cfg, g))
    got = _run_batch(cfgs, grids, u0s, dz, mode)
    for i, (p, cfg, g, u0) in enumerate(zip(picks, cfgs, grids, u0s)):
        su, sr = _single(cfg, g, u0, dz, mode)
        assert np.array_equal(got[i][0], su), (i, p["Nr"], p["Nt"])
        assert np.array_equal(got[i][1], sr), (i, p["Nr"], p["Nt"])
        uo, ro = _fp64(p["Nr"], p["Nt"], p["R_max"], p["w0"], p["T_half"], u0, dz)
        assert rel_l2(got[i][0], uo) < 2e-5, (i, p["Nr"], p["Nt"])
        assert np.abs(got[i][1] - ro).max() <= 1e-3 * max(ro.max(), 1e-30), (i, p["Nr"], p["Nt"])
