"""Run every kernel of libnlse once on the 1024 x 2048 workload (for profiling).

``python -m rapport_gb300.kernel_tour`` builds the measured workload (800 nm in
fused silica, 5 uJ, w0 150 um, f 10 cm, dz 2.5 um, seeded 1 % noise) and calls,
in order: the plain half step, split(), the nonlinear block, update_plasma,
one z-step and a 2-step propagate in each arithmetic (plain FP32, split-BF16,
split-FP16), a 2-step propagate of 8 such pulses in one batch (both split
forms), the record reductions, the exciton-channel march, the full-physics
split / nonlinear block (Raman, self-steepening, space-time focusing) and the
fused full-physics row kernel of the split form on the same grid.  Under a
profiler the launch list then holds every kernel kind at full size; the
program checks only that every call succeeds and the fields stay finite.
"""
import numpy as np
import torch

import rapport_gb300 as R
from rapport_gb300 import _lib

W = dict(Nr=1024, Nt=2048, R_max=2e-3, w0=150e-6, T_half=800e-15, fwhm=100e-15, E=5.0, f=0.1, dz=2.5e-6)


def _setup(**over):
    cfg = R.workload_config(W["Nr"], W["Nt"], W["R_max"], W["w0"], W["T_half"], W["dz"], 2, **over)
    g = R.build_grids(cfg)
    u0 = R.envelope_lens(W["w0"], W["fwhm"], W["E"], W["f"], 0)(g["rr"], g["tt"], cfg, g)
    return cfg, g, np.ascontiguousarray(u0.astype(np.complex64))


def main():
    dev = torch.device("cuda", 0)
    cfg, g, u0 = _setup()
    ctx = _lib.Context(cfg, g)
    lin, nl = R.LinearOperator(cfg, g, ctx), R.NonlinearOperator(cfg, g, ctx)
    u = torch.from_numpy(u0).to(dev)
    rho = torch.zeros(u.shape, dtype=torch.float32, device=dev)
    rs = torch.zeros_like(rho)
    hl = lin.half_linear(u, W["dz"])                      # k_gemm_f32, k_fft_phase_ifft, k_phase_tables
    nl.update_plasma(hl, rho, rs)                          # k_rate_scan
    nl.split(hl, rho, rs)                                  # k_split
    nl.nonlinear_step(hl.clone(), rho, W["dz"])            # k_nonlinear_step
    rec = torch.zeros((W["Nr"], 6), dtype=torch.float64, device=dev)
    ctx.record(hl, rho, rs, None, 0, rec)                  # k_record
    for mode in (_lib.MODE_PLAIN_F32, _lib.MODE_SPLIT_BF16, _lib.MODE_SPLIT_F16):
        v = u.clone()
        ctx.step(v, rho, W["dz"], mode, rs)                # split forms: k_build_E, k_split_E*, k_row_*, k_gemm_tc
        ctx.propagate(v, torch.zeros_like(rho), torch.zeros_like(rho), W["dz"], 2, mode)
        assert bool(torch.isfinite(v).all())
    envs = [R.envelope_lens(W["w0"], W["fwhm"], W["E"], W["f"], i)(g["rr"], g["tt"], cfg, g) for i in range(8)]
    b = _lib.Batch([cfg] * 8, [g] * 8)
    bu = [torch.from_numpy(np.ascontiguousarray(e.astype(np.complex64))).to(dev) for e in envs]
    br = [torch.zeros(u.shape, dtype=torch.float32, device=dev) for _ in envs]
    for mode in (_lib.MODE_SPLIT_BF16, _lib.MODE_SPLIT_F16):
        b.set_mode(mode)
        b.propagate(bu, br, None, W["dz"], 2)              # k_gemm_tc_grouped, k_row_*_b, k_field_bound
    assert b.device_status() == 0 and all(bool(torch.isfinite(x).all()) for x in bu)
    # exciton channel: the two-population march
    cfg_s, g_s, _ = _setup(enable_ste=True, tau_ste=1e-12)
    cs = _lib.Context(cfg_s, g_s)
    r2, s2 = torch.zeros_like(rho), torch.zeros_like(rho)
    cs.update_plasma(u, r2, s2)                            # k_rate_scan (two populations)
    # full-physics split: Raman, self-steepening, space-time focusing
    cfg_f, g_f, _ = _setup(f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True,
                           enable_space_time_focusing=True)
    cf = _lib.Context(cfg_f, g_f)
    out = torch.empty_like(u)
    alpha = torch.empty_like(rho)
    cf.split(u, rho, out, alpha)                           # k_split_full
    v = u.clone()
    cf.nonlinear_step(v, rho, W["dz"])                     # k_nl_full
    cf.half_linear(v, W["dz"])                             # k_phase_table_2d, k_fft_phase_ifft (2-d phase)
    assert bool(torch.isfinite(v).all())
    # Raman + self-steepening in the split form: the fused full-physics row kernel
    cfg_r, g_r, _ = _setup(f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True)
    cr = _lib.Context(cfg_r, g_r)
    v = u.clone()
    cr.step(v, rho, W["dz"], _lib.MODE_SPLIT_BF16)         # k_row_nl_full
    assert bool(torch.isfinite(v).all())
    torch.cuda.synchronize()
    for c in (ctx, cs, cf, cr):
        assert c.device_status() == 0
    print("kernel tour done")


if __name__ == "__main__":
    main()
