"""Benchmark: z-steps/s of the split-step NLSE propagator on one GB300.

Workload (the measured grid): N_r = 1024 radial points (R_max = 2 mm),
N_t = 2048 time points (+-800 fs), 800 nm, 5 uJ, 100 fs FWHM, w0 = 150 um,
lens f = 10 cm, 1 % seeded noise (numpy default_rng(0)), fused silica with K=6
MPI (sigma_K = 1e-71), avalanche, recombination (150 fs), dz = 2.5 um.
Synthetic input of that shape; no dataset is involved.

One bench step = Z z-steps (update_plasma + step each, the reference's z-loop
iteration) advanced by one call of the C ABI (nlse_propagate); the metric is
z-steps/s.  Between timed steps the L2 is flushed (256 MB write) outside the
timed events; inside a step the field stays on-chip as in the reference's own
loop, whose host syncs happen only at _record.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the FP64 CPU restatement of the reference path (the
oracle: numpy complex128 + the C carrier march with OpenMP) on this host's
cores, one z-step per bench step; rank 0 only under torchrun.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "z-steps/s (1 GB300), split-BF16 batched vs plain FP32, at ≤1e-4 L2 err vs FP64"
WORKLOAD = dict(Nr=1024, Nt=2048, R_max=2e-3, w0=150e-6, T_half=800e-15, fwhm=100e-15, E=5.0, f=0.1,
                dz=2.5e-6, seed=0)
CONFIG = {"workload": "single pulse, N_r=1024 (R_max 2 mm) x N_t=2048 (+-800 fs), 5 uJ, 100 fs, w0 150 um, "
                      "f 10 cm, 1% noise seed 0, K=6 MPI + avalanche + recombination, dz 2.5 um",
          "Nr": 1024, "Nt": 2048, "dz_um": 2.5}


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), d.get("bf16_tflops_sustained", 1700.0), \
            "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


TRAFFIC_JSON = os.path.join(HERE, "profiles", "traffic_per_launch.json")


def measured_traffic(kernel, path=TRAFFIC_JSON):
    """DRAM bytes (read + write) per launch of a kernel from the ncu capture in
    profiles/traffic_per_launch.json, if that capture was taken of the kernel
    sources being run (same kernel fingerprint); else (None, why)."""
    from rapport_gb300.build import kernel_fingerprint
    if not os.path.exists(path):
        return None, "no capture"
    with open(path) as f:
        rec = json.load(f)
    ent = rec.get("kernels", {}).get(kernel)
    if ent is None:
        return None, f"no capture of {kernel}"
    fp = kernel_fingerprint()
    if ent.get("kernel_fingerprint") != fp:
        return None, f"capture of {kernel} is of other kernel sources ({ent.get('kernel_fingerprint')} != {fp})"
    return ent["bytes_per_launch"], f"ncu dram__bytes_read.sum + dram__bytes_write.sum, {ent['note']}"


def host_cores():
    """Host threads this process may run on, and the BLAS thread count numpy uses."""
    cores = len(os.sched_getaffinity(0))
    blas = None
    try:
        from threadpoolctl import threadpool_info
        blas = max((d.get("num_threads") or 0 for d in threadpool_info() if d.get("user_api") == "blas"),
                   default=None)
    except ImportError:
        v = os.environ.get("OPENBLAS_NUM_THREADS") or os.environ.get("OMP_NUM_THREADS")
        blas = int(v) if v else cores  # OpenBLAS default: one thread per available core
    return cores, blas


# ------------------------------------------------------------------ clocks
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "100", "-i", str(device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world, local_rank):
    import torch
    import rapport_gb300 as R
    from rapport_gb300 import _lib

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    w = dict(WORKLOAD, Nt=args.nt) if args.nt else WORKLOAD
    Z = args.zsteps
    if args.row_plans:
        _lib.set_row_plans(w["Nt"], *args.row_plans)
    cfg = R.workload_config(w["Nr"], w["Nt"], w["R_max"], w["w0"], w["T_half"], w["dz"], Z, **physics_over(args))
    g = R.build_grids(cfg)
    ctx = _lib.Context(cfg, g)
    u0 = R.envelope_lens(w["w0"], w["fwhm"], w["E"], w["f"], w["seed"])(g["rr"], g["tt"], cfg, g)
    u0 = np.ascontiguousarray(u0.astype(np.complex64))
    modes = {"plain": _lib.MODE_PLAIN_F32, "split_bf16": _lib.MODE_SPLIT_BF16, "split_f16": _lib.MODE_SPLIT_F16}
    want = ["split_bf16", "split_f16", "plain"] if args.mode == "auto" else [args.mode]

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    results = {}
    lead = None
    for name in want:
        mode = modes[name]
        u = torch.from_numpy(u0).to(dev)
        rho = torch.zeros(u.shape, dtype=torch.float32, device=dev)
        rs = torch.zeros_like(rho)
        try:
            ctx.propagate(u, rho, rs, w["dz"], 1, mode)
        except _lib.NLSEError as e:
            if args.mode != "auto":
                raise
            results[name] = {"unavailable": str(e)}
            continue
        lead = lead or name
        K = args.steps if name == lead else max(2, args.steps // 4)
        for _ in range(args.warmup):
            ctx.propagate(u, rho, rs, w["dz"], Z, mode)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        clk = ClockSampler(local_rank) if name == lead else None
        barrier()
        torch.cuda.synchronize()
        for i in range(K):
            flush.fill_(float(i))
            ev[i][0].record()
            ctx.propagate(u, rho, rs, w["dz"], Z, mode)
            ev[i][1].record()
        torch.cuda.synchronize()
        barrier()
        clocks = clk.stop() if clk else None
        # second, identical pass with per-launch events on the launching stream
        # (kept out of the timed pass: recording them costs a few percent)
        ctx.profile_start(K * Z * 16 + 64)
        for i in range(K):
            flush.fill_(float(i))
            ctx.propagate(u, rho, rs, w["dz"], Z, mode)
        prof = ctx.profile_read()
        t_ms = sum(a.elapsed_time(b) for a, b in ev)
        if world > 1:
            import torch.distributed as dist
            tt = torch.tensor([t_ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            t_ms = float(tt.item())
        results[name] = dict(K=K, t_ms=t_ms, zsteps_per_s=world * K * Z / (t_ms * 1e-3), prof=prof,
                             clocks=clocks, finite=bool(torch.isfinite(u).all().item()))
    head = next(n for n in want if "t_ms" in results.get(n, {}))
    r = results[head]
    mode = modes[head]

    # ---------------------------------------------------------- headline: the batched split-BF16 form
    # B pulses of the same 1024 x 2048 grid (seeds 0..B-1) advanced together:
    # one grouped tensor-core launch per half step over all their tiles.
    hbm, bf16, bf16_s, src = peaks()
    Nr, Nt = w["Nr"], w["Nt"]
    B = args.batch if head in ("split_bf16", "split_f16") else 0
    bmode = args.batch_mode if args.mode == "auto" else head
    other_batched = {}
    fallback = {"single_pulse": int(ctx.scan_fallback_rows())}
    batch_variant = None
    if B > 0:
        envs = [np.ascontiguousarray(R.envelope_lens(w["w0"], w["fwhm"], w["E"], w["f"], w["seed"] + i)(
            g["rr"], g["tt"], cfg, g).astype(np.complex64)) for i in range(B)]
        bt = _lib.Batch([cfg] * B, [g] * B)
        bt.set_mode(modes[bmode])
        bu = [torch.from_numpy(e).to(dev) for e in envs]
        br = [torch.zeros(u0.shape, dtype=torch.float32, device=dev) for _ in range(B)]
        # the exciton density, where the channel is on (the batch then requires it)
        bs = [torch.zeros(u0.shape, dtype=torch.float32, device=dev) for _ in range(B)] if cfg.enable_ste else None
        bt.propagate(bu, br, bs, w["dz"], 1)
        for _ in range(args.warmup):
            bt.propagate(bu, br, bs, w["dz"], Z)
        torch.cuda.synchronize()
        K = args.steps
        bev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        clk = ClockSampler(local_rank)
        barrier()
        torch.cuda.synchronize()
        for i in range(K):
            flush.fill_(float(i))
            bev[i][0].record()
            bt.propagate(bu, br, bs, w["dz"], Z)
            bev[i][1].record()
        torch.cuda.synchronize()
        barrier()
        clocks = clk.stop()
        t_ms = sum(a.elapsed_time(b_) for a, b_ in bev)
        if world > 1:
            import torch.distributed as dist
            tt = torch.tensor([t_ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            t_ms = float(tt.item())
        value = world * B * K * Z / (t_ms * 1e-3)
        pctx = bt.context_profile()
        pctx.profile_start(K * Z * 16 + 64)
        for i in range(K):
            flush.fill_(float(i))
            bt.propagate(bu, br, bs, w["dz"], Z)
        prof = pctx.profile_read()
        assert bt.device_status() == 0 and all(bool(torch.isfinite(x).all().item()) for x in bu)
        batch_variant = bt.context(0).gemm_variant()  # the batch's own tuner pick (grouped launch)
        # e2e through the C ABI with host buffers: every step copies each pulse's field in from
        # pinned memory and its field + densities back out.  Two device (and host) buffer sets
        # alternate, so step i's read-back (own stream) overlaps step i + 1's upload (own stream)
        # and compute, as a caller streaming batches would run it; every copy of the K steps is
        # inside the one timed region.  The batch's working set (~0.6 GB) exceeds the L2.
        uh = [torch.from_numpy(e).pin_memory() for e in envs]
        dsets = [(bu, br, bs), ([torch.empty_like(x) for x in bu], [torch.empty_like(x) for x in br],
                                [torch.zeros_like(x) for x in bs] if bs else None)]
        nd = 2 if bs else 1  # densities read back per pulse: rho (and rho_s)
        hsets = [([torch.empty_like(x).pin_memory() for x in uh],
                  [torch.empty(u0.shape, dtype=torch.float32).pin_memory() for _ in range(nd * B)]) for _ in range(2)]
        main = torch.cuda.current_stream()
        s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
        ev_in = [torch.cuda.Event() for _ in range(2)]
        ev_done = [torch.cuda.Event() for _ in range(2)]
        ev_out = [torch.cuda.Event() for _ in range(2)]

        def e2e_step(i):
            k = i % 2
            du, dr, ds = dsets[k]
            ho, hr = hsets[k]
            with torch.cuda.stream(s_in):
                if i >= 2:
                    s_in.wait_event(ev_out[k])   # set k's previous read-back is done
                for j in range(B):
                    du[j].copy_(uh[j], non_blocking=True)
                ev_in[k].record(s_in)
            main.wait_event(ev_in[k])
            bt.propagate(du, dr, ds, w["dz"], Z)
            ev_done[k].record(main)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_done[k])
                for j in range(B):
                    ho[j].copy_(du[j], non_blocking=True)
                    hr[j].copy_(dr[j], non_blocking=True)
                    if ds:
                        hr[B + j].copy_(ds[j], non_blocking=True)
                ev_out[k].record(s_out)

        for i in range(2):                     # untimed: both buffer sets once
            e2e_step(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(main)
        for i in range(K):
            e2e_step(i)
        main.wait_stream(s_out)
        e1.record(main)
        torch.cuda.synchronize()
        e_ms = e0.elapsed_time(e1)
        assert all(np.isfinite(x.numpy()).all() for hs in hsets for x in hs[0])
        e2e = {"value": world * B * K * Z / (e_ms * 1e-3), "unit": "z-steps/s",
               "h2d_bytes_per_step": int(sum(x.numel() * 8 for x in uh)),
               "d2h_bytes_per_step": int(sum(x.numel() * 8 for x in hsets[0][0]) +
                                         sum(x.numel() * 4 for x in hsets[0][1])),
               "overlap": "double-buffered: step i's read-back overlaps step i+1's upload and compute"}
        del dsets[1]
        # rows whose carrier march fell back to the one-thread sequential form (a
        # diagnostic: the Newton scan should solve every row of these workloads)
        fallback["batched"] = int(sum(bt.context(i).scan_fallback_rows() for i in range(B)))
        # the other tensor-core form on the same batch, for the forms table
        for oname in [m for m in ("split_bf16", "split_f16") if m != bmode and args.mode == "auto"]:
            bt.set_mode(modes[oname])
            bt.propagate(bu, br, bs, w["dz"], Z)
            K2 = max(2, K // 2)
            oev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K2)]
            torch.cuda.synchronize()
            for i in range(K2):
                flush.fill_(float(i))
                oev[i][0].record()
                bt.propagate(bu, br, bs, w["dz"], Z)
                oev[i][1].record()
            torch.cuda.synchronize()
            assert bt.device_status() == 0
            o_ms = sum(a.elapsed_time(b_) for a, b_ in oev)
            other_batched[oname + "_batched"] = round(world * B * K2 * Z / (o_ms * 1e-3), 1)
        del bt, bu, br
        gemm_flops = B * 8.0 * Nr * Nr * Nt          # one grouped launch, algorithmic
        form = f"{bmode} batched ({B} pulses of {Nr}x{Nt})"
        ms_per_step = t_ms / K
    else:
        # single-pulse form only (split-BF16 unavailable): e2e through the single-context call
        value, prof, clocks, K = r["zsteps_per_s"], r["prof"], r["clocks"], r["K"]
        uh = torch.from_numpy(u0).pin_memory()
        uo = torch.empty_like(uh).pin_memory()
        rho_h = torch.empty(u0.shape, dtype=torch.float32).pin_memory()
        ud = torch.empty(u0.shape, dtype=torch.complex64, device=dev)
        rd = torch.zeros(u0.shape, dtype=torch.float32, device=dev)
        sd = torch.zeros_like(rd)
        e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        for i in range(K + 1):
            flush.fill_(float(i))
            if i > 0:
                e_ev[i - 1][0].record()
            ud.copy_(uh, non_blocking=True)
            ctx.propagate(ud, rd, sd, w["dz"], Z, mode)
            uo.copy_(ud, non_blocking=True)
            rho_h.copy_(rd, non_blocking=True)
            if i > 0:
                e_ev[i - 1][1].record()
        torch.cuda.synchronize()
        e_ms = sum(a.elapsed_time(b) for a, b in e_ev)
        e2e = {"value": world * K * Z / (e_ms * 1e-3), "unit": "z-steps/s",
               "h2d_bytes_per_step": int(uh.numel() * 8),
               "d2h_bytes_per_step": int(uo.numel() * 8 + rho_h.numel() * 4)}
        gemm_flops = (8.0 if head.startswith("split") else 4.0) * Nr * Nr * Nt
        form = head
        bmode = head
        ms_per_step = r["t_ms"] / r["K"]

    # ---------------------------------------------------------- roofline of the dominant kernel
    top = max(prof, key=lambda k: prof[k][1])
    n_launch, tot = prof[top]
    avg_s = tot / n_launch * 1e-3
    traffic, traffic_note = measured_traffic(top + ("_batched" if B > 0 else ""))
    if top in ("k_gemm_tc", "k_gemm_f32"):
        ach = gemm_flops / avg_s / 1e12
        roof = {"kernel": top, "bound": "tensor", "achieved": ach, "peak": bf16_s, "unit": "TFLOP/s",
                "frac": ach / bf16_s, "traffic": traffic, "peak_source": f"bf16_tflops_sustained ({src})",
                "per_launch": f"{gemm_flops:.3e} algorithmic FLOPs, avg {avg_s * 1e6:.1f} us over {n_launch} launches",
                "executed_tensor_tflops": (3 if bmode == "split_f16" else 4) * ach if top == "k_gemm_tc" else None,
                "traffic_source": traffic_note}
    else:
        npts = (B if B > 0 else 1) * Nr * Nt
        byts = {"k_row_nl": 36.0, "k_row_next": 36.0, "k_rate_scan": 12.0, "k_nonlinear_step": 20.0,
                "k_fft_phase_ifft": 16.0}.get(top, 16.0) * npts
        ach = byts / avg_s / 1e9
        roof = {"kernel": top, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": traffic, "traffic_source": traffic_note, "peak_source": f"hbm_gbs ({src})",
                "per_launch": f"{byts:.3e} algorithmic bytes, avg {avg_s * 1e6:.1f} us over {n_launch} launches"}

    line = {
        "metric": METRIC, "value": value, "unit": "z-steps/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"split_bf16": "bf16x3-split + f32", "split_f16": "f16x2-split + f32"}.get(bmode, "f32"),
        "data": "synthetic (seeded lens-focused Gaussian pulses with 1% noise)",
        "config": dict(CONFIG, Nt=w["Nt"], workload=CONFIG["workload"].replace("N_t=2048", f"N_t={w['Nt']}"),
                       form=form, pulses=max(B, 1), z_steps_per_step=Z, parallelism=f"replicas{world}",
                       space_time_focusing=bool(args.space_time_focusing or args.all_physics),
                       physics=physics_name(args),
                       l2="256 MB flush before each timed step (outside its events); per pulse 24 MB",
                       kernel_times="second identical pass of K steps with per-launch events"),
        "roofline": roof, "e2e": e2e, "gpu_launches": int(sum(v[0] for v in prof.values())),
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()},
        "scan_fallback_rows": fallback,
        "autotuned": {"gemm_variant": ctx.gemm_variant(), "batch_gemm_variant": batch_variant,
                      "row_plans": dict(zip(("row_nl", "row_next"), _lib.row_plans(Nt)))},
        "clocks": clocks,
        "forms": dict({k + "_single_pulse": (round(v["zsteps_per_s"], 1) if "zsteps_per_s" in v else v)
                       for k, v in results.items()},
                      **({bmode + "_batched": round(value, 1)} if B > 0 else {}), **other_batched),
        "speedup_vs_plain_fp32": (value / results["plain"]["zsteps_per_s"])
        if "zsteps_per_s" in results.get("plain", {}) else None,
    }
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_zsteps, args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ------------------------------------------------------------------ 64 pulses on mixed grids
def mixed_pulses(n=64, seed=1):
    """The batch workload: rng = default_rng(seed); per-parameter draws in this
    order -- N_r in {512, 768, 1024}, N_t in {1024, 2048, 4096} (uniform),
    energy log-uniform 1-20 uJ, FWHM uniform 50-200 fs, w0 uniform 80-200 um,
    f uniform 5-20 cm -- then each pulse's noise.  R_max = 10 w0 and a +-4 FWHM
    window (the ratios of the 256 x 512 CPU case); dz = 5 um."""
    rng = np.random.default_rng(seed)
    Nr = rng.choice([512, 768, 1024], n)
    Nt = rng.choice([1024, 2048, 4096], n)
    E = np.exp(rng.uniform(np.log(1.0), np.log(20.0), n))
    fwhm = rng.uniform(50e-15, 200e-15, n)
    w0 = rng.uniform(80e-6, 200e-6, n)
    f = rng.uniform(0.05, 0.20, n)
    return [dict(Nr=int(Nr[i]), Nt=int(Nt[i]), E=float(E[i]), fwhm=float(fwhm[i]), w0=float(w0[i]), f=float(f[i]),
                 R_max=10 * float(w0[i]), T_half=4 * float(fwhm[i]), dz=5e-6, noise_seed=int(rng.integers(1 << 31)))
            for i in range(n)]


def run_mixed(args, rank, world, local_rank):
    import torch
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    from rapport_gb300.replicas import pulse_cost, shard_pulses
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    pulses = mixed_pulses()
    mine = shard_pulses([pulse_cost(p["Nr"], p["Nt"]) for p in pulses], world, rank)
    cfgs, grids, us, rhos = [], [], [], []
    for i in mine:
        p = pulses[i]
        cfg = R.workload_config(p["Nr"], p["Nt"], p["R_max"], p["w0"], p["T_half"], p["dz"], 2000)
        g = R.build_grids(cfg)
        u0 = R.envelope_lens(p["w0"], p["fwhm"], p["E"], p["f"], p["noise_seed"])(g["rr"], g["tt"], cfg, g)
        cfgs.append(cfg)
        grids.append(g)
        us.append(torch.from_numpy(np.ascontiguousarray(u0.astype(np.complex64))).to(dev))
        rhos.append(torch.zeros(u0.shape, dtype=torch.float32, device=dev))
    bt = _lib.Batch(cfgs, grids)
    Z = args.zsteps
    for _ in range(args.warmup):
        bt.propagate(us, rhos, None, 5e-6, Z)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local_rank) if rank == 0 else None
    for i in range(args.steps):
        flush.fill_(float(i))
        ev[i][0].record()
        bt.propagate(us, rhos, None, 5e-6, Z)
        ev[i][1].record()
    torch.cuda.synchronize()
    clocks = clk.stop() if clk else None
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    prof_ctx = bt.context_profile()
    prof_ctx.profile_start(args.steps * Z * 64 + 64)
    for i in range(args.steps):
        bt.propagate(us, rhos, None, 5e-6, Z)
    prof = prof_ctx.profile_read()
    ok = bt.device_status() == 0 and all(bool(torch.isfinite(u).all().item()) for u in us)
    flops = sum(8.0 * pulses[i]["Nr"] ** 2 * pulses[i]["Nt"] for i in range(len(pulses)))
    line = {
        "metric": "pulse-z-steps/s (1 GB300), split-BF16 batched, 64 mixed pulses", "value":
            len(pulses) * args.steps * Z / (t_ms * 1e-3), "unit": "pulse-z-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "dtype": "bf16x3-split + f32", "data": "synthetic (the 64-pulse draws, default_rng(1))",
        "config": {"workload": "64 pulses, N_r in {512,768,1024} x N_t in {1024,2048,4096}, 1-20 uJ, 50-200 fs, "
                               "w0 80-200 um, f 5-20 cm, dz 5 um", "z_steps_per_step": Z,
                   "grids": sorted({(p["Nr"], p["Nt"]) for p in pulses}), "parallelism": f"replicas{world}"},
        "tensor_tflops_algorithmic": 2 * flops * args.steps * Z / (sum(v[1] for k, v in prof.items()
                                                                     if k == "k_gemm_tc") * 1e-3) / 1e12,
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()},
        "finite": ok,
        "row_plans": {str(nt): dict(zip(("row_nl", "row_next"), _lib.row_plans(nt)))
                      for nt in sorted({pulses[i]["Nt"] for i in mine})},
        "gemm_variant": bt.context(0).gemm_variant(),
        "launches_per_z_step": "2 grouped products + 2 row launches per N_t class (one per half step)",
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def physics_over(args):
    """Config overrides of the physics options: none (the measured workload),
    space-time focusing, or every term the reference's Config enables by default."""
    if getattr(args, "all_physics", False):
        return dict(f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True,
                    enable_space_time_focusing=True, enable_ste=True, enable_ste_index=True)
    if args.space_time_focusing:
        return dict(enable_space_time_focusing=True)
    return {}


def physics_name(args):
    if getattr(args, "all_physics", False):
        return "Raman + self-steepening + space-time focusing + exciton channel (the reference's defaults)"
    return "space-time focusing" if args.space_time_focusing else "Kerr, MPI + avalanche + recombination"


# ------------------------------------------------------------------ CPU (oracle) arm
def _oracle_setup(args):
    """The oracle on the GPU arm's workload: the same grid (N_t from --nt), pulse and physics terms."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import nlse_oracle as O
    w = dict(WORKLOAD, Nt=args.nt) if args.nt else WORKLOAD
    og = O.OracleGrid(O.workload_config(w["Nr"], w["Nt"], w["R_max"], w["w0"], w["T_half"], **physics_over(args)))
    u = O.lens_gaussian(og, w["w0"], w["fwhm"], w["E"], w["f"], w["seed"])
    return og, u, w


def cpu_baseline(nz, args):
    og, u, w = _oracle_setup(args)
    rho = np.zeros(u.shape)
    rs = np.zeros(u.shape)
    og.update_plasma(u, rho, rs)
    t = time.perf_counter()
    for _ in range(nz):
        og.update_plasma(u, rho, rs)
        u = og.step(u, rho, rs, WORKLOAD["dz"])
    dt = time.perf_counter() - t
    cores, blas = host_cores()
    return {"value": nz / dt, "unit": "z-steps/s", "cores": cores, "blas_threads": blas, "kind": "port",
            "sample": f"{nz} z-steps of the {w['Nr']}x{w['Nt']} workload (FP64 numpy/OpenBLAS + C carrier march, "
                      f"OpenMP over r; physics: {physics_name(args)})",
            "what": "the oracle: an FP64 restatement of the reference path, pinned to the reference's own "
                    "outputs bit for bit or to 1e-12 (the reference itself needs CuPy and a GPU)"}


def run_reference(args, rank):
    if rank != 0:
        return
    og, u, w = _oracle_setup(args)
    rho = np.zeros(u.shape)
    rs = np.zeros(u.shape)
    for _ in range(args.warmup):
        og.update_plasma(u, rho, rs)
        u = og.step(u, rho, rs, WORKLOAD["dz"])
    t = time.perf_counter()
    for _ in range(args.steps):
        og.update_plasma(u, rho, rs)
        u = og.step(u, rho, rs, WORKLOAD["dz"])
    dt = time.perf_counter() - t
    v = args.steps / dt
    cores, blas = host_cores()
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": "z-steps/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (complex128)", "data": "synthetic",
        "config": dict(CONFIG, Nt=w["Nt"], workload=CONFIG["workload"].replace("N_t=2048", f"N_t={w['Nt']}"),
                       physics=physics_name(args), form="reference CPU path (FP64 restatement)", z_steps_per_step=1),
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "z-steps/s", "cores": cores, "blas_threads": blas, "kind": "port",
                         "sample": f"{args.steps} z-steps of the {w['Nr']}x{w['Nt']} workload ({physics_name(args)})"},
        "e2e": {"value": v, "unit": "z-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ------------------------------------------------------------------ one large pulse (2048 x 8192)
LARGE_PULSE = dict(Nr=2048, Nt=8192, R_max=3e-3, w0=200e-6, T_half=1.5e-12, fwhm=80e-15, E=20.0, f=0.15, dz=1.25e-6,
               seed=0)
# algorithmic bytes per point of the row / elementwise kernels, FLOPs per launch of the products
ROW_BYTES = {"k_row_nl": 36.0, "k_row_next": 36.0, "k_row_entry": 28.0, "k_fft_phase_ifft": 16.0,
             "k_nonlinear_step": 20.0, "k_rate_scan": 12.0, "k_split": 24.0}


def run_large(args, rank, world, local_rank):
    """One 2048 x 8192 pulse (20 uJ, 80 fs, w0 200 um, f 15 cm, dz 1.25 um): z-steps/s of each
    arithmetic and the roofline fraction of every kernel (per-launch CUDA events)."""
    import torch
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    lp = LARGE_PULSE
    Z = args.zsteps
    cfg = R.workload_config(lp["Nr"], lp["Nt"], lp["R_max"], lp["w0"], lp["T_half"], lp["dz"], Z)
    g = R.build_grids(cfg)
    ctx = _lib.Context(cfg, g)
    u0 = R.envelope_lens(lp["w0"], lp["fwhm"], lp["E"], lp["f"], lp["seed"])(g["rr"], g["tt"], cfg, g)
    u0 = np.ascontiguousarray(u0.astype(np.complex64))
    hbm, bf16, bf16_s, src = peaks()
    Nr, Nt = lp["Nr"], lp["Nt"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    modes = [("split_bf16", _lib.MODE_SPLIT_BF16), ("split_f16", _lib.MODE_SPLIT_F16), ("plain", _lib.MODE_PLAIN_F32)]
    forms, kernels, clocks = {}, {}, None
    for name, mode in modes:
        u = torch.from_numpy(u0).to(dev)
        rho = torch.zeros(u.shape, dtype=torch.float32, device=dev)
        rs = torch.zeros_like(rho)
        K = args.steps if name != "plain" else max(2, args.steps // 3)
        for _ in range(args.warmup):
            ctx.propagate(u, rho, rs, lp["dz"], Z, mode)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        clk = ClockSampler(local_rank) if name == "split_bf16" else None
        for i in range(K):
            flush.fill_(float(i))
            ev[i][0].record()
            ctx.propagate(u, rho, rs, lp["dz"], Z, mode)
            ev[i][1].record()
        torch.cuda.synchronize()
        if clk:
            clocks = clk.stop()
        t_ms = sum(a.elapsed_time(b) for a, b in ev)
        forms[name] = round(K * Z / (t_ms * 1e-3), 2)
        ctx.profile_start(K * Z * 16 + 64)
        for i in range(K):
            flush.fill_(float(i))
            ctx.propagate(u, rho, rs, lp["dz"], Z, mode)
        prof = ctx.profile_read()
        assert ctx.device_status() == 0 and bool(torch.isfinite(u).all().item())
        per = {}
        for k, (n, ms) in prof.items():
            avg_s = ms / n * 1e-3
            e = {"launches": n, "avg_us": round(avg_s * 1e6, 1), "share": round(ms / sum(v[1] for v in
                                                                                         prof.values()), 3)}
            if k == "k_gemm_tc":
                ach = 8.0 * Nr * Nr * Nt / avg_s / 1e12
                e.update(bound="tensor", achieved_tflops=round(ach, 1), frac=round(ach / bf16_s, 3),
                         executed_tflops=round((3 if name == "split_f16" else 4) * ach, 1))
            elif k == "k_gemm_f32":
                e.update(bound="fp32 SIMT", achieved_tflops=round(4.0 * Nr * Nr * Nt / avg_s / 1e12, 1))
            elif k in ROW_BYTES:
                ach = ROW_BYTES[k] * Nr * Nt / avg_s / 1e9
                e.update(bound="hbm", achieved_gbs=round(ach, 1), frac=round(ach / hbm, 3))
            per[k] = e
        kernels[name] = per
        del u, rho, rs
    line = {
        "metric": "z-steps/s (1 GB300), one 2048x8192 pulse", "value": forms["split_bf16"],
        "unit": "z-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "dtype": "bf16x3-split + f32", "data": "synthetic (seeded lens-focused Gaussian, 1% noise)",
        "config": {"workload": "single pulse, N_r=2048 (R_max 3 mm) x N_t=8192 (+-1.5 ps), 20 uJ, 80 fs, w0 200 um, "
                               "f 15 cm, 1% noise seed 0, K=6 MPI + avalanche + recombination, dz 1.25 um",
                   "z_steps_per_step": Z, "l2": "256 MB flush before each timed step; field 134 MB"},
        "forms": forms, "speedup_vs_plain_fp32": forms["split_bf16"] / forms["plain"],
        "peaks": {"hbm_gbs": hbm, "bf16_tflops_sustained": bf16_s, "source": src},
        "kernels": kernels, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_tour(args, rank, world, local_rank):
    """Every kernel of libnlse once at the 1024 x 2048 workload, for profiling: the
    plain half step, split(), the nonlinear block, update_plasma, a z-step and
    a 2-step propagate in each arithmetic, a 2-step propagate of 8 pulses in one
    batch (both split forms), the record reductions, the exciton-channel
    march, the full-physics split / nonlinear block (Raman, self-steepening,
    space-time focusing) and the fused full-physics row kernel of the split
    form.  Under ncu the launch list then holds every kernel kind at full size;
    the run checks only that every call succeeds and the fields stay finite."""
    import torch
    import rapport_gb300 as R
    from rapport_gb300 import _lib
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    W = WORKLOAD

    def _setup(**over):
        cfg = R.workload_config(W["Nr"], W["Nt"], W["R_max"], W["w0"], W["T_half"], W["dz"], 2, **over)
        g = R.build_grids(cfg)
        u0 = R.envelope_lens(W["w0"], W["fwhm"], W["E"], W["f"], 0)(g["rr"], g["tt"], cfg, g)
        return cfg, g, np.ascontiguousarray(u0.astype(np.complex64))

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


def record_traffic(csv_path, out_path=TRAFFIC_JSON):
    """Write profiles/traffic_per_launch.json from an ncu CSV of
    gpu__time_duration.sum, dram__bytes_read.sum and dram__bytes_write.sum
    (one row per launch and metric), stamped with the kernel fingerprint of the
    sources in this tree: per kernel kind, the mean DRAM bytes per launch."""
    import csv
    from rapport_gb300.build import kernel_fingerprint
    kinds = {"k_gemm_tc_grouped": "k_gemm_tc_batched", "k_row_nl_b": "k_row_nl_batched",
             "k_row_next_b": "k_row_next_batched", "k_gemm_tc": "k_gemm_tc", "k_row_nl": "k_row_nl",
             "k_row_next": "k_row_next"}
    lines = open(csv_path).read().splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.startswith('"ID"'))
    per = {}
    for row in csv.DictReader(lines[start:]):
        name = row["Kernel Name"].split("(")[0].split("<")[0].replace("void ", "").strip()
        if name not in kinds:
            continue
        v = float(row["Metric Value"].replace(",", ""))
        unit = row.get("Metric Unit", "")
        scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9}.get(unit, 1)
        ent = per.setdefault((kinds[name], row["ID"]), {})
        ent[row["Metric Name"]] = v * scale
    out = {}
    for (kind, _), m in per.items():
        if "dram__bytes_read.sum" in m and "dram__bytes_write.sum" in m:
            out.setdefault(kind, []).append(m["dram__bytes_read.sum"] + m["dram__bytes_write.sum"])
    fp = kernel_fingerprint()
    rec = {"_what": "DRAM bytes read + written per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum), "
                    "mean over the captured launches; valid for the kernel sources with this fingerprint",
           "kernels": {k: {"bytes_per_launch": int(sum(v) / len(v)), "launches": len(v), "kernel_fingerprint": fp,
                           "note": f"mean of {len(v)} launches, capture {os.path.basename(csv_path)}"}
                       for k, v in sorted(out.items())}}
    with open(out_path, "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec, indent=1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="auto", choices=["auto", "plain", "split_bf16", "split_f16"])
    ap.add_argument("--batch-mode", default="split_bf16", choices=["split_bf16", "split_f16"],
                    help="tensor-core form of the batched headline (auto mode)")
    ap.add_argument("--zsteps", type=int, default=50, help="z-steps per bench step")
    ap.add_argument("--cpu-zsteps", type=int, default=2, help="z-steps timed for cpu_baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch", type=int, default=8, help="pulses of the batched (headline) form; 0 = single pulse")
    ap.add_argument("--row-plans", type=int, nargs=2, metavar=("NL", "NEXT"),
                    help="pin the row kernels' plans for the single / batched workload's N_t instead of tuning "
                         "them (for profiling: under ncu the tuner's timings are meaningless)")
    ap.add_argument("--nt", type=int, default=0,
                    help="time points of the single / batched workload instead of 2048 (same +-800 fs window); "
                         "4096 is the reference Config's default")
    ap.add_argument("--space-time-focusing", action="store_true",
                    help="the single / batched workload with space-time focusing on (the reference's default): "
                         "the tensor-core forms run the correction Y (P - 1) Y")
    ap.add_argument("--all-physics", action="store_true",
                    help="the single / batched workload with every term the reference's Config turns on by "
                         "default: Raman (f_R 0.18), self-steepening, space-time focusing, the exciton channel "
                         "and its index term (the measured workload's rate table and grid otherwise)")
    ap.add_argument("--workload", default="single", choices=["single", "mixed64", "large", "tour"],
                    help="mixed64: 64 pulses on mixed grids (N_r 512-1024, N_t 1024-4096) in one batch; "
                         "large: one 2048 x 8192 pulse, every kernel's roofline; "
                         "tour: every kernel once at 1024 x 2048 (for ncu launch lists)")
    ap.add_argument("--record-traffic", metavar="CSV",
                    help="write profiles/traffic_per_launch.json from an ncu CSV and exit")
    args = ap.parse_args()
    if args.record_traffic:
        record_traffic(args.record_traffic)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "mixed64":
        run_mixed(args, rank, world, local_rank)
        return
    if args.workload == "large":
        run_large(args, rank, world, local_rank)
        return
    if args.workload == "tour":
        run_tour(args, rank, world, local_rank)
        return
    run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
