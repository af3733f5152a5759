"""Long-run accuracy against FP64: the metric's "<= 1e-4 L2 field error after 1 cm".

* test_fp64_gpu_reference_is_pinned: the FP64 GPU restatement (oracle/fp64_gpu.py)
  reproduces the numpy oracle (which reproduces the reference bit for bit) to
  1e-11 over several steps -- only then is it used as the long-run reference.
* test_one_cm_accuracy (~3 min): the 1024 x 2048 workload propagated 4000
  z-steps of 2.5 um (1 cm) by the FP64 reference, the plain FP32 form, the
  split-BF16 form (3-term and 2-term operator) and the split-FP16 form.
  Reports the relative L2 field error, peak-fluence error and peak-rho error
  at 0.125, 0.25, 0.5 and 1 cm, writes them as JSON to the directory named by
  NLSE_REPORT_DIR (with the commit named by NLSE_COMMIT), and asserts the
  bounds L2 <= 1e-4 and peak-rho <= 1e-3 at every checkpoint for the tensor-
  core forms the library offers as precise (split-BF16 with the 3-term
  operator, split-FP16).
"""
import json
import os

import numpy as np
import pytest

import nlse_oracle as O
from conftest import rel_l2
from gpu_util import CONFIG2, Case, dev, host

pytestmark = pytest.mark.gpu


def test_fp64_gpu_reference_is_pinned():
    import fp64_gpu
    og = O.OracleGrid(O.workload_config(64, 256, 1e-4, 1e-5, 3e-13))
    u0 = O.lens_gaussian(og, 1e-5, 100e-15, 2.0, 1e-2, 0)
    ref_u, ref_rho, _ = og.propagate(u0.copy(), 5, 5e-6)
    g = fp64_gpu.FP64GPU(og)
    u, rho = g.propagate(u0, 5, 5e-6)
    assert rel_l2(u.cpu().numpy(), ref_u) < 1e-11
    assert np.abs(rho.cpu().numpy() - ref_rho).max() <= 1e-11 * ref_rho.max()


def test_fp64_gpu_space_time_focusing_is_pinned():
    """The FP64 GPU restatement with space-time focusing (the Omega-dependent
    diffraction phase and the U^-1 filter of split) against the numpy oracle."""
    import fp64_gpu
    og = O.OracleGrid(O.workload_config(64, 256, 1e-4, 1e-5, 3e-13, enable_space_time_focusing=True))
    u0 = O.lens_gaussian(og, 1e-5, 100e-15, 2.0, 1e-2, 0)
    ref_u, ref_rho, _ = og.propagate(u0.copy(), 5, 5e-6)
    u, rho = fp64_gpu.FP64GPU(og).propagate(u0, 5, 5e-6)
    assert rel_l2(u.cpu().numpy(), ref_u) < 1e-11
    assert np.abs(rho.cpu().numpy() - ref_rho).max() <= 1e-11 * ref_rho.max()


def _metrics(u, rho, uref, rref, dt, invE2):
    flu = (np.abs(u) ** 2).sum(axis=1) * dt * invE2
    flu_r = (np.abs(uref) ** 2).sum(axis=1) * dt * invE2
    return {"l2": rel_l2(u, uref), "peak_fluence": abs(flu.max() / flu_r.max() - 1),
            "peak_rho": abs(rho.max() / max(rref.max(), 1e-300) - 1) if rref.max() > 0 else 0.0,
            "peak_rho_value": float(rref.max())}


def test_one_cm_accuracy():
    import torch
    import fp64_gpu
    from rapport_gb300._lib import MODE_PLAIN_F32, MODE_SPLIT_BF16, MODE_SPLIT_F16

    c = Case(**CONFIG2)
    ref = fp64_gpu.FP64GPU(c.og)
    forms = {"split_bf16_3term": (MODE_SPLIT_BF16, 3), "split_bf16_2term": (MODE_SPLIT_BF16, 2),
             "split_f16": (MODE_SPLIT_F16, 3), "plain_fp32": (MODE_PLAIN_F32, 3)}
    state = {k: (dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))) for k in forms}
    ur = torch.tensor(c.u0, dtype=torch.complex128, device="cuda")
    rr = torch.zeros(c.u0.shape, dtype=torch.float64, device="cuda")
    report = {"workload": "1024x2048, 5 uJ, w0 150 um, f 10 cm, dz 2.5 um, 1% noise seed 0",
              "commit": os.environ.get("NLSE_COMMIT", "unknown"),
              "reference": "FP64 GPU restatement (oracle/fp64_gpu.py), same seeded input", "checkpoints": {}}
    done = 0
    for stop in (500, 1000, 2000, 4000):
        for _ in range(stop - done):
            ref.update_plasma(ur, rr)
            ur = ref.step(ur, rr, c.dz)
        for name, (mode, terms) in forms.items():
            c.ctx.set_split_terms(terms)
            u, rho, rs = state[name]
            c.ctx.propagate(u, rho, rs, c.dz, stop - done, mode)
        c.ctx.set_split_terms(3)
        done = stop
        urn, rrn = ur.cpu().numpy(), rr.cpu().numpy()
        entry = {}
        for name in forms:
            u, rho, _ = state[name]
            entry[name] = _metrics(host(u), host(rho), urn, rrn, c.og.dt, c.og.invE2)
        report["checkpoints"][f"{stop * c.dz * 100:.3f} cm"] = entry
        print(stop, json.dumps(entry), flush=True)
    assert c.ctx.device_status() == 0
    out = os.environ.get("NLSE_REPORT_DIR")
    if out:
        os.makedirs(out, exist_ok=True)
        with open(os.path.join(out, "accuracy_1cm_1024x2048.json"), "w") as f:
            json.dump(report, f, indent=1)
    for at, entry in report["checkpoints"].items():
        for name in ("split_bf16_3term", "split_f16"):
            m = entry[name]
            assert m["l2"] <= 1e-4 and m["peak_rho"] <= 1e-3, (at, name, m)


def test_space_time_focusing_half_cm_accuracy():
    """The 1024 x 2048 workload with space-time focusing on (the reference's
    default), 2000 z-steps (0.5 cm): the tensor-core sandwich Y P(rho, Omega) Y
    (scaled FP16 terms) and the plain FP32 form against the FP64 reference,
    with the bounds L2 <= 1e-4 and peak-rho <= 1e-3 at every checkpoint for the
    tensor-core form; written to NLSE_REPORT_DIR like the 1 cm report."""
    import torch
    import fp64_gpu
    from rapport_gb300._lib import MODE_PLAIN_F32, MODE_SPLIT_F16

    c = Case(**CONFIG2, enable_space_time_focusing=True)
    ref = fp64_gpu.FP64GPU(c.og)
    forms = {"split_stf_sandwich": MODE_SPLIT_F16, "plain_fp32": MODE_PLAIN_F32}
    state = {k: (dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))) for k in forms}
    ur = torch.tensor(c.u0, dtype=torch.complex128, device="cuda")
    rr = torch.zeros(c.u0.shape, dtype=torch.float64, device="cuda")
    report = {"workload": "1024x2048, 5 uJ, w0 150 um, f 10 cm, dz 2.5 um, 1% noise seed 0, space-time focusing",
              "commit": os.environ.get("NLSE_COMMIT", "unknown"),
              "reference": "FP64 GPU restatement (oracle/fp64_gpu.py), same seeded input", "checkpoints": {}}
    done = 0
    for stop in (500, 1000, 2000):
        for _ in range(stop - done):
            ref.update_plasma(ur, rr)
            ur = ref.step(ur, rr, c.dz)
        for name, mode in forms.items():
            u, rho, rs = state[name]
            c.ctx.propagate(u, rho, rs, c.dz, stop - done, mode)
        done = stop
        urn, rrn = ur.cpu().numpy(), rr.cpu().numpy()
        entry = {name: _metrics(host(state[name][0]), host(state[name][1]), urn, rrn, c.og.dt, c.og.invE2)
                 for name in forms}
        report["checkpoints"][f"{stop * c.dz * 100:.3f} cm"] = entry
        print(stop, json.dumps(entry), flush=True)
    assert c.ctx.device_status() == 0
    out = os.environ.get("NLSE_REPORT_DIR")
    if out:
        os.makedirs(out, exist_ok=True)
        with open(os.path.join(out, "accuracy_stf_halfcm_1024x2048.json"), "w") as f:
            json.dump(report, f, indent=1)
    for at, entry in report["checkpoints"].items():
        m = entry["split_stf_sandwich"]
        assert m["l2"] <= 1e-4 and m["peak_rho"] <= 1e-3, (at, m)


def test_all_physics_accuracy():
    """Every split() term on (Raman, self-steepening, space-time focusing, the
    exciton channel with a 1 ps decay), a 1 uJ pulse focused by a 1 mm lens on
    256 x 1024: 400 z-steps of 2.5 um (0.1 cm, through the focus) in the split-
    BF16 and split-FP16 forms against the FP64 numpy oracle (the reference's
    arithmetic), checkpoints every 100 steps.  Writes
    accuracy_all_physics_256x1024.json to NLSE_REPORT_DIR; asserts relative L2
    <= 1e-4 and peak-rho / peak-rho_s <= 1e-3 at every checkpoint."""
    from conftest import FULL_PHYSICS
    from rapport_gb300 import _lib
    dz, chunk, nchunk = 2.5e-6, 100, 4
    c = Case(256, 1024, 5e-4, 50e-6, 400e-15, 100e-15, 1.0, 1e-3, dz, chunk * nchunk, 0, **FULL_PHYSICS)
    og = c.og
    uo, ro, so = c.u0.copy(), np.zeros(c.u0.shape), np.zeros(c.u0.shape)
    ref = []
    for _ in range(nchunk):
        uo, ro, so = og.propagate(uo, chunk, dz, ro, so)
        ref.append((uo.copy(), ro.copy(), so.copy()))
    report = {"workload": "256x1024, 1 uJ, w0 50 um, f 1 mm, dz 2.5 um, every split() term, 1% noise seed 0",
              "commit": os.environ.get("NLSE_COMMIT", ""), "reference": "FP64 numpy oracle (oracle/nlse_oracle.py)",
              "checkpoints": {}}
    for name, mode in (("split_bf16", _lib.MODE_SPLIT_BF16), ("split_f16", _lib.MODE_SPLIT_F16)):
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        for j in range(nchunk):
            c.ctx.propagate(u, rho, rs, dz, chunk, mode)
            ur, rr, sr = ref[j]
            m = _metrics(host(u), host(rho), ur, rr, 1.0, 1.0)  # the fluence ratio needs no units
            m["peak_rho_s"] = abs(host(rs).max() / max(sr.max(), 1e-300) - 1) if sr.max() > 0 else 0.0
            report["checkpoints"].setdefault(f"{(j + 1) * chunk * dz * 100:.3f} cm", {})[name] = m
        assert c.ctx.device_status() == 0
    out = os.environ.get("NLSE_REPORT_DIR")
    if out:
        os.makedirs(out, exist_ok=True)
        with open(os.path.join(out, "accuracy_all_physics_256x1024.json"), "w") as f:
            json.dump(report, f, indent=1)
    for cp, forms in report["checkpoints"].items():
        for name, m in forms.items():
            assert m["l2"] <= 1e-4 and m["peak_rho"] <= 1e-3 and m["peak_rho_s"] <= 1e-3, (cp, name, m)
