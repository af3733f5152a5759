"""Scenario sweeps: the term-ablation study and the energy sweeps of the
reference notebooks (``notebooks/term_ablation_study.ipynb`` cells 2, 19, 36,
37, 45; ``filament_1030nm_5uJ.ipynb``) as one batched caller.

A scenario is a name and the keyword overrides of ``run()`` on top of shared
base parameters.  ``run_scenarios`` runs every scenario whose ``result.npz`` is
not already cached (with the current code fingerprint) concurrently on one GPU:

* scenarios that the batched tensor-core form accepts (a split linear mode --
  "auto" resolves to split-BF16 -- up to 8192 radial points, no space-time
  focusing) and that share dz, nz, save_stride and that form advance together
  in one ``nlse_batch`` -- one grouped GEMM and one row launch per time-grid
  class per half step for all of them;
* every other scenario runs on its own context and CUDA stream;

and all of them are advanced one save interval at a time, round robin, so the
kernels of different scenarios overlap on the GPU.  Each scenario's record
planes, ``result.npz`` and ``params.json`` are exactly those of
``run(out_dir=..., **params)``.
"""
import json
import os
from pathlib import Path

import numpy as np
import torch

from ._lib import MODE_SPLIT_F16, Batch
from .config import batch_supported, resolved_linear_mode
from .filament_sim import FIELD_TOGGLES, run_config
from .grids import build_grids
from .integrator import Integrator, code_fingerprint


def build_scenarios(toggles=FIELD_TOGGLES):
    """The ablation set: everything on, each field term off in turn, and every
    field term off ("linear_only")."""
    sc = {"full": {}}
    for f in toggles:
        sc[f"no_{f.replace('enable_', '')}"] = {f: False}
    sc["linear_only"] = {f: False for f in toggles}
    return sc


def energy_scenarios(energies_uJ, prefix="sweep"):
    """One scenario per pulse energy: name f"{prefix}_{E:g}uJ"."""
    return {f"{prefix}_{e:g}uJ": {"energy_uJ": float(e)} for e in energies_uJ}


def load_scenario_npz(out_dir, ignore_stale=False):
    """A cached result.npz as a dict, or None when absent, unreadable or made
    by other code (params.json's code_fingerprint differs; ignore_stale=True
    reads it anyway)."""
    npz = Path(out_dir) / "result.npz"
    if not npz.exists():
        return None
    pj = Path(out_dir) / "params.json"
    if not ignore_stale and pj.exists():
        try:
            old = json.loads(pj.read_text()).get("code_fingerprint")
        except (OSError, ValueError):
            old = None
        if old != code_fingerprint():
            return None
    try:
        return dict(np.load(npz, allow_pickle=True))
    except Exception:  # a truncated file from an interrupted write: recompute
        return None


def summarize(results):
    """Per scenario: peak intensity, its z (um) and the on-axis peak electron density."""
    rows = []
    for name, res in results.items():
        Imax = np.asarray(res["Imax_z"])
        r = np.asarray(res["r"])
        i_axis = int(np.argmin(np.abs(r)))
        k = int(np.argmax(Imax))
        rows.append(dict(scenario=name, I_peak_Wcm2=float(Imax[k]), z_at_Ipeak_um=float(np.asarray(res["z"])[k] * 1e6),
                         rho_e_onaxis_max_cm3=float(np.asarray(res["rho_rz"])[:, i_axis].max())))
    return rows


def _batchable(cfg):
    # a batch takes the Raman / self-steepening terms and the exciton channel;
    # space-time focusing has no single radial operator (plain mode, own context)
    return resolved_linear_mode(cfg) in ("split_bf16", "split_f16") and batch_supported(cfg)


class _Group:
    """Scenarios advanced by one stepper on one stream: a single context, or a batch."""

    def __init__(self, names, integs, batch=None):
        self.names, self.integs, self.batch = names, integs, batch
        self.stream = torch.cuda.Stream()
        self.stream.wait_stream(torch.cuda.current_stream())  # the integrators' initial uploads
        self.plan = integs[0].chunks()
        self.pending = None

    def queue(self):
        """Queue the next chunk on the group's stream; False when done."""
        nxt = next(self.plan, None)
        if nxt is None:
            return False
        n = nxt[0]
        with torch.cuda.stream(self.stream):
            if self.batch is None:
                self.integs[0].advance(n)
            else:
                it = self.integs
                self.batch.propagate([x.u for x in it], [x.rho for x in it], [x.rho_s for x in it], it[0].dz, n)
        self.pending = nxt
        return True

    def record(self):
        _, z, i = self.pending
        with torch.cuda.stream(self.stream):
            for x in self.integs:
                x.after_chunk(z, i)


def run_scenarios(base_params, scenarios, out_root, reuse=True, envelope="gaussian_focused", batch=True):
    """Run every scenario (name -> run() overrides on base_params) into
    out_root/name; returns name -> result dict.  Cached results are reused
    when reuse is True (see load_scenario_npz); batch=False keeps every
    scenario on its own context."""
    out_root = Path(out_root)
    results, todo = {}, []
    for name, over in scenarios.items():
        out_dir = str(out_root / name)
        cached = load_scenario_npz(out_dir) if reuse else None
        if cached is not None:
            results[name] = cached
            continue
        params = {**base_params, **over, "out_dir": out_dir}
        params.pop("envelope", None)
        todo.append((name, run_config(**params)))
    env = base_params.get("envelope", envelope)
    groups = []
    # batch groups: same dz / nz / save_stride (they advance in lockstep)
    keyed = {}
    for name, cfg in todo:
        if batch and _batchable(cfg):
            keyed.setdefault((cfg.dz, cfg.nz, max(1, int(cfg.save_stride)), resolved_linear_mode(cfg)),
                             []).append((name, cfg))
        else:
            g = build_grids(cfg)
            groups.append(_Group([name], [Integrator(cfg, envelope=env, g=g)]))
    for members in keyed.values():
        if len(members) == 1:
            name, cfg = members[0]
            groups.append(_Group([name], [Integrator(cfg, envelope=env)]))
            continue
        cfgs = [c for _, c in members]
        grids = [build_grids(c) for c in cfgs]
        b = Batch(cfgs, grids)
        if resolved_linear_mode(cfgs[0]) == "split_f16":
            b.set_mode(MODE_SPLIT_F16)
        integs = [Integrator(c, envelope=env, ctx=b.context(i), g=g) for i, (c, g) in enumerate(zip(cfgs, grids))]
        groups.append(_Group([n for n, _ in members], integs, batch=b))
    active = list(groups)
    while active:
        active = [gr for gr in active if gr.queue()]
        for gr in active:
            gr.record()
    for gr in groups:
        with torch.cuda.stream(gr.stream):
            for name, x in zip(gr.names, gr.integs):
                results[name] = x._results()
    return {name: results[name] for name in scenarios}
