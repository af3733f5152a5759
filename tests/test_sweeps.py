"""Host logic of the scenario-sweep driver (no GPU): scenario sets, the
result cache and its code-fingerprint check, the summary table."""
import json

import numpy as np

import rapport_gb300 as R
from rapport_gb300.integrator import code_fingerprint


def test_ablation_scenarios_follow_the_field_toggles():
    sc = R.build_scenarios()
    assert list(sc)[0] == "full" and sc["full"] == {}
    assert sc["linear_only"] == {f: False for f in R.FIELD_TOGGLES}
    for f in R.FIELD_TOGGLES:
        assert sc["no_" + f.replace("enable_", "")] == {f: False}
    assert len(sc) == len(R.FIELD_TOGGLES) + 2


def test_energy_scenarios():
    sc = R.energy_scenarios([0.25, 1.1, 1.25], prefix="couairon2005")
    assert sc == {"couairon2005_0.25uJ": {"energy_uJ": 0.25}, "couairon2005_1.1uJ": {"energy_uJ": 1.1},
                  "couairon2005_1.25uJ": {"energy_uJ": 1.25}}


def _write(d, fp, payload=None):
    d.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(d / "result.npz", **(payload or {"Imax_z": np.arange(3.0)}))
    (d / "params.json").write_text(json.dumps({"code_fingerprint": fp}))


def test_cache_reuse_and_staleness(tmp_path):
    assert R.load_scenario_npz(tmp_path / "absent") is None
    fresh = tmp_path / "fresh"
    _write(fresh, code_fingerprint())
    got = R.load_scenario_npz(fresh)
    assert got is not None and np.array_equal(got["Imax_z"], np.arange(3.0))
    stale = tmp_path / "stale"
    _write(stale, "0123456789ab")
    assert R.load_scenario_npz(stale) is None
    assert R.load_scenario_npz(stale, ignore_stale=True) is not None
    broken = tmp_path / "broken"
    _write(broken, code_fingerprint())
    (broken / "result.npz").write_bytes(b"PK\x03\x04 truncated")
    assert R.load_scenario_npz(broken) is None


def test_summary_rows():
    res = {"a": dict(Imax_z=np.array([1.0, 5.0, 2.0]), z=np.array([0.0, 1e-6, 2e-6]),
                     r=np.array([-2.0, -1.0, 1.0, 2.0]),
                     rho_rz=np.array([[0, 1, 1, 0], [0, 3, 3, 0], [0, 2, 2, 0]], dtype=float))}
    (row,) = R.summarize(res)
    assert row == dict(scenario="a", I_peak_Wcm2=5.0, z_at_Ipeak_um=1.0, rho_e_onaxis_max_cm3=3.0)
