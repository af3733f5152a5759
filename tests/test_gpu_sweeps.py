"""The scenario-sweep driver on the GPU: scenarios run together (one batch for
the batchable ones -- the exciton channel and the Raman / self-steepening terms
included -- own streams for the rest) give exactly what run() gives for each
alone, and cached results are reused."""
import os

import numpy as np
import pytest

import rapport_gb300 as R

pytestmark = pytest.mark.gpu

BASE = dict(Nz=6, Nt=256, Nr=65, wavelength=800e-9, energy_uJ=1.0, w0=10e-6, delta_t=300e-15 * np.sqrt(2 * np.log(2)) / 5,
            begin=-15e-6, end=15e-6, n2=3.2e-20, Ui_eV=9.0, R_factor=10.0, save_stride=2, verbose=False,
            linear_mode="split_bf16", rate_model="mpi", f_R=0.0, enable_kerr_raman=False,
            enable_self_steepening=False, enable_space_time_focusing=False, enable_ste=False, rho_t_stride=0)
KEYS = ("fluence_rz", "rho_rz", "Imax_z", "absorbed_rz", "E_total_z", "rho_onaxis_t", "I_onaxis_t")


def test_sweep_equals_individual_runs(tmp_path):
    sc = R.energy_scenarios([1.0, 2.0, 3.0], prefix="e")
    sc["plain_2uJ"] = {"energy_uJ": 2.0, "linear_mode": "plain"}            # own stream
    sc["ste_2uJ"] = {"energy_uJ": 2.0, "enable_ste": True}                  # batched: own march launch
    sc["raman_2uJ"] = {"energy_uJ": 2.0, "f_R": 0.18, "enable_kerr_raman": True,
                       "enable_self_steepening": True}                      # batched: own row class
    sc["stf_2uJ"] = {"energy_uJ": 2.0, "enable_space_time_focusing": True,
                     "linear_mode": "plain"}                                # own stream
    got = R.run_scenarios(BASE, sc, tmp_path / "sweep")
    for name, over in sc.items():
        ref = R.run(**{**BASE, **over, "out_dir": str(tmp_path / "single" / name)})
        for k in KEYS:
            assert np.array_equal(np.asarray(got[name][k]), np.asarray(ref[k])), (name, k)
        assert os.path.exists(tmp_path / "sweep" / name / "params.json")
    # the energies really differ
    assert got["e_3uJ"]["Imax_z"].max() > got["e_1uJ"]["Imax_z"].max()


def test_sweep_reuses_cached_results(tmp_path):
    sc = R.energy_scenarios([1.0, 2.0], prefix="e")
    first = R.run_scenarios(BASE, sc, tmp_path)
    stamp = {n: os.path.getmtime(tmp_path / n / "result.npz") for n in sc}
    again = R.run_scenarios(BASE, sc, tmp_path)
    for n in sc:
        assert os.path.getmtime(tmp_path / n / "result.npz") == stamp[n]
        assert np.array_equal(again[n]["Imax_z"], first[n]["Imax_z"])
    rows = R.summarize(again)
    assert [r["scenario"] for r in rows] == list(sc)
