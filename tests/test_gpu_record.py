"""Integrator.propagate() outputs against the reference's own propagate().

record_tiny.npz holds the result dict of the reference Integrator (save stride
2, (z, r, t) cube with strides, absorption time bins, rho snapshot); our
Integrator on the same config and input must return the same keys with the
same shapes and values within FP32 tolerance, and write result.npz +
params.json the same way."""
import json
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELD_KEYS = ("fluence_rz", "Imax_z", "Ipeak_rz", "I_rzt", "I_onaxis_t")
RHO_KEYS = ("rho_rz", "rho_rzt", "rho_onaxis_t", "rho_rz_at")
LOSS_KEYS = ("absorbed_rz", "absorbed_rz_bins", "E_plasma_z", "E_MPI_z", "E_total_z")


@pytest.mark.parametrize("mode", ["plain", "split_bf16", "split_f16", "auto"])
def test_propagate_results_match_reference(mode, tmp_path):
    import rapport_gb300 as R
    from conftest import load_golden
    ref = load_golden("record_tiny.npz")
    Nr, Nt, R_max, w0, T_half, fwhm, E, f, dz, nz, seed = ref["meta"]
    cfg = R.workload_config(int(Nr), int(Nt), R_max, w0, T_half, dz, int(nz), linear_mode=mode,
                            save_stride=2, rho_t_stride=4, rho_r_stride=2,
                            absorb_time_bins_fs=(-100.0, -50.0, 0.0, 50.0, 100.0), rho_snapshot_t_fs=50.0,
                            out_dir=str(tmp_path / "run"))
    integ = R.Integrator(cfg, envelope=R.envelope_lens(w0, fwhm, E, f, int(seed)))
    assert integ.U0_uJ == pytest.approx(float(ref["U0_uJ"]), rel=1e-6)
    out = integ.propagate()
    for k in ("r", "rlist", "z", "t_sub_fs", "r_sub", "absorb_bin_edges_fs", "t_full_fs", "E_STE_z", "rho_s_rz",
              "rho_s_rzt", "rho_s_onaxis_t"):
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-12, atol=0, err_msg=k)
    for k in FIELD_KEYS:
        assert out[k].shape == ref[k].shape, k
        assert rel_l2(out[k], ref[k]) < 2e-4, k
    for k in RHO_KEYS:
        assert out[k].shape == ref[k].shape, k
        assert rel_l2(out[k], ref[k]) < 2e-3, k
    for k in LOSS_KEYS:
        assert np.shape(out[k]) == np.shape(ref[k]), k
        assert rel_l2(out[k], ref[k]) < 2e-3, k
    run = tmp_path / "run"
    saved = np.load(run / "result.npz", allow_pickle=True)
    assert set(saved.files) == set(out.keys())
    params = json.loads((run / "params.json").read_text())
    # "auto" runs the split-BF16 form on this tileable grid (and records it)
    assert params["toggles"]["enable_kerr_raman"] is False
    assert params["linear_mode"] == ("split_bf16" if mode == "auto" else mode)
    assert len(params["code_fingerprint"]) == 12
    assert not os.path.exists(run / "result.npz.tmp.npz")
