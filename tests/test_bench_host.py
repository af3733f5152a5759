"""Host-side logic of bench.py (no GPU): the DRAM-traffic record and its
fingerprint check, the reference arm's JSON line, and the seeded 64-pulse
draws of the mixed-grid workload."""
import json
import os
import subprocess
import sys

import numpy as np

import bench
from conftest import REPO

HEADER = ('"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size",'
          '"Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"')


def _row(i, kernel, metric, unit, value):
    return (f'"{i}","1","python3","127.0.0.1","void {kernel}(const CUtensorMap_st *, int)","1","7","(192, 1, 1)",'
            f'"(152, 1, 1)","0","10.3","Command line profiler metrics","{metric}","{unit}","{value}"')


def test_record_traffic_means_dram_bytes_per_launch_and_stamps_the_fingerprint(tmp_path):
    from rapport_gb300.build import kernel_fingerprint
    lines = ["==PROF== Connected to process 1", HEADER]
    for i, (rd, wr) in enumerate([(100.0, 50.0), (110.0, 40.0)]):  # two launches of the grouped product
        lines += [_row(i, "k_gemm_tc_grouped<3, 32, 4, 0>", "gpu__time_duration.sum", "us", "290.5"),
                  _row(i, "k_gemm_tc_grouped<3, 32, 4, 0>", "dram__bytes_read.sum", "Mbyte", f"{rd:.2f}"),
                  _row(i, "k_gemm_tc_grouped<3, 32, 4, 0>", "dram__bytes_write.sum", "Mbyte", f"{wr:.2f}")]
    lines += [_row(2, "k_row_nl_b<2048, 1>", "dram__bytes_read.sum", "Gbyte", "0.35"),
              _row(2, "k_row_nl_b<2048, 1>", "dram__bytes_write.sum", "Mbyte", "200.00"),
              _row(3, "k_tune_fill", "dram__bytes_read.sum", "byte", "1,024"),
              _row(3, "k_tune_fill", "dram__bytes_write.sum", "byte", "0")]
    csv_path = tmp_path / "traffic.csv"
    csv_path.write_text("\n".join(lines) + "\n")
    out = tmp_path / "traffic.json"
    bench.record_traffic(str(csv_path), out_path=str(out))
    rec = json.loads(out.read_text())["kernels"]
    assert set(rec) == {"k_gemm_tc_batched", "k_row_nl_batched"}
    assert rec["k_gemm_tc_batched"]["bytes_per_launch"] == 150_000_000
    assert rec["k_gemm_tc_batched"]["launches"] == 2
    assert rec["k_row_nl_batched"]["bytes_per_launch"] == 550_000_000
    assert rec["k_gemm_tc_batched"]["kernel_fingerprint"] == kernel_fingerprint()
    v, why = bench.measured_traffic("k_gemm_tc_batched", path=str(out))
    assert v == 150_000_000, why
    # a capture of other kernel sources is not reported
    data = json.loads(out.read_text())
    data["kernels"]["k_gemm_tc_batched"]["kernel_fingerprint"] = "0" * 16
    out.write_text(json.dumps(data))
    v, why = bench.measured_traffic("k_gemm_tc_batched", path=str(out))
    assert v is None and "other kernel sources" in why
    v, why = bench.measured_traffic("k_row_next_batched", path=str(out))
    assert v is None and "no capture" in why


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["unit"] == "z-steps/s" and d["higher_is_better"] is True and d["steps"] == 1
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["config"]["Nr"] == 1024 and d["config"]["Nt"] == 2048


def test_mixed_pulse_draws_are_seeded_and_within_the_workload_ranges():
    a, b = bench.mixed_pulses(), bench.mixed_pulses()
    assert a == b and len(a) == 64
    assert {p["Nr"] for p in a} <= {512, 768, 1024} and {p["Nt"] for p in a} <= {1024, 2048, 4096}
    assert len({(p["Nr"], p["Nt"]) for p in a}) >= 6  # the grids are mixed
    E = np.array([p["E"] for p in a])
    assert E.min() >= 1.0 and E.max() <= 20.0
    assert all(50e-15 <= p["fwhm"] <= 200e-15 and 80e-6 <= p["w0"] <= 200e-6 and 0.05 <= p["f"] <= 0.20
               and p["dz"] == 5e-6 and p["R_max"] == 10 * p["w0"] and p["T_half"] == 4 * p["fwhm"] for p in a)
    assert bench.mixed_pulses(seed=2) != a
