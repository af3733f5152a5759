"""The row FFT's compile-time shared-memory offsets (nlse_internal.cuh), checked
on the host against the padded index they replace.

A Stockham pass of radix R at stride NS gathers points j + r N/R and scatters
to d0 + r NS with d0 = (j - k) R + k, k = j mod NS; the padded slot of point i
is pidx(i) = i + i/16.  The kernels address those R points from one padded base
at compile-time offsets (pass_src_linear / pass_dst_linear / pass_dst_step).
This compiles a host program against the header itself and checks, for every
pass of every row length 16 .. 8192 and every butterfly, that the offsets give
the same slots as pidx."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

PROGRAM = r"""
#include <cstdio>
#include "nlse_internal.cuh"

int main() {
    long checked = 0, bad = 0, linear_passes = 0, passes = 0;
    for (int N = 16; N <= 8192; N *= 2) {
        for (int NS = 1; NS < N; NS *= fft_radix(N, NS)) {
            const int R = fft_radix(N, NS), nb = N / R;
            ++passes;
            if (pass_src_linear(nb) && pass_dst_linear(NS, R)) ++linear_passes;
            for (int j = 0; j < nb; ++j) {
                const int k = j & (NS - 1), d0 = (j - k) * R + k;
                for (int r = 0; r < R; ++r) {
                    if (pass_src_linear(nb)) {
                        ++checked;
                        bad += pidx(j) + r * (nb + nb / 16) != pidx(j + r * nb);
                    }
                    if (pass_dst_linear(NS, R)) {
                        ++checked;
                        bad += pidx(d0) + pass_dst_step(NS, r) != pidx(d0 + r * NS);
                    }
                }
            }
        }
    }
    std::printf("%ld %ld %ld %ld\n", checked, bad, linear_passes, passes);
    return bad != 0;
}
"""


def test_compile_time_pass_offsets_equal_the_padded_index(tmp_path):
    from rapport_gb300 import build as b
    if shutil.which(b.NVCC) is None and not os.path.exists(b.NVCC):
        pytest.skip("nvcc not available")
    src = tmp_path / "pass_offsets.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "pass_offsets"
    cmd = [b.NVCC, *b.ARCH, "-std=c++17", "-I", b.CSRC, "-I", b.INCLUDE, str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    checked, bad, linear, passes = map(int, r.stdout.split())
    assert r.returncode == 0 and bad == 0
    assert checked > 100_000
    # every pass from N = 128 on uses the linear forms; below, the six passes of N = 16, 32, 64 keep pidx
    assert linear == passes - 6
