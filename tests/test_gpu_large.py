"""The large single-pulse grid (N_r = 2048, R_max 3 mm; N_t = 8192, +-1.5 ps; 20 uJ, 80 fs,
w0 200 um, f 15 cm, dz 1.25 um): both arithmetics against the FP64 GPU
reference (pinned to the numpy oracle in test_gpu_accuracy.py) for two
z-steps -- the largest single-GPU grid of the measured workloads (134 MB field,
the 8192-point row kernels, 1024-tile products)."""
import numpy as np
import pytest

from conftest import rel_l2
from gpu_util import Case, dev, host

pytestmark = pytest.mark.gpu

CONFIG5 = dict(Nr=2048, Nt=8192, R_max=3e-3, w0=200e-6, T_half=1.5e-12, fwhm=80e-15, E=20.0, f=0.15,
               dz=1.25e-6)


def test_large_pulse_two_z_steps_both_forms():
    import torch
    import fp64_gpu
    from rapport_gb300._lib import MODE_PLAIN_F32, MODE_SPLIT_BF16
    c = Case(**CONFIG5)
    ref = fp64_gpu.FP64GPU(c.og)
    ur, rr = ref.propagate(c.u0, 2, c.dz)
    ur, rr = ur.cpu().numpy(), rr.cpu().numpy()
    for mode in (MODE_SPLIT_BF16, MODE_PLAIN_F32):
        u, rho, rs = dev(c.u0), dev(np.zeros(c.u0.shape)), dev(np.zeros(c.u0.shape))
        c.ctx.propagate(u, rho, rs, c.dz, 2, mode)
        torch.cuda.synchronize()
        assert rel_l2(host(u), ur) < 2e-5, mode
        assert np.abs(host(rho) - rr).max() <= 1e-3 * max(rr.max(), 1e-30), mode
    assert c.ctx.device_status() == 0
