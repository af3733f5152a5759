"""The allocation-free half step, nlse_half_linear_noalloc, through the C ABI.

It exists for callers that cannot allocate device memory themselves -- a host
application whose memory pool owns every device buffer, a real-time loop that
must not reach the allocator, code that cannot create a context.  It takes the
QDHT matrix, the phase tables and the field as caller-owned device buffers
and keeps its intermediate field in a static device array shared by every
call.  This test checks it against the context entry point nlse_half_linear
on two calls in a row with different fields (the second call must not depend
on what the first left in the shared array), pins both to the FP64 oracle's
half_linear (the reference's LinearOperator.half_linear restated), and checks
that a size beyond the array is refused with a clear error before anything is
launched.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-5  # relative L2, the FP32 tolerance of the parity tests


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_half_linear_matches_context_entry():
    import torch

    import rapport_gb300 as R
    from rapport_gb300 import _lib

    Nr, Nt, dz = 256, 512, 5e-6
    cfg = R.workload_config(Nr, Nt, 1e-3, 100e-6, 400e-15, dz, 1)
    g = R.build_grids(cfg)
    ctx = _lib.Context(cfg, g)
    lib = _lib.load()

    # the caller's own tables, computed in FP64 on the host and rounded once
    rk = (g["R"] ** 2 / g["j1last"]) * (g["j1last"] / g["R"] ** 2)
    Pt = np.exp(1j * g["delta_k"] * dz / 2) * g["spec_mask"] * rk / Nt
    Pr = np.exp(-1j * g["rholist"] ** 2 * dz / (4 * g["komega"]))
    Y = torch.from_numpy(g["Y"].astype(np.float32)).cuda()
    Ptd = torch.from_numpy(Pt.astype(np.complex64)).cuda()
    Prd = torch.from_numpy(Pr.astype(np.complex64)).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    rng = np.random.default_rng(4)
    fields = [R.envelope_lens(100e-6, 100e-15, 1.0, 0.1, 0)(g["rr"], g["tt"], cfg, g),
              (rng.standard_normal((Nr, Nt)) + 1j * rng.standard_normal((Nr, Nt))) * 1e9]
    import nlse_oracle as O
    og = O.OracleGrid(O.workload_config(Nr, Nt, 1e-3, 100e-6, 400e-15))
    for f in fields:  # two calls in a row
        u = torch.from_numpy(f.astype(np.complex64)).cuda()
        want = og.half_linear(u.cpu().numpy().astype(np.complex128), dz)
        ref = u.clone()
        ctx.half_linear(ref, dz)
        out = u.clone()
        st = lib.nlse_half_linear_noalloc(_ptr(Y), _ptr(Ptd), _ptr(Prd), _ptr(out), Nr, Nt, stream)
        assert st == _lib.NLSE_OK
        torch.cuda.synchronize()
        err = float((out - ref).abs().norm() / ref.abs().norm())
        assert err < TOL, err
        got = out.cpu().numpy().astype(np.complex128)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < TOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    from rapport_gb300 import _lib

    lib = _lib.load()
    x = torch.zeros(4, dtype=torch.float32, device="cuda")
    st = lib.nlse_half_linear_noalloc(_ptr(x), _ptr(x), _ptr(x), _ptr(x), 1024, 2048, None)
    assert st == _lib.NLSE_ERR_INVALID_ARG
    buf = ctypes.create_string_buffer(512)
    assert lib.nlse_get_last_error(None, buf, 512) == _lib.NLSE_ERR_INVALID_ARG
    assert b"static scratch" in buf.value
