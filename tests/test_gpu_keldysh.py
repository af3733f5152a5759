"""The reference's default rate model (Keldysh photo-ionisation tables) on the GPU.

tiny_keldysh.npz was written by the reference itself with KeldyshSiO2 filling
the spline and both carrier tables (grids.py:140-161; the 6 eV exciton table is
live because the exciton channel is on), no power-law substitution.  The
product builds the same tables on the host (grids.keldysh_rate; pinned to the
reference's rate on every knot in test_host_grids.py) and propagates through
the C ABI in each arithmetic.

Tolerances as for the power-law fixtures: split() and the carrier march as in
test_gpu_parity.py; 1 and 4 z-steps field relative L2 1e-4, densities 1e-3 of
the peak.
"""
import numpy as np
import pytest

from conftest import meta_case, rel_l2
from gpu_util import dev, host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kel_objs(tiny_keldysh):
    import rapport_gb300 as R
    m = meta_case(tiny_keldysh)
    cfg = R.workload_config(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"], m["dz"], m["nsteps"],
                            rate_model="keldysh", enable_ste=True, tau_ste=1e-12)
    g = R.build_grids(cfg)
    lin = R.LinearOperator(cfg, g)
    nl = R.NonlinearOperator(cfg, g, lin.ctx)
    return m, lin, nl


def test_update_plasma_and_split_match_reference(tiny_keldysh, kel_objs):
    d = tiny_keldysh
    m, lin, nl = kel_objs
    rho, rs = dev(np.zeros(d["u0"].shape)), dev(np.zeros(d["u0"].shape))
    nl.update_plasma(dev(d["u0"]), rho, rs)
    for got, ref in ((host(rho), d["rho_u0"]), (host(rs), d["rho_s_u0"])):
        peak = np.maximum(ref.max(axis=1, keepdims=True), 1e-30)
        assert np.all(np.abs(got - ref) <= 2e-4 * peak + 1e-30)
    assert d["rho_s_u0"].max() > 1e-3 * d["rho_u0"].max() > 0   # both tables matter
    rhs, al = nl.split(dev(d["hl_u0"]), dev(d["rho_u0"]), dev(d["rho_s_u0"]))
    assert rel_l2(host(rhs), d["split_rhs"]) < 2e-5
    assert rel_l2(host(al), d["split_alpha"]) < 2e-5


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_z_steps_match_reference(tiny_keldysh, kel_objs, mode):
    d = tiny_keldysh
    m, lin, _ = kel_objs
    ctx = lin.ctx
    u = dev(d["u0"])
    rho, rs = dev(np.zeros(d["u0"].shape)), dev(np.zeros(d["u0"].shape))
    done = 0
    for j, s in enumerate(d["steps_kept"]):
        ctx.propagate(u, rho, rs, m["dz"], int(s) - done, mode)
        done = int(s)
        assert rel_l2(host(u), d["u_steps"][j]) < 1e-4, (mode, s)
        for got, ref in ((host(rho), d["rho_steps"][j]), (host(rs), d["rho_s_steps"][j])):
            assert np.abs(got - ref).max() <= 1e-3 * max(ref.max(), 1e-30), (mode, s)
    assert ctx.device_status() == 0
