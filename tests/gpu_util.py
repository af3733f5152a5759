"""Helpers shared by the GPU tests: product objects + the oracle on identical inputs."""
import numpy as np

import nlse_oracle as O
import rapport_gb300 as R
from conftest import meta_case


def torch():
    import torch as t
    return t


def dev(u):
    t = torch()
    if np.iscomplexobj(u):
        return t.from_numpy(np.ascontiguousarray(u, dtype=np.complex64)).cuda()
    return t.from_numpy(np.ascontiguousarray(u, dtype=np.float32)).cuda()


def host(x):
    return x.detach().cpu().numpy().astype(np.complex128 if x.is_complex() else np.float64)


class Case:
    """Product context + oracle grid for one workload (tiny / 256 x 512 / ...)."""

    def __init__(self, Nr, Nt, R_max, w0, T_half, fwhm, E, f, dz, nsteps=1, seed=0, **over):
        self.cfg = R.workload_config(Nr, Nt, R_max, w0, T_half, dz, max(nsteps, 1), **over)
        self.g = R.build_grids(self.cfg)
        self.integ = None
        self.lin = R.LinearOperator(self.cfg, self.g)
        self.nl = R.NonlinearOperator(self.cfg, self.g, self.lin.ctx)
        self.ctx = self.lin.ctx
        self.og = O.OracleGrid(O.workload_config(Nr, Nt, R_max, w0, T_half, **over))
        self.dz = dz
        self.u0 = O.lens_gaussian(self.og, w0, fwhm, E, f, seed)

    @classmethod
    def from_fixture(cls, d):
        m = meta_case(d)
        return cls(m["Nr"], m["Nt"], m["R_max"], m["w0"], m["T_half"], m["fwhm"], m["E"], m["f"], m["dz"],
                   m["nsteps"], m["seed"])

    def oracle_nl_block(self, u, rho, rs=None):
        """alpha/2, RK4, alpha/2 of Integrator.step (integrator.py:140-147) in FP64."""
        og, dz = self.og, self.dz
        rs = np.zeros_like(rho) if rs is None else rs
        _, a = og.split(u, rho, rs)
        u = u * np.exp(-0.5 * dz * a)
        k1, _ = og.split(u, rho, rs)
        k2, _ = og.split(u + 0.5 * dz * k1, rho, rs)
        k3, _ = og.split(u + 0.5 * dz * k2, rho, rs)
        k4, _ = og.split(u + dz * k3, rho, rs)
        u = u + dz / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        _, a = og.split(u, rho, rs)
        return u * np.exp(-0.5 * dz * a)


# the measured single-pulse workload: 1024 x 2048, R_max 2 mm, +-800 fs, 5 uJ, w0 150 um, f 10 cm
CONFIG2 = dict(Nr=1024, Nt=2048, R_max=2e-3, w0=150e-6, T_half=800e-15, fwhm=100e-15, E=5.0, f=0.1,
               dz=2.5e-6)
