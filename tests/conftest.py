import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


@pytest.fixture(scope="session")
def tiny():
    return load_golden("tiny.npz")


@pytest.fixture(scope="session")
def hot():
    return load_golden("tiny_hot.npz")


@pytest.fixture(scope="session")
def cfg1():
    return load_golden("config1_prefix.npz")


@pytest.fixture(scope="session")
def full():
    return load_golden("tiny_full.npz")


# every split() term on (tiny_full.npz): Raman with f_R 0.18, self-steepening,
# space-time focusing, excitons with a 1 ps decay
FULL_PHYSICS = dict(f_R=0.18, enable_kerr_raman=True, enable_self_steepening=True,
                    enable_space_time_focusing=True, enable_ste=True, tau_ste=1e-12)


@pytest.fixture(scope="session")
def tiny_keldysh():
    # the reference's default rate model (Keldysh tables) with the exciton channel on
    return load_golden("tiny_keldysh.npz")


@pytest.fixture(scope="session")
def k1edge():
    return load_golden("k1_edge.npz")


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def meta_case(d):
    """Unpack the meta vector of a propagation fixture."""
    Nr, Nt, R_max, w0, T_half, fwhm, E, f, dz, nsteps, seed = d["meta"]
    return dict(Nr=int(Nr), Nt=int(Nt), R_max=R_max, w0=w0, T_half=T_half, fwhm=fwhm, E=E, f=f,
                dz=dz, nsteps=int(nsteps), seed=int(seed))
