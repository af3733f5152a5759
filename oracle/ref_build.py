"""Recipe that compiles the reference's own carrier-rate kernel into oracle/_ref/.

TEST INFRASTRUCTURE ONLY (never imported by the product).

The reference ships its only native component, ``solve_rate_equation_kernel``,
as a CUDA-C source string inside ``deliverable (3)/sim/kernels.py:13-106``.
This recipe compiles that string unmodified as C++ under a few macro shims
(``__global__``/``__device__`` removed, a ``double2`` struct, thread indices
as host globals) into ``oracle/_ref/k1_ref_<hash>.so``; a host loop then plays
the launch grid.  The result is the reference's own arithmetic on the CPU and
is used to pin the oracle's C restatement (``oracle/rate_scan.c``).

The source is read where it lies under the reference checkout (or handed over
by the cupy stand-in's RawKernel); nothing of it is copied into the repository.
``oracle/_ref/`` is git-ignored.
"""
import ctypes
import hashlib
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout (RAPPORT_REFERENCE; the build container's copy by default)
REF_ROOT = os.environ.get("RAPPORT_REFERENCE", "/root/reference")
REF_KERNELS_PY = os.path.join(REF_ROOT, ".github", "deliverable (3)", "sim", "kernels.py")

_PRELUDE = r"""
#include <cmath>
using std::isfinite; using std::exp; using std::log10; using std::fabs;
struct double2 { double x, y; };
struct ref_uint3 { unsigned int x, y, z; };
static ref_uint3 threadIdx, blockIdx, blockDim;
extern "C" void ref_set_thread(unsigned b, unsigned t, unsigned bd) {
    blockIdx.x = b; threadIdx.x = t; blockDim.x = bd;
}
#define __global__
#define __device__
#define __forceinline__ inline
"""


def reference_available():
    return os.path.exists(REF_KERNELS_PY)


def extract_kernel_source(path=REF_KERNELS_PY):
    """Return the raw CUDA-C string assigned to _RATE_KERNEL_SRC in kernels.py."""
    with open(path, "r", encoding="utf-8") as f:
        text = f.read()
    m = re.search(r"_RATE_KERNEL_SRC\s*=\s*r'''(.*?)'''", text, re.S)
    if not m:
        raise RuntimeError("kernel source string not found in " + path)
    return m.group(1)


def compile_kernel_source(src, name):
    """Compile a CUDA-C kernel string as C++; return (lib, kernel function)."""
    os.makedirs(OUT, exist_ok=True)
    h = hashlib.sha256((src + name).encode()).hexdigest()[:12]
    so = os.path.join(OUT, f"k1_ref_{h}.so")
    if not os.path.exists(so):
        cpp = os.path.join(OUT, f"k1_ref_{h}.cpp")
        with open(cpp, "w") as f:
            f.write(_PRELUDE)
            f.write(src)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared",
                               "-o", so, cpp])
        os.remove(cpp)
    lib = ctypes.CDLL(so)
    lib.ref_set_thread.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint]
    fn = getattr(lib, name)
    fn.restype = None
    return lib, fn


def build():
    """Build oracle/_ref from the reference checkout; return the .so path or None."""
    if not reference_available():
        return None
    lib, _ = compile_kernel_source(extract_kernel_source(), "solve_rate_equation_kernel")
    return lib._name


class RefRateKernel:
    """Host launcher for the compiled reference kernel (FP64, one thread per r)."""

    def __init__(self):
        self.lib, self.fn = compile_kernel_source(extract_kernel_source(),
                                                  "solve_rate_equation_kernel")
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        self.fn.argtypes = [P, P, P, I, I, D, D, D, D, D, D, D, I, P, P, I, D, D, D, D]

    def __call__(self, E, ne, ns, dt, field_to_I, beta_g, beta_s, na, inv_tau_r,
                 inv_tau_ste, enable_ste, lut, lut_s, log_min, inv_dlog, Imin, Imax):
        import numpy as np
        E = np.ascontiguousarray(E, dtype=np.complex128)
        Nr, Nt = E.shape
        lut = np.ascontiguousarray(lut, dtype=np.float64)
        lut_s = np.ascontiguousarray(lut_s, dtype=np.float64)
        for ri in range(Nr):
            self.lib.ref_set_thread(0, ri, Nr)
            self.fn(E.ctypes.data, ne.ctypes.data, ns.ctypes.data, Nr, Nt, dt,
                    field_to_I, beta_g, beta_s, na, inv_tau_r, inv_tau_ste,
                    int(enable_ste), lut.ctypes.data, lut_s.ctypes.data, lut.size,
                    log_min, inv_dlog, Imin, Imax)


if __name__ == "__main__":
    print(build())
