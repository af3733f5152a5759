"""numpy stand-in for ``cupy``, used ONLY to run the reference solver on the CPU
when generating golden fixtures (``tests/golden/make_golden.py``) and when
validating the oracle against the reference.  It is test infrastructure; the
product never imports it.

Arrays are plain numpy arrays.  ``RawKernel`` compiles the CUDA-C source string
the reference hands it as C++ under macro shims (see
``oracle/ref_build.py``) and emulates the launch grid with a host loop.
"""
import numpy as _np
from numpy import fft  # noqa: F401  (cp.fft.fft / ifft / fftfreq / ifftshift)


def asnumpy(a):
    return _np.asarray(a)


def ascontiguousarray(a):
    return _np.ascontiguousarray(a)


class RawKernel:
    def __init__(self, src, name):
        import os
        import sys
        here = os.path.dirname(os.path.abspath(__file__))
        repo = os.path.abspath(os.path.join(here, "..", "..", "..", ".."))
        sys.path.insert(0, os.path.join(repo, "oracle"))
        import ref_build  # noqa: E402
        self._lib, self._fn = ref_build.compile_kernel_source(src, name)

    def __call__(self, grid, block, args):
        import ctypes
        cargs = []
        keep = []
        for a in args:
            if isinstance(a, _np.ndarray):
                if not a.flags.c_contiguous:
                    raise ValueError("RawKernel stand-in needs contiguous arrays")
                keep.append(a)
                cargs.append(ctypes.c_void_p(a.ctypes.data))
            elif isinstance(a, (bool, _np.bool_)):
                cargs.append(ctypes.c_int(int(a)))
            elif isinstance(a, (int, _np.integer)):
                cargs.append(ctypes.c_int(int(a)))
            elif isinstance(a, (float, _np.floating)):
                cargs.append(ctypes.c_double(float(a)))
            else:
                raise TypeError(f"unsupported kernel argument {type(a)}")
        gx, bx = int(grid[0]), int(block[0])
        for b in range(gx):
            for t in range(bx):
                self._lib.ref_set_thread(b, t, bx)
                self._fn(*cargs)


def __getattr__(name):
    return getattr(_np, name)
