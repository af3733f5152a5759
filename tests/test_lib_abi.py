"""The C ABI library: built, loadable, exports every declared symbol, and the
ctypes mirror of nlse_grid_desc matches the C layout.  No compute calls."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO
from rapport_gb300 import _lib

HEADER = os.path.join(REPO, "include", "nlse.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char \*)\s*\*?\s*(nlse_\w+)\s*\(", src, re.M)))


def test_header_lists_match():
    assert _declared() == sorted(_lib.EXPORTS)


def test_library_loads_and_exports_all_symbols():
    if not os.path.exists(_lib.LIB_PATH):
        from rapport_gb300 import build
        build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for name in _declared():
        assert hasattr(lib, name), name
    lib.nlse_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.nlse_version()


def test_create_error_path_without_device_or_with_bad_desc():
    lib = _lib.load()
    h = ctypes.c_void_p()
    d = _lib.GridDesc()
    d.Nr, d.Nt = 4, 100          # Nt not a power of two: rejected before any CUDA call
    st = lib.nlse_create(ctypes.byref(d), ctypes.byref(h))
    assert st == _lib.NLSE_ERR_INVALID_ARG
    buf = ctypes.create_string_buffer(256)
    assert lib.nlse_get_last_error(None, buf, 256) == _lib.NLSE_ERR_INVALID_ARG
    assert b"power of two" in buf.value
    d.Nt, d.flags = 64, _lib.F_KERR_RAMAN      # Raman without its R_f table
    assert lib.nlse_create(ctypes.byref(d), ctypes.byref(h)) == _lib.NLSE_ERR_INVALID_ARG
    d.Nt, d.flags = 8192, _lib.F_SELF_STEEP    # the full-physics block holds N_t <= 4096
    assert lib.nlse_create(ctypes.byref(d), ctypes.byref(h)) == _lib.NLSE_ERR_UNSUPPORTED
    d.Nt, d.flags = 64, 1 << 12                 # unknown flag bit
    assert lib.nlse_create(ctypes.byref(d), ctypes.byref(h)) == _lib.NLSE_ERR_INVALID_ARG
    assert lib.nlse_half_linear(None, None, 1.0, None) == _lib.NLSE_ERR_INVALID_ARG


def test_struct_layout_matches_header(tmp_path):
    fields = [f for f, _ in _lib.GridDesc._fields_]
    prog = tmp_path / "layout.c"
    body = "\n".join(f'printf("{f} %zu\\n", offsetof(nlse_grid_desc, {f}));' for f in fields)
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "nlse.h"\nint main(void){\n'
                    f'printf("size %zu\\n", sizeof(nlse_grid_desc));\n{body}\nreturn 0;}}\n')
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(REPO, "include"), str(prog), "-o", str(exe)])
    out = dict(line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())
    assert int(out["size"]) == ctypes.sizeof(_lib.GridDesc)
    for f in fields:
        assert int(out[f]) == getattr(_lib.GridDesc, f).offset, f


def test_context_refuses_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import rapport_gb300 as R
    cfg = R.workload_config(8, 16, 1e-4, 1e-5, 3e-13, 5e-6, 1)
    with pytest.raises(RuntimeError, match="CUDA"):
        _lib.Context(cfg, R.build_grids(cfg))
