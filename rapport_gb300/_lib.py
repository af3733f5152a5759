"""ctypes binding of libnlse.so (the C ABI declared in include/nlse.h).

The library is loaded from ``rapport_gb300/lib/libnlse.so`` (built in-tree by
``rapport_gb300.build``).  There is no fallback: if the library is missing or
a CUDA device is unavailable, constructing a Context raises.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libnlse.so")

NLSE_OK, NLSE_ERR_INVALID_ARG, NLSE_ERR_UNSUPPORTED, NLSE_ERR_CUDA, NLSE_ERR_DEVICE_FLAG, NLSE_ERR_TIMEOUT = range(6)
F_KERR_INSTANT, F_PHOTO_LOSS, F_PLASMA_DEFOC, F_PLASMA_ABSORB = 1, 2, 4, 8
F_KERR_RAMAN, F_SELF_STEEP, F_SPACE_TIME, F_STE = 16, 32, 64, 128
MODE_PLAIN_F32, MODE_SPLIT_BF16, MODE_SPLIT_F16 = 0, 1, 2

# every symbol include/nlse.h declares (checked by the CPU test suite)
EXPORTS = ("nlse_create", "nlse_half_linear", "nlse_half_linear_ex", "nlse_split", "nlse_nonlinear_step",
           "nlse_update_plasma", "nlse_rate_equation", "nlse_step", "nlse_step_batched", "nlse_propagate", "nlse_set_split_terms",
           "nlse_device_status", "nlse_debug_operator_product", "nlse_debug_wait_timeout", "nlse_scan_fallback_rows",
           "nlse_half_linear_noalloc", "nlse_record", "nlse_set_gemm_variant", "nlse_get_gemm_variant", "nlse_get_row_plan", "nlse_set_row_plan", "nlse_batch_create", "nlse_batch_propagate", "nlse_batch_get_context",
           "nlse_batch_set_split_terms", "nlse_batch_set_mode", "nlse_batch_device_status", "nlse_batch_get_last_error",
           "nlse_batch_destroy",
           "nlse_profile_start", "nlse_profile_read", "nlse_kernel_name",
           "nlse_get_last_error", "nlse_destroy", "nlse_version")

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int


class GridDesc(ctypes.Structure):
    """Mirror of nlse_grid_desc."""
    _fields_ = [
        ("Nr", _I), ("Nt", _I), ("flags", _I), ("dt", _D), ("komega", _D),
        ("Y", _P), ("rho_modes", _P), ("delta_k", _P), ("spec_mask", _P), ("mask_r", _P),
        ("Rk_iRk", _D),
        ("invE2", _D), ("kerr_pref", _D), ("kerr_scale", _D), ("plasma_pref", _D),
        ("omega0_tau_c", _D), ("rho_max", _D), ("photo_const", _D),
        ("pchip_n", _I), ("pchip_x", _P), ("pchip_c", _P),
        ("lut_n", _I), ("lut", _P), ("lut_log_min", _D), ("lut_inv_dlog", _D),
        ("lut_Imin", _D), ("lut_Imax", _D), ("beta_g", _D), ("inv_tau_r", _D),
        ("lut_s", _P), ("beta_s", _D), ("inv_tau_ste", _D), ("ste_pref", _D),
        ("f_R", _D), ("R_f", _P), ("T_op", _P), ("inv_U_nl", _P), ("inv_U_op", _P),
    ]


class PulseDesc(ctypes.Structure):
    """Mirror of nlse_pulse_desc."""
    _fields_ = [("u", _P), ("rho", _P), ("rho_s", _P), ("dz", _D), ("nsteps", _I), ("mode", _I)]


_lib = None


def load():
    """Load libnlse.so once and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built: run `python -c \"import __graft_entry__ as g; g.build()\"`")
    lib = ctypes.CDLL(LIB_PATH)
    lib.nlse_create.argtypes = [ctypes.POINTER(GridDesc), ctypes.POINTER(_P)]
    lib.nlse_half_linear.argtypes = [_P, _P, _D, _P]
    lib.nlse_half_linear_ex.argtypes = [_P, _P, _D, _I, _P]
    lib.nlse_set_split_terms.argtypes = [_P, _I]
    lib.nlse_half_linear_noalloc.argtypes = [_P, _P, _P, _P, _I, _I, _P]
    lib.nlse_debug_operator_product.argtypes = [_P, _P, _P, _D, _P]
    lib.nlse_device_status.argtypes = [_P, ctypes.POINTER(_I)]
    lib.nlse_debug_wait_timeout.argtypes = [_P, _I, _P]
    lib.nlse_split.argtypes = [_P, _P, _P, _P, _P, _P, _P]
    lib.nlse_nonlinear_step.argtypes = [_P, _P, _P, _P, _D, _P]
    lib.nlse_update_plasma.argtypes = [_P, _P, _P, _P, _P]
    lib.nlse_rate_equation.argtypes = [_P, _P, _P, _P, _P]
    lib.nlse_step.argtypes = [_P, _P, _P, _P, _D, _I, _P]
    lib.nlse_propagate.argtypes = [_P, _P, _P, _P, _D, _I, _I, _P]
    lib.nlse_step_batched.argtypes = [_P, ctypes.POINTER(PulseDesc), _I, _P]
    lib.nlse_scan_fallback_rows.argtypes = [_P, ctypes.POINTER(_I)]
    lib.nlse_get_last_error.argtypes = [_P, ctypes.c_char_p, ctypes.c_size_t]
    lib.nlse_destroy.argtypes = [_P]
    lib.nlse_destroy.restype = None
    lib.nlse_version.restype = ctypes.c_char_p
    lib.nlse_profile_start.argtypes = [_P, _I]
    lib.nlse_profile_read.argtypes = [_P, ctypes.POINTER(_I), ctypes.POINTER(_D), _I, ctypes.POINTER(_I)]
    lib.nlse_kernel_name.argtypes = [_I]
    lib.nlse_kernel_name.restype = ctypes.c_char_p
    lib.nlse_set_gemm_variant.argtypes = [_P, _I]
    lib.nlse_record.argtypes = [_P, _P, _P, _P, _P, _I, _P, _P]
    lib.nlse_get_gemm_variant.argtypes = [_P]
    lib.nlse_get_row_plan.argtypes = [_I, ctypes.POINTER(_I), ctypes.POINTER(_I)]
    lib.nlse_set_row_plan.argtypes = [_I, _I, _I]
    lib.nlse_batch_create.argtypes = [ctypes.POINTER(GridDesc), _I, ctypes.POINTER(_P)]
    lib.nlse_batch_propagate.argtypes = [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), _D, _I, _P]
    lib.nlse_batch_get_context.argtypes = [_P, _I, ctypes.POINTER(_P)]
    lib.nlse_batch_set_split_terms.argtypes = [_P, _I]
    lib.nlse_batch_set_mode.argtypes = [_P, _I]
    lib.nlse_batch_device_status.argtypes = [_P, ctypes.POINTER(_I)]
    lib.nlse_batch_get_last_error.argtypes = [_P, ctypes.c_char_p, ctypes.c_size_t]
    lib.nlse_batch_destroy.argtypes = [_P]
    lib.nlse_batch_destroy.restype = None
    for name in EXPORTS:
        if name not in ("nlse_destroy", "nlse_version", "nlse_kernel_name", "nlse_batch_destroy"):
            getattr(lib, name).restype = _I
    _lib = lib
    return lib


def row_plans(Nt):
    """(row_nl plan, row_next plan) picked for N_t on the current device (-1: not tuned yet)."""
    lib = load()
    a, b = _I(-1), _I(-1)
    if lib.nlse_get_row_plan(int(Nt), ctypes.byref(a), ctypes.byref(b)) != NLSE_OK:
        raise ValueError(f"Nt={Nt} is not a power of two in [16, 8192]")
    return a.value, b.value


def set_row_plans(Nt, nl_plan, next_plan):
    """Pin the row plans for N_t on the current device (-1: tune again at the next context)."""
    if load().nlse_set_row_plan(int(Nt), int(nl_plan), int(next_plan)) != NLSE_OK:
        raise ValueError((Nt, nl_plan, next_plan))


class NLSEError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libnlse status {status}: {msg}")
        self.status = status


def _check(lib, ctx, status):
    if status != NLSE_OK:
        buf = ctypes.create_string_buffer(512)
        lib.nlse_get_last_error(ctx, buf, 512)
        raise NLSEError(status, buf.value.decode(errors="replace"))


def physics_flags(cfg):
    f = 0
    if cfg.enable_kerr_instantaneous:
        f |= F_KERR_INSTANT
    if cfg.enable_photoionization_loss:
        f |= F_PHOTO_LOSS
    if cfg.enable_plasma_defocusing:
        f |= F_PLASMA_DEFOC
    if cfg.enable_plasma_absorption:
        f |= F_PLASMA_ABSORB
    if cfg.enable_kerr_raman:
        f |= F_KERR_RAMAN
    if cfg.enable_self_steepening:
        f |= F_SELF_STEEP
    if cfg.enable_space_time_focusing:
        f |= F_SPACE_TIME
    if cfg.enable_ste:
        f |= F_STE
    return f


def _arr(a, keep):
    a = np.ascontiguousarray(a, dtype=np.float64)
    keep.append(a)
    return a.ctypes.data


def make_desc(cfg, g):
    """Fill an nlse_grid_desc from a Config and its build_grids() dict.
    Returns (desc, keep-alive list)."""
    from scipy.constants import c, epsilon_0
    keep = []
    kel = g["keldysh"]
    sp = kel["f_spline"]
    Nr, Nt = g["Y"].shape[0], len(g["tlist"])
    d = GridDesc()
    d.Nr, d.Nt, d.flags = Nr, Nt, physics_flags(cfg)
    d.dt, d.komega = g["dt"], g["komega"]
    d.Y = _arr(g["Y"], keep)
    d.rho_modes = _arr(g["rholist"], keep)
    d.delta_k = _arr(g["delta_k"], keep)
    d.spec_mask = _arr(g["spec_mask"], keep)
    d.mask_r = _arr(g["mask_r"][:, 0], keep)
    Rk = g["R"] ** 2 / g["j1last"]
    iRk = g["j1last"] / g["R"] ** 2
    d.Rk_iRk = Rk * iRk
    d.invE2 = g["invE2"]
    d.kerr_pref = 3 * cfg.chi3 * cfg.omega0**2 / (8 * g["komega"] * c**2)
    d.kerr_scale = 1.0 - cfg.f_R
    d.plasma_pref = (g["sigmaomega"] / 2.0) * 100.0
    d.omega0_tau_c = cfg.omega0 * cfg.tau_c
    d.rho_max = cfg.rho_max
    d.photo_const = 1e6 * cfg.Ui / (cfg.n0 * c * epsilon_0)
    d.pchip_n = len(kel["I_knots"])
    d.pchip_x = _arr(kel["I_knots"], keep)
    d.pchip_c = _arr(sp.c, keep)
    d.lut_n = kel["NLUT"]
    d.lut = _arr(kel["W_LUT"], keep)
    d.lut_log_min, d.lut_inv_dlog = kel["logImin"], kel["inv_dlog"]
    d.lut_Imin, d.lut_Imax = kel["Imin"], kel["Imax"]
    d.beta_g = g["avalanche_coef"]
    d.inv_tau_r = g["inv_taur_eff"]
    if cfg.enable_ste:
        d.lut_s = _arr(kel["W_LUT_s"], keep)
        d.beta_s = g["avalanche_coef_s"]
        d.inv_tau_ste = g["inv_tau_ste"]
        d.ste_pref = g["ste_pref"]
    d.f_R = cfg.f_R
    if cfg.enable_kerr_raman:
        d.R_f = _arr(np.ascontiguousarray(np.asarray(g["R_f"], dtype=np.complex128)).view(np.float64), keep)
    if cfg.enable_self_steepening:
        d.T_op = _arr(g["T_op"], keep)
    if cfg.enable_space_time_focusing:
        d.inv_U_nl = _arr(g["inv_U_nl"], keep)
        d.inv_U_op = _arr(g["inv_U_op"], keep)
    return d, keep


class Context:
    """One libnlse context (tables + workspace on the current CUDA device).

    Methods take torch CUDA tensors: fields complex64 (Nr, Nt) C-contiguous,
    densities float32 (Nr, Nt).  Work is queued on torch's current stream."""

    def __init__(self, cfg=None, g=None, desc=None):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("rapport_gb300 needs a CUDA device (no CPU path exists)")
        self.lib = load()
        torch.cuda.init()
        if desc is None:
            desc, keep = make_desc(cfg, g)
        self.Nr, self.Nt = desc.Nr, desc.Nt
        h = _P()
        st = self.lib.nlse_create(ctypes.byref(desc), ctypes.byref(h))
        _check(self.lib, None, st)
        self.h = h
        self.device = torch.cuda.current_device()

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and not getattr(self, "_borrowed", False):
            try:
                self.lib.nlse_destroy(h)
            except Exception:
                pass
            self.h = None

    # ---------------------------------------------------------- checks
    def _stream(self):
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _field(self, t, name, dtype=None):
        import torch
        dtype = dtype or torch.complex64
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise TypeError(f"{name} must be a CUDA tensor")
        if t.dtype != dtype or tuple(t.shape) != (self.Nr, self.Nt) or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous {dtype} tensor of shape {(self.Nr, self.Nt)}, "
                             f"got {t.dtype} {tuple(t.shape)}")
        return ctypes.c_void_p(t.data_ptr())

    def _rho(self, t, name):
        import torch
        return self._field(t, name, torch.float32)

    # ---------------------------------------------------------- ops
    def half_linear(self, u, dz, mode=MODE_PLAIN_F32):
        _check(self.lib, self.h, self.lib.nlse_half_linear_ex(self.h, self._field(u, "u"), float(dz), int(mode),
                                                              self._stream()))

    def debug_operator_product(self, w, out, dz):
        """out = E' w (planar FP32, 2Nr x Nt) through the tensor-core product alone."""
        import torch
        for t, nm in ((w, "w"), (out, "out")):
            if t.dtype != torch.float32 or tuple(t.shape) != (2 * self.Nr, self.Nt) or not t.is_contiguous():
                raise ValueError(f"{nm} must be a contiguous float32 tensor of shape {(2 * self.Nr, self.Nt)}")
        _check(self.lib, self.h, self.lib.nlse_debug_operator_product(
            self.h, ctypes.c_void_p(w.data_ptr()), ctypes.c_void_p(out.data_ptr()), float(dz), self._stream()))

    def record(self, u, rho, rho_s, bin_of_t, nbins, out):
        """Per-radius plane diagnostics into out (float64 CUDA tensor, Nr x (6 + nbins))."""
        import torch
        if out.dtype != torch.float64 or tuple(out.shape) != (self.Nr, 6 + nbins) or not out.is_contiguous():
            raise ValueError("out must be a contiguous float64 CUDA tensor of shape (Nr, 6 + nbins)")
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        b = ctypes.c_void_p(bin_of_t.data_ptr()) if bin_of_t is not None else None
        _check(self.lib, self.h, self.lib.nlse_record(self.h, self._field(u, "u"), self._rho(rho, "rho"), rs, b,
                                                      int(nbins), ctypes.c_void_p(out.data_ptr()), self._stream()))

    def set_split_terms(self, n):
        _check(self.lib, self.h, self.lib.nlse_set_split_terms(self.h, int(n)))

    def set_gemm_variant(self, v):
        _check(self.lib, self.h, self.lib.nlse_set_gemm_variant(self.h, int(v)))

    def gemm_variant(self):
        return self.lib.nlse_get_gemm_variant(self.h)

    def device_status(self):
        w = _I(0)
        _check(self.lib, self.h, self.lib.nlse_device_status(self.h, ctypes.byref(w)))
        return w.value

    def debug_wait_timeout(self, limit_us):
        """Launch the failure-path probe: a device wait bounded by limit_us that
        runs out and raises the context's status bit (read by device_status)."""
        _check(self.lib, self.h, self.lib.nlse_debug_wait_timeout(self.h, int(limit_us), self._stream()))

    def split(self, u, rho, rhs, alpha, rho_s=None):
        a = self._rho(alpha, "alpha") if alpha is not None else None
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        _check(self.lib, self.h, self.lib.nlse_split(self.h, self._field(u, "u"), self._rho(rho, "rho"), rs,
                                                     self._field(rhs, "rhs"), a, self._stream()))

    def nonlinear_step(self, u, rho, dz, rho_s=None):
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        _check(self.lib, self.h, self.lib.nlse_nonlinear_step(self.h, self._field(u, "u"), self._rho(rho, "rho"),
                                                              rs, float(dz), self._stream()))

    def update_plasma(self, u, rho, rho_s=None):
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        _check(self.lib, self.h, self.lib.nlse_update_plasma(self.h, self._field(u, "u"), self._rho(rho, "rho"),
                                                             rs, self._stream()))

    def rate_equation(self, u, rho, rho_s=None):
        """The carrier march alone, from the t = 0 values already in rho / rho_s."""
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        _check(self.lib, self.h, self.lib.nlse_rate_equation(self.h, self._field(u, "u"), self._rho(rho, "rho"),
                                                             rs, self._stream()))

    def step(self, u, rho, dz, mode=MODE_PLAIN_F32, rho_s=None):
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        _check(self.lib, self.h, self.lib.nlse_step(self.h, self._field(u, "u"), self._rho(rho, "rho"), rs,
                                                    float(dz), int(mode), self._stream()))

    def propagate(self, u, rho, rho_s, dz, nsteps, mode=MODE_PLAIN_F32):
        rs = self._rho(rho_s, "rho_s") if rho_s is not None else None
        _check(self.lib, self.h, self.lib.nlse_propagate(self.h, self._field(u, "u"), self._rho(rho, "rho"), rs,
                                                         float(dz), int(nsteps), int(mode), self._stream()))

    def step_batched(self, pulses, dz, nsteps, mode=MODE_PLAIN_F32):
        """pulses: [(u, rho, rho_s or None)] on this context's grid; each advances
        nsteps iterations of update_plasma + step."""
        arr = (PulseDesc * len(pulses))()
        for i, (u, rho, rs) in enumerate(pulses):
            arr[i].u = self._field(u, "u")
            arr[i].rho = self._rho(rho, "rho")
            arr[i].rho_s = self._rho(rs, "rho_s") if rs is not None else None
            arr[i].dz, arr[i].nsteps, arr[i].mode = float(dz), int(nsteps), int(mode)
        _check(self.lib, self.h, self.lib.nlse_step_batched(self.h, arr, len(pulses), self._stream()))

    def profile_start(self, capacity):
        _check(self.lib, self.h, self.lib.nlse_profile_start(self.h, int(capacity)))

    def profile_read(self, nkinds=16):
        """-> {kernel name: (launches, total ms)} of the records since profile_start."""
        L = (_I * nkinds)()
        T = (_D * nkinds)()
        _check(self.lib, self.h, self.lib.nlse_profile_read(self.h, L, T, nkinds, None))
        out = {}
        for k in range(nkinds):
            if L[k]:
                out[self.lib.nlse_kernel_name(k).decode()] = (L[k], T[k])
        return out

    def scan_fallback_rows(self):
        v = _I(0)
        _check(self.lib, self.h, self.lib.nlse_scan_fallback_rows(self.h, ctypes.byref(v)))
        return v.value


class Batch:
    """Many pulses (each its own Config / grid) advanced together in the split-BF16
    form: nlse_batch_create / nlse_batch_propagate."""

    def __init__(self, cfgs, grids):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("rapport_gb300 needs a CUDA device (no CPU path exists)")
        self.lib = load()
        torch.cuda.init()
        descs = (GridDesc * len(cfgs))()
        self._keep = []
        self.shapes = []
        for i, (c, g) in enumerate(zip(cfgs, grids)):
            d, keep = make_desc(c, g)
            descs[i] = d
            self._keep.append(keep)
            self.shapes.append((d.Nr, d.Nt))
        h = _P()
        st = self.lib.nlse_batch_create(descs, len(cfgs), ctypes.byref(h))
        if st != NLSE_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.nlse_batch_get_last_error(None, buf, 512)
            raise NLSEError(st, buf.value.decode(errors="replace"))
        self.h = h
        self.n = len(cfgs)

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                self.lib.nlse_batch_destroy(h)
            except Exception:
                pass
            self.h = None

    def _ptrs(self, ts, dtype, name, allow_none=False):
        import torch
        arr = (_P * self.n)()
        for i, t in enumerate(ts):
            if t is None and allow_none:
                arr[i] = None
                continue
            if t.dtype != dtype or tuple(t.shape) != self.shapes[i] or not t.is_contiguous() or not t.is_cuda:
                raise ValueError(f"{name}[{i}] must be a contiguous CUDA {dtype} tensor of shape {self.shapes[i]}")
            arr[i] = t.data_ptr()
        return arr

    def propagate(self, us, rhos, rho_ss, dz, nsteps):
        import torch
        u = self._ptrs(us, torch.complex64, "u")
        r = self._ptrs(rhos, torch.float32, "rho")
        s = self._ptrs(rho_ss, torch.float32, "rho_s", allow_none=True) if rho_ss is not None else None
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        status = self.lib.nlse_batch_propagate(self.h, u, r, s, float(dz), int(nsteps), st)
        if status != NLSE_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.nlse_batch_get_last_error(self.h, buf, 512)
            raise NLSEError(status, buf.value.decode(errors="replace"))

    def set_split_terms(self, n):
        _check(self.lib, None, self.lib.nlse_batch_set_split_terms(self.h, int(n)))

    def set_mode(self, mode):
        """MODE_SPLIT_BF16 (default) or MODE_SPLIT_F16."""
        _check(self.lib, None, self.lib.nlse_batch_set_mode(self.h, int(mode)))

    def device_status(self):
        """The status word of the batch's bounded waits (0: none gave up);
        raises NLSEError when a wait gave up or a pulse's own device flags
        report an error (e.g. a split-FP16 overflow)."""
        w = _I(0)
        status = self.lib.nlse_batch_device_status(self.h, ctypes.byref(w))
        if status != NLSE_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.nlse_batch_get_last_error(self.h, buf, 512)
            raise NLSEError(status, buf.value.decode(errors="replace"))
        return w.value

    def context(self, i):
        """Pulse i's context (owned by the batch: valid while the batch lives).
        Its single-pulse operations (record, update_plasma, ...) act on that
        pulse's grid and tables."""
        if not 0 <= i < self.n:
            raise IndexError(i)
        c = _P()
        _check(self.lib, None, self.lib.nlse_batch_get_context(self.h, int(i), ctypes.byref(c)))
        ctx = Context.__new__(Context)
        ctx.lib, ctx.h, ctx.Nr, ctx.Nt = self.lib, c, self.shapes[i][0], self.shapes[i][1]
        ctx._borrowed = True
        ctx._owner = self
        return ctx

    def context_profile(self):
        """The first pulse's context (the batch records its launches there)."""
        return self.context(0)
