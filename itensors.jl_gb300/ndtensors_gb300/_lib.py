"""ctypes binding of libndtensors_gb300.so (the C ABI in include/ndtensors_gb300.h).

The library is loaded from this directory.  There is no CPU fallback: if the
shared library is missing or no CUDA device is visible, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
import atexit
import weakref
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libndtensors_gb300.so"

ND_OK, ND_ERR_ARG, ND_ERR_OOM, ND_ERR_NOCONV, ND_ERR_TIMEOUT, ND_ERR_CUDA, ND_ERR_UNSUPPORTED, ND_ERR_NONFINITE = range(8)
STATUS_NAMES = {0: "OK", 1: "ARG", 2: "OOM", 3: "NOCONV", 4: "TIMEOUT", 5: "CUDA", 6: "UNSUPPORTED",
                7: "NONFINITE"}
PRECISIONS = {"fp64": 0, "ozaki": 1, "bf16x3": 2}
MAX_RANK = 8


class NDError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[ND_ERR_{STATUS_NAMES.get(status, status)}] {msg}")
        self.status = status


class NoConvergence(NDError):
    pass


class BlockCopy(C.Structure):
    _fields_ = [("src_off", C.c_int64), ("dst_off", C.c_int64), ("rank", C.c_int32),
                ("dims", C.c_int64 * MAX_RANK), ("src_strides", C.c_int64 * MAX_RANK),
                ("dst_strides", C.c_int64 * MAX_RANK)]


class BsDesc(C.Structure):
    _fields_ = [("rank", C.c_int32), ("nblocks", C.POINTER(C.c_int32)), ("blockdims", C.POINTER(C.c_int64)),
                ("nnzblocks", C.c_int32), ("blocks", C.POINTER(C.c_int32)), ("offsets", C.POINTER(C.c_int64))]


_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64
_D = C.c_double
_PI32 = C.POINTER(C.c_int32)
_PI64 = C.POINTER(C.c_int64)
_PD = C.POINTER(C.c_double)

# name -> argtypes (restype is always int32 status unless listed in _RESTYPE)
SIGNATURES = {
    "nd_create": [_I32, C.POINTER(_P)],
    "nd_destroy": [_P],
    "nd_last_error": [_P],
    "nd_set_stream": [_P, _P],
    "nd_get_stream": [_P, C.POINTER(_P)],
    "nd_sync": [_P],
    "nd_alloc": [_P, C.c_size_t, C.POINTER(_P)],
    "nd_free": [_P, _P],
    "nd_h2d": [_P, _P, _P, C.c_size_t],
    "nd_d2h": [_P, _P, _P, C.c_size_t],
    "nd_memset0": [_P, _P, C.c_size_t],
    "nd_set_ozaki_slices": [_P, _I32],
    "nd_set_split_tile": [_P, _I32],
    "nd_set_plan_placement": [_P, _I32],
    "nd_set_permute_path": [_P, _I32],
    "nd_set_verify": [_P, _I32],
    "nd_verify_last": [_P, _PD],
    "nd_set_spin_limit": [_P, C.c_uint32],
    "nd_set_svd_max_sweeps": [_P, _I32],
    "nd_svd_last_info": [_P, _P, _I32, _P, _I32],
    "nd_block_copy_plan_create": [_P, _I32, _P, _P],
    "nd_block_copy_plan_run": [_P, _P, _P],
    "nd_block_copy_plan_destroy": [_P],
    "nd_tridiag_lowest_f64": [_P, _I32, _P, _P, _P, _P],
    "nd_bs_svd_plan_create": [_P, _I32, _P, _P, _P],
    "nd_bs_svd_plan_exec": [_P, _P, _P, _P, _P, _P, _I32, _I32, _D, _I32, _I32, _I32, _P, _P, _P, _P, _P],
    "nd_bs_svd_plan_destroy": [_P],
    "nd_set_cta_timing": [_P, _I32],
    "nd_cta_times_read": [_P, _P, _P, _P],
    "nd_launch_count": [_P, _PI64],
    "nd_profile_enable": [_P, _I32],
    "nd_profile_read": [_P, _I32, C.c_char_p, _PI64, _PD, _PI32],
    "nd_tune_enable": [_P, _I32],
    "nd_tune_count": [_P, _PI32],
    "nd_tune_save": [_P, C.c_char_p],
    "nd_tune_load": [_P, C.c_char_p],
    "nd_permutedims_f64": [_P, _P, _P, _I32, _PI64, _PI32, _D, _D],
    "nd_contract_dense_f64": [_P, _P, _I32, _PI64, _PI32, _P, _I32, _PI64, _PI32, _P, _I32, _PI64, _PI32,
                              _D, _D, _I32],
    "nd_contract_dense_ozaki_noalloc_f64": [_P, _P, _I32, _PI64, _PI32, _P, _I32, _PI64, _PI32, _P, _I32, _PI64,
                                            _PI32, _D, _D],
    "nd_bs_plan_create": [_P, C.POINTER(BsDesc), _PI32, C.POINTER(BsDesc), _PI32, _I32, _PI32, C.POINTER(_P)],
    "nd_bs_plan_sizes": [_P, _PI32, _PI32, _PI64],
    "nd_bs_plan_get": [_P, _PI32, _PI64, _PI32],
    "nd_bs_plan_destroy": [_P],
    "nd_bs_plan_set_output_offsets": [_P, _PI64],
    "nd_bs_contract_f64": [_P, _P, _P, _P, _P, _D, _I32],
    "nd_bs_contract_adjoint_f64": [_P, _P, _P, _P, _P, _P, _P, _I32],
    "nd_bs_contract_diag_f64": [_P, _P, _P, _P, _P, _PI64, _D],
    "nd_bs_permutedims_f64": [_P, C.POINTER(BsDesc), _P, _PI32, _PI64, _P],
    "nd_bs_svd_f64": [_P, _I32, _PI64, _PI64, _PI64, _P, _P, _P, _P, _I32, _I32, _D, _I32, _I32, _I32,
                      _PI32, _PD, _PI32, _PD, _PD],
    "nd_bs_qr_f64": [_P, _I32, _PI64, _PI64, _PI64, _P, _P, _P, _I32],
    "nd_bs_eigen_f64": [_P, _I32, _PI64, _PI64, _P, _P, _P, _I32, _I32, _D, _I32, _I32, _I32, _PI32, _PD, _PI32,
                        _PD, _PD],
    "nd_truncate_f64": [_P, _P, _I32, _I32, _I32, _D, _I32, _I32, _PI32, _PD, _PD],
    "nd_block_copy_f64": [_P, _I32, C.POINTER(BlockCopy), _P, _P],
    "nd_vec_inner_f64": [_P, _I64, _P, _P, _P],
    "nd_vec_norm_f64": [_P, _I64, _P, _P],
    "nd_vec_scale_f64": [_P, _I64, _P, _P, _D, _P, _I32],
    "nd_vec_add_f64": [_P, _I64, _P, _P, _D, _D],
    "nd_vec_dots_f64": [_P, _I64, _I32, _P, _I64, _P, _P],
    "nd_vec_update_f64": [_P, _I64, _I32, _P, _I64, _P, _D, _P],
    "nd_graph_begin": [_P],
    "nd_graph_end": [_P, C.POINTER(_P)],
    "nd_graph_launch": [_P, _P],
    "nd_graph_destroy": [_P],
}
_RESTYPE = {"nd_last_error": C.c_char_p}

_lib = None
_lock = threading.Lock()
_shutting_down = False
_live_plans = weakref.WeakSet()


@atexit.register
def _teardown():
    """Destroy plans before handles, before the CUDA runtime unloads."""
    global _shutting_down
    for p in list(_live_plans):
        try:
            p.destroy()
        except Exception:
            pass
    for h in list(_handles.values()):
        try:
            h.close()
        except Exception:
            pass
    _handles.clear()
    _shutting_down = True


def load():
    """Load the shared library (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"{LIB_PATH} is missing: build it with itensors.jl_gb300/build.py "
                                   "(there is no CPU fallback)")
            lib = C.CDLL(str(LIB_PATH))
            for name, args in SIGNATURES.items():
                f = getattr(lib, name)
                f.argtypes = args
                f.restype = _RESTYPE.get(name, C.c_int32)
            _lib = lib
    return _lib


def exported_symbols():
    return sorted(SIGNATURES)


class Handle:
    """An nd_handle bound to one CUDA device, driven on torch's current stream."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.ptr = _P()
        self._check(self.lib.nd_create(device, C.byref(self.ptr)), ctx=False)
        self.device = device

    def _check(self, status, ctx=True):
        if status != ND_OK:
            msg = self.lib.nd_last_error(self.ptr if ctx else None)
            msg = msg.decode() if msg else ""
            if status == ND_ERR_NOCONV:
                raise NoConvergence(status, msg)
            raise NDError(status, msg)

    def call(self, name, *args):
        self._check(getattr(self.lib, name)(self.ptr, *args))

    def use_stream(self, stream_ptr):
        self._check(self.lib.nd_set_stream(self.ptr, _P(stream_ptr)))

    def sync(self):
        self._check(self.lib.nd_sync(self.ptr))

    def profile(self, enable=True):
        self._check(self.lib.nd_profile_enable(self.ptr, 1 if enable else 0))

    def profile_read(self):
        """{kernel name: (launches, total ms)} since the last read; synchronises."""
        cap = 64
        names = C.create_string_buffer(64 * cap)
        counts = (C.c_int64 * cap)()
        tot = (C.c_double * cap)()
        n = C.c_int32()
        self._check(self.lib.nd_profile_read(self.ptr, cap, names, counts, tot, C.byref(n)))
        out = {}
        for k in range(min(n.value, cap)):
            nm = names.raw[64 * k:64 * k + 64].split(b"\0", 1)[0].decode()
            out[nm] = (counts[k], tot[k])
        return out

    def tune(self, enable=True):
        """Autotune the execution parameters of contractions built from now on (cached per
        block-size histogram)."""
        self._check(self.lib.nd_tune_enable(self.ptr, 1 if enable else 0))

    def tune_count(self):
        n = C.c_int32()
        self._check(self.lib.nd_tune_count(self.ptr, C.byref(n)))
        return n.value

    def tune_save(self, path):
        self._check(self.lib.nd_tune_save(self.ptr, os.fsencode(str(path))))

    def tune_load(self, path):
        self._check(self.lib.nd_tune_load(self.ptr, os.fsencode(str(path))))

    def verify(self, enable=True):
        """Verify mode: split-precision contractions are recomputed in FP64 and the relative
        Frobenius distance of the two results is recorded (read it with verify_last)."""
        self._check(self.lib.nd_set_verify(self.ptr, 1 if enable else 0))

    def verify_last(self):
        """The relative error of the last verified contraction (0 for FP64, -1 if none)."""
        v = C.c_double()
        self._check(self.lib.nd_verify_last(self.ptr, C.byref(v)))
        return v.value

    def launches(self):
        c = C.c_int64()
        self._check(self.lib.nd_launch_count(self.ptr, C.byref(c)))
        return c.value

    def close(self):
        if self.ptr:
            self.lib.nd_destroy(self.ptr)
            self.ptr = _P()

    def __del__(self):
        if _shutting_down:
            return
        try:
            self.close()
        except Exception:
            pass


_handles = {}


def _current_stream_ptr(device):
    import torch
    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:
        return raw(device)
    return torch.cuda.current_stream(device).cuda_stream


def handle(device: int = 0) -> Handle:
    """Per-device default handle, bound to torch's current CUDA stream."""
    h = _handles.get(device)
    if h is None:
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("ndtensors_gb300 needs a CUDA device (no CPU fallback)")
        h = Handle(device)
        _handles[device] = h
        h._stream = None
    s = _current_stream_ptr(device)
    if s != h._stream:
        h.use_stream(s)
        h._stream = s
    return h


def i64arr(xs):
    xs = list(xs)
    return (C.c_int64 * max(1, len(xs)))(*xs)


def i32arr(xs):
    xs = list(xs)
    return (C.c_int32 * max(1, len(xs)))(*xs)
