"""ctypes binding of ``librascil_gb300.so`` (the C-ABI in
``include/rascil_gb300.h``).

There is no CPU fallback: if the library is missing or a call fails, a
Python exception is raised.  Status codes map to exceptions the way the
reference's GPU sibling reports errors (``ValueError`` for bad arguments,
``rascil/processing_components/imaging/wg.py:52-54,79-85``) and
``RuntimeError`` otherwise.
"""

import ctypes
import os
import threading

from . import build as _build

GB_OK = 0
GB_ERR_INVALID_ARG = 1
GB_ERR_NOT_BOUND = 2
GB_ERR_WORKSPACE = 3
GB_ERR_CUDA = 4
GB_ERR_CUFFT = 5
GB_ERR_TIMEOUT = 6
GB_ERR_INTERNAL = 7
GB_ERR_OUT_OF_GRID = 8
GB_WEIGHT_NATURAL, GB_WEIGHT_UNIFORM, GB_WEIGHT_ROBUST = 0, 1, 2

GB_FP32 = 0
GB_FP64 = 1
GB_LAYOUT_XY = 0
GB_LAYOUT_YX = 1
GB_FLAGS_NONE = 0
GB_FLAGS_U8 = 1
GB_FLAGS_I64 = 2

# Every symbol the header declares, with its ctypes signature.
_c = ctypes
_vp = _c.c_void_p
_dp = _c.POINTER(_c.c_double)


class PlanParams(_c.Structure):
    _fields_ = [
        ("nrows", _c.c_int64),
        ("nchan", _c.c_int32),
        ("npol", _c.c_int32),
        ("npix_x", _c.c_int32),
        ("npix_y", _c.c_int32),
        ("pixsize_x", _c.c_double),
        ("pixsize_y", _c.c_double),
        ("epsilon", _c.c_double),
        ("do_wstacking", _c.c_int32),
        ("precision", _c.c_int32),
        ("sigma", _c.c_double),
        ("support", _c.c_int32),
        ("tile", _c.c_int32),
        ("slab", _c.c_int32),
        ("grid_budget_bytes", _c.c_int64),
        ("fft_mode", _c.c_int32),
        ("phase_shift", _c.c_double * 3),
        ("planes_per_batch", _c.c_int32),
    ]


class PlanInfo(_c.Structure):
    _fields_ = [
        ("support", _c.c_int32),
        ("ngrid_x", _c.c_int32),
        ("ngrid_y", _c.c_int32),
        ("nplanes", _c.c_int32),
        ("planes_per_batch", _c.c_int32),
        ("tile", _c.c_int32),
        ("slab", _c.c_int32),
        ("beta", _c.c_double),
        ("sigma", _c.c_double),
        ("dw", _c.c_double),
        ("w_lo", _c.c_double),
        ("w_hi", _c.c_double),
        ("tc", _c.c_double),
        ("nitems", _c.c_int64),
        ("nbuckets", _c.c_int64),
        ("workspace_bytes", _c.c_int64),
        ("fft_mode", _c.c_int32),
        ("own_rows", _c.c_int32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BatchItem(_c.Structure):
    """gb_batch_item: one solve's arguments in gb_batch_run_items."""
    _fields_ = [
        ("vis", _vp),
        ("npol_vis", _c.c_int32),
        ("psf", _c.c_int32),
        ("wgt", _vp),
        ("flags", _vp),
        ("flags_type", _c.c_int32),
        ("pad0", _c.c_int32),
        ("polmat_in", _dp),
        ("dirty", _vp),
        ("sumwt", _vp),
        ("model", _vp),
        ("polmat_out", _dp),
        ("npol_out", _c.c_int32),
        ("pad1", _c.c_int32),
        ("pred", _vp),
    ]


SIGNATURES = {
    "gb_plan_geometry": (_c.c_int, [_c.POINTER(PlanParams), _c.c_double, _c.c_double,
                                    _c.POINTER(PlanInfo)]),
    "gb_plan_create": (_c.c_int, [_c.POINTER(PlanParams), _vp, _vp, _vp, _c.POINTER(_vp)]),
    "gb_plan_workspace_size": (_c.c_int, [_vp, _c.POINTER(_c.c_size_t)]),
    "gb_plan_bind": (_c.c_int, [_vp, _vp, _c.c_size_t, _vp]),
    "gb_plan_info_get": (_c.c_int, [_vp, _c.POINTER(PlanInfo)]),
    "gb_plan_destroy": (_c.c_int, [_vp]),
    "gb_weight_visibility": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _c.c_int32, _vp,
                                        _c.c_int32, _c.c_int32, _c.c_int32, _c.c_double,
                                        _c.c_double, _vp, _vp, _vp, _c.c_int32, _c.c_int32,
                                        _c.c_double, _vp, _vp, _vp, _vp, _vp]),
    "gb_plan_device_status": (_c.c_int, [_vp, _vp, _c.POINTER(_c.c_int32)]),
    "gb_batch_run": (_c.c_int, [_vp, _c.c_int32, _vp, _vp, _vp, _c.c_int32, _vp, _vp, _vp,
                                _vp, _c.c_int32]),
    "gb_batch_run_items": (_c.c_int, [_vp, _c.POINTER(BatchItem), _c.c_int32, _vp, _vp, _vp,
                                      _c.c_int32, _c.c_int32]),
    "gb_phase_rotate": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _c.c_int32, _vp,
                                   _c.c_int32, _c.c_double, _c.c_double, _c.c_double,
                                   _c.c_int32, _vp]),
    "gb_plan_export_items": (_c.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gb_plan_ms2dirty": (_c.c_int, [_vp, _vp, _c.c_int32, _vp, _vp, _c.c_int32, _dp,
                                    _c.c_int32, _vp, _c.c_int32, _vp, _vp]),
    "gb_plan_dirty2ms": (_c.c_int, [_vp, _vp, _c.c_int32, _vp, _dp, _c.c_int32, _vp, _vp]),
    "gb_ms2dirty": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _vp, _vp, _c.c_int32,
                               _c.c_int32, _c.c_double, _c.c_double, _c.c_double,
                               _c.c_int32, _c.c_int32, _vp, _vp]),
    "gb_dirty2ms": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _vp, _vp, _c.c_int32,
                               _c.c_int32, _c.c_double, _c.c_double, _c.c_double,
                               _c.c_int32, _c.c_int32, _vp, _vp]),
    "gb_dft_components": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _vp, _vp, _c.c_int32,
                                     _c.c_int32, _vp, _c.c_int32, _c.c_int32, _vp]),
    "gb_dft_pixels": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _c.c_int32, _c.c_int32, _vp,
                                 _c.c_int32, _vp, _vp, _c.c_int32, _c.c_int32, _c.c_int32,
                                 _c.c_double, _c.c_double, _c.c_int32, _c.c_int32, _vp, _vp]),
    "gb_profile_enable": (_c.c_int, [_c.c_int32]),
    "gb_profile_reset": (_c.c_int, []),
    "gb_profile_count": (_c.c_int, []),
    "gb_profile_get": (_c.c_int, [_c.c_int32, _c.c_char_p, _c.c_int32, _dp,
                                  _c.POINTER(_c.c_int64), _dp]),
    "gb_profile_updates": (_c.c_int, [_c.c_int32, _dp]),
    "gb_probe_smem_peaks": (_c.c_int, [_dp, _dp, _vp]),
    "gb_apply_gains": (_c.c_int, [_vp, _vp, _vp, _vp, _c.c_int64, _c.c_int32, _c.c_int32,
                                  _c.c_int32, _vp, _vp]),
    "gb_gain_gradient": (_c.c_int, [_vp, _vp, _vp, _vp, _vp, _c.c_int64, _c.c_int32, _c.c_int32,
                                    _c.c_int32, _c.c_int32, _vp, _vp]),
    "gb_wrange_noalloc": (_c.c_int, [_vp, _vp, _c.c_int64, _c.c_int32, _vp, _vp]),
    "gb_last_error_string": (_c.c_char_p, []),
    "gb_version": (_c.c_char_p, []),
}

_lock = threading.Lock()
_lib = None


class GridderError(RuntimeError):
    """A non-argument failure reported by the C-ABI."""


class OutOfGridError(ValueError, AssertionError):
    """A sample's uv cell lies outside the weighting grid (the reference
    asserts there, so this is also an AssertionError)."""


def load(build_if_missing=True):
    """Load (building first if needed) the shared library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise ImportError("rascil_gb300 CUDA library not built: %s" % path)
        lib = ctypes.CDLL(path)
        for name, (restype, argtypes) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
        return lib


def check(status, what=""):
    """Raise the Python exception matching a gb_status."""
    if status == GB_OK:
        return
    msg = load().gb_last_error_string().decode(errors="replace")
    text = "%s: %s" % (what, msg) if what else msg
    if status == GB_ERR_INVALID_ARG:
        raise ValueError(text)
    if status == GB_ERR_OUT_OF_GRID:
        raise OutOfGridError(text)
    raise GridderError("status %d: %s" % (status, text))


def profile_enable(on=True):
    load().gb_profile_enable(1 if on else 0)


def profile_reset():
    load().gb_profile_reset()


def profile_read():
    """{kernel: {"ms": total device ms, "launches": n, "bytes": algorithmic bytes}}"""
    lib = load()
    out = {}
    for i in range(lib.gb_profile_count()):
        name = ctypes.create_string_buffer(64)
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        b = ctypes.c_double()
        check(lib.gb_profile_get(i, name, 64, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(b)))
        u = ctypes.c_double()
        check(lib.gb_profile_updates(i, ctypes.byref(u)))
        if n.value:
            out[name.value.decode()] = {"ms": ms.value, "launches": n.value, "bytes": b.value,
                                        "updates": u.value}
    return out


def smem_peaks(stream=None):
    """Measured (conflict-free 32-bit shared atomic adds per second,
    conflict-free 8-byte shared loads per second) of the current GPU."""
    a, l = ctypes.c_double(), ctypes.c_double()
    check(load().gb_probe_smem_peaks(ctypes.byref(a), ctypes.byref(l), stream),
          "gb_probe_smem_peaks")
    return a.value, l.value
