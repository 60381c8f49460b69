"""The reference's CUDA DFT kernel, built from the reference tree for a same-GPU
comparison (test infrastructure only; see make_ref_dft.py)."""
import ctypes
import os

from . import make_ref_dft

_lib = [None]


def available():
    return os.path.exists(make_ref_dft.KERNEL)


def load():
    if _lib[0] is None:
        path = make_ref_dft.build()
        if path is None:
            raise FileNotFoundError("reference DFT kernel source not extracted")
        lib = ctypes.CDLL(path)
        lib.ref_dft_launch.restype = ctypes.c_int
        lib.ref_dft_launch.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 5
        _lib[0] = lib
    return _lib[0]


def run(dirs, fluxes, uvw_lambda, vis, stream=None):
    """Launch dft_kernel on device tensors: dirs [ncomp, 3] f64, fluxes [ncomp,
    nchan, npol] c128, uvw_lambda [ntimes, nbl, nchan, 3] f64, vis [ntimes, nbl,
    nchan, npol] c128 (written)."""
    ncomp, nchan, npol = fluxes.shape
    ntimes, nbl = uvw_lambda.shape[:2]
    rc = load().ref_dft_launch(ncomp, npol, nchan, nbl, ntimes,
                               ctypes.c_void_p(dirs.data_ptr()),
                               ctypes.c_void_p(fluxes.data_ptr()),
                               ctypes.c_void_p(uvw_lambda.data_ptr()),
                               ctypes.c_void_p(vis.data_ptr()), stream)
    if rc != 0:
        raise RuntimeError("reference dft_kernel launch failed (%d)" % rc)
