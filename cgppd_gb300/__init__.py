"""cgppd_gb300 -- GB300-native replica-exchange Monte Carlo energy engine for CGPPD.

The product is the native library ``_lib/libcgppd_gb300.so`` (C++ host code and
sm_103a CUDA kernels behind a C ABI, declared in ``include/*.h``).  This module only
loads it with ctypes and declares the argument types, for the tests and the
benchmark.  There is no Python or CPU fallback: importing fails loudly when the
library has not been built.
"""
import ctypes
import os

from .build import LIB, build  # noqa: F401

_lib = None

c_int, c_float, c_double, c_void_p, c_char_p, c_size_t = (
    ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t)
P = ctypes.POINTER

# name: (restype, [argtypes])
_SIGNATURES = {
    # drop-in C ABI (include/cgppd_cuda_functions.h)
    "__throwLastCudaError": (None, [c_char_p, c_char_p, c_int]),
    "LJPotentialDataToDevice": (c_void_p, [c_void_p]),
    "copyLJPotentialDataToDevice": (None, [c_void_p, c_void_p]),
    "bindLJTexture": (None, [c_void_p]),
    "unbindLJTexture": (None, []),
    "CUDA_setBoxDimension": (None, [c_float]),
    "CUDA_freeBoxDimension": (None, []),
    "CUDA_EonDevice": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, P(c_double),
                              c_int, c_int, c_int]),
    "CUDA_EonDeviceNC": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, P(c_double),
                                c_int, c_int, c_int]),
    "CUDA_EonDevice_async": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_int, c_int, c_int, c_int, c_void_p]),
    "cgppd_last_energy_components": (c_int, [P(c_double)]),
    "cgppd_set_repulsive_crowding": (c_int, [c_int]),
    "cgppd_get_last_error": (c_int, [c_char_p, c_int]),
    # residue-type tables (include/cgppd_amino_acids.h)
    "cgppd_aminoacids_create": (c_void_p, []),
    "cgppd_aminoacids_destroy": (None, [c_void_p]),
    "cgppd_aminoacids_load": (c_int, [c_void_p, c_char_p, c_char_p]),
    "cgppd_aminoacids_set": (None, [c_void_p, c_int, c_char_p, c_char_p, ctypes.c_char, c_float, c_float]),
    "cgppd_aminoacids_set_table": (None, [c_void_p, P(c_float)]),
    "cgppd_aminoacids_get_table": (None, [c_void_p, P(c_float)]),
    "cgppd_aminoacids_index": (c_int, [c_void_p, c_char_p]),
    "cgppd_aminoacids_lj_offset": (c_size_t, []),
    "cgppd_aminoacids_sizeof": (c_size_t, []),
}


class CgppdError(RuntimeError):
    pass


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise CgppdError("native library %s is missing: run cgppd_gb300.build() (or "
                             "__graft_entry__.build()) first; there is no fallback" % LIB)
        L = ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGNATURES)


def check(where=""):
    """Raise CgppdError if the library recorded an error on this thread."""
    buf = ctypes.create_string_buffer(512)
    code = lib().cgppd_get_last_error(buf, 512)
    if code != 0:
        raise CgppdError("%s%s (code %d)" % (where + ": " if where else "", buf.value.decode(errors="replace"), code))
