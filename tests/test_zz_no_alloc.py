"""CUDA_EonDevice_noalloc: the energy entry point for callers that cannot allocate.

Hosts that run inside another framework's device-memory pool, under a fixed memory
budget, or in a loop that must not allocate, call this variant instead of
CUDA_EonDevice; it uses a static device array as scratch.  Its result must equal
CUDA_EonDevice's on the same inputs, call after call.  This file is collected last
so that a failure here leaves every other test already run; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

import cgppd_gb300
import oracle
from helpers import device_array, ptr

pytestmark = pytest.mark.gpu
REL = 1e-5  # the GPU energy tolerance used throughout the tests


@pytest.fixture(scope="module")
def L(refdata):
    import torch
    assert torch.cuda.is_available()
    cgppd_gb300.build()
    L = cgppd_gb300.lib()
    L.CUDA_EonDevice_noalloc.restype = None
    L.CUDA_EonDevice_noalloc.argtypes = [ctypes.c_void_p] * 6 + [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                                                  ctypes.c_int, ctypes.c_int]
    a = L.cgppd_aminoacids_create()
    t = np.ascontiguousarray(np.array(refdata["lj_table"], np.float32).reshape(-1))
    L.cgppd_aminoacids_set_table(a, t.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    dev = L.LJPotentialDataToDevice(a)
    L.bindLJTexture(dev)
    cgppd_gb300.check("setup")
    yield L
    L.unbindLJTexture()
    L.cgppd_aminoacids_destroy(a)


def energies(L, pos, meta, box):
    L.CUDA_setBoxDimension(box)
    dp, dm = device_array(pos), device_array(meta)
    out = []
    for fn in (L.CUDA_EonDevice, L.CUDA_EonDevice_noalloc, L.CUDA_EonDevice_noalloc):
        res = ctypes.c_double(0.0)
        fn(ptr(dp), ptr(dm), None, None, None, None, ctypes.byref(res), 32, pos.shape[0], 0)
        cgppd_gb300.check(fn.__name__)
        out.append(res.value)
    return out


def test_noalloc_matches_cuda_eondevice_twice(L, refdata):
    for i in (1, 3, 8):
        mols = oracle.build_replica(["conf%d/1a" % i, "conf%d/1b" % i], refdata, 1000.0)
        pos, meta = oracle.pack_replica(mols, 32)
        ref, first, second = energies(L, pos, meta, 1000.0)
        assert abs(first - ref) <= REL * abs(ref) + 1e-12
        assert abs(second - ref) <= REL * abs(ref) + 1e-12


def test_noalloc_large_system_and_limit(L, refdata):
    rng = np.random.default_rng(7)
    n = 6000
    P = -(-n // 32) * 32
    pos = np.zeros((P, 4), np.float32)
    meta = np.zeros((P, 4), np.float32)
    pos[:n, :3] = rng.uniform(0, 200.0, (n, 3))
    pos[:n, 3] = 1.0 + np.arange(n) // 300          # rigid domain per 300 residues
    meta[:n] = np.stack([rng.integers(0, 20, n), rng.choice([-1.0, 0.0, 1.0], n), rng.uniform(4.5, 7, n),
                         np.arange(n) // 300 + 0.25], 1)
    pos[n:, 3] = -2.0
    meta[n:, 0] = 20.0
    ref, first, second = energies(L, pos, meta, 200.0)
    assert abs(first - ref) <= REL * abs(ref) + 1e-12
    assert abs(second - ref) <= REL * abs(ref) + 1e-12
    # above the static scratch's limit the call is refused, not run
    big = np.zeros((16416, 4), np.float32)
    res = ctypes.c_double(3.0)
    L.CUDA_EonDevice_noalloc(None, None, None, None, None, None, ctypes.byref(res), 32, 16416, 0)
    assert res.value == 0.0
    with pytest.raises(cgppd_gb300.CgppdError):
        cgppd_gb300.check("over the limit")
    del big
