"""CUDA_EonDevice_noalloc: the energy entry point for callers that cannot allocate.

Hosts that run inside another framework's device-memory pool, under a fixed memory
budget, or in a loop that must not allocate, call this variant instead of
CUDA_EonDevice; it uses a static device array as scratch.  Its result must equal
CUDA_EonDevice's on the same inputs, call after call, and both must be within 1e-5 of
the FP64 oracle.  The largest accepted size (16384 residues: 128 tiles, 8384 CTAs)
fills the static array exactly; one residue more is refused.  This file is collected
last so that a failure here leaves every other test already run; it also passes alone.
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
    """CUDA_EonDevice once, then CUDA_EonDevice_noalloc twice in a row."""
    L.CUDA_setBoxDimension(box)
    dp, dm = device_array(pos), device_array(meta)
    out = []
    for fn in (L.CUDA_EonDevice, L.CUDA_EonDevice_noalloc, L.CUDA_EonDevice_noalloc):
        res = ctypes.c_double(0.0)
        fn(ptr(dp), ptr(dm), None, None, None, None, ctypes.byref(res), 32, pos.shape[0], 0)
        cgppd_gb300.check(fn.__name__)
        out.append(res.value)
    return out


def check_all(L, refdata, pos, meta, box):
    lib_ref, first, second = energies(L, pos, meta, box)
    e64 = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], box)[2]
    for v in (lib_ref, first, second):
        assert abs(v - e64) <= REL * abs(e64) + 1e-12, (v, e64)
    assert abs(first - lib_ref) <= REL * abs(lib_ref) + 1e-12
    assert abs(second - lib_ref) <= REL * abs(lib_ref) + 1e-12


def test_noalloc_matches_cuda_eondevice_twice(L, refdata):
    for i in (1, 3, 8):
        mols = oracle.build_replica(["conf%d/1a" % i, "conf%d/1b" % i], refdata, 1000.0)
        pos, meta = oracle.pack_replica(mols, 32)
        check_all(L, refdata, pos, meta, 1000.0)


def lattice_packed(n, P, seed, spacing=6.5):
    """n residues in rigid domains of 300 residues on a jittered cubic lattice (no
    clashes, so the sum is not dominated by a few huge repulsive terms), padded to P with
    the reference's padding records.  Returns pos, meta and the periodic box edge."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n ** (1.0 / 3.0)))
    box = side * spacing
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    pos = np.zeros((P, 4), np.float32)
    meta = np.zeros((P, 4), np.float32)
    pos[:n, :3] = g * spacing + rng.uniform(-0.6, 0.6, (n, 3))
    pos[:n, 3] = 1.0 + np.arange(n) // 300          # rigid domain per 300 residues
    meta[:n] = np.stack([rng.integers(0, 20, n), rng.choice([-1.0, 0.0, 1.0], n), rng.uniform(4.5, 7, n),
                         np.arange(n) // 300 + 0.25], 1)
    pos[n:, 3] = -2.0
    meta[n:, 0] = 20.0
    return pos, meta, float(box)


def test_noalloc_large_system(L, refdata):
    pos, meta, box = lattice_packed(6000, 6016, 7)
    check_all(L, refdata, pos, meta, box)


def test_noalloc_at_the_limit_and_above(L, refdata):
    # 16384 residues: 128 tiles of 128, 8384 CTAs -- every CTA slot of the static array
    pos, meta, box = lattice_packed(16384, 16384, 11)
    check_all(L, refdata, pos, meta, box)
    # one residue more is refused before anything is launched (no device memory is read)
    for size in (16385, 16416):
        res = ctypes.c_double(3.0)
        L.CUDA_EonDevice_noalloc(None, None, None, None, None, None, ctypes.byref(res), 32, size, 0)
        assert res.value == 0.0
        with pytest.raises(cgppd_gb300.CgppdError):
            cgppd_gb300.check("over the limit")
