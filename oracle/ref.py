"""ctypes binding of oracle/_ref/libcgppd_ref.so (the reference's own energy code).

TEST INFRASTRUCTURE ONLY.  The library exists only where the reference tree is
mounted (it is built from the reference's sources by oracle/build_ref.py); callers
skip when `available()` is False.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libcgppd_ref.so")
_lib = None


def available():
    if not os.path.exists(LIB):
        try:
            from .build_ref import build
            build()
        except Exception:
            return False
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        f64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.ref_energy.argtypes = [ctypes.c_int, i32, i32, i32, i32, f32, i32, f32, f32, ctypes.c_char_p, i32, i32,
                                 i32, i32, i32, f32, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_float, f64, f64]
        L.ref_graph.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, i32, i32, ctypes.c_int,
                                i32, ctypes.c_int, i32, i32, i32, i32]
        L.ref_lj_offset.restype = ctypes.c_size_t
        _lib = L
    return _lib


def energy(molecules, table, box, torsion_V=None, torsion_phase=None):
    """Reference E() + sum of Molecule::E(true): raw (LJ, DH, bond, angle product,
    torsion) and the inter-molecule (LJ, DH)."""
    t = np.asarray(table, np.float32)
    crowder_raw = float(t[20, 0]) if t.shape[0] > 20 else 0.0
    t20 = np.ascontiguousarray(t[:20, :20]).reshape(-1)
    mstart = np.cumsum([0] + [m.n for m in molecules[:-1]]).astype(np.int32)
    mcount = np.array([m.n for m in molecules], np.int32)
    mflex = np.array([1 if m.all_flexible else 0 for m in molecules], np.int32)
    mcrowd = np.array([1 if m.crowder else 0 for m in molecules], np.int32)
    xyz = np.ascontiguousarray(np.concatenate([m.xyz for m in molecules]).astype(np.float32).reshape(-1))
    types = np.ascontiguousarray(np.concatenate([m.types for m in molecules]).astype(np.int32))
    q = np.ascontiguousarray(np.concatenate([m.charges for m in molecules]).astype(np.float32))
    s = np.ascontiguousarray(np.concatenate([m.radii for m in molecules]).astype(np.float32))
    cid = "".join("".join(m.chain_ids) for m in molecules).encode()
    rseq = np.ascontiguousarray(np.concatenate([m.res_seq for m in molecules]).astype(np.int32))
    cidx = np.ascontiguousarray(np.concatenate([m.chain_index for m in molecules]).astype(np.int32))
    nseg = np.array([len(m.segments) for m in molecules], np.int32)
    seglen = np.ascontiguousarray([len(x) for m in molecules for x in m.segments] or [0], np.int32)
    segres = np.ascontiguousarray([v for m in molecules for x in m.segments for v in x] or [0], np.int32)
    V = np.ascontiguousarray(torsion_V, np.float64) if torsion_V is not None else None
    S = np.ascontiguousarray(torsion_phase, np.float64) if torsion_phase is not None else None
    out = np.zeros(5, np.float64)
    inter = np.zeros(2, np.float64)
    lib().ref_energy(len(molecules), mstart, mcount, mflex, mcrowd, xyz, types, q, s, cid, rseq, cidx, nseg, seglen,
                     segres, t20, crowder_raw, V.ctypes.data if V is not None else None,
                     S.ctypes.data if S is not None else None, float(box), out, inter)
    return out, inter


def graph(chain_ids, all_flexible, segments, num_chains, cap=100000):
    n = len(chain_ids)
    seglen = np.ascontiguousarray([len(x) for x in segments] or [0], np.int32)
    segres = np.ascontiguousarray([v for x in segments for v in x] or [0], np.int32)
    counts = np.zeros(9, np.int32)
    b = np.zeros(cap, np.int32)
    a = np.zeros(cap, np.int32)
    t = np.zeros(cap, np.int32)
    ind = np.zeros(cap, np.int32)
    lib().ref_graph(n, "".join(chain_ids).encode(), int(bool(all_flexible)), len(segments), seglen, segres,
                    num_chains, counts, cap, b, a, t, ind)
    return {"counts": counts.tolist(),
            "bonds": set(map(tuple, b[:2 * counts[0]].reshape(-1, 2).tolist())),
            "angles": set(map(tuple, a[:3 * counts[1]].reshape(-1, 3).tolist())),
            "torsions": set(map(tuple, t[:4 * counts[2]].reshape(-1, 4).tolist())),
            "indirect": set(map(tuple, ind[:2 * counts[5]].reshape(-1, 2).tolist()))}
