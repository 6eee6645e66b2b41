"""Parity of the drop-in CUDA ABI (CUDA_EonDevice / NC / async) on a GB300.

Inputs are packed exactly as the reference's ReplicaDataToDevice does; results are
compared with the golden totals of the reference tests and with the FP64 oracle.
Tolerance: 1e-5 relative to the FP64 oracle (the bound of the GPU path), plus a
1e-9 kcal/mol absolute floor for totals that are themselves ~1e-5.
"""
import ctypes

import numpy as np
import pytest

import cgppd_gb300
import oracle
from helpers import device_array, ptr

pytestmark = pytest.mark.gpu
REL = 1e-5
ABS = 1e-9


@pytest.fixture(scope="module")
def L(refdata):
    import torch
    assert torch.cuda.is_available()
    cgppd_gb300.build()
    L = cgppd_gb300.lib()
    a = L.cgppd_aminoacids_create()
    t = np.ascontiguousarray(np.array(refdata["lj_table"], np.float32).reshape(-1))
    L.cgppd_aminoacids_set_table(a, t.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    dev = L.LJPotentialDataToDevice(a)
    assert dev
    L.bindLJTexture(dev)
    cgppd_gb300.check("setup")
    yield L
    L.unbindLJTexture()
    L.cgppd_aminoacids_destroy(a)


def eon(L, pos, meta, box, nc=False, P=None):
    L.CUDA_setBoxDimension(box)
    dp, dm = device_array(pos), device_array(meta)
    res = ctypes.c_double(0.0)
    fn = L.CUDA_EonDeviceNC if nc else L.CUDA_EonDevice
    fn(ptr(dp), ptr(dm), None, None, None, None, ctypes.byref(res), 32, int(P if P is not None else pos.shape[0]), 0)
    cgppd_gb300.check("EonDevice")
    return res.value


def eon_async(L, pos, meta, box, block=32):
    import torch
    L.CUDA_setBoxDimension(box)
    dp, dm = device_array(pos), device_array(meta)
    rs = pos.shape[0] // block
    out = torch.full((rs * rs,), 7.0, dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    L.CUDA_EonDevice_async(ptr(dp), ptr(dm), None, None, None, None, ptr(out), rs, block, pos.shape[0], 0,
                           ctypes.c_void_p(s.cuda_stream))
    s.synchronize()
    cgppd_gb300.check("EonDevice_async")
    h = out.cpu().numpy().astype(np.float64)
    return h.sum(), h


def test_reference_conformations(L, refdata):
    # tests/testReferenceConformations.cpp:95-101: GPU, NC and async totals
    kat = refdata["kats"]["reference_conformations_exact"]
    for i in range(1, 11):
        mols = oracle.build_replica(["conf%d/1a" % i, "conf%d/1b" % i], refdata, 1000.0)
        pos, meta = oracle.pack_replica(mols, 32)
        ref = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], 1000.0)[2]
        g = eon(L, pos, meta, 1000.0)
        gnc = eon(L, pos, meta, 1000.0, nc=True)
        ga, arr = eon_async(L, pos, meta, 1000.0)
        assert abs(g - ref) <= REL * abs(ref) + ABS, (i, g, ref)
        assert abs(gnc - ref) <= REL * abs(ref) + ABS, (i, gnc, ref)
        assert abs(ga - ref) <= 2e-7 * abs(ref) + REL * abs(ref) + ABS, (i, ga, ref)
        assert np.all(arr[1:] == 0.0)
        exp = sum(kat[i - 1])
        assert g == pytest.approx(exp, rel=1.2e-5, abs=1e-9)


def test_flexible_replica(L, refdata):
    # tests/testReplica.cpp:83-100
    mols = oracle.build_replica(["conf1/1a", "conf1/1b"], refdata, 118.4, segments={1: [[72, 73, 74, 75]]})
    pos, meta = oracle.pack_replica(mols, 32)
    corr = oracle.total(oracle.E_intra(oracle.FP64, mols[1], refdata, include_lj_dh=False))
    flex = sum(refdata["kats"]["replica_flexible"])
    rigid = sum(refdata["kats"]["replica_rigid"])
    assert eon(L, pos, meta, 118.4) + corr == pytest.approx(flex, rel=1.2e-5)
    assert eon(L, pos, meta, 118.4, nc=True) == pytest.approx(rigid, rel=1.2e-5)
    ga, _ = eon_async(L, pos, meta, 118.4)
    assert ga + corr == pytest.approx(flex, rel=1.2e-5)
    pos_r, meta_r = oracle.pack_replica(mols, 32, rigid_only=True)
    assert eon(L, pos_r, meta_r, 118.4) == pytest.approx(rigid, rel=1.2e-5)


def synthetic_packed(rng, nmol, lens, box, flexible_frac=0.0, crowders=0, block=32):
    """Random packed replica: compact random-walk chains, random types, uids as packed floats."""
    recs = []
    dom = 1
    for m in range(nmol + crowders):
        n = int(lens[m % len(lens)])
        c = rng.uniform(0, box, 3)
        steps = rng.normal(size=(n, 3))
        steps = 3.8 * steps / np.linalg.norm(steps, axis=1, keepdims=True)
        xyz = c + np.cumsum(steps, 0) * 0.4
        crowd = m >= nmol
        for i in range(n):
            flexible = (not crowd) and rng.random() < flexible_frac
            pw = 0.0 if flexible else float(dom)
            if rng.random() < 0.05 and not crowd:
                pw += 0.25
            mw = -1.0 if crowd else m + 0.25
            recs.append((xyz[i], pw, rng.integers(0, 20), rng.choice([-1.0, 0.0, 0.0, 0.0, 1.0, 0.5]),
                         rng.uniform(4.5, 7.0), mw))
        dom += 1
    n = len(recs)
    P = -(-n // block) * block
    pos = np.zeros((P, 4), np.float32)
    meta = np.zeros((P, 4), np.float32)
    for k, (xyz, pw, aa, q, s, mw) in enumerate(recs):
        pos[k] = (*xyz, pw)
        meta[k] = (aa, q, s, mw)
    pos[n:, 3] = -2.0
    meta[n:, 0] = 20.0
    return pos, meta


@pytest.mark.parametrize("case", [
    dict(nmol=2, lens=[76], box=150.0),
    dict(nmol=3, lens=[40, 129, 7], box=60.0, flexible_frac=0.3),
    dict(nmol=6, lens=[100, 250], box=120.0, crowders=5, flexible_frac=0.1),
    dict(nmol=1, lens=[3], box=0.0),
    dict(nmol=24, lens=[60, 160, 97], box=250.0, crowders=40),
])
def test_random_systems_vs_oracle(L, refdata, case):
    rng = np.random.default_rng(1234 + case["nmol"])
    box = case["box"]
    pos, meta = synthetic_packed(rng, case["nmol"], case["lens"], box, case.get("flexible_frac", 0.0),
                                 case.get("crowders", 0))
    for nc in (False, True):
        ref = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], box, nc=nc)
        g = eon(L, pos, meta, box, nc=nc)
        comps = (ctypes.c_double * 3)()
        assert L.cgppd_last_energy_components(comps) == 0
        assert comps[2] == g
        # each component within 1e-5 relative of the FP64 oracle, and the total too
        for k in (0, 1):
            assert abs(comps[k] - ref[k]) <= REL * abs(ref[k]) + ABS, (nc, k, comps[k], ref[k])
        assert abs(g - ref[2]) <= REL * abs(ref[2]) + ABS, (nc, g, ref)


def test_async_calls_back_to_back_on_one_stream(L, refdata):
    # consecutive asynchronous calls on one stream share its scratch and are dependent
    # launches (each may be placed before the previous one ends): every call must still
    # see only its own inputs and leave its own total
    import torch
    rng = np.random.default_rng(77)
    box = 120.0
    pos0, meta = synthetic_packed(rng, 6, [100, 250], box, 0.1, 5)
    L.CUDA_setBoxDimension(box)
    systems, outs, refs = [], [], []
    for k in range(8):
        pos = pos0.copy()
        n = int((pos[:, 3] > -2.0).sum())
        pos[:n, :3] += rng.normal(scale=0.3, size=(n, 3)).astype(np.float32)
        refs.append(oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], box)[2])
        systems.append((device_array(pos), device_array(meta)))
    rs = pos0.shape[0] // 32
    s = torch.cuda.Stream()
    for k, (dp, dm) in enumerate(systems):
        out = torch.full((rs * rs,), 7.0, dtype=torch.float32, device="cuda")
        outs.append(out)
        L.CUDA_EonDevice_async(ptr(dp), ptr(dm), None, None, None, None, ptr(out), rs, 32, pos0.shape[0], 0,
                               ctypes.c_void_p(s.cuda_stream))
    s.synchronize()
    cgppd_gb300.check("EonDevice_async burst")
    for k, out in enumerate(outs):
        h = out.cpu().numpy()
        assert np.all(h[1:] == 0.0)
        # float32 output: its rounding on top of the 1e-5 bound
        assert abs(float(h[0]) - refs[k]) <= REL * abs(refs[k]) + 1e-6 * abs(refs[k]) + ABS, (k, h[0], refs[k])
    assert len(set(float(o[0].item()) for o in outs)) > 1  # the inputs differ, so do the totals


def test_empty_and_unbound(L, refdata):
    # empty dataset -> 0 without a launch
    res = ctypes.c_double(5.0)
    L.CUDA_EonDevice(None, None, None, None, None, None, ctypes.byref(res), 32, 0, 0)
    assert res.value == 0.0
    cgppd_gb300.check("empty")


def test_type_index_out_of_range_is_reported(L, refdata):
    pos = np.zeros((32, 4), np.float32)
    meta = np.zeros((32, 4), np.float32)
    pos[:, 3] = -2.0
    meta[:, 0] = 20.0
    pos[0] = (0, 0, 0, 1.0)
    pos[1] = (5, 0, 0, 2.0)
    meta[0] = (3, 0, 5, 0.25)
    meta[1] = (400, 0, 5, 1.5)  # 20*3 + 400 is outside the 20x20 table
    L.CUDA_setBoxDimension(0.0)
    dp, dm = device_array(pos), device_array(meta)
    res = ctypes.c_double(0.0)
    L.CUDA_EonDevice(ptr(dp), ptr(dm), None, None, None, None, ctypes.byref(res), 32, 32, 0)
    with pytest.raises(cgppd_gb300.CgppdError):
        cgppd_gb300.check("bad type")
