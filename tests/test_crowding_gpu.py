"""Repulsive crowding (the reference's REPULSIVE_CROWDING build) on a GB300.

The engine (cgppd_sim_params.repulsive_crowding) and the drop-in energy module
(cgppd_set_repulsive_crowding) against the oracle's restatement: energies within 1e-5
of the FP64 oracle, Monte Carlo trajectories step for step with the reference-loop
oracle (same Philox draws, same decisions, same exchanges).
"""
import ctypes

import numpy as np
import pytest

import cgppd_gb300
import oracle
from cgppd_gb300 import engine as eng
from cgppd_gb300 import workloads
from helpers import device_array, ptr
from oracle.remc import OracleRemc
from test_crowding_cpu import arrays, packed, small_crowded
from test_engine_gpu import compare_runs

pytestmark = pytest.mark.gpu
REL = 1e-5


def engine(table, sim, cluster=1, threads=256, resident=True):
    wl = workloads.Workload("crowded", [sim], table, seed=20261210)
    return eng.from_workload(wl, cluster=cluster, threads=threads, resident=resident), wl


@pytest.mark.parametrize("cluster", [1, 3])
def test_initial_matrix(cluster):
    table, sim = small_crowded()
    e, _ = engine(table, sim, cluster=cluster)
    start, cnt, xyz, aa, q, s, crowd = arrays(sim)
    ref = oracle.E_inter_matrix_rc(oracle.FP64, xyz, aa, q, s, start, cnt, crowd, table, sim.box)
    full = oracle.E_inter_matrix(oracle.FP64, xyz, aa, q, s, start, cnt, table, sim.box)
    assert not np.allclose(ref, full)  # the crowder pairs differ from the full potential
    # crowder entries are sums of positive terms: each within 1e-5 of itself
    cmask = (crowd[:, None] | crowd[None, :]).astype(bool)
    assert ref[cmask].max() > 0.1
    for r in range(len(sim.temperatures)):
        E, _ = e.matrix(0, r)
        scale = np.abs(ref).max()
        assert np.abs(E - ref).max() <= REL * scale
        assert np.all(np.abs(E - ref)[cmask] <= REL * np.abs(ref)[cmask] + 1e-12)
        tot = np.triu(ref, 1).sum()
        assert abs(e.replicas(0)["potential"][r] - tot) <= REL * abs(tot) + 1e-9


@pytest.mark.parametrize("resident,cluster,large", [(True, 1, False), (False, 1, False), (True, 3, False),
                                                   (False, 3, False), (True, 2, True), (False, 2, True)])
def test_trajectory_matches_oracle(cluster, resident, large):
    table, sim = small_crowded(large=large)
    e, wl = engine(table, sim, cluster=cluster, resident=resident)
    assert e.launch_shape()[:1] == (cluster,) and e.launch_shape()[2] == resident
    o = OracleRemc(sim.molecules, table, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                   seed=wl.seed, mode=oracle.REF, repulsive_crowding=True)
    e.run(3, 80, exchange_after_last=True)
    o.run(3, 80, exchange_after_last=True)
    compare_runs(e, o)
    assert e.error_bits() == 0
    assert e.replicas(0)["totalAccept"].sum() > 0  # moves were accepted (counters reset per report)


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
    L.bindLJTexture(dev)
    cgppd_gb300.check("setup")
    yield L
    L.cgppd_set_repulsive_crowding(0)
    L.unbindLJTexture()
    L.cgppd_aminoacids_destroy(a)


def test_dropin_energy(L, refdata):
    table, sim = small_crowded()
    pos4, meta4 = packed(sim)
    t20 = np.array(refdata["lj_table"], np.float32).reshape(20, 20)
    L.CUDA_setBoxDimension(sim.box)
    dp, dm = device_array(pos4), device_array(meta4)
    out = {}
    for rc in (0, 1):
        assert L.cgppd_set_repulsive_crowding(rc) in (0, 1)
        res = ctypes.c_double(0.0)
        L.CUDA_EonDevice(ptr(dp), ptr(dm), None, None, None, None, ctypes.byref(res), 32, pos4.shape[0], 0)
        cgppd_gb300.check("EonDevice")
        ref = oracle.E_packed(oracle.FP64, pos4, meta4, t20, sim.box, repulsive_crowding=bool(rc))[2]
        assert abs(res.value - ref) <= REL * abs(ref) + 1e-9, (rc, res.value, ref)
        out[rc] = res.value
    assert L.cgppd_set_repulsive_crowding(0) == 1
    assert out[0] != out[1]
