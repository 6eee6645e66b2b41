"""The GB300 engine against the reference's own Monte Carlo code.

The recorded trajectories of the reference's Simulation::run (tests/golden/
ref_mc_trajectories.json; the reference's src/Simulation.cpp, Replica.cpp and
Molecule.cpp with the engine's Philox draws, see tests/golden/make_ref_mc_golden.py)
start from the reference's own initial coordinates; the engine starts from the same
state with the same seed and must take the same moves and decisions: identical
temperatures, labels and acceptance counters after every run, coordinates within the
drift of its float rotations (the reference rotates with double quaternions), each
running total within 1e-5 of the FP64 energy of the engine's own coordinates.
"""
import numpy as np
import pytest

import oracle
from cgppd_gb300 import engine as eng
from cgppd_gb300 import workloads
from oracle import ref_mc
from oracle.remc import OracleRemc
from helpers import ref_mc_config

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,blocks", [("bound", 1), ("bound", 3), ("flexible", 1)])
def test_engine_takes_the_reference_trajectory(name, blocks, refdata):
    cfg, mols, cen, rel, temps, tsteps, rsteps = ref_mc_config(name)
    table = np.array(refdata["lj_table"], np.float32)
    V, S = np.array(refdata["torsion_V"]), np.array(refdata["torsion_sigma"])
    sim = workloads.Simulation(mols, cfg["box"], temps, tsteps, rsteps)
    wl = workloads.Workload(name, [sim], table, V, S, seed=cfg["seed"])
    e = eng.from_workload(wl, cluster=1, threads=256, sample_frequency=cfg["sample_frequency"],
                          sample_after=cfg["sample_after"])
    xyz = np.concatenate([m.xyz for m in mols])
    for r in range(len(temps)):
        e.set_state(0, r, xyz, rel, cen)
    e.recompute(write_state=True)
    pot0 = e.replicas(0)["potential"]
    assert np.allclose(pot0, cfg["initial"]["replicas"][0]["potential"], rtol=1e-5, atol=1e-6)
    e.run(blocks, cfg["block"], exchange_after_last=False)
    e.final_report(blocks - 1)
    fin = ref_mc.replicas(cfg["runs"][str(blocks)], "final")
    rep = e.replicas(0)
    assert np.array_equal(rep["temperature"], fin["temperature"])
    assert np.array_equal(rep["label"], fin["label"])
    assert np.array_equal(rep["totalAccept"], fin["totalAccept"]), (rep["totalAccept"], fin["totalAccept"])
    assert np.array_equal(rep["totalAcceptReject"], fin["totalAcceptReject"])
    o = OracleRemc(mols, table, cfg["box"], temps, tsteps, rsteps, (1, 1, 1, 1), 0.5, V, S, seed=cfg["seed"],
                   centers=cen, rel=rel)
    for r in range(len(temps)):
        exyz, _, ecen = e.state(0, r)
        assert np.abs(exyz - fin["xyz"][r]).max() < 2e-3
        assert np.abs(ecen - fin["centers"][r]).max() < 2e-3
        e64 = o.energy_of(exyz, oracle.FP64)
        assert abs(rep["potential"][r] - e64) <= 1e-5 * abs(e64) + 1e-7, (r, rep["potential"][r], e64)
        # and the reference's own total on its own coordinates, to the drift of the rotations
        assert abs(rep["potential"][r] - fin["potential"][r]) <= 1e-4 * abs(fin["potential"][r]) + 1e-5
    e.close()
