"""Checkpoint and resume of the engine (no counterpart in the reference, which stubs it).

A run interrupted by checkpoint -> new engine -> restore continues exactly as the
uninterrupted run: same potentials, coordinates, labels, statistics and report rows
(the Philox step counters travel with the state).
"""
import numpy as np
import pytest

from cgppd_gb300 import CgppdError
from cgppd_gb300 import engine as eng
from cgppd_gb300 import workloads

pytestmark = pytest.mark.gpu


def subset(wl, nrep):
    sim = wl.sims[0]
    return workloads.Simulation(sim.molecules, sim.box, sim.temperatures[:nrep], sim.translate_steps[:nrep],
                                sim.rotate_steps[:nrep], sim.move_weights, sim.rigid_rotate_prob)


def make(wl, nrep, cluster):
    w2 = workloads.Workload(wl.name, [subset(wl, nrep)], wl.lj_raw, wl.torsion_V, wl.torsion_phase, wl.seed)
    return eng.from_workload(w2, cluster=cluster, threads=256)


@pytest.mark.parametrize("config", ["c4", "c1"])
def test_resume_continues_the_run_exactly(tmp_path, config):
    wl = workloads.make(config)
    a = make(wl, 4, 2)
    a.run(2, 80)
    path = tmp_path / "state.ck"
    a.checkpoint(path)
    a.run(2, 80)
    b = make(wl, 4, 2)
    b.restore(path)
    b.run(2, 80)
    ra, rb = a.replicas(0), b.replicas(0)
    for k in ("potential", "temperature", "label", "tindex", "accept", "acceptA", "reject", "totalAccept",
              "totalAcceptReject"):
        assert np.array_equal(ra[k], rb[k]), k
    for r in range(4):
        xa, qa, ca = a.state(0, r)
        xb, qb, cb = b.state(0, r)
        assert np.array_equal(xa, xb) and np.array_equal(qa, qb) and np.array_equal(ca, cb)
    for row in range(3):
        assert np.array_equal(a.report(0, row)[0], b.report(0, row)[0], equal_nan=True)
    assert a.counters() == b.counters()
    a.close()
    b.close()


def test_restore_rejects_another_system(tmp_path):
    a = make(workloads.make("c4"), 4, 1)
    path = tmp_path / "state.ck"
    a.checkpoint(path)
    b = make(workloads.make("c4"), 3, 1)
    with pytest.raises(CgppdError):
        b.restore(path)
    a.close()
    b.close()


def test_restore_clears_report_rows_past_the_checkpoint(tmp_path):
    # an engine that already wrote more report rows than the checkpoint holds shows, after
    # the restore, the checkpoint's rows and then zeros -- never its own earlier rows
    wl = workloads.make("c4")
    a = make(wl, 3, 1)
    a.run(1, 40)
    path = tmp_path / "state.ck"
    a.checkpoint(path)
    b = make(wl, 3, 1)
    b.run(6, 40)
    assert np.any(b.report(0, 4)[0] != 0)
    b.restore(path)
    assert np.array_equal(b.report(0, 0)[0], a.report(0, 0)[0], equal_nan=True)
    for row in range(2, 6):
        rep, ex = b.report(0, row)
        assert np.all(rep == 0) and tuple(ex) == (0, 0), (row, rep, ex)
    a.close()
    b.close()
