"""Self-consistency of the oracle's Monte Carlo restatement (CPU only)."""
import numpy as np
import pytest

from cgppd_gb300 import workloads
from oracle.remc import OracleRemc


def small(config, nrep, steps=40):
    wl = workloads.make(config)
    sim = wl.sims[0]
    o = OracleRemc(sim.molecules, wl.lj_raw, sim.box, sim.temperatures[:nrep], sim.translate_steps[:nrep],
                   sim.rotate_steps[:nrep], sim.move_weights, sim.rigid_rotate_prob, wl.torsion_V,
                   wl.torsion_phase, seed=wl.seed)
    return wl, o


@pytest.mark.parametrize("config", ["c0", "c1"])
def test_running_potential_is_the_energy_of_the_state(config):
    wl, o = small(config, 3)
    o.run(2, 25, exchange_after_last=False)
    for r in range(o.R):
        e, _ = o.energy(r)
        assert e == o.potential[r]  # the reference keeps the recomputed total on accept
    c = o.counters()
    # the closing report has not run, so per-block counters hold the last block only
    assert np.all(c["accept"] + c["acceptA"] + c["reject"] == 25)


def test_moves_keep_rigid_shapes():
    wl, o = small("c0", 2)
    before = o.pos.copy()
    o.run(1, 60)
    for r in range(o.R):
        for m, (s0, n) in enumerate(((0, 76), (76, 76))):
            d0 = np.linalg.norm(before[r, s0:s0 + n, None] - before[r, None, s0:s0 + n], axis=-1)
            d1 = np.linalg.norm(o.pos[r, s0:s0 + n, None] - o.pos[r, None, s0:s0 + n], axis=-1)
            # internal distances survive rotation / translation (wrapping moves whole molecules)
            assert np.allclose(d0, d1, atol=2e-3)


def test_flexible_moves_change_only_the_linker_geometry():
    wl, o = small("c1", 2)
    before = o.pos.copy()
    o.run(1, 80)
    for r in range(o.R):
        for s0, n in ((0, 75), (87, 75)):  # rigid domains keep their shape
            d0 = np.linalg.norm(before[r, s0:s0 + n, None] - before[r, None, s0:s0 + n], axis=-1)
            d1 = np.linalg.norm(o.pos[r, s0:s0 + n, None] - o.pos[r, None, s0:s0 + n], axis=-1)
            assert np.allclose(d0, d1, atol=5e-3)
