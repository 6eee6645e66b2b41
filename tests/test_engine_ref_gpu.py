"""The engine's energies against the reference's own energy code.

tests/golden/ref_energies.json holds totals the reference's energy code produced
(tests/golden/make_ref_golden.py) for the synthetic configurations' initial states
(saved in tests/golden/ref_structures.npz) and rigid perturbations of them; the engine
must reproduce each within 1e-5 relative.
"""
import json
import os

import numpy as np
import pytest

from cgppd_gb300 import engine as eng
from cgppd_gb300 import workloads
from helpers import fixture_workload
from test_ref_pin import perturbed

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "ref_energies.json")))


@pytest.mark.parametrize("cfg", ["c0", "c1", "c2", "c4"])
def test_engine_matches_reference_energies(cfg):
    wl = fixture_workload(cfg)
    sim = wl.sims[0]
    for st in GOLD["configs"][cfg]:
        mols = perturbed(sim, st["transforms"])
        s2 = workloads.Simulation(mols, sim.box, sim.temperatures[:1], sim.translate_steps[:1], sim.rotate_steps[:1],
                                  sim.move_weights, sim.rigid_rotate_prob)
        w2 = workloads.Workload(wl.name, [s2], wl.lj_raw, wl.torsion_V, wl.torsion_phase, wl.seed)
        e = eng.from_workload(w2, cluster=1, threads=256)
        pot = e.replicas(0)["potential"][0]
        ref = st["total_kcal"]
        assert abs(pot - ref) <= 1e-5 * abs(ref) + 1e-9, (cfg, pot, ref)
        e.close()
