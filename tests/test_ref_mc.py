"""The oracle's Monte Carlo restatement against the reference's own MC code.

The reference's Simulation (src/Simulation.cpp init + run, src/Replica.cpp MCSearch,
src/Molecule.cpp moves, unmodified) runs with its GSL calls answered by the GB300
engine's Philox draws (oracle/ref_rng.cpp), so it makes the moves and decisions the
oracle and the engine make from the same seed.  The oracle must then reproduce it: the
same coordinates bit for bit, the same temperatures, labels and counters, and the same
potentials up to the order of the double-precision sums (1e-12 relative).

* Everywhere: the recorded reference trajectories (tests/golden/ref_mc_trajectories.json,
  made by tests/golden/make_ref_mc_golden.py): the reference's REMC regression system
  (tests/remctestfile, flexible) and bound conformation 1 (rigid), 1 and 3 blocks.
* Where the reference tree is mounted (oracle/_ref/cgppd_ref_mc built from its sources):
  a longer run of the regression system live, 10 blocks of 500 steps.
"""
import os

import numpy as np
import pytest

import oracle
from oracle import ref_mc
from oracle.remc import OracleRemc
from helpers import ref_mc_config, write_reference_data_dir


def oracle_from(cfg, mols, cen, rel, temps, tsteps, rsteps, refdata, seed):
    return OracleRemc(mols, np.array(refdata["lj_table"], np.float32), cfg["box"], temps, tsteps, rsteps,
                      (1, 1, 1, 1), 0.5, np.array(refdata["torsion_V"]), np.array(refdata["torsion_sigma"]),
                      seed=seed, mode=oracle.REF, centers=cen, rel=rel, sample_frequency=cfg["sample_frequency"],
                      sample_after=cfg["sample_after"])


def assert_same_state(o, fin):
    assert np.array_equal(o.temperature, fin["temperature"])
    assert np.array_equal(o.label, fin["label"])
    c = o.counters()
    assert np.array_equal(c["totalAccept"], fin["totalAccept"])
    assert np.array_equal(c["totalAcceptReject"], fin["totalAcceptReject"])
    assert np.allclose(o.potential, fin["potential"], rtol=1e-12, atol=0), (o.potential, fin["potential"])
    assert np.array_equal(o.pos, fin["xyz"])
    assert np.array_equal(o.center, fin["centers"])


@pytest.mark.parametrize("name", ["flexible", "bound"])
@pytest.mark.parametrize("blocks", [1, 3])
def test_oracle_reproduces_reference_trajectory(name, blocks, refdata):
    cfg, mols, cen, rel, temps, tsteps, rsteps = ref_mc_config(name)
    o = oracle_from(cfg, mols, cen, rel, temps, tsteps, rsteps, refdata, cfg["seed"])
    assert o.initial_energy == pytest.approx(cfg["initial"]["replicas"][0]["potential"], rel=1e-12)
    o.run(blocks, cfg["block"], exchange_after_last=False)
    o.final_report()
    run = cfg["runs"][str(blocks)]
    assert_same_state(o, ref_mc.replicas(run, "final"))


def test_reference_code_live_long_run(tmp_path, refdata):
    if not ref_mc.available():
        pytest.skip("the reference tree is not mounted here")
    write_reference_data_dir(str(tmp_path), refdata)
    text = refdata["remctestfile"].replace("mcsteps 1000", "mcsteps 5000").replace("resteps 100", "resteps 10")
    (tmp_path / "cfg").write_text(text)
    d = ref_mc.run(str(tmp_path), "cfg", 11)
    assert d["rng_errors"] == 0
    mols, cen, rel = ref_mc.system(d)
    ini = ref_mc.replicas(d, "initial")
    o = oracle_from(d, mols, cen, rel, ini["temperature"], ini["translate_step"].astype(np.float32),
                    ini["rotate_step"].astype(np.float64), refdata, 11)
    o.run(10, 500, exchange_after_last=False)
    o.final_report()
    assert_same_state(o, ref_mc.replicas(d, "final"))
