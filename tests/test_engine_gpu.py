"""Parity of the batched GB300 REMC engine with the oracle.

1. Energies: every replica's molecule-pair matrix, internal energies and total are
   compared with the FP64 oracle on the same coordinates (1e-5 relative bound).
2. Trajectories: the engine and the oracle's restatement of the reference MC loop
   (full recomputation each step, reference precision) draw the same Philox words, so
   they take the same moves and -- except for Metropolis draws that fall within float
   rounding of the acceptance probability -- the same decisions.  Positions are compared
   after whole blocks (tolerance 2e-3 A for the accumulated float rotations), potentials
   within 1e-5 relative, exchange decisions and counters exactly.
3. Statistics: where float rotations part the trajectories from the reference loop's
   double ones (C1), seeded runs of both sample the same per-temperature mean energies
   and acceptance within statistical error.
"""
import numpy as np
import pytest

import oracle
from cgppd_gb300 import engine as eng
from cgppd_gb300 import workloads
from oracle.remc import OracleRemc, float_mean

pytestmark = pytest.mark.gpu
REL = 1e-5


def oracle_matrix(wl, sim, xyz):
    mols = sim.molecules
    start = np.cumsum([0] + [m.n for m in mols[:-1]]).astype(np.int32)
    cnt = np.array([m.n for m in mols], np.int32)
    aa = np.concatenate([m.types for m in mols])
    q = np.concatenate([m.charges for m in mols])
    s = np.concatenate([m.radii for m in mols])
    return oracle.E_inter_matrix(oracle.FP64, xyz, aa, q, s, start, cnt, wl.lj_raw, sim.box)


def subset(wl, nrep):
    sim = wl.sims[0]
    return workloads.Simulation(sim.molecules, sim.box, sim.temperatures[:nrep], sim.translate_steps[:nrep],
                                sim.rotate_steps[:nrep], sim.move_weights, sim.rigid_rotate_prob)


def engine_for(wl, sims, cluster=1, threads=256, sample_frequency=0, sample_after=0, resident=True):
    w2 = workloads.Workload(wl.name, sims, wl.lj_raw, wl.torsion_V, wl.torsion_phase, wl.seed)
    return eng.from_workload(w2, cluster=cluster, threads=threads, sample_frequency=sample_frequency,
                             sample_after=sample_after, resident=resident)


def oracle_for(wl, sim, mode=oracle.REF, **kw):
    return OracleRemc(sim.molecules, wl.lj_raw, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                      sim.move_weights, sim.rigid_rotate_prob, wl.torsion_V, wl.torsion_phase, seed=wl.seed,
                      mode=mode, **kw)


@pytest.mark.parametrize("config", ["c0", "c2", "c4"])
def test_initial_energy_matrix(config):
    wl = workloads.make(config)
    sim = subset(wl, 2)
    e = engine_for(wl, [sim])
    xyz = np.concatenate([m.xyz for m in sim.molecules]).astype(np.float32)
    ref = oracle_matrix(wl, sim, xyz)
    E, intra = e.matrix(0, 1)
    scale = np.abs(ref).max()
    assert np.all(np.abs(E - ref) <= REL * np.abs(ref) + 1e-7 * scale), np.abs(E - ref).max()
    tot_ref = np.triu(ref, 1).sum()
    pot = e.replicas(0)["potential"]
    assert np.all(np.abs(pot - tot_ref) <= REL * abs(tot_ref) + 1e-9)
    # recompute into scratch leaves the state alone and agrees
    assert np.allclose(e.recompute(False), pot, rtol=1e-12, atol=1e-12)


def test_initial_energy_flexible_linker():
    wl = workloads.make("c1")
    sim = subset(wl, 2)
    e = engine_for(wl, [sim])
    o = oracle_for(wl, sim, mode=oracle.FP64)
    pot = e.replicas(0)["potential"]
    assert abs(pot[0] - o.initial_energy) <= REL * abs(o.initial_energy)


def test_reference_flexible_replica_energy(refdata):
    # tests/testReplica.cpp:79-82 through the engine: conf1, 1b residues 73-76 flexible
    mols = []
    for key, segs in (("conf1/1a", []), ("conf1/1b", [[72, 73, 74, 75]])):
        rec = refdata["pdbs"][key]
        aa = np.array([r["aa"] for r in rec["residues"]], np.int32)
        mols.append(workloads.Molecule(np.array([r["xyz"] for r in rec["residues"]], np.float32), aa,
                                       [refdata["amino_acids"][a]["charge"] for a in aa],
                                       [refdata["amino_acids"][a]["radius"] for a in aa], segments=segs,
                                       res_seq=[r["seq"] for r in rec["residues"]]))
    sim = workloads.Simulation(mols, 118.4, [300.0], [0.5], [0.2])
    V = np.array(refdata["torsion_V"])
    S = np.array(refdata["torsion_sigma"])
    wl = workloads.Workload("conf1", [sim], np.array(refdata["lj_table"], np.float32), V, S, seed=1)
    e = eng.from_workload(wl, cluster=1)
    pot = e.replicas(0)["potential"][0]
    assert pot == pytest.approx(sum(refdata["kats"]["replica_flexible"]), rel=1.2e-5)
    E, intra = e.matrix(0, 0)
    assert E[0, 1] == pytest.approx(sum(refdata["kats"]["replica_rigid"]), rel=1.2e-5)


def compare_runs(e, o, sim_index=0, pos_tol=2e-3, traj_rel=REL):
    """Same decisions, same exchanges; coordinates within float drift; the engine's
    running total within 1e-5 of the FP64 oracle evaluated on the engine's own
    coordinates; the two totals within `traj_rel` of each other (they are energies of
    coordinates that differ by the accumulated float rounding of the moves)."""
    R = o.R
    rep = e.replicas(sim_index)
    assert np.array_equal(rep["temperature"], o.temperature)
    assert np.array_equal(rep["label"], o.label)
    c = o.counters()
    for k in ("accept", "acceptA", "reject", "totalAccept", "totalAcceptReject"):
        assert np.array_equal(rep[k], c[k]), (k, rep[k], c[k])
    assert np.all(np.abs(rep["potential"] - o.potential) <= traj_rel * np.abs(o.potential) + 1e-6)
    for r in range(R):
        xyz, rel, cen = e.state(sim_index, r)
        assert np.abs(xyz - o.pos[r]).max() < pos_tol
        assert np.abs(cen - o.center[r]).max() < pos_tol
        e64 = o.energy_of(xyz, oracle.FP64)
        assert abs(rep["potential"][r] - e64) <= REL * abs(e64) + 1e-9, (r, rep["potential"][r], e64)


@pytest.mark.parametrize("resident", [True, False])
# c1 is shorter: its flex moves rotate in float here and in double in the reference loop,
# so the coordinates drift apart by float rounding and, over a few hundred steps, one
# Metropolis draw can land inside that rounding of its acceptance probability.
@pytest.mark.parametrize("config,nrep,blocks,steps", [("c0", 4, 3, 100), ("c4", 4, 2, 60), ("c1", 4, 2, 40),
                                                     ("c2", 3, 2, 20)])
def test_trajectory_matches_oracle(config, nrep, blocks, steps, resident):
    wl = workloads.make(config)
    sim = subset(wl, nrep)
    e = engine_for(wl, [sim], cluster=4 if config == "c2" else 1, resident=resident)
    assert e.launch_shape()[2] == resident
    o = oracle_for(wl, sim)
    e.run(blocks, steps, exchange_after_last=True)
    orep, oex = o.run(blocks, steps, exchange_after_last=True)
    compare_runs(e, o, traj_rel=REL if config != "c1" else 2e-4)
    assert e.error_bits() == 0
    # per-temperature reports and exchange counts of every exchange are identical
    for b in range(blocks):
        er, ex = e.report(0, b)
        assert np.allclose(er, orep[b], equal_nan=True), (b, er, orep[b])
        assert tuple(ex) == tuple(oex[b])


@pytest.mark.parametrize("resident", [True, False])
@pytest.mark.parametrize("cluster", [2, 4])
def test_cluster_split_matches_single_cta(cluster, resident):
    wl = workloads.make("c4")
    sim = subset(wl, 3)
    e1 = engine_for(wl, [sim], cluster=1, resident=resident)
    ec = engine_for(wl, [sim], cluster=cluster, resident=resident)
    assert ec.launch_shape()[0] == cluster
    e1.run(2, 80)
    ec.run(2, 80)
    r1, rc = e1.replicas(0), ec.replicas(0)
    for k in ("accept", "acceptA", "reject", "label"):
        assert np.array_equal(r1[k], rc[k])
    # same decisions; totals differ only by the float grouping of each CTA's slice
    assert np.allclose(r1["potential"], rc["potential"], rtol=1e-7, atol=1e-9)
    for r in range(3):
        assert np.abs(e1.state(0, r)[0] - ec.state(0, r)[0]).max() < 1e-5


def test_running_total_has_no_drift():
    wl = workloads.make("c4")
    sim = subset(wl, 4)
    e = engine_for(wl, [sim], cluster=2)
    e.run(5, 200)
    run_tot = e.replicas(0)["potential"]
    fresh = e.recompute(False)
    # a fresh evaluation sums each molecule pair from the other side: FP32-level noise only
    assert np.allclose(run_tot, fresh, rtol=1e-6, atol=1e-7)
    # and the state's energy agrees with the FP64 oracle on the engine's coordinates
    for r in range(4):
        xyz, _, _ = e.state(0, r)
        ref = np.triu(oracle_matrix(wl, sim, xyz), 1).sum()
        assert abs(run_tot[r] - ref) <= REL * abs(ref) + 1e-9


def test_flexible_running_total_within_bound():
    # local moves keep the internal energy of a flexible molecule incrementally (the
    # moved residue's terms), re-evaluated at every launch: after long blocks the totals
    # stay within 1e-5 of a fresh evaluation and of the FP64 energy
    wl = workloads.make("c1")
    sim = subset(wl, 4)
    e = engine_for(wl, [sim], cluster=4)
    e.run(3, 1000)
    run_tot = e.replicas(0)["potential"]
    assert np.allclose(run_tot, e.recompute(False), rtol=1e-5, atol=1e-7)
    o = oracle_for(wl, sim)
    for r in range(4):
        xyz, _, _ = e.state(0, r)
        e64 = o.energy_of(xyz, oracle.FP64)
        assert abs(run_tot[r] - e64) <= REL * abs(e64) + 1e-9, (r, run_tot[r], e64)


@pytest.mark.parametrize("config", ["c1", "c4"])
def test_flexible_and_rigid_clusters_match_oracle(config):
    # flexible moves and crankshafts split over a cluster, state resident
    wl = workloads.make(config)
    sim = subset(wl, 3)
    e = engine_for(wl, [sim], cluster=2)
    o = oracle_for(wl, sim)
    e.run(2, 80)
    o.run(2, 80)
    compare_runs(e, o, traj_rel=REL if config != "c1" else 2e-4)


def test_flexible_linker_statistics_match_oracle():
    # C1's rigid and flex rotations run in float here and in double in the reference loop
    # (src/Quaternion.cpp:95-112), so trajectories part after a few hundred steps.  What
    # must not change is what they sample: per-temperature mean energies of independent
    # seeded runs of the engine and of the oracle's restatement of the reference loop
    # (reference precision) agree within their statistical error.  No exchanges, so every
    # slot samples its own temperature; one energy per block after a burn-in block.
    wl = workloads.make("c1")
    sim = subset(wl, 8)
    nseed, blocks, steps, burn = 16, 8, 250, 2

    def acceptance(c):  # accepted / proposed over the run (no exchange resets the counters)
        a = c["accept"].sum() + c["acceptA"].sum()
        return a / max(1, a + c["reject"].sum())

    def engine_means(seed):
        w2 = workloads.Workload(wl.name, [sim], wl.lj_raw, wl.torsion_V, wl.torsion_phase, seed)
        e = eng.from_workload(w2, cluster=1, threads=256)
        samples = []
        for b in range(blocks):
            e.run(1, steps, exchange_after_last=False)
            if b >= burn:
                samples.append(e.replicas(0)["potential"].copy())
        c = e.replicas(0)
        e.close()
        return np.mean(samples, 0), acceptance(c)

    def oracle_means(seed):
        o = OracleRemc(sim.molecules, wl.lj_raw, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                       sim.move_weights, sim.rigid_rotate_prob, wl.torsion_V, wl.torsion_phase, seed=seed,
                       mode=oracle.REF)
        samples = []
        for b in range(blocks):
            o.run(1, steps, exchange_after_last=False, threads=8)
            if b >= burn:
                samples.append(o.potential.copy())
        return np.mean(samples, 0), acceptance(o.counters())

    e_runs = [engine_means(1000 + s) for s in range(nseed)]
    o_runs = [oracle_means(2000 + s) for s in range(nseed)]
    em, om = np.array([r[0] for r in e_runs]), np.array([r[0] for r in o_runs])
    err = np.sqrt(em.var(0, ddof=1) / nseed + om.var(0, ddof=1) / nseed)
    z = np.abs(em.mean(0) - om.mean(0)) / np.maximum(err, 1e-3)
    assert np.all(z < 4.5), (em.mean(0), om.mean(0), err)
    ea, oa = np.array([r[1] for r in e_runs]), np.array([r[1] for r in o_runs])
    za = abs(ea.mean() - oa.mean()) / max(np.sqrt(ea.var(ddof=1) / nseed + oa.var(ddof=1) / nseed), 1e-4)
    assert za < 4.5, (ea.mean(), oa.mean())


def test_batched_simulations_match_separate_oracles():
    # three small simulations of different shapes in one launch
    wl0, wl4, wl1 = workloads.make("c0"), workloads.make("c4"), workloads.make("c1")
    sims = [subset(wl0, 3), subset(wl4, 2)]
    e = engine_for(wl0, sims)  # same contact table object is used for both
    e.run(2, 50)
    off = 0
    for s, sim in enumerate(sims):
        o = OracleRemc(sim.molecules, wl0.lj_raw, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                       sim.move_weights, sim.rigid_rotate_prob, None, None, seed=wl0.seed, rep_off=off, sim_index=s)
        o.run(2, 50)
        compare_runs(e, o, sim_index=s)
        off += o.R


def test_fraction_bound_sampling_matches_oracle():
    wl = workloads.make("c4")
    sim = subset(wl, 3)
    e = engine_for(wl, [sim], sample_frequency=10, sample_after=0)
    o = oracle_for(wl, sim, sample_frequency=10, sample_after=0)
    e.run(2, 100, exchange_after_last=False)
    o.run(2, 100, exchange_after_last=False)
    rep = e.replicas(0)
    c = o.counters()
    for k in ("boundSamples", "samplesSinceLastExchange", "totalBoundSamples", "totalSamples"):
        assert np.array_equal(rep[k], c[k]), k
    e.final_report(1)
    fo = o.final_report()
    fe, _ = e.report(0, 1)
    assert np.allclose(fe, fo, equal_nan=True)


def test_counters_and_launches():
    wl = workloads.make("c0")
    sim = subset(wl, 2)
    e = engine_for(wl, [sim])
    e.run(3, 10)
    steps, pairs = e.counters()
    assert steps == 2 * 30
    assert pairs == 2 * 30 * 76 * 76
    assert e.last_launches() == 6


def test_non_finite_coordinates_are_reported_not_propagated():
    # a replica whose coordinates turn non-finite (injected on the host) rejects every
    # move and takes no part in exchanges; the others run on, and each slot reports
    # its own status bits (2: non-finite energy change, 4: non-finite exchange test)
    wl = workloads.make("c0")
    sim = subset(wl, 4)
    e = engine_for(wl, [sim], cluster=2)
    e.run(1, 20)
    bad = 2
    xyz, rel, cen = e.state(0, bad)
    xyz[0, 0] = np.nan
    rel[0, 0] = np.nan
    e.set_state(0, bad, xyz, rel, cen)
    e.recompute(write_state=True)
    before = e.replicas(0)
    e.run(3, 40)
    after = e.replicas(0)
    bits = e.replica_error_bits(0)
    assert bits[bad] & 2
    for r in range(4):
        if r != bad:
            assert not (bits[r] & 2), (r, bits)
            assert np.isfinite(after["potential"][r])
    # the bad replica's temperature never moved and its coordinates never changed
    assert after["temperature"][bad] == before["temperature"][bad]
    xyz2, _, _ = e.state(0, bad)
    assert np.array_equal(np.isnan(xyz2), np.isnan(xyz))
    assert np.array_equal(xyz2[~np.isnan(xyz2)], xyz[~np.isnan(xyz)])
    # its ladder neighbours saw the non-finite exchange test
    assert bits[bad] & 4
    assert e.error_bits() & 6 == 6


def test_tuning_cache_persists_across_processes(tmp_path):
    # CGPPD_TUNING_CACHE: the first process sweeps and records the chosen shape, a second
    # process on the same GPU model reads it and skips the sweep
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from cgppd_gb300 import engine as eng, workloads\n"
            "e = eng.from_workload(workloads.make('c4'))\n"
            "print(len(e.tuning()), *e.launch_shape()[:2])\n" % root)
    env = dict(os.environ, CGPPD_TUNING_CACHE=str(tmp_path / "tuning.jsonl"))
    first = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert first.returncode == 0, first.stderr
    n1, c1, t1 = map(int, first.stdout.split()[-3:])
    assert n1 > 0
    lines = (tmp_path / "tuning.jsonl").read_text().splitlines()
    assert len(lines) == 1 and '"cluster":%d' % c1 in lines[0] and '"threads":%d' % t1 in lines[0]
    second = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert second.returncode == 0, second.stderr
    n2, c2, t2 = map(int, second.stdout.split()[-3:])
    assert (n2, c2, t2) == (0, c1, t1)
    assert len((tmp_path / "tuning.jsonl").read_text().splitlines()) == 1


@pytest.fixture(scope="module")
def c3_subset():
    """Four simulations of the batched uneven configuration, kept in their order there:
    the one with the most pair work per step (12 molecules, 2,157 residues, a 387-residue
    chain, 15 replicas), the one with the longest chain (400 residues), a 12-molecule one
    with 8 replicas and the one with the least pair work (2 molecules, 172 residues)."""
    wl = workloads.make("c3")
    sizes = [sum(m.n for m in s.molecules) ** 2 - sum(m.n ** 2 for m in s.molecules) for s in wl.sims]
    most = int(np.argmax(sizes))
    least = int(np.argmin(sizes))
    longest = max(range(len(wl.sims)), key=lambda i: max(m.n for m in wl.sims[i].molecules))
    eight = next(i for i, s in enumerate(wl.sims) if len(s.temperatures) == 8 and len(s.molecules) == 12)
    ids = sorted({most, least, longest, eight})
    assert len(ids) == 4
    return wl, ids


def test_batched_uneven_subset_matches_oracle(c3_subset):
    wl, ids = c3_subset
    sims = [wl.sims[i] for i in ids]
    e = engine_for(wl, sims, cluster=1, threads=512)
    assert e.launch_shape()[2]  # resident, as in the full configuration
    # initial molecule-pair matrices of the first and last replica of every simulation
    for s, sim in enumerate(sims):
        xyz = np.concatenate([m.xyz for m in sim.molecules]).astype(np.float32)
        ref = oracle_matrix(wl, sim, xyz)
        scale = np.abs(ref).max()
        for r in (0, len(sim.temperatures) - 1):
            E, _ = e.matrix(s, r)
            assert np.all(np.abs(E - ref) <= REL * np.abs(ref) + 1e-7 * scale), (ids[s], r, np.abs(E - ref).max())
    # two exchange blocks, every simulation against its own oracle run (same Philox
    # streams: the engine numbers replicas across simulations in the order added)
    blocks, steps = 2, 30
    e.run(blocks, steps, exchange_after_last=True)
    assert e.error_bits() == 0
    off = 0
    for s, sim in enumerate(sims):
        o = OracleRemc(sim.molecules, wl.lj_raw, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                       sim.move_weights, sim.rigid_rotate_prob, None, None, seed=wl.seed, rep_off=off, sim_index=s)
        orep, oex = o.run(blocks, steps, exchange_after_last=True, threads=o.R)
        # the engine rotates in float, the reference loop in double: the coordinates of
        # the two runs differ by that rounding, and near contact the energies of the two
        # coordinate sets differ by up to ~1e-5 relative; each engine total is still held
        # to 1e-5 of the FP64 energy of its own coordinates
        compare_runs(e, o, sim_index=s, traj_rel=1e-4)
        for b in range(blocks):
            er, ex = e.report(s, b)
            assert np.allclose(er, orep[b], equal_nan=True), (ids[s], b)
            assert tuple(ex) == tuple(oex[b]), (ids[s], b)
        off += o.R
    e.close()


def test_sample_log_records_every_sample():
    # fraction-bound samples every 10 steps: one record per sample and replica slot, in
    # order, with the window's first step; a block-end sample holds the replica's
    # potential and temperature at that point, and the non-crowder energy of a system
    # of two rigid proteins is its total
    wl = workloads.make("c0")
    sim = subset(wl, 3)
    e = engine_for(wl, [sim], sample_frequency=10, sample_after=0)
    e.set_sample_log(25)
    e.run(2, 100, exchange_after_last=False)
    rec = e.take_samples(0)
    rep = e.replicas(0)
    for r in range(3):
        assert list(rec[r]["step"]) == list(range(0, 200, 10))
        assert rec[r]["potential"][-1] == pytest.approx(rep["potential"][r], rel=1e-12)
        assert rec[r]["temperature"][-1] == rep["temperature"][r]
        assert np.allclose(rec[r]["enc"], rec[r]["potential"], rtol=1e-12)
    # the log was emptied; a full log records no more and says so (bit 8)
    assert all(len(x["step"]) == 0 for x in e.take_samples(0))
    e.run(3, 100, exchange_after_last=False)
    assert all(len(x["step"]) == 25 for x in e.take_samples(0))
    assert e.error_bits() & 8
    e.close()


@pytest.mark.parametrize("resident", [True, False])
def test_sample_snapshots_hold_the_sampled_coordinates(resident):
    # with snapshots on, every recorded sample also keeps the leading residues'
    # coordinates (the sample PDB files): a sample on a block's last step holds the
    # coordinates the replica ends the block with; C1's flexible molecule in a cluster
    wl = workloads.make("c1")
    sim = subset(wl, 3)
    e = engine_for(wl, [sim], cluster=2, sample_frequency=50, sample_after=0, resident=resident)
    nres = 100  # a prefix of the molecule: the first residues of the replica
    e.set_sample_log(8)
    e.set_sample_snapshots(nres)
    for b in range(3):
        e.run(1, 50, exchange_after_last=False)
        rec = e.take_samples(0)
        for r in range(3):
            assert list(rec[r]["step"]) == [50 * b]
            xyz, _, _ = e.state(0, r)
            assert np.array_equal(rec[r]["xyz"][0], xyz[:nres])
    assert e.error_bits() == 0
    e.close()
