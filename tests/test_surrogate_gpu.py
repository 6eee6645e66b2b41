"""The learned pair-energy surrogate on a GB300: kernels against the CPU oracle, training,
and delayed-acceptance screening inside the engine.

* forward pass and loss gradient of the tcgen05 training kernels against the float64
  restatement (oracle/mlp.py), both with the GPU's bfloat16 rounding points emulated
  (tight) and as the exact float64 network (loose);
* training samples: pose features and exact pair energies produced by the engine against
  the oracle's features and FP64 pair energies of the same states;
* screening with a network that predicts exactly zero leaves the trajectory identical
  to the plain engine (stage 1 always passes, stage 2 is the plain test);
* the error threshold trips the fallback to the plain test, and a wildly wrong network
  leaves the running totals exact;
* training lowers the held-out error, and the trained network's first stage saves exact
  pair work relative to the plain engine;
* screening with a trained network, and with that network's output negated, samples the
  plain engine's distribution (per-temperature mean energy over 16 simulations).
"""
import numpy as np
import pytest

import oracle
from oracle import mlp
from cgppd_gb300 import engine as eng
from cgppd_gb300 import surrogate as sg
from cgppd_gb300 import workloads

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def pose_like(rng, n):
    X = np.zeros((n, 8), np.float32)
    X[:, :3] = rng.normal(scale=1.2, size=(n, 3))
    X[:, 3] = rng.uniform(0.15, 1.2, n)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    X[:, 4:] = q
    return X


@pytest.fixture(scope="module")
def net():
    s = sg.Surrogate(batch=512, seed=7)
    yield s
    s.close()


def test_forward_matches_oracle(net):
    rng = np.random.default_rng(1)
    X = pose_like(rng, 300)            # not a multiple of 128: padded inside
    out = net.predict(X)
    p = net.params.astype(np.float64)
    ref_bf, _ = mlp.forward(p, X, bf16_path=True)
    ref64, _ = mlp.forward(p, X)
    assert np.max(np.abs(out - ref_bf)) <= 2e-3 * (1 + np.max(np.abs(ref_bf))), np.max(np.abs(out - ref_bf))
    assert rel_err(out, ref64) < 3e-2


def test_gradients_match_oracle(net):
    rng = np.random.default_rng(2)
    X = pose_like(rng, 512)
    y = rng.normal(size=512).astype(np.float32)
    loss, g = net.loss_grad(X, y)
    p = net.params.astype(np.float64)
    lb, gb = mlp.loss_grad(p, X, y, bf16_path=True)
    l64, g64 = mlp.loss_grad(p, X, y)
    assert loss == pytest.approx(lb, rel=2e-3)
    assert loss == pytest.approx(l64, rel=2e-2)
    for k, (o, n) in mlp.OFF.items():
        assert rel_err(g[o:o + n], gb[o:o + n]) < 2e-2, (k, rel_err(g[o:o + n], gb[o:o + n]))
        assert rel_err(g[o:o + n], g64[o:o + n]) < 8e-2, (k, rel_err(g[o:o + n], g64[o:o + n]))
    cos = float(np.dot(g, g64) / (np.linalg.norm(g) * np.linalg.norm(g64)))
    assert cos > 0.998


def subset(wl, nrep):
    sim = wl.sims[0]
    return workloads.Simulation(sim.molecules, sim.box, sim.temperatures[:nrep], sim.translate_steps[:nrep],
                                sim.rotate_steps[:nrep], sim.move_weights, sim.rigid_rotate_prob)


def engine_for(wl, sims, cluster=8, threads=256, resident=True):
    w2 = workloads.Workload(wl.name, sims, wl.lj_raw, wl.torsion_V, wl.torsion_phase, wl.seed)
    return eng.from_workload(w2, cluster=cluster, threads=threads, resident=resident)


def oracle_pair_energies(wl, sim, xyz):
    mols = sim.molecules
    start = np.cumsum([0] + [m.n for m in mols[:-1]]).astype(np.int32)
    cnt = np.array([m.n for m in mols], np.int32)
    aa = np.concatenate([m.types for m in mols])
    q = np.concatenate([m.charges for m in mols])
    s = np.concatenate([m.radii for m in mols])
    return oracle.E_inter_matrix(oracle.FP64, xyz.astype(np.float32), aa, q, s, start, cnt, wl.lj_raw, sim.box)


def test_training_samples_match_oracle():
    wl = workloads.make("c4")
    sim = subset(wl, 2)
    e = engine_for(wl, [sim])
    assert sg.compatible(e, 0)
    e.run(2, 50)                      # two different replica states
    s = sg.Surrogate(batch=128, seed=3)
    s.collect(e, 0, 96, proposal_fraction=0.0, seed=11)
    X, y = s.samples()
    fr = mlp.frame_residues(sim.molecules[0].xyz - sim.molecules[0].xyz.mean(0))
    cands = []
    for r in range(2):
        xyz, rel, cen = e.state(0, r)
        E = oracle_pair_energies(wl, sim, xyz)
        off = np.cumsum([0] + [m.n for m in sim.molecules])
        frames = [mlp.frame(*rel[off[k] + np.array(fr)]) for k in range(len(sim.molecules))]
        for a in range(len(sim.molecules)):
            for b in range(a + 1, len(sim.molecules)):
                cands.append((mlp.features(frames[a], cen[a], frames[b], cen[b], sim.box), E[a, b]))
    CX = np.array([c[0] for c in cands])
    CE = np.array([c[1] for c in cands])
    for x, yy in zip(X, y):
        d = np.max(np.abs(CX - x), axis=1)
        k = int(np.argmin(d))
        assert d[k] < 2e-4, d[k]
        assert abs(yy - CE[k]) <= 1e-5 * abs(CE[k]) + 1e-6, (yy, CE[k])
    s.close()
    e.close()


def run_pair(wl, nrep, blocks, steps, attach_with=None, resident=True, **kw):
    e = engine_for(wl, [subset(wl, nrep)], resident=resident)
    if attach_with is not None:
        assert sg.attach(e, attach_with, **kw) == 1
    e.run(blocks, steps, exchange_after_last=True)
    e.synchronize()
    return e


@pytest.mark.parametrize("resident", [True, False])
def test_zero_surrogate_reproduces_plain_trajectory(resident):
    wl = workloads.make("c4")
    s = sg.Surrogate(batch=128, seed=5)
    s.params = np.zeros(sg.N_PARAMS, np.float32)
    plain = run_pair(wl, 4, 3, 100, resident=resident)
    da = run_pair(wl, 4, 3, 100, attach_with=s, resident=resident, rmse_threshold=1e9)
    assert da.launch_shape()[2] == resident
    rp, rd = plain.replicas(0), da.replicas(0)
    for k in ("accept", "acceptA", "reject", "totalAccept", "totalAcceptReject", "label", "tindex"):
        assert np.array_equal(rp[k], rd[k]), k
    # the screened engine may autotune to another cluster shape: totals agree to float regrouping
    assert np.allclose(rp["potential"], rd["potential"], rtol=1e-7, atol=1e-9)
    for r in range(4):
        assert np.allclose(plain.state(0, r)[0], da.state(0, r)[0], atol=1e-4)
    st = sg.stats(da, 0)
    assert st["proposals"] == 4 * 300 and st["stage1_reject"] == 0 and st["stage2_eval"] == 4 * 300
    assert st["screening"] == 1
    plain.close()
    da.close()
    s.close()


def test_error_threshold_falls_back_to_plain():
    # a network predicting zero passes every proposal to stage 2, whose error is then the
    # exact change itself: with a tiny threshold the simulation must fall back
    wl = workloads.make("c4")
    s = sg.Surrogate(batch=128, seed=9)
    s.params = np.zeros(sg.N_PARAMS, np.float32)
    e = run_pair(wl, 4, 1, 200, attach_with=s, rmse_threshold=1e-6, min_evals=10)
    st = sg.stats(e, 0)
    assert st["n_e2"] >= 10 and st["rmse"] > 1e-6
    assert st["screening"] == 0
    before = st["proposals"]
    e.run(1, 100)
    e.synchronize()
    assert sg.stats(e, 0)["proposals"] == before     # plain steps from now on
    e.close()
    s.close()


def test_bad_surrogate_keeps_exact_bookkeeping():
    # a wildly wrong network only changes which proposals are tried exactly: the running
    # totals still equal a fresh evaluation of the final coordinates
    wl = workloads.make("c4")
    s = sg.Surrogate(batch=128, seed=9)
    p = s.params
    p[mlp.OFF["w5"][0]:mlp.OFF["w5"][0] + 256] *= 50.0
    s.params = p
    e = run_pair(wl, 4, 2, 200, attach_with=s, rmse_threshold=1e9)
    pot = e.replicas(0)["potential"]
    assert np.allclose(e.recompute(False), pot, rtol=1e-6, atol=1e-6)
    st = sg.stats(e, 0)
    assert st["proposals"] == 4 * 400 and st["screening"] == 1
    assert st["stage1_reject"] + st["stage2_eval"] == st["proposals"]
    e.close()
    s.close()


def test_training_lowers_heldout_error():
    wl = workloads.make("c4")
    e = engine_for(wl, [subset(wl, 8)])
    s, hist = sg.train_on_engine(e, 0, n_samples=40960, blocks=4, steps_per_block=100, epochs=6, batch=1024)
    assert s.n_samples == 40960
    assert np.all(np.isfinite(hist))
    assert hist[-1, 1] < hist[0, 1]
    e.close()
    s.close()


def test_trained_surrogate_skips_exact_work():
    # what the trained network gains over the method without it: its first stage rejects
    # proposals the exact test would mostly reject too, so fewer exact pair terms are
    # evaluated per MC step than in the plain engine (no speed claim: the measured
    # throughput of both is in the bench line's surrogate leg)
    wl = workloads.make("c4")
    plain = engine_for(wl, [subset(wl, 8)])
    s, hist = sg.train_on_engine(plain, 0, n_samples=1_000_000, blocks=8, steps_per_block=200, epochs=6,
                                 batch=8192)
    assert hist[-1, 1] < hist[0, 1]
    s0, p0 = plain.counters()
    plain.run(2, 200)
    plain.synchronize()
    s1, p1 = plain.counters()
    plain_per_step = (p1 - p0) / (s1 - s0)
    da = engine_for(wl, [subset(wl, 8)])
    assert sg.attach(da, s, rmse_threshold=1e30) == 1
    a0, q0 = da.counters()
    da.run(2, 200)
    da.synchronize()
    a1, q1 = da.counters()
    da_per_step = (q1 - q0) / (a1 - a0)
    st = sg.stats(da, 0)
    assert st["screening"] == 1 and st["proposals"] == 8 * 400
    assert st["stage1_reject"] >= 0.03 * st["proposals"], st
    assert da_per_step <= 0.97 * plain_per_step, (da_per_step, plain_per_step)
    # the running totals stay exact whatever the first stage decides
    assert np.allclose(da.recompute(False), da.replicas(0)["potential"], rtol=1e-6, atol=1e-6)
    plain.close()
    da.close()
    s.close()


def two_copy_workload(n_sims):
    """`n_sims` independent copies of one small system: two copies of the c4 protein 30 A
    apart in a 60 A box, 8 temperatures 288-450 K (contacts form and break within a few
    thousand steps, so both arms below reach the same stationary state quickly)."""
    wl4 = workloads.make("c4")
    base = wl4.sims[0].molecules[0]
    m2 = workloads.Molecule(base.xyz + np.float32([30.0, 0.0, 0.0]), base.types, base.charges, base.radii)
    sims = [workloads.Simulation([base, m2], 60.0, workloads.ladder(288.0, 450.0, 8),
                                 workloads.ladder(0.5, 2.0, 8), workloads.ladder(0.2, 0.2, 8))
            for _ in range(n_sims)]
    return workloads.Workload("two copies", sims, wl4.lj_raw, seed=wl4.seed)


def mean_energy_by_temperature(e, n_sims, blocks, steps):
    """Per simulation and temperature index: the mean potential at the ends of `blocks`
    exchange blocks."""
    acc = np.zeros((n_sims, 8))
    for _ in range(blocks):
        e.run(1, steps, exchange_after_last=True)
        for s in range(n_sims):
            rep = e.replicas(s)
            acc[s, rep["tindex"]] += rep["potential"]
    return acc / blocks


def test_screening_samples_the_plain_distribution():
    # Delayed acceptance changes which proposals are evaluated exactly, not the sampled
    # distribution: from the same equilibrated states, the plain engine, the engine
    # screened by a trained network and the engine screened by the same network with its
    # output negated (a first stage that prefers uphill moves) give the same mean energy at
    # every temperature within the spread of 16 independent simulations each.
    S, steps = 16, 500
    wl = two_copy_workload(S)
    burn = eng.from_workload(wl, cluster=4, threads=256)
    burn.run(40, steps, exchange_after_last=True)
    s, hist = sg.train_on_engine(burn, 0, n_samples=262144, blocks=4, steps_per_block=steps, epochs=4, batch=8192)
    snap = []
    for k in range(S):
        rep = burn.replicas(k)
        snap.append([(int(rep["tindex"][r]), burn.state(k, r)) for r in range(8)])
    flipped = sg.Surrogate(batch=8192, seed=3)
    p = s.params.copy()
    for name in ("w5", "b5"):  # (offset, length) of the output layer's weights and bias
        off, n = mlp.OFF[name]
        p[off:off + n] *= -1.0
    flipped.params = p

    def arm(net):
        e = eng.from_workload(wl, cluster=4, threads=256)
        for k in range(S):
            for t, (xyz, rel, cen) in snap[k]:
                e.set_state(k, t, xyz, rel, cen)  # slot t holds temperature index t
        e.recompute(write_state=True)
        if net is not None:
            assert sg.attach(e, net, rmse_threshold=1e30) == S
        e.run(10, steps, exchange_after_last=True)
        m = mean_energy_by_temperature(e, S, 60, steps)
        st = sg.stats(e, 0) if net is not None else None
        assert np.allclose(e.recompute(False), np.concatenate([e.replicas(k)["potential"] for k in range(S)]),
                           rtol=1e-6, atol=1e-6)
        e.close()
        return m, st

    plain, _ = arm(None)
    for net in (s, flipped):
        m, st = arm(net)
        assert st["screening"] == 1 and st["stage1_reject"] > 0
        se = np.sqrt(plain.var(0, ddof=1) / S + m.var(0, ddof=1) / S)
        z = np.abs(plain.mean(0) - m.mean(0)) / np.maximum(se, 1e-3)
        assert np.all(z < 4.5), (plain.mean(0), m.mean(0), se)
    burn.close()
    s.close()
    flipped.close()
