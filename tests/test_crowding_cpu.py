"""The oracle's repulsive-crowding terms (the reference's REPULSIVE_CROWDING build).

The reference selects, at compile time (src/definitions.h:18, off by default), a
repulsive-only potential for every pair with a crowder: (6/r)^12 in RT units below
15 A (src/Replica.cpp:416-419, :434-472; src/CudaFunctions.cu:335-338, :492-498) and
no Debye-Hueckel term.  No reference test or golden file covers that build, so these
checks hold the oracle's restatement to the closed form and to the full-potential
oracle on the pairs that do not involve a crowder.
"""
import math

import numpy as np
import pytest

import oracle
from cgppd_gb300 import workloads
from oracle.remc import OracleRemc

RT = oracle.RT_TO_KCAL


def small_crowded(seed=7, rep_crowd=True, large=False):
    # large: proteins of 100+ residues, so the engine reads the mover charged first
    rng = np.random.default_rng(seed)
    sigma_type = rng.uniform(4.5, 7.0, size=21).astype(np.float32)
    table = workloads.contact_table(rng, with_crowder=True, crowder_eps=0.1)
    lengths, box = ([110, 64], 80.0) if large else ([30, 24, 36], 60.0)
    sim = workloads.rigid_sim(rng, lengths, box, 4, sigma_type, crowders=5, crowder_len=12)
    sim.repulsive_crowding = rep_crowd
    return table, sim


def arrays(sim):
    mols = sim.molecules
    start = np.cumsum([0] + [m.n for m in mols[:-1]]).astype(np.int32)
    cnt = np.array([m.n for m in mols], np.int32)
    xyz = np.concatenate([m.xyz for m in mols]).astype(np.float32)
    aa = np.concatenate([m.types for m in mols])
    q = np.concatenate([m.charges for m in mols])
    s = np.concatenate([m.radii for m in mols])
    crowd = np.array([1 if m.crowder else 0 for m in mols], np.int32)
    return start, cnt, xyz, aa, q, s, crowd


def min_image_r(a, b, L):
    d = a.astype(np.float64) - b.astype(np.float64)
    d -= L * np.round(d / L)
    return np.sqrt((d * d).sum(-1))


@pytest.mark.parametrize("mode", [oracle.REF, oracle.FP64])
def test_crowder_term_closed_form(mode):
    for r in (2.5, 4.0, 6.0, 9.3, 14.99):
        assert oracle.crowder_term(mode, r) == pytest.approx((6.0 / r) ** 12, rel=1e-6 if mode == oracle.REF else 1e-14)
    # zero from the cutoff on (r < const_repulsive_cutoff is the condition)
    assert oracle.crowder_term(mode, 15.0) == 0.0
    assert oracle.crowder_term(mode, 40.0) == 0.0


def test_matrix_without_crowders_is_the_full_potential():
    table, sim = small_crowded()
    start, cnt, xyz, aa, q, s, crowd = arrays(sim)
    full = oracle.E_inter_matrix(oracle.FP64, xyz, aa, q, s, start, cnt, table, sim.box)
    none = oracle.E_inter_matrix_rc(oracle.FP64, xyz, aa, q, s, start, cnt, np.zeros_like(crowd), table, sim.box)
    assert np.array_equal(full, none)


def test_crowder_pairs_are_repulsive_only():
    table, sim = small_crowded()
    start, cnt, xyz, aa, q, s, crowd = arrays(sim)
    full = oracle.E_inter_matrix(oracle.FP64, xyz, aa, q, s, start, cnt, table, sim.box)
    rc = oracle.E_inter_matrix_rc(oracle.FP64, xyz, aa, q, s, start, cnt, crowd, table, sim.box)
    M = len(start)
    n_close = 0
    for a in range(M):
        for b in range(a + 1, M):
            if not (crowd[a] or crowd[b]):
                assert rc[a, b] == full[a, b]
                continue
            A = xyz[start[a]:start[a] + cnt[a]]
            B = xyz[start[b]:start[b] + cnt[b]]
            r = min_image_r(A[:, None, :], B[None, :, :], sim.box)
            close = r < 15.0
            n_close += int(close.sum())
            ref = RT * math.fsum(((6.0 / r[close]) ** 12).tolist())
            assert rc[a, b] == pytest.approx(ref, rel=1e-12, abs=1e-300)
            assert rc[a, b] >= 0.0
    assert n_close > 0  # the case exercises the crowder term


def test_mc_oracle_energy_uses_crowder_terms():
    table, sim = small_crowded()
    start, cnt, xyz, aa, q, s, crowd = arrays(sim)
    o = OracleRemc(sim.molecules, table, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                   mode=oracle.FP64, repulsive_crowding=True)
    rc = oracle.E_inter_matrix_rc(oracle.FP64, xyz, aa, q, s, start, cnt, crowd, table, sim.box)
    assert o.energy_of(xyz, oracle.FP64) == pytest.approx(np.triu(rc, 1).sum(), rel=1e-13)
    o_full = OracleRemc(sim.molecules, table, sim.box, sim.temperatures, sim.translate_steps, sim.rotate_steps,
                        mode=oracle.FP64, repulsive_crowding=False)
    full = oracle.E_inter_matrix(oracle.FP64, xyz, aa, q, s, start, cnt, table, sim.box)
    assert o_full.energy_of(xyz, oracle.FP64) == pytest.approx(np.triu(full, 1).sum(), rel=1e-13)


def packed(sim, block=32):
    """The reference's packed upload of rigid molecules: pos.w = molecule id (the rigid
    domain), meta = (type, charge, radius, w) with w = molecule id + a chain fraction
    unique to the molecule, or -1 for a crowder (src/Replica.cpp:748-798)."""
    start, cnt, xyz, aa, q, s, crowd = arrays(sim)
    N = xyz.shape[0]
    P = ((N + block - 1) // block) * block
    pos4 = np.zeros((P, 4), np.float32)
    meta4 = np.zeros((P, 4), np.float32)
    pos4[:, 3] = -2.0
    meta4[:, 0] = 20.0
    for m in range(len(start)):
        sl = slice(start[m], start[m] + cnt[m])
        pos4[sl, :3] = xyz[sl]
        pos4[sl, 3] = m + 1
        meta4[sl, 0] = np.where(crowd[m], 0, aa[sl])  # a crowder's term reads no table entry
        meta4[sl, 1] = q[sl]
        meta4[sl, 2] = s[sl]
        meta4[sl, 3] = -1.0 if crowd[m] else (m + 1) + (m + 1) / 64.0
    return pos4, meta4


def test_packed_kernel_rules_with_repulsive_crowding():
    table, sim = small_crowded()
    start, cnt, xyz, aa, q, s, crowd = arrays(sim)
    pos4, meta4 = packed(sim)
    t20 = np.ascontiguousarray(table[:20, :20])
    off = oracle.E_packed(oracle.FP64, pos4, meta4, t20, sim.box)
    assert np.array_equal(off, oracle.E_packed(oracle.FP64, pos4, meta4, t20, sim.box, repulsive_crowding=False))
    on = oracle.E_packed(oracle.FP64, pos4, meta4, t20, sim.box, repulsive_crowding=True)
    # the same pairs as the molecule-pair matrix, except that the packed kernel's chain
    # rule also excludes residues of two consecutive crowders (both w = -1, chain
    # fraction 0) within 4 indices of each other
    rc = oracle.E_inter_matrix_rc(oracle.FP64, xyz, aa, q, s, start, cnt, crowd, table, sim.box)
    excl = 0.0
    for a in range(len(start) - 1):
        if crowd[a] and crowd[a + 1]:
            for i in range(start[a] + cnt[a] - 3, start[a] + cnt[a]):
                for j in range(start[a + 1], i + 4):
                    excl += oracle.crowder_term(oracle.FP64, min_image_r(xyz[i], xyz[j], sim.box) + 1e-38)
    assert on[2] == pytest.approx(np.triu(rc, 1).sum() - excl * RT, rel=1e-9)
    # pairs with a crowder carry no Debye-Hueckel term: charged crowders change the
    # full-potential sum but not the repulsive-crowding one
    charged = meta4.copy()
    charged[meta4[:, 3] == -1.0, 1] = 0.5
    assert oracle.E_packed(oracle.FP64, pos4, charged, t20, sim.box)[1] != off[1]
    assert oracle.E_packed(oracle.FP64, pos4, charged, t20, sim.box, repulsive_crowding=True)[1] == on[1]
