"""Pin the oracle against the reference tests' known answers (CPU only).

Each test cites the reference assertion it reproduces.  The comparisons use the
reference's own rule where it has one: Potential::almost_equal is 1e-5 absolute on the
raw accumulators (src/Potential.cpp:223-230); Catch's Approx is ~1.2e-5 relative.
"""
import math

import numpy as np
import pytest

import oracle

ALMOST = 1e-5


def almost_equal(raw_a, raw_b, eps=ALMOST):
    return all(abs(float(a) - float(b)) < eps for a, b in zip(raw_a, raw_b))


def conf_replica(refdata, i, box=1000.0):
    return oracle.build_replica(["conf%d/1a" % i, "conf%d/1b" % i], refdata, box)


@pytest.mark.parametrize("mode", [oracle.REF, oracle.FP64])
def test_reference_conformations_exact(refdata, mode):
    # tests/testReferenceConformations.cpp:83-101: CPU E() and E(a,b) of 10 conformations
    kat = refdata["kats"]["reference_conformations_exact"]
    for i in range(1, 11):
        mols = conf_replica(refdata, i)
        lj, dh = oracle.E_inter(mode, mols, refdata["lj_table"], 1000.0)
        exp_raw = oracle.raw_from_kcal([kat[i - 1][0], kat[i - 1][1], 0, 0, 0])[:2]
        assert almost_equal((lj, dh), exp_raw), (i, lj, dh, exp_raw)
        tot = lj * oracle.RT_TO_KCAL + dh * oracle.DH_FACTOR
        exp_tot = kat[i - 1][0] + kat[i - 1][1]
        assert tot == pytest.approx(exp_tot, rel=1.2e-5, abs=1e-9), (i, tot, exp_tot)


def test_published_error_statistics(refdata):
    # tests/testReferenceConformations.cpp:104-189: relative errors vs the published
    # energies.  The asserted statistics (0.001505, ...) are reproduced to all printed
    # digits when the two conversion fudge factors that the test comments out
    # (:111-112: LJ x 0.6/RT_to_kcalmol, DH x 1.00465) are applied; without them the
    # committed test's assertions do not hold (mean LJ error 0.0145).
    kim = refdata["kats"]["reference_conformations_published"]
    stats = refdata["kats"]["published_error_stats"]
    fudge_lj, fudge_dh = 0.6 / oracle.RT_TO_KCAL, 1.00465
    e = {"LJ": [], "DH": [], "total": []}
    for i in range(1, 11):
        lj, dh = oracle.E_inter(oracle.REF, conf_replica(refdata, i), refdata["lj_table"], 1000.0)
        LJ, DH = lj * oracle.RT_TO_KCAL * fudge_lj, dh * oracle.DH_FACTOR * fudge_dh
        kLJ, kDH = kim[i - 1]
        e["LJ"].append(abs(kLJ - LJ) / abs(kLJ))
        e["DH"].append(abs(kDH - DH) / abs(kDH))
        e["total"].append(abs(kLJ + kDH - LJ - DH) / abs(kLJ + kDH))
    for k in ("LJ", "DH", "total"):
        assert np.mean(e[k]) == pytest.approx(stats["mean_" + k], rel=1e-3, abs=1e-6)
        assert max(e[k]) == pytest.approx(stats["max_" + k], rel=1e-3, abs=1e-6)


def flexible_conf1(refdata, rigid_only=False):
    # tests/testReplica.cpp:36-47: conf1 in a 118.4 A box, residues 73-76 of 1b flexible
    return oracle.build_replica(["conf1/1a", "conf1/1b"], refdata, 118.4, segments={1: [[72, 73, 74, 75]]})


@pytest.mark.parametrize("mode", [oracle.REF, oracle.FP64])
def test_replica_flexible_potential(refdata, mode):
    # tests/testReplica.cpp:79-82: (E() + internal_molecule_E(true)).almost_equal(expected)
    mols = flexible_conf1(refdata)
    lj, dh = oracle.E_inter(mode, mols, refdata["lj_table"], 118.4)
    raw = np.array([lj, dh, 0.0, 1.0, 0.0])
    for m in mols:
        if m.is_flexible:
            r = oracle.E_intra(mode, m, refdata)
            raw[0] += r[0]
            raw[1] += r[1]
            raw[2] += r[2]
            raw[3] *= r[3]
            raw[4] += r[4]
    exp = oracle.raw_from_kcal(refdata["kats"]["replica_flexible"])
    assert almost_equal(raw, exp), (raw, exp)
    # rigid-only potential (testReplica.cpp:95-100): inter-molecule terms alone
    exp_r = oracle.raw_from_kcal(refdata["kats"]["replica_rigid"])
    assert almost_equal((lj, dh), exp_r[:2])


def test_replica_uids_and_packing(refdata):
    # tests/testReplica.cpp:112-176
    mols = flexible_conf1(refdata)
    m1, m2 = mols
    k = refdata["kats"]["replica_uids"]
    assert len(m1.graph.rigid_domains) == 1 and len(m2.graph.rigid_domains) == 1
    assert len(m1.graph.segment_bonds) == 0 and len(m2.graph.segment_bonds) == 0
    assert all(m1.domain_uid == 1) and all(m1.chain_uid == 1) and all(m1.bond_uid == 0)
    assert np.allclose(m1.pos_w, k["m1_pos_w"]) and np.allclose(m1.meta_w, k["m1_meta_w"])
    assert all(m2.domain_uid[:73] == 2) and all(m2.domain_uid[73:] == 0)
    assert all(m2.chain_uid == 2)
    assert np.allclose(m2.pos_w[:73], k["m2_domain_pos_w"]) and np.allclose(m2.pos_w[73:], k["m2_linker_pos_w"])
    assert np.allclose(m2.meta_w, k["m2_meta_w"])


def test_packed_gpu_semantics_matches_cpu(refdata):
    # The reference GPU totals equal the CPU ones (testReferenceConformations.cpp:95-101)
    kat = refdata["kats"]["reference_conformations_exact"]
    for i in range(1, 11):
        mols = conf_replica(refdata, i)
        pos, meta = oracle.pack_replica(mols, 32)
        out = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], 1000.0)
        assert out[2] == pytest.approx(sum(kat[i - 1]), rel=1.2e-5, abs=1e-9)
        nc = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], 1000.0, nc=True)
        assert nc[2] == pytest.approx(sum(kat[i - 1]), rel=1.2e-5, abs=1e-9)


def test_packed_flexible_plus_cpu_correction(refdata):
    # tests/testReplica.cpp:83-86: EonDevice() + internal_molecule_E(false) == flexible total,
    # EonDeviceNC() == rigid total
    mols = flexible_conf1(refdata)
    pos, meta = oracle.pack_replica(mols, 32)
    gpu = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], 118.4)
    corr = oracle.E_intra(oracle.FP64, mols[1], refdata, include_lj_dh=False)
    total = gpu[2] + oracle.total(corr)
    assert total == pytest.approx(sum(refdata["kats"]["replica_flexible"]), rel=1.2e-5)
    nc = oracle.E_packed(oracle.FP64, pos, meta, refdata["lj_table"], 118.4, nc=True)
    assert nc[2] == pytest.approx(sum(refdata["kats"]["replica_rigid"]), rel=1.2e-5)
    # calculate_rigid_potential_only repacking (testReplica.cpp:92-100)
    pos_r, meta_r = oracle.pack_replica(mols, 32, rigid_only=True)
    rig = oracle.E_packed(oracle.FP64, pos_r, meta_r, refdata["lj_table"], 118.4)
    assert rig[2] == pytest.approx(sum(refdata["kats"]["replica_rigid"]), rel=1.2e-5)


def single_molecule(refdata, key, box, all_flexible=False, segments=()):
    rec = refdata["pdbs"][key]
    m = oracle.Mol(rec["residues"], rec["chains"], refdata["amino_acids"], box, all_flexible=all_flexible,
                   segments=segments, position=(0.0, 0.0, 0.0), translate=False)
    m.index = 0
    oracle.assign_uids([m])
    return m


@pytest.mark.parametrize("mode", [oracle.REF, oracle.FP64])
def test_molecule_potentials(refdata, mode):
    # tests/testMolecule.cpp:289-307: ala8 (box 15 A) and angiotensin (box 1000 A), all flexible
    ala = single_molecule(refdata, "tests/ala8", 15.0, all_flexible=True)
    ang = single_molecule(refdata, "tests/angiotensin", 1000.0, all_flexible=True)
    for m, key in ((ala, "molecule_ala8"), (ang, "molecule_angiotensin")):
        got = oracle.E_intra(mode, m, refdata)
        exp = oracle.raw_from_kcal(refdata["kats"][key])
        assert almost_equal(got, exp), (key, got, exp)


def test_molecule_start_positions_and_counts(refdata):
    # tests/testMolecule.cpp:45-70 and :311-323
    ala = single_molecule(refdata, "tests/ala8", 15.0, all_flexible=True)
    assert np.allclose(ala.center, 0.0, atol=1e-5)
    assert np.allclose(ala.rel, np.array(refdata["kats"]["ala8_start"]), atol=1e-5)
    ubq = single_molecule(refdata, "tests/1UBQ", 1000.0, segments=[[72, 73, 74, 75]])
    ang = single_molecule(refdata, "tests/angiotensin", 1000.0, all_flexible=True)
    c = refdata["kats"]["molecule_counts"]
    for m, key in ((ubq, "ubiquitin_seg_72_75"), (ala, "ala8_all"), (ang, "angiotensin_all")):
        assert [len(m.graph.bonds), len(m.graph.angles), len(m.graph.torsions)] == c[key]


def test_geometry_graph(refdata):
    # tests/testGeometry.cpp:6-98: synthetic diubiquitin with two segments
    chain_ids = ["A"] * 76 + ["B"] * 76
    g = oracle.Graph(chain_ids, False, [[72, 73, 74, 75, 123], [148, 149, 150, 151]], 2)
    k = refdata["kats"]["geometry"]
    assert g.bonds == set(map(tuple, k["bonds"]))
    assert g.angles == set(map(tuple, k["angles"]))
    assert g.torsions == set(map(tuple, k["torsions"]))
    assert g.MC_crankshaft_residues == k["crankshaft"]
    assert g.MC_local_residues == k["local"]
    assert g.MC_flex_residues == k["flex"]
    for key, (lo, hi) in k["branch"].items():
        i, j = map(int, key.split(","))
        assert g.branch(i, j) == set(range(lo, hi + 1))
    assert g.segment_bonds == list(map(tuple, k["segment_bonds"]))
    assert g.indirect_neighbours == set(map(tuple, k["indirect_neighbours"]))
    assert [set(d) for d in g.rigid_domains] == [set(range(a, b + 1)) for a, b in k["rigid_domains"]]
    for v in (0, 50, 72):
        assert g.rigid_domain_around(v) == set(range(0, 73))
    for v in (76, 100, 123, 148):
        assert g.rigid_domain_around(v) == set(range(76, 149))


def test_philox_known_answers():
    # Published known-answer vectors of Philox4x32-10 (Random123 distribution).
    cases = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, exp in cases:
        assert list(oracle.philox(ctr, key)) == exp


def test_fp64_and_ref_modes_agree(refdata):
    # The FP64 oracle and the reference's mixed precision differ by float rounding only.
    for i in range(1, 11):
        mols = conf_replica(refdata, i)
        a = oracle.E_inter(oracle.REF, mols, refdata["lj_table"], 1000.0)
        b = oracle.E_inter(oracle.FP64, mols, refdata["lj_table"], 1000.0)
        ta = a[0] * oracle.RT_TO_KCAL + a[1] * oracle.DH_FACTOR
        tb = b[0] * oracle.RT_TO_KCAL + b[1] * oracle.DH_FACTOR
        assert math.isclose(ta, tb, rel_tol=1e-5, abs_tol=1e-10)
