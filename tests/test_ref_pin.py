"""Pin the oracle (and the library's graph) against the reference's own code.

* Everywhere: the committed fixtures tests/golden/ref_energies.json (energies the
  reference's own energy code produced for the synthetic configurations, made by
  tests/golden/make_ref_golden.py, on the structures saved beside them in
  tests/golden/ref_structures.npz) against the oracle in reference precision (to
  1e-9 relative) and in FP64 (1e-5).
* Where the reference tree is mounted (oracle/_ref built from its sources): the same
  comparisons live, the reference's Graph::init against the oracle's and the
  library's graph, and the reference's AminoAcids layout against the library's.
"""
import json
import os

import numpy as np
import pytest

import cgppd_gb300
import oracle
from cgppd_gb300 import workloads
from oracle import ref
from oracle.remc import OracleRemc
from helpers import fixture_workload

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "ref_energies.json")))


def perturbed(sim, transforms):
    mols = []
    for m, tr in zip(sim.molecules, transforms):
        xyz = m.xyz.astype(np.float64)
        if tr is not None:
            ax, ang, shift = np.asarray(tr[0]), tr[1], np.asarray(tr[2])
            c = xyz.mean(0)
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            Rm = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
            xyz = (xyz - c) @ Rm.T + c + shift
        mols.append(workloads.Molecule(xyz.astype(np.float32), m.types, m.charges, m.radii, m.segments,
                                       m.all_flexible, m.crowder, m.chain_ids, m.res_seq))
    return mols


def oracle_energy(wl, sim, mols, mode):
    o = OracleRemc(mols, wl.lj_raw, sim.box, sim.temperatures[:1], sim.translate_steps[:1], sim.rotate_steps[:1],
                   sim.move_weights, sim.rigid_rotate_prob, wl.torsion_V, wl.torsion_phase, mode=mode)
    return o.initial_energy


@pytest.mark.parametrize("cfg", ["c0", "c1", "c2", "c4"])
def test_oracle_matches_reference_fixtures(cfg):
    wl = fixture_workload(cfg)
    sim = wl.sims[0]
    for st in GOLD["configs"][cfg]:
        mols = perturbed(sim, st["transforms"])
        e_ref = st["total_kcal"]
        assert oracle_energy(wl, sim, mols, oracle.REF) == pytest.approx(e_ref, rel=1e-9, abs=1e-12)
        assert oracle_energy(wl, sim, mols, oracle.FP64) == pytest.approx(e_ref, rel=1e-5, abs=1e-9)


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference tree not mounted")


@needs_ref
def test_reference_layout_matches_library():
    cgppd_gb300.build()
    assert ref.lib().ref_lj_offset() == cgppd_gb300.lib().cgppd_aminoacids_lj_offset() == 960


@needs_ref
def test_reference_conformations_through_reference_code(refdata):
    kat = refdata["kats"]["reference_conformations_exact"]
    for i in range(1, 11):
        mols = []
        for key in ("conf%d/1a" % i, "conf%d/1b" % i):
            rec = refdata["pdbs"][key]
            aa = np.array([r["aa"] for r in rec["residues"]], np.int32)
            mols.append(workloads.Molecule(np.array([r["xyz"] for r in rec["residues"]], np.float32), aa,
                                           [refdata["amino_acids"][a]["charge"] for a in aa],
                                           [refdata["amino_acids"][a]["radius"] for a in aa],
                                           res_seq=[r["seq"] for r in rec["residues"]]))
        raw, inter = ref.energy(mols, refdata["lj_table"], 1000.0)
        assert raw[0] * oracle.RT_TO_KCAL == pytest.approx(kat[i - 1][0], rel=2e-5, abs=1e-9)
        assert raw[1] * oracle.DH_FACTOR == pytest.approx(kat[i - 1][1], rel=2e-5, abs=1e-9)
        lj, dh = oracle.E_inter(oracle.REF, oracle.build_replica(["conf%d/1a" % i, "conf%d/1b" % i], refdata,
                                                                  1000.0), refdata["lj_table"], 1000.0)
        assert lj == pytest.approx(raw[0], rel=1e-12, abs=1e-15)
        assert dh == pytest.approx(raw[1], rel=1e-12, abs=1e-15)


@needs_ref
@pytest.mark.parametrize("cfg", ["c1", "c4"])
def test_live_reference_energies(cfg):
    wl = workloads.make(cfg)
    sim = wl.sims[0]
    raw, _ = ref.energy(sim.molecules, wl.lj_raw, sim.box, wl.torsion_V, wl.torsion_phase)
    e_ref = oracle.total(raw, cfg == "c1")
    assert oracle_energy(wl, sim, sim.molecules, oracle.REF) == pytest.approx(e_ref, rel=1e-12)


@needs_ref
def test_reference_graph_matches_oracle_and_library(refdata):
    cases = [
        (["A"] * 76 + ["B"] * 76, False, [[72, 73, 74, 75, 123], [148, 149, 150, 151]], 2),
        (["A"] * 162, False, [list(range(75, 87))], 1),
        (["A"] * 10, True, [], 1),
        (["A"] * 30 + ["B"] * 30, False, [[28, 29, 30, 31], [5, 40]], 2),
    ]
    L = cgppd_gb300.lib()
    for chains, allflex, segs, nch in cases:
        r = ref.graph(chains, allflex, segs, nch)
        g = oracle.Graph(chains, allflex, segs, nch)
        assert r["bonds"] == g.bonds and r["angles"] == g.angles and r["torsions"] == g.torsions
        assert r["indirect"] == g.indirect_neighbours
        assert r["counts"][3:] == [len(g.rigid_domains), len(g.segment_bonds), len(g.indirect_neighbours),
                                   len(g.MC_local_residues), len(g.MC_crankshaft_residues), len(g.MC_flex_residues)]
        lib_counts = cgppd_graph_counts(L, chains, allflex, segs, nch)
        assert lib_counts == r["counts"]


def cgppd_graph_counts(L, chains, allflex, segs, nch):
    import ctypes
    seglen = np.ascontiguousarray([len(x) for x in segs] or [0], np.int32)
    segres = np.ascontiguousarray([v for x in segs for v in x] or [0], np.int32)
    out = np.zeros(9, np.int32)
    f = L.cgppd_graph_counts
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p]
    assert f(len(chains), "".join(chains).encode(), int(allflex), len(segs), seglen.ctypes.data, segres.ctypes.data,
             nch, out.ctypes.data) == 0
    return out.tolist()
