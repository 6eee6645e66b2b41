"""CPU oracle for the CGPPD hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import
this package, and only as the checker (or as the timed CPU baseline).  The product
(``cgppd_gb300``) never imports it.

Contents:
* ctypes bindings to ``cgppd_oracle.c`` (energies, Philox) and ``cgppd_oracle_mc.c``
  (the reference CPU Monte Carlo loop);
* a Python restatement of the reference's molecule model: PDB centring
  (src/Molecule.cpp:506-612), the flexible-segment graph (src/Geometry.cpp:34-302),
  replica-wide UIDs and the float packing of the GPU upload
  (src/Residue.cpp:41-59, src/Replica.cpp:705-830).

Parity: the energy functions are pinned against the reference tests' golden values
(tests/testReferenceConformations.cpp, tests/testReplica.cpp, tests/testMolecule.cpp)
and the graph against tests/testGeometry.cpp; see tests/test_oracle_golden.py.
"""
import ctypes
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_data.json")

REF, FP64 = 0, 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        from .build_oracle import build
        L = ctypes.CDLL(build())
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        c_int, c_float = ctypes.c_int, ctypes.c_float
        L.oracle_E_inter.argtypes = [c_int, c_int, i32p, i32p, f32p, i32p, f32p, f32p, f32p, c_int, c_float,
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.oracle_E_inter_matrix.argtypes = [c_int, c_int, i32p, i32p, f32p, i32p, f32p, f32p, f32p, c_int,
                                            c_float, f64p]
        L.oracle_E_intra.argtypes = [c_int, c_int, f32p, i32p, f32p, f32p, i32p, c_int, i32p, c_int, i32p, c_int,
                                     i32p, c_int, i32p, f64p, f64p, c_int, f32p, c_int, c_float, c_int, f64p]
        L.oracle_E_packed.argtypes = [c_int, c_int, c_int, f32p, f32p, f32p, c_float, f64p]
        L.oracle_E_packed_rc.argtypes = [c_int, c_int, c_int, c_int, f32p, f32p, f32p, c_float, f64p]
        L.oracle_E_inter_matrix_rc.argtypes = [c_int, c_int, i32p, i32p, i32p, f32p, i32p, f32p, f32p, f32p, c_int,
                                               c_float, f64p]
        L.or_crowder_term.argtypes = [c_int, ctypes.c_double]
        L.or_crowder_term.restype = ctypes.c_double
        L.oracle_total.argtypes = [f64p, c_int]
        L.oracle_total.restype = ctypes.c_double
        L.oracle_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.oracle_rt_to_kcal.restype = ctypes.c_double
        L.oracle_dh_factor.restype = ctypes.c_double
        _lib = L
    return _lib


RT_TO_KCAL = 0.59218674898147583
DH_FACTOR = 4.1507959365844727
K_SPRING = 378.0
GAMMA_RECIP = 10.0


def load_reference_data(path=GOLDEN):
    with open(path) as f:
        return json.load(f)


# ------------------------------------------------------------------ molecules

class Mol:
    """One molecule as the reference holds it after Molecule::init."""

    def __init__(self, residues, chains, aa_table, box, all_flexible=False, segments=(), crowder=False,
                 position=None, translate=True, rotation=None):
        n = len(residues)
        self.n = n
        self.box = np.float32(box)
        self.aa = np.array([r["aa"] for r in residues], np.int32)
        self.res_seq = np.array([r["seq"] for r in residues], np.int32)
        self.chain_id = [r["chain"] for r in residues]
        self.chain_int = np.array([r["chain_index"] for r in residues], np.int32)
        self.charge = np.array([aa_table[a]["charge"] for a in self.aa], np.float32)
        self.radius = np.array([aa_table[a]["radius"] for a in self.aa], np.float32)
        pos = np.array([r["xyz"] for r in residues], np.float32)
        # centre accumulated in float, then divided (src/Molecule.cpp:590-604)
        c = np.zeros(3, np.float32)
        for p in pos:
            c = (c + p).astype(np.float32)
        c = (c / np.float32(n)).astype(np.float32)
        self.center = c
        self.rel = (pos - c).astype(np.float32)
        self.pos = pos
        self.num_chains = chains
        self.crowder = crowder
        self.all_flexible = all_flexible
        self.segments = [list(s) for s in segments]
        if position is not None:
            if translate:
                if any(position):
                    self.translate(np.array(position, np.float32))
            else:
                self.set_position(np.array(position, np.float32))
        self.graph = Graph(self.chain_id, all_flexible, self.segments, chains)
        self.is_flexible = bool(all_flexible or len(self.segments))

    def set_position(self, c):
        self.center = np.asarray(c, np.float32)
        self.pos = (self.rel + self.center).astype(np.float32)

    def translate(self, v):
        nc = (self.center + np.asarray(v, np.float32)).astype(np.float32)
        nc = np.fmod(nc, self.box).astype(np.float32)
        self.set_position(nc)


class Graph:
    """Restatement of Graph::init and helpers (src/Geometry.cpp:34-302)."""

    def __init__(self, chain_ids, all_flexible, segments, num_chains):
        self.num_chains = num_chains
        self.vertices = set()
        self.edges = set()
        self.adj = {}
        self.flex = {}
        n = len(chain_ids)
        for i in range(n - 1):
            if chain_ids[i] == chain_ids[i + 1]:
                self._add_edge(i, i + 1, all_flexible)
        for s in segments:
            for a, b in zip(s[:-1], s[1:]):
                self._add_edge(a, b, True)
        self.bonds = set()
        self.torsions = set()
        self.angles = set()
        for (j, k) in sorted(self.edges):
            if self.flex.get((j, k), False):
                self.bonds.add((j, k))
            nj, nk = self.adj[j], self.adj[k]
            if len(nj) > 1 and len(nk) > 1:
                for i in sorted(nj):
                    if i == k:
                        continue
                    for l in sorted(nk):
                        if l == j:
                            continue
                        if self.is_flexible(i, j) or self.is_flexible(j, k) or self.is_flexible(k, l):
                            self.torsions.add((i, j, k, l))
        local, crank, flexr = set(), set(), set()
        for j in sorted(self.vertices):
            nb = self.adj[j]
            has_rigid = has_flex = False
            for i in sorted(nb):
                if self.is_flexible(i, j):
                    has_flex = True
                else:
                    has_rigid = True
                for k in sorted(nb):
                    if i < k and (self.is_flexible(i, j) or self.is_flexible(j, k)):
                        self.angles.add((i, j, k))
            if not has_rigid:
                local.add(j)
                if len(nb) > 1:
                    crank.add(j)
            if has_flex:
                flexr.add(j)
        self.MC_local_residues = sorted(local)
        self.MC_crankshaft_residues = sorted(crank)
        self.MC_flex_residues = sorted(flexr)
        self.rigid_domains = []
        todo = set(self.vertices)
        while todo:
            v = min(todo)
            dom = self.rigid_domain_around(v)
            todo -= dom
            if len(dom) > 1:
                self.rigid_domains.append(dom)
        self.segment_bonds = []
        for (i, j) in sorted(self.bonds):
            if chain_ids[i] != chain_ids[j] or abs(i - j) >= 4:
                self.segment_bonds.append((i, j))
        self.indirect_neighbours = set()
        for (pi, pj) in self.segment_bonds:
            around = sorted(t for t in self.torsions if (pi in t and pj in t))
            proposed = set()
            for (ti, tj, tk, tl) in around:
                proposed.add((ti, tl))
                # The reference writes `(t->i, t->j) == (p->i, p->j)`: the comma operator
                # makes that `t->j == p->j`, and likewise for the other three tests.
                if tj == pj or ti == pj:
                    proposed.add((ti, tk))
                if tl == pj or tk == pj:
                    proposed.add((tj, tl))
            for (a, b) in proposed:
                if chain_ids[a] != chain_ids[b] or abs(a - b) >= 4:
                    self.indirect_neighbours.add((a, b) if a < b else (b, a))

    def _add_edge(self, i, j, flexible):
        self.vertices.update((i, j))
        self.edges.add((i, j) if i < j else (j, i))
        self.adj.setdefault(i, set()).add(j)
        self.adj.setdefault(j, set()).add(i)
        self.flex[(i, j)] = flexible
        self.flex[(j, i)] = flexible

    def is_flexible(self, i, j):
        return self.flex.get((i, j), False)

    def neighbours(self, i):
        return sorted(self.adj.get(i, ()))

    def branch(self, i, j, visited=frozenset()):
        out = [(j, k) for k in sorted(self.adj.get(j, ())) if k != i and (j, k) not in visited]
        br = {i, j}
        nv = visited | {(i, j)}
        for (a, b) in out:
            br |= self.branch(a, b, nv)
        return br

    def rigid_domain_around(self, i, visited=frozenset()):
        out = [j for j in sorted(self.adj.get(i, ())) if not self.is_flexible(i, j) and (j, i) not in visited]
        dom = {i}
        for j in out:
            dom |= self.rigid_domain_around(j, visited | {(i, j)})
        return dom


def assign_uids(mols):
    """Graph::assign_uids over a replica (src/Geometry.cpp:256-302, src/Replica.cpp:33-40):
    replica-wide chain/domain/bond UIDs per residue and the packed GPU floats."""
    chain_off = dom_off = bond_off = 1
    for m in mols:
        g = m.graph
        chain_uid = {c: chain_off + c for c in range(g.num_chains)}
        chain_off += g.num_chains
        dom_uid = {d: dom_off + d for d in range(len(g.rigid_domains))}
        dom_off += len(g.rigid_domains)
        bond_uid = {b: bond_off + b for b in range(len(g.segment_bonds))}
        bond_off += len(g.segment_bonds)
        m.domain_uid = np.zeros(m.n, np.int32)
        m.bond_uid = np.zeros(m.n, np.int32)
        m.chain_uid = np.zeros(m.n, np.int32)
        for d, dom in enumerate(g.rigid_domains):
            for i in dom:
                m.domain_uid[i] = dom_uid[d]
        for b, (i, j) in enumerate(g.segment_bonds):
            m.bond_uid[i] = bond_uid[b]
            m.bond_uid[j] = bond_uid[b]
        m.pos_w = np.zeros(m.n, np.float32)
        m.meta_w = np.zeros(m.n, np.float32)
        for i in range(len(g.vertices)):
            m.chain_uid[i] = chain_uid.get(int(m.chain_int[i]), 0)
            bf = 0.0
            if m.bond_uid[i]:
                bf = m.bond_uid[i] / (2.0 ** math.ceil(math.log2(bond_off + 1)))
            cf = m.chain_uid[i] / (2.0 ** math.ceil(math.log2(chain_off + 1)))
            m.pos_w[i] = np.float32(np.float32(m.domain_uid[i]) + np.float32(bf))
            m.meta_w[i] = np.float32(np.float32(m.index) + np.float32(cf))


def pack_replica(mols, block=32, rigid_only=False):
    """ReplicaDataToDevice packing (src/Replica.cpp:705-798): float4 pos/meta, padded
    to a multiple of `block` with w = -2 / type 20."""
    n = sum(m.n for m in mols)
    P = int(math.ceil(n / block)) * block
    pos = np.zeros((P, 4), np.float32)
    meta = np.zeros((P, 4), np.float32)
    k = 0
    for mi, m in enumerate(mols):
        for i in range(m.n):
            pos[k, :3] = m.pos[i]
            w = m.pos_w[i]
            if rigid_only:
                w = np.float32(w - np.float32(int(w)))
                w = np.float32(w + np.float32(mi) + np.float32(1.0))
            pos[k, 3] = w
            meta[k] = (m.aa[i], m.charge[i], m.radius[i], -1.0 if m.crowder else m.meta_w[i])
            k += 1
    pos[k:, 3] = -2.0
    meta[k:, 0] = 20.0
    return pos, meta


def build_replica(pdb_keys, data, box, segments=None, all_flexible=None, crowders=None):
    """Molecules loaded like Replica::init_first_replica with `translate=true` and zero
    offsets (the reference tests' set-up)."""
    mols = []
    for idx, key in enumerate(pdb_keys):
        rec = data["pdbs"][key]
        segs = (segments or {}).get(idx, [])
        af = bool((all_flexible or {}).get(idx, False))
        m = Mol(rec["residues"], rec["chains"], data["amino_acids"], box, all_flexible=af, segments=segs,
                crowder=bool((crowders or {}).get(idx, False)))
        m.index = idx
        mols.append(m)
    assign_uids(mols)
    return mols


# ------------------------------------------------------------------ energies

def _concat(mols):
    xyz = np.ascontiguousarray(np.concatenate([m.pos for m in mols]).astype(np.float32).reshape(-1))
    aa = np.ascontiguousarray(np.concatenate([m.aa for m in mols]).astype(np.int32))
    q = np.ascontiguousarray(np.concatenate([m.charge for m in mols]).astype(np.float32))
    s = np.ascontiguousarray(np.concatenate([m.radius for m in mols]).astype(np.float32))
    start = np.cumsum([0] + [m.n for m in mols[:-1]]).astype(np.int32)
    cnt = np.array([m.n for m in mols], np.int32)
    return xyz, aa, q, s, start, cnt


def E_inter(mode, mols, table, box):
    """Replica::E(): (LJ raw, DH raw) over all inter-molecule residue pairs."""
    xyz, aa, q, s, start, cnt = _concat(mols)
    t = np.ascontiguousarray(np.asarray(table, np.float32).reshape(-1))
    nt = int(round(math.sqrt(t.size)))
    lj, dh = ctypes.c_double(), ctypes.c_double()
    lib().oracle_E_inter(mode, len(mols), start, cnt, xyz, aa, q, s, t, nt, float(box), ctypes.byref(lj),
                         ctypes.byref(dh))
    return lj.value, dh.value


def E_inter_arrays(mode, xyz, aa, q, s, start, cnt, table, box):
    t = np.ascontiguousarray(np.asarray(table, np.float32).reshape(-1))
    nt = int(round(math.sqrt(t.size)))
    lj, dh = ctypes.c_double(), ctypes.c_double()
    lib().oracle_E_inter(mode, len(start), np.ascontiguousarray(start, np.int32), np.ascontiguousarray(cnt, np.int32),
                         np.ascontiguousarray(xyz, np.float32).reshape(-1), np.ascontiguousarray(aa, np.int32),
                         np.ascontiguousarray(q, np.float32), np.ascontiguousarray(s, np.float32), t, nt, float(box),
                         ctypes.byref(lj), ctypes.byref(dh))
    return lj.value, dh.value


def E_inter_matrix(mode, xyz, aa, q, s, start, cnt, table, box):
    t = np.ascontiguousarray(np.asarray(table, np.float32).reshape(-1))
    nt = int(round(math.sqrt(t.size)))
    M = len(start)
    out = np.zeros(M * M, np.float64)
    lib().oracle_E_inter_matrix(mode, M, np.ascontiguousarray(start, np.int32), np.ascontiguousarray(cnt, np.int32),
                                np.ascontiguousarray(xyz, np.float32).reshape(-1), np.ascontiguousarray(aa, np.int32),
                                np.ascontiguousarray(q, np.float32), np.ascontiguousarray(s, np.float32), t, nt,
                                float(box), out)
    return out.reshape(M, M)


def E_inter_matrix_rc(mode, xyz, aa, q, s, start, cnt, crowder, table, box):
    """E_inter_matrix under repulsive crowding (crowder: per-molecule flags)."""
    t = np.ascontiguousarray(np.asarray(table, np.float32).reshape(-1))
    nt = int(round(math.sqrt(t.size)))
    M = len(start)
    out = np.zeros(M * M, np.float64)
    lib().oracle_E_inter_matrix_rc(mode, M, np.ascontiguousarray(start, np.int32),
                                   np.ascontiguousarray(cnt, np.int32), np.ascontiguousarray(crowder, np.int32),
                                   np.ascontiguousarray(xyz, np.float32).reshape(-1),
                                   np.ascontiguousarray(aa, np.int32), np.ascontiguousarray(q, np.float32),
                                   np.ascontiguousarray(s, np.float32), t, nt, float(box), out)
    return out.reshape(M, M)


def crowder_term(mode, r):
    """Repulsive crowder pair term in RT units (REPULSIVE_CROWDING builds)."""
    return lib().or_crowder_term(mode, float(r))


def intra_inputs(m):
    g = m.graph
    excl = np.ascontiguousarray(np.stack([m.chain_uid, m.res_seq, m.domain_uid, m.bond_uid], 1).astype(np.int32))
    ind = np.ascontiguousarray(np.array(sorted(g.indirect_neighbours), np.int32).reshape(-1))
    bonds = np.ascontiguousarray(np.array(sorted(g.bonds), np.int32).reshape(-1))
    angles = np.ascontiguousarray(np.array(sorted(g.angles), np.int32).reshape(-1))
    tors = np.ascontiguousarray(np.array(sorted(g.torsions), np.int32).reshape(-1))
    return excl, ind, bonds, angles, tors


def E_intra(mode, m, data, include_lj_dh=True, table=None, torsV=None, torsS=None, xyz=None):
    """Molecule::E(include): raw (LJ, DH, bond, angle product, torsion)."""
    excl, ind, bonds, angles, tors = intra_inputs(m)
    t = np.ascontiguousarray(np.asarray(table if table is not None else data["lj_table"], np.float32).reshape(-1))
    nt = int(round(math.sqrt(t.size)))
    V = np.ascontiguousarray(np.asarray(torsV if torsV is not None else data["torsion_V"], np.float64).reshape(-1))
    S = np.ascontiguousarray(np.asarray(torsS if torsS is not None else data["torsion_sigma"], np.float64).reshape(-1))
    ntt = int(round(math.sqrt(V.size // 4)))
    out = np.zeros(5, np.float64)
    pos = np.ascontiguousarray((m.pos if xyz is None else xyz).astype(np.float32).reshape(-1))
    lib().oracle_E_intra(mode, m.n, pos, m.aa, m.charge, m.radius, excl, len(ind) // 2, ind, len(bonds) // 2, bonds,
                         len(angles) // 3, angles, len(tors) // 4, tors, V, S, ntt, t, nt, float(m.box),
                         1 if include_lj_dh else 0, out)
    return out


def E_packed(mode, pos4, meta4, table20, box, nc=False, P=None, repulsive_crowding=False):
    """Reference GPU pair rules on packed arrays: (LJ raw, DH raw, total kcal/mol)."""
    pos4 = np.ascontiguousarray(pos4, np.float32)
    meta4 = np.ascontiguousarray(meta4, np.float32)
    out = np.zeros(3, np.float64)
    lib().oracle_E_packed_rc(mode, 1 if nc else 0, 1 if repulsive_crowding else 0,
                             int(P if P is not None else pos4.shape[0]), pos4.reshape(-1), meta4.reshape(-1),
                             np.ascontiguousarray(np.asarray(table20, np.float32).reshape(-1)), float(box), out)
    return out


def total(raw5, flexible=True):
    return lib().oracle_total(np.ascontiguousarray(raw5, np.float64), 1 if flexible else 0)


def kcal(raw5):
    """Component values in kcal/mol from raw accumulators."""
    lj, dh, b, a, t = raw5
    return np.array([lj * RT_TO_KCAL, dh * DH_FACTOR, b * 0.5 * K_SPRING,
                     math.log(a) * -GAMMA_RECIP if a > 0 else float("inf"), t])


def raw_from_kcal(k5):
    lj, dh, b, a, t = k5
    return np.array([lj / RT_TO_KCAL, dh / DH_FACTOR, b / (0.5 * K_SPRING), math.exp(a / -GAMMA_RECIP), t])


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().oracle_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out
