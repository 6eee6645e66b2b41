"""Python driver of the oracle's replica-exchange restatement (cgppd_oracle_mc.c).

TEST INFRASTRUCTURE ONLY (tests/ and bench.py's CPU-baseline leg).  The graph data
(bonds, angles, torsions, indirect neighbours, flex branches, local and crankshaft
sets) is derived here with the oracle's own restatement of Graph (oracle.Graph), not
taken from the engine, so a graph bug in either shows up as a mismatch.
"""
import ctypes

import numpy as np

from . import Graph, lib

c_int, c_float, c_double = ctypes.c_int, ctypes.c_float, ctypes.c_double
P = ctypes.POINTER


class OracleSystem(ctypes.Structure):
    _fields_ = [("N", c_int), ("M", c_int), ("mstart", P(c_int)), ("mcount", P(c_int)), ("mflags", P(c_int)),
                ("aa", P(c_int)), ("q", P(c_float)), ("sig", P(c_float)), ("table", P(c_float)), ("ntypes", c_int),
                ("box", c_float), ("excl", P(c_int)),
                ("ind_off", P(c_int)), ("nind", P(c_int)), ("ind", P(c_int)),
                ("bond_off", P(c_int)), ("nbond", P(c_int)), ("bonds", P(c_int)),
                ("ang_off", P(c_int)), ("nang", P(c_int)), ("angles", P(c_int)),
                ("tor_off", P(c_int)), ("ntor", P(c_int)), ("tors", P(c_int)),
                ("torsV", P(c_double)), ("torsS", P(c_double)), ("tors_types", c_int),
                ("flex_off", P(c_int)), ("nflex", P(c_int)), ("flexres", P(c_int)), ("flexopt", P(c_int)),
                ("branch", P(c_int)), ("local_off", P(c_int)), ("nlocal", P(c_int)), ("localres", P(c_int)),
                ("crank_off", P(c_int)), ("ncrank", P(c_int)), ("crankres", P(c_int)),
                ("w_cum", c_float * 4), ("w1_cum", c_float * 3), ("rigid_rotate_p", c_float),
                ("non_crowders", c_int), ("nc_mode", c_int), ("sample_freq", c_int), ("sample_after", c_int),
                ("bound_threshold", c_float), ("rep_crowd", c_int)]


class OracleStats(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("accept", "acceptA", "reject", "totalAcceptReject", "totalAccept",
                                     "boundSamples", "samplesSinceLastExchange", "totalBoundSamples",
                                     "totalSamples")] + \
               [(n, c_float) for n in ("acceptanceRatio", "accumulativeAcceptanceRatio", "fractionBound",
                                       "accumulativeFractionBound")] + [("pad", c_int * 3)]


class OracleReplicas(ctypes.Structure):
    _fields_ = [("R", c_int), ("pos", P(c_float)), ("rel", P(c_float)), ("center", P(c_float)),
                ("potential", P(c_double)), ("temperature", P(c_float)), ("tstep", P(c_float)),
                ("rstep", P(c_double)), ("tindex", P(c_int)), ("label", P(c_int)), ("slot_of_t", P(c_int)),
                ("stats", P(OracleStats)), ("stepc", P(ctypes.c_ulonglong)), ("seed_lo", ctypes.c_uint32),
                ("seed_hi", ctypes.c_uint32), ("sim_index", c_int), ("rep_off", c_int), ("mode", c_int)]


def _declare():
    L = lib()
    if not getattr(L, "_mc_declared", False):
        L.oracle_remc_run.argtypes = [P(OracleSystem), P(OracleReplicas), c_int, c_int, c_int, c_int, P(c_int),
                                      P(c_int), P(c_float), P(c_int)]
        L.oracle_remc_run.restype = c_int
        L.oracle_final_report.argtypes = [P(OracleReplicas), P(c_float)]
        L.oracle_replica_energy.argtypes = [P(OracleSystem), c_int, P(c_float), P(c_double)]
        L.oracle_replica_energy.restype = c_double
        L._mc_declared = True
    return L


def _i(a):
    return np.ascontiguousarray(a if len(a) else [0], np.int32)


def _ptr(a, t):
    return a.ctypes.data_as(P(t))


def float_mean(xyz):
    """Centre as Molecule::initFromPDB accumulates it: float sums, then a float divide."""
    c = np.zeros(3, np.float32)
    for p in np.asarray(xyz, np.float32):
        c = (c + p).astype(np.float32)
    return (c / np.float32(len(xyz))).astype(np.float32)


class OracleRemc:
    """One simulation's replicas in the oracle."""

    def __init__(self, molecules, table, box, temperatures, translate_steps, rotate_steps, move_weights=(1, 1, 1, 1),
                 rigid_rotate_prob=0.5, torsion_V=None, torsion_phase=None, seed=20261203, mode=0,
                 sample_frequency=0, sample_after=0, bound_threshold=-1.1844, rep_off=0, sim_index=0,
                 repulsive_crowding=False, centers=None, rel=None):
        """`centers` [M, 3] and `rel` [N, 3] give the molecules' centres and relative
        positions where they are not the float mean of the coordinates and the
        differences from it (a state loaded from the reference's own run)."""
        L = _declare()
        self.L = L
        self.keep = []
        M = len(molecules)
        N = sum(m.n for m in molecules)
        self.N, self.M = N, M
        mstart = np.cumsum([0] + [m.n for m in molecules[:-1]]).astype(np.int32)
        mcount = np.array([m.n for m in molecules], np.int32)
        mflags = np.array([(1 if (m.all_flexible or m.segments) else 0) | (2 if m.crowder else 0)
                           for m in molecules], np.int32)
        aa = np.concatenate([m.types for m in molecules]).astype(np.int32)
        q = np.concatenate([m.charges for m in molecules]).astype(np.float32)
        sig = np.concatenate([m.radii for m in molecules]).astype(np.float32)
        tab = np.ascontiguousarray(table, np.float32)
        excl = np.zeros((N, 4), np.int32)
        lists = {k: [] for k in ("ind", "bond", "ang", "tor", "flexres", "flexopt", "branch", "local", "crank")}
        offs = {k: [] for k in ("ind", "bond", "ang", "tor", "flex", "local", "crank")}
        cnts = {k: [] for k in offs}
        chain_off = dom_off = bond_off = 1
        for mi, m in enumerate(molecules):
            g = Graph(list(m.chain_ids), m.all_flexible, m.segments, 1)
            s0 = mstart[mi]
            dom_uid = np.zeros(m.n, np.int32)
            bond_uid = np.zeros(m.n, np.int32)
            for d, dom in enumerate(g.rigid_domains):
                for v in dom:
                    dom_uid[v] = dom_off + d
            dom_off += len(g.rigid_domains)
            for b, (i, j) in enumerate(g.segment_bonds):
                bond_uid[i] = bond_off + b
                bond_uid[j] = bond_off + b
            bond_off += len(g.segment_bonds)
            chain_uid = np.zeros(m.n, np.int32)
            chain_uid[:len(g.vertices)] = chain_off + np.asarray(m.chain_index[:len(g.vertices)])
            chain_off += int(np.max(m.chain_index)) + 1
            excl[s0:s0 + m.n] = np.stack([chain_uid, m.res_seq, dom_uid, bond_uid], 1)
            flexible = mflags[mi] & 1

            def add(key, items, width):
                offs[key].append(len(lists[key if key != "flex" else "flexres"]) // width)
                cnts[key].append(len(items))

            if flexible:
                ind = sorted(g.indirect_neighbours)
                offs["ind"].append(len(lists["ind"]) // 2)
                cnts["ind"].append(len(ind))
                lists["ind"] += [v for p in ind for v in p]
                bonds = sorted(g.bonds)
                offs["bond"].append(len(lists["bond"]) // 2)
                cnts["bond"].append(len(bonds))
                lists["bond"] += [v for p in bonds for v in p]
                angles = sorted(g.angles)
                offs["ang"].append(len(lists["ang"]) // 3)
                cnts["ang"].append(len(angles))
                lists["ang"] += [v for p in angles for v in p]
                tors = sorted(g.torsions)
                offs["tor"].append(len(lists["tor"]) // 4)
                cnts["tor"].append(len(tors))
                lists["tor"] += [v for p in tors for v in p]
                offs["flex"].append(len(lists["flexres"]) // 3)
                cnts["flex"].append(len(g.MC_flex_residues))
                for ri in g.MC_flex_residues:
                    nb = g.neighbours(ri)
                    lists["flexres"] += [ri, len(nb), len(lists["flexopt"]) // 3]
                    dom = g.rigid_domain_around(ri)
                    for nbr in nb:
                        br = set(g.branch(ri, nbr))
                        if nbr in dom:
                            for other in nb:
                                if other != nbr and other in dom:
                                    br |= g.branch(ri, other)
                        lists["flexopt"] += [nbr, len(lists["branch"]), len(br)]
                        lists["branch"] += sorted(br)
                offs["local"].append(len(lists["local"]))
                cnts["local"].append(len(g.MC_local_residues))
                lists["local"] += list(g.MC_local_residues)
                offs["crank"].append(len(lists["crank"]))
                cnts["crank"].append(len(g.MC_crankshaft_residues))
                lists["crank"] += list(g.MC_crankshaft_residues)
            else:
                for k in offs:
                    offs[k].append(0)
                    cnts[k].append(0)
        arrs = {k: _i(v) for k, v in lists.items()}
        offa = {k: _i(v) for k, v in offs.items()}
        cnta = {k: _i(v) for k, v in cnts.items()}
        if torsion_V is not None:
            V = np.ascontiguousarray(torsion_V, np.float64)
            S = np.ascontiguousarray(torsion_phase, np.float64)
            tt = V.shape[0]
        else:
            V = np.zeros(4, np.float64)
            S = np.zeros(4, np.float64)
            tt = 1
        # cumulative move weights, normalised in float
        w = [np.float32(v) for v in move_weights]
        wsum = np.float32(w[0] + w[1] + w[2] + w[3])
        w_cum, acc = [], np.float32(0)
        for v in w:
            acc = np.float32(acc + v)
            w_cum.append(np.float32(acc / wsum))
        w1s = np.float32(w[1] + w[2] + w[3])
        w1_cum = [np.float32(w[1] / w1s), np.float32(np.float32(w[1] + w[2]) / w1s), np.float32(1.0)]
        non_crowders = 0
        for m in molecules:
            if m.crowder:
                break
            non_crowders += 1
        flexible_exists = any(bool(m.all_flexible or m.segments) for m in molecules)
        nc_mode = 0 if M == 1 else (1 if (M != non_crowders or flexible_exists) else 2)
        self.keep += [mstart, mcount, mflags, aa, q, sig, tab, excl, V, S] + list(arrs.values()) + \
            list(offa.values()) + list(cnta.values())
        self.sys = OracleSystem(
            N, M, _ptr(mstart, c_int), _ptr(mcount, c_int), _ptr(mflags, c_int), _ptr(aa, c_int), _ptr(q, c_float),
            _ptr(sig, c_float), _ptr(tab, c_float), tab.shape[0], float(box), _ptr(excl, c_int),
            _ptr(offa["ind"], c_int), _ptr(cnta["ind"], c_int), _ptr(arrs["ind"], c_int),
            _ptr(offa["bond"], c_int), _ptr(cnta["bond"], c_int), _ptr(arrs["bond"], c_int),
            _ptr(offa["ang"], c_int), _ptr(cnta["ang"], c_int), _ptr(arrs["ang"], c_int),
            _ptr(offa["tor"], c_int), _ptr(cnta["tor"], c_int), _ptr(arrs["tor"], c_int),
            _ptr(V, c_double), _ptr(S, c_double), tt,
            _ptr(offa["flex"], c_int), _ptr(cnta["flex"], c_int), _ptr(arrs["flexres"], c_int),
            _ptr(arrs["flexopt"], c_int), _ptr(arrs["branch"], c_int),
            _ptr(offa["local"], c_int), _ptr(cnta["local"], c_int), _ptr(arrs["local"], c_int),
            _ptr(offa["crank"], c_int), _ptr(cnta["crank"], c_int), _ptr(arrs["crank"], c_int),
            (c_float * 4)(*w_cum), (c_float * 3)(*w1_cum), float(rigid_rotate_prob), non_crowders, nc_mode,
            int(sample_frequency), int(sample_after), float(bound_threshold), int(bool(repulsive_crowding)))
        # replicas: every slot starts from the same coordinates
        R = len(temperatures)
        self.R = R
        xyz = np.concatenate([np.asarray(m.xyz, np.float32) for m in molecules])
        cen = np.stack([float_mean(m.xyz) for m in molecules]).astype(np.float32) if centers is None else \
            np.ascontiguousarray(centers, np.float32).reshape(M, 3)
        rel = np.concatenate([(np.asarray(m.xyz, np.float32) - cen[k]).astype(np.float32)
                              for k, m in enumerate(molecules)]) if rel is None else \
            np.ascontiguousarray(rel, np.float32).reshape(N, 3)
        self.pos = np.ascontiguousarray(np.broadcast_to(xyz, (R, N, 3)).copy())
        self.rel = np.ascontiguousarray(np.broadcast_to(rel, (R, N, 3)).copy())
        self.center = np.ascontiguousarray(np.broadcast_to(cen, (R, M, 3)).copy())
        e0 = L.oracle_replica_energy(ctypes.byref(self.sys), mode, _ptr(self.pos[0], c_float), None)
        self.potential = np.full(R, e0, np.float64)
        self.temperature = np.ascontiguousarray(temperatures, np.float32).copy()
        self.tstep = np.ascontiguousarray(translate_steps, np.float32)
        self.rstep = np.ascontiguousarray(rotate_steps, np.float64)
        self.tindex = np.arange(R, dtype=np.int32)
        self.label = np.arange(R, dtype=np.int32)
        self.slot_of_t = np.arange(R, dtype=np.int32)
        self.stats = (OracleStats * R)()
        self.stepc = np.zeros(R, np.uint64)
        self.x = c_int(0)
        self.offset = c_int(0)
        self.reps = OracleReplicas(R, _ptr(self.pos, c_float), _ptr(self.rel, c_float), _ptr(self.center, c_float),
                                   _ptr(self.potential, c_double), _ptr(self.temperature, c_float),
                                   _ptr(self.tstep, c_float), _ptr(self.rstep, c_double), _ptr(self.tindex, c_int),
                                   _ptr(self.label, c_int), _ptr(self.slot_of_t, c_int), self.stats,
                                   _ptr(self.stepc, ctypes.c_ulonglong), seed & 0xffffffff, (seed >> 32) & 0xffffffff,
                                   sim_index, rep_off, mode)
        self.mode = mode
        self.initial_energy = e0

    def run(self, n_blocks, steps_per_block, exchange_after_last=True, threads=1):
        reports = np.zeros((n_blocks, self.R, 4), np.float32)
        exch = np.zeros((n_blocks, 2), np.int32)
        self.L.oracle_remc_run(ctypes.byref(self.sys), ctypes.byref(self.reps), n_blocks, steps_per_block,
                               int(bool(exchange_after_last)), threads, ctypes.byref(self.x),
                               ctypes.byref(self.offset), _ptr(reports, c_float), _ptr(exch, c_int))
        return reports, exch

    def final_report(self):
        out = np.zeros((self.R, 4), np.float32)
        self.L.oracle_final_report(ctypes.byref(self.reps), _ptr(out, c_float))
        return out

    def energy(self, slot, mode=None):
        nc = c_double()
        e = self.L.oracle_replica_energy(ctypes.byref(self.sys), self.mode if mode is None else mode,
                                         _ptr(np.ascontiguousarray(self.pos[slot]), c_float), ctypes.byref(nc))
        return e, nc.value

    def energy_of(self, xyz, mode=1):
        """Total energy (kcal/mol) of arbitrary coordinates [N,3] of this system."""
        x = np.ascontiguousarray(xyz, np.float32)
        return self.L.oracle_replica_energy(ctypes.byref(self.sys), mode, _ptr(x, c_float), None)

    def counters(self):
        return {n: np.array([getattr(self.stats[i], n) for i in range(self.R)])
                for n, _ in OracleStats._fields_ if n != "pad"}
