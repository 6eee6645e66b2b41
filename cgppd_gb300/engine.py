"""ctypes view of the batched REMC engine (include/cgppd_remc.h).

Thin: argument marshalling only.  Everything runs in the native library.
"""
import ctypes

import numpy as np

from . import CgppdError, check, lib

c_int, c_float, c_double, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p
P = ctypes.POINTER


class SimParams(ctypes.Structure):
    _fields_ = [("n_replicas", c_int), ("box", c_float), ("temperatures", P(c_float)),
                ("translate_steps", P(c_float)), ("rotate_steps", P(c_double)), ("move_weights", c_float * 4),
                ("rigid_rotate_prob", c_float), ("sample_frequency", c_int), ("sample_after", c_int),
                ("bound_threshold", c_float), ("rigid_only", c_int), ("repulsive_crowding", c_int)]


_DECL = {
    "cgppd_engine_create": (c_void_p, [P(c_float), c_int, P(c_double), P(c_double), c_int, ctypes.c_uint64]),
    "cgppd_engine_destroy": (None, [c_void_p]),
    "cgppd_engine_add_simulation": (c_int, [c_void_p, P(SimParams)]),
    "cgppd_engine_add_molecule": (c_int, [c_void_p, c_int, c_int, P(c_float), P(c_int), P(c_float), P(c_float),
                                          ctypes.c_char_p, P(c_int), P(c_int), c_int, c_int, c_int, c_int, P(c_int),
                                          P(c_int), P(c_float)]),
    "cgppd_engine_finalize": (c_int, [c_void_p, c_int, c_int]),
    "cgppd_engine_run": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p]),
    "cgppd_engine_final_report": (c_int, [c_void_p, c_int, c_void_p]),
    "cgppd_engine_synchronize": (c_int, [c_void_p]),
    "cgppd_engine_total_replicas": (c_int, [c_void_p]),
    "cgppd_engine_sim_info": (c_int, [c_void_p, c_int, P(c_int), P(c_int), P(c_int)]),
    "cgppd_engine_recompute": (c_int, [c_void_p, P(c_double), c_int]),
    "cgppd_engine_get_replicas": (c_int, [c_void_p, c_int, P(c_double), P(c_float), P(c_int), P(c_int), P(c_int)]),
    "cgppd_engine_get_state": (c_int, [c_void_p, c_int, c_int, P(c_float), P(c_float), P(c_float)]),
    "cgppd_engine_set_state": (c_int, [c_void_p, c_int, c_int, P(c_float), P(c_float), P(c_float)]),
    "cgppd_engine_get_matrix": (c_int, [c_void_p, c_int, c_int, P(c_double), P(c_double)]),
    "cgppd_engine_upload": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "cgppd_engine_download": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "cgppd_engine_get_report": (c_int, [c_void_p, c_int, c_int, P(c_float), P(c_int)]),
    "cgppd_engine_counters": (c_int, [c_void_p, P(ctypes.c_ulonglong), P(ctypes.c_ulonglong)]),
    "cgppd_engine_error_bits": (ctypes.c_uint, [c_void_p]),
    "cgppd_engine_replica_error_bits": (c_int, [c_void_p, c_int, P(ctypes.c_uint)]),
    "cgppd_engine_last_launches": (c_int, [c_void_p]),
    "cgppd_engine_launch_shape": (c_int, [c_void_p, P(c_int), P(c_int)]),
    "cgppd_engine_set_resident": (c_int, [c_void_p, c_int]),
    "cgppd_engine_checkpoint": (c_int, [c_void_p, ctypes.c_char_p]),
    "cgppd_engine_restore": (c_int, [c_void_p, ctypes.c_char_p]),
    "cgppd_engine_set_sample_log": (c_int, [c_void_p, c_int]),
    "cgppd_engine_take_samples": (c_int, [c_void_p, c_int, P(c_int), P(ctypes.c_double), P(ctypes.c_double),
                                          P(c_float), P(c_int)]),
    "cgppd_engine_set_sample_snapshots": (c_int, [c_void_p, c_int]),
    "cgppd_engine_take_sample_xyz": (c_int, [c_void_p, c_int, P(c_float)]),
}


def _L():
    L = lib()
    if not getattr(L, "_engine_declared", False):
        for name, (res, args) in _DECL.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L._engine_declared = True
    return L


def _p(arr, ctype):
    return arr.ctypes.data_as(P(ctype))


def _ok(rc, where):
    if rc < 0:
        check(where)
        raise CgppdError(where + " failed")
    return rc


class Engine:
    """All replicas of one or more simulations resident on the current GPU."""

    def __init__(self, lj_raw, torsion_V=None, torsion_phase=None, seed=20261203):
        L = _L()
        t = np.ascontiguousarray(lj_raw, np.float32)
        nt = t.shape[0]
        self._keep = []
        V = S = None
        tt = 0
        if torsion_V is not None:
            V = np.ascontiguousarray(torsion_V, np.float64)
            S = np.ascontiguousarray(torsion_phase, np.float64)
            tt = V.shape[0]
        h = L.cgppd_engine_create(_p(t, c_float), nt, _p(V, c_double) if V is not None else None,
                                  _p(S, c_double) if S is not None else None, tt, ctypes.c_uint64(seed))
        if not h:
            check("cgppd_engine_create")
            raise CgppdError("cgppd_engine_create failed")
        self.h = h
        self.sims = []

    def close(self):
        if getattr(self, "h", None):
            _L().cgppd_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_simulation(self, temperatures, translate_steps, rotate_steps, box, move_weights=(1, 1, 1, 1),
                       rigid_rotate_prob=0.5, sample_frequency=0, sample_after=0, bound_threshold=-1.1844,
                       rigid_only=False, repulsive_crowding=False):
        T = np.ascontiguousarray(temperatures, np.float32)
        ts = np.ascontiguousarray(translate_steps, np.float32)
        rs = np.ascontiguousarray(rotate_steps, np.float64)
        p = SimParams(len(T), float(box), _p(T, c_float), _p(ts, c_float), _p(rs, c_double),
                      (c_float * 4)(*move_weights), float(rigid_rotate_prob), int(sample_frequency),
                      int(sample_after), float(bound_threshold), int(bool(rigid_only)),
                      int(bool(repulsive_crowding)))
        sim = _ok(_L().cgppd_engine_add_simulation(self.h, ctypes.byref(p)), "add_simulation")
        self.sims.append(len(T))
        return sim

    def add_molecule(self, sim, xyz, types, charges, radii, chain_ids=None, res_seq=None, chain_index=None,
                     num_chains=1, all_flexible=False, crowder=False, segments=(), center=None):
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1)
        n = xyz.size // 3
        types = np.ascontiguousarray(types, np.int32)
        q = np.ascontiguousarray(charges, np.float32)
        s = np.ascontiguousarray(radii, np.float32)
        cid = "".join(chain_ids) if chain_ids is not None else "A" * n
        rseq = np.ascontiguousarray(res_seq if res_seq is not None else np.arange(1, n + 1), np.int32)
        cidx = np.ascontiguousarray(chain_index if chain_index is not None else np.zeros(n), np.int32)
        seglen = np.ascontiguousarray([len(x) for x in segments] or [0], np.int32)
        segres = np.ascontiguousarray([v for x in segments for v in x] or [0], np.int32)
        c = np.ascontiguousarray(center, np.float32) if center is not None else None
        return _ok(_L().cgppd_engine_add_molecule(
            self.h, sim, n, _p(xyz, c_float), _p(types, c_int), _p(q, c_float), _p(s, c_float), cid.encode(),
            _p(rseq, c_int), _p(cidx, c_int), int(num_chains), int(bool(all_flexible)), int(bool(crowder)),
            len(segments), _p(seglen, c_int), _p(segres, c_int), _p(c, c_float) if c is not None else None),
            "add_molecule")

    def finalize(self, cluster=0, threads=0, resident=True):
        _ok(_L().cgppd_engine_set_resident(self.h, int(bool(resident))), "set_resident")
        _ok(_L().cgppd_engine_finalize(self.h, int(cluster), int(threads)), "finalize")

    def run(self, n_blocks, steps_per_block, exchange_after_last=True, stream=None):
        _ok(_L().cgppd_engine_run(self.h, int(n_blocks), int(steps_per_block), int(bool(exchange_after_last)),
                                  c_void_p(stream) if stream else None), "run")

    def final_report(self, row, stream=None):
        _ok(_L().cgppd_engine_final_report(self.h, int(row), c_void_p(stream) if stream else None), "final_report")

    def synchronize(self):
        _ok(_L().cgppd_engine_synchronize(self.h), "synchronize")

    @property
    def total_replicas(self):
        return _L().cgppd_engine_total_replicas(self.h)

    def sim_info(self, sim):
        n, m, r = c_int(), c_int(), c_int()
        _ok(_L().cgppd_engine_sim_info(self.h, sim, ctypes.byref(n), ctypes.byref(m), ctypes.byref(r)), "sim_info")
        return n.value, m.value, r.value

    def recompute(self, write_state=False):
        out = np.zeros(self.total_replicas, np.float64)
        _ok(_L().cgppd_engine_recompute(self.h, _p(out, c_double), int(bool(write_state))), "recompute")
        return out

    def replicas(self, sim):
        _, _, R = self.sim_info(sim)
        pot = np.zeros(R, np.float64)
        T = np.zeros(R, np.float32)
        lab = np.zeros(R, np.int32)
        ti = np.zeros(R, np.int32)
        st = np.zeros((R, 16), np.int32)
        _ok(_L().cgppd_engine_get_replicas(self.h, sim, _p(pot, c_double), _p(T, c_float), _p(lab, c_int),
                                           _p(ti, c_int), _p(st, c_int)), "get_replicas")
        fl = st[:, 9:13].copy().view(np.float32)
        return {"potential": pot, "temperature": T, "label": lab, "tindex": ti, "accept": st[:, 0],
                "acceptA": st[:, 1], "reject": st[:, 2], "totalAcceptReject": st[:, 3], "totalAccept": st[:, 4],
                "boundSamples": st[:, 5], "samplesSinceLastExchange": st[:, 6], "totalBoundSamples": st[:, 7],
                "totalSamples": st[:, 8], "acceptanceRatio": fl[:, 0], "accumulativeAcceptanceRatio": fl[:, 1],
                "fractionBound": fl[:, 2], "accumulativeFractionBound": fl[:, 3]}

    def state(self, sim, replica):
        N, M, _ = self.sim_info(sim)
        xyz = np.zeros((N, 3), np.float32)
        rel = np.zeros((N, 3), np.float32)
        cen = np.zeros((M, 3), np.float32)
        _ok(_L().cgppd_engine_get_state(self.h, sim, replica, _p(xyz, c_float), _p(rel, c_float), _p(cen, c_float)),
            "get_state")
        return xyz, rel, cen

    def set_state(self, sim, replica, xyz, rel, centers):
        xyz = np.ascontiguousarray(xyz, np.float32)
        rel = np.ascontiguousarray(rel, np.float32)
        cen = np.ascontiguousarray(centers, np.float32)
        _ok(_L().cgppd_engine_set_state(self.h, sim, replica, _p(xyz, c_float), _p(rel, c_float), _p(cen, c_float)),
            "set_state")

    def upload(self, sim, pos4_ptr, rel4_ptr, centers4_ptr, recompute=True, stream=None):
        """Enqueue host->device copies of every replica's state (raw host pointers)."""
        _ok(_L().cgppd_engine_upload(self.h, sim, c_void_p(pos4_ptr), c_void_p(rel4_ptr), c_void_p(centers4_ptr),
                                     int(bool(recompute)), c_void_p(stream) if stream else None), "upload")

    def download(self, sim, pos4_ptr, rel4_ptr, centers4_ptr, pot_ptr, stream=None):
        """Enqueue device->host copies of every replica's state and potentials."""
        _ok(_L().cgppd_engine_download(self.h, sim, c_void_p(pos4_ptr), c_void_p(rel4_ptr), c_void_p(centers4_ptr),
                                       c_void_p(pot_ptr), c_void_p(stream) if stream else None), "download")

    def matrix(self, sim, replica):
        _, M, _ = self.sim_info(sim)
        E = np.zeros((M, M), np.float64)
        intra = np.zeros(M, np.float64)
        _ok(_L().cgppd_engine_get_matrix(self.h, sim, replica, _p(E, c_double), _p(intra, c_double)), "get_matrix")
        return E, intra

    def report(self, sim, row):
        _, _, R = self.sim_info(sim)
        out = np.zeros((R, 4), np.float32)
        ex = np.zeros(2, np.int32)
        _ok(_L().cgppd_engine_get_report(self.h, sim, row, _p(out, c_float), _p(ex, c_int)), "get_report")
        return out, ex

    def counters(self):
        a, b = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        _ok(_L().cgppd_engine_counters(self.h, ctypes.byref(a), ctypes.byref(b)), "counters")
        return a.value, b.value

    def error_bits(self):
        return _L().cgppd_engine_error_bits(self.h)

    def replica_error_bits(self, sim):
        """Status bits per replica slot (1 null move, 2 non-finite energy change, 4
        non-finite potential in an exchange test)."""
        _, _, R = self.sim_info(sim)
        out = np.zeros(R, np.uint32)
        _ok(_L().cgppd_engine_replica_error_bits(self.h, sim, _p(out, ctypes.c_uint)), "replica_error_bits")
        return out

    def last_launches(self):
        return _L().cgppd_engine_last_launches(self.h)

    def set_sample_log(self, per_replica):
        """Keep up to `per_replica` fraction-bound samples per replica on the device."""
        self._sample_cap = int(per_replica)
        _ok(_L().cgppd_engine_set_sample_log(self.h, int(per_replica)), "set_sample_log")

    def take_samples(self, sim):
        """The samples recorded since the last call, per replica slot: a list of record
        arrays (step, non-crowder energy, potential, temperature), emptying the log."""
        _, _, R = self.sim_info(sim)
        cap = max(1, getattr(self, "_sample_cap", 0))
        counts = np.zeros(R, np.int32)
        enc = np.zeros(R * cap, np.float64)
        pot = np.zeros(R * cap, np.float64)
        temp = np.zeros(R * cap, np.float32)
        step = np.zeros(R * cap, np.int32)
        _ok(_L().cgppd_engine_take_samples(self.h, sim, _p(counts, c_int), _p(enc, ctypes.c_double),
                                           _p(pot, ctypes.c_double), _p(temp, c_float), _p(step, c_int)),
            "take_samples")
        xyz = None
        if getattr(self, "_sample_nres", 0) > 0 and getattr(self, "_sample_cap", 0) > 0:
            xyz = np.zeros((R, cap, self._sample_nres, 3), np.float32)
            _ok(_L().cgppd_engine_take_sample_xyz(self.h, sim, _p(xyz, c_float)), "take_sample_xyz")
        out = []
        for r in range(R):
            sl = slice(r * cap, r * cap + counts[r])
            rec = {"step": step[sl].copy(), "enc": enc[sl].copy(), "potential": pot[sl].copy(),
                   "temperature": temp[sl].copy()}
            if xyz is not None:
                rec["xyz"] = xyz[r, :counts[r]].copy()
            out.append(rec)
        return out

    def set_sample_snapshots(self, residues):
        """Keep the coordinates of the first `residues` residues with every recorded sample
        (returned by take_samples as "xyz")."""
        self._sample_nres = int(residues)
        _ok(_L().cgppd_engine_set_sample_snapshots(self.h, int(residues)), "set_sample_snapshots")

    def checkpoint(self, path):
        _ok(_L().cgppd_engine_checkpoint(self.h, str(path).encode()), "checkpoint")

    def restore(self, path):
        _ok(_L().cgppd_engine_restore(self.h, str(path).encode()), "restore")

    def launch_shape(self):
        """(CTAs per replica, threads per CTA, state resident in shared memory)."""
        c, t = c_int(), c_int()
        res = _L().cgppd_engine_launch_shape(self.h, ctypes.byref(c), ctypes.byref(t))
        return c.value, t.value, bool(res)


def from_workload(wl, cluster=0, threads=0, seed=None, sample_frequency=0, sample_after=0, finalize=True,
                  resident=True):
    """Engine holding every simulation of a workloads.Workload."""
    e = Engine(wl.lj_raw, wl.torsion_V, wl.torsion_phase, seed=wl.seed if seed is None else seed)
    for sim in wl.sims:
        s = e.add_simulation(sim.temperatures, sim.translate_steps, sim.rotate_steps, sim.box, sim.move_weights,
                             sim.rigid_rotate_prob, sample_frequency, sample_after,
                             repulsive_crowding=getattr(sim, "repulsive_crowding", False))
        for m in sim.molecules:
            e.add_molecule(s, m.xyz, m.types, m.charges, m.radii, chain_ids=m.chain_ids, res_seq=m.res_seq,
                           chain_index=m.chain_index, all_flexible=m.all_flexible, crowder=m.crowder,
                           segments=m.segments)
    if finalize:
        e.finalize(cluster, threads, resident)
    return e


def _tuning(self):
    """Autotuner measurements: list of (CTAs per replica, threads per CTA, us per MC step)."""
    L = _L()
    if not hasattr(L, "_tuning_declared"):
        L.cgppd_engine_tuning.restype = c_int
        L.cgppd_engine_tuning.argtypes = [c_void_p, P(c_int), P(c_int), P(c_int), P(c_float)]
        L._tuning_declared = True
    cap = 64
    n = c_int(cap)
    cl = (c_int * cap)()
    th = (c_int * cap)()
    us = (c_float * cap)()
    L.cgppd_engine_tuning(self.h, ctypes.byref(n), cl, th, us)
    return [(cl[i], th[i], us[i]) for i in range(min(n.value, cap))]


Engine.tuning = _tuning
