"""Driver of oracle/_ref/cgppd_ref_mc: the reference's own Simulation run with the GB300
engine's Philox draws (oracle/ref_rng.cpp), and the same system in the oracle.

TEST INFRASTRUCTURE ONLY.  The binary exists only where the reference tree is mounted
(oracle/build_ref.py builds it); callers skip when `available()` is False.
"""
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "cgppd_ref_mc")


def available():
    if not os.path.exists(BIN):
        try:
            from .build_ref import build_mc
            build_mc()
        except Exception:
            return False
    return os.path.exists(BIN)


def run(workdir, argfile_name, seed, extra=(), timeout=600):
    """Run the reference's Simulation::init + run on `argfile_name` in `workdir` (which
    holds the reference's data/ files and the argfile's PDBs): the initial system and
    the final state as a dict (see oracle/ref_mc_harness.cpp)."""
    out = os.path.join(workdir, "ref_mc_%d.json" % seed)
    r = subprocess.run([BIN, str(seed), out, "-f", argfile_name] + list(extra), cwd=workdir,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("reference MC harness failed (%d):\n%s" % (r.returncode, r.stdout[-3000:]))
    with open(out) as f:
        return json.load(f)


def system(d):
    """The run's molecules (workloads.Molecule) with the reference's initial coordinates,
    and their centres and relative positions, from a harness result."""
    from cgppd_gb300 import workloads
    mols, centers, rel = [], [], []
    for m in d["molecules"]:
        res = np.array(m["residues"], np.float64)
        xyz = res[:, 0:3].astype(np.float32)
        aa = res[:, 6].astype(np.int32)
        q = res[:, 7].astype(np.float32)
        r = res[:, 8].astype(np.float32)
        seq = res[:, 9].astype(np.int32)
        chains = [chr(int(c)) for c in res[:, 10]]
        segs = [] if m["all_flexible"] else m["segments"]
        mol = workloads.Molecule(xyz, aa, q, r, segments=segs, all_flexible=bool(m["all_flexible"]),
                                 crowder=bool(m["crowder"]), chain_ids=chains, res_seq=seq)
        mols.append(mol)
        centers.append(m["center"])
        rel.append(res[:, 3:6])
    return mols, np.array(centers, np.float32), np.concatenate(rel).astype(np.float32)


def replicas(d, which):
    """Per-slot arrays of the 'initial' or 'final' state."""
    reps = d[which]["replicas"]
    out = {k: np.array([r[k] for r in reps]) for k in reps[0] if k not in ("xyz", "centers")}
    out["xyz"] = np.array([r["xyz"] for r in reps], np.float32).reshape(len(reps), -1, 3)
    out["centers"] = np.array([r["centers"] for r in reps], np.float32).reshape(len(reps), -1, 3)
    out["potential"] = out["potential"].astype(np.float64)
    out["temperature"] = out["temperature"].astype(np.float32)
    return out
