#!/usr/bin/env python3
"""Record the reference's own energies for the synthetic configurations.

Runs the reference's energy code (oracle/_ref/libcgppd_ref.so, built from the
reference tree by oracle/build_ref.py; available only where the tree is mounted) on
the seeded initial structures of configurations c0, c1, c2 and c4, and on a few
rigid-body perturbations of each, and writes tests/golden/ref_energies.json.  The
structures themselves go to tests/golden/ref_structures.npz: the seeded generator is
not bit-reproducible across CPU architectures and numpy builds, so the tests read the
exact inputs the energies were computed from.  The GPU tests compare the engine
against these numbers on a machine without the tree.

Usage: python tests/golden/make_ref_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import ref  # noqa: E402
from cgppd_gb300 import workloads  # noqa: E402
from helpers import STRUCTURES, fixture_workload, save_structures  # noqa: E402


def total_kcal(raw5, flexible):
    return oracle.total(np.asarray(raw5, np.float64), flexible)


def perturbed(sim, transforms):
    """Molecules of `sim` moved rigidly by transforms[m] = (axis, angle, shift) about
    their float64 centres (None = unmoved)."""
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


def main():
    assert ref.available(), "the reference tree is needed to build oracle/_ref"
    out = {"source": "reference energy code (src/Potential.cpp, Residue.cpp, Geometry.cpp, ...) via "
                     "oracle/ref_harness.cpp", "configs": {}}
    cfgs = ("c0", "c1", "c2", "c4")
    save_structures(STRUCTURES, {cfg: workloads.make(cfg) for cfg in cfgs})
    print("wrote", STRUCTURES, os.path.getsize(STRUCTURES), "bytes")
    for cfg in cfgs:
        wl = fixture_workload(cfg)
        sim = wl.sims[0]
        rng = np.random.default_rng(99)
        states = []
        for k in range(4):
            transforms = []
            for _m in sim.molecules:
                if k == 0:
                    transforms.append(None)
                    continue
                ax = rng.normal(size=3)
                ax /= np.linalg.norm(ax)
                transforms.append((ax.tolist(), float(rng.uniform(-0.3, 0.3)), rng.normal(scale=1.5, size=3).tolist()))
            mols = perturbed(sim, transforms)
            raw, inter = ref.energy(mols, wl.lj_raw, sim.box, wl.torsion_V, wl.torsion_phase)
            flexible = any(m.all_flexible or m.segments for m in mols)
            states.append({"transforms": transforms, "raw": raw.tolist(), "inter": inter.tolist(),
                           "total_kcal": total_kcal(raw, flexible)})
        out["configs"][cfg] = states
    path = os.path.join(HERE, "ref_energies.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
