"""Shared test helpers: parameter files in the reference's formats, device buffers."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LJ_LABELS = ["Cys", "Met", "Phe", "Ile", "Leu", "Val", "Trp", "Tyr", "Ala", "Gly", "Thr", "Ser", "Asn", "Gln",
             "Asp", "Glu", "His", "Arg", "Lys", "Pro"]


def write_amino_acid_file(path, recs):
    """Residue-type records in the reference's five-line format (data/AminoAcids)."""
    with open(path, "w") as f:
        for r in recs:
            f.write("#Amino acid class initialisation data\n#name\n")
            f.write("%s\n%s\n%s\n%s\n%s\n\n" % (r["name"], r["sname"], r["symbol"], repr(r["radius"]),
                                                repr(r["charge"])))


def write_lj_file(path, recs, table):
    """Upper-triangular contact table with labels (data/pair_potentials_MJ1996 format)."""
    idx = {r["sname"]: i for i, r in enumerate(recs)}
    order = [idx[l] for l in LJ_LABELS]
    with open(path, "w") as f:
        f.write("# contact table\n")
        f.write("     " + " ".join(LJ_LABELS) + "\n")
        for k, a in enumerate(order):
            vals = " ".join("%.6f" % table[a][order[j]] for j in range(k, 20))
            f.write("%s %s\n" % (LJ_LABELS[k], vals))


def write_torsion_file(path, recs, V, S):
    """Torsion table in the reference's `NAME NAME V N SIGMA(deg)` format."""
    with open(path, "w") as f:
        f.write("# NAME NAME V N SIGMA\n")
        for i in range(20):
            for j in range(20):
                for n in range(4):
                    if V[i][j][n] != 0.0 or S[i][j][n] != 0.0:
                        f.write("%s %s %12.6f %d %12.6f\n" % (recs[i]["sname"].upper(), recs[j]["sname"].upper(),
                                                               V[i][j][n], n + 1, S[i][j][n] * 57.29577951308232))


def write_pdb(path, residues):
    """C-alpha records in fixed PDB columns (what Molecule::initFromPDB reads)."""
    with open(path, "w") as f:
        chain = None
        for k, r in enumerate(residues):
            if chain is not None and r["chain_index"] != chain:
                f.write("TER\n")
            chain = r["chain_index"]
            x, y, z = r["xyz"]
            f.write("ATOM  %5d  CA  %3s %c%4d    %8.3f%8.3f%8.3f  1.00  0.00\n" % (k + 1, r["res"], r["chain"],
                                                                                r["seq"], x, y, z))
        f.write("TER\nEND\n")


def write_reference_data_dir(root, refdata):
    """data/AminoAcids, data/pair_potentials_MJ1996, data/torsional_pair_potentials and
    data/application/{ubq,uim}.pdb under `root`, from the fixtures."""
    d = os.path.join(root, "data")
    os.makedirs(os.path.join(d, "application"), exist_ok=True)
    write_amino_acid_file(os.path.join(d, "AminoAcids"), refdata["amino_acids"])
    write_lj_file(os.path.join(d, "pair_potentials_MJ1996"), refdata["amino_acids"], refdata["lj_table"])
    write_torsion_file(os.path.join(d, "torsional_pair_potentials"), refdata["amino_acids"], refdata["torsion_V"],
                       refdata["torsion_sigma"])
    for name in ("ubq", "uim"):
        write_pdb(os.path.join(d, "application", name + ".pdb"), refdata["pdbs"]["application/" + name]["residues"])


STRUCTURES = os.path.join(ROOT, "tests", "golden", "ref_structures.npz")


def save_structures(path, workloads_by_config):
    """Write the first simulation of each seeded workload (molecules, box, contact and
    torsion tables) to one .npz, so that fixtures computed from them do not depend on
    regenerating the structures bit for bit on another machine."""
    arrays = {}
    for cfg, wl in workloads_by_config.items():
        sim = wl.sims[0]
        arrays[cfg + "/box"] = np.float64(sim.box)
        arrays[cfg + "/lj_raw"] = wl.lj_raw
        if wl.torsion_V is not None:
            arrays[cfg + "/torsion_V"] = np.asarray(wl.torsion_V, np.float64)
            arrays[cfg + "/torsion_phase"] = np.asarray(wl.torsion_phase, np.float64)
        arrays[cfg + "/n_mol"] = np.int32(len(sim.molecules))
        for k, m in enumerate(sim.molecules):
            p = "%s/m%d/" % (cfg, k)
            arrays[p + "xyz"] = m.xyz
            arrays[p + "types"] = m.types.astype(np.uint8)
            arrays[p + "charges"] = m.charges.astype(np.int8)
            arrays[p + "radii"] = m.radii
            arrays[p + "flags"] = np.array([m.all_flexible, m.crowder], np.uint8)
            arrays[p + "segments"] = np.array([len(m.segments)] + [len(s) for s in m.segments] +
                                              [v for s in m.segments for v in s], np.int32)
    np.savez_compressed(path, **arrays)


def fixture_workload(cfg, path=STRUCTURES):
    """The workload of `cfg` as saved by save_structures (one simulation, one replica)."""
    from cgppd_gb300 import workloads
    z = np.load(path)
    mols = []
    for k in range(int(z[cfg + "/n_mol"])):
        p = "%s/m%d/" % (cfg, k)
        seg = z[p + "segments"].tolist()       # [count, lengths..., residues...]
        segments, i = [], 1 + seg[0]
        for n in seg[1:1 + seg[0]]:
            segments.append(seg[i:i + n])
            i += n
        fl = z[p + "flags"]
        mols.append(workloads.Molecule(z[p + "xyz"], z[p + "types"].astype(np.int32),
                                       z[p + "charges"].astype(np.float32), z[p + "radii"], segments,
                                       bool(fl[0]), bool(fl[1])))
    V = z[cfg + "/torsion_V"] if cfg + "/torsion_V" in z else None
    S = z[cfg + "/torsion_phase"] if cfg + "/torsion_phase" in z else None
    sim = workloads.Simulation(mols, float(z[cfg + "/box"]), [300.0], [2.0], [0.2])
    return workloads.Workload(cfg, [sim], z[cfg + "/lj_raw"], V, S)


def header_functions():
    """Function names declared in include/*.h."""
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(inc, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{}]*\)\s*;", src):
            name = m.group(1)
            if name in ("if", "while", "for", "return", "sizeof", "defined"):
                continue
            names.append(name)
    return sorted(set(names))


def device_array(arr):
    """A torch CUDA tensor holding `arr` (plumbing only)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


REF_MC = os.path.join(ROOT, "tests", "golden", "ref_mc_trajectories.json")


def ref_mc_config(name):
    """One configuration of the reference trajectory fixtures (make_ref_mc_golden.py):
    (config dict, molecules, centres [M,3], relative positions [N,3], per-replica
    temperatures, translate steps, rotate steps)."""
    import json
    from oracle import ref_mc
    with open(REF_MC) as f:
        d = json.load(f)
    cfg = d["configs"][name]
    cfg["seed"], cfg["block"] = d["seed"], d["block"]
    mols, cen, rel = ref_mc.system(cfg)
    ini = ref_mc.replicas(cfg, "initial")
    return cfg, mols, cen, rel, ini["temperature"], ini["translate_step"].astype(np.float32), \
        ini["rotate_step"].astype(np.float64)
