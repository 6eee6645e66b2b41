#!/usr/bin/env python3
"""Generate the golden fixtures used by the test-suite from the CGPPD reference tree.

This script is test infrastructure. It is run in the build container, where the
reference tree is mounted, and writes ``tests/golden/reference_data.json``; the
GPU machine never sees the reference tree and reads only that JSON file.

What it extracts, with the reference behaviour each parser restates:

* the 20 amino-acid records (name, short name, symbol, vdW radius, charge) in file
  order, which is the residue-type index order (``src/AminoAcids.cpp:29-73``);
* the symmetric 20x20 contact table from the upper-triangular text file, with the
  column labels mapped through ``getAminoAcidIndex`` (``src/AminoAcids.cpp:75-138``,
  ``:145-181``);
* the torsion table ``V[20][20][4]`` and ``Sigma[20][20][4]`` with the phase
  converted from degrees to radians (``src/TorsionalLookupMatrix.cpp:21-51``);
* the C-alpha records of the PDB files the reference tests load: only ``ATOM``
  lines whose atom name is ``CA``; ``TER`` counts chains; ``END`` (prefix match)
  stops reading; a file without ``TER`` gets one chain (``src/Molecule.cpp:506-612``);
* the known-answer values the reference tests assert, with their file:line.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_amino_acids(path):
    """Five non-comment lines per record: name, short name, symbol, radius, charge."""
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    recs = []
    k = 0
    while k < len(lines):
        ln = lines[k]
        if ln == "" or ln.startswith("#"):
            k += 1
            continue
        name = ln[:19]
        sname = lines[k + 1][:3]
        symbol = lines[k + 2][:1]
        radius = float(lines[k + 3].strip() or 0)
        charge = float(lines[k + 4].split()[0])
        recs.append({"name": name, "sname": sname, "symbol": symbol,
                     "radius": radius, "charge": charge})
        k += 5
    assert len(recs) == 20, len(recs)
    return recs


def aa_index(recs, name):
    """Restates AminoAcids::getAminoAcidIndex (src/AminoAcids.cpp:145-181).

    Three-letter names match the short name case-insensitively (first letter upper,
    rest lower), one-letter names match the symbol, anything else matches the full
    name; the search runs from index 19 down and returns -1 when nothing matches."""
    if len(name) < 1:
        return -1
    if len(name) == 3:
        key = name[0].upper() + name[1].lower() + name[2].lower()
        for i in range(19, -1, -1):
            if recs[i]["sname"] == key:
                return i
    elif len(name) == 1:
        key = name[0].upper()
        for i in range(19, -1, -1):
            if recs[i]["symbol"] == key:
                return i
    else:
        key = name[0].upper() + name[1:]
        for i in range(19, -1, -1):
            if recs[i]["name"] == key:
                return i
    return -1


def parse_lj_table(path, recs):
    table = [[0.0] * 20 for _ in range(20)]
    labels = None
    start = 0
    with open(path) as f:
        for ln in f:
            ln = ln.rstrip("\n")
            if ln == "" or ln.startswith("#"):
                continue
            toks = ln.split()
            if labels is None:
                labels = [aa_index(recs, t) for t in toks]
                continue
            vals = toks[1:]
            for n, j in enumerate(range(start, 20)):
                e = float(vals[n])
                table[labels[start]][labels[j]] = e
                table[labels[j]][labels[start]] = e
            start += 1
    return table


def parse_torsions(path, recs):
    V = [[[0.0] * 4 for _ in range(20)] for _ in range(20)]
    S = [[[0.0] * 4 for _ in range(20)] for _ in range(20)]
    with open(path) as f:
        for ln in f:
            ln = ln.rstrip("\n")
            if ln == "" or ln.startswith("#"):
                continue
            a0, a1, v, n, sig = ln.split()[:5]
            i0, i1, n = aa_index(recs, a0[:3]), aa_index(recs, a1[:3]), int(n)
            V[i0][i1][n - 1] = float(v)
            S[i0][i1][n - 1] = float(sig) / 57.29577951308232
    return V, S


def parse_pdb(path, recs):
    """C-alpha records: resName, chainId, resSeq, x, y, z, chain index (TER count)."""
    residues = []
    chains = 0
    with open(path, errors="replace") as f:
        for ln in f:
            ln = ln.rstrip("\n")
            if ln.startswith("ATOM"):
                name = ln[12:].split()[0] if len(ln) > 12 and ln[12:].split() else ""
                if name != "CA":
                    continue
                res_name = ln[17:].split()[0]
                chain_id = ln[21] if len(ln) > 21 else " "
                m = re.match(r"\s*([-+]?\d+)", ln[22:])
                res_seq = int(m.group(1)) if m else 0

                def num(s):
                    m = re.match(r"\s*([-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?)", s)
                    return float(m.group(1)) if m else 0.0
                x, y, z = num(ln[30:]), num(ln[38:]), num(ln[46:])
                residues.append({"res": res_name, "aa": aa_index(recs, res_name),
                                 "chain": chain_id, "seq": res_seq,
                                 "xyz": [x, y, z], "chain_index": chains})
            elif ln.startswith("TER"):
                chains += 1
            elif ln.startswith("END"):
                break
    if residues and chains == 0:
        chains = 1
    return {"residues": residues, "chains": chains}


# Known answers asserted by the reference tests.
KATS = {
    # tests/testReferenceConformations.cpp:83-94 -- Potential(LJ kcal/mol, DH kcal/mol)
    # of the 10 two-molecule conformations in a 1000 A box, CPU E() and GPU totals.
    "reference_conformations_exact": [
        [-0.0796731, -0.212202], [-1.30422, 0.264889], [-8.97201, -1.17831],
        [-5.81976, -1.67169], [-2.08631e-05, -5.76825e-05], [-4.74252, -0.749355],
        [-4.11734, -1.26302], [-9.08724, -1.44068], [-7.83475, -1.94273],
        [-7.34204, -1.06544]],
    # tests/testReferenceConformations.cpp:119-130 -- published energies (LJ, DH)
    "reference_conformations_published": [
        [-0.08092694, -0.21315828], [-1.32250603, 0.26608889], [-9.09456258, -1.18374210],
        [-5.90453581, -1.67963588], [-0.00002116, -0.00005795], [-4.81153585, -0.75302819],
        [-4.18365757, -1.26891119], [-9.22300158, -1.44730149], [-7.95237776, -1.95173336],
        [-7.44768961, -1.07043531]],
    # tests/testReferenceConformations.cpp:183-189 -- relative error statistics
    "published_error_stats": {"mean_LJ": 0.001505, "mean_DH": 0.000078, "mean_total": 0.001073,
                              "max_LJ": 0.002866, "max_DH": 0.000250, "max_total": 0.002202},
    # tests/testReplica.cpp:61-82 -- conf1 in a 118.4 A box with residues 73-76 of 1b flexible:
    # (LJ, DH, bond, angle, torsion) kcal/mol, flexible and rigid-only
    "replica_flexible": [-0.068205, -0.240383, 0.180426, 1.555213, 5.420859],
    "replica_rigid": [-0.079673, -0.212202, 0.0, 0.0, 0.0],
    # tests/testReplica.cpp:115-176 -- UIDs and packed floats
    "replica_uids": {"m1_pos_w": 1.0, "m1_meta_w": 0.25, "m2_domain_pos_w": 2.0,
                     "m2_meta_w": 1.5, "m2_linker_pos_w": 0.0},
    # tests/testMolecule.cpp:289-307 -- intra-molecular components (LJ, DH, bond, angle,
    # torsion) of all-flexible ala8 (box 15 A) and angiotensin (box 1000 A)
    "molecule_ala8": [0.932791, 0.000000, 0.045626, 1.272977, 10.872785],
    "molecule_angiotensin": [-0.250504, 0.052706, 0.642775, 4.887787, 15.871157],
    # tests/testMolecule.cpp:311-323 -- bond/angle/torsion counts
    "molecule_counts": {"ubiquitin_seg_72_75": [3, 3, 3], "ala8_all": [7, 6, 5],
                        "angiotensin_all": [9, 8, 7]},
    # tests/testMolecule.cpp:45-60 -- relative start positions of ala8 (centred on 0)
    "ala8_start": [[-9.29663, -6.96, -0.91625], [-7.38663, -3.879, 0.23775],
                   [-3.76163, -3.302, -0.76025], [-1.79963, -0.311, 0.53375],
                   [1.76937, 0.361, -0.59825], [3.79137, 3.252, 0.82475],
                   [7.29737, 4.029, -0.43125], [9.38637, 6.81, 1.10975]],
    # tests/testGeometry.cpp:9-96 -- synthetic 2x76 diubiquitin graph with segments
    # {72,73,74,75,123} and {148,149,150,151}
    "geometry": {
        "bonds": [[72, 73], [73, 74], [74, 75], [75, 123], [148, 149], [149, 150], [150, 151]],
        "angles": [[71, 72, 73], [72, 73, 74], [73, 74, 75], [74, 75, 123], [75, 123, 122],
                   [75, 123, 124], [147, 148, 149], [148, 149, 150], [149, 150, 151]],
        "torsions": [[70, 71, 72, 73], [71, 72, 73, 74], [72, 73, 74, 75], [73, 74, 75, 123],
                     [74, 75, 123, 122], [74, 75, 123, 124], [75, 123, 124, 125],
                     [121, 122, 123, 75], [146, 147, 148, 149], [147, 148, 149, 150],
                     [148, 149, 150, 151]],
        "crankshaft": [73, 74, 75, 149, 150],
        "local": [73, 74, 75, 149, 150, 151],
        "flex": [72, 73, 74, 75, 123, 148, 149, 150, 151],
        "branch": {"123,122": [76, 123], "75,123": [75, 151], "148,149": [148, 151]},
        "segment_bonds": [[75, 123]],
        "indirect_neighbours": [[73, 123], [74, 123], [74, 122], [74, 124], [75, 122],
                                [75, 121], [75, 124], [75, 125]],
        "rigid_domains": [[0, 72], [76, 148]],
    },
}


def remc_outputs(ref, arch):
    """Statistics of the reference's seeded REMC regression output
    (tests/remctest_<arch>.tgz, checked by tests/testSimulation.cpp:97-150)."""
    import tarfile
    out = {}
    with tarfile.open(os.path.join(ref, "tests", "remctest_%s.tgz" % arch)) as tf:
        def text(name):
            return tf.extractfile("remctest_%s/%s" % (arch, name)).read().decode()
        acc = text("acceptance_ratios").splitlines()
        out["acceptance_header"] = acc[:2]
        rows = [ln for ln in acc[2:] if ":" in ln]
        vals = [[float(x) for x in ln.split(":", 1)[1].replace("|", " ").split()] for ln in rows]
        out["acceptance_rows"] = len(rows)
        out["acceptance_final_cumulative"] = vals[-1][1::2]
        out["acceptance_mean_instantaneous"] = [sum(v[2 * t] for v in vals) / len(vals) for t in range(5)]
        ex = [ln.split() for ln in text("exchange_freq").splitlines()[1:]]
        out["exchange_rows"] = len(ex)
        out["exchange_final_cumulative"] = float(ex[-1][1])
        fb = text("fractionBound").splitlines()
        out["fraction_header"] = fb[:3]
        frows = [ln for ln in fb[3:] if ":" in ln]
        fvals = [[float(x) for x in ln.split(":", 1)[1].replace("|", " ").split()] for ln in frows]
        out["fraction_final_cumulative"] = fvals[-1][1::2]
        out["fileindex"] = text("fileindex").splitlines()
        bc = text("boundconformations").splitlines()
        out["boundconformations_header"] = bc[:2]
        # per-temperature mean of the sampled replica potentials ("step; E_nc (E); T")
        per_t = {}
        for ln in bc[2:]:
            if ";" not in ln:
                continue
            f = ln.split(";")
            e = float(f[1].split("(")[1].split(")")[0])
            per_t.setdefault(f[2].strip(), []).append(e)
        out["sampled_energy_mean_by_temperature"] = {t: sum(v) / len(v) for t, v in per_t.items()}
        out["sampled_energy_count_by_temperature"] = {t: len(v) for t, v in per_t.items()}
        # the sample PDB files (src/Replica.cpp:1082-1087, 1124-1168): how many, and the
        # layout of the first sample's file with its coordinates and values masked
        out["pdb_sample_count"] = sum(1 for n in tf.getnames()
                                      if n.startswith("remctest_%s/pdb/sample_" % arch))
        out["pdb_sample_layout"] = [mask_pdb_line(ln) for ln in
                                    text("pdb/" + os.path.basename(bc[3])).splitlines()]
    return out


def mask_pdb_line(ln):
    """A sample PDB line without what differs between runs: the coordinates of ATOM
    records and the values of the REMARK records."""
    if ln.startswith("ATOM"):
        return ln[:30] + "*" + ln[54:]
    if ln.startswith("REMARK") and ":" in ln and not ln.startswith("REMARK simulation"):
        return ln.split(":")[0] + ":*"
    return ln


def main():
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from oracle.build_ref import reference_root
    ref = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if ref is None:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set CGPPD_REFERENCE_DIR)")
    recs = parse_amino_acids(os.path.join(ref, "data/AminoAcids"))
    lj = parse_lj_table(os.path.join(ref, "data/pair_potentials_MJ1996"), recs)
    V, S = parse_torsions(os.path.join(ref, "data/torsional_pair_potentials"), recs)
    pdbs = {}
    for i in range(1, 11):
        for part in ("1a", "1b"):
            pdbs["conf%d/%s" % (i, part)] = parse_pdb(os.path.join(ref, "data/conf%d/%s.pdb" % (i, part)), recs)
    for name in ("1UBQ", "ala8", "angiotensin"):
        pdbs["tests/" + name] = parse_pdb(os.path.join(ref, "tests/%s.pdb" % name), recs)
    for name in ("ubq", "uim"):
        pdbs["application/" + name] = parse_pdb(os.path.join(ref, "data/application/%s.pdb" % name), recs)
    with open(os.path.join(ref, "data", "torsional_pair_potentials")) as f:
        torsion_text = f.read()
    with open(os.path.join(ref, "tests", "argtestfile")) as f:
        argtestfile = f.read()
    with open(os.path.join(ref, "tests", "remctestfile")) as f:
        remctestfile = f.read()
    out = {"amino_acids": recs, "lj_table": lj, "torsion_V": V, "torsion_sigma": S,
           "pdbs": pdbs, "kats": KATS,
           # the reference's own test inputs (tests/argtestfile, tests/remctestfile) and the
           # statistics of its seeded REMC outputs, CPU and GPU builds
           "argtestfile": argtestfile, "remctestfile": remctestfile,
           "remctest": {"CPU": remc_outputs(ref, "CPU"), "GPU": remc_outputs(ref, "GPU")},
           "torsion_file_lines": len(torsion_text.splitlines()),
           "source": "CGPPD reference data/ and tests/ (see make_golden.py)"}
    path = os.path.join(HERE, "reference_data.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
