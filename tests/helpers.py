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
