"""Build oracle/_ref/libcgppd_ref.so from the reference's own energy sources.

TEST INFRASTRUCTURE ONLY.  Compiles, in place from the reference tree (read-only),
the translation units of the energy layer that need no external library --
src/{Potential,Residue,AminoAcids,AminoAcid,Geometry,Quaternion,vector3f,
TorsionalLookupMatrix}.cpp -- with the reference's own flags for the flexible-linker
CPU build (-O2 -std=c++11 -DEnableFlexibleLinkers, Makefile:5 and :60-62), plus
oracle/ref_harness.cpp.  Output goes only to oracle/_ref/ (git-ignored).  The MC layer
(Molecule, Replica, Simulation) needs GSL and logog, which are not installed here, so
it is not built.

Usage: python oracle/build_ref.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $CGPPD_REFERENCE_DIR, else a directory named `reference`
beside the repository checkout; without either nothing is built.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "libcgppd_ref.so")
UNITS = ["Potential", "Residue", "AminoAcids", "AminoAcid", "Geometry", "Quaternion", "vector3f",
         "TorsionalLookupMatrix"]


def reference_root():
    """The reference tree: $CGPPD_REFERENCE_DIR, else `reference` beside the repository
    checkout, else None."""
    env = os.environ.get("CGPPD_REFERENCE_DIR")
    if env:
        return env if os.path.isdir(env) else None
    sib = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return sib if os.path.isdir(os.path.join(sib, "src")) else None


def build(ref_root=None):
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    src = os.path.join(ref_root, "src")
    if not os.path.isdir(src):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(src, u + ".cpp") for u in UNITS] + [os.path.join(HERE, "ref_harness.cpp")]
    if os.path.exists(OUT) and all(os.path.getmtime(s) < os.path.getmtime(OUT) for s in srcs + [__file__]):
        return OUT
    cmd = ["g++", "-O2", "-std=c++11", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-DEnableFlexibleLinkers",
           "-I" + src, "-o", OUT] + srcs
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference energy layer failed to build:\n" + r.stdout[-4000:])
    return OUT


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
