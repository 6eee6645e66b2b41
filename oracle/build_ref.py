"""Build the reference's own code as a checker, from the reference tree (read-only).

TEST INFRASTRUCTURE ONLY.  Output goes only to oracle/_ref/ (git-ignored):

* oracle/_ref/libcgppd_ref.so -- the energy layer, src/{Potential,Residue,AminoAcids,
  AminoAcid,Geometry,Quaternion,vector3f,TorsionalLookupMatrix}.cpp, with
  oracle/ref_harness.cpp;
* oracle/_ref/cgppd_ref_mc -- the MC layer as well (src/Molecule.cpp, Replica.cpp,
  Simulation.cpp, unmodified), driven by oracle/ref_mc_harness.cpp; two vector
  operators without a return statement are routed to oracle/ref_fixups.cpp at link time.  GSL and logog are
  not installed here: oracle/ref_stubs/ declares the calls the reference makes, and
  oracle/ref_rng.cpp answers its random-number calls with the GB300 engine's Philox
  draws (the Philox itself from oracle/cgppd_oracle.c); logging is compiled out.

* oracle/_ref/cgppd_ref_cuda -- the reference's own program built as its CUDA build
  (`-DEnableCUDA -DEnableStreams`, Makefile:35-39) with libcgppd_gb300.so linked in
  place of its src/CudaFunctions.cu: the drop-in at the link level, through the
  reference's own call sites and src/cudaExterns.h declarations
  (oracle/ref_stubs/cuda/ stands in for the CUDA-samples helper headers).

All use the reference's own flags for the flexible-linker CPU build (-O2 -std=c++11
-DEnableFlexibleLinkers, Makefile:5 and :60-62) plus -ffp-contract=off, so that an
aarch64 host rounds like the x86-64 build the reference was run on.

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
MC_UNITS = UNITS + ["Molecule", "Replica", "Simulation"]
MC_OUT = os.path.join(OUT_DIR, "cgppd_ref_mc")


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


def build_mc(ref_root=None):
    """oracle/_ref/cgppd_ref_mc: the reference's MC layer with the Philox-protocol
    generators, or None without the reference tree."""
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    src = os.path.join(ref_root, "src")
    if not os.path.isdir(src):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    stubs = os.path.join(HERE, "ref_stubs")
    cpp = [os.path.join(src, u + ".cpp") for u in MC_UNITS] + [os.path.join(HERE, f) for f in
                                                                ("ref_rng.cpp", "ref_fixups.cpp",
                                                                 "ref_mc_harness.cpp")]
    philox = os.path.join(HERE, "cgppd_oracle.c")
    deps = cpp + [philox, __file__] + [os.path.join(dp, f) for dp, _, fs in os.walk(stubs) for f in fs]
    if os.path.exists(MC_OUT) and all(os.path.getmtime(d) < os.path.getmtime(MC_OUT) for d in deps):
        return MC_OUT
    obj = os.path.join(OUT_DIR, "philox.o")
    steps = [["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-c", philox, "-o", obj],
             ["g++", "-O2", "-std=c++11", "-ffp-contract=off", "-w", "-DEnableFlexibleLinkers",
              '-DHGVERSION="cgppd reference (checker build)"', "-I" + stubs, "-I" + src, "-o", MC_OUT] + cpp +
             [obj, "-lpthread", "-lm",
              # src/vector3f.cpp:105-117 lack a return statement: calls go to ref_fixups.cpp
              "-Wl,--wrap=_ZN8Vector3fpLES_", "-Wl,--wrap=_ZN8Vector3fmIES_"]]
    for cmd in steps:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference MC layer failed to build:\n" + r.stdout[-4000:])
    return MC_OUT


DROPIN_OUT = os.path.join(OUT_DIR, "cgppd_ref_cuda")


def build_dropin_program(ref_root=None, lib_dir=None):
    """oracle/_ref/cgppd_ref_cuda: the reference's main, Simulation, Replica, Molecule and
    energy layer compiled as its CUDA build and linked against libcgppd_gb300.so (no
    reference CUDA code), or None without the reference tree."""
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    src = os.path.join(ref_root, "src")
    if not os.path.isdir(src):
        return None
    root = os.path.dirname(HERE)
    lib_dir = lib_dir or os.path.join(root, "cgppd_gb300", "_lib")
    lib = os.path.join(lib_dir, "libcgppd_gb300.so")
    if not os.path.exists(lib):
        return None
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    stubs = os.path.join(HERE, "ref_stubs")
    os.makedirs(OUT_DIR, exist_ok=True)
    cpp = [os.path.join(src, u + ".cpp") for u in MC_UNITS + ["main"]] + \
        [os.path.join(HERE, f) for f in ("ref_rng.cpp", "ref_fixups.cpp")]
    philox = os.path.join(HERE, "cgppd_oracle.c")
    deps = cpp + [philox, lib, __file__] + [os.path.join(dp, f) for dp, _, fs in os.walk(stubs) for f in fs]
    if os.path.exists(DROPIN_OUT) and all(os.path.getmtime(d) < os.path.getmtime(DROPIN_OUT) for d in deps):
        return DROPIN_OUT
    obj = os.path.join(OUT_DIR, "philox_cuda.o")
    steps = [["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-c", philox, "-o", obj],
             ["g++", "-O2", "-std=c++11", "-ffp-contract=off", "-w", "-DEnableFlexibleLinkers", "-DEnableCUDA",
              "-DEnableStreams", '-DHGVERSION="cgppd reference (CUDA build on libcgppd_gb300)"',
              "-I" + os.path.join(stubs, "cuda"), "-I" + stubs, "-I" + os.path.join(cuda, "include"), "-I" + src,
              "-o", DROPIN_OUT] + cpp +
             [obj, "-L" + lib_dir, "-lcgppd_gb300", "-L" + os.path.join(cuda, "lib64"), "-lcudart",
              # setup_CUDA (src/Simulation.cpp) calls cuInit of the CUDA driver API: the toolkit's link stub
              "-L" + os.path.join(cuda, "lib64", "stubs"), "-lcuda", "-lpthread",
              "-lm", "-Wl,-rpath," + lib_dir,
              "-Wl,--wrap=_ZN8Vector3fpLES_", "-Wl,--wrap=_ZN8Vector3fmIES_"]]
    for cmd in steps:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference CUDA build against the drop-in library failed:\n" + r.stdout[-4000:])
    return DROPIN_OUT


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else None
    print(build(root))
    print(build_mc(root))
    print(build_dropin_program(root))
