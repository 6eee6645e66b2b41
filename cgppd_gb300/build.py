"""Build the native library in-tree: ``cgppd_gb300/_lib/libcgppd_gb300.so``.

CUDA sources are compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``),
host C++ with g++; translation units compile in parallel and are skipped when their
object is newer than every source and header.  No cmake, no torch extension machinery.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libcgppd_gb300.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cgppd_gb300")


APP = os.path.join(LIBDIR, "cgppd")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "host", "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(CSRC, "host", "*.cpp")))
    return cu, cpp


def _headers():
    hs = []
    for pat in ("*.h", "*.cuh", "*/*.h", "*/*.cuh"):
        hs += glob.glob(os.path.join(CSRC, pat))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(obj, src, newest_header):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or newest_header > t


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, ptxas_info=False):
    """Compile every translation unit that changed and link the shared library."""
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu, cpp = _sources()
    hdrs = _headers()
    newest = max([os.path.getmtime(h) for h in hdrs] + [0.0])
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(home, "include")]
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.relpath(src, CSRC).replace(os.sep, "_") + ".o")
        objs.append(obj)
        if _stale(obj, src, newest):
            cmd = [nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"] + inc + ["-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in cpp:
        obj = os.path.join(BUILD, os.path.relpath(src, CSRC).replace(os.sep, "_") + ".o")
        objs.append(obj)
        if _stale(obj, src, newest):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall",
                         "-Wno-unused-function"] + inc + ["-c", src, "-o", obj])
    outs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc, GENCODE, "-shared", "-o", LIB] + objs + ["-lpthread"])
    # the `cgppd` command, linked against the library (found next to it at run time)
    app_src = os.path.join(CSRC, "app", "cgppd_main.cpp")
    if not os.path.exists(APP) or os.path.getmtime(APP) < max(os.path.getmtime(LIB), os.path.getmtime(app_src)):
        _run(["g++", "-O2", "-o", APP, app_src, "-L" + LIBDIR, "-lcgppd_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
