"""The drop-in at the link level: the reference's own CUDA build on libcgppd_gb300.so.

The reference's program (src/main.cpp, src/Simulation.cpp, src/Replica.cpp,
src/Molecule.cpp and the energy layer, unmodified) compiled as its CUDA build
(-DEnableCUDA -DEnableStreams, Makefile:35-39) links against libcgppd_gb300.so in place
of its src/CudaFunctions.cu, with src/cudaExterns.h as the only declaration of the
entry points it calls.  oracle/build_ref.py builds it as oracle/_ref/cgppd_ref_cuda where
the reference tree is mounted; the test is skipped elsewhere.  The program is x86 code
built from sources that are not on the GPU machine, so only the link and the symbol
binding are checked here; the entry points' results are checked by the GPU tests of
the drop-in (tests/test_dropin_gpu.py, tests/test_zz_no_alloc.py).
"""
import os
import subprocess

import pytest

import cgppd_gb300
from helpers import header_functions
from oracle import build_ref

# what src/Replica.cpp and src/Simulation.cpp call through src/cudaExterns.h in the
# flexible-linker CUDA build with streams
CALLED = {"__throwLastCudaError", "copyLJPotentialDataToDevice", "CUDA_EonDevice", "CUDA_EonDeviceNC",
          "CUDA_EonDevice_async", "CUDA_setBoxDimension", "bindLJTexture", "unbindLJTexture"}


def dynsyms(path, defined):
    flag = "--defined-only" if defined else "--undefined-only"
    out = subprocess.run(["nm", "-D", flag, path], stdout=subprocess.PIPE, text=True, check=True).stdout
    return {line.split()[-1].split("@")[0] for line in out.splitlines() if line.strip()}


@pytest.fixture(scope="module")
def program():
    if build_ref.reference_root() is None:
        pytest.skip("the reference tree is not mounted")
    cgppd_gb300.build()
    path = build_ref.build_dropin_program()
    if path is None:
        pytest.skip("the reference's sources or the library are missing")
    return path


def test_reference_cuda_build_links_against_the_library(program):
    lib = cgppd_gb300.LIB
    taken = dynsyms(program, False) & dynsyms(lib, True)
    assert taken == CALLED, taken ^ CALLED
    # every one of them is declared by the library's own header of the entry points
    assert CALLED <= set(header_functions())
    ldd = subprocess.run(["ldd", program], stdout=subprocess.PIPE, text=True, check=True).stdout
    line = [ln for ln in ldd.splitlines() if "libcgppd_gb300.so" in ln]
    assert line and os.path.realpath(line[0].split("=>")[1].split("(")[0].strip()) == os.path.realpath(lib)


def test_reference_cuda_build_prints_its_usage(program):
    ldd = subprocess.run(["ldd", program], stdout=subprocess.PIPE, text=True, check=True).stdout
    if "not found" in ldd:
        pytest.skip("the CUDA driver library is not installed here: " +
                    ", ".join(ln.split()[0] for ln in ldd.splitlines() if "not found" in ln))
    r = subprocess.run([program, "-h"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert r.returncode == 0, r.stdout
    assert "Usage" in r.stdout or "usage" in r.stdout
