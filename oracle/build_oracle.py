"""Compile the oracle (test infrastructure) into ``oracle/_build/libcgppd_oracle.so``.

``-ffp-contract=off`` keeps float expressions unfused on every host (the reference was
built without FMA contraction on x86-64; aarch64 gcc would otherwise fuse them).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libcgppd_oracle.so")
SRC = [os.path.join(HERE, "cgppd_oracle.c"), os.path.join(HERE, "cgppd_oracle_mc.c")]


def build():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    srcs = [s for s in SRC if os.path.exists(s)]
    if os.path.exists(OUT) and all(os.path.getmtime(s) < os.path.getmtime(OUT) for s in srcs + [__file__]):
        return OUT
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-pthread", "-o", OUT] + srcs + ["-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    return OUT


if __name__ == "__main__":
    print(build())
