"""The C++ Simulation (argfile -> GPU engine -> reference output files) on a GB300.

Input: the reference's own REMC regression configuration (tests/remctestfile: ubiquitin
with a flexible tail and an all-flexible UIM in a 160.7 A box, 5 replicas 240-420 K,
1000 MC steps, 100 exchange blocks, sampling every 10 steps) with the reference's
parameter files and structures (fixtures).  The reference's seeded outputs
(tests/remctest_{CPU,GPU}.tgz) give the file layout, which must match exactly, and one
sample each of the acceptance and exchange statistics, which must fall within the
spread of independent runs here (the random streams differ: GSL MT19937 there,
Philox here): final acceptance ratios, exchange ratio, fraction bound, and the mean
potential of the samples at each temperature (boundconformations).
"""
import ctypes
import os
import re

import numpy as np
import pytest

import cgppd_gb300
from helpers import write_reference_data_dir

pytestmark = pytest.mark.gpu


def run_sim(workdir, argv):
    L = cgppd_gb300.lib()
    f = L.cgppd_simulation_main
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]
    arr = (ctypes.c_char_p * (len(argv) + 1))(*[a.encode() for a in argv], None)
    old = os.getcwd()
    os.chdir(workdir)
    try:
        return f(len(argv), arr, 0)
    finally:
        os.chdir(old)


def parse_rows(path):
    lines = open(path).read().splitlines()
    rows = [ln for ln in lines if ":" in ln and not ln.startswith("Iteration")]
    return lines, [[float(x) for x in ln.split(":", 1)[1].replace("|", " ").split()] for ln in rows]


@pytest.fixture(scope="module")
def workdir(tmp_path_factory, refdata):
    d = tmp_path_factory.mktemp("remc")
    write_reference_data_dir(str(d), refdata)
    return d


def sampled_energy_by_temperature(path):
    """Mean sampled replica potential per temperature label of a boundconformations file
    (lines "step; E_nc (E); T" followed by the sample's PDB name)."""
    per_t = {}
    for ln in open(path).read().splitlines()[2:]:
        if ";" not in ln:
            continue
        f = ln.split(";")
        per_t.setdefault(f[2].strip(), []).append(float(f[1].split("(")[1].split(")")[0]))
    return {t: (float(np.mean(v)), len(v)) for t, v in per_t.items()}


def config(refdata, prefix, seed):
    text = refdata["remctestfile"].replace("prefix remctest", "prefix %s\nseed %d" % (prefix, seed))
    return text


def test_output_files_match_reference_layout(workdir, refdata):
    (workdir / "remc_a").write_text(config(refdata, "remctest", 11))
    assert run_sim(workdir, ["cgppd", "-f", "remc_a"]) == 0
    out = workdir / "output" / "remctest_0"
    gold = refdata["remctest"]["CPU"]
    acc_lines, acc = parse_rows(out / "acceptance_ratios")
    assert acc_lines[:2] == gold["acceptance_header"]
    assert len(acc) == gold["acceptance_rows"] == 100
    fb_lines, fb = parse_rows(out / "fractionBound")
    assert fb_lines[:3] == gold["fraction_header"]
    ex = open(out / "exchange_freq").read().splitlines()
    assert ex[0] == "# Iteration continous_ratio, inst_ratio" and len(ex) - 1 == gold["exchange_rows"]
    assert open(out / "fileindex").read().splitlines() == gold["fileindex"]
    bc = open(out / "boundconformations").read().splitlines()
    assert bc[:2] == gold["boundconformations_header"]
    # one sample per replica and block (sampling every 10 steps, 10-step blocks): the
    # reference's line pairs "step; E_nc (E); T" + PDB name, steps 0, 10, ..., 990
    assert len(bc) - 2 == 2 * 5 * 100
    steps = sorted({int(ln.split(";")[0]) for ln in bc[2::2]})
    assert steps == list(range(0, 1000, 10))
    assert all(ln.startswith("output/remctest_0/pdb/sample_") for ln in bc[3::2])
    counts = {t: n for t, (_, n) in sampled_energy_by_temperature(out / "boundconformations").items()}
    assert counts == gold["sampled_energy_count_by_temperature"]
    # row labels: MC step counts of the blocks, then the closing row
    labels = [int(ln.split(":")[0]) for ln in acc_lines[2:] if ":" in ln]
    assert labels == list(range(10, 1001, 10))
    assert (out / "pdb" / "final_lowest_temperature.pdb").exists()
    # every sample line names its PDB file (the reference records all samples), laid out
    # as the reference's: header, the non-crowders' C-alpha records in replica-wide
    # chains, TER records, END (coordinates and header values masked)
    names = [ln for ln in bc[3::2]]
    assert len(names) == gold["pdb_sample_count"]
    for name in names:
        assert (workdir / name).exists(), name
    first = open(workdir / names[0]).read().splitlines()
    assert [mask_pdb_line(ln) for ln in first] == gold["pdb_sample_layout"]
    # its potential header is the sample line's replica potential (a float printed with
    # 10 decimals; the sample line prints 5)
    pot = float(bc[2].split("(")[1].split(")")[0])
    assert re.fullmatch(r"REMARK potential: -?\d+\.\d{10} ", first[3]), first[3]
    assert abs(float(first[3].split(":")[1]) - pot) <= 5e-6 + 1e-6 * abs(pot)


def mask_pdb_line(ln):
    """tests/golden/make_golden.py: a sample PDB line without the coordinates of ATOM
    records and the values of the REMARK records."""
    if ln.startswith("ATOM"):
        return ln[:30] + "*" + ln[54:]
    if ln.startswith("REMARK") and ":" in ln and not ln.startswith("REMARK simulation"):
        return ln.split(":")[0] + ":*"
    return ln


def test_statistics_within_spread_of_reference(workdir, refdata):
    finals, exch, fbound, energies = [], [], [], []
    for seed in range(1, 33):
        prefix = "stat%d" % seed
        (workdir / prefix).write_text(config(refdata, prefix, seed))
        assert run_sim(workdir, ["cgppd", "-f", prefix]) == 0
        out = workdir / "output" / (prefix + "_0")
        _, acc = parse_rows(out / "acceptance_ratios")
        finals.append(acc[-1][1::2])
        _, fb = parse_rows(out / "fractionBound")
        fbound.append(fb[-1][1::2])
        exch.append(float(open(out / "exchange_freq").read().splitlines()[-1].split()[1]))
        energies.append(sampled_energy_by_temperature(out / "boundconformations"))
    finals = np.array(finals)
    mean, sd = finals.mean(0), finals.std(0, ddof=1)
    em, es = np.mean(exch), np.std(exch, ddof=1)
    for arch in ("CPU", "GPU"):
        g = refdata["remctest"][arch]
        ref_acc = np.array(g["acceptance_final_cumulative"])
        z = np.abs(ref_acc - mean) / np.maximum(sd, 0.01)
        assert np.all(z < 4.5), (arch, ref_acc, mean, sd)
        assert abs(g["exchange_final_cumulative"] - em) / max(es, 0.01) < 4.5, (arch, g["exchange_final_cumulative"],
                                                                                  em, es)
        assert np.allclose(np.array(g["fraction_final_cumulative"]), np.mean(fbound, 0), atol=0.05)
        # per-temperature mean energy of the reference's samples against the spread of
        # the 32 runs' means at the same temperature
        for t, e_ref in g["sampled_energy_mean_by_temperature"].items():
            ours = np.array([run[t][0] for run in energies])
            z = abs(e_ref - ours.mean()) / max(ours.std(ddof=1), 0.05)
            assert z < 4.5, (arch, t, e_ref, ours.mean(), ours.std(ddof=1))
