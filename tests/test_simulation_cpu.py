"""Argfile and command-line parsing of the C++ Simulation (no GPU).

Reproduces the reference's tests/testSimulation.cpp:7-94 on the same inputs: the
argtestfile and command line of that test (the file's text is in the fixtures).
"""
import ctypes

import pytest

import cgppd_gb300


def dump(argv, mode, cwd):
    L = cgppd_gb300.lib()
    f = L.cgppd_args_dump
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    arr = (ctypes.c_char_p * (len(argv) + 1))(*[a.encode() for a in argv], None)
    buf = ctypes.create_string_buffer(1 << 16)
    import os
    old = os.getcwd()
    os.chdir(cwd)
    try:
        rc = f(len(argv), arr, mode, buf, len(buf))
    finally:
        os.chdir(old)
    text = buf.value.decode()
    if rc != 0:
        return rc, text
    return rc, dict(ln.split("=", 1) for ln in text.splitlines() if "=" in ln)


@pytest.fixture()
def argdir(tmp_path, refdata):
    (tmp_path / "tests").mkdir()
    (tmp_path / "tests" / "argtestfile").write_text(refdata["argtestfile"])
    return tmp_path


def test_command_line(argdir):
    # tests/testSimulation.cpp:8-44
    argv = ["my_programname", "-f", "tests/argtestfile", "-p", "-q", "-t", "23", "-s", "23", "-g", "23", "-z", "2",
            "-m", "23", "-e", "23", "-r", "23", "-b", "23", "-n", "23", "-x", "23", "-d", "23"]
    rc, p = dump(argv, 1 | 4, argdir)
    assert rc == 0, p
    assert p["viewConditions"] == "0" and p["skipsimulation"] == "1"
    assert p["cuda_blockSize"] == "23" and p["auto_blockdim"] == "0"
    for k in ("threads", "streams", "gpus", "MCsteps", "REsteps", "replicas"):
        assert p[k] == "23", k
    assert p["gpuoffset"] == "2"
    assert p["sampleFrequency"] == "5000" and p["sampleStartsAfter"] == "5000"
    assert p["inputFile"] == "1" and p["nonCrowders"] == "0" and p["pid"] == "0" and p["resume"] == "0"
    assert float(p["bound"]) == 23.0 and float(p["temperatureMin"]) == 23.0 and float(p["temperatureMax"]) == 23.0
    assert p["prefix"] == "" and p["file"] == "tests/argtestfile"


def test_config_file(argdir):
    # tests/testSimulation.cpp:46-94
    rc, p = dump(["x", "tests/argtestfile"], 2 | 8, argdir)
    assert rc == 0, p
    assert p["skipsimulation"] == "0" and p["auto_blockdim"] == "1"
    assert p["threads"] == "1" and p["streams"] == "1" and p["gpus"] == "1"
    assert p["MCsteps"] == "10000" and p["REsteps"] == "10000" and p["replicas"] == "1"
    assert p["sampleFrequency"] == "1000" and p["sampleStartsAfter"] == "1000"
    assert p["nonCrowders"] == "2"
    assert float(p["bound"]) == 100.0 and float(p["temperatureMin"]) == 288.0 and float(p["temperatureMax"]) == 300.0
    assert p["prefix"] == "" and p["title"] == "Config file for unit tests"
    assert p["molecules"] == "7" and p["named"] == "2"
    mols = [p["mol%d" % i].split() for i in range(7)]
    ubq, uim = mols[0], mols[1]
    assert ubq[1] == "ubiquitin" and uim[1] == "UIM1"
    assert uim[11] == "1" and uim[12] == "0"           # UIM1 all flexible, no segments
    assert ubq[11] == "0" and ubq[12] == "1" and ubq[13] == "[72,73,74,75]"
    assert [m[10] for m in mols] == ["0", "0", "1", "1", "1", "1", "1"]   # crowders
    assert ubq[2] == "0" and mols[2][2] == "1"          # p(...) sets, t(...) translates
    assert [float(v) for v in ubq[3:10]] == [45.0, 45.0, 45.0, 0.0, 1.0, 0.0, pytest.approx(3.142)]


def test_errors_are_reported(tmp_path):
    rc, msg = dump(["x"], 1, tmp_path)
    assert rc == 1 and "No configuration file" in msg
    rc, msg = dump(["x", "-f", "missing"], 1 | 2, tmp_path)
    assert rc == 1 and "Failed to open config file" in msg
    bad = tmp_path / "bad"
    bad.write_text("files\np(1,1,1) r(1,0,0,0) a.pdb named\nsegments\nother 1 2 3\n")
    rc, msg = dump(["x", "-f", "bad"], 1 | 2, tmp_path)
    assert rc == 1 and "unknown molecule" in msg


def test_repulsive_crowding_key(argdir):
    # the run-time form of the reference's compile-time REPULSIVE_CROWDING switch:
    # off unless the argfile sets it
    rc, p = dump(["x", "tests/argtestfile"], 2 | 8, argdir)
    assert rc == 0 and p["repulsiveCrowding"] == "0"
    text = (argdir / "tests" / "argtestfile").read_text()
    (argdir / "tests" / "crowdfile").write_text("repulsivecrowding 1\n" + text)
    rc, p = dump(["x", "tests/crowdfile"], 2 | 8, argdir)
    assert rc == 0, p
    assert p["repulsiveCrowding"] == "1" and p["nonCrowders"] == "2"


def read_pdb(path, aa_handle, capacity=4096):
    L = cgppd_gb300.lib()
    f = L.cgppd_pdb_read
    f.restype = ctypes.c_int
    P = ctypes.POINTER
    f.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, P(ctypes.c_float), P(ctypes.c_int),
                  ctypes.c_char_p, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int)]
    import numpy as np
    xyz = np.zeros(3 * capacity, np.float32)
    types = np.zeros(capacity, np.int32)
    chains = ctypes.create_string_buffer(capacity)
    seq = np.zeros(capacity, np.int32)
    cidx = np.zeros(capacity, np.int32)
    nch = ctypes.c_int(0)
    n = f(str(path).encode(), aa_handle, capacity, xyz.ctypes.data_as(P(ctypes.c_float)),
          types.ctypes.data_as(P(ctypes.c_int)), chains, seq.ctypes.data_as(P(ctypes.c_int)),
          cidx.ctypes.data_as(P(ctypes.c_int)), ctypes.byref(nch))
    if n < 0:
        buf = ctypes.create_string_buffer(512)
        L.cgppd_get_last_error(buf, 512)
        return n, buf.value.decode()
    return n, dict(xyz=xyz[:3 * n].reshape(n, 3), types=types[:n], chains=chains.raw[:n].decode(), seq=seq[:n],
                   chain_index=cidx[:n], num_chains=nch.value)


@pytest.mark.parametrize("case", ["good", "unknown_residue", "no_ca_records", "missing_file"])
def test_pdb_reader(tmp_path, refdata, case):
    # the reading part of Molecule::initFromPDB (src/Molecule.cpp:506-612); bad files
    # fail with a message instead of indexing the tables with -1
    # (src/AminoAcids.cpp:145-181)
    from helpers import write_reference_data_dir
    write_reference_data_dir(str(tmp_path), refdata)
    L = cgppd_gb300.lib()
    a = L.cgppd_aminoacids_create()
    d = tmp_path / "data"
    assert L.cgppd_aminoacids_load(a, str(d / "AminoAcids").encode(), str(d / "pair_potentials_MJ1996").encode()) == 0
    ubq = d / "application" / "ubq.pdb"
    lines = ubq.read_text().splitlines()
    try:
        if case == "good":
            n, r = read_pdb(ubq, a)
            gold = refdata["pdbs"]["application/ubq"]["residues"]
            assert n == len(gold) == 76 and r["num_chains"] == 1
            assert r["seq"][0] == 1 and r["seq"][-1] == 76
            assert all(t >= 0 for t in r["types"])
            return
        if case == "unknown_residue":
            k = next(i for i, ln in enumerate(lines) if ln.startswith("ATOM") and ln[12:16].strip() == "CA")
            lines[k] = lines[k][:17] + "XYZ" + lines[k][20:]
            ubq.write_text("\n".join(lines) + "\n")
            expect = "Unknown residue name"
        elif case == "no_ca_records":
            ubq.write_text("\n".join(ln for ln in lines if not ln.startswith("ATOM")) + "\n")
            expect = "No C-alpha records"
        else:
            ubq.unlink()
            expect = "Failed to open PDB file"
        n, msg = read_pdb(ubq, a)
        assert n == -1 and expect in msg
    finally:
        L.cgppd_aminoacids_destroy(a)


def write_sample(path, aa_handle, title, temperature, sample, potential, xyz, types, seq, chain, mol):
    import numpy as np
    L = cgppd_gb300.lib()
    f = L.cgppd_pdb_write_sample
    f.restype = ctypes.c_int
    P = ctypes.POINTER
    f.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_float, ctypes.c_int, ctypes.c_double,
                  ctypes.c_int, P(ctypes.c_float), P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int)]
    arrs = [np.ascontiguousarray(x, np.int32) for x in (types, seq, chain, mol)]
    xyz = np.ascontiguousarray(xyz, np.float32)
    return f(str(path).encode(), aa_handle, title.encode(), temperature, sample, potential, len(arrs[0]),
             xyz.ctypes.data_as(P(ctypes.c_float)), *[x.ctypes.data_as(P(ctypes.c_int)) for x in arrs])


def test_sample_pdb_layout_matches_reference(tmp_path, refdata):
    # Replica::saveAsSinglePDB (src/Replica.cpp:1124-1168) for the reference's regression
    # system (ubiquitin, then the UIM: replica-wide chains A and B): the layout of the
    # reference's own sample file (tests/remctest_CPU.tgz, coordinates and header values
    # masked), and the header values as the reference prints them
    import numpy as np
    from helpers import write_reference_data_dir
    write_reference_data_dir(str(tmp_path), refdata)
    L = cgppd_gb300.lib()
    a = L.cgppd_aminoacids_create()
    d = tmp_path / "data"
    assert L.cgppd_aminoacids_load(a, str(d / "AminoAcids").encode(), str(d / "pair_potentials_MJ1996").encode()) == 0
    parts = [read_pdb(d / "application" / name, a)[1] for name in ("ubq.pdb", "uim.pdb")]
    types, seq, chain, mol, xyz = [], [], [], [], []
    base = 0
    for k, r in enumerate(parts):
        types += list(r["types"])
        seq += list(r["seq"])
        chain += [base + c for c in r["chain_index"]]
        mol += [k] * len(r["types"])
        xyz.append(r["xyz"])
        base += r["num_chains"]
    out = tmp_path / "sample_0_240.0K_-0.00.pdb"
    pot = 50.3998794556
    assert write_sample(out, a, "remctest_0", 240.0, 0, pot, np.concatenate(xyz), types, seq, chain, mol) == 0
    lines = out.read_text().splitlines()

    def mask(ln):  # tests/golden/make_golden.py
        if ln.startswith("ATOM"):
            return ln[:30] + "*" + ln[54:]
        if ln.startswith("REMARK") and ":" in ln and not ln.startswith("REMARK simulation"):
            return ln.split(":")[0] + ":*"
        return ln
    assert [mask(ln) for ln in lines] == refdata["remctest"]["CPU"]["pdb_sample_layout"]
    assert lines[1:4] == ["REMARK temperature: 240.0 ", "REMARK sample: 0 ",
                          "REMARK potential: %0.10f " % float(np.float32(pot))]
    first = np.concatenate(xyz)[0]
    assert lines[4][30:54] == "%8.3f%8.3f%8.3f" % tuple(float(v) for v in first)
    # bad input is refused with a message
    assert write_sample(out, a, "t", 300.0, 0, 0.0, np.zeros((1, 3)), [25], [1], [0], [0]) == -1
    L.cgppd_aminoacids_destroy(a)
