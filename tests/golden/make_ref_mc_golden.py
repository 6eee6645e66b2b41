#!/usr/bin/env python3
"""Record trajectories of the reference's own Monte Carlo code.

Runs the reference's Simulation (src/Simulation.cpp init + run, with src/Replica.cpp and
src/Molecule.cpp, unmodified) through oracle/_ref/cgppd_ref_mc -- built by
oracle/build_ref.py where the reference tree is mounted -- with its random-number calls
answered by the GB300 engine's Philox draws (oracle/ref_rng.cpp), on the reference's
REMC regression configuration (tests/remctestfile: ubiquitin with a flexible tail and
an all-flexible UIM, 5 replicas 240-420 K, box 160.7 A, sampling every 10 steps) and on
the reference's bound conformation 1 (data/conf1: the UIM and ubiquitin in contact, both
rigid, same settings).  For each, runs of 1 and 3 exchange blocks of
100 MC steps (prefixes of one another: the draws depend only on the seed, replica slot
and step).  Writes tests/golden/ref_mc_trajectories.json: the initial system (the
reference's coordinates after its own PDB loading and placement) and every run's final
per-replica state (potential, temperature, label, counters, coordinates).

Usage: python tests/golden/make_ref_mc_golden.py
"""
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import ref_mc  # noqa: E402
from helpers import write_pdb, write_reference_data_dir  # noqa: E402

SEED = 7
BLOCK = 100
RUNS = (1, 3)


def argfile(base, blocks, bound):
    text = base.replace("mcsteps 1000", "mcsteps %d" % (BLOCK * blocks)).replace("resteps 100", "resteps %d" % blocks)
    if bound:
        # the two chains of bound conformation 1 where the PDB places them, no segments
        text = text[:text.index("files")] + ("files\n\nt(0,0,0) r(0,0,1,0) data/conf1/1a.pdb UIM1\n"
                                             "t(0,0,0) r(0,0,1,0) data/conf1/1b.pdb ubiquitin\n")
    return text


def trim(state):
    keep = ("potential", "temperature", "translate_step", "rotate_step", "label", "accept", "acceptA", "reject",
            "totalAccept", "totalAcceptReject", "steps", "xyz", "centers")
    return {"replicas": [{k: r[k] for k in keep} for r in state["replicas"]]}


def main():
    if not ref_mc.available():
        sys.exit("the reference tree is needed (set CGPPD_REFERENCE_DIR)")
    ref = oracle.load_reference_data()
    out = {"source": "reference Simulation::run (src/Simulation.cpp, src/Replica.cpp, src/Molecule.cpp) with the "
                     "engine's Philox draws, tests/remctestfile system; see tests/golden/make_ref_mc_golden.py",
           "seed": SEED, "block": BLOCK, "configs": {}}
    for name, bound in (("flexible", False), ("bound", True)):
        cfg = {"runs": {}}
        for blocks in RUNS:
            d = tempfile.mkdtemp()
            write_reference_data_dir(d, ref)
            os.makedirs(os.path.join(d, "data", "conf1"), exist_ok=True)
            for part in ("1a", "1b"):
                write_pdb(os.path.join(d, "data", "conf1", part + ".pdb"), ref["pdbs"]["conf1/" + part]["residues"])
            with open(os.path.join(d, "cfg"), "w") as f:
                f.write(argfile(ref["remctestfile"], blocks, bound))
            res = ref_mc.run(d, "cfg", SEED)
            assert res["rng_errors"] == 0
            if "molecules" not in cfg:
                cfg.update({k: res[k] for k in ("box", "direction_order", "sample_frequency", "sample_after",
                                                "molecules")})
                cfg["initial"] = trim(res["initial"])
            cfg["runs"][str(blocks)] = {"final": trim(res["final"]), "exchanges": res["exchanges"],
                                        "tests": res["tests"]}
        out["configs"][name] = cfg
    path = os.path.join(HERE, "ref_mc_trajectories.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
