// ref_mc_harness.cpp -- runs the reference's own Simulation (src/Simulation.cpp,
// src/Replica.cpp, src/Molecule.cpp, unmodified, CPU build with flexible linkers) on an
// argfile with its generators bound to the GB300 engine's Philox draw protocol
// (oracle/ref_rng.cpp), and writes the initial system and the final state as JSON.
// TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.py into oracle/_ref/cgppd_ref_mc
// where the reference tree is mounted; tests/test_ref_mc.py and
// tests/golden/make_ref_mc_golden.py drive it.
//
// Usage: cgppd_ref_mc SEED OUT.json <the reference's own arguments: -f ARGFILE ...>
// (run in a directory holding the reference's data/ files and the argfile's PDBs).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "Simulation.h"

extern "C" {
void ref_rng_set_direction_order(const int order[3]);
void ref_rng_bind_replica(gsl_rng *r, unsigned long long seed, int slot);
void ref_rng_bind_exchange(gsl_rng *r, unsigned long long seed, int sim_index, int replicas);
void ref_rng_probe(gsl_rng *r, const double *values, int n);
int ref_rng_errors();
unsigned long long ref_rng_steps(const gsl_rng *r);
}

namespace {

// Which component of the reference's random direction each of its three draws feeds:
// the three calls sit in one constructor argument list, whose evaluation order the
// compiler picks.  Probe the reference's own function with draws (0.75, 0.5, 0.5):
// only the component fed by the first call is non-zero.
void probe_direction_order(Molecule &mol, int order[3])
{
    gsl_rng *p = gsl_rng_alloc(gsl_rng_mt19937);
    for (int first = 0; first < 3; ++first) {
        // k-th call returns 0.75 (others 0.5): find the component it lands in
        double v[3] = {0.5, 0.5, 0.5};
        v[first] = 0.75;
        ref_rng_probe(p, v, 3);
        Vector3double d = mol.normalised_random_vector_d(p);
        order[first] = (std::fabs(d.x) > 0.5) ? 0 : (std::fabs(d.y) > 0.5) ? 1 : 2;
        ref_rng_probe(p, v, 3);
        Vector3f f = mol.normalised_random_vector_f(p);
        const int of = (std::fabs(f.x) > 0.5f) ? 0 : (std::fabs(f.y) > 0.5f) ? 1 : 2;
        if (of != order[first]) {
            std::fprintf(stderr, "direction draws: float and double vectors disagree\n");
            std::exit(3);
        }
    }
    gsl_rng_free(p);
}

void put_f(FILE *f, float v) { std::fprintf(f, "%.9g", (double)v); }
void put_d(FILE *f, double v) { std::fprintf(f, "%.17g", v); }

void dump_molecules(FILE *f, Simulation &s, Replica &r)
{
    std::fprintf(f, "\"molecules\": [");
    for (int m = 0; m < r.moleculeCount; ++m) {
        Molecule &mol = r.molecules[m];
        const moldata &md = s.parameters.mdata[m];
        std::fprintf(f, "%s{\"name\": \"%s\", \"flexible\": %d, \"all_flexible\": %d, \"crowder\": %d, "
                        "\"segments\": [",
                     m ? ", " : "", md.name, mol.is_flexible ? 1 : 0, md.all_flexible ? 1 : 0,
                     md.crowder ? 1 : 0);
        for (size_t k = 0; k < md.segments.size(); ++k) {
            std::fprintf(f, "%s[", k ? ", " : "");
            for (size_t i = 0; i < md.segments[k].residue_indices.size(); ++i)
                std::fprintf(f, "%s%d", i ? ", " : "", md.segments[k].residue_indices[i]);
            std::fprintf(f, "]");
        }
        std::fprintf(f, "], \"center\": [");
        put_f(f, mol.center.x), std::fprintf(f, ", "), put_f(f, mol.center.y), std::fprintf(f, ", "),
            put_f(f, mol.center.z);
        std::fprintf(f, "], \"residues\": [");
        for (int i = 0; i < mol.residueCount; ++i) {
            const Residue &q = mol.Residues[i];
            std::fprintf(f, "%s[", i ? ", " : "");
            put_f(f, q.position.x), std::fprintf(f, ", "), put_f(f, q.position.y), std::fprintf(f, ", "),
                put_f(f, q.position.z);
            std::fprintf(f, ", ");
            put_f(f, q.relativePosition.x), std::fprintf(f, ", "), put_f(f, q.relativePosition.y),
                std::fprintf(f, ", "), put_f(f, q.relativePosition.z);
            std::fprintf(f, ", %d, ", q.aminoAcidIndex);
            put_f(f, q.electrostaticCharge), std::fprintf(f, ", "), put_f(f, q.vanderWaalRadius);
            std::fprintf(f, ", %d, %d]", q.resSeq, (int)q.chainId);
        }
        std::fprintf(f, "]}");
    }
    std::fprintf(f, "]");
}

void dump_state(FILE *f, Simulation &s)
{
    const int R = s.parameters.replicas;
    std::fprintf(f, "\"replicas\": [");
    for (int i = 0; i < R; ++i) {
        Replica &r = s.replica[i];
        std::fprintf(f, "%s{\"potential\": ", i ? ", " : "");
        put_d(f, r.potential);
        std::fprintf(f, ", \"temperature\": ");
        put_f(f, r.temperature);
        std::fprintf(f, ", \"translate_step\": ");
        put_f(f, r.translateStep);
        std::fprintf(f, ", \"rotate_step\": ");
        put_d(f, r.rotateStep);
        std::fprintf(f, ", \"label\": %d, \"accept\": %d, \"acceptA\": %d, \"reject\": %d, \"totalAccept\": %d, "
                        "\"totalAcceptReject\": %d, \"steps\": %llu, \"xyz\": [",
                     (int)r.label, r.accept, r.acceptA, r.reject, r.totalAccept, r.totalAcceptReject,
                     ref_rng_steps(r.rng));
        bool first = true;
        for (int m = 0; m < r.moleculeCount; ++m)
            for (int k = 0; k < r.molecules[m].residueCount; ++k) {
                const Vector3f &p = r.molecules[m].Residues[k].position;
                std::fprintf(f, "%s", first ? "" : ", ");
                first = false;
                put_f(f, p.x), std::fprintf(f, ", "), put_f(f, p.y), std::fprintf(f, ", "), put_f(f, p.z);
            }
        std::fprintf(f, "], \"centers\": [");
        for (int m = 0; m < r.moleculeCount; ++m) {
            const Vector3f &c = r.molecules[m].center;
            std::fprintf(f, "%s", m ? ", " : "");
            put_f(f, c.x), std::fprintf(f, ", "), put_f(f, c.y), std::fprintf(f, ", "), put_f(f, c.z);
        }
        std::fprintf(f, "]}");
    }
    std::fprintf(f, "]");
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 4) {
        std::fprintf(stderr, "usage: cgppd_ref_mc SEED OUT.json -f ARGFILE [reference options]\n");
        return 2;
    }
    const unsigned long long seed = std::strtoull(argv[1], nullptr, 10);
    const char *out = argv[2];
    // the reference's own argument vector: program name, then the rest
    std::vector<char *> rargv;
    rargv.push_back(argv[0]);
    for (int k = 3; k < argc; ++k)
        rargv.push_back(argv[k]);
    rargv.push_back(nullptr);
    try {
        Simulation s;
        s.init((int)rargv.size() - 1, rargv.data(), 0);
        int order[3];
        probe_direction_order(s.replica[0].molecules[0], order);
        ref_rng_set_direction_order(order);
        const int R = s.parameters.replicas;
        for (int i = 0; i < R; ++i)
            ref_rng_bind_replica(s.replica[i].rng, seed, i);
        ref_rng_bind_exchange(s.REMCRng, seed, 0, R);
        FILE *f = std::fopen(out, "w");
        if (!f) {
            std::fprintf(stderr, "cannot write %s\n", out);
            return 2;
        }
        std::fprintf(f, "{\"seed\": %llu, \"direction_order\": [%d, %d, %d], \"box\": ", seed, order[0], order[1],
                     order[2]);
        put_f(f, s.parameters.bound);
        std::fprintf(f, ", \"mcsteps\": %d, \"resteps\": %d, \"sample_frequency\": %d, \"sample_after\": %d, ",
                     s.parameters.MCsteps, s.parameters.REsteps, s.parameters.sampleFrequency,
                     s.parameters.sampleStartsAfter);
        dump_molecules(f, s, s.replica[0]);
        std::fprintf(f, ", \"initial\": {");
        dump_state(f, s);
        std::fprintf(f, "}");
        std::fflush(f);
        s.run();
        std::fprintf(f, ", \"final\": {");
        dump_state(f, s);
        std::fprintf(f, "}, \"exchanges\": %d, \"tests\": %d, \"rng_errors\": %d}\n", s.totalExchanges,
                     s.totalTests, ref_rng_errors());
        std::fclose(f);
        return ref_rng_errors() == 0 ? 0 : 4;
    } catch (const char *msg) {
        std::fprintf(stderr, "reference threw: %s\n", msg);
        return 5;
    }
}
