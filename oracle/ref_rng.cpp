// ref_rng.cpp -- the GSL calls of the reference's MC layer, answered with the draws of
// the GB300 engine's Philox protocol.  TEST INFRASTRUCTURE ONLY: linked into
// oracle/_ref/cgppd_ref_mc (built by oracle/build_ref.py from the reference's own
// Molecule, Replica and Simulation sources) so that the reference's Replica::MCSearch
// (src/Replica.cpp:350-414) and Simulation::run (src/Simulation.cpp:709-830) make exactly
// the moves and decisions the engine makes from the same seed, and their trajectories
// can be compared step by step with the oracle's restatement and with the engine.
//
// Nothing of GSL is reproduced: the reference asks its generators for uniforms,
// bounded integers, Bernoulli trials and discrete draws in a fixed order per MC step;
// every such call is mapped onto the word of the engine's draw that serves the same
// purpose:
//   per replica slot r, MC step t: Philox4x32-10 with key {seed_lo ^ 0x9E3779B9 (r + 1),
//   seed_hi} and counters {t, t >> 32, b, 'MC'} for b = 0..2 give words w[0..11]:
//     w0 molecule, w1 move type, w2..w4 direction (x, y, z), w5 flex residue / local
//     kind, w6 flex neighbour / local residue, w7 crankshaft flip, w8 Metropolis;
//   exchange sweep x: key {seed_lo ^ 0xB5297A4D, seed_hi ^ 0x68E31DA4 (sim + 1)},
//     counters {x, 0, ti, 'RE'}, word 0 for the test of ladder pair (ti, ti + 1).
// A word w stands for the uniform w / 2^32; a bounded integer is floor(u n); a
// Bernoulli(p) trial is u < p; a discrete draw inverts the float cumulative weights.
// A call that the protocol does not expect at that point is counted as an error.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"

extern "C" void oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]);

struct gsl_rng_type {
    int unused;
};

namespace {
const gsl_rng_type kType = {0};

enum Kind { kUnbound = 0, kReplica = 1, kExchange = 2 };
// the call the protocol expects next (replica generators)
enum Call { kStepStart, kMoveType, kMoveDraws, kAfterMove };
enum Op { kUniform, kInt, kBern, kDiscrete };

struct Expect {
    Op op;
    int word;
};

std::mutex g_mu;
int g_errors = 0;
int g_dir_order[3] = {2, 3, 4};  // word of the 1st, 2nd and 3rd direction draw

double u01(uint32_t w) { return (double)w * 2.3283064365386963e-10; }

int pick(double u, unsigned long n)
{
    unsigned long k = (unsigned long)(u * (double)n);
    return (int)(k < n ? k : n - 1);
}

void error() { ++g_errors; }
}  // namespace

struct gsl_rng {
    int kind = kUnbound;
    uint32_t key[2] = {0, 0};
    // replica slot
    int n_molecules = 1;
    unsigned long long step = 0;   // next MC step
    uint32_t w[12] = {0};
    Call call = kStepStart;
    std::vector<Expect> script;    // draws of the current move still to come
    size_t next = 0;
    // exchange generator
    int R = 0, x = 0, offset = 0, k = 0;
};

struct gsl_ran_discrete_t {
    int K;
    float cum[8];
};

extern "C" {

const gsl_rng_type *gsl_rng_mt19937 = &kType;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *) { return new gsl_rng(); }

void gsl_rng_set(const gsl_rng *, unsigned long) {}

void gsl_rng_free(gsl_rng *r) { delete r; }

// ---------------------------------------------------------------- binding (harness)

// Which evaluation order the compiler gave the three draws of a direction vector
// (the reference builds Vector3(u - 0.5, 0.5 - u, u - 0.5) from three calls in one
// argument list): order[k] = component (0 x, 1 y, 2 z) that the k-th call feeds.
void ref_rng_set_direction_order(const int order[3])
{
    for (int k = 0; k < 3; ++k)
        g_dir_order[k] = 2 + order[k];
}

void ref_rng_bind_replica(gsl_rng *r, unsigned long long seed, int slot)
{
    r->kind = kReplica;
    r->key[0] = (uint32_t)seed ^ (0x9E3779B9u * (uint32_t)(slot + 1));
    r->key[1] = (uint32_t)(seed >> 32);
    r->step = 0;
    r->call = kStepStart;
    r->script.clear();
    r->next = 0;
}

void ref_rng_bind_exchange(gsl_rng *r, unsigned long long seed, int sim_index, int replicas)
{
    r->kind = kExchange;
    r->key[0] = (uint32_t)seed ^ 0xB5297A4Du;
    r->key[1] = (uint32_t)(seed >> 32) ^ (0x68E31DA4u * (uint32_t)(sim_index + 1));
    r->R = replicas;
    r->x = 0;
    r->offset = 0;
    r->k = 0;
}

// A probe generator that returns the given uniforms in turn (direction-order probe).
static std::vector<double> g_probe;
static size_t g_probe_next = 0;

void ref_rng_probe(gsl_rng *r, const double *values, int n)
{
    r->kind = 3;
    g_probe.assign(values, values + n);
    g_probe_next = 0;
}

int ref_rng_errors() { return g_errors; }

unsigned long long ref_rng_steps(const gsl_rng *r) { return r->step; }

}  // extern "C"

namespace {

void begin_step(gsl_rng *r)
{
    const unsigned long long t = r->step++;
    for (int b = 0; b < 3; ++b) {
        const uint32_t ctr[4] = {(uint32_t)t, (uint32_t)(t >> 32), (uint32_t)b, 0x4D43u};
        oracle_philox4x32_10(ctr, r->key, r->w + 4 * b);
    }
    r->call = kMoveType;
    r->script.clear();
    r->next = 0;
}

void push_direction(gsl_rng *r)
{
    for (int k = 0; k < 3; ++k)
        r->script.push_back({kUniform, g_dir_order[k]});
}

// The draws of a move of type `type` after its type draw (src/Molecule.cpp:193-504).
void plan_move(gsl_rng *r, int type)
{
    switch (type) {
    case 0:  // MC_TRANSLATE: normalised_random_vector_f
    case 1:  // MC_ROTATE: normalised_random_vector_d
        push_direction(r);
        break;
    case 2:  // MC_FLEX: axis, residue, neighbour
        push_direction(r);
        r->script.push_back({kInt, 5});
        r->script.push_back({kInt, 6});
        break;
    case 3:  // MC_LOCAL: translate-or-crankshaft, then its own draws (planned when known)
        r->script.push_back({kBern, 5});
        break;
    }
    r->call = kMoveDraws;
}

// The next draw of the current move; `op` is what the reference asks for.
uint32_t move_word(gsl_rng *r, Op op)
{
    if (r->next >= r->script.size() || r->script[r->next].op != op) {
        error();
        return 0;
    }
    const uint32_t w = r->w[r->script[r->next].word];
    ++r->next;
    return w;
}

void move_drawn(gsl_rng *r)
{
    if (r->next >= r->script.size())
        r->call = kAfterMove;
}

}  // namespace

extern "C" {

double gsl_rng_uniform(const gsl_rng *cr)
{
    std::lock_guard<std::mutex> lock(g_mu);
    gsl_rng *r = const_cast<gsl_rng *>(cr);
    if (r->kind == 3)
        return g_probe_next < g_probe.size() ? g_probe[g_probe_next++] : 0.5;
    if (r->kind == kExchange) {
        if (r->R < 2) {
            error();
            return 0.0;
        }
        const int ti = r->offset + 2 * r->k;
        const uint32_t ctr[4] = {(uint32_t)r->x, 0u, (uint32_t)ti, 0x5245u};
        uint32_t o[4];
        oracle_philox4x32_10(ctr, r->key, o);
        ++r->k;
        if (r->offset + 2 * r->k >= r->R - 1) {  // the sweep's last test: next sweep
            do {
                ++r->x;
                r->offset = 1 - r->offset;
            } while (r->offset >= r->R - 1);
            r->k = 0;
        }
        return u01(o[0]);
    }
    if (r->kind != kReplica) {
        error();
        return 0.0;
    }
    if (r->call == kMoveDraws) {
        const double u = u01(move_word(r, kUniform));
        move_drawn(r);
        return u;
    }
    if (r->call == kAfterMove) {  // the Metropolis draw (src/Replica.cpp:395)
        r->call = kStepStart;
        return u01(r->w[8]);
    }
    error();
    return 0.0;
}

unsigned long int gsl_rng_uniform_int(const gsl_rng *cr, unsigned long int n)
{
    std::lock_guard<std::mutex> lock(g_mu);
    gsl_rng *r = const_cast<gsl_rng *>(cr);
    if (r->kind != kReplica || n == 0) {
        error();
        return 0;
    }
    if (r->call == kStepStart || r->call == kAfterMove) {  // the molecule (src/Replica.cpp:355)
        begin_step(r);
        r->n_molecules = (int)n;
        return (unsigned long)pick(u01(r->w[0]), n);
    }
    if (r->call == kMoveDraws) {
        const int k = pick(u01(move_word(r, kInt)), n);
        move_drawn(r);
        return (unsigned long)k;
    }
    error();
    return 0;
}

unsigned int gsl_ran_bernoulli(const gsl_rng *cr, double p)
{
    std::lock_guard<std::mutex> lock(g_mu);
    gsl_rng *r = const_cast<gsl_rng *>(cr);
    if (r->kind != kReplica) {
        error();
        return 0;
    }
    if (r->call == kMoveType) {  // rigid molecule: rotate (1) or translate (0)
        const unsigned v = u01(r->w[1]) < p ? 1u : 0u;
        plan_move(r, (int)v);
        return v;
    }
    if (r->call == kMoveDraws) {
        const bool local_kind = r->next < r->script.size() && r->script[r->next].op == kBern &&
                                r->script[r->next].word == 5;
        const unsigned v = u01(move_word(r, kBern)) < p ? 1u : 0u;
        if (local_kind) {
            // src/Molecule.cpp:415-448: crankshaft (1): residue, flip; translate (0):
            // residue, then the direction
            r->script.push_back({kInt, 6});
            if (v)
                r->script.push_back({kBern, 7});
            else
                push_direction(r);
        }
        move_drawn(r);
        return v;
    }
    error();
    return 0;
}

gsl_ran_discrete_t *gsl_ran_discrete_preproc(size_t K, const double *P)
{
    gsl_ran_discrete_t *g = new gsl_ran_discrete_t();
    g->K = (int)K;
    if (K < 1 || K > 8) {
        error();
        return g;
    }
    // cumulative weights normalised in float, as the engine forms its thresholds
    float sum = 0.0f;
    for (size_t k = 0; k < K; ++k)
        sum += (float)P[k];
    float acc = 0.0f;
    for (size_t k = 0; k < K; ++k) {
        acc += (float)P[k];
        g->cum[k] = acc / sum;
    }
    g->cum[K - 1] = 1.0f;
    return g;
}

size_t gsl_ran_discrete(const gsl_rng *cr, const gsl_ran_discrete_t *g)
{
    std::lock_guard<std::mutex> lock(g_mu);
    gsl_rng *r = const_cast<gsl_rng *>(cr);
    if (r->kind != kReplica || r->call != kMoveType) {
        error();
        return 0;
    }
    const double u = u01(r->w[1]);
    int k = 0;
    while (k < g->K - 1 && !(u < (double)g->cum[k]))
        ++k;
    // the reference shifts the draw by one for a molecule alone in its replica
    // (src/Molecule.cpp:455-458: no translations)
    plan_move(r, r->n_molecules > 1 ? k : k + 1);
    return (size_t)k;
}

void gsl_ran_discrete_free(gsl_ran_discrete_t *g) { delete g; }

}  // extern "C"
