// engine_types.h -- device data layout of the batched replica-exchange engine.
//
// One engine holds S independent simulations.  Simulation s has N residues in M
// molecules (contiguous, argfile order) and R replicas; all replicas of all
// simulations are advanced by one kernel launch (one CTA cluster per replica).
//
// HBM layout (all arrays flat, offsets in DevSim):
//   static, per residue   rstat[res_off+i]  float4 (sigma_i/2, q_i*sqrt(DHF), type bits, mol bits)
//                          rexcl[res_off+i]  int4   (chain uid, resSeq, domain uid, bond uid)
//   static, per molecule  mols[mol_off+m]   DevMol (range, flags, graph list offsets)
//   per replica state     pos/rel[state_off + r*N + i]  float4 (x, y, z, 0)
//                          center[molst_off + r*M + m]   float4
//                          emat[emat_off + r*M*M + a*M + b]  double, pair energy of molecules a, b
//                          intra[molst_off + r*M + m]   double, intra + bonded energy of molecule m
//                          potential/temperature/steps/stats[rep_off + r]
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace cgppd {

enum MoveType { kTranslate = 0, kRotate = 1, kFlex = 2, kLocal = 3 };
enum MolFlags { kMolFlexible = 1, kMolCrowder = 2 };

struct DevSim {
    int N, M, R;
    int res_off;                 // first static residue
    int mol_off;                 // first static molecule
    int rep_off;                 // first global replica
    long long state_off;         // residue state of replica 0 (replicas stride N)
    int molst_off;               // molecule state of replica 0 (replicas stride M)
    long long emat_off;          // energy matrix of replica 0 (replicas stride M*M)
    float box, inv_box;
    float w_cum[4];              // cumulative move weights of a flexible molecule (T, R, F, L)
    float w1_cum[3];             // same when it is the only molecule (R, F, L)
    float rigid_rotate_p;        // P(rotate) for a rigid molecule (Bernoulli, else translate)
    int non_crowders;            // molecules before the first crowder
    int nc_mode;                 // 0: bound test uses 0; 1: non-crowder inter energy; 2: potential
    int sample_freq, sample_after;
    float bound_threshold;       // kcal/mol, BOUND_ENERGY_VALUE
    int max_mol;                 // largest molecule
    int crowd_start;             // repulsive crowding: first residue of the trailing crowders
                                 // (their pairs use (6/r)^12 RT below 15 A, no DH); -1: off
    // The same choices as integer thresholds on the raw 32-bit draw w (u = w / 2^32):
    // u < c  <=>  w < ceil(c * 2^32), so the comparisons are exact without FP64.
    unsigned long long thr4[4];  // cumulative weights, flexible molecule
    unsigned long long thr3[3];  // cumulative weights, only molecule
    unsigned long long thr_rot;  // rigid molecule: rotate below, translate above
    // this simulation's ranges of the static lists (first index, count): bonds, angles,
    // torsions (+ their V / phase), indirect pairs, flex residues, flex options, branch
    // residues, local residues, crankshaft residues, active intra tiles
    int lbase[10], lcount[10];
};

struct DevMol {
    int start, count, flags;
    int bond_off, nbond;
    int ang_off, nang;
    int tor_off, ntor;
    int ind_off, nind;           // indirect-neighbour pairs to subtract (not otherwise excluded)
    int flex_off, nflex;         // flexible residues: int4 (ri, degree, option offset, 0)
    int local_off, nlocal;
    int crank_off, ncrank;
    int nintra;                  // intra pairs that are not excluded (flexible molecules)
    int fr0, fr1, fr2;           // residues (molecule-relative) spanning the body frame
    int tile_off, ntile;         // 32 x 32 intra tiles (ta <= tb) holding an unexcluded pair
    float tors_const;            // sum of V_n over the molecule's torsions (kcal/mol)
    int pair_lanes;              // lanes per other residue in the inter pair loop (set per launch)
    int nq;                      // charged residues: the inter pair loop takes them first
};

// Delayed-acceptance counters of one replica slot (not swapped on exchange).
struct DAStats {
    unsigned long long proposals, stage1_reject, stage2_eval, stage2_accept;
    double sum_e2;               // squared (exact - surrogate) energy changes, |exact| <= window
    unsigned long long n_e2;
    double win_e2;               // the same since the last fallback check
    unsigned long long win_n;
};

// Per-replica counters and ratios, swapped with the temperature on exchange
// (src/Replica.cpp:188-210).
struct ReplicaStats {
    int accept, acceptA, reject;
    int totalAcceptReject, totalAccept;
    int boundSamples, samplesSinceLastExchange;
    int totalBoundSamples, totalSamples;
    float acceptanceRatio, accumulativeAcceptanceRatio;
    float fractionBound, accumulativeFractionBound;
    int pad[3];
};

// One fraction-bound sample of a replica slot, the content of the line
// Replica::sample writes to boundconformations (src/Replica.cpp:1037-1093): the
// non-crowder inter-molecule energy, the replica's potential, the slot's temperature
// and the first MC step of the sampling window.
struct SampleRec {
    double enc, potential;
    float temperature;
    int step;
};

struct EngineArgs {
    const DevSim *sims;
    const int *rep_sim;          // global replica -> simulation
    const int *rep_order;        // launch order of k_mc: cluster index -> global replica
    const unsigned short *rqpos; // per residue: its place in the molecule's charged-first order
    const DevMol *mols;
    const float4 *rstat;
    const int4 *rexcl;
    const int2 *bonds;
    const int4 *angles;          // (i, j, k, 0)
    const int4 *tors;            // (i, j, k, l)
    const float4 *torsV;         // V_n cos(sigma_n), n = 1..4, of each torsion
    const float4 *torsS;         // V_n sin(sigma_n)
    const int2 *indsub;
    const int4 *flexres;         // (ri, degree, first option, 0)
    const int4 *flexopt;         // (neighbour, branch offset, branch count, 0)
    const int *branch;
    const int *localres;
    const int *crankres;
    const int2 *tiles;           // active intra tiles (ta, tb) of flexible molecules
    const float *table;          // -4 Eij in kcal/mol, ntypes x ntypes (row stride 32)
    float4 *pos;
    float4 *rel;
    float4 *center;
    double *emat;
    double *intra;
    double *potential;
    float *temperature;
    float *tstep;
    double *rstep;
    unsigned long long *stepc;   // MC steps done by each replica
    unsigned long long *pairc;   // residue-pair terms evaluated by each replica
    ReplicaStats *stats;
    int *tindex;                 // temperature-ladder index held by each replica slot
    int *label;
    int *slot_of_t;              // [rep_off + t] replica slot holding ladder index t
    int *sim_state;              // per simulation: {offset, exchanges done, exch_total, tests_total}
    float4 *report;              // per exchange and ladder index: (fb, afb, ar, aar)
    int2 *exch_report;           // per exchange: (exchanges, tests)
    int report_capacity;         // exchanges the report buffers hold per simulation
    unsigned *errflags;          // per replica error bits
    SampleRec *sample_log;       // [total replicas][sample_cap] or null
    unsigned *sample_count;      // records held per replica
    int sample_cap;
    float4 *sample_xyz;          // [total replicas][sample_cap][sample_nres] coordinates, or null
    int sample_nres;             // leading residues of a replica kept per record
    uint32_t seed_lo, seed_hi;
    int ntypes;
    int cluster;                 // CTAs per replica
    int resident;                // 1: each CTA keeps its replica's state in shared memory
    int any_flexible;            // some molecule carries internal energy terms
    int qfirst;                  // 1: k_mc<.., .., true> reads rigid movers charged first
    int max_n;                   // largest N
    int max_m;                   // largest M
    int max_mol;                 // largest molecule
    int lmax[10];                // largest per-simulation count of each static list
    // delayed acceptance with the learned surrogate (da != 0: k_mc<.., true, false> is launched)
    int da;
    const float *sur_P;          // FP32 master parameters
    const void *sur_wf;          // BF16 Wf[3][256][256] of layers 2..4
    int *sim_da;                 // per simulation: 1 while screening, 0 after a fallback
    DAStats *dastats;            // per replica slot
    float sur_thr2;              // fallback when mean squared error > sur_thr2
    float sur_window;            // errors counted for |exact change| <= sur_window
    int sur_min;                 // ... once a block has at least sur_min of them
};

}  // namespace cgppd
