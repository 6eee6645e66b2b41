/*
 * cgppd_remc.h -- C ABI of the batched GB300 replica-exchange Monte Carlo engine.
 *
 * The reference runs Replica::MCSearch per replica on host threads, uploading the
 * moved molecule and launching one energy kernel per Monte Carlo step
 * (src/Simulation.cpp:1042-1092, src/Replica.cpp:643-701), and exchanges
 * temperatures on the host (src/Simulation.cpp:770-795).  This engine keeps every
 * replica of every simulation resident on one GPU and runs the move, the energy of
 * the moved molecule, the Metropolis test and the exchange on the device; the host
 * only configures, launches (CUDA-graph replays) and reads results.
 *
 * Units: positions in Angstrom, energies in kcal/mol, temperatures in K.  All
 * functions return 0 (or a non-negative index) on success and -1 on failure, with
 * the message available from cgppd_get_last_error().
 */
#ifndef CGPPD_REMC_H_
#define CGPPD_REMC_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cgppd_engine cgppd_engine;

typedef struct cgppd_sim_params {
    int n_replicas;
    float box;                    /* periodic box edge (> 0), src/structures.h:93 `bound` */
    const float *temperatures;    /* [n_replicas], ladder order */
    const float *translate_steps; /* [n_replicas] A */
    const double *rotate_steps;   /* [n_replicas] rad */
    float move_weights[4];        /* flexible molecules: translate, rotate, flex, local
                                     (reference 1:1:1:1, src/definitions.h:86-89) */
    float rigid_rotate_prob;      /* rigid molecules: P(rotate), else translate (0.5) */
    int sample_frequency;         /* fraction-bound sampling period in MC steps (0 = off) */
    int sample_after;             /* first MC step that samples */
    float bound_threshold;        /* kcal/mol (-1.1844, src/definitions.h:33) */
    int rigid_only;               /* treat flexible molecules as rigid
                                     (Replica::calculate_rigid_potential_only) */
    int repulsive_crowding;       /* pairs with a crowder residue: u = (6/r)^12 RT for
                                     r < 15 A and no Debye-Hueckel term, the reference's
                                     REPULSIVE_CROWDING build (src/Replica.cpp:416-472,
                                     src/definitions.h:18,38); 0 = the full potential.
                                     Crowders must then follow every other molecule and
                                     be rigid. */
} cgppd_sim_params;

/* Replaces the parameter set-up of Simulation::init (src/Simulation.cpp:553) and
 * ::setup_CUDA (src/Simulation.cpp:892-926): a new engine with the raw contact table
 * (ntypes x ntypes, the reference's LJpotentials values, ntypes <= 32), the torsion
 * tables V / phase[nt][nt][4] (src/TorsionalLookupMatrix.h:12-13; may be NULL when no
 * molecule is flexible) and the random seed. */
cgppd_engine *cgppd_engine_create(const float *lj_raw, int ntypes, const double *torsion_V,
                                  const double *torsion_phase, int torsion_types, uint64_t seed);
void cgppd_engine_destroy(cgppd_engine *e);

/* Add a simulation; returns its index. */
int cgppd_engine_add_simulation(cgppd_engine *e, const cgppd_sim_params *p);

/* Replaces Replica::loadMolecule / Molecule::init (src/Replica.cpp:267-299,
 * src/Molecule.cpp:25-64): append a molecule of n residues to simulation `sim`.
 * xyz: placed C-alpha positions [3n]; types/charges/radii per residue; chain_ids,
 * res_seq and chain_index as read from the PDB (chain_index = TER count before the
 * residue); segments: n_segments lists of 0-based residue indices (lengths in
 * seg_lengths, concatenated in seg_residues); center: [3] or NULL for the float mean
 * of xyz.  Returns the molecule index. */
int cgppd_engine_add_molecule(cgppd_engine *e, int sim, int n, const float *xyz, const int *types,
                              const float *charges, const float *radii, const char *chain_ids,
                              const int *res_seq, const int *chain_index, int num_chains, int all_flexible,
                              int crowder, int n_segments, const int *seg_lengths, const int *seg_residues,
                              const float *center);

/* Build the device tables, upload every replica and compute the initial energies
 * (Simulation::init: initialReplica.E() + internal_molecule_E(true), replicated to
 * every replica).  cluster: CTAs per replica (1-8 or 16); threads per CTA (128, 256,
 * 512);
 * 0 for either lets the autotuner pick it from a timed sweep on scratch copies of the
 * state (cached per system shape for the life of the process). */
int cgppd_engine_finalize(cgppd_engine *e, int cluster, int threads);

/* The autotuner's measurements: on input *n is the capacity of the arrays, on output
 * the number of shapes timed (0 if the shape was given). */
int cgppd_engine_tuning(const cgppd_engine *e, int *n, int *clusters, int *threads, float *us_per_step);

/* Replaces MCthreadableFunction's MC loop and Simulation::run's exchange loop
 * (src/Simulation.cpp:737-816, :1044-1092): n_blocks blocks of steps_per_block MC
 * steps per replica, each followed by the per-temperature report (once sampling has
 * started) and an even/odd exchange, except after the last block when
 * exchange_after_last is 0.  Enqueued on `stream` (a cudaStream_t, NULL = the
 * engine's own stream) as CUDA-graph replays; returns without synchronising. */
int cgppd_engine_run(cgppd_engine *e, int n_blocks, int steps_per_block, int exchange_after_last, void *stream);

/* The closing per-temperature report (src/Simulation.cpp:834-848) into report row `row`. */
int cgppd_engine_final_report(cgppd_engine *e, int row, void *stream);

int cgppd_engine_synchronize(cgppd_engine *e);

/* Sizes. */
int cgppd_engine_total_replicas(const cgppd_engine *e);
int cgppd_engine_sim_info(const cgppd_engine *e, int sim, int *n_residues, int *n_molecules, int *n_replicas);

/* Recompute every replica's energy from scratch (molecule-pair matrix and internal
 * energies).  out: [total replicas] or NULL; write_state != 0 also replaces the
 * running totals (removes accumulated rounding). */
int cgppd_engine_recompute(cgppd_engine *e, double *out, int write_state);

/* Per-replica results of one simulation (arrays of n_replicas, replica-slot order):
 * potentials, temperatures, labels, ladder index held, and 16 ints of statistics per
 * replica {accept, acceptA, reject, totalAcceptReject, totalAccept, boundSamples,
 * samplesSinceLastExchange, totalBoundSamples, totalSamples, then the bit patterns of
 * acceptanceRatio, accumulativeAcceptanceRatio, fractionBound,
 * accumulativeFractionBound, 3 unused}.  Any pointer may be NULL. */
int cgppd_engine_get_replicas(cgppd_engine *e, int sim, double *potentials, float *temperatures, int *labels,
                              int *tindex, int *stats16);

/* Coordinates of one replica: positions / relative positions [3N], centres [3M]. */
int cgppd_engine_get_state(cgppd_engine *e, int sim, int replica, float *xyz, float *rel, float *centers);
int cgppd_engine_set_state(cgppd_engine *e, int sim, int replica, const float *xyz, const float *rel,
                           const float *centers);

/* Bulk state transfer of every replica of one simulation, enqueued on `stream`
 * (NULL = the engine's stream) with one copy per array: positions and relative
 * positions as float4 [R*N*4], centres as float4 [R*M*4] (w unused), potentials
 * [R].  Host buffers should be page-locked for the copies to be asynchronous.
 * After an upload, recompute != 0 rebuilds every energy from the new coordinates
 * (required unless the coordinates are the ones last downloaded). */
int cgppd_engine_upload(cgppd_engine *e, int sim, const float *pos4, const float *rel4, const float *centers4,
                        int recompute, void *stream);
int cgppd_engine_download(cgppd_engine *e, int sim, float *pos4, float *rel4, float *centers4, double *potentials,
                          void *stream);

/* Checkpoint and resume.  The reference leaves resuming a stub (src/Simulation.cpp:703-706);
 * here the complete mutable state of a finalized engine -- coordinates, pair matrices,
 * internal energies, potentials, temperature ladder and labels, swapped statistics, the
 * MC step counters that key every replica's Philox stream, exchange bookkeeping, report
 * rows and surrogate counters -- is written to one file, and restoring it into an engine
 * built from the same system continues the run exactly as if it had not stopped.
 * Restore checks the system's shape (simulations, replicas, molecules) and fails on a
 * mismatch.  Both synchronize the engine's stream first. */
int cgppd_engine_checkpoint(cgppd_engine *e, const char *path);
int cgppd_engine_restore(cgppd_engine *e, const char *path);

/* Molecule-pair energies [M*M] and internal energies [M] of one replica. */
int cgppd_engine_get_matrix(cgppd_engine *e, int sim, int replica, double *E, double *intra);

/* Report rows written by the exchanges: per ladder index (fractionBound,
 * accumulativeFractionBound, acceptanceRatio, accumulativeAcceptanceRatio) [4R], and
 * (exchanges, tests) of that exchange. */
int cgppd_engine_get_report(cgppd_engine *e, int sim, int row, float *per_temperature4, int *exch2);

/* Sample records for the reference's boundconformations file (src/Replica.cpp:1037-1093,
 * which writes one line per fraction-bound sample: "step; E_nc (E); T").  After
 * finalize, set_sample_log keeps up to `per_replica` samples per replica slot on the
 * device (0 = none, the default); every sample taken while the log has room is
 * recorded, a full log sets error bit 8.  take_samples copies one simulation's records
 * and empties its logs: counts [n_replicas], and per slot r the records
 * [r * per_replica, r * per_replica + counts[r]) of enc (non-crowder energy, kcal/mol),
 * potential (kcal/mol), temperature (K) and step (first MC step of the sampling
 * window), in the order they were taken.  Any record array may be NULL. */
int cgppd_engine_set_sample_log(cgppd_engine *e, int per_replica);
int cgppd_engine_take_samples(cgppd_engine *e, int sim, int *counts, double *enc, double *potential,
                              float *temperature, int *step);

/* Coordinates of the samples, for the reference's sample PDB files
 * (src/Replica.cpp:1082-1087, 1124-1168): after set_sample_snapshots(residues) every
 * recorded sample also keeps the coordinates of the first `residues` residues of its
 * replica (the non-crowders; 0 = none, the default).  take_sample_xyz copies one
 * simulation's: xyz [n_replicas][per_replica][residues][3], slot r's record k at
 * [r][k] -- the records that take_samples returned last (call it after take_samples and
 * before the next run). */
int cgppd_engine_set_sample_snapshots(cgppd_engine *e, int residues);
int cgppd_engine_take_sample_xyz(cgppd_engine *e, int sim, float *xyz);

/* MC steps done and residue-pair terms evaluated by all replicas since creation. */
int cgppd_engine_counters(cgppd_engine *e, unsigned long long *mc_steps, unsigned long long *pair_evals);

/* OR of the per-replica status bits: 1 a move type with no candidate residue was drawn
 * and left the molecule unchanged; 2 a proposal's energy change was not finite
 * (non-finite coordinates or energies) and the move was rejected; 4 an exchange test
 * met a non-finite potential and the pair did not exchange; 8 a sample was taken while
 * the sample log was full (see cgppd_engine_set_sample_log) and was not recorded. */
unsigned cgppd_engine_error_bits(cgppd_engine *e);

/* The same bits per replica of simulation `sim` (out: [n_replicas], replica-slot order). */
int cgppd_engine_replica_error_bits(cgppd_engine *e, int sim, unsigned *out);

/* Kernel launches enqueued by the last cgppd_engine_run call. */
int cgppd_engine_last_launches(const cgppd_engine *e);

/* Launch shape in use: CTAs per replica and threads per CTA; returns 1 when each
 * CTA keeps its replica's state in shared memory for the whole launch, else 0. */
int cgppd_engine_launch_shape(const cgppd_engine *e, int *cluster, int *threads);

/* Before finalize: allow (1, default) or forbid (0) shared-memory-resident replica
 * state; it is used only when the state fits. */
int cgppd_engine_set_resident(cgppd_engine *e, int allow);

/* Replaces Graph::init for inspection (src/Geometry.cpp:34-192): the flexible-segment
 * graph of one molecule of n residues.  counts9 = {bonds, angles, torsions, rigid
 * domains, segment bonds, indirect neighbours, local residues, crankshaft residues,
 * flex residues}. */
int cgppd_graph_counts(int n, const char *chain_ids, int all_flexible, int n_segments, const int *seg_lengths,
                       const int *seg_residues, int num_chains, int *counts9);

#ifdef __cplusplus
}
#endif

#endif /* CGPPD_REMC_H_ */
