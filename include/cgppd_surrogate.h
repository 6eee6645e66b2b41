/*
 * cgppd_surrogate.h -- learned pair-energy surrogate and delayed-acceptance screening.
 *
 * No counterpart in the reference: the reference evaluates every proposal with the
 * exact potential (src/Replica.cpp:350-414).  Here a small MLP (8 -> 256 x 4 SiLU -> 1)
 * predicts the inter-molecule energy of two copies of one rigid molecule from their
 * relative pose, trained with the library's own CUDA kernels (BF16 tcgen05 GEMMs,
 * FP32 accumulation, Adam) on (pose, exact pair energy) samples the exact engine
 * produces.  Attached to an engine, it screens proposals in a two-stage
 * delayed-acceptance Metropolis test whose second stage is the exact energy, so the
 * sampled distribution is unchanged; the engine also measures the surrogate's error
 * on every second-stage evaluation and falls back to the plain test when the error
 * drifts past a threshold.
 *
 * Pose features (8): the minimum-image centre-to-centre vector in the first molecule's
 * body frame / 20 A, 10 A / distance, and the relative rotation as a unit quaternion
 * with w >= 0.  The body frame is the Gram-Schmidt frame of three fixed residues.
 *
 * All functions return 0 on success and -1 on failure (message via
 * cgppd_get_last_error) unless stated otherwise.
 */
#ifndef CGPPD_SURROGATE_H_
#define CGPPD_SURROGATE_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cgppd_surrogate cgppd_surrogate;
struct cgppd_engine;

/* A surrogate with seeded initial parameters; `batch` (multiple of 128) is the
 * training mini-batch and the inference chunk.  NULL on failure. */
cgppd_surrogate *cgppd_surrogate_create(int batch, unsigned long long seed);
void cgppd_surrogate_destroy(cgppd_surrogate *s);

/* Number of FP32 master parameters and their layout:
 * W1[256][8], b1[256], W2[256][256] (out, in), b2, W3, b3, W4, b4, w5[256], b5[1]. */
int cgppd_surrogate_num_params(void);
int cgppd_surrogate_get_params(cgppd_surrogate *s, float *out);
int cgppd_surrogate_set_params(cgppd_surrogate *s, const float *in);

/* Mean squared error of the network on (X[n][8], y[n]) and, if grad != NULL, its
 * gradient with respect to every master parameter (n % 128 == 0, n <= batch). */
int cgppd_surrogate_loss_grad(cgppd_surrogate *s, const float *X, const float *y, int n, float *loss, float *grad);

/* Predictions for n feature rows (host or device pointers). */
int cgppd_surrogate_predict(cgppd_surrogate *s, const float *X, int n, float *out);

/* Training samples (host arrays), appended in order. */
int cgppd_surrogate_add_samples(cgppd_surrogate *s, const float *X, const float *y, int n);
int cgppd_surrogate_clear_samples(cgppd_surrogate *s);
long long cgppd_surrogate_num_samples(cgppd_surrogate *s);
int cgppd_surrogate_get_samples(cgppd_surrogate *s, float *X, float *y, long long n);

/* Append n (pose, exact pair energy) samples drawn from the current states of the
 * engine's simulation `sim`: per sample a replica and a molecule pair a < b chosen at
 * random, and with probability `proposal_fraction` molecule a displaced by one MC
 * proposal of that replica (translate or rotate with its step sizes).  The energy is
 * the exact FP32-pair / compensated-sum energy of the pair.  The simulation must be
 * surrogate-compatible (cgppd_engine_surrogate_compatible). */
int cgppd_surrogate_collect(cgppd_surrogate *s, struct cgppd_engine *e, int sim, int n, double proposal_fraction,
                            unsigned long long seed);

/* Adam training for `epochs` passes over the first (1 - val_fraction) of the samples
 * (targets clipped to +-clip kcal/mol); history (2 x epochs floats, may be NULL)
 * receives per epoch the training RMSE and the held-out RMSE over |y| <= clip. */
int cgppd_surrogate_train(cgppd_surrogate *s, int epochs, float lr, float clip, float val_fraction, float *history);

/* 1 if every molecule of simulation `sim` is a rigid, non-crowder copy of one molecule
 * (same residue count, types, charges and radii), 2..64 molecules of >= 3 residues;
 * else 0 (or -1 on error). */
int cgppd_engine_surrogate_compatible(struct cgppd_engine *e, int sim);

/* Screen the proposals of every compatible simulation of a finalized engine with `s`
 * (NULL detaches).  The surrogate's parameters are read at each run, so it must outlive
 * the engine or be detached first.  `rmse_threshold` (kcal/mol): a simulation falls
 * back to the plain test once the RMS of (exact - surrogate) energy changes over an
 * exchange block's second-stage evaluations with |exact change| <= `error_window`
 * exceeds it (checked after every block with at least `min_evals` such evaluations).
 * Delayed acceptance needs 4 or 8 CTAs per replica; the launch shape is re-chosen. */
int cgppd_engine_set_surrogate(struct cgppd_engine *e, cgppd_surrogate *s, float rmse_threshold,
                               float error_window, int min_evals);

/* Delayed-acceptance counters of simulation `sim`, summed over its replicas:
 * out[0] proposals screened, out[1] rejected by the surrogate (stage 1),
 * out[2] exact evaluations (stage 2), out[3] accepted at stage 2,
 * out[4] sum of squared errors of the counted stage-2 evaluations, out[5] their number,
 * out[6] 1 while the simulation still screens, 0 after falling back. */
int cgppd_engine_surrogate_stats(struct cgppd_engine *e, int sim, double *out);

#ifdef __cplusplus
}
#endif

#endif /* CGPPD_SURROGATE_H_ */
