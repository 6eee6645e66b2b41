/*
 * cgppd_oracle_mc.c -- CPU restatement of the reference's replica-exchange Monte Carlo
 * loop.  TEST INFRASTRUCTURE ONLY: used by tests/ as the trajectory checker of the GPU
 * engine and by bench.py as the timed CPU baseline ("port" of the reference CPU path).
 *
 * Restates, in the reference's own precision (float coordinates, double quaternions,
 * full energy recomputation every step):
 *   - Replica::MCSearch                 src/Replica.cpp:350-414
 *   - Molecule::make_MC_move and moves  src/Molecule.cpp:146-504
 *   - Quaternion / rotateVector         src/Quaternion.cpp:12-112
 *   - Replica::E() + internal_molecule_E(true) each step (src/Replica.cpp:359-379)
 *   - Simulation::run exchange sweep    src/Simulation.cpp:770-795
 *   - Replica::sample / fraction_bound / acceptance_ratio (src/Replica.cpp:1037-1122)
 * The random draws follow the GPU engine's protocol (Philox4x32-10, nine words per
 * step, one word per exchange test) so the two trajectories can be compared step by
 * step; the reference itself draws from GSL's MT19937, which changes which states
 * are visited but not their distribution.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cgppd_oracle_internal.h"

#define OR_RT_TO_KCAL 0.59218674898147583
#define OR_DHC 4.1507959365844727
#define OR_K_SPRING 378.0
#define OR_GAMMA_RECIP 10.0f
#define OR_EPS 1e-38f
#define OR_KCAL 4184.0f
#define OR_RGAS 8.3144621f

/* The system, with residue indices of the graph lists local to each molecule. */
typedef struct {
    int N, M;
    const int *mstart, *mcount, *mflags; /* flags: 1 flexible, 2 crowder */
    const int *aa;
    const float *q, *sig;
    const float *table; /* raw contact table ntypes x ntypes */
    int ntypes;
    float box;
    const int *excl; /* N*4: chain uid, resSeq, domain uid, bond uid */
    const int *ind_off, *nind, *ind;
    const int *bond_off, *nbond, *bonds;
    const int *ang_off, *nang, *angles;
    const int *tor_off, *ntor, *tors;
    const double *torsV, *torsS;
    int tors_types;
    const int *flex_off, *nflex, *flexres; /* (ri, degree, first option) */
    const int *flexopt;                    /* (neighbour, branch offset, branch count) */
    const int *branch;
    const int *local_off, *nlocal, *localres;
    const int *crank_off, *ncrank, *crankres;
    float w_cum[4], w1_cum[3];
    float rigid_rotate_p;
    int non_crowders, nc_mode, sample_freq, sample_after;
    float bound_threshold;
    int rep_crowd; /* REPULSIVE_CROWDING: pairs with a crowder molecule take the crowder term */
} OracleSystem;

typedef struct {
    int accept, acceptA, reject, totalAcceptReject, totalAccept;
    int boundSamples, samplesSinceLastExchange, totalBoundSamples, totalSamples;
    float acceptanceRatio, accumulativeAcceptanceRatio, fractionBound, accumulativeFractionBound;
    int pad[3];
} OracleStats;

/* Replica states, R slots. */
typedef struct {
    int R;
    float *pos, *rel, *center; /* R*N*3, R*N*3, R*M*3 */
    double *potential;
    float *temperature;
    const float *tstep;
    const double *rstep;
    int *tindex, *label, *slot_of_t;
    OracleStats *stats;
    unsigned long long *stepc;
    uint32_t seed_lo, seed_hi;
    int sim_index;
    int rep_off; /* global index of slot 0 (the engine's replica numbering) */
    int mode;
} OracleReplicas;

/* ------------------------------------------------------------ quaternion */

typedef struct {
    double w, x, y, z;
} Quat;

static Quat quat_axis_angle(double angle, double ax, double ay, double az)
{
    double s = sin(angle / 2.0), c = cos(angle / 2.0);
    Quat q = {c, s * ax, s * ay, s * az};
    return q;
}

static void quat_normalize(Quat *q)
{
    double m = sqrt(q->w * q->w + q->x * q->x + q->y * q->y + q->z * q->z);
    q->w /= m, q->x /= m, q->y /= m, q->z /= m;
}

/* Quaternion::rotateVector: double arithmetic on a float vector, float result. */
static void quat_rotate(const Quat *q, const float *v, float *o)
{
    double w2 = q->w * q->w, x2 = q->x * q->x, y2 = q->y * q->y, z2 = q->z * q->z;
    double wx = q->w * q->x, wy = q->w * q->y, wz = q->w * q->z, xy = q->x * q->y, xz = q->x * q->z,
           yz = q->y * q->z;
    double vx = v[0], vy = v[1], vz = v[2];
    o[0] = (float)(vx * (w2 + x2 - y2 - z2) + (vy * (xy - wz) + vz * (wy + xz)) * 2.0);
    o[1] = (float)((vx * (wz + xy) + vz * (yz - wx)) * 2.0 + vy * (w2 - x2 + y2 - z2));
    o[2] = (float)((vx * (xz - wy) + vy * (yz + wx)) * 2.0 + vz * (w2 - x2 - y2 + z2));
}

/* ------------------------------------------------------------ draws */

static double u01(uint32_t x) { return (double)x * 2.3283064365386963e-10; }

static int pick(double u, int n)
{
    int k = (int)(u * (double)n);
    return k < n ? k : n - 1;
}

static int discrete(double u, const float *cum, int n)
{
    for (int k = 0; k < n - 1; ++k)
        if (u < (double)cum[k])
            return k;
    return n - 1;
}

/* ------------------------------------------------------------ energy */

/* E() + internal_molecule_E(true), total() in kcal/mol; also the non-crowder
 * inter-molecule energy (E(a,b) summed over non-crowder pairs). */
static double replica_energy(const OracleSystem *S, int mode, const float *pos, double *nc_out)
{
    double LJ = 0.0, DH = 0.0, B = 0.0, A = 1.0, T = 0.0, nc = 0.0;
    for (int a = 0; a < S->M; ++a)
        for (int b = a + 1; b < S->M; ++b) {
            double lj = 0.0, dh = 0.0;
            /* REPULSIVE_CROWDING (src/Replica.cpp:434-472): crowder pairs, repulsive only */
            const int crowd = S->rep_crowd && ((S->mflags[a] | S->mflags[b]) & 2);
            for (int i = S->mstart[a]; i < S->mstart[a] + S->mcount[a]; ++i)
                for (int j = S->mstart[b]; j < S->mstart[b] + S->mcount[b]; ++j) {
                    double r = or_dist(mode, pos + 3 * i, pos + 3 * j, S->box) + (double)OR_EPS;
                    if (crowd) {
                        lj += or_crowder_term(mode, r);
                        continue;
                    }
                    lj += or_lj_term(mode, r, S->table[S->aa[i] * S->ntypes + S->aa[j]], S->sig[i], S->sig[j]);
                    dh += or_dh_term(mode, r, S->q[i], S->q[j]);
                }
            LJ += lj;
            DH += dh;
            if (a < S->non_crowders && b < S->non_crowders)
                nc += lj * OR_RT_TO_KCAL + dh * OR_DHC;
        }
    int flexible = 0;
    for (int m = 0; m < S->M; ++m) {
        if (!(S->mflags[m] & 1))
            continue;
        flexible = 1;
        double out[5];
        const int s0 = S->mstart[m];
        oracle_E_intra(mode, S->mcount[m], pos + 3 * s0, S->aa + s0, S->q + s0, S->sig + s0, S->excl + 4 * s0,
                       S->nind[m], S->ind + 2 * S->ind_off[m], S->nbond[m], S->bonds + 2 * S->bond_off[m],
                       S->nang[m], S->angles + 3 * S->ang_off[m], S->ntor[m], S->tors + 4 * S->tor_off[m],
                       S->torsV, S->torsS, S->tors_types, S->table, S->ntypes, S->box, 1, out);
        LJ += out[0];
        DH += out[1];
        B += out[2];
        A *= out[3];
        T += out[4];
    }
    if (nc_out)
        *nc_out = nc;
    double raw[5] = {LJ, DH, B, A, T};
    return oracle_total(raw, flexible);
}

double oracle_replica_energy(const OracleSystem *S, int mode, const float *pos, double *nc_out)
{
    return replica_energy(S, mode, pos, nc_out);
}

/* ------------------------------------------------------------ moves */

static void normalize_f(double dx, double dy, double dz, float *v)
{
    float x = (float)dx, y = (float)dy, z = (float)dz;
    float m = sqrtf(x * x + y * y + z * z);
    if (m != 0.0f)
        x /= m, y /= m, z /= m;
    v[0] = x, v[1] = y, v[2] = z;
}

/* Molecule::wrap_if_necessary after a change of centre. */
static void wrap_and_place(float *c, float box, float *pos, const float *rel, int n)
{
    float w[3] = {fmodf(c[0], box), fmodf(c[1], box), fmodf(c[2], box)};
    if (w[0] != c[0] || w[1] != c[1] || w[2] != c[2]) {
        c[0] = w[0], c[1] = w[1], c[2] = w[2];
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                pos[3 * i + k] = rel[3 * i + k] + c[k];
    }
}

/* Molecule::translate(v, ri) (src/Molecule.cpp:274-301). */
static void local_translate(float *pos, float *rel, float *c, int n, int ri, const float *v, float box)
{
    float vf[3] = {v[0] / (float)n, v[1] / (float)n, v[2] / (float)n};
    for (int k = 0; k < 3; ++k) {
        pos[3 * ri + k] += v[k];
        rel[3 * ri + k] += v[k];
        c[k] = c[k] + vf[k];
    }
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k)
            rel[3 * i + k] -= vf[k];
    wrap_and_place(c, box, pos, rel, n);
}

/* One make_MC_move on molecule m (positions pos/rel of that molecule, centre c). */
static void make_move(const OracleSystem *S, int m, const uint32_t *w, float tstep, double rstep, float *pos,
                      float *rel, float *c)
{
    const int n = S->mcount[m];
    const int flexible = S->mflags[m] & 1;
    const double u1 = u01(w[1]);
    int type;
    if (flexible)
        type = (S->M > 1) ? discrete(u1, S->w_cum, 4) : 1 + discrete(u1, S->w1_cum, 3);
    else
        type = (u1 < (double)S->rigid_rotate_p) ? 1 : 0;
    const double dx = u01(w[2]) - 0.5, dy = 0.5 - u01(w[3]), dz = u01(w[4]) - 0.5;
    if (type == 0) { /* translate */
        float v[3];
        normalize_f(dx, dy, dz, v);
        for (int k = 0; k < 3; ++k) {
            v[k] = v[k] * tstep;
            c[k] = fmodf(c[k] + v[k], S->box);
        }
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                pos[3 * i + k] = rel[3 * i + k] + c[k];
    } else if (type == 1) { /* rotate about the centre */
        double mag = sqrt(dx * dx + dy * dy + dz * dz);
        Quat q = quat_axis_angle(rstep, dx / mag, dy / mag, dz / mag);
        quat_normalize(&q);
        for (int i = 0; i < n; ++i) {
            float o[3];
            quat_rotate(&q, rel + 3 * i, o);
            for (int k = 0; k < 3; ++k) {
                rel[3 * i + k] = o[k];
                pos[3 * i + k] = c[k] + o[k];
            }
        }
    } else if (type == 2) { /* flex a branch */
        if (S->nflex[m] == 0)
            return;
        double mag = sqrt(dx * dx + dy * dy + dz * dz);
        Quat q = quat_axis_angle(rstep, dx / mag, dy / mag, dz / mag);
        const int *fr = S->flexres + 3 * (S->flex_off[m] + pick(u01(w[5]), S->nflex[m]));
        const int *op = S->flexopt + 3 * (fr[2] + pick(u01(w[6]), fr[1]));
        const int ri = fr[0];
        const float pr[3] = {pos[3 * ri], pos[3 * ri + 1], pos[3 * ri + 2]};
        float acc[3] = {0, 0, 0};
        float *d = (float *)calloc((size_t)3 * n, sizeof(float));
        for (int k = 0; k < op[2]; ++k) {
            const int i = S->branch[op[1] + k];
            float rp[3] = {pos[3 * i] - pr[0], pos[3 * i + 1] - pr[1], pos[3 * i + 2] - pr[2]}, o[3];
            quat_rotate(&q, rp, o);
            for (int kk = 0; kk < 3; ++kk) {
                d[3 * i + kk] = (o[kk] + pr[kk]) - pos[3 * i + kk];
                acc[kk] += d[3 * i + kk];
            }
        }
        float vf[3] = {acc[0] / (float)n, acc[1] / (float)n, acc[2] / (float)n};
        for (int k = 0; k < op[2]; ++k) {
            const int i = S->branch[op[1] + k];
            for (int kk = 0; kk < 3; ++kk) {
                pos[3 * i + kk] += d[3 * i + kk];
                rel[3 * i + kk] += d[3 * i + kk];
            }
        }
        for (int kk = 0; kk < 3; ++kk)
            c[kk] = c[kk] + vf[kk];
        for (int i = 0; i < n; ++i)
            for (int kk = 0; kk < 3; ++kk)
                rel[3 * i + kk] -= vf[kk];
        wrap_and_place(c, S->box, pos, rel, n);
        free(d);
    } else { /* local move */
        const int crank = u01(w[5]) < 0.5;
        float v[3];
        int ri;
        if (!crank) {
            if (S->nlocal[m] == 0)
                return;
            ri = S->localres[S->local_off[m] + pick(u01(w[6]), S->nlocal[m])];
            float nv[3];
            normalize_f(dx, dy, dz, nv);
            const double s = (double)0.1f * (double)tstep;
            for (int k = 0; k < 3; ++k)
                v[k] = (float)(nv[k] * s);
        } else {
            if (S->ncrank[m] == 0)
                return;
            ri = S->crankres[S->crank_off[m] + pick(u01(w[6]), S->ncrank[m])];
            if (ri < 1 || ri + 1 >= n)
                return;
            const int flip = u01(w[7]) < 0.5;
            double ax = (double)(pos[3 * (ri + 1)] - pos[3 * (ri - 1)]);
            double ay = (double)(pos[3 * (ri + 1) + 1] - pos[3 * (ri - 1) + 1]);
            double az = (double)(pos[3 * (ri + 1) + 2] - pos[3 * (ri - 1) + 2]);
            double am = sqrt(ax * ax + ay * ay + az * az);
            Quat q = quat_axis_angle(flip ? -rstep : rstep, ax / am, ay / am, az / am);
            quat_normalize(&q);
            float rp[3] = {pos[3 * ri] - pos[3 * (ri - 1)], pos[3 * ri + 1] - pos[3 * (ri - 1) + 1],
                           pos[3 * ri + 2] - pos[3 * (ri - 1) + 2]},
                  o[3];
            quat_rotate(&q, rp, o);
            for (int k = 0; k < 3; ++k)
                v[k] = (o[k] + pos[3 * (ri - 1) + k]) - pos[3 * ri + k];
        }
        local_translate(pos, rel, c, n, ri, v, S->box);
    }
}

/* ------------------------------------------------------------ MC steps */

static void mc_steps(const OracleSystem *S, OracleReplicas *X, int slot, int nsteps)
{
    const int N = S->N, M = S->M;
    float *pos = X->pos + (size_t)slot * N * 3, *rel = X->rel + (size_t)slot * N * 3;
    float *cen = X->center + (size_t)slot * M * 3;
    float *bpos = (float *)malloc(sizeof(float) * 3 * N), *brel = (float *)malloc(sizeof(float) * 3 * N);
    const uint32_t key[2] = {X->seed_lo ^ (0x9E3779B9u * (uint32_t)(X->rep_off + slot + 1)), X->seed_hi};
    OracleStats *st = X->stats + slot;
    for (int s = 0; s < nsteps; ++s) {
        const unsigned long long mcstep = X->stepc[slot] + (unsigned long long)s;
        uint32_t w[12];
        for (int b = 0; b < 3; ++b) {
            uint32_t ctr[4] = {(uint32_t)mcstep, (uint32_t)(mcstep >> 32), (uint32_t)b, 0x4D43u};
            oracle_philox4x32_10(ctr, key, w + 4 * b);
        }
        const int m = pick(u01(w[0]), M);
        const int s0 = S->mstart[m], n = S->mcount[m];
        float bc[3] = {cen[3 * m], cen[3 * m + 1], cen[3 * m + 2]};
        memcpy(bpos, pos + 3 * s0, sizeof(float) * 3 * n);
        memcpy(brel, rel + 3 * s0, sizeof(float) * 3 * n);
        make_move(S, m, w, X->tstep[slot], X->rstep[slot], pos + 3 * s0, rel + 3 * s0, cen + 3 * m);
        double nc = 0.0;
        const double newE = replica_energy(S, X->mode, pos, &nc);
        const float delta = (float)(newE - X->potential[slot]);
        int acc;
        if (delta < 0.0f) {
            acc = 1;
        } else {
            const float boltz = expf(-(delta * OR_KCAL) / (OR_RGAS * X->temperature[slot]));
            acc = u01(w[8]) < (double)boltz ? 2 : 0;
        }
        if (acc) {
            X->potential[slot] = newE;
            if (acc == 1)
                st->accept++;
            else
                st->acceptA++;
        } else {
            st->reject++;
            memcpy(pos + 3 * s0, bpos, sizeof(float) * 3 * n);
            memcpy(rel + 3 * s0, brel, sizeof(float) * 3 * n);
            cen[3 * m] = bc[0], cen[3 * m + 1] = bc[1], cen[3 * m + 2] = bc[2];
        }
        if (S->sample_freq > 0 && (long long)(mcstep % (unsigned long long)S->sample_freq) == S->sample_freq - 1 &&
            (long long)mcstep >= (long long)S->sample_after) {
            double e = 0.0;
            if (S->nc_mode == 1)
                replica_energy(S, X->mode, pos, &e);
            else if (S->nc_mode == 2)
                e = X->potential[slot];
            st->samplesSinceLastExchange++;
            if ((float)e < S->bound_threshold)
                st->boundSamples++;
        }
    }
    X->stepc[slot] += (unsigned long long)nsteps;
    free(bpos);
    free(brel);
}

typedef struct {
    const OracleSystem *S;
    OracleReplicas *X;
    int first, last, nsteps;
} Work;

static void *worker(void *p)
{
    Work *w = (Work *)p;
    for (int r = w->first; r < w->last; ++r)
        mc_steps(w->S, w->X, r, w->nsteps);
    return NULL;
}

static void report_slot(OracleStats *s, float *out4)
{
    s->totalBoundSamples += s->boundSamples;
    s->totalSamples += s->samplesSinceLastExchange;
    s->fractionBound = (float)s->boundSamples / fmaxf(1.0f, (float)s->samplesSinceLastExchange);
    s->accumulativeFractionBound = (float)s->totalBoundSamples / fmaxf(1.0f, (float)s->totalSamples);
    s->boundSamples = 0;
    s->samplesSinceLastExchange = 0;
    s->totalAccept += s->acceptA + s->accept;
    s->totalAcceptReject += s->acceptA + s->accept + s->reject;
    s->acceptanceRatio = (float)(s->acceptA + s->accept) / (float)(s->acceptA + s->accept + s->reject);
    s->accumulativeAcceptanceRatio = (float)s->totalAccept / (float)s->totalAcceptReject;
    s->acceptA = s->accept = s->reject = 0;
    if (out4) {
        out4[0] = s->fractionBound;
        out4[1] = s->accumulativeFractionBound;
        out4[2] = s->acceptanceRatio;
        out4[3] = s->accumulativeAcceptanceRatio;
    }
}

/* Even/odd exchange sweep number x (Simulation::run, src/Simulation.cpp:770-795). */
static void exchange(OracleReplicas *X, int x, int *offset, int *exch_out, int *tests_out)
{
    int exchanges = 0, tests = 0;
    const uint32_t key[2] = {X->seed_lo ^ 0xB5297A4Du, X->seed_hi ^ (0x68E31DA4u * (uint32_t)(X->sim_index + 1))};
    for (int ti = *offset; ti < X->R - 1; ti += 2) {
        const int i = X->slot_of_t[ti], j = X->slot_of_t[ti + 1];
        const double Ti = X->temperature[i], Tj = X->temperature[j];
        const double delta = (1.0 / Ti - 1.0 / Tj) * (X->potential[i] - X->potential[j]) * (double)(OR_KCAL / OR_RGAS);
        uint32_t ctr[4] = {(uint32_t)x, 0u, (uint32_t)ti, 0x5245u}, o[4];
        oracle_philox4x32_10(ctr, key, o);
        double p = exp(delta);
        if (p > 1.0)
            p = 1.0;
        if (u01(o[0]) < p) {
            float tf = X->temperature[i];
            X->temperature[i] = X->temperature[j];
            X->temperature[j] = tf;
            int ti_ = X->tindex[i];
            X->tindex[i] = X->tindex[j];
            X->tindex[j] = ti_;
            int lb = X->label[i];
            X->label[i] = X->label[j];
            X->label[j] = lb;
            OracleStats sv = X->stats[i];
            X->stats[i] = X->stats[j];
            X->stats[j] = sv;
            X->slot_of_t[X->tindex[i]] = i;
            X->slot_of_t[X->tindex[j]] = j;
            ++exchanges;
        }
        ++tests;
    }
    *offset = 1 - *offset;
    *exch_out = exchanges;
    *tests_out = tests;
}

/* Blocks of MC steps with exchanges in between, mirroring cgppd_engine_run.
 * reports: [n_blocks+1][R][4] rows (written when sampling has started); exch: [n_blocks][2].
 * *x_io is the number of exchanges done so far (in/out), *offset_io the sweep parity. */
int oracle_remc_run(const OracleSystem *S, OracleReplicas *X, int n_blocks, int steps_per_block,
                    int exchange_after_last, int nthreads, int *x_io, int *offset_io, float *reports, int *exch)
{
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > X->R)
        nthreads = X->R;
    for (int b = 0; b < n_blocks; ++b) {
        pthread_t th[256];
        Work wk[256];
        int nt = nthreads > 256 ? 256 : nthreads;
        int per = (X->R + nt - 1) / nt;
        int used = 0;
        for (int k = 0; k < nt; ++k) {
            wk[k].S = S;
            wk[k].X = X;
            wk[k].first = k * per;
            wk[k].last = (k + 1) * per < X->R ? (k + 1) * per : X->R;
            wk[k].nsteps = steps_per_block;
            if (wk[k].first >= wk[k].last)
                break;
            if (nt == 1)
                worker(&wk[k]);
            else
                pthread_create(&th[k], NULL, worker, &wk[k]);
            ++used;
        }
        if (nt > 1)
            for (int k = 0; k < used; ++k)
                pthread_join(th[k], NULL);
        const int last = (b + 1 == n_blocks);
        if (!last || exchange_after_last) {
            const int x = *x_io;
            if ((long long)steps_per_block * x >= (long long)S->sample_after && reports)
                for (int t = 0; t < X->R; ++t)
                    report_slot(X->stats + X->slot_of_t[t], reports + ((size_t)b * X->R + t) * 4);
            int e = 0, tt = 0;
            exchange(X, x, offset_io, &e, &tt);
            if (exch) {
                exch[2 * b] = e;
                exch[2 * b + 1] = tt;
            }
            *x_io = x + 1;
        }
    }
    return 0;
}

void oracle_final_report(OracleReplicas *X, float *out)
{
    for (int t = 0; t < X->R; ++t)
        report_slot(X->stats + X->slot_of_t[t], out ? out + (size_t)t * 4 : NULL);
}
