/*
 * cgppd_oracle.c -- CPU oracle for the CGPPD hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls this
 * file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do,
 * and only as the checker (or as the timed CPU baseline).
 *
 * It restates, in plain C, the arithmetic of the reference CPU path:
 *   - Residue::distance            src/Residue.cpp:62-81   (float min-image, sqrtf)
 *   - calculate_LJ / calculate_DH  src/Potential.cpp:5-42
 *   - calculate_bond/angle/torsion src/Potential.cpp:45-98
 *   - Potential totals             src/Potential.cpp:187-221
 *   - Replica::E()                 src/Replica.cpp:421-500  (inter-molecule pairs)
 *   - Replica::E(a,b)              src/Replica.cpp:502-528
 *   - Molecule::E(bool)            src/Molecule.cpp:636-699 (flexible intra + bonded)
 *   - crowderPairPotential and the REPULSIVE_CROWDING branches of Replica::E()
 *                                  src/Replica.cpp:416-472 (off in the reference's
 *                                  default build; selected per call here)
 * and, on the packed float4 layout, the pair rules of the reference GPU kernels
 *   - E_TiledKernel   src/CudaFunctions.cu:346-607 (flexible-linker build)
 *   - E_TiledKernelNC src/CudaFunctions.cu:757-961
 *   - the REPULSIVE_CROWDING branch of E_TiledKernel, src/CudaFunctions.cu:492-498
 *
 * Every energy function takes `mode`:
 *   ORACLE_REF  (0): the reference's own mixed precision -- float coordinates and
 *                    float min-image distance, double pow, float expf; this is the
 *                    mode pinned against the reference's golden vectors.
 *   ORACLE_FP64 (1): the FP64 oracle -- the same formulas with the distance, the
 *                    exponentials and every product in double from the same float
 *                    inputs; the 1e-5 relative bound of the GPU path is taken
 *                    against this mode.
 *
 * Units: functions return the reference's raw accumulators (LJ in RT units, DH as
 * the unscaled q_i q_j e^{-r/xi}/r sum, bond as sum (r-R0)^2, angle as the product
 * of the angle terms, torsion in kcal/mol) so that they compare directly with
 * Potential::almost_equal (src/Potential.cpp:223-230); oracle_total() applies the
 * unit factors of Potential::total().
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cgppd_oracle_internal.h"

#define ORACLE_REF 0
#define ORACLE_FP64 1

/* Physical constants exactly as the reference evaluates them.  In
 * src/constants.h:8-26 every factor is a float literal, so the compiled values are
 * the float results below (printed with %.17g from a g++ build of that header). */
#define OR_RT_TO_KCAL 0.59218674898147583 /* (T_room*Rgas/kcal) in float */
#define OR_DHC 4.1507959365844727         /* DH_CONVERSION_FACTOR in float */
#define OR_R0C 1.1224620342254639         /* pow(2.0f, 1.0f/6.0f) in float */
#define OR_LAMBDA 0.159f                  /* LJ_lambda */
#define OR_E0 (-2.27f)                    /* e0, RT units */
#define OR_XI 10.0f                       /* Debye length, A */
#define OR_EPS 1e-38f                     /* EPS, src/definitions.h:10 */
#define OR_K_SPRING 378.0                 /* src/constants.h:35 */
#define OR_R0 3.81f                       /* src/constants.h:36 */
#define OR_GAMMA 0.1f                     /* src/constants.h:40-46 */
#define OR_GAMMA_RECIP 10.0f
#define OR_EPS_ALPHA 4.3f
#define OR_THETA_ALPHA 1.6f
#define OR_THETA_BETA 2.27f
#define OR_K_ALPHA 106.4f
#define OR_K_BETA 26.3f
#define OR_PADDER (-2.0f)
#define OR_CROWDER (-1.0f)

double oracle_rt_to_kcal(void) { return OR_RT_TO_KCAL; }
double oracle_dh_factor(void) { return OR_DHC; }

/* ---------------------------------------------------------------- distance */

/* Residue::distance (src/Residue.cpp:62-76): float differences, min image with
 * round() (half away from zero), sqrtf.  The reference returns it as double. */
static double dist_ref(const float *a, const float *b, float L)
{
    float X = a[0] - b[0], Y = a[1] - b[1], Z = a[2] - b[2];
    if (L != 0.0f) {
        X = X - L * roundf(X / L);
        Y = Y - L * roundf(Y / L);
        Z = Z - L * roundf(Z / L);
    }
    return (double)sqrtf(X * X + Y * Y + Z * Z);
}

static double dist_fp64(const float *a, const float *b, float L)
{
    double X = (double)a[0] - b[0], Y = (double)a[1] - b[1], Z = (double)a[2] - b[2];
    if (L != 0.0f) {
        X -= (double)L * round(X / L);
        Y -= (double)L * round(Y / L);
        Z -= (double)L * round(Z / L);
    }
    return sqrt(X * X + Y * Y + Z * Z);
}

double or_dist(int mode, const float *a, const float *b, float L)
{
    return mode == ORACLE_REF ? dist_ref(a, b, L) : dist_fp64(a, b, L);
}

/* ---------------------------------------------------------------- pair terms */

/* calculate_LJ (src/Potential.cpp:5-35).  eps_raw is the table value
 * LJpotentials[a][b] (float, RT units, before the lambda/e0 transform). */
double or_lj_term(int mode, double r, float eps_raw, float si, float sj)
{
    if (mode == ORACLE_REF) {
        double Eij = (double)(OR_LAMBDA * (eps_raw - OR_E0));
        double sigmaij = (double)(0.5f * (si + sj));
        double t = pow(sigmaij / r, 6.0);
        double LJ = -4.0 * Eij * t * (t - 1.0);
        if (Eij > 0.0 && r < sigmaij * OR_R0C)
            LJ = -LJ + 2.0 * Eij;
        return LJ;
    } else {
        double Eij = (double)OR_LAMBDA * ((double)eps_raw - (double)OR_E0);
        double sigmaij = 0.5 * ((double)si + (double)sj);
        double t = pow(sigmaij / r, 6.0);
        double LJ = -4.0 * Eij * t * (t - 1.0);
        if (Eij > 0.0 && r < sigmaij * pow(2.0, 1.0 / 6.0))
            LJ = -LJ + 2.0 * Eij;
        return LJ;
    }
}

/* calculate_DH (src/Potential.cpp:37-42): q_i q_j expf(-r/xi) / r. */
double or_dh_term(int mode, double r, float qi, float qj)
{
    if (mode == ORACLE_REF)
        return (double)(qi * qj * expf((float)(-r / OR_XI))) / r;
    return (double)qi * (double)qj * exp(-r / (double)OR_XI) / r;
}

/* Repulsive crowder pair of the reference's REPULSIVE_CROWDING build (off in its
 * default build, src/definitions.h:18): crowderPairPotential (src/Replica.cpp:416-419)
 * = powf(6.0f / r, 12.0f) in RT units, applied when r < const_repulsive_cutoff (15 A,
 * src/definitions.h:38; src/Replica.cpp:443-447 and :464-468), with no Debye-Hueckel
 * term for the pair.  r includes the +EPS of the callers. */
double or_crowder_term(int mode, double r)
{
    if (!(r < 15.0))
        return 0.0;
    if (mode == ORACLE_REF)
        return (double)powf(6.0f / (float)r, 12.0f);
    return pow(6.0 / r, 12.0);
}

/* One residue pair, both terms, in raw units.  r includes the +EPS of the callers. */
void oracle_pair(int mode, const float *pi, const float *pj, float eps_raw, float qi,
                 float qj, float si, float sj, float box, double *lj, double *dh)
{
    double r = or_dist(mode, pi, pj, box) + (double)OR_EPS;
    *lj = or_lj_term(mode, r, eps_raw, si, sj);
    *dh = or_dh_term(mode, r, qi, qj);
}

/* ---------------------------------------------------------------- sums */

/* Replica::E() (src/Replica.cpp:421-500), REPULSIVE_CROWDING off: every residue
 * pair of every molecule pair mI < mJ.  Residues are stored contiguously per
 * molecule: molecule m owns [mstart[m], mstart[m]+mcount[m]).  xyz is n*3 floats,
 * aa the type index into `table` (ntypes x ntypes raw contact values). */
void oracle_E_inter(int mode, int nmol, const int *mstart, const int *mcount,
                    const float *xyz, const int *aa, const float *q, const float *sig,
                    const float *table, int ntypes, float box, double *out_lj, double *out_dh)
{
    double LJ = 0.0, DH = 0.0;
    for (int mI = 0; mI < nmol; mI++)
        for (int mJ = mI + 1; mJ < nmol; mJ++)
            for (int a = mstart[mI]; a < mstart[mI] + mcount[mI]; a++)
                for (int b = mstart[mJ]; b < mstart[mJ] + mcount[mJ]; b++) {
                    double r = or_dist(mode, xyz + 3 * a, xyz + 3 * b, box) + (double)OR_EPS;
                    LJ += or_lj_term(mode, r, table[aa[a] * ntypes + aa[b]], sig[a], sig[b]);
                    DH += or_dh_term(mode, r, q[a], q[b]);
                }
    *out_lj = LJ;
    *out_dh = DH;
}

/* Per molecule-pair energies in kcal/mol: out[mI*nmol+mJ] (symmetric, zero
 * diagonal) -- the decomposition the GPU engine keeps per replica. */
void oracle_E_inter_matrix(int mode, int nmol, const int *mstart, const int *mcount,
                           const float *xyz, const int *aa, const float *q, const float *sig,
                           const float *table, int ntypes, float box, double *out)
{
    memset(out, 0, sizeof(double) * nmol * nmol);
    for (int mI = 0; mI < nmol; mI++)
        for (int mJ = mI + 1; mJ < nmol; mJ++) {
            double LJ = 0.0, DH = 0.0;
            for (int a = mstart[mI]; a < mstart[mI] + mcount[mI]; a++)
                for (int b = mstart[mJ]; b < mstart[mJ] + mcount[mJ]; b++) {
                    double r = or_dist(mode, xyz + 3 * a, xyz + 3 * b, box) + (double)OR_EPS;
                    LJ += or_lj_term(mode, r, table[aa[a] * ntypes + aa[b]], sig[a], sig[b]);
                    DH += or_dh_term(mode, r, q[a], q[b]);
                }
            double e = LJ * OR_RT_TO_KCAL + DH * OR_DHC;
            out[mI * nmol + mJ] = e;
            out[mJ * nmol + mI] = e;
        }
}

/* The same matrix under repulsive crowding: crowder[m] != 0 marks crowder molecules,
 * whose pairs (with any molecule) take or_crowder_term and no Debye-Hueckel term
 * (src/Replica.cpp:434-472). */
void oracle_E_inter_matrix_rc(int mode, int nmol, const int *mstart, const int *mcount, const int *crowder,
                              const float *xyz, const int *aa, const float *q, const float *sig,
                              const float *table, int ntypes, float box, double *out)
{
    memset(out, 0, sizeof(double) * nmol * nmol);
    for (int mI = 0; mI < nmol; mI++)
        for (int mJ = mI + 1; mJ < nmol; mJ++) {
            const int crowd = crowder[mI] || crowder[mJ];
            double LJ = 0.0, DH = 0.0;
            for (int a = mstart[mI]; a < mstart[mI] + mcount[mI]; a++)
                for (int b = mstart[mJ]; b < mstart[mJ] + mcount[mJ]; b++) {
                    double r = or_dist(mode, xyz + 3 * a, xyz + 3 * b, box) + (double)OR_EPS;
                    if (crowd) {
                        LJ += or_crowder_term(mode, r);
                    } else {
                        LJ += or_lj_term(mode, r, table[aa[a] * ntypes + aa[b]], sig[a], sig[b]);
                        DH += or_dh_term(mode, r, q[a], q[b]);
                    }
                }
            double e = LJ * OR_RT_TO_KCAL + DH * OR_DHC;
            out[mI * nmol + mJ] = e;
            out[mJ * nmol + mI] = e;
        }
}

/* Vector3f::angle (src/vector3f.cpp:137-143) as the reference computes it: float
 * magnitudes and dot product, double acos, float result. */
double or_angle_ref(const float *a, const float *b)
{
    float ma = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    float mb = sqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    double cmag = (double)(mb * ma);
    if (cmag < 1e-26)
        return 0.0;
    float dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    return (double)(float)acos(dot / cmag);
}

double or_angle_fp64(const float *pa, const float *pb, const float *pc)
{
    double a[3], b[3];
    for (int k = 0; k < 3; k++) {
        a[k] = (double)pa[k] - pb[k];
        b[k] = (double)pc[k] - pb[k];
    }
    double cmag = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) * sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    if (cmag < 1e-26)
        return 0.0;
    double c = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) / cmag;
    if (c > 1.0) c = 1.0;
    if (c < -1.0) c = -1.0;
    return acos(c);
}

/* calculate_angle (src/Potential.cpp:57-71): the term whose product is stored. */
double or_angle_term(double theta)
{
    double da = theta - (double)OR_THETA_ALPHA, db = theta - (double)OR_THETA_BETA;
    return exp(-(double)OR_GAMMA * ((double)OR_K_ALPHA * da * da + (double)OR_EPS_ALPHA)) +
           exp(-(double)OR_GAMMA * ((double)OR_K_BETA * db * db));
}

static void sub3f(const float *a, const float *b, float *o)
{
    o[0] = a[0] - b[0];
    o[1] = a[1] - b[1];
    o[2] = a[2] - b[2];
}

static void cross3f(const float *a, const float *b, float *o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* The dihedral of calculate_torsion (src/Potential.cpp:73-98). */
double or_torsion_phi(int mode, const float *pi, const float *pj, const float *pk, const float *pl)
{
    if (mode == ORACLE_REF) {
        float b1[3], b2[3], b3[3], c23[3], c12[3];
        sub3f(pj, pi, b1);
        sub3f(pk, pj, b2);
        sub3f(pl, pk, b3);
        cross3f(b2, b3, c23);
        cross3f(b1, b2, c12);
        float mb2 = sqrtf(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
        float y = mb2 * (b1[0] * c23[0] + b1[1] * c23[1] + b1[2] * c23[2]);
        float x = c12[0] * c23[0] + c12[1] * c23[1] + c12[2] * c23[2];
        return (double)atan2f(y, x);
    } else {
        double b1[3], b2[3], b3[3], c23[3], c12[3];
        for (int k = 0; k < 3; k++) {
            b1[k] = (double)pj[k] - pi[k];
            b2[k] = (double)pk[k] - pj[k];
            b3[k] = (double)pl[k] - pk[k];
        }
        c23[0] = b2[1] * b3[2] - b2[2] * b3[1];
        c23[1] = b2[2] * b3[0] - b2[0] * b3[2];
        c23[2] = b2[0] * b3[1] - b2[1] * b3[0];
        c12[0] = b1[1] * b2[2] - b1[2] * b2[1];
        c12[1] = b1[2] * b2[0] - b1[0] * b2[2];
        c12[2] = b1[0] * b2[1] - b1[1] * b2[0];
        double mb2 = sqrt(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
        double y = mb2 * (b1[0] * c23[0] + b1[1] * c23[1] + b1[2] * c23[2]);
        double x = c12[0] * c23[0] + c12[1] * c23[1] + c12[2] * c23[2];
        return atan2(y, x);
    }
}

/* Molecule::E(include_LJ_and_DH) (src/Molecule.cpp:636-699) for ONE flexible
 * molecule of n residues (indices local to the molecule).
 *   excl_ids: n*4 ints per residue {chain_uid, res_seq, domain_uid, bond_uid}
 *   indirect: n_ind pairs (i<j) of indirect neighbours
 *   bonds (i,j), angles (i,j,k), torsions (i,j,k,l): residue index tuples
 *   torsV/torsS: [ntypes_t*ntypes_t*4] torsion amplitudes / phases (radians)
 * out[5] = {LJ raw, DH raw, bond raw, angle product, torsion kcal}. */
void oracle_E_intra(int mode, int n, const float *xyz, const int *aa, const float *q,
                    const float *sig, const int *excl_ids, int n_ind, const int *indirect,
                    int n_bonds, const int *bonds, int n_angles, const int *angles,
                    int n_tors, const int *tors, const double *torsV, const double *torsS,
                    int ntypes_t, const float *table, int ntypes, float box,
                    int include_lj_dh, double *out)
{
    double LJ = 0.0, DH = 0.0, B = 0.0, A = 1.0, T = 0.0;
    if (include_lj_dh) {
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) {
                const int *ei = excl_ids + 4 * i, *ej = excl_ids + 4 * j;
                int same_domain = ei[2] && ei[2] == ej[2];
                int chain_nb = ei[0] == ej[0] && abs(ei[1] - ej[1]) < 4;
                int bonded = ei[3] && ei[3] == ej[3];
                int ind = 0;
                for (int p = 0; p < n_ind; p++)
                    if (indirect[2 * p] == i && indirect[2 * p + 1] == j) {
                        ind = 1;
                        break;
                    }
                if (same_domain || chain_nb || bonded || ind)
                    continue;
                double r = or_dist(mode, xyz + 3 * i, xyz + 3 * j, box) + (double)OR_EPS;
                LJ += or_lj_term(mode, r, table[aa[i] * ntypes + aa[j]], sig[i], sig[j]);
                DH += or_dh_term(mode, r, q[i], q[j]);
            }
    } else {
        for (int p = 0; p < n_ind; p++) {
            int i = indirect[2 * p], j = indirect[2 * p + 1];
            double r = or_dist(mode, xyz + 3 * i, xyz + 3 * j, box) + (double)OR_EPS;
            LJ -= or_lj_term(mode, r, table[aa[i] * ntypes + aa[j]], sig[i], sig[j]);
            DH -= or_dh_term(mode, r, q[i], q[j]);
        }
    }
    for (int b = 0; b < n_bonds; b++) {
        int i = bonds[2 * b], j = bonds[2 * b + 1];
        double r = or_dist(mode, xyz + 3 * j, xyz + 3 * i, box);
        double d = r - (double)OR_R0;
        B += d * d;
    }
    for (int a = 0; a < n_angles; a++) {
        const float *pi = xyz + 3 * angles[3 * a], *pj = xyz + 3 * angles[3 * a + 1],
                    *pk = xyz + 3 * angles[3 * a + 2];
        double theta;
        if (mode == ORACLE_REF) {
            float ab[3], cb[3];
            sub3f(pi, pj, ab);
            sub3f(pk, pj, cb);
            theta = or_angle_ref(ab, cb);
        } else {
            theta = or_angle_fp64(pi, pj, pk);
        }
        A *= or_angle_term(theta);
    }
    for (int t = 0; t < n_tors; t++) {
        const int *tt = tors + 4 * t;
        double phi = or_torsion_phi(mode, xyz + 3 * tt[0], xyz + 3 * tt[1], xyz + 3 * tt[2], xyz + 3 * tt[3]);
        int r1 = aa[tt[1]], r2 = aa[tt[2]];
        const double *V = torsV + 4 * (r1 * ntypes_t + r2), *S = torsS + 4 * (r1 * ntypes_t + r2);
        double pot = 0.0;
        /* phi holds atan2f's float result in a double variable, so n * phi is a double
         * product in both modes (src/Potential.cpp:84-93) */
        for (int k = 0; k < 4; k++)
            pot += (1.0 + cos((k + 1) * phi - S[k])) * V[k];
        T += pot;
    }
    out[0] = LJ;
    out[1] = DH;
    out[2] = B;
    out[3] = A;
    out[4] = T;
}

/* Potential::total() (src/Potential.cpp:214-221) of raw components. */
double oracle_total(const double *raw5, int flexible)
{
    double t = raw5[1] * OR_DHC + raw5[0] * OR_RT_TO_KCAL;
    if (flexible)
        t += raw5[2] * 0.5 * OR_K_SPRING + log(raw5[3]) * -(double)OR_GAMMA_RECIP + raw5[4];
    return t;
}

/* ------------------------------------------------- packed GPU-kernel semantics */

static float frac_part(float w, float *ip)
{
    float i = truncf(w);
    *ip = i;
    return w - i;
}

/* Pair rules of E_TiledKernel (flexible-linker build, src/CudaFunctions.cu:424-468)
 * and E_TiledKernelNC (src/CudaFunctions.cu:823-846) on the packed arrays the
 * reference uploads (src/Replica.cpp:705-830):
 *   pos4[i]  = (x, y, z, w)  w = rigid_domain_uid + bond_fraction, or -2 padding
 *   meta4[i] = (aa, q, sigma, w)  w = molecule_id + chain_fraction, -1 crowder, 0 pad
 * Sums every unordered pair once (the kernel's upper-triangular tiles with halved
 * diagonal tiles).  table20 is the raw 20x20 contact table.  out = {LJ raw, DH raw,
 * total kcal/mol}. */
void oracle_E_packed_rc(int mode, int nc, int rc, int P, const float *pos4, const float *meta4,
                        const float *table20, float box, double *out);

void oracle_E_packed(int mode, int nc, int P, const float *pos4, const float *meta4,
                     const float *table20, float box, double *out)
{
    oracle_E_packed_rc(mode, nc, 0, P, pos4, meta4, table20, box, out);
}

/* rc != 0: the REPULSIVE_CROWDING build of E_TiledKernel (src/CudaFunctions.cu:492-498):
 * a pair that passes the exclusion rules and has a crowder residue (meta w == -1) on
 * either side adds crowderPotential (6/r)^12 in RT units below 15 A and no
 * Debye-Hueckel term. */
void oracle_E_packed_rc(int mode, int nc, int rc, int P, const float *pos4, const float *meta4,
                        const float *table20, float box, double *out)
{
    double LJ = 0.0, DH = 0.0;
    for (int y = 0; y < P; y++) {
        const float *py = pos4 + 4 * y, *my = meta4 + 4 * y;
        if (!(py[3] > OR_PADDER))
            continue;
        if (nc && my[3] == OR_CROWDER)
            continue;
        for (int x = y + 1; x < P; x++) {
            const float *px = pos4 + 4 * x, *mx = meta4 + 4 * x;
            int excluded;
            if (px[3] == OR_PADDER) {
                excluded = 1;
            } else if (nc) {
                excluded = mx[3] == OR_CROWDER || truncf(mx[3]) == truncf(my[3]);
            } else {
                float xdom, ydom, xmol, ymol;
                float xbond = frac_part(px[3], &xdom), ybond = frac_part(py[3], &ydom);
                float xchain = frac_part(mx[3], &xmol), ychain = frac_part(my[3], &ymol);
                excluded = (xdom != 0.0f && xdom == ydom) || (xbond != 0.0f && xbond == ybond) ||
                           (xchain == ychain && fabsf((float)x - (float)y) < 4.0f);
            }
            if (excluded)
                continue;
            double r = or_dist(mode, px, py, box) + (double)OR_EPS;
            if (rc && (mx[3] == OR_CROWDER || my[3] == OR_CROWDER)) {
                LJ += or_crowder_term(mode, r);
                continue;
            }
            int ax = (int)rintf(mx[0]), ay = (int)rintf(my[0]);
            LJ += or_lj_term(mode, r, table20[ay * 20 + ax], my[2], mx[2]);
            DH += or_dh_term(mode, r, my[1], mx[1]);
        }
    }
    out[0] = LJ;
    out[1] = DH;
    out[2] = LJ * OR_RT_TO_KCAL + DH * OR_DHC;
}

/* ---------------------------------------------------------------- Philox */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
 * 1, 2, 3", SC'11): the counter-based generator the GPU engine draws from. */
void oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; round++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}
