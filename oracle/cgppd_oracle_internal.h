/* Shared helpers of the oracle translation units (test infrastructure only). */
#ifndef CGPPD_ORACLE_INTERNAL_H_
#define CGPPD_ORACLE_INTERNAL_H_

#include <stdint.h>

double or_dist(int mode, const float *a, const float *b, float L);
double or_lj_term(int mode, double r, float eps_raw, float si, float sj);
double or_dh_term(int mode, double r, float qi, float qj);
double or_crowder_term(int mode, double r);
double or_angle_ref(const float *a, const float *b);
double or_angle_fp64(const float *pa, const float *pb, const float *pc);
double or_angle_term(double theta);
double or_torsion_phi(int mode, const float *pi, const float *pj, const float *pk, const float *pl);
void oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]);
double oracle_total(const double *raw5, int flexible);
void oracle_E_intra(int mode, int n, const float *xyz, const int *aa, const float *q, const float *sig,
                    const int *excl_ids, int n_ind, const int *indirect, int n_bonds, const int *bonds,
                    int n_angles, const int *angles, int n_tors, const int *tors, const double *torsV,
                    const double *torsS, int ntypes_t, const float *table, int ntypes, float box,
                    int include_lj_dh, double *out);

#endif
