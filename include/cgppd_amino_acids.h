/*
 * cgppd_amino_acids.h -- C helpers around the AminoAcids parameter object that the
 * drop-in ABI takes by pointer (src/cudaExterns.h:20-21).
 *
 * The object has the reference's memory layout (src/AminoAcids.h:7-27): 20 AminoAcid
 * records of 48 bytes, then float LJpotentials[20][20] at byte offset 960.  These
 * helpers let non-C++ hosts create and fill one; C++ hosts may use their own
 * reference-layout AminoAcids directly.
 */
#ifndef CGPPD_AMINO_ACIDS_H_
#define CGPPD_AMINO_ACIDS_H_

#include <stddef.h>

#ifdef __cplusplus
class AminoAcids;
extern "C" {
#else
typedef struct AminoAcids AminoAcids;
#endif

/* New / delete an AminoAcids object (reference constructor: src/AminoAcids.cpp:10-13). */
AminoAcids *cgppd_aminoacids_create(void);
void cgppd_aminoacids_destroy(AminoAcids *a);

/* Replaces AminoAcids::init (src/AminoAcids.cpp:19-22): load the residue-type file and
 * the contact table in the reference's text formats.  Returns 0 on success. */
int cgppd_aminoacids_load(AminoAcids *a, const char *aa_path, const char *lj_path);

/* Fill record i / the raw 20x20 table directly (synthetic parameter sets). */
void cgppd_aminoacids_set(AminoAcids *a, int i, const char *name, const char *sname, char symbol, float radius,
                          float charge);
void cgppd_aminoacids_set_table(AminoAcids *a, const float *table400);
void cgppd_aminoacids_get_table(const AminoAcids *a, float *table400);

/* Replaces AminoAcids::getAminoAcidIndex (src/AminoAcids.cpp:145-181); -1 if unknown. */
int cgppd_aminoacids_index(const AminoAcids *a, const char *name);

/* Layout probes: offset of LJpotentials and sizeof(AminoAcids). */
size_t cgppd_aminoacids_lj_offset(void);
size_t cgppd_aminoacids_sizeof(void);

#ifdef __cplusplus
}
#endif

#endif /* CGPPD_AMINO_ACIDS_H_ */
