/*
 * cgppd_pdb.h -- the C-alpha records of a PDB file, for hosts that build engine
 * molecules themselves (cgppd_engine_add_molecule takes plain arrays).
 */
#ifndef CGPPD_PDB_H_
#define CGPPD_PDB_H_

#include "cgppd_amino_acids.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces the reading part of Molecule::initFromPDB (src/Molecule.cpp:506-612): ATOM
 * records whose atom name is CA, TER records counting chains, END stopping the read.
 * Returns the residue count n and, where the arrays are non-NULL and capacity >= n,
 * fills positions xyz[3n], residue types (indices into `a`), chain identifiers,
 * residue sequence numbers, chain indices (TER records before each residue) and the
 * chain count.  Returns -1, with the message in cgppd_get_last_error, when the file
 * cannot be opened, holds an unknown residue name (the reference indexes its tables
 * with -1 there, src/AminoAcids.cpp:145-181) or has no C-alpha record. */
int cgppd_pdb_read(const char *path, const AminoAcids *a, int capacity, float *xyz, int *types, char *chain_ids,
                   int *res_seq, int *chain_index, int *num_chains);

/* Replaces Replica::saveAsSinglePDB (src/Replica.cpp:1124-1168), the sample PDB the
 * reference writes for every recorded sample: "REMARK simulation/temperature/sample/
 * potential" lines (the potential as a float, 10 decimals), one CA ATOM record per
 * residue (residue name in capitals, chain letter 'A' + chain[i], number res_seq[i],
 * coordinates xyz[3i..3i+2]), a TER record after every chain change inside a molecule
 * and after every molecule (molecule[i] numbers them), END.  Returns 0, or -1 with the
 * message in cgppd_get_last_error (missing arguments, a type outside 0..19, a chain
 * outside A..Z, a file that cannot be opened). */
int cgppd_pdb_write_sample(const char *path, const AminoAcids *a, const char *title, float temperature, int sample,
                           double potential, int n, const float *xyz, const int *types, const int *res_seq,
                           const int *chain, const int *molecule);

#ifdef __cplusplus
}
#endif

#endif /* CGPPD_PDB_H_ */
