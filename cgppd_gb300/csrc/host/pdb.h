// pdb.h -- C-alpha records of a PDB file and the placement of a molecule.
#pragma once

#include <string>
#include <vector>

#include "amino_acids.h"

namespace cgppd {

struct PdbResidue {
    std::string name;  // residue name
    char chain;        // chain identifier (column 22)
    int res_seq;       // residue sequence number
    int chain_index;   // number of TER records before this residue
    int type;          // residue-type index, -1 if the name is unknown
    float x, y, z;
};

// Molecule::initFromPDB (src/Molecule.cpp:506-612): ATOM records whose atom name is CA,
// TER counts chains, a record starting with END stops reading, a file with residues but
// no TER has one chain.  Throws a const char* when the file cannot be opened or holds an
// unknown residue name (the reference would index its tables with -1).
std::vector<PdbResidue> read_pdb(const std::string &path, const AminoAcids &aa, int *num_chains);

// A molecule as Molecule::init leaves it: centre = float mean of the file's positions,
// relative positions, then `p(x,y,z)` (set the centre) or `t(x,y,z)` (translate and
// wrap the centre), then a rotation about the normalised axis by `angle` rad
// (src/Molecule.cpp:25-64, :183-208).
struct PlacedMolecule {
    std::vector<PdbResidue> residues;
    int num_chains = 1;
    std::vector<float> pos, rel;  // 3n each
    float center[3] = {0, 0, 0};
};

PlacedMolecule place_molecule(const std::vector<PdbResidue> &res, int num_chains, bool translate, float px, float py,
                              float pz, float rx, float ry, float rz, float angle, float box);

// Reference PDB output of one molecule's C-alpha trace (src/Replica.cpp:1124-1168 format).
// Chain letters are replica-wide, as the reference's chain UIDs (src/Geometry.cpp:256-297):
// 'A' + chain_base + the residue's chain index, chain_base counting the chains of the
// molecules before this one.
void write_pdb_atoms(FILE *out, const std::vector<PdbResidue> &res, const float *pos, const AminoAcids &aa,
                     int *atom_counter, int chain_base = 0);

// The same records for n residues given as arrays: types, residue numbers, replica-wide
// chain numbers (0 = 'A') and molecule numbers (a TER record follows each molecule and
// every chain change inside one).
void write_pdb_trace(FILE *out, int n, const float *xyz, const int *types, const int *res_seq, const int *chain,
                     const int *molecule, const AminoAcids &aa, int *atom_counter);

// Replica::saveAsSinglePDB (src/Replica.cpp:1124-1168): the sample's header (simulation
// title, temperature, sample step, the replica potential as a float), its C-alpha
// records (write_pdb_trace), END.
void write_sample_pdb(FILE *out, const char *title, float temperature, int sample, double potential, int n,
                      const float *xyz, const int *types, const int *res_seq, const int *chain, const int *molecule,
                      const AminoAcids &aa);

}  // namespace cgppd
