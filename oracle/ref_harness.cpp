// ref_harness.cpp -- C entry points over the reference's own energy code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.py together with the
// reference's sources (Potential, Residue, AminoAcids, AminoAcid, Geometry, Quaternion,
// vector3f, TorsionalLookupMatrix -- read in place from the reference tree) into
// oracle/_ref/libcgppd_ref.so, which exists only where the reference tree is mounted.
// It composes the reference's functions exactly as Replica::E() (src/Replica.cpp:421-500)
// and Molecule::E(true) (src/Molecule.cpp:636-699) do; those two classes themselves
// need GSL and logog, which are not available, so their loops are restated here around
// the reference's own calculate_* functions, Residue predicates and Graph.
#include <cstring>
#include <vector>

#include "Geometry.h"
#include "Potential.h"

namespace {

void fill_table(AminoAcids &aa, const float *table20)
{
    for (int i = 0; i < 20; ++i)
        for (int j = 0; j < 20; ++j)
            aa.LJpotentials[i][j] = table20[i * 20 + j];
}

}  // namespace

extern "C" {

// Total of E() + sum over flexible molecules of Molecule::E(true) in raw accumulators
// {LJ, DH, bond, angle product, torsion} (out5) and the inter-molecule part alone
// (inter2).  Types >= 20 mark crowder residues whose every contact uses crowder_raw.
int ref_energy(int nmol, const int *mstart, const int *mcount, const int *mflex, const int *mcrowder,
               const float *xyz, const int *types, const float *q, const float *sig, const char *chain_ids,
               const int *res_seq, const int *chain_index, const int *nseg, const int *seg_len, const int *seg_res,
               const float *table20, float crowder_raw, const double *torsV, const double *torsS, float box,
               double *out5, double *inter2)
{
    AminoAcids amino, crowd;
    fill_table(amino, table20);
    for (int i = 0; i < 20; ++i)
        for (int j = 0; j < 20; ++j)
            crowd.LJpotentials[i][j] = crowder_raw;
    TorsionalLookupMatrix tors;
    if (torsV)
        for (int i = 0; i < 20; ++i)
            for (int j = 0; j < 20; ++j)
                for (int n = 0; n < 4; ++n) {
                    tors.V[i][j][n] = torsV[(i * 20 + j) * 4 + n];
                    tors.Sigma[i][j][n] = torsS[(i * 20 + j) * 4 + n];
                }
    int total = 0;
    for (int m = 0; m < nmol; ++m)
        total += mcount[m];
    std::vector<Residue> res(total);
    for (int i = 0; i < total; ++i) {
        Residue &r = res[i];
        r.aminoAcidIndex = types[i] >= 20 ? 0 : types[i];
        r.electrostaticCharge = q[i];
        r.vanderWaalRadius = sig[i];
        r.position = Vector3f(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        r.chainId = chain_ids[i];
        r.resSeq = res_seq[i];
        r.chain_int_id = chain_index[i];
    }
    Potential inter;
    for (int a = 0; a < nmol; ++a)
        for (int b = a + 1; b < nmol; ++b) {
            const AminoAcids &tab = (mcrowder[a] || mcrowder[b]) ? crowd : amino;
            for (int i = mstart[a]; i < mstart[a] + mcount[a]; ++i)
                for (int j = mstart[b]; j < mstart[b] + mcount[b]; ++j) {
                    double r = res[i].distance(res[j], box) + EPS;
                    inter.increment_LJ(calculate_LJ(res[i], res[j], r, tab));
                    inter.increment_DH(calculate_DH(res[i], res[j], r));
                }
        }
    Potential pot = inter;
    int chain_off = 1, dom_off = 1, bond_off = 1, seg_pos = 0;
    for (int m = 0; m < nmol; ++m) {
        std::vector<segdata> segs;
        for (int k = 0; k < nseg[m]; ++k) {
            segdata s;
            for (int v = 0; v < seg_len[seg_pos]; ++v)
                s.residue_indices.push_back(*seg_res++);
            segs.push_back(s);
            ++seg_pos;
        }
        if (!mflex[m] && segs.empty())
            continue;
        Residue *R = &res[mstart[m]];
        const int n = mcount[m];
        std::vector<Residue> vr(R, R + n);
        int nchains = 1;
        for (int i = 0; i < n; ++i)
            nchains = std::max(nchains, chain_index[mstart[m] + i] + 1);
        Graph g;
        g.init(vr, mflex[m] != 0, segs, nchains);
        g.assign_uids(R, chain_off, dom_off, bond_off);
        Potential p;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j)
                if (!R[i].same_rigid_domain_as(R[j]) && !R[i].chain_neighbour_of(R[j]) && !R[i].bonded_to(R[j]) &&
                    !g.indirect_neighbours.count(Pair(i, j))) {
                    double r = R[i].distance(R[j], box) + EPS;
                    p.increment_LJ(calculate_LJ(R[i], R[j], r, amino));
                    p.increment_DH(calculate_DH(R[i], R[j], r));
                }
        for (std::set<Bond>::iterator b = g.bonds.begin(); b != g.bonds.end(); ++b)
            p.increment_bond(calculate_bond(R, *b, box));
        for (std::set<Angle>::iterator a = g.angles.begin(); a != g.angles.end(); ++a)
            p.increment_angle(calculate_angle(R, *a));
        for (std::set<Torsion>::iterator t = g.torsions.begin(); t != g.torsions.end(); ++t)
            p.increment_torsion(calculate_torsion(R, *t, tors));
        pot += p;
    }
    out5[0] = pot.LJ;
    out5[1] = pot.DH;
    out5[2] = pot.bond;
    out5[3] = pot.angle;
    out5[4] = pot.torsion;
    inter2[0] = inter.LJ;
    inter2[1] = inter.DH;
    return 0;
}

// Graph::init of one molecule: counts {bonds, angles, torsions, rigid domains, segment
// bonds, indirect neighbours, local, crankshaft, flex} into counts9, and the sorted
// flat lists (pairs/triples/quads) into the given buffers (capacity in cap).
int ref_graph(int n, const char *chain_ids, int all_flexible, int nseg, const int *seg_len, const int *seg_res,
              int num_chains, int *counts9, int cap, int *bonds, int *angles, int *torsions, int *indirect)
{
    std::vector<Residue> vr(n);
    for (int i = 0; i < n; ++i)
        vr[i].chainId = chain_ids[i];
    std::vector<segdata> segs;
    for (int k = 0; k < nseg; ++k) {
        segdata s;
        for (int v = 0; v < seg_len[k]; ++v)
            s.residue_indices.push_back(*seg_res++);
        segs.push_back(s);
    }
    Graph g;
    g.init(vr, all_flexible != 0, segs, num_chains);
    counts9[0] = (int)g.bonds.size();
    counts9[1] = (int)g.angles.size();
    counts9[2] = (int)g.torsions.size();
    counts9[3] = (int)g.rigid_domains.size();
    counts9[4] = (int)g.segment_bonds.size();
    counts9[5] = (int)g.indirect_neighbours.size();
    counts9[6] = (int)g.MC_local_residues.size();
    counts9[7] = (int)g.MC_crankshaft_residues.size();
    counts9[8] = (int)g.MC_flex_residues.size();
    int k = 0;
    for (std::set<Bond>::iterator b = g.bonds.begin(); b != g.bonds.end() && k + 2 <= cap; ++b, k += 2)
        bonds[k] = b->i, bonds[k + 1] = b->j;
    k = 0;
    for (std::set<Angle>::iterator a = g.angles.begin(); a != g.angles.end() && k + 3 <= cap; ++a, k += 3)
        angles[k] = a->i, angles[k + 1] = a->j, angles[k + 2] = a->k;
    k = 0;
    for (std::set<Torsion>::iterator t = g.torsions.begin(); t != g.torsions.end() && k + 4 <= cap; ++t, k += 4)
        torsions[k] = t->i, torsions[k + 1] = t->j, torsions[k + 2] = t->k, torsions[k + 3] = t->l;
    k = 0;
    for (std::set<Pair>::iterator p = g.indirect_neighbours.begin(); p != g.indirect_neighbours.end() && k + 2 <= cap;
         ++p, k += 2)
        indirect[k] = p->i, indirect[k + 1] = p->j;
    return 0;
}

// Byte offset of AminoAcids::LJpotentials in the reference's own class.
size_t ref_lj_offset(void)
{
    static AminoAcids probe;
    return (size_t)(reinterpret_cast<const char *>(&probe.LJpotentials[0][0]) - reinterpret_cast<const char *>(&probe));
}
}
