// graph.h -- flexible-segment graph of one molecule (bonds, angles, torsions, rigid
// domains, segment bonds, indirect neighbours and the Monte Carlo residue sets).
//
// Same definitions as the reference's Graph (src/Geometry.h:131-176,
// src/Geometry.cpp:34-302); residue indices are positions in the molecule.
#pragma once

#include <map>
#include <set>
#include <utility>
#include <vector>

namespace cgppd {

struct Pair {
    int i, j;
    bool operator<(const Pair &o) const { return i != o.i ? i < o.i : j < o.j; }
    bool operator==(const Pair &o) const { return i == o.i && j == o.j; }
};

struct Angle3 {
    int i, j, k;
    bool operator<(const Angle3 &o) const
    {
        if (i != o.i) return i < o.i;
        if (j != o.j) return j < o.j;
        return k < o.k;
    }
};

struct Torsion4 {
    int i, j, k, l;
    bool operator<(const Torsion4 &o) const
    {
        if (i != o.i) return i < o.i;
        if (j != o.j) return j < o.j;
        if (k != o.k) return k < o.k;
        return l < o.l;
    }
    bool contains(int r) const { return r == i || r == j || r == k || r == l; }
};

class Graph {
public:
    // chain_ids: one chain character per residue; segments: residue index lists (0-based)
    // whose consecutive entries are joined by flexible bonds.
    void init(const std::vector<char> &chain_ids, bool all_flexible, const std::vector<std::vector<int>> &segments,
              int num_chains);

    int num_chains = 0;
    std::set<Pair> bonds;
    std::set<Angle3> angles;
    std::set<Torsion4> torsions;
    std::vector<int> MC_local_residues;
    std::vector<int> MC_crankshaft_residues;
    std::vector<int> MC_flex_residues;
    std::vector<std::set<int>> rigid_domains;
    std::vector<Pair> segment_bonds;
    std::set<Pair> indirect_neighbours;

    std::vector<int> neighbours(int i) const;
    // Residues moved when the edge i->j is rotated about i: i, j and everything
    // reachable from j without walking back along an edge already taken.
    std::set<int> branch(int i, int j) const;
    // Residues joined to i through rigid (non-flexible) edges.
    std::set<int> rigid_domain_around(int i) const;
    bool is_flexible(int i, int j) const;
    int vertex_count() const { return (int)vertices_.size(); }

private:
    void add_edge(int i, int j, bool flexible);
    std::set<int> branch_rec(int i, int j, const std::set<std::pair<int, int>> &visited) const;
    std::set<int> domain_rec(int i, const std::set<std::pair<int, int>> &visited) const;

    std::set<int> vertices_;
    std::set<std::pair<int, int>> edges_;
    std::map<int, std::set<int>> adj_;
    std::map<std::pair<int, int>, bool> flexible_;
};

}  // namespace cgppd
