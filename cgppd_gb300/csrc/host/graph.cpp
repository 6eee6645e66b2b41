// graph.cpp -- see graph.h.
#include "graph.h"

#include <cstdlib>

namespace cgppd {

void Graph::add_edge(int i, int j, bool flexible)
{
    vertices_.insert(i);
    vertices_.insert(j);
    edges_.insert(i < j ? std::make_pair(i, j) : std::make_pair(j, i));
    adj_[i].insert(j);
    adj_[j].insert(i);
    flexible_[std::make_pair(i, j)] = flexible;
    flexible_[std::make_pair(j, i)] = flexible;
}

bool Graph::is_flexible(int i, int j) const
{
    auto it = flexible_.find(std::make_pair(i, j));
    return it != flexible_.end() && it->second;
}

std::vector<int> Graph::neighbours(int i) const
{
    auto it = adj_.find(i);
    if (it == adj_.end())
        return {};
    return std::vector<int>(it->second.begin(), it->second.end());
}

void Graph::init(const std::vector<char> &chain_ids, bool all_flexible, const std::vector<std::vector<int>> &segments,
                 int nchains)
{
    num_chains = nchains;
    const int n = (int)chain_ids.size();
    // Backbone edges within a chain (flexible only when the whole molecule is), then
    // the segment edges, which are always flexible and override.
    for (int i = 0; i + 1 < n; ++i)
        if (chain_ids[i] == chain_ids[i + 1])
            add_edge(i, i + 1, all_flexible);
    for (const auto &s : segments)
        for (size_t k = 0; k + 1 < s.size(); ++k)
            add_edge(s[k], s[k + 1], true);

    // Bonds are the flexible edges; a torsion i-j-k-l is recorded around every edge j-k
    // whose ends both have other neighbours, when any of its three edges is flexible.
    for (const auto &e : edges_) {
        const int j = e.first, k = e.second;
        if (is_flexible(j, k))
            bonds.insert(Pair{j, k});
        const std::set<int> &nj = adj_[j], &nk = adj_[k];
        if (nj.size() > 1 && nk.size() > 1)
            for (int i : nj) {
                if (i == k)
                    continue;
                for (int l : nk) {
                    if (l == j)
                        continue;
                    if (is_flexible(i, j) || is_flexible(j, k) || is_flexible(k, l))
                        torsions.insert(Torsion4{i, j, k, l});
                }
            }
    }

    // Angles around each vertex with a flexible edge; MC residue sets.
    std::set<int> local, crank, flex;
    for (int j : vertices_) {
        const std::set<int> &nb = adj_[j];
        bool has_rigid = false, has_flexible = false;
        for (int i : nb) {
            if (is_flexible(i, j))
                has_flexible = true;
            else
                has_rigid = true;
            for (int k : nb)
                if (i < k && (is_flexible(i, j) || is_flexible(j, k)))
                    angles.insert(Angle3{i, j, k});
        }
        if (!has_rigid) {
            local.insert(j);
            if (nb.size() > 1)
                crank.insert(j);
        }
        if (has_flexible)
            flex.insert(j);
    }
    MC_local_residues.assign(local.begin(), local.end());
    MC_crankshaft_residues.assign(crank.begin(), crank.end());
    MC_flex_residues.assign(flex.begin(), flex.end());

    // Rigid domains: connected groups of more than one residue over rigid edges, in order
    // of their lowest residue.
    std::set<int> todo(vertices_);
    while (!todo.empty()) {
        std::set<int> dom = rigid_domain_around(*todo.begin());
        for (int v : dom)
            todo.erase(v);
        if (dom.size() > 1)
            rigid_domains.push_back(dom);
    }

    // Segment bonds join residues that are not backbone neighbours.
    for (const auto &b : bonds)
        if (chain_ids[b.i] != chain_ids[b.j] || std::abs(b.i - b.j) >= 4)
            segment_bonds.push_back(b);

    // Indirect neighbours: end pairs of the torsions around each segment bond.  The
    // reference's tests for the two extra pairs compare C++ comma expressions
    // (`(t->i, t->j) == (p->i, p->j)` and so on, src/Geometry.cpp:175-180), which reduce to
    // comparing the second elements only; that behaviour defines the set and is kept.
    for (const auto &p : segment_bonds) {
        std::set<Pair> proposed;
        for (const auto &t : torsions) {
            if (!(t.contains(p.i) && t.contains(p.j)))
                continue;
            proposed.insert(Pair{t.i, t.l});
            if (t.j == p.j || t.i == p.j)
                proposed.insert(Pair{t.i, t.k});
            if (t.l == p.j || t.k == p.j)
                proposed.insert(Pair{t.j, t.l});
        }
        for (const auto &pr : proposed)
            if (chain_ids[pr.i] != chain_ids[pr.j] || std::abs(pr.i - pr.j) >= 4)
                indirect_neighbours.insert(pr.i < pr.j ? pr : Pair{pr.j, pr.i});
    }
}

std::set<int> Graph::branch_rec(int i, int j, const std::set<std::pair<int, int>> &visited) const
{
    std::set<int> out{i, j};
    auto it = adj_.find(j);
    if (it == adj_.end())
        return out;
    std::set<std::pair<int, int>> nv(visited);
    nv.insert(std::make_pair(i, j));
    for (int k : it->second) {
        if (k == i || visited.count(std::make_pair(j, k)))
            continue;
        std::set<int> sub = branch_rec(j, k, nv);
        out.insert(sub.begin(), sub.end());
    }
    return out;
}

std::set<int> Graph::branch(int i, int j) const { return branch_rec(i, j, {}); }

std::set<int> Graph::domain_rec(int i, const std::set<std::pair<int, int>> &visited) const
{
    std::set<int> dom{i};
    auto it = adj_.find(i);
    if (it == adj_.end())
        return dom;
    for (int j : it->second) {
        if (is_flexible(i, j) || visited.count(std::make_pair(j, i)))
            continue;
        std::set<std::pair<int, int>> nv(visited);
        nv.insert(std::make_pair(i, j));
        std::set<int> sub = domain_rec(j, nv);
        dom.insert(sub.begin(), sub.end());
    }
    return dom;
}

std::set<int> Graph::rigid_domain_around(int i) const { return domain_rec(i, {}); }

}  // namespace cgppd
