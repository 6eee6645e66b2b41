// engine_host.cu -- host side of the batched replica-exchange engine (see cgppd_remc.h).
//
// Builds the device tables from molecules (flexible-segment graph, replica-wide
// UIDs, exclusion keys, move candidate lists), owns the device buffers, and drives
// the kernels as CUDA-graph replays of [MC block, exchange].
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "cgppd_common.cuh"
#include "cgppd_remc.h"
#include "cgppd_surrogate.h"
#include "devbuf.h"
#include "engine_types.h"
#include "host/graph.h"
#include "status.h"
#include "surrogate.cuh"
#include "surrogate_internal.h"

namespace cgppd {
size_t engine_smem_bytes(int max_mol, int max_n, int max_m, int cluster, int resident, int any_flexible, int da,
                         const int *lmax);
cudaError_t launch_pose_samples(const EngineArgs &a, const int4 *items, int n, uint32_t key0, uint32_t key1, float *X,
                                float *Y, cudaStream_t stream);
cudaError_t launch_mc_block(const EngineArgs &a, int total_replicas, int nsteps, int threads, size_t smem,
                            cudaStream_t stream);
cudaError_t set_mc_smem_limit(size_t smem);
cudaError_t launch_init_energy(const EngineArgs &a, int total_replicas, size_t smem, double *potential_out,
                               cudaStream_t stream);
cudaError_t launch_exchange(const EngineArgs &a, int nsims, int total_replicas, int steps_per_block,
                            cudaStream_t stream);
cudaError_t launch_final_report(const EngineArgs &a, int nsims, int total_replicas, int row, cudaStream_t stream);
}  // namespace cgppd

using namespace cgppd;

namespace {

struct HostMolecule {
    int n = 0;
    std::vector<float> xyz, rel;
    float center[3] = {0, 0, 0};
    std::vector<int> types, res_seq, chain_index;
    std::vector<float> charges, radii;
    std::vector<char> chain_ids;
    int num_chains = 1;
    bool all_flexible = false, crowder = false;
    std::vector<std::vector<int>> segments;
};

struct HostSim {
    cgppd_sim_params p{};
    std::vector<float> temps, tsteps;
    std::vector<double> rsteps;
    std::vector<HostMolecule> mols;
};



// Residues spanning a molecule's body frame, from its centred coordinates: the one
// farthest from the centre, the one farthest from it, and the one farthest from the line
// through both (lowest index on ties), so copies of one molecule pick the same residues.
void frame_residues(const HostMolecule &hm, int &f0, int &f1, int &f2)
{
    f0 = f1 = f2 = 0;
    if (hm.n < 3)
        return;
    auto q = [&](int i, int k) { return (double)hm.rel[3 * i + k]; };
    double best = -1.0;
    for (int i = 0; i < hm.n; ++i) {
        const double d = q(i, 0) * q(i, 0) + q(i, 1) * q(i, 1) + q(i, 2) * q(i, 2);
        if (d > best)
            best = d, f0 = i;
    }
    best = -1.0;
    for (int i = 0; i < hm.n; ++i) {
        double d = 0.0;
        for (int k = 0; k < 3; ++k)
            d += (q(i, k) - q(f0, k)) * (q(i, k) - q(f0, k));
        if (d > best)
            best = d, f1 = i;
    }
    double u[3], nu = 0.0;
    for (int k = 0; k < 3; ++k) {
        u[k] = q(f1, k) - q(f0, k);
        nu += u[k] * u[k];
    }
    nu = std::sqrt(nu);
    for (int k = 0; k < 3; ++k)
        u[k] /= (nu > 0.0 ? nu : 1.0);
    best = -1.0;
    for (int i = 0; i < hm.n; ++i) {
        double v[3], dot = 0.0;
        for (int k = 0; k < 3; ++k) {
            v[k] = q(i, k) - q(f0, k);
            dot += v[k] * u[k];
        }
        double d = 0.0;
        for (int k = 0; k < 3; ++k)
            d += (v[k] - dot * u[k]) * (v[k] - dot * u[k]);
        if (d > best)
            best = d, f2 = i;
    }
}

}  // namespace

struct cgppd_engine {
    std::vector<float> table;  // -4 Eij kcal/mol, 32x32
    std::vector<double> torsV, torsS;
    int tors_types = 0;
    int ntypes = 0;
    uint64_t seed = 0;
    std::vector<HostSim> sims;
    bool finalized = false;

    // launch shape
    int cluster = 1, threads = 256;
    size_t smem = 0;
    int total_replicas = 0;
    int max_n = 0, max_m = 0, max_mol = 0;
    int lmax[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // largest per-simulation static list sizes
    int resident = 0, any_flexible = 0;
    int resident_pref = 1;
    // delayed acceptance
    cgppd_surrogate *sur = nullptr;
    int da = 0;
    float sur_thr = 0.5f, sur_window = 25.0f;
    int sur_min = 100;
    int plain_cluster = 1, plain_threads = 256;
    DevBuf<int> d_sim_da;
    DevBuf<DAStats> d_dastats;
    int report_capacity = 0;
    int last_launches = 0;

    cudaStream_t own_stream = nullptr;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (steps, exchange) -> graph

    // device buffers
    DevBuf<DevSim> d_sims;
    DevBuf<int> d_rep_sim, d_rep_order;
    DevBuf<DevMol> d_mols;
    DevBuf<float4> d_rstat;
    DevBuf<unsigned short> d_rqpos;
    DevBuf<int4> d_rexcl;
    DevBuf<int2> d_bonds, d_indsub;
    DevBuf<int4> d_angles, d_tors, d_flexres, d_flexopt;
    DevBuf<float4> d_torsV, d_torsS;
    DevBuf<int> d_branch, d_localres, d_crankres;
    DevBuf<int2> d_tiles;
    DevBuf<float> d_table;
    DevBuf<float4> d_pos, d_rel, d_center;
    DevBuf<double> d_emat, d_intra, d_potential, d_scratch_pot, d_scratch_emat, d_scratch_intra;
    DevBuf<float> d_temperature, d_tstep;
    DevBuf<double> d_rstep;
    DevBuf<unsigned long long> d_stepc, d_pairc;
    DevBuf<ReplicaStats> d_stats;
    DevBuf<int> d_tindex, d_label, d_slot_of_t, d_sim_state;
    DevBuf<float4> d_report;
    DevBuf<int2> d_exch_report;
    DevBuf<unsigned> d_errflags;
    DevBuf<SampleRec> d_sample_log;  // boundconformations records (cgppd_engine_set_sample_log)
    DevBuf<unsigned> d_sample_count;
    int sample_cap = 0;
    DevBuf<float4> d_sample_xyz;     // their coordinates (cgppd_engine_set_sample_snapshots)
    int sample_nres = 0;

    std::vector<DevSim> h_sims;
    std::vector<DevMol> h_mols;

    struct TuneResult {
        int cluster, threads;
        float us_per_step;
    };
    std::vector<TuneResult> tuning;  // the autotuner's measurements (empty if not run)

    ~cgppd_engine()
    {
        for (auto &kv : graphs)
            cudaGraphExecDestroy(kv.second);
        if (own_stream)
            cudaStreamDestroy(own_stream);
    }

    EngineArgs args() const
    {
        EngineArgs a{};
        a.sims = d_sims.ptr;
        a.rep_sim = d_rep_sim.ptr;
        a.rep_order = d_rep_order.ptr;
        a.mols = d_mols.ptr;
        a.rstat = d_rstat.ptr;
        a.rqpos = d_rqpos.ptr;
        a.rexcl = d_rexcl.ptr;
        a.bonds = d_bonds.ptr;
        a.angles = d_angles.ptr;
        a.tors = d_tors.ptr;
        a.torsV = d_torsV.ptr;
        a.torsS = d_torsS.ptr;
        a.indsub = d_indsub.ptr;
        a.flexres = d_flexres.ptr;
        a.flexopt = d_flexopt.ptr;
        a.branch = d_branch.ptr;
        a.localres = d_localres.ptr;
        a.crankres = d_crankres.ptr;
        a.tiles = d_tiles.ptr;
        a.table = d_table.ptr;
        a.pos = d_pos.ptr;
        a.rel = d_rel.ptr;
        a.center = d_center.ptr;
        a.emat = d_emat.ptr;
        a.intra = d_intra.ptr;
        a.potential = d_potential.ptr;
        a.temperature = d_temperature.ptr;
        a.tstep = d_tstep.ptr;
        a.rstep = d_rstep.ptr;
        a.stepc = d_stepc.ptr;
        a.pairc = d_pairc.ptr;
        a.stats = d_stats.ptr;
        a.tindex = d_tindex.ptr;
        a.label = d_label.ptr;
        a.slot_of_t = d_slot_of_t.ptr;
        a.sim_state = d_sim_state.ptr;
        a.report = d_report.ptr;
        a.exch_report = d_exch_report.ptr;
        a.report_capacity = report_capacity;
        a.errflags = d_errflags.ptr;
        a.sample_log = sample_cap > 0 ? d_sample_log.ptr : nullptr;
        a.sample_count = d_sample_count.ptr;
        a.sample_cap = sample_cap;
        a.sample_xyz = (sample_cap > 0 && sample_nres > 0) ? d_sample_xyz.ptr : nullptr;
        a.sample_nres = sample_nres;
        a.seed_lo = (uint32_t)seed;
        a.seed_hi = (uint32_t)(seed >> 32);
        a.ntypes = ntypes;
        a.cluster = cluster;
        a.max_n = max_n;
        a.max_m = max_m;
        a.max_mol = max_mol;
        for (int k = 0; k < 10; ++k)
            a.lmax[k] = lmax[k];
        a.resident = resident;
        a.any_flexible = any_flexible;
        // the charged-first mover order (Debye-Hueckel terms for charged residues only)
        // pays off for rigid systems with long per-thread i loops; elsewhere it lengthens
        // the kernel for nothing (measured: C2 +6 %, C3 +10 %; C4 -3 % and C1 -3 % when
        // compiled into their kernel), so it is a separate instantiation
        a.qfirst = (!any_flexible && max_mol >= 96) ? 1 : 0;
        a.da = da;
        a.sur_P = surrogate_device_params(sur);
        a.sur_wf = surrogate_device_wf(sur);
        a.sim_da = d_sim_da.ptr;
        a.dastats = d_dastats.ptr;
        a.sur_thr2 = sur_thr * sur_thr;
        a.sur_window = sur_window;
        a.sur_min = sur_min;
        return a;
    }

    int build();
};

// Build every static table and the initial replica state.
int cgppd_engine::build()
{
    std::vector<float4> rstat;
    std::vector<int4> rexcl, angles, tors, flexres, flexopt;
    std::vector<int2> bonds, indsub, tiles;
    std::vector<float4> torsVv, torsSv;
    std::vector<int> branch, localres, crankres, rep_sim;
    std::vector<unsigned short> rqpos;
    std::vector<float4> pos, rel, center;
    std::vector<float> temperature, tstep;
    std::vector<double> rstep;
    std::vector<int> tindex, label, slot_of_t;
    const float qscale = std::sqrt(kDHFactor);
    long long state_off = 0, emat_off = 0;
    int molst_off = 0, rep_off = 0, res_off = 0, mol_off = 0;
    h_sims.clear();
    h_mols.clear();

    for (size_t s = 0; s < sims.size(); ++s) {
        HostSim &hs = sims[s];
        DevSim ds{};
        int N = 0;
        for (auto &m : hs.mols)
            N += m.n;
        const int M = (int)hs.mols.size();
        const int R = hs.p.n_replicas;
        if (M == 0 || N == 0)
            return cgppd_fail("engine: a simulation has no molecules");
        if (!(hs.p.box > 0.0f))
            return cgppd_fail("engine: the periodic box edge must be positive");
        ds.N = N, ds.M = M, ds.R = R;
        ds.res_off = res_off, ds.mol_off = mol_off, ds.rep_off = rep_off;
        ds.state_off = state_off, ds.molst_off = molst_off, ds.emat_off = emat_off;
        ds.box = hs.p.box, ds.inv_box = 1.0f / hs.p.box;
        float wsum = 0.f;
        for (int k = 0; k < 4; ++k)
            wsum += hs.p.move_weights[k];
        float acc = 0.f;
        for (int k = 0; k < 4; ++k) {
            acc += hs.p.move_weights[k];
            ds.w_cum[k] = acc / wsum;
        }
        float w1 = hs.p.move_weights[1] + hs.p.move_weights[2] + hs.p.move_weights[3];
        ds.w1_cum[0] = hs.p.move_weights[1] / w1;
        ds.w1_cum[1] = (hs.p.move_weights[1] + hs.p.move_weights[2]) / w1;
        ds.w1_cum[2] = 1.0f;
        ds.rigid_rotate_p = hs.p.rigid_rotate_prob;
        // u < c  <=>  w < ceil(c 2^32) for the 32-bit draw w = u 2^32
        auto thr = [](float c) { return (unsigned long long)std::ceil((double)c * 4294967296.0); };
        for (int k = 0; k < 4; ++k)
            ds.thr4[k] = thr(ds.w_cum[k]);
        for (int k = 0; k < 3; ++k)
            ds.thr3[k] = thr(ds.w1_cum[k]);
        ds.thr_rot = thr(ds.rigid_rotate_p);
        ds.sample_freq = hs.p.sample_frequency;
        ds.sample_after = hs.p.sample_after;
        ds.bound_threshold = hs.p.bound_threshold;

        auto list_sizes = [&]() {
            return std::vector<int>{(int)bonds.size(), (int)angles.size(), (int)tors.size(), (int)indsub.size(),
                                    (int)flexres.size(), (int)flexopt.size(), (int)branch.size(),
                                    (int)localres.size(), (int)crankres.size(), (int)tiles.size()};
        };
        const std::vector<int> lbase = list_sizes();
        // replica-wide UIDs (Graph::assign_uids with running offsets, src/Replica.cpp:33-40)
        int chain_off = 1, dom_off = 1, bond_off = 1;
        int non_crowders = 0;
        bool seen_crowder = false, flexible_exists = false;
        int start = 0;
        for (int mi = 0; mi < M; ++mi) {
            HostMolecule &hm = hs.mols[mi];
            const bool flexible = !hs.p.rigid_only && (hm.all_flexible || !hm.segments.empty());
            if (flexible)
                any_flexible = 1;
            flexible_exists = flexible_exists || (hm.all_flexible || !hm.segments.empty());
            if (hm.crowder)
                seen_crowder = true;
            else if (!seen_crowder)
                ++non_crowders;
            Graph G;
            G.init(hm.chain_ids, hm.all_flexible, hm.segments, hm.num_chains);
            std::vector<int> chain_uid(hm.n, 0), dom_uid(hm.n, 0), bond_uid(hm.n, 0);
            std::map<int, int> cu;
            for (int c = 0; c < G.num_chains; ++c)
                cu[c] = chain_off + c;
            chain_off += G.num_chains;
            for (size_t d = 0; d < G.rigid_domains.size(); ++d)
                for (int v : G.rigid_domains[d])
                    dom_uid[v] = dom_off + (int)d;
            dom_off += (int)G.rigid_domains.size();
            for (size_t b = 0; b < G.segment_bonds.size(); ++b) {
                bond_uid[G.segment_bonds[b].i] = bond_off + (int)b;
                bond_uid[G.segment_bonds[b].j] = bond_off + (int)b;
            }
            bond_off += (int)G.segment_bonds.size();
            for (int i = 0; i < G.vertex_count() && i < hm.n; ++i) {
                auto it = cu.find(hm.chain_index[i]);
                chain_uid[i] = it == cu.end() ? 0 : it->second;
            }
            auto excluded = [&](int i, int j) {
                return (dom_uid[i] && dom_uid[i] == dom_uid[j]) ||
                       (chain_uid[i] == chain_uid[j] && std::abs(hm.res_seq[i] - hm.res_seq[j]) < 4) ||
                       (bond_uid[i] && bond_uid[i] == bond_uid[j]);
            };

            DevMol dm{};
            dm.start = start;
            dm.count = hm.n;
            frame_residues(hm, dm.fr0, dm.fr1, dm.fr2);
            dm.flags = (flexible ? kMolFlexible : 0) | (hm.crowder ? kMolCrowder : 0);
            for (int i = 0; i < hm.n; ++i) {
                float4 r4;
                r4.x = 0.5f * hm.radii[i];
                r4.y = hm.charges[i] * qscale;
                int ty = hm.types[i];
                if (ty < 0 || ty >= ntypes)
                    return cgppd_fail("engine: residue type outside the contact table");
                std::memcpy(&r4.z, &ty, 4);
                int mol = mi;
                std::memcpy(&r4.w, &mol, 4);
                rstat.push_back(r4);
                rexcl.push_back(make_int4(chain_uid[i], hm.res_seq[i], dom_uid[i], bond_uid[i]));
            }
            // charged residues first (stable), so the inter pair loop can take the
            // Debye-Hueckel term for them only
            {
                const size_t r0 = rstat.size() - hm.n;
                int nq = 0;
                for (int i = 0; i < hm.n; ++i)
                    nq += (rstat[r0 + i].y != 0.0f) ? 1 : 0;
                int kq = 0, ku = nq;
                for (int i = 0; i < hm.n; ++i)
                    rqpos.push_back((unsigned short)((rstat[r0 + i].y != 0.0f) ? kq++ : ku++));
                dm.nq = nq;
            }
            if (flexible) {
                dm.bond_off = (int)bonds.size();
                for (const auto &b : G.bonds)
                    bonds.push_back(make_int2(b.i, b.j));
                dm.nbond = (int)bonds.size() - dm.bond_off;
                dm.ang_off = (int)angles.size();
                for (const auto &an : G.angles)
                    angles.push_back(make_int4(an.i, an.j, an.k, 0));
                dm.nang = (int)angles.size() - dm.ang_off;
                dm.tor_off = (int)tors.size();
                double vsum = 0.0;
                for (const auto &t : G.torsions) {
                    tors.push_back(make_int4(t.i, t.j, t.k, t.l));
                    // A_n = V_n cos(sigma_n), B_n = V_n sin(sigma_n) (torsion term by angle addition)
                    float A[4] = {0, 0, 0, 0}, Bv[4] = {0, 0, 0, 0};
                    int a1 = hm.types[t.j], a2 = hm.types[t.k];
                    if (!torsV.empty() && a1 < tors_types && a2 < tors_types) {
                        const double *v = &torsV[4 * (a1 * tors_types + a2)];
                        const double *sg = &torsS[4 * (a1 * tors_types + a2)];
                        for (int q = 0; q < 4; ++q) {
                            A[q] = (float)(v[q] * std::cos(sg[q]));
                            Bv[q] = (float)(v[q] * std::sin(sg[q]));
                            vsum += v[q];
                        }
                    }
                    torsVv.push_back(make_float4(A[0], A[1], A[2], A[3]));
                    torsSv.push_back(make_float4(Bv[0], Bv[1], Bv[2], Bv[3]));
                }
                dm.tors_const = (float)vsum;
                dm.ntor = (int)tors.size() - dm.tor_off;
                dm.ind_off = (int)indsub.size();
                for (const auto &p : G.indirect_neighbours)
                    if (!excluded(p.i, p.j))
                        indsub.push_back(make_int2(p.i, p.j));
                dm.nind = (int)indsub.size() - dm.ind_off;
                long long nintra = 0;
                for (int i = 0; i < hm.n; ++i)
                    for (int j = i + 1; j < hm.n; ++j)
                        if (!excluded(i, j) && !G.indirect_neighbours.count(Pair{i, j}))
                            ++nintra;
                dm.nintra = (int)nintra;
                // 32 x 32 tiles (ta <= tb) with at least one pair i < j that the rules keep
                dm.tile_off = (int)tiles.size();
                const int nt = (hm.n + 31) / 32;
                for (int ta = 0; ta < nt; ++ta)
                    for (int tb = ta; tb < nt; ++tb) {
                        bool any = false;
                        for (int i = ta * 32; i < std::min(hm.n, ta * 32 + 32) && !any; ++i)
                            for (int j = std::max(i + 1, tb * 32); j < std::min(hm.n, tb * 32 + 32); ++j)
                                if (!excluded(i, j)) {
                                    any = true;
                                    break;
                                }
                        if (any)
                            tiles.push_back(make_int2(ta, tb));
                    }
                dm.ntile = (int)tiles.size() - dm.tile_off;
                // flex candidates: branch of each (residue, neighbour) edge, extended by the
                // other branches inside the residue's rigid domain (src/Molecule.cpp:331-360)
                dm.flex_off = (int)flexres.size();
                for (int ri : G.MC_flex_residues) {
                    std::vector<int> nb = G.neighbours(ri);
                    flexres.push_back(make_int4(ri, (int)nb.size(), (int)flexopt.size(), 0));
                    std::set<int> dom = G.rigid_domain_around(ri);
                    for (int nbr : nb) {
                        std::set<int> br = G.branch(ri, nbr);
                        if (dom.count(nbr))
                            for (int other : nb)
                                if (other != nbr && dom.count(other)) {
                                    std::set<int> extra = G.branch(ri, other);
                                    br.insert(extra.begin(), extra.end());
                                }
                        flexopt.push_back(make_int4(nbr, (int)branch.size(), (int)br.size(), 0));
                        branch.insert(branch.end(), br.begin(), br.end());
                    }
                }
                dm.nflex = (int)flexres.size() - dm.flex_off;
                dm.local_off = (int)localres.size();
                localres.insert(localres.end(), G.MC_local_residues.begin(), G.MC_local_residues.end());
                dm.nlocal = (int)localres.size() - dm.local_off;
                dm.crank_off = (int)crankres.size();
                crankres.insert(crankres.end(), G.MC_crankshaft_residues.begin(), G.MC_crankshaft_residues.end());
                dm.ncrank = (int)crankres.size() - dm.crank_off;
            }
            h_mols.push_back(dm);
            start += hm.n;
            max_mol = std::max(max_mol, hm.n);
        }
        const std::vector<int> lend = list_sizes();
        for (int k = 0; k < 10; ++k) {
            ds.lbase[k] = lbase[k];
            ds.lcount[k] = lend[k] - lbase[k];
            lmax[k] = std::max(lmax[k], ds.lcount[k]);
        }
        ds.non_crowders = non_crowders;
        ds.crowd_start = -1;
        if (hs.p.repulsive_crowding) {
            // crowders after every other molecule (the argfile's `crowders` section follows
            // its `files`) and rigid: a crowder pair is then j >= crowd_start or a crowder mover
            int first = 0;
            for (int mi = 0; mi < non_crowders; ++mi)
                first += hs.mols[mi].n;
            for (int mi = non_crowders; mi < M; ++mi) {
                const HostMolecule &hm = hs.mols[mi];
                if (!hm.crowder)
                    return cgppd_fail("engine: repulsive crowding needs the crowders after every other molecule");
                if (!hs.p.rigid_only && (hm.all_flexible || !hm.segments.empty()))
                    return cgppd_fail("engine: repulsive crowding needs rigid crowders");
            }
            ds.crowd_start = first;
        }
        // Replica::sample chooses what the bound test compares (src/Replica.cpp:1043-1075)
        if (M == 1)
            ds.nc_mode = 0;
        else if (M != non_crowders || (flexible_exists && !hs.p.rigid_only))
            ds.nc_mode = 1;
        else
            ds.nc_mode = 2;
        ds.max_mol = 0;
        for (auto &m : hs.mols)
            ds.max_mol = std::max(ds.max_mol, m.n);

        // replicas: every replica starts from the initial replica's coordinates
        for (int r = 0; r < R; ++r) {
            for (auto &hm : hs.mols)
                for (int i = 0; i < hm.n; ++i) {
                    pos.push_back(make_float4(hm.xyz[3 * i], hm.xyz[3 * i + 1], hm.xyz[3 * i + 2], 0.f));
                    rel.push_back(make_float4(hm.rel[3 * i], hm.rel[3 * i + 1], hm.rel[3 * i + 2], 0.f));
                }
            for (auto &hm : hs.mols)
                center.push_back(make_float4(hm.center[0], hm.center[1], hm.center[2], 0.f));
            temperature.push_back(hs.temps[r]);
            tstep.push_back(hs.tsteps[r]);
            rstep.push_back(hs.rsteps[r]);
            tindex.push_back(r);
            label.push_back(r);
            slot_of_t.push_back(r);
            rep_sim.push_back((int)s);
        }
        h_sims.push_back(ds);
        max_n = std::max(max_n, N);
        max_m = std::max(max_m, M);
        res_off += N;
        mol_off += M;
        rep_off += R;
        state_off += (long long)N * R;
        molst_off += M * R;
        emat_off += (long long)M * M * R;
    }
    total_replicas = rep_off;
    std::vector<int> sim_state(4 * sims.size(), 0);
    // k_mc's clusters run each replica to the end of the block and the next waits for
    // a free SM: the replicas with the most pair work per step go first (longest
    // processing time first), so the launch does not end on a few long replicas
    std::vector<double> sim_work(sims.size(), 0.0);
    for (size_t s = 0; s < sims.size(); ++s) {
        const HostSim &hs = sims[s];
        double N = 0.0, w = 0.0;
        for (auto &m : hs.mols)
            N += m.n;
        for (auto &m : hs.mols)
            w += (double)m.n * (N - m.n);
        sim_work[s] = w / (double)hs.mols.size();
    }
    std::vector<int> rep_order(total_replicas);
    for (int g = 0; g < total_replicas; ++g)
        rep_order[g] = g;
    std::stable_sort(rep_order.begin(), rep_order.end(),
                     [&](int x, int y) { return sim_work[rep_sim[x]] > sim_work[rep_sim[y]]; });

    int rc = 0;
    rc |= d_sims.upload(h_sims);
    rc |= d_rep_sim.upload(rep_sim);
    rc |= d_rep_order.upload(rep_order);
    rc |= d_mols.upload(h_mols);
    rc |= d_rstat.upload(rstat);
    rc |= d_rqpos.upload(rqpos);
    rc |= d_rexcl.upload(rexcl);
    rc |= d_bonds.upload(bonds);
    rc |= d_indsub.upload(indsub);
    rc |= d_angles.upload(angles);
    rc |= d_tors.upload(tors);
    rc |= d_torsV.upload(torsVv);
    rc |= d_torsS.upload(torsSv);
    rc |= d_flexres.upload(flexres);
    rc |= d_flexopt.upload(flexopt);
    rc |= d_branch.upload(branch);
    rc |= d_localres.upload(localres);
    rc |= d_crankres.upload(crankres);
    rc |= d_tiles.upload(tiles);
    rc |= d_table.upload(table);
    rc |= d_pos.upload(pos);
    rc |= d_rel.upload(rel);
    rc |= d_center.upload(center);
    rc |= d_emat.zero((size_t)emat_off);
    rc |= d_intra.zero((size_t)molst_off);
    rc |= d_potential.zero((size_t)total_replicas);
    rc |= d_scratch_pot.zero((size_t)total_replicas);
    rc |= d_temperature.upload(temperature);
    rc |= d_tstep.upload(tstep);
    rc |= d_rstep.upload(rstep);
    rc |= d_stepc.zero((size_t)total_replicas);
    rc |= d_pairc.zero((size_t)total_replicas);
    rc |= d_stats.zero((size_t)total_replicas);
    rc |= d_tindex.upload(tindex);
    rc |= d_label.upload(label);
    rc |= d_slot_of_t.upload(slot_of_t);
    rc |= d_sim_state.upload(sim_state);
    rc |= d_errflags.zero((size_t)total_replicas);
    report_capacity = 0;
    return rc ? -1 : 0;
}

// ------------------------------------------------------------------ launch shape

// CTAs per replica C and threads per CTA T; the state is kept in shared memory when the
// per-CTA footprint stays under 210 KB.
static void configure_shape(cgppd_engine *e, int C, int T)
{
    e->cluster = C;
    e->threads = T;
    const int da = e->da;
    const size_t s_res = engine_smem_bytes(e->max_mol, e->max_n, e->max_m, C, 1, e->any_flexible, da, e->lmax);
    const size_t s_da = da ? s_res - engine_smem_bytes(e->max_mol, e->max_n, e->max_m, C, 1, e->any_flexible, 0, e->lmax) : 0;
    e->resident = (e->resident_pref != 0) && s_res <= 210 * 1024 + s_da && s_res <= 226 * 1024;
    e->smem = engine_smem_bytes(e->max_mol, e->max_n, e->max_m, C, e->resident, e->any_flexible, da, e->lmax);
}

// Autotuner: time k_mc for each candidate launch shape on scratch copies of the mutable
// state (the real trajectory is not advanced) and keep the fastest.  Results are cached
// per system shape for the life of the process and, when the environment variable
// CGPPD_TUNING_CACHE names a file, persisted there as JSON lines (one object per tuned
// shape, with the device name and SM count) so that later processes on the same kind
// of GPU skip the sweep.
static std::mutex g_tune_mu;

static std::string device_tag()
{
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p{};
    cudaGetDeviceProperties(&p, dev);
    char buf[320];
    std::snprintf(buf, sizeof(buf), "%s/%d", p.name, p.multiProcessorCount);
    std::string s = buf;
    for (char &c : s)
        if (c == '"' || c == '\\')
            c = '_';
    return s;
}

static void tune_cache_load(std::map<std::vector<long long>, std::pair<int, int>> &cache)
{
    const char *path = std::getenv("CGPPD_TUNING_CACHE");
    if (!path)
        return;
    FILE *f = std::fopen(path, "r");
    if (!f)
        return;
    const std::string dev = device_tag();
    char line[8192];
    while (std::fgets(line, sizeof(line), f)) {
        const char *d = std::strstr(line, "\"device\":\""), *k = std::strstr(line, "\"key\":[");
        const char *c = std::strstr(line, "\"cluster\":"), *t = std::strstr(line, "\"threads\":");
        if (!d || !k || !c || !t)
            continue;
        d += 10;
        const char *de = std::strchr(d, '"');
        if (!de || std::string(d, de) != dev)
            continue;
        std::vector<long long> key;
        const char *q = k + 7;
        while (*q && *q != ']') {
            char *end = nullptr;
            const long long v = std::strtoll(q, &end, 10);
            if (end == q)
                break;
            key.push_back(v);
            q = end;
            if (*q == ',')
                ++q;
        }
        const int C = std::atoi(c + 10), T = std::atoi(t + 10);
        if (!key.empty() && C > 0 && T > 0)
            cache[key] = std::make_pair(C, T);
    }
    std::fclose(f);
}

static void tune_cache_store(const std::vector<long long> &key, int C, int T)
{
    const char *path = std::getenv("CGPPD_TUNING_CACHE");
    if (!path)
        return;
    FILE *f = std::fopen(path, "a");
    if (!f)
        return;
    std::fprintf(f, "{\"format\":1,\"device\":\"%s\",\"key\":[", device_tag().c_str());
    for (size_t i = 0; i < key.size(); ++i)
        std::fprintf(f, "%s%lld", i ? "," : "", key[i]);
    std::fprintf(f, "],\"cluster\":%d,\"threads\":%d}\n", C, T);
    std::fclose(f);
}

static int autotune(cgppd_engine *e, int fixed_cluster, int fixed_threads)
{
    static std::map<std::vector<long long>, std::pair<int, int>> cache;
    static bool loaded = false;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (!loaded) {
        tune_cache_load(cache);
        loaded = true;
    }
    std::vector<long long> key{e->total_replicas, e->max_n, e->max_m, e->max_mol, e->any_flexible, e->resident_pref,
                               fixed_cluster, fixed_threads, e->da};
    for (const auto &s : e->h_sims)
        key.push_back(((long long)s.N << 32) | ((long long)s.M << 16) | s.R);
    auto hit = cache.find(key);
    if (hit != cache.end()) {
        configure_shape(e, hit->second.first, hit->second.second);
        return 0;
    }
    DevBuf<float4> pos, rel, cen;
    DevBuf<double> em, in, pot;
    DevBuf<ReplicaStats> st;
    DevBuf<unsigned long long> sc, pc;
    DevBuf<unsigned> ef;
    auto clone = [](auto &dst, const auto &src) {
        if (dst.alloc(src.n) != 0)
            return -1;
        return cgppd_check(cudaMemcpy(dst.ptr, src.ptr, src.n * sizeof(*src.ptr), cudaMemcpyDeviceToDevice),
                           "autotune copy");
    };
    if (clone(pos, e->d_pos) || clone(rel, e->d_rel) || clone(cen, e->d_center) || clone(em, e->d_emat) ||
        clone(in, e->d_intra) || clone(pot, e->d_potential) || clone(st, e->d_stats) || clone(sc, e->d_stepc) ||
        clone(pc, e->d_pairc) || clone(ef, e->d_errflags))
        return -1;
    DevBuf<DAStats> das;
    if (e->da && clone(das, e->d_dastats))
        return -1;
    EngineArgs base = e->args();
    base.pos = pos.ptr, base.rel = rel.ptr, base.center = cen.ptr, base.emat = em.ptr, base.intra = in.ptr;
    base.potential = pot.ptr, base.stats = st.ptr, base.stepc = sc.ptr, base.pairc = pc.ptr, base.errflags = ef.ptr;
    base.sample_log = nullptr;  // timing launches record no samples
    base.sample_xyz = nullptr;
    if (e->da)
        base.dastats = das.ptr;
    // the clones back to the engine's state (on the engine's stream, before a timed launch)
    auto restore = [&]() -> int {
        auto back = [&](auto &dst, const auto &src) {
            return cudaMemcpyAsync(dst.ptr, src.ptr, src.n * sizeof(*src.ptr), cudaMemcpyDeviceToDevice, e->own_stream);
        };
        cudaError_t err = cudaSuccess;
        for (cudaError_t r : {back(pos, e->d_pos), back(rel, e->d_rel), back(cen, e->d_center), back(em, e->d_emat),
                              back(in, e->d_intra), back(pot, e->d_potential), back(st, e->d_stats),
                              back(sc, e->d_stepc), back(pc, e->d_pairc), back(ef, e->d_errflags)})
            if (err == cudaSuccess)
                err = r;
        if (err == cudaSuccess && e->da)
            err = back(das, e->d_dastats);
        return cgppd_check(err, "autotune restore");
    };
    const int clusters[8] = {1, 2, 3, 4, 5, 6, 8, 16}, thread_opts[3] = {128, 256, 512};
    const int steps = 16;
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    float best = 1e30f;
    int bc = e->da ? 8 : 1, bt = 256;
    e->tuning.clear();
    for (int C : clusters) {
        if (fixed_cluster > 0 && C != fixed_cluster)
            continue;
        if (e->da && (C < 4 || 256 % C != 0))  // the surrogate's 256 units split evenly over 4, 8 or 16 CTAs
            continue;
        for (int T : thread_opts) {
            if (fixed_threads > 0 && T != fixed_threads)
                continue;
            configure_shape(e, C, T);
            if (e->smem > 227 * 1024 || set_mc_smem_limit(e->smem) != cudaSuccess)
                continue;
            EngineArgs a = base;
            a.cluster = C;
            a.resident = e->resident;
            if (launch_mc_block(a, e->total_replicas, 4, T, e->smem, e->own_stream) != cudaSuccess) {
                cudaGetLastError();  // a shape the device cannot schedule: skip it
                continue;
            }
            // the marginal cost of a step: launches of n and 2n steps (n sized so that one
            // takes about 2 ms after a short probe), each the faster of two, differenced so
            // that the per-launch set-up (state load and write-back) drops out.  Every timed
            // launch starts from the same copy of the state, so every shape is timed on the
            // same moves (a step's cost varies several-fold with the molecule it moves).
            auto time_launch = [&](int n_steps, float &ms_out) -> bool {
                if (restore() != 0)
                    return false;
                cudaEventRecord(ev0, e->own_stream);
                cudaError_t err = launch_mc_block(a, e->total_replicas, n_steps, T, e->smem, e->own_stream);
                cudaEventRecord(ev1, e->own_stream);
                if (err != cudaSuccess || cudaEventSynchronize(ev1) != cudaSuccess) {
                    cudaGetLastError();
                    return false;
                }
                cudaEventElapsedTime(&ms_out, ev0, ev1);
                return true;
            };
            float probe = 0.f;
            if (!time_launch(steps, probe))
                continue;
            const float probe_us = 1000.f * probe / steps;
            const int n = std::max(steps, std::min(2048, (int)(2000.f / std::max(probe_us, 1e-3f))));
            float t1 = 1e30f, t2 = 1e30f;
            bool ok = true;
            for (int rep = 0; rep < 2 && ok; ++rep) {
                float u = 0.f, v = 0.f;
                ok = time_launch(n, u) && time_launch(2 * n, v);
                t1 = std::min(t1, u);
                t2 = std::min(t2, v);
            }
            if (!ok)
                continue;
            // (a difference swamped by noise falls back to the plain per-step time)
            const float us = (t2 > t1) ? 1000.f * (t2 - t1) / n : 1000.f * t2 / (2 * n);
            e->tuning.push_back({C, T, us});
            if (us < best * 0.995f) {  // ties (within timing noise) keep the smaller shape
                best = us;
                bc = C;
                bt = T;
            }
        }
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "autotune") != 0)
        return -1;
    configure_shape(e, bc, bt);
    cache[key] = std::make_pair(bc, bt);
    tune_cache_store(key, bc, bt);
    return 0;
}

// ------------------------------------------------------------------ C ABI

extern "C" {

cgppd_engine *cgppd_engine_create(const float *lj_raw, int ntypes, const double *torsion_V,
                                  const double *torsion_phase, int torsion_types, uint64_t seed)
{
    if (lj_raw == nullptr || ntypes <= 0 || ntypes > 32) {
        cgppd_fail("cgppd_engine_create: the contact table must have 1..32 types");
        return nullptr;
    }
    auto *e = new cgppd_engine();
    e->ntypes = ntypes;
    e->seed = seed;
    e->table.assign(32 * 32, 0.0f);
    // Eij = lambda (e_ij - e0) in RT units, as the reference forms it in float
    // (src/Potential.cpp:14), then in kcal/mol.
    for (int i = 0; i < ntypes; ++i)
        for (int j = 0; j < ntypes; ++j)
            e->table[i * 32 + j] = -4.0f * ((kLambda * (lj_raw[i * ntypes + j] - kE0)) * kRTtoKcal);
    if (torsion_V && torsion_phase && torsion_types > 0) {
        e->tors_types = torsion_types;
        e->torsV.assign(torsion_V, torsion_V + 4 * torsion_types * torsion_types);
        e->torsS.assign(torsion_phase, torsion_phase + 4 * torsion_types * torsion_types);
    }
    return e;
}

void cgppd_engine_destroy(cgppd_engine *e) { delete e; }

int cgppd_engine_add_simulation(cgppd_engine *e, const cgppd_sim_params *p)
{
    if (e->finalized)
        return cgppd_fail("cgppd_engine_add_simulation: engine already finalized");
    if (p->n_replicas <= 0 || !p->temperatures || !p->translate_steps || !p->rotate_steps)
        return cgppd_fail("cgppd_engine_add_simulation: replica ladders are required");
    HostSim hs;
    hs.p = *p;
    hs.temps.assign(p->temperatures, p->temperatures + p->n_replicas);
    hs.tsteps.assign(p->translate_steps, p->translate_steps + p->n_replicas);
    hs.rsteps.assign(p->rotate_steps, p->rotate_steps + p->n_replicas);
    hs.p.temperatures = nullptr;
    hs.p.translate_steps = nullptr;
    hs.p.rotate_steps = nullptr;
    e->sims.push_back(hs);
    return (int)e->sims.size() - 1;
}

int cgppd_engine_add_molecule(cgppd_engine *e, int sim, int n, const float *xyz, const int *types,
                              const float *charges, const float *radii, const char *chain_ids,
                              const int *res_seq, const int *chain_index, int num_chains, int all_flexible,
                              int crowder, int n_segments, const int *seg_lengths, const int *seg_residues,
                              const float *center)
{
    if (e->finalized || sim < 0 || sim >= (int)e->sims.size() || n <= 0)
        return cgppd_fail("cgppd_engine_add_molecule: bad arguments");
    if (n > 65535)
        return cgppd_fail("cgppd_engine_add_molecule: a molecule holds at most 65535 residues");
    HostMolecule m;
    m.n = n;
    m.xyz.assign(xyz, xyz + 3 * n);
    m.types.assign(types, types + n);
    m.charges.assign(charges, charges + n);
    m.radii.assign(radii, radii + n);
    m.chain_ids.assign(chain_ids, chain_ids + n);
    m.res_seq.assign(res_seq, res_seq + n);
    m.chain_index.assign(chain_index, chain_index + n);
    m.num_chains = num_chains > 0 ? num_chains : 1;
    m.all_flexible = all_flexible != 0;
    m.crowder = crowder != 0;
    int off = 0;
    for (int k = 0; k < n_segments; ++k) {
        std::vector<int> seg(seg_residues + off, seg_residues + off + seg_lengths[k]);
        for (int v : seg)
            if (v < 0 || v >= n)
                return cgppd_fail("cgppd_engine_add_molecule: segment residue out of range");
        m.segments.push_back(seg);
        off += seg_lengths[k];
    }
    if (center) {
        std::memcpy(m.center, center, sizeof(m.center));
    } else {
        // float accumulation then division, as Molecule::initFromPDB (src/Molecule.cpp:590-604)
        float c[3] = {0, 0, 0};
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                c[k] += xyz[3 * i + k];
        for (int k = 0; k < 3; ++k)
            m.center[k] = c[k] / (float)n;
    }
    m.rel.resize(3 * n);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k)
            m.rel[3 * i + k] = xyz[3 * i + k] - m.center[k];
    e->sims[sim].mols.push_back(m);
    return (int)e->sims[sim].mols.size() - 1;
}

int cgppd_engine_finalize(cgppd_engine *e, int cluster, int threads)
{
    if (e->finalized)
        return 0;
    if (e->sims.empty())
        return cgppd_fail("cgppd_engine_finalize: no simulation");
    if (e->build() != 0)
        return -1;
    const bool tune = cluster <= 0 || threads <= 0;
    configure_shape(e, std::min(16, std::max(1, cluster > 0 ? cluster : 1)),
                    threads == 128 ? 128 : threads == 512 ? 512 : 256);
    const size_t s_init = engine_smem_bytes(e->max_mol, e->max_n, e->max_m, 1, 0, e->any_flexible, 0, nullptr);
    if (std::max(e->smem, s_init) > 227 * 1024)
        return cgppd_fail("cgppd_engine_finalize: system too large for shared memory (reduce molecule size or N)");
    if (cgppd_check(set_mc_smem_limit(std::max(e->smem, s_init)), "engine shared-memory limit") != 0)
        return -1;
    if (cgppd_check(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking), "engine stream") != 0)
        return -1;
    EngineArgs a = e->args();
    if (cgppd_check(launch_init_energy(a, e->total_replicas, s_init, e->d_potential.ptr, e->own_stream),
                    "initial energy") != 0)
        return -1;
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "initial energy") != 0)
        return -1;
    if (tune && autotune(e, cluster, threads) != 0)
        return -1;
    if (e->d_sim_da.zero(e->sims.size()) != 0 || e->d_dastats.zero((size_t)e->total_replicas) != 0)
        return -1;
    e->plain_cluster = e->cluster;
    e->plain_threads = e->threads;
    e->finalized = true;
    return 0;
}

int cgppd_engine_tuning(const cgppd_engine *e, int *n, int *clusters, int *threads, float *us_per_step)
{
    const int k = (int)e->tuning.size();
    for (int i = 0; i < k && i < *n; ++i) {
        clusters[i] = e->tuning[i].cluster;
        threads[i] = e->tuning[i].threads;
        us_per_step[i] = e->tuning[i].us_per_step;
    }
    *n = k;
    return 0;
}

static int ensure_reports(cgppd_engine *e, int rows)
{
    if (rows <= e->report_capacity)
        return 0;
    // keep existing rows
    const int cap = std::max(rows, 2 * e->report_capacity);
    DevBuf<float4> nr;
    DevBuf<int2> ne;
    if (nr.zero((size_t)cap * e->total_replicas) != 0 || ne.zero((size_t)cap * e->sims.size()) != 0)
        return -1;
    if (e->report_capacity > 0) {
        cudaMemcpy(nr.ptr, e->d_report.ptr, sizeof(float4) * (size_t)e->report_capacity * e->total_replicas,
                   cudaMemcpyDeviceToDevice);
        cudaMemcpy(ne.ptr, e->d_exch_report.ptr, sizeof(int2) * (size_t)e->report_capacity * e->sims.size(),
                   cudaMemcpyDeviceToDevice);
    }
    std::swap(e->d_report.ptr, nr.ptr);
    std::swap(e->d_report.n, nr.n);
    std::swap(e->d_exch_report.ptr, ne.ptr);
    std::swap(e->d_exch_report.n, ne.n);
    e->report_capacity = cap;
    for (auto &kv : e->graphs)  // graphs captured the old buffer pointers
        cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
    return 0;
}

static int exchanges_done(cgppd_engine *e)
{
    int st[4] = {0, 0, 0, 0};
    cudaMemcpy(st, e->d_sim_state.ptr, sizeof(st), cudaMemcpyDeviceToHost);
    return st[1];
}

int cgppd_engine_run(cgppd_engine *e, int n_blocks, int steps_per_block, int exchange_after_last, void *stream)
{
    if (!e->finalized)
        return cgppd_fail("cgppd_engine_run: engine not finalized");
    if (n_blocks <= 0 || steps_per_block <= 0)
        return 0;
    cudaStream_t st = stream ? (cudaStream_t)stream : e->own_stream;
    // report rows: one per exchange (+1 for a closing report)
    const int need = exchanges_done(e) + n_blocks + 1;
    if (ensure_reports(e, need) != 0)
        return -1;
    EngineArgs a = e->args();
    const int nsims = (int)e->sims.size();
    int launches = 0;
    for (int b = 0; b < n_blocks; ++b) {
        const bool exch = (b + 1 < n_blocks) || exchange_after_last;
        const auto key = std::make_pair(steps_per_block, exch ? 1 : 0);
        auto it = e->graphs.find(key);
        if (it == e->graphs.end()) {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            if (cgppd_check(cudaStreamBeginCapture(e->own_stream, cudaStreamCaptureModeThreadLocal), "capture") != 0)
                return -1;
            cudaError_t err = launch_mc_block(a, e->total_replicas, steps_per_block, e->threads, e->smem, e->own_stream);
            if (err == cudaSuccess && exch)
                err = launch_exchange(a, nsims, e->total_replicas, steps_per_block, e->own_stream);
            cudaError_t err2 = cudaStreamEndCapture(e->own_stream, &g);
            if (cgppd_check(err, "MC block launch") != 0 || cgppd_check(err2, "end capture") != 0)
                return -1;
            if (cgppd_check(cudaGraphInstantiate(&ge, g, 0), "graph instantiate") != 0)
                return -1;
            cudaGraphDestroy(g);
            it = e->graphs.emplace(key, ge).first;
        }
        if (cgppd_check(cudaGraphLaunch(it->second, st), "graph launch") != 0)
            return -1;
        launches += exch ? 2 : 1;
    }
    e->last_launches = launches;
    return 0;
}

int cgppd_engine_final_report(cgppd_engine *e, int row, void *stream)
{
    if (ensure_reports(e, row + 1) != 0)
        return -1;
    cudaStream_t st = stream ? (cudaStream_t)stream : e->own_stream;
    return cgppd_check(launch_final_report(e->args(), (int)e->sims.size(), e->total_replicas, row, st),
                       "final report");
}

int cgppd_engine_synchronize(cgppd_engine *e)
{
    int rc = cgppd_check(cudaStreamSynchronize(e->own_stream), "engine synchronize");
    if (rc == 0)
        rc = cgppd_check(cudaDeviceSynchronize(), "engine synchronize");
    return rc;
}

int cgppd_engine_total_replicas(const cgppd_engine *e) { return e->total_replicas; }

int cgppd_engine_sim_info(const cgppd_engine *e, int sim, int *n_residues, int *n_molecules, int *n_replicas)
{
    if (sim < 0 || sim >= (int)e->sims.size())
        return cgppd_fail("cgppd_engine_sim_info: bad simulation index");
    int N = 0;
    for (auto &m : e->sims[sim].mols)
        N += m.n;
    if (n_residues)
        *n_residues = N;
    if (n_molecules)
        *n_molecules = (int)e->sims[sim].mols.size();
    if (n_replicas)
        *n_replicas = e->sims[sim].p.n_replicas;
    return 0;
}

int cgppd_engine_recompute(cgppd_engine *e, double *out, int write_state)
{
    if (!e->finalized)
        return cgppd_fail("cgppd_engine_recompute: engine not finalized");
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "recompute") != 0)
        return -1;
    EngineArgs a = e->args();
    const size_t s_init = engine_smem_bytes(e->max_mol, e->max_n, e->max_m, 1, 0, e->any_flexible, 0, nullptr);
    double *dst = write_state ? e->d_potential.ptr : e->d_scratch_pot.ptr;
    if (!write_state) {
        // evaluate into scratch copies so the running state is untouched
        if (e->d_scratch_emat.n < e->d_emat.n && e->d_scratch_emat.zero(e->d_emat.n) != 0)
            return -1;
        if (e->d_scratch_intra.n < e->d_intra.n && e->d_scratch_intra.zero(e->d_intra.n) != 0)
            return -1;
        a.emat = e->d_scratch_emat.ptr;
        a.intra = e->d_scratch_intra.ptr;
    }
    if (cgppd_check(launch_init_energy(a, e->total_replicas, s_init, dst, e->own_stream), "recompute") != 0)
        return -1;
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "recompute") != 0)
        return -1;
    if (out)
        return cgppd_check(cudaMemcpy(out, dst, sizeof(double) * e->total_replicas, cudaMemcpyDeviceToHost),
                           "recompute copy");
    return 0;
}

int cgppd_engine_get_replicas(cgppd_engine *e, int sim, double *potentials, float *temperatures, int *labels,
                              int *tindex, int *stats16)
{
    if (sim < 0 || sim >= (int)e->h_sims.size())
        return cgppd_fail("cgppd_engine_get_replicas: bad simulation index");
    cudaDeviceSynchronize();
    const DevSim &S = e->h_sims[sim];
    int rc = 0;
    if (potentials)
        rc |= cgppd_check(cudaMemcpy(potentials, e->d_potential.ptr + S.rep_off, sizeof(double) * S.R,
                                     cudaMemcpyDeviceToHost), "copy");
    if (temperatures)
        rc |= cgppd_check(cudaMemcpy(temperatures, e->d_temperature.ptr + S.rep_off, sizeof(float) * S.R,
                                     cudaMemcpyDeviceToHost), "copy");
    if (labels)
        rc |= cgppd_check(cudaMemcpy(labels, e->d_label.ptr + S.rep_off, sizeof(int) * S.R, cudaMemcpyDeviceToHost),
                          "copy");
    if (tindex)
        rc |= cgppd_check(cudaMemcpy(tindex, e->d_tindex.ptr + S.rep_off, sizeof(int) * S.R, cudaMemcpyDeviceToHost),
                          "copy");
    if (stats16) {
        static_assert(sizeof(ReplicaStats) == 64, "ReplicaStats is 16 words");
        rc |= cgppd_check(cudaMemcpy(stats16, e->d_stats.ptr + S.rep_off, sizeof(ReplicaStats) * S.R,
                                     cudaMemcpyDeviceToHost), "copy");
    }
    return rc ? -1 : 0;
}

int cgppd_engine_get_state(cgppd_engine *e, int sim, int replica, float *xyz, float *rel, float *centers)
{
    if (sim < 0 || sim >= (int)e->h_sims.size() || replica < 0 || replica >= e->h_sims[sim].R)
        return cgppd_fail("cgppd_engine_get_state: bad index");
    cudaDeviceSynchronize();
    const DevSim &S = e->h_sims[sim];
    std::vector<float4> buf(std::max(S.N, S.M));
    const long long off = S.state_off + (long long)replica * S.N;
    if (xyz) {
        if (cgppd_check(cudaMemcpy(buf.data(), e->d_pos.ptr + off, sizeof(float4) * S.N, cudaMemcpyDeviceToHost),
                        "copy") != 0)
            return -1;
        for (int i = 0; i < S.N; ++i)
            xyz[3 * i] = buf[i].x, xyz[3 * i + 1] = buf[i].y, xyz[3 * i + 2] = buf[i].z;
    }
    if (rel) {
        if (cgppd_check(cudaMemcpy(buf.data(), e->d_rel.ptr + off, sizeof(float4) * S.N, cudaMemcpyDeviceToHost),
                        "copy") != 0)
            return -1;
        for (int i = 0; i < S.N; ++i)
            rel[3 * i] = buf[i].x, rel[3 * i + 1] = buf[i].y, rel[3 * i + 2] = buf[i].z;
    }
    if (centers) {
        if (cgppd_check(cudaMemcpy(buf.data(), e->d_center.ptr + S.molst_off + (long long)replica * S.M,
                                   sizeof(float4) * S.M, cudaMemcpyDeviceToHost), "copy") != 0)
            return -1;
        for (int m = 0; m < S.M; ++m)
            centers[3 * m] = buf[m].x, centers[3 * m + 1] = buf[m].y, centers[3 * m + 2] = buf[m].z;
    }
    return 0;
}

int cgppd_engine_set_state(cgppd_engine *e, int sim, int replica, const float *xyz, const float *rel,
                           const float *centers)
{
    if (sim < 0 || sim >= (int)e->h_sims.size() || replica < 0 || replica >= e->h_sims[sim].R)
        return cgppd_fail("cgppd_engine_set_state: bad index");
    const DevSim &S = e->h_sims[sim];
    std::vector<float4> buf(std::max(S.N, S.M));
    const long long off = S.state_off + (long long)replica * S.N;
    int rc = 0;
    if (xyz) {
        for (int i = 0; i < S.N; ++i)
            buf[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.f);
        rc |= cgppd_check(cudaMemcpy(e->d_pos.ptr + off, buf.data(), sizeof(float4) * S.N, cudaMemcpyHostToDevice),
                          "copy");
    }
    if (rel) {
        for (int i = 0; i < S.N; ++i)
            buf[i] = make_float4(rel[3 * i], rel[3 * i + 1], rel[3 * i + 2], 0.f);
        rc |= cgppd_check(cudaMemcpy(e->d_rel.ptr + off, buf.data(), sizeof(float4) * S.N, cudaMemcpyHostToDevice),
                          "copy");
    }
    if (centers) {
        for (int m = 0; m < S.M; ++m)
            buf[m] = make_float4(centers[3 * m], centers[3 * m + 1], centers[3 * m + 2], 0.f);
        rc |= cgppd_check(cudaMemcpy(e->d_center.ptr + S.molst_off + (long long)replica * S.M, buf.data(),
                                     sizeof(float4) * S.M, cudaMemcpyHostToDevice), "copy");
    }
    return rc ? -1 : 0;
}

int cgppd_engine_upload(cgppd_engine *e, int sim, const float *pos4, const float *rel4, const float *centers4,
                        int recompute, void *stream)
{
    if (!e->finalized || sim < 0 || sim >= (int)e->h_sims.size())
        return cgppd_fail("cgppd_engine_upload: bad simulation index");
    const DevSim &S = e->h_sims[sim];
    cudaStream_t st = stream ? (cudaStream_t)stream : e->own_stream;
    const size_t nres = (size_t)S.N * S.R;
    int rc = 0;
    if (pos4)
        rc |= cgppd_check(cudaMemcpyAsync(e->d_pos.ptr + S.state_off, pos4, sizeof(float4) * nres,
                                          cudaMemcpyHostToDevice, st), "upload positions");
    if (rel4)
        rc |= cgppd_check(cudaMemcpyAsync(e->d_rel.ptr + S.state_off, rel4, sizeof(float4) * nres,
                                          cudaMemcpyHostToDevice, st), "upload relative positions");
    if (centers4)
        rc |= cgppd_check(cudaMemcpyAsync(e->d_center.ptr + S.molst_off, centers4, sizeof(float4) * S.M * S.R,
                                          cudaMemcpyHostToDevice, st), "upload centres");
    if (rc == 0 && recompute) {
        const size_t s_init = engine_smem_bytes(e->max_mol, e->max_n, e->max_m, 1, 0, e->any_flexible, 0, nullptr);
        rc |= cgppd_check(launch_init_energy(e->args(), e->total_replicas, s_init, e->d_potential.ptr, st),
                          "upload recompute");
    }
    return rc ? -1 : 0;
}

int cgppd_engine_download(cgppd_engine *e, int sim, float *pos4, float *rel4, float *centers4, double *potentials,
                          void *stream)
{
    if (!e->finalized || sim < 0 || sim >= (int)e->h_sims.size())
        return cgppd_fail("cgppd_engine_download: bad simulation index");
    const DevSim &S = e->h_sims[sim];
    cudaStream_t st = stream ? (cudaStream_t)stream : e->own_stream;
    const size_t nres = (size_t)S.N * S.R;
    int rc = 0;
    if (pos4)
        rc |= cgppd_check(cudaMemcpyAsync(pos4, e->d_pos.ptr + S.state_off, sizeof(float4) * nres,
                                          cudaMemcpyDeviceToHost, st), "download positions");
    if (rel4)
        rc |= cgppd_check(cudaMemcpyAsync(rel4, e->d_rel.ptr + S.state_off, sizeof(float4) * nres,
                                          cudaMemcpyDeviceToHost, st), "download relative positions");
    if (centers4)
        rc |= cgppd_check(cudaMemcpyAsync(centers4, e->d_center.ptr + S.molst_off, sizeof(float4) * S.M * S.R,
                                          cudaMemcpyDeviceToHost, st), "download centres");
    if (potentials)
        rc |= cgppd_check(cudaMemcpyAsync(potentials, e->d_potential.ptr + S.rep_off, sizeof(double) * S.R,
                                          cudaMemcpyDeviceToHost, st), "download potentials");
    return rc ? -1 : 0;
}

}  // extern "C"

// ---- checkpoint / restore: every mutable device buffer of the engine in one file.
// Layout: magic "CGPPDCK1", u64 fingerprint length + fingerprint (the system's shape),
// then for each buffer u64 byte count + bytes, in a fixed order.
static std::vector<long long> engine_fingerprint(const cgppd_engine *e)
{
    std::vector<long long> f{(long long)e->sims.size(), e->total_replicas, e->max_n, e->max_m};
    for (const auto &s : e->h_sims) {
        f.push_back(s.N);
        f.push_back(s.M);
        f.push_back(s.R);
    }
    for (const auto &m : e->h_mols) {
        f.push_back(m.start);
        f.push_back(m.count);
        f.push_back(m.flags);
    }
    return f;
}

template <typename F>
static int for_each_state_buffer(cgppd_engine *e, F &&f)
{
    int rc = 0;
    rc |= f(e->d_pos.ptr, e->d_pos.n * sizeof(float4));
    rc |= f(e->d_rel.ptr, e->d_rel.n * sizeof(float4));
    rc |= f(e->d_center.ptr, e->d_center.n * sizeof(float4));
    rc |= f(e->d_emat.ptr, e->d_emat.n * sizeof(double));
    rc |= f(e->d_intra.ptr, e->d_intra.n * sizeof(double));
    rc |= f(e->d_potential.ptr, e->d_potential.n * sizeof(double));
    rc |= f(e->d_temperature.ptr, e->d_temperature.n * sizeof(float));
    rc |= f(e->d_tstep.ptr, e->d_tstep.n * sizeof(float));
    rc |= f(e->d_rstep.ptr, e->d_rstep.n * sizeof(double));
    rc |= f(e->d_stepc.ptr, e->d_stepc.n * sizeof(unsigned long long));
    rc |= f(e->d_pairc.ptr, e->d_pairc.n * sizeof(unsigned long long));
    rc |= f(e->d_stats.ptr, e->d_stats.n * sizeof(ReplicaStats));
    rc |= f(e->d_tindex.ptr, e->d_tindex.n * sizeof(int));
    rc |= f(e->d_label.ptr, e->d_label.n * sizeof(int));
    rc |= f(e->d_slot_of_t.ptr, e->d_slot_of_t.n * sizeof(int));
    rc |= f(e->d_sim_state.ptr, e->d_sim_state.n * sizeof(int));
    rc |= f(e->d_errflags.ptr, e->d_errflags.n * sizeof(unsigned));
    rc |= f(e->d_dastats.ptr, e->d_dastats.n * sizeof(DAStats));
    rc |= f(e->d_sim_da.ptr, e->d_sim_da.n * sizeof(int));
    rc |= f(e->d_report.ptr, (size_t)e->report_capacity * e->total_replicas * sizeof(float4));
    rc |= f(e->d_exch_report.ptr, (size_t)e->report_capacity * e->sims.size() * sizeof(int2));
    return rc;
}

extern "C" int cgppd_engine_checkpoint(cgppd_engine *e, const char *path)
{
    if (!e || !e->finalized || !path)
        return cgppd_fail("cgppd_engine_checkpoint: engine not finalized or no path");
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "checkpoint") != 0 ||
        cgppd_check(cudaDeviceSynchronize(), "checkpoint") != 0)
        return -1;
    FILE *fp = std::fopen(path, "wb");
    if (!fp)
        return cgppd_fail("cgppd_engine_checkpoint: cannot open the file for writing");
    const std::vector<long long> fpr = engine_fingerprint(e);
    const uint64_t nf = fpr.size(), cap = (uint64_t)e->report_capacity;
    bool ok = std::fwrite("CGPPDCK1", 1, 8, fp) == 8 && std::fwrite(&nf, 8, 1, fp) == 1 &&
              std::fwrite(fpr.data(), sizeof(long long), nf, fp) == nf && std::fwrite(&cap, 8, 1, fp) == 1;
    std::vector<unsigned char> host;
    const int rc = for_each_state_buffer(e, [&](void *dptr, size_t bytes) -> int {
        const uint64_t nb = bytes;
        if (!ok || std::fwrite(&nb, 8, 1, fp) != 1) {
            ok = false;
            return -1;
        }
        if (bytes == 0)
            return 0;
        host.resize(bytes);
        if (cgppd_check(cudaMemcpy(host.data(), dptr, bytes, cudaMemcpyDeviceToHost), "checkpoint copy") != 0)
            return -1;
        if (std::fwrite(host.data(), 1, bytes, fp) != bytes) {
            ok = false;
            return -1;
        }
        return 0;
    });
    ok = (std::fclose(fp) == 0) && ok;
    if (rc != 0 || !ok)
        return cgppd_fail("cgppd_engine_checkpoint: write failed");
    return 0;
}

extern "C" int cgppd_engine_restore(cgppd_engine *e, const char *path)
{
    if (!e || !e->finalized || !path)
        return cgppd_fail("cgppd_engine_restore: engine not finalized or no path");
    if (cgppd_check(cudaDeviceSynchronize(), "restore") != 0)
        return -1;
    FILE *fp = std::fopen(path, "rb");
    if (!fp)
        return cgppd_fail("cgppd_engine_restore: cannot open the file");
    char magic[8];
    uint64_t nf = 0, cap = 0;
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, "CGPPDCK1", 8) == 0 &&
              std::fread(&nf, 8, 1, fp) == 1 && nf < (1u << 26);
    std::vector<long long> fpr(ok ? nf : 0);
    ok = ok && std::fread(fpr.data(), sizeof(long long), nf, fp) == nf && std::fread(&cap, 8, 1, fp) == 1;
    if (!ok || fpr != engine_fingerprint(e)) {
        std::fclose(fp);
        return cgppd_fail("cgppd_engine_restore: not a checkpoint of an engine with this system");
    }
    if (cap > (uint64_t)e->report_capacity && ensure_reports(e, (int)cap) != 0) {
        std::fclose(fp);
        return -1;
    }
    std::vector<unsigned char> host;
    const int saved_cap = e->report_capacity;
    e->report_capacity = (int)cap;  // the report buffers are read for the saved rows only
    const int rc = for_each_state_buffer(e, [&](void *dptr, size_t bytes) -> int {
        uint64_t nb = 0;
        if (!ok || std::fread(&nb, 8, 1, fp) != 1 || nb != bytes) {
            ok = false;
            return -1;
        }
        if (bytes == 0)
            return 0;
        host.resize(bytes);
        if (std::fread(host.data(), 1, bytes, fp) != bytes) {
            ok = false;
            return -1;
        }
        return cgppd_check(cudaMemcpy(dptr, host.data(), bytes, cudaMemcpyHostToDevice), "restore copy");
    });
    e->report_capacity = saved_cap;
    std::fclose(fp);
    if (rc != 0 || !ok)
        return cgppd_fail("cgppd_engine_restore: truncated or mismatched checkpoint");
    // rows past the checkpoint's capacity held this engine's earlier run: clear them, as
    // in the engine that wrote the checkpoint (report rows start zeroed)
    if ((int)cap < e->report_capacity) {
        const size_t rows = (size_t)(e->report_capacity - (int)cap);
        if (cgppd_check(cudaMemset(e->d_report.ptr + cap * e->total_replicas, 0,
                                   sizeof(float4) * rows * e->total_replicas), "restore clear") != 0 ||
            cgppd_check(cudaMemset(e->d_exch_report.ptr + cap * e->sims.size(), 0,
                                   sizeof(int2) * rows * e->sims.size()), "restore clear") != 0)
            return -1;
    }
    return 0;
}

extern "C" {

int cgppd_engine_get_matrix(cgppd_engine *e, int sim, int replica, double *E, double *intra)
{
    if (sim < 0 || sim >= (int)e->h_sims.size() || replica < 0 || replica >= e->h_sims[sim].R)
        return cgppd_fail("cgppd_engine_get_matrix: bad index");
    cudaDeviceSynchronize();
    const DevSim &S = e->h_sims[sim];
    int rc = 0;
    if (E)
        rc |= cgppd_check(cudaMemcpy(E, e->d_emat.ptr + S.emat_off + (long long)replica * S.M * S.M,
                                     sizeof(double) * S.M * S.M, cudaMemcpyDeviceToHost), "copy");
    if (intra)
        rc |= cgppd_check(cudaMemcpy(intra, e->d_intra.ptr + S.molst_off + (long long)replica * S.M,
                                     sizeof(double) * S.M, cudaMemcpyDeviceToHost), "copy");
    return rc ? -1 : 0;
}

int cgppd_engine_get_report(cgppd_engine *e, int sim, int row, float *per_temperature4, int *exch2)
{
    if (sim < 0 || sim >= (int)e->h_sims.size() || row < 0 || row >= e->report_capacity)
        return cgppd_fail("cgppd_engine_get_report: bad index");
    cudaDeviceSynchronize();
    const DevSim &S = e->h_sims[sim];
    int rc = 0;
    if (per_temperature4)
        rc |= cgppd_check(cudaMemcpy(per_temperature4, e->d_report.ptr + (long long)row * e->total_replicas + S.rep_off,
                                     sizeof(float4) * S.R, cudaMemcpyDeviceToHost), "copy");
    if (exch2)
        rc |= cgppd_check(cudaMemcpy(exch2, e->d_exch_report.ptr + (long long)row * e->sims.size() + sim, sizeof(int2),
                                     cudaMemcpyDeviceToHost), "copy");
    return rc ? -1 : 0;
}

int cgppd_engine_set_sample_log(cgppd_engine *e, int per_replica)
{
    if (!e || !e->finalized || per_replica < 0)
        return cgppd_fail("cgppd_engine_set_sample_log: engine not finalized or negative capacity");
    if (cgppd_check(cudaDeviceSynchronize(), "sample log") != 0)
        return -1;
    e->sample_cap = 0;
    e->d_sample_log.release();
    e->d_sample_xyz.release();
    if (per_replica > 0) {
        if (e->d_sample_log.alloc((size_t)per_replica * e->total_replicas) != 0 ||
            e->d_sample_count.zero((size_t)e->total_replicas) != 0 ||
            (e->sample_nres > 0 &&
             e->d_sample_xyz.alloc((size_t)per_replica * e->total_replicas * e->sample_nres) != 0))
            return -1;
        e->sample_cap = per_replica;
    }
    for (auto &kv : e->graphs)  // graphs captured the old arguments
        cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
    return 0;
}

int cgppd_engine_set_sample_snapshots(cgppd_engine *e, int residues)
{
    if (!e || !e->finalized || residues < 0)
        return cgppd_fail("cgppd_engine_set_sample_snapshots: engine not finalized or negative residue count");
    if (cgppd_check(cudaDeviceSynchronize(), "sample snapshots") != 0)
        return -1;
    e->d_sample_xyz.release();
    e->sample_nres = 0;
    if (residues > 0 && e->sample_cap > 0 &&
        e->d_sample_xyz.alloc((size_t)e->sample_cap * e->total_replicas * residues) != 0)
        return -1;
    e->sample_nres = residues;
    for (auto &kv : e->graphs)  // graphs captured the old arguments
        cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
    return 0;
}

int cgppd_engine_take_sample_xyz(cgppd_engine *e, int sim, float *xyz)
{
    if (!e || sim < 0 || sim >= (int)e->h_sims.size() || !xyz)
        return cgppd_fail("cgppd_engine_take_sample_xyz: bad simulation index or output");
    if (e->sample_cap <= 0 || e->sample_nres <= 0)
        return 0;
    if (cgppd_check(cudaDeviceSynchronize(), "take sample coordinates") != 0)
        return -1;
    const DevSim &S = e->h_sims[sim];
    const size_t n = (size_t)S.R * e->sample_cap * e->sample_nres;
    std::vector<float4> h(n);
    if (cgppd_check(cudaMemcpy(h.data(), e->d_sample_xyz.ptr + (size_t)S.rep_off * e->sample_cap * e->sample_nres,
                               sizeof(float4) * n, cudaMemcpyDeviceToHost),
                    "take sample coordinates") != 0)
        return -1;
    for (size_t i = 0; i < n; ++i) {
        xyz[3 * i] = h[i].x;
        xyz[3 * i + 1] = h[i].y;
        xyz[3 * i + 2] = h[i].z;
    }
    return 0;
}

int cgppd_engine_take_samples(cgppd_engine *e, int sim, int *counts, double *enc, double *potential,
                              float *temperature, int *step)
{
    if (!e || sim < 0 || sim >= (int)e->h_sims.size())
        return cgppd_fail("cgppd_engine_take_samples: bad simulation index");
    const DevSim &S = e->h_sims[sim];
    if (e->sample_cap <= 0) {
        for (int r = 0; r < S.R; ++r)
            counts[r] = 0;
        return 0;
    }
    if (cgppd_check(cudaDeviceSynchronize(), "take samples") != 0)
        return -1;
    std::vector<unsigned> cnt(S.R);
    std::vector<SampleRec> rec((size_t)S.R * e->sample_cap);
    if (cgppd_check(cudaMemcpy(cnt.data(), e->d_sample_count.ptr + S.rep_off, sizeof(unsigned) * S.R,
                               cudaMemcpyDeviceToHost), "take samples") != 0 ||
        cgppd_check(cudaMemcpy(rec.data(), e->d_sample_log.ptr + (size_t)S.rep_off * e->sample_cap,
                               sizeof(SampleRec) * rec.size(), cudaMemcpyDeviceToHost), "take samples") != 0 ||
        cgppd_check(cudaMemset(e->d_sample_count.ptr + S.rep_off, 0, sizeof(unsigned) * S.R), "take samples") != 0)
        return -1;
    for (int r = 0; r < S.R; ++r) {
        counts[r] = (int)cnt[r];
        for (unsigned k = 0; k < cnt[r]; ++k) {
            const SampleRec &x = rec[(size_t)r * e->sample_cap + k];
            const size_t o = (size_t)r * e->sample_cap + k;
            if (enc)
                enc[o] = x.enc;
            if (potential)
                potential[o] = x.potential;
            if (temperature)
                temperature[o] = x.temperature;
            if (step)
                step[o] = x.step;
        }
    }
    return 0;
}

int cgppd_engine_counters(cgppd_engine *e, unsigned long long *mc_steps, unsigned long long *pair_evals)
{
    cudaDeviceSynchronize();
    std::vector<unsigned long long> a(e->total_replicas), b(e->total_replicas);
    if (cgppd_check(cudaMemcpy(a.data(), e->d_stepc.ptr, sizeof(unsigned long long) * a.size(), cudaMemcpyDeviceToHost),
                    "copy") != 0 ||
        cgppd_check(cudaMemcpy(b.data(), e->d_pairc.ptr, sizeof(unsigned long long) * b.size(), cudaMemcpyDeviceToHost),
                    "copy") != 0)
        return -1;
    unsigned long long sa = 0, sb = 0;
    for (size_t i = 0; i < a.size(); ++i)
        sa += a[i], sb += b[i];
    if (mc_steps)
        *mc_steps = sa;
    if (pair_evals)
        *pair_evals = sb;
    return 0;
}

unsigned cgppd_engine_error_bits(cgppd_engine *e)
{
    cudaDeviceSynchronize();
    std::vector<unsigned> f(e->total_replicas);
    cudaMemcpy(f.data(), e->d_errflags.ptr, sizeof(unsigned) * f.size(), cudaMemcpyDeviceToHost);
    unsigned o = 0;
    for (unsigned v : f)
        o |= v;
    return o;
}

int cgppd_engine_replica_error_bits(cgppd_engine *e, int sim, unsigned *out)
{
    if (!e->finalized || sim < 0 || sim >= (int)e->h_sims.size() || !out)
        return cgppd_fail("cgppd_engine_replica_error_bits: bad index");
    const DevSim &S = e->h_sims[sim];
    if (cgppd_check(cudaDeviceSynchronize(), "replica error bits") != 0)
        return -1;
    return cgppd_check(cudaMemcpy(out, e->d_errflags.ptr + S.rep_off, sizeof(unsigned) * S.R, cudaMemcpyDeviceToHost),
                       "replica error bits");
}

int cgppd_engine_last_launches(const cgppd_engine *e) { return e->last_launches; }

int cgppd_engine_set_resident(cgppd_engine *e, int allow)
{
    if (e->finalized)
        return cgppd_fail("cgppd_engine_set_resident: engine already finalized");
    e->resident_pref = allow ? 1 : 0;
    return 0;
}

int cgppd_engine_launch_shape(const cgppd_engine *e, int *cluster, int *threads)
{
    if (cluster)
        *cluster = e->cluster;
    if (threads)
        *threads = e->threads;
    return e->resident;
}

}  // extern "C"

// ------------------------------------------------------------------ learned surrogate

// Every molecule a rigid, non-crowder copy of the first (count, types, charges, radii and
// frame residues), 2..64 molecules of at least 3 residues.
static bool sim_compatible(const cgppd_engine *e, int sim)
{
    const HostSim &hs = e->sims[sim];
    const int M = (int)hs.mols.size();
    if (M < 2 || M > 64)
        return false;
    const HostMolecule &m0 = hs.mols[0];
    const int mol_off = e->h_sims[sim].mol_off;
    const DevMol &d0 = e->h_mols[mol_off];
    if (m0.n < 3)
        return false;
    for (int k = 0; k < M; ++k) {
        const HostMolecule &mk = hs.mols[k];
        const DevMol &dk = e->h_mols[mol_off + k];
        if (mk.crowder || (dk.flags & kMolFlexible))
            return false;
        if (mk.n != m0.n || mk.types != m0.types || mk.charges != m0.charges || mk.radii != m0.radii)
            return false;
        if (dk.fr0 != d0.fr0 || dk.fr1 != d0.fr1 || dk.fr2 != d0.fr2)
            return false;
    }
    return true;
}

extern "C" {

int cgppd_engine_surrogate_compatible(cgppd_engine *e, int sim)
{
    if (!e || !e->finalized || sim < 0 || sim >= (int)e->sims.size())
        return cgppd_fail("cgppd_engine_surrogate_compatible: bad engine or simulation index");
    return sim_compatible(e, sim) ? 1 : 0;
}

int cgppd_engine_set_surrogate(cgppd_engine *e, cgppd_surrogate *s, float rmse_threshold, float error_window,
                               int min_evals)
{
    if (!e || !e->finalized)
        return cgppd_fail("cgppd_engine_set_surrogate: engine not finalized");
    if (s && (!(rmse_threshold > 0.f) || !(error_window > 0.f) || min_evals < 1))
        return cgppd_fail("cgppd_engine_set_surrogate: threshold and window must be positive, min_evals >= 1");
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "set surrogate") != 0)
        return -1;
    std::vector<int> on(e->sims.size(), 0);
    int count = 0;
    if (s)
        for (size_t k = 0; k < e->sims.size(); ++k) {
            on[k] = sim_compatible(e, (int)k) ? 1 : 0;
            count += on[k];
        }
    if (e->d_sim_da.upload(on) != 0 || e->d_dastats.zero((size_t)e->total_replicas) != 0)
        return -1;
    e->da = count > 0 ? 1 : 0;
    e->sur = e->da ? s : nullptr;
    if (s) {
        e->sur_thr = rmse_threshold;
        e->sur_window = error_window;
        e->sur_min = min_evals;
    }
    for (auto &kv : e->graphs)
        cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
    if (e->da) {
        if (autotune(e, 0, 0) != 0)
            return -1;
    } else {
        configure_shape(e, e->plain_cluster, e->plain_threads);
    }
    if (e->smem > 227 * 1024)
        return cgppd_fail("cgppd_engine_set_surrogate: the screened kernel does not fit in shared memory");
    if (cgppd_check(set_mc_smem_limit(e->smem), "engine shared-memory limit") != 0)
        return -1;
    return count;
}

int cgppd_engine_surrogate_stats(cgppd_engine *e, int sim, double *out)
{
    if (!e || !e->finalized || sim < 0 || sim >= (int)e->sims.size() || !out)
        return cgppd_fail("cgppd_engine_surrogate_stats: bad argument");
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "surrogate stats") != 0)
        return -1;
    const DevSim &S = e->h_sims[sim];
    for (int k = 0; k < 7; ++k)
        out[k] = 0.0;
    if (!e->da)
        return 0;
    std::vector<DAStats> d(S.R);
    int flag = 0;
    if (cgppd_check(cudaMemcpy(d.data(), e->d_dastats.ptr + S.rep_off, sizeof(DAStats) * S.R, cudaMemcpyDeviceToHost),
                    "surrogate stats") != 0 ||
        cgppd_check(cudaMemcpy(&flag, e->d_sim_da.ptr + sim, sizeof(int), cudaMemcpyDeviceToHost), "surrogate flag"))
        return -1;
    for (const DAStats &x : d) {
        out[0] += (double)x.proposals;
        out[1] += (double)x.stage1_reject;
        out[2] += (double)x.stage2_eval;
        out[3] += (double)x.stage2_accept;
        out[4] += x.sum_e2;
        out[5] += (double)x.n_e2;
    }
    out[6] = flag;
    return 0;
}

int cgppd_surrogate_collect(cgppd_surrogate *s, cgppd_engine *e, int sim, int n, double proposal_fraction,
                            unsigned long long seed)
{
    if (!s || !e || !e->finalized || sim < 0 || sim >= (int)e->sims.size() || n <= 0)
        return cgppd_fail("cgppd_surrogate_collect: bad argument");
    if (!sim_compatible(e, sim))
        return cgppd_fail("cgppd_surrogate_collect: the simulation is not made of copies of one rigid molecule");
    const DevSim &S = e->h_sims[sim];
    uint64_t rs = seed;
    auto next = [&rs]() {
        uint64_t z = (rs += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    std::vector<int4> items(n);
    for (int i = 0; i < n; ++i) {
        const int g = S.rep_off + (int)(next() % (uint64_t)S.R);
        int a = (int)(next() % (uint64_t)S.M), b = (int)(next() % (uint64_t)(S.M - 1));
        if (b >= a)
            ++b;
        if (a > b)
            std::swap(a, b);
        const double u = (double)(next() >> 11) * (1.0 / 9007199254740992.0);
        const int mode = (u < proposal_fraction) ? 1 + (int)(next() & 1) : 0;
        items[i] = make_int4(g, a, b, mode);
    }
    DevBuf<int4> d_items;
    DevBuf<float> dX, dY;
    if (d_items.upload(items) != 0 || dX.alloc((size_t)n * kSurIn) != 0 || dY.alloc((size_t)n) != 0)
        return -1;
    if (cgppd_check(cudaStreamSynchronize(e->own_stream), "collect") != 0)
        return -1;
    const uint32_t k0 = (uint32_t)(seed ^ 0x51A7u), k1 = (uint32_t)(seed >> 32) ^ 0x2545F491u;
    if (cgppd_check(launch_pose_samples(e->args(), d_items.ptr, n, k0, k1, dX.ptr, dY.ptr, e->own_stream),
                    "pose samples") != 0 ||
        cgppd_check(cudaStreamSynchronize(e->own_stream), "pose samples") != 0)
        return -1;
    return surrogate_append_device_samples(s, dX.ptr, dY.ptr, n);
}

}  // extern "C"

extern "C" int cgppd_graph_counts(int n, const char *chain_ids, int all_flexible, int n_segments,
                                  const int *seg_lengths, const int *seg_residues, int num_chains, int *counts9)
{
    if (n <= 0)
        return cgppd_fail("cgppd_graph_counts: empty molecule");
    std::vector<char> chains(chain_ids, chain_ids + n);
    std::vector<std::vector<int>> segs;
    int off = 0;
    for (int k = 0; k < n_segments; ++k) {
        segs.emplace_back(seg_residues + off, seg_residues + off + seg_lengths[k]);
        for (int v : segs.back())
            if (v < 0 || v >= n)
                return cgppd_fail("cgppd_graph_counts: segment residue out of range");
        off += seg_lengths[k];
    }
    Graph g;
    g.init(chains, all_flexible != 0, segs, num_chains);
    counts9[0] = (int)g.bonds.size();
    counts9[1] = (int)g.angles.size();
    counts9[2] = (int)g.torsions.size();
    counts9[3] = (int)g.rigid_domains.size();
    counts9[4] = (int)g.segment_bonds.size();
    counts9[5] = (int)g.indirect_neighbours.size();
    counts9[6] = (int)g.MC_local_residues.size();
    counts9[7] = (int)g.MC_crankshaft_residues.size();
    counts9[8] = (int)g.MC_flex_residues.size();
    return 0;
}
