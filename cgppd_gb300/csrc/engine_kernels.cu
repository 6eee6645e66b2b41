// engine_kernels.cu -- device side of the batched replica-exchange Monte Carlo engine.
//
// k_mc<RES, DA, QF>: one thread-block cluster per replica runs `nsteps` Monte Carlo steps of
// that replica with no inter-replica traffic (replicas are independent between
// exchanges); every replica of every simulation is in the one launch.  A step restates
// Replica::MCSearch (src/Replica.cpp:350-414):
//   1. pick a molecule and a move (src/Molecule.cpp:451-504) from Philox draws (drawn one
//      step ahead by an idle warp),
//   2. build the moved molecule's proposed coordinates in shared memory,
//   3. evaluate the moved molecule against every other residue (its row of the
//      molecule-pair energy matrix) and, for a flexible molecule, its internal
//      non-bonded + bonded energy (src/Molecule.cpp:636-699; a local move evaluates only
//      the moved residue's terms, every other term being unchanged bit for bit),
//   4. new total = old total - old row + new row; Metropolis on the float delta with
//      the float Boltzmann factor, as the reference does (src/Replica.cpp:385-410),
//   5. on accept, commit coordinates and the row (copy-on-accept; nothing to undo).
// The reference recomputes every pair each step; only the moved molecule's pairs
// change, so the engine evaluates those and keeps the rest in the matrix.
//
// RES = true: every CTA copies its replica's state (coordinates, static residue
// records, centres, the pair matrix, internal energies and row sums as float-float,
// and the simulation's static move/bond/tile lists) into shared memory at launch,
// updates it in place, and rank 0 writes it back at the end -- no global-memory latency
// and no FP64 arithmetic on the step's serial path.  RES = false (large systems): state
// stays in global memory (L2) and rank 0 commits there.
//
// Within a cluster every CTA builds the same proposal (same draws, same arithmetic),
// takes an even slice of the other residues, and pushes its per-molecule partial rows
// (float-float) into every CTA's shared memory before one cluster barrier; every CTA sums
// them in the same rank order, so every CTA takes the same Metropolis decision.
//
// DA = true: delayed-acceptance screening with the learned surrogate (see below).
//
// QF = true: a rigid mover is also kept in charged-first order, and the pair loop takes
// the Debye-Hueckel term for its charged residues only (most residues carry no charge).
//
// k_exchange: one warp per simulation performs the even/odd temperature exchange of
// Simulation::run (src/Simulation.cpp:770-795), the per-temperature bookkeeping of
// Replica::fraction_bound / acceptance_ratio (src/Replica.cpp:1095-1122) and the
// surrogate's fallback check.
#include <array>
#include <cooperative_groups.h>

#include "cgppd_common.cuh"
#include "engine_types.h"
#include "surrogate.cuh"

namespace cg = cooperative_groups;

namespace cgppd {

constexpr int kTableStride = 32;
// Contact table in shared memory: -4 Eij in kcal/mol per type pair (4 bytes: a warp's
// lookups of one row fall in one 128-byte line).
constexpr int kTableBytes = kTableStride * kTableStride * (int)sizeof(float);
constexpr int kMaxThreads = 512;
constexpr int kMaxWarps = kMaxThreads / 32;
// Slack (A) on top of two bounding radii before a molecule pair skips the per-pair
// minimum image: covers the float rounding of positions, centres and rotations.
constexpr float kImageMargin = 0.05f;

struct MoveDesc {
    int m, start, n, type, kind;
    int ri, br_off, br_cnt;
    int flexible, wrapped, null_move, nintra;
    float R[9];
    float vx, vy, vz;        // translation of the molecule (translate) or of residue ri (local)
    float fx, fy, fz;        // displacement / n (local, flex)
    float cx, cy, cz;        // centre before the move
    float wcx, wcy, wcz;     // centre after the move (wrapped)
    float px, py, pz;        // flex pivot position
    uint32_t w_metro;
    uint32_t w_stage1;       // delayed acceptance: the surrogate stage's uniform draw
};

// The part of a move decision that depends on the draws alone (src/Molecule.cpp:146-504:
// the molecule, the move type, the direction and its rotation, the flex residue and
// branch, the local residue and the crankshaft flip), taken for 32 steps at a time by
// the lanes of one warp; finish_move adds the part that reads the state.
struct MovePre {
    int m, ri, br_off, br_cnt;
    int bits;       // type | kind << 4 | null move << 8 | crankshaft flip << 9
    float R[9];     // the rotation (rotate, flex) or the unit direction in R[0..2]
    uint32_t w_metro, w_stage1;
};

// Ring of draw-only decisions in shared memory: the entries of steps [32k, 32k + 32)
// are filled during step 32k - 17 (the first 32 before the loop), half a ring ahead of
// the step that reads them.
constexpr int kRing = 64;

struct SmemLayout {
    int table, mols, ipos, irel, iexcl, idisp, iq, ipq, iqq, ej, rowp, row;  // always
    int rcv;                                                         // clusters: pushed partial rows
    int rad;                                                         // bounding radius per molecule
    int ring;                                                        // draw-only decisions (kRing)
    int lst[12];                                                     // resident + flexible: static lists
    int P, Q, ST, EX, CEN, EM, INTRA, ROWSUM, QP;                    // resident only
    int daW, daW1, daB, daW5, daH, daHS, daX, daP, daF, daSM;        // delayed acceptance only
    int total;
};

// Delayed acceptance: each CTA of a replica's cluster holds the output columns
// [rank * S, rank * S + S) of layers 1..4 (S = 256 / C); rows of the pose batch are
// padded to multiples of 16 (one mma.sync m-tile); BF16 rows are padded to 264 elements
// so that the fragment loads of 8 consecutive rows hit distinct banks.
constexpr int kDaWS = kSurH + 8;

__host__ __device__ inline int da_rows(int max_m) { return (((max_m - 1 > 1 ? max_m - 1 : 1) + 15) / 16) * 16; }

__host__ __device__ inline int align16(int v) { return (v + 15) & ~15; }

// Lanes per other residue j in the inter-pair loop of a move of an n-residue molecule
// (N residues in the simulation, C CTAs of W warps): g lanes share one j and take every
// g-th residue i of the mover, a warp holds floor(32 / g) such groups.  Cost of the busiest
// thread: passes over the CTA's slice x (ceil(n / g) pairs + a per-j overhead for the
// loads, the periodic image and the log2(g)-step reduction); the cheapest g wins, ties
// to the smaller g.
__host__ __device__ inline int pair_lanes(int n, int N, int C, int W) {
    const int sl = (N - n + C - 1) / C;
    int best = 1, best_cost = 0x7fffffff;
    for (int g = 1; g <= 32 && g <= (n > 1 ? n : 1); ++g) {
        const int per = W * (32 / g);
        const int passes = (sl + per - 1) / per;
        int lg = 0;
        while ((1 << lg) < g)
            ++lg;
        const int cost = passes * ((n + g - 1) / g + 2 + lg);
        if (cost < best_cost) {
            best_cost = cost;
            best = g;
        }
    }
    return best;
}

enum ListId { kLBond = 0, kLAng, kLTor, kLInd, kLFlex, kLFopt, kLBranch, kLLocal, kLCrank, kLTile };
constexpr int kNumLists = 10;

__host__ __device__ inline SmemLayout smem_layout(int max_mol, int slice, int max_m, int max_n, int resident,
                                                  int any_flexible, int da = 0, int C = 1,
                                                  const int *lmax = nullptr)
{
    SmemLayout L;
    int off = 0;
    L.table = off;  off += kTableBytes;
    L.mols = off;   off = align16(off + (int)sizeof(DevMol) * max_m);
    L.ipos = off;   off += 16 * max_mol;
    L.irel = off;   off += 16 * max_mol;
    L.iexcl = off;  off += 16 * max_mol;
    L.idisp = off;  off += 16 * max_mol;
    L.iq = off;     off = align16(off + 8 * max_mol);
    L.ipq = off;    off += 16 * max_mol;  // the rigid mover in charged-first order
    L.iqq = off;    off = align16(off + 8 * max_mol);
    L.ej = off;     off = align16(off + 8 * slice);
    L.rowp = off;   off = align16(off + 8 * (max_m + 1));
    L.row = off;    off = align16(off + 8 * (max_m + 1));
    // [2 step parities][C source ranks][max_m + 1] (last entry: internal energy)
    L.rcv = off;    off = align16(off + (C > 1 ? 2 * C * (max_m + 1) * 8 : 0));
    L.rad = off;    off = align16(off + 4 * max_m);
    L.ring = off;   off = align16(off + kRing * (int)sizeof(MovePre));
    L.P = L.Q = L.ST = L.EX = L.CEN = L.EM = L.INTRA = L.ROWSUM = L.QP = 0;
    if (resident) {
        L.P = off;      off += 16 * max_n;
        L.Q = off;      off += 16 * max_n;
        L.ST = off;     off = align16(off + max_n);  // residue types (sigma/2 in P.w, charge in Q.w)
        L.EX = off;     off += any_flexible ? 16 * max_n : 0;
        L.CEN = off;    off += 16 * max_m;
        L.EM = off;     off = align16(off + 8 * max_m * max_m);
        L.INTRA = off;  off = align16(off + 8 * max_m);
        L.ROWSUM = off; off = align16(off + 8 * max_m);
        L.QP = off;     off = align16(off + 2 * max_n);  // charged-first positions
    }
    for (int k = 0; k < 12; ++k)
        L.lst[k] = 0;
    if (resident && any_flexible && lmax) {
        // bonds, angles, torsions, torsion V, torsion phases, indirect pairs, flex residues,
        // flex options, branch residues, local residues, crankshaft residues, intra tiles
        const int bytes[12] = {8 * lmax[kLBond], 16 * lmax[kLAng], 16 * lmax[kLTor], 16 * lmax[kLTor],
                               16 * lmax[kLTor], 8 * lmax[kLInd], 16 * lmax[kLFlex], 16 * lmax[kLFopt],
                               4 * lmax[kLBranch], 4 * lmax[kLLocal], 4 * lmax[kLCrank], 8 * lmax[kLTile]};
        for (int k = 0; k < 12; ++k) {
            L.lst[k] = off;
            off = align16(off + bytes[k]);
        }
    }
    L.daW = L.daW1 = L.daB = L.daW5 = L.daH = L.daHS = L.daX = L.daP = L.daF = L.daSM = 0;
    if (da) {
        const int S = kSurH / C, RP = da_rows(max_m);
        L.daW = off;   off += 3 * S * kDaWS * 2;
        L.daW1 = off;  off += S * kSurIn * 4;
        L.daB = off;   off += 4 * S * 4;
        L.daW5 = off;  off = align16(off + S * 4);
        L.daH = off;   off += RP * kDaWS * 2;
        L.daHS = off;  off += 2 * RP * S * 2;
        L.daX = off;   off += RP * kSurIn * 4;
        L.daP = off;   off += RP * 4;
        L.daF = off;   off = align16(off + RP * 4);
        L.daSM = off;  off = align16(off + 4 * max_m * max_m);
    }
    L.total = off;
    return L;
}

size_t engine_smem_bytes(int max_mol, int max_n, int max_m, int cluster, int resident, int any_flexible, int da,
                         const int *lmax)
{
    const int slice = (max_n + cluster - 1) / cluster;
    return (size_t)smem_layout(max_mol, slice, max_m, max_n, resident, any_flexible, da, cluster, lmax).total;
}

// Static per-molecule lists (DevMol offsets index the global arrays).  Resident launches
// read shared-memory copies of their simulation's ranges, shifted by the range starts.
struct Lists {
    const int2 *bonds;
    const int4 *angles, *tors;
    const float4 *torsV, *torsS;
    const int2 *indsub;
    const int4 *flexres, *flexopt;
    const int *branch, *localres, *crankres;
    const int2 *tiles;
    int base[kNumLists];
};

__device__ __forceinline__ Lists global_lists(const EngineArgs &a)
{
    Lists Ls{a.bonds, a.angles, a.tors, a.torsV, a.torsS, a.indsub, a.flexres, a.flexopt, a.branch, a.localres,
             a.crankres, a.tiles, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
    return Ls;
}

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ FF ff_from(double d)
{
    const float hi = (float)d;
    return FF{hi, (float)(d - (double)hi)};
}

// Block-wide FF sum in a fixed order, returned (identically) in every thread.
__device__ FF block_sum_ff_ff(FF v, FF *red)
{
    const int t = threadIdx.x, nw = blockDim.x >> 5;
    v = ff_warp_sum(v);
    __syncthreads();
    if ((t & 31) == 0)
        red[t >> 5] = v;
    __syncthreads();
    FF s{0.f, 0.f};
    for (int w = 0; w < nw; ++w)
        ff_add_ff(s, red[w]);
    return s;
}

// Block-wide FF sum in a fixed order, complete in every lane of warp 0 (a butterfly over
// the warp sums; the other warps' return value is unspecified).
__device__ FF block_sum_ff_warp0(FF v, FF *red)
{
    const int t = threadIdx.x, nw = blockDim.x >> 5, lane = t & 31;
    v = ff_warp_sum(v);
    __syncthreads();
    if (lane == 0)
        red[t >> 5] = v;
    __syncthreads();
    FF s{0.f, 0.f};
    if (t < 32) {
        if (lane < nw)
            s = red[lane];
        s = ff_warp_sum(s);
    }
    return s;
}

// Block-wide FF sum in a fixed order, returned as double in every thread.
__device__ double block_sum_ff(FF v, FF *red)
{
    const int t = threadIdx.x, nw = blockDim.x >> 5;
    v = ff_warp_sum(v);
    __syncthreads();
    if ((t & 31) == 0)
        red[t >> 5] = v;
    __syncthreads();
    FF s{0.f, 0.f};
    for (int w = 0; w < nw; ++w)
        ff_add_ff(s, red[w]);
    return ff_value(s);
}

__device__ __forceinline__ float3 rot_apply(const float *R, float x, float y, float z)
{
    return make_float3(fmaf(R[0], x, fmaf(R[1], y, R[2] * z)), fmaf(R[3], x, fmaf(R[4], y, R[5] * z)),
                       fmaf(R[6], x, fmaf(R[7], y, R[8] * z)));
}

// Rotation matrix of the quaternion (cos(a/2), sin(a/2) axis) (src/Quaternion.cpp:12-21,
// :95-112), optionally normalised first (Quaternion::normalize, :30-38).
// Rotation matrix of the quaternion (cos(angle/2), sin(angle/2) * axis); (s, c) are
// sin/cos of angle/2 (precomputed per launch for the replica's fixed step angle).
__device__ void axis_angle_matrix_sc(float s, float c, float ax, float ay, float az, bool normalize, float *R)
{
    float w = c, x = s * ax, y = s * ay, z = s * az;
    if (normalize) {
        const float inv = 1.0f / sqrtf(w * w + x * x + y * y + z * z);
        w *= inv, x *= inv, y *= inv, z *= inv;
    }
    const float w2 = w * w, x2 = x * x, y2 = y * y, z2 = z * z;
    const float wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
    R[0] = w2 + x2 - y2 - z2;
    R[1] = (xy - wz) * 2.0f;
    R[2] = (wy + xz) * 2.0f;
    R[3] = (wz + xy) * 2.0f;
    R[4] = w2 - x2 + y2 - z2;
    R[5] = (yz - wx) * 2.0f;
    R[6] = (xz - wy) * 2.0f;
    R[7] = (yz + wx) * 2.0f;
    R[8] = w2 - x2 - y2 + z2;
}

__device__ void axis_angle_matrix(float angle, float ax, float ay, float az, bool normalize, float *R)
{
    float s, c;
    sincosf(0.5f * angle, &s, &c);
    axis_angle_matrix_sc(s, c, ax, ay, az, normalize, R);
}

// Molecule::wrapped_centre: fmod per component (keeps the sign).  Centres move by a few
// A per step, so |c| < 2 box: then fmod is c, c - box or c + box, each exact (Sterbenz);
// c == -box (fmod gives -0) and larger |c| take fmodf itself.
__device__ __forceinline__ float wrapf(float c, float box)
{
    if (fabsf(c) < box)
        return c;
    if (c >= box && c < 2.0f * box)
        return c - box;
    if (c < -box && c > -2.0f * box)
        return c + box;
    return fmodf(c, box);
}

// floor(u * n) for u = w / 2^32, exactly.
__device__ __forceinline__ int pickw(uint32_t w, int n) { return (int)(((unsigned long long)w * (unsigned)n) >> 32); }

// The draw u - 0.5 (or 0.5 - u) rounded once to float, exactly as (float)(u - 0.5).
__device__ __forceinline__ float centred(uint32_t w, bool negate)
{
    const long long d = negate ? (2147483648LL - (long long)w) : ((long long)w - 2147483648LL);
    return (float)d * 2.3283064365386963e-10f;
}

__device__ __forceinline__ float3 normalized(float x, float y, float z)
{
    const float mag = sqrtf(x * x + y * y + z * z);
    if (mag != 0.0f)
        return make_float3(x / mag, y / mag, z / mag);
    return make_float3(x, y, z);
}


__device__ __forceinline__ void load_table(float *s_table, const float *table, int t, int T)
{
    for (int k = t; k < kTableStride * kTableStride; k += T)
        s_table[k] = table[k];
}

// Pair energy in kcal/mol of residue records a (position, sigma/2) and b, with the
// charge q*sqrt(DHF) of a in qa.x and its type in qa.y (int bits), b's charge in qb and
// `col` the table column of b's type (col[type_a * kTableStride]).  The LJ term is
// u = (-4 Eij) s6 (s6 - 1), and 2 Eij - u on the repulsive branch (Eij > 0, s6 > 1/2),
// the same values as lj_term with one multiplication less (power-of-two scaling).
// MI: the axes (bit 0 x, 1 y, 2 z) that take the minimum image; on the others the caller
// has already moved b to the periodic image that every pair takes (see the inter-pair
// loop of k_mc), so a - b is the minimum-image difference itself.
template <bool DH, int MI>
__device__ __forceinline__ float pair_term(float4 a, float2 qa, float4 b, float qb, const float *col, float L,
                                           float invL)
{
    const float dx = (MI & 1) ? min_image(a.x - b.x, L, invL) : a.x - b.x;
    const float dy = (MI & 2) ? min_image(a.y - b.y, L, invL) : a.y - b.y;
    const float dz = (MI & 4) ? min_image(a.z - b.z, L, invL) : a.z - b.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float inv_r = rsqrt_sfu(r2);
    const float m4e = col[__float_as_int(qa.y) * kTableStride];
    const float so = (a.w + b.w) * inv_r;  // sigma_ij / r
    const float s2 = so * so;
    const float s6 = s2 * s2 * s2;
    float u = m4e * fmaf(s6, s6, -s6);
    if (m4e < 0.0f && s6 > 0.5f)
        u = fmaf(-0.5f, m4e, -u);
    if (!DH)  // one of the pair uncharged: no Debye-Hueckel term
        return u;
    return u + qa.x * qb * ex2_sfu(r2 * inv_r * (-kLog2e / kXi)) * inv_r;
}

template <bool DH = true>
__device__ __forceinline__ float pair_kcal(float4 a, float2 qa, float4 b, float2 qb, const float *table, float L,
                                           float invL)
{
    return pair_term<DH, 7>(a, qa, b, qb.x, table + __float_as_int(qb.y), L, invL);
}

// Pair terms of residues i = i0, i0 + g, ... < i1 of the mover (records ipv / iqv) with
// one residue b of another molecule: four independent partial sums, folded into the
// float-float accumulator every 32 terms.  Returns the first index of the sequence at or
// past i1 (where the next span of the same sequence starts).
template <bool DH, int MI>
__device__ __forceinline__ int pair_span(const float4 *ipv, const float2 *iqv, int i0, int i1, int g, float4 b,
                                          float qb, const float *col, float L, float invL, FF &acc, float &p0,
                                          float &p1, float &p2, float &p3)
{
    int i = i0, cntp = 0;
    for (; i + 3 * g < i1; i += 4 * g) {
        p0 += pair_term<DH, MI>(ipv[i], iqv[i], b, qb, col, L, invL);
        p1 += pair_term<DH, MI>(ipv[i + g], iqv[i + g], b, qb, col, L, invL);
        p2 += pair_term<DH, MI>(ipv[i + 2 * g], iqv[i + 2 * g], b, qb, col, L, invL);
        p3 += pair_term<DH, MI>(ipv[i + 3 * g], iqv[i + 3 * g], b, qb, col, L, invL);
        if (++cntp == 8) {
            ff_add(acc, (p0 + p1) + (p2 + p3));
            p0 = p1 = p2 = p3 = 0.f;
            cntp = 0;
        }
    }
    for (; i < i1; i += g)
        p0 += pair_term<DH, MI>(ipv[i], iqv[i], b, qb, col, L, invL);
    return i;
}

// Every pair of the mover (its charged residues first: the full term, then the
// Lennard-Jones part alone) with the residue b, residues i = sub, sub + g, ... of the
// mover, into acc.
template <int MI>
__device__ __forceinline__ void mover_spans(const float4 *ipv, const float2 *iqv, int sub, int nqm, int n, int g,
                                            float4 b, float qb, const float *col, float L, float invL, FF &acc)
{
    float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
    const int i2 = pair_span<true, MI>(ipv, iqv, sub, nqm, g, b, qb, col, L, invL, acc, p0, p1, p2, p3);
    ff_add(acc, (p0 + p1) + (p2 + p3));
    p0 = p1 = p2 = p3 = 0.f;
    pair_span<false, MI>(ipv, iqv, i2, n, g, b, qb, col, L, invL, acc, p0, p1, p2, p3);
    ff_add(acc, (p0 + p1) + (p2 + p3));
}

// Repulsive crowder pair in kcal/mol, the reference's REPULSIVE_CROWDING build
// (src/Replica.cpp:416-419 and :434-472, src/CudaFunctions.cu:335-338 and :492-498):
// (6/r)^12 RT below const_repulsive_cutoff (15 A, src/definitions.h:38), zero beyond,
// and no Debye-Hueckel term.
__device__ __forceinline__ float crowder_kcal(float4 a, float4 b, float L, float invL)
{
    const float dx = min_image(a.x - b.x, L, invL);
    const float dy = min_image(a.y - b.y, L, invL);
    const float dz = min_image(a.z - b.z, L, invL);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float inv_r = rsqrt_sfu(r2);
    const float s = 6.0f * inv_r;
    const float s2 = s * s;
    const float s6 = s2 * s2 * s2;
    return (r2 * inv_r < kRepulsiveCutoff) ? kRTtoKcal * (s6 * s6) : 0.0f;
}

__device__ __forceinline__ bool intra_excluded(int4 ei, int4 ej)
{
    // same rigid domain, backbone neighbours (|resSeq| < 4 on one chain), or bonded
    // across a segment (src/Molecule.cpp:655, src/Residue.cpp:101-114)
    return (ei.z != 0 && ei.z == ej.z) || (ei.x == ej.x && abs(ei.y - ej.y) < 4) || (ei.w != 0 && ei.w == ej.w);
}

// One bonded term (kcal/mol) of a molecule at coordinates `p`: kind 0 bond, 1 angle,
// 2 torsion (src/Potential.cpp:45-98 with Potential::total's factors).
__device__ float bonded_item(const Lists &a, const DevMol &mol, const float4 *p, float L, float invL, int kind,
                             int k)
{
    if (kind == 0) {  // 0.5 K (r - R0)^2, minimum-image distance
        const int2 b = a.bonds[mol.bond_off + k - a.base[kLBond]];
        const float4 pi = p[b.x], pj = p[b.y];
        const float dx = min_image(pj.x - pi.x, L, invL), dy = min_image(pj.y - pi.y, L, invL),
                    dz = min_image(pj.z - pi.z, L, invL);
        const float rr = sqrtf(dx * dx + dy * dy + dz * dz) - kR0;
        return 0.5f * kKSpring * rr * rr;
    }
    if (kind == 1) {  // -(1/gamma) log(exp(-gamma(ka(t-ta)^2 + ea)) + exp(-gamma kb (t-tb)^2))
        const int4 an = a.angles[mol.ang_off + k - a.base[kLAng]];
        const float4 pi = p[an.x], pj = p[an.y], pk = p[an.z];
        const float abx = pi.x - pj.x, aby = pi.y - pj.y, abz = pi.z - pj.z;
        const float cbx = pk.x - pj.x, cby = pk.y - pj.y, cbz = pk.z - pj.z;
        const float cm = sqrtf(cbx * cbx + cby * cby + cbz * cbz) * sqrtf(abx * abx + aby * aby + abz * abz);
        float th = 0.f;
        if (cm >= 1e-26f)
            th = acosf(fminf(1.f, fmaxf(-1.f, (abx * cbx + aby * cby + abz * cbz) / cm)));
        const float da = th - kThetaAlpha, db = th - kThetaBeta;
        const float term =
            expf(-kGammaAngle * (kKAlpha * da * da + kEpsAlpha)) + expf(-kGammaAngle * (kKBeta * db * db));
        return -kGammaAngleRecip * logf(term);
    }
    // sum_n V_n (1 + cos(n phi - sigma_n))
    // sum_n V_n (1 + cos(n phi - sigma_n)) = sum_n V_n + sum_n A_n cos(n phi) + B_n sin(n phi)
    // with A_n = V_n cos(sigma_n), B_n = V_n sin(sigma_n) (precomputed); cos/sin(phi) from
    // the dihedral's dot and cross products and cos/sin(n phi) by angle addition, so no
    // atan2 or cos call sits on the step's path.  The molecule's sum of V_n is added once.
    const int ti = mol.tor_off + k - a.base[kLTor];
    const int4 tq = a.tors[ti];
    const float4 A = a.torsV[ti], B = a.torsS[ti];
    const float4 p1 = p[tq.x], p2 = p[tq.y], p3 = p[tq.z], p4 = p[tq.w];
    const float b1x = p2.x - p1.x, b1y = p2.y - p1.y, b1z = p2.z - p1.z;
    const float b2x = p3.x - p2.x, b2y = p3.y - p2.y, b2z = p3.z - p2.z;
    const float b3x = p4.x - p3.x, b3y = p4.y - p3.y, b3z = p4.z - p3.z;
    const float c23x = b2y * b3z - b2z * b3y, c23y = b2z * b3x - b2x * b3z, c23z = b2x * b3y - b2y * b3x;
    const float c12x = b1y * b2z - b1z * b2y, c12y = b1z * b2x - b1x * b2z, c12z = b1x * b2y - b1y * b2x;
    const float mb2 = sqrtf(b2x * b2x + b2y * b2y + b2z * b2z);
    const float y = mb2 * (b1x * c23x + b1y * c23y + b1z * c23z), x = c12x * c23x + c12y * c23y + c12z * c23z;
    const float h2 = x * x + y * y;
    float c1 = 1.f, s1 = 0.f;  // atan2(0, 0) = 0
    if (h2 > 0.f) {
        const float inv = rsqrt_refined(h2);
        c1 = x * inv;
        s1 = y * inv;
    }
    const float c2 = c1 * c1 - s1 * s1, s2 = 2.f * s1 * c1;
    const float c3 = c2 * c1 - s2 * s1, s3 = s2 * c1 + c2 * s1;
    const float c4 = c3 * c1 - s3 * s1, s4 = s3 * c1 + c3 * s1;
    const float e = ((A.x * c1 + B.x * s1) + (A.y * c2 + B.y * s2)) + ((A.z * c3 + B.z * s3) + (A.w * c4 + B.w * s4));
    return (k == 0) ? e + mol.tors_const : e;
}

// Bonded terms of one molecule, one flat index over bonds, angles and torsions so that
// each thread evaluates one term: thread-strided from t0 by `stride`.
__device__ void bonded_terms(const Lists &a, const DevMol &mol, const float4 *p, float L, float invL, int t0,
                             int stride, FF &acc)
{
    const int nb = mol.nbond, na = mol.nang, nt = mol.ntor;
    for (int k = t0; k < nb + na + nt; k += stride) {
        const int kind = (k < nb) ? 0 : (k < nb + na) ? 1 : 2;
        const int kk = (kind == 0) ? k : (kind == 1) ? k - nb : k - nb - na;
        ff_add(acc, bonded_item(a, mol, p, L, invL, kind, kk));
    }
}

// Whether bonded term (kind, k) of a molecule involves residue ri.
__device__ __forceinline__ bool bonded_has(const Lists &a, const DevMol &mol, int kind, int k, int ri)
{
    if (kind == 0) {
        const int2 b = a.bonds[mol.bond_off + k - a.base[kLBond]];
        return b.x == ri || b.y == ri;
    }
    if (kind == 1) {
        const int4 an = a.angles[mol.ang_off + k - a.base[kLAng]];
        return an.x == ri || an.y == ri || an.z == ri;
    }
    const int4 tq = a.tors[mol.tor_off + k - a.base[kLTor]];
    return tq.x == ri || tq.y == ri || tq.z == ri || tq.w == ri;
}

// Change of the bonded terms that involve residue ri between positions pold and pnew
// (molecule-relative arrays), thread-strided from t0.
__device__ void bonded_delta(const Lists &a, const DevMol &mol, const float4 *pnew, const float4 *pold, int ri,
                             float L, float invL, int t0, int stride, FF &acc)
{
    const int nb = mol.nbond, na = mol.nang, nt = mol.ntor;
    for (int k = t0; k < nb + na + nt; k += stride) {
        const int kind = (k < nb) ? 0 : (k < nb + na) ? 1 : 2;
        const int kk = (kind == 0) ? k : (kind == 1) ? k - nb : k - nb - na;
        if (bonded_has(a, mol, kind, kk, ri))
            ff_add(acc, bonded_item(a, mol, pnew, L, invL, kind, kk) - bonded_item(a, mol, pold, L, invL, kind, kk));
    }
}

// Full internal energy (unexcluded pairs over the molecule's active tiles, indirect
// subtraction, bonded terms) of a molecule at the state's positions, by one CTA; the
// same value in every thread.
__device__ FF intra_full_cta(const Lists &Ls, const DevMol &mol, const float4 *P, const float4 *Q,
                             const unsigned char *TY, const int4 *EX, const float *table, float L, float invL,
                             FF *red)
{
    const int t = threadIdx.x, T = blockDim.x, warp = t >> 5, lane = t & 31, NW = T >> 5;
    const int n = mol.count, st = mol.start;
    FF acc{0.f, 0.f};
    for (int k = warp; k < mol.ntile; k += NW) {
        const int2 tl = Ls.tiles[mol.tile_off + k - Ls.base[kLTile]];
        const int j = tl.y * 32 + lane;
        float part = 0.f;
        if (j < n) {
            const float4 pj = P[st + j];  // resident records: sigma/2 in P.w, charge in Q.w
            const float2 qj = make_float2(Q[st + j].w, __int_as_float((int)TY[st + j]));
            const int4 ej = EX[st + j];
            const int iend = (tl.x == tl.y) ? j : min(n, tl.x * 32 + 32);
            for (int i = tl.x * 32; i < iend; ++i) {
                if (intra_excluded(EX[st + i], ej))
                    continue;
                part += pair_kcal(P[st + i], make_float2(Q[st + i].w, __int_as_float((int)TY[st + i])), pj, qj, table,
                                  L, invL);
            }
        }
        ff_add(acc, part);
    }
    for (int k = t; k < mol.nind; k += T) {
        const int2 pr = Ls.indsub[mol.ind_off + k - Ls.base[kLInd]];
        const int ia = st + pr.x, ib = st + pr.y;
        ff_add(acc, -pair_kcal(P[ia], make_float2(Q[ia].w, __int_as_float((int)TY[ia])), P[ib],
                               make_float2(Q[ib].w, __int_as_float((int)TY[ib])), table, L, invL));
    }
    bonded_terms(Ls, mol, P + st, L, invL, t, T, acc);
    return block_sum_ff_ff(acc, red);
}

// ------------------------------------------------------------------ move decision

// Loads of mutable state: plain shared-memory loads when resident, L2 loads otherwise
// (another CTA of the cluster may have committed them).
template <bool RES, typename T>
__device__ __forceinline__ T ld_state(const T *p)
{
    if (RES)
        return *p;
    return __ldcg(p);
}

__device__ void predecide_move(const Lists &a, const DevSim &S, const DevMol *mols, const float4 rsc,
                               const uint32_t *w, MovePre &pre)
{
    const int M = S.M;
    const int m = pickw(w[0], M);
    const DevMol &mol = mols[m];
    pre.m = m;
    pre.ri = 0, pre.br_off = 0, pre.br_cnt = 0;
    int kind = 0, null_move = 0, flip = 0;
    int type;
    if (mol.flags & kMolFlexible) {
        int k = 0;
        if (M > 1) {
            while (k < 3 && (unsigned long long)w[1] >= S.thr4[k])
                ++k;
            type = k;
        } else {
            while (k < 2 && (unsigned long long)w[1] >= S.thr3[k])
                ++k;
            type = 1 + k;
        }
    } else {
        type = ((unsigned long long)w[1] < S.thr_rot) ? kRotate : kTranslate;  // gsl_ran_bernoulli
    }
    const float dx = centred(w[2], false), dy = centred(w[3], true), dz = centred(w[4], false);
    switch (type) {
    case kTranslate: {
        // Molecule::translate(rng, step) (src/Molecule.cpp:146-159, :262-266)
        const float3 u = normalized(dx, dy, dz);
        pre.R[0] = u.x, pre.R[1] = u.y, pre.R[2] = u.z;
        break;
    }
    case kRotate: {
        // Molecule::rotate(rng, step) -> setRotation (src/Molecule.cpp:193-208, :255-260)
        const float3 u = normalized(dx, dy, dz);
        axis_angle_matrix_sc(rsc.x, rsc.y, u.x, u.y, u.z, true, pre.R);
        break;
    }
    case kFlex: {
        // Molecule::flex(rng, step) (src/Molecule.cpp:331-413)
        if (mol.nflex == 0) {
            null_move = 1;
            break;
        }
        const float3 u = normalized(dx, dy, dz);
        axis_angle_matrix_sc(rsc.x, rsc.y, u.x, u.y, u.z, false, pre.R);
        const int4 fr = a.flexres[mol.flex_off + pickw(w[5], mol.nflex) - a.base[kLFlex]];
        if (fr.y <= 0) {
            null_move = 1;
            break;
        }
        const int4 op = a.flexopt[fr.z + pickw(w[6], fr.y) - a.base[kLFopt]];
        pre.ri = fr.x;
        pre.br_off = op.y;
        pre.br_cnt = op.z;
        break;
    }
    case kLocal: {
        // Molecule::make_local_moves (src/Molecule.cpp:415-448): Bernoulli(0.5) picks a
        // crankshaft (1) or a local translation (0) of one residue.
        kind = (w[5] < 2147483648u) ? 1 : 0;
        if (kind == 0) {
            if (mol.nlocal == 0) {
                null_move = 1;
                break;
            }
            pre.ri = a.localres[mol.local_off + pickw(w[6], mol.nlocal) - a.base[kLLocal]];
            const float3 u = normalized(dx, dy, dz);
            pre.R[0] = u.x, pre.R[1] = u.y, pre.R[2] = u.z;
        } else {
            if (mol.ncrank == 0) {
                null_move = 1;
                break;
            }
            const int ri = a.crankres[mol.crank_off + pickw(w[6], mol.ncrank) - a.base[kLCrank]];
            if (ri < 1 || ri + 1 >= mol.count) {  // needs both backbone neighbours in the array
                null_move = 1;
                break;
            }
            pre.ri = ri;
            flip = w[7] < 2147483648u;
        }
        break;
    }
    }
    pre.bits = type | (kind << 4) | (null_move << 8) | (flip << 9);
    pre.w_metro = w[8];
    pre.w_stage1 = w[9];
}

// The move of this step from its draw-only part and the current state: the centre,
// the translation and its wrap, the flex pivot, the crankshaft rotation.
template <bool RES>
__device__ void finish_move(const DevSim &S, const DevMol *mols, const float4 *CEN, const float4 *P, float tstep,
                            const float4 rsc, const MovePre &pre, MoveDesc &mv)
{
    const int m = pre.m;
    const DevMol &mol = mols[m];
    const int ptype = pre.bits & 15, pkind = (pre.bits >> 4) & 15, pnull = (pre.bits >> 8) & 1,
              pflip = (pre.bits >> 9) & 1;
    mv.m = m;
    mv.start = mol.start;
    mv.n = mol.count;
    mv.flexible = (mol.flags & kMolFlexible) != 0;
    mv.nintra = mol.nintra;
    mv.type = ptype;
    mv.kind = pkind;
    mv.ri = pre.ri;
    mv.br_off = pre.br_off;
    mv.br_cnt = pre.br_cnt;
    mv.null_move = pnull;
    mv.wrapped = 0;
    mv.w_metro = pre.w_metro;
    mv.w_stage1 = pre.w_stage1;
    const float box = S.box;
    const float4 c = ld_state<RES>(&CEN[m]);
    mv.cx = c.x, mv.cy = c.y, mv.cz = c.z;
    mv.wcx = c.x, mv.wcy = c.y, mv.wcz = c.z;
    const float4 *Pm = P + mv.start;
    switch (ptype) {
    case kTranslate:
        mv.vx = pre.R[0] * tstep, mv.vy = pre.R[1] * tstep, mv.vz = pre.R[2] * tstep;
        mv.wcx = wrapf(c.x + mv.vx, box);
        mv.wcy = wrapf(c.y + mv.vy, box);
        mv.wcz = wrapf(c.z + mv.vz, box);
        break;
    case kRotate:
#pragma unroll
        for (int k = 0; k < 9; ++k)
            mv.R[k] = pre.R[k];
        break;
    case kFlex: {
        if (pnull)
            break;
#pragma unroll
        for (int k = 0; k < 9; ++k)
            mv.R[k] = pre.R[k];
        const float4 p = ld_state<RES>(&Pm[pre.ri]);
        mv.px = p.x, mv.py = p.y, mv.pz = p.z;
        break;
    }
    case kLocal: {
        if (pnull)
            break;
        float vx, vy, vz;
        if (pkind == 0) {
            const float s = (float)((double)0.1f * (double)tstep);
            vx = pre.R[0] * s, vy = pre.R[1] * s, vz = pre.R[2] * s;
        } else {
            const int ri = pre.ri;
            const float4 pm = ld_state<RES>(&Pm[ri - 1]);
            const float4 p0 = ld_state<RES>(&Pm[ri]);
            const float4 pp = ld_state<RES>(&Pm[ri + 1]);
            const float3 ax = normalized(pp.x - pm.x, pp.y - pm.y, pp.z - pm.z);
            float Rm[9];
            axis_angle_matrix_sc(pflip ? rsc.z : rsc.x, pflip ? rsc.w : rsc.y, ax.x, ax.y, ax.z, true, Rm);
            const float3 rr = rot_apply(Rm, p0.x - pm.x, p0.y - pm.y, p0.z - pm.z);
            vx = (rr.x + pm.x) - p0.x;
            vy = (rr.y + pm.y) - p0.y;
            vz = (rr.z + pm.z) - p0.z;
        }
        // Molecule::translate(v, ri) (src/Molecule.cpp:274-301)
        const float nf = (float)mv.n;
        mv.vx = vx, mv.vy = vy, mv.vz = vz;
        mv.fx = vx / nf, mv.fy = vy / nf, mv.fz = vz / nf;
        const float ncx = c.x + mv.fx, ncy = c.y + mv.fy, ncz = c.z + mv.fz;
        const float wx = wrapf(ncx, box), wy = wrapf(ncy, box), wz = wrapf(ncz, box);
        mv.wrapped = (wx != ncx) || (wy != ncy) || (wz != ncz);
        mv.wcx = mv.wrapped ? wx : ncx;
        mv.wcy = mv.wrapped ? wy : ncy;
        mv.wcz = mv.wrapped ? wz : ncz;
        break;
    }
    }
}

// ------------------------------------------------------------------ surrogate screening
//
// Delayed acceptance (two-stage Metropolis): stage 1 accepts a proposal with
// min(1, exp(-beta dS)), dS = the surrogate's change of sum_{a<b} f(pose_ab); only
// stage-1 survivors are evaluated exactly, and stage 2 accepts them with
// min(1, exp(-beta (dE - dS))).  The product of the two is a Metropolis-Hastings kernel
// for the exact Boltzmann distribution.  f of every pair is kept in SM (shared memory,
// rebuilt at each launch with the same code that scores proposals), so dS needs only
// the moved molecule's M - 1 new poses: one batch of the MLP per proposal, split over
// the replica's cluster by output columns with activations exchanged through DSMEM.

struct DaView {
    __nv_bfloat16 *W;   // [3][S][kDaWS] rows = this CTA's output units of layers 2..4
    float *W1;          // [S][8]
    float *B;           // [4][S] biases of layers 1..4
    float *W5;          // [S]
    __nv_bfloat16 *H;   // [RP][kDaWS] full activations of the previous layer
    __nv_bfloat16 *hs;  // [2][RP][S] this CTA's outputs (double buffer)
    float *X;           // [RP][8] pose features
    float *P;           // [RP] partial outputs of this CTA
    float *F;           // [RP] predictions
    float *SM;          // [M][M] f of every pair
    float b5;
    int S, RP;
};

__device__ DaView da_view(unsigned char *smem, const SmemLayout &Ly, int C, int max_m)
{
    DaView v;
    v.W = reinterpret_cast<__nv_bfloat16 *>(smem + Ly.daW);
    v.W1 = reinterpret_cast<float *>(smem + Ly.daW1);
    v.B = reinterpret_cast<float *>(smem + Ly.daB);
    v.W5 = reinterpret_cast<float *>(smem + Ly.daW5);
    v.H = reinterpret_cast<__nv_bfloat16 *>(smem + Ly.daH);
    v.hs = reinterpret_cast<__nv_bfloat16 *>(smem + Ly.daHS);
    v.X = reinterpret_cast<float *>(smem + Ly.daX);
    v.P = reinterpret_cast<float *>(smem + Ly.daP);
    v.F = reinterpret_cast<float *>(smem + Ly.daF);
    v.SM = reinterpret_cast<float *>(smem + Ly.daSM);
    v.S = kSurH / C;
    v.RP = da_rows(max_m);
    v.b5 = 0.f;
    return v;
}

// This CTA's slices of the parameters (once per launch).
__device__ void da_load_weights(const EngineArgs &a, DaView &v, int rank, int t, int T)
{
    const int S = v.S, c0 = rank * S;
    const uint4 *wf = reinterpret_cast<const uint4 *>(a.sur_wf);
    for (int idx = t; idx < 3 * S * 32; idx += T) {
        const int l = idx / (S * 32), rem = idx - l * S * 32, r = rem >> 5, q = rem & 31;
        *reinterpret_cast<uint4 *>(v.W + ((size_t)l * S + r) * kDaWS + q * 8) = wf[((size_t)l * kSurH + c0 + r) * 32 + q];
    }
    for (int idx = t; idx < S * kSurIn; idx += T)
        v.W1[idx] = a.sur_P[kOffW1 + c0 * kSurIn + idx];
    for (int idx = t; idx < 4 * S; idx += T) {
        const int l = idx / S, c = idx - l * S;
        v.B[idx] = a.sur_P[sur_b_off(l + 1) + c0 + c];
    }
    for (int c = t; c < S; c += T)
        v.W5[c] = a.sur_P[kOffW5 + c0 + c];
    if (t == 0)
        v.b5 = a.sur_P[kOffB5];
}

// Predictions F[0..R) of the pose rows X[0..R) (R <= RP).  Every CTA of the cluster
// ends with the same values.  Holds cluster barriers: call uniformly across the cluster.
__device__ void da_eval(DaView &v, int R, int C, int t, int T)
{
    cg::cluster_group cl = cg::this_cluster();
    const int S = v.S, RPc = ((R + 15) >> 4) << 4;
    const int warp = t >> 5, lane = t & 31, NW = T >> 5;
    __nv_bfloat16 *cur = v.hs, *nxt = v.hs + v.RP * S;
    // layer 1 in FP32 (same operation order as the training kernel)
    for (int idx = t; idx < RPc * S; idx += T) {
        const int j = idx / S, c = idx - j * S;
        float z = v.B[c];
#pragma unroll
        for (int i = 0; i < kSurIn; ++i)
            z = fmaf(v.W1[c * kSurIn + i], v.X[j * kSurIn + i], z);
        cur[idx] = __float2bfloat16_rn(silu(z));
    }
    cl.sync();
    for (int layer = 2; layer <= 4; ++layer) {
        // all 256 inputs of this layer, gathered from the cluster in rank order
        for (int idx = t; idx < RPc * 32; idx += T) {
            const int j = idx >> 5, col = (idx & 31) * 8, r = col / S, c = col - r * S;
            const __nv_bfloat16 *src = cl.map_shared_rank(cur, r) + j * S + c;
            *reinterpret_cast<uint4 *>(v.H + j * kDaWS + col) = *reinterpret_cast<const uint4 *>(src);
        }
        __syncthreads();
        const __nv_bfloat16 *Wl = v.W + (size_t)(layer - 2) * S * kDaWS;
        const float *bl = v.B + (layer - 1) * S;
        const int mt = RPc >> 4, nt = S >> 3, g = lane >> 2, tig = lane & 3;
        for (int task = warp; task < mt * nt; task += NW) {
            const int tm = task / nt, tn = task - tm * nt;
            const int r0 = tm * 16 + g, n = tn * 8 + g;
            float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
            for (int kt = 0; kt < kSurH / 16; ++kt) {
                const int k0 = kt * 16 + 2 * tig;
                uint32_t af[4], bf[2];
                af[0] = *reinterpret_cast<const uint32_t *>(v.H + r0 * kDaWS + k0);
                af[1] = *reinterpret_cast<const uint32_t *>(v.H + (r0 + 8) * kDaWS + k0);
                af[2] = *reinterpret_cast<const uint32_t *>(v.H + r0 * kDaWS + k0 + 8);
                af[3] = *reinterpret_cast<const uint32_t *>(v.H + (r0 + 8) * kDaWS + k0 + 8);
                bf[0] = *reinterpret_cast<const uint32_t *>(Wl + n * kDaWS + k0);
                bf[1] = *reinterpret_cast<const uint32_t *>(Wl + n * kDaWS + k0 + 8);
                mma_bf16_16816(d, af, bf);
            }
            const int col = tn * 8 + 2 * tig;
            *reinterpret_cast<uint32_t *>(nxt + r0 * S + col) =
                pack_bf16(silu(d[0] + bl[col]), silu(d[1] + bl[col + 1]));
            *reinterpret_cast<uint32_t *>(nxt + (r0 + 8) * S + col) =
                pack_bf16(silu(d[2] + bl[col]), silu(d[3] + bl[col + 1]));
        }
        __nv_bfloat16 *tmp = cur;
        cur = nxt;
        nxt = tmp;
        if (layer < 4)
            cl.sync();
    }
    __syncthreads();
    for (int j = t; j < RPc; j += T) {
        float s = 0.f;
        for (int c = 0; c < S; ++c)
            s = fmaf(__bfloat162float(cur[j * S + c]), v.W5[c], s);
        v.P[j] = s;
    }
    cl.sync();
    for (int j = t; j < R; j += T) {
        float f = 0.f;
        for (int r = 0; r < C; ++r)
            f += cl.map_shared_rank(v.P, r)[j];
        v.F[j] = f + v.b5;
    }
    __syncthreads();
}

template <bool RES>
__device__ __forceinline__ Frame mol_frame(const float4 *Q, const DevMol &mb)
{
    return frame_from(ld_state<RES>(&Q[mb.start + mb.fr0]), ld_state<RES>(&Q[mb.start + mb.fr1]),
                      ld_state<RES>(&Q[mb.start + mb.fr2]));
}

__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }

// Pose rows of the proposal: the moved molecule (new centre and frame) against every
// other molecule, ordered pairs (lower index first); rows up to the next multiple of 16
// are zeroed.
template <bool RES>
__device__ void da_step_features(const DevMol *mols, const float4 *Q, const float4 *CEN, const MoveDesc &mv, int M,
                                 float box, float invbox, float *X, int t, int T)
{
    const int R = M - 1, RPc = ((R + 15) >> 4) << 4;
    for (int j = t; j < RPc; j += T) {
        float *x = X + j * kSurIn;
        if (j >= R) {
#pragma unroll
            for (int i = 0; i < kSurIn; ++i)
                x[i] = 0.f;
            continue;
        }
        const int b = (j < mv.m) ? j : j + 1;
        const DevMol &mm = mols[mv.m];
        float4 q[3] = {ld_state<RES>(&Q[mm.start + mm.fr0]), ld_state<RES>(&Q[mm.start + mm.fr1]),
                       ld_state<RES>(&Q[mm.start + mm.fr2])};
        if (mv.type == kRotate)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float3 rr = rot_apply(mv.R, q[k].x, q[k].y, q[k].z);
                q[k] = make_float4(rr.x, rr.y, rr.z, 0.f);
            }
        const Frame Fm = frame_from(q[0], q[1], q[2]);
        const Frame Fb = mol_frame<RES>(Q, mols[b]);
        const float3 cm = make_float3(mv.wcx, mv.wcy, mv.wcz), cb = f3(ld_state<RES>(&CEN[b]));
        if (mv.m < b)
            pair_features(Fm, cm, Fb, cb, box, invbox, x);
        else
            pair_features(Fb, cb, Fm, cm, box, invbox, x);
    }
}

// SM[a][b] = f(pose_ab) for every pair of the current state, in chunks of RP rows.
template <bool RES>
__device__ void da_init_matrix(DaView &v, const DevMol *mols, const float4 *Q, const float4 *CEN, int M, float box,
                               float invbox, int C, int t, int T)
{
    const int npairs = M * (M - 1) / 2;
    for (int p0 = 0; p0 < npairs; p0 += v.RP) {
        const int R = min(v.RP, npairs - p0);
        for (int j = t; j < v.RP; j += T) {
            float *x = v.X + j * kSurIn;
            if (j >= R) {
                for (int i = 0; i < kSurIn; ++i)
                    x[i] = 0.f;
                continue;
            }
            int pa = 0, rem = p0 + j;
            while (rem >= M - 1 - pa) {
                rem -= M - 1 - pa;
                ++pa;
            }
            const int pb = pa + 1 + rem;
            pair_features(mol_frame<RES>(Q, mols[pa]), f3(ld_state<RES>(&CEN[pa])), mol_frame<RES>(Q, mols[pb]),
                          f3(ld_state<RES>(&CEN[pb])), box, invbox, x);
        }
        __syncthreads();
        da_eval(v, R, C, t, T);
        for (int j = t; j < R; j += T) {
            int pa = 0, rem = p0 + j;
            while (rem >= M - 1 - pa) {
                rem -= M - 1 - pa;
                ++pa;
            }
            const int pb = pa + 1 + rem;
            v.SM[pa * M + pb] = v.F[j];
            v.SM[pb * M + pa] = v.F[j];
        }
        __syncthreads();
    }
    for (int k = t; k < M; k += T)
        v.SM[k * M + k] = 0.f;
    __syncthreads();
}

// ------------------------------------------------------------------ MC kernel

template <bool RES, bool DA, bool QF>
__global__ void __launch_bounds__(kMaxThreads) k_mc(EngineArgs a, int nsteps)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ MoveDesc mv;
    __shared__ FF s_red[kMaxWarps];
    __shared__ float s_fred[3 * kMaxWarps];
    // running total, old/new row of the moved molecule and its internal energy, all as
    // float-float pairs so that the step's decision path has no FP64 arithmetic
    __shared__ FF s_pot, s_old_row, s_intrap, s_intra_new, s_new_row;
    __shared__ int s_accept;
    __shared__ DevSim S;           // this replica's simulation (read by thread 0 mostly)
    __shared__ ReplicaStats st;    // counters, updated by thread 0
    __shared__ double s_ds;        // delayed acceptance: surrogate energy change of the proposal
    __shared__ int s_skip;         // ... 1 when stage 1 rejected it
    __shared__ DAStats s_da;
    __shared__ Lists s_lists;      // static-list views (shared: keeps them out of registers)
    __shared__ DaView s_dv;

    const int C = a.cluster;
    const int t = threadIdx.x, T = blockDim.x, lane = t & 31, warp = t >> 5, NW = T >> 5;
    int rank = 0;
    if (C > 1)
        rank = (int)cg::this_cluster().block_rank();
    const int g = a.rep_order[blockIdx.x / C];
    const int s = a.rep_sim[g];
    if (t == 0) {
        S = a.sims[s];
        st = a.stats[g];
        if (DA)
            s_da = a.dastats[g];
    }
    __syncthreads();
    const int r = g - S.rep_off;
    const int N = S.N, M = S.M;
    const int slice = (a.max_n + C - 1) / C;
    const SmemLayout Ly =
        smem_layout(a.max_mol, slice, a.max_m, a.max_n, RES ? 1 : 0, a.any_flexible, DA ? 1 : 0, C, a.lmax);
    // screening is on for this simulation (uniform over the cluster: one simulation)
    const bool da_on = DA && a.sim_da[s] != 0;
    float *s_table = reinterpret_cast<float *>(smem + Ly.table);
    DevMol *s_mols = reinterpret_cast<DevMol *>(smem + Ly.mols);
    float4 *s_ipos = reinterpret_cast<float4 *>(smem + Ly.ipos);
    float4 *s_irel = reinterpret_cast<float4 *>(smem + Ly.irel);
    int4 *s_iexcl = reinterpret_cast<int4 *>(smem + Ly.iexcl);
    float4 *s_disp = reinterpret_cast<float4 *>(smem + Ly.idisp);
    float2 *s_iq = reinterpret_cast<float2 *>(smem + Ly.iq);
    float4 *s_ipq = reinterpret_cast<float4 *>(smem + Ly.ipq);
    float2 *s_iqq = reinterpret_cast<float2 *>(smem + Ly.iqq);
    unsigned short *s_qpos = reinterpret_cast<unsigned short *>(smem + Ly.QP);
    float *s_rad = reinterpret_cast<float *>(smem + Ly.rad);
    float2 *s_ej = reinterpret_cast<float2 *>(smem + Ly.ej);
    FF *s_rowp = reinterpret_cast<FF *>(smem + Ly.rowp);
    FF *s_row = reinterpret_cast<FF *>(smem + Ly.row);
    MovePre *s_ring = reinterpret_cast<MovePre *>(smem + Ly.ring);

    const long long st0 = S.state_off + (long long)r * N;
    float4 *gP = a.pos + st0;
    float4 *gQ = a.rel + st0;
    float4 *gCEN = a.center + S.molst_off + (long long)r * M;
    double *gE = a.emat + S.emat_off + (long long)r * M * M;
    double *gINTRA = a.intra + S.molst_off + (long long)r * M;
    const float4 *gST = a.rstat + S.res_off;
    const int4 *gEX = a.rexcl + S.res_off;

    // state views: shared-memory copies when resident, global memory otherwise
    float4 *P = RES ? reinterpret_cast<float4 *>(smem + Ly.P) : gP;
    float4 *Q = RES ? reinterpret_cast<float4 *>(smem + Ly.Q) : gQ;
    // static residue records: global float4 (sigma/2, charge, type, molecule) when not
    // resident; resident CTAs pack sigma/2 into P.w, the charge into Q.w and the type
    // into a byte (33 instead of 48 bytes per residue)
    const float4 *ST = gST;
    const unsigned char *TY = RES ? reinterpret_cast<const unsigned char *>(smem + Ly.ST) : nullptr;
    const int4 *EX = (RES && a.any_flexible) ? reinterpret_cast<const int4 *>(smem + Ly.EX) : gEX;
    float4 *CEN = RES ? reinterpret_cast<float4 *>(smem + Ly.CEN) : gCEN;
    // resident copies of the pair matrix, internal energies and row sums are float-float
    // (converted from / to the global doubles at launch start and end)
    FF *EMf = reinterpret_cast<FF *>(smem + Ly.EM);
    FF *INTRAf = reinterpret_cast<FF *>(smem + Ly.INTRA);
    FF *ROWSUMf = reinterpret_cast<FF *>(smem + Ly.ROWSUM);

    load_table(s_table, a.table, t, T);
    for (int k = t; k < M; k += T) {
        DevMol mk = a.mols[S.mol_off + k];
        mk.pair_lanes = pair_lanes(mk.count, N, C, NW);
        s_mols[k] = mk;
    }
    if (RES) {
        float4 *sP = P, *sQ = Q, *sC = CEN;
        unsigned char *sTY = reinterpret_cast<unsigned char *>(smem + Ly.ST);
        for (int i = t; i < N; i += T) {
            const float4 p = __ldcg(&gP[i]), q = __ldcg(&gQ[i]), sr = gST[i];
            sP[i] = make_float4(p.x, p.y, p.z, sr.x);
            sQ[i] = make_float4(q.x, q.y, q.z, sr.y);
            sTY[i] = (unsigned char)__float_as_int(sr.z);
            if (QF)
                s_qpos[i] = a.rqpos[S.res_off + i];
        }
        if (a.any_flexible) {
            int4 *sEX = reinterpret_cast<int4 *>(smem + Ly.EX);
            for (int i = t; i < N; i += T)
                sEX[i] = gEX[i];
        }
        for (int k = t; k < M; k += T) {
            sC[k] = __ldcg(&gCEN[k]);
            INTRAf[k] = ff_from(__ldcg(&gINTRA[k]));
        }
        for (int k = t; k < M * M; k += T)
            EMf[k] = ff_from(__ldcg(&gE[k]));
        __syncthreads();
    }
    // bounding radius of every rigid molecule about its centre (rotations keep it up to
    // float rounding, which kImageMargin covers); flexible molecules change shape and get
    // none.  One warp per molecule, after every thread has stored its DevMol records (the
    // resident load above ends with a barrier; the global-state path has none).
    __syncthreads();
    for (int k = warp; k < M; k += NW) {
        const DevMol &mk = s_mols[k];
        float rmax = 0.0f;
        for (int i = lane; i < mk.count; i += 32) {
            const float4 q = RES ? Q[mk.start + i] : __ldcg(&gQ[mk.start + i]);
            rmax = fmaxf(rmax, sqrtf(fmaf(q.x, q.x, fmaf(q.y, q.y, q.z * q.z))));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        if (lane == 0)
            s_rad[k] = (mk.flags & kMolFlexible) ? __int_as_float(0x7f800000) : rmax;
    }
    __syncthreads();
    const float L = S.box, invL = (S.box != 0.0f) ? 1.0f / S.box : 0.0f;
    const float tstep = a.tstep[g];
    const float rstep = (float)a.rstep[g];
    const float temperature = a.temperature[g];
    const uint32_t key0 = a.seed_lo ^ (0x9E3779B9u * (uint32_t)(g + 1)), key1 = a.seed_hi;
    const unsigned long long step0 = a.stepc[g];
    // sin/cos of +-rstep/2, the replica's fixed rotation half-angles
    float4 rsc;
    sincosf(0.5f * rstep, &rsc.x, &rsc.y);
    sincosf(-(0.5f * rstep), &rsc.z, &rsc.w);
    // pair and error counters live in registers of thread 0 (rank 0 writes them back)
    unsigned long long pairs = 0;
    unsigned errbits = 0;
    if (t == 0)
        s_lists = global_lists(a);
    if (RES && a.any_flexible) {
        // this simulation's static lists into shared memory
        int2 *lb = reinterpret_cast<int2 *>(smem + Ly.lst[0]);
        int4 *la = reinterpret_cast<int4 *>(smem + Ly.lst[1]);
        int4 *lt = reinterpret_cast<int4 *>(smem + Ly.lst[2]);
        float4 *ltv = reinterpret_cast<float4 *>(smem + Ly.lst[3]);
        float4 *lts = reinterpret_cast<float4 *>(smem + Ly.lst[4]);
        int2 *li = reinterpret_cast<int2 *>(smem + Ly.lst[5]);
        int4 *lf = reinterpret_cast<int4 *>(smem + Ly.lst[6]);
        int4 *lfo = reinterpret_cast<int4 *>(smem + Ly.lst[7]);
        int *lbr = reinterpret_cast<int *>(smem + Ly.lst[8]);
        int *ll = reinterpret_cast<int *>(smem + Ly.lst[9]);
        int *lc = reinterpret_cast<int *>(smem + Ly.lst[10]);
        int2 *ltl = reinterpret_cast<int2 *>(smem + Ly.lst[11]);
        const int *B = S.lbase, *Nn = S.lcount;
        for (int k = t; k < Nn[kLBond]; k += T)
            lb[k] = a.bonds[B[kLBond] + k];
        for (int k = t; k < Nn[kLAng]; k += T)
            la[k] = a.angles[B[kLAng] + k];
        for (int k = t; k < Nn[kLTor]; k += T) {
            lt[k] = a.tors[B[kLTor] + k];
            ltv[k] = a.torsV[B[kLTor] + k];
            lts[k] = a.torsS[B[kLTor] + k];
        }
        for (int k = t; k < Nn[kLInd]; k += T)
            li[k] = a.indsub[B[kLInd] + k];
        for (int k = t; k < Nn[kLFlex]; k += T)
            lf[k] = a.flexres[B[kLFlex] + k];
        for (int k = t; k < Nn[kLFopt]; k += T)
            lfo[k] = a.flexopt[B[kLFopt] + k];
        for (int k = t; k < Nn[kLBranch]; k += T)
            lbr[k] = a.branch[B[kLBranch] + k];
        for (int k = t; k < Nn[kLLocal]; k += T)
            ll[k] = a.localres[B[kLLocal] + k];
        for (int k = t; k < Nn[kLCrank]; k += T)
            lc[k] = a.crankres[B[kLCrank] + k];
        for (int k = t; k < Nn[kLTile]; k += T)
            ltl[k] = a.tiles[B[kLTile] + k];
        if (t == 0)
            s_lists = Lists{lb, la, lt, ltv, lts, li, lf, lfo, lbr, ll, lc, ltl,
                            {B[0], B[1], B[2], B[3], B[4], B[5], B[6], B[7], B[8], B[9]}};
    }
    const Lists &Ls = s_lists;
    if (t == 0)
        s_pot = ff_from(__ldcg(&a.potential[g]));
    __syncthreads();
    if (RES) {
        // Local moves keep flexible molecules' internal energies incrementally: re-evaluate
        // them from the state once per launch (bounding the float-float accumulation of the
        // increments) and carry the difference into the running total.  Every CTA of the
        // cluster evaluates the same sums in the same order.
        if (a.any_flexible)
            for (int k = 0; k < M; ++k) {
                if (!(s_mols[k].flags & kMolFlexible))
                    continue;
                const FF v = intra_full_cta(Ls, s_mols[k], P, Q, TY, EX, s_table, L, invL, s_red);
                if (t == 0) {
                    const FF old = INTRAf[k];
                    FF pot = s_pot;
                    ff_add_ff(pot, v);
                    ff_add_ff(pot, FF{-old.hi, -old.lo});
                    s_pot = pot;
                    INTRAf[k] = v;
                }
                __syncthreads();
            }
        // row sums: S[m] = intra[m] + sum_b E[m][b]
        for (int k = t; k < M; k += T) {
            FF v = INTRAf[k];
            for (int b = 0; b < M; ++b)
                if (b != k)
                    ff_add_ff(v, EMf[(long long)k * M + b]);
            ROWSUMf[k] = v;
        }
        __syncthreads();
    }
    DaView &dv = s_dv;
    if (DA) {
        if (t == 0)
            dv = da_view(smem, Ly, C, a.max_m);
        __syncthreads();
        if (da_on) {
            da_load_weights(a, dv, rank, t, T);
            __syncthreads();
            da_init_matrix<RES>(dv, s_mols, Q, CEN, M, L, invL, C, t, T);
            cg::this_cluster().sync();  // no CTA leaves while another reads its shared memory
        }
    }

    // Draw-only decisions of the 32 steps from `first` (local step index), lane k taking
    // step first + k: its Philox words (counter (step, step_hi, word block, 'MC')) and
    // predecide_move, into the ring.  The last warp fills it: the first 32 steps here,
    // the next ones during the Metropolis test of every 32nd step.
    auto fill_ring = [&](int first) {
        const int k = first + lane;
        const unsigned long long ms = step0 + (unsigned long long)k;
        uint32_t w[12];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const U4 ctr{(uint32_t)ms, (uint32_t)(ms >> 32), (uint32_t)b, 0x4D43u};
            const U4 res = philox4x32_10(ctr, key0, key1);
            w[4 * b + 0] = res.x, w[4 * b + 1] = res.y, w[4 * b + 2] = res.z, w[4 * b + 3] = res.w;
        }
        predecide_move(Ls, S, s_mols, rsc, w, s_ring[k & (kRing - 1)]);
    };
    if (warp == NW - 1)
        fill_ring(0);
    __syncthreads();

    for (int step = 0; step < nsteps; ++step) {
        const unsigned long long mcstep = step0 + (unsigned long long)step;
        // ---- the move decision (thread 0): the state-dependent part of the decision
        // whose draw-only part waits in the ring
        if (t == 0) {
            finish_move<RES>(S, s_mols, CEN, P, tstep, rsc, s_ring[step & (kRing - 1)], mv);
            if (RES)
                s_old_row = ROWSUMf[mv.m];
        }
        __syncthreads();
        const int n = mv.n, start = mv.start, type = mv.type, m = mv.m;
        const bool nullm = mv.null_move != 0;
        const bool flexmol = mv.flexible != 0;

        // ---- delayed acceptance, stage 1: the surrogate's energy change of the proposal
        const bool screened = da_on && !nullm && !flexmol;
        bool skip = false;
        if (DA && screened) {
            da_step_features<RES>(s_mols, Q, CEN, mv, M, L, invL, dv.X, t, T);
            __syncthreads();
            da_eval(dv, M - 1, C, t, T);
            if (t == 0) {
                double fnew = 0.0, fold = 0.0;
                for (int j = 0; j < M - 1; ++j) {
                    const int b = (j < m) ? j : j + 1;
                    fnew += (double)dv.F[j];
                    fold += (double)dv.SM[m * M + b];
                }
                const double ds = fnew - fold;
                s_ds = ds;
                const float dsf = (float)ds;
                int pass = 1;
                if (!(dsf < 0.0f)) {
                    const float boltz = expf(-(dsf * kKcal) / (kRgas * temperature));
                    const unsigned long long thr = (unsigned long long)ceilf(boltz * 4294967296.0f);
                    pass = ((unsigned long long)mv.w_stage1 < thr) ? 1 : 0;
                }
                s_skip = !pass;
                s_da.proposals++;
                if (!pass) {
                    s_da.stage1_reject++;
                    st.reject++;
                }
            }
            __syncthreads();
            skip = s_skip != 0;
        }

        if (!skip) {
        if (!RES && warp == 0) {
            // old row from the global matrix (read before anyone commits this step)
            double v = 0.0;
            for (int b = lane; b < M; b += 32)
                if (b != m)
                    v += __ldcg(&gE[(long long)m * M + b]);
            v = warp_sum_d(v);
            if (lane == 0)
                s_old_row = ff_from(v + __ldcg(&gINTRA[m]));
        }

        // ---- proposal of the moved molecule
        for (int i = t; i < n; i += T) {
            const float4 p = ld_state<RES>(&P[start + i]);
            const float4 q = ld_state<RES>(&Q[start + i]);
            const float4 sr = RES ? make_float4(p.w, q.w, __int_as_float((int)TY[start + i]), 0.f) : ST[start + i];
            s_iq[i] = make_float2(sr.y, sr.z);
            if (flexmol)
                s_iexcl[i] = EX[start + i];
            float4 np = p, nq = q;
            if (!nullm) {
                if (type == kTranslate) {
                    np = make_float4(q.x + mv.wcx, q.y + mv.wcy, q.z + mv.wcz, 0.f);
                } else if (type == kRotate) {
                    const float3 rr = rot_apply(mv.R, q.x, q.y, q.z);
                    nq = make_float4(rr.x, rr.y, rr.z, 0.f);
                    np = make_float4(mv.cx + rr.x, mv.cy + rr.y, mv.cz + rr.z, 0.f);
                } else if (type == kLocal) {
                    if (i == mv.ri) {
                        nq = make_float4(q.x + mv.vx, q.y + mv.vy, q.z + mv.vz, 0.f);
                        np = make_float4(p.x + mv.vx, p.y + mv.vy, p.z + mv.vz, 0.f);
                    }
                    nq = make_float4(nq.x - mv.fx, nq.y - mv.fy, nq.z - mv.fz, 0.f);
                    if (mv.wrapped)
                        np = make_float4(nq.x + mv.wcx, nq.y + mv.wcy, nq.z + mv.wcz, 0.f);
                } else {  // kFlex: displacement pass below
                    s_disp[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            np.w = sr.x;
            s_ipos[i] = np;
            s_irel[i] = nq;
            if (QF && !flexmol) {  // the rigid mover also in charged-first order (its final positions)
                const int k = RES ? s_qpos[start + i] : a.rqpos[S.res_off + start + i];
                s_ipq[k] = np;
                s_iqq[k] = make_float2(sr.y, sr.z);
            }
        }
        __syncthreads();
        if (type == kFlex && !nullm) {
            // rotate the branch about the pivot, accumulate the displacement
            for (int k = t; k < mv.br_cnt; k += T) {
                const int i = Ls.branch[mv.br_off + k - Ls.base[kLBranch]];
                const float4 p = s_ipos[i];
                const float3 rr = rot_apply(mv.R, p.x - mv.px, p.y - mv.py, p.z - mv.pz);
                s_disp[i] = make_float4((rr.x + mv.px) - p.x, (rr.y + mv.py) - p.y, (rr.z + mv.pz) - p.z, 0.f);
            }
            __syncthreads();
            float sx = 0.f, sy = 0.f, sz = 0.f;
            for (int i = t; i < n; i += T) {
                const float4 d = s_disp[i];
                sx += d.x, sy += d.y, sz += d.z;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sx += __shfl_xor_sync(0xffffffffu, sx, o);
                sy += __shfl_xor_sync(0xffffffffu, sy, o);
                sz += __shfl_xor_sync(0xffffffffu, sz, o);
            }
            if (lane == 0) {
                s_fred[3 * warp + 0] = sx;
                s_fred[3 * warp + 1] = sy;
                s_fred[3 * warp + 2] = sz;
            }
            __syncthreads();
            if (t == 0) {
                float ax = 0.f, ay = 0.f, az = 0.f;
                for (int w = 0; w < NW; ++w)
                    ax += s_fred[3 * w], ay += s_fred[3 * w + 1], az += s_fred[3 * w + 2];
                const float nf = (float)n;
                mv.fx = ax / nf, mv.fy = ay / nf, mv.fz = az / nf;
                const float ncx = mv.cx + mv.fx, ncy = mv.cy + mv.fy, ncz = mv.cz + mv.fz;
                const float wx = wrapf(ncx, L), wy = wrapf(ncy, L), wz = wrapf(ncz, L);
                mv.wrapped = (wx != ncx) || (wy != ncy) || (wz != ncz);
                mv.wcx = mv.wrapped ? wx : ncx;
                mv.wcy = mv.wrapped ? wy : ncy;
                mv.wcz = mv.wrapped ? wz : ncz;
            }
            __syncthreads();
            for (int i = t; i < n; i += T) {
                const float4 d = s_disp[i];
                float4 p = s_ipos[i], q = s_irel[i];
                q = make_float4((q.x + d.x) - mv.fx, (q.y + d.y) - mv.fy, (q.z + d.z) - mv.fz, 0.f);
                if (mv.wrapped)
                    p = make_float4(q.x + mv.wcx, q.y + mv.wcy, q.z + mv.wcz, p.w);
                else
                    p = make_float4(p.x + d.x, p.y + d.y, p.z + d.z, p.w);
                s_ipos[i] = p;
                s_irel[i] = q;
            }
            __syncthreads();
        }

        // ---- inter-molecule pairs: this CTA's slice of the other residues
        // the other N - n residues split evenly over the cluster for this move (the
        // shared-memory slice buffers are sized for the largest system, slice >= sl)
        const int nother = N - n;
        const int sl = (nother + C - 1) / C;
        const int o0 = rank * sl, o1 = min(nother, o0 + sl);
        const int cnt = max(0, o1 - o0);
        // g lanes per j (each takes every g-th i), floor(32 / g) groups of lanes per warp;
        // the lanes past the last whole group idle
        const int g = s_mols[m].pair_lanes, jw = 32 / g;
        // a rigid mover is read in charged-first order: its first nqm residues take the
        // full pair term, the rest the Lennard-Jones part alone (no charge, no Debye-Hueckel)
        const bool qfirst = QF && !flexmol;
        const float4 *ipv = qfirst ? s_ipq : s_ipos;
        const float2 *iqv = qfirst ? s_iqq : s_iq;
        const int nqm = qfirst ? s_mols[m].nq : n;
        // repulsive crowding: pairs with a crowder (j >= cstart, or a crowder mover) take
        // the crowder term
        const int cstart = (S.crowd_start >= 0) ? S.crowd_start : 0x7fffffff;
        const bool mcrowd = S.crowd_start >= 0 && m >= S.non_crowders;
        const int sub = lane % g, grp = lane / g;
        const int jl = warp * jw + grp, jstride = NW * jw;
        const bool lane_on = grp < jw;
        // Periodic images without a minimum image per pair: each other residue j is moved
        // once to its image nearest the mover's centre.  Where that image lies more than
        // the mover's bounding radius inside the half box around the centre on every
        // axis, no mover residue is more than half a box from it, so the per-pair rule
        // (src/CudaFunctions.cu:321-333) takes exactly that image for every pair and the
        // loop takes the plain differences; on an axis where some j of the warp lies in the
        // outer shell the warp keeps the per-pair minimum image for that axis.  (Flexible
        // movers have no fixed radius: always the per-pair rule.)
        const float hlim = (L != 0.0f && !flexmol) ? 0.5f * L - (s_rad[m] + kImageMargin) : -1.0f;
        auto stat_of = [&](int j) -> float4 {
            return RES ? make_float4(0.f, Q[j].w, __int_as_float((int)TY[j]), 0.f) : ST[j];
        };
        // residue record of this thread's next j, loaded one iteration ahead
        float4 npj = make_float4(0.f, 0.f, 0.f, 0.f), nsj = npj;
        if (lane_on && jl < cnt) {
            const int o = o0 + jl, j = (o < start) ? o : o + n;
            npj = ld_state<RES>(&P[j]);
            nsj = stat_of(j);
        }
        for (int base = 0; base < cnt; base += jstride) {
            const int o = o0 + base + jl;
            const bool valid = lane_on && (base + jl) < cnt;
            const bool crowd = mcrowd || ((o < start) ? o : o + n) >= cstart;
            const float4 pj = npj, sj = nsj;
            if (lane_on && base + jstride + jl < cnt) {
                const int on = o + jstride, jn = (on < start) ? on : on + n;
                npj = ld_state<RES>(&P[jn]);
                nsj = stat_of(jn);
            }
            // j's image nearest the mover's centre (the minimum-image rule applied once;
            // exactly pj where that image is pj itself)
            const float kx = __fadd_rn(__fmaf_rn(pj.x - mv.wcx, invL, 12582912.0f), -12582912.0f);
            const float ky = __fadd_rn(__fmaf_rn(pj.y - mv.wcy, invL, 12582912.0f), -12582912.0f);
            const float kz = __fadd_rn(__fmaf_rn(pj.z - mv.wcz, invL, 12582912.0f), -12582912.0f);
            const float bx = fmaf(-L, kx, pj.x), by = fmaf(-L, ky, pj.y), bz = fmaf(-L, kz, pj.z);
            // the axes on which some j of the warp lies outside the inner region
            const bool use = valid && !crowd && L != 0.0f;
            const int outer = (__any_sync(0xffffffffu, use && !(fabsf(bx - mv.wcx) < hlim)) ? 1 : 0) |
                              (__any_sync(0xffffffffu, use && !(fabsf(by - mv.wcy) < hlim)) ? 2 : 0) |
                              (__any_sync(0xffffffffu, use && !(fabsf(bz - mv.wcz) < hlim)) ? 4 : 0);
            FF acc{0.f, 0.f};
            if (valid && crowd) {
                float p0 = 0.f;
                int cntp = 0;
                for (int i = sub; i < n; i += g) {
                    p0 += crowder_kcal(ipv[i], pj, L, invL);
                    if (++cntp == 32) {
                        ff_add(acc, p0);
                        p0 = 0.f;
                        cntp = 0;
                    }
                }
                ff_add(acc, p0);
            } else if (valid) {
                const float qj = sj.y;
                const float *col = s_table + __float_as_int(sj.z);
                const float sw = RES ? pj.w : sj.x;
                // j's image nearest the mover's centre; the minimum image per pair only on
                // the axes where the warp needs it (most outer warps are outer on one axis)
                const float4 rj = make_float4(bx, by, bz, sw);
                if (outer == 0)
                    mover_spans<0>(ipv, iqv, sub, nqm, n, g, rj, qj, col, L, invL, acc);
                else if (outer == 1)
                    mover_spans<1>(ipv, iqv, sub, nqm, n, g, rj, qj, col, L, invL, acc);
                else if (outer == 2)
                    mover_spans<2>(ipv, iqv, sub, nqm, n, g, rj, qj, col, L, invL, acc);
                else if (outer == 4)
                    mover_spans<4>(ipv, iqv, sub, nqm, n, g, rj, qj, col, L, invL, acc);
                else
                    mover_spans<7>(ipv, iqv, sub, nqm, n, g, make_float4(pj.x, pj.y, pj.z, sw), qj, col, L, invL,
                                   acc);
            }
            // segmented tree sum towards the group's first lane: after the step with offset
            // d, lane sub holds the lanes [sub, min(sub + 2d, g)) of its group
            for (int d = 1; d < g; d <<= 1) {
                const FF w{__shfl_down_sync(0xffffffffu, acc.hi, d), __shfl_down_sync(0xffffffffu, acc.lo, d)};
                if (sub + d < g)
                    ff_add_ff(acc, w);
            }
            if (valid && sub == 0)
                s_ej[o - o0] = make_float2(acc.hi, acc.lo);
        }

        // ---- internal energy of a flexible molecule (intra pairs split over the cluster).
        // A local move of residue ri (resident launches, centre not wrapped) leaves every
        // other position bit for bit unchanged, so the new value is the old one plus
        // new - old over ri's unexcluded pairs, indirect-neighbour corrections and bonded
        // terms.  Other moves recompute it: a rigid rotation or translation changes the
        // float positions, and with them the energy, at rounding level, which a running
        // total must follow to stay within 1e-5 of the energy of its own coordinates.
        FF iacc{0.f, 0.f};
        const bool incr = RES && flexmol && !nullm && type == kLocal && !mv.wrapped;
        if (incr && type == kLocal) {
            const DevMol &mol = s_mols[m];
            const int ri = mv.ri;
            const float4 pn = s_ipos[ri], po4 = P[start + ri];
            const float4 po = make_float4(po4.x, po4.y, po4.z, pn.w);
            const float2 qr = s_iq[ri];
            const int4 er = s_iexcl[ri];
            for (int j = rank * T + t; j < n; j += C * T) {
                if (j == ri || intra_excluded(er, s_iexcl[j]))
                    continue;
                const float4 pj = s_ipos[j];  // unmoved: the state's position
                const float2 qj = s_iq[j];
                ff_add(iacc, pair_kcal(pn, qr, pj, qj, s_table, L, invL) - pair_kcal(po, qr, pj, qj, s_table, L, invL));
            }
            for (int k = rank * T + t; k < mol.nind; k += C * T) {
                const int2 pr = Ls.indsub[mol.ind_off + k - Ls.base[kLInd]];
                if (pr.x != ri && pr.y != ri)
                    continue;
                const int o = (pr.x == ri) ? pr.y : pr.x;
                ff_add(iacc, pair_kcal(po, qr, s_ipos[o], s_iq[o], s_table, L, invL) -
                                 pair_kcal(pn, qr, s_ipos[o], s_iq[o], s_table, L, invL));
            }
            bonded_delta(Ls, mol, s_ipos, P + start, ri, L, invL, rank * T + t, C * T, iacc);
        } else if (flexmol && !incr) {
            // the molecule's active 32 x 32 tiles (on and above the diagonal, holding at least
            // one unexcluded pair); when the cluster has spare warps each tile's i range is
            // split into sf chunks (shorter serial chains)
            const DevMol &mt = s_mols[m];
            const int ntiles = mt.ntile;
            int sf = 1;
            while (sf < 4 && ntiles * sf * 2 <= C * NW)
                sf <<= 1;
            const int il = 32 / sf;
            for (int k = rank * NW + warp; k < ntiles * sf; k += C * NW) {
                const int tk = k / sf, ck = k - tk * sf;
                const int2 tl = Ls.tiles[mt.tile_off + tk - Ls.base[kLTile]];
                const int ta = tl.x, tb = tl.y;
                const int j = tb * 32 + lane;
                float part = 0.f;
                if (j < n) {
                    const float4 pj = s_ipos[j];
                    const float2 qj = s_iq[j];
                    const int4 ej = s_iexcl[j];
                    const int ib = ta * 32 + ck * il;
                    const int iend = min((ta == tb) ? j : n, ib + il);
                    float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
                    int i = ib;
                    // excluded pairs are evaluated and dropped (select, no divergence)
                    for (; i + 3 < iend; i += 4) {
                        const float e0 = pair_kcal(s_ipos[i], s_iq[i], pj, qj, s_table, L, invL);
                        const float e1 = pair_kcal(s_ipos[i + 1], s_iq[i + 1], pj, qj, s_table, L, invL);
                        const float e2 = pair_kcal(s_ipos[i + 2], s_iq[i + 2], pj, qj, s_table, L, invL);
                        const float e3 = pair_kcal(s_ipos[i + 3], s_iq[i + 3], pj, qj, s_table, L, invL);
                        p0 += intra_excluded(s_iexcl[i], ej) ? 0.f : e0;
                        p1 += intra_excluded(s_iexcl[i + 1], ej) ? 0.f : e1;
                        p2 += intra_excluded(s_iexcl[i + 2], ej) ? 0.f : e2;
                        p3 += intra_excluded(s_iexcl[i + 3], ej) ? 0.f : e3;
                    }
                    for (; i < iend; ++i) {
                        const float e0 = pair_kcal(s_ipos[i], s_iq[i], pj, qj, s_table, L, invL);
                        p0 += intra_excluded(s_iexcl[i], ej) ? 0.f : e0;
                    }
                    part = (p0 + p1) + (p2 + p3);
                }
                ff_add(iacc, part);
            }
            {
                // indirect neighbours not caught by the rules above, and the bonded terms:
                // on the cluster's warps that hold no tile task when there are any (so
                // no warp carries both), else over every thread
                const DevMol &mol = s_mols[m];
                const int gw = rank * NW + warp, ntask = ntiles * sf, nwarps = C * NW;
                int b0 = rank * T + t, bstride = C * T;
                if (ntask < nwarps) {
                    b0 = (gw >= ntask) ? (gw - ntask) * 32 + lane : 0x7fffffff;
                    bstride = (nwarps - ntask) * 32;
                }
                for (int k = b0; k < mol.nind; k += bstride) {
                    const int2 pr = Ls.indsub[mol.ind_off + k - Ls.base[kLInd]];
                    ff_add(iacc, -pair_kcal(s_ipos[pr.x], s_iq[pr.x], s_ipos[pr.y], s_iq[pr.y], s_table, L, invL));
                }
                if (b0 != 0x7fffffff)
                    bonded_terms(Ls, mol, s_ipos, L, invL, b0, bstride, iacc);
            }
        }
        __syncthreads();

        // ---- per-molecule partial rows of this CTA's slice (float-float, then double).
        // In a cluster every CTA pushes its partials into every CTA's receive slots
        // (step parity, source rank) before the barrier, so nothing is read remotely after it.
        const int M1 = a.max_m + 1;
        FF *rcv = reinterpret_cast<FF *>(smem + Ly.rcv) + (step & 1) * C * M1;
        for (int b = warp; b < M; b += NW) {
            if (b == m)  // the mover's own row is not read
                continue;
            FF acc{0.f, 0.f};
            const DevMol &mb = s_mols[b];
            const int ob0 = (mb.start < start) ? mb.start : mb.start - n;
            const int lo = max(ob0, o0), hi = min(ob0 + mb.count, o1);
            for (int o = lo + lane; o < hi; o += 32) {
                const float2 e = s_ej[o - o0];
                ff_add_ff(acc, FF{e.x, e.y});
            }
            acc = ff_warp_sum(acc);
            // lane 0's value for every receiver (lanes may differ in the low word)
            const FF v{__shfl_sync(0xffffffffu, acc.hi, 0), __shfl_sync(0xffffffffu, acc.lo, 0)};
            if (C > 1) {
                if (lane < C)
                    cg::this_cluster().map_shared_rank(rcv, lane)[rank * M1 + b] = v;
            } else if (lane == 0) {
                s_rowp[b] = v;
            }
        }
        if (flexmol) {
            const FF v = block_sum_ff_warp0(iacc, s_red);
            if (C > 1) {
                if (t < C)
                    cg::this_cluster().map_shared_rank(rcv, t)[rank * M1 + a.max_m] = v;
            } else if (t == 0) {
                s_intrap = v;
            }
        }
        if (C > 1)
            cg::this_cluster().sync();
        else
            __syncthreads();

        // ---- sum the cluster's partials (fixed rank order, local reads) and take the
        // Metropolis decision, all in warp 0 (no CTA barrier before the decision) and in
        // float-float arithmetic (FP32 pipe; the FP64 unit is slow on this part)
        const FF *rowv = (C > 1) ? s_row : s_rowp;
        if (warp == 0) {
            FF v{0.f, 0.f};
            for (int b = lane; b < M; b += 32) {
                if (b == m)
                    continue;
                FF rb{0.f, 0.f};
                if (C > 1) {
                    for (int k = 0; k < C; ++k)
                        ff_add_ff(rb, rcv[k * M1 + b]);
                    s_row[b] = rb;
                } else {
                    rb = s_rowp[b];
                }
                ff_add_ff(v, rb);
            }
            if (M > 1)
                v = ff_warp_sum(v);
            // the internal energy's partials of the C ranks: lane k holds rank k's, summed
            // in a fixed tree towards lane 0
            FF intra_new{0.f, 0.f};
            if (flexmol) {
                if (C > 1) {
                    if (lane < C)
                        intra_new = rcv[lane * M1 + a.max_m];
                    for (int d = 1; d < C; d <<= 1) {
                        const FF w{__shfl_down_sync(0xffffffffu, intra_new.hi, d),
                                   __shfl_down_sync(0xffffffffu, intra_new.lo, d)};
                        if (lane + d < C)
                            ff_add_ff(intra_new, w);
                    }
                } else {
                    intra_new = s_intrap;
                }
            }
            if (lane == 0) {
                if (flexmol && incr)  // the partials are the change: add the molecule's current value
                    ff_add_ff(intra_new, INTRAf[m]);
                s_intra_new = intra_new;
                FF new_row = v;
                ff_add_ff(new_row, intra_new);
                s_new_row = new_row;
                FF dEf = new_row;  // newPotential - oldPotential = new row - old row
                ff_add_ff(dEf, FF{-s_old_row.hi, -s_old_row.lo});
                float delta = dEf.hi + dEf.lo;
                if (DA && screened)  // stage 2: exact change less the surrogate's
                    delta = (float)(ff_value(dEf) - s_ds);
                int acc = 0;
                if (!isfinite(dEf.hi) || !isfinite(delta)) {
                    // a non-finite energy change (non-finite coordinates): rejected, and
                    // reported in the replica's status bits
                    errbits |= 2u;
                } else if (delta < 0.0f) {
                    acc = 1;
                } else {
                    // u = w / 2^32 < boltz  <=>  w < boltz 2^32, exact in float (power-of-two
                    // scaling) and compared as integers
                    const float boltz = expf(-(delta * kKcal) / (kRgas * temperature));
                    const unsigned long long thr = (unsigned long long)ceilf(boltz * 4294967296.0f);
                    acc = ((unsigned long long)mv.w_metro < thr) ? 2 : 0;
                }
                if (DA && screened) {
                    const double dE = ff_value(dEf), e = dE - s_ds;
                    s_da.stage2_eval++;
                    if (acc)
                        s_da.stage2_accept++;
                    if (fabs(dE) <= (double)a.sur_window && isfinite(e)) {
                        s_da.sum_e2 += e * e;
                        s_da.n_e2++;
                        s_da.win_e2 += e * e;
                        s_da.win_n++;
                    }
                }
                s_accept = acc;
                if (acc) {
                    FF pot = s_pot;
                    ff_add_ff(pot, dEf);
                    s_pot = pot;
                }
                if (acc == 1)
                    st.accept++;
                else if (acc == 2)
                    st.acceptA++;
                else
                    st.reject++;
                pairs += (unsigned long long)n * (unsigned long long)(N - n) +
                         (flexmol ? (incr ? 2ull * (unsigned long long)(n - 1) : (unsigned long long)mv.nintra)
                                  : 0ull);
                if (nullm)
                    errbits |= 1u;
            }
        } else if (warp == NW - 1 && (step & 31) == 15) {
            fill_ring(step + 17);  // the steps of the next block of 32, half a ring ahead
        }
        __syncthreads();

        // ---- commit
        const int acc = s_accept;
        const bool writer = RES || rank == 0;
        if (acc && writer) {
            for (int i = t; i < n; i += T) {
                float4 p = s_ipos[i], q = s_irel[i];  // s_ipos.w = sigma/2
                p.w = RES ? p.w : 0.f;
                q.w = RES ? s_iq[i].x : 0.f;
                P[start + i] = p;
                Q[start + i] = q;
            }
            for (int b = t; b < M; b += T) {
                if (b != m) {
                    if (RES) {
                        const FF nv = rowv[b], ov = EMf[(long long)m * M + b];
                        FF rs = ROWSUMf[b];
                        ff_add_ff(rs, nv);
                        ff_add_ff(rs, FF{-ov.hi, -ov.lo});
                        ROWSUMf[b] = rs;
                        EMf[(long long)m * M + b] = nv;
                        EMf[(long long)b * M + m] = nv;
                    } else {
                        const double nv = ff_value(rowv[b]);
                        gE[(long long)m * M + b] = nv;
                        gE[(long long)b * M + m] = nv;
                    }
                } else {
                    if (RES)
                        ROWSUMf[m] = s_new_row;
                    if (flexmol) {
                        if (RES)
                            INTRAf[m] = s_intra_new;
                        else
                            gINTRA[m] = ff_value(s_intra_new);
                    }
                }
            }
            if (t == 0)
                CEN[m] = make_float4(mv.wcx, mv.wcy, mv.wcz, 0.f);
        }
        if (DA && screened && acc) {  // every CTA keeps its own copy of the surrogate matrix
            for (int j = t; j < M - 1; j += T) {
                const int b = (j < m) ? j : j + 1;
                dv.SM[m * M + b] = dv.F[j];
                dv.SM[b * M + m] = dv.F[j];
            }
        }
        }  // !skip
        // a step the surrogate rejected skipped the Metropolis slot: the ring's refill here
        // (the end-of-step barrier publishes it)
        if (skip && warp == NW - 1 && (step & 31) == 15)
            fill_ring(step + 17);
        // fraction-bound sample (src/Simulation.cpp:1063-1073, src/Replica.cpp:1037-1063)
        const int freq = S.sample_freq;
        if (freq > 0 && (long long)(mcstep % (unsigned long long)freq) == freq - 1 &&
            (long long)mcstep >= (long long)S.sample_after) {
            __syncthreads();
            if (warp == 0) {
                double e = 0.0;
                if (S.nc_mode == 1) {
                    const int nc = S.non_crowders;
                    for (int k = lane; k < nc * nc; k += 32) {
                        const int aa = k / nc, bb = k % nc;
                        if (aa < bb)
                            e += RES ? ff_value(EMf[(long long)aa * M + bb]) : __ldcg(&gE[(long long)aa * M + bb]);
                    }
                    e = warp_sum_d(e);
                } else if (S.nc_mode == 2) {
                    e = ff_value(s_pot);
                }
                int slot = -1;  // this sample's record in the log
                if (lane == 0) {
                    st.samplesSinceLastExchange++;
                    if ((float)e < S.bound_threshold)
                        st.boundSamples++;
                    // the sample's line of boundconformations, when the host keeps them
                    if (a.sample_log != nullptr && rank == 0) {
                        const unsigned k = a.sample_count[g];
                        if ((int)k < a.sample_cap) {
                            a.sample_log[(long long)g * a.sample_cap + k] =
                                SampleRec{e, ff_value(s_pot), temperature, (int)(mcstep + 1 - (unsigned)freq)};
                            a.sample_count[g] = k + 1;
                            slot = (int)k;
                        } else {
                            errbits |= 8u;  // log full: the sample is counted but not recorded
                        }
                    }
                }
                // and its coordinates (the sample PDB of src/Replica.cpp:1082-1087, 1124-1168),
                // when the host keeps them: the leading residues, the non-crowders
                slot = __shfl_sync(0xffffffffu, slot, 0);
                if (slot >= 0 && a.sample_xyz != nullptr) {
                    const int nres = min(a.sample_nres, N);
                    float4 *dst = a.sample_xyz + ((long long)g * a.sample_cap + slot) * a.sample_nres;
                    for (int i = lane; i < nres; i += 32) {
                        const float4 p = ld_state<RES>(&P[i]);
                        dst[i] = make_float4(p.x, p.y, p.z, 0.f);
                    }
                }
            }
        }
        // Resident CTAs own their state copies and every cross-CTA value of a step
        // travels through the receive slots (double-buffered by step parity), so a CTA
        // barrier suffices; without residency rank 0's global commit must be visible
        // to the cluster before the next step reads it.
        if (C > 1 && !RES)
            cg::this_cluster().sync();
        else
            __syncthreads();
    }
    if (C > 1)  // no CTA leaves while another may still read its shared memory
        cg::this_cluster().sync();

    // ---- write back (rank 0)
    if (rank == 0) {
        if (RES) {
            for (int i = t; i < N; i += T) {
                const float4 p = P[i], q = Q[i];
                gP[i] = make_float4(p.x, p.y, p.z, 0.f);
                gQ[i] = make_float4(q.x, q.y, q.z, 0.f);
            }
            for (int k = t; k < M; k += T) {
                gCEN[k] = CEN[k];
                gINTRA[k] = ff_value(INTRAf[k]);
            }
            for (int k = t; k < M * M; k += T)
                gE[k] = ff_value(EMf[k]);
        }
        if (t == 0) {
            a.potential[g] = ff_value(s_pot);
            a.stats[g] = st;
            if (DA)
                a.dastats[g] = s_da;
            a.stepc[g] = step0 + (unsigned long long)nsteps;
            a.pairc[g] += pairs;
            if (errbits)
                atomicOr(&a.errflags[g], errbits);
        }
    }
}

// ------------------------------------------------------------------ initial energies

// CTA (g, a): row a of replica g's matrix for b > a, and the internal energy of a.
__global__ void __launch_bounds__(256) k_init_rows(EngineArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ FF s_red[kMaxWarps];
    const int t = threadIdx.x, T = blockDim.x;
    const int g = blockIdx.x / a.max_m, am = blockIdx.x % a.max_m;
    const int s = a.rep_sim[g];
    const DevSim S = a.sims[s];
    if (am >= S.M)
        return;
    const int r = g - S.rep_off, N = S.N, M = S.M;
    const SmemLayout Ly = smem_layout(a.max_mol, a.max_n, a.max_m, a.max_n, 0, a.any_flexible);
    float *s_table = reinterpret_cast<float *>(smem + Ly.table);
    float4 *s_ipos = reinterpret_cast<float4 *>(smem + Ly.ipos);
    float2 *s_iq = reinterpret_cast<float2 *>(smem + Ly.iq);
    int4 *s_iexcl = reinterpret_cast<int4 *>(smem + Ly.iexcl);
    load_table(s_table, a.table, t, T);
    const DevMol mol = a.mols[S.mol_off + am];
    const long long st0 = S.state_off + (long long)r * N;
    const float4 *stat = a.rstat + S.res_off;
    const int4 *excl = a.rexcl + S.res_off;
    const int n = mol.count, start = mol.start;
    for (int i = t; i < n; i += T) {
        const float4 p = a.pos[st0 + start + i];
        const float4 sr = stat[start + i];
        s_ipos[i] = make_float4(p.x, p.y, p.z, sr.x);
        s_iq[i] = make_float2(sr.y, sr.z);
        s_iexcl[i] = excl[start + i];
    }
    __syncthreads();
    const float L = S.box, invL = (S.box != 0.0f) ? 1.0f / S.box : 0.0f;
    double *E = a.emat + S.emat_off + (long long)r * M * M;
    for (int b = am + 1; b < M; ++b) {
        const DevMol mb = a.mols[S.mol_off + b];
        const bool crowd = S.crowd_start >= 0 && (am >= S.non_crowders || b >= S.non_crowders);
        FF acc{0.f, 0.f};
        for (int jj = t; jj < mb.count; jj += T) {
            const int j = mb.start + jj;
            const float4 pj = a.pos[st0 + j];
            const float4 sj = stat[j];
            const float4 rj = make_float4(pj.x, pj.y, pj.z, sj.x);
            const float2 qj = make_float2(sj.y, sj.z);
            float part = 0.f;
            for (int i = 0; i < n; ++i) {
                part += crowd ? crowder_kcal(s_ipos[i], rj, L, invL)
                              : pair_kcal(s_ipos[i], s_iq[i], rj, qj, s_table, L, invL);
                if ((i & 31) == 31) {
                    ff_add(acc, part);
                    part = 0.f;
                }
            }
            ff_add(acc, part);
        }
        const double v = block_sum_ff(acc, s_red);
        if (t == 0) {
            E[(long long)am * M + b] = v;
            E[(long long)b * M + am] = v;
        }
    }
    if (t == 0)
        E[(long long)am * M + am] = 0.0;
    FF iacc{0.f, 0.f};
    if (mol.flags & kMolFlexible) {
        for (int j = t; j < n; j += T) {
            const float4 pj = s_ipos[j];
            const float2 qj = s_iq[j];
            const int4 ej = s_iexcl[j];
            float part = 0.f;
            for (int i = 0; i < j; ++i) {
                if (!intra_excluded(s_iexcl[i], ej))
                    part += pair_kcal(s_ipos[i], s_iq[i], pj, qj, s_table, L, invL);
                if ((i & 31) == 31) {
                    ff_add(iacc, part);
                    part = 0.f;
                }
            }
            ff_add(iacc, part);
        }
        for (int k = t; k < mol.nind; k += T) {
            const int2 pr = a.indsub[mol.ind_off + k];
            ff_add(iacc, -pair_kcal(s_ipos[pr.x], s_iq[pr.x], s_ipos[pr.y], s_iq[pr.y], s_table, L, invL));
        }
        bonded_terms(global_lists(a), mol, s_ipos, L, invL, t, T, iacc);
    }
    const double v = block_sum_ff(iacc, s_red);
    if (t == 0)
        a.intra[S.molst_off + (long long)r * M + am] = (mol.flags & kMolFlexible) ? v : 0.0;
}

// potential[g] = sum_{a<b} E[a][b] + sum_a intra[a]
__global__ void k_sum_potential(EngineArgs a, double *out)
{
    const int g = blockIdx.x, lane = threadIdx.x;
    const DevSim S = a.sims[a.rep_sim[g]];
    const int r = g - S.rep_off, M = S.M;
    const double *E = a.emat + S.emat_off + (long long)r * M * M;
    const double *in = a.intra + S.molst_off + (long long)r * M;
    double v = 0.0;
    for (int k = lane; k < M * M; k += 32) {
        const int x = k / M, y = k % M;
        if (x < y)
            v += E[k];
    }
    for (int k = lane; k < M; k += 32)
        v += in[k];
    v = warp_sum_d(v);
    if (lane == 0)
        out[g] = v;
}

// ------------------------------------------------------------------ exchange

__device__ void report_slot(ReplicaStats &s, float4 &out)
{
    // Replica::fraction_bound and Replica::acceptance_ratio (src/Replica.cpp:1095-1122)
    s.totalBoundSamples += s.boundSamples;
    s.totalSamples += s.samplesSinceLastExchange;
    s.fractionBound = (float)s.boundSamples / fmaxf(1.0f, (float)s.samplesSinceLastExchange);
    s.accumulativeFractionBound = (float)s.totalBoundSamples / fmaxf(1.0f, (float)s.totalSamples);
    s.boundSamples = 0;
    s.samplesSinceLastExchange = 0;
    s.totalAccept += s.acceptA + s.accept;
    s.totalAcceptReject += s.acceptA + s.accept + s.reject;
    s.acceptanceRatio = (float)(s.acceptA + s.accept) / (float)(s.acceptA + s.accept + s.reject);
    s.accumulativeAcceptanceRatio = (float)s.totalAccept / (float)s.totalAcceptReject;
    s.acceptA = s.accept = s.reject = 0;
    out = make_float4(s.fractionBound, s.accumulativeFractionBound, s.acceptanceRatio, s.accumulativeAcceptanceRatio);
}

// One warp per simulation: the per-temperature report (once sampling has started),
// then the even/odd exchange sweep.  Lanes take temperatures (report) and neighbour
// pairs (exchange) in parallel: the pairs of one sweep are disjoint, so every swap
// touches its own two slots.
__global__ void k_exchange(EngineArgs a, int total_replicas, int steps_per_block)
{
    const int s = blockIdx.x, lane = threadIdx.x;
    const DevSim S = a.sims[s];
    int *st = a.sim_state + 4 * s;
    const int x = st[1];
    const int R = S.R;
    // delayed acceptance: fall back to the plain test when the surrogate's error over
    // the block's second-stage evaluations drifts past the threshold
    if (a.da && a.sim_da[s]) {
        double e2 = 0.0;
        unsigned long long cnt = 0;
        for (int k = lane; k < R; k += 32) {
            DAStats &d = a.dastats[S.rep_off + k];
            e2 += d.win_e2;
            cnt += d.win_n;
            d.win_e2 = 0.0;
            d.win_n = 0;
        }
        for (int o = 16; o > 0; o >>= 1) {
            e2 += __shfl_xor_sync(0xffffffffu, e2, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0 && cnt >= (unsigned long long)a.sur_min && e2 > (double)a.sur_thr2 * (double)cnt)
            a.sim_da[s] = 0;
    }
    // reporting happens when sampling has started (src/Simulation.cpp:751-768)
    if ((long long)steps_per_block * x >= (long long)S.sample_after && x < a.report_capacity) {
        for (int tt = lane; tt < R; tt += 32) {
            const int slot = a.slot_of_t[S.rep_off + tt];
            float4 o;
            report_slot(a.stats[S.rep_off + slot], o);
            a.report[(long long)x * total_replicas + S.rep_off + tt] = o;
        }
    }
    __syncwarp();  // the sweep swaps statistics the report has just updated
    int exchanges = 0, tests = 0;
    const int offset = st[0];
    for (int ti = offset + 2 * lane; ti < R - 1; ti += 64) {
        const int i = a.slot_of_t[S.rep_off + ti], j = a.slot_of_t[S.rep_off + ti + 1];
        const int gi = S.rep_off + i, gj = S.rep_off + j;
        const double Ti = a.temperature[gi], Tj = a.temperature[gj];
        const double delta =
            (1.0 / Ti - 1.0 / Tj) * (a.potential[gi] - a.potential[gj]) * (double)(kKcal / kRgas);
        U4 ctr{(uint32_t)x, 0u, (uint32_t)ti, 0x5245u};
        const U4 o = philox4x32_10(ctr, a.seed_lo ^ 0xB5297A4Du, a.seed_hi ^ (0x68E31DA4u * (uint32_t)(s + 1)));
        if (!isfinite(delta)) {
            // a non-finite potential takes no part in exchanges; both slots report it
            atomicOr(&a.errflags[gi], 4u);
            atomicOr(&a.errflags[gj], 4u);
        } else if (u01(o.x) < fmin(1.0, exp(delta))) {
            // Replica::exchangeReplicas: swap temperature, label and statistics
            float tf = a.temperature[gi];
            a.temperature[gi] = a.temperature[gj];
            a.temperature[gj] = tf;
            int ti_ = a.tindex[gi];
            a.tindex[gi] = a.tindex[gj];
            a.tindex[gj] = ti_;
            int lb = a.label[gi];
            a.label[gi] = a.label[gj];
            a.label[gj] = lb;
            ReplicaStats sv = a.stats[gi];
            a.stats[gi] = a.stats[gj];
            a.stats[gj] = sv;
            a.slot_of_t[S.rep_off + a.tindex[gi]] = i;
            a.slot_of_t[S.rep_off + a.tindex[gj]] = j;
            ++exchanges;
        }
        ++tests;
    }
    exchanges = __reduce_add_sync(0xffffffffu, exchanges);
    tests = __reduce_add_sync(0xffffffffu, tests);
    if (lane == 0) {
        st[0] = 1 - offset;
        if (x < a.report_capacity)
            a.exch_report[(long long)x * gridDim.x + s] = make_int2(exchanges, tests);
        st[2] += exchanges;
        st[3] += tests;
        st[1] = x + 1;
    }
}

// Final per-temperature report after the last block (src/Simulation.cpp:834-848).
__global__ void k_final_report(EngineArgs a, int total_replicas, int row)
{
    const int s = blockIdx.x;
    const DevSim S = a.sims[s];
    for (int tt = threadIdx.x; tt < S.R; tt += blockDim.x) {
        const int slot = a.slot_of_t[S.rep_off + tt];
        float4 o;
        report_slot(a.stats[S.rep_off + slot], o);
        if (row < a.report_capacity)
            a.report[(long long)row * total_replicas + S.rep_off + tt] = o;
    }
}

// ------------------------------------------------------------------ surrogate samples

// Training sample `si` = (replica g, molecules a < b, mode): the pose features of the
// pair (a', b) and its exact inter-molecule energy, where a' is molecule a unchanged
// (mode 0) or displaced by one MC proposal of replica g drawn from Philox (mode 1
// translate by the replica's step along a cube-biased direction, mode 2 rotate by its
// angle about such an axis; src/Molecule.cpp:193-221).
__global__ void __launch_bounds__(128) k_pose_samples(EngineArgs a, const int4 *items, uint32_t key0, uint32_t key1,
                                                      float *X, float *Y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ FF s_red[kMaxWarps];
    __shared__ float s_R[9], s_c[3];
    const int si = blockIdx.x, t = threadIdx.x, T = blockDim.x;
    const int4 it = items[si];
    const int g = it.x, ma = it.y, mb = it.z, mode = it.w;
    const DevSim S = a.sims[a.rep_sim[g]];
    const int r = g - S.rep_off, N = S.N, M = S.M;
    const DevMol A = a.mols[S.mol_off + ma], B = a.mols[S.mol_off + mb];
    const long long st0 = S.state_off + (long long)r * N;
    const float4 *Q = a.rel + st0, *P = a.pos + st0;
    const float4 *CEN = a.center + S.molst_off + (long long)r * M;
    const float4 *stat = a.rstat + S.res_off;
    float *s_table = reinterpret_cast<float *>(smem);
    float4 *s_pa = reinterpret_cast<float4 *>(smem + kTableBytes);
    float2 *s_qa = reinterpret_cast<float2 *>(smem + kTableBytes + 16 * a.max_mol);
    const float L = S.box, invL = (S.box != 0.0f) ? 1.0f / S.box : 0.0f;
    load_table(s_table, a.table, t, T);
    if (t == 0) {
        const float4 c = CEN[ma];
        float R[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
        float cx = c.x, cy = c.y, cz = c.z;
        if (mode != 0) {
            const U4 w = philox4x32_10(U4{(uint32_t)si, 0u, 0u, 0x504Fu}, key0, key1);
            const float3 u = normalized(centred(w.x, false), centred(w.y, true), centred(w.z, false));
            if (mode == 1) {
                const float ts = a.tstep[g];
                cx = wrapf(c.x + u.x * ts, L);
                cy = wrapf(c.y + u.y * ts, L);
                cz = wrapf(c.z + u.z * ts, L);
            } else {
                axis_angle_matrix((float)a.rstep[g], u.x, u.y, u.z, true, R);
            }
        }
        for (int k = 0; k < 9; ++k)
            s_R[k] = R[k];
        s_c[0] = cx, s_c[1] = cy, s_c[2] = cz;
    }
    __syncthreads();
    for (int i = t; i < A.count; i += T) {
        const float4 q = Q[A.start + i];
        const float3 rr = (mode == 2) ? rot_apply(s_R, q.x, q.y, q.z) : make_float3(q.x, q.y, q.z);
        const float4 sr = stat[A.start + i];
        s_pa[i] = make_float4(s_c[0] + rr.x, s_c[1] + rr.y, s_c[2] + rr.z, sr.x);
        s_qa[i] = make_float2(sr.y, sr.z);
    }
    __syncthreads();
    FF acc{0.f, 0.f};
    for (int jj = t; jj < B.count; jj += T) {
        const int j = B.start + jj;
        const float4 pj = P[j], sj = stat[j];
        const float4 rj = make_float4(pj.x, pj.y, pj.z, sj.x);
        const float2 qj = make_float2(sj.y, sj.z);
        float part = 0.f;
        for (int i = 0; i < A.count; ++i) {
            part += pair_kcal(s_pa[i], s_qa[i], rj, qj, s_table, L, invL);
            if ((i & 31) == 31) {
                ff_add(acc, part);
                part = 0.f;
            }
        }
        ff_add(acc, part);
    }
    const double e = block_sum_ff(acc, s_red);
    if (t == 0) {
        Y[si] = (float)e;
        float4 q[3] = {Q[A.start + A.fr0], Q[A.start + A.fr1], Q[A.start + A.fr2]};
        if (mode == 2)
            for (int k = 0; k < 3; ++k) {
                const float3 rr = rot_apply(s_R, q[k].x, q[k].y, q[k].z);
                q[k] = make_float4(rr.x, rr.y, rr.z, 0.f);
            }
        const Frame Fa = frame_from(q[0], q[1], q[2]);
        const Frame Fb = frame_from(Q[B.start + B.fr0], Q[B.start + B.fr1], Q[B.start + B.fr2]);
        pair_features(Fa, make_float3(s_c[0], s_c[1], s_c[2]), Fb, f3(CEN[mb]), L, invL, X + (size_t)si * kSurIn);
    }
}

// ------------------------------------------------------------------ launchers

cudaError_t launch_pose_samples(const EngineArgs &a, const int4 *items, int n, uint32_t key0, uint32_t key1, float *X,
                                float *Y, cudaStream_t stream)
{
    const size_t smem = (size_t)kTableBytes + 24 * (size_t)a.max_mol;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_pose_samples, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    k_pose_samples<<<n, 128, smem, stream>>>(a, items, key0, key1, X, Y);
    return cudaGetLastError();
}

// Every instantiation of k_mc a launch can pick: resident or not x delayed acceptance x
// charged-first mover order (the last only without delayed acceptance).
static const std::array<const void *, 6> &mc_kernels()
{
    static const std::array<const void *, 6> k = {
        (const void *)k_mc<true, false, false>, (const void *)k_mc<false, false, false>,
        (const void *)k_mc<true, true, false>,  (const void *)k_mc<false, true, false>,
        (const void *)k_mc<true, false, true>,  (const void *)k_mc<false, false, true>};
    return k;
}

cudaError_t launch_mc_block(const EngineArgs &a, int total_replicas, int nsteps, int threads, size_t smem,
                            cudaStream_t stream)
{
    const int C = a.cluster;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(total_replicas * C);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (C > 1) ? 1 : 0;
    if (C > 8) {  // 16-CTA clusters are a non-portable size: opt in once per kernel
        static bool allowed = false;
        if (!allowed) {
            for (const void *f : mc_kernels()) {
                const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
                if (e != cudaSuccess)
                    return e;
            }
            allowed = true;
        }
    }
    if (a.da) {
        if (a.resident)
            return cudaLaunchKernelEx(&cfg, k_mc<true, true, false>, a, nsteps);
        return cudaLaunchKernelEx(&cfg, k_mc<false, true, false>, a, nsteps);
    }
    if (a.qfirst) {
        if (a.resident)
            return cudaLaunchKernelEx(&cfg, k_mc<true, false, true>, a, nsteps);
        return cudaLaunchKernelEx(&cfg, k_mc<false, false, true>, a, nsteps);
    }
    if (a.resident)
        return cudaLaunchKernelEx(&cfg, k_mc<true, false, false>, a, nsteps);
    return cudaLaunchKernelEx(&cfg, k_mc<false, false, false>, a, nsteps);
}

cudaError_t set_mc_smem_limit(size_t smem)
{
    // The attribute belongs to the kernel, not to an engine: never lower it below what an
    // engine created earlier (and its captured graphs) needs.
    static size_t s_max = 0;
    if (smem <= s_max)
        return cudaSuccess;
    s_max = smem;
    cudaError_t e = cudaSuccess;
    for (const void *f : mc_kernels())
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_init_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e;
}

cudaError_t launch_init_energy(const EngineArgs &a, int total_replicas, size_t smem, double *potential_out,
                               cudaStream_t stream)
{
    k_init_rows<<<total_replicas * a.max_m, 256, smem, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    k_sum_potential<<<total_replicas, 32, 0, stream>>>(a, potential_out);
    return cudaGetLastError();
}

cudaError_t launch_exchange(const EngineArgs &a, int nsims, int total_replicas, int steps_per_block,
                            cudaStream_t stream)
{
    k_exchange<<<nsims, 32, 0, stream>>>(a, total_replicas, steps_per_block);
    return cudaGetLastError();
}

cudaError_t launch_final_report(const EngineArgs &a, int nsims, int total_replicas, int row, cudaStream_t stream)
{
    k_final_report<<<nsims, 32, 0, stream>>>(a, total_replicas, row);
    return cudaGetLastError();
}

}  // namespace cgppd
