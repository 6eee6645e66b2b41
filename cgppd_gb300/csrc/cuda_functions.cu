// cuda_functions.cu -- the drop-in C ABI of the reference's CUDA energy module
// (src/cudaExterns.h:14-90, src/CudaFunctions.cu:20-277, :724-961), rebuilt for sm_103a.
//
// Callers keep the reference's packed layout: float4 pos[P] = (x, y, z, w) with
// w = rigid_domain_uid + bond_fraction (-2 for padding), float4 meta[P] =
// (type, charge, vdW radius, w) with w = molecule_id + chain_fraction (-1 for a
// crowder).  The pair rules are those of the reference's flexible-linker build.
//
// Kernel: one CTA per (y-tile, x-tile) pair of 128-residue tiles on or above the
// diagonal, two (one per 64-residue half of the y tile) for the diagonal pairs.  The x
// tile is decoded once into shared memory (position and radius; the exclusion keys of
// its w fields; charge, type and flags) next to the 20x20 table, and copied in the
// order [charged | uncharged] real residues (padding left out), each part split into
// the residues that cannot form an excluded pair with this CTA's y residues (their keys
// outside the y residues' key ranges) and those that may: the Debye-Hueckel term is
// taken for charged x residues only, and only the second kind takes the exclusion tests.
// Per warp of y residues the tests are dropped altogether when none of its residues can
// meet an excluded pair, or when the others share every x residue's domain (their sums
// are discarded); the crowder forms keep a general loop where pairs may be excluded.
// Two or four threads own each y residue and sweep alternate x residues.  Pair terms
// are FP32, summed per 32 pairs and folded into float-float accumulators, reduced per
// CTA in float-float.  The last CTA to finish (ticket counter) reduces all CTA partials
// in a fixed order, so the total is deterministic.  Scratch (partials + ticket +
// result) is per (device, stream), allocated on first use and reused.
#include <cstdio>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "cgppd_common.cuh"
#include "host/amino_acids.h"
#include "status.h"
#include "cgppd_cuda_functions.h"

using namespace cgppd;

namespace {

// (64-residue tiles, four times the CTAs for a one-wave call, measured no faster:
// 26.5-27.5 us against 24.7 us for a 6 M-pair call, with 12 % more instructions.)
constexpr int kTile = 128;                 // residues per tile side
constexpr int kThreads = 2 * kTile;        // two threads per y residue (four for a half y tile)
constexpr int kWarps = kThreads / 32;

__constant__ float c_boxdim;  // CUDA_setBoxDimension, module state per device
// cgppd_set_repulsive_crowding: the reference's compile-time REPULSIVE_CROWDING
// (src/definitions.h:18) as process-wide module state, read at each launch
std::atomic<int> g_repulsive_crowding{0};

// CTAs are reduced in groups of kGroup: the last CTA of a group to finish sums the
// group's partials, the last group to finish sums the group sums.
constexpr int kGroup = 32;

struct Scratch {
    unsigned *ticket = nullptr;   // group completion counter, self-resetting
    unsigned *flags = nullptr;    // bit 0: residue type index out of range
    double *result = nullptr;     // {LJ raw, DH raw, total kcal/mol}
    double *partials = nullptr;   // 16 bytes per CTA: its LJ and DH sums as float-float
    float4 *gsums = nullptr;      // 16 bytes per group: its LJ and DH sums as float-float
    unsigned *gtickets = nullptr; // CTA completion counter per group, self-resetting
    size_t capacity = 0;          // CTAs the partials can hold
};

// Scratch layout for `cap` CTAs: [ticket, flags | pad to 256] [result: 4 doubles | pad]
// [partials: 16 bytes per CTA] [group sums: 16 bytes per group] [group tickets: 4 bytes
// per group]; the counters (the first 8 bytes and the group tickets) start at zero.
constexpr size_t scratch_groups(size_t cap) { return (cap + kGroup - 1) / kGroup; }
constexpr size_t scratch_gsums_at(size_t cap) { return 512 + 16 * cap; }
constexpr size_t scratch_gtickets_at(size_t cap) { return scratch_gsums_at(cap) + 16 * scratch_groups(cap); }
constexpr size_t scratch_bytes(size_t cap) { return scratch_gtickets_at(cap) + 4 * scratch_groups(cap); }

void scratch_view(unsigned char *base, size_t cap, Scratch &s)
{
    s.ticket = reinterpret_cast<unsigned *>(base);
    s.flags = reinterpret_cast<unsigned *>(base + 4);
    s.result = reinterpret_cast<double *>(base + 256);
    s.partials = reinterpret_cast<double *>(base + 512);
    s.gsums = reinterpret_cast<float4 *>(base + scratch_gsums_at(cap));
    s.gtickets = reinterpret_cast<unsigned *>(base + scratch_gtickets_at(cap));
    s.capacity = cap;
}

std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, Scratch> g_scratch;
std::map<int, const float *> g_bound_table;  // bindLJTexture, per device

__device__ __forceinline__ float frac_int(float w, float &ip)
{
    ip = truncf(w);
    return w - ip;
}

// 1/x on the SFU (PTX rcp.approx.ftz.f32, max relative error about 2^-23).
__device__ __forceinline__ float rcp_sfu(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The Lennard-Jones part of lj_term with the table value m4e = -4 Eij (RT units) and the
// mixed radius sigma_ij: u = m4e s6 (s6 - 1), and 2 Eij - u on the repulsive branch
// (Eij > 0, s6 > 1/2); one multiplication less than lj_term.
__device__ __forceinline__ float lj_m4(float m4e, float sigma_ij, float inv_r2)
{
    const float s2 = sigma_ij * sigma_ij * inv_r2;
    const float s6 = s2 * s2 * s2;
    float u = m4e * fmaf(s6, s6, -s6);
    if (m4e < 0.0f && s6 > 0.5f)
        u = fmaf(-0.5f, m4e, -u);
    return u;
}

// What the charged-first loop needs of its y residue.
struct PairCtx {
    float4 py;
    float yh, yq;             // half radius, charge
    const float *m4row;       // -4 Eij (RT units) row of the y type
    float L, invL;
    int yl, x0, y;            // y's place in its tile, the x tile's first index, y's index
    bool diag, near;
    float ydom, ybond, ychain;
    bool ydom_nz, ybond_nz;
};

// The y residue against a span of the copied x tile, the S threads of a y residue
// taking every S-th x residue of the sequence j, j + S, ... below `end` (returns where
// the sequence continues).  Charged spans take the full term, the others the
// Lennard-Jones part alone (1/r^2 from the SFU reciprocal: no 1/r needed there).
// TESTED spans hold the x residues that may form a pair the reference excludes (same
// rigid domain, same bond, chain neighbours |x - y| < 4, the diagonal tile's lower
// half), with the rules of the general loop: charged spans skip those pairs (a warp's y
// residues mostly share a molecule, so the branch is mostly uniform), the others
// evaluate them two at a time and select them away.
template <bool TESTED>
__device__ __forceinline__ bool pair_excluded(const PairCtx &c, const float4 *s_qk, int j)
{
    if (!TESTED)
        return false;
    const float4 k = s_qk[j];
    const int xi = __float_as_int(k.w);
    return (c.diag && xi <= c.yl) || (c.ydom_nz && k.x == c.ydom) || (c.ybond_nz && k.y == c.ybond) ||
           (c.near && k.z == c.ychain && abs(c.x0 + xi - c.y) < 4);
}

template <bool TESTED, int S>
__device__ __forceinline__ int charged_span(const PairCtx &c, const float4 *s_pq, const float2 *s_qt,
                                            const float4 *s_qk, int j, int end, FF &lj, FF &dh)
{
    const float4 py = c.py;
    const float L = c.L, invL = c.invL;
    float l0 = 0.f, d0 = 0.f;
    int cnt = 0;
    for (; j < end; j += S) {
        if (pair_excluded<TESTED>(c, s_qk, j))
            continue;
        const float4 px = s_pq[j];
        const float2 qt = s_qt[j];
        const float dx = min_image(py.x - px.x, L, invL);
        const float dyy = min_image(py.y - px.y, L, invL);
        const float dz = min_image(py.z - px.z, L, invL);
        const float r2 = fmaf(dx, dx, fmaf(dyy, dyy, dz * dz));
        const float inv_r = rsqrt_sfu(r2);
        const float u = lj_m4(c.m4row[__float_as_int(qt.y)], c.yh + px.w, inv_r * inv_r);
        const float d = dh_term(c.yq * qt.x, r2 * inv_r, inv_r);
        l0 += u;
        d0 += d;
        if (++cnt == 32) {
            ff_add(lj, l0);
            ff_add(dh, d0);
            l0 = d0 = 0.f;
            cnt = 0;
        }
    }
    ff_add(lj, l0);
    ff_add(dh, d0);
    return j;
}

template <bool TESTED, int S>
__device__ __forceinline__ int lj_span(const PairCtx &c, const float4 *s_pq, const float2 *s_qt, const float4 *s_qk,
                                       int j, int end, FF &lj)
{
    const float4 py = c.py;
    const float L = c.L, invL = c.invL;
    float l0 = 0.f, l1 = 0.f;
    int cnt = 0;
    for (; j + S < end; j += 2 * S) {
        const float4 pa = s_pq[j], pb = s_pq[j + S];
        const int ta = __float_as_int(s_qt[j].y), tb = __float_as_int(s_qt[j + S].y);
        const float ax = min_image(py.x - pa.x, L, invL), bx = min_image(py.x - pb.x, L, invL);
        const float ay = min_image(py.y - pa.y, L, invL), by = min_image(py.y - pb.y, L, invL);
        const float az = min_image(py.z - pa.z, L, invL), bz = min_image(py.z - pb.z, L, invL);
        const float ra = fmaf(ax, ax, fmaf(ay, ay, az * az)), rb = fmaf(bx, bx, fmaf(by, by, bz * bz));
        const float ua = lj_m4(c.m4row[ta], c.yh + pa.w, rcp_sfu(ra));
        const float ub = lj_m4(c.m4row[tb], c.yh + pb.w, rcp_sfu(rb));
        l0 += pair_excluded<TESTED>(c, s_qk, j) ? 0.f : ua;
        l1 += pair_excluded<TESTED>(c, s_qk, j + S) ? 0.f : ub;
        if (++cnt == 16) {
            ff_add(lj, l0 + l1);
            l0 = l1 = 0.f;
            cnt = 0;
        }
    }
    for (; j < end; j += S) {
        const float4 pa = s_pq[j];
        const float ax = min_image(py.x - pa.x, L, invL);
        const float ay = min_image(py.y - pa.y, L, invL);
        const float az = min_image(py.z - pa.z, L, invL);
        const float ra = fmaf(ax, ax, fmaf(ay, ay, az * az));
        const float ua = lj_m4(c.m4row[__float_as_int(s_qt[j].y)], c.yh + pa.w, rcp_sfu(ra));
        l0 += pair_excluded<TESTED>(c, s_qk, j) ? 0.f : ua;
    }
    ff_add(lj, l0 + l1);
    return j;
}

// The y residue against the copied x tile: its real residues in the order [charged
// safe | charged tested | uncharged safe | uncharged tested] with the group ends e[0..3]
// (padding after e[3] is not visited); TESTED: the tested groups take the exclusion
// tests (else the warp's y residues need none, and skip_tested residues skip them).
template <int S, bool TESTED>
__device__ __forceinline__ void charged_first_pairs(const PairCtx &c, const float4 *s_pq, const float2 *s_qt,
                                                    const float4 *s_qk, const int *e, int sub, bool skip_tested,
                                                    FF &lj, FF &dh)
{
    // the first index of the sequence j, j + S, ... at or past `end`
    auto past = [](int j, int end) { return j < end ? j + ((end - j + S - 1) / S) * S : j; };
    int j = sub;
    j = charged_span<false, S>(c, s_pq, s_qt, s_qk, j, e[0], lj, dh);
    j = skip_tested ? past(j, e[1]) : charged_span<TESTED, S>(c, s_pq, s_qt, s_qk, j, e[1], lj, dh);
    j = lj_span<false, S>(c, s_pq, s_qt, s_qk, j, e[2], lj);
    if (!skip_tested)
        lj_span<TESTED, S>(c, s_pq, s_qt, s_qk, j, e[3], lj);
}

// One warp's residues' exclusion-key ranges and flags, stored by lane 0 into wk[0..8]:
// [nonzero domain min/max, nonzero bond min/max, chain min/max, molecule min/max] as
// bit patterns, then the OR of the flags (bit 0 padding, bit 1 crowder).  Ranges are of
// the keys' bit patterns: two sets of floats whose bit-pattern ranges are disjoint share
// no value.
__device__ __forceinline__ void warp_keys(int *wk, float dom, float bond, float chain, float mol, int flags)
{
    const int inf = 0x7fffffff;
    // + 0.0f turns -0 into +0: the exclusion tests compare keys as floats, where -0 == +0
    const int d = __float_as_int(dom + 0.0f), b = __float_as_int(bond + 0.0f), c = __float_as_int(chain + 0.0f),
              m = __float_as_int(mol + 0.0f);
    const bool real = (flags & 1) == 0;  // padding records carry no keys
    const int v[8] = {real && dom != 0.f ? d : inf, real && dom != 0.f ? d : -1,
                      real && bond != 0.f ? b : inf, real && bond != 0.f ? b : -1,
                      real ? c : inf, real ? c : -1, real && mol >= 0.f ? m : inf, real && mol >= 0.f ? m : -1};
    int r[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        r[k] = (k & 1) ? __reduce_max_sync(0xffffffffu, v[k]) : __reduce_min_sync(0xffffffffu, v[k]);
    const int f = (int)__reduce_or_sync(0xffffffffu, (unsigned)flags);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            wk[k] = r[k];
        wk[8] = f;
    }
}

constexpr int kKeys = 9;

// Key k of a tile from the nw warps that stored theirs (min for even k, max for odd k,
// OR for the flags, k = 8).
__device__ __forceinline__ int tile_key(const int (*wk)[kKeys], int nw, int k)
{
    int v = wk[0][k];
    for (int w = 1; w < nw; ++w)
        v = (k == 8) ? (v | wk[w][k]) : (k & 1) ? max(v, wk[w][k]) : min(v, wk[w][k]);
    return v;
}

__device__ __forceinline__ bool ranges_disjoint(int amin, int amax, int bmin, int bmax)
{
    return amax < bmin || bmax < amin;  // an empty range (min > max) is disjoint from all
}

// CTAs of a call on nt tiles: every tile pair on or above the diagonal, the nt diagonal
// pairs twice.
__host__ __device__ constexpr int energy_ctas(int nt) { return nt * (nt + 1) / 2 + nt; }

// CTA b -> tile pair (ty <= tx) and y part: part 1, 2 are the halves of the y tile of a
// diagonal pair (CTAs 0 .. 2 nt - 1), part 0 the whole y tile of an off-diagonal pair
// (row-major).
__device__ __forceinline__ void cta_work(int b, int nt, int &ty, int &tx, int &part)
{
    if (b < 2 * nt) {
        part = 1 + (b & 1);
        ty = tx = b >> 1;
        return;
    }
    part = 0;
    int rem = b - 2 * nt;
    ty = 0;
    while (ty < nt - 1 && rem >= nt - ty - 1) {  // row ty holds nt - ty - 1 such pairs
        rem -= nt - ty - 1;
        ++ty;
    }
    tx = ty + 1 + rem;
}

// kNC: non-crowder pairs of different molecules only (E_TiledKernelNC).  kRC: the
// REPULSIVE_CROWDING form of the crowder pairs.
template <bool kNC, bool kRC>
__global__ void __launch_bounds__(kThreads) k_tile_energy(const float4 *__restrict__ pos, const float4 *__restrict__ meta,
                                                          int P, int nt, const float *__restrict__ lj_raw,
                                                          double *__restrict__ partials, unsigned *__restrict__ ticket,
                                                          unsigned *__restrict__ flags, double *__restrict__ result,
                                                          float4 *__restrict__ gsums, unsigned *__restrict__ gtickets,
                                                          float *__restrict__ async_out, int async_count)
{
    // x tile, decoded once per CTA: position and vdW radius; exclusion keys (rigid
    // domain, bond fraction, chain fraction, molecule id); charge, type, flags
    __shared__ float4 s_px[kTile];
    __shared__ float4 s_xk[kTile];
    __shared__ float4 s_xm[kTile];
    __shared__ float s_eij[400];
    __shared__ float s_m4[400];   // -4 Eij in RT units (the clean-tile loop's form)
    __shared__ FF s_red[2][kWarps];
    __shared__ bool s_last, s_last_group;
    // the x tile's real residues again in charged-first order (position + half radius,
    // charge + type), for the charged-first loop
    __shared__ float4 s_pq[kTile];
    __shared__ float2 s_qt[kTile];
    // ... and their exclusion keys (domain, bond, chain, original index), for the pairs
    // that take the exclusion tests
    __shared__ float4 s_qk[kTile];
    // per-warp key ranges and flags of the x tile and of this CTA's y residues (warp_keys)
    __shared__ int s_wk[2][kTile / 32][kKeys];
    // per x warp, key ranges of its residues that take the exclusion tests: [nonzero domain
    // min/max, nonzero bond min/max, chain min/max, domain min/max] (bit patterns)
    __shared__ int s_tk[kTile / 32][8];
    // counts of the x tile's copy groups per warp (charged safe, charged tested, uncharged
    // safe, uncharged tested, padding)
    __shared__ int s_gcnt[kTile / 32][5];

    // a dependent launch (see launch_energy): nothing global is touched before the
    // stream's previous kernel has completed
    asm volatile("griddepcontrol.wait;" ::: "memory");
    int ty, tx, part;
    cta_work(blockIdx.x, nt, ty, tx, part);
    const int t = threadIdx.x;
    // y residue of this thread (place in its tile) and its share of the x tile: the
    // whole y tile with two threads per residue, or one half with four
    const int ny = part ? kTile / 2 : kTile;
    const int yl = (part ? (part - 1) * (kTile / 2) : 0) + (t & (ny - 1)), sub = t / ny;
    // the x and y records first, so that their loads overlap the table's
    const int x0 = tx * kTile;
    const int y = ty * kTile + yl;
    float4 px_in = make_float4(0.f, 0.f, 0.f, kPadder), mx_in = make_float4(0.f, 0.f, 0.f, 0.f);
    if (t < kTile && x0 + t < P) {
        px_in = pos[x0 + t];
        mx_in = meta[x0 + t];
    }
    const float4 py = (y < P) ? pos[y] : make_float4(0.f, 0.f, 0.f, kPadder);
    const float4 my = (y < P) ? meta[y] : make_float4(0.f, 0.f, 0.f, 0.f);
    // the async form's output other than the total: zeroed by every CTA, a slice each
    if (async_out != nullptr && async_count > 1) {
        const int per = (async_count - 1 + (int)gridDim.x - 1) / (int)gridDim.x;
        const int k0 = 1 + (int)blockIdx.x * per, k1 = min(async_count, k0 + per);
        for (int k = k0 + t; k < k1; k += kThreads)
            async_out[k] = 0.0f;
    }

    for (int k = t; k < 400; k += kThreads)
    {
        const float e = kLambda * (lj_raw[k] - kE0);  // Eij in RT units, as the kernel forms it
        s_eij[k] = e;
        s_m4[k] = -4.0f * e;
    }
    __syncthreads();
    // residue types are checked once per residue (0..19; padding is excluded anyway):
    // the pair loop then indexes the table without a bounds test
    unsigned bad = 0;
    unsigned qb = 0, rb = 0;  // this x warp's charged and real (not padding) residues
    if (t < kTile) {
        const float4 px = px_in, mx = mx_in;
        float xdom, xmol;
        const float xbond = frac_int(px.w, xdom);
        const float xchain = frac_int(mx.w, xmol);
        const bool pad = px.w == kPadder;
        const bool crowd = mx.w == kCrowder;
        int xt = __float2int_rn(mx.x);
        if ((unsigned)xt >= 20u) {
            // crowders read no table entry where they are excluded (kNC) or repulsive
            // only (kRC; the reference then gives them the type -1)
            bad |= (pad || (crowd && (kNC || kRC))) ? 0u : 1u;
            xt = 0;
        }
        const int xflags = (pad ? 1 : 0) | (crowd ? 2 : 0);
        s_px[t] = make_float4(px.x, px.y, px.z, mx.z);
        s_xk[t] = make_float4(xdom, xbond, xchain, xmol);
        s_xm[t] = make_float4(mx.y, __int_as_float(xt), __int_as_float(xflags), 0.f);
        warp_keys(s_wk[0][t >> 5], xdom, xbond, xchain, xmol, xflags);
        qb = __ballot_sync(0xffffffffu, !pad && mx.y != 0.0f);
        rb = __ballot_sync(0xffffffffu, !pad);
    }
    if (sub == 0) {
        float ydom0, ymol0;
        const float ybond0 = frac_int(py.w, ydom0);
        const float ychain0 = frac_int(my.w, ymol0);
        warp_keys(s_wk[1][t >> 5], ydom0, ybond0, ychain0, ymol0,
                  (py.w == kPadder ? 1 : 0) | (my.w == kCrowder ? 2 : 0));
    }
    __syncthreads();
    const int nyw = ny / 32;  // warps that stored y keys
    // No pair of the two tiles can be excluded when they are different tiles (where
    // crowders are treated apart, without crowders), their nonzero rigid-domain and bond
    // keys share no value, and the chain rule (|x - y| < 4 on one chain) cannot apply
    // (tiles two or more apart, or no common chain key); for the non-crowder sum also no
    // common molecule.  Disjoint key ranges show the first ones.  (Padding carries no
    // keys and is left out of the charged-first copy.)
    // (Only the crowder forms decide per tile pair; the default potential per x residue.)
    bool clean = false;
    if (kNC || kRC) {
        auto kx = [&](int k) { return tile_key(s_wk[0], kTile / 32, k); };
        auto ky = [&](int k) { return tile_key(s_wk[1], nyw, k); };
        clean = tx != ty && ((kx(8) | ky(8)) & 2) == 0;
        if (kNC)
            clean = clean && ranges_disjoint(kx(6), kx(7), ky(6), ky(7));
        else
            clean = clean && ranges_disjoint(kx(0), kx(1), ky(0), ky(1)) && ranges_disjoint(kx(2), kx(3), ky(2), ky(3)) &&
                    (tx - ty >= 2 || ranges_disjoint(kx(4), kx(5), ky(4), ky(5)));
    }
    // The default potential always takes the charged-first loop: each x residue that may
    // form an excluded pair with this CTA's y residues (a diagonal tile; its nonzero domain
    // or bond key inside the y residues' ranges; its chain key inside theirs where the
    // chain rule can apply) is tested per pair, the others are not.  The crowder forms
    // take it for clean tile pairs only, the general loop otherwise.
    const bool cfirst = clean || (!kNC && !kRC);
    int e[4] = {0, 0, 0, 0};  // ends of the copy's groups (see charged_first_pairs)
    if (cfirst) {
        // the x tile's real residues in the order [charged safe | charged tested | uncharged
        // safe | uncharged tested] (stable within each group), padding after them: the
        // Debye-Hueckel term is then taken for the charged x residues only
        unsigned gm[5] = {0u, 0u, 0u, 0u, 0u};  // this x warp's residues by group
        if (t < kTile) {
            bool u = false;
            if (!kNC && !kRC) {
                const float4 xk = s_xk[t];
                const int d = __float_as_int(xk.x + 0.0f), b = __float_as_int(xk.y + 0.0f),
                          ch = __float_as_int(xk.z + 0.0f);
                u = tx == ty || (xk.x != 0.f && tile_key(s_wk[1], nyw, 0) <= d && d <= tile_key(s_wk[1], nyw, 1)) ||
                    (xk.y != 0.f && tile_key(s_wk[1], nyw, 2) <= b && b <= tile_key(s_wk[1], nyw, 3)) ||
                    (tx - ty <= 1 && tile_key(s_wk[1], nyw, 4) <= ch && ch <= tile_key(s_wk[1], nyw, 5));
            }
            const unsigned ub = __ballot_sync(0xffffffffu, u);
            {
                const float4 xk = s_xk[t];
                const bool tst = u && ((rb >> (t & 31)) & 1u);
                const int inf = 0x7fffffff;
                const int d = __float_as_int(xk.x + 0.0f), b = __float_as_int(xk.y + 0.0f),
                          ch = __float_as_int(xk.z + 0.0f);
                const int v[8] = {tst && xk.x != 0.f ? d : inf, tst && xk.x != 0.f ? d : -1,
                                  tst && xk.y != 0.f ? b : inf, tst && xk.y != 0.f ? b : -1,
                                  tst ? ch : inf, tst ? ch : -1, tst ? d : inf, tst ? d : -1};
                int r[8];
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    r[k] = (k & 1) ? __reduce_max_sync(0xffffffffu, v[k]) : __reduce_min_sync(0xffffffffu, v[k]);
                if ((t & 31) == 0)
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        s_tk[t >> 5][k] = r[k];
            }
            gm[0] = qb & ~ub;
            gm[1] = qb & ub;
            gm[2] = rb & ~qb & ~ub;
            gm[3] = rb & ~qb & ub;
            gm[4] = ~rb;
            if ((t & 31) == 0)
#pragma unroll
                for (int g = 0; g < 5; ++g)
                    s_gcnt[t >> 5][g] = __popc(gm[g]);
        }
        __syncthreads();
        int acc = 0;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            for (int w = 0; w < kTile / 32; ++w)
                acc += s_gcnt[w][g];
            e[g] = acc;
        }
        if (t < kTile) {
            // this residue's group g, its members in this warp (mg) and the group's start
            const int w0 = t >> 5;
            const unsigned me = 1u << (t & 31);
            const int g = (gm[0] & me) ? 0 : (gm[1] & me) ? 1 : (gm[2] & me) ? 2 : (gm[3] & me) ? 3 : 4;
            const unsigned mg = g == 0 ? gm[0] : g == 1 ? gm[1] : g == 2 ? gm[2] : g == 3 ? gm[3] : gm[4];
            int k = (g == 0 ? 0 : g == 1 ? e[0] : g == 2 ? e[1] : g == 3 ? e[2] : e[3]) + __popc(mg & (me - 1u));
            for (int w = 0; w < w0; ++w)
                k += s_gcnt[w][g];
            const float4 xm = s_xm[t];
            float4 pw = s_px[t];
            pw.w *= 0.5f;  // half the radius: sigma_ij = half_y + half_x
            s_pq[k] = pw;
            s_qt[k] = make_float2(xm.x, xm.y);
            const float4 xk = s_xk[t];
            s_qk[k] = make_float4(xk.x, xk.y, xk.z, __int_as_float(t));
        }
        __syncthreads();
    }

    FF lj{0.f, 0.f}, dh{0.f, 0.f};
    const bool ycrowd = my.w == kCrowder;
    const bool active = (py.w > kPadder) && (!kNC || !ycrowd);
    // Default potential, per y residue against the tested x residues (keys s_tk): it is
    // safe when none of its keys can meet theirs (an off-diagonal tile; its nonzero domain
    // and bond keys outside their ranges; its chain key too where the chain rule can
    // apply), and all-excluded when they all share its nonzero domain.  A warp whose y
    // residues are all one or the other takes the tested groups without tests (the
    // all-excluded residues skip them); otherwise it tests per pair.
    bool skip_tested = false, wtested = true;
    if (!kNC && !kRC && cfirst) {
        // the tested residues' key k: lane k combines the x warps' values, then a broadcast
        int tk = 0;
        if ((t & 31) < 8) {
            const int k = t & 31;
            tk = s_tk[0][k];
            for (int w = 1; w < kTile / 32; ++w)
                tk = (k & 1) ? max(tk, s_tk[w][k]) : min(tk, s_tk[w][k]);
        }
        int T[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            T[k] = __shfl_sync(0xffffffffu, tk, k);
        float yd0, ym0;
        const float yb0 = frac_int(py.w, yd0);
        const float yc0 = frac_int(my.w, ym0);
        const int yd = __float_as_int(yd0 + 0.0f), yb = __float_as_int(yb0 + 0.0f), yc = __float_as_int(yc0 + 0.0f);
        const bool lsafe = tx != ty && !(yd0 != 0.f && T[0] <= yd && yd <= T[1]) &&
                           !(yb0 != 0.f && T[2] <= yb && yb <= T[3]) && !(tx - ty <= 1 && T[4] <= yc && yc <= T[5]);
        skip_tested = yd0 != 0.f && T[6] == yd && T[7] == yd;
        wtested = __any_sync(0xffffffffu, active && !lsafe && !skip_tested);
    }
    if (active) {
        const float L = c_boxdim;
        const float invL = (L != 0.0f) ? 1.0f / L : 0.0f;
        float ydom, ymol;
        const float ybond = frac_int(py.w, ydom);
        const float ychain = frac_int(my.w, ymol);
        const bool ydom_nz = ydom != 0.f, ybond_nz = ybond != 0.f;
        const bool diag = (tx == ty);
        // the chain rule (|x - y| < 4) can only hold on and next to the diagonal
        const bool near = (tx - ty) <= 1;
        int yt = __float2int_rn(my.x);
        if ((unsigned)yt >= 20u) {
            bad |= (kRC && ycrowd) ? 0u : 1u;
            yt = 0;
        }
        const float *erow = s_eij + 20 * yt;
        const float yq = my.y, ys = my.z;
        if (cfirst) {
            const PairCtx c{py, 0.5f * ys, yq, s_m4 + 20 * yt, L, invL, yl, x0, y, diag, near, ydom, ybond, ychain,
                            ydom_nz, ybond_nz};
            if (wtested) {
                if (part == 0)
                    charged_first_pairs<2, true>(c, s_pq, s_qt, s_qk, e, sub, false, lj, dh);
                else
                    charged_first_pairs<4, true>(c, s_pq, s_qt, s_qk, e, sub, false, lj, dh);
            } else {
                if (part == 0)
                    charged_first_pairs<2, false>(c, s_pq, s_qt, s_qk, e, sub, skip_tested, lj, dh);
                else
                    charged_first_pairs<4, false>(c, s_pq, s_qt, s_qk, e, sub, skip_tested, lj, dh);
            }
        }
        // the general loop: this thread's share of the x tile, kTile / S consecutive residues
        const int jw = part ? kTile / 4 : kTile / 2, jb0 = sub * jw;
        for (int jb = jb0; !cfirst && jb < jb0 + jw; jb += 32) {
            float l0 = 0.f, l1 = 0.f, d0 = 0.f, d1 = 0.f;
            // branch-free: every pair is evaluated and the excluded ones (padding, the
            // pair itself on the diagonal: possibly inf / NaN) are selected away
#pragma unroll 4
            for (int jj = 0; jj < 32; ++jj) {
                const int j = jb + jj;
                const float4 xk = s_xk[j];
                const float4 xm = s_xm[j];
                const float4 px = s_px[j];
                const int xflags = __float_as_int(xm.z);
                bool excl = (xflags & 1) || (diag && j <= yl);
                if (kNC)
                    excl = excl || (xflags & 2) || xk.w == ymol;
                else
                    excl = excl || (ydom_nz && xk.x == ydom) || (ybond_nz && xk.y == ybond) ||
                           (near && xk.z == ychain && abs(x0 + j - y) < 4);
                const float dx = min_image(py.x - px.x, L, invL);
                const float dyy = min_image(py.y - px.y, L, invL);
                const float dz = min_image(py.z - px.z, L, invL);
                const float r2 = fmaf(dx, dx, fmaf(dyy, dyy, dz * dz));
                const float inv_r = rsqrt_sfu(r2);
                const float r = r2 * inv_r;
                float lt = lj_term(erow[__float_as_int(xm.y)], (ys + px.w) * 0.5f, inv_r * inv_r);
                float dt = dh_term(yq * xm.x, r, inv_r);
                if (kRC && (ycrowd || (xflags & 2))) {
                    // REPULSIVE_CROWDING (src/CudaFunctions.cu:335-338, :492-498):
                    // (6/r)^12 in RT units below 15 A, no Debye-Hueckel term
                    const float sc = 6.0f * inv_r, s2 = sc * sc, s6 = s2 * s2 * s2;
                    lt = (r < kRepulsiveCutoff) ? s6 * s6 : 0.f;
                    dt = 0.f;
                }
                lt = excl ? 0.f : lt;
                dt = excl ? 0.f : dt;
                if (jj & 1) {
                    l1 += lt;
                    d1 += dt;
                } else {
                    l0 += lt;
                    d0 += dt;
                }
            }
            ff_add(lj, l0 + l1);
            ff_add(dh, d0 + d1);
        }
    }

    // the stream's next call may be scheduled once every CTA is past its pair work: its
    // CTAs then spread over SMs that are mostly idle, and wait for this kernel to end
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // CTA reduction in float-float on the FP32 pipe (the FP64 unit is slow on this part).
    // Each CTA leaves (LJ hi, LJ lo, DH hi, DH lo) in its 16-byte partials slot.
    float4 *part4 = reinterpret_cast<float4 *>(partials);
    lj = ff_warp_sum(lj);
    dh = ff_warp_sum(dh);
    bad = __any_sync(0xffffffffu, bad) ? 1u : 0u;
    if ((t & 31) == 0) {
        s_red[0][t >> 5] = lj;
        s_red[1][t >> 5] = dh;
        if (bad)
            atomicOr(flags, 1u);
    }
    __syncthreads();
    if (t == 0) {
        FF a = s_red[0][0], b = s_red[1][0];
        for (int w = 1; w < kWarps; ++w) {
            ff_add_ff(a, s_red[0][w]);
            ff_add_ff(b, s_red[1][w]);
        }
        part4[blockIdx.x] = make_float4(a.hi, a.lo, b.hi, b.lo);
        __threadfence();
        const int g = blockIdx.x / kGroup, gsize = min(kGroup, (int)gridDim.x - g * kGroup);
        const unsigned done = atomicAdd(&gtickets[g], 1u);
        s_last = (done == (unsigned)gsize - 1u);
    }
    __syncthreads();
    if (!s_last)
        return;

    // Last CTA of its group: the group's partials in a fixed order (float-float, one warp).
    __threadfence();
    const int ngroups = ((int)gridDim.x + kGroup - 1) / kGroup;
    if (t < 32) {
        const int g = blockIdx.x / kGroup, c0 = g * kGroup, gsize = min(kGroup, (int)gridDim.x - c0);
        FF a{0.f, 0.f}, b{0.f, 0.f};
        if (t < gsize) {
            const float4 p = __ldcg(&part4[c0 + t]);
            a = FF{p.x, p.y};
            b = FF{p.z, p.w};
        }
        a = ff_warp_sum(a);
        b = ff_warp_sum(b);
        if (t == 0) {
            gsums[g] = make_float4(a.hi, a.lo, b.hi, b.lo);
            gtickets[g] = 0u;
            __threadfence();
            const unsigned done = atomicAdd(ticket, 1u);
            s_last_group = (done == (unsigned)ngroups - 1u);
        }
    }
    __syncthreads();
    if (!s_last_group)
        return;

    // Last group: every group's sum in a fixed order, float-float, then FP64 once.
    __threadfence();
    if (t < 32) {
        FF a{0.f, 0.f}, b{0.f, 0.f};
        for (int g = t; g < ngroups; g += 32) {
            const float4 p = __ldcg(&gsums[g]);
            ff_add_ff(a, FF{p.x, p.y});
            ff_add_ff(b, FF{p.z, p.w});
        }
        a = ff_warp_sum(a);
        b = ff_warp_sum(b);
        if (t == 0) {
            const double lj_raw_sum = ff_value(a), dh_raw_sum = ff_value(b);
            const double total = lj_raw_sum * (double)kRTtoKcal + dh_raw_sum * (double)kDHFactor;
            result[0] = lj_raw_sum;
            result[1] = dh_raw_sum;
            result[2] = total;
            if (async_out != nullptr && async_count > 0)
                async_out[0] = (float)total;
            *ticket = 0u;
        }
    }
}

int current_device()
{
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

// Scratch for `blocks` CTAs on (current device, stream); g_mu must be held.
Scratch *scratch_for(cudaStream_t stream, size_t blocks)
{
    Scratch &s = g_scratch[std::make_pair(current_device(), stream)];
    if (s.capacity < blocks) {
        if (s.ticket != nullptr)
            cudaFree(s.ticket);
        size_t cap = blocks < 256 ? 256 : blocks;
        unsigned char *base = nullptr;
        if (cgppd_check(cudaMalloc(&base, scratch_bytes(cap)), "scratch allocation") != 0)
            return nullptr;
        cudaMemset(base, 0, scratch_bytes(cap));
        scratch_view(base, cap, s);
    }
    return &s;
}

const float *bound_table()
{
    auto it = g_bound_table.find(current_device());
    return it == g_bound_table.end() ? nullptr : it->second;
}

// Launch the tile kernel on `stream`.  Returns 0 on success.
// Launch the tile kernel on `stream`.  Returns 0 on success.  On a stream of the caller
// (the asynchronous entry point) the launch is a programmatic dependent one: the grid
// may be scheduled once every CTA of the stream's previous kernel has finished its pair
// work (for a previous call of this kernel), and each CTA waits for that kernel's
// completion (griddepcontrol.wait) before it reads or writes global memory, so the
// ordering the caller sees is that of a plain launch.
int launch_energy(bool nc, const float4 *pos, const float4 *meta, int P, const float *table, Scratch *s,
                  float *async_out, int async_count, cudaStream_t stream)
{
    const int nt = (P + kTile - 1) / kTile;
    // crowders take no part in the non-crowder sum, so its form has no crowder variant
    const bool rc = g_repulsive_crowding.load() != 0;
    auto kern = nc ? k_tile_energy<true, false> : rc ? k_tile_energy<false, true> : k_tile_energy<false, false>;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)energy_ctas(nt));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    const bool dependent = stream != cudaStreamLegacy && stream != nullptr;
    cfg.attrs = dependent ? attr : nullptr;
    cfg.numAttrs = dependent ? 1 : 0;
    return cgppd_check(cudaLaunchKernelEx(&cfg, kern, pos, meta, P, nt, table, s->partials, s->ticket, s->flags,
                                          s->result, s->gsums, s->gtickets, async_out, async_count),
                       "energy kernel launch");
}

// Synchronous total on the legacy default stream (the reference's stream 0).
void eon_device_sync(bool nc, float4 *pos, float4 *meta, double *result, int datasetSize)
{
    *result = 0.0;
    if (datasetSize <= 0)
        return;
    std::lock_guard<std::mutex> lock(g_mu);
    const float *table = bound_table();
    if (table == nullptr) {
        cgppd_fail("CUDA_EonDevice: no contact table bound (call bindLJTexture first)");
        return;
    }
    const int nt = (datasetSize + kTile - 1) / kTile;
    Scratch *s = scratch_for(cudaStreamLegacy, (size_t)energy_ctas(nt));
    if (s == nullptr)
        return;
    if (launch_energy(nc, pos, meta, datasetSize, table, s, nullptr, 0, cudaStreamLegacy) != 0)
        return;
    double host[3];
    unsigned flags = 0;
    if (cgppd_check(cudaMemcpy(host, s->result, sizeof(host), cudaMemcpyDeviceToHost), "energy result copy") != 0)
        return;
    cudaMemcpy(&flags, s->flags, sizeof(flags), cudaMemcpyDeviceToHost);
    if (flags != 0u) {
        cudaMemset(s->flags, 0, sizeof(unsigned));
        cgppd_fail("CUDA_EonDevice: residue type index outside the 20x20 table");
    }
    *result = host[2];
}

}  // namespace

extern "C" {

// Reference src/CudaFunctions.cu:20-32: report the last CUDA error and throw.
void __throwLastCudaError(const char *errorMessage, const char *file, const int line)
{
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        std::fprintf(stderr, "%s(%i) : getLastCudaError() CUDA error : %s : (%d) %s.\n", file, line, errorMessage,
                     (int)err, cudaGetErrorString(err));
        throw errorMessage;
    }
}

// Reference src/CudaFunctions.cu:75-104: a device copy of the contact table.
float *LJPotentialDataToDevice(AminoAcids *a)
{
    float *dev = nullptr;
    if (cgppd_check(cudaMalloc(&dev, sizeof(float) * 400), "LJPotentialDataToDevice") != 0)
        return nullptr;
    cgppd_check(cudaMemcpy(dev, &a->LJpotentials[0][0], sizeof(float) * 400, cudaMemcpyHostToDevice),
                "LJPotentialDataToDevice copy");
    return dev;
}

// Reference src/CudaFunctions.cu:106-125: copy the table into a caller-allocated buffer.
void copyLJPotentialDataToDevice(float *dev_LJPotentialData, AminoAcids *a)
{
    cgppd_check(cudaMemcpy(dev_LJPotentialData, &a->LJpotentials[0][0], sizeof(float) * 400, cudaMemcpyHostToDevice),
                "Failed to copy contact potentials");
}

// Reference src/CudaFunctions.cu:36-47: make `ljp` the table the energy kernels read on
// the current device.  The kernels read it through the read-only path after staging it
// in shared memory; there is no texture object to bind.
void bindLJTexture(float *ljp)
{
    std::lock_guard<std::mutex> lock(g_mu);
    g_bound_table[current_device()] = ljp;
}

void unbindLJTexture()
{
    std::lock_guard<std::mutex> lock(g_mu);
    g_bound_table.erase(current_device());
}

// Reference src/CudaFunctions.cu:157-167: periodic box edge, module state per device.
void CUDA_setBoxDimension(float value)
{
    cgppd_check(cudaMemcpyToSymbol(c_boxdim, &value, sizeof(value)), "Set boxdim");
}

void CUDA_freeBoxDimension()
{
    float zero = 0.0f;
    cudaMemcpyToSymbol(c_boxdim, &zero, sizeof(zero));
}

// Reference src/CudaFunctions.cu:198-277.  `LJPotentials` is never dereferenced (the
// reference callers pass an uninitialised pointer); the bound table is used.  The
// residue/molecule count arguments are accepted and unused, as in the reference.
void CUDA_EonDevice(float4 *residuePositions, float4 *residueMeta, int *residueCount, int *moleculePositions,
                    int *moleculeCount, float *LJPotentials, double *result, int blockSize, int datasetSize,
                    int sharedMemSize)
{
    (void)residueCount, (void)moleculePositions, (void)moleculeCount, (void)LJPotentials, (void)blockSize,
        (void)sharedMemSize;
    eon_device_sync(false, residuePositions, residueMeta, result, datasetSize);
}

// Reference src/CudaFunctions.cu:724-754: non-crowder, different-molecule pairs only.
void CUDA_EonDeviceNC(float4 *residuePositions, float4 *residueMeta, int *residueCount, int *moleculePositions,
                      int *moleculeCount, float *LJPotentials, double *result, int blockSize, int datasetSize,
                      int sharedMemSize)
{
    (void)residueCount, (void)moleculePositions, (void)moleculeCount, (void)LJPotentials, (void)blockSize,
        (void)sharedMemSize;
    eon_device_sync(true, residuePositions, residueMeta, result, datasetSize);
}

// Reference src/CudaFunctions.cu:176-190.  The caller owns `device_result`
// (resultSize*resultSize floats) and sums it after syncing `stream`; this writes the
// total to element 0 and zero everywhere else, which sums to the same value.
void CUDA_EonDevice_async(float4 *residuePositions, float4 *residueMeta, int *residueCount, int *moleculePositions,
                          int *moleculeCount, float *LJPotentials, float *device_result, int resultSize,
                          int blockSize, int datasetSize, int sharedMemSize, cudaStream_t stream)
{
    (void)residueCount, (void)moleculePositions, (void)moleculeCount, (void)LJPotentials, (void)blockSize,
        (void)sharedMemSize;
    if (datasetSize <= 0 || resultSize <= 0)
        return;
    std::lock_guard<std::mutex> lock(g_mu);
    const float *table = bound_table();
    if (table == nullptr) {
        cgppd_fail("CUDA_EonDevice_async: no contact table bound (call bindLJTexture first)");
        return;
    }
    const int nt = (datasetSize + kTile - 1) / kTile;
    Scratch *s = scratch_for(stream, (size_t)energy_ctas(nt));
    if (s == nullptr)
        return;
    launch_energy(false, residuePositions, residueMeta, datasetSize, table, s, device_result,
                  resultSize * resultSize, stream);
}

// The reference selects the crowder potential at compile time (REPULSIVE_CROWDING,
// src/definitions.h:18; off in its default build); this library selects it at run
// time for every later energy call of the process: 0 (default) the full potential for
// crowder pairs, 1 the repulsive (6/r)^12 term below 15 A without Debye-Hueckel.
// Returns the previous setting.
int cgppd_set_repulsive_crowding(int on)
{
    return g_repulsive_crowding.exchange(on ? 1 : 0);
}

// Components of the last synchronous call on the current device (LJ raw, DH raw,
// total): a library extension used by the tests.
int cgppd_last_energy_components(double *out3)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_scratch.find(std::make_pair(current_device(), cudaStreamLegacy));
    if (it == g_scratch.end())
        return -1;
    return cgppd_check(cudaMemcpy(out3, it->second.result, 3 * sizeof(double), cudaMemcpyDeviceToHost),
                       "component copy");
}

}  // extern "C"

// ------------------------------------------------------------------ allocation-free variant
//
// Some hosts of this library cannot allocate device memory while they evaluate
// energies: code that runs inside another framework's memory pool or under a fixed
// device-memory budget, and callers that must not introduce allocation calls into a
// timed or real-time loop.  CUDA_EonDevice_noalloc gives them the CUDA_EonDevice
// result without any allocation: its scratch (CTA partials, completion ticket, error
// flags, result slot) is a file-scope __device__ array, which every GPU that loads the
// library holds until the process exits.
namespace {

constexpr int kNoAllocMaxResidues = 16384;                       // datasetSize limit
constexpr int kNoAllocMaxTiles = kNoAllocMaxResidues / kTile;    // 128-residue tiles
constexpr int kNoAllocMaxCtas = energy_ctas(kNoAllocMaxTiles);
constexpr size_t kNoAllocBytes = scratch_bytes(kNoAllocMaxCtas);  // 139,896 bytes (layout: scratch_view)
static_assert(kNoAllocBytes == 139896, "the documented size of the static scratch");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
// Calls on one device share that device's array and are serialised; each device has
// its own copy of the array, so calls on different devices do not wait for each other.
std::mutex g_noalloc_mu[kMaxDevices];

// In host code g_noalloc_scratch names a host-side stand-in, not device memory; the
// kernel needs the device address, looked up with the device current.  The lookup
// allocates nothing and is repeated on every call, so the address stays valid after a
// cudaDeviceReset (which reloads the module, possibly elsewhere); the first lookup on a
// device also loads the library's device code there.
unsigned char *noalloc_scratch()
{
    void *p = nullptr;
    if (cgppd_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "CUDA_EonDevice_noalloc set-up") != 0)
        return nullptr;
    return static_cast<unsigned char *>(p);
}

}  // namespace

extern "C" {

// Same arguments and result as CUDA_EonDevice.  The first call on a device loads the
// library's device code there if nothing else has, and should come before any stream
// capture.  datasetSize above 16384 residues is rejected with an error (result 0).
// Every call on a device shares that device's array and leaves the last call's data in
// it; the ticket and error flags are cleared before each launch.  Two calls whose
// kernels overlap on the GPU would race on the array: this function holds a per-device
// lock and returns only after its kernel and result copy have finished, so calls made
// through it on one device do not overlap.
void CUDA_EonDevice_noalloc(float4 *residuePositions, float4 *residueMeta, int *residueCount,
                            int *moleculePositions, int *moleculeCount, float *LJPotentials, double *result,
                            int blockSize, int datasetSize, int sharedMemSize)
{
    (void)residueCount, (void)moleculePositions, (void)moleculeCount, (void)LJPotentials, (void)blockSize,
        (void)sharedMemSize;
    *result = 0.0;
    if (datasetSize <= 0)
        return;
    if (datasetSize > kNoAllocMaxResidues) {
        cgppd_fail("CUDA_EonDevice_noalloc: datasetSize exceeds the 16384-residue limit of its static scratch");
        return;
    }
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) {
        cgppd_fail("CUDA_EonDevice_noalloc: device ordinal above 63");
        return;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu[dev]);
    const float *table = nullptr;
    {
        std::lock_guard<std::mutex> tlock(g_mu);
        table = bound_table();
    }
    if (table == nullptr) {
        cgppd_fail("CUDA_EonDevice_noalloc: no contact table bound (call bindLJTexture first)");
        return;
    }
    unsigned char *base = noalloc_scratch();
    if (base == nullptr)
        return;
    Scratch s;
    scratch_view(base, kNoAllocMaxCtas, s);
    if (cgppd_check(cudaMemsetAsync(base, 0, 8, cudaStreamLegacy), "CUDA_EonDevice_noalloc clear") != 0 ||
        cgppd_check(cudaMemsetAsync(s.gtickets, 0, 4 * scratch_groups(kNoAllocMaxCtas), cudaStreamLegacy),
                    "CUDA_EonDevice_noalloc clear") != 0)
        return;
    if (launch_energy(false, residuePositions, residueMeta, datasetSize, table, &s, nullptr, 0, cudaStreamLegacy) != 0)
        return;
    double host[3];
    unsigned flags = 0;
    if (cgppd_check(cudaMemcpy(host, s.result, sizeof(host), cudaMemcpyDeviceToHost), "CUDA_EonDevice_noalloc copy") != 0)
        return;
    if (cgppd_check(cudaMemcpy(&flags, s.flags, sizeof(flags), cudaMemcpyDeviceToHost), "CUDA_EonDevice_noalloc copy") != 0)
        return;
    if (flags != 0u) {
        cgppd_fail("CUDA_EonDevice_noalloc: residue type index outside the 20x20 table");
        return;
    }
    *result = host[2];
}

}  // extern "C"
