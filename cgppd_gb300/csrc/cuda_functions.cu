// cuda_functions.cu -- the drop-in C ABI of the reference's CUDA energy module
// (src/cudaExterns.h:14-90, src/CudaFunctions.cu:20-277, :724-961), rebuilt for sm_103a.
//
// Callers keep the reference's packed layout: float4 pos[P] = (x, y, z, w) with
// w = rigid_domain_uid + bond_fraction (-2 for padding), float4 meta[P] =
// (type, charge, vdW radius, w) with w = molecule_id + chain_fraction (-1 for a
// crowder).  The pair rules are those of the reference's flexible-linker build.
//
// Kernel: one CTA per (y-tile, x-tile) pair of 128-residue tiles on or above the
// diagonal.  The x tile is decoded once into shared memory (position and radius; the
// exclusion keys of its w fields; charge, type and flags) next to the 20x20 table; two
// threads own each y residue and sweep one half of the x tile each.  Pair terms are
// FP32, summed per 32 pairs in two alternating partial sums and folded into
// float-float accumulators, reduced per CTA in FP64.  The last CTA
// to finish (ticket counter) reduces all CTA partials in a fixed order, so the total
// is deterministic.  Scratch (partials + ticket + result) is per (device, stream),
// allocated on first use and reused.
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

constexpr int kTile = 128;                 // residues per tile side
constexpr int kThreads = 2 * kTile;        // two threads per y residue (x-tile halves)
constexpr int kWarps = kThreads / 32;

__constant__ float c_boxdim;  // CUDA_setBoxDimension, module state per device
// cgppd_set_repulsive_crowding: the reference's compile-time REPULSIVE_CROWDING
// (src/definitions.h:18) as process-wide module state, read at each launch
std::atomic<int> g_repulsive_crowding{0};

struct Scratch {
    unsigned *ticket = nullptr;   // CTA completion counter, self-resetting
    unsigned *flags = nullptr;    // bit 0: residue type index out of range
    double *result = nullptr;     // {LJ raw, DH raw, total kcal/mol}
    double *partials = nullptr;   // 2 doubles per CTA
    size_t capacity = 0;          // CTAs the partials can hold
};

std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, Scratch> g_scratch;
std::map<int, const float *> g_bound_table;  // bindLJTexture, per device

__device__ __forceinline__ float frac_int(float w, float &ip)
{
    ip = truncf(w);
    return w - ip;
}

// kNC: non-crowder pairs of different molecules only (E_TiledKernelNC).  kRC: the
// REPULSIVE_CROWDING form of the crowder pairs.
template <bool kNC, bool kRC>
__global__ void __launch_bounds__(kThreads) k_tile_energy(const float4 *__restrict__ pos, const float4 *__restrict__ meta,
                                                          int P, int nt, const float *__restrict__ lj_raw,
                                                          double *__restrict__ partials, unsigned *__restrict__ ticket,
                                                          unsigned *__restrict__ flags, double *__restrict__ result,
                                                          float *__restrict__ async_out, int async_count)
{
    // x tile, decoded once per CTA: position and vdW radius; exclusion keys (rigid
    // domain, bond fraction, chain fraction, molecule id); charge, type, flags
    __shared__ float4 s_px[kTile];
    __shared__ float4 s_xk[kTile];
    __shared__ float4 s_xm[kTile];
    __shared__ float s_eij[400];
    __shared__ double s_red[2][kWarps];
    __shared__ bool s_last;

    // Tile pair (ty <= tx) of this CTA, row-major over the upper triangle.
    int rem = blockIdx.x, ty = 0;
    while (rem >= nt - ty) {
        rem -= nt - ty;
        ++ty;
    }
    const int tx = ty + rem;
    const int t = threadIdx.x;
    const int yl = t & (kTile - 1), half = t / kTile;  // y residue, half of the x tile

    for (int k = t; k < 400; k += kThreads)
        s_eij[k] = kLambda * (lj_raw[k] - kE0);  // Eij in RT units, as the kernel forms it
    // residue types are checked once per residue (0..19; padding is excluded anyway):
    // the pair loop then indexes the table without a bounds test
    unsigned bad = 0;
    const int x0 = tx * kTile;
    if (t < kTile) {
        const float4 px = (x0 + t < P) ? pos[x0 + t] : make_float4(0.f, 0.f, 0.f, kPadder);
        const float4 mx = (x0 + t < P) ? meta[x0 + t] : make_float4(0.f, 0.f, 0.f, 0.f);
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
    }
    const int y = ty * kTile + yl;
    const float4 py = (y < P) ? pos[y] : make_float4(0.f, 0.f, 0.f, kPadder);
    const float4 my = (y < P) ? meta[y] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();

    FF lj{0.f, 0.f}, dh{0.f, 0.f};
    const bool ycrowd = my.w == kCrowder;
    const bool active = (py.w > kPadder) && (!kNC || !ycrowd);
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
        const int jb0 = half * (kTile / 2);
        for (int jb = jb0; jb < jb0 + kTile / 2; jb += 32) {
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

    // CTA reduction in FP64.
    double v0 = ff_value(lj), v1 = ff_value(dh);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, o);
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
    }
    bad = __any_sync(0xffffffffu, bad) ? 1u : 0u;
    if ((t & 31) == 0) {
        s_red[0][t >> 5] = v0;
        s_red[1][t >> 5] = v1;
        if (bad)
            atomicOr(flags, 1u);
    }
    __syncthreads();
    if (t == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kWarps; ++w) {
            a += s_red[0][w];
            b += s_red[1][w];
        }
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
        __threadfence();
        const unsigned done = atomicAdd(ticket, 1u);
        s_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last)
        return;

    // Last CTA: ordered reduction of every CTA's partials.
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int k = t; k < (int)gridDim.x; k += kThreads) {
        a += __ldcg(&partials[2 * k]);
        b += __ldcg(&partials[2 * k + 1]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    __syncthreads();
    if ((t & 31) == 0) {
        s_red[0][t >> 5] = a;
        s_red[1][t >> 5] = b;
    }
    __syncthreads();
    if (t == 0) {
        double A = 0.0, B = 0.0;
        for (int w = 0; w < kWarps; ++w) {
            A += s_red[0][w];
            B += s_red[1][w];
        }
        const double total = A * (double)kRTtoKcal + B * (double)kDHFactor;
        result[0] = A;
        result[1] = B;
        result[2] = total;
        if (async_out != nullptr && async_count > 0)
            async_out[0] = (float)total;
        *ticket = 0u;
    }
    if (async_out != nullptr)
        for (int k = 1 + t; k < async_count; k += kThreads)
            async_out[k] = 0.0f;
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
        char *base = nullptr;
        // [ticket, flags | pad to 256] [result: 4 doubles | pad] [partials]
        size_t bytes = 256 + 256 + 2 * sizeof(double) * cap;
        if (cgppd_check(cudaMalloc(&base, bytes), "scratch allocation") != 0)
            return nullptr;
        cudaMemset(base, 0, 512);
        s.ticket = reinterpret_cast<unsigned *>(base);
        s.flags = reinterpret_cast<unsigned *>(base + 4);
        s.result = reinterpret_cast<double *>(base + 256);
        s.partials = reinterpret_cast<double *>(base + 512);
        s.capacity = cap;
    }
    return &s;
}

const float *bound_table()
{
    auto it = g_bound_table.find(current_device());
    return it == g_bound_table.end() ? nullptr : it->second;
}

// Launch the tile kernel on `stream`.  Returns 0 on success.
int launch_energy(bool nc, const float4 *pos, const float4 *meta, int P, const float *table, Scratch *s,
                  float *async_out, int async_count, cudaStream_t stream)
{
    const int nt = (P + kTile - 1) / kTile;
    const int blocks = nt * (nt + 1) / 2;
    // crowders take no part in the non-crowder sum, so its form has no crowder variant
    const bool rc = g_repulsive_crowding.load() != 0;
    if (nc)
        k_tile_energy<true, false><<<blocks, kThreads, 0, stream>>>(pos, meta, P, nt, table, s->partials, s->ticket,
                                                                    s->flags, s->result, async_out, async_count);
    else if (rc)
        k_tile_energy<false, true><<<blocks, kThreads, 0, stream>>>(pos, meta, P, nt, table, s->partials, s->ticket,
                                                                    s->flags, s->result, async_out, async_count);
    else
        k_tile_energy<false, false><<<blocks, kThreads, 0, stream>>>(pos, meta, P, nt, table, s->partials, s->ticket,
                                                                     s->flags, s->result, async_out, async_count);
    return cgppd_check(cudaGetLastError(), "energy kernel launch");
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
    Scratch *s = scratch_for(cudaStreamLegacy, (size_t)nt * (nt + 1) / 2);
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
    Scratch *s = scratch_for(stream, (size_t)nt * (nt + 1) / 2);
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
constexpr int kNoAllocMaxCtas = kNoAllocMaxTiles * (kNoAllocMaxTiles + 1) / 2;
// layout: [0] ticket, [4] flags, [256] result (3 doubles), [512] 2 doubles per CTA
constexpr size_t kNoAllocBytes = 512 + 2 * sizeof(double) * kNoAllocMaxCtas;  // 132,608 bytes

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
    s.ticket = reinterpret_cast<unsigned *>(base);
    s.flags = reinterpret_cast<unsigned *>(base + 4);
    s.result = reinterpret_cast<double *>(base + 256);
    s.partials = reinterpret_cast<double *>(base + 512);
    s.capacity = kNoAllocMaxCtas;
    if (cgppd_check(cudaMemsetAsync(base, 0, 8, cudaStreamLegacy), "CUDA_EonDevice_noalloc clear") != 0)
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
