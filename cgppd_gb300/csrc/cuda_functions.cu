// cuda_functions.cu -- the drop-in C ABI of the reference's CUDA energy module
// (src/cudaExterns.h:14-90, src/CudaFunctions.cu:20-277, :724-961), rebuilt for sm_103a.
//
// Callers keep the reference's packed layout: float4 pos[P] = (x, y, z, w) with
// w = rigid_domain_uid + bond_fraction (-2 for padding), float4 meta[P] =
// (type, charge, vdW radius, w) with w = molecule_id + chain_fraction (-1 for a
// crowder).  The pair rules are those of the reference's flexible-linker build.
//
// Kernel: one CTA per (y-tile, x-tile) pair of 128-residue tiles on or above the
// diagonal.  The x tile and the 20x20 table are staged in shared memory, each thread
// owns one y residue and sweeps the x tile; pair terms are FP32, summed per 32 pairs
// and folded into float-float accumulators, reduced per CTA in FP64.  The last CTA
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

constexpr int kTile = 128;
constexpr int kWarps = kTile / 32;

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

template <bool kNC>
__global__ void __launch_bounds__(kTile) k_tile_energy(const float4 *__restrict__ pos, const float4 *__restrict__ meta,
                                                       int P, int nt, const float *__restrict__ lj_raw,
                                                       double *__restrict__ partials, unsigned *__restrict__ ticket,
                                                       unsigned *__restrict__ flags, double *__restrict__ result,
                                                       float *__restrict__ async_out, int async_count, int rc)
{
    __shared__ float4 s_pos[kTile];
    __shared__ float4 s_meta[kTile];
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

    for (int k = t; k < 400; k += kTile)
        s_eij[k] = kLambda * (lj_raw[k] - kE0);  // Eij in RT units, as the kernel forms it
    const float4 pad = make_float4(0.f, 0.f, 0.f, kPadder);
    const float4 padm = make_float4(20.f, 0.f, 0.f, 0.f);
    const int x0 = tx * kTile;
    s_pos[t] = (x0 + t < P) ? pos[x0 + t] : pad;
    s_meta[t] = (x0 + t < P) ? meta[x0 + t] : padm;
    const int y = ty * kTile + t;
    const float4 py = (y < P) ? pos[y] : pad;
    const float4 my = (y < P) ? meta[y] : padm;
    __syncthreads();

    FF lj{0.f, 0.f}, dh{0.f, 0.f};
    unsigned bad = 0;
    const bool active = (py.w > kPadder) && (!kNC || my.w != kCrowder);
    if (active) {
        const float L = c_boxdim;
        const float invL = (L != 0.0f) ? 1.0f / L : 0.0f;
        float ydom, ymol;
        const float ybond = frac_int(py.w, ydom);
        const float ychain = frac_int(my.w, ymol);
        const bool diag = (tx == ty);
        const bool ycrowd = rc && (my.w == kCrowder);
        for (int jb = 0; jb < kTile; jb += 32) {
            float lj_t = 0.f, dh_t = 0.f;
#pragma unroll 4
            for (int jj = 0; jj < 32; ++jj) {
                const int j = jb + jj;
                const float4 px = s_pos[j];
                const float4 mx = s_meta[j];
                bool excl = (px.w == kPadder) || (diag && j <= t);
                if (kNC) {
                    excl = excl || (mx.w == kCrowder) || (truncf(mx.w) == ymol);
                } else {
                    float xdom, xmol;
                    const float xbond = frac_int(px.w, xdom);
                    const float xchain = frac_int(mx.w, xmol);
                    excl = excl || (xdom != 0.f && xdom == ydom) || (xbond != 0.f && xbond == ybond) ||
                           (xchain == ychain && fabsf((float)(x0 + j) - (float)y) < 4.0f);
                }
                if (!excl) {
                    const float dx = min_image(py.x - px.x, L, invL);
                    const float dy = min_image(py.y - px.y, L, invL);
                    const float dz = min_image(py.z - px.z, L, invL);
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float inv_r = rsqrt_refined(r2);
                    const float r = r2 * inv_r;
                    if (ycrowd || (rc && mx.w == kCrowder)) {
                        // REPULSIVE_CROWDING (src/CudaFunctions.cu:335-338, :492-498):
                        // (6/r)^12 in RT units below 15 A, no Debye-Hueckel term
                        if (r < kRepulsiveCutoff) {
                            const float sc = 6.0f * inv_r, s2 = sc * sc, s6 = s2 * s2 * s2;
                            lj_t += s6 * s6;
                        }
                    } else {
                        int idx = __float2int_rn(20.0f * my.x + mx.x);
                        if ((unsigned)idx >= 400u) {
                            bad = 1u;
                            idx = 0;
                        }
                        const float eij = s_eij[idx];
                        const float sig = (my.z + mx.z) * 0.5f;
                        lj_t += lj_term(eij, sig, inv_r * inv_r);
                        dh_t += dh_term(my.y * mx.y, r, inv_r);
                    }
                }
            }
            ff_add(lj, lj_t);
            ff_add(dh, dh_t);
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
    for (int k = t; k < (int)gridDim.x; k += kTile) {
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
        for (int k = 1 + t; k < async_count; k += kTile)
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
    const int rc = g_repulsive_crowding.load();
    if (nc)
        k_tile_energy<true><<<blocks, kTile, 0, stream>>>(pos, meta, P, nt, table, s->partials, s->ticket, s->flags,
                                                           s->result, async_out, async_count, rc);
    else
        k_tile_energy<false><<<blocks, kTile, 0, stream>>>(pos, meta, P, nt, table, s->partials, s->ticket, s->flags,
                                                            s->result, async_out, async_count, rc);
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
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[kMaxDevices] = {nullptr};  // device address of the array, per device

// In host code g_noalloc_scratch names a host-side stand-in, not device memory; the
// kernel needs the device address, looked up once per device with that device current.
unsigned char *noalloc_scratch(int dev)
{
    if (dev < 0 || dev >= kMaxDevices) {
        cgppd_fail("CUDA_EonDevice_noalloc: device ordinal above 63");
        return nullptr;
    }
    if (g_noalloc_addr[dev] == nullptr) {
        void *p = nullptr;
        if (cgppd_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "CUDA_EonDevice_noalloc set-up") != 0)
            return nullptr;
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    return g_noalloc_addr[dev];
}

}  // namespace

extern "C" {

// Same arguments and result as CUDA_EonDevice.  The first call on a device performs
// the one-time set-up (the device address of the static scratch) and should come
// before any stream capture.  datasetSize above 16384 residues is rejected with an
// error (result 0).  Every call shares the one array and leaves the last call's data
// in it; the ticket and error flags are cleared before each launch.  Two calls whose
// kernels overlap on the GPU would race on the array: this function holds a
// process-wide lock and returns only after its kernel and result copy have finished,
// so calls made through it do not overlap.
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
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    const int dev = current_device();
    const float *table = nullptr;
    {
        std::lock_guard<std::mutex> tlock(g_mu);
        table = bound_table();
    }
    if (table == nullptr) {
        cgppd_fail("CUDA_EonDevice_noalloc: no contact table bound (call bindLJTexture first)");
        return;
    }
    unsigned char *base = noalloc_scratch(dev);
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
