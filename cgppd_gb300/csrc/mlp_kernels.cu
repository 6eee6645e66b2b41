// mlp_kernels.cu -- training and batched inference of the pair-energy surrogate.
//
// The three 256x256 layers run as BF16 GEMMs on the tcgen05 tensor cores with FP32
// accumulation in tensor memory: C[M x 256] = A[M x K] * B[256 x K]^T, both operands
// K-major, one 128 x 256 tile per CTA (accumulator = 256 TMEM columns x 128 lanes).
// 64-wide K chunks are staged into shared memory by the CTA's 256 threads in the
// no-swizzle core-matrix layout (tc05.cuh), then one thread issues four K = 16 MMAs and
// commits them to an mbarrier; the next chunk's global loads are issued into registers
// while those MMAs run.  Epilogues read the accumulator back with tcgen05.ld
// (warp w owns lanes 32(w % 4)..+31 = rows of the tile, columns of half w / 4) and
// fuse what the layer needs:
//   kGemmFwd   z = acc + bias -> Z (f32), h = silu(z) -> H (bf16) and H^T (bf16)
//   kGemmBwd   d = acc * silu'(Zprev) -> dZ (bf16) and dZ^T (bf16)
//   kGemmStore acc -> C[z] (f32 split-K partial, reduced in a fixed order afterwards)
// Every orientation a GEMM needs is produced by an epilogue, so no GEMM reads a
// transposed operand.  Layer 1 (K = 8) and the output dot product stay in FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "surrogate.cuh"
#include "surrogate_internal.h"
#include "tc05.cuh"

namespace cgppd {

constexpr int kGemmN = 256;
constexpr int kGemmThreads = 256;   // 8 warps: two per TMEM lane quadrant, one per column half
constexpr int kGemmLoadsA = 128 * 8 / kGemmThreads;     // 16-byte pieces of A per thread and chunk
constexpr int kGemmLoadsB = kGemmN * 8 / kGemmThreads;  // and of B
constexpr int kGemmTileA = 128 * tc05::kChunkK * 2;       // 16 KB
constexpr int kGemmTileB = kGemmN * tc05::kChunkK * 2;    // 32 KB
// Requested dynamic shared memory: the tiles plus slack so that at most two CTAs share
// an SM (2 x 256 TMEM columns = the SM's 512).
constexpr int kGemmSmem = 100 * 1024;

template <int MODE>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_tc(GemmArgs g)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int m0 = blockIdx.x * 128;
    const int kb = blockIdx.z * g.k_split, ke = kb + g.k_split;
    unsigned char *sA = smem, *sB = smem + kGemmTileA;

    if (warp == 0)
        tc05::tmem_alloc(&tmem_base, kGemmN);
    if (t == 0)
        tc05::mbar_init(&mbar, 1);
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t aaddr = tc05::smem_u32(sA), baddr = tc05::smem_u32(sB);
    constexpr uint32_t idesc = tc05::idesc_bf16_f32(128, kGemmN);

    // software pipeline: the next chunk's global loads are in flight (in registers) while
    // the tensor cores work on this one; the shared tiles are rewritten only after the
    // MMAs that read them have completed
    uint4 ra[kGemmLoadsA], rb[kGemmLoadsB];
    auto load_chunk = [&](int k0) {
#pragma unroll
        for (int i = 0; i < kGemmLoadsA; ++i) {
            const int idx = t + kGemmThreads * i, r = idx >> 3, c = idx & 7;
            ra[i] = *reinterpret_cast<const uint4 *>(g.A + (size_t)(m0 + r) * g.K + k0 + c * 8);
        }
#pragma unroll
        for (int i = 0; i < kGemmLoadsB; ++i) {
            const int idx = t + kGemmThreads * i, r = idx >> 3, c = idx & 7;
            rb[i] = *reinterpret_cast<const uint4 *>(g.B + (size_t)r * g.K + k0 + c * 8);
        }
    };
    uint32_t phase = 0;
    int ok = 1;
    bool pending = false;
    load_chunk(kb);
    for (int k0 = kb; k0 < ke; k0 += tc05::kChunkK) {
        if (pending) {
            const int done = tc05::mbar_wait(&mbar, phase) ? 1 : 0;
            phase ^= 1u;
            tc05::fence_after_sync();
            ok = __syncthreads_and(done);
            if (!ok)
                break;
        }
        // stage the A (128 rows) and B (256 rows) chunks: 16-byte pieces, 8 per row
#pragma unroll
        for (int i = 0; i < kGemmLoadsA; ++i) {
            const int idx = t + kGemmThreads * i, r = idx >> 3, c = idx & 7;
            *reinterpret_cast<uint4 *>(sA + tc05::tile_offset(r, c)) = ra[i];
        }
#pragma unroll
        for (int i = 0; i < kGemmLoadsB; ++i) {
            const int idx = t + kGemmThreads * i, r = idx >> 3, c = idx & 7;
            *reinterpret_cast<uint4 *>(sB + tc05::tile_offset(r, c)) = rb[i];
        }
        tc05::fence_proxy_async();
        __syncthreads();
        if (t == 0) {
            tc05::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < tc05::kChunkK / 16; ++kk)
                tc05::mma_f16(tmem, tc05::smem_desc(aaddr + 256u * kk), tc05::smem_desc(baddr + 256u * kk), idesc,
                              (k0 > kb) || (kk > 0));
            tc05::mma_commit(&mbar);
        }
        pending = true;
        if (k0 + tc05::kChunkK < ke)
            load_chunk(k0 + tc05::kChunkK);
    }
    if (ok && pending) {  // the accumulator is read only after the last MMAs completed
        const int done = tc05::mbar_wait(&mbar, phase) ? 1 : 0;
        phase ^= 1u;
        tc05::fence_after_sync();
        ok = __syncthreads_and(done);
    }

    if (ok) {
        // warp w reads TMEM lane quadrant w % 4 (rows 32(w % 4) .. +31 of the tile) and
        // column half w / 4
        const int quad = warp & 3, chalf = warp >> 2;
        const int row = m0 + quad * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16);
        for (int n0 = chalf * (kGemmN / 2); n0 < (chalf + 1) * (kGemmN / 2); n0 += 16) {
            float v[16];
            tc05::tmem_ld16(lane_base + (uint32_t)n0, v);
            if (MODE == kGemmStore) {
                float *c = g.C + ((size_t)blockIdx.z * g.M + row) * kGemmN + n0;
#pragma unroll
                for (int i = 0; i < 16; i += 4)
                    *reinterpret_cast<float4 *>(c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            } else if (MODE == kGemmFwd) {
                float *z = g.Z + (size_t)row * kGemmN + n0;
                uint32_t hp[8];
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const float z0 = v[i] + g.bias[n0 + i], z1 = v[i + 1] + g.bias[n0 + i + 1];
                    z[i] = z0;
                    z[i + 1] = z1;
                    const __nv_bfloat16 h0 = __float2bfloat16_rn(silu(z0)), h1 = __float2bfloat16_rn(silu(z1));
                    g.HT[(size_t)(n0 + i) * g.M + row] = h0;
                    g.HT[(size_t)(n0 + i + 1) * g.M + row] = h1;
                    hp[i >> 1] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
                }
                uint4 *h = reinterpret_cast<uint4 *>(g.H + (size_t)row * kGemmN + n0);
                h[0] = make_uint4(hp[0], hp[1], hp[2], hp[3]);
                h[1] = make_uint4(hp[4], hp[5], hp[6], hp[7]);
            } else {
                const float *zp = g.Zp + (size_t)row * kGemmN + n0;
                uint32_t hp[8];
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const __nv_bfloat16 d0 = __float2bfloat16_rn(v[i] * silu_grad(zp[i]));
                    const __nv_bfloat16 d1 = __float2bfloat16_rn(v[i + 1] * silu_grad(zp[i + 1]));
                    g.HT[(size_t)(n0 + i) * g.M + row] = d0;
                    g.HT[(size_t)(n0 + i + 1) * g.M + row] = d1;
                    hp[i >> 1] = (uint32_t)__bfloat16_as_ushort(d0) | ((uint32_t)__bfloat16_as_ushort(d1) << 16);
                }
                uint4 *h = reinterpret_cast<uint4 *>(g.H + (size_t)row * kGemmN + n0);
                h[0] = make_uint4(hp[0], hp[1], hp[2], hp[3]);
                h[1] = make_uint4(hp[4], hp[5], hp[6], hp[7]);
            }
        }
    } else {
        if (t == 0)
            atomicOr(g.err, 1u);
        // give MMAs still in flight a second bounded wait before the columns are freed
        if (t == 0)
            tc05::mbar_wait(&mbar, phase ^ 1u);
    }
    tc05::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc05::fence_after_sync();
        tc05::tmem_dealloc(tmem, kGemmN);
    }
}

// ------------------------------------------------------------------ FP32 parts

// Z1 = X W1^T + b1, H1 = silu(Z1) (bf16, both orientations); one thread per (row, unit).
__global__ void k_layer1_fwd(const float *X, const float *P, float *Z, __nv_bfloat16 *H, __nv_bfloat16 *HT, int B)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * kSurH)
        return;
    const int b = idx / kSurH, o = idx % kSurH;
    float z = P[kOffB1 + o];
#pragma unroll
    for (int i = 0; i < kSurIn; ++i)
        z = fmaf(P[kOffW1 + o * kSurIn + i], X[b * kSurIn + i], z);
    Z[idx] = z;
    const __nv_bfloat16 h = __float2bfloat16_rn(silu(z));
    H[idx] = h;
    HT[(size_t)o * B + b] = h;
}

// o = H4 . w5 + b5 (one warp per row); with targets: r = o - y, dO = 2 r / B, r2 = r^2.
__global__ void k_out_fwd(const __nv_bfloat16 *H4, const float *P, const float *y, float *o, float *dO, float *r2,
                          int B)
{
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (row >= B)
        return;
    float s = 0.f;
    for (int k = lane; k < kSurH; k += 32)
        s = fmaf(__bfloat162float(H4[(size_t)row * kSurH + k]), P[kOffW5 + k], s);
#pragma unroll
    for (int w = 16; w > 0; w >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, w);
    if (lane == 0) {
        const float out = s + P[kOffB5];
        o[row] = out;
        if (y) {
            const float r = out - y[row];
            dO[row] = 2.0f * r / (float)B;
            r2[row] = r * r;
        }
    }
}

// dZ4 = (dO w5^T) * silu'(Z4), both orientations.
__global__ void k_out_bwd(const float *dO, const float *P, const float *Z4, __nv_bfloat16 *dZ, __nv_bfloat16 *dZT,
                          int B)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * kSurH)
        return;
    const int b = idx / kSurH, k = idx % kSurH;
    const __nv_bfloat16 d = __float2bfloat16_rn(dO[b] * P[kOffW5 + k] * silu_grad(Z4[idx]));
    dZ[idx] = d;
    dZT[(size_t)k * B + b] = d;
}

// Fixed-order block reduction (256 threads).
__device__ float block_sum256(float v, float *red)
{
#pragma unroll
    for (int w = 16; w > 0; w >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, w);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.f;
    if (threadIdx.x == 0)
        for (int w = 0; w < 8; ++w)
            s += red[w];
    __syncthreads();
    return s;
}

// Row k of a [rows][B] bf16 matrix: sum (bias gradient) and, optionally, dot products
// with up to 8 f32 columns X[b][i] (layer-1 weight gradient) or with one vector u.
__global__ void __launch_bounds__(256) k_row_reduce(const __nv_bfloat16 *MT, int B, const float *X, int nx,
                                                    const float *u, float *sum_out, float *dot_out)
{
    __shared__ float red[8];
    const int k = blockIdx.x;
    float s = 0.f, d[kSurIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, du = 0.f;
    for (int b = threadIdx.x; b < B; b += 256) {
        const float v = __bfloat162float(MT[(size_t)k * B + b]);
        s += v;
        if (X)
            for (int i = 0; i < nx; ++i)
                d[i] = fmaf(v, X[b * kSurIn + i], d[i]);
        if (u)
            du = fmaf(v, u[b], du);
    }
    const float ts = block_sum256(s, red);
    if (sum_out && threadIdx.x == 0)
        sum_out[k] = ts;
    if (X)
        for (int i = 0; i < nx; ++i) {
            const float ti = block_sum256(d[i], red);
            if (threadIdx.x == 0)
                dot_out[k * kSurIn + i] = ti;
        }
    if (u) {
        const float tu = block_sum256(du, red);
        if (threadIdx.x == 0)
            dot_out[k] = tu;
    }
}

// sum over rows of a f32 vector (one block): the output-bias gradient and the loss.
__global__ void __launch_bounds__(256) k_vec_sum(const float *v, int n, float *out)
{
    __shared__ float red[8];
    float s = 0.f;
    for (int i = threadIdx.x; i < n; i += 256)
        s += v[i];
    const float t = block_sum256(s, red);
    if (threadIdx.x == 0)
        *out = t;
}

__global__ void k_splitk_reduce(const float *part, int splits, int n, float *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z)
        s += part[(size_t)z * n + i];
    out[i] = s;
}

// Adam on the FP32 master parameters (bias-corrected), then the BF16 GEMM copies.
__global__ void k_adam(float *P, const float *G, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float gi = G[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Wf[l][out][in] and Wt[l][in][out] (bf16) of layers 2..4 from the master weights.
__global__ void k_bf16_copies(const float *P, __nv_bfloat16 *Wf, __nv_bfloat16 *Wt)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * kSurH * kSurH)
        return;
    const int l = idx / (kSurH * kSurH), e = idx % (kSurH * kSurH), o = e / kSurH, i = e % kSurH;
    const __nv_bfloat16 w = __float2bfloat16_rn(P[sur_w_off(l + 2) + e]);
    Wf[idx] = w;
    Wt[(size_t)l * kSurH * kSurH + (size_t)i * kSurH + o] = w;
}

__global__ void k_gather_rows(const float *X, const float *y, const int *perm, int n, float *Xb, float *yb,
                              float clip)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int s = perm[i];
#pragma unroll
    for (int k = 0; k < kSurIn; ++k)
        Xb[i * kSurIn + k] = X[(size_t)s * kSurIn + k];
    yb[i] = fminf(clip, fmaxf(-clip, y[s]));
}

// ------------------------------------------------------------------ launchers

cudaError_t launch_gemm(int mode, const GemmArgs &g, cudaStream_t st)
{
    static bool attr_set[3] = {false, false, false};
    const dim3 grid(g.M / 128, 1, g.K / g.k_split);
    cudaError_t e = cudaSuccess;
    switch (mode) {
    case kGemmStore:
        if (!attr_set[0])
            e = cudaFuncSetAttribute(k_gemm_tc<kGemmStore>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
        attr_set[0] = (e == cudaSuccess);
        if (e == cudaSuccess)
            k_gemm_tc<kGemmStore><<<grid, kGemmThreads, kGemmSmem, st>>>(g);
        break;
    case kGemmFwd:
        if (!attr_set[1])
            e = cudaFuncSetAttribute(k_gemm_tc<kGemmFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
        attr_set[1] = (e == cudaSuccess);
        if (e == cudaSuccess)
            k_gemm_tc<kGemmFwd><<<grid, kGemmThreads, kGemmSmem, st>>>(g);
        break;
    default:
        if (!attr_set[2])
            e = cudaFuncSetAttribute(k_gemm_tc<kGemmBwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
        attr_set[2] = (e == cudaSuccess);
        if (e == cudaSuccess)
            k_gemm_tc<kGemmBwd><<<grid, kGemmThreads, kGemmSmem, st>>>(g);
        break;
    }
    if (e != cudaSuccess)
        return e;
    return cudaGetLastError();
}

void launch_layer1_fwd(const float *X, const float *P, float *Z, __nv_bfloat16 *H, __nv_bfloat16 *HT, int B,
                       cudaStream_t st)
{
    k_layer1_fwd<<<(B * kSurH + 255) / 256, 256, 0, st>>>(X, P, Z, H, HT, B);
}

void launch_out_fwd(const __nv_bfloat16 *H4, const float *P, const float *y, float *o, float *dO, float *r2, int B,
                    cudaStream_t st)
{
    k_out_fwd<<<(B + 7) / 8, 256, 0, st>>>(H4, P, y, o, dO, r2, B);
}

void launch_out_bwd(const float *dO, const float *P, const float *Z4, __nv_bfloat16 *dZ, __nv_bfloat16 *dZT, int B,
                    cudaStream_t st)
{
    k_out_bwd<<<(B * kSurH + 255) / 256, 256, 0, st>>>(dO, P, Z4, dZ, dZT, B);
}

void launch_row_reduce(const __nv_bfloat16 *MT, int rows, int B, const float *X, int nx, const float *u,
                       float *sum_out, float *dot_out, cudaStream_t st)
{
    k_row_reduce<<<rows, 256, 0, st>>>(MT, B, X, nx, u, sum_out, dot_out);
}

void launch_vec_sum(const float *v, int n, float *out, cudaStream_t st) { k_vec_sum<<<1, 256, 0, st>>>(v, n, out); }

void launch_splitk_reduce(const float *part, int splits, int n, float *out, cudaStream_t st)
{
    k_splitk_reduce<<<(n + 255) / 256, 256, 0, st>>>(part, splits, n, out);
}

void launch_adam(float *P, const float *G, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                 float c1, float c2, cudaStream_t st)
{
    k_adam<<<(n + 255) / 256, 256, 0, st>>>(P, G, m, v, n, lr, b1, b2, eps, c1, c2);
}

void launch_bf16_copies(const float *P, __nv_bfloat16 *Wf, __nv_bfloat16 *Wt, cudaStream_t st)
{
    k_bf16_copies<<<(3 * kSurH * kSurH + 255) / 256, 256, 0, st>>>(P, Wf, Wt);
}

void launch_gather_rows(const float *X, const float *y, const int *perm, int n, float *Xb, float *yb, float clip,
                        cudaStream_t st)
{
    k_gather_rows<<<(n + 255) / 256, 256, 0, st>>>(X, y, perm, n, Xb, yb, clip);
}

}  // namespace cgppd
