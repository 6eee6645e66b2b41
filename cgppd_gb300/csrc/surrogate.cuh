// surrogate.cuh -- the learned pair-energy surrogate: pose features and the MLP layout.
//
// The surrogate predicts the inter-molecule energy E(a, b) (kcal/mol) of two copies of
// one rigid molecule from their relative pose.  Input (8 numbers):
//   d_body / 20 A      the minimum-image centre-to-centre vector b - a in a's body frame
//   10 A / |d|         inverse distance
//   q_rel              the rotation taking a's body frame to b's (unit quaternion, w >= 0)
// A molecule's body frame is the Gram-Schmidt frame of three fixed residues of its
// centred coordinates (e1 along f1 - f0, e2 from f2 - f0, e3 = e1 x e2); copies of one
// molecule share the residue choice, so the frame moves rigidly with the molecule.
//
// Network: 8 -> 256 -> 256 -> 256 -> 256 -> 1, SiLU after each hidden layer.  Layer 1
// (K = 8) and the output dot product run in FP32; layers 2-4 are BF16 tensor-core
// GEMMs with FP32 accumulation.  Master parameters are FP32 (Adam); the GEMM layers
// also keep BF16 copies: Wf[out][in] (forward operand) and Wt[in][out] (backward).
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace cgppd {

constexpr int kSurIn = 8;
constexpr int kSurH = 256;

// FP32 master parameter offsets
constexpr int kOffW1 = 0;                          // [256][8]
constexpr int kOffB1 = kOffW1 + kSurH * kSurIn;    // [256]
constexpr int kOffW2 = kOffB1 + kSurH;             // [256][256] (out, in)
constexpr int kOffB2 = kOffW2 + kSurH * kSurH;
constexpr int kOffW3 = kOffB2 + kSurH;
constexpr int kOffB3 = kOffW3 + kSurH * kSurH;
constexpr int kOffW4 = kOffB3 + kSurH;
constexpr int kOffB4 = kOffW4 + kSurH * kSurH;
constexpr int kOffW5 = kOffB4 + kSurH;             // [256]
constexpr int kOffB5 = kOffW5 + kSurH;             // [1]
constexpr int kSurParams = kOffB5 + 1;
constexpr int kSurParamsPad = (kSurParams + 3) & ~3;

__host__ __device__ constexpr int sur_w_off(int layer) { return layer == 2 ? kOffW2 : layer == 3 ? kOffW3 : kOffW4; }
__host__ __device__ constexpr int sur_b_off(int layer) { return layer == 1 ? kOffB1 : layer == 2 ? kOffB2 : layer == 3 ? kOffB3 : kOffB4; }

constexpr float kSurPosScale = 1.0f / 20.0f;
constexpr float kSurInvScale = 10.0f;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ float silu_grad(float z)
{
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

struct Frame {
    float e[3][3];   // rows: e1, e2, e3
};

__device__ __forceinline__ Frame frame_from(float4 q0, float4 q1, float4 q2)
{
    Frame F;
    float ax = q1.x - q0.x, ay = q1.y - q0.y, az = q1.z - q0.z;
    float n = rsqrtf(ax * ax + ay * ay + az * az);
    ax *= n, ay *= n, az *= n;
    float bx = q2.x - q0.x, by = q2.y - q0.y, bz = q2.z - q0.z;
    const float d = ax * bx + ay * by + az * bz;
    bx -= d * ax, by -= d * ay, bz -= d * az;
    n = rsqrtf(bx * bx + by * by + bz * bz);
    bx *= n, by *= n, bz *= n;
    F.e[0][0] = ax, F.e[0][1] = ay, F.e[0][2] = az;
    F.e[1][0] = bx, F.e[1][1] = by, F.e[1][2] = bz;
    F.e[2][0] = ay * bz - az * by;
    F.e[2][1] = az * bx - ax * bz;
    F.e[2][2] = ax * by - ay * bx;
    return F;
}

// Features of the ordered pair (a, b): centres ca, cb (wrapped), frames Fa, Fb.
__device__ __forceinline__ void pair_features(const Frame &Fa, float3 ca, const Frame &Fb, float3 cb, float box,
                                              float invbox, float *x)
{
    float dx = cb.x - ca.x, dy = cb.y - ca.y, dz = cb.z - ca.z;
    if (box > 0.f) {
        dx -= box * rintf(dx * invbox);
        dy -= box * rintf(dy * invbox);
        dz -= box * rintf(dz * invbox);
    }
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    x[0] = (Fa.e[0][0] * dx + Fa.e[0][1] * dy + Fa.e[0][2] * dz) * kSurPosScale;
    x[1] = (Fa.e[1][0] * dx + Fa.e[1][1] * dy + Fa.e[1][2] * dz) * kSurPosScale;
    x[2] = (Fa.e[2][0] * dx + Fa.e[2][1] * dy + Fa.e[2][2] * dz) * kSurPosScale;
    x[3] = kSurInvScale / fmaxf(r, 1.0f);
    // R = Fa Fb^T maps b's body coordinates to a's: R_ij = e_i(a) . e_j(b)
    float R[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            R[i][j] = Fa.e[i][0] * Fb.e[j][0] + Fa.e[i][1] * Fb.e[j][1] + Fa.e[i][2] * Fb.e[j][2];
    // rotation matrix -> quaternion (largest-component branch), then w >= 0
    float w, qx, qy, qz;
    const float tr = R[0][0] + R[1][1] + R[2][2];
    if (tr > 0.f) {
        const float s = sqrtf(tr + 1.0f) * 2.f;
        w = 0.25f * s;
        qx = (R[2][1] - R[1][2]) / s;
        qy = (R[0][2] - R[2][0]) / s;
        qz = (R[1][0] - R[0][1]) / s;
    } else if (R[0][0] > R[1][1] && R[0][0] > R[2][2]) {
        const float s = sqrtf(1.0f + R[0][0] - R[1][1] - R[2][2]) * 2.f;
        w = (R[2][1] - R[1][2]) / s;
        qx = 0.25f * s;
        qy = (R[0][1] + R[1][0]) / s;
        qz = (R[0][2] + R[2][0]) / s;
    } else if (R[1][1] > R[2][2]) {
        const float s = sqrtf(1.0f + R[1][1] - R[0][0] - R[2][2]) * 2.f;
        w = (R[0][2] - R[2][0]) / s;
        qx = (R[0][1] + R[1][0]) / s;
        qy = 0.25f * s;
        qz = (R[1][2] + R[2][1]) / s;
    } else {
        const float s = sqrtf(1.0f + R[2][2] - R[0][0] - R[1][1]) * 2.f;
        w = (R[1][0] - R[0][1]) / s;
        qx = (R[0][2] + R[2][0]) / s;
        qy = (R[1][2] + R[2][1]) / s;
        qz = 0.25f * s;
    }
    if (w < 0.f)
        w = -w, qx = -qx, qy = -qy, qz = -qz;
    x[4] = w, x[5] = qx, x[6] = qy, x[7] = qz;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// D(16x8, f32) += A(16x16 bf16, row) * B(16x8 bf16, col)
__device__ __forceinline__ void mma_bf16_16816(float *d, const uint32_t *a, const uint32_t *b)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

}  // namespace cgppd
