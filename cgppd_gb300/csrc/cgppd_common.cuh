// cgppd_common.cuh -- constants and device arithmetic shared by the CGPPD GB300 kernels.
//
// Physical constants carry the values the reference compiles (src/constants.h:8-46):
// every factor there is a float literal, so e.g. RT_to_kcalmol is the float result of
// 298*8.3144621/4184 and DH_CONVERSION_FACTOR the float CCELEC/80 expression.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cgppd {

constexpr float kRTtoKcal = 0.59218674898147583f;   // (T_room * Rgas / kcal)
constexpr float kDHFactor = 4.1507959365844727f;    // DH_CONVERSION_FACTOR
constexpr float kLambda = 0.159f;                   // LJ_lambda
constexpr float kE0 = -2.27f;                       // e0, RT units
constexpr float kXi = 10.0f;                        // Debye screening length, A
constexpr float kKcal = 4184.0f;                    // J per kcal
constexpr float kRgas = 8.3144621f;                 // J / (mol K)
constexpr float kKSpring = 378.0f;                  // bond spring, kcal/(mol A^2)
constexpr float kR0 = 3.81f;                        // bond length, A
constexpr float kGammaAngle = 0.1f;                 // angle term constants
constexpr float kGammaAngleRecip = 10.0f;
constexpr float kEpsAlpha = 4.3f;
constexpr float kThetaAlpha = 1.6f;
constexpr float kThetaBeta = 2.27f;
constexpr float kKAlpha = 106.4f;
constexpr float kKBeta = 26.3f;
constexpr float kPadder = -2.0f;                    // PADDER_IDENTIFIER
constexpr float kCrowder = -1.0f;                   // CROWDER_IDENTIFIER
constexpr float kRepulsiveCutoff = 15.0f;           // const_repulsive_cutoff, A
constexpr float kLog2e = 1.4426950408889634f;

// ------------------------------------------------------------------ float-float sums
// A (hi, lo) pair accumulated with Knuth's TwoSum: the rounding error of every add is
// carried in `lo`.  Pair terms are first summed in plain FP32 over a short tile, then
// folded in here (6 FP32 ops per tile), which keeps the per-residue sums at ~1e-7
// relative of the sum of magnitudes without FP64 arithmetic in the inner loop.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ void ff_add(FF &a, float b)
{
    float s = a.hi + b;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b - bb);
    a.hi = s;
    a.lo += err;
}

__device__ __forceinline__ double ff_value(const FF &a) { return (double)a.hi + (double)a.lo; }

// a += b for two float-float values (TwoSum of the high parts, the low parts added).
__device__ __forceinline__ void ff_add_ff(FF &a, FF b)
{
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b.hi - bb);
    a.hi = s;
    a.lo += err + b.lo;
}

// Sum over the warp (butterfly: every lane ends with the same value, in a fixed order).
__device__ __forceinline__ FF ff_warp_sum(FF v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        ff_add_ff(v, w);
    }
    return v;
}

// ------------------------------------------------------------------ geometry
__device__ __forceinline__ float min_image(float d, float L, float invL)
{
    // d - L*rint(d/L) (src/CudaFunctions.cu:321-333); L == 0 means no periodic box.  The
    // nearest integer to d/L comes from adding and removing 1.5 * 2^23 (exact for
    // |d/L| < 2^22), which keeps the whole term on the FMA pipe.
    const float k = __fadd_rn(__fmaf_rn(d, invL, 12582912.0f), -12582912.0f);
    return fmaf(-L, k, d);
}

// 1/sqrt(r2) on the SFU (PTX rsqrt.approx.ftz.f32, max relative error 2^-22.9) for the
// pair terms: a residue pair closer than 1e-19 A does not occur, and the error stays two
// orders below the 1e-5 energy bound.  (A Newton step on top, as rsqrt_refined does,
// lengthens each pair's dependency chain by four operations: 7-13 % of the MC kernel's
// throughput.)
__device__ __forceinline__ float rsqrt_sfu(float r2)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(r2));
    return y;
}

// 1/sqrt(r2) with one Newton step on top of the MUFU estimate (~0.5 ulp).
__device__ __forceinline__ float rsqrt_refined(float r2)
{
    float y = rsqrtf(r2);
    float h = 0.5f * r2 * y;
    return y * fmaf(-h, y, 1.5f);
}

// ------------------------------------------------------------------ pair energy
// Kim-Hummer pair term (src/Potential.cpp:5-42; src/CudaFunctions.cu:515-543):
//   Eij > 0 and r < 2^(1/6) sigma_ij : u = 4 Eij (s^12 - s^6) + 2 Eij
//   otherwise                         : u = -4 Eij (s^12 - s^6)
// with s = sigma_ij / r.  r < 2^(1/6) sigma_ij is tested as s^6 > 1/2, and both
// branches meet at that point (u = Eij), so the test's rounding does not matter.
// Returns the LJ part in the unit of `eij` and writes r, 1/r for the DH part.
__device__ __forceinline__ float lj_term(float eij, float sigma_ij, float inv_r2)
{
    float s2 = sigma_ij * sigma_ij * inv_r2;
    float s6 = s2 * s2 * s2;
    float u = -4.0f * eij * s6 * (s6 - 1.0f);
    if (eij > 0.0f && s6 > 0.5f)
        u = fmaf(2.0f, eij, -u);
    return u;
}

// 2^x on the SFU (PTX ex2.approx.ftz.f32, max relative error 2^-22); the Debye-Hueckel
// argument -r log2(e) / xi reaches the denormal range only beyond r = 873 A, where the
// term (< 1e-37 kcal/mol) flushes to zero.
__device__ __forceinline__ float ex2_sfu(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// q_i q_j exp(-r/xi) / r, with exp as ex2 on the SFU.
__device__ __forceinline__ float dh_term(float qq, float r, float inv_r)
{
    return qq * ex2_sfu(r * (-kLog2e / kXi)) * inv_r;
}

// ------------------------------------------------------------------ Philox4x32-10
// Counter-based generator (Salmon et al., SC'11).  Engine draws are
// philox(key = {seed ^ stream, seed_hi}, ctr = {step, step_hi, block, domain}).
struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        U4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// uniform double in [0, 1) from one 32-bit word (the resolution of a 32-bit
// Mersenne Twister draw, which is what the reference's gsl_rng_uniform returns).
__host__ __device__ __forceinline__ double u01(uint32_t x) { return (double)x * 2.3283064365386963e-10; }

}  // namespace cgppd
