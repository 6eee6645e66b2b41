// surrogate_internal.h -- declarations shared by the surrogate's kernels and host code.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

struct cgppd_surrogate;

namespace cgppd {

enum GemmMode { kGemmStore = 0, kGemmFwd = 1, kGemmBwd = 2 };

// C = A * B^T on the tcgen05 tensor cores, A [M][K], B [256][K] (bf16, K-major).
struct GemmArgs {
    const __nv_bfloat16 *A;   // [M][K]
    const __nv_bfloat16 *B;   // [256][K]
    int M, K, k_split;        // M % 128 == 0, K % k_split == 0, k_split % 64 == 0
    float *C;                 // store: [K / k_split][M][256]
    const float *bias;        // fwd
    float *Z;                 // fwd: [M][256]
    __nv_bfloat16 *H, *HT;    // fwd: [M][256], [256][M]; bwd: dZ, dZ^T
    const float *Zp;          // bwd: pre-activation of the layer below, [M][256]
    unsigned *err;
};

cudaError_t launch_gemm(int mode, const GemmArgs &g, cudaStream_t st);
void launch_layer1_fwd(const float *X, const float *P, float *Z, __nv_bfloat16 *H, __nv_bfloat16 *HT, int B,
                       cudaStream_t st);
void launch_out_fwd(const __nv_bfloat16 *H4, const float *P, const float *y, float *o, float *dO, float *r2, int B,
                    cudaStream_t st);
void launch_out_bwd(const float *dO, const float *P, const float *Z4, __nv_bfloat16 *dZ, __nv_bfloat16 *dZT, int B,
                    cudaStream_t st);
void launch_row_reduce(const __nv_bfloat16 *MT, int rows, int B, const float *X, int nx, const float *u,
                       float *sum_out, float *dot_out, cudaStream_t st);
void launch_vec_sum(const float *v, int n, float *out, cudaStream_t st);
void launch_splitk_reduce(const float *part, int splits, int n, float *out, cudaStream_t st);
void launch_adam(float *P, const float *G, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                 float c1, float c2, cudaStream_t st);
void launch_bf16_copies(const float *P, __nv_bfloat16 *Wf, __nv_bfloat16 *Wt, cudaStream_t st);
void launch_gather_rows(const float *X, const float *y, const int *perm, int n, float *Xb, float *yb, float clip,
                        cudaStream_t st);

// The engine reads a trained surrogate's FP32 parameters and BF16 forward weights.
const float *surrogate_device_params(const cgppd_surrogate *s);
const __nv_bfloat16 *surrogate_device_wf(const cgppd_surrogate *s);
// Append n samples held in device memory (features [n][8], energies [n]).
int surrogate_append_device_samples(cgppd_surrogate *s, const float *dX, const float *dY, int n);

}  // namespace cgppd
