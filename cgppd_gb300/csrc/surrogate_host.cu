// surrogate_host.cu -- the pair-energy surrogate object: parameters, dataset, training.
//
// Training is plain mini-batch Adam on the mean squared error against targets clipped
// to +-clip kcal/mol (clashes only need to read as "large").  Every step runs the
// project's own kernels (mlp_kernels.cu): FP32 layer 1, three tcgen05 BF16 GEMMs with
// fused bias/SiLU epilogues, FP32 output, then the backward pass as split-K tcgen05
// GEMMs for the weight gradients (reduced in a fixed order) and GEMMs with fused SiLU'
// epilogues for the activation gradients.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "cgppd_surrogate.h"
#include "devbuf.h"
#include "status.h"
#include "surrogate.cuh"
#include "surrogate_internal.h"


using namespace cgppd;

namespace {

uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

float uniform_pm(uint64_t &s, float a)
{
    const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
    return (float)((2.0 * u - 1.0) * a);
}

}  // namespace

struct cgppd_surrogate {
    int batch = 0;
    int k_split = 0;
    uint64_t seed = 0;
    int adam_t = 0;
    cudaStream_t stream = nullptr;

    DevBuf<float> P, G, am, av;
    DevBuf<__nv_bfloat16> Wf, Wt;
    // activations of one batch
    DevBuf<float> X, y, Z, o, dO, r2, Cpart, scalars;
    DevBuf<__nv_bfloat16> H, HT, dZ, dZT;
    DevBuf<unsigned> err;
    // dataset
    DevBuf<float> dsX, dsY;
    DevBuf<int> perm;
    std::vector<float> hX, hY;   // host mirror of the dataset (appended by collect/set)
    bool ds_dirty = true;

    ~cgppd_surrogate()
    {
        if (stream)
            cudaStreamDestroy(stream);
    }

    int init(int b, uint64_t sd)
    {
        batch = b;
        seed = sd;
        k_split = std::min(batch, 1024);
        if (cgppd_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "surrogate stream") != 0)
            return -1;
        const size_t BH = (size_t)batch * kSurH;
        if (P.zero(kSurParamsPad) || G.zero(kSurParamsPad) || am.zero(kSurParamsPad) || av.zero(kSurParamsPad) ||
            Wf.alloc(3 * kSurH * kSurH) || Wt.alloc(3 * kSurH * kSurH) || X.zero((size_t)batch * kSurIn) ||
            y.zero(batch) || Z.alloc(4 * BH) || o.alloc(batch) || dO.alloc(batch) || r2.alloc(batch) ||
            Cpart.alloc((size_t)(batch / k_split) * kSurH * kSurH) || scalars.zero(4) || H.alloc(4 * BH) ||
            HT.alloc(4 * BH) || dZ.alloc(2 * BH) || dZT.alloc(2 * BH) || err.zero(1))
            return -1;
        // PyTorch-Linear-style initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in))
        std::vector<float> p(kSurParamsPad, 0.f);
        uint64_t s = seed ^ 0x5EED5EEDull;
        auto fill = [&](int off, int count, int fan_in) {
            const float a = 1.0f / std::sqrt((float)fan_in);
            for (int i = 0; i < count; ++i)
                p[off + i] = uniform_pm(s, a);
        };
        fill(kOffW1, kSurH * kSurIn, kSurIn);
        fill(kOffB1, kSurH, kSurIn);
        for (int l = 2; l <= 4; ++l) {
            fill(sur_w_off(l), kSurH * kSurH, kSurH);
            fill(sur_b_off(l), kSurH, kSurH);
        }
        fill(kOffW5, kSurH, kSurH);
        fill(kOffB5, 1, kSurH);
        return set_params(p.data());
    }

    int set_params(const float *host)
    {
        if (cgppd_check(cudaMemcpy(P.ptr, host, kSurParams * sizeof(float), cudaMemcpyHostToDevice), "surrogate params"))
            return -1;
        launch_bf16_copies(P.ptr, Wf.ptr, Wt.ptr, stream);
        return cgppd_check(cudaStreamSynchronize(stream), "surrogate bf16 copies");
    }

    // forward (and backward when `grad`) over the batch in X/y (n rows, n % 128 == 0,
    // n <= batch).  Returns 0 or -1.
    int step(int n, bool with_targets, bool grad, float *loss_out)
    {
        const size_t BH = (size_t)n * kSurH;
        cudaStream_t st = stream;
        float *Zl[4];
        __nv_bfloat16 *Hl[4], *HTl[4];
        for (int l = 0; l < 4; ++l) {
            Zl[l] = Z.ptr + l * BH;
            Hl[l] = H.ptr + l * BH;
            HTl[l] = HT.ptr + l * BH;
        }
        launch_layer1_fwd(X.ptr, P.ptr, Zl[0], Hl[0], HTl[0], n, st);
        for (int l = 2; l <= 4; ++l) {
            GemmArgs g{};
            g.A = Hl[l - 2];
            g.B = Wf.ptr + (size_t)(l - 2) * kSurH * kSurH;
            g.M = n;
            g.K = kSurH;
            g.k_split = kSurH;
            g.bias = P.ptr + sur_b_off(l);
            g.Z = Zl[l - 1];
            g.H = Hl[l - 1];
            g.HT = HTl[l - 1];
            g.err = err.ptr;
            if (cgppd_check(launch_gemm(kGemmFwd, g, st), "surrogate forward GEMM"))
                return -1;
        }
        launch_out_fwd(Hl[3], P.ptr, with_targets ? y.ptr : nullptr, o.ptr, dO.ptr, r2.ptr, n, st);
        if (with_targets)
            launch_vec_sum(r2.ptr, n, scalars.ptr, st);
        if (grad) {
            const int ks = std::min(n, k_split);
            if (n % ks != 0 || ks % 64 != 0)
                return cgppd_fail("surrogate: batch must be a multiple of 64 (and of the split size)");
            // output layer
            launch_row_reduce(HTl[3], kSurH, n, nullptr, 0, dO.ptr, nullptr, G.ptr + kOffW5, st);
            launch_vec_sum(dO.ptr, n, G.ptr + kOffB5, st);
            __nv_bfloat16 *dZl[2] = {dZ.ptr, dZ.ptr + BH}, *dZTl[2] = {dZT.ptr, dZT.ptr + BH};
            launch_out_bwd(dO.ptr, P.ptr, Zl[3], dZl[0], dZTl[0], n, st);
            int cur = 0;
            for (int l = 4; l >= 2; --l) {
                GemmArgs gw{};
                gw.A = dZTl[cur];
                gw.B = HTl[l - 2];
                gw.M = kSurH;
                gw.K = n;
                gw.k_split = ks;
                gw.C = Cpart.ptr;
                gw.err = err.ptr;
                if (cgppd_check(launch_gemm(kGemmStore, gw, st), "surrogate weight-gradient GEMM"))
                    return -1;
                launch_splitk_reduce(Cpart.ptr, n / ks, kSurH * kSurH, G.ptr + sur_w_off(l), st);
                launch_row_reduce(dZTl[cur], kSurH, n, nullptr, 0, nullptr, G.ptr + sur_b_off(l), nullptr, st);
                GemmArgs gb{};
                gb.A = dZl[cur];
                gb.B = Wt.ptr + (size_t)(l - 2) * kSurH * kSurH;
                gb.M = n;
                gb.K = kSurH;
                gb.k_split = kSurH;
                gb.Zp = Zl[l - 2];
                gb.H = dZl[cur ^ 1];
                gb.HT = dZTl[cur ^ 1];
                gb.err = err.ptr;
                if (cgppd_check(launch_gemm(kGemmBwd, gb, st), "surrogate activation-gradient GEMM"))
                    return -1;
                cur ^= 1;
            }
            launch_row_reduce(dZTl[cur], kSurH, n, X.ptr, kSurIn, nullptr, G.ptr + kOffB1, G.ptr + kOffW1, st);
        }
        if (cgppd_check(cudaGetLastError(), "surrogate kernels"))
            return -1;
        if (loss_out && with_targets) {
            float v = 0.f;
            if (cgppd_check(cudaMemcpyAsync(&v, scalars.ptr, sizeof(float), cudaMemcpyDeviceToHost, st), "loss") ||
                cgppd_check(cudaStreamSynchronize(st), "surrogate step"))
                return -1;
            *loss_out = v / (float)n;
        }
        return check_err();
    }

    int check_err()
    {
        unsigned e = 0;
        if (cgppd_check(cudaMemcpyAsync(&e, err.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, stream), "err") ||
            cgppd_check(cudaStreamSynchronize(stream), "surrogate sync"))
            return -1;
        if (e)
            return cgppd_fail("surrogate: a tensor-core GEMM timed out waiting for its MMAs");
        return 0;
    }

    void adam(float lr)
    {
        ++adam_t;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
        launch_adam(P.ptr, G.ptr, am.ptr, av.ptr, kSurParams, lr, b1, b2, 1e-8f, c1, c2, stream);
        launch_bf16_copies(P.ptr, Wf.ptr, Wt.ptr, stream);
    }

    int upload_dataset()
    {
        if (!ds_dirty)
            return 0;
        if (dsX.upload(hX) || dsY.upload(hY))
            return -1;
        ds_dirty = false;
        return 0;
    }

    // predictions for rows [0, n) of host or device features (host if `host`)
    int predict(const float *Xsrc, int n, float *out_host)
    {
        for (int s0 = 0; s0 < n; s0 += batch) {
            const int cnt = std::min(batch, n - s0);
            const int padded = (cnt + 127) / 128 * 128;
            if (cgppd_check(cudaMemsetAsync(X.ptr, 0, (size_t)padded * kSurIn * sizeof(float), stream), "memset") ||
                cgppd_check(cudaMemcpyAsync(X.ptr, Xsrc + (size_t)s0 * kSurIn, (size_t)cnt * kSurIn * sizeof(float),
                                            cudaMemcpyDefault, stream),
                            "features"))
                return -1;
            if (step(padded, false, false, nullptr))
                return -1;
            if (cgppd_check(cudaMemcpyAsync(out_host + s0, o.ptr, cnt * sizeof(float), cudaMemcpyDeviceToHost, stream),
                            "predictions") ||
                cgppd_check(cudaStreamSynchronize(stream), "predict"))
                return -1;
        }
        return 0;
    }
};

// ------------------------------------------------------------------ C ABI

extern "C" {

cgppd_surrogate *cgppd_surrogate_create(int batch, unsigned long long seed)
{
    if (batch <= 0 || batch % 128 != 0) {
        cgppd_fail("cgppd_surrogate_create: batch must be a positive multiple of 128");
        return nullptr;
    }
    auto *s = new cgppd_surrogate();
    if (s->init(batch, seed) != 0) {
        delete s;
        return nullptr;
    }
    return s;
}

void cgppd_surrogate_destroy(cgppd_surrogate *s) { delete s; }

int cgppd_surrogate_num_params(void) { return kSurParams; }

int cgppd_surrogate_get_params(cgppd_surrogate *s, float *out)
{
    if (!s || !out)
        return cgppd_fail("cgppd_surrogate_get_params: null argument");
    return cgppd_check(cudaMemcpy(out, s->P.ptr, kSurParams * sizeof(float), cudaMemcpyDeviceToHost), "get params");
}

int cgppd_surrogate_set_params(cgppd_surrogate *s, const float *in)
{
    if (!s || !in)
        return cgppd_fail("cgppd_surrogate_set_params: null argument");
    return s->set_params(in);
}

int cgppd_surrogate_loss_grad(cgppd_surrogate *s, const float *X, const float *y, int n, float *loss, float *grad)
{
    if (!s || !X || !y)
        return cgppd_fail("cgppd_surrogate_loss_grad: null argument");
    if (n <= 0 || n > s->batch || n % 128 != 0)
        return cgppd_fail("cgppd_surrogate_loss_grad: n must be a multiple of 128 no larger than the batch");
    if (cgppd_check(cudaMemcpy(s->X.ptr, X, (size_t)n * kSurIn * sizeof(float), cudaMemcpyHostToDevice), "X") ||
        cgppd_check(cudaMemcpy(s->y.ptr, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice), "y"))
        return -1;
    if (s->step(n, true, grad != nullptr, loss))
        return -1;
    if (grad)
        return cgppd_check(cudaMemcpy(grad, s->G.ptr, kSurParams * sizeof(float), cudaMemcpyDeviceToHost), "grad");
    return 0;
}

int cgppd_surrogate_predict(cgppd_surrogate *s, const float *X, int n, float *out)
{
    if (!s || (!X && n > 0) || (!out && n > 0))
        return cgppd_fail("cgppd_surrogate_predict: null argument");
    return s->predict(X, n, out);
}

int cgppd_surrogate_add_samples(cgppd_surrogate *s, const float *X, const float *y, int n)
{
    if (!s || n < 0 || (n > 0 && (!X || !y)))
        return cgppd_fail("cgppd_surrogate_add_samples: bad argument");
    s->hX.insert(s->hX.end(), X, X + (size_t)n * kSurIn);
    s->hY.insert(s->hY.end(), y, y + n);
    s->ds_dirty = true;
    return 0;
}

int cgppd_surrogate_clear_samples(cgppd_surrogate *s)
{
    if (!s)
        return cgppd_fail("cgppd_surrogate_clear_samples: null surrogate");
    s->hX.clear();
    s->hY.clear();
    s->ds_dirty = true;
    return 0;
}

long long cgppd_surrogate_num_samples(cgppd_surrogate *s) { return s ? (long long)s->hY.size() : -1; }

int cgppd_surrogate_get_samples(cgppd_surrogate *s, float *X, float *y, long long n)
{
    if (!s || n > (long long)s->hY.size())
        return cgppd_fail("cgppd_surrogate_get_samples: bad argument");
    std::memcpy(X, s->hX.data(), (size_t)n * kSurIn * sizeof(float));
    std::memcpy(y, s->hY.data(), (size_t)n * sizeof(float));
    return 0;
}

// Train on the first (1 - val_fraction) of the samples (in their stored order, which
// the collector already randomises), `epochs` passes in a seeded shuffled order.
// history[2 * e] = training RMSE of epoch e (clipped targets, running over its
// batches), history[2 * e + 1] = RMSE on the held-out samples with |y| <= clip.
int cgppd_surrogate_train(cgppd_surrogate *s, int epochs, float lr, float clip, float val_fraction, float *history)
{
    if (!s || epochs < 0 || !(lr > 0.f) || !(clip > 0.f) || val_fraction < 0.f || val_fraction >= 1.f)
        return cgppd_fail("cgppd_surrogate_train: bad argument");
    const long long total = (long long)s->hY.size();
    const long long nval = (long long)(val_fraction * (double)total);
    const long long ntrain = total - nval;
    const int B = s->batch;
    if (ntrain < B)
        return cgppd_fail("cgppd_surrogate_train: fewer training samples than one batch");
    if (s->upload_dataset())
        return -1;
    if (s->perm.alloc(ntrain))
        return -1;
    std::vector<int> perm(ntrain);
    uint64_t rs = s->seed ^ 0x7A11ull;
    const long long nb = ntrain / B;
    for (int e = 0; e < epochs; ++e) {
        std::iota(perm.begin(), perm.end(), 0);
        for (long long i = ntrain - 1; i > 0; --i) {
            const long long j = (long long)(splitmix64(rs) % (uint64_t)(i + 1));
            std::swap(perm[i], perm[j]);
        }
        if (cgppd_check(cudaMemcpyAsync(s->perm.ptr, perm.data(), ntrain * sizeof(int), cudaMemcpyHostToDevice,
                                        s->stream),
                        "permutation"))
            return -1;
        double sse = 0.0;
        long long nlog = 0;
        for (long long b = 0; b < nb; ++b) {
            launch_gather_rows(s->dsX.ptr, s->dsY.ptr, s->perm.ptr + b * B, B, s->X.ptr, s->y.ptr, clip, s->stream);
            float loss = 0.f;
            const bool want_loss = (b == nb - 1) || (b % 16 == 0);
            if (s->step(B, true, true, want_loss ? &loss : nullptr))
                return -1;
            s->adam(lr);
            if (want_loss) {
                sse += (double)loss;
                ++nlog;
            }
        }
        if (cgppd_check(cudaStreamSynchronize(s->stream), "training epoch"))
            return -1;
        if (history) {
            history[2 * e] = (float)std::sqrt(sse / (double)std::max(1ll, nlog));
            history[2 * e + 1] = -1.f;
        }
        if (history && nval > 0) {
            std::vector<float> pred(nval);
            if (s->predict(s->dsX.ptr + ntrain * kSurIn, (int)nval, pred.data()))
                return -1;
            double se = 0.0;
            long long cnt = 0;
            for (long long i = 0; i < nval; ++i) {
                const float yt = s->hY[ntrain + i];
                if (std::fabs(yt) <= clip) {
                    se += (double)(pred[i] - yt) * (double)(pred[i] - yt);
                    ++cnt;
                }
            }
            history[2 * e + 1] = cnt ? (float)std::sqrt(se / (double)cnt) : -1.f;
        }
    }
    return 0;
}

}  // extern "C"

namespace cgppd {
const float *surrogate_device_params(const cgppd_surrogate *s) { return s ? s->P.ptr : nullptr; }
const __nv_bfloat16 *surrogate_device_wf(const cgppd_surrogate *s) { return s ? s->Wf.ptr : nullptr; }
int surrogate_append_device_samples(cgppd_surrogate *s, const float *dX, const float *dY, int n)
{
    std::vector<float> x((size_t)n * kSurIn), y(n);
    if (cgppd_check(cudaMemcpy(x.data(), dX, x.size() * sizeof(float), cudaMemcpyDeviceToHost), "samples") ||
        cgppd_check(cudaMemcpy(y.data(), dY, y.size() * sizeof(float), cudaMemcpyDeviceToHost), "samples"))
        return -1;
    return cgppd_surrogate_add_samples(s, x.data(), y.data(), n);
}
}  // namespace cgppd
