// Learned Strassen scheduler: a 2 x 64 MLP that predicts, per candidate node
// of the Strassen decision tree (matmult_strassen_dryrun, strassen.hpp:
// 511-679), log(t_strassen / t_sparse) from the node's features, trained on
// timings the library takes of its own Strassen and sparse paths.  The
// reference's cost model (nf >= cost, strassen.hpp:602-640) is the fallback
// for nodes the network does not cover.
//
// Everything runs on the device with hand-written kernels: feature
// extraction from the block norms, the forward pass, the backward pass
// (per-sample gradients summed in a fixed order, so training is
// deterministic) and Adam.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>

#include "bsg_sched.cuh"

namespace bsg {

// ---- parameter layout (float) ----
constexpr int kW1 = 0;                          // [H][IN]
constexpr int kB1 = kW1 + kSchedH * kSchedIn;   // [H]
constexpr int kW2 = kB1 + kSchedH;              // [H][H]
constexpr int kB2 = kW2 + kSchedH * kSchedH;    // [H]
constexpr int kW3 = kB2 + kSchedH;              // [H]
constexpr int kB3 = kW3 + kSchedH;              // [1]
static_assert(kB3 + 1 == kSchedParams, "parameter count");

// forward: one CTA of kSchedH threads per sample (sample index idx[b] or b)
__global__ void __launch_bounds__(kSchedH) k_mlp_fwd(const float *__restrict__ X, const int *__restrict__ idx, int n,
                                                     const float *__restrict__ P, float *__restrict__ H1,
                                                     float *__restrict__ H2, float *__restrict__ Y) {
    const int b = blockIdx.x, j = threadIdx.x;
    if (b >= n) return;
    const int src = idx ? idx[b] : b;
    __shared__ float x[kSchedIn], h1[kSchedH], h2[kSchedH], part[2];
    if (j < kSchedIn) x[j] = X[(size_t)src * kSchedIn + j];
    __syncthreads();
    float a = P[kB1 + j];
    for (int i = 0; i < kSchedIn; ++i) a = fmaf(P[kW1 + j * kSchedIn + i], x[i], a);
    h1[j] = fmaxf(a, 0.f);
    __syncthreads();
    a = P[kB2 + j];
    for (int i = 0; i < kSchedH; ++i) a = fmaf(P[kW2 + j * kSchedH + i], h1[i], a);
    h2[j] = fmaxf(a, 0.f);
    if (H1) H1[(size_t)b * kSchedH + j] = h1[j];
    if (H2) H2[(size_t)b * kSchedH + j] = h2[j];
    // output: fixed-order tree over the 64 products
    float t = P[kW3 + j] * h2[j];
    for (int o = 16; o >= 1; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((j & 31) == 0) part[j >> 5] = t;
    __syncthreads();
    if (j == 0) Y[b] = P[kB3] + (part[0] + part[1]);
}

// backward of the mean squared error: per-sample gradient rows G[b][param]
__global__ void __launch_bounds__(kSchedH) k_mlp_bwd(const float *__restrict__ X, const int *__restrict__ idx, int n,
                                                     const float *__restrict__ P, const float *__restrict__ H1,
                                                     const float *__restrict__ H2, const float *__restrict__ Y,
                                                     const float *__restrict__ T, float *__restrict__ G) {
    const int b = blockIdx.x, j = threadIdx.x;
    if (b >= n) return;
    const int src = idx ? idx[b] : b;
    __shared__ float x[kSchedIn], h1[kSchedH], dh2[kSchedH];
    if (j < kSchedIn) x[j] = X[(size_t)src * kSchedIn + j];
    h1[j] = H1[(size_t)b * kSchedH + j];
    const float h2 = H2[(size_t)b * kSchedH + j];
    const float dy = 2.f * (Y[b] - T[src]) / (float)n;
    float *g = G + (size_t)b * kSchedParams;
    g[kW3 + j] = dy * h2;
    if (j == 0) g[kB3] = dy;
    dh2[j] = h2 > 0.f ? dy * P[kW3 + j] : 0.f;
    __syncthreads();
    for (int i = 0; i < kSchedH; ++i) g[kW2 + j * kSchedH + i] = dh2[j] * h1[i];
    g[kB2 + j] = dh2[j];
    // dh1[j] = sum_k W2[k][j] dh2[k] where h1[j] > 0
    float a = 0.f;
    for (int k = 0; k < kSchedH; ++k) a = fmaf(P[kW2 + k * kSchedH + j], dh2[k], a);
    const float dh1 = h1[j] > 0.f ? a : 0.f;
    for (int i = 0; i < kSchedIn; ++i) g[kW1 + j * kSchedIn + i] = dh1 * x[i];
    g[kB1 + j] = dh1;
}

// grad[p] = sum_b G[b][p] in sample order
__global__ void k_mlp_gsum(const float *__restrict__ G, int n, float *__restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kSchedParams) return;
    float a = 0.f;
    for (int b = 0; b < n; ++b) a += G[(size_t)b * kSchedParams + p];
    grad[p] = a;
}

// loss = mean (Y - T)^2, one thread, sample order
__global__ void k_mlp_loss(const float *__restrict__ Y, const float *__restrict__ T, const int *__restrict__ idx, int n,
                           float *__restrict__ loss) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float a = 0.f;
    for (int b = 0; b < n; ++b) {
        const float d = Y[b] - T[idx ? idx[b] : b];
        a = fmaf(d, d, a);
    }
    *loss = a / (float)n;
}

// Adam (Kingma & Ba 2015) with bias correction
__global__ void k_adam(float *__restrict__ P, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kSchedParams) return;
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.f - b1) * g, vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    P[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// ---- node features ----
// For node (si, sj, sk) of level L (super-blocks of sb = 2^(L+1) blocks):
//  0 level / 8            1 log2(sb) / 8          2 log2(1 + nf) / 64
//  3 log2(cost) / 64      4 log2(nf / cost) / 8   5 nf / dense flops
//  6 A density            7 B density             8 C density
//  9..16  histogram of log10 ||A_ik|| over [-20, 4) in 8 bins (fractions of present blocks)
// 17..24  the same for B
// and eligibility (all A, B, C blocks present, not an edge node).
__device__ __forceinline__ int hist_bin(double nrm) {
    if (!(nrm > 0.0)) return 0;
    const double l = log10(nrm);
    const int b = (int)floor((l + 20.0) / 3.0);
    return b < 0 ? 0 : (b > 7 ? 7 : b);
}

__global__ void k_node_features(double *const *__restrict__ A, const double *__restrict__ An, size_t a_nrb,
                                double *const *__restrict__ B, const double *__restrict__ Bn, size_t b_nrb,
                                double *const *__restrict__ C, size_t c_nrb, size_t nib, size_t njb, size_t nkb,
                                int level, size_t nsi, size_t nsj, size_t nsk, size_t bs,
                                const unsigned long long *__restrict__ nf, const uint8_t *__restrict__ edge,
                                unsigned long long cost, float *__restrict__ F, uint8_t *__restrict__ ok) {
    const size_t node = blockIdx.x;
    if (node >= nsi * nsj * nsk) return;
    const size_t si = node % nsi, sj = (node / nsi) % nsj, sk = node / (nsi * nsj);
    const size_t sb = (size_t)1 << (level + 1);
    const size_t ib0 = si * sb, jb0 = sj * sb, kb0 = sk * sb;
    const size_t ib1 = min(ib0 + sb, nib), jb1 = min(jb0 + sb, njb), kb1 = min(kb0 + sb, nkb);
    const size_t nA = (ib1 - ib0) * (kb1 - kb0), nB = (kb1 - kb0) * (jb1 - jb0), nC = (ib1 - ib0) * (jb1 - jb0);
    unsigned cA = 0, cB = 0, cC = 0, hA[8] = {0}, hB[8] = {0};
    for (size_t e = threadIdx.x; e < nA; e += blockDim.x) {
        const size_t r = ib0 + e % (ib1 - ib0), c = kb0 + e / (ib1 - ib0);
        if (A[r + c * a_nrb]) {
            ++cA;
            ++hA[hist_bin(An[r + c * a_nrb])];
        }
    }
    for (size_t e = threadIdx.x; e < nB; e += blockDim.x) {
        const size_t r = kb0 + e % (kb1 - kb0), c = jb0 + e / (kb1 - kb0);
        if (B[r + c * b_nrb]) {
            ++cB;
            ++hB[hist_bin(Bn[r + c * b_nrb])];
        }
    }
    for (size_t e = threadIdx.x; e < nC; e += blockDim.x) {
        const size_t r = ib0 + e % (ib1 - ib0), c = jb0 + e / (ib1 - ib0);
        if (C[r + c * c_nrb]) ++cC;
    }
    // block reduction of the 19 counters (fixed order)
    __shared__ unsigned red[19][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned vals[19] = {cA, cB, cC, hA[0], hA[1], hA[2], hA[3], hA[4], hA[5], hA[6], hA[7],
                         hB[0], hB[1], hB[2], hB[3], hB[4], hB[5], hB[6], hB[7]};
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        unsigned t = vals[q];
        for (int o = 16; o >= 1; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) red[q][w] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned tot[19];
        for (int q = 0; q < 19; ++q) {
            tot[q] = 0;
            for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) tot[q] += red[q][ww];
        }
        const double nfl = (double)nf[node], cst = (double)cost;
        const double dense = 2.0 * (double)bs * bs * bs * (double)((ib1 - ib0) * (jb1 - jb0) * (kb1 - kb0));
        float *f = F + node * kSchedNodeIn;
        f[0] = (float)level / 8.f;
        f[1] = (float)log2((double)sb) / 8.f;
        f[2] = (float)(log2(1.0 + nfl) / 64.0);
        f[3] = (float)(log2(cst) / 64.0);
        f[4] = (float)(log2((nfl + 1.0) / cst) / 8.0);
        f[5] = (float)(nfl / dense);
        f[6] = nA ? (float)tot[0] / (float)nA : 0.f;
        f[7] = nB ? (float)tot[1] / (float)nB : 0.f;
        f[8] = nC ? (float)tot[2] / (float)nC : 0.f;
        for (int q = 0; q < 8; ++q) {
            f[9 + q] = tot[0] ? (float)tot[3 + q] / (float)tot[0] : 0.f;
            f[17 + q] = tot[1] ? (float)tot[11 + q] / (float)tot[1] : 0.f;
        }
        ok[node] = !edge[node] && tot[0] == nA && tot[1] == nB && tot[2] == nC;
    }
}

// option rows: node features, then the option's one-hot
__global__ void k_option_rows(const float *__restrict__ F, size_t n, float *__restrict__ X) {
    const size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n * kSchedOpts) return;
    const size_t i = r / kSchedOpts;
    const int o = (int)(r % kSchedOpts);
    float *x = X + r * kSchedIn;
    for (int j = 0; j < kSchedNodeIn; ++j) x[j] = F[i * kSchedNodeIn + j];
    for (int j = 0; j < kSchedOpts; ++j) x[kSchedNodeIn + j] = j == o ? 1.f : 0.f;
}

void launch_option_rows(bsg_ctx ctx, const float *F, size_t n, float *X) {
    if (!n) return;
    k_option_rows<<<(unsigned)ceil_div(n * kSchedOpts, (size_t)256), 256, 0, ctx->stream>>>(F, n, X);
    ctx->note_launch();
    ctx->check_launch("scheduler option rows");
}

// per node the option the network predicts fastest, where it beats the
// sparse recursion (options in order, ties to the first)
__global__ void k_sched_decide(const uint8_t *__restrict__ ok, const float *__restrict__ y, size_t n, int level,
                               uint8_t *__restrict__ tree) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int best = -1;
    float yb = 0.f;
    for (int o = 0; o < kSchedOpts; ++o) {
        const bool valid = o == kSchedOpts - 1 || o <= level;  // depth o + 1 needs 2^o | 2^level
        const float v = y[i * kSchedOpts + o];
        if (valid && v < yb) {
            yb = v;
            best = o;
        }
    }
    tree[i] = (ok[i] && best >= 0) ? (uint8_t)(kNodeDepth1 + best) : kNodeSparse;
}

void launch_sched_decide(bsg_ctx ctx, const uint8_t *ok, const float *y, size_t n, int level, uint8_t *tree) {
    if (!n) return;
    k_sched_decide<<<(unsigned)ceil_div(n, (size_t)256), 256, 0, ctx->stream>>>(ok, y, n, level, tree);
    ctx->note_launch();
    ctx->check_launch("scheduler decisions");
}

void launch_node_features(bsg_bsm A, bsg_bsm B, bsg_bsm C, int level, size_t nsi, size_t nsj, size_t nsk,
                          const unsigned long long *nf, const uint8_t *edge, unsigned long long cost, float *F,
                          uint8_t *ok) {
    const size_t n = nsi * nsj * nsk;
    if (!n) return;
    k_node_features<<<(unsigned)n, 128, 0, A->ctx->stream>>>(A->dptr, A->dnorm, A->nrb, B->dptr, B->dnorm, B->nrb,
                                                            C->dptr, C->nrb, A->nrb, B->ncb, A->ncb, level, nsi, nsj,
                                                            nsk, A->bsr, nf, edge, cost, F, ok);
    A->ctx->note_launch();
    A->ctx->check_launch("scheduler features");
}

}  // namespace bsg

using namespace bsg;

// ---- scheduler object ----
bsg_sched_s::bsg_sched_s(bsg_ctx c) : ctx(c) {
    ctx_retain(c);
    BSG_CUDA(cudaMalloc(&params, kSchedParams * 4));
    BSG_CUDA(cudaMalloc(&m, kSchedParams * 4));
    BSG_CUDA(cudaMalloc(&v, kSchedParams * 4));
    init(1234);
}
bsg_sched_s::~bsg_sched_s() {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(params);
    cudaFree(m);
    cudaFree(v);
    ctx_release(ctx);
}

void bsg_sched_s::init(uint64_t seed) {
    // He-uniform weights, zero biases
    std::vector<float> h(kSchedParams, 0.f);
    std::mt19937_64 g(seed);
    auto fill = [&](int off, int fan_in, int count) {
        const float lim = std::sqrt(6.f / (float)fan_in);
        std::uniform_real_distribution<float> U(-lim, lim);
        for (int i = 0; i < count; ++i) h[off + i] = U(g);
    };
    fill(kW1, kSchedIn, kSchedH * kSchedIn);
    fill(kW2, kSchedH, kSchedH * kSchedH);
    fill(kW3, kSchedH, kSchedH);
    set(h.data());
    trained = false;
}

void bsg_sched_s::set(const float *host) {
    BSG_CUDA(cudaMemcpyAsync(params, host, kSchedParams * 4, cudaMemcpyHostToDevice, ctx->stream));
    BSG_CUDA(cudaMemsetAsync(m, 0, kSchedParams * 4, ctx->stream));
    BSG_CUDA(cudaMemsetAsync(v, 0, kSchedParams * 4, ctx->stream));
    BSG_CUDA(cudaStreamSynchronize(ctx->stream));
    adam_t = 0;
}

void bsg_sched_s::predict_dev(const float *dX, int n, float *dY) {
    if (n <= 0) return;
    k_mlp_fwd<<<n, kSchedH, 0, ctx->stream>>>(dX, nullptr, n, params, nullptr, nullptr, dY);
    ctx->note_launch();
    ctx->check_launch("scheduler forward");
}

float bsg_sched_s::fwd_bwd_dev(const float *dX, const int *didx, const float *dT, int n, float *dgrad) {
    cudaStream_t s = ctx->stream;
    DevBuf H1((size_t)n * kSchedH * 4, s), H2((size_t)n * kSchedH * 4, s), Y((size_t)n * 4, s),
        G((size_t)n * kSchedParams * 4, s), L(4, s);
    k_mlp_fwd<<<n, kSchedH, 0, s>>>(dX, didx, n, params, H1.as<float>(), H2.as<float>(), Y.as<float>());
    k_mlp_bwd<<<n, kSchedH, 0, s>>>(dX, didx, n, params, H1.as<float>(), H2.as<float>(), Y.as<float>(), dT,
                                     G.as<float>());
    k_mlp_gsum<<<(kSchedParams + 255) / 256, 256, 0, s>>>(G.as<float>(), n, dgrad);
    k_mlp_loss<<<1, 32, 0, s>>>(Y.as<float>(), dT, didx, n, L.as<float>());
    ctx->note_launch(4);
    ctx->check_launch("scheduler backward");
    float loss = 0.f;
    BSG_CUDA(cudaMemcpyAsync(&loss, L.p, 4, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    return loss;
}

float bsg_sched_s::train(const float *hX, const float *hT, int n, int epochs, int batch, float lr, uint64_t seed) {
    BSG_REQUIRE(n > 0 && epochs >= 0 && batch > 0, BSG_ERR_ARG, "scheduler training arguments");
    cudaStream_t s = ctx->stream;
    DevBuf dX((size_t)n * kSchedIn * 4, s), dT((size_t)n * 4, s), didx((size_t)n * 4, s), dgrad(kSchedParams * 4, s);
    BSG_CUDA(cudaMemcpyAsync(dX.p, hX, (size_t)n * kSchedIn * 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dT.p, hT, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::mt19937_64 g(seed);
    float last = 0.f;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(order.begin(), order.end(), g);
        BSG_CUDA(cudaMemcpyAsync(didx.p, order.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
        float tot = 0.f;
        int nb = 0;
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int nbat = std::min(batch, n - b0);
            tot += fwd_bwd_dev(dX.as<float>(), didx.as<int>() + b0, dT.as<float>(), nbat, dgrad.as<float>());
            ++nb;
            ++adam_t;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
            k_adam<<<(kSchedParams + 255) / 256, 256, 0, s>>>(params, dgrad.as<float>(), m, v, lr, b1, b2, 1e-8f, c1,
                                                              c2);
            ctx->note_launch();
        }
        last = tot / (float)std::max(nb, 1);
    }
    BSG_CUDA(cudaStreamSynchronize(s));
    trained = true;
    return last;
}

extern "C" bsg_status bsg_sched_create(bsg_ctx ctx, bsg_sched *out) {
    return guard([&] {
        BSG_REQUIRE(ctx && out, BSG_ERR_ARG, "NULL argument");
        *out = new bsg_sched_s(ctx);
    });
}

extern "C" bsg_status bsg_sched_destroy(bsg_sched sc) {
    return guard([&] { delete sc; });
}

extern "C" bsg_status bsg_sched_param_count(int *out) {
    return guard([&] {
        BSG_REQUIRE(out, BSG_ERR_ARG, "NULL argument");
        *out = kSchedParams;
    });
}

extern "C" bsg_status bsg_sched_set_params(bsg_sched sc, const float *params) {
    return guard([&] {
        BSG_REQUIRE(sc && params, BSG_ERR_ARG, "NULL argument");
        sc->set(params);
        sc->trained = true;
    });
}

extern "C" bsg_status bsg_sched_get_params(bsg_sched sc, float *params) {
    return guard([&] {
        BSG_REQUIRE(sc && params, BSG_ERR_ARG, "NULL argument");
        BSG_CUDA(cudaMemcpyAsync(params, sc->params, kSchedParams * 4, cudaMemcpyDeviceToHost, sc->ctx->stream));
        BSG_CUDA(cudaStreamSynchronize(sc->ctx->stream));
    });
}

extern "C" bsg_status bsg_sched_init(bsg_sched sc, uint64_t seed) {
    return guard([&] {
        BSG_REQUIRE(sc, BSG_ERR_ARG, "NULL argument");
        sc->init(seed);
    });
}

extern "C" bsg_status bsg_sched_predict(bsg_sched sc, const float *X, int n, float *Y) {
    return guard([&] {
        BSG_REQUIRE(sc && (n == 0 || (X && Y)) && n >= 0, BSG_ERR_ARG, "bad arguments");
        if (!n) return;
        cudaStream_t s = sc->ctx->stream;
        DevBuf dX((size_t)n * kSchedIn * 4, s), dY((size_t)n * 4, s);
        BSG_CUDA(cudaMemcpyAsync(dX.p, X, (size_t)n * kSchedIn * 4, cudaMemcpyHostToDevice, s));
        sc->predict_dev(dX.as<float>(), n, dY.as<float>());
        BSG_CUDA(cudaMemcpyAsync(Y, dY.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" bsg_status bsg_sched_loss_grad(bsg_sched sc, const float *X, const float *T, int n, float *loss,
                                          float *grad) {
    return guard([&] {
        BSG_REQUIRE(sc && X && T && n > 0, BSG_ERR_ARG, "bad arguments");
        cudaStream_t s = sc->ctx->stream;
        DevBuf dX((size_t)n * kSchedIn * 4, s), dT((size_t)n * 4, s), dg(kSchedParams * 4, s);
        BSG_CUDA(cudaMemcpyAsync(dX.p, X, (size_t)n * kSchedIn * 4, cudaMemcpyHostToDevice, s));
        BSG_CUDA(cudaMemcpyAsync(dT.p, T, (size_t)n * 4, cudaMemcpyHostToDevice, s));
        const float l = sc->fwd_bwd_dev(dX.as<float>(), nullptr, dT.as<float>(), n, dg.as<float>());
        if (loss) *loss = l;
        if (grad) {
            BSG_CUDA(cudaMemcpyAsync(grad, dg.p, kSchedParams * 4, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaStreamSynchronize(s));
        }
    });
}

extern "C" bsg_status bsg_sched_train(bsg_sched sc, const float *X, const float *T, int n, int epochs, int batch,
                                      float lr, uint64_t seed, float *final_loss) {
    return guard([&] {
        BSG_REQUIRE(sc && X && T, BSG_ERR_ARG, "NULL argument");
        const float l = sc->train(X, T, n, epochs, batch, lr, seed);
        if (final_loss) *final_loss = l;
    });
}
