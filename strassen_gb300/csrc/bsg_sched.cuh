// Learned Strassen scheduler (see bsg_sched.cu).
#pragma once
#include "bsg_internal.cuh"

namespace bsg {

constexpr int kSchedIn = 25;  // node features
constexpr int kSchedH = 64;   // hidden width (two hidden layers)
constexpr int kSchedParams = kSchedH * kSchedIn + kSchedH + kSchedH * kSchedH + kSchedH + kSchedH + 1;

// features (kSchedIn floats per node, row-major) and eligibility of every node
// of one level of the Strassen decision tree; nf / edge / cost from the dry run
void launch_node_features(bsg_bsm A, bsg_bsm B, bsg_bsm C, int level, size_t nsi, size_t nsj, size_t nsk,
                          const unsigned long long *nf, const uint8_t *edge, unsigned long long cost, float *F,
                          uint8_t *ok);

// tree[i] = ok[i] && y[i] < 0
void launch_sched_decide(bsg_ctx ctx, const uint8_t *ok, const float *y, size_t n, uint8_t *tree);

}  // namespace bsg

// The MLP: parameters and Adam moments on the device.
struct bsg_sched_s {
    bsg_ctx ctx;
    float *params = nullptr, *m = nullptr, *v = nullptr;
    int adam_t = 0;
    bool trained = false;
    explicit bsg_sched_s(bsg_ctx c);
    ~bsg_sched_s();
    void init(uint64_t seed);
    void set(const float *host);
    void predict_dev(const float *dX, int n, float *dY);
    // forward + backward on samples idx[0..n) (or 0..n): loss, gradient into dgrad
    float fwd_bwd_dev(const float *dX, const int *didx, const float *dT, int n, float *dgrad);
    float train(const float *hX, const float *hT, int n, int epochs, int batch, float lr, uint64_t seed);
};
