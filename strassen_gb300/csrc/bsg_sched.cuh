// Learned Strassen scheduler (see bsg_sched.cu).
#pragma once
#include "bsg_internal.cuh"

namespace bsg {

constexpr int kSchedNodeIn = 25;  // node features
// options the network scores per node (one-hot after the node features):
// Strassen-Winograd of depth 1, 2, 3 at the node, or the node's product as
// one dense tile (every block product, unscreened)
constexpr int kSchedOpts = 4;
constexpr int kSchedIn = kSchedNodeIn + kSchedOpts;  // network input
constexpr int kSchedH = 64;   // hidden width (two hidden layers)

// Decision-tree byte of a node: 0 screened sparse recursion, 1 Strassen with
// the call's min_size_for_strassen, 2..4 Strassen of depth 1..3 at the node,
// 5 dense tile
constexpr uint8_t kNodeSparse = 0, kNodeStrassen = 1, kNodeDepth1 = 2, kNodeDense = 5;
constexpr int kSchedParams = kSchedH * kSchedIn + kSchedH + kSchedH * kSchedH + kSchedH + kSchedH + 1;

// features (kSchedNodeIn floats per node, row-major) and eligibility of every
// node of one level of the Strassen decision tree; nf / edge / cost from the
// dry run
void launch_node_features(bsg_bsm A, bsg_bsm B, bsg_bsm C, int level, size_t nsi, size_t nsj, size_t nsk,
                          const unsigned long long *nf, const uint8_t *edge, unsigned long long cost, float *F,
                          uint8_t *ok);

// network inputs X (n * kSchedOpts rows of kSchedIn: node i's features with
// option o one-hot at row i * kSchedOpts + o) from the node features F
void launch_option_rows(bsg_ctx ctx, const float *F, size_t n, float *X);

// tree[i]: the option with the smallest predicted log(t_option / t_sparse)
// among those valid at the level (depth t needs 2^(t-1) to divide the half
// side 2^level), kNodeDepth1 + o, where ok[i] and that prediction is < 0;
// kNodeSparse otherwise
void launch_sched_decide(bsg_ctx ctx, const uint8_t *ok, const float *y, size_t n, int level, uint8_t *tree);

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
