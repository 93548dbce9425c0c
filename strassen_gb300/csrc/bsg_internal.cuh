// Internal declarations of the bsgpu library (GB300, sm_103a).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <atomic>
#include <cstring>
#include <memory>
#include <mutex>
#include <map>
#include <array>
#include <string>
#include <vector>

#include "../../include/bsgpu.h"

namespace bsg {

struct Error {
    int code;
    std::string msg;
};

void set_error(int code, const std::string &msg);
void clear_error();

#define BSG_CUDA(x)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess)                                                                        \
            throw ::bsg::Error{BSG_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_) + " at " + \
                                                 __FILE__ + ":" + std::to_string(__LINE__)};          \
    } while (0)

#define BSG_REQUIRE(cond, code, msg)                                  \
    do {                                                              \
        if (!(cond)) throw ::bsg::Error{(code), std::string(msg)};    \
    } while (0)

// Runs f, converting exceptions to a status + last-error message.
template <class F>
int guard(F &&f) {
    try {
        clear_error();
        f();
        return BSG_OK;
    } catch (const Error &e) {
        set_error(e.code, e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error(BSG_ERR_NOMEM, "host allocation failed");
        return BSG_ERR_NOMEM;
    } catch (const std::exception &e) {
        set_error(BSG_ERR_ARG, e.what());
        return BSG_ERR_ARG;
    }
}

inline size_t ceil_div(size_t a, size_t b) { return a == 0 ? 0 : 1 + (a - 1) / b; }  // utils.hpp:6-12

// Device memory owned by RAII (stream-ordered free).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t s = 0;
    DevBuf() = default;
    DevBuf(size_t n, cudaStream_t st);
    ~DevBuf();
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept { *this = std::move(o); }
    DevBuf &operator=(DevBuf &&o) noexcept {
        std::swap(p, o.p);
        std::swap(bytes, o.bytes);
        std::swap(s, o.s);
        return *this;
    }
    template <class T>
    T *as() const { return reinterpret_cast<T *>(p); }
};

}  // namespace bsg

// Reference counted: the caller's handle, every pool and every matrix created
// on the context hold one reference; the stream is released with the last.
struct bsg_ctx_s {
    std::atomic<int> refs{1};
    int device = 0;
    cudaStream_t stream = 0;
    bool own_stream = false;
    int sm_count = 0;
    uint64_t launches = 0;
    // timing of the tensor-core GEMM launches (CUDA events on `stream`)
    bool timing = false;
    double oz_ms = 0.0;
    uint64_t oz_launches = 0;
    double oz_useful_macs = 0.0;  // unpadded block-product multiply-adds (FP64-equivalent)
    uint64_t oz_stall[12] = {};    // pipeline stall counters of the GEMM kernel (SM cycles over CTAs)
    // timeout flag of the tensor-core GEMM launches: set on the device, read
    // once per public call (gemm_check) instead of after every launch
    int *d_gemm_err = nullptr;
    bool gemm_err_pending = false;
    // autotuned tile height (slots) and pipeline stages of the mixed-form
    // GEMM per (block rows, block k, block cols, digits)
    bool autotune = true;
    std::map<std::array<int, 4>, std::array<int, 2>> oz_tune;
    // SMs the tensor-core GEMM leaves free for a kernel that runs beside it
    // (the host-memory fetch of the 3c->2c upload path); 0 otherwise
    int oz_sm_reserve = 0;
    // second stream for host->device uploads that overlap compute on `stream`
    // (created on first use, released with the context)
    cudaStream_t copy_stream = 0;
    cudaStream_t upload_stream();
    // a highest-priority stream for a dependent kernel chain and a lowest-
    // priority one for work overlapped with it: with the chain's persistent
    // GEMM at the higher priority, blocks of the side work never hold it back
    // (both created on first use, released with the context)
    cudaStream_t chain_hi = 0, side_lo = 0;
    cudaStream_t chain_stream();
    cudaStream_t side_stream();
    void note_launch(uint64_t n = 1) { launches += n; }
    void check_launch(const char *what);
    int *gemm_err_flag();  // the device flag, cleared before the first launch of a call
    void gemm_check();     // synchronizes if launches are pending; throws BSG_ERR_TIMEOUT if one timed out
};

// BlockMemoryPool<double> on the device (blockallocator.h:8-25).
struct PoolImpl {
    bsg_ctx ctx;
    size_t block_elems;
    std::vector<double *> slabs;
    std::vector<double *> free_list;
    size_t total_blocks = 0;
    std::mutex mu;
    PoolImpl(bsg_ctx c, size_t be);
    ~PoolImpl();
    double *allocate(size_t n_elems);
    void deallocate(double *p);
    void grow();  // blockallocator.hpp:27-49
    void release_all();
};

struct bsg_pool_s {
    std::shared_ptr<PoolImpl> p;
};

struct bsg_bsm_s {
    bsg_ctx ctx;
    size_t nr, nc, bsr, bsc, nrb, ncb;
    double thresh;
    std::shared_ptr<PoolImpl> pool;
    std::vector<double *> hptr;  // host mirror of the block table (nullptr = absent)
    double **dptr = nullptr;     // device block table, block (r,c) at r + c*nrb
    double *dnorm = nullptr;     // device cached Frobenius norms
    size_t nblocks() const { return nrb * ncb; }
    size_t rows_of(size_t rb) const { return (rb + 1) * bsr <= nr ? bsr : nr - rb * bsr; }
    size_t cols_of(size_t cb) const { return (cb + 1) * bsc <= nc ? bsc : nc - cb * bsc; }
    void upload_table();       // hptr -> dptr (stream ordered)
    void release_block(size_t b);
    void ensure_block(size_t b);  // allocate if absent (content undefined)
};

namespace bsg {
void ctx_retain(bsg_ctx c);
void ctx_release(bsg_ctx c);
// kernels + launchers shared between translation units
void launch_block_norms(bsg_bsm m, const uint8_t *d_sel, cudaStream_t s);  // recompute norms where sel (all if null)
void launch_zero_blocks(bsg_bsm m, const uint8_t *d_sel, cudaStream_t s);
}  // namespace bsg

// ---- device helpers ----
// Frobenius norm of an rs x cs column-major block with leading dimension ld,
// computed by one full warp in the fixed order (the deterministic nrm2 the
// FP64 form shares with the oracle): lane l accumulates fma(x_i, x_i, s) over
// column-major element indices i = l, l+32, ...; then s_l += s_{l+o} for
// o = 16..1; lane 0 returns sqrt(s_0).
//
// The lane's chain s_l (the first half of the definition):
__device__ __forceinline__ double warp_norm_chain(const double *__restrict__ p, int rs, int cs, size_t ld) {
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    const int n = rs * cs;
    for (int i = lane; i < n; i += 32) {
        const int r = i % rs, c = i / rs;
        const double v = p[(size_t)r + (size_t)c * ld];
        acc = fma(v, v, acc);
    }
    return acc;
}

__device__ __forceinline__ double warp_block_norm(const double *__restrict__ p, int rs, int cs, size_t ld) {
    double acc = warp_norm_chain(p, rs, cs, ld);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, o));
    return sqrt(acc);
}

// The same norm from the 32 chains s[0..31] of one block, by one thread: the
// shuffle tree above as plain adds (level o adds s_{l+o} to s_l, l < o, o =
// 16 .. 1) and the square root.  Kernels that hold several blocks' chains in
// shared memory let lane q finish block q, so the FP64 pipe (the bound of the
// norm passes on this part) runs the tree and the square root once per
// kNormBlocks blocks instead of warp-wide for every block.
__device__ __forceinline__ double norm_from_chains(const double *s) {
    double t[16];
#pragma unroll
    for (int l = 0; l < 16; ++l) t[l] = __dadd_rn(s[l], s[l + 16]);
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1)
#pragma unroll
        for (int l = 0; l < o; ++l) t[l] = __dadd_rn(t[l], t[l + o]);
    return sqrt(t[0]);
}

// blocks per warp of the batched norm passes, and the per-warp table of their
// chains (33 doubles per block: lane q reading row q meets no bank conflict)
constexpr int kNormBlocks = 8;
using NormTable = double[kNormBlocks][33];
