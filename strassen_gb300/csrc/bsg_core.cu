// Context, device block pool and BlockSparseMatrix container operations.
//
// Reference: blockallocator.{h,hpp} (pool), blocksparsematrix.{h,hpp}
// (container).  The host keeps the authoritative block table (which blocks
// exist and where they live in the pool); a device copy of the table and the
// cached norms live on the context's stream.  Container kernels reproduce
// the reference's element operations exactly (see bsgpu.h).
#include <cmath>
#include <numeric>

#include "bsg_internal.cuh"

namespace bsg {

// the message of the last failed call on this host thread (the status code
// itself is what the call returns)
static thread_local std::string g_msg;

void set_error(int, const std::string &msg) { g_msg = msg; }
void clear_error() { g_msg.clear(); }

DevBuf::DevBuf(size_t n, cudaStream_t st) : bytes(n), s(st) {
    if (n) {
        cudaError_t e = cudaMallocAsync(&p, n, st);
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error{BSG_ERR_NOMEM, std::string("device allocation of ") + std::to_string(n) +
                                           " bytes failed: " + cudaGetErrorString(e)};
        }
    }
}
DevBuf::~DevBuf() {
    if (p) cudaFreeAsync(p, s);
}

void ctx_retain(bsg_ctx c) {
    if (c) c->refs.fetch_add(1);
}

void ctx_release(bsg_ctx c) {
    if (!c) return;
    if (c->refs.fetch_sub(1) == 1) {
        cudaStreamSynchronize(c->stream);
        if (c->d_gemm_err) cudaFree(c->d_gemm_err);
        for (cudaStream_t x : {c->copy_stream, c->chain_hi, c->side_lo})
            if (x) {
                cudaStreamSynchronize(x);
                cudaStreamDestroy(x);
            }
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
    }
}

}  // namespace bsg

using namespace bsg;

extern "C" const char *bsg_last_error(void) { return g_msg.c_str(); }
extern "C" int bsg_version(void) { return 10000; }

void bsg_ctx_s::check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error{BSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

cudaStream_t bsg_ctx_s::upload_stream() {
    if (!copy_stream) BSG_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
    return copy_stream;
}

cudaStream_t bsg_ctx_s::chain_stream() {
    if (!chain_hi) {
        int least = 0, greatest = 0;
        BSG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        BSG_CUDA(cudaStreamCreateWithPriority(&chain_hi, cudaStreamNonBlocking, greatest));
    }
    return chain_hi;
}

cudaStream_t bsg_ctx_s::side_stream() {
    if (!side_lo) {
        int least = 0, greatest = 0;
        BSG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        BSG_CUDA(cudaStreamCreateWithPriority(&side_lo, cudaStreamNonBlocking, least));
    }
    return side_lo;
}

int *bsg_ctx_s::gemm_err_flag() {
    if (!d_gemm_err) BSG_CUDA(cudaMalloc(&d_gemm_err, sizeof(int)));
    if (!gemm_err_pending) {
        BSG_CUDA(cudaMemsetAsync(d_gemm_err, 0, sizeof(int), stream));
        gemm_err_pending = true;
    }
    return d_gemm_err;
}

void bsg_ctx_s::gemm_check() {
    if (!gemm_err_pending) return;
    int h = 0;
    BSG_CUDA(cudaMemcpyAsync(&h, d_gemm_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    BSG_CUDA(cudaStreamSynchronize(stream));
    gemm_err_pending = false;
    BSG_REQUIRE(!h, BSG_ERR_TIMEOUT, "Ozaki GEMM: a pipeline wait timed out");
}

extern "C" bsg_status bsg_ctx_create(int device, void *cuda_stream, bsg_ctx *out) {
    return guard([&] {
        BSG_REQUIRE(out, BSG_ERR_ARG, "out is NULL");
        int ndev = 0;
        BSG_CUDA(cudaGetDeviceCount(&ndev));
        BSG_REQUIRE(device >= 0 && device < ndev, BSG_ERR_ARG, "no such CUDA device");
        BSG_CUDA(cudaSetDevice(device));
        auto *c = new bsg_ctx_s();
        c->device = device;
        if (cuda_stream) {
            c->stream = (cudaStream_t)cuda_stream;
        } else {
            BSG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
            c->own_stream = true;
        }
        BSG_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
        // keep freed stream-ordered allocations cached in this process (the
        // default pool would hand them back at every synchronization and map
        // them again on the next call); this process's own runtime state only
        cudaMemPool_t mp;
        if (cudaDeviceGetDefaultMemPool(&mp, device) == cudaSuccess) {
            uint64_t keep = 64ull << 30;
            cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        *out = c;
    });
}

extern "C" bsg_status bsg_ctx_destroy(bsg_ctx ctx) {
    return guard([&] {
        ctx_release(ctx);
    });
}

extern "C" bsg_status bsg_ctx_sync(bsg_ctx ctx) {
    return guard([&] {
        BSG_REQUIRE(ctx, BSG_ERR_ARG, "ctx is NULL");
        BSG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

extern "C" bsg_status bsg_ctx_launch_count(bsg_ctx ctx, uint64_t *out) {
    return guard([&] {
        BSG_REQUIRE(ctx && out, BSG_ERR_ARG, "NULL argument");
        *out = ctx->launches;
    });
}

extern "C" bsg_status bsg_ctx_set_timing(bsg_ctx ctx, int on) {
    return guard([&] {
        BSG_REQUIRE(ctx, BSG_ERR_ARG, "ctx is NULL");
        ctx->timing = on != 0;
        ctx->oz_ms = 0.0;
        ctx->oz_launches = 0;
        ctx->oz_useful_macs = 0.0;
        for (auto &v : ctx->oz_stall) v = 0;
    });
}

extern "C" bsg_status bsg_ctx_gemm_timing(bsg_ctx ctx, uint64_t *launches, double *ms, double *useful_macs) {
    return guard([&] {
        BSG_REQUIRE(ctx, BSG_ERR_ARG, "ctx is NULL");
        if (launches) *launches = ctx->oz_launches;
        if (ms) *ms = ctx->oz_ms;
        if (useful_macs) *useful_macs = ctx->oz_useful_macs;
    });
}

extern "C" bsg_status bsg_ctx_gemm_stalls(bsg_ctx ctx, uint64_t out[12]) {
    return guard([&] {
        BSG_REQUIRE(ctx && out, BSG_ERR_ARG, "NULL argument");
        for (int i = 0; i < 12; ++i) out[i] = ctx->oz_stall[i];
    });
}

// ---------------------------------------------------------------------------
// Block pool (blockallocator.hpp:7-62)
// ---------------------------------------------------------------------------

PoolImpl::PoolImpl(bsg_ctx c, size_t be) : ctx(c), block_elems(be) { ctx_retain(c); }

PoolImpl::~PoolImpl() {
    release_all();
    ctx_release(ctx);
}

void PoolImpl::grow() {
    // 16 MB first slab, doubling up to 1 GB per slab (blockallocator.hpp:27-49)
    const size_t min_bytes = 16ull << 20;
    const size_t shift = std::min<size_t>(6, slabs.size());
    const size_t bytes = min_bytes << shift;
    const size_t n = std::max<size_t>(1, bytes / (block_elems * sizeof(double)));
    double *p = nullptr;
    cudaError_t e = cudaMalloc(&p, n * block_elems * sizeof(double));
    if (e != cudaSuccess) throw Error{BSG_ERR_NOMEM, std::string("block pool growth failed: ") + cudaGetErrorString(e)};
    slabs.push_back(p);
    free_list.reserve(free_list.size() + n);
    for (size_t i = n; i-- > 0;) free_list.push_back(p + i * block_elems);
    total_blocks += n;
}

double *PoolImpl::allocate(size_t n_elems) {
    BSG_REQUIRE(n_elems <= block_elems, BSG_ERR_ARG, "block larger than the pool's block size");
    std::lock_guard<std::mutex> lk(mu);
    if (free_list.empty()) grow();
    double *p = free_list.back();
    free_list.pop_back();
    return p;
}

void PoolImpl::deallocate(double *p) {
    std::lock_guard<std::mutex> lk(mu);
    free_list.push_back(p);
}

void PoolImpl::release_all() {
    std::lock_guard<std::mutex> lk(mu);
    if (!slabs.empty() && ctx) cudaStreamSynchronize(ctx->stream);
    for (double *p : slabs) cudaFree(p);
    slabs.clear();
    free_list.clear();
    total_blocks = 0;
}

extern "C" bsg_status bsg_pool_create(bsg_ctx ctx, size_t block_elems, bsg_pool *out) {
    return guard([&] {
        BSG_REQUIRE(ctx && out, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(block_elems > 0, BSG_ERR_ARG, "block size must be positive");
        *out = new bsg_pool_s{std::make_shared<PoolImpl>(ctx, block_elems)};
    });
}

extern "C" bsg_status bsg_pool_release(bsg_pool pool) {
    return guard([&] { delete pool; });
}

extern "C" bsg_status bsg_pool_adjust_blocksize(bsg_pool pool, size_t block_elems) {
    return guard([&] {
        BSG_REQUIRE(pool, BSG_ERR_ARG, "pool is NULL");
        // only works if no blocks are allocated yet (blockallocator.hpp:51-56)
        BSG_REQUIRE(pool->p->slabs.empty(), BSG_ERR_PRECOND, "adjust_blocksize on a pool that holds memory");
        pool->p->block_elems = block_elems;
    });
}

extern "C" bsg_status bsg_pool_release_all_memory(bsg_pool pool) {
    return guard([&] {
        BSG_REQUIRE(pool, BSG_ERR_ARG, "pool is NULL");
        BSG_REQUIRE(pool->p->free_list.size() == pool->p->total_blocks, BSG_ERR_PRECOND,
                    "release_all_memory while matrices still hold blocks");
        pool->p->release_all();
    });
}

extern "C" bsg_status bsg_pool_stats(bsg_pool pool, size_t *total, size_t *nfree, size_t *bytes) {
    return guard([&] {
        BSG_REQUIRE(pool, BSG_ERR_ARG, "pool is NULL");
        std::lock_guard<std::mutex> lk(pool->p->mu);
        if (total) *total = pool->p->total_blocks;
        if (nfree) *nfree = pool->p->free_list.size();
        if (bytes) *bytes = pool->p->total_blocks * pool->p->block_elems * sizeof(double);
    });
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// One warp per block: norm of each input block of a dense column-major
// matrix, keep flag = !(norm < tpb) (blocksparsematrix.hpp:38,58-59).
__global__ void k_dense_block_norms(const double *__restrict__ in, size_t ld, size_t nr, size_t nc, size_t bsr,
                                    size_t bsc, size_t nrb, size_t nblk, double tpb, double *__restrict__ norm,
                                    uint8_t *__restrict__ keep) {
    const size_t b = (size_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (b >= nblk) return;
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    const double est = warp_block_norm(in + rb * bsr + cb * bsc * ld, rs, cs, ld);
    if ((threadIdx.x & 31) == 0) {
        norm[b] = est;
        keep[b] = !(est < tpb);
    }
}

// Copy kept blocks of a dense column-major matrix into their pool slots
// (block storage is column-major with ld = block rows).
__global__ void k_dense_to_blocks(const double *__restrict__ in, size_t ld, size_t nr, size_t nc, size_t bsr,
                                  size_t bsc, size_t nrb, double *const *__restrict__ dptr) {
    const size_t b = blockIdx.x;
    double *dst = dptr[b];
    if (!dst) return;
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    const double *src = in + rb * bsr + cb * bsc * ld;
    for (int i = threadIdx.x; i < rs * cs; i += blockDim.x) {
        const int r = i % rs, c = i / rs;
        dst[i] = src[(size_t)r + (size_t)c * ld];
    }
}

__global__ void k_blocks_to_dense(double *__restrict__ out, size_t ld, size_t nr, size_t nc, size_t bsr, size_t bsc,
                                  size_t nrb, double *const *__restrict__ dptr) {
    const size_t b = blockIdx.x;
    const double *src = dptr[b];
    if (!src) return;
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    double *dst = out + rb * bsr + cb * bsc * ld;
    for (int i = threadIdx.x; i < rs * cs; i += blockDim.x) {
        const int r = i % rs, c = i / rs;
        dst[(size_t)r + (size_t)c * ld] = src[i];
    }
}

// fill_with_values: every block = val, norm = sqrt(rows*cols)*val (matrix.hpp:27-33)
__global__ void k_fill_blocks(double *const *__restrict__ dptr, double *__restrict__ norm, size_t nr, size_t nc,
                              size_t bsr, size_t bsc, size_t nrb, double val) {
    const size_t b = blockIdx.x;
    double *dst = dptr[b];
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    for (int i = threadIdx.x; i < rs * cs; i += blockDim.x) dst[i] = val;
    if (threadIdx.x == 0) norm[b] = __dmul_rn(sqrt((double)((size_t)rs * (size_t)cs)), val);
}

// scale: present blocks *= s; every cached norm *= s*s (blocksparsematrix.hpp:71-77)
__global__ void k_scale_blocks(double *const *__restrict__ dptr, double *__restrict__ norm, size_t nr, size_t nc,
                               size_t bsr, size_t bsc, size_t nrb, double s) {
    const size_t b = blockIdx.x;
    double *dst = dptr[b];
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    if (dst)
        for (int i = threadIdx.x; i < rs * cs; i += blockDim.x) dst[i] = __dmul_rn(dst[i], s);
    if (threadIdx.x == 0) norm[b] = __dmul_rn(norm[b], __dmul_rn(s, s));
}

// y = fma(a, x, y) on blocks where op[b] == 1 (daxpy, matrix.hpp:107-117);
// op[b] == 2: y = x with norm copied (absent lhs in +=), op[b] == 3: y = x
// (absent lhs in -=).  Blocks with op[b] != 0 get their norm refreshed when
// refresh_norm is set (operator-= blocksparsematrix.hpp:217).
__global__ void k_axpy_blocks(double *const *__restrict__ y, double *__restrict__ ynorm,
                              double *const *__restrict__ x, const double *__restrict__ xnorm,
                              const uint8_t *__restrict__ op, size_t nr, size_t nc, size_t bsr, size_t bsc,
                              size_t nrb, double a, int refresh_norm) {
    const size_t b = blockIdx.x;
    const int o = op[b];
    if (!o) return;
    double *yd = y[b];
    const double *xd = x[b];
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    for (int i = threadIdx.x; i < rs * cs; i += blockDim.x) yd[i] = (o == 1) ? fma(a, xd[i], yd[i]) : xd[i];
    __syncthreads();
    if (refresh_norm) {
        if (threadIdx.x < 32) {
            double est = warp_block_norm(yd, rs, cs, rs);
            if (threadIdx.x == 0) ynorm[b] = est;
        }
    } else if (o == 2 && threadIdx.x == 0) {
        ynorm[b] = xnorm[b];
    }
}

// add_transpose (blocksparsematrix.hpp:224-248, matrix.hpp:179-187): for
// every lhs block (ib, jb) whose rhs partner (jb, ib) exists: a fresh lhs
// block starts at zero; lhs(r,c) += rhs(c,r); norm refreshed.
__global__ void k_add_transpose(double *const *__restrict__ d, double *__restrict__ dnorm,
                                double *const *__restrict__ r, const uint8_t *__restrict__ fresh, size_t nr,
                                size_t nc, size_t bsr, size_t bsc, size_t nrb, size_t r_nrb) {
    const size_t b = blockIdx.x;
    const size_t ib = b % nrb, jb = b / nrb;
    const double *rd = r[jb + ib * r_nrb];
    if (!rd) return;
    double *dd = d[b];
    const int rs = (int)(((ib + 1) * bsr <= nr) ? bsr : nr - ib * bsr);
    const int cs = (int)(((jb + 1) * bsc <= nc) ? bsc : nc - jb * bsc);
    const bool fr = fresh[b] != 0;
    for (int i = threadIdx.x; i < rs * cs; i += blockDim.x) {
        const int rr = i % rs, cc = i / rs;
        const double base = fr ? 0.0 : dd[i];
        dd[i] = __dadd_rn(base, rd[cc + rr * cs]);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double est = warp_block_norm(dd, rs, cs, rs);
        if (threadIdx.x == 0) dnorm[b] = est;
    }
}

__global__ void k_block_norms(double *const *__restrict__ dptr, double *__restrict__ norm,
                              const uint8_t *__restrict__ sel, size_t nr, size_t nc, size_t bsr, size_t bsc,
                              size_t nrb, size_t nblk) {
    const size_t b = (size_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (b >= nblk) return;
    if (sel && !sel[b]) return;
    const double *p = dptr[b];
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    double est = p ? warp_block_norm(p, rs, cs, rs) : 0.0;
    if ((threadIdx.x & 31) == 0) norm[b] = est;
}

__global__ void k_zero_blocks(double *const *__restrict__ dptr, double *__restrict__ norm,
                              const uint8_t *__restrict__ sel, size_t nblk) {
    const size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    if (sel && !sel[b]) return;
    norm[b] = 0.0;
}

// per-block dot with std::inner_product order (matrix.hpp:99-103)
__global__ void k_block_dots(double *const *__restrict__ a, const double *__restrict__ an,
                             double *const *__restrict__ bq, const double *__restrict__ bn, size_t nr, size_t nc,
                             size_t bsr, size_t bsc, size_t nrb, size_t nblk, double tpb, double *__restrict__ out,
                             uint8_t *__restrict__ used) {
    const size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const double *x = a[b], *y = bq[b];
    used[b] = 0;
    out[b] = 0.0;
    if (!x || !y) return;
    if (!(__dmul_rn(an[b], bn[b]) >= tpb)) return;
    const size_t rb = b % nrb, cb = b / nrb;
    const int rs = (int)(((rb + 1) * bsr <= nr) ? bsr : nr - rb * bsr);
    const int cs = (int)(((cb + 1) * bsc <= nc) ? bsc : nc - cb * bsc);
    double d = 0.0;
    for (int i = 0; i < rs * cs; ++i) d = __dadd_rn(d, __dmul_rn(x[i], y[i]));
    out[b] = d;
    used[b] = 1;
}

namespace bsg {
void launch_block_norms(bsg_bsm m, const uint8_t *d_sel, cudaStream_t s) {
    if (!m->nblocks()) return;
    const int wpb = 8;
    k_block_norms<<<(unsigned)ceil_div(m->nblocks(), wpb), wpb * 32, 0, s>>>(m->dptr, m->dnorm, d_sel, m->nr, m->nc,
                                                                             m->bsr, m->bsc, m->nrb, m->nblocks());
    m->ctx->note_launch();
    m->ctx->check_launch("block norms");
}
void launch_zero_blocks(bsg_bsm m, const uint8_t *d_sel, cudaStream_t s) {
    if (!m->nblocks()) return;
    k_zero_blocks<<<(unsigned)ceil_div(m->nblocks(), 256), 256, 0, s>>>(m->dptr, m->dnorm, d_sel, m->nblocks());
    m->ctx->note_launch();
    m->ctx->check_launch("zero norms");
}
}  // namespace bsg

// ---------------------------------------------------------------------------
// BlockSparseMatrix
// ---------------------------------------------------------------------------

void bsg_bsm_s::upload_table() {
    if (!nblocks()) return;
    BSG_CUDA(cudaMemcpyAsync(dptr, hptr.data(), nblocks() * sizeof(double *), cudaMemcpyHostToDevice, ctx->stream));
}

void bsg_bsm_s::release_block(size_t b) {
    if (hptr[b]) {
        pool->deallocate(hptr[b]);
        hptr[b] = nullptr;
    }
}

void bsg_bsm_s::ensure_block(size_t b) {
    if (!hptr[b]) hptr[b] = pool->allocate(bsr * bsc);
}

static unsigned tpb_for(size_t n) {
    size_t t = std::min<size_t>(256, ((n + 31) / 32) * 32);
    return (unsigned)std::max<size_t>(32, t);
}

extern "C" bsg_status bsg_bsm_create(bsg_ctx ctx, size_t nr, size_t nc, size_t bsr, size_t bsc, double thresh,
                                     bsg_pool pool, bsg_bsm *out) {
    return guard([&] {
        BSG_REQUIRE(ctx && out, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(bsr > 0 && bsc > 0, BSG_ERR_ARG, "block sizes must be positive");
        if (pool) {
            BSG_REQUIRE(pool->p->ctx == ctx, BSG_ERR_ARG, "pool belongs to another context");
            BSG_REQUIRE(pool->p->block_elems >= bsr * bsc, BSG_ERR_ARG, "pool block size smaller than bsr*bsc");
        }
        auto *m = new bsg_bsm_s();
        m->ctx = ctx;
        ctx_retain(ctx);
        m->nr = nr;
        m->nc = nc;
        m->bsr = bsr;
        m->bsc = bsc;
        m->nrb = ceil_div(nr, bsr);
        m->ncb = ceil_div(nc, bsc);
        m->thresh = thresh;
        m->pool = pool ? pool->p : std::make_shared<PoolImpl>(ctx, bsr * bsc);
        m->hptr.assign(m->nblocks(), nullptr);
        if (m->nblocks()) {
            cudaError_t e1 = cudaMalloc(&m->dptr, m->nblocks() * sizeof(double *));
            cudaError_t e2 = cudaMalloc(&m->dnorm, m->nblocks() * sizeof(double));
            if (e1 != cudaSuccess || e2 != cudaSuccess) {
                cudaFree(m->dptr);
                cudaFree(m->dnorm);
                m->pool.reset();
                ctx_release(ctx);
                delete m;
                throw Error{BSG_ERR_NOMEM, "matrix table allocation failed"};
            }
            cudaMemsetAsync(m->dptr, 0, m->nblocks() * sizeof(double *), ctx->stream);
            cudaMemsetAsync(m->dnorm, 0, m->nblocks() * sizeof(double), ctx->stream);
        }
        *out = m;
    });
}

extern "C" bsg_status bsg_bsm_destroy(bsg_bsm m) {
    return guard([&] {
        if (!m) return;
        bsg_ctx c = m->ctx;
        cudaStreamSynchronize(c->stream);
        for (size_t b = 0; b < m->nblocks(); ++b) m->release_block(b);
        cudaFree(m->dptr);
        cudaFree(m->dnorm);
        m->pool.reset();
        delete m;
        ctx_release(c);
    });
}

extern "C" bsg_status bsg_bsm_info(bsg_bsm m, size_t dims[6], double *thresh) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        if (dims) {
            dims[0] = m->nr;
            dims[1] = m->nc;
            dims[2] = m->bsr;
            dims[3] = m->bsc;
            dims[4] = m->nrb;
            dims[5] = m->ncb;
        }
        if (thresh) *thresh = m->thresh;
    });
}

extern "C" bsg_status bsg_bsm_pool(bsg_bsm m, bsg_pool *out) {
    return guard([&] {
        BSG_REQUIRE(m && out, BSG_ERR_ARG, "NULL argument");
        *out = new bsg_pool_s{m->pool};
    });
}

extern "C" bsg_status bsg_bsm_assign(bsg_bsm dst, bsg_bsm src) {
    return guard([&] {
        BSG_REQUIRE(dst && src, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(dst->ctx == src->ctx, BSG_ERR_ARG, "matrices belong to different contexts");
        if (dst == src) return;
        cudaStream_t s = dst->ctx->stream;
        // the copy shares the source's pool, as std::vector copy-assignment of
        // the pool-allocated blocks does
        if (dst->nblocks() != src->nblocks()) {
            for (size_t b = 0; b < dst->nblocks(); ++b) dst->release_block(b);
            cudaFree(dst->dptr);
            cudaFree(dst->dnorm);
            dst->dptr = nullptr;
            dst->dnorm = nullptr;
            dst->hptr.assign(src->nblocks(), nullptr);
            if (src->nblocks()) {
                BSG_CUDA(cudaMalloc(&dst->dptr, src->nblocks() * sizeof(double *)));
                BSG_CUDA(cudaMalloc(&dst->dnorm, src->nblocks() * sizeof(double)));
            }
        }
        if (dst->pool != src->pool) {
            for (size_t b = 0; b < dst->nblocks(); ++b) dst->release_block(b);
            dst->pool = src->pool;
        }
        dst->nr = src->nr;
        dst->nc = src->nc;
        dst->bsr = src->bsr;
        dst->bsc = src->bsc;
        dst->nrb = src->nrb;
        dst->ncb = src->ncb;
        dst->thresh = src->thresh;
        std::vector<uint8_t> op(dst->nblocks(), 0);
        for (size_t b = 0; b < dst->nblocks(); ++b) {
            if (src->hptr[b]) {
                dst->ensure_block(b);
                op[b] = 2;
            } else {
                dst->release_block(b);
            }
        }
        if (!dst->nblocks()) return;
        dst->upload_table();
        DevBuf dop(op.size(), s);
        BSG_CUDA(cudaMemcpyAsync(dop.p, op.data(), op.size(), cudaMemcpyHostToDevice, s));
        k_axpy_blocks<<<(unsigned)dst->nblocks(), tpb_for(dst->bsr * dst->bsc), 0, s>>>(
            dst->dptr, dst->dnorm, src->dptr, src->dnorm, dop.as<uint8_t>(), dst->nr, dst->nc, dst->bsr, dst->bsc,
            dst->nrb, 1.0, 0);
        dst->ctx->note_launch();
        dst->ctx->check_launch("assign");
        // norms of absent source blocks are copied too (0 for absent blocks)
        BSG_CUDA(cudaMemcpyAsync(dst->dnorm, src->dnorm, dst->nblocks() * sizeof(double), cudaMemcpyDeviceToDevice, s));
        BSG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" bsg_status bsg_bsm_copy_from_dense(bsg_bsm m, const double *in, int where) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        const size_t n = m->nr * m->nc, nb = m->nblocks();
        if (!nb) return;
        BSG_REQUIRE(in, BSG_ERR_ARG, "input is NULL");
        cudaStream_t s = m->ctx->stream;
        DevBuf staged;
        const double *din = in;
        if (where == BSG_HOST) {
            staged = DevBuf(n * sizeof(double), s);
            BSG_CUDA(cudaMemcpyAsync(staged.p, in, n * sizeof(double), cudaMemcpyHostToDevice, s));
            din = staged.as<double>();
        }
        DevBuf keep(nb, s);
        // thresh_per_block = thresh * (bsc*bsr) (blocksparsematrix.hpp:38)
        const double tpb = m->thresh * (double)(m->bsc * m->bsr);
        const int wpb = 8;
        k_dense_block_norms<<<(unsigned)ceil_div(nb, wpb), wpb * 32, 0, s>>>(din, m->nr, m->nr, m->nc, m->bsr, m->bsc,
                                                                          m->nrb, nb, tpb, m->dnorm, keep.as<uint8_t>());
        m->ctx->note_launch();
        m->ctx->check_launch("dense block norms");
        std::vector<uint8_t> hk(nb);
        BSG_CUDA(cudaMemcpyAsync(hk.data(), keep.p, nb, cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
        for (size_t b = 0; b < nb; ++b) {
            if (hk[b])
                m->ensure_block(b);
            else
                m->release_block(b);
        }
        m->upload_table();
        k_dense_to_blocks<<<(unsigned)nb, tpb_for(m->bsr * m->bsc), 0, s>>>(din, m->nr, m->nr, m->nc, m->bsr, m->bsc,
                                                                            m->nrb, m->dptr);
        m->ctx->note_launch();
        m->ctx->check_launch("dense to blocks");
        // dropped blocks get norm 0 (a fresh Mat, matrix.h:71)
        std::vector<uint8_t> drop(nb);
        for (size_t b = 0; b < nb; ++b) drop[b] = !hk[b];
        DevBuf dd(nb, s);
        BSG_CUDA(cudaMemcpyAsync(dd.p, drop.data(), nb, cudaMemcpyHostToDevice, s));
        launch_zero_blocks(m, dd.as<uint8_t>(), s);
        BSG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" bsg_status bsg_bsm_fill(bsg_bsm m, double val) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        if (!m->nblocks()) return;
        for (size_t b = 0; b < m->nblocks(); ++b) m->ensure_block(b);
        m->upload_table();
        k_fill_blocks<<<(unsigned)m->nblocks(), tpb_for(m->bsr * m->bsc), 0, m->ctx->stream>>>(
            m->dptr, m->dnorm, m->nr, m->nc, m->bsr, m->bsc, m->nrb, val);
        m->ctx->note_launch();
        m->ctx->check_launch("fill");
    });
}

extern "C" bsg_status bsg_bsm_zero(bsg_bsm m) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        if (!m->nblocks()) return;
        BSG_CUDA(cudaStreamSynchronize(m->ctx->stream));
        for (size_t b = 0; b < m->nblocks(); ++b) m->release_block(b);
        m->upload_table();
        BSG_CUDA(cudaMemsetAsync(m->dnorm, 0, m->nblocks() * sizeof(double), m->ctx->stream));
    });
}

extern "C" bsg_status bsg_bsm_scale(bsg_bsm m, double sc) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        if (!m->nblocks()) return;
        k_scale_blocks<<<(unsigned)m->nblocks(), tpb_for(m->bsr * m->bsc), 0, m->ctx->stream>>>(
            m->dptr, m->dnorm, m->nr, m->nc, m->bsr, m->bsc, m->nrb, sc);
        m->ctx->note_launch();
        m->ctx->check_launch("scale");
    });
}

static void add_impl(bsg_bsm m, bsg_bsm r, double a, bool refresh) {
    BSG_REQUIRE(m && r, BSG_ERR_ARG, "NULL argument");
    BSG_REQUIRE(m->ctx == r->ctx, BSG_ERR_ARG, "matrices belong to different contexts");
    BSG_REQUIRE(m->nrb == r->nrb && m->ncb == r->ncb && m->nr == r->nr && m->nc == r->nc, BSG_ERR_ARG,
                "operator+=/-=: dimensions do not match");
    const size_t nb = m->nblocks();
    if (!nb) return;
    std::vector<uint8_t> op(nb, 0);
    for (size_t b = 0; b < nb; ++b) {
        if (!r->hptr[b]) continue;
        if (m->hptr[b]) {
            op[b] = 1;
        } else {
            m->ensure_block(b);
            op[b] = refresh ? 3 : 2;
        }
    }
    cudaStream_t s = m->ctx->stream;
    m->upload_table();
    DevBuf dop(nb, s);
    BSG_CUDA(cudaMemcpyAsync(dop.p, op.data(), nb, cudaMemcpyHostToDevice, s));
    k_axpy_blocks<<<(unsigned)nb, tpb_for(m->bsr * m->bsc), 0, s>>>(m->dptr, m->dnorm, r->dptr, r->dnorm,
                                                                     dop.as<uint8_t>(), m->nr, m->nc, m->bsr, m->bsc,
                                                                     m->nrb, a, refresh ? 1 : 0);
    m->ctx->note_launch();
    m->ctx->check_launch("axpy blocks");
    BSG_CUDA(cudaStreamSynchronize(s));
}

extern "C" bsg_status bsg_bsm_add(bsg_bsm m, bsg_bsm rhs) {
    return guard([&] { add_impl(m, rhs, 1.0, false); });
}
extern "C" bsg_status bsg_bsm_sub(bsg_bsm m, bsg_bsm rhs) {
    return guard([&] { add_impl(m, rhs, -1.0, true); });
}

extern "C" bsg_status bsg_bsm_add_transpose(bsg_bsm m, bsg_bsm r) {
    return guard([&] {
        BSG_REQUIRE(m && r, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(m->ctx == r->ctx, BSG_ERR_ARG, "matrices belong to different contexts");
        BSG_REQUIRE(m->nrb == r->ncb && m->ncb == r->nrb && m->nr == r->nc && m->nc == r->nr && m->bsr == r->bsc &&
                        m->bsc == r->bsr,
                    BSG_ERR_ARG, "add_transpose: dimensions do not match");
        BSG_REQUIRE(m != r, BSG_ERR_ARG, "add_transpose with itself is not supported");
        const size_t nb = m->nblocks();
        if (!nb) return;
        std::vector<uint8_t> fresh(nb, 0);
        for (size_t ib = 0; ib < m->nrb; ++ib)
            for (size_t jb = 0; jb < m->ncb; ++jb) {
                const size_t b = ib + jb * m->nrb;
                if (!r->hptr[jb + ib * r->nrb]) continue;
                if (!m->hptr[b]) {
                    m->ensure_block(b);
                    fresh[b] = 1;
                }
            }
        cudaStream_t s = m->ctx->stream;
        m->upload_table();
        DevBuf df(nb, s);
        BSG_CUDA(cudaMemcpyAsync(df.p, fresh.data(), nb, cudaMemcpyHostToDevice, s));
        k_add_transpose<<<(unsigned)nb, tpb_for(m->bsr * m->bsc), 0, s>>>(m->dptr, m->dnorm, r->dptr,
                                                                          df.as<uint8_t>(), m->nr, m->nc, m->bsr,
                                                                          m->bsc, m->nrb, r->nrb);
        m->ctx->note_launch();
        m->ctx->check_launch("add_transpose");
        BSG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" bsg_status bsg_bsm_calc_norms(bsg_bsm m) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        launch_block_norms(m, nullptr, m->ctx->stream);
    });
}

extern "C" bsg_status bsg_bsm_recompress(bsg_bsm m) {
    return guard([&] {
        BSG_REQUIRE(m, BSG_ERR_ARG, "matrix is NULL");
        const size_t nb = m->nblocks();
        if (!nb) return;
        std::vector<double> nrm(nb);
        BSG_CUDA(cudaMemcpyAsync(nrm.data(), m->dnorm, nb * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
        BSG_CUDA(cudaStreamSynchronize(m->ctx->stream));
        const double tpb = m->thresh * (double)(m->bsc * m->bsr);
        std::vector<uint8_t> drop(nb, 0);
        for (size_t b = 0; b < nb; ++b)
            if (nrm[b] < tpb) {
                m->release_block(b);
                drop[b] = 1;
            }
        m->upload_table();
        DevBuf dd(nb, m->ctx->stream);
        BSG_CUDA(cudaMemcpyAsync(dd.p, drop.data(), nb, cudaMemcpyHostToDevice, m->ctx->stream));
        launch_zero_blocks(m, dd.as<uint8_t>(), m->ctx->stream);
        BSG_CUDA(cudaStreamSynchronize(m->ctx->stream));
    });
}

extern "C" bsg_status bsg_bsm_frobenius_norm(bsg_bsm m, double *out) {
    return guard([&] {
        BSG_REQUIRE(m && out, BSG_ERR_ARG, "NULL argument");
        std::vector<double> nrm(m->nblocks());
        if (!nrm.empty()) {
            BSG_CUDA(cudaMemcpyAsync(nrm.data(), m->dnorm, nrm.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                     m->ctx->stream));
            BSG_CUDA(cudaStreamSynchronize(m->ctx->stream));
        }
        // std::accumulate(norm*norm + acc) in block order (blocksparsematrix.hpp:256-261)
        volatile double acc = 0.0;
        for (double v : nrm) {
            volatile double sq = v * v;
            acc = sq + acc;
        }
        *out = std::sqrt((double)acc);
    });
}

extern "C" bsg_status bsg_bsm_no_of_alloc_blocks(bsg_bsm m, size_t *out) {
    return guard([&] {
        BSG_REQUIRE(m && out, BSG_ERR_ARG, "NULL argument");
        size_t n = 0;
        for (auto *p : m->hptr) n += p != nullptr;
        *out = n;
    });
}

extern "C" bsg_status bsg_bsm_calc_alloc_dim(bsg_bsm m, size_t *out) {
    return guard([&] {
        BSG_REQUIRE(m && out, BSG_ERR_ARG, "NULL argument");
        size_t n = 0;
        for (size_t b = 0; b < m->nblocks(); ++b)
            if (m->hptr[b]) n += m->rows_of(b % m->nrb) * m->cols_of(b / m->nrb);
        *out = n;
    });
}

extern "C" bsg_status bsg_bsm_to_dense(bsg_bsm m, double *out, int where) {
    return guard([&] {
        BSG_REQUIRE(m && out, BSG_ERR_ARG, "NULL argument");
        const size_t n = m->nr * m->nc;
        if (!n) return;
        cudaStream_t s = m->ctx->stream;
        DevBuf staged;
        double *dout = out;
        if (where == BSG_HOST) {
            staged = DevBuf(n * sizeof(double), s);
            dout = staged.as<double>();
        }
        BSG_CUDA(cudaMemsetAsync(dout, 0, n * sizeof(double), s));
        k_blocks_to_dense<<<(unsigned)m->nblocks(), tpb_for(m->bsr * m->bsc), 0, s>>>(dout, m->nr, m->nr, m->nc,
                                                                                      m->bsr, m->bsc, m->nrb, m->dptr);
        m->ctx->note_launch();
        m->ctx->check_launch("blocks to dense");
        if (where == BSG_HOST) BSG_CUDA(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" bsg_status bsg_bsm_get_mask(bsg_bsm m, uint8_t *mask) {
    return guard([&] {
        BSG_REQUIRE(m && mask, BSG_ERR_ARG, "NULL argument");
        for (size_t b = 0; b < m->nblocks(); ++b) mask[b] = m->hptr[b] != nullptr;
    });
}

extern "C" bsg_status bsg_bsm_get_norms(bsg_bsm m, double *norms) {
    return guard([&] {
        BSG_REQUIRE(m && norms, BSG_ERR_ARG, "NULL argument");
        if (!m->nblocks()) return;
        BSG_CUDA(cudaMemcpyAsync(norms, m->dnorm, m->nblocks() * sizeof(double), cudaMemcpyDeviceToHost,
                                 m->ctx->stream));
        BSG_CUDA(cudaStreamSynchronize(m->ctx->stream));
    });
}

extern "C" bsg_status bsg_dot(bsg_bsm a, bsg_bsm b, double thresh, double *out) {
    return guard([&] {
        BSG_REQUIRE(a && b && out, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(a->nrb == b->nrb && a->ncb == b->ncb && a->nr == b->nr && a->nc == b->nc, BSG_ERR_ARG,
                    "dot: dimensions do not match");
        const size_t nb = a->nblocks();
        double acc = 0.0;
        if (nb) {
            cudaStream_t s = a->ctx->stream;
            DevBuf d(nb * sizeof(double), s), u(nb, s);
            const double tpb = thresh * (double)(a->bsr * a->bsc);
            k_block_dots<<<(unsigned)ceil_div(nb, 128), 128, 0, s>>>(a->dptr, a->dnorm, b->dptr, b->dnorm, a->nr,
                                                                     a->nc, a->bsr, a->bsc, a->nrb, nb, tpb,
                                                                     d.as<double>(), u.as<uint8_t>());
            a->ctx->note_launch();
            a->ctx->check_launch("block dots");
            std::vector<double> hd(nb);
            std::vector<uint8_t> hu(nb);
            BSG_CUDA(cudaMemcpyAsync(hd.data(), d.p, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(hu.data(), u.p, nb, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaStreamSynchronize(s));
            // the reference's loop order: ijb -> (ib = ijb / ncb, jb = ijb % ncb)
            for (size_t ijb = 0; ijb < nb; ++ijb) {
                const size_t ib = ijb / a->ncb, jb = ijb % a->ncb, bi = ib + jb * a->nrb;
                if (hu[bi]) {
                    volatile double t = acc + hd[bi];
                    acc = t;
                }
            }
        }
        *out = acc;
    });
}
