// Screened block-sparse GEMM, FP64 form (blocksparsematrix.hpp:293-414) and the
// 3-index tensor products built on it (blocksparse3d_tensor.h:11-24).
//
// Pipeline per call: beta handling on C -> count kernel (one thread per
// output block counts surviving (slice, k) block triples) -> host allocates
// the C blocks that become non-empty and lays out the pair list (prefix sum of
// the counts) -> fill kernel writes each output block's pairs in
// accumulation order -> one grouped GEMM launch over all output blocks.
#include <algorithm>

#include "bsg_gemm64.cuh"
#include "bsg_ozaki.cuh"

namespace bsg {

constexpr int kEPT = 16;  // output elements per thread in the FP64 block kernel

// For every output element: t = 0; t = fma(opA(i,l), opB(l,j), t) over l;
// then C = alpha*t (first pair of a fresh block) or C = alpha*t + C.
__global__ void __launch_bounds__(1024) k_gemm64(const GemmItem *__restrict__ items,
                                                 const GemmPair *__restrict__ pairs, int tA, int tB, double alpha) {
    const GemmItem it = items[blockIdx.x];
    const int rows = it.rows, n = it.rows * it.cols;
    double acc[kEPT];
    int ii[kEPT], jj[kEPT];
    const int nt = blockDim.x;
#pragma unroll
    for (int s = 0; s < kEPT; ++s) {
        const int e = threadIdx.x + s * nt;
        ii[s] = e < n ? e % rows : 0;
        jj[s] = e < n ? e / rows : 0;
        acc[s] = (e < n && !it.fresh) ? it.c[e] : 0.0;
    }
    bool first = it.fresh != 0;
    for (uint32_t p = it.p0; p < it.p1; ++p) {
        const GemmPair pr = pairs[p];
        double t[kEPT];
#pragma unroll
        for (int s = 0; s < kEPT; ++s) t[s] = 0.0;
        for (int l = 0; l < pr.k; ++l) {
#pragma unroll
            for (int s = 0; s < kEPT; ++s) {
                if (threadIdx.x + s * nt < n) {
                    const double a = tA ? __ldg(pr.a + l + (size_t)ii[s] * pr.lda) : __ldg(pr.a + ii[s] + (size_t)l * pr.lda);
                    const double b = tB ? __ldg(pr.b + jj[s] + (size_t)l * pr.ldb) : __ldg(pr.b + l + (size_t)jj[s] * pr.ldb);
                    t[s] = fma(a, b, t[s]);
                }
            }
        }
#pragma unroll
        for (int s = 0; s < kEPT; ++s) acc[s] = first ? __dmul_rn(alpha, t[s]) : __dadd_rn(__dmul_rn(alpha, t[s]), acc[s]);
        first = false;
    }
#pragma unroll
    for (int s = 0; s < kEPT; ++s) {
        const int e = threadIdx.x + s * nt;
        if (e < n) it.c[e] = acc[s];
    }
    if (it.fresh && it.c_norm && threadIdx.x == 0) *it.c_norm = 0.0;
}

void launch_gemm64(bsg_ctx ctx, const GemmItem *d_items, size_t n_items, const GemmPair *d_pairs, int tA, int tB,
                   double alpha, int max_rows, int max_cols, cudaStream_t s) {
    if (!n_items) return;
    const size_t elems = (size_t)max_rows * (size_t)max_cols;
    BSG_REQUIRE(elems <= (size_t)kEPT * 1024, BSG_ERR_UNSUPPORTED, "FP64 block kernel supports blocks up to 16384 elements");
    const unsigned nt = (unsigned)std::max<size_t>(32, ((ceil_div(elems, kEPT) + 31) / 32) * 32);
    for (size_t off = 0; off < n_items; off += 2147483647ull) {
        const unsigned g = (unsigned)std::min<size_t>(n_items - off, 2147483647ull);
        k_gemm64<<<g, nt, 0, s>>>(d_items + off, d_pairs, tA, tB, alpha);
        ctx->note_launch();
        ctx->check_launch("gemm64");
    }
}

using Geom = ScreenGeom;

__device__ __forceinline__ bool survives(const SliceOps &s, const Geom &g, size_t ib, size_t jb, size_t kb,
                                         size_t *ai_out, size_t *bi_out) {
    const size_t ai = g.tA ? kb + ib * s.a_nrb : ib + kb * s.a_nrb;
    const size_t bi = g.tB ? jb + kb * s.b_nrb : kb + jb * s.b_nrb;
    *ai_out = ai;
    *bi_out = bi;
    if (!s.a[ai] || !s.b[bi]) return false;
    return __dmul_rn(s.an[ai], s.bn[bi]) >= g.tpb;
}

// one thread per output block (c, ib, jb): number of surviving triples
__global__ void k_count(const SliceOps *__restrict__ sl, const uint32_t *__restrict__ lo,
                        const uint32_t *__restrict__ hi, Geom g, size_t n_c, uint32_t *__restrict__ count) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = g.nib * g.njb;
    if (x >= per * n_c) return;
    const size_t c = x / per, r = x % per, ib = r % g.nib, jb = r / g.nib;
    uint32_t n = 0;
    for (uint32_t l = lo[c]; l < hi[c]; ++l) {
        const SliceOps s = sl[l];
        for (size_t kb = 0; kb < g.nkb; ++kb) {
            size_t ai, bi;
            n += survives(s, g, ib, jb, kb, &ai, &bi);
        }
    }
    count[x] = n;
}

// writes the pairs of every output block at its offset, in (slice, kb) order
__global__ void k_fill(const SliceOps *__restrict__ sl, const uint32_t *__restrict__ lo,
                       const uint32_t *__restrict__ hi, Geom g, size_t n_c, const uint32_t *__restrict__ offset,
                       GemmPair *__restrict__ pairs) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = g.nib * g.njb;
    if (x >= per * n_c) return;
    const size_t c = x / per, r = x % per, ib = r % g.nib, jb = r / g.nib;
    uint32_t o = offset[x];
    const int rows_i = (int)(((ib + 1) * g.ibs <= g.ni) ? g.ibs : g.ni - ib * g.ibs);
    const int cols_j = (int)(((jb + 1) * g.jbs <= g.nj) ? g.jbs : g.nj - jb * g.jbs);
    for (uint32_t l = lo[c]; l < hi[c]; ++l) {
        const SliceOps s = sl[l];
        for (size_t kb = 0; kb < g.nkb; ++kb) {
            size_t ai, bi;
            if (!survives(s, g, ib, jb, kb, &ai, &bi)) continue;
            const int k = (int)(((kb + 1) * g.kbs <= g.nk) ? g.kbs : g.nk - kb * g.kbs);
            GemmPair p;
            p.a = s.a[ai];
            p.b = s.b[bi];
            p.k = k;
            p.lda = g.tA ? k : rows_i;
            p.ldb = g.tB ? cols_j : k;
            pairs[o++] = p;
        }
    }
}

uint64_t screened_product(bsg_ctx ctx, const std::vector<bsg_bsm> &Cs, const std::vector<bsg_bsm> &As, int tA,
                          const std::vector<bsg_bsm> &Bs, int tB, const std::vector<std::pair<size_t, size_t>> &ranges,
                          double thresh, double alpha, double beta, int form, int n_digits) {
    BSG_REQUIRE(!Cs.empty() && As.size() == Bs.size() && ranges.size() == Cs.size(), BSG_ERR_ARG, "bad operand lists");
    const bsg_bsm A0 = As[0], B0 = Bs[0], C0 = Cs[0];
    for (auto *m : As) BSG_REQUIRE(m && m->ctx == ctx, BSG_ERR_ARG, "operand on another context");
    for (auto *m : Bs) BSG_REQUIRE(m && m->ctx == ctx, BSG_ERR_ARG, "operand on another context");
    for (auto *m : Cs) BSG_REQUIRE(m && m->ctx == ctx, BSG_ERR_ARG, "output on another context");
    Geom g;
    g.tA = tA;
    g.tB = tB;
    g.ni = tA ? A0->nc : A0->nr;
    g.nj = tB ? B0->nr : B0->nc;
    const size_t nk1 = tA ? A0->nr : A0->nc, nk2 = tB ? B0->nc : B0->nr;
    BSG_REQUIRE(nk1 == nk2, BSG_ERR_ARG, "matmult: inner dimensions do not match");
    g.nk = nk1;
    g.ibs = tA ? A0->bsc : A0->bsr;
    g.jbs = tB ? B0->bsr : B0->bsc;
    const size_t kbs1 = tA ? A0->bsr : A0->bsc, kbs2 = tB ? B0->bsc : B0->bsr;
    BSG_REQUIRE(kbs1 == kbs2, BSG_ERR_ARG, "matmult: inner block sizes do not match");
    g.kbs = kbs1;
    for (auto *m : As)
        BSG_REQUIRE(m->nr == A0->nr && m->nc == A0->nc && m->bsr == A0->bsr && m->bsc == A0->bsc, BSG_ERR_ARG,
                    "A slices differ in shape");
    for (auto *m : Bs)
        BSG_REQUIRE(m->nr == B0->nr && m->nc == B0->nc && m->bsr == B0->bsr && m->bsc == B0->bsc, BSG_ERR_ARG,
                    "B slices differ in shape");
    for (auto *m : Cs)
        BSG_REQUIRE(m->bsr == g.ibs && m->bsc == g.jbs && m->nr == g.ni && m->nc == g.nj, BSG_ERR_ARG,
                    "matmult: output dimensions or block sizes do not match");
    g.nib = ceil_div(g.ni, g.ibs);
    g.njb = ceil_div(g.nj, g.jbs);
    g.nkb = ceil_div(g.nk, g.kbs);
    // thresh_per_block = thresh * (bs_i*bs_j*bs_k) (blocksparsematrix.hpp:350)
    g.tpb = thresh * (double)(g.ibs * g.jbs * g.kbs);
    BSG_REQUIRE(form == BSG_FORM_FP64 || form == BSG_FORM_OZAKI, BSG_ERR_ARG, "unknown arithmetic form");

    cudaStream_t s = ctx->stream;
    // beta handling (blocksparsematrix.hpp:299-305)
    for (auto *C : Cs) {
        if (beta == 1.0) {
        } else if (beta == 0.0) {
            BSG_REQUIRE(bsg_bsm_zero(C) == BSG_OK, BSG_ERR_CUDA, bsg_last_error());
        } else {
            BSG_REQUIRE(bsg_bsm_scale(C, beta) == BSG_OK, BSG_ERR_CUDA, bsg_last_error());
        }
    }
    const size_t n_c = Cs.size(), per = g.nib * g.njb, n_out = per * n_c;
    if (!n_out || !g.nkb) return 0;

    std::vector<SliceOps> hs(As.size());
    for (size_t l = 0; l < As.size(); ++l)
        hs[l] = SliceOps{As[l]->dptr, As[l]->dnorm, As[l]->nrb, Bs[l]->dptr, Bs[l]->dnorm, Bs[l]->nrb};
    std::vector<uint32_t> hlo(n_c), hhi(n_c);
    for (size_t c = 0; c < n_c; ++c) {
        hlo[c] = (uint32_t)ranges[c].first;
        hhi[c] = (uint32_t)ranges[c].second;
    }
    DevBuf dsl(hs.size() * sizeof(SliceOps), s), dlo(n_c * 4, s), dhi(n_c * 4, s), dcount(n_out * 4, s);
    BSG_CUDA(cudaMemcpyAsync(dsl.p, hs.data(), hs.size() * sizeof(SliceOps), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dlo.p, hlo.data(), n_c * 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dhi.p, hhi.data(), n_c * 4, cudaMemcpyHostToDevice, s));
    k_count<<<(unsigned)ceil_div(n_out, 128), 128, 0, s>>>(dsl.as<SliceOps>(), dlo.as<uint32_t>(), dhi.as<uint32_t>(),
                                                            g, n_c, dcount.as<uint32_t>());
    ctx->note_launch();
    ctx->check_launch("pair count");
    std::vector<uint32_t> cnt(n_out);
    BSG_CUDA(cudaMemcpyAsync(cnt.data(), dcount.p, n_out * 4, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));

    // exclusive scan of the counts = pair-list layout; allocate C blocks that
    // become non-empty (fresh: first pair assigns, norm 0)
    std::vector<uint32_t> off(n_out);
    uint64_t total = 0;
    std::vector<GemmItem> items;
    int max_r = 0, max_c = 0;
    std::vector<bool> touched(Cs.size(), false);
    std::vector<uint32_t> item_ib, item_jb;
    for (size_t x = 0; x < n_out; ++x) {
        off[x] = (uint32_t)total;
        if (!cnt[x]) continue;
        BSG_REQUIRE(total + cnt[x] < 0xffffffffull, BSG_ERR_UNSUPPORTED, "more than 2^32 block products in one call");
        const size_t c = x / per, r = x % per, ib = r % g.nib, jb = r / g.nib;
        bsg_bsm C = Cs[c];
        const size_t cbk = ib + jb * C->nrb;
        GemmItem it;
        it.fresh = C->hptr[cbk] == nullptr;
        C->ensure_block(cbk);
        touched[c] = true;
        it.c = C->hptr[cbk];
        it.c_norm = C->dnorm + cbk;
        it.rows = (int)C->rows_of(ib);
        it.cols = (int)C->cols_of(jb);
        it.p0 = (uint32_t)total;
        it.p1 = (uint32_t)(total + cnt[x]);
        max_r = std::max(max_r, it.rows);
        max_c = std::max(max_c, it.cols);
        items.push_back(it);
        item_ib.push_back((uint32_t)ib);
        item_jb.push_back((uint32_t)jb);
        total += cnt[x];
    }
    for (size_t c = 0; c < Cs.size(); ++c)
        if (touched[c]) Cs[c]->upload_table();
    if (!total) return 0;
    if (form == BSG_FORM_OZAKI) {
        BSG_REQUIRE(As.size() == 1 && Cs.size() == 1, BSG_ERR_UNSUPPORTED, "Ozaki form: single products only");
        ozaki_screened(ctx, C0, A0, B0, g, items, item_ib, item_jb, alpha, n_digits, s);
        BSG_CUDA(cudaStreamSynchronize(s));
        return total;
    }
    DevBuf doff(n_out * 4, s), dpairs(total * sizeof(GemmPair), s), ditems(items.size() * sizeof(GemmItem), s);
    BSG_CUDA(cudaMemcpyAsync(doff.p, off.data(), n_out * 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(ditems.p, items.data(), items.size() * sizeof(GemmItem), cudaMemcpyHostToDevice, s));
    k_fill<<<(unsigned)ceil_div(n_out, 128), 128, 0, s>>>(dsl.as<SliceOps>(), dlo.as<uint32_t>(), dhi.as<uint32_t>(), g,
                                                           n_c, doff.as<uint32_t>(), dpairs.as<GemmPair>());
    ctx->note_launch();
    ctx->check_launch("pair fill");
    launch_gemm64(ctx, ditems.as<GemmItem>(), items.size(), dpairs.as<GemmPair>(), tA, tB, alpha, max_r, max_c, s);
    BSG_CUDA(cudaStreamSynchronize(s));
    return total;
}

ScreenItems screen_items(bsg_ctx ctx, bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh, double beta) {
    BSG_REQUIRE(C && A && B, BSG_ERR_ARG, "NULL matrix");
    BSG_REQUIRE(A->ctx == ctx && B->ctx == ctx && C->ctx == ctx, BSG_ERR_ARG, "operand on another context");
    ScreenItems R;
    ScreenGeom &g = R.g;
    g.tA = tA;
    g.tB = tB;
    g.ni = tA ? A->nc : A->nr;
    g.nj = tB ? B->nr : B->nc;
    const size_t nk1 = tA ? A->nr : A->nc, nk2 = tB ? B->nc : B->nr;
    BSG_REQUIRE(nk1 == nk2, BSG_ERR_ARG, "matmult: inner dimensions do not match");
    g.nk = nk1;
    g.ibs = tA ? A->bsc : A->bsr;
    g.jbs = tB ? B->bsr : B->bsc;
    const size_t kbs1 = tA ? A->bsr : A->bsc, kbs2 = tB ? B->bsc : B->bsr;
    BSG_REQUIRE(kbs1 == kbs2, BSG_ERR_ARG, "matmult: inner block sizes do not match");
    g.kbs = kbs1;
    BSG_REQUIRE(C->bsr == g.ibs && C->bsc == g.jbs && C->nr == g.ni && C->nc == g.nj, BSG_ERR_ARG,
                "matmult: output dimensions or block sizes do not match");
    g.nib = ceil_div(g.ni, g.ibs);
    g.njb = ceil_div(g.nj, g.jbs);
    g.nkb = ceil_div(g.nk, g.kbs);
    g.tpb = thresh * (double)(g.ibs * g.jbs * g.kbs);  // blocksparsematrix.hpp:350
    cudaStream_t s = ctx->stream;
    if (beta == 0.0) {  // blocksparsematrix.hpp:299-305
        BSG_REQUIRE(bsg_bsm_zero(C) == BSG_OK, BSG_ERR_CUDA, bsg_last_error());
    } else if (beta != 1.0) {
        BSG_REQUIRE(bsg_bsm_scale(C, beta) == BSG_OK, BSG_ERR_CUDA, bsg_last_error());
    }
    const size_t n_out = g.nib * g.njb;
    if (!n_out || !g.nkb) return R;
    SliceOps h{A->dptr, A->dnorm, A->nrb, B->dptr, B->dnorm, B->nrb};
    const uint32_t lo = 0, hi = 1;
    DevBuf dsl(sizeof(SliceOps), s), dlo(4, s), dhi(4, s), dcount(n_out * 4, s);
    BSG_CUDA(cudaMemcpyAsync(dsl.p, &h, sizeof(SliceOps), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dlo.p, &lo, 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dhi.p, &hi, 4, cudaMemcpyHostToDevice, s));
    k_count<<<(unsigned)ceil_div(n_out, 128), 128, 0, s>>>(dsl.as<SliceOps>(), dlo.as<uint32_t>(), dhi.as<uint32_t>(),
                                                            g, 1, dcount.as<uint32_t>());
    ctx->note_launch();
    ctx->check_launch("pair count");
    std::vector<uint32_t> cnt(n_out);
    BSG_CUDA(cudaMemcpyAsync(cnt.data(), dcount.p, n_out * 4, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    bool touched = false;
    for (size_t x = 0; x < n_out; ++x) {
        if (!cnt[x]) continue;
        const size_t ib = x % g.nib, jb = x / g.nib, cbk = ib + jb * C->nrb;
        GemmItem it;
        it.fresh = C->hptr[cbk] == nullptr;
        C->ensure_block(cbk);
        touched = true;
        it.c = C->hptr[cbk];
        it.c_norm = C->dnorm + cbk;
        it.rows = (int)C->rows_of(ib);
        it.cols = (int)C->cols_of(jb);
        it.p0 = (uint32_t)R.total;
        it.p1 = (uint32_t)(R.total + cnt[x]);
        R.items.push_back(it);
        R.item_ib.push_back((uint32_t)ib);
        R.item_jb.push_back((uint32_t)jb);
        R.total += cnt[x];
    }
    if (touched) C->upload_table();
    return R;
}

}  // namespace bsg

using namespace bsg;

extern "C" bsg_status bsg_matmult_form(bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh, double alpha,
                                       double beta, int form, int n_digits, uint64_t *nsig_out) {
    return guard([&] {
        BSG_REQUIRE(C && A && B, BSG_ERR_ARG, "NULL matrix");
        uint64_t n = screened_product(C->ctx, {C}, {A}, tA ? 1 : 0, {B}, tB ? 1 : 0, {{0, 1}}, thresh, alpha, beta,
                                      form, n_digits);
        if (nsig_out) *nsig_out = n;
    });
}

extern "C" bsg_status bsg_matmult(bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh, double alpha,
                                  double beta, uint64_t *nsig_out) {
    return bsg_matmult_form(C, A, tA, B, tB, thresh, alpha, beta, BSG_FORM_FP64, 0, nsig_out);
}

extern "C" bsg_status bsg_tensormult_contract(bsg_bsm C, const bsg_bsm *A, int tA, const bsg_bsm *B, int tB,
                                              size_t n_slices, double thresh, double alpha, double beta) {
    return guard([&] {
        BSG_REQUIRE(C && A && B && n_slices > 0, BSG_ERR_ARG, "NULL argument or no slices");
        std::vector<bsg_bsm> as(A, A + n_slices), bs(B, B + n_slices);
        screened_product(C->ctx, {C}, as, tA ? 1 : 0, bs, tB ? 1 : 0, {{0, n_slices}}, thresh, alpha, beta,
                         BSG_FORM_FP64, 0);
    });
}

extern "C" bsg_status bsg_tensormult_batched(const bsg_bsm *C, bsg_bsm A, int tA, const bsg_bsm *B, int tB,
                                             size_t n_slices, double thresh, double alpha, double beta) {
    return guard([&] {
        BSG_REQUIRE(C && A && B && n_slices > 0, BSG_ERR_ARG, "NULL argument or no slices");
        std::vector<bsg_bsm> cs(C, C + n_slices), as(n_slices, A), bs(B, B + n_slices);
        std::vector<std::pair<size_t, size_t>> rg(n_slices);
        for (size_t l = 0; l < n_slices; ++l) rg[l] = {l, l + 1};
        screened_product(A->ctx, cs, as, tA ? 1 : 0, bs, tB ? 1 : 0, rg, thresh, alpha, beta, BSG_FORM_FP64, 0);
    });
}
