// Hybrid Strassen-Winograd / sparse block recursion (strassen.hpp).
//
// GPU schedule (FP64 form, bit-identical to the reference):
//  1. dry run (matmult_strassen_dryrun :511-679) on the device: level-0 flop
//     cells from the block norms, then one launch per level that sums the
//     2x2x2 children, applies the Strassen cost model and writes the tree.
//  2. the host reads the tree and lists the ACTIVE Strassen nodes (tree bit
//     set, no ancestor set: the nodes hybrid_recurse :418-508 hands to
//     strassen_recurse).
//  3. all active nodes run their Winograd recursion at once, level by level:
//     the fused pre-sums (:153-213) of every frame of a depth in one launch,
//     the leaf products of the deepest frames as grouped block GEMMs
//     (M1..M4, then the fused post-sum :215-237, then M5..M7), and on the way
//     up the `X += S` accumulations (:345-351) around each frame's post-sum.
//  4. one apply launch walks every C block's k axis in order and adds, per
//     position, either a screened single-pair leaf product (:435-446) or a
//     Strassen node's S grid block (accumulate_into_bsm :249-256) -- the same
//     order in which the reference's depth-first walk reaches C.
#include <algorithm>
#include <cmath>

#include "bsg_gemm64.cuh"
#include "bsg_ozaki.cuh"
#include "bsg_sched.cuh"

namespace bsg {

static const double kStrassenFac[20] = {10, 10, 10, 25, 35, 35, 35, 35, 35, 35,
                                        35, 35, 35, 35, 35, 35, 35, 35, 35, 35};  // strassen.hpp:582

__global__ void k_dry_level0(double *const *__restrict__ A, const double *__restrict__ An, size_t a_nrb,
                             double *const *__restrict__ B, const double *__restrict__ Bn, size_t b_nrb, size_t nib,
                             size_t njb, size_t nkb, size_t ni, size_t nj, size_t nk, size_t ibs, size_t jbs,
                             size_t kbs, double tpb, unsigned long long *__restrict__ nfl,
                             unsigned long long *__restrict__ total) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long f = 0;
    if (x < nib * njb * nkb) {
        const size_t ib = x % nib, jb = (x / nib) % njb, kb = x / (nib * njb);
        const size_t ai = ib + kb * a_nrb, bi = kb + jb * b_nrb;
        const double est = __dmul_rn(An[ai], Bn[bi]);
        const unsigned long long r = A[ai] ? (((ib + 1) * ibs <= ni) ? ibs : ni - ib * ibs) : 0;
        const unsigned long long kk = A[ai] ? (((kb + 1) * kbs <= nk) ? kbs : nk - kb * kbs) : 0;
        const unsigned long long c = B[bi] ? (((jb + 1) * jbs <= nj) ? jbs : nj - jb * jbs) : 0;
        f = (est >= tpb) ? 2ull * r * c * kk : 0ull;
        nfl[x] = f;
    }
    // block-level sum of the flops on level 0 (for the per-level report)
    for (int o = 16; o >= 1; o >>= 1) f += __shfl_down_sync(0xffffffffu, f, o);
    if ((threadIdx.x & 31) == 0 && f) atomicAdd(total, f);
}

struct DryLevel {
    size_t psb, sb, nsi, nsj, nsk, pni, pnj;
    unsigned long long cost;
};

__global__ void k_dry_level(const unsigned long long *__restrict__ prev, unsigned long long *__restrict__ next,
                            uint8_t *__restrict__ tree, DryLevel L, size_t nib, size_t njb, size_t nkb, size_t ni,
                            size_t nj, size_t nk, size_t ibs, size_t jbs, size_t kbs,
                            unsigned long long *__restrict__ total, unsigned long long *__restrict__ nf_out,
                            uint8_t *__restrict__ edge_out) {
    const size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long out = 0;
    if (s < L.nsi * L.nsj * L.nsk) {
        const size_t si = s % L.nsi, sj = (s / L.nsi) % L.nsj, sk = s / (L.nsi * L.nsj);
        const size_t ib0 = si * L.sb, jb0 = sj * L.sb, kb0 = sk * L.sb;
        const size_t ib1 = min(ib0 + L.sb, nib), jb1 = min(jb0 + L.sb, njb), kb1 = min(kb0 + L.sb, nkb);
        const size_t i1 = min(ib1 * ibs, ni), j1 = min(jb1 * jbs, nj), k1 = min(kb1 * kbs, nk);
        const bool edge = (i1 - ib0 * ibs) != ibs * L.sb || (j1 - jb0 * jbs) != jbs * L.sb || (k1 - kb0 * kbs) != kbs * L.sb;
        const size_t isub = (ib1 - ib0 + L.psb - 1) / L.psb, jsub = (jb1 - jb0 + L.psb - 1) / L.psb,
                     ksub = (kb1 - kb0 + L.psb - 1) / L.psb;
        unsigned long long nf = 0;
        for (size_t a = 0; a < isub; ++a)
            for (size_t b = 0; b < jsub; ++b)
                for (size_t c = 0; c < ksub; ++c)
                    nf += prev[(2 * si + a) + (2 * sj + b) * L.pni + (2 * sk + c) * L.pni * L.pnj];
        const bool go = (nf >= L.cost) && !edge;
        tree[si + sj * L.nsi + sk * L.nsi * L.nsj] = go;
        if (nf_out) {  // the node's cost below it (sparse recursion), for the scheduler's features
            nf_out[si + sj * L.nsi + sk * L.nsi * L.nsj] = nf;
            edge_out[si + sj * L.nsi + sk * L.nsi * L.nsj] = edge;
        }
        out = go ? L.cost : nf;
        next[si + sj * L.nsi + sk * L.nsi * L.nsj] = out;
    }
    for (int o = 16; o >= 1; o >>= 1) out += __shfl_down_sync(0xffffffffu, out, o);
    if ((threadIdx.x & 31) == 0 && out) atomicAdd(total, out);
}

struct DryResult {
    int n_levels = 0;
    std::vector<std::vector<uint8_t>> tree;
    std::vector<uint64_t> flops;
    std::vector<uint64_t> cost;                     // Strassen cost of a node per level
    std::vector<DevBuf> nf, edge;                   // per level, kept when asked for (scheduler)
};

static void check_square(bsg_bsm A, bsg_bsm B) {
    BSG_REQUIRE(A && B, BSG_ERR_ARG, "NULL matrix");
    BSG_REQUIRE(A->ctx == B->ctx, BSG_ERR_ARG, "matrices on different contexts");
    BSG_REQUIRE(A->nc == B->nr && A->bsc == B->bsr, BSG_ERR_ARG, "strassen: inner dimensions do not match");
    // only quadratic so far (strassen.hpp:547-551)
    BSG_REQUIRE(A->nr == B->nc && A->nr == A->nc && A->nrb == B->ncb && A->nrb == A->ncb, BSG_ERR_ARG,
                "strassen: only square products are supported (strassen.hpp:547-551)");
}

static DryResult dryrun(bsg_bsm A, bsg_bsm B, double tpb, bool keep_nodes = false) {
    check_square(A, B);
    bsg_ctx ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    const size_t ni = A->nr, nj = B->nc, nk = A->nc;
    const size_t ibs = A->bsr, jbs = B->bsc, kbs = A->bsc;
    const size_t nib = A->nrb, njb = B->ncb, nkb = A->ncb;
    DryResult R;
    const size_t max_level = (size_t)std::log2((double)nib + 0.5);
    R.n_levels = (int)max_level;
    R.flops.assign(max_level + 1, 0);
    if (!nib) return R;
    DevBuf tot((max_level + 1) * 8, s);
    BSG_CUDA(cudaMemsetAsync(tot.p, 0, (max_level + 1) * 8, s));
    auto *T = tot.as<unsigned long long>();
    DevBuf prev(nib * njb * nkb * 8, s);
    k_dry_level0<<<(unsigned)ceil_div(nib * njb * nkb, 256), 256, 0, s>>>(
        A->dptr, A->dnorm, A->nrb, B->dptr, B->dnorm, B->nrb, nib, njb, nkb, ni, nj, nk, ibs, jbs, kbs, tpb,
        prev.as<unsigned long long>(), T);
    ctx->note_launch();
    ctx->check_launch("dryrun level 0");
    const unsigned long long max_mult = 2ull * ibs * jbs * kbs, max_add = ibs * jbs;
    std::vector<DevBuf> trees;
    for (size_t level = 0; level < max_level; ++level) {
        DryLevel L;
        L.psb = (size_t)std::exp2((double)level);
        L.sb = (size_t)std::exp2((double)(level + 1));
        const unsigned long long cm = (unsigned long long)std::round(std::pow(7.0, (double)(level + 1))) * max_mult;
        const unsigned long long ca =
            (unsigned long long)(15e0 * kStrassenFac[level] * std::pow(4.0, (double)(level + 1)) * (double)max_add);
        L.cost = cm + ca;
        L.nsi = ceil_div(nib, L.sb);
        L.nsj = ceil_div(njb, L.sb);
        L.nsk = ceil_div(nkb, L.sb);
        L.pni = ceil_div(nib, L.psb);
        L.pnj = ceil_div(njb, L.psb);
        const size_t n = L.nsi * L.nsj * L.nsk;
        DevBuf next(n * 8, s), tr(n, s);
        R.cost.push_back(L.cost);
        if (keep_nodes) {
            R.nf.emplace_back(n * 8, s);
            R.edge.emplace_back(n, s);
        }
        k_dry_level<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(
            prev.as<unsigned long long>(), next.as<unsigned long long>(), tr.as<uint8_t>(), L, nib, njb, nkb, ni, nj,
            nk, ibs, jbs, kbs, T + level + 1, keep_nodes ? R.nf.back().as<unsigned long long>() : nullptr,
            keep_nodes ? R.edge.back().as<uint8_t>() : nullptr);
        ctx->note_launch();
        ctx->check_launch("dryrun level");
        R.tree.emplace_back(n);
        BSG_CUDA(cudaMemcpyAsync(R.tree.back().data(), tr.p, n, cudaMemcpyDeviceToHost, s));
        trees.push_back(std::move(tr));
        prev = std::move(next);
    }
    std::vector<unsigned long long> h(max_level + 1);
    BSG_CUDA(cudaMemcpyAsync(h.data(), T, (max_level + 1) * 8, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    for (size_t l = 0; l <= max_level; ++l) R.flops[l] = h[l];
    return R;
}

// ---------------------------------------------------------------------------
// Winograd frames
// ---------------------------------------------------------------------------

enum { OP_PREP_A = 0, OP_PREP_B = 1, OP_POST = 2, OP_ADD = 3 };

struct QuadOp {
    const double *in[4];
    double *out[4];
};

// strassen_prepare_A_side / _B_side / post_process_C_side / `X += S` on
// whole blocks, with the reference's expression order.
__global__ void k_quad(const QuadOp *__restrict__ ops, int op, int bs2) {
    const QuadOp q = ops[blockIdx.x];
    for (int i = threadIdx.x; i < bs2; i += blockDim.x) {
        if (op == OP_PREP_A) {  // in = a,b,c,d; out = c-a, c+d, (c+d)-a, b-((c+d)-a)
            const double a = q.in[0][i], b = q.in[1][i], c = q.in[2][i], d = q.in[3][i];
            q.out[0][i] = __dsub_rn(c, a);
            const double v = __dadd_rn(c, d);
            q.out[1][i] = v;
            const double w = __dsub_rn(v, a);
            q.out[2][i] = w;
            q.out[3][i] = __dsub_rn(b, w);
        } else if (op == OP_PREP_B) {  // in = A,B,C,D; out = C-D, C-A, D-(C-A), B-(D-(C-A))
            const double A = q.in[0][i], B = q.in[1][i], C = q.in[2][i], D = q.in[3][i];
            q.out[0][i] = __dsub_rn(C, D);
            const double v = __dsub_rn(C, A);
            q.out[1][i] = v;
            const double w = __dsub_rn(D, v);
            q.out[2][i] = w;
            q.out[3][i] = __dsub_rn(B, w);
        } else if (op == OP_POST) {  // out = nw, C00, C01, C10
            double *nw = q.out[0], *c00 = q.out[1], *c01 = q.out[2], *c10 = q.out[3];
            const double t = __dadd_rn(nw[i], c00[i]);
            const double n10 = __dadd_rn(c10[i], t);
            c10[i] = n10;
            nw[i] = __dadd_rn(c01[i], n10);
            c01[i] = __dadd_rn(c01[i], t);
        } else {  // X = fma(1, S, X)  (daxpy, matrix.hpp:107-117)
            q.out[0][i] = fma(1.0, q.in[0][i], q.out[0][i]);
        }
    }
}

// a square grid of bs x bs blocks, block (r, c) at blk[r + c*n]
struct Grid {
    std::vector<double *> blk;
    size_t n = 0;
    double *at(size_t r, size_t c) const { return blk[r + c * n]; }
    Grid quad(size_t r0, size_t c0, size_t h) const {
        Grid g;
        g.n = h;
        g.blk.resize(h * h);
        for (size_t c = 0; c < h; ++c)
            for (size_t r = 0; r < h; ++r) g.blk[r + c * h] = at(r0 + r, c0 + c);
        return g;
    }
};

struct Frame {
    Grid out[4];             // C00, C01, C10, C11
    Grid a, b, c, d, A, C, B, D;
    Grid pa[4], pb[4];       // na_pc, pc_pd, na_pc_pd, pa_pb_nc_nd / pC_nD, nA_pC, pA_nC_pD, nA_pB_pC_nD
    int child[7] = {-1, -1, -1, -1, -1, -1, -1};
};

// (X, P, Q) of product i of a frame, strassen.hpp:392-402
static void product(const Frame &f, int i, const Grid **X, const Grid **P, const Grid **Q) {
    switch (i) {
        case 0: *X = &f.out[0]; *P = &f.a; *Q = &f.A; break;        // M1 -> C00
        case 1: *X = &f.out[2]; *P = &f.pa[0]; *Q = &f.pb[0]; break; // M2 -> C10
        case 2: *X = &f.out[1]; *P = &f.pa[1]; *Q = &f.pb[1]; break; // M3 -> C01
        case 3: *X = &f.out[3]; *P = &f.pa[2]; *Q = &f.pb[2]; break; // M4 -> nw
        case 4: *X = &f.out[1]; *P = &f.pa[3]; *Q = &f.D; break;     // M5 -> C01
        case 5: *X = &f.out[2]; *P = &f.d; *Q = &f.pb[3]; break;     // M6 -> C10
        default: *X = &f.out[0]; *P = &f.b; *Q = &f.B; break;        // M7 -> C00
    }
}

struct Arena {
    DevBuf buf;
    size_t used = 0, bs2 = 0;
    double *take(size_t nblocks) {
        double *p = buf.as<double>() + used * bs2;
        used += nblocks;
        return p;
    }
    Grid grid(size_t n) {
        Grid g;
        g.n = n;
        g.blk.resize(n * n);
        double *p = take(n * n);
        for (size_t i = 0; i < n * n; ++i) g.blk[i] = p + i * bs2;
        return g;
    }
};

static void run_quads(bsg_ctx ctx, const std::vector<QuadOp> &ops, int op, int bs2, cudaStream_t s) {
    if (ops.empty()) return;
    DevBuf d(ops.size() * sizeof(QuadOp), s);
    BSG_CUDA(cudaMemcpyAsync(d.p, ops.data(), ops.size() * sizeof(QuadOp), cudaMemcpyHostToDevice, s));
    for (size_t off = 0; off < ops.size(); off += 1u << 30) {
        const unsigned g = (unsigned)std::min<size_t>(ops.size() - off, 1u << 30);
        k_quad<<<g, 256, 0, s>>>(d.as<QuadOp>() + off, op, bs2);
        ctx->note_launch();
    }
    ctx->check_launch("winograd sums");
    BSG_CUDA(cudaStreamSynchronize(s));
}

// dense 8-product `X(rb,cb) += sum_kb P(rb,kb) Q(kb,cb)` (strassen.hpp:311-323)
static void leaf_products(bsg_ctx ctx, const std::vector<std::tuple<const Grid *, const Grid *, const Grid *>> &prods,
                          int bs, int form, int n_digits, cudaStream_t s) {
    if (form != BSG_FORM_FP64) {
        // mixed form: bf16 digit products on the tensor cores; the Winograd
        // sums around them stay FP64
        if (prods.empty()) return;
        const size_t n = std::get<0>(prods[0])->n;
        std::vector<double *> X, P, Q;
        for (auto &t : prods) {
            BSG_REQUIRE(std::get<0>(t)->n == n, BSG_ERR_PRECOND, "leaf grids of one depth share their side");
            X.insert(X.end(), std::get<0>(t)->blk.begin(), std::get<0>(t)->blk.end());
            P.insert(P.end(), std::get<1>(t)->blk.begin(), std::get<1>(t)->blk.end());
            Q.insert(Q.end(), std::get<2>(t)->blk.begin(), std::get<2>(t)->blk.end());
        }
        ozaki_grid_products(ctx, prods.size(), n, X, P, Q, bs, n_digits, s);
        return;
    }
    std::vector<GemmItem> items;
    std::vector<GemmPair> pairs;
    for (auto &t : prods) {
        const Grid &X = *std::get<0>(t), &P = *std::get<1>(t), &Q = *std::get<2>(t);
        const size_t n = X.n;
        for (size_t cb = 0; cb < n; ++cb)
            for (size_t rb = 0; rb < n; ++rb) {
                GemmItem it;
                it.c = X.at(rb, cb);
                it.c_norm = nullptr;
                it.rows = it.cols = bs;
                it.fresh = 0;
                it.p0 = (uint32_t)pairs.size();
                for (size_t kb = 0; kb < n; ++kb) pairs.push_back(GemmPair{P.at(rb, kb), Q.at(kb, cb), bs, bs, bs});
                it.p1 = (uint32_t)pairs.size();
                items.push_back(it);
            }
    }
    if (items.empty()) return;
    DevBuf di(items.size() * sizeof(GemmItem), s), dp(pairs.size() * sizeof(GemmPair), s);
    BSG_CUDA(cudaMemcpyAsync(di.p, items.data(), items.size() * sizeof(GemmItem), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dp.p, pairs.data(), pairs.size() * sizeof(GemmPair), cudaMemcpyHostToDevice, s));
    launch_gemm64(ctx, di.as<GemmItem>(), items.size(), dp.as<GemmPair>(), 0, 0, 1.0, bs, bs, s);
    BSG_CUDA(cudaStreamSynchronize(s));
}

// Runs strassen_recurse for every root frame (same grid side h).
static void winograd(bsg_ctx ctx, std::vector<Frame> &roots, size_t h, size_t bs, size_t min_size, int form,
                     int n_digits, cudaStream_t s) {
    const size_t bs2 = bs * bs;
    // depth schedule: products at depth d act on grids of side g_d
    std::vector<size_t> g{h};
    while (true) {
        const size_t gd = g.back();
        const bool recurse = !(gd == 1) && !(gd % 2 != 0 || gd * bs <= min_size);
        if (!recurse) break;
        g.push_back(gd / 2);
    }
    const size_t D = g.size() - 1;  // frames at depth D have leaf products
    // arena: per frame 8 prepared grids; frames at depth d>0 also own 4 outputs
    size_t nblocks = 0, nframes = roots.size();
    for (size_t d = 0; d <= D; ++d) {
        nblocks += nframes * 8 * g[d] * g[d];
        if (d > 0) nblocks += nframes * 4 * g[d] * g[d];
        nframes *= 7;
    }
    Arena ar;
    ar.bs2 = bs2;
    ar.buf = DevBuf(nblocks * bs2 * 8, s);
    std::vector<std::vector<Frame>> frames(D + 1);
    frames[0] = roots;
    for (size_t d = 0; d <= D; ++d) {
        auto &fr = frames[d];
        std::vector<QuadOp> qa, qb;
        for (auto &f : fr) {
            for (int i = 0; i < 4; ++i) {
                f.pa[i] = ar.grid(g[d]);
                f.pb[i] = ar.grid(g[d]);
            }
            for (size_t e = 0; e < g[d] * g[d]; ++e) {
                qa.push_back(QuadOp{{f.a.blk[e], f.b.blk[e], f.c.blk[e], f.d.blk[e]},
                                    {f.pa[0].blk[e], f.pa[1].blk[e], f.pa[2].blk[e], f.pa[3].blk[e]}});
                qb.push_back(QuadOp{{f.A.blk[e], f.B.blk[e], f.C.blk[e], f.D.blk[e]},
                                    {f.pb[0].blk[e], f.pb[1].blk[e], f.pb[2].blk[e], f.pb[3].blk[e]}});
            }
        }
        run_quads(ctx, qa, OP_PREP_A, (int)bs2, s);
        run_quads(ctx, qb, OP_PREP_B, (int)bs2, s);
        if (d == D) break;
        // children: fresh zero outputs, operands = quadrants of P and Q
        auto &next = frames[d + 1];
        const size_t hh = g[d + 1];
        for (auto &f : fr) {
            for (int i = 0; i < 7; ++i) {
                const Grid *X, *P, *Q;
                product(f, i, &X, &P, &Q);
                Frame c;
                for (int q = 0; q < 4; ++q) {
                    c.out[q] = ar.grid(hh);
                    BSG_CUDA(cudaMemsetAsync(c.out[q].blk[0], 0, hh * hh * bs2 * 8, s));
                }
                c.a = P->quad(0, 0, hh);
                c.b = P->quad(0, hh, hh);
                c.c = P->quad(hh, 0, hh);
                c.d = P->quad(hh, hh, hh);
                c.A = Q->quad(0, 0, hh);
                c.C = Q->quad(0, hh, hh);
                c.B = Q->quad(hh, 0, hh);
                c.D = Q->quad(hh, hh, hh);
                f.child[i] = (int)next.size();
                next.push_back(std::move(c));
            }
        }
    }
    auto post_ops = [&](const std::vector<Frame> &fr) {
        std::vector<QuadOp> q;
        for (auto &f : fr)
            for (size_t e = 0; e < f.out[0].blk.size(); ++e)
                q.push_back(QuadOp{{nullptr, nullptr, nullptr, nullptr},
                                   {f.out[3].blk[e], f.out[0].blk[e], f.out[1].blk[e], f.out[2].blk[e]}});
        run_quads(ctx, q, OP_POST, (int)bs2, s);
    };
    // leaf frames: M1..M4, post, M5..M7
    {
        std::vector<std::tuple<const Grid *, const Grid *, const Grid *>> pA, pB;
        for (auto &f : frames[D])
            for (int i = 0; i < 7; ++i) {
                const Grid *X, *P, *Q;
                product(f, i, &X, &P, &Q);
                (i < 4 ? pA : pB).emplace_back(X, P, Q);
            }
        leaf_products(ctx, pA, (int)bs, form, n_digits, s);
        post_ops(frames[D]);
        leaf_products(ctx, pB, (int)bs, form, n_digits, s);
    }
    // upward: X += S_child around each frame's post-sum
    for (size_t d = D; d-- > 0;) {
        const size_t hh = g[d + 1];
        auto add_ops = [&](int lo, int hi) {
            std::vector<QuadOp> q;
            for (auto &f : frames[d])
                for (int i = lo; i < hi; ++i) {
                    const Grid *X, *P, *Q;
                    product(f, i, &X, &P, &Q);
                    const Frame &c = frames[d + 1][f.child[i]];
                    for (size_t cb = 0; cb < hh; ++cb)
                        for (size_t rb = 0; rb < hh; ++rb) {
                            const size_t e = rb + cb * hh;
                            q.push_back(QuadOp{{c.out[0].blk[e]}, {X->at(rb, cb)}});
                            q.push_back(QuadOp{{c.out[1].blk[e]}, {X->at(rb, cb + hh)}});
                            q.push_back(QuadOp{{c.out[2].blk[e]}, {X->at(rb + hh, cb)}});
                            q.push_back(QuadOp{{c.out[3].blk[e]}, {X->at(rb + hh, cb + hh)}});
                        }
                }
            run_quads(ctx, q, OP_ADD, (int)bs2, s);
        };
        add_ops(0, 4);
        post_ops(frames[d]);
        add_ops(4, 7);
    }
    for (size_t i = 0; i < roots.size(); ++i) roots[i] = frames[0][i];
}

// ---------------------------------------------------------------------------
// ordered application into C
// ---------------------------------------------------------------------------

struct ApplyGeom {
    size_t nib, njb, nkb, bs, a_nrb, b_nrb, c_nrb;
    int n_levels;
    double tpb;
};

// Per C block: walk kb in order; a (ib,jb,kb) covered by an active Strassen
// node contributes that node's S block once (at the node's first k block),
// an uncovered triple is a screened leaf: C = t + C.
__global__ void __launch_bounds__(256) k_apply(double *const *__restrict__ Cp, double *const *__restrict__ Ap,
                                               const double *__restrict__ An, double *const *__restrict__ Bp,
                                               const double *__restrict__ Bn, const uint8_t *__restrict__ tree,
                                               const int *__restrict__ node_of, const size_t *__restrict__ lvl_off,
                                               const size_t *__restrict__ lvl_n, double *const *__restrict__ node_S,
                                               ApplyGeom g, unsigned long long *__restrict__ nsig) {
    const size_t ib = blockIdx.x % g.nib, jb = blockIdx.x / g.nib;
    double *C = Cp[ib + jb * g.c_nrb];
    if (!C) return;  // a size-0 C view makes the leaf BLAS call a no-op
    const int bs = (int)g.bs, n = bs * bs;
    constexpr int EPT = 16;
    double acc[EPT];
    int ii[EPT], jj[EPT];
#pragma unroll
    for (int s = 0; s < EPT; ++s) {
        const int e = threadIdx.x + s * blockDim.x;
        ii[s] = e < n ? e % bs : 0;
        jj[s] = e < n ? e / bs : 0;
        acc[s] = e < n ? C[e] : 0.0;
    }
    unsigned long long cnt = 0;
    for (size_t kb = 0; kb < g.nkb; ++kb) {
        int node = -1;
        size_t sbn = 0;
        for (int L = g.n_levels - 1; L >= 0; --L) {
            const size_t sh = (size_t)L + 1;
            const size_t nL = lvl_n[L];
            const size_t idx = (ib >> sh) + (jb >> sh) * nL + (kb >> sh) * nL * nL;
            if (tree[lvl_off[L] + idx]) {
                node = node_of[lvl_off[L] + idx];
                sbn = (size_t)1 << sh;
                break;
            }
        }
        if (node >= 0) {
            const size_t h = sbn / 2, ri = ib % sbn, rj = jb % sbn;
            const int q = (ri >= h ? 2 : 0) + (rj >= h ? 1 : 0);  // S00, S01, S10, S11
            const double *S = node_S[node] + ((size_t)q * h * h + (ri % h) + (rj % h) * h) * n;
#pragma unroll
            for (int s = 0; s < EPT; ++s)
                if (threadIdx.x + s * blockDim.x < n) acc[s] = fma(1.0, S[threadIdx.x + s * blockDim.x], acc[s]);
            kb = (kb / sbn) * sbn + sbn - 1;  // the node covers the rest of this k range
            continue;
        }
        const size_t ai = ib + kb * g.a_nrb, bi = kb + jb * g.b_nrb;
        const double *A = Ap[ai], *B = Bp[bi];
        if (!A || !B) continue;
        if (__dmul_rn(An[ai], Bn[bi]) < g.tpb) continue;
        double t[EPT];
#pragma unroll
        for (int s = 0; s < EPT; ++s) t[s] = 0.0;
        for (int l = 0; l < bs; ++l) {
#pragma unroll
            for (int s = 0; s < EPT; ++s)
                if (threadIdx.x + s * blockDim.x < n) t[s] = fma(__ldg(A + ii[s] + l * bs), __ldg(B + l + jj[s] * bs), t[s]);
        }
#pragma unroll
        for (int s = 0; s < EPT; ++s) acc[s] = __dadd_rn(t[s], acc[s]);
        ++cnt;
    }
#pragma unroll
    for (int s = 0; s < EPT; ++s) {
        const int e = threadIdx.x + s * blockDim.x;
        if (e < n) C[e] = acc[s];
    }
    if (threadIdx.x == 0 && cnt) atomicAdd(nsig, cnt);
}

// Features (host copy, kSchedNodeIn floats per node) and eligibility of the
// nodes of one dry-run level.
static void level_features(bsg_bsm C, bsg_bsm A, bsg_bsm B, const DryResult &R, int L, std::vector<float> &F,
                           std::vector<uint8_t> &ok, DevBuf *dF_keep = nullptr) {
    cudaStream_t s = A->ctx->stream;
    const size_t sb = (size_t)1 << (L + 1);
    const size_t nsi = ceil_div(A->nrb, sb), nsj = ceil_div(B->ncb, sb), nsk = ceil_div(A->ncb, sb);
    const size_t n = nsi * nsj * nsk;
    DevBuf dF(n * kSchedNodeIn * 4, s), dok(n, s);
    launch_node_features(A, B, C, L, nsi, nsj, nsk, R.nf[L].as<unsigned long long>(), R.edge[L].as<uint8_t>(),
                         R.cost[L], dF.as<float>(), dok.as<uint8_t>());
    F.resize(n * kSchedNodeIn);
    ok.resize(n);
    BSG_CUDA(cudaMemcpyAsync(F.data(), dF.p, n * kSchedNodeIn * 4, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaMemcpyAsync(ok.data(), dok.p, n, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    if (dF_keep) *dF_keep = std::move(dF);
}

// Replaces the cost model's tree per the scheduling policy (the cost model's
// own tree is BSG_SCHED_COST and the fallback of BSG_SCHED_MLP on levels with
// more than kSchedMaxNodes nodes).
constexpr size_t kSchedMaxNodes = 65536;
static void apply_policy(bsg_bsm C, bsg_bsm A, bsg_bsm B, DryResult &R, int policy, bsg_sched sched) {
    const int NL = R.n_levels;
    if (policy == BSG_SCHED_COST) return;
    if (policy == BSG_SCHED_NONE) {
        for (auto &t : R.tree) std::fill(t.begin(), t.end(), 0);
        return;
    }
    if (policy == BSG_SCHED_ROOT || policy == BSG_SCHED_DENSE) {
        for (auto &t : R.tree) std::fill(t.begin(), t.end(), 0);
        if (NL == 0 || R.tree[NL - 1].size() != 1) return;  // no single root node
        std::vector<float> F;
        std::vector<uint8_t> ok;
        level_features(C, A, B, R, NL - 1, F, ok);
        R.tree[NL - 1][0] = ok[0] ? (policy == BSG_SCHED_ROOT ? kNodeStrassen : kNodeDense) : kNodeSparse;
        return;
    }
    BSG_REQUIRE(policy == BSG_SCHED_MLP && sched, BSG_ERR_ARG, "BSG_SCHED_MLP needs a scheduler");
    BSG_REQUIRE(sched->ctx == A->ctx, BSG_ERR_ARG, "scheduler on another context");
    // features, forward pass and decisions of every covered level on the
    // device; one synchronization for all the levels' trees
    cudaStream_t s = A->ctx->stream;
    std::vector<DevBuf> keep;
    std::vector<int> levels;
    for (int L = 0; L < NL; ++L) {
        const size_t n = R.tree[L].size();
        if (n > kSchedMaxNodes || !n) continue;  // cost model (its Strassen nodes use the call's min_size)
        const size_t sb = (size_t)1 << (L + 1);
        DevBuf dF(n * kSchedNodeIn * 4, s), dX(n * kSchedOpts * kSchedIn * 4, s), dok(n, s),
            dY(n * kSchedOpts * 4, s), dT(n, s);
        launch_node_features(A, B, C, L, ceil_div(A->nrb, sb), ceil_div(B->ncb, sb), ceil_div(A->ncb, sb),
                             R.nf[L].as<unsigned long long>(), R.edge[L].as<uint8_t>(), R.cost[L], dF.as<float>(),
                             dok.as<uint8_t>());
        launch_option_rows(A->ctx, dF.as<float>(), n, dX.as<float>());
        // predicted log(t_option / t_sparse) of every (node, option)
        sched->predict_dev(dX.as<float>(), (int)(n * kSchedOpts), dY.as<float>());
        launch_sched_decide(A->ctx, dok.as<uint8_t>(), dY.as<float>(), n, L, dT.as<uint8_t>());
        BSG_CUDA(cudaMemcpyAsync(R.tree[L].data(), dT.p, n, cudaMemcpyDeviceToHost, s));
        keep.push_back(std::move(dF));
        keep.push_back(std::move(dX));
        keep.push_back(std::move(dok));
        keep.push_back(std::move(dY));
        keep.push_back(std::move(dT));
    }
    BSG_CUDA(cudaStreamSynchronize(s));
}

static void strassen_sparse(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh, size_t min_size, int form, int n_digits,
                            int policy = BSG_SCHED_COST, bsg_sched sched = nullptr, uint64_t *n_nodes = nullptr) {
    check_square(A, B);
    BSG_REQUIRE(C && C->ctx == A->ctx, BSG_ERR_ARG, "output on another context");
    BSG_REQUIRE(C->nrb == A->nrb && C->ncb == B->ncb && C->nr == A->nr && C->nc == B->nc, BSG_ERR_ARG,
                "strassen: output dimensions do not match");
    BSG_REQUIRE(A->bsr == A->bsc && B->bsr == B->bsc && A->bsr == B->bsr && C->bsr == A->bsr && C->bsc == A->bsr,
                BSG_ERR_ARG, "strassen: square blocks of one size are required");
    bsg_ctx ctx = A->ctx;
    cudaStream_t s = ctx->stream;
    const size_t bs = A->bsr, nib = A->nrb;
    BSG_REQUIRE(bs * bs <= 16 * 256, BSG_ERR_UNSUPPORTED, "strassen kernels support bs <= 64");
    const double tpb = thresh * (double)(A->bsr * B->bsc * A->bsc);  // strassen.hpp:710
    DryResult R = dryrun(A, B, tpb, policy != BSG_SCHED_COST);
    apply_policy(C, A, B, R, policy, sched);
    const int NL = R.n_levels;
    // active nodes: tree bit set and no ancestor set
    std::vector<size_t> lvl_n(NL), lvl_off(NL);
    size_t tot = 0;
    for (int L = 0; L < NL; ++L) {
        lvl_n[L] = ceil_div(nib, (size_t)1 << (L + 1));
        lvl_off[L] = tot;
        tot += R.tree[L].size();
    }
    std::vector<int> node_of(std::max<size_t>(tot, 1), -1);
    struct Node {
        int L;
        size_t si, sj, sk;
        uint8_t opt;  // decision-tree byte: Strassen (the call's min_size or a depth) or dense tile
    };
    std::vector<Node> nodes;
    std::vector<std::vector<uint8_t>> cov(NL);
    for (int L = NL - 1; L >= 0; --L) {
        const size_t n = lvl_n[L];
        cov[L].assign(n * n * n, 0);
        for (size_t sk = 0; sk < n; ++sk)
            for (size_t sj = 0; sj < n; ++sj)
                for (size_t si = 0; si < n; ++si) {
                    const size_t idx = si + sj * n + sk * n * n;
                    bool above = false;
                    if (L + 1 < NL) {
                        const size_t pn = lvl_n[L + 1];
                        above = cov[L + 1][(si / 2) + (sj / 2) * pn + (sk / 2) * pn * pn] != 0;
                    }
                    const bool t = R.tree[L][idx] != 0;
                    cov[L][idx] = above || t;
                    if (t && !above) {
                        node_of[lvl_off[L] + idx] = (int)nodes.size();
                        nodes.push_back(Node{L, si, sj, sk, R.tree[L][idx]});
                    }
                }
    }
    if (n_nodes) *n_nodes = nodes.size();
    // preconditions of the Strassen path: full, present A/B/C blocks
    for (auto &nd : nodes) {
        const size_t sb = (size_t)1 << (nd.L + 1), ib0 = nd.si * sb, jb0 = nd.sj * sb, kb0 = nd.sk * sb;
        for (size_t x = 0; x < sb; ++x)
            for (size_t y = 0; y < sb; ++y) {
                BSG_REQUIRE(A->hptr[(ib0 + x) + (kb0 + y) * A->nrb] && B->hptr[(kb0 + x) + (jb0 + y) * B->nrb],
                            BSG_ERR_PRECOND, "strassen: an operand block on a Strassen node is absent");
                BSG_REQUIRE(C->hptr[(ib0 + x) + (jb0 + y) * C->nrb], BSG_ERR_PRECOND,
                            "strassen: C must be fully allocated (fill_with_values) on Strassen nodes");
            }
    }
    // Winograd recursion per node size and depth; dense tiles per node size
    std::vector<DevBuf> sbufs;
    std::vector<double *> node_S(std::max<size_t>(nodes.size(), 1), nullptr);
    for (int L = 0; L < NL; ++L) {
        for (uint8_t opt = kNodeStrassen; opt <= kNodeDense; ++opt) {
            std::vector<Frame> roots;
            std::vector<int> ids;
            const size_t sb = (size_t)1 << (L + 1), h = sb / 2;
            // a node of depth t recurses while the grid side exceeds h / 2^(t-1)
            const size_t ms = opt == kNodeStrassen ? min_size
                                                   : std::max<size_t>(1, h >> (opt - kNodeDepth1)) * bs;
            std::vector<std::tuple<const Grid *, const Grid *, const Grid *>> dense;
            std::vector<Grid> dgrids;
            dgrids.reserve(3 * nodes.size());
            for (size_t i = 0; i < nodes.size(); ++i) {
                if (nodes[i].L != L || nodes[i].opt != opt) continue;
                const Node &nd = nodes[i];
                const size_t ib0 = nd.si * sb, jb0 = nd.sj * sb, kb0 = nd.sk * sb;
                DevBuf sbuf(4 * h * h * bs * bs * 8, s);
                BSG_CUDA(cudaMemsetAsync(sbuf.p, 0, sbuf.bytes, s));  // S00..S11 start at 0.0 (:468-471)
                node_S[i] = sbuf.as<double>();
                auto view = [&](bsg_bsm M, size_t r0, size_t c0, size_t side) {
                    Grid g;
                    g.n = side;
                    g.blk.resize(side * side);
                    for (size_t c = 0; c < side; ++c)
                        for (size_t r = 0; r < side; ++r) g.blk[r + c * side] = M->hptr[(r0 + r) + (c0 + c) * M->nrb];
                    return g;
                };
                if (opt == kNodeDense) {
                    // the node's product as one dense tile: S (the node's quadrants
                    // S00, S01, S10, S11, as k_apply reads them) += A_node B_node over
                    // every block product, unscreened
                    Grid X;
                    X.n = sb;
                    X.blk.resize(sb * sb);
                    for (size_t c = 0; c < sb; ++c)
                        for (size_t r = 0; r < sb; ++r) {
                            const size_t q = (r >= h ? 2 : 0) + (c >= h ? 1 : 0);
                            X.blk[r + c * sb] = sbuf.as<double>() + (q * h * h + (r % h) + (c % h) * h) * bs * bs;
                        }
                    dgrids.push_back(std::move(X));
                    dgrids.push_back(view(A, ib0, kb0, sb));
                    dgrids.push_back(view(B, kb0, jb0, sb));
                    const size_t k = dgrids.size();
                    dense.emplace_back(&dgrids[k - 3], &dgrids[k - 2], &dgrids[k - 1]);
                    sbufs.push_back(std::move(sbuf));
                    continue;
                }
                Frame f;
                for (int q = 0; q < 4; ++q) {
                    f.out[q].n = h;
                    f.out[q].blk.resize(h * h);
                    for (size_t e = 0; e < h * h; ++e) f.out[q].blk[e] = sbuf.as<double>() + (q * h * h + e) * bs * bs;
                }
                f.a = view(A, ib0, kb0, h);
                f.b = view(A, ib0, kb0 + h, h);
                f.c = view(A, ib0 + h, kb0, h);
                f.d = view(A, ib0 + h, kb0 + h, h);
                f.A = view(B, kb0, jb0, h);
                f.C = view(B, kb0, jb0 + h, h);
                f.B = view(B, kb0 + h, jb0, h);
                f.D = view(B, kb0 + h, jb0 + h, h);
                roots.push_back(std::move(f));
                ids.push_back((int)i);
                sbufs.push_back(std::move(sbuf));
            }
            if (!roots.empty()) winograd(ctx, roots, h, bs, ms, form, n_digits, s);
            if (!dense.empty()) leaf_products(ctx, dense, (int)bs, form, n_digits, s);
        }
    }
    // ordered application
    std::vector<uint8_t> tree_flat(std::max<size_t>(tot, 1), 0);
    for (int L = 0; L < NL; ++L) std::copy(R.tree[L].begin(), R.tree[L].end(), tree_flat.begin() + lvl_off[L]);
    DevBuf dtree(tree_flat.size(), s), dnode(node_of.size() * 4, s), doff(std::max(NL, 1) * 8, s),
        dn(std::max(NL, 1) * 8, s), dS(node_S.size() * 8, s), dcnt(8, s);
    BSG_CUDA(cudaMemcpyAsync(dtree.p, tree_flat.data(), tree_flat.size(), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(dnode.p, node_of.data(), node_of.size() * 4, cudaMemcpyHostToDevice, s));
    if (NL) {
        BSG_CUDA(cudaMemcpyAsync(doff.p, lvl_off.data(), NL * 8, cudaMemcpyHostToDevice, s));
        BSG_CUDA(cudaMemcpyAsync(dn.p, lvl_n.data(), NL * 8, cudaMemcpyHostToDevice, s));
    }
    BSG_CUDA(cudaMemcpyAsync(dS.p, node_S.data(), node_S.size() * 8, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemsetAsync(dcnt.p, 0, 8, s));
    ApplyGeom ag{nib, B->ncb, A->ncb, bs, A->nrb, B->nrb, C->nrb, NL, tpb};
    const unsigned nt = (unsigned)std::max<size_t>(32, ((ceil_div(bs * bs, 16) + 31) / 32) * 32);
    // sparse single-pair leaves stay FP64 in every form (they are screened,
    // few, and their order against the node contributions is fixed here)
    k_apply<<<(unsigned)(nib * B->ncb), nt, 0, s>>>(C->dptr, A->dptr, A->dnorm, B->dptr, B->dnorm,
                                                     dtree.as<uint8_t>(), dnode.as<int>(), doff.as<size_t>(),
                                                     dn.as<size_t>(), dS.as<double *>(), ag,
                                                     dcnt.as<unsigned long long>());
    ctx->note_launch();
    ctx->check_launch("strassen apply");
    BSG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace bsg

using namespace bsg;

extern "C" bsg_status bsg_strassen_dryrun(bsg_bsm A, bsg_bsm B, double tpb, int *n_levels, uint8_t *tree_host,
                                          size_t tree_cap, uint64_t *flops) {
    return guard([&] {
        BSG_REQUIRE(n_levels, BSG_ERR_ARG, "n_levels is NULL");
        DryResult R = dryrun(A, B, tpb);
        *n_levels = R.n_levels;
        size_t off = 0;
        for (auto &lv : R.tree) {
            if (tree_host) {
                BSG_REQUIRE(off + lv.size() <= tree_cap, BSG_ERR_ARG, "tree buffer too small");
                std::copy(lv.begin(), lv.end(), tree_host + off);
            }
            off += lv.size();
        }
        if (flops)
            for (size_t l = 0; l < R.flops.size(); ++l) flops[l] = R.flops[l];
    });
}

extern "C" bsg_status bsg_matmult_strassen_sparse(bsg_bsm C, bsg_bsm A, int tA, bsg_bsm B, int tB, double thresh,
                                                  double alpha, double beta, size_t min_size) {
    return guard([&] {
        // strassen.hpp:693: no transposes, alpha == 1; beta is ignored (:694-697)
        BSG_REQUIRE(!tA && !tB, BSG_ERR_PRECOND, "matmult_strassen_sparse: transposes are not supported");
        BSG_REQUIRE(alpha == 1.0, BSG_ERR_PRECOND, "matmult_strassen_sparse: alpha must be 1");
        (void)beta;
        strassen_sparse(C, A, B, thresh, min_size, BSG_FORM_FP64, 0);
    });
}

extern "C" bsg_status bsg_matmult_strassen_sparse_form(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh,
                                                       size_t min_size, int form, int n_digits) {
    return guard([&] {
        BSG_REQUIRE(form == BSG_FORM_FP64 || form == BSG_FORM_OZAKI, BSG_ERR_ARG, "unknown form");
        strassen_sparse(C, A, B, thresh, min_size, form, n_digits);
    });
}

extern "C" bsg_status bsg_matmult_strassen_sparse_sched(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh, size_t min_size,
                                                        int form, int n_digits, int policy, bsg_sched sched,
                                                        uint64_t *n_strassen_nodes) {
    return guard([&] {
        BSG_REQUIRE(form == BSG_FORM_FP64 || form == BSG_FORM_OZAKI, BSG_ERR_ARG, "unknown form");
        BSG_REQUIRE(policy >= BSG_SCHED_COST && policy <= BSG_SCHED_DENSE, BSG_ERR_ARG, "unknown policy");
        strassen_sparse(C, A, B, thresh, min_size, form, n_digits, policy, sched, n_strassen_nodes);
    });
}

extern "C" bsg_status bsg_strassen_root_features(bsg_bsm C, bsg_bsm A, bsg_bsm B, double thresh, float *features,
                                                 int *eligible) {
    return guard([&] {
        check_square(A, B);
        BSG_REQUIRE(C && features && eligible, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(C->nrb == A->nrb && C->ncb == B->ncb, BSG_ERR_ARG, "output dimensions do not match");
        const double tpb = thresh * (double)(A->bsr * B->bsc * A->bsc);
        DryResult R = dryrun(A, B, tpb, true);
        BSG_REQUIRE(R.n_levels > 0 && R.tree[R.n_levels - 1].size() == 1, BSG_ERR_PRECOND,
                    "the decision tree has no single root node (block count not a power of two)");
        std::vector<float> F;
        std::vector<uint8_t> ok;
        level_features(C, A, B, R, R.n_levels - 1, F, ok);
        std::copy(F.begin(), F.begin() + kSchedNodeIn, features);
        *eligible = ok[0];
    });
}
