// Batched screened products: n independent C_i = alpha A_i B_i + beta C_i
// (each with matmult's semantics, blocksparsematrix.hpp:293-414), of any
// sizes and block sizes.
//
// Mixed form: the products are grouped by (block rows, block k, block cols);
// each group's digit images and exponents go into shared buffers (per-product
// index bases), the tiles of every group into one list (group after group),
// and ONE persistent k_ozgemm launch runs every tile of every product of the
// batch, each tile in its group's geometry (up to 8 groups per launch).  The
// tile height (slots per tile) of each group is picked by an autotuner that
// times the candidates on the group's own tiles in a launch of their own
// (writing scratch blocks) and caches the winner in the context.  A plan
// captures the device work of a batch in a CUDA graph for replay.
//
// FP64 form: one grouped FP64 launch per product (the reference's order).
#include <algorithm>
#include <cstring>

#include "bsg_gemm64.cuh"
#include "bsg_ozaki.cuh"

namespace bsg {

using bf16 = __nv_bfloat16;

struct BatchProd {
    bsg_bsm C, A, B;
    ScreenItems si;
};

struct ClassRun {
    OzShape sh;                      // with the tuned R and S
    std::vector<size_t> prods;       // members of the batch
    OzTilePlan tp;                   // host tile lists (kept alive by plans)
    std::vector<size_t> tile0;       // first tile of each member
};

// images and exponents of a group (device buffers owned by the caller)
struct ClassImages {
    DevBuf rexp, cexp, aimg, bimg;
    std::vector<size_t> roff, coff;
    std::vector<uint32_t> abase, bbase;
};

// exponents and digit images of the members into the group's buffers
static void class_images_compute(bsg_ctx ctx, std::vector<BatchProd> &P, const std::vector<size_t> &members,
                                 const OzShape &sh, ClassImages &im) {
    const size_t ai = (size_t)sh.nd * sh.mp * sh.kp, bi = (size_t)sh.nd * sh.np * sh.kp;
    for (size_t q = 0; q < members.size(); ++q) {
        BatchProd &p = P[members[q]];
        oz_operand_images(ctx, p.A, p.B, p.si.g, sh, im.rexp.as<int>() + im.roff[q], im.cexp.as<int>() + im.coff[q],
                          im.aimg.as<bf16>() + (size_t)im.abase[q] * ai, im.bimg.as<bf16>() + (size_t)im.bbase[q] * bi);
    }
}

// allocates the group's buffers and computes them
static void class_images(bsg_ctx ctx, std::vector<BatchProd> &P, const std::vector<size_t> &members,
                         const OzShape &sh, ClassImages &im) {
    cudaStream_t s = ctx->stream;
    size_t nr = 0, nc = 0, na = 0, nb = 0;
    for (size_t m : members) {
        const ScreenGeom &g = P[m].si.g;
        im.roff.push_back(nr);
        im.coff.push_back(nc);
        im.abase.push_back((uint32_t)na);
        im.bbase.push_back((uint32_t)nb);
        nr += g.nib * g.ibs;
        nc += g.njb * g.jbs;
        na += P[m].A->nblocks();
        nb += P[m].B->nblocks();
    }
    BSG_REQUIRE(na < 0xffffffffull && nb < 0xffffffffull, BSG_ERR_UNSUPPORTED, "too many blocks in one batch group");
    const size_t ai = (size_t)sh.nd * sh.mp * sh.kp, bi = (size_t)sh.nd * sh.np * sh.kp;
    im.rexp = DevBuf(std::max<size_t>(nr, 1) * 4, s);
    im.cexp = DevBuf(std::max<size_t>(nc, 1) * 4, s);
    im.aimg = DevBuf(std::max<size_t>(na, 1) * ai * 2, s);
    im.bimg = DevBuf(std::max<size_t>(nb, 1) * bi * 2, s);
    class_images_compute(ctx, P, members, sh, im);
}

// tiles of every member (scratch: trial runs write scratch blocks)
static void class_tiles(bsg_ctx ctx, std::vector<BatchProd> &P, ClassRun &cr, const ClassImages &im, bool all_fresh,
                        double *scratch, uint64_t step_base = 0) {
    cr.tp = OzTilePlan();
    cr.tile0.clear();
    uint64_t steps = step_base;
    size_t scratch_items = 0;
    for (size_t q = 0; q < cr.prods.size(); ++q) {
        BatchProd &p = P[cr.prods[q]];
        cr.tile0.push_back(cr.tp.tiles.size());
        const size_t before = cr.tp.tiles.size();
        oz_build_tiles(ctx, p.si, cr.sh, im.rexp.as<int>() + im.roff[q], im.cexp.as<int>() + im.coff[q],
                       (uint32_t)steps, all_fresh,
                       scratch ? scratch + scratch_items * p.si.g.ibs * p.si.g.jbs : nullptr, cr.tp);
        steps += (uint64_t)(cr.tp.tiles.size() - before) * p.si.g.nkb;
        scratch_items += (size_t)(cr.tp.tiles.size() - before) * cr.sh.R;
        BSG_REQUIRE(steps < 0xffffffffull, BSG_ERR_UNSUPPORTED, "too many Ozaki steps in one batch group");
    }
    cr.tile0.push_back(cr.tp.tiles.size());
}

static uint64_t class_steps(const std::vector<BatchProd> &P, const ClassRun &cr) {
    uint64_t n = 0;
    for (size_t q = 0; q < cr.prods.size(); ++q) n += (uint64_t)(cr.tile0[q + 1] - cr.tile0[q]) * P[cr.prods[q]].si.g.nkb;
    return n;
}

// device copies of a group's tile lists (the tiles' step counts are filled
// in by the step kernel, so a replay starts from these)
struct ClassLists {
    DevBuf tiles, tib, tjb;
};
static void class_upload(bsg_ctx ctx, const ClassRun &cr, ClassLists &L) {
    cudaStream_t s = ctx->stream;
    const size_t nt = cr.tp.tiles.size();
    L.tiles = DevBuf(std::max<size_t>(nt, 1) * sizeof(OzTile), s);
    L.tib = DevBuf(std::max<size_t>(cr.tp.tib.size(), 1) * 4, s);
    L.tjb = DevBuf(std::max<size_t>(nt, 1) * 4, s);
    if (!nt) return;
    BSG_CUDA(cudaMemcpyAsync(L.tiles.p, cr.tp.tiles.data(), nt * sizeof(OzTile), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(L.tib.p, cr.tp.tib.data(), cr.tp.tib.size() * 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(L.tjb.p, cr.tp.tjb.data(), nt * 4, cudaMemcpyHostToDevice, s));
}

// enqueues steps + the persistent launch of one group (no synchronization;
// with `lists` the tile lists are already on the device)
static void class_launch(bsg_ctx ctx, std::vector<BatchProd> &P, const ClassRun &cr, const ClassImages &im,
                         double alpha, const ClassLists *lists = nullptr) {
    cudaStream_t s = ctx->stream;
    const size_t nt = cr.tp.tiles.size();
    if (!nt) return;
    ClassLists own;
    if (!lists) {
        class_upload(ctx, cr, own);
        lists = &own;
    }
    DevBuf dst(std::max<uint64_t>(class_steps(P, cr), 1) * sizeof(OzStep), s), dmacs(8, s);
    BSG_CUDA(cudaMemsetAsync(dmacs.p, 0, 8, s));
    OzTile *dtl = const_cast<OzTile *>(lists->tiles.as<OzTile>());
    const uint32_t *dib = lists->tib.as<uint32_t>(), *djb = lists->tjb.as<uint32_t>();
    for (size_t q = 0; q < cr.prods.size(); ++q) {
        BatchProd &p = P[cr.prods[q]];
        const size_t t0 = cr.tile0[q], t1 = cr.tile0[q + 1];
        oz_launch_steps(ctx, dtl + t0, t1 - t0, dib + t0 * kOzMaxSlots, djb + t0, p.A, p.B, p.si.g, cr.sh.R,
                        dst.as<OzStep>(), dmacs.as<unsigned long long>(), im.abase[q], im.bbase[q]);
    }
    oz_run(ctx, cr.sh, dtl, nt, dst.as<OzStep>(), im.aimg.as<bf16>(), im.bimg.as<bf16>(), alpha, s,
           dmacs.as<unsigned long long>());
}

// The tiles of groups [c0, c1) of a batch in one list, group after group
// (step indices continue from group to group), uploaded once.
struct BatchLists {
    DevBuf tiles, tib, tjb;
    size_t c0 = 0, c1 = 0;
    std::vector<size_t> tile0;  // first tile of each group, then the total
    uint64_t steps = 0;
};
constexpr size_t kGroupsPerLaunch = 8;  // tile geometries one launch can hold

static void batch_tiles(bsg_ctx ctx, std::vector<BatchProd> &P, std::vector<ClassRun> &classes,
                        const std::vector<ClassImages> &ims, size_t c0, size_t c1, bool all_fresh, BatchLists &L) {
    cudaStream_t s = ctx->stream;
    L.c0 = c0;
    L.c1 = c1;
    L.tile0.clear();
    L.steps = 0;
    std::vector<OzTile> tiles;
    std::vector<uint32_t> tib, tjb;
    for (size_t c = c0; c < c1; ++c) {
        ClassRun &cr = classes[c];
        class_tiles(ctx, P, cr, ims[c], all_fresh, nullptr, L.steps);
        L.tile0.push_back(tiles.size());
        tiles.insert(tiles.end(), cr.tp.tiles.begin(), cr.tp.tiles.end());
        tib.insert(tib.end(), cr.tp.tib.begin(), cr.tp.tib.end());
        tjb.insert(tjb.end(), cr.tp.tjb.begin(), cr.tp.tjb.end());
        L.steps += class_steps(P, cr);
        BSG_REQUIRE(L.steps < 0xffffffffull, BSG_ERR_UNSUPPORTED, "too many Ozaki steps in one batch launch");
    }
    L.tile0.push_back(tiles.size());
    const size_t nt = tiles.size();
    L.tiles = DevBuf(std::max<size_t>(nt, 1) * sizeof(OzTile), s);
    L.tib = DevBuf(std::max<size_t>(tib.size(), 1) * 4, s);
    L.tjb = DevBuf(std::max<size_t>(nt, 1) * 4, s);
    if (!nt) return;
    BSG_CUDA(cudaMemcpyAsync(L.tiles.p, tiles.data(), nt * sizeof(OzTile), cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(L.tib.p, tib.data(), tib.size() * 4, cudaMemcpyHostToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(L.tjb.p, tjb.data(), nt * 4, cudaMemcpyHostToDevice, s));
    // the host vectors are released on return: they must be copied first
    BSG_CUDA(cudaStreamSynchronize(s));
}

// steps of every tile of the list, then one persistent launch over all of
// them (no synchronization)
static void batch_launch(bsg_ctx ctx, std::vector<BatchProd> &P, const std::vector<ClassRun> &classes,
                         const std::vector<ClassImages> &ims, const BatchLists &L, double alpha) {
    cudaStream_t s = ctx->stream;
    const size_t nt = L.tile0.back();
    if (!nt) return;
    DevBuf dst(std::max<uint64_t>(L.steps, 1) * sizeof(OzStep), s), dmacs(8, s);
    BSG_CUDA(cudaMemsetAsync(dmacs.p, 0, 8, s));
    OzTile *dtl = const_cast<OzTile *>(L.tiles.as<OzTile>());
    const uint32_t *dib = L.tib.as<uint32_t>(), *djb = L.tjb.as<uint32_t>();
    std::vector<OzRun> runs;
    for (size_t c = L.c0; c < L.c1; ++c) {
        const ClassRun &cr = classes[c];
        const size_t T0 = L.tile0[c - L.c0];
        for (size_t q = 0; q < cr.prods.size(); ++q) {
            BatchProd &p = P[cr.prods[q]];
            const size_t t0 = T0 + cr.tile0[q], t1 = T0 + cr.tile0[q + 1];
            oz_launch_steps(ctx, dtl + t0, t1 - t0, dib + t0 * kOzMaxSlots, djb + t0, p.A, p.B, p.si.g, cr.sh.R,
                            dst.as<OzStep>(), dmacs.as<unsigned long long>(), ims[c].abase[q], ims[c].bbase[q]);
        }
        runs.push_back(OzRun{cr.sh, ims[c].aimg.as<bf16>(), ims[c].bimg.as<bf16>(), L.tile0[c - L.c0 + 1]});
    }
    oz_run_groups(ctx, runs, dtl, nt, dst.as<OzStep>(), alpha, s, dmacs.as<unsigned long long>());
}

// picks (slots per tile, stages) for the group's shape: cached, or timed on
// the group's own tiles writing scratch blocks
static void class_tune(bsg_ctx ctx, std::vector<BatchProd> &P, ClassRun &cr, const ClassImages &im, double alpha) {
    const std::array<int, 4> key{cr.sh.mp, cr.sh.kp, cr.sh.np, cr.sh.nd};
    auto it = ctx->oz_tune.find(key);
    if (it != ctx->oz_tune.end()) {
        cr.sh.R = it->second[0];
        cr.sh.S = it->second[1];
        return;
    }
    const int Rmax = cr.sh.R;
    if (!ctx->autotune) return;
    size_t items = 0;
    for (size_t m : cr.prods) items += P[m].si.items.size();
    if (!items) return;
    cudaStream_t s = ctx->stream;
    // candidates: full or half tile height, as many stages as fit or two
    std::vector<std::array<int, 2>> cand{{Rmax, 0}, {Rmax, 2}, {(Rmax + 1) / 2, 0}, {(Rmax + 1) / 2, 2}};
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    const size_t blk = (size_t)P[cr.prods[0]].si.g.ibs * P[cr.prods[0]].si.g.jbs;
    DevBuf scratch(items * (size_t)Rmax * blk * 8 + 8, s);  // at most one scratch block per slot of every tile
    cudaEvent_t e0, e1;
    BSG_CUDA(cudaEventCreate(&e0));
    BSG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    std::array<int, 2> pick{Rmax, 0};
    for (auto &c : cand) {
        ClassRun trial = cr;
        trial.sh.R = c[0];
        trial.sh.S = c[1];
        class_tiles(ctx, P, trial, im, true, scratch.as<double>());
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {  // first run warms caches and the launch
            BSG_CUDA(cudaEventRecord(e0, s));
            class_launch(ctx, P, trial, im, alpha);
            BSG_CUDA(cudaEventRecord(e1, s));
            ctx->gemm_check();
            BSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        }
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->oz_tune[key] = pick;
    cr.sh.R = pick[0];
    cr.sh.S = pick[1];
}

// groups of the batch's products by block sizes (mixed form)
static std::vector<ClassRun> make_classes(std::vector<BatchProd> &P, int n_digits) {
    std::vector<ClassRun> out;
    std::vector<std::array<int, 3>> keys;
    for (size_t i = 0; i < P.size(); ++i) {
        const ScreenGeom &g = P[i].si.g;
        if (P[i].si.items.empty()) continue;
        BSG_REQUIRE(g.ibs <= 64 && g.jbs <= 64 && g.kbs <= 64, BSG_ERR_UNSUPPORTED,
                    "Ozaki form supports blocks up to 64");
        const std::array<int, 3> k{(int)g.ibs, (int)g.kbs, (int)g.jbs};
        size_t c = std::find(keys.begin(), keys.end(), k) - keys.begin();
        if (c == keys.size()) {
            keys.push_back(k);
            ClassRun cr;
            const int nd = oz_default_digits(n_digits, k[0], k[1], k[2]);
            cr.sh = oz_shape(k[0], k[1], k[2], nd);
            out.push_back(std::move(cr));
        }
        out[c].prods.push_back(i);
    }
    return out;
}

static std::vector<BatchProd> screen_batch(size_t n, const bsg_bsm *C, const bsg_bsm *A, const bsg_bsm *B,
                                           double thresh, double beta, uint64_t *nsig) {
    BSG_REQUIRE(n == 0 || (C && A && B), BSG_ERR_ARG, "NULL operand arrays");
    std::vector<BatchProd> P(n);
    uint64_t tot = 0;
    bsg_ctx ctx = n ? A[0]->ctx : nullptr;
    for (size_t i = 0; i < n; ++i) {
        BSG_REQUIRE(C[i] && A[i] && B[i], BSG_ERR_ARG, "NULL matrix in the batch");
        BSG_REQUIRE(A[i]->ctx == ctx, BSG_ERR_ARG, "batch on several contexts");
        P[i].C = C[i];
        P[i].A = A[i];
        P[i].B = B[i];
        P[i].si = screen_items(ctx, C[i], A[i], 0, B[i], 0, thresh, beta);
        tot += P[i].si.total;
    }
    if (nsig) *nsig = tot;
    return P;
}

}  // namespace bsg

using namespace bsg;

extern "C" bsg_status bsg_matmult_batched(size_t n, const bsg_bsm *C, const bsg_bsm *A, const bsg_bsm *B,
                                          double thresh, double alpha, double beta, int form, int n_digits,
                                          uint64_t *nsig_total) {
    return guard([&] {
        BSG_REQUIRE(form == BSG_FORM_FP64 || form == BSG_FORM_OZAKI, BSG_ERR_ARG, "unknown form");
        if (form == BSG_FORM_FP64) {
            uint64_t tot = 0;
            for (size_t i = 0; i < n; ++i) {
                BSG_REQUIRE(C && A && B && C[i] && A[i] && B[i], BSG_ERR_ARG, "NULL matrix in the batch");
                tot += screened_product(C[i]->ctx, {C[i]}, {A[i]}, 0, {B[i]}, 0, {{0, 1}}, thresh, alpha, beta,
                                        BSG_FORM_FP64, 0);
            }
            if (nsig_total) *nsig_total = tot;
            return;
        }
        std::vector<BatchProd> P = screen_batch(n, C, A, B, thresh, beta, nsig_total);
        if (P.empty()) return;
        bsg_ctx ctx = A[0]->ctx;
        std::vector<ClassRun> classes = make_classes(P, n_digits);
        std::vector<ClassImages> ims(classes.size());
        for (size_t c = 0; c < classes.size(); ++c) {
            class_images(ctx, P, classes[c].prods, classes[c].sh, ims[c]);
            class_tune(ctx, P, classes[c], ims[c], alpha);
        }
        for (size_t c0 = 0; c0 < classes.size(); c0 += kGroupsPerLaunch) {
            BatchLists L;
            batch_tiles(ctx, P, classes, ims, c0, std::min(classes.size(), c0 + kGroupsPerLaunch), false, L);
            batch_launch(ctx, P, classes, ims, L, alpha);
        }
        ctx->gemm_check();
    });
}

// A captured batch: the device work (exponents, digit images, step lists,
// one persistent launch over every block-size group) of C_i = alpha A_i B_i
// as a CUDA graph.  The C block structure is fixed when the plan is made (beta 0:
// every output block is overwritten); a replay recomputes everything from the
// operands' current values and cached norms.
struct bsg_batch_plan_s {
    bsg_ctx ctx = nullptr;
    std::vector<BatchProd> prods;
    std::vector<ClassRun> classes;
    std::vector<ClassImages> images;  // exponents and digit images the tiles point into
    std::vector<BatchLists> lists;    // device tile lists the graph reads (up to 8 groups each)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t nsig = 0;
    ~bsg_batch_plan_s() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (ctx) ctx_release(ctx);
    }
};

extern "C" bsg_status bsg_batched_plan_create(size_t n, const bsg_bsm *C, const bsg_bsm *A, const bsg_bsm *B,
                                              double thresh, double alpha, int n_digits, bsg_batch_plan *out) {
    return guard([&] {
        BSG_REQUIRE(out && n > 0, BSG_ERR_ARG, "empty batch or NULL output");
        auto plan = std::make_unique<bsg_batch_plan_s>();
        plan->prods = screen_batch(n, C, A, B, thresh, 0.0, &plan->nsig);
        bsg_ctx ctx = A[0]->ctx;
        ctx_retain(ctx);
        plan->ctx = ctx;
        plan->classes = make_classes(plan->prods, n_digits);
        // buffers the plan owns; tune and run once outside the capture
        // (first-use initialisation, and the plan's own first result)
        const size_t nc = plan->classes.size();
        plan->images.resize(nc);
        for (size_t c = 0; c < nc; ++c) {
            ClassRun &cr = plan->classes[c];
            class_images(ctx, plan->prods, cr.prods, cr.sh, plan->images[c]);
            class_tune(ctx, plan->prods, cr, plan->images[c], alpha);
        }
        plan->lists.resize((nc + kGroupsPerLaunch - 1) / kGroupsPerLaunch);
        for (size_t k = 0; k < plan->lists.size(); ++k) {
            batch_tiles(ctx, plan->prods, plan->classes, plan->images, k * kGroupsPerLaunch,
                        std::min(nc, (k + 1) * kGroupsPerLaunch), true, plan->lists[k]);
            batch_launch(ctx, plan->prods, plan->classes, plan->images, plan->lists[k], alpha);
        }
        ctx->gemm_check();
        ctx->gemm_err_flag();  // allocated and armed before the capture
        cudaStream_t s = ctx->stream;
        BSG_CUDA(cudaStreamSynchronize(s));
        BSG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
            for (size_t c = 0; c < nc; ++c) {
                ClassRun &cr = plan->classes[c];
                class_images_compute(ctx, plan->prods, cr.prods, cr.sh, plan->images[c]);
            }
            for (const BatchLists &L : plan->lists)
                batch_launch(ctx, plan->prods, plan->classes, plan->images, L, alpha);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        BSG_CUDA(cudaStreamEndCapture(s, &plan->graph));
        BSG_CUDA(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
        ctx->gemm_check();
        *out = plan.release();
    });
}

extern "C" bsg_status bsg_batched_plan_run(bsg_batch_plan plan) {
    return guard([&] {
        BSG_REQUIRE(plan && plan->exec, BSG_ERR_ARG, "NULL plan");
        bsg_ctx ctx = plan->ctx;
        ctx->gemm_err_flag();
        BSG_CUDA(cudaGraphLaunch(plan->exec, ctx->stream));
        ctx->note_launch();
        ctx->gemm_check();
    });
}

extern "C" bsg_status bsg_batched_plan_destroy(bsg_batch_plan plan) {
    return guard([&] { delete plan; });
}

extern "C" bsg_status bsg_ctx_set_autotune(bsg_ctx ctx, int on) {
    return guard([&] {
        BSG_REQUIRE(ctx, BSG_ERR_ARG, "ctx is NULL");
        ctx->autotune = on != 0;
        if (on < 0) ctx->oz_tune.clear();
    });
}

extern "C" bsg_status bsg_ctx_autotune_entries(bsg_ctx ctx, int *entries, int cap, int *n) {
    return guard([&] {
        BSG_REQUIRE(ctx && n, BSG_ERR_ARG, "NULL argument");
        *n = (int)ctx->oz_tune.size();
        int i = 0;
        for (auto &kv : ctx->oz_tune) {
            if (i >= cap || !entries) break;
            int *e = entries + 6 * i;
            e[0] = kv.first[0];
            e[1] = kv.first[1];
            e[2] = kv.first[2];
            e[3] = kv.first[3];
            e[4] = kv.second[0];
            e[5] = kv.second[1];
            ++i;
        }
    });
}
