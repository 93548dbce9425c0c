// 3c->2c transform (3c_2c_transform.cpp:44-57), Ozaki form, on dense device
// operands: out = X * V^{-1/2} over the block triples that survive
// ||X_ik|| ||V_kj|| >= thresh*bs^3, written straight into the dense output.
//
// The reference builds block-sparse copies of both inputs at threshold 0
// (every block kept), pre-fills the output with zeros and accumulates; this
// path computes the same block norms (the deterministic 32-lane order), the
// same screen, and writes each output block as the sum of its surviving
// products (blocks without any are written as zeros) -- no block pool, no
// host loops over blocks.
#include <algorithm>

#include "bsg_ozaki.cuh"

namespace bsg {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ int ext3(size_t blk, size_t bs, size_t n) {
    return (int)(((blk + 1) * bs <= n) ? bs : n - blk * bs);
}

// one warp per block of a dense column-major matrix: deterministic norm
__global__ void k_dense_norms(const double *__restrict__ M, size_t ld, size_t nr, size_t nc, size_t bs, size_t nrb,
                              size_t nblk, double *__restrict__ norm) {
    const size_t b = (size_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (b >= nblk) return;
    const size_t rb = b % nrb, cb = b / nrb;
    const double est = warp_block_norm(M + rb * bs + cb * bs * ld, ext3(rb, bs, nr), ext3(cb, bs, nc), ld);
    if ((threadIdx.x & 31) == 0) norm[b] = est;
}

// block norms of X (the deterministic order) and the blocks' row maxima
// folded into row_bits (bit patterns of |x|, atomicMax), one pass;
// kNormBlocks consecutive blocks per warp, their norms finished from the
// warp's table of chains (norm_from_chains), kXnWarps warps per CTA
constexpr int kXnWarps = 8;
__global__ void k_xnorm_rowmax(const double *__restrict__ X, size_t ld, size_t nr, size_t nc, size_t bs, size_t nrb,
                               size_t nblk, double *__restrict__ norm, unsigned long long *__restrict__ row_bits) {
    __shared__ NormTable tab[kXnWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t b0 = ((size_t)blockIdx.x * kXnWarps + w) * kNormBlocks;
    if (b0 >= nblk) return;
    const int nq = (int)min((size_t)kNormBlocks, nblk - b0);
    for (int q = 0; q < nq; ++q) {
        const size_t b = b0 + q, rb = b % nrb, cb = b / nrb;
        const int rows = ext3(rb, bs, nr), cols = ext3(cb, bs, nc);
        const double *M = X + rb * bs + cb * bs * ld;
        tab[w][q][lane] = warp_norm_chain(M, rows, cols, ld);
        for (int r = lane; r < rows; r += 32) {
            long long mx = 0;
            for (int l = 0; l < cols; ++l) {
                const long long v = oz_absbits(M[r + (size_t)l * ld]);
                mx = v > mx ? v : mx;
            }
            if (mx) atomicMax(&row_bits[rb * bs + r], (unsigned long long)mx);
        }
    }
    __syncwarp();
    if (lane < nq) norm[b0 + lane] = norm_from_chains(tab[w][lane]);
}

// exponent of every column of V (over all rows); one block per column
__global__ void k_colexp_dense(const double *__restrict__ V, size_t nr, int *__restrict__ cexp) {
    const size_t c = blockIdx.x;
    long long mx = 0;
    for (size_t r = threadIdx.x; r < nr; r += blockDim.x) {
        const long long b = oz_absbits(V[r + c * nr]);
        mx = b > mx ? b : mx;
    }
    for (int o = 16; o >= 1; o >>= 1) {
        const long long other = __shfl_down_sync(0xffffffffu, mx, o);
        mx = other > mx ? other : mx;
    }
    __shared__ long long wmax[32];
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long m = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = wmax[w] > m ? wmax[w] : m;
        cexp[c] = oz_exp_of_bits(m);
    }
}

struct Dense3c {
    size_t n_vec2, n_aux, bs, nib, nkb, njb;
    size_t ldx, ldo;  // leading dimensions of X and of the output
    int mp, kp, np, nd, R;
    int J;        // X block rows per N-side group (np = J * bs rounded to 8)
    size_t nibp;  // groups of J block rows
};

// The tile is transposed with respect to the output: its slots (the MMA's M
// side) are R output block columns jb, fed by V^T blocks, and its columns
// (the N side) one output block row ib, fed by the X block of each k step.
// V^{-1/2} has no block locality, so whether a triple survives the screen is
// decided by ||X_ib,kb|| for all R slots alike and a step's slots are nearly
// always all live; with block rows as slots a step would carry the
// insignificant X blocks of its other rows as zero images.

// The screen ||X_ib,kb|| ||V_kb,jb|| >= tpb keeps no product of block
// (ib, kb) of X in any tile when it fails for the largest ||V_kb,jb|| of the
// k step (a correctly rounded product is monotone in each factor), so the
// test against vmax[kb] decides it for every slot at once.
__device__ __forceinline__ bool x_block_dead(double xn, double vmax, double tpb) { return !(__dmul_rn(xn, vmax) >= tpb); }

// vmax[kb] = max over jb of ||V_kb,jb|| (vn column-major, nkb rows)
__global__ void k_vn_rowmax(const double *__restrict__ vn, size_t nkb, size_t njb, double *__restrict__ vmax) {
    const size_t kb = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= nkb) return;
    double m = 0.0;
    for (size_t jb = 0; jb < njb; ++jb) m = fmax(m, vn[kb + jb * nkb]);
    vmax[kb] = m;
}

// N-side images of X: J consecutive block rows stacked along N, one image
// per (group ibp, kb), index ibp*nkb + kb (a group's k steps back to back, so
// that the two steps of a stage pair are one copy); block ib = J*ibp + j
// fills rows j*bs.. of its group's image (rows of missing blocks are never
// read).  A block that the screen drops in every tile gets an all-zero
// image where the other block row of its group survives: a step may then
// copy the group's whole image (one copy) and the MMA adds exact zeros for
// it.  Where neither survives, no step reads the image and it is not written.
// kImgXBlocks consecutive blocks x = ib + kb*nib per warp.
constexpr int kImgXBlocks = 4;
__global__ void k_img_X(const double *__restrict__ X, const int *__restrict__ rexp, const double *__restrict__ xn,
                        const double *__restrict__ vmax, double tpb, Dense3c D, bf16 *__restrict__ img) {
    __shared__ OzImgJob sj[kOzImgWarps][kImgXBlocks];
    const size_t x0 = oz_warp_id() * kImgXBlocks, n = D.nib * D.nkb;
    if (x0 >= n) return;
    oz_jobs_image(
        kImgXBlocks,
        [&](int q, OzImgJob &J) {
            const size_t x = x0 + q;
            if (x >= n) return false;
            const size_t ib = x % D.nib, kb = x / D.nib, ibp = ib / D.J, j = ib % D.J;
            bool zero = false;
            if (x_block_dead(xn[x], vmax[kb], tpb)) {
                // zeros where the group's other block row survives (else no step reads the image)
                const size_t iq = ibp * D.J + (1 - j);
                if (D.J != 2 || iq >= D.nib || x_block_dead(xn[iq + kb * D.nib], vmax[kb], tpb)) return false;
                zero = true;
            }
            J.get = OzDenseGet{X + ib * D.bs + kb * D.bs * D.ldx, D.ldx, false};
            J.rows = zero ? 0 : ext3(ib, D.bs, D.n_vec2);  // 0 rows: all digits zero
            J.k = ext3(kb, D.bs, D.n_aux);
            J.exps = rexp + ib * D.bs;
            J.dst = img + (ibp * D.nkb + kb) * D.nd * (size_t)D.np * D.kp + j * D.bs * (size_t)D.kp;
            J.m_side = false;
            J.plane_rows = D.np;
            return true;
        },
        (int)D.bs, D.kp, D.nd, sj[threadIdx.x >> 5]);
}

// M-side images of V^T blocks (jb, kb): image row = output column, index
// (jg*nkb + kb)*R + s for jb = jg*R + s (a tile's slots are consecutive
// images, and so are the slots of consecutive k steps)
__global__ void k_img_V(const double *__restrict__ V, const int *__restrict__ cexp, Dense3c D, bf16 *__restrict__ img) {
    const size_t x = oz_warp_id();
    if (x >= D.nkb * D.njb) return;
    const size_t jb = x % D.njb, kb = x / D.njb;
    const size_t idx = ((jb / D.R) * D.nkb + kb) * D.R + jb % D.R;
    oz_block_image(V + kb * D.bs + jb * D.bs * D.n_aux, D.n_aux, true, ext3(jb, D.bs, D.n_aux), ext3(kb, D.bs, D.n_aux),
                   cexp + jb * D.bs, D.mp, D.kp, D.nd, img + idx * D.nd * (size_t)D.mp * D.kp, true);
}

// tiles and their steps; tile t covers output block rows J*ibp .. J*ibp+J-1
// (N side) and block columns jg*R .. jg*R+R-1 (slots).  Order: column groups
// of Gj slot groups (their V^T images, Gj*R*nkb of them, stay resident in
// L2), within a group every block-row group with its Gj tiles together.
// A step k carries the slots and N-side sub-blocks of a rectangle of
// surviving (slot, sub-block) pairs: whether (jb, ib, kb) survives is
// ||X_ib,kb|| ||V_kb,jb|| >= tpb, so for fixed kb the slot sets of the
// sub-blocks are nested and split into at most J exact rectangles.
__global__ void k_tiles_3c(size_t n_tiles, size_t n_jg, size_t Gj, const double *__restrict__ xn,
                           const double *__restrict__ vn, const double *__restrict__ vmax,
                           const int *__restrict__ rexp, const int *__restrict__ cexp,
                           double *__restrict__ out, Dense3c D, double tpb, OzTile *__restrict__ tiles,
                           OzStep *__restrict__ steps, unsigned long long *__restrict__ nsig,
                           unsigned long long *__restrict__ macs) {
    const size_t t = oz_warp_id();  // one warp per tile, lanes over the k steps
    if (t >= n_tiles) return;
    const int lane = threadIdx.x & 31;
    const size_t q = t / (D.nibp * Gj), rem = t % (D.nibp * Gj);
    const size_t gsz = min(Gj, n_jg - q * Gj);  // only the last group is smaller
    const size_t ibp = rem / gsz, jg = q * Gj + rem % gsz;
    OzTile T;
    for (int s = 0; s < kOzMaxSlots; ++s) {
        T.c[s] = nullptr;
        T.cnorm[s] = nullptr;
        T.rexp[s] = nullptr;
        T.rows[s] = 0;
        T.ldc[s] = 0;
    }
    int nsub = 0, rows = 0, sub_rows[8];
    for (int j = 0; j < D.J && ibp * D.J + j < D.nib; ++j) {
        sub_rows[j] = ext3(ibp * D.J + j, D.bs, D.n_vec2);
        rows += sub_rows[j];
        ++nsub;
    }
    for (int s = 0; s < D.R; ++s) {
        const size_t jb = jg * D.R + s;
        if (jb >= D.njb) break;
        T.c[s] = out + ibp * D.J * D.bs + jb * D.bs * D.ldo;
        T.ldc[s] = (int)D.ldo;
        T.rows[s] = ext3(jb, D.bs, D.n_aux);  // slot rows are output columns
        T.rexp[s] = cexp + jb * D.bs;
    }
    T.cols = rows;  // tile columns are output rows (J consecutive block rows)
    T.cexp = rexp + ibp * D.J * D.bs;
    T.trans = 1;
    T.fresh_mask = 0xFFu;  // out = 0 + sum of the surviving products
    T.s0 = (uint32_t)(t * D.nkb * D.J);
    uint32_t n = 0;
    unsigned long long cnt = 0, m = 0;
    for (size_t base = 0; base < D.nkb; base += 32) {
        const size_t kb = base + lane;
        OzStep mine[2];
        uint32_t c = 0;
        if (kb < D.nkb) {
            uint32_t live[2] = {0, 0}, phantom = 0;
            for (int j = 0; j < nsub; ++j) {
                const double x = xn[ibp * D.J + j + kb * D.nib];
                // a block dropped in every tile has a zero image: its
                // sub-block may ride along in a whole-image copy (and no slot
                // needs a test)
                if (x_block_dead(x, vmax[kb], tpb)) {
                    phantom |= 1u << j;
                    continue;
                }
                for (int s = 0; s < D.R; ++s) {
                    const size_t jb = jg * D.R + s;
                    if (jb >= D.njb) break;
                    if (__dmul_rn(x, vn[kb + jb * D.nkb]) >= tpb) {
                        live[j] |= 1u << s;
                        ++cnt;
                        m += (unsigned long long)sub_rows[j] * T.rows[s] * ext3(kb, D.bs, D.n_aux);
                    }
                }
            }
            uint32_t a_idx[kOzMaxSlots];
            for (int s = 0; s < kOzMaxSlots; ++s) a_idx[s] = (uint32_t)((jg * D.nkb + kb) * D.R + s);
            // exact rectangles (the slot sets of a norm-product screen are nested)
            c = emit_rect_steps(live, D.J, phantom, (uint32_t)(ibp * D.nkb + kb), a_idx, mine);
        }
        warp_append_steps(mine, c, steps + T.s0, n);
    }
    cnt = warp_sum_u64(cnt);
    m = warp_sum_u64(m);
    if (lane == 0) {
        T.ns = n;
        tiles[t] = T;
        if (cnt) atomicAdd(nsig, cnt);
        if (m) atomicAdd(macs, m);
    }
}

namespace {

// V-side operands (block norms, column exponents, M-side digit images of
// V^T), shared by every row range of X
struct Oz3cV {
    DevBuf vn, vmax, cexp, ai;
};

Dense3c oz3c_dims(size_t n_aux, size_t bs, int nd, OzShape &sh) {
    // X block rows per tile on the N side.  Two rows (nd * 2*bs TMEM columns,
    // bs % 8 == 0) halve the shared-memory bytes of the V^T operand per
    // product; 35% of the steps split into two rectangles (the rows' screens
    // differ).  Measured on the 40-atom workload: 5 digits 34.1 ms with two
    // rows against 36.2 with one; 6 digits 41.1 against 39.5 (the two
    // accumulator sets no longer fit TMEM together), so two rows only where
    // both sets fit.
    int J = (bs % 8 == 0 && 2 * bs <= 64 && nd * 2 * (int)bs + 8 <= 256) ? 2 : 1;
    sh = oz_shape((int)bs, (int)bs, (int)bs * J, nd);
    if (J == 2) {  // the V^T images are laid out for the one-row shape's k steps
        const OzShape s1 = oz_shape((int)bs, (int)bs, (int)bs, nd);
        if (s1.kp != sh.kp || s1.pair != sh.pair) {
            J = 1;
            sh = s1;
        }
    }
    sh.J = J;
    Dense3c D;
    D.n_vec2 = D.ldx = D.ldo = 0;
    D.n_aux = n_aux;
    D.bs = bs;
    D.nib = D.nibp = 0;
    D.nkb = D.njb = ceil_div(n_aux, bs);
    D.mp = sh.mp;
    D.kp = sh.kp;
    D.np = sh.np;
    D.nd = nd;
    D.R = sh.R;
    D.J = J;
    return D;
}

void oz3c_prepare_v(bsg_ctx ctx, const double *V, const Dense3c &D, Oz3cV &v) {
    cudaStream_t s = ctx->stream;
    const size_t n_aux = D.n_aux, a_img = (size_t)D.nd * D.mp * D.kp;
    v.vn = DevBuf(D.nkb * D.njb * 8, s);
    v.cexp = DevBuf(n_aux * 4, s);
    v.ai = DevBuf(ceil_div(D.njb, (size_t)D.R) * D.R * D.nkb * a_img * 2, s);  // whole slot groups
    const int wpb = 8;
    k_dense_norms<<<(unsigned)ceil_div(D.nkb * D.njb, wpb), wpb * 32, 0, s>>>(V, n_aux, n_aux, n_aux, D.bs, D.nkb,
                                                                              D.nkb * D.njb, v.vn.as<double>());
    v.vmax = DevBuf(D.nkb * 8, s);
    k_vn_rowmax<<<(unsigned)ceil_div(D.nkb, (size_t)128), 128, 0, s>>>(v.vn.as<double>(), D.nkb, D.njb,
                                                                      v.vmax.as<double>());
    k_colexp_dense<<<(unsigned)n_aux, 256, 0, s>>>(V, n_aux, v.cexp.as<int>());
    k_img_V<<<oz_img_grid(D.nkb * D.njb), 32 * kOzImgWarps, 0, s>>>(V, v.cexp.as<int>(), D, v.ai.as<bf16>());
    ctx->note_launch(4);
    ctx->check_launch("3c2c ozaki V prep");
}

// rows [0, rows) of X (leading dimension ldx) into the same rows of out
// (leading dimension ldo); stream-ordered on the context's stream, no sync
void oz3c_rows(bsg_ctx ctx, Dense3c D, const OzShape &sh, const Oz3cV &v, const double *X, size_t ldx, size_t rows,
               double *out, size_t ldo, double thresh, unsigned long long *cnt) {
    cudaStream_t s = ctx->stream;
    const size_t bs = D.bs, n_aux = D.n_aux;
    D.n_vec2 = rows;
    D.ldx = ldx;
    D.ldo = ldo;
    D.nib = ceil_div(rows, bs);
    D.nibp = ceil_div(D.nib, (size_t)D.J);
    const size_t a_img = (size_t)D.nd * sh.mp * sh.kp, b_img = (size_t)D.nd * sh.np * sh.kp;
    DevBuf xn(D.nib * D.nkb * 8, s), rexp(rows * 4, s), bi(D.nibp * D.nkb * b_img * 2, s);
    DevBuf rbits(rows * 8, s);
    BSG_CUDA(cudaMemsetAsync(rbits.p, 0, rows * 8, s));
    k_xnorm_rowmax<<<(unsigned)ceil_div(D.nib * D.nkb, (size_t)kXnWarps * kNormBlocks), kXnWarps * 32, 0, s>>>(
        X, ldx, rows, n_aux, bs, D.nib, D.nib * D.nkb, xn.as<double>(), rbits.as<unsigned long long>());
    k_bits_to_exp<<<(unsigned)ceil_div(rows, (size_t)256), 256, 0, s>>>(rbits.as<unsigned long long>(), rows,
                                                                        rexp.as<int>());
    const double tpb = thresh * (double)(bs * bs * bs);
    k_img_X<<<oz_img_grid(ceil_div(D.nib * D.nkb, (size_t)kImgXBlocks)), 32 * kOzImgWarps, 0, s>>>(
        X, rexp.as<int>(), xn.as<double>(), v.vmax.as<double>(), tpb, D, bi.as<bf16>());
    ctx->note_launch(3);
    ctx->check_launch("3c2c ozaki X prep");
    const size_t n_jg = ceil_div(D.njb, (size_t)D.R), n_tiles = D.nibp * n_jg;
    BSG_REQUIRE(n_tiles * D.nkb * D.J < 0xffffffffull, BSG_ERR_UNSUPPORTED, "too many Ozaki steps in one call");
    DevBuf dt(n_tiles * sizeof(OzTile), s), dst(n_tiles * D.nkb * D.J * sizeof(OzStep), s);
    // V^T images of one slot group: R * nkb images; keep about 48 MB of them in L2
    const size_t grp_bytes = (size_t)D.R * D.nkb * a_img * 2;
    const size_t Gj = std::max<size_t>(1, std::min<size_t>(n_jg, (48ull << 20) / std::max<size_t>(grp_bytes, 1)));
    k_tiles_3c<<<oz_img_grid(n_tiles), 32 * kOzImgWarps, 0, s>>>(n_tiles, n_jg, Gj, xn.as<double>(), v.vn.as<double>(),
                                                                v.vmax.as<double>(), rexp.as<int>(),
                                                                v.cexp.as<int>(), out, D, tpb,
                                                                dt.as<OzTile>(), dst.as<OzStep>(), cnt, cnt + 1);
    ctx->note_launch();
    ctx->check_launch("3c2c ozaki tiles");
    // tiles go round-robin (chunk 1): the Gj tiles of one block row run on
    // neighbouring CTAs at about the same time and share its X images in L2
    // (a chunk of Gj tiles per CTA puts 152 block rows in flight at once and
    // measured more DRAM traffic)
    oz_run(ctx, sh, dt.as<OzTile>(), n_tiles, dst.as<OzStep>(), v.ai.as<bf16>(), bi.as<bf16>(), 1.0, s, cnt + 1, 1);
}

// Rows [0, rows) of every column of a column-major host matrix (leading
// dimension ld, pinned and mapped into the device's address space) into a
// rows x ncols device buffer, read by the SMs over the host link: one CTA
// per column at a time, eight 16-byte loads in flight per thread.  The copy
// engine takes a strided copy one row of the 2D copy at a time, well below
// the link's rate; a handful of SMs reach it.  vec: every column start on
// both sides 16-byte aligned and rows even (else 8-byte loads).
__global__ void __launch_bounds__(1024) k_fetch_host_rows(const double *__restrict__ src, size_t ld, size_t rows,
                                                          size_t ncols, double *__restrict__ dst, int vec) {
    for (size_t c = blockIdx.x; c < ncols; c += gridDim.x) {
        const double *sc = src + c * ld;
        double *dc = dst + c * rows;
        if (vec) {
            const double2 *s2 = reinterpret_cast<const double2 *>(sc);
            double2 *d2 = reinterpret_cast<double2 *>(dc);
            const size_t n2 = rows / 2, step = blockDim.x;
            size_t i = threadIdx.x;
            for (; i + 7 * step < n2; i += 8 * step) {
                double2 v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = s2[i + u * step];
#pragma unroll
                for (int u = 0; u < 8; ++u) d2[i + u * step] = v[u];
            }
            for (; i < n2; i += step) d2[i] = s2[i];
        } else {
            for (size_t i = threadIdx.x; i < rows; i += blockDim.x) dc[i] = sc[i];
        }
    }
}

// SMs left to the host fetch beside the GEMM, one CTA of 1024 threads each:
// a CTA this size does not fit beside a GEMM CTA, and the block scheduler
// spreads a grid over idle SMs first, so any more CTAs would land on SMs a
// GEMM CTA needs
constexpr int kFetchSms = 16;

struct EventPair {
    cudaEvent_t e[2] = {nullptr, nullptr};
    EventPair() {
        for (auto &x : e) BSG_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    }
    ~EventPair() {
        for (auto &x : e)
            if (x) cudaEventDestroy(x);
    }
};

}  // namespace

void transform_3c2c_ozaki(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *X, const double *V, size_t bs,
                          double thresh, int n_digits, double *out, uint64_t *nsig_out) {
    cudaStream_t s = ctx->stream;
    BSG_REQUIRE(bs <= 64, BSG_ERR_UNSUPPORTED, "Ozaki form supports blocks up to 64");
    const int nd = oz_default_digits(n_digits, (int)bs, (int)bs, (int)bs);
    OzShape sh;
    const Dense3c D = oz3c_dims(n_aux, bs, nd, sh);
    if (!n_vec2 || !n_aux) return;
    DevBuf cnt(16, s);
    BSG_CUDA(cudaMemsetAsync(cnt.p, 0, 16, s));
    Oz3cV v;
    oz3c_prepare_v(ctx, V, D, v);
    // row ranges whose X digit images stay within 16 GB (one range for the
    // 40-atom workload); the rows are independent, so ranges change nothing
    const size_t row_img = D.nkb * (size_t)D.nd * sh.np * sh.kp * 2 / (size_t)D.J;  // image bytes per block row
    const size_t nib = ceil_div(n_vec2, bs);
    const size_t rb = std::max<size_t>(1, std::min(nib, (size_t)(16ull << 30) / std::max<size_t>(row_img, 1)));
    const size_t rr = (rb >= nib ? nib : rb / (size_t)D.J * (size_t)D.J + (rb < (size_t)D.J ? (size_t)D.J : 0)) * bs;
    for (size_t r0 = 0; r0 < n_vec2; r0 += rr)
        oz3c_rows(ctx, D, sh, v, X + r0, n_vec2, std::min(rr, n_vec2 - r0), out + r0, n_vec2, thresh,
                  cnt.as<unsigned long long>());
    ctx->gemm_check();
    if (nsig_out) {
        BSG_CUDA(cudaMemcpyAsync(nsig_out, cnt.p, 8, cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
    }
}

// Host X: uploaded in row ranges on the context's upload stream, each range
// transformed on the compute stream while the next one is in flight (two
// device range buffers).  A range of the column-major X is strided: from
// pinned host memory that the device can address, k_fetch_host_rows reads it
// on kFetchSms SMs that the GEMM launches of the call leave free (about 190
// GB/s on GB300 against about 140 for the copy engine's 2D copy); other
// host memory goes through cudaMemcpy2DAsync.  The rows of the output are
// independent, so the result equals transform_3c2c_ozaki's bit for bit.
void transform_3c2c_ozaki_upload(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *X_host, const double *V,
                                 size_t bs, double thresh, int n_digits, double *out, uint64_t *nsig_out) {
    cudaStream_t s = ctx->stream;
    BSG_REQUIRE(bs <= 64, BSG_ERR_UNSUPPORTED, "Ozaki form supports blocks up to 64");
    const int nd = oz_default_digits(n_digits, (int)bs, (int)bs, (int)bs);
    OzShape sh;
    const Dense3c D = oz3c_dims(n_aux, bs, nd, sh);
    if (!n_vec2 || !n_aux) return;
    // about eight ranges of whole block rows
    const size_t nib = ceil_div(n_vec2, bs), rc = std::max<size_t>(1, ceil_div(nib, (size_t)8)) * bs;
    const size_t n_ch = ceil_div(n_vec2, rc);
    DevBuf cnt(16, s), xb0(rc * n_aux * 8, s), xb1(n_ch > 1 ? rc * n_aux * 8 : 0, s);
    double *xb[2] = {xb0.as<double>(), xb1.as<double>()};
    cudaStream_t up = ctx->upload_stream();
    EventPair copied, used, ready;
    // the range buffers exist (stream-ordered allocation): the first range's
    // upload may start, beside the V operands' preparation
    BSG_CUDA(cudaEventRecord(ready.e[0], s));
    BSG_CUDA(cudaStreamWaitEvent(up, ready.e[0], 0));
    BSG_CUDA(cudaMemsetAsync(cnt.p, 0, 16, s));
    Oz3cV v;
    oz3c_prepare_v(ctx, V, D, v);
    // pinned host memory the device can address, first and last element
    // alike (so the matrix does not reach past a registered region): fetched
    // by SMs
    const double *X_mapped = nullptr;
    {
        auto mapped = [](const double *h) -> const double * {
            cudaPointerAttributes at{};
            if (cudaPointerGetAttributes(&at, h) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
                return static_cast<const double *>(at.devicePointer);
            cudaGetLastError();  // not a registered pointer: clear the error, copy with the copy engine
            return nullptr;
        };
        const size_t last = n_vec2 * n_aux - 1;
        const double *first_d = mapped(X_host), *last_d = mapped(X_host + last);
        if (first_d && last_d == first_d + last) X_mapped = first_d;
    }
    const bool fetch = X_mapped && ctx->sm_count > 4 * kFetchSms;
    struct Reserve {  // GEMM launches beside a fetch leave kFetchSms SMs free (restored on exit)
        bsg_ctx c;
        int prev;
        ~Reserve() { c->oz_sm_reserve = prev; }
    } reserve{ctx, ctx->oz_sm_reserve};
    auto upload = [&](size_t c) {
        const size_t r0 = c * rc, rows = std::min(rc, n_vec2 - r0);
        if (fetch) {
            const int vec = ((reinterpret_cast<uintptr_t>(X_mapped + r0) | reinterpret_cast<uintptr_t>(xb[c & 1]) |
                              (n_vec2 * 8) | (rows * 8)) &
                             15u) == 0;
            k_fetch_host_rows<<<kFetchSms, 1024, 0, up>>>(X_mapped + r0, n_vec2, rows, n_aux, xb[c & 1], vec);
            ctx->note_launch();
            ctx->check_launch("3c2c host fetch");
        } else {
            BSG_CUDA(cudaMemcpy2DAsync(xb[c & 1], rows * 8, X_host + r0, n_vec2 * 8, rows * 8, n_aux,
                                       cudaMemcpyHostToDevice, up));
        }
        BSG_CUDA(cudaEventRecord(copied.e[c & 1], up));
    };
    upload(0);
    for (size_t c = 0; c < n_ch; ++c) {
        if (c + 1 < n_ch) {
            if (c >= 1) BSG_CUDA(cudaStreamWaitEvent(up, used.e[(c + 1) & 1], 0));  // range c-1 is done with it
            upload(c + 1);
        }
        BSG_CUDA(cudaStreamWaitEvent(s, copied.e[c & 1], 0));
        const size_t r0 = c * rc, rows = std::min(rc, n_vec2 - r0);
        // the last range runs with no fetch beside it: its GEMM takes every SM
        ctx->oz_sm_reserve = (fetch && c + 1 < n_ch) ? kFetchSms : reserve.prev;
        oz3c_rows(ctx, D, sh, v, xb[c & 1], rows, rows, out + r0, n_vec2, thresh, cnt.as<unsigned long long>());
        BSG_CUDA(cudaEventRecord(used.e[c & 1], s));
    }
    ctx->gemm_check();
    if (nsig_out) {
        BSG_CUDA(cudaMemcpyAsync(nsig_out, cnt.p, 8, cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
    }
}

}  // namespace bsg
