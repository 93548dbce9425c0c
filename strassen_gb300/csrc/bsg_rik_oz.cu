// occ-RI-K exchange step, Ozaki form: the three block products of every P run
// on tcgen05 tensor cores as bf16 digit slices with exact fp32 chains; the
// screening (block norms, masks, surviving pairs), the transpose-add and the
// K accumulation stay FP64.
//
// Per chunk of aux functions P (N-side groups of two blocks where both TMEM
// accumulator sets fit):
//   U_P                  block norms, flags, row maxima and dense copies of the
//                        occupied blocks, gathered once from the compressed
//                        integrals (bit-identical FP64 norms)
//   mui_P = U_P C        as mui_P^T = C^T U_P^T: tiles (P pair, a, 5 occupied
//                        block columns j), steps over the present U_P(a, b)
//   mui statistics       FP64 norms, row and column maxima in one pass; all
//                        digit images of mui in one pass
//   ij_P  = C^T mui_P    tiles (P, jb pair, 5 block rows ib), steps over a
//   ijs_P = ij + ij^T    FP64 (shared kernel)
//   K    += mui_P ijs_P  tiles (P sub-range, jb pair, 5 block rows a), steps
//                        over (P, ib); per-tile partial blocks summed in order
//   Kmn  += mui_P mui_P^T  (optional) tiles (P sub-range, b pair, block rows
//                        a >= b), steps over (P, jb); lower blocks, mirrored
//                        at the end
// The U pass of chunk c+1 runs on a low-priority side stream beside chunk c's
// statistics and image passes (two U sets, ordered by events); the products
// run on a high-priority chain stream; both join the caller's stream.
// Steps whose N-side sub-blocks have different surviving slot sets split into
// exact rectangles, so every product the FP64 screen drops stays out.
// Operand scales: U rows per (P, mu); C columns per i (also the rows of C^T);
// mui columns per (P, j) for the ij product; mui rows and ijs columns per
// (P sub-range, mu / j) for the K product.  Every tile has one scale set, so
// its steps chain exactly (<= 512 k per chain).
#include <algorithm>

#include "bsg_ozaki.cuh"
#include "bsg_rik.cuh"

namespace bsg {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ int ext_r(size_t blk, size_t bs, size_t n) {
    return (int)(((blk + 1) * bs <= n) ? bs : n - blk * bs);
}

// ---- scale exponents ----

// ---- U_p straight from the compressed integrals ----
// The reference rebuilds a dense n_bf x n_bf U_P for every aux function from
// the significant-pair storage (decompress_integrals, occ_ri_k_step.cpp:
// 133-146) and then blocks and screens it (:102-104).  Here the dense U is
// never formed: an inverse key map gives, for every (mu, nu), the index v of
// its compressed entry (or none), and the block norms, row exponents and
// digit images gather U_P(mu, nu) = ints[v, P] from column P.

// inv[key] = the last v carrying that key (the reference's sequential scatter
// keeps the last write), -1 where no entry exists; occ[a + b*nb] = 1 for the
// blocks of U that hold any entry (the others are zero for every P)
__global__ void k_key_inverse(const uint64_t *__restrict__ keys, size_t n_vec2, size_t n_bf, size_t bs, size_t nb,
                              int *__restrict__ inv, uint8_t *__restrict__ occ) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_vec2) return;
    const uint64_t key = keys[v];
    atomicMax(&inv[key], (int)v);
    occ[(key % n_bf) / bs + (key / n_bf) / bs * nb] = 1;
}

// U_P(r0 + r, c0 + l) from column P of the compressed integrals
struct UGet {
    const int *inv;
    const double *col;
    size_t n_bf, r0, c0;
    __device__ __forceinline__ double operator()(int r, int l) const {
        const int v = inv[(r0 + r) + (c0 + l) * n_bf];
        return v >= 0 ? col[v] : 0.0;
    }
};

// block norms and keep flags of U_p, one warp per (p, occupied block w =
// p*n_ob + ob); the elements are visited in the order of the dense block norm
// (lane-strided column-major), so the result is bit-identical to it.  Blocks
// without any integral keep the zero norm and flag the caller cleared.  The
// gathered elements are also stored densely (ucomp + w*bs*bs, column-major
// with the block's row count as leading dimension) for the row maxima and
// the digit images.
__global__ void k_unorms_c(const double *__restrict__ ints, const int *__restrict__ inv,
                           const uint32_t *__restrict__ ob_list, size_t n_ob, size_t n_vec2, size_t P0, size_t n_bf,
                           size_t bs, size_t nb, size_t n_p, double tpb, double *__restrict__ norm,
                           uint8_t *__restrict__ flag, double *__restrict__ ucomp,
                           unsigned long long *__restrict__ row_bits) {
    const size_t w = oz_warp_id();
    if (w >= n_p * n_ob) return;
    const size_t p = w / n_ob, rr = ob_list[w % n_ob], a = rr % nb, b = rr / nb;
    const size_t x = p * nb * nb + rr;
    const int rs = ext_r(a, bs, n_bf), cs = ext_r(b, bs, n_bf);
    const UGet get{inv, ints + (P0 + p) * n_vec2, n_bf, a * bs, b * bs};
    double *dense = ucomp + w * bs * bs;
    const int lane = threadIdx.x & 31, n = rs * cs;
    double acc = 0.0;
    for (int i0 = lane; i0 < n; i0 += 32 * 8) {
        double v[8];  // eight independent gathers in flight, then the chain in the same order
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = i0 + 32 * u;
            v[u] = i < n ? get(i % rs, i / rs) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (i0 + 32 * u < n) {
                acc = fma(v[u], v[u], acc);
                dense[i0 + 32 * u] = v[u];
            }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, o));
    const double est = sqrt(__shfl_sync(0xffffffffu, acc, 0));
    const bool keep = !(est < tpb);
    if (lane == 0) {
        norm[x] = est;
        flag[x] = keep;
    }
    if (!keep) return;
    // row maxima of the kept block (the scale exponents of U's rows), from
    // the dense copy this warp just wrote
    __syncwarp();
    for (int r = lane; r < rs; r += 32) {
        long long mx = 0;
        for (int l = 0; l < cs; ++l) {
            const long long bb_ = oz_absbits(dense[r + l * rs]);
            mx = bb_ > mx ? bb_ : mx;
        }
        if (mx) atomicMax(&row_bits[p * n_bf + a * bs + r], (unsigned long long)mx);
    }
}

// columns of C over every row; grid jb
__global__ void k_cexp_C(const double *__restrict__ C, size_t n_bf, size_t n_occ, size_t bs, int *__restrict__ cexp) {
    const size_t jb = blockIdx.x;
    const int c = threadIdx.x;
    if (c >= ext_r(jb, bs, n_occ)) return;
    long long mx = 0;
    for (size_t mu = 0; mu < n_bf; ++mu) { const long long bb_ = oz_absbits(C[mu + (jb * bs + c) * n_bf]); mx = bb_ > mx ? bb_ : mx; }
    cexp[jb * bs + c] = oz_exp_of_bits(mx);
}

// ---- row / column maxima, one warp per present block ----
// Bit patterns of |x| (non-negative doubles order like their bits) are
// combined with atomicMax; the exponents follow from the maxima.

// columns of ijs over the aux sub-range p / Q
__global__ void k_colmax_ijs_sub(const double *__restrict__ ijs, const uint8_t *__restrict__ sflag, size_t n_occ,
                                 size_t bs, size_t nob, size_t Q, size_t n, unsigned long long *__restrict__ bits) {
    const size_t x = oz_warp_id();
    if (x >= n || !sflag[x]) return;
    const size_t p = x / (nob * nob), ib = x % nob, jb = (x / nob) % nob;
    const int k = ext_r(ib, bs, n_occ), cols = ext_r(jb, bs, n_occ);
    const double *S = ijs + p * n_occ * n_occ;
    for (int c = threadIdx.x & 31; c < cols; c += 32) {
        long long mx = 0;
        for (int l = 0; l < k; ++l) {
            const long long bb_ = oz_absbits(S[ib * bs + l + (jb * bs + c) * n_occ]);
            mx = bb_ > mx ? bb_ : mx;
        }
        if (mx) atomicMax(&bits[(p / Q) * n_occ + jb * bs + c], (unsigned long long)mx);
    }
}

// ---- digit images ----

struct OzDims {
    size_t n_bf, n_occ, bs, nb, nob;
    int mp, kp, np, nd, R;
    // N side of the ij and K products: J occupied block columns per tile
    // (stacked along N in one image of npJ rows per digit plane), nobp groups
    int J, npJ;
    size_t nobp;
    // N side of mui^T = C^T U^T: U blocks of Jm consecutive aux functions per
    // image (npm rows per digit plane)
    int Jm, npm;
    // N side of K_mn = mui mui^T: Jk consecutive basis block rows per image
    // (npk rows per digit plane), nbp groups
    int Jk, npk;
    size_t nbp;
};

// N-side image rows of occupied block column jb = J*jbp + j inside its
// group's image start at j*bs (J = 1: the image's own np rows)
__device__ __forceinline__ int rows_in_group(const OzDims &D) { return D.J == 1 ? D.npJ : (int)D.bs; }



// Sub-blocks that the screen drops in every tile.  A product's N-side
// sub-block survives with slot s when nA_s nB >= tpb; a correctly rounded
// product is monotone in each factor, so the test against the largest slot
// norm any tile can hold decides it for every tile at once.  Such a
// sub-block gets an all-zero image where the other sub-block of its image
// does survive somewhere, so that the tile builders may count it as present
// (one whole-image copy per step instead of one per digit plane and
// sub-block) while the MMA adds exact zeros for it.
__device__ __forceinline__ bool sub_dead(bool present, double nslot_max, double nb_, double tpb) {
    return !present || !(__dmul_rn(nslot_max, nb_) >= tpb);
}

// cmax[x] = max over occupied block columns ib of ||C(x, ib)|| (cnorm: x + ib*nb)
__global__ void k_cnorm_rowmax(const double *__restrict__ cnorm, size_t nb, size_t nob, double *__restrict__ cmax) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nb) return;
    double m = 0.0;
    for (size_t ib = 0; ib < nob; ++ib) m = fmax(m, cnorm[x + ib * nb]);
    cmax[x] = m;
}

// mmax[p*nob + ib] = max over basis blocks a of the present ||mui_p(a, ib)||
__global__ void k_mnorm_max(const double *__restrict__ mnorm, const uint8_t *__restrict__ mflag, size_t np, size_t nb,
                            size_t nob, double *__restrict__ mmax) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= np * nob) return;
    const size_t p = x / nob, ib = x % nob, base = p * nb * nob + ib * nb;
    double m = 0.0;
    for (size_t a = 0; a < nb; ++a)
        if (mflag[base + a]) m = fmax(m, mnorm[base + a]);
    mmax[x] = m;
}

// U_p blocks (a, b) as the N side of mui^T = C^T U^T (image rows = the
// block's rows mu, k = its columns), from the dense copies; kImgUBlocks
// consecutive occupied blocks w per warp.  The blocks of Jm consecutive aux
// functions p = Jm*pp + j share one image (index pp*nb*nb + a + b*nb), aux
// function j at rows j*bs.
constexpr int kImgUBlocks = 4;
__global__ void k_img_U(const double *__restrict__ ucomp, const uint32_t *__restrict__ ob_list, size_t n_ob,
                        size_t n_p, const uint8_t *__restrict__ uflag, const double *__restrict__ unorm,
                        const double *__restrict__ cmax, double tpb, const int *__restrict__ rexp, OzDims D,
                        bf16 *__restrict__ img) {
    __shared__ OzImgJob sj[kOzImgWarps][kImgUBlocks];
    const size_t w0 = oz_warp_id() * kImgUBlocks, nw = n_p * n_ob;
    if (w0 >= nw) return;
    oz_jobs_image(
        kImgUBlocks,
        [&](int q, OzImgJob &J) {
            const size_t w = w0 + q;
            if (w >= nw) return false;
            const size_t p = w / n_ob, rr = ob_list[w % n_ob], a = rr % D.nb, b = rr / D.nb;
            const size_t pp = p / D.Jm, j = p % D.Jm;
            const size_t u = p * D.nb * D.nb + rr;
            bool zero = false;
            if (sub_dead(uflag[u], cmax[b], unorm[u], tpb)) {
                // zeros where the pair's other aux function survives
                const size_t q = pp * D.Jm + (1 - j), uq = q * D.nb * D.nb + rr;
                if (D.Jm != 2 || q >= n_p || sub_dead(uflag[uq], cmax[b], unorm[uq], tpb)) return false;
                zero = true;
            }
            const int rows = ext_r(a, D.bs, D.n_bf);
            J.get = OzDenseGet{ucomp + w * D.bs * D.bs, (size_t)rows, false};
            J.rows = zero ? 0 : rows;  // 0 rows: all digits zero
            J.k = ext_r(b, D.bs, D.n_bf);
            J.exps = rexp + p * D.n_bf + a * D.bs;
            J.dst = img + (pp * D.nb * D.nb + rr) * D.nd * (size_t)D.npm * D.kp + j * D.bs * (size_t)D.kp;
            J.m_side = false;
            J.plane_rows = D.npm;
            return true;
        },
        D.Jm == 1 ? D.npm : (int)D.bs, D.kp, D.nd, sj[threadIdx.x >> 5]);
}

// C^T blocks (ib, a) in the A role of ij = C^T mui and of mui^T = C^T U^T; index ib + a*nob
__global__ void k_img_Ct_A(const double *__restrict__ C, const int *__restrict__ cexp, OzDims D, bf16 *__restrict__ img) {
    const size_t x = oz_warp_id();
    if (x >= D.nob * D.nb) return;
    const size_t ib = x % D.nob, a = x / D.nob;
    oz_block_image(C + a * D.bs + ib * D.bs * D.n_bf, D.n_bf, true, ext_r(ib, D.bs, D.n_occ), ext_r(a, D.bs, D.n_bf),
                cexp + ib * D.bs, D.mp, D.kp, D.nd, img + x * D.nd * (size_t)D.mp * D.kp, true);
}

// All digit images of mui_p blocks x = (p, a, jb), jb < nobp*J, kImgMBlocks
// consecutive blocks per warp: the A image of the K and K_mn products (rows
// a, row exponents per aux sub-range, index p*nb*nob + a + jb*nb), the
// J-grouped B image of ij (imgB, rows jb, column exponents per aux function;
// columns past n_occ get zero rows) and the B image of K_mn (imgT, rows a);
// null images are skipped.  A block's B and A images are neighbouring jobs,
// so the block is read from DRAM once and the second split hits L1.
constexpr int kImgMBlocks = 2;
__global__ void k_img_mui_all(const double *__restrict__ mui, const uint8_t *__restrict__ mflag,
                              const double *__restrict__ mnorm, const double *__restrict__ cmax, double tpb,
                              const int *__restrict__ rexp, size_t Q, const int *__restrict__ cexp, OzDims D, size_t n,
                              bf16 *__restrict__ imgA, bf16 *__restrict__ imgB, bf16 *__restrict__ imgT) {
    __shared__ OzImgJob sj[kOzImgWarps][2 * kImgMBlocks];
    const size_t x0 = oz_warp_id() * kImgMBlocks;
    if (x0 >= n) return;
    const size_t nj = D.nobp * D.J;
    // job 2q: B image of block x0 + q, job 2q + 1: its A image
    auto job = [&](int jj, OzImgJob &J) {
        const size_t x = x0 + jj / 2;
        if (x >= n) return false;
        const size_t a = x % D.nb, jb = (x / D.nb) % nj, p = x / (D.nb * nj);
        const bool real = jb < D.nob;
        const size_t xb = p * D.nb * D.nob + a + jb * D.nb;
        const size_t jc = real ? jb : 0;
        const double *M = mui + p * D.n_bf * D.n_occ + a * D.bs + jc * D.bs * D.n_bf;
        const int ra = ext_r(a, D.bs, D.n_bf), rj = real ? ext_r(jb, D.bs, D.n_occ) : 0;
        if (jj & 1) {
            if (!real || !mflag[xb] || !imgA) return false;
            J.get = OzDenseGet{M, D.n_bf, false};
            J.rows = ra;
            J.k = rj;
            J.exps = rexp + (p / Q) * D.n_bf + a * D.bs;
            J.dst = imgA + xb * D.nd * (size_t)D.mp * D.kp;
            J.m_side = true;
            J.plane_rows = 0;
        } else {
            if (!imgB) return false;
            const size_t jbp = jb / D.J, j = jb % D.J;
            bool zero = false;
            if (real && sub_dead(mflag[xb], cmax[a], mnorm[xb], tpb)) {
                // zeros where the group's other block column survives in ij
                const size_t jq = jbp * D.J + (1 - j), xq = p * D.nb * D.nob + a + jq * D.nb;
                if (D.J != 2 || jq >= D.nob || sub_dead(mflag[xq], cmax[a], mnorm[xq], tpb)) return false;
                zero = true;
            }
            J.get = OzDenseGet{M, D.n_bf, true};
            J.rows = zero ? 0 : rj;  // 0 rows: all digits zero
            J.k = real ? ra : 0;
            J.exps = cexp + p * D.n_occ + jc * D.bs;
            J.dst = imgB + ((p * D.nobp + jbp) * D.nb + a) * D.nd * (size_t)D.npJ * D.kp + j * D.bs * (size_t)D.kp;
            J.m_side = false;
            J.plane_rows = D.npJ;
        }
        return true;
    };
    OzImgJob *tab = sj[threadIdx.x >> 5];
    const int mpB = rows_in_group(D);
    if (mpB == D.mp) {
        oz_jobs_image(2 * kImgMBlocks, job, D.mp, D.kp, D.nd, tab);
    } else {  // different image heights: the B images, then the A images
        oz_jobs_image(kImgMBlocks, [&](int q, OzImgJob &J) { return job(2 * q, J); }, mpB, D.kp, D.nd, tab);
        oz_jobs_image(kImgMBlocks, [&](int q, OzImgJob &J) { return job(2 * q + 1, J); }, D.mp, D.kp, D.nd, tab);
    }
    if (!imgT) return;
    for (int q = 0; q < kImgMBlocks; ++q) {
        // K_mn's N side: block rows a of Jk-groups, image (p, jb, a / Jk), rows (a % Jk) * bs
        const size_t x = x0 + q;
        if (x >= n) break;
        const size_t a = x % D.nb, jb = (x / D.nb) % nj, p = x / (D.nb * nj);
        if (jb >= D.nob || !mflag[p * D.nb * D.nob + a + jb * D.nb]) continue;
        const double *M = mui + p * D.n_bf * D.n_occ + a * D.bs + jb * D.bs * D.n_bf;
        oz_block_image_g(OzDenseGet{M, D.n_bf, false}, ext_r(a, D.bs, D.n_bf), ext_r(jb, D.bs, D.n_occ),
                         rexp + (p / Q) * D.n_bf + a * D.bs, D.Jk == 1 ? D.npk : (int)D.bs, D.kp, D.nd,
                         imgT + ((p * D.nob + jb) * D.nbp + a / D.Jk) * D.nd * (size_t)D.npk * D.kp +
                             (a % D.Jk) * D.bs * (size_t)D.kp,
                         false, threadIdx.x & 31, 32, D.npk);
    }
}

// ijs_p blocks (ib, jb) in the B role of the K product, J block columns per
// image: index p*nob*nobp + ib + jbp*nob; blocks x = (p, ib, jb), jb < nobp*J,
// kImgSBlocks consecutive blocks per warp
constexpr int kImgSBlocks = 4;
__global__ void k_img_ijs_B(const double *__restrict__ ijs, const uint8_t *__restrict__ sflag,
                            const double *__restrict__ snorm, const double *__restrict__ mmax, double tpb,
                            const int *__restrict__ cexp, size_t Q, OzDims D, size_t n, bf16 *__restrict__ img) {
    __shared__ OzImgJob sj[kOzImgWarps][kImgSBlocks];
    const size_t x0 = oz_warp_id() * kImgSBlocks;
    if (x0 >= n) return;
    oz_jobs_image(
        kImgSBlocks,
        [&](int q, OzImgJob &J) {
            const size_t x = x0 + q;
            if (x >= n) return false;
            const size_t nj = D.nobp * D.J, ib = x % D.nob, jb = (x / D.nob) % nj, p = x / (D.nob * nj);
            const size_t jbp = jb / D.J, j = jb % D.J;
            const bool real = jb < D.nob;
            bool zero = !real;
            const size_t sb = p * D.nob * D.nob + ib + jb * D.nob;
            if (real && sub_dead(sflag[sb], mmax[p * D.nob + ib], snorm[sb], tpb)) {
                // zeros where the group's other block column survives in K
                const size_t jq = jbp * D.J + (1 - j), sq = p * D.nob * D.nob + ib + jq * D.nob;
                if (D.J != 2 || jq >= D.nob || sub_dead(sflag[sq], mmax[p * D.nob + ib], snorm[sq], tpb)) return false;
                zero = true;
            }
            const size_t jc = real ? jb : 0;
            J.get = OzDenseGet{ijs + p * D.n_occ * D.n_occ + ib * D.bs + jc * D.bs * D.n_occ, D.n_occ, true};
            J.rows = zero ? 0 : ext_r(jb, D.bs, D.n_occ);  // 0 rows: all digits zero
            J.k = real ? ext_r(ib, D.bs, D.n_occ) : 0;
            J.exps = cexp + (p / Q) * D.n_occ + jc * D.bs;
            J.dst = img + ((p * D.nobp + jbp) * D.nob + ib) * D.nd * (size_t)D.npJ * D.kp + j * D.bs * (size_t)D.kp;
            J.m_side = false;
            J.plane_rows = D.npJ;
            return true;
        },
        rows_in_group(D), D.kp, D.nd, sj[threadIdx.x >> 5]);
}

// ---- tiles and steps (one thread per tile) ----

__device__ __forceinline__ void tile_clear(OzTile &T) {
    for (int s = 0; s < kOzMaxSlots; ++s) {
        T.c[s] = nullptr;
        T.cnorm[s] = nullptr;
        T.rexp[s] = nullptr;
        T.rows[s] = 0;
        T.ldc[s] = 0;
    }
    T.fresh_mask = 0xFFu;
}

// mui tiles, transposed: mui_p^T(j, a) = sum_b C^T(j, b) U_p(a, b)^T, so the
// dense C^T blocks fill the slots (R occupied block columns j) and the
// block-sparse U_p supplies the N side: per step the present U blocks (a, b)
// of Jm consecutive aux functions p = Jm*pp + j (their C^T operand is the
// same).  t = (pp, a, group g of R block columns j), written transposed; the
// aux functions' outputs are n_bf*n_occ apart (sub-blocks stored apart).
__global__ void k_tiles_mui(const uint8_t *__restrict__ uflag, const double *__restrict__ unorm,
                            const double *__restrict__ cnorm, const double *__restrict__ cmax,
                            const int *__restrict__ rexp_U,
                            const int *__restrict__ cexp_C, double *__restrict__ mui, OzDims D, size_t np,
                            size_t n_tiles, double tpb, OzTile *__restrict__ tiles, OzStep *__restrict__ steps,
                            uint8_t *__restrict__ mflag, unsigned long long *__restrict__ nsig,
                            unsigned long long *__restrict__ macs) {
    const size_t t = oz_warp_id();  // one warp per tile, lanes over b
    if (t >= n_tiles) return;
    const int lane = threadIdx.x & 31;
    const size_t ng = (D.nob + D.R - 1) / D.R;
    const size_t g = t % ng, a = (t / ng) % D.nb, pp = t / (ng * D.nb), p0 = pp * D.Jm;
    const int nsub = (int)min((size_t)D.Jm, np - p0);
    unsigned long long m = 0;
    OzTile T;
    tile_clear(T);
    int cnt[kOzMaxSlots][2] = {};
    for (int s = 0; s < D.R; ++s) {
        const size_t j = g * D.R + s;
        if (j >= D.nob) break;
        T.c[s] = mui + p0 * D.n_bf * D.n_occ + a * D.bs + j * D.bs * D.n_bf;
        T.ldc[s] = (int)D.n_bf;
        T.rows[s] = ext_r(j, D.bs, D.n_occ);  // slot rows are mui columns
        T.rexp[s] = cexp_C + j * D.bs;
    }
    const int npj = D.npm / D.Jm;
    T.trans = 1;
    T.cexp = rexp_U + p0 * D.n_bf + a * D.bs;
    if (D.Jm == 1) {
        T.cols = ext_r(a, D.bs, D.n_bf);  // tile columns are mui rows
    } else {
        T.cols = nsub * npj;  // no columns of an aux function past the chunk
        T.sub_cols = ext_r(a, D.bs, D.n_bf);
        T.sub_stride = (long long)(D.n_bf * D.n_occ);
        T.cexp_sub = (int)D.n_bf;
    }
    T.s0 = (uint32_t)(t * D.nb * D.Jm);
    uint32_t n = 0;
    for (size_t base = 0; base < D.nb; base += 32) {
        const size_t b = base + lane;
        OzStep mine[2];
        uint32_t c = 0;
        if (b < D.nb) {
            uint32_t live[2] = {0, 0}, phantom = 0;
            uint32_t a_idx[kOzMaxSlots];
            for (int s = 0; s < kOzMaxSlots; ++s) a_idx[s] = (uint32_t)(g * D.R + s + b * D.nob);
            for (int js = 0; js < nsub; ++js) {
                const size_t ub = (p0 + js) * D.nb * D.nb + a + b * D.nb;
                // dropped in every tile: a zero image where the other aux function survives
                // (and no slot needs a test)
                if (sub_dead(uflag[ub], cmax[b], unorm[ub], tpb)) {
                    if (D.Jm == 2) phantom |= 1u << js;
                    continue;
                }
                for (int s = 0; s < D.R; ++s) {
                    if (!T.c[s]) continue;
                    const size_t j = g * D.R + s;
                    if (!(__dmul_rn(unorm[ub], cnorm[b + j * D.nb]) >= tpb)) continue;
                    live[js] |= 1u << s;
                    m += (unsigned long long)T.rows[s] * ext_r(a, D.bs, D.n_bf) * ext_r(b, D.bs, D.n_bf);
                    ++cnt[s][js];
                }
            }
            // a missing aux function (odd chunk end) counts as absent: its image rows are never written
            c = emit_rect_steps(live, D.Jm, phantom, (uint32_t)(pp * D.nb * D.nb + a + b * D.nb), a_idx, mine);
        }
        warp_append_steps(mine, c, steps + T.s0, n);
    }
    unsigned long long tot = 0;
    for (int s = 0; s < D.R; ++s) {
        const size_t j = g * D.R + s;
        if (j >= D.nob) break;
        for (int js = 0; js < nsub; ++js) {
            const unsigned long long cs = warp_sum_u64((unsigned long long)cnt[s][js]);  // lane 0 holds the sum
            if (lane == 0) mflag[(p0 + js) * D.nb * D.nob + a + j * D.nb] = cs > 0;
            tot += cs;
        }
    }
    m = warp_sum_u64(m);
    if (lane == 0) {
        T.ns = n;
        tiles[t] = T;
        if (tot) atomicAdd(nsig, tot);
        if (m) atomicAdd(macs, m);
    }
}

// ij tiles: t = (p, jbp, group of R block rows ib), N side J block columns
// jb = J*jbp + j, steps over a (split into exact rectangles); one warp per
// tile, lanes over a
__global__ void k_tiles_ij(const uint8_t *__restrict__ mflag, const double *__restrict__ mnorm,
                           const double *__restrict__ cnorm, const double *__restrict__ cmax,
                           const int *__restrict__ cexp_C,
                           const int *__restrict__ cexp_mui, double *__restrict__ ij, OzDims D, size_t n_tiles,
                           double tpb, OzTile *__restrict__ tiles, OzStep *__restrict__ steps,
                           uint8_t *__restrict__ ijflag, unsigned long long *__restrict__ nsig,
                           unsigned long long *__restrict__ macs) {
    const size_t t = oz_warp_id();
    if (t >= n_tiles) return;
    const int lane = threadIdx.x & 31;
    const size_t ng = (D.nob + D.R - 1) / D.R;
    const size_t g = t % ng, jbp = (t / ng) % D.nobp, p = t / (ng * D.nobp);
    unsigned long long m = 0;
    OzTile T;
    tile_clear(T);
    for (int s = 0; s < D.R; ++s) {
        const size_t ib = g * D.R + s;
        if (ib >= D.nob) break;
        T.c[s] = ij + p * D.n_occ * D.n_occ + ib * D.bs + jbp * D.J * D.bs * D.n_occ;
        T.ldc[s] = (int)D.n_occ;
        T.rows[s] = ext_r(ib, D.bs, D.n_occ);
        T.rexp[s] = cexp_C + ib * D.bs;
    }
    int cols = 0;
    uint32_t phantom = 0;
    for (int j = 0; j < D.J; ++j) {
        const size_t jb = jbp * D.J + j;
        if (jb < D.nob) cols = j * (int)D.bs + ext_r(jb, D.bs, D.n_occ);
        else phantom |= 1u << j;
    }
    T.cols = cols;
    T.trans = 0;
    T.cexp = cexp_mui + p * D.n_occ + jbp * D.J * D.bs;
    T.s0 = (uint32_t)(t * D.nb * D.J);
    uint32_t n = 0, seen[kOzMaxSlots][2] = {};  // per (slot, sub-block): products in this lane
    for (size_t base = 0; base < D.nb; base += 32) {
        const size_t a = base + lane;
        OzStep mine[2];
        uint32_t cnt = 0;
        if (a < D.nb) {
            uint32_t live[2] = {0, 0}, ph = phantom;
            uint32_t a_idx[kOzMaxSlots];
            for (int s = 0; s < kOzMaxSlots; ++s) a_idx[s] = (uint32_t)(g * D.R + s + a * D.nob);
            for (int j = 0; j < D.J; ++j) {
                const size_t jb = jbp * D.J + j;
                if (jb >= D.nob) continue;
                const size_t mb = p * D.nb * D.nob + a + jb * D.nb;
                // dropped in every tile: a zero image where the other block column survives
                // (and no slot needs a test)
                if (sub_dead(mflag[mb], cmax[a], mnorm[mb], tpb)) {
                    if (D.J == 2) ph |= 1u << j;
                    continue;
                }
                for (int s = 0; s < D.R; ++s) {
                    if (!T.c[s]) continue;
                    const size_t ib = g * D.R + s;
                    if (!(__dmul_rn(cnorm[a + ib * D.nb], mnorm[mb]) >= tpb)) continue;
                    live[j] |= 1u << s;
                    m += (unsigned long long)T.rows[s] * ext_r(jb, D.bs, D.n_occ) * ext_r(a, D.bs, D.n_bf);
                    ++seen[s][j];
                }
            }
            cnt = emit_rect_steps(live, D.J, ph, (uint32_t)((p * D.nobp + jbp) * D.nb + a), a_idx, mine);
        }
        warp_append_steps(mine, cnt, steps + T.s0, n);
    }
    unsigned long long tot = 0;
    for (int s = 0; s < D.R; ++s) {
        const size_t ib = g * D.R + s;
        if (ib >= D.nob) break;
        for (int j = 0; j < D.J; ++j) {
            const size_t jb = jbp * D.J + j;
            const unsigned long long c = warp_sum_u64(seen[s][j]);  // lane 0 holds the tile's count
            if (jb >= D.nob) continue;
            if (lane == 0) ijflag[p * D.nob * D.nob + ib + jb * D.nob] = c > 0;
            tot += c;
        }
    }
    m = warp_sum_u64(m);
    if (lane == 0) {
        T.ns = n;
        tiles[t] = T;
        if (tot) atomicAdd(nsig, tot);
        if (m) atomicAdd(macs, m);
    }
}

// K tiles: t = (sub-range, jbp, group of R block rows a), N side J block
// columns jb = J*jbp + j, steps over (p, ib) split into exact rectangles;
// partial blocks of a tile: Kpart + ((sub*nobp + jbp)*nb + a) * bs * J*bs,
// column-major with ld = the block's rows.  One warp per tile, lanes over
// the (p, ib) steps.
__global__ void k_tiles_K(const uint8_t *__restrict__ mflag, const double *__restrict__ mnorm,
                          const uint8_t *__restrict__ sflag, const double *__restrict__ snorm,
                          const double *__restrict__ mmax,
                          const int *__restrict__ rexp_sub, const int *__restrict__ cexp_sub, double *__restrict__ Kpart,
                          OzDims D, size_t np, size_t Q, size_t n_tiles, double tpb, OzTile *__restrict__ tiles,
                          OzStep *__restrict__ steps, unsigned long long *__restrict__ nsig,
                          unsigned long long *__restrict__ macs) {
    const size_t t = oz_warp_id();
    if (t >= n_tiles) return;
    const int lane = threadIdx.x & 31;
    const size_t ng = (D.nb + D.R - 1) / D.R;
    const size_t g = t % ng, jbp = (t / ng) % D.nobp, sub = t / (ng * D.nobp);
    unsigned long long m = 0, tot = 0;
    OzTile T;
    tile_clear(T);
    const size_t blk = D.bs * D.bs * D.J;
    for (int s = 0; s < D.R; ++s) {
        const size_t a = g * D.R + s;
        if (a >= D.nb) break;
        T.c[s] = Kpart + ((sub * D.nobp + jbp) * D.nb + a) * blk;
        T.rows[s] = ext_r(a, D.bs, D.n_bf);
        T.ldc[s] = T.rows[s];
        T.rexp[s] = rexp_sub + sub * D.n_bf + a * D.bs;
    }
    int cols = 0;
    uint32_t phantom = 0;
    for (int j = 0; j < D.J; ++j) {
        const size_t jb = jbp * D.J + j;
        if (jb < D.nob) cols = j * (int)D.bs + ext_r(jb, D.bs, D.n_occ);
        else phantom |= 1u << j;
    }
    T.cols = cols;
    T.trans = 0;
    T.cexp = cexp_sub + sub * D.n_occ + jbp * D.J * D.bs;
    T.s0 = (uint32_t)(t * Q * D.nob * D.J);
    uint32_t n = 0;
    const size_t p0 = sub * Q, p1 = min(np, (sub + 1) * Q), n_k = (p1 - p0) * D.nob;
    for (size_t base = 0; base < n_k; base += 32) {
        const size_t idx = base + lane;
        OzStep mine[2];
        uint32_t cnt = 0;
        if (idx < n_k) {
            const size_t p = p0 + idx / D.nob, ib = idx % D.nob;
            uint32_t live[2] = {0, 0}, ph = phantom;
            uint32_t a_idx[kOzMaxSlots];
            for (int s = 0; s < kOzMaxSlots; ++s) a_idx[s] = (uint32_t)(p * D.nb * D.nob + g * D.R + s + ib * D.nb);
            for (int j = 0; j < D.J; ++j) {
                const size_t jb = jbp * D.J + j;
                if (jb >= D.nob) continue;
                const size_t sb = p * D.nob * D.nob + ib + jb * D.nob;
                // dropped in every tile: a zero image where the other block column survives
                // (and no slot needs a test)
                if (sub_dead(sflag[sb], mmax[p * D.nob + ib], snorm[sb], tpb)) {
                    if (D.J == 2) ph |= 1u << j;
                    continue;
                }
                for (int s = 0; s < D.R; ++s) {
                    if (!T.c[s]) continue;
                    const size_t mb = p * D.nb * D.nob + g * D.R + s + ib * D.nb;
                    if (!mflag[mb]) continue;
                    if (!(__dmul_rn(mnorm[mb], snorm[sb]) >= tpb)) continue;
                    live[j] |= 1u << s;
                    m += (unsigned long long)T.rows[s] * ext_r(jb, D.bs, D.n_occ) * ext_r(ib, D.bs, D.n_occ);
                    ++tot;
                }
            }
            cnt = emit_rect_steps(live, D.J, ph, (uint32_t)((p * D.nobp + jbp) * D.nob + ib), a_idx, mine);
        }
        warp_append_steps(mine, cnt, steps + T.s0, n);
    }
    m = warp_sum_u64(m);
    tot = warp_sum_u64(tot);
    if (lane == 0) {
        T.ns = n;
        tiles[t] = T;
        if (tot) atomicAdd(nsig, tot);
        if (m) atomicAdd(macs, m);
    }
}

// K(a, jb) += sum over sub-ranges (in order) of the tiles' partial blocks
__global__ void k_K_reduce(const double *__restrict__ Kpart, size_t n_sub, OzDims D, double *__restrict__ K) {
    const size_t x = blockIdx.x;  // (jb, a)
    const size_t a = x % D.nb, jb = x / D.nb, jbp = jb / D.J, j = jb % D.J;
    const int rows = ext_r(a, D.bs, D.n_bf), cols = ext_r(jb, D.bs, D.n_occ);
    const size_t blk = D.bs * D.bs * D.J;
    for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
        const int r = e % rows, c = e / rows;
        const size_t pe = (size_t)r + (j * D.bs + c) * (size_t)rows;
        double acc = K[a * D.bs + r + (jb * D.bs + c) * D.n_bf];
        for (size_t sub = 0; sub < n_sub; ++sub) acc += Kpart[((sub * D.nobp + jbp) * D.nb + a) * blk + pe];
        K[a * D.bs + r + (jb * D.bs + c) * D.n_bf] = acc;
    }
}

// (bp, g) pairs of the K_mn tiles: a group of Jk block columns b = Jk*bp + j
// and a group g of R block rows a = g R .. g R + R - 1 with at least one
// a >= Jk*bp; pairs ordered by bp, then g
__host__ __device__ inline size_t kmn_pairs(size_t nbp, size_t Jk, size_t nb, size_t R) {
    const size_t ng = (nb + R - 1) / R;
    size_t n = 0;
    for (size_t bp = 0; bp < nbp; ++bp) n += ng - (Jk * bp) / R;
    return n;
}

// K_mn tiles: t = (sub-range, pair (bp, g)), N side Jk block columns, steps
// over (p, jb) split into exact rectangles; a product (a, b) enters only for
// a >= b (the upper blocks are the mirrors).  Partial blocks of a tile:
// Kpart + ((sub*nbp + bp)*nb + a) * bs * Jk*bs, column-major, ld = rows.
__global__ void k_tiles_Kmn(const uint8_t *__restrict__ mflag, const double *__restrict__ mnorm,
                            const int *__restrict__ rexp_sub, double *__restrict__ Kpart, OzDims D, size_t np,
                            size_t Q, size_t n_pairs, size_t n_tiles, double tpb, OzTile *__restrict__ tiles,
                            OzStep *__restrict__ steps, unsigned long long *__restrict__ nsig,
                            unsigned long long *__restrict__ macs) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    const size_t ng = (D.nb + D.R - 1) / D.R, sub = t / n_pairs;
    size_t rem = t % n_pairs, bp = 0, g = 0;
    for (; bp < D.nbp; ++bp) {
        const size_t c = ng - (D.Jk * bp) / D.R;
        if (rem < c) {
            g = (D.Jk * bp) / D.R + rem;
            break;
        }
        rem -= c;
    }
    const size_t b0 = bp * D.Jk;
    unsigned long long m = 0;
    OzTile T;
    tile_clear(T);
    const size_t blk = D.bs * D.bs * D.Jk;
    for (int s = 0; s < D.R; ++s) {
        const size_t a = g * D.R + s;
        if (a >= D.nb) break;
        if (a < b0) continue;
        T.c[s] = Kpart + ((sub * D.nbp + bp) * D.nb + a) * blk;
        T.rows[s] = ext_r(a, D.bs, D.n_bf);
        T.ldc[s] = T.rows[s];
        T.rexp[s] = rexp_sub + sub * D.n_bf + a * D.bs;
    }
    int cols = 0;
    for (int j = 0; j < D.Jk; ++j)
        if (b0 + j < D.nb) cols = j * (int)D.bs + ext_r(b0 + j, D.bs, D.n_bf);
    T.cols = cols;
    T.trans = 0;
    T.cexp = rexp_sub + sub * D.n_bf + b0 * D.bs;
    T.s0 = (uint32_t)(t * Q * D.nob * D.Jk);
    uint32_t n = 0;
    unsigned long long tot = 0;
    const size_t p1 = min(np, (sub + 1) * Q);
    for (size_t p = sub * Q; p < p1; ++p)
        for (size_t jb = 0; jb < D.nob; ++jb) {
            uint32_t live[2] = {0, 0};
            uint32_t a_idx[kOzMaxSlots];
            for (int s = 0; s < kOzMaxSlots; ++s) a_idx[s] = (uint32_t)(p * D.nb * D.nob + g * D.R + s + jb * D.nb);
            for (int j = 0; j < D.Jk; ++j) {
                const size_t b = b0 + j;
                if (b >= D.nb) continue;
                const size_t mb = p * D.nb * D.nob + b + jb * D.nb;
                if (!mflag[mb]) continue;
                for (int s = 0; s < D.R; ++s) {
                    if (!T.c[s]) continue;
                    const size_t a = g * D.R + s, ma = p * D.nb * D.nob + a + jb * D.nb;
                    if (a < b || !mflag[ma]) continue;
                    if (!(__dmul_rn(mnorm[ma], mnorm[mb]) >= tpb)) continue;
                    live[j] |= 1u << s;
                    m += (unsigned long long)T.rows[s] * ext_r(b, D.bs, D.n_bf) * ext_r(jb, D.bs, D.n_occ);
                    ++tot;
                }
            }
            n += emit_rect_steps(live, D.Jk, 0u, (uint32_t)((p * D.nob + jb) * D.nbp + bp), a_idx, steps + T.s0 + n);
        }
    T.ns = n;
    tiles[t] = T;
    if (tot) atomicAdd(nsig, tot);
    if (m) atomicAdd(macs, m);
}

// K_mn(a, b) += sum over sub-ranges (in order) of the tiles' partial blocks, a >= b
__global__ void k_Kmn_reduce(const double *__restrict__ Kpart, size_t n_sub, OzDims D, double *__restrict__ K) {
    const size_t x = blockIdx.x;  // (b, a)
    const size_t a = x % D.nb, b = x / D.nb, bp = b / D.Jk, j = b % D.Jk;
    if (a < b) return;
    const int rows = ext_r(a, D.bs, D.n_bf), cols = ext_r(b, D.bs, D.n_bf);
    const size_t blk = D.bs * D.bs * D.Jk;
    for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
        const int r = e % rows, c = e / rows;
        const size_t pe = (size_t)r + (j * D.bs + c) * (size_t)rows;
        double acc = K[a * D.bs + r + (b * D.bs + c) * D.n_bf];
        for (size_t sub = 0; sub < n_sub; ++sub) acc += Kpart[((sub * D.nbp + bp) * D.nb + a) * blk + pe];
        K[a * D.bs + r + (b * D.bs + c) * D.n_bf] = acc;
    }
}

// upper triangle of K_mn from the lower one (diagonal blocks by element)
__global__ void k_Kmn_mirror(double *__restrict__ K, size_t n_bf, size_t bs) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_bf * n_bf) return;
    const size_t gi = e % n_bf, gj = e / n_bf;
    const size_t bi = gi / bs, bj = gj / bs;
    if (bi < bj || (bi == bj && gi < gj)) K[e] = K[gj + gi * n_bf];
}

// One pass over each present mui_p block (kNormBlocks consecutive blocks per
// warp): its FP64 norm (the deterministic block-norm order, finished from the
// warp's table of chains), its row maxima per aux sub-range p/Q (rows of the
// A operand of K and K_mn) and, when col_bits is given, its column maxima per
// p (columns of the B operand of ij).  The block is read from DRAM once; the
// maxima walk hits L1.
__global__ void k_mui_stats(const double *__restrict__ mui, const uint8_t *__restrict__ mflag, size_t n_bf,
                            size_t n_occ, size_t bs, size_t nb, size_t nob, size_t Q, size_t n,
                            double *__restrict__ mnorm, unsigned long long *__restrict__ row_bits,
                            unsigned long long *__restrict__ col_bits) {
    __shared__ NormTable tab[kOzImgWarps];
    const size_t x0 = oz_warp_id() * kNormBlocks;
    if (x0 >= n) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nq = (int)min((size_t)kNormBlocks, n - x0);
    for (int q = 0; q < nq; ++q) {
        const size_t x = x0 + q;
        if (!mflag[x]) continue;
        const size_t p = x / (nb * nob), a = x % nb, jb = (x / nb) % nob;
        const int rows = ext_r(a, bs, n_bf), cols = ext_r(jb, bs, n_occ);
        const double *M = mui + p * n_bf * n_occ + a * bs + jb * bs * n_bf;
        tab[w][q][lane] = warp_norm_chain(M, rows, cols, n_bf);
        // one walk over the columns with the lanes over rows (bs <= 64: rows
        // lane and lane + 32), so every step reads one column coalesced; a
        // column's maximum is a warp reduction, kept by lane l % 32
        unsigned long long rmx[2] = {0, 0}, cmx[2] = {0, 0};
#pragma unroll 4
        for (int l = 0; l < cols; ++l) {
            const double *col = M + (size_t)l * n_bf;
            unsigned long long cm = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = lane + 32 * h;
                if (r < rows) {
                    const unsigned long long bb = (unsigned long long)oz_absbits(col[r]);
                    rmx[h] = bb > rmx[h] ? bb : rmx[h];
                    cm = bb > cm ? bb : cm;
                }
            }
            if (col_bits) {
                cm = warp_max_u64(cm);
                if (lane == (l & 31)) (l < 32 ? cmx[0] : cmx[1]) = cm;
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = lane + 32 * h;
            if (r < rows && rmx[h]) atomicMax(&row_bits[(p / Q) * n_bf + a * bs + r], rmx[h]);
            if (col_bits && r < cols && cmx[h]) atomicMax(&col_bits[p * n_occ + jb * bs + r], cmx[h]);
        }
    }
    __syncwarp();
    if (lane < nq && mflag[x0 + lane]) mnorm[x0 + lane] = norm_from_chains(tab[w][lane]);
}

// Two streams forked off a caller's stream: both wait for the caller's work
// so far; join() makes the caller's stream wait for both.  The destructor
// joins too when join() was not reached (an error path), so no kernel of the
// fork outlives the stream-ordered frees of the caller's buffers.  Also holds
// the events that order the U sets between the two streams.
struct StreamFork {
    cudaStream_t base, a, b;
    cudaEvent_t start = nullptr, end_a = nullptr, end_b = nullptr;
    cudaEvent_t u_ready[2] = {nullptr, nullptr}, u_done[2] = {nullptr, nullptr};
    bool joined = false;
    StreamFork(cudaStream_t base_, cudaStream_t a_, cudaStream_t b_) : base(base_), a(a_), b(b_) {
        for (cudaEvent_t *e : {&start, &end_a, &end_b, &u_ready[0], &u_ready[1], &u_done[0], &u_done[1]})
            if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
                *e = nullptr;
                release();
                throw Error{BSG_ERR_CUDA, "stream fork: event creation failed"};
            }
        if (cudaEventRecord(start, base) != cudaSuccess || cudaStreamWaitEvent(a, start, 0) != cudaSuccess ||
            cudaStreamWaitEvent(b, start, 0) != cudaSuccess) {
            release();
            throw Error{BSG_ERR_CUDA, "stream fork: ordering the streams failed"};
        }
    }
    void join() {
        BSG_CUDA(cudaEventRecord(end_a, a));
        BSG_CUDA(cudaEventRecord(end_b, b));
        BSG_CUDA(cudaStreamWaitEvent(base, end_a, 0));
        BSG_CUDA(cudaStreamWaitEvent(base, end_b, 0));
        joined = true;
    }
    void release() {
        for (cudaEvent_t e : {start, end_a, end_b, u_ready[0], u_ready[1], u_done[0], u_done[1]})
            if (e) cudaEventDestroy(e);
        start = end_a = end_b = u_ready[0] = u_ready[1] = u_done[0] = u_done[1] = nullptr;
    }
    ~StreamFork() {
        if (!joined && end_a && end_b) {  // error path; nothing here throws
            cudaEventRecord(end_a, a);
            cudaEventRecord(end_b, b);
            cudaStreamWaitEvent(base, end_a, 0);
            cudaStreamWaitEvent(base, end_b, 0);
        }
        release();
    }
    StreamFork(const StreamFork &) = delete;
    StreamFork &operator=(const StreamFork &) = delete;
};

void rik_ozaki(bsg_ctx ctx, const RikDev &d, double *K_dev, double *Kmn_dev, uint64_t stats[6]) {
    cudaStream_t s = ctx->stream;
    const size_t n_bf = d.n_bf, n_occ = d.n_occ, bs = d.bs, n_aux = d.n_aux;
    BSG_REQUIRE(bs <= 64, BSG_ERR_UNSUPPORTED, "RI-K Ozaki form supports bs <= 64");
    const int nd = oz_default_digits(d.n_digits, (int)bs, (int)bs, (int)bs);
    const OzShape sh = oz_shape((int)bs, (int)bs, (int)bs, nd);
    OzDims D;
    D.n_bf = n_bf;
    D.n_occ = n_occ;
    D.bs = bs;
    D.nb = ceil_div(n_bf, bs);
    D.nob = ceil_div(n_occ, bs);
    D.mp = sh.mp;
    D.kp = sh.kp;
    D.np = sh.np;
    D.nd = nd;
    D.R = sh.R;
    // ij and K products: two occupied block columns per tile where they fit
    // (N = 2 bs per digit plane, both accumulator sets in TMEM): the A images
    // then serve twice the columns per copy and per MMA
    int J = (bs % 8 == 0 && 2 * bs <= 64 && nd * 2 * (int)bs + 8 <= 256) ? 2 : 1;
    OzShape shJ = oz_shape((int)bs, (int)bs, (int)bs * J, nd);
    if (shJ.kp != sh.kp || shJ.pair != sh.pair) {  // the A images are laid out for sh's k steps
        J = 1;
        shJ = sh;
    }
    shJ.J = J;
    D.J = J;
    // mui^T = C^T U^T: the U blocks of two aux functions per tile on the N side
    int Jm = (bs % 8 == 0 && 2 * bs <= 64 && nd * 2 * (int)bs + 8 <= 256) ? 2 : 1;
    OzShape shM = oz_shape((int)bs, (int)bs, (int)bs * Jm, nd);
    if (shM.kp != sh.kp || shM.pair != sh.pair) {
        Jm = 1;
        shM = sh;
    }
    shM.J = Jm;
    D.Jm = Jm;
    D.npm = shM.np;
    // K_mn: two basis block rows per tile on the N side where they fit
    int Jk = Jm;
    OzShape shK = Jk == 2 ? shM : sh;
    shK.J = Jk;
    D.Jk = Jk;
    D.npk = shK.np;
    D.nbp = ceil_div(D.nb, (size_t)Jk);
    const size_t b_imgK = (size_t)nd * shK.np * shK.kp;
    const size_t b_imgM = (size_t)nd * shM.np * shM.kp;  // elements per U image (Jm aux functions)
    D.npJ = shJ.np;
    D.nobp = ceil_div(D.nob, (size_t)J);
    const size_t nb = D.nb, nob = D.nob, nobp = D.nobp;
    const size_t a_img = (size_t)nd * sh.mp * sh.kp, b_img = (size_t)nd * sh.np * sh.kp;  // elements per image
    const size_t b_imgJ = (size_t)nd * shJ.np * shJ.kp;  // J-group images (N side of ij and K)
    // bytes per aux function of every per-chunk buffer
    const bool want_k = K_dev != nullptr, want_kmn = Kmn_dev != nullptr;
    const size_t Q = 8;  // aux functions per K-product tile
    const size_t per_p = nb * nb * 9 + nb * nb * b_img * 2 + n_bf * n_occ * 8 + nb * nob * 9 +
                         nb * nob * a_img * 2 + nb * nobp * b_imgJ * 2 + 3 * n_occ * n_occ * 8 + 3 * nob * nob * 9 +
                         nob * nobp * b_imgJ * 2 + (want_kmn ? nb * nob * b_img * 2 + nb * nb * bs * bs * 8 / Q : 0);
    size_t pc = d.p_chunk ? d.p_chunk : std::max<size_t>(1, (size_t)(8ull << 30) / per_p);
    pc = std::max<size_t>(1, std::min(pc, n_aux));
    const size_t n_sub_max = ceil_div(pc, Q);

    DevBuf dinv(n_bf * n_bf * 4, s), docc(nb * nb, s);
    // the U set (norms, flags, row maxima, row exponents, dense copies,
    // images) twice: the next chunk's U pass runs on a side stream while this
    // chunk's products run
    DevBuf dun[2] = {DevBuf(pc * nb * nb * 8, s), DevBuf(pc * nb * nb * 8, s)};
    DevBuf duf[2] = {DevBuf(pc * nb * nb, s), DevBuf(pc * nb * nb, s)};
    DevBuf dmui(pc * n_bf * n_occ * 8, s), dmn(pc * nb * nob * 8, s), dmf(pc * nb * nob, s);
    DevBuf dij(pc * n_occ * n_occ * 8, s), dijf(pc * nob * nob, s);
    DevBuf dijs(pc * n_occ * n_occ * 8, s), dsn(pc * nob * nob * 8, s), dsf(pc * nob * nob, s);
    DevBuf dcn(nb * nob * 8, s), dcexpC(nob * bs * 4, s), dimgCtA(nob * nb * a_img * 2, s);
    DevBuf dcmax(nb * 8, s), dmmax(pc * nob * 8, s);  // largest slot norms of the N-side screens
    DevBuf drexpU[2] = {DevBuf(pc * n_bf * 4, s), DevBuf(pc * n_bf * 4, s)};
    DevBuf dbitsU[2] = {DevBuf(pc * n_bf * 8, s), DevBuf(pc * n_bf * 8, s)};
    const size_t u_img_bytes = ceil_div(pc, (size_t)Jm) * nb * nb * b_imgM * 2;
    DevBuf dimgU[2] = {DevBuf(u_img_bytes, s), DevBuf(u_img_bytes, s)};
    DevBuf dcexpM(pc * n_occ * 4, s), dimgMB(pc * nb * nobp * b_imgJ * 2, s);
    DevBuf drexpMs(n_sub_max * n_bf * 4, s), dcexpSs(n_sub_max * n_occ * 4, s);
    // maxima bit patterns for the three exponent sets of a chunk's mui and ijs
    const size_t nbits = pc * n_occ + n_sub_max * n_bf + n_sub_max * n_occ;
    DevBuf dbits(nbits * 8, s);
    auto *bitsM = dbits.as<unsigned long long>(), *bitsMs = bitsM + pc * n_occ, *bitsSs = bitsMs + n_sub_max * n_bf;
    DevBuf dimgMA(pc * nb * nob * a_img * 2, s), dimgSB(pc * nob * nobp * b_imgJ * 2, s);
    DevBuf dKp(want_k ? n_sub_max * nobp * nb * bs * bs * J * 8 : 0, s), dcnt(6 * 8, s), dmacs(4 * 8, s);
    const size_t ng_a = ceil_div(nb, (size_t)D.R), ng_i = ceil_div(nob, (size_t)D.R);
    const size_t tiles_mui = ceil_div(pc, (size_t)Jm) * nb * ng_i, tiles_ij = pc * nobp * ng_i, tiles_K = n_sub_max * nobp * ng_a;
    DevBuf dtm(tiles_mui * sizeof(OzTile), s), dsm(tiles_mui * nb * Jm * sizeof(OzStep), s);
    DevBuf dti(tiles_ij * sizeof(OzTile), s), dsi(tiles_ij * nb * J * sizeof(OzStep), s);
    DevBuf dtk(tiles_K * sizeof(OzTile), s), dsk(tiles_K * Q * nob * J * sizeof(OzStep), s);
    // K_mn: images of mui in the B role, tiles over (sub-range, lower pair), partials
    const size_t n_pairs = kmn_pairs(D.nbp, (size_t)Jk, nb, (size_t)D.R);
    const size_t tiles_Kmn = want_kmn ? n_sub_max * n_pairs : 0;
    DevBuf dimgMT(want_kmn ? pc * nob * D.nbp * b_imgK * 2 : 0, s);
    DevBuf dKmnp(want_kmn ? n_sub_max * D.nbp * nb * bs * bs * Jk * 8 : 0, s);
    DevBuf dtkm(tiles_Kmn * sizeof(OzTile), s), dskm(tiles_Kmn * Q * nob * Jk * sizeof(OzStep), s);
    if (want_k) BSG_CUDA(cudaMemsetAsync(K_dev, 0, n_bf * n_occ * 8, s));
    if (want_kmn) BSG_CUDA(cudaMemsetAsync(Kmn_dev, 0, n_bf * n_bf * 8, s));
    BSG_CUDA(cudaMemsetAsync(dcnt.p, 0, 6 * 8, s));
    auto *cnt = dcnt.as<unsigned long long>();
    auto *macs = dmacs.as<unsigned long long>();
    const unsigned tb = (unsigned)std::max<size_t>(32, ((bs + 31) / 32) * 32);

    // call-constant operands: C norms, C column exponents, C^T images
    const int wpb = 8;
    k_cnorms<<<(unsigned)ceil_div(nb * nob, wpb), wpb * 32, 0, s>>>(d.c_occ, n_bf, n_occ, bs, nb, nob, dcn.as<double>());
    if (d.tr_c_norm) BSG_CUDA(cudaMemcpyAsync(d.tr_c_norm, dcn.p, nb * nob * 8, cudaMemcpyDeviceToDevice, s));
    k_cnorm_rowmax<<<(unsigned)ceil_div(nb, (size_t)128), 128, 0, s>>>(dcn.as<double>(), nb, nob, dcmax.as<double>());
    k_cexp_C<<<(unsigned)nob, tb, 0, s>>>(d.c_occ, n_bf, n_occ, bs, dcexpC.as<int>());
    k_img_Ct_A<<<oz_img_grid(nob * nb), 32 * kOzImgWarps, 0, s>>>(d.c_occ, dcexpC.as<int>(), D, dimgCtA.as<bf16>());
    // inverse key map of the compressed integrals (replaces the per-P dense rebuild)
    BSG_CUDA(cudaMemsetAsync(dinv.p, 0xFF, n_bf * n_bf * 4, s));
    BSG_CUDA(cudaMemsetAsync(docc.p, 0, nb * nb, s));
    if (d.n_vec2)
        k_key_inverse<<<(unsigned)ceil_div(d.n_vec2, 256), 256, 0, s>>>(d.keys, d.n_vec2, n_bf, bs, nb, dinv.as<int>(),
                                                                        docc.as<uint8_t>());
    ctx->note_launch(5);
    // the U blocks that hold any integral (the same for every P), in block order
    std::vector<uint8_t> hocc(nb * nb);
    BSG_CUDA(cudaMemcpyAsync(hocc.data(), docc.p, nb * nb, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    std::vector<uint32_t> hob;
    for (size_t rr = 0; rr < nb * nb; ++rr)
        if (hocc[rr]) hob.push_back((uint32_t)rr);
    const size_t n_ob = hob.size();
    const size_t ucomp_bytes = std::max<size_t>(1, pc * n_ob) * bs * bs * 8;
    DevBuf dob(std::max<size_t>(1, n_ob) * 4, s), ducomp[2] = {DevBuf(ucomp_bytes, s), DevBuf(ucomp_bytes, s)};
    if (n_ob) BSG_CUDA(cudaMemcpyAsync(dob.p, hob.data(), n_ob * 4, cudaMemcpyHostToDevice, s));
    const double tpb_u = 1e-20 * (double)(bs * bs);
    const double tpb = d.thresh * (double)(bs * bs * bs);

    // Two streams from here on: the products of each chunk on a high-priority
    // chain stream, the U pass of the next chunk on a low-priority side
    // stream.  u_ready[x]: U set x written; u_done[x]: the mui product that
    // read U set x finished (the set may be overwritten).  Both join the
    // caller's stream before the checks and the statistics, and on any exit.
    ctx->gemm_err_flag();  // cleared on the caller's stream, ahead of the fork
    const cudaStream_t hs = ctx->chain_stream(), ss = ctx->side_stream();
    StreamFork fork(s, hs, ss);
    auto u_pass = [&](size_t P0, int x) {
        // U_p block norms, keep flags, row exponents and digit images, all
        // gathered from the compressed integrals
        const size_t np = std::min(pc, n_aux - P0);
        BSG_CUDA(cudaMemsetAsync(dun[x].p, 0, np * nb * nb * 8, ss));
        BSG_CUDA(cudaMemsetAsync(duf[x].p, 0, np * nb * nb, ss));
        BSG_CUDA(cudaMemsetAsync(dbitsU[x].p, 0, np * n_bf * 8, ss));
        auto *bitsU = dbitsU[x].as<unsigned long long>();
        if (n_ob) {
            k_unorms_c<<<oz_img_grid(np * n_ob), 32 * kOzImgWarps, 0, ss>>>(
                d.ints, dinv.as<int>(), dob.as<uint32_t>(), n_ob, d.n_vec2, P0, n_bf, bs, nb, np, tpb_u,
                dun[x].as<double>(), duf[x].as<uint8_t>(), ducomp[x].as<double>(), bitsU);
        }
        k_bits_to_exp<<<(unsigned)ceil_div(np * n_bf, (size_t)256), 256, 0, ss>>>(bitsU, np * n_bf,
                                                                                   drexpU[x].as<int>());
        if (n_ob)
            k_img_U<<<oz_img_grid(ceil_div(np * n_ob, (size_t)kImgUBlocks)), 32 * kOzImgWarps, 0, ss>>>(
                ducomp[x].as<double>(), dob.as<uint32_t>(), n_ob, np, duf[x].as<uint8_t>(), dun[x].as<double>(),
                dcmax.as<double>(), tpb, drexpU[x].as<int>(), D, dimgU[x].as<bf16>());
        ctx->note_launch(n_ob ? 3 : 1);
        ctx->check_launch("rik ozaki U pass");
        BSG_CUDA(cudaEventRecord(fork.u_ready[x], ss));
    };
    s = hs;
    u_pass(0, 0);
    int ux = 0;  // U set of the current chunk
    for (size_t P0 = 0; P0 < n_aux; P0 += pc, ux ^= 1) {
        const size_t np = std::min(pc, n_aux - P0), n_sub = ceil_div(np, Q);
        BSG_CUDA(cudaStreamWaitEvent(s, fork.u_ready[ux], 0));
        auto &dun_ = dun[ux], &duf_ = duf[ux], &drexpU_ = drexpU[ux], &dimgU_ = dimgU[ux];
        BSG_CUDA(cudaMemsetAsync(macs, 0, 4 * 8, s));
        // mui = U C
        BSG_CUDA(cudaMemsetAsync(dbits.p, 0, nbits * 8, s));
        const size_t tm = ceil_div(np, (size_t)Jm) * nb * ng_i;
        k_tiles_mui<<<oz_img_grid(tm), 32 * kOzImgWarps, 0, s>>>(
            duf_.as<uint8_t>(), dun_.as<double>(), dcn.as<double>(), dcmax.as<double>(), drexpU_.as<int>(),
            dcexpC.as<int>(),
            dmui.as<double>(), D, np, tm, tpb, dtm.as<OzTile>(), dsm.as<OzStep>(), dmf.as<uint8_t>(), cnt + 0,
            macs + 0);
        ctx->note_launch();
        ctx->check_launch("rik ozaki mui prep");
        oz_run(ctx, shM, dtm.as<OzTile>(), tm, dsm.as<OzStep>(), dimgCtA.as<bf16>(), dimgU_.as<bf16>(), 1.0, s,
               macs + 0);
        BSG_CUDA(cudaEventRecord(fork.u_done[ux], s));
        if (P0 + pc < n_aux) {
            // the next chunk's U pass into the other set (the chunk before
            // this one has finished reading it), issued after this chunk's
            // mui product so that it runs beside the statistics and image
            // passes rather than beside a persistent GEMM's start
            if (P0 > 0) BSG_CUDA(cudaStreamWaitEvent(ss, fork.u_done[ux ^ 1], 0));
            u_pass(P0 + pc, ux ^ 1);
        }
        // mui norms, row exponents per sub-range (A operand of K and of K_mn)
        // and column exponents per aux function (B operand of ij)
        k_mui_stats<<<oz_img_grid(ceil_div(np * nb * nob, (size_t)kNormBlocks)), 32 * kOzImgWarps, 0, s>>>(
            dmui.as<double>(), dmf.as<uint8_t>(), n_bf, n_occ, bs, nb, nob, Q, np * nb * nob, dmn.as<double>(), bitsMs,
            want_k ? bitsM : nullptr);
        k_bits_to_exp<<<(unsigned)ceil_div(n_sub * n_bf, (size_t)256), 256, 0, s>>>(bitsMs, n_sub * n_bf,
                                                                                 drexpMs.as<int>());
        if (want_k)
            k_bits_to_exp<<<(unsigned)ceil_div(np * n_occ, (size_t)256), 256, 0, s>>>(bitsM, np * n_occ,
                                                                                     dcexpM.as<int>());
        // every digit image of mui in one pass
        k_img_mui_all<<<oz_img_grid(ceil_div(np * nb * nobp * J, (size_t)kImgMBlocks)), 32 * kOzImgWarps, 0, s>>>(
            dmui.as<double>(), dmf.as<uint8_t>(), dmn.as<double>(), dcmax.as<double>(), tpb, drexpMs.as<int>(), Q,
            dcexpM.as<int>(), D, np * nb * nobp * J, dimgMA.as<bf16>(), want_k ? dimgMB.as<bf16>() : nullptr,
            want_kmn ? dimgMT.as<bf16>() : nullptr);
        if (want_k)
            k_mnorm_max<<<(unsigned)ceil_div(np * nob, (size_t)128), 128, 0, s>>>(dmn.as<double>(), dmf.as<uint8_t>(),
                                                                                 np, nb, nob, dmmax.as<double>());
        ctx->note_launch(want_k ? 5 : 3);
        if (want_kmn) {
            // K_mn += mui mui^T
            const size_t tkm = n_sub * n_pairs;
            k_tiles_Kmn<<<(unsigned)ceil_div(tkm, 128), 128, 0, s>>>(
                dmf.as<uint8_t>(), dmn.as<double>(), drexpMs.as<int>(), dKmnp.as<double>(), D, np, Q, n_pairs, tkm,
                tpb, dtkm.as<OzTile>(), dskm.as<OzStep>(), cnt + 5, macs + 3);
            ctx->note_launch();
            ctx->check_launch("rik ozaki Kmn prep");
            oz_run(ctx, shK, dtkm.as<OzTile>(), tkm, dskm.as<OzStep>(), dimgMA.as<bf16>(), dimgMT.as<bf16>(), 1.0, s,
                   macs + 3);
            k_Kmn_reduce<<<(unsigned)(nb * nb), 256, 0, s>>>(dKmnp.as<double>(), n_sub, D, Kmn_dev);
            ctx->note_launch();
            ctx->check_launch("rik ozaki Kmn reduce");
        }
        if (!want_k) continue;
        // ij = C^T mui
        const size_t ti = np * nobp * ng_i;
        k_tiles_ij<<<oz_img_grid(ti), 32 * kOzImgWarps, 0, s>>>(
            dmf.as<uint8_t>(), dmn.as<double>(), dcn.as<double>(), dcmax.as<double>(), dcexpC.as<int>(),
            dcexpM.as<int>(), dij.as<double>(), D, ti, tpb, dti.as<OzTile>(), dsi.as<OzStep>(), dijf.as<uint8_t>(), cnt + 1, macs + 1);
        ctx->note_launch();
        ctx->check_launch("rik ozaki ij prep");
        oz_run(ctx, shJ, dti.as<OzTile>(), ti, dsi.as<OzStep>(), dimgCtA.as<bf16>(), dimgMB.as<bf16>(), 1.0, s,
               macs + 1);
        // ijs = ij + ij^T (FP64, with the reference's norm bookkeeping)
        k_ijs<<<(unsigned)(np * nob * nob), 128, 0, s>>>(dij.as<double>(), dijf.as<uint8_t>(), n_occ, bs, nob,
                                                          dijs.as<double>(), dsn.as<double>(), dsf.as<uint8_t>());
        rik_trace_chunk(d, P0, np, dmn.as<double>(), dmf.as<uint8_t>(), dijf.as<uint8_t>(), dsn.as<double>(),
                        dsf.as<uint8_t>(), s);
        // K += mui ijs
        k_colmax_ijs_sub<<<oz_img_grid(np * nob * nob), 32 * kOzImgWarps, 0, s>>>(
            dijs.as<double>(), dsf.as<uint8_t>(), n_occ, bs, nob, Q, np * nob * nob, bitsSs);
        k_bits_to_exp<<<(unsigned)ceil_div(n_sub * n_occ, (size_t)256), 256, 0, s>>>(bitsSs, n_sub * n_occ,
                                                                                  dcexpSs.as<int>());
        k_img_ijs_B<<<oz_img_grid(ceil_div(np * nob * nobp * J, (size_t)kImgSBlocks)), 32 * kOzImgWarps, 0, s>>>(
            dijs.as<double>(), dsf.as<uint8_t>(), dsn.as<double>(), dmmax.as<double>(), tpb, dcexpSs.as<int>(), Q, D,
            np * nob * nobp * J, dimgSB.as<bf16>());
        const size_t tk = n_sub * nobp * ng_a;
        k_tiles_K<<<oz_img_grid(tk), 32 * kOzImgWarps, 0, s>>>(
            dmf.as<uint8_t>(), dmn.as<double>(), dsf.as<uint8_t>(), dsn.as<double>(), dmmax.as<double>(),
            drexpMs.as<int>(), dcexpSs.as<int>(), dKp.as<double>(), D, np, Q, tk, tpb, dtk.as<OzTile>(), dsk.as<OzStep>(), cnt + 2,
            macs + 2);
        ctx->note_launch(5);
        ctx->check_launch("rik ozaki K prep");
        oz_run(ctx, shJ, dtk.as<OzTile>(), tk, dsk.as<OzStep>(), dimgMA.as<bf16>(), dimgSB.as<bf16>(), 1.0, s,
               macs + 2);
        k_K_reduce<<<(unsigned)(nb * nob), 256, 0, s>>>(dKp.as<double>(), n_sub, D, K_dev);
        ctx->note_launch();
        ctx->check_launch("rik ozaki K reduce");
    }
    if (want_kmn) {
        k_Kmn_mirror<<<(unsigned)ceil_div(n_bf * n_bf, (size_t)256), 256, 0, s>>>(Kmn_dev, n_bf, bs);
        ctx->note_launch();
    }
    fork.join();
    s = ctx->stream;
    ctx->gemm_check();
    if (stats) {
        unsigned long long h[6];
        BSG_CUDA(cudaMemcpyAsync(h, cnt, 6 * 8, cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i < 6; ++i) stats[i] = h[i];
    }
}

}  // namespace bsg
