// Ozaki-scheme split-precision block products on tcgen05 tensor cores.
//
// Every FP64 operand row of A (column of B) is scaled by a power of two 2^e
// (max |x| < 2^e) and split into nd bf16 "digits":
//   x * 2^(7-e) = D0 + D1 + D2 + ...,  D0 = d0, D1 = d1 2^-8, D2 = d2 2^-16, ...
// with integers |d| <= 128 (7 + 8 + 8 + ... bits).  A digit product D_i E_j
// is then an integer multiple of 2^-8(i+j) bounded by 2^14 2^-8(i+j), so a
// fp32 tensor-core accumulation of the weight-0 products (D0 E0) is exact up
// to K = 1024 and of the weight-1 products (D0 E1 + D1 E0) up to K = 512;
// weight 2 is exact while its partial sums stay below 2^8, and lower weights
// carry < 2^-24 of the result.  Products of equal weight share one TMEM
// region; one MMA per A digit covers all its partners at once: D_i x
// [E_0 .. E_{nd-1-i}] stacked along N.  Chains of at most 512 k are drained
// into an int64 (weights 0-2) and an FP32 (lower weights) accumulator and
// combined in FP64 once per tile, scaled by 2^(e_r + f_c - 14).  With nd
// digits the representation error is below 2^-(8 nd - 1) of each row/column
// maximum.
#pragma once
#include <cuda_bf16.h>

#include "bsg_digits.h"
#include "bsg_gemm64.cuh"

namespace bsg {

constexpr int kOzMaxSlots = 8;
constexpr int kOzMaxDigits = 8;
constexpr uint32_t kOzNone = 0xFFFFFFFFu;

// Padded tile geometry for one block size.
struct OzShape {
    int mp;  // rows per slot (block rows rounded up to 8)
    int kp;  // k per step (block k rounded up to 16, or to 8 in pair mode)
    int np;  // output columns (block cols rounded up to 8)
    int R;   // slots per 128-row tile
    int nd;  // digits per operand
    int F;   // steps per exact chain (F kp <= 512; even in pair mode)
    int S = 0;  // pipeline stages (0: as many as fit, at most 4)
    int J = 1;  // N-side sub-blocks of np / J rows each (a B image holds J blocks)
    // Pair mode (kp = 8 mod 16, e.g. 24-wide blocks): a stage holds two steps
    // side by side and the MMA's k16 slices run across them (the one slice
    // that straddles the two takes its second core matrix from the other
    // half through the descriptor's leading byte offset), so no step is
    // padded to a multiple of 16 in k.
    int pair = 0;
};
OzShape oz_shape(int bs_rows, int bs_k, int bs_cols, int nd);
// digits to use: `requested` (validated) or, for 0, 5 where it fits else 4
int oz_default_digits(int requested, int bs_rows, int bs_k, int bs_cols);

struct OzTile {
    double *c[kOzMaxSlots];        // output block per slot (column-major, ld = ldc), null = unused slot
    double *cnorm[kOzMaxSlots];    // cached-norm slot zeroed when the block is fresh (may be null)
    const int *rexp[kOzMaxSlots];  // row exponents of the slot's rows
    const int *cexp;               // column exponents of the tile's columns
    int rows[kOzMaxSlots];
    int ldc[kOzMaxSlots];          // leading dimension of each output block
    int cols;
    int trans;                     // 1: slot rows are output columns, tile columns output rows
    uint32_t fresh_mask;           // slot s overwrites C (bit set) or adds to it
    uint32_t s0, ns;               // step range
    // N-side sub-blocks stored apart (0: the tile's columns are contiguous):
    // with J = 2 sub-blocks of NP/2 columns, sub-block js holds sub_cols
    // valid columns at output offset js * sub_stride (elements) with column
    // exponents at cexp + js * cexp_sub
    int sub_cols = 0;
    long long sub_stride = 0;
    int cexp_sub = 0;
};

struct OzStep {
    uint32_t b;                  // B image index
    uint32_t a[kOzMaxSlots];     // A image index per slot, kOzNone = zero
    uint32_t bmask;              // N-side sub-blocks taken from B (bit j); the others are zero
};
constexpr uint32_t kOzAllSub = 0xFFFFFFFFu;

// Runs the tiles: C_slot = alpha * sum_steps A_slot,step * B_step (+ C_slot
// unless fresh).  a_img / b_img hold nd planes per image in the UMMA layout.
// d_macs (may be null): device counter of the unpadded multiply-adds the
// tiles perform, read for the context's GEMM timing.  Each persistent CTA
// takes `chunk` consecutive tiles at a time.
void oz_run(bsg_ctx ctx, const OzShape &sh, const OzTile *d_tiles, size_t n_tiles, const OzStep *d_steps,
            const __nv_bfloat16 *a_img, const __nv_bfloat16 *b_img, double alpha, cudaStream_t s,
            const unsigned long long *d_macs = nullptr, uint32_t chunk = 1);

// A run of tiles of one geometry inside a larger tile list: tiles below
// tile_end (and at or above the previous run's tile_end) have shape sh and
// take their operands from a_img / b_img.
struct OzRun {
    OzShape sh;
    const __nv_bfloat16 *a_img, *b_img;
    size_t tile_end;
};
// One persistent launch over the tiles of several geometries (at most 8
// runs, block widths up to 64): the tiles of a batch of products of
// different block sizes, in run order.  Step indices are absolute; each
// step's image indices refer to its run's images.
void oz_run_groups(bsg_ctx ctx, const std::vector<OzRun> &runs, const OzTile *d_tiles, size_t n_tiles,
                   const OzStep *d_steps, double alpha, cudaStream_t s, const unsigned long long *d_macs = nullptr);

// ---- building blocks of a mixed-form screened product ----
// row exponents of op(A), column exponents of op(B) and their digit images
// (one image per stored block, at the block's table index)
void oz_operand_images(bsg_ctx ctx, bsg_bsm A, bsg_bsm B, const ScreenGeom &g, const OzShape &sh, int *rexp,
                       int *cexp, __nv_bfloat16 *aimg, __nv_bfloat16 *bimg);
// host tile lists (tile, slot block rows, block column) appended to a plan
struct OzTilePlan {
    std::vector<OzTile> tiles;
    std::vector<uint32_t> tib, tjb;
};
// Tiles of up to sh.R items of one block column, in super-tile order; step
// ranges start at step_base (nkb per tile).  all_fresh: every item overwrites
// its block; scratch (may be null): slots write consecutive scratch blocks
// instead of C (autotuning trials).
void oz_build_tiles(bsg_ctx ctx, const ScreenItems &si, const OzShape &sh, const int *rexp, const int *cexp,
                    uint32_t step_base, bool all_fresh, double *scratch, OzTilePlan &out);
// steps of every tile (the FP64 form's screen), image indices offset by the bases
void oz_launch_steps(bsg_ctx ctx, OzTile *d_tiles, size_t n_tiles, const uint32_t *d_tib, const uint32_t *d_tjb,
                     bsg_bsm A, bsg_bsm B, const ScreenGeom &g, int R, OzStep *d_steps, unsigned long long *d_macs,
                     uint32_t a_base, uint32_t b_base);

// Ozaki form of one screened product (single slice): same screening and C
// block bookkeeping as the FP64 form; items come from screened_product.
void ozaki_screened(bsg_ctx ctx, bsg_bsm C, bsg_bsm A, bsg_bsm B, const ScreenGeom &g, const std::vector<GemmItem> &items,
                    const std::vector<uint32_t> &item_ib, const std::vector<uint32_t> &item_jb, double alpha,
                    int n_digits, cudaStream_t s);

// Dense grid products X_i += P_i Q_i (the Strassen-Winograd leaves): n_prod
// products of n x n grids of bs x bs blocks; X, P, Q hold the device block
// pointers of every grid, column-major, product after product.
void ozaki_grid_products(bsg_ctx ctx, size_t n_prod, size_t n, const std::vector<double *> &X,
                         const std::vector<double *> &P, const std::vector<double *> &Q, int bs, int n_digits,
                         cudaStream_t s);

// ---- device helpers shared with the RI-K pipeline ----

// |x| as an ordered integer (non-negative doubles compare like their bits)
__device__ __forceinline__ long long oz_absbits(double x) {
    return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFll;
}

// scale exponent e of a row/column whose largest |x| has bit pattern mb:
// max < 2^e, i.e. the frexp exponent (0 for an all-zero row)
__device__ __forceinline__ int oz_exp_of_bits(long long mb) {
    if (mb == 0) return 0;
    const int E = (int)((mb >> 52) & 0x7FF);
    if (E) return E - 1022;
    return ilogb(__longlong_as_double(mb)) + 1;  // subnormal
}
__device__ __forceinline__ int oz_exp_of(double mx) { return oz_exp_of_bits(oz_absbits(mx)); }

// Digit-image layouts (UMMA K-major canonical form without swizzle: core
// matrices of 8 rows x 16 bytes, the kp/8 core matrices of an 8-row group
// adjacent along k).
//  N side (B operand): digit planes one after another, each mpad rows
//    (8-row groups kp*8 elements apart) -- a block's planes stack along N.
//  M side (A operand): digits interleaved per 8-row group (group g holds
//    digit 0..nd-1 of its 8 rows, kp*8 elements each), so that a block's full
//    image is one contiguous run and consecutive blocks of a tile's slots
//    are one contiguous run too; digit i is then addressed at offset
//    i*kp*8 with an 8-row-group stride of nd*kp*8.
__device__ __forceinline__ size_t oz_rg_stride(bool m_side, int nd, int kp) {
    return m_side ? (size_t)nd * kp * 8 : (size_t)kp * 8;
}
__device__ __forceinline__ size_t oz_plane_stride(bool m_side, int mpad, int kp) {
    return m_side ? (size_t)kp * 8 : (size_t)mpad * kp;
}

// Fixed-point value of v with row/column exponent e, integer arithmetic only:
// N = round(v 2^(K - e)) with ties to even (|N| <= 2^K); see bsg_digits.h.
__device__ __forceinline__ long long oz_fixed(double v, int e, int K) {
    return oz_fixed_bits((unsigned long long)__double_as_longlong(v), e, K);
}

// Split into nd balanced base-256 digits: N = d_0 256^(nd-1) + ... + d_{nd-1}
// with d_1.. in [-128, 127] and d_0 in [-128, 128], K = 7 + 8(nd-1).  Adding
// 128 to each of the nd-1 low bytes (the constant 0x80..80) makes them plain
// bytes of T = N + C (d_i = byte - 128) and leaves d_0 = T >> 8(nd-1).  Up to
// 5 digits the low bytes sit in T's low 32 bits and are read from there.
struct OzDigits {
    long long T;
    int lowb;  // 8 (nd - 1)
    __device__ __forceinline__ OzDigits(double v, int e, int nd) {
        lowb = 8 * (nd - 1);
        const long long C = nd > 1 ? (long long)(0x8080808080808080ull >> (64 - lowb)) : 0;
        T = oz_fixed(v, e, 7 + lowb) + C;
        neg = __double_as_longlong(v) < 0;  // the sign bit (an integer test, not an FP64 compare)
    }
    bool neg;
    __device__ __forceinline__ int digit(int i) const {
        if (i == 0) {
            const int d0 = (int)(T >> lowb);
            // only at 8 digits can T overflow (N = +2^63 wraps)
            return (lowb == 56 && d0 < 0 && !neg) ? d0 + 256 : d0;
        }
        if (lowb <= 32) return (int)(((unsigned int)T >> (lowb - 8 * i)) & 255u) - 128;
        return (int)((T >> (lowb - 8 * i)) & 255) - 128;
    }
    // float bits of d_i 2^(-8i), sc = 2^(-8i): exact (a digit has at most 8
    // significant bits, the product stays a normal float for i <= 7, zero
    // stays zero), and the high half is the bf16 of the same value.  FP32
    // multiplies and fmas stand in for integer subtracts and zero tests: the
    // split is bound by the integer pipe.  Up to 5 digits a low digit is a
    // byte of T's low word (one byte permute) and (byte - 128) sc is one fma.
    __device__ __forceinline__ uint32_t digit_f32(int i, float sc) const {
        if (i > 0 && lowb <= 32) {
            const uint32_t b = __byte_perm((uint32_t)T, 0u, 0x4440u | (uint32_t)((lowb >> 3) - i));
            return __float_as_uint(fmaf((float)b, sc, -128.0f * sc));
        }
        return __float_as_uint((float)digit(i) * sc);
    }
};

// One item of a block's digit image from a value source get(r, l) (image row
// r, k l): image row r = idx % mpad, 8 consecutive k from h*8, h = idx / mpad,
// one 16-byte store per digit plane.  exps[r] is the scale exponent of image
// row r; rows >= `rows` and k >= `k` are zero.  m_side selects the layout (M
// side of the MMA, or N side); plane_rows (N side): rows of the image the
// block is part of (a group of blocks stacked along N), 0 = mpad.
template <class Get>
__device__ __forceinline__ void oz_image_item(const Get &get, int rows, int k, const int *__restrict__ exps, int mpad,
                                              int kp, int nd, __nv_bfloat16 *__restrict__ dst, bool m_side,
                                              int plane_rows, int idx) {
    const size_t plane = oz_plane_stride(m_side, plane_rows ? plane_rows : mpad, kp), rgs = oz_rg_stride(m_side, nd, kp);
    const int r = idx % mpad, h = idx / mpad;
    const size_t off = (size_t)(r >> 3) * rgs + (size_t)h * 64 + (size_t)(r & 7) * 8;
    if (r >= rows || h * 8 >= k) {  // padding: all digits zero
        for (int i = 0; i < nd; ++i) *reinterpret_cast<uint4 *>(dst + i * plane + off) = make_uint4(0, 0, 0, 0);
        return;
    }
    const int e = exps[r];
    double v[8];  // the eight loads first, then the splits
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = h * 8 + j < k ? get(r, h * 8 + j) : 0.0;
    OzDigits D[8] = {OzDigits(v[0], e, nd), OzDigits(v[1], e, nd), OzDigits(v[2], e, nd), OzDigits(v[3], e, nd),
                     OzDigits(v[4], e, nd), OzDigits(v[5], e, nd), OzDigits(v[6], e, nd), OzDigits(v[7], e, nd)};
    // one digit plane at a time: four packed words live, not nd x 4
    for (int i = 0; i < nd; ++i) {
        const float sc = __int_as_float((127 - 8 * i) << 23);  // 2^(-8i)
        uint32_t w[4];  // two bf16 = the high halves of two floats (one byte permute)
#pragma unroll
        for (int q = 0; q < 4; ++q) w[q] = __byte_perm(D[2 * q].digit_f32(i, sc), D[2 * q + 1].digit_f32(i, sc), 0x7632);
        *reinterpret_cast<uint4 *>(dst + i * plane + off) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// Digit image of one block, items spread over threads tid, tid + nthr, ...
template <class Get>
__device__ __forceinline__ void oz_block_image_g(const Get &get, int rows, int k, const int *__restrict__ exps, int mpad,
                                                 int kp, int nd, __nv_bfloat16 *__restrict__ dst, bool m_side, int tid,
                                                 int nthr, int plane_rows = 0) {
    for (int idx = tid; idx < mpad * (kp >> 3); idx += nthr)
        oz_image_item(get, rows, k, exps, mpad, kp, nd, dst, m_side, plane_rows, idx);
}

// value source of a column-major block: b_role false: src[r + l*ld] (image
// row = block row); true: src[l + r*ld] (image row = block column)
struct OzDenseGet {
    const double *src;
    size_t ld;
    bool b_role;
    __device__ __forceinline__ double operator()(int r, int l) const {
        return b_role ? src[l + (size_t)r * ld] : src[r + (size_t)l * ld];
    }
};

// Digit image of one column-major block, built by one warp.
__device__ __forceinline__ void oz_block_image(const double *__restrict__ src, size_t ld, bool b_role, int rows,
                                               int k, const int *__restrict__ exps, int mpad, int kp, int nd,
                                               __nv_bfloat16 *__restrict__ dst, bool m_side) {
    oz_block_image_g(OzDenseGet{src, ld, b_role}, rows, k, exps, mpad, kp, nd, dst, m_side, threadIdx.x & 31, 32);
}

// One block image of a warp's job list (see oz_jobs_image); rows < 0: none
struct OzImgJob {
    OzDenseGet get;
    int rows, k;
    const int *exps;
    __nv_bfloat16 *dst;
    int plane_rows;
    bool m_side;
};

// Digit images of n_jobs <= 32 blocks by one warp, the items of consecutive
// jobs back to back: a 24 x 24 block has 72 items, so one block per warp
// leaves a quarter of the lanes idle in its last pass (the image kernels are
// bound by the integer pipe).  Lane j describes job j once, job(j, J)
// returning false for a job without an image, into the warp's table sj in
// shared memory, which the items read.  Every job has the same mpad, kp and
// nd.  The whole warp calls this.
template <class JobFn>
__device__ __forceinline__ void oz_jobs_image(int n_jobs, const JobFn &job, int mpad, int kp, int nd,
                                              OzImgJob *__restrict__ sj) {
    const int lane = threadIdx.x & 31, per = mpad * (kp >> 3);
    if (lane < n_jobs) {
        OzImgJob J;
        if (!job(lane, J)) J.rows = -1;
        sj[lane] = J;
    }
    __syncwarp();
    for (int it = lane; it < n_jobs * per; it += 32) {
        const int j = it / per;
        const OzImgJob &J = sj[j];
        if (J.rows >= 0)
            oz_image_item(J.get, J.rows, J.k, J.exps, mpad, kp, nd, J.dst, J.m_side, J.plane_rows, it - j * per);
    }
    __syncwarp();
}

// One k step of a tile whose N side holds J block columns: live[j] = slots
// whose product with sub-block j survives.  The pairs are split into exact
// rectangles (slot set x sub-block set), each one step: the slots common to
// every sub-block that still has some, then the rest (at most J steps).
// Sub-blocks past the last block column count as present: their image rows
// are zero, so a rectangle may include them and keep the single B copy.
__device__ __forceinline__ uint32_t emit_rect_steps(uint32_t (&live)[2], int J, uint32_t phantom, uint32_t b,
                                                    const uint32_t (&a_idx)[kOzMaxSlots], OzStep *__restrict__ out) {
    uint32_t n = 0;
    for (int guard = 0; guard < 2 * 2; ++guard) {
        uint32_t common = 0xFFFFFFFFu, jset = 0;
        for (int j = 0; j < J; ++j)
            if (live[j]) {
                common &= live[j];
                jset |= 1u << j;
            }
        if (!jset) break;
        if (!common) {
            for (int j = 0; j < J; ++j)
                if (live[j]) {
                    common = live[j];
                    jset = 1u << j;
                    break;
                }
        }
        OzStep st;
        st.b = b;
        st.bmask = ((jset | phantom) == (1u << J) - 1u) ? kOzAllSub : jset;
        for (int sl = 0; sl < kOzMaxSlots; ++sl) st.a[sl] = ((common >> sl) & 1u) ? a_idx[sl] : kOzNone;
        out[n++] = st;
        for (int j = 0; j < J; ++j)
            if ((jset >> j) & 1u) live[j] &= ~common;
    }
    return n;
}

// Warp-built step lists: lane l holds the (at most 2) steps of the tile's
// k step base + l; they are written after the n steps already there, in
// lane order, which is the order a serial loop over the k steps gives.
__device__ __forceinline__ void warp_append_steps(const OzStep (&mine)[2], uint32_t cnt, OzStep *__restrict__ out,
                                                  uint32_t &n) {
    const int lane = threadIdx.x & 31;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t excl = incl - cnt;
    for (uint32_t i = 0; i < cnt; ++i) out[n + excl + i] = mine[i];
    n += __shfl_sync(0xffffffffu, incl, 31);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// warp maximum of a 64-bit value by two 32-bit reductions: the high words,
// then the low words of the lanes that hold the high maximum
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    const uint32_t hi = __reduce_max_sync(0xffffffffu, (uint32_t)(v >> 32));
    const uint32_t lo = __reduce_max_sync(0xffffffffu, (uint32_t)(v >> 32) == hi ? (uint32_t)v : 0u);
    return ((unsigned long long)hi << 32) | lo;
}

// exponents from maxima bit patterns (bsg_ozaki.cu): exps[i] = frexp exponent of bits[i]
__global__ void k_bits_to_exp(const unsigned long long *__restrict__ bits, size_t n, int *__restrict__ exps);

// one warp per item: global warp index and a guard for launches of 8 warps per CTA
constexpr int kOzImgWarps = 8;
__device__ __forceinline__ size_t oz_warp_id() { return (size_t)blockIdx.x * kOzImgWarps + (threadIdx.x >> 5); }
inline unsigned oz_img_grid(size_t n) { return (unsigned)((n + kOzImgWarps - 1) / kOzImgWarps); }

}  // namespace bsg
