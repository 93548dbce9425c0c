// Ozaki-scheme split-precision block products on tcgen05 tensor cores.
//
// Every FP64 operand row of A (column of B) is scaled by a power of two 2^e
// (max |x| < 2^e) and split into nd bf16 "digits":
//   x * 2^(7-e) = D1 + D2 + D3 + D4,  D1 = d1, D2 = d2 2^-8, D3 = d3 2^-16, ...
// with integers |d| <= 128 (7 + 8 + 8 + 8 bits).  A digit product D_i E_j is
// then an integer multiple of 2^-8(i+j-2) bounded by 2^14 2^-8(i+j-2), so a
// fp32 tensor-core accumulation of the weight-2 products (D1 E1) is exact up
// to K = 1024 and of the weight-3 products (D1 E2 + D2 E1) up to K = 512;
// lower weights carry < 2^-16 of the result and round harmlessly.  Products
// of equal weight share one TMEM region; one MMA per A digit covers all its
// partners at once: D_i x [E_1 .. E_{nd+1-i}] stacked along N.  Chains of at
// most 512 k are flushed to FP64 registers, scaled by 2^(e_r + f_c - 14) and
// summed.  With nd = 4 the representation error is below 2^-31 of each
// row/column maximum.
#pragma once
#include <cuda_bf16.h>

#include "bsg_gemm64.cuh"

namespace bsg {

constexpr int kOzMaxSlots = 8;
constexpr int kOzMaxDigits = 8;
constexpr uint32_t kOzNone = 0xFFFFFFFFu;

// Padded tile geometry for one block size.
struct OzShape {
    int mp;  // rows per slot (block rows rounded up to 8)
    int kp;  // k per step (block k rounded up to 16)
    int np;  // output columns (block cols rounded up to 8)
    int R;   // slots per 128-row tile
    int nd;  // digits per operand
    int F;   // steps per exact chain (512 / kp)
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
};

struct OzStep {
    uint32_t b;                  // B image index
    uint32_t a[kOzMaxSlots];     // A image index per slot, kOzNone = zero
};

// Runs the tiles: C_slot = alpha * sum_steps A_slot,step * B_step (+ C_slot
// unless fresh).  a_img / b_img hold nd planes per image in the UMMA layout.
// d_macs (may be null): device counter of the unpadded multiply-adds the
// tiles perform, read for the context's GEMM timing
void oz_run(bsg_ctx ctx, const OzShape &sh, const OzTile *d_tiles, size_t n_tiles, const OzStep *d_steps,
            const __nv_bfloat16 *a_img, const __nv_bfloat16 *b_img, double alpha, cudaStream_t s,
            const unsigned long long *d_macs = nullptr);

// Ozaki form of one screened product (single slice): same screening and C
// block bookkeeping as the FP64 form; items come from screened_product.
void ozaki_screened(bsg_ctx ctx, bsg_bsm C, bsg_bsm A, bsg_bsm B, const ScreenGeom &g, const std::vector<GemmItem> &items,
                    const std::vector<uint32_t> &item_ib, const std::vector<uint32_t> &item_jb, double alpha,
                    int n_digits, cudaStream_t s);

// Grouped products given as items and pairs (Strassen leaves).
void ozaki_grouped_gemm(bsg_ctx ctx, const std::vector<GemmItem> &items, const GemmItem *d_items,
                        const GemmPair *d_pairs, uint64_t n_pairs, int tA, int tB, double alpha, int max_r, int max_c,
                        size_t kbs, int n_digits, cudaStream_t s);

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

// Fixed-point split of v with row/column exponent e into nd balanced base-256
// digits, integer arithmetic only: N = round(v 2^(7 + 8(nd-1) - e)) (ties to
// even), then d_{nd-1}, ..., d_1 from the low end and d_0 = the rest
// (|d_i| <= 128).  Digit i is stored as d_i 2^(-8i).
__device__ __forceinline__ void oz_split(double v, int e, int nd, int (&d)[kOzMaxDigits]) {
    const long long bits = __double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7FF);
    long long M = (bits & 0xFFFFFFFFFFFFFll) | (E ? (1ll << 52) : 0ll);
    const int Eb = E ? E : 1;
    const int K = 7 + 8 * (nd - 1);
    const int sh = Eb - 1075 + K - e;  // N = M * 2^sh
    long long N;
    if (M == 0) {
        N = 0;
    } else if (sh >= 0) {
        N = M << sh;
    } else {
        const int s = -sh;
        if (s > 54) {
            N = 0;
        } else {
            const long long q = M >> s, rem = M & ((1ll << s) - 1), half = 1ll << (s - 1);
            N = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
        }
    }
    if (bits < 0) N = -N;
#pragma unroll
    for (int i = kOzMaxDigits - 1; i >= 1; --i) {
        if (i < nd) {
            const long long di = ((N + 128) & 255) - 128;
            d[i] = (int)di;
            N = (N - di) >> 8;
        } else {
            d[i] = 0;
        }
    }
    d[0] = (int)N;
}

// Digit image of one block, 8 consecutive k per thread and one 16-byte store
// per digit plane.  b_role false: image row r = block row, value
// src[r + l*ld]; true: image row r = output column, value src[l + r*ld].
// exps[r] is the scale exponent of image row r; rows >= `rows` and k >= `k`
// are zero.  m_side selects the layout (M side of the MMA, or N side).
__device__ __forceinline__ void oz_block_image(const double *__restrict__ src, size_t ld, bool b_role, int rows,
                                               int k, const int *__restrict__ exps, int mpad, int kp, int nd,
                                               __nv_bfloat16 *__restrict__ dst, bool m_side) {
    const size_t plane = oz_plane_stride(m_side, mpad, kp), rgs = oz_rg_stride(m_side, nd, kp);
    const int hk = kp >> 3;
    for (int idx = threadIdx.x; idx < mpad * hk; idx += blockDim.x) {
        const int r = idx % mpad, h = idx / mpad;
        const int e = r < rows ? exps[r] : 0;
        int dig[8][kOzMaxDigits];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int l = h * 8 + j;
            double v = 0.0;
            if (r < rows && l < k) v = b_role ? src[l + (size_t)r * ld] : src[r + (size_t)l * ld];
            oz_split(v, e, nd, dig[j]);
        }
        const size_t off = (size_t)(r >> 3) * rgs + (size_t)h * 64 + (size_t)(r & 7) * 8;
#pragma unroll
        for (int i = 0; i < kOzMaxDigits; ++i) {
            if (i < nd) {
                const float sc = __int_as_float((127 - 8 * i) << 23);  // 2^(-8i)
                __align__(16) __nv_bfloat16 w[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) w[j] = __float2bfloat16_rn((float)dig[j][i] * sc);
                *reinterpret_cast<uint4 *>(dst + i * plane + off) = *reinterpret_cast<const uint4 *>(w);
            }
        }
    }
}

}  // namespace bsg
