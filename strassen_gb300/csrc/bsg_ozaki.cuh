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
    int mp;  // rows per slot (block rows rounded up to 16; 24 and 48 kept)
    int kp;  // k per step (block k rounded up to 16)
    int np;  // output columns (block cols rounded up to 16)
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

// device helpers shared with the RI-K pipeline
__device__ __forceinline__ int oz_exp_of(double mx) { return mx > 0.0 ? ilogb(mx) + 1 : 0; }

// element offset of (row r, k l) inside one digit plane of an image with kp
// columns: core matrices of 8x8, row groups outer, k groups inner
__device__ __forceinline__ int oz_img_off(int r, int l, int kp) {
    return (((r >> 3) * (kp >> 3) + (l >> 3)) << 6) + ((r & 7) << 3) + (l & 7);
}

// writes the nd digit planes of x (already scaled by 2^-e) at offset off
__device__ __forceinline__ void oz_digits(double x, int nd, __nv_bfloat16 *img, size_t plane_elems, size_t off) {
    double y = x * 128.0;
    double scale = 1.0;
#pragma unroll
    for (int i = 0; i < kOzMaxDigits; ++i) {
        if (i < nd) {
            const double d = rint(y);
            img[i * plane_elems + off] = __float2bfloat16_rn((float)(d * scale));
            y = (y - d) * 256.0;
            scale *= 1.0 / 256.0;
        }
    }
}

}  // namespace bsg
