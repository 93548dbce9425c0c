// occ-RI-K exchange step (occ_ri_k_step.cpp:83-130) and the 3c->2c transform
// (3c_2c_transform.cpp:44-57), batched over the auxiliary index P.
//
// The reference runs one P at a time per OpenMP thread: scatter the
// compressed integrals of P into an N_bf^2 matrix (decompress_integrals,
// :133-146), block it with input screening, and run three screened block
// GEMMs plus a transpose-add.  Here a chunk of P values is processed per
// launch, every stage a grid over (P, block-row, block-col):
//
//   scatter  ints[:, P] -> U_P                     (HBM-bound)
//   norms    ||U_P(a,b)||, keep if >= 1e-20*bs^2   (HBM-bound)
//   mui      mui_P = U_P * C       screened, fma chains, + block norms
//   ij       ij_P  = C^T * mui_P   screened
//   ijs      ijs_P = ij_P + ij_P^T with the reference's norm bookkeeping
//   kupd     Ksub[t] += mui_P * ijs_P, P in order within partition t
//   kmn      Kmn_sub[t] += mui_P * mui_P^T (optional symmetric K_mn)
//
// and finally K = sum_t Ksub[t] in partition order (the critical section of
// :119-122 with a fixed order).  The FP64 form performs the reference's
// operation sequence element by element, so K is bit-identical to the
// reference on the deterministic BLAS definition for the same partitioning.
#include <algorithm>

#include "bsg_gemm64.cuh"
#include "bsg_rik.cuh"

namespace bsg {

constexpr int kREPT = 16;

__global__ void k_check_keys(const uint64_t *__restrict__ keys, size_t n, uint64_t limit, int *__restrict__ bad) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n && keys[v] >= limit) atomicExch(bad, 1);
}

// decompress_integrals for a chunk of P: U_p[key[v]] = ints[v + P*n_vec2]
__global__ void k_scatter(const double *__restrict__ ints, const uint64_t *__restrict__ keys, size_t n_vec2,
                          size_t P0, size_t u_stride, double *__restrict__ U) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t p = blockIdx.y;
    if (v >= n_vec2) return;
    U[p * u_stride + keys[v]] = ints[v + (P0 + p) * n_vec2];
}

// one warp per (p, a, b) block of U_p: norm and keep flag
__global__ void k_unorms(const double *__restrict__ U, size_t n_bf, size_t bs, size_t nb, size_t n_p, double tpb,
                         double *__restrict__ norm, uint8_t *__restrict__ flag) {
    const size_t x = (size_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (x >= n_p * nb * nb) return;
    const size_t p = x / (nb * nb), r = x % (nb * nb), a = r % nb, b = r / nb;
    const int rs = (int)(((a + 1) * bs <= n_bf) ? bs : n_bf - a * bs);
    const int cs = (int)(((b + 1) * bs <= n_bf) ? bs : n_bf - b * bs);
    const double est = warp_block_norm(U + p * n_bf * n_bf + a * bs + b * bs * n_bf, rs, cs, n_bf);
    if ((threadIdx.x & 31) == 0) {
        norm[x] = est;
        flag[x] = !(est < tpb);
    }
}

struct ElemMap {
    int ii[kREPT], jj[kREPT];
};

__device__ __forceinline__ void elem_map(ElemMap &m, int rows, int n) {
#pragma unroll
    for (int s = 0; s < kREPT; ++s) {
        const int e = threadIdx.x + s * blockDim.x;
        m.ii[s] = e < n ? e % rows : 0;
        m.jj[s] = e < n ? e / rows : 0;
    }
}

// acc = (first ? t : t + acc) with t the fma chain of one block product;
// opA(i,l) = tA ? A[l + i*lda] : A[i + l*lda], opB(l,j) likewise.
template <bool TA, bool TB>
__device__ __forceinline__ void chain(double (&acc)[kREPT], bool first, const ElemMap &m, int n,
                                      const double *__restrict__ A, size_t lda, const double *__restrict__ B,
                                      size_t ldb, int k) {
    double t[kREPT];
#pragma unroll
    for (int s = 0; s < kREPT; ++s) t[s] = 0.0;
    for (int l = 0; l < k; ++l) {
#pragma unroll
        for (int s = 0; s < kREPT; ++s) {
            if (threadIdx.x + s * blockDim.x < n) {
                const double a = TA ? __ldg(A + l + (size_t)m.ii[s] * lda) : __ldg(A + m.ii[s] + (size_t)l * lda);
                const double b = TB ? __ldg(B + m.jj[s] + (size_t)l * ldb) : __ldg(B + l + (size_t)m.jj[s] * ldb);
                t[s] = fma(a, b, t[s]);
            }
        }
    }
#pragma unroll
    for (int s = 0; s < kREPT; ++s) acc[s] = first ? t[s] : __dadd_rn(t[s], acc[s]);
}

__device__ __forceinline__ int ext(size_t blk, size_t bs, size_t n) {
    return (int)(((blk + 1) * bs <= n) ? bs : n - blk * bs);
}

// block norm of an output block just written by this CTA (warp 0)
__device__ __forceinline__ void cta_norm(const double *p, int rs, int cs, size_t ld, double *out) {
    __syncthreads();
    if (threadIdx.x < 32) {
        const double est = warp_block_norm(p, rs, cs, ld);
        if (threadIdx.x == 0) *out = est;
    }
}

// mui_p(a, j) = sum over surviving b of U_p(a,b) * C(b,j) (matmult with beta 0,
// occ_ri_k_step.cpp:107) followed by its block norm (:108)
__global__ void __launch_bounds__(256) k_mui(const double *__restrict__ U, const double *__restrict__ unorm,
                                             const uint8_t *__restrict__ uflag, const double *__restrict__ C,
                                             const double *__restrict__ cnorm, size_t n_bf, size_t n_occ, size_t bs,
                                             size_t nb, size_t nob, double tpb, double *__restrict__ mui,
                                             double *__restrict__ mnorm, uint8_t *__restrict__ mflag,
                                             unsigned long long *__restrict__ nsig) {
    const size_t x = blockIdx.x;  // (p, a, j)
    const size_t p = x / (nb * nob), r = x % (nb * nob), a = r % nb, j = r / nb;
    const int rows = ext(a, bs, n_bf), cols = ext(j, bs, n_occ), n = rows * cols;
    ElemMap m;
    elem_map(m, rows, n);
    double acc[kREPT];
    bool first = true;
    uint32_t cnt = 0;
    const double *Up = U + p * n_bf * n_bf;
    for (size_t b = 0; b < nb; ++b) {
        const size_t ub = p * nb * nb + a + b * nb;
        if (!uflag[ub]) continue;
        if (!(__dmul_rn(unorm[ub], cnorm[b + j * nb]) >= tpb)) continue;
        chain<false, false>(acc, first, m, n, Up + a * bs + b * bs * n_bf, n_bf, C + b * bs + j * bs * n_bf, n_bf,
                            ext(b, bs, n_bf));
        first = false;
        ++cnt;
    }
    if (threadIdx.x == 0) mflag[x] = cnt > 0;
    if (!cnt) return;
    double *out = mui + p * n_bf * n_occ + a * bs + j * bs * n_bf;
#pragma unroll
    for (int s = 0; s < kREPT; ++s)
        if (threadIdx.x + s * blockDim.x < n) out[m.ii[s] + (size_t)m.jj[s] * n_bf] = acc[s];
    cta_norm(out, rows, cols, n_bf, mnorm + x);
    if (threadIdx.x == 0) atomicAdd(nsig, (unsigned long long)cnt);
}

// ij_p(ib, jb) = sum over surviving a of C(a,ib)^T * mui_p(a,jb)  (:110)
__global__ void __launch_bounds__(256) k_ij(const double *__restrict__ C, const double *__restrict__ cnorm,
                                            const double *__restrict__ mui, const double *__restrict__ mnorm,
                                            const uint8_t *__restrict__ mflag, size_t n_bf, size_t n_occ, size_t bs,
                                            size_t nb, size_t nob, double tpb, double *__restrict__ ij,
                                            uint8_t *__restrict__ ijflag, unsigned long long *__restrict__ nsig) {
    const size_t x = blockIdx.x;  // (p, ib, jb)
    const size_t p = x / (nob * nob), r = x % (nob * nob), ib = r % nob, jb = r / nob;
    const int rows = ext(ib, bs, n_occ), cols = ext(jb, bs, n_occ), n = rows * cols;
    ElemMap m;
    elem_map(m, rows, n);
    double acc[kREPT];
    bool first = true;
    uint32_t cnt = 0;
    const double *Mp = mui + p * n_bf * n_occ;
    for (size_t a = 0; a < nb; ++a) {
        const size_t mb = p * nb * nob + a + jb * nb;
        if (!mflag[mb]) continue;
        if (!(__dmul_rn(cnorm[a + ib * nb], mnorm[mb]) >= tpb)) continue;
        chain<true, false>(acc, first, m, n, C + a * bs + ib * bs * n_bf, n_bf, Mp + a * bs + jb * bs * n_bf, n_bf,
                           ext(a, bs, n_bf));
        first = false;
        ++cnt;
    }
    if (threadIdx.x == 0) ijflag[x] = cnt > 0;
    if (!cnt) return;
    double *out = ij + p * n_occ * n_occ + ib * bs + jb * bs * n_occ;
#pragma unroll
    for (int s = 0; s < kREPT; ++s)
        if (threadIdx.x + s * blockDim.x < n) out[m.ii[s] + (size_t)m.jj[s] * n_occ] = acc[s];
    if (threadIdx.x == 0) atomicAdd(nsig, (unsigned long long)cnt);
}

// ijs = ij; ijs.add_transpose(ij) (:112-113, blocksparsematrix.hpp:224-248):
// block (ib,jb) holds [ij(ib,jb) or a fresh zero block] + ij(jb,ib)^T when
// the partner exists (norm refreshed); otherwise a copy of ij(ib,jb) whose
// cached norm stays the 0 a fresh matmult block carries.
__global__ void k_ijs(const double *__restrict__ ij, const uint8_t *__restrict__ ijflag, size_t n_occ, size_t bs,
                      size_t nob, double *__restrict__ ijs, double *__restrict__ snorm, uint8_t *__restrict__ sflag) {
    const size_t x = blockIdx.x;
    const size_t p = x / (nob * nob), r = x % (nob * nob), ib = r % nob, jb = r / nob;
    const bool self = ijflag[x] != 0;
    const bool tr = ijflag[p * nob * nob + jb + ib * nob] != 0;
    if (threadIdx.x == 0) sflag[x] = self || tr;
    if (!self && !tr) return;
    const int rows = ext(ib, bs, n_occ), cols = ext(jb, bs, n_occ);
    const double *S = ij + p * n_occ * n_occ;
    double *out = ijs + p * n_occ * n_occ + ib * bs + jb * bs * n_occ;
    for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
        const int i = e % rows, j = e / rows;
        const size_t gi = ib * bs + i, gj = jb * bs + j;
        double v = self ? S[gi + gj * n_occ] : 0.0;
        if (tr) v = __dadd_rn(v, S[gj + gi * n_occ]);
        out[i + (size_t)j * n_occ] = v;
    }
    if (tr) {
        cta_norm(out, rows, cols, n_occ, snorm + x);
    } else if (threadIdx.x == 0) {
        snorm[x] = 0.0;
    }
}

// Ksub[t](a, jb) += mui_p(a,ib) * ijs_p(ib,jb) over p of partition t in this
// chunk (in order) and surviving ib (:116; K_sub pre-filled, so beta' = 1)
__global__ void __launch_bounds__(256) k_kupd(const double *__restrict__ mui, const double *__restrict__ mnorm,
                                              const uint8_t *__restrict__ mflag, const double *__restrict__ ijs,
                                              const double *__restrict__ snorm, const uint8_t *__restrict__ sflag,
                                              size_t n_bf, size_t n_occ, size_t bs, size_t nb, size_t nob,
                                              double tpb, const uint32_t *__restrict__ plo,
                                              const uint32_t *__restrict__ phi, double *__restrict__ Ksub,
                                              unsigned long long *__restrict__ nsig) {
    const size_t x = blockIdx.x;  // (t, a, jb)
    const size_t t = x / (nb * nob), r = x % (nb * nob), a = r % nb, jb = r / nb;
    const uint32_t lo = plo[t], hi = phi[t];
    if (lo >= hi) return;
    const int rows = ext(a, bs, n_bf), cols = ext(jb, bs, n_occ), n = rows * cols;
    ElemMap m;
    elem_map(m, rows, n);
    double *K = Ksub + t * n_bf * n_occ + a * bs + jb * bs * n_bf;
    double acc[kREPT];
#pragma unroll
    for (int s = 0; s < kREPT; ++s) acc[s] = (threadIdx.x + s * blockDim.x < n) ? K[m.ii[s] + (size_t)m.jj[s] * n_bf] : 0.0;
    uint32_t cnt = 0;
    for (uint32_t p = lo; p < hi; ++p) {
        for (size_t ib = 0; ib < nob; ++ib) {
            const size_t mb = (size_t)p * nb * nob + a + ib * nb;
            const size_t sb = (size_t)p * nob * nob + ib + jb * nob;
            if (!mflag[mb] || !sflag[sb]) continue;
            if (!(__dmul_rn(mnorm[mb], snorm[sb]) >= tpb)) continue;
            chain<false, false>(acc, false, m, n, mui + (size_t)p * n_bf * n_occ + a * bs + ib * bs * n_bf, n_bf,
                                ijs + (size_t)p * n_occ * n_occ + ib * bs + jb * bs * n_occ, n_occ,
                                ext(ib, bs, n_occ));
            ++cnt;
        }
    }
#pragma unroll
    for (int s = 0; s < kREPT; ++s)
        if (threadIdx.x + s * blockDim.x < n) K[m.ii[s] + (size_t)m.jj[s] * n_bf] = acc[s];
    if (threadIdx.x == 0 && cnt) atomicAdd(nsig, (unsigned long long)cnt);
}

// K = 0; K += Ksub[t] for t in order (daxpy with a = 1, :119-122)
__global__ void k_kreduce(const double *__restrict__ Ksub, size_t n, int T, double *__restrict__ K) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    double acc = 0.0;
    for (int t = 0; t < T; ++t) acc = fma(1.0, Ksub[(size_t)t * n + e], acc);
    K[e] = acc;
}

// Kmn_sub[t](a, b) += mui_p(a,jb) * mui_p(b,jb)^T over p of partition t in
// this chunk (in order) and surviving jb: matmult(Kmn_sub, mui, N, mui, T,
// thresh, 1, 1) per P on a pre-filled Kmn_sub, the way :116 adds mui ijs.
// Lower blocks a >= b only: an upper block's chains multiply the same pairs
// in the same order (fma's product commutes), so it is the transpose bit for
// bit and the reduce mirrors it.
__global__ void __launch_bounds__(256) k_kmn_upd(const double *__restrict__ mui, const double *__restrict__ mnorm,
                                                 const uint8_t *__restrict__ mflag, size_t n_bf, size_t n_occ,
                                                 size_t bs, size_t nb, size_t nob, double tpb,
                                                 const uint32_t *__restrict__ plo, const uint32_t *__restrict__ phi,
                                                 double *__restrict__ Ksub, unsigned long long *__restrict__ nsig) {
    const size_t x = blockIdx.x;  // (t, a, b)
    const size_t t = x / (nb * nb), r = x % (nb * nb), a = r % nb, b = r / nb;
    const uint32_t lo = plo[t], hi = phi[t];
    if (a < b || lo >= hi) return;
    const int rows = ext(a, bs, n_bf), cols = ext(b, bs, n_bf), n = rows * cols;
    ElemMap m;
    elem_map(m, rows, n);
    double *K = Ksub + t * n_bf * n_bf + a * bs + b * bs * n_bf;
    double acc[kREPT];
#pragma unroll
    for (int s = 0; s < kREPT; ++s) acc[s] = (threadIdx.x + s * blockDim.x < n) ? K[m.ii[s] + (size_t)m.jj[s] * n_bf] : 0.0;
    uint32_t cnt = 0;
    for (uint32_t p = lo; p < hi; ++p) {
        const double *Mp = mui + (size_t)p * n_bf * n_occ;
        for (size_t jb = 0; jb < nob; ++jb) {
            const size_t ma = (size_t)p * nb * nob + a + jb * nb, mb = (size_t)p * nb * nob + b + jb * nb;
            if (!mflag[ma] || !mflag[mb]) continue;
            if (!(__dmul_rn(mnorm[ma], mnorm[mb]) >= tpb)) continue;
            chain<false, true>(acc, false, m, n, Mp + a * bs + jb * bs * n_bf, n_bf, Mp + b * bs + jb * bs * n_bf, n_bf,
                               ext(jb, bs, n_occ));
            ++cnt;
        }
    }
#pragma unroll
    for (int s = 0; s < kREPT; ++s)
        if (threadIdx.x + s * blockDim.x < n) K[m.ii[s] + (size_t)m.jj[s] * n_bf] = acc[s];
    if (threadIdx.x == 0 && cnt) atomicAdd(nsig, (unsigned long long)cnt);
}

// K_mn = sum_t Kmn_sub[t] in partition order; upper blocks from the lower
__global__ void k_kmn_reduce(const double *__restrict__ Ksub, size_t n_bf, size_t bs, int T, double *__restrict__ K) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_bf * n_bf) return;
    const size_t gi = e % n_bf, gj = e / n_bf;
    const size_t src = (gi / bs >= gj / bs) ? e : gj + gi * n_bf;
    double acc = 0.0;
    for (int t = 0; t < T; ++t) acc = fma(1.0, Ksub[(size_t)t * n_bf * n_bf + src], acc);
    K[e] = acc;
}

// per-block norms of the dense occupied coefficients (BlockSparseMatrix(C, bs, bs, 0.0), :85)
__global__ void k_cnorms(const double *__restrict__ C, size_t n_bf, size_t n_occ, size_t bs, size_t nb, size_t nob,
                         double *__restrict__ cnorm) {
    const size_t x = (size_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (x >= nb * nob) return;
    const size_t a = x % nb, j = x / nb;
    const double est = warp_block_norm(C + a * bs + j * bs * n_bf, ext(a, bs, n_bf), ext(j, bs, n_occ), n_bf);
    if ((threadIdx.x & 31) == 0) cnorm[x] = est;
}

static unsigned threads_for(int rows, int cols) {
    const size_t e = (size_t)rows * cols;
    return (unsigned)std::max<size_t>(32, ((ceil_div(e, kREPT) + 31) / 32) * 32);
}

void rik_trace_chunk(const RikDev &d, size_t P0, size_t np, const double *mnorm, const uint8_t *mflag,
                     const uint8_t *ijflag, const double *snorm, const uint8_t *sflag, cudaStream_t s) {
    if (!d.tr_mui_norm) return;
    const size_t nb = ceil_div(d.n_bf, d.bs), nob = ceil_div(d.n_occ, d.bs);
    const size_t m = nb * nob, o = nob * nob;
    BSG_CUDA(cudaMemcpyAsync(d.tr_mui_norm + P0 * m, mnorm, np * m * 8, cudaMemcpyDeviceToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(d.tr_mui_flag + P0 * m, mflag, np * m, cudaMemcpyDeviceToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(d.tr_ij_flag + P0 * o, ijflag, np * o, cudaMemcpyDeviceToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(d.tr_ijs_norm + P0 * o, snorm, np * o * 8, cudaMemcpyDeviceToDevice, s));
    BSG_CUDA(cudaMemcpyAsync(d.tr_ijs_flag + P0 * o, sflag, np * o, cudaMemcpyDeviceToDevice, s));
}

void rik_fp64(bsg_ctx ctx, const RikDev &d, double *K_dev, double *Kmn_dev, uint64_t stats[6]) {
    cudaStream_t s = ctx->stream;
    const size_t n_bf = d.n_bf, n_occ = d.n_occ, bs = d.bs, n_aux = d.n_aux;
    const size_t nb = ceil_div(n_bf, bs), nob = ceil_div(n_occ, bs);
    const int T = d.n_part;
    BSG_REQUIRE((size_t)bs * bs <= (size_t)kREPT * 256, BSG_ERR_UNSUPPORTED, "RI-K FP64 kernels support bs <= 64");
    // P partitions (libgomp static schedule)
    std::vector<uint32_t> plo_all(T), phi_all(T);
    for (int t = 0; t < T; ++t) {
        const size_t q = n_aux / T, r = n_aux % T, tt = (size_t)t;
        plo_all[t] = (uint32_t)(tt * q + std::min(tt, r));
        phi_all[t] = (uint32_t)(plo_all[t] + q + (tt < r ? 1 : 0));
    }
    size_t pc = d.p_chunk;
    if (!pc) pc = std::max<size_t>(1, std::min<size_t>(n_aux, (size_t)(2ull << 30) / (n_bf * n_bf * 8)));
    pc = std::min(pc, n_aux);

    DevBuf dU(pc * n_bf * n_bf * 8, s), dun(pc * nb * nb * 8, s), duf(pc * nb * nb, s);
    DevBuf dmui(pc * n_bf * n_occ * 8, s), dmn(pc * nb * nob * 8, s), dmf(pc * nb * nob, s);
    DevBuf dij(pc * n_occ * n_occ * 8, s), dijf(pc * nob * nob, s);
    DevBuf dijs(pc * n_occ * n_occ * 8, s), dsn(pc * nob * nob * 8, s), dsf(pc * nob * nob, s);
    const bool want_k = K_dev != nullptr, want_kmn = Kmn_dev != nullptr;
    DevBuf dK(want_k ? (size_t)T * n_bf * n_occ * 8 : 0, s), dcn(nb * nob * 8, s);
    DevBuf dKmn(want_kmn ? (size_t)T * n_bf * n_bf * 8 : 0, s);
    DevBuf dplo(T * 4, s), dphi(T * 4, s), dcnt(6 * 8, s);
    if (want_k) BSG_CUDA(cudaMemsetAsync(dK.p, 0, (size_t)T * n_bf * n_occ * 8, s));  // K_sub.fill_with_values(0) (:98)
    if (want_kmn) BSG_CUDA(cudaMemsetAsync(dKmn.p, 0, (size_t)T * n_bf * n_bf * 8, s));
    BSG_CUDA(cudaMemsetAsync(dcnt.p, 0, 6 * 8, s));
    auto *cnt = dcnt.as<unsigned long long>();

    const int wpb = 8;
    k_cnorms<<<(unsigned)ceil_div(nb * nob, wpb), wpb * 32, 0, s>>>(d.c_occ, n_bf, n_occ, bs, nb, nob, dcn.as<double>());
    ctx->note_launch();
    if (d.tr_c_norm) BSG_CUDA(cudaMemcpyAsync(d.tr_c_norm, dcn.p, nb * nob * 8, cudaMemcpyDeviceToDevice, s));
    const double tpb_u = 1e-20 * (double)(bs * bs);     // U_bsm threshold 1e-20 (:93)
    const double tpb = d.thresh * (double)(bs * bs * bs);  // matmult per-block threshold
    std::vector<uint32_t> plo(T), phi(T);
    for (size_t P0 = 0; P0 < n_aux; P0 += pc) {
        const size_t np = std::min(pc, n_aux - P0);
        BSG_CUDA(cudaMemsetAsync(dU.p, 0, np * n_bf * n_bf * 8, s));
        if (d.n_vec2) {
            dim3 g((unsigned)ceil_div(d.n_vec2, 256), (unsigned)np);
            k_scatter<<<g, 256, 0, s>>>(d.ints, d.keys, d.n_vec2, P0, n_bf * n_bf, dU.as<double>());
            ctx->note_launch();
        }
        k_unorms<<<(unsigned)ceil_div(np * nb * nb, wpb), wpb * 32, 0, s>>>(dU.as<double>(), n_bf, bs, nb, np, tpb_u,
                                                                            dun.as<double>(), duf.as<uint8_t>());
        ctx->note_launch();
        k_mui<<<(unsigned)(np * nb * nob), threads_for((int)bs, (int)bs), 0, s>>>(
            dU.as<double>(), dun.as<double>(), duf.as<uint8_t>(), d.c_occ, dcn.as<double>(), n_bf, n_occ, bs, nb, nob,
            tpb, dmui.as<double>(), dmn.as<double>(), dmf.as<uint8_t>(), cnt + 0);
        ctx->note_launch();
        if (want_k) {
            k_ij<<<(unsigned)(np * nob * nob), threads_for((int)bs, (int)bs), 0, s>>>(
                d.c_occ, dcn.as<double>(), dmui.as<double>(), dmn.as<double>(), dmf.as<uint8_t>(), n_bf, n_occ, bs,
                nb, nob, tpb, dij.as<double>(), dijf.as<uint8_t>(), cnt + 1);
            k_ijs<<<(unsigned)(np * nob * nob), 128, 0, s>>>(dij.as<double>(), dijf.as<uint8_t>(), n_occ, bs, nob,
                                                              dijs.as<double>(), dsn.as<double>(), dsf.as<uint8_t>());
            ctx->note_launch(2);
            rik_trace_chunk(d, P0, np, dmn.as<double>(), dmf.as<uint8_t>(), dijf.as<uint8_t>(), dsn.as<double>(),
                            dsf.as<uint8_t>(), s);
        }
        for (int t = 0; t < T; ++t) {
            const size_t lo = std::max<size_t>(plo_all[t], P0), hi = std::min<size_t>(phi_all[t], P0 + np);
            plo[t] = lo < hi ? (uint32_t)(lo - P0) : 0;
            phi[t] = lo < hi ? (uint32_t)(hi - P0) : 0;
        }
        BSG_CUDA(cudaMemcpyAsync(dplo.p, plo.data(), T * 4, cudaMemcpyHostToDevice, s));
        BSG_CUDA(cudaMemcpyAsync(dphi.p, phi.data(), T * 4, cudaMemcpyHostToDevice, s));
        if (want_k) {
            k_kupd<<<(unsigned)((size_t)T * nb * nob), threads_for((int)bs, (int)bs), 0, s>>>(
                dmui.as<double>(), dmn.as<double>(), dmf.as<uint8_t>(), dijs.as<double>(), dsn.as<double>(),
                dsf.as<uint8_t>(), n_bf, n_occ, bs, nb, nob, tpb, dplo.as<uint32_t>(), dphi.as<uint32_t>(),
                dK.as<double>(), cnt + 2);
            ctx->note_launch();
        }
        if (want_kmn) {
            k_kmn_upd<<<(unsigned)((size_t)T * nb * nb), threads_for((int)bs, (int)bs), 0, s>>>(
                dmui.as<double>(), dmn.as<double>(), dmf.as<uint8_t>(), n_bf, n_occ, bs, nb, nob, tpb,
                dplo.as<uint32_t>(), dphi.as<uint32_t>(), dKmn.as<double>(), cnt + 5);
            ctx->note_launch();
        }
        ctx->check_launch("rik chunk");
        // the host-side partition table is reused by the next chunk
        BSG_CUDA(cudaStreamSynchronize(s));
    }
    if (want_k) {
        k_kreduce<<<(unsigned)ceil_div(n_bf * n_occ, 256), 256, 0, s>>>(dK.as<double>(), n_bf * n_occ, T, K_dev);
        ctx->note_launch();
    }
    if (want_kmn) {
        k_kmn_reduce<<<(unsigned)ceil_div(n_bf * n_bf, 256), 256, 0, s>>>(dKmn.as<double>(), n_bf, bs, T, Kmn_dev);
        ctx->note_launch();
    }
    ctx->check_launch("rik reduce");
    if (stats) {
        unsigned long long h[6];
        BSG_CUDA(cudaMemcpyAsync(h, cnt, 6 * 8, cudaMemcpyDeviceToHost, s));
        BSG_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i < 6; ++i) stats[i] = h[i];
    }
}

void check_keys(bsg_ctx ctx, const uint64_t *dkeys, size_t n, uint64_t limit) {
    if (!n) return;
    cudaStream_t s = ctx->stream;
    DevBuf bad(4, s);
    BSG_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
    k_check_keys<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(dkeys, n, limit, bad.as<int>());
    ctx->note_launch();
    int h = 0;
    BSG_CUDA(cudaMemcpyAsync(&h, bad.p, 4, cudaMemcpyDeviceToHost, s));
    BSG_CUDA(cudaStreamSynchronize(s));
    // decompress_integrals asserts max key <= N_bf^2 (occ_ri_k_step.cpp:140); a
    // key equal to N_bf^2 would write past the matrix, so it is rejected too
    BSG_REQUIRE(!h, BSG_ERR_ARG, "v2m key outside the N_bf x N_bf matrix");
}

}  // namespace bsg

using namespace bsg;

namespace {

// shared body of the two RI-K entry points: either output may be NULL
bsg_status rik_entry(bsg_ctx ctx, const bsg_rik_args *a, double *K_out, double *Kmn_out, int out_where,
                     uint64_t *stats_out, int n_stats, const bsg_rik_screen_trace *trace = nullptr) {
    return guard([&] {
        BSG_REQUIRE(ctx && a && (K_out || Kmn_out), BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(a->bs > 0 && a->n_part >= 1, BSG_ERR_ARG, "block size and partition count must be positive");
        BSG_REQUIRE(a->n_bf > 0 && a->n_occ > 0, BSG_ERR_ARG, "empty basis");
        BSG_REQUIRE(a->n_vec2 == 0 || (a->ints && a->keys), BSG_ERR_ARG, "integrals or keys missing");
        BSG_REQUIRE(a->c_occ, BSG_ERR_ARG, "occupied coefficients missing");
        BSG_REQUIRE(a->form == BSG_FORM_FP64 || a->form == BSG_FORM_OZAKI, BSG_ERR_ARG, "unknown form");
        cudaStream_t s = ctx->stream;
        RikDev d;
        d.n_bf = a->n_bf;
        d.n_aux = a->n_aux;
        d.n_occ = a->n_occ;
        d.n_vec2 = a->n_vec2;
        d.bs = a->bs;
        d.thresh = a->thresh;
        d.n_part = a->n_part;
        d.p_chunk = a->p_chunk;
        d.n_digits = a->n_digits;
        DevBuf dints, dkeys, dc, dk, dkmn;
        if (a->where == BSG_HOST) {
            dints = DevBuf(a->n_vec2 * a->n_aux * 8, s);
            dkeys = DevBuf(a->n_vec2 * 8, s);
            dc = DevBuf(a->n_bf * a->n_occ * 8, s);
            if (a->n_vec2 && a->n_aux)
                BSG_CUDA(cudaMemcpyAsync(dints.p, a->ints, a->n_vec2 * a->n_aux * 8, cudaMemcpyHostToDevice, s));
            if (a->n_vec2) BSG_CUDA(cudaMemcpyAsync(dkeys.p, a->keys, a->n_vec2 * 8, cudaMemcpyHostToDevice, s));
            BSG_CUDA(cudaMemcpyAsync(dc.p, a->c_occ, a->n_bf * a->n_occ * 8, cudaMemcpyHostToDevice, s));
            d.ints = dints.as<double>();
            d.keys = dkeys.as<uint64_t>();
            d.c_occ = dc.as<double>();
        } else {
            d.ints = a->ints;
            d.keys = a->keys;
            d.c_occ = a->c_occ;
        }
        check_keys(ctx, d.keys, d.n_vec2, (uint64_t)(a->n_bf * a->n_bf));
        const size_t nk = a->n_bf * a->n_occ, nkmn = a->n_bf * a->n_bf;
        double *Kd = K_out, *Kmnd = Kmn_out;
        if (out_where == BSG_HOST) {
            if (K_out) {
                dk = DevBuf(nk * 8, s);
                Kd = dk.as<double>();
            }
            if (Kmn_out) {
                dkmn = DevBuf(nkmn * 8, s);
                Kmnd = dkmn.as<double>();
            }
        }
        // screen trace: device copies of the per-P screening state, read back at the end
        const size_t nb = ceil_div(a->n_bf, a->bs), nob = ceil_div(a->n_occ, a->bs);
        const size_t tm = a->n_aux * nb * nob, to = a->n_aux * nob * nob;
        DevBuf tmn, tmf, tif, tsn, tsf, tcn;
        if (trace) {
            BSG_REQUIRE(K_out && trace->mui_norm && trace->mui_flag && trace->ij_flag && trace->ijs_norm &&
                            trace->ijs_flag && trace->c_norm,
                        BSG_ERR_ARG, "screen trace: every array is required");
            tmn = DevBuf(tm * 8, s);
            tmf = DevBuf(tm, s);
            tif = DevBuf(to, s);
            tsn = DevBuf(to * 8, s);
            tsf = DevBuf(to, s);
            tcn = DevBuf(nb * nob * 8, s);
            BSG_CUDA(cudaMemsetAsync(tmf.p, 0, tm, s));
            BSG_CUDA(cudaMemsetAsync(tif.p, 0, to, s));
            BSG_CUDA(cudaMemsetAsync(tsf.p, 0, to, s));
            d.tr_mui_norm = tmn.as<double>();
            d.tr_mui_flag = tmf.as<uint8_t>();
            d.tr_ij_flag = tif.as<uint8_t>();
            d.tr_ijs_norm = tsn.as<double>();
            d.tr_ijs_flag = tsf.as<uint8_t>();
            d.tr_c_norm = tcn.as<double>();
        }
        uint64_t st[6] = {0, 0, 0, 0, 0, 0};
        if (d.n_aux == 0) {
            if (Kd) BSG_CUDA(cudaMemsetAsync(Kd, 0, nk * 8, s));
            if (Kmnd) BSG_CUDA(cudaMemsetAsync(Kmnd, 0, nkmn * 8, s));
        } else if (a->form == BSG_FORM_FP64) {
            rik_fp64(ctx, d, Kd, Kmnd, st);
        } else {
            rik_ozaki(ctx, d, Kd, Kmnd, st);
        }
        if (out_where == BSG_HOST) {
            if (K_out) BSG_CUDA(cudaMemcpyAsync(K_out, Kd, nk * 8, cudaMemcpyDeviceToHost, s));
            if (Kmn_out) BSG_CUDA(cudaMemcpyAsync(Kmn_out, Kmnd, nkmn * 8, cudaMemcpyDeviceToHost, s));
        }
        if (trace && d.n_aux) {
            BSG_CUDA(cudaMemcpyAsync(trace->mui_norm, tmn.p, tm * 8, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(trace->mui_flag, tmf.p, tm, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(trace->ij_flag, tif.p, to, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(trace->ijs_norm, tsn.p, to * 8, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(trace->ijs_flag, tsf.p, to, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(trace->c_norm, tcn.p, nb * nob * 8, cudaMemcpyDeviceToHost, s));
        }
        BSG_CUDA(cudaStreamSynchronize(s));
        if (stats_out)
            for (int i = 0; i < n_stats; ++i) stats_out[i] = st[i];
    });
}

}  // namespace

extern "C" bsg_status bsg_rik_occ_step(bsg_ctx ctx, const bsg_rik_args *a, double *K_out, int out_where,
                                       uint64_t stats_out[5]) {
    if (!K_out) return guard([] { BSG_REQUIRE(false, BSG_ERR_ARG, "NULL argument"); });
    return rik_entry(ctx, a, K_out, nullptr, out_where, stats_out, 5);
}

extern "C" bsg_status bsg_rik_occ_step_trace(bsg_ctx ctx, const bsg_rik_args *a, double *K_out, int out_where,
                                             uint64_t stats_out[5], const bsg_rik_screen_trace *trace) {
    if (!K_out || !trace) return guard([] { BSG_REQUIRE(false, BSG_ERR_ARG, "NULL argument"); });
    return rik_entry(ctx, a, K_out, nullptr, out_where, stats_out, 5, trace);
}

extern "C" bsg_status bsg_rik_kmn_step(bsg_ctx ctx, const bsg_rik_args *a, double *Kmn_out, double *K_out,
                                       int out_where, uint64_t stats_out[6]) {
    if (!Kmn_out) return guard([] { BSG_REQUIRE(false, BSG_ERR_ARG, "NULL argument"); });
    return rik_entry(ctx, a, K_out, Kmn_out, out_where, stats_out, 6);
}

extern "C" bsg_status bsg_3c2c_transform(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *ints_3c,
                                         const double *v_m12, int where, size_t bs, double thresh, int form,
                                         int n_digits, double *out, int out_where) {
    return bsg_3c2c_transform_nsig(ctx, n_vec2, n_aux, ints_3c, v_m12, where, bs, thresh, form, n_digits, out,
                                   out_where, nullptr);
}

extern "C" bsg_status bsg_3c2c_transform_nsig(bsg_ctx ctx, size_t n_vec2, size_t n_aux, const double *ints_3c,
                                              const double *v_m12, int where, size_t bs, double thresh, int form,
                                              int n_digits, double *out, int out_where, uint64_t *nsig_out) {
    return guard([&] {
        BSG_REQUIRE(ctx && ints_3c && v_m12 && out, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(bs > 0, BSG_ERR_ARG, "block size must be positive");
        if (form == BSG_FORM_OZAKI) {
            // dense device path: same norms and screen as the block-sparse
            // path below, products on tensor cores, output written directly
            cudaStream_t s = ctx->stream;
            DevBuf dv, dout;
            const double *v = v_m12;
            double *o = out;
            if (where == BSG_HOST) {
                dv = DevBuf(n_aux * n_aux * 8, s);
                BSG_CUDA(cudaMemcpyAsync(dv.p, v_m12, n_aux * n_aux * 8, cudaMemcpyHostToDevice, s));
                v = dv.as<double>();
            }
            if (out_where == BSG_HOST) {
                dout = DevBuf(n_vec2 * n_aux * 8, s);
                o = dout.as<double>();
            }
            if (where == BSG_HOST)  // the integrals stream in by row ranges, overlapping the transform
                transform_3c2c_ozaki_upload(ctx, n_vec2, n_aux, ints_3c, v, bs, thresh, n_digits, o, nsig_out);
            else
                transform_3c2c_ozaki(ctx, n_vec2, n_aux, ints_3c, v, bs, thresh, n_digits, o, nsig_out);
            if (out_where == BSG_HOST)
                BSG_CUDA(cudaMemcpyAsync(out, o, n_vec2 * n_aux * 8, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaStreamSynchronize(s));
            return;
        }
        bsg_bsm X = nullptr, V = nullptr, O = nullptr;
        auto cleanup = [&] {
            bsg_bsm_destroy(X);
            bsg_bsm_destroy(V);
            bsg_bsm_destroy(O);
        };
        try {
            // BlockSparseMatrix(ints, bs, bs, 0.0) for both inputs (3c_2c_transform.cpp:44-47)
            BSG_REQUIRE(bsg_bsm_create(ctx, n_vec2, n_aux, bs, bs, 0.0, nullptr, &X) == BSG_OK, BSG_ERR_NOMEM, bsg_last_error());
            BSG_REQUIRE(bsg_bsm_create(ctx, n_aux, n_aux, bs, bs, 0.0, nullptr, &V) == BSG_OK, BSG_ERR_NOMEM, bsg_last_error());
            BSG_REQUIRE(bsg_bsm_create(ctx, n_vec2, n_aux, bs, bs, 0.0, nullptr, &O) == BSG_OK, BSG_ERR_NOMEM, bsg_last_error());
            int st = bsg_bsm_copy_from_dense(X, ints_3c, where);
            if (st) throw Error{st, bsg_last_error()};
            st = bsg_bsm_copy_from_dense(V, v_m12, where);
            if (st) throw Error{st, bsg_last_error()};
            st = bsg_bsm_fill(O, 0.0);  // :54
            if (st) throw Error{st, bsg_last_error()};
            const uint64_t n = screened_product(ctx, {O}, {X}, 0, {V}, 0, {{0, 1}}, thresh, 1.0, 1.0, form, n_digits);  // :56
            if (nsig_out) *nsig_out = n;
            st = bsg_bsm_to_dense(O, out, out_where);
            if (st) throw Error{st, bsg_last_error()};
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
    });
}

// ---------------------------------------------------------------------------
// Allocation-free RI-K step.
//
// For callers that must not allocate device memory themselves: code running
// under a framework whose caching allocator owns the whole device heap (a
// cudaMalloc/cudaFree behind its back fragments that heap, and cudaFree
// synchronizes the device), services with a fixed per-process memory budget,
// and code on latency-critical streams where an allocation's implicit
// synchronization is not acceptable.  All intermediates live in one
// file-scope device array of kRikScratchBytes; every GPU that loads this
// library keeps that array until the process exits.  The first call on a
// device looks up the array's device address (cudaGetSymbolAddress) with
// that device current; make that first call before any stream capture.
// Every call reuses the same array, so calls that overlap on the GPU (other
// streams, other host threads) race on it: serialize them.  The kernels go to
// the caller's stream and use the current device's copy of the array, so the
// current device must own the stream and every buffer (checked for the
// buffers).  Without stats_out the call only enqueues work and does not wait
// for the stream: integral keys are checked on the device, a key outside the
// N_bf x N_bf matrix is skipped and K is set to NaN; with stats_out the call
// waits for its stream once and also returns BSG_ERR_ARG for such a key.
// ---------------------------------------------------------------------------

namespace bsg {

constexpr size_t kRikScratchBytes = 32ull << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_rik_scratch[kRikScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_rik_scratch_mu;
static void *g_rik_scratch_addr[kMaxDevices] = {};

// device address of g_rik_scratch on the current device (looked up once)
static void *rik_scratch_address() {
    int dev = 0;
    BSG_CUDA(cudaGetDevice(&dev));
    BSG_REQUIRE(dev >= 0 && dev < kMaxDevices, BSG_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_rik_scratch_mu);
    if (!g_rik_scratch_addr[dev]) {
        void *p = nullptr;
        BSG_CUDA(cudaGetSymbolAddress(&p, g_rik_scratch));
        BSG_REQUIRE(p != nullptr, BSG_ERR_CUDA, "cudaGetSymbolAddress returned NULL for the RI-K scratch array");
        g_rik_scratch_addr[dev] = p;
    }
    return g_rik_scratch_addr[dev];
}

// per-partition P range inside a chunk (libgomp static schedule), on device
__global__ void k_part_table(uint32_t *plo, uint32_t *phi, int T, size_t n_aux, size_t P0, size_t np) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const size_t q = n_aux / (size_t)T, r = n_aux % (size_t)T, tt = (size_t)t;
    const size_t lo_all = tt * q + (tt < r ? tt : r), hi_all = lo_all + q + (tt < r ? 1 : 0);
    const size_t lo = lo_all > P0 ? lo_all : P0, hi = hi_all < P0 + np ? hi_all : P0 + np;
    plo[t] = lo < hi ? (uint32_t)(lo - P0) : 0;
    phi[t] = lo < hi ? (uint32_t)(hi - P0) : 0;
}

// decompress_integrals without a host-side key check: a key outside the
// N_bf x N_bf matrix is skipped (never written) and raises *bad
__global__ void k_scatter_guarded(const double *__restrict__ ints, const uint64_t *__restrict__ keys, size_t n_vec2,
                                  size_t P0, size_t u_stride, double *__restrict__ U, int *__restrict__ bad) {
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t p = blockIdx.y;
    if (v >= n_vec2) return;
    const uint64_t key = keys[v];
    if (key >= (uint64_t)u_stride) {
        if (p == 0) atomicExch(bad, 1);
        return;
    }
    U[p * u_stride + key] = ints[v + (P0 + p) * n_vec2];
}

// K = NaN everywhere when a key was bad, so the error shows in the output of
// a call that does not wait for its stream
__global__ void k_poison_if_bad(double *__restrict__ K, size_t n, const int *__restrict__ bad) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n && *bad) K[e] = __longlong_as_double(0x7FF8000000000000ll);
}

// the device that owns a pointer (-1: host memory or unknown)
static int owner_device(const void *p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) ? at.device : -1;
}

struct ScratchLayout {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~size_t(255);
        return o;
    }
};

}  // namespace bsg

extern "C" bsg_status bsg_rik_occ_step_noalloc(const bsg_rik_args *a, double *K_dev, void *cuda_stream,
                                               uint64_t stats_out[5]) {
    return guard([&] {
        BSG_REQUIRE(a && K_dev, BSG_ERR_ARG, "NULL argument");
        BSG_REQUIRE(a->where == BSG_DEVICE, BSG_ERR_ARG, "the allocation-free RI-K step takes device inputs only");
        BSG_REQUIRE(a->form == BSG_FORM_FP64, BSG_ERR_UNSUPPORTED, "the allocation-free RI-K step is FP64 only");
        BSG_REQUIRE(a->bs > 0 && a->n_part >= 1 && a->n_bf > 0 && a->n_occ > 0, BSG_ERR_ARG, "bad dimensions");
        BSG_REQUIRE(a->n_vec2 == 0 || (a->ints && a->keys), BSG_ERR_ARG, "integrals or keys missing");
        BSG_REQUIRE(a->c_occ, BSG_ERR_ARG, "occupied coefficients missing");
        BSG_REQUIRE((size_t)a->bs * a->bs <= (size_t)kREPT * 256, BSG_ERR_UNSUPPORTED, "bs <= 64 required");
        int cur = 0;
        BSG_CUDA(cudaGetDevice(&cur));
        // the kernels use the current device's copy of the scratch array, so the
        // buffers (and with them the stream's work) must live on that device
        for (const void *ptr : {(const void *)K_dev, (const void *)a->c_occ, (const void *)a->ints})
            if (ptr) {
                const int od = owner_device(ptr);
                BSG_REQUIRE(od < 0 || od == cur, BSG_ERR_ARG,
                            "allocation-free RI-K step: a device buffer belongs to another device than the current one");
            }
        cudaStream_t s = (cudaStream_t)cuda_stream;
        const size_t n_bf = a->n_bf, n_occ = a->n_occ, bs = a->bs, n_aux = a->n_aux, n_vec2 = a->n_vec2;
        const size_t nb = ceil_div(n_bf, bs), nob = ceil_div(n_occ, bs);
        const int T = a->n_part;
        // fixed part, then as many aux functions per chunk as fit
        ScratchLayout fixed;
        const size_t oK = fixed.take((size_t)T * n_bf * n_occ * 8), oCn = fixed.take(nb * nob * 8),
                     oLo = fixed.take((size_t)T * 4), oHi = fixed.take((size_t)T * 4), oCnt = fixed.take(5 * 8),
                     oBad = fixed.take(8);
        auto per_chunk = [&](size_t pc) {
            ScratchLayout l;
            l.off = fixed.off;
            l.take(pc * n_bf * n_bf * 8);
            l.take(pc * nb * nb * 8);
            l.take(pc * nb * nb);
            l.take(pc * n_bf * n_occ * 8);
            l.take(pc * nb * nob * 8);
            l.take(pc * nb * nob);
            l.take(pc * n_occ * n_occ * 8);
            l.take(pc * nob * nob);
            l.take(pc * n_occ * n_occ * 8);
            l.take(pc * nob * nob * 8);
            l.take(pc * nob * nob);
            return l.off;
        };
        BSG_REQUIRE(per_chunk(1) <= kRikScratchBytes, BSG_ERR_ARG,
                    "RI-K problem too large for the 32 MiB allocation-free scratch (needs " +
                        std::to_string(per_chunk(1)) + " bytes for one aux function)");
        size_t pc = a->p_chunk ? a->p_chunk : n_aux;
        pc = std::max<size_t>(1, std::min(pc, std::max<size_t>(1, n_aux)));
        while (pc > 1 && per_chunk(pc) > kRikScratchBytes) pc = std::max<size_t>(1, pc / 2);
        unsigned char *base = static_cast<unsigned char *>(rik_scratch_address());
        ScratchLayout l;
        l.off = fixed.off;
        double *dU = (double *)(base + l.take(pc * n_bf * n_bf * 8));
        double *dun = (double *)(base + l.take(pc * nb * nb * 8));
        uint8_t *duf = base + l.take(pc * nb * nb);
        double *dmui = (double *)(base + l.take(pc * n_bf * n_occ * 8));
        double *dmn = (double *)(base + l.take(pc * nb * nob * 8));
        uint8_t *dmf = base + l.take(pc * nb * nob);
        double *dij = (double *)(base + l.take(pc * n_occ * n_occ * 8));
        uint8_t *dijf = base + l.take(pc * nob * nob);
        double *dijs = (double *)(base + l.take(pc * n_occ * n_occ * 8));
        double *dsn = (double *)(base + l.take(pc * nob * nob * 8));
        uint8_t *dsf = base + l.take(pc * nob * nob);
        double *dK = (double *)(base + oK);
        double *dcn = (double *)(base + oCn);
        uint32_t *dplo = (uint32_t *)(base + oLo), *dphi = (uint32_t *)(base + oHi);
        auto *cnt = (unsigned long long *)(base + oCnt);
        int *bad = (int *)(base + oBad);
        // the array keeps the previous call's contents: clear what accumulates
        BSG_CUDA(cudaMemsetAsync(dK, 0, (size_t)T * n_bf * n_occ * 8, s));
        BSG_CUDA(cudaMemsetAsync(cnt, 0, 5 * 8, s));
        BSG_CUDA(cudaMemsetAsync(bad, 0, 4, s));
        // keys are checked on the device (no wait for the stream here): a key
        // outside the N_bf x N_bf matrix is never written, and K becomes NaN
        const int wpb = 8;
        k_cnorms<<<(unsigned)ceil_div(nb * nob, wpb), wpb * 32, 0, s>>>(a->c_occ, n_bf, n_occ, bs, nb, nob, dcn);
        const double tpb_u = 1e-20 * (double)(bs * bs);
        const double tpb = a->thresh * (double)(bs * bs * bs);
        for (size_t P0 = 0; P0 < n_aux; P0 += pc) {
            const size_t np = std::min(pc, n_aux - P0);
            BSG_CUDA(cudaMemsetAsync(dU, 0, np * n_bf * n_bf * 8, s));
            if (n_vec2) {
                dim3 g((unsigned)ceil_div(n_vec2, 256), (unsigned)np);
                k_scatter_guarded<<<g, 256, 0, s>>>(a->ints, a->keys, n_vec2, P0, n_bf * n_bf, dU, bad);
            }
            k_unorms<<<(unsigned)ceil_div(np * nb * nb, wpb), wpb * 32, 0, s>>>(dU, n_bf, bs, nb, np, tpb_u, dun, duf);
            k_mui<<<(unsigned)(np * nb * nob), threads_for((int)bs, (int)bs), 0, s>>>(
                dU, dun, duf, a->c_occ, dcn, n_bf, n_occ, bs, nb, nob, tpb, dmui, dmn, dmf, cnt + 0);
            k_ij<<<(unsigned)(np * nob * nob), threads_for((int)bs, (int)bs), 0, s>>>(
                a->c_occ, dcn, dmui, dmn, dmf, n_bf, n_occ, bs, nb, nob, tpb, dij, dijf, cnt + 1);
            k_ijs<<<(unsigned)(np * nob * nob), 128, 0, s>>>(dij, dijf, n_occ, bs, nob, dijs, dsn, dsf);
            k_part_table<<<(unsigned)ceil_div((size_t)T, 128), 128, 0, s>>>(dplo, dphi, T, n_aux, P0, np);
            k_kupd<<<(unsigned)((size_t)T * nb * nob), threads_for((int)bs, (int)bs), 0, s>>>(
                dmui, dmn, dmf, dijs, dsn, dsf, n_bf, n_occ, bs, nb, nob, tpb, dplo, dphi, dK, cnt + 2);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) throw Error{BSG_ERR_CUDA, std::string("rik (no-alloc) chunk: ") + cudaGetErrorString(e)};
        }
        if (n_aux)
            k_kreduce<<<(unsigned)ceil_div(n_bf * n_occ, 256), 256, 0, s>>>(dK, n_bf * n_occ, T, K_dev);
        else
            BSG_CUDA(cudaMemsetAsync(K_dev, 0, n_bf * n_occ * 8, s));
        if (n_vec2 && n_aux)
            k_poison_if_bad<<<(unsigned)ceil_div(n_bf * n_occ, 256), 256, 0, s>>>(K_dev, n_bf * n_occ, bad);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) throw Error{BSG_ERR_CUDA, std::string("rik (no-alloc) reduce: ") + cudaGetErrorString(e)};
        if (stats_out) {
            // the one wait of the call: counters and the key check's verdict
            unsigned long long h[5];
            int hb = 0;
            BSG_CUDA(cudaMemcpyAsync(h, cnt, 5 * 8, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, s));
            BSG_CUDA(cudaStreamSynchronize(s));
            BSG_REQUIRE(!hb, BSG_ERR_ARG, "v2m key outside the N_bf x N_bf matrix (K set to NaN)");
            for (int i = 0; i < 5; ++i) stats_out[i] = h[i];
        }
    });
}
