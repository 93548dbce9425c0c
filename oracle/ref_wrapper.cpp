// C entry points over the UNMODIFIED reference headers (test infrastructure
// only).  Compiled by oracle/build_ref.sh straight from the reference's source
// directory into oracle/_ref/libref.so, linked with the deterministic BLAS
// shim (naive_blas.c) instead of MKL.  Used to pin the C restatement
// (bsm_oracle.c) and to generate golden fixtures; never shipped.
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

// same include order as the reference drivers (occ_ri_k_step.cpp:1-5)
#include "matrix.h"
#include "matrix.hpp"
#include "blocksparsematrix.h"
#include "blocksparsematrix.hpp"
#include "strassen.hpp"

// The reference defines this knob in main.cpp:9, whose main() is disabled.
size_t min_size_for_strassen = 0;

using BSM = BlockSparseMatrix<double>;

static void export_bsm(const BSM& m, double* dense, uint8_t* mask, double* norms) {
    if (dense) {
        auto d = m.to_matrix();
        std::memcpy(dense, d.data_ptr(), sizeof(double) * m.nrow() * m.ncol());
    }
    for (size_t b = 0; b < m.nblocks(); ++b) {
        const size_t rb = b % m.nrowblocks(), cb = b / m.nrowblocks();
        if (mask) mask[b] = m.block(rb, cb).size() != 0;
        if (norms) norms[b] = m.block(rb, cb).frobenius_norm();
    }
}

extern "C" {

// C = alpha*op(A)*op(B) + beta*C via matmult(BSM) blocksparsematrix.hpp:293.
// c_mode: 0 = C empty, 1 = C.fill_with_values(c_fill), 2 = C from c_in with
// threshold c_thresh.  A and B are built from dense inputs with a_thresh /
// b_thresh (blocksparsematrix.hpp:35-61).  Returns C dense, its block mask and
// its cached block norms.
int ref_matmult(size_t a_nr, size_t a_nc, const double* a_in, double a_thresh, size_t a_bsr, size_t a_bsc,
                size_t b_nr, size_t b_nc, const double* b_in, double b_thresh, size_t b_bsr, size_t b_bsc, int tA,
                int tB, int c_mode, double c_fill, const double* c_in, double c_thresh, double thresh, double alpha,
                double beta, double* c_out, uint8_t* c_mask, double* c_norms) {
    omp_set_num_threads(1);
    BSM A(a_in, a_nr, a_nc, a_bsr, a_bsc, a_thresh);
    BSM B(b_in, b_nr, b_nc, b_bsr, b_bsc, b_thresh);
    const size_t c_nr = tA ? a_nc : a_nr, c_nc = tB ? b_nr : b_nc;
    const size_t c_bsr = tA ? a_bsc : a_bsr, c_bsc = tB ? b_bsr : b_bsc;
    BSM C(c_nr, c_nc, c_bsr, c_bsc, c_thresh);
    if (c_mode == 1) C.fill_with_values(c_fill);
    if (c_mode == 2) C.copy_from_input_array(c_in);
    matmult(C, A, tA != 0, B, tB != 0, thresh, alpha, beta);
    export_bsm(C, c_out, c_mask, c_norms);
    return 0;
}

// matmult_strassen_sparse strassen.hpp:688 on A, B built from dense inputs
// at threshold in_thresh; C.fill_with_values(0) first (main.cpp:57).
int ref_strassen(size_t n, size_t bs, const double* a_in, const double* b_in, double in_thresh, double thresh,
                 size_t min_size, double* c_out) {
    omp_set_num_threads(1);
    min_size_for_strassen = min_size;
    BSM A(a_in, n, n, bs, bs, in_thresh);
    BSM B(b_in, n, n, bs, bs, in_thresh);
    BSM C(n, n, bs, bs, 0.0);
    C.fill_with_values(0.0);
    matmult_strassen_sparse(C, A, false, B, false, thresh, 1.0, 1.0);
    export_bsm(C, c_out, nullptr, nullptr);
    return 0;
}

// matmult_strassen_dryrun strassen.hpp:511; tree bits of all levels
// concatenated (level l has ceil(nb/2^(l+1))^3 entries).
int ref_dryrun(size_t n, size_t bs, const double* a_in, const double* b_in, double in_thresh,
               double thresh_per_block, int* n_levels, uint8_t* tree_out, size_t tree_cap) {
    omp_set_num_threads(1);
    BSM A(a_in, n, n, bs, bs, in_thresh);
    BSM B(b_in, n, n, bs, bs, in_thresh);
    auto tree = matmult_strassen_dryrun(A, B, thresh_per_block);
    *n_levels = (int)tree.size();
    size_t off = 0;
    for (auto& lv : tree) {
        if (off + lv.size() > tree_cap) return 2;
        for (size_t i = 0; i < lv.size(); ++i) tree_out[off + i] = lv[i] ? 1 : 0;
        off += lv.size();
    }
    return 0;
}

// The block-sparse loop of occ_ri_k_step.cpp:83-130 written against the
// reference classes, with the P loop split into n_part static partitions run
// one after another and summed in partition order (the deterministic reading
// of the OpenMP team + critical section).
int ref_rik_occ_step(size_t N_bf, size_t N_aux, size_t N_occ, size_t N_vec2, const double* ints,
                     const uint64_t* keys, const double* c_occ, size_t bs, double thresh, int n_part,
                     double* k_out) {
    omp_set_num_threads(1);
    Matrix<double> ints_3c(ints, N_vec2, N_aux);
    Matrix<double> occ_MOs(c_occ, N_bf, N_occ);
    Matrix<size_t> v2m_keys(N_vec2, 1);
    for (size_t v = 0; v < N_vec2; ++v) v2m_keys.elem(v, 0) = (size_t)keys[v];
    BSM K_bsm(N_bf, N_occ, bs, bs, 0.0);
    BSM C_bsm(occ_MOs, bs, bs, 0.0);
    K_bsm.fill_with_values(0.e0);
    for (int t = 0; t < n_part; ++t) {
        Matrix<double> U(0.e0, N_bf, N_bf);
        BSM U_bsm(N_bf, N_bf, bs, bs, 1e-20);
        BSM mui(N_bf, N_occ, bs, bs, 0.0);
        BSM ij(N_occ, N_occ, bs, bs, 0.0);
        BSM ijs(ij);
        BSM Ksub(N_bf, N_occ, bs, bs, 0.0);
        Ksub.fill_with_values(0.e0);
        const size_t q = N_aux / (size_t)n_part, r = N_aux % (size_t)n_part, tt = (size_t)t;
        const size_t lo = tt * q + (tt < r ? tt : r), hi = lo + q + (tt < r ? 1 : 0);
        for (size_t P = lo; P < hi; ++P) {
            double* u = U.data_ptr();
            const double* cp = &ints_3c.elem(0, P);
            for (size_t v = 0; v < N_vec2; ++v) u[v2m_keys.elem(v, 0)] = cp[v];
            U_bsm.copy_from_input_matrix(U);
            matmult(mui, U_bsm, false, C_bsm, false, thresh, 1.0, 0.0);
            mui.calc_frobenius_norms();
            matmult(ij, C_bsm, true, mui, false, thresh, 1.0, 0.0);
            ijs = ij;
            ijs.add_transpose(ij);
            matmult(Ksub, mui, false, ijs, false, thresh, 1.0, 1.0);
        }
        K_bsm += Ksub;
    }
    export_bsm(K_bsm, k_out, nullptr, nullptr);
    return 0;
}

// K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i) on the reference classes: the occ
// step's mui_P (occ_ri_k_step.cpp:102-108) followed by the screened
// matmult(Kmn_sub, mui, N, mui, T, thresh, 1, 1), partitions as above.
int ref_rik_kmn_step(size_t N_bf, size_t N_aux, size_t N_occ, size_t N_vec2, const double* ints,
                     const uint64_t* keys, const double* c_occ, size_t bs, double thresh, int n_part,
                     double* kmn_out) {
    omp_set_num_threads(1);
    Matrix<double> ints_3c(ints, N_vec2, N_aux);
    Matrix<double> occ_MOs(c_occ, N_bf, N_occ);
    Matrix<size_t> v2m_keys(N_vec2, 1);
    for (size_t v = 0; v < N_vec2; ++v) v2m_keys.elem(v, 0) = (size_t)keys[v];
    BSM K_bsm(N_bf, N_bf, bs, bs, 0.0);
    BSM C_bsm(occ_MOs, bs, bs, 0.0);
    K_bsm.fill_with_values(0.e0);
    for (int t = 0; t < n_part; ++t) {
        Matrix<double> U(0.e0, N_bf, N_bf);
        BSM U_bsm(N_bf, N_bf, bs, bs, 1e-20);
        BSM mui(N_bf, N_occ, bs, bs, 0.0);
        BSM Ksub(N_bf, N_bf, bs, bs, 0.0);
        Ksub.fill_with_values(0.e0);
        const size_t q = N_aux / (size_t)n_part, r = N_aux % (size_t)n_part, tt = (size_t)t;
        const size_t lo = tt * q + (tt < r ? tt : r), hi = lo + q + (tt < r ? 1 : 0);
        for (size_t P = lo; P < hi; ++P) {
            double* u = U.data_ptr();
            const double* cp = &ints_3c.elem(0, P);
            for (size_t v = 0; v < N_vec2; ++v) u[v2m_keys.elem(v, 0)] = cp[v];
            U_bsm.copy_from_input_matrix(U);
            matmult(mui, U_bsm, false, C_bsm, false, thresh, 1.0, 0.0);
            mui.calc_frobenius_norms();
            matmult(Ksub, mui, false, mui, true, thresh, 1.0, 1.0);
        }
        K_bsm += Ksub;
    }
    export_bsm(K_bsm, kmn_out, nullptr, nullptr);
    return 0;
}

// Sequence of container operations for parity of the block-level API:
// op 0: lhs += rhs, 1: lhs -= rhs, 2: lhs.add_transpose(rhs), 3: lhs *= s,
// 4: lhs.recompress(), 5: lhs.calc_frobenius_norms().  lhs/rhs built from
// dense at their thresholds.  Returns lhs dense, mask, norms and the
// accumulated frobenius_norm().
int ref_bsm_op(int op, size_t nr, size_t nc, size_t bsr, size_t bsc, const double* lhs_in, double lhs_thresh,
               const double* rhs_in, double rhs_thresh, double s, double* out, uint8_t* mask, double* norms,
               double* fro) {
    omp_set_num_threads(1);
    BSM L(lhs_in, nr, nc, bsr, bsc, lhs_thresh);
    const bool tr = op == 2;
    BSM R(rhs_in, tr ? nc : nr, tr ? nr : nc, tr ? bsc : bsr, tr ? bsr : bsc, rhs_thresh);
    switch (op) {
        case 0: L += R; break;
        case 1: L -= R; break;
        case 2: L.add_transpose(R); break;
        case 3: L *= s; break;
        case 4: L.recompress(); break;
        case 5: L.calc_frobenius_norms(); break;
        default: return 1;
    }
    export_bsm(L, out, mask, norms);
    *fro = L.frobenius_norm();
    return 0;
}

}  // extern "C"
