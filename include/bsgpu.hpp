/* C++ facade over libbsgpu's C ABI with the reference's interface:
 * Matrix<T> (matrix.h: host column-major storage and its binary file format,
 * matrix.hpp:200-227), BlockSparseMatrix<double> (blocksparsematrix.h:24-99),
 * matmult (blocksparsematrix.hpp:293-414), matmult_strassen_sparse
 * (strassen.hpp:687-753) with the global min_size_for_strassen (main.cpp:9).
 *
 * Error behaviour is the reference's: a failed call prints its message and
 * exits with status 1 (the reference asserts or calls exit(1) on dimension
 * mismatches, matrix.hpp:64-74); nothing is thrown.
 *
 * Header-only; link with -lbsgpu. */
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <type_traits>
#include <utility>
#include <vector>

#include "bsgpu.h"

namespace bsgpu {

inline void check(bsg_status st, const char *what) {
    if (st != BSG_OK) {
        std::fprintf(stderr, "%s failed: %s\n", what, bsg_last_error());
        std::exit(1);
    }
}

/* one context (device 0, library-owned stream) shared by every object */
inline bsg_ctx default_ctx() {
    static bsg_ctx ctx = [] {
        bsg_ctx c = nullptr;
        check(bsg_ctx_create(0, nullptr, &c), "bsg_ctx_create");
        return c;
    }();
    return ctx;
}

/* Host column-major matrix (the subset of matrix.h the drivers use) and the
 * reference's raw binary format: nrow*ncol elements of T, column-major, no
 * header, read or written at an element offset (matrix.hpp:200-227). */
template <typename T>
class Matrix {
  public:
    Matrix() = default;
    Matrix(size_t nr, size_t nc) : nr_(nr), nc_(nc), d_(nr * nc) {}
    Matrix(T v, size_t nr, size_t nc) : nr_(nr), nc_(nc), d_(nr * nc, v) {}
    size_t nrow() const { return nr_; }
    size_t ncol() const { return nc_; }
    size_t size() const { return d_.size(); }
    T *data_ptr() { return d_.data(); }
    const T *data_ptr() const { return d_.data(); }
    T &operator()(size_t r, size_t c) { return d_[r + c * nr_]; }
    const T &operator()(size_t r, size_t c) const { return d_[r + c * nr_]; }
    void fill_with_values(T v) { std::fill(d_.begin(), d_.end(), v); }
    double calc_frobenius_norm() const {
        double s = 0.0;
        for (const T &x : d_) s += (double)x * (double)x;
        return std::sqrt(s);
    }
    Matrix operator-(const Matrix &o) const {
        if (o.nr_ != nr_ || o.nc_ != nc_) {
            std::fprintf(stderr, "Matrix::operator-: dimension mismatch\n");
            std::exit(1);
        }
        Matrix r(nr_, nc_);
        for (size_t i = 0; i < d_.size(); ++i) r.d_[i] = d_[i] - o.d_[i];
        return r;
    }
    /* matrix.hpp:200-218: the file must hold at least size() elements past the offset */
    void read_from_file(const char *filename, size_t start_offset_in_file = 0) {
        FILE *f = std::fopen(filename, "rb");
        if (!f) {
            std::printf("File %s not available\n", filename);
            std::exit(1);
        }
        std::fseek(f, 0, SEEK_END);
        const size_t file_elems = (size_t)std::ftell(f) / sizeof(T);
        if (file_elems < start_offset_in_file || file_elems - start_offset_in_file < size()) {
            std::fprintf(stderr, "read_from_file: %s is too small for %zu x %zu\n", filename, nr_, nc_);
            std::exit(1);
        }
        std::fseek(f, (long)(start_offset_in_file * sizeof(T)), SEEK_SET);
        if (size() && std::fread(d_.data(), sizeof(T), size(), f) == 0) {
            std::fprintf(stderr, "read_from_file: read error on %s\n", filename);
            std::exit(1);
        }
        std::fclose(f);
    }
    /* matrix.hpp:220-226 */
    void write_to_file(const char *filename, size_t start_offset_in_file = 0) const {
        FILE *f = std::fopen(filename, "wb");
        if (!f) {
            std::printf("File %s not available\n", filename);
            std::exit(1);
        }
        std::fseek(f, (long)(start_offset_in_file * sizeof(T)), SEEK_SET);
        std::fwrite(d_.data(), sizeof(T), size(), f);
        std::fclose(f);
    }

  private:
    size_t nr_ = 0, nc_ = 0;
    std::vector<T> d_;
};

/* BlockMemoryPool<double> (blockallocator.h:8-25): a device block pool shared by matrices */
class BlockMemoryPool {
  public:
    explicit BlockMemoryPool(size_t block_elems) { check(bsg_pool_create(default_ctx(), block_elems, &p_), "pool"); }
    ~BlockMemoryPool() { bsg_pool_release(p_); }
    BlockMemoryPool(const BlockMemoryPool &) = delete;
    BlockMemoryPool &operator=(const BlockMemoryPool &) = delete;
    bsg_pool handle() const { return p_; }

  private:
    bsg_pool p_ = nullptr;
};

template <typename Num>
class BlockSparseMatrix {
    static_assert(std::is_same<Num, double>::value, "the device library is double only");

  public:
    BlockSparseMatrix(size_t nr, size_t nc, size_t bsr, size_t bsc, double thresh,
                      const std::shared_ptr<BlockMemoryPool> &pool = nullptr) {
        check(bsg_bsm_create(default_ctx(), nr, nc, bsr, bsc, thresh, pool ? pool->handle() : nullptr, &h_),
              "BlockSparseMatrix");
    }
    BlockSparseMatrix(const Matrix<double> &m, size_t bsr, size_t bsc, double thresh,
                      const std::shared_ptr<BlockMemoryPool> &pool = nullptr)
        : BlockSparseMatrix(m.nrow(), m.ncol(), bsr, bsc, thresh, pool) {
        copy_from_input_matrix(m);
    }
    /* copies share the pool (occ_ri_k_step.cpp:96) */
    BlockSparseMatrix(const BlockSparseMatrix &o) {
        size_t dims[6];
        double thr;
        check(bsg_bsm_info(o.h_, dims, &thr), "bsg_bsm_info");
        bsg_pool p = nullptr;
        check(bsg_bsm_pool(o.h_, &p), "bsg_bsm_pool");
        check(bsg_bsm_create(default_ctx(), dims[0], dims[1], dims[2], dims[3], thr, p, &h_), "BlockSparseMatrix");
        check(bsg_bsm_assign(h_, o.h_), "operator=");
    }
    BlockSparseMatrix &operator=(const BlockSparseMatrix &o) {
        if (this != &o) check(bsg_bsm_assign(h_, o.h_), "operator=");
        return *this;
    }
    ~BlockSparseMatrix() {
        if (h_) bsg_bsm_destroy(h_);
    }
    bsg_bsm handle() const { return h_; }

    void copy_from_input_matrix(const Matrix<double> &m) {
        check(bsg_bsm_copy_from_dense(h_, m.data_ptr(), BSG_HOST), "copy_from_input_matrix");
    }
    void fill_with_values(double v) { check(bsg_bsm_fill(h_, v), "fill_with_values"); }
    void zero() { check(bsg_bsm_zero(h_), "zero"); }
    void scale(double s) { check(bsg_bsm_scale(h_, s), "scale"); }
    BlockSparseMatrix &operator*=(double s) {
        scale(s);
        return *this;
    }
    BlockSparseMatrix &operator+=(const BlockSparseMatrix &o) {
        check(bsg_bsm_add(h_, o.h_), "operator+=");
        return *this;
    }
    BlockSparseMatrix &operator-=(const BlockSparseMatrix &o) {
        check(bsg_bsm_sub(h_, o.h_), "operator-=");
        return *this;
    }
    void add_transpose(const BlockSparseMatrix &o) { check(bsg_bsm_add_transpose(h_, o.h_), "add_transpose"); }
    void calc_frobenius_norms() { check(bsg_bsm_calc_norms(h_), "calc_frobenius_norms"); }
    void recompress() { check(bsg_bsm_recompress(h_), "recompress"); }
    double frobenius_norm() const {
        double n = 0.0;
        check(bsg_bsm_frobenius_norm(h_, &n), "frobenius_norm");
        return n;
    }
    size_t no_of_alloc_blocks() const {
        size_t n = 0;
        check(bsg_bsm_no_of_alloc_blocks(h_, &n), "no_of_alloc_blocks");
        return n;
    }
    Matrix<double> to_matrix() const {
        size_t dims[6];
        double thr;
        check(bsg_bsm_info(h_, dims, &thr), "bsg_bsm_info");
        Matrix<double> m(dims[0], dims[1]);
        check(bsg_bsm_to_dense(h_, m.data_ptr(), BSG_HOST), "to_matrix");
        return m;
    }

  private:
    bsg_bsm h_ = nullptr;
};

/* the reference's global knob (main.cpp:9) */
inline size_t min_size_for_strassen = 1024;

template <typename Num>
void matmult(BlockSparseMatrix<Num> &C, const BlockSparseMatrix<Num> &A, bool transA, const BlockSparseMatrix<Num> &B,
             bool transB, Num thresh, Num alpha, Num beta) {
    check(bsg_matmult(C.handle(), A.handle(), transA, B.handle(), transB, thresh, alpha, beta, nullptr), "matmult");
}

template <typename Num>
void matmult_strassen_sparse(BlockSparseMatrix<Num> &C, const BlockSparseMatrix<Num> &A, bool transA,
                             const BlockSparseMatrix<Num> &B, bool transB, Num thresh, Num alpha, Num beta) {
    check(bsg_matmult_strassen_sparse(C.handle(), A.handle(), transA, B.handle(), transB, thresh, alpha, beta,
                                      min_size_for_strassen),
          "matmult_strassen_sparse");
}

}  // namespace bsgpu
