// The reference's Strassen benchmark driver (main.cpp) against libbsgpu:
// screened block-sparse matmult and the hybrid Strassen-Winograd / sparse
// recursion of two N x N matrices read from files in the reference's binary
// format, compared with the unscreened product (threshold 0).
#include <chrono>
#include <cstdio>
#include <string>

#include "bsgpu.hpp"

using bsgpu::BlockSparseMatrix;
using bsgpu::Matrix;

int main(int argc, char **argv) {
    if (argc < 8) {
        puts("Usage: <program> <blocksize> <strassen_min> <thresh> <n_runs> <N> <matrix 1 file> <matrix 2 file>");
        return 1;
    }
    const size_t bs = (size_t)std::stoi(argv[1]);
    bsgpu::min_size_for_strassen = (size_t)std::stoi(argv[2]);
    const double thresh = std::stod(argv[3]);
    const int n_runs = std::stoi(argv[4]);
    const size_t N = (size_t)std::stol(argv[5]);

    Matrix<double> mat1(N, N), mat2(N, N);
    mat1.read_from_file(argv[6]);
    mat2.read_from_file(argv[7]);
    BlockSparseMatrix<double> bsmat1(mat1, bs, bs, 0.0);
    BlockSparseMatrix<double> bsmat2(mat2, bs, bs, 0.0);
    BlockSparseMatrix<double> bsmat3(Matrix<double>(N, N), bs, bs, 0.0);
    const double flops = 2.0 * (double)N * N * N;

    // unscreened product (every block pair): the reference's dense result
    bsmat3.fill_with_values(0.0);
    bsgpu::matmult(bsmat3, bsmat1, false, bsmat2, false, 0.0, 1.0, 0.0);
    const Matrix<double> mat3_dense = bsmat3.to_matrix();
    const double L2_norm_of_output = mat3_dense.calc_frobenius_norm();

    printf("--- BSM matmult on the GPU (thresh=%.2e) ---\n", thresh);
    for (int i = 0; i < n_runs; ++i) {
        bsmat3.fill_with_values(0.0);
        const auto t0 = std::chrono::steady_clock::now();
        bsgpu::matmult(bsmat3, bsmat1, false, bsmat2, false, thresh, 1.0, 0.0);
        const auto t1 = std::chrono::steady_clock::now();
        const double us = (double)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
        printf("  [%d] %.4f s  (%.4f GFLOPs)", i + 1, 1e-6 * us, 1e-3 * flops / us);
        printf("relative RMSD = %e\n", (bsmat3.to_matrix() - mat3_dense).calc_frobenius_norm() / L2_norm_of_output);
    }
    printf("\n--- Strassen-Sparse on the GPU (thresh=%.2e) ---\n", thresh);
    for (int i = 0; i < n_runs; ++i) {
        bsmat3.fill_with_values(0.0);
        const auto t0 = std::chrono::steady_clock::now();
        bsgpu::matmult_strassen_sparse(bsmat3, bsmat1, false, bsmat2, false, thresh, 1.0, 0.0);
        const auto t1 = std::chrono::steady_clock::now();
        const double us = (double)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
        printf("  [%d] %.4f s  (%.4f GFLOPs)", i + 1, 1e-6 * us, 1e-3 * flops / us);
        printf("relative RMSD = %e\n", (bsmat3.to_matrix() - mat3_dense).calc_frobenius_norm() / L2_norm_of_output);
    }
    return 0;
}
