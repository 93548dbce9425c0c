// The reference's occ-RI-K driver (occ_ri_k_step.cpp) against libbsgpu: same
// arguments and data files, the block-sparse step on the GPU in the FP64
// form (bit-identical to the reference on the deterministic BLAS) and in the
// mixed form (bf16 digit products on the tensor cores).
#include <chrono>
#include <cstdio>
#include <string>

#include "bsgpu.hpp"

using bsgpu::Matrix;

static double run(const Matrix<double> &ints, const Matrix<size_t> &keys, const Matrix<double> &occ, size_t n_bf,
                  size_t n_aux, size_t n_occ, size_t n_vec2, size_t bs, double thresh, int form, int digits,
                  Matrix<double> &K) {
    bsg_rik_args a{};
    a.n_bf = n_bf;
    a.n_aux = n_aux;
    a.n_occ = n_occ;
    a.n_vec2 = n_vec2;
    a.ints = ints.data_ptr();
    a.keys = reinterpret_cast<const uint64_t *>(keys.data_ptr());
    a.c_occ = occ.data_ptr();
    a.where = BSG_HOST;
    a.bs = bs;
    a.thresh = thresh;
    a.n_part = 1;
    a.form = form;
    a.n_digits = digits;
    const auto t0 = std::chrono::steady_clock::now();
    bsgpu::check(bsg_rik_occ_step(bsgpu::default_ctx(), &a, K.data_ptr(), BSG_HOST, nullptr), "rik_occ_step");
    const auto t1 = std::chrono::steady_clock::now();
    return (double)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
}

int main(int argc, char **argv) {
    if (argc < 10) {
        puts("Usage: <program> <N_bf> <N_aux> <N_occ> <N_vec2> <3c filename> <MO filename> <v2m_key_filename> "
             "<blocksize> <threshold>");
        return 1;
    }
    const size_t N_bf = (size_t)std::stol(argv[1]);
    const size_t N_aux = (size_t)std::stol(argv[2]);
    const size_t N_occ = (size_t)std::stol(argv[3]);
    const size_t N_vec2 = (size_t)std::stol(argv[4]);
    const size_t bs = (size_t)std::stol(argv[8]);
    const double thresh_mult = std::stod(argv[9]);

    Matrix<double> ints(N_vec2, N_aux);
    ints.read_from_file(argv[5]);
    Matrix<double> occ(N_bf, N_occ);
    occ.read_from_file(argv[6]);
    Matrix<size_t> keys(N_vec2, 1);
    keys.read_from_file(argv[7]);
    const size_t total_flops = 2 * (N_bf * N_bf * N_occ * N_aux + 2 * N_bf * N_occ * N_occ * N_aux);

    Matrix<double> K(0.0, N_bf, N_occ);
    printf("--- sparse occ-RIK, GPU FP64 form ---\n");
    for (int i = 0; i < 3; ++i) {
        const double us = run(ints, keys, occ, N_bf, N_aux, N_occ, N_vec2, bs, thresh_mult, BSG_FORM_FP64, 0, K);
        printf("  [%d] %.4f s  (%.4f GFLOPs)\n", i + 1, 1e-6 * us, 2e-3 * (double)total_flops / us);
    }
    const double L2_norm_of_output = K.calc_frobenius_norm();
    printf("L2 norm of output = %e\n", L2_norm_of_output);

    Matrix<double> Km(0.0, N_bf, N_occ);
    printf("--- sparse occ-RIK, GPU mixed form (bf16 x 5 digits) ---\n");
    for (int i = 0; i < 3; ++i) {
        const double us = run(ints, keys, occ, N_bf, N_aux, N_occ, N_vec2, bs, thresh_mult, BSG_FORM_OZAKI, 5, Km);
        printf("  [%d] %.4f s  (%.4f GFLOPs)\n", i + 1, 1e-6 * us, 2e-3 * (double)total_flops / us);
        printf("relative RMSD = %e\n", (Km - K).calc_frobenius_norm() / L2_norm_of_output);
    }
    return 0;
}
