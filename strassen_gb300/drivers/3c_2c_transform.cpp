// The reference's 3c->2c driver (3c_2c_transform.cpp) against libbsgpu: same
// arguments and data files; the screened product on the GPU in the FP64 form
// and in the mixed form, compared with each other.
#include <chrono>
#include <cstdio>
#include <string>

#include "bsgpu.hpp"

using bsgpu::Matrix;

int main(int argc, char **argv) {
    if (argc < 8) {
        puts("Usage: <program> <N_bf> <N_aux> <N_vec2> <3c filename> <2c filename> <blocksize> <threshold>");
        return 1;
    }
    const size_t N_aux = (size_t)std::stol(argv[2]);
    const size_t N_vec2 = (size_t)std::stol(argv[3]);
    const size_t bs = (size_t)std::stol(argv[6]);
    const double thresh_mult = std::stod(argv[7]);

    Matrix<double> ints_3c(N_vec2, N_aux);
    ints_3c.read_from_file(argv[4]);
    Matrix<double> ints_2c(N_aux, N_aux);
    ints_2c.read_from_file(argv[5]);
    const double flops = 2.0 * (double)N_vec2 * N_aux * N_aux;

    Matrix<double> out64(N_vec2, N_aux), outmx(N_vec2, N_aux);
    const int forms[2] = {BSG_FORM_FP64, BSG_FORM_OZAKI};
    Matrix<double> *outs[2] = {&out64, &outmx};
    const char *names[2] = {"FP64 form", "mixed form (bf16 x 6 digits)"};
    double L2 = 0.0;
    for (int f = 0; f < 2; ++f) {
        printf("--- BSM matmult on the GPU, %s (thresh=%.2e) ---\n", names[f], thresh_mult);
        const auto t0 = std::chrono::steady_clock::now();
        bsgpu::check(bsg_3c2c_transform(bsgpu::default_ctx(), N_vec2, N_aux, ints_3c.data_ptr(), ints_2c.data_ptr(),
                                        BSG_HOST, bs, thresh_mult, forms[f], f ? 6 : 0, outs[f]->data_ptr(), BSG_HOST),
                     "3c2c_transform");
        const auto t1 = std::chrono::steady_clock::now();
        const double us = (double)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
        printf("  [1] %.4f s  (%.4f GFLOPs)\n", 1e-6 * us, 1e-3 * flops / us);
        if (f == 0) {
            L2 = out64.calc_frobenius_norm();
            printf("L2 norm of output = %e\n", L2);
        } else {
            printf("relative RMSD = %e\n", (outmx - out64).calc_frobenius_norm() / L2);
        }
    }
    return 0;
}
