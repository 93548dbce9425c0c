// Fixed-point value of an FP64 number for the mixed form's digit split,
// computed from its bit pattern with integer operations only.  Host and
// device compile the same code (the host build checks it against exact
// rounding), so this header includes nothing from CUDA.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define BSG_HD __host__ __device__ __forceinline__
#else
#define BSG_HD inline
#endif

namespace bsg {

// N = round(v 2^(K - e)), ties to even, for the double with bit pattern
// `bits` (|N| <= 2^K when |v| < 2^e).  The value is M 2^(E' - 1075) with the
// 53-bit integer M (the implicit bit set for normal numbers, E' = max(E, 1)),
// so N = M 2^sh with sh = E' - 1075 + K - e.  For a right shift by s = -sh,
// with q = M >> s the rounded quotient is (M + 2^(s-1) - 1 + (q & 1)) >> s:
// one add chain, no compares or branches.  s is capped at 63 (any s >= 54
// rounds to 0 either way).  A word-wise form with the rounding decided by
// compares measured slower on the image kernels (its branches diverge).
BSG_HD long long oz_fixed_bits(unsigned long long bits, int e, int K) {
    const int E = (int)((bits >> 52) & 0x7FF);
    const unsigned long long M = (bits & 0xFFFFFFFFFFFFFull) | (E ? (1ull << 52) : 0ull);
    const int sh = (E ? E : 1) - 1075 + K - e;  // N = M * 2^sh
    unsigned long long N;
    if (sh >= 0) {
        N = M << sh;
    } else {
        const int s = -sh < 63 ? -sh : 63;
        N = (M + ((1ull << (s - 1)) - 1ull) + ((M >> s) & 1ull)) >> s;
    }
    return (bits >> 63) ? -(long long)N : (long long)N;
}

}  // namespace bsg
