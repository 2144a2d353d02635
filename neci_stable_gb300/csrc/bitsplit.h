// bitsplit.h -- threshold tests and the integer/fraction split of a walker
// sign done on the IEEE-754 bit pattern, for the per-determinant sweeps.
//
// GB300 runs FP64 instructions at about 1/128 of the FP32 rate, and the sweeps
// over CurrentDets test |C| against thresholds and split |C| into whole and
// fractional walkers for every determinant.  For finite doubles of equal
// sign the order of the values is the order of their bit patterns read as
// integers, and a double is mantissa x 2^exponent, so these steps are exact
// in integer arithmetic.  Every function here returns what the FP64
// expression it names returns, for every finite input (checked against that
// expression on the host by the tests).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define NECI_HD __host__ __device__ __forceinline__
#else
#define NECI_HD inline
#endif

namespace neci {

NECI_HD uint64_t dbl_bits(double x) {
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
}

// Bits of |x|: for finite x, y >= 0:  |x| > y  <=>  abs_bits(x) > dbl_bits(y).
NECI_HD uint64_t abs_bits(double x) { return dbl_bits(x) & 0x7FFFFFFFFFFFFFFFull; }

// x < 0 and x != 0 (a negative value, not -0.0).
NECI_HD bool is_negative(double x) { return (dbl_bits(x) >> 63) && abs_bits(x) != 0; }
// x > 0.
NECI_HD bool is_positive(double x) { return !(dbl_bits(x) >> 63) && abs_bits(x) != 0; }

// a * b < 0.0 for finite a, b: opposite signs, both non-zero, and a product
// that does not round to zero.  Exponents that keep |a b| >= 2^-1073 answer
// in integers; smaller products (not met by walker signs) take the FP64 form.
NECI_HD bool prod_negative(double a, double b) {
    const uint64_t x = dbl_bits(a), y = dbl_bits(b);
    const uint64_t ax = x & 0x7FFFFFFFFFFFFFFFull, ay = y & 0x7FFFFFFFFFFFFFFFull;
    if (!((x ^ y) >> 63) || ax == 0 || ay == 0) return false;
    const int ea = (int)(ax >> 52), eb = (int)(ay >> 52);
    if (ea >= 1 && eb >= 1 && ea + eb - 2046 >= -1073) return true;
    return a * b < 0.0;
}

// The split of decide_num_to_spawn (fcimc_helper.F90:2160-2174) with
// AvMCExcits = 1, for |c| < 2^31:
//   whole  = abs(int(c))
//   extra  = (|c| - whole > 1e-12)                 (an extra attempt is drawn)
//   thresh = prob_thresh(|c| - whole) = floor((|c| - whole) * 2^64)
// Returns false (and leaves the outputs alone) for |c| >= 2^31, where the
// caller takes the FP64 form.
NECI_HD bool split_count(double c, uint32_t &whole, bool &extra, uint64_t &thresh) {
    const uint64_t a = abs_bits(c);
    const int E = (int)(a >> 52);
    const uint64_t m = (a & 0xFFFFFFFFFFFFFull) | (E ? (1ull << 52) : 0ull);
    if (E >= 1023 + 31) return false;
    if (E >= 1023) {
        // |c| = m 2^(E-1075), 1 <= |c| < 2^31: the fraction has sh = 1075 - E bits
        const int sh = 1075 - E;  // 22 .. 52
        whole = (uint32_t)(m >> sh);
        const uint64_t F = (m & ((1ull << sh) - 1)) << (64 - sh);  // fraction * 2^64, exact
        // F is an integer and 1e-12 * 2^64 = 18446744.07..., so F > it <=> F >= 18446745
        extra = F >= 18446745ull;
        thresh = F;
        return true;
    }
    whole = 0;
    extra = a > dbl_bits(1e-12);
    // floor(|c| 2^64) = floor(m 2^(E-1011)), E <= 1022
    const int s = E - 1011;
    thresh = s >= 0 ? (m << s) : (s > -64 ? (m >> -s) : 0ull);
    return true;
}

// The spawn amplitude's fixed point: q = llrint(x * 2^32) (round half to
// even) with the overflow rule !(|x * 2^32| < 9.2e18) -> false.  The product
// by 2^32 is exact for normal x, so q follows from the bits of x alone: with
// x = m 2^(E-1075), x 2^32 = m 2^(E-1043), shifted with round-half-even.
// Subnormal x give 0 (|x 2^32| < 2^-990).  NaN and infinities overflow.
NECI_HD bool fixed32_from_double(double x, int64_t &q) {
    const uint64_t b = dbl_bits(x);
    const uint64_t a = b & 0x7FFFFFFFFFFFFFFFull;
    // 9.2e18 * 2^-32 is exact, so |x| 2^32 < 9.2e18 <=> |x| < 9.2e18 * 2^-32
    if (!(a < dbl_bits(9.2e18 * 2.3283064365386962890625e-10))) return false;
    const int E = (int)(a >> 52);
    if (E == 0) {
        q = 0;
        return true;
    }
    const uint64_t m = (a & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = E - 1043;
    uint64_t v;
    if (sh >= 0) {
        v = m << sh;  // |x 2^32| < 2^63 bounds sh by 10
    } else if (sh <= -54) {
        v = 0;  // below 1/2
    } else {
        const int k = -sh;
        const uint64_t ip = m >> k, rem = m & ((1ull << k) - 1), half = 1ull << (k - 1);
        v = ip + ((rem > half || (rem == half && (ip & 1ull))) ? 1ull : 0ull);
    }
    q = (b >> 63) ? -(int64_t)v : (int64_t)v;
    return true;
}

// prob_thresh(p) = floor(p 2^64) as a 64-bit threshold (0 for p <= 0 or
// NaN, all ones for p >= 1), from the bits of p: the product by 2^64 is
// exact, so for p = m 2^(E-1075) in (0, 1) it is m shifted by E - 1011
// (at most 11 places left) and truncated.  Subnormal p give 0.
NECI_HD uint64_t prob_thresh_bits(double p) {
    const uint64_t b = dbl_bits(p);
    if ((b >> 63) || b == 0) return 0ull;
    if (b >= 0x3FF0000000000000ull) return b > 0x7FF0000000000000ull ? 0ull : ~0ull;
    const int E = (int)(b >> 52);
    if (E == 0) return 0ull;
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = E - 1011;
    return sh >= 0 ? m << sh : (sh > -64 ? m >> -sh : 0ull);
}

// a <= b for finite a and b >= 0 (b not -0.0 unless a is negative or zero):
// a negative or -0.0 is below any b >= 0; non-negative doubles order like
// their bit patterns.
NECI_HD bool le_nonneg(double a, double b) {
    const uint64_t x = dbl_bits(a);
    return (x >> 63) || x <= dbl_bits(b);
}

// a > b for b > 0 finite: a positive and above b in bit order (NaN with the
// sign bit clear counts as above).
NECI_HD bool gt_pos(double a, double b) {
    const uint64_t x = dbl_bits(a);
    return !(x >> 63) && x > dbl_bits(b);
}

}  // namespace neci
