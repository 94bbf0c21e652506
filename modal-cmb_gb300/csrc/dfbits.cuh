// dfbits.cuh -- exact float/double conversions by integer arithmetic.
//
// GB300 issues one FP64 warp instruction per 16 cycles per SM, and the
// double -> float and double -> integer conversions share that rate.  Kernels
// that touch every element of a large matrix once -- the (head, tail) float
// copy of the trailing matrix in the tridiagonalisation, the 7-bit digit
// slicing of the FP64-accurate tensor-core products, the row maxima that set
// the slices' exponents -- were bound by those few instructions per element.
// The functions here produce the same bits with integer instructions, which
// issue at the full rate, and decline the rare inputs they do not cover
// (denormal or huge exponents); the caller then takes the FP64 route.
//
// The header compiles with nvcc (device and host) and with a plain C++
// compiler, so that the CPU tests check it bit for bit against IEEE rounding.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define DFB_HD __host__ __device__ __forceinline__
#else
#define DFB_HD static inline
#endif

namespace dfb {

DFB_HD uint64_t bits64(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

DFB_HD double from64(uint64_t u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

DFB_HD int clz64(uint64_t a)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)a);
#else
    return __builtin_clzll(a);
#endif
}

// Head and tail of x as floats: hi = RN(x), lo = RN(x - hi) (round to nearest
// even, the bits of __double2float_rn(x) and __double2float_rn(x - (double)hi)).
// Covers zero and |x| in [2^-74, 2^127) (both parts then normal floats);
// returns false otherwise.
DFB_HD bool split(double x, uint32_t *hi, uint32_t *lo)
{
    const uint64_t u = bits64(x);
    const uint32_t sg = (uint32_t)(u >> 63);
    if ((u << 1) == 0) {  // +-0: hi keeps the sign, x - hi = +0
        *hi = sg << 31;
        *lo = 0u;
        return true;
    }
    const int E = (int)((u >> 52) & 0x7ffu) - 1023;
    if (E < -74 || E > 126) return false;
    const uint64_t M = (u & 0xfffffffffffffull) | (1ull << 52);  // 53-bit significand
    uint64_t q = M >> 29;                                         // its top 24 bits
    const uint64_t r = M & ((1ull << 29) - 1);
    if (r > (1ull << 28) || (r == (1ull << 28) && (q & 1u))) q++;
    const int64_t d = (int64_t)M - (int64_t)(q << 29);  // x - hi in units of 2^(E-52), |d| <= 2^28
    int Eh = E;
    if (q == (1ull << 24)) {  // rounded up to the next power of two
        q >>= 1;
        Eh++;
    }
    *hi = (sg << 31) | ((uint32_t)(Eh + 127) << 23) | ((uint32_t)q & 0x7fffffu);
    if (d == 0) {
        *lo = 0u;
        return true;
    }
    const uint32_t sl = sg ^ (d < 0 ? 1u : 0u);
    const uint64_t a = (uint64_t)(d < 0 ? -d : d);
    const int p = 63 - clz64(a);  // leading bit, 0 .. 28
    int El = E - 52 + p;          // >= -126: normal
    uint64_t ql;
    if (p <= 23) {
        ql = a << (23 - p);
    } else {
        const int sh = p - 23;
        ql = a >> sh;
        const uint64_t rr = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rr > half || (rr == half && (ql & 1u))) ql++;
        if (ql == (1ull << 24)) {
            ql >>= 1;
            El++;
        }
    }
    *lo = (sl << 31) | ((uint32_t)(El + 127) << 23) | ((uint32_t)ql & 0x7fffffu);
    return true;
}

// x 2^sh rounded to the nearest integer, ties to even: the value of
// __double2ll_rn(ldexp(x, sh)).  Covers zero and normal x with |x 2^sh| < 2^62;
// returns false otherwise (denormal, infinite or NaN x, or too large).
DFB_HD bool scaled_rint(double x, int sh, long long *F)
{
    const uint64_t u = bits64(x);
    const uint64_t a = u & 0x7fffffffffffffffull;
    if (a == 0) {
        *F = 0;
        return true;
    }
    const int e11 = (int)(a >> 52);
    if (e11 == 0 || e11 == 2047) return false;
    const int E = e11 - 1023 + sh;  // x 2^sh = M 2^(E - 52), M the 53-bit significand
    if (E >= 62) return false;
    const uint64_t M = (a & 0xfffffffffffffull) | (1ull << 52);
    uint64_t q;
    if (E >= 52) {
        q = M << (E - 52);
    } else if (52 - E >= 64) {
        q = 0;  // below 2^-11
    } else {
        const int shift = 52 - E;
        q = M >> shift;
        const uint64_t rem = M & ((1ull << shift) - 1), half = 1ull << (shift - 1);
        if (rem > half || (rem == half && (q & 1u))) q++;
    }
    *F = (u >> 63) ? -(long long)q : (long long)q;
    return true;
}

// max(m, |x|) on the bit patterns (m the bits of a non-negative double): for
// non-negative doubles the unsigned integer order is the numeric order.  NaNs
// are skipped, as fmax skips them; infinities count.  Start from 0 (+0.0).
DFB_HD uint64_t absmax_bits(uint64_t m, double x)
{
    const uint64_t b = bits64(x) & 0x7fffffffffffffffull;
    return (b <= 0x7ff0000000000000ull && b > m) ? b : m;
}

}  // namespace dfb
