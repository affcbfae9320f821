// Block-floating fixed-point arithmetic for FP64 amplitudes on the integer pipes.
//
// GB300 issues about 2 FP64 FMAs per clock per SM, so a general complex 2x2 gate on
// an FP64 statevector (16 real products per amplitude pair) is bound by the FP64 pipe
// at roughly a third of HBM bandwidth.  The integer multiply-add pipe is many times
// wider.  This header applies a real 4x4 operator (the real form of a complex 2x2
// matrix) to the four doubles of an amplitude pair in 64-bit fixed point:
//
//  * the pair shares one scale: e = the largest biased exponent among its four doubles;
//    each value becomes x = v * 2^(1082 - e), |x| < 2^60 (denormals are exact: they
//    enter with exponent 1 and no implicit bit);
//  * the operator's coefficients share one scale E (|c| < 2^E): m = c * 2^(60 - E);
//  * x and m split into balanced 32-bit limbs, x = xh*2^32 + xl with xl in
//    [-2^31, 2^31); each output is R = sum(xh*mh) + (sum(xh*ml + xl*mh) >> 32), the
//    top 64 bits of the exact 128-bit sum of products minus the dropped xl*ml terms;
//  * R converts back to a double rounded to nearest (ties away): value = R * 2^(e+E-1078).
//
// Error per output: at most 2 units of R plus the input truncation, i.e. below
// 2^-54 of (largest |v| in the pair) * (largest |c|).  IEEE FP64 evaluation of the same
// 4-term sums has a bound of the same order.  A pair holding Inf or NaN, or whose result
// would leave the normal double range, returns false and the caller uses FP64.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define QG_HD __host__ __device__ __forceinline__
#else
#define QG_HD inline
#endif

namespace qgfx {

// one real operator coefficient row-set: out[r] = sum_j C[r][j] * in[j], in the limb form
struct Op4 {
    int32_t h[4][4];    // high limbs, |h| <= 2^28 + 1
    int32_t l[4][4];    // low limbs in [-2^31, 2^31)
    int32_t expo;       // E: every |C[r][j]| < 2^E
    int32_t pad;
};

QG_HD uint64_t f64_bits(double v) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t u;
    __builtin_memcpy(&u, &v, 8);
    return u;
#endif
}

QG_HD double bits_f64(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double v;
    __builtin_memcpy(&v, &u, 8);
    return v;
#endif
}

QG_HD int clz64(uint64_t a) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)a);
#else
    return a ? __builtin_clzll(a) : 64;
#endif
}

// biased exponent with denormals (and zero) counted as exponent 1
QG_HD int eff_exponent(uint64_t u) {
    int ei = (int)((u >> 52) & 0x7FF);
    return ei + (ei == 0);
}

// v (bits u) at the pair scale e: x = v * 2^(1082 - e), split into balanced limbs
QG_HD void to_limbs(uint64_t u, int e, int32_t& xh, int32_t& xl) {
    const int ei = (int)((u >> 52) & 0x7FF);
    const uint64_t mant = (u & 0xFFFFFFFFFFFFFull) | (ei ? (1ull << 52) : 0ull);
    const int d = e - (ei + (ei == 0));
    const uint64_t x = d < 64 ? (mant << 7) >> d : 0ull;
    const int64_t sx = (u >> 63) ? -(int64_t)x : (int64_t)x;
    const uint32_t lo = (uint32_t)sx;
    xl = (int32_t)lo;
    xh = (int32_t)(uint32_t)((uint64_t)sx >> 32) + (int32_t)(lo >> 31);
}

// R * 2^(ebase - 1086) as a double (ebase = e + E + 8); ok = false when the result
// is not a normal double (the caller then recomputes in FP64)
QG_HD double from_fixed(int64_t R, int ebase, bool& ok) {
    if (R == 0) return 0.0;
    const uint64_t sgn = (uint64_t)R >> 63;
    const uint64_t a = sgn ? (uint64_t)(-R) : (uint64_t)R;
    const int lz = clz64(a);
    const uint64_t nrm = a << lz;                         // bit 63 set
    uint64_t q = (nrm >> 11) + ((nrm >> 10) & 1ull);      // 53 significant bits, rounded
    int be = ebase - lz;
    if (q >> 53) { q >>= 1; be += 1; }
    ok = ok && be >= 1 && be <= 2046;
    return bits_f64((sgn << 63) | ((uint64_t)(uint32_t)be << 52) | (q & 0xFFFFFFFFFFFFFull));
}

// out[r] = sum_j C[r][j] * in[j]; false (outputs undefined) if FP64 must be used
QG_HD bool apply_op4(const Op4& C, const double in[4], double out[4]) {
    uint64_t u[4];
    int e = 1;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        u[j] = f64_bits(in[j]);
        const int ej = eff_exponent(u[j]);
        e = ej > e ? ej : e;
    }
    if (e == 2047) return false;          // Inf or NaN in the pair
    int32_t xh[4], xl[4];
#pragma unroll
    for (int j = 0; j < 4; j++) to_limbs(u[j], e, xh[j], xl[j]);
    bool ok = true;
    const int ebase = e + C.expo + 8;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int64_t hh = 0, mid = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            hh += (int64_t)xh[j] * C.h[r][j];
            mid += (int64_t)xh[j] * C.l[r][j];
            mid += (int64_t)xl[j] * C.h[r][j];
        }
        out[r] = from_fixed(hh + (mid >> 32), ebase, ok);
    }
    return ok;
}

}  // namespace qgfx
