// Block-floating fixed-point arithmetic for FP64 amplitudes on the integer pipes.
//
// GB300 issues about 2 FP64 FMAs per clock per SM, so a general complex 2x2 gate on
// an FP64 statevector (16 real products per amplitude pair) is bound by the FP64 pipe
// at roughly a third of HBM bandwidth.  The integer multiply-add pipe is many times
// wider.  This header applies a real N x N operator (N = 4: the real form of a complex
// 2x2 matrix on an amplitude pair; N = 2: a complex scalar on one amplitude) to N
// doubles in 64-bit fixed point:
//
//  * the input shares one scale: e = the largest biased exponent among its N doubles;
//    each value becomes x = v * 2^(S + 1075 - e), |x| < 2^(53+S) with S from 7 (N <= 4)
//    down to 4 (N = 32) (denormals are exact: they enter with exponent 1 and no implicit bit);
//  * the operator's coefficients share one scale E (|c| < 2^E): m = c * 2^(Q - E);
//  * x and m split into balanced 32-bit limbs, x = xh*2^32 + xl with xl in
//    [-2^31, 2^31); each output is R = sum(xh*mh) + (sum(xh*ml + xl*mh) >> 32), the
//    top 64 bits of the exact 128-bit sum of products minus the dropped xl*ml terms;
//  * R converts back to a double rounded to nearest: value = R * 2^(e+E-S-Q-1011).
//    apply_op does that with integer instructions only (ties away from zero);
//    apply_op_cvt, which the GPU kernels use, lets the hardware int64 -> double
//    conversion round (ties to even) and adds the scale to the exponent field.
//
// Error per output, relative to (largest |v| in the input) x (largest |c|): N input
// truncations of 2^-(52+S), N coefficient roundings of 2^-Q, and N/4 + 1 units of R
// (2^(13-S-Q) each) for the dropped low x low products; plus half an ulp of the result.
// That is below 2^-54 for N = 4 and 2^-48.8 for N = 32, the order of IEEE FP64's own
// bound for the same N-term sums (tests/fx_check.cpp checks it on random operators).  An input holding Inf or NaN, or whose
// result could leave the normal double range, returns false and the caller uses FP64.
#pragma once
#include <stdint.h>
#include <cmath>

#if defined(__CUDACC__)
#define QG_HD __host__ __device__ __forceinline__
#else
#define QG_HD inline
#endif

namespace qgfx {

// a real N x N operator, out[r] = sum_j C[r][j] * in[j], in the limb form (N = 2: a
// complex scalar acting on one amplitude; N = 4: a complex 2x2 acting on a pair)
template <int N>
struct OpN {
    int32_t h[N][N];    // high limbs, |h| <= 2^28 + 1
    int32_t l[N][N];    // low limbs in [-2^31, 2^31)
    int32_t expo;       // E: every |C[r][j]| < 2^E
    int32_t pad;
};
typedef OpN<4> Op4;
typedef OpN<2> Op2;

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

// Scales that leave headroom for the 2N middle products of one output: inputs
// |x| < 2^(53+S), coefficients |m| <= 2^Q, so |xh*ml| <= 2^(S+52) and
// |xl*mh| <= 2^(Q-1) (+2^31) and N of each stay below 2^63:
//   N <= 4: S = 7, Q = 60;  N = 8: S = 6, Q = 60;  N = 16: S = 5, Q = 59;  N = 32: S = 4, Q = 58.
// |R| <= N * 2^(S+Q-11) = 2^RL, and value = R * 2^(e + E - S - Q - 1011).
template <int N>
struct FxShift {
    static_assert(N >= 1 && N <= 32, "operator size");
    static constexpr int S = (N <= 4) ? 7 : (N <= 8) ? 6 : (N <= 16) ? 5 : 4;
    static constexpr int Q = (N <= 8) ? 60 : (N <= 16) ? 59 : 58;
    static constexpr int RL = (N <= 2 ? 1 : N <= 4 ? 2 : N <= 8 ? 3 : N <= 16 ? 4 : 5) + S + Q - 11;
    static constexpr int TOFF = S + Q + 1011;     // value = R * 2^(e + E - TOFF)
};

// v (bits u) at the pair scale e: x = v * 2^(S + 1075 - e), split into balanced limbs
QG_HD void to_limbs(uint64_t u, int e, int32_t& xh, int32_t& xl, int S = 7) {
    const int ei = (int)((u >> 52) & 0x7FF);
    const uint64_t mant = (u & 0xFFFFFFFFFFFFFull) | (ei ? (1ull << 52) : 0ull);
    const int d = e - (ei + (ei == 0));
    const uint64_t x = d < 64 ? (mant << S) >> d : 0ull;
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

// out[r] = sum_j C[r][j] * in[j]; false (outputs undefined) if FP64 must be used.
// Bounds: |x| < 2^60 and |m| <= 2^60 give |xh*ml|, |xl*mh| < 2^59 + 2^31, so the
// 2N middle terms sum below 2^63 for N <= 4.
template <int N>
QG_HD bool apply_op(const OpN<N>& C, const double in[N], double out[N]) {
    constexpr int S = FxShift<N>::S;
    uint64_t u[N];
    int e = 1;
#pragma unroll
    for (int j = 0; j < N; j++) {
        u[j] = f64_bits(in[j]);
        const int ej = eff_exponent(u[j]);
        e = ej > e ? ej : e;
    }
    if (e == 2047) return false;          // Inf or NaN in the input
    int32_t xh[N], xl[N];
#pragma unroll
    for (int j = 0; j < N; j++) to_limbs(u[j], e, xh[j], xl[j], S);
    bool ok = true;
    const int ebase = e + C.expo + 1086 - FxShift<N>::TOFF;
#pragma unroll
    for (int r = 0; r < N; r++) {
        int64_t hh = 0, mid = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            hh += (int64_t)xh[j] * C.h[r][j];
            mid += (int64_t)xh[j] * C.l[r][j];
            mid += (int64_t)xl[j] * C.h[r][j];
        }
        out[r] = from_fixed(hh + (mid >> 32), ebase, ok);
    }
    return ok;
}

QG_HD bool apply_op4(const Op4& C, const double in[4], double out[4]) { return apply_op<4>(C, in, out); }

// The same arithmetic with the output step done by the hardware int64 -> double
// conversion (round to nearest) and the scale applied by an integer add to the
// exponent field: out_r = double(R) * 2^t, t = e + E - S - Q - 1011.  On GB300 that conversion
// runs on the FP64 unit, which the integer arithmetic leaves idle, and replaces
// about 30 integer ALU instructions per output.  Falls back (returns false) for
// Inf/NaN and when some output could leave the normal range (scale checked once
// per input: double(R) lies in [1, 2^58] or is 0).
QG_HD double i64_to_double(int64_t v) {
#if defined(__CUDA_ARCH__)
    return __ll2double_rn((long long)v);
#else
    return (double)v;
#endif
}

template <int N>
QG_HD bool apply_op_cvt(const OpN<N>& C, const double in[N], double out[N]) {
    constexpr int S = FxShift<N>::S;
    uint64_t u[N];
    int e = 1;
#pragma unroll
    for (int j = 0; j < N; j++) {
        u[j] = f64_bits(in[j]);
        const int ej = eff_exponent(u[j]);
        e = ej > e ? ej : e;
    }
    const int t = e + C.expo - FxShift<N>::TOFF;
    if (1023 + t < 1 || 1023 + FxShift<N>::RL + t > 2046 || e == 2047) {
        uint64_t any = 0;
#pragma unroll
        for (int j = 0; j < N; j++) any |= u[j] << 1;     // ignores the signs of zeros
        if (any) return false;
#pragma unroll
        for (int r = 0; r < N; r++) out[r] = 0.0;       // all zero: the common case in sparse states
        return true;
    }
    int32_t xh[N], xl[N];
#pragma unroll
    for (int j = 0; j < N; j++) to_limbs(u[j], e, xh[j], xl[j], S);
    const uint32_t down = (uint32_t)t << 20;           // adds t to the exponent field
#pragma unroll
    for (int r = 0; r < N; r++) {
        int64_t hh = 0, mid = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            hh += (int64_t)xh[j] * C.h[r][j];
            mid += (int64_t)xh[j] * C.l[r][j];
            mid += (int64_t)xl[j] * C.h[r][j];
        }
        const uint64_t d = f64_bits(i64_to_double(hh + (mid >> 32)));
        const uint32_t dh = (uint32_t)(d >> 32);
        out[r] = bits_f64(dh ? ((uint64_t)(dh + down) << 32 | (uint32_t)d) : 0ull);
    }
    return true;
}

// x = v * 2^(S + 1075 - e) for a normal v whose exponent is within 31 of e (d = e - e_v),
// from its two 32-bit words with 32-bit funnel shifts, split into balanced limbs
template <int S>
QG_HD void to_limbs_near(uint32_t hi, uint32_t lo, int d, int32_t& xh, int32_t& xl) {
    const uint32_t mh = (hi & 0xFFFFFu) | 0x100000u;            // 21 high mantissa bits with the implicit 1
#if defined(__CUDA_ARCH__)
    const uint32_t ah = __funnelshift_l(lo, mh, S);              // (mantissa << S): 53 + S bits
    const uint32_t al = lo << S;
    const uint32_t yl = __funnelshift_r(al, ah, d);              // >> d, d in [0, 31]
#else
    const uint32_t ah = (mh << S) | (lo >> (32 - S));
    const uint32_t al = lo << S;
    const uint32_t yl = d ? (al >> d) | (ah << (32 - d)) : al;
#endif
    const uint32_t yh = ah >> d;
    const uint32_t s = (uint32_t)((int32_t)hi >> 31);            // 0 or all ones
    const uint64_t y = ((uint64_t)(yh ^ s) << 32 | (yl ^ s)) - (uint64_t)(int64_t)(int32_t)s;   // +-y
    const uint32_t x0 = (uint32_t)y;
    xl = (int32_t)x0;
    xh = (int32_t)(uint32_t)(y >> 32) + (int32_t)(x0 >> 31);
}

// apply_op_cvt for the usual input: every value normal and within 2^31 of the largest
// (no zeros, denormals, Inf/NaN or wide spreads), output scale in range.  Returns false
// (outputs untouched) otherwise; the caller then uses apply_op_cvt.
template <int N>
QG_HD bool apply_op_near(const OpN<N>& C, const double in[N], double out[N]) {
    uint32_t hi[N], lo[N];
    int ex[N];
    int e = 0, emin = 4096;
#pragma unroll
    for (int j = 0; j < N; j++) {
        const uint64_t u = f64_bits(in[j]);
        hi[j] = (uint32_t)(u >> 32);
        lo[j] = (uint32_t)u;
        ex[j] = (int)((hi[j] >> 20) & 0x7FFu);
        e = ex[j] > e ? ex[j] : e;
        emin = ex[j] < emin ? ex[j] : emin;
    }
    constexpr int S = FxShift<N>::S;
    const int t = e + C.expo - FxShift<N>::TOFF;
    if (emin < 1 || e > 2046 || e - emin > 31 || 1023 + t < 1 || 1023 + FxShift<N>::RL + t > 2046) return false;
    int32_t xh[N], xl[N];
#pragma unroll
    for (int j = 0; j < N; j++) to_limbs_near<S>(hi[j], lo[j], e - ex[j], xh[j], xl[j]);
    const uint32_t down = (uint32_t)t << 20;
#pragma unroll
    for (int r = 0; r < N; r++) {
        int64_t hh = 0, mid = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            hh += (int64_t)xh[j] * C.h[r][j];
            mid += (int64_t)xh[j] * C.l[r][j];
            mid += (int64_t)xl[j] * C.h[r][j];
        }
        const uint64_t d = f64_bits(i64_to_double(hh + (mid >> 32)));
        const uint32_t dh = (uint32_t)(d >> 32);
        out[r] = bits_f64(dh ? ((uint64_t)(dh + down) << 32 | (uint32_t)d) : 0ull);
    }
    return true;
}

// The same arithmetic split in two, for callers that store each output as it is
// formed (wide operators, whose N outputs would not fit in registers at once):
// fx_prepare puts the N inputs at their common scale as limbs (false: use FP64);
// fx_row then forms output r.  The results equal apply_op_best's bit for bit.
template <int N>
QG_HD bool fx_prepare_e(int expo, const double in[N], int32_t xh[N], int32_t xl[N], uint32_t& down, bool& zero) {
    constexpr int S = FxShift<N>::S;
    // two passes over the inputs (scale, then limbs) so that no per-input state beyond
    // the inputs themselves stays live: at N = 32 registers are the limit
    int e = 0, emin = 4096, eg = 1;
    uint64_t any = 0;
#pragma unroll
    for (int j = 0; j < N; j++) {
        const uint64_t u = f64_bits(in[j]);
        any |= u << 1;
        const int ej = (int)((u >> 52) & 0x7FF);
        e = ej > e ? ej : e;
        emin = ej < emin ? ej : emin;
        const int ejg = ej + (ej == 0);
        eg = ejg > eg ? ejg : eg;
    }
    zero = false;
    const int t = e + expo - FxShift<N>::TOFF;
    if (emin >= 1 && e <= 2046 && e - emin <= 31 && 1023 + t >= 1 && 1023 + FxShift<N>::RL + t <= 2046) {
#pragma unroll
        for (int j = 0; j < N; j++) {
            const uint64_t u = f64_bits(in[j]);
            const uint32_t hi = (uint32_t)(u >> 32);
            to_limbs_near<S>(hi, (uint32_t)u, e - (int)((hi >> 20) & 0x7FFu), xh[j], xl[j]);
        }
        down = (uint32_t)t << 20;
        return true;
    }
    // the general form: exponents counted with denormals as 1
    const int tg = eg + expo - FxShift<N>::TOFF;
    if (1023 + tg < 1 || 1023 + FxShift<N>::RL + tg > 2046 || eg == 2047) {
        if (any) return false;
        zero = true;                      // all zero: every output is zero
        return true;
    }
#pragma unroll
    for (int j = 0; j < N; j++) to_limbs(f64_bits(in[j]), eg, xh[j], xl[j], S);
    down = (uint32_t)tg << 20;
    return true;
}

template <int N>
QG_HD bool fx_prepare(const OpN<N>& C, const double in[N], int32_t xh[N], int32_t xl[N], uint32_t& down, bool& zero) {
    return fx_prepare_e<N>(C.expo, in, xh, xl, down, zero);
}

template <int N>
QG_HD double fx_row(const OpN<N>& C, int r, const int32_t xh[N], const int32_t xl[N], uint32_t down, bool zero) {
    if (zero) return 0.0;
    int64_t hh = 0, mid = 0;
#pragma unroll
    for (int j = 0; j < N; j++) {
        hh += (int64_t)xh[j] * C.h[r][j];
        mid += (int64_t)xh[j] * C.l[r][j];
        mid += (int64_t)xl[j] * C.h[r][j];
    }
    const uint64_t d = f64_bits(i64_to_double(hh + (mid >> 32)));
    const uint32_t dh = (uint32_t)(d >> 32);
    return bits_f64(dh ? ((uint64_t)(dh + down) << 32 | (uint32_t)d) : 0ull);
}

// ---------------------------------------------------------------- complex operators, 3 products
// A complex D x D matrix U = A + iB on D complex inputs X = x + iy, with Gauss's
// three-product form per term: A(x+y), (A+B)y and (B-A)x give
//   Re Y = sum A(x+y) - sum (A+B)y,   Im Y = sum A(x+y) + sum (B-A)x,
// and the first sum is shared by both parts: 3D products per complex output instead
// of the 4D of the real 2D x 2D form.  The scales are those of OpN<2D>: (x+y) and
// (A+B), (B-A) carry one more bit, and each sum has D terms instead of 2D, so the
// middle sums stay below 2^63.
template <int D>
struct CopN {
    int32_t ah[D][D], al[D][D];   // A
    int32_t ph[D][D], pl[D][D];   // A + B
    int32_t qh[D][D], ql[D][D];   // B - A
    int32_t expo;                 // E: |A|, |B| < 2^E  (so |A+B|, |B-A| < 2^(E+1))
    int32_t pad;
};

// Host: the limb form of a complex D x D matrix (row-major, interleaved re/im)
template <int D>
inline bool make_cop(const double* u, CopN<D>& op) {
    constexpr int Q = FxShift<2 * D>::Q;
    int E = -100000;
    for (int i = 0; i < 2 * D * D; i++) {
        if (!(u[i] - u[i] == 0.0)) return false;
        if (u[i] != 0.0) {
            int ex;
            std::frexp(u[i], &ex);
            E = ex > E ? ex : E;
        }
    }
    if (E == -100000) E = 0;
    op.expo = E;
    op.pad = 0;
    auto limbs = [](int64_t m, int32_t& h, int32_t& l) {
        const uint32_t lo = (uint32_t)m;
        l = (int32_t)lo;
        h = (int32_t)((m - (int64_t)(int32_t)lo) >> 32);
    };
    for (int r = 0; r < D; r++)
        for (int j = 0; j < D; j++) {
            // A and B rounded once to the fixed-point quantum; A + B and B - A formed
            // exactly from those integers (a sum in double would round at 2^-53)
            const int64_t a = (int64_t)std::llround(std::ldexp(u[2 * (D * r + j)], Q - E));
            const int64_t b = (int64_t)std::llround(std::ldexp(u[2 * (D * r + j) + 1], Q - E));
            limbs(a, op.ah[r][j], op.al[r][j]);
            limbs(a + b, op.ph[r][j], op.pl[r][j]);
            limbs(b - a, op.qh[r][j], op.ql[r][j]);
        }
    return true;
}

QG_HD void split_limbs(int64_t v, int32_t& h, int32_t& l) {
    const uint32_t lo = (uint32_t)v;
    l = (int32_t)lo;
    h = (int32_t)(uint32_t)((uint64_t)v >> 32) + (int32_t)(lo >> 31);
}

// The D complex inputs (2D doubles) at their common scale as limbs of x, y and x + y;
// false: use FP64.  Same scale rules as fx_prepare<2D>.
template <int D>
QG_HD bool cfx_prepare(const CopN<D>& C, const double in[2 * D], int32_t xh[D], int32_t xl[D], int32_t yh[D],
                       int32_t yl[D], int32_t sh[D], int32_t sl[D], uint32_t& down, bool& zero) {
    constexpr int N = 2 * D;
    int32_t h[N], l[N];
    if (!fx_prepare_e<N>(C.expo, in, h, l, down, zero)) return false;
#pragma unroll
    for (int j = 0; j < D; j++) {
        const int64_t x = ((int64_t)h[2 * j] << 32) + (int64_t)l[2 * j];
        const int64_t y = ((int64_t)h[2 * j + 1] << 32) + (int64_t)l[2 * j + 1];
        xh[j] = h[2 * j]; xl[j] = l[2 * j];
        yh[j] = h[2 * j + 1]; yl[j] = l[2 * j + 1];
        split_limbs(x + y, sh[j], sl[j]);
    }
    return true;
}

// top 64 bits of sum_j (mh*2^32 + ml) * (vh*2^32 + vl) without the low x low terms
template <int D>
QG_HD int64_t limb_dot(const int32_t (&mh)[D][D], const int32_t (&ml)[D][D], int r, const int32_t* vh, const int32_t* vl) {
    int64_t hh = 0, mid = 0;
#pragma unroll
    for (int j = 0; j < D; j++) {
        hh += (int64_t)vh[j] * mh[r][j];
        mid += (int64_t)vh[j] * ml[r][j];
        mid += (int64_t)vl[j] * mh[r][j];
    }
    return hh + (mid >> 32);
}

QG_HD double fx_to_double(int64_t R, uint32_t down) {
    const uint64_t d = f64_bits(i64_to_double(R));
    const uint32_t dh = (uint32_t)(d >> 32);
    return bits_f64(dh ? ((uint64_t)(dh + down) << 32 | (uint32_t)d) : 0ull);
}

// complex output r: (re, im)
template <int D>
QG_HD void cfx_row(const CopN<D>& C, int r, const int32_t* xh, const int32_t* xl, const int32_t* yh, const int32_t* yl,
                   const int32_t* sh, const int32_t* sl, uint32_t down, bool zero, double& re, double& im) {
    if (zero) { re = 0.0; im = 0.0; return; }
    const int64_t t1 = limb_dot<D>(C.ah, C.al, r, sh, sl);
    const int64_t t2 = limb_dot<D>(C.ph, C.pl, r, yh, yl);
    const int64_t t3 = limb_dot<D>(C.qh, C.ql, r, xh, xl);
    re = fx_to_double(t1 - t2, down);
    im = fx_to_double(t1 + t3, down);
}

// the fast form when it applies, else the general one; false: use FP64
template <int N>
QG_HD bool apply_op_best(const OpN<N>& C, const double in[N], double out[N]) {
    return apply_op_near<N>(C, in, out) || apply_op_cvt<N>(C, in, out);
}

// Host: the limb form of a real N x N operator C (row-major).  Returns false when a
// coefficient is not finite (the caller then keeps FP64).
template <int N>
inline bool make_op(const double* C, OpN<N>& op) {
    int E = -100000;
    for (int i = 0; i < N * N; i++) {
        if (!(C[i] - C[i] == 0.0)) return false;   // Inf or NaN
        if (C[i] != 0.0) {
            int ex;
            std::frexp(C[i], &ex);                   // |C| < 2^ex
            E = ex > E ? ex : E;
        }
    }
    if (E == -100000) E = 0;                         // the zero operator
    op.expo = E;
    op.pad = 0;
    for (int r = 0; r < N; r++)
        for (int j = 0; j < N; j++) {
            const int64_t m = (int64_t)std::llround(std::ldexp(C[N * r + j], FxShift<N>::Q - E));
            const uint32_t lo = (uint32_t)m;
            op.l[r][j] = (int32_t)lo;
            op.h[r][j] = (int32_t)((m - (int64_t)(int32_t)lo) >> 32);
        }
    return true;
}

inline bool make_op4(const double C[16], Op4& op) { return make_op<4>(C, op); }

// Host: multiplication by the complex scalar f = (re, im) on (a.re, a.im)
inline bool make_scalar_op(double re, double im, Op2& op) {
    const double C[4] = {re, -im, im, re};
    return make_op<2>(C, op);
}

// Host: the real form (2D x 2D, row-major) of a complex D x D matrix u (row-major,
// interleaved re/im); in/out order (a0.re, a0.im, a1.re, a1.im, ...)
inline void real_form(const double* u, int D, double* C) {
    const int W = 2 * D;
    for (int r = 0; r < D; r++)
        for (int j = 0; j < D; j++) {
            const double re = u[2 * (D * r + j)], im = u[2 * (D * r + j) + 1];
            C[W * (2 * r) + 2 * j] = re;
            C[W * (2 * r) + 2 * j + 1] = -im;
            C[W * (2 * r + 1) + 2 * j] = im;
            C[W * (2 * r + 1) + 2 * j + 1] = re;
        }
}

// Host: the real form of out = U * (a0, a1) for a complex 2x2 U given as
// {re00, im00, re01, im01, re10, im10, re11, im11}; in/out order (a0.re, a0.im, a1.re, a1.im)
inline void real_form_2x2(const double u[8], double C[16]) {
    for (int r = 0; r < 2; r++)
        for (int j = 0; j < 2; j++) {
            const double re = u[2 * (2 * r + j)], im = u[2 * (2 * r + j) + 1];
            C[4 * (2 * r) + 2 * j] = re;           // out_r.re += re * a_j.re
            C[4 * (2 * r) + 2 * j + 1] = -im;      //           - im * a_j.im
            C[4 * (2 * r + 1) + 2 * j] = im;       // out_r.im += im * a_j.re
            C[4 * (2 * r + 1) + 2 * j + 1] = re;   //           + re * a_j.im
        }
}

}  // namespace qgfx
