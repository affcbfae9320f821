// Exact 8-bit slices: FP64 dense products on the fp16 tensor cores.
//
// A multi-target dense gate applies the real KR x KR form R of its complex matrix to each
// group of KR/2 amplitudes (KR reals x_k, re/im interleaved): y_n = sum_k R[n][k] x_k.
// GB300's FP64 pipe issues about 2 FMAs per clock per SM and its integer multiply-add pipe
// a few times more, far below what HBM can feed for 16 or 32 products per real; its fp16
// tensor cores run thousands.  An fp16 value holds any integer of magnitude <= 2048
// exactly, and the tensor cores multiply fp16 exactly and add in FP32, which is exact
// while every partial sum is an integer below 2^24.  So both operands are cut into signed
// 8-bit digits and the digit products are summed on the tensor cores, exactly; the exact
// digit sums are then combined in 64-bit integers (the idea of the Ozaki scheme, with
// fixed-point slices).
//
//  * Inputs share one scale per group: Eg = the largest biased exponent among the group's
//    KR reals.  Each real v (biased exponent e, 53-bit significand m with the implicit bit)
//    becomes |V| = trunc(m 2^(1 - (Eg - e))) = trunc(|v| 2^(1076 - Eg)) < 2^54, and
//    W = |V| + CX (CX = 0x80 in each of 7 bytes), 0 <= W < 2^56.  Digit i (i = 0 most
//    significant) is sign(v) (byte 6 - i of W minus 128), in [-128, 128], and
//    V = sign(v) |V| = sum_i d_i 2^(8(6-i)).  Zeros and denormals enter as V = 0 (Eg >= 56
//    below, so a denormal is below 2^-55 of the group's largest value).
//  * The operator shares one scale: eR with every |R| < 2^eR; Vr = round(R * 2^(61 - eR)),
//    |Vr| <= 2^61, Wr = Vr + CR (0x80 in each of 8 bytes), digit j = byte 7 - j of Wr minus
//    128, and Vr = sum_j r_j 2^(8(7-j)).
//  * sum_k V_k Vr_nk = sum_s acc_s 2^(104 - 8s) with acc_s = sum over i + j = s of
//    sum_k d_i[k] r_j[n][k].  The sums s = 0..7 are kept (s = i + j >= 8 is dropped).
//    Each acc_s has at most 7 digit pairs of KR <= 32 products of magnitude <= 128 x 128:
//    |acc_s| < 2^22, exact in FP32 and through the tensor cores' FP32 sums.
//  * Y = sum_{s<=7} acc_s 2^(8(7-s)) (|Y| <= 2^72), Y' = floor(Y / 2^11) in int64, and
//    y = (double)Y' * 2^(Eg + eR - 1078), the conversion rounding to nearest even and the
//    power of two added to the exponent field.
//
// Error per output, relative to M = 2^(Eg-1023) x 2^eR (the bounds of the largest |x| in
// the group and of the largest |R|): the inputs' truncation below KR x 2^-53, the dropped
// digit sums below 2^-52.4 (KR = 32), the floor 2^-55 and the operator's rounding
// KR x 2^-62, in all below (KR + 2) 2^-53 M; plus half an ulp of the result.  That is the
// order of an FP64 FMA chain's own bound for the same KR-term sums (tests/slices_check.cpp
// checks it on random, general and sparse operators and on groups whose members differ by
// up to 2^80).
//
// A group holding Inf or NaN, whose largest value is denormal, or whose scale leaves the
// range where every output is a normal double or zero (Eg < 56, or Eg + eR outside
// [56, 2039]), is evaluated in FP64 instead; an all-zero group gives zeros.
//
// Everything here is plain C++ usable on the host (the operator's digits, and the tests'
// restatement of the kernel, which must match it bit for bit) and in CUDA device code.
#pragma once

#include <stdint.h>

#include <cmath>

#include "qg_fixed.cuh"   // QG_HD, f64_bits, bits_f64

namespace qgsl {

const int XD = 7;                            // digits of an input
const int RD = 8;                            // digits of an operator coefficient
const int NSUM = 8;                          // digit sums kept: s = i + j = 0..7
const uint64_t CX = 0x80808080808080ull;     // 128 in each of the 7 input digit positions
const uint64_t CR = 0x8080808080808080ull;   // 128 in each of the 8 operator digit positions
const int YSHIFT = 11;                       // Y' = floor(Y / 2^11)
const int SCALE_OFF = 1078;                  // y = Y' * 2^(Eg + eR - 1078)
const int EMIN = 56, EMAX = 2039;            // normal groups: EMIN <= Eg + eR <= EMAX

// W = |V| + CX of the real with bits u at the group scale Eg (Eg >= its biased exponent)
QG_HD uint64_t input_word(uint64_t u, int Eg) {
    const int d = Eg - (int)((u >> 52) & 0x7FF);
    const uint64_t m2 = ((u & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 1;
    return (d < 64 ? m2 >> d : 0ull) + CX;
}

// digit i of the real with bits u and word W
QG_HD int input_digit(uint64_t u, uint64_t W, int i) {
    const int b = (int)((W >> (8 * (6 - i))) & 0xFF) - 128;
    return (u >> 63) ? -b : b;
}

// Y' from the eight exact digit sums acc[0..7] (acc[s] for s = i + j)
QG_HD int64_t combine(const int32_t* acc) {
    const int32_t h1 = acc[0] * 256 + acc[1], h2 = acc[2] * 256 + acc[3];
    const int32_t l1 = acc[4] * 256 + acc[5], l2 = acc[6] * 256 + acc[7];
    // Y = h1 2^48 + h2 2^32 + l1 2^16 + l2; the first three are multiples of 2^11
    return (int64_t)h1 * ((int64_t)1 << 37) + (int64_t)h2 * ((int64_t)1 << 21) + (int64_t)l1 * 32 + (int64_t)(l2 >> 11);
}

// Y' * 2^shift as a double (shift = Eg + eR - 1078, inside the normal range by the group test)
QG_HD double to_output(int64_t Y, int shift) {
    if (Y == 0) return 0.0;
    const double d = (double)Y;
    return qgfx::bits_f64(qgfx::f64_bits(d) + ((uint64_t)(int64_t)shift << 52));
}

// Host: the operator's digits, dig[(j * N + n) * N + k] = r_j of R[n][k] (R row-major N x N),
// and its scale eR.  false when a coefficient is not finite.
inline bool operator_digits(const double* R, int N, int8_t* dig, int* eR) {
    int E = -100000;
    for (int i = 0; i < N * N; i++) {
        if (!(R[i] - R[i] == 0.0)) return false;
        if (R[i] != 0.0) {
            int ex;
            std::frexp(R[i], &ex);   // |R| < 2^ex
            E = ex > E ? ex : E;
        }
    }
    if (E == -100000) E = 0;
    *eR = E;
    for (int n = 0; n < N; n++)
        for (int k = 0; k < N; k++) {
            const int64_t v = (int64_t)std::llround(std::ldexp(R[n * N + k], 61 - E));
            const uint64_t w = (uint64_t)v + CR;
            for (int j = 0; j < RD; j++) dig[(j * N + n) * N + k] = (int8_t)((int)((w >> (8 * (7 - j))) & 0xFF) - 128);
        }
    return true;
}

// Host: fp16 bits of a digit (an integer of magnitude <= 128)
inline uint16_t digit_half(int v) {
    if (v == 0) return 0;
    const uint16_t sgn = v < 0 ? 0x8000 : 0;
    int a = v < 0 ? -v : v, p = 0;
    while ((a >> (p + 1)) != 0) p++;                    // a = 1.f x 2^p
    return (uint16_t)(sgn | (uint16_t)((p + 15) << 10) | (uint16_t)(((a << (10 - p)) & 0x3FF)));
}

// Host restatement of the kernel for one group: y = R x with the operator's digits and
// scale, the group's KR reals x (re/im interleaved).  Returns false for a group that the
// kernel evaluates in FP64 (the caller then does so, in the kernel's order).
inline bool apply_group(const int8_t* dig, int eR, int KR, const double* x, double* y) {
    int Eg = 0;
    bool nonzero = false;
    for (int k = 0; k < KR; k++) {
        const uint64_t u = qgfx::f64_bits(x[k]);
        const int e = (int)((u >> 52) & 0x7FF);
        Eg = e > Eg ? e : Eg;
        nonzero = nonzero || (u << 1) != 0;
    }
    if (Eg == 2047) return false;                       // Inf or NaN
    if (Eg == 0) {
        if (nonzero) return false;                      // denormals only
        Eg = 1023;                                      // all zero: zero digits, zero outputs
    } else if (Eg < EMIN || Eg + eR < EMIN || Eg + eR > EMAX) {
        return false;
    }
    uint64_t U[64], W[64];
    for (int k = 0; k < KR; k++) {
        U[k] = qgfx::f64_bits(x[k]);
        W[k] = input_word(U[k], Eg);
    }
    for (int n = 0; n < KR; n++) {
        int32_t acc[NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < XD; i++)
            for (int j = 0; j < RD && i + j < NSUM; j++) {
                int32_t s = 0;
                for (int k = 0; k < KR; k++) s += input_digit(U[k], W[k], i) * dig[(j * KR + n) * KR + k];
                acc[i + j] += s;
            }
        y[n] = to_output(combine(acc), Eg + eR - SCALE_OFF);
    }
    return true;
}

}  // namespace qgsl
