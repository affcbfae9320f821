// Host check of the exact 8-bit slice arithmetic of the tensor-core dense kernel
// (quest_gb300/csrc/qg_slices.h):
//  * the digits of every input and operator coefficient add back to its fixed-point value;
//  * every digit sum acc_s stays below 2^22 (so it is exact in FP32, and the kernel's
//    float-to-integer step is exact);
//  * each output is within the stated bound of a long-double evaluation: (KR + 2) 2^-53
//    of (2^(Eg-1023) x 2^eR), the bounds of the largest input and coefficient, plus half an
//    ulp of the result;
//  * groups with Inf/NaN or scales outside [EMIN, EMAX] are refused (the kernel's FP64
//    path), an all-zero group gives zeros.
// Prints one summary line starting "OK" when every case passes.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "qg_slices.h"

typedef long double ld;

static int failures = 0;
static long numChecked = 0, numRefused = 0;
static double worstRatio = 0, worstRatioF64 = 0;

static void fail(const char* what) {
    if (failures < 10) std::printf("FAIL: %s\n", what);
    failures++;
}

// Haar-like D x D unitary (Gram-Schmidt on Gaussian columns), row-major, re/im interleaved
static std::vector<double> unitary(std::mt19937_64& g, int D) {
    std::normal_distribution<double> nd;
    std::vector<std::complex<double>> m(D * D);
    for (auto& z : m) z = {nd(g), nd(g)};
    for (int c = 0; c < D; c++) {
        for (int p = 0; p < c; p++) {
            std::complex<double> dot = 0;
            for (int r = 0; r < D; r++) dot += std::conj(m[r * D + p]) * m[r * D + c];
            for (int r = 0; r < D; r++) m[r * D + c] -= dot * m[r * D + p];
        }
        double nrm = 0;
        for (int r = 0; r < D; r++) nrm += std::norm(m[r * D + c]);
        nrm = std::sqrt(nrm);
        for (int r = 0; r < D; r++) m[r * D + c] /= nrm;
    }
    std::vector<double> u(2 * D * D);
    for (int i = 0; i < D * D; i++) { u[2 * i] = m[i].real(); u[2 * i + 1] = m[i].imag(); }
    return u;
}

static void check_operator_digits(const std::vector<double>& R, int KR, const std::vector<int8_t>& dig, int eR) {
    for (int n = 0; n < KR; n++)
        for (int k = 0; k < KR; k++) {
            const int64_t v = (int64_t)std::llround(std::ldexp(R[n * KR + k], 61 - eR));
            if (v > ((int64_t)1 << 61) || v < -((int64_t)1 << 61)) fail("operator value above 2^61");
            __int128 sum = 0;
            for (int j = 0; j < qgsl::RD; j++) sum = sum * 256 + dig[(j * KR + n) * KR + k];
            if (sum != (__int128)v) fail("operator digits do not add back");
        }
}

// one group: digit identities, sum bounds, and the output error against long double
static void check_group(const std::vector<double>& R, int KR, const std::vector<int8_t>& dig, int eR, const double* x,
                        ld maxR) {
    std::vector<double> y(KR);
    if (!qgsl::apply_group(dig.data(), eR, KR, x, y.data())) { numRefused++; return; }
    int Eg = 1;
    bool nonzero = false;
    for (int k = 0; k < KR; k++) {
        const uint64_t u = qgfx::f64_bits(x[k]);
        const int ei = (int)((u >> 52) & 0x7FF);
        Eg = std::max(Eg, ei + (ei == 0));
        nonzero = nonzero || (u << 1) != 0;
    }
    if (!nonzero) {
        for (int n = 0; n < KR; n++)
            if (y[n] != 0.0) fail("all-zero group gave a nonzero output");
        return;
    }
    // digits of the inputs add back to V = trunc(x 2^(1076 - Eg))
    for (int k = 0; k < KR; k++) {
        const uint64_t u = qgfx::f64_bits(x[k]), W = qgsl::input_word(u, Eg);
        int64_t sum = 0;
        for (int i = 0; i < qgsl::XD; i++) {
            const int dgt = qgsl::input_digit(u, W, i);
            if (dgt < -128 || dgt > 128) fail("input digit out of range");
            sum = sum * 256 + dgt;
        }
        const ld V = std::trunc(std::ldexp((ld)x[k], 1076 - Eg));
        if ((ld)sum != V) fail("input digits do not add back");
        if (std::fabs(V) >= std::ldexp((ld)1, 54)) fail("input value above 2^54");
    }
    // every digit sum below 2^22
    for (int n = 0; n < KR; n++)
        for (int s = 0; s < qgsl::NSUM; s++) {
            int64_t acc = 0;
            for (int i = 0; i < qgsl::XD; i++) {
                const int j = s - i;
                if (j < 0 || j >= qgsl::RD) continue;
                for (int k = 0; k < KR; k++)
                    acc += (int64_t)qgsl::input_digit(qgfx::f64_bits(x[k]), qgsl::input_word(qgfx::f64_bits(x[k]), Eg), i) *
                           dig[(j * KR + n) * KR + k];
            }
            if (acc >= ((int64_t)1 << 22) || acc <= -((int64_t)1 << 22)) fail("digit sum reached 2^22");
        }
    const ld M = std::ldexp((ld)1, Eg - 1023) * std::ldexp((ld)1, eR);
    (void)maxR;
    for (int n = 0; n < KR; n++) {
        ld ref = 0;
        double f64 = 0;
        for (int k = 0; k < KR; k++) {
            ref += (ld)R[n * KR + k] * (ld)x[k];
            f64 = std::fma(R[n * KR + k], x[k], f64);
        }
        const ld bound = (ld)(KR + 2) * std::ldexp((ld)1, -53) * M + std::ldexp(std::fabs(ref), -53) + 1e-320L;
        const ld err = std::fabs((ld)y[n] - ref);
        numChecked++;
        if (err > bound) {
            if (failures < 10)
                std::printf("out of bound: KR=%d n=%d got %.17g want %.20Lg err %Lg bound %Lg\n", KR, n, y[n], ref, err, bound);
            failures++;
        }
        worstRatio = std::max(worstRatio, (double)(err / bound));
        worstRatioF64 = std::max(worstRatioF64, (double)(std::fabs((ld)f64 - ref) / bound));
    }
}

template <int K>
static void run(std::mt19937_64& g, int operators, int groups) {
    constexpr int D = 1 << K, KR = 2 * D;
    std::normal_distribution<double> nd;
    std::uniform_int_distribution<int> wide(-80, 0), scale(-60, 60), pick(0, 9);
    for (int o = 0; o < operators; o++) {
        std::vector<double> u = unitary(g, D);
        if (o % 5 == 1)   // a general (non-unitary) operator with entries of mixed size
            for (auto& v : u) v = std::ldexp(nd(g), scale(g) / 4);
        if (o % 7 == 3)   // a sparse operator (a permutation with phases)
            for (int i = 0; i < D * D; i++) {
                const bool on = (i / D) == ((i % D) * 5 + 3) % D;
                u[2 * i] = on ? std::cos(0.3 * i) : 0.0;
                u[2 * i + 1] = on ? std::sin(0.3 * i) : 0.0;
            }
        std::vector<double> R(KR * KR);
        qgfx::real_form(u.data(), D, R.data());
        std::vector<int8_t> dig(qgsl::RD * KR * KR);
        int eR = 0;
        if (!qgsl::operator_digits(R.data(), KR, dig.data(), &eR)) { fail("finite operator refused"); continue; }
        check_operator_digits(R, KR, dig, eR);
        ld maxR = 0;
        for (double v : R) maxR = std::max(maxR, std::fabs((ld)v));
        if (maxR >= std::ldexp((ld)1, eR) || (maxR > 0 && maxR < std::ldexp((ld)1, eR - 1))) fail("operator scale");
        for (int t = 0; t < groups; t++) {
            std::vector<double> x(KR);
            const int style = pick(g);
            const int base = scale(g);
            for (int k = 0; k < KR; k++) {
                double v = std::ldexp(nd(g), base);
                if (style == 1) v = std::ldexp(nd(g), base + wide(g));          // members up to 2^80 apart
                if (style == 2 && (k % 3)) v = 0.0;                              // zeros among them
                if (style == 3 && k) v = std::ldexp(nd(g), -1060);              // denormals beside one normal
                if (style == 4) v = std::ldexp(nd(g), -1060);                   // all denormal: refused
                if (style == 5) v = (k % 2) ? -0.0 : 0.0;                       // all zero
                if (style == 6 && k == 3) v = std::ldexp(1.0, base) * (1 - std::ldexp(1.0, -53));   // a largest mantissa
                x[k] = v;
            }
            check_group(R, KR, dig, eR, x.data(), maxR);
        }
        // refused: Inf, NaN, scales beyond the normal range of the result
        std::vector<double> x(KR, 0.5);
        std::vector<double> y(KR);
        x[1] = INFINITY;
        if (qgsl::apply_group(dig.data(), eR, KR, x.data(), y.data())) fail("Inf not refused");
        x[1] = NAN;
        if (qgsl::apply_group(dig.data(), eR, KR, x.data(), y.data())) fail("NaN not refused");
        x[1] = std::ldexp(1.0, 1020 - eR);
        if (eR >= 0 && qgsl::apply_group(dig.data(), eR, KR, x.data(), y.data())) fail("huge scale not refused");
    }
}

// fp16 bits of every digit value decode back to it
static void check_digit_half() {
    for (int v = -128; v <= 128; v++) {
        const uint16_t h = qgsl::digit_half(v);
        const int e = (h >> 10) & 0x1F, f = h & 0x3FF;
        const double back = (h & 0x8000 ? -1.0 : 1.0) * (e ? std::ldexp(1.0 + f / 1024.0, e - 15) : std::ldexp(f / 1024.0, -14));
        if (back != (double)v) fail("fp16 digit does not decode to its value");
    }
}

int main() {
    std::mt19937_64 g(20261204);
    check_digit_half();
    run<3>(g, 60, 400);
    run<4>(g, 60, 400);
    if (numRefused == 0) fail("no group took the FP64 path");
    std::printf("%s checked %ld outputs, %ld groups to FP64, worst error / bound %.3f (FP64 FMA chain %.3f), %d failures\n",
                failures ? "FAIL" : "OK", numChecked, numRefused, worstRatio, worstRatioF64, failures);
    return failures ? 1 : 0;
}
