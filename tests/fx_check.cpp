// Host check of the block-floating fixed-point amplitude-pair arithmetic
// (quest_gb300/csrc/qg_fixed.cuh) against long-double evaluation.
// Prints one summary line; exit status 0 when every case is within its bound.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>
#include <complex>
#include <vector>

#include "qg_fixed.cuh"

typedef long double ld;

static int failures = 0;
static double worstRatio = 0, worstRatioF64 = 0;
static long numChecked = 0, numFallback = 0;

static int variant = 0;   // 0: integer conversions (apply_op), 1: hardware output conversion (apply_op_cvt),
                          // 2: its fast form for near-equal exponents with the general one behind it

static void check_case(const double C[16], const double in[4], bool expectFast) {
    qgfx::Op4 op;
    if (!qgfx::make_op4(C, op)) { failures++; std::printf("make_op4 refused a finite operator\n"); return; }
    double out[4];
    bool ok = variant == 2 ? qgfx::apply_op_best<4>(op, in, out)
              : variant ? qgfx::apply_op_cvt<4>(op, in, out) : qgfx::apply_op4(op, in, out);
    if (variant == 2) {   // where the fast form applies it gives the general form's bits
        double o1[4], o2[4];
        if (qgfx::apply_op_near<4>(op, in, o1) && qgfx::apply_op_cvt<4>(op, in, o2))
            for (int r = 0; r < 4; r++)
                if (qgfx::f64_bits(o1[r]) != qgfx::f64_bits(o2[r])) { failures++; std::printf("fast form differs\n"); break; }
    }
    if (!ok) {
        numFallback++;
        if (expectFast) { failures++; std::printf("unexpected fallback: in %g %g %g %g\n", in[0], in[1], in[2], in[3]); }
        return;
    }
    ld maxIn = 0, maxC = 0;
    for (int j = 0; j < 4; j++) maxIn = std::fmax(maxIn, std::fabs((ld)in[j]));
    for (int i = 0; i < 16; i++) maxC = std::fmax(maxC, std::fabs((ld)C[i]));
    for (int r = 0; r < 4; r++) {
        ld ref = 0;
        double f64 = 0;
        for (int j = 0; j < 4; j++) { ref += (ld)C[4 * r + j] * (ld)in[j]; f64 = std::fma(C[4 * r + j], in[j], f64); }
        // bound: 1.5 * 2^-53 of (max |in| * max |C|) + half an ulp of the result
        ld bound = std::ldexp((ld)1.5, -53) * maxIn * maxC + std::ldexp(std::fabs(ref), -53) + 1e-320L;
        ld err = std::fabs((ld)out[r] - ref);
        ld errF64 = std::fabs((ld)f64 - ref);
        numChecked++;
        if (err > bound) {
            failures++;
            if (failures < 10) std::printf("out of bound: r=%d got %.17g want %.17Lg err %Lg bound %Lg\n", r, out[r], ref, err, bound);
        }
        worstRatio = std::fmax(worstRatio, (double)(err / bound));
        worstRatioF64 = std::fmax(worstRatioF64, (double)(errF64 / bound));
    }
}

static void haar2(std::mt19937_64& g, double u[8]) {
    std::normal_distribution<double> nd;
    std::complex<double> a(nd(g), nd(g)), b(nd(g), nd(g)), c(nd(g), nd(g)), d(nd(g), nd(g));
    double n0 = std::sqrt(std::norm(a) + std::norm(c));
    a /= n0; c /= n0;
    std::complex<double> p = std::conj(a) * b + std::conj(c) * d;
    b -= p * a; d -= p * c;
    double n1 = std::sqrt(std::norm(b) + std::norm(d));
    b /= n1; d /= n1;
    std::complex<double> m[4] = {a, b, c, d};
    for (int i = 0; i < 4; i++) { u[2 * i] = m[i].real(); u[2 * i + 1] = m[i].imag(); }
}

// D x D complex (N = 2D real) Haar-like unitaries on random inputs; the error bound
// grows with the number of terms and the bits given up for headroom
template <int N>
static void check_wide(std::mt19937_64& g, int cases) {
    constexpr int D = N / 2;
    std::normal_distribution<double> nd;
    std::uniform_int_distribution<int> scale(-70, 8);
    for (int t = 0; t < cases; t++) {
        std::vector<std::complex<double>> m(D * D);
        for (auto& v : m) v = std::complex<double>(nd(g), nd(g));
        for (int c = 0; c < D; c++) {
            for (int p = 0; p < c; p++) {
                std::complex<double> dot = 0;
                for (int r = 0; r < D; r++) dot += std::conj(m[D * r + p]) * m[D * r + c];
                for (int r = 0; r < D; r++) m[D * r + c] -= dot * m[D * r + p];
            }
            double nrm = 0;
            for (int r = 0; r < D; r++) nrm += std::norm(m[D * r + c]);
            for (int r = 0; r < D; r++) m[D * r + c] /= std::sqrt(nrm);
        }
        std::vector<double> u(2 * D * D), C(N * N), in(N), out(N);
        for (int i = 0; i < D * D; i++) { u[2 * i] = m[i].real(); u[2 * i + 1] = m[i].imag(); }
        qgfx::real_form(u.data(), D, C.data());
        qgfx::OpN<N> op;
        if (!qgfx::make_op<N>(C.data(), op)) { failures++; continue; }
        const int s0 = scale(g);
        for (int j = 0; j < N; j++) in[j] = std::ldexp(nd(g), s0 - (int)(g() % 3));
        bool ok = variant == 2 ? qgfx::apply_op_best<N>(op, in.data(), out.data())
                  : variant ? qgfx::apply_op_cvt<N>(op, in.data(), out.data()) : qgfx::apply_op<N>(op, in.data(), out.data());
        if (!ok) { failures++; std::printf("%dx%d fell back\n", N, N); continue; }
        if (variant == 2) {   // the streaming split gives apply_op_best's bits
            int32_t xh[N], xl[N];
            uint32_t down;
            bool zero;
            if (!qgfx::fx_prepare<N>(op, in.data(), xh, xl, down, zero)) { failures++; continue; }
            for (int r = 0; r < N; r++)
                if (qgfx::f64_bits(qgfx::fx_row<N>(op, r, xh, xl, down, zero)) != qgfx::f64_bits(out[r])) {
                    failures++;
                    std::printf("streaming split differs\n");
                    break;
                }
        }
        ld maxIn = 0, maxC = 0;
        for (int j = 0; j < N; j++) maxIn = std::fmax(maxIn, std::fabs((ld)in[j]));
        for (int i = 0; i < N * N; i++) maxC = std::fmax(maxC, std::fabs((ld)C[i]));
        for (int r = 0; r < N; r++) {
            ld ref = 0;
            for (int j = 0; j < N; j++) ref += (ld)C[N * r + j] * (ld)in[j];
            // N terms, each input truncated at 2^-(52+S) of the largest and each coefficient
            // rounded at 2^-Q of the largest; the dropped low x low products and the shift
            // of the middle sum cost N/4 + 1 units of R, one unit being 2^(13-S-Q) of
            // (largest input) x (largest coefficient); half an ulp for the final rounding
            constexpr int S = qgfx::FxShift<N>::S, Q = qgfx::FxShift<N>::Q;
            ld bound = (ld)N * (std::ldexp((ld)1, -(52 + S)) + std::ldexp((ld)1, -Q)) * maxIn * maxC
                       + (ld)(N / 4 + 1) * std::ldexp((ld)1, 13 - S - Q) * maxIn * maxC
                       + std::ldexp(std::fabs(ref), -53) + 1e-320L;
            ld err = std::fabs((ld)out[r] - ref);
            numChecked++;
            if (err > bound) { failures++; if (failures < 10) std::printf("%dx%d out of bound %Lg %Lg\n", N, N, err, bound); }
            worstRatio = std::fmax(worstRatio, (double)(err / bound));
        }
    }
}

// complex D x D operators in the three-product form against long double, and against
// the real-form (four-product) result
template <int D>
static void check_complex(std::mt19937_64& g, int cases) {
    constexpr int N = 2 * D;
    std::normal_distribution<double> nd;
    std::uniform_int_distribution<int> scale(-70, 8);
    for (int t = 0; t < cases; t++) {
        std::vector<double> u(2 * D * D), C(N * N), in(N);
        for (auto& v : u) v = nd(g) * (t & 1 ? 0.3 : 1.0);
        qgfx::real_form(u.data(), D, C.data());
        qgfx::CopN<D> op;
        if (!qgfx::make_cop<D>(u.data(), op)) { failures++; continue; }
        const int s0 = scale(g);
        for (int j = 0; j < N; j++) in[j] = std::ldexp(nd(g), s0 - (int)(g() % 3));
        int32_t xh[D], xl[D], yh[D], yl[D], sh[D], sl[D];
        uint32_t down;
        bool zero;
        if (!qgfx::cfx_prepare<D>(op, in.data(), xh, xl, yh, yl, sh, sl, down, zero)) { failures++; continue; }
        ld maxIn = 0, maxC = 0;
        for (int j = 0; j < N; j++) maxIn = std::fmax(maxIn, std::fabs((ld)in[j]));
        for (int i = 0; i < N * N; i++) maxC = std::fmax(maxC, std::fabs((ld)C[i]));
        constexpr int S = qgfx::FxShift<N>::S, Q = qgfx::FxShift<N>::Q;
        for (int r = 0; r < D; r++) {
            double out[2];
            qgfx::cfx_row<D>(op, r, xh, xl, yh, yl, sh, sl, down, zero, out[0], out[1]);
            for (int c = 0; c < 2; c++) {
                ld ref = 0;
                for (int j = 0; j < N; j++) ref += (ld)C[N * (2 * r + c)] * 0 + (ld)C[N * (2 * r + c) + j] * (ld)in[j];
                // as the real form, with twice the coefficient rounding (A + B, B - A) and
                // two sums' dropped terms per part
                ld bound = (ld)N * (std::ldexp((ld)1, -(52 + S)) + std::ldexp((ld)2, -Q)) * maxIn * maxC
                           + (ld)(2 * (D / 4 + 1)) * std::ldexp((ld)1, 13 - S - Q) * maxIn * maxC
                           + std::ldexp(std::fabs(ref), -53) + 1e-320L;
                ld err = std::fabs((ld)out[c] - ref);
                numChecked++;
                if (err > bound) { failures++; if (failures < 10) std::printf("complex %d out of bound %Lg %Lg\n", D, err, bound); }
                worstRatio = std::fmax(worstRatio, (double)(err / bound));
            }
        }
    }
}

static void run_all();

int main() {
    for (variant = 0; variant < 3; variant++) run_all();
    return failures ? 1 : 0;
}

static void run_all() {
    worstRatio = worstRatioF64 = 0;
    numChecked = numFallback = 0;
    std::mt19937_64 g(20261204);
    std::normal_distribution<double> nd;
    std::uniform_int_distribution<int> scale(-70, 8), spread(0, 80);
    double u[8], C[16], in[4];
    // Haar unitaries on Gaussian pairs, the pair's members at independent scales
    for (int t = 0; t < 200000; t++) {
        haar2(g, u);
        qgfx::real_form_2x2(u, C);
        int s0 = scale(g), s1 = s0 - spread(g) * (t & 1);
        for (int j = 0; j < 4; j++) in[j] = std::ldexp(nd(g), j < 2 ? s0 : s1);
        check_case(C, in, true);
    }
    // general (non-unitary) complex matrices with entries at mixed scales
    for (int t = 0; t < 50000; t++) {
        for (int i = 0; i < 8; i++) u[i] = std::ldexp(nd(g), (int)(g() % 40) - 20);
        qgfx::real_form_2x2(u, C);
        for (int j = 0; j < 4; j++) in[j] = std::ldexp(nd(g), scale(g));
        check_case(C, in, true);
    }
    // exact zeros, signed zeros and exactly representable small integers
    {
        haar2(g, u);
        qgfx::real_form_2x2(u, C);
        double z[4] = {0.0, -0.0, 0.0, 0.0};
        check_case(C, z, true);
        double ints[4] = {1.0, -2.0, 3.0, 0.5};
        double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        qgfx::Op4 op;
        qgfx::make_op4(I, op);
        double out[4];
        if (!qgfx::apply_op4(op, ints, out) || out[0] != 1.0 || out[1] != -2.0 || out[2] != 3.0 || out[3] != 0.5) {
            failures++;
            std::printf("identity does not reproduce exact inputs\n");
        }
    }
    // denormal inputs next to normal ones: exact conversion, normal results
    for (int t = 0; t < 1000; t++) {
        haar2(g, u);
        qgfx::real_form_2x2(u, C);
        in[0] = nd(g); in[1] = nd(g);
        in[2] = std::ldexp(nd(g), -1060); in[3] = std::ldexp(nd(g), -1070);
        check_case(C, in, true);
    }
    // Inf / NaN in the pair, and results leaving the normal range, must fall back
    {
        haar2(g, u);
        qgfx::real_form_2x2(u, C);
        qgfx::Op4 op;
        qgfx::make_op4(C, op);
        double out[4];
        double bad[3][4] = {{INFINITY, 0, 1, 0}, {NAN, 0, 0, 0}, {1e-310, 1e-311, -1e-310, 0}};
        for (auto& b : bad)
            if (variant == 2 ? qgfx::apply_op_best<4>(op, b, out)
                : variant ? qgfx::apply_op_cvt<4>(op, b, out) : qgfx::apply_op4(op, b, out)) {
                failures++;
                std::printf("special input not sent to FP64\n");
            }
        double big[16];
        for (int i = 0; i < 16; i++) big[i] = C[i] * 1e300;
        qgfx::make_op4(big, op);
        double huge[4] = {1e300, -1e300, 1e300, 1e300};
        if (variant == 2 ? qgfx::apply_op_best<4>(op, huge, out)
            : variant ? qgfx::apply_op_cvt<4>(op, huge, out) : qgfx::apply_op4(op, huge, out)) {
            failures++;
            std::printf("overflow not sent to FP64\n");
        }
    }
    // complex scalars (phases and general factors) on single amplitudes
    for (int t = 0; t < 100000; t++) {
        double th = std::uniform_real_distribution<double>(0, 6.283185307179586)(g);
        double re = std::cos(th), im = std::sin(th);
        if (t & 1) { re = std::ldexp(nd(g), (int)(g() % 20) - 10); im = std::ldexp(nd(g), (int)(g() % 20) - 10); }
        qgfx::Op2 op;
        if (!qgfx::make_scalar_op(re, im, op)) { failures++; continue; }
        double a[2] = {std::ldexp(nd(g), scale(g)), std::ldexp(nd(g), scale(g) - spread(g) * (t & 2))};
        double out[2];
        if (!(variant == 2 ? qgfx::apply_op_best<2>(op, a, out)
              : variant ? qgfx::apply_op_cvt<2>(op, a, out) : qgfx::apply_op<2>(op, a, out))) {
            failures++;
            std::printf("scalar fell back\n");
            continue;
        }
        ld maxIn = std::fmax(std::fabs((ld)a[0]), std::fabs((ld)a[1]));
        ld maxC = std::fmax(std::fabs((ld)re), std::fabs((ld)im));
        ld ref[2] = {(ld)re * a[0] - (ld)im * a[1], (ld)im * a[0] + (ld)re * a[1]};
        for (int r = 0; r < 2; r++) {
            ld bound = std::ldexp((ld)1.5, -53) * maxIn * maxC + std::ldexp(std::fabs(ref[r]), -53) + 1e-320L;
            ld err = std::fabs((ld)out[r] - ref[r]);
            numChecked++;
            if (err > bound) { failures++; if (failures < 10) std::printf("scalar out of bound %Lg %Lg\n", err, bound); }
            worstRatio = std::fmax(worstRatio, (double)(err / bound));
        }
    }
    // 8x8 real operators (complex 4x4: two-qubit gates) on four amplitudes
    for (int t = 0; t < 50000; t++) {
        std::complex<double> m[16];
        for (auto& v : m) v = std::complex<double>(nd(g), nd(g));
        for (int c = 0; c < 4; c++) {           // Gram-Schmidt on the columns: a Haar-like unitary
            for (int p = 0; p < c; p++) {
                std::complex<double> dot = 0;
                for (int r = 0; r < 4; r++) dot += std::conj(m[4 * r + p]) * m[4 * r + c];
                for (int r = 0; r < 4; r++) m[4 * r + c] -= dot * m[4 * r + p];
            }
            double nrm = 0;
            for (int r = 0; r < 4; r++) nrm += std::norm(m[4 * r + c]);
            for (int r = 0; r < 4; r++) m[4 * r + c] /= std::sqrt(nrm);
        }
        if (t & 1)
            for (auto& v : m) v *= std::ldexp(1.0, (int)(g() % 12) - 6);   // non-unitary scales too
        double u16[32], C8[64], in8[8], out8[8];
        for (int i = 0; i < 16; i++) { u16[2 * i] = m[i].real(); u16[2 * i + 1] = m[i].imag(); }
        qgfx::real_form(u16, 4, C8);
        qgfx::OpN<8> op;
        if (!qgfx::make_op<8>(C8, op)) { failures++; continue; }
        const int s0 = scale(g);
        for (int j = 0; j < 8; j++) in8[j] = std::ldexp(nd(g), s0 - (int)(g() % 4) * spread(g) / 8);
        bool ok = variant == 2 ? qgfx::apply_op_best<8>(op, in8, out8)
                  : variant ? qgfx::apply_op_cvt<8>(op, in8, out8) : qgfx::apply_op<8>(op, in8, out8);
        if (!ok) { failures++; std::printf("8x8 fell back\n"); continue; }
        ld maxIn = 0, maxC = 0;
        for (int j = 0; j < 8; j++) maxIn = std::fmax(maxIn, std::fabs((ld)in8[j]));
        for (int i = 0; i < 64; i++) maxC = std::fmax(maxC, std::fabs((ld)C8[i]));
        for (int r = 0; r < 8; r++) {
            ld ref = 0;
            for (int j = 0; j < 8; j++) ref += (ld)C8[8 * r + j] * (ld)in8[j];
            // the 8-term bound: one more input bit dropped, twice the terms
            ld bound = std::ldexp((ld)3.0, -53) * maxIn * maxC + std::ldexp(std::fabs(ref), -53) + 1e-320L;
            ld err = std::fabs((ld)out8[r] - ref);
            numChecked++;
            if (err > bound) { failures++; if (failures < 10) std::printf("8x8 out of bound %Lg %Lg\n", err, bound); }
            worstRatio = std::fmax(worstRatio, (double)(err / bound));
        }
    }
    // 16x16 and 32x32 real operators (three- and four-target matrices, two-qubit
    // superoperators) on 8 and 16 amplitudes
    check_wide<16>(g, 20000);
    check_wide<32>(g, 10000);
    check_complex<2>(g, 20000);
    check_complex<4>(g, 20000);
    check_complex<8>(g, 10000);
    check_complex<16>(g, 5000);
    std::printf("%s variant=%d checked=%ld fallback=%ld worst_err_over_bound=%.3f fp64_fma_worst_over_bound=%.3f failures=%d\n",
                failures ? "FAIL" : "OK", variant, numChecked, numFallback, worstRatio, worstRatioF64, failures);
}
