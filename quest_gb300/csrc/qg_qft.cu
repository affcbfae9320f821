// Steps of the quantum Fourier transform on a statevector in one pass: the Hadamard on
// target t followed by its controlled phases.  QuEST's applyQuantumFourierTransform
// (quest/src/api/operations.cpp:1934-1952) applies, for each target t[n] from the top,
// applyHadamard(t[n]) and then applyTwoQubitPhaseShift(t[n], t[n-m-1], pi / 2^(m+1)) for
// m < n: one pass per gate, n + 1 passes for this step.  For contiguous targets
// t[j] = t0 + j those phases multiply every amplitude whose bit t[n] is set by
//     exp(i pi sum_{m<n} x_{t[n-m-1]} / 2^(m+1)) = exp(i pi L / 2^n),
// L = (index >> t0) & (2^n - 1), so the step is a radix-2 butterfly with a twiddle:
//     out0 = (a0 + a1) / sqrt2,   out1 = w^L (a0 - a1) / sqrt2,   w = exp(i pi / 2^n),
// for each pair (a0, a1) of amplitudes that differ in bit t[n] only.
//
// Products in 60-bit block-floating fixed point on the integer pipes (as the one-target
// kernels of qg_fixed.cuh; GB300's FP64 rate would bound the twiddle products): the pair's
// four reals share the largest exponent and become integers below 2^60, sums and
// differences are exact, the twiddle w^L / sqrt2 is the product of up to five tables of
// 256 values at scale 2^62 (indices: the bytes of L), and each output is the top 64 bits
// of its products (from 32-bit limbs), converted to double with the scale added to the
// exponent field.  Error per output: a few units of 2^-57 of the pair's largest
// |amplitude|.  Pairs holding Inf/NaN or with scales near the ends of the double range
// are evaluated in FP64.
//
// Targets from qubit 0 take two or three steps per pass (k_qft_two_steps_*,
// k_qft_three_steps_*): a thread holds the 4 or 8 amplitudes that differ in the steps'
// target bits, every twiddle of the steps comes from the first step's tables, and the
// values stay in fixed point between the steps.  The transform's closing swaps on qubits
// 0..n-1 are one in-place bit-reversal pass (k_reverse_low_bits).
//
// The same fixed-point steps apply a set of controlled phases in one pass (k_phase_set):
// phase gates commute, so the API defers them (diagonal gates whose only factor != 1 is on
// the all-ones state of their qubits: CPhase, CZ, phase shifts, S, T, Z) and applies a set
// of up to 32 at once, each amplitude multiplied by the product of the factors whose mask
// it contains.  The products of every subset of 8 factors are tables of 256 values at
// scale 2^62, so an amplitude takes one table value per 8 factors.  Statevectors of at
// least 8 qubits (the API defers phases from 19 qubits on).
#include "qg_common.cuh"
#include "qg_fixed.cuh"

#include <cmath>
#include <complex>
#include <vector>

#define QFT_MAX_TABLES 5         // twiddle index L of up to 40 bits
struct QftTables {
    long long t[QFT_MAX_TABLES][256][2];   // table k, entry j: exp(i pi j 2^(8k) / 2^n) (k = 0: / sqrt2), (re, im) x 2^62
};

// the top 64 bits of a * b (signed), to within 2 units: balanced 32-bit limbs a = ah 2^32 + al
// (al in [-2^31, 2^31)), three 32 x 32 -> 64 products, the low x low one dropped (a full
// 64-bit high product takes several times the instructions on the integer pipe)
__device__ __forceinline__ void limbs(long long a, int& h, int& l) {
    l = (int)(unsigned)a;
    h = (int)((a - (long long)l) >> 32);
}
__device__ __forceinline__ long long mulhi(long long a, long long b) {
    int ah, al, bh, bl;
    limbs(a, ah, al);
    limbs(b, bh, bl);
    const long long mid = (long long)ah * bl + (long long)al * bh;
    return (long long)ah * bh + (mid >> 32);
}

// (a * b) for complex values at scale 2^62 (|a|, |b| <= 1): the product at scale 2^62
__device__ __forceinline__ void cmul62(long long ar, long long ai, long long br, long long bi, long long& cr, long long& ci) {
    cr = (mulhi(ar, br) - mulhi(ai, bi)) * 4;
    ci = (mulhi(ar, bi) + mulhi(ai, br)) * 4;
}

// v (bits u) at the pair scale eb: mant * 2^(7 + eff - eb), below 2^60 in magnitude
__device__ __forceinline__ long long qft_fixed(uint64_t u, int eb) {
    const int ei = (int)((u >> 52) & 0x7FF);
    const uint64_t mant = (u & 0xFFFFFFFFFFFFFull) | (ei ? (1ull << 52) : 0ull);
    const int d = eb - (ei + (ei == 0));
    const uint64_t x = d < 64 ? (mant << 7) >> d : 0ull;
    return (u >> 63) ? -(long long)x : (long long)x;
}

// Y * 2^t as a double (t = eb - 1080 keeps every nonzero output normal for 58 <= eb <= 2043)
__device__ __forceinline__ double qft_double(long long Y, int t) {
    if (Y == 0) return 0.0;
    const double d = __ll2double_rn(Y);
    return __hiloint2double(__double2hiint(d) + t * (1 << 20), __double2loint(d));
}

#define QFT_THREADS 256
#define QFT_C (3260954456333195553LL)    // round(2^62 / sqrt2)

// One butterfly at the pair's own scale: o0 = (v0 + v1) / sqrt2, o1 = w (v0 - v1), with
// (wr, wi) = w at scale 2^62 (the 1/sqrt2 included, |w| <= 1/sqrt2).  The pair's four reals
// share the largest exponent eb and become integers below 2^60; sums and differences are
// exact and each output is the top 64 bits of its products.  Pairs holding Inf/NaN or with
// scales near the ends of the double range are evaluated in FP64.
__device__ __forceinline__ void qft_butterfly(const double2 v0, const double2 v1, long long wr, long long wi, double2& o0,
                                              double2& o1) {
    const uint64_t u[4] = {qgfx::f64_bits(v0.x), qgfx::f64_bits(v0.y), qgfx::f64_bits(v1.x), qgfx::f64_bits(v1.y)};
    int eb = 1;
    uint64_t any = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int ei = (int)((u[k] >> 52) & 0x7FF);
        eb = max(eb, ei + (ei == 0));
        any |= u[k] << 1;
    }
    if (any == 0) {
        o0 = make_double2(0.0, 0.0);
        o1 = o0;
    } else if (eb >= 58 && eb <= 2043) {
        const long long x0r = qft_fixed(u[0], eb), x0i = qft_fixed(u[1], eb);
        const long long x1r = qft_fixed(u[2], eb), x1i = qft_fixed(u[3], eb);
        const long long sr = x0r + x1r, si = x0i + x1i, dr = x0r - x1r, di = x0i - x1i;
        // values * 2^(1082 - eb) / 4: (a0 + a1) / sqrt2 and w (a0 - a1)
        const long long y0r = mulhi(sr, QFT_C), y0i = mulhi(si, QFT_C);
        const long long y1r = mulhi(dr, wr) - mulhi(di, wi), y1i = mulhi(dr, wi) + mulhi(di, wr);
        const int t = eb - 1080;
        o0 = make_double2(qft_double(y0r, t), qft_double(y0i, t));
        o1 = make_double2(qft_double(y1r, t), qft_double(y1i, t));
    } else {
        const double s = 0.70710678118654752440;
        const double cr = (double)wr * 0x1p-62 / s, ci = (double)wi * 0x1p-62 / s;   // w sqrt2
        o0 = make_double2((v0.x + v1.x) * s, (v0.y + v1.y) * s);
        const double dr = (v0.x - v1.x) * s, di = (v0.y - v1.y) * s;
        o1 = make_double2(fma(dr, cr, -di * ci), fma(dr, ci, di * cr));
    }
}

// The butterfly kept in fixed point, for a second step that follows in the same pass.
// qft_fly_fx: a pair of doubles in, y = (o0.re, o0.im, o1.re, o1.im) out as integers at the
// pair's scale, value = y 2^(eb - 1080) (|y| < 2^59); eb = 0 for an all-zero pair; false
// when the pair needs FP64.  qft_fly_int: the same on integer inputs below 2^59 at one
// scale, outputs at that scale divided by 4.
__device__ __forceinline__ bool qft_fly_fx(const double2 v0, const double2 v1, long long wr, long long wi, long long (&y)[4],
                                           int& eb) {
    const uint64_t u[4] = {qgfx::f64_bits(v0.x), qgfx::f64_bits(v0.y), qgfx::f64_bits(v1.x), qgfx::f64_bits(v1.y)};
    eb = 1;
    uint64_t any = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int ei = (int)((u[k] >> 52) & 0x7FF);
        eb = max(eb, ei + (ei == 0));
        any |= u[k] << 1;
    }
    if (any == 0) {
        eb = 0;
        y[0] = y[1] = y[2] = y[3] = 0;
        return true;
    }
    if (eb < 58 || eb > 2043) return false;
    const long long x0r = qft_fixed(u[0], eb), x0i = qft_fixed(u[1], eb);
    const long long x1r = qft_fixed(u[2], eb), x1i = qft_fixed(u[3], eb);
    const long long sr = x0r + x1r, si = x0i + x1i, dr = x0r - x1r, di = x0i - x1i;
    y[0] = mulhi(sr, QFT_C);
    y[1] = mulhi(si, QFT_C);
    y[2] = mulhi(dr, wr) - mulhi(di, wi);
    y[3] = mulhi(dr, wi) + mulhi(di, wr);
    return true;
}
__device__ __forceinline__ void qft_fly_int(long long x0r, long long x0i, long long x1r, long long x1i, long long wr, long long wi,
                                            long long (&y)[4]) {
    const long long sr = x0r + x1r, si = x0i + x1i, dr = x0r - x1r, di = x0i - x1i;
    y[0] = mulhi(sr, QFT_C);
    y[1] = mulhi(si, QFT_C);
    y[2] = mulhi(dr, wr) - mulhi(di, wi);
    y[3] = mulhi(dr, wi) + mulhi(di, wr);
}
__device__ __forceinline__ long long qft_align(long long y, int shift) { return shift >= 63 ? 0 : (y >> shift); }

// the two steps in FP64 butterflies, for a quadruple with a pair that needs them (out of
// line: it is rare, and inlined it took registers from the fixed-point path)
__device__ __noinline__ void qft_two_flies_fp64(const double2 v00, const double2 v01, const double2 v10, const double2 v11,
                                                long long wr, long long wi, long long vr, long long vi, double2& y00,
                                                double2& y01, double2& y10, double2& y11) {
    double2 x00, x01, x10, x11;
    qft_butterfly(v00, v10, wr, wi, x00, x10);
    qft_butterfly(v01, v11, -wi, wr, x01, x11);
    qft_butterfly(x00, x01, vr, vi, y00, y01);
    qft_butterfly(x10, x11, vr, vi, y10, y11);
}

// Two steps on one quadruple (v_xy: bit T = x, bit T - 1 = y): step T on the pairs
// (v_0y, v_1y) with twiddles W and i W, then step T - 1 on (x_x0, x_x1) with twiddle V.
// The values stay in fixed point between the steps: the second step takes the first's
// integer outputs, aligned to the larger of the two pairs' scales (an arithmetic shift of
// the smaller), so the quadruple is converted from and to double once.  A quadruple with a
// pair that needs FP64 takes four FP64 butterflies.
__device__ __forceinline__ void qft_two_flies(const double2 v00, const double2 v01, const double2 v10, const double2 v11,
                                              long long wr, long long wi, long long vr, long long vi, double2& y00,
                                              double2& y01, double2& y10, double2& y11) {
    long long ya[4], yb[4];
    int ea, eb;
    const bool okA = qft_fly_fx(v00, v10, wr, wi, ya, ea);
    const bool okB = qft_fly_fx(v01, v11, -wi, wr, yb, eb);
    if (okA && okB) {
        const int e = max(ea, eb), sa = e - ea, sb = e - eb;
        long long z0[4], z1[4];
        qft_fly_int(qft_align(ya[0], sa), qft_align(ya[1], sa), qft_align(yb[0], sb), qft_align(yb[1], sb), vr, vi, z0);
        qft_fly_int(qft_align(ya[2], sa), qft_align(ya[3], sa), qft_align(yb[2], sb), qft_align(yb[3], sb), vr, vi, z1);
        const int t = e - 1078;      // value = z 2^(e - 1078)
        y00 = make_double2(qft_double(z0[0], t), qft_double(z0[1], t));
        y01 = make_double2(qft_double(z0[2], t), qft_double(z0[3], t));
        y10 = make_double2(qft_double(z1[0], t), qft_double(z1[1], t));
        y11 = make_double2(qft_double(z1[2], t), qft_double(z1[3], t));
    } else {
        qft_two_flies_fp64(v00, v01, v10, v11, wr, wi, vr, vi, y00, y01, y10, y11);
    }
}

// NT tables (compile time, so that every loop over them unrolls)
template <int NT>
__global__ void __launch_bounds__(QFT_THREADS) k_qft_step(double2* __restrict__ a, qidx numPairs, int tb, int lb, qidx lmask,
                                                          const __grid_constant__ QftTables T) {
    constexpr int numTables = NT;
    __shared__ long long sT[NT][256][2];
    for (int e = threadIdx.x; e < numTables * 512; e += QFT_THREADS) (&sT[0][0][0])[e] = (&T.t[0][0][0])[e];
    __syncthreads();
    const qidx stride = (qidx)gridDim.x * QFT_THREADS;
    const qidx lowMask = ((qidx)1 << tb) - 1;
    for (qidx p = blockIdx.x * (qidx)QFT_THREADS + threadIdx.x; p < numPairs; p += stride) {
        const qidx i0 = ((p & ~lowMask) << 1) | (p & lowMask), i1 = i0 | ((qidx)1 << tb);
        const double2 v0 = ld_amp(a + i0), v1 = ld_amp(a + i1);
        // the twiddle w^L / sqrt2 at scale 2^62
        const qidx L = (i0 >> lb) & lmask;
        long long wr = sT[0][L & 255][0], wi = sT[0][L & 255][1];
#pragma unroll
        for (int k = 1; k < numTables; k++) {
            const int j = (int)((L >> (8 * k)) & 255);
            cmul62(wr, wi, sT[k][j][0], sT[k][j][1], wr, wi);
        }
        double2 o0, o1;
        qft_butterfly(v0, v1, wr, wi, o0, o1);
        st_amp(a + i0, o0);
        st_amp(a + i1, o1);
    }
}

// The same step for targets from qubit 0 (lb = 0) and tb >= 8: a warp takes chunks of 256
// consecutive pairs (lane l, round r: pair 256 c + 32 r + l), whose twiddle index L keeps its
// bytes above the lowest across the chunk, so their product H is formed once per chunk and
// each pair takes one complex product T0[L & 255] H instead of NT - 1.
template <int NT>
__global__ void __launch_bounds__(QFT_THREADS) k_qft_step_chunks(double2* __restrict__ a, qidx numChunks, int tb, qidx lmask,
                                                                 const __grid_constant__ QftTables T) {
    __shared__ long long sT[NT][256][2];
    for (int e = threadIdx.x; e < NT * 512; e += QFT_THREADS) (&sT[0][0][0])[e] = (&T.t[0][0][0])[e];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const qidx lowMask = ((qidx)1 << tb) - 1;
    const qidx warps = (qidx)gridDim.x * (QFT_THREADS / 32);
    for (qidx c = blockIdx.x * (qidx)(QFT_THREADS / 32) + (threadIdx.x >> 5); c < numChunks; c += warps) {
        const qidx Lh = (c << 8) & lmask;                       // L's bytes above the lowest
        long long hr = sT[1][(Lh >> 8) & 255][0], hi = sT[1][(Lh >> 8) & 255][1];
#pragma unroll
        for (int k = 2; k < NT; k++) {
            const int j = (int)((Lh >> (8 * k)) & 255);
            cmul62(hr, hi, sT[k][j][0], sT[k][j][1], hr, hi);
        }
#pragma unroll 2
        for (int r = 0; r < 8; r++) {
            const int k0 = 32 * r + lane;                       // L & 255
            const qidx p = (c << 8) + k0;
            const qidx i0 = ((p & ~lowMask) << 1) | (p & lowMask), i1 = i0 | ((qidx)1 << tb);
            const double2 v0 = ld_amp(a + i0), v1 = ld_amp(a + i1);
            long long wr, wi;
            cmul62(sT[0][k0][0], sT[0][k0][1], hr, hi, wr, wi);
            double2 o0, o1;
            qft_butterfly(v0, v1, wr, wi, o0, o1);
            st_amp(a + i0, o0);
            st_amp(a + i1, o1);
        }
    }
}

// Two steps in one pass, targets from qubit 0: the step of target T (twiddle index L = the
// T bits below it) and then the step of target T - 1 (the T - 1 bits below it).  A thread
// takes the four amplitudes a_xy that differ in bits T (x) and T - 1 (y) only; with B = their
// index bits below T - 1 and w = exp(i pi / 2^T):
//     step T:     pairs (a_0y, a_1y), twiddle w^(B + y 2^(T-1)) / sqrt2 = i^y W,  W = w^B / sqrt2
//     step T - 1: pairs (x_x0, x_x1), twiddle exp(i pi B / 2^(T-1)) / sqrt2 = w^(2B) / sqrt2 = V
// Both twiddles come from the tables of step T: W from the bytes of B and V from those of 2B.
// Between the steps the values stay in fixed point (qft_two_flies).
//
// T - 1 >= 8: a warp takes chunks of 256 consecutive quadruples (lane l, round r: B's low
// byte b = 32 r + l).  B's higher bytes are fixed across the chunk, so W's product of the
// higher tables (HW) is formed once per chunk, and V's as well: the bytes of 2B above the
// lowest are those of 2 (B - b) with bit 8 set when b >= 128: two products (H0, H1).
template <int NT>
__global__ void __launch_bounds__(QFT_THREADS, 2) k_qft_two_steps_chunks(double2* __restrict__ a, qidx numChunks, int tb,
                                                                      const __grid_constant__ QftTables T) {
    static_assert(NT >= 2, "T - 1 >= 8 needs two tables");
    __shared__ long long sT[NT][256][2];
    for (int e = threadIdx.x; e < NT * 512; e += QFT_THREADS) (&sT[0][0][0])[e] = (&T.t[0][0][0])[e];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const qidx bMask = ((qidx)1 << (tb - 1)) - 1, half = (qidx)1 << (tb - 1), top = (qidx)1 << tb;
    const qidx warps = (qidx)gridDim.x * (QFT_THREADS / 32);
    for (qidx c = blockIdx.x * (qidx)(QFT_THREADS / 32) + (threadIdx.x >> 5); c < numChunks; c += warps) {
        const qidx Bh = (c << 8) & bMask;                       // B with its low byte cleared
        const qidx B2 = Bh << 1;                                // 2 B with its low 9 bits cleared
        long long hwr = sT[1][(Bh >> 8) & 255][0], hwi = sT[1][(Bh >> 8) & 255][1];
        const int j1 = (int)((B2 >> 8) & 255);
        long long h0r = sT[1][j1][0], h0i = sT[1][j1][1], h1r = sT[1][j1 | 1][0], h1i = sT[1][j1 | 1][1];
#pragma unroll
        for (int k = 2; k < NT; k++) {
            const int j = (int)((Bh >> (8 * k)) & 255), j2 = (int)((B2 >> (8 * k)) & 255);
            cmul62(hwr, hwi, sT[k][j][0], sT[k][j][1], hwr, hwi);
            cmul62(h0r, h0i, sT[k][j2][0], sT[k][j2][1], h0r, h0i);
            cmul62(h1r, h1i, sT[k][j2][0], sT[k][j2][1], h1r, h1i);
        }
#pragma unroll 1
        for (int r = 0; r < 8; r++) {
            const int b = 32 * r + lane;                        // B & 255
            const qidx qd = (c << 8) + b;
            const qidx i00 = ((qd & ~bMask) << 2) | (qd & bMask);
            const double2 v00 = ld_amp(a + i00), v01 = ld_amp(a + i00 + half);
            const double2 v10 = ld_amp(a + i00 + top), v11 = ld_amp(a + i00 + top + half);
            long long wr, wi, vr, vi;
            cmul62(sT[0][b][0], sT[0][b][1], hwr, hwi, wr, wi);
            const bool hi = r >= 4;                             // b >= 128: bit 8 of 2B set
            cmul62(sT[0][(2 * b) & 255][0], sT[0][(2 * b) & 255][1], hi ? h1r : h0r, hi ? h1i : h0i, vr, vi);
            double2 y00, y01, y10, y11;
            qft_two_flies(v00, v01, v10, v11, wr, wi, vr, vi, y00, y01, y10, y11);
            st_amp(a + i00, y00);
            st_amp(a + i00 + half, y01);
            st_amp(a + i00 + top, y10);
            st_amp(a + i00 + top + half, y11);
        }
    }
}

// The same for 1 <= T <= 8: B < 128 and 2B < 256, one table (W = T0[B], V = T0[2B]).
__global__ void __launch_bounds__(QFT_THREADS) k_qft_two_steps_small(double2* __restrict__ a, qidx numQuads, int tb,
                                                                     const __grid_constant__ QftTables T) {
    __shared__ long long sT[256][2];
    for (int e = threadIdx.x; e < 512; e += QFT_THREADS) (&sT[0][0])[e] = (&T.t[0][0][0])[e];
    __syncthreads();
    const qidx bMask = ((qidx)1 << (tb - 1)) - 1, half = (qidx)1 << (tb - 1), top = (qidx)1 << tb;
    const qidx stride = (qidx)gridDim.x * QFT_THREADS;
    for (qidx qd = blockIdx.x * (qidx)QFT_THREADS + threadIdx.x; qd < numQuads; qd += stride) {
        const int b = (int)(qd & bMask);
        const qidx i00 = ((qd & ~bMask) << 2) | (qidx)b;
        const double2 v00 = ld_amp(a + i00), v01 = ld_amp(a + i00 + half);
        const double2 v10 = ld_amp(a + i00 + top), v11 = ld_amp(a + i00 + top + half);
        const long long wr = sT[b][0], wi = sT[b][1], vr = sT[2 * b][0], vi = sT[2 * b][1];
        double2 y00, y01, y10, y11;
        qft_two_flies(v00, v01, v10, v11, wr, wi, vr, vi, y00, y01, y10, y11);
        st_amp(a + i00, y00);
        st_amp(a + i00 + half, y01);
        st_amp(a + i00 + top, y10);
        st_amp(a + i00 + top + half, y11);
    }
}

// Three steps in one pass, targets from qubit 0: the steps of T, T - 1 and T - 2 on the
// eight amplitudes a_pqr that differ in bits T (p), T - 1 (q) and T - 2 (r) only.  With B =
// their index bits below T - 2 and w = exp(i pi / 2^T):
//     step T:     pairs over p, twiddle w^(B + r 2^(T-2) + q 2^(T-1)) / sqrt2 = W omega^r i^q,
//                 W = w^B / sqrt2, omega = exp(i pi / 4)
//     step T - 1: pairs over q, twiddle exp(i pi (B + r 2^(T-2)) / 2^(T-1)) / sqrt2 = V i^r,
//                 V = w^(2B) / sqrt2
//     step T - 2: pairs over r, twiddle U = w^(4B) / sqrt2
// All from the tables of step T.  The first step's four pairs are converted at their own
// scales; their outputs are aligned to the largest and the next two steps run on integers
// at that one scale (each halving it twice: the outputs are converted with 2^(e - 1076)).
// An octet with a pair that needs FP64, or whose scale would leave no headroom for the
// double conversion at the end, takes twelve FP64 butterflies.
__device__ __noinline__ void qft_three_flies_fp64(double2* __restrict__ p, qidx quarter, long long w0r, long long w0i,
                                                  long long w1r, long long w1i, long long vr, long long vi, long long ur,
                                                  long long ui) {
    double2 v[8], x[8];
#pragma unroll
    for (int o = 0; o < 8; o++) v[o] = ld_amp(p + o * quarter);
#pragma unroll
    for (int qr = 0; qr < 4; qr++) {        // step T: pairs (0qr, 1qr), twiddle W omega^r i^q
        const int q = qr >> 1, r = qr & 1;
        const long long wr = r ? w1r : w0r, wi = r ? w1i : w0i;
        qft_butterfly(v[qr], v[4 + qr], q ? -wi : wr, q ? wr : wi, x[qr], x[4 + qr]);
    }
#pragma unroll
    for (int pr = 0; pr < 4; pr++) {        // step T - 1: pairs (p0r, p1r), twiddle V i^r
        const int pp = pr >> 1, r = pr & 1, o = 4 * pp + r;
        qft_butterfly(x[o], x[o + 2], r ? -vi : vr, r ? vr : vi, v[o], v[o + 2]);
    }
#pragma unroll
    for (int pq = 0; pq < 4; pq++) {        // step T - 2: pairs (pq0, pq1), twiddle U
        qft_butterfly(v[2 * pq], v[2 * pq + 1], ur, ui, x[2 * pq], x[2 * pq + 1]);
        st_amp(p + 2 * pq * quarter, x[2 * pq]);
        st_amp(p + (2 * pq + 1) * quarter, x[2 * pq + 1]);
    }
}

// The octet at p (amplitude o = 4p + 2q + r at p + o * quarter), its values already in v:
// the three steps in fixed point, written back; with twiddles W, W omega, V, U.  The
// octet's sixteen reals share one scale, the largest exponent among them (block floating
// point over the octet: each output's error is a few units of 2^-56 of the octet's largest
// |amplitude|), so they are converted once and every butterfly runs on integers.  An octet
// that needs FP64 (Inf/NaN, or scales near the ends of the range) goes to
// qft_three_flies_fp64, which reads it again.
__device__ __forceinline__ void qft_three_flies(double2* __restrict__ p, qidx quarter, const double2 (&v)[8], long long w0r,
                                                long long w0i, long long w1r, long long w1i, long long vr, long long vi,
                                                long long ur, long long ui) {
    int eb = 1;
    uint64_t any = 0;
#pragma unroll
    for (int o = 0; o < 8; o++) {
        const uint64_t ux = qgfx::f64_bits(v[o].x), uy = qgfx::f64_bits(v[o].y);
        const int ex = (int)((ux >> 52) & 0x7FF), ey = (int)((uy >> 52) & 0x7FF);
        eb = max(eb, max(ex + (ex == 0), ey + (ey == 0)));
        any |= (ux << 1) | (uy << 1);
    }
    if (any == 0) {
#pragma unroll
        for (int o = 0; o < 8; o++) st_amp(p + o * quarter, make_double2(0.0, 0.0));
        return;
    }
    if (eb < 58 || eb > 2040) {
        qft_three_flies_fp64(p, quarter, w0r, w0i, w1r, w1i, vr, vi, ur, ui);
        return;
    }
    // z[4p + 2q + r] (re, im), values x 2^(1082 - eb) below 2^60
    long long z[8][2];
#pragma unroll
    for (int o = 0; o < 8; o++) {
        z[o][0] = qft_fixed(qgfx::f64_bits(v[o].x), eb);
        z[o][1] = qft_fixed(qgfx::f64_bits(v[o].y), eb);
    }
#pragma unroll
    for (int qr = 0; qr < 4; qr++) {        // step T: pairs (0qr, 1qr), twiddle W omega^r i^q
        const int q = qr >> 1, r = qr & 1;
        const long long wr = r ? w1r : w0r, wi = r ? w1i : w0i;
        long long out[4];
        qft_fly_int(z[qr][0], z[qr][1], z[4 + qr][0], z[4 + qr][1], q ? -wi : wr, q ? wr : wi, out);
        z[qr][0] = out[0];
        z[qr][1] = out[1];
        z[4 + qr][0] = out[2];
        z[4 + qr][1] = out[3];
    }
#pragma unroll
    for (int pr = 0; pr < 4; pr++) {        // step T - 1: pairs (p0r, p1r), twiddle V i^r
        const int pp = pr >> 1, r = pr & 1, o = 4 * pp + r;
        long long out[4];
        qft_fly_int(z[o][0], z[o][1], z[o + 2][0], z[o + 2][1], r ? -vi : vr, r ? vr : vi, out);
        z[o][0] = out[0];
        z[o][1] = out[1];
        z[o + 2][0] = out[2];
        z[o + 2][1] = out[3];
    }
    const int t = eb - 1076;                 // value = z 2^(eb - 1076) after three steps (2^-2 each)
#pragma unroll
    for (int pq = 0; pq < 4; pq++) {        // step T - 2: pairs (pq0, pq1), twiddle U
        long long out[4];
        qft_fly_int(z[2 * pq][0], z[2 * pq][1], z[2 * pq + 1][0], z[2 * pq + 1][1], ur, ui, out);
        st_amp(p + 2 * pq * quarter, make_double2(qft_double(out[0], t), qft_double(out[1], t)));
        st_amp(p + (2 * pq + 1) * quarter, make_double2(qft_double(out[2], t), qft_double(out[3], t)));
    }
}

// T - 2 >= 8: a warp takes chunks of 256 consecutive octets (B's low byte b = 32 r + lane);
// the products of the higher tables are formed once per chunk, by seven lanes, into shared
// memory: for W (the bytes of B), for V (those of 2B: bit 8 from b's bit 7, two variants) and
// for U (those of 4B: bits 8-9 from b's bits 6-7, four variants).
template <int NT>
__global__ void __launch_bounds__(QFT_THREADS, 2) k_qft_three_steps_chunks(double2* __restrict__ a, qidx numChunks, int tb,
                                                                        const __grid_constant__ QftTables T) {
    static_assert(NT >= 2, "T - 2 >= 8 needs two tables");
    __shared__ long long sT[NT][256][2];
    __shared__ long long sH[QFT_THREADS / 32][8][2];        // per warp: HW, HV[2], HU[4] of its chunk
    for (int e = threadIdx.x; e < NT * 512; e += QFT_THREADS) (&sT[0][0][0])[e] = (&T.t[0][0][0])[e];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const qidx bMask = ((qidx)1 << (tb - 2)) - 1, quarter = (qidx)1 << (tb - 2);
    const qidx warps = (qidx)gridDim.x * (QFT_THREADS / 32);
    for (qidx c = blockIdx.x * (qidx)(QFT_THREADS / 32) + wid; c < numChunks; c += warps) {
        // lane k < 7 forms product k: 0 for W (the bytes of B), 1-2 for V (those of 2B, bit 8
        // = 0 or 1), 3-6 for U (those of 4B, bits 8-9 = 0..3); the low 8, 9 and 10 bits of B,
        // 2B and 4B are clear here
        if (lane < 7) {
            const qidx Bh = (c << 8) & bMask;
            const qidx X = lane == 0 ? Bh : lane < 3 ? Bh << 1 : Bh << 2;
            const int low = lane == 0 ? 0 : lane < 3 ? lane - 1 : lane - 3;
            const int j = (int)((X >> 8) & 255) | low;
            long long hr = sT[1][j][0], hi = sT[1][j][1];
#pragma unroll
            for (int k = 2; k < NT; k++) {
                const int jk = (int)((X >> (8 * k)) & 255);
                cmul62(hr, hi, sT[k][jk][0], sT[k][jk][1], hr, hi);
            }
            sH[wid][lane][0] = hr;
            sH[wid][lane][1] = hi;
        }
        __syncwarp();
#pragma unroll 1
        for (int r = 0; r < 8; r++) {
            const int b = 32 * r + lane;                        // B & 255
            const qidx oc = (c << 8) + b;
            const qidx i0 = ((oc & ~bMask) << 3) | (oc & bMask);
            double2 v[8];
#pragma unroll
            for (int o = 0; o < 8; o++) v[o] = ld_amp(a + i0 + o * quarter);
            long long w0r, w0i, w1r, w1i, vr, vi, ur, ui;
            const int hv = 1 + (r >> 2), hu = 3 + (r >> 1);    // b's bit 7; b's bits 6-7
            cmul62(sT[0][b][0], sT[0][b][1], sH[wid][0][0], sH[wid][0][1], w0r, w0i);
            cmul62(w0r, w0i, QFT_C, QFT_C, w1r, w1i);                                           // W omega
            cmul62(sT[0][(2 * b) & 255][0], sT[0][(2 * b) & 255][1], sH[wid][hv][0], sH[wid][hv][1], vr, vi);
            cmul62(sT[0][(4 * b) & 255][0], sT[0][(4 * b) & 255][1], sH[wid][hu][0], sH[wid][hu][1], ur, ui);
            qft_three_flies(a + i0, quarter, v, w0r, w0i, w1r, w1i, vr, vi, ur, ui);
        }
        __syncwarp();                                           // sH is rewritten for the next chunk
    }
}

// The same for 2 <= T <= 8: B < 64 and 4B < 256, one table (W = T0[B], V = T0[2B], U = T0[4B]).
__global__ void __launch_bounds__(QFT_THREADS, 2) k_qft_three_steps_small(double2* __restrict__ a, qidx numOctets, int tb,
                                                                       const __grid_constant__ QftTables T) {
    __shared__ long long sT[256][2];
    for (int e = threadIdx.x; e < 512; e += QFT_THREADS) (&sT[0][0])[e] = (&T.t[0][0][0])[e];
    __syncthreads();
    const qidx bMask = ((qidx)1 << (tb - 2)) - 1, quarter = (qidx)1 << (tb - 2);
    const qidx stride = (qidx)gridDim.x * QFT_THREADS;
    for (qidx oc = blockIdx.x * (qidx)QFT_THREADS + threadIdx.x; oc < numOctets; oc += stride) {
        const int b = (int)(oc & bMask);
        const qidx i0 = ((oc & ~bMask) << 3) | (qidx)b;
        double2 v[8];
#pragma unroll
        for (int o = 0; o < 8; o++) v[o] = ld_amp(a + i0 + o * quarter);
        long long w1r, w1i;
        cmul62(sT[b][0], sT[b][1], QFT_C, QFT_C, w1r, w1i);
        qft_three_flies(a + i0, quarter, v, sT[b][0], sT[b][1], w1r, w1i, sT[2 * b][0], sT[2 * b][1], sT[4 * b][0], sT[4 * b][1]);
    }
}

struct PhaseSet {
    long long t[4][256][2];     // table g, entry j: product of the factors 8g + k with bit k of j set, x 2^62
    qidx mask[32];              // the qubits of factor i (all must be 1)
};

// NT tables of 8 factors.  A warp takes chunks of 256 consecutive amplitudes (lane l, round
// r: amplitude 256 c + 32 r + l).  Whether factor f applies, (index & mask_f) == mask_f,
// splits into the bits above 8 (the same for the whole chunk: lane f tests them once per
// chunk and a ballot gathers the 32 answers) and the 8 low bits (fixed per lane and round:
// computed once per thread); their AND gives, byte g, the index into table g.
template <int NT>
__global__ void __launch_bounds__(QFT_THREADS) k_phase_set(double2* __restrict__ a, qidx numChunks, int num,
                                                           const __grid_constant__ PhaseSet P) {
    constexpr int numTables = NT;
    __shared__ long long sT[NT][256][2];
    for (int e = threadIdx.x; e < numTables * 512; e += QFT_THREADS) (&sT[0][0][0])[e] = (&P.t[0][0][0])[e];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const qidx myHigh = lane < num ? (P.mask[lane] & ~(qidx)255) : 0;     // lane f: factor f's bits above 8
    uint32_t low[8];                                                      // round r: the factors whose low bits hold
#pragma unroll
    for (int r = 0; r < 8; r++) {
        uint32_t w = 0;
        const int lo = 32 * r + lane;
        for (int f = 0; f < num; f++) {
            const int m = (int)(P.mask[f] & 255);
            if ((lo & m) == m) w |= 1u << f;
        }
        low[r] = w;
    }
    const qidx warps = (qidx)gridDim.x * (QFT_THREADS / 32);
    for (qidx c = blockIdx.x * (qidx)(QFT_THREADS / 32) + (threadIdx.x >> 5); c < numChunks; c += warps) {
        const qidx base = c << 8;
        const uint32_t high = __ballot_sync(0xffffffffu, lane < num && (base & myHigh) == myHigh);
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const uint32_t j4 = high & low[r];
            if (j4 == 0) continue;                   // every factor is 1 here: nothing to write
            const qidx i = base + 32 * r + lane;
            long long wr = sT[0][j4 & 255][0], wi = sT[0][j4 & 255][1];
#pragma unroll
            for (int g = 1; g < numTables; g++) {
                const uint32_t j = (j4 >> (8 * g)) & 255;
                cmul62(wr, wi, sT[g][j][0], sT[g][j][1], wr, wi);
            }
            const double2 v = ld_amp(a + i);
            const uint64_t u0 = qgfx::f64_bits(v.x), u1 = qgfx::f64_bits(v.y);
            const int e0 = (int)((u0 >> 52) & 0x7FF), e1 = (int)((u1 >> 52) & 0x7FF);
            const int eb = max(max(e0 + (e0 == 0), e1 + (e1 == 0)), 1);
            double2 o;
            if (((u0 | u1) << 1) == 0) {
                o = v;
            } else if (eb >= 58 && eb <= 2043) {
                const long long xr = qft_fixed(u0, eb), xi = qft_fixed(u1, eb);
                // value * 2^(1082 - eb) / 4
                const long long yr = mulhi(xr, wr) - mulhi(xi, wi), yi = mulhi(xr, wi) + mulhi(xi, wr);
                const int t = eb - 1080;
                o = make_double2(qft_double(yr, t), qft_double(yi, t));
            } else {
                const double cr = (double)wr * 0x1p-62, ci = (double)wi * 0x1p-62;
                o = make_double2(fma(v.x, cr, -v.y * ci), fma(v.x, ci, v.y * cr));
            }
            st_amp(a + i, o);
        }
    }
}

// the twiddle tables of a step with n low bits: table k, entry j = exp(i pi j 2^(8k) / 2^n)
// at scale 2^62, table 0 with 1/sqrt2; returns the number of tables (at least one)
static int qft_tables(int n, QftTables& T) {
    const int numTables = n <= 8 ? 1 : (n + 7) / 8;
    const long double PI = 3.141592653589793238462643383279502884L;
    for (int k = 0; k < numTables; k++)
        for (int j = 0; j < 256; j++) {
            const long double ang = PI * std::ldexp((long double)j, 8 * k - n);
            const long double sc = (k == 0 ? 1.0L / std::sqrt(2.0L) : 1.0L) * 4611686018427387904.0L;   // 2^62
            T.t[k][j][0] = (long long)std::llroundl(std::cos(ang) * sc);
            T.t[k][j][1] = (long long)std::llroundl(std::sin(ang) * sc);
        }
    return numTables;
}

// The closing swaps of a QFT on qubits 0..n-1 (n >= 10) as one in-place permutation: index
// bits [0, n) reversed.  The index splits into o (bits above n), h (bits n-5..n-1), m (the
// n - 10 middle bits) and l (bits 0..4); (o, h, m, l) goes to (o, rev5 l, rev m, rev5 h).  So
// the 32 x 32 tile of (o, m) goes, transposed and with both 5-bit fields reversed, to the
// tile of (o, rev m): a block reads a tile and its partner (one tile when m = rev m) into
// shared memory -- rows of 32 consecutive amplitudes, 512 bytes -- and then writes both,
// again in rows of 512 bytes.  Every tile belongs to one block, so nothing else reads or
// writes it meanwhile.  In shared memory, element (h, l) sits in column l ^ (rev5(h) & 7):
// the eight lanes of a 16-byte access phase then hit eight distinct bank groups both when a
// row is written (l = the lane) and when a column is read back (h = rev5 of the lane).
#define REV_THREADS 256
__global__ void __launch_bounds__(REV_THREADS, 6) k_reverse_low_bits(double2* __restrict__ a, qidx numTiles, int n) {
    __shared__ double2 s[2][32][32];
    const int midBits = n - 10;
    const int lane = threadIdx.x & 31, row0 = threadIdx.x >> 5;
    const int rl = (int)(__brev((unsigned)lane) >> 27);               // rev5(lane)
    const qidx rowStride = (qidx)1 << (n - 5);
    for (qidx tile = blockIdx.x; tile < numTiles; tile += gridDim.x) {
        const qidx o = tile >> midBits, m = tile & (((qidx)1 << midBits) - 1);
        const qidx rm = midBits ? (qidx)(__brevll((unsigned long long)m) >> (64 - midBits)) : 0;
        if (rm < m) continue;                                            // the partner's tile does this pair
        const bool two = rm != m;
        const qidx baseM = (o << n) | (m << 5), baseR = (o << n) | (rm << 5);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int h = row0 + 8 * k;
            const int col = lane ^ (int)((__brev((unsigned)h) >> 27) & 7);
            s[0][h][col] = ld_amp(a + baseM + h * rowStride + lane);
            if (two) s[1][h][col] = ld_amp(a + baseR + h * rowStride + lane);
        }
        __syncthreads();
        // destination row r (= rev5 of the source's l), column lane (= rev5 of its h)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = row0 + 8 * k;
            const int sl = (int)(__brev((unsigned)r) >> 27);
            const int col = sl ^ (lane & 7);                             // rev5(rl) & 7 = lane & 7
            st_amp(a + baseR + r * rowStride + lane, s[0][rl][col]);
            if (two) st_amp(a + baseM + r * rowStride + lane, s[1][rl][col]);
        }
        __syncthreads();
    }
}

extern "C" {

// Reverses the low numBits bits of every amplitude index (the closing swaps of a QFT on
// qubits 0..numBits-1), in place, in one pass.
int qg_sv_reverseLowBits(void* amps, int numQubits, int numBits, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (numBits < 10 || numBits > numQubits)
        return qg_fail(QG_ERR_ARG, "reverseLowBits: %d bits of a %d-qubit register (10 <= bits <= qubits)", numBits, numQubits);
    const qidx numTiles = (qidx)1 << (numQubits - 10);
    int perSm = 0;
    QG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_reverse_low_bits, REV_THREADS, 0));
    const unsigned grid = (unsigned)std::min<qidx>(numTiles, (qidx)qg_num_sms() * std::max(1, perSm));
    k_reverse_low_bits<<<grid, REV_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numTiles, numBits);
    qg_note_launch();
    return qg_check_launch("k_reverse_low_bits");
}

// A set of controlled phases on a statevector: every amplitude whose index contains
// masks[f] (all those bits 1) is multiplied by factors[f], for each f < num (num <= 32;
// each |factors[f]| = 1).  The phases commute, so their order does not matter.
int qg_sv_phaseSet(void* amps, int numQubits, const int64_t* masks, const qg_cplx* factors, int num, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (num < 0 || num > 32 || (num > 0 && (!masks || !factors)))
        return qg_fail(QG_ERR_ARG, "phaseSet: %d phases (at most 32)", num);
    if (num == 0) return QG_OK;
    PhaseSet P;
    const qidx all = ((qidx)1 << numQubits) - 1;
    for (int f = 0; f < num; f++) {
        if (masks[f] <= 0 || (masks[f] & ~all) != 0) return qg_fail(QG_ERR_ARG, "phaseSet: mask %lld", (long long)masks[f]);
        const double m = std::hypot(factors[f].re, factors[f].im);
        if (!(std::fabs(m - 1.0) < 1e-6)) return qg_fail(QG_ERR_ARG, "phaseSet: a factor of modulus %g (must be 1)", m);
        P.mask[f] = masks[f];
    }
    for (int f = num; f < 32; f++) P.mask[f] = 0;
    const int numTables = (num + 7) / 8;
    for (int g = 0; g < numTables; g++)
        for (int j = 0; j < 256; j++) {
            std::complex<long double> prod(1.0L, 0.0L);
            for (int k = 0; k < 8; k++)
                if ((j >> k) & 1 && 8 * g + k < num)
                    prod *= std::complex<long double>(factors[8 * g + k].re, factors[8 * g + k].im);
            P.t[g][j][0] = (long long)std::llroundl(prod.real() * 4611686018427387904.0L);
            P.t[g][j][1] = (long long)std::llroundl(prod.imag() * 4611686018427387904.0L);
        }
    if (numQubits < 8) return qg_fail(QG_ERR_ARG, "phaseSet: at least 8 qubits (chunks of 256 amplitudes)");
    const qidx numChunks = ((qidx)1 << numQubits) >> 8;
    const unsigned grid = (unsigned)std::min<qidx>((numChunks + QFT_THREADS / 32 - 1) / (QFT_THREADS / 32), (qidx)qg_num_sms() * 8);
    double2* A = (double2*)amps;
    cudaStream_t st = qg_stream(stream);
    switch (numTables) {
        case 1: k_phase_set<1><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, num, P); break;
        case 2: k_phase_set<2><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, num, P); break;
        case 3: k_phase_set<3><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, num, P); break;
        default: k_phase_set<4><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, num, P); break;
    }
    qg_note_launch();
    return qg_check_launch("k_phase_set");
}

// One QFT step on a statevector: Hadamard on `target`, then for every amplitude whose bit
// `target` is set the phase exp(i pi L / 2^numLowBits), L = (index >> lowTarget) &
// (2^numLowBits - 1), with lowTarget + numLowBits == target (the step of
// applyQuantumFourierTransform on the contiguous targets lowTarget..target).
int qg_sv_qftStep(void* amps, int numQubits, int target, int lowTarget, int numLowBits, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (target < 0 || target >= numQubits || lowTarget < 0 || numLowBits < 0 || lowTarget + numLowBits != target ||
        numLowBits > 8 * QFT_MAX_TABLES)
        return qg_fail(QG_ERR_ARG, "qftStep: target %d, low target %d, %d low bits", target, lowTarget, numLowBits);
    QftTables T;
    const int numTables = qft_tables(numLowBits, T);
    const qidx numPairs = (qidx)1 << (numQubits - 1);
    const qidx lmask = numLowBits >= 63 ? -1 : (((qidx)1 << numLowBits) - 1);
    const unsigned grid = (unsigned)std::min<qidx>((numPairs + QFT_THREADS - 1) / QFT_THREADS, (qidx)qg_num_sms() * 8);
    double2* A = (double2*)amps;
    cudaStream_t st = qg_stream(stream);
    if (lowTarget == 0 && target >= 8 && numTables >= 3) {
        const qidx numChunks = numPairs >> 8;
        const unsigned g2 = (unsigned)std::min<qidx>((numChunks + QFT_THREADS / 32 - 1) / (QFT_THREADS / 32), (qidx)qg_num_sms() * 8);
        if (numTables == 3) k_qft_step_chunks<3><<<g2, QFT_THREADS, 0, st>>>(A, numChunks, target, lmask, T);
        else if (numTables == 4) k_qft_step_chunks<4><<<g2, QFT_THREADS, 0, st>>>(A, numChunks, target, lmask, T);
        else k_qft_step_chunks<5><<<g2, QFT_THREADS, 0, st>>>(A, numChunks, target, lmask, T);
        qg_note_launch();
        return qg_check_launch("k_qft_step_chunks");
    }
    switch (numTables) {
        case 1: k_qft_step<1><<<grid, QFT_THREADS, 0, st>>>(A, numPairs, target, lowTarget, lmask, T); break;
        case 2: k_qft_step<2><<<grid, QFT_THREADS, 0, st>>>(A, numPairs, target, lowTarget, lmask, T); break;
        case 3: k_qft_step<3><<<grid, QFT_THREADS, 0, st>>>(A, numPairs, target, lowTarget, lmask, T); break;
        case 4: k_qft_step<4><<<grid, QFT_THREADS, 0, st>>>(A, numPairs, target, lowTarget, lmask, T); break;
        default: k_qft_step<5><<<grid, QFT_THREADS, 0, st>>>(A, numPairs, target, lowTarget, lmask, T); break;
    }
    qg_note_launch();
    return qg_check_launch("k_qft_step");
}

// The QFT steps of targets `target` and then `target` - 1 on the contiguous targets from
// qubit 0 (qg_sv_qftStep(target, 0, target), then qg_sv_qftStep(target - 1, 0, target - 1))
// in one pass.
int qg_sv_qftTwoSteps(void* amps, int numQubits, int target, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (target < 1 || target >= numQubits || target > 8 * QFT_MAX_TABLES)
        return qg_fail(QG_ERR_ARG, "qftTwoSteps: target %d of %d qubits", target, numQubits);
    QftTables T;
    const int numTables = qft_tables(target, T);
    const qidx numQuads = (qidx)1 << (numQubits - 2);
    double2* A = (double2*)amps;
    cudaStream_t st = qg_stream(stream);
    if (target <= 8) {
        const unsigned grid = (unsigned)std::min<qidx>((numQuads + QFT_THREADS - 1) / QFT_THREADS, (qidx)qg_num_sms() * 8);
        k_qft_two_steps_small<<<grid, QFT_THREADS, 0, st>>>(A, numQuads, target, T);
        qg_note_launch();
        return qg_check_launch("k_qft_two_steps_small");
    }
    const qidx numChunks = numQuads >> 8;
    const unsigned grid = (unsigned)std::min<qidx>((numChunks + QFT_THREADS / 32 - 1) / (QFT_THREADS / 32), (qidx)qg_num_sms() * 8);
    switch (numTables) {
        case 2: k_qft_two_steps_chunks<2><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
        case 3: k_qft_two_steps_chunks<3><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
        case 4: k_qft_two_steps_chunks<4><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
        default: k_qft_two_steps_chunks<5><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
    }
    qg_note_launch();
    return qg_check_launch("k_qft_two_steps_chunks");
}

// The QFT steps of `target`, `target` - 1 and `target` - 2 on the contiguous targets from
// qubit 0 in one pass: 2 <= target <= 8 or 10 <= target <= 40.
int qg_sv_qftThreeSteps(void* amps, int numQubits, int target, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (target < 2 || target >= numQubits || target == 9 || target > 8 * QFT_MAX_TABLES)
        return qg_fail(QG_ERR_ARG, "qftThreeSteps: target %d of %d qubits (2..8 or 10..40)", target, numQubits);
    QftTables T;
    const int numTables = qft_tables(target, T);
    const qidx numOctets = (qidx)1 << (numQubits - 3);
    double2* A = (double2*)amps;
    cudaStream_t st = qg_stream(stream);
    if (target <= 8) {
        const unsigned grid = (unsigned)std::min<qidx>((numOctets + QFT_THREADS - 1) / QFT_THREADS, (qidx)qg_num_sms() * 8);
        k_qft_three_steps_small<<<grid, QFT_THREADS, 0, st>>>(A, numOctets, target, T);
        qg_note_launch();
        return qg_check_launch("k_qft_three_steps_small");
    }
    const qidx numChunks = numOctets >> 8;
    const unsigned grid = (unsigned)std::min<qidx>((numChunks + QFT_THREADS / 32 - 1) / (QFT_THREADS / 32), (qidx)qg_num_sms() * 8);
    switch (numTables) {
        case 2: k_qft_three_steps_chunks<2><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
        case 3: k_qft_three_steps_chunks<3><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
        case 4: k_qft_three_steps_chunks<4><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
        default: k_qft_three_steps_chunks<5><<<grid, QFT_THREADS, 0, st>>>(A, numChunks, target, T); break;
    }
    qg_note_launch();
    return qg_check_launch("k_qft_three_steps_chunks");
}

}  // extern "C"
