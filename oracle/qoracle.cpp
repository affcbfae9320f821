/*
 * qoracle.cpp -- CPU oracle (TEST INFRASTRUCTURE ONLY; see qoracle.h).
 *
 * Each routine restates the algorithm of the named QuEST v4.1.0 function on a
 * single, non-distributed node (rank 0, every qubit in the "suffix"), so the
 * prefix/communication branches of the reference do not arise.  Loops are
 * OpenMP-parallel like the reference's CPU backend, so the same code serves as
 * the timed CPU baseline.  Arithmetic is std::complex<double>, as qcomp is at
 * FLOAT_PRECISION=2 (quest/include/precision.h:43-107).
 */
#include "qoracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cplx;
typedef long long idx;
using std::vector;

/* ------------------------------------------------------------------------ */
/* bit helpers: quest/src/core/bitwise.hpp:84-215                            */
/* ------------------------------------------------------------------------ */

static inline idx pow2(int k) { return ((idx)1) << k; }
static inline int getBit(idx n, int b) { return (int)((n >> b) & 1); }
static inline idx flipBit(idx n, int b) { return n ^ pow2(b); }

/* insertBit: bitwise.hpp:99-105 -- open a gap at bitIndex holding bitValue */
static inline idx insertBit(idx n, int b, int v) {
    idx low = n & (pow2(b) - 1);
    idx high = (n >> b) << (b + 1);
    return high | ((idx)v << b) | low;
}
/* insertBits with strictly increasing indices: bitwise.hpp:164-171 */
static inline idx insertZeroBits(idx n, const int* sorted, int k) {
    for (int i = 0; i < k; i++) n = insertBit(n, sorted[i], 0);
    return n;
}
/* setBits: bitwise.hpp:174-183 */
static inline idx setBits(idx n, const int* inds, int k, idx value) {
    for (int i = 0; i < k; i++) {
        idx one = pow2(inds[i]);
        n = getBit(value, i) ? (n | one) : (n & ~one);
    }
    return n;
}
/* getValueOfBits: bitwise.hpp:186-195 */
static inline idx getValueOfBits(idx n, const int* inds, int k) {
    idx v = 0;
    for (int i = 0; i < k; i++) v |= ((idx)getBit(n, inds[i])) << i;
    return v;
}
static inline int parity(idx n) { return __builtin_parityll((unsigned long long)n); }
/* fast_getPlusOrMinusMaskedBitParity: fastmath.hpp:52-58 */
static inline int signOfParity(idx n, idx mask) { return 1 - 2 * parity(n & mask); }

static idx maskOf(const int* q, int n) { idx m = 0; for (int i = 0; i < n; i++) m |= pow2(q[i]); return m; }

/* util_getSorted(ctrls, targs) + util_getBitMask(ctrls, states, targs, targStates):
 * quest/src/core/utilities.cpp (qubit-list helpers). Missing states default to 1
 * (setDefaultCtrlStates, localiser.cpp:58-67). */
struct QubitSet {
    vector<int> sorted;
    idx stateMask = 0;
};
static QubitSet makeSet(const int* ctrls, const int* states, int nc, const int* targs, const int* targStates, int nt) {
    QubitSet s;
    for (int i = 0; i < nc; i++) {
        s.sorted.push_back(ctrls[i]);
        int st = states ? states[i] : 1;
        if (st) s.stateMask |= pow2(ctrls[i]);
    }
    for (int i = 0; i < nt; i++) {
        s.sorted.push_back(targs[i]);
        if (targStates && targStates[i]) s.stateMask |= pow2(targs[i]);
    }
    std::sort(s.sorted.begin(), s.sorted.end());
    return s;
}
/* insertBitsWithMaskedValues: bitwise.hpp:206-210 */
static inline idx insertWithMask(idx n, const QubitSet& s) {
    return s.stateMask | insertZeroBits(n, s.sorted.data(), (int)s.sorted.size());
}

/* The reference unrolls insertBits at compile time for up to five bits
 * (SET_VAR_AT_COMPILE_TIME with the NumCtrls template parameter, cpu_subroutines.cpp);
 * the same here, so that the port runs as fast as the reference's CPU build. */
struct FixedSet {
    int num;
    int sorted[64];
    idx mask;
    explicit FixedSet(const QubitSet& s) : num((int)s.sorted.size()), mask(s.stateMask) {
        for (int i = 0; i < num; i++) sorted[i] = s.sorted[i];
    }
};
template <int K>
static inline idx insertK(idx n, const FixedSet& f) {
    if (K >= 0) {
        for (int i = 0; i < (K >= 0 ? K : 0); i++) n = insertBit(n, f.sorted[i], 0);
    } else {
        for (int i = 0; i < f.num; i++) n = insertBit(n, f.sorted[i], 0);
    }
    return n | f.mask;
}
#define ORC_DISPATCH_K(num, ...)                          \
    switch (num) {                                        \
        case 0: { constexpr int K = 0; __VA_ARGS__ } break;  \
        case 1: { constexpr int K = 1; __VA_ARGS__ } break;  \
        case 2: { constexpr int K = 2; __VA_ARGS__ } break;  \
        case 3: { constexpr int K = 3; __VA_ARGS__ } break;  \
        case 4: { constexpr int K = 4; __VA_ARGS__ } break;  \
        case 5: { constexpr int K = 5; __VA_ARGS__ } break;  \
        default: { constexpr int K = -1; __VA_ARGS__ } break; \
    }
#define ORC_PARALLEL_FOR _Pragma("omp parallel for num_threads(orc_get_num_threads())")

static inline cplx* C(double* a) { return reinterpret_cast<cplx*>(a); }
static inline const cplx* C(const double* a) { return reinterpret_cast<const cplx*>(a); }

static int g_threads = 0;
extern "C" void orc_set_num_threads(int n) { g_threads = n; }
extern "C" int orc_get_num_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#define NT num_threads(orc_get_num_threads())

/* ------------------------------------------------------------------------ */
/* statevector subroutines                                                   */
/* ------------------------------------------------------------------------ */

/* cpu_statevec_anyCtrlSwap_subA: cpu_subroutines.cpp:255-280 (targ1 < targ2 after
 * localiser_statevec_anyCtrlSwap, localiser.cpp:872-897) */
extern "C" void orc_sv_swap(double* amps, int nq, const int* ctrls, const int* states, int nc, int t1, int t2) {
    if (t1 > t2) std::swap(t1, t2);
    int targs[2] = {t2, t1}, ts[2] = {0, 1};
    FixedSet f(makeSet(ctrls, states, nc, targs, ts, 2));
    idx numIts = pow2(nq) >> (nc + 2);
    cplx* a = C(amps);
    ORC_DISPATCH_K(f.num,
        ORC_PARALLEL_FOR
        for (idx n = 0; n < numIts; n++) {
            idx i01 = insertK<K>(n, f);
            idx i10 = flipBit(flipBit(i01, t2), t1);
            std::swap(a[i01], a[i10]);
        })
}

/* cpu_statevec_anyCtrlOneTargDenseMatr_subA: cpu_subroutines.cpp:355-383 */
extern "C" void orc_sv_dense1(double* amps, int nq, const int* ctrls, const int* states, int nc, int t, const double* mm) {
    const cplx* m = C(mm);
    int ts = 0;
    FixedSet f(makeSet(ctrls, states, nc, &t, &ts, 1));
    idx numIts = pow2(nq) >> (nc + 1);
    cplx* a = C(amps);
    const cplx m0 = m[0], m1 = m[1], m2 = m[2], m3 = m[3];
    ORC_DISPATCH_K(f.num,
        ORC_PARALLEL_FOR
        for (idx n = 0; n < numIts; n++) {
            idx i0 = insertK<K>(n, f);
            idx i1 = flipBit(i0, t);
            cplx a0 = a[i0], a1 = a[i1];
            a[i0] = m0 * a0 + m1 * a1;
            a[i1] = m2 * a0 + m3 * a1;
        })
}

/* cpu_statevec_anyCtrlTwoTargDenseMatr_sub: cpu_subroutines.cpp:433-470 */
extern "C" void orc_sv_dense2(double* amps, int nq, const int* ctrls, const int* states, int nc, int t1, int t2, const double* mm) {
    const cplx* m = C(mm);
    int targs[2] = {t1, t2}, ts[2] = {0, 0};
    QubitSet s = makeSet(ctrls, states, nc, targs, ts, 2);
    idx numIts = pow2(nq) >> (nc + 2);
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx i00 = insertWithMask(n, s);
        idx i01 = flipBit(i00, t1), i10 = flipBit(i00, t2), i11 = flipBit(i01, t2);
        cplx v[4] = {a[i00], a[i01], a[i10], a[i11]};
        idx ii[4] = {i00, i01, i10, i11};
        for (int r = 0; r < 4; r++)
            a[ii[r]] = m[4*r+0]*v[0] + m[4*r+1]*v[1] + m[4*r+2]*v[2] + m[4*r+3]*v[3];
    }
}

/* cpu_statevec_anyCtrlAnyTargDenseMatr_sub: cpu_subroutines.cpp:482-569.
 * Targets keep their given order: matrix index bit i is targs[i]. */
extern "C" void orc_sv_denseK(double* amps, int nq, const int* ctrls, const int* states, int nc, const int* targs, int nt, const double* mm, int conj) {
    const cplx* m = C(mm);
    vector<int> zeros(nt, 0);
    QubitSet s = makeSet(ctrls, states, nc, targs, zeros.data(), nt);
    idx numIts = pow2(nq) >> (nc + nt);
    idx dim = pow2(nt);
    cplx* a = C(amps);
    #pragma omp parallel NT
    {
        vector<cplx> cache(dim);
        #pragma omp for
        for (idx n = 0; n < numIts; n++) {
            idx i0 = insertWithMask(n, s);
            for (idx j = 0; j < dim; j++) cache[j] = a[setBits(i0, targs, nt, j)];
            for (idx k = 0; k < dim; k++) {
                idx i = setBits(i0, targs, nt, k);
                cplx acc = 0;
                for (idx j = 0; j < dim; j++) {
                    cplx e = m[k * dim + j];
                    if (conj) e = std::conj(e);
                    acc += e * cache[j];
                }
                a[i] = acc;
            }
        }
    }
}

/* cpu_statevec_anyCtrlOneTargDiagMatr_sub: cpu_subroutines.cpp:581-610 */
extern "C" void orc_sv_diag1(double* amps, int nq, const int* ctrls, const int* states, int nc, int t, const double* dd) {
    const cplx* d = C(dd);
    FixedSet f(makeSet(ctrls, states, nc, nullptr, nullptr, 0));
    idx numIts = pow2(nq) >> nc;
    cplx* a = C(amps);
    const cplx d2[2] = {d[0], d[1]};
    ORC_DISPATCH_K(f.num,
        ORC_PARALLEL_FOR
        for (idx n = 0; n < numIts; n++) {
            idx j = insertK<K>(n, f);
            a[j] *= d2[getBit(j, t)];
        })
}

/* cpu_statevec_anyCtrlTwoTargDiagMatr_sub: cpu_subroutines.cpp:622-651 (k = bit t2 bit t1) */
extern "C" void orc_sv_diag2(double* amps, int nq, const int* ctrls, const int* states, int nc, int t1, int t2, const double* dd) {
    const cplx* d = C(dd);
    QubitSet s = makeSet(ctrls, states, nc, nullptr, nullptr, 0);
    idx numIts = pow2(nq) >> nc;
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx j = insertWithMask(n, s);
        int k = (getBit(j, t2) << 1) | getBit(j, t1);
        a[j] *= d[k];
    }
}

/* cpu_statevec_anyCtrlAnyTargDiagMatr_sub: cpu_subroutines.cpp:663-701
 * (std::pow(qcomp,qcomp) when an exponent is given; conj after the power) */
extern "C" void orc_sv_diagK(double* amps, int nq, const int* ctrls, const int* states, int nc, const int* targs, int nt, const double* dd, int conj, const double* exponent) {
    const cplx* d = C(dd);
    QubitSet s = makeSet(ctrls, states, nc, nullptr, nullptr, 0);
    idx numIts = pow2(nq) >> nc;
    cplx* a = C(amps);
    cplx ex = exponent ? cplx(exponent[0], exponent[1]) : cplx(1, 0);
    bool hasPower = exponent && ex != cplx(1, 0);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx j = insertWithMask(n, s);
        cplx e = d[getValueOfBits(j, targs, nt)];
        if (hasPower) e = std::pow(e, ex);
        if (conj) e = std::conj(e);
        a[j] *= e;
    }
}

/* cpu_statevec_allTargDiagMatr_sub: cpu_subroutines.cpp:713-738
 * (a_n *= d_n, or d_n^p with std::pow(qcomp,qcomp) when an exponent is given) */
extern "C" void orc_sv_allTargDiag(double* amps, int nq, const double* elems, const double* exponent) {
    const cplx* d = C(elems);
    cplx* a = C(amps);
    cplx ex = exponent ? cplx(exponent[0], exponent[1]) : cplx(1, 0);
    bool hasPower = exponent && ex != cplx(1, 0);
    idx numIts = pow2(nq);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        cplx e = d[n];
        if (hasPower) e = std::pow(e, ex);
        a[n] *= e;
    }
}

/* cpu_densmatr_allTargDiagMatr_sub: cpu_subroutines.cpp:740-784
 * (rho[r][c] *= d_r^p, and unless multiplyOnly also *= conj(d_c^p); flat n = c*dim + r) */
extern "C" void orc_dm_allTargDiag(double* amps, int nKet, const double* elems, const double* exponent, int multiplyOnly) {
    const cplx* d = C(elems);
    cplx* a = C(amps);
    cplx ex = exponent ? cplx(exponent[0], exponent[1]) : cplx(1, 0);
    bool hasPower = exponent && ex != cplx(1, 0);
    idx dim = pow2(nKet), numIts = dim * dim;
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        cplx fac = d[n % dim];
        if (hasPower) fac = std::pow(fac, ex);
        if (!multiplyOnly) {
            cplx term = d[n / dim];
            if (hasPower) term = std::pow(term, ex);
            fac *= std::conj(term);
        }
        a[n] *= fac;
    }
}

/* the diagonal element raised as the expectation routines do: cpu_subroutines.cpp:2194-2200 */
static cplx expecElem(cplx e, cplx ex, bool hasPower, bool useRealPow) {
    if (hasPower && !useRealPow) return std::pow(e, ex);
    if (hasPower && useRealPow) return cplx(std::pow(std::real(e), std::real(ex)), 0);
    return e;
}

/* cpu_statevec_calcExpecFullStateDiagMatr_sub: cpu_subroutines.cpp:2175-2212
 * (sum_n d_n^p |a_n|^2; hasPower iff the exponent differs from 1, accelerator.cpp:1020-1021) */
extern "C" void orc_sv_expecAllTargDiag(double* out, const double* amps, int nq, const double* elems, const double* exponent, int useRealPow) {
    const cplx* d = C(elems);
    const cplx* a = C(amps);
    cplx ex = exponent ? cplx(exponent[0], exponent[1]) : cplx(1, 0);
    bool hasPower = ex != cplx(1, 0);
    bool realPow = useRealPow && hasPower;
    double re = 0, im = 0;
    idx numIts = pow2(nq);
    #pragma omp parallel for reduction(+:re,im) NT
    for (idx n = 0; n < numIts; n++) {
        cplx t = expecElem(d[n], ex, hasPower, realPow) * std::norm(a[n]);
        re += std::real(t);
        im += std::imag(t);
    }
    out[0] = re;
    out[1] = im;
}

/* cpu_densmatr_calcExpecFullStateDiagMatr_sub: cpu_subroutines.cpp:2215-2258 (sum_r d_r^p rho[r][r]) */
extern "C" void orc_dm_expecAllTargDiag(double* out, const double* amps, int nKet, const double* elems, const double* exponent, int useRealPow) {
    const cplx* d = C(elems);
    const cplx* a = C(amps);
    cplx ex = exponent ? cplx(exponent[0], exponent[1]) : cplx(1, 0);
    bool hasPower = ex != cplx(1, 0);
    bool realPow = useRealPow && hasPower;
    double re = 0, im = 0;
    idx dim = pow2(nKet);
    #pragma omp parallel for reduction(+:re,im) NT
    for (idx n = 0; n < dim; n++) {
        cplx t = expecElem(d[n], ex, hasPower, realPow) * a[n * (dim + 1)];
        re += std::real(t);
        im += std::imag(t);
    }
    out[0] = re;
    out[1] = im;
}

/* cpu_statevector_anyCtrlPauliTensorOrGadget_subA + applyPauliUponAmpPair:
 * cpu_subroutines.cpp:802-906 */
extern "C" void orc_sv_pauliTensorOrGadget(double* amps, int nq, const int* ctrls, const int* states, int nc,
                                           const int* x, int nx, const int* y, int ny, const int* z, int nz,
                                           const double* ampFacP, const double* pairFacP) {
    vector<int> xy(x, x + nx);
    xy.insert(xy.end(), y, y + ny);
    std::sort(xy.begin(), xy.end());
    int nxy = (int)xy.size();
    vector<int> zeros(nxy, 0);
    QubitSet s = makeSet(ctrls, states, nc, xy.data(), zeros.data(), nxy);
    idx maskXY = maskOf(xy.data(), nxy);
    idx maskYZ = maskOf(y, ny) | maskOf(z, nz);
    cplx ampFac(ampFacP[0], ampFacP[1]);
    static const cplx powI[4] = {cplx(1, 0), cplx(0, 1), cplx(-1, 0), cplx(0, -1)}; /* util_getPowerOfI, utilities.cpp:333-338 */
    cplx pairFac = cplx(pairFacP[0], pairFacP[1]) * powI[ny % 4];
    idx numOuter = pow2(nq) >> (nc + nxy);
    idx numInner = pow2(nxy) / 2;
    cplx* a = C(amps);
    #pragma omp parallel for NT collapse(2)
    for (idx n = 0; n < numOuter; n++) {
        for (idx v = 0; v < numInner; v++) {
            idx i0 = insertWithMask(n, s);
            idx iA = setBits(i0, xy.data(), nxy, v);
            idx iB = iA ^ maskXY;
            int signA = signOfParity(iA, maskYZ), signB = signOfParity(iB, maskYZ);
            cplx aA = a[iA], aB = a[iB];
            a[iA] = (ampFac * aA) + (pairFac * (double)signB * aB);
            a[iB] = (ampFac * aB) + (pairFac * (double)signA * aA);
        }
    }
}

/* cpu_statevector_anyCtrlAnyTargZOrPhaseGadget_sub: cpu_subroutines.cpp:962-990 */
extern "C" void orc_sv_zOrPhaseGadget(double* amps, int nq, const int* ctrls, const int* states, int nc, const int* targs, int nt, const double* f0, const double* f1) {
    cplx facs[2] = {cplx(f0[0], f0[1]), cplx(f1[0], f1[1])};
    QubitSet s = makeSet(ctrls, states, nc, nullptr, nullptr, 0);
    idx tmask = maskOf(targs, nt);
    idx numIts = pow2(nq) >> nc;
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx i = insertWithMask(n, s);
        a[i] *= facs[parity(i & tmask)];
    }
}

/* cpu_statevec_multiQubitProjector_sub: cpu_subroutines.cpp:2281-2306 */
extern "C" void orc_sv_projector(double* amps, int nq, const int* qubits, const int* outcomes, int n, double prob) {
    double renorm = 1 / std::sqrt(prob);
    idx retain = 0;
    for (int i = 0; i < n; i++) retain |= ((idx)outcomes[i]) << i;
    cplx* a = C(amps);
    idx numIts = pow2(nq);
    #pragma omp parallel for NT
    for (idx k = 0; k < numIts; k++) {
        idx v = getValueOfBits(k, qubits, n);
        cplx fac = renorm * (double)(v == retain);
        a[k] *= fac;
    }
}

/* ------------------------------------------------------------------------ */
/* density-matrix subroutines (bra qubit = ket qubit + nKet, utilities.cpp:50-55) */
/* ------------------------------------------------------------------------ */

/* insertTwoBits(n, hi, bhi, lo, blo) for hi > lo (bitwise.hpp) */
static inline idx insertTwo(idx n, int hi, int bhi, int lo, int blo) {
    return insertBit(insertBit(n, lo, blo), hi, bhi);
}

/* cpu_densmatr_oneQubitDepolarising_subA: cpu_subroutines.cpp:1183-1215;
 * factors util_getOneQubitDepolarisingFactors: utilities.cpp:932-947 */
extern "C" void orc_dm_depolarising1(double* amps, int nKet, int ket, double prob) {
    int bra = ket + nKet;
    double facAA = 1 - (2 * prob / 3), facBB = 2 * prob / 3, facAB = 1 - (4 * prob / 3);
    idx numIts = pow2(2 * nKet) / 4;
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx i00 = insertTwo(n, bra, 0, ket, 0);
        idx i01 = flipBit(i00, ket), i10 = flipBit(i00, bra), i11 = flipBit(i01, bra);
        cplx a00 = a[i00], a11 = a[i11];
        a[i00] = (facAA * a00) + (facBB * a11);
        a[i01] *= facAB;
        a[i10] *= facAB;
        a[i11] = (facAA * a11) + (facBB * a00);
    }
}

/* localiser_densmatr_twoQubitDepolarising (localiser.cpp:1535-1556) with
 * cpu_densmatr_twoQubitDepolarising_subA/subB (cpu_subroutines.cpp:1262-1325);
 * factors utilities.cpp:949-960 */
extern "C" void orc_dm_depolarising2(double* amps, int nKet, int q1, int q2, double prob) {
    if (q1 > q2) std::swap(q1, q2);
    int b1 = q1 + nKet, b2 = q2 + nKet;
    double c1 = 1 - (4 * prob / 5), c2 = 4 * prob / 15, c3 = -(16 * prob / 15);
    cplx* a = C(amps);
    idx N = pow2(2 * nKet);
    #pragma omp parallel for NT
    for (idx n = 0; n < N; n++) {
        bool f1 = getBit(n, q1) == getBit(n, b1);
        bool f2 = getBit(n, q2) == getBit(n, b2);
        bool mod = !(f1 & f2);
        a[n] *= 1 + c3 * mod;
    }
    c1 -= c2;
    int srt[4] = {q1, q2, b1, b2};
    std::sort(srt, srt + 4);
    #pragma omp parallel for NT
    for (idx n = 0; n < N / 16; n++) {
        idx i0000 = insertZeroBits(n, srt, 4);
        idx i0101 = flipBit(flipBit(i0000, b1), q1);
        idx i1010 = flipBit(flipBit(i0000, b2), q2);
        idx i1111 = flipBit(flipBit(i0101, b2), q2);
        cplx term = a[i0000] + a[i0101] + a[i1010] + a[i1111];
        a[i0000] = c1 * a[i0000] + c2 * term;
        a[i0101] = c1 * a[i0101] + c2 * term;
        a[i1010] = c1 * a[i1010] + c2 * term;
        a[i1111] = c1 * a[i1111] + c2 * term;
    }
}

/* cpu_densmatr_oneQubitDephasing_subA: cpu_subroutines.cpp:1072-1105; factor utilities.cpp:918-921 */
extern "C" void orc_dm_dephasing1(double* amps, int nKet, int ket, double prob) {
    int bra = ket + nKet;
    double fac = 1 - (2 * prob);
    idx numIts = pow2(2 * nKet) / 4;
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx i01 = insertTwo(n, bra, 0, ket, 1);
        idx i10 = insertTwo(n, bra, 1, ket, 0);
        a[i01] *= fac;
        a[i10] *= fac;
    }
}

/* cpu_densmatr_twoQubitDephasing_subB: cpu_subroutines.cpp:1143-1170; term utilities.cpp:923-926 */
extern "C" void orc_dm_dephasing2(double* amps, int nKet, int qA, int qB, double prob) {
    double term = -4 * prob / 3;
    int bA = qA + nKet, bB = qB + nKet;
    cplx* a = C(amps);
    idx N = pow2(2 * nKet);
    #pragma omp parallel for NT
    for (idx n = 0; n < N; n++) {
        int flag = (getBit(n, qA) ^ getBit(n, bA)) | (getBit(n, qB) ^ getBit(n, bB));
        a[n] *= 1 + (flag * term);
    }
}

/* cpu_densmatr_oneQubitDamping_subA: cpu_subroutines.cpp:1550-1575; factors utilities.cpp:977-988 */
extern "C" void orc_dm_damping1(double* amps, int nKet, int ket, double prob) {
    int bra = ket + nKet;
    double c1 = std::sqrt(1 - prob), c2 = 1 - prob;
    idx numIts = pow2(2 * nKet) / 4;
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx i00 = insertTwo(n, bra, 0, ket, 0);
        idx i01 = flipBit(i00, ket), i10 = flipBit(i00, bra), i11 = flipBit(i01, bra);
        a[i00] += prob * a[i11];
        a[i01] *= c1;
        a[i10] *= c1;
        a[i11] *= c2;
    }
}

/* localiser_densmatr_oneQubitPauliChannel (localiser.cpp:1575-1585) and
 * cpu_densmatr_oneQubitPauliChannel_subA (cpu_subroutines.cpp:1455-1496);
 * factors utilities.cpp:962-975 */
extern "C" void orc_dm_pauliChannel1(double* amps, int nKet, int ket, double pX, double pY, double pZ) {
    double pI = 1 - pX - pY - pZ;
    int bra = ket + nKet;
    double fAA = pI + pZ, fBB = pX + pY, fAB = pI - pZ, fBA = pX - pY;
    idx numIts = pow2(2 * nKet) / 4;
    cplx* a = C(amps);
    #pragma omp parallel for NT
    for (idx n = 0; n < numIts; n++) {
        idx i00 = insertTwo(n, bra, 0, ket, 0);
        idx i01 = flipBit(i00, ket), i10 = flipBit(i00, bra), i11 = flipBit(i01, bra);
        cplx a00 = a[i00], a01 = a[i01], a10 = a[i10], a11 = a[i11];
        a[i00] = (fAA * a00) + (fBB * a11);
        a[i01] = (fAB * a01) + (fBA * a10);
        a[i10] = (fAB * a10) + (fBA * a01);
        a[i11] = (fAA * a11) + (fBB * a00);
    }
}

/* cpu_densmatr_multiQubitProjector_sub: cpu_subroutines.cpp:2309-2343 */
extern "C" void orc_dm_projector(double* amps, int nKet, const int* qubits, const int* outcomes, int n, double prob) {
    double renorm = 1 / prob;
    idx retain = 0;
    for (int i = 0; i < n; i++) retain |= ((idx)outcomes[i]) << i;
    cplx* a = C(amps);
    idx N = pow2(2 * nKet);
    idx rowMask = pow2(nKet) - 1;
    #pragma omp parallel for NT
    for (idx k = 0; k < N; k++) {
        idx r = k & rowMask, c = k >> nKet;
        idx v1 = getValueOfBits(r, qubits, n), v2 = getValueOfBits(c, qubits, n);
        cplx fac = renorm * (double)(v1 == v2) * (double)(retain == v1);
        a[k] *= fac;
    }
}

/* ------------------------------------------------------------------------ */
/* reductions                                                                */
/* ------------------------------------------------------------------------ */

/* cpu_statevec_calcTotalProb_sub: cpu_subroutines.cpp:1704-1727 */
extern "C" double orc_sv_totalProb(const double* amps, int nq) {
    const cplx* a = C(amps);
    double prob = 0;
    idx N = pow2(nq);
    #pragma omp parallel for reduction(+:prob) NT
    for (idx n = 0; n < N; n++) prob += std::norm(a[n]);
    return prob;
}

/* cpu_densmatr_calcTotalProb_sub: cpu_subroutines.cpp:1730-1757 (diagonal stride 2^n + 1) */
extern "C" double orc_dm_totalProb(const double* amps, int nKet) {
    const cplx* a = C(amps);
    double prob = 0;
    idx dim = pow2(nKet);
    #pragma omp parallel for reduction(+:prob) NT
    for (idx n = 0; n < dim; n++) prob += std::real(a[n * (dim + 1)]);
    return prob;
}

/* cpu_statevec_calcProbOfMultiQubitOutcome_sub: cpu_subroutines.cpp:1760-1786 */
extern "C" double orc_sv_probOfOutcome(const double* amps, int nq, const int* qubits, const int* outcomes, int n) {
    QubitSet s = makeSet(nullptr, nullptr, 0, qubits, outcomes, n);
    const cplx* a = C(amps);
    double prob = 0;
    idx numIts = pow2(nq) >> n;
    #pragma omp parallel for reduction(+:prob) NT
    for (idx k = 0; k < numIts; k++) prob += std::norm(a[insertWithMask(k, s)]);
    return prob;
}

/* cpu_densmatr_calcProbOfMultiQubitOutcome_sub: cpu_subroutines.cpp:1789-1824 */
extern "C" double orc_dm_probOfOutcome(const double* amps, int nKet, const int* qubits, const int* outcomes, int n) {
    QubitSet s = makeSet(nullptr, nullptr, 0, qubits, outcomes, n);
    const cplx* a = C(amps);
    double prob = 0;
    idx dim = pow2(nKet);
    idx numIts = pow2(nKet - n);
    #pragma omp parallel for reduction(+:prob) NT
    for (idx k = 0; k < numIts; k++) {
        idx i = insertWithMask(k, s);
        prob += std::real(a[i * (dim + 1)]);
    }
    return prob;
}

/* cpu_statevec_calcProbsOfAllMultiQubitOutcomes_sub: cpu_subroutines.cpp:1827-1860 */
extern "C" void orc_sv_probsOfAllOutcomes(double* out, const double* amps, int nq, const int* qubits, int n) {
    const cplx* a = C(amps);
    idx numOut = pow2(n);
    for (idx i = 0; i < numOut; i++) out[i] = 0;
    idx N = pow2(nq);
    for (idx k = 0; k < N; k++) out[getValueOfBits(k, qubits, n)] += std::norm(a[k]);
}

/* cpu_densmatr_calcProbsOfAllMultiQubitOutcomes_sub: cpu_subroutines.cpp:1865-1904 (one diagonal
 * element per column, added to the bin of its outcome) */
extern "C" void orc_dm_probsOfAllOutcomes(double* out, const double* amps, int nKet, const int* qubits, int n) {
    const cplx* a = C(amps);
    idx numOut = pow2(n);
    for (idx i = 0; i < numOut; i++) out[i] = 0;
    idx dim = pow2(nKet);
    for (idx k = 0; k < dim; k++) out[getValueOfBits(k, qubits, n)] += std::real(a[k * (dim + 1)]);
}

/* cpu_statevec_calcExpecAnyTargZ_sub: cpu_subroutines.cpp:2006-2025 */
extern "C" double orc_sv_expecZ(const double* amps, int nq, const int* targs, int nt) {
    const cplx* a = C(amps);
    idx tmask = maskOf(targs, nt);
    double v = 0;
    idx N = pow2(nq);
    #pragma omp parallel for reduction(+:v) NT
    for (idx n = 0; n < N; n++) v += signOfParity(n, tmask) * std::norm(a[n]);
    return v;
}

/* cpu_densmatr_calcExpecAnyTargZ_sub: cpu_subroutines.cpp:2028-2056 */
extern "C" void orc_dm_expecZ(double* out, const double* amps, int nKet, const int* targs, int nt) {
    const cplx* a = C(amps);
    idx tmask = maskOf(targs, nt);
    idx dim = pow2(nKet);
    double re = 0, im = 0;
    #pragma omp parallel for reduction(+:re,im) NT
    for (idx n = 0; n < dim; n++) {
        cplx term = (double)signOfParity(n, tmask) * a[n * (dim + 1)];
        re += term.real(); im += term.imag();
    }
    out[0] = re; out[1] = im;
}

/* cpu_statevec_calcExpecPauliStr_subA: cpu_subroutines.cpp:2059-2085 */
extern "C" void orc_sv_expecPauli(double* out, const double* amps, int nq, const int* x, int nx, const int* y, int ny, const int* z, int nz) {
    const cplx* a = C(amps);
    idx maskXY = maskOf(x, nx) | maskOf(y, ny);
    idx maskYZ = maskOf(y, ny) | maskOf(z, nz);
    double re = 0, im = 0;
    idx N = pow2(nq);
    #pragma omp parallel for reduction(+:re,im) NT
    for (idx n = 0; n < N; n++) {
        idx j = n ^ maskXY;
        cplx term = (double)signOfParity(j, maskYZ) * std::conj(a[n]) * a[j];
        re += term.real(); im += term.imag();
    }
    static const cplx powI[4] = {cplx(1, 0), cplx(0, 1), cplx(-1, 0), cplx(0, -1)};
    cplx v = cplx(re, im) * powI[ny % 4];
    out[0] = v.real(); out[1] = v.imag();
}

/* cpu_densmatr_calcExpecPauliStr_sub: cpu_subroutines.cpp:2121-2160 */
extern "C" void orc_dm_expecPauli(double* out, const double* amps, int nKet, const int* x, int nx, const int* y, int ny, const int* z, int nz) {
    const cplx* a = C(amps);
    idx maskXY = maskOf(x, nx) | maskOf(y, ny);
    idx maskYZ = maskOf(y, ny) | maskOf(z, nz);
    idx dim = pow2(nKet);
    double re = 0, im = 0;
    #pragma omp parallel for reduction(+:re,im) NT
    for (idx n = 0; n < dim; n++) {
        idx i = n ^ maskXY;
        idx m = i + n * dim;
        cplx term = (double)signOfParity(i, maskYZ) * a[m];
        re += term.real(); im += term.imag();
    }
    static const cplx powI[4] = {cplx(1, 0), cplx(0, 1), cplx(-1, 0), cplx(0, -1)};
    cplx v = cplx(re, im) * powI[ny % 4];
    out[0] = v.real(); out[1] = v.imag();
}

/* util_setSuperoperator: utilities.cpp:770-801 -- superop[r][c] += conj(K[i][j]) K[k][l],
 * r = i*dim + k, c = j*dim + l */
extern "C" void orc_build_superop(double* outP, const double* krausP, int numOps, int k) {
    idx dim = pow2(k), sdim = dim * dim;
    cplx* out = C(outP);
    const cplx* kr = C(krausP);
    for (idx i = 0; i < sdim * sdim; i++) out[i] = 0;
    for (int n = 0; n < numOps; n++) {
        const cplx* K = kr + n * dim * dim;
        for (idx i = 0; i < dim; i++)
            for (idx j = 0; j < dim; j++)
                for (idx kk = 0; kk < dim; kk++)
                    for (idx l = 0; l < dim; l++) {
                        idx r = i * dim + kk, c = j * dim + l;
                        out[r * sdim + c] += std::conj(K[i * dim + j]) * K[kk * dim + l];
                    }
    }
}

/* ------------------------------------------------------------------------ */
/* API-level decomposition and the text circuit runner                        */
/* ------------------------------------------------------------------------ */

namespace {

struct Runner {
    int n;          /* qubits of the Qureg (ket qubits for a density matrix) */
    int isDM;
    int nsv;        /* qubits of the underlying statevector (2n for a density matrix) */
    double* amps;
    vector<double> results;
    vector<int> outcomes;
    std::mt19937_64 gen;
    std::string err;

    vector<int> bra(const vector<int>& q) const { vector<int> o(q); for (auto& v : o) v += n; return o; }

    static vector<double> conjOf(const vector<double>& m) { vector<double> o(m); for (size_t i = 1; i < o.size(); i += 2) o[i] = -o[i]; return o; }

    /* validateAndApplyAnyCtrlAnyTargUnitaryMatrix + localiser_statevec_anyCtrlAnyTargAnyMatr:
     * operations.cpp:36-63, localiser.cpp:1051-1076 (1 and 2 targets divert to bespoke routines) */
    void denseOnSV(const vector<int>& c, const vector<int>& s, const vector<int>& t, const vector<double>& m, bool conj) {
        const int* sp = s.empty() ? nullptr : s.data();
        vector<double> mm = conj ? conjOf(m) : m;
        if (t.size() == 1) orc_sv_dense1(amps, nsv, c.data(), sp, (int)c.size(), t[0], mm.data());
        else if (t.size() == 2) orc_sv_dense2(amps, nsv, c.data(), sp, (int)c.size(), t[0], t[1], mm.data());
        else orc_sv_denseK(amps, nsv, c.data(), sp, (int)c.size(), t.data(), (int)t.size(), m.data(), conj ? 1 : 0);
    }
    void dense(const vector<int>& c, const vector<int>& s, const vector<int>& t, const vector<double>& m) {
        denseOnSV(c, s, t, m, false);
        if (isDM) denseOnSV(bra(c), s, bra(t), m, true);
    }
    void diagOnSV(const vector<int>& c, const vector<int>& s, const vector<int>& t, const vector<double>& d, bool conj, const double* ex) {
        const int* sp = s.empty() ? nullptr : s.data();
        if (ex == nullptr && t.size() == 1) { vector<double> dd = conj ? conjOf(d) : d; orc_sv_diag1(amps, nsv, c.data(), sp, (int)c.size(), t[0], dd.data()); }
        else if (ex == nullptr && t.size() == 2) { vector<double> dd = conj ? conjOf(d) : d; orc_sv_diag2(amps, nsv, c.data(), sp, (int)c.size(), t[0], t[1], dd.data()); }
        else orc_sv_diagK(amps, nsv, c.data(), sp, (int)c.size(), t.data(), (int)t.size(), d.data(), conj ? 1 : 0, ex);
    }
    void diag(const vector<int>& c, const vector<int>& s, const vector<int>& t, const vector<double>& d, const double* ex) {
        diagOnSV(c, s, t, d, false, ex);
        if (isDM) diagOnSV(bra(c), s, bra(t), d, true, ex);
    }
    /* Pauli string as per-qubit codes 0..3 (I,X,Y,Z) over nsv qubits */
    static void split(const vector<int>& codes, vector<int>& x, vector<int>& y, vector<int>& z) {
        for (size_t q = 0; q < codes.size(); q++) {
            if (codes[q] == 1) x.push_back((int)q);
            if (codes[q] == 2) y.push_back((int)q);
            if (codes[q] == 3) z.push_back((int)q);
        }
    }
    static bool oddY(const vector<int>& codes) { int k = 0; for (int v : codes) k += (v == 2); return k % 2; }
    vector<int> shifted(const vector<int>& codes) const { vector<int> o(nsv, 0); for (size_t q = 0; q < codes.size() && (int)q < n; q++) o[q + n] = codes[q]; return o; }
    vector<int> padded(const vector<int>& codes) const { vector<int> o(nsv, 0); for (size_t q = 0; q < codes.size() && (int)q < nsv; q++) o[q] = codes[q]; return o; }

    /* localiser_statevec_anyCtrlPauliTensor / ZTensorOrGadget / PauliGadget: localiser.cpp:1247-1360 */
    void pauliTensorSV(const vector<int>& c, const vector<int>& s, const vector<int>& codes, cplx factor) {
        vector<int> x, y, z; split(codes, x, y, z);
        const int* sp = s.empty() ? nullptr : s.data();
        if (!x.empty() || !y.empty()) {
            cplx af = 0.0 * factor, pf = 1.0 * factor;
            double a2[2] = {af.real(), af.imag()}, p2[2] = {pf.real(), pf.imag()};
            orc_sv_pauliTensorOrGadget(amps, nsv, c.data(), sp, (int)c.size(), x.data(), (int)x.size(), y.data(), (int)y.size(), z.data(), (int)z.size(), a2, p2);
        } else {
            double f0[2] = {1, 0}, f1[2] = {-1, 0};
            orc_sv_zOrPhaseGadget(amps, nsv, c.data(), sp, (int)c.size(), z.data(), (int)z.size(), f0, f1);
        }
    }
    void phaseGadgetSV(const vector<int>& c, const vector<int>& s, const vector<int>& t, double phase) {
        const int* sp = s.empty() ? nullptr : s.data();
        cplx f0 = std::exp(cplx(0, +phase)), f1 = std::exp(cplx(0, -phase));
        double a[2] = {f0.real(), f0.imag()}, b[2] = {f1.real(), f1.imag()};
        orc_sv_zOrPhaseGadget(amps, nsv, c.data(), sp, (int)c.size(), t.data(), (int)t.size(), a, b);
    }
    void pauliGadgetSV(const vector<int>& c, const vector<int>& s, const vector<int>& codes, double phase) {
        vector<int> x, y, z; split(codes, x, y, z);
        if (x.empty() && y.empty()) { phaseGadgetSV(c, s, z, phase); return; }
        const int* sp = s.empty() ? nullptr : s.data();
        cplx af = std::cos(phase), pf = std::sin(phase) * cplx(0, 1);
        double a2[2] = {af.real(), af.imag()}, p2[2] = {pf.real(), pf.imag()};
        orc_sv_pauliTensorOrGadget(amps, nsv, c.data(), sp, (int)c.size(), x.data(), (int)x.size(), y.data(), (int)y.size(), z.data(), (int)z.size(), a2, p2);
    }
    /* applyMultiStateControlledPauliStr: operations.cpp:1061-1090 */
    void pauliStr(const vector<int>& c, const vector<int>& s, const vector<int>& codesIn) {
        vector<int> codes = padded(codesIn);
        if (isDM && c.empty()) {
            cplx factor = oddY(codes) ? -1.0 : 1.0;
            vector<int> both = codes, sh = shifted(codes);
            for (int q = 0; q < nsv; q++) both[q] |= sh[q];
            pauliTensorSV(c, s, both, factor);
            return;
        }
        pauliTensorSV(c, s, codes, 1.0);
        if (isDM) {
            cplx factor = oddY(codes) ? -1.0 : 1.0;
            pauliTensorSV(bra(c), s, shifted(codes), factor);
        }
    }
    /* applyMultiStateControlledPauliGadget: operations.cpp:1449-1476 (phase = -angle/2, utilities.cpp:911-914) */
    void pauliGadget(const vector<int>& c, const vector<int>& s, const vector<int>& codesIn, double angle) {
        vector<int> codes = padded(codesIn);
        bool isId = true; for (int v : codes) if (v) isId = false;
        if (isId && c.empty() && isDM) return;
        double phase = -angle / 2;
        pauliGadgetSV(c, s, codes, phase);
        if (!isDM) return;
        phase *= oddY(codes) ? 1 : -1;
        pauliGadgetSV(bra(c), s, shifted(codes), phase);
    }
    /* applyMultiStateControlledPhaseGadget: operations.cpp:1532-1549 */
    void phaseGadget(const vector<int>& c, const vector<int>& s, const vector<int>& t, double angle) {
        double phase = -angle / 2;
        phaseGadgetSV(c, s, t, phase);
        if (!isDM) return;
        phaseGadgetSV(bra(c), s, bra(t), -phase);
    }
    /* applyMultiStateControlledSwap: operations.cpp:778-796 */
    void swap(const vector<int>& c, const vector<int>& s, int a, int b) {
        const int* sp = s.empty() ? nullptr : s.data();
        orc_sv_swap(amps, nsv, c.data(), sp, (int)c.size(), a, b);
        if (!isDM) return;
        vector<int> bc = bra(c);
        orc_sv_swap(amps, nsv, bc.data(), sp, (int)bc.size(), a + n, b + n);
    }
    double probOfOutcome(const vector<int>& q, const vector<int>& o) {
        return isDM ? orc_dm_probOfOutcome(amps, n, q.data(), o.data(), (int)q.size())
                    : orc_sv_probOfOutcome(amps, n, q.data(), o.data(), (int)q.size());
    }
    void projector(const vector<int>& q, const vector<int>& o, double prob) {
        if (isDM) orc_dm_projector(amps, n, q.data(), o.data(), (int)q.size(), prob);
        else orc_sv_projector(amps, n, q.data(), o.data(), (int)q.size(), prob);
    }
    /* calcExpecPauliStr: calculations.cpp:133-144 -> localiser.cpp:1963-2049 */
    double expec(const vector<int>& codesIn) {
        vector<int> codes(n, 0);
        for (size_t q = 0; q < codesIn.size() && (int)q < n; q++) codes[q] = codesIn[q];
        vector<int> x, y, z; split(codes, x, y, z);
        double out[2];
        if (!isDM) {
            if (x.empty() && y.empty() && z.empty()) return orc_sv_totalProb(amps, n);
            if (x.empty() && y.empty()) return orc_sv_expecZ(amps, n, z.data(), (int)z.size());
            orc_sv_expecPauli(out, amps, n, x.data(), (int)x.size(), y.data(), (int)y.size(), z.data(), (int)z.size());
            return out[0];
        }
        if (x.empty() && y.empty() && z.empty()) return orc_dm_totalProb(amps, n);
        if (x.empty() && y.empty()) { orc_dm_expecZ(out, amps, n, z.data(), (int)z.size()); return out[0]; }
        orc_dm_expecPauli(out, amps, n, x.data(), (int)x.size(), y.data(), (int)y.size(), z.data(), (int)z.size());
        return out[0];
    }

    /* the complex term value of one string (localiser.cpp:1963-2049, the value before the
     * real part is taken) */
    cplx expecC(const vector<int>& codesIn) {
        vector<int> codes(n, 0);
        for (size_t q = 0; q < codesIn.size() && (int)q < n; q++) codes[q] = codesIn[q];
        vector<int> x, y, z; split(codes, x, y, z);
        double out[2] = {0, 0};
        if (!isDM) {
            if (x.empty() && y.empty() && z.empty()) return orc_sv_totalProb(amps, n);
            if (x.empty() && y.empty()) return orc_sv_expecZ(amps, n, z.data(), (int)z.size());
            orc_sv_expecPauli(out, amps, n, x.data(), (int)x.size(), y.data(), (int)y.size(), z.data(), (int)z.size());
            return cplx(out[0], out[1]);
        }
        if (x.empty() && y.empty() && z.empty()) return orc_dm_totalProb(amps, n);
        if (x.empty() && y.empty()) orc_dm_expecZ(out, amps, n, z.data(), (int)z.size());
        else orc_dm_expecPauli(out, amps, n, x.data(), (int)x.size(), y.data(), (int)y.size(), z.data(), (int)z.size());
        return cplx(out[0], out[1]);
    }
    /* calcProbsOfAllMultiQubitOutcomes: calculations.cpp:265-275 */
    vector<double> probsOfAll(const vector<int>& q) {
        vector<double> p(pow2((int)q.size()));
        if (isDM) orc_dm_probsOfAllOutcomes(p.data(), amps, n, q.data(), (int)q.size());
        else orc_sv_probsOfAllOutcomes(p.data(), amps, n, q.data(), (int)q.size());
        return p;
    }

    bool run(const std::string& text);
};

static vector<int> parsePauli(const std::string& s) {
    vector<int> codes;
    for (char ch : s) {
        switch (ch) {
            case 'I': case '0': codes.push_back(0); break;
            case 'X': case '1': codes.push_back(1); break;
            case 'Y': case '2': codes.push_back(2); break;
            case 'Z': case '3': codes.push_back(3); break;
            default: break;
        }
    }
    return codes;
}

bool Runner::run(const std::string& text) {
    std::istringstream lines(text);
    std::string line;
    int lineNo = 0;
    auto rdInts = [](std::istringstream& is, int k) { vector<int> v(k); for (int i = 0; i < k; i++) is >> v[i]; return v; };
    auto rdDbl = [](std::istringstream& is, int k) { vector<double> v(k); for (int i = 0; i < k; i++) is >> v[i]; return v; };
    while (std::getline(lines, line)) {
        lineNo++;
        std::istringstream is(line);
        std::string op;
        if (!(is >> op) || op[0] == '#') continue;
        const double PI = 3.141592653589793238462643383279502884;
        if (op == "H") {                 /* operations.cpp:716-723 */
            int t; is >> t; double a = 1 / std::sqrt(2);
            dense({}, {}, {t}, {a, 0, a, 0, a, 0, -a, 0});
        } else if (op == "X" || op == "Y") {
            int t; is >> t; vector<int> codes(t + 1, 0); codes[t] = (op == "X") ? 1 : 2;
            pauliStr({}, {}, codes);
        } else if (op == "Z") {          /* operations.cpp:977-985 */
            int t; is >> t; diag({}, {}, {t}, {1, 0, -1, 0}, nullptr);
        } else if (op == "S") {          /* operations.cpp:614-618 */
            int t; is >> t; diag({}, {}, {t}, {1, 0, 0, 1}, nullptr);
        } else if (op == "T") {          /* operations.cpp:665-669 */
            int t; is >> t; double r = 1 / std::sqrt(2); diag({}, {}, {t}, {1, 0, r, r}, nullptr);
        } else if (op == "RX" || op == "RY" || op == "RZ") {   /* operations.cpp:1283-1308 */
            int t; double th; is >> t >> th; vector<int> codes(t + 1, 0); codes[t] = op[1] - 'W';
            pauliGadget({}, {}, codes, th);
        } else if (op == "CRX" || op == "CRY" || op == "CRZ") {
            int c, t; double th; is >> c >> t >> th; vector<int> codes(t + 1, 0); codes[t] = op[2] - 'W';
            pauliGadget({c}, {}, codes, th);
        } else if (op == "PS") {         /* applyPhaseShift: operations.cpp:1588-1613 */
            int t; double th; is >> t >> th; cplx e = std::exp(cplx(0, 1) * th);
            diag({}, {}, {t}, {1, 0, e.real(), e.imag()}, nullptr);
        } else if (op == "CPS") {        /* applyTwoQubitPhaseShift: operations.cpp:1596-1613 */
            int t1, t2; double th; is >> t1 >> t2 >> th; cplx e = std::exp(cplx(0, 1) * th);
            diag({t2}, {}, {t1}, {1, 0, e.real(), e.imag()}, nullptr);
        } else if (op == "MPS") {        /* applyMultiQubitPhaseShift: operations.cpp:1605-1613 */
            int k; is >> k; auto t = rdInts(is, k); double th; is >> th; cplx e = std::exp(cplx(0, 1) * th);
            diag(vector<int>(t.begin() + 1, t.end()), {}, {t[0]}, {1, 0, e.real(), e.imag()}, nullptr);
        } else if (op == "CX") {         /* applyControlledPauliX: operations.cpp:911-916 */
            int c, t; is >> c >> t; vector<int> codes(t + 1, 0); codes[t] = 1; pauliStr({c}, {}, codes);
        } else if (op == "CZ") {         /* applyControlledPauliZ: operations.cpp:927-932 */
            int c, t; is >> c >> t; diag({c}, {}, {t}, {1, 0, -1, 0}, nullptr);
        } else if (op == "SWAP") {
            int a, b; is >> a >> b; swap({}, {}, a, b);
        } else if (op == "CSWAP") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int a, b; is >> a >> b; swap(c, s, a, b);
        } else if (op == "U1") {
            int t; is >> t; dense({}, {}, {t}, rdDbl(is, 8));
        } else if (op == "CU1") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int t; is >> t; dense(c, s, {t}, rdDbl(is, 8));
        } else if (op == "U2") {
            int t1, t2; is >> t1 >> t2; dense({}, {}, {t1, t2}, rdDbl(is, 32));
        } else if (op == "CU2") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int t1, t2; is >> t1 >> t2; dense(c, s, {t1, t2}, rdDbl(is, 32));
        } else if (op == "UK") {
            int k; is >> k; auto t = rdInts(is, k); dense({}, {}, t, rdDbl(is, 2 << (2 * k)));
        } else if (op == "CUK") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int k; is >> k; auto t = rdInts(is, k);
            dense(c, s, t, rdDbl(is, 2 << (2 * k)));
        } else if (op == "D1") {
            int t; is >> t; diag({}, {}, {t}, rdDbl(is, 4), nullptr);
        } else if (op == "D2") {
            int t1, t2; is >> t1 >> t2; diag({}, {}, {t1, t2}, rdDbl(is, 8), nullptr);
        } else if (op == "DK") {
            int k; is >> k; auto t = rdInts(is, k); diag({}, {}, t, rdDbl(is, 2 << k), nullptr);
        } else if (op == "CDK") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int k; is >> k; auto t = rdInts(is, k);
            diag(c, s, t, rdDbl(is, 2 << k), nullptr);
        } else if (op == "DKP") {        /* applyMultiStateControlledDiagMatrPower: operations.cpp:468-500 */
            int k; is >> k; auto t = rdInts(is, k); auto d = rdDbl(is, 2 << k); auto ex = rdDbl(is, 2);
            diag({}, {}, t, d, ex.data());
        } else if (op == "FSD") {        /* (apply|multiply)FullStateDiagMatr[Power]: operations.cpp:537-576 */
            int mult, hasPow; is >> mult >> hasPow;
            vector<double> ex = hasPow ? rdDbl(is, 2) : vector<double>{1.0, 0.0};
            auto d = rdDbl(is, 2 * (size_t)pow2(n));
            if (isDM) orc_dm_allTargDiag(amps, n, d.data(), ex.data(), mult);
            else orc_sv_allTargDiag(amps, n, d.data(), ex.data());
        } else if (op == "EXPFSD") {     /* calcExpec[NonHermitian]FullStateDiagMatr[Power]: calculations.cpp:85-215 */
            int kind; is >> kind;        /* 0: Hermitian, 1: Hermitian power (real p), 2: non-Hermitian, 3: non-Hermitian power */
            vector<double> ex = {1.0, 0.0};
            if (kind == 1) { double p; is >> p; ex = {p, 0.0}; }
            if (kind == 3) ex = rdDbl(is, 2);
            auto d = rdDbl(is, 2 * (size_t)pow2(n));
            double v[2];
            int useRealPow = kind == 1;
            if (isDM) orc_dm_expecAllTargDiag(v, amps, n, d.data(), ex.data(), useRealPow);
            else orc_sv_expecAllTargDiag(v, amps, n, d.data(), ex.data(), useRealPow);
            results.push_back(v[0]);
            if (kind >= 2) results.push_back(v[1]);
        } else if (op == "PSTR") {
            std::string s; is >> s; pauliStr({}, {}, parsePauli(s));
        } else if (op == "CPSTR") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); std::string p; is >> p; pauliStr(c, s, parsePauli(p));
        } else if (op == "PG") {
            std::string s; double th; is >> s >> th; pauliGadget({}, {}, parsePauli(s), th);
        } else if (op == "CPG") {
            int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); std::string p; double th; is >> p >> th;
            pauliGadget(c, s, parsePauli(p), th);
        } else if (op == "PHG") {
            int k; is >> k; auto t = rdInts(is, k); double th; is >> th; phaseGadget({}, {}, t, th);
        } else if (op == "QFT" || op == "FQFT") {   /* operations.cpp:1934-1966 */
            vector<int> t;
            if (op == "QFT") { int k; is >> k; t = rdInts(is, k); }
            else { for (int q = 0; q < n; q++) t.push_back(q); }
            int k = (int)t.size();
            double a = 1 / std::sqrt(2);
            for (int m = k - 1; m >= 0; m--) {
                dense({}, {}, {t[m]}, {a, 0, a, 0, a, 0, -a, 0});
                for (int j = 0; j < m; j++) {
                    double arg = PI / (double)pow2(j + 1);
                    cplx e = std::exp(cplx(0, 1) * arg);
                    diag({t[m - j - 1]}, {}, {t[m]}, {1, 0, e.real(), e.imag()}, nullptr);
                }
            }
            for (int m = 0; m < k / 2; m++) swap({}, {}, t[m], t[k - 1 - m]);
        } else if (op == "DEPOL") {      /* mixDepolarising: decoherence.cpp:61-74 */
            int q; double p; is >> q >> p; if (p != 0) orc_dm_depolarising1(amps, n, q, p);
        } else if (op == "DEPOL2") {
            int a, b; double p; is >> a >> b >> p; if (p != 0) orc_dm_depolarising2(amps, n, a, b, p);
        } else if (op == "DEPHASE") {
            int q; double p; is >> q >> p; if (p != 0) orc_dm_dephasing1(amps, n, q, p);
        } else if (op == "DEPHASE2") {
            int a, b; double p; is >> a >> b >> p; if (p != 0) orc_dm_dephasing2(amps, n, a, b, p);
        } else if (op == "DAMP") {
            int q; double p; is >> q >> p; if (p != 0) orc_dm_damping1(amps, n, q, p);
        } else if (op == "PAULIS") {
            int q; double px, py, pz; is >> q >> px >> py >> pz;
            if (!(px == 0 && py == 0 && pz == 0)) orc_dm_pauliChannel1(amps, n, q, px, py, pz);
        } else if (op == "KRAUS") {      /* mixKrausMap: decoherence.cpp:121-131, localiser.cpp:1670-1686 */
            int k; is >> k; auto t = rdInts(is, k); int nops; is >> nops;
            auto kr = rdDbl(is, nops * (2 << (2 * k)));
            vector<double> sup(2 << (4 * k));
            orc_build_superop(sup.data(), kr.data(), nops, k);
            vector<int> all = t; for (int q : t) all.push_back(q + n);
            denseOnSV({}, {}, all, sup, false);
        } else if (op == "PROJ") {       /* applyMultiQubitProjector: operations.cpp:1766-1780 */
            int k; is >> k; auto q = rdInts(is, k); auto o = rdInts(is, k); projector(q, o, 1.0);
        } else if (op == "SEED") {       /* setSeeds -> rand_setSeeds: randomiser.cpp:59-86 */
            vector<unsigned> seeds; unsigned v; while (is >> v) seeds.push_back(v);
            std::seed_seq seq(seeds.begin(), seeds.end()); gen.seed(seq);
        } else if (op == "MEAS") {       /* applyQubitMeasurementAndGetProb: operations.cpp:1804-1826 */
            int q; is >> q;
            double p0 = probOfOutcome({q}, {0}), p1 = probOfOutcome({q}, {1});
            std::uniform_real_distribution<double> distrib(0, 1);   /* randomiser.cpp:125-137 */
            double sample = distrib(gen);
            int outcome = sample > p0;
            projector({q}, {outcome}, outcome ? p1 : p0);
            outcomes.push_back(outcome);
        } else if (op == "MEASM") {      /* applyMultiQubitMeasurementAndGetProb: operations.cpp:1858-1891 */
            int k; is >> k; auto q = rdInts(is, k);
            vector<double> probs = probsOfAll(q);
            double total = 0, comp = 0;              /* util_getSum: Kahan (utilities.cpp:346-360) */
            for (double x : probs) { double y = x - comp, t = total + y; comp = (t - total) - y; total = t; }
            if (std::abs(total - 1) > 1e-12) { err = "MEASM: outcome probabilities do not sum to one"; return false; }
            std::uniform_real_distribution<double> distrib(0, 1);   /* rand_getRandomMultiQubitOutcome: randomiser.cpp:140-166 */
            double sample = distrib(gen), cum = 0;
            idx outcome = (idx)probs.size();
            for (size_t i = 0; i < probs.size(); i++) { cum += probs[i]; if (sample < cum) { outcome = (idx)i; break; } }
            if (outcome == (idx)probs.size()) {
                if (1 - cum <= 1e-12) outcome = (idx)probs.size() - 1;
                else { err = "MEASM: non-normalised probabilities"; return false; }
            }
            vector<int> o(k);
            for (int i = 0; i < k; i++) o[i] = (int)((outcome >> i) & 1);   /* getBitsFromInteger */
            projector(q, o, probs[(size_t)outcome]);
            outcomes.push_back((int)outcome);
            results.push_back(probs[(size_t)outcome]);
        } else if (op == "FMEAS") {      /* applyForcedQubitMeasurement: operations.cpp:1829-1846 */
            int q, o; is >> q >> o;
            double p = probOfOutcome({q}, {o});
            if (p < 1e-12) { err = "FMEAS: outcome impossibly unlikely"; return false; }
            projector({q}, {o}, p);
            results.push_back(p);
        } else if (op == "FMEASM") {     /* applyForcedMultiQubitMeasurement: operations.cpp:1893-1912 */
            int k; is >> k; auto q = rdInts(is, k); auto o = rdInts(is, k);
            double p = probOfOutcome(q, o);
            if (p < 1e-12) { err = "FMEASM: outcome impossibly unlikely"; return false; }
            projector(q, o, p);
            results.push_back(p);
        } else if (op == "PROBALL") {    /* calcProbsOfAllMultiQubitOutcomes: calculations.cpp:265-275 */
            int k; is >> k; auto q = rdInts(is, k);
            for (double v : probsOfAll(q)) results.push_back(v);
        } else if (op == "EXPSUM") {     /* calcExpecPauliStrSum: calculations.cpp:146-159, localiser.cpp:2052-2148 */
            int T; is >> T;
            cplx total = 0;
            for (int t = 0; t < T; t++) {
                double cr, ci; std::string ps; is >> cr >> ci >> ps;
                total += cplx(cr, ci) * expecC(parsePauli(ps));
            }
            results.push_back(total.real());
        } else if (op == "TOTALPROB") {  /* calcTotalProb: calculations.cpp:278-284 */
            results.push_back(isDM ? orc_dm_totalProb(amps, n) : orc_sv_totalProb(amps, n));
        } else if (op == "PURITY") {     /* calcPurity: calculations.cpp:293-300 */
            double p = orc_sv_totalProb(amps, nsv);
            results.push_back(isDM ? p : p * p);
        } else if (op == "PROBQ") {
            int q, o; is >> q >> o; results.push_back(probOfOutcome({q}, {o}));
        } else if (op == "PROBMQ") {
            int k; is >> k; auto q = rdInts(is, k); auto o = rdInts(is, k); results.push_back(probOfOutcome(q, o));
        } else if (op == "EXPEC") {
            std::string s; is >> s; results.push_back(expec(parsePauli(s)));
        } else {
            err = "unknown op '" + op + "' on line " + std::to_string(lineNo);
            return false;
        }
    }
    return true;
}

thread_local std::string g_err;

} // namespace

extern "C" const char* orc_last_error(void) { return g_err.c_str(); }

static double g_lastSeconds = 0;
/* seconds spent in the ops of the last orc_run_circuit call (no state copies) */
extern "C" double orc_last_run_seconds(void) { return g_lastSeconds; }

extern "C" int orc_run_circuit(const char* text, int numQubits, int isDensMatr, double* amps,
                               double* results, int maxResults, int* numResults,
                               int* outcomes, int maxOutcomes, int* numOutcomes) {
    Runner r;
    r.n = numQubits;
    r.isDM = isDensMatr;
    r.nsv = isDensMatr ? 2 * numQubits : numQubits;
    r.amps = amps;
    std::seed_seq seq{0u};
    r.gen.seed(seq);
    const auto t0 = std::chrono::steady_clock::now();
    bool ok = r.run(text ? std::string(text) : std::string());
    g_lastSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (numResults) *numResults = (int)r.results.size();
    if (numOutcomes) *numOutcomes = (int)r.outcomes.size();
    for (int i = 0; i < (int)r.results.size() && i < maxResults; i++) results[i] = r.results[i];
    for (int i = 0; i < (int)r.outcomes.size() && i < maxOutcomes; i++) outcomes[i] = r.outcomes[i];
    if (!ok) { g_err = r.err; return -1; }
    return 0;
}
