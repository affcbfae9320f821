// Density-matrix channel kernels of the sm_103a backend (FP64).
//
// A density matrix of N qubits is its column-major Choi vector of 2N qubits
// (row = low N bits, column = high N bits; quest/src/core/fastmath.hpp:68-93),
// so the bra partner of ket qubit q is bit q+N.  A one-qubit channel mixes the
// four amplitudes {i00, i01, i10, i11} over (ket q, bra q+N): one thread owns
// one such group, found by inserting zeros at q and q+N.  For q near N the two
// strides are 2^q and 2^(q+N) apart; consecutive threads still walk consecutive
// addresses within each of the four streams.
//
// Reference algorithms: quest/src/cpu/cpu_subroutines.cpp:1060-1600 and the
// factors of quest/src/core/utilities.cpp:916-990.
#include "qg_common.cuh"

#include <algorithm>
#include <cmath>

namespace {

__device__ __forceinline__ qidx insert_zero(qidx n, int b) {
    qidx lo = n & (((qidx)1 << b) - 1);
    return ((n ^ lo) << 1) | lo;
}
// positions lo < hi
__device__ __forceinline__ qidx insert_two_zeros(qidx n, int lo, int hi) { return insert_zero(insert_zero(n, lo), hi); }

__device__ __forceinline__ double2 lin2(double c1, double2 x, double c2, double2 y) {
    return make_double2(fma(c1, x.x, c2 * y.x), fma(c1, x.y, c2 * y.y));
}

}  // namespace

// One-qubit channels on the 4-amplitude groups {i00, i01, i10, i11} over (ket q, bra q+N).
// Each thread takes G groups per iteration of a grid-stride loop and issues all their
// loads before any arithmetic, so that G x 64 B per thread are in flight.
enum { CH_DEPOL = 0, CH_PAULI = 1, CH_DAMP = 2, CH_DEPHASE = 3 };

template <int KIND, int G>
__global__ void __launch_bounds__(QG_THREADS) k_dm_channel1(double2* __restrict__ a, qidx numIts, int ket, int bra,
                                                            double f0, double f1, double f2, double f3) {
    const qidx bk = (qidx)1 << ket, bb = (qidx)1 << bra;
    const qidx stride = (qidx)gridDim.x * QG_THREADS * G;
    for (qidx n0 = blockIdx.x * (qidx)QG_THREADS * G + threadIdx.x; n0 < numIts; n0 += stride) {
        qidx i00[G];
        double2 x00[G], x01[G], x10[G], x11[G];
#pragma unroll
        for (int g = 0; g < G; g++) {
            qidx n = n0 + (qidx)g * QG_THREADS;
            i00[g] = insert_two_zeros(n < numIts ? n : n0, ket, bra);
            if (KIND != CH_DEPHASE) {
                x00[g] = ld_amp(a + i00[g]);
                x11[g] = ld_amp(a + (i00[g] | bk | bb));
            }
            x01[g] = ld_amp(a + (i00[g] | bk));
            x10[g] = ld_amp(a + (i00[g] | bb));
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (n0 + (qidx)g * QG_THREADS >= numIts) break;
            const qidx i = i00[g];
            if (KIND == CH_DEPOL) {
                // cpu_densmatr_oneQubitDepolarising_subA (cpu_subroutines.cpp:1183-1215):
                // a00' = cAA a00 + cBB a11 with cAA = 1 - cBB, written a00 + cBB (a11 - a00)
                // (3 FP64 operations per real pair instead of 4); off-diagonals times cAB
                double2 d = make_double2(x11[g].x - x00[g].x, x11[g].y - x00[g].y);
                st_amp(a + i, make_double2(fma(f0, d.x, x00[g].x), fma(f0, d.y, x00[g].y)));
                st_amp(a + (i | bk | bb), make_double2(fma(-f0, d.x, x11[g].x), fma(-f0, d.y, x11[g].y)));
                st_amp(a + (i | bk), cscale(f1, x01[g]));
                st_amp(a + (i | bb), cscale(f1, x10[g]));
            } else if (KIND == CH_PAULI) {
                // cpu_densmatr_oneQubitPauliChannel_subA (cpu_subroutines.cpp:1455-1496)
                st_amp(a + i, lin2(f0, x00[g], f1, x11[g]));
                st_amp(a + (i | bk), lin2(f2, x01[g], f3, x10[g]));
                st_amp(a + (i | bb), lin2(f2, x10[g], f3, x01[g]));
                st_amp(a + (i | bk | bb), lin2(f0, x11[g], f1, x00[g]));
            } else if (KIND == CH_DAMP) {
                // cpu_densmatr_oneQubitDamping_subA (cpu_subroutines.cpp:1550-1575)
                st_amp(a + i, make_double2(fma(f0, x11[g].x, x00[g].x), fma(f0, x11[g].y, x00[g].y)));
                st_amp(a + (i | bk), cscale(f1, x01[g]));
                st_amp(a + (i | bb), cscale(f1, x10[g]));
                st_amp(a + (i | bk | bb), cscale(f2, x11[g]));
            } else {
                // cpu_densmatr_oneQubitDephasing_subA (cpu_subroutines.cpp:1072-1105): only the two
                // off-diagonal amplitudes of each group change
                st_amp(a + (i | bk), cscale(f0, x01[g]));
                st_amp(a + (i | bb), cscale(f0, x10[g]));
            }
        }
    }
}

// cpu_densmatr_twoQubitDephasing_subB (cpu_subroutines.cpp:1143-1170): amplitudes
// whose ket and bra differ on either qubit are scaled by 1 + term.
__global__ void k_dephase2(double2* __restrict__ a, qidx numAmps, int kA, int bA, int kB, int bB, double fac) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numAmps) return;
    int flag = (int)(((n >> kA) ^ (n >> bA)) | ((n >> kB) ^ (n >> bB))) & 1;
    if (flag) st_amp(a + n, cscale(fac, ld_amp(a + n)));
}

// cpu_densmatr_twoQubitDepolarising_subA followed by _subB (cpu_subroutines.cpp:1262-1325),
// fused: one thread owns the 16 amplitudes sharing all other bits.  The four with
// ket == bra on both qubits are mixed; the other twelve are scaled by 1 + c3.
__global__ void k_depol2(double2* __restrict__ a, qidx numIts, Ins ins, int q1, int q2, int b1, int b2,
                         double c1m, double c2, double s) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx base = insert_bits<4>(n, ins);
    qidx bq1 = (qidx)1 << q1, bq2 = (qidx)1 << q2, bb1 = (qidx)1 << b1, bb2 = (qidx)1 << b2;
    qidx i0000 = base, i0101 = base | bq1 | bb1, i1010 = base | bq2 | bb2, i1111 = i0101 | bq2 | bb2;
    double2 x0 = ld_amp(a + i0000), x1 = ld_amp(a + i0101), x2 = ld_amp(a + i1010), x3 = ld_amp(a + i1111);
    double2 t = make_double2(x0.x + x1.x + x2.x + x3.x, x0.y + x1.y + x2.y + x3.y);
    st_amp(a + i0000, lin2(c1m, x0, c2, t));
    st_amp(a + i0101, lin2(c1m, x1, c2, t));
    st_amp(a + i1010, lin2(c1m, x2, c2, t));
    st_amp(a + i1111, lin2(c1m, x3, c2, t));
#pragma unroll
    for (int m = 0; m < 16; m++) {
        // m's bits: (q1, q2, b1, b2); skip the four "ket == bra on both" combinations
        int k1 = m & 1, k2 = (m >> 1) & 1, r1 = (m >> 2) & 1, r2 = (m >> 3) & 1;
        if (k1 == r1 && k2 == r2) continue;
        qidx i = base | (k1 ? bq1 : 0) | (k2 ? bq2 : 0) | (r1 ? bb1 : 0) | (r2 ? bb2 : 0);
        st_amp(a + i, cscale(s, ld_amp(a + i)));
    }
}

// cpu_densmatr_multiQubitProjector_sub (cpu_subroutines.cpp:2309-2343)
__global__ void k_dm_projector(double2* __restrict__ a, qidx numAmps, int nKet, qidx qmask, qidx retainBits, double renorm) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i >= numAmps) return;
    qidx r = i & ((((qidx)1) << nKet) - 1), c = i >> nKet;
    bool keep = ((r & qmask) == retainBits) && ((c & qmask) == retainBits);
    if (keep) st_amp(a + i, cscale(renorm, ld_amp(a + i)));
    else st_amp(a + i, make_double2(0.0, 0.0));
}

namespace {

const int CH_G = 2;   // groups per thread per iteration

template <int KIND>
int launch_channel1(void* amps, int nKet, int qubit, double f0, double f1, double f2, double f3, void* stream, const char* what) {
    qidx numIts = ((qidx)1 << (2 * nKet)) / 4;
    qidx need = (numIts + (qidx)QG_THREADS * CH_G - 1) / ((qidx)QG_THREADS * CH_G);
    unsigned grid = (unsigned)std::max<qidx>(1, std::min<qidx>(need, (qidx)qg_num_sms() * 16));
    k_dm_channel1<KIND, CH_G><<<grid, QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numIts, qubit, qubit + nKet, f0, f1, f2, f3);
    qg_note_launch();
    return qg_check_launch(what);
}

int check_dm(void* amps, int nKet, int qubit) {
    if (nKet < 1 || 2 * nKet > QG_MAX_QUBITS) return qg_fail(QG_ERR_ARG, "density matrix of %d qubits is unsupported", nKet);
    QG_TRY(qg_check_amps(amps, 2 * nKet));
    if (qubit < 0 || qubit >= nKet) return qg_fail(QG_ERR_ARG, "qubit %d outside [0, %d)", qubit, nKet);
    return QG_OK;
}

}  // namespace

extern "C" {

int qg_dm_oneQubitDepolarising(void* amps, int nKet, int qubit, double prob, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit));
    // util_getOneQubitDepolarisingFactors (utilities.cpp:932-947)
    // (cAA = 1 - cBB is folded into the kernel's arithmetic)
    double cBB = 2 * prob / 3, cAB = 1 - (4 * prob / 3);
    return launch_channel1<CH_DEPOL>(amps, nKet, qubit, cBB, cAB, 0, 0, stream, "depol1");
}

int qg_dm_twoQubitDepolarising(void* amps, int nKet, int qubit1, int qubit2, double prob, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit1));
    QG_TRY(check_dm(amps, nKet, qubit2));
    if (qubit1 == qubit2) return qg_fail(QG_ERR_ARG, "the two qubits must differ");
    if (qubit1 > qubit2) { int t = qubit1; qubit1 = qubit2; qubit2 = t; }
    // util_getTwoQubitDepolarisingFactors (utilities.cpp:949-960); c1 -= c2 as in _subB
    double c1 = 1 - (4 * prob / 5), c2 = 4 * prob / 15, c3 = -(16 * prob / 15);
    int b1 = qubit1 + nKet, b2 = qubit2 + nKet;
    int srt[4] = {qubit1, qubit2, b1, b2};   // already ascending: q1 < q2 < b1 < b2
    Ins ins;
    ins.num = 4;
    for (int i = 0; i < 4; i++) ins.low[i] = ((qidx)1 << srt[i]) - 1;
    qidx numIts = ((qidx)1 << (2 * nKet)) / 16;
    k_depol2<<<qg_blocks(numIts), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numIts, ins, qubit1, qubit2, b1, b2,
                                                                       c1 - c2, c2, 1 + c3);
    qg_note_launch();
    return qg_check_launch("depol2");
}

int qg_dm_oneQubitDephasing(void* amps, int nKet, int qubit, double prob, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit));
    double fac = 1 - (2 * prob);   // util_getOneQubitDephasingFactor (utilities.cpp:918-921)
    return launch_channel1<CH_DEPHASE>(amps, nKet, qubit, fac, 0, 0, 0, stream, "dephase1");
}

int qg_dm_twoQubitDephasing(void* amps, int nKet, int qubit1, int qubit2, double prob, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit1));
    QG_TRY(check_dm(amps, nKet, qubit2));
    if (qubit1 == qubit2) return qg_fail(QG_ERR_ARG, "the two qubits must differ");
    double term = -4 * prob / 3;   // util_getTwoQubitDephasingTerm (utilities.cpp:923-926)
    qidx n = (qidx)1 << (2 * nKet);
    k_dephase2<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, n, qubit1, qubit1 + nKet, qubit2, qubit2 + nKet, 1 + term);
    qg_note_launch();
    return qg_check_launch("dephase2");
}

int qg_dm_oneQubitDamping(void* amps, int nKet, int qubit, double prob, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit));
    double c1 = std::sqrt(1 - prob), c2 = 1 - prob;   // util_getOneQubitDampingFactors (utilities.cpp:977-988)
    return launch_channel1<CH_DAMP>(amps, nKet, qubit, prob, c1, c2, 0, stream, "damping1");
}

int qg_dm_oneQubitPauliChannel(void* amps, int nKet, int qubit, double pX, double pY, double pZ, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit));
    double pI = 1 - pX - pY - pZ;   // localiser.cpp:1575-1585
    // util_getOneQubitPauliChannelFactors (utilities.cpp:962-975)
    double fAA = pI + pZ, fBB = pX + pY, fAB = pI - pZ, fBA = pX - pY;
    return launch_channel1<CH_PAULI>(amps, nKet, qubit, fAA, fBB, fAB, fBA, stream, "pauli_channel1");
}

int qg_dm_multiQubitProjector(void* amps, int nKet, const int* qubits, const int* outcomes, int num, double prob, void* stream) {
    if (nKet < 1 || 2 * nKet > QG_MAX_QUBITS) return qg_fail(QG_ERR_ARG, "density matrix of %d qubits is unsupported", nKet);
    QG_TRY(qg_check_amps(amps, 2 * nKet));
    QG_TRY(qg_check_qubits(nKet, qubits, num, "projector qubits"));
    qidx qmask = 0, retain = 0;
    for (int i = 0; i < num; i++) {
        if (outcomes[i] != 0 && outcomes[i] != 1) return qg_fail(QG_ERR_ARG, "outcome %d is not 0 or 1", outcomes[i]);
        qmask |= (qidx)1 << qubits[i];
        if (outcomes[i]) retain |= (qidx)1 << qubits[i];
    }
    qidx n = (qidx)1 << (2 * nKet);
    k_dm_projector<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, n, nKet, qmask, retain, 1 / prob);
    qg_note_launch();
    return qg_check_launch("dm_projector");
}

}  // extern "C"
