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

// cpu_densmatr_oneQubitDepolarising_subA (cpu_subroutines.cpp:1183-1215)
__global__ void k_depol1(double2* __restrict__ a, qidx numIts, int ket, int bra, double cAA, double cBB, double cAB) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i00 = insert_two_zeros(n, ket, bra);
    qidx i01 = i00 | ((qidx)1 << ket), i10 = i00 | ((qidx)1 << bra), i11 = i01 | ((qidx)1 << bra);
    double2 a00 = ld_amp(a + i00), a01 = ld_amp(a + i01), a10 = ld_amp(a + i10), a11 = ld_amp(a + i11);
    st_amp(a + i00, lin2(cAA, a00, cBB, a11));
    st_amp(a + i01, cscale(cAB, a01));
    st_amp(a + i10, cscale(cAB, a10));
    st_amp(a + i11, lin2(cAA, a11, cBB, a00));
}

// cpu_densmatr_oneQubitPauliChannel_subA (cpu_subroutines.cpp:1455-1496)
__global__ void k_pauli_channel1(double2* __restrict__ a, qidx numIts, int ket, int bra, double fAA, double fBB, double fAB, double fBA) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i00 = insert_two_zeros(n, ket, bra);
    qidx i01 = i00 | ((qidx)1 << ket), i10 = i00 | ((qidx)1 << bra), i11 = i01 | ((qidx)1 << bra);
    double2 a00 = ld_amp(a + i00), a01 = ld_amp(a + i01), a10 = ld_amp(a + i10), a11 = ld_amp(a + i11);
    st_amp(a + i00, lin2(fAA, a00, fBB, a11));
    st_amp(a + i01, lin2(fAB, a01, fBA, a10));
    st_amp(a + i10, lin2(fAB, a10, fBA, a01));
    st_amp(a + i11, lin2(fAA, a11, fBB, a00));
}

// cpu_densmatr_oneQubitDamping_subA (cpu_subroutines.cpp:1550-1575)
__global__ void k_damping1(double2* __restrict__ a, qidx numIts, int ket, int bra, double prob, double c1, double c2) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i00 = insert_two_zeros(n, ket, bra);
    qidx i01 = i00 | ((qidx)1 << ket), i10 = i00 | ((qidx)1 << bra), i11 = i01 | ((qidx)1 << bra);
    double2 a00 = ld_amp(a + i00), a01 = ld_amp(a + i01), a10 = ld_amp(a + i10), a11 = ld_amp(a + i11);
    st_amp(a + i00, make_double2(fma(prob, a11.x, a00.x), fma(prob, a11.y, a00.y)));
    st_amp(a + i01, cscale(c1, a01));
    st_amp(a + i10, cscale(c1, a10));
    st_amp(a + i11, cscale(c2, a11));
}

// cpu_densmatr_oneQubitDephasing_subA (cpu_subroutines.cpp:1072-1105): only the two
// off-diagonal amplitudes of each group change.
__global__ void k_dephase1(double2* __restrict__ a, qidx numIts, int ket, int bra, double fac) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i00 = insert_two_zeros(n, ket, bra);
    qidx i01 = i00 | ((qidx)1 << ket), i10 = i00 | ((qidx)1 << bra);
    st_amp(a + i01, cscale(fac, ld_amp(a + i01)));
    st_amp(a + i10, cscale(fac, ld_amp(a + i10)));
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
    double cAA = 1 - (2 * prob / 3), cBB = 2 * prob / 3, cAB = 1 - (4 * prob / 3);
    qidx numIts = ((qidx)1 << (2 * nKet)) / 4;
    k_depol1<<<qg_blocks(numIts), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numIts, qubit, qubit + nKet, cAA, cBB, cAB);
    qg_note_launch();
    return qg_check_launch("depol1");
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
    qidx numIts = ((qidx)1 << (2 * nKet)) / 4;
    k_dephase1<<<qg_blocks(numIts), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numIts, qubit, qubit + nKet, fac);
    qg_note_launch();
    return qg_check_launch("dephase1");
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
    qidx numIts = ((qidx)1 << (2 * nKet)) / 4;
    k_damping1<<<qg_blocks(numIts), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numIts, qubit, qubit + nKet, prob, c1, c2);
    qg_note_launch();
    return qg_check_launch("damping1");
}

int qg_dm_oneQubitPauliChannel(void* amps, int nKet, int qubit, double pX, double pY, double pZ, void* stream) {
    QG_TRY(check_dm(amps, nKet, qubit));
    double pI = 1 - pX - pY - pZ;   // localiser.cpp:1575-1585
    // util_getOneQubitPauliChannelFactors (utilities.cpp:962-975)
    double fAA = pI + pZ, fBB = pX + pY, fAB = pI - pZ, fBA = pX - pY;
    qidx numIts = ((qidx)1 << (2 * nKet)) / 4;
    k_pauli_channel1<<<qg_blocks(numIts), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, numIts, qubit, qubit + nKet, fAA, fBB, fAB, fBA);
    qg_note_launch();
    return qg_check_launch("pauli_channel1");
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
