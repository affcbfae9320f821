// Drop-in replacement for QuEST v4.1.0's quest/src/gpu/gpu_subroutines.cpp.
//
// Built INSIDE a QuEST tree (FLOAT_PRECISION=2, COMPILE_CUDA=1, COMPILE_MPI=0,
// COMPILE_CUQUANTUM=0) in place of that file, it keeps every signature of
// quest/src/gpu/gpu_subroutines.hpp -- so accelerator.cpp's function-pointer
// tables bind unchanged -- and forwards each call on the single-GPU gate path to
// the C ABI of include/quest_gb300.h.  The template parameters that the
// reference uses for compile-time unrolling (NumCtrls, NumTargs, ApplyConj,
// HasPower) become runtime arguments of the backend.  Routines that only serve
// distribution (the _subB/_subC buffer variants, buffer packing) or lie outside
// the gate path report an internal error if reached.
#include "quest/include/modes.h"
#include "quest/include/types.h"
#include "quest/include/qureg.h"
#include "quest/include/paulis.h"
#include "quest/include/matrices.h"

#include "quest/src/core/errors.hpp"
#include "quest/src/core/accelerator.hpp"
#include "quest/src/gpu/gpu_subroutines.hpp"

#include "quest_gb300.h"

#include <string>
#include <vector>

using std::vector;

static_assert(sizeof(qcomp) == sizeof(qg_cplx), "the backend needs FLOAT_PRECISION=2 (qcomp = two doubles)");

namespace {

inline void ok(int rc, const char* caller) {
    if (rc != QG_OK) error_cudaCallFailed(qg_get_last_error(), "qg_*", caller, __FILE__, __LINE__);
}
inline const qg_cplx* C(const qcomp* p) { return reinterpret_cast<const qg_cplx*>(p); }
inline qg_cplx C(qcomp c) { return qg_cplx{std::real(c), std::imag(c)}; }
inline const int* P(const vector<int>& v) { return v.empty() ? nullptr : v.data(); }
inline int nq(const Qureg& q) { return (int)q.logNumAmpsPerNode; }   // qubits of the local amplitude vector
[[noreturn]] void unsupported(const char* func) {
    std::string m = std::string(func) + " is not provided by the GB300 single-GPU backend";
    error_cudaCallFailed(m.c_str(), func, func, __FILE__, __LINE__);
    throw 0;   // not reached: error_* exits
}

}  // namespace

qcomp gpu_statevec_getAmp_sub(Qureg qureg, qindex ind) {
    qcomp v;
    ok(qg_copy_d2h(&v, qureg.gpuAmps + ind, sizeof(qcomp), nullptr), __func__);
    return v;
}

void gpu_densmatr_setAmpsToPauliStrSum_sub(Qureg, PauliStrSum) { unsupported(__func__); }
void gpu_fullstatediagmatr_setElemsToPauliStrSum(FullStateDiagMatr, PauliStrSum) { unsupported(__func__); }

template <int NumQubits> qindex gpu_statevec_packAmpsIntoBuffer(Qureg, vector<int>, vector<int>) { unsupported(__func__); }
qindex gpu_statevec_packPairSummedAmpsIntoBuffer(Qureg, int, int, int, int) { unsupported(__func__); }
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(qindex, gpu_statevec_packAmpsIntoBuffer, (Qureg, vector<int>, vector<int>))

// ---------------------------------------------------------------- swaps

template <int NumCtrls>
void gpu_statevec_anyCtrlSwap_subA(Qureg q, vector<int> c, vector<int> s, int t1, int t2) {
    ok(qg_sv_anyCtrlSwap(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), t1, t2, nullptr), __func__);
}
template <int NumCtrls> void gpu_statevec_anyCtrlSwap_subB(Qureg, vector<int>, vector<int>) { unsupported(__func__); }
template <int NumCtrls> void gpu_statevec_anyCtrlSwap_subC(Qureg, vector<int>, vector<int>, int, int) { unsupported(__func__); }
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlSwap_subA, (Qureg, vector<int>, vector<int>, int, int))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlSwap_subB, (Qureg, vector<int>, vector<int>))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlSwap_subC, (Qureg, vector<int>, vector<int>, int, int))

// ---------------------------------------------------------------- dense matrices

template <int NumCtrls>
void gpu_statevec_anyCtrlOneTargDenseMatr_subA(Qureg q, vector<int> c, vector<int> s, int t, CompMatr1 m) {
    ok(qg_sv_anyCtrlOneTargDenseMatr(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), t, C(&m.elems[0][0]), nullptr), __func__);
}
template <int NumCtrls> void gpu_statevec_anyCtrlOneTargDenseMatr_subB(Qureg, vector<int>, vector<int>, qcomp, qcomp) { unsupported(__func__); }
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlOneTargDenseMatr_subA, (Qureg, vector<int>, vector<int>, int, CompMatr1))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlOneTargDenseMatr_subB, (Qureg, vector<int>, vector<int>, qcomp, qcomp))

template <int NumCtrls>
void gpu_statevec_anyCtrlTwoTargDenseMatr_sub(Qureg q, vector<int> c, vector<int> s, int t1, int t2, CompMatr2 m) {
    ok(qg_sv_anyCtrlTwoTargDenseMatr(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), t1, t2, C(&m.elems[0][0]), nullptr), __func__);
}
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlTwoTargDenseMatr_sub, (Qureg, vector<int>, vector<int>, int, int, CompMatr2))

template <int NumCtrls, int NumTargs, bool ApplyConj>
void gpu_statevec_anyCtrlAnyTargDenseMatr_sub(Qureg q, vector<int> c, vector<int> s, vector<int> t, CompMatr m) {
    ok(qg_sv_anyCtrlAnyTargDenseMatr(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), P(t), (int)t.size(),
                                     C(m.cpuElemsFlat), ApplyConj ? 1 : 0, nullptr), __func__);
}
INSTANTIATE_CONJUGABLE_FUNC_OPTIMISED_FOR_NUM_CTRLS_AND_TARGS(void, gpu_statevec_anyCtrlAnyTargDenseMatr_sub, (Qureg, vector<int>, vector<int>, vector<int>, CompMatr))

// ---------------------------------------------------------------- diagonal matrices

template <int NumCtrls>
void gpu_statevec_anyCtrlOneTargDiagMatr_sub(Qureg q, vector<int> c, vector<int> s, int t, DiagMatr1 m) {
    ok(qg_sv_anyCtrlOneTargDiagMatr(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), t, C(m.elems), nullptr), __func__);
}
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlOneTargDiagMatr_sub, (Qureg, vector<int>, vector<int>, int, DiagMatr1))

template <int NumCtrls>
void gpu_statevec_anyCtrlTwoTargDiagMatr_sub(Qureg q, vector<int> c, vector<int> s, int t1, int t2, DiagMatr2 m) {
    ok(qg_sv_anyCtrlTwoTargDiagMatr(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), t1, t2, C(m.elems), nullptr), __func__);
}
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevec_anyCtrlTwoTargDiagMatr_sub, (Qureg, vector<int>, vector<int>, int, int, DiagMatr2))

template <int NumCtrls, int NumTargs, bool ApplyConj, bool HasPower>
void gpu_statevec_anyCtrlAnyTargDiagMatr_sub(Qureg q, vector<int> c, vector<int> s, vector<int> t, DiagMatr m, qcomp exponent) {
    qg_cplx ex = C(exponent);
    ok(qg_sv_anyCtrlAnyTargDiagMatr(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), P(t), (int)t.size(), C(m.cpuElems),
                                    ApplyConj ? 1 : 0, HasPower ? &ex : nullptr, nullptr), __func__);
}
INSTANTIATE_EXPONENTIABLE_CONJUGABLE_FUNC_OPTIMISED_FOR_NUM_CTRLS_AND_TARGS(void, gpu_statevec_anyCtrlAnyTargDiagMatr_sub, (Qureg, vector<int>, vector<int>, vector<int>, DiagMatr, qcomp))

template <bool HasPower> void gpu_statevec_allTargDiagMatr_sub(Qureg q, FullStateDiagMatr m, qcomp e) {
    ok(qg_sv_allTargDiagMatr(q.gpuAmps, nq(q), m.gpuElems, C(e), HasPower, nullptr), __func__);
}
template <bool HasPower, bool MultiplyOnly> void gpu_densmatr_allTargDiagMatr_sub(Qureg q, FullStateDiagMatr m, qcomp e) {
    ok(qg_dm_allTargDiagMatr(q.gpuAmps, q.numQubits, m.gpuElems, C(e), HasPower, MultiplyOnly, nullptr), __func__);
}
template void gpu_statevec_allTargDiagMatr_sub<true>(Qureg, FullStateDiagMatr, qcomp);
template void gpu_statevec_allTargDiagMatr_sub<false>(Qureg, FullStateDiagMatr, qcomp);
template void gpu_densmatr_allTargDiagMatr_sub<true, true>(Qureg, FullStateDiagMatr, qcomp);
template void gpu_densmatr_allTargDiagMatr_sub<true, false>(Qureg, FullStateDiagMatr, qcomp);
template void gpu_densmatr_allTargDiagMatr_sub<false, true>(Qureg, FullStateDiagMatr, qcomp);
template void gpu_densmatr_allTargDiagMatr_sub<false, false>(Qureg, FullStateDiagMatr, qcomp);

// ---------------------------------------------------------------- Pauli tensors and gadgets

template <int NumCtrls, int NumTargs>
void gpu_statevector_anyCtrlPauliTensorOrGadget_subA(Qureg q, vector<int> c, vector<int> s, vector<int> x, vector<int> y, vector<int> z,
                                                     qcomp ampFac, qcomp pairAmpFac) {
    ok(qg_sv_anyCtrlPauliTensorOrGadget(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), P(x), (int)x.size(), P(y), (int)y.size(),
                                        P(z), (int)z.size(), C(ampFac), C(pairAmpFac), nullptr), __func__);
}
template <int NumCtrls>
void gpu_statevector_anyCtrlPauliTensorOrGadget_subB(Qureg, vector<int>, vector<int>, vector<int>, vector<int>, vector<int>, qcomp, qcomp, qindex) { unsupported(__func__); }
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS_AND_TARGS(void, gpu_statevector_anyCtrlPauliTensorOrGadget_subA, (Qureg, vector<int>, vector<int>, vector<int>, vector<int>, vector<int>, qcomp, qcomp))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevector_anyCtrlPauliTensorOrGadget_subB, (Qureg, vector<int>, vector<int>, vector<int>, vector<int>, vector<int>, qcomp, qcomp, qindex))

template <int NumCtrls>
void gpu_statevector_anyCtrlAnyTargZOrPhaseGadget_sub(Qureg q, vector<int> c, vector<int> s, vector<int> t, qcomp fac0, qcomp fac1) {
    ok(qg_sv_anyCtrlAnyTargZOrPhaseGadget(q.gpuAmps, nq(q), P(c), P(s), (int)c.size(), P(t), (int)t.size(), C(fac0), C(fac1), nullptr), __func__);
}
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_CTRLS(void, gpu_statevector_anyCtrlAnyTargZOrPhaseGadget_sub, (Qureg, vector<int>, vector<int>, vector<int>, qcomp, qcomp))

// ---------------------------------------------------------------- qureg combination (outside the gate path)

void gpu_statevec_setQuregToSuperposition_sub(qcomp, Qureg, qcomp, Qureg, qcomp, Qureg) { unsupported(__func__); }
void gpu_densmatr_mixQureg_subA(qreal, Qureg, qreal, Qureg) { unsupported(__func__); }
void gpu_densmatr_mixQureg_subB(qreal, Qureg, qreal, Qureg) { unsupported(__func__); }
void gpu_densmatr_mixQureg_subC(qreal, Qureg, qreal) { unsupported(__func__); }

// ---------------------------------------------------------------- decoherence

void gpu_densmatr_oneQubitDephasing_subA(Qureg q, int qubit, qreal p) { ok(qg_dm_oneQubitDephasing(q.gpuAmps, q.numQubits, qubit, p, nullptr), __func__); }
void gpu_densmatr_oneQubitDephasing_subB(Qureg, int, qreal) { unsupported(__func__); }
void gpu_densmatr_twoQubitDephasing_subA(Qureg q, int a, int b, qreal p) { ok(qg_dm_twoQubitDephasing(q.gpuAmps, q.numQubits, a, b, p, nullptr), __func__); }
void gpu_densmatr_twoQubitDephasing_subB(Qureg q, int a, int b, qreal p) { ok(qg_dm_twoQubitDephasing(q.gpuAmps, q.numQubits, a, b, p, nullptr), __func__); }
void gpu_densmatr_oneQubitDepolarising_subA(Qureg q, int qubit, qreal p) { ok(qg_dm_oneQubitDepolarising(q.gpuAmps, q.numQubits, qubit, p, nullptr), __func__); }
void gpu_densmatr_oneQubitDepolarising_subB(Qureg, int, qreal) { unsupported(__func__); }
// the localiser calls _subA then _subB on one node (localiser.cpp:1535-1556); the backend fuses
// both into one pass, run at _subA, so _subB has nothing left to do
void gpu_densmatr_twoQubitDepolarising_subA(Qureg q, int a, int b, qreal p) { ok(qg_dm_twoQubitDepolarising(q.gpuAmps, q.numQubits, a, b, p, nullptr), __func__); }
void gpu_densmatr_twoQubitDepolarising_subB(Qureg, int, int, qreal) {}
void gpu_densmatr_twoQubitDepolarising_subC(Qureg, int, int, qreal) { unsupported(__func__); }
void gpu_densmatr_twoQubitDepolarising_subD(Qureg, int, int, qreal) { unsupported(__func__); }
void gpu_densmatr_twoQubitDepolarising_subE(Qureg, int, int, qreal) { unsupported(__func__); }
void gpu_densmatr_twoQubitDepolarising_subF(Qureg, int, int, qreal) { unsupported(__func__); }
void gpu_densmatr_oneQubitPauliChannel_subA(Qureg q, int qubit, qreal pI, qreal pX, qreal pY, qreal pZ) {
    (void)pI;   // the backend infers pI = 1 - pX - pY - pZ, as the localiser does
    ok(qg_dm_oneQubitPauliChannel(q.gpuAmps, q.numQubits, qubit, pX, pY, pZ, nullptr), __func__);
}
void gpu_densmatr_oneQubitPauliChannel_subB(Qureg, int, qreal, qreal, qreal, qreal) { unsupported(__func__); }
void gpu_densmatr_oneQubitDamping_subA(Qureg q, int qubit, qreal p) { ok(qg_dm_oneQubitDamping(q.gpuAmps, q.numQubits, qubit, p, nullptr), __func__); }
void gpu_densmatr_oneQubitDamping_subB(Qureg, int, qreal) { unsupported(__func__); }
void gpu_densmatr_oneQubitDamping_subC(Qureg, int, qreal) { unsupported(__func__); }
void gpu_densmatr_oneQubitDamping_subD(Qureg, int, qreal) { unsupported(__func__); }

template <int NumTargs> void gpu_densmatr_partialTrace_sub(Qureg, Qureg, vector<int>, vector<int>) { unsupported(__func__); }
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(void, gpu_densmatr_partialTrace_sub, (Qureg, Qureg, vector<int>, vector<int>))

// ---------------------------------------------------------------- probabilities

qreal gpu_statevec_calcTotalProb_sub(Qureg q) { double v = 0; ok(qg_sv_calcTotalProb(q.gpuAmps, nq(q), &v, nullptr), __func__); return v; }
qreal gpu_densmatr_calcTotalProb_sub(Qureg q) { double v = 0; ok(qg_dm_calcTotalProb(q.gpuAmps, q.numQubits, &v, nullptr), __func__); return v; }

template <int NumQubits>
qreal gpu_statevec_calcProbOfMultiQubitOutcome_sub(Qureg q, vector<int> qs, vector<int> os) {
    double v = 0;
    ok(qg_sv_calcProbOfMultiQubitOutcome(q.gpuAmps, nq(q), P(qs), P(os), (int)qs.size(), &v, nullptr), __func__);
    return v;
}
template <int NumQubits>
qreal gpu_densmatr_calcProbOfMultiQubitOutcome_sub(Qureg q, vector<int> qs, vector<int> os) {
    double v = 0;
    ok(qg_dm_calcProbOfMultiQubitOutcome(q.gpuAmps, q.numQubits, P(qs), P(os), (int)qs.size(), &v, nullptr), __func__);
    return v;
}
template <int NumQubits>
void gpu_statevec_calcProbsOfAllMultiQubitOutcomes_sub(qreal* out, Qureg q, vector<int> qs) {
    ok(qg_sv_calcProbsOfAllMultiQubitOutcomes(out, q.gpuAmps, nq(q), P(qs), (int)qs.size(), nullptr), __func__);
}
template <int NumQubits>
void gpu_densmatr_calcProbsOfAllMultiQubitOutcomes_sub(qreal* out, Qureg q, vector<int> qs) {
    ok(qg_dm_calcProbsOfAllMultiQubitOutcomes(out, q.gpuAmps, q.numQubits, P(qs), (int)qs.size(), nullptr), __func__);
}
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(qreal, gpu_statevec_calcProbOfMultiQubitOutcome_sub, (Qureg, vector<int>, vector<int>))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(qreal, gpu_densmatr_calcProbOfMultiQubitOutcome_sub, (Qureg, vector<int>, vector<int>))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(void, gpu_statevec_calcProbsOfAllMultiQubitOutcomes_sub, (qreal*, Qureg, vector<int>))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(void, gpu_densmatr_calcProbsOfAllMultiQubitOutcomes_sub, (qreal*, Qureg, vector<int>))

// ---------------------------------------------------------------- inner products (outside the gate path)

qcomp gpu_statevec_calcInnerProduct_sub(Qureg, Qureg) { unsupported(__func__); }
qreal gpu_densmatr_calcHilbertSchmidtDistance_sub(Qureg, Qureg) { unsupported(__func__); }
template <bool Conj> qcomp gpu_densmatr_calcFidelityWithPureState_sub(Qureg, Qureg) { unsupported(__func__); }
template qcomp gpu_densmatr_calcFidelityWithPureState_sub<true>(Qureg, Qureg);
template qcomp gpu_densmatr_calcFidelityWithPureState_sub<false>(Qureg, Qureg);

// ---------------------------------------------------------------- expectation values

qreal gpu_statevec_calcExpecAnyTargZ_sub(Qureg q, vector<int> t) {
    double v = 0;
    ok(qg_sv_calcExpecAnyTargZ(q.gpuAmps, nq(q), P(t), (int)t.size(), &v, nullptr), __func__);
    return v;
}
qcomp gpu_densmatr_calcExpecAnyTargZ_sub(Qureg q, vector<int> t) {
    qg_cplx v;
    ok(qg_dm_calcExpecAnyTargZ(q.gpuAmps, q.numQubits, P(t), (int)t.size(), &v, nullptr), __func__);
    return qcomp(v.re, v.im);
}
qcomp gpu_statevec_calcExpecPauliStr_subA(Qureg q, vector<int> x, vector<int> y, vector<int> z) {
    qg_cplx v;
    ok(qg_sv_calcExpecPauliStr(q.gpuAmps, nq(q), P(x), (int)x.size(), P(y), (int)y.size(), P(z), (int)z.size(), &v, nullptr), __func__);
    return qcomp(v.re, v.im);
}
qcomp gpu_statevec_calcExpecPauliStr_subB(Qureg, vector<int>, vector<int>, vector<int>) { unsupported(__func__); }
qcomp gpu_densmatr_calcExpecPauliStr_sub(Qureg q, vector<int> x, vector<int> y, vector<int> z) {
    qg_cplx v;
    ok(qg_dm_calcExpecPauliStr(q.gpuAmps, q.numQubits, P(x), (int)x.size(), P(y), (int)y.size(), P(z), (int)z.size(), &v, nullptr), __func__);
    return qcomp(v.re, v.im);
}
template <bool HasPower, bool UseRealPow> qcomp gpu_statevec_calcExpecFullStateDiagMatr_sub(Qureg q, FullStateDiagMatr m, qcomp e) {
    qg_cplx v{0, 0};
    ok(qg_sv_calcExpecFullStateDiagMatr(q.gpuAmps, nq(q), m.gpuElems, C(e), HasPower, UseRealPow, &v, nullptr), __func__);
    return qcomp(v.re, v.im);
}
template <bool HasPower, bool UseRealPow> qcomp gpu_densmatr_calcExpecFullStateDiagMatr_sub(Qureg q, FullStateDiagMatr m, qcomp e) {
    qg_cplx v{0, 0};
    ok(qg_dm_calcExpecFullStateDiagMatr(q.gpuAmps, q.numQubits, m.gpuElems, C(e), HasPower, UseRealPow, &v, nullptr), __func__);
    return qcomp(v.re, v.im);
}
template qcomp gpu_statevec_calcExpecFullStateDiagMatr_sub<true, true>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_statevec_calcExpecFullStateDiagMatr_sub<true, false>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_statevec_calcExpecFullStateDiagMatr_sub<false, true>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_statevec_calcExpecFullStateDiagMatr_sub<false, false>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_densmatr_calcExpecFullStateDiagMatr_sub<true, true>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_densmatr_calcExpecFullStateDiagMatr_sub<true, false>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_densmatr_calcExpecFullStateDiagMatr_sub<false, true>(Qureg, FullStateDiagMatr, qcomp);
template qcomp gpu_densmatr_calcExpecFullStateDiagMatr_sub<false, false>(Qureg, FullStateDiagMatr, qcomp);

// ---------------------------------------------------------------- projectors

template <int NumQubits>
void gpu_statevec_multiQubitProjector_sub(Qureg q, vector<int> qs, vector<int> os, qreal prob) {
    ok(qg_sv_multiQubitProjector(q.gpuAmps, nq(q), P(qs), P(os), (int)qs.size(), prob, nullptr), __func__);
}
template <int NumQubits>
void gpu_densmatr_multiQubitProjector_sub(Qureg q, vector<int> qs, vector<int> os, qreal prob) {
    ok(qg_dm_multiQubitProjector(q.gpuAmps, q.numQubits, P(qs), P(os), (int)qs.size(), prob, nullptr), __func__);
}
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(void, gpu_statevec_multiQubitProjector_sub, (Qureg, vector<int>, vector<int>, qreal))
INSTANTIATE_FUNC_OPTIMISED_FOR_NUM_TARGS(void, gpu_densmatr_multiQubitProjector_sub, (Qureg, vector<int>, vector<int>, qreal))

// ---------------------------------------------------------------- state initialisation

void gpu_statevec_initUniformState_sub(Qureg q, qcomp amp) { ok(qg_sv_initUniformState(q.gpuAmps, nq(q), C(amp), nullptr), __func__); }
void gpu_statevec_initDebugState_sub(Qureg q) { ok(qg_sv_initDebugState(q.gpuAmps, nq(q), nullptr), __func__); }
void gpu_statevec_initUnnormalisedUniformlyRandomPureStateAmps_sub(Qureg) { unsupported(__func__); }
