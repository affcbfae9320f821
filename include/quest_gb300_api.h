/*
 * quest_gb300_api.h -- the QuEST v4 API functions of the gate-application path,
 * implemented on the GB300 backend (include/quest_gb300.h).
 *
 * Names, argument order and meaning, and the validation/error behaviour follow
 * QuEST v4.1.0's public headers (quest/include/qureg.h, operations.h,
 * decoherence.h, calculations.h, matrices.h, channels.h, paulis.h, debug.h);
 * each declaration cites the reference definition it mirrors.  Structs keep the
 * reference's field order so a caller's Qureg/CompMatr1/... bytes mean the same
 * thing on both sides.  Every Qureg created here is GPU-resident (gpuAmps) with
 * a host mirror (cpuAmps), as in qureg.cpp:157-168; there is no CPU execution path.
 *
 * Errors: invalid input calls the handler installed with setInputErrorHandler()
 * (default: print and exit(EXIT_FAILURE), as validation.cpp:1073-1096); if a
 * user handler returns, the offending call returns without acting.  Backend
 * (CUDA) failures are reported the same way with function name "qg_backend".
 */
#ifndef QUEST_GB300_API_H
#define QUEST_GB300_API_H

#include <stdint.h>
#include "quest_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef long long int qindex;         /* quest/include/types.h (FLOAT_PRECISION=2) */
typedef double qreal;
typedef qg_cplx qcomp_t;              /* layout of qcomp: (re, im) doubles */
typedef unsigned long long int PAULI_MASK_TYPE;

/* quest/include/qureg.h:49-79 */
typedef struct {
    int isMultithreaded;
    int isGpuAccelerated;
    int isDistributed;
    int rank;
    int numNodes;
    int logNumNodes;
    int isDensityMatrix;
    int numQubits;
    qindex numAmps;
    qindex logNumAmps;
    qindex numAmpsPerNode;
    qindex logNumAmpsPerNode;
    qindex logNumColsPerNode;
    qcomp_t* cpuAmps;
    qcomp_t* gpuAmps;
    qcomp_t* cpuCommBuffer;
    qcomp_t* gpuCommBuffer;
} Qureg;

/* quest/include/matrices.h:68-86 */
typedef struct { int numQubits; qindex numRows; qcomp_t elems[2][2]; } CompMatr1;
typedef struct { int numQubits; qindex numRows; qcomp_t elems[4][4]; } CompMatr2;
/* quest/include/matrices.h:136-154 */
typedef struct { int numQubits; qindex numElems; qcomp_t elems[2]; } DiagMatr1;
typedef struct { int numQubits; qindex numElems; qcomp_t elems[4]; } DiagMatr2;

/* quest/include/matrices.h:90-125 */
typedef struct {
    int numQubits;
    qindex numRows;
    int* isApproxUnitary;
    int* isApproxHermitian;
    int* wasGpuSynced;
    qcomp_t** cpuElems;
    qcomp_t* cpuElemsFlat;
    qcomp_t* gpuElemsFlat;
} CompMatr;

/* quest/include/matrices.h:158-186 */
typedef struct {
    int numQubits;
    qindex numElems;
    int* isApproxUnitary;
    int* isApproxHermitian;
    int* isApproxNonZero;
    int* isStrictlyNonNegative;
    int* wasGpuSynced;
    qcomp_t* cpuElems;
    qcomp_t* gpuElems;
} DiagMatr;

/* quest/include/matrices.h:195-230 */
typedef struct {
    int numQubits;
    qindex numElems;
    int isGpuAccelerated;
    int isMultithreaded;
    int isDistributed;
    qindex numElemsPerNode;
    int* isApproxUnitary;
    int* isApproxHermitian;
    int* isApproxNonZero;
    int* isStrictlyNonNegative;
    int* wasGpuSynced;
    qcomp_t* cpuElems;
    qcomp_t* gpuElems;
} FullStateDiagMatr;

/* quest/include/channels.h:74-101 */
typedef struct {
    int numQubits;
    qindex numRows;
    qcomp_t** cpuElems;
    qcomp_t* cpuElemsFlat;
    qcomp_t* gpuElemsFlat;
    int* wasGpuSynced;
} SuperOp;

typedef struct {
    int numQubits;
    int numMatrices;
    qindex numRows;
    qcomp_t*** matrices;
    SuperOp superop;
    int* isApproxCPTP;
} KrausMap;

/* quest/include/paulis.h:53-60: base-4 digits, 2 bits per qubit */
typedef struct { PAULI_MASK_TYPE lowPaulis; PAULI_MASK_TYPE highPaulis; } PauliStr;

/* quest/include/paulis.h:64-80 */
typedef struct {
    qindex numTerms;
    PauliStr* strings;
    qcomp_t* coeffs;
    int* isApproxHermitian;
} PauliStrSum;

/* environment (quest/include/environment.h:48-56) */
void initQuESTEnv(void);
void initCustomQuESTEnv(int useDistrib, int useGpuAccel, int useMultithread);
void finalizeQuESTEnv(void);
int  isQuESTEnvInit(void);
void syncQuESTEnv(void);                                                          /* environment.cpp -> gpu_sync */
void setInputErrorHandler(void (*callback)(const char* func, const char* msg));  /* debug.h */
void setSeeds(unsigned* seeds, int numSeeds);                                     /* debug.cpp:37 */
void setValidationEpsilon(qreal eps);                                             /* debug.h:98 */
void setValidationEpsilonToDefault(void);
/* the stream every API call of this thread enqueues on (NULL: legacy default stream) */
void setQuESTStream(void* cudaStream);

/* qureg lifecycle (quest/src/api/qureg.cpp:276-333) */
Qureg createQureg(int numQubits);
Qureg createDensityQureg(int numQubits);
Qureg createCustomQureg(int numQubits, int isDensMatr, int useDistrib, int useGpuAccel, int useMultithread);
Qureg createCloneQureg(Qureg qureg);
void  destroyQureg(Qureg qureg);
void  syncQuregToGpu(Qureg qureg);                                               /* qureg.cpp:395 */
void  syncQuregFromGpu(Qureg qureg);                                             /* qureg.cpp:402 */
void  getQuregAmps(qcomp_t* outAmps, Qureg qureg, qindex startInd, qindex numAmps);        /* qureg.cpp:451 */
qcomp_t getQuregAmp(Qureg qureg, qindex index);
/* 1 if the Qureg's host mirror (cpuAmps) is page-locked, so that syncQuregToGpu /
 * syncQuregFromGpu copy at the host link's rate; 0 if the pinned allocation was refused
 * and the mirror is pageable.  No reference counterpart (the reference's mirror is
 * always pageable, qureg.cpp:157-168). */
int   isQuregHostMirrorPinned(Qureg qureg);
/* Applies the Qureg's deferred operations now, on the current stream, without waiting for
 * them.  One-qubit unitaries and channels on density matrices, and one-qubit dense
 * unitaries on statevectors of at least one tensor-core tile of amplitude groups per SM,
 * are deferred and applied together (two or four qubits per pass) when any other call on
 * the Qureg needs its state; every API call that reads or changes the state does that
 * itself, so this is for callers that hand the amplitudes to other code (the C ABI, their
 * own kernels, a stream-ordered copy).  No reference counterpart. */
void  flushQuregDeferredOps(Qureg qureg);

/* initialisations (quest/src/api/initialisations.cpp) */
void initZeroState(Qureg qureg);
void initPlusState(Qureg qureg);
void initClassicalState(Qureg qureg, qindex stateInd);
void initDebugState(Qureg qureg);
void setQuregAmps(Qureg qureg, qindex startInd, qcomp_t* amps, qindex numAmps);             /* :151 */
void setDensityQuregFlatAmps(Qureg qureg, qindex startInd, qcomp_t* amps, qindex numAmps);  /* :169 */

/* matrices and channels (quest/src/api/matrices.cpp, channels.cpp) */
CompMatr createCompMatr(int numQubits);
void destroyCompMatr(CompMatr matr);
void setCompMatrFlat(CompMatr matr, const qcomp_t* rowMajorElems);              /* setCompMatr from a flat array */
void syncCompMatr(CompMatr matr);
DiagMatr createDiagMatr(int numQubits);
void destroyDiagMatr(DiagMatr matr);
void setDiagMatrFlat(DiagMatr matr, const qcomp_t* elems);
void syncDiagMatr(DiagMatr matr);
KrausMap createKrausMap(int numQubits, int numOperators);
void setKrausMapFlat(KrausMap map, const qcomp_t* ops /* numOps x 2^k x 2^k row-major */);
void syncKrausMap(KrausMap map);
void destroyKrausMap(KrausMap map);
PauliStr getPauliStrFromCodes(const int* paulis, const int* indices, int numPaulis);  /* getPauliStr(int*,int*,int), paulis.h:151 */
PauliStrSum createPauliStrSum(PauliStr* strings, qcomp_t* coeffs, qindex numTerms);    /* paulis.cpp:396-417 */
void destroyPauliStrSum(PauliStrSum sum);                                               /* paulis.cpp */

/* operations (quest/src/api/operations.cpp) */
void applyCompMatr1(Qureg qureg, int target, CompMatr1 matrix);                                          /* :81 */
void applyControlledCompMatr1(Qureg qureg, int control, int target, CompMatr1 matrix);                   /* :86 */
void applyMultiControlledCompMatr1(Qureg qureg, int* controls, int numControls, int target, CompMatr1 matrix);
void applyMultiStateControlledCompMatr1(Qureg qureg, int* controls, int* states, int numControls, int target, CompMatr1 matrix); /* :96 */
void applyCompMatr2(Qureg qureg, int target1, int target2, CompMatr2 matrix);                             /* :132 */
void applyControlledCompMatr2(Qureg qureg, int control, int target1, int target2, CompMatr2 matrix);
void applyMultiStateControlledCompMatr2(Qureg qureg, int* controls, int* states, int numControls, int target1, int target2, CompMatr2 matrix); /* :150 */
void applyCompMatr(Qureg qureg, int* targets, int numTargets, CompMatr matrix);                           /* :187 */
void applyMultiStateControlledCompMatr(Qureg qureg, int* controls, int* states, int numControls, int* targets, int numTargets, CompMatr matrix); /* :202 */
void applyDiagMatr1(Qureg qureg, int target, DiagMatr1 matrix);                                          /* :252 */
void applyMultiStateControlledDiagMatr1(Qureg qureg, int* controls, int* states, int numControls, int target, DiagMatr1 matrix); /* :267 */
void applyDiagMatr2(Qureg qureg, int target1, int target2, DiagMatr2 matrix);                             /* :302 */
void applyMultiStateControlledDiagMatr2(Qureg qureg, int* controls, int* states, int numControls, int target1, int target2, DiagMatr2 matrix);
void applyDiagMatr(Qureg qureg, int* targets, int numTargets, DiagMatr matrix);                           /* :357 */
void applyMultiStateControlledDiagMatr(Qureg qureg, int* controls, int* states, int numControls, int* targets, int numTargets, DiagMatr matrix); /* :372 */
void applyDiagMatrPower(Qureg qureg, int* targets, int numTargets, DiagMatr matrix, qcomp_t exponent);    /* :426 */
void applyMultiStateControlledDiagMatrPower(Qureg qureg, int* controls, int* states, int numControls, int* targets, int numTargets, DiagMatr matrix, qcomp_t exponent); /* :468 */
void applyS(Qureg qureg, int target);                                                                    /* :590 */
void applyT(Qureg qureg, int target);                                                                    /* :641 */
void applyHadamard(Qureg qureg, int target);                                                             /* :692 */
void applyMultiStateControlledHadamard(Qureg qureg, int* controls, int* states, int numControls, int target); /* :716 */
void applySwap(Qureg qureg, int qubit1, int qubit2);                                                     /* :754 */
void applyMultiStateControlledSwap(Qureg qureg, int* controls, int* states, int numControls, int qubit1, int qubit2); /* :778 */
void applyPauliX(Qureg qureg, int target);                                                               /* :887 */
void applyPauliY(Qureg qureg, int target);                                                               /* :895 */
void applyPauliZ(Qureg qureg, int target);                                                               /* :903 */
void applyControlledPauliX(Qureg qureg, int control, int target);                                        /* :911 */
void applyControlledPauliZ(Qureg qureg, int control, int target);                                        /* :927 */
void applyPauliStr(Qureg qureg, PauliStr str);                                                           /* :1037 */
void applyMultiStateControlledPauliStr(Qureg qureg, int* controls, int* states, int numControls, PauliStr str); /* :1061 */
void applyRotateX(Qureg qureg, int target, qreal angle);                                                 /* :1211 */
void applyRotateY(Qureg qureg, int target, qreal angle);                                                 /* :1219 */
void applyRotateZ(Qureg qureg, int target, qreal angle);                                                 /* :1227 */
void applyControlledRotateX(Qureg qureg, int control, int target, qreal angle);                          /* :1235 */
void applyControlledRotateY(Qureg qureg, int control, int target, qreal angle);
void applyControlledRotateZ(Qureg qureg, int control, int target, qreal angle);
void applyPauliGadget(Qureg qureg, PauliStr str, qreal angle);                                           /* :1428 */
void applyMultiStateControlledPauliGadget(Qureg qureg, int* controls, int* states, int numControls, PauliStr str, qreal angle); /* :1449 */
void applyPhaseGadget(Qureg qureg, int* targets, int numTargets, qreal angle);                           /* :1508 */
void applyMultiStateControlledPhaseGadget(Qureg qureg, int* controls, int* states, int numControls, int* targets, int numTargets, qreal angle); /* :1532 */
void applyPhaseShift(Qureg qureg, int target, qreal angle);                                              /* :1588 */
void applyTwoQubitPhaseShift(Qureg qureg, int target1, int target2, qreal angle);                        /* :1596 */
void applyMultiQubitPhaseShift(Qureg qureg, int* targets, int numTargets, qreal angle);                  /* :1605 */
void applyPhaseFlip(Qureg qureg, int target);                                                            /* :1631 */
void applyTwoQubitPhaseFlip(Qureg qureg, int target1, int target2);                                      /* :1639 */
void applyQuantumFourierTransform(Qureg qureg, int* targets, int numTargets);                            /* :1934 */
void applyFullQuantumFourierTransform(Qureg qureg);                                                      /* :1955 */
void applyQubitProjector(Qureg qureg, int target, int outcome);                                          /* :1754 */
void applyMultiQubitProjector(Qureg qureg, int* qubits, int* outcomes, int numQubits);                   /* :1766 */
int  applyQubitMeasurement(Qureg qureg, int target);                                                     /* :1796 */
int  applyQubitMeasurementAndGetProb(Qureg qureg, int target, qreal* probability);                       /* :1804 */
qreal applyForcedQubitMeasurement(Qureg qureg, int target, int outcome);                                 /* :1829 */
qindex applyMultiQubitMeasurement(Qureg qureg, int* qubits, int numQubits);                              /* :1848 */
qindex applyMultiQubitMeasurementAndGetProb(Qureg qureg, int* qubits, int numQubits, qreal* probability); /* :1858 */
qreal applyForcedMultiQubitMeasurement(Qureg qureg, int* qubits, int* outcomes, int numQubits);           /* :1893 */

/* decoherence (quest/src/api/decoherence.cpp) */
void mixDephasing(Qureg qureg, int qubit, qreal prob);                                                   /* :31 */
void mixTwoQubitDephasing(Qureg qureg, int qubit1, int qubit2, qreal prob);                              /* :46 */
void mixDepolarising(Qureg qureg, int qubit, qreal prob);                                                /* :61 */
void mixTwoQubitDepolarising(Qureg qureg, int qubit1, int qubit2, qreal prob);                           /* :76 */
void mixDamping(Qureg qureg, int qubit, qreal prob);                                                     /* :91 */
void mixPaulis(Qureg qureg, int qubit, qreal probX, qreal probY, qreal probZ);                           /* :106 */
void mixKrausMap(Qureg qureg, int* qubits, int numQubits, KrausMap map);                                 /* :121 */

/* calculations (quest/src/api/calculations.cpp) */
qreal calcExpecPauliStr(Qureg qureg, PauliStr str);                                                      /* :133 */
/* :146; every term through the batched kernels (several strings per pass over the state) */
qreal calcExpecPauliStrSum(Qureg qureg, PauliStrSum sum);
/* many strings of one Qureg in as few passes as the backend allows (per-term loop of
 * localiser_statevec_calcExpecPauliStrSum, localiser.cpp:2052-2148) */
void  calcExpecPauliStrs(qreal* out, Qureg qureg, const PauliStr* strs, int numStrs);
qreal calcProbOfQubitOutcome(Qureg qureg, int qubit, int outcome);                                       /* :241 */
qreal calcProbOfMultiQubitOutcome(Qureg qureg, int* qubits, int* outcomes, int numQubits);               /* :251 */
void  calcProbsOfAllMultiQubitOutcomes(qreal* outcomeProbs, Qureg qureg, int* qubits, int numQubits);    /* :265 */
qreal calcTotalProb(Qureg qureg);                                                                        /* :278 */
qreal calcPurity(Qureg qureg);                                                                           /* :293 */

/* FullStateDiagMatr: matrices.h:755-923, operations.h:970-990, calculations.h:170-318 */
FullStateDiagMatr createFullStateDiagMatr(int numQubits);
void destroyFullStateDiagMatr(FullStateDiagMatr matr);
void setFullStateDiagMatr(FullStateDiagMatr out, qindex startInd, const qcomp_t* in, qindex numElems);
void syncFullStateDiagMatr(FullStateDiagMatr matr);
void multiplyFullStateDiagMatr(Qureg qureg, FullStateDiagMatr matrix);
void multiplyFullStateDiagMatrPower(Qureg qureg, FullStateDiagMatr matrix, qcomp_t exponent);
void applyFullStateDiagMatr(Qureg qureg, FullStateDiagMatr matrix);
void applyFullStateDiagMatrPower(Qureg qureg, FullStateDiagMatr matrix, qcomp_t exponent);
qreal calcExpecFullStateDiagMatr(Qureg qureg, FullStateDiagMatr matrix);
qreal calcExpecFullStateDiagMatrPower(Qureg qureg, FullStateDiagMatr matrix, qreal exponent);
qcomp_t calcExpecNonHermitianFullStateDiagMatr(Qureg qureg, FullStateDiagMatr matrix);
qcomp_t calcExpecNonHermitianFullStateDiagMatrPower(Qureg qureg, FullStateDiagMatr matrix, qcomp_t exponent);

#ifdef __cplusplus
}
#endif
#endif /* QUEST_GB300_API_H */
