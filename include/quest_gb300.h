/*
 * quest_gb300.h -- C ABI of the GB300 (sm_103a) gate-application backend.
 *
 * Each entry point replaces one GPU backend function of QuEST v4.1.0, named in
 * its comment (file:line within the QuEST project).  A QuEST build reaches these
 * through a thin shim that keeps the signatures of quest/src/gpu/gpu_subroutines.hpp
 * and quest/src/gpu/gpu_config.hpp (quest_gb300/shim/); the localiser and the
 * accelerator above it are unchanged.
 *
 * Conventions
 *  - amps: DEVICE pointer to interleaved complex amplitudes, FP64 (qg_cplx, the
 *    layout of qcomp at FLOAT_PRECISION=2) unless the name ends in _f32.
 *  - numQubits: qubits of the amplitude vector; for a density matrix routine
 *    (qg_dm_*) numKetQubits is the Qureg's qubit count and the vector holds
 *    4^numKetQubits amps (column-major Choi vector: row = low bits).
 *  - ctrls / ctrlStates / targs / qubits: HOST int arrays.  ctrlStates may be
 *    NULL, meaning every control must be 1 (the reference's default,
 *    quest/src/core/localiser.cpp:58-67).
 *  - matrices and factors: HOST pointers, read during the call.
 *  - stream: a cudaStream_t (NULL = the legacy default stream).  Amplitude
 *    routines are asynchronous like the reference's kernel launches; reductions
 *    return a host value and therefore synchronise the stream, as the reference's
 *    Thrust reductions do.
 *  - Every function returns QG_OK (0) or a negative QG_ERR_* code; the message
 *    of the last failure on the calling thread is in qg_get_last_error().
 */
#ifndef QUEST_GB300_H
#define QUEST_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } qg_cplx;   /* = qcomp at FLOAT_PRECISION=2 */
typedef struct { float re, im; } qg_cplxf;   /* = qcomp at FLOAT_PRECISION=1 */

#define QG_OK            0
#define QG_ERR_CUDA     -1   /* a CUDA runtime call failed (reference: error_cudaCallFailed, errors.cpp:630) */
#define QG_ERR_ARG      -2   /* invalid argument (qubit out of range, overlapping qubits, bad size ...) */
#define QG_ERR_OOM      -3   /* device allocation failed (reference: gpu_allocArray returns nullptr, gpu_config.cpp:407-412) */
#define QG_ERR_TIMEOUT  -4   /* a bounded device-side wait gave up */
#define QG_ERR_NOTSUP   -5   /* configuration not supported by this build */

const char* qg_get_last_error(void);
const char* qg_get_error_string(int code);
int  qg_get_version(void);                 /* 100*major + minor */

/* ------------------------------------------------------------------ runtime
 * replaces quest/src/gpu/gpu_config.hpp (gpu_config.cpp:124-663)            */

int qg_init(int device);                                   /* gpu_bindLocalGPUsToNodes (gpu_config.cpp:332) + queries */
int qg_get_num_devices(int* out);                          /* gpu_getNumberOfLocalGpus (gpu_config.cpp:124) */
int qg_get_device_info(int* numSMs, int64_t* totalMem, int64_t* freeMem, int* ccMajor, int* ccMinor);
/* The context's L2 fetch-granularity hint (cudaLimitMaxL2FetchGranularity): 0, 32, 64
 * or 128 bytes.  qg_init sets 32: gates that visit every other short run of amplitudes
 * then fetch only the sectors they use.  The limit belongs to the device's primary
 * context, so it applies to every library of the host process on that device until the
 * process exits.  qg_init keeps the value it found; qg_restore_l2_fetch_granularity puts
 * that value back on the current device (a host application that shares the context and
 * wants its own setting calls it after qg_init).  No reference counterpart (the
 * reference leaves the limit alone). */
int qg_set_l2_fetch_granularity(int bytes);
int qg_get_l2_fetch_granularity(int* bytes);
int qg_restore_l2_fetch_granularity(void);
int qg_alloc(void** out, int64_t numBytes);                /* gpu_allocArray (gpu_config.cpp:399-421) */
int qg_free(void* ptr);                                    /* gpu_deallocArray (gpu_config.cpp:424-436) */
int qg_copy_h2d(void* dst, const void* src, int64_t numBytes, void* stream);   /* gpu_copyCpuToGpu (gpu_config.cpp:535) */
int qg_copy_d2h(void* dst, const void* src, int64_t numBytes, void* stream);   /* gpu_copyGpuToCpu (gpu_config.cpp:449-533) */
int qg_copy_d2d(void* dst, const void* src, int64_t numBytes, void* stream);   /* gpu_copyArray (gpu_config.cpp:521-532) */
int qg_sync(void);                                         /* gpu_sync (gpu_config.cpp:382-390) */
int qg_stream_sync(void* stream);
int qg_get_cache_size(int64_t* out);                       /* getGpuCacheSize (quest/src/api/debug.cpp:180) */
int qg_clear_cache(void);                                  /* gpu_clearCache (gpu_config.cpp:665) */
int qg_get_launch_count(int64_t* out);                     /* kernels launched by this library so far */
/* Streams and events for host harnesses (no reference counterpart; the reference runs
 * everything on the legacy default stream): a non-blocking stream, so that work on it
 * never waits implicitly for the legacy stream; a stream that waits for an event
 * recorded on another, so that copies on one stream and gates on another can be
 * overlapped and still ordered. */
int qg_stream_create(void** out);
int qg_stream_destroy(void* stream);
int qg_stream_wait_event(void* stream, void* event);
/* CUDA events on the launching stream, for timing kernels from a host harness */
int qg_event_create(void** out);
int qg_event_destroy(void* event);
int qg_event_record(void* event, void* stream);
int qg_event_elapsed_ms(void* start, void* stop, float* ms); /* waits for `stop` */
/* FP64 fused multiply-adds per second this GPU sustains (a short probe kernel);
 * the issue rate that bounds the general complex FP64 gates */
int qg_measure_fp64_fma_rate(double* fmaPerSecond);
/* How general complex FP64 gates form their products (no counterpart in the reference,
 * whose GPU kernels use FP64 FMAs):
 *   0 (default) block-floating 60-bit fixed point on the integer pipes: each amplitude
 *     pair shares one exponent; per output the error is below 2^-54 of (largest |amp| in
 *     the pair) x (largest |matrix entry|), the order of IEEE FP64's own bound; pairs
 *     holding Inf/NaN or with results outside the normal range are evaluated in FP64;
 *   1 IEEE FP64 fused multiply-adds throughout.
 * Applies to one-target dense matrices (applyCompMatr1, Hadamard, rotations and their
 * controlled forms) and one-target diagonals (phase gates, controlled phases);
 * process-wide. */
int qg_set_fp64_products(int mode);
int qg_get_fp64_products(int* mode);
/* Three- and four-target dense gates in product mode 0 (no counterpart in the reference):
 *   1 (default) on the bf16 tensor cores as exact 8-bit slices when the register holds at
 *     least one tile of 128 amplitude groups per SM: each group's inputs share one exponent,
 *     are cut into seven signed 8-bit digits and multiplied with the matrix's eight digits,
 *     every digit product and sum exact (FP32 sums of integers below 2^22), and combined in
 *     int64; per output the error is below (2^(K+1) + 2) 2^-53 of (largest |amp| in the
 *     group) x (largest |matrix entry|), as for mode 0's integer form; groups holding Inf/NaN
 *     or with extreme scales are evaluated in FP64;
 *   2 the same at every register size;
 *   0 the integer-pipe fixed-point kernels.
 * A launch whose bounded wait runs out sets the tensor-core error flag (qg_tc_get_error_flag);
 * the next such launch returns QG_ERR_TIMEOUT.  Process-wide. */
int qg_set_tensor_slices(int mode);
int qg_get_tensor_slices(int* mode);
/* CUDA events around every tensor-core dense launch, for a caller's roofline: enable = 1
 * starts recording (dropping earlier records), 0 stops; _read waits for the recorded
 * launches and returns their durations in ms (numOut = how many were recorded, of which
 * the first maxOut are written). */
int qg_dense_tc_timing(int enable);
int qg_dense_tc_timing_read(float* msOut, int maxOut, int* numOut);

/* ------------------------------------------------------------------ launch-shape autotuner
 * (no counterpart in the reference, whose launch sizes are fixed formulas,
 * gpu_subroutines.cpp getNumBlocks)  Kernel 0 = the one-target dense kernel, 1 = the
 * one-target diagonal kernel, 2 = the two-target dense kernel, all with fixed-point
 * products.  A shape is (items per thread per iteration -- for kernel 2, groups in
 * flight per thread -- , threads per block) from {(1,256), (1,128), (2,256), (2,128)};
 * default (1,256). */
#define QG_TUNE_KERNEL_DENSE1 0
#define QG_TUNE_KERNEL_DIAG1 1
#define QG_TUNE_KERNEL_DENSE2 2
int qg_set_kernel_shape(int kernel, int pairsPerThread, int threadsPerBlock);
int qg_get_kernel_shape(int kernel, int* pairsPerThread, int* threadsPerBlock);
/* times every candidate of every tunable kernel on a scratch register of numQubits
 * (16 B x 2^numQubits of device memory for the duration of the call) and keeps the
 * fastest per kernel; msOut[kernel * 4 + candidate] receives milliseconds per launch,
 * candidates in the order above */
int qg_autotune_fp64(int numQubits, double* msOut, int maxOut, int* numOut);
/* text file: "qg-tune 1", then "<device name> <kernel> <ppt> <threads>" per line;
 * load applies only the lines for the current device's name */
int qg_tune_save(const char* path);
int qg_tune_load(const char* path, int* numApplied);

/* ------------------------------------------------------------------ initialisation
 * replaces gpu_statevec_initUniformState_sub / initDebugState_sub
 * (gpu_subroutines.hpp:189-193; gpu_thrust.cuh:1053-1070)                    */

int qg_sv_initUniformState(void* amps, int numQubits, qg_cplx amp, void* stream);
int qg_sv_initClassicalState(void* amps, int numQubits, int64_t index, void* stream);   /* initZeroState / initClassicalState */
int qg_sv_initDebugState(void* amps, int numQubits, void* stream);

/* ------------------------------------------------------------------ statevector gates
 * (a density matrix's Choi vector is passed here too, with numQubits = 2*numKetQubits) */

/* gpu_statevec_anyCtrlSwap_subA (gpu_subroutines.hpp:50; gpu_subroutines.cpp:197-222) */
int qg_sv_anyCtrlSwap(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                      int targ1, int targ2, void* stream);

/* gpu_statevec_anyCtrlOneTargDenseMatr_subA (gpu_subroutines.hpp:59; gpu_subroutines.cpp:286-315)
 * matr: 2x2 row-major */
int qg_sv_anyCtrlOneTargDenseMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                  int targ, const qg_cplx* matr, void* stream);

/* gpu_statevec_anyCtrlTwoTargDenseMatr_sub (gpu_subroutines.hpp:62; gpu_subroutines.cpp:354-385)
 * matr: 4x4 row-major; matrix index bit 0 is targ1 */
int qg_sv_anyCtrlTwoTargDenseMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                  int targ1, int targ2, const qg_cplx* matr, void* stream);

/* gpu_statevec_anyCtrlAnyTargDenseMatr_sub<NumCtrls,NumTargs,ApplyConj> (gpu_subroutines.hpp:64;
 * gpu_subroutines.cpp:396-507).  matr: 2^k x 2^k row-major HOST elements; matrix
 * index bit i is targs[i].  applyConj conjugates every element. */
int qg_sv_anyCtrlAnyTargDenseMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                  const int* targs, int numTargs, const qg_cplx* matr, int applyConj, void* stream);
/* A set of controlled phases: every amplitude whose index has all bits of masks[f] set is
 * multiplied by factors[f] (|factors[f]| = 1), f < num <= 32, in one pass (the phases
 * commute); statevectors of at least 8 qubits.  Products in fixed point; the API defers
 * CPhase, CZ, phase shifts, S, T and Z on large statevectors and applies them with this. */
int qg_sv_phaseSet(void* amps, int numQubits, const int64_t* masks, const qg_cplx* factors, int num, void* stream);
/* One step of the quantum Fourier transform on contiguous targets lowTarget..target
 * (lowTarget + numLowBits == target): the Hadamard on `target`, then, for every amplitude
 * whose bit `target` is set, the phase exp(i pi L / 2^numLowBits) with L = (index >>
 * lowTarget) & (2^numLowBits - 1) -- the target's controlled phases of
 * applyQuantumFourierTransform (operations.cpp:1934-1952), one pass instead of
 * numLowBits + 1.  numLowBits <= 40.  Fixed-point products (Inf/NaN and extreme scales in FP64). */
int qg_sv_qftStep(void* amps, int numQubits, int target, int lowTarget, int numLowBits, void* stream);
/* The QFT steps of `target` and then `target` - 1 on contiguous targets from qubit 0
 * (qg_sv_qftStep(target, 0, target) followed by qg_sv_qftStep(target - 1, 0, target - 1)) in
 * one pass over quadruples of amplitudes: 2 * target + 1 gates of
 * applyQuantumFourierTransform (operations.cpp:1934-1949).  1 <= target <= 40. */
int qg_sv_qftTwoSteps(void* amps, int numQubits, int target, void* stream);
/* The QFT steps of `target`, `target` - 1 and `target` - 2 on contiguous targets from qubit 0
 * in one pass over octets of amplitudes (3 * target gates of applyQuantumFourierTransform).
 * 2 <= target <= 8 or 10 <= target <= 40. */
int qg_sv_qftThreeSteps(void* amps, int numQubits, int target, void* stream);
/* The closing swaps of a quantum Fourier transform on the targets 0..numBits-1 (qubit j
 * with qubit numBits-1-j, j < numBits/2: applySwap in applyQuantumFourierTransform,
 * operations.cpp:1950-1952) as one in-place pass: every amplitude index has its low numBits
 * bits reversed.  10 <= numBits <= numQubits.  A permutation: bit-exact. */
int qg_sv_reverseLowBits(void* amps, int numQubits, int numBits, void* stream);

/* gpu_statevec_anyCtrlOneTargDiagMatr_sub (gpu_subroutines.hpp:71; gpu_subroutines.cpp:516-572) */
int qg_sv_anyCtrlOneTargDiagMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                 int targ, const qg_cplx* elems, void* stream);

/* gpu_statevec_anyCtrlTwoTargDiagMatr_sub (gpu_subroutines.hpp:73; gpu_subroutines.cpp:584-641)
 * elems index = (bit targ2) * 2 + (bit targ1) */
int qg_sv_anyCtrlTwoTargDiagMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                 int targ1, int targ2, const qg_cplx* elems, void* stream);

/* gpu_statevec_anyCtrlAnyTargDiagMatr_sub<C,T,ApplyConj,HasPower> (gpu_subroutines.hpp:75;
 * gpu_subroutines.cpp:653-709).  exponent == NULL (or 1+0i) means no power; the power
 * is applied before the conjugation, as in the reference. */
int qg_sv_anyCtrlAnyTargDiagMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                 const int* targs, int numTargs, const qg_cplx* elems, int applyConj,
                                 const qg_cplx* exponent, void* stream);

/* gpu_statevector_anyCtrlPauliTensorOrGadget_subA<C,T> (gpu_subroutines.hpp:86;
 * gpu_subroutines.cpp:779-820): amp pairs (iA, iA ^ maskXY) mixed as
 * a'A = ampFac*aA + pairAmpFac*i^#Y*sign(iB)*aB */
int qg_sv_anyCtrlPauliTensorOrGadget(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                     const int* targsX, int numX, const int* targsY, int numY, const int* targsZ, int numZ,
                                     qg_cplx ampFac, qg_cplx pairAmpFac, void* stream);

/* gpu_statevector_anyCtrlAnyTargZOrPhaseGadget_sub<C> (gpu_subroutines.hpp:90;
 * gpu_subroutines.cpp:864-887): a *= (parity of targs even) ? fac0 : fac1 */
int qg_sv_anyCtrlAnyTargZOrPhaseGadget(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                       const int* targs, int numTargs, qg_cplx fac0, qg_cplx fac1, void* stream);

/* gpu_statevec_multiQubitProjector_sub<N> (gpu_subroutines.hpp:183; gpu_thrust.cuh:1014-1030) */
int qg_sv_multiQubitProjector(void* amps, int numQubits, const int* qubits, const int* outcomes, int numQubitsProj,
                              double prob, void* stream);

/* ------------------------------------------------------------------ density-matrix channels */

/* gpu_densmatr_multiQubitProjector_sub<N> (gpu_subroutines.hpp:184; gpu_thrust.cuh:1033-1048) */
int qg_dm_multiQubitProjector(void* amps, int numKetQubits, const int* qubits, const int* outcomes, int numQubitsProj,
                              double prob, void* stream);
/* gpu_densmatr_oneQubitDepolarising_subA (gpu_subroutines.hpp:114; gpu_subroutines.cpp:1069-1086) */
int qg_dm_oneQubitDepolarising(void* amps, int numKetQubits, int qubit, double prob, void* stream);
/* gpu_densmatr_twoQubitDepolarising_subA + subB (gpu_subroutines.hpp:117-118), fused into one pass */
int qg_dm_twoQubitDepolarising(void* amps, int numKetQubits, int qubit1, int qubit2, double prob, void* stream);
/* gpu_densmatr_oneQubitDephasing_subA (gpu_subroutines.hpp:108) */
int qg_dm_oneQubitDephasing(void* amps, int numKetQubits, int qubit, double prob, void* stream);
/* gpu_densmatr_twoQubitDephasing_subA (gpu_subroutines.hpp:111) */
int qg_dm_twoQubitDephasing(void* amps, int numKetQubits, int qubit1, int qubit2, double prob, void* stream);
/* gpu_densmatr_oneQubitDamping_subA (gpu_subroutines.hpp:127) */
int qg_dm_oneQubitDamping(void* amps, int numKetQubits, int qubit, double prob, void* stream);
/* gpu_densmatr_oneQubitPauliChannel_subA (gpu_subroutines.hpp:124); probI = 1 - pX - pY - pZ */
int qg_dm_oneQubitPauliChannel(void* amps, int numKetQubits, int qubit, double probX, double probY, double probZ, void* stream);

/* ------------------------------------------------------------------ reductions (FP64 accumulation,
 * fixed reduction tree: the same input gives the same bits on every run) */

/* gpu_statevec_calcTotalProb_sub (gpu_subroutines.hpp:144; gpu_thrust.cuh:745-764) */
int qg_sv_calcTotalProb(const void* amps, int numQubits, double* out, void* stream);
/* gpu_densmatr_calcTotalProb_sub (gpu_subroutines.hpp:145; gpu_thrust.cuh:767-785) */
int qg_dm_calcTotalProb(const void* amps, int numKetQubits, double* out, void* stream);
/* gpu_statevec_calcProbOfMultiQubitOutcome_sub<N> (gpu_subroutines.hpp:147; gpu_thrust.cuh:788-805) */
int qg_sv_calcProbOfMultiQubitOutcome(const void* amps, int numQubits, const int* qubits, const int* outcomes, int num,
                                      double* out, void* stream);
/* gpu_densmatr_calcProbOfMultiQubitOutcome_sub<N> (gpu_subroutines.hpp:148; gpu_thrust.cuh:808-832) */
int qg_dm_calcProbOfMultiQubitOutcome(const void* amps, int numKetQubits, const int* qubits, const int* outcomes, int num,
                                      double* out, void* stream);
/* gpu_statevec_calcProbsOfAllMultiQubitOutcomes_sub<N> (gpu_subroutines.hpp:150; gpu_kernels.cuh:1145-1171);
 * deterministic (no atomics on the probabilities). outProbs: HOST array of 2^num */
int qg_sv_calcProbsOfAllMultiQubitOutcomes(double* outProbs, const void* amps, int numQubits, const int* qubits, int num,
                                           void* stream);
/* gpu_densmatr_calcProbsOfAllMultiQubitOutcomes_sub<N> (gpu_subroutines.hpp:150; gpu_subroutines.cpp:1550-1580):
 * the histogram of the diagonal, deterministic like the statevector form */
int qg_dm_calcProbsOfAllMultiQubitOutcomes(double* outProbs, const void* amps, int numKetQubits, const int* qubits, int num,
                                           void* stream);
/* ------------------------------------------------------------------ all-target diagonals (FullStateDiagMatr)
 * elems: DEVICE array of 2^n complex (n ket qubits for a density matrix), 16-byte aligned.
 * With hasPower the elements are raised to `exponent` (complex pow, exp(w log z)). */
/* gpu_statevec_allTargDiagMatr_sub (gpu_subroutines.hpp:76; gpu_thrust.cuh:729-742): a_i *= d_i^p */
int qg_sv_allTargDiagMatr(void* amps, int numQubits, const void* elems, qg_cplx exponent, int hasPower, void* stream);
/* gpu_densmatr_allTargDiagMatr_sub (gpu_subroutines.hpp:78; gpu_kernels.cuh:556-588):
 * rho[r][c] *= d_r^p, and unless multiplyOnly also *= conj(d_c^p) */
int qg_dm_allTargDiagMatr(void* amps, int numKetQubits, const void* elems, qg_cplx exponent, int hasPower, int multiplyOnly,
                          void* stream);
/* gpu_statevec_calcExpecFullStateDiagMatr_sub (gpu_subroutines.hpp:176; gpu_thrust.cuh:977-988):
 * sum_i f(d_i) |a_i|^2 with f = d^p (complex pow) or, with useRealPow, re(d)^re(p) */
int qg_sv_calcExpecFullStateDiagMatr(const void* amps, int numQubits, const void* elems, qg_cplx exponent, int hasPower,
                                     int useRealPow, qg_cplx* out, void* stream);
/* gpu_densmatr_calcExpecFullStateDiagMatr_sub (gpu_subroutines.hpp:177; gpu_thrust.cuh:991-1008): sum_r f(d_r) rho[r][r] */
int qg_dm_calcExpecFullStateDiagMatr(const void* amps, int numKetQubits, const void* elems, qg_cplx exponent, int hasPower,
                                     int useRealPow, qg_cplx* out, void* stream);

/* gpu_statevec_calcExpecAnyTargZ_sub (gpu_subroutines.hpp:169; gpu_thrust.cuh:888-900) */
int qg_sv_calcExpecAnyTargZ(const void* amps, int numQubits, const int* targs, int numTargs, double* out, void* stream);
/* gpu_densmatr_calcExpecAnyTargZ_sub (gpu_subroutines.hpp:170; gpu_thrust.cuh:903-915) */
int qg_dm_calcExpecAnyTargZ(const void* amps, int numKetQubits, const int* targs, int numTargs, qg_cplx* out, void* stream);
/* gpu_statevec_calcExpecPauliStr_subA (gpu_subroutines.hpp:173; gpu_thrust.cuh:918-932) */
int qg_sv_calcExpecPauliStr(const void* amps, int numQubits, const int* targsX, int numX, const int* targsY, int numY,
                            const int* targsZ, int numZ, qg_cplx* out, void* stream);
/* gpu_densmatr_calcExpecPauliStr_sub (gpu_subroutines.hpp:175; gpu_thrust.cuh:953-974) */
int qg_dm_calcExpecPauliStr(const void* amps, int numKetQubits, const int* targsX, int numX, const int* targsY, int numY,
                            const int* targsZ, int numZ, qg_cplx* out, void* stream);
/* Many Pauli strings in ONE pass over a statevector (batched calcExpecPauliStr, the
 * per-term loop of localiser_statevec_calcExpecPauliStrSum, localiser.cpp:2052-2148).
 * Strings are given as (maskXY, maskYZ, numY) triples; out[s] is string s's value. */
int qg_sv_calcExpecPauliStrBatch(const void* amps, int numQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                 const int* numsY, int numStrings, qg_cplx* out, void* stream);
/* the density-matrix form (no one-pass counterpart in the reference, which runs one
 * gpu_densmatr_calcExpecPauliStr_sub per string, gpu_subroutines.hpp:174): masks on the
 * ket qubits; up to 16 strings per pass over the 2^N columns */
int qg_dm_calcExpecPauliStrBatch(const void* amps, int numKetQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                 const int* numsY, int numStrings, qg_cplx* out, void* stream);

/* The same batched Pauli expectation values, for callers that cannot allocate
 * device or pinned memory during the call (their HBM is reserved up front by
 * another allocator, or they cannot afford cudaMalloc's implicit
 * synchronisation).  No counterpart in the reference.  Allocates nothing: its
 * scratch is a fixed device array inside the library (about 264 KiB per GPU
 * that loads the library, held until exit).  At most QG_NOALLOC_MAX_STRINGS
 * strings per call; more is rejected with QG_ERR_ARG.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and should
 * come before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race. */
#define QG_NOALLOC_MAX_STRINGS 64
int qg_sv_calcExpecPauliStrBatch_noalloc(const void* amps, int numQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                         const int* numsY, int numStrings, qg_cplx* out, void* stream);

/* ------------------------------------------------------------------ FP32 fused-block path
 * A circuit of small dense unitaries is fused on the host into blocks of at most
 * k <= 5 qubits (each block's matrix formed in FP64), then applied to an FP32
 * (complex64) statevector one block per pass.  A block is the few-target dense
 * primitive of gpu_statevec_anyCtrlAnyTargDenseMatr_sub (gpu_kernels.cuh:296-356)
 * in FP32; 5-qubit blocks can run on the tensor cores as 3xTF32 GEMM tiles. */

typedef struct qg_circuit qg_circuit;

int qg_circuit_create(qg_circuit** out, int numQubits);
int qg_circuit_destroy(qg_circuit* circuit);
/* appends a dense unitary on 1..5 qubits; matr row-major 2^k x 2^k, index bit i <-> targs[i] */
int qg_circuit_add_matrix(qg_circuit* circuit, const int* targs, int numTargs, const qg_cplx* matr);
/* appends numGates 1- or 2-qubit unitaries at once: gate g acts on numTargs[g] qubits
 * targs[2g], targs[2g+1] with the row-major matrix in the first 4^numTargs[g] entries of
 * matrs[16g .. 16g+15] */
int qg_circuit_add_matrices(qg_circuit* circuit, int numGates, const int* numTargs, const int* targs, const qg_cplx* matrs);
/* greedy fusion into blocks of at most maxFusedQubits (1..5) qubits; matrices upload at the first apply */
int qg_circuit_fuse(qg_circuit* circuit, int maxFusedQubits);
int qg_circuit_get_num_gates(const qg_circuit* circuit, int* out);
int qg_circuit_get_num_blocks(const qg_circuit* circuit, int* out);
/* block i: its ascending targets and (if matr != NULL) its 2^k x 2^k FP64 matrix */
int qg_circuit_get_block(const qg_circuit* circuit, int i, int* targs, int* numTargs, qg_cplx* matr);
/* impl: 0 automatic (tensor cores for 5-qubit blocks on >= 12 qubits), 1 SIMT FP32, 2 tensor cores,
 * 3 tensor cores in the self-test of their failure path (no operand buffer is ever signalled
 * full: every 5-qubit block launch gives up after about 2 s and leaves the register untouched).
 * Asynchronous.  A tensor-core launch whose bounded wait runs out sets the device's error flag;
 * the next qg_sv32_apply_circuit or qg_graph_launch on that device returns QG_ERR_TIMEOUT for
 * it (and clears the flag) before launching anything.  Callers that need the outcome of their
 * own launches synchronise the stream and read qg_tc_get_error_flag. */
int qg_sv32_apply_circuit(qg_circuit* circuit, void* amps32, int numQubits, int impl, void* stream);
/* the current device's flag: 1 if a tensor-core launch gave up a bounded wait since it was
 * last cleared (a host read of mapped memory: no copy, no synchronisation) */
int qg_tc_get_error_flag(int* out);
int qg_tc_clear_error_flag(void);
/* Self-test of that failure path: one launch (12..20 qubits, five targets) in which no
 * operand buffer is ever signalled full, so the kernel's bounded waits run out (about
 * 2 s).  flagOut: the error flag it left (1 expected, then cleared); secondsOut: the
 * launch's wall time; unchangedOut: 1 if the scratch register was left untouched. */
int qg_tc_selftest_timeout(int numQubits, const int* targs, int* flagOut, double* secondsOut, int* unchangedOut);

/* Fusion autotuner (no counterpart in the reference): times the circuit fused at each
 * width k from its widest gate to 5 with the SIMT kernel, and at k = 5 with the
 * tensor-core kernel (>= 12 qubits), on a scratch FP32 register of the circuit's size
 * (8 B x 2^n for the duration of the call).  Leaves the circuit fused at the fastest
 * width, with that kernel used by applies that pass impl = 0; a later qg_circuit_fuse
 * clears the preference.  Candidate i (in the order tried, at most maxOut reported) is
 * (candK[i], candImpl[i]) and took msOut[i] ms per circuit; any output may be NULL. */
int qg_circuit_autotune(qg_circuit* circuit, int* bestK, int* bestImpl, int* candK, int* candImpl, double* msOut,
                        int maxOut, int* numOut);

/* CUDA graph of one application of a fused circuit to one FP32 register (no
 * counterpart in the reference).  The graph holds the register's address and the
 * circuit's device copy: it stays valid while both live and the circuit is not
 * re-fused.  Launching it replays every block kernel with one host call. */
typedef struct qg_graph qg_graph;
int qg_circuit_graph_create(qg_circuit* circuit, void* amps32, int numQubits, int impl, qg_graph** out);
int qg_graph_launch(qg_graph* graph, void* stream);
int qg_graph_get_num_kernels(const qg_graph* graph, int* out);
int qg_graph_destroy(qg_graph* graph);

int qg_sv32_initUniformState(void* amps32, int numQubits, qg_cplxf amp, void* stream);
int qg_sv32_initClassicalState(void* amps32, int numQubits, int64_t index, void* stream);
int qg_sv_convert_f64_to_f32(void* dst32, const void* src64, int numQubits, void* stream);
int qg_sv_convert_f32_to_f64(void* dst64, const void* src32, int numQubits, void* stream);
/* FP64-accumulated reductions of an FP32 statevector */
int qg_sv32_calcTotalProb(const void* amps32, int numQubits, double* out, void* stream);
/* scales the state so that its FP64-summed total probability is targetProb (> 0); stays on
   `stream` (no host round trip).  Removes the norm drift of FP32 products after a unitary circuit. */
int qg_sv32_normalise(void* amps32, int numQubits, double targetProb, void* stream);
int qg_sv32_calcExpecPauliStrBatch(const void* amps32, int numQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                   const int* numsY, int numStrings, qg_cplx* out, void* stream);

/* ------------------------------------------------------------------ continuous-batching server
 * Requests are fused circuits on FP32 registers starting in |0>, each returning up to
 * 16 Pauli expectation values.  Registers of <= 14 qubits run whole in shared memory,
 * one thread block per request, all admitted small requests in one launch; larger
 * registers are admitted against an HBM byte budget (sub-allocated from one arena) and
 * run on a pool of non-blocking streams.  poll() is one non-blocking scheduling step. */

typedef struct qg_server qg_server;

/* impl: the block kernel choice of qg_sv32_apply_circuit (0..3) for the large registers */
int qg_server_create(qg_server** out, int64_t hbmBudgetBytes, int maxInFlight, int impl);
int qg_server_destroy(qg_server* server);
/* queues a request (the fused circuit must outlive it); returns its id */
int qg_server_submit(qg_server* server, qg_circuit* circuit, const int64_t* masksXY, const int64_t* masksYZ,
                     const int* numsY, int numStrings, int64_t* id);
/* retires finished requests, admits queued ones in arrival order as slots and memory free up, launches their work */
int qg_server_poll(qg_server* server, int* numDone);
/* *done = 1 once finished; values = the request's expectation values.  When every gate of
   the circuit is unitary (max|U^dagger U - I| <= 1e-10) they are <P>/<psi|psi>, with the norm
   of the final FP32 state summed in FP64; otherwise <psi|P|psi> unnormalised.  A finished
   request one of whose tensor-core launches gave up a bounded wait returns QG_ERR_TIMEOUT
   (with *done = 1 and no values); each request has a timeout word of its own, so the others
   in flight are unaffected. */
int qg_server_result(qg_server* server, int64_t id, double* values, int* done);
int qg_server_release(qg_server* server, int64_t id);
/* the client went away: a queued request is dropped at once (its circuit is no longer
 * needed); one on the GPU is dropped when it completes, its slot and memory returned
 * then; a finished one is released.  The id is unknown afterwards. */
int qg_server_cancel(qg_server* server, int64_t id);
int qg_server_stats(qg_server* server, int64_t* queued, int64_t* inFlight, int64_t* hbmInUse, int64_t* finished);

#ifdef __cplusplus
}
#endif
#endif /* QUEST_GB300_H */
