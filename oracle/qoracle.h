/*
 * qoracle.h -- CPU oracle for the QuEST gate-application path.
 *
 * TEST INFRASTRUCTURE ONLY. This library restates, on the host and in FP64,
 * the algorithm of QuEST v4.1.0's OpenMP CPU backend for the gate path
 * (quest/src/cpu/cpu_subroutines.cpp) and the API-level decompositions above it
 * (quest/src/api/operations.cpp, decoherence.cpp, calculations.cpp).
 * It is used by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg as the checker; the product path never calls it.
 *
 * Parity is pinned: tests/golden/ holds final states and reduction results
 * produced by the reference library itself (built from its own sources by
 * `make -C oracle ref`), and tests/test_oracle_golden.py checks this oracle
 * against them.
 *
 * Complex numbers are interleaved (re, im) doubles, the layout of
 * std::complex<double> / QuEST's qcomp at FLOAT_PRECISION=2.
 */
#ifndef QORACLE_H
#define QORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- subroutines on a single-node statevector of 2^numQubits amps ---- */

void orc_sv_swap(double* amps, int nq, const int* ctrls, const int* states, int nc, int t1, int t2);
void orc_sv_dense1(double* amps, int nq, const int* ctrls, const int* states, int nc, int t, const double* m /*2x2 row-major*/);
void orc_sv_dense2(double* amps, int nq, const int* ctrls, const int* states, int nc, int t1, int t2, const double* m /*4x4*/);
void orc_sv_denseK(double* amps, int nq, const int* ctrls, const int* states, int nc, const int* targs, int nt, const double* m, int conj);
void orc_sv_diag1(double* amps, int nq, const int* ctrls, const int* states, int nc, int t, const double* d /*2*/);
void orc_sv_diag2(double* amps, int nq, const int* ctrls, const int* states, int nc, int t1, int t2, const double* d /*4*/);
void orc_sv_diagK(double* amps, int nq, const int* ctrls, const int* states, int nc, const int* targs, int nt, const double* d, int conj, const double* exponent /*NULL = no power*/);
void orc_sv_pauliTensorOrGadget(double* amps, int nq, const int* ctrls, const int* states, int nc,
                                const int* x, int nx, const int* y, int ny, const int* z, int nz,
                                const double* ampFac, const double* pairAmpFac);
void orc_sv_zOrPhaseGadget(double* amps, int nq, const int* ctrls, const int* states, int nc, const int* targs, int nt, const double* fac0, const double* fac1);
void orc_sv_projector(double* amps, int nq, const int* qubits, const int* outcomes, int n, double prob);

/* density matrices: a Choi vector of 2^(2*nKet) amps, column-major (row = low nKet bits) */
void orc_dm_depolarising1(double* amps, int nKet, int qubit, double prob);
void orc_dm_depolarising2(double* amps, int nKet, int q1, int q2, double prob);
void orc_dm_dephasing1(double* amps, int nKet, int qubit, double prob);
void orc_dm_dephasing2(double* amps, int nKet, int q1, int q2, double prob);
void orc_dm_damping1(double* amps, int nKet, int qubit, double prob);
void orc_dm_pauliChannel1(double* amps, int nKet, int qubit, double pX, double pY, double pZ);
void orc_dm_projector(double* amps, int nKet, const int* qubits, const int* outcomes, int n, double prob);
/* FullStateDiagMatr: elems are 2^n complex; exponent NULL = no power */
void orc_sv_allTargDiag(double* amps, int nq, const double* elems, const double* exponent);
void orc_dm_allTargDiag(double* amps, int nKet, const double* elems, const double* exponent, int multiplyOnly);
void orc_sv_expecAllTargDiag(double* out2, const double* amps, int nq, const double* elems, const double* exponent, int useRealPow);
void orc_dm_expecAllTargDiag(double* out2, const double* amps, int nKet, const double* elems, const double* exponent, int useRealPow);

double orc_sv_totalProb(const double* amps, int nq);
double orc_dm_totalProb(const double* amps, int nKet);
double orc_sv_probOfOutcome(const double* amps, int nq, const int* qubits, const int* outcomes, int n);
double orc_dm_probOfOutcome(const double* amps, int nKet, const int* qubits, const int* outcomes, int n);
void   orc_sv_probsOfAllOutcomes(double* out, const double* amps, int nq, const int* qubits, int n);
void   orc_dm_probsOfAllOutcomes(double* out, const double* amps, int nKet, const int* qubits, int n);
double orc_sv_expecZ(const double* amps, int nq, const int* targs, int nt);
void   orc_dm_expecZ(double* out /*2*/, const double* amps, int nKet, const int* targs, int nt);
void   orc_sv_expecPauli(double* out /*2*/, const double* amps, int nq, const int* x, int nx, const int* y, int ny, const int* z, int nz);
void   orc_dm_expecPauli(double* out /*2*/, const double* amps, int nKet, const int* x, int nx, const int* y, int ny, const int* z, int nz);

/* superoperator sum_k conj(K_k) (x) K_k of numOps 2^k x 2^k Kraus matrices (row-major, interleaved) */
void orc_build_superop(double* out /*4^k x 4^k*/, const double* kraus, int numOps, int k);

/* ---- text circuit runner (the API-level decomposition of QuEST v4) ----
 * Runs the circuit text on the state in place. Reductions append one double
 * each to results; measurements append one int each to outcomes.
 * Returns 0 on success, else a negative code (message via orc_last_error()).
 */
int orc_run_circuit(const char* text, int numQubits, int isDensMatr, double* amps,
                    double* results, int maxResults, int* numResults,
                    int* outcomes, int maxOutcomes, int* numOutcomes);
const char* orc_last_error(void);
double orc_last_run_seconds(void);   /* time in the ops of the last run (no state copies) */
void orc_set_num_threads(int n);
int  orc_get_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
