/*
 * ref_harness.cpp -- runs the text circuit format of qoracle.h through the
 * REFERENCE QuEST v4.1.0 library itself (its OpenMP CPU build, FLOAT_PRECISION=2),
 * so that the oracle and the golden fixtures can be pinned to the reference's
 * own outputs.  TEST INFRASTRUCTURE ONLY: built by `make -C oracle ref` into
 * oracle/_ref/ when the reference sources are present; never part of the product.
 *
 * Every op calls the public QuEST API function that the op names
 * (quest/include/operations.h, decoherence.h, calculations.h).
 */
#include "quest/include/modes.h"
#include "quest/include/precision.h"
#include "quest/include/types.h"
#include "quest/include/environment.h"
#include "quest/include/qureg.h"
#include "quest/include/matrices.h"
#include "quest/include/channels.h"
#include "quest/include/paulis.h"
#include "quest/include/operations.h"
#include "quest/include/decoherence.h"
#include "quest/include/calculations.h"
#include "quest/include/initialisations.h"
#include "quest/include/debug.h"

#include <chrono>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

using std::vector;

static std::string g_err;
static double g_lastSeconds = 0;

// seconds spent in the ops of the last ref_run_circuit call (no Qureg creation or copies)
extern "C" double ref_last_run_seconds(void) { return g_lastSeconds; }

static vector<int> rdInts(std::istringstream& is, int k) { vector<int> v(k); for (int i = 0; i < k; i++) is >> v[i]; return v; }
static vector<double> rdDbl(std::istringstream& is, int k) { vector<double> v(k); for (int i = 0; i < k; i++) is >> v[i]; return v; }
static vector<qcomp> toC(const vector<double>& d) { vector<qcomp> c(d.size() / 2); for (size_t i = 0; i < c.size(); i++) c[i] = qcomp(d[2*i], d[2*i+1]); return c; }

static PauliStr pauliOf(const std::string& s) {
    vector<int> codes, inds;
    for (size_t q = 0; q < s.size(); q++) {
        int c = (s[q] == 'X') ? 1 : (s[q] == 'Y') ? 2 : (s[q] == 'Z') ? 3 : 0;
        codes.push_back(c); inds.push_back((int)q);
    }
    return getPauliStr(codes.data(), inds.data(), (int)codes.size());
}

static CompMatr1 m1(const vector<double>& d) { auto c = toC(d); return getCompMatr1(vector<vector<qcomp>>{{c[0], c[1]}, {c[2], c[3]}}); }
static CompMatr2 m2(const vector<double>& d) {
    auto c = toC(d); vector<vector<qcomp>> r(4, vector<qcomp>(4));
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r[i][j] = c[4*i+j];
    return getCompMatr2(r);
}
static CompMatr mK(int k, const vector<double>& d) {
    auto c = toC(d); int dim = 1 << k; vector<vector<qcomp>> r(dim, vector<qcomp>(dim));
    for (int i = 0; i < dim; i++) for (int j = 0; j < dim; j++) r[i][j] = c[dim*i+j];
    CompMatr m = createCompMatr(k); setCompMatr(m, r); return m;
}
static DiagMatr dK(int k, const vector<double>& d) { DiagMatr m = createDiagMatr(k); setDiagMatr(m, toC(d)); return m; }

// REF_HARNESS_GPU=1 builds the same runner against a QuEST built with its GPU backend
// (the drop-in of this repository): GPU-accelerated Quregs, amplitudes moved through the
// host mirror with syncQuregToGpu / syncQuregFromGpu (no-ops for CPU Quregs).
#ifndef REF_HARNESS_GPU
#define REF_HARNESS_GPU 0
#endif

extern "C" int ref_run_circuit(const char* text, int numQubits, int isDensMatr, double* amps,
                               double* results, int maxResults, int* numResults,
                               int* outcomes, int maxOutcomes, int* numOutcomes) {
    static bool envUp = false;
    if (!envUp) { initCustomQuESTEnv(0, REF_HARNESS_GPU, !REF_HARNESS_GPU); envUp = true; }
    Qureg q = createCustomQureg(numQubits, isDensMatr, 0, REF_HARNESS_GPU, !REF_HARNESS_GPU);
    std::memcpy(q.cpuAmps, amps, sizeof(qcomp) * q.numAmps);
    syncQuregToGpu(q);
    vector<double> res; vector<int> outs;
    { unsigned s0 = 0; setSeeds(&s0, 1); }

    std::istringstream lines(text);
    std::string line;
    int rc = 0;
    const auto t0 = std::chrono::steady_clock::now();
    while (std::getline(lines, line)) {
        std::istringstream is(line);
        std::string op;
        if (!(is >> op) || op[0] == '#') continue;
        if (op == "H") { int t; is >> t; applyHadamard(q, t); }
        else if (op == "X") { int t; is >> t; applyPauliX(q, t); }
        else if (op == "Y") { int t; is >> t; applyPauliY(q, t); }
        else if (op == "Z") { int t; is >> t; applyPauliZ(q, t); }
        else if (op == "S") { int t; is >> t; applyS(q, t); }
        else if (op == "T") { int t; is >> t; applyT(q, t); }
        else if (op == "RX") { int t; double a; is >> t >> a; applyRotateX(q, t, a); }
        else if (op == "RY") { int t; double a; is >> t >> a; applyRotateY(q, t, a); }
        else if (op == "RZ") { int t; double a; is >> t >> a; applyRotateZ(q, t, a); }
        else if (op == "CRX") { int c, t; double a; is >> c >> t >> a; applyControlledRotateX(q, c, t, a); }
        else if (op == "CRY") { int c, t; double a; is >> c >> t >> a; applyControlledRotateY(q, c, t, a); }
        else if (op == "CRZ") { int c, t; double a; is >> c >> t >> a; applyControlledRotateZ(q, c, t, a); }
        else if (op == "PS") { int t; double a; is >> t >> a; applyPhaseShift(q, t, a); }
        else if (op == "CPS") { int a, b; double th; is >> a >> b >> th; applyTwoQubitPhaseShift(q, a, b, th); }
        else if (op == "MPS") { int k; is >> k; auto t = rdInts(is, k); double a; is >> a; applyMultiQubitPhaseShift(q, t.data(), k, a); }
        else if (op == "CX") { int c, t; is >> c >> t; applyControlledPauliX(q, c, t); }
        else if (op == "CZ") { int c, t; is >> c >> t; applyControlledPauliZ(q, c, t); }
        else if (op == "SWAP") { int a, b; is >> a >> b; applySwap(q, a, b); }
        else if (op == "CSWAP") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int a, b; is >> a >> b; applyMultiStateControlledSwap(q, c.data(), s.data(), nc, a, b); }
        else if (op == "U1") { int t; is >> t; applyCompMatr1(q, t, m1(rdDbl(is, 8))); }
        else if (op == "CU1") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int t; is >> t; applyMultiStateControlledCompMatr1(q, c.data(), s.data(), nc, t, m1(rdDbl(is, 8))); }
        else if (op == "U2") { int a, b; is >> a >> b; applyCompMatr2(q, a, b, m2(rdDbl(is, 32))); }
        else if (op == "CU2") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int a, b; is >> a >> b; applyMultiStateControlledCompMatr2(q, c.data(), s.data(), nc, a, b, m2(rdDbl(is, 32))); }
        else if (op == "UK") { int k; is >> k; auto t = rdInts(is, k); CompMatr m = mK(k, rdDbl(is, 2 << (2*k))); applyCompMatr(q, t.data(), k, m); destroyCompMatr(m); }
        else if (op == "CUK") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int k; is >> k; auto t = rdInts(is, k); CompMatr m = mK(k, rdDbl(is, 2 << (2*k))); applyMultiStateControlledCompMatr(q, c.data(), s.data(), nc, t.data(), k, m); destroyCompMatr(m); }
        else if (op == "D1") { int t; is >> t; auto c = toC(rdDbl(is, 4)); applyDiagMatr1(q, t, getDiagMatr1(c)); }
        else if (op == "D2") { int a, b; is >> a >> b; auto c = toC(rdDbl(is, 8)); applyDiagMatr2(q, a, b, getDiagMatr2(c)); }
        else if (op == "DK") { int k; is >> k; auto t = rdInts(is, k); DiagMatr m = dK(k, rdDbl(is, 2 << k)); applyDiagMatr(q, t.data(), k, m); destroyDiagMatr(m); }
        else if (op == "CDK") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); int k; is >> k; auto t = rdInts(is, k); DiagMatr m = dK(k, rdDbl(is, 2 << k)); applyMultiStateControlledDiagMatr(q, c.data(), s.data(), nc, t.data(), k, m); destroyDiagMatr(m); }
        else if (op == "DKP") { int k; is >> k; auto t = rdInts(is, k); DiagMatr m = dK(k, rdDbl(is, 2 << k)); auto e = rdDbl(is, 2); applyDiagMatrPower(q, t.data(), k, m, qcomp(e[0], e[1])); destroyDiagMatr(m); }
        else if (op == "PSTR") { std::string s; is >> s; applyPauliStr(q, pauliOf(s)); }
        else if (op == "CPSTR") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); std::string p; is >> p; applyMultiStateControlledPauliStr(q, c.data(), s.data(), nc, pauliOf(p)); }
        else if (op == "PG") { std::string s; double a; is >> s >> a; applyPauliGadget(q, pauliOf(s), a); }
        else if (op == "CPG") { int nc; is >> nc; auto c = rdInts(is, nc); auto s = rdInts(is, nc); std::string p; double a; is >> p >> a; applyMultiStateControlledPauliGadget(q, c.data(), s.data(), nc, pauliOf(p), a); }
        else if (op == "PHG") { int k; is >> k; auto t = rdInts(is, k); double a; is >> a; applyPhaseGadget(q, t.data(), k, a); }
        else if (op == "QFT") { int k; is >> k; auto t = rdInts(is, k); applyQuantumFourierTransform(q, t.data(), k); }
        else if (op == "FQFT") { applyFullQuantumFourierTransform(q); }
        else if (op == "DEPOL") { int a; double p; is >> a >> p; mixDepolarising(q, a, p); }
        else if (op == "DEPOL2") { int a, b; double p; is >> a >> b >> p; mixTwoQubitDepolarising(q, a, b, p); }
        else if (op == "DEPHASE") { int a; double p; is >> a >> p; mixDephasing(q, a, p); }
        else if (op == "DEPHASE2") { int a, b; double p; is >> a >> b >> p; mixTwoQubitDephasing(q, a, b, p); }
        else if (op == "DAMP") { int a; double p; is >> a >> p; mixDamping(q, a, p); }
        else if (op == "PAULIS") { int a; double x, y, z; is >> a >> x >> y >> z; mixPaulis(q, a, x, y, z); }
        else if (op == "KRAUS") {
            int k; is >> k; auto t = rdInts(is, k); int nops; is >> nops;
            auto d = toC(rdDbl(is, nops * (2 << (2*k))));
            int dim = 1 << k;
            vector<vector<vector<qcomp>>> ops(nops, vector<vector<qcomp>>(dim, vector<qcomp>(dim)));
            for (int n = 0; n < nops; n++) for (int i = 0; i < dim; i++) for (int j = 0; j < dim; j++) ops[n][i][j] = d[(n*dim + i)*dim + j];
            KrausMap m = createKrausMap(k, nops); setKrausMap(m, ops);
            mixKrausMap(q, t.data(), k, m); destroyKrausMap(m);
        }
        else if (op == "PROJ") { int k; is >> k; auto a = rdInts(is, k); auto o = rdInts(is, k); applyMultiQubitProjector(q, a.data(), o.data(), k); }
        else if (op == "SEED") { vector<unsigned> s; unsigned v; while (is >> v) s.push_back(v); setSeeds(s.data(), (int)s.size()); }
        else if (op == "MEAS") { int a; is >> a; outs.push_back(applyQubitMeasurement(q, a)); }
        else if (op == "MEASM") {
            int k; is >> k; auto a = rdInts(is, k); qreal p = 0;
            qindex o = applyMultiQubitMeasurementAndGetProb(q, a.data(), k, &p);
            outs.push_back((int)o); res.push_back(p);
        }
        else if (op == "FMEAS") { int a, o; is >> a >> o; res.push_back(applyForcedQubitMeasurement(q, a, o)); }
        else if (op == "FMEASM") { int k; is >> k; auto a = rdInts(is, k); auto o = rdInts(is, k); res.push_back(applyForcedMultiQubitMeasurement(q, a.data(), o.data(), k)); }
        else if (op == "PROBALL") {
            int k; is >> k; auto a = rdInts(is, k);
            vector<qreal> p((size_t)1 << k);
            calcProbsOfAllMultiQubitOutcomes(p.data(), q, a.data(), k);
            for (qreal v : p) res.push_back(v);
        }
        else if (op == "EXPSUM") {
            int T; is >> T;
            vector<PauliStr> strs; vector<qcomp> cs;
            for (int t = 0; t < T; t++) { double cr, ci; std::string ps; is >> cr >> ci >> ps; cs.push_back(qcomp(cr, ci)); strs.push_back(pauliOf(ps)); }
            PauliStrSum sum = createPauliStrSum(strs.data(), cs.data(), (qindex)T);
            res.push_back(calcExpecPauliStrSum(q, sum));
            destroyPauliStrSum(sum);
        }
        else if (op == "TOTALPROB") res.push_back(calcTotalProb(q));
        else if (op == "PURITY") res.push_back(calcPurity(q));
        else if (op == "PROBQ") { int a, o; is >> a >> o; res.push_back(calcProbOfQubitOutcome(q, a, o)); }
        else if (op == "PROBMQ") { int k; is >> k; auto a = rdInts(is, k); auto o = rdInts(is, k); res.push_back(calcProbOfMultiQubitOutcome(q, a.data(), o.data(), k)); }
        else if (op == "EXPEC") { std::string s; is >> s; res.push_back(calcExpecPauliStr(q, pauliOf(s))); }
        else if (op == "FSD") {
            int mult, hasPow; is >> mult >> hasPow;
            vector<double> e = hasPow ? rdDbl(is, 2) : vector<double>{1.0, 0.0};
            qindex dim = (qindex)1 << numQubits;
            FullStateDiagMatr m = createFullStateDiagMatr(numQubits);
            auto d = rdDbl(is, 2 * (size_t)dim);
            setFullStateDiagMatr(m, 0, toC(d).data(), dim);
            qcomp ex(e[0], e[1]);
            if (mult && hasPow) multiplyFullStateDiagMatrPower(q, m, ex);
            else if (mult) multiplyFullStateDiagMatr(q, m);
            else if (hasPow) applyFullStateDiagMatrPower(q, m, ex);
            else applyFullStateDiagMatr(q, m);
            destroyFullStateDiagMatr(m);
        }
        else if (op == "EXPFSD") {
            int kind; is >> kind;
            double p = 1;
            vector<double> e = {1.0, 0.0};
            if (kind == 1) is >> p;
            if (kind == 3) e = rdDbl(is, 2);
            qindex dim = (qindex)1 << numQubits;
            FullStateDiagMatr m = createFullStateDiagMatr(numQubits);
            auto d = rdDbl(is, 2 * (size_t)dim);
            setFullStateDiagMatr(m, 0, toC(d).data(), dim);
            if (kind == 0) res.push_back(calcExpecFullStateDiagMatr(q, m));
            if (kind == 1) res.push_back(calcExpecFullStateDiagMatrPower(q, m, p));
            if (kind == 2) { qcomp v = calcExpecNonHermitianFullStateDiagMatr(q, m); res.push_back(std::real(v)); res.push_back(std::imag(v)); }
            if (kind == 3) { qcomp v = calcExpecNonHermitianFullStateDiagMatrPower(q, m, qcomp(e[0], e[1])); res.push_back(std::real(v)); res.push_back(std::imag(v)); }
            destroyFullStateDiagMatr(m);
        }
        else { g_err = "unknown op " + op; rc = -1; break; }
    }
    syncQuESTEnv();
    g_lastSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    syncQuregFromGpu(q);
    std::memcpy(amps, q.cpuAmps, sizeof(qcomp) * q.numAmps);
    destroyQureg(q);
    if (numResults) *numResults = (int)res.size();
    if (numOutcomes) *numOutcomes = (int)outs.size();
    for (int i = 0; i < (int)res.size() && i < maxResults; i++) results[i] = res[i];
    for (int i = 0; i < (int)outs.size() && i < maxOutcomes; i++) outcomes[i] = outs[i];
    return rc;
}

extern "C" const char* ref_last_error(void) { return g_err.c_str(); }
