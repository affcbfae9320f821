// Host check of the API's deferral of statevector gates (quest_gb300/csrc/quest_api.cpp):
// the API file is compiled here with the pass kernels it calls replaced by plain CPU loops
// (one-, two- and k-target dense matrices, phase sets), and random layers of one-qubit
// unitaries (on every qubit, or on a subset), two-qubit phase shifts on disjoint pairs (or on
// a few pairs), three-qubit and one-qubit phase shifts, on 8 to 14 qubits, go through the
// public calls (applyCompMatr1, applyTwoQubitPhaseShift, applyMultiQubitPhaseShift,
// applyPhaseShift, flushQuregDeferredOps).  The state must equal the gate-by-gate product to
// 1e-12 of its largest amplitude, and the circuits shaped like the benchmark layers (a gate
// on every qubit, phases on disjoint pairs covering all of them) must take no phase pass and
// ceil(n / 4) passes per layer, the last partial group staying pending to the next layer
// when it has one or two qubits.  Prints one line starting "OK" when every case passes.
#include "quest_api.cpp"
#include <random>
typedef std::complex<double> cx;
static long g_passes = 0, g_phasePasses = 0;
static void applyK(cx* a, int n, const int* t, int k, const qcomp_t* m) {
    const long long N = 1LL << n;
    const int D = 1 << k;
    std::vector<cx> in(D), out(D);
    for (long long i = 0; i < N; i++) {
        bool base = true;
        for (int b = 0; b < k; b++) base = base && !((i >> t[b]) & 1);
        if (!base) continue;
        for (int j = 0; j < D; j++) {
            long long idx = i;
            for (int b = 0; b < k; b++) if ((j >> b) & 1) idx |= 1LL << t[b];
            in[j] = a[idx];
        }
        for (int r = 0; r < D; r++) {
            cx acc = 0;
            for (int c = 0; c < D; c++) acc += cx(m[r * D + c].re, m[r * D + c].im) * in[c];
            out[r] = acc;
        }
        for (int j = 0; j < D; j++) {
            long long idx = i;
            for (int b = 0; b < k; b++) if ((j >> b) & 1) idx |= 1LL << t[b];
            a[idx] = out[j];
        }
    }
}
extern "C" {
int qg_sv_anyCtrlOneTargDenseMatr(void* amps, int n, const int*, const int*, int nc, int t, const qg_cplx* m, void*) {
    if (nc) { printf("FAIL: unexpected controls\n"); exit(2); }
    g_passes++; applyK((cx*)amps, n, &t, 1, (const qcomp_t*)m); return 0;
}
int qg_sv_anyCtrlTwoTargDenseMatr(void* amps, int n, const int*, const int*, int nc, int t1, int t2, const qg_cplx* m, void*) {
    if (nc) { printf("FAIL: unexpected controls\n"); exit(2); }
    int t[2] = {t1, t2}; g_passes++; applyK((cx*)amps, n, t, 2, (const qcomp_t*)m); return 0;
}
int qg_sv_anyCtrlAnyTargDenseMatr(void* amps, int n, const int*, const int*, int nc, const int* t, int k, const qg_cplx* m, int conj, void*) {
    if (nc || conj) { printf("FAIL: unexpected controls\n"); exit(2); }
    g_passes++; applyK((cx*)amps, n, t, k, (const qcomp_t*)m); return 0;
}
int qg_sv_phaseSet(void* amps, int n, const int64_t* masks, const qg_cplx* f, int num, void*) {
    g_passes++; g_phasePasses++;
    cx* a = (cx*)amps;
    for (long long i = 0; i < (1LL << n); i++)
        for (int k = 0; k < num; k++) if ((i & masks[k]) == masks[k]) a[i] *= cx(f[k].re, f[k].im);
    return 0;
}
}
int qg_fp64_products_mode() { return 0; }
bool qg_dense_tc_wanted(long long) { return true; }
int main() {
    g_envInit = true;
    std::mt19937_64 g(7);
    std::normal_distribution<double> nd;
    int bad = 0;
    for (int trial = 0; trial < 40; trial++) {
        const int n = 8 + trial % 7;   // 8..14 qubits
        const long long N = 1LL << n;
        std::vector<cx> st(N), ref;
        for (auto& v : st) v = cx(nd(g), nd(g));
        ref = st;
        Qureg q{};
        q.numQubits = n; q.isDensityMatrix = 0; q.numAmps = N; q.gpuAmps = (qcomp_t*)st.data();
        g_passes = 0; g_phasePasses = 0;
        long long gates = 0;
        const int layers = 6;
        for (int L = 0; L < layers; L++) {
            // one-qubit gates on all (or a subset of) qubits
            for (int t = 0; t < n; t++) {
                if (trial % 3 == 2 && (g() % 3 == 0)) continue;
                CompMatr1 m{};
                m.numQubits = 1; m.numRows = 2;
                // a random unitary from four angles
                double a = nd(g), b = nd(g), c = nd(g), d = nd(g);
                cx u00 = std::polar(1.0, a) * std::cos(b), u01 = std::polar(1.0, c) * std::sin(b);
                cx u10 = -std::conj(u01) * std::polar(1.0, d), u11 = std::conj(u00) * std::polar(1.0, d);
                m.elems[0][0] = {u00.real(), u00.imag()}; m.elems[0][1] = {u01.real(), u01.imag()};
                m.elems[1][0] = {u10.real(), u10.imag()}; m.elems[1][1] = {u11.real(), u11.imag()};
                applyCompMatr1(q, t, m);
                qcomp_t mm[4] = {m.elems[0][0], m.elems[0][1], m.elems[1][0], m.elems[1][1]};
                applyK(ref.data(), n, &t, 1, mm);
                gates++;
            }
            // phases: disjoint pairs, sometimes a 3-qubit one and a single
            std::vector<int> perm(n);
            for (int i = 0; i < n; i++) perm[i] = i;
            std::shuffle(perm.begin(), perm.end(), g);
            const int np_ = (trial % 4 == 3) ? n / 4 : n / 2;
            for (int p = 0; p < np_; p++) {
                double th = nd(g);
                applyTwoQubitPhaseShift(q, perm[2 * p], perm[2 * p + 1], th);
                qcomp_t dm[4] = {{1, 0}, {0, 0}, {0, 0}, {std::cos(th), std::sin(th)}};
                int t2[2] = {perm[2 * p], perm[2 * p + 1]};
                qcomp_t M[16] = {};
                M[0] = {1, 0}; M[5] = {1, 0}; M[10] = {1, 0}; M[15] = dm[3];
                applyK(ref.data(), n, t2, 2, M);
                gates++;
            }
            if (trial % 5 == 1) {
                int t3[3] = {perm[0], perm[3], perm[5]};
                double th = nd(g);
                applyMultiQubitPhaseShift(q, t3, 3, th);
                qcomp_t M[64] = {};
                for (int i = 0; i < 8; i++) M[i * 9] = {1, 0};
                M[63] = {std::cos(th), std::sin(th)};
                applyK(ref.data(), n, t3, 3, M);
                int one = perm[1];
                applyPhaseShift(q, one, th * 0.5);
                qcomp_t M1[4] = {{1, 0}, {0, 0}, {0, 0}, {std::cos(th * 0.5), std::sin(th * 0.5)}};
                applyK(ref.data(), n, &one, 1, M1);
            }
        }
        flushQuregDeferredOps(q);
        double err = 0, mx = 0;
        for (long long i = 0; i < N; i++) { err = std::max(err, std::abs(st[i] - ref[i])); mx = std::max(mx, std::abs(ref[i])); }
        bool ok = err <= 1e-12 * mx;
        // layers shaped like the benchmark's: ceil(n / 4) passes per layer at most, or one
        // fewer when the last group (of one or two qubits) stays pending, plus that group's
        // pass at the end; no phase pass
        const bool benchShaped = n % 2 == 0 && trial % 3 != 2 && trial % 4 != 3 && trial % 5 != 1;
        if (benchShaped) {
            const int full = n / 4, rem = n % 4;
            const long want = rem == 0 ? (long)layers * full : rem <= 2 ? (long)layers * full + 1 : (long)layers * (full + 1);
            ok = ok && g_phasePasses == 0 && g_passes == want;
        }
        if (!ok) bad++;
        printf("n=%2d trial=%2d gates=%lld passes=%ld (phase passes %ld) err/max=%.2e %s\n", n, trial, gates, g_passes, g_phasePasses, err / mx, ok ? "" : "FAIL");
    }
    printf("%s %d circuits\n", bad ? "FAIL" : "OK", 40);
    return bad != 0;
}
