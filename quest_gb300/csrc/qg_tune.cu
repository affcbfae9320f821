// Launch-shape autotuner for the streaming FP64 kernels.
//
// A shape is (pairs per thread per loop iteration, threads per block).  The search
// times every candidate shape with CUDA events on a scratch register on the current
// device and keeps the fastest; choices can be saved to and loaded from a small text
// file keyed by the device name, so a deployment tunes once per GPU model.
#include "qg_common.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

namespace {

struct Candidate { int ppt, threads; };
const Candidate kCandidates[] = {{1, 256}, {1, 128}, {2, 256}, {2, 128}};
const char* kKernelNames[QG_TUNE_NUM] = {"dense1_fx", "diag1_fx", "dense2_fx"};

std::atomic<int> g_shape[QG_TUNE_NUM] = {{1 * 1000 + 256}, {1 * 1000 + 256}, {1 * 1000 + 256}};

bool is_candidate(int ppt, int threads) {
    for (const auto& c : kCandidates)
        if (c.ppt == ppt && c.threads == threads) return true;
    return false;
}

std::string device_name() {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    std::string s = prop.name;
    for (auto& ch : s)
        if (ch == ' ') ch = '_';
    return s;
}

}  // namespace

QgShape qg_tuned_shape(int kernel) {
    int v = (kernel >= 0 && kernel < QG_TUNE_NUM) ? g_shape[kernel].load() : 1256;
    return QgShape{v / 1000, v % 1000};
}

extern "C" {

int qg_set_kernel_shape(int kernel, int ppt, int threads) {
    if (kernel < 0 || kernel >= QG_TUNE_NUM) return qg_fail(QG_ERR_ARG, "no tunable kernel %d", kernel);
    if (!is_candidate(ppt, threads))
        return qg_fail(QG_ERR_ARG, "shape (%d pairs per thread, %d threads) is not one of the compiled shapes", ppt, threads);
    g_shape[kernel] = ppt * 1000 + threads;
    return QG_OK;
}

int qg_get_kernel_shape(int kernel, int* ppt, int* threads) {
    if (kernel < 0 || kernel >= QG_TUNE_NUM || !ppt || !threads) return qg_fail(QG_ERR_ARG, "bad argument");
    QgShape s = qg_tuned_shape(kernel);
    *ppt = s.ppt;
    *threads = s.threads;
    return QG_OK;
}

// Times every candidate shape of the tunable kernels on a scratch register of
// numQubits (16 B x 2^numQubits of device memory, freed before returning): the
// one-target dense kernel (fixed-point products) on a fixed unitary, and the
// one-target diagonal kernel on a controlled phase, the two-target dense kernel
// (fixed-point products) on near and far target pairs.  Keeps the fastest shape per
// kernel and reports milliseconds per launch in msOut, kernel-major: msOut[k * 4 + c]
// for candidate c (up to maxOut entries).
int qg_autotune_fp64(int numQubits, double* msOut, int maxOut, int* numOut) {
    if (numQubits < 10 || numQubits > 32) return qg_fail(QG_ERR_ARG, "tune on 10..32 qubits, not %d", numQubits);
    const int64_t bytes = (int64_t)16 << numQubits;
    void* amps = nullptr;
    QG_TRY(qg_alloc(&amps, bytes));
    int rc = QG_OK;
    const qg_cplx amp = {1.0 / std::sqrt((double)((int64_t)1 << numQubits)), 0.0};
    // a fixed non-trivial unitary (phase * rotation) and a phase
    const double c = std::cos(0.37), s = std::sin(0.37), pc = std::cos(0.11), ps = std::sin(0.11);
    const qg_cplx m[4] = {{c * pc, c * ps}, {-s * pc, -s * ps}, {s * pc, s * ps}, {c * pc, c * ps}};
    const qg_cplx phase[2] = {{1.0, 0.0}, {std::cos(0.23), std::sin(0.23)}};
    qg_cplx m4[16];   // the Kronecker product of the 2x2 above with itself (unitary)
    for (int r = 0; r < 4; r++)
        for (int q = 0; q < 4; q++) {
            const qg_cplx x = m[(r >> 1) * 2 + (q >> 1)], y = m[(r & 1) * 2 + (q & 1)];
            m4[r * 4 + q] = qg_cplx{x.re * y.re - x.im * y.im, x.re * y.im + x.im * y.re};
        }
    void* ev0 = nullptr;
    void* ev1 = nullptr;
    int saved[QG_TUNE_NUM], best[QG_TUNE_NUM];
    for (int k = 0; k < QG_TUNE_NUM; k++) saved[k] = best[k] = g_shape[k].load();
    int n = 0;
    if ((rc = qg_event_create(&ev0)) == QG_OK) rc = qg_event_create(&ev1);
    if (rc == QG_OK) rc = qg_sv_initUniformState(amps, numQubits, amp, nullptr);
    for (int kern = 0; kern < QG_TUNE_NUM && rc == QG_OK; kern++) {
        double bestMs = 1e30;
        int ci = 0;
        for (const auto& cand : kCandidates) {
            g_shape[kern] = cand.ppt * 1000 + cand.threads;
            auto run = [&](int r) {
                const int t = (r * 7) % (numQubits - 2) + 2;
                if (kern == QG_TUNE_DENSE1)
                    return qg_sv_anyCtrlOneTargDenseMatr(amps, numQubits, nullptr, nullptr, 0, t, m, nullptr);
                if (kern == QG_TUNE_DENSE2) {
                    // near pairs and pairs half the register apart (a density matrix's ket/bra pair)
                    const int t2 = (r & 1) ? (t + numQubits / 2) % numQubits : (t + 1) % numQubits;
                    return qg_sv_anyCtrlTwoTargDenseMatr(amps, numQubits, nullptr, nullptr, 0, t, t2 == t ? (t + 1) % numQubits : t2,
                                                         m4, nullptr);
                }
                const int ctrl = (t + 3) % numQubits == t ? 0 : (t + 3) % numQubits;
                return qg_sv_anyCtrlOneTargDiagMatr(amps, numQubits, &ctrl, nullptr, 1, t, phase, nullptr);
            };
            const int reps = 6;
            for (int w = 0; w < 2 && rc == QG_OK; w++) rc = run(w);
            if (rc == QG_OK) rc = qg_event_record(ev0, nullptr);
            for (int r = 0; r < reps && rc == QG_OK; r++) rc = run(r);
            if (rc == QG_OK) rc = qg_event_record(ev1, nullptr);
            float ms = 0;
            if (rc == QG_OK) rc = qg_event_elapsed_ms(ev0, ev1, &ms);
            if (rc != QG_OK) break;
            const double per = ms / reps;
            const int slot = kern * 4 + ci;
            if (msOut && slot < maxOut) msOut[slot] = per;
            n = std::max(n, slot + 1);
            if (per < bestMs) { bestMs = per; best[kern] = cand.ppt * 1000 + cand.threads; }
            ci++;
        }
    }
    for (int k = 0; k < QG_TUNE_NUM; k++) g_shape[k] = rc == QG_OK ? best[k] : saved[k];
    if (numOut) *numOut = n;
    if (ev0) qg_event_destroy(ev0);
    if (ev1) qg_event_destroy(ev1);
    qg_free(amps);
    return rc;
}

// "qg-tune 1", then one line per kernel: <device> <kernel> <ppt> <threads>
int qg_tune_save(const char* path) {
    if (!path) return qg_fail(QG_ERR_ARG, "null path");
    FILE* f = std::fopen(path, "w");
    if (!f) return qg_fail(QG_ERR_ARG, "cannot write %s", path);
    std::string dev = device_name();
    std::fprintf(f, "qg-tune 1\n");
    for (int k = 0; k < QG_TUNE_NUM; k++) {
        QgShape s = qg_tuned_shape(k);
        std::fprintf(f, "%s %s %d %d\n", dev.c_str(), kKernelNames[k], s.ppt, s.threads);
    }
    std::fclose(f);
    return QG_OK;
}

// applies the lines for this device's name; lines for other devices are skipped
int qg_tune_load(const char* path, int* numApplied) {
    if (!path) return qg_fail(QG_ERR_ARG, "null path");
    FILE* f = std::fopen(path, "r");
    if (!f) return qg_fail(QG_ERR_ARG, "cannot read %s", path);
    char line[512];
    int applied = 0, rc = QG_OK;
    if (!std::fgets(line, sizeof line, f) || std::strncmp(line, "qg-tune 1", 9) != 0) {
        std::fclose(f);
        return qg_fail(QG_ERR_ARG, "%s is not a tuning file", path);
    }
    std::string dev = device_name();
    while (std::fgets(line, sizeof line, f)) {
        char d[256], kname[64];
        int ppt, threads;
        if (std::sscanf(line, "%255s %63s %d %d", d, kname, &ppt, &threads) != 4) continue;
        if (dev != d) continue;
        for (int k = 0; k < QG_TUNE_NUM; k++)
            if (std::strcmp(kname, kKernelNames[k]) == 0) {
                if ((rc = qg_set_kernel_shape(k, ppt, threads)) != QG_OK) break;
                applied++;
            }
        if (rc != QG_OK) break;
    }
    std::fclose(f);
    if (numApplied) *numApplied = applied;
    return rc;
}

}  // extern "C"
