// Host restatement of the tensor-core dense kernel (quest_gb300/csrc/qg_dense_tc.cu) over a
// whole register, for the GPU tests' bit-for-bit comparison: every group through
// qg_slices.h's apply_group, and the groups it refuses in FP64 with the kernel's order of
// fused multiply-adds.  Built by the tests as a shared library.
#include <cmath>
#include <cstdint>
#include <vector>

#include "qg_slices.h"

extern "C" int slices_apply_state(int numQubits, int K, const int* targs, int numCtrls, const int* ctrls,
                                  const int* ctrlStates, const double* matr, double* amps) {
    const int D = 1 << K, KR = 2 * D;
    std::vector<double> R(KR * KR);
    qgfx::real_form(matr, D, R.data());
    std::vector<int8_t> dig(qgsl::RD * KR * KR);
    int eR = 0;
    if (!qgsl::operator_digits(R.data(), KR, dig.data(), &eR)) return 1;
    int64_t tmask = 0, cmask = 0, cval = 0;
    for (int b = 0; b < K; b++) tmask |= (int64_t)1 << targs[b];
    for (int c = 0; c < numCtrls; c++) {
        cmask |= (int64_t)1 << ctrls[c];
        if (ctrlStates[c]) cval |= (int64_t)1 << ctrls[c];
    }
    std::vector<int64_t> off(D);
    for (int j = 0; j < D; j++) {
        int64_t o = 0;
        for (int b = 0; b < K; b++)
            if ((j >> b) & 1) o |= (int64_t)1 << targs[b];
        off[j] = o;
    }
    std::vector<double> x(KR), y(KR);
    const int64_t N = (int64_t)1 << numQubits;
    for (int64_t base = 0; base < N; base++) {
        if ((base & tmask) || (base & cmask) != cval) continue;
        for (int j = 0; j < D; j++) {
            x[2 * j] = amps[2 * (base + off[j])];
            x[2 * j + 1] = amps[2 * (base + off[j]) + 1];
        }
        if (!qgsl::apply_group(dig.data(), eR, KR, x.data(), y.data())) {
            // the kernel's FP64 path: acc = m[r][j] * in[j] + acc for j = 0.. in order
            for (int r = 0; r < D; r++) {
                double re = 0.0, im = 0.0;
                for (int j = 0; j < D; j++) {
                    const double mr = matr[2 * (r * D + j)], mi = matr[2 * (r * D + j) + 1];
                    const double xr = x[2 * j], xi = x[2 * j + 1];
                    const double nre = std::fma(mr, xr, std::fma(-mi, xi, re));
                    const double nim = std::fma(mr, xi, std::fma(mi, xr, im));
                    re = nre;
                    im = nim;
                }
                y[2 * r] = re;
                y[2 * r + 1] = im;
            }
        }
        for (int j = 0; j < D; j++) {
            amps[2 * (base + off[j])] = y[2 * j];
            amps[2 * (base + off[j]) + 1] = y[2 * j + 1];
        }
    }
    return 0;
}
