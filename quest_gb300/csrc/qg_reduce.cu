// Reductions of the sm_103a backend: total probability, outcome probabilities and
// Pauli expectation values (replacing the Thrust transform_reduce calls of
// quest/src/gpu/gpu_thrust.cuh:745-1011).
//
// Every reduction is one launch of a fixed grid (a multiple of the SM count).
// Each thread accumulates a fixed, strided subset of the terms in FP64; the block
// combines its threads with warp shuffles and a shared-memory tree; the block's
// partial sums go to library scratch, and the last block to finish (found with
// an atomic ticket after a memory fence) adds the partials in block order and
// resets the ticket.  The grid, the assignment of terms to threads and every
// addition order are fixed, so the same input always gives the same bits.
#include "qg_reduce.cuh"

#include <algorithm>
#include <vector>

// ----------------------------------------------------------------- kernels

// sum |a_i|^2 over i = insert(m) | mask, m in [0, numIts)  (calcTotalProb / calcProbOfMultiQubitOutcome)
template <int NB>
__global__ void __launch_bounds__(RED_THREADS) k_sum_norm(const double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, RedOut out) {
    double v[1] = {0.0};
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    qidx m = blockIdx.x * (qidx)RED_THREADS + threadIdx.x;
    for (; m + 3 * stride < numIts; m += 4 * stride) {
        double2 x0 = ld_amp(a + (insert_bits<NB>(m, ins) | mask));
        double2 x1 = ld_amp(a + (insert_bits<NB>(m + stride, ins) | mask));
        double2 x2 = ld_amp(a + (insert_bits<NB>(m + 2 * stride, ins) | mask));
        double2 x3 = ld_amp(a + (insert_bits<NB>(m + 3 * stride, ins) | mask));
        v[0] = fma(x0.x, x0.x, fma(x0.y, x0.y, v[0]));
        v[0] = fma(x1.x, x1.x, fma(x1.y, x1.y, v[0]));
        v[0] = fma(x2.x, x2.x, fma(x2.y, x2.y, v[0]));
        v[0] = fma(x3.x, x3.x, fma(x3.y, x3.y, v[0]));
    }
    for (; m < numIts; m += stride) {
        double2 x = ld_amp(a + (insert_bits<NB>(m, ins) | mask));
        v[0] = fma(x.x, x.x, fma(x.y, x.y, v[0]));
    }
    block_reduce_and_finish<1>(v, out);
}

// sum Re a[d(i)] over diagonal elements, i = insert(m) | mask, d(i) = i * (2^nKet + 1)
template <int NB>
__global__ void __launch_bounds__(RED_THREADS) k_sum_diag(const double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx diagStride, RedOut out) {
    double v[1] = {0.0};
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx m = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; m < numIts; m += stride) {
        qidx i = insert_bits<NB>(m, ins) | mask;
        v[0] += __ldg(&a[i * diagStride].x);
    }
    block_reduce_and_finish<1>(v, out);
}

// sum (-1)^parity(i & tmask) |a_i|^2
__global__ void __launch_bounds__(RED_THREADS) k_expec_z(const double2* __restrict__ a, qidx numAmps, qidx tmask, RedOut out) {
    double v[1] = {0.0};
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx i = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; i < numAmps; i += stride) {
        double2 x = ld_amp(a + i);
        double p = fma(x.x, x.x, x.y * x.y);
        v[0] += parity64(i & tmask) ? -p : p;
    }
    block_reduce_and_finish<1>(v, out);
}

// density matrix: sum (-1)^parity(n & tmask) a[n * (dim + 1)]  (complex)
__global__ void __launch_bounds__(RED_THREADS) k_dm_expec_z(const double2* __restrict__ a, qidx dim, qidx tmask, RedOut out) {
    double v[2] = {0.0, 0.0};
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx n = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; n < dim; n += stride) {
        double2 x = __ldg(a + n * (dim + 1));
        if (parity64(n & tmask)) { v[0] -= x.x; v[1] -= x.y; }
        else { v[0] += x.x; v[1] += x.y; }
    }
    block_reduce_and_finish<2>(v, out);
}

// Statevector Pauli string, pair form.  The reference sums, over every n,
// sign(j & maskYZ) conj(a_n) a_j with j = n ^ maskXY (cpu_subroutines.cpp:2059-2085).
// Each unordered pair {n, j} contributes sign(j) x + sign(n) conj(x), x = conj(a_n) a_j;
// with sign(j) = sign(n) (-1)^numY this is 2 sign(n) Re x (even #Y) or
// -2i sign(n) Im x (odd #Y).  Pairs are enumerated by n with the top X/Y bit zero,
// so every amplitude is read once.  Result before the i^numY factor: v[0] + i v[1].
template <int NB>
__global__ void __launch_bounds__(RED_THREADS) k_expec_pauli(const double2* __restrict__ a, qidx numIts, Ins ins,
                                                            qidx maskXY, qidx maskYZ, int oddY, RedOut out) {
    double v[2] = {0.0, 0.0};
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx m = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; m < numIts; m += stride) {
        qidx n = insert_bits<NB>(m, ins);
        qidx j = n ^ maskXY;
        double2 an = ld_amp(a + n), aj = ld_amp(a + j);
        // x = conj(an) * aj
        double xr = fma(an.x, aj.x, an.y * aj.y);
        double xi = fma(an.x, aj.y, -an.y * aj.x);
        double s = parity64(n & maskYZ) ? -2.0 : 2.0;
        if (oddY) v[1] -= s * xi;
        else v[0] += s * xr;
    }
    block_reduce_and_finish<2>(v, out);
}

// density matrix Pauli string (cpu_subroutines.cpp:2121-2160): sum_n sign(i & maskYZ) a[i + n*dim], i = n ^ maskXY
__global__ void __launch_bounds__(RED_THREADS) k_dm_expec_pauli(const double2* __restrict__ a, qidx dim, qidx maskXY, qidx maskYZ, RedOut out) {
    double v[2] = {0.0, 0.0};
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx n = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; n < dim; n += stride) {
        qidx i = n ^ maskXY;
        double2 x = __ldg(a + i + n * dim);
        if (parity64(i & maskYZ)) { v[0] -= x.x; v[1] -= x.y; }
        else { v[0] += x.x; v[1] += x.y; }
    }
    block_reduce_and_finish<2>(v, out);
}

// Density-matrix form of the batch: per column n and string s the element
// rho[n ^ maskXY_s][n] with its sign; NS strings per pass over the 2^N columns.
template <int NS>
__global__ void __launch_bounds__(RED_THREADS) k_dm_expec_pauli_batch(const double2* __restrict__ a, qidx dim,
                                                                     const qidx* __restrict__ mXY, const qidx* __restrict__ mYZ,
                                                                     int numStrings, RedOut out) {
    double v[2 * NS];
#pragma unroll
    for (int k = 0; k < 2 * NS; k++) v[k] = 0.0;
    __shared__ qidx sXY[NS], sYZ[NS];
    if (threadIdx.x < NS) {
        sXY[threadIdx.x] = threadIdx.x < numStrings ? mXY[threadIdx.x] : 0;
        sYZ[threadIdx.x] = threadIdx.x < numStrings ? mYZ[threadIdx.x] : 0;
    }
    __syncthreads();
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx n = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; n < dim; n += stride) {
#pragma unroll
        for (int s = 0; s < NS; s++) {
            if (s < numStrings) {
                qidx i = n ^ sXY[s];
                double2 x = __ldg(a + i + n * dim);
                double sg = parity64(i & sYZ[s]) ? -1.0 : 1.0;
                v[2 * s] += sg * x.x;
                v[2 * s + 1] += sg * x.y;
            }
        }
    }
    block_reduce_and_finish<2 * NS>(v, out);
}

// histogram of all outcomes of `num` qubits, one bin per blockIdx.y (deterministic: no
// atomics, a fixed assignment of terms to threads and a fixed addition order).
// Statevector (DIAG = false): sum of |a_i|^2; density matrix (DIAG = true): sum of
// Re rho_ii, the element i * diagStride of the Choi vector.
template <int NB, bool DIAG>
__global__ void __launch_bounds__(RED_THREADS) k_probs_all(const double2* __restrict__ a, qidx numIts, Ins ins,
                                                          const qidx* __restrict__ binMasks, qidx diagStride,
                                                          double* __restrict__ partials) {
    __shared__ double sh[RED_THREADS / 32];
    qidx mask = binMasks[blockIdx.y];
    double v = 0;
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx m = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; m < numIts; m += stride) {
        if (DIAG) {
            v += __ldg(&a[(insert_bits<NB>(m, ins) | mask) * diagStride].x);
        } else {
            double2 x = ld_amp(a + (insert_bits<NB>(m, ins) | mask));
            v = fma(x.x, x.x, fma(x.y, x.y, v));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < RED_THREADS / 32; w++) s += sh[w];
        partials[(qidx)blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void k_probs_all_finish(const double* __restrict__ partials, int perBin, qidx numBins, double* __restrict__ out) {
    qidx b = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (b >= numBins) return;
    double s = 0;
    for (int k = 0; k < perBin; k++) s += partials[b * perBin + k];
    out[b] = s;
}

// ----------------------------------------------------------------- host side

namespace {

int sum_norm(const void* amps, int numQubits, const QubitPlan& p, double* out, cudaStream_t st) {
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    int grid = red_grid(numIts);
    RedOut r;
    QG_TRY(red_setup(grid, 1, &r));
#define L(NBV) k_sum_norm<NBV><<<grid, RED_THREADS, 0, st>>>((const double2*)amps, numIts, p.ins, p.stateMask, r)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    return red_fetch(r, 1, out, st);
}

int sum_diag(const void* amps, int nKet, const QubitPlan& p, double* out, cudaStream_t st) {
    qidx numIts = ((qidx)1 << nKet) >> p.numFixed;
    int grid = red_grid(numIts);
    RedOut r;
    QG_TRY(red_setup(grid, 1, &r));
    qidx ds = ((qidx)1 << nKet) + 1;
#define L(NBV) k_sum_diag<NBV><<<grid, RED_THREADS, 0, st>>>((const double2*)amps, numIts, p.ins, p.stateMask, ds, r)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    return red_fetch(r, 1, out, st);
}

int check_dm_amps(const void* amps, int nKet) {
    if (nKet < 1 || 2 * nKet > QG_MAX_QUBITS) return qg_fail(QG_ERR_ARG, "density matrix of %d qubits is unsupported", nKet);
    return qg_check_amps(amps, 2 * nKet);
}

int pauli_masks(int limit, const int* x, int nx, const int* y, int ny, const int* z, int nz, qidx* mXY, qidx* mYZ, int* top) {
    std::vector<int> all;
    *mXY = 0; *mYZ = 0; *top = -1;
    for (int i = 0; i < nx; i++) { all.push_back(x[i]); *mXY |= (qidx)1 << x[i]; *top = std::max(*top, x[i]); }
    for (int i = 0; i < ny; i++) { all.push_back(y[i]); *mXY |= (qidx)1 << y[i]; *mYZ |= (qidx)1 << y[i]; *top = std::max(*top, y[i]); }
    for (int i = 0; i < nz; i++) { all.push_back(z[i]); *mYZ |= (qidx)1 << z[i]; }
    return qg_check_qubits(limit, all.data(), (int)all.size(), "Pauli targets");
}

}  // namespace

extern "C" {

int qg_sv_calcTotalProb(const void* amps, int numQubits, double* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, nullptr, nullptr, 0, nullptr, nullptr, 0, &p));
    return sum_norm(amps, numQubits, p, out, qg_stream(stream));
}

int qg_dm_calcTotalProb(const void* amps, int nKet, double* out, void* stream) {
    QG_TRY(check_dm_amps(amps, nKet));
    QubitPlan p;
    QG_TRY(qg_make_plan(nKet, nullptr, nullptr, 0, nullptr, nullptr, 0, &p));
    return sum_diag(amps, nKet, p, out, qg_stream(stream));
}

int qg_sv_calcProbOfMultiQubitOutcome(const void* amps, int numQubits, const int* qubits, const int* outcomes, int num,
                                      double* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, nullptr, nullptr, 0, qubits, outcomes, num, &p));
    return sum_norm(amps, numQubits, p, out, qg_stream(stream));
}

int qg_dm_calcProbOfMultiQubitOutcome(const void* amps, int nKet, const int* qubits, const int* outcomes, int num,
                                      double* out, void* stream) {
    QG_TRY(check_dm_amps(amps, nKet));
    QubitPlan p;
    QG_TRY(qg_make_plan(nKet, nullptr, nullptr, 0, qubits, outcomes, num, &p));
    return sum_diag(amps, nKet, p, out, qg_stream(stream));
}

}  // extern "C"

namespace {

// histogram over the outcomes of `num` qubits: statevector (nKet = 0) or the diagonal of a
// density matrix of nKet qubits (its Choi vector has 2 nKet qubits)
int probs_all(double* outProbs, const void* amps, int numQubits, bool dm, const int* qubits, int num, void* stream) {
    if (num < 1 || num > 20) return qg_fail(QG_ERR_ARG, "outcome histogram over %d qubits is unsupported", num);
    if (!outProbs) return qg_fail(QG_ERR_ARG, "null output");
    std::vector<int> zeros(num, 0);
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, nullptr, nullptr, 0, qubits, zeros.data(), num, &p));
    qidx numBins = (qidx)1 << num;
    std::vector<qidx> masks((size_t)numBins);
    for (qidx b = 0; b < numBins; b++) {
        qidx m = 0;
        for (int i = 0; i < num; i++)
            if ((b >> i) & 1) m |= (qidx)1 << qubits[i];
        masks[(size_t)b] = m;
    }
    qidx numIts = ((qidx)1 << numQubits) >> num;
    qidx diagStride = dm ? ((qidx)1 << numQubits) + 1 : 1;
    int gx = (int)std::max<qidx>(1, std::min<qidx>((qidx)qg_num_sms() * 4 / numBins + 1, (numIts + RED_THREADS - 1) / RED_THREADS));
    cudaStream_t st = qg_stream(stream);
    void* s = nullptr;
    size_t need = 8 * (size_t)numBins + 8 * (size_t)numBins * gx + 8 * (size_t)numBins;
    QG_TRY(qg_scratch_get(&s, need + 512));
    // the first 512 bytes hold the completion ticket of the other reductions: keep clear of them
    qidx* dMasks = (qidx*)((char*)s + 512);
    double* partials = (double*)((char*)s + 512 + 8 * numBins);
    double* result = partials + numBins * gx;
    QG_CUDA(cudaMemcpyAsync(dMasks, masks.data(), 8 * (size_t)numBins, cudaMemcpyHostToDevice, st));
    for (qidx b0 = 0; b0 < numBins; b0 += 65535) {
        unsigned gy = (unsigned)std::min<qidx>(65535, numBins - b0);
        dim3 grid(gx, gy);
        if (dm) {
#define L(NBV) k_probs_all<NBV, true><<<grid, RED_THREADS, 0, st>>>((const double2*)amps, numIts, p.ins, dMasks + b0, diagStride, partials + b0 * gx)
            QG_DISPATCH_NB(p.numFixed, L)
#undef L
        } else {
#define L(NBV) k_probs_all<NBV, false><<<grid, RED_THREADS, 0, st>>>((const double2*)amps, numIts, p.ins, dMasks + b0, diagStride, partials + b0 * gx)
            QG_DISPATCH_NB(p.numFixed, L)
#undef L
        }
        qg_note_launch();
    }
    k_probs_all_finish<<<qg_blocks(numBins), QG_THREADS, 0, st>>>(partials, gx, numBins, result);
    qg_note_launch();
    QG_TRY(qg_check_launch("probs_all"));
    QG_CUDA(cudaMemcpyAsync(outProbs, result, 8 * (size_t)numBins, cudaMemcpyDeviceToHost, st));
    QG_CUDA(cudaStreamSynchronize(st));
    return QG_OK;
}

}  // namespace

extern "C" {

int qg_sv_calcProbsOfAllMultiQubitOutcomes(double* outProbs, const void* amps, int numQubits, const int* qubits, int num,
                                           void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    return probs_all(outProbs, amps, numQubits, false, qubits, num, stream);
}

int qg_dm_calcProbsOfAllMultiQubitOutcomes(double* outProbs, const void* amps, int numKetQubits, const int* qubits, int num,
                                           void* stream) {
    QG_TRY(check_dm_amps(amps, numKetQubits));
    return probs_all(outProbs, amps, numKetQubits, true, qubits, num, stream);
}

int qg_sv_calcExpecAnyTargZ(const void* amps, int numQubits, const int* targs, int numTargs, double* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QG_TRY(qg_check_qubits(numQubits, targs, numTargs, "targets"));
    qidx tmask = 0;
    for (int i = 0; i < numTargs; i++) tmask |= (qidx)1 << targs[i];
    qidx n = (qidx)1 << numQubits;
    int grid = red_grid(n);
    RedOut r;
    QG_TRY(red_setup(grid, 1, &r));
    cudaStream_t st = qg_stream(stream);
    k_expec_z<<<grid, RED_THREADS, 0, st>>>((const double2*)amps, n, tmask, r);
    return red_fetch(r, 1, out, st);
}

int qg_dm_calcExpecAnyTargZ(const void* amps, int nKet, const int* targs, int numTargs, qg_cplx* out, void* stream) {
    QG_TRY(check_dm_amps(amps, nKet));
    QG_TRY(qg_check_qubits(nKet, targs, numTargs, "targets"));
    qidx tmask = 0;
    for (int i = 0; i < numTargs; i++) tmask |= (qidx)1 << targs[i];
    qidx dim = (qidx)1 << nKet;
    int grid = red_grid(dim);
    RedOut r;
    QG_TRY(red_setup(grid, 2, &r));
    cudaStream_t st = qg_stream(stream);
    k_dm_expec_z<<<grid, RED_THREADS, 0, st>>>((const double2*)amps, dim, tmask, r);
    double v[2];
    QG_TRY(red_fetch(r, 2, v, st));
    out->re = v[0];
    out->im = v[1];
    return QG_OK;
}

int qg_sv_calcExpecPauliStr(const void* amps, int numQubits, const int* x, int nx, const int* y, int ny,
                            const int* z, int nz, qg_cplx* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    qidx mXY, mYZ;
    int top;
    QG_TRY(pauli_masks(numQubits, x, nx, y, ny, z, nz, &mXY, &mYZ, &top));
    cudaStream_t st = qg_stream(stream);
    if (nx + ny == 0) {
        // identity -> total probability; Z-only -> the Z routine (localiser.cpp:1963-1976)
        double v;
        if (nz == 0) QG_TRY(qg_sv_calcTotalProb(amps, numQubits, &v, stream));
        else QG_TRY(qg_sv_calcExpecAnyTargZ(amps, numQubits, z, nz, &v, stream));
        out->re = v;
        out->im = 0;
        return QG_OK;
    }
    int tv = 0;
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, nullptr, nullptr, 0, &top, &tv, 1, &p));
    qidx numIts = ((qidx)1 << numQubits) >> 1;
    int grid = red_grid(numIts);
    RedOut r;
    QG_TRY(red_setup(grid, 2, &r));
    k_expec_pauli<1><<<grid, RED_THREADS, 0, st>>>((const double2*)amps, numIts, p.ins, mXY, mYZ, ny & 1, r);
    double v[2];
    QG_TRY(red_fetch(r, 2, v, st));
    times_power_of_i(&v[0], &v[1], ny);
    out->re = v[0];
    out->im = v[1];
    return QG_OK;
}

int qg_dm_calcExpecPauliStr(const void* amps, int nKet, const int* x, int nx, const int* y, int ny,
                            const int* z, int nz, qg_cplx* out, void* stream) {
    QG_TRY(check_dm_amps(amps, nKet));
    qidx mXY, mYZ;
    int top;
    QG_TRY(pauli_masks(nKet, x, nx, y, ny, z, nz, &mXY, &mYZ, &top));
    cudaStream_t st = qg_stream(stream);
    if (nx + ny == 0) {
        if (nz == 0) {
            double v;
            QG_TRY(qg_dm_calcTotalProb(amps, nKet, &v, stream));
            out->re = v;
            out->im = 0;
            return QG_OK;
        }
        return qg_dm_calcExpecAnyTargZ(amps, nKet, z, nz, out, stream);
    }
    qidx dim = (qidx)1 << nKet;
    int grid = red_grid(dim);
    RedOut r;
    QG_TRY(red_setup(grid, 2, &r));
    k_dm_expec_pauli<<<grid, RED_THREADS, 0, st>>>((const double2*)amps, dim, mXY, mYZ, r);
    double v[2];
    QG_TRY(red_fetch(r, 2, v, st));
    times_power_of_i(&v[0], &v[1], ny);
    out->re = v[0];
    out->im = v[1];
    return QG_OK;
}

}  // extern "C"

namespace {
int expec_pauli_batch(const void* amps, int numQubits, bool dm, const int64_t* masksXY, const int64_t* masksYZ,
                      const int* numsY, int numStrings, qg_cplx* out, void* stream);
}  // namespace

extern "C" {

int qg_sv_calcExpecPauliStrBatch(const void* amps, int numQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                 const int* numsY, int numStrings, qg_cplx* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    return expec_pauli_batch(amps, numQubits, false, masksXY, masksYZ, numsY, numStrings, out, stream);
}

int qg_dm_calcExpecPauliStrBatch(const void* amps, int numKetQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                 const int* numsY, int numStrings, qg_cplx* out, void* stream) {
    QG_TRY(check_dm_amps(amps, numKetQubits));
    return expec_pauli_batch(amps, numKetQubits, true, masksXY, masksYZ, numsY, numStrings, out, stream);
}

}  // extern "C"

template <typename AMP>
int qg_pauli_tile_batch(const AMP* amps, int n, const int64_t* mXY, const int64_t* mYZ, const int* numsY, int num,
                        qg_cplx* out, cudaStream_t st);

namespace {

// statevector: the tiled kernel of qg_pauli_tile.cu (each amplitude read once per group
// of strings); density matrix: up to 16 strings per pass over the columns, where each
// string reads one element per column; numQubits = the ket qubits of a density matrix
int expec_pauli_batch(const void* amps, int numQubits, bool dm, const int64_t* masksXY, const int64_t* masksYZ,
                      const int* numsY, int numStrings, qg_cplx* out, void* stream) {
    if (numStrings < 0) return qg_fail(QG_ERR_ARG, "negative string count");
    if (numStrings > 0 && (!masksXY || !masksYZ || !numsY || !out)) return qg_fail(QG_ERR_ARG, "null argument");
    qidx lim = ((qidx)1 << numQubits) - 1;
    for (int s = 0; s < numStrings; s++)
        if ((masksXY[s] & ~lim) || (masksYZ[s] & ~lim)) return qg_fail(QG_ERR_ARG, "Pauli string %d targets a qubit beyond %d", s, numQubits);
    cudaStream_t st = qg_stream(stream);
    if (!dm) return numStrings ? qg_pauli_tile_batch<double2>((const double2*)amps, numQubits, masksXY, masksYZ, numsY, numStrings, out, st) : QG_OK;
    const int NS = 16;
    qidx n = (qidx)1 << numQubits;
    for (int s0 = 0; s0 < numStrings; s0 += NS) {
        int cnt = std::min(NS, numStrings - s0);
        int grid = red_grid(n);
        void* s = nullptr;
        // scratch: masks (2*NS qidx) then the reduction area
        RedOut r;
        size_t bytes = 512 + 8 * 2 * NS + 8 * (size_t)(2 * NS) * grid + 8 * 2 * NS + 1024;
        QG_TRY(qg_scratch_get(&s, bytes));
        char* base = (char*)s;
        r.ticket = (unsigned int*)base;
        r.result = (double*)(base + 256);
        qidx* dmask = (qidx*)(base + 256 + 8 * 2 * NS);
        r.partials = (double*)(base + 256 + 8 * 2 * NS + 8 * 2 * NS);
        std::vector<qidx> hm(2 * NS, 0);
        for (int k = 0; k < cnt; k++) { hm[k] = masksXY[s0 + k]; hm[NS + k] = masksYZ[s0 + k]; }
        QG_CUDA(cudaMemcpyAsync(dmask, hm.data(), 8 * 2 * NS, cudaMemcpyHostToDevice, st));
        k_dm_expec_pauli_batch<NS><<<grid, RED_THREADS, 0, st>>>((const double2*)amps, n, dmask, dmask + NS, cnt, r);
        qg_note_launch();
        double v[2 * NS];
        QG_TRY(red_fetch(r, 2 * NS, v, st));
        for (int k = 0; k < cnt; k++) {
            double re = v[2 * k], im = v[2 * k + 1];
            times_power_of_i(&re, &im, numsY[s0 + k]);
            out[s0 + k].re = re;
            out[s0 + k].im = im;
        }
    }
    return QG_OK;
}

}  // namespace

