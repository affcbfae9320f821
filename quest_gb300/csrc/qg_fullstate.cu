// All-target diagonal matrices (QuEST's FullStateDiagMatr) on FP64 registers:
// application to statevectors and density matrices, with an optional complex power,
// and the expectation value of the diagonal.
//
// Replaces gpu_statevec_allTargDiagMatr_sub / gpu_densmatr_allTargDiagMatr_sub
// (quest/src/gpu/gpu_subroutines.cpp, kernels in gpu_kernels.cuh:556-588 and
// gpu_thrust.cuh:729-742) and gpu_statevec/densmatr_calcExpecFullStateDiagMatr_sub
// (gpu_thrust.cuh:977-1011).  The element array lives in device memory (the matrix's
// gpuElems), 2^n complex values for an n-qubit register (n ket qubits for a density
// matrix).
//
// Traffic: a statevector update reads the element and the amplitude and writes the
// amplitude (48 B per amplitude); a density-matrix update streams the 2^(2N) flat
// amplitudes while the row factors (2^N elements) stay in L2.  Powers use
// pow(z, w) = exp(w log z), the formula of std::pow on complex arguments.
#include "qg_common.cuh"
#include "qg_reduce.cuh"

namespace {

__device__ __forceinline__ double2 cpow_(double2 z, double2 w) {
    if (z.x == 0.0 && z.y == 0.0) return make_double2(0.0, 0.0);
    const double lr = log(hypot(z.x, z.y)), th = atan2(z.y, z.x);   // log z = lr + i th
    const double re = w.x * lr - w.y * th, im = w.x * th + w.y * lr;
    double s, c;
    sincos(im, &s, &c);
    const double m = exp(re);
    return make_double2(m * c, m * s);
}

template <bool HasPower>
__device__ __forceinline__ double2 elem_pow(double2 d, double2 ex) {
    return HasPower ? cpow_(d, ex) : d;
}

template <bool HasPower>
__global__ void k_sv_alltarg_diag(double2* __restrict__ a, const double2* __restrict__ d, qidx n, double2 ex) {
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    for (qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x; i < n; i += stride)
        st_amp(a + i, cmul(elem_pow<HasPower>(ld_amp(d + i), ex), ld_amp(a + i)));
}

// flat index i = c * dim + r: rho[r][c] *= f(d_r) (* conj(f(d_c)) unless MultiplyOnly)
template <bool HasPower, bool MultiplyOnly>
__global__ void k_dm_alltarg_diag(double2* __restrict__ a, const double2* __restrict__ d, int nKet, double2 ex) {
    const qidx dim = (qidx)1 << nKet, n = dim << nKet;
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    for (qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x; i < n; i += stride) {
        double2 fac = elem_pow<HasPower>(__ldg(d + (i & (dim - 1))), ex);
        if (!MultiplyOnly) {
            double2 t = elem_pow<HasPower>(__ldg(d + (i >> nKet)), ex);
            fac = cmul(fac, make_double2(t.x, -t.y));
        }
        st_amp(a + i, cmul(fac, ld_amp(a + i)));
    }
}

// the element as the expectation routines raise it (real power: pow of the real part)
template <bool HasPower, bool RealPow>
__device__ __forceinline__ double2 expec_elem(double2 d, double2 ex) {
    if (HasPower && RealPow) return make_double2(pow(d.x, ex.x), 0.0);
    if (HasPower) return cpow_(d, ex);
    return d;
}

template <bool HasPower, bool RealPow>
__global__ void __launch_bounds__(RED_THREADS) k_sv_expec_alltarg(const double2* __restrict__ a, const double2* __restrict__ d,
                                                                  qidx n, double2 ex, RedOut out) {
    double v[2] = {0.0, 0.0};
    const qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx i = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; i < n; i += stride) {
        const double2 x = __ldg(a + i);
        const double nrm = x.x * x.x + x.y * x.y;
        const double2 e = expec_elem<HasPower, RealPow>(__ldg(d + i), ex);
        v[0] += e.x * nrm;
        v[1] += e.y * nrm;
    }
    block_reduce_and_finish<2>(v, out);
}

template <bool HasPower, bool RealPow>
__global__ void __launch_bounds__(RED_THREADS) k_dm_expec_alltarg(const double2* __restrict__ a, const double2* __restrict__ d,
                                                                  int nKet, double2 ex, RedOut out) {
    double v[2] = {0.0, 0.0};
    const qidx dim = (qidx)1 << nKet;
    const qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx r = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; r < dim; r += stride) {
        const double2 rho = __ldg(a + r * (dim + 1));
        const double2 e = expec_elem<HasPower, RealPow>(__ldg(d + r), ex);
        v[0] += e.x * rho.x - e.y * rho.y;
        v[1] += e.x * rho.y + e.y * rho.x;
    }
    block_reduce_and_finish<2>(v, out);
}

inline double2 d2c(qg_cplx c) { return make_double2(c.re, c.im); }

int check_elems(const void* elems) {
    if (!elems) return qg_fail(QG_ERR_ARG, "null diagonal element array");
    if (((uintptr_t)elems & 15) != 0) return qg_fail(QG_ERR_ARG, "the diagonal element array must be 16-byte aligned");
    return QG_OK;
}

}  // namespace

extern "C" {

int qg_sv_allTargDiagMatr(void* amps, int numQubits, const void* elems, qg_cplx exponent, int hasPower, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QG_TRY(check_elems(elems));
    const qidx n = (qidx)1 << numQubits;
    cudaStream_t st = qg_stream(stream);
    if (hasPower)
        k_sv_alltarg_diag<true><<<qg_blocks(n), QG_THREADS, 0, st>>>((double2*)amps, (const double2*)elems, n, d2c(exponent));
    else
        k_sv_alltarg_diag<false><<<qg_blocks(n), QG_THREADS, 0, st>>>((double2*)amps, (const double2*)elems, n, d2c(exponent));
    qg_note_launch();
    return qg_check_launch("sv_allTargDiagMatr");
}

int qg_dm_allTargDiagMatr(void* amps, int numKetQubits, const void* elems, qg_cplx exponent, int hasPower, int multiplyOnly,
                          void* stream) {
    QG_TRY(qg_check_amps(amps, 2 * numKetQubits));
    QG_TRY(check_elems(elems));
    const qidx n = (qidx)1 << (2 * numKetQubits);
    cudaStream_t st = qg_stream(stream);
    const double2 ex = d2c(exponent);
    double2* a = (double2*)amps;
    const double2* d = (const double2*)elems;
    const unsigned g = qg_blocks(n);
    if (hasPower && multiplyOnly) k_dm_alltarg_diag<true, true><<<g, QG_THREADS, 0, st>>>(a, d, numKetQubits, ex);
    else if (hasPower) k_dm_alltarg_diag<true, false><<<g, QG_THREADS, 0, st>>>(a, d, numKetQubits, ex);
    else if (multiplyOnly) k_dm_alltarg_diag<false, true><<<g, QG_THREADS, 0, st>>>(a, d, numKetQubits, ex);
    else k_dm_alltarg_diag<false, false><<<g, QG_THREADS, 0, st>>>(a, d, numKetQubits, ex);
    qg_note_launch();
    return qg_check_launch("dm_allTargDiagMatr");
}

int qg_sv_calcExpecFullStateDiagMatr(const void* amps, int numQubits, const void* elems, qg_cplx exponent, int hasPower,
                                     int useRealPow, qg_cplx* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QG_TRY(check_elems(elems));
    if (!out) return qg_fail(QG_ERR_ARG, "null output");
    const qidx n = (qidx)1 << numQubits;
    const int grid = red_grid(n);
    RedOut r;
    QG_TRY(red_setup(grid, 2, &r));
    cudaStream_t st = qg_stream(stream);
    const double2 ex = d2c(exponent);
    const double2* a = (const double2*)amps;
    const double2* d = (const double2*)elems;
    if (hasPower && useRealPow) k_sv_expec_alltarg<true, true><<<grid, RED_THREADS, 0, st>>>(a, d, n, ex, r);
    else if (hasPower) k_sv_expec_alltarg<true, false><<<grid, RED_THREADS, 0, st>>>(a, d, n, ex, r);
    else k_sv_expec_alltarg<false, false><<<grid, RED_THREADS, 0, st>>>(a, d, n, ex, r);
    qg_note_launch();
    double v[2];
    QG_TRY(red_fetch(r, 2, v, st));
    out->re = v[0];
    out->im = v[1];
    return QG_OK;
}

int qg_dm_calcExpecFullStateDiagMatr(const void* amps, int numKetQubits, const void* elems, qg_cplx exponent, int hasPower,
                                     int useRealPow, qg_cplx* out, void* stream) {
    QG_TRY(qg_check_amps(amps, 2 * numKetQubits));
    QG_TRY(check_elems(elems));
    if (!out) return qg_fail(QG_ERR_ARG, "null output");
    const qidx dim = (qidx)1 << numKetQubits;
    const int grid = red_grid(dim);
    RedOut r;
    QG_TRY(red_setup(grid, 2, &r));
    cudaStream_t st = qg_stream(stream);
    const double2 ex = d2c(exponent);
    const double2* a = (const double2*)amps;
    const double2* d = (const double2*)elems;
    if (hasPower && useRealPow) k_dm_expec_alltarg<true, true><<<grid, RED_THREADS, 0, st>>>(a, d, numKetQubits, ex, r);
    else if (hasPower) k_dm_expec_alltarg<true, false><<<grid, RED_THREADS, 0, st>>>(a, d, numKetQubits, ex, r);
    else k_dm_expec_alltarg<false, false><<<grid, RED_THREADS, 0, st>>>(a, d, numKetQubits, ex, r);
    qg_note_launch();
    double v[2];
    QG_TRY(red_fetch(r, 2, v, st));
    out->re = v[0];
    out->im = v[1];
    return QG_OK;
}

}  // extern "C"
