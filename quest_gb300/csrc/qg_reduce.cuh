// Deterministic single-launch reductions shared by the FP64 and FP32 kernels:
// per-thread FP64 accumulation over a fixed strided subset, warp shuffles, a
// shared-memory tree, per-block partials in library scratch, and a last-block
// (atomic ticket) final sum in block order.
#pragma once

#include "qg_common.cuh"

#include <algorithm>

#define RED_THREADS 256
#define RED_MAX_VALUES 34   // up to 17 complex values per launch

struct RedOut {
    double* partials;        // [NV][gridDim.x]
    unsigned int* ticket;
    double* result;          // [NV]
};

template <int NV>
__device__ __forceinline__ void block_reduce_and_finish(double (&v)[NV], const RedOut& out) {
    __shared__ double sh[NV][RED_THREADS / 32];
    __shared__ bool amLast;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[k][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0;
            for (int w = 0; w < RED_THREADS / 32; w++) s += sh[k][w];
            out.partials[k * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        unsigned int t = atomicAdd(out.ticket, 1u);
        amLast = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    // the last block adds every block's partial in a fixed order
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += RED_THREADS) s += ((volatile double*)out.partials)[k * gridDim.x + b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[k][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0;
            for (int w = 0; w < RED_THREADS / 32; w++) s += sh[k][w];
            out.result[k] = s;
        }
        *out.ticket = 0;
    }
}


// scratch layout: [ticket (256 B)] [results (NV doubles, 256 B aligned)] [partials]
static inline int red_setup_at(void* s, int grid, int nv, RedOut* out) {
    char* base = (char*)s;
    out->ticket = (unsigned int*)base;
    out->result = (double*)(base + 256);
    out->partials = (double*)(base + 256 + ((8 * (size_t)nv + 255) / 256) * 256);
    (void)grid;
    return QG_OK;
}
static inline size_t red_scratch_bytes(int grid, int nv) {
    return 256 + ((8 * (size_t)nv + 255) / 256) * 256 + 8 * (size_t)nv * grid + 256;
}
static inline int red_setup(int grid, int nv, RedOut* out) {
    void* s = nullptr;
    QG_TRY(qg_scratch_get(&s, red_scratch_bytes(grid, nv)));
    return red_setup_at(s, grid, nv, out);
}
static inline int red_grid(qidx work) {
    qidx g = (qidx)qg_num_sms() * 4;
    qidx need = (work + RED_THREADS - 1) / RED_THREADS;
    if (need < g) g = std::max<qidx>(1, need);
    return (int)g;
}
static inline int red_fetch(const RedOut& out, int nv, double* host, cudaStream_t st) {
    QG_TRY(qg_check_launch("reduction"));
    void* pinned = nullptr;
    QG_TRY(qg_pinned_result(&pinned, 8 * (size_t)nv));
    QG_CUDA(cudaMemcpyAsync(pinned, out.result, 8 * (size_t)nv, cudaMemcpyDeviceToHost, st));
    QG_CUDA(cudaStreamSynchronize(st));
    std::copy((double*)pinned, (double*)pinned + nv, host);
    qg_note_launch();
    return QG_OK;
}
// i^k applied to (re, im)
static inline void times_power_of_i(double* re, double* im, int k) {
    double r = *re, i = *im;
    switch (((k % 4) + 4) % 4) {
        case 0: break;
        case 1: *re = -i; *im = r; break;
        case 2: *re = -r; *im = -i; break;
        default: *re = i; *im = -r; break;
    }
}
