// Shared device/host helpers of the sm_103a gate-application backend.
//
// Amplitudes are FP64 complex numbers stored as double2 (16 bytes: one 128-bit
// load or store per amplitude).  Index arithmetic is 64-bit.  A gate enumerates
// the amplitude groups it touches by "bit insertion": the n-th group's base
// index is n with a zero (or fixed control value) opened at each sorted control
// and target position, which is the index map of QuEST's
// insertBitsWithMaskedValues (quest/src/core/bitwise.hpp:206-210).  Consecutive
// threads take consecutive n, so every warp touches contiguous runs of memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/quest_gb300.h"

typedef long long qidx;

#define QG_MAX_QUBITS 50          // amplitude vectors of up to 2^50 elements
#define QG_THREADS 256            // threads per block for the streaming kernels

// ---------------------------------------------------------------- host-side error state

void qg_set_error(const char* fmt, ...);
int qg_fail(int code, const char* fmt, ...);
int qg_check_cuda(cudaError_t e, const char* what);
int qg_check_launch(const char* what);
void qg_note_launch(int n = 1);
int qg_num_sms();

// How general complex FP64 gate products are evaluated (qg_set_fp64_products)
#define QG_FP64_PRODUCTS_FIXED 0   // block-floating 60-bit fixed point on the integer pipes
#define QG_FP64_PRODUCTS_FP64 1    // IEEE FP64 fused multiply-adds
int qg_fp64_products_mode();

// Launch shapes chosen by the autotuner (qg_tune.cu): pairs per thread per loop
// iteration and threads per block, per tunable kernel
struct QgShape { int ppt; int threads; };
#define QG_TUNE_DENSE1 0
#define QG_TUNE_DIAG1 1
#define QG_TUNE_DENSE2 2
#define QG_TUNE_NUM 3
QgShape qg_tuned_shape(int kernel);

#define QG_CUDA(call)                                                      \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) return qg_check_cuda(_e, #call);            \
    } while (0)

#define QG_TRY(expr)                                                       \
    do {                                                                   \
        int _rc = (expr);                                                  \
        if (_rc != QG_OK) return _rc;                                      \
    } while (0)

static inline cudaStream_t qg_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Library-owned device scratch (a growing cache, like QuEST's gpu_getCacheOfSize,
// quest/src/gpu/gpu_config.cpp:639-663).  Reductions keep their per-block partial
// sums and their completion counter here.
int qg_scratch_get(void** out, size_t bytes);
// Pinned host slot for reduction results.
int qg_pinned_result(void** out, size_t bytes);

// ---------------------------------------------------------------- bit insertion

// Low-bit masks (2^q - 1) of up to MAXB sorted qubit positions.
template <int MAXB>
struct InsertList {
    int num;
    qidx low[MAXB];
};

#define QG_MAX_INSERT 24
typedef InsertList<QG_MAX_INSERT> Ins;

// Opens a zero at each listed (ascending) position: the map of QuEST's
// insertBits(n, sortedQubits, k, 0) (bitwise.hpp:164-171).
template <int NB>
__device__ __forceinline__ qidx insert_bits(qidx n, const Ins& ins) {
    if (NB >= 0) {
#pragma unroll
        for (int i = 0; i < (NB >= 0 ? NB : 0); i++) {
            qidx lo = n & ins.low[i];
            n = ((n ^ lo) << 1) | lo;
        }
    } else {
        for (int i = 0; i < ins.num; i++) {
            qidx lo = n & ins.low[i];
            n = ((n ^ lo) << 1) | lo;
        }
    }
    return n;
}

__device__ __forceinline__ int parity64(qidx x) { return __popcll((unsigned long long)x) & 1; }

// ---------------------------------------------------------------- complex arithmetic (FMA form)

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a*b + c
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfmaf(float2 a, float2 b, float2 c) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

// Streaming loads/stores: each amplitude is touched once per kernel, so keep it
// out of L1 and mark it as evict-first in L2.
__device__ __forceinline__ double2 ld_amp(const double2* p) { return __ldcs(p); }
__device__ __forceinline__ void st_amp(double2* p, double2 v) { __stcs(p, v); }

// ---------------------------------------------------------------- host-side qubit bookkeeping

struct QubitPlan {
    Ins ins;          // sorted positions of ctrls (+ fixed targets)
    qidx stateMask;   // bits forced to 1 (ctrls in state 1, fixed target values)
    int numFixed;     // ctrls + fixed targets
};

// Validates and sorts ctrls (+extra fixed bits), building the insertion plan.
// extraQubits/extraValues: targets whose value is fixed in the enumeration.
int qg_make_plan(int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                 const int* extraQubits, const int* extraValues, int numExtra, QubitPlan* plan);
int qg_check_qubits(int numQubits, const int* qubits, int num, const char* what);
int qg_check_amps(const void* amps, int numQubits);

// Launch geometry for `items` work items of one thread each.
static inline unsigned qg_blocks(qidx items, int threads = QG_THREADS) {
    return (unsigned)((items + threads - 1) / threads);
}

// Dispatches a templated launch on the number of inserted bits (0..8, else generic).
#define QG_DISPATCH_NB(nb, LAUNCH)                 \
    switch (nb) {                                  \
        case 0: LAUNCH(0); break;                  \
        case 1: LAUNCH(1); break;                  \
        case 2: LAUNCH(2); break;                  \
        case 3: LAUNCH(3); break;                  \
        case 4: LAUNCH(4); break;                  \
        case 5: LAUNCH(5); break;                  \
        case 6: LAUNCH(6); break;                  \
        default: LAUNCH(-1); break;                \
    }
