// Statevector amplitude kernels of the sm_103a backend (FP64).
//
// One thread owns one amplitude group (a pair for one-target gates, a quad for
// two-target gates, a 2^k block for k-target dense matrices, a single amplitude
// for diagonals).  Group bases come from bit insertion over the sorted control
// and target positions (qg_common.cuh), so a warp reads 32 consecutive groups:
// coalesced 16-byte loads for every target position.  Matrices of up to five
// targets travel in the kernel's parameter space, which the whole warp reads
// with uniform (broadcast) constant-bank loads.  Gates whose structure permits
// it (real matrices, gadgets with a real diagonal factor, permutations, unit
// diagonal entries) run reduced-arithmetic variants, because FP64 issue rate
// rather than HBM bandwidth bounds general complex gates on this part.
//
// Reference algorithms: quest/src/cpu/cpu_subroutines.cpp (index maps and
// arithmetic of each cpu_statevec_* routine) and quest/src/gpu/gpu_kernels.cuh.
#include "qg_common.cuh"
#include "qg_fixed.cuh"

#include <cmath>
#include <complex>
#include <algorithm>
#include <cstring>
#include <vector>
#include <map>
#include <mutex>

// ============================================================== initialisation

__global__ void k_init_uniform(double2* __restrict__ a, qidx n, double2 v) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i < n) st_amp(a + i, v);
}

__global__ void k_set_one(double2* __restrict__ a, qidx index, double2 v) { a[index] = v; }

// initDebugState: amp_k = (2k + i(2k+1)) / 10 (cpu_subroutines.cpp:2364-2376)
__global__ void k_init_debug(double2* __restrict__ a, qidx n) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i < n) st_amp(a + i, make_double2((2.0 * i) / 10.0, (2.0 * i + 1.0) / 10.0));
}

// ============================================================== swap
// cpu_statevec_anyCtrlSwap_subA (cpu_subroutines.cpp:255-280): i01 has the higher
// target at 0 and the lower at 1; it trades places with i10.

template <int NB>
__global__ void k_swap(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx flip) {
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i01 = insert_bits<NB>(n, ins) | mask;
    double2 x = ld_amp(a + i01), y = ld_amp(a + (i01 ^ flip));
    for (;;) {
        // software pipeline: the next group's loads are in flight while this one is stored
        const qidx nn = n + stride;
        const bool more = nn < numIts;
        qidx j01 = 0;
        double2 xn, yn;
        if (more) {
            j01 = insert_bits<NB>(nn, ins) | mask;
            xn = ld_amp(a + j01);
            yn = ld_amp(a + (j01 ^ flip));
        }
        st_amp(a + i01, y);
        st_amp(a + (i01 ^ flip), x);
        if (!more) break;
        n = nn; i01 = j01; x = xn; y = yn;
    }
}

// ============================================================== one-target dense

struct Mat1 { double2 m[4]; };

// MODE 0: general complex 2x2; MODE 1: real 2x2 (imaginary parts all zero).
// Persistent grid-stride loop with the next pair's loads issued before this
// pair's FP64 work, so the FP64 pipe is not left idle while warps wait on memory.
template <int MODE>
__device__ __forceinline__ void dense1_pair(const Mat1& M, double2 x, double2 y, double2& o0, double2& o1) {
    if (MODE == 1) {
        o0 = make_double2(fma(M.m[0].x, x.x, M.m[1].x * y.x), fma(M.m[0].x, x.y, M.m[1].x * y.y));
        o1 = make_double2(fma(M.m[2].x, x.x, M.m[3].x * y.x), fma(M.m[2].x, x.y, M.m[3].x * y.y));
    } else {
        o0 = cfma(M.m[0], x, cmul(M.m[1], y));
        o1 = cfma(M.m[2], x, cmul(M.m[3], y));
    }
}

template <int NB, int MODE>
__global__ void k_dense1(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx tbit, Mat1 M) {
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i0 = insert_bits<NB>(n, ins) | mask;
    double2 x = ld_amp(a + i0), y = ld_amp(a + (i0 | tbit));
    for (;;) {
        const qidx nn = n + stride;
        const bool more = nn < numIts;
        qidx j0 = 0;
        double2 xn, yn;
        if (more) {
            j0 = insert_bits<NB>(nn, ins) | mask;
            xn = ld_amp(a + j0);
            yn = ld_amp(a + (j0 | tbit));
        }
        double2 o0, o1;
        dense1_pair<MODE>(M, x, y, o0, o1);
        st_amp(a + i0, o0);
        st_amp(a + (i0 | tbit), o1);
        if (!more) break;
        n = nn; i0 = j0; x = xn; y = yn;
    }
}

// General complex 2x2 through the integer pipes: each pair is evaluated in
// block-floating 60-bit fixed point (qg_fixed.cuh); a pair holding Inf/NaN or with a
// result outside the normal double range is evaluated in FP64 instead.  Each thread
// takes PPT pairs per iteration (independent work for the integer pipes) and loads
// the next iteration's pairs before computing the current ones.
__device__ __forceinline__ void dense1_fx_pair(const qgfx::Op4& C, const Mat1& M, double2 x, double2 y, double2& o0,
                                               double2& o1) {
    const double in[4] = {x.x, x.y, y.x, y.y};
    double out[4];
    if (qgfx::apply_op_best<4>(C, in, out)) {
        o0 = make_double2(out[0], out[1]);
        o1 = make_double2(out[2], out[3]);
    } else {
        dense1_pair<0>(M, x, y, o0, o1);
    }
}

// The launch bound asks for half the SM's thread slots resident (4 blocks of 256):
// it caps registers at 64, and the extra warps take the kernel from 0.86 to 0.94 of
// the measured HBM rate at 30 qubits.  Each thread keeps NBUF rounds of PPT pairs in
// registers: the loads of the next NBUF - 1 rounds are in flight while one round is
// computed, and the loop is unrolled NBUF times so that no buffer is ever copied (a
// register copy of a pending load would wait for it).
template <int NB, int PPT, int THREADS, int NBUF = 2>
__global__ void __launch_bounds__(THREADS, 2048 / THREADS / 2) k_dense1_fx(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask,
                                                      qidx tbit, qgfx::Op4 C, Mat1 M) {
    const qidx stride = (qidx)gridDim.x * THREADS;
    const qidx span = PPT * stride;
    const qidx tid = blockIdx.x * (qidx)THREADS + threadIdx.x;
    const qidx groups = numIts / span;      // rounds in which all PPT pairs of every thread exist
    if (groups > 0) {
        qidx i0[NBUF][PPT];
        double2 x[NBUF][PPT], y[NBUF][PPT];
        auto load = [&](qidx (&ib)[PPT], double2 (&xb)[PPT], double2 (&yb)[PPT], qidx g) {
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                ib[k] = insert_bits<NB>(g * span + tid + k * stride, ins) | mask;
                xb[k] = ld_amp(a + ib[k]);
                yb[k] = ld_amp(a + (ib[k] | tbit));
            }
        };
#pragma unroll
        for (int b = 0; b < NBUF - 1; b++)
            if (b < groups) load(i0[b], x[b], y[b], b);
        for (qidx g0 = 0; g0 < groups; g0 += NBUF) {
#pragma unroll
            for (int b = 0; b < NBUF; b++) {
                const qidx g = g0 + b;
                if (g >= groups) break;
                const int nb = (b + NBUF - 1) % NBUF;
                if (g + NBUF - 1 < groups) load(i0[nb], x[nb], y[nb], g + NBUF - 1);
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    double2 o0, o1;
                    dense1_fx_pair(C, M, x[b][k], y[b][k], o0, o1);
                    st_amp(a + i0[b][k], o0);
                    st_amp(a + (i0[b][k] | tbit), o1);
                }
            }
        }
    }
    // the remaining pairs, one at a time
    for (qidx n = groups * span + tid; n < numIts; n += stride) {
        const qidx i = insert_bits<NB>(n, ins) | mask;
        double2 o0, o1;
        dense1_fx_pair(C, M, ld_amp(a + i), ld_amp(a + (i | tbit)), o0, o1);
        st_amp(a + i, o0);
        st_amp(a + (i | tbit), o1);
    }
}

// ============================================================== two-target dense

struct Mat2 { double2 m[16]; };

template <int NB>
__global__ void k_dense2(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx b1, qidx b2, Mat2 M) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i00 = insert_bits<NB>(n, ins) | mask;
    qidx idx[4] = {i00, i00 | b1, i00 | b2, i00 | b1 | b2};
    double2 v[4];
#pragma unroll
    for (int j = 0; j < 4; j++) v[j] = ld_amp(a + idx[j]);
#pragma unroll
    for (int r = 0; r < 4; r++) {
        double2 acc = cmul(M.m[4 * r], v[0]);
#pragma unroll
        for (int j = 1; j < 4; j++) acc = cfma(M.m[4 * r + j], v[j], acc);
        st_amp(a + idx[r], acc);
    }
}

// k_dense2 through the integer pipes: the real 8x8 form of the matrix on each group
// of four amplitudes in block-floating fixed point (qg_fixed.cuh); groups holding
// Inf/NaN or with results outside the normal range take the FP64 products.
// NBUF = 1: one group per thread at a time (registers capped at 64 for 4 resident
// blocks of 256).  NBUF = 2: two groups per thread in rotating register buffers, the
// next group's loads in flight while the current one is computed (the loop is unrolled
// over the buffers, so no buffer is copied: a register copy of a pending load would
// wait for it); 3 resident blocks of 256.  The autotuner picks the shape per GPU.
__device__ __forceinline__ void dense2_fx_group(double2* __restrict__ a, qidx i00, qidx b1, qidx b2, const double2 (&v)[4],
                                                const qgfx::OpN<8>& C, const Mat2& M) {
    const double in[8] = {v[0].x, v[0].y, v[1].x, v[1].y, v[2].x, v[2].y, v[3].x, v[3].y};
    double out[8];
    if (qgfx::apply_op_best<8>(C, in, out)) {
        st_amp(a + i00, make_double2(out[0], out[1]));
        st_amp(a + (i00 | b1), make_double2(out[2], out[3]));
        st_amp(a + (i00 | b2), make_double2(out[4], out[5]));
        st_amp(a + (i00 | b1 | b2), make_double2(out[6], out[7]));
    } else {
        const qidx idx[4] = {i00, i00 | b1, i00 | b2, i00 | b1 | b2};
#pragma unroll
        for (int r = 0; r < 4; r++) {
            double2 acc = cmul(M.m[4 * r], v[0]);
#pragma unroll
            for (int j = 1; j < 4; j++) acc = cfma(M.m[4 * r + j], v[j], acc);
            st_amp(a + idx[r], acc);
        }
    }
}

template <int NB, int NBUF, int THREADS>
__global__ void __launch_bounds__(THREADS, (NBUF == 1 ? 1024 : 768) / THREADS) k_dense2_fx(double2* __restrict__ a, qidx numIts,
                                                                                         Ins ins, qidx mask, qidx b1, qidx b2,
                                                                                         qgfx::OpN<8> C, Mat2 M) {
    const qidx stride = (qidx)gridDim.x * THREADS;
    const qidx tid = blockIdx.x * (qidx)THREADS + threadIdx.x;
    auto load = [&](qidx& i00, double2 (&v)[4], qidx n) {
        i00 = insert_bits<NB>(n, ins) | mask;
        v[0] = ld_amp(a + i00);
        v[1] = ld_amp(a + (i00 | b1));
        v[2] = ld_amp(a + (i00 | b2));
        v[3] = ld_amp(a + (i00 | b1 | b2));
    };
    if (NBUF == 1) {
        for (qidx n = tid; n < numIts; n += stride) {
            qidx i00;
            double2 v[4];
            load(i00, v, n);
            dense2_fx_group(a, i00, b1, b2, v, C, M);
        }
        return;
    }
    // rounds g = 0, 1, ...: this thread's group of round g is tid + g * stride
    const qidx rounds = numIts > tid ? (numIts - tid + stride - 1) / stride : 0;
    qidx i0[2];
    double2 v[2][4];
    if (rounds > 0) load(i0[0], v[0], tid);
    for (qidx g = 0; g < rounds; g += 2) {
        if (g + 1 < rounds) load(i0[1], v[1], tid + (g + 1) * stride);
        dense2_fx_group(a, i0[0], b1, b2, v[0], C, M);
        if (g + 1 >= rounds) break;
        if (g + 2 < rounds) load(i0[0], v[0], tid + (g + 2) * stride);
        dense2_fx_group(a, i0[1], b1, b2, v[1], C, M);
    }
}

// ============================================================== few-target dense (3..5 targets)
// Each thread caches its 2^K amplitudes in registers; the matrix (already
// conjugated if requested) sits in parameter space.

template <int K>
struct MatK {
    double2 m[1 << (2 * K)];
    qidx off[1 << K];   // offset of matrix index j from the group base
};

template <int K, int NB>
__global__ void __launch_bounds__(128) k_denseK(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, MatK<K> M) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    constexpr int D = 1 << K;
    qidx base = insert_bits<NB>(n, ins) | mask;
    double2 v[D];
#pragma unroll
    for (int j = 0; j < D; j++) v[j] = ld_amp(a + base + M.off[j]);
#pragma unroll
    for (int r = 0; r < D; r++) {
        double2 acc = cmul(M.m[r * D], v[0]);
#pragma unroll
        for (int j = 1; j < D; j++) acc = cfma(M.m[r * D + j], v[j], acc);
        st_amp(a + base + M.off[r], acc);
    }
}

// k_denseK through the integer pipes (K = 3, 4): the real 2^(K+1)-square form of the
// matrix on each group, inputs put at their common scale once, each output formed and
// stored in turn (qg_fixed.cuh fx_prepare / fx_row); groups that need FP64 use M.
// The operator form per width, as measured on GB300 (28 qubits): three targets run
// 12 % faster with the three-product complex form; four targets keep the real form
// (the complex form's extra (x+y) limbs spill there).
template <int K>
struct DenseKOp { typedef qgfx::OpN<2 << K> type; static constexpr bool complex = false; };
template <>
struct DenseKOp<3> { typedef qgfx::CopN<8> type; static constexpr bool complex = true; };

// Four targets (a 16-amplitude group, the real 32x32 operator): each thread owns a group,
// as k_denseK_fx does, and forms its 32 outputs one row at a time; the operator sits in
// shared memory and every row is read as 16-byte broadcasts (all threads of a warp are on
// the same row), not from the parameter bank, where a row chosen at run time becomes a
// constant-bank load per coefficient.  The limbs and the integer sums are fx_prepare /
// fx_row's, so the bits equal k_denseK_fx's.
template <int NB>
__global__ void __launch_bounds__(128) k_dense4_fx(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, MatK<4> M,
                                                   qgfx::OpN<32> C) {
    constexpr int D = 16, N = 32;
    __shared__ __align__(16) int32_t sh[N][N], sl[N][N];
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
        sh[e / N][e % N] = C.h[e / N][e % N];
        sl[e / N][e % N] = C.l[e / N][e % N];
    }
    __syncthreads();
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    for (qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x; n < numIts; n += stride) {
        const qidx base = insert_bits<NB>(n, ins) | mask;
        double in[N];
#pragma unroll
        for (int j = 0; j < D; j++) {
            const double2 v = ld_amp(a + base + M.off[j]);
            in[2 * j] = v.x;
            in[2 * j + 1] = v.y;
        }
        int32_t xh[N], xl[N];
        uint32_t down;
        bool zero;
        if (qgfx::fx_prepare<N>(C, in, xh, xl, down, zero)) {
#pragma unroll 1
            for (int r = 0; r < D; r++) {
                double out[2];
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const int4* hr = (const int4*)sh[2 * r + c];
                    const int4* lr = (const int4*)sl[2 * r + c];
                    // four independent integer sums (exact, so their order does not matter):
                    // short dependency chains for the integer multiply-add pipe
                    int64_t h0 = 0, h1 = 0, m0 = 0, m1 = 0;
#pragma unroll
                    for (int q = 0; q < N / 4; q++) {
                        const int4 H = hr[q], Lo = lr[q];
                        h0 += (int64_t)xh[4 * q] * H.x;     m0 += (int64_t)xh[4 * q] * Lo.x;     m1 += (int64_t)xl[4 * q] * H.x;
                        h1 += (int64_t)xh[4 * q + 1] * H.y; m0 += (int64_t)xh[4 * q + 1] * Lo.y; m1 += (int64_t)xl[4 * q + 1] * H.y;
                        h0 += (int64_t)xh[4 * q + 2] * H.z; m0 += (int64_t)xh[4 * q + 2] * Lo.z; m1 += (int64_t)xl[4 * q + 2] * H.z;
                        h1 += (int64_t)xh[4 * q + 3] * H.w; m0 += (int64_t)xh[4 * q + 3] * Lo.w; m1 += (int64_t)xl[4 * q + 3] * H.w;
                    }
                    out[c] = zero ? 0.0 : qgfx::fx_to_double((h0 + h1) + ((m0 + m1) >> 32), down);
                }
                st_amp(a + base + M.off[r], make_double2(out[0], out[1]));
            }
        } else {
            // nothing has been stored: reload the group and use FP64
            double2 v[D];
#pragma unroll
            for (int j = 0; j < D; j++) v[j] = a[base + M.off[j]];
#pragma unroll 1
            for (int r = 0; r < D; r++) {
                double2 acc = cmul(M.m[r * D], v[0]);
#pragma unroll
                for (int j = 1; j < D; j++) acc = cfma(M.m[r * D + j], v[j], acc);
                st_amp(a + base + M.off[r], acc);
            }
        }
    }
}

template <int K, int NB>
__global__ void __launch_bounds__(128) k_denseK_fx(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, MatK<K> M,
                                                  typename DenseKOp<K>::type C) {
    constexpr int D = 1 << K, N = 2 << K;
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    for (qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x; n < numIts; n += stride) {
        const qidx base = insert_bits<NB>(n, ins) | mask;
        double in[N];
#pragma unroll
        for (int j = 0; j < D; j++) {
            const double2 v = ld_amp(a + base + M.off[j]);
            in[2 * j] = v.x;
            in[2 * j + 1] = v.y;
        }
        bool done = false;
        if constexpr (DenseKOp<K>::complex) {
            int32_t xh[D], xl[D], yh[D], yl[D], sh[D], sl[D];
            uint32_t down;
            bool zero;
            if (qgfx::cfx_prepare<D>(C, in, xh, xl, yh, yl, sh, sl, down, zero)) {
#pragma unroll
                for (int r = 0; r < D; r++) {
                    double re, im;
                    qgfx::cfx_row<D>(C, r, xh, xl, yh, yl, sh, sl, down, zero, re, im);
                    st_amp(a + base + M.off[r], make_double2(re, im));
                }
                done = true;
            }
        } else {
            int32_t xh[N], xl[N];
            uint32_t down;
            bool zero;
            if (qgfx::fx_prepare<N>(C, in, xh, xl, down, zero)) {
                // rows one after another (fully unrolled, the schedule runs out of registers)
#pragma unroll 1
                for (int r = 0; r < D; r++)
                    st_amp(a + base + M.off[r], make_double2(qgfx::fx_row<N>(C, 2 * r, xh, xl, down, zero),
                                                             qgfx::fx_row<N>(C, 2 * r + 1, xh, xl, down, zero)));
                done = true;
            }
        }
        if (!done) {
            // nothing has been stored: reload the group (keeping the inputs live across the
            // fixed-point path would not fit in registers at K = 4)
            double2 v[D];
#pragma unroll
            for (int j = 0; j < D; j++) v[j] = a[base + M.off[j]];
#pragma unroll
            for (int r = 0; r < D; r++) {
                double2 acc = cmul(M.m[r * D], v[0]);
#pragma unroll
                for (int j = 1; j < D; j++) acc = cfma(M.m[r * D + j], v[j], acc);
                st_amp(a + base + M.off[r], acc);
            }
        }
    }
}

// ============================================================== many-target dense (>= 6 targets)
// One CTA per 2^K block: the block's amplitudes are staged in `cache` (shared
// memory, or a per-CTA slot of global scratch beyond shared capacity), then each
// thread forms whole output rows from the column-major matrix in global memory.

__global__ void k_denseMany(double2* __restrict__ a, qidx numBlocks, int K, Ins ins, qidx mask,
                            const qidx* __restrict__ off, const double2* __restrict__ McolMajor,
                            double2* __restrict__ globalCache) {
    extern __shared__ double2 smem[];
    const int D = 1 << K;
    double2* cache = globalCache ? globalCache + (qidx)blockIdx.x * D : smem;
    for (qidx blk = blockIdx.x; blk < numBlocks; blk += gridDim.x) {
        qidx base = insert_bits<-1>(blk, ins) | mask;
        for (int j = threadIdx.x; j < D; j += blockDim.x) cache[j] = a[base + off[j]];
        __syncthreads();
        for (int r = threadIdx.x; r < D; r += blockDim.x) {
            double2 acc = make_double2(0, 0);
            for (int j = 0; j < D; j++) acc = cfma(McolMajor[(qidx)j * D + r], cache[j], acc);
            a[base + off[r]] = acc;
        }
        __syncthreads();
    }
}

// ============================================================== diagonals

// MODE 0: factor d[bit t]; MODE 1: single factor d0 on every visited amplitude
template <int NB, int MODE>
__global__ void k_diag1(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx tbit, double2 d0, double2 d1) {
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i = insert_bits<NB>(n, ins) | mask;
    double2 x = ld_amp(a + i);
    for (;;) {
        const qidx nn = n + stride;
        const bool more = nn < numIts;
        qidx j = 0;
        double2 xn;
        if (more) {
            j = insert_bits<NB>(nn, ins) | mask;
            xn = ld_amp(a + j);
        }
        double2 f = (MODE == 1) ? d0 : ((i & tbit) ? d1 : d0);
        st_amp(a + i, cmul(f, x));
        if (!more) break;
        n = nn; i = j; x = xn;
    }
}

// k_diag1 through the integer pipes: each amplitude times its factor in block-floating
// fixed point (qg_fixed.cuh); amplitudes holding Inf/NaN or with a result outside the
// normal range take the FP64 product instead.
__device__ __forceinline__ double2 diag1_fx_amp(const qgfx::Op2& F, double2 f, double2 x) {
    const double in[2] = {x.x, x.y};
    double out[2];
    if (qgfx::apply_op_best<2>(F, in, out)) return make_double2(out[0], out[1]);
    return cmul(f, x);
}

// MODE 1: every visited amplitude times F0 (the target bit is part of the fixed mask);
// MODE 0: F0 or F1 by the target bit.  PPT amplitudes per thread per round, NBUF rounds
// in registers: the next NBUF - 1 rounds' loads are in flight while one round's
// products are formed (the loop is unrolled NBUF times, so no buffer is copied).
template <int NB, int MODE, int PPT, int THREADS, int NBUF = 2>
__global__ void __launch_bounds__(THREADS) k_diag1_fx(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx tbit,
                                                     double2 d0, double2 d1, qgfx::Op2 F0, qgfx::Op2 F1) {
    const qidx stride = (qidx)gridDim.x * THREADS;
    const qidx span = PPT * stride;
    const qidx tid = blockIdx.x * (qidx)THREADS + threadIdx.x;
    const qidx groups = numIts / span;
    if (groups > 0) {
        qidx i[NBUF][PPT];
        double2 x[NBUF][PPT];
        auto load = [&](qidx (&ib)[PPT], double2 (&xb)[PPT], qidx g) {
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                ib[k] = insert_bits<NB>(g * span + tid + k * stride, ins) | mask;
                xb[k] = a[ib[k]];   // default caching: the amplitude's sector stays in L2 until it is stored
            }
        };
#pragma unroll
        for (int b = 0; b < NBUF - 1; b++)
            if (b < groups) load(i[b], x[b], b);
        for (qidx g0 = 0; g0 < groups; g0 += NBUF) {
#pragma unroll
            for (int b = 0; b < NBUF; b++) {
                const qidx g = g0 + b;
                if (g >= groups) break;
                const int nb = (b + NBUF - 1) % NBUF;
                if (g + NBUF - 1 < groups) load(i[nb], x[nb], g + NBUF - 1);
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    const bool second = (MODE == 0) && (i[b][k] & tbit);
                    st_amp(a + i[b][k], diag1_fx_amp(second ? F1 : F0, second ? d1 : d0, x[b][k]));
                }
            }
        }
    }
    for (qidx n = groups * span + tid; n < numIts; n += stride) {
        const qidx ii = insert_bits<NB>(n, ins) | mask;
        const bool second = (MODE == 0) && (ii & tbit);
        st_amp(a + ii, diag1_fx_amp(second ? F1 : F0, second ? d1 : d0, a[ii]));
    }
}

struct Diag4 { double2 d[4]; };

template <int NB>
__global__ void k_diag2(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, int t1, int t2, Diag4 D) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i = insert_bits<NB>(n, ins) | mask;
    int k = (int)(((i >> t2) & 1) << 1 | ((i >> t1) & 1));
    st_amp(a + i, cmul(D.d[k], ld_amp(a + i)));
}

#define QG_DIAG_PARAM_MAX 10   // up to 2^10 diagonal elements in parameter space

struct DiagK {
    double2 d[1 << QG_DIAG_PARAM_MAX];
    int t[QG_DIAG_PARAM_MAX];
    int k;
};
struct DiagKDev {
    const double2* d;
    int t[QG_MAX_QUBITS];
    int k;
};

template <int NB, typename DT>
__device__ __forceinline__ double2 diagk_elem(const DT& D, qidx i);

template <int NB>
__global__ void k_diagK(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, DiagK D) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i = insert_bits<NB>(n, ins) | mask;
    int v = 0;
    for (int b = 0; b < D.k; b++) v |= (int)((i >> D.t[b]) & 1) << b;
    st_amp(a + i, cmul(D.d[v], ld_amp(a + i)));
}

template <int NB>
__global__ void k_diagKdev(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, DiagKDev D) {
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i = insert_bits<NB>(n, ins) | mask;
    qidx v = 0;
    for (int b = 0; b < D.k; b++) v |= ((i >> D.t[b]) & 1) << b;
    st_amp(a + i, cmul(__ldg(D.d + v), ld_amp(a + i)));
}

// ============================================================== Pauli tensors and gadgets
// Pairs (iA, iB = iA ^ maskXY), enumerated by fixing the highest X/Y target of
// iA to zero: the same set of pairs as cpu_statevector_anyCtrlPauliTensorOrGadget_subA
// (cpu_subroutines.cpp:802-906), each visited once.
//   a'A = f0*aA + f1*sign(iB)*aB,  a'B = f0*aB + f1*sign(iA)*aA
// with sign(i) = (-1)^parity(i & maskYZ) and f1 already scaled by i^numY.

__device__ __forceinline__ double neg_if(double x, int s) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)s << 63));
}

// MODE 0: general complex f0, f1.  MODE 1: f0 real, f1 real (f1.y == 0).
// MODE 2: f0 real, f1 imaginary (f1.x == 0).  MODE 3: f0 == 0, f1 in {1,i,-1,-i}: pure permutation.
template <int MODE>
__device__ __forceinline__ void pauli_pair(double2 f0, double2 f1, int sA, int sB, double2 x, double2 y, double2& oA, double2& oB) {
    if (MODE == 0) {
        double2 gA = make_double2(neg_if(f1.x, sB), neg_if(f1.y, sB));
        double2 gB = make_double2(neg_if(f1.x, sA), neg_if(f1.y, sA));
        oA = cfma(f0, x, cmul(gA, y));
        oB = cfma(f0, y, cmul(gB, x));
    } else if (MODE == 1) {
        double gA = neg_if(f1.x, sB), gB = neg_if(f1.x, sA);
        oA = make_double2(fma(f0.x, x.x, gA * y.x), fma(f0.x, x.y, gA * y.y));
        oB = make_double2(fma(f0.x, y.x, gB * x.x), fma(f0.x, y.y, gB * x.y));
    } else if (MODE == 2) {
        // f1 = i*g: (i g) * (yr + i yi) = (-g yi, g yr)
        double gA = neg_if(f1.y, sB), gB = neg_if(f1.y, sA);
        oA = make_double2(fma(f0.x, x.x, -gA * y.y), fma(f0.x, x.y, gA * y.x));
        oB = make_double2(fma(f0.x, y.x, -gB * x.y), fma(f0.x, y.y, gB * x.x));
    } else {
        // f1 in {1, i, -1, -i}: multiply by a unit of the Gaussian integers without FP work
        bool imag = (f1.y != 0.0);
        int neg = imag ? (f1.y < 0) : (f1.x < 0);
        if (imag) {   // (i s)(yr + i yi) = (-s yi, s yr)
            oA = make_double2(neg_if(y.y, !(neg ^ sB)), neg_if(y.x, neg ^ sB));
            oB = make_double2(neg_if(x.y, !(neg ^ sA)), neg_if(x.x, neg ^ sA));
        } else {
            oA = make_double2(neg_if(y.x, neg ^ sB), neg_if(y.y, neg ^ sB));
            oB = make_double2(neg_if(x.x, neg ^ sA), neg_if(x.y, neg ^ sA));
        }
    }
}

template <int NB, int MODE>
__global__ void k_pauli(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx maskXY, qidx maskYZ,
                        double2 f0, double2 f1) {
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx iA = insert_bits<NB>(n, ins) | mask;
    double2 x = ld_amp(a + iA), y = ld_amp(a + (iA ^ maskXY));
    for (;;) {
        const qidx nn = n + stride;
        const bool more = nn < numIts;
        qidx jA = 0;
        double2 xn, yn;
        if (more) {
            jA = insert_bits<NB>(nn, ins) | mask;
            xn = ld_amp(a + jA);
            yn = ld_amp(a + (jA ^ maskXY));
        }
        const qidx iB = iA ^ maskXY;
        const int sA = parity64(iA & maskYZ), sB = parity64(iB & maskYZ);   // 1 means minus
        double2 oA, oB;
        pauli_pair<MODE>(f0, f1, sA, sB, x, y, oA, oB);
        st_amp(a + iA, oA);
        st_amp(a + iB, oB);
        if (!more) break;
        n = nn; iA = jA; x = xn; y = yn;
    }
}

// cpu_statevector_anyCtrlAnyTargZOrPhaseGadget_sub (cpu_subroutines.cpp:962-990).
// MODE 0: general complex factors.  MODE 1: f0 = 1 and f1 = -1 (Z tensor): only
// odd-parity amplitudes change, by a sign flip.
template <int NB, int MODE>
__global__ void k_zphase(double2* __restrict__ a, qidx numIts, Ins ins, qidx mask, qidx tmask, double2 f0, double2 f1) {
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx i = insert_bits<NB>(n, ins) | mask;
    double2 x = ld_amp(a + i);
    for (;;) {
        const qidx nn = n + stride;
        const bool more = nn < numIts;
        qidx j = 0;
        double2 xn;
        if (more) {
            j = insert_bits<NB>(nn, ins) | mask;
            xn = ld_amp(a + j);
        }
        const int p = parity64(i & tmask);
        if (MODE == 1) st_amp(a + i, make_double2(neg_if(x.x, p), neg_if(x.y, p)));
        else st_amp(a + i, cmul(p ? f1 : f0, x));
        if (!more) break;
        n = nn; i = j; x = xn;
    }
}

// cpu_statevec_multiQubitProjector_sub (cpu_subroutines.cpp:2281-2306)
__global__ void k_projector(double2* __restrict__ a, qidx numAmps, qidx qmask, qidx retainBits, double renorm) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i >= numAmps) return;
    if ((i & qmask) == retainBits) {
        double2 x = ld_amp(a + i);
        st_amp(a + i, make_double2(renorm * x.x, renorm * x.y));
    } else {
        st_amp(a + i, make_double2(0.0, 0.0));
    }
}

// ============================================================== host side

namespace {

double2 d2(qg_cplx c) { return make_double2(c.re, c.im); }

#define QG_LAUNCH_PLAIN(KERNEL, NBV, ...) \
    KERNEL<NBV><<<qg_blocks(numIts), QG_THREADS, 0, st>>>(__VA_ARGS__)

// One resident wave of 256-thread blocks (8 per SM), or fewer when there is less work:
// the grid-stride kernels below then stream their groups with loads in flight.
unsigned persistent_blocks(qidx items) {
    qidx full = (qidx)qg_num_sms() * 8;
    qidx need = (items + QG_THREADS - 1) / QG_THREADS;
    return (unsigned)(need < full ? need : full);
}

// a persistent grid of as many QG_THREADS-blocks as stay resident on every SM
// (the fixed-point kernels hold more registers than the FP64 ones)
template <typename Kernel>
unsigned resident_blocks(Kernel k, qidx items, int threads = QG_THREADS) {
    static std::mutex mu;
    static std::map<const void*, int> perSm;
    int b = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = perSm.find((const void*)k);
        if (it == perSm.end()) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, threads, 0) != cudaSuccess || b < 1) b = 1;
            perSm[(const void*)k] = b;
        } else {
            b = it->second;
        }
    }
    qidx full = (qidx)qg_num_sms() * b;
    qidx need = (items + threads - 1) / threads;
    return (unsigned)(need < full ? need : full);
}

// k_dense1_fx with a launch shape (pairs per thread per iteration, threads per block)
template <int PPT, int THREADS>
int launch_dense1_fx_shape(const QubitPlan& p, qidx numIts, double2* amps, qidx tbit, const qgfx::Op4& C, const Mat1& M,
                           cudaStream_t st) {
    const qidx groups = (numIts + PPT - 1) / PPT;
#define L(NBV) k_dense1_fx<NBV, PPT, THREADS><<<resident_blocks(k_dense1_fx<NBV, PPT, THREADS>, groups, THREADS), THREADS, 0, st>>>(amps, numIts, p.ins, p.stateMask, tbit, C, M)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    return QG_OK;
}

int launch_dense1_fx(QgShape shape, const QubitPlan& p, qidx numIts, double2* amps, qidx tbit, const qgfx::Op4& C,
                     const Mat1& M, cudaStream_t st) {
    switch (shape.ppt * 1000 + shape.threads) {
        case 1128: return launch_dense1_fx_shape<1, 128>(p, numIts, amps, tbit, C, M, st);
        case 2128: return launch_dense1_fx_shape<2, 128>(p, numIts, amps, tbit, C, M, st);
        case 2256: return launch_dense1_fx_shape<2, 256>(p, numIts, amps, tbit, C, M, st);
        default: return launch_dense1_fx_shape<1, 256>(p, numIts, amps, tbit, C, M, st);
    }
}

// k_dense2_fx with a launch shape (groups in flight per thread, threads per block)
template <int NBUF, int THREADS>
int launch_dense2_fx_shape(const QubitPlan& p, qidx numIts, double2* amps, qidx b1, qidx b2, const qgfx::OpN<8>& C,
                           const Mat2& M, cudaStream_t st) {
#define L(NBV) k_dense2_fx<NBV, NBUF, THREADS><<<resident_blocks(k_dense2_fx<NBV, NBUF, THREADS>, numIts, THREADS), THREADS, 0, st>>>(amps, numIts, p.ins, p.stateMask, b1, b2, C, M)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    return QG_OK;
}

int launch_dense2_fx(QgShape shape, const QubitPlan& p, qidx numIts, double2* amps, qidx b1, qidx b2, const qgfx::OpN<8>& C,
                     const Mat2& M, cudaStream_t st) {
    switch (shape.ppt * 1000 + shape.threads) {
        case 1128: return launch_dense2_fx_shape<1, 128>(p, numIts, amps, b1, b2, C, M, st);
        case 2128: return launch_dense2_fx_shape<2, 128>(p, numIts, amps, b1, b2, C, M, st);
        case 2256: return launch_dense2_fx_shape<2, 256>(p, numIts, amps, b1, b2, C, M, st);
        default: return launch_dense2_fx_shape<1, 256>(p, numIts, amps, b1, b2, C, M, st);
    }
}

template <int MODE, int PPT, int THREADS>
int launch_diag1_fx_shape(const QubitPlan& p, qidx numIts, double2* amps, qidx tbit, double2 d0, double2 d1,
                          const qgfx::Op2& F0, const qgfx::Op2& F1, cudaStream_t st) {
    const qidx groups = (numIts + PPT - 1) / PPT;
#define L(NBV) k_diag1_fx<NBV, MODE, PPT, THREADS><<<resident_blocks(k_diag1_fx<NBV, MODE, PPT, THREADS>, groups, THREADS), THREADS, 0, st>>>(amps, numIts, p.ins, p.stateMask, tbit, d0, d1, F0, F1)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    return QG_OK;
}

template <int MODE>
int launch_diag1_fx(QgShape shape, const QubitPlan& p, qidx numIts, double2* amps, qidx tbit, double2 d0, double2 d1,
                    const qgfx::Op2& F0, const qgfx::Op2& F1, cudaStream_t st) {
    switch (shape.ppt * 1000 + shape.threads) {
        case 1128: return launch_diag1_fx_shape<MODE, 1, 128>(p, numIts, amps, tbit, d0, d1, F0, F1, st);
        case 2128: return launch_diag1_fx_shape<MODE, 2, 128>(p, numIts, amps, tbit, d0, d1, F0, F1, st);
        case 2256: return launch_diag1_fx_shape<MODE, 2, 256>(p, numIts, amps, tbit, d0, d1, F0, F1, st);
        default: return launch_diag1_fx_shape<MODE, 1, 256>(p, numIts, amps, tbit, d0, d1, F0, F1, st);
    }
}

// the limb form of a complex 2x2 (row-major) for k_dense1_fx; false: keep FP64
bool make_fx(const qg_cplx* matr, qgfx::Op4& C) {
    double u[8], R[16];
    for (int i = 0; i < 4; i++) { u[2 * i] = matr[i].re; u[2 * i + 1] = matr[i].im; }
    qgfx::real_form_2x2(u, R);
    return qgfx::make_op4(R, C);
}

}  // namespace

extern "C" {

int qg_sv_initUniformState(void* amps, int numQubits, qg_cplx amp, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    qidx n = (qidx)1 << numQubits;
    k_init_uniform<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, n, d2(amp));
    qg_note_launch();
    return qg_check_launch("init_uniform");
}

int qg_sv_initClassicalState(void* amps, int numQubits, int64_t index, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    qidx n = (qidx)1 << numQubits;
    if (index < 0 || index >= n) return qg_fail(QG_ERR_ARG, "basis index %lld outside [0, %lld)", (long long)index, n);
    k_init_uniform<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, n, make_double2(0, 0));
    k_set_one<<<1, 1, 0, qg_stream(stream)>>>((double2*)amps, index, make_double2(1, 0));
    qg_note_launch(2);
    return qg_check_launch("init_classical");
}

int qg_sv_initDebugState(void* amps, int numQubits, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    qidx n = (qidx)1 << numQubits;
    k_init_debug<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, n);
    qg_note_launch();
    return qg_check_launch("init_debug");
}

int qg_sv_anyCtrlSwap(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                      int targ1, int targ2, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (targ1 == targ2) return qg_fail(QG_ERR_ARG, "swap targets must differ");
    if (targ1 > targ2) { int t = targ1; targ1 = targ2; targ2 = t; }
    int tq[2] = {targ2, targ1}, tv[2] = {0, 1};
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, tq, tv, 2, &p));
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    qidx flip = ((qidx)1 << targ1) | ((qidx)1 << targ2);
    cudaStream_t st = qg_stream(stream);
#define L(NBV) k_swap<NBV><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, flip)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    qg_note_launch();
    return qg_check_launch("swap");
}

int qg_sv_anyCtrlOneTargDenseMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                  int targ, const qg_cplx* matr, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (!matr) return qg_fail(QG_ERR_ARG, "null matrix");
    int tv = 0;
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, &targ, &tv, 1, &p));
    Mat1 M;
    qgfx::Op4 C;
    bool real = true;
    for (int i = 0; i < 4; i++) {
        M.m[i] = d2(matr[i]);
        if (matr[i].im != 0.0) real = false;
    }
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    qidx tbit = (qidx)1 << targ;
    cudaStream_t st = qg_stream(stream);
    if (qg_fp64_products_mode() == QG_FP64_PRODUCTS_FIXED && make_fx(matr, C)) {
        QG_TRY(launch_dense1_fx(qg_tuned_shape(QG_TUNE_DENSE1), p, numIts, (double2*)amps, tbit, C, M, st));
    } else if (real) {
#define L(NBV) k_dense1<NBV, 1><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, tbit, M)
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
    } else {
#define L(NBV) k_dense1<NBV, 0><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, tbit, M)
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
    }
    qg_note_launch();
    return qg_check_launch("dense1");
}

int qg_sv_anyCtrlTwoTargDenseMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                  int targ1, int targ2, const qg_cplx* matr, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (!matr) return qg_fail(QG_ERR_ARG, "null matrix");
    int tq[2] = {targ1, targ2}, tv[2] = {0, 0};
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, tq, tv, 2, &p));
    Mat2 M;
    for (int i = 0; i < 16; i++) M.m[i] = d2(matr[i]);
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    qidx b1 = (qidx)1 << targ1, b2 = (qidx)1 << targ2;
    cudaStream_t st = qg_stream(stream);
    double u[32], R[64];
    for (int i = 0; i < 16; i++) { u[2 * i] = matr[i].re; u[2 * i + 1] = matr[i].im; }
    qgfx::real_form(u, 4, R);
    qgfx::OpN<8> C;
    if (qg_fp64_products_mode() == QG_FP64_PRODUCTS_FIXED && qgfx::make_op<8>(R, C)) {
        QG_TRY(launch_dense2_fx(qg_tuned_shape(QG_TUNE_DENSE2), p, numIts, (double2*)amps, b1, b2, C, M, st));
    } else {
#define L(NBV) QG_LAUNCH_PLAIN(k_dense2, NBV, (double2*)amps, numIts, p.ins, p.stateMask, b1, b2, M)
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
    }
    qg_note_launch();
    return qg_check_launch("dense2");
}

}  // extern "C"

bool qg_dense_tc_wanted(qidx numIts);
template <int K>
int qg_dense_tc_launch(double2* amps, qidx numIts, const Ins& ins, qidx mask, const double2* m, const qidx* off,
                       cudaStream_t st, bool* used);

namespace {

template <int K>
int launch_denseK(double2* amps, qidx numIts, const QubitPlan& p, const qg_cplx* matr, const int* targs, int conj, cudaStream_t st) {
    MatK<K> M;
    constexpr int D = 1 << K;
    for (int i = 0; i < D * D; i++) M.m[i] = make_double2(matr[i].re, conj ? -matr[i].im : matr[i].im);
    for (int j = 0; j < D; j++) {
        qidx o = 0;
        for (int b = 0; b < K; b++)
            if ((j >> b) & 1) o |= (qidx)1 << targs[b];
        M.off[j] = o;
    }
    if constexpr (K == 3 || K == 4) {
        // exact 8-bit slices on the tensor cores (qg_dense_tc.cu)
        if (qg_fp64_products_mode() == QG_FP64_PRODUCTS_FIXED && qg_dense_tc_wanted(numIts)) {
            bool used = false;
            QG_TRY(qg_dense_tc_launch<K>(amps, numIts, p.ins, p.stateMask, M.m, M.off, st, &used));
            if (used) return QG_OK;
        }
    }
    if constexpr (K <= 4) {
        if (qg_fp64_products_mode() == QG_FP64_PRODUCTS_FIXED) {
            std::vector<double> u(2 * D * D), R(4 * D * D);
            for (int i = 0; i < D * D; i++) { u[2 * i] = M.m[i].x; u[2 * i + 1] = M.m[i].y; }
            typename DenseKOp<K>::type C;
            bool ok;
            if constexpr (DenseKOp<K>::complex) {
                ok = qgfx::make_cop<D>(u.data(), C);
            } else {
                qgfx::real_form(u.data(), D, R.data());
                ok = qgfx::make_op<2 * D>(R.data(), C);
            }
            if constexpr (K == 4) {
                if (ok) {
                    // the operator as shared-memory broadcasts
#define L(NBV) k_dense4_fx<NBV><<<resident_blocks(k_dense4_fx<NBV>, numIts, 128), 128, 0, st>>>(amps, numIts, p.ins, p.stateMask, M, C)
                    QG_DISPATCH_NB(p.numFixed, L)
#undef L
                    return QG_OK;
                }
            } else if (ok) {
#define L(NBV) k_denseK_fx<K, NBV><<<resident_blocks(k_denseK_fx<K, NBV>, numIts, 128), 128, 0, st>>>(amps, numIts, p.ins, p.stateMask, M, C)
                QG_DISPATCH_NB(p.numFixed, L)
#undef L
                return QG_OK;
            }
        }
    }
    unsigned blocks = (unsigned)((numIts + 127) / 128);
#define L(NBV) k_denseK<K, NBV><<<blocks, 128, 0, st>>>(amps, numIts, p.ins, p.stateMask, M)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    return QG_OK;
}

}  // namespace

extern "C" {

int qg_sv_anyCtrlAnyTargDenseMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                  const int* targs, int numTargs, const qg_cplx* matr, int applyConj, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (!matr) return qg_fail(QG_ERR_ARG, "null matrix");
    if (numTargs < 1) return qg_fail(QG_ERR_ARG, "at least one target is required");
    if (numTargs <= 2) {
        // the bespoke one- and two-target kernels (as localiser.cpp:1051-1076 diverts)
        int D = 1 << numTargs;
        qg_cplx m[16];
        for (int i = 0; i < D * D; i++) m[i] = {matr[i].re, applyConj ? -matr[i].im : matr[i].im};
        if (numTargs == 1) return qg_sv_anyCtrlOneTargDenseMatr(amps, numQubits, ctrls, ctrlStates, numCtrls, targs[0], m, stream);
        return qg_sv_anyCtrlTwoTargDenseMatr(amps, numQubits, ctrls, ctrlStates, numCtrls, targs[0], targs[1], m, stream);
    }
    std::vector<int> zeros(numTargs, 0);
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, targs, zeros.data(), numTargs, &p));
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    cudaStream_t st = qg_stream(stream);
    switch (numTargs) {
        case 3: QG_TRY(launch_denseK<3>((double2*)amps, numIts, p, matr, targs, applyConj, st)); break;
        case 4: QG_TRY(launch_denseK<4>((double2*)amps, numIts, p, matr, targs, applyConj, st)); break;
        case 5: QG_TRY(launch_denseK<5>((double2*)amps, numIts, p, matr, targs, applyConj, st)); break;
        default: {
            // matrix (column-major, conjugated if asked) and target offsets in stream-ordered device memory
            int K = numTargs;
            qidx D = (qidx)1 << K;
            std::vector<double2> colMajor((size_t)(D * D));
            for (qidx r = 0; r < D; r++)
                for (qidx c = 0; c < D; c++) {
                    qg_cplx e = matr[r * D + c];
                    colMajor[(size_t)(c * D + r)] = make_double2(e.re, applyConj ? -e.im : e.im);
                }
            std::vector<qidx> off((size_t)D);
            for (qidx j = 0; j < D; j++) {
                qidx o = 0;
                for (int b = 0; b < K; b++)
                    if ((j >> b) & 1) o |= (qidx)1 << targs[b];
                off[(size_t)j] = o;
            }
            size_t matBytes = sizeof(double2) * (size_t)(D * D), offBytes = sizeof(qidx) * (size_t)D;
            int sms = qg_num_sms();
            bool useSmem = (size_t)D * sizeof(double2) <= 96 * 1024;
            qidx grid = std::min<qidx>(numIts, (qidx)sms * 8);
            size_t cacheBytes = useSmem ? 0 : sizeof(double2) * (size_t)(D * grid);
            char* dev = nullptr;
            QG_CUDA(cudaMallocAsync((void**)&dev, matBytes + offBytes + cacheBytes, st));
            QG_CUDA(cudaMemcpyAsync(dev, colMajor.data(), matBytes, cudaMemcpyHostToDevice, st));
            QG_CUDA(cudaMemcpyAsync(dev + matBytes, off.data(), offBytes, cudaMemcpyHostToDevice, st));
            size_t smemBytes = useSmem ? (size_t)D * sizeof(double2) : 0;
            if (smemBytes > 48 * 1024)
                QG_CUDA(cudaFuncSetAttribute(k_denseMany, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes));
            k_denseMany<<<(unsigned)grid, 256, smemBytes, st>>>((double2*)amps, numIts, K, p.ins, p.stateMask,
                                                                 (const qidx*)(dev + matBytes), (const double2*)dev,
                                                                 useSmem ? nullptr : (double2*)(dev + matBytes + offBytes));
            QG_TRY(qg_check_launch("denseMany"));
            QG_CUDA(cudaFreeAsync(dev, st));
        }
    }
    qg_note_launch();
    return qg_check_launch("denseK");
}

int qg_sv_anyCtrlOneTargDiagMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                 int targ, const qg_cplx* elems, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (!elems) return qg_fail(QG_ERR_ARG, "null diagonal");
    QG_TRY(qg_check_qubits(numQubits, &targ, 1, "target"));
    for (int i = 0; i < numCtrls; i++)
        if (ctrls[i] == targ) return qg_fail(QG_ERR_ARG, "control %d is also the target", targ);
    bool one0 = elems[0].re == 1.0 && elems[0].im == 0.0;
    bool one1 = elems[1].re == 1.0 && elems[1].im == 0.0;
    cudaStream_t st = qg_stream(stream);
    if (one0 && one1) return QG_OK;   // the identity: nothing changes
    if (one0 || one1) {
        // only amplitudes whose factor differs from 1 are visited
        int tv = one0 ? 1 : 0;
        QubitPlan p;
        QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, &targ, &tv, 1, &p));
        qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
        double2 f = d2(one0 ? elems[1] : elems[0]);
        qgfx::Op2 F;
        if (qg_fp64_products_mode() == QG_FP64_PRODUCTS_FIXED && qgfx::make_scalar_op(f.x, f.y, F)) {
            QG_TRY(launch_diag1_fx<1>(qg_tuned_shape(QG_TUNE_DIAG1), p, numIts, (double2*)amps, 0, f, f, F, F, st));
        } else {
#define L(NBV) k_diag1<NBV, 1><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, 0, f, f)
            QG_DISPATCH_NB(p.numFixed, L)
#undef L
        }
    } else {
        QubitPlan p;
        QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, nullptr, nullptr, 0, &p));
        qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
        qidx tbit = (qidx)1 << targ;
        qgfx::Op2 F0, F1;
        if (qg_fp64_products_mode() == QG_FP64_PRODUCTS_FIXED && qgfx::make_scalar_op(elems[0].re, elems[0].im, F0) &&
            qgfx::make_scalar_op(elems[1].re, elems[1].im, F1)) {
            QG_TRY(launch_diag1_fx<0>(qg_tuned_shape(QG_TUNE_DIAG1), p, numIts, (double2*)amps, tbit, d2(elems[0]),
                                      d2(elems[1]), F0, F1, st));
        } else {
#define L(NBV) k_diag1<NBV, 0><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, tbit, d2(elems[0]), d2(elems[1]))
            QG_DISPATCH_NB(p.numFixed, L)
#undef L
        }
    }
    qg_note_launch();
    return qg_check_launch("diag1");
}

int qg_sv_anyCtrlTwoTargDiagMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                 int targ1, int targ2, const qg_cplx* elems, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (!elems) return qg_fail(QG_ERR_ARG, "null diagonal");
    int tq[2] = {targ1, targ2};
    QG_TRY(qg_check_qubits(numQubits, tq, 2, "targets"));
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, nullptr, nullptr, 0, &p));
    for (int i = 0; i < numCtrls; i++)
        if (ctrls[i] == targ1 || ctrls[i] == targ2) return qg_fail(QG_ERR_ARG, "control %d is also a target", ctrls[i]);
    Diag4 D;
    for (int i = 0; i < 4; i++) D.d[i] = d2(elems[i]);
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    cudaStream_t st = qg_stream(stream);
#define L(NBV) QG_LAUNCH_PLAIN(k_diag2, NBV, (double2*)amps, numIts, p.ins, p.stateMask, targ1, targ2, D)
    QG_DISPATCH_NB(p.numFixed, L)
#undef L
    qg_note_launch();
    return qg_check_launch("diag2");
}

int qg_sv_anyCtrlAnyTargDiagMatr(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                 const int* targs, int numTargs, const qg_cplx* elems, int applyConj,
                                 const qg_cplx* exponent, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (!elems) return qg_fail(QG_ERR_ARG, "null diagonal");
    QG_TRY(qg_check_qubits(numQubits, targs, numTargs, "targets"));
    for (int i = 0; i < numCtrls; i++)
        for (int j = 0; j < numTargs; j++)
            if (ctrls[i] == targs[j]) return qg_fail(QG_ERR_ARG, "control %d is also a target", ctrls[i]);
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, nullptr, nullptr, 0, &p));
    // the 2^k elements are prepared once on the host: the power (std::pow on qcomp, as
    // cpu_subroutines.cpp:663-701 evaluates it per amplitude) then the conjugation
    qidx D = (qidx)1 << numTargs;
    bool hasPower = exponent && !(exponent->re == 1.0 && exponent->im == 0.0);
    std::vector<double2> el((size_t)D);
    for (qidx v = 0; v < D; v++) {
        std::complex<double> e(elems[v].re, elems[v].im);
        if (hasPower) e = std::pow(e, std::complex<double>(exponent->re, exponent->im));
        if (applyConj) e = std::conj(e);
        el[(size_t)v] = make_double2(e.real(), e.imag());
    }
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    cudaStream_t st = qg_stream(stream);
    if (numTargs <= QG_DIAG_PARAM_MAX) {
        DiagK Dk;
        Dk.k = numTargs;
        for (int b = 0; b < numTargs; b++) Dk.t[b] = targs[b];
        for (qidx v = 0; v < D; v++) Dk.d[v] = el[(size_t)v];
#define L(NBV) QG_LAUNCH_PLAIN(k_diagK, NBV, (double2*)amps, numIts, p.ins, p.stateMask, Dk)
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
    } else {
        double2* dev = nullptr;
        QG_CUDA(cudaMallocAsync((void**)&dev, sizeof(double2) * (size_t)D, st));
        QG_CUDA(cudaMemcpyAsync(dev, el.data(), sizeof(double2) * (size_t)D, cudaMemcpyHostToDevice, st));
        DiagKDev Dk;
        Dk.d = dev;
        Dk.k = numTargs;
        for (int b = 0; b < numTargs; b++) Dk.t[b] = targs[b];
#define L(NBV) QG_LAUNCH_PLAIN(k_diagKdev, NBV, (double2*)amps, numIts, p.ins, p.stateMask, Dk)
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
        QG_TRY(qg_check_launch("diagKdev"));
        QG_CUDA(cudaFreeAsync(dev, st));
    }
    qg_note_launch();
    return qg_check_launch("diagK");
}

int qg_sv_anyCtrlPauliTensorOrGadget(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                     const int* targsX, int numX, const int* targsY, int numY, const int* targsZ, int numZ,
                                     qg_cplx ampFac, qg_cplx pairAmpFac, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (numX + numY == 0) return qg_fail(QG_ERR_ARG, "a Pauli tensor or gadget needs an X or Y target");
    std::vector<int> all;
    qidx maskXY = 0, maskYZ = 0;
    int top = -1;
    for (int i = 0; i < numX; i++) { all.push_back(targsX[i]); maskXY |= (qidx)1 << targsX[i]; top = std::max(top, targsX[i]); }
    for (int i = 0; i < numY; i++) { all.push_back(targsY[i]); maskXY |= (qidx)1 << targsY[i]; maskYZ |= (qidx)1 << targsY[i]; top = std::max(top, targsY[i]); }
    for (int i = 0; i < numZ; i++) { all.push_back(targsZ[i]); maskYZ |= (qidx)1 << targsZ[i]; }
    for (int i = 0; i < numCtrls; i++) all.push_back(ctrls[i]);
    QG_TRY(qg_check_qubits(numQubits, all.data(), (int)all.size(), "Pauli targets and controls"));
    int tv = 0;
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, &top, &tv, 1, &p));
    // scale the pair factor by i^numY (util_getPowerOfI, utilities.cpp:333-338)
    static const double pr[4] = {1, 0, -1, 0}, pi[4] = {0, 1, 0, -1};
    int r = numY % 4;
    double2 f1 = make_double2(pairAmpFac.re * pr[r] - pairAmpFac.im * pi[r], pairAmpFac.re * pi[r] + pairAmpFac.im * pr[r]);
    double2 f0 = d2(ampFac);
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    cudaStream_t st = qg_stream(stream);
    int mode = 0;
    bool unit1 = (std::fabs(f1.x) == 1.0 && f1.y == 0.0) || (f1.x == 0.0 && std::fabs(f1.y) == 1.0);
    if (f0.x == 0.0 && f0.y == 0.0 && unit1) mode = 3;
    else if (f0.y == 0.0 && f1.y == 0.0) mode = 1;
    else if (f0.y == 0.0 && f1.x == 0.0) mode = 2;
#define L0(NBV) k_pauli<NBV, 0><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, maskXY, maskYZ, f0, f1)
#define L1(NBV) k_pauli<NBV, 1><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, maskXY, maskYZ, f0, f1)
#define L2(NBV) k_pauli<NBV, 2><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, maskXY, maskYZ, f0, f1)
#define L3(NBV) k_pauli<NBV, 3><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, maskXY, maskYZ, f0, f1)
    switch (mode) {
        case 0: QG_DISPATCH_NB(p.numFixed, L0) break;
        case 1: QG_DISPATCH_NB(p.numFixed, L1) break;
        case 2: QG_DISPATCH_NB(p.numFixed, L2) break;
        default: QG_DISPATCH_NB(p.numFixed, L3) break;
    }
#undef L0
#undef L1
#undef L2
#undef L3
    qg_note_launch();
    return qg_check_launch("pauli");
}

int qg_sv_anyCtrlAnyTargZOrPhaseGadget(void* amps, int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                                       const int* targs, int numTargs, qg_cplx fac0, qg_cplx fac1, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QG_TRY(qg_check_qubits(numQubits, targs, numTargs, "targets"));
    for (int i = 0; i < numCtrls; i++)
        for (int j = 0; j < numTargs; j++)
            if (ctrls[i] == targs[j]) return qg_fail(QG_ERR_ARG, "control %d is also a target", ctrls[i]);
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, ctrls, ctrlStates, numCtrls, nullptr, nullptr, 0, &p));
    qidx tmask = 0;
    for (int j = 0; j < numTargs; j++) tmask |= (qidx)1 << targs[j];
    qidx numIts = ((qidx)1 << numQubits) >> p.numFixed;
    cudaStream_t st = qg_stream(stream);
    bool ztensor = fac0.re == 1.0 && fac0.im == 0.0 && fac1.re == -1.0 && fac1.im == 0.0;
    if (ztensor) {
#define L(NBV) k_zphase<NBV, 1><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, tmask, d2(fac0), d2(fac1))
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
    } else {
#define L(NBV) k_zphase<NBV, 0><<<persistent_blocks(numIts), QG_THREADS, 0, st>>>((double2*)amps, numIts, p.ins, p.stateMask, tmask, d2(fac0), d2(fac1))
        QG_DISPATCH_NB(p.numFixed, L)
#undef L
    }
    qg_note_launch();
    return qg_check_launch("zphase");
}

int qg_sv_multiQubitProjector(void* amps, int numQubits, const int* qubits, const int* outcomes, int num,
                              double prob, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    QG_TRY(qg_check_qubits(numQubits, qubits, num, "projector qubits"));
    qidx qmask = 0, retain = 0;
    for (int i = 0; i < num; i++) {
        if (outcomes[i] != 0 && outcomes[i] != 1) return qg_fail(QG_ERR_ARG, "outcome %d is not 0 or 1", outcomes[i]);
        qmask |= (qidx)1 << qubits[i];
        if (outcomes[i]) retain |= (qidx)1 << qubits[i];
    }
    qidx n = (qidx)1 << numQubits;
    double renorm = 1 / std::sqrt(prob);
    k_projector<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)amps, n, qmask, retain, renorm);
    qg_note_launch();
    return qg_check_launch("projector");
}

}  // extern "C"
