// Many Pauli-string expectation values of one statevector, each amplitude read from
// HBM once per group of strings (the batched form of the per-term loop of
// localiser_statevec_calcExpecPauliStrSum, quest/src/core/localiser.cpp:2052-2148, whose
// terms are cpu_statevec_calcExpecPauliStr_subA, quest/src/cpu/cpu_subroutines.cpp:2059-2085).
//
// A string pairs amplitude n with j = n ^ maskXY.  Split every index into column bits
// (the t lowest, a run of 2^t contiguous amplitudes) and row bits.  The row parts of the
// group's XY masks span a space V of dimension d over GF(2); a tile is one coset of V
// times all 2^t columns, 2^(d+t) amplitudes, and it holds the partner of every member
// for every string of the group.  One CTA loads a tile into shared memory (rows of 2^t
// contiguous amplitudes: coalesced), then evaluates every string on it, each unordered
// pair {n, j} once:
//   term(n) + term(j) = sign(j) x + sign(n) conj(x),   x = conj(a_n) a_j,
//   sign(j) = sign(n) (-1)^numY,
// so a pair adds 2 sign(n) Re x (even numY) or -2i sign(n) Im x (odd numY): two FP64
// FMAs per pair and string, with the sign folded into a_n's sign bit.  Strings without
// X or Y (j = n) add sign(n) |a_n|^2 per amplitude.
//
// The tile coordinates and the grouping of strings into passes are the host plan of
// qg_pauli_plan.h (checked on the CPU by tests/pauli_plan_check.cpp with these index
// expressions).  sign(n) = parity(n & maskYZ) splits into a per-tile bit
// parity(base & maskYZ) and parity(L & W_s) for local index L.
//
// Bytes: a group of strings reads the state once; strings group while their row parts
// span at most PT_DMAX dimensions (and PT_NS strings), so 16 random strings on n qubits
// take ceil(16 / PT_DMAX) passes.  The FP64 work (one FMA per amplitude and string) is
// the bound on GB300, whose FP64 rate is about 2 FMA per clock per SM.
//
// Deterministic: a fixed grid, a fixed assignment of tiles and pairs to threads and the
// fixed reduction tree of qg_reduce.cuh.
#include "qg_reduce.cuh"
#include "qg_pauli_plan.h"

#include <algorithm>
#include <vector>

#define PT_THREADS 256

template <typename AMP>
__device__ __forceinline__ double2 ld_d2(const AMP* p) {
    const AMP v = __ldcs(p);          // streamed: each amplitude is read once per pass
    return make_double2((double)v.x, (double)v.y);
}

__device__ __forceinline__ double flip_sign(double x, unsigned long long s) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)s);
}

template <typename AMP>
__global__ void __launch_bounds__(PT_THREADS, 3) k_expec_pauli_tile(const AMP* __restrict__ a, qidx numTiles,
                                                                    const qgpt::Tile P, RedOut out) {
    extern __shared__ __align__(16) unsigned char pt_smem[];
    double2* tile = (double2*)pt_smem;
    qidx* vtab = (qidx*)(pt_smem + (sizeof(double2) << (P.d + P.t)));   // v(r) of every row
    const int t = P.t, d = P.d;
    const int L = 1 << (d + t);
    const int colMask = (1 << t) - 1;
    for (int r = threadIdx.x; r < (1 << d); r += PT_THREADS) {
        qidx v = 0;
        for (int i = 0; i < d; i++)
            if ((r >> i) & 1) v ^= P.basis[i];
        vtab[r] = v;
    }
    double acc[qgpt::NS];
#pragma unroll
    for (int s = 0; s < qgpt::NS; s++) acc[s] = 0.0;
    for (qidx k = blockIdx.x; k < numTiles; k += gridDim.x) {
        qidx base = k << t;
        for (int i = 0; i < d; i++) {
            qidx lo = base & P.pivLow[i];
            base = ((base ^ lo) << 1) | lo;
        }
        __syncthreads();   // the previous tile is consumed (and vtab written, on the first)
        // consecutive threads take consecutive columns of a row: 2^t contiguous amplitudes
        for (int e = threadIdx.x; e < L; e += PT_THREADS)
            tile[e] = ld_d2(a + ((base ^ vtab[e >> t]) | (qidx)(e & colMask)));
        __syncthreads();
#pragma unroll
        for (int s = 0; s < qgpt::NS; s++) {
            if (s >= P.numStrings) break;
            const unsigned long long pb = (unsigned long long)parity64(base & P.yz[s]);
            const qidx W = P.W[s];
            if (P.top[s] < 0) {
                // no X or Y: sum of sign(n) |a_n|^2
                for (int e = threadIdx.x; e < L; e += PT_THREADS) {
                    const double2 x = tile[e];
                    const unsigned long long sg = (pb ^ (unsigned long long)parity64((qidx)e & W)) << 63;
                    acc[s] = fma(flip_sign(x.x, sg), x.x, fma(flip_sign(x.y, sg), x.y, acc[s]));
                }
            } else {
                const int top = P.top[s];
                const int Ds = (int)P.D[s];
                const int lowMask = (1 << top) - 1;
                const bool odd = P.odd[s] != 0;
                for (int m = threadIdx.x; m < (L >> 1); m += PT_THREADS) {
                    const int e = ((m & ~lowMask) << 1) | (m & lowMask);     // bit `top` of e is zero
                    const double2 an = tile[e], aj = tile[e ^ Ds];
                    const unsigned long long sg = (pb ^ (unsigned long long)parity64((qidx)e & W)) << 63;
                    const double nx = flip_sign(an.x, sg), ny = flip_sign(an.y, sg);
                    if (odd) acc[s] = fma(nx, aj.y, fma(-ny, aj.x, acc[s]));   // sign(n) Im(conj(a_n) a_j)
                    else acc[s] = fma(nx, aj.x, fma(ny, aj.y, acc[s]));        // sign(n) Re(conj(a_n) a_j)
                }
            }
        }
    }
    block_reduce_and_finish<qgpt::NS>(acc, out);
}

// out[s] = <P_s> (the i^numY factor included), one launch per pass of the plan
template <typename AMP>
int qg_pauli_tile_batch(const AMP* amps, int n, const int64_t* mXY, const int64_t* mYZ, const int* numsY, int num,
                        qg_cplx* out, cudaStream_t st) {
    const std::vector<qgpt::Pass> passes = qgpt::make_passes(n, mXY, mYZ, numsY, num);
    double raw[qgpt::NS];
    for (const qgpt::Pass& ps : passes) {
        const qgpt::Tile& P = ps.tile;
        const size_t smem = (sizeof(double2) << (P.d + P.t)) + sizeof(qidx) * ((size_t)1 << P.d);
        QG_CUDA(cudaFuncSetAttribute(k_expec_pauli_tile<AMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        // every resident block busy: while some load their tile, the others keep the FP64 pipe fed
        int perSM = 0;
        QG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_expec_pauli_tile<AMP>, PT_THREADS, smem));
        const int grid = (int)std::max<qidx>(1, std::min<qidx>(ps.numTiles, (qidx)qg_num_sms() * std::max(1, perSM)));
        RedOut r;
        QG_TRY(red_setup(grid, qgpt::NS, &r));
        k_expec_pauli_tile<AMP><<<grid, PT_THREADS, smem, st>>>(amps, ps.numTiles, P, r);
        qg_note_launch();
        QG_TRY(red_fetch(r, qgpt::NS, raw, st));
        for (int k = 0; k < P.numStrings; k++) {
            const int s = ps.members[k];
            qgpt::finish_value(P, k, numsY[s], raw[k], &out[s].re, &out[s].im);
        }
    }
    return QG_OK;
}

template int qg_pauli_tile_batch<double2>(const double2*, int, const int64_t*, const int64_t*, const int*, int, qg_cplx*, cudaStream_t);
template int qg_pauli_tile_batch<float2>(const float2*, int, const int64_t*, const int64_t*, const int*, int, qg_cplx*, cudaStream_t);
