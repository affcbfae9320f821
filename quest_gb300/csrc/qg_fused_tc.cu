// Tensor-core application of a fused 5-qubit block to an FP32 statevector:
// 3xTF32 products on the 5th-generation tensor cores (tcgen05.mma, kind::tf32),
// accumulators in tensor memory.
//
// For a block on targets t0<...<t4, group r (the r-th index with the five target
// bits cleared) holds 32 amplitudes x_r[j] = a[base(r) + off(j)].  With complex
// numbers interleaved (re, im), the block is one real GEMM per tile of 128 groups:
//     Y (128 x 64) = X (128 x 64) * B (64 x 64),
//     B[2j+c][2k+d] = real form of U[k][j]  (re->re: Re U, im->re: -Im U, re->im: Im U, im->im: Re U).
// FP32 accuracy comes from the 3xTF32 split: X = Xh + Xl, B = Bh + Bl with each
// part a TF32 value, and D = Xl*Bh + Xh*Bl + Xh*Bh accumulated in FP32 (the
// Xl*Bl term is below FP32 rounding).  Bh/Bl are built once per block on the host.
//
// Per tile, the producers split the 128 groups' amplitudes into TF32 hi/lo parts and
// store both into shared memory in the no-swizzle K-major core-matrix layout (8 rows x
// 16 bytes per core matrix); one thread issues the 24 MMAs (3 products x 8 K-steps of
// 8) into two 128-lane x 64-column TMEM accumulators (large term, small terms); the
// epilogue reads its TMEM lane (tcgen05.ld 32x32b), adds the two accumulators in FP32
// and writes the group's 32 outputs back.  Every wait is bounded: a wait that runs out
// sets the error flag, waits for the tensor core, frees the TMEM and returns.
#include "qg_common.cuh"
#include "qg_tc_plan.h"
#include "qg_tcgen05.cuh"

#include <chrono>
#include <mutex>
#include <vector>

#include <cmath>
#include <complex>
#include <cstring>

#define TC_M 128              // groups per tile (MMA M)
#define TC_K 64               // real K (32 complex amplitudes)
#define TC_N 64               // real N
#define TC_WAIT_NS 2000000000ull   // a tile's MMAs take microseconds; 2 s means they never completed

// shared-memory operand sizes (bytes)
#define TC_A_BYTES (TC_M * TC_K * 4)      // 32 KiB per part
#define TC_B_BYTES (TC_N * TC_K * 4)      // 16 KiB per part

namespace {

// byte offset of element (row, kk) in the K-major no-swizzle core-matrix layout of a
// (rows x 64) tile: core matrices are 8 rows x 16 bytes; cores are ordered
// [k-core (16)][row-group (rows/8)], so K-adjacent cores are (rows/8)*128 bytes apart
// (the descriptor's leading byte offset) and row-adjacent cores 128 bytes apart
// (its stride byte offset).
__host__ __device__ __forceinline__ unsigned core_offset(int row, int kk, int rows) {
    return (unsigned)(((kk >> 2) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (kk & 3) * 4);
}

}  // namespace

// ---------------------------------------------------------------- host: operands

size_t qg_tc_operand_floats() { return 2 * (size_t)TC_N * TC_K; }

// round-to-nearest (ties away) to TF32: keep 10 explicit mantissa bits
static float tf32_round(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) {
        u += 0x1000u;
        u &= 0xffffe000u;
    }
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// out: Bh then Bl, each 64x64 floats in the tile layout of the B operand (N x K, K-major)
void qg_tc_build_operands(const std::complex<double>* m, float* out) {
    float* bh = out;
    float* bl = out + TC_N * TC_K;
    std::memset(out, 0, sizeof(float) * 2 * TC_N * TC_K);
    for (int k = 0; k < 32; k++)
        for (int j = 0; j < 32; j++) {
            std::complex<double> u = m[k * 32 + j];
            // B_int[2j+c][2k+d]; operand element (n = 2k+d, kk = 2j+c)
            double vals[2][2] = {{u.real(), u.imag()}, {-u.imag(), u.real()}};   // [c][d]
            for (int c = 0; c < 2; c++)
                for (int d = 0; d < 2; d++) {
                    int n = 2 * k + d, kk = 2 * j + c;
                    float f = (float)vals[c][d];
                    float h = tf32_round(f);
                    float l = tf32_round(f - h);
                    unsigned off = core_offset(n, kk, TC_N) / 4;
                    bh[off] = h;
                    bl[off] = l;
                }
        }
}

// ---------------------------------------------------------------- device helpers

// kind::tf32 instruction descriptor: D=F32, A=B=TF32, both K-major, N=64, M=128
__device__ __forceinline__ uint32_t make_idesc() {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

// bounded wait with this kernel's limit
__device__ __forceinline__ bool mbar_wait_tc(uint32_t bar, uint32_t parity) { return mbar_wait_bounded(bar, parity, TC_WAIT_NS); }

// ---------------------------------------------------------------- kernel

struct TcArgs {
    float2* amps;
    qidx numTiles;     // groups / 128
    Ins ins;           // the five sorted targets, as insertion masks
    qidx off[32];      // amplitude offset of matrix index j within a group
    const float* ops;  // Bh, Bl (global)
    int* errorFlag;    // set to 1 if a bounded wait ran out
    // Staged mode, for blocks whose lowest target is below 5 (a warp's 32 groups are
    // then not 32 adjacent amplitudes).  A tile's 4096 amplitudes are numbered in
    // address order by a 12-bit local index L: bit p of L sits at amplitude bit P[p],
    // P = the five targets and the seven lowest other bits, ascending.
    int stage;
    qidx lbit[12];     // 2^P[p]
    int lrow[7];       // L bit holding bit i of the group row
    int lj[5];         // L bit holding bit b of the matrix index j
    qidx kp[16];       // producer element k: amplitude offset of the L bits above the producer index = k
    qidx ke[32];       // epilogue element k: amplitude offset of L bits 7..11 = k
    int sj[32];        // stage_slot of the L bits of matrix index j (the slot map is linear over XOR)
    int holdOperands;  // self-test of the bounded waits: producers never signal "A full"
};

// ---------------------------------------------------------------- kernel
//
// One persistent CTA per SM with three roles that hand tiles to one another through
// mbarriers, so that loads, tensor-core work and stores of different tiles overlap:
// * producers: TPR threads per group row load the row's 32 amplitudes, split them into
//   TF32 hi/lo parts and write them into one of two A operand buffers.  Each holds
//   NBUF tiles of loads in registers: NBUF - 1 tiles are in flight while one is split;
// * one MMA warp (one elected thread): the 24 MMAs of a tile into one of two TMEM
//   accumulator sets, committed to that buffer's "MMA done" barrier;
// * 4 epilogue warps: one thread per group row (TMEM lane) reads the two accumulators,
//   adds them and stores the row's 32 outputs.
// Barriers per buffer s: aFull[s] (one arrival per producer), mmaDone[s] (the commit;
// it also frees A[s]), tmemEmpty[s] (128 epilogue arrivals).  Tile i of a CTA uses
// buffer i & 1 for the (i >> 1)-th time, which gives every wait's phase parity.
#define WS_EPILOGUE 128
// launch shapes: producer threads per group row and register buffers per producer
// (tiles of loads in flight + 1), for the direct and the staged mode
#define TC_TPR 2
#define TC_NBUF 3
#define TC_TPR_STAGED 4
#define TC_NBUF_STAGED 2
#define WS_TMEM_COLS 256
#define WS_STAGE_BYTES (TC_M * 32 * 8)     // one tile of amplitudes (32 KiB)
// shared memory: A[2] (hi, lo), Bh, Bl, the staging buffers the mode uses, barriers.
// Shared memory and L1 share one array per SM, and L1 holds the loads in flight, so a
// launch asks only for what its mode uses.
#define WS_SMEM_BYTES(nstage) (4 * TC_A_BYTES + 2 * TC_B_BYTES + (nstage) * WS_STAGE_BYTES + 128 + 1024)

// staging-buffer slot of local index e: the low five bits are XORed with the next
// five, so that both address-order and group-row-order accesses of a warp spread
// over the banks
__device__ __forceinline__ int stage_slot(int e) { return e ^ ((e >> 5) & 31); }

// TPR producer threads per group row, each holding 32 / TPR amplitudes of it; NBUF
// register buffers per producer, so NBUF - 1 tiles of loads are in flight while one
// tile is split (the loop is unrolled NBUF times so buffers are never copied).
template <int TPR, int NBUF>
struct WsShape {
    static constexpr int PRODUCERS = 128 * TPR;
    static constexpr int PBITS = TPR == 1 ? 7 : TPR == 2 ? 8 : 9;   // log2(PRODUCERS)
    static constexpr int AMPS = 32 / TPR;
    static constexpr int MMA_WARP = PRODUCERS / 32;
    static constexpr int THREADS = PRODUCERS + 32 + WS_EPILOGUE;
};

// STAGED: the producers load in address order through a staging buffer; STAGED_OUT:
// the epilogue stores in address order through a second one.
template <int TPR, int NBUF, bool STAGED, bool STAGED_OUT>
__global__ void __launch_bounds__(WsShape<TPR, NBUF>::THREADS, 1) k32_fused_tc(TcArgs args) {
    using S = WsShape<TPR, NBUF>;
    constexpr int AMPS = S::AMPS;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // A[s] = hi part then lo part (TC_A_BYTES each), s = 0, 1; Bh, Bl; the producers'
    // and the epilogue's staging buffers; barriers
    float* sB = (float*)(smem + 4 * TC_A_BYTES);
    float2* sStageP = (float2*)(smem + 4 * TC_A_BYTES + 2 * TC_B_BYTES);
    float2* sStageE = (float2*)(smem + 4 * TC_A_BYTES + 2 * TC_B_BYTES + (STAGED ? WS_STAGE_BYTES : 0));
    uint64_t* bars = (uint64_t*)(smem + 4 * TC_A_BYTES + 2 * TC_B_BYTES + ((int)STAGED + (int)STAGED_OUT) * WS_STAGE_BYTES);   // aFull[2], mmaDone[2], tmemEmpty[2]
    uint32_t* tmemSlot = (uint32_t*)(bars + 6);
    volatile int* abortFlag = (volatile int*)(tmemSlot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    {
        const float4* src = (const float4*)args.ops;
        float4* dst = (float4*)sB;
        for (int i = tid; i < (2 * TC_B_BYTES) / 16; i += S::THREADS) dst[i] = __ldg(src + i);
    }
    if (tid == 0) {
        for (int s = 0; s < 2; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bars + s)), "r"(S::PRODUCERS));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bars + 2 + s)), "r"(1));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bars + 4 + s)), "r"(WS_EPILOGUE));
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
        *abortFlag = 0;
    }
    if (warp == S::MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_addr(tmemSlot)), "r"(WS_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmemSlot;
    const qidx first = blockIdx.x, step = gridDim.x;
    const qidx nLocal = args.numTiles > first ? (args.numTiles - first + step - 1) / step : 0;
    const uint32_t aFull = smem_addr(bars), mmaDone = smem_addr(bars + 2), tmemEmpty = smem_addr(bars + 4);

    if (warp < S::MMA_WARP) {
        // ---------------- producers.  Direct mode: thread (row, part) loads amplitudes
        // [AMPS*part, AMPS*part + AMPS) of its row.  Staged mode: it loads the tile's
        // elements L = tid + PRODUCERS * k (address order) into the staging buffer, then
        // reads its row's amplitudes back from there.
        const int row = tid & (TC_M - 1), part = tid >> 7;
        qidx tOff = 0;
        int sRow = 0, sTid = 0;
        if constexpr (STAGED) {
            int eRow = 0;
#pragma unroll
            for (int p = 0; p < S::PBITS; p++) tOff += ((tid >> p) & 1) ? args.lbit[p] : 0;
#pragma unroll
            for (int i = 0; i < 7; i++) eRow |= ((row >> i) & 1) << args.lrow[i];
            sRow = stage_slot(eRow);
            sTid = stage_slot(tid);
        } else {
            tOff = insert_bits<5>(row, args.ins);
        }
        const float2* src = args.amps + tOff;
        const qidx* off = STAGED ? args.kp : args.off + AMPS * part;
        float2 x[NBUF][AMPS];
        auto load = [&](float2 (&dst)[AMPS], qidx i) {
            const float2* p = src + insert_bits<5>((first + i * step) * TC_M, args.ins);
#pragma unroll
            for (int k = 0; k < AMPS; k++) dst[k] = __ldcs(p + off[k]);
        };
#pragma unroll
        for (int b = 0; b < NBUF - 1; b++)
            if (b < nLocal) load(x[b], b);
        bool stop = false;
        for (qidx i0 = 0; i0 < nLocal && !stop; i0 += NBUF) {
#pragma unroll
            for (int b = 0; b < NBUF; b++) {
                const qidx i = i0 + b;
                if (i >= nLocal) break;
                if (i + NBUF - 1 < nLocal) load(x[(b + NBUF - 1) % NBUF], i + NBUF - 1);
                const int s = (int)(i & 1);
                const uint32_t u = (uint32_t)(i >> 1);
                bool bad = u >= 1 && !mbar_wait_tc(mmaDone + 8 * s, (u - 1) & 1);
                if (bad) *abortFlag = 1;
                if constexpr (STAGED) {
                    // all producers have finished reading the previous tile's staging
                    if (named_sync_or(1, S::PRODUCERS, bad || *abortFlag)) { stop = true; break; }
                    // slot(tid + PRODUCERS k) = slot(tid) ^ slot(PRODUCERS k), the second a constant
#pragma unroll
                    for (int k = 0; k < AMPS; k++) sStageP[sTid ^ stage_slot(S::PRODUCERS * k)] = x[b][k];
                    named_sync(1, S::PRODUCERS);
                } else if (*abortFlag) {
                    stop = true;
                    break;
                }
                unsigned char* sAh = smem + (2 * s) * TC_A_BYTES;
                unsigned char* sAl = sAh + TC_A_BYTES;
#pragma unroll
                for (int q = 0; q < AMPS / 2; q++) {
                    float2 p0, p1;
                    if constexpr (STAGED) {
                        const int* sj = args.sj + AMPS * part + 2 * q;
                        p0 = sStageP[sRow ^ sj[0]];
                        p1 = sStageP[sRow ^ sj[1]];
                    } else {
                        p0 = x[b][2 * q];
                        p1 = x[b][2 * q + 1];
                    }
                    float4 h, l;
                    h.x = tf32_hi(p0.x); l.x = tf32_hi(p0.x - h.x);
                    h.y = tf32_hi(p0.y); l.y = tf32_hi(p0.y - h.y);
                    h.z = tf32_hi(p1.x); l.z = tf32_hi(p1.x - h.z);
                    h.w = tf32_hi(p1.y); l.w = tf32_hi(p1.y - h.w);
                    const unsigned o = core_offset(row, 4 * ((AMPS / 2) * part + q), TC_M);
                    *(float4*)(sAh + o) = h;
                    *(float4*)(sAl + o) = l;
                }
                asm volatile("fence.proxy.async.shared::cta;");
                if (!args.holdOperands) mbar_arrive(aFull + 8 * s);
            }
        }
    } else if (warp == S::MMA_WARP) {
        // ---------------- MMA issue (one thread)
        if (lane == 0) {
            const uint32_t idesc = make_idesc();
            const uint32_t lboA = (TC_M / 8) * 128, lboB = (TC_N / 8) * 128, sbo = 128;
            const uint32_t bH = smem_addr(sB), bL = bH + TC_B_BYTES;
            qidx issued = 0;
            for (qidx i = 0; i < nLocal; i++) {
                const int s = (int)(i & 1);
                const uint32_t u = (uint32_t)(i >> 1);
                if (!mbar_wait_tc(aFull + 8 * s, u & 1)) *abortFlag = 1;
                if (!*abortFlag && u >= 1 && !mbar_wait_tc(tmemEmpty + 8 * s, (u - 1) & 1)) *abortFlag = 1;
                if (*abortFlag) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t aH = smem_addr(smem + (2 * s) * TC_A_BYTES), aL = aH + TC_A_BYTES;
                const uint32_t dBase = tmem + (uint32_t)s * 128;
                for (int prod = 0; prod < 3; prod++) {
                    const uint32_t a = (prod == 0) ? aL : aH;
                    const uint32_t b = (prod == 1) ? bL : bH;
                    const uint32_t d = (prod == 2) ? dBase : dBase + TC_N;
                    uint32_t acc = (prod == 1) ? 1u : 0u;
#pragma unroll
                    for (int k = 0; k < TC_K / 8; k++) {
                        mma_tf32(d, make_desc(a + k * 2 * lboA, lboA, sbo), make_desc(b + k * 2 * lboB, lboB, sbo), idesc, acc);
                        acc = 1;
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mmaDone + 8 * s) : "memory");
                issued = i + 1;
            }
            // no MMA may still be running when the accumulators are freed
            if (issued > 0) {
                const qidx l = issued - 1;
                if (!mbar_wait_tc(mmaDone + 8 * (int)(l & 1), (uint32_t)(l >> 1) & 1)) *abortFlag = 1;
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: TMEM lane quarter = warp % 4, one group row per
        // thread.  Direct mode stores the row's 32 outputs; staged mode writes them into
        // the staging buffer and stores the tile's elements L = row + 128 k in address order.
        const int quarter = warp & 3;
        const int row = 32 * quarter + lane;
        qidx eOff = 0;
        int sRow = 0;
        if constexpr (STAGED_OUT) {
            int eRow = 0;
#pragma unroll
            for (int p = 0; p < 7; p++) eOff += ((row >> p) & 1) ? args.lbit[p] : 0;
#pragma unroll
            for (int i = 0; i < 7; i++) eRow |= ((row >> i) & 1) << args.lrow[i];
            sRow = stage_slot(eRow);
        } else {
            eOff = insert_bits<5>(row, args.ins);
        }
        float2* dstRow = args.amps + eOff;
        const int sOut = stage_slot(row);
        for (qidx i = 0; i < nLocal; i++) {
            const int s = (int)(i & 1);
            const uint32_t u = (uint32_t)(i >> 1);
            const bool waited = mbar_wait_tc(mmaDone + 8 * s, u & 1);
            if constexpr (STAGED_OUT) {
                // the whole epilogue leaves together (named barriers below); this barrier
                // also orders the previous tile's staging reads before this tile's writes
                const bool bad = named_sync_or(2, WS_EPILOGUE, !waited || *abortFlag);
                if (!waited) *abortFlag = 1;
                if (bad) break;
            } else {
                // the warp leaves together: it runs warp-collective TMEM loads
                const bool ok = __all_sync(0xffffffffu, waited);
                if (!ok && lane == 0) *abortFlag = 1;
                if (!ok || __shfl_sync(0xffffffffu, lane == 0 ? *abortFlag : 0, 0)) break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            float2* dst = dstRow + insert_bits<5>((first + i * step) * TC_M, args.ins);
            const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)s * 128;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                uint32_t big[16], small[16];
                TMEM_LD16(taddr + 16 * c, big);
                TMEM_LD16(taddr + TC_N + 16 * c, small);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (c == 3) {
                    asm volatile("tcgen05.fence::before_thread_sync;");
                    mbar_arrive(tmemEmpty + 8 * s);
                }
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const float re = __uint_as_float(small[2 * k]) + __uint_as_float(big[2 * k]);
                    const float im = __uint_as_float(small[2 * k + 1]) + __uint_as_float(big[2 * k + 1]);
                    if constexpr (STAGED_OUT)
                        sStageE[sRow ^ args.sj[8 * c + k]] = make_float2(re, im);
                    else
                        __stcs(dst + args.off[8 * c + k], make_float2(re, im));
                }
            }
            if constexpr (STAGED_OUT) {
                named_sync(2, WS_EPILOGUE);
                // slot(row + 128 k) = slot(row) ^ slot(128 k)
#pragma unroll 8
                for (int k = 0; k < 32; k++) __stcs(dst + args.ke[k], sStageE[sOut ^ stage_slot(WS_EPILOGUE * k)]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0 && *abortFlag) {
        *(volatile int*)args.errorFlag = 1;     // a plain store: the word may be mapped host memory
        __threadfence_system();
    }
    if (warp == S::MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(WS_TMEM_COLS));
}

// ---------------------------------------------------------------- host: launch

namespace {
// Per device: the error flag that launches without a flag of their own report to, and
// whether the kernel's shared-memory limit has been raised there.  The flag lives in
// mapped pinned host memory, so the host reads it without a copy or a synchronisation.
struct TcDevice {
    int* hostFlag = nullptr;   // host view
    int* devFlag = nullptr;    // the same word as the device sees it
    bool attr = false;
};
const int TC_MAX_DEVICES = 64;
TcDevice g_tcdev[TC_MAX_DEVICES];
std::mutex g_tcmu;

int tc_current(TcDevice** out) {
    int dev = 0;
    QG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= TC_MAX_DEVICES) return qg_fail(QG_ERR_NOTSUP, "device %d is beyond this build's device table", dev);
    *out = &g_tcdev[dev];
    return QG_OK;
}
}  // namespace

bool qg_tc_supported(int numQubits) { return numQubits >= 12; }

// one-time set-up per device (the error flag, the kernel's shared-memory limit); done
// before the first launch on that device and before any stream capture of one
int qg_tc_prepare() {
    std::lock_guard<std::mutex> lock(g_tcmu);
    TcDevice* d = nullptr;
    QG_TRY(tc_current(&d));
    if (!d->hostFlag) {
        int* h = nullptr;
        QG_CUDA(cudaHostAlloc((void**)&h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable));
        *(volatile int*)h = 0;
        int* dp = nullptr;
        cudaError_t e = cudaHostGetDevicePointer((void**)&dp, h, 0);
        if (e != cudaSuccess) {
            cudaFreeHost(h);
            return qg_check_cuda(e, "cudaHostGetDevicePointer(tensor-core error flag)");
        }
        d->hostFlag = h;
        d->devFlag = dp;
    }
    if (!d->attr) {
        QG_CUDA(cudaFuncSetAttribute(k32_fused_tc<TC_TPR, TC_NBUF, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, WS_SMEM_BYTES(0)));
        QG_CUDA(cudaFuncSetAttribute(k32_fused_tc<TC_TPR_STAGED, TC_NBUF_STAGED, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, WS_SMEM_BYTES(1)));
        QG_CUDA(cudaFuncSetAttribute(k32_fused_tc<TC_TPR_STAGED, TC_NBUF_STAGED, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, WS_SMEM_BYTES(2)));
        d->attr = true;
    }
    return QG_OK;
}

// the current device's error flag as the device sees it (prepared on first use)
int qg_tc_device_flag(int** out) {
    TcDevice* d = nullptr;
    QG_TRY(tc_current(&d));
    if (!d->hostFlag) QG_TRY(qg_tc_prepare());
    *out = d->devFlag;
    return QG_OK;
}

// Reports, and clears, a timeout that an earlier launch on the current device left in the
// device's flag: QG_ERR_TIMEOUT if there was one.  A host read of mapped memory: no copy,
// no synchronisation, so launches still in flight are not waited for.
int qg_tc_take_error() {
    TcDevice* d = nullptr;
    QG_TRY(tc_current(&d));
    if (!d->hostFlag || *(volatile int*)d->hostFlag == 0) return QG_OK;
    *(volatile int*)d->hostFlag = 0;
    return qg_fail(QG_ERR_TIMEOUT, "an earlier tensor-core block launch on this device gave up a bounded wait "
                                   "(its register was left partly updated); the flag is now cleared");
}

// errorFlag: the device word a timeout is reported to (nullptr: the device's own flag)
int qg_tc_apply_block(float2* amps, int numQubits, const int* targs, const float* devOperands, cudaStream_t st,
                      bool holdOperands = false, int* errorFlag = nullptr) {
    if (numQubits < 12) return qg_fail(QG_ERR_ARG, "the tensor-core block kernel needs at least 12 qubits (one 128-group tile)");
    TcDevice* dev = nullptr;
    QG_TRY(tc_current(&dev));
    if (!dev->attr) QG_TRY(qg_tc_prepare());
    int zeros[5] = {0, 0, 0, 0, 0};
    QubitPlan p;
    QG_TRY(qg_make_plan(numQubits, nullptr, nullptr, 0, targs, zeros, 5, &p));
    TcArgs a;
    a.amps = amps;
    a.numTiles = (((qidx)1 << numQubits) >> 5) / TC_M;
    a.ins = p.ins;
    for (int j = 0; j < 32; j++) {
        qidx o = 0;
        for (int b = 0; b < 5; b++) if ((j >> b) & 1) o |= (qidx)1 << targs[b];
        a.off[j] = o;
    }
    a.ops = devOperands;
    a.errorFlag = errorFlag ? errorFlag : dev->devFlag;
    a.holdOperands = holdOperands ? 1 : 0;
    // the mode and the staged modes' index tables (qg_tc_plan.h)
    qgtc::Plan plan;
    if (!qgtc::make_plan(numQubits, targs, WsShape<TC_TPR_STAGED, TC_NBUF_STAGED>::PBITS, &plan))
        return qg_fail(QG_ERR_ARG, "bad targets for a tensor-core block");
    a.stage = plan.stage;
    for (int i = 0; i < 12; i++) a.lbit[i] = plan.lbit[i];
    for (int i = 0; i < 7; i++) a.lrow[i] = plan.lrow[i];
    for (int i = 0; i < 5; i++) a.lj[i] = plan.lj[i];
    for (int i = 0; i < 16; i++) a.kp[i] = plan.kp[i];
    for (int i = 0; i < 32; i++) {
        a.ke[i] = plan.ke[i];
        a.sj[i] = plan.sj[i];
    }
    const unsigned grid = (unsigned)std::min<qidx>(a.numTiles, (qidx)qg_num_sms());
    using SS = WsShape<TC_TPR_STAGED, TC_NBUF_STAGED>;
    if (a.stage == 2)
        k32_fused_tc<TC_TPR_STAGED, TC_NBUF_STAGED, true, true><<<grid, SS::THREADS, WS_SMEM_BYTES(2), st>>>(a);
    else if (a.stage == 1)
        k32_fused_tc<TC_TPR_STAGED, TC_NBUF_STAGED, true, false><<<grid, SS::THREADS, WS_SMEM_BYTES(1), st>>>(a);
    else
        k32_fused_tc<TC_TPR, TC_NBUF, false, false><<<grid, WsShape<TC_TPR, TC_NBUF>::THREADS, WS_SMEM_BYTES(0), st>>>(a);
    qg_note_launch();
    return qg_check_launch("k32_fused_tc");
}

extern "C" int qg_tc_get_error_flag(int* out) {
    if (!out) return qg_fail(QG_ERR_ARG, "null argument");
    TcDevice* d = nullptr;
    QG_TRY(tc_current(&d));
    *out = d->hostFlag ? *(volatile int*)d->hostFlag : 0;
    return QG_OK;
}

extern "C" int qg_tc_clear_error_flag(void) {
    TcDevice* d = nullptr;
    QG_TRY(tc_current(&d));
    if (d->hostFlag) *(volatile int*)d->hostFlag = 0;
    return QG_OK;
}

// Self-test of the kernel's failure path.  One launch on a scratch FP32 register of
// numQubits (12..20) with the given five targets, in which the producers never signal
// that an operand buffer is full.  The MMA warp's and the epilogue's bounded waits then
// run out: no MMA is issued, nothing is stored, the TMEM is freed, and the kernel
// returns with the error flag set.  Reports that flag (1 expected), the launch's
// wall time and whether the register came back unchanged, then clears the flag.
extern "C" int qg_tc_selftest_timeout(int numQubits, const int* targs, int* flagOut, double* secondsOut,
                                      int* unchangedOut) {
    if (numQubits < 12 || numQubits > 20 || !targs || !flagOut) return qg_fail(QG_ERR_ARG, "self-test on 12..20 qubits");
    QG_TRY(qg_tc_prepare());
    const size_t n = (size_t)1 << numQubits;
    std::vector<float2> host(n);
    for (size_t i = 0; i < n; i++) host[i] = make_float2((float)(i % 7) * 0.125f, -(float)(i % 5) * 0.25f);
    void* amps = nullptr;
    void* ops = nullptr;
    QG_TRY(qg_alloc(&amps, (int64_t)(n * sizeof(float2))));
    int rc = qg_alloc(&ops, (int64_t)(qg_tc_operand_floats() * sizeof(float)));
    if (rc == QG_OK && cudaMemcpy(amps, host.data(), n * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = qg_fail(QG_ERR_CUDA, "copy failed");
    if (rc == QG_OK && cudaMemset(ops, 0, qg_tc_operand_floats() * sizeof(float)) != cudaSuccess)
        rc = qg_fail(QG_ERR_CUDA, "memset failed");
    const auto t0 = std::chrono::steady_clock::now();
    if (rc == QG_OK) rc = qg_tc_apply_block((float2*)amps, numQubits, targs, (const float*)ops, nullptr, true);
    if (rc == QG_OK && cudaDeviceSynchronize() != cudaSuccess) rc = qg_fail(QG_ERR_CUDA, "self-test launch failed");
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc == QG_OK) rc = qg_tc_get_error_flag(flagOut);
    if (rc == QG_OK && unchangedOut) {
        std::vector<float2> back(n);
        if (cudaMemcpy(back.data(), amps, n * sizeof(float2), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = qg_fail(QG_ERR_CUDA, "copy failed");
        *unchangedOut = rc == QG_OK && std::memcmp(back.data(), host.data(), n * sizeof(float2)) == 0;
    }
    if (rc == QG_OK) qg_tc_clear_error_flag();
    if (secondsOut) *secondsOut = secs;
    qg_free(ops);
    qg_free(amps);
    return rc;
}
