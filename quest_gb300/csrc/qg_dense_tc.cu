// Three- and four-target dense gates on an FP64 statevector through the fp16 tensor cores,
// as exact 8-bit slices (the arithmetic is qg_slices.h's).  The same operation as
// gpu_statevec_anyCtrlAnyTargDenseMatr_sub (quest/src/gpu/gpu_subroutines.cpp), whose
// kernel forms each output with FP64 multiply-adds (quest/src/gpu/gpu_kernels.cuh).
//
// A tile is 128 amplitude groups (KR = 16 or 32 reals each).  Per tile:
//   A_i (128 x KR, fp16) = digit i of the groups' inputs, i = 0..6,
//   B   (8 KR x KR, fp16) = the operator's digits r_j[n][k] stacked by j (row j KR + n),
//   D   (128 x 8 KR, FP32 in TMEM): column s KR + n accumulates acc_s[n] = sum over
//       i + j = s of A_i . r_j[n].
// Slice i contributes to the sums s = i..7 only, so its MMA writes D columns i KR .. 8 KR
// with the first (8 - i) KR rows of B: seven MMAs of N = (8 - i) KR per K step of 16, and
// no partial product that the result drops is ever formed.
//
// One persistent CTA per SM, warp-specialised like the FP32 block kernel (qg_fused_tc.cu):
// * producers (8 warps, two threads per group): load the group's amplitudes, find the
//   group's scale (the partner's half by a shuffle), cut the inputs into digits and store
//   them into one of two A buffers (bulk prefetches of later tiles into L2 were measured
//   and made it slower); a group that needs FP64 (Inf/NaN, extreme scales) is
//   evaluated by its two producer threads directly;
// * one MMA warp: one thread issues the tile's MMAs into one of two accumulator sets;
// * epilogue (8 warps: TMEM lane quarter x half of the outputs): reads its eight digit
//   sums per output, combines them in int64 and stores the outputs.
// Barriers per buffer s: aFull (the producers' arrivals), infoReady (the MMA thread,
// after it has seen aFull: the group scales are then visible to the epilogue), mmaDone
// (the MMAs' commit; also frees A[s]), tmemEmpty (the epilogue's arrivals).  Every wait
// is bounded: one that runs out sets the error flag, the CTA stops, waits for its MMAs,
// frees the TMEM and returns; the register is then partly updated.
#include "qg_common.cuh"
#include "qg_slices.h"
#include "qg_tcgen05.cuh"

#include <cuda_fp16.h>

#include <atomic>
#include <climits>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#define DT_WAIT_NS 2000000000ull   // a tile takes microseconds; 2 s means it never completes
#define DT_SKIP INT_MIN            // epilogue: nothing to store for this group (else the scale << 20)

// KR reals per group; STG: the producers' inputs pass through a shared-memory stage
// filled by cp.async (else they load into registers, the next tile's loads issued per
// k-core as its digits are formed)
template <int KR, bool STG>
struct DtShape {
    static constexpr int D = KR / 2;                      // amplitudes per group
    static constexpr int AMPS = D / 2;                    // amplitudes per producer thread
    static constexpr int NV = KR / 2;                     // reals per producer thread
    static constexpr int PRODUCERS = 256;
    static constexpr int MMA_WARP = PRODUCERS / 32;
    static constexpr int EPI = 256;
    static constexpr int THREADS = PRODUCERS + 32 + EPI;
    static constexpr int SLICE = 128 * KR * 2;            // bytes of one digit slice of a tile
    static constexpr int A_BYTES = qgsl::XD * SLICE;
    static constexpr int B_ROWS = qgsl::RD * KR;
    static constexpr int B_BYTES = B_ROWS * KR * 2;
    static constexpr int DCOLS = qgsl::NSUM * KR;         // accumulator columns per tile
    static constexpr int TMEM_COLS = 2 * DCOLS;           // 512 (KR = 32) or 256
    static constexpr int INFO_BYTES = 4 * 128 * 4 + 8 * (KR / 2);   // + the offsets off[j]
    // the producers' input staging: NSTAGE tiles of their amplitudes (NSTAGE - 1 in flight
    // while one is cut into digits), filled by cp.async, so the bytes in flight per SM do
    // not depend on registers
    static constexpr int TILE_IN = 128 * D * 16;          // input bytes of one tile
    static constexpr int NSTAGE = (96 * 1024) / TILE_IN;  // 3 (four targets) or 6 (three)
    static constexpr int STAGE_BYTES = STG ? NSTAGE * TILE_IN : 0;
    static constexpr int CHUNK = STG ? 8 : 4;             // output reals per TMEM-load round of the epilogue
    // 128 bytes of barriers, TMEM address and abort flag; 128 of alignment slack
    static constexpr int SMEM_USED = 2 * A_BYTES + B_BYTES + STAGE_BYTES + INFO_BYTES + 128 + 128;
    // one CTA per SM: at least 120 KiB asked for, so that a second never fits beside it
    static constexpr int SMEM = SMEM_USED > 120 * 1024 ? SMEM_USED : 120 * 1024;
    static_assert(SMEM_USED <= 232448, "shared memory per block");
};

template <int KR>
struct DtArgs {
    double2* amps;
    qidx numIts;                  // groups
    qidx numTiles;                // ceil(groups / 128)
    Ins ins;                      // controls and targets, sorted, as insertion masks
    qidx mask;                    // control bits set to 1
    qidx off[KR / 2];             // amplitude offset of matrix index j within a group
    int elo, ehi;                 // a group is normal when elo <= Eg <= ehi
    int eR;                       // the operator's scale
    int* errorFlag;
    double2 m[(KR / 2) * (KR / 2)];                 // the matrix, for groups evaluated in FP64
    uint4 bops[DtShape<KR, false>::B_BYTES / 16];  // the operator's digits in the B tile layout
};

// byte offset of element (row, k) in the K-major no-swizzle layout of a tile of `rows`
// rows of 16-bit values: core matrices of 8 rows x 16 bytes, ordered [k-core][row group], so
// K-adjacent cores are rows/8 x 128 bytes apart (the descriptor's leading byte offset)
// and row-adjacent ones 128 bytes (its stride byte offset)
__host__ __device__ __forceinline__ unsigned dt_core_offset(int row, int k, int rows) {
    return (unsigned)(((k >> 3) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// kind::f16 instruction descriptor: D = F32, A = B = F16, both K-major, M = 128
__device__ __forceinline__ uint32_t dt_idesc(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

// |V| + CX of a real with high and low words (hi, lo) at group scale Eg (qg_slices.h
// input_word; Eg >= 2047 + 64 gives CX, all digits zero)
__device__ __forceinline__ uint64_t dt_word(uint32_t hi, uint32_t lo, int Eg) {
    const int d = Eg - (int)((hi >> 20) & 0x7FFu);
    const uint64_t m2 = ((uint64_t)((hi & 0xFFFFFu) | 0x100000u) << 33) | ((uint64_t)lo << 1);
    return (d < 64 ? m2 >> d : 0ull) + qgsl::CX;
}

// fp16x2 (sign0 (byte b0 of g - 128), sign1 (byte b1 of g - 128)): 0x64XX is 1024 + XX in
// fp16, exactly, and sgn (1024 + XX) - sgn 1152 = sgn (XX - 128) in one exact FMA
__device__ __forceinline__ uint32_t dt_pair(uint32_t g, uint32_t sel, __half2 sgn, __half2 nc) {
    const uint32_t h = __byte_perm(g, 0x64646464u, sel);
    const __half2 v = __hfma2(*reinterpret_cast<const __half2*>(&h), sgn, nc);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// the 7 digit words (fp16x2: digit i of real k, digit i of real k + 1) of two reals with
// high words hi0, hi1 (their signs) and magnitude words w0, w1
__device__ __forceinline__ void dt_digits2(uint32_t hi0, uint32_t hi1, uint64_t w0, uint64_t w1, uint32_t (&out)[qgsl::XD]) {
    const uint32_t sb = 0x3C003C00u | ((hi0 >> 16) & 0x8000u) | (hi1 & 0x80000000u);   // (+-1, +-1)
    const uint32_t nb = 0xE480E480u ^ (sb & 0x80008000u);                              // (-+1152, -+1152)
    const __half2 sgn = *reinterpret_cast<const __half2*>(&sb), nc = *reinterpret_cast<const __half2*>(&nb);
    const uint32_t lo0 = (uint32_t)w0, lo1 = (uint32_t)w1, h0 = (uint32_t)(w0 >> 32), h1 = (uint32_t)(w1 >> 32);
    const uint32_t gl01 = __byte_perm(lo0, lo1, 0x5140u);   // W bytes 0, 1 of both: digits 6, 5
    const uint32_t gl23 = __byte_perm(lo0, lo1, 0x7362u);   // W bytes 2, 3: digits 4, 3
    const uint32_t gh01 = __byte_perm(h0, h1, 0x5140u);     // W bytes 4, 5: digits 2, 1
    const uint32_t gh2 = __byte_perm(h0, h1, 0x6262u);      // W byte 6: digit 0
    out[0] = dt_pair(gh2, 0x4140u, sgn, nc);
    out[1] = dt_pair(gh01, 0x4342u, sgn, nc);
    out[2] = dt_pair(gh01, 0x4140u, sgn, nc);
    out[3] = dt_pair(gl23, 0x4342u, sgn, nc);
    out[4] = dt_pair(gl23, 0x4140u, sgn, nc);
    out[5] = dt_pair(gl01, 0x4342u, sgn, nc);
    out[6] = dt_pair(gl01, 0x4140u, sgn, nc);
}

// the output from this lane's eight digit sums (column q of each).  Each sum s is an
// integer below 2^22, so 1.5 * 2^23 + acc_s has unit spacing and its bits are
// 0x4B400000 + acc_s.  The four pair sums t_2m * 256 + t_2m+1 are then acc-pair sums plus
// c = 257 * 0x4B400000 mod 2^32 = 0x8B400000, without wrapping as unsigned values (the
// pair sums stay below 2^30 + 2^22 in magnitude), and c is a multiple of 2^11, so
// Y' = h1 2^37 + h2 2^21 + l1 2^5 + floor(l2 / 2^11) is formed from them modulo 2^64
// with one constant, DT_K, taken off (qg_slices.h combine states the same value).
#define DT_K 0x6811681168116800ull
template <int W>
__device__ __forceinline__ double dt_output(const uint32_t (&r)[qgsl::NSUM][W], int q, int shift20) {
    uint32_t t[qgsl::NSUM];
#pragma unroll
    for (int s = 0; s < qgsl::NSUM; s++) t[s] = __float_as_uint(__uint_as_float(r[s][q]) + 12582912.0f);
    const uint32_t h1 = t[0] * 256u + t[1], h2 = t[2] * 256u + t[3], l1 = t[4] * 256u + t[5], l2 = t[6] * 256u + t[7];
    const uint64_t y = (uint64_t)(l2 >> 11) + (uint64_t)l1 * 32u + (uint64_t)h2 * (1ull << 21) + ((uint64_t)h1 << 37) - DT_K;
    const double d = (double)(int64_t)y;
    const int hi = __double2hiint(d);
    return hi == 0 ? 0.0 : __hiloint2double(hi + shift20, __double2loint(d));
}

template <int KR, bool STG>
__global__ void __launch_bounds__(DtShape<KR, STG>::THREADS, 1) k_dense_tc(const __grid_constant__ DtArgs<KR> args) {
    using S = DtShape<KR, STG>;
    constexpr int D = S::D, AMPS = S::AMPS;
    extern __shared__ __align__(128) unsigned char dt_smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)dt_smem_raw + 127) & ~(uintptr_t)127);
    unsigned char* sA = smem;                                   // A[2], XD slices each
    unsigned char* sB = smem + 2 * S::A_BYTES;
    double2* sStage = (double2*)(sB + S::B_BYTES);              // [stage][amplitude a][producer]
    int* sInfo = (int*)(sB + S::B_BYTES + S::STAGE_BYTES);      // [tile & 3][row]: output scale or DT_SKIP
    qidx* sOff = (qidx*)(sInfo + 4 * 128);                      // off[j] (a per-lane index into the parameters would be a serial constant load)
    uint64_t* bars = (uint64_t*)(sB + S::B_BYTES + S::STAGE_BYTES + S::INFO_BYTES);   // aFull[2], infoReady[2], mmaDone[2], tmemEmpty[2]
    uint32_t* tmemSlot = (uint32_t*)(bars + 8);
    volatile int* abortFlag = (volatile int*)(tmemSlot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < S::B_BYTES / 16; i += S::THREADS) ((uint4*)sB)[i] = args.bops[i];
    if (tid < D) sOff[tid] = args.off[tid];
    if (tid == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(smem_addr(bars + s), S::PRODUCERS);
            mbar_init(smem_addr(bars + 2 + s), 1);
            mbar_init(smem_addr(bars + 4 + s), 1);
            mbar_init(smem_addr(bars + 6 + s), S::EPI);
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
        *abortFlag = 0;
    }
    if (warp == S::MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_addr(tmemSlot)), "r"(S::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmemSlot;
    const qidx first = blockIdx.x, step = gridDim.x;
    const qidx nLocal = args.numTiles > first ? (args.numTiles - first + step - 1) / step : 0;
    const uint32_t aFull = smem_addr(bars), infoReady = smem_addr(bars + 2), mmaDone = smem_addr(bars + 4),
                   tmemEmpty = smem_addr(bars + 6);
    // group g = 128 t + r of tile t starts at insert(128 t) | insert(r) | mask: the first
    // part is the same for the whole CTA, the second is fixed per thread
    auto tile_base = [&](qidx i) { return insert_bits<-1>((first + i * step) * 128, args.ins) | args.mask; };

    if (warp < S::MMA_WARP) {
        // ---------------- producers: thread (row, part) holds amplitudes part*AMPS .. of its
        // group; the two halves of a group are lanes l and l + 16 of one warp, so that the 8
        // lanes of each shared-store phase write 8 consecutive rows of one core column
        const int row = warp * 16 + (lane & 15), part = lane >> 4;
        const qidx rowOff = insert_bits<-1>((qidx)row, args.ins);
        // STG: tile i's amplitudes of this thread go to stage i % NSTAGE by cp.async, NSTAGE - 1
        // tiles ahead; each thread reads back only what it copied, so one wait_group per
        // tile orders them (one commit per tile, empty past the last).  Otherwise the loads of
        // tile i + 1 go into the registers of a k-core of tile i as soon as its digits are
        // formed.  (Staging gains where a warp's loads cover consecutive amplitudes and
        // qubit 0 is neither a target nor a control.)
        auto issue = [&](qidx i) {
            if (i < nLocal && (first + i * step) * 128 + row < args.numIts) {
                const double2* src = args.amps + (tile_base(i) + rowOff);
                double2* dst = sStage + (size_t)(i % S::NSTAGE) * AMPS * S::PRODUCERS + tid;
#pragma unroll
                for (int a = 0; a < AMPS; a++)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                                 :: "r"(smem_addr(dst + a * S::PRODUCERS)), "l"(src + sOff[part * AMPS + a]) : "memory");
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        double2 x[AMPS];
        auto load4 = [&](qidx i, int c) {
            const bool ok = (first + i * step) * 128 + row < args.numIts;
            const double2* src = args.amps + (tile_base(i) + rowOff);
#pragma unroll
            for (int a = 4 * c; a < 4 * c + 4; a++) x[a] = ok ? __ldcs(src + sOff[part * AMPS + a]) : make_double2(0.0, 0.0);
        };
        if constexpr (STG) {
#pragma unroll 1
            for (int j = 0; j < S::NSTAGE - 1; j++) issue(j);
        } else if (nLocal > 0) {
#pragma unroll
            for (int c = 0; c < AMPS / 4; c++) load4(0, c);
        }
        for (qidx i = 0; i < nLocal; i++) {
            const qidx g = (first + i * step) * 128 + row;
            const bool valid = g < args.numIts;
            double2* p = args.amps + (tile_base(i) + rowOff);
            if constexpr (STG) {
                issue(i + S::NSTAGE - 1);
                asm volatile("cp.async.wait_group %0;" :: "n"(S::NSTAGE - 1) : "memory");
                const double2* src = sStage + (size_t)(i % S::NSTAGE) * AMPS * S::PRODUCERS + tid;
#pragma unroll
                for (int a = 0; a < AMPS; a++) x[a] = valid ? src[a * S::PRODUCERS] : make_double2(0.0, 0.0);
            }
            const int s = (int)(i & 1);
            const uint32_t u = (uint32_t)(i >> 1);
            // the group's scale: the largest biased exponent of this half, then of the partner's
            uint32_t em = 0;
#pragma unroll
            for (int a = 0; a < AMPS; a++)
                em = max(em, max((uint32_t)__double2hiint(x[a].x) & 0x7FF00000u, (uint32_t)__double2hiint(x[a].y) & 0x7FF00000u));
            em = max(em, __shfl_xor_sync(0xffffffffu, em, 16));
            const int E = (int)(em >> 20);
            int nz = 0;
            if (E == 0) {      // zeros and denormals only: is any of them nonzero?
#pragma unroll
                for (int a = 0; a < AMPS; a++)
                    nz |= ((__double_as_longlong(x[a].x) << 1) | (__double_as_longlong(x[a].y) << 1)) != 0;
            }
            nz |= __shfl_xor_sync(0xffffffffu, nz, 16);
            const bool fp64 = valid && (E == 2047 || (E == 0 && nz) || (E != 0 && (E < args.elo || E > args.ehi)));
            const bool digits = valid && !fp64;
            const int Eg = E == 0 ? 1023 : E;
            const int Ew = digits ? Eg : 4095;           // 4095: every V is 0, W = CX
            // A[s] is free once the MMAs of tile i - 2 are done
            const bool bad = u >= 1 && !mbar_wait_bounded(mmaDone + 8 * s, (u - 1) & 1, DT_WAIT_NS);
            if (bad) *abortFlag = 1;
            if (__any_sync(0xffffffffu, bad || *abortFlag)) break;
            if (part == 0) sInfo[(i & 3) * 128 + row] = digits ? (Eg + args.eR - qgsl::SCALE_OFF) * (1 << 20) : DT_SKIP;
            // one k-core (8 reals, 4 amplitudes) at a time: its digit words, stored slice by slice
            unsigned char* aBuf = sA + s * S::A_BYTES;
#pragma unroll
            for (int c = 0; c < S::NV / 8; c++) {
                uint32_t dg[4][qgsl::XD];
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const double2 v = x[4 * c + a];
                    const uint32_t hx = (uint32_t)__double2hiint(v.x), hy = (uint32_t)__double2hiint(v.y);
                    dt_digits2(hx, hy, dt_word(hx, (uint32_t)__double2loint(v.x), Ew), dt_word(hy, (uint32_t)__double2loint(v.y), Ew), dg[a]);
                }
                if constexpr (!STG) {
                    if (i + 1 < nLocal) load4(i + 1, c);
                }
                unsigned char* dst = aBuf + dt_core_offset(row, part * S::NV + 8 * c, 128);
#pragma unroll
                for (int d = 0; d < qgsl::XD; d++) *(uint4*)(dst + d * S::SLICE) = make_uint4(dg[0][d], dg[1][d], dg[2][d], dg[3][d]);
            }
            asm volatile("fence.proxy.async.shared::cta;");
            mbar_arrive(aFull + 8 * s);
            // FP64 groups: both threads form their outputs before either stores
            const unsigned fm = __ballot_sync(0xffffffffu, fp64);
            if (fp64) {
                double2 out[AMPS];
#pragma unroll
                for (int a = 0; a < AMPS; a++) {
                    const int r = part * AMPS + a;
                    double2 acc = make_double2(0.0, 0.0);
#pragma unroll 1
                    for (int j = 0; j < D; j++) acc = cfma(args.m[r * D + j], p[sOff[j]], acc);
                    out[a] = acc;
                }
                __syncwarp(fm);
#pragma unroll
                for (int a = 0; a < AMPS; a++) p[sOff[part * AMPS + a]] = out[a];
            }
        }
        if constexpr (STG) asm volatile("cp.async.wait_all;" ::: "memory");      // none left in flight at exit
    } else if (warp == S::MMA_WARP) {
        // ---------------- MMA issue (one thread)
        if (lane == 0) {
            const uint32_t lboA = (128 / 8) * 128, lboB = (S::B_ROWS / 8) * 128, sbo = 128;
            const uint32_t bBase = smem_addr(sB);
            qidx issued = 0;
            for (qidx i = 0; i < nLocal; i++) {
                const int s = (int)(i & 1);
                const uint32_t u = (uint32_t)(i >> 1);
                if (!mbar_wait_bounded(aFull + 8 * s, u & 1, DT_WAIT_NS)) *abortFlag = 1;
                if (!*abortFlag && u >= 1 && !mbar_wait_bounded(tmemEmpty + 8 * s, (u - 1) & 1, DT_WAIT_NS)) *abortFlag = 1;
                if (*abortFlag) break;
                mbar_arrive(infoReady + 8 * s);      // the producers' scales, seen through aFull
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t aBase = smem_addr(sA + s * S::A_BYTES);
                const uint32_t dBase = tmem + (uint32_t)(s * S::DCOLS);
#pragma unroll
                for (int d = 0; d < qgsl::XD; d++) {
                    const uint32_t idesc = dt_idesc((qgsl::NSUM - d) * KR);
#pragma unroll
                    for (int kk = 0; kk < KR / 16; kk++)
                        mma_f16(dBase + (uint32_t)(d * KR), make_desc(aBase + d * S::SLICE + kk * 2 * lboA, lboA, sbo),
                                 make_desc(bBase + kk * 2 * lboB, lboB, sbo), idesc, (d > 0 || kk > 0) ? 1u : 0u);
                }
                mma_commit(mmaDone + 8 * s);
                issued = i + 1;
            }
            // no MMA may still be running when the accumulators are freed
            if (issued > 0) {
                const qidx l = issued - 1;
                if (!mbar_wait_bounded(mmaDone + 8 * (int)(l & 1), (uint32_t)(l >> 1) & 1, DT_WAIT_NS)) *abortFlag = 1;
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: TMEM lane quarter = warp % 4, half of the outputs = which four warps
        const int quarter = warp & 3, half = (warp - S::MMA_WARP - 1) >> 2;
        const int row = 32 * quarter + lane;
        const qidx rowOff = insert_bits<-1>((qidx)row, args.ins);
        const qidx* offs = sOff + half * (D / 2);
        for (qidx i = 0; i < nLocal; i++) {
            const int s = (int)(i & 1);
            const uint32_t u = (uint32_t)(i >> 1);
            const bool waited = mbar_wait_bounded(infoReady + 8 * s, u & 1, DT_WAIT_NS) &&
                                mbar_wait_bounded(mmaDone + 8 * s, u & 1, DT_WAIT_NS);
            // the warp leaves together: it runs warp-collective TMEM loads
            const bool ok = __all_sync(0xffffffffu, waited);
            if (!ok && lane == 0) *abortFlag = 1;
            if (!ok || __shfl_sync(0xffffffffu, lane == 0 ? *abortFlag : 0, 0)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const int shift20 = sInfo[(i & 3) * 128 + row];
            double2* dst = args.amps + (tile_base(i) + rowOff);
            const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(s * S::DCOLS + half * (KR / 2));
            // chunks of CHUNK output reals: 8 digit sums x CHUNK columns in registers (a loop,
            // not unrolled: the smaller body was measured faster)
            constexpr int CH = S::CHUNK;
#pragma unroll 1
            for (int c = 0; c < KR / 2 / CH; c++) {
                uint32_t r[qgsl::NSUM][CH];
#pragma unroll
                for (int sd = 0; sd < qgsl::NSUM; sd++) {
                    if constexpr (CH == 8) TMEM_LD8(taddr + (uint32_t)(sd * KR + CH * c), r[sd]);
                    else TMEM_LD4(taddr + (uint32_t)(sd * KR + CH * c), r[sd]);
                }
                tmem_wait_ld();
                if (c == KR / 2 / CH - 1) {
                    asm volatile("tcgen05.fence::before_thread_sync;");
                    mbar_arrive(tmemEmpty + 8 * s);
                }
                if (shift20 != DT_SKIP) {
#pragma unroll
                    for (int q = 0; q < CH / 2; q++)
                        __stcs(dst + offs[CH / 2 * c + q],
                               make_double2(dt_output(r, 2 * q, shift20), dt_output(r, 2 * q + 1, shift20)));
                }
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
    if (warp == S::MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(S::TMEM_COLS));
}

// ---------------------------------------------------------------- host

int qg_tc_prepare();
int qg_tc_take_error();
int qg_tc_device_flag(int** out);

namespace {
std::atomic<int> g_slices{1};

// optional CUDA events around each launch (qg_dense_tc_timing), for a caller's roofline
std::mutex g_timeMu;
bool g_timing = false;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_times;

template <int KR, bool STG>
int dt_set_attr() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    QG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return qg_fail(QG_ERR_NOTSUP, "device %d is beyond this build's device table", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!done[dev]) {
        QG_CUDA(cudaFuncSetAttribute(k_dense_tc<KR, STG>, cudaFuncAttributeMaxDynamicSharedMemorySize, DtShape<KR, STG>::SMEM));
        done[dev] = true;
    }
    return QG_OK;
}
}  // namespace

// whether a K-target gate on numIts groups takes the tensor-core slices (mode 1: at least
// one tile of 128 groups per SM; mode 2: any size, for tests of small registers)
bool qg_dense_tc_wanted(qidx numIts) {
    const int mode = g_slices.load();
    return mode == 2 || (mode == 1 && numIts >= (qidx)128 * qg_num_sms());
}

// The launch for a K-target gate (K = 3, 4) on numIts groups (the plan's insertion of
// controls and targets, matrix m row-major with the gate's conjugation applied, off[j]
// the offset of matrix index j).  *used = false (nothing launched) when the matrix is
// not finite; the caller then keeps FP64.
template <int K>
int qg_dense_tc_launch(double2* amps, qidx numIts, const Ins& ins, qidx mask, const double2* m, const qidx* off,
                       cudaStream_t st, bool* used) {
    constexpr int KR = 2 << K, D = 1 << K;
    using S = DtShape<KR, false>;
    *used = false;
    // A target on qubit 0 becomes the matrix's top index bit (the operator and the offsets
    // permuted to match): the two threads of a group then hold its halves with qubit 0 clear
    // and set, so lanes l and l + 16 read adjacent amplitudes (4-8 % faster than qubit 0 as the
    // lowest index bit for targets 0..3 and 0, 3, 4, 17 at 28 qubits; within 2 % elsewhere).
    int zb = -1;
    for (int b = 0; b < K; b++)
        if (off[1 << b] == 1) zb = b;
    std::vector<double2> mp(m, m + D * D);
    std::vector<qidx> op(off, off + D);
    if (zb >= 0 && zb != K - 1) {
        int oldBit[K], k2 = 0;
        for (int b = 0; b < K; b++)
            if (b != zb) oldBit[k2++] = b;
        oldBit[K - 1] = zb;
        auto oldIndex = [&](int jn) {
            int jo = 0;
            for (int b = 0; b < K; b++) jo |= ((jn >> b) & 1) << oldBit[b];
            return jo;
        };
        for (int jn = 0; jn < D; jn++) {
            op[jn] = off[oldIndex(jn)];
            for (int cn = 0; cn < D; cn++) mp[jn * D + cn] = m[oldIndex(jn) * D + oldIndex(cn)];
        }
        m = mp.data();
        off = op.data();
    }
    std::vector<double> u(2 * D * D), R(KR * KR);
    for (int i = 0; i < D * D; i++) { u[2 * i] = m[i].x; u[2 * i + 1] = m[i].y; }
    qgfx::real_form(u.data(), D, R.data());
    std::vector<int8_t> dig(qgsl::RD * KR * KR);
    int eR = 0;
    if (!qgsl::operator_digits(R.data(), KR, dig.data(), &eR)) return QG_OK;
    QG_TRY(qg_tc_take_error());
    QG_TRY(qg_tc_prepare());
    std::unique_ptr<DtArgs<KR>> a(new DtArgs<KR>());
    a->amps = amps;
    a->numIts = numIts;
    a->numTiles = (numIts + 127) / 128;
    a->ins = ins;
    a->mask = mask;
    for (int j = 0; j < D; j++) a->off[j] = off[j];
    a->eR = eR;
    a->elo = std::max(qgsl::EMIN, qgsl::EMIN - eR);
    a->ehi = qgsl::EMAX - eR;
    QG_TRY(qg_tc_device_flag(&a->errorFlag));
    for (int i = 0; i < D * D; i++) a->m[i] = m[i];
    std::vector<uint16_t> bt(S::B_BYTES / 2, 0);
    for (int j = 0; j < qgsl::RD; j++)
        for (int n = 0; n < KR; n++)
            for (int k = 0; k < KR; k++)
                bt[dt_core_offset(j * KR + n, k, S::B_ROWS) / 2] = qgsl::digit_half(dig[(j * KR + n) * KR + k]);
    std::memcpy(a->bops, bt.data(), S::B_BYTES);
    const unsigned grid = (unsigned)std::min<qidx>(a->numTiles, (qidx)qg_num_sms());
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_timeMu);
        if (g_timing) {
            QG_CUDA(cudaEventCreate(&ev0));
            QG_CUDA(cudaEventCreate(&ev1));
            g_times.push_back({ev0, ev1});
            QG_CUDA(cudaEventRecord(ev0, st));
        }
    }
    bool staged = false;
    if constexpr (KR == 32) {
        // qubit 0 neither a target nor a control: with a control there, a warp's loads take
        // every other amplitude; with a target there (the top index bit), the staged form
        // measured 2-4 % slower than the register form on most placements at 28 qubits
        staged = ins.num == 0 || ins.low[0] != 0;
        if (staged) {
            QG_TRY((dt_set_attr<KR, true>()));
            k_dense_tc<KR, true><<<grid, DtShape<KR, true>::THREADS, DtShape<KR, true>::SMEM, st>>>(*a);
        }
    }
    if (!staged) {
        QG_TRY((dt_set_attr<KR, false>()));
        k_dense_tc<KR, false><<<grid, S::THREADS, S::SMEM, st>>>(*a);
    }
    if (ev1) QG_CUDA(cudaEventRecord(ev1, st));
    *used = true;      // the launch is counted by the caller (qg_sv_anyCtrlAnyTargDenseMatr), once per call
    return qg_check_launch("k_dense_tc");
}

template int qg_dense_tc_launch<3>(double2*, qidx, const Ins&, qidx, const double2*, const qidx*, cudaStream_t, bool*);
template int qg_dense_tc_launch<4>(double2*, qidx, const Ins&, qidx, const double2*, const qidx*, cudaStream_t, bool*);

extern "C" {

int qg_set_tensor_slices(int enable) {
    if (enable < 0 || enable > 2) return qg_fail(QG_ERR_ARG, "tensor slices: 0, 1 or 2, not %d", enable);
    g_slices.store(enable);
    return QG_OK;
}

int qg_get_tensor_slices(int* enable) {
    if (!enable) return qg_fail(QG_ERR_ARG, "null argument");
    *enable = g_slices.load();
    return QG_OK;
}

int qg_dense_tc_timing(int enable) {
    std::lock_guard<std::mutex> lock(g_timeMu);
    for (auto& e : g_times) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    g_times.clear();
    g_timing = enable != 0;
    return QG_OK;
}

int qg_dense_tc_timing_read(float* msOut, int maxOut, int* numOut) {
    if (!numOut || (maxOut > 0 && !msOut)) return qg_fail(QG_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lock(g_timeMu);
    int n = 0;
    for (auto& e : g_times) {
        float ms = 0;
        QG_CUDA(cudaEventSynchronize(e.second));
        QG_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
        if (n < maxOut) msOut[n] = ms;
        n++;
    }
    *numOut = n;
    return QG_OK;
}

}  // extern "C"
