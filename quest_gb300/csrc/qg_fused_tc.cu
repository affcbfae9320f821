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
// Per CTA tile: 256 threads, two per group row, each load 16 of the group's 32
// amplitudes (coalesced 8-byte loads: consecutive threads own consecutive groups),
// split them into TF32 hi/lo parts and store both into shared memory in the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix); one thread issues the
// 24 MMAs (3 products x 8 K-steps of 8) into two 128-lane x 64-column TMEM
// accumulators (large term, small terms) and commits them to an mbarrier; every
// warp then reads its 32 TMEM lanes (tcgen05.ld 32x32b) in its half of the columns,
// adds the two accumulators in FP32 and writes its groups' 16 outputs back.
// Every wait is bounded: a wait that runs out sets the error flag, frees the
// TMEM and returns.
#include "qg_common.cuh"

#include <mutex>

#include <cmath>
#include <complex>
#include <cstring>

#define TC_M 128              // groups per tile (MMA M)
#define TC_K 64               // real K (32 complex amplitudes)
#define TC_N 64               // real N
#define TC_THREADS 256           // two threads per group row: each holds 16 of its 32 amplitudes
#define TC_TMEM_COLS 128          // two 64-column accumulators: the large and the small 3xTF32 terms
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

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version for tcgen05
    return d;                 // base offset 0, relative LBO, no swizzle
}

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

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

// bounded wait on an mbarrier phase; false if it ran out.  The clock is read once
// per 256 polls, not per poll.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        for (int i = 0; i < 256; i++)
            if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > TC_WAIT_NS) return false;
    }
}

#define TMEM_LD16(taddr, r)                                                                              \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),    \
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]) \
                 : "r"(taddr))

// ---------------------------------------------------------------- kernel

struct TcArgs {
    float2* amps;
    qidx numTiles;     // groups / 128
    Ins ins;           // the five sorted targets, as insertion masks
    qidx off[32];      // amplitude offset of matrix index j within a group
    const float* ops;  // Bh, Bl (global)
    int* errorFlag;    // set to 1 if a bounded wait ran out
};

__global__ void __launch_bounds__(TC_THREADS, 2) k32_fused_tc(TcArgs args) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float* sAh = (float*)smem;
    float* sAl = (float*)(smem + TC_A_BYTES);
    float* sBh = (float*)(smem + 2 * TC_A_BYTES);
    float* sBl = (float*)(smem + 2 * TC_A_BYTES + TC_B_BYTES);
    uint64_t* bar = (uint64_t*)(smem + 2 * TC_A_BYTES + 2 * TC_B_BYTES);
    uint32_t* tmemSlot = (uint32_t*)(bar + 1);
    volatile int* abortFlag = (volatile int*)(tmemSlot + 1);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid & (TC_M - 1), half = tid >> 7;   // thread (row g, half h): j in [16h, 16h+16)

    // stage Bh, Bl once (already in the tile layout)
    {
        const float4* src = (const float4*)args.ops;
        float4* dst = (float4*)sBh;   // sBh and sBl are contiguous
        for (int i = tid; i < (2 * TC_B_BYTES) / 16; i += TC_THREADS) dst[i] = __ldg(src + i);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;");
        *abortFlag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_addr(tmemSlot)), "r"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmemSlot;
    const uint32_t idesc = make_idesc();
    const uint32_t aH = smem_addr(sAh), aL = smem_addr(sAl), bH = smem_addr(sBh), bL = smem_addr(sBl);
    const uint32_t barAddr = smem_addr(bar);
    uint32_t phase = 0;

    // Software pipeline: the next tile's 32 amplitudes per thread are loaded into
    // registers while this tile's MMAs run and its results are written back.
    qidx tile = blockIdx.x;
    float2 x[16];
    qidx base = 0;
    if (tile < args.numTiles) {
        base = insert_bits<5>(tile * TC_M + row, args.ins);
#pragma unroll
        for (int i = 0; i < 16; i++) x[i] = __ldcs(args.amps + base + args.off[16 * half + i]);
    }
    for (; tile < args.numTiles; tile += gridDim.x) {
        // ---- split into TF32 hi/lo and store in the K-major core layout (kk = 2j + c)
#pragma unroll
        for (int q = 0; q < 8; q++) {
            float4 h, l;
            h.x = tf32_hi(x[2 * q].x);     l.x = tf32_hi(x[2 * q].x - h.x);
            h.y = tf32_hi(x[2 * q].y);     l.y = tf32_hi(x[2 * q].y - h.y);
            h.z = tf32_hi(x[2 * q + 1].x); l.z = tf32_hi(x[2 * q + 1].x - h.z);
            h.w = tf32_hi(x[2 * q + 1].y); l.w = tf32_hi(x[2 * q + 1].y - h.w);
            unsigned o = core_offset(row, 4 * (8 * half + q), TC_M);
            *(float4*)((unsigned char*)sAh + o) = h;
            *(float4*)((unsigned char*)sAl + o) = l;
        }
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");

        // ---- one thread issues the 24 MMAs (8 K-steps per product) and commits them:
        //      columns 64..127 accumulate the small terms Al*Bh + Ah*Bl, columns 0..63 the
        //      large term Ah*Bh; the epilogue adds the two in FP32
        if (tid == 0) {
            const uint32_t lboA = (TC_M / 8) * 128, lboB = (TC_N / 8) * 128, sbo = 128;
            for (int part = 0; part < 3; part++) {
                uint32_t a = (part == 0) ? aL : aH;
                uint32_t b = (part == 1) ? bL : bH;
                uint32_t d = (part == 2) ? tmem : tmem + TC_N;
                uint32_t acc = (part == 1) ? 1u : 0u;
#pragma unroll
                for (int s = 0; s < TC_K / 8; s++) {
                    uint64_t ad = make_desc(a + s * 2 * lboA, lboA, sbo);
                    uint64_t bd = make_desc(b + s * 2 * lboB, lboB, sbo);
                    mma_tf32(d, ad, bd, idesc, acc);
                    acc = 1;
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(barAddr) : "memory");
        }

        // ---- while the MMAs run: load the next tile (registers only; shared memory is busy)
        const qidx cur = base;
        const qidx next = tile + gridDim.x;
        if (next < args.numTiles) {
            base = insert_bits<5>(next * TC_M + row, args.ins);
#pragma unroll
            for (int i = 0; i < 16; i++) x[i] = __ldcs(args.amps + base + args.off[16 * half + i]);
        }

        // ---- every thread waits for the MMAs (bounded by %globaltimer)
        if (!mbar_wait_bounded(barAddr, phase)) *abortFlag = 1;
        phase ^= 1;
        __syncthreads();
        if (*abortFlag) {
            if (tid == 0) atomicExch(args.errorFlag, 1);
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");

        // ---- epilogue: warp w reads TMEM lanes 32(w mod 4).. (its groups) and the 32
        //      columns of its half (outputs k in [16h, 16h+16)), 16 at a time
        const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + 32 * half;
#pragma unroll
        for (int c = 0; c < 2; c++) {
            uint32_t big[16], small[16];
            TMEM_LD16(taddr + 16 * c, big);
            TMEM_LD16(taddr + TC_N + 16 * c, small);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float re = __uint_as_float(small[2 * k]) + __uint_as_float(big[2 * k]);
                float im = __uint_as_float(small[2 * k + 1]) + __uint_as_float(big[2 * k + 1]);
                __stcs(args.amps + cur + args.off[16 * half + 8 * c + k], make_float2(re, im));
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();   // TMEM and the A buffers may now be overwritten
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TC_TMEM_COLS));
}

// ---------------------------------------------------------------- host: launch

namespace {
int* g_tc_error = nullptr;
}

bool qg_tc_supported(int numQubits) { return numQubits >= 12; }

// one-time set-up (the error flag's memory, the kernel's shared-memory limit); done
// before the first launch and before any stream capture of one
int qg_tc_prepare() {
    static std::mutex mu;
    static bool attr = false;
    std::lock_guard<std::mutex> lock(mu);
    if (!g_tc_error) {
        QG_CUDA(cudaMalloc(&g_tc_error, sizeof(int)));
        QG_CUDA(cudaMemset(g_tc_error, 0, sizeof(int)));
    }
    if (!attr) {
        const size_t smem = 2 * TC_A_BYTES + 2 * TC_B_BYTES + 64 + 1024;
        QG_CUDA(cudaFuncSetAttribute(k32_fused_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    return QG_OK;
}

int qg_tc_apply_block(float2* amps, int numQubits, const int* targs, const float* devOperands, cudaStream_t st) {
    if (numQubits < 12) return qg_fail(QG_ERR_ARG, "the tensor-core block kernel needs at least 12 qubits (one 128-group tile)");
    if (!g_tc_error) QG_TRY(qg_tc_prepare());
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
    a.errorFlag = g_tc_error;
    int sms = qg_num_sms();
    size_t smem = 2 * TC_A_BYTES + 2 * TC_B_BYTES + 64 + 1024;
    qidx grid = std::min<qidx>(a.numTiles, (qidx)sms * 2);
    k32_fused_tc<<<(unsigned)grid, TC_THREADS, smem, st>>>(a);
    qg_note_launch();
    return qg_check_launch("k32_fused_tc");
}

extern "C" int qg_tc_get_error_flag(int* out) {
    if (!g_tc_error) { *out = 0; return QG_OK; }
    QG_CUDA(cudaMemcpy(out, g_tc_error, sizeof(int), cudaMemcpyDeviceToHost));
    return QG_OK;
}
