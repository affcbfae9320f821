// Batched Pauli expectation values of an FP64 statevector that allocate nothing.
//
// The regular reductions keep their partial sums in a library scratch buffer
// that grows on demand with cudaMalloc (and read results back through a pinned
// buffer from cudaMallocHost).  Some callers cannot allow that: a process whose
// device memory is handed wholesale to another allocator (a framework's caching
// allocator or a serving engine that reserves HBM up front), or a latency-bound
// loop that must not hit cudaMalloc's implicit device synchronisation.  This
// entry point serves them: its scratch is a fixed array in this file's device
// memory, which every GPU that loads the library holds until the process exits.
//
// Host code must not pass `g_noalloc_scratch` itself to a kernel: on the host
// that name is only a stand-in for the device array.  Its device address is
// looked up once per device with cudaGetSymbolAddress (with that device
// current) at the first call made on that device, so that first call does the
// set-up and should come before any stream capture.  All calls share the one
// array and it keeps the last call's contents: the completion ticket is cleared
// at every call, and calls that overlap on the GPU (on different streams) race.
#include "qg_reduce.cuh"

#define NOALLOC_NS 16                     // strings per launch
#define NOALLOC_MAX_GRID 1024             // blocks per launch
#define NOALLOC_MAX_DEVICES 64

// [ticket 256 B][results: 2*QG_NOALLOC_MAX_STRINGS doubles][partials: 2*NS*MAX_GRID doubles]
#define NOALLOC_RESULTS_OFF 256
#define NOALLOC_PARTIALS_OFF (256 + 8 * 2 * QG_NOALLOC_MAX_STRINGS)
#define NOALLOC_BYTES (NOALLOC_PARTIALS_OFF + 8 * 2 * NOALLOC_NS * NOALLOC_MAX_GRID)

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

struct NoallocMasks {
    qidx xy[NOALLOC_NS];
    qidx yz[NOALLOC_NS];
};

// the reference's per-n term sign(j & maskYZ) conj(a_n) a_j, j = n ^ maskXY
// (cpu_subroutines.cpp:2059-2085), for up to 16 strings in one pass
__global__ void __launch_bounds__(RED_THREADS) k_noalloc_expec_pauli(const double2* __restrict__ a, qidx n, NoallocMasks m,
                                                                    int numStrings, RedOut out) {
    double v[2 * NOALLOC_NS];
#pragma unroll
    for (int k = 0; k < 2 * NOALLOC_NS; k++) v[k] = 0.0;
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx i = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; i < n; i += stride) {
        double2 an = __ldg(a + i);
#pragma unroll
        for (int s = 0; s < NOALLOC_NS; s++) {
            if (s < numStrings) {
                qidx j = i ^ m.xy[s];
                double2 aj = __ldg(a + j);
                double sg = parity64(j & m.yz[s]) ? -1.0 : 1.0;
                v[2 * s] += sg * fma(an.x, aj.x, an.y * aj.y);
                v[2 * s + 1] += sg * fma(an.x, aj.y, -an.y * aj.x);
            }
        }
    }
    block_reduce_and_finish<2 * NOALLOC_NS>(v, out);
}

namespace {

unsigned char* g_scratchAddr[NOALLOC_MAX_DEVICES];   // device address of g_noalloc_scratch, per device
int g_numSMs[NOALLOC_MAX_DEVICES];

int noalloc_setup(int dev, unsigned char** addr, int* sms) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return qg_fail(QG_ERR_NOTSUP, "device %d beyond the %d supported", dev, NOALLOC_MAX_DEVICES);
    if (!g_scratchAddr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return qg_check_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return qg_check_cuda(e, "cudaDeviceGetAttribute");
        g_numSMs[dev] = n > 0 ? n : 1;
        g_scratchAddr[dev] = (unsigned char*)p;
    }
    *addr = g_scratchAddr[dev];
    *sms = g_numSMs[dev];
    return QG_OK;
}

}  // namespace

extern "C" int qg_sv_calcExpecPauliStrBatch_noalloc(const void* amps, int numQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                                    const int* numsY, int numStrings, qg_cplx* out, void* stream) {
    QG_TRY(qg_check_amps(amps, numQubits));
    if (numStrings < 0 || numStrings > QG_NOALLOC_MAX_STRINGS)
        return qg_fail(QG_ERR_ARG, "%d Pauli strings requested; this entry point takes at most %d per call",
                       numStrings, QG_NOALLOC_MAX_STRINGS);
    if (numStrings > 0 && (!masksXY || !masksYZ || !numsY || !out)) return qg_fail(QG_ERR_ARG, "null argument");
    qidx lim = ((qidx)1 << numQubits) - 1;
    for (int s = 0; s < numStrings; s++)
        if ((masksXY[s] & ~lim) || (masksYZ[s] & ~lim)) return qg_fail(QG_ERR_ARG, "Pauli string %d targets a qubit beyond %d", s, numQubits);
    if (numStrings == 0) return QG_OK;
    int dev = 0;
    QG_CUDA(cudaGetDevice(&dev));
    unsigned char* base = nullptr;
    int sms = 1;
    QG_TRY(noalloc_setup(dev, &base, &sms));
    cudaStream_t st = qg_stream(stream);
    qidx n = (qidx)1 << numQubits;
    qidx need = (n + RED_THREADS - 1) / RED_THREADS;
    int grid = (int)std::min<qidx>(std::min<qidx>((qidx)sms * 4, NOALLOC_MAX_GRID), std::max<qidx>(1, need));
    QG_CUDA(cudaMemsetAsync(base, 0, 256, st));   // the completion ticket starts at zero
    for (int s0 = 0; s0 < numStrings; s0 += NOALLOC_NS) {
        int cnt = std::min(NOALLOC_NS, numStrings - s0);
        NoallocMasks m;
        for (int k = 0; k < NOALLOC_NS; k++) {
            m.xy[k] = k < cnt ? masksXY[s0 + k] : 0;
            m.yz[k] = k < cnt ? masksYZ[s0 + k] : 0;
        }
        RedOut r;
        r.ticket = (unsigned int*)base;
        r.result = (double*)(base + NOALLOC_RESULTS_OFF) + 2 * s0;
        r.partials = (double*)(base + NOALLOC_PARTIALS_OFF);
        k_noalloc_expec_pauli<<<grid, RED_THREADS, 0, st>>>((const double2*)amps, n, m, cnt, r);
        qg_note_launch();
        QG_TRY(qg_check_launch("k_noalloc_expec_pauli"));
    }
    double v[2 * QG_NOALLOC_MAX_STRINGS];
    QG_CUDA(cudaMemcpyAsync(v, base + NOALLOC_RESULTS_OFF, sizeof(double) * 2 * numStrings, cudaMemcpyDeviceToHost, st));
    QG_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < numStrings; s++) {
        double re = v[2 * s], im = v[2 * s + 1];
        times_power_of_i(&re, &im, numsY[s]);
        out[s].re = re;
        out[s].im = im;
    }
    return QG_OK;
}
