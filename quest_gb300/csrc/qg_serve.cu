// Continuous-batching circuit server on one GPU (the serving form of the gate path).
//
// Requests are compiled circuits (qg_circuit, fused into <=5-qubit blocks) on
// FP32 statevectors starting in |0>, each returning a list of Pauli expectation
// values (FP64 accumulation).  The server keeps two execution paths:
//
//  * small registers (<= 14 qubits, <= 128 KiB of amplitudes): every request runs
//    whole inside ONE thread block -- state in shared memory, all its fused blocks,
//    then its expectation values -- and every small request admitted since the
//    last scheduling step goes into ONE launch (one CTA per request, uneven qubit
//    counts side by side);
//  * large registers: the state lives in an HBM arena sub-allocated from a budget
//    fixed at creation (admission control by bytes), each request gets a
//    non-blocking stream from a pool, and its fused blocks run as whole-state
//    passes (tensor-core 3xTF32 kernel for 5-qubit blocks) followed by an
//    asynchronous batched expectation reduction.
//
// qg_server_poll() is one non-blocking scheduling step: it admits queued
// requests in arrival order while the byte budget and the slot count allow,
// launches their work, and retires requests whose completion event has fired.
// Requests that arrive while others are on the GPU are admitted as soon as
// memory frees up, and their work overlaps with the work already in flight.
// Each request's arithmetic is independent of what else runs, so its results
// are the same alone and in any mix.
#include "qg_circuit.cuh"
#include "qg_reduce.cuh"

#include <algorithm>
#include <deque>
#include <map>
#include <vector>

#define SERVE_MAX_STRINGS 16
// per result slot: (re, im) per string, then <psi|psi> and a zero
#define SERVE_RESULT_DOUBLES (2 * SERVE_MAX_STRINGS + 2)
#define SERVE_SMALL_MAX_QUBITS 14
#define SERVE_SMALL_THREADS 256
#define SERVE_STREAMS 16

extern "C" int qg_sv32_apply_circuit_flag(qg_circuit* c, void* amps, int numQubits, int impl, cudaStream_t st, int* errorFlag);

// ============================================================== device: small registers in shared memory

struct SmallJob {
    const QgBlockInfo* info;   // the circuit's blocks
    const float2* mats;        // the circuit's FP32 block matrices
    int numBlocks;
    int nq;
    int numStrings;
    int pad;
    qidx xy[SERVE_MAX_STRINGS];
    qidx yz[SERVE_MAX_STRINGS];
    double* out;               // SERVE_RESULT_DOUBLES: (re, im) per string before the i^numY factor, then the norm
    float2* stateOut;          // optional copy of the final state (nullptr: none)
};

template <int K>
__device__ __forceinline__ void smem_block(float2* st, int N, const QgBlockInfo& b, const float2* M) {
    constexpr int D = 1 << K;
    qidx low[K];
    int off[D];
#pragma unroll
    for (int i = 0; i < K; i++) low[i] = ((qidx)1 << b.t[i]) - 1;
#pragma unroll
    for (int j = 0; j < D; j++) {
        int o = 0;
#pragma unroll
        for (int i = 0; i < K; i++) if ((j >> i) & 1) o |= 1 << b.t[i];
        off[j] = o;
    }
    const int groups = N >> K;
    for (int g = threadIdx.x; g < groups; g += blockDim.x) {
        qidx base = g;
#pragma unroll
        for (int i = 0; i < K; i++) { qidx lo = base & low[i]; base = ((base ^ lo) << 1) | lo; }
        float2 v[D];
#pragma unroll
        for (int j = 0; j < D; j++) v[j] = st[base + off[j]];
#pragma unroll
        for (int r = 0; r < D; r++) {
            float2 acc = cmulf(M[r * D], v[0]);
#pragma unroll
            for (int j = 1; j < D; j++) acc = cfmaf(M[r * D + j], v[j], acc);
            st[base + off[r]] = acc;
        }
    }
}

__global__ void __launch_bounds__(SERVE_SMALL_THREADS) k_serve_small(const SmallJob* __restrict__ jobs) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const SmallJob J = jobs[blockIdx.x];
    const int N = 1 << J.nq;
    float2* mat = (float2*)smraw;                 // 32 x 32 staged block matrix (8 KiB)
    float2* st = (float2*)(smraw + 8192);         // the register
    for (int i = threadIdx.x; i < N; i += blockDim.x) st[i] = make_float2(i == 0 ? 1.f : 0.f, 0.f);
    for (int b = 0; b < J.numBlocks; b++) {
        const QgBlockInfo info = J.info[b];
        const int D = 1 << info.k;
        __syncthreads();
        for (int i = threadIdx.x; i < D * D; i += blockDim.x) mat[i] = J.mats[info.off32 + i];
        __syncthreads();
        switch (info.k) {
            case 1: smem_block<1>(st, N, info, mat); break;
            case 2: smem_block<2>(st, N, info, mat); break;
            case 3: smem_block<3>(st, N, info, mat); break;
            case 4: smem_block<4>(st, N, info, mat); break;
            default: smem_block<5>(st, N, info, mat); break;
        }
    }
    __syncthreads();
    if (J.stateOut)
        for (int i = threadIdx.x; i < N; i += blockDim.x) J.stateOut[i] = st[i];
    // <psi|psi> then the expectation values sum_i sign(j & yz) conj(a_i) a_j, j = i ^ xy, in FP64
    __shared__ double red[SERVE_SMALL_THREADS / 32][2];
    {
        double nrm = 0;
        for (int i = threadIdx.x; i < N; i += blockDim.x) nrm += (double)st[i].x * st[i].x + (double)st[i].y * st[i].y;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nrm += __shfl_down_sync(0xffffffffu, nrm, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][0] = nrm;
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0;
            for (int w = 0; w < SERVE_SMALL_THREADS / 32; w++) a += red[w][0];
            J.out[2 * SERVE_MAX_STRINGS] = a;
            J.out[2 * SERVE_MAX_STRINGS + 1] = 0;
        }
        __syncthreads();
    }
    for (int s = 0; s < J.numStrings; s++) {
        double re = 0, im = 0;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            int j = i ^ (int)J.xy[s];
            float2 ai = st[i], aj = st[j];
            double sg = parity64(j & J.yz[s]) ? -1.0 : 1.0;
            re += sg * ((double)ai.x * aj.x + (double)ai.y * aj.y);
            im += sg * ((double)ai.x * aj.y - (double)ai.y * aj.x);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_down_sync(0xffffffffu, re, o);
            im += __shfl_down_sync(0xffffffffu, im, o);
        }
        if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5][0] = re; red[threadIdx.x >> 5][1] = im; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0, c = 0;
            for (int w = 0; w < SERVE_SMALL_THREADS / 32; w++) { a += red[w][0]; c += red[w][1]; }
            J.out[2 * s] = a;
            J.out[2 * s + 1] = c;
        }
        __syncthreads();
    }
}

// ============================================================== device: expectation values of a large register

struct ExpecMasks {
    qidx xy[SERVE_MAX_STRINGS];
    qidx yz[SERVE_MAX_STRINGS];
};

__global__ void __launch_bounds__(RED_THREADS) k_serve_expec(const float2* __restrict__ a, qidx n, ExpecMasks m,
                                                            int numStrings, RedOut out) {
    double v[SERVE_RESULT_DOUBLES];
#pragma unroll
    for (int k = 0; k < SERVE_RESULT_DOUBLES; k++) v[k] = 0.0;
    qidx stride = (qidx)gridDim.x * RED_THREADS;
    for (qidx i = blockIdx.x * (qidx)RED_THREADS + threadIdx.x; i < n; i += stride) {
        float2 ai = __ldg(a + i);
        v[2 * SERVE_MAX_STRINGS] += (double)ai.x * ai.x + (double)ai.y * ai.y;
#pragma unroll
        for (int s = 0; s < SERVE_MAX_STRINGS; s++) {
            if (s < numStrings) {
                qidx j = i ^ m.xy[s];
                float2 aj = __ldg(a + j);
                double sg = parity64(j & m.yz[s]) ? -1.0 : 1.0;
                v[2 * s] += sg * ((double)ai.x * aj.x + (double)ai.y * aj.y);
                v[2 * s + 1] += sg * ((double)ai.x * aj.y - (double)ai.y * aj.x);
            }
        }
    }
    block_reduce_and_finish<SERVE_RESULT_DOUBLES>(v, out);
}

// ============================================================== host: the server

namespace {

struct Request {
    int64_t id;
    qg_circuit* circ;
    int nq;
    int numStrings;
    qidx xy[SERVE_MAX_STRINGS], yz[SERVE_MAX_STRINGS];
    int ny[SERVE_MAX_STRINGS];
    int slot = -1;           // device / pinned result slot
    size_t arenaOff = 0, arenaBytes = 0;     // state + reduction scratch (large) and the circuit copy
    int stream = -1;         // large requests: index into the stream pool
    cudaEvent_t done = nullptr;
    bool small = false;
    bool unitary = true;     // every gate of the circuit is unitary: results are normalised
    bool finished = false;
    bool cancelled = false;  // the client went away while it ran: dropped when it completes
    bool timedOut = false;   // a tensor-core launch of it gave up a bounded wait: no values
    std::vector<double> values;
};

struct Batch {
    std::vector<int64_t> ids;
    cudaEvent_t done;
    SmallJob* devJobs;
};

}  // namespace

struct qg_server {
    int impl = 0;
    int maxSlots = 0;
    char* arena = nullptr;
    size_t arenaBytes = 0;
    std::map<size_t, size_t> freeList;        // offset -> size
    size_t inUse = 0;
    double* devResults = nullptr;             // [maxSlots][2*16]
    double* hostResults = nullptr;            // pinned mirror
    int* devFlags = nullptr;                  // [maxSlots] tensor-core timeout word of the slot's request
    int* hostFlags = nullptr;                 // pinned mirror
    std::vector<int> freeSlots;
    cudaStream_t streams[SERVE_STREAMS];
    cudaStream_t smallStream;
    int nextStream = 0;
    int64_t nextId = 1;
    std::deque<int64_t> queue;                // submitted, not yet admitted
    std::vector<int64_t> pendingSmall;        // admitted small requests awaiting the next batch launch
    std::map<int64_t, Request> reqs;
    std::vector<Batch> batches;
    int64_t numFinished = 0;
};

namespace {

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

bool arena_alloc(qg_server* s, size_t bytes, size_t* off) {
    for (auto it = s->freeList.begin(); it != s->freeList.end(); ++it) {
        if (it->second >= bytes) {
            *off = it->first;
            size_t rest = it->second - bytes;
            size_t newOff = it->first + bytes;
            s->freeList.erase(it);
            if (rest) s->freeList[newOff] = rest;
            s->inUse += bytes;
            return true;
        }
    }
    return false;
}

void arena_free(qg_server* s, size_t off, size_t bytes) {
    s->inUse -= bytes;
    auto it = s->freeList.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != s->freeList.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        s->freeList.erase(nx);
    }
    if (it != s->freeList.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            s->freeList.erase(it);
        }
    }
}

size_t small_smem_bytes(int nq) { return 8192 + ((size_t)8 << nq); }

// The server's copy of a circuit lives in the request's arena region, which is freed when
// the request finishes: forget it, so a later standalone apply uploads a copy of its own.
void release_transient_copy(qg_circuit* c) {
    c->devInfo = nullptr;
    c->devF32 = nullptr;
    c->devTC = nullptr;
    c->uploaded = false;
    c->ownsDevice = false;
}

size_t state_bytes(const Request& r) {
    return r.small ? 0 : round_up((size_t)8 << r.nq, 256) + red_scratch_bytes(red_grid((qidx)1 << r.nq), SERVE_RESULT_DOUBLES);
}

int launch_large(qg_server* s, Request& r) {
    cudaStream_t st = s->streams[r.stream];
    QG_TRY(qg_circuit_upload_to(r.circ, s->arena + r.arenaOff + state_bytes(r), st));
    float2* amps = (float2*)(s->arena + r.arenaOff);
    qidx n = (qidx)1 << r.nq;
    QG_TRY(qg_sv32_initClassicalState(amps, r.nq, 0, st));
    int* flag = s->devFlags + r.slot;
    QG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    QG_TRY(qg_sv32_apply_circuit_flag(r.circ, amps, r.nq, s->impl, st, flag));
    release_transient_copy(r.circ);
    // expectation values into the request's own reduction scratch, then its result slot
    char* scratch = s->arena + r.arenaOff + round_up((size_t)8 << r.nq, 256);
    int grid = red_grid(n);
    RedOut ro;
    ro.ticket = (unsigned int*)scratch;
    ro.result = s->devResults + (size_t)r.slot * SERVE_RESULT_DOUBLES;
    ro.partials = (double*)(scratch + 256);
    QG_CUDA(cudaMemsetAsync(scratch, 0, 256, st));
    ExpecMasks m;
    for (int k = 0; k < SERVE_MAX_STRINGS; k++) {
        m.xy[k] = k < r.numStrings ? r.xy[k] : 0;
        m.yz[k] = k < r.numStrings ? r.yz[k] : 0;
    }
    k_serve_expec<<<grid, RED_THREADS, 0, st>>>(amps, n, m, r.numStrings, ro);
    qg_note_launch();
    QG_TRY(qg_check_launch("k_serve_expec"));
    QG_CUDA(cudaMemcpyAsync(s->hostResults + (size_t)r.slot * SERVE_RESULT_DOUBLES, ro.result,
                            sizeof(double) * SERVE_RESULT_DOUBLES, cudaMemcpyDeviceToHost, st));
    QG_CUDA(cudaMemcpyAsync(s->hostFlags + r.slot, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    QG_CUDA(cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming));
    QG_CUDA(cudaEventRecord(r.done, st));
    return QG_OK;
}

int launch_small_batch(qg_server* s) {
    if (s->pendingSmall.empty()) return QG_OK;
    // one launch per shared-memory size bucket, so tiny registers are not limited by the largest
    std::vector<int64_t> ids = s->pendingSmall;
    s->pendingSmall.clear();
    std::sort(ids.begin(), ids.end(), [&](int64_t a, int64_t b) { return s->reqs[a].nq < s->reqs[b].nq; });
    std::vector<SmallJob> jobs(ids.size());
    for (size_t i = 0; i < ids.size(); i++) {
        Request& r = s->reqs[ids[i]];
        QG_TRY(qg_circuit_upload_to(r.circ, s->arena + r.arenaOff, s->smallStream));
        SmallJob& j = jobs[i];
        j.info = r.circ->devInfo;
        j.mats = r.circ->devF32;
        j.numBlocks = (int)r.circ->blocks.size();
        j.nq = r.nq;
        j.numStrings = r.numStrings;
        j.pad = 0;
        for (int k = 0; k < SERVE_MAX_STRINGS; k++) {
            j.xy[k] = k < r.numStrings ? r.xy[k] : 0;
            j.yz[k] = k < r.numStrings ? r.yz[k] : 0;
        }
        j.out = s->devResults + (size_t)r.slot * SERVE_RESULT_DOUBLES;
        j.stateOut = nullptr;
        release_transient_copy(r.circ);
    }
    Batch b;
    b.ids = ids;
    QG_CUDA(cudaMallocAsync((void**)&b.devJobs, sizeof(SmallJob) * jobs.size(), s->smallStream));
    QG_CUDA(cudaMemcpyAsync(b.devJobs, jobs.data(), sizeof(SmallJob) * jobs.size(), cudaMemcpyHostToDevice, s->smallStream));
    size_t i0 = 0;
    while (i0 < ids.size()) {
        int nq = s->reqs[ids[i0]].nq;
        int bucketMax = nq <= 10 ? 10 : nq;       // <=10 qubits share one launch
        size_t i1 = i0;
        while (i1 < ids.size() && s->reqs[ids[i1]].nq <= bucketMax) i1++;
        size_t smem = small_smem_bytes(bucketMax);
        if (smem > 48 * 1024)
            QG_CUDA(cudaFuncSetAttribute(k_serve_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem_bytes(SERVE_SMALL_MAX_QUBITS)));
        k_serve_small<<<(unsigned)(i1 - i0), SERVE_SMALL_THREADS, smem, s->smallStream>>>(b.devJobs + i0);
        qg_note_launch();
        QG_TRY(qg_check_launch("k_serve_small"));
        i0 = i1;
    }
    for (int64_t id : ids) {
        Request& r = s->reqs[id];
        QG_CUDA(cudaMemcpyAsync(s->hostResults + (size_t)r.slot * SERVE_RESULT_DOUBLES,
                                s->devResults + (size_t)r.slot * SERVE_RESULT_DOUBLES,
                                sizeof(double) * SERVE_RESULT_DOUBLES, cudaMemcpyDeviceToHost, s->smallStream));
    }
    QG_CUDA(cudaFreeAsync(b.devJobs, s->smallStream));
    QG_CUDA(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming));
    QG_CUDA(cudaEventRecord(b.done, s->smallStream));
    s->batches.push_back(b);
    return QG_OK;
}

void finish(qg_server* s, Request& r) {
    const double* h = s->hostResults + (size_t)r.slot * SERVE_RESULT_DOUBLES;
    // small requests run in shared memory without tensor-core launches: no timeout word
    r.timedOut = !r.small && s->hostFlags[r.slot] != 0;
    r.values.resize(r.numStrings);
    // A unitary circuit keeps the norm of |0>, so values are divided by the FP64 norm of
    // the final FP32 state: this removes the drift of the FP32 products to first order.
    double scale = r.unitary ? 1.0 / h[2 * SERVE_MAX_STRINGS] : 1.0;
    for (int k = 0; k < r.numStrings; k++) {
        double re = h[2 * k], im = h[2 * k + 1];
        times_power_of_i(&re, &im, r.ny[k]);
        r.values[k] = re * scale;
    }
    r.finished = true;
    s->freeSlots.push_back(r.slot);
    arena_free(s, r.arenaOff, r.arenaBytes);
    s->numFinished++;
}

}  // namespace

extern "C" {

int qg_server_create(qg_server** out, int64_t hbmBudgetBytes, int maxInFlight, int impl) {
    if (!out || hbmBudgetBytes < (1 << 20) || maxInFlight < 1) return qg_fail(QG_ERR_ARG, "bad server arguments");
    if (impl < 0 || impl > 3) return qg_fail(QG_ERR_ARG, "unknown block kernel choice %d", impl);
    qg_server* s = new qg_server();
    s->impl = impl;
    s->maxSlots = maxInFlight;
    s->arenaBytes = (size_t)hbmBudgetBytes;
    cudaError_t e = cudaMalloc(&s->arena, s->arenaBytes);
    if (e != cudaSuccess) {
        delete s;
        return qg_check_cuda(e, "cudaMalloc(server arena)");
    }
    s->freeList[0] = s->arenaBytes;
    QG_CUDA(cudaMalloc(&s->devResults, sizeof(double) * SERVE_RESULT_DOUBLES * maxInFlight));
    QG_CUDA(cudaMallocHost(&s->hostResults, sizeof(double) * SERVE_RESULT_DOUBLES * maxInFlight));
    QG_CUDA(cudaMalloc(&s->devFlags, sizeof(int) * maxInFlight));
    QG_CUDA(cudaMallocHost(&s->hostFlags, sizeof(int) * maxInFlight));
    for (int i = 0; i < maxInFlight; i++) s->hostFlags[i] = 0;
    for (int i = maxInFlight - 1; i >= 0; i--) s->freeSlots.push_back(i);
    for (int i = 0; i < SERVE_STREAMS; i++) QG_CUDA(cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking));
    QG_CUDA(cudaStreamCreateWithFlags(&s->smallStream, cudaStreamNonBlocking));
    *out = s;
    return QG_OK;
}

int qg_server_destroy(qg_server* s) {
    if (!s) return QG_OK;
    cudaDeviceSynchronize();
    for (auto& kv : s->reqs) if (kv.second.done) cudaEventDestroy(kv.second.done);
    for (auto& b : s->batches) cudaEventDestroy(b.done);
    for (int i = 0; i < SERVE_STREAMS; i++) cudaStreamDestroy(s->streams[i]);
    cudaStreamDestroy(s->smallStream);
    cudaFree(s->arena);
    cudaFree(s->devResults);
    cudaFreeHost(s->hostResults);
    cudaFree(s->devFlags);
    cudaFreeHost(s->hostFlags);
    delete s;
    return QG_OK;
}

int qg_server_submit(qg_server* s, qg_circuit* c, const int64_t* masksXY, const int64_t* masksYZ, const int* numsY,
                     int numStrings, int64_t* id) {
    if (!s || !c || !id) return qg_fail(QG_ERR_ARG, "null argument");
    if (numStrings < 0 || numStrings > SERVE_MAX_STRINGS) return qg_fail(QG_ERR_ARG, "at most %d Pauli strings per request", SERVE_MAX_STRINGS);
    if (c->blocks.empty() && !c->gates.empty()) return qg_fail(QG_ERR_ARG, "the circuit is not fused");
    qidx lim = ((qidx)1 << c->numQubits) - 1;
    for (int k = 0; k < numStrings; k++)
        if ((masksXY[k] & ~lim) || (masksYZ[k] & ~lim)) return qg_fail(QG_ERR_ARG, "Pauli string beyond the register");
    Request r;
    r.nq = c->numQubits;
    r.small = r.nq <= SERVE_SMALL_MAX_QUBITS;
    size_t need = state_bytes(r) + round_up(qg_circuit_device_bytes(c), 256);
    if (need > s->arenaBytes)
        return qg_fail(QG_ERR_ARG, "a %d-qubit request needs %zu bytes, above the server's budget", c->numQubits, need);
    r.id = s->nextId++;
    r.circ = c;
    r.numStrings = numStrings;
    r.unitary = c->allUnitary;
    for (int k = 0; k < numStrings; k++) { r.xy[k] = masksXY[k]; r.yz[k] = masksYZ[k]; r.ny[k] = numsY[k]; }
    r.arenaBytes = need;
    s->reqs[r.id] = r;
    s->queue.push_back(r.id);
    *id = r.id;
    return QG_OK;
}

int qg_server_poll(qg_server* s, int* numDone) {
    if (!s) return qg_fail(QG_ERR_ARG, "null server");
    int done = 0;
    // retire finished work
    std::vector<int64_t> dropped;    // cancelled requests that completed: nobody reads them
    for (auto it = s->batches.begin(); it != s->batches.end();) {
        cudaError_t q = cudaEventQuery(it->done);
        if (q == cudaSuccess) {
            for (int64_t id : it->ids) {
                Request& r = s->reqs[id];
                finish(s, r);
                if (r.cancelled) dropped.push_back(id);
                else done++;
            }
            cudaEventDestroy(it->done);
            it = s->batches.erase(it);
        } else if (q == cudaErrorNotReady) {
            ++it;
        } else {
            return qg_check_cuda(q, "cudaEventQuery(small batch)");
        }
    }
    for (auto& kv : s->reqs) {
        Request& r = kv.second;
        if (r.small || r.finished || !r.done) continue;
        cudaError_t q = cudaEventQuery(r.done);
        if (q == cudaSuccess) {
            cudaEventDestroy(r.done);
            r.done = nullptr;
            finish(s, r);
            if (r.cancelled) dropped.push_back(r.id);
            else done++;
        } else if (q != cudaErrorNotReady) {
            return qg_check_cuda(q, "cudaEventQuery(request)");
        }
    }
    for (int64_t id : dropped) s->reqs.erase(id);
    // admit in arrival order while slots and memory allow (a large request that does not
    // fit yet blocks the queue, so admission stays first-come first-served)
    while (!s->queue.empty() && !s->freeSlots.empty()) {
        Request& r = s->reqs[s->queue.front()];
        size_t off;
        if (!arena_alloc(s, r.arenaBytes, &off)) break;
        r.arenaOff = off;
        r.slot = s->freeSlots.back();
        s->freeSlots.pop_back();
        s->queue.pop_front();
        if (r.small) {
            s->pendingSmall.push_back(r.id);
        } else {
            r.stream = s->nextStream;
            s->nextStream = (s->nextStream + 1) % SERVE_STREAMS;
            QG_TRY(launch_large(s, r));
        }
    }
    QG_TRY(launch_small_batch(s));
    if (numDone) *numDone = done;
    return QG_OK;
}

int qg_server_result(qg_server* s, int64_t id, double* values, int* done) {
    if (!s || !done) return qg_fail(QG_ERR_ARG, "null argument");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return qg_fail(QG_ERR_ARG, "unknown request %lld", (long long)id);
    *done = it->second.finished ? 1 : 0;
    if (it->second.finished && it->second.timedOut)
        return qg_fail(QG_ERR_TIMEOUT, "request %lld failed: a tensor-core block launch gave up a bounded wait", (long long)id);
    if (it->second.finished && values)
        for (int k = 0; k < it->second.numStrings; k++) values[k] = it->second.values[k];
    return QG_OK;
}

int qg_server_release(qg_server* s, int64_t id) {
    if (!s) return qg_fail(QG_ERR_ARG, "null server");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second.finished) return qg_fail(QG_ERR_ARG, "request %lld is not finished", (long long)id);
    s->reqs.erase(it);
    return QG_OK;
}

int qg_server_cancel(qg_server* s, int64_t id) {
    if (!s) return qg_fail(QG_ERR_ARG, "null server");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second.cancelled) return qg_fail(QG_ERR_ARG, "unknown request %lld", (long long)id);
    Request& r = it->second;
    if (r.finished) {                        // done already: same as releasing it
        s->reqs.erase(it);
        return QG_OK;
    }
    if (r.slot < 0) {                        // still queued: nothing on the GPU
        for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
            if (*q == id) { s->queue.erase(q); break; }
        s->reqs.erase(it);
        return QG_OK;
    }
    r.cancelled = true;                      // in flight: its slot and memory return when it completes
    return QG_OK;
}

int qg_server_stats(qg_server* s, int64_t* queued, int64_t* inFlight, int64_t* hbmInUse, int64_t* finished) {
    if (!s) return qg_fail(QG_ERR_ARG, "null server");
    int64_t flight = 0;
    for (auto& kv : s->reqs)
        if (!kv.second.finished && kv.second.slot >= 0) flight++;
    if (queued) *queued = (int64_t)s->queue.size();
    if (inFlight) *inFlight = flight;
    if (hbmInUse) *hbmInUse = (int64_t)s->inUse;
    if (finished) *finished = s->numFinished;
    return QG_OK;
}

}  // extern "C"
