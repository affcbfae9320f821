// Runtime services of the backend: device binding, allocation, copies, error
// reporting and the library-owned scratch cache.  Replaces the role of QuEST's
// quest/src/gpu/gpu_config.cpp for the gate path (allocation gpu_config.cpp:399-436,
// copies :449-633, sync :382-390, the scratch cache :639-669).
#include "qg_common.cuh"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <vector>

namespace {
thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};
std::atomic<int> g_fp64_products{QG_FP64_PRODUCTS_FIXED};

struct DeviceCache {
    void* scratch = nullptr;
    size_t scratchBytes = 0;
    void* pinned = nullptr;
    size_t pinnedBytes = 0;
    int numSMs = 0;
};
std::mutex g_cache_mutex;
std::vector<DeviceCache> g_caches;

DeviceCache& cache_for_current() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_cache_mutex);
    if ((int)g_caches.size() <= dev) g_caches.resize(dev + 1);
    return g_caches[dev];
}
}  // namespace

void qg_set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int qg_fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int qg_check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return QG_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return qg_fail(QG_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    }
    return qg_fail(QG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int qg_check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return qg_fail(QG_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    return QG_OK;
}

void qg_note_launch(int n) { g_launches += n; }
int qg_fp64_products_mode() { return g_fp64_products.load(); }

int qg_num_sms() {
    DeviceCache& c = cache_for_current();
    if (c.numSMs == 0) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        c.numSMs = n > 0 ? n : 1;
    }
    return c.numSMs;
}

int qg_scratch_get(void** out, size_t bytes) {
    DeviceCache& c = cache_for_current();
    if (c.scratchBytes < bytes) {
        if (c.scratch) {
            // the old cache may still be read by queued kernels on any stream
            QG_CUDA(cudaDeviceSynchronize());
            QG_CUDA(cudaFree(c.scratch));
            c.scratch = nullptr;
            c.scratchBytes = 0;
        }
        size_t want = std::max(bytes, (size_t)1 << 20);
        QG_CUDA(cudaMalloc(&c.scratch, want));
        QG_CUDA(cudaMemset(c.scratch, 0, want));
        c.scratchBytes = want;
    }
    *out = c.scratch;
    return QG_OK;
}

int qg_pinned_result(void** out, size_t bytes) {
    DeviceCache& c = cache_for_current();
    if (c.pinnedBytes < bytes) {
        if (c.pinned) QG_CUDA(cudaFreeHost(c.pinned));
        c.pinned = nullptr;
        size_t want = std::max(bytes, (size_t)4096);
        QG_CUDA(cudaMallocHost(&c.pinned, want));
        c.pinnedBytes = want;
    }
    *out = c.pinned;
    return QG_OK;
}

int qg_check_qubits(int numQubits, const int* qubits, int num, const char* what) {
    if (num < 0) return qg_fail(QG_ERR_ARG, "%s: negative count", what);
    if (num > 0 && qubits == nullptr) return qg_fail(QG_ERR_ARG, "%s: null qubit list", what);
    unsigned long long seen = 0;
    for (int i = 0; i < num; i++) {
        int q = qubits[i];
        if (q < 0 || q >= numQubits) return qg_fail(QG_ERR_ARG, "%s: qubit %d is outside [0, %d)", what, q, numQubits);
        if (seen & (1ULL << q)) return qg_fail(QG_ERR_ARG, "%s: qubit %d appears twice", what, q);
        seen |= 1ULL << q;
    }
    return QG_OK;
}

int qg_check_amps(const void* amps, int numQubits) {
    if (amps == nullptr) return qg_fail(QG_ERR_ARG, "null amplitude pointer");
    if (numQubits < 1 || numQubits > QG_MAX_QUBITS) return qg_fail(QG_ERR_ARG, "numQubits %d outside [1, %d]", numQubits, QG_MAX_QUBITS);
    if (((uintptr_t)amps) & 15) return qg_fail(QG_ERR_ARG, "amplitude pointer is not 16-byte aligned");
    return QG_OK;
}

int qg_make_plan(int numQubits, const int* ctrls, const int* ctrlStates, int numCtrls,
                 const int* extraQubits, const int* extraValues, int numExtra, QubitPlan* plan) {
    int all[64];
    int n = numCtrls + numExtra;
    if (n > QG_MAX_INSERT) return qg_fail(QG_ERR_NOTSUP, "%d controls+targets exceed the supported %d", n, QG_MAX_INSERT);
    if (n > numQubits) return qg_fail(QG_ERR_ARG, "%d controls+targets exceed %d qubits", n, numQubits);
    plan->stateMask = 0;
    for (int i = 0; i < numCtrls; i++) {
        all[i] = ctrls[i];
        int st = ctrlStates ? ctrlStates[i] : 1;
        if (st != 0 && st != 1) return qg_fail(QG_ERR_ARG, "control state %d is not 0 or 1", st);
        if (st) plan->stateMask |= (qidx)1 << ctrls[i];
    }
    for (int i = 0; i < numExtra; i++) {
        all[numCtrls + i] = extraQubits[i];
        if (extraValues && extraValues[i]) plan->stateMask |= (qidx)1 << extraQubits[i];
    }
    QG_TRY(qg_check_qubits(numQubits, all, n, "controls/targets"));
    std::sort(all, all + n);
    plan->ins.num = n;
    for (int i = 0; i < n; i++) plan->ins.low[i] = ((qidx)1 << all[i]) - 1;
    plan->numFixed = n;
    return QG_OK;
}

extern "C" {

const char* qg_get_last_error(void) { return g_last_error.c_str(); }

const char* qg_get_error_string(int code) {
    switch (code) {
        case QG_OK: return "success";
        case QG_ERR_CUDA: return "CUDA runtime error";
        case QG_ERR_ARG: return "invalid argument";
        case QG_ERR_OOM: return "device allocation failed";
        case QG_ERR_TIMEOUT: return "device-side wait timed out";
        case QG_ERR_NOTSUP: return "not supported";
        default: return "unknown error";
    }
}

int qg_get_version(void) { return 100; }

namespace {
// the context's L2 fetch-granularity limit as qg_init found it, per device (-1: not saved)
const int L2_MAX_DEVICES = 64;
int g_l2Saved[L2_MAX_DEVICES] = {};
bool g_l2SavedInit = false;
std::mutex g_l2mu;
}  // namespace

int qg_init(int device) {
    int n = 0;
    QG_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return qg_fail(QG_ERR_ARG, "device %d outside [0, %d)", device, n);
    QG_CUDA(cudaSetDevice(device));
    QG_CUDA(cudaFree(0));  // create the primary context now
    qg_num_sms();
    // L2 fetches of 32 bytes: gates that visit every other 16-, 32- or 64-byte run (a
    // controlled phase on qubits 1 or 2) otherwise pull whole 64- or 128-byte units for
    // half their bytes.  Measured on GB300 at 28 qubits: 0.553 -> 0.372 ms for such a
    // phase, streaming kernels unchanged.  The limit belongs to the primary context, which
    // every library of the process shares, and lasts until the process exits; the value
    // found here is kept so that qg_restore_l2_fetch_granularity can put it back.
    {
        std::lock_guard<std::mutex> lock(g_l2mu);
        if (!g_l2SavedInit) {
            for (int i = 0; i < L2_MAX_DEVICES; i++) g_l2Saved[i] = -1;
            g_l2SavedInit = true;
        }
        if (device < L2_MAX_DEVICES && g_l2Saved[device] < 0) {
            size_t v = 0;
            QG_CUDA(cudaDeviceGetLimit(&v, cudaLimitMaxL2FetchGranularity));
            g_l2Saved[device] = (int)v;
        }
    }
    return qg_set_l2_fetch_granularity(32);
}

int qg_set_l2_fetch_granularity(int bytes) {
    if (bytes != 0 && bytes != 32 && bytes != 64 && bytes != 128)
        return qg_fail(QG_ERR_ARG, "L2 fetch granularity %d: use 0, 32, 64 or 128", bytes);
    QG_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes));
    return QG_OK;
}

int qg_restore_l2_fetch_granularity(void) {
    int dev = 0;
    QG_CUDA(cudaGetDevice(&dev));
    int v = -1;
    {
        std::lock_guard<std::mutex> lock(g_l2mu);
        if (g_l2SavedInit && dev < L2_MAX_DEVICES) v = g_l2Saved[dev];
    }
    if (v < 0) return QG_OK;    // qg_init never changed this device's limit
    QG_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)v));
    return QG_OK;
}

int qg_get_l2_fetch_granularity(int* bytes) {
    if (!bytes) return qg_fail(QG_ERR_ARG, "null output");
    size_t v = 0;
    QG_CUDA(cudaDeviceGetLimit(&v, cudaLimitMaxL2FetchGranularity));
    *bytes = (int)v;
    return QG_OK;
}

int qg_get_num_devices(int* out) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *out = n;
    return QG_OK;
}

int qg_get_device_info(int* numSMs, int64_t* totalMem, int64_t* freeMem, int* ccMajor, int* ccMinor) {
    int dev = 0;
    QG_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp p;
    QG_CUDA(cudaGetDeviceProperties(&p, dev));
    size_t fr = 0, tot = 0;
    QG_CUDA(cudaMemGetInfo(&fr, &tot));
    if (numSMs) *numSMs = p.multiProcessorCount;
    if (totalMem) *totalMem = (int64_t)tot;
    if (freeMem) *freeMem = (int64_t)fr;
    if (ccMajor) *ccMajor = p.major;
    if (ccMinor) *ccMinor = p.minor;
    return QG_OK;
}

int qg_alloc(void** out, int64_t numBytes) {
    if (!out) return qg_fail(QG_ERR_ARG, "null output pointer");
    *out = nullptr;
    if (numBytes <= 0) return qg_fail(QG_ERR_ARG, "allocation of %lld bytes", (long long)numBytes);
    cudaError_t e = cudaMalloc(out, (size_t)numBytes);
    if (e != cudaSuccess) {
        *out = nullptr;
        return qg_check_cuda(e, "cudaMalloc");
    }
    return QG_OK;
}

int qg_free(void* ptr) {
    if (ptr) QG_CUDA(cudaFree(ptr));
    return QG_OK;
}

int qg_copy_h2d(void* dst, const void* src, int64_t numBytes, void* stream) {
    if (numBytes < 0 || (numBytes > 0 && (!dst || !src))) return qg_fail(QG_ERR_ARG, "bad copy arguments");
    if (numBytes == 0) return QG_OK;
    QG_CUDA(cudaMemcpyAsync(dst, src, (size_t)numBytes, cudaMemcpyHostToDevice, qg_stream(stream)));
    return QG_OK;
}

int qg_copy_d2h(void* dst, const void* src, int64_t numBytes, void* stream) {
    if (numBytes < 0 || (numBytes > 0 && (!dst || !src))) return qg_fail(QG_ERR_ARG, "bad copy arguments");
    if (numBytes == 0) return QG_OK;
    QG_CUDA(cudaMemcpyAsync(dst, src, (size_t)numBytes, cudaMemcpyDeviceToHost, qg_stream(stream)));
    QG_CUDA(cudaStreamSynchronize(qg_stream(stream)));
    return QG_OK;
}

int qg_copy_d2d(void* dst, const void* src, int64_t numBytes, void* stream) {
    if (numBytes < 0 || (numBytes > 0 && (!dst || !src))) return qg_fail(QG_ERR_ARG, "bad copy arguments");
    if (numBytes == 0) return QG_OK;
    QG_CUDA(cudaMemcpyAsync(dst, src, (size_t)numBytes, cudaMemcpyDeviceToDevice, qg_stream(stream)));
    return QG_OK;
}

int qg_sync(void) {
    QG_CUDA(cudaDeviceSynchronize());
    return QG_OK;
}

int qg_stream_sync(void* stream) {
    QG_CUDA(cudaStreamSynchronize(qg_stream(stream)));
    return QG_OK;
}

int qg_get_cache_size(int64_t* out) {
    DeviceCache& c = cache_for_current();
    *out = (int64_t)c.scratchBytes;
    return QG_OK;
}

int qg_clear_cache(void) {
    DeviceCache& c = cache_for_current();
    if (c.scratch) {
        QG_CUDA(cudaDeviceSynchronize());
        QG_CUDA(cudaFree(c.scratch));
    }
    c.scratch = nullptr;
    c.scratchBytes = 0;
    return QG_OK;
}

int qg_stream_create(void** out) {
    if (!out) return qg_fail(QG_ERR_ARG, "null output");
    cudaStream_t s;
    QG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *out = (void*)s;
    return QG_OK;
}

int qg_stream_destroy(void* stream) {
    if (stream) QG_CUDA(cudaStreamDestroy((cudaStream_t)stream));
    return QG_OK;
}

int qg_stream_wait_event(void* stream, void* ev) {
    if (!ev) return qg_fail(QG_ERR_ARG, "null event");
    QG_CUDA(cudaStreamWaitEvent(qg_stream(stream), (cudaEvent_t)ev, 0));
    return QG_OK;
}

int qg_event_create(void** out) {
    cudaEvent_t e;
    QG_CUDA(cudaEventCreate(&e));
    *out = (void*)e;
    return QG_OK;
}

int qg_event_destroy(void* ev) {
    if (ev) QG_CUDA(cudaEventDestroy((cudaEvent_t)ev));
    return QG_OK;
}

int qg_event_record(void* ev, void* stream) {
    QG_CUDA(cudaEventRecord((cudaEvent_t)ev, qg_stream(stream)));
    return QG_OK;
}

int qg_event_elapsed_ms(void* start, void* stop, float* ms) {
    QG_CUDA(cudaEventSynchronize((cudaEvent_t)stop));
    QG_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop));
    return QG_OK;
}

int qg_get_launch_count(int64_t* out) {
    *out = (int64_t)g_launches.load();
    return QG_OK;
}

int qg_set_fp64_products(int mode) {
    if (mode != QG_FP64_PRODUCTS_FIXED && mode != QG_FP64_PRODUCTS_FP64)
        return qg_fail(QG_ERR_ARG, "FP64 product mode %d is neither 0 (fixed point) nor 1 (FP64)", mode);
    g_fp64_products = mode;
    return QG_OK;
}

int qg_get_fp64_products(int* mode) {
    if (!mode) return qg_fail(QG_ERR_ARG, "null argument");
    *mode = g_fp64_products.load();
    return QG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- FP64 issue-rate probe
// Eight independent FMA chains per thread, enough warps to fill every SM: the
// kernel's FP64 throughput is the rate that bounds the general complex gates.
__global__ void k_fp64_fma_rate(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

extern "C" int qg_measure_fp64_fma_rate(double* fmaPerSecond) {
    int blocks = qg_num_sms() * 8, threads = 256, iters = 1 << 13;
    double* out = nullptr;
    QG_CUDA(cudaMalloc(&out, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1;
    QG_CUDA(cudaEventCreate(&e0));
    QG_CUDA(cudaEventCreate(&e1));
    k_fp64_fma_rate<<<blocks, threads>>>(out, 64, 1.0000001, 1e-9);   // warm-up
    QG_CUDA(cudaEventRecord(e0));
    k_fp64_fma_rate<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    QG_CUDA(cudaEventRecord(e1));
    QG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    QG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    QG_CUDA(cudaFree(out));
    qg_note_launch(2);
    *fmaPerSecond = (double)blocks * threads * iters * 8 / (ms * 1e-3);
    return QG_OK;
}
