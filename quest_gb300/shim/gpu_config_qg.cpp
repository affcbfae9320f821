// Drop-in replacement for QuEST v4.1.0's quest/src/gpu/gpu_config.cpp on one
// GB300: keeps every signature of quest/src/gpu/gpu_config.hpp and forwards to
// the runtime entry points of include/quest_gb300.h (device binding, allocation,
// copies, synchronisation, the scratch cache).  cuQuantum hooks are no-ops: the
// backend never uses cuStateVec.
#include "quest/include/modes.h"
#include "quest/include/types.h"
#include "quest/include/qureg.h"
#include "quest/include/matrices.h"
#include "quest/include/channels.h"

#include "quest/src/core/errors.hpp"
#include "quest/src/gpu/gpu_config.hpp"

#include "quest_gb300.h"

namespace {
inline void ok(int rc, const char* caller) {
    if (rc != QG_OK) error_cudaCallFailed(qg_get_last_error(), "qg_*", caller, __FILE__, __LINE__);
}
int g_device = 0;
}  // namespace

bool gpu_isGpuCompiled() { return true; }
bool gpu_isCuQuantumCompiled() { return false; }
bool gpu_isGpuAvailable() { int n = 0; qg_get_num_devices(&n); return n > 0; }
bool gpu_isDirectGpuCommPossible() { return false; }
int gpu_getNumberOfLocalGpus() { int n = 0; qg_get_num_devices(&n); return n; }
int gpu_getComputeCapability() { int a = 0, b = 0; ok(qg_get_device_info(nullptr, nullptr, nullptr, &a, &b), __func__); return 10 * a + b; }
size_t gpu_getCurrentAvailableMemoryInBytes() { int64_t f = 0; ok(qg_get_device_info(nullptr, nullptr, &f, nullptr, nullptr), __func__); return (size_t)f; }
size_t gpu_getTotalMemoryInBytes() { int64_t t = 0; ok(qg_get_device_info(nullptr, &t, nullptr, nullptr, nullptr), __func__); return (size_t)t; }
bool gpu_doesGpuSupportMemPools() { return true; }
qindex gpu_getMaxNumConcurrentThreads() { int sms = 0; ok(qg_get_device_info(&sms, nullptr, nullptr, nullptr, nullptr), __func__); return (qindex)sms * 2048; }

void gpu_bindLocalGPUsToNodes() { ok(qg_init(g_device), __func__); }
bool gpu_areAnyNodesBoundToSameGpu() { return false; }
void gpu_sync() { ok(qg_sync(), __func__); }
void gpu_initCuQuantum() {}
void gpu_finalizeCuQuantum() {}

// gpu_allocArray returns nullptr on failure, which validation reports (gpu_config.cpp:399-421)
qcomp* gpu_allocArray(qindex numLocalAmps) {
    void* p = nullptr;
    if (qg_alloc(&p, (int64_t)(numLocalAmps * sizeof(qcomp))) != QG_OK) return nullptr;
    return (qcomp*)p;
}
void gpu_deallocArray(qcomp* amps) { ok(qg_free(amps), __func__); }

void gpu_copyArray(qcomp* dest, qcomp* src, qindex dim) {
    ok(qg_copy_d2d(dest, src, (int64_t)(dim * sizeof(qcomp)), nullptr), __func__);
    ok(qg_sync(), __func__);
}
void gpu_copyCpuToGpu(qcomp* cpuArr, qcomp* gpuArr, qindex n) { ok(qg_copy_h2d(gpuArr, cpuArr, (int64_t)(n * sizeof(qcomp)), nullptr), __func__); ok(qg_sync(), __func__); }
void gpu_copyGpuToCpu(qcomp* gpuArr, qcomp* cpuArr, qindex n) { ok(qg_copy_d2h(cpuArr, gpuArr, (int64_t)(n * sizeof(qcomp)), nullptr), __func__); }
void gpu_copyGpuToCpu(Qureg, qcomp* gpuArr, qcomp* cpuArr, qindex n) { gpu_copyGpuToCpu(gpuArr, cpuArr, n); }
void gpu_copyGpuToCpu(Qureg q) { gpu_copyGpuToCpu(q.gpuAmps, q.cpuAmps, q.numAmpsPerNode); }
void gpu_copyCpuToGpu(Qureg, qcomp* cpuArr, qcomp* gpuArr, qindex n) { gpu_copyCpuToGpu(cpuArr, gpuArr, n); }
void gpu_copyCpuToGpu(Qureg q) { gpu_copyCpuToGpu(q.cpuAmps, q.gpuAmps, q.numAmpsPerNode); }

// Heap matrices: the backend reads dense and diagonal elements from the host copy at
// each call (small matrices travel as kernel parameters), so the device copies that
// QuEST keeps in sync are filled only when QuEST allocated them.
void gpu_copyCpuToGpu(CompMatr m) { if (m.gpuElemsFlat) gpu_copyCpuToGpu(m.cpuElemsFlat, m.gpuElemsFlat, m.numRows * m.numRows); }
void gpu_copyGpuToCpu(CompMatr m) { if (m.gpuElemsFlat) gpu_copyGpuToCpu(m.gpuElemsFlat, m.cpuElemsFlat, m.numRows * m.numRows); }
void gpu_copyCpuToGpu(DiagMatr m) { if (m.gpuElems) gpu_copyCpuToGpu(m.cpuElems, m.gpuElems, m.numElems); }
void gpu_copyGpuToCpu(DiagMatr m) { if (m.gpuElems) gpu_copyGpuToCpu(m.gpuElems, m.cpuElems, m.numElems); }
void gpu_copyCpuToGpu(SuperOp op) { if (op.gpuElemsFlat) gpu_copyCpuToGpu(op.cpuElemsFlat, op.gpuElemsFlat, op.numRows * op.numRows); }
void gpu_copyGpuToCpu(SuperOp op) { if (op.gpuElemsFlat) gpu_copyGpuToCpu(op.gpuElemsFlat, op.cpuElemsFlat, op.numRows * op.numRows); }
void gpu_copyCpuToGpu(FullStateDiagMatr m) { if (m.gpuElems) gpu_copyCpuToGpu(m.cpuElems, m.gpuElems, m.numElemsPerNode); }

// the backend manages its own scratch; QuEST's many-target cache is never needed
qcomp* gpu_getCacheOfSize(qindex, qindex) { return nullptr; }
void gpu_clearCache() { ok(qg_clear_cache(), __func__); }
size_t gpu_getCacheMemoryInBytes() { int64_t b = 0; qg_get_cache_size(&b); return (size_t)b; }
