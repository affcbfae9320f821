// The compiled-circuit object shared by the fused-block path and the server.
#pragma once

#include "qg_common.cuh"

#include <complex>
#include <vector>

typedef std::complex<double> cd;

// per block, as the device-side runners read it
struct QgBlockInfo {
    int k;          // targets (1..5)
    int t[5];       // ascending target qubits
    int off32;      // offset (in float2) of the block's FP32 matrix in qg_circuit::devF32
    int pad;
};

struct QgGate {
    std::vector<int> targs;   // matrix index bit i <-> targs[i]
    std::vector<cd> m;        // row-major 2^k x 2^k
};

struct QgBlock {
    std::vector<int> targs;   // ascending
    std::vector<cd> m;        // row-major, index bit i <-> targs[i]
    size_t off32 = 0;         // offset (in float2) of the FP32 matrix in devF32
    size_t offTC = 0;         // offset (in floats) of the tensor-core operand pair in devTC (k == 5 only)
};

struct qg_circuit {
    int numQubits = 0;
    std::vector<QgGate> gates;
    std::vector<QgBlock> blocks;
    int fusedK = 0;
    float2* devF32 = nullptr;   // concatenated FP32 block matrices
    float* devTC = nullptr;     // per k=5 block: Bhi, Blo (64x64 real each) in tensor-core layout
    size_t tcFloats = 0;
    QgBlockInfo* devInfo = nullptr;   // per-block k, targets and matrix offset (start of the device copy)
    bool uploaded = false;      // block matrices are copied to the device at the first apply
    bool ownsDevice = false;    // the device copy was allocated here (else it lives in a caller's arena)
    bool allUnitary = true;     // every gate satisfies max|U^dagger U - I| <= 1e-10
    int preferredImpl = 0;      // set by qg_circuit_autotune: the kernel an automatic apply uses
};

// bytes of the device copy of the fused blocks (descriptors, FP32 matrices, tensor-core operands)
size_t qg_circuit_device_bytes(qg_circuit* c);
// writes that copy into caller-owned device memory `dev`, copying on `stream`
int qg_circuit_upload_to(qg_circuit* c, char* dev, cudaStream_t stream);
// allocates the device copy and uploads it (synchronises `stream`)
int qg_circuit_upload(qg_circuit* c, cudaStream_t stream);

