// FP32 fused-block path: circuits compiled into dense blocks of up to k qubits
// and applied to FP32 (complex64) statevectors.
//
// The gate path of QuEST applies one kernel per gate.  Here a circuit (a list of
// small dense unitaries) is first fused on the host: gates are greedily merged
// into blocks acting on at most k qubits, each block's 2^k x 2^k matrix is
// formed in FP64 (the product of its gates, in order), and the matrices are
// uploaded once.  Applying a block is the dense-matrix primitive of
// quest/src/gpu/gpu_kernels.cuh:296-356 (anyCtrlFewTargDenseMatr) on FP32
// amplitudes; each pass reads and writes every amplitude once, so a circuit
// costs (number of blocks) passes instead of (number of gates).
//
// Two block kernels: a SIMT kernel (each thread holds one 2^k-amplitude group
// in registers and the matrix is read from shared memory as warp broadcasts),
// and the tensor-core kernel of qg_fused_tc.cu (k = 5, 3xTF32 on tcgen05).
// Norms and expectation values of FP32 states accumulate in FP64.
#include "qg_reduce.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

// ============================================================== circuit object (host)

#include "qg_circuit.cuh"

// tensor-core operand builder, defined in qg_fused_tc.cu
size_t qg_tc_operand_floats();
void qg_tc_build_operands(const std::complex<double>* m32x32, float* out);
int qg_tc_apply_block(float2* amps, int numQubits, const int* targs, const float* devOperands, cudaStream_t st,
                      bool holdOperands = false, int* errorFlag = nullptr);
bool qg_tc_supported(int numQubits);
int qg_tc_prepare();
int qg_tc_take_error();
template <typename AMP>
int qg_pauli_tile_batch(const AMP* amps, int n, const int64_t* mXY, const int64_t* mYZ, const int* numsY, int num,
                        qg_cplx* out, cudaStream_t st);

namespace {

bool is_diagonal(const QgGate& g) {
    size_t GD = (size_t)1 << g.targs.size();
    for (size_t r = 0; r < GD; r++)
        for (size_t c = 0; c < GD; c++)
            if (r != c && g.m[r * GD + c] != cd(0, 0)) return false;
    return true;
}

// M <- G M on the space of `qs` (sorted); G acts on its targets, a subset of qs
void apply_gate_to_columns(std::vector<cd>& M, const std::vector<int>& qs, const QgGate& g) {
    const int m = (int)qs.size();
    const size_t D = (size_t)1 << m;
    const int gk = (int)g.targs.size();
    const size_t GD = (size_t)1 << gk;
    size_t gbit[5], gmask = 0;
    for (int i = 0; i < gk; i++) {
        gbit[i] = (size_t)1 << (std::find(qs.begin(), qs.end(), g.targs[i]) - qs.begin());
        gmask |= gbit[i];
    }
    size_t offs[32];
    for (size_t j = 0; j < GD; j++) {
        size_t o = 0;
        for (int i = 0; i < gk; i++) if ((j >> i) & 1) o |= gbit[i];
        offs[j] = o;
    }
    if (is_diagonal(g)) {
        // a diagonal gate scales whole rows of M
        for (size_t r = 0; r < D; r++) {
            size_t j = 0;
            for (int i = 0; i < gk; i++) if (r & gbit[i]) j |= (size_t)1 << i;
            cd d = g.m[j * GD + j];
            if (d == cd(1, 0)) continue;
            cd* row = &M[r * D];
            for (size_t c = 0; c < D; c++) row[c] *= d;
        }
        return;
    }
    cd in[32];
    for (size_t base = 0; base < D; base++) {
        if (base & gmask) continue;
        for (size_t col = 0; col < D; col++) {
            for (size_t j = 0; j < GD; j++) in[j] = M[(base | offs[j]) * D + col];
            for (size_t r2 = 0; r2 < GD; r2++) {
                cd acc = 0;
                const cd* grow = &g.m[r2 * GD];
                for (size_t j = 0; j < GD; j++) acc += grow[j] * in[j];
                M[(base | offs[r2]) * D + col] = acc;
            }
        }
    }
}

// Runs of one-qubit gates on the same qubit collapse into one 2x2 gate (their product),
// so the block fuser sees fewer, denser gates.
std::vector<QgGate> merge_single_qubit_runs(const std::vector<QgGate>& gates, int numQubits) {
    std::vector<QgGate> out;
    std::vector<int> pending(numQubits, -1);   // index in `out` of an open 1q gate per qubit
    for (const QgGate& g : gates) {
        if (g.targs.size() == 1) {
            int q = g.targs[0];
            if (pending[q] >= 0) {
                QgGate& p = out[pending[q]];
                cd a = g.m[0], b = g.m[1], c = g.m[2], d = g.m[3];
                cd e = p.m[0], f = p.m[1], h = p.m[2], k = p.m[3];
                p.m = {a * e + b * h, a * f + b * k, c * e + d * h, c * f + d * k};   // g * p
            } else {
                pending[q] = (int)out.size();
                out.push_back(g);
            }
            continue;
        }
        for (int q : g.targs) pending[q] = -1;
        out.push_back(g);
    }
    return out;
}

// re-express M (over qs) on the larger sorted set qs2 (M tensor identity)
std::vector<cd> expand(const std::vector<cd>& M, const std::vector<int>& qs, const std::vector<int>& qs2) {
    int m = (int)qs.size(), m2 = (int)qs2.size();
    size_t D = (size_t)1 << m, D2 = (size_t)1 << m2;
    std::vector<int> pos(m);
    for (int i = 0; i < m; i++) pos[i] = (int)(std::find(qs2.begin(), qs2.end(), qs[i]) - qs2.begin());
    size_t inMask = 0;
    for (int i = 0; i < m; i++) inMask |= (size_t)1 << pos[i];
    std::vector<cd> out(D2 * D2, cd(0, 0));
    auto sub = [&](size_t x) { size_t v = 0; for (int i = 0; i < m; i++) if ((x >> pos[i]) & 1) v |= (size_t)1 << i; return v; };
    for (size_t r = 0; r < D2; r++)
        for (size_t c = 0; c < D2; c++) {
            if ((r & ~inMask) != (c & ~inMask)) continue;
            out[r * D2 + c] = M[sub(r) * D + sub(c)];
        }
    return out;
}

struct OpenBlock {
    std::vector<int> qs;   // sorted
    std::vector<cd> m;
    int order;             // creation order, for deterministic emission
};

void absorb(OpenBlock& b, const QgGate& g) {
    std::vector<int> u = b.qs;
    for (int q : g.targs) if (std::find(u.begin(), u.end(), q) == u.end()) u.push_back(q);
    std::sort(u.begin(), u.end());
    if (u != b.qs) {
        b.m = expand(b.m, b.qs, u);
        b.qs = u;
    }
    apply_gate_to_columns(b.m, b.qs, g);
}

OpenBlock block_from(const QgGate& g, int order) {
    OpenBlock b;
    b.qs = g.targs;
    std::sort(b.qs.begin(), b.qs.end());
    size_t D = (size_t)1 << b.qs.size();
    b.m.assign(D * D, cd(0, 0));
    for (size_t i = 0; i < D; i++) b.m[i * D + i] = 1;
    b.order = order;
    apply_gate_to_columns(b.m, b.qs, g);
    return b;
}

void emit(std::vector<QgBlock>& out, OpenBlock& b) {
    QgBlock q;
    q.targs = b.qs;
    q.m = b.m;
    out.push_back(q);
}

}  // namespace

// Greedy fusion.  Open blocks have pairwise disjoint qubits (so they commute).  A
// gate joins the single open block it overlaps if the union still fits in k qubits,
// merges the blocks it overlaps when they fit together, joins the nearest block
// with room when it overlaps none, and otherwise closes what it overlaps and starts
// a new block.  Diagonal gates (CZ, controlled phases, RZ ...) that would force a
// closure are held back instead: a diagonal gate commutes with every diagonal gate
// and with every gate on other qubits, so it may wait until the first non-diagonal
// gate on one of its qubits, which places it first.  Every reordering swaps
// commuting gates, so the product of the emitted blocks equals the circuit.
namespace {

struct Fuser {
    int k;
    std::vector<OpenBlock> open;
    std::vector<QgBlock>& out;
    int order = 0;

    std::vector<int> hits(const QgGate& g) const {
        std::vector<int> hit;
        for (int i = 0; i < (int)open.size(); i++)
            for (int q : g.targs)
                if (std::find(open[i].qs.begin(), open[i].qs.end(), q) != open[i].qs.end()) { hit.push_back(i); break; }
        return hit;
    }

    // places g without closing any block; false if that is impossible
    bool try_place(const QgGate& g) {
        std::vector<int> hit = hits(g);
        std::vector<int> uni = g.targs;
        for (int i : hit)
            for (int q : open[i].qs)
                if (std::find(uni.begin(), uni.end(), q) == uni.end()) uni.push_back(q);
        if (!hit.empty()) {
            if ((int)uni.size() > k) return false;
            // merge every hit block into the first, then absorb the gate
            OpenBlock& b0 = open[hit[0]];
            for (size_t h = 1; h < hit.size(); h++) {
                QgGate as;
                as.targs = open[hit[h]].qs;
                as.m = open[hit[h]].m;
                absorb(b0, as);
            }
            absorb(b0, g);
            for (int h = (int)hit.size() - 1; h >= 1; h--) open.erase(open.begin() + hit[h]);
            return true;
        }
        // join the open block with room whose qubits lie nearest (contiguous windows keep
        // later nearest-neighbour gates inside one block); ties go to the larger block
        int best = -1, bestDist = 1 << 30;
        for (int i = 0; i < (int)open.size(); i++) {
            if ((int)(open[i].qs.size() + g.targs.size()) > k) continue;
            int dist = 1 << 30;
            for (int a : open[i].qs)
                for (int b : g.targs) dist = std::min(dist, std::abs(a - b));
            if (best < 0 || dist < bestDist || (dist == bestDist && open[i].qs.size() > open[best].qs.size())) {
                best = i;
                bestDist = dist;
            }
        }
        if (best >= 0) absorb(open[best], g);
        else open.push_back(block_from(g, order++));
        return true;
    }

    // places g, closing the blocks it overlaps (in creation order) if it must
    void place(const QgGate& g) {
        if (try_place(g)) return;
        std::vector<int> hit = hits(g);
        std::sort(hit.begin(), hit.end(), [&](int a, int b) { return open[a].order < open[b].order; });
        for (int i : hit) emit(out, open[i]);
        std::sort(hit.begin(), hit.end());
        for (int h = (int)hit.size() - 1; h >= 0; h--) open.erase(open.begin() + hit[h]);
        open.push_back(block_from(g, order++));
    }
};

bool shares_qubit(const QgGate& a, const QgGate& b) {
    for (int q : a.targs)
        if (std::find(b.targs.begin(), b.targs.end(), q) != b.targs.end()) return true;
    return false;
}

}  // namespace

static void fuse_gates(const std::vector<QgGate>& gatesIn, int numQubits, int k, std::vector<QgBlock>& out) {
    const std::vector<QgGate> gates = merge_single_qubit_runs(gatesIn, numQubits);
    Fuser f{k, {}, out};
    std::vector<QgGate> pending;   // diagonal gates held back
    for (const QgGate& g : gates) {
        const bool diag = is_diagonal(g);
        if (!diag) {
            for (size_t i = 0; i < pending.size();) {
                if (shares_qubit(pending[i], g)) {
                    f.place(pending[i]);
                    pending.erase(pending.begin() + i);
                } else {
                    i++;
                }
            }
            f.place(g);
            continue;
        }
        if (!f.try_place(g)) pending.push_back(g);
    }
    for (const QgGate& p : pending) f.place(p);
    std::sort(f.open.begin(), f.open.end(), [](const OpenBlock& a, const OpenBlock& b) { return a.order < b.order; });
    for (auto& b : f.open) emit(out, b);
}

// ============================================================== FP32 kernels

__device__ __forceinline__ float2 ld32(const float2* p) { return __ldcs(p); }
__device__ __forceinline__ void st32(float2* p, float2 v) { __stcs(p, v); }

__global__ void k32_init_uniform(float2* __restrict__ a, qidx n, float2 v) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i < n) st32(a + i, v);
}
__global__ void k32_set_one(float2* __restrict__ a, qidx i, float2 v) { a[i] = v; }

__global__ void k_f64_to_f32(float2* __restrict__ dst, const double2* __restrict__ src, qidx n) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i < n) { double2 v = __ldcs(src + i); st32(dst + i, make_float2((float)v.x, (float)v.y)); }
}
__global__ void k_f32_to_f64(double2* __restrict__ dst, const float2* __restrict__ src, qidx n) {
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (i < n) { float2 v = ld32(src + i); __stcs(dst + i, make_double2(v.x, v.y)); }
}

// One 2^K-amplitude group per thread.  off[j]: offset of matrix index j from the
// group base.  The FP32 matrix is staged in shared memory (warp-uniform reads).
template <int K, int NB>
__global__ void __launch_bounds__(128) k32_fused(float2* __restrict__ a, qidx numIts, Ins ins, const float2* __restrict__ M, InsertList<8> offs) {
    constexpr int D = 1 << K;
    __shared__ float2 sm[D * D];
    __shared__ qidx soff[D];
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) sm[i] = M[i];
    if (threadIdx.x < D) {
        qidx o = 0;
        for (int b = 0; b < K; b++) if ((threadIdx.x >> b) & 1) o |= offs.low[b];
        soff[threadIdx.x] = o;
    }
    __syncthreads();
    qidx n = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (n >= numIts) return;
    qidx base = insert_bits<NB>(n, ins);
    float2 v[D];
#pragma unroll
    for (int j = 0; j < D; j++) v[j] = ld32(a + base + soff[j]);
#pragma unroll
    for (int r = 0; r < D; r++) {
        float2 acc = cmulf(sm[r * D], v[0]);
#pragma unroll
        for (int j = 1; j < D; j++) acc = cfmaf(sm[r * D + j], v[j], acc);
        st32(a + base + soff[r], acc);
    }
}

// sum |a_i|^2 in FP64 over an FP32 vector (n even): two amplitudes per 16-byte load,
// four loads in flight per thread, four independent FP64 accumulators.  Each square
// is exact in FP64; the FP64 adds (two per amplitude) bound the kernel near 2.5 TB/s
// on GB300.
__device__ __forceinline__ double sq4(float4 x) {
    return fma((double)x.x, (double)x.x, fma((double)x.y, (double)x.y, fma((double)x.z, (double)x.z, (double)x.w * x.w)));
}

__global__ void __launch_bounds__(RED_THREADS) k32_sum_norm(const float2* __restrict__ a, qidx n, bool vec16, RedOut out) {
    const qidx stride = (qidx)gridDim.x * RED_THREADS;
    qidx i = blockIdx.x * (qidx)RED_THREADS + threadIdx.x;
    if (!vec16) {   // a pointer that is 8- but not 16-byte aligned: one amplitude per load
        double v[1] = {0.0};
        for (; i < n; i += stride) {
            const float2 x = __ldcs(a + i);
            v[0] += (double)x.x * x.x + (double)x.y * x.y;
        }
        block_reduce_and_finish<1>(v, out);
        return;
    }
    const float4* a4 = (const float4*)a;
    const qidx n4 = n >> 1;
    double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        const float4 x0 = __ldcs(a4 + i), x1 = __ldcs(a4 + i + stride);
        const float4 x2 = __ldcs(a4 + i + 2 * stride), x3 = __ldcs(a4 + i + 3 * stride);
        v0 += sq4(x0);
        v1 += sq4(x1);
        v2 += sq4(x2);
        v3 += sq4(x3);
    }
    for (; i < n4; i += stride) v0 += sq4(__ldcs(a4 + i));
    double v[1] = {(v0 + v1) + (v2 + v3)};
    block_reduce_and_finish<1>(v, out);
}

// a_i *= sqrt(target / sum), the sum read from device memory (written by k32_sum_norm);
// the factor is computed once per block, and each thread moves 16-byte pairs
__global__ void __launch_bounds__(256) k32_scale_to_norm(float2* __restrict__ a, qidx n, bool vec16, const double* __restrict__ sum, double target) {
    __shared__ float sf;
    if (threadIdx.x == 0) {
        const double s = *sum;
        sf = s > 0 ? (float)sqrt(target / s) : 1.0f;
    }
    __syncthreads();
    const float f = sf;
    const qidx stride = (qidx)gridDim.x * blockDim.x;
    qidx i = blockIdx.x * (qidx)blockDim.x + threadIdx.x;
    if (!vec16) {
        for (; i < n; i += stride) {
            float2 x = __ldcs(a + i);
            x.x *= f; x.y *= f;
            __stcs(a + i, x);
        }
        return;
    }
    float4* a4 = (float4*)a;
    const qidx n4 = n >> 1;
    for (; i + stride < n4; i += 2 * stride) {
        float4 x0 = __ldcs(a4 + i), x1 = __ldcs(a4 + i + stride);
        x0.x *= f; x0.y *= f; x0.z *= f; x0.w *= f;
        x1.x *= f; x1.y *= f; x1.z *= f; x1.w *= f;
        __stcs(a4 + i, x0);
        __stcs(a4 + i + stride, x1);
    }
    for (; i < n4; i += stride) {
        float4 x = __ldcs(a4 + i);
        x.x *= f; x.y *= f; x.z *= f; x.w *= f;
        __stcs(a4 + i, x);
    }
}

// ============================================================== host side

namespace {

int check32(const void* amps, int nq) {
    if (amps == nullptr) return qg_fail(QG_ERR_ARG, "null amplitude pointer");
    if (nq < 1 || nq > QG_MAX_QUBITS) return qg_fail(QG_ERR_ARG, "numQubits %d outside [1, %d]", nq, QG_MAX_QUBITS);
    if (((uintptr_t)amps) & 7) return qg_fail(QG_ERR_ARG, "FP32 amplitude pointer is not 8-byte aligned");
    return QG_OK;
}

int launch_fused_simt(float2* amps, int nq, const std::vector<int>& targs, const float2* devM, cudaStream_t st) {
    int k = (int)targs.size();
    std::vector<int> zeros(k, 0);
    QubitPlan p;
    QG_TRY(qg_make_plan(nq, nullptr, nullptr, 0, targs.data(), zeros.data(), k, &p));
    InsertList<8> offs;
    offs.num = k;
    for (int b = 0; b < k; b++) offs.low[b] = (qidx)1 << targs[b];
    qidx numIts = ((qidx)1 << nq) >> k;
    unsigned blocks = (unsigned)((numIts + 127) / 128);
#define LK(KV, NBV) k32_fused<KV, NBV><<<blocks, 128, 0, st>>>(amps, numIts, p.ins, devM, offs)
    switch (k) {
        case 1: LK(1, 1); break;
        case 2: LK(2, 2); break;
        case 3: LK(3, 3); break;
        case 4: LK(4, 4); break;
        case 5: LK(5, 5); break;
        default: return qg_fail(QG_ERR_NOTSUP, "FP32 fused blocks of %d qubits are not supported (max 5)", k);
    }
#undef LK
    qg_note_launch();
    return qg_check_launch("k32_fused");
}

}  // namespace

namespace {

size_t round256(size_t x) { return (x + 255) / 256 * 256; }

// assigns each block its matrix offsets; returns (info, f32, tc) byte sizes
void layout_blocks(qg_circuit* c, size_t* infoBytes, size_t* f32Bytes, size_t* tcBytes) {
    size_t n32 = 0, nTC = 0, tcPer = qg_tc_operand_floats();
    for (auto& b : c->blocks) {
        size_t D = (size_t)1 << b.targs.size();
        b.off32 = n32;
        n32 += D * D;
        if (b.targs.size() == 5) { b.offTC = nTC; nTC += tcPer; }
    }
    *infoBytes = round256(c->blocks.size() * sizeof(QgBlockInfo));
    *f32Bytes = round256(n32 * sizeof(float2));
    *tcBytes = round256(nTC * sizeof(float));
    c->tcFloats = nTC;
}

void free_owned(qg_circuit* c) {
    if (c->ownsDevice && c->devInfo) cudaFree(c->devInfo);
    c->devInfo = nullptr;
    c->devF32 = nullptr;
    c->devTC = nullptr;
    c->ownsDevice = false;
    c->uploaded = false;
}

}  // namespace

size_t qg_circuit_device_bytes(qg_circuit* c) {
    size_t a, b, t;
    layout_blocks(c, &a, &b, &t);
    return a + b + t;
}

// Writes the block descriptors, FP32 matrices and tensor-core operands into `dev`
// (qg_circuit_device_bytes bytes) with copies on `st`, in stream order.
int qg_circuit_upload_to(qg_circuit* c, char* dev, cudaStream_t st) {
    free_owned(c);
    size_t infoBytes, f32Bytes, tcBytes;
    layout_blocks(c, &infoBytes, &f32Bytes, &tcBytes);
    std::vector<QgBlockInfo> hInfo(c->blocks.size());
    std::vector<float2> h32(f32Bytes / sizeof(float2));
    std::vector<float> hTC(tcBytes / sizeof(float));
    for (size_t i = 0; i < c->blocks.size(); i++) {
        auto& b = c->blocks[i];
        size_t D = (size_t)1 << b.targs.size();
        for (size_t j = 0; j < D * D; j++) h32[b.off32 + j] = make_float2((float)b.m[j].real(), (float)b.m[j].imag());
        if (b.targs.size() == 5) qg_tc_build_operands(b.m.data(), hTC.data() + b.offTC);
        hInfo[i].k = (int)b.targs.size();
        for (int j = 0; j < 5; j++) hInfo[i].t[j] = j < hInfo[i].k ? b.targs[j] : 0;
        hInfo[i].off32 = (int)b.off32;
        hInfo[i].pad = 0;
    }
    c->devInfo = (QgBlockInfo*)dev;
    c->devF32 = (float2*)(dev + infoBytes);
    c->devTC = (float*)(dev + infoBytes + f32Bytes);
    if (!hInfo.empty()) QG_CUDA(cudaMemcpyAsync(c->devInfo, hInfo.data(), hInfo.size() * sizeof(QgBlockInfo), cudaMemcpyHostToDevice, st));
    if (!h32.empty()) QG_CUDA(cudaMemcpyAsync(c->devF32, h32.data(), h32.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
    if (!hTC.empty()) QG_CUDA(cudaMemcpyAsync(c->devTC, hTC.data(), hTC.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    // copies from pageable memory are staged by the driver before cudaMemcpyAsync returns,
    // so the vectors may die now; the device copy is complete in stream order
    c->uploaded = true;
    return QG_OK;
}

int qg_circuit_upload(qg_circuit* c, cudaStream_t st) {
    free_owned(c);
    size_t bytes = qg_circuit_device_bytes(c);
    char* dev = nullptr;
    QG_CUDA(cudaMalloc(&dev, std::max<size_t>(bytes, 256)));
    QG_TRY(qg_circuit_upload_to(c, dev, st));
    c->ownsDevice = true;
    QG_CUDA(cudaStreamSynchronize(st));
    return QG_OK;
}

extern "C" {

int qg_circuit_create(qg_circuit** out, int numQubits) {
    if (!out) return qg_fail(QG_ERR_ARG, "null output");
    if (numQubits < 1 || numQubits > QG_MAX_QUBITS) return qg_fail(QG_ERR_ARG, "numQubits %d outside [1, %d]", numQubits, QG_MAX_QUBITS);
    *out = new qg_circuit();
    (*out)->numQubits = numQubits;
    return QG_OK;
}

int qg_circuit_destroy(qg_circuit* c) {
    if (!c) return QG_OK;
    free_owned(c);
    delete c;
    return QG_OK;
}

// max |(U^dagger U - I)_ij| <= 1e-10, in FP64
static bool is_unitary(const cd* u, size_t D) {
    for (size_t i = 0; i < D; i++)
        for (size_t j = 0; j < D; j++) {
            cd s = 0;
            for (size_t r = 0; r < D; r++) s += std::conj(u[r * D + i]) * u[r * D + j];
            if (std::abs(s - (i == j ? cd(1) : cd(0))) > 1e-10) return false;
        }
    return true;
}

int qg_circuit_add_matrix(qg_circuit* c, const int* targs, int numTargs, const qg_cplx* matr) {
    if (!c || !matr) return qg_fail(QG_ERR_ARG, "null circuit or matrix");
    if (numTargs < 1 || numTargs > 5) return qg_fail(QG_ERR_ARG, "a circuit gate acts on 1..5 qubits, not %d", numTargs);
    QG_TRY(qg_check_qubits(c->numQubits, targs, numTargs, "gate targets"));
    QgGate g;
    g.targs.assign(targs, targs + numTargs);
    size_t D = (size_t)1 << numTargs;
    g.m.resize(D * D);
    for (size_t i = 0; i < D * D; i++) g.m[i] = cd(matr[i].re, matr[i].im);
    if (c->allUnitary && !is_unitary(g.m.data(), D)) c->allUnitary = false;
    c->gates.push_back(std::move(g));
    c->blocks.clear();
    free_owned(c);
    return QG_OK;
}

int qg_circuit_add_matrices(qg_circuit* c, int numGates, const int* numTargs, const int* targs, const qg_cplx* matrs) {
    if (!c || numGates < 0 || (numGates > 0 && (!numTargs || !targs || !matrs))) return qg_fail(QG_ERR_ARG, "bad gate list");
    for (int g = 0; g < numGates; g++) {
        int k = numTargs[g];
        if (k < 1 || k > 2) return qg_fail(QG_ERR_ARG, "gate %d: the bulk call takes 1- and 2-qubit gates", g);
        QG_TRY(qg_circuit_add_matrix(c, targs + 2 * g, k, matrs + 16 * (size_t)g));
    }
    return QG_OK;
}

int qg_circuit_fuse(qg_circuit* c, int maxFusedQubits) {
    if (!c) return qg_fail(QG_ERR_ARG, "null circuit");
    if (maxFusedQubits < 1 || maxFusedQubits > 5) return qg_fail(QG_ERR_ARG, "fusion width %d outside [1, 5]", maxFusedQubits);
    for (auto& g : c->gates)
        if ((int)g.targs.size() > maxFusedQubits) return qg_fail(QG_ERR_ARG, "a gate is wider than the fusion width");
    c->blocks.clear();
    fuse_gates(c->gates, c->numQubits, maxFusedQubits, c->blocks);
    c->fusedK = maxFusedQubits;
    c->preferredImpl = 0;
    free_owned(c);
    return QG_OK;
}

int qg_circuit_get_num_gates(const qg_circuit* c, int* out) {
    if (!c || !out) return qg_fail(QG_ERR_ARG, "null argument");
    *out = (int)c->gates.size();
    return QG_OK;
}

int qg_circuit_get_num_blocks(const qg_circuit* c, int* out) {
    if (!c || !out) return qg_fail(QG_ERR_ARG, "null argument");
    *out = (int)c->blocks.size();
    return QG_OK;
}

int qg_circuit_get_block(const qg_circuit* c, int i, int* targs, int* numTargs, qg_cplx* matr) {
    if (!c || i < 0 || i >= (int)c->blocks.size()) return qg_fail(QG_ERR_ARG, "block index out of range");
    const QgBlock& b = c->blocks[i];
    *numTargs = (int)b.targs.size();
    for (size_t j = 0; j < b.targs.size(); j++) targs[j] = b.targs[j];
    if (matr)
        for (size_t j = 0; j < b.m.size(); j++) matr[j] = qg_cplx{b.m[j].real(), b.m[j].imag()};
    return QG_OK;
}

// impl: 0 = automatic (tensor cores for 5-qubit blocks on large states), 1 = SIMT FP32, 2 = tensor cores,
// 3 = tensor cores in the self-test of their failure path (operand buffers are never signalled
// full, so every 5-qubit block launch gives up its bounded waits after about 2 s and leaves the
// register untouched).  errorFlag: the device word a timed-out launch reports to (nullptr: the
// device's own flag, reported by the next qg_sv32_apply_circuit or qg_graph_launch).
int qg_sv32_apply_circuit_flag(qg_circuit* c, void* amps, int numQubits, int impl, cudaStream_t st, int* errorFlag) {
    QG_TRY(check32(amps, numQubits));
    if (!c) return qg_fail(QG_ERR_ARG, "null circuit");
    if (impl < 0 || impl > 3) return qg_fail(QG_ERR_ARG, "unknown block kernel choice %d", impl);
    if (!c->uploaded) QG_TRY(qg_circuit_upload(c, st));
    if (numQubits != c->numQubits) return qg_fail(QG_ERR_ARG, "circuit has %d qubits, state has %d", c->numQubits, numQubits);
    if (c->blocks.empty() && !c->gates.empty()) return qg_fail(QG_ERR_ARG, "circuit was not fused (qg_circuit_fuse)");
    if (impl == 0 && c->preferredImpl != 0) impl = c->preferredImpl;
    for (const QgBlock& b : c->blocks) {
        bool tc = b.targs.size() == 5 && (impl >= 2 || (impl == 0 && qg_tc_supported(numQubits)));
        if (tc) {
            QG_TRY(qg_tc_apply_block((float2*)amps, numQubits, b.targs.data(), c->devTC + b.offTC, st, impl == 3, errorFlag));
        } else {
            QG_TRY(launch_fused_simt((float2*)amps, numQubits, b.targs, c->devF32 + b.off32, st));
        }
    }
    return QG_OK;
}

int qg_sv32_apply_circuit(qg_circuit* c, void* amps, int numQubits, int impl, void* stream) {
    // a timeout left by an earlier launch on this device is reported here, before more work goes out
    QG_TRY(qg_tc_take_error());
    return qg_sv32_apply_circuit_flag(c, amps, numQubits, impl, qg_stream(stream), nullptr);
}

// ---------------------------------------------------------------- CUDA graphs of a circuit

struct qg_graph {
    cudaGraphExec_t exec = nullptr;
    int numKernels = 0;
};

int qg_circuit_graph_create(qg_circuit* c, void* amps, int numQubits, int impl, qg_graph** out) {
    QG_TRY(check32(amps, numQubits));
    if (!c || !out) return qg_fail(QG_ERR_ARG, "null argument");
    if (numQubits != c->numQubits) return qg_fail(QG_ERR_ARG, "circuit has %d qubits, state has %d", c->numQubits, numQubits);
    if (c->blocks.empty() && !c->gates.empty()) return qg_fail(QG_ERR_ARG, "circuit was not fused (qg_circuit_fuse)");
    // everything that allocates or synchronises happens before the capture
    if (!c->uploaded) QG_TRY(qg_circuit_upload(c, nullptr));
    if (numQubits >= 12) QG_TRY(qg_tc_prepare());
    cudaStream_t s = nullptr;
    QG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int64_t before = 0, after = 0;
    qg_get_launch_count(&before);
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return qg_check_cuda(e, "cudaStreamBeginCapture");
    }
    int rc = qg_sv32_apply_circuit_flag(c, amps, numQubits, impl, s, nullptr);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    qg_get_launch_count(&after);
    qg_note_launch(-(int)(after - before));        // captured, not launched
    cudaStreamDestroy(s);
    if (rc != QG_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rc != QG_OK ? rc : qg_check_cuda(e, "cudaStreamEndCapture");
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return qg_check_cuda(e, "cudaGraphInstantiate");
    qg_graph* g = new qg_graph;
    g->exec = exec;
    g->numKernels = (int)(after - before);
    *out = g;
    return QG_OK;
}

int qg_graph_launch(qg_graph* g, void* stream) {
    if (!g) return qg_fail(QG_ERR_ARG, "null graph");
    QG_TRY(qg_tc_take_error());
    QG_CUDA(cudaGraphLaunch(g->exec, qg_stream(stream)));
    qg_note_launch(g->numKernels);
    return QG_OK;
}

int qg_graph_get_num_kernels(const qg_graph* g, int* out) {
    if (!g || !out) return qg_fail(QG_ERR_ARG, "null argument");
    *out = g->numKernels;
    return QG_OK;
}

int qg_graph_destroy(qg_graph* g) {
    if (!g) return QG_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    delete g;
    return QG_OK;
}

// ---------------------------------------------------------------- fusion autotuner

// Times the circuit fused at every width k in [widest gate, 5] with the SIMT kernel,
// and at k = 5 with the tensor-core kernel (12 qubits and up), on a scratch register
// of the circuit's size; leaves the circuit fused at the fastest width with that
// kernel preferred by automatic applies.  Candidate i (in the order tried) is
// (candK[i], candImpl[i]) and took msOut[i] milliseconds per circuit.
int qg_circuit_autotune(qg_circuit* c, int* bestK, int* bestImpl, int* candK, int* candImpl, double* msOut, int maxOut,
                        int* numOut) {
    if (!c) return qg_fail(QG_ERR_ARG, "null circuit");
    const int nq = c->numQubits;
    if (nq < 5) return qg_fail(QG_ERR_ARG, "autotuning needs at least 5 qubits");
    int widest = 1;
    for (const auto& g : c->gates) widest = std::max(widest, (int)g.targs.size());
    void* amps = nullptr;
    QG_TRY(qg_alloc(&amps, (int64_t)8 << nq));
    void* ev0 = nullptr;
    void* ev1 = nullptr;
    int rc = QG_OK, n = 0, kBest = 5, iBest = 1;
    double tBest = 1e300;
    if ((rc = qg_event_create(&ev0)) == QG_OK) rc = qg_event_create(&ev1);
    for (int k = std::max(3, widest); k <= 5 && rc == QG_OK; k++) {
        for (int impl = 1; impl <= 2 && rc == QG_OK; impl++) {
            if (impl == 2 && (k != 5 || nq < 12)) continue;
            if ((rc = qg_circuit_fuse(c, k)) != QG_OK) break;
            if ((rc = qg_circuit_upload(c, nullptr)) != QG_OK) break;
            if ((rc = qg_sv32_initClassicalState(amps, nq, 0, nullptr)) != QG_OK) break;
            if ((rc = qg_sv32_apply_circuit(c, amps, nq, impl, nullptr)) != QG_OK) break;    // warm-up
            const int reps = 2;
            if ((rc = qg_event_record(ev0, nullptr)) != QG_OK) break;
            for (int r = 0; r < reps && rc == QG_OK; r++) rc = qg_sv32_apply_circuit(c, amps, nq, impl, nullptr);
            if (rc == QG_OK) rc = qg_event_record(ev1, nullptr);
            float ms = 0;
            if (rc == QG_OK) rc = qg_event_elapsed_ms(ev0, ev1, &ms);
            if (rc != QG_OK) break;
            const double per = ms / reps;
            if (n < maxOut) {
                if (msOut) msOut[n] = per;
                if (candK) candK[n] = k;
                if (candImpl) candImpl[n] = impl;
            }
            n++;
            if (per < tBest) { tBest = per; kBest = k; iBest = impl; }
        }
    }
    if (ev0) qg_event_destroy(ev0);
    if (ev1) qg_event_destroy(ev1);
    qg_free(amps);
    if (rc != QG_OK) return rc;
    QG_TRY(qg_circuit_fuse(c, kBest));
    c->preferredImpl = iBest;
    if (bestK) *bestK = kBest;
    if (bestImpl) *bestImpl = iBest;
    if (numOut) *numOut = n;
    return QG_OK;
}

int qg_sv32_initUniformState(void* amps, int numQubits, qg_cplxf amp, void* stream) {
    QG_TRY(check32(amps, numQubits));
    qidx n = (qidx)1 << numQubits;
    k32_init_uniform<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((float2*)amps, n, make_float2(amp.re, amp.im));
    qg_note_launch();
    return qg_check_launch("k32_init_uniform");
}

int qg_sv32_initClassicalState(void* amps, int numQubits, int64_t index, void* stream) {
    QG_TRY(check32(amps, numQubits));
    qidx n = (qidx)1 << numQubits;
    if (index < 0 || index >= n) return qg_fail(QG_ERR_ARG, "basis index outside the state");
    k32_init_uniform<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((float2*)amps, n, make_float2(0, 0));
    k32_set_one<<<1, 1, 0, qg_stream(stream)>>>((float2*)amps, index, make_float2(1, 0));
    qg_note_launch(2);
    return qg_check_launch("k32_init_classical");
}

int qg_sv_convert_f64_to_f32(void* dst32, const void* src64, int numQubits, void* stream) {
    QG_TRY(check32(dst32, numQubits));
    QG_TRY(qg_check_amps(src64, numQubits));
    qidx n = (qidx)1 << numQubits;
    k_f64_to_f32<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((float2*)dst32, (const double2*)src64, n);
    qg_note_launch();
    return qg_check_launch("k_f64_to_f32");
}

int qg_sv_convert_f32_to_f64(void* dst64, const void* src32, int numQubits, void* stream) {
    QG_TRY(check32(src32, numQubits));
    QG_TRY(qg_check_amps(dst64, numQubits));
    qidx n = (qidx)1 << numQubits;
    k_f32_to_f64<<<qg_blocks(n), QG_THREADS, 0, qg_stream(stream)>>>((double2*)dst64, (const float2*)src32, n);
    qg_note_launch();
    return qg_check_launch("k_f32_to_f64");
}

int qg_sv32_calcTotalProb(const void* amps, int numQubits, double* out, void* stream) {
    QG_TRY(check32(amps, numQubits));
    qidx n = (qidx)1 << numQubits;
    int grid = red_grid(n);
    RedOut r;
    QG_TRY(red_setup(grid, 1, &r));
    cudaStream_t st = qg_stream(stream);
    k32_sum_norm<<<grid, RED_THREADS, 0, st>>>((const float2*)amps, n, ((uintptr_t)amps & 15) == 0, r);
    return red_fetch(r, 1, out, st);
}

int qg_sv32_normalise(void* amps, int numQubits, double targetProb, void* stream) {
    QG_TRY(check32(amps, numQubits));
    if (!(targetProb > 0)) return qg_fail(QG_ERR_ARG, "target probability must be positive");
    qidx n = (qidx)1 << numQubits;
    int grid = red_grid(n);
    RedOut r;
    QG_TRY(red_setup(grid, 1, &r));
    cudaStream_t st = qg_stream(stream);
    const bool vec16 = ((uintptr_t)amps & 15) == 0;
    k32_sum_norm<<<grid, RED_THREADS, 0, st>>>((const float2*)amps, n, vec16, r);
    qg_note_launch();
    QG_TRY(qg_check_launch("k32_sum_norm"));
    const unsigned sgrid = (unsigned)std::min<qidx>(qg_blocks(n / 2, 256), (qidx)qg_num_sms() * 8);
    k32_scale_to_norm<<<sgrid, 256, 0, st>>>((float2*)amps, n, vec16, r.result, targetProb);
    qg_note_launch();
    return qg_check_launch("k32_scale_to_norm");
}

int qg_sv32_calcExpecPauliStrBatch(const void* amps, int numQubits, const int64_t* masksXY, const int64_t* masksYZ,
                                   const int* numsY, int numStrings, qg_cplx* out, void* stream) {
    QG_TRY(check32(amps, numQubits));
    if (numStrings < 0) return qg_fail(QG_ERR_ARG, "negative string count");
    qidx lim = ((qidx)1 << numQubits) - 1;
    for (int s = 0; s < numStrings; s++)
        if ((masksXY[s] & ~lim) || (masksYZ[s] & ~lim)) return qg_fail(QG_ERR_ARG, "Pauli string %d targets a qubit beyond %d", s, numQubits);
    if (numStrings > 0 && (!masksXY || !masksYZ || !numsY || !out)) return qg_fail(QG_ERR_ARG, "null argument");
    // the tiled kernel of qg_pauli_tile.cu: FP32 amplitudes, FP64 products and sums
    return numStrings ? qg_pauli_tile_batch<float2>((const float2*)amps, numQubits, masksXY, masksYZ, numsY, numStrings, out,
                                                    qg_stream(stream))
                      : QG_OK;
}

}  // extern "C"
