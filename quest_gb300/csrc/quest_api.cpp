// QuEST v4 API functions of the gate-application path, on the GB300 backend.
//
// This file is the host side above the C ABI (include/quest_gb300.h).  It keeps
// the reference's observable behaviour: the same validation (and error handler
// contract), the same decomposition of each API call into backend calls
// (quest/src/api/operations.cpp, decoherence.cpp, calculations.cpp and the
// single-node branches of quest/src/core/localiser.cpp), the same gate
// constants, and the same host random-number stream for measurements
// (std::mt19937_64 seeded through std::seed_seq, a uniform double in [0,1)
// compared with the zero-outcome probability; quest/src/core/randomiser.cpp:59-137).
// Every Qureg lives on the GPU; nothing here evaluates amplitudes on the CPU.
#include "quest_gb300_api.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

using std::vector;
typedef std::complex<double> cd;

// backend internals (quest_gb300/csrc): the product mode, and whether a gate on numIts
// amplitude groups takes the tensor-core slices
int qg_fp64_products_mode();
bool qg_dense_tc_wanted(long long numIts);

namespace {

const int QG_MAX_QUBITS_API = 40;    // 2^40 FP64 amplitudes = 16 TiB: far above one GPU
const double DEFAULT_EPS = 1e-12;            // precision.h:131-140 at FLOAT_PRECISION=2
const double REDUCTION_EPS_FACTOR = 100;     // validation.cpp:1137
double g_eps = DEFAULT_EPS;
bool g_envInit = false;
thread_local void* g_stream = nullptr;
// how each Qureg's host mirror was allocated (keyed by cpuAmps)
enum { MIRROR_PINNED = 0, MIRROR_REGISTERED = 1, MIRROR_PAGEABLE = 2 };
std::map<void*, int> g_mirrorKind;
std::mutex g_mirrorMu;
std::mt19937_64 g_rng;

void default_handler(const char* func, const char* msg) {
    std::fprintf(stderr, "\nQuEST encountered a validation error during function '%s':\n%s\nExiting...\n", func, msg);
    std::exit(EXIT_FAILURE);
}
void (*g_handler)(const char*, const char*) = default_handler;

// Reports a failed check; returns false so callers can `if (!check(...)) return;`
bool fail(const char* func, const std::string& msg) {
    g_handler(func, msg.c_str());
    return false;
}
bool check(bool cond, const char* func, const std::string& msg) { return cond ? true : fail(func, msg); }
bool backend(int rc, const char* func) {
    if (rc == QG_OK) return true;
    std::string m = std::string("GPU backend call failed in ") + func + ": " + qg_get_last_error();
    g_handler("qg_backend", m.c_str());
    return false;
}

inline int nsv(const Qureg& q) { return q.isDensityMatrix ? 2 * q.numQubits : q.numQubits; }
inline cd C(qcomp_t c) { return cd(c.re, c.im); }
inline qcomp_t Q(cd c) { return qcomp_t{c.real(), c.imag()}; }

bool checkEnv(const char* func) { return check(g_envInit, func, "The QuEST environment has not been initialised."); }

// ------------------------------------------------------------------ deferred one-qubit superoperators
// On a density matrix, a one-qubit unitary and a one-qubit channel act on the pair
// (ket q, bra q+N) of the Choi vector as a 4x4 superoperator (matrix index bit 0 = ket,
// bit 1 = bra).  Such operations are not applied at once: per ket qubit they are
// multiplied into one pending 4x4 in FP64 on the host, and the product is applied in
// one pass when something needs the state -- any other API call on the Qureg (all
// pending qubits), or a multi-qubit operation (only the qubits it touches: operations on
// other qubits commute with it).  A unitary followed by depolarising on the same qubit
// then costs one pass instead of two.  A qubit whose only pending operation is a single
// channel is applied with that channel's own kernel.
enum { PEND_GENERAL = 0, PEND_DEPOL, PEND_DEPHASE, PEND_DAMP, PEND_PAULIS, PEND_SV };
struct PendingOp {
    int kind;
    double p[3];      // the channel's parameters when kind is not PEND_GENERAL
    cd m[16];         // the product of the qubit's pending superoperators, row-major
};
typedef std::vector<std::pair<long long, cd>> PhaseList;
struct PendingSet {
    int numQubits;                      // the Qureg's (ket) qubits
    bool dm;                            // a density matrix (else a statevector: PEND_SV ops)
    std::map<int, PendingOp> ops;       // ket qubit -> its pending op
    // statevectors: pending controlled phases (qubit mask, factor), which commute with one
    // another and come after every pending one-qubit op and the block (a one-qubit gate on
    // a qubit of a pending phase applies everything pending first)
    PhaseList phases;
    // statevectors: a pending two-qubit unitary (blockQ[0] < blockQ[1], -1 when none; 4x4,
    // index bit i = qubit blockQ[i]), whose qubits have no entry in `ops`
    int blockQ[2] = {-1, -1};
    cd block[16];
};
std::map<const void*, PendingSet> g_pending;   // keyed by gpuAmps
std::mutex g_pendingMu;

bool backend(int rc, const char* func);

bool applyPendingOp(const Qureg& q, int qubit, const PendingOp& op, const char* func) {
    const int N = q.numQubits;
    switch (op.kind) {
        case PEND_DEPOL: return backend(qg_dm_oneQubitDepolarising(q.gpuAmps, N, qubit, op.p[0], g_stream), func);
        case PEND_DEPHASE: return backend(qg_dm_oneQubitDephasing(q.gpuAmps, N, qubit, op.p[0], g_stream), func);
        case PEND_DAMP: return backend(qg_dm_oneQubitDamping(q.gpuAmps, N, qubit, op.p[0], g_stream), func);
        case PEND_PAULIS: return backend(qg_dm_oneQubitPauliChannel(q.gpuAmps, N, qubit, op.p[0], op.p[1], op.p[2], g_stream), func);
        case PEND_SV:       // statevector ops are applied in groups (applySVUnits), never here
            return check(false, func, "Internal error: a statevector's pending gate reached the density-matrix path.");
        default: {
            qcomp_t k[16];
            for (int i = 0; i < 16; i++) k[i] = qcomp_t{op.m[i].real(), op.m[i].imag()};
            return backend(qg_sv_anyCtrlTwoTargDenseMatr(q.gpuAmps, 2 * N, nullptr, nullptr, 0, qubit, qubit + N, k, g_stream), func);
        }
    }
}

// Two qubits' superoperators, or a two-qubit unitary's, as one 16x16 superoperator on the
// Choi targets (a, b, a + N, b + N): matrix index bit 0 = ket a, 1 = ket b, 2 = bra a,
// 3 = bra b.  One pass of the four-target tensor-core kernel costs about what one pass of a
// one-qubit superoperator does, so when that kernel runs (product mode 0, registers of at
// least one tile per SM) pairs of pending qubits are applied together.
bool pairSuperops(const Qureg& q) {
    return q.isDensityMatrix && q.numQubits >= 3 && q.numQubits <= QG_MAX_QUBITS_API / 2 && qg_fp64_products_mode() == 0 &&
           qg_dense_tc_wanted((long long)1 << (2 * q.numQubits - 4));
}

bool applyPairOp(const Qureg& q, int a, int b, const cd (&M)[256], const char* func) {
    qcomp_t k[256];
    for (int i = 0; i < 256; i++) k[i] = qcomp_t{M[i].real(), M[i].imag()};
    const int t[4] = {a, b, a + q.numQubits, b + q.numQubits};
    return backend(qg_sv_anyCtrlAnyTargDenseMatr(q.gpuAmps, 2 * q.numQubits, nullptr, nullptr, 0, t, 4, k, 0, g_stream), func);
}

// Sa on qubit a and Sb on qubit b (4x4, index bit 0 = ket, bit 1 = bra), as the 16x16 above
void kronPair(const cd (&Sa)[16], const cd (&Sb)[16], cd (&M)[256]) {
    for (int j = 0; j < 16; j++)
        for (int k = 0; k < 16; k++) {
            const int ja = (j & 1) | (((j >> 2) & 1) << 1), jb = ((j >> 1) & 1) | (((j >> 3) & 1) << 1);
            const int ka = (k & 1) | (((k >> 2) & 1) << 1), kb = ((k >> 1) & 1) | (((k >> 3) & 1) << 1);
            M[j * 16 + k] = Sa[ja * 4 + ka] * Sb[jb * 4 + kb];
        }
}

// A two-qubit superoperator M (16x16 on (a, b, a + N, b + N)) applied after the pending
// one-qubit superoperators of ket qubits a and b: those are taken out of the pending set
// and multiplied in (M <- M (Sa (x) Sb), a missing one the identity), so that the qubits'
// pending work costs no pass of its own.  Other pending qubits commute with M.
void composePendingPair(const Qureg& q, int a, int b, cd (&M)[256]) {
    cd S[2][16];
    bool any = false;
    {
        std::lock_guard<std::mutex> lock(g_pendingMu);
        auto it = g_pending.find(q.gpuAmps);
        for (int i = 0; i < 2; i++) {
            for (int e = 0; e < 16; e++) S[i][e] = (e % 5 == 0) ? cd(1) : cd(0);
            if (it == g_pending.end()) continue;
            auto jt = it->second.ops.find(i == 0 ? a : b);
            if (jt == it->second.ops.end()) continue;
            for (int e = 0; e < 16; e++) S[i][e] = jt->second.m[e];
            it->second.ops.erase(jt);
            any = true;
        }
        if (it != g_pending.end() && it->second.ops.empty() && it->second.phases.empty() && it->second.blockQ[0] < 0)
            g_pending.erase(it);
    }
    if (!any) return;
    cd P[256], R[256];
    kronPair(S[0], S[1], P);
    for (int j = 0; j < 16; j++)
        for (int k = 0; k < 16; k++) {
            cd acc = 0;
            for (int m = 0; m < 16; m++) acc += M[j * 16 + m] * P[m * 16 + k];
            R[j * 16 + k] = acc;
        }
    for (int i = 0; i < 256; i++) M[i] = R[i];
}

// Statevectors: one-qubit dense unitaries are deferred the same way (a pending 2x2 per
// qubit, composed on the host) when the tensor-core kernel runs for four targets, and the
// pending qubits are applied four at a time as the Kronecker product of their unitaries
// (one pass instead of four), then three, two or one.
bool deferSV(const Qureg& q) {
    return !q.isDensityMatrix && q.numQubits >= 5 && q.numQubits <= QG_MAX_QUBITS_API && qg_fp64_products_mode() == 0 &&
           qg_dense_tc_wanted((long long)1 << (q.numQubits - 4));
}

// U applied after the qubit's pending unitary: pending = U * pending (the block's, when the
// qubit is one of the pending two-qubit block's)
void addPendingSV(const Qureg& q, int qubit, const cd (&U)[4]) {
    std::lock_guard<std::mutex> lock(g_pendingMu);
    PendingSet& set = g_pending[q.gpuAmps];
    set.numQubits = q.numQubits;
    set.dm = false;
    if (qubit == set.blockQ[0] || qubit == set.blockQ[1]) {
        const int bit = qubit == set.blockQ[0] ? 0 : 1;
        cd nb[16];
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) {
                cd acc = 0;
                for (int v = 0; v < 2; v++) {
                    const int sr = (r & ~(1 << bit)) | (v << bit);     // r with its `bit` set to v
                    acc += U[((r >> bit) & 1) * 2 + v] * set.block[sr * 4 + c];
                }
                nb[r * 4 + c] = acc;
            }
        for (int i = 0; i < 16; i++) set.block[i] = nb[i];
        return;
    }
    auto it = set.ops.find(qubit);
    if (it == set.ops.end()) {
        PendingOp op;
        op.kind = PEND_SV;
        op.p[0] = op.p[1] = op.p[2] = 0;
        for (int i = 0; i < 16; i++) op.m[i] = i < 4 ? U[i] : cd(0);
        set.ops[qubit] = op;
        return;
    }
    cd* P = it->second.m;
    const cd r0 = U[0] * P[0] + U[1] * P[2], r1 = U[0] * P[1] + U[1] * P[3];
    const cd r2 = U[2] * P[0] + U[3] * P[2], r3 = U[2] * P[1] + U[3] * P[3];
    P[0] = r0; P[1] = r1; P[2] = r2; P[3] = r3;
}

// a pending statevector unitary on one qubit or on two (q[0] < q[1]; 2^k x 2^k, index bit i
// = qubit q[i])
struct SVUnit {
    int k;
    int q[2];
    cd m[16];
};

// Groups of at most four pending statevector qubits (indices into `units`, whose units
// stay whole), one pass each.  A pending phase whose qubits all have pending units and fall
// into one group is folded into that group's matrix (it acts after the group's unitaries and
// commutes with every other group), which saves the phase pass when all of them fold.  So
// the units joined by such phases (clusters of at most four qubits) are packed into the
// groups first-fit, largest first, into as many groups as the plain split needs (n/4 groups
// of four qubits and one of n % 4); the cluster holding qubit 0 goes to the smaller group
// when it fits there and the rest still packs, since a four-qubit pass without qubit 0 takes
// the faster (staged) tensor-core form.  When the clusters do not pack into that many
// groups, the units are packed in ascending order of their qubits, qubit 0 last.
std::vector<std::vector<int>> groupSV(const std::vector<SVUnit>& units, const PhaseList& phases) {
    const int nu = (int)units.size();
    int n = 0;
    for (auto& u : units) n += u.k;
    auto holdsZero = [&](int i) { return units[i].q[0] == 0 || (units[i].k == 2 && units[i].q[1] == 0); };
    std::vector<std::vector<int>> plain;
    {
        std::vector<int> order(nu);
        for (int i = 0; i < nu; i++) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            if (holdsZero(x) != holdsZero(y)) return holdsZero(y);
            return units[x].q[0] < units[y].q[0];
        });
        int room = 0;
        for (int i : order) {
            if (room < units[i].k) {
                plain.emplace_back();
                room = 4;
            }
            plain.back().push_back(i);
            room -= units[i].k;
        }
    }
    if (phases.empty() || nu < 2) return plain;
    long long pendingMask = 0;
    int at[64];
    for (int i = 0; i < nu; i++)
        for (int b = 0; b < units[i].k; b++) {
            pendingMask |= 1LL << units[i].q[b];
            at[units[i].q[b]] = i;
        }
    std::vector<int> parent(nu);
    for (int i = 0; i < nu; i++) parent[i] = i;
    auto find = [&](int i) {
        while (parent[i] != i) i = parent[i] = parent[parent[i]];
        return i;
    };
    for (auto& ph : phases) {
        const long long m = ph.first;
        if ((m & ~pendingMask) != 0 || __builtin_popcountll((unsigned long long)m) > 4) continue;
        int first = -1;
        for (int b = 0; b < 64; b++) {
            if (!((m >> b) & 1)) continue;
            if (first < 0) first = find(at[b]);
            else parent[find(at[b])] = first;
        }
    }
    std::map<int, std::vector<int>> byRoot;
    for (int i = 0; i < nu; i++) byRoot[find(i)].push_back(i);
    struct Item {
        std::vector<int> members;
        int size;
    };
    std::vector<Item> items;
    for (auto& kv : byRoot) {
        int size = 0;
        for (int i : kv.second) size += units[i].k;
        if (size <= 4) items.push_back({kv.second, size});
        else for (int i : kv.second) items.push_back({{i}, units[i].k});
    }
    const int numFull = n / 4, rem = n % 4;
    std::stable_sort(items.begin(), items.end(), [](const Item& x, const Item& y) { return x.size > y.size; });
    // first-fit, largest first; with `zeroLast`, the item holding qubit 0 goes first to the
    // smaller group
    auto pack = [&](bool zeroLast, std::vector<std::vector<int>>& groups) {
        groups.assign(numFull + (rem ? 1 : 0), std::vector<int>());
        std::vector<int> room(groups.size(), 4);
        if (rem) room.back() = rem;
        std::vector<char> placed(items.size(), 0);
        for (size_t k = 0; zeroLast && k < items.size(); k++) {
            bool zero = false;
            for (int i : items[k].members) zero = zero || holdsZero(i);
            if (rem && zero && items[k].size <= rem) {
                groups.back() = items[k].members;
                room.back() -= items[k].size;
                placed[k] = 1;
                break;
            }
        }
        for (size_t k = 0; k < items.size(); k++) {
            if (placed[k]) continue;
            size_t g = 0;
            while (g < groups.size() && room[g] < items[k].size) g++;
            if (g == groups.size()) return false;
            groups[g].insert(groups[g].end(), items[k].members.begin(), items[k].members.end());
            room[g] -= items[k].size;
        }
        return true;
    };
    std::vector<std::vector<int>> groups;
    if (pack(true, groups) || pack(false, groups)) return groups;
    return plain;
}

// The matrix of a group of units (qubits ascending; bit b of an index = the group's b-th
// qubit), with the not yet applied phases that lie inside the group folded in (a phase
// multiplies the rows whose bits of its mask are all set).
struct SVGroupOp {
    int k;
    int t[4];
    std::vector<cd> m;
};
SVGroupOp svGroupOp(const std::vector<SVUnit>& units, const std::vector<int>& grp, const PhaseList& phases,
                    std::vector<char>& applied) {
    SVGroupOp g;
    g.k = 0;
    for (int i : grp)
        for (int b = 0; b < units[i].k; b++) g.t[g.k++] = units[i].q[b];
    std::sort(g.t, g.t + g.k);
    int pos[64];
    long long groupMask = 0;
    for (int b = 0; b < g.k; b++) {
        pos[g.t[b]] = b;
        groupMask |= 1LL << g.t[b];
    }
    const int D = 1 << g.k;
    std::vector<cd> rowFactor(D, cd(1));
    for (size_t p = 0; p < phases.size(); p++) {
        if (applied[p] || (phases[p].first & ~groupMask) != 0) continue;
        int local = 0;
        for (int b = 0; b < g.k; b++)
            if ((phases[p].first >> g.t[b]) & 1) local |= 1 << b;
        for (int j = 0; j < D; j++)
            if ((j & local) == local) rowFactor[j] *= phases[p].second;
        applied[p] = 1;
    }
    g.m.assign((size_t)D * D, cd(0));
    for (int j = 0; j < D; j++)
        for (int c = 0; c < D; c++) {
            cd v = rowFactor[j];
            for (int i : grp) {
                const SVUnit& u = units[i];
                int jj = 0, cc = 0;
                for (int b = 0; b < u.k; b++) {
                    jj |= ((j >> pos[u.q[b]]) & 1) << b;
                    cc |= ((c >> pos[u.q[b]]) & 1) << b;
                }
                v *= u.m[jj * (1 << u.k) + cc];
            }
            g.m[(size_t)j * D + c] = v;
        }
    return g;
}

bool applySVGroupOp(const Qureg& q, const SVGroupOp& g, const char* func) {
    std::vector<qcomp_t> M(g.m.size());
    for (size_t i = 0; i < g.m.size(); i++) M[i] = qcomp_t{g.m[i].real(), g.m[i].imag()};
    if (g.k == 1) return backend(qg_sv_anyCtrlOneTargDenseMatr(q.gpuAmps, q.numQubits, nullptr, nullptr, 0, g.t[0], M.data(), g_stream), func);
    if (g.k == 2) return backend(qg_sv_anyCtrlTwoTargDenseMatr(q.gpuAmps, q.numQubits, nullptr, nullptr, 0, g.t[0], g.t[1], M.data(), g_stream), func);
    return backend(qg_sv_anyCtrlAnyTargDenseMatr(q.gpuAmps, q.numQubits, nullptr, nullptr, 0, g.t, g.k, M.data(), 0, g_stream), func);
}

// applies a set of pending phases, 32 per pass
bool applyPhases(const Qureg& q, const PhaseList& ph, const char* func) {
    for (size_t i = 0; i < ph.size(); i += 32) {
        const int num = (int)std::min<size_t>(32, ph.size() - i);
        int64_t masks[32];
        qcomp_t f[32];
        for (int k = 0; k < num; k++) {
            masks[k] = ph[i + k].first;
            f[k] = qcomp_t{ph[i + k].second.real(), ph[i + k].second.imag()};
        }
        if (!backend(qg_sv_phaseSet(q.gpuAmps, q.numQubits, masks, f, num, g_stream), func)) return false;
    }
    return true;
}

// Applies a statevector's pending units in the groups of groupSV, with the phases that fit
// in a group folded into its pass, then the other phases together.  With `keepLast`, a last
// group of one or two qubits that no remaining phase touches is not applied but stays
// pending (as the two-qubit block, or a one-qubit op): the next flush packs it with the
// units that later phases join it to, which saves a pass per flush when the qubit count is
// not a multiple of four (the gates of the next layer on its qubits join it meanwhile).
bool applySVUnits(const Qureg& q, const std::vector<SVUnit>& units, const PhaseList& phases, bool keepLast, const char* func) {
    std::vector<char> applied(phases.size(), 0);
    std::vector<std::vector<int>> groups = groupSV(units, phases);
    std::vector<SVGroupOp> ops;
    for (auto& grp : groups) ops.push_back(svGroupOp(units, grp, phases, applied));
    bool keep = keepLast && !ops.empty() && ops.back().k <= 2;
    if (keep) {
        long long lastMask = 0;
        for (int b = 0; b < ops.back().k; b++) lastMask |= 1LL << ops.back().t[b];
        for (size_t p = 0; p < phases.size(); p++) keep = keep && (applied[p] || (phases[p].first & lastMask) == 0);
    }
    for (size_t i = 0; i + (keep ? 1 : 0) < ops.size(); i++)
        if (!applySVGroupOp(q, ops[i], func)) return false;
    if (keep) {
        const SVGroupOp& g = ops.back();
        std::lock_guard<std::mutex> lock(g_pendingMu);
        PendingSet& set = g_pending[q.gpuAmps];
        set.numQubits = q.numQubits;
        set.dm = false;
        if (g.k == 2) {
            set.blockQ[0] = g.t[0];
            set.blockQ[1] = g.t[1];
            for (int i = 0; i < 16; i++) set.block[i] = g.m[i];
        } else {
            PendingOp op;
            op.kind = PEND_SV;
            op.p[0] = op.p[1] = op.p[2] = 0;
            for (int i = 0; i < 16; i++) op.m[i] = i < 4 ? g.m[i] : cd(0);
            set.ops[g.t[0]] = op;
        }
    }
    PhaseList rest;
    for (size_t p = 0; p < phases.size(); p++)
        if (!applied[p]) rest.push_back(phases[p]);
    return applyPhases(q, rest, func);
}

// applies a density matrix's pending ops: in pairs when that pays (general superoperators
// first, a remaining one with a channel), the rest one by one
bool applyPendingList(const Qureg& q, std::vector<std::pair<int, PendingOp>>& todo, const char* func) {
    if (todo.size() >= 2 && pairSuperops(q)) {
        std::stable_partition(todo.begin(), todo.end(), [](const std::pair<int, PendingOp>& x) { return x.second.kind == PEND_GENERAL; });
        size_t i = 0;
        for (; i + 1 < todo.size(); i += 2) {
            if (todo[i].second.kind != PEND_GENERAL) break;    // two channels: their own kernels are cheaper
            cd M[256];
            kronPair(todo[i].second.m, todo[i + 1].second.m, M);
            if (!applyPairOp(q, todo[i].first, todo[i + 1].first, M, func)) return false;
        }
        for (; i < todo.size(); i++)
            if (!applyPendingOp(q, todo[i].first, todo[i].second, func)) return false;
        return true;
    }
    for (auto& kv : todo)
        if (!applyPendingOp(q, kv.first, kv.second, func)) return false;
    return true;
}

// applies the pending ops of the listed ket qubits (all of them when `qubits` is null); when
// a statevector's pending phase involves a listed qubit, everything pending is applied
// (the phases come after the pending ops of their qubits); `keepLast` as in applySVUnits
bool flushPending(const Qureg& q, const std::vector<int>* qubits, const char* func, bool keepLast = false) {
    std::vector<std::pair<int, PendingOp>> todo;
    PhaseList phases;
    std::vector<SVUnit> units;
    bool dm = true;
    {
        std::lock_guard<std::mutex> lock(g_pendingMu);
        auto it = g_pending.find(q.gpuAmps);
        if (it == g_pending.end()) return true;
        PendingSet& set = it->second;
        dm = set.dm;
        long long touched = 0;
        if (qubits)
            for (int b : *qubits) touched |= 1LL << b;
        bool all = !qubits;
        for (auto& ph : set.phases) all = all || (ph.first & touched) != 0;
        bool takeBlock = set.blockQ[0] >= 0 && (all || ((touched >> set.blockQ[0]) & 1) || ((touched >> set.blockQ[1]) & 1));
        if (all) {
            phases.swap(set.phases);
            for (auto& kv : set.ops) todo.push_back(kv);
            set.ops.clear();
        } else {
            for (int b : *qubits) {
                auto jt = set.ops.find(b);
                if (jt == set.ops.end()) continue;
                todo.push_back(*jt);
                set.ops.erase(jt);
            }
        }
        if (!dm) {
            for (auto& kv : todo) {
                SVUnit u;
                u.k = 1;
                u.q[0] = kv.first;
                u.q[1] = -1;
                for (int i = 0; i < 16; i++) u.m[i] = kv.second.m[i];
                units.push_back(u);
            }
            if (takeBlock) {
                SVUnit u;
                u.k = 2;
                u.q[0] = set.blockQ[0];
                u.q[1] = set.blockQ[1];
                for (int i = 0; i < 16; i++) u.m[i] = set.block[i];
                units.push_back(u);
                set.blockQ[0] = set.blockQ[1] = -1;
            }
        }
        if (set.ops.empty() && set.phases.empty() && set.blockQ[0] < 0) g_pending.erase(it);
    }
    if (dm) return applyPendingList(q, todo, func);
    return applySVUnits(q, units, phases, keepLast, func);
}

// a pending phase on a statevector involves this qubit
bool phasePendingOn(const Qureg& q, int qubit) {
    std::lock_guard<std::mutex> lock(g_pendingMu);
    auto it = g_pending.find(q.gpuAmps);
    if (it == g_pending.end()) return false;
    for (auto& ph : it->second.phases)
        if ((ph.first >> qubit) & 1) return true;
    return false;
}

// defers a controlled phase of a statevector (it acts after the pending one-qubit ops)
void addPendingPhase(const Qureg& q, long long mask, cd factor) {
    std::lock_guard<std::mutex> lock(g_pendingMu);
    PendingSet& set = g_pending[q.gpuAmps];
    set.numQubits = q.numQubits;
    set.dm = false;
    set.phases.push_back({mask, factor});
}

// forgets the pending ops of a Qureg whose state is about to be overwritten or freed
void discardPending(const Qureg& q) {
    std::lock_guard<std::mutex> lock(g_pendingMu);
    g_pending.erase(q.gpuAmps);
}

// S applied after the qubit's pending op: pending = S * pending
void addPending(const Qureg& q, int qubit, const cd (&S)[16], int kind, double p0 = 0, double p1 = 0, double p2 = 0) {
    std::lock_guard<std::mutex> lock(g_pendingMu);
    PendingSet& set = g_pending[q.gpuAmps];
    set.numQubits = q.numQubits;
    set.dm = true;
    auto& ops = set.ops;
    auto it = ops.find(qubit);
    if (it == ops.end()) {
        PendingOp op;
        op.kind = kind;
        op.p[0] = p0; op.p[1] = p1; op.p[2] = p2;
        for (int i = 0; i < 16; i++) op.m[i] = S[i];
        ops[qubit] = op;
        return;
    }
    PendingOp& op = it->second;
    cd prod[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            cd acc = 0;
            for (int k = 0; k < 4; k++) acc += S[r * 4 + k] * op.m[k * 4 + c];
            prod[r * 4 + c] = acc;
        }
    for (int i = 0; i < 16; i++) op.m[i] = prod[i];
    op.kind = PEND_GENERAL;
}

// checks the Qureg and, unless `keepPending`, applies its deferred ops first
bool checkQureg(const Qureg& q, const char* func, bool keepPending = false) {
    if (!checkEnv(func)) return false;
    if (!check(q.gpuAmps != nullptr && q.numQubits >= 1, func, "Invalid Qureg; it was not created, or was destroyed.")) return false;
    return keepPending || flushPending(q, nullptr, func);
}

bool checkQubits(const Qureg& q, const int* qs, int n, const char* func, const char* what) {
    if (!check(n >= 0, func, std::string("Invalid number of ") + what + ".")) return false;
    if (n > 0 && !check(qs != nullptr, func, std::string("Null list of ") + what + ".")) return false;
    for (int i = 0; i < n; i++) {
        if (!check(qs[i] >= 0 && qs[i] < q.numQubits, func,
                   std::string("Invalid ") + what + " index " + std::to_string(qs[i]) + ". Must be >=0 and <" +
                       std::to_string(q.numQubits) + "."))
            return false;
        for (int j = 0; j < i; j++)
            if (!check(qs[i] != qs[j], func, std::string("The ") + what + " contain a duplicate qubit."))
                return false;
    }
    return true;
}

bool checkCtrlsTargs(const Qureg& q, const int* c, int nc, const int* t, int nt, const char* func) {
    if (!checkQubits(q, c, nc, func, "control qubits")) return false;
    if (!checkQubits(q, t, nt, func, "target qubits")) return false;
    for (int i = 0; i < nc; i++)
        for (int j = 0; j < nt; j++)
            if (!check(c[i] != t[j], func, "A control qubit was also a target qubit.")) return false;
    return true;
}

bool checkStates(const int* s, int n, const char* func) {
    if (!s) return true;
    for (int i = 0; i < n; i++)
        if (!check(s[i] == 0 || s[i] == 1, func, "Invalid control-qubit state; must be 0 or 1.")) return false;
    return true;
}

bool isUnitaryDense(const qcomp_t* m, qindex dim) {
    for (qindex r = 0; r < dim; r++)
        for (qindex c = 0; c < dim; c++) {
            cd e = 0;
            for (qindex i = 0; i < dim; i++) e += C(m[r * dim + i]) * std::conj(C(m[c * dim + i]));
            if (std::norm(e - cd(r == c, 0)) > g_eps) return false;
        }
    return true;
}
bool isUnitaryDiag(const qcomp_t* d, qindex dim) {
    for (qindex i = 0; i < dim; i++)
        if (std::abs(std::abs(C(d[i])) - 1) > g_eps) return false;
    return true;
}

vector<int> V(const int* p, int n) { return p ? vector<int>(p, p + n) : vector<int>(); }
vector<int> braOf(const Qureg& q, vector<int> v) { for (auto& x : v) x += q.numQubits; return v; }
const int* P(const vector<int>& v) { return v.empty() ? nullptr : v.data(); }
const int* S(const vector<int>& s) { return s.empty() ? nullptr : s.data(); }

// ------------------------------------------------------------------ dense / diagonal on the Choi or state vector

bool denseSV(const Qureg& q, const vector<int>& c, const vector<int>& s, const vector<int>& t, const qcomp_t* m, bool conj, const char* func) {
    int k = (int)t.size();
    qindex D = (qindex)1 << k;
    if (k <= 2) {
        vector<qcomp_t> mm(m, m + D * D);
        if (conj) for (auto& e : mm) e.im = -e.im;
        if (k == 1) return backend(qg_sv_anyCtrlOneTargDenseMatr(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), t[0], mm.data(), g_stream), func);
        return backend(qg_sv_anyCtrlTwoTargDenseMatr(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), t[0], t[1], mm.data(), g_stream), func);
    }
    return backend(qg_sv_anyCtrlAnyTargDenseMatr(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), t.data(), k, m, conj ? 1 : 0, g_stream), func);
}

// validateAndApplyAnyCtrlAnyTargUnitaryMatrix: operations.cpp:36-63
void applyDense(const Qureg& q, const int* ctrls, const int* states, int nc, const int* targs, int nt, const qcomp_t* m, bool checkUnitary, const char* func) {
    const bool defer = deferSV(q);
    if (!checkQureg(q, func, q.isDensityMatrix != 0 || defer)) return;
    if (!checkCtrlsTargs(q, ctrls, nc, targs, nt, func)) return;
    if (!checkStates(states, nc, func)) return;
    if (!check(nt >= 1, func, "At least one target qubit is required.")) return;
    if (checkUnitary && !check(isUnitaryDense(m, (qindex)1 << nt), func, "The given matrix was not (approximately) unitary.")) return;
    vector<int> c = V(ctrls, nc), s = V(states, nc), t = V(targs, nt);
    if (q.isDensityMatrix && nt == 1 && nc == 0) {
        // U rho U^dagger as one superoperator: U on the ket qubit and conj(U) on its bra
        // partner commute, and together they are the 4x4 operator conj(U) (x) U on the pair
        // (t, t + N) -- the same 16 complex products per 4 amplitudes as the reference's two
        // passes (localiser_statevec_anyCtrlOneTargDenseMatr on the ket, then on the
        // conjugated bra).  It joins the qubit's pending superoperator (applied in one pass).
        cd k[16];
        for (int r1 = 0; r1 < 2; r1++)
            for (int r0 = 0; r0 < 2; r0++)
                for (int c1 = 0; c1 < 2; c1++)
                    for (int c0 = 0; c0 < 2; c0++)
                        k[((r1 << 1) | r0) * 4 + ((c1 << 1) | c0)] = std::conj(C(m[r1 * 2 + c1])) * C(m[r0 * 2 + c0]);
        addPending(q, t[0], k, PEND_GENERAL);
        return;
    }
    if (defer) {
        if (nt == 1 && nc == 0) {
            // pending phases on this qubit come first (a last group of one or two qubits may
            // stay pending: the gate then joins it)
            if (phasePendingOn(q, t[0])) {
                const vector<int> one = {t[0]};
                if (!flushPending(q, &one, func, true)) return;
            }
            const cd U[4] = {C(m[0]), C(m[1]), C(m[2]), C(m[3])};
            addPendingSV(q, t[0], U);
            return;
        }
        vector<int> touched = c;          // other pending qubits commute with this gate
        touched.insert(touched.end(), t.begin(), t.end());
        if (!flushPending(q, &touched, func)) return;
    }
    if (q.isDensityMatrix) {
        if (nt == 2 && nc == 0 && pairSuperops(q)) {
            // U rho U^dagger in one pass: conj(U) (x) U on (t0, t1, t0 + N, t1 + N), the
            // reference's two passes (ket, then conjugated bra) as one superoperator, with
            // the pending superoperators of t0 and t1 multiplied in
            cd M[256];
            for (int j = 0; j < 16; j++)
                for (int k = 0; k < 16; k++)
                    M[j * 16 + k] = C(m[(j & 3) * 4 + (k & 3)]) * std::conj(C(m[(j >> 2) * 4 + (k >> 2)]));
            composePendingPair(q, t[0], t[1], M);
            applyPairOp(q, t[0], t[1], M, func);
            return;
        }
        vector<int> touched = c;
        touched.insert(touched.end(), t.begin(), t.end());
        if (!flushPending(q, &touched, func)) return;
    }
    if (!denseSV(q, c, s, t, m, false, func)) return;
    if (!q.isDensityMatrix) return;
    denseSV(q, braOf(q, c), s, braOf(q, t), m, true, func);
}

bool diagSV(const Qureg& q, const vector<int>& c, const vector<int>& s, const vector<int>& t, const qcomp_t* d, bool conj, const qcomp_t* ex, bool anyTarg, const char* func) {
    int k = (int)t.size();
    if (!anyTarg && !ex && k <= 2) {
        qcomp_t dd[4];
        for (int i = 0; i < (1 << k); i++) dd[i] = qcomp_t{d[i].re, conj ? -d[i].im : d[i].im};
        if (k == 1) return backend(qg_sv_anyCtrlOneTargDiagMatr(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), t[0], dd, g_stream), func);
        return backend(qg_sv_anyCtrlTwoTargDiagMatr(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), t[0], t[1], dd, g_stream), func);
    }
    return backend(qg_sv_anyCtrlAnyTargDiagMatr(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), t.data(), k, d, conj ? 1 : 0, ex, g_stream), func);
}

void applyDiag(const Qureg& q, const int* ctrls, const int* states, int nc, const int* targs, int nt, const qcomp_t* d,
               const qcomp_t* ex, bool anyTarg, const char* func) {
    // a controlled phase (one target, factor 1 on |0>, a factor of modulus 1 on |1>, every
    // control state 1) on a statevector of at least 8 qubits that defers one-qubit gates is
    // deferred too
    bool phase = !q.isDensityMatrix && !ex && !anyTarg && nt == 1 && d[0].re == 1 && d[0].im == 0 &&
                 std::fabs(std::abs(C(d[1])) - 1.0) < 1e-9 && q.numQubits >= 8 && deferSV(q);
    for (int i = 0; phase && states && i < nc; i++) phase = states[i] == 1;
    if (!checkQureg(q, func, phase)) return;
    if (!checkCtrlsTargs(q, ctrls, nc, targs, nt, func)) return;
    if (!checkStates(states, nc, func)) return;
    if (!check(nt >= 1, func, "At least one target qubit is required.")) return;
    if (!check(isUnitaryDiag(d, (qindex)1 << nt), func, "The given matrix was not (approximately) unitary.")) return;
    if (ex && !check(std::abs(ex->im) <= g_eps, func, "The exponent of a unitary diagonal matrix must be real.")) return;
    if (phase) {
        // waits with the other pending phases, after the pending one-qubit ops
        long long mask = 1LL << targs[0];
        for (int i = 0; i < nc; i++) mask |= 1LL << ctrls[i];
        if (!(d[1].re == 1 && d[1].im == 0)) addPendingPhase(q, mask, C(d[1]));
        return;
    }
    vector<int> c = V(ctrls, nc), s = V(states, nc), t = V(targs, nt);
    if (!diagSV(q, c, s, t, d, false, ex, anyTarg, func)) return;
    if (!q.isDensityMatrix) return;
    diagSV(q, braOf(q, c), s, braOf(q, t), d, true, ex, anyTarg, func);
}

// ------------------------------------------------------------------ Pauli strings (paulis.h:53-60)

int pauliAt(const PauliStr& p, int q) {
    return q < 32 ? (int)((p.lowPaulis >> (2 * q)) & 3) : (int)((p.highPaulis >> (2 * (q - 32))) & 3);
}
vector<int> codesOf(const PauliStr& p, int n) { vector<int> v(n); for (int q = 0; q < n; q++) v[q] = pauliAt(p, q); return v; }
bool strFits(const PauliStr& p, int n) {
    for (int q = n; q < 64; q++) if (pauliAt(p, q)) return false;
    return true;
}
void splitXYZ(const vector<int>& codes, vector<int>& x, vector<int>& y, vector<int>& z) {
    for (size_t q = 0; q < codes.size(); q++) {
        if (codes[q] == 1) x.push_back((int)q);
        else if (codes[q] == 2) y.push_back((int)q);
        else if (codes[q] == 3) z.push_back((int)q);
    }
}
int numY(const vector<int>& codes) { int k = 0; for (int v : codes) k += v == 2; return k; }

// localiser_statevec_anyCtrlPauliTensor (localiser.cpp:1319-1339) on codes over the whole vector
bool pauliTensorSV(const Qureg& q, const vector<int>& c, const vector<int>& s, const vector<int>& codes, cd factor, const char* func) {
    vector<int> x, y, z;
    splitXYZ(codes, x, y, z);
    if (!x.empty() || !y.empty())
        return backend(qg_sv_anyCtrlPauliTensorOrGadget(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), P(x), (int)x.size(), P(y), (int)y.size(),
                                                         P(z), (int)z.size(), Q(0.0 * factor), Q(1.0 * factor), g_stream), func);
    return backend(qg_sv_anyCtrlAnyTargZOrPhaseGadget(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), P(z), (int)z.size(),
                                                       qcomp_t{1, 0}, qcomp_t{-1, 0}, g_stream), func);
}

// localiser_statevec_anyCtrlPhaseGadget / PauliGadget (localiser.cpp:1342-1360)
bool phaseGadgetSV(const Qureg& q, const vector<int>& c, const vector<int>& s, const vector<int>& t, double phase, const char* func) {
    cd f0 = std::exp(cd(0, +phase)), f1 = std::exp(cd(0, -phase));
    return backend(qg_sv_anyCtrlAnyTargZOrPhaseGadget(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), P(t), (int)t.size(), Q(f0), Q(f1), g_stream), func);
}
bool pauliGadgetSV(const Qureg& q, const vector<int>& c, const vector<int>& s, const vector<int>& codes, double phase, const char* func) {
    vector<int> x, y, z;
    splitXYZ(codes, x, y, z);
    if (x.empty() && y.empty()) return phaseGadgetSV(q, c, s, z, phase, func);
    cd f0 = std::cos(phase), f1 = std::sin(phase) * cd(0, 1);
    return backend(qg_sv_anyCtrlPauliTensorOrGadget(q.gpuAmps, nsv(q), P(c), S(s), (int)c.size(), P(x), (int)x.size(), P(y), (int)y.size(),
                                                     P(z), (int)z.size(), Q(f0), Q(f1), g_stream), func);
}

vector<int> shiftedCodes(const Qureg& q, const vector<int>& ket) {
    vector<int> v(nsv(q), 0);
    for (int i = 0; i < q.numQubits; i++) v[i + q.numQubits] = ket[i];
    return v;
}
vector<int> paddedCodes(const Qureg& q, const vector<int>& ket) {
    vector<int> v(nsv(q), 0);
    for (int i = 0; i < q.numQubits; i++) v[i] = ket[i];
    return v;
}

bool checkPauliTargs(const Qureg& q, const int* ctrls, int nc, const PauliStr& str, const char* func) {
    if (!check(strFits(str, q.numQubits), func, "The Pauli string targets a qubit beyond the Qureg.")) return false;
    if (!checkQubits(q, ctrls, nc, func, "control qubits")) return false;
    for (int i = 0; i < nc; i++)
        if (!check(pauliAt(str, ctrls[i]) == 0, func, "A control qubit was also a target qubit.")) return false;
    return true;
}

// ------------------------------------------------------------------ probabilities

bool probOf(const Qureg& q, const vector<int>& qs, const vector<int>& os, double* out, const char* func) {
    if (q.isDensityMatrix)
        return backend(qg_dm_calcProbOfMultiQubitOutcome(q.gpuAmps, q.numQubits, P(qs), P(os), (int)qs.size(), out, g_stream), func);
    return backend(qg_sv_calcProbOfMultiQubitOutcome(q.gpuAmps, q.numQubits, P(qs), P(os), (int)qs.size(), out, g_stream), func);
}
bool project(const Qureg& q, const vector<int>& qs, const vector<int>& os, double prob, const char* func) {
    if (q.isDensityMatrix)
        return backend(qg_dm_multiQubitProjector(q.gpuAmps, q.numQubits, P(qs), P(os), (int)qs.size(), prob, g_stream), func);
    return backend(qg_sv_multiQubitProjector(q.gpuAmps, q.numQubits, P(qs), P(os), (int)qs.size(), prob, g_stream), func);
}

bool checkDensMatr(const Qureg& q, const char* func) {
    return check(q.isDensityMatrix, func, "Expected a density matrix Qureg but received a statevector.");
}
bool checkProb(double p, double maxP, const char* func) {
    if (!check(p >= 0 && p <= 1, func, "The given probability is invalid; it must lie in [0, 1].")) return false;
    return check(p <= maxP, func, "The given probability exceeds the maximal mixing of this channel.");
}

}  // namespace

extern "C" {

// ====================================================================== environment

void initQuESTEnv(void) { initCustomQuESTEnv(0, 1, 0); }

void initCustomQuESTEnv(int useDistrib, int useGpuAccel, int useMultithread) {
    (void)useMultithread;
    const char* func = "initCustomQuESTEnv";
    if (!check(!g_envInit, func, "The QuEST environment has already been initialised.")) return;
    if (!check(useDistrib == 0 || useDistrib == -1, func, "This build runs on one GPU; distribution is compiled out.")) return;
    if (!check(useGpuAccel != 0, func, "This build has no CPU backend; GPU acceleration cannot be disabled.")) return;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!backend(qg_init(dev), func)) return;
    std::random_device rd;   // rand_setSeedsToDefault (randomiser.cpp:89-106)
    vector<unsigned> seeds(4);
    for (auto& s : seeds) s = rd();
    std::seed_seq seq(seeds.begin(), seeds.end());
    g_rng.seed(seq);
    g_envInit = true;
}

void finalizeQuESTEnv(void) {
    if (!g_envInit) return;
    qg_sync();
    g_envInit = false;
}

int isQuESTEnvInit(void) { return g_envInit ? 1 : 0; }

void syncQuESTEnv(void) {
    // deferred one-qubit superoperators of every density matrix are applied first
    std::vector<std::pair<const void*, PendingSet>> all;
    {
        std::lock_guard<std::mutex> lock(g_pendingMu);
        for (auto& kv : g_pending) all.push_back(kv);
    }
    for (auto& kv : all) {
        Qureg q;
        std::memset(&q, 0, sizeof(q));
        q.gpuAmps = (qcomp_t*)kv.first;
        q.numQubits = kv.second.numQubits;
        q.isDensityMatrix = kv.second.dm ? 1 : 0;
        if (!flushPending(q, nullptr, "syncQuESTEnv")) return;
    }
    backend(qg_sync(), "syncQuESTEnv");
}

void setInputErrorHandler(void (*callback)(const char*, const char*)) { g_handler = callback ? callback : default_handler; }

void setSeeds(unsigned* seeds, int numSeeds) {
    if (!check(numSeeds > 0 && seeds != nullptr, "setSeeds", "Invalid number of seeds.")) return;
    std::seed_seq seq(seeds, seeds + numSeeds);
    g_rng.seed(seq);
}

void setValidationEpsilon(qreal eps) {
    if (!check(eps >= 0, "setValidationEpsilon", "The validation epsilon must be non-negative.")) return;
    g_eps = eps;
}
void setValidationEpsilonToDefault(void) { g_eps = DEFAULT_EPS; }
void setQuESTStream(void* s) { g_stream = s; }

// ====================================================================== qureg lifecycle

Qureg createCustomQureg(int numQubits, int isDensMatr, int useDistrib, int useGpuAccel, int useMultithread) {
    (void)useMultithread;
    const char* func = "createCustomQureg";
    Qureg q;
    std::memset(&q, 0, sizeof(q));
    if (!checkEnv(func)) return q;
    if (!check(numQubits >= 1, func, "Invalid number of qubits; must be >= 1.")) return q;
    if (!check(useDistrib == 0 || useDistrib == -1, func, "This build runs on one GPU; distribution is compiled out.")) return q;
    if (!check(useGpuAccel != 0, func, "This build has no CPU backend; GPU acceleration cannot be disabled.")) return q;
    int n = isDensMatr ? 2 * numQubits : numQubits;
    if (!check(n <= QG_MAX_QUBITS_API, func, "Too many qubits for one GPU.")) return q;
    qindex numAmps = (qindex)1 << n;
    size_t bytes = sizeof(qcomp_t) * (size_t)numAmps;
    // qureg_populateNonHeapFields (qureg.cpp:37-88), single node
    q.isMultithreaded = 0;
    q.isGpuAccelerated = 1;
    q.isDistributed = 0;
    q.rank = 0;
    q.numNodes = 1;
    q.logNumNodes = 0;
    q.isDensityMatrix = isDensMatr ? 1 : 0;
    q.numQubits = numQubits;
    q.numAmps = numAmps;
    q.logNumAmps = n;
    q.numAmpsPerNode = numAmps;
    q.logNumAmpsPerNode = n;
    q.logNumColsPerNode = isDensMatr ? numQubits : 0;
    void* dev = nullptr;
    int rc = qg_alloc(&dev, (int64_t)bytes);
    if (rc != QG_OK) {
        fail(func, std::string("Could not allocate ") + std::to_string(bytes) + " bytes of GPU memory: " + qg_get_last_error());
        std::memset(&q, 0, sizeof(q));
        return q;
    }
    void* host = nullptr;
    int kind = MIRROR_PINNED;
    if (cudaMallocHost(&host, bytes) != cudaSuccess) {
        // pinned allocation refused (a memlock limit, say): page-lock ordinary memory, and
        // only if that fails too keep a pageable mirror (copies then run through staging)
        cudaGetLastError();
        host = std::calloc(1, bytes);
        kind = MIRROR_PAGEABLE;
        if (host && cudaHostRegister(host, bytes, cudaHostRegisterDefault) == cudaSuccess) kind = MIRROR_REGISTERED;
        else cudaGetLastError();
    }
    if (!host) {
        qg_free(dev);
        fail(func, "Could not allocate the host copy of the amplitudes.");
        std::memset(&q, 0, sizeof(q));
        return q;
    }
    {
        std::lock_guard<std::mutex> lock(g_mirrorMu);
        g_mirrorKind[host] = kind;
    }
    q.gpuAmps = (qcomp_t*)dev;
    q.cpuAmps = (qcomp_t*)host;
    initZeroState(q);
    return q;
}

Qureg createQureg(int numQubits) { return createCustomQureg(numQubits, 0, 0, 1, 0); }
Qureg createDensityQureg(int numQubits) { return createCustomQureg(numQubits, 1, 0, 1, 0); }

Qureg createCloneQureg(Qureg qureg) {
    Qureg q;
    std::memset(&q, 0, sizeof(q));
    if (!checkQureg(qureg, "createCloneQureg")) return q;
    q = createCustomQureg(qureg.numQubits, qureg.isDensityMatrix, 0, 1, 0);
    if (q.gpuAmps) backend(qg_copy_d2d(q.gpuAmps, qureg.gpuAmps, (int64_t)(sizeof(qcomp_t) * qureg.numAmps), g_stream), "createCloneQureg");
    return q;
}

void destroyQureg(Qureg qureg) {
    if (!checkQureg(qureg, "destroyQureg", true)) return;
    discardPending(qureg);
    qg_sync();
    qg_free(qureg.gpuAmps);
    int kind = MIRROR_PINNED;
    {
        std::lock_guard<std::mutex> lock(g_mirrorMu);
        auto it = g_mirrorKind.find(qureg.cpuAmps);
        if (it != g_mirrorKind.end()) {
            kind = it->second;
            g_mirrorKind.erase(it);
        }
    }
    if (kind == MIRROR_PINNED) {
        if (cudaFreeHost(qureg.cpuAmps) != cudaSuccess) cudaGetLastError();
        return;
    }
    if (kind == MIRROR_REGISTERED && cudaHostUnregister(qureg.cpuAmps) != cudaSuccess) cudaGetLastError();
    std::free(qureg.cpuAmps);
}

// 1 if the Qureg's host mirror is page-locked (pinned or registered), so that
// syncQuregToGpu / syncQuregFromGpu copy at the host link's rate; 0 if it is pageable
int isQuregHostMirrorPinned(Qureg qureg) {
    if (!checkQureg(qureg, "isQuregHostMirrorPinned")) return 0;
    std::lock_guard<std::mutex> lock(g_mirrorMu);
    auto it = g_mirrorKind.find(qureg.cpuAmps);
    return it != g_mirrorKind.end() && it->second != MIRROR_PAGEABLE ? 1 : 0;
}

// applies the Qureg's deferred operations now, on the current stream, without waiting
void flushQuregDeferredOps(Qureg q) {
    checkQureg(q, "flushQuregDeferredOps");
}

void syncQuregToGpu(Qureg q) {
    if (!checkQureg(q, "syncQuregToGpu", true)) return;
    discardPending(q);      // the host copy replaces the whole state
    backend(qg_copy_h2d(q.gpuAmps, q.cpuAmps, (int64_t)(sizeof(qcomp_t) * q.numAmps), g_stream), "syncQuregToGpu");
}

void syncQuregFromGpu(Qureg q) {
    if (!checkQureg(q, "syncQuregFromGpu")) return;
    backend(qg_copy_d2h(q.cpuAmps, q.gpuAmps, (int64_t)(sizeof(qcomp_t) * q.numAmps), g_stream), "syncQuregFromGpu");
}

void getQuregAmps(qcomp_t* out, Qureg q, qindex start, qindex num) {
    const char* func = "getQuregAmps";
    if (!checkQureg(q, func)) return;
    if (!check(start >= 0 && num >= 0 && start + num <= q.numAmps, func, "Invalid amplitude range.")) return;
    backend(qg_copy_d2h(out, q.gpuAmps + start, (int64_t)(sizeof(qcomp_t) * num), g_stream), func);
}

qcomp_t getQuregAmp(Qureg q, qindex index) {
    qcomp_t v{0, 0};
    getQuregAmps(&v, q, index, 1);
    return v;
}

// ====================================================================== initialisations

void initZeroState(Qureg q) { initClassicalState(q, 0); }

void initPlusState(Qureg q) {
    const char* func = "initPlusState";
    if (!checkQureg(q, func, true)) return;
    discardPending(q);
    double v = q.isDensityMatrix ? 1.0 / (double)((qindex)1 << q.numQubits) : 1.0 / std::sqrt((double)((qindex)1 << q.numQubits));
    backend(qg_sv_initUniformState(q.gpuAmps, nsv(q), qcomp_t{v, 0}, g_stream), func);
}

void initClassicalState(Qureg q, qindex ind) {
    const char* func = "initClassicalState";
    if (!checkQureg(q, func, true)) return;
    qindex dim = (qindex)1 << q.numQubits;
    if (!check(ind >= 0 && ind < dim, func, "Invalid basis state index.")) return;
    qindex flat = q.isDensityMatrix ? ind * (dim + 1) : ind;
    discardPending(q);
    backend(qg_sv_initClassicalState(q.gpuAmps, nsv(q), flat, g_stream), func);
}

void initDebugState(Qureg q) {
    if (!checkQureg(q, "initDebugState", true)) return;
    discardPending(q);
    backend(qg_sv_initDebugState(q.gpuAmps, nsv(q), g_stream), "initDebugState");
}

void setQuregAmps(Qureg q, qindex start, qcomp_t* amps, qindex num) {
    const char* func = "setQuregAmps";
    if (!checkQureg(q, func, true)) return;
    if (!check(start >= 0 && num >= 0 && start + num <= q.numAmps, func, "Invalid amplitude range.")) return;
    if (start == 0 && num == q.numAmps) discardPending(q);      // every amplitude is overwritten
    else if (!flushPending(q, nullptr, func)) return;
    backend(qg_copy_h2d(q.gpuAmps + start, amps, (int64_t)(sizeof(qcomp_t) * num), g_stream), func);
}

void setDensityQuregFlatAmps(Qureg q, qindex start, qcomp_t* amps, qindex num) {
    const char* func = "setDensityQuregFlatAmps";
    if (!checkQureg(q, func, true) || !checkDensMatr(q, func)) return;
    if (!check(start >= 0 && num >= 0 && start + num <= q.numAmps, func, "Invalid amplitude range.")) return;
    if (start == 0 && num == q.numAmps) discardPending(q);
    else if (!flushPending(q, nullptr, func)) return;
    backend(qg_copy_h2d(q.gpuAmps + start, amps, (int64_t)(sizeof(qcomp_t) * num), g_stream), func);
}

// ====================================================================== matrices and channels

CompMatr createCompMatr(int k) {
    CompMatr m;
    std::memset(&m, 0, sizeof(m));
    if (!check(k >= 1 && k <= 16, "createCompMatr", "Invalid number of qubits for a CompMatr.")) return m;
    qindex D = (qindex)1 << k;
    m.numQubits = k;
    m.numRows = D;
    m.isApproxUnitary = (int*)std::malloc(sizeof(int));
    m.isApproxHermitian = (int*)std::malloc(sizeof(int));
    m.wasGpuSynced = (int*)std::malloc(sizeof(int));
    *m.isApproxUnitary = -1;
    *m.isApproxHermitian = -1;
    *m.wasGpuSynced = 0;
    m.cpuElemsFlat = (qcomp_t*)std::calloc((size_t)(D * D), sizeof(qcomp_t));
    m.cpuElems = (qcomp_t**)std::malloc(sizeof(qcomp_t*) * (size_t)D);
    for (qindex r = 0; r < D; r++) m.cpuElems[r] = m.cpuElemsFlat + r * D;
    m.gpuElemsFlat = nullptr;   // the backend stages dense matrices itself
    return m;
}

void destroyCompMatr(CompMatr m) {
    std::free(m.isApproxUnitary);
    std::free(m.isApproxHermitian);
    std::free(m.wasGpuSynced);
    std::free(m.cpuElems);
    std::free(m.cpuElemsFlat);
}

void syncCompMatr(CompMatr m) {
    *m.wasGpuSynced = 1;
    *m.isApproxUnitary = -1;
}

void setCompMatrFlat(CompMatr m, const qcomp_t* elems) {
    std::memcpy(m.cpuElemsFlat, elems, sizeof(qcomp_t) * (size_t)(m.numRows * m.numRows));
    syncCompMatr(m);
}

DiagMatr createDiagMatr(int k) {
    DiagMatr m;
    std::memset(&m, 0, sizeof(m));
    if (!check(k >= 1 && k <= 30, "createDiagMatr", "Invalid number of qubits for a DiagMatr.")) return m;
    m.numQubits = k;
    m.numElems = (qindex)1 << k;
    int** flags[] = {&m.isApproxUnitary, &m.isApproxHermitian, &m.isApproxNonZero, &m.isStrictlyNonNegative, &m.wasGpuSynced};
    for (auto f : flags) { *f = (int*)std::malloc(sizeof(int)); **f = -1; }
    *m.wasGpuSynced = 0;
    m.cpuElems = (qcomp_t*)std::calloc((size_t)m.numElems, sizeof(qcomp_t));
    m.gpuElems = nullptr;
    return m;
}

void destroyDiagMatr(DiagMatr m) {
    std::free(m.isApproxUnitary);
    std::free(m.isApproxHermitian);
    std::free(m.isApproxNonZero);
    std::free(m.isStrictlyNonNegative);
    std::free(m.wasGpuSynced);
    std::free(m.cpuElems);
}

void syncDiagMatr(DiagMatr m) {
    *m.wasGpuSynced = 1;
    *m.isApproxUnitary = -1;
}

void setDiagMatrFlat(DiagMatr m, const qcomp_t* elems) {
    std::memcpy(m.cpuElems, elems, sizeof(qcomp_t) * (size_t)m.numElems);
    syncDiagMatr(m);
}

KrausMap createKrausMap(int k, int numOps) {
    KrausMap m;
    std::memset(&m, 0, sizeof(m));
    if (!check(k >= 1 && k <= 8 && numOps >= 1, "createKrausMap", "Invalid Kraus map dimensions.")) return m;
    qindex D = (qindex)1 << k, SD = D * D;
    m.numQubits = k;
    m.numMatrices = numOps;
    m.numRows = D;
    m.matrices = (qcomp_t***)std::malloc(sizeof(qcomp_t**) * numOps);
    for (int n = 0; n < numOps; n++) {
        m.matrices[n] = (qcomp_t**)std::malloc(sizeof(qcomp_t*) * (size_t)D);
        for (qindex r = 0; r < D; r++) m.matrices[n][r] = (qcomp_t*)std::calloc((size_t)D, sizeof(qcomp_t));
    }
    m.superop.numQubits = 2 * k;
    m.superop.numRows = SD;
    m.superop.cpuElemsFlat = (qcomp_t*)std::calloc((size_t)(SD * SD), sizeof(qcomp_t));
    m.superop.cpuElems = (qcomp_t**)std::malloc(sizeof(qcomp_t*) * (size_t)SD);
    for (qindex r = 0; r < SD; r++) m.superop.cpuElems[r] = m.superop.cpuElemsFlat + r * SD;
    m.superop.gpuElemsFlat = nullptr;
    m.superop.wasGpuSynced = (int*)std::malloc(sizeof(int));
    *m.superop.wasGpuSynced = 0;
    m.isApproxCPTP = (int*)std::malloc(sizeof(int));
    *m.isApproxCPTP = -1;
    return m;
}

// syncKrausMap: rebuilds the superoperator sum_n conj(K_n) (x) K_n on the host
// (channels.cpp:228-240, util_setSuperoperator utilities.cpp:770-801)
void syncKrausMap(KrausMap m) {
    qindex D = m.numRows, SD = D * D;
    for (qindex i = 0; i < SD * SD; i++) m.superop.cpuElemsFlat[i] = qcomp_t{0, 0};
    for (int n = 0; n < m.numMatrices; n++)
        for (qindex i = 0; i < D; i++)
            for (qindex j = 0; j < D; j++)
                for (qindex k = 0; k < D; k++)
                    for (qindex l = 0; l < D; l++) {
                        qindex r = i * D + k, c = j * D + l;
                        cd v = C(m.superop.cpuElemsFlat[r * SD + c]) + std::conj(C(m.matrices[n][i][j])) * C(m.matrices[n][k][l]);
                        m.superop.cpuElemsFlat[r * SD + c] = Q(v);
                    }
    *m.superop.wasGpuSynced = 1;
    *m.isApproxCPTP = -1;
}

void setKrausMapFlat(KrausMap m, const qcomp_t* ops) {
    qindex D = m.numRows;
    for (int n = 0; n < m.numMatrices; n++)
        for (qindex r = 0; r < D; r++)
            for (qindex c = 0; c < D; c++) m.matrices[n][r][c] = ops[(n * D + r) * D + c];
    syncKrausMap(m);
}

void destroyKrausMap(KrausMap m) {
    for (int n = 0; n < m.numMatrices; n++) {
        for (qindex r = 0; r < m.numRows; r++) std::free(m.matrices[n][r]);
        std::free(m.matrices[n]);
    }
    std::free(m.matrices);
    std::free(m.superop.cpuElems);
    std::free(m.superop.cpuElemsFlat);
    std::free(m.superop.wasGpuSynced);
    std::free(m.isApproxCPTP);
}

PauliStr getPauliStrFromCodes(const int* paulis, const int* indices, int num) {
    PauliStr p{0, 0};
    for (int i = 0; i < num; i++) {
        if (!check(paulis[i] >= 0 && paulis[i] <= 3, "getPauliStr", "Invalid Pauli code; must be 0 (I), 1 (X), 2 (Y) or 3 (Z).")) return PauliStr{0, 0};
        if (!check(indices[i] >= 0 && indices[i] < 64, "getPauliStr", "Invalid Pauli index.")) return PauliStr{0, 0};
        int q = indices[i];
        PAULI_MASK_TYPE code = (PAULI_MASK_TYPE)paulis[i];
        if (q < 32) p.lowPaulis |= code << (2 * q);
        else p.highPaulis |= code << (2 * (q - 32));
    }
    return p;
}

// ====================================================================== operations

void applyCompMatr1(Qureg q, int t, CompMatr1 m) { applyDense(q, nullptr, nullptr, 0, &t, 1, &m.elems[0][0], true, "applyCompMatr1"); }
void applyControlledCompMatr1(Qureg q, int c, int t, CompMatr1 m) { applyDense(q, &c, nullptr, 1, &t, 1, &m.elems[0][0], true, "applyControlledCompMatr1"); }
void applyMultiControlledCompMatr1(Qureg q, int* c, int nc, int t, CompMatr1 m) { applyDense(q, c, nullptr, nc, &t, 1, &m.elems[0][0], true, "applyMultiControlledCompMatr1"); }
void applyMultiStateControlledCompMatr1(Qureg q, int* c, int* s, int nc, int t, CompMatr1 m) { applyDense(q, c, s, nc, &t, 1, &m.elems[0][0], true, "applyMultiStateControlledCompMatr1"); }

void applyCompMatr2(Qureg q, int t1, int t2, CompMatr2 m) { int t[2] = {t1, t2}; applyDense(q, nullptr, nullptr, 0, t, 2, &m.elems[0][0], true, "applyCompMatr2"); }
void applyControlledCompMatr2(Qureg q, int c, int t1, int t2, CompMatr2 m) { int t[2] = {t1, t2}; applyDense(q, &c, nullptr, 1, t, 2, &m.elems[0][0], true, "applyControlledCompMatr2"); }
void applyMultiStateControlledCompMatr2(Qureg q, int* c, int* s, int nc, int t1, int t2, CompMatr2 m) { int t[2] = {t1, t2}; applyDense(q, c, s, nc, t, 2, &m.elems[0][0], true, "applyMultiStateControlledCompMatr2"); }

void applyCompMatr(Qureg q, int* t, int nt, CompMatr m) {
    if (!check(m.cpuElemsFlat && m.numQubits == nt, "applyCompMatr", "The matrix size does not match the number of targets.")) return;
    applyDense(q, nullptr, nullptr, 0, t, nt, m.cpuElemsFlat, true, "applyCompMatr");
}
void applyMultiStateControlledCompMatr(Qureg q, int* c, int* s, int nc, int* t, int nt, CompMatr m) {
    if (!check(m.cpuElemsFlat && m.numQubits == nt, "applyMultiStateControlledCompMatr", "The matrix size does not match the number of targets.")) return;
    applyDense(q, c, s, nc, t, nt, m.cpuElemsFlat, true, "applyMultiStateControlledCompMatr");
}

void applyDiagMatr1(Qureg q, int t, DiagMatr1 m) { applyDiag(q, nullptr, nullptr, 0, &t, 1, m.elems, nullptr, false, "applyDiagMatr1"); }
void applyMultiStateControlledDiagMatr1(Qureg q, int* c, int* s, int nc, int t, DiagMatr1 m) { applyDiag(q, c, s, nc, &t, 1, m.elems, nullptr, false, "applyMultiStateControlledDiagMatr1"); }
void applyDiagMatr2(Qureg q, int t1, int t2, DiagMatr2 m) { int t[2] = {t1, t2}; applyDiag(q, nullptr, nullptr, 0, t, 2, m.elems, nullptr, false, "applyDiagMatr2"); }
void applyMultiStateControlledDiagMatr2(Qureg q, int* c, int* s, int nc, int t1, int t2, DiagMatr2 m) { int t[2] = {t1, t2}; applyDiag(q, c, s, nc, t, 2, m.elems, nullptr, false, "applyMultiStateControlledDiagMatr2"); }
void applyDiagMatr(Qureg q, int* t, int nt, DiagMatr m) {
    if (!check(m.cpuElems && m.numQubits == nt, "applyDiagMatr", "The matrix size does not match the number of targets.")) return;
    applyDiag(q, nullptr, nullptr, 0, t, nt, m.cpuElems, nullptr, true, "applyDiagMatr");
}
void applyMultiStateControlledDiagMatr(Qureg q, int* c, int* s, int nc, int* t, int nt, DiagMatr m) {
    if (!check(m.cpuElems && m.numQubits == nt, "applyMultiStateControlledDiagMatr", "The matrix size does not match the number of targets.")) return;
    applyDiag(q, c, s, nc, t, nt, m.cpuElems, nullptr, true, "applyMultiStateControlledDiagMatr");
}
void applyDiagMatrPower(Qureg q, int* t, int nt, DiagMatr m, qcomp_t ex) {
    if (!check(m.cpuElems && m.numQubits == nt, "applyDiagMatrPower", "The matrix size does not match the number of targets.")) return;
    applyDiag(q, nullptr, nullptr, 0, t, nt, m.cpuElems, &ex, true, "applyDiagMatrPower");
}
void applyMultiStateControlledDiagMatrPower(Qureg q, int* c, int* s, int nc, int* t, int nt, DiagMatr m, qcomp_t ex) {
    if (!check(m.cpuElems && m.numQubits == nt, "applyMultiStateControlledDiagMatrPower", "The matrix size does not match the number of targets.")) return;
    applyDiag(q, c, s, nc, t, nt, m.cpuElems, &ex, true, "applyMultiStateControlledDiagMatrPower");
}

// S = diag(1, i) (operations.cpp:614-618); T = diag(1, 1/sqrt2 + i/sqrt2) (:665-669)
void applyS(Qureg q, int t) { qcomp_t d[2] = {{1, 0}, {0, 1}}; applyDiag(q, nullptr, nullptr, 0, &t, 1, d, nullptr, false, "applyS"); }
void applyT(Qureg q, int t) { double r = 1 / std::sqrt(2); qcomp_t d[2] = {{1, 0}, {r, r}}; applyDiag(q, nullptr, nullptr, 0, &t, 1, d, nullptr, false, "applyT"); }

// operations.cpp:716-723: a = 1/sqrt(2)
void applyMultiStateControlledHadamard(Qureg q, int* c, int* s, int nc, int t) {
    double a = 1 / std::sqrt(2);
    qcomp_t m[4] = {{a, 0}, {a, 0}, {a, 0}, {-a, 0}};
    applyDense(q, c, s, nc, &t, 1, m, false, "applyHadamard");
}
void applyHadamard(Qureg q, int t) { applyMultiStateControlledHadamard(q, nullptr, nullptr, 0, t); }

// operations.cpp:778-796
void applyMultiStateControlledSwap(Qureg q, int* c, int* s, int nc, int a, int b) {
    const char* func = "applySwap";
    if (!checkQureg(q, func)) return;
    int t[2] = {a, b};
    if (!checkCtrlsTargs(q, c, nc, t, 2, func) || !checkStates(s, nc, func)) return;
    vector<int> cv = V(c, nc), sv = V(s, nc);
    if (!backend(qg_sv_anyCtrlSwap(q.gpuAmps, nsv(q), P(cv), S(sv), nc, a, b, g_stream), func)) return;
    if (!q.isDensityMatrix) return;
    vector<int> bc = braOf(q, cv);
    backend(qg_sv_anyCtrlSwap(q.gpuAmps, nsv(q), P(bc), S(sv), nc, a + q.numQubits, b + q.numQubits, g_stream), func);
}
void applySwap(Qureg q, int a, int b) { applyMultiStateControlledSwap(q, nullptr, nullptr, 0, a, b); }

// applyMultiStateControlledPauliStr: operations.cpp:1061-1090
void applyMultiStateControlledPauliStr(Qureg q, int* c, int* s, int nc, PauliStr str) {
    const char* func = "applyPauliStr";
    if (!checkQureg(q, func) || !checkPauliTargs(q, c, nc, str, func) || !checkStates(s, nc, func)) return;
    vector<int> cv = V(c, nc), sv = V(s, nc);
    vector<int> ket = codesOf(str, q.numQubits);
    bool oddY = numY(ket) % 2;
    if (q.isDensityMatrix && nc == 0) {
        vector<int> both = paddedCodes(q, ket), sh = shiftedCodes(q, ket);
        for (size_t i = 0; i < both.size(); i++) both[i] |= sh[i];
        pauliTensorSV(q, cv, sv, both, oddY ? -1.0 : 1.0, func);
        return;
    }
    if (!pauliTensorSV(q, cv, sv, q.isDensityMatrix ? paddedCodes(q, ket) : ket, 1.0, func)) return;
    if (q.isDensityMatrix) pauliTensorSV(q, braOf(q, cv), sv, shiftedCodes(q, ket), oddY ? -1.0 : 1.0, func);
}
void applyPauliStr(Qureg q, PauliStr str) { applyMultiStateControlledPauliStr(q, nullptr, nullptr, 0, str); }

void applyPauliX(Qureg q, int t) {
    if (!checkQureg(q, "applyPauliX") || !checkQubits(q, &t, 1, "applyPauliX", "target qubits")) return;
    int code = 1; applyPauliStr(q, getPauliStrFromCodes(&code, &t, 1));
}
void applyPauliY(Qureg q, int t) {
    if (!checkQureg(q, "applyPauliY") || !checkQubits(q, &t, 1, "applyPauliY", "target qubits")) return;
    int code = 2; applyPauliStr(q, getPauliStrFromCodes(&code, &t, 1));
}
// Z = DiagMatr1 {1, -1} (operations.cpp:977-985)
void applyPauliZ(Qureg q, int t) { qcomp_t d[2] = {{1, 0}, {-1, 0}}; applyDiag(q, nullptr, nullptr, 0, &t, 1, d, nullptr, false, "applyPauliZ"); }
void applyControlledPauliX(Qureg q, int c, int t) {
    if (!checkQureg(q, "applyControlledPauliX") || !checkCtrlsTargs(q, &c, 1, &t, 1, "applyControlledPauliX")) return;
    int code = 1; applyMultiStateControlledPauliStr(q, &c, nullptr, 1, getPauliStrFromCodes(&code, &t, 1));
}
void applyControlledPauliZ(Qureg q, int c, int t) { qcomp_t d[2] = {{1, 0}, {-1, 0}}; applyDiag(q, &c, nullptr, 1, &t, 1, d, nullptr, false, "applyControlledPauliZ"); }

// applyMultiStateControlledPauliGadget: operations.cpp:1449-1476 (phase = -angle/2, utilities.cpp:911-914)
void applyMultiStateControlledPauliGadget(Qureg q, int* c, int* s, int nc, PauliStr str, qreal angle) {
    const char* func = "applyPauliGadget";
    if (!checkQureg(q, func) || !checkPauliTargs(q, c, nc, str, func) || !checkStates(s, nc, func)) return;
    vector<int> ket = codesOf(str, q.numQubits);
    bool isId = std::all_of(ket.begin(), ket.end(), [](int v) { return v == 0; });
    if (isId && nc == 0 && q.isDensityMatrix) return;
    double phase = -angle / 2;
    vector<int> cv = V(c, nc), sv = V(s, nc);
    if (!pauliGadgetSV(q, cv, sv, q.isDensityMatrix ? paddedCodes(q, ket) : ket, phase, func)) return;
    if (!q.isDensityMatrix) return;
    phase *= (numY(ket) % 2) ? 1 : -1;
    pauliGadgetSV(q, braOf(q, cv), sv, shiftedCodes(q, ket), phase, func);
}
void applyPauliGadget(Qureg q, PauliStr str, qreal angle) { applyMultiStateControlledPauliGadget(q, nullptr, nullptr, 0, str, angle); }

// A one-target rotation exp(-i angle/2 P) (operations.cpp:1283-1310: a Pauli gadget) as its
// 2x2 unitary through applyDense where one-qubit gates are deferred -- statevectors that
// defer them, and density matrices -- so that it joins the qubit's pending unitary (or
// superoperator) instead of taking a pass of its own.  False where the gadget applies.
bool rotationDeferred(const Qureg& q, int t, qreal a, int pauli, const char* func) {
    if (!(q.isDensityMatrix ? q.gpuAmps != nullptr : deferSV(q))) return false;
    const double c = std::cos(a / 2), s = std::sin(a / 2);
    qcomp_t m[4];
    if (pauli == 1) { m[0] = {c, 0}; m[1] = {0, -s}; m[2] = {0, -s}; m[3] = {c, 0}; }
    else if (pauli == 2) { m[0] = {c, 0}; m[1] = {-s, 0}; m[2] = {s, 0}; m[3] = {c, 0}; }
    else { m[0] = {c, -s}; m[1] = {0, 0}; m[2] = {0, 0}; m[3] = {c, s}; }
    applyDense(q, nullptr, nullptr, 0, &t, 1, m, false, func);
    return true;
}
void applyRotateX(Qureg q, int t, qreal a) { if (rotationDeferred(q, t, a, 1, "applyRotateX")) return; if (!checkQureg(q, "applyRotateX") || !checkQubits(q, &t, 1, "applyRotateX", "target qubits")) return; int p = 1; applyPauliGadget(q, getPauliStrFromCodes(&p, &t, 1), a); }
void applyRotateY(Qureg q, int t, qreal a) { if (rotationDeferred(q, t, a, 2, "applyRotateY")) return; if (!checkQureg(q, "applyRotateY") || !checkQubits(q, &t, 1, "applyRotateY", "target qubits")) return; int p = 2; applyPauliGadget(q, getPauliStrFromCodes(&p, &t, 1), a); }
void applyRotateZ(Qureg q, int t, qreal a) { if (rotationDeferred(q, t, a, 3, "applyRotateZ")) return; if (!checkQureg(q, "applyRotateZ") || !checkQubits(q, &t, 1, "applyRotateZ", "target qubits")) return; int p = 3; applyPauliGadget(q, getPauliStrFromCodes(&p, &t, 1), a); }
void applyControlledRotateX(Qureg q, int c, int t, qreal a) { if (!checkQureg(q, "applyControlledRotateX") || !checkCtrlsTargs(q, &c, 1, &t, 1, "applyControlledRotateX")) return; int p = 1; applyMultiStateControlledPauliGadget(q, &c, nullptr, 1, getPauliStrFromCodes(&p, &t, 1), a); }
void applyControlledRotateY(Qureg q, int c, int t, qreal a) { if (!checkQureg(q, "applyControlledRotateY") || !checkCtrlsTargs(q, &c, 1, &t, 1, "applyControlledRotateY")) return; int p = 2; applyMultiStateControlledPauliGadget(q, &c, nullptr, 1, getPauliStrFromCodes(&p, &t, 1), a); }
void applyControlledRotateZ(Qureg q, int c, int t, qreal a) { if (!checkQureg(q, "applyControlledRotateZ") || !checkCtrlsTargs(q, &c, 1, &t, 1, "applyControlledRotateZ")) return; int p = 3; applyMultiStateControlledPauliGadget(q, &c, nullptr, 1, getPauliStrFromCodes(&p, &t, 1), a); }

// applyMultiStateControlledPhaseGadget: operations.cpp:1532-1549
void applyMultiStateControlledPhaseGadget(Qureg q, int* c, int* s, int nc, int* t, int nt, qreal angle) {
    const char* func = "applyPhaseGadget";
    if (!checkQureg(q, func) || !checkCtrlsTargs(q, c, nc, t, nt, func) || !checkStates(s, nc, func)) return;
    double phase = -angle / 2;
    vector<int> cv = V(c, nc), sv = V(s, nc), tv = V(t, nt);
    if (!phaseGadgetSV(q, cv, sv, tv, phase, func)) return;
    if (!q.isDensityMatrix) return;
    phaseGadgetSV(q, braOf(q, cv), sv, braOf(q, tv), -phase, func);
}
void applyPhaseGadget(Qureg q, int* t, int nt, qreal angle) { applyMultiStateControlledPhaseGadget(q, nullptr, nullptr, 0, t, nt, angle); }

// applyMultiQubitPhaseShift: a (n-1)-controlled DiagMatr1 {1, e^(i angle)} (operations.cpp:1605-1613)
void applyMultiQubitPhaseShift(Qureg q, int* t, int nt, qreal angle) {
    const char* func = "applyMultiQubitPhaseShift";
    if (!checkQureg(q, func, true) || !checkQubits(q, t, nt, func, "target qubits")) return;
    if (!check(nt >= 1, func, "At least one target qubit is required.")) return;
    cd e = std::exp(cd(0, 1) * angle);
    qcomp_t d[2] = {{1, 0}, Q(e)};
    applyDiag(q, t + 1, nullptr, nt - 1, &t[0], 1, d, nullptr, false, func);
}
void applyPhaseShift(Qureg q, int t, qreal a) { applyMultiQubitPhaseShift(q, &t, 1, a); }
void applyTwoQubitPhaseShift(Qureg q, int t1, int t2, qreal a) { int t[2] = {t1, t2}; applyMultiQubitPhaseShift(q, t, 2, a); }
void applyPhaseFlip(Qureg q, int t) { qcomp_t d[2] = {{1, 0}, {-1, 0}}; applyDiag(q, nullptr, nullptr, 0, &t, 1, d, nullptr, false, "applyPhaseFlip"); }
void applyTwoQubitPhaseFlip(Qureg q, int t1, int t2) { qcomp_t d[2] = {{1, 0}, {-1, 0}}; applyDiag(q, &t2, nullptr, 1, &t1, 1, d, nullptr, false, "applyTwoQubitPhaseFlip"); }

// applyQuantumFourierTransform: operations.cpp:1934-1952
void applyQuantumFourierTransform(Qureg q, int* t, int nt) {
    const char* func = "applyQuantumFourierTransform";
    if (!checkQureg(q, func) || !checkQubits(q, t, nt, func, "target qubits")) return;
    bool contiguous = true;
    for (int j = 1; j < nt; j++) contiguous = contiguous && t[j] == t[0] + j;
    if (!q.isDensityMatrix && contiguous && qg_fp64_products_mode() == 0) {
        // each step (Hadamard on t[n], then its n controlled phases) as one pass, or for
        // targets from qubit 0 three steps per pass (two where three do not fit: the pass
        // of three takes targets 2..8 and 10..40); their closing swaps as one permutation
        for (int n = nt - 1; n >= 0; n--) {
            if (t[0] == 0 && n >= 2 && n != 9) {
                if (!backend(qg_sv_qftThreeSteps(q.gpuAmps, q.numQubits, t[n], g_stream), func)) return;
                n -= 2;
                continue;
            }
            if (t[0] == 0 && n >= 1) {
                if (!backend(qg_sv_qftTwoSteps(q.gpuAmps, q.numQubits, t[n], g_stream), func)) return;
                n--;
                continue;
            }
            if (!backend(qg_sv_qftStep(q.gpuAmps, q.numQubits, t[n], t[0], n, g_stream), func)) return;
        }
        if (t[0] == 0 && nt >= 10) {
            backend(qg_sv_reverseLowBits(q.gpuAmps, q.numQubits, nt, g_stream), func);
            return;
        }
        for (int n = 0; n < nt / 2; n++) applySwap(q, t[n], t[nt - 1 - n]);
        return;
    }
    const double PI = 3.141592653589793238462643383279502884;
    for (int n = nt - 1; n >= 0; n--) {
        applyHadamard(q, t[n]);
        for (int m = 0; m < n; m++) {
            double arg = PI / (double)((qindex)1 << (m + 1));
            applyTwoQubitPhaseShift(q, t[n], t[n - m - 1], arg);
        }
    }
    for (int n = 0; n < nt / 2; n++) applySwap(q, t[n], t[nt - 1 - n]);
}
void applyFullQuantumFourierTransform(Qureg q) {
    if (!checkQureg(q, "applyFullQuantumFourierTransform")) return;
    vector<int> t(q.numQubits);
    for (int i = 0; i < q.numQubits; i++) t[i] = i;
    applyQuantumFourierTransform(q, t.data(), (int)t.size());
}

// projectors and measurement: operations.cpp:1754-1826, localiser.cpp:2295-2322
void applyMultiQubitProjector(Qureg q, int* qs, int* os, int n) {
    const char* func = "applyMultiQubitProjector";
    if (!checkQureg(q, func) || !checkQubits(q, qs, n, func, "target qubits")) return;
    for (int i = 0; i < n; i++)
        if (!check(os[i] == 0 || os[i] == 1, func, "Invalid measurement outcome; must be 0 or 1.")) return;
    project(q, V(qs, n), V(os, n), 1.0, func);
}
void applyQubitProjector(Qureg q, int t, int o) { applyMultiQubitProjector(q, &t, &o, 1); }

int applyQubitMeasurementAndGetProb(Qureg q, int t, qreal* probability) {
    const char* func = "applyQubitMeasurement";
    if (!checkQureg(q, func) || !checkQubits(q, &t, 1, func, "target qubits")) return -1;
    double p[2];
    if (!probOf(q, {t}, {0}, &p[0], func) || !probOf(q, {t}, {1}, &p[1], func)) return -1;
    if (!check(std::abs(p[0] + p[1] - 1) <= g_eps, func, "The outcome probabilities do not sum to one; the state is not normalised.")) return -1;
    std::uniform_real_distribution<double> distrib(0, 1);
    double sample = distrib(g_rng);
    int outcome = sample > p[0];
    if (probability) *probability = p[outcome];
    project(q, {t}, {outcome}, p[outcome], func);
    return outcome;
}
int applyQubitMeasurement(Qureg q, int t) { qreal p = 0; return applyQubitMeasurementAndGetProb(q, t, &p); }

// applyMultiQubitMeasurementAndGetProb: operations.cpp:1858-1891.  Every outcome's
// probability (one deterministic histogram pass), a Kahan-summed normalisation check
// (util_getSum, utilities.cpp:346-360), one uniform sample walked along the cumulative
// probabilities (rand_getRandomMultiQubitOutcome, randomiser.cpp:140-166), then the
// projector onto the outcome's bits (bit i of the outcome for qubits[i]).
qindex applyMultiQubitMeasurementAndGetProb(Qureg q, int* qs, int n, qreal* probability) {
    const char* func = "applyMultiQubitMeasurementAndGetProb";
    if (!checkQureg(q, func) || !checkQubits(q, qs, n, func, "target qubits")) return -1;
    if (!check(n >= 1 && n <= 20, func, "This build measures at most 20 qubits at once.")) return -1;
    vector<double> probs((size_t)1 << n);
    calcProbsOfAllMultiQubitOutcomes(probs.data(), q, qs, n);
    double total = 0, comp = 0;
    for (double x : probs) { double y = x - comp, t = total + y; comp = (t - total) - y; total = t; }
    if (!check(std::abs(total - 1) <= g_eps, func, "The outcome probabilities do not sum to one; the state is not normalised.")) return -1;
    std::uniform_real_distribution<double> distrib(0, 1);
    double sample = distrib(g_rng), cum = 0;
    qindex outcome = (qindex)probs.size();
    for (size_t i = 0; i < probs.size(); i++) {
        cum += probs[i];
        if (sample < cum) { outcome = (qindex)i; break; }
    }
    if (outcome == (qindex)probs.size()) {
        if (!check(1 - cum <= g_eps, func, "The outcome probabilities are not normalised.")) return -1;
        outcome = (qindex)probs.size() - 1;
    }
    vector<int> qv(qs, qs + n), ov(n);
    for (int i = 0; i < n; i++) ov[i] = (int)((outcome >> i) & 1);
    if (probability) *probability = probs[(size_t)outcome];
    project(q, qv, ov, probs[(size_t)outcome], func);
    return outcome;
}
qindex applyMultiQubitMeasurement(Qureg q, int* qs, int n) { qreal p = 0; return applyMultiQubitMeasurementAndGetProb(q, qs, n, &p); }

// applyForcedMultiQubitMeasurement: operations.cpp:1893-1912 (the outcome's probability must
// be at least epsilon; the state is projected and renormalised by it)
qreal applyForcedMultiQubitMeasurement(Qureg q, int* qs, int* os, int n) {
    const char* func = "applyForcedMultiQubitMeasurement";
    if (!checkQureg(q, func) || !checkQubits(q, qs, n, func, "target qubits")) return 0;
    for (int i = 0; i < n; i++)
        if (!check(os[i] == 0 || os[i] == 1, func, "Invalid measurement outcome; must be 0 or 1.")) return 0;
    double p = 0;
    if (!probOf(q, V(qs, n), V(os, n), &p, func)) return 0;
    if (!check(p >= g_eps, func, "The forced measurement outcome is impossibly unlikely.")) return 0;
    project(q, V(qs, n), V(os, n), p, func);
    return p;
}
// applyForcedQubitMeasurement: operations.cpp:1829-1846
qreal applyForcedQubitMeasurement(Qureg q, int t, int o) {
    const char* func = "applyForcedQubitMeasurement";
    if (!checkQureg(q, func) || !checkQubits(q, &t, 1, func, "target qubits")) return 0;
    if (!check(o == 0 || o == 1, func, "Invalid measurement outcome; must be 0 or 1.")) return 0;
    double p = 0;
    if (!probOf(q, {t}, {o}, &p, func)) return 0;
    if (!check(p >= g_eps, func, "The forced measurement outcome is impossibly unlikely.")) return 0;
    project(q, {t}, {o}, p, func);
    return p;
}

// ====================================================================== decoherence (decoherence.cpp:31-131)

// The one-qubit channels join the qubit's pending superoperator (index bit 0 = ket,
// bit 1 = bra); their factors are those of the reference's kernels
// (utilities.cpp:916-990, cpu_subroutines.cpp:1060-1600).
void mixDephasing(Qureg q, int qubit, qreal prob) {
    const char* func = "mixDephasing";
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkQubits(q, &qubit, 1, func, "target qubits") || !checkProb(prob, 0.5, func)) return;
    if (prob == 0) return;
    if (!checkDensMatr(q, func)) return;
    const double f = 1 - 2 * prob;    // util_getOneQubitDephasingFactor (utilities.cpp:918-921)
    cd S[16] = {};
    S[0] = 1; S[5] = f; S[10] = f; S[15] = 1;
    addPending(q, qubit, S, PEND_DEPHASE, prob);
}
void mixTwoQubitDephasing(Qureg q, int a, int b, qreal prob) {
    const char* func = "mixTwoQubitDephasing";
    int t[2] = {a, b};
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkQubits(q, t, 2, func, "target qubits") || !checkProb(prob, 0.75, func)) return;
    if (prob == 0) return;
    if (!checkDensMatr(q, func)) return;
    vector<int> touched = {a, b};
    if (!flushPending(q, &touched, func)) return;
    backend(qg_dm_twoQubitDephasing(q.gpuAmps, q.numQubits, a, b, prob, g_stream), func);
}
void mixDepolarising(Qureg q, int qubit, qreal prob) {
    const char* func = "mixDepolarising";
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkQubits(q, &qubit, 1, func, "target qubits") || !checkProb(prob, 0.75, func)) return;
    if (prob == 0) return;
    if (!checkDensMatr(q, func)) return;
    // util_getOneQubitDepolarisingFactors (utilities.cpp:932-947)
    const double c1 = 1 - 2 * prob / 3, c2 = 2 * prob / 3, c3 = 1 - 4 * prob / 3;
    cd S[16] = {};
    S[0] = c1; S[3] = c2; S[5] = c3; S[10] = c3; S[12] = c2; S[15] = c1;
    addPending(q, qubit, S, PEND_DEPOL, prob);
}
void mixTwoQubitDepolarising(Qureg q, int a, int b, qreal prob) {
    const char* func = "mixTwoQubitDepolarising";
    int t[2] = {a, b};
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkQubits(q, t, 2, func, "target qubits") || !checkProb(prob, 15.0 / 16, func)) return;
    if (prob == 0) return;
    if (!checkDensMatr(q, func)) return;
    vector<int> touched = {a, b};
    if (!flushPending(q, &touched, func)) return;
    backend(qg_dm_twoQubitDepolarising(q.gpuAmps, q.numQubits, a, b, prob, g_stream), func);
}
void mixDamping(Qureg q, int qubit, qreal prob) {
    const char* func = "mixDamping";
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkQubits(q, &qubit, 1, func, "target qubits") || !checkProb(prob, 1.0, func)) return;
    if (prob == 0) return;
    if (!checkDensMatr(q, func)) return;
    const double c1 = std::sqrt(1 - prob), c2 = 1 - prob;   // util_getOneQubitDampingFactors (utilities.cpp:977-988)
    cd S[16] = {};
    S[0] = 1; S[3] = prob; S[5] = c1; S[10] = c1; S[15] = c2;
    addPending(q, qubit, S, PEND_DAMP, prob);
}
void mixPaulis(Qureg q, int qubit, qreal px, qreal py, qreal pz) {
    const char* func = "mixPaulis";
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkQubits(q, &qubit, 1, func, "target qubits")) return;
    if (!checkProb(px, 1, func) || !checkProb(py, 1, func) || !checkProb(pz, 1, func)) return;
    if (px == 0 && py == 0 && pz == 0) return;
    if (!checkDensMatr(q, func)) return;
    // util_getOneQubitPauliChannelFactors (utilities.cpp:962-975)
    const double pI = 1 - px - py - pz;
    const double fAA = pI + pz, fBB = px + py, fAB = pI - pz, fBA = px - py;
    cd S[16] = {};
    S[0] = fAA; S[3] = fBB; S[5] = fAB; S[6] = fBA; S[9] = fBA; S[10] = fAB; S[12] = fBB; S[15] = fAA;
    addPending(q, qubit, S, PEND_PAULIS, px, py, pz);
}

// mixKrausMap: the superoperator as a dense matrix on targets {ket..., bra...}
// (localiser_densmatr_superoperator, localiser.cpp:1670-1686), not conjugated
void mixKrausMap(Qureg q, int* qubits, int n, KrausMap map) {
    const char* func = "mixKrausMap";
    if (!checkQureg(q, func, q.isDensityMatrix != 0) || !checkDensMatr(q, func) || !checkQubits(q, qubits, n, func, "target qubits")) return;
    if (!check(map.numQubits == n && map.superop.cpuElemsFlat, func, "The Kraus map size does not match the number of targets.")) return;
    // util_isCPTP (utilities.cpp:729-768): sum_n K_n^dagger K_n = I within eps (squared distance)
    if (*map.isApproxCPTP == -1) {
        int ok = 1;
        for (qindex r = 0; r < map.numRows && ok; r++)
            for (qindex c = 0; c < map.numRows && ok; c++) {
                cd e = 0;
                for (int k = 0; k < map.numMatrices; k++)
                    for (qindex i = 0; i < map.numRows; i++) e += std::conj(C(map.matrices[k][i][r])) * C(map.matrices[k][i][c]);
                if (std::norm(e - cd(r == c, 0)) > g_eps) ok = 0;
            }
        *map.isApproxCPTP = ok;
    }
    if (!check(*map.isApproxCPTP == 1, func, "The Kraus map is not (approximately) completely positive and trace preserving.")) return;
    if (n == 1) {
        // a one-qubit map joins the qubit's pending superoperator
        cd S[16];
        for (int i = 0; i < 16; i++) S[i] = C(map.superop.cpuElemsFlat[i]);
        addPending(q, qubits[0], S, PEND_GENERAL);
        return;
    }
    if (n == 2 && pairSuperops(q)) {
        // the superoperator with the pending superoperators of its two qubits multiplied in
        cd M[256];
        for (int i = 0; i < 256; i++) M[i] = C(map.superop.cpuElemsFlat[i]);
        composePendingPair(q, qubits[0], qubits[1], M);
        applyPairOp(q, qubits[0], qubits[1], M, func);
        return;
    }
    vector<int> touched(qubits, qubits + n);
    if (!flushPending(q, &touched, func)) return;
    vector<int> t(qubits, qubits + n);
    for (int i = 0; i < n; i++) t.push_back(qubits[i] + q.numQubits);
    denseSV(q, {}, {}, t, map.superop.cpuElemsFlat, false, func);
}

// ====================================================================== calculations

qreal calcTotalProb(Qureg q) {
    const char* func = "calcTotalProb";
    if (!checkQureg(q, func)) return 0;
    double v = 0;
    if (q.isDensityMatrix) backend(qg_dm_calcTotalProb(q.gpuAmps, q.numQubits, &v, g_stream), func);
    else backend(qg_sv_calcTotalProb(q.gpuAmps, q.numQubits, &v, g_stream), func);
    return v;
}

// calcPurity: calculations.cpp:293-300
qreal calcPurity(Qureg q) {
    const char* func = "calcPurity";
    if (!checkQureg(q, func)) return 0;
    double v = 0;
    backend(qg_sv_calcTotalProb(q.gpuAmps, nsv(q), &v, g_stream), func);
    return q.isDensityMatrix ? v : v * v;
}

// ---------------------------------------------------------------- FullStateDiagMatr
// createFullStateDiagMatr / setFullStateDiagMatr / syncFullStateDiagMatr: matrices.cpp;
// the GPU copy is made at creation and refreshed by every set or sync.

FullStateDiagMatr createFullStateDiagMatr(int k) {
    const char* func = "createFullStateDiagMatr";
    FullStateDiagMatr m;
    std::memset(&m, 0, sizeof(m));
    if (!check(k >= 1 && k <= 33, func, "Invalid number of qubits for a FullStateDiagMatr.")) return m;
    m.numQubits = k;
    m.numElems = (qindex)1 << k;
    m.numElemsPerNode = m.numElems;
    m.isGpuAccelerated = 1;
    int** flags[] = {&m.isApproxUnitary, &m.isApproxHermitian, &m.isApproxNonZero, &m.isStrictlyNonNegative, &m.wasGpuSynced};
    for (auto f : flags) { *f = (int*)std::malloc(sizeof(int)); **f = -1; }
    *m.wasGpuSynced = 0;
    m.cpuElems = (qcomp_t*)std::calloc((size_t)m.numElems, sizeof(qcomp_t));
    void* g = nullptr;
    if (!backend(qg_alloc(&g, (int64_t)sizeof(qcomp_t) * m.numElems), func)) return m;
    m.gpuElems = (qcomp_t*)g;
    backend(qg_copy_h2d(m.gpuElems, m.cpuElems, (int64_t)sizeof(qcomp_t) * m.numElems, nullptr), func);
    return m;
}

void destroyFullStateDiagMatr(FullStateDiagMatr m) {
    int* flags[] = {m.isApproxUnitary, m.isApproxHermitian, m.isApproxNonZero, m.isStrictlyNonNegative, m.wasGpuSynced};
    for (auto f : flags) std::free(f);
    std::free(m.cpuElems);
    if (m.gpuElems) qg_free(m.gpuElems);
}

void syncFullStateDiagMatr(FullStateDiagMatr m) {
    const char* func = "syncFullStateDiagMatr";
    if (!check(m.cpuElems && m.gpuElems, func, "The FullStateDiagMatr was not created.")) return;
    backend(qg_copy_h2d(m.gpuElems, m.cpuElems, (int64_t)sizeof(qcomp_t) * m.numElems, nullptr), func);
    *m.wasGpuSynced = 1;
    *m.isApproxUnitary = *m.isApproxHermitian = *m.isApproxNonZero = *m.isStrictlyNonNegative = -1;
}

void setFullStateDiagMatr(FullStateDiagMatr m, qindex start, const qcomp_t* in, qindex num) {
    const char* func = "setFullStateDiagMatr";
    if (!check(m.cpuElems && m.gpuElems, func, "The FullStateDiagMatr was not created.")) return;
    if (!check(start >= 0 && num >= 0 && start + num <= m.numElems, func,
               "The start index and number of elements exceed the matrix's elements.")) return;
    std::memcpy(m.cpuElems + start, in, sizeof(qcomp_t) * (size_t)num);
    backend(qg_copy_h2d(m.gpuElems + start, in, (int64_t)sizeof(qcomp_t) * num, nullptr), func);
    *m.wasGpuSynced = 1;
    *m.isApproxUnitary = *m.isApproxHermitian = *m.isApproxNonZero = *m.isStrictlyNonNegative = -1;
}

namespace {

// validate_matrixFields + validate_matrixAndQuregAreCompatible (validation.cpp)
bool fsdCompatible(const Qureg& q, const FullStateDiagMatr& m, const char* func) {
    if (!checkQureg(q, func)) return false;
    if (!check(m.cpuElems && m.gpuElems, func, "The FullStateDiagMatr was not created.")) return false;
    return check(m.numQubits == q.numQubits, func,
                 "The FullStateDiagMatr has a different number of qubits than the Qureg.");
}

// every |d_i|^2 within epsilon of 1 (the diagonal of a unitary)
bool fsdUnitary(const FullStateDiagMatr& m, const char* func) {
    if (*m.isApproxUnitary == -1) {
        int ok = 1;
        for (qindex i = 0; i < m.numElems && ok; i++) ok = std::abs(std::norm(C(m.cpuElems[i])) - 1) <= g_eps;
        *m.isApproxUnitary = ok;
    }
    return check(*m.isApproxUnitary == 1, func, "The given matrix was not (approximately) unitary.");
}

bool fsdHermitian(const FullStateDiagMatr& m, const char* func) {
    if (*m.isApproxHermitian == -1) {
        int ok = 1;
        for (qindex i = 0; i < m.numElems && ok; i++) ok = std::abs(m.cpuElems[i].im) <= g_eps;
        *m.isApproxHermitian = ok;
    }
    return check(*m.isApproxHermitian == 1, func, "The given matrix was not (approximately) Hermitian.");
}

// validate_matrixExpIsNonDiverging: a (near) zero element under a negative power
bool fsdNonDiverging(const FullStateDiagMatr& m, cd p, const char* func) {
    if (p.real() >= 0) return true;
    for (qindex i = 0; i < m.numElems; i++)
        if (std::abs(C(m.cpuElems[i])) <= g_eps)
            return fail(func, "The given exponent is negative and the matrix has a (near) zero element, "
                              "so the matrix power diverges.");
    return true;
}

void fsdApply(Qureg q, FullStateDiagMatr m, cd p, bool multiplyOnly, const char* func) {
    const bool hasPower = p != cd(1, 0);
    qg_cplx ex = {p.real(), p.imag()};
    if (q.isDensityMatrix)
        backend(qg_dm_allTargDiagMatr(q.gpuAmps, q.numQubits, m.gpuElems, ex, hasPower, multiplyOnly, g_stream), func);
    else
        backend(qg_sv_allTargDiagMatr(q.gpuAmps, q.numQubits, m.gpuElems, ex, hasPower, g_stream), func);
}

// accelerator.cpp:1010-1030: no power (and so no real-power) when the exponent is 1
cd fsdExpec(Qureg q, FullStateDiagMatr m, cd p, bool useRealPow, const char* func) {
    const bool hasPower = p != cd(1, 0);
    qg_cplx ex = {p.real(), p.imag()}, out = {0, 0};
    if (q.isDensityMatrix)
        backend(qg_dm_calcExpecFullStateDiagMatr(q.gpuAmps, q.numQubits, m.gpuElems, ex, hasPower, useRealPow && hasPower, &out, g_stream), func);
    else
        backend(qg_sv_calcExpecFullStateDiagMatr(q.gpuAmps, q.numQubits, m.gpuElems, ex, hasPower, useRealPow && hasPower, &out, g_stream), func);
    return cd(out.re, out.im);
}

}  // namespace

// operations.cpp:537-576
void multiplyFullStateDiagMatr(Qureg q, FullStateDiagMatr m) {
    const char* func = "multiplyFullStateDiagMatr";
    if (!fsdCompatible(q, m, func)) return;
    fsdApply(q, m, cd(1, 0), true, func);
}

void multiplyFullStateDiagMatrPower(Qureg q, FullStateDiagMatr m, qcomp_t e) {
    const char* func = "multiplyFullStateDiagMatrPower";
    if (!fsdCompatible(q, m, func) || !fsdNonDiverging(m, C(e), func)) return;
    fsdApply(q, m, C(e), true, func);
}

void applyFullStateDiagMatr(Qureg q, FullStateDiagMatr m) {
    const char* func = "applyFullStateDiagMatr";
    if (!fsdCompatible(q, m, func) || !fsdUnitary(m, func)) return;
    fsdApply(q, m, cd(1, 0), false, func);
}

void applyFullStateDiagMatrPower(Qureg q, FullStateDiagMatr m, qcomp_t e) {
    const char* func = "applyFullStateDiagMatrPower";
    if (!fsdCompatible(q, m, func) || !fsdUnitary(m, func)) return;
    if (!check(std::abs(e.im) <= g_eps, func, "The exponent of a unitary matrix must be real so that the result stays unitary."))
        return;
    if (!fsdNonDiverging(m, C(e), func)) return;
    fsdApply(q, m, C(e), false, func);
}

// calculations.cpp:85-215
qcomp_t calcExpecNonHermitianFullStateDiagMatr(Qureg q, FullStateDiagMatr m) {
    const char* func = "calcExpecNonHermitianFullStateDiagMatr";
    if (!fsdCompatible(q, m, func)) return qcomp_t{0, 0};
    return Q(fsdExpec(q, m, cd(1, 0), false, func));
}

qcomp_t calcExpecNonHermitianFullStateDiagMatrPower(Qureg q, FullStateDiagMatr m, qcomp_t e) {
    const char* func = "calcExpecNonHermitianFullStateDiagMatrPower";
    if (!fsdCompatible(q, m, func) || !fsdNonDiverging(m, C(e), func)) return qcomp_t{0, 0};
    return Q(fsdExpec(q, m, C(e), false, func));
}

qreal calcExpecFullStateDiagMatr(Qureg q, FullStateDiagMatr m) {
    const char* func = "calcExpecFullStateDiagMatr";
    if (!fsdCompatible(q, m, func) || !fsdHermitian(m, func)) return 0;
    cd v = fsdExpec(q, m, cd(1, 0), false, func);
    if (q.isDensityMatrix && !check(std::abs(v.imag()) <= REDUCTION_EPS_FACTOR * g_eps, func,
                                    "The calculated expectation value was not approximately real.")) return 0;
    return v.real();
}

qreal calcExpecFullStateDiagMatrPower(Qureg q, FullStateDiagMatr m, qreal p) {
    const char* func = "calcExpecFullStateDiagMatrPower";
    if (!fsdCompatible(q, m, func) || !fsdHermitian(m, func) || !fsdNonDiverging(m, cd(p, 0), func)) return 0;
    // validate_matrixExpIsHermitian: a non-integer power of a negative element is not real
    if (p != std::floor(p))
        for (qindex i = 0; i < m.numElems; i++)
            if (!check(m.cpuElems[i].re >= -g_eps, func,
                       "The matrix has a negative element, so a non-integer power of it is not Hermitian.")) return 0;
    cd v = fsdExpec(q, m, cd(p, 0), true, func);
    if (q.isDensityMatrix && !check(std::abs(v.imag()) <= REDUCTION_EPS_FACTOR * g_eps, func,
                                    "The calculated expectation value was not approximately real.")) return 0;
    return v.real();
}

qreal calcProbOfMultiQubitOutcome(Qureg q, int* qs, int* os, int n) {
    const char* func = "calcProbOfMultiQubitOutcome";
    if (!checkQureg(q, func) || !checkQubits(q, qs, n, func, "target qubits")) return 0;
    for (int i = 0; i < n; i++)
        if (!check(os[i] == 0 || os[i] == 1, func, "Invalid measurement outcome; must be 0 or 1.")) return 0;
    double v = 0;
    probOf(q, V(qs, n), V(os, n), &v, func);
    return v;
}
qreal calcProbOfQubitOutcome(Qureg q, int qubit, int outcome) { return calcProbOfMultiQubitOutcome(q, &qubit, &outcome, 1); }

void calcProbsOfAllMultiQubitOutcomes(qreal* out, Qureg q, int* qs, int n) {
    const char* func = "calcProbsOfAllMultiQubitOutcomes";
    if (!checkQureg(q, func) || !checkQubits(q, qs, n, func, "target qubits")) return;
    if (q.isDensityMatrix)
        backend(qg_dm_calcProbsOfAllMultiQubitOutcomes(out, q.gpuAmps, q.numQubits, qs, n, g_stream), func);
    else
        backend(qg_sv_calcProbsOfAllMultiQubitOutcomes(out, q.gpuAmps, q.numQubits, qs, n, g_stream), func);
}

// calcExpecPauliStr: calculations.cpp:133-144 and localiser.cpp:1963-2049
qreal calcExpecPauliStr(Qureg q, PauliStr str) {
    const char* func = "calcExpecPauliStr";
    if (!checkQureg(q, func)) return 0;
    if (!check(strFits(str, q.numQubits), func, "The Pauli string targets a qubit beyond the Qureg.")) return 0;
    vector<int> x, y, z;
    splitXYZ(codesOf(str, q.numQubits), x, y, z);
    qcomp_t v{0, 0};
    bool ok = q.isDensityMatrix
                  ? backend(qg_dm_calcExpecPauliStr(q.gpuAmps, q.numQubits, P(x), (int)x.size(), P(y), (int)y.size(), P(z), (int)z.size(), &v, g_stream), func)
                  : backend(qg_sv_calcExpecPauliStr(q.gpuAmps, q.numQubits, P(x), (int)x.size(), P(y), (int)y.size(), P(z), (int)z.size(), &v, g_stream), func);
    if (!ok) return 0;
    if (!check(std::abs(v.im) <= REDUCTION_EPS_FACTOR * g_eps, func, "The expectation value was not approximately real.")) return 0;
    return v.re;
}

}  // extern "C"

namespace {

// The complex value of every string (the term before its real part is taken), through the
// batched kernels: many strings per pass over the amplitudes (statevector) or the columns
// (density matrix).  The reference evaluates one pass per string
// (localiser_statevec_calcExpecPauliStrSum, localiser.cpp:2052-2148; its density-matrix
// form, :2151-2171); the values are the same terms.
bool pauliValues(const Qureg& q, const PauliStr* strs, qindex num, vector<cd>& vals, const char* func) {
    vector<int64_t> mxy((size_t)num), myz((size_t)num);
    vector<int> ny((size_t)num);
    for (qindex s = 0; s < num; s++) {
        if (!check(strFits(strs[s], q.numQubits), func, "A Pauli string targets a qubit beyond the Qureg.")) return false;
        vector<int> codes = codesOf(strs[s], q.numQubits);
        int64_t a = 0, b = 0;
        for (int i = 0; i < q.numQubits; i++) {
            if (codes[i] == 1 || codes[i] == 2) a |= (int64_t)1 << i;
            if (codes[i] == 2 || codes[i] == 3) b |= (int64_t)1 << i;
        }
        mxy[(size_t)s] = a;
        myz[(size_t)s] = b;
        ny[(size_t)s] = numY(codes);
    }
    vector<qcomp_t> v((size_t)num);
    const int CHUNK = 1 << 20;
    for (qindex s0 = 0; s0 < num; s0 += CHUNK) {
        int cnt = (int)std::min<qindex>(CHUNK, num - s0);
        int rc = q.isDensityMatrix
                     ? qg_dm_calcExpecPauliStrBatch(q.gpuAmps, q.numQubits, mxy.data() + s0, myz.data() + s0, ny.data() + s0, cnt, v.data() + s0, g_stream)
                     : qg_sv_calcExpecPauliStrBatch(q.gpuAmps, q.numQubits, mxy.data() + s0, myz.data() + s0, ny.data() + s0, cnt, v.data() + s0, g_stream);
        if (!backend(rc, func)) return false;
    }
    vals.resize((size_t)num);
    for (qindex s = 0; s < num; s++) vals[(size_t)s] = C(v[(size_t)s]);
    return true;
}

}  // namespace

extern "C" {

void calcExpecPauliStrs(qreal* out, Qureg q, const PauliStr* strs, int num) {
    const char* func = "calcExpecPauliStrs";
    if (!checkQureg(q, func)) return;
    if (!check(num >= 0 && (num == 0 || (strs && out)), func, "Invalid list of Pauli strings.")) return;
    vector<cd> v;
    if (!pauliValues(q, strs, num, v, func)) return;
    for (int s = 0; s < num; s++) {
        if (!check(std::abs(v[s].imag()) <= REDUCTION_EPS_FACTOR * g_eps, func, "The expectation value was not approximately real.")) return;
        out[s] = v[s].real();
    }
}

// createPauliStrSum: paulis.cpp:396-417 (the strings need not be unique)
PauliStrSum createPauliStrSum(PauliStr* strings, qcomp_t* coeffs, qindex numTerms) {
    const char* func = "createPauliStrSum";
    PauliStrSum sum;
    std::memset(&sum, 0, sizeof(sum));
    if (!check(numTerms > 0, func, "The number of terms must be a positive integer.")) return sum;
    if (!check(strings != nullptr && coeffs != nullptr, func, "Null list of Pauli strings or coefficients.")) return sum;
    sum.numTerms = numTerms;
    sum.strings = (PauliStr*)std::malloc(sizeof(PauliStr) * (size_t)numTerms);
    sum.coeffs = (qcomp_t*)std::malloc(sizeof(qcomp_t) * (size_t)numTerms);
    sum.isApproxHermitian = (int*)std::malloc(sizeof(int));
    if (!sum.strings || !sum.coeffs || !sum.isApproxHermitian) {
        std::free(sum.strings);
        std::free(sum.coeffs);
        std::free(sum.isApproxHermitian);
        std::memset(&sum, 0, sizeof(sum));
        fail(func, "Could not allocate the memory of the Pauli string sum.");
        return sum;
    }
    std::memcpy(sum.strings, strings, sizeof(PauliStr) * (size_t)numTerms);
    std::memcpy(sum.coeffs, coeffs, sizeof(qcomp_t) * (size_t)numTerms);
    *sum.isApproxHermitian = -1;
    return sum;
}

void destroyPauliStrSum(PauliStrSum sum) {
    std::free(sum.strings);
    std::free(sum.coeffs);
    std::free(sum.isApproxHermitian);
}

// calcExpecPauliStrSum: calculations.cpp:146-159.  Validation as validate_pauliStrSumFields,
// _pauliStrSumTargets and _pauliStrSumIsHermitian (validation.cpp:3255-3293: every coefficient
// real within epsilon, the flag cached in the sum); the value is sum_t coeff_t * <P_t> added
// in term order, and must be real within the reduction epsilon.
qreal calcExpecPauliStrSum(Qureg q, PauliStrSum sum) {
    const char* func = "calcExpecPauliStrSum";
    if (!checkQureg(q, func)) return 0;
    if (!check(sum.numTerms > 0 && sum.strings && sum.coeffs && sum.isApproxHermitian, func,
               "Invalid PauliStrSum; it was not created, or was destroyed.")) return 0;
    for (qindex t = 0; t < sum.numTerms; t++)
        if (!check(strFits(sum.strings[t], q.numQubits), func, "The PauliStrSum targets a qubit beyond the Qureg.")) return 0;
    if (*sum.isApproxHermitian == -1) {
        int herm = 1;
        for (qindex t = 0; t < sum.numTerms && herm; t++) herm = std::abs(sum.coeffs[t].im) <= g_eps;
        *sum.isApproxHermitian = herm;
    }
    if (!check(*sum.isApproxHermitian == 1, func, "The PauliStrSum is not Hermitian (a coefficient is not real).")) return 0;
    vector<cd> v;
    if (!pauliValues(q, sum.strings, sum.numTerms, v, func)) return 0;
    cd total = 0;
    for (qindex t = 0; t < sum.numTerms; t++) total += C(sum.coeffs[t]) * v[(size_t)t];
    if (!check(std::abs(total.imag()) <= REDUCTION_EPS_FACTOR * g_eps, func, "The expectation value was not approximately real.")) return 0;
    return total.real();
}

}  // extern "C"
