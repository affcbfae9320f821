// Host-side plan of the tensor-core block kernel (qg_fused_tc.cu): which mode a block
// runs in and the index tables of its staged modes.  Plain C++ (no CUDA), so that the
// CPU tests check the same tables the launches use.
//
// A block on targets t0..t4 (any order; bit b of the matrix index j is target targs[b])
// works on tiles of 128 groups.  Group r holds the 32 amplitudes base(r) + off(j), with
// base(r) = r with a zero bit opened at each target.  A tile's 4096 amplitudes are
// numbered in address order by a 12-bit local index L: bit p of L sits at amplitude
// bit P[p], where P is the five targets and the seven lowest other bits, ascending.
#pragma once

#include <stdint.h>

namespace qgtc {

struct Plan {
    int stage;          // 0: row by row; 1: staged loads; 2: staged loads and stores
    int lines;          // 128-byte lines one warp instruction touches row by row
    int64_t lbit[12];   // 2^P[p]
    int lrow[7];        // L bit holding bit i of the group row
    int lj[5];          // L bit holding bit b of the matrix index j
    int64_t kp[16];     // producer element k: amplitude offset of the L bits above the producer index
    int64_t ke[32];     // epilogue element k: amplitude offset of L bits 7..11 = k
    int sj[32];         // stage_slot of the L bits of matrix index j
};

// staging-buffer slot of local index e: the low five bits XORed with the next five
inline int stage_slot(int e) { return e ^ ((e >> 5) & 31); }

// a zero bit opened at each of the (ascending) positions
inline int64_t insert_zeros(int64_t n, const int* sortedPos, int num) {
    for (int i = 0; i < num; i++) {
        const int64_t lo = n & (((int64_t)1 << sortedPos[i]) - 1);
        n = ((n ^ lo) << 1) | lo;
    }
    return n;
}

// numQubits >= 12, five distinct targets in [0, numQubits); producerBits = log2 of the
// staged producers' thread count (9 for 512 threads).  Returns false on bad arguments.
inline bool make_plan(int numQubits, const int targs[5], int producerBits, Plan* out) {
    if (numQubits < 12 || numQubits > 62 || producerBits < 7 || producerBits > 11) return false;
    int sorted[5];
    for (int b = 0; b < 5; b++) {
        if (targs[b] < 0 || targs[b] >= numQubits) return false;
        for (int c = 0; c < b; c++)
            if (targs[c] == targs[b]) return false;
        sorted[b] = targs[b];
    }
    for (int i = 1; i < 5; i++)
        for (int k = i; k > 0 && sorted[k - 1] > sorted[k]; k--) {
            const int t = sorted[k];
            sorted[k] = sorted[k - 1];
            sorted[k - 1] = t;
        }
    Plan& p = *out;
    // Row-by-row, lane r of a warp loads amplitude base(r) + off(j): count the distinct
    // 128-byte lines (16 FP32 amplitudes) of r = 0..31.  Measured on GB300 at 30
    // qubits: 32 lines run fastest fully staged (5.3 ms against 8.9 ms row by row), 16
    // lines with staged loads only (4.7 against 5.1), 8 or fewer row by row (2.8-3.9
    // against 3.4-5.4 staged).
    int64_t seen[32];
    p.lines = 0;
    for (int r = 0; r < 32; r++) {
        const int64_t line = insert_zeros(r, sorted, 5) >> 4;
        bool dup = false;
        for (int q = 0; q < p.lines; q++) dup |= seen[q] == line;
        if (!dup) seen[p.lines++] = line;
    }
    p.stage = p.lines >= 32 ? 2 : p.lines >= 16 ? 1 : 0;
    // local bit positions: the targets and the seven lowest other bits, ascending
    int pos[12], n = 0, rows = 0;
    for (int q = 0; q < numQubits && n < 12; q++) {
        bool isTarg = false;
        for (int b = 0; b < 5; b++) isTarg |= targs[b] == q;
        if (isTarg || rows < 7) {
            if (!isTarg) rows++;
            pos[n++] = q;
        }
    }
    int r = 0;
    for (int pb = 0; pb < 12; pb++) {
        p.lbit[pb] = (int64_t)1 << pos[pb];
        int jb = -1;
        for (int b = 0; b < 5; b++)
            if (targs[b] == pos[pb]) jb = b;
        if (jb >= 0) p.lj[jb] = pb;
        else p.lrow[r++] = pb;
    }
    for (int k = 0; k < 16; k++) {
        p.kp[k] = 0;
        if (k < (1 << (12 - producerBits)))
            for (int c = 0; c < 12 - producerBits; c++)
                if ((k >> c) & 1) p.kp[k] += p.lbit[producerBits + c];
    }
    for (int k = 0; k < 32; k++) {
        p.ke[k] = 0;
        int ej = 0;
        for (int c = 0; c < 5; c++)
            if ((k >> c) & 1) {
                p.ke[k] += p.lbit[7 + c];
                ej |= 1 << p.lj[c];
            }
        p.sj[k] = stage_slot(ej);
    }
    return true;
}

}  // namespace qgtc
