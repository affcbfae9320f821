// Host-side plan of the tiled Pauli-expectation kernel (qg_pauli_tile.cu): how a list of
// strings is split into groups (one pass over the state each) and each group's tile
// coordinates.  Plain C++ (no CUDA), so that the CPU tests check the same plans the
// launches use, with the kernel's own index expressions.
//
// A string pairs amplitude n with j = n ^ maskXY.  Index bits split into t column bits
// (the lowest) and row bits.  The row parts of a group's XY masks span V (over GF(2)),
// kept in reduced row-echelon form B_0..B_{d-1}: B_i's highest bit p_i (its pivot) is
// set in no other B_k; the basis is stored in ascending pivot order and padded with unit
// vectors at the lowest free bits up to `rows` dimensions.  Tile k covers the amplitudes
//     base(k) ^ v(r) | c,   r < 2^d, c < 2^t,
// with base(k) = k << t with zeros opened at the pivots, v(r) = XOR of the B_i whose bit
// i is set in r.  v(r)'s pivot bits are r, so (k, r, c) -> index is one-to-one, and every
// string's partner j of a tile member lies in the same tile at local index
// L ^ D_s (L = (r << t) | c).
#pragma once

#include <stdint.h>

#include <algorithm>
#include <vector>

namespace qgpt {

const int T_MAX = 5;      // column bits: 32 contiguous amplitudes per row
const int D_MAX = 7;      // row bits: at most 2^12 amplitudes per tile
const int NS = 16;        // strings per pass

struct Tile {
    int t, d, numStrings, pad;
    int64_t basis[D_MAX];     // B_i in ascending pivot order (zero in the column bits)
    int64_t pivLow[D_MAX];    // 2^p_i - 1 (zero insertion at the pivots, ascending)
    int64_t D[NS];            // local partner offset of each member (0: no X or Y)
    int64_t yz[NS];           // maskYZ
    int64_t W[NS];            // local sign mask: parity(n & yz) = parity(base & yz) ^ parity(L & W)
    int top[NS];              // highest set bit of D (-1 when D = 0)
    int odd[NS];              // numY odd
};

struct Pass {
    Tile tile;
    std::vector<int> members;  // the caller's string indices, in tile order
    int64_t numTiles;
};

inline int highest_bit(int64_t x) {
    int b = -1;
    for (int i = 0; i < 64; i++)
        if ((x >> i) & 1) b = i;
    return b;
}
inline int parity(int64_t x) {
    int p = 0;
    for (; x; x &= x - 1) p ^= 1;
    return p;
}

struct Basis {
    std::vector<int64_t> vec;
    std::vector<int> piv;
    // clears every pivot bit of x (reduced form: a pivot appears in one vector only)
    int64_t reduce(int64_t x) const {
        for (size_t i = 0; i < vec.size(); i++)
            if ((x >> piv[i]) & 1) x ^= vec[i];
        return x;
    }
    // x reduced and nonzero: its highest bit becomes a new pivot
    void add(int64_t x) {
        const int p = highest_bit(x);
        for (size_t i = 0; i < vec.size(); i++)
            if ((vec[i] >> p) & 1) vec[i] ^= x;
        vec.push_back(x);
        piv.push_back(p);
    }
};

// The passes for `num` strings on an n-qubit statevector (n >= 1): strings in order, a new
// pass whenever one more would exceed NS strings or D_MAX row dimensions.
inline std::vector<Pass> make_passes(int n, const int64_t* mXY, const int64_t* mYZ, const int* numsY, int num) {
    const int t = std::min(n, T_MAX);
    const int rows = std::min(D_MAX, n - t);
    const int64_t colMask = ((int64_t)1 << t) - 1;
    std::vector<Pass> passes;
    std::vector<Basis> bases;
    for (int s = 0; s < num; s++) {
        const int64_t row = mXY[s] & ~colMask;
        bool fits = !passes.empty() && (int)passes.back().members.size() < NS;
        int64_t red = fits ? bases.back().reduce(row) : row;
        if (fits && red != 0 && (int)bases.back().vec.size() >= rows) fits = false;
        if (!fits) {
            passes.emplace_back();
            bases.emplace_back();
            red = row;
        }
        if (red != 0) bases.back().add(red);
        passes.back().members.push_back(s);
    }
    for (size_t g = 0; g < passes.size(); g++) {
        Basis& B = bases[g];
        for (int b = t; b < n && (int)B.vec.size() < rows; b++) {     // pad with free unit vectors
            const int64_t e = (int64_t)1 << b;
            if (B.reduce(e) == e) B.add(e);
        }
        const int d = (int)B.vec.size();
        std::vector<int> order(d);
        for (int i = 0; i < d; i++) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int x, int y) { return B.piv[x] < B.piv[y]; });
        Tile& P = passes[g].tile;
        P = Tile();
        P.t = t;
        P.d = d;
        P.numStrings = (int)passes[g].members.size();
        for (int i = 0; i < d; i++) {
            P.basis[i] = B.vec[order[i]];
            P.pivLow[i] = ((int64_t)1 << B.piv[order[i]]) - 1;
        }
        for (int k = 0; k < P.numStrings; k++) {
            const int s = passes[g].members[k];
            const int64_t xy = mXY[s], yz = mYZ[s];
            int64_t r = 0, w = 0;
            for (int i = 0; i < d; i++) {
                if ((xy >> B.piv[order[i]]) & 1) r |= (int64_t)1 << i;
                if (parity(P.basis[i] & yz)) w |= (int64_t)1 << i;
            }
            P.D[k] = (r << t) | (xy & colMask);
            P.yz[k] = yz;
            P.W[k] = (w << t) | (yz & colMask);
            P.top[k] = highest_bit(P.D[k]);
            P.odd[k] = numsY[s] & 1;
        }
        passes[g].numTiles = ((int64_t)1 << n) >> (t + d);
    }
    return passes;
}

// the kernel's address of local index e in tile k (vtab[r] = v(r))
inline int64_t tile_base(const Tile& P, int64_t k) {
    int64_t base = k << P.t;
    for (int i = 0; i < P.d; i++) {
        const int64_t lo = base & P.pivLow[i];
        base = ((base ^ lo) << 1) | lo;
    }
    return base;
}
inline int64_t row_offset(const Tile& P, int r) {
    int64_t v = 0;
    for (int i = 0; i < P.d; i++)
        if ((r >> i) & 1) v ^= P.basis[i];
    return v;
}

// The value of string k of a pass from its accumulated sum (the kernel's per-member
// total): the pair sum doubled, or -2i times it for odd numY, or the plain sum for a
// string without X or Y; then the i^numY factor of the Pauli string.
inline void finish_value(const Tile& P, int k, int numY, double acc, double* re, double* im) {
    double r, i;
    if (P.D[k] == 0 && P.top[k] < 0) { r = acc; i = 0; }
    else if (P.odd[k]) { r = 0; i = -2 * acc; }
    else { r = 2 * acc; i = 0; }
    switch (((numY % 4) + 4) % 4) {
        case 0: *re = r; *im = i; break;
        case 1: *re = -i; *im = r; break;
        case 2: *re = -r; *im = -i; break;
        default: *re = i; *im = -r; break;
    }
}

}  // namespace qgpt
