// Host check of the tiled Pauli-expectation kernel's plan (qg_pauli_plan.h): for random
// statevectors and string lists, every pass's tiles, evaluated with the kernel's own index
// expressions (tile base, row offsets, partner offset, sign masks, the pair enumeration
// that skips bit `top`), cover every amplitude exactly once and give the expectation
// values of the direct sum over n of sign(j & maskYZ) conj(a_n) a_j, j = n ^ maskXY.
#include "qg_pauli_plan.h"

#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

typedef std::complex<double> cd;
static int failures = 0;

#define CHECK(c, ...)                                      \
    do {                                                   \
        if (!(c)) {                                        \
            if (failures++ < 10) std::printf(__VA_ARGS__); \
        }                                                  \
    } while (0)

static void check_case(int n, int num, std::mt19937_64& g, int style) {
    const int64_t N = (int64_t)1 << n;
    std::normal_distribution<double> nd;
    std::vector<cd> a(N);
    for (auto& x : a) x = cd(nd(g), nd(g));
    std::vector<int64_t> xy(num), yz(num);
    std::vector<int> ny(num);
    for (int s = 0; s < num; s++) {
        int64_t x = 0, z = 0;
        int y = 0;
        for (int q = 0; q < n; q++) {
            int code = (int)(g() % 4);
            if (style == 1 && q >= 3) code = (code == 1 || code == 2) ? 0 : code;   // XY only on low qubits
            if (style == 2 && (code == 1 || code == 2) && q < n - 3) code = 3;      // XY only on high qubits
            if (style == 3 && s % 3 == 0) code = (code == 3) ? 3 : 0;               // Z-only / identity strings
            if (code == 1 || code == 2) x |= (int64_t)1 << q;
            if (code == 2 || code == 3) z |= (int64_t)1 << q;
            y += code == 2;
        }
        if (style == 4 && s > 0 && s % 2 == 0) { x = xy[s - 1]; z = yz[s - 1]; y = ny[s - 1]; }   // repeats
        xy[s] = x;
        yz[s] = z;
        ny[s] = y;
    }
    const std::vector<qgpt::Pass> passes = qgpt::make_passes(n, xy.data(), yz.data(), ny.data(), num);
    std::vector<int> seen(num, 0);
    for (const qgpt::Pass& ps : passes) {
        const qgpt::Tile& P = ps.tile;
        CHECK(P.numStrings >= 1 && P.numStrings <= qgpt::NS, "bad pass size %d\n", P.numStrings);
        CHECK(P.d <= qgpt::D_MAX && P.t + P.d <= n, "bad tile shape t=%d d=%d n=%d\n", P.t, P.d, n);
        CHECK(ps.numTiles == (N >> (P.t + P.d)), "bad tile count\n");
        const int L = 1 << (P.d + P.t);
        std::vector<int> cover(N, 0);
        std::vector<double> acc(P.numStrings, 0.0);
        for (int64_t k = 0; k < ps.numTiles; k++) {
            const int64_t base = qgpt::tile_base(P, k);
            std::vector<cd> tile(L);
            for (int e = 0; e < L; e++) {
                const int64_t idx = (base ^ qgpt::row_offset(P, e >> P.t)) | (int64_t)(e & ((1 << P.t) - 1));
                CHECK(idx >= 0 && idx < N, "index %lld out of range (n=%d)\n", (long long)idx, n);
                if (idx < 0 || idx >= N) return;
                cover[idx]++;
                tile[e] = a[idx];
            }
            for (int s = 0; s < P.numStrings; s++) {
                const int pb = qgpt::parity(base & P.yz[s]);
                if (P.top[s] < 0) {
                    for (int e = 0; e < L; e++) {
                        const int64_t idx = (base ^ qgpt::row_offset(P, e >> P.t)) | (int64_t)(e & ((1 << P.t) - 1));
                        const int sg = pb ^ qgpt::parity((int64_t)e & P.W[s]);
                        CHECK(sg == qgpt::parity(idx & P.yz[s]), "sign split wrong\n");
                        acc[s] += (sg ? -1.0 : 1.0) * std::norm(tile[e]);
                    }
                } else {
                    const int top = P.top[s], Ds = (int)P.D[s], lowMask = (1 << top) - 1;
                    CHECK(Ds > 0 && Ds < L, "partner offset outside the tile\n");
                    for (int m = 0; m < (L >> 1); m++) {
                        const int e = ((m & ~lowMask) << 1) | (m & lowMask);
                        const int ep = e ^ Ds;
                        const int64_t idx = (base ^ qgpt::row_offset(P, e >> P.t)) | (int64_t)(e & ((1 << P.t) - 1));
                        const int64_t jdx = (base ^ qgpt::row_offset(P, ep >> P.t)) | (int64_t)(ep & ((1 << P.t) - 1));
                        CHECK(jdx == (idx ^ xy[ps.members[s]]), "partner of %lld is %lld, not %lld\n", (long long)idx,
                              (long long)jdx, (long long)(idx ^ xy[ps.members[s]]));
                        const int sg = pb ^ qgpt::parity((int64_t)e & P.W[s]);
                        const cd x = std::conj(tile[e]) * tile[ep];
                        acc[s] += (sg ? -1.0 : 1.0) * (P.odd[s] ? x.imag() : x.real());
                    }
                }
            }
        }
        for (int64_t i = 0; i < N; i++) CHECK(cover[i] == 1, "amplitude %lld covered %d times\n", (long long)i, cover[i]);
        for (int k = 0; k < P.numStrings; k++) {
            const int s = ps.members[k];
            seen[s]++;
            double re, im;
            qgpt::finish_value(P, k, ny[s], acc[k], &re, &im);
            cd direct = 0;
            for (int64_t i = 0; i < N; i++) {
                const int64_t j = i ^ xy[s];
                direct += (qgpt::parity(j & yz[s]) ? -1.0 : 1.0) * std::conj(a[i]) * a[j];
            }
            static const cd powI[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
            direct *= powI[ny[s] % 4];
            const double scale = 1e-12 * (double)N;
            CHECK(std::abs(re - direct.real()) <= scale && std::abs(im - direct.imag()) <= scale,
                  "n=%d string %d: (%g, %g) vs direct (%g, %g)\n", n, s, re, im, direct.real(), direct.imag());
        }
    }
    for (int s = 0; s < num; s++) CHECK(seen[s] == 1, "string %d in %d passes\n", s, seen[s]);
}

int main() {
    std::mt19937_64 g(2027);
    for (int n = 1; n <= 16; n++)
        for (int style = 0; style < 5; style++) {
            const int num = 1 + (int)(g() % 40);
            check_case(n, num, g, style);
        }
    for (int rep = 0; rep < 20; rep++) check_case(10 + (int)(g() % 7), 16, g, 0);
    if (failures) {
        std::printf("FAILED: %d checks\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
