// Host check of the tensor-core block kernel's plan (qg_tc_plan.h): the mode chosen for
// a target set, and the staged modes' index tables, evaluated with the same expressions
// as the kernel (producer loads in address order into a staging buffer, row-order
// read-back; the epilogue's row-order writes and address-order stores).
#include "qg_tc_plan.h"

#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

static int failures = 0;

#define CHECK(c, ...)                                  \
    do {                                               \
        if (!(c)) {                                    \
            if (failures++ < 10) std::printf(__VA_ARGS__); \
        }                                              \
    } while (0)

static const int kProducers = 512, kProducerBits = 9, kEpilogue = 128;

static void check_tables(int nq, const int targs[5], std::mt19937_64& g) {
    qgtc::Plan p;
    if (!qgtc::make_plan(nq, targs, kProducerBits, &p)) {
        CHECK(false, "plan refused valid targets\n");
        return;
    }
    int sorted[5];
    std::copy(targs, targs + 5, sorted);
    std::sort(sorted, sorted + 5);
    int64_t off[32];
    for (int j = 0; j < 32; j++) {
        off[j] = 0;
        for (int b = 0; b < 5; b++)
            if ((j >> b) & 1) off[j] += (int64_t)1 << targs[b];
    }
    const int64_t numTiles = ((int64_t)1 << nq) / 32 / 128;
    for (int rep = 0; rep < 3; rep++) {
        const int64_t T = (int64_t)(g() % (uint64_t)numTiles);
        const int64_t tileBase = qgtc::insert_zeros(T * 128, sorted, 5);
        std::vector<int64_t> want(128 * 32);
        for (int r = 0; r < 128; r++)
            for (int j = 0; j < 32; j++) want[r * 32 + j] = qgtc::insert_zeros(T * 128 + r, sorted, 5) + off[j];
        // producers: element L = tid + 512 k at tileBase + tOff(tid) + kp[k], into slot
        // stage_slot(tid) ^ stage_slot(512 k)
        std::vector<int64_t> stage(4096, -1);
        for (int tid = 0; tid < kProducers; tid++) {
            int64_t tOff = 0;
            for (int b = 0; b < kProducerBits; b++)
                if ((tid >> b) & 1) tOff += p.lbit[b];
            for (int k = 0; k < 4096 / kProducers; k++) {
                const int64_t addr = tileBase + tOff + p.kp[k];
                CHECK(addr >= 0 && addr < ((int64_t)1 << nq), "load out of range\n");
                const int slot = qgtc::stage_slot(tid) ^ qgtc::stage_slot(kProducers * k);
                CHECK(slot == qgtc::stage_slot(tid + kProducers * k), "slot map not linear (producer)\n");
                CHECK(stage[slot] == -1, "staging slot written twice\n");
                stage[slot] = addr;
            }
        }
        std::vector<int64_t> a(stage), b(want);
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        CHECK(a == b, "tile coverage differs (targets %d %d %d %d %d)\n", targs[0], targs[1], targs[2], targs[3], targs[4]);
        // producer read-back: (row, j) at stage_slot(eRow) ^ sj[j]
        std::vector<int64_t> epi(4096, -1);
        for (int r = 0; r < 128; r++) {
            int eRow = 0;
            for (int i = 0; i < 7; i++)
                if ((r >> i) & 1) eRow |= 1 << p.lrow[i];
            const int sRow = qgtc::stage_slot(eRow);
            for (int j = 0; j < 32; j++) {
                CHECK(stage[sRow ^ p.sj[j]] == want[r * 32 + j], "producer read-back wrong (row %d, j %d)\n", r, j);
                epi[sRow ^ p.sj[j]] = want[r * 32 + j];   // the epilogue's row-order write
            }
        }
        // epilogue stores: element L = row + 128 k from slot stage_slot(row) ^ stage_slot(128 k)
        for (int r = 0; r < kEpilogue; r++) {
            int64_t eOff = 0;
            for (int b = 0; b < 7; b++)
                if ((r >> b) & 1) eOff += p.lbit[b];
            for (int k = 0; k < 32; k++) {
                const int slot = qgtc::stage_slot(r) ^ qgtc::stage_slot(kEpilogue * k);
                CHECK(slot == qgtc::stage_slot(r + kEpilogue * k), "slot map not linear (epilogue)\n");
                CHECK(tileBase + eOff + p.ke[k] == epi[slot], "epilogue store wrong (row %d, k %d)\n", r, k);
            }
        }
    }
}

int main() {
    std::vector<int> seen(4096, 0);
    for (int e = 0; e < 4096; e++) seen[qgtc::stage_slot(e)]++;
    CHECK(std::all_of(seen.begin(), seen.end(), [](int v) { return v == 1; }), "stage_slot is not a bijection\n");

    // modes of the target sets measured on GB300
    struct Case { int t[5]; int stage; };
    const Case cases[] = {{{0, 1, 2, 3, 4}, 2}, {{0, 1, 2, 3, 9}, 2}, {{1, 2, 3, 4, 5}, 1}, {{1, 2, 3, 4, 10}, 1},
                          {{2, 3, 4, 5, 6}, 0}, {{0, 1, 7, 13, 19}, 0}, {{2, 3, 9, 15, 21}, 0}, {{5, 6, 7, 8, 9}, 0},
                          {{25, 26, 27, 28, 29}, 0}, {{4, 3, 2, 1, 0}, 2}};
    for (const auto& c : cases) {
        qgtc::Plan p;
        CHECK(qgtc::make_plan(30, c.t, kProducerBits, &p) && p.stage == c.stage,
              "mode of targets %d %d %d %d %d: got %d, want %d\n", c.t[0], c.t[1], c.t[2], c.t[3], c.t[4], p.stage, c.stage);
    }
    // refused arguments
    {
        qgtc::Plan p;
        const int dup[5] = {0, 1, 2, 3, 3}, out[5] = {0, 1, 2, 3, 14}, ok[5] = {0, 1, 2, 3, 4};
        CHECK(!qgtc::make_plan(14, dup, kProducerBits, &p), "duplicate target accepted\n");
        CHECK(!qgtc::make_plan(14, out, kProducerBits, &p), "target out of range accepted\n");
        CHECK(!qgtc::make_plan(11, ok, kProducerBits, &p), "register below one tile accepted\n");
    }
    // the staged tables on the measured sets and on random sets at 12..24 qubits
    std::mt19937_64 g(20260512);
    for (const auto& c : cases) check_tables(30, c.t, g);
    int tables = (int)(sizeof(cases) / sizeof(cases[0]));
    for (int rep = 0; rep < 60; rep++) {
        const int nq = 12 + (int)(g() % 13);
        int t[5], n = 0;
        while (n < 5) {
            const int q = (int)(g() % (uint64_t)nq);
            if (std::find(t, t + n, q) == t + n) t[n++] = q;
        }
        check_tables(nq, t, g);
        tables++;
    }
    std::printf("%s target sets=%d failures=%d\n", failures ? "FAIL" : "OK", tables, failures);
    return failures ? 1 : 0;
}
