// CPU unit test of the integer helpers the kernels use (bitops.cuh compiled as
// host code): the bit-parallel edit distance against a plain DP, the diagonal
// values used by the kernels' early exit, and the triangular unit decode.
// Exit status 0 = all checks passed.
#include "bitops.cuh"

#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

using namespace idb;

static int dp(const uint8_t *a, int m, const uint8_t *b, int n) {
    std::vector<int> p(n + 1), c(n + 1);
    for (int j = 0; j <= n; j++) p[j] = j;
    for (int i = 1; i <= m; i++) {
        c[0] = i;
        for (int j = 1; j <= n; j++)
            c[j] = std::min({p[j - 1] + (a[i - 1] != b[j - 1]), p[j] + 1, c[j - 1] + 1});
        std::swap(p, c);
    }
    return p[n];
}

int main() {
    std::mt19937 rng(1);
    int bad = 0;
    // multi-block recurrence, patterns up to 128
    for (int it = 0; it < 100000; it++) {
        int m = rng() % 129, n = rng() % 140;
        int A = 1 + rng() % 5;
        std::vector<uint8_t> a(m), b(n);
        for (auto &x : a) x = rng() % A;
        for (auto &x : b) x = rng() % A;
        if (rng() % 2)
            for (int k = 0; k < std::min(m, n); k++)
                if (rng() % 4) b[k] = a[k];
        int d = dp(a.data(), m, b.data(), n), e;
        if (m <= 32) e = myers_distance<1>(a.data(), m, b.data(), n);
        else if (m <= 64) e = myers_distance<2>(a.data(), m, b.data(), n);
        else if (m <= 96) e = myers_distance<3>(a.data(), m, b.data(), n);
        else e = myers_distance<4>(a.data(), m, b.data(), n);
        if (d != e) {
            if (bad < 5) printf("myers m=%d n=%d dp=%d bitpar=%d\n", m, n, d, e);
            bad++;
        }
    }
    // single-block step and every intermediate D[i][j]
    for (int it = 0; it < 20000; it++) {
        int m = rng() % 33, n = rng() % 40;
        std::vector<uint8_t> a(m), b(n);
        for (auto &x : a) x = rng() % 4;
        for (auto &x : b) x = rng() % 4;
        uint32_t Pv = ~0u, Mv = 0;
        for (int j = 0; j < n; j++) {
            uint32_t eq = 0;
            for (int i = 0; i < m; i++)
                if (a[i] == b[j]) eq |= 1u << i;
            myers_step1(Pv, Mv, eq);
            uint32_t P1[1] = {Pv}, M1[1] = {Mv};
            for (int i = 0; i <= m; i++)
                if (dp(a.data(), i, b.data(), j + 1) != myers_value<1>(P1, M1, i, j + 1)) bad++;
        }
    }
    // triangular work-unit numbering
    for (uint32_t ncx = 1; ncx < 60; ncx++)
        for (uint32_t q = 1; q < 9; q++) {
            uint32_t ncy = (ncx + q - 1) / q;
            std::vector<std::pair<uint32_t, uint32_t>> ref;
            for (uint32_t cy = 0; cy < ncy; cy++)
                for (uint32_t cx = 0; cx < ncx; cx++)
                    if (cx < (cy + 1) * q) ref.push_back({cx, cy});
            uint64_t T = tri_units(ncx, ncy, q);
            if (T != ref.size()) { bad++; continue; }
            for (uint64_t k = 0; k < T; k++) {
                uint32_t cx, cy;
                tri_decode(k, ncx, q, cx, cy);
                if (cx != ref[k].first || cy != ref[k].second) bad++;
            }
        }
    printf("bitops failures: %d\n", bad);
    return bad ? 1 : 0;
}
