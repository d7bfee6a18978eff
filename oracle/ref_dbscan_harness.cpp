// ref_dbscan_harness.cpp -- TEST INFRASTRUCTURE: runs the reference's own
// clustering path, InterlinkClass (cuda/Interlink.hpp:54-67, body
// cuda/Interlink.cu:34-95), on the host execution model of ref_emu.h, for one
// input file, and writes its getters' results.  Built by oracle/build_ref.py
// into oracle/_ref/ref_dbscan; driven by oracle/ref_run.py.
//
//   ref_dbscan IN OUT
//
// IN  (little endian): "IDBR", n_rows, then n_rows V calls, n_rows J calls,
//     n_rows sequences (each u32 length + bytes), n_v + V names, n_j + J names
//     (same encoding), f32 threshold, u32 minPts, u32 use_hamming,
//     u32 eval_trees.
// OUT: n_rows, n_uniques, clusters[n_rows], cores[n_rows], copies[n_rows],
//     uniques[n_uniques], n_hist, hist[n_hist] (the "Number of trees with depth
//     d" messages of cuda/PSDBSCAN.hcu:1020-1040 when eval_trees is set).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "Interlink.hpp"
#include "../cpp/BenchmarkSingleton.hpp"

namespace {

uint32_t rd32(std::istream &in) {
    unsigned char b[4];
    if (!in.read(reinterpret_cast<char *>(b), 4)) throw std::runtime_error("short input");
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}

std::string rdstr(std::istream &in) {
    uint32_t n = rd32(in);
    std::string s(n, '\0');
    if (n && !in.read(&s[0], n)) throw std::runtime_error("short input");
    return s;
}

void wr32(std::ostream &out, uint32_t v) {
    unsigned char b[4] = {(unsigned char)v, (unsigned char)(v >> 8), (unsigned char)(v >> 16),
                          (unsigned char)(v >> 24)};
    out.write(reinterpret_cast<char *>(b), 4);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    if (rd32(in) != 0x52424449u) throw std::runtime_error("bad magic");
    const uint32_t n = rd32(in);
    thrust::host_vector<std::string> v(n), j(n), seq(n), vg, jg;
    for (uint32_t i = 0; i < n; ++i) v[i] = rdstr(in);
    for (uint32_t i = 0; i < n; ++i) j[i] = rdstr(in);
    for (uint32_t i = 0; i < n; ++i) seq[i] = rdstr(in);
    vg.resize(rd32(in));
    for (auto &g : vg) g = rdstr(in);
    jg.resize(rd32(in));
    for (auto &g : jg) g = rdstr(in);
    uint32_t tb = rd32(in);
    float threshold;
    std::memcpy(&threshold, &tb, 4);
    const uint32_t min_pts = rd32(in), use_hamming = rd32(in), eval_trees = rd32(in);

    // the call of cpp/TableHolder.hpp:337-343
    NormalStringVectorZipIteratorType rows =
        thrust::make_zip_iterator(thrust::make_tuple(v.begin(), j.begin(), seq.begin()));
    InterlinkClass link(rows, n, vg.begin(), (unsigned)vg.size(), jg.begin(), (unsigned)jg.size(),
                        threshold, min_pts, use_hamming != 0, eval_trees != 0);

    std::vector<uint32_t> hist;
    if (eval_trees) {
        const std::string tsv = std::string(argv[2]) + ".tsv";
        BenchmarkSingleton::Instance().write_map(tsv);
        std::ifstream t(tsv);
        std::string line;
        const std::string key = "Number of trees with depth ";
        while (std::getline(t, line)) {
            size_t p = line.find(key);
            if (p == std::string::npos) continue;
            std::istringstream ss(line.substr(p + key.size()));
            unsigned d;
            char colon;
            unsigned long long c;
            ss >> d >> colon >> c;
            if (hist.size() <= d) hist.resize(d + 1, 0);
            hist[d] = (uint32_t)c;
        }
        std::remove(tsv.c_str());
    }

    std::ofstream out(argv[2], std::ios::binary);
    const uint32_t nu = link.get_n_uniques();
    wr32(out, n);
    wr32(out, nu);
    for (uint32_t i = 0; i < n; ++i) wr32(out, link.get_clusters_iterator()[i]);
    for (uint32_t i = 0; i < n; ++i) wr32(out, (uint32_t)link.get_cores_iterator()[i]);
    for (uint32_t i = 0; i < n; ++i) wr32(out, link.get_copies_iterator()[i]);
    for (uint32_t i = 0; i < nu; ++i) wr32(out, link.get_uniques_iterator()[i]);
    wr32(out, (uint32_t)hist.size());
    for (uint32_t h : hist) wr32(out, h);
    return out.good() ? 0 : 1;
}
