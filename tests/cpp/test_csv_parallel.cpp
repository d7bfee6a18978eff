// The parallel CSV reader and writer against their one-thread forms
// (read_csv_serial / write_csv_serial in host/csv.hpp): identical tables and
// byte-identical files on generated inputs large enough for every host thread
// to take part, with the reader's quirks (trailing '\r', quoted separators,
// escapes, short rows, a final empty row or none, header-only files).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "csv.hpp"

using namespace psdb;

static int failures = 0;
#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::cerr << "FAIL " << __FILE__ << ":" << __LINE__ << " " #c "\n"; \
            ++failures;                                                   \
        }                                                                 \
    } while (0)

static std::string slurp(const std::string &f) {
    std::ifstream in(f, std::ios::binary);
    std::stringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

static std::string make_file(std::mt19937_64 &rng, size_t rows, bool final_eol, bool cr, char sep) {
    const char *alpha = "ACDEFGHIKLMNPQRSTVWY";
    std::string s = std::string("ID") + sep + "junction_aa" + sep + "v_call" + sep + "extra" +
                    (cr ? "\r\n" : "\n");
    for (size_t r = 0; r < rows; ++r) {
        std::string seq;
        const int L = (int)(rng() % 20);
        for (int k = 0; k < L; ++k) seq.push_back(alpha[rng() % 20]);
        std::string v = "IGHV" + std::to_string(rng() % 60) + "*0" + std::to_string(rng() % 3);
        switch (rng() % 10) {
            case 0: v = "\"IGHV1" + std::string(1, sep) + "x\""; break;   // quoted separator
            case 1: v = "a\\nb\\\\c"; break;                             // escapes
            case 2: v = ""; break;
            default: break;
        }
        s += std::to_string(r);
        if (rng() % 50 == 0) {               // a short row: fields missing
            s += sep + seq;
        } else {
            s += sep + seq + sep + v + sep + "e" + std::to_string(r % 7);
        }
        if (r + 1 < rows || final_eol) s += cr && rng() % 2 ? "\r\n" : "\n";
    }
    return s;
}

int main(int argc, char **argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    std::mt19937_64 rng(7);
    const std::vector<std::string> wanted{"v_call", "junction_aa", "ID"};
    int case_no = 0;
    for (size_t rows : {0ul, 1ul, 5ul, 3000ul, 200000ul}) {
        for (bool final_eol : {true, false}) {
            for (bool cr : {false, true}) {
                const char sep = case_no % 2 ? '\t' : ',';
                const std::string f = dir + "/p" + std::to_string(case_no++) + ".csv";
                std::ofstream(f, std::ios::binary) << make_file(rng, rows, final_eol, cr, sep);
                std::vector<std::vector<std::string>> a, b;
                read_csv(f, sep, '\n', '"', wanted, a);
                read_csv_serial(f, sep, '\n', '"', wanted, b);
                CHECK(a == b);
                // two files appended
                read_csv(f, sep, '\n', '"', wanted, a);
                read_csv_serial(f, sep, '\n', '"', wanted, b);
                CHECK(a == b);
                std::vector<const std::vector<std::string> *> cols;
                for (auto &c : a) cols.push_back(&c);
                const std::vector<std::string> hdr{"file", "V", "J", "I"};
                for (char q : {'"', '\0'}) {
                    write_csv(f + ".par", cols, hdr, sep, '\n', q);
                    write_csv_serial(f + ".ser", cols, hdr, sep, '\n', q);
                    CHECK(slurp(f + ".par") == slurp(f + ".ser"));
                }
            }
        }
    }
    // header only, with and without its end of line; an empty file
    for (const char *content : {"ID,junction_aa,v_call", "ID,junction_aa,v_call\n", ""}) {
        const std::string f = dir + "/h.csv";
        std::ofstream(f, std::ios::binary) << content;
        std::vector<std::vector<std::string>> a, b;
        std::string ea, eb;
        try { read_csv(f, ',', '\n', '"', wanted, a); } catch (const std::exception &e) { ea = e.what(); }
        try { read_csv_serial(f, ',', '\n', '"', wanted, b); } catch (const std::exception &e) { eb = e.what(); }
        CHECK(a == b);
        CHECK(ea == eb);
    }
    if (failures) {
        std::cerr << failures << " failure(s)\n";
        return 1;
    }
    std::cout << "ok\n";
    return 0;
}
