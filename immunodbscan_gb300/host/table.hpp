// table.hpp -- the psdbscan host: configuration keys, the column table, the
// clustering call and the output file.  Same flow and keys as the reference's
// ConfigHolderClass / TableHolderClass (cpp/ConfigHolder.hpp, cpp/TableHolder.hpp),
// with InterlinkClass replaced by the C ABI call idb_cluster.
#pragma once
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "csv.hpp"
#include "immunodbscan_gb300.h"
#include "info.hpp"

namespace psdb {

// ---------------------------------------------------------------------------
// Timers and messages (cpp/BenchmarkSingleton.hpp): written as a two-column
// TSV "Timer/Message<TAB>Value" to the benchmark file.
// ---------------------------------------------------------------------------
class Benchmark {
    using clock = std::chrono::high_resolution_clock;
    std::map<std::string, std::pair<clock::time_point, clock::time_point>> timers_;
    std::vector<std::pair<std::string, std::string>> data_;
    clock::time_point start_ = clock::now();
    bool verbose_ = false;

  public:
    static Benchmark &instance() {
        static Benchmark b;
        return b;
    }
    void be_verbose() { verbose_ = true; }
    void start(const std::string &name) { timers_[name].first = clock::now(); }
    void stop(const std::string &name) {
        auto it = timers_.find(name);
        if (it == timers_.end()) return;
        it->second.second = clock::now();
        const double s = std::chrono::duration<double>(it->second.second - it->second.first).count();
        data_.emplace_back(name, std::to_string(s) + " sec");
        if (verbose_) std::cout << "\nTimer " << name << ": " << s << " sec";
    }
    void message(const std::string &msg) {
        const double s = std::chrono::duration<double>(clock::now() - start_).count();
        data_.emplace_back("At " + std::to_string(s) + " sec", msg);
        if (verbose_) std::cout << "\n" << msg;
    }
    void write(const std::string &filename) const {
        std::ofstream out(filename);
        out << "Timer/Message" << "\t" << "Value" << "\n";
        for (const auto &d : data_) out << d.first << "\t" << d.second << "\n";
    }
};

// ---------------------------------------------------------------------------
// Configuration keys (cpp/ConfigHolder.hpp:65-259).  Added optional keys:
//   maximum_absolute_edit_distance  int, caps eps (or replaces the relative key)
//   work_schedule                   "static" (default) or "learned"
//   candidate_pairs                 "auto" (default) or "buckets"
// ---------------------------------------------------------------------------
class Config {
    InfoNode tree_;

  public:
    enum FileSel { Input, Output, Bench };
    explicit Config(const std::string &file) : tree_(read_info(file)) {}
    explicit Config(InfoNode tree) : tree_(std::move(tree)) {}
    const InfoNode &tree() const { return tree_; }

    char special(FileSel f, const std::string &what) const {
        static const char *names[] = {"input_settings", "output_settings", "benchmark_output_settings"};
        return as_char(tree_.child(names[f]).get(what), std::string(names[f]) + "." + what);
    }
    std::string filename(const std::string &main, FileSel f) const {
        // path + prefix + stem + suffix + filetype (cpp/ConfigHolder.hpp:42-48, 89-113)
        const std::string path = main.substr(0, main.find_last_of('/') + 1);
        std::string stem = main.substr(0, main.find_last_of('.'));
        stem = stem.substr(stem.find_last_of('/') + 1);
        const std::string k = f == Output ? "output_" : "benchmark_output_";
        if (f == Input) throw std::runtime_error("Bad File Selection!");
        return path + tree_.get(k + "prefix") + stem + tree_.get(k + "suffix") + tree_.get(k + "filetype");
    }
    std::vector<std::pair<std::string, std::string>> columns(const std::string &block) const {
        std::vector<std::pair<std::string, std::string>> out;
        for (const auto &c : tree_.child(block).children) out.emplace_back(c.key, c.data);
        return out;
    }
    float threshold() const {
        if (!tree_.has("maximum_relative_edit_distance") && tree_.has("maximum_absolute_edit_distance"))
            return NAN;
        return as_float(tree_.get("maximum_relative_edit_distance"), "maximum_relative_edit_distance");
    }
    int32_t abs_eps() const {
        if (!tree_.has("maximum_absolute_edit_distance")) return -1;
        return (int32_t)as_int(tree_.get("maximum_absolute_edit_distance"), "maximum_absolute_edit_distance");
    }
    uint32_t min_pts() const {
        return (uint32_t)as_int(tree_.get("minimum_number_of_neighbors"), "minimum_number_of_neighbors");
    }
    bool flag(const std::string &k, bool dflt) const {
        return tree_.has(k) ? as_bool(tree_.get(k), k) : dflt;
    }
    bool remove_noise() const { return as_bool(tree_.get("remove_noise_from_output"), "remove_noise_from_output"); }
    int schedule() const {
        if (!tree_.has("work_schedule")) return 0;
        const std::string &s = tree_.get("work_schedule");
        if (s == "static") return 0;
        if (s == "learned") return 1;
        throw std::runtime_error("work_schedule must be static or learned");
    }
    int candidates() const {
        if (!tree_.has("candidate_pairs")) return 0;
        const std::string &s = tree_.get("candidate_pairs");
        if (s == "auto") return 0;
        if (s == "buckets") return 1;
        throw std::runtime_error("candidate_pairs must be auto or buckets");
    }
    // gene_columns.first_gene.name etc.; "" when not configured
    std::string opt(const std::string &p) const { return tree_.has(p) ? tree_.get(p) : std::string(); }
};

// ---------------------------------------------------------------------------
// One row column as idb_cluster takes it (blob + int64 offsets), in page-locked
// memory when the library can provide it, packed by all host threads.
// ---------------------------------------------------------------------------
class HostColumn {
    void *mem_ = nullptr;   // page-locked: offsets then bytes
    std::vector<char> heap_;
    int64_t *off_ = nullptr;
    char *blob_ = nullptr;

  public:
    HostColumn() = default;
    HostColumn(const HostColumn &) = delete;
    HostColumn &operator=(const HostColumn &) = delete;
    ~HostColumn() {
        if (mem_) idb_host_free(mem_);
    }
    void pack(const std::vector<std::string> &v) {
        const size_t n = v.size();
        std::vector<int64_t> off(n + 1, 0);
        // offsets: per-range sums, then a scan over the ranges
        const size_t nt = std::max<size_t>(1, std::min<size_t>(host_threads(), n / 65536));
        std::vector<int64_t> part(nt + 1, 0);
        parallel_ranges(nt, [&](size_t lo, size_t hi) {
            for (size_t t = lo; t < hi; ++t) {
                int64_t acc = 0;
                for (size_t r = n * t / nt; r < n * (t + 1) / nt; ++r) {
                    acc += (int64_t)v[r].size();
                    off[r + 1] = acc;
                }
                part[t + 1] = acc;
            }
        }, 1);
        for (size_t t = 0; t < nt; ++t) part[t + 1] += part[t];
        const size_t bytes = (size_t)part[nt];
        const size_t need = 8 * (n + 1) + bytes;
        if (idb_host_alloc(need, &mem_) == IDB_OK) {
            off_ = static_cast<int64_t *>(mem_);
            blob_ = static_cast<char *>(mem_) + 8 * (n + 1);
        } else {
            mem_ = nullptr;
            heap_.resize(need + 8);
            off_ = reinterpret_cast<int64_t *>((reinterpret_cast<uintptr_t>(heap_.data()) + 7) & ~(uintptr_t)7);
            blob_ = reinterpret_cast<char *>(off_ + n + 1);
        }
        off_[0] = 0;
        parallel_ranges(nt, [&](size_t lo, size_t hi) {
            for (size_t t = lo; t < hi; ++t)
                for (size_t r = n * t / nt; r < n * (t + 1) / nt; ++r) {
                    off_[r + 1] = off[r + 1] + part[t];
                    if (!v[r].empty()) std::memcpy(blob_ + off_[r + 1] - v[r].size(), v[r].data(), v[r].size());
                }
        }, 1);
    }
    const char *blob() const { return blob_; }
    const int64_t *offsets() const { return off_; }
};

// ---------------------------------------------------------------------------
// The column table (cpp/TableHolder.hpp).
// ---------------------------------------------------------------------------
class Table {
    const Config &cfg_;
    std::vector<std::string> names_;                 // column denominators
    std::vector<std::vector<std::string>> cols_;
    std::string first_file_;

    size_t index(const std::string &name) const {
        for (size_t k = 0; k < names_.size(); ++k)
            if (names_[k] == name) return k;
        throw std::runtime_error("Column " + name + " not contained in TableHolder!");
    }

  public:
    Table(const std::vector<std::string> &files, const Config &cfg) : cfg_(cfg) {
        const char sep = cfg.special(Config::Input, "separator");
        const char eol = cfg.special(Config::Input, "endline");
        const char quote = cfg.special(Config::Input, "quotation");
        names_.push_back("file_origin");
        std::vector<std::string> wanted;
        for (const auto &c : cfg.columns("select_columns_to_read")) {
            names_.push_back(c.first);
            wanted.push_back(c.second);
        }
        first_file_ = files.at(0);
        for (const auto &f : files) read_csv(f, sep, eol, quote, wanted, cols_);
        if (cols_.empty()) cols_.assign(names_.size(), {});
    }

    size_t rows() const { return cols_.empty() ? 0 : cols_[0].size(); }
    const std::vector<std::string> &column(const std::string &name) const { return cols_[index(name)]; }

    void delete_rows(const std::vector<char> &del) {
        size_t n = 0;
        for (char d : del) n += d != 0;
        Benchmark::instance().message("Deleting " + std::to_string(n) + " rows");
        for (auto &col : cols_) {
            size_t t = 0;
            for (size_t r = 0; r < col.size(); ++r) {
                if (del[r]) continue;
                if (t != r) col[t] = std::move(col[r]);   // no self-move: it may empty the string
                ++t;
            }
            col.resize(t);
        }
    }
    void delete_empty(const std::string &name) {
        const auto &col = cols_[index(name)];
        std::vector<char> del(col.size());
        for (size_t r = 0; r < col.size(); ++r) del[r] = col[r].empty();
        Benchmark::instance().message("Deleting empty rows for column " + name);
        delete_rows(del);
    }
    // append_column with make_output_string = std::to_string (cpp/TableHolder.hpp:56-66, 126-131)
    template <typename T>
    void append(const std::string &name, const std::vector<T> &v) {
        std::vector<std::string> col(rows());
        for (size_t r = 0; r < col.size(); ++r) col[r] = std::to_string(v[r]);
        append_strings(name, std::move(col));
    }
    void append_strings(const std::string &name, std::vector<std::string> col) {
        names_.push_back(name);
        cols_.push_back(std::move(col));
    }

    // cpp/TableHolder.hpp:275-348
    void cluster() {
        Benchmark &bm = Benchmark::instance();
        bm.start("Deleting Empty Rows");
        const std::string vcol = cfg_.opt("gene_columns.first_gene.name");
        const std::string jcol = cfg_.opt("gene_columns.second_gene.name");
        const std::string scol = cfg_.opt("sequence_columns.name");
        if (!scol.empty()) delete_empty(scol);
        if (!vcol.empty()) delete_empty(vcol);
        if (!jcol.empty()) delete_empty(jcol);
        bm.stop("Deleting Empty Rows");
        bm.start("Transferring data to device");
        const size_t n = rows();
        std::string vgb, jgb;
        std::vector<int64_t> vgo, jgo;
        // the three row columns are packed by all host threads into page-locked
        // blobs (idb_host_alloc), which idb_cluster copies at the link's full rate
        HostColumn vcolumn, jcolumn, scolumn;
        auto pack = [](const std::vector<std::string> &v, std::string &blob, std::vector<int64_t> &off) {
            off.assign(1, 0);
            size_t total = 0;
            for (const auto &x : v) total += x.size();
            blob.reserve(total);
            for (const auto &x : v) { blob += x; off.push_back((int64_t)blob.size()); }
        };
        auto genes = [](const std::string &file, std::vector<std::string> &out) {
            // cpp/GeneReader.hpp:65-76: one name per line, empty lines skipped
            std::ifstream f(file);
            if (!f.is_open()) throw std::runtime_error("Cannot read from file " + file);
            std::string line;
            while (std::getline(f, line))
                if (!line.empty()) out.push_back(line);
        };
        idb_input in = {};
        in.n_rows = (uint32_t)n;
        std::vector<std::string> vnames, jnames;
        if (!vcol.empty()) {
            vcolumn.pack(column(vcol));
            genes(cfg_.opt("gene_columns.first_gene.ref"), vnames);
            pack(vnames, vgb, vgo);
            in.v_calls = vcolumn.blob(); in.v_offsets = vcolumn.offsets();
            in.v_genes = vgb.data(); in.v_gene_offsets = vgo.data(); in.n_v_genes = (uint32_t)vnames.size();
        }
        if (!jcol.empty()) {
            jcolumn.pack(column(jcol));
            genes(cfg_.opt("gene_columns.second_gene.ref"), jnames);
            pack(jnames, jgb, jgo);
            in.j_calls = jcolumn.blob(); in.j_offsets = jcolumn.offsets();
            in.j_genes = jgb.data(); in.j_gene_offsets = jgo.data(); in.n_j_genes = (uint32_t)jnames.size();
        }
        if (!scol.empty()) {
            scolumn.pack(column(scol));
            in.seqs = scolumn.blob(); in.seq_offsets = scolumn.offsets();
        }
        bm.stop("Transferring data to device");
        idb_params prm = {};
        prm.threshold = cfg_.threshold();
        prm.abs_eps = cfg_.abs_eps();
        prm.min_pts = cfg_.min_pts();
        prm.use_hamming = cfg_.flag("use_hamming", false);
        prm.eval_trees = cfg_.flag("get_tree_depth_statistics", false);
        prm.schedule = cfg_.schedule();
        prm.candidates = cfg_.candidates();
        bm.message("DBSCAN settings: epsilon = " + std::to_string(prm.threshold));
        bm.message("DBSCAN settings: minPts = " + std::to_string(prm.min_pts));
        if (prm.use_hamming)
            bm.message("DBSCAN settings: using Hamming distance measure instead of Levenshtein distance");
        std::vector<uint32_t> clone(n), copies(n), hist(51);
        std::vector<int32_t> cores(n);
        idb_stats st = {};
        uint32_t nu = 0;
        idb_output out = {};
        out.clone_id = clone.data(); out.core = cores.data(); out.copies = copies.data();
        out.n_uniques = &nu;
        out.tree_depth_hist = prm.eval_trees ? hist.data() : nullptr;
        out.stats = &st;
        bm.start("Clustering core process");
        const idb_status rc = idb_cluster(nullptr, &in, &prm, &out);
        bm.stop("Clustering core process");
        if (rc != IDB_OK) {
            char msg[512];
            idb_last_error(msg, sizeof msg);
            throw std::runtime_error(std::string("clustering failed: ") + idb_status_string(rc) + ": " + msg);
        }
        bm.message("Total number of sequences = " + std::to_string(n));
        bm.message("Number of uniques = " + std::to_string(nu));
        bm.message("Number of core points = " + std::to_string(st.n_cores));
        if (prm.eval_trees) {
            bm.message("Union find tree depth structure");
            for (int d = 0; d <= 50; ++d)
                bm.message("Number of trees with depth " + std::to_string(d) + ": " + std::to_string(hist[d]));
        }
        bm.message("Total number of clusters = " + std::to_string(st.n_clusters));
        bm.message("Number of noise points = " + std::to_string(st.n_noise_rows));
        bm.message("Percentage of noise points = " +
                   std::to_string(n ? (100 * (uint64_t)st.n_noise_rows) / n : 0) + "%");
        append("clone_id", clone);
        append("copies", copies);
        append("cores", cores);
    }

    // cpp/TableHolder.hpp:217-271
    void write() {
        const char sep = cfg_.special(Config::Output, "separator");
        const char eol = cfg_.special(Config::Output, "endline");
        const char quote = cfg_.special(Config::Output, "quotation");
        if (cfg_.remove_noise()) {
            const auto &cid = cols_[index("clone_id")];
            std::vector<char> del(cid.size());
            for (size_t r = 0; r < cid.size(); ++r) del[r] = cid[r] == "0";
            Benchmark::instance().message("Deleting noise points");
            delete_rows(del);
        }
        std::vector<std::string> header;
        std::vector<const std::vector<std::string> *> sel;
        const auto outcols = cfg_.columns("select_columns_to_write");
        for (const auto &c : outcols) {
            bool present = false;
            for (const auto &nm : names_) present |= nm == c.first;
            if (!present) append_strings(c.first, std::vector<std::string>(rows()));
        }
        for (const auto &c : outcols) {
            header.push_back(c.second);
            sel.push_back(&cols_[index(c.first)]);
        }
        const std::string fn = cfg_.filename(first_file_, Config::Output);
        Benchmark::instance().message("Writing to file " + fn);
        write_csv(fn, sel, header, sep, eol, quote);
    }

    const std::string &first_file() const { return first_file_; }
};

}  // namespace psdb
