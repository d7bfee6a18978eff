// csv.hpp -- the CSV in/out surface of psdbscan.
//
// Tokenizer: the rules of boost::escaped_list_separator<char>('\\', sep, quote)
// that the reference uses for headers and rows (cpp/csvreader.hpp:56, 108):
// the separator splits fields outside quotes; the quote character toggles
// quoting and is dropped; the escape character '\\' followed by 'n' gives a
// newline, followed by the quote or the escape character gives that character,
// and anything else is an error.  An empty line has no fields.
//
// Reader (cpp/csvreader.hpp:101-189): the header line selects columns by name;
// every following line (split on the configured end-of-line character, one
// trailing '\r' removed) becomes a row -- including the empty row produced by a
// file that ends with an end-of-line character, as in the reference.
//
// Writer (cpp/csvwriter.hpp:37-73): header names unquoted, every value wrapped
// in the quotation character unless it is '\0'.
//
// The reference reads a file line by line, starting one task per line and
// waiting for it before the next (cpp/csvreader.hpp:152-180), and writes cell
// by cell through a stream (cpp/csvwriter.hpp:57-71).  Here a file is read in
// one piece, its lines are found and tokenized by all host threads (every
// line is independent: the reader splits on the end-of-line character before
// any quoting applies), and the output is formatted by all threads into
// per-range buffers written in order.  read_csv_serial / write_csv_serial keep
// the one-thread form as the check of the parallel one.
#pragma once
#include <algorithm>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace psdb {

// Threads for the host-side passes (at least 1).
inline unsigned host_threads() {
    const unsigned t = std::thread::hardware_concurrency();
    return t ? t : 1;
}

// Runs f(lo, hi) over [0, n) in contiguous ranges on up to host_threads()
// threads; exceptions are rethrown in the caller.
template <typename F>
void parallel_ranges(size_t n, F f, size_t min_per_thread = 4096) {
    const size_t t = std::max<size_t>(1, std::min<size_t>(host_threads(), n / min_per_thread));
    if (t <= 1) {
        f((size_t)0, n);
        return;
    }
    std::vector<std::thread> pool;
    std::vector<std::exception_ptr> err(t);
    for (size_t k = 0; k < t; ++k)
        pool.emplace_back([&, k] {
            try {
                f(n * k / t, n * (k + 1) / t);
            } catch (...) {
                err[k] = std::current_exception();
            }
        });
    for (auto &th : pool) th.join();
    for (auto &e : err)
        if (e) std::rethrow_exception(e);
}

inline std::vector<std::string> tokenize(const std::string &line, char sep, char quote,
                                         char esc = '\\') {
    std::vector<std::string> out;
    if (line.empty()) return out;
    std::string tok;
    bool in_quote = false;
    for (size_t i = 0; i < line.size(); ++i) {
        const char c = line[i];
        if (c == esc) {
            if (i + 1 >= line.size()) throw std::runtime_error("cannot end with escape");
            const char n = line[++i];
            if (n == 'n') tok.push_back('\n');
            else if (n == quote || n == esc) tok.push_back(n);
            else throw std::runtime_error("unknown escape sequence");
        } else if (c == sep && !in_quote) {
            out.push_back(tok);
            tok.clear();
        } else if (c == quote) {
            in_quote = !in_quote;
        } else {
            tok.push_back(c);
        }
    }
    out.push_back(tok);
    return out;
}

inline void purify_line(std::string &line) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
}

// Header line -> column order (order[t] = table column of field t, -1 = unused).
inline std::vector<int> header_order(const std::string &header_line, char sep, char quote,
                                     const std::vector<std::string> &wanted,
                                     const std::string &filename) {
    const std::vector<std::string> header = tokenize(header_line, sep, quote);
    std::vector<int> order(header.size(), -1);
    for (size_t k = 0; k < wanted.size(); ++k) {
        size_t pos = 0;
        while (pos < header.size() && header[pos] != wanted[k]) ++pos;
        if (pos == header.size())
            throw std::runtime_error("Required column " + wanted[k] + " not found in " + filename);
        order[pos] = (int)k + 1;
    }
    return order;
}

// Reads one input file into the column table.  cols[0] is "file_origin";
// cols[1..] follow `wanted` (header strings of select_columns_to_read).  Rows
// of several files are appended in file order.
inline void read_csv(const std::string &filename, char sep, char eol, char quote,
                     const std::vector<std::string> &wanted,
                     std::vector<std::vector<std::string>> &cols) {
    std::ifstream f(filename, std::ios::binary | std::ios::ate);
    if (!f.is_open()) throw std::runtime_error("Cannot read from file " + filename);
    const std::streamoff size = f.tellg();
    std::string buf((size_t)std::max<std::streamoff>(size, 0), '\0');
    f.seekg(0);
    if (size > 0 && !f.read(&buf[0], size)) throw std::runtime_error("Cannot read from file " + filename);
    // line starts: the header ends at the first eol; the byte after it and
    // after every later eol starts a row (so a file ending in an eol has a
    // final empty row, as the reference's reader produces); a file without an
    // eol has the header only
    const size_t n = buf.size();
    const char *b = buf.data();
    const char *h = static_cast<const char *>(std::memchr(b, eol, n));
    const size_t hdr_end = h ? (size_t)(h - b) : n;
    std::string hline(b, hdr_end);
    purify_line(hline);
    const std::vector<int> order = header_order(hline, sep, quote, wanted, filename);
    if (cols.size() != wanted.size() + 1) cols.assign(wanted.size() + 1, {});
    std::vector<size_t> starts;
    if (h) {
        const size_t body = hdr_end + 1;
        const unsigned t = (unsigned)std::max<size_t>(1, std::min<size_t>(host_threads(), (n - body) >> 16));
        std::vector<std::vector<size_t>> part(t);
        parallel_ranges(t, [&](size_t lo, size_t hi) {
            for (size_t k = lo; k < hi; ++k) {
                const size_t a = body + (n - body) * k / t, z = body + (n - body) * (k + 1) / t;
                for (const char *p = b + a; (p = static_cast<const char *>(std::memchr(p, eol, (size_t)(b + z - p))));
                     ++p)
                    part[k].push_back((size_t)(p - b) + 1);
            }
        }, 1);
        starts.push_back(body);
        for (auto &pv : part) starts.insert(starts.end(), pv.begin(), pv.end());
    }
    const size_t rows = starts.size(), base = cols[0].size();
    for (auto &c : cols) c.resize(base + rows);
    parallel_ranges(rows, [&](size_t lo, size_t hi) {
        std::string line;
        for (size_t r = lo; r < hi; ++r) {
            const size_t a = starts[r];
            const size_t z = r + 1 < rows ? starts[r + 1] - 1 : n;   // the eol is not part of the line
            line.assign(b + a, z > a ? z - a : 0);
            purify_line(line);
            const std::vector<std::string> tok = tokenize(line, sep, quote);
            cols[0][base + r] = filename;
            for (size_t t = 0; t < tok.size() && t < order.size(); ++t)
                if (order[t] >= 0) cols[order[t]][base + r] = tok[t];
        }
    }, 1024);
}

// The one-thread reader (getline per row), kept as the check of read_csv.
inline void read_csv_serial(const std::string &filename, char sep, char eol, char quote,
                            const std::vector<std::string> &wanted,
                            std::vector<std::vector<std::string>> &cols) {
    std::ifstream f(filename, std::ios::binary);
    if (!f.is_open()) throw std::runtime_error("Cannot read from file " + filename);
    std::string line;
    std::getline(f, line, eol);
    purify_line(line);
    const std::vector<int> order = header_order(line, sep, quote, wanted, filename);
    if (cols.size() != wanted.size() + 1) cols.assign(wanted.size() + 1, {});
    // every line after the header, including a final empty one
    while (!f.eof()) {
        std::getline(f, line, eol);
        purify_line(line);
        const std::vector<std::string> tok = tokenize(line, sep, quote);
        for (auto &c : cols) c.emplace_back();
        cols[0].back() = filename;
        for (size_t t = 0; t < tok.size() && t < order.size(); ++t)
            if (order[t] >= 0) cols[order[t]].back() = tok[t];
    }
}

// Rows [lo, hi) formatted as the writer formats them.
inline void format_rows(std::string &buf, const std::vector<const std::vector<std::string> *> &cols,
                        size_t lo, size_t hi, char sep, char eol, char quote) {
    for (size_t r = lo; r < hi; ++r) {
        for (size_t k = 0; k < cols.size(); ++k) {
            if (quote != '\0') buf.push_back(quote);
            buf += (*cols[k])[r];
            if (quote != '\0') buf.push_back(quote);
            if (k + 1 < cols.size()) buf.push_back(sep);
        }
        buf.push_back(eol);
    }
}

inline void write_csv(const std::string &filename, const std::vector<const std::vector<std::string> *> &cols,
                      const std::vector<std::string> &header, char sep, char eol, char quote) {
    std::ofstream out(filename, std::ios::binary);
    if (!out.is_open()) throw std::runtime_error("Cannot write to file " + filename);
    std::string head;
    for (size_t k = 0; k < header.size(); ++k) {
        head += header[k];
        if (k + 1 < header.size()) head.push_back(sep);
    }
    head.push_back(eol);
    out.write(head.data(), (std::streamsize)head.size());
    const size_t n = cols.empty() ? 0 : cols[0]->size();
    // blocks of rows, each formatted by one thread, written in order
    const size_t block = 1u << 16;
    const size_t nblocks = (n + block - 1) / block;
    const size_t wave = std::max<size_t>(1, host_threads());
    std::vector<std::string> bufs(wave);
    for (size_t b0 = 0; b0 < nblocks; b0 += wave) {
        const size_t nb = std::min(wave, nblocks - b0);
        parallel_ranges(nb, [&](size_t lo, size_t hi) {
            for (size_t k = lo; k < hi; ++k) {
                bufs[k].clear();
                const size_t r0 = (b0 + k) * block;
                format_rows(bufs[k], cols, r0, std::min(n, r0 + block), sep, eol, quote);
            }
        }, 1);
        for (size_t k = 0; k < nb; ++k) out.write(bufs[k].data(), (std::streamsize)bufs[k].size());
    }
    if (!out) throw std::runtime_error("Cannot write to file " + filename);
}

// The one-thread writer, kept as the check of write_csv.
inline void write_csv_serial(const std::string &filename,
                             const std::vector<const std::vector<std::string> *> &cols,
                             const std::vector<std::string> &header, char sep, char eol, char quote) {
    std::ofstream out(filename, std::ios::binary);
    if (!out.is_open()) throw std::runtime_error("Cannot write to file " + filename);
    std::string buf;
    for (size_t k = 0; k < header.size(); ++k) {
        buf += header[k];
        if (k + 1 < header.size()) buf.push_back(sep);
    }
    buf.push_back(eol);
    const size_t n = cols.empty() ? 0 : cols[0]->size();
    for (size_t r = 0; r < n; ++r) {
        for (size_t k = 0; k < cols.size(); ++k) {
            if (quote != '\0') buf.push_back(quote);
            buf += (*cols[k])[r];
            if (quote != '\0') buf.push_back(quote);
            if (k + 1 < cols.size()) buf.push_back(sep);
        }
        buf.push_back(eol);
        if (buf.size() > (1u << 22)) {
            out.write(buf.data(), (std::streamsize)buf.size());
            buf.clear();
        }
    }
    out.write(buf.data(), (std::streamsize)buf.size());
}

}  // namespace psdb
