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
#pragma once
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace psdb {

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

// Reads one input file into the column table.  cols[0] is "file_origin";
// cols[1..] follow `wanted` (header strings of select_columns_to_read).
inline void read_csv(const std::string &filename, char sep, char eol, char quote,
                     const std::vector<std::string> &wanted,
                     std::vector<std::vector<std::string>> &cols) {
    std::ifstream f(filename, std::ios::binary);
    if (!f.is_open()) throw std::runtime_error("Cannot read from file " + filename);
    std::string line;
    std::getline(f, line, eol);
    purify_line(line);
    const std::vector<std::string> header = tokenize(line, sep, quote);
    std::vector<int> order(header.size(), -1);
    for (size_t k = 0; k < wanted.size(); ++k) {
        size_t pos = 0;
        while (pos < header.size() && header[pos] != wanted[k]) ++pos;
        if (pos == header.size())
            throw std::runtime_error("Required column " + wanted[k] + " not found in " + filename);
        order[pos] = (int)k + 1;
    }
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

inline void write_csv(const std::string &filename, const std::vector<const std::vector<std::string> *> &cols,
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
