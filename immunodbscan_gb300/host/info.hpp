// info.hpp -- reader for the INFO configuration format of psdbscan.
//
// The reference reads its configuration with boost::property_tree::read_info
// (cpp/ConfigHolder.hpp:57-60, 325); Boost is not a dependency here, so this is
// a reader for the same format:
//   key value            ; a comment runs to the end of the line
//   key "quoted value"   ; escapes \0 \a \b \f \n \r \t \v \' \" \\ (\0 = NUL)
//   key { child 1 }      ; children, also with '{' on the following line
//   #include "file"      ; relative to the including file
// Children keep their order (select_columns_to_read / _write depend on it) and
// keys may repeat.  Paths use '.' as separator (property_tree's default).
#pragma once
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace psdb {

struct InfoNode {
    std::string key;
    std::string data;
    std::vector<InfoNode> children;

    const InfoNode *find(const std::string &k) const {
        for (const auto &c : children)
            if (c.key == k) return &c;
        return nullptr;
    }
    // dotted path lookup; nullptr if absent
    const InfoNode *path(const std::string &p) const {
        const InfoNode *n = this;
        size_t pos = 0;
        while (n && pos <= p.size()) {
            size_t dot = p.find('.', pos);
            std::string part = p.substr(pos, dot == std::string::npos ? std::string::npos : dot - pos);
            n = n->find(part);
            if (dot == std::string::npos) break;
            pos = dot + 1;
        }
        return n;
    }
    const InfoNode &child(const std::string &p) const {
        const InfoNode *n = path(p);
        if (!n) throw std::runtime_error("No such node (" + p + ")");
        return *n;
    }
    const std::string &get(const std::string &p) const { return child(p).data; }
    bool has(const std::string &p) const { return path(p) != nullptr; }
};

class InfoError : public std::runtime_error {
  public:
    InfoError(const std::string &file, int line, const std::string &msg)
        : std::runtime_error(file + "(" + std::to_string(line) + "): " + msg) {}
};

namespace detail {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

inline void skip_ws(const std::string &s, size_t &i) {
    while (i < s.size() && is_space(s[i])) ++i;
}

inline char unescape(char c, const std::string &file, int line) {
    switch (c) {
        case '0': return '\0';
        case 'a': return '\a';
        case 'b': return '\b';
        case 'f': return '\f';
        case 'n': return '\n';
        case 'r': return '\r';
        case 't': return '\t';
        case 'v': return '\v';
        case '"': return '"';
        case '\'': return '\'';
        case '\\': return '\\';
    }
    throw InfoError(file, line, std::string("unknown escape sequence \\") + c);
}

// a bare word or a quoted string starting at s[i]; returns false at end / comment / brace
inline bool token(const std::string &s, size_t &i, std::string &out, const std::string &file,
                  int line) {
    skip_ws(s, i);
    if (i >= s.size() || s[i] == ';' || s[i] == '{' || s[i] == '}') return false;
    out.clear();
    if (s[i] == '"') {
        ++i;
        while (true) {
            if (i >= s.size()) throw InfoError(file, line, "unterminated string");
            char c = s[i++];
            if (c == '"') break;
            if (c == '\\') {
                if (i >= s.size()) throw InfoError(file, line, "unterminated escape");
                out.push_back(unescape(s[i++], file, line));
            } else {
                out.push_back(c);
            }
        }
        return true;
    }
    while (i < s.size() && !is_space(s[i]) && s[i] != ';' && s[i] != '{' && s[i] != '}')
        out.push_back(s[i++]);
    return true;
}

inline std::string dir_of(const std::string &f) {
    size_t p = f.find_last_of('/');
    return p == std::string::npos ? std::string() : f.substr(0, p + 1);
}

inline void parse_stream(std::istream &in, const std::string &file, InfoNode &root, int depth);

inline void parse_file(const std::string &file, InfoNode &root, int depth) {
    if (depth > 32) throw InfoError(file, 0, "#include nesting too deep");
    std::ifstream f(file);
    if (!f.is_open()) throw InfoError(file, 0, "cannot open file");
    parse_stream(f, file, root, depth);
}

inline void parse_stream(std::istream &in, const std::string &file, InfoNode &root, int depth) {
    std::vector<InfoNode *> stack{&root};
    InfoNode *last = nullptr;   // the node a following '{' opens
    std::string line;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        size_t i = 0;
        skip_ws(line, i);
        if (i < line.size() && line[i] == '#') {
            const std::string kw = "#include";
            if (line.compare(i, kw.size(), kw) != 0) throw InfoError(file, lineno, "unknown directive");
            i += kw.size();
            std::string inc;
            if (!token(line, i, inc, file, lineno)) throw InfoError(file, lineno, "#include without file");
            parse_file(inc.size() && inc[0] == '/' ? inc : dir_of(file) + inc, *stack.back(), depth + 1);
            last = nullptr;
            continue;
        }
        while (true) {
            skip_ws(line, i);
            if (i >= line.size() || line[i] == ';') break;
            if (line[i] == '{') {
                if (!last) throw InfoError(file, lineno, "'{' without a key");
                stack.push_back(last);
                last = nullptr;
                ++i;
                continue;
            }
            if (line[i] == '}') {
                if (stack.size() <= 1) throw InfoError(file, lineno, "unmatched '}'");
                stack.pop_back();
                last = nullptr;
                ++i;
                continue;
            }
            std::string key, data;
            token(line, i, key, file, lineno);
            token(line, i, data, file, lineno);
            stack.back()->children.push_back(InfoNode{key, data, {}});
            last = &stack.back()->children.back();
            // a further token on the same line would be a syntax error in INFO
            skip_ws(line, i);
            if (i < line.size() && line[i] != ';' && line[i] != '{' && line[i] != '}')
                throw InfoError(file, lineno, "unexpected text after value");
        }
    }
    if (stack.size() != 1) throw InfoError(file, lineno, "missing '}'");
}

}  // namespace detail

inline InfoNode read_info(const std::string &file) {
    InfoNode root;
    detail::parse_file(file, root, 0);
    return root;
}

inline InfoNode read_info_string(const std::string &text, const std::string &name = "<string>") {
    InfoNode root;
    std::istringstream in(text);
    detail::parse_stream(in, name, root, 0);
    return root;
}

// value conversions with property_tree's meaning
inline char as_char(const std::string &v, const std::string &what) {
    if (v.size() != 1) throw std::runtime_error("conversion of data to type \"char\" failed (" + what + ")");
    return v[0];
}

inline bool as_bool(const std::string &v, const std::string &what) {
    if (v == "true" || v == "1") return true;
    if (v == "false" || v == "0") return false;
    throw std::runtime_error("conversion of data to type \"bool\" failed (" + what + ")");
}

inline float as_float(const std::string &v, const std::string &what) {
    char *end = nullptr;
    const float f = std::strtof(v.c_str(), &end);
    if (v.empty() || *end) throw std::runtime_error("conversion of data to type \"float\" failed (" + what + ")");
    return f;
}

inline long long as_int(const std::string &v, const std::string &what) {
    char *end = nullptr;
    const long long x = std::strtoll(v.c_str(), &end, 10);
    if (v.empty() || *end) throw std::runtime_error("conversion of data to an integer failed (" + what + ")");
    return x;
}

}  // namespace psdb
