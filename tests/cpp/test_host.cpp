// CPU test of the psdbscan host surface: INFO reader, CSV tokenizer, reader and
// writer.  Exit status 0 = all checks passed.  argv[1] = scratch directory.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "csv.hpp"
#include "info.hpp"

static int g_fail = 0;
#define CHECK(cond)                                                             \
    do {                                                                        \
        if (!(cond)) {                                                          \
            std::cerr << __FILE__ << ":" << __LINE__ << ": " #cond "\n";        \
            ++g_fail;                                                           \
        }                                                                       \
    } while (0)

template <typename F>
static bool throws(F f) {
    try {
        f();
    } catch (const std::exception &) {
        return true;
    }
    return false;
}

static std::string slurp(const std::string &f) {
    std::ifstream in(f, std::ios::binary);
    std::ostringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

int main(int argc, char **argv) {
    using namespace psdb;
    const std::string dir = argc > 1 ? argv[1] : ".";

    // ---- INFO reader -------------------------------------------------------
    const std::string conf =
        "; comment line\n"
        "input_settings\n"
        "{\n"
        "\tseparator \"\\t\"     ; tab\n"
        "\tendline   \"\\n\"\n"
        "\tquotation \"\\\"\"\n"
        "}\n"
        "output_settings {\n quotation \"\\0\"\n separator \",\" }\n"
        "select_columns_to_read\n"
        "{\n"
        "\tb_col  \"Second\"\n"
        "\ta_col  \"First name\"\n"
        "\tb_col  \"dup\"\n"
        "}\n"
        "gene_columns\n"
        "{\n"
        "\tfirst_gene\n"
        "\t{\n"
        "\t\tname\tv_col\n"
        "\t\tref\t\"genes.txt\"\n"
        "\t}\n"
        ";\tsecond_gene { name j }\n"
        "}\n"
        "sequence_columns\n"
        "{\n"
        ";\tname  cdr3\n"
        "}\n"
        "maximum_relative_edit_distance 0.15\n"
        "use_hamming false\n"
        "flag1 1\n"
        "empty_value\n";
    InfoNode t = read_info_string(conf);
    CHECK(as_char(t.get("input_settings.separator"), "") == '\t');
    CHECK(as_char(t.get("input_settings.endline"), "") == '\n');
    CHECK(as_char(t.get("input_settings.quotation"), "") == '"');
    CHECK(t.get("output_settings.quotation").size() == 1 && t.get("output_settings.quotation")[0] == '\0');
    CHECK(as_char(t.get("output_settings.separator"), "") == ',');
    const auto &cols = t.child("select_columns_to_read").children;
    CHECK(cols.size() == 3);
    CHECK(cols[0].key == "b_col" && cols[0].data == "Second");
    CHECK(cols[1].key == "a_col" && cols[1].data == "First name");
    CHECK(cols[2].data == "dup");
    CHECK(t.get("gene_columns.first_gene.name") == "v_col");
    CHECK(t.get("gene_columns.first_gene.ref") == "genes.txt");
    CHECK(!t.has("gene_columns.second_gene.name"));
    CHECK(!t.has("sequence_columns.name"));
    CHECK(as_float(t.get("maximum_relative_edit_distance"), "") == 0.15f);
    CHECK(as_bool(t.get("use_hamming"), "") == false);
    CHECK(as_bool(t.get("flag1"), "") == true);
    CHECK(t.get("empty_value").empty());
    CHECK(throws([&] { as_char("ab", "x"); }));
    CHECK(throws([&] { as_bool("yes", "x"); }));
    CHECK(throws([&] { read_info_string("a {\n b 1\n"); }));       // missing '}'
    CHECK(throws([&] { read_info_string("}\n"); }));                // unmatched
    CHECK(throws([&] { read_info_string("a \"unterminated\n"); }));
    CHECK(throws([&] { read_info_string("a \"\\q\"\n"); }));        // bad escape
    CHECK(throws([&] { read_info_string("a 1 b 2\n"); }));             // two pairs on a line
    // #include relative to the including file
    {
        std::ofstream(dir + "/inc_child.conf") << "included_key 42\nblock { x 1 }\n";
        std::ofstream(dir + "/inc_main.conf") << "top 1\n#include \"inc_child.conf\"\nlast 2\n";
        InfoNode m = read_info(dir + "/inc_main.conf");
        CHECK(m.get("included_key") == "42");
        CHECK(m.get("block.x") == "1");
        CHECK(m.children.size() == 4 && m.children[3].key == "last");
    }

    // ---- tokenizer: boost::escaped_list_separator rules ---------------------
    CHECK(tokenize("", ',', '"').empty());
    CHECK((tokenize("a,b,,c", ',', '"') == std::vector<std::string>{"a", "b", "", "c"}));
    CHECK((tokenize(",", ',', '"') == std::vector<std::string>{"", ""}));
    CHECK((tokenize("\"a,b\",c", ',', '"') == std::vector<std::string>{"a,b", "c"}));
    CHECK((tokenize("x\"y\"z", ',', '"') == std::vector<std::string>{"xyz"}));
    CHECK((tokenize("a\\nb,c\\\\d,\\\"q", ',', '"') == std::vector<std::string>{"a\nb", "c\\d", "\"q"}));
    CHECK((tokenize("a\tb", '\t', '"') == std::vector<std::string>{"a", "b"}));
    CHECK(throws([] { tokenize("a\\x", ',', '"'); }));
    CHECK(throws([] { tokenize("a\\", ',', '"'); }));

    // ---- reader --------------------------------------------------------------
    {
        const std::string f = dir + "/in.tsv";
        std::ofstream(f, std::ios::binary) << "ID\tSeq\tV\r\n1\tCAR\tIGHV1*01\r\n2\t\tIGHV2*01\n3\t\"CA\tK\"\tx\n";
        std::vector<std::vector<std::string>> c;
        read_csv(f, '\t', '\n', '"', {"V", "Seq"}, c);
        CHECK(c.size() == 3);
        // 3 data lines + the trailing empty row of the final newline
        CHECK(c[0].size() == 4);
        CHECK(c[0][0] == f);
        CHECK(c[1][0] == "IGHV1*01" && c[2][0] == "CAR");
        CHECK(c[2][1].empty());
        CHECK(c[2][2] == "CA\tK");
        CHECK(c[1][3].empty() && c[2][3].empty());
        // a second file appends
        read_csv(f, '\t', '\n', '"', {"V", "Seq"}, c);
        CHECK(c[0].size() == 8);
        CHECK(throws([&] {
            std::vector<std::vector<std::string>> d;
            read_csv(f, '\t', '\n', '"', {"Missing"}, d);
        }));
        CHECK(throws([&] {
            std::vector<std::vector<std::string>> d;
            read_csv(dir + "/does_not_exist.tsv", '\t', '\n', '"', {"V"}, d);
        }));
        // no trailing newline: no extra row
        std::ofstream(dir + "/in2.tsv", std::ios::binary) << "A,B\n1,2\n3,4";
        std::vector<std::vector<std::string>> e;
        read_csv(dir + "/in2.tsv", ',', '\n', '"', {"B"}, e);
        CHECK(e[0].size() == 2 && e[1][1] == "4");
    }

    // ---- writer --------------------------------------------------------------
    {
        std::vector<std::string> a{"1", "2"}, b{"x", ""};
        write_csv(dir + "/out1.csv", {&a, &b}, {"A", "B"}, '\t', '\n', '\0');
        CHECK(slurp(dir + "/out1.csv") == "A\tB\n1\tx\n2\t\n");
        write_csv(dir + "/out2.csv", {&a, &b}, {"A", "B"}, ',', '\n', '"');
        CHECK(slurp(dir + "/out2.csv") == "A,B\n\"1\",\"x\"\n\"2\",\"\"\n");
    }

    std::printf("host failures: %d\n", g_fail);
    return g_fail ? 1 : 0;
}
