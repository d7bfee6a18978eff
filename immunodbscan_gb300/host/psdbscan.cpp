// psdbscan -- command-line host of the GB300 clone-collapsing path.
//
// Same options and defaults as the reference's psdbscan (cpp/psdbscan.cpp:25-106):
//   psdbscan [--help] [--input f1 [f2 ...]] [--config_file f] [--verbose]
// defaults data/psdbscan.conf and data/ExampleData.csv.  Reads the input
// table(s), clusters through the C ABI (idb_cluster), writes the output table
// and the benchmark log named by the configuration.
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "table.hpp"

namespace {

void usage() {
    std::cout << "Allowed options:\n"
                 "  --help                produce help message\n"
                 "  --input arg           set input file (csv format, settings may need to be "
                 "adjusted in config file)\n"
                 "  --config_file arg     set config file (boost property_tree info file data "
                 "format)\n"
                 "  --verbose             Print some status information during data processing.\n";
}

}  // namespace

int main(int argc, char **argv) {
    // more hardware work queues than CUDA's default 8, before the first CUDA
    // call: the library's copy, side and main streams then never share a
    // queue with one another (a shared queue serialises unrelated streams and
    // stalled single calls by tens of milliseconds); a value the user set wins
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    using psdb::Benchmark;
    Benchmark &bm = Benchmark::instance();
    bm.start("Overall");
    std::vector<std::string> inputs;
    std::string conf = "data/psdbscan.conf";
    bool help = false;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        std::string val;
        const size_t eq = a.find('=');
        if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
            val = a.substr(eq + 1);
            a = a.substr(0, eq);
        }
        if (a == "--help") {
            help = true;
        } else if (a == "--verbose") {
            bm.be_verbose();
        } else if (a == "--config_file") {
            if (val.empty()) {
                if (i + 1 >= argc) { std::cerr << "the required argument for option '--config_file' is missing\n"; return 1; }
                val = argv[++i];
            }
            conf = val;
        } else if (a == "--input") {
            if (!val.empty()) inputs.push_back(val);
            while (i + 1 < argc && std::string(argv[i + 1]).rfind("--", 0) != 0) inputs.push_back(argv[++i]);
            if (inputs.empty()) { std::cerr << "the required argument for option '--input' is missing\n"; return 1; }
        } else {
            std::cerr << "unrecognised option '" << a << "'\n";
            return 1;
        }
    }
    if (help) {
        usage();
        return 1;
    }
    if (inputs.empty()) inputs.push_back("data/ExampleData.csv");
    std::cout << "\n\n***************************************** PSDBSCAN "
                 "************************************************\n";
    try {
        psdb::Config cfg(conf);
        for (const auto &f : inputs) bm.message("Input file(s) " + f);
        bm.message("Using configuration file " + conf);
        std::cout << "\nReading files ... \n";
        bm.start("Reading Files");
        psdb::Table table(inputs, cfg);
        bm.stop("Reading Files");
        std::cout << "\nStarting clustering process... \n";
        bm.start("Do clustering");
        table.cluster();
        bm.stop("Do clustering");
        std::cout << "\nWriting output ... \n";
        bm.start("Writing Output");
        table.write();
        bm.stop("Writing Output");
        std::cout << "\nFinished!\n\n";
        bm.stop("Overall");
        std::cout << "\n\n***************************************************************************************************\n";
        bm.write(cfg.filename(inputs[0], psdb::Config::Bench));
    } catch (const std::exception &e) {
        std::cerr << "psdbscan: " << e.what() << "\n";
        return 2;
    }
    return 0;
}
