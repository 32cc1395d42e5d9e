// vx3g_sim -- command-line runner in the manner of voxcraft-sim / vx3_node_worker
// (src/Executables/voxcraft-sim.cpp:25-132, vx3_node_worker.cu:32-142):
//
//   vx3g_sim -i <input_dir> -o <report.xml> [--mixed] [--max-steps N]
//
// <input_dir> holds base.vxa and the *.vxd files to simulate (one robot each);
// every VXD runs on device 0 as one batch; the report lists the results sorted
// by fitness, and RecordHistory settings print the history text to stdout.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "../../include/vx3_simulation_manager.h"
#include "../../include/vx3g.h"

namespace fs = std::filesystem;

int main(int argc, char **argv) {
    std::string in, out = "output.xml";
    int precision = VX3G_PRECISION_FP64;
    long max_steps = 1000000;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
        else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
        else if (a == "--mixed") precision = VX3G_PRECISION_MIXED;
        else if (a == "--max-steps" && i + 1 < argc) max_steps = std::atol(argv[++i]);
        else {
            fprintf(stderr, "usage: %s -i <input_dir> -o <report.xml> [--mixed] [--max-steps N]\n", argv[0]);
            return 2;
        }
    }
    fs::path dir(in);
    if (in.empty() || !fs::exists(dir / "base.vxa")) {
        fprintf(stderr, "ERROR: no base.vxa in %s\n", in.c_str());
        return 1;
    }
    std::vector<fs::path> files;
    for (auto &e : fs::directory_iterator(dir))
        if (e.path().extension() == ".vxd") files.push_back(e.path().filename());
    std::sort(files.begin(), files.end());
    if (files.empty()) {
        fprintf(stderr, "ERROR: no .vxd files in %s\n", in.c_str());
        return 1;
    }
    try {
        VX3_SimulationManager sm({files}, dir / "base.vxa", dir, 1);
        sm.precision = precision;
        sm.max_steps = max_steps;
        sm.start();
        vx3_write_report(out, dir.filename().string(), sm.h_results);
    } catch (const std::exception &e) {
        fprintf(stderr, "ERROR: %s\n", e.what());
        return 1;
    }
    return 0;
}
