// vx3g_sim -- command-line runner in the manner of voxcraft-sim / vx3_node_worker
// (src/Executables/voxcraft-sim.cpp:25-132, vx3_node_worker.cu:32-142):
//
//   vx3g_sim -i <input_dir> -o <report.xml> [--mixed] [--max-steps N]
//            [--devices N] [--device-map d0,d1,...]
//
// <input_dir> holds base.vxa and the *.vxd files to simulate (one robot each).  The
// files are dealt round-robin into N sub-batches (vx3_node_worker.cu:88-93; default
// one per visible GPU), sub-batch i runs on device i (or the i-th entry of
// --device-map), all sub-batches at once; the report lists the results sorted by
// fitness, and RecordHistory settings print the history text to stdout.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "../../include/vx3_simulation_manager.h"
#include "../../include/vx3g.h"

#include <cuda_runtime.h>

namespace fs = std::filesystem;

int main(int argc, char **argv) {
    std::string in, out = "output.xml";
    int precision = VX3G_PRECISION_FP64;
    long max_steps = 1000000;
    int n_dev = 0;
    std::vector<int> device_map;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
        else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
        else if (a == "--mixed") precision = VX3G_PRECISION_MIXED;
        else if (a == "--max-steps" && i + 1 < argc) max_steps = std::atol(argv[++i]);
        else if (a == "--devices" && i + 1 < argc) n_dev = std::atoi(argv[++i]);
        else if (a == "--device-map" && i + 1 < argc) {
            std::string m = argv[++i];
            for (size_t p = 0; p <= m.size();) {
                size_t q = m.find(',', p);
                if (q == std::string::npos) q = m.size();
                device_map.push_back(std::atoi(m.substr(p, q - p).c_str()));
                p = q + 1;
            }
        } else {
            fprintf(stderr, "usage: %s -i <input_dir> -o <report.xml> [--mixed] [--max-steps N] [--devices N] "
                            "[--device-map d0,d1,...]\n", argv[0]);
            return 2;
        }
    }
    if (n_dev <= 0) {
        int visible = 0;
        if (cudaGetDeviceCount(&visible) != cudaSuccess || visible <= 0) {
            fprintf(stderr, "ERROR: No GPU found.\n");
            return 1;
        }
        n_dev = visible;
    }
    if (!device_map.empty() && (int)device_map.size() < n_dev) {
        fprintf(stderr, "ERROR: --device-map needs %d entries\n", n_dev);
        return 2;
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
    std::vector<std::vector<fs::path>> sub_batches(n_dev);
    for (size_t i = 0; i < files.size(); i++) sub_batches[i % n_dev].push_back(files[i]);
    try {
        VX3_SimulationManager sm(sub_batches, dir / "base.vxa", dir, n_dev);
        sm.devices = device_map;
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
