// vx3_simulation_manager.h -- C++ drop-in for the reference's
// VX3_SimulationManager (src/VX3/VX3_SimulationManager.cuh:15-48), running the
// GB300 step of libvx3g.so underneath.
//
// Same constructor shape, same start() and h_results; std::filesystem::path
// stands in for boost::filesystem::path.  Each sub-batch (one per device) is
// read the way readVXD does it (base VXA + each VXD merged by its
// replace="..." children, src/Utils/ctool.h:49-57), simulated as one vx3g
// batch until each robot's StopConditionFormula holds (or it diverges; the formula
// reads the centre of mass as the reference samples it, every int(TempPeriod / dt)
// steps, src/VX3/VX3_VoxelyzeKernel.cu:313-320), and
// collected into VX3_SimulationResult records sorted by fitness
// (VX3_SimulationResult.h:26-33).  With RecordStepSize > 0 the history text of
// CUDA_Simulation (src/VX3/VX3_SimulationManager.cu:40-114) is written to
// `history` (stdout by default).  Simulator/SecondaryExperiment: material removal
// runs inside the step, the initial-position reset
// (ReinitializeInitialPositionAfterThisManySeconds, :344-348) here between chunks.
#pragma once

#include <cstdio>
#include <filesystem>
#include <string>
#include <vector>

struct VX3_Vec3 {
    double x = 0, y = 0, z = 0;
};

struct VX3_SimulationResult {
    double x = 0, y = 0, z = 0;
    double voxSize = 0;
    double currentTime = 0.0;
    int num_voxel = 0;
    int num_measured_voxel = 0;
    double fitness_score = 0;
    std::string vxa_filename;
    bool SavePositionOfAllVoxels = false;
    std::vector<int> voxel_mats;
    std::vector<VX3_Vec3> voxel_init_pos;
    std::vector<VX3_Vec3> voxel_position;
    double total_distance_of_all_voxels = 0.0;
    VX3_Vec3 initialCenterOfMass;
    VX3_Vec3 currentCenterOfMass;
    int numClosePairs = 0;
    int status = 0;  // vx3g per-robot status word at the end (VX3G_ROBOT_*)
    long steps = 0;

    static bool compareFitnessScore(const VX3_SimulationResult &i1, const VX3_SimulationResult &i2);
};

class VX3_SimulationManager {
  public:
    VX3_SimulationManager(std::vector<std::vector<std::filesystem::path>> in_sub_batches, std::filesystem::path in_base,
                          std::filesystem::path in_input_dir, int in_num_of_devices);
    ~VX3_SimulationManager();

    // Runs every sub-batch to its stop conditions, all at once: one host thread per
    // sub-batch, each driving its own device (sub-batch i on device i, or devices[i]);
    // fills and sorts h_results.  Throws std::runtime_error with the library's message
    // on failure (the first failing sub-batch's, after all have finished).
    void start();

    std::vector<std::vector<std::filesystem::path>> sub_batches;
    std::filesystem::path base;
    std::filesystem::path input_dir;
    int num_of_devices;
    std::vector<VX3_SimulationResult> h_results;

    // GB300 options (no counterpart in the reference)
    int precision = 0;           // VX3G_PRECISION_FP64 or VX3G_PRECISION_MIXED
    long max_steps = 1000000;    // CUDA_Simulation's loop bound
    FILE *history = stdout;      // history text sink when RecordStepSize > 0
    std::vector<int> devices;    // device of each sub-batch (empty: sub-batch i on device i)

  private:
    std::vector<VX3_SimulationResult> run_sub_batch(int index, int device, const void *base_doc);
};

// Writes the vx3_node_worker report (src/Executables/vx3_node_worker.cu:98-141).
void vx3_write_report(const std::string &path, const std::string &input_dir_name,
                      const std::vector<VX3_SimulationResult> &results);
