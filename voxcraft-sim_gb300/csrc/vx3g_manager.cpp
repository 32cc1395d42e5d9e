// vx3g_manager.cpp -- VX3_SimulationManager drop-in (include/vx3_simulation_manager.h).
//
// VXA/VXD -> vx3g_robot_desc follows what the reference reads:
//   <Simulator>   CVX_Sim::ReadXML (src/VXA/VX_Sim.cpp:185-294) and the VX3 keys of
//                 VX3_SimulationManager::readVXD (src/VX3/VX3_SimulationManager.cu:326-367)
//   <Environment> CVX_Environment::ReadXML (src/old/VX_Environment.cpp:150-172), constructor
//                 defaults when an element is absent (:22-37)
//   <VXC>         palette and structure (src/VXA/VX_Object.cpp:1373-1456, 1760-1884)
// Math trees (StopConditionFormula, FitnessFunction) are evaluated on the host
// with the operator set of VX3_MathTree::eval (src/Utils/VX3_MathTree.h:50-192).
#include "../../include/vx3_simulation_manager.h"

#include <algorithm>
#include <exception>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <stdexcept>

#include "../../include/vx3g.h"
#include "vx3g_xml.h"

using vx3g::xml::Node;
namespace fs = std::filesystem;

bool VX3_SimulationResult::compareFitnessScore(const VX3_SimulationResult &i1, const VX3_SimulationResult &i2) {
    if (std::isnan(i2.fitness_score)) return true;
    if (std::isnan(i1.fitness_score)) return false;
    return i1.fitness_score > i2.fitness_score;
}

namespace {

struct MathVars {
    double x = 0, y = 0, z = 0, hit = 0, t = 0, angle = 0, closeness = 0, close_pairs = 0, num_voxel = 0;
};

// Evaluates a math tree whose operands are the element's children in document
// order (the queue order of the reference's token interpreter).
double eval_tree(const Node *n, const MathVars &v) {
    const std::string &op = n->name;
    auto arg = [&](size_t i) -> double {
        if (i >= n->children.size()) throw std::runtime_error("math tree: " + op + " lacks an operand");
        return eval_tree(n->children[i].get(), v);
    };
    if (op == "mtCONST") return std::strtod(vx3g::xml::trim(n->text).c_str(), nullptr);
    if (op == "mtE") return 2.71828182845904523536;
    if (op == "mtPI") return 3.14159265358979323846;
    if (op == "mtVAR") {
        std::string s = vx3g::xml::trim(n->text);
        if (s == "x") return v.x;
        if (s == "y") return v.y;
        if (s == "z") return v.z;
        if (s == "hit") return v.hit;
        if (s == "t") return v.t;
        if (s == "angle") return v.angle;
        if (s == "targetCloseness") return v.closeness;
        if (s == "numClosePairs") return v.close_pairs;
        if (s == "num_voxel") return v.num_voxel;
        throw std::runtime_error("math tree: unknown variable " + s);
    }
    if (op == "mtSIN") return std::sin(arg(0));
    if (op == "mtCOS") return std::cos(arg(0));
    if (op == "mtTAN") return std::tan(arg(0));
    if (op == "mtATAN") return std::atan(arg(0));
    if (op == "mtLOG") return std::log(arg(0));
    if (op == "mtINT") return std::rint(arg(0));
    if (op == "mtNORMALCDF") return 0.5 * std::erfc(-arg(0) / std::sqrt(2.0));
    if (op == "mtSQRT") return std::sqrt(arg(0));
    if (op == "mtABS") return std::fabs(arg(0));
    if (op == "mtNOT") return !arg(0);
    if (op == "mtADD") return arg(0) + arg(1);
    if (op == "mtSUB") return arg(0) - arg(1);
    if (op == "mtMUL") return arg(0) * arg(1);
    if (op == "mtDIV") return arg(0) / arg(1);
    if (op == "mtPOW") return std::pow(arg(0), arg(1));
    if (op == "mtGREATERTHAN") return arg(0) > arg(1);
    if (op == "mtLESSTHAN") return arg(0) < arg(1);
    if (op == "mtAND") return arg(0) && arg(1);
    if (op == "mtOR") return arg(0) || arg(1);
    throw std::runtime_error("math tree: operation not implemented: " + op);
}

bool uses_only_time(const Node *n) {
    if (n->name == "mtVAR") {
        std::string s = vx3g::xml::trim(n->text);
        return s == "t" || s == "num_voxel";
    }
    for (auto &c : n->children)
        if (!uses_only_time(c.get())) return false;
    return true;
}

// The token program VX3_SimulationManager::ParseMathTree (src/VX3/VX3_SimulationManager.cu:
// 157-275) writes for a formula element: every element below it, breadth first in
// document order, pushed on a stack above mtEND and popped back (leaves first, mtEND
// last); operator codes and variable indices as in include/vx3g.h.
std::vector<vx3g_math_token> math_program(const Node *holder, const std::string &where) {
    static const char *ops[] = {"mtEND", "mtCONST", "mtE", "mtPI", "mtVAR", "mtADD", "mtSUB", "mtMUL",
                                "mtDIV", "mtPOW", "mtSQRT", "mtSIN", "mtCOS", "mtTAN", "mtATAN", "mtLOG",
                                "mtINT", "mtABS", "mtNOT", "mtGREATERTHAN", "mtLESSTHAN", "mtAND", "mtOR", "mtNORMALCDF"};
    static const char *vars[] = {"x", "y", "z", "hit", "t", "angle", "targetCloseness", "numClosePairs", "num_voxel"};
    std::vector<const Node *> order, frontier{holder};
    while (!frontier.empty()) {
        std::vector<const Node *> next;
        for (const Node *n : frontier)
            for (auto &c : n->children) {
                order.push_back(c.get());
                next.push_back(c.get());
            }
        frontier.swap(next);
    }
    std::vector<vx3g_math_token> prog;
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        const Node *n = *it;
        vx3g_math_token t{};
        int op = -1;
        for (int k = 1; k < 24; k++)
            if (n->name == ops[k]) op = k;
        if (op < 0) throw std::runtime_error(where + ": unknown math-tree operator " + n->name);
        t.op = op;
        const std::string text = vx3g::xml::trim(n->text);
        if (op == 1) t.value = std::strtod(text.c_str(), nullptr);
        if (op == 4) {
            int v = -1;
            for (int k = 0; k < 9; k++)
                if (text == vars[k]) v = k;
            if (v < 0) throw std::runtime_error(where + ": unknown math-tree variable " + text);
            t.value = v;
        }
        prog.push_back(t);
    }
    prog.push_back(vx3g_math_token{});  // mtEND
    return prog;
}

const Node *formula_root(const Node *holder) {  // the single operator element inside a formula holder
    if (!holder) return nullptr;
    for (auto &c : holder->children)
        if (c->name.rfind("mt", 0) == 0) return c.get();
    return nullptr;
}

std::string from_base64(const std::string &in) {
    static const std::string tbl = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::string out;
    int val = 0, bits = -8;
    for (char c : in) {
        size_t p = tbl.find(c);
        if (p == std::string::npos) continue;
        val = (val << 6) + (int)p;
        bits += 6;
        if (bits >= 0) {
            out.push_back((char)((val >> bits) & 0xFF));
            bits -= 8;
        }
    }
    return out;
}

struct RobotSpec {
    std::string filename;
    std::vector<uint8_t> lattice;
    std::vector<double> phase;
    std::vector<double> cilia_base, cilia_shift;  // 3 per cell, or empty
    std::vector<vx3g_material> mats;
    std::vector<std::vector<double>> ss_strain, ss_stress;  // SSData points per material (mats[i] points here)
    std::vector<int> mat_rgba;  // 4 ints per material
    vx3g_robot_desc desc{};
    const Node *stop = nullptr, *fitness = nullptr;
    std::vector<vx3g_math_token> ff[3];  // force-field programs (desc.force_field points here)
    std::vector<vx3g_math_token> ac[5];  // attach-condition programs (desc.attach_condition points here)
    std::vector<vx3g_bc_region> bcs;     // Environment/Boundary_Conditions (desc.bcs points here)
    std::unique_ptr<Node> doc;
    int record_step = 0, record_voxel = 1, record_link = 0, save_all = 0;
    double reinit_after = 0.0;  // ReinitializeInitialPositionAfterThisManySeconds (SecondaryExperiment)
};

void read_spec(RobotSpec &S) {
    const Node *root = S.doc.get();
    const Node *vxa = root->child("VXA");
    if (!vxa) throw std::runtime_error(S.filename + ": no <VXA> element");
    vx3g_robot_desc &d = S.desc;
    // Simulator
    d.dt_frac = vx3g::xml::get_double(root, "VXA.Simulator.Integration.DtFrac", 0.9);
    if (vx3g::xml::find(root, "VXA.Simulator.Damping")) {
        d.bond_damping = vx3g::xml::get_double(root, "VXA.Simulator.Damping.BondDampingZ", 0.1);
        d.col_damping = vx3g::xml::get_double(root, "VXA.Simulator.Damping.ColDampingZ", 1.0);
        d.slow_damping = vx3g::xml::get_double(root, "VXA.Simulator.Damping.SlowDampingZ", 1.0);
    } else {  // the reference leaves these uninitialised; the <Damping> defaults are used instead
        d.bond_damping = 0.1;
        d.col_damping = 1.0;
        d.slow_damping = 1.0;
    }
    d.volume_effects = vx3g::xml::get_bool(root, "VXA.Simulator.Features.VolumeEffectsEnabled", false);
    d.enable_collision = vx3g::xml::get_bool(root, "VXA.Simulator.AttachDetach.EnableCollision", true);
    // EnableAttach, SafetyGuard and AttachCondition/Condition_0..4 (VX3_SimulationManager.cu:329-343)
    d.enable_attach = vx3g::xml::get_bool(root, "VXA.Simulator.AttachDetach.EnableAttach", false);
    d.safety_guard = vx3g::xml::get_int(root, "VXA.Simulator.AttachDetach.SafetyGuard", 500);
    for (int k = 0; k < 5; k++) {
        const std::string key = "VXA.Simulator.AttachDetach.AttachCondition.Condition_" + std::to_string(k);
        const Node *holder = vx3g::xml::find(root, key);
        if (!holder || !formula_root(holder)) continue;
        S.ac[k] = math_program(holder, S.filename + ": " + key);
        d.attach_condition[k] = S.ac[k].data();
    }
    d.enable_detach = vx3g::xml::get_bool(root, "VXA.Simulator.AttachDetach.EnableDetach", false);  // :330
    d.enable_signals = vx3g::xml::get_int(root, "VXA.Simulator.EnableSignals", 0);  // :361
    // SecondaryExperiment (VX3_SimulationManager.cu:364-365): material removal on the device,
    // the initial-position reset here
    d.secondary_experiment = vx3g::xml::get_int(root, "VXA.Simulator.SecondaryExperiment", 0);
    S.reinit_after = vx3g::xml::get_double(root, "VXA.Simulator.ReinitializeInitialPositionAfterThisManySeconds", 0.0);
    d.enable_cilia = vx3g::xml::get_int(root, "VXA.Simulator.EnableCilia", 0);  // VX3_SimulationManager.cu:360
    const char *axes[3] = {"x_forcefield", "y_forcefield", "z_forcefield"};
    for (int k = 0; k < 3; k++) {  // Simulator/ForceField (VX3_SimulationManager.cu:349-354)
        const std::string key = std::string("VXA.Simulator.ForceField.") + axes[k];
        const Node *holder = vx3g::xml::find(root, key);
        if (!holder || !formula_root(holder)) continue;
        S.ff[k] = math_program(holder, S.filename + ": " + key);
        d.force_field[k] = S.ff[k].data();
    }
    d.enable_expansion = vx3g::xml::get_int(root, "VXA.Simulator.EnableExpansion", 0);
    S.record_step = vx3g::xml::get_int(root, "VXA.Simulator.RecordHistory.RecordStepSize", 0);
    S.record_voxel = vx3g::xml::get_int(root, "VXA.Simulator.RecordHistory.RecordVoxel", 1);
    S.record_link = vx3g::xml::get_int(root, "VXA.Simulator.RecordHistory.RecordLink", 0);
    S.save_all = vx3g::xml::get_int(root, "VXA.Simulator.SavePositionOfAllVoxels", 0);
    S.stop = formula_root(vx3g::xml::find(root, "VXA.Simulator.StopCondition.StopConditionFormula"));
    S.fitness = formula_root(vx3g::xml::find(root, "VXA.Simulator.FitnessFunction"));
    // Environment
    d.grav_acc = -9.81;
    d.floor_enabled = 1;
    d.temp_enabled = 1;
    d.vary_temp = 0;
    d.temp_amplitude = 0;
    d.temp_base = 25;
    d.temp_period = 0.1;
    if (vx3g::xml::find(root, "VXA.Environment.Gravity")) {
        d.grav_acc = vx3g::xml::get_double(root, "VXA.Environment.Gravity.GravAcc", -9.81);
        d.floor_enabled = vx3g::xml::get_bool(root, "VXA.Environment.Gravity.FloorEnabled", false);
    }
    if (vx3g::xml::find(root, "VXA.Environment.Thermal")) {
        d.temp_enabled = vx3g::xml::get_bool(root, "VXA.Environment.Thermal.TempEnabled", false);
        d.temp_base = vx3g::xml::get_double(root, "VXA.Environment.Thermal.TempBase", 25.0);
        double amp;
        if (vx3g::xml::get_double(root, "VXA.Environment.Thermal.TempAmplitude", &amp)) d.temp_amplitude = amp;
        else if (vx3g::xml::get_double(root, "VXA.Environment.Thermal.TempAmp", &amp)) d.temp_amplitude = amp - d.temp_base;
        else d.temp_amplitude = 0;
        d.vary_temp = vx3g::xml::get_bool(root, "VXA.Environment.Thermal.VaryTempEnabled", false);
        d.temp_period = vx3g::xml::get_double(root, "VXA.Environment.Thermal.TempPeriod", 0.1);
    }
    // Environment/Boundary_Conditions: NumBCs FRegion elements (CVX_Environment::ReadXML,
    // src/old/VX_Environment.cpp:101-117; CVX_FRegion::ReadXML, src/old/VX_FRegion.cpp:165-219)
    if (const Node *bc = vx3g::xml::find(root, "VXA.Environment.Boundary_Conditions")) {
        const int n = vx3g::xml::get_int(bc, "NumBCs", 0);
        const std::vector<const Node *> regs = bc->all("FRegion");
        if ((int)regs.size() < n) throw std::runtime_error(S.filename + ": fewer FRegion elements than NumBCs");
        for (int i = 0; i < n; i++) {
            const Node *f = regs[i];
            vx3g_bc_region b{};
            double prim;
            if (!vx3g::xml::get_double(f, "PrimType", &prim)) throw std::runtime_error(S.filename + ": FRegion without PrimType");
            b.prim = (int)prim;
            const char *geo[7] = {"X", "Y", "Z", "dX", "dY", "dZ", "Radius"};
            float *dst[7] = {&b.x, &b.y, &b.z, &b.dx, &b.dy, &b.dz, &b.radius};
            for (int k = 0; k < 7; k++) *dst[k] = (float)vx3g::xml::get_double(f, geo[k], 0.0);
            double dof;
            if (vx3g::xml::get_double(f, "DofFixed", &dof)) b.dof_fixed = (int)dof & 0x3F;
            else b.dof_fixed = vx3g::xml::get_bool(f, "Fixed", false) ? 0x3F : 0;  // older files: a binary Fixed
            const char *ax = "XYZ";
            for (int k = 0; k < 3; k++) {
                const std::string a(1, ax[k]);
                b.force[k] = vx3g::xml::get_double(f, "Force" + a, 0.0);
                b.torque[k] = vx3g::xml::get_double(f, "Torque" + a, 0.0);
                b.displace[k] = vx3g::xml::get_double(f, "Displace" + a, 0.0);
                b.ang_displace[k] = vx3g::xml::get_double(f, "AngDisplace" + a, 0.0);
            }
            S.bcs.push_back(b);
        }
    }
    // VXC
    const Node *vxc = vxa->child("VXC");
    if (!vxc) throw std::runtime_error(S.filename + ": no <VXC> element");
    double dim = vx3g::xml::get_double(vxc, "Lattice.Lattice_Dim", 0.001);
    d.vox_size = dim * vx3g::xml::get_double(vxc, "Lattice.X_Dim_Adj", 1.0);
    if (!S.bcs.empty()) {  // regions are placed on a cubic lattice without offsets
        for (const char *k : {"Lattice.X_Dim_Adj", "Lattice.Y_Dim_Adj", "Lattice.Z_Dim_Adj"})
            if (vx3g::xml::get_double(vxc, k, 1.0) != 1.0)
                throw std::runtime_error(S.filename + ": boundary conditions need lattice dimension adjustments of 1");
        for (const char *k : {"Lattice.X_Line_Offset", "Lattice.Y_Line_Offset", "Lattice.X_Layer_Offset",
                              "Lattice.Y_Layer_Offset"})
            if (vx3g::xml::get_double(vxc, k, 0.0) != 0.0)
                throw std::runtime_error(S.filename + ": boundary conditions need a lattice without line or layer offsets");
    }
    const Node *pal = vxc->child("Palette");
    if (pal) {
        for (const Node *m : pal->all("Material")) {
            const Node *mech = m->child("Mechanical");
            vx3g_material M{};
            int model = mech ? vx3g::xml::get_int(mech, "MatModel", 0) : 0;
            if (model < 0 || model > 3) throw std::runtime_error(S.filename + ": MatModel " + std::to_string(model) + " is not supported");
            M.model = model;
            M.E = vx3g::xml::get_double(mech, "Elastic_Mod", 0.0);
            M.fail_stress = vx3g::xml::get_double(mech, "Fail_Stress", 0.0);
            M.plastic_mod = vx3g::xml::get_double(mech, "Plastic_Mod", 0.0);  // VX_Object.cpp:1439-1440
            M.yield_stress = vx3g::xml::get_double(mech, "Yield_Stress", 0.0);
            // <SSData><NumDataPts/><StrainData><Strain/>...</StrainData><StressData>...</StressData></SSData>
            // (VX_Object.cpp:1397-1418): the first NumDataPts values of each list
            std::vector<double> se, ss;
            if (const Node *sd = mech ? mech->child("SSData") : nullptr) {
                const int n = vx3g::xml::get_int(sd, "NumDataPts", 0);
                auto values = [&](const char *list, const char *item, std::vector<double> &dst) {
                    if (const Node *ln = sd->child(list))
                        for (const Node *v : ln->all(item))
                            if ((int)dst.size() < n) dst.push_back(std::atof(v->text.c_str()));
                };
                values("StrainData", "Strain", se);
                values("StressData", "Stress", ss);
                if ((int)se.size() != n || (int)ss.size() != n)
                    throw std::runtime_error(S.filename + ": SSData holds fewer points than NumDataPts");
                if (n > VX3G_MAX_MODEL_POINTS)
                    throw std::runtime_error(S.filename + ": SSData holds more than " +
                                             std::to_string(VX3G_MAX_MODEL_POINTS) + " points");
            }
            S.ss_strain.push_back(se);
            S.ss_stress.push_back(ss);
            M.rho = vx3g::xml::get_double(mech, "Density", 0.0);
            M.nu = vx3g::xml::get_double(mech, "Poissons_Ratio", 0.0);
            M.cte = vx3g::xml::get_double(mech, "CTE", 0.0);
            M.mu_static = vx3g::xml::get_double(mech, "uStatic", 0.0);
            M.mu_kinetic = vx3g::xml::get_double(mech, "uDynamic", 0.0);
            M.fixed = vx3g::xml::get_int(mech, "Fixed", 0);
            M.sticky = vx3g::xml::get_int(mech, "Sticky", 0);  // VX_Object.cpp:1436
            M.is_measured = vx3g::xml::get_int(mech, "isMeasured", 1);
            M.thermal_on_after = vx3g::xml::get_double(mech, "TurnOnThermalExpansionAfterThisManySeconds", 0.0);
            M.cilia = vx3g::xml::get_double(mech, "Cilia", 0.0);  // VX_Object.cpp:1429, 1437
            M.cilia_on_after = vx3g::xml::get_double(mech, "TurnOnCiliaAfterThisManySeconds", 0.0);
            M.remove_after = vx3g::xml::get_double(mech, "RemoveFromSimulationAfterThisManySeconds", 0.0);  // :1427
            // signals (VX_Object.cpp:1420-1424)
            M.is_pacemaker = vx3g::xml::get_int(mech, "isPaceMaker", 0);
            M.pacemaker_period = vx3g::xml::get_double(mech, "PaceMakerPeriod", 0.0);
            M.signal_value_decay = vx3g::xml::get_double(mech, "signalValueDecay", 0.9);
            M.signal_time_delay = vx3g::xml::get_double(mech, "signalTimeDelay", 0.03);
            M.inactive_period = vx3g::xml::get_double(mech, "inactivePeriod", 0.03);
            if (vx3g::xml::get_int(mech, "isTarget", 0))  // collisions with targets count hits and signal
                throw std::runtime_error(S.filename + ": target materials (isTarget) are not supported");
            S.mats.push_back(M);
            const Node *disp = m->child("Display");
            for (const char *c : {"Red", "Green", "Blue", "Alpha"})
                S.mat_rgba.push_back((int)(vx3g::xml::get_double(disp, c, std::strcmp(c, "Alpha") ? 0.5 : 1.0) * 255));
        }
        for (size_t i = 0; i < S.mats.size(); i++) {  // the SSData arrays live in S
            S.mats[i].n_data = (int)S.ss_strain[i].size();
            S.mats[i].strain_data = S.ss_strain[i].empty() ? nullptr : S.ss_strain[i].data();
            S.mats[i].stress_data = S.ss_stress[i].empty() ? nullptr : S.ss_stress[i].data();
        }
    }
    const Node *st = vxc->child("Structure");
    if (!st) throw std::runtime_error(S.filename + ": no <Structure>");
    d.nx = vx3g::xml::get_int(st, "X_Voxels", 1);
    d.ny = vx3g::xml::get_int(st, "Y_Voxels", 1);
    d.nz = vx3g::xml::get_int(st, "Z_Voxels", 1);
    const std::string *comp = st->attr("Compression");
    std::string compression = comp ? *comp : "BASE64";
    const size_t layer = (size_t)d.nx * d.ny;
    S.lattice.assign(layer * d.nz, 0);
    const Node *data = st->child("Data");
    auto layers = data ? data->all("Layer") : std::vector<const Node *>{};
    if ((int)layers.size() < d.nz) throw std::runtime_error(S.filename + ": structure has fewer layers than Z_Voxels");
    for (int z = 0; z < d.nz; z++) {
        std::string raw = layers[z]->text, bytes;
        if (compression == "ASCII_READABLE") {
            raw = vx3g::xml::trim(raw);
            for (char c : raw) bytes.push_back((char)(c - 48));
        } else if (compression == "RAW_DATA") {
            bytes = raw;
        } else if (compression == "BASE64" || compression.empty()) {
            bytes = from_base64(raw);
        } else {
            throw std::runtime_error(S.filename + ": structure compression " + compression + " is not supported");
        }
        if (bytes.size() != layer) throw std::runtime_error(S.filename + ": layer size does not match X_Voxels*Y_Voxels");
        for (size_t k = 0; k < layer; k++) S.lattice[z * layer + k] = (uint8_t)bytes[k];
    }
    S.phase.assign(S.lattice.size(), 0.0);
    if (const Node *po = st->child("PhaseOffset")) {  // comma-separated, one value per cell, read for occupied cells
        auto rows = po->all("Layer");
        for (int z = 0; z < d.nz && z < (int)rows.size(); z++) {
            std::string row = rows[z]->text;
            size_t k = 0, a = 0;
            while (k < layer && a <= row.size()) {
                size_t b = row.find(',', a);
                if (b == std::string::npos) b = row.size();
                if (S.lattice[z * layer + k] > 0) S.phase[z * layer + k] = std::atof(row.substr(a, b - a).c_str());
                k++;
                a = b + 1;
            }
        }
    }
    // BaseCiliaForce / ShiftCiliaForce (VX_Object.cpp:1886-1958): three comma-separated values
    // per cell of each layer, read for occupied cells, 0 where a row is short
    for (int which = 0; which < 2; which++) {
        const Node *cf = st->child(which ? "ShiftCiliaForce" : "BaseCiliaForce");
        std::vector<double> &dst = which ? S.cilia_shift : S.cilia_base;
        if (!cf) continue;
        dst.assign(3 * S.lattice.size(), 0.0);
        auto rows = cf->all("Layer");
        for (int z = 0; z < d.nz && z < (int)rows.size(); z++) {
            std::vector<double> vals;
            const std::string &row = rows[z]->text;
            size_t a = 0;
            while (a <= row.size()) {
                size_t b = row.find(',', a);
                if (b == std::string::npos) b = row.size();
                vals.push_back(std::atof(row.substr(a, b - a).c_str()));
                a = b + 1;
            }
            for (size_t k = 0; k < layer; k++)
                if (S.lattice[z * layer + k] > 0 && vals.size() > 3 * k + 2)
                    for (int j = 0; j < 3; j++) dst[3 * (z * layer + k) + j] = vals[3 * k + j];
        }
    }
    d.cilia_base = S.cilia_base.empty() ? nullptr : S.cilia_base.data();
    d.cilia_shift = S.cilia_shift.empty() ? nullptr : S.cilia_shift.data();
    d.lattice = S.lattice.data();
    d.phase = S.phase.data();
    d.n_materials = (int)S.mats.size();
    d.materials = S.mats.data();
    d.n_bcs = (int)S.bcs.size();
    d.bcs = S.bcs.empty() ? nullptr : S.bcs.data();
}

void check(int rc, const char *what) {
    if (rc != VX3G_OK) throw std::runtime_error(std::string(what) + ": " + vx3g_last_error());
}

// CUDA_Simulation's history record (src/VX3/VX3_SimulationManager.cu:74-112)
void print_history(FILE *out, vx3g_ctx *ctx, int robot, const RobotSpec &S, long step, double t,
                   const std::vector<int> &voff, const std::vector<int> &loff) {
    int nv, nl, ns;
    check(vx3g_counts(ctx, &nv, &nl, &ns), "vx3g_counts");
    std::vector<double> pos(3 * (size_t)nv), orient(4 * (size_t)nv);
    std::vector<float> tempe(nv), strain(nl), maxs(nl);
    std::vector<double> signal(nv);
    check(vx3g_get_signals(ctx, signal.data()), "vx3g_get_signals");
    std::vector<int32_t> ends(2 * (size_t)nl), axis(nl), vmat(nv), surf(ns), lflag(nl);
    check(vx3g_get_state(ctx, pos.data(), orient.data(), nullptr, nullptr), "vx3g_get_state");
    check(vx3g_get_voxel_aux(ctx, tempe.data(), nullptr, nullptr), "vx3g_get_voxel_aux");
    check(vx3g_get_links(ctx, strain.data(), maxs.data(), nullptr, nullptr, lflag.data()), "vx3g_get_links");
    check(vx3g_get_topology(ctx, nullptr, vmat.data(), ends.data(), axis.data()), "vx3g_get_topology");
    check(vx3g_get_surface(ctx, surf.data()), "vx3g_get_surface");
    // per voxel: link in each direction (detached and removed links are no voxel's any more)
    std::vector<int> slot(6 * (size_t)nv, -1);
    for (int l = loff[robot]; l < loff[robot + 1]; l++) {
        if (lflag[l] & 2) continue;
        slot[6 * (size_t)ends[2 * l] + 2 * axis[l]] = l;
        slot[6 * (size_t)ends[2 * l + 1] + 2 * axis[l] + 1] = l;
    }
    const double vs = 1 / 0.001;
    if (S.record_voxel) {
        fprintf(out, "<<<Step%ld Time:%f>>>", step, t);
        for (int s : surf) {
            if (s < voff[robot] || s >= voff[robot + 1]) continue;
            const double *p = &pos[3 * (size_t)s], *q = &orient[4 * (size_t)s];
            fprintf(out, "%.1f,%.1f,%.1f,", p[0] * vs, p[1] * vs, p[2] * vs);
            const double w = q[0] > 1 ? 1 : q[0];
            fprintf(out, "%.1f,%.2f,%.2f,%.2f,", 2.0 * std::acos(w) * 57.29577951308232, q[1], q[2], q[3]);
            // cornerOffset (VX3_Voxel.cu:147-159)
            const vx3g_material &M = S.mats[vmat[s]];
            const float cte = (float)M.cte;
            const double bs = S.desc.vox_size * (1 + tempe[s] * cte);
            double corner[2][3];
            for (int c = 0; c < 2; c++) {
                for (int i = 0; i < 3; i++) {
                    const bool posLink = c == 1;
                    const int l = slot[6 * (size_t)s + 2 * i + (posLink ? 0 : 1)];
                    float st;
                    const float Eneg = (float)S.mats[vmat[l >= 0 ? ends[2 * l] : s]].E;
                    const float Epos = (float)S.mats[vmat[l >= 0 ? ends[2 * l + 1] : s]].E;
                    const float ratio = Epos / Eneg;
                    if (l >= 0) {
                        const float a = posLink ? 2.0f * strain[l] * ratio / (1.0f + ratio) : 2.0f * strain[l] / (1.0f + ratio);
                        st = (1 + a) * (posLink ? 1 : -1);
                    } else {
                        st = posLink ? 1.0f : -1.0f;
                    }
                    corner[c][i] = (float)(0.5 * bs * st);
                }
            }
            fprintf(out, "%.1f,%.1f,%.1f,%.1f,%.1f,%.1f,", corner[0][0] * vs, corner[0][1] * vs, corner[0][2] * vs,
                    corner[1][0] * vs, corner[1][1] * vs, corner[1][2] * vs);
            fprintf(out, "%d,", vmat[s] + 1);
            fprintf(out, "%.1f,", signal[s]);  // localSignal, for colouring (:88)
            fprintf(out, ";");
        }
        fprintf(out, "<<<>>>");
    }
    if (S.record_link) {
        fprintf(out, "|[[[%ld]]]", step);
        for (int l = loff[robot]; l < loff[robot + 1]; l++) {
            if (lflag[l] & 2) continue;  // removed or detached (:98-103)
            const double *a = &pos[3 * (size_t)ends[2 * l + 1]], *b = &pos[3 * (size_t)ends[2 * l]];
            fprintf(out, "%.4f,%.4f,%.4f,%.4f,%.4f,%.4f,;", a[0], a[1], a[2], b[0], b[1], b[2]);
        }
        fprintf(out, "[[[]]]");
    }
    fprintf(out, "\n");
}

}  // namespace

VX3_SimulationManager::VX3_SimulationManager(std::vector<std::vector<fs::path>> in_sub_batches, fs::path in_base,
                                             fs::path in_input_dir, int in_num_of_devices)
    : sub_batches(std::move(in_sub_batches)), base(std::move(in_base)), input_dir(std::move(in_input_dir)),
      num_of_devices(in_num_of_devices) {}

VX3_SimulationManager::~VX3_SimulationManager() {}

// One device's sub-batch: read (base VXA + each VXD), simulated as one vx3g batch until
// every robot's stop condition holds, collected into result records.  Runs on its own
// host thread (one per device); the history text of concurrent sub-batches is written
// under one lock, a record at a time.
static std::mutex g_history_lock;

std::vector<VX3_SimulationResult> VX3_SimulationManager::run_sub_batch(int index, int dev, const void *base_doc_p) {
    const Node *base_doc = static_cast<const Node *>(base_doc_p);
    std::vector<VX3_SimulationResult> h_results;
    {
        auto &files = sub_batches[index];
        if (files.empty()) return h_results;
        std::vector<std::unique_ptr<RobotSpec>> specs;
        for (auto &f : files) {
            auto S = std::make_unique<RobotSpec>();
            S->filename = f.filename().string();
            S->doc = base_doc->clone();
            auto vxd = vx3g::xml::parse_file((input_dir / f).string());
            vx3g::xml::merge_vxd(vxd.get(), S->doc.get());
            read_spec(*S);
            specs.push_back(std::move(S));
        }
        std::vector<vx3g_robot_desc> descs;
        for (auto &S : specs) descs.push_back(S->desc);
        vx3g_batch_desc bd{(int)descs.size(), descs.data(), precision, dev, 100};
        int status = 0;
        vx3g_ctx *ctx = vx3g_create(&bd, &status);
        if (!ctx) throw std::runtime_error(std::string("vx3g_create: ") + vx3g_last_error());
        const int R = (int)specs.size();
        std::vector<int> voff(R + 1), loff(R + 1);
        check(vx3g_offsets(ctx, voff.data(), loff.data()), "vx3g_offsets");
        std::vector<double> com(3 * R), com0(3 * R), t(R), dt(R);
        std::vector<int32_t> st(R);
        check(vx3g_com(ctx, com0.data()), "vx3g_com");
        check(vx3g_dt(ctx, dt.data()), "vx3g_dt");
        std::vector<char> done(R, 0);
        std::vector<long> steps(R, 0);
        // history stride: int(RecordStepSize/(10000*recommendedTimeStep*DtFrac))+1 (:56)
        std::vector<long> stride(R, 0);
        for (int r = 0; r < R; r++)
            if (specs[r]->record_step) stride[r] = (long)(specs[r]->record_step / (10000 * (dt[r] / specs[r]->desc.dt_frac) * specs[r]->desc.dt_frac)) + 1;
        auto stop_met = [&](int r, double time, const double *c) {
            if (!specs[r]->stop) return false;
            MathVars v;
            v.x = c[0]; v.y = c[1]; v.z = c[2];
            v.t = time;
            v.num_voxel = voff[r + 1] - voff[r];
            return eval_tree(specs[r]->stop, v) > 0;
        };
        // currentCenterOfMass, which StopConditionMet reads before every step
        // (VX3_SimulationManager.cu:62-64), is refreshed only at the end of every step whose
        // count is a multiple of CycleStep = int(TempPeriod / dt) (VX3_VoxelyzeKernel.cu:313-320);
        // com_s is that value.  (CycleStep 0, TempPeriod below dt, leaves the reference with a
        // modulo by zero; here the value then stays the initial one.)
        std::vector<long> cycle(R, 0);
        for (int r = 0; r < R; r++) cycle[r] = (long)(specs[r]->desc.temp_period / (double)(float)dt[r]);
        std::vector<double> com_s(com0);
        // SecondaryExperiment: the initial centre of mass (that value) and the voxels' initial
        // positions are taken again at the end of the first step that starts later than
        // ReinitializeInitialPositionAfterThisManySeconds (:344-348)
        std::vector<long> reinit_step(R, -1);
        std::vector<std::vector<double>> init_pos(R);
        for (int r = 0; r < R; r++) {
            if (!specs[r]->desc.secondary_experiment) continue;
            double tt = 0.0;  // start time of step n
            long n = 1;
            while (!(specs[r]->reinit_after < tt) && n <= max_steps) {
                tt += (float)dt[r];
                n++;
            }
            if (n <= max_steps) reinit_step[r] = n;
        }
        long loop = 0;
        const bool history = std::any_of(stride.begin(), stride.end(), [](long s) { return s > 0; });
        while (true) {
            check(vx3g_time(ctx, t.data()), "vx3g_time");
            check(vx3g_status(ctx, st.data()), "vx3g_status");
            check(vx3g_com(ctx, com.data()), "vx3g_com");
            bool snap = false;
            for (int r = 0; r < R; r++) {  // the end of step `loop` for the robots still stepping
                if (done[r] || loop == 0) continue;
                if (cycle[r] > 0 && loop % cycle[r] == 0)
                    for (int k = 0; k < 3; k++) com_s[3 * r + k] = com[3 * r + k];
                if (loop == reinit_step[r]) {
                    for (int k = 0; k < 3; k++) com0[3 * r + k] = com_s[3 * r + k];
                    snap = true;
                }
            }
            if (snap) {
                int nv_all = 0;
                check(vx3g_counts(ctx, &nv_all, nullptr, nullptr), "vx3g_counts");
                std::vector<double> p(3 * (size_t)nv_all);
                check(vx3g_get_state(ctx, p.data(), nullptr, nullptr, nullptr), "vx3g_get_state");
                for (int r = 0; r < R; r++)
                    if (!done[r] && loop == reinit_step[r])
                        init_pos[r].assign(p.begin() + 3 * (size_t)voff[r], p.begin() + 3 * (size_t)voff[r + 1]);
            }
            int active = 0;
            long chunk = 100;
            for (int r = 0; r < R; r++) {
                if (done[r]) continue;
                if (st[r] != VX3G_ROBOT_OK || loop >= max_steps || stop_met(r, t[r], &com_s[3 * r])) {
                    done[r] = 1;
                    continue;
                }
                active++;
                if (specs[r]->stop) {
                    // the exact number of steps before the condition holds: time accumulates the
                    // float dt in double, and the COM it reads changes only at the next CycleStep
                    long lim = chunk;
                    if (!uses_only_time(specs[r]->stop) && cycle[r] > 0) lim = std::min(lim, (loop / cycle[r] + 1) * cycle[r] - loop);
                    double tt = t[r];
                    long k = 0;
                    while (k < lim && !stop_met(r, tt, &com_s[3 * r])) {
                        tt += (float)dt[r];
                        k++;
                    }
                    chunk = std::max(1L, std::min(chunk, k));
                }
                if (reinit_step[r] > loop) {  // the reset reads the COM sampled at the last CycleStep before it
                    chunk = std::min(chunk, reinit_step[r] - loop);
                    if (cycle[r] > 0) chunk = std::min(chunk, (loop / cycle[r] + 1) * cycle[r] - loop);
                }
            }
            if (!active) break;
            if (history) {  // end the chunk on the next loop index j with j % stride == 0
                for (int r = 0; r < R; r++) {
                    if (!stride[r] || done[r]) continue;
                    const long next_j = (loop % stride[r] == 0) ? loop : (loop / stride[r] + 1) * stride[r];
                    chunk = std::min(chunk, next_j - loop + 1);
                }
            }
            chunk = std::min(chunk, max_steps - loop);
            // robots that are done stop stepping
            for (int r = 0; r < R; r++)
                if (done[r] && st[r] == VX3G_ROBOT_OK) check(vx3g_stop_robot(ctx, r), "vx3g_stop_robot");
            check(vx3g_step(ctx, (int)chunk), "vx3g_step");
            for (int r = 0; r < R; r++)
                if (!done[r]) steps[r] += chunk;
            if (history) {
                check(vx3g_time(ctx, t.data()), "vx3g_time");
                const long j = loop + chunk - 1;
                for (int r = 0; r < R; r++)
                    if (stride[r] && !done[r] && j % stride[r] == 0) {
                        std::lock_guard<std::mutex> g(g_history_lock);
                        print_history(this->history, ctx, r, *specs[r], j, t[r], voff, loff);
                    }
            }
            loop += chunk;
        }
        check(vx3g_com(ctx, com.data()), "vx3g_com");
        check(vx3g_time(ctx, t.data()), "vx3g_time");
        check(vx3g_status(ctx, st.data()), "vx3g_status");
        int nv, nl, ns;
        check(vx3g_counts(ctx, &nv, &nl, &ns), "vx3g_counts");
        std::vector<double> pos(3 * (size_t)nv);
        std::vector<int32_t> ijk(3 * (size_t)nv), vmat(nv);
        check(vx3g_get_state(ctx, pos.data(), nullptr, nullptr, nullptr), "vx3g_get_state");
        check(vx3g_get_topology(ctx, ijk.data(), vmat.data(), nullptr, nullptr), "vx3g_get_topology");
        for (int r = 0; r < R; r++) {
            VX3_SimulationResult res;
            const RobotSpec &S = *specs[r];
            res.vxa_filename = S.filename;
            res.currentTime = t[r];
            res.voxSize = S.desc.vox_size;
            res.num_voxel = voff[r + 1] - voff[r];
            res.x = com[3 * r]; res.y = com[3 * r + 1]; res.z = com[3 * r + 2];
            res.currentCenterOfMass = {com[3 * r], com[3 * r + 1], com[3 * r + 2]};
            res.initialCenterOfMass = {com0[3 * r], com0[3 * r + 1], com0[3 * r + 2]};
            res.SavePositionOfAllVoxels = S.save_all != 0;
            res.status = st[r];
            res.steps = steps[r];
            for (int v = voff[r]; v < voff[r + 1]; v++) {
                // saveInitialPosition (VX3_VoxelyzeKernel.cu:155-161): the lattice positions, or
                // the positions at the SecondaryExperiment reset
                VX3_Vec3 p0{ijk[3 * v] * S.desc.vox_size, ijk[3 * v + 1] * S.desc.vox_size, ijk[3 * v + 2] * S.desc.vox_size};
                if (!init_pos[r].empty()) {
                    const double *q = &init_pos[r][3 * (size_t)(v - voff[r])];
                    p0 = VX3_Vec3{q[0], q[1], q[2]};
                }
                VX3_Vec3 p{pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
                res.voxel_init_pos.push_back(p0);
                res.voxel_position.push_back(p);
                res.voxel_mats.push_back(vmat[v] + 1);
                if (S.mats[vmat[v]].is_measured) {
                    res.num_measured_voxel++;
                    res.total_distance_of_all_voxels +=
                        std::sqrt((p.x - p0.x) * (p.x - p0.x) + (p.y - p0.y) * (p.y - p0.y) + (p.z - p0.z) * (p.z - p0.z));
                }
            }
            // computeFitness (VX3_VoxelyzeKernel.cu:530-534): offset COM as x, y, z
            MathVars v;
            v.x = com[3 * r] - com0[3 * r];
            v.y = com[3 * r + 1] - com0[3 * r + 1];
            v.z = com[3 * r + 2] - com0[3 * r + 2];
            v.t = t[r];
            v.num_voxel = res.num_voxel;
            res.fitness_score = S.fitness ? eval_tree(S.fitness, v) : 0.0;
            if (st[r] & VX3G_ROBOT_DIVERGED) res.fitness_score = NAN;
            h_results.push_back(res);
        }
        vx3g_destroy(ctx);
    }
    return h_results;
}

// All sub-batches at once, one host thread (and so one CUDA context stream) per device,
// as the reference launches every device's kernel before its one synchronisation
// (VX3_SimulationManager.cu:138-155); the results are merged in sub-batch order and sorted.
void VX3_SimulationManager::start() {
    auto base_doc = vx3g::xml::parse_file(base.string());
    const int n = std::min(num_of_devices, (int)sub_batches.size());
    if (!devices.empty() && (int)devices.size() < n)
        throw std::runtime_error("devices: one device per sub-batch is needed");
    std::vector<std::vector<VX3_SimulationResult>> per(n);
    std::vector<std::exception_ptr> errs(n);
    std::vector<std::thread> threads;
    for (int i = 0; i < n; i++) {
        const int dev = devices.empty() ? i : devices[i];
        threads.emplace_back([this, i, dev, &per, &errs, &base_doc] {
            try {
                per[i] = run_sub_batch(i, dev, base_doc.get());
            } catch (...) {
                errs[i] = std::current_exception();
            }
        });
    }
    for (auto &t : threads) t.join();
    for (auto &e : errs)
        if (e) std::rethrow_exception(e);
    for (auto &v : per) h_results.insert(h_results.end(), v.begin(), v.end());
    std::sort(h_results.begin(), h_results.end(), VX3_SimulationResult::compareFitnessScore);
}

void vx3_write_report(const std::string &path, const std::string &input_dir_name,
                      const std::vector<VX3_SimulationResult> &results) {
    std::ofstream o(path);
    if (!o) throw std::runtime_error("cannot write " + path);
    auto num = [](double v) {
        char b[64];
        snprintf(b, sizeof b, "%.17g", v);
        return std::string(b);
    };
    o << "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n<report>";
    o << "<inputdir>" << input_dir_name << "</inputdir>";
    if (!results.empty())
        o << "<bestfit><filename>" << results[0].vxa_filename << "</filename><fitness_score>"
          << num(results[0].fitness_score) << "</fitness_score></bestfit>";
    o << "<detail>";
    for (auto &r : results) {
        std::string name = r.vxa_filename.substr(0, r.vxa_filename.find('.'));
        o << "<" << name << ">";
        o << "<currentTime>" << num(r.currentTime) << "</currentTime>";
        o << "<fitness_score>" << num(r.fitness_score) << "</fitness_score>";
        o << "<num_voxel>" << r.num_voxel << "</num_voxel>";
        o << "<num_measured_voxel>" << r.num_measured_voxel << "</num_measured_voxel>";
        o << "<voxSize>" << num(r.voxSize) << "</voxSize>";
        o << "<numClosePairs>" << r.numClosePairs << "</numClosePairs>";
        o << "<initialCenterOfMass><x>" << num(r.initialCenterOfMass.x) << "</x><y>" << num(r.initialCenterOfMass.y)
          << "</y><z>" << num(r.initialCenterOfMass.z) << "</z></initialCenterOfMass>";
        o << "<currentCenterOfMass><x>" << num(r.currentCenterOfMass.x) << "</x><y>" << num(r.currentCenterOfMass.y)
          << "</y><z>" << num(r.currentCenterOfMass.z) << "</z></currentCenterOfMass>";
        o << "<total_distance_of_all_voxels>" << num(r.total_distance_of_all_voxels) << "</total_distance_of_all_voxels>";
        if (r.SavePositionOfAllVoxels) {
            o << "<init_pos>";
            for (auto &p : r.voxel_init_pos) o << std::to_string(p.x) << "," << std::to_string(p.y) << "," << std::to_string(p.z) << ";";
            o << "</init_pos><pos>";
            for (auto &p : r.voxel_position) o << std::to_string(p.x) << "," << std::to_string(p.y) << "," << std::to_string(p.z) << ";";
            o << "</pos><mats>";
            for (int m : r.voxel_mats) o << m << ";";
            o << "</mats>";
        }
        o << "</" << name << ">";
    }
    o << "</detail></report>\n";
}
