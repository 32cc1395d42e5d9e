// vx3g_host.cpp -- host side of the C ABI: lattice building, material
// constants, device memory, the step loop as CUDA graphs, and state access.
//
// Lattice building follows CVX_Sim::Import / CVoxelyze::addVoxel / addLink
// (src/VXA/VX_Sim.cpp:88-107, src/old/Voxelyze.cpp:439-539, src/old/VX_Link.cpp:21-54):
// voxels in x-fastest scan order; a new voxel links to the neighbours that
// already exist, in direction order X_NEG, Y_NEG, Z_NEG, with the lower lattice
// index as the link's negative end.  Material constants follow CVX_Material /
// CVX_MaterialVoxel / CVX_MaterialLink (src/old/VX_Material*.cpp) in float, as the
// reference computes them before copying them into its VX3 objects.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vx3g.h"
#include "vx3g_adjoint.h"
#include "vx3g_internal.h"
#include "vx3g_bc.h"
#include "vx3g_material.h"

using namespace vx3g;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(VX3G_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

struct HostVMat {
    float E, nu, rho, cte, mu_s, mu_k, z_int, z_glob, z_col, eHat, sigma_fail, grav_mult;
    float mass, mass_inv, sqrt_mass, mom, mom_inv, c2m, c2i;
    double nom;
    MatModel model;  // stress-strain model (E and sigma_fail above are its values)
};

// the stress-strain model of a palette entry as CVX_Sim::CopyMat sets it (src/VXA/VX_Sim.cpp:390-409)
MatModel material_model(const vx3g_material &in) {
    MatModel m;
    bool ok = false;
    switch (in.model) {
        case 0: ok = model_linear(m, (float)in.E, -1.0f); break;
        case 1: ok = model_linear(m, (float)in.E, (float)in.fail_stress); break;
        case 2: ok = model_bilinear(m, (float)in.E, (float)in.plastic_mod, (float)in.yield_stress, (float)in.fail_stress); break;
        case 3: {
            std::vector<float> e(in.n_data), s(in.n_data);
            for (int i = 0; i < in.n_data; i++) e[i] = (float)in.strain_data[i], s[i] = (float)in.stress_data[i];
            ok = model_data(m, in.n_data, e.data(), s.data());
            break;
        }
    }
    if (!ok) m = MatModel();  // the setter failed: the material keeps addMaterial's default model
    return m;
}

float ehat(float E, float nu) { return E / ((1 - 2 * nu) * (1 + nu)); }

// CVX_Sim::CopyMat + Import damping + EnableVolumeEffects + CVX_MaterialVoxel::updateDerived
HostVMat import_material(const vx3g_material &in, const vx3g_robot_desc &r) {
    HostVMat m{};
    m.model = material_model(in);
    m.E = m.model.E;
    m.sigma_fail = m.model.sigma_fail;
    float nu = (float)in.nu;
    if (nu < 0) nu = 0;
    if (nu >= 0.5) nu = 0.5 - FLT_EPSILON * 2;
    if (!r.volume_effects) nu = 0;
    m.nu = nu;
    float rho = (float)in.rho;
    if (rho <= 0) rho = FLT_MIN;
    m.rho = rho;
    m.cte = (float)in.cte;
    float ms = (float)in.mu_static, mk = (float)in.mu_kinetic;
    m.mu_s = ms <= 0 ? 0 : ms;
    m.mu_k = mk <= 0 ? 0 : mk;
    float zi = (float)r.bond_damping, zg = (float)r.slow_damping, zc = (float)r.col_damping;
    m.z_int = zi <= 0 ? 0 : zi;
    m.z_glob = zg <= 0 ? 0 : zg;
    m.z_col = zc <= 0 ? 0 : zc;
    m.nom = r.vox_size;
    float ga = (float)r.grav_acc;
    m.grav_mult = (float)(-ga / 9.80665);  // CVX_Sim::SetGravityAccel (VX_Sim.cpp:485)
    m.eHat = ehat(m.E, m.nu);
    double volume = m.nom * m.nom * m.nom;
    m.mass = (float)(volume * m.rho);
    m.mom = (float)(m.mass * m.nom * m.nom / 6.0f);
    if (volume == 0 || m.mass == 0 || m.mom == 0) return m;
    m.mass_inv = 1.0f / m.mass;
    m.sqrt_mass = sqrtf(m.mass);
    m.mom_inv = 1.0f / m.mom;
    m.c2m = (float)(2.0f * std::sqrt((double)(m.mass * m.E) * m.nom));
    m.c2i = (float)(2.0f * std::sqrt((double)(m.mom * m.E) * m.nom * m.nom * m.nom));
    return m;
}

// CVX_MaterialLink::updateAll + updateDerived (src/old/VX_MaterialLink.cpp:47-140);
// vox1 is the material of the voxel being added, vox2 its existing neighbour's.
VMat to_vmat(const HostVMat &m, const vx3g_material &in) {
    VMat v{};
    v.mass = m.mass; v.mass_inv = m.mass_inv; v.mom_inv = m.mom_inv;
    v.c_glob = m.z_glob * m.c2m;
    v.c_glob_rot = m.z_glob * m.c2i;
    v.c_col = m.z_col * m.c2m;
    v.grav_force = -m.mass * 9.80665f * m.grav_mult;
    v.pstiff = (float)(2 * m.E * m.nom);
    v.mu_s = m.mu_s; v.mu_k = m.mu_k; v.cte = m.cte;
    v.dmc = 2 * m.sqrt_mass * m.z_int;
    v.E = m.E; v.nu = m.nu;
    v.nom_hi = (float)m.nom;
    v.nom_lo = (float)(m.nom - (double)v.nom_hi);
    v.fixed = in.fixed ? 1 : 0;
    v.is_measured = in.is_measured ? 1 : 0;
    v.nom_size = m.nom;
    v.thermal_on_after = in.thermal_on_after;
    v.toa_pos = in.thermal_on_after > 0 ? 1 : 0;
    v.pacemaker = in.is_pacemaker ? 1 : 0;
    v.pace_period = in.pacemaker_period;
    v.sig_decay = in.signal_value_decay;
    v.sig_delay = in.signal_time_delay;
    v.inactive = in.inactive_period;
    v.alm = -1;  // set for Sticky materials of robots with EnableAttach
    return v;
}

LMat combine(const HostVMat &v1, const HostVMat &v2, std::vector<float2> &pts) {
    LMat l{};
    const MatModel lm = model_link(v1.model, v2.model);
    const float E = lm.E;
    l.E = E;
    l.eps_fail = lm.eps_fail;
    l.lin = lm.linear ? 1 : 0;
    l.ssn = (int)lm.strain.size() + 1;
    l.sso = 0;
    if (!lm.linear) {
        // the data points of the curve as the reference's device copy holds them:
        // VX3_Material::syncVectors (VX3_Material.cu:463-481) puts one more (0,0) in front,
        // which the stress function's segment tests then see
        l.sso = (int)pts.size();
        pts.push_back(make_float2(0.0f, 0.0f));
        for (size_t i = 0; i < lm.strain.size(); i++) pts.push_back(make_float2(lm.strain[i], lm.stress[i]));
    }
    float nu;
    if (v1.nu == 0 && v2.nu == 0) {
        nu = 0;
    } else {
        float tmpEHat = 2 * v1.eHat * v2.eHat / (v1.eHat + v2.eHat);
        float c2 = (float)((tmpEHat - E) / (2 * tmpEHat) + 0.0625);
        nu = (float)(sqrtf(c2) - 0.25);
    }
    l.nu = nu;
    l.eHat = ehat(E, nu);
    float L = (float)(0.5 * (v1.nom + v2.nom));
    l.a1 = E * L;
    l.a2 = E * L * L * L / (12.0f * (1 + nu));
    l.b1 = E * L;
    l.b2 = E * L * L / 2.0f;
    l.b3 = E * L * L * L / 6.0f;
    l.sqA1 = sqrtf(l.a1);
    l.sqA2xIp = sqrtf(l.a2 * L * L / 6.0f);
    l.sqB1 = sqrtf(l.b1);
    l.sqB2xFMp = sqrtf(l.b2 * L / 2.0f);
    l.sqB3xIp = sqrtf(l.b3 * L * L / 6.0f);
    // transverse area/strain sum at creation (CVX_Link::updateTransverseInfo, unstrained voxels)
    float s1 = (float)v1.nom, s2 = (float)v2.nom;
    l.area = 0.5f * (s2 * s2 + s1 * s1);
    l.tss = 0.0f;
    return l;
}

// A 32-byte voxel-state slot: four doubles, or (mixed precision) a float4 hi
// followed by a float4 lo whose sum is the value.
double4 to_slot(double a, double b, double c, double w, bool mixed) {
    if (!mixed) return make_double4(a, b, c, w);
    const double v[4] = {a, b, c, w};
    float f[8];
    for (int k = 0; k < 4; k++) {
        f[k] = (float)v[k];
        f[4 + k] = (float)(v[k] - (double)f[k]);
    }
    double4 out;
    memcpy(&out, f, sizeof out);
    return out;
}

void from_slot(const double4 &s, bool mixed, double out[4]) {
    if (!mixed) {
        out[0] = s.x; out[1] = s.y; out[2] = s.z; out[3] = s.w;
        return;
    }
    float f[8];
    memcpy(f, &s, sizeof f);
    for (int k = 0; k < 4; k++) out[k] = (double)f[k] + (double)f[4 + k];
}

}  // namespace

struct vx3g_ctx {
    int precision = 0, chunk = 100, device = 0, nr = 0;
    cudaStream_t stream = nullptr;
    // mixed precision with collisions: the contact evaluation runs on `side`, beside the
    // link pass (both read only the state the step starts with), forked and joined by events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool overlap = false;
    // where the side stream forks: 0 after the cooperative rebuild kernel (best when
    // rebuilds are rare), 1 before the displacement check, so that the check, any rebuild
    // and the contact evaluation all run beside the link pass (best when some robot
    // rebuilds in most steps); chosen by vx3g_autotune, results do not depend on it
    int fork_early = 0;
    Dev d{};
    std::vector<void *> allocs;
    double *scratch = nullptr;  // dt reduction / com output
    // host copies of static topology
    std::vector<int> voff, loff;
    std::vector<int2> ends;
    std::vector<uint32_t> laxis;
    std::vector<short4> ijk;
    std::vector<int> vmat_local, surface;
    std::vector<unsigned char> vfixed;
    int64_t steps = 0;
    int shape_links = 0, shape_voxels = 0;  // launch shapes of the mixed passes (vx3g_autotune)
    bool ff_pos = false;  // some robot's force field reads the voxel position
    bool any_ff = false;  // some robot has a force field
    bool any_cilia = false;  // some robot has cilia
    bool any_detach = false;  // some robot has EnableDetach
    bool any_remove = false;  // some robot removes voxels (SecondaryExperiment)
    bool any_dyn = false;     // some robot's surface follows its link table (detach or removal)
    bool any_nonlinear = false;  // some material has a non-linear stress-strain model
    bool any_bcs = false;        // some voxel has a boundary-condition external
    bool any_signals = false;    // some robot has EnableSignals
    bool any_attach = false;     // some robot has EnableAttach (runtime links)
    bool any_acond = false;      // some robot has an attach condition
    std::vector<double> mass_tot;  // per robot: mass of the measured voxels (the COM's weights)
    bool any_collision = false;
    // recorded run (vx3g_record) and the adjoint's buffers (vx3g_backward)
    std::vector<void *> rec_mem;
    std::vector<Snap> rec_ck, rec_store;
    Snap rec_end{};
    void *rec_slots = nullptr;
    int64_t rec_start = -1;
    int rec_n = 0, rec_k = 0;
    void *adj_mem = nullptr;
    AdjBufs ab{};
    std::vector<std::pair<long, cudaGraphExec_t>> adj_graphs;  // backward intervals, by (len, parity)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    void *flush = nullptr;
    size_t flush_bytes = 0;
    double *stage = nullptr;  // 4 doubles per voxel: host state exchange

    template <class T> int alloc(T **p, size_t n) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, n ? n * sizeof(T) : 16);
        if (e != cudaSuccess) return fail(VX3G_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(q);
        *p = (T *)q;
        return cudaMemsetAsync(q, 0, n ? n * sizeof(T) : 16, stream) == cudaSuccess ? VX3G_OK : fail(VX3G_ERR_CUDA, "memset");
    }
    template <class T> int upload(T **p, const std::vector<T> &h) {
        int rc = alloc(p, h.size());
        if (rc) return rc;
        if (!h.empty()) CU(cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
        return VX3G_OK;
    }
    void free_record() {
        if (stream) cudaStreamSynchronize(stream);
        for (auto &g : adj_graphs) cudaGraphExecDestroy(g.second);
        adj_graphs.clear();
        for (void *p : rec_mem) cudaFree(p);
        rec_mem.clear();
        rec_ck.clear();
        rec_store.clear();
        rec_slots = nullptr;
        rec_start = -1;
    }
    ~vx3g_ctx() {
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g);
        if (stream) cudaStreamSynchronize(stream);
        free_record();
        if (adj_mem) cudaFree(adj_mem);
        for (void *p : allocs) cudaFree(p);
        if (flush) cudaFree(flush);
        if (stage) cudaFree(stage);
        if (side) cudaStreamSynchronize(side);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// Checks a math-tree program the way VX3_MathTree::eval would run it
// (src/Utils/VX3_MathTree.h:50-191): known operators and variables, operators never
// consume values not yet produced, mtEND within VX3G_MAX_MATH_TOKENS with exactly one
// value left.  Sets *len (tokens including mtEND) and *reads_pos (x, y or z read).
int check_math_program(const vx3g_math_token *t, int *len, bool *reads_pos, std::string *why) {
    int vc = 0, pc = 0;
    *reads_pos = false;
    for (int i = 0; i < VX3G_MAX_MATH_TOKENS; i++) {
        const int op = t[i].op;
        if (op == 0) {
            if (vc - pc != 1) {
                *why = "the program leaves " + std::to_string(vc - pc) + " values (1 expected)";
                return VX3G_ERR_INVALID;
            }
            *len = i + 1;
            return VX3G_OK;
        }
        if (op == 4) {
            const double w = t[i].value;
            if (!(w >= -0.5 && w < 8.5)) {
                *why = "mtVAR names no variable";
                return VX3G_ERR_INVALID;
            }
            if (w < 2.5) *reads_pos = true;
            if (w >= 4.5 && w < 7.5) {
                *why = "variables angle, targetCloseness and numClosePairs (target tracking) are not supported";
                return VX3G_ERR_UNSUPPORTED;
            }
        } else if ((op >= 5 && op <= 9) || (op >= 19 && op <= 22)) {
            pc += 2;
        } else if ((op >= 10 && op <= 18) || op == 23) {
            pc += 1;
        } else if (op < 1 || op > 3) {
            *why = "unknown operator " + std::to_string(op);
            return VX3G_ERR_INVALID;
        }
        if (pc > vc) {
            *why = "an operator at token " + std::to_string(i) + " lacks operands";
            return VX3G_ERR_INVALID;
        }
        vc++;
    }
    *why = "no mtEND within " + std::to_string(VX3G_MAX_MATH_TOKENS) + " tokens";
    return VX3G_ERR_INVALID;
}

int build(vx3g_ctx *c, const vx3g_batch_desc *desc) {
    if (!desc || desc->n_robots <= 0 || !desc->robots) return fail(VX3G_ERR_INVALID, "empty batch descriptor");
    if (desc->precision != VX3G_PRECISION_FP64 && desc->precision != VX3G_PRECISION_MIXED)
        return fail(VX3G_ERR_INVALID, "unknown precision");
    c->precision = desc->precision;
    c->chunk = desc->graph_chunk > 0 ? desc->graph_chunk : 100;
    if (c->chunk & 1) c->chunk++;  // even chunks keep the time-buffer parity aligned
    if (desc->graph_chunk < 0) c->chunk = INT32_MAX;  // no graphs: single steps only
    c->device = desc->device;
    c->nr = desc->n_robots;
    CU(cudaSetDevice(c->device));
    CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));

    std::vector<VMat> vmats;
    std::vector<LMat> lmats;
    std::vector<RobotP> rps(c->nr);
    std::vector<double4> pos, quat;
    std::vector<float> tempe;
    std::vector<double> phase;
    std::vector<uint2> vinfo, linfo;
    std::vector<int> csurf;
    std::vector<MathTok> ftok;
    std::vector<double4> cil_h, cils_h;  // BaseCiliaForce (w: Cilia), ShiftCiliaForce
    std::vector<double> cil_on_h;
    std::vector<int> vnb_h, sigrob_h;    // signals: the voxel across each link, robots with signals
    std::vector<int> arob_h;             // robots with EnableAttach
    std::vector<double> rm_h;  // per voxel: removal time (+inf: never)
    std::vector<float2> ss_h;  // stress-strain points of the non-linear link materials
    std::vector<ExtBC> ext_h;  // boundary-condition externals
    std::vector<int> vext_h;   // per voxel: index into ext_h or -1
    c->voff.assign(c->nr + 1, 0);
    c->loff.assign(c->nr + 1, 0);

    for (int r = 0; r < c->nr; r++) {
        const vx3g_robot_desc &R = desc->robots[r];
        if (R.nx <= 0 || R.ny <= 0 || R.nz <= 0 || !R.lattice)
            return fail(VX3G_ERR_INVALID, "robot " + std::to_string(r) + ": empty lattice");
        if (R.nx > 32767 || R.ny > 32767 || R.nz > 32767) return fail(VX3G_ERR_INVALID, "lattice too large");
        if (R.n_materials < 1 || R.n_materials > 16 || !R.materials)
            return fail(VX3G_ERR_INVALID, "robot " + std::to_string(r) + ": palette must hold 1..16 materials");
        if (!(R.vox_size > 0)) return fail(VX3G_ERR_INVALID, "vox_size must be positive");
        std::vector<HostVMat> hm(R.n_materials);
        const int vbase = (int)vmats.size(), lbase = (int)lmats.size();
        double cte_max = 0;
        for (int i = 0; i < R.n_materials; i++) {
            const vx3g_material &in = R.materials[i];
            if (in.model < 0 || in.model > 3)
                return fail(VX3G_ERR_UNSUPPORTED, "material model (MatModel) must be 0, 1, 2 or 3");
            if (in.model == 3 && (in.n_data < 0 || in.n_data > VX3G_MAX_MODEL_POINTS ||
                                  (in.n_data > 0 && (!in.strain_data || !in.stress_data))))
                return fail(VX3G_ERR_INVALID, "MatModel 3 needs 0.." + std::to_string(VX3G_MAX_MODEL_POINTS) +
                                                  " stress-strain points and both arrays");
            if (R.log10E && in.model > 1)
                return fail(VX3G_ERR_UNSUPPORTED, "per-voxel moduli (log10E) need linear material models");
            hm[i] = import_material(in, R);
            if (!hm[i].model.linear) c->any_nonlinear = true;
            if (!R.log10E) vmats.push_back(to_vmat(hm[i], in));
            cte_max = std::fmax(cte_max, std::fabs((double)hm[i].cte));
        }
        const int nx = R.nx, ny = R.ny, nz = R.nz;
        const long long ncell = (long long)nx * ny * nz;
        std::vector<int> vid(ncell, -1);
        const int v0 = (int)pos.size();
        c->voff[r] = v0;
        c->loff[r] = (int)c->ends.size();
        int nvr = 0;
        for (long long i = 0; i < ncell; i++) {
            int p = R.lattice[i];
            if (p > R.n_materials) return fail(VX3G_ERR_INVALID, "lattice names a missing palette entry");
            if (p > 0) vid[i] = v0 + nvr++;
        }
        std::vector<int> pair_lmat(R.n_materials * R.n_materials, -1);  // unordered pair -> combined values
        std::vector<int> ori_lmat(R.n_materials * R.n_materials, -1);   // (neg, pos) -> oriented material
        std::vector<LMat> pair_vals;
        std::vector<HostVMat> hv;  // per voxel when the robot carries per-voxel moduli
        if (R.log10E) hv.resize(nvr);
        // initial temperature: UpdateMatTemps at import (VX_Sim.cpp:462-478, VX_Environment.cpp:326-345)
        float temp0 = 0.0f;
        if (R.temp_enabled) {
            double cur = R.vary_temp ? (R.temp_period == 0 ? 0.0 : R.temp_base + R.temp_amplitude * std::sin(0.0))
                                     : R.temp_base + R.temp_amplitude;
            temp0 = (float)((float)cur - R.temp_base);
        }
        for (long long i = 0; i < ncell; i++) {
            if (vid[i] < 0) continue;
            const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long long)nx * ny));
            const int mi = R.lattice[i] - 1;
            const bool mx = c->precision == VX3G_PRECISION_MIXED;
            pos.push_back(to_slot(x * R.vox_size, y * R.vox_size, z * R.vox_size, 0.0, mx));
            quat.push_back(to_slot(1, 0, 0, 0, mx));
            tempe.push_back(temp0);
            phase.push_back(R.phase ? R.phase[i] : 0.0);
            c->ijk.push_back(make_short4((short)x, (short)y, (short)z, 0));
            c->vmat_local.push_back(mi);
            uint32_t fl = VF_STATIC | (R.materials[mi].fixed ? VF_FIXED : 0u);
            int vm = vbase + mi;
            if (R.log10E) {  // this voxel's own material: the palette entry with E = 10^log10E
                if (!std::isfinite(R.log10E[i])) return fail(VX3G_ERR_INVALID, "log10E must be finite");
                vx3g_material mm = R.materials[mi];
                mm.E = std::pow(10.0, R.log10E[i]);
                hv[vid[i] - v0] = import_material(mm, R);
                vm = (int)vmats.size();
                vmats.push_back(to_vmat(hv[vid[i] - v0], mm));
            }
            vinfo.push_back(make_uint2((unsigned)r, fl | ((uint32_t)vm << 8)));
            c->vfixed.push_back(R.materials[mi].fixed ? 1 : 0);
            const long long nb[3] = {x > 0 ? i - 1 : -1, y > 0 ? i - nx : -1, z > 0 ? i - (long long)nx * ny : -1};
            for (int a = 0; a < 3; a++) {
                if (nb[a] < 0 || vid[nb[a]] < 0) continue;
                const int vn = vid[nb[a]], vp = vid[i];
                const int mn = c->vmat_local[vn], mp = mi;
                // each ends' damping numerator and Fixed flag ride with the link material, so the
                // link pass needs no per-voxel material lookups
                auto orient = [&](LMat l, const HostVMat &neg, const HostVMat &pos, bool fneg, bool fpos) {
                    l.dmcN = 2 * neg.sqrt_mass * neg.z_int;
                    l.dmcP = 2 * pos.sqrt_mass * pos.z_int;
                    l.fixN = fneg ? 1 : 0;
                    l.fixP = fpos ? 1 : 0;
                    return l;
                };
                int lm;
                if (R.log10E) {  // one link material per link
                    lm = (int)lmats.size() - lbase;
                    lmats.push_back(orient(combine(hv[vp - v0], hv[vn - v0], ss_h), hv[vn - v0], hv[vp - v0],
                                           R.materials[mn].fixed, R.materials[mp].fixed));
                } else {
                    // the combined constants come from the pair's first use (vox1 = the new voxel);
                    // oriented entries (negative end's material first) share them
                    int &base = pair_lmat[mp * R.n_materials + mn];
                    if (base < 0) {
                        base = (int)pair_vals.size();
                        pair_lmat[mn * R.n_materials + mp] = base;
                        pair_vals.push_back(combine(hm[mp], hm[mn], ss_h));
                    }
                    int &ori = ori_lmat[mn * R.n_materials + mp];
                    if (ori < 0) {
                        ori = (int)lmats.size() - lbase;
                        lmats.push_back(orient(pair_vals[base], hm[mn], hm[mp], R.materials[mn].fixed,
                                               R.materials[mp].fixed));
                    }
                    lm = ori;
                }
                const int l = (int)c->ends.size();
                c->ends.push_back(make_int2(vn, vp));
                c->laxis.push_back((uint32_t)a);
                const bool bothFixed = R.materials[mn].fixed && R.materials[mp].fixed;
                linfo.push_back(make_uint2((unsigned)r, (uint32_t)a | LF_SMALL | (bothFixed ? LF_BOTH_FIXED : 0u) |
                                                            ((uint32_t)(lbase + lm) << 8)));
                vinfo[vn].y |= 1u << (2 * a);       // neighbour: link in its positive direction
                vinfo[vp].y |= 1u << (2 * a + 1);   // new voxel: link in its negative direction
                (void)l;
            }
        }
        RobotP &rp = rps[r];
        rp.vox_size = R.vox_size;
        rp.temp_amp = R.temp_amplitude;
        rp.temp_period = R.temp_period;
        rp.inv_period = R.temp_period > 0 ? 1.0 / R.temp_period : 0.0;
        rp.cyc_rate = (float)(rp.inv_period * kCycle);
        rp.amp_f = (float)R.temp_amplitude;
        rp.dt_frac = R.dt_frac;
        rp.voff = v0;
        rp.nv = nvr;
        rp.loff = c->loff[r];
        rp.nl = (int)c->ends.size() - rp.loff;
        rp.floor = R.floor_enabled ? 1 : 0;
        rp.vary_temp = R.vary_temp ? 1 : 0;
        rp.expansion = R.enable_expansion ? 1 : 0;
        rp.collision = R.enable_collision ? 1 : 0;
        rp.detach = R.enable_detach ? 1 : 0;
        c->any_detach |= R.enable_detach != 0;
        // SecondaryExperiment: the voxels of a material with RemoveFromSimulationAfterThisManySeconds > 0
        // leave at the end of the first step that starts later (removeVoxels, VX3_VoxelyzeKernel.cu:365-397)
        rm_h.resize(pos.size(), INFINITY);
        rp.remove = 0;
        if (R.secondary_experiment) {
            for (int k = 0; k < nvr; k++) {
                const double ra = R.materials[c->vmat_local[v0 + k]].remove_after;
                if (ra > 0) {
                    rm_h[v0 + k] = ra;
                    rp.remove = 1;
                }
            }
        }
        c->any_remove |= rp.remove != 0;
        // Environment/Boundary_Conditions: the externals of the voxels the regions touch
        vext_h.resize(pos.size(), -1);
        rp.bcs = 0;
        if (R.n_bcs < 0 || (R.n_bcs > 0 && !R.bcs)) return fail(VX3G_ERR_INVALID, "n_bcs needs the regions");
        for (int j = 0; j < R.n_bcs; j++) {
            if (R.bcs[j].prim == 3)
                return fail(VX3G_ERR_UNSUPPORTED, "mesh boundary-condition regions (PrimType 3) are not supported");
            if (R.bcs[j].prim < 0 || R.bcs[j].prim > 3) return fail(VX3G_ERR_INVALID, "unknown PrimType");
        }
        if (R.n_bcs > 0) {
            std::vector<int> ix(nvr), iy(nvr), iz(nvr);
            for (int k = 0; k < nvr; k++) {
                const short4 l = c->ijk[v0 + k];
                ix[k] = l.x, iy[k] = l.y, iz[k] = l.z;
            }
            const std::vector<VoxelExt> ex = bc_externals(R, ix, iy, iz);
            for (int k = 0; k < nvr; k++) {
                if (!ex[k].any) continue;
                const VoxelExt &e = ex[k];
                ExtBC b{};
                b.t = make_double4(e.t[0], e.t[1], e.t[2], 0.0);
                b.q = make_double4(e.q[0], e.q[1], e.q[2], e.q[3]);
                for (int k = 0; k < 3; k++) b.f[k] = e.f[k], b.m[k] = e.m[k];
                b.dof = e.dof;
                vext_h[v0 + k] = (int)ext_h.size();
                ext_h.push_back(b);
                rp.bcs = 1;
            }
        }
        c->any_bcs |= rp.bcs != 0;
        rp.dyn = rp.detach || rp.remove ? 1 : 0;
        c->any_dyn |= rp.dyn != 0;
        rp.ff_pos = 0;
        for (int k = 0; k < 3; k++) {  // Simulator/ForceField programs
            rp.ff[k] = -1;
            if (!R.force_field[k]) continue;
            int len = 0, rc;
            bool reads_pos = false;
            std::string why;
            if ((rc = check_math_program(R.force_field[k], &len, &reads_pos, &why)))
                return fail(rc, "robot " + std::to_string(r) + ": force_field[" + std::to_string(k) + "]: " + why);
            rp.ff[k] = (int)ftok.size();
            for (int i = 0; i < len; i++) ftok.push_back(MathTok{R.force_field[k][i].op, 0, R.force_field[k][i].value});
            rp.ff_pos |= reads_pos ? 1 : 0;
            rp.ff_any = 1;
            c->ff_pos |= reads_pos;
            c->any_ff = true;
        }
        // largest base size over the run bounds the envelope cutoff 1.25*bs
        // the envelope cutoff (bsa1+bsa2)*0.625 is at most 1.25*vox_size*fmax, fmax the largest
        // base-size factor 1+T*cte any voxel can reach: T spans the initial temperature and,
        // with actuation, [-|A|, 0] (or [-|A|, |A|] with expansion enabled)
        double tlo = temp0, thi = temp0;
        if (R.vary_temp && R.temp_period > 0) {
            tlo = std::fmin(tlo, -std::fabs(R.temp_amplitude));
            thi = std::fmax(thi, R.enable_expansion ? std::fabs(R.temp_amplitude) : 0.0);
        }
        double fmax = 0.0;
        for (int i = 0; i < R.n_materials; i++)
            fmax = std::fmax(fmax, std::fmax(1.0 + tlo * hm[i].cte, 1.0 + thi * hm[i].cte));
        rp.cell_size = 1.25 * R.vox_size * fmax * (1.0 + 1e-6);
        rp.skin = 0.3 * R.vox_size;
        rp.inv_list_cell = 1.0 / (rp.cell_size + rp.skin);
        (void)cte_max;
        rp.soff = (int)csurf.size();
        for (int k = 0; k < nvr; k++) {
            const int v = v0 + k;
            const bool interior = (vinfo[v].y & VF_LINKMASK) == VF_LINKMASK;
            if (!interior) c->surface.push_back(v);
            // detach or removal: any voxel may become a surface voxel, so all take part
            // (interior ones are skipped while their six links hold, removed ones for good);
            // attachment alone only turns surface voxels into interior ones
            if ((!interior || rp.detach || rp.remove) && R.enable_collision) csurf.push_back(v);
        }
        rp.ns = (int)csurf.size() - rp.soff;
        // cilia (gpu_update_cilia_force, VX3_VoxelyzeKernel.cu:846-859): surface voxels of a
        // material with Cilia != 0, once TurnOnCiliaAfterThisManySeconds has passed (k_extra_forces
        // reads the surface from the current link table)
        cil_h.resize(pos.size(), make_double4(0, 0, 0, 0));
        cil_on_h.resize(pos.size(), INFINITY);
        rp.cilia = 0;
        if (R.enable_cilia) {
            for (int k = 0; k < nvr; k++) {
                const int v = v0 + k;
                const vx3g_material &M = R.materials[c->vmat_local[v]];
                const short4 q = c->ijk[v];
                const size_t cell = (size_t)q.x + (size_t)R.nx * ((size_t)q.y + (size_t)R.ny * (size_t)q.z);
                double b[3] = {0, 0, 0}, sh[3] = {0, 0, 0};
                for (int j = 0; j < 3; j++) {
                    if (R.cilia_base) b[j] = R.cilia_base[3 * cell + j];
                    if (R.cilia_shift) sh[j] = R.cilia_shift[3 * cell + j];
                }
                cil_h[v] = make_double4(b[0], b[1], b[2], M.cilia);  // + localSignal * shift on the device
                if (R.enable_signals) {
                    cils_h.resize(pos.size(), make_double4(0, 0, 0, 0));
                    cils_h[v] = make_double4(sh[0], sh[1], sh[2], 0.0);
                }
                if (M.cilia != 0) {
                    cil_on_h[v] = M.cilia_on_after;
                    rp.cilia = 1;
                }
            }
            c->any_cilia |= rp.cilia != 0;
        }
        // signals (the partner across each face: vnb, below)
        rp.signals = R.enable_signals ? 1 : 0;
        if (rp.signals) sigrob_h.push_back(r);
        // EnableAttach: Sticky materials get the link material of their runtime links (the pair
        // (m, m), VX3_VoxelyzeKernel::combinedMaterial), the robot a reserve of links after its
        // lattice's, each face's partner voxel is kept (vnb), and the surface follows the link table
        rp.attach = 0;
        if (R.enable_attach) {
            if (!R.enable_collision)
                return fail(VX3G_ERR_UNSUPPORTED, "robot " + std::to_string(r) + ": enable_attach needs enable_collision");
            for (int k = 0; k < 5; k++) {  // AttachCondition/Condition_k programs
                rp.acond[k] = -1;
                if (!R.attach_condition[k]) continue;
                int len = 0, rc;
                bool reads_pos = false;
                std::string why;
                if ((rc = check_math_program(R.attach_condition[k], &len, &reads_pos, &why)))
                    return fail(rc, "robot " + std::to_string(r) + ": attach_condition[" + std::to_string(k) + "]: " + why);
                rp.acond[k] = (int)ftok.size();
                for (int i = 0; i < len; i++)
                    ftok.push_back(MathTok{R.attach_condition[k][i].op, 0, R.attach_condition[k][i].value});
                c->any_acond = true;
            }
            int sticky_lm = -1;
            for (int i = 0; i < R.n_materials; i++) {
                const vx3g_material &M = R.materials[i];
                if (!M.sticky || R.log10E) continue;  // per-voxel moduli: no two voxels share a material
                if (!hm[i].model.linear || hm[i].nu != 0)
                    return fail(VX3G_ERR_UNSUPPORTED, "robot " + std::to_string(r) + ": a Sticky material must be linear "
                                "(MatModel 0/1) with Poisson's ratio 0 for attachment");
                int &ori = ori_lmat[i * R.n_materials + i];
                if (ori < 0) {
                    ori = (int)lmats.size() - lbase;
                    LMat l = combine(hm[i], hm[i], ss_h);
                    l.dmcN = l.dmcP = 2 * hm[i].sqrt_mass * hm[i].z_int;
                    l.fixN = l.fixP = M.fixed ? 1 : 0;
                    lmats.push_back(l);
                }
                vmats[vbase + i].alm = lbase + ori;
                if (sticky_lm < 0) sticky_lm = lbase + ori;
            }
            // reserve: a runtime link takes a free face of two Sticky voxels; twice the free faces
            // leave room for faces freed again by detach
            long long faces = 0;
            for (int k = 0; k < nvr && sticky_lm >= 0; k++) {
                const int v = v0 + k;
                const vx3g_material &M = R.materials[c->vmat_local[v]];
                if (!M.sticky || M.fixed || R.log10E) continue;
                faces += 6 - __builtin_popcount(vinfo[v].y & VF_LINKMASK);
            }
            rp.ares = (int)c->ends.size();
            rp.acap = faces ? (int)std::min<long long>(faces + 16, INT32_MAX / 4) : 0;
            for (int k = 0; k < rp.acap; k++) {  // unused slots: gone, ends on a voxel of the robot
                c->ends.push_back(make_int2(v0, v0));
                c->laxis.push_back(0u);
                linfo.push_back(make_uint2((unsigned)r, LF_GONE | LF_RUNTIME | LF_SMALL | ((uint32_t)sticky_lm << 8)));
            }
            rp.nl = (int)c->ends.size() - rp.loff;
            rp.guard = R.safety_guard;
            rp.attach = 1;
            rp.dyn = 1;
            c->any_dyn = true;
            c->any_attach = true;
            arob_h.push_back(r);
        }
        if (rp.signals || rp.attach) {  // the voxel across each face's link (lattice links)
            vnb_h.resize(6 * pos.size(), -1);
            for (int l = c->loff[r]; l < rp.loff + rp.nl; l++) {
                if (linfo[l].y & LF_RUNTIME) continue;
                const int a = (int)c->laxis[l];
                vnb_h[6 * (size_t)c->ends[l].x + 2 * a] = c->ends[l].y;      // negative end: toward +axis
                vnb_h[6 * (size_t)c->ends[l].y + 2 * a + 1] = c->ends[l].x;  // positive end: toward -axis
            }
        }
        // lists in shared memory when the robot fits (lattice coordinates below 512, packed in 10 bits each)
        int cmax = 0;
        for (int k = 0; k < nvr; k++) {
            const short4 q = c->ijk[v0 + k];
            cmax = std::max(cmax, (int)std::max(q.x, std::max(q.y, q.z)));
        }
        rp.lchunks = rp.ns > 0 && rp.ns <= kLocalListMax && cmax < 512 ? (rp.ns + kLocalListChunk - 1) / kLocalListChunk : 0;
        // Verlet skin: a robot rebuilt on the global hashed grid (a whole large body at a time)
        // keeps a wider skin than one rebuilt in shared memory, trading longer candidate lists
        // for fewer rebuilds (measured on the 64^3 body and the 256-robot batch)
        if (rp.ns > 0 && !rp.lchunks) {
            rp.skin = 0.5 * R.vox_size;
            rp.inv_list_cell = 1.0 / (rp.cell_size + rp.skin);
        }
    }
    c->voff[c->nr] = (int)pos.size();
    c->loff[c->nr] = (int)c->ends.size();
    if (vmats.size() >= (1u << 24) || lmats.size() >= (1u << 24))
        return fail(VX3G_ERR_INVALID, "more than 2^24 materials (per-voxel moduli on a very large batch)");
    c->mass_tot.assign(c->nr, 0.0);
    for (size_t v = 0; v < vinfo.size(); v++) {
        const VMat &m = vmats[vinfo[v].y >> 8];
        if (m.is_measured) c->mass_tot[vinfo[v].x] += (double)m.mass;
    }
    c->any_collision = !csurf.empty();
    if (pos.size() > (size_t)INT32_MAX / 8) return fail(VX3G_ERR_INVALID, "batch too large");

    Dev &d = c->d;
    std::vector<float> tempe2(tempe);  // two parity buffers of the per-voxel temperature
    tempe2.insert(tempe2.end(), tempe.begin(), tempe.end());
    d.nv = (int)pos.size();
    d.mixed = c->precision == VX3G_PRECISION_MIXED ? 1 : 0;
    d.nl = (int)c->ends.size();
    d.nr = c->nr;
    d.ns = (int)csurf.size();
    int rc;
    if ((rc = c->upload(&d.pos, pos)) || (rc = c->upload(&d.quat, quat)) || (rc = c->alloc(&d.linmom, d.nv)) ||
        (rc = c->alloc(&d.angmom, d.nv)) || (rc = c->alloc(&d.contact, d.nv)) || (rc = c->upload(&d.tempe, tempe2)) ||
        (rc = c->upload(&d.phase, phase)) || (rc = c->upload(&d.vinfo, vinfo)) || (rc = c->upload(&d.ijk, c->ijk)) ||
        (rc = c->upload(&d.ends, c->ends)) || (rc = c->upload(&d.linfo, linfo)) || (rc = c->alloc(&d.strain, d.nl)))
        return rc;
    d.tcyc = d.phc = nullptr;
    if (d.mixed) {  // actuation cycles: the robots' (zero at time 0) and the voxels' phases
        std::vector<float2> phc(phase.size());
        for (size_t i = 0; i < phase.size(); i++) {
            double cy = phase[i] * kCycle;
            cy -= std::floor(cy);
            phc[i].x = (float)cy;
            phc[i].y = (float)(cy - (double)phc[i].x);
        }
        if ((rc = c->upload(&d.phc, phc)) || (rc = c->alloc(&d.tcyc, 2 * (size_t)d.nr))) return rc;
    }
    const size_t rsz = c->precision == VX3G_PRECISION_FP64 ? sizeof(double) : sizeof(float);
    char *ls = nullptr, *sl = nullptr;
    if ((rc = c->alloc(&ls, 9 * (size_t)d.nl * rsz)) || (rc = c->alloc(&sl, 6 * (size_t)d.nv * 6 * rsz))) return rc;
    d.lstate = ls;
    d.slots = sl;
    d.ext = nullptr;
    d.vext = nullptr;
    d.xbc = nullptr;
    d.nxbc = 0;
    if (c->any_bcs) {
        ExtBC *dext;
        if ((rc = c->upload(&dext, ext_h)) || (rc = c->upload(&d.vext, vext_h))) return rc;
        d.ext = dext;
        std::vector<int> xbc;  // the voxels with an external
        for (size_t v = 0; v < vext_h.size(); v++)
            if (vext_h[v] >= 0) xbc.push_back((int)v);
        if ((rc = c->upload(&d.xbc, xbc))) return rc;
        d.nxbc = (int)xbc.size();
    }
    d.soff = nullptr;
    d.ss = nullptr;
    if (!ss_h.empty()) {  // non-linear link materials: their curves and a plastic strain offset per link
        float2 *dss;
        if ((rc = c->upload(&dss, ss_h)) || (rc = c->alloc(&d.soff, d.nl))) return rc;
        d.ss = dss;
    }
    RobotP *drp;
    VMat *dvm;
    LMat *dlm;
    int words = 0;  // attachment: each robot's words of the collision-surface bitmap
    for (int r : arob_h) {
        rps[r].abit = words;
        words += (rps[r].ns + 31) / 32;
    }
    if ((rc = c->upload(&drp, rps)) || (rc = c->upload(&dvm, vmats)) || (rc = c->upload(&dlm, lmats))) return rc;
    d.rp = drp;
    d.vmat = dvm;
    d.lmat = dlm;
    MathTok *dft;
    if ((rc = c->upload(&dft, ftok))) return rc;
    d.ftok = dft;
    d.ffv = nullptr;
    if (c->any_ff && (rc = c->alloc(&d.ffv, d.nv))) return rc;
    d.cil = nullptr;
    d.cil_on = nullptr;
    d.cfv = nullptr;
    d.cils = nullptr;
    d.sig = nullptr;
    d.vnb = nullptr;
    d.sigrob = nullptr;
    d.nsigrob = (int)sigrob_h.size();
    if (d.nsigrob || !arob_h.empty()) {
        vnb_h.resize(6 * pos.size(), -1);
        if ((rc = c->upload(&d.vnb, vnb_h))) return rc;
    }
    if (d.nsigrob) {
        if ((rc = c->alloc(&d.sig, 6 * pos.size())) || (rc = c->upload(&d.sigrob, sigrob_h))) return rc;
        if (!cils_h.empty()) {
            cils_h.resize(pos.size(), make_double4(0, 0, 0, 0));
            if ((rc = c->upload(&d.cils, cils_h))) return rc;
        }
    }
    c->any_signals = d.nsigrob > 0;
    // attachment: enableAttach (true at first, VX3_Voxel.h:302), isNewLink, the scan's marks
    d.vatt = nullptr;
    d.lnew = nullptr;
    d.amask = nullptr;
    d.abits = nullptr;
    d.aflag = d.anum = d.acnt = nullptr;
    d.arob = nullptr;
    d.narob = (int)arob_h.size();
    d.any_acond = c->any_acond ? 1 : 0;
    if (d.narob) {
        if ((rc = c->upload(&d.vatt, std::vector<unsigned char>(pos.size(), 1))) || (rc = c->alloc(&d.lnew, d.nl)) ||
            (rc = c->alloc(&d.amask, d.ns)) || (rc = c->alloc(&d.abits, words)) || (rc = c->alloc(&d.aflag, d.nr)) ||
            (rc = c->alloc(&d.anum, d.nr)) || (rc = c->alloc(&d.acnt, d.nr)) || (rc = c->upload(&d.arob, arob_h)))
            return rc;
    }
    if (c->any_cilia &&
        ((rc = c->upload(&d.cil, cil_h)) || (rc = c->upload(&d.cil_on, cil_on_h)) || (rc = c->alloc(&d.cfv, d.nv))))
        return rc;
    {  // large-robot grid: empty bounding boxes (min keys at the top, max keys at the bottom)
        std::vector<unsigned> box(6 * (size_t)d.nr, 0u);
        for (size_t r = 0; r < (size_t)d.nr; r++) box[6 * r] = box[6 * r + 1] = box[6 * r + 2] = 0xffffffffu;
        if ((rc = c->upload(&d.gbox, box))) return rc;
    }
    d.any_detach = c->any_detach ? 1 : 0;
    d.any_remove = c->any_remove ? 1 : 0;
    d.any_dyn = c->any_dyn ? 1 : 0;
    d.vgone = nullptr;
    d.rm_at = nullptr;
    if (c->any_remove && ((rc = c->alloc(&d.vgone, (size_t)d.nv)) || (rc = c->upload(&d.rm_at, rm_h)))) return rc;
    if ((rc = c->alloc(&d.srf, (size_t)d.nr))) return rc;
    if ((rc = c->alloc(&d.dt, d.nr)) || (rc = c->alloc(&d.T, 2 * (size_t)d.nr)) || (rc = c->alloc(&d.status, d.nr)) ||
        (rc = c->alloc(&d.err, 1)) || (rc = c->alloc(&c->scratch, 4 * (size_t)d.nr + 4)))
        return rc;
    int nvmax = 1;
    for (const RobotP &q : rps) nvmax = std::max(nvmax, q.nv);
    d.com_tiles = (nvmax + kComTile - 1) / kComTile;
    if ((rc = c->alloc(&d.com_part, (size_t)d.nr * d.com_tiles * 4))) return rc;
    // collision tables: robots on the shared-memory path (lchunks > 0) and the global hashed grid
    d.lmax = 0;
    d.nhash = 0;
    std::vector<unsigned> cpk(csurf.size(), 0u);
    for (const RobotP &q : rps) {
        if (q.lchunks) d.lmax = std::max(d.lmax, q.ns);
        else d.nhash += q.ns;
        for (int k = 0; q.lchunks && k < q.ns; k++) {
            const int v = csurf[q.soff + k];
            const short4 l = c->ijk[v];
            cpk[q.soff + k] = (unsigned)l.x | (unsigned)l.y << 10 | (unsigned)l.z << 20 | ((vinfo[v].y & VF_FIXED) ? kPackFixed : 0u);
        }
    }
    int hs = 1024;
    while (hs < 2 * (long long)d.nhash) hs <<= 1;  // room for a dense grid over the robots' boxes
    d.hsize = hs;
    if ((rc = c->upload(&d.csurf, csurf)) || (rc = c->alloc(&d.ccell, d.ns)) || (rc = c->alloc(&d.cposf, d.ns)) ||
        (rc = c->alloc(&d.nbr, (size_t)d.ns * kNbrCap)) || (rc = c->alloc(&d.nnb, d.ns)) || (rc = c->alloc(&d.cflag, 1 + (size_t)d.nr)) || (rc = c->upload(&d.gbar, std::vector<unsigned>{0u, 0u, kBarrierPolls})) ||
        (rc = c->upload(&d.cref, std::vector<float4>((size_t)d.ns, make_float4(1e30f, 1e30f, 1e30f, 0.0f)))) ||
        (rc = c->alloc(&d.hcount, hs)) ||
        (rc = c->alloc(&d.hstart, hs)) || (rc = c->alloc(&d.hfill, hs)) || (rc = c->alloc(&d.spos, d.ns)) || (rc = c->alloc(&d.sij, d.ns)) ||
        (rc = c->alloc(&d.ssurf, d.ns)) || (rc = c->alloc(&d.ggrid, (size_t)d.nr)) || (rc = c->alloc(&d.gmode, 3)) ||
        (rc = c->alloc(&d.hblock, hs / 1024)) || (rc = c->alloc(&d.lwork, (size_t)d.nr)) || (rc = c->upload(&d.cpk, cpk)) ||
        (rc = c->alloc(&d.lwork_ctr, 1)))
        return rc;
    d.crec = nullptr;
    if (d.mixed && d.ns && (rc = c->alloc(&d.crec, 3 * (size_t)d.nv))) return rc;
    CU(init_collision(d));
    // the contact evaluation beside the link pass, except with attachment (its links are made
    // between the check and the evaluation and must not race the link pass's reads)
    if (d.mixed && d.ns && !c->any_attach) {
        CU(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
        c->overlap = true;
    }

    launch_init_temperature(d, c->precision == VX3G_PRECISION_MIXED, c->stream);
    launch_dt(d, c->scratch, c->stream);
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(c->stream));
    return VX3G_OK;
}

void enqueue_links(vx3g_ctx *c) {
    if (c->precision == VX3G_PRECISION_FP64) launch_links_fp64(c->d, c->stream);
    else launch_links_mixed(c->d, c->stream, c->shape_links, !c->any_remove);  // removal writes link info
}
void enqueue_voxels(vx3g_ctx *c, int parity, bool extra = true) {
    if (extra) launch_extra_forces(c->d, parity, c->stream);  // robots with a force field or cilia only
    launch_detach(c->d, c->stream);                // EnableDetach robots only (after the collision pass)
    if (c->precision == VX3G_PRECISION_FP64) launch_voxels_fp64(c->d, parity, c->stream);
    else {
        launch_voxels_mixed(c->d, parity, c->stream, c->shape_voxels, !c->any_detach);  // detach writes voxel info
        launch_voxels_bc_mixed(c->d, parity, c->stream);  // voxels with a boundary condition, if any
    }
    launch_attach_cond(c->d, parity, c->stream);   // robots with attach conditions: enableAttach
    launch_signals(c->d, parity, c->stream);       // EnableSignals robots only (the end of timeStep)
    launch_remove(c->d, parity, c->stream);        // SecondaryExperiment robots only (end of the step)
}

cudaError_t enqueue_step(vx3g_ctx *c, int parity) {
    if (!c->overlap) {
        enqueue_links(c);
        // with attachment the cilia force is taken before any link is made: from the surface the
        // step started with, which the reference's cilia pass walks (VX3_VoxelyzeKernel.cu:296-303)
        if (c->any_attach) launch_extra_forces(c->d, parity, c->stream);
        const cudaError_t e = launch_collision(c->d, c->stream);
        enqueue_voxels(c, parity, !c->any_attach);
        return e;
    }
    // the check / list rebuild, then the contact evaluation on the side stream beside the
    // link pass (disjoint outputs: contact forces; link forces and link state), joined
    // before the voxel pass, which reads both
    cudaError_t e = c->fork_early ? cudaSuccess : launch_coll_prepare(c->d, c->stream);
    if (e != cudaSuccess || (e = cudaEventRecord(c->ev_fork, c->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(c->side, c->ev_fork, 0)) != cudaSuccess ||
        (c->fork_early && (e = launch_coll_prepare(c->d, c->side)) != cudaSuccess))
        return e;
    launch_coll_eval(c->d, c->side);
    launch_links_mixed(c->d, c->stream, c->shape_links, false);
    if ((e = cudaEventRecord(c->ev_join, c->side)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(c->stream, c->ev_join, 0)) != cudaSuccess)
        return e;
    launch_extra_forces(c->d, parity, c->stream);
    launch_detach(c->d, c->stream);
    launch_voxels_mixed(c->d, parity, c->stream, c->shape_voxels, false);
    launch_voxels_bc_mixed(c->d, parity, c->stream);
    launch_signals(c->d, parity, c->stream);
    launch_remove(c->d, parity, c->stream);
    return cudaSuccess;
}

int get_graph(vx3g_ctx *c, int parity, cudaGraphExec_t *out) {
    if (!c->graph[parity]) {
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaSuccess;
        for (int i = 0; i < c->chunk && ce == cudaSuccess; i++) ce = enqueue_step(c, (parity + i) & 1);
        cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
        if (ce != cudaSuccess) {
            if (ee == cudaSuccess) cudaGraphDestroy(g);
            return fail(VX3G_ERR_CUDA, std::string("step graph capture: ") + cudaGetErrorString(ce));
        }
        CU(ee);
        cudaError_t e = cudaGraphInstantiate(&c->graph[parity], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(VX3G_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    *out = c->graph[parity];
    return VX3G_OK;
}

template <class T> int download(vx3g_ctx *c, std::vector<T> &h, const T *dptr, size_t n) {
    h.resize(n);
    if (n) CU(cudaMemcpyAsync(h.data(), dptr, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    return VX3G_OK;
}

}  // namespace

extern "C" {

const char *vx3g_last_error(void) { return g_err.c_str(); }

vx3g_ctx *vx3g_create(const vx3g_batch_desc *desc, int *status) {
    vx3g_ctx *c = new (std::nothrow) vx3g_ctx();
    if (!c) {
        if (status) *status = fail(VX3G_ERR_NOMEM, "host allocation failed");
        return nullptr;
    }
    int rc = build(c, desc);
    if (status) *status = rc;
    if (rc != VX3G_OK) {
        delete c;
        return nullptr;
    }
    return c;
}

void vx3g_destroy(vx3g_ctx *c) { delete c; }

int vx3g_step(vx3g_ctx *c, int n) {
    if (!c || n < 0) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_step");
    CU(cudaSetDevice(c->device));
    while (n > 0) {
        const int parity = (int)(c->steps & 1);
        if (n >= c->chunk) {
            cudaGraphExec_t g;
            int rc = get_graph(c, parity, &g);
            if (rc) return rc;
            CU(cudaGraphLaunch(g, c->stream));
            n -= c->chunk;
            c->steps += c->chunk;
        } else {
            CU(enqueue_step(c, parity));
            n -= 1;
            c->steps += 1;
        }
    }
    CU(cudaGetLastError());
    return VX3G_OK;
}

int vx3g_prepare_graphs(vx3g_ctx *c) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    if (c->chunk == INT32_MAX) return VX3G_OK;  // graphs off
    CU(cudaSetDevice(c->device));
    cudaGraphExec_t g;
    for (int parity = 0; parity < 2; parity++)
        if (int rc = get_graph(c, parity, &g)) return rc;
    return VX3G_OK;
}

int vx3g_synchronize(vx3g_ctx *c) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    CU(cudaStreamSynchronize(c->stream));
    return VX3G_OK;
}

void *vx3g_stream(vx3g_ctx *c) { return c ? (void *)c->stream : nullptr; }
int64_t vx3g_steps_taken(vx3g_ctx *c) { return c ? c->steps : -1; }

// The surface voxels (fewer than six links, not removed) in voxel order: fixed at
// creation, or read from the current link table when links can detach or voxels leave.
static int current_surface(vx3g_ctx *c, std::vector<int> &out) {
    if (!c->any_dyn) {
        out = c->surface;
        return VX3G_OK;
    }
    std::vector<uint2> vi((size_t)c->d.nv);
    std::vector<unsigned char> gone((size_t)c->d.nv, 0);
    if (c->d.nv) CU(cudaMemcpyAsync(vi.data(), c->d.vinfo, sizeof(uint2) * vi.size(), cudaMemcpyDeviceToHost, c->stream));
    if (c->d.nv && c->d.vgone)
        CU(cudaMemcpyAsync(gone.data(), c->d.vgone, gone.size(), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    out.clear();
    for (size_t v = 0; v < vi.size(); v++)
        if ((vi[v].y & VF_LINKMASK) != VF_LINKMASK && !gone[v]) out.push_back((int)v);
    return VX3G_OK;
}

// The link table as it stands: the host copy of the lattice's links, or, with attachment,
// the device's (runtime links made so far, unused reserve slots with ends -1).
static int current_links(vx3g_ctx *c, std::vector<int2> &ends, std::vector<uint32_t> &axis) {
    if (!c->any_attach) {
        ends = c->ends;
        axis = c->laxis;
        return VX3G_OK;
    }
    std::vector<uint2> li;
    std::vector<int> made;
    std::vector<RobotP> rps;
    int rc;
    if ((rc = download(c, ends, c->d.ends, c->d.nl)) || (rc = download(c, li, c->d.linfo, c->d.nl)) ||
        (rc = download(c, made, c->d.anum, c->nr)) || (rc = download(c, rps, c->d.rp, c->nr)))
        return rc;
    CU(cudaStreamSynchronize(c->stream));
    axis.resize(ends.size());
    for (size_t l = 0; l < ends.size(); l++) {
        axis[l] = li[l].y & LF_AXIS;
        const RobotP &q = rps[li[l].x];
        if ((li[l].y & LF_RUNTIME) && (int)l >= q.ares + made[li[l].x]) ends[l] = make_int2(-1, -1);
    }
    return VX3G_OK;
}

int vx3g_links_in_use(vx3g_ctx *c, int32_t *n) {
    if (!c || !n) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_links_in_use");
    std::vector<int> made(c->nr, 0);
    std::vector<RobotP> rps;
    int rc;
    if ((rc = download(c, rps, c->d.rp, c->nr))) return rc;
    if (c->any_attach && (rc = download(c, made, c->d.anum, c->nr))) return rc;
    CU(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < c->nr; r++) n[r] = (rps[r].attach ? rps[r].ares - rps[r].loff : rps[r].nl) + made[r];
    return VX3G_OK;
}

int vx3g_counts(vx3g_ctx *c, int *nv, int *nl, int *ns) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    if (nv) *nv = c->d.nv;
    if (nl) *nl = c->d.nl;
    if (ns) {
        std::vector<int> cur;
        int rc = current_surface(c, cur);
        if (rc) return rc;
        *ns = (int)cur.size();
    }
    return VX3G_OK;
}

int vx3g_offsets(vx3g_ctx *c, int *vo, int *lo) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    for (int r = 0; r <= c->nr; r++) {
        if (vo) vo[r] = c->voff[r];
        if (lo) lo[r] = c->loff[r];
    }
    return VX3G_OK;
}

static int ensure_stage(vx3g_ctx *c) {
    if (c->stage) return VX3G_OK;
    cudaError_t e = cudaMalloc(&c->stage, 4 * sizeof(double) * (size_t)(c->d.nv ? c->d.nv : 1));
    if (e != cudaSuccess) {
        c->stage = nullptr;
        return fail(VX3G_ERR_NOMEM, std::string("cudaMalloc (state staging): ") + cudaGetErrorString(e));
    }
    return VX3G_OK;
}

// The device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister), or
// nullptr for pageable or device memory: vx3g_set_state's kernel reads page-locked
// buffers in place instead of staging them through a device copy (0.17 -> 0.12 ms for
// the 16 MB of a 64^3 body).  vx3g_get_state stages its writes: kernel stores into host
// memory were slower than the copy engine (0.21 -> 0.31 ms).
static const void *pinned_device_pointer(const void *p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // not a CUDA pointer: clear the error
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int vx3g_get_state(vx3g_ctx *c, double *pos, double *orient, double *linmom, double *angmom) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    CU(cudaSetDevice(c->device));
    int rc = ensure_stage(c);
    if (rc) return rc;
    const size_t n = c->d.nv;
    double *out[4] = {pos, orient, linmom, angmom};
    const double4 *src[4] = {c->d.pos, c->d.quat, c->d.linmom, c->d.angmom};
    for (int k = 0; k < 4; k++) {
        if (!out[k]) continue;
        const int comps = k == 1 ? 4 : 3;
        launch_unpack_state(c->d, c->stage, src[k], comps, c->stream);
        CU(cudaMemcpyAsync(out[k], c->stage, comps * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaGetLastError());
    return VX3G_OK;
}

int vx3g_set_state(vx3g_ctx *c, const double *pos, const double *orient, const double *linmom, const double *angmom) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    CU(cudaSetDevice(c->device));
    int rc = ensure_stage(c);
    if (rc) return rc;
    const size_t n = c->d.nv;
    const double *in[4] = {pos, orient, linmom, angmom};
    double4 *dst[4] = {c->d.pos, c->d.quat, c->d.linmom, c->d.angmom};
    for (int k = 0; k < 4; k++) {
        if (!in[k]) continue;
        const int comps = k == 1 ? 4 : 3;
        const double *from = (const double *)pinned_device_pointer(in[k]);  // page-locked: read in place
        if (!from) {
            CU(cudaMemcpyAsync(c->stage, in[k], comps * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
            from = c->stage;
        }
        launch_pack_state(c->d, dst[k], from, comps, k == 0, c->stream);  // pos keeps its base size
    }
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaGetLastError());
    return VX3G_OK;
}

int vx3g_get_voxel_aux(vx3g_ctx *c, float *tempe, int32_t *flags, double *contact) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    const size_t n = c->d.nv;
    std::vector<float> t;
    std::vector<uint2> vi;
    std::vector<double4> ct;
    std::vector<RobotP> rps;
    int rc;
    // the buffer of the last step taken holds the temperature that step used
    const size_t tb = c->steps > 0 ? (size_t)((c->steps - 1) & 1) : 0;
    if (tempe && (rc = download(c, t, c->d.tempe + tb * n, n))) return rc;
    if (flags && ((rc = download(c, vi, c->d.vinfo, n)) || (rc = download(c, rps, c->d.rp, (size_t)c->nr)))) return rc;
    if (contact && (rc = download(c, ct, c->d.contact, n))) return rc;
    CU(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; i++) {
        if (tempe) tempe[i] = t[i];
        if (flags) {
            const uint32_t f = vi[i].y;
            // reference voxState bits: SURFACE(2, set for interior voxels), FLOOR_ENABLED(4), FLOOR_STATIC_FRICTION(8)
            flags[i] = (((f & VF_LINKMASK) == VF_LINKMASK) ? 2 : 0) | (rps[vi[i].x].floor ? 4 : 0) | ((f & VF_STATIC) ? 8 : 0);
        }
        if (contact && c->d.mixed) {  // mixed precision: float4 per voxel in the first half of the buffer
            const float4 f = reinterpret_cast<const float4 *>(ct.data())[i];
            contact[3 * i] = f.x; contact[3 * i + 1] = f.y; contact[3 * i + 2] = f.z;
        } else if (contact) {
            contact[3 * i] = ct[i].x; contact[3 * i + 1] = ct[i].y; contact[3 * i + 2] = ct[i].z;
        }
    }
    return VX3G_OK;
}

int vx3g_get_links(vx3g_ctx *c, float *strain, float *max_strain, double *local9, double *forces12, int32_t *small) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    const size_t nl = c->d.nl, nv = c->d.nv;
    std::vector<int2> lends;
    std::vector<uint32_t> laxis;
    if (forces12) {
        int rc = current_links(c, lends, laxis);
        if (rc) return rc;
    }
    const bool fp64 = c->precision == VX3G_PRECISION_FP64;
    const size_t rsz = fp64 ? 8 : 4;
    std::vector<float2> sm;
    std::vector<uint2> li;
    std::vector<char> ls, sl;
    int rc;
    if ((strain || max_strain) && (rc = download(c, sm, c->d.strain, nl))) return rc;
    if (small && (rc = download(c, li, c->d.linfo, nl))) return rc;
    if (local9 && (rc = download(c, ls, (const char *)c->d.lstate, 9 * nl * rsz))) return rc;
    if (forces12 && (rc = download(c, sl, (const char *)c->d.slots, 36 * nv * rsz))) return rc;
    CU(cudaStreamSynchronize(c->stream));
    auto rd = [&](const std::vector<char> &buf, size_t idx) -> double {
        if (fp64) return ((const double *)buf.data())[idx];
        return (double)((const float *)buf.data())[idx];
    };
    for (size_t l = 0; l < nl; l++) {
        if (strain) strain[l] = sm[l].x;
        if (max_strain) max_strain[l] = sm[l].y;
        if (small) small[l] = ((li[l].y & LF_SMALL) ? 1 : 0) | ((li[l].y & LF_GONE) ? 2 : 0) | ((li[l].y & LF_LVV) ? 4 : 0);
        if (local9) {  // pos2, angle1v, angle2v
            if (fp64) {
                for (int k = 0; k < 9; k++) local9[9 * l + k] = rd(ls, (size_t)k * nl + l);
            } else {  // mixed: rows {pos2, angle2v.x}, {angle2v.y, angle2v.z}, then angle1v component-major
                for (int k = 0; k < 3; k++) local9[9 * l + k] = rd(ls, 4 * l + k);
                for (int k = 0; k < 3; k++) local9[9 * l + 3 + k] = rd(ls, 6 * nl + (size_t)k * nl + l);
                local9[9 * l + 6] = rd(ls, 4 * l + 3);
                local9[9 * l + 7] = rd(ls, 4 * nl + 2 * l);
                local9[9 * l + 8] = rd(ls, 4 * nl + 2 * l + 1);
            }
        }
        if (forces12 && lends[l].x < 0) {  // an unused reserve slot
            std::fill(forces12 + 12 * l, forces12 + 12 * l + 12, 0.0);
        } else if (forces12) {
            const int a = (int)laxis[l];
            const size_t in = (size_t)(2 * a) * nv + lends[l].x, ip = (size_t)(2 * a + 1) * nv + lends[l].y;
            // the six components (force x, y, z, moment x, y, z) of slot i: FP64 Slot<double>;
            // mixed precision: a 16-byte row {f, m.x} then, after all of those, an 8-byte row {m.y, m.z}
            auto comp = [&](size_t i, int k) -> double {
                if (fp64) return rd(sl, i * 6 + k);
                return k < 4 ? rd(sl, i * 4 + k) : rd(sl, 24 * nv + i * 2 + (k - 4));
            };
            for (int k = 0; k < 3; k++) {
                forces12[12 * l + k] = comp(in, k);          // forceNeg
                forces12[12 * l + 3 + k] = comp(ip, k);      // forcePos
                forces12[12 * l + 6 + k] = comp(in, 3 + k);  // momentNeg
                forces12[12 * l + 9 + k] = comp(ip, 3 + k);  // momentPos
            }
        }
    }
    return VX3G_OK;
}

int vx3g_get_signals(vx3g_ctx *c, double *local) {
    if (!c || !local) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_get_signals");
    const size_t n = c->d.nv;
    if (!c->d.sig) {
        std::fill(local, local + n, 0.0);
        return VX3G_OK;
    }
    std::vector<double> h;
    int rc;
    if ((rc = download(c, h, c->d.sig, 6 * n))) return rc;
    CU(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; i++) local[i] = h[6 * i];
    return VX3G_OK;
}

int vx3g_get_topology(vx3g_ctx *c, int32_t *ijk, int32_t *vmat, int32_t *ends, int32_t *axis) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    std::vector<int2> lends;
    std::vector<uint32_t> laxis;
    if (ends || axis) {
        int rc = current_links(c, lends, laxis);
        if (rc) return rc;
    }
    for (size_t i = 0; i < (size_t)c->d.nv; i++) {
        if (ijk) { ijk[3 * i] = c->ijk[i].x; ijk[3 * i + 1] = c->ijk[i].y; ijk[3 * i + 2] = c->ijk[i].z; }
        if (vmat) vmat[i] = c->vmat_local[i];
    }
    for (size_t l = 0; l < (size_t)c->d.nl; l++) {
        if (ends) { ends[2 * l] = lends[l].x; ends[2 * l + 1] = lends[l].y; }
        if (axis) axis[l] = (int32_t)laxis[l];
    }
    return VX3G_OK;
}

int vx3g_get_surface(vx3g_ctx *c, int32_t *surface) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    std::vector<int> cur;
    int rc = current_surface(c, cur);
    if (rc) return rc;
    for (size_t i = 0; i < cur.size(); i++) surface[i] = cur[i];
    return VX3G_OK;
}

int vx3g_com(vx3g_ctx *c, double *com) {
    if (!c || !com) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_com");
    std::vector<double> out;
    double *dout = c->scratch;  // 4*nr doubles
    launch_com(c->d, dout, c->stream);
    CU(cudaGetLastError());
    int rc = download(c, out, (const double *)dout, 3 * (size_t)c->nr);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    memcpy(com, out.data(), 3 * c->nr * sizeof(double));
    return VX3G_OK;
}

int vx3g_dt(vx3g_ctx *c, double *dt) {
    if (!c || !dt) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_dt");
    std::vector<float> h;
    int rc = download(c, h, c->d.dt, (size_t)c->nr);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < c->nr; r++) dt[r] = h[r];
    return VX3G_OK;
}

int vx3g_time(vx3g_ctx *c, double *t) {
    if (!c || !t) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_time");
    std::vector<double> h;
    int rc = download(c, h, c->d.T + (size_t)(c->steps & 1) * c->nr, (size_t)c->nr);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    memcpy(t, h.data(), c->nr * sizeof(double));
    return VX3G_OK;
}

int vx3g_status(vx3g_ctx *c, int32_t *st) {
    if (!c || !st) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_status");
    std::vector<int> h, err;
    int rc = download(c, h, c->d.status, (size_t)c->nr);
    if (rc || (rc = download(c, err, c->d.err, 1))) return rc;
    CU(cudaStreamSynchronize(c->stream));
    memcpy(st, h.data(), c->nr * sizeof(int));
    if (err[0] & 1) {
        // a grid barrier gave up: CTAs that left early may have left a stale arrival count
        // and half-built candidate lists.  With nothing in flight (the stream is idle),
        // clear the barrier words and the error word and make every robot's lists due, so
        // the next step rebuilds them from scratch; the report stands for the steps taken.
        CU(cudaMemsetAsync(c->d.gbar, 0, 2 * sizeof(unsigned), c->stream));
        CU(cudaMemsetAsync(c->d.err, 0, sizeof(int), c->stream));
        if (c->d.ns) {
            const std::vector<float4> far((size_t)c->d.ns, make_float4(1e30f, 1e30f, 1e30f, 0.0f));
            CU(cudaMemcpyAsync(c->d.cref, far.data(), far.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
        }
        CU(cudaStreamSynchronize(c->stream));
        return fail(VX3G_ERR_DEVICE, "collision pass: a grid barrier of k_coll_prepare timed out");
    }
    return VX3G_OK;
}

int vx3g_debug_barrier(vx3g_ctx *c, uint32_t polls, uint32_t arrivals) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    CU(cudaSetDevice(c->device));
    const unsigned w[3] = {arrivals, 0u, polls ? polls : kBarrierPolls};
    CU(cudaMemcpyAsync(c->d.gbar, w, sizeof w, cudaMemcpyHostToDevice, c->stream));
    if (polls && c->d.ns) {  // make every robot's lists due, so the next step runs the barriers
        const std::vector<float4> far((size_t)c->d.ns, make_float4(1e30f, 1e30f, 1e30f, 0.0f));
        CU(cudaMemcpyAsync(c->d.cref, far.data(), far.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    }
    CU(cudaStreamSynchronize(c->stream));
    return VX3G_OK;
}

int vx3g_stop_robot(vx3g_ctx *c, int robot) {
    if (!c || robot < 0 || robot >= c->nr) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_stop_robot");
    launch_or_status(c->d, robot, VX3G_ROBOT_STOPPED, c->stream);
    CU(cudaGetLastError());
    return VX3G_OK;
}

int vx3g_time_steps(vx3g_ctx *c, int n, float *ms) {
    if (!c || !ms || n < 0) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_time_steps");
    cudaEvent_t a, b;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    CU(cudaEventRecord(a, c->stream));
    int rc = vx3g_step(c, n);
    CU(cudaEventRecord(b, c->stream));
    CU(cudaEventSynchronize(b));
    CU(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

int vx3g_flush_l2(vx3g_ctx *c, size_t bytes) {
    if (!c) return fail(VX3G_ERR_INVALID, "null context");
    if (bytes > c->flush_bytes) {
        if (c->flush) cudaFree(c->flush);
        c->flush = nullptr;
        c->flush_bytes = 0;
        CU(cudaMalloc(&c->flush, bytes));
        c->flush_bytes = bytes;
    }
    static unsigned char v = 0;
    CU(cudaMemsetAsync(c->flush, ++v, bytes, c->stream));
    return VX3G_OK;
}

int vx3g_time_passes(vx3g_ctx *c, int iters, float *ms4) {
    if (!c || !ms4 || iters <= 0) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_time_passes");
    CU(cudaSetDevice(c->device));
    cudaEvent_t a, b;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    const Dev &d = c->d;
    for (int pass = 0; pass < 4; pass++) {
        // each pass repeated `iters` times inside one CUDA graph, as the step graphs run it
        const int p0 = (int)(c->steps & 1);
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < iters; i++) {
            if (pass == 0) enqueue_links(c);
            else if (pass == 1) launch_collision(d, c->stream);
            else if (pass == 2) enqueue_voxels(c, (p0 + i) & 1);
            else launch_coll_eval(d, c->stream);
        }
        CU(cudaStreamEndCapture(c->stream, &g));
        cudaGraphExec_t ex = nullptr;
        cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(VX3G_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        CU(cudaEventRecord(a, c->stream));
        CU(cudaGraphLaunch(ex, c->stream));
        CU(cudaEventRecord(b, c->stream));
        CU(cudaEventSynchronize(b));
        cudaGraphExecDestroy(ex);
        if (pass == 2) c->steps += iters;
        float ms = 0;
        CU(cudaEventElapsedTime(&ms, a, b));
        ms4[pass] = ms / iters;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    CU(cudaGetLastError());
    return VX3G_OK;
}

int vx3g_autotune(vx3g_ctx *c, int n_steps, const char *cache_json) {
    if (!c || n_steps < 0) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_autotune");
    if (c->precision != VX3G_PRECISION_MIXED) return vx3g_step(c, n_steps);  // one shape per FP64 pass
    CU(cudaSetDevice(c->device));
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, c->device));
    const std::string key = std::string(prop.name) + "|mixed|" + std::to_string(c->d.nv) + "|" +
                            std::to_string(c->d.nl) + "|" + std::to_string(c->d.ns);
    std::string cache;
    if (cache_json) {
        if (FILE *f = fopen(cache_json, "rb")) {
            char buf[4096];
            size_t k;
            while ((k = fread(buf, 1, sizeof buf, f)) > 0) cache.append(buf, k);
            fclose(f);
        }
        const size_t at = cache.find("\"" + key + "\": [");
        int a = -1, b = -1, fk = 0;
        if (at != std::string::npos &&
            sscanf(cache.c_str() + at + key.size() + 5, "%d, %d, %d", &a, &b, &fk) >= 2 && a >= 0 && a < kMixedShapes &&
            b >= 0 && b < kMixedShapes) {
            fk = (fk == 1 && c->overlap) ? 1 : 0;
            if (a != c->shape_links || b != c->shape_voxels || fk != c->fork_early) {
                for (auto &g : c->graph)
                    if (g) cudaGraphExecDestroy(g), g = nullptr;
            }
            c->shape_links = a;
            c->shape_voxels = b;
            c->fork_early = fk;
            return vx3g_step(c, n_steps);
        }
    }
    // time the passes of real steps, cycling through the shapes (results do not depend on them),
    // then whole steps alternating the fork point of the overlapped step
    const int warm = 2 * kMixedShapes;
    if (n_steps < warm + 2 * kMixedShapes) return vx3g_step(c, n_steps);
    const int n_fork = c->overlap && n_steps >= 2 * (warm + 2 * kMixedShapes) ? std::min(n_steps / 2, 64) : 0;
    const int n_shape = n_steps - n_fork;
    std::vector<cudaEvent_t> ev(4 * (size_t)n_steps);
    for (auto &e : ev) CU(cudaEventCreate(&e));
    for (int i = 0; i < n_shape; i++) {
        const int parity = (int)(c->steps & 1);
        c->shape_links = c->shape_voxels = i % kMixedShapes;
        CU(cudaEventRecord(ev[4 * i], c->stream));
        enqueue_links(c);
        CU(cudaEventRecord(ev[4 * i + 1], c->stream));
        CU(launch_collision(c->d, c->stream));
        CU(cudaEventRecord(ev[4 * i + 2], c->stream));
        enqueue_voxels(c, parity);
        CU(cudaEventRecord(ev[4 * i + 3], c->stream));
        c->steps++;
    }
    CU(cudaStreamSynchronize(c->stream));
    double tl[kMixedShapes] = {}, tv[kMixedShapes] = {};
    for (int i = warm; i < n_shape; i++) {
        float a = 0, b = 0;
        CU(cudaEventElapsedTime(&a, ev[4 * i], ev[4 * i + 1]));
        CU(cudaEventElapsedTime(&b, ev[4 * i + 2], ev[4 * i + 3]));
        tl[i % kMixedShapes] += a;
        tv[i % kMixedShapes] += b;
    }
    int bl = 0, bv = 0;
    for (int k = 1; k < kMixedShapes; k++) {
        if (tl[k] < tl[bl]) bl = k;
        if (tv[k] < tv[bv]) bv = k;
    }
    c->shape_links = bl;
    c->shape_voxels = bv;
    // the fork point: graphs of G whole overlapped steps (the form vx3g_step runs them in),
    // one per fork point, launched alternately; the first launch of each is not counted
    constexpr int G = 8;
    const int reps = n_fork / (2 * G);
    double tf[2] = {0.0, 0.0};
    if (reps >= 2) {
        cudaGraphExec_t gx[2] = {nullptr, nullptr};
        const int p0 = (int)(c->steps & 1);  // G is even: every launch starts at this parity
        for (int m = 0; m < 2; m++) {
            c->fork_early = m;
            cudaGraph_t gr;
            CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t ce = cudaSuccess;
            for (int i = 0; i < G && ce == cudaSuccess; i++) ce = enqueue_step(c, (p0 + i) & 1);
            const cudaError_t ee = cudaStreamEndCapture(c->stream, &gr);
            if (ce != cudaSuccess || ee != cudaSuccess) {
                if (ee == cudaSuccess) cudaGraphDestroy(gr);
                if (gx[0]) cudaGraphExecDestroy(gx[0]);
                return fail(VX3G_ERR_CUDA, "autotune graph capture");
            }
            const cudaError_t ie = cudaGraphInstantiate(&gx[m], gr, 0);
            cudaGraphDestroy(gr);
            if (ie != cudaSuccess) {
                if (gx[0]) cudaGraphExecDestroy(gx[0]);
                return fail(VX3G_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
            }
        }
        for (int k = 0; k < 2 * reps; k++) {
            CU(cudaEventRecord(ev[2 * k], c->stream));
            CU(cudaGraphLaunch(gx[k & 1], c->stream));
            CU(cudaEventRecord(ev[2 * k + 1], c->stream));
            c->steps += G;
        }
        CU(cudaStreamSynchronize(c->stream));
        for (int k = 2; k < 2 * reps; k++) {
            float a = 0;
            CU(cudaEventElapsedTime(&a, ev[2 * k], ev[2 * k + 1]));
            tf[k & 1] += a;
        }
        cudaGraphExecDestroy(gx[0]);
        cudaGraphExecDestroy(gx[1]);
    }
    c->fork_early = reps >= 2 && tf[1] < tf[0] ? 1 : 0;
    for (int i = 2 * reps * G; i < n_fork; i++) {  // the rest of the n_steps, at the chosen point
        CU(enqueue_step(c, (int)(c->steps & 1)));
        c->steps++;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (auto &g : c->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    if (cache_json) {  // flat JSON object {"<gpu>|mixed|nv|nl|ns": [link shape, voxel shape, fork point], ...}
        std::string body = cache;
        const size_t close = body.rfind('}');
        const std::string entry = "\"" + key + "\": [" + std::to_string(bl) + ", " + std::to_string(bv) + ", " +
                                  std::to_string(c->fork_early) + "]";
        if (close == std::string::npos || body.find('"') == std::string::npos) {
            body = "{\n  " + entry + "\n}\n";
        } else {
            body = body.substr(0, close);
            while (!body.empty() && (body.back() == '\n' || body.back() == ' ')) body.pop_back();
            body += ",\n  " + entry + "\n}\n";
        }
        if (FILE *f = fopen(cache_json, "wb")) {
            fwrite(body.data(), 1, body.size(), f);
            fclose(f);
        }
    }
    return VX3G_OK;
}

int vx3g_launch_shapes(vx3g_ctx *c, int32_t *shapes4) {
    if (!c || !shapes4) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_launch_shapes");
    const bool mx = c->precision == VX3G_PRECISION_MIXED;
    shapes4[0] = mx ? kLinkShapes[c->shape_links].threads : 256;
    shapes4[1] = mx ? kLinkShapes[c->shape_links].min_blocks : 1;
    shapes4[2] = mx ? kVoxelShapes[c->shape_voxels].threads : 256;
    shapes4[3] = mx ? kVoxelShapes[c->shape_voxels].min_blocks : 1;
    return VX3G_OK;
}

int vx3g_recommended_dt_noalloc(vx3g_ctx *c, double *rdt) {
    if (!c || !rdt) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_recommended_dt_noalloc");
    CU(cudaSetDevice(c->device));
    const char *why = "";
    const int rc = recommended_dt_noalloc(c->d, c->device, rdt, c->stream, &why);
    if (rc == -1) return fail(VX3G_ERR_INVALID, why);
    if (rc != 0) return fail(VX3G_ERR_CUDA, why);
    return VX3G_OK;
}

// ---- differentiation: recorded run with checkpoints, adjoint run backwards

}  // extern "C"

namespace {

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t snap_bytes(const Dev &d) {
    const size_t nv = d.nv, nl = d.nl, nr = d.nr;
    return 4 * al256(nv * sizeof(double4)) + al256(nv * sizeof(uint2)) + al256(2 * nv * sizeof(float)) +
           al256(9 * nl * sizeof(double)) + al256(nl * sizeof(float2)) + al256(nl * sizeof(uint2)) +
           al256(2 * nr * sizeof(double)) + al256(nr * sizeof(int));
}

Snap carve(const Dev &d, char *p) {
    const size_t nv = d.nv, nl = d.nl, nr = d.nr;
    auto take = [&p](size_t n) {
        char *q = p;
        p += al256(n);
        return q;
    };
    Snap s;
    s.pos = (double4 *)take(nv * sizeof(double4));
    s.quat = (double4 *)take(nv * sizeof(double4));
    s.linmom = (double4 *)take(nv * sizeof(double4));
    s.angmom = (double4 *)take(nv * sizeof(double4));
    s.vinfo = (uint2 *)take(nv * sizeof(uint2));
    s.tempe = (float *)take(2 * nv * sizeof(float));
    s.lstate = (double *)take(9 * nl * sizeof(double));
    s.strain = (float2 *)take(nl * sizeof(float2));
    s.linfo = (uint2 *)take(nl * sizeof(uint2));
    s.T = (double *)take(2 * nr * sizeof(double));
    s.status = (int *)take(nr * sizeof(int));
    return s;
}

Snap live_snap(const Dev &d) {
    Snap s;
    s.pos = d.pos; s.quat = d.quat; s.linmom = d.linmom; s.angmom = d.angmom;
    s.vinfo = d.vinfo; s.tempe = d.tempe;
    s.lstate = (double *)d.lstate; s.strain = d.strain; s.linfo = d.linfo;
    s.T = d.T; s.status = d.status;
    return s;
}

int alloc_snaps(vx3g_ctx *c, std::vector<Snap> &out, int n) {
    const size_t sb = snap_bytes(c->d);
    for (int i = 0; i < n; i++) {
        void *m = nullptr;
        cudaError_t e = cudaMalloc(&m, sb);
        if (e != cudaSuccess) return fail(VX3G_ERR_NOMEM, std::string("cudaMalloc (state snapshots): ") + cudaGetErrorString(e));
        c->rec_mem.push_back(m);
        out.push_back(carve(c->d, (char *)m));
    }
    return VX3G_OK;
}

// One checkpoint interval of the backward pass as a CUDA graph: recompute the
// interval's len states from the live state (the checkpoint, copied in just before),
// then run the reverse steps over them.  Cached per (len, parity of the first step).
cudaError_t enqueue_adj_segment(vx3g_ctx *c, const AdjBufs &a0, int len, int p0) {
    const Dev &d = c->d;
    const Snap live = live_snap(d);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < len && e == cudaSuccess; i++) {
        launch_snap_copy(c->rec_store[i], live, d.nv, d.nl, d.nr, c->stream);
        e = enqueue_step(c, (p0 + i) & 1);
    }
    AdjBufs a = a0;
    if (!c->any_collision) {
        launch_adj_slots(d, c->rec_store[len - 1], a, c->stream);
        for (int i = len - 1; i >= 0; i--) {
            a.parity = (p0 + i) & 1;
            launch_adj_voxel_link(d, c->rec_store[i], a, c->stream);
            launch_adj_gather_slots(d, c->rec_store[i], i > 0 ? &c->rec_store[i - 1] : nullptr, a, c->stream);
        }
        return e;
    }
    // with collisions, per reverse step: the step's contact forces from its stored state
    // (the candidate lists checked and rebuilt against that state as the forward pass
    // does), then the link-force recompute, the voxel and link adjoints, the contact
    // adjoint and the gather
    for (int i = len - 1; i >= 0 && e == cudaSuccess; i--) {
        const Snap &st = c->rec_store[i];
        Dev ds = d;
        ds.pos = st.pos;
        ds.linmom = st.linmom;
        ds.vinfo = st.vinfo;
        ds.status = st.status;
        e = launch_collision(ds, c->stream);
        a.parity = (p0 + i) & 1;
        launch_adj_slots(d, st, a, c->stream);
        launch_adj_voxel_link(d, st, a, c->stream);
        launch_adj_contact(d, st, a, c->stream);
        launch_adj_gather_slots(d, st, nullptr, a, c->stream);
    }
    return e;
}

int adj_segment_graph(vx3g_ctx *c, const AdjBufs &a, int len, int p0, cudaGraphExec_t *out) {
    const long key = 2L * len + p0;
    for (auto &e : c->adj_graphs)
        if (e.first == key) {
            *out = e.second;
            return VX3G_OK;
        }
    cudaGraph_t g;
    CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t ce = enqueue_adj_segment(c, a, len, p0);
    const cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
    if (ce != cudaSuccess) {
        if (ee == cudaSuccess) cudaGraphDestroy(g);
        return fail(VX3G_ERR_CUDA, std::string("backward graph capture: ") + cudaGetErrorString(ce));
    }
    CU(ee);
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(VX3G_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    c->adj_graphs.push_back({key, ex});
    *out = ex;
    return VX3G_OK;
}

}  // namespace

extern "C" {

int vx3g_record(vx3g_ctx *c, int n, int k) {
    if (!c || n < 0 || k <= 0) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_record");
    if (c->precision != VX3G_PRECISION_FP64) return fail(VX3G_ERR_UNSUPPORTED, "the adjoint runs on FP64 contexts");
    if (c->ff_pos)
        return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of a force field that reads the voxel position is not implemented");
    if (c->any_cilia) return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of cilia forces is not implemented");
    if (c->any_nonlinear)
        return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of non-linear material models is not implemented");
    if (c->any_bcs) return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of boundary conditions is not implemented");
    if (c->any_signals) return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of signals is not implemented");
    if (c->any_attach) return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of attachment is not implemented");
    if (c->any_detach || c->any_remove)
        return fail(VX3G_ERR_UNSUPPORTED, "the adjoint of a changing link table (detach, removal) is not implemented");
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    c->free_record();
    const int nck = (n + k - 1) / k;
    int rc = alloc_snaps(c, c->rec_ck, nck);
    if (rc) {
        c->free_record();
        return rc;
    }
    const Dev &d = c->d;
    const Snap live = live_snap(d);
    c->rec_start = c->steps;
    c->rec_n = n;
    c->rec_k = k;
    for (int j = 0; j < nck; j++) {
        launch_snap_copy(c->rec_ck[j], live, d.nv, d.nl, d.nr, c->stream);
        rc = vx3g_step(c, std::min(k, n - j * k));
        if (rc) {
            c->free_record();
            return rc;
        }
    }
    CU(cudaGetLastError());
    return VX3G_OK;
}

int vx3g_backward(vx3g_ctx *c, const double *dL_dcom, double *dL_dphase, double *dL_dlog10E) {
    if (!c || !dL_dcom) return fail(VX3G_ERR_INVALID, "bad arguments to vx3g_backward");
    if (c->rec_start < 0 || c->steps != c->rec_start + c->rec_n)
        return fail(VX3G_ERR_INVALID, "no recorded run ends at the current state (call vx3g_record first)");
    CU(cudaSetDevice(c->device));
    const Dev &d = c->d;
    const size_t nv = d.nv, nl = d.nl, nr = d.nr;
    int rc;
    if (!c->adj_mem) {  // adjoint buffers, kept for later calls
        const size_t bytes = al256(13 * nv * 8) * 2 + al256(6 * nv * 8) + al256(nv * 8) * 4 + al256(9 * nl * 8) +
                             al256(54 * nv * 8) + al256(3 * nr * 8) + al256(nr * 8) + al256(3 * nv * 8) +
                             al256(8 * nv * 8);
        cudaError_t e = cudaMalloc(&c->adj_mem, bytes);
        if (e != cudaSuccess) {
            c->adj_mem = nullptr;
            return fail(VX3G_ERR_NOMEM, std::string("cudaMalloc (adjoint buffers): ") + cudaGetErrorString(e));
        }
        char *p = (char *)c->adj_mem;
        auto take = [&p](size_t n) {
            char *q = p;
            p += al256(n);
            return (double *)q;
        };
        AdjBufs &a = c->ab;
        a.lv = take(13 * nv * 8);
        a.lown = take(13 * nv * 8);
        a.lF = take(6 * nv * 8);
        a.lbs = take(nv * 8);
        a.lE = take(nv * 8);
        a.gphase = take(nv * 8);
        a.glogE = take(nv * 8);
        a.lloc = take(9 * nl * 8);
        a.aslot = take(54 * nv * 8);
        a.w = take(3 * nr * 8);
        a.mass_tot = take(nr * 8);
        a.lcon = take(3 * nv * 8);
        a.lcc = take(8 * nv * 8);
        CU(cudaMemsetAsync(a.lcon, 0, 3 * nv * 8, c->stream));
        CU(cudaMemsetAsync(a.lcc, 0, 8 * nv * 8, c->stream));  // stays zero off the collision surface
        CU(cudaMemcpyAsync((void *)a.mass_tot, c->mass_tot.data(), nr * 8, cudaMemcpyHostToDevice, c->stream));
    }
    const int n = c->rec_n, k = c->rec_k;
    const int store = std::min(n, k);
    if ((int)c->rec_store.size() < store || !c->rec_slots) {  // recompute store + the end state
        for (auto &g : c->adj_graphs) cudaGraphExecDestroy(g.second);
        c->adj_graphs.clear();
        c->rec_store.clear();
        std::vector<Snap> end;
        if ((rc = alloc_snaps(c, c->rec_store, store)) || (rc = alloc_snaps(c, end, 1))) return rc;
        c->rec_end = end[0];
        void *m = nullptr;
        cudaError_t e = cudaMalloc(&m, (36 + 4) * nv * sizeof(double));  // slots + contact forces
        if (e != cudaSuccess) return fail(VX3G_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        c->rec_mem.push_back(m);
        c->rec_slots = m;
    }
    AdjBufs a = c->ab;
    CU(cudaMemcpyAsync((void *)a.w, dL_dcom, 3 * nr * 8, cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemsetAsync(a.gphase, 0, nv * 8, c->stream));
    CU(cudaMemsetAsync(a.glogE, 0, nv * 8, c->stream));
    const Snap live = live_snap(d);
    launch_snap_copy(c->rec_end, live, d.nv, d.nl, d.nr, c->stream);
    CU(cudaMemcpyAsync(c->rec_slots, d.slots, 36 * nv * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync((double *)c->rec_slots + 36 * nv, d.contact, nv * sizeof(double4), cudaMemcpyDeviceToDevice,
                       c->stream));
    launch_adj_seed(d, a, c->stream);
    const int nck = (n + k - 1) / k;
    for (int j = nck - 1; j >= 0; j--) {
        const int len = std::min(k, n - j * k);
        const int p0 = (int)((c->rec_start + (int64_t)j * k) & 1);
        launch_snap_copy(live, c->rec_ck[j], d.nv, d.nl, d.nr, c->stream);
        cudaGraphExec_t g = nullptr;
        if ((rc = adj_segment_graph(c, a, len, p0, &g))) return rc;
        CU(cudaGraphLaunch(g, c->stream));
    }
    launch_snap_copy(live, c->rec_end, d.nv, d.nl, d.nr, c->stream);
    CU(cudaMemcpyAsync(d.slots, c->rec_slots, 36 * nv * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(d.contact, (double *)c->rec_slots + 36 * nv, nv * sizeof(double4), cudaMemcpyDeviceToDevice,
                       c->stream));
    if (dL_dphase) CU(cudaMemcpyAsync(dL_dphase, a.gphase, nv * 8, cudaMemcpyDeviceToHost, c->stream));
    if (dL_dlog10E) CU(cudaMemcpyAsync(dL_dlog10E, a.glogE, nv * 8, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaGetLastError());
    return VX3G_OK;
}

}  // extern "C"
