// Host build of the FP64 step and its adjoint (vx3g_step.cuh, vx3g_adjoint.cuh) for
// checking the adjoint's algebra against finite differences without a GPU.
//
// The forward here is the product's own link_update<double> / voxel_update<double>
// run as serial loops over a small fully filled body; material constants follow the
// reference's scaling with E (beam stiffnesses ~ E, damping constants ~ sqrt(E),
// floor stiffness 2*E*L).  Test infrastructure only; nothing here ships.
//
//   adjoint_check step  N nx ny nz amp   one-step VJP at the state after N steps,
//                                        random cotangent on every state component
//   adjoint_check param N nx ny nz amp floor   dCOM_x(N)/d(phase, log10E) vs central FD
// Prints one line per check class: "<name> <max relative error>" (error relative to
// |fd| + 1% of the class's largest |fd|).  Quaternions are stored {w,x,y,z}, the
// order of the adjoint's quaternion entries.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

static inline int atomicOr(int *a, int v) {
    const int o = *a;
    *a |= v;
    return o;
}
static inline float sinpif(float x) { return (float)std::sin(M_PI * (double)x); }
static uint3 blockIdx, threadIdx;
static dim3 blockDim;
#define __launch_bounds__(x)
#include "../../voxcraft-sim_gb300/csrc/vx3g_adjoint.cuh"

using namespace vx3g;

namespace {

const double kL = 0.01;  // voxel size

VMat voxel_material(double Ed) {
    const float E = (float)Ed, rho = 1e3f;
    const double vol = kL * kL * kL;
    VMat v{};
    const float mass = (float)(vol * rho), mom = (float)(mass * kL * kL / 6.0f);
    v.mass = mass;
    v.mass_inv = 1.0f / mass;
    v.mom_inv = 1.0f / mom;
    const float c2m = (float)(2.0f * std::sqrt((double)(mass * E) * kL));
    const float c2i = (float)(2.0f * std::sqrt((double)(mom * E) * kL * kL * kL));
    v.c_glob = 0.1f * c2m;
    v.c_glob_rot = 0.1f * c2i;
    v.c_col = 1.0f * c2m;
    v.grav_force = -mass * 9.80665f;
    v.pstiff = (float)(2 * E * kL);
    v.mu_s = 1.0f;
    v.mu_k = 0.5f;
    v.cte = 0.01f;
    v.dmc = 2 * sqrtf(mass) * 1.0f;
    v.E = E;
    v.nom_size = kL;
    v.is_measured = 1;
    return v;
}

LMat link_material(const VMat &a, const VMat &b) {
    LMat l{};
    const float E = 2.0f * a.E * b.E / (a.E + b.E), L = (float)kL;
    l.E = E;
    l.eps_fail = -1.0f;
    l.lin = 1;  // linear model: no stress-strain points
    l.eHat = E;
    l.a1 = E * L;
    l.a2 = E * L * L * L / 12.0f;
    l.b1 = E * L;
    l.b2 = E * L * L / 2.0f;
    l.b3 = E * L * L * L / 6.0f;
    l.sqA1 = sqrtf(l.a1);
    l.sqA2xIp = sqrtf(l.a2 * L * L / 6.0f);
    l.sqB1 = sqrtf(l.b1);
    l.sqB2xFMp = sqrtf(l.b2 * L / 2.0f);
    l.sqB3xIp = sqrtf(l.b3 * L * L / 6.0f);
    l.area = L * L;
    return l;
}

struct World {
    int nx, ny, nz, nv = 0, nl = 0, floor = 1;
    double amp = 39.0;
    std::vector<double4> pos, quat, lm, am, contact;
    std::vector<float> tempe;
    std::vector<double> phase, lstate, slots;
    std::vector<uint2> vinfo, linfo;
    std::vector<int2> ends;
    std::vector<float2> strain;
    std::vector<VMat> vm;
    std::vector<LMat> lmt;
    RobotP rp{};
    float dt = 0;
    double T[2] = {0, 0};
    int status = 0;
    Dev d{};

    void build(const std::vector<double> &ph, const std::vector<double> &le, float dtf) {
        nv = nx * ny * nz;
        phase = ph;
        pos.clear(); quat.clear(); vinfo.clear(); linfo.clear(); ends.clear(); vm.clear(); lmt.clear();
        for (int i = 0; i < nv; i++) {
            const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
            pos.push_back(make_double4(x * kL, y * kL, z * kL, 0));
            quat.push_back(make_double4(1, 0, 0, 0));
            vm.push_back(voxel_material(std::pow(10.0, le[i])));
            vinfo.push_back(make_uint2(0, VF_STATIC | ((uint32_t)i << 8)));
            const int nb[3] = {x > 0 ? i - 1 : -1, y > 0 ? i - nx : -1, z > 0 ? i - nx * ny : -1};
            for (int a = 0; a < 3; a++) {
                if (nb[a] < 0) continue;
                lmt.push_back(link_material(vm[i], vm[nb[a]]));
                ends.push_back(make_int2(nb[a], i));
                linfo.push_back(make_uint2(0, (uint32_t)a | LF_SMALL | ((uint32_t)(lmt.size() - 1) << 8)));
                vinfo[nb[a]].y |= 1u << (2 * a);
                vinfo[i].y |= 1u << (2 * a + 1);
            }
        }
        nl = (int)ends.size();
        lm.assign(nv, make_double4(0, 0, 0, 0));
        am = lm;
        contact = lm;
        tempe.assign(2 * nv, 0.0f);
        lstate.assign(9 * (size_t)nl, 0.0);
        slots.assign(36 * (size_t)nv, 0.0);
        strain.assign(nl, make_float2(0, 0));
        rp = RobotP{};
        rp.vox_size = kL; rp.temp_amp = amp; rp.temp_period = 0.2; rp.inv_period = 5.0; rp.dt_frac = 0.9;
        rp.nv = nv; rp.nl = nl; rp.floor = floor; rp.vary_temp = 1;
        dt = dtf;
        T[0] = T[1] = 0;
        status = 0;
        d = Dev{};
        d.pos = pos.data(); d.quat = quat.data(); d.linmom = lm.data(); d.angmom = am.data();
        d.contact = contact.data(); d.tempe = tempe.data(); d.phase = phase.data(); d.vinfo = vinfo.data();
        d.ends = ends.data(); d.linfo = linfo.data(); d.lstate = lstate.data(); d.strain = strain.data();
        d.slots = slots.data(); d.rp = &rp; d.dt = &dt; d.T = T; d.status = &status; d.vmat = vm.data();
        d.lmat = lmt.data(); d.nv = nv; d.nl = nl; d.nr = 1;
        for (int v = 0; v < nv; v++) {  // initial temperature (k_init_temperature)
            float te = tempe[v];
            double bs = vm[v].nom_size * (1 + te * vm[v].cte);
            bs = temperature_base_size<true>(rp, vm[v], phase[v], 0.0, bs, &te);
            pos[v].w = bs;
            tempe[v] = tempe[nv + v] = te;
        }
    }
    void step(long k) {
        for (int l = 0; l < nl; l++) link_update<double>(d, l);
        for (int v = 0; v < nv; v++) voxel_update<double>(d, v, (int)(k & 1));
    }
    double com_x() const {
        double sx = 0, sm = 0;
        for (int v = 0; v < nv; v++) { sx += vm[v].mass * pos[v].x; sm += vm[v].mass; }
        return sx / sm;
    }
};

// a stored state (what the checkpoints hold)
struct Stored {
    std::vector<double4> pos, quat, lm, am;
    std::vector<uint2> vinfo, linfo;
    std::vector<float> tempe;
    std::vector<double> lstate;
    std::vector<float2> strain;
    double T[2];
    int status;
    Snap s;
    void take(const World &w) {
        pos = w.pos; quat = w.quat; lm = w.lm; am = w.am; vinfo = w.vinfo; linfo = w.linfo; tempe = w.tempe;
        lstate = w.lstate; strain = w.strain; T[0] = w.T[0]; T[1] = w.T[1]; status = w.status;
        s = Snap{pos.data(), quat.data(), lm.data(), am.data(), vinfo.data(), tempe.data(), lstate.data(),
                 strain.data(), linfo.data(), T, &status};
    }
    void put(World &w) const {
        w.pos = pos; w.quat = quat; w.lm = lm; w.am = am; w.vinfo = vinfo; w.linfo = linfo; w.tempe = tempe;
        w.lstate = lstate; w.strain = strain; w.T[0] = T[0]; w.T[1] = T[1]; w.status = status;
        w.d.pos = w.pos.data(); w.d.quat = w.quat.data(); w.d.linmom = w.lm.data(); w.d.angmom = w.am.data();
        w.d.vinfo = w.vinfo.data(); w.d.linfo = w.linfo.data(); w.d.tempe = w.tempe.data();
        w.d.lstate = w.lstate.data(); w.d.strain = w.strain.data();
    }
};

struct Adj {
    std::vector<double> lv, lown, lF, lbs, lE, lloc, aslot, gph, gle, lcon, lcc, w, mt;
    AdjBufs a{};
    Adj(int nv, int nl) : lv(13 * nv), lown(13 * nv), lF(6 * nv), lbs(nv), lE(nv), lloc(9 * nl), aslot(54 * nv),
                          gph(nv), gle(nv), lcon(3 * nv), lcc(8 * nv), w{1, 0, 0}, mt{0} {
        a = AdjBufs{};
        a.lv = lv.data(); a.lown = lown.data(); a.lF = lF.data(); a.lbs = lbs.data(); a.lE = lE.data();
        a.lloc = lloc.data(); a.aslot = aslot.data(); a.gphase = gph.data(); a.glogE = gle.data();
        a.lcon = lcon.data(); a.lcc = lcc.data(); a.w = w.data(); a.mass_tot = mt.data(); a.parity = 0;
    }
    void reverse_step(const World &w, const Snap &s, int parity) {
        a.parity = parity;
        for (int l = 0; l < w.nl; l++) adj::adj_link_slots(w.d, s, a, l);
        for (int v = 0; v < w.nv; v++) adj::adj_voxel(w.d, s, a, v);
        for (int l = 0; l < w.nl; l++) adj::adj_link(w.d, s, a, l);
        for (int v = 0; v < w.nv; v++) adj::adj_gather(w.d, s, a, v);
    }
};

double state_value(const World &w, int v, int i) {
    if (i < 3) return (&w.pos[v].x)[i];
    if (i < 7) return (&w.quat[v].x)[i - 3];
    if (i < 10) return (&w.lm[v].x)[i - 7];
    return (&w.am[v].x)[i - 10];
}
double *state_ref(World &w, int v, int i) {
    if (i < 3) return &w.pos[v].x + i;
    if (i < 7) return &w.quat[v].x + (i - 3);
    if (i < 10) return &w.lm[v].x + (i - 7);
    return &w.am[v].x + (i - 10);
}

float stable_dt(const std::vector<double> &le) {
    double emax = 0;
    for (double x : le) emax = std::fmax(emax, std::pow(10.0, x));
    return (float)(0.9 / (6.283185307179586 * std::sqrt(emax * kL / (1e3 * kL * kL * kL))));
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 7) {
        fprintf(stderr, "usage: adjoint_check step|param N nx ny nz amp [floor]\n");
        return 2;
    }
    const bool param = std::string(argv[1]) == "param";
    const int N = atoi(argv[2]);
    World w;
    w.nx = atoi(argv[3]); w.ny = atoi(argv[4]); w.nz = atoi(argv[5]);
    w.amp = atof(argv[6]);
    w.floor = argc > 7 ? atoi(argv[7]) : 1;
    const int nv = w.nx * w.ny * w.nz;
    std::mt19937_64 rng(1);
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<double> ph(nv), le(nv);
    for (int i = 0; i < nv; i++) {
        ph[i] = (double)(float)U(rng);
        le[i] = (double)(float)(5 + 2 * U(rng));
    }
    const float dt = stable_dt(le);
    w.build(ph, le, dt);
    const int nl = w.nl;
    if (!param) {
        for (int k = 0; k < N; k++) w.step(k);
        Stored base;
        base.take(w);
        std::mt19937_64 r2(7);
        std::normal_distribution<double> G(0, 1);
        std::vector<double> lam(13 * nv), laml(9 * nl);
        for (auto &x : lam) x = G(r2);
        for (auto &x : laml) x = 1e-2 * G(r2);
        auto J = [&](const World &ww) {
            double acc = 0;
            for (int v = 0; v < nv; v++)
                for (int i = 0; i < 13; i++) acc += lam[13 * v + i] * state_value(ww, v, i);
            for (int l = 0; l < nl; l++)
                for (int k = 0; k < 9; k++) acc += laml[9 * l + k] * ww.lstate[(size_t)k * nl + l];
            return acc;
        };
        Adj A(nv, nl);
        A.lv = lam;
        A.lloc = laml;
        A.a.lv = A.lv.data();
        A.a.lloc = A.lloc.data();
        A.reverse_step(w, base.s, N & 1);
        // finite-difference steps per component class (positions, quaternions, momenta)
        const double hs[4] = {1e-9, 1e-8, 1e-10, 1e-14};
        const char *names[4] = {"pos", "quat", "linmom", "angmom"};
        double worst[5] = {0, 0, 0, 0, 0}, scale[5] = {0, 0, 0, 0, 0};
        std::vector<double> fdv(13 * nv), fdl(9 * nl);
        for (int v = 0; v < nv; v++)
            for (int i = 0; i < 13; i++) {
                const int cls = i < 3 ? 0 : (i < 7 ? 1 : (i < 10 ? 2 : 3));
                double f[2];
                for (int sg = 0; sg < 2; sg++) {
                    base.put(w);
                    *state_ref(w, v, i) += sg ? -hs[cls] : hs[cls];
                    w.step(N);
                    f[sg] = J(w);
                }
                fdv[13 * v + i] = (f[0] - f[1]) / (2 * hs[cls]);
                scale[cls] = std::fmax(scale[cls], std::fabs(fdv[13 * v + i]));
            }
        for (int l = 0; l < nl; l++)
            for (int k = 0; k < 9; k++) {
                double f[2];
                for (int sg = 0; sg < 2; sg++) {
                    base.put(w);
                    w.lstate[(size_t)k * nl + l] += sg ? -1e-9 : 1e-9;
                    w.step(N);
                    f[sg] = J(w);
                }
                fdl[9 * l + k] = (f[0] - f[1]) / 2e-9;
                scale[4] = std::fmax(scale[4], std::fabs(fdl[9 * l + k]));
            }
        for (int v = 0; v < nv; v++)
            for (int i = 0; i < 13; i++) {
                const int cls = i < 3 ? 0 : (i < 7 ? 1 : (i < 10 ? 2 : 3));
                const double e = std::fabs(A.lv[13 * v + i] - fdv[13 * v + i]) /
                                 (std::fabs(fdv[13 * v + i]) + 1e-2 * scale[cls]);
                worst[cls] = std::fmax(worst[cls], e);
            }
        for (size_t i = 0; i < fdl.size(); i++)
            worst[4] = std::fmax(worst[4], std::fabs(A.lloc[i] - fdl[i]) / (std::fabs(fdl[i]) + 1e-2 * scale[4]));
        for (int c = 0; c < 4; c++) printf("%s %.3e\n", names[c], worst[c]);
        printf("link_state %.3e\n", worst[4]);
        return 0;
    }
    // parameter gradient over N steps
    std::vector<Stored> st(N);
    const double c0 = w.com_x();
    for (int k = 0; k < N; k++) {
        st[k].take(w);
        w.step(k);
    }
    Adj A(nv, nl);
    for (int v = 0; v < nv; v++) A.mt[0] += w.vm[v].mass;
    for (int v = 0; v < nv; v++) adj::adj_seed(w.d, A.a, v);
    for (int l = 0; l < 9 * nl; l++) A.lloc[l] = 0;
    for (int k = N - 1; k >= 0; k--) A.reverse_step(w, st[k].s, k & 1);
    auto loss = [&](const std::vector<double> &p, const std::vector<double> &e) {
        World u;
        u.nx = w.nx; u.ny = w.ny; u.nz = w.nz; u.amp = w.amp; u.floor = w.floor;
        u.build(p, e, dt);
        for (int k = 0; k < N; k++) u.step(k);
        return u.com_x() - c0;
    };
    const double eps = 1e-4;
    double worst_p = 0, worst_e = 0, sp = 0, se = 0;
    std::vector<double> fp(nv), fe(nv);
    for (int v = 0; v < nv; v++) {
        std::vector<double> p1 = ph, p2 = ph, e1 = le, e2 = le;
        p1[v] += eps; p2[v] -= eps; e1[v] += eps; e2[v] -= eps;
        fp[v] = (loss(p1, le) - loss(p2, le)) / (2 * eps);
        fe[v] = (loss(ph, e1) - loss(ph, e2)) / (2 * eps);
        sp = std::fmax(sp, std::fabs(fp[v]));
        se = std::fmax(se, std::fabs(fe[v]));
    }
    for (int v = 0; v < nv; v++) {
        worst_p = std::fmax(worst_p, std::fabs(A.gph[v] - fp[v]) / (std::fabs(fp[v]) + 1e-2 * sp));
        worst_e = std::fmax(worst_e, std::fabs(A.gle[v] - fe[v]) / (std::fabs(fe[v]) + 1e-2 * se));
    }
    printf("phase %.3e\nlog10E %.3e\n", worst_p, worst_e);
    return 0;
}
