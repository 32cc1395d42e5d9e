// vx3g_aux.cu -- set-up and per-step passes other than the link/voxel passes:
// initial temperature, stable time step, surface-voxel collision, centre of mass.
// FP64 arithmetic throughout, compiled with --fmad=false.
#include <mutex>

#include "vx3g_step.cuh"

namespace vx3g {

// ---------------------------------------------------------------- temperature at t = 0
// The reference's first doTimeStep updates temperatures before anything else
// (VX3_VoxelyzeKernel.cu:240, :625-650); the base size of every voxel for step 0
// follows from that update (or from the initial temperature where it is skipped).
template <bool EXACT> __global__ void k_init_temperature(Dev d) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d.nv) return;
    const uint2 vi = d.vinfo[v];
    const VMat m = d.vmat[vi.y >> 8];
    const RobotP &rp = d.rp[vi.x];
    float te = d.tempe[v];
    double bs = m.nom_size * (1 + te * m.cte);
    bs = temperature_base_size<EXACT>(rp, m, d.phase[v], 0.0, bs, &te);
    d.pos[v].w = bs;
    d.tempe[v] = te;              // parity-0 buffer: the temperature step 0 uses
    d.tempe[d.nv + v] = te;       // parity-1 buffer: unchanged for robots without actuation
}

void launch_init_temperature(const Dev &d, int mixed, cudaStream_t s) {
    if (!d.nv) return;
    if (mixed) launch_init_temperature_mixed(d, s);
    else k_init_temperature<true><<<(d.nv + 255) / 256, 256, 0, s>>>(d);
}

// ---------------------------------------------------------------- stable time step
// recommendedTimeStep (VX3_VoxelyzeKernel.cu:184-217) with VX3_Link::axialStiffness
// (VX3_Link.cu:269-278): max over links of k/min(m1,m2), as a per-robot max of the
// non-negative doubles' bit patterns (order independent, so deterministic).
__global__ void k_dt_links(Dev d, unsigned long long *mx) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= d.nl) return;
    const uint2 li = d.linfo[l];
    if (li.y & LF_RUNTIME) return;  // the reference's loop covers the lattice's links (d_links) only
    const LMat &m = d.lmat[li.y >> 8];
    const int2 e = d.ends[l];
    const double m1 = d.vmat[d.vinfo[e.x].y >> 8].mass, m2 = d.vmat[d.vinfo[e.y].y >> 8].mass;
    float k;
    if (m.nu == 0.0f) {
        k = m.a1;
    } else {
        const double rest = 0.5 * (load_state(d, d.pos, e.x).w + load_state(d, d.pos, e.y).w);
        k = (float)(m.eHat * m.area / ((d.strain[l].x + 1) * rest));
    }
    const double f2 = k / (m1 < m2 ? m1 : m2);
    if (f2 > 0) atomicMax(&mx[2 * li.x], (unsigned long long)__double_as_longlong(f2));
}

__global__ void k_dt_voxels(Dev d, unsigned long long *mx) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d.nv) return;
    const uint2 vi = d.vinfo[v];
    const VMat &m = d.vmat[vi.y >> 8];
    const double f2 = m.E * m.nom_size / m.mass;
    if (f2 > 0) atomicMax(&mx[2 * vi.x + 1], (unsigned long long)__double_as_longlong(f2));
}

__global__ void k_dt_final(Dev d, const unsigned long long *mx) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= d.nr) return;
    double f2 = __longlong_as_double((long long)mx[2 * r]);
    if (f2 <= 0.0f) f2 = __longlong_as_double((long long)mx[2 * r + 1]);
    double opt = (f2 <= 0.0f) ? 0.0f : 1.0f / (6.283185f * sqrt(f2));
    if (opt < 1e-10) opt = 1e-10;  // doTimeStep (VX3_VoxelyzeKernel.cu:248-252)
    d.dt[r] = (float)(d.rp[r].dt_frac * opt);
}

void launch_dt(const Dev &d, double *scratch, cudaStream_t s) {
    unsigned long long *mx = (unsigned long long *)scratch;
    cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * 2 * d.nr, s);
    if (d.nl) k_dt_links<<<(d.nl + 255) / 256, 256, 0, s>>>(d, mx);
    if (d.nv) k_dt_voxels<<<(d.nv + 255) / 256, 256, 0, s>>>(d, mx);
    k_dt_final<<<(d.nr + 255) / 256, 256, 0, s>>>(d, mx);
}

// ---------------------------------------------------------------- stable time step, no allocation
// vx3g_recommended_dt_noalloc computes recommendedTimeStep for every robot with its
// reduction scratch in device memory reserved when the module loads, not in memory
// the context or the call allocates: 2 per-robot maxima (link and voxel terms) and
// the per-robot result, for at most kNoAllocMaxRobots robots (96 KB).
constexpr int kNoAllocMaxRobots = 4096;
static __device__ __align__(256) unsigned long long g_dt_noalloc[3 * kNoAllocMaxRobots];

// recommendedTimeStep from the maxima (VX3_VoxelyzeKernel.cu:184-217), without DtFrac
__global__ void k_dt_recommended(int nr, const unsigned long long *mx, double *out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    double f2 = __longlong_as_double((long long)mx[2 * r]);
    if (f2 <= 0.0f) f2 = __longlong_as_double((long long)mx[2 * r + 1]);
    out[r] = (f2 <= 0.0f) ? 0.0f : 1.0f / (6.283185f * sqrt(f2));
}

int recommended_dt_noalloc(const Dev &d, int device, double *out_host, cudaStream_t s, const char **why) {
    if (d.nr > kNoAllocMaxRobots) {
        *why = "vx3g_recommended_dt_noalloc: at most 4096 robots per context";
        return -1;
    }
    // the scratch address, looked up once per device (with that device current)
    static std::mutex lock;
    static void *addr[64] = {};
    if (device < 0 || device >= 64) {
        *why = "vx3g_recommended_dt_noalloc: device ordinal out of range";
        return -1;
    }
    void *base;
    {
        std::lock_guard<std::mutex> g(lock);
        if (!addr[device]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_dt_noalloc) != cudaSuccess) {
                *why = "vx3g_recommended_dt_noalloc: cudaGetSymbolAddress failed";
                return -3;
            }
            addr[device] = p;
        }
        base = addr[device];
    }
    unsigned long long *mx = (unsigned long long *)base;  // 2*nr maxima: must start at zero
    double *res = (double *)(mx + 2 * kNoAllocMaxRobots);
    if (cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * 2 * d.nr, s) != cudaSuccess) {
        *why = "vx3g_recommended_dt_noalloc: cudaMemsetAsync failed";
        return -3;
    }
    if (d.nl) k_dt_links<<<(d.nl + 255) / 256, 256, 0, s>>>(d, mx);
    if (d.nv) k_dt_voxels<<<(d.nv + 255) / 256, 256, 0, s>>>(d, mx);
    if (d.nr) k_dt_recommended<<<(d.nr + 255) / 256, 256, 0, s>>>(d.nr, mx, res);
    if (cudaMemcpyAsync(out_host, res, sizeof(double) * d.nr, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        *why = "vx3g_recommended_dt_noalloc: CUDA error";
        return -3;
    }
    return 0;
}

// ---------------------------------------------------------------- force field and cilia
// VX3_Voxel::timeStep adds the three force-field programs evaluated at the voxel's
// position and the current time (VX3_Voxel.cu:178-184), and force() adds
// CiliaForce * Cilia (:376), CiliaForce being set for surface voxels by
// gpu_update_cilia_force (VX3_VoxelyzeKernel.cu:846-859) as R(orient) (base + signal
// * shift), the signal staying 0 here.  Both are evaluated in FP64 before the voxel
// pass and the step's detach (from the position, orientation and time the step starts
// with), so the voxel kernels only add the stored forces at the reference's places in
// the sum.
__global__ void k_extra_forces(Dev d, int parity) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d.nv) return;
    const int r = (int)d.vinfo[v].x;
    const RobotP &rp = d.rp[r];
    if (!rp.ff_any && !rp.cilia) return;
    const double t = d.T[(size_t)parity * d.nr + r];
    if (rp.cilia) {
        const double4 c = d.cil[v];
        V3<double> cf{0, 0, 0};
        // surface voxels only; a voxel joins the surface once it has lost a link (detach,
        // removal of a neighbour) -- this kernel runs before the step's detach, so with the
        // link table the reference regenerated its surface list from
        const bool surface = (d.vinfo[v].y & VF_LINKMASK) != VF_LINKMASK;
        if (surface && !(d.cil_on[v] > t)) {
            const double4 q = load_state(d, d.quat, v);
            V3<double> b{c.x, c.y, c.z};  // baseCiliaForce + localSignal * shiftCiliaForce
            if (rp.signals) {
                const double sl = d.sig[6 * (size_t)v];
                const double4 sh = d.cils[v];
                b = V3<double>{c.x + sl * sh.x, c.y + sl * sh.y, c.z + sl * sh.z};
            }
            cf = qrot(Q4<double>{q.x, q.y, q.z, q.w}, b);
        }
        d.cfv[v] = make_double4(cf.x * c.w, cf.y * c.w, cf.z * c.w, 0.0);
    }
    if (rp.ff_any) {
        const double4 p = load_state(d, d.pos, v);
        const V3<double> f = force_field(d, rp, p.x, p.y, p.z, t);
        d.ffv[v] = make_double4(f.x, f.y, f.z, 0.0);
    }
}

void launch_extra_forces(const Dev &d, int parity, cudaStream_t s) {
    if ((d.ffv || d.cfv) && d.nv) k_extra_forces<<<(d.nv + 255) / 256, 256, 0, s>>>(d, parity);
}

// ---------------------------------------------------------------- signals
// The end of VX3_Voxel::timeStep with EnableSignals (VX3_Voxel.cu:271-348): propagateSignal
// (the pending signal, once due, passed to the voxel across each link in direction order,
// each receiver taking it unless refractory), packMaker, localSignalDecay.  A voxel writes
// its neighbours' signal state, so the voxels of a robot take their turns in voxel order, as
// a serial loop over the voxel pass does: one warp per robot walks its voxels 32 at a time;
// a group in which no voxel passes a signal on touches only each voxel's own state and runs
// in parallel, a group with one runs voxel by voxel on lane 0.  The physics of the step does
// not read signal state, so this runs after the voxel pass.
__device__ __forceinline__ void sig_receive(const Dev &d, int v, double value, double at, bool force) {
    double *S = d.sig + 6 * (size_t)v;
    const VMat &m = d.vmat[d.vinfo[v].y >> 8];
    if (!force && S[3] > at) return;
    if (value < 0.1) return;
    S[3] = at + m.inactive;  // inactiveUntil
    S[0] = value;            // localSignal
    double sv = value * m.sig_decay;
    if (sv < 0.1) sv = 0;
    S[4] = sv;
    S[5] = at;
}

// the voxel reached the end of timeStep this step (stepped, not fixed in all DOFs)
__device__ __forceinline__ bool sig_turn(const Dev &d, const RobotP &rp, int v) {
    if (d.vinfo[v].y & VF_FIXED) return false;  // material Fixed, or removed
    if (rp.bcs && d.vext[v] >= 0 && d.ext[d.vext[v]].dof == EXT_ALL) return false;
    return true;
}

__device__ __forceinline__ bool sig_sends(const Dev &d, int v, double t) {
    const double *S = d.sig + 6 * (size_t)v;
    return !(S[5] > t) && !(S[4] < 0.1);
}

__device__ void sig_own(const Dev &d, int v, double t) {  // packMaker, localSignalDecay
    double *S = d.sig + 6 * (size_t)v;
    const VMat &m = d.vmat[d.vinfo[v].y >> 8];
    if (m.pacemaker && !(S[2] > t)) {
        sig_receive(d, v, 100, t, true);
        S[2] = t + m.pace_period;
    }
    if (!(S[1] > t)) {
        if (S[0] < 0.1) S[0] = 0;
        else {
            S[0] = S[0] * 0.9;
            S[1] = t + 0.01;
        }
    }
}

__device__ void sig_send(const Dev &d, int v, double t) {  // propagateSignal
    double *S = d.sig + 6 * (size_t)v;
    const uint2 vi = d.vinfo[v];
    const VMat &m = d.vmat[vi.y >> 8];
    for (int dir = 0; dir < 6; dir++) {
        const int u = d.vnb[6 * (size_t)v + dir];
        if (u >= 0 && ((vi.y >> dir) & 1u)) sig_receive(d, u, S[4], t + m.sig_delay, false);
    }
    S[4] = 0;
    S[5] = 0;
    S[3] = t + 2 * m.sig_delay + m.inactive;
}

__global__ void k_signals(Dev d, int parity) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= d.nsigrob) return;
    const int r = d.sigrob[w];
    const RobotP &rp = d.rp[r];
    if (d.status[r] != 0 || d.dt[r] == 0.0f) return;
    const double t = d.T[(size_t)parity * d.nr + r];
    const int end = rp.voff + rp.nv;
    for (int base = rp.voff; base < end; base += 32) {
        const int v = base + lane;
        const bool mine = v < end && sig_turn(d, rp, v);
        const unsigned sends = __ballot_sync(0xffffffffu, mine && sig_sends(d, v, t));
        if (!sends) {
            if (mine) sig_own(d, v, t);
        } else if (lane == 0) {
            for (int u = base; u < min(base + 32, end); u++) {
                if (!sig_turn(d, rp, u)) continue;
                if (sig_sends(d, u, t)) sig_send(d, u, t);
                sig_own(d, u, t);
            }
        }
        __syncwarp();
    }
}

void launch_signals(const Dev &d, int parity, cudaStream_t s) {
    if (d.nsigrob) k_signals<<<(d.nsigrob + 3) / 4, 128, 0, s>>>(d, parity);
}

// ---------------------------------------------------------------- detach
// gpu_update_detach (VX3_VoxelyzeKernel.cu:946-967), after the collision pass: a link
// that has failed (VX3_Link::isFailed, maxStrain past the failure strain, VX3_Link.cu:78)
// leaves the link tables of both voxels; the robot's surface, and so its contact
// candidate lists, change from the next step on (regenerateSurfaceVoxels, :283-286).
__global__ void k_detach(Dev d) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= d.nl) return;
    const uint2 li = d.linfo[l];
    const int r = (int)li.x;
    if (!d.rp[r].detach || d.status[r] != 0) return;
    const uint32_t fl = li.y;
    if (fl & LF_GONE) return;
    const LMat &m = d.lmat[fl >> 8];
    if (!(m.eps_fail != -1.0f && d.strain[l].y > m.eps_fail)) return;
    d.linfo[l].y = fl | LF_GONE;
    const int a = (int)(fl & LF_AXIS);
    const int2 e = d.ends[l];
    atomicAnd(&d.vinfo[e.x].y, ~(1u << (2 * a)));      // the negative end's link toward +axis
    atomicAnd(&d.vinfo[e.y].y, ~(1u << (2 * a + 1)));  // the positive end's link toward -axis
    d.srf[r] = 1;
}

void launch_detach(const Dev &d, cudaStream_t s) {
    if (d.any_detach && d.nl) k_detach<<<(d.nl + 255) / 256, 256, 0, s>>>(d);
}

// ---------------------------------------------------------------- material removal
// removeVoxels (VX3_VoxelyzeKernel.cu:365-397), at the end of a SecondaryExperiment step
// (:335-349): once the step's start time is past a material's
// RemoveFromSimulationAfterThisManySeconds (> 0), each voxel of it leaves the simulation.
// It no longer steps (VF_FIXED: the voxel pass skips it, as gpu_update_voxels skips a
// removed voxel, :586), keeps the temperature of the step just taken (gpu_update_temperature
// skips it, :632), still counts toward the centre of mass (:477-493), and every link of it
// leaves the lattice (LF_GONE, the direction bits of both ends cleared).  Its robot's
// contact lists are rebuilt in the next step without it.  Whether a voxel leaves in this
// step depends on its own time test only, so link threads and voxel threads need no
// ordering among themselves.
__device__ __forceinline__ bool removed_by(const Dev &d, int v, int parity) {
    const int r = (int)d.vinfo[v].x;
    return d.status[r] == 0 && d.rm_at[v] < d.T[(size_t)parity * d.nr + r];
}

__global__ void k_remove(Dev d, int parity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.nl) {
        const uint2 li = d.linfo[i];
        if (d.rp[li.x].remove && !(li.y & LF_GONE)) {
            const int2 e = d.ends[i];
            if (removed_by(d, e.x, parity) || removed_by(d, e.y, parity)) {
                d.linfo[i].y = li.y | LF_GONE;
                const int a = (int)(li.y & LF_AXIS);
                atomicAnd(&d.vinfo[e.x].y, ~(1u << (2 * a)));      // the negative end's link toward +axis
                atomicAnd(&d.vinfo[e.y].y, ~(1u << (2 * a + 1)));  // the positive end's toward -axis
            }
        }
    }
    if (i < d.nv && !d.vgone[i] && removed_by(d, i, parity)) {
        d.vgone[i] = 1;
        atomicOr(&d.vinfo[i].y, VF_FIXED);
        d.tempe[(size_t)(parity ^ 1) * d.nv + i] = d.tempe[(size_t)parity * d.nv + i];
        d.srf[d.vinfo[i].x] = 1;
    }
}

void launch_remove(const Dev &d, int parity, cudaStream_t s) {
    const int n = d.nv > d.nl ? d.nv : d.nl;
    if (d.any_remove && n) k_remove<<<(n + 255) / 256, 256, 0, s>>>(d, parity);
}

// ---------------------------------------------------------------- collision
// The reference tests every pair of surface voxels each step (gpu_update_attach,
// VX3_VoxelyzeKernel.cu:833-843).  Here each surface voxel keeps a list of the
// surface voxels of its robot that were within cutoff + skin when the list was
// built (a Verlet list over a uniform grid of cell edge cutoff + skin).  A robot's
// lists are rebuilt in a step where any of its voxels has moved more than half the
// skin since its last build (robots never collide with each other, so the others
// keep theirs); every pair within the cutoff is therefore listed.  Robots of up to
// kLocalListMax collision-surface voxels build their lists in shared memory, one
// CTA per chunk of the robot (coll_list_robots, from a work list of the robots
// due); larger ones use one hashed grid in global memory with a counting sort
// (coll_bin .. coll_list).  The check and the rebuild run in one cooperative kernel
// (k_coll_prepare).  Each step the reference's exact test
// (handle_collision_attachment, :682-704) runs on the listed pairs and the contact
// forces of VX3_Collision (VX3_Collision.cu:3-31) are summed in ascending partner
// order -- the order in which the reference's serial pair loop accumulates them --
// without atomics.  A list may hold pairs that are out of reach; they add nothing,
// so the forces are the reference's, pair for pair, whichever path built the list.
__device__ __forceinline__ unsigned cell_hash(int cx, int cy, int cz, int r, int hmask) {
    unsigned h = (unsigned)cx * 73856093u ^ (unsigned)cy * 19349663u ^ (unsigned)cz * 83492791u ^ (unsigned)r * 2654435761u;
    h ^= h >> 15;
    h *= 0x2c1b3c6du;
    h ^= h >> 12;
    return h & (unsigned)hmask;
}

__device__ __forceinline__ float4 pos_f(const Dev &d, int v) {
    if (d.mixed) {
        const float4 *f = reinterpret_cast<const float4 *>(d.pos) + 2 * (size_t)v;
        const float4 h = f[0], l = f[1];
        return make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
    }
    const double4 p = d.pos[v];
    return make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
}

// robot r's lists are rebuilt this step; the first voxel to say so puts a robot of the
// shared-memory path on the work list of coll_list_robots
__device__ __forceinline__ void flag_robot(const Dev &d, int r) {
    if (*(volatile int *)&d.cflag[1 + r]) return;
    if (atomicOr(&d.cflag[1 + r], 1) != 0) return;
    atomicOr(d.cflag, 1);
    const int k = d.rp[r].lchunks;
    if (k) {
        const unsigned long long old = atomicAdd(d.lwork_ctr, (1ull << 32) | (unsigned long long)k);
        if ((old >> 32) < (unsigned long long)d.nr) d.lwork[old >> 32] = make_int2(r, (int)(old & 0xffffffffull));
    }
}

// 1. has surface voxel s moved more than half the skin since its robot's last build?
__device__ __forceinline__ void coll_check(const Dev &d, int s) {
    const int v = d.csurf[s];
    const float4 p = pos_f(d, v), q = d.cref[s];  // q.w: squared displacement limit
    d.cposf[s] = p;  // the positions a rebuild on the shared-memory path lists from
    if (d.crec) {  // mixed precision: this step's contact record of the voxel (k_coll_eval_mixed)
        const float4 *P = reinterpret_cast<const float4 *>(d.pos) + 2 * (size_t)v;
        const float4 h = P[0], l = P[1];
        const float4 lm = reinterpret_cast<const float4 *>(d.linmom)[2 * (size_t)v];
        const VMat &m = d.vmat[d.vinfo[v].y >> 8];
        float4 *R = d.crec + 2 * (size_t)v;
        R[0] = make_float4(h.x, h.y, h.z, h.w + l.w);
        R[1] = make_float4(l.x, l.y, l.z, m.pstiff);
        d.crec[2 * (size_t)d.nv + v] = make_float4(lm.x * m.mass_inv, lm.y * m.mass_inv, lm.z * m.mass_inv, m.c_col);
    }
    if (d.any_dyn) {  // robots whose surface follows their link table
        const uint2 vi = d.vinfo[v];
        const RobotP &rp = d.rp[vi.x];
        if (rp.dyn && s == rp.soff && d.srf[vi.x]) {  // a link or a voxel left last step: new surface
            d.srf[vi.x] = 0;
            flag_robot(d, (int)vi.x);
        }
        // interior or removed: not a surface voxel now
        if ((vi.y & VF_LINKMASK) == VF_LINKMASK || (d.vgone && d.vgone[v])) return;
    }
    const float ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
    if (ex * ex + ey * ey + ez * ez > q.w) flag_robot(d, (int)d.vinfo[v].x);
}

// exclusive scan of the inclusive-to-be value x over the kLocalListThreads threads of
// the block; returns the exclusive prefix, *total the block's sum (wsum: NW ints)
__device__ __forceinline__ int block_scan(int x, int *wsum, int *total) {
    constexpr int NW = kLocalListThreads / 32;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    int y = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += t;
    }
    __syncthreads();  // wsum is free
    if (lane == 31) wsum[wp] = y;
    __syncthreads();
    if (wp == 0) {
        int t = lane < NW ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += u;
        }
        if (lane < NW) wsum[lane] = t;
    }
    __syncthreads();
    *total = wsum[NW - 1];
    return y - x + (wp ? wsum[wp - 1] : 0);
}

// exclusive scan of hcount segment b (1024 buckets; hsize is a multiple of 1024), two
// buckets per thread; the segment's sum goes to hblock[b]
__device__ __forceinline__ void coll_scan_segment(const Dev &d, int b, int *wsum) {
    const int i = b * 1024 + 2 * (int)threadIdx.x;
    const int x0 = d.hcount[i], x1 = d.hcount[i + 1];
    int total;
    const int e = block_scan(x0 + x1, wsum, &total);
    d.hstart[i] = e;
    d.hstart[i + 1] = e + x0;
    if (threadIdx.x == 0) d.hblock[b] = total;
}

// add the sums of the segments before b to segment b; fill cursors start there
__device__ __forceinline__ void coll_scan_add(const Dev &d, int b, int *wsum) {
    if (threadIdx.x < 32) {
        int acc = 0;
        for (int k = threadIdx.x; k < b; k += 32) acc += d.hblock[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        __syncwarp();
        if (threadIdx.x == 0) wsum[0] = acc;
    }
    __syncthreads();
    const int base = wsum[0];
    const int i = b * 1024 + 2 * (int)threadIdx.x;
    const int v0 = d.hstart[i] + base, v1 = d.hstart[i + 1] + base;
    d.hstart[i] = v0;
    d.hstart[i + 1] = v1;
    d.hfill[i] = v0;
    d.hfill[i + 1] = v1;
    __syncthreads();  // wsum is reused
}

// the link-table bit of a voxel toward a face neighbour at lattice offset (dx, dy, dz):
// bit 2a for +a, 2a + 1 for -a
__device__ __forceinline__ int link_bit(int dx, int dy, int dz) {
    return dx ? (dx > 0 ? 0 : 1) : dy ? (dy > 0 ? 2 : 3) : (dz > 0 ? 4 : 5);
}

// 2. lists of the robots too large for shared memory (the 64^3 body): one grid over all
// of them in global memory.  Each due robot's surface voxels are binned into a dense
// cell grid over its bounding box (cells of edge cutoff + skin), the robots' grids
// back to back in the bucket table; if they do not fit, cells are hashed with the
// robot id instead and each candidate's cell is compared.  A counting sort stores every
// binned voxel's position and voxel index (spos) and lattice word (sij) in cell order,
// so a candidate costs two independent loads; in a dense grid the 3 x 3 x 3
// neighbourhood is 9 contiguous runs of buckets.  Three lanes per voxel scan one
// dz-plane each, voxels taken in cell order, appending partners to sub-lists in shared
// memory that are sorted and merged by rank, as on the shared-memory path.
__device__ __forceinline__ unsigned fkey(float f) {  // order-preserving float -> unsigned
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ bool grid_voxel(const Dev &d, int s, int *v, int *r) {  // a due voxel of a large robot
    *v = d.csurf[s];
    const uint2 vi = d.vinfo[*v];
    *r = (int)vi.x;
    return d.cflag[1 + *r] && !d.rp[*r].lchunks;
}

__device__ __forceinline__ int3 grid_cell(const GridP &g, float4 p, bool dense) {
    int3 c = make_int3((int)floorf((p.x - g.mnx) * g.ic), (int)floorf((p.y - g.mny) * g.ic), (int)floorf((p.z - g.mnz) * g.ic));
    if (dense) {
        c.x = min(max(c.x, 0), g.gx - 1);
        c.y = min(max(c.y, 0), g.gy - 1);
        c.z = min(max(c.z, 0), g.gz - 1);
    }
    return c;
}

__device__ __forceinline__ int grid_bucket(const Dev &d, const GridP &g, int3 c, int r, bool dense) {
    return dense ? g.base + (c.z * g.gy + c.y) * g.gx + c.x : (int)cell_hash(c.x, c.y, c.z, r, d.hsize - 1);
}

// (a) bounding boxes of the due robots' surface voxels.  Each thread keeps a running box
// of its voxels while they belong to one robot; warps, then the CTA, reduce the boxes of
// one robot before the atomics, so a single large body costs a few atomics per CTA (the
// per-warp atomics on six words serialised to ~20 us for a 64^3 body)
__device__ __forceinline__ void box_atomics(const Dev &d, int r, const unsigned k[6]) {
    unsigned *b = d.gbox + 6 * (size_t)r;
    atomicMin(b + 0, k[0]), atomicMin(b + 1, k[1]), atomicMin(b + 2, k[2]);
    atomicMax(b + 3, k[3]), atomicMax(b + 4, k[4]), atomicMax(b + 5, k[5]);
}

__device__ void grid_boxes(const Dev &d, int gt, int gs) {
    __shared__ int wr[kLocalListThreads / 32];
    __shared__ unsigned wk[kLocalListThreads / 32][6];
    unsigned k[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    int rc = -1;
    for (int s = gt; s < d.ns; s += gs) {
        int v, r;
        if (!grid_voxel(d, s, &v, &r) || (d.vinfo[v].y & VF_LINKMASK) == VF_LINKMASK || (d.vgone && d.vgone[v]))
            continue;
        if (rc >= 0 && r != rc) {  // the thread's voxels changed robot: flush the box so far
            box_atomics(d, rc, k);
            k[0] = k[1] = k[2] = 0xffffffffu;
            k[3] = k[4] = k[5] = 0u;
        }
        rc = r;
        const float4 p = d.cposf[s];
        k[0] = min(k[0], fkey(p.x)), k[1] = min(k[1], fkey(p.y)), k[2] = min(k[2], fkey(p.z));
        k[3] = max(k[3], fkey(p.x)), k[4] = max(k[4], fkey(p.y)), k[5] = max(k[5], fkey(p.z));
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const unsigned any = __ballot_sync(0xffffffffu, rc >= 0);
    int wrob = -1;
    if (any) {
        const int r0 = __shfl_sync(0xffffffffu, rc, __ffs(any) - 1);
        if (__all_sync(0xffffffffu, rc < 0 || rc == r0)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                k[0] = min(k[0], __shfl_xor_sync(0xffffffffu, k[0], o));
                k[1] = min(k[1], __shfl_xor_sync(0xffffffffu, k[1], o));
                k[2] = min(k[2], __shfl_xor_sync(0xffffffffu, k[2], o));
                k[3] = max(k[3], __shfl_xor_sync(0xffffffffu, k[3], o));
                k[4] = max(k[4], __shfl_xor_sync(0xffffffffu, k[4], o));
                k[5] = max(k[5], __shfl_xor_sync(0xffffffffu, k[5], o));
            }
            wrob = r0;
        } else if (rc >= 0) {
            box_atomics(d, rc, k);  // robots mixed within the warp: one flush per thread
        }
    }
    if (lane == 0) {
        wr[wp] = wrob;
        for (int c = 0; c < 6; c++) wk[wp][c] = k[c];
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // merge the warps' boxes of one robot, flushing when the robot changes
        int br = -1;
        unsigned bk[6];
        for (int w = 0; w < kLocalListThreads / 32; w++) {
            if (wr[w] < 0) continue;
            if (br >= 0 && wr[w] != br) box_atomics(d, br, bk);
            if (wr[w] != br) {
                br = wr[w];
                for (int c = 0; c < 6; c++) bk[c] = wk[w][c];
            } else {
                for (int c = 0; c < 3; c++) bk[c] = min(bk[c], wk[w][c]);
                for (int c = 3; c < 6; c++) bk[c] = max(bk[c], wk[w][c]);
            }
        }
        if (br >= 0) box_atomics(d, br, bk);
    }
    __syncthreads();
}

// (b) one thread: grid of every due robot, cells of the list cutoff: dense if every due
// robot's box fits the bucket table, else hashed.  gmode[0] = the reach in cells of a
// dense grid's neighbourhood (1), 0 hashed.  (Cells of half the cutoff with a reach of 2
// scan 58% of the candidates, but leave one or two voxels per cell to share a staged
// neighbourhood: the 64^3 body's lists took 243 us instead of 126 us.)
__device__ void grid_params(const Dev &d) {
    int reach = 1;
    long long total = 0;
    for (; reach >= 0; reach--) {  // 1: dense, 0: hashed
        total = 0;
        bool fits = true;
        for (int r = 0; r < d.nr; r++) {
            const RobotP &rp = d.rp[r];
            if (rp.lchunks || !rp.ns || !d.cflag[1 + r]) continue;
            const unsigned *b = d.gbox + 6 * (size_t)r;
            GridP g;
            g.ic = (float)rp.inv_list_cell;
            g.mnx = fkey_inv(b[0]), g.mny = fkey_inv(b[1]), g.mnz = fkey_inv(b[2]);
            const float ex = (fkey_inv(b[3]) - g.mnx) * g.ic, ey = (fkey_inv(b[4]) - g.mny) * g.ic,
                        ez = (fkey_inv(b[5]) - g.mnz) * g.ic;
            g.gx = g.gy = g.gz = 1;
            g.base = 0;
            if (ex >= 0.0f && ey >= 0.0f && ez >= 0.0f && ex < 65536.0f && ey < 65536.0f && ez < 65536.0f) {
                g.gx = (int)ex + 1, g.gy = (int)ey + 1, g.gz = (int)ez + 1;
                const long long cells = (long long)g.gx * g.gy * g.gz;
                g.base = (int)min(total, (long long)INT_MAX);
                total += cells;
            } else {
                if (!(ex >= 0.0f && ey >= 0.0f && ez >= 0.0f)) g.mnx = g.mny = g.mnz = 0.0f;  // no finite box
                fits = false;
            }
            d.ggrid[r] = g;
        }
        if (reach == 0 || (fits && total <= d.hsize)) break;
    }
    for (int r = 0; r < d.nr; r++) {  // the boxes are ready for the next rebuild
        const RobotP &rp = d.rp[r];
        if (rp.lchunks || !rp.ns || !d.cflag[1 + r]) continue;
        unsigned *b = d.gbox + 6 * (size_t)r;
        b[0] = b[1] = b[2] = 0xffffffffu;
        b[3] = b[4] = b[5] = 0u;
    }
    d.gmode[0] = reach;
    d.gmode[1] = reach ? (int)((total + 1023) / 1024 * 1024) : d.hsize;
}

// (c) count the due surface voxels per bucket
__device__ __forceinline__ void grid_count(const Dev &d, int s) {
    int v, r;
    if (!grid_voxel(d, s, &v, &r)) return;
    const RobotP &rp = d.rp[r];
    const float4 p = d.cposf[s];
    if ((d.vinfo[v].y & VF_LINKMASK) == VF_LINKMASK || (d.vgone && d.vgone[v])) {  // interior or removed: lists nothing
        const float lim = 0.49f * (float)rp.skin;
        d.nnb[s] = 0;
        d.cref[s] = make_float4(p.x, p.y, p.z, lim * lim);
        d.ccell[s].x = -1;
        return;
    }
    const bool dense = d.gmode[0] != 0;
    const GridP g = d.ggrid[r];
    const int bk = grid_bucket(d, g, grid_cell(g, p, dense), r, dense);
    d.ccell[s].x = bk;
    atomicAdd(&d.hcount[bk], 1);
}

// (d) scatter into cell order: position + voxel index, lattice word, surface index
__device__ __forceinline__ void grid_scatter(const Dev &d, int s) {
    int v, r;
    if (!grid_voxel(d, s, &v, &r)) return;
    const int bk = d.ccell[s].x;
    if (bk < 0) return;
    const int slot = atomicAdd(&d.hfill[bk], 1);
    if (slot < 0 || slot >= d.ns) return;
    const float4 p = d.cposf[s];
    const short4 ij = d.ijk[v];
    d.spos[slot] = make_float4(p.x, p.y, p.z, __int_as_float(v));
    d.sij[slot] = make_short4(ij.x, ij.y, ij.z, (d.vinfo[v].y & VF_FIXED) ? 1 : 0);
    d.ssurf[slot] = s;
}

// (e) the lists of the binned voxels, a kernel of its own after k_coll_prepare.
// Dense grid: every warp takes an equal contiguous range of the binned voxels (cell
// order) and works through it cell by cell.  Every voxel of a cell has the same 3 x 3 x 3
// neighbourhood -- nine runs of three buckets in the binned order -- so the warp streams
// the candidates through its lanes 32 at a time (one independent load each) and, in each
// round, tests each of its voxels of the cell against them: one round trip to memory per
// 32 candidates serves all of them.  The voxels and their partner lists sit in shared
// memory (32 voxels at a time); the partners found are compacted by ballot and written
// out in ascending voxel order, each at its rank.  A hashed grid (a bucket may hold
// several cells) is listed voxel by voxel with the same tests, each candidate's cell
// compared.  The 64^3 body's lists at step 4,700: 126 us (three lanes per voxel with
// sorted sub-lists in shared memory, inside the cooperative kernel at 16 warps per SM
// with a third of the lanes active: 190 us; one warp per voxel: 152 us; a warp per cell
// with each CTA a contiguous range of buckets: 380 us, the occupied cells of a folded
// body falling to few CTAs; staging only the candidates near a cell's voxels: 165 us).
constexpr int kGridListThreads = 128;
constexpr int kGridListWarps = kGridListThreads / 32;

struct ListScratch {
    int found[32][kNbrCap];  // the partners of the cell's voxels (32 at a time), in the order found
    int nfound[32];
    float4 pv[32];           // those voxels: FP32 position, voxel index in w
    short4 ij[32];           // lattice coordinates, w = fixed
    uint32_t viy[32];        // link bits
    int s[32];               // collision-surface index
    int lst[kNbrCap];        // one voxel's partners (voxel indices) for the per-voxel path
};

// the partner tests of one pair (voxel v: position pv, lattice word ij, link bits vi_y,
// robot parameters rp) for a candidate u at pu / ik within the cutoff
__device__ __forceinline__ bool list_pair(const Dev &d, bool attach, int v, float4 pv, short4 ij, uint32_t vi_y,
                                          float cut2, int u, float4 pu, short4 ik) {
    const float ex = pu.x - pv.x, ey = pu.y - pv.y, ez = pu.z - pv.z;
    if (!(u != v && ex * ex + ey * ey + ez * ez <= cut2)) return false;
    // is_neighbor depth 1 (VX3_VoxelyzeKernel.cu:651-680): a link joins them
    // (a runtime link may join any two voxels: the face partners say)
    const int ddx = ik.x - ij.x, ddy = ik.y - ij.y, ddz = ik.z - ij.z;
    if (attach) {
        if (linked_to(d, v, u)) return false;
    } else if (abs(ddx) + abs(ddy) + abs(ddz) == 1 && ((vi_y >> link_bit(ddx, ddy, ddz)) & 1u)) {
        return false;
    }
    return !((ij.w & 1) && (ik.w & 1));  // not both fixed
}

// the found partners (n of them, the first kNbrCap kept in L) written in ascending order
__device__ __forceinline__ void list_write(const Dev &d, int lane, int s, int r, float4 pv, float skin, int n,
                                           const int *L) {
    __syncwarp();
    const int nc = min(n, kNbrCap);
    const size_t ns = (size_t)d.ns;
    for (int a = lane; a < nc; a += 32) {  // entries are distinct voxel indices: ranks are a permutation
        const int x = L[a];
        int rank = 0;
        for (int i = 0; i < nc; i++) rank += L[i] < x ? 1 : 0;
        d.nbr[s + (size_t)rank * ns] = x;
    }
    if (lane == 0) {
        d.nnb[s] = nc;
        if (n > kNbrCap) atomicOr(&d.status[r], 2);
        const float lim = 0.49f * skin;  // rebuild when a voxel has moved farther than this
        d.cref[s] = make_float4(pv.x, pv.y, pv.z, lim * lim);
    }
    __syncwarp();
}

// one binned voxel k, its candidates read from global memory, 32 at a time
__device__ void list_voxel(const Dev &d, int k, int nbin, bool dense, int lane, int *L) {
    const int s = d.ssurf[k];
    const float4 pv = d.spos[k];
    const int v = __float_as_int(pv.w);
    const short4 ij = d.sij[k];
    const uint2 vi = d.vinfo[v];
    const int r = (int)vi.x;
    const RobotP &rp = d.rp[r];
    const GridP g = d.ggrid[r];
    const int3 c = grid_cell(g, pv, dense);
    // 1e-3 relative margin: FP32 positions up to ~100 m from the origin lose no true pair
    const float cut = (float)(rp.cell_size + rp.skin) * 1.001f, cut2 = cut * cut;
    const bool attach = rp.attach != 0;
    const int R = dense ? d.gmode[0] : 1, w = 2 * R + 1;  // reach in cells
    const int nruns = dense ? w * w : 27;
    // run `lane`: [rb, rb + rl) of the binned order; hashed grid: its cell (cx, cy, cz)
    int rb = 0, rl = 0, cx = 0, cy = 0, cz = 0;
    if (lane < nruns) {
        int e = 0;
        if (dense) {
            const int z = c.z + lane / w - R, y = c.y + lane % w - R;
            if (z >= 0 && z < g.gz && y >= 0 && y < g.gy) {
                const int rw = g.base + (z * g.gy + y) * g.gx;
                rb = d.hstart[rw + max(c.x - R, 0)];
                e = d.hfill[rw + min(c.x + R, g.gx - 1)];  // the bucket's end after the scatter
            }
        } else {
            cz = c.z + lane / 9 - 1, cy = c.y + (lane / 3) % 3 - 1, cx = c.x + lane % 3 - 1;
            const int h = (int)cell_hash(cx, cy, cz, r, d.hsize - 1);
            rb = d.hstart[h];
            e = d.hfill[h];
        }
        rl = max(min(e, nbin) - rb, 0);
    }
    int ro = rl;  // inclusive, then exclusive prefix of the run lengths
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, ro, o);
        if (lane >= o) ro += t;
    }
    const int total = __shfl_sync(0xffffffffu, ro, 31);
    ro -= rl;
    int n = 0;  // partners found so far (the same in every lane)
    for (int t0 = 0; t0 < total; t0 += 32) {
        const int t = t0 + lane;
        int run = 0;  // the last run starting at or before t (empty runs share the next one's start)
        for (int i = 1; i < nruns; i++) run += __shfl_sync(0xffffffffu, ro, i) <= t ? 1 : 0;
        const int jb = __shfl_sync(0xffffffffu, rb, run), jo = __shfl_sync(0xffffffffu, ro, run);
        const int ex_x = __shfl_sync(0xffffffffu, cx, run), ex_y = __shfl_sync(0xffffffffu, cy, run),
                  ex_z = __shfl_sync(0xffffffffu, cz, run);
        bool acc = false;
        int u = 0;
        if (t < total) {
            const int j = jb + (t - jo);
            const float4 pu = d.spos[j];
            const short4 ik = d.sij[j];
            u = __float_as_int(pu.w);
            acc = list_pair(d, attach, v, pv, ij, vi.y, cut2, u, pu, ik);
            if (acc && !dense) {  // another cell in the same bucket, or another robot
                const int3 cu = grid_cell(g, pu, false);
                acc = cu.x == ex_x && cu.y == ex_y && cu.z == ex_z && (int)d.vinfo[u].x == r;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        if (acc) {
            const int p = n + __popc(m & ((1u << lane) - 1u));
            if (p < kNbrCap) L[p] = u;
        }
        n += __popc(m);
    }
    list_write(d, lane, s, r, pv, (float)rp.skin, n, L);
}

__global__ void __launch_bounds__(kGridListThreads) k_grid_list(Dev d) {
    __shared__ ListScratch scratch[kGridListWarps];
    if (!*(volatile int *)d.cflag) return;   // no robot is due this step
    if (*(volatile int *)d.err & 1) return;  // a grid barrier of k_coll_prepare gave up
    const int used = d.gmode[1];  // 0 when no large robot is due this step
    if (used <= 0) return;
    const int nbin = min(d.hstart[used - 1] + d.hcount[used - 1], d.ns);  // voxels binned this step
    if (nbin <= 0) return;
    const bool dense = d.gmode[0] != 0;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    ListScratch &S = scratch[wp];
    if (!dense) {  // voxel by voxel, each CTA a contiguous range in cell order
        const int per_cta = (nbin + gridDim.x - 1) / gridDim.x;
        const int k1 = min(nbin, (blockIdx.x + 1) * per_cta);
        for (int k = blockIdx.x * per_cta + wp; k < k1; k += kGridListWarps) list_voxel(d, k, nbin, false, lane, S.lst);
        return;
    }
    // dense: each warp an equal contiguous range of the binned voxels (cell order), taken
    // cell by cell (consecutive warps of a CTA take consecutive ranges: shared L1 lines)
    const int R = d.gmode[0], w = 2 * R + 1, nruns = w * w;  // reach in cells, rows of the neighbourhood
    const int nw = gridDim.x * kGridListWarps;
    const int per_w = (nbin + nw - 1) / nw;
    const int kend = min(nbin, (blockIdx.x * kGridListWarps + wp + 1) * per_w);
    for (int k = (blockIdx.x * kGridListWarps + wp) * per_w; k < kend;) {
        const int b = d.ccell[d.ssurf[k]].x;  // the bucket (cell) of voxel k
        const int cnt = min(min(d.hfill[b], nbin), kend) - k;  // this warp's voxels of the cell
        const int beg = k;
        k += max(cnt, 1);
        if (cnt <= 0) continue;
        // the cell's robot (one robot per dense cell) and its coordinates
        const int r = (int)d.vinfo[__float_as_int(d.spos[beg].w)].x;
        const RobotP &rp = d.rp[r];
        const GridP g = d.ggrid[r];
        const int loc = b - g.base;
        const int3 c = make_int3(loc % g.gx, (loc / g.gx) % g.gy, loc / (g.gx * g.gy));
        int rb = 0, rl = 0;  // run `lane`: row (dz, dy) of the neighbourhood, cells x-R .. x+R
        if (lane < nruns) {
            const int z = c.z + lane / w - R, y = c.y + lane % w - R;
            if (z >= 0 && z < g.gz && y >= 0 && y < g.gy) {
                const int rw = g.base + (z * g.gy + y) * g.gx;
                rb = d.hstart[rw + max(c.x - R, 0)];
                rl = max(min(d.hfill[rw + min(c.x + R, g.gx - 1)], nbin) - rb, 0);  // bucket ends after the scatter
            }
        }
        int ro = rl;  // inclusive, then exclusive prefix of the run lengths
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, ro, o);
            if (lane >= o) ro += t;
        }
        const int total = __shfl_sync(0xffffffffu, ro, 31);
        ro -= rl;
        const float cut = (float)(rp.cell_size + rp.skin) * 1.001f, cut2 = cut * cut;
        const bool attach = rp.attach != 0;
        for (int i0 = 0; i0 < cnt; i0 += 32) {  // the voxels, 32 at a time
            const int m = min(32, cnt - i0);
            if (lane < m) {
                const int kk = beg + i0 + lane;
                const float4 p = d.spos[kk];
                S.s[lane] = d.ssurf[kk];
                S.pv[lane] = p;
                S.ij[lane] = d.sij[kk];
                S.viy[lane] = d.vinfo[__float_as_int(p.w)].y;
                S.nfound[lane] = 0;
            }
            __syncwarp();
            for (int t0 = 0; t0 < total; t0 += 32) {  // candidate rounds
                const int t = t0 + lane;
                int run = 0;  // the last run starting at or before t (empty runs share the next one's start)
                for (int i = 1; i < nruns; i++) run += __shfl_sync(0xffffffffu, ro, i) <= t ? 1 : 0;
                const int j = __shfl_sync(0xffffffffu, rb, run) + (t - __shfl_sync(0xffffffffu, ro, run));
                float4 pu = make_float4(0.f, 0.f, 0.f, 0.f);
                short4 ik = make_short4(0, 0, 0, 0);
                if (t < total) {
                    pu = d.spos[j];
                    ik = d.sij[j];
                }
                const int u = __float_as_int(pu.w);
                for (int i = 0; i < m; i++) {
                    const bool acc = t < total && list_pair(d, attach, __float_as_int(S.pv[i].w), S.pv[i], S.ij[i],
                                                            S.viy[i], cut2, u, pu, ik);
                    const unsigned hit = __ballot_sync(0xffffffffu, acc);
                    if (hit) {
                        const int n = S.nfound[i];
                        if (acc) {
                            const int q = n + __popc(hit & ((1u << lane) - 1u));
                            if (q < kNbrCap) S.found[i][q] = u;
                        }
                        __syncwarp();
                        if (lane == 0) S.nfound[i] = n + __popc(hit);
                        __syncwarp();
                    }
                }
            }
            for (int i = 0; i < m; i++) list_write(d, lane, S.s[i], r, S.pv[i], (float)rp.skin, S.nfound[i], S.found[i]);
        }
    }
}

// 2'. lists of the robots on the shared-memory path.  The work list holds the robots
// due this step, each with its chunks of kLocalListChunk collision-surface voxels;
// CTA b takes a contiguous range of those chunks.  For a chunk it bins every
// collision-surface voxel of the chunk's robot into a cell grid in shared memory
// (counting sort; kept while consecutive chunks belong to the same robot), then three
// threads list the partners of each voxel of the chunk, in ascending order.  The grid
// is dense over the robot's bounding box when that has at most kLocalHash cells (the
// 3 x 3 x 3 neighbourhood is then 9 contiguous runs of buckets), else hashed, with
// each candidate's cell compared.
// Shared memory: P[lmax] (FP32 position from the displacement check; w holds the
// packed lattice coordinates and fixed flag, cpk), cur/beg[kLocalHash] (bucket
// ends and starts), srt[lmax] (local indices sorted by bucket),
// cand[kNbrCap][kLocalListThreads] (each thread's sorted sub-list).
size_t local_list_smem(int lmax) {
    return (size_t)lmax * sizeof(float4) + 2 * (size_t)kLocalHash * sizeof(int) + (size_t)((lmax + 7) & ~7) * 2 +
           (size_t)kNbrCap * kLocalListThreads * 2;
}

struct LocalGrid {
    float3 mn;    // bounding-box corner
    float ic;     // 1 / cell edge
    int3 g;       // cells per axis (dense grid)
    int dense;
};

__device__ __forceinline__ int3 local_cell(float4 p, const LocalGrid &G) {
    int3 c = make_int3((int)floorf((p.x - G.mn.x) * G.ic), (int)floorf((p.y - G.mn.y) * G.ic),
                       (int)floorf((p.z - G.mn.z) * G.ic));
    if (G.dense) {
        c.x = min(max(c.x, 0), G.g.x - 1);
        c.y = min(max(c.y, 0), G.g.y - 1);
        c.z = min(max(c.z, 0), G.g.z - 1);
    }
    return c;
}

__device__ __forceinline__ int local_bucket(int3 c, const LocalGrid &G) {
    return G.dense ? (c.z * G.g.y + c.y) * G.g.x + c.x : (int)cell_hash(c.x, c.y, c.z, 0, kLocalHash - 1);
}

__device__ __forceinline__ void coll_list_robots(const Dev &d, unsigned char *lsm, int *wsum) {
    constexpr int T = kLocalListThreads, NW = T / 32;
    __shared__ float wbox[6][NW];
    __shared__ LocalGrid G;
    float4 *P = reinterpret_cast<float4 *>(lsm);
    int *cur = reinterpret_cast<int *>(P + d.lmax);
    int *beg = cur + kLocalHash;
    unsigned short *srt = reinterpret_cast<unsigned short *>(beg + kLocalHash);
    unsigned short *cand = srt + ((d.lmax + 7) & ~7);
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
    const unsigned long long w = *(volatile unsigned long long *)d.lwork_ctr;
    const int nrob = (int)min(w >> 32, (unsigned long long)d.nr), nitem = (int)(w & 0xffffffffull);
    const int i0 = (int)((long long)nitem * blockIdx.x / gridDim.x);
    const int i1 = (int)((long long)nitem * (blockIdx.x + 1) / gridDim.x);
    int built = -1;
    for (int item = i0; item < i1; item++) {
        int lo = 0, hi = nrob - 1;  // the last work entry whose first chunk is <= item
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldcg(&d.lwork[mid].y) <= item) lo = mid;
            else hi = mid - 1;
        }
        const int2 wk = __ldcg(&d.lwork[lo]);
        const int r = wk.x;
        if (r < 0 || r >= d.nr || item < wk.y) continue;  // (uniform) a work list the check did not write
        const RobotP &rp = d.rp[r];
        const int n = rp.ns, s0 = rp.soff;
        if (!rp.lchunks || n > d.lmax) continue;
        if (r != built) {  // uniform across the CTA
            __syncthreads();  // the previous robot's table is no longer read
            for (int h = tid; h < kLocalHash; h += T) cur[h] = 0;
            float bx0 = INFINITY, by0 = INFINITY, bz0 = INFINITY, bx1 = -INFINITY, by1 = -INFINITY, bz1 = -INFINITY;
            for (int i = tid; i < n; i += T) {
                const float4 q = __ldcg(&d.cposf[s0 + i]);
                unsigned pk = d.cpk[s0 + i];
                if (rp.dyn) {  // interior or removed: neither lists nor is listed
                    const int v = d.csurf[s0 + i];
                    if ((d.vinfo[v].y & VF_LINKMASK) == VF_LINKMASK || (d.vgone && d.vgone[v])) pk |= kPackInterior;
                }
                P[i] = make_float4(q.x, q.y, q.z, __uint_as_float(pk));
                bx0 = fminf(bx0, q.x), by0 = fminf(by0, q.y), bz0 = fminf(bz0, q.z);
                bx1 = fmaxf(bx1, q.x), by1 = fmaxf(by1, q.y), bz1 = fmaxf(bz1, q.z);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
                by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
                bz0 = fminf(bz0, __shfl_xor_sync(0xffffffffu, bz0, o));
                bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
                by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
                bz1 = fmaxf(bz1, __shfl_xor_sync(0xffffffffu, bz1, o));
            }
            if (lane == 0) {
                wbox[0][wp] = bx0, wbox[1][wp] = by0, wbox[2][wp] = bz0;
                wbox[3][wp] = bx1, wbox[4][wp] = by1, wbox[5][wp] = bz1;
            }
            __syncthreads();
            if (tid == 0) {
                for (int k = 1; k < NW; k++) {
                    bx0 = fminf(bx0, wbox[0][k]), by0 = fminf(by0, wbox[1][k]), bz0 = fminf(bz0, wbox[2][k]);
                    bx1 = fmaxf(bx1, wbox[3][k]), by1 = fmaxf(by1, wbox[4][k]), bz1 = fmaxf(bz1, wbox[5][k]);
                }
                LocalGrid g;
                g.ic = (float)rp.inv_list_cell;
                g.mn = make_float3(bx0, by0, bz0);
                const float ex = (bx1 - bx0) * g.ic, ey = (by1 - by0) * g.ic, ez = (bz1 - bz0) * g.ic;
                g.dense = 0;
                g.g = make_int3(1, 1, 1);
                // finite extents below kLocalHash cells per axis (NaN fails every comparison)
                if (ex >= 0.0f && ey >= 0.0f && ez >= 0.0f && ex < (float)kLocalHash && ey < (float)kLocalHash &&
                    ez < (float)kLocalHash) {
                    const int gx = (int)ex + 1, gy = (int)ey + 1, gz = (int)ez + 1;
                    if ((long long)gx * gy * gz <= kLocalHash) {
                        g.g = make_int3(gx, gy, gz);
                        g.dense = 1;
                    }
                }
                if (!g.dense && !(bx0 <= bx1 && by0 <= by1 && bz0 <= bz1))
                    g.mn = make_float3(0.0f, 0.0f, 0.0f);  // non-finite box: absolute cells
                G = g;
            }
            __syncthreads();
            const LocalGrid g = G;
            for (int i = tid; i < n; i += T) atomicAdd(&cur[local_bucket(local_cell(P[i], g), g)], 1);
            __syncthreads();
            // exclusive scan of the bucket counts, kLocalHash / T buckets per thread
            constexpr int per = kLocalHash / T;
            int sum = 0;
#pragma unroll
            for (int k = 0; k < per; k++) sum += cur[tid * per + k];
            int x = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) wsum[wp] = x;
            __syncthreads();
            if (wp == 0) {
                int t = lane < NW ? wsum[lane] : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, t, o);
                    if (lane >= o) t += y;
                }
                if (lane < NW) wsum[lane] = t;
            }
            __syncthreads();
            int e = x - sum + (wp ? wsum[wp - 1] : 0);
#pragma unroll
            for (int k = 0; k < per; k++) {
                const int ck = cur[tid * per + k];
                beg[tid * per + k] = e;
                cur[tid * per + k] = e;
                e += ck;
            }
            __syncthreads();
            for (int i = tid; i < n; i += T) {
                const int slot = atomicAdd(&cur[local_bucket(local_cell(P[i], g), g)], 1);
                if (slot < n) srt[slot] = (unsigned short)i;  // bucket h: srt[beg[h] .. cur[h])
            }
            __syncthreads();
            built = r;
        }
        // three threads per voxel (a trio), thread q of the trio scanning the plane
        // dz = q - 1 of the 3 x 3 x 3 neighbourhood; ten trios per warp, the voxels taken
        // in bucket order so that a warp's trios work on neighbouring cells
        const int trio = lane / 3, q = lane - 3 * trio, tb = lane - q;
        const int pos = (item - wk.y) * kLocalListChunk + wp * 10 + trio;
        const bool valid = lane < 30 && pos < n && item - wk.y < rp.lchunks;
        unsigned short *my = cand + tid;  // this thread's sub-list, entry j at my[j*T]
        int nc = 0, i = 0;
        float4 pi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (valid) {
            i = srt[pos];
            pi = P[i];
        }
        if (valid && !(__float_as_uint(pi.w) & kPackInterior)) {  // interior voxels list nothing
            const LocalGrid g = G;
            const unsigned ki = __float_as_uint(pi.w);
            // the voxel's link table: face neighbours are excluded only while a link joins them
            const unsigned imask = rp.dyn ? d.vinfo[d.csurf[s0 + i]].y & VF_LINKMASK : VF_LINKMASK;
            const int3 c = local_cell(pi, g);
            // 1e-3 relative margin: FP32 positions up to ~100 m from the origin lose no true pair
            const float cut = (float)(rp.cell_size + rp.skin) * 1.001f, cut2 = cut * cut;
            const int z = c.z + q - 1;
            if (!g.dense || (z >= 0 && z < g.g.z)) {
                for (int dy = -1; dy <= 1; dy++) {
                    const int y = c.y + dy;
                    if (g.dense && (y < 0 || y >= g.g.y)) continue;
                    // dense grid: one run of buckets, cells x-1 .. x+1; hashed grid: the three
                    // cells one by one, each candidate's cell compared
                    for (int dx = -1; dx <= (g.dense ? -1 : 1); dx++) {
                        int b, e;
                        if (g.dense) {
                            const int rw = (z * g.g.y + y) * g.g.x;
                            b = beg[rw + max(c.x - 1, 0)];
                            e = cur[rw + min(c.x + 1, g.g.x - 1)];
                        } else {
                            const int h = (int)cell_hash(c.x + dx, y, z, 0, kLocalHash - 1);
                            b = beg[h];
                            e = cur[h];
                        }
                        e = min(e, n);
                        for (int k = b; k < e; k++) {
                            const int t = srt[k];
                            const float4 pt = P[t];
                            const float ex = pt.x - pi.x, ey = pt.y - pi.y, ez = pt.z - pi.z;
                            const unsigned kt = __float_as_uint(pt.w);
                            // is_neighbor depth 1 (VX3_VoxelyzeKernel.cu:651-680): a link joins them;
                            // face neighbours have a packed lattice difference of +-1, +-2^10 or +-2^20
                            const int dl = (int)(ki & kPackMask) - (int)(kt & kPackMask);
                            const int ad = abs(dl);
                            const bool face = ad == 1 || ad == (1 << 10) || ad == (1 << 20);
                            const int bit = (ad == 1 ? 0 : ad == (1 << 10) ? 2 : 4) + (dl > 0 ? 1 : 0);
                            bool linked = face && ((imask >> bit) & 1u);
                            bool acc = ex * ex + ey * ey + ez * ez <= cut2 && t != i &&
                                       !(ki & kt & kPackFixed) && !(kt & kPackInterior);
                            // a runtime link may join any two voxels: the face partners say
                            if (acc && rp.attach) linked = linked_to(d, d.csurf[s0 + i], d.csurf[s0 + t]);
                            acc = acc && !linked;
                            if (!g.dense) {
                                const int3 ct = local_cell(pt, g);
                                acc = acc && ct.x == c.x + dx && ct.y == y && ct.z == z;  // same bucket, other cell
                            }
                            if (acc) {
                                if (nc < kNbrCap) my[nc * T] = (unsigned short)t;
                                nc++;
                            }
                        }
                    }
                }
            }
        }
        const bool overflow = nc > kNbrCap;
        nc = min(nc, kNbrCap);
        for (int a2 = 1; a2 < nc; a2++) {  // ascending
            const int x = my[a2 * T];
            int j = a2;
            while (j > 0 && my[(j - 1) * T] > x) {
                my[j * T] = my[(j - 1) * T];
                j--;
            }
            my[j * T] = (unsigned short)x;
        }
        // merge the trio's three disjoint sorted sub-lists: an entry's place in the list
        // is its index in its own sub-list plus the entries below it in the other two
        int c3[3];
        bool ov3 = false;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            c3[k] = __shfl_sync(0xffffffffu, nc, (tb + k) & 31);
            ov3 |= __shfl_sync(0xffffffffu, overflow ? 1 : 0, (tb + k) & 31) != 0;
        }
        __syncwarp();
        if (valid) {
            // the robot's collision-surface voxels are in ascending voxel order, so
            // ascending local index is the ascending partner order of the reference
            const int s = s0 + i;
            int *out = d.nbr + s;
            const size_t ns = (size_t)d.ns;
            for (int j = 0; j < nc; j++) {
                const int e = my[j * T];
                int rank = j;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    if (k == q) continue;
                    const unsigned short *o = cand + (tid - q + k);
                    int m = 0;
                    while (m < c3[k] && o[m * T] < e) m++;
                    rank += m;
                }
                if (rank < kNbrCap) out[rank * ns] = d.csurf[s0 + e];
            }
            if (q == 0) {
                const int total = c3[0] + c3[1] + c3[2];
                d.nnb[s] = min(total, kNbrCap);
                if (ov3 || total > kNbrCap) atomicOr(&d.status[r], 2);
                const float lim = 0.49f * (float)rp.skin;  // rebuild when a voxel has moved farther than this
                d.cref[s] = make_float4(pi.x, pi.y, pi.z, lim * lim);
            }
        }
    }
}

// Barrier across the CTAs of the cooperative k_coll_prepare (a cooperative launch
// keeps them all resident).  gbar[0] counts arrivals, gbar[1] is the generation; the
// last CTA to arrive resets the count and advances the generation.  A CTA that has
// waited gbar[2] polls (kBarrierPolls unless a test lowered it) records bit 1 in d.err
// and returns false; vx3g_status reports it and clears gbar[0..1] and the error word.
__device__ bool grid_barrier(const Dev &d) {
    __shared__ int passed;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = d.gbar + 1;
        const unsigned g = *gen;
        const unsigned limit = *(volatile unsigned *)(d.gbar + 2);
        __threadfence();
        if (atomicAdd(d.gbar, 1u) == gridDim.x - 1) {
            atomicExch(d.gbar, 0u);
            __threadfence();
            atomicAdd(d.gbar + 1, 1u);
            passed = 1;
        } else {
            unsigned k = 0;
            while (*gen == g && ++k < limit) __nanosleep(32);
            passed = *gen != g;
            if (!passed) atomicOr(d.err, 1);
        }
        __threadfence();
    }
    __syncthreads();
    return passed != 0;
}

// The collision pass before the narrow phase, one cooperative launch per step: the
// displacement check of every surface voxel; then, only in a step where some robot
// is due, the rebuild of its lists (hashed-grid phases separated by grid barriers,
// and the shared-memory path).  No host or graph decision sits between them.
// the displacement check of every collision-surface voxel, at full occupancy, just
// before k_coll_prepare
__global__ void __launch_bounds__(256) k_coll_check(Dev d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < d.ns) coll_check(d, s);
}

__global__ void __launch_bounds__(kLocalListThreads, 1) k_coll_prepare(Dev d) {
    extern __shared__ __align__(16) unsigned char lsm[];
    __shared__ int wsum[kLocalListThreads / 32];
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    if (!*(volatile int *)d.cflag) return;  // (uniform: k_coll_check has finished) no robot is due
    // a barrier gave up in an earlier launch and vx3g_status has not cleared it yet: the
    // arrival count may be stale, so no barrier of this launch could be trusted
    if (*(volatile int *)d.err & 1) return;
    if (d.nhash) {  // robots too large for shared memory, if any is due (their lists: k_grid_list)
        grid_boxes(d, gt, gs);
        if (!grid_barrier(d)) return;
        if (gt == 0) grid_params(d);
        if (!grid_barrier(d)) return;
        const int used = d.gmode[1];
        for (int i = gt; i < used; i += gs) d.hcount[i] = 0;
        if (!grid_barrier(d)) return;
        for (int s = gt; s < d.ns; s += gs) grid_count(d, s);
        if (!grid_barrier(d)) return;
        for (int b = blockIdx.x; b < used / 1024; b += gridDim.x) coll_scan_segment(d, b, wsum);
        if (!grid_barrier(d)) return;
        for (int b = blockIdx.x; b < used / 1024; b += gridDim.x) coll_scan_add(d, b, wsum);
        if (!grid_barrier(d)) return;
        for (int s = gt; s < d.ns; s += gs) grid_scatter(d, s);
    }
    if (d.lmax) coll_list_robots(d, lsm, wsum);
}

// dynamic shared memory of k_coll_prepare: the shared-memory path's tables
static size_t coll_prepare_smem(const Dev &d) { return d.lmax ? local_list_smem(d.lmax) : 0; }

cudaError_t init_collision(Dev &d) {
    d.cgrid = 0;
    if (!d.ns) return cudaSuccess;
    const size_t sm = coll_prepare_smem(d);
    cudaError_t e = cudaFuncSetAttribute(k_coll_prepare, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 0, occ = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_coll_prepare, kLocalListThreads, sm)) !=
        cudaSuccess)
        return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    d.cgrid = nsm * occ;  // every CTA resident: the grid barrier's premise
    d.glgrid = 0;
    if (d.nhash) {  // k_grid_list: as many CTAs as fit at once
        int gocc = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gocc, k_grid_list, kGridListThreads, 0)) != cudaSuccess)
            return e;
        d.glgrid = nsm * std::max(gocc, 1);
    }
    return cudaSuccess;
}

// force on voxel1 from the pair (voxel1, voxel2) as VX3_Collision computes it
__device__ __forceinline__ V3<double> pair_force(const Dev &d, int v1, int v2, double bsa1, double bsa2) {
    const VMat &m1 = d.vmat[d.vinfo[v1].y >> 8];
    const VMat &m2 = d.vmat[d.vinfo[v2].y >> 8];
    const double pstiff = 2.0f / (1.0f / m1.pstiff + 1.0f / m2.pstiff);
    const double dampC = 0.5f * (m1.c_col + m2.c_col);
    const double4 p1 = load_state(d, d.pos, v1), p2 = load_state(d, d.pos, v2);
    const V3<double> offset{p2.x - p1.x, p2.y - p1.y, p2.z - p1.z};
    const double nom = (bsa1 + bsa2) * 0.625;
    const double rel = nom - len(offset);
    if (!(rel > 0)) return V3<double>{0, 0, 0};
    const V3<double> u = normalized(offset);
    const double4 l1 = load_state(d, d.linmom, v1), l2 = load_state(d, d.linmom, v2);
    const V3<double> w1 = scl(V3<double>{l1.x, l1.y, l1.z}, m1.mass_inv);
    const V3<double> w2 = scl(V3<double>{l2.x, l2.y, l2.z}, m2.mass_inv);
    const double rv = (w1.x * u.x + w1.y * u.y + w1.z * u.z) - (w2.x * u.x + w2.y * u.y + w2.z * u.z);
    return scl(u, pstiff * rel + dampC * rv);
}

// 3. exact test and contact forces on the listed pairs, ascending partner order
__global__ void k_coll_eval(Dev d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) {  // the rebuild (if any) is done; the next check starts clear
        *d.cflag = 0;
        *d.lwork_ctr = 0ull;
    }
    if (s >= d.ns) return;
    const int v = d.csurf[s];
    const uint2 vi = d.vinfo[v];
    const int r = (int)vi.x;
    if (d.cflag[1 + r]) d.cflag[1 + r] = 0;
    if (d.status[r] != 0) return;
    const int n = d.nnb[s];
    const int *lst = d.nbr + s;  // slot-major: entry k at lst[k*ns]
    const size_t ns = (size_t)d.ns;
    // attachment linked some pairs this step: their contact is added, then taken back
    // (VX3_VoxelyzeKernel.cu:824-826); a listed pair with a link was linked this step
    // (a link makes its robot rebuild its lists in the next step)
    const bool att = d.narob && d.rp[r].attach && d.acnt[r] > 0;
    V3<double> acc{0, 0, 0};
    if (!runs_force(d, d.rp[r].bcs, v, vi.y)) {  // its contactForce is never cleared: the pairs add to it
        const double4 c = d.contact[v];
        acc = V3<double>{c.x, c.y, c.z};
    }
    if (n) {
        const float4 pf = pos_f(d, v);
        const double4 pv = load_state(d, d.pos, v);
        double bsa = 0;
        bool have_bsa = false;
        for (int k = 0; k < n; k++) {
            const int u = lst[k * ns];  // partner voxel, ascending
            // FP32 prefilter against the current cutoff: only pairs within 0.1% of it reach FP64
            const float4 tf = pos_f(d, u);
            const float ex = tf.x - pf.x, ey = tf.y - pf.y, ez = tf.z - pf.z;
            const float cw = (pf.w + tf.w) * 0.625f * 1.001f;
            if (ex * ex + ey * ey + ez * ez > cw * cw) continue;
            if (!have_bsa) {
                bsa = (pv.w + pv.w + pv.w) / 3.0f;  // baseSizeAverage (VX3_Voxel.h:102-105)
                have_bsa = true;
            }
            const double4 pu = load_state(d, d.pos, u);
            const double bu = (pu.w + pu.w + pu.w) / 3.0f;
            // exact envelope test, voxel1 = the later surface voxel
            const double4 &pa = u < v ? pv : pu, &pb = u < v ? pu : pv;
            const double ba = u < v ? bsa : bu, bb = u < v ? bu : bsa;
            const V3<double> diff{pa.x - pb.x, pa.y - pb.y, pa.z - pb.z};
            const double wd = (ba + bb) * 0.625;
            if (diff.x > wd || diff.x < -wd) continue;
            if (diff.y > wd || diff.y < -wd) continue;
            if (diff.z > wd || diff.z < -wd) continue;
            if (len(diff) > wd) continue;
            // v.contactForce += force (v is voxel1) or += -force (v is voxel2)
            const V3<double> f = u < v ? pair_force(d, v, u, bsa, bu) : neg(pair_force(d, u, v, bu, bsa));
            acc = add(acc, f);
            if (att && linked_to(d, v, u)) acc = sub(acc, f);
        }
    }
    d.contact[v] = make_double4(acc.x, acc.y, acc.z, 0.0);
}

cudaError_t launch_coll_prepare(const Dev &d, cudaStream_t s) {
    if (!d.ns) return cudaSuccess;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cs);
    if (e != cudaSuccess) return e;
    if (cs == cudaStreamCaptureStatusNone) {
        // single steps start from clear flags (inside graphs the narrow phase clears them)
        if ((e = cudaMemsetAsync(d.cflag, 0, sizeof(int) * (1 + (size_t)d.nr), s)) != cudaSuccess ||
            (e = cudaMemsetAsync(d.lwork_ctr, 0, sizeof(unsigned long long), s)) != cudaSuccess)
            return e;
    }
    k_coll_check<<<(d.ns + 255) / 256, 256, 0, s>>>(d);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)d.cgrid);
    cfg.blockDim = dim3(kLocalListThreads);
    cfg.dynamicSmemBytes = coll_prepare_smem(d);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if ((e = cudaLaunchKernelEx(&cfg, k_coll_prepare, d)) != cudaSuccess) return e;
    if (d.glgrid) k_grid_list<<<d.glgrid, kGridListThreads, 0, s>>>(d);  // the large robots' lists, if rebuilt
    return cudaSuccess;
}

cudaError_t launch_collision(const Dev &d, cudaStream_t s) {
    if (!d.ns) return cudaSuccess;
    const cudaError_t e = launch_coll_prepare(d, s);
    if (e != cudaSuccess) return e;
    launch_attach(d, s);  // robots with EnableAttach: links made in the pair order, before the contacts
    launch_coll_eval(d, s);
    return cudaGetLastError();
}

void launch_coll_eval(const Dev &d, cudaStream_t s) {
    if (!d.ns) return;
    if (d.mixed) launch_coll_eval_mixed(d, s);
    else k_coll_eval<<<(d.ns + 255) / 256, 256, 0, s>>>(d);
}

// ---------------------------------------------------------------- host state exchange
// vx3g_set_state / vx3g_get_state convert between plain doubles (comps per voxel)
// and the 32-byte state slots on the device: double4, or float4 hi + float4 lo
// (mixed).  keep_w keeps the slot's 4th component (the base size of pos).
__device__ __forceinline__ void put_slot(double4 *dst, size_t i, int mixed, double a, double b, double c, double w) {
    if (!mixed) {
        dst[i] = make_double4(a, b, c, w);
        return;
    }
    float4 *f = reinterpret_cast<float4 *>(dst) + 2 * i;
    const float ha = (float)a, hb = (float)b, hc = (float)c, hw = (float)w;
    f[0] = make_float4(ha, hb, hc, hw);
    f[1] = make_float4((float)(a - (double)ha), (float)(b - (double)hb), (float)(c - (double)hc), (float)(w - (double)hw));
}

__global__ void k_pack_state(Dev d, double4 *dst, const double *src, int comps, int keep_w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nv) return;
    const double *x = src + (size_t)comps * i;
    const double w = comps == 4 ? x[3] : (keep_w ? load_state(d, dst, i).w : 0.0);
    put_slot(dst, i, d.mixed, x[0], x[1], x[2], w);
}

__global__ void k_unpack_state(Dev d, double *dst, const double4 *src, int comps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nv) return;
    const double4 v = load_state(d, src, i);
    double *x = dst + (size_t)comps * i;
    x[0] = v.x;
    x[1] = v.y;
    x[2] = v.z;
    if (comps == 4) x[3] = v.w;
}

void launch_pack_state(const Dev &d, double4 *dst, const double *staged, int comps, int keep_w, cudaStream_t s) {
    if (d.nv) k_pack_state<<<(d.nv + 255) / 256, 256, 0, s>>>(d, dst, staged, comps, keep_w);
}
void launch_unpack_state(const Dev &d, double *staged, const double4 *src, int comps, cudaStream_t s) {
    if (d.nv) k_unpack_state<<<(d.nv + 255) / 256, 256, 0, s>>>(d, staged, src, comps);
}

// ---------------------------------------------------------------- centre of mass
// updateCurrentCenterOfMass (VX3_VoxelyzeKernel.cu:477-493): mass-weighted mean
// of measured voxels, FP64.  Two passes with a fixed partition and order (so the
// result does not depend on scheduling): block (tile, robot) sums kComTile voxels
// of the robot into partial[(r * com_tiles + tile) * 4 + {x, y, z, mass}]; then one
// thread per robot and component adds the robot's tiles in tile order.
__global__ void __launch_bounds__(256) k_com_tiles(Dev d) {
    __shared__ double sh[4][256];
    const int r = blockIdx.y, tile = blockIdx.x;
    const RobotP &rp = d.rp[r];
    const int i0 = tile * kComTile;
    if (i0 >= rp.nv) return;  // (uniform) past the robot's voxels
    const int i1 = min(rp.nv, i0 + kComTile);
    double sx = 0, sy = 0, sz = 0, sm = 0;
    for (int i = i0 + threadIdx.x; i < i1; i += 256) {
        const int v = rp.voff + i;
        const VMat &m = d.vmat[d.vinfo[v].y >> 8];
        if (!m.is_measured) continue;
        const double mass = m.mass;
        const double4 p = load_state(d, d.pos, v);
        sx += mass * p.x;
        sy += mass * p.y;
        sz += mass * p.z;
        sm += mass;
    }
    sh[0][threadIdx.x] = sx; sh[1][threadIdx.x] = sy; sh[2][threadIdx.x] = sz; sh[3][threadIdx.x] = sm;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 4) d.com_part[((size_t)r * d.com_tiles + tile) * 4 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_com_sum(Dev d, double *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * d.nr) return;
    const int r = t >> 2, k = t & 3;
    const int nt = (d.rp[r].nv + kComTile - 1) / kComTile;
    const double *p = d.com_part + (size_t)r * d.com_tiles * 4;
    double acc = 0;
    for (int j = 0; j < nt; j++) acc += p[4 * j + k];
    double tot = 0;
    for (int j = 0; j < nt; j++) tot += p[4 * j + 3];
    if (k < 3) out[3 * r + k] = tot != 0 ? (1.0 / tot) * acc : 0.0;
}

void launch_com(const Dev &d, double *out, cudaStream_t s) {
    if (!d.nr) return;
    k_com_tiles<<<dim3((unsigned)d.com_tiles, (unsigned)d.nr), 256, 0, s>>>(d);
    k_com_sum<<<(4 * d.nr + 255) / 256, 256, 0, s>>>(d, out);
}

__global__ void k_or_status(Dev d, int r, int bits) { d.status[r] |= bits; }

void launch_or_status(const Dev &d, int robot, int bits, cudaStream_t s) { k_or_status<<<1, 1, 0, s>>>(d, robot, bits); }

}  // namespace vx3g
