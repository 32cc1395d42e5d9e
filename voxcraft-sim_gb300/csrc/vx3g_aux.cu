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

// ---------------------------------------------------------------- collision
// The reference tests every pair of surface voxels each step (gpu_update_attach,
// VX3_VoxelyzeKernel.cu:833-843).  Here each surface voxel keeps a list of the
// surface voxels of its robot that were within cutoff + skin when the list was
// built (a Verlet list: uniform grid of cell edge cutoff + skin, hashed, counting
// sort).  The lists are rebuilt in a step where any voxel has moved more than
// half the skin since the last build, so every pair within the cutoff is in the
// lists; each step the reference's exact test (handle_collision_attachment,
// :682-704) runs on the listed pairs and the contact forces of VX3_Collision
// (VX3_Collision.cu:3-31) are summed in ascending partner order -- the order in
// which the reference's serial pair loop accumulates them -- without atomics.
// The candidate set is therefore the reference's, pair for pair.
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

// 1. has any voxel moved more than half the skin since the last build?
__global__ void k_coll_check(Dev d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.ns) return;
    const int v = d.csurf[s];
    const float4 p = pos_f(d, v), q = d.cref[s];  // q.w: squared displacement limit
    const float ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
    if (ex * ex + ey * ey + ez * ez > q.w) atomicOr(d.cflag, 1);
}

__global__ void k_coll_clear(Dev d) {
    if (!*d.cflag) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.hsize; i += gridDim.x * blockDim.x) d.hcount[i] = 0;
}

__global__ void k_coll_bin(Dev d) {
    if (!*d.cflag) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.ns) return;
    const int v = d.csurf[s];
    const int r = (int)d.vinfo[v].x;
    const double ic = d.rp[r].inv_list_cell;
    const double4 p = load_state(d, d.pos, v);
    const int4 c = make_int4((int)floor(p.x * ic), (int)floor(p.y * ic), (int)floor(p.z * ic), r);
    d.ccell[s] = c;
    d.cposf[s] = make_float4((float)p.x, (float)p.y, (float)p.z, 0.0f);
    atomicAdd(&d.hcount[cell_hash(c.x, c.y, c.z, c.w, d.hsize - 1)], 1);
}

// exclusive scan of hcount in blocks of 1024 (hsize is a multiple of 1024)
__global__ void __launch_bounds__(1024) k_scan_blocks(Dev d) {
    if (!*d.cflag) return;
    __shared__ int sh[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int x = d.hcount[i];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int y = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += y;
        __syncthreads();
    }
    d.hstart[i] = sh[threadIdx.x] - x;
    if (threadIdx.x == 1023) d.hblock[blockIdx.x] = sh[1023];
}

__global__ void __launch_bounds__(1024) k_scan_add(Dev d) {
    if (!*d.cflag) return;
    __shared__ int base;
    if (threadIdx.x < 32) {
        int acc = 0;
        for (int b = threadIdx.x; b < (int)blockIdx.x; b += 32) acc += d.hblock[b];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) base = acc;
    }
    __syncthreads();
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int v = d.hstart[i] + base;
    d.hstart[i] = v;
    d.hfill[i] = v;
}

__global__ void k_coll_scatter(Dev d) {
    if (!*d.cflag) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.ns) return;
    const int4 c = d.ccell[s];
    const int slot = atomicAdd(&d.hfill[cell_hash(c.x, c.y, c.z, c.w, d.hsize - 1)], 1);
    d.hsorted[slot] = s;
}

// 2. list every unlinked surface voxel of the same robot within cutoff + skin, ascending
__global__ void k_coll_list(Dev d) {
    if (!*d.cflag) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.ns) return;
    const int v = d.csurf[s];
    const int r = (int)d.vinfo[v].x;
    const int4 c = d.ccell[s];
    const float4 pf = d.cposf[s];
    const RobotP &rp = d.rp[r];
    // 1e-3 relative margin: FP32 positions up to ~100 m from the origin lose no true pair
    const float cut = (float)(rp.cell_size + rp.skin) * 1.001f, cut2 = cut * cut;
    const bool fixed = (d.vinfo[v].y & VF_FIXED) != 0;
    const short4 ij = d.ijk[v];
    int *out = d.nbr + s;  // entry j at out[j*ns]: slot-major, so list reads coalesce across a warp
    const size_t ns = (size_t)d.ns;
    int nc = 0;
    bool overflow = false;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int cx = c.x + dx, cy = c.y + dy, cz = c.z + dz;
                const unsigned h = cell_hash(cx, cy, cz, r, d.hsize - 1);
                const int b = d.hstart[h], n = d.hcount[h];
                for (int k = 0; k < n; k++) {
                    const int t = d.hsorted[b + k];
                    if (t == s) continue;
                    const int4 ct = d.ccell[t];
                    if (ct.x != cx || ct.y != cy || ct.z != cz || ct.w != r) continue;
                    const float4 tf = d.cposf[t];
                    const float ex = tf.x - pf.x, ey = tf.y - pf.y, ez = tf.z - pf.z;
                    if (ex * ex + ey * ey + ez * ez > cut2) continue;
                    const int u = d.csurf[t];
                    // is_neighbor depth 1 (VX3_VoxelyzeKernel.cu:651-680): linked <=> face-adjacent in the lattice
                    const short4 ik = d.ijk[u];
                    if (abs(ik.x - ij.x) + abs(ik.y - ij.y) + abs(ik.z - ij.z) == 1) continue;
                    if (fixed && (d.vinfo[u].y & VF_FIXED)) continue;
                    if (nc == kNbrCap) {
                        overflow = true;
                        continue;
                    }
                    // the list holds voxel indices in ascending order: csurf is ascending, so
                    // this is the ascending surface-index order of the reference's pair loop
                    int j = nc++;
                    while (j > 0 && out[(j - 1) * ns] > u) {
                        out[j * ns] = out[(j - 1) * ns];
                        j--;
                    }
                    out[j * ns] = u;
                }
            }
    if (overflow) atomicOr(&d.status[r], 2);
    d.nnb[s] = nc;
    const float lim = 0.49f * (float)rp.skin;  // rebuild when a voxel has moved farther than this
    d.cref[s] = make_float4(pf.x, pf.y, pf.z, lim * lim);
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
    if (s == 0) *d.cflag = 0;  // the rebuild (if any) is done; the next check starts clear
    if (s >= d.ns) return;
    const int v = d.csurf[s];
    const int r = (int)d.vinfo[v].x;
    if (d.status[r] != 0) return;
    const int n = d.nnb[s];
    const int *lst = d.nbr + s;  // slot-major: entry k at lst[k*ns]
    const size_t ns = (size_t)d.ns;
    V3<double> acc{0, 0, 0};
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
            if (u < v) acc = add(acc, pair_force(d, v, u, bsa, bu));    // v.contactForce += force
            else acc = add(acc, neg(pair_force(d, u, v, bu, bsa)));      // v.contactForce += -force
        }
    }
    d.contact[v] = make_double4(acc.x, acc.y, acc.z, 0.0);
}

// 1'. the displacement check inside a CUDA graph: the last block to finish sets the
// conditional node that runs the list rebuild (threadfence-reduction pattern, no wait)
__global__ void k_coll_check_cond(Dev d, cudaGraphConditionalHandle h) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < d.ns) {
        const int v = d.csurf[s];
        const float4 p = pos_f(d, v), q = d.cref[s];  // q.w: squared displacement limit
        const float ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
        if (ex * ex + ey * ey + ez * ez > q.w) atomicOr(d.cflag, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(d.ccount, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            cudaGraphSetConditional(h, atomicOr(d.cflag, 0) ? 1u : 0u);
            *d.ccount = 0;
        }
    }
}

static void enqueue_rebuild(const Dev &d, int g, cudaStream_t s) {
    k_coll_clear<<<152 * 4, 256, 0, s>>>(d);
    k_coll_bin<<<g, 256, 0, s>>>(d);
    k_scan_blocks<<<d.hsize / 1024, 1024, 0, s>>>(d);
    k_scan_add<<<d.hsize / 1024, 1024, 0, s>>>(d);
    k_coll_scatter<<<g, 256, 0, s>>>(d);
    k_coll_list<<<g, 256, 0, s>>>(d);
}

cudaError_t launch_collision(const Dev &d, cudaStream_t s, cudaStream_t side) {
    if (!d.ns) return cudaSuccess;
    const int g = (d.ns + 255) / 256;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cs);
    if (e != cudaSuccess) return e;
    if (cs == cudaStreamCaptureStatusActive && side) {
        // in a graph: check, then IF(rebuild due) { rebuild }, then the narrow phase
        cudaGraph_t graph;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        if ((e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, nullptr, nullptr, nullptr)) != cudaSuccess) return e;
        cudaGraphConditionalHandle h;
        if ((e = cudaGraphConditionalHandleCreate(&h, graph, 0, 0)) != cudaSuccess) return e;
        k_coll_check_cond<<<g, 256, 0, s>>>(d, h);
        if ((e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &nd)) != cudaSuccess) return e;
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeIf;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        if ((e = cudaGraphAddNode(&node, graph, deps, nullptr, nd, &p)) != cudaSuccess) return e;
        cudaGraph_t body = p.conditional.phGraph_out[0];
        if ((e = cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
            cudaSuccess)
            return e;
        enqueue_rebuild(d, g, side);
        if ((e = cudaStreamEndCapture(side, &body)) != cudaSuccess) return e;
        if ((e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
            cudaSuccess)
            return e;
    } else {
        // outside a graph: every rebuild kernel runs and returns at once unless the flag is set
        cudaMemsetAsync(d.cflag, 0, sizeof(int), s);
        k_coll_check<<<g, 256, 0, s>>>(d);
        enqueue_rebuild(d, g, s);
    }
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
// of measured voxels, FP64, one block per robot with a fixed reduction order.
__global__ void __launch_bounds__(256) k_com(Dev d, double *out) {
    __shared__ double sh[4][256];
    const int r = blockIdx.x;
    const RobotP &rp = d.rp[r];
    double sx = 0, sy = 0, sz = 0, sm = 0;
    for (int i = threadIdx.x; i < rp.nv; i += 256) {
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
    if (threadIdx.x == 0) {
        const double tot = sh[3][0];
        double inv = tot != 0 ? 1.0 / tot : 0.0;
        out[3 * r] = tot != 0 ? inv * sh[0][0] : 0.0;
        out[3 * r + 1] = tot != 0 ? inv * sh[1][0] : 0.0;
        out[3 * r + 2] = tot != 0 ? inv * sh[2][0] : 0.0;
    }
}

void launch_com(const Dev &d, double *out, cudaStream_t s) {
    if (d.nr) k_com<<<d.nr, 256, 0, s>>>(d, out);
}

__global__ void k_or_status(Dev d, int r, int bits) { d.status[r] |= bits; }

void launch_or_status(const Dev &d, int robot, int bits, cudaStream_t s) { k_or_status<<<1, 1, 0, s>>>(d, robot, bits); }

}  // namespace vx3g
