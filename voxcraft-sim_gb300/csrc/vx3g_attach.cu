// vx3g_attach.cu -- runtime link creation (attachment) for robots with EnableAttach.
//
// The reference decides attachment inside the surface-pair pass of each step
// (handle_collision_attachment, src/VX3/VX3_VoxelyzeKernel.cu:729-830): a pair that passed
// the envelope and direct-neighbour tests, whose voxels both allow attaching
// (enableAttach), are unfixed, of one Sticky material and more than five links apart
// (is_neighbor, :651-680), gets a new link along the dominant axis of voxel2's offset in
// voxel1's frame if both faces are free; the pair's contact of this step is taken back.
// All pairs run at once there, so which of two competing links is made depends on thread
// timing.  Here the pairs take their turns in the order of the serial loop over surface
// pairs (first ascending, second ascending below it), which makes the outcome unique:
//
//   k_attach_scan   one thread per collision-surface voxel v: every listed partner u < v
//                   (v is voxel1) is put through the tests that links made in this step
//                   cannot turn from fail to pass -- all but the free faces and the
//                   five-link distance, which only shrink.  Pairs that fail here fail in the
//                   serial order too; the survivors are marked in a per-voxel mask of list
//                   entries and a per-robot bitmap of voxels.
//   k_attach_commit one warp per robot: the marked pairs in serial order (voxels ascending,
//                   list entries ascending), each re-tested for free faces and, once the
//                   step has made a link, for the five-link distance, then linked.
//
// A new link takes the next slot of the robot's reserve (LF_RUNTIME, GONE until made): the
// device constructor's state after reset() (VX3_Link.cu:31-70) -- zero pos2/angles/strain,
// small-angle, no valid local velocity, isNewLink = SafetyGuard -- with the link material
// of the material pair, its faces set in both voxels' link bits and partner table, and
// both face slots zeroed (the step's voxel pass sums them: the new link's forces are 0
// until its first update, as after reset()).  The robot's contact lists and surface
// follow from the next step (isSurfaceChanged).
//
// enableAttach of each voxel is the AND of the attach conditions at its position after
// its step (gpu_update_voxels, :606-621), evaluated after the voxel pass.
//
// Arithmetic is FP64 and compiled with --fmad=false: the tests and the direction are the
// reference's expressions on the voxels' state (the hi+lo sums in mixed precision).
#include "vx3g_step.cuh"

namespace vx3g {

// is_neighbor(a, b, NULL, depth) for depth <= 5: b is reached from a over at most `depth`
// links without going straight back over the link just taken (the two faces of a link
// are opposite directions, so the way back from a face d is the face d ^ 1)
constexpr int kNeighborDepth = 5;
__device__ bool within_links(const Dev &d, int a, int b, int depth) {
    if (a == b) return true;
    int node[kNeighborDepth], from[kNeighborDepth], next[kNeighborDepth];
    int lv = 0;
    node[0] = a;
    from[0] = -1;
    next[0] = 0;
    while (lv >= 0) {
        if (next[lv] == 6) {
            lv--;
            continue;
        }
        const int dir = next[lv]++;
        const int x = node[lv];
        if (from[lv] >= 0 && dir == (from[lv] ^ 1)) continue;
        if (!((d.vinfo[x].y >> dir) & 1u)) continue;
        const int y = d.vnb[6 * (size_t)x + dir];
        if (y == b) return true;
        if (lv + 1 < depth) {
            lv++;
            node[lv] = y;
            from[lv] = dir;
            next[lv] = 0;
        }
    }
    return false;
}

// the link direction of the pair (voxel1 = v1): the dominant axis of ea = voxel2's offset
// rotated into voxel1's frame (ties to x, then y), rev = 1 when voxel2 lies on the
// negative side (voxel1 becomes the link's positive end)
__device__ __forceinline__ void attach_direction(const Dev &d, int v1, int v2, int *axis, int *rev) {
    const double4 p1 = load_state(d, d.pos, v1), p2 = load_state(d, d.pos, v2);
    const double4 q = load_state(d, d.quat, v1);
    const V3<double> e{p1.x - p2.x, p1.y - p2.y, p1.z - p2.z};
    const V3<double> ea = qrotinv(Q4<double>{q.x, q.y, q.z, q.w}, V3<double>{-e.x, -e.y, -e.z});
    const double fx = fabs(ea.x), fy = fabs(ea.y), fz = fabs(ea.z);
    if (fx >= fy && fx >= fz) {
        *axis = 0;
        *rev = ea.x < 0;
    } else if (fy >= fx && fy >= fz) {
        *axis = 1;
        *rev = ea.y < 0;
    } else {
        *axis = 2;
        *rev = ea.z < 0;
    }
}

// the tests a pair (voxel1 = v1 > v2 in voxel order) must pass whatever links the step
// makes before it, with the faces it would take free at the start of the pass
__device__ bool attach_candidate(const Dev &d, int v1, int v2) {
    const uint2 i1 = d.vinfo[v1], i2 = d.vinfo[v2];
    if ((i1.y >> 8) != (i2.y >> 8)) return false;  // one material (the same palette entry)
    const VMat &m = d.vmat[i1.y >> 8];
    if (m.alm < 0 || m.fixed) return false;        // Sticky (of an attaching robot), not Fixed
    if (!d.vatt[v1] || !d.vatt[v2]) return false;  // enableAttach
    if ((i2.y & VF_LINKMASK) == VF_LINKMASK || (d.vgone && d.vgone[v2])) return false;  // not on the surface
    // the envelope test of the collision half (:688-699)
    const double4 p1 = load_state(d, d.pos, v1), p2 = load_state(d, d.pos, v2);
    const double b1 = (p1.w + p1.w + p1.w) / 3.0f, b2 = (p2.w + p2.w + p2.w) / 3.0f;  // baseSizeAverage
    const V3<double> diff{p1.x - p2.x, p1.y - p2.y, p1.z - p2.z};
    const double wd = (b1 + b2) * 0.625;
    if (diff.x > wd || diff.x < -wd) return false;
    if (diff.y > wd || diff.y < -wd) return false;
    if (diff.z > wd || diff.z < -wd) return false;
    if (len(diff) > wd) return false;
    if (linked_to(d, v1, v2)) return false;  // direct neighbours: neither contact nor link
    if (within_links(d, v1, v2, kNeighborDepth)) return false;
    int axis, rev;
    attach_direction(d, v1, v2, &axis, &rev);
    const int f1 = 2 * axis + rev, f2 = 2 * axis + (rev ^ 1);
    return !((i1.y >> f1) & 1u) && !((i2.y >> f2) & 1u);
}

__global__ void k_attach_scan(Dev d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.ns) return;
    const int v = d.csurf[s];
    const uint2 vi = d.vinfo[v];
    const int r = (int)vi.x;
    const RobotP &rp = d.rp[r];
    if (!rp.attach) return;
    unsigned long long mask = 0ull;
    const VMat &m = d.vmat[vi.y >> 8];
    if (d.status[r] == 0 && m.alm >= 0 && !m.fixed && d.vatt[v] && (vi.y & VF_LINKMASK) != VF_LINKMASK &&
        !(d.vgone && d.vgone[v])) {
        const int n = d.nnb[s];
        const int *lst = d.nbr + s;
        for (int k = 0; k < n; k++) {
            const int u = lst[(size_t)k * d.ns];  // ascending partners
            if (u >= v) break;                    // v is voxel1 of its pairs with earlier voxels
            if (attach_candidate(d, v, u)) mask |= 1ull << k;
        }
    }
    d.amask[s] = mask;
    if (mask) {
        const int i = s - rp.soff;
        atomicOr(&d.abits[rp.abit + (i >> 5)], 1u << (i & 31));
        d.aflag[r] = 1;
    }
}

// a new link between v1 (voxel1) and v2 along `axis` (rev: v1 is the positive end) in the
// robot's next reserve slot; false when the reserve is used up
__device__ bool make_link(const Dev &d, const RobotP &rp, int r, int v1, int v2, int axis, int rev) {
    if (d.anum[r] >= rp.acap) {
        atomicOr(&d.status[r], kStatusLinkCapacity);
        return false;
    }
    const int l = rp.ares + d.anum[r]++;
    const int neg = rev ? v2 : v1, pos = rev ? v1 : v2;
    const int lm = d.vmat[d.vinfo[v1].y >> 8].alm;
    d.ends[l] = make_int2(neg, pos);
    d.linfo[l] = make_uint2((unsigned)r, (uint32_t)axis | LF_SMALL | LF_RUNTIME | ((uint32_t)lm << 8));
    const size_t NL = (size_t)d.nl;
    if (d.mixed) {
        mixed_lstate_a(d)[l] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        mixed_lstate_b(d)[l] = make_float2(0.0f, 0.0f);
        float *c = mixed_lstate_c(d);
        for (int k = 0; k < 3; k++) c[k * NL + l] = 0.0f;
    } else {
        double *ls = (double *)d.lstate;
        for (int k = 0; k < 9; k++) ls[k * NL + l] = 0.0;
    }
    d.strain[l] = make_float2(0.0f, 0.0f);
    if (d.soff) d.soff[l] = 0.0f;
    d.lnew[l] = rp.guard;
    d.vinfo[neg].y |= 1u << (2 * axis);      // the negative end's face toward +axis
    d.vinfo[pos].y |= 1u << (2 * axis + 1);  // the positive end's face toward -axis
    d.vnb[6 * (size_t)neg + 2 * axis] = pos;
    d.vnb[6 * (size_t)pos + 2 * axis + 1] = neg;
    const size_t sn = (size_t)(2 * axis) * d.nv + neg, sp = (size_t)(2 * axis + 1) * d.nv + pos;
    if (d.mixed) {
        const V3<float> z{0, 0, 0};
        store_slot_mx(d, 2 * axis, neg, z, z);
        store_slot_mx(d, 2 * axis + 1, pos, z, z);
    } else {
        Slot<double> *S = (Slot<double> *)d.slots;
        S[sn] = Slot<double>{{0, 0, 0}, {0, 0, 0}};
        S[sp] = Slot<double>{{0, 0, 0}, {0, 0, 0}};
    }
    d.srf[r] = 1;  // isSurfaceChanged: the surface and the contact lists follow next step
    return true;
}

__global__ void k_attach_commit(Dev d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= d.narob) return;
    const int r = d.arob[w];
    const RobotP &rp = d.rp[r];
    if (!d.aflag[r]) {
        if (lane == 0) d.acnt[r] = 0;
        return;
    }
    int made = 0;  // lane 0's count
    bool full = false;
    const int nwords = (rp.ns + 31) >> 5;
    for (int w0 = 0; w0 < nwords; w0 += 32) {
        const int wi = w0 + lane;
        const unsigned bits = wi < nwords ? d.abits[rp.abit + wi] : 0u;
        unsigned any = __ballot_sync(0xffffffffu, bits != 0u);
        while (any) {  // words with marked voxels, ascending
            const int src = __ffs(any) - 1;
            any &= any - 1;
            const unsigned wb = __shfl_sync(0xffffffffu, bits, src);
            if (lane == 0) {
                unsigned b = wb;
                while (b) {
                    const int bit = __ffs(b) - 1;
                    b &= b - 1;
                    const int s = rp.soff + ((w0 + src) << 5) + bit;
                    const int v = d.csurf[s];
                    unsigned long long mask = d.amask[s];
                    d.amask[s] = 0ull;
                    while (mask && !full) {
                        const int k = __ffsll((long long)mask) - 1;
                        mask &= mask - 1;
                        const int u = d.nbr[s + (size_t)k * d.ns];
                        int axis, rev;
                        attach_direction(d, v, u, &axis, &rev);
                        const int f1 = 2 * axis + rev, f2 = 2 * axis + (rev ^ 1);
                        if (((d.vinfo[v].y >> f1) & 1u) || ((d.vinfo[u].y >> f2) & 1u)) continue;
                        if (made > 0 && within_links(d, v, u, kNeighborDepth)) continue;
                        if (!make_link(d, rp, r, v, u, axis, rev)) full = true;
                        else made++;
                    }
                }
            }
        }
        if (bits) d.abits[rp.abit + wi] = 0u;
    }
    if (lane == 0) {
        d.acnt[r] = made;
        d.aflag[r] = 0;
    }
}

void launch_attach(const Dev &d, cudaStream_t s) {
    if (!d.narob || !d.ns) return;
    k_attach_scan<<<(d.ns + 255) / 256, 256, 0, s>>>(d);
    k_attach_commit<<<(d.narob + 3) / 4, 128, 0, s>>>(d);
}

// gpu_update_voxels (:606-621): after a voxel's step, enableAttach = every attach condition
// > 0 at its new position, the step's start time and the robot's voxel count; Fixed and
// removed voxels are not stepped and keep theirs
__global__ void k_attach_cond(Dev d, int parity) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d.nv) return;
    const uint2 vi = d.vinfo[v];
    const int r = (int)vi.x;
    const RobotP &rp = d.rp[r];
    if (!rp.attach || (vi.y & VF_FIXED) || d.status[r] != 0) return;
    const double4 p = load_state(d, d.pos, v);
    const double t = d.T[(size_t)parity * d.nr + r];
    bool ok = true;
    for (int k = 0; k < 5 && ok; k++)
        if (rp.acond[k] >= 0 && !(math_eval(d.ftok + rp.acond[k], p.x, p.y, p.z, t, (double)rp.nv) > 0)) ok = false;
    d.vatt[v] = ok ? 1 : 0;
}

void launch_attach_cond(const Dev &d, int parity, cudaStream_t s) {
    if (d.any_acond && d.nv) k_attach_cond<<<(d.nv + 255) / 256, 256, 0, s>>>(d, parity);
}

}  // namespace vx3g
