// vx3g_adjoint.h -- state snapshots and buffers of the FP64 adjoint (vx3g_adjoint.cuh/.cu).
#pragma once

#include "vx3g_internal.h"

namespace vx3g {

// One copy of everything a step reads and changes (FP64 layout).  The recorded
// run keeps one every K steps (checkpoints); the backward pass recomputes the K
// states of an interval from its checkpoint into a store of K snapshots.
struct Snap {
    double4 *pos, *quat, *linmom, *angmom;
    uint2 *vinfo;
    float *tempe;     // 2*NV (both parity buffers)
    double *lstate;   // 9*NL, component-major
    float2 *strain;
    uint2 *linfo;
    double *T;        // 2*NR
    int *status;      // NR
};

struct AdjBufs {
    double *lv;     // 13 per voxel: dL/d(pos3, quat4 w,x,y,z, linMom3, angMom3)
    double *lown;   // 13 per voxel: the voxel pass's own part of dL/ds_k
    double *lF;     // 6 per voxel: dL/d(sum of link forces), dL/d(sum of link moments)
    double *lbs;    // per voxel: dL/d(base size) from the voxel pass
    double *lE;     // per voxel: dL/dE from the voxel pass
    double *lloc;   // 9 per link: dL/d(local state pos2, angle1v, angle2v)
    double *aslot;  // 9 per voxel-direction: a link's dL/d(pos3, quat4), dL/d(base size), dL/dE for that end
    double *gphase; // per voxel: accumulated dL/d(phase)
    double *glogE;  // per voxel: accumulated dL/d(log10 E)
    double *lcon;   // 3 per voxel: dL/d(contact force) of this step (the voxel pass consumes it)
    double *lcc;    // 8 per voxel: the contact adjoint's dL/d(pos3, linMom3, base size, E) for that voxel
    const double *w;         // 3 per robot: dL/dCOM
    const double *mass_tot;  // per robot: total mass of the measured voxels
    int parity;     // step parity of the step being reversed (time buffer)
};

// copies one state: n voxels, l links, r robots
void launch_snap_copy(const Snap &dst, const Snap &src, int nv, int nl, int nr, cudaStream_t st);
// reverse of one step, in three launches per step when steps are chained:
// slots(k) first; then per step voxel+link(k); then gather(k) fused with slots(k-1)
// (ss = nullptr for the last gather of a sweep)
void launch_adj_slots(const Dev &d, const Snap &s, const AdjBufs &a, cudaStream_t st);
void launch_adj_voxel_link(const Dev &d, const Snap &s, const AdjBufs &a, cudaStream_t st);
void launch_adj_gather_slots(const Dev &d, const Snap &sg, const Snap *ss, const AdjBufs &a, cudaStream_t st);
// with collisions: the contact forces of the step must be in d.contact (and the candidate
// lists valid) for the voxel adjoint; then the contact adjoint, then the gather
void launch_adj_contact(const Dev &d, const Snap &s, const AdjBufs &a, cudaStream_t st);
// dL/d(final state) for L = sum_r w_r . COM_r(end); also zeroes the link-state adjoint
void launch_adj_seed(const Dev &d, const AdjBufs &a, cudaStream_t st);

}  // namespace vx3g
