// vx3g_internal.h -- device data layout shared by the host code and kernels.
//
// HBM layout (all arrays packed over the whole batch; robots back to back in
// the reference's voxel order, x fastest):
//   voxel v : pos[v]    double4 {x, y, z, baseSize}   baseSize = nomSize*(1+tempe*cte) of the
//                                                      current step (VX3_Voxel::baseSize, VX3_Voxel.h:96-100)
//             quat[v]   double4 {w, x, y, z}
//             linmom[v] double4 {x, y, z, -}, angmom[v] double4 {x, y, z, -}
//             vinfo[v]  uint2 {robot, flags | vmat<<8}
//             contact[v] double4 (float4 in mixed precision), tempe[v] float, phase[v] double,
//             ijk[v] short4
//   link l  : ends[l] int2 {neg, pos}, linfo[l] uint2 {robot, flags | lmat<<8},
//             local state (pos2, angle1v, angle2v): 9 component-major arrays of R,
//             strain[l] float2 {strain, maxStrain}
//   slots   : slot[dir*NV + v] = {force, moment} of the link attached to voxel v in
//             direction dir (X_POS..Z_NEG), written by the link pass, read in order 0..5 by
//             the voxel pass (the summation order of VX3_Voxel::force/moment).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vx3g {

// voxel flag bits (low 8 bits of vinfo.y)
enum : uint32_t {
    VF_LINKMASK = 0x3F,   // bit d set: a link exists in direction d
    VF_STATIC = 1u << 6,  // FLOOR_STATIC_FRICTION
    VF_FIXED = 1u << 7,   // material Fixed (voxel never steps)
};
// link flag bits (low 8 bits of linfo.y)
enum : uint32_t {
    LF_AXIS = 0x3,
    LF_SMALL = 1u << 2,       // smallAngle
    LF_LVV = 1u << 3,         // LOCAL_VELOCITY_VALID
    LF_BOTH_FIXED = 1u << 4,  // both ends fixed: gpu_update_links skips the link
    LF_GONE = 1u << 5,        // detached (gpu_update_detach): no longer updated, no voxel's link
    LF_RUNTIME = 1u << 6,     // made by attachment, or a reserve slot for one (GONE until made)
};

// the actuation argument 2*3.1415926f*(t/period + phase) (gpu_update_temperature,
// VX3_VoxelyzeKernel.cu:625-650) in cycles of 2*pi: (t/period + phase) * kCycle
constexpr double kCycle = (double)(2 * 3.1415926f) * (1.0 / 6.283185307179586);

// robot status bit (VX3G_ROBOT_LINK_CAPACITY): attachment found the robot's link reserve used up
constexpr int kStatusLinkCapacity = 8;

struct VMat {  // one voxel material (global index), constants as the reference derives them
    float mass, mass_inv, mom_inv;
    float c_glob;      // zetaGlobal*_2xSqMxExS          globalDampingTranslateC
    float c_glob_rot;  // zetaGlobal*_2xSqIxExSxSxS      globalDampingRotateC
    float c_col;       // zetaCollision*_2xSqMxExS       collisionDampingTranslateC
    float grav_force;  // -_mass*9.80665f*gravMult       gravityForce
    float pstiff;      // (float)(2*E*nomSize)           penetrationStiffness
    float mu_s, mu_k, cte;
    float dmc;         // 2*_sqrtMass*zetaInternal       dampingMultiplier numerator
    float E, nu;
    float nom_hi, nom_lo;  // nomSize as an FP32 hi/lo pair (mixed precision)
    int fixed, is_measured;
    double nom_size;
    double thermal_on_after;
    int toa_pos;       // thermal_on_after > 0: only then is it compared with the time (in FP64)
    int pacemaker;     // isPaceMaker
    double pace_period, sig_decay, sig_delay, inactive;  // PaceMakerPeriod, signalValueDecay, signalTimeDelay, inactivePeriod
    int alm;           // Sticky material of a robot with EnableAttach: the link material of its runtime
                       // links (VX3_VoxelyzeKernel::combinedMaterial of the pair); -1 otherwise
};

struct LMat {  // one link material (global index), oriented: (negative end, positive end) materials
    float E, nu, eHat, eps_fail;
    float a1, a2, b1, b2, b3;
    float sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp;
    float area, tss;  // transverse area / strain sum frozen at link creation
    float dmcN, dmcP; // the ends' dampingMultiplier numerators 2*sqrt(m)*zetaInternal (VMat.dmc)
    int fixN, fixP;   // the ends' materials are Fixed
    int lin;          // 1: linear model (VX3_Material::linear); 0: data points d.ss[sso .. sso+ssn)
    int ssn, sso;     // stress-strain points of a non-linear model: (0,0), then the model's from (0,0) on
};

struct RobotP {
    double vox_size, temp_amp, temp_period, inv_period, dt_frac;
    float cyc_rate, amp_f;  // mixed precision: actuation cycles per second (inv_period * kCycle), amplitude
    double cell_size;      // upper bound of the envelope cutoff (bsa1+bsa2)*0.625
    double skin;           // Verlet skin of the contact-candidate lists
    double inv_list_cell;  // 1 / (cell_size + skin): grid used to build the lists
    int voff, nv, loff, nl, soff, ns;
    int floor, vary_temp, expansion, collision;
    int lchunks;  // > 0: lists built in shared memory (coll_list_robots), in this many chunks; 0: global hashed grid
    int ff[3] = {-1, -1, -1};  // force-field programs (x, y, z): token offset in Dev::ftok, or -1 for none
    int ff_pos = 0;            // 1: a force-field program reads the voxel position
    int ff_any = 0;            // 1: the robot has a force field (k_extra_forces fills Dev::ffv)
    int cilia = 0;             // 1: EnableCilia with some cilia voxel (k_extra_forces fills Dev::cfv)
    int detach = 0;            // 1: EnableDetach (failed links leave)
    int remove = 0;            // 1: SecondaryExperiment with a material that leaves (k_remove)
    int dyn = 0;               // detach || remove: the surface follows the link table
    int bcs = 0;               // 1: some voxel has a boundary-condition external (Dev::vext)
    int signals = 0;           // 1: EnableSignals (k_signals; the cilia force reads the signal)
    int attach = 0;            // 1: EnableAttach (k_attach_scan / k_attach_commit)
    int acond[5] = {-1, -1, -1, -1, -1};  // attach-condition programs: token offset in Dev::ftok, or -1
    int guard = 0;             // SafetyGuard: a runtime link's first updates scaled by 0.01
    int ares = 0, acap = 0;    // the robot's reserve of runtime links: first link index, size
    int abit = 0;              // first word of its collision-surface bitmap (Dev::abits)
};

// a voxel's boundary-condition external (VX3_External): fixed DOFs with their prescribed
// translation and rotation, applied force and moment
struct ExtBC {
    double4 t;   // extTranslation {x, y, z, -}
    double4 q;   // _extRotationQ {w, x, y, z}
    float f[3];  // extForce
    float m[3];  // extMoment
    int dof;     // fixed DOFs: bits 0-2 translation x, y, z; 3-5 rotation x, y, z
    int pad;
};
enum : int { EXT_T = 0x7, EXT_R = 0x38, EXT_ALL = 0x3F };

// grid of one robot on the large-robot list path (bounding box in cells of cutoff + skin)
struct GridP {
    float mnx, mny, mnz, ic;  // bounding-box corner, 1 / cell edge
    int gx, gy, gz, base;     // cells per axis, first bucket (dense grid)
};

// a math-tree token as vx3g_math_token lays it out (op, reserved, value)
struct MathTok {
    int op, reserved;
    double value;
};

template <class R> struct Slot { R f[3]; R m[3]; };

constexpr int kNbrCap = 64;  // contact candidates kept per collision-surface voxel
constexpr int kComTile = 2048;  // voxels per block of the centre-of-mass reduction
// per-robot list build in shared memory: robots with at most kLocalListMax collision-surface
// voxels and lattice coordinates below 512, chunks of kLocalListChunk voxels (ten per warp,
// three threads per voxel)
constexpr int kLocalListMax = 6144;
constexpr int kLocalListThreads = 512;
constexpr int kLocalListChunk = kLocalListThreads / 32 * 10;
// packed lattice word of a voxel on that path: x | y << 10 | z << 20 | fixed << 31 (coordinates
// below 512, so the difference of two packed words is face-adjacent iff it is +-1, +-2^10 or +-2^20)
constexpr unsigned kPackMask = 0x3fffffffu, kPackFixed = 0x80000000u;
// set while a voxel of a robot whose surface follows its link table has six links, or
// after it was removed: it neither lists nor is listed
constexpr unsigned kPackInterior = 0x40000000u;
constexpr int kLocalHash = 4096;  // buckets of the shared-memory grid (power of two)
// polls (each with a 32 ns back-off) after which a CTA waiting at a grid barrier of
// k_coll_prepare gives up, records the error and returns
constexpr unsigned kBarrierPolls = 1u << 22;

struct Dev {
    // voxels
    double4 *pos, *quat, *linmom, *angmom, *contact;
    float *tempe;
    double *phase;
    uint2 *vinfo;
    short4 *ijk;
    // links
    int2 *ends;
    uint2 *linfo;
    void *lstate;   // 9*NL of R, component-major
    float2 *strain;
    float *soff;    // per link: strainOffset of a non-linear link material (VX3_Link.cu:231-258), or NULL
    const float2 *ss;  // stress-strain points {strain, stress} of the non-linear link materials
    void *slots;    // 6*NV Slot<R>
    // robots
    const RobotP *rp;
    float *dt;
    double *T;      // [2][NR] time, double-buffered by step parity
    // mixed precision: [2][NR] the actuation cycles frac(T * inv_period * kCycle) as an FP32
    // hi + lo pair, written with T; per voxel the phase cycles frac(phase * kCycle) as hi + lo
    // (NULL in FP64)
    float2 *tcyc, *phc;
    int *status;
    // materials
    const VMat *vmat;
    const LMat *lmat;
    // collision
    int *csurf;     // collision surface list (global voxel index), NS entries
    int4 *ccell;    // x: the bucket of a collision-surface voxel in the large-robot grid (-1: not binned)
    float4 *cposf;  // FP32 position per collision-surface voxel, written by the displacement check
    // mixed precision: per voxel, the contact record of the collision-surface voxels for this
    // step, written by the displacement check: [2v] {position hi x, y, z; base size},
    // [2v+1] {position lo x, y, z; penetrationStiffness} -- one aligned 32-byte sector per
    // contact candidate, four voxels to a cache line -- and [2NV+v] {velocity (linMom hi /
    // m); collision damping}, read for the candidates in contact (NULL in FP64)
    float4 *crec;
    unsigned *cpk;  // per collision-surface voxel: packed lattice word (kPackMask, kPackFixed; shared-memory path)
    float4 *cref;   // position at the last list build (w: squared displacement that forces a rebuild)
    int *nbr;       // candidate lists, slot-major [kNbrCap][NS]: partner voxel indices, ascending
    int *nnb;       // candidate count per collision-surface voxel
    int *cflag;     // [1 + NR]: [0] some robot's lists are rebuilt this step, [1 + r] robot r's are
    unsigned *gbar;  // [3] grid barrier of k_coll_prepare: arrivals, generation, poll limit
    int2 *lwork;    // [NR] robots whose lists are rebuilt in shared memory this step: (robot, first chunk)
    unsigned long long *lwork_ctr;  // (robots << 32) | chunks listed in lwork; cleared by the narrow phase
    int lmax;       // most collision-surface voxels of a robot on the shared-memory path (0: none)
    int cgrid;      // CTAs of the cooperative k_coll_prepare (all resident)
    int glgrid;     // CTAs of k_grid_list (the lists of robots on the global hashed grid), 0: none
    int nhash;      // collision-surface voxels on the global hashed-grid path
    int *hcount, *hstart, *hfill, *hblock;  // bucket counts, starts, ends (after the scatter), segment sums
    unsigned *gbox;      // [NR][6] bounding-box accumulators of the large-robot grid (order-preserving keys)
    GridP *ggrid;        // [NR] that grid's corner, cell edge, size and first bucket
    int *gmode;          // [3] reach of a dense grid's neighbourhood in cells (1), 0 hashed; buckets in use
    float4 *spos;        // [NS] binned voxels in cell order: FP32 position, voxel index in w
    short4 *sij;         // [NS] their lattice coordinates, w = fixed
    int *ssurf;          // [NS] their collision-surface index
    int hsize;      // power of two
    int *err;       // device error word
    const MathTok *ftok;  // force-field programs of all robots, back to back
    double4 *ffv;         // per voxel: this step's force-field force (robots with ff_any), or NULL
    double4 *cil;         // per voxel: BaseCiliaForce + 0 * ShiftCiliaForce, material Cilia (robots with cilia)
    double *cil_on;       // per voxel: the time cilia switch on (+inf: never; interior or Cilia 0)
    double4 *cfv;         // per voxel: this step's CiliaForce * Cilia (robots with cilia), or NULL
    double4 *cils;        // per voxel: ShiftCiliaForce (robots with cilia and signals), or NULL
    // signals: per voxel {localSignal, localSignaldt, packmakerNextPulse, inactiveUntil, pending
    // value, pending activeTime} (VX3_Voxel.h:304-309), and the voxel across each direction's
    // link (-1: none); robots with signals: sigrob[nsigrob]
    double *sig;
    int *vnb;
    int *sigrob;
    int nsigrob;
    int *srf;             // [NR] a link of the robot detached or a voxel left this step: rebuild its lists next step
    int any_detach;       // some robot has EnableDetach
    int any_remove;       // some robot removes voxels (k_remove)
    int any_dyn;          // some robot's surface follows its link table (detach or removal)
    unsigned char *vgone; // per voxel: removed (removeVoxels), or NULL when no robot removes voxels
    double *rm_at;        // per voxel: the time after which it is removed (+inf: never), or NULL
    const ExtBC *ext;  // boundary-condition externals, or NULL when no robot has any
    int *vext;         // per voxel: its index in ext, or -1 (NULL when no robot has any)
    int *xbc;          // the voxels with an external, in voxel order (mixed precision: k_voxels_bc_mixed)
    int nxbc;
    // attachment (robots with EnableAttach): per voxel enableAttach (VX3_Voxel.h:302); per link
    // isNewLink (VX3_Link.h:240, runtime links only); per collision-surface voxel the candidate
    // list entries that passed the parallel tests this step (bit k: entry k), with a bitmap of
    // those voxels per robot; per robot: a pair passed this step, runtime links made so far,
    // links made this step; the robots with EnableAttach
    unsigned char *vatt;
    int *lnew;
    unsigned long long *amask;
    unsigned *abits;
    int *aflag, *anum, *acnt;
    int *arob;
    int narob;
    int any_acond;     // some robot has an attach condition (k_attach_cond after the voxel pass)
    double *com_part;  // [NR][com_tiles][4] partial sums of the centre of mass
    int com_tiles;     // tiles of kComTile voxels of the largest robot
    int nv, nl, nr, ns;
    int mixed;      // 1: voxel state is compensated FP32 (see below)
};

// In the mixed-precision layout each 32-byte double4 slot of pos/quat/linmom/angmom
// holds two float4 {hi, lo}: the value is hi + lo (an unevaluated sum of two
// floats, ~48 significant bits), advanced with two-sum arithmetic.
#ifdef __CUDACC__
__device__ __forceinline__ double4 load_state(const Dev &d, const double4 *a, int v) {
    if (!d.mixed) return a[v];
    const float4 *f = reinterpret_cast<const float4 *>(a) + 2 * (size_t)v;
    const float4 h = f[0], l = f[1];
    return make_double4((double)h.x + l.x, (double)h.y + l.y, (double)h.z + l.z, (double)h.w + l.w);
}
#endif

// launchers (defined in the .cu files)
void launch_links_fp64(const Dev &d, cudaStream_t s);
void launch_voxels_fp64(const Dev &d, int parity, cudaStream_t s);
// launch shapes of the mixed-precision passes (vx3g_mixed.cu), chosen by vx3g_autotune
struct LaunchShape { int threads, min_blocks; };
constexpr int kMixedShapes = 6;
extern const LaunchShape kLinkShapes[kMixedShapes], kVoxelShapes[kMixedShapes];
// pdl = false when the kernel before it wrote link info (removal): no early start
void launch_links_mixed(const Dev &d, cudaStream_t s, int shape = 0, bool pdl = true);
// pdl = false when the kernel before it wrote voxel info (detach): no early start
void launch_voxels_mixed(const Dev &d, int parity, cudaStream_t s, int shape = 0, bool pdl = true);
void launch_init_temperature(const Dev &d, int mixed, cudaStream_t s);
// the mixed-precision voxel pass of the voxels with a boundary-condition external (after
// the main pass, which skips them)
void launch_voxels_bc_mixed(const Dev &d, int parity, cudaStream_t s);
void launch_init_temperature_mixed(const Dev &d, cudaStream_t s);
void launch_dt(const Dev &d, double *maxfreq2_scratch, cudaStream_t s);
// surface-voxel collision of one step: displacement check and list rebuild (one
// cooperative kernel), then the narrow phase
cudaError_t launch_collision(const Dev &d, cudaStream_t s);
cudaError_t launch_coll_prepare(const Dev &d, cudaStream_t s);  // the check / rebuild kernel alone
// the force field (d.ffv) and the cilia force (d.cfv) of the voxels of robots that have
// them, at the start of the step of the given time parity
void launch_extra_forces(const Dev &d, int parity, cudaStream_t s);
// gpu_update_detach (VX3_VoxelyzeKernel.cu:946-967) for robots with EnableDetach
void launch_detach(const Dev &d, cudaStream_t s);
// removeVoxels (VX3_VoxelyzeKernel.cu:365-397) at the end of the step of the given parity
void launch_remove(const Dev &d, int parity, cudaStream_t s);
// the signals of the step of the given parity (the end of VX3_Voxel::timeStep), after the voxel pass
void launch_signals(const Dev &d, int parity, cudaStream_t s);
// attachment (robots with EnableAttach), between the contact-list check and the contact
// evaluation: the parallel pair tests, then the links made in the serial pair order
void launch_attach(const Dev &d, cudaStream_t s);
// enableAttach of every stepped voxel of robots with attach conditions, after the voxel pass
void launch_attach_cond(const Dev &d, int parity, cudaStream_t s);
// one-time setup of the collision kernels (shared-memory size, grid); fills d.cgrid
cudaError_t init_collision(Dev &d);
void launch_coll_eval_mixed(const Dev &d, cudaStream_t s);
void launch_coll_eval(const Dev &d, cudaStream_t s);  // the contact evaluation alone
void launch_com(const Dev &d, double *out4, cudaStream_t s);
// state exchange with plain doubles (comps = 3 or 4 per voxel) in device memory, or, for
// the pack, in page-locked host memory it reads in place
void launch_pack_state(const Dev &d, double4 *dst, const double *staged, int comps, int keep_w, cudaStream_t s);
void launch_unpack_state(const Dev &d, double *staged, const double4 *src, int comps, cudaStream_t s);
void launch_or_status(const Dev &d, int robot, int bits, cudaStream_t s);
// stable time step of every robot with module-static scratch (vx3g_recommended_dt_noalloc);
// returns 0, -1 (invalid) or -3 (CUDA error, message in *why)
int recommended_dt_noalloc(const Dev &d, int device, double *out_host, cudaStream_t s, const char **why);

}  // namespace vx3g
