/* vx3g.h -- C ABI of the GB300-native VX3 voxel-physics step.
 *
 * One context holds a batch of independent simulations ("robots"), each the
 * equivalent of one VX3_VoxelyzeKernel built from one merged VXA document in
 * the reference.  All state lives in GPU memory owned by the context; every
 * call below takes and returns plain host pointers and sizes.  No call throws;
 * every call returns VX3G_OK (0) or a negative error code, and
 * vx3g_last_error() gives a one-line reason for the calling thread's last
 * failure.  A context is not re-entrant: use one context per host thread.
 *
 * Reference interfaces each entry point replaces (voxcraft-sim source tree):
 *   vx3g_create       VX3_VoxelyzeKernel::VX3_VoxelyzeKernel(CVX_Sim*)   src/VX3/VX3_VoxelyzeKernel.cu:27-105
 *                     + the per-file setup of VX3_SimulationManager::readVXD  src/VX3/VX3_SimulationManager.cu:277-381
 *   vx3g_step         VX3_VoxelyzeKernel::doTimeStep(float dt = -1), called in the
 *                     CUDA_Simulation step loop                           src/VX3/VX3_VoxelyzeKernel.cu:237-359,
 *                                                                         src/VX3/VX3_SimulationManager.cu:62-115
 *   vx3g_dt           VX3_VoxelyzeKernel::recommendedTimeStep()*DtFrac    src/VX3/VX3_VoxelyzeKernel.cu:184-217,241-254
 *   vx3g_com          VX3_VoxelyzeKernel::updateCurrentCenterOfMass()     src/VX3/VX3_VoxelyzeKernel.cu:477-493
 *   vx3g_get_state    the device->host copy of voxel state in
 *                     VX3_SimulationManager::collectResults               src/VX3/VX3_SimulationManager.cu:428-470
 *   vx3g_status       doTimeStep's false return on divergence             src/VX3/VX3_VoxelyzeKernel.cu:271-281
 *   vx3g_destroy      VX3_VoxelyzeKernel::cleanup()                       src/VX3/VX3_VoxelyzeKernel.cu:107-119
 */
#ifndef VX3G_H
#define VX3G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------ */
#define VX3G_OK 0
#define VX3G_ERR_INVALID (-1)      /* bad argument or descriptor */
#define VX3G_ERR_UNSUPPORTED (-2)  /* input uses a feature outside the supported scope */
#define VX3G_ERR_CUDA (-3)         /* CUDA runtime error (no device, launch failure, ...) */
#define VX3G_ERR_NOMEM (-4)        /* device or host allocation failed */
#define VX3G_ERR_DEVICE (-5)       /* a kernel reported an internal error (see vx3g_status) */

/* ---- per-robot status words (vx3g_status) -------------------------------- */
#define VX3G_ROBOT_OK 0
#define VX3G_ROBOT_DIVERGED 1          /* a link strain exceeded 100; the robot stops stepping */
#define VX3G_ROBOT_CONTACT_OVERFLOW 2  /* more contact candidates than one voxel can hold */
#define VX3G_ROBOT_STOPPED 4           /* stopped by the caller (vx3g_stop_robot) */
#define VX3G_ROBOT_LINK_CAPACITY 8     /* attachment wanted a runtime link beyond the robot's reserve
                                          (links that detached keep their slots); the robot stops */

/* ---- precision of the step ---------------------------------------------- */
#define VX3G_PRECISION_FP64 0   /* the reference's arithmetic: FP64 vectors, FP32 scalars where it uses float */
#define VX3G_PRECISION_MIXED 1  /* FP32 link forces/moments, FP64 position/orientation/momentum integration */

/* One palette entry, with the values of the VXA <Material><Mechanical> element. */
typedef struct vx3g_material {
    double E;             /* Elastic_Mod (Pa) */
    double nu;            /* Poissons_Ratio */
    double rho;           /* Density (kg/m^3) */
    double cte;           /* CTE (1/degC) */
    double mu_static;     /* uStatic */
    double mu_kinetic;    /* uDynamic */
    double fail_stress;   /* Fail_Stress (Pa): models 1 and 2 (-1: no failure) */
    int model;            /* MatModel: 0 linear, 1 linear with failure, 2 bilinear (elastic-plastic),
                             3 stress-strain data points; others -> VX3G_ERR_UNSUPPORTED.  A model
                             the reference's setters reject (E <= 0; model 1 with fail_stress <= 0;
                             model 2 unless 0 < plastic_mod < E, yield_stress > 0 and fail_stress
                             > yield_stress or -1; model 3 without a positive first point or with
                             strain not increasing) leaves the reference's default material model,
                             as VX3_SimulationManager does: linear, E = 1e6 Pa, no failure
                             (src/old/VX_Material.cpp:300-446, src/old/Voxelyze.cpp:357-365) */
    int fixed;            /* Fixed */
    int is_measured;      /* isMeasured (counts toward the centre of mass) */
    double thermal_on_after; /* TurnOnThermalExpansionAfterThisManySeconds */
    double cilia;            /* Cilia: scale of the cilia force (VX3_Voxel::force, src/VX3/VX3_Voxel.cu:376) */
    double cilia_on_after;   /* TurnOnCiliaAfterThisManySeconds */
    double remove_after;     /* RemoveFromSimulationAfterThisManySeconds: with secondary_experiment, the
                                material's voxels leave the simulation at the end of the first step that
                                starts later than this (> 0; 0 never) */
    double plastic_mod;      /* Plastic_Mod (Pa), model 2: the modulus past yield */
    double yield_stress;     /* Yield_Stress (Pa), model 2 */
    int n_data;              /* model 3: SSData NumDataPts (a leading (0,0) point is skipped), at most
                                VX3G_MAX_MODEL_POINTS */
    const double *strain_data, *stress_data; /* model 3: SSData StrainData / StressData values */
    int is_pacemaker;         /* isPaceMaker: with enable_signals, emits a signal of 100 every pacemaker_period s */
    double pacemaker_period;  /* PaceMakerPeriod (s) */
    double signal_value_decay; /* signalValueDecay: a received signal is passed on scaled by this (VXA default 0.9) */
    double signal_time_delay; /* signalTimeDelay (s): delay before a voxel passes a signal on (VXA default 0.03) */
    double inactive_period;   /* inactivePeriod (s): refractory time after a signal (VXA default 0.03) */
    int sticky;               /* Sticky: with enable_attach, touching voxels of this material link up.  A
                                 sticky material of an attaching robot must be linear (model 0/1) with
                                 Poisson's ratio 0 (or volume effects off), else VX3G_ERR_UNSUPPORTED */
} vx3g_material;
#define VX3G_MAX_MODEL_POINTS 32

/* One token of a math-tree program, the reference's VX3_MathTreeToken
 * (src/Utils/VX3_MathTree.h:29-36) as VX3_SimulationManager::ParseMathTree
 * (src/VX3/VX3_SimulationManager.cu:157-275) lays a formula out: op is the
 * VX3_MathTreeOperator value -- mtEND 0, mtCONST 1, mtE 2, mtPI 3, mtVAR 4, mtADD 5,
 * mtSUB 6, mtMUL 7, mtDIV 8, mtPOW 9, mtSQRT 10, mtSIN 11, mtCOS 12, mtTAN 13,
 * mtATAN 14, mtLOG 15, mtINT 16, mtABS 17, mtNOT 18, mtGREATERTHAN 19, mtLESSTHAN 20,
 * mtAND 21, mtOR 22, mtNORMALCDF 23 -- and value is mtCONST's constant or mtVAR's
 * variable: x 0, y 1, z 2, hit 3, t 4, angle 5, targetCloseness 6, numClosePairs 7,
 * num_voxel 8.  A program ends with mtEND and holds at most VX3G_MAX_MATH_TOKENS
 * tokens including it. */
typedef struct vx3g_math_token {
    int32_t op;
    int32_t reserved;
    double value;
} vx3g_math_token;
#define VX3G_MAX_MATH_TOKENS 256

/* One boundary-condition region of the VXA <Environment><Boundary_Conditions>
 * (CVX_FRegion, src/old/VX_FRegion.cpp:165-219).  Every voxel the region touches
 * gets an external (VX3_External): the fixed degrees of freedom held at their
 * prescribed displacement, and an equal share of the region's force and torque
 * (CVX_Sim::Import, src/VXA/VX_Sim.cpp:109-141). */
typedef struct vx3g_bc_region {
    int prim;            /* PrimType: 0 box, 1 cylinder, 2 sphere (3, a mesh, -> VX3G_ERR_UNSUPPORTED) */
    int dof_fixed;       /* DofFixed: 1 X, 2 Y, 4 Z translation, 8 X, 16 Y, 32 Z rotation */
    float x, y, z;       /* X, Y, Z: the region's corner (box, cylinder) or centre (sphere) in
                            fractions of the workspace (the lattice's extent) */
    float dx, dy, dz;    /* dX, dY, dZ: box size; cylinder length along its one non-zero axis */
    float radius;        /* Radius (sphere, cylinder), in fractions of the workspace's largest side */
    double force[3];     /* ForceX..Z (N), divided equally among the voxels it touches */
    double torque[3];    /* TorqueX..Z (N m), likewise */
    double displace[3];  /* DisplaceX..Z (m): translation of the fixed translational DOFs */
    double ang_displace[3]; /* AngDisplaceX..Z (rad): rotation vector of the fixed rotational DOFs */
} vx3g_bc_region;

/* One simulation: the content of a merged VXA document. */
typedef struct vx3g_robot_desc {
    int nx, ny, nz;                 /* X_Voxels, Y_Voxels, Z_Voxels */
    const uint8_t *lattice;         /* nx*ny*nz palette ids, x fastest then y then z; 0 = empty */
    const double *phase;            /* nx*ny*nz PhaseOffset values (cycles) or NULL for 0 */
    int n_materials;                /* palette ids 1..n_materials, at most 16 */
    const vx3g_material *materials;
    double vox_size;                /* Lattice_Dim (m) */
    double dt_frac;                 /* Integration/DtFrac */
    double grav_acc;                /* Gravity/GravAcc (m/s^2); the reference applies it whatever GravEnabled says */
    int floor_enabled;              /* Gravity/FloorEnabled */
    double temp_amplitude, temp_period, temp_base; /* Thermal/TempAmplitude, TempPeriod, TempBase */
    int temp_enabled;               /* Thermal/TempEnabled (only the initial temperature uses it) */
    int vary_temp;                  /* Thermal/VaryTempEnabled */
    int enable_expansion;           /* Simulator/EnableExpansion */
    int enable_collision;           /* Simulator/AttachDetach/EnableCollision */
    int volume_effects;             /* Simulator/Features/VolumeEffectsEnabled (0 forces Poisson's ratio to 0) */
    double bond_damping, col_damping, slow_damping; /* Simulator/Damping/{Bond,Col,Slow}DampingZ */
    const double *log10E;           /* nx*ny*nz per-voxel log10 Young's modulus overriding the palette's,
                                       or NULL (per-voxel stiffness is not expressible in a VXA palette) */
    const vx3g_math_token *force_field[3]; /* Simulator/ForceField/{x,y,z}_forcefield programs or NULL
                                       (0): the force added to every voxel each step
                                       (VX3_Voxel::timeStep, src/VX3/VX3_Voxel.cu:178-184).  Variables
                                       x, y, z (the voxel's position), t (the time at the start of the
                                       step), num_voxel, and hit (the reference keeps it 0); programs
                                       that read angle, targetCloseness or numClosePairs (target
                                       tracking, not supported) are rejected with VX3G_ERR_UNSUPPORTED */
    int enable_cilia;               /* Simulator/EnableCilia: gpu_update_cilia_force (VX3_VoxelyzeKernel.cu:846-859) */
    const double *cilia_base;       /* nx*ny*nz*3 Structure/BaseCiliaForce vectors (per cell) or NULL for 0 */
    const double *cilia_shift;      /* nx*ny*nz*3 Structure/ShiftCiliaForce vectors or NULL; scaled by the
                                       voxel's localSignal (0 unless enable_signals) */
    int enable_detach;              /* Simulator/AttachDetach/EnableDetach: a failed link leaves both voxels'
                                       link tables after the collision pass (gpu_update_detach,
                                       VX3_VoxelyzeKernel.cu:946-967); the surface, the contact
                                       candidates and the cilia follow from the next step */
    int secondary_experiment;       /* Simulator/SecondaryExperiment: material removal (removeVoxels,
                                       VX3_VoxelyzeKernel.cu:335-397): a removed voxel is no longer
                                       stepped, loses its links, leaves the surface and the contact
                                       candidates, and keeps counting toward the centre of mass; the
                                       initial-position reset of the same block is the caller's (it
                                       touches only the report) */
    int n_bcs;                      /* Environment/Boundary_Conditions regions, applied in order */
    const vx3g_bc_region *bcs;      /* (the lattice's cells are vox_size cubes: Lattice_Dim with all
                                       dimension adjustments 1 and no line or layer offsets) */
    int enable_signals;             /* Simulator/EnableSignals: pacemaker voxels emit signals that spread
                                       along links, decaying; a voxel's signal scales its ShiftCiliaForce
                                       (VX3_Voxel.cu:271-348, VX3_VoxelyzeKernel.cu:857).  The reference
                                       lets each voxel thread write its neighbours' signal state without
                                       synchronisation; here voxels take their turns in voxel order, the
                                       order of a serial loop over the voxel pass */
    int enable_attach;              /* Simulator/AttachDetach/EnableAttach: two voxels of one Sticky material
                                       that come within the contact envelope, both allowed by the attach
                                       conditions, unfixed and more than five links apart, get a new link
                                       along the dominant axis of their offset in the first one's frame
                                       when both faces are free (handle_collision_attachment,
                                       VX3_VoxelyzeKernel.cu:729-830).  The reference runs all pairs of
                                       a step at once; here they take their turns in the order of its
                                       serial loop over surface pairs.  Needs enable_collision. */
    int safety_guard;               /* Simulator/AttachDetach/SafetyGuard (VXA default 500): a new link's
                                       forces and moments are scaled by 0.01 for its first this many
                                       updates (VX3_Link.cu:206-213) */
    const vx3g_math_token *attach_condition[5]; /* AttachCondition/Condition_0..4 programs or NULL: a
                                       voxel may attach while every given program is > 0 at its
                                       position after its last step (x, y, z), t (that step's start
                                       time), num_voxel; an absent condition holds (the reference reads
                                       an unset value there) */
} vx3g_robot_desc;

typedef struct vx3g_batch_desc {
    int n_robots;
    const vx3g_robot_desc *robots;
    int precision;                  /* VX3G_PRECISION_* */
    int device;                     /* CUDA device ordinal */
    int graph_chunk;                /* steps captured per CUDA graph launch (0 -> 100; < 0: no
                                       graphs, every step's kernels launched one by one, e.g.
                                       for a per-kernel profiler) */
} vx3g_batch_desc;

typedef struct vx3g_ctx vx3g_ctx;

/* Builds the lattice (voxel order, link order and Neg/Pos ends exactly as the
 * reference's CVoxelyze), derives material constants, uploads the batch and
 * computes each robot's time step.  Returns NULL on failure with *status set. */
vx3g_ctx *vx3g_create(const vx3g_batch_desc *desc, int *status);
void vx3g_destroy(vx3g_ctx *ctx);
const char *vx3g_last_error(void);

/* Advances every robot by n_steps time steps (asynchronous on the context's
 * stream; robots that diverged stay frozen).  Full chunks run as CUDA graphs. */
int vx3g_step(vx3g_ctx *ctx, int n_steps);
int vx3g_synchronize(vx3g_ctx *ctx);
/* Captures and instantiates the CUDA graphs vx3g_step replays (both step parities)
 * without running them, so that the first vx3g_step of a latency-sensitive loop does
 * not pay for the capture.  Optional; no counterpart in the reference. */
int vx3g_prepare_graphs(vx3g_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for event timing by the caller. */
void *vx3g_stream(vx3g_ctx *ctx);

/* Sizes: totals over the batch, and per-robot offsets into the packed arrays. */
int vx3g_counts(vx3g_ctx *ctx, int *n_voxels, int *n_links, int *n_surface);
int vx3g_offsets(vx3g_ctx *ctx, int *voxel_offset /* n_robots+1 */, int *link_offset /* n_robots+1 */);

/* Host copies of the packed state (voxel order of each robot, robots
 * back to back).  Any pointer may be NULL to skip that array.
 *   pos, linmom, angmom: 3 doubles per voxel; orient: 4 doubles (w,x,y,z) per voxel. */
int vx3g_get_state(vx3g_ctx *ctx, double *pos, double *orient, double *linmom, double *angmom);
int vx3g_set_state(vx3g_ctx *ctx, const double *pos, const double *orient, const double *linmom,
                   const double *angmom);
/* tempe: float per voxel; flags: reference voxel bool-state bits (FLOOR_ENABLED 4,
 * FLOOR_STATIC_FRICTION 8); contact: 3 doubles per voxel (last step's contact force; on a
 * voxel of a Fixed material or with all DOFs fixed by a boundary condition, which never
 * reaches VX3_Voxel::force() where the reference clears it, the sum over all steps so far). */
int vx3g_get_voxel_aux(vx3g_ctx *ctx, float *tempe, int32_t *flags, double *contact);
/* Link state in the reference's link order (each robot's lattice links, then its runtime
 * links in creation order, then its unused reserve, reported as gone): strain, maxStrain (float),
 * local9 = pos2, angle1v, angle2v (9 doubles), forces12 = forceNeg, forcePos,
 * momentNeg, momentPos (12 doubles), small = small-angle flag (bit 0) | 2 once the
 * link has left the lattice (detached or removed: no voxel's link any more) | 4 while
 * its local velocity is valid (LOCAL_VELOCITY_VALID: the damping terms apply). */
int vx3g_get_links(vx3g_ctx *ctx, float *strain, float *max_strain, double *local9, double *forces12,
                   int32_t *small);
/* Topology: voxel lattice indices (3 ints), voxel palette index (0-based),
 * link ends (neg, pos voxel indices, packed global; -1 for an unused reserve slot),
 * link axis (0 x, 1 y, 2 z). */
int vx3g_get_topology(vx3g_ctx *ctx, int32_t *voxel_ijk, int32_t *voxel_mat, int32_t *link_ends,
                      int32_t *link_axis);
/* Per voxel: its localSignal (VX3_Voxel::localSignal; 0 in robots without signals). */
int vx3g_get_signals(vx3g_ctx *ctx, double *local_signal);
/* Surface voxels (fewer than six links, not removed), global voxel indices in voxel
 * order; with enable_detach or secondary_experiment the set follows the link table
 * (vx3g_counts gives its current size). */
int vx3g_get_surface(vx3g_ctx *ctx, int32_t *surface);
/* Per robot: links in use, the lattice's plus those made by attachment so far (each
 * robot's link range of vx3g_offsets holds these first, then its unused reserve). */
int vx3g_links_in_use(vx3g_ctx *ctx, int32_t *n_links /* per robot */);

int vx3g_com(vx3g_ctx *ctx, double *com /* 3 per robot */);
int vx3g_dt(vx3g_ctx *ctx, double *dt /* per robot: the float step, widened */);
int vx3g_time(vx3g_ctx *ctx, double *t /* per robot */);
/* Per-robot status words.  Returns VX3G_ERR_DEVICE (status still filled) if a device
 * wait of the collision pass gave up (bounded grid barrier; the state is then suspect). */
int vx3g_status(vx3g_ctx *ctx, int32_t *status /* per robot */);
/* Stops one robot: it no longer steps (CUDA_Simulation's per-simulation loop
 * exit when StopConditionMet(), src/VX3/VX3_SimulationManager.cu:63-64). */
int vx3g_stop_robot(vx3g_ctx *ctx, int robot);
/* Steps taken so far by the context (every robot that has not diverged). */
int64_t vx3g_steps_taken(vx3g_ctx *ctx);

/* ---- differentiation (no counterpart in the reference) ---------------------
 * vx3g_record: advances n_steps (exactly like vx3g_step) and keeps the state
 *   every `checkpoint_every` steps, as the forward pass of a gradient.  FP64
 *   contexts only (VX3G_ERR_UNSUPPORTED otherwise); self-collision included.
 * vx3g_backward: gradient of L = sum_r w_r . (COM_r(end) - COM_r(start)) over the
 *   recorded run with respect to every voxel's actuation phase (in cycles, the
 *   unit of vx3g_robot_desc.phase) and log10 of its Young's modulus, by the
 *   hand-written adjoint of the step run backwards over the recorded steps; each
 *   checkpoint interval is recomputed from its checkpoint.  dL_dcom: w, 3 per
 *   robot; dL_dphase, dL_dlog10E: one per voxel (either may be NULL).  The
 *   discrete events of the run (friction stick/slip, floor and voxel-voxel
 *   contact, the small/large angle switch of each link, the temperature clamp)
 *   are held as the run took them, and the time step is held fixed.  The context keeps the recorded end
 *   state; backward may be called again with other weights. */
int vx3g_record(vx3g_ctx *ctx, int n_steps, int checkpoint_every);
int vx3g_backward(vx3g_ctx *ctx, const double *dL_dcom, double *dL_dphase, double *dL_dlog10E);

/* ---- stable time step without allocation (no counterpart in the reference as
 * an entry point; the reference evaluates recommendedTimeStep inside its first
 * doTimeStep, VX3_VoxelyzeKernel.cu:184-217, 248-253) ----------------------------
 * vx3g_recommended_dt_noalloc: rdt[r] = recommendedTimeStep of robot r in its
 *   current state (seconds, before DtFrac and the 1e-10 floor; vx3g_create sets
 *   the context's dt to (float)(DtFrac * max(rdt, 1e-10))).  With Poisson's ratio
 *   on, the stiffness term eHat*A/((strain+1)*L) takes the links' current strain
 *   and rest length, so the value changes as the robot deforms, and the transverse
 *   area A fixed when the link was created -- the area the step itself uses (the
 *   reference's link update never refreshes it, VX3_Link.cu:147-150).  The
 *   reference's VX3_Link::axialStiffness refreshes A from the voxels' current
 *   Poisson strain (VX3_Link.cu:269-278); the two agree at step 0, where the
 *   reference calls it.
 *   For callers that must not allocate device memory at this point: a control
 *   loop re-checking the stable step between chunks in a process whose device
 *   memory budget is fixed, or code that runs while the device is in use by work
 *   that an allocation (which can synchronise the device) would disturb.  Its
 *   reduction scratch is a fixed 96 KB array in the library's device image; the
 *   call allocates nothing and frees nothing.  At most 4096 robots per context
 *   (VX3G_ERR_INVALID beyond).  The first call on a device looks the scratch up
 *   (once per device); make that first call before any stream capture.  Calls
 *   that overlap in time on the same device share the one scratch array and race
 *   (wrong results): serialise them.  Blocking: returns when rdt is filled. */
int vx3g_recommended_dt_noalloc(vx3g_ctx *ctx, double *rdt);

/* ---- launch-shape autotuning (no counterpart in the reference) ---------------
 * vx3g_autotune: advances n_steps exactly like vx3g_step (results identical),
 *   timing the link and voxel passes of a mixed-precision context under each of
 *   their compiled launch shapes (threads per block x minimum resident blocks),
 *   and keeps the fastest.  With cache_json (a path, or NULL) the choice is read
 *   from / appended to a flat JSON object keyed by GPU name and batch size; a
 *   cached choice is applied without timing.  FP64 contexts just step.
 * vx3g_launch_shapes: the shapes in use: {link threads, link min blocks, voxel
 *   threads, voxel min blocks}. */
int vx3g_autotune(vx3g_ctx *ctx, int n_steps, const char *cache_json);
int vx3g_launch_shapes(vx3g_ctx *ctx, int32_t *shapes4);

/* ---- measurement helpers (no counterpart in the reference) ---------------
 * vx3g_time_steps: runs vx3g_step(ctx, n_steps) between two CUDA events on the
 *   context's stream and returns the device time in milliseconds.
 * vx3g_flush_l2: overwrites a context-owned buffer of `bytes` bytes on the
 *   context's stream (evicts the L2 cache between timed iterations).
 * vx3g_time_passes: runs each per-step pass `iters` times on its own, captured
 *   in one CUDA graph as the step graphs run it, between CUDA events, and
 *   returns the mean device time per pass in milliseconds (ms4[4]) for: [0] link pass, [1] collision passes (all kernels of the
 *   broad and narrow phase together), [2] voxel pass, [3] the contact evaluation
 *   kernel alone.  It advances the state like extra steps would; use it after
 *   the measured run. */
int vx3g_time_steps(vx3g_ctx *ctx, int n_steps, float *ms);
int vx3g_flush_l2(vx3g_ctx *ctx, size_t bytes);
int vx3g_time_passes(vx3g_ctx *ctx, int iters, float *ms4);

/* ---- fault-path test hook (no counterpart in the reference) ---------------
 * vx3g_debug_barrier: sets the grid barrier of the collision list rebuild to give up
 *   after `polls` polls of 32 ns or more each (0: the default limit, 2^22 polls)
 *   with `arrivals` arrivals already counted, and, for polls > 0, makes every
 *   robot's contact lists due so that the next step runs the barrier.  A large
 *   pre-counted arrival makes every wait run out: the kernel returns, later rebuilds
 *   are skipped until the next vx3g_status reports VX3G_ERR_DEVICE and clears the
 *   barrier and the error, and the step after that rebuilds every list.  Tests only. */
int vx3g_debug_barrier(vx3g_ctx *ctx, uint32_t polls, uint32_t arrivals);

#ifdef __cplusplus
}
#endif
#endif
