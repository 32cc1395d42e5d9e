/* vx3_oracle.h -- CPU restatement of the reference VX3 time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300
 * kernels: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it; nothing in the shipped library links or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py compares this restatement,
 * bit for bit, against golden vectors produced by the reference's own
 * sources compiled on the host (oracle/Makefile target `ref`,
 * tests/golden/make_golden.py).
 */
#ifndef VX3_ORACLE_H
#define VX3_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* One palette entry, values as read from the VXA <Material> element. */
typedef struct vxo_material {
    double E, nu, rho, cte, mu_static, mu_kinetic;
    double fail_stress;      /* models 1 and 2 (-1: none) */
    int model;               /* 0 MDL_LINEAR, 1 MDL_LINEAR_FAIL, 2 MDL_BILINEAR, 3 MDL_DATA */
    int fixed, is_measured;
    double thermal_on_after; /* TurnOnThermalExpansionAfterThisManySeconds */
    double cilia, cilia_on_after; /* Cilia, TurnOnCiliaAfterThisManySeconds */
    double remove_after;          /* RemoveFromSimulationAfterThisManySeconds (SecondaryExperiment) */
    double plastic_mod, yield_stress; /* Plastic_Mod, Yield_Stress (model 2, MDL_BILINEAR) */
    int n_data;                       /* model 3 (MDL_DATA): SSData points */
    const double *strain_data, *stress_data;
    int is_pacemaker;                 /* isPaceMaker */
    double pacemaker_period, signal_value_decay, signal_time_delay, inactive_period;
    int sticky;                       /* Sticky: runtime links with touching voxels of this material */
} vxo_material;

/* A math-tree token (VX3_MathTreeToken, src/Utils/VX3_MathTree.h:29-36): op is the
 * VX3_MathTreeOperator value, value the constant or the variable index. */
typedef struct vxo_math_token {
    int op, reserved;
    double value;
} vxo_math_token;

/* A boundary-condition region (CVX_FRegion): PrimType 0 box, 1 cylinder, 2 sphere;
 * DofFixed bits 1,2,4 translation x,y,z and 8,16,32 rotation x,y,z; coordinates in
 * fractions of the workspace (floats, as the reference keeps them). */
typedef struct vxo_bc_region {
    int prim, dof_fixed;
    float x, y, z, dx, dy, dz, radius;
    double force[3], torque[3], displace[3], ang_displace[3];
} vxo_bc_region;

/* One simulation (one merged VXA). */
typedef struct vxo_robot {
    int nx, ny, nz;
    const unsigned char *lattice; /* nx*ny*nz palette ids, x fastest, then y, then z */
    const double *phase;          /* nx*ny*nz phase offsets (cycles) or NULL */
    int n_materials;
    const vxo_material *materials;
    double vox_size, dt_frac, grav_acc;
    int floor_enabled;
    double temp_amplitude, temp_period, temp_base;
    int temp_enabled, vary_temp, enable_expansion, enable_collision, volume_effects;
    double bond_damping, col_damping, slow_damping;
    const vxo_math_token *force_field[3]; /* ForceField x/y/z programs (mtEND-terminated) or NULL */
    int enable_cilia;                     /* Simulator/EnableCilia */
    const double *cilia_base, *cilia_shift; /* nx*ny*nz*3 Base/ShiftCiliaForce per cell, or NULL */
    int enable_detach;                    /* Simulator/AttachDetach/EnableDetach */
    int secondary_experiment;             /* Simulator/SecondaryExperiment: material removal */
    int n_bcs;                            /* Environment/Boundary_Conditions regions */
    const vxo_bc_region *bcs;
    int enable_signals;                   /* Simulator/EnableSignals */
    int enable_attach;                    /* Simulator/AttachDetach/EnableAttach */
    int safety_guard;                     /* Simulator/AttachDetach/SafetyGuard (the reference's default is 500) */
    const vxo_math_token *attach_cond[5]; /* AttachCondition/Condition_0..4 programs, or NULL (no condition) */
} vxo_robot;

void *vxo_create(const vxo_robot *r);
void vxo_destroy(void *h);
void vxo_counts(void *h, int *nv, int *nl, int *nsurf);
int vxo_step(void *h, int n);
double vxo_time(void *h);
float vxo_dt(void *h);
void vxo_voxels(void *h, double *pos, double *orient, double *linmom, double *angmom, float *tempe, int *flags);
void vxo_set_voxels(void *h, const double *pos, const double *orient, const double *linmom, const double *angmom);
/* the rest of a run's state (time, temperatures, static friction, link state) to continue
 * a run taken elsewhere: link_flags bit 0 smallAngle, bit 2 LOCAL_VELOCITY_VALID */
void vxo_set_run_state(void *h, double t, const float *tempe, const int *static_flag, const double *local9,
                       const float *strain, const float *maxstrain, const int *link_flags);
void vxo_topology(void *h, int *mat, int *ijk, int *slots);
void vxo_link_topology(void *h, int *negpos, int *axis, int *small, int *states);
void vxo_links(void *h, float *strain, float *maxstrain, double *rest, double *local9, double *forces12);
void vxo_voxel_mats(void *h, float *f16, double *nomsize, int *fixed_measured);
void vxo_link_mats(void *h, float *f16, int *lmat_of_link);
int vxo_num_link_mats(void *h);
void vxo_surface(void *h, int *idx);
/* per link: the plastic strain offset; link material i's stress-strain points as the
 * reference's device copy holds them (0, 0, then the model's points from (0,0) on; at
 * most cap copied), returning their count */
void vxo_link_offsets(void *h, float *off);
/* per voxel: localSignal */
void vxo_signals(void *h, double *local_signal);
int vxo_link_curve(void *h, int i, float *strain, float *stress, int cap);
void vxo_last_contact(void *h, double *c3);
void vxo_com(void *h, double *c3);
double vxo_recommended_dt(void *h);
/* timing helpers for the CPU baseline (not used for parity) */
void vxo_set_threads(void *h, int n);
/* n threads with results bit-identical to the serial step (contact forces gathered per
 * voxel in the serial loop's order); for large parity cases */
void vxo_set_exact_threads(void *h, int n);
double vxo_time_collision_rows(void *h, int begin, int end);
int vxo_step_no_collision(void *h, int n);

#ifdef __cplusplus
}
#endif
#endif
