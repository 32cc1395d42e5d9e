/* vx3_oracle.c -- CPU restatement of the reference VX3 time step (plain C).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GB300 kernels, never linked
 * into the shipped library.  Every function cites the reference file:line it
 * restates (paths relative to the voxcraft-sim source tree).  Arithmetic is
 * written so that C's usual conversions reproduce the reference's mix of
 * float and double exactly (build with -ffp-contract=off).
 *
 * Scope: material models 0-3 (linear, linear with failure, bilinear, data points);
 * boundary-condition regions; signals and cilia; the link table changes by detach,
 * by material removal and by attachment (runtime links between touching Sticky
 * voxels of one material whose Poisson's ratio is 0, in the serial pair loop's
 * order); force field and attach conditions: math-tree programs (force field 0
 * when absent, the reference default, VX3_ForceField.h:10-20; an absent attach
 * condition holds), target-tracking variables 0.
 */
#include "vx3_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y, z; } vec;
typedef struct { double w, x, y, z; } quat;

static vec V(double x, double y, double z) { vec r = {x, y, z}; return r; }
static vec vadd(vec a, vec b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static vec vsub(vec a, vec b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static vec vneg(vec a) { return V(-a.x, -a.y, -a.z); }
/* VX3_Vec3D operator*(f): (f*x, f*y, f*z)  (VX3_Vec3D.h:49,61) */
static vec vscale(vec a, double f) { return V(f * a.x, f * a.y, f * a.z); }
/* VX3_Vec3D operator/(f): Inv = 1/f; (Inv*x, ...)  (VX3_Vec3D.h:63) */
static vec vdiv(vec a, double f) { double inv = 1.0 / f; return V(inv * a.x, inv * a.y, inv * a.z); }
static double vlen(vec a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static double vdot(vec a, vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* Normalized (VX3_Vec3D.h:94) */
static vec vnormalized(vec a) { double l = sqrt(a.x * a.x + a.y * a.y + a.z * a.z); return l > 0 ? vdiv(a, l) : a; }

static quat Q(double w, double x, double y, double z) { quat q = {w, x, y, z}; return q; }
static quat qident(void) { return Q(1, 0, 0, 0); }
static quat qconj(quat q) { return Q(q.w, -q.x, -q.y, -q.z); }
/* VX3_Quat3D.h:217-222 */
static quat qmul(quat a, quat f) {
    return Q(a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z,
             a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
             a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x,
             a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w);
}
/* VX3_Quat3D.h:439-447 */
static vec qrot(quat q, vec f) {
    double fx = f.x, fy = f.y, fz = f.z;
    double tw = fx * q.x + fy * q.y + fz * q.z;
    double tx = fx * q.w - fy * q.z + fz * q.y;
    double ty = fx * q.z + fy * q.w - fz * q.x;
    double tz = -fx * q.y + fy * q.x + fz * q.w;
    return V(q.w * tx + q.x * tw + q.y * tz - q.z * ty,
             q.w * ty - q.x * tz + q.y * tw + q.z * tx,
             q.w * tz + q.x * ty - q.y * tx + q.z * tw);
}
/* VX3_Quat3D.h:465-473 */
static vec qrotinv(quat q, vec f) {
    double fx = f.x, fy = f.y, fz = f.z;
    double tw = q.x * fx + q.y * fy + q.z * fz;
    double tx = q.w * fx - q.y * fz + q.z * fy;
    double ty = q.w * fy + q.x * fz - q.z * fx;
    double tz = q.w * fz - q.x * fy + q.y * fx;
    return V(tw * q.x + tx * q.w + ty * q.z - tz * q.y,
             tw * q.y - tx * q.z + ty * q.w + tz * q.x,
             tw * q.z + tx * q.y - ty * q.x + tz * q.w);
}
/* ToRotationVector (VX3_Quat3D.h:347-359) */
static vec q_to_rotvec(quat q) {
    if (q.w >= 1.0 || q.w <= -1.0) return V(0, 0, 0);
    double sq = 1.0 - q.w * q.w;
    vec v = V(q.x, q.y, q.z);
    if (sq < 2.4e-3)
        return vscale(vscale(v, 2.0), sqrt((2 - 2 * q.w) / sq));
    return vdiv(vscale(vscale(v, 2.0), acos(q.w)), sqrt(sq));
}
/* FromRotationVector (VX3_Quat3D.h:363-377) */
static quat q_from_rotvec(vec in) {
    vec theta = vdiv(in, 2);
    double s, m2 = theta.x * theta.x + theta.y * theta.y + theta.z * theta.z;
    quat q;
    if (m2 * m2 < 5.328e-15) {
        q.w = 1.0 - 0.5 * m2;
        s = 1.0 - m2 / 6.0;
    } else {
        double m = sqrt(m2);
        q.w = cos(m);
        s = sin(m) / m;
    }
    q.x = theta.x * s;
    q.y = theta.y * s;
    q.z = theta.z * s;
    return q;
}
/* FromAngleToPosX (VX3_Quat3D.h:384-432); q is left unchanged for a zero vector */
static quat q_from_angle_to_posx(quat q, vec r) {
    if (r.x == 0 && r.y == 0 && r.z == 0) return q;
    double yx = r.y / r.x, zx = r.z / r.x;
    if (yx < 1.732e-2 && yx > -1.732e-2 && zx < 1.732e-2 && zx > -1.732e-2) {
        q.x = 0;
        q.y = 0.5 * zx;
        q.z = -0.5 * yx;
        q.w = 1 + 0.5 * (-q.y * q.y - q.z * q.z);
        return q;
    }
    vec n = r; /* NormalizeFast (VX3_Vec3D.h:84) */
    double l = sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
    if (l > 0) { double li = 1.0 / l; n.x *= li; n.y *= li; n.z *= li; }
    double theta = acos(n.x);
    if (theta > 3.14159265358979 - 1e-7) return Q(0, 0, 1, 0);
    double axis_inv = 1.0 / sqrt(n.z * n.z + n.y * n.y);
    double a = 0.5 * theta, s = sin(a);
    return Q(cos(a), 0, n.z * axis_inv * s, -n.y * axis_inv * s);
}

/* VX3_Link.h:134-153 and :156-191 */
static vec to_axis_x(int axis, vec v) {
    if (axis == 1) return V(v.y, -v.x, v.z);
    if (axis == 2) return V(v.z, v.y, -v.x);
    return v;
}
static quat to_axis_xq(int axis, quat q) {
    if (axis == 1) return Q(q.w, q.y, -q.x, q.z);
    if (axis == 2) return Q(q.w, q.z, q.y, -q.x);
    return q;
}
static vec to_axis_original(int axis, vec v) {
    if (axis == 1) return V(-v.y, v.x, v.z);
    if (axis == 2) return V(-v.z, v.y, v.x);
    return v;
}

/* ------------------------------------------------------- stress-strain curves */
/* The piecewise-linear stress-strain model of a material: points (0,0),
 * (strain[1], stress[1]), ... in float, initial modulus E, failure stress and
 * strain (-1: none), linear flag.  Setters as CVX_Material's
 * (src/old/VX_Material.cpp:300-446); each returns 0 where the reference's setter
 * returns false, the caller then keeping the default curve (setModelLinear(1e6),
 * the CVX_Material constructor's, src/old/VX_Material.cpp:15-22). */
#define VXO_MAX_PTS 72
typedef struct {
    int linear, n;
    float E, sigma_fail, eps_fail;
    float strain[VXO_MAX_PTS], stress[VXO_MAX_PTS];
} curve;

static int curve_linear(curve *c, float E, float fail) {
    if (E <= 0) return 0;
    if (fail != -1.0f && fail <= 0) return 0;
    float fs = fail == -1.0f ? 1000000.0f : fail;
    float fe = fs / E;
    c->n = 2;
    c->strain[0] = 0.0f; c->stress[0] = 0.0f;
    c->strain[1] = fe; c->stress[1] = fs;
    c->linear = 1;
    c->E = E;
    c->sigma_fail = fail;
    c->eps_fail = fail == -1.0f ? -1.0f : fe;
    return 1;
}

static void curve_default(curve *c) { curve_linear(c, 1e6f, -1.0f); }

static int curve_bilinear(curve *c, float E, float Ep, float sy, float fail) {
    if (E <= 0 || Ep <= 0 || Ep >= E || sy <= 0) return 0;
    if (fail != -1.0f && fail <= sy) return 0;
    float ys = sy / E;
    float fs = fail == -1.0f ? 3 * sy : fail;
    float b = sy - Ep * ys;
    float fe = (fs - b) / Ep;
    c->n = 3;
    c->strain[0] = 0.0f; c->stress[0] = 0.0f;
    c->strain[1] = ys; c->stress[1] = sy;
    c->strain[2] = fe; c->stress[2] = fs;
    c->linear = 0;
    c->E = E;
    c->sigma_fail = fail;
    c->eps_fail = fail == -1.0f ? -1.0f : fe;
    return 1;
}

/* setModel: a leading (0,0) is dropped; the rest must begin positive with strictly
 * increasing strain; the point (0,0) is put back in front */
static int curve_points(curve *c, int n, const float *e, const float *s) {
    int k = 0;
    if (n > 0 && e[0] == 0 && s[0] == 0) k = 1;
    int m = n - k;
    if (m <= 0 || m + 1 > VXO_MAX_PTS) return 0;
    if (e[k] <= 0 || s[k] <= 0) return 0;
    float last = 0.0f;
    for (int i = k; i < n; i++) {
        if (e[i] <= last) return 0;
        last = e[i];
    }
    c->n = m + 1;
    c->strain[0] = 0.0f; c->stress[0] = 0.0f;
    for (int i = 0; i < m; i++) { c->strain[i + 1] = e[k + i]; c->stress[i + 1] = s[k + i]; }
    c->E = c->stress[1] / c->strain[1];
    c->sigma_fail = c->stress[c->n - 1];
    c->eps_fail = c->strain[c->n - 1];
    c->linear = m == 1;
    return 1;
}

static int curve_failed(const curve *c, float eps) { return c->eps_fail != -1.0f && eps > c->eps_fail; }

/* CVX_Material::modulus (src/old/VX_Material.cpp:231-243) */
static float curve_modulus(const curve *c, float eps) {
    if (curve_failed(c, eps)) return 0.0f;
    if (eps <= c->strain[1] || c->linear) return c->E;
    for (int i = 2; i < c->n; i++)
        if (eps <= c->strain[i] || i == c->n - 1) return (c->stress[i] - c->stress[i - 1]) / (c->strain[i] - c->strain[i - 1]);
    return 0.0f;
}

/* CVX_Material::strain(stress) (src/old/VX_Material.cpp:214-228) */
static float curve_strain_of(const curve *c, float sig) {
    if (sig <= c->stress[1] || c->linear) return sig / c->E;
    for (int i = 2; i < c->n; i++) {
        if (sig <= c->stress[i] || i == c->n - 1) {
            float perc = (sig - c->stress[i - 1]) / (c->stress[i] - c->stress[i - 1]);
            return c->strain[i - 1] + perc * (c->strain[i] - c->strain[i - 1]);
        }
    }
    return 0.0f;
}

/* VX3_Material::stress (src/VX3/VX3_Material.cu:90-124) on the device copy of the
 * curve: VX3_Material::syncVectors (VX3_Material.cu:463-481) puts one more 0 in front
 * of the host points, so the device arrays read 0, 0, strain_1, ... and the stress
 * function's first-segment test compares with that second 0 */
static float curve_stress(const curve *c, float nu, float eHat, float eps, float tss, int force_linear) {
    float ds[VXO_MAX_PTS + 1], dS[VXO_MAX_PTS + 1];
    int n = c->n + 1;
    ds[0] = 0.0f; dS[0] = 0.0f;
    for (int i = 0; i < c->n; i++) { ds[i + 1] = c->strain[i]; dS[i + 1] = c->stress[i]; }
    if (curve_failed(c, eps)) return 0.0f;
    if (eps <= ds[1] || c->linear || force_linear) {
        if (nu == 0.0f) return c->E * eps;
        return eHat * ((1 - nu) * eps + nu * tss);
    }
    for (int i = 2; i < n; i++) {
        if (eps <= ds[i] || i == n - 1) {
            float perc = (eps - ds[i - 1]) / (ds[i] - ds[i - 1]);
            float basic = dS[i - 1] + perc * (dS[i] - dS[i - 1]);
            if (nu == 0.0f) return basic;
            float modulus = (dS[i] - dS[i - 1]) / (ds[i] - ds[i - 1]);
            float modulusHat = modulus / ((1 - 2 * nu) * (1 + nu));
            float eff = basic / modulus;
            float effT = tss * (eff / eps);
            return modulusHat * ((1 - nu) * eff + nu * effT);
        }
    }
    return 0.0f;
}

/* the link curve of CVX_MaterialLink::updateAll (src/old/VX_MaterialLink.cpp:66-97) */
static void curve_link(curve *out, const curve *a, const curve *b) {
    float fail;
    if (a->sigma_fail == -1.0f) fail = b->sigma_fail;
    else if (b->sigma_fail == -1.0f) fail = a->sigma_fail;
    else fail = a->sigma_fail < b->sigma_fail ? a->sigma_fail : b->sigma_fail;
    if (a->linear && b->linear) {
        if (!curve_linear(out, 2.0f * a->E * b->E / (a->E + b->E), fail)) curve_default(out);
        return;
    }
    float e[VXO_MAX_PTS], s[VXO_MAX_PTS];
    int n = 1, ia = 1, ib = 1;
    e[0] = 0.0f; s[0] = 0.0f;
    while (ia < a->n && ib < b->n && n < VXO_MAX_PTS) {
        float x = a->strain[ia];
        if (b->strain[ib] < x) x = b->strain[ib];
        if (x == a->strain[ia]) ia++;
        if (x == b->strain[ib]) ib++;
        float k1 = curve_modulus(a, x - FLT_EPSILON), k2 = curve_modulus(b, x - FLT_EPSILON);
        float k = 2.0f * k1 * k2 / (k1 + k2);
        e[n] = x;
        s[n] = s[n - 1] + k * (x - e[n - 1]);
        n++;
    }
    if (!curve_points(out, n, e, s)) curve_default(out);
    out->sigma_fail = fail;
    out->eps_fail = fail == -1.0f ? -1.0f : curve_strain_of(out, fail);
}

/* ------------------------------------------------------------- materials */
typedef struct {
    float E, nu, rho, cte, mu_s, mu_k, z_int, z_glob, z_col, eHat;
    float sigma_fail, eps_fail;
    curve cv;
    double nom_size;
    float grav_mult;
    float mass, mass_inv, sqrt_mass, mom_inertia, mom_inertia_inv, c2xSqMxExS, c2xSqIxExSxSxS;
    int fixed, is_measured;
    double thermal_on_after;
    double cilia, cilia_on_after; /* Cilia, TurnOnCiliaAfterThisManySeconds (VX_Object.cpp:1429,1437) */
    double remove_after;          /* RemoveFromSimulationAfterThisManySeconds (VX_Object.cpp:1427) */
    int pacemaker;                /* isPaceMaker */
    double pace_period, sig_decay, sig_delay, inactive; /* PaceMakerPeriod, signalValueDecay, signalTimeDelay, inactivePeriod */
    int sticky;                   /* Sticky (VX_Object.cpp:1436) */
} vmat;

typedef struct {
    int m1, m2; /* vox1Mat, vox2Mat indices */
    float E, nu, eHat, eps_fail, cte;
    float a1, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp;
    curve cv;
} lmat;

/* CVX_Material::updateDerived _eHat (src/old/VX_Material.cpp:542-549) */
static float ehat(float E, float nu) { return E / ((1 - 2 * nu) * (1 + nu)); }

/* CVX_MaterialVoxel::updateDerived (src/old/VX_MaterialVoxel.cpp:57-79) */
static void vmat_derive(vmat *m) {
    double volume = m->nom_size * m->nom_size * m->nom_size;
    m->eHat = ehat(m->E, m->nu);
    m->mass = (float)(volume * m->rho);
    m->mom_inertia = (float)(m->mass * m->nom_size * m->nom_size / 6.0f);
    if (volume == 0 || m->mass == 0 || m->mom_inertia == 0) {
        m->mass_inv = m->sqrt_mass = m->mom_inertia_inv = m->c2xSqMxExS = m->c2xSqIxExSxSxS = 0.0f;
        return;
    }
    m->mass_inv = 1.0f / m->mass;
    m->sqrt_mass = sqrtf(m->mass);
    m->mom_inertia_inv = 1.0f / m->mom_inertia;
    m->c2xSqMxExS = (float)(2.0f * sqrt(m->mass * m->E * m->nom_size));
    m->c2xSqIxExSxSxS = (float)(2.0f * sqrt(m->mom_inertia * m->E * m->nom_size * m->nom_size * m->nom_size));
}

/* Material import as CVX_Sim::Import + CopyMat do it (src/VXA/VX_Sim.cpp:73-86, 365-420,
 * 145-148; setters src/old/VX_Material.cpp:372-532). */
static void vmat_import(vmat *m, const vxo_material *in, const vxo_robot *r) {
    memset(m, 0, sizeof(*m));
    m->cilia = in->cilia;
    m->cilia_on_after = in->cilia_on_after;
    m->pacemaker = in->is_pacemaker;
    m->pace_period = in->pacemaker_period;
    m->sig_decay = in->signal_value_decay;
    m->sig_delay = in->signal_time_delay;
    m->inactive = in->inactive_period;
    m->remove_after = in->remove_after;
    m->sticky = in->sticky != 0;
    /* the model as CVX_Sim::CopyMat sets it (VX_Sim.cpp:390-409) */
    int ok = 0;
    if (in->model == 0) ok = curve_linear(&m->cv, (float)in->E, -1.0f);
    else if (in->model == 1) ok = curve_linear(&m->cv, (float)in->E, (float)in->fail_stress);
    else if (in->model == 2)
        ok = curve_bilinear(&m->cv, (float)in->E, (float)in->plastic_mod, (float)in->yield_stress, (float)in->fail_stress);
    else if (in->model == 3 && in->n_data > 0 && in->n_data < VXO_MAX_PTS) {
        float e[VXO_MAX_PTS], sg[VXO_MAX_PTS];
        for (int i = 0; i < in->n_data; i++) { e[i] = (float)in->strain_data[i]; sg[i] = (float)in->stress_data[i]; }
        ok = curve_points(&m->cv, in->n_data, e, sg);
    }
    if (!ok) curve_default(&m->cv);
    m->E = m->cv.E;
    m->sigma_fail = m->cv.sigma_fail;
    m->eps_fail = m->cv.eps_fail;
    float nu = (float)in->nu;
    if (nu < 0) nu = 0;
    if (nu >= 0.5) nu = 0.5 - FLT_EPSILON * 2;
    if (!r->volume_effects) nu = 0; /* EnableVolumeEffects(false) (VX_Sim.cpp:445-459) */
    m->nu = nu;
    float rho = (float)in->rho;
    if (rho <= 0) rho = FLT_MIN;
    m->rho = rho;
    m->cte = (float)in->cte;
    float ms = (float)in->mu_static, mk = (float)in->mu_kinetic;
    m->mu_s = ms <= 0 ? 0 : ms;
    m->mu_k = mk <= 0 ? 0 : mk;
    float zi = (float)r->bond_damping, zg = (float)r->slow_damping, zc = (float)r->col_damping;
    m->z_int = zi <= 0 ? 0 : zi;
    m->z_glob = zg <= 0 ? 0 : zg;
    m->z_col = zc <= 0 ? 0 : zc;
    m->nom_size = r->vox_size;
    /* CVX_Sim::SetGravityAccel (VX_Sim.cpp:485): gravity multiplier from GravAcc */
    float ga = (float)r->grav_acc;
    m->grav_mult = (float)(-ga / 9.80665);
    m->fixed = in->fixed;
    m->is_measured = in->is_measured;
    m->thermal_on_after = in->thermal_on_after;
    vmat_derive(m);
}

/* CVX_MaterialLink::updateAll + updateDerived (src/old/VX_MaterialLink.cpp:47-140) */
static void lmat_make(lmat *l, const vmat *v1, const vmat *v2, int i1, int i2) {
    l->m1 = i1;
    l->m2 = i2;
    curve_link(&l->cv, &v1->cv, &v2->cv);
    float E = l->cv.E;
    l->E = E;
    l->eps_fail = l->cv.eps_fail;
    l->cte = 0.5f * (v1->cte + v2->cte);
    float nu;
    if (v1->nu == 0 && v2->nu == 0) nu = 0;
    else {
        float tmpEHat = 2 * v1->eHat * v2->eHat / (v1->eHat + v2->eHat);
        float tmpE = E;
        float c2 = (tmpEHat - tmpE) / (2 * tmpEHat) + 0.0625;
        nu = sqrtf(c2) - 0.25;
    }
    l->nu = nu;
    l->eHat = ehat(E, nu);
    double nom = 0.5 * (v1->nom_size + v2->nom_size);
    float L = (float)nom;
    l->a1 = E * L;
    l->a2 = E * L * L * L / (12.0f * (1 + nu));
    l->b1 = E * L;
    l->b2 = E * L * L / 2.0f;
    l->b3 = E * L * L * L / 6.0f;
    l->sqA1 = sqrtf(l->a1);
    l->sqA2xIp = sqrtf(l->a2 * L * L / 6.0f);
    l->sqB1 = sqrtf(l->b1);
    l->sqB2xFMp = sqrtf(l->b2 * L / 2.0f);
    l->sqB3xIp = sqrtf(l->b3 * L * L / 6.0f);
}

/* ------------------------------------------------- boundary conditions */
/* A voxel's external (VX3_External): fixed DOFs with translation and rotation,
 * force and moment. */
typedef struct {
    int any, dof;
    float f[3], m[3];
    double t[3], r[3];
    quat q;
} vext;

/* CP_Box / CP_Cylinder / CP_Sphere ::IsTouching(P, Dist, Envelope) (src/old/VX_FRegion.cpp:395-605),
 * with Dist the half-cell vector: region coordinates in float, the rest in double */
static int bc_touch(const vxo_bc_region *b, const double P[3], const double D[3], const double W[3]) {
    if (b->prim == 0) {
        float hx = b->x + b->dx, hy = b->y + b->dy, hz = b->z + b->dz;
        double px = P[0] / W[0], py = P[1] / W[1], pz = P[2] / W[2];
        double dx = D[0] / W[0], dy = D[1] / W[1], dz = D[2] / W[2];
        return px + dx > b->x && px - dx < hx && py + dy > b->y && py - dy < hy && pz + dz > b->z && pz - dz < hz;
    }
    double wm = W[0] > W[1] ? W[0] : W[1];
    if (W[2] > wm) wm = W[2];
    double cx = b->x * W[0], cy = b->y * W[1], cz = b->z * W[2];
    double rad = b->radius * wm;
    if (b->prim == 2) {
        double dist = sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
        return sqrt((P[0] - cx) * (P[0] - cx) + (P[1] - cy) * (P[1] - cy) + (P[2] - cz) * (P[2] - cz)) < rad + dist;
    }
    double sx = b->dx * W[0], sy = b->dy * W[1], sz = b->dz * W[2];
    if (b->dx != 0) return P[0] > cx && P[0] < cx + sx && sqrt((P[1] - cy) * (P[1] - cy) + (P[2] - cz) * (P[2] - cz)) < rad;
    if (b->dy != 0) return P[1] > cy && P[1] < cy + sy && sqrt((P[0] - cx) * (P[0] - cx) + (P[2] - cz) * (P[2] - cz)) < rad;
    if (b->dz != 0) return P[2] > cz && P[2] < cz + sz && sqrt((P[0] - cx) * (P[0] - cx) + (P[1] - cy) * (P[1] - cy)) < rad;
    return 0;
}

/* ---------------------------------------------------------------- state */
enum { F_SURFACE = 1 << 1, F_FLOOR = 1 << 2, F_STATIC = 1 << 3 };
enum { L_LVV = 1 };

typedef struct {
    int mat, ix, iy, iz, links[6];
    vec pos, linMom, angMom, contact;
    quat orient;
    float tempe, prevDt;
    int flags;
    int removed; /* removeVoxels (SecondaryExperiment): no longer stepped, linked or collided */
    double phase;
    /* signals (VX3_Voxel.h:304-309): localSignal, localSignaldt, packmakerNextPulse,
     * inactiveUntil, the pending signal d_signal {value, activeTime}; all 0 at the start */
    double sig_local, sig_local_dt, pace_next, inactive_until, sig_value, sig_active;
    int stepped; /* reached the end of timeStep this step (signals run only there) */
    int attach_ok; /* VX3_Voxel::enableAttach: the attach conditions held after its last step (true at first) */
} voxel;

typedef struct {
    int neg, pos, axis, mat;
    vec pos2, a1v, a2v;
    vec fNeg, fPos, mNeg, mPos;
    float strain, maxStrain, area, tss;
    float strainOffset; /* plastic offset of a non-linear material (VX3_Link::strainOffset) */
    double rest;
    int small, states;
    int gone; /* detached (gpu_update_detach): no longer updated, no longer any voxel's link */
    int is_new; /* VX3_Link::isNewLink: updates left whose forces are scaled by 0.01 (runtime links) */
} link;

typedef struct {
    vxo_robot r;
    int nv, nl, nvm, nlm, ns;
    int nl0, lcap;            /* links of the lattice (recommendedTimeStep reads only those); capacity */
    vmat *vm;
    lmat *lm;
    voxel *v;
    link *l;
    int *surf;
    double *last_contact;
    double t, optimal_dt;
    float dt;
    int surface_stale, diverged;
    int threads; /* > 1: loops run under OpenMP */
    int exact;   /* with threads > 1: contact sums in the serial loop's order (else timing mode) */
    vxo_math_token *ff[3]; /* force-field programs (copies) or NULL */
    vec *cilia_base;       /* per voxel: BaseCiliaForce, or NULL */
    vec *cilia_shift;      /* per voxel: ShiftCiliaForce (scaled by localSignal), or NULL */
    int *mat_removed;      /* per material: removeVoxels has removed it (VX3_MaterialVoxel::removed) */
    vext *ext;             /* per voxel: boundary-condition externals, or NULL without regions */
    vxo_math_token *acond[5]; /* attach-condition programs (copies) or NULL */
} sim;

/* VX3_MathTree::eval (src/Utils/VX3_MathTree.h:50-191): tokens in order, each result
 * appended to a value queue, operators consuming the oldest unconsumed values (binary:
 * values[pc + 1] op values[pc]); hit, angle, targetCloseness, numClosePairs are 0 here
 * (the reference keeps collisionCount at 0; target tracking is not restated). */
#define VXO_MAX_TOKENS 256
static double math_eval(const vxo_math_token *tok, double x, double y, double z, double t, double num_voxel) {
    double vals[VXO_MAX_TOKENS];
    int vc = 0, pc = 0;
    for (int i = 0; i < VXO_MAX_TOKENS; i++) {
        double r, w;
        switch (tok[i].op) {
        case 0: return vals[pc < vc ? pc : 0];
        case 1: r = tok[i].value; break;
        case 2: r = 2.71828182845904523536; break;
        case 3: r = 3.14159265358979323846; break;
        case 4:
            w = tok[i].value;
            r = w < 0.5 ? x : w < 1.5 ? y : w < 2.5 ? z : (w >= 3.5 && w < 4.5) ? t : (w >= 7.5 && w < 8.5) ? num_voxel : 0.0;
            break;
        case 5: r = vals[pc + 1] + vals[pc]; pc += 2; break;
        case 6: r = vals[pc + 1] - vals[pc]; pc += 2; break;
        case 7: r = vals[pc + 1] * vals[pc]; pc += 2; break;
        case 8: r = vals[pc + 1] / vals[pc]; pc += 2; break;
        case 9: r = pow(vals[pc + 1], vals[pc]); pc += 2; break;
        case 10: r = sqrt(vals[pc]); pc++; break;
        case 11: r = sin(vals[pc]); pc++; break;
        case 12: r = cos(vals[pc]); pc++; break;
        case 13: r = tan(vals[pc]); pc++; break;
        case 14: r = atan(vals[pc]); pc++; break;
        case 15: r = log(vals[pc]); pc++; break;
        case 16: r = rint(vals[pc]); pc++; break;
        case 17: r = fabs(vals[pc]); pc++; break;
        case 18: r = !vals[pc]; pc++; break;
        case 19: r = vals[pc + 1] > vals[pc]; pc += 2; break;
        case 20: r = vals[pc + 1] < vals[pc]; pc += 2; break;
        case 21: r = vals[pc + 1] && vals[pc]; pc += 2; break;
        case 22: r = vals[pc + 1] || vals[pc]; pc += 2; break;
        case 23: r = 0.5 * erfc(-vals[pc] / sqrt(2.0)); pc++; break;
        default: return 0.0;
        }
        if (pc > vc) return 0.0;
        vals[vc++] = r;
    }
    return 0.0;
}

/* VX3_Voxel::baseSize(axis) (VX3_Voxel.h:96-100); material size() = nomSize*extScale(1,1,1) */
static double base_size(const sim *S, const voxel *v) {
    const vmat *m = &S->vm[v->mat];
    return m->nom_size * (1 + v->tempe * m->cte);
}
/* VX3_Voxel::baseSizeAverage (VX3_Voxel.h:102-105) */
static double base_size_avg(const sim *S, const voxel *v) {
    double b = base_size(S, v);
    return (b + b + b) / 3.0f;
}
/* VX3_Voxel::floorPenetration (VX3_Voxel.h:185-188) */
static float floor_pen(const sim *S, const voxel *v) {
    return (float)(base_size_avg(S, v) / 2 - S->vm[v->mat].nom_size / 2 - v->pos.z);
}
/* VX3_Link::updateRestLength (VX3_Link.cu:80-83) */
static void update_rest(sim *S, link *L) {
    L->rest = 0.5 * (base_size(S, &S->v[L->neg]) + base_size(S, &S->v[L->pos]));
}

/* Lattice -> voxels and links, CVX_Sim::Import / CVoxelyze::addVoxel / addLink
 * order (src/VXA/VX_Sim.cpp:88-107, src/old/Voxelyze.cpp:439-462, 508-539,
 * src/old/VX_Link.cpp:21-54): voxels in x-fastest scan order; each new voxel
 * links to already-present neighbours in direction order X_NEG, Y_NEG, Z_NEG
 * (the only earlier ones), pVNeg being the lower lattice index. */
void *vxo_create(const vxo_robot *r) {
    sim *S = (sim *)calloc(1, sizeof(sim));
    S->r = *r;
    S->r.cilia_base = S->r.cilia_shift = NULL;
    for (int k = 0; k < 3; k++) {
        S->r.force_field[k] = NULL;
        if (!r->force_field[k]) continue;
        int n = 0;
        while (n < VXO_MAX_TOKENS - 1 && r->force_field[k][n].op != 0) n++;
        S->ff[k] = (vxo_math_token *)calloc((size_t)n + 1, sizeof(vxo_math_token));
        memcpy(S->ff[k], r->force_field[k], sizeof(vxo_math_token) * (size_t)n);
    }
    for (int k = 0; k < 5; k++) {
        S->r.attach_cond[k] = NULL;
        if (!r->attach_cond[k]) continue;
        int n = 0;
        while (n < VXO_MAX_TOKENS - 1 && r->attach_cond[k][n].op != 0) n++;
        S->acond[k] = (vxo_math_token *)calloc((size_t)n + 1, sizeof(vxo_math_token));
        memcpy(S->acond[k], r->attach_cond[k], sizeof(vxo_math_token) * (size_t)n);
    }
    int nx = r->nx, ny = r->ny, nz = r->nz, ncell = nx * ny * nz;
    S->nvm = r->n_materials;
    S->vm = (vmat *)calloc(S->nvm ? S->nvm : 1, sizeof(vmat));
    for (int i = 0; i < S->nvm; i++) vmat_import(&S->vm[i], &r->materials[i], r);
    S->mat_removed = (int *)calloc(S->nvm ? S->nvm : 1, sizeof(int));

    /* initial temperature with Thermal/TempEnabled: CVX_Sim::UpdateMatTemps at import
     * (VXA/VX_Sim.cpp:467-478) sets every voxel to CVX_Environment::UpdateCurTemp(0) - TempBase
     * (old/VX_Environment.cpp:327-346): TempBase + TempAmplitude without VaryTempEnabled,
     * TempBase + TempAmplitude*sin(0) with it, 0 for a TempPeriod of 0; VX3_Voxel takes it over
     * (VX3_Voxel.cu:12) and, without varying temperature, keeps it */
    float temp0 = 0.0f;
    if (r->temp_enabled) {
        const double cur = r->vary_temp ? (r->temp_period == 0 ? 0.0 : r->temp_base + r->temp_amplitude * sin(0.0))
                                        : r->temp_base + r->temp_amplitude;
        temp0 = (float)((float)cur - r->temp_base);
    }
    int *vid = (int *)malloc(sizeof(int) * (ncell ? ncell : 1));
    S->nv = 0;
    for (int c = 0; c < ncell; c++) vid[c] = r->lattice[c] > 0 ? S->nv++ : -1;
    S->v = (voxel *)calloc(S->nv ? S->nv : 1, sizeof(voxel));
    S->lcap = 3 * (S->nv ? S->nv : 1);
    S->l = (link *)calloc((size_t)S->lcap, sizeof(link));
    S->lm = (lmat *)calloc((size_t)S->nvm * S->nvm + 1, sizeof(lmat));
    S->nl = 0;
    S->nlm = 0;
    for (int c = 0; c < ncell; c++) {
        if (vid[c] < 0) continue;
        int x = c % nx, y = (c / nx) % ny, z = c / (nx * ny);
        voxel *v = &S->v[vid[c]];
        v->mat = r->lattice[c] - 1;
        v->ix = x; v->iy = y; v->iz = z;
        /* CVoxelyze::addVoxel pos (Voxelyze.cpp:447); CVX_Voxel::reset (VX_Voxel.cpp:48-57) */
        v->pos = V(x * r->vox_size, y * r->vox_size, z * r->vox_size);
        v->orient = qident();
        v->flags = F_STATIC | (r->floor_enabled ? F_FLOOR : 0);
        v->tempe = temp0;
        v->prevDt = 0.0f;
        v->phase = r->phase ? r->phase[c] : 0.0;
        v->attach_ok = 1; /* VX3_Voxel.h:302 */
        for (int d = 0; d < 6; d++) v->links[d] = -1;
        int nb[3] = {x > 0 ? vid[c - 1] : -1, y > 0 ? vid[c - nx] : -1, z > 0 ? vid[c - nx * ny] : -1};
        for (int a = 0; a < 3; a++) {
            if (nb[a] < 0) continue;
            link *L = &S->l[S->nl];
            L->neg = nb[a];
            L->pos = vid[c];
            L->axis = a;
            /* CVoxelyze::combinedMaterial (Voxelyze.cpp:626-641): first use of a pair fixes
             * (vox1Mat, vox2Mat) = (new voxel's material, neighbour's material) */
            int m_new = v->mat, m_nb = S->v[nb[a]].mat, found = -1;
            for (int k = 0; k < S->nlm; k++)
                if ((S->lm[k].m1 == m_new && S->lm[k].m2 == m_nb) || (S->lm[k].m1 == m_nb && S->lm[k].m2 == m_new)) found = k;
            if (found < 0) {
                lmat_make(&S->lm[S->nlm], &S->vm[m_new], &S->vm[m_nb], m_new, m_nb);
                found = S->nlm++;
            }
            L->mat = found;
            L->small = 1;
            L->states = 0;
            /* CVX_Link::reset transverse info (VX_Link.cpp:56-71): voxels unstrained */
            float sz = (float)S->vm[v->mat].nom_size, sz2 = (float)S->vm[m_nb].nom_size;
            L->area = 0.5f * (sz2 * sz2 + sz * sz);
            L->tss = 0.0f;
            v->links[2 * a + 1] = S->nl;           /* new voxel: negative direction */
            S->v[nb[a]].links[2 * a] = S->nl;      /* neighbour: positive direction */
            S->nl++;
        }
    }
    if (r->enable_cilia) { /* VX_Sim.cpp:102-105: per-voxel cilia vectors in voxel order */
        S->cilia_base = (vec *)calloc(S->nv ? S->nv : 1, sizeof(vec));
        S->cilia_shift = (vec *)calloc(S->nv ? S->nv : 1, sizeof(vec));
        for (int c = 0; c < ncell; c++) {
            if (vid[c] < 0) continue;
            vec b = V(0, 0, 0), sh = V(0, 0, 0);
            if (r->cilia_base) b = V(r->cilia_base[3 * c], r->cilia_base[3 * c + 1], r->cilia_base[3 * c + 2]);
            if (r->cilia_shift) sh = V(r->cilia_shift[3 * c], r->cilia_shift[3 * c + 1], r->cilia_shift[3 * c + 2]);
            S->cilia_base[vid[c]] = b;
            S->cilia_shift[vid[c]] = sh;
        }
    }
    free(vid);
    /* boundary conditions (CVX_Sim::Import, src/VXA/VX_Sim.cpp:109-141): regions counted on
     * the GetXYZ cell centres (1e-6 lattice units further in x and y), applied to each voxel
     * touched at its position plus half a cell, in voxel then region order */
    S->r.bcs = NULL;
    if (r->n_bcs > 0) {
        double vs = r->vox_size;
        double W[3] = {vs * (double)nx, vs * (double)ny, vs * (double)nz}, H[3] = {0.5 * vs, 0.5 * vs, 0.5 * vs};
        int *size = (int *)calloc((size_t)r->n_bcs, sizeof(int));
        for (int j = 0; j < r->n_bcs; j++)
            for (int i = 0; i < S->nv; i++) {
                const voxel *v = &S->v[i];
                double P[3] = {vs * ((0.5 + v->ix) + 1e-6), vs * ((0.5 + v->iy) + 1e-6), vs * (0.5 + v->iz)};
                if (bc_touch(&r->bcs[j], P, H, W)) size[j]++;
            }
        S->ext = (vext *)calloc(S->nv ? S->nv : 1, sizeof(vext));
        for (int i = 0; i < S->nv; i++) {
            const voxel *v = &S->v[i];
            vext *e = &S->ext[i];
            e->q = qident();
            double P[3] = {v->ix * vs + H[0], v->iy * vs + H[1], v->iz * vs + H[2]};
            for (int j = 0; j < r->n_bcs; j++) {
                const vxo_bc_region *b = &r->bcs[j];
                if (!bc_touch(b, P, H, W)) continue;
                e->any = 1;
                for (int k = 0; k < 6; k++) { /* CVX_External::setDisplacement */
                    if (!(b->dof_fixed & (1 << k))) continue;
                    e->dof |= 1 << k;
                    double d = k < 3 ? b->displace[k] : b->ang_displace[k - 3];
                    if (d != 0.0f) { if (k < 3) e->t[k] = d; else e->r[k - 3] = d; }
                }
                double inv = 1.0 / (double)size[j];
                for (int k = 0; k < 3; k++) { /* addForce(force() + Force/Size): float sums */
                    float fa = (float)((double)e->f[k] + inv * b->force[k]);
                    float ma = (float)((double)e->m[k] + inv * b->torque[k]);
                    e->f[k] += fa;
                    e->m[k] += ma;
                }
            }
            if (e->r[0] != 0.0 || e->r[1] != 0.0 || e->r[2] != 0.0) e->q = q_from_rotvec(V(e->r[0], e->r[1], e->r[2]));
        }
        free(size);
    }
    for (int i = 0; i < S->nl; i++) update_rest(S, &S->l[i]);
    S->nl0 = S->nl;
    S->surf = (int *)malloc(sizeof(int) * (S->nv ? S->nv : 1));
    S->last_contact = (double *)calloc(3 * (size_t)(S->nv ? S->nv : 1), sizeof(double));
    S->surface_stale = 1;
    S->threads = 1;
    S->ns = 0;
    for (int i = 0; i < S->nv; i++) {
        int interior = 1;
        for (int d = 0; d < 6; d++) if (S->v[i].links[d] < 0) interior = 0;
        if (!interior) S->surf[S->ns++] = i;
    }
    return S;
}

void vxo_destroy(void *h) {
    sim *S = (sim *)h;
    if (!S) return;
    free(S->vm); free(S->lm); free(S->v); free(S->l); free(S->surf); free(S->last_contact);
    free(S->ff[0]); free(S->ff[1]); free(S->ff[2]); free(S->cilia_base); free(S->cilia_shift); free(S->mat_removed); free(S->ext);
    for (int k = 0; k < 5; k++) free(S->acond[k]);
    free(S);
}

/* VX3_Link::updateStrain (VX3_Link.cu:220-260): linear materials follow their law and
 * track maxStrain; non-linear ones follow the curve on new ground (recording the
 * strainOffset of the unloading line) and unload linearly below maxStrain */
static float link_strain_update(link *L, const lmat *m, float eps) {
    L->strain = eps;
    if (m->cv.linear) {
        if (eps > L->maxStrain) L->maxStrain = eps;
        return curve_stress(&m->cv, m->nu, m->eHat, eps, L->tss, 0);
    }
    if (eps > L->maxStrain) {
        L->maxStrain = eps;
        float st = curve_stress(&m->cv, m->nu, m->eHat, eps, L->tss, 0);
        if (m->nu != 0.0f)
            L->strainOffset = L->maxStrain - curve_stress(&m->cv, m->nu, m->eHat, eps, 0.0f, 0) / (m->eHat * (1 - m->nu));
        else
            L->strainOffset = L->maxStrain - st / m->E;
        return st;
    }
    float rel = eps - L->strainOffset;
    if (m->nu != 0.0f) return curve_stress(&m->cv, m->nu, m->eHat, rel, L->tss, 1);
    return m->E * rel;
}

/* VX3_Voxel::dampingMultiplier (VX3_Voxel.h:206-208) */
static float damping_mult(const sim *S, const voxel *v) {
    const vmat *m = &S->vm[v->mat];
    return 2 * m->sqrt_mass * m->z_int / v->prevDt;
}

/* VX3_Link::orientLink + updateForces + updateStrain (VX3_Link.cu:90-260) */
static void link_update(sim *S, link *L) {
    voxel *vn = &S->v[L->neg], *vp = &S->v[L->pos];
    const lmat *m = &S->lm[L->mat];
    vec oldPos2 = L->pos2, oldA1 = L->a1v, oldA2 = L->a2v;

    /* orientLink (:90-133) */
    vec pos2 = to_axis_x(L->axis, vsub(vp->pos, vn->pos));
    quat angle1 = to_axis_xq(L->axis, vn->orient);
    quat angle2 = to_axis_xq(L->axis, vp->orient);
    quat totalRot = qconj(angle1);
    pos2 = qrot(totalRot, pos2);
    angle2 = qmul(totalRot, angle2);
    angle1 = qident();
    float SmallTurn = (float)((fabs(pos2.z) + fabs(pos2.y)) / pos2.x);
    float ExtendPerc = (float)(fabs(1 - pos2.x / L->rest));
    const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;
    if (!L->small && SmallTurn < BEND && ExtendPerc < EXT) {
        L->small = 1;
        L->states &= ~L_LVV;
    } else if (L->small && (SmallTurn > HF * BEND || ExtendPerc > HF * EXT)) {
        L->small = 0;
        L->states &= ~L_LVV;
    }
    if (L->small) {
        pos2.x -= L->rest;
    } else {
        angle1 = q_from_angle_to_posx(angle1, pos2);
        angle2 = qmul(angle1, angle2);
        pos2 = V(vlen(pos2) - L->rest, 0, 0);
    }
    vec a1v = q_to_rotvec(angle1), a2v = q_to_rotvec(angle2);
    L->pos2 = pos2; L->a1v = a1v; L->a2v = a2v;

    /* updateForces (:135-218) */
    vec dPos2 = vscale(vsub(pos2, oldPos2), 0.5);
    vec dA1 = vscale(vsub(a1v, oldA1), 0.5);
    vec dA2 = vscale(vsub(a2v, oldA2), 0.5);
    /* updateStrain (:220-260) */
    float axialStrain = (float)(pos2.x / L->rest);
    float stress = link_strain_update(L, m, axialStrain);
    if (m->eps_fail != -1.0f && L->maxStrain > m->eps_fail) { /* isFailed */
        L->fNeg = L->fPos = L->mNeg = L->mPos = V(0, 0, 0);
        return;
    }
    float b1 = m->b1, b2 = m->b2, b3 = m->b3, a2 = m->a2;
    vec fNeg = V(stress * L->area, b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y));
    vec fPos = vneg(fNeg);
    vec mNeg = V(a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z));
    vec mPos = V(a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z));
    if (L->states & L_LVV) {
        float sqA1 = m->sqA1, sqA2xIp = m->sqA2xIp, sqB1 = m->sqB1, sqB2xFMp = m->sqB2xFMp, sqB3xIp = m->sqB3xIp;
        vec posCalc = V(sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z), sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y));
        float dmN = damping_mult(S, vn), dmP = damping_mult(S, vp);
        fNeg = vadd(fNeg, vscale(posCalc, dmN));
        fPos = vsub(fPos, vscale(posCalc, dmP));
        mNeg = vsub(mNeg, vscale(V(-sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (2 * dA1.y + dA2.y),
                                   -sqB2xFMp * dPos2.y + sqB3xIp * (2 * dA1.z + dA2.z)), 0.5 * dmN));
        mPos = vsub(mPos, vscale(V(sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (dA1.y + 2 * dA2.y),
                                   -sqB2xFMp * dPos2.y + sqB3xIp * (dA1.z + 2 * dA2.z)), 0.5 * dmP));
    } else {
        L->states |= L_LVV;
    }
    if (!L->small) {
        fNeg = qrotinv(angle1, fNeg);
        mNeg = qrotinv(angle1, mNeg);
    }
    fPos = qrotinv(angle2, fPos);
    mPos = qrotinv(angle2, mPos);
    L->fNeg = to_axis_original(L->axis, fNeg);
    L->fPos = to_axis_original(L->axis, fPos);
    L->mNeg = to_axis_original(L->axis, mNeg);
    L->mPos = to_axis_original(L->axis, mPos);
    if (L->is_new) { /* a runtime link's first SafetyGuard updates (VX3_Link.cu:206-213) */
        L->fNeg = vscale(L->fNeg, 0.01);
        L->fPos = vscale(L->fPos, 0.01);
        L->mNeg = vscale(L->mNeg, 0.01);
        L->mPos = vscale(L->mPos, 0.01);
        L->is_new -= 1;
    }
}

/* VX3_Voxel::floorForce (VX3_Voxel.cu:399-426) */
static void floor_force(const sim *S, voxel *v, vec *F) {
    const vmat *m = &S->vm[v->mat];
    float pen = floor_pen(S, v);
    if (pen >= 0) {
        vec vel = vscale(v->linMom, m->mass_inv);
        vec hv = V(vel.x, vel.y, 0);
        float pstiff = (float)(2 * m->E * m->nom_size);
        float normal = pstiff * pen;
        F->z += normal - (m->z_col * m->c2xSqMxExS) * vel.z;
        if (v->flags & F_STATIC) {
            float surf = (float)(F->x * F->x + F->y * F->y);
            float fric = (m->mu_s * normal) * (m->mu_s * normal);
            if (surf > fric) v->flags &= ~F_STATIC;
        } else {
            *F = vsub(*F, vscale(vnormalized(hv), m->mu_k * normal));
        }
    } else {
        v->flags &= ~F_STATIC;
    }
}

/* VX3_Voxel::timeStep with force()/moment() (VX3_Voxel.cu:162-277, 350-397) */
static void voxel_update(sim *S, voxel *v, float dtf) {
    const vmat *m = &S->vm[v->mat];
    double dt = dtf;
    v->prevDt = (float)dt;
    v->stepped = 0;
    if (dt == 0.0f) return;
    const vext *ex = S->ext && S->ext[v - S->v].any ? &S->ext[v - S->v] : NULL;
    if (ex && ex->dof == 0x3F) { /* isFixedAll (VX3_Voxel.cu:167-173) */
        double s = m->nom_size;
        v->pos = V(v->ix * s + ex->t[0], v->iy * s + ex->t[1], v->iz * s + ex->t[2]);
        v->orient = ex->q;
        v->linMom = v->angMom = V(0, 0, 0);
        return;
    }
    /* force() */
    vec F = V(0, 0, 0);
    for (int i = 0; i < 6; i++) {
        if (v->links[i] < 0) continue;
        const link *L = &S->l[v->links[i]];
        F = vadd(F, (i % 2 == 1) ? L->fPos : L->fNeg);
    }
    F = qrot(v->orient, F);
    if (ex) F = vadd(F, V(ex->f[0], ex->f[1], ex->f[2])); /* external force (VX3_Voxel.cu:363-364) */
    vec vel = vscale(v->linMom, m->mass_inv);
    F = vsub(F, vscale(vel, m->z_glob * m->c2xSqMxExS));
    F.z += -m->mass * 9.80665f * m->grav_mult;
    F = vsub(F, v->contact);
    v->contact = V(0, 0, 0);
    {   /* CiliaForce * Cilia (VX3_Voxel.cu:376); CiliaForce from gpu_update_cilia_force
         * (VX3_VoxelyzeKernel.cu:846-859) for surface voxels, before the voxel pass */
        vec cf = V(0, 0, 0);
        if (S->cilia_base && !(v->flags & F_SURFACE) && m->cilia != 0 && !(m->cilia_on_after > S->t))
            cf = qrot(v->orient, vadd(S->cilia_base[v - S->v], vscale(S->cilia_shift[v - S->v], v->sig_local)));
        F = vadd(F, vscale(cf, m->cilia));
    }
    /* force field (VX3_Voxel.cu:178-184; constant 0 unless the VXA gives one) */
    F.x += S->ff[0] ? math_eval(S->ff[0], v->pos.x, v->pos.y, v->pos.z, S->t, S->nv) : 0.0;
    F.y += S->ff[1] ? math_eval(S->ff[1], v->pos.x, v->pos.y, v->pos.z, S->t, S->nv) : 0.0;
    F.z += S->ff[2] ? math_eval(S->ff[2], v->pos.x, v->pos.y, v->pos.z, S->t, S->nv) : 0.0;
    vec fric = F;
    if (v->flags & F_FLOOR) floor_force(S, v, &F);
    fric = vsub(F, fric);
    v->linMom = vadd(v->linMom, vscale(F, dt));
    vec translate = vscale(v->linMom, dt * m->mass_inv);
    if ((v->flags & F_FLOOR) && floor_pen(S, v) >= 0) {
        double work = fric.x * translate.x + fric.y * translate.y;
        double hKe = 0.5 * m->mass_inv * (v->linMom.x * v->linMom.x + v->linMom.y * v->linMom.y);
        if (hKe + work <= 0) v->flags |= F_STATIC;
        if (v->flags & F_STATIC) {
            v->linMom.x = v->linMom.y = 0;
            translate.x = translate.y = 0;
        }
    } else {
        v->flags &= ~F_STATIC;
    }
    v->pos = vadd(v->pos, translate);
    /* moment() */
    vec M = V(0, 0, 0);
    for (int i = 0; i < 6; i++) {
        if (v->links[i] < 0) continue;
        const link *L = &S->l[v->links[i]];
        M = vadd(M, (i % 2 == 1) ? L->mPos : L->mNeg);
    }
    M = qrot(v->orient, M);
    if (ex) M = vadd(M, V(ex->m[0], ex->m[1], ex->m[2])); /* external moment (:393-394) */
    vec angVel = vscale(v->angMom, m->mom_inertia_inv);
    M = vsub(M, vscale(angVel, m->z_glob * m->c2xSqIxExSxSxS));
    v->angMom = vadd(v->angMom, vscale(M, dt));
    v->orient = qmul(q_from_rotvec(vscale(v->angMom, dt * m->mom_inertia_inv)), v->orient);
    if (ex) { /* fixed DOFs (VX3_Voxel.cu:222-257) */
        double s = m->nom_size;
        if (ex->dof & 1) { v->pos.x = v->ix * s + ex->t[0]; v->linMom.x = 0; }
        if (ex->dof & 2) { v->pos.y = v->iy * s + ex->t[1]; v->linMom.y = 0; }
        if (ex->dof & 4) { v->pos.z = v->iz * s + ex->t[2]; v->linMom.z = 0; }
        if (ex->dof & 0x38) {
            if ((ex->dof & 0x38) == 0x38) {
                v->orient = ex->q;
                v->angMom = V(0, 0, 0);
            } else {
                vec rv = q_to_rotvec(v->orient);
                if (ex->dof & 8) { rv.x = 0; v->angMom.x = 0; }
                if (ex->dof & 16) { rv.y = 0; v->angMom.y = 0; }
                if (ex->dof & 32) { rv.z = 0; v->angMom.z = 0; }
                v->orient = q_from_rotvec(rv);
            }
        }
    }
    if ((v->flags & F_FLOOR) && floor_pen(S, v) >= 0) {
        if (v->flags & F_STATIC) v->angMom = V(0, 0, 0);
    }
    v->stepped = 1;
}

/* ------------------------------------------------------------------ signals */
/* VX3_Voxel::receiveSignal (VX3_Voxel.cu:301-322): the receiving voxel's material */
static void sig_receive(sim *S, voxel *v, double value, double active_time, int force) {
    const vmat *m = &S->vm[v->mat];
    if (!force && v->inactive_until > active_time) return;
    if (value < 0.1) return;
    v->inactive_until = active_time + m->inactive;
    v->sig_local = value;
    v->sig_value = value * m->sig_decay;
    if (v->sig_value < 0.1) v->sig_value = 0;
    v->sig_active = active_time;
}

/* the end of VX3_Voxel::timeStep with EnableSignals (VX3_Voxel.cu:271-276): propagateSignal
 * (:323-348; to the voxel at the other end of each link, in direction order), packMaker
 * (:291-299), localSignalDecay (:279-289).  They change only signal state, which the step's
 * physics does not read, so running them for every voxel in voxel order after the voxel
 * pass is the serial loop's result. */
static void voxel_signals(sim *S, voxel *v) {
    const vmat *m = &S->vm[v->mat];
    const double t = S->t;
    if (!(v->sig_active > t) && !(v->sig_value < 0.1)) {
        for (int d = 0; d < 6; d++) {
            if (v->links[d] < 0) continue;
            const link *L = &S->l[v->links[d]];
            voxel *o = &S->v[(&S->v[L->neg] == v) ? L->pos : L->neg];
            sig_receive(S, o, v->sig_value, t + m->sig_delay, 0);
        }
        v->sig_value = 0;
        v->sig_active = 0;
        v->inactive_until = t + 2 * m->sig_delay + m->inactive;
    }
    if (m->pacemaker && !(v->pace_next > t)) {
        sig_receive(S, v, 100, t, 1);
        v->pace_next = t + m->pace_period;
    }
    if (!(v->sig_local_dt > t)) {
        if (v->sig_local < 0.1) v->sig_local = 0;
        else {
            v->sig_local = v->sig_local * 0.9;
            v->sig_local_dt = t + 0.01;
        }
    }
}

/* recommendedTimeStep with axialStiffness (VX3_VoxelyzeKernel.cu:184-217, VX3_Link.cu:269-278) */
double vxo_recommended_dt(void *h) {
    sim *S = (sim *)h;
    double MaxFreq2 = 0.0f;
    for (int i = 0; i < S->nl0; i++) { /* the lattice's links (num_d_links), not runtime ones */
        link *L = &S->l[i];
        const lmat *m = &S->lm[L->mat];
        double m1 = S->vm[S->v[L->neg].mat].mass, m2 = S->vm[S->v[L->pos].mat].mass;
        float k;
        if (m->nu == 0.0f) k = m->a1;
        else {
            update_rest(S, L);
            k = (float)(m->eHat * L->area / ((L->strain + 1) * L->rest));
        }
        double f2 = k / (m1 < m2 ? m1 : m2);
        if (f2 > MaxFreq2) MaxFreq2 = f2;
    }
    if (MaxFreq2 <= 0.0f) {
        for (int i = 0; i < S->nv; i++) {
            const vmat *m = &S->vm[S->v[i].mat];
            double f2 = m->E * m->nom_size / m->mass;
            if (f2 > MaxFreq2) MaxFreq2 = f2;
        }
    }
    if (MaxFreq2 <= 0.0f) return 0.0f;
    return 1.0f / (6.283185f * sqrt(MaxFreq2));
}

static int is_linked(const sim *S, int a, int b) {
    for (int d = 0; d < 6; d++) {
        int li = S->v[a].links[d];
        if (li < 0) continue;
        int o = S->l[li].neg == a ? S->l[li].pos : S->l[li].neg;
        if (o == b) return 1;
    }
    return 0;
}

/* handle_collision_attachment (collision half) + VX3_Collision
 * (VX3_VoxelyzeKernel.cu:682-727, VX3_Collision.cu:3-31) */
/* the contact force of one surface pair (voxel1 = v1, the later in surface order): 1 with
 * the force in *out; 0 where the reference's handle_collision_attachment leaves the pair
 * before any contact (VX3_VoxelyzeKernel.cu:682-727, VX3_Collision.cu:3-31); 2 where it
 * passes the pair on to the attachment half without a contact (EnableCollision off) */
static int pair_force(const sim *S, const voxel *v1, const voxel *v2, int i1, int i2, double bsa1, double bsa2,
                      vec *out) {
    const vmat *m1 = &S->vm[v1->mat], *m2 = &S->vm[v2->mat];
    if (m1->fixed && m2->fixed) return 0;
    vec diff = vsub(v1->pos, v2->pos);
    double wd = (bsa1 + bsa2) * 0.625;
    if (diff.x > wd || diff.x < -wd) return 0;
    if (diff.y > wd || diff.y < -wd) return 0;
    if (diff.z > wd || diff.z < -wd) return 0;
    if (vlen(diff) > wd) return 0;
    if (is_linked(S, i1, i2)) return 0;
    if (!S->r.enable_collision) return 2;
    float k1 = (float)(2 * m1->E * m1->nom_size), k2 = (float)(2 * m2->E * m2->nom_size);
    double pstiff = 2.0f / (1.0f / k1 + 1.0f / k2);
    double dampC = 0.5f * (m1->z_col * m1->c2xSqMxExS + m2->z_col * m2->c2xSqMxExS);
    vec offset = vsub(v2->pos, v1->pos);
    double nom = (double)((bsa1 + bsa2) * 0.625);
    double rel = nom - vlen(offset);
    vec f = V(0, 0, 0);
    if (rel > 0) {
        vec u = vnormalized(offset);
        double rv = vdot(vscale(v1->linMom, m1->mass_inv), u) - vdot(vscale(v2->linMom, m2->mass_inv), u);
        f = vscale(u, pstiff * rel + dampC * rv);
    }
    *out = f;
    return 1;
}

static void attach_pair(sim *S, int i1, int i2, int had_contact, vec f);

static void collide(sim *S, voxel *v1, voxel *v2, int i1, int i2) {
    vec f = V(0, 0, 0);
    const int rc = pair_force(S, v1, v2, i1, i2, base_size_avg(S, v1), base_size_avg(S, v2), &f);
    if (!rc) return;
    if (rc == 1) {
        v1->contact = vadd(v1->contact, f);
        v2->contact = vadd(v2->contact, vneg(f));
    }
    if (S->r.enable_attach) attach_pair(S, i1, i2, rc == 1, f);
}

/* is_neighbor (VX3_VoxelyzeKernel.cu:651-680): b within `depth` links of a, never going
 * straight back over the link just taken */
static int within_links(const sim *S, int a, int b, int incoming, int depth) {
    if (a == b) return 1;
    if (depth <= 0) return 0;
    for (int d = 0; d < 6; d++) {
        const int li = S->v[a].links[d];
        if (li < 0 || li == incoming) continue;
        const link *L = &S->l[li];
        if (within_links(S, L->neg == a ? L->pos : L->neg, b, li, depth - 1)) return 1;
    }
    return 0;
}

/* VX3_VoxelyzeKernel::combinedMaterial (:515-528) for two voxels of one material m: the
 * link material of the pair (m, m), made on first use */
static int lmat_same(sim *S, int m) {
    for (int k = 0; k < S->nlm; k++)
        if (S->lm[k].m1 == m && S->lm[k].m2 == m) return k;
    lmat_make(&S->lm[S->nlm], &S->vm[m], &S->vm[m], m, m);
    return S->nlm++;
}

/* the attachment half of handle_collision_attachment (VX3_VoxelyzeKernel.cu:729-830), for a
 * pair that passed the envelope and direct-neighbour tests: two enableAttach voxels of one
 * Sticky, unfixed material more than five links apart get a new link along the dominant
 * axis of voxel2's offset in voxel1's frame, if both of those faces are free; the pair's
 * contact of this step is taken back.  The new link is the device constructor's
 * (VX3_Link.cu:31-56) after reset() (:58-70): zero state, small-angle, no valid local
 * velocity, rest length from both base sizes, transverse area of two unstrained faces
 * (the material's Poisson's ratio is 0), isNewLink = SafetyGuard. */
static void attach_pair(sim *S, int i1, int i2, int had_contact, vec f) {
    voxel *v1 = &S->v[i1], *v2 = &S->v[i2];
    if (!v1->attach_ok || !v2->attach_ok) return;
    const vmat *m1 = &S->vm[v1->mat];
    if (m1->fixed || S->vm[v2->mat].fixed) return;
    if (v1->mat != v2->mat) return;
    if (!m1->sticky) return;
    if (within_links(S, i1, i2, -1, 5)) return;
    const vec ea = qrotinv(v1->orient, vneg(vsub(v1->pos, v2->pos)));
    const vec fa = V(fabs(ea.x), fabs(ea.y), fabs(ea.z));
    int axis, rev;
    if (fa.x >= fa.y && fa.x >= fa.z) axis = 0, rev = ea.x < 0;
    else if (fa.y >= fa.x && fa.y >= fa.z) axis = 1, rev = ea.y < 0;
    else axis = 2, rev = ea.z < 0;
    const int d1 = 2 * axis + (rev ? 1 : 0), d2 = 2 * axis + (rev ? 0 : 1);
    if (v1->links[d1] >= 0 || v2->links[d2] >= 0) return;
    if (S->nl == S->lcap) {
        S->lcap *= 2;
        S->l = (link *)realloc(S->l, sizeof(link) * (size_t)S->lcap);
    }
    link *L = &S->l[S->nl];
    memset(L, 0, sizeof(*L));
    L->neg = rev ? i2 : i1; /* the voxel on the axis' negative side */
    L->pos = rev ? i1 : i2;
    L->axis = axis;
    L->mat = lmat_same(S, v1->mat);
    L->small = 1;
    L->states = 0;
    update_rest(S, L);
    const float sz = (float)m1->nom_size;
    L->area = 0.5f * (sz * sz + sz * sz);
    L->tss = 0.0f;
    L->is_new = S->r.safety_guard;
    v1->links[d1] = S->nl;
    v2->links[d2] = S->nl;
    S->nl++;
    S->surface_stale = 1;
    if (had_contact) {
        v1->contact = vsub(v1->contact, f);
        v2->contact = vsub(v2->contact, vneg(f));
    }
}

/* The serial pair loop adds to the contact of surface voxel k first its pairs (k, b),
 * b < k ascending, as voxel1, then the pairs (a, k), a > k ascending, as voxel2.  Each
 * voxel gathers its own sum in that order here, so rows run in parallel with the serial
 * loop's result bit for bit (every pair's force is evaluated once from each side). */
static void collide_gather_threaded(sim *S) {
    /* surface positions and base sizes, compact, for the box test that rejects most pairs
     * (the same doubles and comparisons as pair_force, which repeats them for the rest) */
    const int ns = S->ns;
    double *c = (double *)malloc(sizeof(double) * 4 * (ns ? ns : 1));
    for (int k = 0; k < ns; k++) {
        const voxel *v = &S->v[S->surf[k]];
        c[4 * k] = v->pos.x; c[4 * k + 1] = v->pos.y; c[4 * k + 2] = v->pos.z;
        c[4 * k + 3] = base_size_avg(S, v);
    }
#pragma omp parallel for schedule(dynamic, 32)
    for (int k = 0; k < ns; k++) {
        const int ik = S->surf[k];
        voxel *vk = &S->v[ik];
        const double *ck = c + 4 * k;
        vec acc = vk->contact, f;
        for (int b = 0; b < k; b++) {  /* (k, b): k is voxel1 */
            const double *cb = c + 4 * b;
            double wd = (ck[3] + cb[3]) * 0.625, dx = ck[0] - cb[0], dy = ck[1] - cb[1], dz = ck[2] - cb[2];
            if (dx > wd || dx < -wd || dy > wd || dy < -wd || dz > wd || dz < -wd) continue;
            if (pair_force(S, vk, &S->v[S->surf[b]], ik, S->surf[b], ck[3], cb[3], &f)) acc = vadd(acc, f);
        }
        for (int a = k + 1; a < ns; a++) {  /* (a, k): k is voxel2 */
            const double *ca = c + 4 * a;
            double wd = (ca[3] + ck[3]) * 0.625, dx = ca[0] - ck[0], dy = ca[1] - ck[1], dz = ca[2] - ck[2];
            if (dx > wd || dx < -wd || dy > wd || dy < -wd || dz > wd || dz < -wd) continue;
            if (pair_force(S, &S->v[S->surf[a]], vk, S->surf[a], ik, ca[3], ck[3], &f)) acc = vadd(acc, vneg(f));
        }
        vk->contact = acc;
    }
    free(c);
}

/* The same all-pairs loop with rows spread over threads (timing mode only:
 * contact sums then depend on thread interleaving). */
static void collide_rows_threaded(sim *S, int row_begin, int row_end) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int a = row_begin; a < row_end; a++) {
        for (int b = 0; b < a; b++) {
            voxel *v1 = &S->v[S->surf[a]], *v2 = &S->v[S->surf[b]];
            vec c1 = v1->contact, c2 = v2->contact;
            collide(S, v1, v2, S->surf[a], S->surf[b]);
            vec d1 = vsub(v1->contact, c1), d2 = vsub(v2->contact, c2);
            if (d1.x != 0 || d1.y != 0 || d1.z != 0) {
#pragma omp critical(vxo_contact)
                {
                    v1->contact = vadd(c1, d1);
                    v2->contact = vadd(c2, d2);
                }
            }
        }
    }
}

/* removeVoxels (VX3_VoxelyzeKernel.cu:365-397), at the end of a step of a SecondaryExperiment
 * (:335-349), before the time advances: every voxel of a material whose
 * RemoveFromSimulationAfterThisManySeconds (> 0) is below the current time leaves the
 * simulation together with its links; the surface is regenerated in the next step. */
static void remove_voxels(sim *S) {
    for (int i = 0; i < S->nvm; i++) {
        const vmat *m = &S->vm[i];
        if (S->mat_removed[i] || !(m->remove_after > 0) || !(m->remove_after < S->t)) continue;
        for (int j = 0; j < S->nv; j++) {
            voxel *v = &S->v[j];
            if (v->mat != i || v->removed) continue;
            v->removed = 1;
            for (int k = 0; k < 6; k++) {
                const int li = v->links[k];
                if (li < 0) continue;
                link *L = &S->l[li];
                L->gone = 1; /* VX3_Link::removed: skipped by the link and detach passes */
                voxel *nb = &S->v[L->neg == j ? L->pos : L->neg];
                for (int q = 0; q < 6; q++)
                    if (nb->links[q] == li) { nb->links[q] = -1; break; }
                v->links[k] = -1;
            }
        }
        S->mat_removed[i] = 1;
        S->surface_stale = 1;
    }
}

/* doTimeStep (VX3_VoxelyzeKernel.cu:237-359) */
static int do_step(sim *S) {
    const vxo_robot *r = &S->r;
    /* gpu_update_temperature (:625-650) + setTemperature (VX3_Voxel.cu:107-113) */
    if (r->vary_temp && r->temp_period > 0 && S->threads > 1) {
        /* threaded: every temperature first, then every rest length (the values the serial
         * loop leaves, each link's later end seeing both new temperatures) */
#pragma omp parallel for schedule(static)
        for (int i = 0; i < S->nv; i++) {
            voxel *v = &S->v[i];
            const vmat *m = &S->vm[v->mat];
            if (v->removed || m->thermal_on_after > S->t || m->fixed) continue;
            double T = r->temp_amplitude * sin(2 * 3.1415926f * (S->t / r->temp_period + v->phase));
            if (!r->enable_expansion && T > 0) T = 0;
            v->tempe = (float)T;
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < S->nl; i++) {
            const link *L = &S->l[i];
            const voxel *a = &S->v[L->neg], *b = &S->v[L->pos];
            const vmat *ma = &S->vm[a->mat], *mb = &S->vm[b->mat];
            int ua = !(a->removed || ma->thermal_on_after > S->t || ma->fixed);
            int ub = !(b->removed || mb->thermal_on_after > S->t || mb->fixed);
            int attached = 0;
            for (int d = 0; d < 6; d++) attached |= (ua && a->links[d] == i) || (ub && b->links[d] == i);
            if (attached) update_rest(S, &S->l[i]);
        }
    } else if (r->vary_temp && r->temp_period > 0) {
        for (int i = 0; i < S->nv; i++) {
            voxel *v = &S->v[i];
            const vmat *m = &S->vm[v->mat];
            if (v->removed) continue;
            if (m->thermal_on_after > S->t) continue;
            if (m->fixed) continue;
            double T = r->temp_amplitude * sin(2 * 3.1415926f * (S->t / r->temp_period + v->phase));
            if (!r->enable_expansion && T > 0) T = 0;
            v->tempe = (float)T;
            for (int d = 0; d < 6; d++)
                if (v->links[d] >= 0) update_rest(S, &S->l[v->links[d]]);
        }
    }
    if (!S->optimal_dt) S->optimal_dt = vxo_recommended_dt(S);
    if (S->optimal_dt < 1e-10) S->optimal_dt = 1e-10;
    float dt = S->r.dt_frac * S->optimal_dt;
    S->dt = dt;
    /* gpu_update_links (:566-581), divergence over every link */
    int div = 0;
#pragma omp parallel for if (S->threads > 1) schedule(static) reduction(| : div)
    for (int i = 0; i < S->nl; i++) {
        link *L = &S->l[i];
        if (L->gone) continue;
        if (S->vm[S->v[L->neg].mat].fixed && S->vm[S->v[L->pos].mat].fixed) continue;
        link_update(S, L);
        if (L->strain > 100) div = 1;
    }
    if (div) return 0;
    /* regenerateSurfaceVoxels (:495-513, VX3_Voxel.cu:515-524) */
    if (S->surface_stale) {
        S->surface_stale = 0;
        S->ns = 0;
        for (int i = 0; i < S->nv; i++) {
            int interior = 1;
            for (int d = 0; d < 6; d++) if (S->v[i].links[d] < 0) interior = 0;
            if (interior) S->v[i].flags |= F_SURFACE; else S->v[i].flags &= ~F_SURFACE;
            if (!interior && !S->v[i].removed) S->surf[S->ns++] = i;
        }
    }
    /* gpu_update_attach (:833-843): pairs first > second in surface order; with
     * attachment the serial loop itself (links made by earlier pairs count for later ones) */
    if (r->enable_attach) {
        for (int a = 0; a < S->ns; a++)
            for (int b = 0; b < a; b++) collide(S, &S->v[S->surf[a]], &S->v[S->surf[b]], S->surf[a], S->surf[b]);
    } else if (r->enable_collision) {
        if (S->threads > 1 && S->exact) collide_gather_threaded(S);
        else if (S->threads > 1) collide_rows_threaded(S, 0, S->ns);
        else
            for (int a = 0; a < S->ns; a++)
                for (int b = 0; b < a; b++) collide(S, &S->v[S->surf[a]], &S->v[S->surf[b]], S->surf[a], S->surf[b]);
    }
    /* gpu_update_detach (:946-967), after the collision pass: a failed link leaves both
     * voxels' link tables; the surface is regenerated at the start of the next step */
    if (r->enable_detach) {
        for (int i = 0; i < S->nl; i++) {
            link *L = &S->l[i];
            if (L->gone) continue;
            const lmat *m = &S->lm[L->mat];
            if (!(m->eps_fail != -1.0f && L->maxStrain > m->eps_fail)) continue; /* VX3_Link::isFailed */
            L->gone = 1;
            for (int d = 0; d < 6; d++) {
                if (S->v[L->neg].links[d] == i) S->v[L->neg].links[d] = -1;
                if (S->v[L->pos].links[d] == i) S->v[L->pos].links[d] = -1;
            }
            S->surface_stale = 1;
        }
    }
    for (int i = 0; i < S->nv; i++) {
        S->last_contact[3 * i] = S->v[i].contact.x;
        S->last_contact[3 * i + 1] = S->v[i].contact.y;
        S->last_contact[3 * i + 2] = S->v[i].contact.z;
    }
    /* gpu_update_voxels (:582-623) */
#pragma omp parallel for if (S->threads > 1) schedule(static)
    for (int i = 0; i < S->nv; i++) {
        if (S->v[i].removed) continue;
        if (S->vm[S->v[i].mat].fixed) continue;
        voxel_update(S, &S->v[i], dt);
    }
    if (r->enable_attach) /* gpu_update_voxels (:606-621): enableAttach after the voxel's step */
        for (int i = 0; i < S->nv; i++) {
            voxel *v = &S->v[i];
            if (v->removed || S->vm[v->mat].fixed) continue;
            int ok = 1;
            for (int k = 0; k < 5 && ok; k++)
                if (S->acond[k] && !(math_eval(S->acond[k], v->pos.x, v->pos.y, v->pos.z, S->t, S->nv) > 0)) ok = 0;
            v->attach_ok = ok;
        }
    if (r->enable_signals)  /* in voxel order, after the voxel pass (see voxel_signals) */
        for (int i = 0; i < S->nv; i++)
            if (S->v[i].stepped && !S->v[i].removed && !S->vm[S->v[i].mat].fixed) voxel_signals(S, &S->v[i]);
    if (r->secondary_experiment) remove_voxels(S);
    S->t += dt;
    return 1;
}

void vxo_signals(void *h, double *out) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nv; i++) out[i] = S->v[i].sig_local;
}

int vxo_step(void *h, int n) {
    sim *S = (sim *)h;
    int done = 0;
    for (int i = 0; i < n && !S->diverged; i++) {
        if (!do_step(S)) { S->diverged = 1; break; }
        done++;
    }
    return done;
}

void vxo_set_threads(void *h, int n) {
    sim *S = (sim *)h;
    S->threads = n > 1 ? n : 1;
    S->exact = 0;
#ifdef _OPENMP
    if (n > 1) omp_set_num_threads(n);
#endif
}

void vxo_set_exact_threads(void *h, int n) {
    vxo_set_threads(h, n);
    ((sim *)h)->exact = 1;
}

/* Seconds spent by the all-pairs collision loop over surface rows [begin, end)
 * (each row tests all earlier surface voxels); used to time a bounded sample
 * of the O(S^2) broad phase. Contact sums are cleared afterwards. */
double vxo_time_collision_rows(void *h, int begin, int end) {
    sim *S = (sim *)h;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (S->threads > 1) collide_rows_threaded(S, begin, end);
    else
        for (int a = begin; a < end; a++)
            for (int b = 0; b < a; b++) collide(S, &S->v[S->surf[a]], &S->v[S->surf[b]], S->surf[a], S->surf[b]);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    for (int i = 0; i < S->nv; i++) S->v[i].contact = V(0, 0, 0);
    return (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
}

/* Steps without the collision pass (to time the link and voxel passes alone). */
int vxo_step_no_collision(void *h, int n) {
    sim *S = (sim *)h;
    int saved = S->r.enable_collision;
    S->r.enable_collision = 0;
    int done = vxo_step(h, n);
    S->r.enable_collision = saved;
    return done;
}

void vxo_counts(void *h, int *nv, int *nl, int *ns) {
    sim *S = (sim *)h;
    *nv = S->nv; *nl = S->nl; *ns = S->ns;
}
double vxo_time(void *h) { return ((sim *)h)->t; }
float vxo_dt(void *h) { return ((sim *)h)->dt; }

void vxo_voxels(void *h, double *pos, double *orient, double *linmom, double *angmom, float *tempe, int *flags) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nv; i++) {
        voxel *v = &S->v[i];
        pos[3 * i] = v->pos.x; pos[3 * i + 1] = v->pos.y; pos[3 * i + 2] = v->pos.z;
        orient[4 * i] = v->orient.w; orient[4 * i + 1] = v->orient.x; orient[4 * i + 2] = v->orient.y; orient[4 * i + 3] = v->orient.z;
        linmom[3 * i] = v->linMom.x; linmom[3 * i + 1] = v->linMom.y; linmom[3 * i + 2] = v->linMom.z;
        angmom[3 * i] = v->angMom.x; angmom[3 * i + 1] = v->angMom.y; angmom[3 * i + 2] = v->angMom.z;
        tempe[i] = v->tempe;
        flags[i] = v->flags;
    }
}

void vxo_set_voxels(void *h, const double *pos, const double *orient, const double *linmom, const double *angmom) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nv; i++) {
        voxel *v = &S->v[i];
        v->pos = V(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        v->orient = Q(orient[4 * i], orient[4 * i + 1], orient[4 * i + 2], orient[4 * i + 3]);
        v->linMom = V(linmom[3 * i], linmom[3 * i + 1], linmom[3 * i + 2]);
        v->angMom = V(angmom[3 * i], angmom[3 * i + 1], angmom[3 * i + 2]);
    }
}

/* The rest of a run's state, to continue another implementation's run: time,
 * per voxel the temperature of the last step and the static-friction flag, per link
 * pos2/angle1v/angle2v, strain, maxStrain and flags (bit 0 smallAngle, bit 2
 * LOCAL_VELOCITY_VALID).  The time step stays the one recommended for the created
 * (unstrained) robot, as in a run from the start; voxels that stepped have it as
 * previousDt; rest lengths follow the temperatures. */
void vxo_set_run_state(void *h, double t, const float *tempe, const int *static_flag, const double *local9,
                       const float *strain, const float *maxstrain, const int *link_flags) {
    sim *S = (sim *)h;
    if (!S->optimal_dt) {
        /* as the first step takes it: after the temperatures of time 0 (do_step) */
        const vxo_robot *r = &S->r;
        if (r->vary_temp && r->temp_period > 0)
            for (int i = 0; i < S->nv; i++) {
                voxel *v = &S->v[i];
                const vmat *m = &S->vm[v->mat];
                if (v->removed || m->thermal_on_after > 0.0 || m->fixed) continue;
                double T = r->temp_amplitude * sin(2 * 3.1415926f * (0.0 / r->temp_period + v->phase));
                if (!r->enable_expansion && T > 0) T = 0;
                v->tempe = (float)T;
            }
        for (int i = 0; i < S->nl; i++) update_rest(S, &S->l[i]);
        S->optimal_dt = vxo_recommended_dt(S);
    }
    if (S->optimal_dt < 1e-10) S->optimal_dt = 1e-10;
    float dt = S->r.dt_frac * S->optimal_dt;
    S->dt = dt;
    S->t = t;
    for (int i = 0; i < S->nv; i++) {
        voxel *v = &S->v[i];
        v->tempe = tempe[i];
        v->flags = static_flag[i] ? (v->flags | F_STATIC) : (v->flags & ~F_STATIC);
        v->prevDt = S->vm[v->mat].fixed ? 0.0f : dt;
        v->contact = V(0, 0, 0);
    }
    for (int i = 0; i < S->nl; i++) {
        link *L = &S->l[i];
        const double *q = local9 + 9 * (size_t)i;
        L->pos2 = V(q[0], q[1], q[2]);
        L->a1v = V(q[3], q[4], q[5]);
        L->a2v = V(q[6], q[7], q[8]);
        L->strain = strain[i];
        L->maxStrain = maxstrain[i];
        L->small = link_flags[i] & 1;
        L->states = (link_flags[i] & 4) ? (L->states | L_LVV) : (L->states & ~L_LVV);
        update_rest(S, L);
    }
}

void vxo_topology(void *h, int *mat, int *ijk, int *slots) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nv; i++) {
        mat[i] = S->v[i].mat;
        ijk[3 * i] = S->v[i].ix; ijk[3 * i + 1] = S->v[i].iy; ijk[3 * i + 2] = S->v[i].iz;
        for (int d = 0; d < 6; d++) slots[6 * i + d] = S->v[i].links[d];
    }
}

void vxo_link_topology(void *h, int *negpos, int *axis, int *small, int *states) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nl; i++) {
        negpos[2 * i] = S->l[i].neg; negpos[2 * i + 1] = S->l[i].pos;
        axis[i] = S->l[i].axis; small[i] = S->l[i].small; states[i] = S->l[i].states;
    }
}

void vxo_links(void *h, float *strain, float *maxstrain, double *rest, double *local9, double *forces12) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nl; i++) {
        link *L = &S->l[i];
        strain[i] = L->strain; maxstrain[i] = L->maxStrain; rest[i] = L->rest;
        double *p = local9 + 9 * i;
        p[0] = L->pos2.x; p[1] = L->pos2.y; p[2] = L->pos2.z;
        p[3] = L->a1v.x; p[4] = L->a1v.y; p[5] = L->a1v.z;
        p[6] = L->a2v.x; p[7] = L->a2v.y; p[8] = L->a2v.z;
        double *f = forces12 + 12 * i;
        f[0] = L->fNeg.x; f[1] = L->fNeg.y; f[2] = L->fNeg.z;
        f[3] = L->fPos.x; f[4] = L->fPos.y; f[5] = L->fPos.z;
        f[6] = L->mNeg.x; f[7] = L->mNeg.y; f[8] = L->mNeg.z;
        f[9] = L->mPos.x; f[10] = L->mPos.y; f[11] = L->mPos.z;
    }
}

void vxo_voxel_mats(void *h, float *f16, double *nomsize, int *fm) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nvm; i++) {
        vmat *m = &S->vm[i];
        float *f = f16 + 16 * i;
        f[0] = m->mass; f[1] = m->mass_inv; f[2] = m->sqrt_mass; f[3] = m->mom_inertia; f[4] = m->mom_inertia_inv;
        f[5] = m->c2xSqMxExS; f[6] = m->c2xSqIxExSxSxS; f[7] = m->z_int; f[8] = m->z_glob; f[9] = m->z_col;
        f[10] = m->mu_s; f[11] = m->mu_k; f[12] = m->E; f[13] = m->nu; f[14] = m->cte; f[15] = m->grav_mult;
        nomsize[i] = m->nom_size;
        fm[2 * i] = m->fixed; fm[2 * i + 1] = m->is_measured;
    }
}

int vxo_num_link_mats(void *h) { return ((sim *)h)->nlm; }

void vxo_link_mats(void *h, float *f16, int *lmat_of_link) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nlm; i++) {
        lmat *m = &S->lm[i];
        float *f = f16 + 16 * i;
        f[0] = m->E; f[1] = m->nu; f[2] = m->eHat; f[3] = m->a1; f[4] = m->a2; f[5] = m->b1; f[6] = m->b2; f[7] = m->b3;
        f[8] = m->sqA1; f[9] = m->sqA2xIp; f[10] = m->sqB1; f[11] = m->sqB2xFMp; f[12] = m->sqB3xIp;
        f[13] = m->eps_fail; f[14] = m->cv.linear ? 1.0f : 0.0f; f[15] = m->cte;
    }
    for (int i = 0; i < S->nl; i++) lmat_of_link[i] = S->l[i].mat;
}

void vxo_link_offsets(void *h, float *off) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->nl; i++) off[i] = S->l[i].strainOffset;
}

int vxo_link_curve(void *h, int i, float *strain, float *stress, int cap) {
    const curve *c = &((sim *)h)->lm[i].cv;  /* as the device copy holds it: one more 0 in front */
    if (cap > 0) strain[0] = stress[0] = 0.0f;
    for (int j = 0; j < c->n && j + 1 < cap; j++) {
        strain[j + 1] = c->strain[j];
        stress[j + 1] = c->stress[j];
    }
    return c->n + 1;
}

void vxo_surface(void *h, int *idx) {
    sim *S = (sim *)h;
    for (int i = 0; i < S->ns; i++) idx[i] = S->surf[i];
}

void vxo_last_contact(void *h, double *c3) {
    sim *S = (sim *)h;
    memcpy(c3, S->last_contact, sizeof(double) * 3 * (size_t)S->nv);
}

/* updateCurrentCenterOfMass (VX3_VoxelyzeKernel.cu:477-493) */
void vxo_com(void *h, double *c3) {
    sim *S = (sim *)h;
    double total = 0;
    vec sum = V(0, 0, 0);
    for (int i = 0; i < S->nv; i++) {
        const vmat *m = &S->vm[S->v[i].mat];
        if (!m->is_measured) continue;
        double mass = m->mass;
        sum = vadd(sum, vscale(S->v[i].pos, mass));
        total += mass;
    }
    vec c = V(0, 0, 0);
    if (total != 0) c = vdiv(sum, total);
    c3[0] = c.x; c3[1] = c.y; c3[2] = c.z;
}
