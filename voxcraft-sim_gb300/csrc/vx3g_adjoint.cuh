// vx3g_adjoint.cuh -- hand-written reverse-mode adjoint of one FP64 step, per element.
//
// A step maps the state s_k (voxel pos/quat/linMom/angMom, link local state
// pos2/angle1v/angle2v) to s_{k+1} through the link pass (VX3_Link::orientLink,
// updateForces, src/VX3/VX3_Link.cu:90-218) and the voxel pass (VX3_Voxel::timeStep,
// src/VX3/VX3_Voxel.cu:162-277).  Given lambda = dL/ds_{k+1}, the functions below
// give dL/ds_k and add this step's share of dL/d(phase) and dL/d(log10 E) per voxel.
//
// The discrete branches (small-angle hysteresis, LOCAL_VELOCITY_VALID, floor
// contact, static/kinetic friction, temperature clamp, link failure) are taken as
// the forward pass took them, recomputed bit for bit from the stored state: the
// adjoint is that of the piecewise-smooth map the forward run followed.  Both
// orientLink branches (small angle, and large angle through FromAngleToPosX) are
// differentiated.
//
// Parameter paths.  A voxel's phase enters through its base size
// nomSize*(1 + T*cte), T = A*sin(2*3.1415926f*(t/P + phase)) (gpu_update_temperature,
// VX3_VoxelyzeKernel.cu:625-650), which sets the rest length of its links
// (VX3_Link.cu:80-83) and its floor penetration (VX3_Voxel.h:185-188).  Its Young's
// modulus E enters its links' combined modulus 2*E1*E2/(E1+E2)
// (src/old/VX_MaterialLink.cpp:82; every beam stiffness is proportional to the link
// modulus, every beam damping constant to its square root), its floor stiffness
// 2*E*L and its damping coefficients 2*sqrt(m*E*L)*zeta (proportional to sqrt(E)).
// The time step is held fixed.
#pragma once

#include "vx3g_adjoint.h"
#include "vx3g_step.cuh"

namespace vx3g {
namespace adj {

using V = V3<double>;
using Q = Q4<double>;

__device__ __forceinline__ V vload(const double *p) { return V{p[0], p[1], p[2]}; }
__device__ __forceinline__ double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ Q qload(double4 q) { return Q{q.x, q.y, q.z, q.w}; }  // stored {w,x,y,z}

// adjoint of y = qrot(q, f): adds dL/dq, dL/df for a given dL/dy
__device__ __forceinline__ void qrot_adj(Q q, V f, V ly, Q &lq, V &lf) {
    const double tw = f.x * q.x + f.y * q.y + f.z * q.z;
    const double tx = f.x * q.w - f.y * q.z + f.z * q.y;
    const double ty = f.x * q.z + f.y * q.w - f.z * q.x;
    const double tz = -f.x * q.y + f.y * q.x + f.z * q.w;
    // y.x = q.w*tx + q.x*tw + q.y*tz - q.z*ty, y.y = q.w*ty - q.x*tz + q.y*tw + q.z*tx,
    // y.z = q.w*tz + q.x*ty - q.y*tx + q.z*tw
    const double ltw = q.x * ly.x + q.y * ly.y + q.z * ly.z;
    const double ltx = q.w * ly.x + q.z * ly.y - q.y * ly.z;
    const double lty = -q.z * ly.x + q.w * ly.y + q.x * ly.z;
    const double ltz = q.y * ly.x - q.x * ly.y + q.w * ly.z;
    lq.w += tx * ly.x + ty * ly.y + tz * ly.z + f.x * ltx + f.y * lty + f.z * ltz;
    lq.x += tw * ly.x - tz * ly.y + ty * ly.z + f.x * ltw - f.z * lty + f.y * ltz;
    lq.y += tz * ly.x + tw * ly.y - tx * ly.z + f.y * ltw + f.z * ltx - f.x * ltz;
    lq.z += -ty * ly.x + tx * ly.y + tw * ly.z + f.z * ltw - f.y * ltx + f.x * lty;
    lf.x += q.x * ltw + q.w * ltx + q.z * lty - q.y * ltz;
    lf.y += q.y * ltw - q.z * ltx + q.w * lty + q.x * ltz;
    lf.z += q.z * ltw + q.y * ltx - q.x * lty + q.w * ltz;
}

// adjoint of y = qrotinv(q, f)
__device__ __forceinline__ void qrotinv_adj(Q q, V f, V ly, Q &lq, V &lf) {
    const double tw = q.x * f.x + q.y * f.y + q.z * f.z;
    const double tx = q.w * f.x - q.y * f.z + q.z * f.y;
    const double ty = q.w * f.y + q.x * f.z - q.z * f.x;
    const double tz = q.w * f.z - q.x * f.y + q.y * f.x;
    // y.x = tw*q.x + tx*q.w + ty*q.z - tz*q.y, y.y = tw*q.y - tx*q.z + ty*q.w + tz*q.x,
    // y.z = tw*q.z + tx*q.y - ty*q.x + tz*q.w
    const double ltw = q.x * ly.x + q.y * ly.y + q.z * ly.z;
    const double ltx = q.w * ly.x - q.z * ly.y + q.y * ly.z;
    const double lty = q.z * ly.x + q.w * ly.y - q.x * ly.z;
    const double ltz = -q.y * ly.x + q.x * ly.y + q.w * ly.z;
    lq.w += tx * ly.x + ty * ly.y + tz * ly.z + f.x * ltx + f.y * lty + f.z * ltz;
    lq.x += tw * ly.x + tz * ly.y - ty * ly.z + f.x * ltw + f.z * lty - f.y * ltz;
    lq.y += -tz * ly.x + tw * ly.y + tx * ly.z + f.y * ltw - f.z * ltx + f.x * ltz;
    lq.z += ty * ly.x - tx * ly.y + tw * ly.z + f.z * ltw + f.y * ltx - f.x * lty;
    lf.x += q.x * ltw + q.w * ltx - q.z * lty + q.y * ltz;
    lf.y += q.y * ltw + q.z * ltx + q.w * lty - q.x * ltz;
    lf.z += q.z * ltw - q.y * ltx + q.x * lty + q.w * ltz;
}

// adjoint of y = qmul(a, b)
__device__ __forceinline__ void qmul_adj(Q a, Q b, Q l, Q &la, Q &lb) {
    la.w += b.w * l.w + b.x * l.x + b.y * l.y + b.z * l.z;
    la.x += -b.x * l.w + b.w * l.x - b.z * l.y + b.y * l.z;
    la.y += -b.y * l.w + b.z * l.x + b.w * l.y - b.x * l.z;
    la.z += -b.z * l.w - b.y * l.x + b.x * l.y + b.w * l.z;
    lb.w += a.w * l.w + a.x * l.x + a.y * l.y + a.z * l.z;
    lb.x += -a.x * l.w + a.w * l.x + a.z * l.y - a.y * l.z;
    lb.y += -a.y * l.w - a.z * l.x + a.w * l.y + a.x * l.z;
    lb.z += -a.z * l.w + a.y * l.x - a.x * l.y + a.w * l.z;
}

// adjoint of v = ToRotationVector(q) (VX3_Quat3D.h:347-359): v = (x,y,z)*g(w)
// At w >= 1 (no rotation, or one too small to move w off 1 in FP64) the forward
// returns 0; the adjoint uses the limit g = 2 of the smooth function there, which
// is what any perturbation that registers a rotation sees.
__device__ __forceinline__ void rotvec_adj(Q q, V lv, Q &lq) {
    if (q.w <= -1.0) return;
    if (q.w >= 1.0) {
        lq.x += 2.0 * lv.x;
        lq.y += 2.0 * lv.y;
        lq.z += 2.0 * lv.z;
        lq.w += -0.5 * (q.x * lv.x + q.y * lv.y + q.z * lv.z);
        return;
    }
    const double sq = 1.0 - q.w * q.w;
    double g, dg;
    if (sq < 2.4e-3) {  // g = 2*sqrt((2-2w)/(1-w^2)) = 2*sqrt(2/(1+w))
        g = 2.0 * sqrt((2 - 2 * q.w) / sq);
        dg = -g / (2.0 * (1.0 + q.w));
    } else {            // g = 2*acos(w)/sqrt(1-w^2)
        const double s = sqrt(sq), ac = acos(q.w);
        g = 2.0 * ac / s;
        dg = 2.0 * (-1.0 / sq + q.w * ac / (sq * s));
    }
    lq.x += g * lv.x;
    lq.y += g * lv.y;
    lq.z += g * lv.z;
    lq.w += dg * (q.x * lv.x + q.y * lv.y + q.z * lv.z);
}

// adjoint of q = FromRotationVector(in) (VX3_Quat3D.h:363-377): returns dL/d(in)
__device__ __forceinline__ V from_rotvec_adj(V in, Q lq) {
    const V th{0.5 * in.x, 0.5 * in.y, 0.5 * in.z};
    const double m2 = dot(th, th);
    const V lxyz{lq.x, lq.y, lq.z};
    V lth;
    if (m2 * m2 < 5.328e-15) {  // w = 1 - m2/2, xyz = th*(1 - m2/6)
        const double s = 1.0 - m2 / 6.0;
        const double lm2 = -0.5 * lq.w - dot(th, lxyz) / 6.0;
        lth = V{s * lxyz.x + 2 * th.x * lm2, s * lxyz.y + 2 * th.y * lm2, s * lxyz.z + 2 * th.z * lm2};
    } else {                    // w = cos(m), xyz = th*sin(m)/m
        const double m = sqrt(m2), sn = sin(m), cs = cos(m);
        const double s = sn / m, ds = (m * cs - sn) / m2;
        const double lm = -sn * lq.w + dot(th, lxyz) * ds;
        lth = V{s * lxyz.x + lm * th.x / m, s * lxyz.y + lm * th.y / m, s * lxyz.z + lm * th.z / m};
    }
    return V{0.5 * lth.x, 0.5 * lth.y, 0.5 * lth.z};
}

// toAxisX / toAxisOriginal are signed permutations; each is the other's transpose
__device__ __forceinline__ Q axis_q_T(int axis, Q l) {
    const V v = to_axis_original(axis, V{l.x, l.y, l.z});
    return Q{l.w, v.x, v.y, v.z};
}

// adjoint of q = FromAngleToPosX(identity, r) (VX3_Quat3D.h:384-432): adds dL/dr
__device__ __forceinline__ void from_angle_to_posx_adj(V r, Q lq, V &lr) {
    if (r.x == 0 && r.y == 0 && r.z == 0) return;
    const double yx = r.y / r.x, zx = r.z / r.x;
    const double SA = 1.732e-2;
    if (yx < SA && yx > -SA && zx < SA && zx > -SA) {
        // q = (1 + (-qy^2 - qz^2)/2, 0, zx/2, -yx/2)
        const double qy = 0.5 * zx, qz = -0.5 * yx;
        const double lqy = lq.y - qy * lq.w, lqz = lq.z - qz * lq.w;
        const double lzx = 0.5 * lqy, lyx = -0.5 * lqz;
        lr.x += -(yx * lyx + zx * lzx) / r.x;
        lr.y += lyx / r.x;
        lr.z += lzx / r.x;
        return;
    }
    const double l = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    const V n{r.x / l, r.y / l, r.z / l};
    const double theta = acos(n.x);
    if (theta > 3.14159265358979 - 1e-7) return;  // constant (0, 0, 1, 0)
    // q = (cos(a), 0, n.z*ai*sin(a), -n.y*ai*sin(a)), a = theta/2, ai = 1/sqrt(n.y^2 + n.z^2)
    const double ai = 1.0 / sqrt(n.z * n.z + n.y * n.y), a = 0.5 * theta, sa = sin(a), ca = cos(a);
    double la = -sa * lq.w, lsa = n.z * ai * lq.y - n.y * ai * lq.z, lai = n.z * sa * lq.y - n.y * sa * lq.z;
    V ln{0, ai * -sa * lq.z, ai * sa * lq.y};
    la += ca * lsa;
    const double ltheta = 0.5 * la;
    ln.x += -ltheta / sqrt(1.0 - n.x * n.x);
    const double ai3 = ai * ai * ai;
    ln.y += -ai3 * n.y * lai;
    ln.z += -ai3 * n.z * lai;
    const double nl = dot(n, ln);  // n = r/|r|
    lr.x += (ln.x - n.x * nl) / l;
    lr.y += (ln.y - n.y * nl) / l;
    lr.z += (ln.z - n.z * nl) / l;
}

// ------------------------------------------------------------ link forward recompute
// link_update<double> on a stored state, without writing the state: the values the
// adjoint needs.  Same operations in the same order as the forward pass, so every
// branch decision is the forward run's.
struct LinkFwd {
    int state;        // 0: not updated, 1: updated
    bool small, lvv, failed;
    double L, sc, dmN, dmP;
    V p0, P, pos2, a1v, a2v, dP, dA1, dA2;
    Q a1, a2, c, A2, B1, B2;  // B1/B2: the frames of the two ends after orientLink
    V fN0, mN0, mP0;  // elastic parts in the link frame
    V pc, uN, uP;     // damping parts (with lvv)
    V fN, mN, fP, mP; // end forces/moments before the rotations by B1 (large angle) and B2
    V sN_f, sN_m, sP_f, sP_m;  // slot values (original frame)
};

__device__ __forceinline__ void link_forward(const Dev &d, const Snap &s, int l, LinkFwd &o) {
    const uint2 li = s.linfo[l];
    const int r = (int)li.x;
    const uint32_t fl = li.y;
    o.state = 0;
    if (s.status[r] != 0 || (fl & LF_BOTH_FIXED)) return;
    o.state = 1;
    const int axis = fl & LF_AXIS;
    const int2 e = d.ends[l];
    const double4 pn = s.pos[e.x], pp = s.pos[e.y];
    const double rest = 0.5 * (pn.w + pp.w);
    const LMat &m = d.lmat[fl >> 8];
    const double *ls = s.lstate;
    const size_t NL = (size_t)d.nl;
    const V oldPos2{ls[l], ls[NL + l], ls[2 * NL + l]};
    const V oldA1{ls[3 * NL + l], ls[4 * NL + l], ls[5 * NL + l]};
    const V oldA2{ls[6 * NL + l], ls[7 * NL + l], ls[8 * NL + l]};
    o.p0 = to_axis_x(axis, V{pp.x - pn.x, pp.y - pn.y, pp.z - pn.z});
    o.a1 = to_axis_xq(axis, qload(s.quat[e.x]));
    o.a2 = to_axis_xq(axis, qload(s.quat[e.y]));
    o.c = qconj(o.a1);
    V pos2 = qrot(o.c, o.p0);
    o.P = pos2;
    o.A2 = qmul(o.c, o.a2);
    Q angle1{1, 0, 0, 0}, angle2 = o.A2;
    const double restR = rest;
    o.L = restR;
    const float SmallTurn = (float)((fabs(pos2.z) + fabs(pos2.y)) / pos2.x);
    const float ExtendPerc = (float)(fabs(1 - pos2.x / restR));
    const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;
    bool small = (fl & LF_SMALL) != 0, lvv = (fl & LF_LVV) != 0;
    if (!small && SmallTurn < BEND && ExtendPerc < EXT) {
        small = true;
        lvv = false;
    } else if (small && (SmallTurn > HF * BEND || ExtendPerc > HF * EXT)) {
        small = false;
        lvv = false;
    }
    o.small = small;
    if (small) {
        pos2.x -= restR;
    } else {
        angle1 = from_angle_to_posx(angle1, pos2);
        angle2 = qmul(angle1, angle2);
        pos2 = V{len(pos2) - restR, 0, 0};
    }
    o.B1 = angle1;
    o.B2 = angle2;
    o.pos2 = pos2;
    const V a1v = to_rotvec(angle1), a2v = to_rotvec(angle2);
    o.a1v = a1v;
    o.a2v = a2v;
    const double half = 0.5;
    o.dP = scl(sub(pos2, oldPos2), half);
    o.dA1 = scl(sub(a1v, oldA1), half);
    o.dA2 = scl(sub(a2v, oldA2), half);
    const float axialStrain = (float)(pos2.x / restR);
    const float maxs = axialStrain > s.strain[l].y ? axialStrain : s.strain[l].y;
    float stress;
    if (m.eps_fail != -1.0f && axialStrain > m.eps_fail) {
        stress = 0.0f;
        o.sc = 0.0;
    } else if (m.nu == 0.0f) {
        stress = m.E * axialStrain;
        o.sc = m.E;
    } else {
        stress = m.eHat * ((1 - m.nu) * axialStrain + m.nu * m.tss);
        o.sc = (double)m.eHat * (double)(1 - m.nu);
    }
    o.failed = m.eps_fail != -1.0f && maxs > m.eps_fail;
    o.lvv = lvv;
    const V z{0, 0, 0};
    o.sN_f = o.sN_m = o.sP_f = o.sP_m = z;
    o.pc = o.uN = o.uP = z;
    o.dmN = o.dmP = 0;
    if (o.failed) return;
    const float b1 = m.b1, b2 = m.b2, b3 = m.b3, a2 = m.a2;
    V fNeg{(double)(stress * m.area), b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y)};
    V fPos = neg(fNeg);
    V mNeg{a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z)};
    V mPos{a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z)};
    o.fN0 = fNeg;
    o.mN0 = mNeg;
    o.mP0 = mPos;
    if (lvv) {
        const float sqA1 = m.sqA1, sqA2xIp = m.sqA2xIp, sqB1 = m.sqB1, sqB2xFMp = m.sqB2xFMp, sqB3xIp = m.sqB3xIp;
        const V dPos2 = o.dP, dA1 = o.dA1, dA2 = o.dA2;
        const V posCalc{sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z),
                        sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y)};
        const float dtf = d.dt[li.x];
        const uint32_t fnv = s.vinfo[e.x].y, fpv = s.vinfo[e.y].y;
        const float dmN = d.vmat[fnv >> 8].dmc / ((fnv & VF_FIXED) ? 0.0f : dtf);
        const float dmP = d.vmat[fpv >> 8].dmc / ((fpv & VF_FIXED) ? 0.0f : dtf);
        fNeg = add(fNeg, scl(posCalc, dmN));
        fPos = sub(fPos, scl(posCalc, dmP));
        const V uN{-sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (2 * dA1.y + dA2.y),
                   -sqB2xFMp * dPos2.y + sqB3xIp * (2 * dA1.z + dA2.z)};
        const V uP{sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (dA1.y + 2 * dA2.y),
                   -sqB2xFMp * dPos2.y + sqB3xIp * (dA1.z + 2 * dA2.z)};
        mNeg = sub(mNeg, scl(uN, (double)(half * dmN)));
        mPos = sub(mPos, scl(uP, (double)(half * dmP)));
        o.pc = posCalc;
        o.uN = uN;
        o.uP = uP;
        // a fixed end's force is never used; its (infinite) multiplier is left out of the adjoint
        o.dmN = (fnv & VF_FIXED) ? 0.0 : (double)dmN;
        o.dmP = (fpv & VF_FIXED) ? 0.0 : (double)dmP;
    }
    o.fN = fNeg;
    o.mN = mNeg;
    o.fP = fPos;
    o.mP = mPos;
    if (!small) {
        fNeg = qrotinv(angle1, fNeg);
        mNeg = qrotinv(angle1, mNeg);
    }
    fPos = qrotinv(angle2, fPos);
    mPos = qrotinv(angle2, mPos);
    o.sN_f = to_axis_original(axis, fNeg);
    o.sN_m = to_axis_original(axis, mNeg);
    o.sP_f = to_axis_original(axis, fPos);
    o.sP_m = to_axis_original(axis, mPos);
}

// The step's link forces into d.slots (what the forward link pass wrote).
__device__ __forceinline__ void adj_link_slots(const Dev &d, const Snap &s, const AdjBufs &a, int l) {
    LinkFwd o;
    link_forward(d, s, l, o);
    if (o.state == 0) return;  // the forward pass wrote nothing (both ends then stay still)
    const int axis = s.linfo[l].y & LF_AXIS;
    const int2 e = d.ends[l];
    Slot<double> *S = (Slot<double> *)d.slots;
    store_slot(&S[(size_t)(2 * axis) * d.nv + e.x], o.sN_f, o.sN_m);
    store_slot(&S[(size_t)(2 * axis + 1) * d.nv + e.y], o.sP_f, o.sP_m);
}

// ------------------------------------------------------------ voxel pass adjoint
__device__ __forceinline__ void adj_voxel(const Dev &d, const Snap &s, const AdjBufs &a, int v) {
    const double *lv = a.lv + 13 * (size_t)v;
    double *lo = a.lown + 13 * (size_t)v, *lF = a.lF + 6 * (size_t)v;
    for (int i = 0; i < 6; i++) lF[i] = 0.0;
    a.lbs[v] = 0.0;
    a.lE[v] = 0.0;
    a.lcon[3 * (size_t)v] = a.lcon[3 * (size_t)v + 1] = a.lcon[3 * (size_t)v + 2] = 0.0;
    const uint2 vi = s.vinfo[v];
    const int r = (int)vi.x;
    const uint32_t fl = vi.y;
    const float dtf = d.dt[r];
    if (s.status[r] != 0 || (fl & VF_FIXED) || dtf == 0.0f) {  // the state passes through unchanged
        for (int i = 0; i < 13; i++) lo[i] = lv[i];
        return;
    }
    const RobotP &rp = d.rp[r];
    const VMat m = d.vmat[fl >> 8];
    const double dt = dtf;
    const double4 p4 = s.pos[v], l4 = s.linmom[v], a4 = s.angmom[v];
    const Q o = qload(s.quat[v]);
    const V lm{l4.x, l4.y, l4.z}, am{a4.x, a4.y, a4.z};
    // ---- forward recompute (voxel_update<double>, same operation order)
    V F0{0, 0, 0}, M0{0, 0, 0};
    const Slot<double> *S = (const Slot<double> *)d.slots;
    for (int dir = 0; dir < 6; dir++)
        if (fl & (1u << dir)) {
            const Slot<double> sl = S[(size_t)dir * d.nv + v];
            F0 = add(F0, V{sl.f[0], sl.f[1], sl.f[2]});
            M0 = add(M0, V{sl.m[0], sl.m[1], sl.m[2]});
        }
    bool stat = (fl & VF_STATIC) != 0;
    const bool floorOn = rp.floor != 0;
    const double bs = p4.w;
    const double bsa = (bs + bs + bs) / 3.0f;
    const float pen = (float)(bsa / 2 - m.nom_size / 2 - p4.z);
    V F = qrot(o, F0);
    const V vel = scl(lm, m.mass_inv);
    F = sub(F, scl(vel, m.c_glob));
    F.z += m.grav_force;
    if (rp.collision) {  // this step's contact force (recomputed into d.contact for this state)
        const double4 c = d.contact[v];
        F = sub(F, V{c.x, c.y, c.z});
    }
    F = add(F, V{0.0, 0.0, 0.0});
    if (rp.ff[0] >= 0 || rp.ff[1] >= 0 || rp.ff[2] >= 0) {  // force field: depends on time only (record checks)
        const V ff = force_field(d, rp, p4.x, p4.y, p4.z, s.T[(size_t)a.parity * d.nr + r]);
        F.x += ff.x;
        F.y += ff.y;
        F.z += ff.z;
    }
    V fric = F;
    bool contact = false, kinetic = false;
    V u{0, 0, 0};
    double vxy = 0;
    float normal = 0;
    if (floorOn) {
        if (pen >= 0) {
            contact = true;
            normal = m.pstiff * pen;
            F.z += normal - m.c_col * vel.z;
            if (stat) {
                const float surf = (float)(F.x * F.x + F.y * F.y);
                const float fr = (m.mu_s * normal) * (m.mu_s * normal);
                if (surf > fr) stat = false;
            } else {
                kinetic = true;
                const V vxy3{vel.x, vel.y, 0};
                vxy = sqrt(vxy3.x * vxy3.x + vxy3.y * vxy3.y);
                u = normalized(vxy3);
                F = sub(F, scl(u, m.mu_k * normal));
            }
        } else {
            stat = false;
        }
    }
    fric = sub(F, fric);
    const V lm1 = add(lm, scl(F, dt));
    V tr = scl(lm1, dt * m.mass_inv);
    bool zero_xy = false;
    if (floorOn && pen >= 0) {
        const double work = fric.x * tr.x + fric.y * tr.y;
        const double hKe = 0.5 * m.mass_inv * (lm1.x * lm1.x + lm1.y * lm1.y);
        if (hKe + work <= 0) stat = true;
        if (stat) tr.x = tr.y = 0;
        // Held with no normal force and no tangential momentum, a voxel sits on the
        // edge of the static-friction region: any tangential perturbation frees it.
        // The adjoint takes the free side there (the initial resting state has this).
        if (stat && normal == 0.0f && lm1.x == 0 && lm1.y == 0) stat = false;
        zero_xy = stat;
    } else {
        stat = false;
    }
    const double pz1 = p4.z + tr.z;
    V M = qrot(o, M0);
    M = sub(M, scl(scl(am, m.mom_inv), m.c_glob_rot));
    const V am1 = add(am, scl(M, dt));
    const double ki = dt * m.mom_inv;
    const V theta = scl(am1, ki);
    const Q dq = from_rotvec(theta);
    const bool zero_am = floorOn && (float)(bsa / 2 - m.nom_size / 2 - pz1) >= 0 && stat;
    // ---- reverse
    const V lpos1 = vload(lv), llm_out = vload(lv + 7), lam_out = vload(lv + 10);
    const Q lo1{lv[3], lv[4], lv[5], lv[6]};
    V lpos = lpos1, llm{0, 0, 0}, lam{0, 0, 0};
    Q lq{0, 0, 0, 0}, ldq{0, 0, 0, 0};
    qmul_adj(dq, o, lo1, ldq, lq);  // q1 = dq*q
    V lam1 = zero_am ? V{0, 0, 0} : lam_out;
    lam1 = add(lam1, scl(from_rotvec_adj(theta, ldq), ki));
    lam = add(lam, lam1);
    const V lM = scl(lam1, dt);
    lam = sub(lam, scl(lM, (double)m.mom_inv * (double)m.c_glob_rot));
    double lE = -dot(scl(am, m.mom_inv), lM) * (double)m.c_glob_rot / (2.0 * (double)m.E);
    V lM0{0, 0, 0};
    qrot_adj(o, M0, lM, lq, lM0);
    V ltr = lpos1;
    if (zero_xy) ltr.x = ltr.y = 0;
    V llm1 = add(llm_out, scl(ltr, dt * (double)m.mass_inv));
    if (zero_xy) llm1.x = llm1.y = 0;
    llm = add(llm, llm1);
    const V lFt = scl(llm1, dt);  // dL/dF (total force)
    if (rp.collision) {  // F = ... - contact
        a.lcon[3 * (size_t)v] = -lFt.x;
        a.lcon[3 * (size_t)v + 1] = -lFt.y;
        a.lcon[3 * (size_t)v + 2] = -lFt.z;
    }
    V lvel{0, 0, 0};
    double lbs = 0;
    if (contact) {
        double lnormal = lFt.z;
        lvel.z += -(double)m.c_col * lFt.z;
        lE += -vel.z * lFt.z * (double)m.c_col / (2.0 * (double)m.E);
        if (kinetic) {
            lnormal += -(double)m.mu_k * (u.x * lFt.x + u.y * lFt.y);
            if (vxy > 0) {
                const V lu{-(double)m.mu_k * normal * lFt.x, -(double)m.mu_k * normal * lFt.y, 0};
                const double ul = u.x * lu.x + u.y * lu.y;
                lvel.x += (lu.x - u.x * ul) / vxy;
                lvel.y += (lu.y - u.y * ul) / vxy;
            }
        }
        const double lpen = (double)m.pstiff * lnormal;
        lE += (double)pen * lnormal * 2.0 * m.nom_size;  // d(2*E*L)/dE
        lpos.z += -lpen;
        lbs += 0.5 * lpen;  // pen = bs/2 - nomSize/2 - z
    }
    lvel = sub(lvel, scl(lFt, m.c_glob));
    lE += -dot(vel, lFt) * (double)m.c_glob / (2.0 * (double)m.E);
    llm = add(llm, scl(lvel, m.mass_inv));
    V lF0{0, 0, 0};
    qrot_adj(o, F0, lFt, lq, lF0);
    lo[0] = lpos.x; lo[1] = lpos.y; lo[2] = lpos.z;
    lo[3] = lq.w; lo[4] = lq.x; lo[5] = lq.y; lo[6] = lq.z;
    lo[7] = llm.x; lo[8] = llm.y; lo[9] = llm.z;
    lo[10] = lam.x; lo[11] = lam.y; lo[12] = lam.z;
    lF[0] = lF0.x; lF[1] = lF0.y; lF[2] = lF0.z;
    lF[3] = lM0.x; lF[4] = lM0.y; lF[5] = lM0.z;
    a.lbs[v] = lbs;
    a.lE[v] = lE;
}

// ------------------------------------------------------------ link pass adjoint
__device__ __forceinline__ void put_aslot(const AdjBufs &a, const Dev &d, int dir, int v, V lp, Q lq, double lbs,
                                          double lE) {
    double *o = a.aslot + 9 * ((size_t)dir * d.nv + v);
    o[0] = lp.x; o[1] = lp.y; o[2] = lp.z;
    o[3] = lq.w; o[4] = lq.x; o[5] = lq.y; o[6] = lq.z;
    o[7] = lbs; o[8] = lE;
}

__device__ __forceinline__ void adj_link(const Dev &d, const Snap &s, const AdjBufs &a, int l) {
    const uint32_t fl = s.linfo[l].y;
    const int axis = fl & LF_AXIS;
    const int2 e = d.ends[l];
    double *lloc = a.lloc + 9 * (size_t)l;
    LinkFwd o;
    link_forward(d, s, l, o);
    if (o.state == 0) {  // not updated: the local state passes through, no force
        const V zero{0, 0, 0};
        const Q zq{0, 0, 0, 0};
        put_aslot(a, d, 2 * axis, e.x, zero, zq, 0, 0);
        put_aslot(a, d, 2 * axis + 1, e.y, zero, zq, 0, 0);
        return;
    }
    const LMat &m = d.lmat[fl >> 8];
    const double b1 = m.b1, b2 = m.b2, b3 = m.b3, ka2 = m.a2;
    const double sqA1 = m.sqA1, sqA2 = m.sqA2xIp, sqB1 = m.sqB1, sqB2 = m.sqB2xFMp, sqB3 = m.sqB3xIp;
    const double L = o.L;
    // lambda of the new local state (pos2, angle1v, angle2v) from the next step
    V lpos2 = vload(lloc), la1v = vload(lloc + 3), la2v = vload(lloc + 6);
    V loP{0, 0, 0}, loA1{0, 0, 0}, loA2{0, 0, 0};
    Q lB1{0, 0, 0, 0}, lB2{0, 0, 0, 0};
    double lL = 0, lEl = 0;
    if (!o.failed) {
        const double *lFn = a.lF + 6 * (size_t)e.x, *lFp = a.lF + 6 * (size_t)e.y;
        const V lfNr = to_axis_x(axis, vload(lFn)), lmNr = to_axis_x(axis, vload(lFn + 3));
        const V lfPr = to_axis_x(axis, vload(lFp)), lmPr = to_axis_x(axis, vload(lFp + 3));
        V lfN{0, 0, 0}, lmN{0, 0, 0}, lfP{0, 0, 0}, lmP{0, 0, 0};
        if (o.small) {
            lfN = lfNr;
            lmN = lmNr;
        } else {
            qrotinv_adj(o.B1, o.fN, lfNr, lB1, lfN);
            qrotinv_adj(o.B1, o.mN, lmNr, lB1, lmN);
        }
        qrotinv_adj(o.B2, o.fP, lfPr, lB2, lfP);
        qrotinv_adj(o.B2, o.mP, lmPr, lB2, lmP);
        // fN = fN0 + dmN*pc, fP = -fN0 - dmP*pc, mN = mN0 - dmN/2*uN, mP = mP0 - dmP/2*uP
        const V lfN0 = sub(lfN, lfP);
        const V lmN0 = lmN, lmP0 = lmP;
        V ldP{0, 0, 0}, ldA1{0, 0, 0}, ldA2{0, 0, 0};
        if (o.lvv) {
            const V lpc = sub(scl(lfN, o.dmN), scl(lfP, o.dmP));
            const V luN = scl(lmN, -0.5 * o.dmN), luP = scl(lmP, -0.5 * o.dmP);
            // pc = {sqA1*dP.x, sqB1*dP.y - sqB2*(dA1.z+dA2.z), sqB1*dP.z + sqB2*(dA1.y+dA2.y)}
            ldP.x += sqA1 * lpc.x;
            ldP.y += sqB1 * lpc.y;
            ldA1.z += -sqB2 * lpc.y;
            ldA2.z += -sqB2 * lpc.y;
            ldP.z += sqB1 * lpc.z;
            ldA1.y += sqB2 * lpc.z;
            ldA2.y += sqB2 * lpc.z;
            // uN = {-sqA2*(dA2.x-dA1.x), sqB2*dP.z + sqB3*(2dA1.y+dA2.y), -sqB2*dP.y + sqB3*(2dA1.z+dA2.z)}
            // uP = { sqA2*(dA2.x-dA1.x), sqB2*dP.z + sqB3*(dA1.y+2dA2.y), -sqB2*dP.y + sqB3*(dA1.z+2dA2.z)}
            ldA2.x += -sqA2 * luN.x + sqA2 * luP.x;
            ldA1.x += sqA2 * luN.x - sqA2 * luP.x;
            ldP.z += sqB2 * luN.y + sqB2 * luP.y;
            ldA1.y += 2 * sqB3 * luN.y + sqB3 * luP.y;
            ldA2.y += sqB3 * luN.y + 2 * sqB3 * luP.y;
            ldP.y += -sqB2 * luN.z - sqB2 * luP.z;
            ldA1.z += 2 * sqB3 * luN.z + sqB3 * luP.z;
            ldA2.z += sqB3 * luN.z + 2 * sqB3 * luP.z;
            lEl += 0.5 * (dot(lpc, o.pc) + dot(luN, o.uN) + dot(luP, o.uP)) / m.E;
        }
        lEl += (dot(lfN0, o.fN0) + dot(lmN0, o.mN0) + dot(lmP0, o.mP0)) / m.E;
        // dP = (pos2 - oldPos2)/2, dA1 = (a1v - oldA1)/2, dA2 = (a2v - oldA2)/2
        lpos2 = add(lpos2, scl(ldP, 0.5));
        la1v = add(la1v, scl(ldA1, 0.5));
        la2v = add(la2v, scl(ldA2, 0.5));
        loP = scl(ldP, -0.5);
        loA1 = scl(ldA1, -0.5);
        loA2 = scl(ldA2, -0.5);
        // fN0 = {sc*(pos2.x/L)*area, b1*p.y - b2*(a1.z+a2.z), b1*p.z + b2*(a1.y+a2.y)}
        // mN0 = {a2*(a2.x-a1.x), -b2*p.z - b3*(2a1.y+a2.y), b2*p.y - b3*(2a1.z+a2.z)}
        // mP0 = {a2*(a1.x-a2.x), -b2*p.z - b3*(a1.y+2a2.y), b2*p.y - b3*(a1.z+2a2.z)}
        const double lstress = (double)m.area * lfN0.x;
        lpos2.x += o.sc * lstress / L;
        lL += -o.sc * lstress * o.pos2.x / (L * L);
        lpos2.y += b1 * lfN0.y + b2 * lmN0.z + b2 * lmP0.z;
        lpos2.z += b1 * lfN0.z - b2 * lmN0.y - b2 * lmP0.y;
        la1v.x += -ka2 * lmN0.x + ka2 * lmP0.x;
        la2v.x += ka2 * lmN0.x - ka2 * lmP0.x;
        la1v.y += b2 * lfN0.z - 2 * b3 * lmN0.y - b3 * lmP0.y;
        la2v.y += b2 * lfN0.z - b3 * lmN0.y - 2 * b3 * lmP0.y;
        la1v.z += -b2 * lfN0.y - 2 * b3 * lmN0.z - b3 * lmP0.z;
        la2v.z += -b2 * lfN0.y - b3 * lmN0.z - 2 * b3 * lmP0.z;
    }
    rotvec_adj(o.B2, la2v, lB2);
    V lP{0, 0, 0};
    Q lA2{0, 0, 0, 0};
    lL += -lpos2.x;
    if (o.small) {  // B1 = identity, B2 = A2, pos2 = P - (L, 0, 0)
        lA2 = lB2;
        lP = lpos2;
    } else {        // B1 = FromAngleToPosX(P), B2 = B1*A2, pos2 = (|P| - L, 0, 0)
        rotvec_adj(o.B1, la1v, lB1);
        qmul_adj(o.B1, o.A2, lB2, lB1, lA2);
        const double lp = len(o.P);
        lP = scl(o.P, lpos2.x / lp);
        from_angle_to_posx_adj(o.P, lB1, lP);
    }
    // P = qrot(c, p0), A2 = c*a2, c = conj(a1)
    Q lc{0, 0, 0, 0}, la2{0, 0, 0, 0};
    qmul_adj(o.c, o.a2, lA2, lc, la2);
    V lp0{0, 0, 0};
    qrot_adj(o.c, o.p0, lP, lc, lp0);
    const Q la1{lc.w, -lc.x, -lc.y, -lc.z};
    const Q lqn = axis_q_T(axis, la1), lqp = axis_q_T(axis, la2);
    const V lD = to_axis_original(axis, lp0);  // p0 = toAxisX(pos_pos - pos_neg)
    // the local state this step's damping terms consumed
    lloc[0] = loP.x; lloc[1] = loP.y; lloc[2] = loP.z;
    lloc[3] = loA1.x; lloc[4] = loA1.y; lloc[5] = loA1.z;
    lloc[6] = loA2.x; lloc[7] = loA2.y; lloc[8] = loA2.z;
    // L = (bs_neg + bs_pos)/2; link modulus 2*E1*E2/(E1+E2)
    const VMat &mn = d.vmat[s.vinfo[e.x].y >> 8], &mp = d.vmat[s.vinfo[e.y].y >> 8];
    const double En = mn.E, Ep = mp.E, den = (En + Ep) * (En + Ep);
    put_aslot(a, d, 2 * axis, e.x, neg(lD), lqn, 0.5 * lL, lEl * 2 * Ep * Ep / den);
    put_aslot(a, d, 2 * axis + 1, e.y, lD, lqp, 0.5 * lL, lEl * 2 * En * En / den);
}

// ------------------------------------------------------------ gather + parameter gradients
__device__ __forceinline__ void adj_gather(const Dev &d, const Snap &s, const AdjBufs &a, int v) {
    const uint2 vi = s.vinfo[v];
    const uint32_t fl = vi.y;
    const int r = (int)vi.x;
    double acc[13];
    const double *lo = a.lown + 13 * (size_t)v;
    for (int i = 0; i < 13; i++) acc[i] = lo[i];
    double lbs = a.lbs[v], lE = a.lE[v];
    for (int dir = 0; dir < 6; dir++)
        if (fl & (1u << dir)) {
            const double *o = a.aslot + 9 * ((size_t)dir * d.nv + v);
            for (int i = 0; i < 7; i++) acc[i] += o[i];
            lbs += o[7];
            lE += o[8];
        }
    if (d.rp[r].collision) {  // contact forces (zero for voxels off the collision surface)
        const double *c = a.lcc + 8 * (size_t)v;
        acc[0] += c[0]; acc[1] += c[1]; acc[2] += c[2];
        acc[7] += c[3]; acc[8] += c[4]; acc[9] += c[5];
        lbs += c[6];
        lE += c[7];
    }
    double *lv = a.lv + 13 * (size_t)v;
    for (int i = 0; i < 13; i++) lv[i] = acc[i];
    if (s.status[r] != 0) return;
    const VMat &m = d.vmat[fl >> 8];
    const RobotP &rp = d.rp[r];
    // this step's base size nomSize*(1 + T(t_k)*cte) (temperature_base_size at t_k)
    const double t = s.T[(size_t)a.parity * d.nr + r];
    if (rp.vary_temp && rp.temp_period > 0 && !(m.thermal_on_after > t) && !m.fixed) {
        const double arg = 2 * 3.1415926f * (t / rp.temp_period + d.phase[v]);
        const double T = rp.temp_amp * sin(arg);
        if (rp.expansion || !(T > 0))
            a.gphase[v] += lbs * m.nom_size * (double)m.cte * rp.temp_amp * cos(arg) * (double)(2 * 3.1415926f);
    }
    a.glogE[v] += lE * (double)m.E * 2.302585092994046;  // dE/dlog10(E) = E ln 10
}

// ------------------------------------------------------------ contact forces
// The force on surface voxel v from a listed partner u in contact
// (handle_collision_attachment + VX3_Collision::updateContactForce,
// src/VX3/VX3_VoxelyzeKernel.cu:682-727, src/VX3/VX3_Collision.cu:3-31) is, whichever
// is voxel1, G = uh*s with D = p_u - p_v, d = |D|, uh = D/d, s = k*rel + c*rv,
// rel = 0.625*(bs_v + bs_u) - d, rv = (w_v - w_u).uh, w = linMom/m,
// k = 2/(1/k_v + 1/k_u), k_i = 2*E_i*L_i, c = (c_v + c_u)/2, c_i ~ sqrt(E_i); and
// -G on u.  With mu = dL/dcontact_v - dL/dcontact_u and a = mu.uh:
//   dL/dD  = (s*(mu - a*uh) + a*c*((w_v - w_u) - rv*uh))/d - a*k*uh   (p_u: +, p_v: -)
//   dL/dw_v = a*c*uh,  dL/dbs_v = 0.625*a*k,
//   dL/dE_v = a*rel * 2*k_u^2/(k_v + k_u)^2 * 2*L_v + a*rv * c_v/(4*E_v).
// Each surface voxel gathers its own share from its partners in ascending order, with
// the reference's exact test deciding contact as in the forward pass.
__device__ __forceinline__ void adj_contact(const Dev &d, const Snap &s, const AdjBufs &a, int si) {
    const int v = d.csurf[si];
    double *out = a.lcc + 8 * (size_t)v;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint2 vi = s.vinfo[v];
    const int n = d.nnb[si];
    if (s.status[vi.x] == 0 && n > 0) {
        const int *lst = d.nbr + si;  // slot-major: entry k at lst[k*ns]
        const size_t ns = (size_t)d.ns;
        const double4 pv = s.pos[v], lmv4 = s.linmom[v];
        const double bsa = (pv.w + pv.w + pv.w) / 3.0f;
        const VMat &mv = d.vmat[vi.y >> 8];
        const V lcv{a.lcon[3 * (size_t)v], a.lcon[3 * (size_t)v + 1], a.lcon[3 * (size_t)v + 2]};
        const V wv = scl(V{lmv4.x, lmv4.y, lmv4.z}, mv.mass_inv);
        for (int k = 0; k < n; k++) {
            const int u = lst[k * ns];
            const double4 pu = s.pos[u];
            const double bu = (pu.w + pu.w + pu.w) / 3.0f;
            // the forward pass's exact test, voxel1 = the later surface voxel
            const double4 &p1 = u < v ? pv : pu, &p2 = u < v ? pu : pv;
            const double b1 = u < v ? bsa : bu, b2 = u < v ? bu : bsa;
            const V diff{p1.x - p2.x, p1.y - p2.y, p1.z - p2.z};
            const double wd = (b1 + b2) * 0.625;
            if (diff.x > wd || diff.x < -wd || diff.y > wd || diff.y < -wd || diff.z > wd || diff.z < -wd) continue;
            if (len(diff) > wd) continue;
            const V off{p2.x - p1.x, p2.y - p1.y, p2.z - p1.z};
            const double relf = (b1 + b2) * 0.625 - len(off);
            if (!(relf > 0)) continue;
            // the pair's force on v and its derivatives
            const uint2 ui = s.vinfo[u];
            const VMat &mu_ = d.vmat[ui.y >> 8];
            const double kk = 2.0f / (1.0f / mv.pstiff + 1.0f / mu_.pstiff);
            const double cc = 0.5f * (mv.c_col + mu_.c_col);
            const V D{pu.x - pv.x, pu.y - pv.y, pu.z - pv.z};
            const double dd = len(D);
            const V uh = scl(D, 1.0 / dd);
            const double rel = (bsa + bu) * 0.625 - dd;
            const double4 lmu4 = s.linmom[u];
            const V wu = scl(V{lmu4.x, lmu4.y, lmu4.z}, mu_.mass_inv);
            const V wvu = sub(wv, wu);
            const double rv = dot(wvu, uh);
            const double sf = kk * rel + cc * rv;
            const V mu{lcv.x - a.lcon[3 * (size_t)u], lcv.y - a.lcon[3 * (size_t)u + 1],
                       lcv.z - a.lcon[3 * (size_t)u + 2]};
            const double am = dot(mu, uh);
            const V gD = sub(scl(add(scl(sub(mu, scl(uh, am)), sf), scl(sub(wvu, scl(uh, rv)), am * cc)), 1.0 / dd),
                             scl(uh, am * kk));
            acc[0] -= gD.x; acc[1] -= gD.y; acc[2] -= gD.z;  // D = p_u - p_v
            const double lw = am * cc * (double)mv.mass_inv;
            acc[3] += lw * uh.x; acc[4] += lw * uh.y; acc[5] += lw * uh.z;
            acc[6] += 0.625 * am * kk;
            const double kv = mv.pstiff, ku = mu_.pstiff;
            acc[7] += am * rel * 2.0 * ku * ku / ((kv + ku) * (kv + ku)) * 2.0 * mv.nom_size +
                      am * rv * (double)mv.c_col / (4.0 * (double)mv.E);
        }
    }
    for (int i = 0; i < 8; i++) out[i] = acc[i];
}

// dL/d(final state) for L = sum_r w_r . COM_r(end): m_v/M_r * w_r on each measured voxel (k_com)
__device__ __forceinline__ void adj_seed(const Dev &d, const AdjBufs &a, int v) {
    const uint2 vi = d.vinfo[v];
    const int r = (int)vi.x;
    const VMat &m = d.vmat[vi.y >> 8];
    double *lv = a.lv + 13 * (size_t)v;
    for (int i = 0; i < 13; i++) lv[i] = 0.0;
    if (m.is_measured && a.mass_tot[r] > 0) {
        const double f = (double)m.mass / a.mass_tot[r];
        lv[0] = f * a.w[3 * r];
        lv[1] = f * a.w[3 * r + 1];
        lv[2] = f * a.w[3 * r + 2];
    }
}

}  // namespace adj
}  // namespace vx3g
