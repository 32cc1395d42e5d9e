// vx3g_step.cuh -- the two per-step passes, templated on the link-math type R.
//
//   R = double : the reference's arithmetic (FP64 vectors; float wherever the
//                reference uses float).  Compiled with --fmad=false so that the
//                rounding sequence matches the reference step op for op.
//   R = float  : FP32 link forces/moments and FP32 force/moment sums; positions,
//                momenta and quaternions stay FP64 and are advanced in FP64.
//
// Link pass  : VX3_Link::orientLink + updateForces + updateStrain
//              (src/VX3/VX3_Link.cu:90-260), one thread per link.
// Voxel pass : VX3_Voxel::timeStep with force()/moment()/floorForce()
//              (src/VX3/VX3_Voxel.cu:162-277, 350-426), one thread per voxel, plus the
//              next step's temperature (gpu_update_temperature, VX3_VoxelyzeKernel.cu:625-650).
#pragma once

#include <type_traits>

#include "vx3g_internal.h"

namespace vx3g {

template <class R> struct V3 { R x, y, z; };
template <class R> struct Q4 { R w, x, y, z; };

template <class R> __device__ __forceinline__ V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> __device__ __forceinline__ V3<R> add(V3<R> a, V3<R> b) { return V3<R>{a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> __device__ __forceinline__ V3<R> sub(V3<R> a, V3<R> b) { return V3<R>{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> __device__ __forceinline__ V3<R> neg(V3<R> a) { return V3<R>{-a.x, -a.y, -a.z}; }
// VX3_Vec3D::operator*(f) -> (f*x, f*y, f*z)   (VX3_Vec3D.h:49,61)
template <class R, class F> __device__ __forceinline__ V3<R> scl(V3<R> a, F f) {
    return V3<R>{(R)(f * a.x), (R)(f * a.y), (R)(f * a.z)};
}
// VX3_Vec3D::operator/(f) -> Inv = 1/f; (Inv*x, ...)   (VX3_Vec3D.h:63)
template <class R> __device__ __forceinline__ V3<R> vdiv(V3<R> a, R f) {
    R inv = (R)1.0 / f;
    return V3<R>{inv * a.x, inv * a.y, inv * a.z};
}
template <class R> __device__ __forceinline__ R len(V3<R> a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <class R> __device__ __forceinline__ V3<R> normalized(V3<R> a) {
    R l = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return l > 0 ? vdiv(a, l) : a;
}

template <class R> __device__ __forceinline__ Q4<R> qconj(Q4<R> q) { return Q4<R>{q.w, -q.x, -q.y, -q.z}; }
// VX3_Quat3D.h:217-222
template <class R> __device__ __forceinline__ Q4<R> qmul(Q4<R> a, Q4<R> f) {
    return Q4<R>{a.w * f.w - a.x * f.x - a.y * f.y - a.z * f.z, a.w * f.x + a.x * f.w + a.y * f.z - a.z * f.y,
                 a.w * f.y - a.x * f.z + a.y * f.w + a.z * f.x, a.w * f.z + a.x * f.y - a.y * f.x + a.z * f.w};
}
// VX3_Quat3D.h:439-447
template <class R> __device__ __forceinline__ V3<R> qrot(Q4<R> q, V3<R> f) {
    R tw = f.x * q.x + f.y * q.y + f.z * q.z;
    R tx = f.x * q.w - f.y * q.z + f.z * q.y;
    R ty = f.x * q.z + f.y * q.w - f.z * q.x;
    R tz = -f.x * q.y + f.y * q.x + f.z * q.w;
    return V3<R>{q.w * tx + q.x * tw + q.y * tz - q.z * ty, q.w * ty - q.x * tz + q.y * tw + q.z * tx,
                 q.w * tz + q.x * ty - q.y * tx + q.z * tw};
}
// VX3_Quat3D.h:465-473
template <class R> __device__ __forceinline__ V3<R> qrotinv(Q4<R> q, V3<R> f) {
    R tw = q.x * f.x + q.y * f.y + q.z * f.z;
    R tx = q.w * f.x - q.y * f.z + q.z * f.y;
    R ty = q.w * f.y + q.x * f.z - q.z * f.x;
    R tz = q.w * f.z - q.x * f.y + q.y * f.x;
    return V3<R>{tw * q.x + tx * q.w + ty * q.z - tz * q.y, tw * q.y - tx * q.z + ty * q.w + tz * q.x,
                 tw * q.z + tx * q.y - ty * q.x + tz * q.w};
}

// ToRotationVector (VX3_Quat3D.h:347-359).  The FP64 form is the reference's;
// the FP32 form computes 1-w^2 as |xyz|^2 and acos(w) as atan2(|xyz|, w), the
// same function without the cancellation that FP32 would suffer near w = 1.
template <class R> __device__ __forceinline__ V3<R> to_rotvec(Q4<R> q) {
    V3<R> v{q.x, q.y, q.z};
    if constexpr (std::is_same<R, double>::value) {
        if (q.w >= 1.0 || q.w <= -1.0) return V3<R>{0, 0, 0};
        double sq = 1.0 - q.w * q.w;
        if (sq < 2.4e-3) return scl(scl(v, 2.0), sqrt((2 - 2 * q.w) / sq));
        return vdiv(scl(scl(v, 2.0), acos(q.w)), sqrt(sq));
    } else {
        const float s2 = q.x * q.x + q.y * q.y + q.z * q.z;
        if (!(s2 > 0.0f)) return V3<R>{0, 0, 0};
        const float s = sqrtf(s2);
        return scl(v, 2.0f * atan2f(s, q.w) / s);
    }
}

// FromRotationVector (VX3_Quat3D.h:363-377)
template <class R> __device__ __forceinline__ Q4<R> from_rotvec(V3<R> in) {
    V3<R> th = vdiv(in, (R)2);
    R s, m2 = th.x * th.x + th.y * th.y + th.z * th.z;
    Q4<R> q;
    if (m2 * m2 < (R)5.328e-15) {
        q.w = (R)1.0 - (R)0.5 * m2;
        s = (R)1.0 - m2 / (R)6.0;
    } else {
        R m = sqrt(m2);
        q.w = cos(m);
        s = sin(m) / m;
    }
    q.x = th.x * s;
    q.y = th.y * s;
    q.z = th.z * s;
    return q;
}

// FromAngleToPosX (VX3_Quat3D.h:384-432); q unchanged for a zero vector
template <class R> __device__ __forceinline__ Q4<R> from_angle_to_posx(Q4<R> q, V3<R> r) {
    if (r.x == 0 && r.y == 0 && r.z == 0) return q;
    R yx = r.y / r.x, zx = r.z / r.x;
    const R SA = (R)1.732e-2;
    if (yx < SA && yx > -SA && zx < SA && zx > -SA) {
        q.x = 0;
        q.y = (R)0.5 * zx;
        q.z = (R)-0.5 * yx;
        q.w = 1 + (R)0.5 * (-q.y * q.y - q.z * q.z);
        return q;
    }
    V3<R> n = r;
    R l = sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
    if (l > 0) {
        R li = (R)1.0 / l;
        n.x *= li; n.y *= li; n.z *= li;
    }
    R theta = acos(n.x);
    if (theta > (R)(3.14159265358979 - 1e-7)) return Q4<R>{0, 0, 1, 0};
    R axis_inv = (R)1.0 / sqrt(n.z * n.z + n.y * n.y);
    R a = (R)0.5 * theta, s = sin(a);
    return Q4<R>{cos(a), 0, n.z * axis_inv * s, -n.y * axis_inv * s};
}

// VX3_Link.h:134-191 (bond-local +X frame and back)
// written as per-component selects (no branches: a warp's links mix the three axes)
template <class R> __device__ __forceinline__ V3<R> to_axis_x(int axis, V3<R> v) {
    const bool a1 = axis == 1, a2 = axis == 2;
    return V3<R>{a1 ? v.y : (a2 ? v.z : v.x), a1 ? -v.x : v.y, a2 ? -v.x : v.z};
}
template <class R> __device__ __forceinline__ Q4<R> to_axis_xq(int axis, Q4<R> q) {
    const bool a1 = axis == 1, a2 = axis == 2;
    return Q4<R>{q.w, a1 ? q.y : (a2 ? q.z : q.x), a1 ? -q.x : q.y, a2 ? -q.x : q.z};
}
template <class R> __device__ __forceinline__ V3<R> to_axis_original(int axis, V3<R> v) {
    const bool a1 = axis == 1, a2 = axis == 2;
    return V3<R>{a1 ? -v.y : (a2 ? -v.z : v.x), a1 ? v.x : v.y, a2 ? v.x : v.z};
}

// The voxel runs VX3_Voxel::force() in its timeStep (VX3_Voxel.cu:162-176): not of a Fixed
// material, not fixed in all DOFs by a boundary condition.  force() clears the voxel's
// contactForce (VX3_Voxel.cu:373-374); on those two kinds of voxel the contacts add up over the
// steps.  (A removed voxel, also flagged VF_FIXED, has no contacts and reports none.)
__device__ __forceinline__ bool runs_force(const Dev &d, int bcs, int v, uint32_t vflags) {
    if ((vflags & VF_FIXED) && d.vmat[vflags >> 8].fixed) return false;
    if (bcs && d.vext[v] >= 0 && d.ext[d.vext[v]].dof == EXT_ALL) return false;
    return true;
}

// Mixed-precision link state, in the 36 bytes per link of nine floats: a 16-byte row
// {pos2.x, pos2.y, pos2.z, angle2v.x} per link, an 8-byte row {angle2v.y, angle2v.z} per
// link, then angle1v's three components, component-major (read and written only for
// links in the large-angle branch)
__device__ __forceinline__ float4 *mixed_lstate_a(const Dev &d) { return reinterpret_cast<float4 *>(d.lstate); }
__device__ __forceinline__ float2 *mixed_lstate_b(const Dev &d) {
    return reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(d.lstate) + d.nl);
}
__device__ __forceinline__ float *mixed_lstate_c(const Dev &d) {
    return reinterpret_cast<float *>(reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(d.lstate) + d.nl) + d.nl);
}

// Mixed-precision slots: the slot of (direction dir, voxel v) is split into a 16-byte row
// {force x, y, z, moment x} and an 8-byte row {moment y, z}: six 16-byte rows per voxel
// direction-major, then six 8-byte rows, in the same 24 bytes per slot as Slot<float>,
// so that the link pass stores and the voxel pass loads each slot with two wide accesses
__device__ __forceinline__ void store_slot_mx(const Dev &d, int dir, int v, V3<float> f, V3<float> m) {
    const size_t i = (size_t)dir * d.nv + v;
    reinterpret_cast<float4 *>(d.slots)[i] = make_float4(f.x, f.y, f.z, m.x);
    reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(d.slots) + 6 * (size_t)d.nv)[i] = make_float2(m.y, m.z);
}
__device__ __forceinline__ void load_slot_mx(const Dev &d, int dir, int v, V3<float> *f, V3<float> *m) {
    const size_t i = (size_t)dir * d.nv + v;
    const float4 a = reinterpret_cast<const float4 *>(d.slots)[i];
    const float2 b = reinterpret_cast<const float2 *>(reinterpret_cast<const float4 *>(d.slots) + 6 * (size_t)d.nv)[i];
    *f = V3<float>{a.x, a.y, a.z};
    *m = V3<float>{a.w, b.x, b.y};
}

template <class R> __device__ __forceinline__ void store_slot(Slot<R> *s, V3<R> f, V3<R> m) {
    Slot<R> o;
    o.f[0] = f.x; o.f[1] = f.y; o.f[2] = f.z;
    o.m[0] = m.x; o.m[1] = m.y; o.m[2] = m.z;
    *s = o;
}

// VX3_MathTree::eval (src/Utils/VX3_MathTree.h:50-191): the token program is read in
// order; each token's result is appended to a value queue and operators consume the
// oldest unconsumed values (binary: values[pc + 1] op values[pc]).  Programs are
// validated when the context is created (known operators, the consumption cursor
// never passes the append cursor, mtEND within VX3G_MAX_MATH_TOKENS with exactly one
// value left), so the queue indices stay in bounds.  Variables hit, angle,
// targetCloseness and numClosePairs are 0 (the validated programs read none but hit,
// which the reference never changes from 0).
constexpr int kMaxMathTokens = 256;
#if !defined(__CUDACC__)
// host builds of this header (the host-compiled adjoint checks): Phi(x) = erfc(-x/sqrt 2)/2
inline double normcdf(double x) { return 0.5 * std::erfc(-x / std::sqrt(2.0)); }
#endif

__device__ inline double math_eval(const MathTok *tok, double x, double y, double z, double t, double num_voxel) {
    double vals[kMaxMathTokens];
    int vc = 0, pc = 0;
    for (int i = 0; i < kMaxMathTokens; i++) {
        const MathTok k = tok[i];
        double r;
        switch (k.op) {
            case 0: return vals[pc < vc ? pc : 0];  // mtEND
            case 1: r = k.value; break;
            case 2: r = 2.71828182845904523536; break;
            case 3: r = 3.14159265358979323846; break;
            case 4: {
                const double w = k.value;
                r = w < 0.5 ? x : w < 1.5 ? y : w < 2.5 ? z : (w >= 3.5 && w < 4.5) ? t : (w >= 7.5 && w < 8.5) ? num_voxel : 0.0;
                break;
            }
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
            case 23: r = normcdf(vals[pc]); pc++; break;
            default: return 0.0;
        }
        vals[vc++] = r;
    }
    return 0.0;
}

// v has a link to u (is_neighbor depth 1, VX3_VoxelyzeKernel.cu:651-680) in the current link
// table: robots whose links can be made at runtime keep each face's partner in Dev::vnb
__device__ __forceinline__ bool linked_to(const Dev &d, int v, int u) {
    const uint32_t m = d.vinfo[v].y & VF_LINKMASK;
    for (int k = 0; k < 6; k++)
        if (((m >> k) & 1u) && d.vnb[6 * (size_t)v + k] == u) return true;
    return false;
}

// the force field of robot rp at position (x, y, z) and time t (VX3_Voxel.cu:178-184)
__device__ inline V3<double> force_field(const Dev &d, const RobotP &rp, double x, double y, double z, double t) {
    const double nv = (double)rp.nv;
    return V3<double>{rp.ff[0] >= 0 ? math_eval(d.ftok + rp.ff[0], x, y, z, t, nv) : 0.0,
                      rp.ff[1] >= 0 ? math_eval(d.ftok + rp.ff[1], x, y, z, t, nv) : 0.0,
                      rp.ff[2] >= 0 ? math_eval(d.ftok + rp.ff[2], x, y, z, t, nv) : 0.0};
}

// ------------------------------------------------------------- link material models
// VX3_Material::stress (src/VX3/VX3_Material.cu:90-124) of link material m at strain eps:
// zero past failure; the linear law for linear models, in compression and on the first
// segment (or when forced); else the segment of the data points holding eps (the last
// one extrapolated), with the volumetric variant when Poisson's ratio is on.  The data
// points are read only on a non-linear segment.
__device__ __forceinline__ float model_stress(const LMat &m, const float2 *pts, float eps, float tss, bool force_linear) {
    if (m.eps_fail != -1.0f && eps > m.eps_fail) return 0.0f;
    if (m.lin || force_linear || eps <= pts[1].x) {
        if (m.nu == 0.0f) return m.E * eps;
        return m.eHat * ((1 - m.nu) * eps + m.nu * tss);
    }
    for (int i = 2; i < m.ssn; i++) {
        const float2 a = pts[i - 1], b = pts[i];
        if (eps <= b.x || i == m.ssn - 1) {
            const float perc = (eps - a.x) / (b.x - a.x);
            const float basic = a.y + perc * (b.y - a.y);
            if (m.nu == 0.0f) return basic;
            const float modulus = (b.y - a.y) / (b.x - a.x);
            const float mod_hat = modulus / ((1 - 2 * m.nu) * (1 + m.nu));
            const float eff = basic / modulus;  // strain where the segment's line from 0 reaches the stress
            const float eff_tss = tss * (eff / eps);
            return mod_hat * ((1 - m.nu) * eff + m.nu * eff_tss);
        }
    }
    return 0.0f;
}

// VX3_Link::updateStrain (src/VX3/VX3_Link.cu:220-260): the link's stress at axial strain
// eps, with maxStrain (*max_strain) and, for non-linear materials, the plastic
// strainOffset (d.soff[l]): on new ground the curve is followed and the offset of the
// unloading line recorded; below the largest strain reached the material unloads
// linearly from that offset.
__device__ __forceinline__ float link_stress(const Dev &d, const LMat &m, int l, float eps, float *max_strain) {
    if (m.lin) {
        if (eps > *max_strain) *max_strain = eps;
        return model_stress(m, nullptr, eps, m.tss, false);
    }
    const float2 *pts = d.ss + m.sso;
    if (eps > *max_strain) {
        *max_strain = eps;
        const float st = model_stress(m, pts, eps, m.tss, false);
        d.soff[l] = m.nu != 0.0f ? *max_strain - model_stress(m, pts, eps, 0.0f, false) / (m.eHat * (1 - m.nu))
                                 : *max_strain - st / m.E;
        return st;
    }
    const float rel = eps - d.soff[l];
    return m.nu != 0.0f ? model_stress(m, pts, rel, m.tss, true) : m.E * rel;
}

// ------------------------------------------------------------- link pass
// isNewLink (VX3_Link.cu:206-213): a runtime link's forces and moments, just stored, are
// scaled by 0.01 for its first SafetyGuard updates (the product of the stored value is the
// product the reference forms before storing).  The slots are read back through volatile
// pointers, so the common path's values need not stay live across this rare branch.
template <class R> __device__ __forceinline__ void new_link_scale(const Dev &d, int l, Slot<R> *sNeg, Slot<R> *sPos) {
    const int n = d.lnew[l];
    if (n == 0) return;
    const R k = (R)0.01;
    volatile R *a = reinterpret_cast<volatile R *>(sNeg), *b = reinterpret_cast<volatile R *>(sPos);
    for (int c = 0; c < 6; c++) {
        a[c] = a[c] * k;
        b[c] = b[c] * k;
    }
    d.lnew[l] = n - 1;
}

// the same for a runtime link's two mixed-precision slots (negative end: direction dneg)
__device__ __forceinline__ void new_link_scale_mx(const Dev &d, int l, int dneg, int vneg, int vpos) {
    const int n = d.lnew[l];
    if (n == 0) return;
    for (int e = 0; e < 2; e++) {
        const size_t i = (size_t)(dneg + e) * d.nv + (e ? vpos : vneg);
        volatile float *a = reinterpret_cast<volatile float *>(reinterpret_cast<float4 *>(d.slots) + i);
        volatile float *b =
            reinterpret_cast<volatile float *>(reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(d.slots) + 6 * (size_t)d.nv) + i);
        for (int c = 0; c < 4; c++) a[c] = a[c] * 0.01f;
        for (int c = 0; c < 2; c++) b[c] = b[c] * 0.01f;
    }
    d.lnew[l] = n - 1;
}

template <class R> __device__ __forceinline__ void link_update(const Dev &d, int l) {
    const uint2 li = d.linfo[l];
    const int r = (int)li.x;
    if (d.status[r] != 0) return;
    uint32_t fl = li.y;
    if (fl & (LF_BOTH_FIXED | LF_GONE)) return;  // gpu_update_links skips both-fixed and detached links
    const int axis = fl & LF_AXIS;
    const int2 e = d.ends[l];
    const double4 pn = d.pos[e.x], pp = d.pos[e.y];
    const double4 qn = d.quat[e.x], qp = d.quat[e.y];
    const double rest = 0.5 * (pn.w + pp.w);  // VX3_Link::updateRestLength (VX3_Link.cu:80-83)
    const LMat &m = d.lmat[fl >> 8];
    R *ls = (R *)d.lstate;
    const size_t NL = (size_t)d.nl;
    const V3<R> oldPos2{ls[l], ls[NL + l], ls[2 * NL + l]};
    const V3<R> oldA1{ls[3 * NL + l], ls[4 * NL + l], ls[5 * NL + l]};
    const V3<R> oldA2{ls[6 * NL + l], ls[7 * NL + l], ls[8 * NL + l]};

    // orientLink (VX3_Link.cu:90-133)
    V3<R> pos2 = to_axis_x(axis, V3<R>{(R)(pp.x - pn.x), (R)(pp.y - pn.y), (R)(pp.z - pn.z)});
    Q4<R> angle1 = to_axis_xq(axis, Q4<R>{(R)qn.x, (R)qn.y, (R)qn.z, (R)qn.w});
    Q4<R> angle2 = to_axis_xq(axis, Q4<R>{(R)qp.x, (R)qp.y, (R)qp.z, (R)qp.w});
    const Q4<R> tot = qconj(angle1);
    pos2 = qrot(tot, pos2);
    angle2 = qmul(tot, angle2);
    angle1 = Q4<R>{1, 0, 0, 0};
    const R restR = (R)rest;
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
    if (small) {
        pos2.x -= restR;
    } else {
        angle1 = from_angle_to_posx(angle1, pos2);
        angle2 = qmul(angle1, angle2);
        pos2 = V3<R>{len(pos2) - restR, 0, 0};
    }
    const V3<R> a1v = to_rotvec(angle1), a2v = to_rotvec(angle2);
    ls[l] = pos2.x; ls[NL + l] = pos2.y; ls[2 * NL + l] = pos2.z;
    ls[3 * NL + l] = a1v.x; ls[4 * NL + l] = a1v.y; ls[5 * NL + l] = a1v.z;
    ls[6 * NL + l] = a2v.x; ls[7 * NL + l] = a2v.y; ls[8 * NL + l] = a2v.z;

    // updateForces (VX3_Link.cu:135-218) + updateStrain (:220-260), linear model
    const R half = (R)0.5;
    const V3<R> dPos2 = scl(sub(pos2, oldPos2), half);
    const V3<R> dA1 = scl(sub(a1v, oldA1), half);
    const V3<R> dA2 = scl(sub(a2v, oldA2), half);
    const float axialStrain = (float)(pos2.x / restR);
    float2 sm = d.strain[l];
    sm.x = axialStrain;
    const float stress = link_stress(d, m, l, axialStrain, &sm.y);
    d.strain[l] = sm;
    if (axialStrain > 100) atomicOr(&d.status[r], 1);  // divergence (VX3_VoxelyzeKernel.cu:271-281)

    Slot<R> *S = (Slot<R> *)d.slots;
    Slot<R> *sNeg = &S[(size_t)(2 * axis) * d.nv + e.x];
    Slot<R> *sPos = &S[(size_t)(2 * axis + 1) * d.nv + e.y];
    uint32_t nfl = (fl & ~(LF_SMALL | LF_LVV)) | (small ? LF_SMALL : 0u);
    if (m.eps_fail != -1.0f && sm.y > m.eps_fail) {  // isFailed: forces zero (lvv unchanged)
        const V3<R> z{0, 0, 0};
        store_slot(sNeg, z, z);
        store_slot(sPos, z, z);
        nfl |= lvv ? LF_LVV : 0u;
        if (nfl != fl) d.linfo[l].y = nfl;
        return;
    }
    const float b1 = m.b1, b2 = m.b2, b3 = m.b3, a2 = m.a2;
    V3<R> fNeg{(R)(stress * m.area), b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y)};
    V3<R> fPos = neg(fNeg);
    V3<R> mNeg{a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z)};
    V3<R> mPos{a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z)};
    if (lvv) {
        const float sqA1 = m.sqA1, sqA2xIp = m.sqA2xIp, sqB1 = m.sqB1, sqB2xFMp = m.sqB2xFMp, sqB3xIp = m.sqB3xIp;
        const V3<R> posCalc{sqA1 * dPos2.x, sqB1 * dPos2.y - sqB2xFMp * (dA1.z + dA2.z),
                            sqB1 * dPos2.z + sqB2xFMp * (dA1.y + dA2.y)};
        // VX3_Voxel::dampingMultiplier (VX3_Voxel.h:206-208); previousDt is this robot's dt
        // once a voxel has stepped, 0 for fixed voxels (they never step)
        const float dtf = d.dt[r];
        const uint32_t fnv = d.vinfo[e.x].y, fpv = d.vinfo[e.y].y;
        const float dmN = d.vmat[fnv >> 8].dmc / ((fnv & VF_FIXED) ? 0.0f : dtf);
        const float dmP = d.vmat[fpv >> 8].dmc / ((fpv & VF_FIXED) ? 0.0f : dtf);
        fNeg = add(fNeg, scl(posCalc, dmN));
        fPos = sub(fPos, scl(posCalc, dmP));
        mNeg = sub(mNeg, scl(V3<R>{-sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (2 * dA1.y + dA2.y),
                                   -sqB2xFMp * dPos2.y + sqB3xIp * (2 * dA1.z + dA2.z)},
                            (R)(half * dmN)));
        mPos = sub(mPos, scl(V3<R>{sqA2xIp * (dA2.x - dA1.x), sqB2xFMp * dPos2.z + sqB3xIp * (dA1.y + 2 * dA2.y),
                                   -sqB2xFMp * dPos2.y + sqB3xIp * (dA1.z + 2 * dA2.z)},
                            (R)(half * dmP)));
    } else {
        lvv = true;
    }
    nfl |= lvv ? LF_LVV : 0u;
    if (!small) {
        fNeg = qrotinv(angle1, fNeg);
        mNeg = qrotinv(angle1, mNeg);
    }
    fPos = qrotinv(angle2, fPos);
    mPos = qrotinv(angle2, mPos);
    store_slot(sNeg, to_axis_original(axis, fNeg), to_axis_original(axis, mNeg));
    store_slot(sPos, to_axis_original(axis, fPos), to_axis_original(axis, mPos));
    if (fl & LF_RUNTIME) new_link_scale(d, l, sNeg, sPos);
    if (nfl != fl) d.linfo[l].y = nfl;
}

template <class R> __global__ void __launch_bounds__(256) k_links(Dev d) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < d.nl) link_update<R>(d, l);
}

// ------------------------------------------------------------ voxel pass
// Temperature of a voxel at time t (gpu_update_temperature, VX3_VoxelyzeKernel.cu:625-650)
// returned as the base size nomSize*(1+T*cte) (VX3_Voxel::baseSize); tempe gets T.
template <bool EXACT> __device__ __forceinline__ double temperature_base_size(const RobotP &rp, const VMat &m,
                                                                              double phase, double t,
                                                                              double cur_bs, float *tempe) {
    if (!(rp.vary_temp && rp.temp_period > 0)) return cur_bs;
    if (m.thermal_on_after > t || m.fixed) return cur_bs;
    double T;
    if (EXACT) {
        T = rp.temp_amp * sin(2 * 3.1415926f * (t / rp.temp_period + phase));
    } else {
        // same phase in cycles, reduced to [0,1) in FP64, sine in FP32
        double c = (double)(2 * 3.1415926f) * (t / rp.temp_period + phase) * (1.0 / 6.283185307179586);
        c -= floor(c);
        T = rp.temp_amp * (double)sinpif(2.0f * (float)c);
    }
    if (!rp.expansion && T > 0) T = 0;
    const float tf = (float)T;
    *tempe = tf;
    return m.nom_size * (1 + tf * m.cte);
}

template <class R> __device__ __forceinline__ void voxel_update(const Dev &d, int v, int parity) {
    constexpr bool EXACT = std::is_same<R, double>::value;
    const uint2 vi = d.vinfo[v];
    const int r = (int)vi.x;
    const RobotP &rp = d.rp[r];
    const double Tcur = d.T[(size_t)parity * d.nr + r];
    const int st = d.status[r];
    const float dtf = d.dt[r];
    if (v == rp.voff) d.T[(size_t)(parity ^ 1) * d.nr + r] = (st == 0) ? Tcur + dtf : Tcur;  // currentTime += dt
    if (st != 0) return;
    uint32_t fl = vi.y;
    if (fl & VF_FIXED) return;
    const VMat m = d.vmat[fl >> 8];
    const double dt = dtf;
    double4 p = d.pos[v];
    const double4 q = d.quat[v];
    const double4 lm = d.linmom[v];
    const double4 am = d.angmom[v];
    const double tn = Tcur + dt;

    const bool actuated = rp.vary_temp && rp.temp_period > 0;
    float *tcur = d.tempe + (size_t)parity * d.nv, *tnext = d.tempe + (size_t)(parity ^ 1) * d.nv;
    if (dt == 0.0f) {  // VX3_Voxel::timeStep returns before moving; temperature still follows time
        if (actuated) {
            float te = tcur[v];
            p.w = temperature_base_size<EXACT>(rp, m, d.phase[v], tn, p.w, &te);
            d.pos[v] = p;
            tnext[v] = te;
        }
        return;
    }

    // boundary-condition external (VX3_External), if any
    const int xi = rp.bcs ? d.vext[v] : -1;
    ExtBC ex{};
    if (xi >= 0) ex = d.ext[xi];
    const int dof = ex.dof;
    if (dof == EXT_ALL) {  // isFixedAll (VX3_Voxel.cu:167-173): at its prescribed pose, motion halted
        const short4 l = d.ijk[v];
        p.x = l.x * m.nom_size + ex.t.x;
        p.y = l.y * m.nom_size + ex.t.y;
        p.z = l.z * m.nom_size + ex.t.z;
        d.quat[v] = ex.q;
        d.linmom[v] = make_double4(0, 0, 0, 0);
        d.angmom[v] = make_double4(0, 0, 0, 0);
        if (actuated) {
            float te = tcur[v];
            p.w = temperature_base_size<EXACT>(rp, m, d.phase[v], tn, p.w, &te);
            tnext[v] = te;
        }
        d.pos[v] = p;
        return;
    }

    // link force/moment sums in direction order 0..5 (VX3_Voxel::force/moment, VX3_Voxel.cu:350-397)
    V3<R> Fs{0, 0, 0}, Ms{0, 0, 0};
    const Slot<R> *S = (const Slot<R> *)d.slots;
#pragma unroll
    for (int dir = 0; dir < 6; dir++) {
        if (fl & (1u << dir)) {
            const Slot<R> s = S[(size_t)dir * d.nv + v];
            Fs = add(Fs, V3<R>{s.f[0], s.f[1], s.f[2]});
            Ms = add(Ms, V3<R>{s.m[0], s.m[1], s.m[2]});
        }
    }
    bool stat = (fl & VF_STATIC) != 0;
    const bool floorOn = rp.floor != 0;
    const double bs = p.w;
    const double bsa = (bs + bs + bs) / 3.0f;  // baseSizeAverage (VX3_Voxel.h:102-105)
    // floorPenetration (VX3_Voxel.h:185-188), before the position update
    const float pen = (float)(bsa / 2 - m.nom_size / 2 - p.z);
    V3<double> lmv{lm.x, lm.y, lm.z}, amv{am.x, am.y, am.z};
    V3<double> tr;

    if constexpr (EXACT) {
        const Q4<double> o{q.x, q.y, q.z, q.w};
        V3<double> F = qrot(o, Fs);
        if (xi >= 0) F = add(F, V3<double>{ex.f[0], ex.f[1], ex.f[2]});  // external force (:363-364)
        const V3<double> vel = scl(lmv, m.mass_inv);
        F = sub(F, scl(vel, m.c_glob));
        F.z += m.grav_force;
        if (rp.collision) {
            const double4 c = d.contact[v];
            F = sub(F, V3<double>{c.x, c.y, c.z});
        }
        if (rp.cilia) {  // CiliaForce * Cilia (VX3_Voxel.cu:376), from k_extra_forces
            const double4 c = d.cfv[v];
            F = add(F, V3<double>{c.x, c.y, c.z});
        } else {
            F = add(F, V3<double>{0.0, 0.0, 0.0});  // no cilia: CiliaForce is 0
        }
        if (rp.ff_any) {  // force field (VX3_Voxel.cu:178-184), evaluated by k_extra_forces
            const double4 ff = d.ffv[v];
            F.x += ff.x;
            F.y += ff.y;
            F.z += ff.z;
        }
        V3<double> fric = F;
        if (floorOn) {  // floorForce (VX3_Voxel.cu:399-426)
            if (pen >= 0) {
                const float normal = m.pstiff * pen;
                F.z += normal - m.c_col * vel.z;
                if (stat) {
                    const float surf = (float)(F.x * F.x + F.y * F.y);
                    const float fr = (m.mu_s * normal) * (m.mu_s * normal);
                    if (surf > fr) stat = false;
                } else {
                    F = sub(F, scl(normalized(V3<double>{vel.x, vel.y, 0}), m.mu_k * normal));
                }
            } else {
                stat = false;
            }
        }
        fric = sub(F, fric);
        lmv = add(lmv, scl(F, dt));
        tr = scl(lmv, dt * m.mass_inv);
        if (floorOn && pen >= 0) {
            const double work = fric.x * tr.x + fric.y * tr.y;
            const double hKe = 0.5 * m.mass_inv * (lmv.x * lmv.x + lmv.y * lmv.y);
            if (hKe + work <= 0) stat = true;
            if (stat) {
                lmv.x = lmv.y = 0;
                tr.x = tr.y = 0;
            }
        } else {
            stat = false;
        }
        p.x += tr.x; p.y += tr.y; p.z += tr.z;
        V3<double> M = qrot(o, Ms);
        if (xi >= 0) M = add(M, V3<double>{ex.m[0], ex.m[1], ex.m[2]});  // external moment (:393-394)
        M = sub(M, scl(scl(amv, m.mom_inv), m.c_glob_rot));
        amv = add(amv, scl(M, dt));
        Q4<double> on = qmul(from_rotvec(scl(amv, dt * m.mom_inv)), o);
        if (dof) {  // fixed DOFs (VX3_Voxel.cu:222-257)
            const short4 l = d.ijk[v];
            if (dof & 1) { p.x = l.x * m.nom_size + ex.t.x; lmv.x = 0; }
            if (dof & 2) { p.y = l.y * m.nom_size + ex.t.y; lmv.y = 0; }
            if (dof & 4) { p.z = l.z * m.nom_size + ex.t.z; lmv.z = 0; }
            if (dof & EXT_R) {
                if ((dof & EXT_R) == EXT_R) {  // all rotations: the prescribed orientation
                    on = Q4<double>{ex.q.x, ex.q.y, ex.q.z, ex.q.w};
                    amv = V3<double>{0, 0, 0};
                } else {  // some: zero those components of the rotation vector
                    V3<double> rv = to_rotvec(on);
                    if (dof & 8) { rv.x = 0; amv.x = 0; }
                    if (dof & 16) { rv.y = 0; amv.y = 0; }
                    if (dof & 32) { rv.z = 0; amv.z = 0; }
                    on = from_rotvec(rv);
                }
            }
        }
        d.quat[v] = make_double4(on.w, on.x, on.y, on.z);
    } else {
        const Q4<float> o{(float)q.x, (float)q.y, (float)q.z, (float)q.w};
        V3<float> F = qrot(o, Fs);
        const V3<float> vel{(float)lm.x * m.mass_inv, (float)lm.y * m.mass_inv, (float)lm.z * m.mass_inv};
        F = sub(F, scl(vel, m.c_glob));
        F.z += m.grav_force;
        if (rp.collision) {
            const double4 c = d.contact[v];
            F = sub(F, V3<float>{(float)c.x, (float)c.y, (float)c.z});
        }
        if (rp.cilia) {
            const double4 c = d.cfv[v];
            F = add(F, V3<float>{(float)c.x, (float)c.y, (float)c.z});
        }
        if (rp.ff_any) {
            const double4 ff = d.ffv[v];
            F = add(F, V3<float>{(float)ff.x, (float)ff.y, (float)ff.z});
        }
        V3<float> fric = F;
        if (floorOn) {
            if (pen >= 0) {
                const float normal = m.pstiff * pen;
                F.z += normal - m.c_col * vel.z;
                if (stat) {
                    if (F.x * F.x + F.y * F.y > (m.mu_s * normal) * (m.mu_s * normal)) stat = false;
                } else {
                    F = sub(F, scl(normalized(V3<float>{vel.x, vel.y, 0}), m.mu_k * normal));
                }
            } else {
                stat = false;
            }
        }
        fric = sub(F, fric);
        lmv.x += (double)F.x * dt; lmv.y += (double)F.y * dt; lmv.z += (double)F.z * dt;
        tr = scl(lmv, dt * (double)m.mass_inv);
        if (floorOn && pen >= 0) {
            const float work = fric.x * (float)tr.x + fric.y * (float)tr.y;
            const float hKe = 0.5f * m.mass_inv * ((float)lmv.x * (float)lmv.x + (float)lmv.y * (float)lmv.y);
            if (hKe + work <= 0) stat = true;
            if (stat) {
                lmv.x = lmv.y = 0;
                tr.x = tr.y = 0;
            }
        } else {
            stat = false;
        }
        p.x += tr.x; p.y += tr.y; p.z += tr.z;
        V3<float> M = qrot(o, Ms);
        const V3<float> avel{(float)am.x * m.mom_inv, (float)am.y * m.mom_inv, (float)am.z * m.mom_inv};
        M = sub(M, scl(avel, m.c_glob_rot));
        amv.x += (double)M.x * dt; amv.y += (double)M.y * dt; amv.z += (double)M.z * dt;
        // q' = dq*q = q + (dq - 1)*q : the small increment in FP32, the sum in FP64
        const float k = (float)(dt * (double)m.mom_inv);
        const Q4<float> dq = from_rotvec(V3<float>{(float)amv.x * k, (float)amv.y * k, (float)amv.z * k});
        const float th2 = dq.x * dq.x + dq.y * dq.y + dq.z * dq.z;
        const float dw = (dq.w > 0.999f) ? -th2 / (1.0f + dq.w) : dq.w - 1.0f;  // dq.w - 1 without cancellation
        const Q4<float> delta = qmul(Q4<float>{dw, dq.x, dq.y, dq.z}, o);
        d.quat[v] = make_double4(q.x + delta.w, q.y + delta.x, q.z + delta.y, q.w + delta.z);
    }
    // static friction freezes rotation (VX3_Voxel.cu:259-264), penetration after the move
    if (floorOn && (float)(bsa / 2 - m.nom_size / 2 - p.z) >= 0 && stat) amv = V3<double>{0, 0, 0};

    // next step's temperature; tempe is double-buffered by step parity so that the
    // buffer of the step just taken keeps the value that step used (the reference's tempe)
    if (actuated) {
        float te = tcur[v];
        p.w = temperature_base_size<EXACT>(rp, m, d.phase[v], tn, bs, &te);
        tnext[v] = te;
    }
    d.pos[v] = p;
    d.linmom[v] = make_double4(lmv.x, lmv.y, lmv.z, 0.0);
    d.angmom[v] = make_double4(amv.x, amv.y, amv.z, 0.0);
    const uint32_t nfl = stat ? (fl | VF_STATIC) : (fl & ~VF_STATIC);
    if (nfl != fl) d.vinfo[v].y = nfl;
}

template <class R> __global__ void __launch_bounds__(256) k_voxels(Dev d, int parity) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < d.nv) voxel_update<R>(d, v, parity);
}

}  // namespace vx3g
