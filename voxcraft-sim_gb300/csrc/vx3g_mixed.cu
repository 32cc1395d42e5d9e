// vx3g_mixed.cu -- the mixed-precision step: FP32 link forces and moments,
// compensated FP32 (hi + lo float pairs, two-sum arithmetic) for positions,
// orientations and momenta.  No FP64 arithmetic runs per link or per voxel (the actuation
// phase is reduced in FP64 once per robot and step).  Quotients and square roots on the
// hot paths use the hardware reciprocal and reciprocal square root (__fdividef, rsqrtf:
// within 2 ulp), fixed instructions, so every compiled launch shape computes the same
// values; the FP64 step keeps the reference's correctly rounded operations.
//
// The link pass restates VX3_Link::orientLink/updateForces (src/VX3/VX3_Link.cu:90-218)
// without the cancellations FP32 would suffer:
//  * pos2 = R(conj(q1)) * toAxisX(pPos - pNeg) is formed as
//      L*R(conj(q1))e_x + R(conj(q1)) * toAxisX(delta),  delta = (pPos - pNeg) - L*e_axis,
//    with delta taken from the hi/lo pairs (exact differences of nearby values) and
//    R(q)e_x - e_x = (-2(y^2+z^2), 2(xy-wz), 2(xz+wy)) evaluated directly, so the axial
//    deviation pos2.x - L never subtracts two nearly equal FP32 numbers;
//  * angle2 = conj(q1)*q2 = |q1|^2 + conj(q1)*(q2 - q1), the difference again from the
//    hi/lo pairs; the rotation vector uses 2*atan2(|v|, w)/|v|.
// The voxel pass restates VX3_Voxel::timeStep (src/VX3/VX3_Voxel.cu:162-277) with the
// same sums in FP32 and every accumulation (p += F dt, x += p dt/m, L += M dt,
// q += (dq - 1) q) done as a two-sum into the hi/lo pair.
#include <math_constants.h>

#include "vx3g_step.cuh"

namespace vx3g {

__device__ __forceinline__ void quick_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// (hi, lo) += x
__device__ __forceinline__ void df_add(float &hi, float &lo, float x) {
    float s, e;
    two_sum(hi, x, s, e);
    e += lo;
    quick_two_sum(s, e, hi, lo);
}
// (ah + al) - (bh + bl) to FP32 accuracy: the rounding of ah - bh is at most half an ulp of
// the difference itself (and none when ah and bh are within a factor 2), so no two-sum is
// needed when nothing is subtracted from the result afterwards
__device__ __forceinline__ float df_diff(float ah, float al, float bh, float bl) { return (ah - bh) + (al - bl); }
// (ah + al) - (bh + bl) - (ch + cl): the axial deviation of a link (a - b ~= c).  The
// rounding of ah - bh is kept (two-sum): it can be as large as the deviation; s - ch is
// exact (Sterbenz) while the link's strain lies between -50% and +100%, and otherwise
// rounds a deviation as large as the rest length
__device__ __forceinline__ float df_diff3(float ah, float al, float bh, float bl, float ch, float cl) {
    float s, e;
    two_sum(ah, -bh, s, e);
    return (s - ch) + (e + ((al - bl) - cl));
}

// ToRotationVector (src/VX3/VX3_Quat3D.h:347-359) of a unit quaternion (w, v) in FP32.
// The reference takes 1 - w^2 as the squared sine of the half angle and, below
// 2.4e-3 (rotations under about 0.098 rad), does not evaluate the rotation vector
// 2*acos(w)/sin(theta/2) * v but the approximation 2*sqrt((2 - 2w)/(1 - w^2)) * v =
// 2*sqrt(2/(1 + w)) * v, which is smaller by about theta^2/96 relative: 2.6e-5 at
// 0.05 rad, far above FP32 rounding, in every link's bending and torsion terms.  The
// same two branches are taken here, with 1 - w^2 formed as |v|^2 (no cancellation)
// and acos(w)/sin as atan2(|v|, w)/|v|.
__device__ __forceinline__ V3<float> rotvec_f(float w, V3<float> v) {
    const float s2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (!(s2 > 0.0f)) return V3<float>{0, 0, 0};
    if (s2 < 2.4e-3f) return scl(v, 2.82842712f * rsqrtf(1.0f + w));
    const float is = rsqrtf(s2);  // s2 >= 2.4e-3 here
    return scl(v, 2.0f * atan2f(s2 * is, w) * is);
}

// FromAngleToPosX (src/VX3/VX3_Quat3D.h:384-432) in FP32: the rotation taking r to
// +x.  The reference forms theta = acos(n.x) for n = r/|r| and returns
// (cos(theta/2), 0, n.z sin(theta/2)/|(n.y, n.z)|, -n.y sin(theta/2)/|(n.y, n.z)|).
// With the half-angle identities cos(theta/2) = sqrt((1 + n.x)/2) and
// sin(theta/2)/|(n.y, n.z)| = sqrt((1 - n.x)/2)/sqrt(1 - n.x^2) = 1/sqrt(2(1 + n.x))
// that is (c/2, 0, n.z/c, -n.y/c) with c = sqrt(2(1 + n.x)): one square root and one
// reciprocal instead of acos, sin and cos.  The small-angle shortcut and the
// turned-around case (theta within 1e-7 of pi, where 1 + n.x underflows in FP32)
// are the reference's.
__device__ __forceinline__ Q4<float> from_angle_to_posx_f(Q4<float> q, V3<float> r) {
    if (r.x == 0 && r.y == 0 && r.z == 0) return q;
    const float yx = __fdividef(r.y, r.x), zx = __fdividef(r.z, r.x);
    const float SA = 1.732e-2f;
    if (yx < SA && yx > -SA && zx < SA && zx > -SA) {
        q.x = 0;
        q.y = 0.5f * zx;
        q.z = -0.5f * yx;
        q.w = 1 + 0.5f * (-q.y * q.y - q.z * q.z);
        return q;
    }
    const float il = rsqrtf(r.x * r.x + r.y * r.y + r.z * r.z);
    const float nx = r.x * il, ny = r.y * il, nz = r.z * il;
    const float t = 2.0f * (1.0f + nx);
    if (!(t > 0.0f)) return Q4<float>{0, 0, 1, 0};
    const float ic = rsqrtf(t), c = t * ic;
    return Q4<float>{0.5f * c, 0, nz * ic, -ny * ic};
}

// ------------------------------------------------------------- collision narrow phase
// handle_collision_attachment + VX3_Collision::updateContactForce
// (src/VX3/VX3_VoxelyzeKernel.cu:682-727, src/VX3/VX3_Collision.cu:3-31) on the
// listed pairs, in FP32: the pair offset is taken from the hi/lo pairs (one rounding
// of an exact difference), the envelope test and the force in FP32, contacts summed
// in ascending partner order as the FP64 pass does.
// ATTACH: the batch has robots with EnableAttach (their pairs linked this step have their
// contact added, then taken back); the other instance carries none of that code
template <bool ATTACH> __global__ void __launch_bounds__(256) k_coll_eval_mixed(Dev d) {
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
    // stopped robots and robots flagged before this step keep their contact forces; the
    // divergence bit is left out because the link pass, which may set it, runs beside
    // this kernel (a diverged robot never steps again, so its contacts feed nothing)
    if (d.status[r] & ~1) return;
    const int n = d.nnb[s];
    const int *lst = d.nbr + s;  // slot-major: entry k at lst[k*ns]
    const size_t ns = (size_t)d.ns;
    const float4 *R = d.crec;  // contact records of this step (written by the displacement check)
    // pairs linked by this step's attachment: contact added, then taken back
    const bool att = ATTACH && d.rp[r].attach && d.acnt[r] > 0;
    V3<float> acc{0, 0, 0};
    if (!runs_force(d, d.rp[r].bcs, v, vi.y)) {  // its contactForce is never cleared: the pairs add to it
        const float4 c = reinterpret_cast<const float4 *>(d.contact)[v];
        acc = V3<float>{c.x, c.y, c.z};
    }
    if (n) {
        const float4 pvH = R[2 * v], pvL = R[2 * v + 1], wv = R[2 * d.nv + v];
        const float bv = pvH.w;  // baseSizeAverage = baseSize (isotropic)
        for (int k = 0; k < n; k++) {
            const int u = lst[k * ns];  // partner voxel, ascending
            const float4 puH = R[2 * u], puL = R[2 * u + 1];  // one 32-byte sector
            // offset from the later surface voxel (voxel1) to the earlier one (voxel2)
            const float sg = u < v ? 1.0f : -1.0f;
            const float ox = sg * df_diff(puH.x, puL.x, pvH.x, pvL.x);
            const float oy = sg * df_diff(puH.y, puL.y, pvH.y, pvL.y);
            const float oz = sg * df_diff(puH.z, puL.z, pvH.z, pvL.z);
            const float bu = puH.w;
            const float wd = (bv + bu) * 0.625f;
            // |offset| and its reciprocal from one hardware reciprocal square root (coincident
            // voxels, d2 = 0, give dist = NaN and are skipped; the reference's force is NaN there)
            const float d2 = ox * ox + oy * oy + oz * oz;
            const float inv = rsqrtf(d2);
            const float dist = d2 * inv;
            if (!(dist <= wd)) continue;
            const float rel = wd - dist;
            if (!(rel > 0)) continue;
            const float4 wu = R[2 * d.nv + u];
            const float pstiff = __fdividef(2.0f * pvL.w * puL.w, pvL.w + puL.w);  // 2 / (1/a + 1/b)
            const float dampC = 0.5f * (wv.w + wu.w);
            const float ux = ox * inv, uy = oy * inv, uz = oz * inv;
            const float w1x = wv.x, w1y = wv.y, w1z = wv.z;
            const float w2x = wu.x, w2y = wu.y, w2z = wu.z;
            // voxel1 = the later one: rv = w1.u - w2.u with (1, 2) = (v, u) when u < v, else (u, v)
            const float rv = sg * ((w1x * ux + w1y * uy + w1z * uz) - (w2x * ux + w2y * uy + w2z * uz));
            const float f = pstiff * rel + dampC * rv;
            // v.contactForce += force (v is voxel1) or -= force (v is voxel2); force along u
            if (ATTACH && att && linked_to(d, v, u)) {  // (acc + c) - c
                const float cx = sg * ux * f, cy = sg * uy * f, cz = sg * uz * f;
                acc.x = (acc.x + cx) - cx;
                acc.y = (acc.y + cy) - cy;
                acc.z = (acc.z + cz) - cz;
                continue;
            }
            acc.x += sg * ux * f;
            acc.y += sg * uy * f;
            acc.z += sg * uz * f;
        }
    }
    reinterpret_cast<float4 *>(d.contact)[v] = make_float4(acc.x, acc.y, acc.z, 0.0f);
}

void launch_coll_eval_mixed(const Dev &d, cudaStream_t s) {
    if (!d.ns) return;
    if (d.narob) k_coll_eval_mixed<true><<<(d.ns + 255) / 256, 256, 0, s>>>(d);
    else k_coll_eval_mixed<false><<<(d.ns + 255) / 256, 256, 0, s>>>(d);
}

// ------------------------------------------------------------- programmatic dependent launch
// The link and voxel kernels are launched with programmatic stream serialization:
// a kernel may start while the previous one finishes.  Each first issues the loads
// that do not depend on the previous kernel, then waits for it to complete
// (griddepcontrol.wait: a no-op when launched without the attribute), and only then
// lets the next kernel launch, so a kernel never starts before the one two places
// earlier has finished.  Every store comes after the wait.
__device__ __forceinline__ void pdl_wait_then_release() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ------------------------------------------------------------- link pass
__device__ __forceinline__ void links_mixed_body(const Dev &d, int l) {
    // every load that depends only on l is issued before the first branch, then the
    // endpoint state: two dependent load levels instead of four (latency-bound kernel)
    const uint2 li = d.linfo[l];
    const int2 e = d.ends[l];
    // link state (mixed precision): a 16-byte row {pos2, angle2v.x} and an 8-byte row
    // {angle2v.y, angle2v.z} per link, then angle1v component-major (mixed_lstate_*)
    float4 *lsA = mixed_lstate_a(d);
    float2 *lsB = mixed_lstate_b(d);
    float *lsC = mixed_lstate_c(d);
    const size_t NL = (size_t)d.nl;
    const float4 sa = lsA[l];
    const float2 sb = lsB[l];
    const V3<float> oldPos2{sa.x, sa.y, sa.z};
    // angle1v is zero while a link is in the small-angle branch (the flag it entered
    // this step with says so); it is read and written only for large-angle links and
    // zeroed once when a link returns to the small branch
    const bool wasSmall = (li.y & LF_SMALL) != 0;
    V3<float> oldA1{0, 0, 0};
    if (!wasSmall) oldA1 = V3<float>{lsC[l], lsC[NL + l], lsC[2 * NL + l]};
    const V3<float> oldA2{sa.w, sb.x, sb.y};
    float2 sm = d.strain[l];
    pdl_wait_then_release();  // the previous voxel pass has moved the endpoints
    const float4 *P = reinterpret_cast<const float4 *>(d.pos);
    const float4 *Q = reinterpret_cast<const float4 *>(d.quat);
    const float4 pnH = P[2 * e.x], pnL = P[2 * e.x + 1], ppH = P[2 * e.y], ppL = P[2 * e.y + 1];
    const float4 qnH = Q[2 * e.x], qnL = Q[2 * e.x + 1], qpH = Q[2 * e.y], qpL = Q[2 * e.y + 1];
    const int r = (int)li.x;
    if (d.status[r] != 0) return;
    const uint32_t fl = li.y;
    if (fl & (LF_BOTH_FIXED | LF_GONE)) return;
    const int axis = fl & LF_AXIS;
    const LMat &m = d.lmat[fl >> 8];

    // rest length L = 0.5*(bsNeg + bsPos) as a hi/lo pair (VX3_Link::updateRestLength)
    float Lh, Ll;
    two_sum(pnH.w, ppH.w, Lh, Ll);
    Ll += pnL.w + ppL.w;
    quick_two_sum(0.5f * Lh, 0.5f * Ll, Lh, Ll);
    // delta = (pPos - pNeg) - L*e_axis in the global frame
    const float ax = axis == 0 ? Lh : 0.0f, ay = axis == 1 ? Lh : 0.0f, az = axis == 2 ? Lh : 0.0f;
    const float axl = axis == 0 ? Ll : 0.0f, ayl = axis == 1 ? Ll : 0.0f, azl = axis == 2 ? Ll : 0.0f;
    const V3<float> delta{df_diff3(ppH.x, ppL.x, pnH.x, pnL.x, ax, axl), df_diff3(ppH.y, ppL.y, pnH.y, pnL.y, ay, ayl),
                          df_diff3(ppH.z, ppL.z, pnH.z, pnL.z, az, azl)};
    const Q4<float> a1 = to_axis_xq(axis, Q4<float>{qnH.x, qnH.y, qnH.z, qnH.w});
    const Q4<float> dq = to_axis_xq(axis, Q4<float>{df_diff(qpH.x, qpL.x, qnH.x, qnL.x), df_diff(qpH.y, qpL.y, qnH.y, qnL.y),
                                                   df_diff(qpH.z, qpL.z, qnH.z, qnL.z), df_diff(qpH.w, qpL.w, qnH.w, qnL.w)});
    const Q4<float> c = qconj(a1);
    const Q4<float> cd = qmul(c, dq);  // angle2 = conj(q1)*q2 = |q1|^2 + conj(q1)*(q2-q1), |q1| = 1
    const V3<float> rd = qrot(c, to_axis_x(axis, delta));
    const float L = Lh;
    float pxm = -2.0f * L * (a1.y * a1.y + a1.z * a1.z) + rd.x;  // pos2.x - L
    float py = 2.0f * L * (a1.x * a1.y - a1.w * a1.z) + rd.y;
    float pz = 2.0f * L * (a1.x * a1.z + a1.w * a1.y) + rd.z;
    const float px = L + pxm;
    // hysteresis on SmallTurn = (|pz| + |py|)/px and ExtendPerc = |pxm/L| (L > 0),
    // compared without dividing: px < 0 (bent past 90 degrees) gives SmallTurn <= 0,
    // px = 0 gives +inf (or NaN when the numerator is 0 too)
    const float HF = 1.2f, BEND = 0.05f, EXT = 0.50f;
    const float turn = fabsf(pz) + fabsf(py), ext = fabsf(pxm);
    const bool turnBelow = px > 0.0f ? turn < BEND * px : px < 0.0f;
    const bool turnAbove = px > 0.0f ? turn > (HF * BEND) * px : (px == 0.0f && turn > 0.0f);
    bool small = (fl & LF_SMALL) != 0, lvv = (fl & LF_LVV) != 0;
    if (!small && turnBelow && ext < EXT * L) {
        small = true;
        lvv = false;
    } else if (small && (turnAbove || ext > (HF * EXT) * L)) {
        small = false;
        lvv = false;
    }
    Q4<float> angle1{1, 0, 0, 0};
    float w2 = 1.0f + cd.w;
    V3<float> v2{cd.x, cd.y, cd.z};
    V3<float> pos2;
    if (small) {
        pos2 = V3<float>{pxm, py, pz};
    } else {
        angle1 = from_angle_to_posx_f(angle1, V3<float>{px, py, pz});
        const Q4<float> a2 = qmul(angle1, Q4<float>{w2, v2.x, v2.y, v2.z});
        w2 = a2.w;
        v2 = V3<float>{a2.x, a2.y, a2.z};
        const float l2 = px * px + py * py + pz * pz;
        const float len2 = l2 > 0.0f ? l2 * rsqrtf(l2) : 0.0f;
        pos2 = V3<float>{__fdividef(pxm * (px + L) + py * py + pz * pz, len2 + L), 0, 0};  // |pos2| - L
    }
    const V3<float> a1v = small ? V3<float>{0, 0, 0} : rotvec_f(angle1.w, V3<float>{angle1.x, angle1.y, angle1.z});
    const V3<float> a2v = rotvec_f(w2, v2);
    lsA[l] = make_float4(pos2.x, pos2.y, pos2.z, a2v.x);
    lsB[l] = make_float2(a2v.y, a2v.z);
    if (!(small && wasSmall)) {
        lsC[l] = a1v.x; lsC[NL + l] = a1v.y; lsC[2 * NL + l] = a1v.z;
    }

    const V3<float> dPos2 = scl(sub(pos2, oldPos2), 0.5f);
    const V3<float> dA1 = scl(sub(a1v, oldA1), 0.5f);
    const V3<float> dA2 = scl(sub(a2v, oldA2), 0.5f);
    // FP32 quotients in the hot paths use the hardware reciprocal (__fdividef: within 2 ulp, one
    // fixed instruction pair, so every launch shape computes the same value)
    const float axialStrain = __fdividef(pos2.x, L);
    sm.x = axialStrain;
    const float stress = link_stress(d, m, l, axialStrain, &sm.y);  // updateStrain (VX3_Link.cu:220-260)
    d.strain[l] = sm;
    if (axialStrain > 100) atomicOr(&d.status[r], 1);

    uint32_t nfl = (fl & ~(LF_SMALL | LF_LVV)) | (small ? LF_SMALL : 0u);
    if (m.eps_fail != -1.0f && sm.y > m.eps_fail) {
        const V3<float> z{0, 0, 0};
        store_slot_mx(d, 2 * axis, e.x, z, z);
        store_slot_mx(d, 2 * axis + 1, e.y, z, z);
        nfl |= lvv ? LF_LVV : 0u;
        if (nfl != fl) d.linfo[l].y = nfl;
        return;
    }
    const float b1 = m.b1, b2 = m.b2, b3 = m.b3, a2 = m.a2;
    V3<float> fNeg{stress * m.area, b1 * pos2.y - b2 * (a1v.z + a2v.z), b1 * pos2.z + b2 * (a1v.y + a2v.y)};
    V3<float> fPos = neg(fNeg);
    V3<float> mNeg{a2 * (a2v.x - a1v.x), -b2 * pos2.z - b3 * (2 * a1v.y + a2v.y), b2 * pos2.y - b3 * (2 * a1v.z + a2v.z)};
    V3<float> mPos{a2 * (a1v.x - a2v.x), -b2 * pos2.z - b3 * (a1v.y + 2 * a2v.y), b2 * pos2.y - b3 * (a1v.z + 2 * a2v.z)};
    if (lvv) {
        const V3<float> posCalc{m.sqA1 * dPos2.x, m.sqB1 * dPos2.y - m.sqB2xFMp * (dA1.z + dA2.z),
                                m.sqB1 * dPos2.z + m.sqB2xFMp * (dA1.y + dA2.y)};
        // dampingMultiplier / dt, infinite for a Fixed end (its numerator over a zero time step)
        const float idt = __fdividef(1.0f, d.dt[r]);
        const float dmN = m.dmcN * (m.fixN ? CUDART_INF_F : idt);
        const float dmP = m.dmcP * (m.fixP ? CUDART_INF_F : idt);
        fNeg = add(fNeg, scl(posCalc, dmN));
        fPos = sub(fPos, scl(posCalc, dmP));
        mNeg = sub(mNeg, scl(V3<float>{-m.sqA2xIp * (dA2.x - dA1.x), m.sqB2xFMp * dPos2.z + m.sqB3xIp * (2 * dA1.y + dA2.y),
                                       -m.sqB2xFMp * dPos2.y + m.sqB3xIp * (2 * dA1.z + dA2.z)},
                             0.5f * dmN));
        mPos = sub(mPos, scl(V3<float>{m.sqA2xIp * (dA2.x - dA1.x), m.sqB2xFMp * dPos2.z + m.sqB3xIp * (dA1.y + 2 * dA2.y),
                                       -m.sqB2xFMp * dPos2.y + m.sqB3xIp * (dA1.z + 2 * dA2.z)},
                             0.5f * dmP));
    } else {
        lvv = true;
    }
    nfl |= lvv ? LF_LVV : 0u;
    if (!small) {
        fNeg = qrotinv(angle1, fNeg);
        mNeg = qrotinv(angle1, mNeg);
    }
    const Q4<float> angle2{w2, v2.x, v2.y, v2.z};
    fPos = qrotinv(angle2, fPos);
    mPos = qrotinv(angle2, mPos);
    store_slot_mx(d, 2 * axis, e.x, to_axis_original(axis, fNeg), to_axis_original(axis, mNeg));
    store_slot_mx(d, 2 * axis + 1, e.y, to_axis_original(axis, fPos), to_axis_original(axis, mPos));
    if (fl & LF_RUNTIME) new_link_scale_mx(d, l, 2 * axis, e.x, e.y);
    if (nfl != fl) d.linfo[l].y = nfl;
}

// base size nomSize*(1 + T*cte) as a hi/lo pair
__device__ __forceinline__ void base_size_df(const VMat &m, float te, float &hi, float &lo) {
    const float f = 1 + te * m.cte;
    const float p = m.nom_hi * f;
    const float err = fmaf(m.nom_hi, f, -p) + m.nom_lo * f;
    quick_two_sum(p, err, hi, lo);
}

// temperature at the end of a step (gpu_update_temperature, VX3_VoxelyzeKernel.cu:625-650)
// from the cycles of the phase 2*3.1415926f*(t/P + phase) / (2 pi): the robot's cycles at
// the step's start tc and the voxel's phase cycles ph, each frac(.) reduced in FP64 once
// (by the writer of the robot's time, and at create) and held as FP32 hi + lo pairs, plus
// the step's dt * cycles per second (about 5e-4 cycles, rounded to 3e-11).  The sum c_hi +
// c_lo is formed with two-sums, and sin(2 pi c) = sin(2 pi c_hi) + 2 pi c_lo cos(2 pi c_hi),
// the second term dropping (2 pi c_lo)^2 / 2 < 1e-13.  The FP32 sine of a rounded c alone
// would carry up to 3.7e-7 rad of phase; with the correction the temperature is within
// about one FP32 rounding of the FP64 step's, and no FP64 arithmetic runs per voxel.
__device__ __forceinline__ float temperature_mx(const RobotP &rp, float2 tc, float2 ph, float dtf) {
    float s, e;
    two_sum(tc.x, ph.x, s, e);
    s -= floorf(s);  // exact: s lies in [0, 2]
    e += (tc.y + ph.y) + dtf * rp.cyc_rate;
    float ch, cl;
    two_sum(s, e, ch, cl);
    float sn, cs;
    sincospif(2.0f * ch, &sn, &cs);
    float T = rp.amp_f * fmaf(6.28318531f * cl, cs, sn);
    if (!rp.expansion && T > 0) T = 0;
    return T;
}

// frac(c) as an FP32 hi + lo pair
__device__ __forceinline__ float2 cycles_df(double c) {
    c -= floor(c);
    const float h = (float)c;
    return make_float2(h, (float)(c - (double)h));
}

// The FP64 arithmetic of the mixed voxel pass, kept out of line: if-converted into the
// pass, it would issue in every warp (GB300 runs FP64 at about 1/64 of the FP32 rate).
// The robot's time and actuation cycles of the next step (one thread per robot):
__device__ __noinline__ void advance_time(const Dev &d, const RobotP &rp, int r, int parity, float dtf, int st) {
    const double Tcur = d.T[(size_t)parity * d.nr + r];
    const double Tn = (st == 0) ? Tcur + dtf : Tcur;
    d.T[(size_t)(parity ^ 1) * d.nr + r] = Tn;
    d.tcyc[(size_t)(parity ^ 1) * d.nr + r] = cycles_df(Tn * rp.inv_period * kCycle);
}
// a material with TurnOnThermalExpansionAfterThisManySeconds > 0: is expansion on at the
// end of this step?
__device__ __noinline__ bool thermal_on(const Dev &d, double toa, int r, int parity, float dtf) {
    return !(toa > d.T[(size_t)parity * d.nr + r] + dtf);
}

__global__ void k_init_temperature_mixed(Dev d) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d.nv) return;
    const uint2 vi = d.vinfo[v];
    const VMat m = d.vmat[vi.y >> 8];
    const RobotP &rp = d.rp[vi.x];
    float te = d.tempe[v];
    if (rp.vary_temp && rp.temp_period > 0 && !(m.thermal_on_after > 0.0) && !m.fixed)
        te = temperature_mx(rp, make_float2(0.0f, 0.0f), d.phc[v], 0.0f);
    float4 *P = reinterpret_cast<float4 *>(d.pos);
    base_size_df(m, te, P[2 * v].w, P[2 * v + 1].w);
    d.tempe[v] = te;
    d.tempe[d.nv + v] = te;
}

// ------------------------------------------------------------ voxel pass
// a double as an FP32 hi/lo pair
__device__ __forceinline__ void set_df(float &hi, float &lo, double x) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// BC = false: every voxel without a boundary-condition external (the main pass, which
// compiles without the external code).  BC = true: the voxels with one (Dev::xbc), after
// the main pass, with the external force and moment, the fixed DOFs and the fixed-all
// pose (VX3_Voxel.cu:167-173, 222-257, 363-364, 393-394).
template <bool BC> __device__ __forceinline__ void voxels_mixed_body(const Dev &d, int v, int parity) {
    // the voxel's own state is loaded together with its info word, before any branch
    // (latency-bound kernel: one dependent level fewer)
    const uint2 vi = d.vinfo[v];
    float4 *P = reinterpret_cast<float4 *>(d.pos);
    float4 *Qa = reinterpret_cast<float4 *>(d.quat);
    float4 *LM = reinterpret_cast<float4 *>(d.linmom);
    float4 *AM = reinterpret_cast<float4 *>(d.angmom);
    float4 pH = P[2 * v], pL = P[2 * v + 1];
    float4 qH = Qa[2 * v], qL = Qa[2 * v + 1];
    float4 lH = LM[2 * v], lL = LM[2 * v + 1];
    float4 aH = AM[2 * v], aL = AM[2 * v + 1];
    pdl_wait_then_release();  // the link pass (or the contact evaluation) of this step is done
    const int r = (int)vi.x;
    const RobotP &rp = d.rp[r];
    const int st = d.status[r];
    const float dtf = d.dt[r];
    if (!BC && v == rp.voff) advance_time(d, rp, r, parity, dtf, st);
    if (st != 0) return;
    uint32_t fl = vi.y;
    if (fl & VF_FIXED) return;
    if (!BC && rp.bcs && d.vext[v] >= 0) return;  // stepped by the BC pass
    const VMat m = d.vmat[fl >> 8];
    const bool actuated = rp.vary_temp && rp.temp_period > 0;
    float *tcur = d.tempe + (size_t)parity * d.nv, *tnext = d.tempe + (size_t)(parity ^ 1) * d.nv;
    const int xi = BC ? d.vext[v] : -1;  // boundary-condition external
    const int dof = BC ? d.ext[xi].dof : 0;
    if (BC && dtf != 0.0f && dof == EXT_ALL) {  // isFixedAll (VX3_Voxel.cu:167-173)
        const ExtBC &e = d.ext[xi];
        const short4 l = d.ijk[v];
        set_df(pH.x, pL.x, l.x * m.nom_size + e.t.x);
        set_df(pH.y, pL.y, l.y * m.nom_size + e.t.y);
        set_df(pH.z, pL.z, l.z * m.nom_size + e.t.z);
        set_df(qH.x, qL.x, e.q.x);
        set_df(qH.y, qL.y, e.q.y);
        set_df(qH.z, qL.z, e.q.z);
        set_df(qH.w, qL.w, e.q.w);
        Qa[2 * v] = qH;
        Qa[2 * v + 1] = qL;
        const float4 z4 = make_float4(0, 0, 0, 0);
        LM[2 * v] = z4;
        LM[2 * v + 1] = z4;
        AM[2 * v] = z4;
        AM[2 * v + 1] = z4;
    } else if (dtf != 0.0f) {
        V3<float> Fs{0, 0, 0}, Ms{0, 0, 0};
#pragma unroll
        for (int dir = 0; dir < 6; dir++) {
            if (fl & (1u << dir)) {
                V3<float> sf, sm;
                load_slot_mx(d, dir, v, &sf, &sm);
                Fs = add(Fs, sf);
                Ms = add(Ms, sm);
            }
        }
        bool stat = (fl & VF_STATIC) != 0;
        const bool floorOn = rp.floor != 0;
        const Q4<float> o{qH.x, qH.y, qH.z, qH.w};
        V3<float> F = qrot(o, Fs);
        if (BC) F = add(F, V3<float>{d.ext[xi].f[0], d.ext[xi].f[1], d.ext[xi].f[2]});  // external force
        const V3<float> vel{(lH.x + lL.x) * m.mass_inv, (lH.y + lL.y) * m.mass_inv, (lH.z + lL.z) * m.mass_inv};
        F = sub(F, scl(vel, m.c_glob));
        F.z += m.grav_force;
        if (rp.collision) {
            const float4 c = reinterpret_cast<const float4 *>(d.contact)[v];
            F = sub(F, V3<float>{c.x, c.y, c.z});
        }
        if (rp.cilia) {  // CiliaForce * Cilia (VX3_Voxel.cu:376), evaluated in FP64 by k_extra_forces
            const double4 c = d.cfv[v];
            F = add(F, V3<float>{(float)c.x, (float)c.y, (float)c.z});
        }
        if (rp.ff_any) {  // force field (VX3_Voxel.cu:178-184), evaluated in FP64 by k_extra_forces
            const double4 ff = d.ffv[v];
            F = add(F, V3<float>{(float)ff.x, (float)ff.y, (float)ff.z});
        }
        // floor penetration bsa/2 - nom/2 - z with bsa = base size (VX3_Voxel.h:185-188)
        const float pen = 0.5f * ((pH.w - m.nom_hi) + (pL.w - m.nom_lo)) - (pH.z + pL.z);
        V3<float> fric = F;
        if (floorOn) {
            if (pen >= 0) {
                const float normal = m.pstiff * pen;
                F.z += normal - m.c_col * vel.z;
                if (stat) {
                    if (F.x * F.x + F.y * F.y > (m.mu_s * normal) * (m.mu_s * normal)) stat = false;
                } else {
                    // the horizontal velocity's direction (normalized(): unchanged when zero)
                    const float h2 = vel.x * vel.x + vel.y * vel.y;
                    const float k = h2 > 0.0f ? rsqrtf(h2) : 1.0f;
                    F = sub(F, scl(V3<float>{vel.x * k, vel.y * k, 0}, m.mu_k * normal));
                }
            } else {
                stat = false;
            }
        }
        fric = sub(F, fric);
        df_add(lH.x, lL.x, F.x * dtf);
        df_add(lH.y, lL.y, F.y * dtf);
        df_add(lH.z, lL.z, F.z * dtf);
        const float km = dtf * m.mass_inv;
        V3<float> tr{(lH.x + lL.x) * km, (lH.y + lL.y) * km, (lH.z + lL.z) * km};
        if (floorOn && pen >= 0) {
            const float lx = lH.x + lL.x, ly = lH.y + lL.y;
            const float work = fric.x * tr.x + fric.y * tr.y;
            const float hKe = 0.5f * m.mass_inv * (lx * lx + ly * ly);
            if (hKe + work <= 0) stat = true;
            if (stat) {
                lH.x = lL.x = lH.y = lL.y = 0;
                tr.x = tr.y = 0;
            }
        } else {
            stat = false;
        }
        df_add(pH.x, pL.x, tr.x);
        df_add(pH.y, pL.y, tr.y);
        df_add(pH.z, pL.z, tr.z);
        V3<float> M = qrot(o, Ms);
        if (BC) M = add(M, V3<float>{d.ext[xi].m[0], d.ext[xi].m[1], d.ext[xi].m[2]});  // external moment
        const V3<float> avel{(aH.x + aL.x) * m.mom_inv, (aH.y + aL.y) * m.mom_inv, (aH.z + aL.z) * m.mom_inv};
        M = sub(M, scl(avel, m.c_glob_rot));
        df_add(aH.x, aL.x, M.x * dtf);
        df_add(aH.y, aL.y, M.y * dtf);
        df_add(aH.z, aL.z, M.z * dtf);
        // q' = Quat(angMom*dt/I)*q = q + (dq - 1)*q (FromRotationVector, VX3_Quat3D.h:363-377)
        const float ki = dtf * m.mom_inv;
        const V3<float> th{0.5f * (aH.x + aL.x) * ki, 0.5f * (aH.y + aL.y) * ki, 0.5f * (aH.z + aL.z) * ki};
        const float m2 = th.x * th.x + th.y * th.y + th.z * th.z;
        float dw, sfac;
        if (m2 * m2 < 5.328e-15f) {
            dw = -0.5f * m2;
            sfac = 1.0f - m2 * (1.0f / 6.0f);
        } else if (m2 < 0.25f) {
            // |theta| < 0.5 rad: cos|theta| - 1 and sin|theta| / |theta| as their Taylor series in
            // m2 = |theta|^2, truncated where the next term is below 3e-10 (no square root,
            // sine or division; the same values to FP32 rounding)
            dw = m2 * (-0.5f + m2 * (1.0f / 24 + m2 * (-1.0f / 720 + m2 * (1.0f / 40320 - m2 * (1.0f / 3628800)))));
            sfac = 1.0f + m2 * (-1.0f / 6 + m2 * (1.0f / 120 + m2 * (-1.0f / 5040 + m2 * (1.0f / 362880))));
        } else {
            const float im = rsqrtf(m2);  // 1 / |theta|, m2 >= 0.25 here
            float sn, cs;
            sincospif(m2 * im * 0.159154943f, &sn, &cs);  // sin, cos of |theta| / 2
            dw = -2.0f * sn * sn;
            sfac = 2.0f * sn * cs * im;
        }
        const Q4<float> delta = qmul(Q4<float>{dw, th.x * sfac, th.y * sfac, th.z * sfac}, o);
        df_add(qH.x, qL.x, delta.w);
        df_add(qH.y, qL.y, delta.x);
        df_add(qH.z, qL.z, delta.y);
        df_add(qH.w, qL.w, delta.z);
        if (BC && dof) {  // fixed DOFs (VX3_Voxel.cu:222-257), in FP64 on the hi/lo pairs
            const ExtBC &e = d.ext[xi];
            if (dof & EXT_T) {
                const short4 l = d.ijk[v];
                if (dof & 1) { set_df(pH.x, pL.x, l.x * m.nom_size + e.t.x); lH.x = lL.x = 0; }
                if (dof & 2) { set_df(pH.y, pL.y, l.y * m.nom_size + e.t.y); lH.y = lL.y = 0; }
                if (dof & 4) { set_df(pH.z, pL.z, l.z * m.nom_size + e.t.z); lH.z = lL.z = 0; }
            }
            if ((dof & EXT_R) == EXT_R) {  // all rotations: the prescribed orientation
                set_df(qH.x, qL.x, e.q.x);
                set_df(qH.y, qL.y, e.q.y);
                set_df(qH.z, qL.z, e.q.z);
                set_df(qH.w, qL.w, e.q.w);
                aH.x = aH.y = aH.z = aL.x = aL.y = aL.z = 0;
            } else if (dof & EXT_R) {  // some: those rotation-vector components zeroed
                V3<double> rv = to_rotvec(Q4<double>{(double)qH.x + qL.x, (double)qH.y + qL.y, (double)qH.z + qL.z,
                                                     (double)qH.w + qL.w});
                if (dof & 8) { rv.x = 0; aH.x = aL.x = 0; }
                if (dof & 16) { rv.y = 0; aH.y = aL.y = 0; }
                if (dof & 32) { rv.z = 0; aH.z = aL.z = 0; }
                const Q4<double> q = from_rotvec(rv);
                set_df(qH.x, qL.x, q.w);
                set_df(qH.y, qL.y, q.x);
                set_df(qH.z, qL.z, q.y);
                set_df(qH.w, qL.w, q.z);
            }
        }
        const float pen2 = 0.5f * ((pH.w - m.nom_hi) + (pL.w - m.nom_lo)) - (pH.z + pL.z);
        if (floorOn && pen2 >= 0 && stat) aH.x = aH.y = aH.z = aL.x = aL.y = aL.z = 0;
        const uint32_t nfl = stat ? (fl | VF_STATIC) : (fl & ~VF_STATIC);
        if (nfl != fl) d.vinfo[v].y = nfl;
        Qa[2 * v] = qH;
        Qa[2 * v + 1] = qL;
        LM[2 * v] = lH;
        LM[2 * v + 1] = lL;
        AM[2 * v] = aH;
        AM[2 * v + 1] = aL;
    }
    if (actuated) {  // next step's temperature and base size
        float te = tcur[v];
        if (!m.toa_pos || thermal_on(d, m.thermal_on_after, r, parity, dtf))
            te = temperature_mx(rp, d.tcyc[(size_t)parity * d.nr + r], d.phc[v], dtf);
        base_size_df(m, te, pH.w, pL.w);
        tnext[v] = te;
    }
    P[2 * v] = pH;
    P[2 * v + 1] = pL;
}

// the voxels with a boundary-condition external, after the main voxel pass
__global__ void __launch_bounds__(128) k_voxels_bc_mixed(Dev d, int parity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.nxbc) voxels_mixed_body<true>(d, d.xbc[i], parity);
}

void launch_voxels_bc_mixed(const Dev &d, int parity, cudaStream_t s) {
    if (d.nxbc) k_voxels_bc_mixed<<<(d.nxbc + 127) / 128, 128, 0, s>>>(d, parity);
}

// Launch-shape variants (threads per block, minimum resident blocks): the same body,
// so every variant computes bit-identical results; they trade registers for
// occupancy (both passes are latency-bound gathers).  vx3g_autotune picks one per
// context by timing real steps.
template <int TPB, int MINB> __global__ void __launch_bounds__(TPB, MINB) k_links_mixed(Dev d) {
    const int l = blockIdx.x * TPB + threadIdx.x;
    if (l < d.nl) links_mixed_body(d, l);
}
template <int TPB, int MINB> __global__ void __launch_bounds__(TPB, MINB) k_voxels_mixed(Dev d, int parity) {
    const int v = blockIdx.x * TPB + threadIdx.x;
    if (v < d.nv) voxels_mixed_body<false>(d, v, parity);
}

const LaunchShape kLinkShapes[kMixedShapes] = {{256, 1}, {256, 4}, {128, 9}, {128, 10}, {64, 20}, {256, 5}};
const LaunchShape kVoxelShapes[kMixedShapes] = {{256, 1}, {256, 3}, {128, 7}, {128, 8}, {64, 14}, {64, 16}};

// launch with programmatic stream serialization (see pdl_wait_then_release)
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), int n, int threads, cudaStream_t s, bool pdl, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((n + threads - 1) / threads));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

void launch_links_mixed(const Dev &d, cudaStream_t s, int shape, bool pdl) {
    if (!d.nl) return;
    switch (shape) {
        case 1: launch_pdl(k_links_mixed<256, 4>, d.nl, 256, s, pdl, d); break;
        case 2: launch_pdl(k_links_mixed<128, 9>, d.nl, 128, s, pdl, d); break;
        case 3: launch_pdl(k_links_mixed<128, 10>, d.nl, 128, s, pdl, d); break;
        case 4: launch_pdl(k_links_mixed<64, 20>, d.nl, 64, s, pdl, d); break;
        case 5: launch_pdl(k_links_mixed<256, 5>, d.nl, 256, s, pdl, d); break;
        default: launch_pdl(k_links_mixed<256, 1>, d.nl, 256, s, pdl, d); break;
    }
}
void launch_voxels_mixed(const Dev &d, int parity, cudaStream_t s, int shape, bool pdl) {
    if (!d.nv) return;
    switch (shape) {
        case 1: launch_pdl(k_voxels_mixed<256, 3>, d.nv, 256, s, pdl, d, parity); break;
        case 2: launch_pdl(k_voxels_mixed<128, 7>, d.nv, 128, s, pdl, d, parity); break;
        case 3: launch_pdl(k_voxels_mixed<128, 8>, d.nv, 128, s, pdl, d, parity); break;
        case 4: launch_pdl(k_voxels_mixed<64, 14>, d.nv, 64, s, pdl, d, parity); break;
        case 5: launch_pdl(k_voxels_mixed<64, 16>, d.nv, 64, s, pdl, d, parity); break;
        default: launch_pdl(k_voxels_mixed<256, 1>, d.nv, 256, s, pdl, d, parity); break;
    }
}
void launch_init_temperature_mixed(const Dev &d, cudaStream_t s) {
    if (d.nv) k_init_temperature_mixed<<<(d.nv + 255) / 256, 256, 0, s>>>(d);
}

}  // namespace vx3g
