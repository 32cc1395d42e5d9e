// vx3g_bc.h -- boundary-condition regions to per-voxel externals (host side).
//
// CVX_Sim::Import (src/VXA/VX_Sim.cpp:109-141) gives every voxel that a region of
// <Boundary_Conditions> touches an external (CVX_External, src/old/VX_External.cpp):
// each fixed DOF of the region is fixed with the region's displacement (a zero
// displacement leaves an earlier region's value), and the region's force and torque,
// divided by the number of voxels it touches, are added -- in the reference's own
// form, extForce += (float)(extForce + Force/Size), which doubles what earlier regions
// added.  The touching tests are CP_Box/CP_Cylinder/CP_Sphere::IsTouching
// (src/old/VX_FRegion.cpp:395-605) in the reference's arithmetic: region coordinates are
// floats, positions and the workspace doubles.  Two different voxel positions enter,
// as in the reference: the count of touched voxels uses CVX_Object::GetXYZ (cell
// centres shifted by 1e-6 lattice units in x and y, src/VXA/VX_Object.cpp:525-558),
// the assignment uses the voxel's position plus half a cell.
#pragma once

#include <cmath>
#include <vector>

#include "../../include/vx3g.h"

namespace vx3g {

struct VoxelExt {
    bool any = false;       // the voxel has an external (touched by some region)
    int dof = 0;            // fixed DOFs: bits 0-2 translation x, y, z; 3-5 rotation x, y, z
    float f[3] = {0, 0, 0}, m[3] = {0, 0, 0};  // extForce, extMoment
    double t[3] = {0, 0, 0}, r[3] = {0, 0, 0}; // extTranslation, extRotation (rotation vector)
    double q[4] = {1, 0, 0, 0};                 // _extRotationQ (w, x, y, z)
};

// CP_*::IsTouching(P, Dist, Envelope) with the half-cell vector Dist
inline bool bc_touching(const vx3g_bc_region &b, const double P[3], const double D[3], const double W[3]) {
    if (b.prim == 0) {  // box: in workspace fractions
        const double ps[3] = {P[0] / W[0], P[1] / W[1], P[2] / W[2]};
        const double ds[3] = {D[0] / W[0], D[1] / W[1], D[2] / W[2]};
        const float lo[3] = {b.x, b.y, b.z};
        const float hi[3] = {b.x + b.dx, b.y + b.dy, b.z + b.dz};  // float sums, as X+dX in the reference
        for (int k = 0; k < 3; k++)
            if (!(ps[k] + ds[k] > (double)lo[k] && ps[k] - ds[k] < (double)hi[k])) return false;
        return true;
    }
    const double wmax = std::fmax(W[0], std::fmax(W[1], W[2]));
    const double pos[3] = {b.x * W[0], b.y * W[1], b.z * W[2]};
    const double rad = b.radius * wmax;
    if (b.prim == 2) {  // sphere: distance from the centre against radius + |Dist|
        const double dist = std::sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
        const double e0 = P[0] - pos[0], e1 = P[1] - pos[1], e2 = P[2] - pos[2];
        return std::sqrt(e0 * e0 + e1 * e1 + e2 * e2) < rad + dist;
    }
    // cylinder (CP_Cylinder::IsIn): along the first non-zero of dX, dY, dZ
    const double size[3] = {b.dx * W[0], b.dy * W[1], b.dz * W[2]};
    int a;
    if (b.dx != 0) a = 0;
    else if (b.dy != 0) a = 1;
    else if (b.dz != 0) a = 2;
    else return false;
    const int u = a == 0 ? 1 : 0, w = a == 2 ? 1 : 2;
    const double e0 = P[u] - pos[u], e1 = P[w] - pos[w];
    return P[a] > pos[a] && P[a] < pos[a] + size[a] && std::sqrt(e0 * e0 + e1 * e1) < rad;
}

// Quat3D(rotation vector): Quat3D::FromRotationVector (src/old/Quat3D.h:128-143)
inline void quat_from_rotvec(const double r[3], double q[4]) {
    const double h[3] = {0.5 * r[0], 0.5 * r[1], 0.5 * r[2]};
    const double m2 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
    double s;
    if (m2 * m2 < 5.328e-15) {  // DBL_EPSILONx24 of the reference
        q[0] = 1.0 - 0.5 * m2;
        s = 1.0 - m2 / 6.0;
    } else {
        const double m = std::sqrt(m2);
        q[0] = std::cos(m);
        s = std::sin(m) / m;
    }
    q[1] = h[0] * s;
    q[2] = h[1] * s;
    q[3] = h[2] * s;
}

// Externals of a robot's voxels (cells: occupied lattice cells in voxel order, with
// their lattice indices), as the reference's Import derives them.
inline std::vector<VoxelExt> bc_externals(const vx3g_robot_desc &R, const std::vector<int> &ix,
                                          const std::vector<int> &iy, const std::vector<int> &iz) {
    const double vs = R.vox_size;
    const double W[3] = {vs * (double)R.nx, vs * (double)R.ny, vs * (double)R.nz};  // GetWorkSpace
    const double half[3] = {0.5 * vs, 0.5 * vs, 0.5 * vs};                          // GetLatDimEnv()/2
    const size_t nv = ix.size();
    std::vector<int> sizes((size_t)R.n_bcs, 0);
    for (int j = 0; j < R.n_bcs; j++)  // CVX_Environment::GetNumTouching: GetXYZ of every occupied cell
        for (size_t v = 0; v < nv; v++) {
            const double P[3] = {vs * ((0.5 + ix[v]) + 1e-6), vs * ((0.5 + iy[v]) + 1e-6), vs * (0.5 + iz[v])};
            if (bc_touching(R.bcs[j], P, half, W)) sizes[j]++;
        }
    std::vector<VoxelExt> out(nv);
    for (size_t v = 0; v < nv; v++) {
        VoxelExt &e = out[v];
        const double P[3] = {ix[v] * vs + half[0], iy[v] * vs + half[1], iz[v] * vs + half[2]};
        for (int j = 0; j < R.n_bcs; j++) {
            const vx3g_bc_region &b = R.bcs[j];
            if (!bc_touching(b, P, half, W)) continue;
            e.any = true;
            for (int k = 0; k < 6; k++) {  // setDisplacement(dof, displacement)
                if (!(b.dof_fixed & (1 << k))) continue;
                e.dof |= 1 << k;
                const double disp = k < 3 ? b.displace[k] : b.ang_displace[k - 3];
                if (disp != 0.0f) (k < 3 ? e.t[k] : e.r[k - 3]) = disp;
            }
            const double inv = 1.0 / (double)sizes[j];  // Vec3D<double> / int
            for (int k = 0; k < 3; k++) {
                const float fa = (float)((double)e.f[k] + inv * b.force[k]);
                const float ma = (float)((double)e.m[k] + inv * b.torque[k]);
                e.f[k] += fa;
                e.m[k] += ma;
            }
        }
        if (e.r[0] != 0.0 || e.r[1] != 0.0 || e.r[2] != 0.0) quat_from_rotvec(e.r, e.q);  // rotationChanged
    }
    return out;
}

}  // namespace vx3g
