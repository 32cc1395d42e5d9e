// vx3g_material.h -- stress-strain models of voxel and link materials (host side).
//
// A model is the piecewise-linear stress-strain curve the reference keeps per
// material: data points (0,0), (strain_1, stress_1), ... in FP32, the initial modulus
// E, the failure stress and strain (-1: none) and whether the model is linear.  The
// constructors follow the reference's setters and their validations:
//   linear (MatModel 0, 1)      CVX_Material::setModelLinear    src/old/VX_Material.cpp:372-400
//   bilinear (MatModel 2)       CVX_Material::setModelBilinear  src/old/VX_Material.cpp:406-446
//   data points (MatModel 3)    CVX_Material::setModel          src/old/VX_Material.cpp:300-366
// A model the reference's setter rejects leaves the material as CVoxelyze::addMaterial
// created it (src/old/Voxelyze.cpp:357-365, src/old/VX_Material.cpp:15-22): linear,
// E = 1e6 Pa, no failure.  The link material of two voxel materials follows
// CVX_MaterialLink::updateAll (src/old/VX_MaterialLink.cpp:47-112): two linear models
// give a linear model of modulus 2*E1*E2/(E1+E2); otherwise the data points of both
// curves are merged and each segment's modulus is the springs-in-series modulus of the
// two materials just below that strain.
#pragma once

#include <cfloat>
#include <vector>

namespace vx3g {

struct MatModel {
    bool linear = true;
    float E = 1e6f;
    float sigma_fail = -1.0f, eps_fail = -1.0f;
    std::vector<float> strain{0.0f, 1.0f}, stress{0.0f, 1e6f};  // the constructor's setModelLinear(1e6)

    // CVX_Material::isFailed
    bool failed(float eps) const { return eps_fail != -1.0f && eps > eps_fail; }
    // CVX_Material::modulus (src/old/VX_Material.cpp:231-243)
    float modulus(float eps) const {
        if (failed(eps)) return 0.0f;
        if (eps <= strain[1] || linear) return E;
        const int n = (int)strain.size();
        for (int i = 2; i < n; i++)
            if (eps <= strain[i] || i == n - 1) return (stress[i] - stress[i - 1]) / (strain[i] - strain[i - 1]);
        return 0.0f;
    }
    // CVX_Material::strain(stress) (src/old/VX_Material.cpp:214-228)
    float strain_of(float sig) const {
        if (sig <= stress[1] || linear) return sig / E;
        const int n = (int)stress.size();
        for (int i = 2; i < n; i++) {
            if (sig <= stress[i] || i == n - 1) {
                const float perc = (sig - stress[i - 1]) / (stress[i] - stress[i - 1]);
                return strain[i - 1] + perc * (strain[i] - strain[i - 1]);
            }
        }
        return 0.0f;
    }
};

// setModelLinear(youngsModulus, failureStress = -1); false where the reference's setter fails
inline bool model_linear(MatModel &m, float E, float fail_stress) {
    if (E <= 0) return false;
    if (fail_stress != -1.0f && fail_stress <= 0) return false;
    const float fs = fail_stress == -1.0f ? 1000000.0f : fail_stress;
    const float fe = fs / E;
    m.strain = {0.0f, fe};
    m.stress = {0.0f, fs};
    m.linear = true;
    m.E = E;
    m.sigma_fail = fail_stress;
    m.eps_fail = fail_stress == -1.0f ? -1.0f : fe;
    return true;
}

// setModelBilinear(youngsModulus, plasticModulus, yieldStress, failureStress)
inline bool model_bilinear(MatModel &m, float E, float Ep, float sy, float fail_stress) {
    if (E <= 0) return false;
    if (Ep <= 0 || Ep >= E) return false;
    if (sy <= 0) return false;
    if (fail_stress != -1.0f && fail_stress <= sy) return false;
    const float ys = sy / E;
    const float fs = fail_stress == -1.0f ? 3 * sy : fail_stress;
    const float tB = sy - Ep * ys;
    const float fe = (fs - tB) / Ep;
    m.strain = {0.0f, ys, fe};
    m.stress = {0.0f, sy, fs};
    m.linear = false;
    m.E = E;
    m.sigma_fail = fail_stress;
    m.eps_fail = fail_stress == -1.0f ? -1.0f : fe;
    return true;
}

// setModel(dataPointCount, strain, stress): a leading (0,0) point is skipped, the rest
// must start positive with strictly increasing strain (the stress-order and slope checks
// of the reference do not reject: the first only records a message, the second compares
// with 0/0)
inline bool model_data(MatModel &m, int n, const float *eps, const float *sig) {
    if (n > 0 && eps[0] == 0 && sig[0] == 0) {
        eps++;
        sig++;
        n--;
    }
    if (n <= 0) return false;
    if (eps[0] <= 0 || sig[0] <= 0) return false;
    std::vector<float> se{0.0f}, ss{0.0f};
    float sweep = 0.0f;
    for (int i = 0; i < n; i++) {
        if (eps[i] <= sweep) return false;
        sweep = eps[i];
        se.push_back(eps[i]);
        ss.push_back(sig[i]);
    }
    m.strain = se;
    m.stress = ss;
    m.E = ss[1] / se[1];
    m.sigma_fail = ss.back();
    m.eps_fail = se.back();
    m.linear = (n == 1);
    return true;
}

// CVX_MaterialLink::updateAll's model for voxel materials m1 (the voxel being added)
// and m2 (its existing neighbour)
inline MatModel model_link(const MatModel &m1, const MatModel &m2) {
    float fail;
    if (m1.sigma_fail == -1.0f) fail = m2.sigma_fail;
    else if (m2.sigma_fail == -1.0f) fail = m1.sigma_fail;
    else fail = m1.sigma_fail < m2.sigma_fail ? m1.sigma_fail : m2.sigma_fail;
    MatModel l;
    if (m1.linear && m2.linear) {
        if (!model_linear(l, 2.0f * m1.E * m2.E / (m1.E + m2.E), fail)) l = MatModel();
        return l;
    }
    std::vector<float> se{0.0f}, ss{0.0f};
    size_t i1 = 1, i2 = 1;
    while (i1 < m1.strain.size() && i2 < m2.strain.size()) {
        float eps = m1.strain[i1];
        if (m2.strain[i2] < eps) eps = m2.strain[i2];
        if (eps == m1.strain[i1]) i1++;
        if (eps == m2.strain[i2]) i2++;
        const float k1 = m1.modulus(eps - FLT_EPSILON), k2 = m2.modulus(eps - FLT_EPSILON);
        const float k = 2.0f * k1 * k2 / (k1 + k2);
        const float last_e = se.back(), last_s = ss.back();
        se.push_back(eps);
        ss.push_back(last_s + k * (eps - last_e));
    }
    if (!model_data(l, (int)se.size(), se.data(), ss.data())) l = MatModel();
    l.sigma_fail = fail;
    l.eps_fail = fail == -1.0f ? -1.0f : l.strain_of(fail);
    return l;
}

}  // namespace vx3g
