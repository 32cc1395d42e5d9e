// Reference-build driver for the oracle (TEST INFRASTRUCTURE ONLY).
//
// This translation unit is compiled together with the reference's own
// sources (src/VX3/VX3_{Link,Voxel,Collision,Material,MaterialVoxel,
// MaterialLink,External}.cu as host C++, plus src/old and src/VXA for the
// VXA import path) by oracle/Makefile into oracle/_ref/libvx3ref.so.  It is
// only used to generate golden fixtures (tests/golden/) and to pin the C
// restatement in oracle/vx3_oracle.c; nothing shipped calls it.
//
// What lives here is the part of the reference that cannot be compiled on
// the host as-is, restated call for call:
//  * VX3_VoxelyzeKernel(CVX_Sim*) host constructor (src/VX3/VX3_VoxelyzeKernel.cu:27-105)
//  * doTimeStep's child-kernel sequence, run as serial loops
//    (src/VX3/VX3_VoxelyzeKernel.cu:237-359, kernels at :566-650, :682-727, :833-843)
//  * recommendedTimeStep (:184-217), regenerateSurfaceVoxels (:495-513),
//    updateCurrentCenterOfMass (:477-493), is_neighbor (:651-680),
//    combinedMaterial (:515-528), the attachment half of handle_collision_attachment
//    (:729-830) and the attach conditions of gpu_update_voxels (:606-621)
//  * the VXA read of src/VX3/VX3_SimulationManager.cu:298-308
// Every physics function called below (VX3_Link::updateForces,
// VX3_Voxel::timeStep, VX3_Collision::updateContactForce, ...) is the
// reference's own code.
//
// Deviations (documented): the reference probes ONE random link per step for
// strain > 100 (VX3_VoxelyzeKernel.cu:271-281); this driver checks every link,
// which is what the GB300 kernels do as well.  The reference runs every surface pair
// of a step at once, so which of two competing attachments wins (and the order of
// contact sums) depends on thread timing; this driver runs the pairs in the serial
// loop's order, first ascending, second ascending below it.  An AttachCondition the
// VXA does not give leaves the reference reading an unset value (VX3_MathTree::eval
// returns values[0] of an empty program); here an absent condition holds.

#include "VX3_VoxelyzeKernel.cuh"
#include "VX3_MemoryCleaner.h"
#include "VX_Sim.h"
#include "XML_Rip.h"

#include <algorithm>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

// globals declared extern by src/old/VX3_MemoryCleaner.h
bool VX3_MemoryCleaner_running = false;
boost::mutex MemoryCleaner_mutex;
std::vector<void *> MemoryCleaner_toBeFreedCUDAPointer;

// d_v_linkMats of each kernel object: the link materials of the lattice, then those
// made at runtime (VX3_VoxelyzeKernel.cuh:91-93)
static std::map<VX3_VoxelyzeKernel *, std::vector<VX3_MaterialLink *>> g_link_mats;

// VX3_VoxelyzeKernel.cu:515-528: the link material of a voxel-material pair, made with the
// reference's device constructor on first use
VX3_MaterialLink *VX3_VoxelyzeKernel::combinedMaterial(VX3_MaterialVoxel *mat1, VX3_MaterialVoxel *mat2) {
    std::vector<VX3_MaterialLink *> &v = g_link_mats[this];
    for (VX3_MaterialLink *m : v)
        if ((m->vox1Mat == mat1 && m->vox2Mat == mat2) || (m->vox1Mat == mat2 && m->vox2Mat == mat1)) return m;
    VX3_MaterialLink *m = new VX3_MaterialLink(mat1, mat2);
    v.push_back(m);
    return m;
}

namespace {

struct RefSim {
    CVX_Environment env;
    CVX_Object obj;
    CVX_Sim sim;
    VX3_VoxelyzeKernel *k = nullptr;
    std::vector<VX3_Voxel *> surface;        // d_surface_voxels
    std::vector<double> last_contact;        // contact force per voxel captured before the voxel pass
    std::vector<VX3_Link *> new_links;       // links made at runtime (the tail of d_v_links), in creation order
    bool cond_set[5] = {false, false, false, false, false};  // AttachCondition/Condition_k given
    float last_dt = 0.0f;
    int steps_done = 0;
    bool diverged = false;
};

// VX3_VoxelyzeKernel.cu:27-105, restated with the public CVoxelyze accessors.
void build_kernel(RefSim &S) {
    CVoxelyze &Vx = S.sim.Vx;
    VX3_VoxelyzeKernel *k = new VX3_VoxelyzeKernel();
    S.k = k;
    k->voxSize = Vx.voxelSize();

    k->num_d_voxelMats = Vx.materialCount();
    VcudaMalloc((void **)&k->d_voxelMats, k->num_d_voxelMats * sizeof(VX3_MaterialVoxel));
    for (int i = 0; i < k->num_d_voxelMats; i++) k->h_voxelMats.push_back((CVX_MaterialVoxel *)Vx.material(i));
    for (int i = 0; i < k->num_d_voxelMats; i++) {
        VX3_MaterialVoxel tmp(k->h_voxelMats[i], k);
        VcudaMemcpy(k->d_voxelMats + i, &tmp, sizeof(VX3_MaterialVoxel), VcudaMemcpyHostToDevice);
    }

    // link materials in order of first use by the link list
    std::vector<CVX_MaterialLink *> lmats;
    for (int i = 0; i < Vx.linkCount(); i++) {
        CVX_MaterialLink *m = Vx.link(i)->mat;
        bool seen = false;
        for (auto *q : lmats) seen |= (q == m);
        if (!seen) lmats.push_back(m);
    }
    k->num_d_linkMats = (int)lmats.size();
    VcudaMalloc((void **)&k->d_linkMats, (k->num_d_linkMats ? k->num_d_linkMats : 1) * sizeof(VX3_MaterialLink));
    for (int i = 0; i < k->num_d_linkMats; i++) {
        VX3_MaterialLink tmp(lmats[i], k);
        VcudaMemcpy(k->d_linkMats + i, &tmp, sizeof(VX3_MaterialLink), VcudaMemcpyHostToDevice);
        k->h_linkMats.push_back(lmats[i]);
    }
    std::vector<VX3_MaterialLink *> &known = g_link_mats[k];
    for (int i = 0; i < k->num_d_linkMats; i++) known.push_back(k->d_linkMats + i);

    k->num_d_voxels = Vx.voxelCount();
    VcudaMalloc((void **)&k->d_voxels, (k->num_d_voxels ? k->num_d_voxels : 1) * sizeof(VX3_Voxel));
    for (int i = 0; i < k->num_d_voxels; i++) {
        k->h_voxels.push_back(Vx.voxel(i));
        k->h_lookup_voxels[Vx.voxel(i)] = k->d_voxels + i;
    }
    k->num_d_links = Vx.linkCount();
    VcudaMalloc((void **)&k->d_links, (k->num_d_links ? k->num_d_links : 1) * sizeof(VX3_Link));
    for (int i = 0; i < k->num_d_links; i++) {
        VX3_Link tmp(Vx.link(i), k);
        memcpy((void *)(k->d_links + i), (void *)&tmp, sizeof(VX3_Link));
        k->h_links.push_back(Vx.link(i));
        k->h_lookup_links[Vx.link(i)] = k->d_links + i;
    }
    for (int i = 0; i < k->num_d_voxels; i++) {
        VX3_Voxel tmp(Vx.voxel(i), k);
        memcpy((void *)(k->d_voxels + i), (void *)&tmp, sizeof(VX3_Voxel));
        tmp.ext = NULL; // ownership moved to the array copy
        // the constructor leaves the pending signal uninitialised (VX3_Voxel.cu:10-14); a
        // voxel starts with none here, as the other signal members start at 0 (VX3_Voxel.h:306-309)
        k->d_voxels[i].d_signal.value = 0.0;
        k->d_voxels[i].d_signal.activeTime = 0.0;
    }
    k->DtFrac = S.sim.DtFrac;
    k->TempEnabled = S.sim.pEnv->IsTempEnabled();
    k->VaryTempEnabled = S.sim.pEnv->IsTempVaryEnabled();
    k->TempBase = S.sim.pEnv->GetTempBase();
    k->TempAmplitude = S.sim.pEnv->GetTempAmplitude();
    k->TempPeriod = S.sim.pEnv->GetTempPeriod();
    k->d_surface_voxels = NULL;

    // CUDA_Simulation prologue (VX3_SimulationManager.cu:20-23): device vectors
    for (int i = 0; i < k->num_d_voxelMats; i++) k->d_voxelMats[i].syncVectors();
    for (int i = 0; i < k->num_d_linkMats; i++) k->d_linkMats[i].syncVectors();
    for (int i = 0; i < k->num_d_voxels; i++) k->d_voxels[i].syncVectors();
    k->currentTime = 0.0;
    k->OptimalDt = 0.0;
    k->CurStepCount = 0;
    k->isSurfaceChanged = true;
}

// VX3_VoxelyzeKernel.cu:184-217
double recommended_dt(VX3_VoxelyzeKernel *k) {
    double MaxFreq2 = 0.0f;
    for (int i = 0; i < k->num_d_links; i++) {
        VX3_Link *pL = k->d_links + i;
        double m1 = pL->pVNeg->mat->mass(), m2 = pL->pVPos->mat->mass();
        double thisMaxFreq2 = pL->axialStiffness() / (m1 < m2 ? m1 : m2);
        if (thisMaxFreq2 > MaxFreq2) MaxFreq2 = thisMaxFreq2;
    }
    if (MaxFreq2 <= 0.0f) {
        for (int i = 0; i < k->num_d_voxels; i++) {
            double thisMaxFreq2 = k->d_voxels[i].mat->youngsModulus() * k->d_voxels[i].mat->nomSize / k->d_voxels[i].mat->mass();
            if (thisMaxFreq2 > MaxFreq2) MaxFreq2 = thisMaxFreq2;
        }
    }
    if (MaxFreq2 <= 0.0f) return 0.0f;
    return 1.0f / (6.283185f * sqrt(MaxFreq2));
}

// VX3_VoxelyzeKernel.cu:495-513
void regenerate_surface(RefSim &S) {
    VX3_VoxelyzeKernel *k = S.k;
    S.surface.clear();
    for (int i = 0; i < k->num_d_voxels; i++) {
        k->d_voxels[i].updateSurface();
        if (k->d_voxels[i].isSurface() && !k->d_voxels[i].removed) S.surface.push_back(&k->d_voxels[i]);
    }
}

// VX3_VoxelyzeKernel.cu:651-680
bool is_neighbor(VX3_Voxel *voxel1, VX3_Voxel *voxel2, VX3_Link *incoming_link, int depth) {
    if (voxel1 == voxel2) return true;
    if (depth <= 0) return false;
    for (int i = 0; i < 6; i++) {
        VX3_Link *L = voxel1->links[i];
        if (L && L != incoming_link) {
            VX3_Voxel *other = (L->pVNeg == voxel1) ? L->pVPos : L->pVNeg;
            if (is_neighbor(other, voxel2, L, depth - 1)) return true;
        }
    }
    return false;
}

// handle_collision_attachment (VX3_VoxelyzeKernel.cu:682-830), collision then attachment
void collide_pair(RefSim &S, VX3_Voxel *voxel1, VX3_Voxel *voxel2, VX3_VoxelyzeKernel *k) {
    if (voxel1->mat->fixed && voxel2->mat->fixed) return;
    VX3_Vec3D<double> diff = voxel1->pos - voxel2->pos;
    double watchDistance = (voxel1->baseSizeAverage() + voxel2->baseSizeAverage()) * COLLISION_ENVELOPE_RADIUS;
    if (diff.x > watchDistance || diff.x < -watchDistance) return;
    if (diff.y > watchDistance || diff.y < -watchDistance) return;
    if (diff.z > watchDistance || diff.z < -watchDistance) return;
    if (diff.Length() > watchDistance) return;
    if (is_neighbor(voxel1, voxel2, NULL, 1)) return;
    VX3_Vec3D<> c1, c2;
    if (k->EnableCollision) {
        VX3_Collision collision(voxel1, voxel2);
        collision.updateContactForce();
        c1 = collision.contactForce(voxel1);
        c2 = collision.contactForce(voxel2);
        voxel1->contactForce += c1;
        voxel2->contactForce += c2;
    }
    if (!k->enableAttach) return;
    // the attachment half (:729-830)
    if (!voxel1->enableAttach || !voxel2->enableAttach) return;
    if (voxel1->mat->fixed || voxel2->mat->fixed) return;
    if (voxel1->mat != voxel2->mat) return;
    if (!voxel1->mat->sticky) return;
    if (is_neighbor(voxel1, voxel2, NULL, 5)) return;
    linkDirection dir1, dir2;
    linkAxis axis;
    VX3_Vec3D<double> e = voxel1->position() - voxel2->position();
    VX3_Vec3D<double> ea = voxel1->orientation().RotateVec3DInv(-e);
    VX3_Vec3D<double> f = ea.Abs();
    bool reverse = false;
    if (f.x >= f.y && f.x >= f.z) {
        axis = X_AXIS;
        if (ea.x < 0) dir1 = X_NEG, dir2 = X_POS, reverse = true;
        else dir1 = X_POS, dir2 = X_NEG;
    } else if (f.y >= f.x && f.y >= f.z) {
        axis = Y_AXIS;
        if (ea.y < 0) dir1 = Y_NEG, dir2 = Y_POS, reverse = true;
        else dir1 = Y_POS, dir2 = Y_NEG;
    } else {
        axis = Z_AXIS;
        if (ea.z < 0) dir1 = Z_NEG, dir2 = Z_POS, reverse = true;
        else dir1 = Z_POS, dir2 = Z_NEG;
    }
    if (voxel1->links[dir1] != NULL || voxel2->links[dir2] != NULL) return;
    VX3_Link *pL = reverse ? new VX3_Link(voxel1, dir1, voxel2, dir2, axis, k)
                           : new VX3_Link(voxel2, dir2, voxel1, dir1, axis, k);
    pL->isNewLink = k->SafetyGuard;
    S.new_links.push_back(pL);
    k->isSurfaceChanged = true;
    voxel1->contactForce -= c1;
    voxel2->contactForce -= c2;
}

// every link of the kernel: the lattice's (d_links), then the runtime ones
int link_count(const RefSim &S) { return S.k->num_d_links + (int)S.new_links.size(); }
VX3_Link *link_at(const RefSim &S, int i) {
    return i < S.k->num_d_links ? S.k->d_links + i : S.new_links[(size_t)(i - S.k->num_d_links)];
}
int link_index(const RefSim &S, const VX3_Link *L) {
    if (L >= S.k->d_links && L < S.k->d_links + S.k->num_d_links) return (int)(L - S.k->d_links);
    for (size_t j = 0; j < S.new_links.size(); j++)
        if (S.new_links[j] == L) return S.k->num_d_links + (int)j;
    return -1;
}

// removeVoxels (VX3_VoxelyzeKernel.cu:365-397), restated over the kernel's arrays: once a
// material's RemoveFromSimulationAfterThisManySeconds (> 0) is below the current time,
// every voxel of it and each of their links leave the simulation
void remove_voxels(VX3_VoxelyzeKernel *k) {
    for (int i = 0; i < k->num_d_voxelMats; i++) {
        VX3_MaterialVoxel *m = &k->d_voxelMats[i];
        if (m->removed || !(m->RemoveFromSimulationAfterThisManySeconds > 0) ||
            !(m->RemoveFromSimulationAfterThisManySeconds < k->currentTime))
            continue;
        for (int j = 0; j < k->num_d_voxels; j++) {
            VX3_Voxel *v = &k->d_voxels[j];
            if (v->mat != m || v->removed) continue;
            v->removed = true;
            for (int d = 0; d < 6; d++) {
                VX3_Link *L = v->links[d];
                if (!L) continue;
                L->removed = true;
                VX3_Voxel *other = (L->pVNeg == v) ? L->pVPos : L->pVNeg;
                for (int q = 0; q < 6; q++)
                    if (other->links[q] == L) {
                        other->links[q] = NULL;
                        break;
                    }
                v->links[d] = NULL;
            }
        }
        m->removed = true;
        k->isSurfaceChanged = true;
    }
}

// doTimeStep (VX3_VoxelyzeKernel.cu:237-359) with dt = -1
bool do_time_step(RefSim &S) {
    VX3_VoxelyzeKernel *k = S.k;
    // updateTemperature (:219-235) -> gpu_update_temperature (:625-650)
    if (k->VaryTempEnabled && k->TempPeriod > 0) {
        for (int i = 0; i < k->num_d_voxels; i++) {
            VX3_Voxel *t = &k->d_voxels[i];
            if (t->removed) continue;
            if (t->mat->TurnOnThermalExpansionAfterThisManySeconds > k->currentTime) continue;
            if (t->mat->fixed) continue;
            double currentTemperature =
                k->TempAmplitude * sin(2 * 3.1415926f * (k->currentTime / k->TempPeriod + t->phaseOffset));
            if (!k->EnableExpansion) {
                if (currentTemperature > 0) currentTemperature = 0;
            }
            t->setTemperature(currentTemperature);
        }
    }
    k->CurStepCount++;
    float dt;
    if (!k->OptimalDt) k->OptimalDt = recommended_dt(k);
    if (k->OptimalDt < 1e-10) k->OptimalDt = 1e-10;
    dt = k->DtFrac * k->OptimalDt;
    S.last_dt = dt;

    // gpu_update_links (:566-581) over d_v_links
    bool diverged = false;
    for (int i = 0; i < link_count(S); i++) {
        VX3_Link *t = link_at(S, i);
        if (t->removed) continue;
        if (t->pVPos->mat->fixed && t->pVNeg->mat->fixed) continue;
        if (t->isDetached) continue;
        t->updateForces();
        if (t->axialStrain() > 100) diverged = true;
    }
    if (diverged) return false;

    if (k->isSurfaceChanged) {
        k->isSurfaceChanged = false;
        regenerate_surface(S);
    }
    if (k->enableAttach || k->EnableCollision) {
        // gpu_update_attach (:833-843): first in [0,S), second < first
        int num = (int)S.surface.size();
        for (int first = 0; first < num; first++)
            for (int second = 0; second < first; second++) {
                VX3_Voxel *voxel1 = S.surface[first];
                VX3_Voxel *voxel2 = S.surface[second];
                if (voxel1->removed || voxel2->removed) continue;
                collide_pair(S, voxel1, voxel2, k);
            }
    }
    S.last_contact.assign((size_t)k->num_d_voxels * 3, 0.0);
    for (int i = 0; i < k->num_d_voxels; i++) {
        S.last_contact[3 * i + 0] = k->d_voxels[i].contactForce.x;
        S.last_contact[3 * i + 1] = k->d_voxels[i].contactForce.y;
        S.last_contact[3 * i + 2] = k->d_voxels[i].contactForce.z;
    }

    // updateDetach / gpu_update_detach (:292-294, :946-967), after the collision pass
    if (k->enableDetach) {
        for (int i = 0; i < link_count(S); i++) {
            VX3_Link *t = link_at(S, i);
            if (t->removed || t->isDetached) continue;
            if (t->isFailed()) {
                t->isDetached = true;
                for (int j = 0; j < 6; j++) {
                    if (t->pVNeg->links[j] == t) t->pVNeg->links[j] = NULL;
                    if (t->pVPos->links[j] == t) t->pVPos->links[j] = NULL;
                }
                k->isSurfaceChanged = true;
            }
        }
    }

    // gpu_update_cilia_force (:846-859), before the voxel pass (:296-303)
    if (k->EnableCilia) {
        for (VX3_Voxel *v : S.surface) {
            if (v->removed) continue;
            if (v->mat->Cilia == 0) continue;
            if (v->mat->TurnOnCiliaAfterThisManySeconds > k->currentTime) continue;
            v->CiliaForce = v->orient.RotateVec3D(v->baseCiliaForce + v->localSignal * v->shiftCiliaForce);
        }
    }

    // gpu_update_voxels (:582-623), physics part
    for (int i = 0; i < k->num_d_voxels; i++) {
        VX3_Voxel *t = &k->d_voxels[i];
        if (t->removed) continue;
        if (t->mat->fixed) continue;
        t->timeStep(dt, k->currentTime, k);
        if (k->enableAttach) {  // update sticky status (:606-621); an absent condition holds
            bool ok = true;
            for (int c = 0; c < 5 && ok; c++)
                if (S.cond_set[c] && !(VX3_MathTree::eval(t->pos.x, t->pos.y, t->pos.z, k->collisionCount, k->currentTime,
                                                          k->recentAngle, k->targetCloseness, k->numClosePairs,
                                                          k->num_d_voxels, k->AttachCondition[c]) > 0))
                    ok = false;
            t->enableAttach = ok;
        }
    }
    // SecondaryExperiment (:335-349): material removal at the end of the step, before the
    // time advances (the initial-position reset there is the caller's bookkeeping)
    if (k->SecondaryExperiment) remove_voxels(k);
    k->currentTime += dt;
    return true;
}

// VX3_VoxelyzeKernel.cu:477-493
void center_of_mass(VX3_VoxelyzeKernel *k, double *out) {
    double TotalMass = 0;
    VX3_Vec3D<> Sum(0, 0, 0);
    for (int i = 0; i < k->num_d_voxels; i++) {
        if (!k->d_voxels[i].mat->isMeasured) continue;
        double ThisMass = k->d_voxels[i].material()->mass();
        Sum += k->d_voxels[i].position() * ThisMass;
        TotalMass += ThisMass;
    }
    VX3_Vec3D<> c;
    if (TotalMass != 0) c = Sum / TotalMass;
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}

int vidx(VX3_VoxelyzeKernel *k, VX3_Voxel *v) { return (int)(v - k->d_voxels); }

} // namespace

extern "C" {

// Reads a self-contained VXA document (no VXD merge) the way
// VX3_SimulationManager::readVXD does (:298-308), then builds the kernel
// object.  enable_collision / enable_expansion stand for the VX3-only keys
// VXA.Simulator.AttachDetach.EnableCollision and VXA.Simulator.EnableExpansion
// (:328, :367) that the reference reads through boost::property_tree.
void *vx3ref_create(const char *vxa_text, int enable_collision, int enable_expansion) {
    RefSim *S = new RefSim();
    S->env.pObj = &S->obj;
    S->sim.pEnv = &S->env;
    std::string text(vxa_text);
    CXML_Rip XML;
    XML.fromXMLText(&text);
    std::string msg;
    S->sim.ReadVXA(&XML, &msg);
    S->sim.Import(NULL, NULL, &msg);
    build_kernel(*S);
    S->k->EnableCollision = enable_collision != 0;
    S->k->enableAttach = false;
    S->k->enableDetach = false;
    S->k->SecondaryExperiment = 0;
    S->k->EnableExpansion = enable_expansion;
    // CUDA_Simulation prologue (:54-57): initial COM and two recommendedTimeStep calls
    double c[3];
    center_of_mass(S->k, c);
    recommended_dt(S->k);
    return S;
}

// Sets one force-field program (axis 0/1/2 = x/y/z) the way ParseMathTree fills
// VX3_ForceField's token arrays (VX3_SimulationManager.cu:349-354): n tokens laid out
// as {int op, int reserved, double value}, the last one mtEND.
int vx3ref_set_force_field(void *h, int axis, const void *tokens, int n) {
    struct Tok { int op, reserved; double value; };
    VX3_VoxelyzeKernel *k = ((RefSim *)h)->k;
    VX3_MathTreeToken *dst = axis == 0 ? k->force_field.token_x_forcefield
                             : axis == 1 ? k->force_field.token_y_forcefield
                                         : k->force_field.token_z_forcefield;
    if (axis < 0 || axis > 2 || n < 1 || n > 1024) return -1;
    const Tok *t = (const Tok *)tokens;
    for (int i = 0; i < n; i++) dst[i].set((VX3_MathTreeOperator)t[i].op, t[i].value);
    return 0;
}

// VXA.Simulator.EnableCilia, read by VX3_SimulationManager::readVXD through the
// property tree (VX3_SimulationManager.cu:360)
void vx3ref_set_cilia(void *h, int enable) { ((RefSim *)h)->k->EnableCilia = enable; }
// VXA.Simulator.AttachDetach.EnableDetach (VX3_SimulationManager.cu:330)
void vx3ref_set_detach(void *h, int enable) { ((RefSim *)h)->k->enableDetach = enable != 0; }
// VXA.Simulator.SecondaryExperiment (VX3_SimulationManager.cu:364)
void vx3ref_set_secondary(void *h, int enable) { ((RefSim *)h)->k->SecondaryExperiment = enable; }
// VXA.Simulator.AttachDetach.EnableAttach and SafetyGuard (VX3_SimulationManager.cu:329,333)
void vx3ref_set_attach(void *h, int enable, int safety_guard) {
    ((RefSim *)h)->k->enableAttach = enable != 0;
    ((RefSim *)h)->k->SafetyGuard = safety_guard;
}
// AttachCondition/Condition_k (VX3_SimulationManager.cu:334-343), tokens laid out as for
// vx3ref_set_force_field
int vx3ref_set_attach_condition(void *h, int k, const void *tokens, int n) {
    struct Tok { int op, reserved; double value; };
    RefSim *S = (RefSim *)h;
    if (k < 0 || k > 4 || n < 1 || n > 1024) return -1;
    const Tok *t = (const Tok *)tokens;
    for (int i = 0; i < n; i++) S->k->AttachCondition[k][i].set((VX3_MathTreeOperator)t[i].op, t[i].value);
    S->cond_set[k] = true;
    return 0;
}
// VXA.Simulator.EnableSignals (VX3_SimulationManager.cu:361)
void vx3ref_set_signals(void *h, int enable) { ((RefSim *)h)->k->EnableSignals = enable; }
// per voxel: localSignal
void vx3ref_signals(void *h, double *out) {
    VX3_VoxelyzeKernel *k = ((RefSim *)h)->k;
    for (int i = 0; i < k->num_d_voxels; i++) out[i] = k->d_voxels[i].localSignal;
}

void vx3ref_destroy(void *h) { /* the reference frees nothing reliably either; leak in tests */ (void)h; }

void vx3ref_counts(void *h, int *nv, int *nl, int *nsurf) {
    RefSim *S = (RefSim *)h;
    *nv = S->k->num_d_voxels;
    *nl = link_count(*S);
    *nsurf = (int)S->surface.size();
}

// returns number of steps completed (< n if the sim diverged)
int vx3ref_step(void *h, int n) {
    RefSim *S = (RefSim *)h;
    int done = 0;
    for (int i = 0; i < n; i++) {
        if (S->diverged) break;
        if (!do_time_step(*S)) { S->diverged = true; break; }
        done++;
        S->steps_done++;
    }
    return done;
}

double vx3ref_time(void *h) { return ((RefSim *)h)->k->currentTime; }
float vx3ref_dt(void *h) { return ((RefSim *)h)->last_dt; }
double vx3ref_optimal_dt(void *h) { return ((RefSim *)h)->k->OptimalDt; }
double vx3ref_recommended_dt(void *h) { return recommended_dt(((RefSim *)h)->k); }
double vx3ref_dtfrac(void *h) { return ((RefSim *)h)->k->DtFrac; }

// pos[3n], orient[4n] (w,x,y,z), linmom[3n], angmom[3n], tempe[n], flags[n] (boolStates)
void vx3ref_voxels(void *h, double *pos, double *orient, double *linmom, double *angmom, float *tempe, int *flags) {
    VX3_VoxelyzeKernel *k = ((RefSim *)h)->k;
    for (int i = 0; i < k->num_d_voxels; i++) {
        VX3_Voxel &v = k->d_voxels[i];
        pos[3 * i] = v.pos.x; pos[3 * i + 1] = v.pos.y; pos[3 * i + 2] = v.pos.z;
        orient[4 * i] = v.orient.w; orient[4 * i + 1] = v.orient.x; orient[4 * i + 2] = v.orient.y; orient[4 * i + 3] = v.orient.z;
        linmom[3 * i] = v.linMom.x; linmom[3 * i + 1] = v.linMom.y; linmom[3 * i + 2] = v.linMom.z;
        angmom[3 * i] = v.angMom.x; angmom[3 * i + 1] = v.angMom.y; angmom[3 * i + 2] = v.angMom.z;
        tempe[i] = v.tempe;
        flags[i] = v.boolStates;
    }
}

// per voxel: material index (into the voxel material list), lattice indices, 6 link slots (-1 if none)
void vx3ref_topology(void *h, int *mat, int *ijk, int *slots) {
    RefSim *S = (RefSim *)h;
    VX3_VoxelyzeKernel *k = S->k;
    for (int i = 0; i < k->num_d_voxels; i++) {
        VX3_Voxel &v = k->d_voxels[i];
        mat[i] = (int)(v.mat - k->d_voxelMats);
        ijk[3 * i] = v.ix; ijk[3 * i + 1] = v.iy; ijk[3 * i + 2] = v.iz;
        for (int d = 0; d < 6; d++) slots[6 * i + d] = v.links[d] ? link_index(*S, v.links[d]) : -1;
    }
}

// per link: neg, pos voxel index, axis, small-angle flag, bool states
void vx3ref_link_topology(void *h, int *negpos, int *axis, int *small, int *states) {
    RefSim *S = (RefSim *)h;
    VX3_VoxelyzeKernel *k = S->k;
    for (int i = 0; i < link_count(*S); i++) {
        VX3_Link &L = *link_at(*S, i);
        negpos[2 * i] = vidx(k, L.pVNeg);
        negpos[2 * i + 1] = vidx(k, L.pVPos);
        axis[i] = (int)L.axis;
        small[i] = L.smallAngle ? 1 : 0;
        states[i] = L.boolStates;
    }
}

// per link: strain, maxStrain, restLength, pos2/angle1v/angle2v (9), forceNeg/forcePos/momentNeg/momentPos (12)
void vx3ref_links(void *h, float *strain, float *maxstrain, double *rest, double *local9, double *forces12) {
    RefSim *S = (RefSim *)h;
    for (int i = 0; i < link_count(*S); i++) {
        VX3_Link &L = *link_at(*S, i);
        strain[i] = L.strain;
        maxstrain[i] = L.maxStrain;
        rest[i] = L.currentRestLength;
        double *p = local9 + 9 * i;
        p[0] = L.pos2.x; p[1] = L.pos2.y; p[2] = L.pos2.z;
        p[3] = L.angle1v.x; p[4] = L.angle1v.y; p[5] = L.angle1v.z;
        p[6] = L.angle2v.x; p[7] = L.angle2v.y; p[8] = L.angle2v.z;
        double *f = forces12 + 12 * i;
        f[0] = L.forceNeg.x; f[1] = L.forceNeg.y; f[2] = L.forceNeg.z;
        f[3] = L.forcePos.x; f[4] = L.forcePos.y; f[5] = L.forcePos.z;
        f[6] = L.momentNeg.x; f[7] = L.momentNeg.y; f[8] = L.momentNeg.z;
        f[9] = L.momentPos.x; f[10] = L.momentPos.y; f[11] = L.momentPos.z;
    }
}

// derived material constants as the kernels see them
// voxel mats: 16 floats each: mass, massInv, sqrtMass, momentInertia, momentInertiaInv, 2xSqMxExS, 2xSqIxExSxSxS,
//   zetaInternal, zetaGlobal, zetaCollision, muStatic, muKinetic, E, nu, alphaCTE, gravMult ; plus nomSize (double)
void vx3ref_voxel_mats(void *h, float *f16, double *nomsize, int *fixed_measured) {
    VX3_VoxelyzeKernel *k = ((RefSim *)h)->k;
    for (int i = 0; i < k->num_d_voxelMats; i++) {
        VX3_MaterialVoxel &m = k->d_voxelMats[i];
        float *f = f16 + 16 * i;
        f[0] = m._mass; f[1] = m._massInverse; f[2] = m._sqrtMass; f[3] = m._momentInertia; f[4] = m._momentInertiaInverse;
        f[5] = m._2xSqMxExS; f[6] = m._2xSqIxExSxSxS; f[7] = m.zetaInternal; f[8] = m.zetaGlobal; f[9] = m.zetaCollision;
        f[10] = m.muStatic; f[11] = m.muKinetic; f[12] = m.E; f[13] = m.nu; f[14] = m.alphaCTE; f[15] = m.gravMult;
        nomsize[i] = m.nomSize;
        fixed_measured[2 * i] = m.fixed ? 1 : 0;
        fixed_measured[2 * i + 1] = m.isMeasured ? 1 : 0;
    }
}
int vx3ref_num_voxel_mats(void *h) { return ((RefSim *)h)->k->num_d_voxelMats; }
int vx3ref_num_link_mats(void *h) { return (int)g_link_mats[((RefSim *)h)->k].size(); }

// link mats: 16 floats each: E, nu, eHat, a1, a2, b1, b2, b3, sqA1, sqA2xIp, sqB1, sqB2xFMp, sqB3xIp, epsilonFail, linear, alphaCTE
void vx3ref_link_mats(void *h, float *f16, int *lmat_of_link) {
    RefSim *S = (RefSim *)h;
    const std::vector<VX3_MaterialLink *> &all = g_link_mats[S->k];
    for (size_t i = 0; i < all.size(); i++) {
        VX3_MaterialLink &m = *all[i];
        float *f = f16 + 16 * i;
        f[0] = m.E; f[1] = m.nu; f[2] = m._eHat; f[3] = m._a1; f[4] = m._a2; f[5] = m._b1; f[6] = m._b2; f[7] = m._b3;
        f[8] = m._sqA1; f[9] = m._sqA2xIp; f[10] = m._sqB1; f[11] = m._sqB2xFMp; f[12] = m._sqB3xIp;
        f[13] = m.epsilonFail; f[14] = m.linear ? 1.0f : 0.0f; f[15] = m.alphaCTE;
    }
    for (int i = 0; i < link_count(*S); i++) {
        VX3_MaterialLink *m = link_at(*S, i)->mat;
        lmat_of_link[i] = (int)(std::find(all.begin(), all.end(), m) - all.begin());
    }
}

// per link: the plastic strain offset (VX3_Link::strainOffset) of non-linear materials
void vx3ref_link_offsets(void *h, float *off) {
    RefSim *S = (RefSim *)h;
    for (int i = 0; i < link_count(*S); i++) off[i] = link_at(*S, i)->strainOffset;
}

// stress-strain points of link material i ((0,0) first); returns their count, copies at most cap
int vx3ref_link_curve(void *h, int i, float *strain, float *stress, int cap) {
    VX3_MaterialLink &m = *g_link_mats[((RefSim *)h)->k][(size_t)i];
    const int n = (int)m.d_strainData.size();
    for (int j = 0; j < n && j < cap; j++) {
        strain[j] = m.d_strainData[j];
        stress[j] = m.d_stressData[j];
    }
    return n;
}

// link transverse info frozen at init: area, strainSum
void vx3ref_link_transverse(void *h, float *area, float *ssum) {
    RefSim *S = (RefSim *)h;
    for (int i = 0; i < link_count(*S); i++) {
        area[i] = link_at(*S, i)->currentTransverseArea;
        ssum[i] = link_at(*S, i)->currentTransverseStrainSum;
    }
}

void vx3ref_surface(void *h, int *idx) {
    RefSim *S = (RefSim *)h;
    for (size_t i = 0; i < S->surface.size(); i++) idx[i] = vidx(S->k, S->surface[i]);
}

// contact force per voxel as accumulated by the last step's collision pass
void vx3ref_last_contact(void *h, double *c3) {
    RefSim *S = (RefSim *)h;
    for (size_t i = 0; i < S->last_contact.size(); i++) c3[i] = S->last_contact[i];
}

void vx3ref_com(void *h, double *c3) { center_of_mass(((RefSim *)h)->k, c3); }

// environment as imported: gravity multiplier of material 0, floor flag, temp settings
void vx3ref_env(void *h, double *out8) {
    RefSim *S = (RefSim *)h;
    VX3_VoxelyzeKernel *k = S->k;
    out8[0] = k->voxSize;
    out8[1] = k->DtFrac;
    out8[2] = k->VaryTempEnabled ? 1 : 0;
    out8[3] = k->TempAmplitude;
    out8[4] = k->TempPeriod;
    out8[5] = k->num_d_voxels ? (k->d_voxels[0].isFloorEnabled() ? 1 : 0) : 0;
    out8[6] = k->EnableCollision ? 1 : 0;
    out8[7] = k->EnableExpansion;
}

// per voxel phase offset (cycles)
void vx3ref_phase(void *h, double *ph) {
    VX3_VoxelyzeKernel *k = ((RefSim *)h)->k;
    for (int i = 0; i < k->num_d_voxels; i++) ph[i] = k->d_voxels[i].phaseOffset;
}

} // extern "C"
