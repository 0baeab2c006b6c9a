// ORACLE (test infrastructure only): C entry points over the CPU restatement, loaded by the
// tests and by bench.py's CPU-baseline leg through ctypes.  Uses the POD layouts of
// include/jbgpu.h so that oracle and GPU library exchange identical state buffers.
#include <cstring>
#include <vector>
#include "../include/jbgpu.h"
#include "jb_world.h"

// status_flags bit of orc_counters: an explicit solver order was not a permutation of the
// manifolds the oracle itself would solve.
static const int ORC_ORDER_MISMATCH = 1 << 16;
// status_flags bit: a CCD sweep reached a static plane (the reference throws there); the same
// bit value as the library's JBGPU status report uses for it.
static const int ORC_CCD_PLANE = 32;

using namespace jb;

static Xf xf_from12(const float* t) {
    Xf x;
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) x.b.m[r][c] = t[r * 3 + c];
    x.o = v3(t[9], t[10], t[11]);
    return x;
}
static void xf_to12(const Xf& x, float* t) {
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) t[r * 3 + c] = x.b.m[r][c];
    t[9] = x.o.x; t[10] = x.o.y; t[11] = x.o.z;
}
static Shape shape_from_desc(const jbgpu_shape_desc* d) {
    switch (d->type) {
    case JBGPU_SHAPE_BOX: return make_box(v3(d->params[0], d->params[1], d->params[2]));
    case JBGPU_SHAPE_SPHERE: return make_sphere(d->params[0]);
    case JBGPU_SHAPE_CAPSULE: return make_capsule(d->params[0], d->params[1]);
    case JBGPU_SHAPE_CONVEX_HULL: return make_hull(d->points, d->num_points);
    case JBGPU_SHAPE_TRIANGLE_MESH:
        return make_mesh(d->points, d->num_points, d->indices, d->num_triangles, d->params[0],
                         v3(d->params[1], d->params[2], d->params[3]));
    case JBGPU_SHAPE_COMPOUND: {
        std::vector<Shape> ch;
        std::vector<Xf> xf;
        for (int i = 0; i < d->num_children; i++) {
            ch.push_back(shape_from_desc(&d->children[i]));
            xf.push_back(xf_from12(d->child_transforms + 12 * i));
        }
        return make_compound(ch, xf, d->params[0]);
    }
    default: return make_plane(v3(d->params[0], d->params[1], d->params[2]), d->params[3]);
    }
}

extern "C" {

void* orc_create(const jbgpu_config* c) {
    World* w = new World();
    if (c) {
        w->cfg.gravity = v3(c->gravity[0], c->gravity[1], c->gravity[2]);
        w->cfg.contactBreakingThreshold = c->contact_breaking_threshold;
        w->cfg.deactivationTime = c->deactivation_time;
        w->cfg.disableDeactivation = c->disable_deactivation != 0;
        w->cfg.numIterations = c->num_iterations;
        w->cfg.erp = c->erp;
        w->cfg.warmstartingFactor = c->warmstarting_factor;
        w->cfg.linearSlop = c->linear_slop;
        w->cfg.solverMode = c->solver_mode;
        w->cfg.residualTol = c->solver_residual;
        w->cfg.maxIterations = c->solver_max_iterations > 0 ? c->solver_max_iterations : 200;
        w->cfg.residualScope = c->solver_residual_scope != 0 ? 1 : 0;
    }
    return w;
}
void orc_destroy(void* h) { delete (World*)h; }

int orc_add_shape(void* h, const jbgpu_shape_desc* d) {
    World* w = (World*)h;
    w->shapes.push_back(shape_from_desc(d));
    return (int)w->shapes.size() - 1;
}

// The world's current tree of a TRIANGLE_MESH shape (after any refit) in the library's node
// layout; returns the node count, -1 for a shape that is not a triangle mesh.
int orc_world_mesh_bvh(void* h, int shape, int* nodes, int cap, float* aabb) {
    World* w = (World*)h;
    if (shape < 0 || shape >= (int)w->shapes.size() || w->shapes[shape].type != TRIANGLE_MESH) return -1;
    const Shape& s = w->shapes[shape];
    const QuantizedBvh& t = s.mesh->bvh;
    for (int i = 0; i < t.curNodeIndex && i < cap; i++) {
        const uint16_t* q = &t.q[6 * i];
        nodes[4 * i] = (int)((unsigned)q[0] | ((unsigned)q[1] << 16));
        nodes[4 * i + 1] = (int)((unsigned)q[2] | ((unsigned)q[3] << 16));
        nodes[4 * i + 2] = (int)((unsigned)q[4] | ((unsigned)q[5] << 16));
        nodes[4 * i + 3] = t.escOrTri[i];
    }
    if (aabb) {
        aabb[0] = s.localAabbMin.x; aabb[1] = s.localAabbMin.y; aabb[2] = s.localAabbMin.z;
        aabb[3] = s.localAabbMax.x; aabb[4] = s.localAabbMax.y; aabb[5] = s.localAabbMax.z;
    }
    return t.curNodeIndex;
}

// BvhTriangleMeshShape.refitTree over new vertex positions, then CollisionWorld.updateSingleAabb
// (CollisionWorld.java:195-224) for every body of the shape; -1 for a shape that is not a
// triangle mesh or another vertex count.
int orc_refit_mesh(void* h, int shape, const float* points, int n) {
    World* w = (World*)h;
    if (shape < 0 || shape >= (int)w->shapes.size() || w->shapes[shape].type != TRIANGLE_MESH || !points ||
        n != w->shapes[shape].mesh->numVertices)
        return -1;
    mesh_refit(w->shapes[shape], points);
    const float t = w->cfg.contactBreakingThreshold;
    for (Body& b : w->bodies) {
        if (b.shape != shape) continue;
        V3 mn, mx;
        shape_aabb(w->shapes[shape], b.xf, mn, mx);
        mn = sub(mn, v3(t, t, t));
        mx = add(mx, v3(t, t, t));
        V3 d = sub(mx, mn);
        if (b.isStatic() || (len2(d) < 1e12f)) { b.aabbMin = mn; b.aabbMax = mx; }
        else b.setActivationState(DISABLE_SIMULATION);
    }
    return 0;
}

// The quantized tree of a TRIANGLE_MESH descriptor in the library's node layout
// (jbgpu_shape_mesh_bvh); returns the node count.
int orc_mesh_bvh(const jbgpu_shape_desc* d, int* nodes, int cap, float* aabb) {
    Shape s = shape_from_desc(d);
    const QuantizedBvh& t = s.mesh->bvh;
    for (int i = 0; i < t.curNodeIndex && i < cap; i++) {
        const uint16_t* q = &t.q[6 * i];
        nodes[4 * i] = (int)((unsigned)q[0] | ((unsigned)q[1] << 16));
        nodes[4 * i + 1] = (int)((unsigned)q[2] | ((unsigned)q[3] << 16));
        nodes[4 * i + 2] = (int)((unsigned)q[4] | ((unsigned)q[5] << 16));
        nodes[4 * i + 3] = t.escOrTri[i];
    }
    if (aabb) {
        aabb[0] = s.localAabbMin.x; aabb[1] = s.localAabbMin.y; aabb[2] = s.localAabbMin.z;
        aabb[3] = s.localAabbMax.x; aabb[4] = s.localAabbMax.y; aabb[5] = s.localAabbMax.z;
    }
    return t.curNodeIndex;
}

// OptimizedBvh.reportAabbOverlappingNodex on a TRIANGLE_MESH descriptor: the triangles in report
// order; returns their count.
int orc_mesh_query(const jbgpu_shape_desc* d, const float* mn, const float* mx, int* out, int cap) {
    Shape s = shape_from_desc(d);
    std::vector<int> tris;
    mesh_overlapping_triangles(*s.mesh, v3(mn[0], mn[1], mn[2]), v3(mx[0], mx[1], mx[2]), tris);
    for (size_t i = 0; i < tris.size() && (int)i < cap; i++) out[i] = tris[i];
    return (int)tris.size();
}

int orc_shape_local_inertia(const jbgpu_shape_desc* d, float mass, float* out) {
    Shape s = shape_from_desc(d);
    V3 i = shape_local_inertia(s, mass);
    out[0] = i.x; out[1] = i.y; out[2] = i.z;
    return 0;
}

int orc_add_bodies(void* h, const jbgpu_body_desc* b, int n) {
    World* w = (World*)h;
    for (int i = 0; i < n; i++) {
        const jbgpu_body_desc& d = b[i];
        add_body(*w, d.mass, d.shape, xf_from12(d.transform), v3(d.local_inertia[0], d.local_inertia[1], d.local_inertia[2]),
                 d.linear_damping, d.angular_damping, d.friction, d.restitution, d.linear_sleeping_threshold,
                 d.angular_sleeping_threshold, v3(d.linear_velocity[0], d.linear_velocity[1], d.linear_velocity[2]),
                 v3(d.angular_velocity[0], d.angular_velocity[1], d.angular_velocity[2]), d.collision_group, d.collision_mask,
                 d.world, d.collision_flags, d.activation_state);
    }
    return (int)w->bodies.size();
}

int orc_step_simulation(void* h, float ts, int maxSub, float fixed) { return step_simulation(*(World*)h, ts, maxSub, fixed); }
void orc_step(void* h, float dt, int substeps) { step_fixed(*(World*)h, dt, substeps); }

void orc_stage(void* h, int stage, float dt) {
    World& w = *(World*)h;
    switch (stage) {
    case JBGPU_STAGE_APPLY_GRAVITY: stage_apply_gravity(w); break;
    case JBGPU_STAGE_PREDICT: stage_predict(w, dt); break;
    case JBGPU_STAGE_AABB: stage_aabbs(w); break;
    case JBGPU_STAGE_PAIRS: stage_pairs(w); break;
    case JBGPU_STAGE_NARROWPHASE: stage_narrowphase(w); break;
    case JBGPU_STAGE_ISLANDS: stage_islands(w); break;
    case JBGPU_STAGE_SOLVE: stage_solve(w, dt); break;
    case JBGPU_STAGE_INTEGRATE: stage_integrate(w, dt); break;
    case JBGPU_STAGE_ACTIVATION: stage_activation(w, dt); break;
    case JBGPU_STAGE_CLEAR_FORCES: stage_clear_forces(w); break;
    case JBGPU_STAGE_SAVE_KINEMATIC: stage_save_kinematic(w, dt); break;
    }
}

int orc_add_point2point(void* h, int a, int b, const float* pivA, const float* pivB) {
    World* w = (World*)h;
    Joint j;
    j.a = a;
    j.b = b;
    j.pivotA = v3(pivA[0], pivA[1], pivA[2]);
    j.pivotB = v3(pivB[0], pivB[1], pivB[2]);
    w->joints.push_back(j);
    return (int)w->joints.size() - 1;
}
void orc_set_joint_setting(void* h, int id, float tau, float damping, float clamp) {
    Joint& j = ((World*)h)->joints[id];
    j.tau = tau;
    j.damping = damping;
    j.impulseClamp = clamp;
}
// frames: basis row-major (9 floats) then origin (3), as HingeConstraint holds rbAFrame/rbBFrame
int orc_add_hinge(void* h, int a, int b, const float* frameA, const float* frameB) {
    World* w = (World*)h;
    Joint j;
    j.type = JOINT_HINGE;
    j.a = a;
    j.b = b;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            j.frameA.m[r][c] = frameA[r * 3 + c];
            j.frameB.m[r][c] = frameB[r * 3 + c];
        }
    j.pivotA = v3(frameA[9], frameA[10], frameA[11]);
    j.pivotB = v3(frameB[9], frameB[10], frameB[11]);
    w->joints.push_back(j);
    return (int)w->joints.size() - 1;
}
void orc_set_hinge_limit(void* h, int id, float low, float high, float softness, float bias, float relaxation) {
    Joint& j = ((World*)h)->joints[id];
    j.lowerLimit = low;
    j.upperLimit = high;
    j.limitSoftness = softness;
    j.biasFactor = bias;
    j.relaxationFactor = relaxation;
}
void orc_enable_hinge_motor(void* h, int id, int enable, float target, float maxImpulse) {
    Joint& j = ((World*)h)->joints[id];
    j.enableMotor = enable != 0;
    j.motorTarget = target;
    j.maxMotorImpulse = maxImpulse;
}
void orc_set_hinge_angular_only(void* h, int id, int on) { ((World*)h)->joints[id].angularOnly = on != 0; }
// CollisionWorld.rayTest with a ClosestRayResultCallback per ray; out: jbgpu_ray_hit records.
void orc_ray_test(void* h, const float* from, const float* to, const int* world, int n, int group, int mask,
                  jbgpu_ray_hit* out) {
    const World& w = *(const World*)h;
    for (int i = 0; i < n; i++) {
        RayResult r = ray_test(w, v3(from[3 * i], from[3 * i + 1], from[3 * i + 2]), v3(to[3 * i], to[3 * i + 1], to[3 * i + 2]),
                               group, mask, world ? world[i] : 0);
        out[i].body = r.body;
        out[i].fraction = r.fraction;
        out[i].normal[0] = r.normal.x; out[i].normal[1] = r.normal.y; out[i].normal[2] = r.normal.z;
        out[i].point[0] = r.point.x; out[i].point[1] = r.point.y; out[i].point[2] = r.point.z;
    }
}
int orc_add_generic6dof(void* h, int a, int b, const float* frameA, const float* frameB, int useA) {
    int id = orc_add_hinge(h, a, b, frameA, frameB);
    Joint& j = ((World*)h)->joints[id];
    j.type = JOINT_6DOF;
    j.useLinearReferenceFrameA = useA != 0;
    return id;
}
void orc_set_6dof_limit(void* h, int id, int axis, float lo, float hi) {   // Generic6DofConstraint.setLimit
    Joint& j = ((World*)h)->joints[id];
    if (axis < 3) { set_coord(j.linLower, axis, lo); set_coord(j.linUpper, axis, hi); }
    else { j.rot[axis - 3].loLimit = lo; j.rot[axis - 3].hiLimit = hi; }
}
void orc_set_6dof_linear_motor(void* h, int id, float softness, float damping, float restitution) {
    Joint& j = ((World*)h)->joints[id];
    j.linSoftness = softness;
    j.linDamping = damping;
    j.linRestitution = restitution;
}
void orc_set_6dof_angular_motor(void* h, int id, int axis, int enable, float targetVelocity, float maxMotorForce,
                                float maxLimitForce, float damping, float softness, float erp, float bounce) {
    RotMotor& m = ((World*)h)->joints[id].rot[axis];
    m.enableMotor = enable != 0;
    m.targetVelocity = targetVelocity;
    m.maxMotorForce = maxMotorForce;
    m.maxLimitForce = maxLimitForce;
    m.damping = damping;
    m.limitSoftness = softness;
    m.ERP = erp;
    m.bounce = bounce;
}
int orc_add_cone_twist(void* h, int a, int b, const float* frameA, const float* frameB) {
    int id = orc_add_hinge(h, a, b, frameA, frameB);
    Joint& j = ((World*)h)->joints[id];
    j.type = JOINT_CONE;
    j.biasFactor = 0.3f;
    j.relaxationFactor = 1.0f;
    return id;
}
void orc_set_cone_limit(void* h, int id, float swing1, float swing2, float twist, float softness, float bias,
                        float relaxation) {
    Joint& j = ((World*)h)->joints[id];
    j.swingSpan1 = swing1;
    j.swingSpan2 = swing2;
    j.twistSpan = twist;
    j.coneSoftness = softness;
    j.biasFactor = bias;
    j.relaxationFactor = relaxation;
}
int orc_add_slider(void* h, int a, int b, const float* frameA, const float* frameB, int useA) {
    int id = orc_add_hinge(h, a, b, frameA, frameB);
    Joint& j = ((World*)h)->joints[id];
    j.type = JOINT_SLIDER;
    j.useLinearReferenceFrameA = useA != 0;
    return id;
}
// p: lowerLin, upperLin, lowerAng, upperAng, then softness / restitution / damping for dir lin, dir
// ang, lim lin, lim ang, ortho lin, ortho ang (18), then lin motor on, target, max force, ang motor
// on, target, max force
void orc_set_slider_params(void* h, int id, const float* p) {
    SliderParams& P = ((World*)h)->joints[id].slider;
    P.lowerLin = p[0]; P.upperLin = p[1]; P.lowerAng = p[2]; P.upperAng = p[3];
    for (int k = 0; k < 6; k++) { P.soft[k] = p[4 + 3 * k]; P.rest[k] = p[5 + 3 * k]; P.damp[k] = p[6 + 3 * k]; }
    P.linMotor = p[22] != 0.0f; P.linTarget = p[23]; P.linMaxForce = p[24];
    P.angMotor = p[25] != 0.0f; P.angTarget = p[26]; P.angMaxForce = p[27];
}
// convexSweepTest with a ClosestConvexResultCallback per sweep of the world's shape `shape`:
// from / to 12 floats each (basis row-major, origin); returns the number of sweeps that reached
// a static plane (the reference throws there).
int orc_convex_sweep(void* h, int shape, const float* from, const float* to, const int* world, int n, int group,
                     int mask, jbgpu_ray_hit* out) {
    const World& w = *(const World*)h;
    int planes = 0;
    auto xf12 = [](const float* f) {
        Xf t;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) t.b.m[r][c] = f[r * 3 + c];
        t.o = v3(f[9], f[10], f[11]);
        return t;
    };
    for (int i = 0; i < n; i++) {
        bool plane = false;
        RayResult r = convex_sweep(w, w.shapes[shape], xf12(from + 12 * i), xf12(to + 12 * i), group, mask,
                                   world ? world[i] : 0, &plane);
        planes += plane ? 1 : 0;
        if (plane) r = RayResult();     // the reference throws: no result, the record marked -2
        out[i].body = plane ? -2 : r.body;
        out[i].fraction = r.fraction;
        out[i].normal[0] = r.normal.x; out[i].normal[1] = r.normal.y; out[i].normal[2] = r.normal.z;
        out[i].point[0] = r.point.x; out[i].point[1] = r.point.y; out[i].point[2] = r.point.z;
    }
    return planes;
}
int orc_get_joint_impulses(void* h, float* out, int cap) {
    const World* w = (const World*)h;
    const int n = (int)w->joints.size();
    for (int k = 0; k < n && k < cap; k++) out[k] = w->joints[k].appliedImpulse;
    return n;
}
void orc_set_order_mode(void* h, int mode) { ((World*)h)->orderMode = mode; }
void orc_set_explicit_order(void* h, const int* order, int n) { ((World*)h)->explicitOrder.assign(order, order + n); }
void orc_set_brute_force(void* h, int on) { ((World*)h)->bruteForcePairs = on != 0; }
int orc_num_bodies(void* h) { return (int)((World*)h)->bodies.size(); }

int orc_get_state(void* h, jbgpu_state* s) {
    World& w = *(World*)h;
    int n = (int)w.bodies.size();
    s->n_bodies = n;
    for (int i = 0; i < n; i++) {
        const Body& b = w.bodies[i];
        if (s->transform) xf_to12(b.xf, s->transform + 12 * i);
        if (s->linear_velocity) { float* p = s->linear_velocity + 3 * i; p[0] = b.linvel.x; p[1] = b.linvel.y; p[2] = b.linvel.z; }
        if (s->angular_velocity) { float* p = s->angular_velocity + 3 * i; p[0] = b.angvel.x; p[1] = b.angvel.y; p[2] = b.angvel.z; }
        if (s->inv_inertia_world) for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) s->inv_inertia_world[9 * i + 3 * r + c] = b.invInertiaWorld.m[r][c];
        if (s->total_force) { float* p = s->total_force + 3 * i; p[0] = b.totalForce.x; p[1] = b.totalForce.y; p[2] = b.totalForce.z; }
        if (s->total_torque) { float* p = s->total_torque + 3 * i; p[0] = b.totalTorque.x; p[1] = b.totalTorque.y; p[2] = b.totalTorque.z; }
        if (s->aabb) { float* p = s->aabb + 6 * i; p[0] = b.aabbMin.x; p[1] = b.aabbMin.y; p[2] = b.aabbMin.z; p[3] = b.aabbMax.x; p[4] = b.aabbMax.y; p[5] = b.aabbMax.z; }
        if (s->activation_state) s->activation_state[i] = b.activation;
        if (s->deactivation_time) s->deactivation_time[i] = b.deactivationTime;
        if (s->island_tag) s->island_tag[i] = b.islandTag;
    }
    return 0;
}

// DiscreteDynamicsWorld.removeRigidBody -> CollisionWorld.removeCollisionObject
// (CollisionWorld.java:157-176): the pairs (with their manifolds) that involve a removed body go,
// the bodies after it move down in the collision object list and the remaining keys are
// renumbered; -1 for a bad or repeated index or a body a joint uses.
int orc_remove_bodies(void* h, const int* bodies, int n) {
    World* w = (World*)h;
    const int nOld = (int)w->bodies.size();
    std::vector<int> newIndex(nOld, 0);
    for (int k = 0; k < n; k++) {
        if (bodies[k] < 0 || bodies[k] >= nOld || newIndex[bodies[k]] < 0) return -1;
        newIndex[bodies[k]] = -1;
    }
    for (const Joint& j : w->joints)
        if ((j.a >= 0 && newIndex[j.a] < 0) || (j.b >= 0 && newIndex[j.b] < 0)) return -1;
    int m = 0;
    std::vector<Body> kept;
    for (int i = 0; i < nOld; i++)
        if (newIndex[i] >= 0) { newIndex[i] = m++; kept.push_back(w->bodies[i]); }
    w->bodies.swap(kept);
    std::vector<uint64_t> keys;
    std::vector<uint8_t> has;
    std::vector<Manifold> mf;
    for (size_t p = 0; p < w->pairKeys.size(); p++) {
        const uint64_t k = w->pairKeys[p];
        const int o = newIndex[key_owner(k)], q = newIndex[key_partner(k)];
        if (o < 0 || q < 0) continue;
        keys.push_back(((uint64_t)(unsigned)o << 32) | ((uint64_t)key_sub(k) << 24) | (uint64_t)(unsigned)q);
        has.push_back(w->pairHasAlgo[p]);
        Manifold f = w->pairMf[p];
        if (f.body0 >= 0) f.body0 = newIndex[f.body0];
        if (f.body1 >= 0) f.body1 = newIndex[f.body1];
        mf.push_back(f);
    }
    w->pairKeys.swap(keys);
    w->pairHasAlgo.swap(has);
    w->pairMf.swap(mf);
    for (Joint& j : w->joints) {
        if (j.a >= 0) j.a = newIndex[j.a];
        if (j.b >= 0) j.b = newIndex[j.b];
    }
    w->solveList.clear();
    w->lastOrder.clear();
    w->lastColour.clear();
    w->explicitOrder.clear();
    return 0;
}

// RigidBody.applyCentralImpulse / applyImpulse / applyTorqueImpulse (RigidBody.java:395-430) with
// linear and angular factors 1, in list order; -1 for a bad index.
int orc_apply_impulses(void* h, const int* bodies, const float* imp, const float* rel, const float* tq, int n) {
    World* w = (World*)h;
    for (int k = 0; k < n; k++)
        if (bodies[k] < 0 || bodies[k] >= (int)w->bodies.size()) return -1;
    for (int k = 0; k < n; k++) {
        Body& b = w->bodies[bodies[k]];
        if (imp) {
            const V3 J = v3(imp[3 * k], imp[3 * k + 1], imp[3 * k + 2]);
            if (!rel || b.invMass != 0.0f) b.linvel = add(b.linvel, scl(J, b.invMass));
            if (rel && b.invMass != 0.0f) {
                const V3 r = v3(rel[3 * k], rel[3 * k + 1], rel[3 * k + 2]);
                b.angvel = add(b.angvel, mulMv(crs(r, J), b.invInertiaWorld));
            }
        }
        if (tq) b.angvel = add(b.angvel, mulMv(v3(tq[3 * k], tq[3 * k + 1], tq[3 * k + 2]), b.invInertiaWorld));
    }
    return 0;
}

// RigidBody.setDamping (RigidBody.java:224-227, clamped to [0, 1]), CollisionObject.setFriction /
// setRestitution (CollisionObject.java:186-196), RigidBody.setSleepingThresholds (RigidBody.java:371-374)
// for distinct bodies; null arrays leave their property unchanged.
int orc_set_body_properties(void* h, const int* bodies, int n, const float* ld, const float* ad, const float* fr,
                            const float* re, const float* ls, const float* as) {
    World* w = (World*)h;
    std::vector<char> seen(w->bodies.size(), 0);
    for (int k = 0; k < n; k++) {
        if (bodies[k] < 0 || bodies[k] >= (int)w->bodies.size() || seen[bodies[k]]) return -1;
        seen[bodies[k]] = 1;
    }
    auto clamp01 = [](float x) { return x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x); };
    for (int k = 0; k < n; k++) {
        Body& b = w->bodies[bodies[k]];
        if (ld) b.linearDamping = clamp01(ld[k]);
        if (ad) b.angularDamping = clamp01(ad[k]);
        if (fr) b.friction = fr[k];
        if (re) b.restitution = re[k];
        if (ls) b.linSleep = ls[k];
        if (as) b.angSleep = as[k];
    }
    return 0;
}

// DiscreteDynamicsWorld.synchronizeMotionStates (DiscreteDynamicsWorld.java:251-276): the transform
// handed to each dynamic body's MotionState; static and kinematic bodies get their world transform.
void orc_get_interpolated_transforms(void* h, float* out) {
    World* w = (World*)h;
    for (size_t i = 0; i < w->bodies.size(); i++) {
        const Body& b = w->bodies[i];
        const Xf x = b.isStaticOrKinematic() ? b.xf
                                             : integrate_transform(b.ixf, b.ilv, b.iav, w->localTime * b.hitFraction);
        xf_to12(x, out + 12 * i);
    }
}

// DiscreteDynamicsWorld.removeConstraint (DiscreteDynamicsWorld.java:524-528): the joints after it move down.
int orc_remove_joint(void* h, int id) {
    World* w = (World*)h;
    if (id < 0 || id >= (int)w->joints.size()) return -1;
    w->joints.erase(w->joints.begin() + id);
    return 0;
}

// DynamicsWorld.setInternalTickCallback (DynamicsWorld.java:141-144): cb(world handle, timeStep, user)
// after every internal single step.
void orc_set_tick_callback(void* h, void (*cb)(void*, float, void*), void* user) {
    World* w = (World*)h;
    w->tickCb = cb;
    w->tickUser = user;
}

// DiscreteDynamicsWorld.setGravity (DiscreteDynamicsWorld.java:403-412) and RigidBody.setGravity
// (RigidBody.java:213-217): gravity = acceleration scaled by 1 / inverseMass when that is nonzero.
static void set_body_gravity(Body& b, V3 acc) {
    if (b.invMass != 0.0f) b.gravity = scl(acc, 1.0f / b.invMass);
}
void orc_set_gravity(void* h, const float* g) {
    World* w = (World*)h;
    w->cfg.gravity = v3(g[0], g[1], g[2]);
    for (Body& b : w->bodies) set_body_gravity(b, w->cfg.gravity);
}
int orc_set_body_gravity(void* h, const int* bodies, const float* acc, int n) {
    World* w = (World*)h;
    for (int k = 0; k < n; k++)
        if (bodies[k] < 0 || bodies[k] >= (int)w->bodies.size()) return -1;
    for (int k = 0; k < n; k++) set_body_gravity(w->bodies[bodies[k]], v3(acc[3 * k], acc[3 * k + 1], acc[3 * k + 2]));
    return 0;
}

int orc_set_ccd(void* h, const int* bodies, const float* threshold, const float* radius, int n) {
    World& w = *(World*)h;
    for (int k = 0; k < n; k++) {
        if (bodies[k] < 0 || bodies[k] >= (int)w.bodies.size()) return JBGPU_ERR_INVALID_ARGUMENT;
        w.bodies[bodies[k]].ccdMotionThreshold = threshold[k];
        w.bodies[bodies[k]].ccdSweptSphereRadius = radius[k];
    }
    return JBGPU_OK;
}

int orc_set_state(void* h, const jbgpu_state* s) {
    World& w = *(World*)h;
    int n = (int)w.bodies.size();
    if (s->n_bodies != n) return JBGPU_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; i++) {
        Body& b = w.bodies[i];
        if (s->transform) b.xf = xf_from12(s->transform + 12 * i);
        if (s->linear_velocity) { const float* p = s->linear_velocity + 3 * i; b.linvel = v3(p[0], p[1], p[2]); }
        if (s->angular_velocity) { const float* p = s->angular_velocity + 3 * i; b.angvel = v3(p[0], p[1], p[2]); }
        if (s->inv_inertia_world) for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) b.invInertiaWorld.m[r][c] = s->inv_inertia_world[9 * i + 3 * r + c];
        if (s->total_force) { const float* p = s->total_force + 3 * i; b.totalForce = v3(p[0], p[1], p[2]); }
        if (s->total_torque) { const float* p = s->total_torque + 3 * i; b.totalTorque = v3(p[0], p[1], p[2]); }
        if (s->aabb) { const float* p = s->aabb + 6 * i; b.aabbMin = v3(p[0], p[1], p[2]); b.aabbMax = v3(p[3], p[4], p[5]); }
        if (s->activation_state) b.activation = s->activation_state[i];
        if (s->deactivation_time) b.deactivationTime = s->deactivation_time[i];
    }
    return 0;
}

static void point_to(const ManifoldPoint& p, float* f) {
    std::memset(f, 0, sizeof(float) * JBGPU_POINT_FLOATS);
    V3 vs[5] = {p.localA, p.localB, p.worldA, p.worldB, p.normal};
    for (int k = 0; k < 5; k++) { f[3 * k] = vs[k].x; f[3 * k + 1] = vs[k].y; f[3 * k + 2] = vs[k].z; }
    f[15] = p.distance; f[16] = p.friction; f[17] = p.restitution;
    f[18] = p.appliedImpulse; f[19] = p.lat1; f[20] = p.lat2;
    f[21] = p.latInit ? 1.0f : 0.0f; f[22] = (float)p.lifeTime;
    f[23] = p.latDir1.x; f[24] = p.latDir1.y; f[25] = p.latDir1.z;
    f[26] = p.latDir2.x; f[27] = p.latDir2.y; f[28] = p.latDir2.z;
}
static void point_from(ManifoldPoint& p, const float* f) {
    V3* vs[5] = {&p.localA, &p.localB, &p.worldA, &p.worldB, &p.normal};
    for (int k = 0; k < 5; k++) *vs[k] = v3(f[3 * k], f[3 * k + 1], f[3 * k + 2]);
    p.distance = f[15]; p.friction = f[16]; p.restitution = f[17];
    p.appliedImpulse = f[18]; p.lat1 = f[19]; p.lat2 = f[20];
    p.latInit = f[21] != 0.0f; p.lifeTime = (int)f[22];
    p.latDir1 = v3(f[23], f[24], f[25]);
    p.latDir2 = v3(f[26], f[27], f[28]);
}

int orc_get_manifolds(void* h, jbgpu_manifolds* m) {
    World& w = *(World*)h;
    int n = (int)w.pairKeys.size();
    m->n_pairs = n;
    if (n > m->capacity) return JBGPU_ERR_CAPACITY;
    for (int i = 0; i < n; i++) {
        if (m->keys) m->keys[i] = w.pairKeys[i];
        if (m->flags) m->flags[i] = w.pairHasAlgo[i] ? 1 : 0;
        if (m->num_points) m->num_points[i] = w.pairHasAlgo[i] ? w.pairMf[i].n : 0;
        if (m->points)
            for (int j = 0; j < 4; j++) {
                float* f = m->points + ((size_t)i * 4 + j) * JBGPU_POINT_FLOATS;
                if (w.pairHasAlgo[i] && j < w.pairMf[i].n) point_to(w.pairMf[i].pts[j], f);
                else std::memset(f, 0, sizeof(float) * JBGPU_POINT_FLOATS);
            }
    }
    return 0;
}

// Manifold body order is implied by the key (pair_manifold_bodies): convex before plane or mesh,
// a compound's side first, (lo, hi) otherwise.
int orc_set_manifolds(void* h, const jbgpu_manifolds* m) {
    World& w = *(World*)h;
    int n = m->n_pairs;
    w.pairKeys.assign(m->keys, m->keys + n);
    w.pairHasAlgo.assign(n, 0);
    w.pairMf.assign(n, Manifold());
    for (int i = 0; i < n; i++) {
        Manifold& mf = w.pairMf[i];
        int mb0 = -1, mb1 = -1;
        pair_manifold_bodies(w, m->keys[i], mb0, mb1);
        mf.body0 = mb0;
        mf.body1 = mb1;
        w.pairHasAlgo[i] = (m->flags[i] & 1) ? 1 : 0;
        mf.n = w.pairHasAlgo[i] ? m->num_points[i] : 0;
        for (int j = 0; j < mf.n; j++) point_from(mf.pts[j], m->points + ((size_t)i * 4 + j) * JBGPU_POINT_FLOATS);
    }
    return 0;
}

int orc_get_solver_order(void* h, int* out, int cap) {
    World& w = *(World*)h;
    int n = (int)w.lastOrder.size();
    for (int i = 0; i < n && i < cap; i++) out[i] = w.lastOrder[i];
    return n;
}

void orc_counters(void* h, jbgpu_counters* c) {
    World& w = *(World*)h;
    std::memset(c, 0, sizeof(*c));
    c->steps = w.counters.steps;
    c->bodies = (int)w.bodies.size();
    c->pairs = w.counters.pairs;
    c->manifolds = w.counters.manifolds;
    c->contacts = w.counters.contacts;
    c->solver_manifolds = w.counters.solverManifolds;
    c->solver_rows = w.counters.solverRows;
    c->colours = w.counters.colours;
    c->islands = w.counters.islands;
    c->gjk_calls = w.counters.gjk;
    c->epa_calls = w.counters.epa;
    c->status_flags = (w.counters.orderMismatch ? ORC_ORDER_MISMATCH : 0) | (w.counters.ccdPlane ? ORC_CCD_PLANE : 0);
    c->ccd_clamped = w.counters.ccdClamped;
    c->solver_iterations = w.counters.solverIterations;
}

void orc_phase_seconds(void* h, double* out) {
    World& w = *(World*)h;
    for (int i = 0; i < 10; i++) out[i] = w.phaseSeconds[i];
}

// GjkPairDetector.getClosestPoints between two shapes at given transforms (12 floats each).
// out: normal(3), pointOnB(3), distance, valid, usedEpa
int orc_gjk(const jbgpu_shape_desc* da, const float* ta, const jbgpu_shape_desc* db, const float* tb, float maxDist2, float* out) {
    Shape sa = shape_from_desc(da), sb = shape_from_desc(db);
    GjkOut g = gjk_closest_points(sa, xf_from12(ta), sb, xf_from12(tb), maxDist2);
    out[0] = g.valid ? g.normal.x : 0; out[1] = g.valid ? g.normal.y : 0; out[2] = g.valid ? g.normal.z : 0;
    out[3] = g.valid ? g.pointOnB.x : 0; out[4] = g.valid ? g.pointOnB.y : 0; out[5] = g.valid ? g.pointOnB.z : 0;
    out[6] = g.valid ? g.distance : 0;
    out[7] = g.valid ? 1.0f : 0.0f;
    out[8] = (float)g.usedEpa;
    return g.valid ? 1 : 0;
}

// TransformUtil.integrateTransform on one transform, for unit checks of the libGDX boundary.
void orc_integrate_transform(const float* t12, const float* lin, const float* ang, float dt, float* out12) {
    Xf x = integrate_transform(xf_from12(t12), v3(lin[0], lin[1], lin[2]), v3(ang[0], ang[1], ang[2]), dt);
    xf_to12(x, out12);
}

}  // extern "C"
