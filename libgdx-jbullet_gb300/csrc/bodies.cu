// Per-body phases of the step: applyGravity, predictUnconstraintMotion, updateAabbs,
// integrateTransforms, updateActivationState, clearForces.  One thread per body; every
// kernel streams structure-of-arrays body records (HBM bound).
// Citations relative to src/com/bulletphysics/ of the reference.
#include "shapes.cuh"

namespace jbg {
using namespace jbd;

static inline int grid_for(int n, int block) { return (n + block - 1) / block; }

// DiscreteDynamicsWorld.applyGravity (dynamics/DiscreteDynamicsWorld.java:239-249)
__global__ void k_apply_gravity(DevWorld w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    if (!is_active_state(w.act[i]) || is_static_or_kin(w.flags[i])) return;
    float4 f = w.force[i], g = w.gravity[i];
    w.force[i] = make_float4(__fadd_rn(f.x, g.x), __fadd_rn(f.y, g.y), __fadd_rn(f.z, g.z), 0.0f);
}

// predictUnconstraintMotion (DiscreteDynamicsWorld.java:741-767):
// RigidBody.integrateVelocities + applyDamping (dynamics/RigidBody.java:246-299,323-342)
__global__ void k_predict(DevWorld w, float dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    if (is_static_or_kin(w.flags[i]) || !is_active_state(w.act[i])) return;
    const float MAX_ANGVEL = __fmul_rn(SIMD_2_PI, 0.25f);
    float im = w.iloc[i].w;
    float4 F = w.force[i];
    V lv = mk4(w.linvel[i]);
    float imdt = __fmul_rn(im, dt);
    lv.x = __fadd_rn(lv.x, __fmul_rn(imdt, F.x));
    lv.y = __fadd_rn(lv.y, __fmul_rn(imdt, F.y));
    lv.z = __fadd_rn(lv.z, __fmul_rn(imdt, F.z));
    V av = mk4(w.angvel[i]);
    V tmp = scl(mulMv(mk4(w.torque[i]), load_iw(w, i)), dt);
    av = add(av, tmp);
    float a = len(av);
    if (__fmul_rn(a, dt) > MAX_ANGVEL) av = scl(av, jdiv(jdiv(MAX_ANGVEL, dt), a));
    // (float)Math.pow(1 - damping, dt); pow(1, y) == 1 exactly, so zero damping skips the FP64 call
    float ld = __fsub_rn(1.0f, w.linDamp[i]), ad = __fsub_rn(1.0f, w.angDamp[i]);
    lv = scl(lv, ld == 1.0f ? 1.0f : jpow(ld, dt));
    av = scl(av, ad == 1.0f ? 1.0f : jpow(ad, dt));
    w.linvel[i] = f4(lv, 0.0f);
    w.angvel[i] = f4(av, 0.0f);
}

// CollisionWorld.updateSingleAabb (collision/dispatch/CollisionWorld.java:195-229)
__global__ void k_aabb(DevWorld w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    int act = w.act[i];
    if (!is_active_state(act)) return;
    Xf t = load_xf(w, i);
    V mn, mx;
    shape_aabb(w.sh, w.shape[i], t, mn, mx);
    float c = w.cbt;
    mn = sub(mn, mk(c, c, c));
    mx = add(mx, mk(c, c, c));
    V d = sub(mx, mn);
    if ((w.flags[i] & CF_STATIC) || (len2(d) < 1e12f)) {
        w.amin[i] = f4(mn, 0.0f);
        w.amax[i] = f4(mx, 0.0f);
    } else {
        w.act[i] = set_activation(act, DISABLE_SIMULATION);
    }
}

// integrateTransforms (DiscreteDynamicsWorld.java:679-739), CCD off; then
// RigidBody.setCenterOfMassTransform -> updateInertiaTensor (dynamics/RigidBody.java:344-354,449-459)
__global__ void k_integrate(DevWorld w, float dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    w.hitf[i] = 1.0f;
    if (!is_active_state(w.act[i]) || is_static_or_kin(w.flags[i])) return;
    Xf t = load_xf(w, i);
    Xf p = integrate_transform(t, mk4(w.linvel[i]), mk4(w.angvel[i]), dt);
    store_xf(w, i, p);
    store_interpolation(w, i, p);
    M m1 = scaleM(p.b, mk4(w.iloc[i]));
    M iw = mulMM(m1, transpose(p.b));
    w.iw0[i] = f4(iw.r[0], 0.0f);
    w.iw1[i] = f4(iw.r[1], 0.0f);
    w.iw2[i] = f4(iw.r[2], 0.0f);
}

// updateActivationState (DiscreteDynamicsWorld.java:475-512) with RigidBody.updateDeactivation /
// wantsSleeping (dynamics/RigidBody.java:543-576)
__global__ void k_activation(DevWorld w, float dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    int act = w.act[i];
    float dtime = w.deact[i];
    V lv = mk4(w.linvel[i]), av = mk4(w.angvel[i]);
    if (!(act == ISLAND_SLEEPING || act == DISABLE_DEACTIVATION)) {
        float ls = w.linSleep[i], as = w.angSleep[i];
        if (len2(lv) < __fmul_rn(ls, ls) && len2(av) < __fmul_rn(as, as)) {
            dtime = __fadd_rn(dtime, dt);
        } else {
            dtime = 0.0f;
            act = set_activation(act, 0);
        }
    }
    bool wants;
    if (act == DISABLE_DEACTIVATION) wants = false;
    else if (w.disableDeact || w.deactTime == 0.0f) wants = false;
    else if (act == ISLAND_SLEEPING || act == WANTS_DEACTIVATION) wants = true;
    else wants = dtime > w.deactTime;
    if (wants) {
        if (is_static_or_kin(w.flags[i])) {
            act = set_activation(act, ISLAND_SLEEPING);
        } else {
            if (act == ACTIVE_TAG) act = set_activation(act, WANTS_DEACTIVATION);
            if (act == ISLAND_SLEEPING) {
                w.linvel[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                w.angvel[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
    } else {
        if (act != DISABLE_DEACTIVATION) act = set_activation(act, ACTIVE_TAG);
    }
    w.act[i] = act;
    w.deact[i] = dtime;
}

__global__ void k_clear_forces(DevWorld w) {   // DiscreteDynamicsWorld.clearForces (java:226-236)
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    w.force[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w.torque[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// DiscreteDynamicsWorld.saveKinematicState (DiscreteDynamicsWorld.java:105-119) ->
// RigidBody.saveKinematicState (RigidBody.java:190-205): a kinematic body that is not
// ISLAND_SLEEPING takes the velocities that carry its last saved transform to its current one,
// which becomes the saved transform.
__global__ void k_save_kinematic(DevWorld w, float timeStep) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    if (!(w.flags[i] & CF_KINEMATIC) || w.act[i] == ISLAND_SLEEPING || timeStep == 0.0f) return;
    const Xf cur = load_xf(w, i);
    Xf prev;
    const float4 a = w.kx0[i], b = w.kx1[i], c = w.kx2[i];
    prev.b.r[0] = mk(a.x, a.y, a.z);
    prev.b.r[1] = mk(b.x, b.y, b.z);
    prev.b.r[2] = mk(c.x, c.y, c.z);
    prev.o = mk(a.w, b.w, c.w);
    V lin, ang;
    calc_velocity(prev, cur, timeStep, lin, ang);
    w.linvel[i] = f4(lin, 0.0f);
    w.angvel[i] = f4(ang, 0.0f);
    w.ilv[i] = f4(lin, 0.0f);
    w.iav[i] = f4(ang, 0.0f);
    w.kx0[i] = w.xr0[i];
    w.kx1[i] = w.xr1[i];
    w.kx2[i] = w.xr2[i];
}

void launch_save_kinematic(const DevWorld& w, float timeStep, cudaStream_t s) {
    if (w.nBodies) { k_save_kinematic<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w, timeStep); note_launch(); }
}
// RigidBody.applyCentralImpulse / applyImpulse / applyTorqueImpulse (RigidBody.java:395-430),
// linear and angular factors 1: a thread per listed body (distinct bodies).
__global__ void k_apply_impulses(DevWorld w, const int* bodies, const float* imp, const float* rel, const float* tq, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = bodies[k];
    const float im = w.iloc[i].w;
    const float4 a = w.iw0[i], b = w.iw1[i], c = w.iw2[i];
    M iw;
    iw.r[0] = mk(a.x, a.y, a.z);
    iw.r[1] = mk(b.x, b.y, b.z);
    iw.r[2] = mk(c.x, c.y, c.z);
    V lin = mk4(w.linvel[i]), ang = mk4(w.angvel[i]);
    if (imp) {
        const V J = mk(imp[3 * k], imp[3 * k + 1], imp[3 * k + 2]);
        if (!rel || im != 0.0f) lin = add(lin, scl(J, im));                    // applyCentralImpulse
        if (rel && im != 0.0f) {                                                  // applyImpulse's torque part
            const V r = mk(rel[3 * k], rel[3 * k + 1], rel[3 * k + 2]);
            ang = add(ang, mulMv(crs(r, J), iw));
        }
    }
    if (tq) ang = add(ang, mulMv(mk(tq[3 * k], tq[3 * k + 1], tq[3 * k + 2]), iw));   // applyTorqueImpulse
    w.linvel[i] = f4(lin, 0.0f);
    w.angvel[i] = f4(ang, 0.0f);
}
void launch_apply_impulses(const DevWorld& w, const int* bodies, const float* imp, const float* rel, const float* tq, int n,
                           cudaStream_t s) {
    if (n > 0) { k_apply_impulses<<<grid_for(n, 128), 128, 0, s>>>(w, bodies, imp, rel, tq, n); note_launch(); }
}

void launch_apply_gravity(const DevWorld& w, cudaStream_t s) {
    if (w.nBodies) { k_apply_gravity<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w); note_launch(); }
}
void launch_predict(const DevWorld& w, float dt, cudaStream_t s) {
    if (w.nBodies) { k_predict<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w, dt); note_launch(); }
}
void launch_aabb(const DevWorld& w, cudaStream_t s) {
    if (w.nBodies) { k_aabb<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w); note_launch(); }
}
void launch_integrate(const DevWorld& w, float dt, cudaStream_t s) {
    if (w.nBodies) { k_integrate<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w, dt); note_launch(); }
}
void launch_activation(const DevWorld& w, float dt, cudaStream_t s) {
    if (w.nBodies) { k_activation<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w, dt); note_launch(); }
}
void launch_clear_forces(const DevWorld& w, cudaStream_t s) {
    if (w.nBodies) { k_clear_forces<<<grid_for(w.nBodies, 256), 256, 0, s>>>(w); note_launch(); }
}

}  // namespace jbg
