// Device-side layout of a world: structure-of-arrays in HBM, one entry per body / shape /
// pair / manifold point.  Kernels receive a DevWorld by value (plain device pointers).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "jbm.cuh"

namespace jbg {

enum { SHAPE_BOX = 0, SHAPE_TRIANGLE = 1, SHAPE_HULL = 4, SHAPE_SPHERE = 6, SHAPE_CAPSULE = 8, SHAPE_MESH = 16,
       SHAPE_PLANE = 23, SHAPE_COMPOUND = 25 };
__host__ __device__ inline bool shape_is_convex(int t) { return t < 15; }      // BroadphaseNativeType.isConvex
__host__ __device__ inline bool shape_is_concave(int t) { return t > 15 && t < 24; }
enum { ACTIVE_TAG = 1, ISLAND_SLEEPING = 2, WANTS_DEACTIVATION = 3, DISABLE_DEACTIVATION = 4, DISABLE_SIMULATION = 5 };
// CF_LISTED: a static plane or triangle mesh - kept out of the broadphase tree and paired through
// its world's list by every other body of the world (a plane's box is infinite, a terrain's spans
// the world: either would make one tree leaf own and walk to all pairs).
enum { CF_STATIC = 1, CF_KINEMATIC = 2, CF_NO_CONTACT_RESPONSE = 4, CF_LISTED = 64 };
enum { ST_CAPACITY = 1, ST_EPA_POOL = 2, ST_TIMEOUT = 4, ST_NONFINITE = 8, ST_BAD_WORLD = 16, ST_CCD_PLANE = 32 };

// Counters kept on the device (indices into DevWorld::ctr).
enum {
    C_PAIRS = 0, C_FILL_OVERFLOW, C_EPA_QUEUE, C_GJK, C_EPA, C_SOLVE_N, C_COLOURS, C_ISLANDS,
    C_MANIFOLDS, C_CONTACTS, C_ROWS, C_STATUS, C_BAR_COUNT, C_BAR_GEN, C_CUT_DONE, C_WIN0, C_WIN1, C_WIN2,
    C_PGS_ITERS, C_CUT_COLOURS, C_CUT_MANIFOLDS, C_RES0, C_RES1, C_RES2, C_ISL_N, C_ISL_CONV, C_ISL_ITERS,
    C_PART_NEXT0, C_PART_NEXT1, C_CCD_N, C_CCD_BEST, C_NCTR = 32
};

struct DevShapes {
    int* type;
    float* margin;        // getMargin() (sphere: radius)
    float4* dims;         // implicitShapeDimensions xyz; w: capsule up axis
    float4* laabb_min;    // hull local aabb (PolyhedralConvexShape.recalcLocalAabb)
    float4* laabb_max;
    float4* plane;        // static plane normal xyz, constant w
    int* hull_off;
    int* hull_cnt;
    float4* hull_pts;
    // CompoundShape: children child_off[s] .. + child_cnt[s] (0 for other shapes) of the child
    // table: the child's shape index and transform (basis rows, origin in .w; 3 per child)
    int* child_off;
    int* child_cnt;
    int* child_shape;
    float4* child_xf;
    // BvhTriangleMeshShape: quantized nodes mesh_node_off[s] .. + mesh_node_cnt[s] in walk order
    // (x: min.x | min.y << 16, y: min.z | max.x << 16, z: max.y | max.z << 16, w: triangle index
    // of a leaf or -escapeIndex), triangles from mesh_tri_off[s] (3 vertices each), and per
    // shape 3 float4: bvhAabbMin, bvhAabbMax, bvhQuantization
    int* mesh_node_off;
    int* mesh_node_cnt;
    int* mesh_tri_off;
    float4* mesh_q;
    int4* mesh_nodes;
    float4* mesh_tris;
};

// Pair key fields: (owner << 32) | (sub << 24) | partner (sub: child combination of a pair with
// a compound body).
__host__ __device__ inline int key_owner(uint64_t k) { return (int)(k >> 32); }
__host__ __device__ inline int key_partner(uint64_t k) { return (int)(k & 0xffffffu); }
__host__ __device__ inline int key_sub(uint64_t k) { return (int)((k >> 24) & 0xffu); }
constexpr int MAX_BODIES_KEYED = 1 << 24;

// The bodies of the manifold a pair's collision algorithm creates, from the two bodies' shape
// types (DefaultCollisionConfiguration.getCollisionAlgorithmCreateFunc java:160-215 with the
// algorithms' constructors): a compound's side first (with two compounds the higher body, whose
// child the swapped CompoundCollisionAlgorithm puts first), else the convex body before a plane
// or mesh, else (lower, higher).
__host__ __device__ inline void manifold_bodies(int a, int b, int typeLo, int typeHi, int& mb0, int& mb1) {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    bool hiFirst = typeHi == SHAPE_COMPOUND ||
                   (typeLo != SHAPE_COMPOUND && shape_is_convex(typeHi) && !shape_is_convex(typeLo));
    mb0 = hiFirst ? hi : lo;
    mb1 = hiFirst ? lo : hi;
}

// Manifold point, one record spread over eight float4 arrays indexed [pair * 4 + point]:
//  pA  = localPointA.xyz, distance1        pB  = localPointB.xyz, lifeTime (int bits)
//  wA  = positionWorldOnA.xyz, friction    wB  = positionWorldOnB.xyz, restitution
//  nrm = normalWorldOnB.xyz, appliedImpulse
//  imp = appliedImpulseLateral1, appliedImpulseLateral2, lateralFrictionInitialized, 0
//  d1  = lateralFrictionDir1.xyz           d2  = lateralFrictionDir2.xyz
struct DevPairs {
    uint64_t* keys;       // sorted canonical keys (owner << 32 | sub << 24 | partner)
    int* has;             // pair owns an algorithm + manifold
    int* n;               // manifold points
    int* b0;              // manifold body0 / body1
    int* b1;
    float4 *pA, *pB, *wA, *wB, *nrm, *imp, *d1, *d2;
};

// Solver rows, one normal row per contact point with distance <= 0, stored compactly: the
// points of solve slot s are rows [pt0, pt0 + popcount(mask)) with slot_desc[s].z = pt0 << 4 |
// mask; friction rows at 2 * row + k.  Slots are grouped by part and local colour, then by cut
// colour.
struct DevRows {
    float4* n_nrm;    // contactNormal, jacDiagABInv
    float4* n_rp1;    // relpos1CrossNormal, penetration
    float4* n_rp2;    // relpos2CrossNormal, restitution
    float4* n_angA;   // angularComponentA, friction
    float4* n_angB;   // angularComponentB, appliedImpulse
    float4* f_nrm;    // friction rows: direction, jacDiagABInv
    float4* f_rp1;    // relpos1CrossNormal, appliedImpulse
    float4* f_rp2;
    float4* f_angA;
    float4* f_angB;
    int* slot_pair;   // pair index of the manifold in each solve slot
    int4* slot_desc;  // body0, body1, first row << 4 | point mask, local body indices
    float2* slot_im;  // inverse masses of body0, body1
    int* slot_pt0;    // per slot: point count, then (scanned) first row
    int* pt_key;      // per row: slot << 2 | point
    int* nPts;        // device scalar: rows
};

struct DevWorld {
    int nBodies;
    int nPairs;           // pairs of the current pair arrays (device copy in ctr[C_PAIRS])
    // body state
    float4 *xr0, *xr1, *xr2;        // basis rows; origin in .w
    float4 *kx0, *kx1, *kx2;        // interpolationWorldTransform (saveKinematicState, proceedToTransform), same layout
    float4 *ilv, *iav;              // interpolationLinearVelocity / interpolationAngularVelocity
    float* hitf;                    // CollisionObject.hitFraction (1, or 0 after a CCD clamp)
    float4 *linvel, *angvel;
    float4 *iw0, *iw1, *iw2;        // inverse inertia tensor (world) rows
    float4 *iloc;                   // inverse inertia (local) xyz, inverse mass w
    float *ccdThr, *ccdRad;         // CollisionObject.ccdMotionThreshold / ccdSweptSphereRadius
    float4 *force, *torque, *gravity;
    float4 *amin, *amax;            // broadphase proxy aabb
    int* act;
    float* deact;
    int* flags;
    int* shape;
    int* group;
    int* mask;
    int* world;                     // batch world index (0 for single worlds)
    float* friction;
    float* restitution;
    float* linSleep;
    float* angSleep;
    float* linDamp;
    float* angDamp;
    int* island;                    // island root body (min index), -1 static/kinematic
    DevShapes sh;
    int* ctr;                       // device counters
    // config
    float gravityAcc[3];
    float cbt;
    float deactTime;
    int disableDeact;
    int numIter;
    float resTol;         // > 0: residual-terminated PGS
    int maxIter;          // iteration cap when resTol > 0
    int resScope;         // 0: residual per island, 1: one residual over the world's rows
    int hasCompound;      // some shape is a compound: pairs expand to child combinations
    float erp, warm, slop;
    int solverMode;
};

JBD jbd::Xf load_xf(const DevWorld& w, int i) {
    float4 a = w.xr0[i], b = w.xr1[i], c = w.xr2[i];
    jbd::Xf t;
    t.b.r[0] = jbd::mk(a.x, a.y, a.z);
    t.b.r[1] = jbd::mk(b.x, b.y, b.z);
    t.b.r[2] = jbd::mk(c.x, c.y, c.z);
    t.o = jbd::mk(a.w, b.w, c.w);
    return t;
}
JBD void store_xf(const DevWorld& w, int i, const jbd::Xf& t) {
    w.xr0[i] = make_float4(t.b.r[0].x, t.b.r[0].y, t.b.r[0].z, t.o.x);
    w.xr1[i] = make_float4(t.b.r[1].x, t.b.r[1].y, t.b.r[1].z, t.o.y);
    w.xr2[i] = make_float4(t.b.r[2].x, t.b.r[2].y, t.b.r[2].z, t.o.z);
}
// RigidBody.setCenterOfMassTransform of a dynamic body (proceedToTransform): the interpolation
// transform and velocities follow the new transform and the current velocities.
JBD void store_interpolation(const DevWorld& w, int i, const jbd::Xf& t) {
    w.kx0[i] = make_float4(t.b.r[0].x, t.b.r[0].y, t.b.r[0].z, t.o.x);
    w.kx1[i] = make_float4(t.b.r[1].x, t.b.r[1].y, t.b.r[1].z, t.o.y);
    w.kx2[i] = make_float4(t.b.r[2].x, t.b.r[2].y, t.b.r[2].z, t.o.z);
    w.ilv[i] = w.linvel[i];
    w.iav[i] = w.angvel[i];
}
JBD jbd::M load_iw(const DevWorld& w, int i) {
    jbd::M m;
    m.r[0] = jbd::mk4(w.iw0[i]);
    m.r[1] = jbd::mk4(w.iw1[i]);
    m.r[2] = jbd::mk4(w.iw2[i]);
    return m;
}
JBD bool is_active_state(int a) { return a != ISLAND_SLEEPING && a != DISABLE_SIMULATION; }
JBD bool is_static_or_kin(int f) { return (f & (CF_STATIC | CF_KINEMATIC)) != 0; }
JBD bool merges_islands(int f) { return (f & (CF_STATIC | CF_KINEMATIC | CF_NO_CONTACT_RESPONSE)) == 0; }
JBD int set_activation(int cur, int s) { return (cur != DISABLE_DEACTIVATION && cur != DISABLE_SIMULATION) ? s : cur; }

// ---- per-phase event timing ---------------------------------------------------------------
enum { PH_PREDICT = 0, PH_AABB, PH_PAIR_COUNT, PH_PAIR_FILL, PH_NARROW, PH_EPA, PH_ISLANDS, PH_COLOUR, PH_SETUP, PH_PGS,
       PH_INTEGRATE, PH_ACTIVATION, PH_OTHER, PH_CONCAVE, NUM_PHASES };

struct Prof {
    int maxSteps = 0;
    int step = 0;                 // profiled steps recorded so far
    cudaEvent_t* ev = nullptr;    // [maxSteps][NUM_PHASES][2]
    bool active() const { return step < maxSteps && ev != nullptr; }
    void mark(int phase, int which, cudaStream_t s) const {
        if (active()) cudaEventRecord(ev[((size_t)step * NUM_PHASES + phase) * 2 + which], s);
    }
};

// Counts a kernel launch of this library (process-wide, reported by jbgpu_launch_count).
void note_launch();

// ---- launchers (one per translation unit) ------------------------------------------------
struct BroadphaseScratch;   // world.cu owns the buffers; broadphase.cu reads them
void launch_apply_gravity(const DevWorld& w, cudaStream_t s);
void launch_predict(const DevWorld& w, float dt, cudaStream_t s);
void launch_aabb(const DevWorld& w, cudaStream_t s);
void launch_integrate(const DevWorld& w, float dt, cudaStream_t s);
void launch_activation(const DevWorld& w, float dt, cudaStream_t s);
void launch_clear_forces(const DevWorld& w, cudaStream_t s);
void launch_save_kinematic(const DevWorld& w, float timeStep, cudaStream_t s);
void launch_apply_impulses(const DevWorld& w, const int* bodies, const float* imp, const float* rel, const float* tq, int n,
                           cudaStream_t s);

int num_sms();

}  // namespace jbg
