/*
 * jbgpu.h -- C ABI of the GB300 rigid-body step (JBullet's DiscreteDynamicsWorld
 * per-step pipeline: broadphase pairs, narrowphase + persistent manifolds,
 * sequential-impulse contact solver, transform integration).
 *
 * Every entry point returns an int status (JBGPU_OK == 0).  Plain pointers and
 * sizes only; host buffers are owned by the caller, device memory by the library.
 * One world per host thread; each world owns one CUDA stream.
 *
 * Reference interfaces replaced (paths relative to src/com/bulletphysics/):
 *   jbgpu_world_create            DiscreteDynamicsWorld(dispatcher, broadphase, solver, config)
 *                                 dynamics/DiscreteDynamicsWorld.java:86-102 with the defaults of
 *                                 ContactSolverInfo (dynamics/constraintsolver/ContactSolverInfo.java:33-48)
 *                                 and BulletGlobals (BulletGlobals.java:59-66)
 *   jbgpu_world_add_shape         BoxShape/SphereShape/CapsuleShape/ConvexHullShape/StaticPlaneShape constructors
 *                                 (collision/shapes/BoxShape.java:46-50, SphereShape.java:38-41,
 *                                 CapsuleShape.java:55-58, ConvexHullShape.java:44-50, StaticPlaneShape.java:45-48)
 *   jbgpu_world_refit_mesh        BvhTriangleMeshShape.refitTree + CollisionWorld.updateSingleAabb
 *                                 (collision/shapes/BvhTriangleMeshShape.java:172-178,
 *                                 collision/dispatch/CollisionWorld.java:195-224)
 *   jbgpu_shape_local_inertia     CollisionShape.calculateLocalInertia (BoxShape.java:153-167,
 *                                 SphereShape.java:72-76, CapsuleShape.java:125-153, PolyhedralConvexShape.java:133-159)
 *   jbgpu_world_add_bodies        new RigidBody(RigidBodyConstructionInfo) + DiscreteDynamicsWorld.addRigidBody
 *                                 (dynamics/RigidBody.java:121-164, dynamics/DiscreteDynamicsWorld.java:426-440,
 *                                 collision/dispatch/CollisionWorld.java:103-121; uid = ++gid at
 *                                 collision/broadphase/DbvtBroadphase.java:179)
 *   jbgpu_world_step_simulation   DynamicsWorld.stepSimulation(timeStep, maxSubSteps, fixedTimeStep)
 *                                 (dynamics/DiscreteDynamicsWorld.java:290-354)
 *   jbgpu_world_step              stepSimulation with maxSubSteps == substeps and an exact substep count
 *   jbgpu_world_stage             the protected phase methods of DiscreteDynamicsWorld that a subclass
 *                                 overrides (dynamics/DiscreteDynamicsWorld.java:356-400, 620-767)
 *   jbgpu_world_get_pairs         OverlappingPairCache.getOverlappingPairArray
 *                                 (collision/broadphase/OverlappingPairCache.java:34-54)
 *   jbgpu_world_get_manifolds     Dispatcher.getNumManifolds/getManifoldByIndexInternal
 *                                 (collision/broadphase/Dispatcher.java:38-67)
 *   jbgpu_world_get/set_state     RigidBody getters/setters (dynamics/RigidBody.java:480-520) and
 *                                 CollisionObject activation state (collision/dispatch/CollisionObject.java:145-180)
 *   jbgpu_world_counters          BulletStats counters (BulletStats.java:34-56)
 */
#ifndef JBGPU_H
#define JBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define JBGPU_OK                   0
#define JBGPU_ERR_INVALID_ARGUMENT 1  /* bad pointer, size, shape id or config value */
#define JBGPU_ERR_CAPACITY         2  /* a device buffer could not be grown */
#define JBGPU_ERR_CUDA             3  /* a CUDA runtime call failed (see jbgpu_last_error) */
#define JBGPU_ERR_NAN              4  /* a non-finite body state was detected after a step */
#define JBGPU_ERR_TIMEOUT          5  /* a bounded device-side wait gave up */
#define JBGPU_ERR_UNSUPPORTED      6  /* feature of the reference not on this path */
#define JBGPU_ERR_EPA_OVERFLOW     7  /* an EPA polytope outgrew its fixed face pool */
#define JBGPU_ERR_NO_DEVICE        8  /* no CUDA device could be used */

/* ---- shape types: BroadphaseNativeType ordinals (collision/broadphase/BroadphaseNativeType.java:34-112) */
#define JBGPU_SHAPE_BOX          0
#define JBGPU_SHAPE_CONVEX_HULL  4
#define JBGPU_SHAPE_SPHERE       6
#define JBGPU_SHAPE_CAPSULE      8
#define JBGPU_SHAPE_TRIANGLE_MESH 16  /* BvhTriangleMeshShape, static or kinematic bodies only */
#define JBGPU_SHAPE_STATIC_PLANE 23
#define JBGPU_SHAPE_COMPOUND     25
#define JBGPU_COMPOUND_MAX_CHILDREN 16

/* ---- activation states (collision/dispatch/CollisionObject.java:43-47) ------------ */
#define JBGPU_ACTIVE_TAG           1
#define JBGPU_ISLAND_SLEEPING      2
#define JBGPU_WANTS_DEACTIVATION   3
#define JBGPU_DISABLE_DEACTIVATION 4
#define JBGPU_DISABLE_SIMULATION   5

/* ---- collision flags a body may be given (collision/dispatch/CollisionFlags.java:31-36) -- */
#define JBGPU_CF_KINEMATIC_OBJECT     2   /* moved by the caller; saveKinematicState gives it velocities */
#define JBGPU_CF_NO_CONTACT_RESPONSE  4   /* contacts are found, never solved (trigger volumes) */

/* ---- SolverMode bits (dynamics/constraintsolver/SolverMode.java:33-36) ------------ */
#define JBGPU_SOLVER_RANDMIZE_ORDER    1  /* rejected: the GPU order is the colour order */
#define JBGPU_SOLVER_FRICTION_SEPARATE 2
#define JBGPU_SOLVER_USE_WARMSTARTING  4
#define JBGPU_SOLVER_CACHE_FRIENDLY    8

/* ---- phases of internalSingleStepSimulation, for jbgpu_world_stage --------------- */
#define JBGPU_STAGE_APPLY_GRAVITY 0 /* DiscreteDynamicsWorld.applyGravity               */
#define JBGPU_STAGE_PREDICT       1 /* predictUnconstraintMotion                        */
#define JBGPU_STAGE_AABB          2 /* CollisionWorld.updateAabbs                       */
#define JBGPU_STAGE_PAIRS         3 /* BroadphaseInterface.calculateOverlappingPairs    */
#define JBGPU_STAGE_NARROWPHASE   4 /* Dispatcher.dispatchAllCollisionPairs             */
#define JBGPU_STAGE_ISLANDS       5 /* calculateSimulationIslands + buildIslands        */
#define JBGPU_STAGE_SOLVE         6 /* solveConstraints (colour, setup, PGS, write-back) */
#define JBGPU_STAGE_INTEGRATE     7 /* integrateTransforms                              */
#define JBGPU_STAGE_ACTIVATION    8 /* updateActivationState                            */
#define JBGPU_STAGE_CLEAR_FORCES  9 /* clearForces                                      */
#define JBGPU_STAGE_SAVE_KINEMATIC 10 /* saveKinematicState(dt): velocities of kinematic bodies */

/* Floats per manifold point in jbgpu_manifolds.points (ManifoldPoint,
 * collision/narrowphase/ManifoldPoint.java:36-62):
 *  0-2 localPointA   3-5 localPointB   6-8 positionWorldOnA   9-11 positionWorldOnB
 *  12-14 normalWorldOnB  15 distance1  16 combinedFriction  17 combinedRestitution
 *  18 appliedImpulse  19 appliedImpulseLateral1  20 appliedImpulseLateral2
 *  21 lateralFrictionInitialized (0/1)  22 lifeTime (integer value)
 *  23-25 lateralFrictionDir1  26-28 lateralFrictionDir2  29-31 unused (0)          */
#define JBGPU_POINT_FLOATS 32
#define JBGPU_MANIFOLD_POINTS 4

/* Pair keys.  A pair of bodies (a, b) (body index = uid - 1) is stored under the
 * canonical key (owner << 32) | (sub << 24) | partner, where the owner is the other body when
 * exactly one body is a static plane or a triangle mesh, else min(a, b).  sub numbers the child
 * combinations of a pair with a compound body, each with its own manifold as
 * CompoundCollisionAlgorithm keeps one child algorithm per child
 * (collision/dispatch/CompoundCollisionAlgorithm.java:49-67): sub = i * n1 + j for child i of
 * body min(a, b) and child j of body max(a, b) (n1 = the latter's child count, 1 when it is
 * not a compound; i, j = 0 for a body that is not one); sub is 0 for every other pair.  Body
 * indices stay below 2^24.  Keys are unique and pair arrays are always sorted by key.  The
 * reference keeps the same set of body pairs
 * (collision/broadphase/HashedOverlappingPairCache.java:291-347) in hash order. */

typedef struct jbgpu_config {
    float   gravity[3];                 /* default (0,-10,0)  DiscreteDynamicsWorld.java:71 */
    float   contact_breaking_threshold; /* default 0.02       BulletGlobals.java:61 */
    float   deactivation_time;          /* default 2.0        BulletGlobals.java:63 */
    int32_t disable_deactivation;       /* default 0          BulletGlobals.java:64 */
    int32_t num_iterations;             /* default 10         ContactSolverInfo.java:38 */
    float   erp;                        /* default 0.2        ContactSolverInfo.java:41 */
    float   warmstarting_factor;        /* default 0.85       ContactSolverInfo.java:46 */
    float   linear_slop;                /* default 0          ContactSolverInfo.java:45 */
    int32_t solver_mode;                /* default CACHE_FRIENDLY|USE_WARMSTARTING */
    int32_t device;                     /* CUDA device ordinal, default 0 */
    int32_t initial_body_capacity;      /* device arrays grow on demand; default 1024 */
    int32_t pairs_per_body;             /* initial pair capacity per body, default 16 */
    int32_t solver_parts;               /* 0 (default): one solver part per batch world when every
                                           world has at most 2048 finite bodies, else ranges of
                                           the Morton order; > 0: that many range parts (at least
                                           finite bodies / 2048).  No counterpart in the reference. */
    int32_t solver_threads;             /* threads per solver block: 0 (default 256), 64, 128 or 256.
                                           No counterpart in the reference. */
    float   solver_residual;            /* 0 (default): num_iterations PGS iterations, as the reference.
                                           > 0: the rows of an island (the group one reference
                                           solveGroup call receives) iterate until its residual
                                           max|lambda_k - lambda_k-1| / max(max|lambda_k|, 1e-6) is
                                           <= this value, at most solver_max_iterations. */
    int32_t solver_max_iterations;      /* cap for solver_residual > 0; 0 means 200 */
    int32_t solver_smem_bodies;         /* solver parts of at most this many bodies keep their
                                           velocities in shared memory (0: 2048).  No counterpart
                                           in the reference; a tuning knob. */
    int32_t broadphase_rebuild_interval;/* rebuild the broadphase tree every this many steps and
                                           refit it in between (0 or 1: every step; default 4).  The
                                           pair set is the same either way.  A tuning knob. */
    int32_t step_graphs;                /* 1 (default): internal steps replay captured CUDA graphs
                                           (jbgpu_world_set_graph); 0: their kernels are launched one
                                           by one.  Bit-identical results.  No counterpart in the
                                           reference. */
    int32_t solver_residual_scope;      /* with solver_residual > 0: 0 (default) tests the residual of
                                           each island on its own rows (islands stop independently);
                                           1 tests it once over all rows of the world (every island
                                           iterates until max|lambda_k - lambda_k-1| over the world
                                           / max(max|lambda_k| over the world, 1e-6) <= solver_residual).
                                           No counterpart in the reference. */
} jbgpu_config;

typedef struct jbgpu_shape_desc {
    int32_t      type;       /* JBGPU_SHAPE_* */
    float        params[4];  /* BOX: half extents xyz (BoxShape(Vector3)); SPHERE: radius;
                                CAPSULE: radius, height (CapsuleShape(radius, height), up axis y);
                                STATIC_PLANE: normal xyz, plane constant; CONVEX_HULL: unused;
                                TRIANGLE_MESH, COMPOUND: params[0] = collision margin
                                (setMargin; the reference's default is 0);
                                TRIANGLE_MESH: params[1..3] = local scaling
                                (setLocalScaling before setMargin; all zero: none) */
    const float* points;     /* CONVEX_HULL: num_points * 3 floats (ConvexHullShape(points));
                                TRIANGLE_MESH: the vertex array, num_points * 3 floats */
    int32_t      num_points;
    /* TRIANGLE_MESH: BvhTriangleMeshShape(new TriangleIndexVertexArray(num_triangles, indices,
       12, num_points, points, 12), true) - one part, the quantized tree
       (collision/shapes/BvhTriangleMeshShape.java:69-93, OptimizedBvh.java:283-342); a scaling
       given in params[1..3] is applied as setLocalScaling does (BvhTriangleMeshShape.java:195-212:
       ignored within a squared distance of SIMD_EPSILON from (1,1,1), else every vertex is
       multiplied by it and the tree rebuilt). */
    const int32_t* indices;  /* 3 vertex indices per triangle */
    int32_t      num_triangles;
    /* COMPOUND: CompoundShape with addChildShape(child_transforms[i], children[i]) in order
       (collision/shapes/CompoundShape.java:59-91); children are BOX, SPHERE, CAPSULE or
       CONVEX_HULL, at most JBGPU_COMPOUND_MAX_CHILDREN. */
    const struct jbgpu_shape_desc* children;
    const float* child_transforms;   /* 12 floats per child: basis rows (row-major 3x3), origin */
    int32_t      num_children;
} jbgpu_shape_desc;

/* RigidBodyConstructionInfo (dynamics/RigidBodyConstructionInfo.java:46-79) plus the
 * velocities a caller sets with setLinearVelocity/setAngularVelocity before stepping. */
typedef struct jbgpu_body_desc {
    float   mass;                       /* 0 => static object */
    int32_t shape;                      /* id from jbgpu_world_add_shape */
    float   transform[12];              /* basis row-major (9), origin (3) */
    float   local_inertia[3];           /* usually from jbgpu_shape_local_inertia */
    float   linear_damping;             /* 0 */
    float   angular_damping;            /* 0 */
    float   friction;                   /* 0.5 */
    float   restitution;                /* 0 */
    float   linear_sleeping_threshold;  /* 0.8 */
    float   angular_sleeping_threshold; /* 1.0 */
    float   linear_velocity[3];
    float   angular_velocity[3];
    int32_t collision_group;            /* -1: DEFAULT (dynamic) / STATIC (static) */
    int32_t collision_mask;             /* -1: ALL / ALL^STATIC  (DiscreteDynamicsWorld.java:426-440) */
    int32_t world;                      /* batch world index: bodies of different worlds never collide
                                           (0 for an ordinary single world) */
    int32_t collision_flags;            /* CollisionObject.setCollisionFlags before addRigidBody:
                                           JBGPU_CF_KINEMATIC_OBJECT, JBGPU_CF_NO_CONTACT_RESPONSE (0: none;
                                           STATIC_OBJECT follows from mass 0) */
    int32_t activation_state;           /* setActivationState before addRigidBody (0: the constructor's
                                           JBGPU_ACTIVE_TAG) */
} jbgpu_body_desc;

/* Body state, structure of arrays.  Any pointer may be NULL (field skipped). */
typedef struct jbgpu_state {
    int32_t  n_bodies;            /* get: written; set: must equal the world's body count */
    float*   transform;           /* 12 per body */
    float*   linear_velocity;     /* 3 */
    float*   angular_velocity;    /* 3 */
    float*   inv_inertia_world;   /* 9 (row-major) */
    float*   total_force;         /* 3 */
    float*   total_torque;        /* 3 */
    float*   aabb;                /* 6: broadphase proxy aabb min xyz, max xyz */
    int32_t* activation_state;    /* JBGPU_ACTIVE_TAG ... */
    float*   deactivation_time;
    int32_t* island_tag;          /* get only: island root body index, -1 for static/kinematic */
} jbgpu_state;

/* Overlapping pairs with their persistent manifolds (one per pair). */
typedef struct jbgpu_manifolds {
    int32_t   n_pairs;     /* get: written; set: number of entries provided */
    int32_t   capacity;    /* get: entries the caller's arrays can hold */
    uint64_t* keys;        /* canonical keys, sorted ascending */
    int32_t*  flags;       /* bit0: the pair owns a collision algorithm and manifold */
    int32_t*  num_points;  /* 0..4 */
    float*    points;      /* capacity * 4 * JBGPU_POINT_FLOATS */
} jbgpu_manifolds;

typedef struct jbgpu_counters {
    int64_t steps;            /* internal single steps taken */
    int32_t bodies;
    int32_t pairs;            /* overlapping pairs after the last broadphase */
    int32_t manifolds;        /* pairs owning a manifold */
    int32_t contacts;         /* manifold points over all manifolds */
    int32_t solver_manifolds; /* manifolds with >= 1 solver row in the last solve */
    int32_t solver_rows;      /* normal rows (each adds 2 friction rows) */
    int32_t colours;          /* colours of the last solve */
    int32_t islands;          /* islands with >= 1 dynamic body */
    int32_t gjk_calls;        /* BulletStats.gNumGjkChecks for the last step */
    int32_t epa_calls;        /* BulletStats.gNumDeepPenetrationChecks for the last step */
    int32_t status_flags;     /* bit0 capacity, bit1 EPA pool, bit2 timeout, bit3 non-finite */
    int32_t solver_iterations;/* PGS iterations of the last solve (the largest over worlds) */
    int32_t cut_colours;      /* colours of manifolds cut between solver parts (GPU only) */
    int32_t cut_manifolds;    /* manifolds cut between solver parts (GPU only) */
    int32_t solver_islands;   /* residual mode: islands with solver rows in the last solve */
    int32_t solver_islands_converged;  /* ... of which reached the residual */
    int32_t solver_island_iterations;  /* ... sum over them of the iterations they took */
    int32_t ray_replays;      /* rays of the last jbgpu_world_ray_test replayed in body order */
    int32_t ccd_clamped;      /* bodies of the last integrateTransforms that ran a CCD sweep
                                 (BulletStats.gNumClampedCcdMotions for one step) */
} jbgpu_counters;

/* One ray of a batch: CollisionWorld.ClosestRayResultCallback after the ray
 * (collision/dispatch/CollisionWorld.java:697-729). */
typedef struct jbgpu_ray_hit {
    int32_t body;       /* collisionObject hit (body index), -1 when nothing was hit (hasHit() false) */
    float   fraction;   /* closestHitFraction: 1 when nothing was hit */
    float   normal[3];  /* hitNormalWorld: unit for convex shapes; for a static plane the triangle
                           normal rotated to world space, not normalised, as the reference leaves it */
    float   point[3];   /* hitPointWorld: from + fraction (to - from); 0 when nothing was hit */
} jbgpu_ray_hit;

/* ---- library -------------------------------------------------------------------- */
const char* jbgpu_version(void);
int64_t     jbgpu_launch_count(void);        /* kernels this library has launched in the process */
const char* jbgpu_last_error(void);          /* thread-local message for the last failure */
void        jbgpu_config_default(jbgpu_config* cfg);

/* CollisionShape.calculateLocalInertia for a shape description (host arithmetic). */
int jbgpu_shape_local_inertia(const jbgpu_shape_desc* shape, float mass, float inertia_out[3]);
/* The quantized tree of a TRIANGLE_MESH descriptor as the library builds it (OptimizedBvh's
 * quantizedContiguousNodes in walk order, collision/shapes/OptimizedBvh.java:283-342, and the
 * shape's local aabb, TriangleMeshShape.localAabbMin/Max): 4 int32 per node - min.x | min.y << 16,
 * min.z | max.x << 16, max.y | max.z << 16 (quantized, unsigned 16-bit), then the triangle index
 * of a leaf or -escapeIndex of an internal node.  Host only.  n_nodes > capacity is
 * JBGPU_ERR_CAPACITY with *n_nodes set; local_aabb (nullable): min xyz, max xyz. */
int jbgpu_shape_mesh_bvh(const jbgpu_shape_desc* mesh, int32_t* nodes, int32_t capacity, int32_t* n_nodes,
                         float local_aabb[6]);

/* ---- world ---------------------------------------------------------------------- */
typedef struct jbgpu_world jbgpu_world;

int jbgpu_world_create(const jbgpu_config* cfg, jbgpu_world** out);
int jbgpu_world_destroy(jbgpu_world* world);
int jbgpu_world_add_shape(jbgpu_world* world, const jbgpu_shape_desc* shape, int32_t* shape_id);
/* n shapes at once; ids_out (may be NULL) receives consecutive ids. */
int jbgpu_world_add_shapes(jbgpu_world* world, const jbgpu_shape_desc* shapes, int32_t n, int32_t* ids_out);
/* BvhTriangleMeshShape.refitTree (collision/shapes/BvhTriangleMeshShape.java:172-178) after the
 * positions of a TRIANGLE_MESH shape's vertices changed: points holds num_points * 3 floats (the
 * shape's vertex count; its triangle indices and scaling stay).  The tree keeps its topology and
 * is requantized as OptimizedBvh.refit does (OptimizedBvh.java:344-367,411-470), the local aabb is
 * recomputed with the shape's margin, and every body with the shape gets
 * CollisionWorld.updateSingleAabb (CollisionWorld.java:195-224) before the next step. */
int jbgpu_world_refit_mesh(jbgpu_world* world, int32_t shape, const float* points, int32_t num_points);
/* The current tree and local aabb of a TRIANGLE_MESH shape of the world (after any refit), in
 * jbgpu_shape_mesh_bvh's layout.  Host only. */
int jbgpu_world_mesh_bvh(const jbgpu_world* world, int32_t shape, int32_t* nodes, int32_t capacity, int32_t* n_nodes,
                         float local_aabb[6]);
int jbgpu_world_add_bodies(jbgpu_world* world, const jbgpu_body_desc* bodies, int32_t n, int32_t* uids_out);
/* DiscreteDynamicsWorld.removeRigidBody for n distinct bodies (dynamics/DiscreteDynamicsWorld.java:
 * 442-445 -> CollisionWorld.removeCollisionObject, collision/dispatch/CollisionWorld.java:157-176):
 * the pairs and manifolds that involve them go (cleanProxyFromPairs, destroyProxy), and the bodies
 * after each removed one move down as in the reference's collisionObjects list - a body's index
 * drops by the number of removed bodies before it.  A body that a joint uses is refused
 * (JBGPU_ERR_INVALID_ARGUMENT). */
int jbgpu_world_remove_bodies(jbgpu_world* world, const int32_t* bodies, int32_t n);
int jbgpu_world_num_bodies(const jbgpu_world* world, int32_t* n);

/* stepSimulation: the reference's fixed-timestep accumulator, applyGravity once per call,
 * then min(numSubSteps, maxSubSteps) internal single steps, then clearForces. */
int jbgpu_world_step_simulation(jbgpu_world* world, float time_step, int32_t max_sub_steps,
                                float fixed_time_step, int32_t* num_sub_steps);
/* applyGravity, `substeps` internal single steps of `fixed_time_step`, clearForces. */
int jbgpu_world_step(jbgpu_world* world, float fixed_time_step, int32_t substeps);
/* One phase of internalSingleStepSimulation (JBGPU_STAGE_*), for open-loop checks. */
int jbgpu_world_stage(jbgpu_world* world, int32_t stage, float time_step);
/* The narrowphase stage, as jbgpu_world_stage(world, JBGPU_STAGE_NARROWPHASE, dt) computes it,
 * for callers that may not allocate device memory on this path: its EPA pass takes scratch
 * from a fixed array compiled into the library (JBGPU_STATIC_EPA_SLOTS_MAX slots of 95.1 KiB,
 * 2.97 MiB per device) instead of the world's EPA arena, and the call allocates nothing.
 * epa_slots (1..JBGPU_STATIC_EPA_SLOTS_MAX) EPA warps share the queued pairs; a larger value
 * is rejected with JBGPU_ERR_CAPACITY.  The first call on a device looks the array up once
 * (cudaGetSymbolAddress with the world's device current); make that first call before any
 * stream capture begins.  The array is shared by every world of a device: calls that overlap in
 * time on one device race on it and must be serialised by the caller.  Shapes or bodies added
 * since the last step or stage are refused (uploading them allocates).  No counterpart in the
 * reference. */
#define JBGPU_STATIC_EPA_SLOTS_MAX 32
int jbgpu_world_narrowphase_static(jbgpu_world* world, int32_t epa_slots);

/* CollisionObject.setCcdMotionThreshold / setCcdSweptSphereRadius for n bodies
 * (collision/dispatch/CollisionObject.java:278-300; both 0 by default).  integrateTransforms
 * (dynamics/DiscreteDynamicsWorld.java:679-739) then sweeps a sphere of the swept radius along
 * the predicted motion of an active dynamic body whose displacement squared exceeds threshold^2,
 * and moves the body only to the first time of impact above 0.0001 (ClosestNotMeConvexResult-
 * Callback: not itself, the filters, objects it already touches with contact points - found only
 * when the body precedes the object, as the reference's pair lookup does - and hits whose
 * normal opposes the motion).  Bodies are clamped in index order, each sweep seeing the bodies
 * before it where they ended.  A sweep that reaches a static plane, where the reference throws,
 * makes the step return JBGPU_ERR_UNSUPPORTED (the body moves unclamped by the plane). */
int jbgpu_world_set_ccd(jbgpu_world* world, const int32_t* bodies, const float* motion_threshold,
                        const float* swept_sphere_radius, int32_t n);

/* RigidBody impulses for n distinct bodies (dynamics/RigidBody.java:395-430), 3 floats each:
 * impulses with rel_pos NULL is applyCentralImpulse (v += impulse * inverseMass), with rel_pos
 * applyImpulse (for a body of nonzero inverse mass: the central impulse, then applyTorqueImpulse of
 * rel_pos x impulse); torque_impulses (nullable) then applyTorqueImpulse
 * (w += invInertiaTensorWorld * torque).  impulses may be NULL when only torque impulses are given. */
int jbgpu_world_apply_impulses(jbgpu_world* world, const int32_t* bodies, const float* impulses, const float* rel_pos,
                               const float* torque_impulses, int32_t n);

/* Body properties after the bodies were added, for n distinct bodies, each array nullable (one
 * value per body): RigidBody.setDamping (dynamics/RigidBody.java:224-227; both values clamped to
 * [0, 1] by MiscUtil.GEN_clamped), CollisionObject.setFriction / setRestitution
 * (collision/dispatch/CollisionObject.java:186-196; they enter the combined values of contact
 * points made from then on, points already in a manifold keep theirs, as in the reference) and
 * RigidBody.setSleepingThresholds (RigidBody.java:371-374). */
int jbgpu_world_set_body_properties(jbgpu_world* world, const int32_t* bodies, int32_t n, const float* linear_damping,
                                    const float* angular_damping, const float* friction, const float* restitution,
                                    const float* linear_sleeping_threshold, const float* angular_sleeping_threshold);

/* DiscreteDynamicsWorld.synchronizeMotionStates (dynamics/DiscreteDynamicsWorld.java:251-276): per
 * body 12 floats (basis row-major, origin) of the transform the reference passes to
 * MotionState.setWorldTransform - the interpolation transform integrated by the interpolation
 * velocities over localTime * hitFraction (TransformUtil.integrateTransform); for static and
 * kinematic bodies, which it skips, the world transform. */
int jbgpu_world_get_interpolated_transforms(jbgpu_world* world, float* out);

/* DynamicsWorld.setInternalTickCallback (dynamics/DynamicsWorld.java:141-144), called at the end of
 * every internalSingleStepSimulation (DiscreteDynamicsWorld.java:393-395): cb(world, time_step, user)
 * runs on the calling thread after each substep of jbgpu_world_step_simulation and jbgpu_world_step,
 * with the world's stream synchronised.  It may read state and change it (impulses, forces, gravity,
 * state, body properties, bodies added or removed): the next substep sees the change.  It may not
 * step the world (jbgpu_world_step, _step_simulation and _stage return JBGPU_ERR_INVALID_ARGUMENT
 * inside it).  NULL removes the callback. */
typedef void (*jbgpu_tick_callback)(jbgpu_world* world, float time_step, void* user);
int jbgpu_world_set_internal_tick_callback(jbgpu_world* world, jbgpu_tick_callback cb, void* user);

/* DiscreteDynamicsWorld.setGravity (dynamics/DiscreteDynamicsWorld.java:403-412): the gravity of
 * bodies added later, and RigidBody.setGravity for every body already in the world. */
int jbgpu_world_set_gravity(jbgpu_world* world, const float gravity[3]);
/* RigidBody.setGravity (dynamics/RigidBody.java:213-217) for n bodies, acceleration 3 floats each:
 * the body's gravity force becomes acceleration scaled by 1 / inverseMass; a body of inverse mass 0
 * keeps its own. */
int jbgpu_world_set_body_gravity(jbgpu_world* world, const int32_t* bodies, const float* acceleration, int32_t n);

/* Wait for the world's stream. */
int jbgpu_world_synchronize(jbgpu_world* world);

/* CollisionWorld.rayTest(rayFromWorld, rayToWorld, new ClosestRayResultCallback(from, to)) for n
 * rays at once (collision/dispatch/CollisionWorld.java:553-591, rayTestSingle 260-331):
 * from and to hold n points (3 floats each); ray_world (NULL: every ray in world 0) the batch
 * world each ray is cast in; filter_group / filter_mask are the callback's
 * collisionFilterGroup / collisionFilterMask (the reference's defaults: 1 and -1).  Rays see the
 * bodies' transforms after the last step.  hits receives one record per ray.  device_buffers
 * != 0: from, to, ray_world and hits are device pointers (the call returns when the hits are
 * written to device memory); else host pointers.  Errors: a ray world outside [0, worlds) is
 * JBGPU_ERR_INVALID_ARGUMENT (host buffers: checked before any work; device buffers: such a ray
 * finds nothing and the call reports it); a tree walk deeper than its stack, or a batch with more
 * (ray, body) candidates than an int counts, is JBGPU_ERR_CAPACITY (split the batch). */
int jbgpu_world_ray_test(jbgpu_world* world, const float* from, const float* to, const int32_t* ray_world, int32_t n,
                         int32_t filter_group, int32_t filter_mask, int32_t device_buffers, jbgpu_ray_hit* hits);
/* CollisionWorld.convexSweepTest(castShape, convexFromWorld, convexToWorld,
 * new ClosestConvexResultCallback(...)) for n sweeps of one cast shape
 * (collision/dispatch/CollisionWorld.java:596-645, objectQuerySingle 391-490): shape is a convex
 * shape id of the world; from and to hold n transforms of 12 floats (basis rows, then origin);
 * sweep_world, filter_group, filter_mask, device_buffers and hits as for jbgpu_world_ray_test.
 * Each hit's fraction is GjkConvexCast's time of impact, normal the normalised hit normal and
 * point the hit point on the body.  A sweep whose path reaches a static plane gets body -2: the
 * reference throws there (its concave branch calls a null caster).  Errors as for
 * jbgpu_world_ray_test. */
int jbgpu_world_convex_sweep_test(jbgpu_world* world, int32_t shape, const float* from, const float* to,
                                  const int32_t* sweep_world, int32_t n, int32_t filter_group, int32_t filter_mask,
                                  int32_t device_buffers, jbgpu_ray_hit* hits);
/* CUDA graphs for the step (no counterpart in the reference).  on != 0: every internal step
 * replays two captured graphs (the launches before the pair-count readback and those after it)
 * instead of launching its kernels one by one; results are bit-identical to the launch path.
 * A graph is captured the first time a buffer arrangement occurs and is dropped whenever
 * buffers or settings change.  Profiling, the learned warm start and sample logging use the
 * launch path.  If a capture fails the world goes back to launches and
 * jbgpu_world_graph_status reports why. */
int jbgpu_world_set_graph(jbgpu_world* world, int32_t on);
/* Graphs held (*graphs) and the capture failure that turned graphs off ("" when none; the
 * string lives until the next jbgpu_world_set_graph). */
int jbgpu_world_graph_status(jbgpu_world* world, int32_t* graphs, const char** error);
/* Verification switch, no counterpart in the reference: all != 0 sends every ray of later
 * jbgpu_world_ray_test calls through the in-order replay of the reference's object loop (the
 * path rays take when the tree walk cannot decide them); results are the same either way. */
int jbgpu_world_set_ray_replay(jbgpu_world* world, int32_t all);

/* The iteration fields of the world's ContactSolverInfo, changed between steps as a caller of
 * the reference changes getSolverInfo().numIterations (dynamics/constraintsolver/
 * ContactSolverInfo.java:38): num_iterations (> 0), and solver_residual / solver_max_iterations
 * with the meaning of jbgpu_config. */
/* Residual trace of the last step's solve, no counterpart in the reference (residual mode
 * only): for iteration k = 0 .. *n - 1, out[2k] = max |lambda_k - lambda_k-1| and out[2k + 1] =
 * max |lambda_k| over the rows still iterating (islands not yet converged; every row with
 * solver_residual_scope 1), so out[2k] / max(out[2k + 1], 1e-6) is the residual the stopping
 * test saw.  At most JBGPU_RESIDUAL_TRACE_MAX iterations are kept; out == NULL returns *n only. */
#define JBGPU_RESIDUAL_TRACE_MAX 4096
int jbgpu_world_get_residual_trace(jbgpu_world* world, float* out, int32_t cap, int32_t* n);
int jbgpu_world_set_solver_iterations(jbgpu_world* world, int32_t num_iterations, float residual,
                                      int32_t max_iterations);

/* ---- learned warm start (no counterpart in the reference) ---------------------------
 * A per-contact MLP 24 -> 64 -> 64 -> 3 (GELU, BF16 weights and activations on the tensor
 * cores, FP32 accumulation) predicts each contact point's converged normal and two friction
 * impulses from its features; the PGS then starts from the prediction instead of
 * warmstarting_factor x last step's impulses, and runs to jbgpu_config.solver_residual.
 * Features of a point (JBGPU_MLP_INPUTS floats): normal (3), distance (1), relative velocity
 * at the contact (3), relative angular velocity (3), inverse masses (2), inverse-inertia-
 * projected normals of both bodies (6), last applied / lateral impulses (3), friction,
 * restitution (2), lifetime (1).  Targets (JBGPU_MLP_OUTPUTS floats): the converged impulses of
 * the normal row and both friction rows. */
#define JBGPU_MLP_INPUTS  24
#define JBGPU_MLP_OUTPUTS 3
#define JBGPU_MLP_PARAMS  5955  /* W1[64][24] b1[64] W2[64][64] b2[64] W3[3][64] b3[3] */
#define JBGPU_MLP_NORM    55    /* in_mean[24] in_scale[24] out_mean[3] out_scale[3] unit:
                                   x' = asinh((x - in_mean) * in_scale);  y = y' * out_scale + out_mean;
                                   unit: impulse scale of the warm-start transform below */
typedef struct jbgpu_mlp jbgpu_mlp;
int jbgpu_mlp_create(int32_t device, uint64_t seed, jbgpu_mlp** out);   /* Xavier weights, identity normalisation */
int jbgpu_mlp_destroy(jbgpu_mlp* mlp);
int jbgpu_mlp_get_params(jbgpu_mlp* mlp, float* params, float* normalization);       /* either may be NULL */
int jbgpu_mlp_set_params(jbgpu_mlp* mlp, const float* params, const float* normalization);
/* y[n][3] = MLP(x[n][24]) in raw units (host buffers). */
int jbgpu_mlp_forward(jbgpu_mlp* mlp, const float* x, int32_t n, float* y);
/* Gradient (JBGPU_MLP_PARAMS floats) and value of the mean squared error of the normalised
 * outputs over the n samples (host buffers). */
int jbgpu_mlp_gradients(jbgpu_mlp* mlp, const float* x, const float* t, int32_t n, float* grad, float* loss);
/* Training set to the device, then Adam (0.9, 0.999, 1e-8) over shuffled mini-batches. */
int jbgpu_mlp_load_samples(jbgpu_mlp* mlp, const float* x, const float* t, int32_t n);
int jbgpu_mlp_train(jbgpu_mlp* mlp, int32_t epochs, int32_t batch, float learning_rate, uint64_t seed,
                    float* loss_per_epoch);
/* Warm-start impulses from `mlp` (NULL: the reference warm start).  With b the point's last
 * normal impulse, mu its friction, u = unit / (invMass0 + invMass1) and y = 0.01 sinh(output),
 * the outputs map to normal = max(0, b + y0 (b + u)) and friction k = y(1+k) mu (b + u), clamped
 * to the cone.  The MLP must live on the world's device and outlive its use by the world. */
int jbgpu_world_set_warmstart_mlp(jbgpu_world* world, jbgpu_mlp* mlp);
/* Record features before and impulses after every solve (training data): on 1 keeps, with
 * solver_residual > 0, only points of islands that reached the residual; on 2 keeps every point
 * (its impulses after the last iteration run, converged or not); 0 stops. */
int jbgpu_world_set_sample_logging(jbgpu_world* world, int32_t on);
/* The last solve's samples: x[n][24], t[n][3] (host buffers); with x or t NULL only *n is set;
 * n > capacity is JBGPU_ERR_CAPACITY with *n set.  With solver_residual > 0 and logging mode 1
 * only points of islands that reached the residual are samples. */
int jbgpu_world_get_samples(jbgpu_world* world, float* x, float* t, int32_t capacity, int32_t* n);

/* Point-to-point (ball-socket) joint: DiscreteDynamicsWorld.addConstraint(new
 * Point2PointConstraint(rbA, rbB, pivotInA, pivotInB), false)
 * (dynamics/constraintsolver/Point2PointConstraint.java:37-171, DiscreteDynamicsWorld.java:515-521).
 * body_b = -1 is TypedConstraint's fixed body (static, at the origin; the reference's
 * one-body constructor passes pivotInB = rbA's transform applied to pivotInA).  Joints join
 * islands (DiscreteDynamicsWorld.java:649-677) and are solved in every iteration before the
 * contact rows (SequentialImpulseConstraintSolver.java:823-842), in the order of their colours
 * (first fit in index order over their dynamic bodies).  Linked bodies still collide
 * (disableCollisionsBetweenLinkedBodies = false).  *id receives the joint's index. */
int jbgpu_world_add_point2point(jbgpu_world* world, int32_t body_a, int32_t body_b, const float pivot_a[3],
                                const float pivot_b[3], int32_t* id);
/* Point2PointConstraint.ConstraintSetting (tau 0.3, damping 1, impulse clamp 0 by default);
 * JBGPU_ERR_INVALID_ARGUMENT for a hinge. */
int jbgpu_world_set_joint_setting(jbgpu_world* world, int32_t id, float tau, float damping, float impulse_clamp);
/* Hinge joint: DiscreteDynamicsWorld.addConstraint(new HingeConstraint(...), false)
 * (dynamics/constraintsolver/HingeConstraint.java:44-533).  frame_a, frame_b: the constraint
 * frames as the constructed HingeConstraint holds them (getAFrame / getBFrame: basis row-major,
 * 9 floats, then the origin; z is the hinge axis, B's axis column already negated by the
 * constructor), in the bodies' centre-of-mass spaces; body_b = -1 is the fixed body.  Starts
 * free (no limit), without motor, not angular-only.  Islands, colouring and solve order as for
 * point-to-point joints; getAppliedImpulse sums the three linear rows' impulses. */
int jbgpu_world_add_hinge(jbgpu_world* world, int32_t body_a, int32_t body_b, const float frame_a[12],
                          const float frame_b[12], int32_t* id);
/* HingeConstraint.setLimit(low, high, softness, biasFactor, relaxationFactor) (java:565-577);
 * the reference's two-argument form passes 0.9, 0.3, 1.0. */
int jbgpu_world_set_hinge_limit(jbgpu_world* world, int32_t id, float low, float high, float softness,
                                float bias_factor, float relaxation_factor);
/* HingeConstraint.enableAngularMotor(enable, targetVelocity, maxMotorImpulse) (java:559-563). */
int jbgpu_world_enable_hinge_motor(jbgpu_world* world, int32_t id, int32_t enable, float target_velocity,
                                   float max_motor_impulse);
/* HingeConstraint.setAngularOnly (java:555-557): no linear rows, the axes alone are held. */
int jbgpu_world_set_hinge_angular_only(jbgpu_world* world, int32_t id, int32_t angular_only);
/* Cone-twist joint: addConstraint(new ConeTwistConstraint(rbA, rbB, rbAFrame, rbBFrame), false)
 * (dynamics/constraintsolver/ConeTwistConstraint.java:43-412), frames as for the hinge (12 floats
 * each; x is the twist axis); body_b = -1 is the fixed body (the reference's one-body constructor
 * passes rbBFrame = rbAFrame unchanged).  Spans start at 1e30 and limitSoftness at 0, as the
 * reference's constructors leave them. */
int jbgpu_world_add_cone_twist(jbgpu_world* world, int32_t body_a, int32_t body_b, const float frame_a[12],
                               const float frame_b[12], int32_t* id);
/* ConeTwistConstraint.setLimit(swingSpan1, swingSpan2, twistSpan, softness, biasFactor,
 * relaxationFactor) (java:379-389); the three-argument form passes 0.8, 0.3, 1.0. */
int jbgpu_world_set_cone_twist_limit(jbgpu_world* world, int32_t id, float swing_span1, float swing_span2,
                                     float twist_span, float softness, float bias_factor, float relaxation_factor);
/* ConeTwistConstraint.setAngularOnly (java:371-373). */
int jbgpu_world_set_cone_twist_angular_only(jbgpu_world* world, int32_t id, int32_t angular_only);
/* Slider joint: addConstraint(new SliderConstraint(rbA, rbB, frameInA, frameInB,
 * useLinearReferenceFrameA), false) (dynamics/constraintsolver/SliderConstraint.java:130-685); frames
 * as for the 6-dof joint, x is the sliding axis; body_b = -1 is the fixed body.  Parameters as
 * SliderConstraint.initParams leaves them (java:139-172). */
int jbgpu_world_add_slider(jbgpu_world* world, int32_t body_a, int32_t body_b, const float frame_a[12],
                           const float frame_b[12], int32_t use_linear_reference_frame_a, int32_t* id);
/* The slider's setters (java:217-439) as one record of JBGPU_SLIDER_PARAMS floats: lower / upper
 * linear limit, lower / upper angular limit; softness, restitution, damping of the directional
 * linear, directional angular, linear limit, angular limit, orthogonal linear and orthogonal
 * angular rows (18); powered linear motor (0/1), its target velocity and max force; powered
 * angular motor, its target velocity and max force. */
#define JBGPU_SLIDER_PARAMS 28
int jbgpu_world_set_slider_params(jbgpu_world* world, int32_t id, const float* params);
int jbgpu_world_get_slider_params(jbgpu_world* world, int32_t id, float* params);
/* Generic 6-dof joint: addConstraint(new Generic6DofConstraint(rbA, rbB, frameInA, frameInB,
 * useLinearReferenceFrameA), false) (dynamics/constraintsolver/Generic6DofConstraint.java:88-490).
 * Frames as 12 floats (basis row-major, origin) in the bodies' centre-of-mass spaces; body_b = -1
 * is the fixed body.  Defaults as the reference: the three linear axes locked (limits 0, 0),
 * softness 0.7, damping 1, restitution 0.5; the angular axes free (limits -FLT_MAX, FLT_MAX), motors
 * off with maxMotorForce 0.1, maxLimitForce 300, damping 1, limitSoftness 0.5, ERP 0.5, bounce 0. */
int jbgpu_world_add_generic6dof(jbgpu_world* world, int32_t body_a, int32_t body_b, const float frame_a[12],
                                const float frame_b[12], int32_t use_linear_reference_frame_a, int32_t* id);
/* Generic6DofConstraint.setLimit(axis, lo, hi) (java:436-446): axes 0-2 linear, 3-5 angular; lo > hi
 * frees an axis, lo == hi locks it. */
int jbgpu_world_set_6dof_limit(jbgpu_world* world, int32_t id, int32_t axis, float lo, float hi);
/* TranslationalLimitMotor.limitSoftness / damping / restitution (TranslationalLimitMotor.java:43-45). */
int jbgpu_world_set_6dof_linear_motor(jbgpu_world* world, int32_t id, float softness, float damping, float restitution);
/* RotationalLimitMotor fields of angular axis 0-2 (RotationalLimitMotor.java:44-53): enableMotor,
 * targetVelocity, maxMotorForce, maxLimitForce, damping, limitSoftness, ERP, bounce. */
int jbgpu_world_set_6dof_angular_motor(jbgpu_world* world, int32_t id, int32_t axis, int32_t enable,
                                       float target_velocity, float max_motor_force, float max_limit_force,
                                       float damping, float limit_softness, float erp, float bounce);
/* DiscreteDynamicsWorld.removeConstraint (dynamics/DiscreteDynamicsWorld.java:524-528): joint id
 * leaves the world; the joints after it move down (id - 1), as in the reference's constraint list,
 * and keep their settings and last applied impulses. */
int jbgpu_world_remove_joint(jbgpu_world* world, int32_t id);
/* TypedConstraint.getAppliedImpulse of every joint after the last solve; with out NULL only *n
 * is set; n > capacity is JBGPU_ERR_CAPACITY with *n set. */
int jbgpu_world_get_joint_impulses(jbgpu_world* world, float* out, int32_t capacity, int32_t* n);

int jbgpu_world_get_state(jbgpu_world* world, jbgpu_state* state);
int jbgpu_world_set_state(jbgpu_world* world, const jbgpu_state* state);
int jbgpu_world_get_pairs(jbgpu_world* world, uint64_t* keys, int32_t capacity, int32_t* n_pairs);
int jbgpu_world_get_manifolds(jbgpu_world* world, jbgpu_manifolds* m);
int jbgpu_world_set_manifolds(jbgpu_world* world, const jbgpu_manifolds* m);
/* Pair indices of the manifolds of the last solve, in the sequential order the colour
 * phases are equivalent to (the order fed to the reference solver for parity). */
int jbgpu_world_get_solver_order(jbgpu_world* world, int32_t* pair_index, int32_t capacity, int32_t* n);
int jbgpu_world_counters(jbgpu_world* world, jbgpu_counters* counters);

/* RigidBody.applyCentralForce / applyTorque for every body (dynamics/RigidBody.java:362-376):
 * adds n_bodies * 3 floats of force and torque (either may be NULL) read from host memory
 * (pinned memory makes the copy asynchronous) to the accumulators cleared by clearForces. */
int jbgpu_world_apply_forces(jbgpu_world* world, const float* force, const float* torque);
/* Copies the n_bodies * 12 floats of body transforms (basis row-major, origin) to host memory;
 * the transform part of jbgpu_world_get_state, for MotionState synchronisation. */
int jbgpu_world_get_transforms(jbgpu_world* world, float* transforms);

/* Per-phase device timing with CUDA events on the world's stream (profiling builds the
 * reference's CProfileManager table, linearmath/CProfileManager.java:41-100).  Phases:
 * 0 predict, 1 aabb, 2 pair count (bounds, morton, sort, tree, count, scan), 3 pair fill
 * (fill, sort, persist), 4 narrowphase GJK pass, 5 EPA pass, 6 islands, 7 colouring,
 * 8 solver setup, 9 PGS, 10 integrate, 11 activation, 12 gravity + clear forces, 13 the
 * triangle-mesh pass of the narrowphase (worlds with meshes). */
#define JBGPU_NUM_PHASES 14
int jbgpu_world_set_profiling(jbgpu_world* world, int32_t max_steps);   /* 0 turns it off */
/* Sum of each phase's device milliseconds over the profiled steps so far (waits for them).
 * With n_phases > JBGPU_NUM_PHASES, ms[JBGPU_NUM_PHASES] receives the device time of the whole
 * profiled window (first phase mark of the first step to the last mark of the last step). */
int jbgpu_world_phase_times(jbgpu_world* world, double* ms, int32_t n_phases, int32_t* steps);
/* The step counters of each profiled step (pairs, contacts, solver rows, ...). */
int jbgpu_world_profile_counters(jbgpu_world* world, jbgpu_counters* per_step, int32_t capacity, int32_t* steps);
/* Device timer on the world's stream (no counterpart in the reference; measurement): mark 0
 * records the start event; mark 1 records the end event, waits for it and writes the device
 * milliseconds between the two into *ms. */
int jbgpu_world_timer(jbgpu_world* world, int32_t mark, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* JBGPU_H */
