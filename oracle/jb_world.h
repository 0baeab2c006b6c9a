// ORACLE (test infrastructure only): single-threaded CPU restatement of JBullet's per-step
// rigid-body pipeline (vbousquet/libgdx-jbullet).  It is the parity checker for the GPU
// library and the timed CPU baseline; the product never links it.
// Citations are relative to src/com/bulletphysics/ of the reference.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>
#include "jb_math.h"

namespace jb {

// BroadphaseNativeType ordinals (collision/broadphase/BroadphaseNativeType.java:36-72)
enum ShapeType { BOX = 0, TRIANGLE = 1, CONVEX_HULL = 4, SPHERE = 6, CAPSULE = 8, TRIANGLE_MESH = 16, STATIC_PLANE = 23,
                 COMPOUND = 25 };
enum ActState { ACTIVE_TAG = 1, ISLAND_SLEEPING = 2, WANTS_DEACTIVATION = 3, DISABLE_DEACTIVATION = 4, DISABLE_SIMULATION = 5 };
enum { CF_STATIC_OBJECT = 1, CF_KINEMATIC_OBJECT = 2, CF_NO_CONTACT_RESPONSE = 4 };
enum { SOLVER_RANDMIZE_ORDER = 1, SOLVER_USE_WARMSTARTING = 4, SOLVER_CACHE_FRIENDLY = 8 };

// OptimizedBvh with quantized aabb compression (collision/shapes/OptimizedBvh.java), the node
// array in the order buildTree writes it (depth first, left subtree first).  A node's
// escOrTri is (partId << 21) | triangleIndex for a leaf, -escapeIndex for an internal node
// (QuantizedBvhNodes.java).
struct QuantizedBvh {
    V3 bvhAabbMin{0, 0, 0}, bvhAabbMax{0, 0, 0}, bvhQuantization{0, 0, 0};
    std::vector<uint16_t> q;          // 6 per node: quantized min xyz, max xyz
    std::vector<int> escOrTri;
    int curNodeIndex = 0;
};
// BvhTriangleMeshShape over a TriangleIndexVertexArray of one part: the triangles' vertices by
// triangle index (times the scaling when setLocalScaling applied one), and the quantized tree
// over them; the indices and scaling are kept for refitTree.
struct MeshData {
    std::vector<V3> tri;              // 3 per triangle
    QuantizedBvh bvh;
    std::vector<int> idx;             // 3 vertex indices per triangle
    int numVertices = 0;
    V3 scaling{1, 1, 1};
    bool scaled = false;
};

// collision/shapes/*.java: one record for the shape classes on the path.
struct Shape {
    int type = BOX;
    float collisionMargin = 0.04f;          // ConvexInternalShape.collisionMargin (BulletGlobals.CONVEX_DISTANCE_MARGIN)
    V3 implicitDims = {0, 0, 0};            // ConvexInternalShape.implicitShapeDimensions
    V3 localScaling = {1, 1, 1};
    int upAxis = 1;                         // CapsuleShape.upAxis
    std::vector<V3> points;                 // ConvexHullShape.points
    V3 localAabbMin = {1, 1, 1}, localAabbMax = {-1, -1, -1};  // PolyhedralConvexShape local aabb
    V3 planeNormal = {0, 1, 0};             // StaticPlaneShape
    float planeConstant = 0;
    std::shared_ptr<const MeshData> mesh;   // BvhTriangleMeshShape (TriangleMeshShape.localAabbMin/Max above)
    std::vector<Shape> children;            // CompoundShape children (localAabbMin/Max above)
    std::vector<Xf> childXf;                // CompoundShapeChild.transform
    V3 tri[3];                              // TriangleShape.vertices1 (a mesh triangle during a query)
    bool isConvex() const { return type < 15; }   // BroadphaseNativeType.isConvex
    bool isConcave() const { return type > 15 && type < 24; }
    bool isCompound() const { return type == COMPOUND; }
    float getMargin() const;                // SphereShape.getMargin returns the radius
    float capsuleRadius() const { return coord(implicitDims, (upAxis + 2) % 3); }
    float capsuleHalfHeight() const { return coord(implicitDims, upAxis); }
};

Shape make_box(V3 halfExtents);
Shape make_sphere(float radius);
Shape make_capsule(float radius, float height);
Shape make_hull(const float* pts, int n);
Shape make_plane(V3 normal, float constant);
// BvhTriangleMeshShape(new TriangleIndexVertexArray(...), true) with ConcaveShape.setMargin(margin)
// scaling: BvhTriangleMeshShape.setLocalScaling before setMargin ((0, 0, 0): not called)
Shape make_mesh(const float* vertices, int numVertices, const int* indices, int numTriangles, float margin,
                V3 scaling = V3{0.0f, 0.0f, 0.0f});
// BvhTriangleMeshShape.refitTree over new positions of the mesh's vertices (same count)
void mesh_refit(Shape& s, const float* vertices);
// CompoundShape with addChildShape(transform, child) for each child in order, then setMargin(margin)
Shape make_compound(const std::vector<Shape>& children, const std::vector<Xf>& xf, float margin);
// OptimizedBvh.reportAabbOverlappingNodex: triangle indices in the order the walk reports them
void mesh_overlapping_triangles(const MeshData& m, V3 aabbMin, V3 aabbMax, std::vector<int>& out);
V3 shape_local_inertia(const Shape& s, float mass);
void shape_aabb(const Shape& s, const Xf& t, V3& mn, V3& mx);
V3 support_without_margin(const Shape& s, V3 vec);
V3 support_with_margin(const Shape& s, V3 vec);

struct ManifoldPoint {   // collision/narrowphase/ManifoldPoint.java:36-62
    V3 localA{0, 0, 0}, localB{0, 0, 0}, worldA{0, 0, 0}, worldB{0, 0, 0}, normal{0, 0, 0};
    float distance = 0, friction = 0, restitution = 0;
    float appliedImpulse = 0, lat1 = 0, lat2 = 0;
    bool latInit = false;
    int lifeTime = 0;
    V3 latDir1{0, 0, 0}, latDir2{0, 0, 0};
};

struct Manifold {        // collision/narrowphase/PersistentManifold.java
    int body0 = -1, body1 = -1;
    int n = 0;
    ManifoldPoint pts[4];
};

struct Body {            // dynamics/RigidBody.java + collision/dispatch/CollisionObject.java
    Xf xf;
    Xf ixf;                                 // interpolationWorldTransform (saveKinematicState, proceedToTransform)
    V3 ilv{0, 0, 0}, iav{0, 0, 0};          // interpolationLinearVelocity / interpolationAngularVelocity
    float hitFraction = 1.0f;               // CollisionObject.hitFraction
    V3 linvel{0, 0, 0}, angvel{0, 0, 0};
    float invMass = 0;
    V3 invInertiaLocal{0, 0, 0};
    M3 invInertiaWorld;
    V3 gravity{0, 0, 0}, totalForce{0, 0, 0}, totalTorque{0, 0, 0};
    V3 linearFactor{1, 1, 1}, angularFactor{1, 1, 1};
    float linearDamping = 0, angularDamping = 0;
    float linSleep = 0.8f, angSleep = 1.0f;
    float friction = 0.5f, restitution = 0;
    int flags = 0;
    int activation = ACTIVE_TAG;
    float deactivationTime = 0;
    int islandTag = -1, companionId = -1;
    int shape = -1;
    int group = 1, mask = -1;
    int world = 0;                          // batch world index: bodies of different worlds never pair
    V3 aabbMin{0, 0, 0}, aabbMax{0, 0, 0};  // broadphase proxy aabb
    float ccdMotionThreshold = 0.0f;        // CollisionObject.ccdMotionThreshold (0: no CCD)
    float ccdSweptSphereRadius = 0.0f;      // CollisionObject.ccdSweptSphereRadius
    bool isStaticOrKinematic() const { return (flags & (CF_STATIC_OBJECT | CF_KINEMATIC_OBJECT)) != 0; }
    bool isStatic() const { return (flags & CF_STATIC_OBJECT) != 0; }
    bool isKinematic() const { return (flags & CF_KINEMATIC_OBJECT) != 0; }
    bool isActive() const { return activation != ISLAND_SLEEPING && activation != DISABLE_SIMULATION; }
    bool mergesIslands() const { return (flags & (CF_STATIC_OBJECT | CF_KINEMATIC_OBJECT | CF_NO_CONTACT_RESPONSE)) == 0; }
    bool hasContactResponse() const { return (flags & CF_NO_CONTACT_RESPONSE) == 0; }
    void setActivationState(int s) { if (activation != DISABLE_DEACTIVATION && activation != DISABLE_SIMULATION) activation = s; }
};

// Point2PointConstraint (dynamics/constraintsolver/Point2PointConstraint.java:37-70) with its
// ConstraintSetting (java:202-206).  b = -1 stands for TypedConstraint's fixed body: static, at
// the origin with the identity basis, zero mass and inertia (TypedConstraint.java:44-49).
// HingeConstraint (dynamics/constraintsolver/HingeConstraint.java:44-620) holds the two
// constraint frames as its constructors leave them (rbAFrame, rbBFrame: z is the hinge axis,
// B's axis column already flipped), its limit (free: lower 1e30 > upper -1e30), motor and
// angularOnly switch.
// Generic6DofConstraint (dynamics/constraintsolver/Generic6DofConstraint.java:88-490) with its
// TranslationalLimitMotor (TranslationalLimitMotor.java) and three RotationalLimitMotors
// (RotationalLimitMotor.java): frames in frameA / frameB with origins in pivotA / pivotB.
// ConeTwistConstraint (dynamics/constraintsolver/ConeTwistConstraint.java:43-412): frames in
// frameA / frameB (origins in pivotA / pivotB), swing spans, twist span, softness, bias and
// relaxation in the hinge's limit fields (swing1 -> lowerLimit, swing2 -> upperLimit, twist ->
// twistSpan).
// SliderConstraint (dynamics/constraintsolver/SliderConstraint.java:44-777): frames as for the
// 6-dof joint, its parameters in `slider` (SliderParams), with useLinearReferenceFrameA == false
// swapping the bodies' roles.
enum JointType { JOINT_P2P = 0, JOINT_HINGE = 1, JOINT_6DOF = 2, JOINT_CONE = 3, JOINT_SLIDER = 4 };
struct SliderParams {   // SliderConstraint.initParams (java:139-172)
    float lowerLin = 1.0f, upperLin = -1.0f, lowerAng = 0.0f, upperAng = 0.0f;
    // softness, restitution, damping of: dir lin, dir ang, lim lin, lim ang, ortho lin, ortho ang
    float soft[6] = {1, 1, 1, 1, 1, 1};
    float rest[6] = {0.7f, 0.7f, 0.7f, 0.7f, 0.7f, 0.7f};
    float damp[6] = {0.0f, 0.0f, 1.0f, 1.0f, 1.0f, 1.0f};
    bool linMotor = false, angMotor = false;
    float linTarget = 0.0f, linMaxForce = 0.0f, angTarget = 0.0f, angMaxForce = 0.0f;
};
enum { SL_DIR_LIN = 0, SL_DIR_ANG, SL_LIM_LIN, SL_LIM_ANG, SL_ORTHO_LIN, SL_ORTHO_ANG };
struct RotMotor {     // RotationalLimitMotor defaults
    float loLimit = -SIMD_INFINITY, hiLimit = SIMD_INFINITY, targetVelocity = 0.0f, maxMotorForce = 0.1f;
    float maxLimitForce = 300.0f, damping = 1.0f, limitSoftness = 0.5f, ERP = 0.5f, bounce = 0.0f;
    bool enableMotor = false;
    int currentLimit = 0;
    float currentLimitError = 0.0f, accumulatedImpulse = 0.0f;
};
struct Joint {
    int type = JOINT_P2P;
    int a = -1, b = -1;
    V3 pivotA{0, 0, 0}, pivotB{0, 0, 0};   // pivotInA, pivotInB (hinge: the frames' origins)
    float tau = 0.3f, damping = 1.0f, impulseClamp = 0.0f;
    float appliedImpulse = 0.0f;           // TypedConstraint.appliedImpulse after the last solve
    float adiag[3] = {0, 0, 0};            // JacobianEntry.Adiag per axis, from buildJacobian
    // hinge
    M3 frameA = m3_identity(), frameB = m3_identity();   // rbAFrame.basis, rbBFrame.basis
    bool angularOnly = false, enableMotor = false;
    float motorTarget = 0.0f, maxMotorImpulse = 0.0f;
    float lowerLimit = 1e30f, upperLimit = -1e30f, limitSoftness = 0.9f, biasFactor = 0.3f, relaxationFactor = 1.0f;
    V3 normal[3];                          // buildJacobian: the linear rows' axes
    float kHinge = 0.0f, correction = 0.0f, limitSign = 0.0f, accLimitImpulse = 0.0f;
    bool solveLimit = false;
    // cone twist (limitSoftness starts at 0: the constructors leave it unset)
    float swingSpan1 = 1e30f, swingSpan2 = 1e30f, twistSpan = 1e30f, coneSoftness = 0.0f;
    V3 swingAxis{0, 0, 0}, twistAxis{0, 0, 0};
    float kSwing = 0.0f, kTwist = 0.0f, swingCorrection = 0.0f, twistCorrection = 0.0f;
    float accSwing = 0.0f, accTwist = 0.0f;
    bool solveSwing = false, solveTwist = false;
    // slider
    SliderParams slider;
    V3 slRelA{0, 0, 0}, slRelB{0, 0, 0}, slDepth{0, 0, 0};
    float slInv[3] = {0, 0, 0}, slAngDepth = 0.0f, slKAngle = 0.0f, slAccLin = 0.0f, slAccAng = 0.0f;
    bool slSolveLin = false, slSolveAng = false;
    // generic 6-dof
    bool useLinearReferenceFrameA = true;
    V3 linLower{0, 0, 0}, linUpper{0, 0, 0}, linAcc{0, 0, 0};
    float linSoftness = 0.7f, linDamping = 1.0f, linRestitution = 0.5f;
    RotMotor rot[3];
    Xf calcA, calcB;                       // calculateTransforms
    V3 angleDiff{0, 0, 0}, calcAxis[3], anchor{0, 0, 0};
    float adiagAng[3] = {0, 0, 0};
};

struct Config {
    V3 gravity{0, -10, 0};
    float contactBreakingThreshold = 0.02f;
    float deactivationTime = 2.0f;
    bool disableDeactivation = false;
    int numIterations = 10;
    float erp = 0.2f, warmstartingFactor = 0.85f, linearSlop = 0.0f;
    int solverMode = SOLVER_CACHE_FRIENDLY | SOLVER_USE_WARMSTARTING;
    float residualTol = 0.0f;         // > 0: iterate to this residual per world (jbgpu_config.solver_residual)
    int maxIterations = 200;
    int residualScope = 0;            // 1: one residual over the world's rows (jbgpu_config.solver_residual_scope)
};

struct Counters {
    long long steps = 0;
    int pairs = 0, manifolds = 0, contacts = 0, solverManifolds = 0, solverRows = 0, colours = 0, islands = 0;
    int gjk = 0, epa = 0;
    int orderMismatch = 0;   // solves whose explicit order was not a permutation of the candidates
    int solverIterations = 0;
    int ccdClamped = 0;      // CCD sweeps of the last integrateTransforms (BulletStats.gNumClampedCcdMotions)
    int ccdPlane = 0;        // CCD sweeps that reached a static plane, where the reference throws
};

// Solver order policy (the reference's F8 hook, SequentialImpulseConstraintSolver.java:769-779):
//  ORDER_REFERENCE: manifolds quick-sorted by island exactly as SimulationIslandManager does,
//                   islands solved one after the other (dispatcher order stands in for the
//                   reference's hash-dependent manifold creation order: ascending pair key);
//  ORDER_COLOUR:    the GPU's deterministic colour order when every batch world is one solver
//                   part (world, then colour, then pair index), all islands in one group
//                   (equivalent because islands share no body);
//  ORDER_EXPLICIT:  a caller-provided list of pair indices.
enum { ORDER_REFERENCE = 0, ORDER_COLOUR = 1, ORDER_EXPLICIT = 2 };

struct World {
    Config cfg;
    std::vector<Shape> shapes;
    std::vector<Body> bodies;
    // overlapping pairs sorted by canonical key, each owning its algorithm/manifold state
    std::vector<uint64_t> pairKeys;
    std::vector<uint8_t> pairHasAlgo;
    std::vector<Manifold> pairMf;
    float localTime = 1.0f / 60.0f;       // DiscreteDynamicsWorld.localTime
    void (*tickCb)(void* world, float timeStep, void* user) = nullptr;   // DynamicsWorld.internalTickCallback
    void* tickUser = nullptr;
    int orderMode = ORDER_COLOUR;
    std::vector<int> explicitOrder;
    std::vector<int> solveList;           // pair indices of islandmanifold (after ISLANDS stage)
    std::vector<int> lastOrder;           // pair indices in the order the last solve used
    std::vector<int> lastColour;          // colour per entry of lastOrder (ORDER_COLOUR)
    bool bruteForcePairs = false;         // SimpleBroadphase-style O(n^2) pair search
    std::vector<Joint> joints;            // DiscreteDynamicsWorld.constraints, in insertion order
    std::vector<int> lastJointOrder;      // joints in the order the last solve used
    Counters counters;
    double phaseSeconds[10] = {0};        // CProfile-like per-phase timers
};

// Pair keys: (owner << 32) | (sub << 24) | partner.  sub numbers the child combinations of a
// pair with a compound body (0 otherwise): sub = i * n1 + j for child i of the lower-index body
// and child j of the higher one (n1 = the higher body's child count, 1 when it is not a compound).
uint64_t pair_key(const World& w, int a, int b);
int pair_subs(const World& w, int a, int b);   // child combinations of a pair (1 without compounds)
static inline int key_owner(uint64_t k) { return (int)(k >> 32); }
static inline int key_partner(uint64_t k) { return (int)(k & 0xffffffu); }
static inline int key_sub(uint64_t k) { return (int)((k >> 24) & 0xffu); }
constexpr int MAX_COMPOUND_CHILDREN = 16;
// Joint colours: first fit in index order over the joints' dynamic bodies (neither static nor
// kinematic); the solve order is (colour, index), the GPU's order.
std::vector<int> joint_colour_order(const World& w);
void stage_apply_gravity(World& w);
void stage_predict(World& w, float dt);
void stage_aabbs(World& w);
// CollisionWorld.rayTest(from, to, ClosestRayResultCallback) over the bodies of one batch world,
// with the callback's collisionFilterGroup / collisionFilterMask.
struct RayResult { int body = -1; float fraction = 1.0f; V3 normal{0, 0, 0}, point{0, 0, 0}; };
RayResult ray_test(const World& w, V3 from, V3 to, int group, int mask, int world);
void stage_pairs(World& w);
void stage_narrowphase(World& w);
void stage_islands(World& w);
void stage_solve(World& w, float dt);
void stage_integrate(World& w, float dt);
void stage_activation(World& w, float dt);
void stage_clear_forces(World& w);
void internal_single_step(World& w, float dt);
int step_simulation(World& w, float timeStep, int maxSubSteps, float fixedTimeStep);
void stage_save_kinematic(World& w, float timeStep);
void calculate_velocity(const Xf& t0, const Xf& t1, float timeStep, V3& linVel, V3& angVel);
void step_fixed(World& w, float dt, int substeps);
// collisionFlags: setCollisionFlags (KINEMATIC_OBJECT, NO_CONTACT_RESPONSE) and activationState:
// setActivationState (0: ACTIVE_TAG), both called before addRigidBody
int add_body(World& w, float mass, int shape, const Xf& xf, V3 localInertia, float linDamp, float angDamp,
             float friction, float restitution, float linSleep, float angSleep, V3 linvel, V3 angvel, int group, int mask,
             int world = 0, int collisionFlags = 0, int activationState = 0);

// narrowphase entry (collision/dispatch/DefaultNearCallback.java:39-66 for one pair)
void process_pair(World& w, int pairIndex);
// The bodies of the manifold a pair's algorithm creates (false: EmptyAlgorithm, no manifold).
bool pair_manifold_bodies(const World& w, uint64_t key, int& mb0, int& mb1);
// GJK/EPA closest points between two convex bodies (GjkPairDetector.getClosestPoints), exposed for tests.
struct GjkOut { bool valid; V3 normal; V3 pointOnB; float distance; int usedEpa; };
GjkOut gjk_closest_points(const Shape& sa, const Xf& ta, const Shape& sb, const Xf& tb, float maxDist2, bool withEpa = true);
RayResult convex_sweep(const World& w, const Shape& cast, const Xf& from, const Xf& to, int group, int mask, int world,
                       bool* planeHit);
// integrateTransforms' CCD sweep of body `me` from its transform to `to` (a sphere of its swept
// radius, ClosestNotMeConvexResultCallback): true with the closest accepted fraction.
bool ccd_sweep(const World& w, int me, const Xf& to, float& fraction, bool* planeHit);

}  // namespace jb
