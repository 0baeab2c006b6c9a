// ORACLE (test infrastructure only): world step of the reference, restated.
// Citations relative to src/com/bulletphysics/.
#include <algorithm>
#include <chrono>
#include <climits>
#include <tuple>
#include <unordered_map>
#include "jb_world.h"

namespace jb {

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
struct PhaseTimer {
    World& w; int i; double t0;
    PhaseTimer(World& ww, int ii) : w(ww), i(ii), t0(now_s()) {}
    ~PhaseTimer() { w.phaseSeconds[i] += now_s() - t0; }
};

// RigidBody.updateInertiaTensor (dynamics/RigidBody.java:449-459)
static void update_inertia_tensor(Body& b) {
    M3 mat1 = scaleM(b.xf.b, b.invInertiaLocal);
    M3 mat2 = transpose(b.xf.b);
    b.invInertiaWorld = mulMM(mat1, mat2);
}

static float gen_clamped(float a, float lb, float ub) { return a < lb ? lb : (ub < a ? ub : a); }   // MiscUtil.GEN_clamped

// RigidBody.setupRigidBody + DiscreteDynamicsWorld.addRigidBody + CollisionWorld.addCollisionObject
// (dynamics/RigidBody.java:121-164,301-312; dynamics/DiscreteDynamicsWorld.java:426-440;
//  collision/dispatch/CollisionWorld.java:103-121)
int add_body(World& w, float mass, int shape, const Xf& xf, V3 inertia, float linDamp, float angDamp, float friction,
             float restitution, float linSleep, float angSleep, V3 linvel, V3 angvel, int group, int mask, int world,
             int collisionFlags, int activationState) {
    Body b;
    b.world = world;
    b.xf = xf;
    b.ixf = xf;   // RigidBody.setupRigidBody: interpolationWorldTransform = worldTransform
    b.flags |= collisionFlags & (CF_KINEMATIC_OBJECT | CF_NO_CONTACT_RESPONSE);
    if (activationState != 0) b.activation = activationState;
    b.shape = shape;
    b.friction = friction;
    b.restitution = restitution;
    b.linSleep = linSleep;
    b.angSleep = angSleep;
    if (mass == 0.0f) { b.flags |= CF_STATIC_OBJECT; b.invMass = 0.0f; }
    else { b.flags &= ~CF_STATIC_OBJECT; b.invMass = 1.0f / mass; }
    b.invInertiaLocal = v3(inertia.x != 0.0f ? 1.0f / inertia.x : 0.0f, inertia.y != 0.0f ? 1.0f / inertia.y : 0.0f,
                           inertia.z != 0.0f ? 1.0f / inertia.z : 0.0f);
    b.linearDamping = gen_clamped(linDamp, 0.0f, 1.0f);
    b.angularDamping = gen_clamped(angDamp, 0.0f, 1.0f);
    update_inertia_tensor(b);
    if (!b.isStaticOrKinematic()) {
        if (b.invMass != 0.0f) b.gravity = scl(w.cfg.gravity, 1.0f / b.invMass);   // RigidBody.setGravity
    }
    bool isDynamic = !(b.isStatic() || b.isKinematic());
    b.group = group != -1 ? group : (isDynamic ? 1 : 2);
    b.mask = mask != -1 ? mask : (isDynamic ? -1 : (short)(-1 ^ 2));
    b.linvel = linvel;
    b.angvel = angvel;
    shape_aabb(w.shapes[shape], b.xf, b.aabbMin, b.aabbMax);   // createProxy with the shape aabb
    w.bodies.push_back(b);
    return (int)w.bodies.size() - 1;
}

// Static planes and triangle meshes: paired by every other body of the world, which owns the key.
static bool is_listed(const World& w, int i) {
    const int t = w.shapes[w.bodies[i].shape].type;
    return t == STATIC_PLANE || t == TRIANGLE_MESH;
}

uint64_t pair_key(const World& w, int a, int b) {
    bool pa = is_listed(w, a), pb = is_listed(w, b);
    int owner, partner;
    if (pa && !pb) { owner = b; partner = a; }
    else if (pb && !pa) { owner = a; partner = b; }
    else { owner = a < b ? a : b; partner = a < b ? b : a; }
    return ((uint64_t)(uint32_t)owner << 32) | (uint32_t)partner;
}

int pair_subs(const World& w, int a, int b) {
    const Shape& sa = w.shapes[w.bodies[a].shape];
    const Shape& sb = w.shapes[w.bodies[b].shape];
    int na = sa.isCompound() ? (int)sa.children.size() : 1, nb = sb.isCompound() ? (int)sb.children.size() : 1;
    return na * nb;
}

// A broadphase pair with its child combinations (one key each; CompoundCollisionAlgorithm keeps
// one child algorithm, and so one manifold, per combination).
static void push_pair(const World& w, std::vector<uint64_t>& keys, int a, int b) {
    uint64_t k = pair_key(w, a, b);
    int n = pair_subs(w, a, b);
    for (int s = 0; s < n; s++) keys.push_back(k | ((uint64_t)s << 24));
}

// ---------------------------------------------------------------------------------------
// DiscreteDynamicsWorld.applyGravity (dynamics/DiscreteDynamicsWorld.java:239-249)
void stage_apply_gravity(World& w) {
    for (Body& b : w.bodies) {
        if (b.isActive() && !b.isStaticOrKinematic()) {   // RigidBody.applyGravity -> applyCentralForce
            b.totalForce.x += b.gravity.x * b.linearFactor.x;
            b.totalForce.y += b.gravity.y * b.linearFactor.y;
            b.totalForce.z += b.gravity.z * b.linearFactor.z;
        }
    }
}

// predictUnconstraintMotion (DiscreteDynamicsWorld.java:741-767): integrateVelocities + applyDamping.
// The predicted transform it computes goes into a temporary and is discarded (CollisionObject.java:230-233).
void stage_predict(World& w, float dt) {
    PhaseTimer pt(w, 1);
    const float MAX_ANGVEL = SIMD_HALF_PI;
    for (Body& b : w.bodies) {
        if (b.isStaticOrKinematic() || !b.isActive()) continue;
        // RigidBody.integrateVelocities (dynamics/RigidBody.java:323-342)
        b.linvel.x += b.invMass * dt * b.totalForce.x;
        b.linvel.y += b.invMass * dt * b.totalForce.y;
        b.linvel.z += b.invMass * dt * b.totalForce.z;
        V3 tmp = scl(mulMv(b.totalTorque, b.invInertiaWorld), dt);
        b.angvel = add(b.angvel, tmp);
        float angvel = len(b.angvel);
        if (angvel * dt > MAX_ANGVEL) b.angvel = scl(b.angvel, (MAX_ANGVEL / dt) / angvel);
        // RigidBody.applyDamping (dynamics/RigidBody.java:246-299), additionalDamping off
        b.linvel = scl(b.linvel, jpow(1.0f - b.linearDamping, dt));
        b.angvel = scl(b.angvel, jpow(1.0f - b.angularDamping, dt));
    }
}

// CollisionWorld.updateAabbs / updateSingleAabb (collision/dispatch/CollisionWorld.java:195-245)
void stage_aabbs(World& w) {
    PhaseTimer pt(w, 2);
    const float t = w.cfg.contactBreakingThreshold;
    for (Body& b : w.bodies) {
        if (!b.isActive()) continue;
        V3 mn, mx;
        shape_aabb(w.shapes[b.shape], b.xf, mn, mx);
        mn = sub(mn, v3(t, t, t));
        mx = add(mx, v3(t, t, t));
        V3 d = sub(mx, mn);
        if (b.isStatic() || (len2(d) < 1e12f)) { b.aabbMin = mn; b.aabbMax = mx; }
        else b.setActivationState(DISABLE_SIMULATION);
    }
}

// DbvtAabbMm.Intersect (collision/broadphase/DbvtAabbMm.java:209-212), inclusive
static inline bool aabb_overlap(const Body& a, const Body& b) {
    return (a.aabbMin.x <= b.aabbMax.x) && (a.aabbMax.x >= b.aabbMin.x) && (a.aabbMin.y <= b.aabbMax.y) &&
           (a.aabbMax.y >= b.aabbMin.y) && (a.aabbMin.z <= b.aabbMax.z) && (a.aabbMax.z >= b.aabbMin.z);
}
// HashedOverlappingPairCache.needsBroadphaseCollision (java:179-188)
static inline bool filter_pass(const Body& a, const Body& b) {
    return a.world == b.world && ((short)a.group & (short)b.mask) != 0 && ((short)b.group & (short)a.mask) != 0;
}

// The pair set the DBVT broadphase holds after collide() (collision/broadphase/DbvtBroadphase.java:89-150):
// every filter-passing pair whose proxy aabbs intersect inclusively.  Found here with a
// median-split box tree over the finite proxies; static planes are tested against all.
namespace {
struct BNode { V3 mn, mx; int left, right, first, count; };
struct BTree {
    std::vector<BNode> nodes;
    std::vector<int> idx;
    const World* w;
    int build(int first, int count) {
        BNode n;
        n.mn = v3(3e38f, 3e38f, 3e38f); n.mx = v3(-3e38f, -3e38f, -3e38f);
        for (int i = first; i < first + count; i++) {
            const Body& b = w->bodies[idx[i]];
            n.mn = v3(std::min(n.mn.x, b.aabbMin.x), std::min(n.mn.y, b.aabbMin.y), std::min(n.mn.z, b.aabbMin.z));
            n.mx = v3(std::max(n.mx.x, b.aabbMax.x), std::max(n.mx.y, b.aabbMax.y), std::max(n.mx.z, b.aabbMax.z));
        }
        n.left = n.right = -1; n.first = first; n.count = count;
        int id = (int)nodes.size();
        nodes.push_back(n);
        if (count > 4) {
            V3 e = sub(n.mx, n.mn);
            int axis = (e.x >= e.y && e.x >= e.z) ? 0 : (e.y >= e.z ? 1 : 2);
            int mid = first + count / 2;
            std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count, [&](int a, int b) {
                const Body& A = w->bodies[a]; const Body& B = w->bodies[b];
                float ca = coord(A.aabbMin, axis) + coord(A.aabbMax, axis), cb = coord(B.aabbMin, axis) + coord(B.aabbMax, axis);
                return ca < cb || (ca == cb && a < b);
            });
            int l = build(first, mid - first);
            int r = build(mid, first + count - mid);
            nodes[id].left = l; nodes[id].right = r;
        }
        return id;
    }
};
}  // namespace

void stage_pairs(World& w) {
    PhaseTimer pt(w, 3);
    const int n = (int)w.bodies.size();
    std::vector<uint64_t> keys;
    std::vector<int> planes, finite;
    for (int i = 0; i < n; i++) (is_listed(w, i) ? planes : finite).push_back(i);
    if (w.bruteForcePairs) {   // SimpleBroadphase.calculateOverlappingPairs-style O(n^2) (SimpleBroadphase.java:87-110)
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++)
                if (!(is_listed(w, i) && is_listed(w, j)) && aabb_overlap(w.bodies[i], w.bodies[j]) && filter_pass(w.bodies[i], w.bodies[j]))
                    push_pair(w, keys, i, j);
    } else {
        for (int p : planes)
            for (int j = 0; j < n; j++)
                if (j != p && !is_listed(w, j) && aabb_overlap(w.bodies[p], w.bodies[j]) && filter_pass(w.bodies[p], w.bodies[j]))
                    push_pair(w, keys, p, j);
        if (!finite.empty()) {
            BTree t;
            t.w = &w;
            t.idx = finite;
            t.nodes.reserve(2 * finite.size() / 4 + 8);
            t.build(0, (int)finite.size());
            std::vector<int> stack;
            for (int i : finite) {
                const Body& bi = w.bodies[i];
                stack.clear();
                stack.push_back(0);
                while (!stack.empty()) {
                    const BNode& nd = t.nodes[stack.back()];
                    stack.pop_back();
                    if (!(bi.aabbMin.x <= nd.mx.x && bi.aabbMax.x >= nd.mn.x && bi.aabbMin.y <= nd.mx.y &&
                          bi.aabbMax.y >= nd.mn.y && bi.aabbMin.z <= nd.mx.z && bi.aabbMax.z >= nd.mn.z)) continue;
                    if (nd.left < 0) {
                        for (int k = nd.first; k < nd.first + nd.count; k++) {
                            int j = t.idx[k];
                            if (j > i && aabb_overlap(bi, w.bodies[j]) && filter_pass(bi, w.bodies[j])) push_pair(w, keys, i, j);
                        }
                    } else {
                        stack.push_back(nd.left);
                        stack.push_back(nd.right);
                    }
                }
            }
        }
    }
    std::sort(keys.begin(), keys.end());
    // carry algorithms/manifolds of pairs that persist; others are released
    // (HashedOverlappingPairCache.removeOverlappingPair -> cleanOverlappingPair, java:77-177,222-228)
    std::vector<uint8_t> has(keys.size(), 0);
    std::vector<Manifold> mf(keys.size());
    size_t o = 0;
    for (size_t k = 0; k < keys.size(); k++) {
        while (o < w.pairKeys.size() && w.pairKeys[o] < keys[k]) o++;
        if (o < w.pairKeys.size() && w.pairKeys[o] == keys[k]) { has[k] = w.pairHasAlgo[o]; mf[k] = w.pairMf[o]; }
    }
    w.pairKeys.swap(keys);
    w.pairHasAlgo.swap(has);
    w.pairMf.swap(mf);
    w.counters.pairs = (int)w.pairKeys.size();
}

// CollisionDispatcher.dispatchAllCollisionPairs (collision/dispatch/CollisionDispatcher.java:252-257)
void stage_narrowphase(World& w) {
    PhaseTimer pt(w, 4);
    w.counters.gjk = 0;
    w.counters.epa = 0;
    for (size_t i = 0; i < w.pairKeys.size(); i++) process_pair(w, (int)i);
    int nm = 0, nc = 0;
    for (size_t i = 0; i < w.pairKeys.size(); i++) if (w.pairHasAlgo[i]) { nm++; nc += w.pairMf[i].n; }
    w.counters.manifolds = nm;
    w.counters.contacts = nc;
}

// ---------------------------------------------------------------------------------------
// UnionFind (collision/dispatch/UnionFind.java:55-143), path-compressing find
namespace {
struct UF {
    std::vector<int> id, sz;
    void reset(int n) { id.resize(n); sz.assign(n, 1); for (int i = 0; i < n; i++) id[i] = i; }
    int find(int x) { while (x != id[x]) { id[x] = id[id[x]]; x = id[x]; } return x; }
    void unite(int p, int q) { int i = find(p), j = find(q); if (i == j) return; id[i] = j; sz[j] += sz[i]; }
};
// MiscUtil.quickSortInternal (linearmath/MiscUtil.java:187-209)
template <class T, class C> static void quick_sort(std::vector<T>& a, int lo, int hi, C cmp) {
    int i = lo, j = hi;
    T x = a[(lo + hi) / 2];
    do {
        while (cmp(a[i], x) < 0) i++;
        while (cmp(x, a[j]) < 0) j--;
        if (i <= j) { std::swap(a[i], a[j]); i++; j--; }
    } while (i <= j);
    if (lo < j) quick_sort(a, lo, j, cmp);
    if (i < hi) quick_sort(a, i, hi, cmp);
}
}  // namespace

static std::vector<int> g_islandManifolds;    // islandmanifold of the last ISLANDS stage (pair indices)
static std::vector<int> g_jointIsland;   // per joint: its processed island, -1 when not solved this step

// calculateSimulationIslands + SimulationIslandManager.buildIslands
// (dynamics/DiscreteDynamicsWorld.java:649-677; collision/dispatch/SimulationIslandManager.java:57-240)
void stage_islands(World& w) {
    PhaseTimer pt(w, 5);
    const int n = (int)w.bodies.size();
    UF uf;
    uf.reset(n);
    for (int i = 0; i < n; i++) { w.bodies[i].islandTag = i; w.bodies[i].companionId = -1; }
    for (size_t k = 0; k < w.pairKeys.size(); k++) {   // findUnions over the pair array
        int a = key_owner(w.pairKeys[k]), b = key_partner(w.pairKeys[k]);
        int lo = a < b ? a : b, hi = a < b ? b : a;
        if (w.bodies[lo].mergesIslands() && w.bodies[hi].mergesIslands()) uf.unite(w.bodies[lo].islandTag, w.bodies[hi].islandTag);
    }
    // calculateSimulationIslands (DiscreteDynamicsWorld.java:649-677): joints between two
    // dynamic bodies, at least one active, join their islands
    for (const Joint& j : w.joints) {
        if (j.b < 0) continue;
        const Body& A = w.bodies[j.a];
        const Body& B = w.bodies[j.b];
        if (!A.isStaticOrKinematic() && !B.isStaticOrKinematic() && (A.isActive() || B.isActive()))
            uf.unite(A.islandTag, B.islandTag);
    }
    for (int i = 0; i < n; i++) {   // storeIslandActivationState
        Body& b = w.bodies[i];
        if (!b.isStaticOrKinematic()) { b.islandTag = uf.find(i); b.companionId = -1; }
        else { b.islandTag = -1; b.companionId = -2; }
    }
    // per island: sleep if no member is ACTIVE_TAG or DISABLE_DEACTIVATION, else wake sleepers
    std::vector<uint8_t> keepAwake(n, 0), hasMember(n, 0);
    for (int i = 0; i < n; i++) {
        const Body& b = w.bodies[i];
        if (b.islandTag < 0) continue;
        hasMember[b.islandTag] = 1;
        if (b.activation == ACTIVE_TAG || b.activation == DISABLE_DEACTIVATION) keepAwake[b.islandTag] = 1;
    }
    int islands = 0;
    for (int i = 0; i < n; i++) islands += hasMember[i];
    w.counters.islands = islands;
    for (int i = 0; i < n; i++) {
        Body& b = w.bodies[i];
        if (b.islandTag < 0) continue;
        if (!keepAwake[b.islandTag]) b.setActivationState(ISLAND_SLEEPING);
        else if (b.activation == ISLAND_SLEEPING) b.setActivationState(WANTS_DEACTIVATION);
    }
    // islandmanifold: manifolds with a non-sleeping body that need a response
    g_islandManifolds.clear();
    for (size_t k = 0; k < w.pairKeys.size(); k++) {
        if (!w.pairHasAlgo[k]) continue;
        const Manifold& m = w.pairMf[k];
        const Body& b0 = w.bodies[m.body0];
        const Body& b1 = w.bodies[m.body1];
        if (b0.activation != ISLAND_SLEEPING || b1.activation != ISLAND_SLEEPING) {
            bool resp = b0.hasContactResponse() && b1.hasContactResponse() && (!b0.isStaticOrKinematic() || !b1.isStaticOrKinematic());
            if (resp) g_islandManifolds.push_back((int)k);
        }
    }
    // islands whose members are all active are processed (SimulationIslandManager.java:283-296)
    std::vector<uint8_t> inactive(n, 0);
    for (int i = 0; i < n; i++) if (w.bodies[i].islandTag >= 0 && !w.bodies[i].isActive()) inactive[w.bodies[i].islandTag] = 1;
    w.solveList.clear();
    for (int k : g_islandManifolds) {
        const Manifold& m = w.pairMf[k];
        int isl = w.bodies[m.body0].islandTag >= 0 ? w.bodies[m.body0].islandTag : w.bodies[m.body1].islandTag;
        if (!inactive[isl]) w.solveList.push_back(k);
    }
    // joints of processed islands (DiscreteDynamicsWorld.getConstraintIslandId, java:549-557)
    g_jointIsland.assign(w.joints.size(), -1);
    for (size_t k = 0; k < w.joints.size(); k++) {
        const Joint& j = w.joints[k];
        const int ta = w.bodies[j.a].islandTag, tb = j.b >= 0 ? w.bodies[j.b].islandTag : -1;
        const int isl = ta >= 0 ? ta : tb;
        if (isl >= 0 && !inactive[isl]) g_jointIsland[k] = isl;
    }
}

std::vector<int> joint_colour_order(const World& w) {
    const size_t n = w.joints.size();
    std::vector<std::vector<int>> used(w.bodies.size());
    std::vector<std::pair<int, int>> ck(n);
    auto dynBody = [&](int b) { return b >= 0 && !w.bodies[b].isStaticOrKinematic(); };
    for (size_t k = 0; k < n; k++) {
        const Joint& j = w.joints[k];
        int c = 0;
        for (;; c++) {
            bool clash = false;
            for (int b : {j.a, j.b})
                if (dynBody(b))
                    for (int u : used[b]) clash = clash || u == c;
            if (!clash) break;
        }
        for (int b : {j.a, j.b})
            if (dynBody(b)) used[b].push_back(c);
        ck[k] = {c, (int)k};
    }
    std::sort(ck.begin(), ck.end());
    std::vector<int> order(n);
    for (size_t k = 0; k < n; k++) order[k] = ck[k].second;
    return order;
}

// ---------------------------------------------------------------------------------------
// SequentialImpulseConstraintSolver (dynamics/constraintsolver/SequentialImpulseConstraintSolver.java)
namespace {
struct SolverBody {   // dynamics/constraintsolver/SolverBody.java:36-119
    V3 angvel, linvel, angularFactor, linearFactor;
    float invMass;
    int original;
    void apply(V3 lin, V3 ang, float imp) {   // internalApplyImpulse
        if (invMass != 0.0f) {
            linvel.x += imp * linearFactor.x * lin.x;
            linvel.y += imp * linearFactor.y * lin.y;
            linvel.z += imp * linearFactor.z * lin.z;
            angvel.x += imp * angularFactor.x * ang.x;
            angvel.y += imp * angularFactor.y * ang.y;
            angvel.z += imp * angularFactor.z * ang.z;
        }
    }
};
struct Row {          // dynamics/constraintsolver/SolverConstraint.java:34-58
    V3 rp1xn, normal, rp2xn, angA, angB;
    float pushImpulse = 0, impulse = 0, friction = 0, restitution = 0, jacDiagABInv = 0, penetration = 0;
    int bodyA = -1, bodyB = -1, frictionIndex = -1;
    int mfPair = -1, mfPoint = -1;
};
}  // namespace

// TypedConstraint's fixed body (TypedConstraint.java:44-49): static, identity transform.
static Body fixed_body() {
    Body b;
    b.xf = xf_identity();
    b.invInertiaWorld = m3_identity();
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) b.invInertiaWorld.m[r][c] = 0.0f;
    b.flags = CF_STATIC_OBJECT;
    return b;
}

// RigidBody.applyImpulse (dynamics/RigidBody.java:401-417): applyCentralImpulse, then the
// torque impulse rel_pos x impulse through the world inverse inertia.
static void apply_impulse(Body& b, V3 impulse, V3 relPos) {
    if (b.invMass == 0.0f) return;
    V3 si = v3(impulse.x * b.linearFactor.x, impulse.y * b.linearFactor.y, impulse.z * b.linearFactor.z);
    b.linvel = add(b.linvel, scl(si, b.invMass));
    V3 t = crs(relPos, v3(impulse.x * b.linearFactor.x, impulse.y * b.linearFactor.y, impulse.z * b.linearFactor.z));
    t.x *= b.angularFactor.x;
    t.y *= b.angularFactor.y;
    t.z *= b.angularFactor.z;
    b.angvel = add(b.angvel, mulMv(t, b.invInertiaWorld));
}

// Point2PointConstraint.buildJacobian (java:72-101) with JacobianEntry.init (JacobianEntry.java:
// 63-78).  The port's `bJ.set(rel_pos2).crs(bJ)` crosses rel_pos2 with itself, so the B-side
// angular Jacobian is the zero vector: kept, as the reference computes it.
static void joint_build(Joint& j, const Body& A, const Body& B) {
    j.appliedImpulse = 0.0f;
    V3 normal = v3(0, 0, 0);
    for (int i = 0; i < 3; i++) {
        set_coord(normal, i, 1.0f);
        M3 w2A = transpose(A.xf.b), w2B = transpose(B.xf.b);
        V3 r1 = sub(xf_apply(A.xf, j.pivotA), A.xf.o);
        V3 r2 = sub(xf_apply(B.xf, j.pivotB), B.xf.o);
        V3 aJ = mulMv(crs(r1, normal), w2A);
        V3 bJ = mulMv(crs(r2, r2), w2B);
        V3 m0 = v3(A.invInertiaLocal.x * aJ.x, A.invInertiaLocal.y * aJ.y, A.invInertiaLocal.z * aJ.z);
        V3 m1 = v3(B.invInertiaLocal.x * bJ.x, B.invInertiaLocal.y * bJ.y, B.invInertiaLocal.z * bJ.z);
        j.adiag[i] = A.invMass + dot(m0, aJ) + B.invMass + dot(m1, bJ);
        set_coord(normal, i, 0.0f);
    }
}

// Point2PointConstraint.solveConstraint (java:103-171): per axis, the positional error and the
// relative velocity at the pivots give an impulse applied to both bodies.
static void joint_solve(Joint& j, Body& A, Body& B, float timeStep) {
    V3 pA = xf_apply(A.xf, j.pivotA), pB = xf_apply(B.xf, j.pivotB);
    V3 normal = v3(0, 0, 0);
    for (int i = 0; i < 3; i++) {
        set_coord(normal, i, 1.0f);
        float jacDiagABInv = 1.0f / j.adiag[i];
        V3 r1 = sub(pA, A.xf.o), r2 = sub(pB, B.xf.o);
        V3 vel1 = add(crs(A.angvel, r1), A.linvel);   // RigidBody.getVelocityInLocalPoint
        V3 vel2 = add(crs(B.angvel, r2), B.linvel);
        V3 vel = sub(vel1, vel2);
        float relVel = dot(normal, vel);
        float depth = -dot(sub(pA, pB), normal);
        float impulse = depth * j.tau / timeStep * jacDiagABInv - j.damping * relVel * jacDiagABInv;
        if (j.impulseClamp > 0.0f) {
            if (impulse < -j.impulseClamp) impulse = -j.impulseClamp;
            if (impulse > j.impulseClamp) impulse = j.impulseClamp;
        }
        j.appliedImpulse += impulse;
        V3 iv = scl(normal, impulse);
        apply_impulse(A, iv, sub(pA, A.xf.o));
        apply_impulse(B, scl(iv, -1.0f), sub(pB, B.xf.o));
        set_coord(normal, i, 0.0f);
    }
}

// ScalarUtil.atan2Fast (linearmath/ScalarUtil.java:43-57): a first-order approximation.
static float atan2_fast(float y, float x) {
    const float c1 = SIMD_PI / 4.0f, c2 = 3.0f * c1;
    const float ay = std::fabs(y);
    float angle;
    if (x >= 0.0f) {
        float r = (x - ay) / (x + ay);
        angle = c1 - c1 * r;
    } else {
        float r = (x + ay) / (ay - x);
        angle = c2 - c1 * r;
    }
    return y < 0.0f ? -angle : angle;
}

static V3 col(const M3& m, int c) { return v3(m.m[0][c], m.m[1][c], m.m[2][c]); }

// RigidBody.computeAngularImpulseDenominator (dynamics/RigidBody.java:534-541)
static float ang_denom(const Body& b, V3 axis) { return dot(axis, mulMTv(axis, b.invInertiaWorld)); }

// RigidBody.applyTorqueImpulse (dynamics/RigidBody.java:405-411): no mass check; a static
// body's zero inverse inertia leaves its angular velocity as it is.
static void apply_torque(Body& b, V3 t) { b.angvel = add(b.angvel, mulMv(t, b.invInertiaWorld)); }

// HingeConstraint.getHingeAngle (HingeConstraint.java:535-555)
static float hinge_angle(const Joint& j, const Body& A, const Body& B) {
    V3 ref0 = mulMv(col(j.frameA, 0), A.xf.b);
    V3 ref1 = mulMv(col(j.frameA, 1), A.xf.b);
    V3 swing = mulMv(col(j.frameB, 1), B.xf.b);
    return atan2_fast(dot(swing, ref0), dot(swing, ref1));
}

// HingeConstraint.buildJacobian (HingeConstraint.java:240-340): three linear rows along the
// pivots' separation and its plane space (JacobianEntry.init, with the port's zero B-side
// angular Jacobian), the limit state from the hinge angle and kHinge = 1 / (J W J') about
// the hinge axis.  The angular JacobianEntries it also builds are never read by the solve.
static void hinge_build(Joint& j, const Body& A, const Body& B) {
    j.appliedImpulse = 0.0f;
    if (!j.angularOnly) {
        V3 pA = xf_apply(A.xf, j.pivotA), pB = xf_apply(B.xf, j.pivotB);
        V3 relPos = sub(pB, pA);
        if (len2(relPos) > FLT_EPS) j.normal[0] = nor(relPos);
        else j.normal[0] = v3(1.0f, 0.0f, 0.0f);
        plane_space1(j.normal[0], j.normal[1], j.normal[2]);
        for (int i = 0; i < 3; i++) {
            M3 w2A = transpose(A.xf.b), w2B = transpose(B.xf.b);
            V3 r1 = sub(pA, A.xf.o), r2 = sub(pB, B.xf.o);
            V3 aJ = mulMv(crs(r1, j.normal[i]), w2A);
            V3 bJ = mulMv(crs(r2, r2), w2B);
            V3 m0 = mulc(A.invInertiaLocal, aJ), m1 = mulc(B.invInertiaLocal, bJ);
            j.adiag[i] = A.invMass + dot(m0, aJ) + B.invMass + dot(m1, bJ);
        }
    }
    float angle = hinge_angle(j, A, B);
    j.correction = 0.0f;
    j.limitSign = 0.0f;
    j.solveLimit = false;
    j.accLimitImpulse = 0.0f;
    if (j.lowerLimit < j.upperLimit) {
        if (angle <= j.lowerLimit * j.limitSoftness) {
            j.correction = j.lowerLimit - angle;
            j.limitSign = 1.0f;
            j.solveLimit = true;
        } else if (angle >= j.upperLimit * j.limitSoftness) {
            j.correction = j.upperLimit - angle;
            j.limitSign = -1.0f;
            j.solveLimit = true;
        }
    }
    V3 axisA = mulMv(col(j.frameA, 2), A.xf.b);
    j.kHinge = 1.0f / (ang_denom(A, axisA) + ang_denom(B, axisA));
}

// HingeConstraint.solveConstraint (HingeConstraint.java:342-533): the linear rows (tau 0.3,
// the pivots' relative velocity taken once before the three rows), then the angular part on
// the angular velocities as they stand after it: the relative angular velocity orthogonal to
// the hinge axes and the axes' misalignment removed by torque impulses, the limit with its
// clamped accumulated impulse, the motor clipped per solve.
static void hinge_solve(Joint& j, Body& A, Body& B, float timeStep) {
    V3 pA = xf_apply(A.xf, j.pivotA), pB = xf_apply(B.xf, j.pivotB);
    const float tau = 0.3f;
    if (!j.angularOnly) {
        V3 r1 = sub(pA, A.xf.o), r2 = sub(pB, B.xf.o);
        V3 vel = sub(add(crs(A.angvel, r1), A.linvel), add(crs(B.angvel, r2), B.linvel));
        for (int i = 0; i < 3; i++) {
            V3 n = j.normal[i];
            float jacDiagABInv = 1.0f / j.adiag[i];
            float relVel = dot(n, vel);
            float depth = -dot(sub(pA, pB), n);
            float impulse = depth * tau / timeStep * jacDiagABInv - relVel * jacDiagABInv;
            j.appliedImpulse += impulse;
            V3 iv = scl(n, impulse);
            apply_impulse(A, iv, sub(pA, A.xf.o));
            apply_impulse(B, scl(iv, -1.0f), sub(pB, B.xf.o));
        }
    }
    V3 axisA = mulMv(col(j.frameA, 2), A.xf.b);
    V3 axisB = mulMv(col(j.frameB, 2), B.xf.b);
    V3 angVelA = A.angvel, angVelB = B.angvel;
    V3 aroundA = scl(axisA, dot(axisA, angVelA));
    V3 aroundB = scl(axisB, dot(axisB, angVelB));
    V3 velrelOrthog = sub(sub(angVelA, aroundA), sub(angVelB, aroundB));
    const float relaxation = 1.0f;
    if (len(velrelOrthog) > 0.00001f) {
        V3 n = nor(velrelOrthog);
        float denom = ang_denom(A, n) + ang_denom(B, n);
        velrelOrthog = scl(velrelOrthog, (1.0f / denom) * j.relaxationFactor);
    }
    V3 angularError = scl(scl(crs(axisA, axisB), -1.0f), 1.0f / timeStep);
    if (len(angularError) > 0.00001f) {
        V3 n2 = nor(angularError);
        float denom2 = ang_denom(A, n2) + ang_denom(B, n2);
        angularError = scl(angularError, (1.0f / denom2) * relaxation);
    }
    apply_torque(A, add(scl(velrelOrthog, -1.0f), angularError));
    apply_torque(B, sub(velrelOrthog, angularError));
    if (j.solveLimit) {
        float amplitude = (dot(sub(angVelB, angVelA), axisA) * j.relaxationFactor + j.correction * (1.0f / timeStep) * j.biasFactor) * j.limitSign;
        float impulseMag = amplitude * j.kHinge;
        float temp = j.accLimitImpulse;
        j.accLimitImpulse = jmax(j.accLimitImpulse + impulseMag, 0.0f);
        impulseMag = j.accLimitImpulse - temp;
        V3 imp = scl(axisA, impulseMag * j.limitSign);
        apply_torque(A, imp);
        apply_torque(B, scl(imp, -1.0f));
    }
    if (j.enableMotor) {
        const V3 angularLimit = v3(0.0f, 0.0f, 0.0f);
        float projRelVel = dot(sub(aroundA, aroundB), axisA);
        float motorRelVel = j.motorTarget - projRelVel;
        float unclipped = j.kHinge * motorRelVel;
        float clipped = unclipped > j.maxMotorImpulse ? j.maxMotorImpulse : unclipped;
        clipped = clipped < -j.maxMotorImpulse ? -j.maxMotorImpulse : clipped;
        V3 motorImp = scl(axisA, clipped);
        apply_torque(A, add(motorImp, angularLimit));
        apply_torque(B, sub(scl(motorImp, -1.0f), angularLimit));
    }
}

// Generic6DofConstraint.matrixToEulerXYZ (Generic6DofConstraint.java:125-159): element `index`
// is row index % 3, column index / 3; atan2 / asin in double, rounded to float.
static V3 matrix_to_euler_xyz(const M3& m) {
    auto e = [&](int index) { return m.m[index % 3][index / 3]; };
    V3 xyz;
    if (e(2) < 1.0f) {
        if (e(2) > -1.0f) {
            xyz.x = (float)std::atan2((double)-e(5), (double)e(8));
            xyz.y = (float)std::asin((double)e(2));
            xyz.z = (float)std::atan2((double)-e(1), (double)e(0));
        } else {
            xyz.x = -(float)std::atan2((double)e(3), (double)e(4));
            xyz.y = -SIMD_HALF_PI;
            xyz.z = 0.0f;
        }
    } else {
        xyz.x = (float)std::atan2((double)e(3), (double)e(4));
        xyz.y = SIMD_HALF_PI;
        xyz.z = 0.0f;
    }
    return xyz;
}

// RotationalLimitMotor.testLimitValue (RotationalLimitMotor.java:110-130)
static void rot_test_limit(RotMotor& m, float v) {
    if (m.loLimit > m.hiLimit) { m.currentLimit = 0; return; }
    if (v < m.loLimit) { m.currentLimit = 1; m.currentLimitError = v - m.loLimit; return; }
    if (v > m.hiLimit) { m.currentLimit = 2; m.currentLimitError = v - m.hiLimit; return; }
    m.currentLimit = 0;
}
static bool rot_need_torques(const RotMotor& m) { return !(m.currentLimit == 0 && !m.enableMotor); }

// Generic6DofConstraint.buildJacobian (java:275-323): accumulators cleared, calculateTransforms
// and calculateAngleInfo (relative Euler angles, the three constraint axes), calcAnchorPos, the
// linear rows of the limited axes (JacobianEntry.init with the port's zero B-side angular part)
// and the angular rows of the axes whose motor or limit applies.
static void d6_build(Joint& j, const Body& A, const Body& B) {
    j.linAcc = v3(0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 3; i++) j.rot[i].accumulatedImpulse = 0.0f;
    Xf fA, fB;
    fA.b = j.frameA; fA.o = j.pivotA;
    fB.b = j.frameB; fB.o = j.pivotB;
    j.calcA = xf_mul(A.xf, fA);
    j.calcB = xf_mul(B.xf, fB);
    M3 rel = mulMM(m3_invert(j.calcA.b), j.calcB.b);
    j.angleDiff = matrix_to_euler_xyz(rel);
    V3 axis0 = col(j.calcB.b, 0), axis2 = col(j.calcA.b, 2);
    j.calcAxis[1] = crs(axis2, axis0);
    j.calcAxis[0] = crs(j.calcAxis[1], axis2);
    j.calcAxis[2] = crs(axis0, j.calcAxis[1]);
    float imA = A.invMass, imB = B.invMass;
    float weight = imB == 0.0f ? 1.0f : imA / (imA + imB);
    j.anchor = add(scl(j.calcA.o, weight), scl(j.calcB.o, 1.0f - weight));
    M3 w2A = transpose(A.xf.b), w2B = transpose(B.xf.b);
    for (int i = 0; i < 3; i++) {
        if (!(coord(j.linUpper, i) >= coord(j.linLower, i))) continue;
        V3 n = col(j.useLinearReferenceFrameA ? j.calcA.b : j.calcB.b, i);
        V3 r1 = sub(j.anchor, A.xf.o), r2 = sub(j.anchor, B.xf.o);
        V3 aJ = mulMv(crs(r1, n), w2A);
        V3 bJ = mulMv(crs(r2, r2), w2B);
        V3 m0 = mulc(A.invInertiaLocal, aJ), m1 = mulc(B.invInertiaLocal, bJ);
        j.adiag[i] = A.invMass + dot(m0, aJ) + B.invMass + dot(m1, bJ);
    }
    for (int i = 0; i < 3; i++) {
        rot_test_limit(j.rot[i], coord(j.angleDiff, i));
        if (!rot_need_torques(j.rot[i])) continue;
        V3 aJ = mulMv(j.calcAxis[i], w2A);
        V3 bJ = mulMv(scl(j.calcAxis[i], -1.0f), w2B);
        V3 m0 = mulc(A.invInertiaLocal, aJ), m1 = mulc(B.invInertiaLocal, bJ);
        j.adiagAng[i] = dot(m0, aJ) + dot(m1, bJ);
    }
}

// Generic6DofConstraint.solveConstraint (java:325-365) with
// TranslationalLimitMotor.solveLinearAxis (TranslationalLimitMotor.java:70-150) and
// RotationalLimitMotor.solveAngularLimits (RotationalLimitMotor.java:135-203).
static void d6_solve(Joint& j, Body& A, Body& B, float timeStep) {
    const V3 pointInA = j.calcA.o, pointInB = j.calcB.o;
    for (int i = 0; i < 3; i++) {
        if (!(coord(j.linUpper, i) >= coord(j.linLower, i))) continue;
        float jacDiagABInv = 1.0f / j.adiag[i];
        V3 axis = col(j.useLinearReferenceFrameA ? j.calcA.b : j.calcB.b, i);
        V3 r1 = sub(j.anchor, A.xf.o), r2 = sub(j.anchor, B.xf.o);
        V3 vel = sub(add(crs(A.angvel, r1), A.linvel), add(crs(B.angvel, r2), B.linvel));
        float relVel = dot(axis, vel);
        float depth = -dot(sub(pointInA, pointInB), axis);
        float lo = -1e30f, hi = 1e30f;
        float minLimit = coord(j.linLower, i), maxLimit = coord(j.linUpper, i);
        if (minLimit < maxLimit) {
            if (depth > maxLimit) { depth -= maxLimit; lo = 0.0f; }
            else if (depth < minLimit) { depth -= minLimit; hi = 0.0f; }
            else continue;
        }
        float normalImpulse = j.linSoftness * (j.linRestitution * depth / timeStep - j.linDamping * relVel) * jacDiagABInv;
        float old = coord(j.linAcc, i);
        float sum = old + normalImpulse;
        set_coord(j.linAcc, i, sum > hi ? 0.0f : (sum < lo ? 0.0f : sum));
        normalImpulse = coord(j.linAcc, i) - old;
        V3 iv = scl(axis, normalImpulse);
        apply_impulse(A, iv, r1);
        apply_impulse(B, scl(iv, -1.0f), r2);
    }
    for (int i = 0; i < 3; i++) {
        RotMotor& m = j.rot[i];
        if (!rot_need_torques(m)) continue;
        V3 axis = j.calcAxis[i];
        float jacDiagABInv = 1.0f / j.adiagAng[i];
        float targetVelocity = m.targetVelocity, maxMotorForce = m.maxMotorForce;
        if (m.currentLimit != 0) {
            targetVelocity = -m.ERP * m.currentLimitError / timeStep;
            maxMotorForce = m.maxLimitForce;
        }
        maxMotorForce *= timeStep;
        float relVel = dot(axis, sub(A.angvel, B.angvel));
        float motorRelVel = m.limitSoftness * (targetVelocity - m.damping * relVel);
        if (motorRelVel < FLT_EPS && motorRelVel > -FLT_EPS) continue;
        float unclipped = (1.0f + m.bounce) * motorRelVel * jacDiagABInv;
        float clipped;
        if (unclipped > 0.0f) clipped = unclipped > maxMotorForce ? maxMotorForce : unclipped;
        else clipped = unclipped < -maxMotorForce ? -maxMotorForce : unclipped;
        const float lo = -1e30f, hi = 1e30f;
        float old = m.accumulatedImpulse;
        float sum = old + clipped;
        m.accumulatedImpulse = sum > hi ? 0.0f : (sum < lo ? 0.0f : sum);
        clipped = m.accumulatedImpulse - old;
        V3 motorImp = scl(axis, clipped);
        apply_torque(A, motorImp);
        apply_torque(B, scl(motorImp, -1.0f));
    }
}

// ConeTwistConstraint.buildJacobian (ConeTwistConstraint.java:111-265): the hinge's linear rows,
// the swing angles about A's frame axes 1 and 2 (atan2Fast damped by the "fact" factor) against
// the elliptic cone of the two swing spans, the twist about the frames' x axes from
// shortestArcQuat / quatRotate.  For a swing span below 0.05 the reference reads a stack vector it
// never set (Stack.allocVector3 does not clear it); here that axis is A's frame axis.
static void cone_build(Joint& j, const Body& A, const Body& B) {
    j.appliedImpulse = 0.0f;
    j.swingCorrection = 0.0f;
    j.solveTwist = false;
    j.solveSwing = false;
    j.accTwist = 0.0f;
    j.accSwing = 0.0f;
    if (!j.angularOnly) {
        V3 pA = xf_apply(A.xf, j.pivotA), pB = xf_apply(B.xf, j.pivotB);
        V3 relPos = sub(pB, pA);
        if (len2(relPos) > FLT_EPS) j.normal[0] = nor(relPos);
        else j.normal[0] = v3(1.0f, 0.0f, 0.0f);
        plane_space1(j.normal[0], j.normal[1], j.normal[2]);
        for (int i = 0; i < 3; i++) {
            M3 w2A = transpose(A.xf.b), w2B = transpose(B.xf.b);
            V3 r1 = sub(pA, A.xf.o), r2 = sub(pB, B.xf.o);
            V3 aJ = mulMv(crs(r1, j.normal[i]), w2A);
            V3 bJ = mulMv(crs(r2, r2), w2B);
            V3 m0 = mulc(A.invInertiaLocal, aJ), m1 = mulc(B.invInertiaLocal, bJ);
            j.adiag[i] = A.invMass + dot(m0, aJ) + B.invMass + dot(m1, bJ);
        }
    }
    V3 b1Axis1 = mulMv(col(j.frameA, 0), A.xf.b);
    V3 b2Axis1 = mulMv(col(j.frameB, 0), B.xf.b);
    V3 b1Axis2 = mulMv(col(j.frameA, 1), A.xf.b);
    V3 b1Axis3 = mulMv(col(j.frameA, 2), A.xf.b);
    float swing1 = 0.0f, swing2 = 0.0f;
    const float thresh = 10.0f;
    if (j.swingSpan1 >= 0.05f) {
        float swx = dot(b2Axis1, b1Axis1), swy = dot(b2Axis1, b1Axis2);
        swing1 = atan2_fast(swy, swx);
        float fact = (swy * swy + swx * swx) * thresh * thresh;
        fact = fact / (fact + 1.0f);
        swing1 *= fact;
    }
    if (j.swingSpan2 >= 0.05f) {
        float swx = dot(b2Axis1, b1Axis1), swy = dot(b2Axis1, b1Axis3);
        swing2 = atan2_fast(swy, swx);
        float fact = (swy * swy + swx * swx) * thresh * thresh;
        fact = fact / (fact + 1.0f);
        swing2 *= fact;
    }
    float r1sq = 1.0f / (j.swingSpan1 * j.swingSpan1);
    float r2sq = 1.0f / (j.swingSpan2 * j.swingSpan2);
    float ellipse = std::fabs(swing1 * swing1) * r1sq + std::fabs(swing2 * swing2) * r2sq;
    if (ellipse > 1.0f) {
        j.swingCorrection = ellipse - 1.0f;
        j.solveSwing = true;
        V3 t = add(scl(b1Axis2, dot(b2Axis1, b1Axis2)), scl(b1Axis3, dot(b2Axis1, b1Axis3)));
        j.swingAxis = nor(crs(b2Axis1, t));
        float sign = dot(b2Axis1, b1Axis1) >= 0.0f ? 1.0f : -1.0f;
        j.swingAxis = scl(j.swingAxis, sign);
        j.kSwing = 1.0f / (ang_denom(A, j.swingAxis) + ang_denom(B, j.swingAxis));
    }
    if (j.twistSpan >= 0.0f) {
        V3 b2Axis2 = mulMv(col(j.frameB, 1), B.xf.b);
        // QuaternionUtil.shortestArcQuat (linearmath/QuaternionUtil.java:49-68), quatRotate (78-90)
        V3 c = crs(b2Axis1, b1Axis1);
        float d = dot(b2Axis1, b1Axis1);
        Quat q;
        if ((double)d < -1.0 + (double)FLT_EPS) q = quat(0.0f, 1.0f, 0.0f, 0.0f);
        else {
            float sq = jsqrt((1.0f + d) * 2.0f);
            float rs = 1.0f / sq;
            q = quat(c.x * rs, c.y * rs, c.z * rs, sq * 0.5f);
        }
        Quat qw = quat(q.w * b2Axis2.x + q.y * b2Axis2.z - q.z * b2Axis2.y, q.w * b2Axis2.y + q.z * b2Axis2.x - q.x * b2Axis2.z,
                       q.w * b2Axis2.z + q.x * b2Axis2.y - q.y * b2Axis2.x, -q.x * b2Axis2.x - q.y * b2Axis2.y - q.z * b2Axis2.z);
        Quat r = qmul(qw, quat(-q.x, -q.y, -q.z, q.w));
        V3 twistRef = v3(r.x, r.y, r.z);
        float twist = atan2_fast(dot(twistRef, b1Axis3), dot(twistRef, b1Axis2));
        float lockedFreeFactor = j.twistSpan > 0.05f ? j.coneSoftness : 0.0f;
        if (twist <= -j.twistSpan * lockedFreeFactor) {
            j.twistCorrection = -(twist + j.twistSpan);
            j.solveTwist = true;
            j.twistAxis = scl(nor(scl(add(b2Axis1, b1Axis1), 0.5f)), -1.0f);
            j.kTwist = 1.0f / (ang_denom(A, j.twistAxis) + ang_denom(B, j.twistAxis));
        } else if (twist > j.twistSpan * lockedFreeFactor) {
            j.twistCorrection = twist - j.twistSpan;
            j.solveTwist = true;
            j.twistAxis = nor(scl(add(b2Axis1, b1Axis1), 0.5f));
            j.kTwist = 1.0f / (ang_denom(A, j.twistAxis) + ang_denom(B, j.twistAxis));
        }
    }
}

// ConeTwistConstraint.solveConstraint (ConeTwistConstraint.java:267-368): the hinge's linear
// rows, then the swing and twist limits with clamped accumulated impulses, both on the angular
// velocities as the linear rows left them.
static void cone_solve(Joint& j, Body& A, Body& B, float timeStep) {
    V3 pA = xf_apply(A.xf, j.pivotA), pB = xf_apply(B.xf, j.pivotB);
    const float tau = 0.3f;
    if (!j.angularOnly) {
        V3 r1 = sub(pA, A.xf.o), r2 = sub(pB, B.xf.o);
        V3 vel = sub(add(crs(A.angvel, r1), A.linvel), add(crs(B.angvel, r2), B.linvel));
        for (int i = 0; i < 3; i++) {
            V3 n = j.normal[i];
            float jacDiagABInv = 1.0f / j.adiag[i];
            float relVel = dot(n, vel);
            float depth = -dot(sub(pA, pB), n);
            float impulse = depth * tau / timeStep * jacDiagABInv - relVel * jacDiagABInv;
            j.appliedImpulse += impulse;
            V3 iv = scl(n, impulse);
            apply_impulse(A, iv, sub(pA, A.xf.o));
            apply_impulse(B, scl(iv, -1.0f), sub(pB, B.xf.o));
        }
    }
    V3 angVelA = A.angvel, angVelB = B.angvel;
    if (j.solveSwing) {
        float amplitude = dot(sub(angVelB, angVelA), j.swingAxis) * j.relaxationFactor * j.relaxationFactor +
                          j.swingCorrection * (1.0f / timeStep) * j.biasFactor;
        float impulseMag = amplitude * j.kSwing;
        float temp = j.accSwing;
        j.accSwing = jmax(j.accSwing + impulseMag, 0.0f);
        impulseMag = j.accSwing - temp;
        V3 imp = scl(j.swingAxis, impulseMag);
        apply_torque(A, imp);
        apply_torque(B, scl(imp, -1.0f));
    }
    if (j.solveTwist) {
        float amplitude = dot(sub(angVelB, angVelA), j.twistAxis) * j.relaxationFactor * j.relaxationFactor +
                          j.twistCorrection * (1.0f / timeStep) * j.biasFactor;
        float impulseMag = amplitude * j.kTwist;
        float temp = j.accTwist;
        j.accTwist = jmax(j.accTwist + impulseMag, 0.0f);
        impulseMag = j.accTwist - temp;
        V3 imp = scl(j.twistAxis, impulseMag);
        apply_torque(A, imp);
        apply_torque(B, scl(imp, -1.0f));
    }
}

// SliderConstraint.buildJacobianInt (SliderConstraint.java:465-526) with testLinLimits (714-730)
// and testAngLimits (732-756); "A" and "B" are the joint's bodies, swapped when
// useLinearReferenceFrameA is false (buildJacobian, java:175-182).
static void slider_build(Joint& j, const Body& A, const Body& B, const M3& frA, V3 oA, const M3& frB, V3 oB) {
    Xf fA, fB;
    fA.b = frA; fA.o = oA;
    fB.b = frB; fB.o = oB;
    j.calcA = xf_mul(A.xf, fA);
    j.calcB = xf_mul(B.xf, fB);
    V3 pivA = j.calcA.o, pivB = j.calcB.o;
    V3 axis = col(j.calcA.b, 0);
    V3 delta = sub(pivB, pivA);
    V3 proj = v3(pivA.x + dot(axis, delta) * axis.x, pivA.y + dot(axis, delta) * axis.y, pivA.z + dot(axis, delta) * axis.z);
    j.slRelA = sub(proj, A.xf.o);
    j.slRelB = sub(pivB, B.xf.o);
    M3 w2A = transpose(A.xf.b), w2B = transpose(B.xf.b);
    for (int i = 0; i < 3; i++) {
        V3 n = col(j.calcA.b, i);
        V3 aJ = mulMv(crs(j.slRelA, n), w2A);
        V3 bJ = mulMv(crs(j.slRelB, j.slRelB), w2B);
        V3 m0 = mulc(A.invInertiaLocal, aJ), m1 = mulc(B.invInertiaLocal, bJ);
        j.slInv[i] = 1.0f / (A.invMass + dot(m0, aJ) + B.invMass + dot(m1, bJ));
        set_coord(j.slDepth, i, dot(delta, n));
    }
    const SliderParams& P = j.slider;
    j.slSolveLin = false;
    if (P.lowerLin <= P.upperLin) {
        if (j.slDepth.x > P.upperLin) { j.slDepth.x -= P.upperLin; j.slSolveLin = true; }
        else if (j.slDepth.x < P.lowerLin) { j.slDepth.x -= P.lowerLin; j.slSolveLin = true; }
        else j.slDepth.x = 0.0f;
    } else {
        j.slDepth.x = 0.0f;
    }
    j.slAngDepth = 0.0f;
    j.slSolveAng = false;
    if (P.lowerAng <= P.upperAng) {
        V3 a0 = col(j.calcA.b, 1), a1 = col(j.calcA.b, 2), b0 = col(j.calcB.b, 1);
        float rot = (float)std::atan2((double)dot(b0, a1), (double)dot(b0, a0));
        if (rot < P.lowerAng) { j.slAngDepth = rot - P.lowerAng; j.slSolveAng = true; }
        else if (rot > P.upperAng) { j.slAngDepth = rot - P.upperAng; j.slSolveAng = true; }
    }
    j.slKAngle = 1.0f / (ang_denom(A, axis) + ang_denom(B, axis));
    j.slAccLin = 0.0f;
    j.slAccAng = 0.0f;
}

// SliderConstraint.solveConstraintInt (SliderConstraint.java:528-685).
static void slider_solve(Joint& j, Body& A, Body& B, float timeStep) {
    const SliderParams& P = j.slider;
    V3 vel = sub(add(crs(A.angvel, j.slRelA), A.linvel), add(crs(B.angvel, j.slRelB), B.linvel));
    for (int i = 0; i < 3; i++) {
        V3 n = col(j.calcA.b, i);
        float relVel = dot(n, vel);
        float depth = coord(j.slDepth, i);
        int k = i != 0 ? SL_ORTHO_LIN : (j.slSolveLin ? SL_LIM_LIN : SL_DIR_LIN);
        float normalImpulse = P.soft[k] * (P.rest[k] * depth / timeStep - P.damp[k] * relVel) * j.slInv[i];
        V3 iv = scl(n, normalImpulse);
        apply_impulse(A, iv, j.slRelA);
        apply_impulse(B, scl(iv, -1.0f), j.slRelB);
        if (P.linMotor && i == 0 && j.slAccLin < P.linMaxForce) {
            float motorRelVel = P.linTarget + relVel;
            normalImpulse = -motorRelVel * j.slInv[i];
            float newAcc = j.slAccLin + std::fabs(normalImpulse);
            if (newAcc > P.linMaxForce) newAcc = P.linMaxForce;
            float del = newAcc - j.slAccLin;
            normalImpulse = normalImpulse < 0.0f ? -del : del;
            j.slAccLin = newAcc;
            iv = scl(n, normalImpulse);
            apply_impulse(A, iv, j.slRelA);
            apply_impulse(B, scl(iv, -1.0f), j.slRelB);
        }
    }
    V3 axisA = col(j.calcA.b, 0), axisB = col(j.calcB.b, 0);
    V3 angVelA = A.angvel, angVelB = B.angvel;
    V3 aroundA = scl(axisA, dot(axisA, angVelA)), aroundB = scl(axisB, dot(axisB, angVelB));
    V3 velrelOrthog = sub(sub(angVelA, aroundA), sub(angVelB, aroundB));
    if (len(velrelOrthog) > 0.00001f) {
        V3 n = nor(velrelOrthog);
        float denom = ang_denom(A, n) + ang_denom(B, n);
        velrelOrthog = scl(velrelOrthog, (1.0f / denom) * P.damp[SL_ORTHO_ANG] * P.soft[SL_ORTHO_ANG]);
    }
    V3 angularError = scl(crs(axisA, axisB), 1.0f / timeStep);
    if (len(angularError) > 0.00001f) {
        V3 n2 = nor(angularError);
        float denom2 = ang_denom(A, n2) + ang_denom(B, n2);
        angularError = scl(angularError, (1.0f / denom2) * P.rest[SL_ORTHO_ANG] * P.soft[SL_ORTHO_ANG]);
    }
    apply_torque(A, add(scl(velrelOrthog, -1.0f), angularError));
    apply_torque(B, sub(velrelOrthog, angularError));
    int k = j.slSolveAng ? SL_LIM_ANG : SL_DIR_ANG;
    float impulseMag = dot(sub(angVelB, angVelA), axisA) * P.damp[k] + j.slAngDepth * P.rest[k] / timeStep;
    impulseMag *= j.slKAngle * P.soft[k];
    V3 imp = scl(axisA, impulseMag);
    apply_torque(A, imp);
    apply_torque(B, scl(imp, -1.0f));
    if (P.angMotor && j.slAccAng < P.angMaxForce) {
        float projRelVel = dot(sub(aroundA, aroundB), axisA);
        float motorRelVel = P.angTarget - projRelVel;
        float angImpulse = j.slKAngle * motorRelVel;
        float newAcc = j.slAccAng + std::fabs(angImpulse);
        if (newAcc > P.angMaxForce) newAcc = P.angMaxForce;
        float del = newAcc - j.slAccAng;
        angImpulse = angImpulse < 0.0f ? -del : del;
        j.slAccAng = newAcc;
        V3 mi = scl(axisA, angImpulse);
        apply_torque(A, mi);
        apply_torque(B, scl(mi, -1.0f));
    }
}

static void solve_group(World& w, const std::vector<int>& manifolds, const std::vector<int>& joints, float dt) {
    const Config& cfg = w.cfg;
    std::vector<SolverBody> sb;
    std::vector<Row> rows, frows;
    sb.reserve(manifolds.size() * 2);
    auto init_sb = [&](int bi) {   // initSolverBody (java:151-177)
        const Body& b = w.bodies[bi];
        SolverBody s;
        s.angvel = b.angvel;
        s.invMass = b.invMass;
        s.linvel = b.linvel;
        s.original = bi;
        s.angularFactor = b.angularFactor;
        s.linearFactor = b.linearFactor;
        sb.push_back(s);
        return (int)sb.size() - 1;
    };
    auto get_sb = [&](int bi) {
        Body& b = w.bodies[bi];
        if (b.islandTag >= 0) {
            if (b.companionId >= 0) return b.companionId;
            int id = init_sb(bi);
            b.companionId = id;
            return id;
        }
        return init_sb(bi);   // static body: a private solver body per manifold
    };
    // addFrictionConstraint (java:349-416)
    auto add_friction = [&](V3 normalAxis, int sbA, int sbB, int frictionIndex, const ManifoldPoint& cp, V3 rp1, V3 rp2,
                            const Body& b0, const Body& b1) {
        Row r;
        r.normal = normalAxis;
        r.bodyA = sbA; r.bodyB = sbB;
        r.frictionIndex = frictionIndex;
        r.friction = cp.friction;
        r.impulse = 0; r.pushImpulse = 0; r.penetration = 0;
        V3 ft = crs(rp1, r.normal);
        r.rp1xn = ft;
        r.angA = mulMv(ft, b0.invInertiaWorld);
        ft = crs(rp2, r.normal);
        r.rp2xn = ft;
        r.angB = mulMv(ft, b1.invInertiaWorld);
        float denom0 = b0.invMass + dot(normalAxis, crs(r.angA, rp1));
        float denom1 = b1.invMass + dot(normalAxis, crs(r.angB, rp2));
        r.jacDiagABInv = 1.0f / (denom0 + denom1);
        frows.push_back(r);
    };
    const bool warm = (cfg.solverMode & SOLVER_USE_WARMSTARTING) != 0;
    // solveGroupCacheFriendlySetup (java:418-786)
    for (int pi : manifolds) {
        Manifold& m = w.pairMf[pi];
        const Body& b0 = w.bodies[m.body0];
        const Body& b1 = w.bodies[m.body1];
        int sbA = -1, sbB = -1;
        if (m.n != 0) { sbA = get_sb(m.body0); sbB = get_sb(m.body1); }
        for (int j = 0; j < m.n; j++) {
            ManifoldPoint& cp = m.pts[j];
            if (!(cp.distance <= 0.0f)) continue;
            V3 pos1 = cp.worldA, pos2 = cp.worldB;
            V3 rp1 = sub(pos1, b0.xf.o), rp2 = sub(pos2, b1.xf.o);
            float relaxation = 1.0f;
            int frictionIndex = (int)rows.size();
            Row r;
            r.bodyA = sbA; r.bodyB = sbB;
            r.mfPair = pi; r.mfPoint = j;
            V3 ta0 = crs(rp1, cp.normal);
            r.angA = mulMv(ta0, b0.invInertiaWorld);
            V3 ta1 = crs(rp2, cp.normal);
            r.angB = mulMv(ta1, b1.invInertiaWorld);
            {
                float denom0 = b0.invMass + dot(cp.normal, crs(r.angA, rp1));
                float denom1 = b1.invMass + dot(cp.normal, crs(r.angB, rp2));
                r.jacDiagABInv = relaxation / (denom0 + denom1);
            }
            r.normal = cp.normal;
            r.rp1xn = crs(rp1, cp.normal);
            r.rp2xn = crs(rp2, cp.normal);
            V3 vel1 = add(crs(b0.angvel, rp1), b0.linvel);   // RigidBody.getVelocityInLocalPoint
            V3 vel2 = add(crs(b1.angvel, rp2), b1.linvel);
            V3 vel = sub(vel1, vel2);
            float rel_vel = dot(cp.normal, vel);
            r.penetration = jmin(cp.distance + cfg.linearSlop, 0.0f);
            r.friction = cp.friction;
            r.restitution = cp.restitution * -rel_vel;   // restitutionCurve
            if (r.restitution <= 0.0f) r.restitution = 0.0f;
            float penVel = -r.penetration / dt;
            if (r.restitution > penVel) r.penetration = 0.0f;
            if (warm) {
                r.impulse = cp.appliedImpulse * cfg.warmstartingFactor;
                sb[r.bodyA].apply(scl(r.normal, b0.invMass), r.angA, r.impulse);
                sb[r.bodyB].apply(scl(r.normal, b1.invMass), r.angB, -r.impulse);
            } else {
                r.impulse = 0.0f;
            }
            r.pushImpulse = 0.0f;
            r.frictionIndex = (int)frows.size();
            rows.push_back(r);
            if (!cp.latInit) {
                cp.latDir1 = sub(vel, scl(cp.normal, rel_vel));
                float lat_rel_vel = len2(cp.latDir1);
                if (lat_rel_vel > FLT_EPS) {
                    cp.latDir1 = scl(cp.latDir1, 1.0f / jsqrt(lat_rel_vel));
                    add_friction(cp.latDir1, sbA, sbB, frictionIndex, cp, rp1, rp2, b0, b1);
                    cp.latDir2 = nor(crs(cp.latDir1, cp.normal));
                    add_friction(cp.latDir2, sbA, sbB, frictionIndex, cp, rp1, rp2, b0, b1);
                } else {
                    plane_space1(cp.normal, cp.latDir1, cp.latDir2);
                    add_friction(cp.latDir1, sbA, sbB, frictionIndex, cp, rp1, rp2, b0, b1);
                    add_friction(cp.latDir2, sbA, sbB, frictionIndex, cp, rp1, rp2, b0, b1);
                }
                cp.latInit = true;
            } else {
                add_friction(cp.latDir1, sbA, sbB, frictionIndex, cp, rp1, rp2, b0, b1);
                add_friction(cp.latDir2, sbA, sbB, frictionIndex, cp, rp1, rp2, b0, b1);
            }
            Row& nr = rows.back();
            for (int f = 0; f < 2; f++) {
                Row& fr = frows[nr.frictionIndex + f];
                if (warm) {
                    fr.impulse = (f == 0 ? cp.lat1 : cp.lat2) * cfg.warmstartingFactor;
                    sb[nr.bodyA].apply(scl(fr.normal, b0.invMass), fr.angA, fr.impulse);
                    sb[nr.bodyB].apply(scl(fr.normal, b1.invMass), fr.angB, -fr.impulse);
                } else {
                    fr.impulse = 0.0f;
                }
            }
        }
    }
    w.counters.solverRows += (int)rows.size();
    Body fixedB = fixed_body();
    auto jointBody = [&](int b) -> Body& { return b >= 0 ? w.bodies[b] : fixedB; };
    for (int jk : joints) {
        Joint& J = w.joints[jk];
        if (J.type == JOINT_HINGE) hinge_build(J, jointBody(J.a), jointBody(J.b));
        else if (J.type == JOINT_6DOF) d6_build(J, jointBody(J.a), jointBody(J.b));
        else if (J.type == JOINT_CONE) cone_build(J, jointBody(J.a), jointBody(J.b));
        else if (J.type == JOINT_SLIDER) {
            if (J.useLinearReferenceFrameA) slider_build(J, jointBody(J.a), jointBody(J.b), J.frameA, J.pivotA, J.frameB, J.pivotB);
            else slider_build(J, jointBody(J.b), jointBody(J.a), J.frameB, J.pivotB, J.frameA, J.pivotA);
        }
        else joint_build(J, jointBody(J.a), jointBody(J.b));
    }
    // solveGroupCacheFriendlyIterations (java:788-890), split impulse off.  With a residual
    // tolerance the iterations of an island (the group a reference solveGroup call receives)
    // stop once max|delta lambda| / max(max|lambda|, 1e-6) over its rows is within it (the
    // GPU's residual-terminated mode); rows of converged islands are skipped.
    const bool byResidual = cfg.residualTol > 0.0f;
    const int maxIt = byResidual ? cfg.maxIterations : cfg.numIterations;
    std::vector<int> rowIsl;            // residual mode: compact island index of each normal row
    int nIsl = 0;
    if (byResidual) {
        std::unordered_map<int, int> index;
        rowIsl.resize(rows.size());
        for (size_t r = 0; r < rows.size(); r++) {
            const Manifold& m = w.pairMf[rows[r].mfPair];
            int tag = w.bodies[m.body0].islandTag >= 0 ? w.bodies[m.body0].islandTag : w.bodies[m.body1].islandTag;
            if (cfg.residualScope) tag = 0;   // one group: the residual over all rows of the world
            auto it = index.find(tag);
            if (it == index.end()) it = index.emplace(tag, nIsl++).first;
            rowIsl[r] = it->second;
        }
    }
    std::vector<uint8_t> converged(nIsl, 0);
    std::vector<float> dmax(nIsl), lmax(nIsl);
    auto track = [&](int wi, float d, float l) {
        d = d < 0.0f ? -d : d;
        l = l < 0.0f ? -l : l;
        if (d > dmax[wi]) dmax[wi] = d;
        if (l > lmax[wi]) lmax[wi] = l;
    };
    int itersUsed = 0;
    for (int it = 0; it < maxIt && (!rows.empty() || !joints.empty()); it++) {
        if (byResidual && !rows.empty()) {
            bool any = false;
            for (int k = 0; k < nIsl; k++) { dmax[k] = 0.0f; lmax[k] = 0.0f; any = any || !converged[k]; }
            if (!any) break;
        }
        itersUsed = it + 1;
        // joints first (java:823-842): the solver bodies' velocities are written to the rigid
        // bodies around each joint's solve
        for (int jk : joints) {
            Joint& J = w.joints[jk];
            Body& A = jointBody(J.a);
            Body& B = jointBody(J.b);
            for (Body* b : {&A, &B})
                if (b->islandTag >= 0 && b->companionId >= 0 && sb[b->companionId].invMass != 0.0f) {
                    b->linvel = sb[b->companionId].linvel;
                    b->angvel = sb[b->companionId].angvel;
                }
            if (J.type == JOINT_HINGE) hinge_solve(J, A, B, dt);
            else if (J.type == JOINT_6DOF) d6_solve(J, A, B, dt);
            else if (J.type == JOINT_CONE) cone_solve(J, A, B, dt);
            else if (J.type == JOINT_SLIDER) {
                if (J.useLinearReferenceFrameA) slider_solve(J, A, B, dt);
                else slider_solve(J, B, A, dt);
            }
            else joint_solve(J, A, B, dt);
            for (Body* b : {&A, &B})
                if (b->islandTag >= 0 && b->companionId >= 0 && sb[b->companionId].invMass != 0.0f) {
                    sb[b->companionId].linvel = b->linvel;
                    sb[b->companionId].angvel = b->angvel;
                }
        }
        for (size_t r = 0; r < rows.size(); r++) {   // resolveSingleCollisionCombinedCacheFriendly (java:234-284)
            Row& c = rows[r];
            if (byResidual && converged[rowIsl[r]]) continue;
            SolverBody& A = sb[c.bodyA];
            SolverBody& B = sb[c.bodyB];
            float vel1Dotn = dot(c.normal, A.linvel) + dot(c.rp1xn, A.angvel);
            float vel2Dotn = dot(c.normal, B.linvel) + dot(c.rp2xn, B.angvel);
            float rel_vel = vel1Dotn - vel2Dotn;
            float positionalError = -c.penetration * cfg.erp / dt;
            float velocityError = c.restitution - rel_vel;
            float penetrationImpulse = positionalError * c.jacDiagABInv;
            float velocityImpulse = velocityError * c.jacDiagABInv;
            float normalImpulse = penetrationImpulse + velocityImpulse;
            float oldImpulse = c.impulse;
            float sum = oldImpulse + normalImpulse;
            c.impulse = 0.0f > sum ? 0.0f : sum;
            normalImpulse = c.impulse - oldImpulse;
            A.apply(scl(c.normal, A.invMass), c.angA, normalImpulse);
            B.apply(scl(c.normal, B.invMass), c.angB, -normalImpulse);
            if (byResidual) track(rowIsl[r], normalImpulse, c.impulse);
        }
        for (Row& c : frows) {  // resolveSingleFrictionCacheFriendly (java:286-346)
            const int wi = byResidual ? rowIsl[c.frictionIndex] : 0;
            if (byResidual && converged[wi]) continue;
            float total = rows[c.frictionIndex].impulse + rows[c.frictionIndex].pushImpulse;
            float limit = total * c.friction;
            if (byResidual && !(total > 0.0f)) track(wi, 0.0f, c.impulse);
            if (total > 0.0f) {
                SolverBody& A = sb[c.bodyA];
                SolverBody& B = sb[c.bodyB];
                float vel1Dotn = dot(c.normal, A.linvel) + dot(c.rp1xn, A.angvel);
                float vel2Dotn = dot(c.normal, B.linvel) + dot(c.rp2xn, B.angvel);
                float rel_vel = vel1Dotn - vel2Dotn;
                float j1 = -rel_vel * c.jacDiagABInv;
                float old = c.impulse;
                c.impulse = old + j1;
                if (limit < c.impulse) c.impulse = limit;
                else if (c.impulse < -limit) c.impulse = -limit;
                j1 = c.impulse - old;
                A.apply(scl(c.normal, A.invMass), c.angA, j1);
                B.apply(scl(c.normal, B.invMass), c.angB, -j1);
                if (byResidual) track(wi, j1, c.impulse);
            }
        }
        if (byResidual)
            for (int k = 0; k < nIsl; k++)
                if (!converged[k] && dmax[k] / (lmax[k] > 1e-6f ? lmax[k] : 1e-6f) <= cfg.residualTol) converged[k] = 1;
    }
    if (itersUsed > w.counters.solverIterations) w.counters.solverIterations = itersUsed;
    // write-back (java:901-924): appliedImpulseLateral1 is assigned twice, lateral2 never
    for (const Row& c : rows) {
        ManifoldPoint& pt = w.pairMf[c.mfPair].pts[c.mfPoint];
        pt.appliedImpulse = c.impulse;
        pt.lat1 = frows[c.frictionIndex].impulse;
        pt.lat1 = frows[c.frictionIndex + 1].impulse;
    }
    for (const SolverBody& s : sb) {
        if (s.invMass != 0.0f) { w.bodies[s.original].linvel = s.linvel; w.bodies[s.original].angvel = s.angvel; }
    }
}

static int island_of(const World& w, int pi) {   // SimulationIslandManager.getIslandId (java:111-117)
    const Manifold& m = w.pairMf[pi];
    return w.bodies[m.body0].islandTag >= 0 ? w.bodies[m.body0].islandTag : w.bodies[m.body1].islandTag;
}

static bool has_rows(const World& w, int pi) {
    const Manifold& m = w.pairMf[pi];
    for (int j = 0; j < m.n; j++) if (m.pts[j].distance <= 0.0f) return true;
    return false;
}

// Deterministic colouring (the GPU's, when every batch world forms one solver part).  Colours
// are grown round by round into maximal sets by claim passes: each dynamic body is claimed by the
// lowest pair index among the eligible manifolds touching it (uncoloured, no dynamic body taken
// by the round); manifolds holding all their claims join the round's colour and take their
// bodies; a round ends after a pass that adds nothing, or after 16 passes.  Returns the
// manifolds ordered by (world, colour, pair index).
static std::vector<int> colour_order(World& w, const std::vector<int>& cand, std::vector<int>& colourOut) {
    const int kMaxPasses = 16;
    const size_t n = cand.size();
    std::vector<int> colour(n, -1), taken(w.bodies.size(), -1), claim(w.bodies.size(), INT_MAX);
    auto dyn = [&](int b) { return w.bodies[b].islandTag >= 0; };
    size_t done = 0;
    int round = 0;
    std::vector<size_t> elig;
    while (done < n) {
        for (int pass = 0; pass < kMaxPasses; pass++) {
            elig.clear();
            for (size_t i = 0; i < n; i++) {
                if (colour[i] >= 0) continue;
                const Manifold& m = w.pairMf[cand[i]];
                if ((dyn(m.body0) && taken[m.body0] == round) || (dyn(m.body1) && taken[m.body1] == round)) continue;
                elig.push_back(i);
            }
            for (size_t i : elig) {
                const Manifold& m = w.pairMf[cand[i]];
                if (dyn(m.body0)) claim[m.body0] = std::min(claim[m.body0], cand[i]);
                if (dyn(m.body1)) claim[m.body1] = std::min(claim[m.body1], cand[i]);
            }
            size_t won = 0;
            for (size_t i : elig) {
                const Manifold& m = w.pairMf[cand[i]];
                bool win = (!dyn(m.body0) || claim[m.body0] == cand[i]) && (!dyn(m.body1) || claim[m.body1] == cand[i]);
                if (!win) continue;
                colour[i] = round;
                if (dyn(m.body0)) taken[m.body0] = round;
                if (dyn(m.body1)) taken[m.body1] = round;
                won++;
            }
            for (size_t i : elig) {
                const Manifold& m = w.pairMf[cand[i]];
                claim[m.body0] = INT_MAX;
                claim[m.body1] = INT_MAX;
            }
            done += won;
            if (won == 0) break;
        }
        round++;
    }
    std::vector<std::tuple<int, int, int>> cm(n);
    for (size_t i = 0; i < n; i++) cm[i] = std::make_tuple(w.bodies[w.pairMf[cand[i]].body0].world, colour[i], cand[i]);
    std::sort(cm.begin(), cm.end());
    std::vector<int> order;
    colourOut.clear();
    for (auto& t : cm) { order.push_back(std::get<2>(t)); colourOut.push_back(std::get<1>(t)); }
    w.counters.colours = round;
    return order;
}

// solveConstraints -> buildAndProcessIslands (DiscreteDynamicsWorld.java:620-647; SimulationIslandManager.java:242-333)
void stage_solve(World& w, float dt) {
    PhaseTimer pt(w, 6);
    w.counters.solverRows = 0;
    w.counters.solverIterations = 0;
    w.lastOrder.clear();
    w.lastColour.clear();
    // joints solved this step, in colour order (islands share no dynamic body, so one order
    // over all of them is equivalent to per-island orders)
    std::vector<int> jointOrder;
    for (int k : joint_colour_order(w)) if (g_jointIsland[k] >= 0) jointOrder.push_back(k);
    w.lastJointOrder = jointOrder;
    if (w.orderMode == ORDER_REFERENCE) {
        std::vector<int> im = g_islandManifolds;
        if (im.size() > 1)
            quick_sort(im, 0, (int)im.size() - 1, [&](int a, int b) { return island_of(w, a) < island_of(w, b) ? -1 : +1; });
        std::vector<uint8_t> inactive(w.bodies.size(), 0);
        for (const Body& b : w.bodies) if (b.islandTag >= 0 && !b.isActive()) inactive[b.islandTag] = 1;
        size_t s = 0;
        while (s < im.size()) {
            int isl = island_of(w, im[s]);
            size_t e = s + 1;
            while (e < im.size() && island_of(w, im[e]) == isl) e++;
            if (!inactive[isl]) {
                std::vector<int> grp(im.begin() + s, im.begin() + e), gj;
                for (int k : jointOrder) if (g_jointIsland[k] == isl) gj.push_back(k);
                solve_group(w, grp, gj, dt);
                for (int k : grp) if (has_rows(w, k)) w.lastOrder.push_back(k);
            }
            s = e;
        }
        // islands with joints and no manifold
        std::vector<uint8_t> withMf(w.bodies.size(), 0);
        for (int k : im) withMf[island_of(w, k)] = 1;
        std::vector<int> rest;
        for (int k : jointOrder) if (!withMf[g_jointIsland[k]]) rest.push_back(k);
        std::vector<int> isls;
        for (int k : rest) isls.push_back(g_jointIsland[k]);
        std::sort(isls.begin(), isls.end());
        isls.erase(std::unique(isls.begin(), isls.end()), isls.end());
        for (int isl : isls) {
            std::vector<int> gj;
            for (int k : rest) if (g_jointIsland[k] == isl) gj.push_back(k);
            solve_group(w, std::vector<int>(), gj, dt);
        }
        w.counters.colours = 0;
    } else {
        std::vector<int> order;
        std::vector<int> cand;
        for (int k : w.solveList) if (has_rows(w, k)) cand.push_back(k);
        if (w.orderMode == ORDER_EXPLICIT) {
            order = w.explicitOrder;
            std::vector<int> a(order), b(cand);
            std::sort(a.begin(), a.end());
            std::sort(b.begin(), b.end());
            if (a != b) w.counters.orderMismatch++;
        } else {
            order = colour_order(w, cand, w.lastColour);
        }
        solve_group(w, order, jointOrder, dt);
        w.lastOrder = order;
    }
    w.counters.solverManifolds = (int)w.lastOrder.size();
}

// integrateTransforms (dynamics/DiscreteDynamicsWorld.java:679-739) with the CCD motion clamping
// of bodies whose predicted displacement squared exceeds ccdMotionThreshold^2 (the reference's
// getCcdSquareMotionThreshold, CollisionObject.java:290-292): the body moves only to the sweep's
// first accepted time of impact when that is above 0.0001.  Bodies are moved one after the
// other, so a later body's sweep sees the earlier ones where they ended.
void stage_integrate(World& w, float dt) {
    PhaseTimer pt(w, 7);
    w.counters.ccdClamped = 0;
    w.counters.ccdPlane = 0;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        Body& b = w.bodies[i];
        b.hitFraction = 1.0f;          // java:692
        if (b.isActive() && !b.isStaticOrKinematic()) {
            Xf p = integrate_transform(b.xf, b.linvel, b.angvel, dt);
            const float sq = b.ccdMotionThreshold * b.ccdMotionThreshold;
            const float squareMotion = len2(sub(p.o, b.xf.o));
            if (sq != 0.0f && sq < squareMotion && w.shapes[b.shape].isConvex()) {
                w.counters.ccdClamped++;
                float f = 1.0f;
                bool plane = false;
                if (ccd_sweep(w, (int)i, p, f, &plane) && f > 0.0001f) {
                    p = integrate_transform(b.xf, b.linvel, b.angvel, dt * f);
                    b.hitFraction = 0.0f;   // java:717
                }
                if (plane) w.counters.ccdPlane++;
            }
            b.xf = p;                  // RigidBody.setCenterOfMassTransform
            b.ixf = p;
            b.ilv = b.linvel;
            b.iav = b.angvel;
            update_inertia_tensor(b);
        }
    }
}

// updateActivationState (dynamics/DiscreteDynamicsWorld.java:475-512) with
// RigidBody.updateDeactivation / wantsSleeping (dynamics/RigidBody.java:543-576)
void stage_activation(World& w, float dt) {
    PhaseTimer pt(w, 8);
    for (Body& b : w.bodies) {
        if (!(b.activation == ISLAND_SLEEPING || b.activation == DISABLE_DEACTIVATION)) {
            if (len2(b.linvel) < b.linSleep * b.linSleep && len2(b.angvel) < b.angSleep * b.angSleep) {
                b.deactivationTime += dt;
            } else {
                b.deactivationTime = 0.0f;
                b.setActivationState(0);
            }
        }
        bool wants;
        if (b.activation == DISABLE_DEACTIVATION) wants = false;
        else if (w.cfg.disableDeactivation || w.cfg.deactivationTime == 0.0f) wants = false;
        else if (b.activation == ISLAND_SLEEPING || b.activation == WANTS_DEACTIVATION) wants = true;
        else wants = b.deactivationTime > w.cfg.deactivationTime;
        if (wants) {
            if (b.isStaticOrKinematic()) {
                b.setActivationState(ISLAND_SLEEPING);
            } else {
                if (b.activation == ACTIVE_TAG) b.setActivationState(WANTS_DEACTIVATION);
                if (b.activation == ISLAND_SLEEPING) { b.angvel = v3(0, 0, 0); b.linvel = v3(0, 0, 0); }
            }
        } else {
            if (b.activation != DISABLE_DEACTIVATION) b.setActivationState(ACTIVE_TAG);
        }
    }
}

void stage_clear_forces(World& w) {   // DiscreteDynamicsWorld.clearForces (java:226-236)
    for (Body& b : w.bodies) { b.totalForce = v3(0, 0, 0); b.totalTorque = v3(0, 0, 0); }
}

// internalSingleStepSimulation (dynamics/DiscreteDynamicsWorld.java:356-400)
void internal_single_step(World& w, float dt) {
    stage_predict(w, dt);
    stage_aabbs(w);
    stage_pairs(w);
    stage_narrowphase(w);
    stage_islands(w);
    stage_solve(w, dt);
    stage_integrate(w, dt);
    stage_activation(w, dt);
    w.counters.steps++;
    if (w.tickCb) w.tickCb(&w, dt, w.tickUser);   // java:393-395
}

// stepSimulation (dynamics/DiscreteDynamicsWorld.java:290-354)
// DiscreteDynamicsWorld.saveKinematicState (DiscreteDynamicsWorld.java:105-119): every kinematic
// body that is not ISLAND_SLEEPING takes the velocities that carry its last saved transform to
// its current one (RigidBody.saveKinematicState, RigidBody.java:190-205).
void stage_save_kinematic(World& w, float timeStep) {
    for (Body& b : w.bodies) {
        if (b.activation == ISLAND_SLEEPING || !b.isKinematic() || timeStep == 0.0f) continue;
        calculate_velocity(b.ixf, b.xf, timeStep, b.linvel, b.angvel);
        b.ilv = b.linvel;   // RigidBody.java:200-202
        b.iav = b.angvel;
        b.ixf = b.xf;
    }
}

int step_simulation(World& w, float timeStep, int maxSubSteps, float fixedTimeStep) {
    int num = 0;
    if (maxSubSteps != 0) {
        w.localTime += timeStep;
        if (w.localTime >= fixedTimeStep) {
            num = (int)(w.localTime / fixedTimeStep);
            w.localTime -= num * fixedTimeStep;
        }
    } else {
        fixedTimeStep = timeStep;
        w.localTime = timeStep;
        if (std::fabs(timeStep) < FLT_EPS) { num = 0; maxSubSteps = 0; }
        else { num = 1; maxSubSteps = 1; }
    }
    if (num != 0) {
        stage_save_kinematic(w, fixedTimeStep);
        stage_apply_gravity(w);
        int clamped = num > maxSubSteps ? maxSubSteps : num;
        for (int i = 0; i < clamped; i++) internal_single_step(w, fixedTimeStep);
    }
    stage_clear_forces(w);
    return num;
}

void step_fixed(World& w, float dt, int substeps) {
    stage_save_kinematic(w, dt);
    stage_apply_gravity(w);
    for (int i = 0; i < substeps; i++) internal_single_step(w, dt);
    stage_clear_forces(w);
}

}  // namespace jb
