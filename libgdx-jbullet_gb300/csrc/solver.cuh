#pragma once
#include <vector>
#include "jbgpu_internal.cuh"

namespace jbg {

constexpr int MAX_COLOURS = 1024;     // grid-wide colours of cut manifolds
constexpr int MAX_LOCAL = 128;        // colours of the manifolds internal to one part
constexpr int MAX_SUB = 16;
constexpr int COL_REG = 4;            // internal-colouring candidates a thread keeps in registers           // claim passes that grow one colour towards a maximal set
constexpr int SOLVER_THREADS = 256;
constexpr int PART_MAX_BODIES = 2048; // bodies of one part (velocities staged in 64 KB of shared memory)

// Solver parts.  Dynamic bodies are split into parts of consecutive positions in a body order
// (the broadphase's sorted leaf order: Morton code with the batch world in the high bits).
// World parts: every world holds at most PART_MAX_BODIES finite bodies, and each world is one
// part.  Range parts otherwise: nParts equal ranges of the order.
// Joints (jbgpu_world_add_point2point, jbgpu_world_add_hinge), uploaded by the host when they
// change.
constexpr int JOINT_P2P = 0;
constexpr int JOINT_HINGE = 1;
constexpr int JOINT_6DOF = 2;
constexpr int JOINT_CONE = 3;
constexpr int JOINT_SLIDER = 4;
constexpr int JK_TYPE = 0xff;         // kind: type in the low byte, hinge switches above it
constexpr int JK_ANGULAR_ONLY = 1 << 8;
constexpr int JK_MOTOR = 1 << 9;
constexpr int JOINT_STEP_F4 = 13;     // float4s of a hinge's or 6-dof joint's per-step state
constexpr int D6_SET_F4 = 12;         // float4s of a 6-dof joint's settings
struct DevJoints {
    int n = 0;                    // joints
    int nCol = 0;                 // colours: first fit in index order over the joints' dynamic bodies
    int* kind = nullptr;          // JOINT_P2P / JOINT_HINGE | JK_ANGULAR_ONLY | JK_MOTOR
    int* a = nullptr;             // body A of each joint
    int* b = nullptr;             // body B, -1 for the fixed body
    float4* pivA = nullptr;       // pivotInA, pivotInB (xyz); a hinge's frame origins
    float4* pivB = nullptr;
    float4* set = nullptr;        // p2p: tau, damping, impulse clamp; hinge: lower, upper limit, softness, bias;
                                  // cone twist: swing span 1, swing span 2, twist span, softness
    float4* set2 = nullptr;       // hinge: relaxation factor, motor target velocity, max motor impulse;
                                  // cone twist: bias factor, relaxation factor
    float4* frame = nullptr;      // hinge: rbAFrame basis rows (3), then rbBFrame basis rows (3)
    float4* hs = nullptr;         // per step (JOINT_STEP_F4 each).  Hinge: axis n_i with 1/Adiag_i (3),
                                  // world hinge axis of A with kHinge, of B with the limit correction,
                                  // (limit sign, accumulated limit impulse, 0, 0).  6-dof: the two
                                  // calculated frame origins, the anchor, linear axes with 1/Adiag
                                  // (3), angular axes with 1/Adiag (3), (limit state, limit error)
                                  // per angular axis (2), accumulated linear and angular impulses
    float4* d6set = nullptr;      // slider: its 28 parameters (jbgpu_world_set_slider_params order);
                                  // 6-dof settings (D6_SET_F4 each): linear lower xyz | use frame A,
                                  // upper xyz | softness, (damping, restitution), then per angular axis
                                  // (lo, hi, target velocity, max motor force), (max limit force,
                                  // damping, softness, ERP), (bounce, motor enabled)
    int* order = nullptr;         // joints by (colour, index)
    int* colStart = nullptr;      // nCol + 1 offsets into order
    float4* r1 = nullptr;         // per step: pivot A - centre of A, 1/Adiag of axis 0 in .w
    float4* r2 = nullptr;         // pivot B - centre of B, 1/Adiag of axis 1 in .w
    float4* dep = nullptr;        // depth per axis, 1/Adiag of axis 2 in .w
    float* imp = nullptr;         // appliedImpulse
    int* act = nullptr;           // solved this step (its island is processed)
};

struct SolverBuffers {
    int* parent = nullptr;        // union-find (bodies)
    int* keepAwake = nullptr;     // per island root
    int* inactive = nullptr;      // per island root
    int* flag = nullptr;          // per pair: manifold is solved this step
    int* candIdx = nullptr;       // exclusive scan of flag
    int* cand = nullptr;          // pair index of candidate k (ascending)
    int* colourOf = nullptr;      // colour of candidate k (local colour for internal ones)
    int* bucket = nullptr;        // part of candidate k, nParts when cut
    int* bucketList = nullptr;    // candidates grouped by bucket
    int* candLocal = nullptr;     // per candidate: its dynamic bodies' indices within its part
    unsigned long long* claim = nullptr;  // per body
    int* taken = nullptr;         // per body: colouring round that took it
    int* posOf = nullptr;         // per body: position in the body order (-1 none)
    int* colourCount = nullptr;   // per cut colour (MAX_COLOURS + 1)
    int* colourFill = nullptr;
    int* colourStart = nullptr;
    int* nCand = nullptr;         // device scalars
    int* nColours = nullptr;      // cut colours
    void* scanScratch = nullptr;
    // part tables (capacity partsCap)
    int* bucketCount = nullptr;   // nParts + 2
    int* bucketFill = nullptr;
    int* bucketStart = nullptr;
    int* lcCount = nullptr;       // nParts * (MAX_LOCAL + 1)
    int* lcFill = nullptr;
    int* lcStart = nullptr;
    int* nLocal = nullptr;        // nParts
    int* partStart = nullptr;     // nParts + 1 positions of the body order
    int* partOrder = nullptr;     // parts by decreasing size (the order blocks take them in)
    int* orderFallback = nullptr; // body order built on the host when the broadphase order is stale
    // residual mode: per slot maxima and island grouping (slots by island root)
    float* md = nullptr;          // per slot: largest |delta lambda| of the iteration
    float* ml = nullptr;          // per slot: largest |lambda|
    int* slotIsl = nullptr;       // per slot: island root
    int* islList = nullptr;       // slots grouped by island (pair capacity)
    int* islCount = nullptr;      // per body index (island root): slots, nBodies + 1
    int* islFill = nullptr;
    int* islStart = nullptr;
    int* segFlag = nullptr;       // per body index: chunks of the island's slots
    int* segIdx = nullptr;        // first chunk of the island
    int2* islChunk = nullptr;     // (island root, chunk) for every chunk; capacity pairs + bodies
    int* islConv = nullptr;       // per island root: converged this solve
    int* islAcc = nullptr;        // per island root: chunk maxima (float bits), 2 per island
    int* islDone = nullptr;       // per island root: chunks reduced this iteration
    int* nIslChunks = nullptr;    // device scalar
    unsigned* resTrace = nullptr; // per iteration: max |delta lambda|, max |lambda| (float bits) of the rows tested
    void* islScratch = nullptr;   // scan scratch for nBodies + 1
    const int* order = nullptr;   // body order in use
    int nFinite = 0;
    int nParts = 0;
    int partsCap = 0;
    int partMax = 0;              // largest part, bodies
    int partSmem = 0;             // velocities of internal manifolds staged in shared memory
    int smemCap = 0;              // parts of at most this many bodies are staged
    int poolPts = 0;              // entries of each of k_pgs's two point pools (0: none)
    int worldParts = 0;
    int gridColour = 0;           // co-resident blocks of the cooperative kernels
    int gridPgs = 0;
    int threads = SOLVER_THREADS;
    DevJoints J;                  // point-to-point joints
};

// (Re)plans the parts for nFinite ordered bodies.  worldCounts: finite bodies per batch world;
// rangeParts > 0 asks for that many range parts; threads per block of the colouring and PGS;
// smemBodies > 0 caps the parts whose velocities are staged in shared memory.
int solver_configure(SolverBuffers& sb, int nFinite, const std::vector<int>& worldCounts, int sms, int rangeParts,
                     int threads, int smemBodies);
void islands_launch(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s);
void islands_launch_unions(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s,
                           const int* cntp);
void islands_launch_select(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s,
                           const int* cntp);
void solve_launch(const DevWorld& w, DevPairs& P, int nPairs, DevRows& rows, SolverBuffers& sb, float dt, cudaStream_t s,
                  const Prof* prof = nullptr);
void solver_free(SolverBuffers& sb);

// Learned warm start and contact samples (solver.cu): per contact point q = slot * 4 + point,
// 24 features (X) before the solve and the 3 converged impulses (T) after it.
struct MlpDev;
struct SolverLearn {
    const MlpDev* mlp = nullptr;    // non-null: warm-start impulses predicted by the MLP
    float* sampleX = nullptr;       // non-null: features written (capacity rows * 4 * 24)
    float* sampleT = nullptr;       // non-null: converged impulses written (rows * 4 * 3)
    int allPoints = 0;              // 1: every point's impulses, also of islands not converged
};
int solver_learn_configure();     // once per world: shared-memory size of the warm-start kernel
void solve_launch_learn(const DevWorld& w, DevPairs& P, int nPairs, DevRows& rows, SolverBuffers& sb, float dt,
                        cudaStream_t s, const Prof* prof, const SolverLearn& learn);

}  // namespace jbg
