#pragma once
#include "jbgpu_internal.cuh"

namespace jbg {

struct SolverBuffers {
    int* parent = nullptr;        // union-find (bodies)
    int* keepAwake = nullptr;     // per island root
    int* inactive = nullptr;      // per island root
    int* flag = nullptr;          // per pair: manifold is solved this step
    int* candIdx = nullptr;       // exclusive scan of flag
    int* cand = nullptr;          // pair index of candidate k (ascending)
    int* colourOf = nullptr;      // colour of candidate k
    int* remA = nullptr;          // colouring work lists
    int* remB = nullptr;
    unsigned long long* claim = nullptr;  // per body
    int* colourCount = nullptr;   // per colour (MAX_COLOURS + 1)
    int* colourFill = nullptr;
    int* colourStart = nullptr;
    int* nCand = nullptr;         // device scalars
    int* nColours = nullptr;
    void* scanScratch = nullptr;
    int coopBlocksColour = 0;
    int coopBlocksPgs = 0;
};

constexpr int MAX_COLOURS = 1024;

void islands_launch(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s);
void solve_launch(const DevWorld& w, DevPairs& P, int nPairs, DevRows& rows, SolverBuffers& sb, float dt, cudaStream_t s,
                  const Prof* prof = nullptr);
int solver_coop_blocks(bool pgs);

}  // namespace jbg
