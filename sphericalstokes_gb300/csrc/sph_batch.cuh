// Batched correction sweeps over many grids of uneven size in one launch.
//
// A batch of mixed-precision solves advances in lockstep: every solve whose
// correction problem is being iterated runs the same number of FP32 sweeps per
// round.  One sweep of all of them is one launch of k_fused_tma_batch per
// geometry over a work list of (solve, tile x, tile y, x3 chunk) items — the
// blocks each solve's own k_fused_tma launch would have — followed by one
// launch per BC stage over the (solve, face block) items of that stage; a
// round of sweeps is replayed from one CUDA graph.  The kernels run the
// single-grid bodies (fused_tma_body, bc_body, velocity_norm_body), so each
// solve computes exactly what it computes alone.
//
// Per-solve data live in device memory (BatchSweep), read by the kernels at
// run time, so the captured graph stays valid while solves enter and leave the
// correction phase: the host rewrites a solve's entry and its active flag,
// and blocks of inactive solves return at once.
#pragma once
#include "sph_fused.cuh"

namespace sph {

constexpr int kBatchMaxBc = 4;  // BC stages per sweep (after the fused x1-face stage)

struct BatchSweep {
    KP<float> p[2];                // correction problem in both ping-pong arrangements (a: the sweep reads p[a])
    FusedOut<float> o[2];          // outputs of a sweep reading arrangement a (the other buffer set)
    const CUtensorMap* maps[2];    // TMA maps of the arrangement a sweep reads
    int* err;                      // the solve's bounded-wait error word
    int kchunk;                    // x3 planes per block
    int nbc;                       // BC stages launched after each sweep (on the new arrangement)
    BcStage bc[kBatchMaxBc];
};

// one correction sweep of every active solve of geometry G (items: x = solve, y, z, w = tile x, y, chunk)
template <int G>
__global__ void __launch_bounds__(FNT, 3) k_fused_tma_batch(const BatchSweep* __restrict__ b, const int4* __restrict__ items,
                                                             const int* __restrict__ active, int a) {
    pdl_wait();  // as k_fused_tma: no early release of the next grid
    const int4 it = items[blockIdx.x];
    if (!active[it.x]) return;  // whole block: no barrier is reached
    const BatchSweep& s = b[it.x];
    fused_tma_body<G, 1>(s.p[a], s.o[a], s.kchunk, s.maps[a], s.err, it.y, it.z, it.w);
}

// BC stage t of every active solve of geometry G after a sweep that read arrangement a (the
// stage acts on arrangement a ^ 1); items: x = solve, y, z = face block; 32 x 8 threads
template <int G>
__global__ void k_bc_batch(const BatchSweep* __restrict__ b, const int4* __restrict__ items, const int* __restrict__ active, int a,
                           int t) {
    pdl_enter();  // as k_bc
    const int4 it = items[blockIdx.x];
    if (!active[it.x]) return;
    const BatchSweep& s = b[it.x];
    if (t >= s.nbc) return;
    bc_body<float, G>(s.p[a ^ 1], s.bc[t], 1, it.y * blockDim.x + threadIdx.x, it.z * blockDim.y + threadIdx.y);
}

// inner stopping test of every active solve of geometry G: max |dV + rV| of arrangement 0 into
// red[solve]; items: x = solve, y, z, w = velocity-node block; 32 x 8 threads
template <int G>
__global__ void __launch_bounds__(256) k_velocity_norm_batch(const BatchSweep* __restrict__ b, const int4* __restrict__ items,
                                                             const int* __restrict__ active, unsigned long long* __restrict__ red) {
    const int4 it = items[blockIdx.x];
    if (!active[it.x]) return;
    velocity_norm_body<float, G>(b[it.x].p[0], it.y, it.z, it.w, red + it.x);
}

}  // namespace sph
