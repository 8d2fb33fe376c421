// Fused FP32 PT sweep: compute_P! and compute_V! of one PT iteration in a
// single launch (SphericalStokes_diapir.jl:416-422), bandwidth-bound design.
//
// A block owns a TX x TY column of cells in (x1, x2) and marches along x3
// over a chunk of planes (2.5D blocking).  Per plane K it
//   1. issues asynchronous copies (cp.async, Ampere-style LDGSTS) of the input
//      plane K+2 (V1, V2, V3, η, ηSM on the tile + halo) into a 3-slot ring, and
//      of the old P, τ (and rP or ρ) of plane K+1 plus the right-hand side rV
//      of plane K+1 into 2-slot rings, so DRAM latency overlaps the compute of
//      plane K;
//   2. updates P, τ11..τ33 (cells) and τ12, τ13, τ23 (edges) of plane K on the
//      tile plus a one-point halo on the low x1/x2 sides (one point per thread:
//      (TX+1)(TY+1) <= threads), keeping them in a 2-plane shared ring and
//      writing the owned points to the output state;
//   3. updates V1, V2, V3 of plane K from the shared stresses of planes K-1, K.
// Every state field is read once and written once per sweep (halo re-reads
// hit L2); the old and new states are different buffers (ping-pong) and the
// boundary-condition stages run afterwards on the new state.  The arithmetic
// of k_fused is the shared core of sph_core.cuh: results equal those of
// k_stress + k_velocity.  k_fused_tma (below) feeds the same march by TMA and
// evaluates the edge-strain and momentum terms on per-thread coefficients
// (SweepCoef): the same values up to FP32 rounding.
//
// MODE 0: reference iteration (ρg body force).  MODE 1: correction problem of
// the mixed-precision solve (right-hand sides rP, rV; η and ηSM frozen).
#pragma once
#include <type_traits>

#include "sph_core.cuh"

namespace sph {

template <typename T>
struct FusedOut {
    T *P, *V1, *V2, *V3, *t11, *t22, *t33, *t12, *t13, *t23;
    // k_fused_tma only: ghost velocities on the two x1 faces written with the new values,
    // ghost = xg[f] x (its interior neighbour) for the fields f of bit f in xg_mask (the
    // first stage of the homogeneous BC program, which the launch then skips)
    int xg_mask;
    T xg[3];
};

constexpr int FTX = 32, FTY = 8;                  // owned tile (cells) per block
constexpr int FLX = FTX + 2, FLY = FTY + 2;       // input tile with halo
constexpr int FSX = FTX + 1, FSY = FTY + 1;       // stage-1 points (tile + low halo)
constexpr int FNT = 320;                          // threads: >= FSX*FSY = 297 and a multiple of 32
constexpr int F_IN = 5;                           // V1 V2 V3 η ηSM
constexpr int F_OLD = 8;                          // P τ11 τ22 τ33 τ12 τ13 τ23 + (rP | ρ)
constexpr int F_RV = 3;                           // rV1 rV2 rV3

struct FusedSmem {
    float in[3][F_IN][FLY][FLX];    // input ring (planes K, K+1, K+2)
    float old[2][F_OLD][FSY][FSX];  // old state ring (planes K, K+1)
    float rv[2][F_RV][FTY][FTX];    // right-hand side ring (planes K, K+1)
    float st[2][8][FSY][FSX];       // new stresses ring (planes K-1, K): P t11 t22 t33 t12 t13 t23 DT_R
};

__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int sz = valid ? 4 : 0;  // 0: zero-fill, nothing read
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int G, int MODE>
__global__ void __launch_bounds__(FNT, 3) k_fused(KP<float> p, FusedOut<float> o, int kchunk) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    FusedSmem& S = *reinterpret_cast<FusedSmem*>(smem_raw);
    enum { IP = 0, I11, I22, I33, I12, I13, I23, IX };  // old-ring / stress-ring field slots (IX: rP | ρ, or DT_R)

    const Dims d = p.d;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * FTX, y0 = blockIdx.y * FTY;
    const int kA = blockIdx.z * kchunk;
    const int kB = min(kA + kchunk, d.n3);
    const int n1 = d.n1, n2 = d.n2, n3 = d.n3;
    const float d1 = p.d1, d2 = p.d2, d3 = p.d3, gsc = p.gsc, kbc = p.kbc, vpdt2 = p.vpdt2;
    if (kA >= kB) return;

    // asynchronous loads of one plane (zero fill outside the box / for z outside [0, pz))
    auto issue_inputs = [&](int z) {
        const int sl = (z + 3) % 3;
        const bool zok = z >= 0 && z < d.pz;
        for (int q = tid; q < FLX * FLY; q += FNT) {
            const int lx = q % FLX, ly = q / FLX;
            const int x = x0 - 1 + lx, y = y0 - 1 + ly;
            const bool ok = zok && x >= 0 && x < d.px && y >= 0 && y < d.py;
            const int g = ok ? x + d.sy * y + d.sz * z : 0;
            cp_async4(&S.in[sl][0][ly][lx], p.V1 + g, ok);
            cp_async4(&S.in[sl][1][ly][lx], p.V2 + g, ok);
            cp_async4(&S.in[sl][2][ly][lx], p.V3 + g, ok);
            cp_async4(&S.in[sl][3][ly][lx], p.eta + g, ok);
            cp_async4(&S.in[sl][4][ly][lx], p.etaSM + g, ok);
        }
    };
    auto issue_old = [&](int z) {
        const int sl = z & 1;
        if (tid < FSX * FSY) {
            const int a = tid % FSX, b = tid / FSX;
            const int x = x0 - 1 + a, y = y0 - 1 + b;
            const bool ok = z >= 0 && z < d.n3 && x >= 0 && x < d.n1 && y >= 0 && y < d.n2;
            const int g = ok ? x + d.sy * y + d.sz * z : 0;
            cp_async4(&S.old[sl][IP][b][a], p.P + g, ok);
            cp_async4(&S.old[sl][I11][b][a], p.t11 + g, ok);
            cp_async4(&S.old[sl][I22][b][a], p.t22 + g, ok);
            cp_async4(&S.old[sl][I33][b][a], p.t33 + g, ok);
            cp_async4(&S.old[sl][I12][b][a], p.t12 + g, ok);
            cp_async4(&S.old[sl][I13][b][a], p.t13 + g, ok);
            cp_async4(&S.old[sl][I23][b][a], p.t23 + g, ok);
            cp_async4(&S.old[sl][IX][b][a], (MODE == 1 ? p.rP : p.rho) + g, ok);
        }
    };
    auto issue_rv = [&](int z) {
        if (MODE != 1) return;
        const int sl = z & 1;
        if (tid < FTX * FTY) {
            const int a = tid % FTX, b = tid / FTX;
            const int x = x0 + a, y = y0 + b;
            const bool ok = z >= 0 && z < d.pz && x < d.px && y < d.py;
            const int g = ok ? x + d.sy * y + d.sz * z : 0;
            cp_async4(&S.rv[sl][0][b][a], p.rV1 + g, ok);
            cp_async4(&S.rv[sl][1][b][a], p.rV2 + g, ok);
            cp_async4(&S.rv[sl][2][b][a], p.rV3 + g, ok);
        }
    };

    // per-thread constants of the whole march (see k_fused_tma)
    const int a = tid % FSX, b = tid / FSX;
    const int x = x0 - 1 + a, y = y0 - 1 + b;
    const bool s1_in = tid < FSX * FSY && x >= 0 && y >= 0 && x < n1 && y < n2;
    const bool s1_own = a >= 1 && b >= 1;
    const bool e12_xy = x < n1 - 1 && y < n2 - 1, e13_xy = x < n1 - 1 && y < n2 - 2, e23_xy = x < n1 - 2 && y < n2 - 1;
    const CellMetric<float> cm = cell_metric_t<float, G>(p.geo, d2, d3, clampi(x, 0, n1 - 1), clampi(y, 0, n2 - 1));
    const EdgeMetric<float> em = edge_metric<float, G>(p.geo, x, y, n1, n2);
    const int gxy = x + d.sy * y;
    const int tx = tid % FTX, ty = tid / FTX;
    const int I = x0 + tx, J = y0 + ty;
    const bool v_ok = tid < FTX * FTY && I >= 1 && J >= 1 && I <= n1 - 1 && J <= n2 - 1;
    const bool m1_xy = J <= n2 - 2, m2_xy = I <= n1 - 2, m3_xy = I <= n1 - 2 && J <= n2 - 2;
    const MomMetric<float> mm = mom_metric<float, G>(p.geo, I, J, n1, n2);
    const int gIJ = I + d.sy * J;

    // stresses of plane k at this thread's stage-1 point; owned points go to the output state
    auto stage1 = [&](int k, bool own_plane) {
        if (tid >= FSX * FSY) return;
        const int ik = (k + 3) % 3, ik1 = (k + 4) % 3, so = k & 1, ol = k & 1;
        const bool own = own_plane && s1_own;
        const int g = gxy + d.sz * k;
        float (*I0)[FLY][FLX] = S.in[ik];
        float (*I1)[FLY][FLX] = S.in[ik1];
        float (*O)[FSY][FSX] = S.old[ol];
        float vP = 0.f, v11 = 0.f, v22 = 0.f, v33 = 0.f, vdt = 0.f, v12 = 0.f, v13 = 0.f, v23 = 0.f;
        if (s1_in) {
            {
                const CellD<float> D = cell_strain_m<float, G>(cm, d1, I0[0][b][a], I0[0][b][a + 1], I0[1][b][a], I0[1][b + 1][a],
                                                               I0[2][b][a], I1[2][b][a]);
                const float sm = I0[4][b][a], e = I0[3][b][a];
                const float gs = gsc * sm, kb = kbc * sm;
                const float f = pdiv(e, e + gs);
                float dv = D.div;
                if (MODE == 1) dv += O[IX][b][a];
                vP = O[IP][b][a] - kb * dv;
                v11 = (O[I11][b][a] + 2.f * gs * D.D11) * f;
                v22 = (O[I22][b][a] + 2.f * gs * D.D22) * f;
                v33 = (O[I33][b][a] + 2.f * gs * D.D33) * f;
                if (p.traction) traction_pressure(y, k, n2, n3, v22, v33, p.sig2, p.sig3, vP);
                if (p.fs && x == n1 - 1)
                    vP = fs_pressure(v11, p.top_load ? p.top_load[g] : 0.f, p.fs_kappa, I0[0][b][a], I0[0][b][a + 1]);
                vdt = pdiv(vpdt2, kb + gs * f);
                if (own) { o.P[g] = vP; o.t11[g] = v11; o.t22[g] = v22; o.t33[g] = v33; }
            }
            if (e12_xy && k < n3 - 2) {
                const float D = edge12_m<float, G>(em, d1, d2, I1[1][b + 1][a], I1[1][b + 1][a + 1], I1[0][b][a + 1], I1[0][b + 1][a + 1]);
                v12 = edge_update(O[I12][b][a], gsc, I1[4][b][a] + I1[4][b + 1][a] + I1[4][b][a + 1] + I1[4][b + 1][a + 1],
                                  I1[3][b][a] + I1[3][b + 1][a] + I1[3][b][a + 1] + I1[3][b + 1][a + 1], D);
                if (own) o.t12[g] = v12;
            }
            if (e13_xy && k < n3 - 1) {
                const float D = edge13_m<float, G>(em, d1, d3, I1[2][b + 1][a], I1[2][b + 1][a + 1], I0[0][b + 1][a + 1], I1[0][b + 1][a + 1]);
                v13 = edge_update(O[I13][b][a], gsc, I0[4][b + 1][a] + I1[4][b + 1][a] + I0[4][b + 1][a + 1] + I1[4][b + 1][a + 1],
                                  I0[3][b + 1][a] + I1[3][b + 1][a] + I0[3][b + 1][a + 1] + I1[3][b + 1][a + 1], D);
                if (own) o.t13[g] = v13;
            }
            if (e23_xy && k < n3 - 1) {
                const float D = edge23_m<float, G>(em, d2, d3, I1[2][b][a + 1], I1[2][b + 1][a + 1], I0[1][b + 1][a + 1], I1[1][b + 1][a + 1]);
                v23 = edge_update(O[I23][b][a], gsc, I0[4][b][a + 1] + I1[4][b][a + 1] + I0[4][b + 1][a + 1] + I1[4][b + 1][a + 1],
                                  I0[3][b][a + 1] + I1[3][b][a + 1] + I0[3][b + 1][a + 1] + I1[3][b + 1][a + 1], D);
                if (own) o.t23[g] = v23;
            }
        }
        float (*W)[FSY][FSX] = S.st[so];
        W[IP][b][a] = vP; W[I11][b][a] = v11; W[I22][b][a] = v22; W[I33][b][a] = v33;
        W[I12][b][a] = v12; W[I13][b][a] = v13; W[I23][b][a] = v23; W[IX][b][a] = vdt;
    };

    // velocities of plane K from the stresses of planes K-1 and K
    auto velocity = [&](int K) {
        if (!v_ok || K < 1 || K > n3 - 1) return;
        const int g = gIJ + d.sz * K;
        const float h = 0.5f;
        float (*C0)[FSY][FSX] = S.st[K & 1];
        float (*C1)[FSY][FSX] = S.st[(K - 1) & 1];
        float (*Vin)[FLY][FLX] = S.in[K % 3];
        const float Pc = C0[IP][ty + 1][tx + 1];
        const float q11 = C0[I11][ty + 1][tx + 1] - Pc, q22 = C0[I22][ty + 1][tx + 1] - Pc, q33 = C0[I33][ty + 1][tx + 1] - Pc;
        const float dtc = C0[IX][ty + 1][tx + 1];
        if (m1_xy && K <= n3 - 2) {  // V1 (I-1/2, J, K), cell m = (I-1, J, K)
            const float Pm = C0[IP][ty + 1][tx];
            float r = mom1_m<float, G>(mm, d1, d2, d3, C0[I11][ty + 1][tx] - Pm, q11, C0[I22][ty + 1][tx] - Pm, q22, C0[I33][ty + 1][tx] - Pm,
                                       q33, C1[I12][ty + 1][tx], C1[I12][ty][tx], C0[I13][ty][tx], C1[I13][ty][tx]);
            if (G != CART && MODE == 0) {
                const float* rho = &S.old[K & 1][IX][0][0];
                r -= (rho[(ty + 1) * FSX + tx] * p.g + rho[(ty + 1) * FSX + tx + 1] * p.g) * h;
            }
            if (MODE == 1) r += S.rv[K & 1][0][ty][tx];
            o.V1[g] = Vin[0][ty + 1][tx + 1] + r * ((C0[IX][ty + 1][tx] + dtc) * h);
        }
        if (m2_xy && K <= n3 - 2) {  // V2 (I, J-1/2, K), cell m = (I, J-1, K)
            const float Pm = C0[IP][ty][tx + 1];
            float r = mom2_m<float, G>(mm, d1, d2, d3, C0[I22][ty][tx + 1] - Pm, q22, C0[I33][ty][tx + 1] - Pm, q33, C1[I12][ty][tx + 1],
                                       C1[I12][ty][tx], C0[I23][ty][tx], C1[I23][ty][tx]);
            if (MODE == 1) r += S.rv[K & 1][1][ty][tx];
            o.V2[g] = Vin[1][ty + 1][tx + 1] + r * ((C0[IX][ty][tx + 1] + dtc) * h);
        }
        if (m3_xy) {  // V3 (I, J, K-1/2), cell m = (I, J, K-1)
            float r = mom3_m<float, G>(mm, d1, d2, d3, C1[I33][ty + 1][tx + 1] - C1[IP][ty + 1][tx + 1], q33, C1[I13][ty][tx + 1],
                                       C1[I13][ty][tx], C1[I23][ty + 1][tx], C1[I23][ty][tx]);
            if (G == CART && MODE == 0) r -= p.g * (h * (p.rho[g - d.sz] + S.old[K & 1][IX][ty + 1][tx + 1]));  // plane K-1's slot is being refilled
            if (MODE == 1) r += S.rv[K & 1][2][ty][tx];
            o.V3[g] = Vin[2][ty + 1][tx + 1] + r * ((C1[IX][ty + 1][tx + 1] + dtc) * h);
        }
    };

    // prologue: inputs kA-1, kA and old kA-1 (group A); inputs kA+1, old kA, rV kA (group B)
    issue_inputs(kA - 1);
    issue_inputs(kA);
    issue_old(kA - 1);
    cp_async_commit();
    issue_inputs(kA + 1);
    issue_old(kA);
    issue_rv(kA);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    if (kA >= 1) stage1(kA - 1, false);
    for (int K = kA; K < kB; ++K) {
        __syncthreads();  // slots of plane K-1 are free
        issue_inputs(K + 2);
        issue_old(K + 1);
        issue_rv(K + 1);
        cp_async_commit();
        cp_async_wait<1>();  // inputs K+1, old K, rV K have landed
        __syncthreads();
        stage1(K, true);
        __syncthreads();
        velocity(K);
    }
    cp_async_wait<0>();
}

inline size_t fused_smem_bytes() { return sizeof(FusedSmem); }

}  // namespace sph

// ===========================================================================
// TMA variant: the same sweep with the tile loads done by the Tensor Memory
// Accelerator (cp.async.bulk.tensor.3d, one elected thread per block, mbarrier
// transaction counts) instead of one cp.async per float.  Tiles start at
// x0-4 so the innermost coordinate is 16-byte aligned; out-of-range parts of
// a box (negative or past the end) are zero-filled by the TMA unit.
#include <cuda.h>

namespace sph {

enum TmaMap {
    TM_V1 = 0, TM_V2, TM_V3, TM_ETA, TM_ETASM,              // input boxes 40 x 10
    TM_P, TM_T11, TM_T22, TM_T33, TM_T12, TM_T13, TM_T23,  // old-state boxes 36 x 9
    TM_RP, TM_RHO,                                          // (36 x 9)
    TM_RV1, TM_RV2, TM_RV3,                                 // 32 x 8
    TM_COUNT
};
constexpr int TIN_X = 40, TIN_Y = 10, TOLD_X = 36, TOLD_Y = 9;
constexpr int TIN_TILE = 416;   // floats per input tile (400 used), 1664 B = 13 x 128 B
constexpr int TOLD_TILE = 352;  // floats per old-state tile (324 used), 1408 B = 11 x 128 B
constexpr int TRV_TILE = FTX * FTY;

struct TmaSmem {
    alignas(128) float in[3][F_IN][TIN_TILE];
    alignas(128) float old[2][F_OLD][TOLD_TILE];
    alignas(128) float rv[2][F_RV][TRV_TILE];
    float st[2][7][FSY][FSX];  // τ11-P, τ22-P, τ33-P, τ12, τ13, τ23, DT_R of planes K-1, K
    unsigned long long bar_in[3];
    unsigned long long bar_old[2];
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// bounded wait on the phase with the given parity; false if the bound ran out.
// Each try_wait suspends the thread until the phase completes or the suspend hint
// (kMbarSuspendNs) passes, so a waiting warp does not re-issue polls; kMbarMaxPolls
// of them bound the wait to about 2 s.  The bound is a count of polls, so the wait
// ends whatever the hint does.
constexpr unsigned kMbarSuspendNs = 200000;
constexpr int kMbarMaxPolls = 10000;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int max_polls = kMbarMaxPolls,
                                          unsigned suspend_ns = kMbarSuspendNs) {
    const unsigned a = smem_u32(bar);
    for (int it = 0; it < max_polls; ++it) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(a), "r"(parity), "r"(suspend_ns) : "memory");
        if (done) return true;
    }
    return false;
}

// Self-test of the bounded-wait error path of the TMA sweeps: one block waits on an
// mbarrier that nothing completes (initialised for one arrival, never arrived at, no
// copy issued), with the sweeps' wait at max_polls polls of suspend_ns; when the
// bound runs out it records 1 in *err as the sweep kernels do, and returns.
__global__ void k_wait_selftest(int* err, int max_polls, unsigned suspend_ns) {
    __shared__ unsigned long long bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(&bar, 0u, max_polls, suspend_ns)) atomicExch(err, 1);
}
__device__ __forceinline__ void tma_load3d(float* dst, const CUtensorMap* map, int x, int y, int z, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// store at a 32-bit unsigned byte offset from a field's base: the address is the
// base plus a zero-extended register, with no 64-bit index arithmetic per store
__device__ __forceinline__ void st_at(float* base, unsigned byte_off, float v) {
    *reinterpret_cast<float*>(reinterpret_cast<char*>(base) + byte_off) = v;
}

// Per-thread coefficients of the FP32 sweep's edge-strain and momentum stencils:
// the metric factors of sph_core.cuh (EdgeMetric at the stage-1 point, MomMetric
// at the velocity node) multiplied out with the spacings once per thread, so that
// each update below is a short chain of FMAs.  The expressions are those of
// edge12_m .. mom3_m regrouped (2 (x h) = x, 3 (x h) = 1.5 x): the same values up
// to FP32 rounding.
struct SweepCoef {
    float e12_d2, e12_h;          // τ12: iRh d2, iRh / 2
    float e13_d3, e13_h;          // τ13: iRh iSc1 d3, iRh / 2
    float e23_d2, e23_d3, e23_h;  // τ23: iRc1 d2, iRc1 iSh d3, iRc1 ctH / 2
    float m1_d2, m1_d3, m1_n, m1_t;  // V1: iR1 d2, iR1 iS1 d3, normal-stress and shear metric terms
    float m2_d2, m2_d3, m2_s, m2_n;  // V2: iR2 d2, iR2 iS2 d3, shear and normal-stress metric terms
    float m3_d3, m3_s, m3_n;         // V3: iR2 iS3 d3, shear metric terms
};
template <int G>
__device__ __forceinline__ SweepCoef sweep_coef(const EdgeMetric<float>& e, const MomMetric<float>& m, float d2, float d3) {
    SweepCoef c;
    if (G == SPH) {
        c.e12_d2 = e.iRh * d2; c.e12_h = 0.5f * e.iRh;
        c.e13_d3 = e.iRh * e.iSc1 * d3; c.e13_h = 0.5f * e.iRh;
        c.e23_d2 = e.iRc1 * d2; c.e23_d3 = e.iRc1 * e.iSh * d3; c.e23_h = 0.5f * e.iRc1 * e.ctH;
        c.m1_d2 = m.iR1 * d2; c.m1_d3 = m.iR1 * m.iS1 * d3; c.m1_n = m.iR1; c.m1_t = 0.5f * m.iR1 * m.ct1;
        c.m2_d2 = m.iR2 * d2; c.m2_d3 = m.iR2 * m.iS2 * d3; c.m2_s = 1.5f * m.iR2; c.m2_n = 0.5f * m.iR2 * m.ct2;
        c.m3_d3 = m.iR2 * m.iS3 * d3; c.m3_s = 1.5f * m.iR2; c.m3_n = m.iR2 * m.ct3;
    } else if (G == CYL) {
        c.e12_d2 = e.iRh * d2; c.e12_h = 0.5f * e.iRh;
        c.e13_d3 = d3; c.e13_h = 0.f;
        c.e23_d2 = e.iRc1 * d2; c.e23_d3 = d3; c.e23_h = 0.f;
        c.m1_d2 = m.iR1 * d2; c.m1_d3 = d3; c.m1_n = 0.5f * m.iR1; c.m1_t = 0.f;
        c.m2_d2 = m.iR2 * d2; c.m2_d3 = d3; c.m2_s = m.iR2; c.m2_n = 0.f;
        c.m3_d3 = d3; c.m3_s = 0.5f * m.iR2; c.m3_n = 0.f;
    } else {
        c.e12_d2 = d2; c.e12_h = 0.f; c.e13_d3 = d3; c.e13_h = 0.f; c.e23_d2 = d2; c.e23_d3 = d3; c.e23_h = 0.f;
        c.m1_d2 = d2; c.m1_d3 = d3; c.m1_n = 0.f; c.m1_t = 0.f;
        c.m2_d2 = d2; c.m2_d3 = d3; c.m2_s = 0.f; c.m2_n = 0.f;
        c.m3_d3 = d3; c.m3_s = 0.f; c.m3_n = 0.f;
    }
    return c;
}
// engineering shear strain rates at the edges (arguments as edge12_m .. edge23_m)
template <int G>
__device__ __forceinline__ float sw_edge12(const SweepCoef& c, float d1, float v2a, float v2b, float v1a, float v1b) {
    const float t = fmaf(c.e12_d2, v1b - v1a, (v2b - v2a) * d1);
    return G != CART ? fmaf(-c.e12_h, v2a + v2b, t) : t;
}
template <int G>
__device__ __forceinline__ float sw_edge13(const SweepCoef& c, float d1, float v3a, float v3b, float v1a, float v1b) {
    const float t = fmaf(c.e13_d3, v1b - v1a, (v3b - v3a) * d1);
    return G == SPH ? fmaf(-c.e13_h, v3a + v3b, t) : t;
}
template <int G>
__device__ __forceinline__ float sw_edge23(const SweepCoef& c, float v3a, float v3b, float v2a, float v2b) {
    const float t = fmaf(c.e23_d3, v2b - v2a, c.e23_d2 * (v3b - v3a));
    return G == SPH ? fmaf(-c.e23_h, v3a + v3b, t) : t;
}
// momentum residuals (arguments as mom1_m .. mom3_m)
template <int G>
__device__ __forceinline__ float sw_mom1(const SweepCoef& c, float d1, float s11m, float s11, float s22m, float s22, float s33m, float s33,
                                         float ta, float tb, float ua, float ub) {
    float r = fmaf(c.m1_d3, ua - ub, fmaf(c.m1_d2, ta - tb, (s11 - s11m) * d1));
    if (G == SPH) r = fmaf(c.m1_t, ta + tb, fmaf(c.m1_n, fmaf(-0.5f, (s22m + s22) + (s33m + s33), s11m + s11), r));
    if (G == CYL) r = fmaf(c.m1_n, (s11m + s11) - (s22m + s22), r);
    return r;
}
template <int G>
__device__ __forceinline__ float sw_mom2(const SweepCoef& c, float d1, float s22m, float s22, float s33m, float s33, float ta, float tb,
                                         float ua, float ub) {
    float r = fmaf(c.m2_d3, ua - ub, fmaf(c.m2_d2, s22 - s22m, (ta - tb) * d1));
    if (G != CART) r = fmaf(c.m2_s, ta + tb, r);
    if (G == SPH) r = fmaf(c.m2_n, (s22m + s22) - (s33m + s33), r);
    return r;
}
template <int G>
__device__ __forceinline__ float sw_mom3(const SweepCoef& c, float d1, float s33m, float s33, float ta, float tb, float ua, float ub) {
    float r = fmaf(c.m3_d3, s33 - s33m, fmaf(c.m2_d2, ua - ub, (ta - tb) * d1));
    if (G != CART) r = fmaf(c.m3_s, ta + tb, r);
    if (G == SPH) r = fmaf(c.m3_n, ua + ub, r);
    return r;
}

// edge stress update from the sums of the 4 surrounding cells' ηSM and η with
// gsc4 = GSDT/ηSM / 4: (τ + aG D) aE / (aE + aG), aG = gsc4 s4, aE = e4 / 4
__device__ __forceinline__ float edge_update_q(float told, float gsc4, float s4, float e4, float D) {
    const float aG = gsc4 * s4;
    return (told + aG * D) * pdiv(e4, fmaf(4.f, aG, e4));
}

// Waiting: warp 0 alone waits on the mbarriers of the planes a step needs and
// the block barrier that follows passes the completed copies on to the other
// warps, so nine of ten warps never poll.  A chunk copies only the planes it
// uses (inputs kA-1 .. kB, old state and rV kA-1 .. kB-1), so nothing is in
// flight when the march ends (unless a bounded wait ran out, see the end).
//
// Per-plane work is kept free of per-thread branching, which this kernel pays
// for in issue slots (it is instruction-bound): every stage-1 thread evaluates
// the cell and all three edges and every row thread all three velocity updates
// (the tiles hold finite or zero-filled values outside the box); validity masks
// only the stores and the stress-ring writes.  Planes 1 .. n3-3 run a body
// without the x3 conditions.  Stores take 32-bit unsigned byte offsets.  The
// x1-face ghost velocities of the homogeneous BC program's first stage are
// written here with the new values (FusedOut::xg_mask), so that stage is not
// launched.
//
// Thread roles (10 warps): warp w < 8 owns the row J = y0 + w of the tile, lane
// l the column I = x0 + l: it computes the stage-1 point (I, J) (a = l+1,
// b = w+1) and then the velocity node (I, J), taking its own point's stresses,
// step and velocities from registers.  Warp 8 computes the low-x2 halo row
// (b = 0), lanes 0..8 of warp 9 the low-x1 halo column (a = 0).  Shared-memory
// rows are then read by whole warps at consecutive addresses.
//
// The body takes the block's tile (bx, by) and x3 chunk (bz) as arguments, so that the
// single-grid kernel (block indices) and the batched kernel over many grids (a work
// list, sph_batch.cuh) run the same code.
template <int G, int MODE>
__device__ __forceinline__ void fused_tma_body(const KP<float>& p, const FusedOut<float>& o, int kchunk,
                                               const CUtensorMap* __restrict__ maps, int* __restrict__ err, int bx, int by, int bz) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TmaSmem& S = *reinterpret_cast<TmaSmem*>(smem_raw);
    enum { IP = 0, I11, I22, I33, I12, I13, I23, IX };  // old-tile slots (IX: rP | ρ)
    enum { Q11 = 0, Q22, Q33, E12, E13, E23, QDT };     // stress-ring slots

    const Dims d = p.d;
    const int tid = threadIdx.x;
    const int x0 = bx * FTX, y0 = by * FTY;
    const int kA = bz * kchunk;
    const int kB = min(kA + kchunk, d.n3);
    const int n1 = d.n1, n2 = d.n2, n3 = d.n3;
    const float d1 = p.d1, d2 = p.d2, d3 = p.d3, gsc = p.gsc, kbc = p.kbc, vpdt2 = p.vpdt2;
    if (kA >= kB) return;

    if (tid == 0) {
        for (int i = 0; i < 3; ++i) mbar_init(&S.bar_in[i], 1);
        for (int i = 0; i < 2; ++i) mbar_init(&S.bar_old[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    const unsigned in_bytes = F_IN * TIN_X * TIN_Y * 4;
    const unsigned old_bytes = F_OLD * TOLD_X * TOLD_Y * 4 + (MODE == 1 ? F_RV * FTX * FTY * 4 : 0);
    auto issue_inputs = [&](int z) {  // thread 0 only
        const int sl = (z + 3) % 3;
        mbar_expect_tx(&S.bar_in[sl], in_bytes);
        for (int f = 0; f < F_IN; ++f) tma_load3d(S.in[sl][f], maps + TM_V1 + f, x0 - 4, y0 - 1, z, &S.bar_in[sl]);
    };
    auto issue_old = [&](int z) {  // thread 0 only: old state + rV of plane z
        const int sl = z & 1;
        mbar_expect_tx(&S.bar_old[sl], old_bytes);
        for (int f = 0; f < 7; ++f) tma_load3d(S.old[sl][f], maps + TM_P + f, x0 - 4, y0 - 1, z, &S.bar_old[sl]);
        tma_load3d(S.old[sl][IX], maps + (MODE == 1 ? TM_RP : TM_RHO), x0 - 4, y0 - 1, z, &S.bar_old[sl]);
        if (MODE == 1)
            for (int f = 0; f < F_RV; ++f) tma_load3d(S.rv[sl][f], maps + TM_RV1 + f, x0, y0, z, &S.bar_old[sl]);
    };
    unsigned ph_in = 0, ph_old = 0;  // parity bit per ring slot
    // false once a bounded wait ran out: from then on this thread neither waits nor (thread 0)
    // issues copies, so the block finishes its march on whatever the tiles hold and exits
    bool ok = true;
    auto wait_in = [&](int z) {
        if (!ok) return;
        const int sl = (z + 3) % 3;
        ok = mbar_wait(&S.bar_in[sl], (ph_in >> sl) & 1u);
        ph_in ^= 1u << sl;
    };
    auto wait_old = [&](int z) {
        if (!ok) return;
        const int sl = z & 1;
        ok = mbar_wait(&S.bar_old[sl], (ph_old >> sl) & 1u);
        ph_old ^= 1u << sl;
    };

    // per-thread constants of the whole march
    const int warp = tid >> 5, lane = tid & 31;
    const int a = warp < FTY ? lane + 1 : (warp == FTY ? lane + 1 : 0);
    const int b = warp < FTY ? warp + 1 : (warp == FTY ? 0 : lane);
    const bool s1_thread = warp <= FTY || lane <= FTY;
    const int x = x0 - 1 + a, y = y0 - 1 + b;
    const bool s1_in = s1_thread && x >= 0 && y >= 0 && x < n1 && y < n2;
    const bool s1_own = warp < FTY;
    const bool e12_xy = x < n1 - 1 && y < n2 - 1, e13_xy = x < n1 - 1 && y < n2 - 2, e23_xy = x < n1 - 2 && y < n2 - 1;
    const CellMetric<float> cm = cell_metric_t<float, G>(p.geo, d2, d3, clampi(x, 0, n1 - 1), clampi(y, 0, n2 - 1));
    const int gxy = x + d.sy * y;
    const bool y_face = y == 0 || y == n2 - 1;  // stage-1 point on an x2 face of the box
    const bool fs_top = p.fs && x == n1 - 1;    // stage-1 point in a free-surface top cell
    const int iin = b * TIN_X + a + 3;   // input-tile index of the stage-1 point
    const int iold = b * TOLD_X + a + 3; // old-tile index of the stage-1 point
    const int tx = lane, ty = warp;      // velocity node (warps < FTY)
    const int I = x0 + tx, J = y0 + ty;
    const bool v_ok = warp < FTY && I >= 1 && J >= 1 && I <= n1 - 1 && J <= n2 - 1;
    const bool m1_xy = J <= n2 - 2, m2_xy = I <= n1 - 2, m3_xy = I <= n1 - 2 && J <= n2 - 2;
    const SweepCoef sc = sweep_coef<G>(edge_metric<float, G>(p.geo, x, y, n1, n2), mom_metric<float, G>(p.geo, I, J, n1, n2), d2, d3);
    const int gIJ = I + d.sy * J;

    // this thread's stage-1 point of the current plane, and carried values of the previous plane
    float o11 = 0.f, o22 = 0.f, o33 = 0.f, odt = 0.f, ov1 = 0.f, ov2 = 0.f, ov3 = 0.f;
    float p33 = 0.f, pdt = 0.f, p13 = 0.f, p23 = 0.f;
    const float gsc4 = 0.25f * gsc;
    // stage1 / velocity of an interior plane (1 <= k <= n3 - 3: every x3 condition holds
    // and no x3 face is a traction face) when `inner` is std::true_type
    auto stage1 = [&](int k, bool own_plane, int sk, auto inner) {
        constexpr bool IN = decltype(inner)::value;
        if (!s1_thread) return;
        const float* I0 = S.in[sk][0] + iin;
        const float* I1 = S.in[sk == 2 ? 0 : sk + 1][0] + iin;
        auto in0 = [&](int f, int db, int da) { return I0[f * TIN_TILE + db * TIN_X + da]; };
        auto in1 = [&](int f, int db, int da) { return I1[f * TIN_TILE + db * TIN_X + da]; };
        const float* O = &S.old[k & 1][0][0] + iold;
        auto old = [&](int f) { return O[f * TOLD_TILE]; };
        const bool own = own_plane && s1_own;
        const int g = gxy + d.sz * k;
        const unsigned gb = 4u * (unsigned)g;  // byte offset (owned points only: g >= 0)
        // every stage-1 thread evaluates all stencils (the tiles hold finite or zero-filled
        // values at points outside the box); validity masks only the stores and the ring
        const bool k12 = IN || k < n3 - 2, k1x = IN || k < n3 - 1;
        ov1 = in0(0, 0, 0); ov2 = in0(1, 0, 0); ov3 = in0(2, 0, 0);
        float vP, v11, v22, v33, vdt, v12, v13, v23;
        {
            const CellD<float> D = cell_strain_m<float, G>(cm, d1, ov1, in0(0, 0, 1), ov2, in0(1, 1, 0), ov3, in1(2, 0, 0));
            const float sm = in0(4, 0, 0), e = in0(3, 0, 0);
            const float gs = gsc * sm, kb = kbc * sm;
            const float f = pdiv(e, e + gs);
            float dv = D.div;
            if (MODE == 1) dv += old(IX);
            vP = old(IP) - kb * dv;
            v11 = (old(I11) + 2.f * gs * D.D11) * f;
            v22 = (old(I22) + 2.f * gs * D.D22) * f;
            v33 = (old(I33) + 2.f * gs * D.D33) * f;
            if (IN) {
                if (p.traction && y_face) vP = v22 - p.sig2;
            } else if (p.traction) {
                traction_pressure(y, k, n2, n3, v22, v33, p.sig2, p.sig3, vP);
            }
            // free-surface top cell (the correction problem is homogeneous: no load)
            if (fs_top) vP = fs_pressure(v11, MODE == 1 ? 0.f : p.top_load[g], p.fs_kappa, ov1, in0(0, 0, 1));
            vdt = pdiv(vpdt2, kb + gs * f);
        }
        {
            const float D = sw_edge12<G>(sc, d1, in1(1, 1, 0), in1(1, 1, 1), in1(0, 0, 1), in1(0, 1, 1));
            v12 = edge_update_q(old(I12), gsc4, in1(4, 0, 0) + in1(4, 1, 0) + in1(4, 0, 1) + in1(4, 1, 1),
                                in1(3, 0, 0) + in1(3, 1, 0) + in1(3, 0, 1) + in1(3, 1, 1), D);
        }
        {
            const float D = sw_edge13<G>(sc, d1, in1(2, 1, 0), in1(2, 1, 1), in0(0, 1, 1), in1(0, 1, 1));
            v13 = edge_update_q(old(I13), gsc4, in0(4, 1, 0) + in1(4, 1, 0) + in0(4, 1, 1) + in1(4, 1, 1),
                                in0(3, 1, 0) + in1(3, 1, 0) + in0(3, 1, 1) + in1(3, 1, 1), D);
        }
        {
            const float D = sw_edge23<G>(sc, in1(2, 0, 1), in1(2, 1, 1), in0(1, 1, 1), in1(1, 1, 1));
            v23 = edge_update_q(old(I23), gsc4, in0(4, 0, 1) + in1(4, 0, 1) + in0(4, 1, 1) + in1(4, 1, 1),
                                in0(3, 0, 1) + in1(3, 0, 1) + in0(3, 1, 1) + in1(3, 1, 1), D);
        }
        const bool ok12 = s1_in && e12_xy && k12, ok13 = s1_in && e13_xy && k1x, ok23 = s1_in && e23_xy && k1x;
        if (own && s1_in) { st_at(o.P, gb, vP); st_at(o.t11, gb, v11); st_at(o.t22, gb, v22); st_at(o.t33, gb, v33); }
        if (own && ok12) st_at(o.t12, gb, v12);
        if (own && ok13) st_at(o.t13, gb, v13);
        if (own && ok23) st_at(o.t23, gb, v23);
        if (!s1_in) { vP = 0.f; v11 = 0.f; v22 = 0.f; v33 = 0.f; vdt = 0.f; }
        if (!ok12) v12 = 0.f;
        if (!ok13) v13 = 0.f;
        if (!ok23) v23 = 0.f;
        o11 = v11 - vP; o22 = v22 - vP; o33 = v33 - vP; odt = vdt;
        float (*W)[FSY][FSX] = S.st[k & 1];
        W[Q11][b][a] = o11; W[Q22][b][a] = o22; W[Q33][b][a] = o33;
        W[E12][b][a] = v12; W[E13][b][a] = v13; W[E23][b][a] = v23; W[QDT][b][a] = vdt;
    };

    // velocities of plane K from the stresses of planes K-1 and K
    auto velocity = [&](int K, auto inner) {
        constexpr bool IN = decltype(inner)::value;
        if (warp >= FTY) return;
        float (*C0)[FSY][FSX] = S.st[K & 1];
        float (*C1)[FSY][FSX] = S.st[(K - 1) & 1];
        if (!IN && K == kA) { p13 = C1[E13][ty][tx]; p23 = C1[E23][ty][tx]; }
        const float c13 = C0[E13][ty][tx], c23 = C0[E23][ty][tx];
        if (IN || (K >= 1 && K <= n3 - 1)) {
            // all three updates evaluated by every row thread; validity masks the stores
            const unsigned gb = 4u * (unsigned)(gIJ + d.sz * K);  // byte offset (valid nodes only: >= 0)
            const float h = 0.5f;
            const float t12a = C1[E12][ty + 1][tx], t12b = C1[E12][ty][tx];
            // V1 (I-1/2, J, K), cell m = (I-1, J, K)
            float r1 = sw_mom1<G>(sc, d1, C0[Q11][ty + 1][tx], o11, C0[Q22][ty + 1][tx], o22, C0[Q33][ty + 1][tx], o33,
                                        t12a, t12b, c13, p13);
            // V2 (I, J-1/2, K), cell m = (I, J-1, K)
            float r2 = sw_mom2<G>(sc, d1, C0[Q22][ty][tx + 1], o22, C0[Q33][ty][tx + 1], o33, C1[E12][ty][tx + 1], t12b,
                                        c23, p23);
            // V3 (I, J, K-1/2), cell m = (I, J, K-1)
            float r3 = sw_mom3<G>(sc, d1, p33, o33, C1[E13][ty][tx + 1], p13, C1[E23][ty + 1][tx], p23);
            if (MODE == 1) {
                r1 += S.rv[K & 1][0][ty * FTX + tx];
                r2 += S.rv[K & 1][1][ty * FTX + tx];
                r3 += S.rv[K & 1][2][ty * FTX + tx];
            }
            const bool kin = IN || K <= n3 - 2;
            const float v1 = ov1 + r1 * ((C0[QDT][ty + 1][tx] + odt) * h);
            const float v2 = ov2 + r2 * ((C0[QDT][ty][tx + 1] + odt) * h);
            const float v3 = ov3 + r3 * ((pdt + odt) * h);
            if (v_ok && m1_xy && kin) {
                st_at(o.V1, gb, v1);
                if ((o.xg_mask & 1) && (I == 1 || I == n1 - 1)) st_at(o.V1, I == 1 ? gb - 4u : gb + 4u, o.xg[0] * v1);
            }
            if (v_ok && m2_xy && kin) {
                st_at(o.V2, gb, v2);
                if ((o.xg_mask & 2) && (I == 1 || I == n1 - 2)) st_at(o.V2, I == 1 ? gb - 4u : gb + 4u, o.xg[1] * v2);
            }
            if (v_ok && m3_xy) {
                st_at(o.V3, gb, v3);
                if ((o.xg_mask & 4) && (I == 1 || I == n1 - 2)) st_at(o.V3, I == 1 ? gb - 4u : gb + 4u, o.xg[2] * v3);
            }
        }
        p13 = c13; p23 = c23; p33 = o33; pdt = odt;
    };

    // prologue: inputs kA-1, kA, kA+1; old kA-1, kA
    if (tid == 0) {
        issue_inputs(kA - 1);
        issue_inputs(kA);
        issue_old(kA - 1);
        issue_inputs(kA + 1);
        issue_old(kA);
    }
    const bool waiter = warp == 0;
    if (waiter) {
        wait_in(kA - 1);
        wait_in(kA);
        wait_old(kA - 1);
    }
    __syncthreads();
    int sk = (kA + 2) % 3;  // input-ring slot of plane kA - 1
    if (kA >= 1) {
        stage1(kA - 1, false, sk, std::false_type{});
        p33 = o33;
        pdt = odt;
    }
    auto step = [&](int K, auto inner) {
        if (waiter) {
            wait_in(K + 1);
            wait_old(K);
        }
        __syncthreads();  // every thread is done with the slots of plane K-1; inputs K+1 and old K have landed
        if (tid == 0 && ok) {  // only planes the chunk uses: inputs up to kB, old state and rV up to kB - 1
            if (K + 2 <= kB) issue_inputs(K + 2);
            if (K + 1 <= kB - 1) issue_old(K + 1);
        }
        sk = sk == 2 ? 0 : sk + 1;
        stage1(K, true, sk, inner);
        __syncthreads();
        velocity(K, inner);
    };
    step(kA, std::false_type{});  // (sets the carried edge stresses of plane kA - 1)
    for (int K = kA + 1; K < kB; ++K) {
        if (K <= n3 - 3) step(K, std::true_type{});
        else step(K, std::false_type{});
    }
    // Without a time-out every issued copy has been waited for, so none is in flight when the
    // block exits.  After a time-out copies issued before it may still be landing in this
    // block's shared memory as it exits and the state it wrote is suspect: the host reads the
    // flag after the launch and treats it as fatal for the context.
    if (waiter && !ok && err) atomicExch(err, 1);
}

template <int G, int MODE>
__global__ void __launch_bounds__(FNT, 3) k_fused_tma(KP<float> p, FusedOut<float> o, int kchunk, const CUtensorMap* __restrict__ maps,
                                                       int* __restrict__ err) {
    pdl_wait();  // no early release of the next grid: its blocks would take SM slots in this grid's tail
    fused_tma_body<G, MODE>(p, o, kchunk, maps, err, blockIdx.x, blockIdx.y, blockIdx.z);
}

inline size_t fused_tma_smem_bytes() { return sizeof(TmaSmem); }

}  // namespace sph
