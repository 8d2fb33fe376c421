// Fused FP32 PT correction sweep, two x1-adjacent points per thread.
//
// The same 2.5D march, TMA tile loads and ring buffers as k_fused_tma
// (sph_fused.cuh): tile 32 x 8 cells per block, inputs of planes K..K+2 in a
// 3-slot ring, old state of planes K, K+1 in a 2-slot ring, new stresses of
// planes K-1, K in a shared ring.  What changes is the work of a thread: it
// owns the pair of points (a, a+1) of one row and evaluates the shared
// stencil templates with T = F2, so every arithmetic instruction serves two
// points (paired FP32 instructions), pairs of neighbours come from one 8-byte
// shared-memory load where the pair is 8-byte aligned, and the owned results
// go to HBM as 8-byte stores.
//
// Thread roles (5 warps):
//   warps 0..3   lane l: row b = 2w + l/16 + 1, points a = 2(l%16) + 1, +2
//                (x1 = x0 + 2(l%16), +1); afterwards the velocity nodes
//                (x0 + 2(l%16) + {0,1}, y0 + b - 1), whose own stage-1 points
//                these are;
//   warp 4       lanes 0..15: halo row b = 0, points a = 2l + 1, +2;
//                lanes 16..24: halo column, points (a = -1, 0) of row b = l-16
//                (a = -1 is computed and discarded; it keeps the pair aligned).
// Stage-1 point (a, b) is the cell (x0 - 1 + a, y0 - 1 + b).  Stress-ring
// rows hold a = -1..32 at offset a + 1 (34 floats), so the pairs a = 2l+1,
// 2l+2 are 8-byte aligned there as in the TMA tiles (offset a + 3, x0 - 4
// box origin) and in HBM (rows of 32-multiple pitch).
//
// Correction problem only (right-hand sides rP, rV; η, ηSM frozen):
// SphericalStokes_diapir.jl:209-241 and :267-329 with the right-hand sides of
// the defect-correction step.
#pragma once
#include "sph_f2.cuh"
#include "sph_fused.cuh"

namespace sph {

constexpr int X2_NT = 160;   // threads per block
constexpr int X2_SROW = 34;  // stress-ring row: a = -1..32

struct X2Smem {
    alignas(128) float in[3][F_IN][TIN_TILE];
    alignas(128) float old[2][F_OLD][TOLD_TILE];
    alignas(128) float rv[2][F_RV][TRV_TILE];
    alignas(16) float st[2][7][FSY * X2_SROW];  // τ11-P, τ22-P, τ33-P, τ12, τ13, τ23, DT_R of planes K-1, K
    unsigned long long bar_in[3];
    unsigned long long bar_old[2];
};

inline size_t sweep_x2_smem_bytes() { return sizeof(X2Smem); }

template <int G>
__device__ __forceinline__ CellMetric<F2> cell_metric_pair(const Geo<float>& geo, float d2, float d3, int xa, int y, int n1, int n2) {
    const CellMetric<float> p = cell_metric_t<float, G>(geo, d2, d3, clampi(xa, 0, n1 - 1), clampi(y, 0, n2 - 1));
    const CellMetric<float> q = cell_metric_t<float, G>(geo, d2, d3, clampi(xa + 1, 0, n1 - 1), clampi(y, 0, n2 - 1));
    CellMetric<F2> m;
    m.a2 = F2(p.a2, q.a2); m.a3 = F2(p.a3, q.a3); m.c1 = F2(p.c1, q.c1); m.c2 = F2(p.c2, q.c2);
    m.e1 = F2(p.e1, q.e1); m.e1b = F2(p.e1b, q.e1b); m.e2 = F2(p.e2, q.e2);
    return m;
}
template <int G>
__device__ __forceinline__ EdgeMetric<F2> edge_metric_pair(const Geo<float>& geo, int xa, int y, int n1, int n2) {
    const EdgeMetric<float> p = edge_metric<float, G>(geo, xa, y, n1, n2);
    const EdgeMetric<float> q = edge_metric<float, G>(geo, xa + 1, y, n1, n2);
    EdgeMetric<F2> m;
    m.iRh = F2(p.iRh, q.iRh); m.iSc1 = F2(p.iSc1, q.iSc1); m.iRc1 = F2(p.iRc1, q.iRc1);
    m.iSh = F2(p.iSh, q.iSh); m.ctH = F2(p.ctH, q.ctH);
    return m;
}
template <int G>
__device__ __forceinline__ MomMetric<F2> mom_metric_pair(const Geo<float>& geo, int Ia, int J, int n1, int n2) {
    const MomMetric<float> p = mom_metric<float, G>(geo, Ia, J, n1, n2);
    const MomMetric<float> q = mom_metric<float, G>(geo, Ia + 1, J, n1, n2);
    MomMetric<F2> m;
    m.iR1 = F2(p.iR1, q.iR1); m.iS1 = F2(p.iS1, q.iS1); m.ct1 = F2(p.ct1, q.ct1);
    m.iR2 = F2(p.iR2, q.iR2); m.iS2 = F2(p.iS2, q.iS2); m.ct2 = F2(p.ct2, q.ct2);
    m.iS3 = F2(p.iS3, q.iS3); m.ct3 = F2(p.ct3, q.ct3);
    return m;
}

// 8-byte store of a pair when both lanes are wanted, else lane by lane; `off` is the
// 32-bit unsigned byte offset of the first point from the field's base
__device__ __forceinline__ void store_pair(float* base, unsigned off, F2 v, bool m0, bool m1) {
    char* q = reinterpret_cast<char*>(base) + off;
    if (m0 && m1) {
        *reinterpret_cast<float2*>(q) = v.v;
    } else {
        if (m0) *reinterpret_cast<float*>(q) = v.v.x;
        if (m1) *reinterpret_cast<float*>(q + 4) = v.v.y;
    }
}

template <int G>
__global__ void __launch_bounds__(X2_NT, 3) k_sweep_x2(KP<float> p, FusedOut<float> o, int kchunk, const CUtensorMap* __restrict__ maps,
                                                        int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    X2Smem& S = *reinterpret_cast<X2Smem*>(smem_raw);
    enum { IP = 0, I11, I22, I33, I12, I13, I23, IX };  // old-tile slots (IX: rP)
    enum { Q11 = 0, Q22, Q33, E12, E13, E23, QDT };     // stress-ring slots

    const Dims d = p.d;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * FTX, y0 = blockIdx.y * FTY;
    const int kA = blockIdx.z * kchunk;
    const int kB = min(kA + kchunk, d.n3);
    const int n1 = d.n1, n2 = d.n2, n3 = d.n3;
    if (kA >= kB) return;

    if (tid == 0) {
        for (int i = 0; i < 3; ++i) mbar_init(&S.bar_in[i], 1);
        for (int i = 0; i < 2; ++i) mbar_init(&S.bar_old[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    const unsigned in_bytes = F_IN * TIN_X * TIN_Y * 4;
    const unsigned old_bytes = F_OLD * TOLD_X * TOLD_Y * 4 + F_RV * FTX * FTY * 4;
    auto issue_inputs = [&](int z) {  // thread 0 only
        const int sl = (z + 3) % 3;
        mbar_expect_tx(&S.bar_in[sl], in_bytes);
        for (int f = 0; f < F_IN; ++f) tma_load3d(S.in[sl][f], maps + TM_V1 + f, x0 - 4, y0 - 1, z, &S.bar_in[sl]);
    };
    auto issue_old = [&](int z) {  // thread 0 only: old state, rP and rV of plane z
        const int sl = z & 1;
        mbar_expect_tx(&S.bar_old[sl], old_bytes);
        for (int f = 0; f < 7; ++f) tma_load3d(S.old[sl][f], maps + TM_P + f, x0 - 4, y0 - 1, z, &S.bar_old[sl]);
        tma_load3d(S.old[sl][IX], maps + TM_RP, x0 - 4, y0 - 1, z, &S.bar_old[sl]);
        for (int f = 0; f < F_RV; ++f) tma_load3d(S.rv[sl][f], maps + TM_RV1 + f, x0, y0, z, &S.bar_old[sl]);
    };
    unsigned ph_in = 0, ph_old = 0;  // parity bit per ring slot
    // false once a bounded wait ran out: no further waits or copies (as in k_fused_tma)
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

    // ---- per-thread constants of the whole march
    const int warp = tid >> 5, lane = tid & 31, lp = lane & 15;
    const bool main_warp = warp < 4;
    int a, b;
    bool s1_thread = true;
    if (main_warp) { a = 2 * lp + 1; b = 2 * warp + (lane >> 4) + 1; }
    else if (lane < 16) { a = 2 * lp + 1; b = 0; }
    else { a = -1; b = lane - 16; s1_thread = b <= FTY; }
    const int x = x0 - 1 + a, y = y0 - 1 + b;  // first point of the pair
    const bool yin = y >= 0 && y < n2;
    const bool in0 = s1_thread && a >= 0 && x >= 0 && x < n1 && yin;  // a = -1 is never a result
    const bool in1 = s1_thread && x + 1 >= 0 && x + 1 < n1 && yin;
    const bool e12_0 = x < n1 - 1 && y < n2 - 1, e12_1 = x + 1 < n1 - 1 && y < n2 - 1;
    const bool e13_0 = x < n1 - 1 && y < n2 - 2, e13_1 = x + 1 < n1 - 1 && y < n2 - 2;
    const bool e23_0 = x < n1 - 2 && y < n2 - 1, e23_1 = x + 1 < n1 - 2 && y < n2 - 1;
    const CellMetric<F2> cm = cell_metric_pair<G>(p.geo, p.d2, p.d3, x, y, n1, n2);
    const EdgeMetric<F2> em = edge_metric_pair<G>(p.geo, x, y, n1, n2);
    const int gxy = x + d.sy * y;
    const int iin = b * TIN_X + a + 3;       // input-tile offset of the first point (even)
    const int iold = b * TOLD_X + a + 3;     // old-tile offset (even)
    const int ist = b * X2_SROW + a + 1;     // stress-ring offset (even)
    const F2 d1(p.d1), d2(p.d2), d3(p.d3), gsc(p.gsc), kbc(p.kbc), vpdt2(p.vpdt2);

    // velocity nodes (main warps): (I, J), (I+1, J) with I = x, J = y; own stage-1 points
    const int I = x, J = y;
    const bool vrow = main_warp && J >= 1 && J <= n2 - 1;
    const bool v0 = vrow && I >= 1 && I <= n1 - 1, v1 = vrow && I + 1 >= 1 && I + 1 <= n1 - 1;
    const bool m1_xy = J <= n2 - 2;
    const bool m2_0 = I <= n1 - 2, m2_1 = I + 1 <= n1 - 2;
    const MomMetric<F2> mm = mom_metric_pair<G>(p.geo, I, J, n1, n2);
    const int irv = (b - 1) * FTX + (a - 1);  // rV-tile offset of node I (even)

    // this thread's pair at the current plane, and carried values of the previous plane
    F2 o11(0.f), o22(0.f), o33(0.f), odt(0.f), ov1(0.f), ov2(0.f), ov3(0.f);
    float o12 = 0.f, o23 = 0.f;                 // own first point's τ12, τ23 (ring values of the node's -x neighbour)
    F2 p13(0.f), p23(0.f), p33(0.f), pdt(0.f);  // previous plane: ring τ13, τ23 at (a-1, b-1), (a, b-1); own τ33-P, DT_R
    float pe12 = 0.f, pe23 = 0.f;               // previous plane: own first point's τ12, τ23

    auto stage1 = [&](int k, bool own_plane) {
        if (!s1_thread) return;
        const float* A0 = S.in[(k + 3) % 3][0] + iin;  // plane k
        const float* A1 = S.in[(k + 4) % 3][0] + iin;  // plane k+1
        // the pair (da, da+1) of field f, row offset db, of plane A (da compile-time after inlining)
        auto pr = [&](const float* A, int f, int db, int da) {
            const float* q = A + f * TIN_TILE + db * TIN_X + da;
            if ((da & 1) == 0) return F2(*reinterpret_cast<const float2*>(q));
            return F2(q[0], q[1]);
        };
        const float* O = &S.old[k & 1][0][0] + iold;
        auto old = [&](int f) { return F2(*reinterpret_cast<const float2*>(O + f * TOLD_TILE)); };
        const bool own = own_plane && main_warp;
        const unsigned g = 4u * (unsigned)(gxy + d.sz * k);  // byte offset (stored points only: >= 0)
        F2 vP(0.f), v11(0.f), v22(0.f), v33(0.f), vdt(0.f), v12(0.f), v13(0.f), v23(0.f);
        if (in0 || in1) {
            {
                const F2 v1m = pr(A0, 0, 0, 0), v1p = pr(A0, 0, 0, 1);
                const F2 v2m = pr(A0, 1, 0, 0), v2p = pr(A0, 1, 1, 0);
                const F2 v3m = pr(A0, 2, 0, 0), v3p = pr(A1, 2, 0, 0);
                ov1 = v1m; ov2 = v2m; ov3 = v3m;
                const CellD<F2> D = cell_strain_m<F2, G>(cm, d1, v1m, v1p, v2m, v2p, v3m, v3p);
                const F2 sm = pr(A0, 4, 0, 0), e = pr(A0, 3, 0, 0);
                const F2 gs = gsc * sm, kb = kbc * sm;
                const F2 f = pdiv(e, e + gs);
                const F2 gs2 = gs + gs;
                vP = old(IP) - kb * (D.div + old(IX));
                v11 = (old(I11) + gs2 * D.D11) * f;
                v22 = (old(I22) + gs2 * D.D22) * f;
                v33 = (old(I33) + gs2 * D.D33) * f;
                if (p.traction) {  // far-field normal stress on the x2 / x3 faces (same y, k for both lanes)
                    const bool b2 = (y == 0 || y == n2 - 1), b3 = (k == 0 || k == n3 - 1);
                    if (b2 && b3) vP = ((v22 - F2(p.sig2)) + (v33 - F2(p.sig3))) * F2(0.5f);
                    else if (b2) vP = v22 - F2(p.sig2);
                    else if (b3) vP = v33 - F2(p.sig3);
                }
                vdt = pdiv(vpdt2, kb + gs * f);
                if (!(in0 && in1)) {
                    vP = keep(vP, in0, in1); v11 = keep(v11, in0, in1); v22 = keep(v22, in0, in1);
                    v33 = keep(v33, in0, in1); vdt = keep(vdt, in0, in1);
                }
                if (own) {
                    store_pair(o.P, g, vP, in0, in1); store_pair(o.t11, g, v11, in0, in1);
                    store_pair(o.t22, g, v22, in0, in1); store_pair(o.t33, g, v33, in0, in1);
                }
            }
            if ((e12_0 || e12_1) && k < n3 - 2) {
                const F2 s0 = pr(A1, 4, 0, 0), s1 = pr(A1, 4, 1, 0), s2 = pr(A1, 4, 0, 1), s3 = pr(A1, 4, 1, 1);
                const F2 t0 = pr(A1, 3, 0, 0), t1 = pr(A1, 3, 1, 0), t2 = pr(A1, 3, 0, 1), t3 = pr(A1, 3, 1, 1);
                const F2 D = edge12_m<F2, G>(em, d1, d2, pr(A1, 1, 1, 0), pr(A1, 1, 1, 1), pr(A1, 0, 0, 1), pr(A1, 0, 1, 1));
                v12 = keep(edge_update(old(I12), gsc, s0 + s1 + s2 + s3, t0 + t1 + t2 + t3, D), e12_0 && in0, e12_1 && in1);
                if (own) store_pair(o.t12, g, v12, e12_0 && in0, e12_1 && in1);
            }
            if ((e13_0 || e13_1) && k < n3 - 1) {
                const F2 s0 = pr(A0, 4, 1, 0), s1 = pr(A1, 4, 1, 0), s2 = pr(A0, 4, 1, 1), s3 = pr(A1, 4, 1, 1);
                const F2 t0 = pr(A0, 3, 1, 0), t1 = pr(A1, 3, 1, 0), t2 = pr(A0, 3, 1, 1), t3 = pr(A1, 3, 1, 1);
                const F2 D = edge13_m<F2, G>(em, d1, d3, pr(A1, 2, 1, 0), pr(A1, 2, 1, 1), pr(A0, 0, 1, 1), pr(A1, 0, 1, 1));
                v13 = keep(edge_update(old(I13), gsc, s0 + s1 + s2 + s3, t0 + t1 + t2 + t3, D), e13_0 && in0, e13_1 && in1);
                if (own) store_pair(o.t13, g, v13, e13_0 && in0, e13_1 && in1);
            }
            if ((e23_0 || e23_1) && k < n3 - 1) {
                const F2 s0 = pr(A0, 4, 0, 1), s1 = pr(A1, 4, 0, 1), s2 = pr(A0, 4, 1, 1), s3 = pr(A1, 4, 1, 1);
                const F2 t0 = pr(A0, 3, 0, 1), t1 = pr(A1, 3, 0, 1), t2 = pr(A0, 3, 1, 1), t3 = pr(A1, 3, 1, 1);
                const F2 D = edge23_m<F2, G>(em, d2, d3, pr(A1, 2, 0, 1), pr(A1, 2, 1, 1), pr(A0, 1, 1, 1), pr(A1, 1, 1, 1));
                v23 = keep(edge_update(old(I23), gsc, s0 + s1 + s2 + s3, t0 + t1 + t2 + t3, D), e23_0 && in0, e23_1 && in1);
                if (own) store_pair(o.t23, g, v23, e23_0 && in0, e23_1 && in1);
            }
        }
        o11 = v11 - vP; o22 = v22 - vP; o33 = v33 - vP; odt = vdt;
        o12 = v12.v.x; o23 = v23.v.x;
        float* W = &S.st[k & 1][0][0] + ist;
        constexpr int RS = FSY * X2_SROW;
        *reinterpret_cast<float2*>(W + Q11 * RS) = o11.v;
        *reinterpret_cast<float2*>(W + Q22 * RS) = o22.v;
        *reinterpret_cast<float2*>(W + Q33 * RS) = o33.v;
        *reinterpret_cast<float2*>(W + E12 * RS) = v12.v;
        *reinterpret_cast<float2*>(W + E13 * RS) = v13.v;
        *reinterpret_cast<float2*>(W + E23 * RS) = v23.v;
        *reinterpret_cast<float2*>(W + QDT * RS) = vdt.v;
    };

    // velocities of plane K at the nodes (I, J), (I+1, J) from the stresses of planes K-1 and K
    auto velocity = [&](int K) {
        if (!main_warp) return;
        constexpr int RS = FSY * X2_SROW;
        const float* C0 = &S.st[K & 1][0][0];
        const float* C1 = &S.st[(K - 1) & 1][0][0];
        // ring offsets: node row (b-1 = J - y0) and own row b, columns a-1 (-x neighbour), a (own), a+1
        const int rUp = ist - X2_SROW;  // (a, b-1)
        const int rOwn = ist;           // (a, b)
        auto pairU = [&](const float* C, int f, int da) {  // row b-1, columns a-1+da, a+da
            const float* q = C + f * RS + rUp - 1 + da;
            if ((da & 1) == 1) return F2(*reinterpret_cast<const float2*>(q));
            return F2(q[0], q[1]);
        };
        if (K == kA) { p13 = pairU(C1, E13, 0); p23 = pairU(C1, E23, 0); }
        const F2 c13 = pairU(C0, E13, 0), c23 = pairU(C0, E23, 0);
        if ((v0 || v1) && K >= 1 && K <= n3 - 1) {
            const unsigned g = 4u * (unsigned)(gxy + d.sz * K);  // byte offset of node I = x, J = y
            const F2 h(0.5f);
            const F2 t12a = F2(C1[E12 * RS + rOwn - 1], pe12);  // τ12 at (a-1, b), (a, b) of plane K-1
            const F2 t12b = pairU(C1, E12, 0);                   // τ12 at (a-1, b-1), (a, b-1)
            const float* RV = &S.rv[K & 1][0][0] + irv;
            if (m1_xy && K <= n3 - 2) {  // V1 (I-1/2, J, K): cell m = (I-1, J, K)
                const F2 s11m = F2(C0[Q11 * RS + rOwn - 1], o11.v.x), s22m = F2(C0[Q22 * RS + rOwn - 1], o22.v.x);
                const F2 s33m = F2(C0[Q33 * RS + rOwn - 1], o33.v.x), dtm = F2(C0[QDT * RS + rOwn - 1], odt.v.x);
                F2 r = mom1_m<F2, G>(mm, d1, d2, d3, s11m, o11, s22m, o22, s33m, o33, t12a, t12b, c13, p13);
                r = r + F2(*reinterpret_cast<const float2*>(RV));
                store_pair(o.V1, g, ov1 + r * ((dtm + odt) * h), v0, v1);
            }
            if ((m2_0 || m2_1) && K <= n3 - 2) {  // V2 (I, J-1/2, K): cell m = (I, J-1, K)
                const F2 s22m = pairU(C0, Q22, 1), s33m = pairU(C0, Q33, 1), dtm = pairU(C0, QDT, 1);
                F2 r = mom2_m<F2, G>(mm, d1, d2, d3, s22m, o22, s33m, o33, pairU(C1, E12, 1), t12b, c23, p23);
                r = r + F2(*reinterpret_cast<const float2*>(RV + F_RV * 0 + TRV_TILE));
                store_pair(o.V2, g, ov2 + r * ((dtm + odt) * h), v0 && m2_0, v1 && m2_1);
            }
            if ((m2_0 || m2_1) && m1_xy) {  // V3 (I, J, K-1/2): cell m = (I, J, K-1)
                const F2 t23a = F2(C1[E23 * RS + rOwn - 1], pe23);  // τ23 at (a-1, b), (a, b) of plane K-1
                F2 r = mom3_m<F2, G>(mm, d1, d2, d3, p33, o33, pairU(C1, E13, 1), p13, t23a, p23);
                r = r + F2(*reinterpret_cast<const float2*>(RV + 2 * TRV_TILE));
                store_pair(o.V3, g, ov3 + r * ((pdt + odt) * h), v0 && m2_0, v1 && m2_1);
            }
        }
        p13 = c13; p23 = c23; p33 = o33; pdt = odt; pe12 = o12; pe23 = o23;
    };

    // prologue: inputs kA-1, kA, kA+1; old kA-1, kA
    if (tid == 0) {
        issue_inputs(kA - 1);
        issue_inputs(kA);
        issue_old(kA - 1);
        issue_inputs(kA + 1);
        issue_old(kA);
    }
    // warp 0 alone waits on the mbarriers; the block barrier after its wait passes the landed
    // copies on to the other warps
    const bool waiter = warp == 0;
    if (waiter) {
        wait_in(kA - 1);
        wait_in(kA);
        wait_old(kA - 1);
    }
    __syncthreads();
    if (kA >= 1) {
        stage1(kA - 1, false);
        p33 = o33; pdt = odt; pe12 = o12; pe23 = o23;
    }
    for (int K = kA; K < kB; ++K) {
        if (waiter) {
            wait_in(K + 1);
            wait_old(K);
        }
        __syncthreads();  // every thread is done with the slots of plane K-1; inputs K+1 and old K have landed
        if (tid == 0 && ok) {
            issue_inputs(K + 2);
            issue_old(K + 1);
        }
        stage1(K, true);
        __syncthreads();
        velocity(K);
    }
    // drain the copies still in flight (planes kB+1 inputs, kB old) before the block exits;
    // after a time-out some may still be landing (the host treats the flag as fatal)
    if (waiter) {
        wait_in(kB + 1);
        wait_old(kB);
        if (!ok && err) atomicExch(err, 1);
    }
}

}  // namespace sph
