// Stencil arithmetic shared by every kernel (simple, fused, residual).
//
// Each function takes the already-loaded neighbour values and the metric
// factors of its point (1D-table values, see *_metric below), so the one-
// thread-per-point kernels (sph_pt.cuh) and the shared-memory fused sweeps
// (sph_fused.cuh) evaluate exactly the same expressions.  The fused sweeps
// load the metric factors once per block (a thread keeps its (x1, x2)
// position for the whole x3 march) instead of once per point.
// Formulas: SphericalStokes_diapir.jl:184-208 (strain rates), :218-238 (stress
// update), :287-307 (momentum); cylindrical CylindricalStokes_diapir.jl:153-166,
// :199-204; Cartesian CartesianStokes_diapir.jl:156-191, :223-235.
#pragma once
#include "sph_common.cuh"

namespace sph {

// division of the stress / pseudo-step updates: IEEE in FP64, the fast
// intrinsic in FP32 (operands are O(1)-scaled viscosities and steps)
__device__ __forceinline__ double pdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float pdiv(float a, float b) { return __fdividef(a, b); }

template <typename T>
struct CellD {
    T div, D11, D22, D33;
};

// metric factors of a cell (i, j) — see CellMetric in sph_common.cuh
template <typename T, int G>
__device__ __forceinline__ CellMetric<T> cell_metric_t(const Geo<T>& geo, T d2, T d3, int i, int j) {
    CellMetric<T> m;
    m.a2 = d2; m.a3 = d3; m.c1 = T(0); m.c2 = T(0); m.e1 = T(0); m.e1b = T(0); m.e2 = T(0);
    if (G == SPH) {
        const T iR = geo.invRc[i], iS = geo.invSinC[j], ct = geo.cotC[j];
        m.a2 = d2 * iR; m.a3 = d3 * iR * iS; m.c1 = T(2) * iR; m.c2 = ct * iR; m.e1 = iR; m.e1b = iR; m.e2 = ct * iR;
    } else if (G == CYL) {
        const T iR = geo.invRc[i];
        m.a2 = d2 * iR; m.c1 = iR; m.e1 = iR;
    }
    return m;
}

// divergence and normal strain rates of a cell from its six face velocities
// (deviatoric for spherical / cylindrical, plain for Cartesian)
template <typename T, int G>
__device__ __forceinline__ CellD<T> cell_strain_m(const CellMetric<T>& m, T d1, T v1m, T v1p, T v2m, T v2p, T v3m, T v3p) {
    const T h = T(0.5);
    const T d1v = v1p - v1m, d2v = v2p - v2m, d3v = v3p - v3m;
    const T avx = (v1m + v1p) * h, avy = (v2m + v2p) * h;
    CellD<T> r;
    r.div = d1 * d1v + m.a2 * d2v + m.a3 * d3v + m.c1 * avx + m.c2 * avy;
    if (G != CART) {
        const T t3 = r.div * T(1.0 / 3.0);
        r.D11 = d1 * d1v - t3;
        r.D22 = m.a2 * d2v + m.e1 * avx - t3;
        r.D33 = m.a3 * d3v + m.e1b * avx + m.e2 * avy - t3;
    } else {
        r.D11 = d1 * d1v; r.D22 = m.a2 * d2v; r.D33 = m.a3 * d3v;
    }
    return r;
}
template <typename T, int G>
__device__ __forceinline__ CellD<T> cell_strain(const Geo<T>& geo, T d1, T d2, T d3, int i, int j, T v1m, T v1p, T v2m, T v2p,
                                                T v3m, T v3p) {
    return cell_strain_m<T, G>(cell_metric_t<T, G>(geo, d2, d3, i, j), d1, v1m, v1p, v2m, v2p, v3m, v3p);
}

// metric factors of the three edge stencils at index (i, j)
template <typename T>
struct EdgeMetric {
    T iRh;    // 1/x1 at i+1/2                          (τ12, τ13)
    T iSc1;   // 1/sin(x2) at cell j+1                   (τ13)
    T iRc1;   // 1/x1 at cell i+1                        (τ23)
    T iSh;    // 1/sin(x2) at j+1/2                      (τ23)
    T ctH;    // cot(x2) at j+1/2                        (τ23)
};
template <typename T, int G>
__device__ __forceinline__ EdgeMetric<T> edge_metric(const Geo<T>& geo, int i, int j, int n1, int n2) {
    EdgeMetric<T> e;
    e.iRh = e.iSc1 = e.iRc1 = e.iSh = e.ctH = T(1);
    if (G != CART) {
        e.iRh = geo.invRh[clampi(i, 0, n1 - 2)];
        e.iRc1 = geo.invRc[clampi(i + 1, 0, n1 - 1)];
    }
    if (G == SPH) {
        e.iSc1 = geo.invSinC[clampi(j + 1, 0, n2 - 1)];
        e.iSh = geo.invSinH[clampi(j, 0, n2 - 2)];
        e.ctH = geo.cotH[clampi(j, 0, n2 - 2)];
    }
    return e;
}

// engineering shear strain rate at the τ12 edge (i+1/2, j+1/2, k+1):
// v2a,v2b = V2(i|i+1, j+1, k+1); v1a,v1b = V1(i+1, j|j+1, k+1)
template <typename T, int G>
__device__ __forceinline__ T edge12_m(const EdgeMetric<T>& e, T d1, T d2, T v2a, T v2b, T v1a, T v1b) {
    if (G != CART) {
        const T iR = e.iRh;
        return (v2b - v2a) * d1 + iR * (v1b - v1a) * d2 - (v2a + v2b) * T(0.5) * iR;
    }
    return (v1b - v1a) * d2 + (v2b - v2a) * d1;
}
// τ13 edge (i+1/2, j+1, k+1/2): v3a,v3b = V3(i|i+1, j+1, k+1); v1a,v1b = V1(i+1, j+1, k|k+1)
template <typename T, int G>
__device__ __forceinline__ T edge13_m(const EdgeMetric<T>& e, T d1, T d3, T v3a, T v3b, T v1a, T v1b) {
    if (G == SPH) {
        const T iR = e.iRh;
        return (v3b - v3a) * d1 + iR * e.iSc1 * (v1b - v1a) * d3 - (v3a + v3b) * T(0.5) * iR;
    }
    return (v3b - v3a) * d1 + (v1b - v1a) * d3;
}
// τ23 edge (i+1, j+1/2, k+1/2): v3a,v3b = V3(i+1, j|j+1, k+1); v2a,v2b = V2(i+1, j+1, k|k+1)
template <typename T, int G>
__device__ __forceinline__ T edge23_m(const EdgeMetric<T>& e, T d2, T d3, T v3a, T v3b, T v2a, T v2b) {
    if (G == SPH) {
        const T iR = e.iRc1;
        return iR * (v3b - v3a) * d2 + iR * e.iSh * (v2b - v2a) * d3 - (v3a + v3b) * T(0.5) * iR * e.ctH;
    }
    if (G == CYL) return e.iRc1 * (v3b - v3a) * d2 + (v2b - v2a) * d3;
    return (v3b - v3a) * d2 + (v2b - v2a) * d3;
}
template <typename T, int G>
__device__ __forceinline__ T edge12(const Geo<T>& geo, T d1, T d2, int i, T v2a, T v2b, T v1a, T v1b) {
    EdgeMetric<T> e;
    e.iRh = G != CART ? geo.invRh[i] : T(1);
    return edge12_m<T, G>(e, d1, d2, v2a, v2b, v1a, v1b);
}
template <typename T, int G>
__device__ __forceinline__ T edge13(const Geo<T>& geo, T d1, T d3, int i, int j, T v3a, T v3b, T v1a, T v1b) {
    EdgeMetric<T> e;
    if (G == SPH) { e.iRh = geo.invRh[i]; e.iSc1 = geo.invSinC[j + 1]; }
    return edge13_m<T, G>(e, d1, d3, v3a, v3b, v1a, v1b);
}
template <typename T, int G>
__device__ __forceinline__ T edge23(const Geo<T>& geo, T d2, T d3, int i, int j, T v3a, T v3b, T v2a, T v2b) {
    EdgeMetric<T> e;
    if (G != CART) e.iRc1 = geo.invRc[i + 1];
    if (G == SPH) { e.iSh = geo.invSinH[j]; e.ctH = geo.cotH[j]; }
    return edge23_m<T, G>(e, d2, d3, v3a, v3b, v2a, v2b);
}

// stress update of an edge from the 4 surrounding cells (ηSM sum s4, η sum e4)
template <typename T>
__device__ __forceinline__ T edge_update(T told, T gsc, T s4, T e4, T D) {
    const T aG = gsc * (s4 * T(0.25));
    const T aE = e4 * T(0.25);
    return (told + aG * D) * pdiv(aE, aE + aG);
}

// metric factors of the three momentum stencils at velocity nodes (I, J)
template <typename T>
struct MomMetric {
    T iR1, iS1, ct1;  // V1: 1/x1 at I-1/2, 1/sin, cot at J
    T iR2, iS2, ct2;  // V2: 1/x1 at I, 1/sin, cot at J-1/2
    T iS3, ct3;       // V3: 1/x1 at I (= iR2), 1/sin, cot at J
};
template <typename T, int G>
__device__ __forceinline__ MomMetric<T> mom_metric(const Geo<T>& geo, int I, int J, int n1, int n2) {
    MomMetric<T> m;
    m.iR1 = m.iS1 = m.ct1 = m.iR2 = m.iS2 = m.ct2 = m.iS3 = m.ct3 = T(1);
    if (G != CART) {
        m.iR1 = geo.invRh[clampi(I - 1, 0, n1 - 2)];
        m.iR2 = geo.invRc[clampi(I, 0, n1 - 1)];
    }
    if (G == SPH) {
        const int Jc = clampi(J, 0, n2 - 1), Jh = clampi(J - 1, 0, n2 - 2);
        m.iS1 = geo.invSinC[Jc]; m.ct1 = geo.cotC[Jc];
        m.iS2 = geo.invSinH[Jh]; m.ct2 = geo.cotH[Jh];
        m.iS3 = m.iS1; m.ct3 = m.ct1;
    }
    return m;
}

// momentum residual at V1 (I-1/2, J, K): cells I-1 (m) and I; τ12 (I-1, J|J-1, K-1) = ta, tb;
// τ13 (I-1, J-1, K|K-1) = ua, ub
template <typename T, int G>
__device__ __forceinline__ T mom1_m(const MomMetric<T>& mm, T d1, T d2, T d3, T s11m, T s11, T s22m, T s22, T s33m, T s33, T ta, T tb,
                                    T ua, T ub) {
    const T h = T(0.5);
    if (G == SPH) {
        const T iR = mm.iR1, iS = mm.iS1, ct = mm.ct1;
        return (s11 - s11m) * d1 + iR * (ta - tb) * d2 + iR * iS * (ua - ub) * d3 +
               (T(2) * ((s11m + s11) * h) - (((s22m + s22) * h) + ((s33m + s33) * h))) * iR + ((tb + ta) * h) * iR * ct;
    } else if (G == CYL) {
        const T iR = mm.iR1;
        return (s11 - s11m) * d1 + iR * (ta - tb) * d2 + (ua - ub) * d3 + (((s11m + s11) * h) - ((s22m + s22) * h)) * iR;
    }
    return (s11 - s11m) * d1 + (ta - tb) * d2 + (ua - ub) * d3;
}
// V2 (I, J-1/2, K): cells J-1 (m) and J; τ12 (I|I-1, J-1, K-1) = ta, tb; τ23 (I-1, J-1, K|K-1) = ua, ub
template <typename T, int G>
__device__ __forceinline__ T mom2_m(const MomMetric<T>& mm, T d1, T d2, T d3, T s22m, T s22, T s33m, T s33, T ta, T tb, T ua, T ub) {
    const T h = T(0.5);
    if (G == SPH) {
        const T iR = mm.iR2, iS = mm.iS2, ct = mm.ct2;
        return (ta - tb) * d1 + iR * (s22 - s22m) * d2 + iR * iS * (ua - ub) * d3 + T(3) * ((tb + ta) * h) * iR +
               (((s22m + s22) * h) - ((s33m + s33) * h)) * iR * ct;
    } else if (G == CYL) {
        const T iR = mm.iR2;
        return (ta - tb) * d1 + iR * (s22 - s22m) * d2 + (ua - ub) * d3 + T(2) * ((tb + ta) * h) * iR;
    }
    return (ta - tb) * d1 + (s22 - s22m) * d2 + (ua - ub) * d3;
}
// V3 (I, J, K-1/2): cells K-1 (m) and K; τ13 (I|I-1, J-1, K-1) = ta, tb; τ23 (I-1, J|J-1, K-1) = ua, ub
template <typename T, int G>
__device__ __forceinline__ T mom3_m(const MomMetric<T>& mm, T d1, T d2, T d3, T s33m, T s33, T ta, T tb, T ua, T ub) {
    const T h = T(0.5);
    if (G == SPH) {
        const T iR = mm.iR2, iS = mm.iS3, ct = mm.ct3;
        return (ta - tb) * d1 + iR * (ua - ub) * d2 + iR * iS * (s33 - s33m) * d3 + T(3) * ((tb + ta) * h) * iR +
               T(2) * ((ub + ua) * h) * iR * ct;
    } else if (G == CYL) {
        const T iR = mm.iR2;
        return (ta - tb) * d1 + iR * (ua - ub) * d2 + (s33 - s33m) * d3 + ((tb + ta) * h) * iR;
    }
    return (ta - tb) * d1 + (ua - ub) * d2 + (s33 - s33m) * d3;
}
template <typename T, int G>
__device__ __forceinline__ T mom1(const Geo<T>& geo, T d1, T d2, T d3, int I, int J, T s11m, T s11, T s22m, T s22, T s33m, T s33,
                                  T ta, T tb, T ua, T ub) {
    MomMetric<T> mm;
    mm.iR1 = G != CART ? geo.invRh[I - 1] : T(1);
    mm.iS1 = G == SPH ? geo.invSinC[J] : T(1);
    mm.ct1 = G == SPH ? geo.cotC[J] : T(1);
    return mom1_m<T, G>(mm, d1, d2, d3, s11m, s11, s22m, s22, s33m, s33, ta, tb, ua, ub);
}
template <typename T, int G>
__device__ __forceinline__ T mom2(const Geo<T>& geo, T d1, T d2, T d3, int I, int J, T s22m, T s22, T s33m, T s33, T ta, T tb, T ua,
                                  T ub) {
    MomMetric<T> mm;
    mm.iR2 = G != CART ? geo.invRc[I] : T(1);
    mm.iS2 = G == SPH ? geo.invSinH[J - 1] : T(1);
    mm.ct2 = G == SPH ? geo.cotH[J - 1] : T(1);
    return mom2_m<T, G>(mm, d1, d2, d3, s22m, s22, s33m, s33, ta, tb, ua, ub);
}
template <typename T, int G>
__device__ __forceinline__ T mom3(const Geo<T>& geo, T d1, T d2, T d3, int I, int J, T s33m, T s33, T ta, T tb, T ua, T ub) {
    MomMetric<T> mm;
    mm.iR2 = G != CART ? geo.invRc[I] : T(1);
    mm.iS3 = G == SPH ? geo.invSinC[J] : T(1);
    mm.ct3 = G == SPH ? geo.cotC[J] : T(1);
    return mom3_m<T, G>(mm, d1, d2, d3, s33m, s33, ta, tb, ua, ub);
}

}  // namespace sph
