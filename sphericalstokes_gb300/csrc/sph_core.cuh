// Stencil arithmetic shared by every kernel (simple, fused, residual).
//
// Each function takes the already-loaded neighbour values, so the one-thread-
// per-point kernels (sph_pt.cuh) and the shared-memory fused sweep
// (sph_fused.cuh) evaluate exactly the same expressions and agree bitwise.
// Formulas: SphericalStokes_diapir.jl:184-208 (strain rates), :218-238 (stress
// update), :287-307 (momentum); cylindrical CylindricalStokes_diapir.jl:153-166,
// :199-204; Cartesian CartesianStokes_diapir.jl:156-191, :223-235.
#pragma once
#include "sph_common.cuh"

namespace sph {

template <typename T>
struct CellD {
    T div, D11, D22, D33;
};

// divergence and normal strain rates of a cell from its six face velocities
// (deviatoric for spherical / cylindrical, plain for Cartesian)
template <typename T, int G>
__device__ __forceinline__ CellD<T> cell_strain(const Geo<T>& geo, T d1, T d2, T d3, int i, int j, T v1m, T v1p, T v2m, T v2p,
                                                T v3m, T v3p) {
    T a2 = d2, a3 = d3, c1 = T(0), c2 = T(0), e1 = T(0), e1b = T(0), e2 = T(0);
    if (G == SPH) {
        const T iR = geo.invRc[i], iS = geo.invSinC[j], ct = geo.cotC[j];
        a2 = d2 * iR; a3 = d3 * iR * iS; c1 = T(2) * iR; c2 = ct * iR; e1 = iR; e1b = iR; e2 = ct * iR;
    } else if (G == CYL) {
        const T iR = geo.invRc[i];
        a2 = d2 * iR; c1 = iR; e1 = iR;
    }
    const T h = T(0.5);
    const T d1v = v1p - v1m, d2v = v2p - v2m, d3v = v3p - v3m;
    const T avx = (v1m + v1p) * h, avy = (v2m + v2p) * h;
    CellD<T> r;
    r.div = d1 * d1v + a2 * d2v + a3 * d3v + c1 * avx + c2 * avy;
    if (G != CART) {
        const T t3 = r.div * T(1.0 / 3.0);
        r.D11 = d1 * d1v - t3;
        r.D22 = a2 * d2v + e1 * avx - t3;
        r.D33 = a3 * d3v + e1b * avx + e2 * avy - t3;
    } else {
        r.D11 = d1 * d1v; r.D22 = a2 * d2v; r.D33 = a3 * d3v;
    }
    return r;
}

// engineering shear strain rate at the τ12 edge (i+1/2, j+1/2, k+1):
// v2a,v2b = V2(i|i+1, j+1, k+1); v1a,v1b = V1(i+1, j|j+1, k+1)
template <typename T, int G>
__device__ __forceinline__ T edge12(const Geo<T>& geo, T d1, T d2, int i, T v2a, T v2b, T v1a, T v1b) {
    if (G != CART) {
        const T iR = geo.invRh[i];
        return (v2b - v2a) * d1 + iR * (v1b - v1a) * d2 - (v2a + v2b) * T(0.5) * iR;
    }
    return (v1b - v1a) * d2 + (v2b - v2a) * d1;
}
// τ13 edge (i+1/2, j+1, k+1/2): v3a,v3b = V3(i|i+1, j+1, k+1); v1a,v1b = V1(i+1, j+1, k|k+1)
template <typename T, int G>
__device__ __forceinline__ T edge13(const Geo<T>& geo, T d1, T d3, int i, int j, T v3a, T v3b, T v1a, T v1b) {
    if (G == SPH) {
        const T iR = geo.invRh[i];
        return (v3b - v3a) * d1 + iR * geo.invSinC[j + 1] * (v1b - v1a) * d3 - (v3a + v3b) * T(0.5) * iR;
    }
    return (v3b - v3a) * d1 + (v1b - v1a) * d3;
}
// τ23 edge (i+1, j+1/2, k+1/2): v3a,v3b = V3(i+1, j|j+1, k+1); v2a,v2b = V2(i+1, j+1, k|k+1)
template <typename T, int G>
__device__ __forceinline__ T edge23(const Geo<T>& geo, T d2, T d3, int i, int j, T v3a, T v3b, T v2a, T v2b) {
    if (G == SPH) {
        const T iR = geo.invRc[i + 1];
        return iR * (v3b - v3a) * d2 + iR * geo.invSinH[j] * (v2b - v2a) * d3 - (v3a + v3b) * T(0.5) * iR * geo.cotH[j];
    }
    if (G == CYL) return geo.invRc[i + 1] * (v3b - v3a) * d2 + (v2b - v2a) * d3;
    return (v3b - v3a) * d2 + (v2b - v2a) * d3;
}

// stress update of an edge from the 4 surrounding cells (ηSM sum s4, η sum e4)
template <typename T>
__device__ __forceinline__ T edge_update(T told, T gsc, T s4, T e4, T D) {
    const T aG = gsc * (s4 * T(0.25));
    const T aE = e4 * T(0.25);
    return (told + aG * D) * (aE / (aE + aG));
}

// momentum residual at V1 (I-1/2, J, K): cells I-1 (m) and I; τ12 (I-1, J|J-1, K-1) = ta, tb;
// τ13 (I-1, J-1, K|K-1) = ua, ub
template <typename T, int G>
__device__ __forceinline__ T mom1(const Geo<T>& geo, T d1, T d2, T d3, int I, int J, T s11m, T s11, T s22m, T s22, T s33m,
                                  T s33, T ta, T tb, T ua, T ub) {
    const T h = T(0.5);
    if (G == SPH) {
        const T iR = geo.invRh[I - 1], iS = geo.invSinC[J], ct = geo.cotC[J];
        return (s11 - s11m) * d1 + iR * (ta - tb) * d2 + iR * iS * (ua - ub) * d3 +
               (T(2) * ((s11m + s11) * h) - (((s22m + s22) * h) + ((s33m + s33) * h))) * iR + ((tb + ta) * h) * iR * ct;
    } else if (G == CYL) {
        const T iR = geo.invRh[I - 1];
        return (s11 - s11m) * d1 + iR * (ta - tb) * d2 + (ua - ub) * d3 + (((s11m + s11) * h) - ((s22m + s22) * h)) * iR;
    }
    return (s11 - s11m) * d1 + (ta - tb) * d2 + (ua - ub) * d3;
}
// V2 (I, J-1/2, K): cells J-1 (m) and J; τ12 (I|I-1, J-1, K-1) = ta, tb; τ23 (I-1, J-1, K|K-1) = ua, ub
template <typename T, int G>
__device__ __forceinline__ T mom2(const Geo<T>& geo, T d1, T d2, T d3, int I, int J, T s22m, T s22, T s33m, T s33, T ta, T tb,
                                  T ua, T ub) {
    const T h = T(0.5);
    if (G == SPH) {
        const T iR = geo.invRc[I], iS = geo.invSinH[J - 1], ct = geo.cotH[J - 1];
        return (ta - tb) * d1 + iR * (s22 - s22m) * d2 + iR * iS * (ua - ub) * d3 + T(3) * ((tb + ta) * h) * iR +
               (((s22m + s22) * h) - ((s33m + s33) * h)) * iR * ct;
    } else if (G == CYL) {
        const T iR = geo.invRc[I];
        return (ta - tb) * d1 + iR * (s22 - s22m) * d2 + (ua - ub) * d3 + T(2) * ((tb + ta) * h) * iR;
    }
    return (ta - tb) * d1 + (s22 - s22m) * d2 + (ua - ub) * d3;
}
// V3 (I, J, K-1/2): cells K-1 (m) and K; τ13 (I|I-1, J-1, K-1) = ta, tb; τ23 (I-1, J|J-1, K-1) = ua, ub
template <typename T, int G>
__device__ __forceinline__ T mom3(const Geo<T>& geo, T d1, T d2, T d3, int I, int J, T s33m, T s33, T ta, T tb, T ua, T ub) {
    const T h = T(0.5);
    if (G == SPH) {
        const T iR = geo.invRc[I], iS = geo.invSinC[J], ct = geo.cotC[J];
        return (ta - tb) * d1 + iR * (ua - ub) * d2 + iR * iS * (s33 - s33m) * d3 + T(3) * ((tb + ta) * h) * iR +
               T(2) * ((ub + ua) * h) * iR * ct;
    } else if (G == CYL) {
        const T iR = geo.invRc[I];
        return (ta - tb) * d1 + iR * (ua - ub) * d2 + (s33 - s33m) * d3 + ((tb + ta) * h) * iR;
    }
    return (ta - tb) * d1 + (ua - ub) * d2 + (s33 - s33m) * d3;
}

}  // namespace sph
