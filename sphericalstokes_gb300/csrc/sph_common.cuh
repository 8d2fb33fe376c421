// Shared definitions of the libsphstokes CUDA kernels (sm_103a).
//
// Device layout: every field of a grid with n1 x n2 x n3 cells lives in the
// same padded box of (n1+1) x (n2+1) x (n3+1) entries, x1 fastest, row pitch
// px = round_up(n1+1, 32) elements so every row starts on a 128-byte (FP32) /
// 256-byte (FP64) boundary.  Entry (i,j,k) (0-based) of every field is at
// i + px*(j + py*k), py = n2+1, whatever the field's own extent; entries
// outside a field's extent are padding and stay zero.  One index therefore
// addresses the cell, its faces and its edges in all arrays, and stencil
// offsets are the same constants (1, px, px*py) for every field.
//
// Staggering (0-based, cell centres at integer coordinates):
//   P, τ11, τ22, τ33, η, ρ ...   cell (i, j, k)            extent n1   x n2   x n3
//   V1 (VR)                       (i-1/2, j, k)             extent n1+1 x n2   x n3
//   V2 (Vθ)                       (i, j-1/2, k)             extent n1   x n2+1 x n3
//   V3 (Vφ)                       (i, j, k-1/2)             extent n1   x n2   x n3+1
//   τ12 (τ_Rθ)                    (i+1/2, j+1/2, k+1)       extent n1-1 x n2-1 x n3-2
//   τ13 (τ_Rφ)                    (i+1/2, j+1, k+1/2)       extent n1-1 x n2-2 x n3-1
//   τ23 (τ_θφ)                    (i+1, j+1/2, k+1/2)       extent n1-2 x n2-1 x n3-1
// which is the reference's array (ix,iy,iz) -> (ix-1,iy-1,iz-1)
// (SphericalStokes_diapir.jl:381-399).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sph {

enum Geom { SPH = 0, CYL = 1, CART = 2 };

struct Dims {
    int n1, n2, n3;     // cells
    int px, py, pz;     // box: px (pitched n1+1), n2+1, n3+1
    int sy, sz;         // strides of x2 and x3
    long long vol;      // px*py*pz
};

// metric tables (per precision) — functions of x1 or x2 only
template <typename T>
struct Geo {
    const T* invRc;    // 1/x1 at cell centres             [n1]
    const T* invRh;    // 1/x1 at half points i+1/2        [n1-1]
    const T* invSinC;  // 1/sin(x2) at cell centres        [n2]
    const T* invSinH;  // 1/sin(x2) at half points j+1/2   [n2-1]
    const T* cotC;     // cot(x2) at cell centres          [n2]
    const T* cotH;     // cot(x2) at half points           [n2-1]
    const T* x1c;      // coordinates of the cell centres  [n1], [n2], [n3]
    const T* x2c;
    const T* x3c;
};

// all fields and scalars one PT kernel may touch
template <typename T>
struct KP {
    Dims d;
    Geo<T> geo;
    T *P, *V1, *V2, *V3;
    T *t11, *t22, *t33, *t12, *t13, *t23;
    T *eta, *eta_ini, *etaSM, *DT_R, *tII, *rho, *eta_pl, *eta_out;
    const uint8_t* phase;
    T *rP, *rV1, *rV2, *rV3;           // right-hand sides of the correction problem / residual outputs
    T *sDD, *s12, *s13, *s23;          // strain-rate scratch (0.5 sum D_ii^2, engineering shear at edges)
    T d1, d2, d3;                      // inverse spacings
    T kbc, gsc, vpdt2;                 // KBDT = kbc*ηSM, GSDT = gsc*ηSM, vpdt^2
    T g;
    T tau_C, n_exp, relax, edot_bg;
    T sig2, sig3;                      // prescribed total normal stress on x2 / x3 faces
    int traction;                      // 1: boundary cells on x2/x3 faces take P = τ_nn - σ_bc
    int fs;                            // 1: top cells (i = n1-1) take the free-surface pressure (fs_pressure)
    T fs_kappa;                        // free-surface stabilisation coefficient
    const T* top_load;                 // surface load per top cell (NULL: 0, the homogeneous problem)
    unsigned long long* red;           // reduction slots (max of |x| as ordered bits)
};

// Programmatic dependent launch: wait until the preceding grid of the stream has
// completed and its writes are visible (returns at once for a launch without a
// programmatic dependency), then allow the next grid of the stream to be
// scheduled, so its launch overlaps this grid instead of following it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
    pdl_wait();
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

__host__ __device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// pressure of a boundary cell under the far-field normal-stress BC: the total
// normal stress -P + τ_nn equals the prescribed σ on the x2 faces (j = 0, n2-1)
// and x3 faces (k = 0, n3-1); the average of both conditions on cells of both.
// Returns false (P unchanged) for cells on no such face.
template <typename T>
__device__ __forceinline__ bool traction_pressure(int j, int k, int n2, int n3, T t22, T t33, T sig2, T sig3, T& P) {
    const bool b2 = (j == 0 || j == n2 - 1), b3 = (k == 0 || k == n3 - 1);
    if (!b2 && !b3) return false;
    if (b2 && b3) P = ((t22 - sig2) + (t33 - sig3)) / T(2);
    else P = b2 ? (t22 - sig2) : (t33 - sig3);
    return true;
}

// pressure of a top cell under the free-surface BC: the normal traction balances the surface
// load q and the stabilisation term, -P + τ11 = -(q + κ V_r), V_r at the cell centre = the mean
// of the cell's inner radial face v_in and its ghost v_out
template <typename T>
__device__ __forceinline__ T fs_pressure(T t11, T q, T kappa, T v_in, T v_out) {
    return t11 + q + kappa * (T(0.5) * (v_in + v_out));
}

// Order-preserving bits of |x|: for non-negative doubles the unsigned order of the
// bit patterns is the numeric order, and every NaN is mapped to the canonical
// positive quiet NaN 0x7ff8000000000000, which lies above +inf.  A max taken on
// these bits (shuffles, atomicMax) therefore propagates NaN, as Julia's maximum
// does, instead of dropping it (fmax) or folding it into +inf.
__device__ __forceinline__ unsigned long long ord_bits(double x) {
    x = fabs(x);
    return x != x ? 0x7ff8000000000000ULL : (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

// max with NaN propagation (Julia's `max`)
template <typename T>
__device__ __forceinline__ T jmax(T a, T b) {
    return (a != a || b != b) ? (a + b) : (a > b ? a : b);
}

// metric coefficients of a cell (i, j): divergence and deviatoric normal strain rates
//   div  = d1*Δ1 + a2*Δ2 + a3*Δ3 + c1*avx(V1) + c2*avy(V2)
//   D11  = d1*Δ1 - div/3
//   D22  = a2*Δ2 + e1*avx(V1) - div/3
//   D33  = a3*Δ3 + e1b*avx(V1) + e2*avy(V2) - div/3
// spherical (SphericalStokes_diapir.jl:184-197), cylindrical (CylindricalStokes_diapir.jl:153-156),
// Cartesian (CartesianStokes_diapir.jl:156-158: no metric, no deviatoric projection)
template <typename T>
struct CellMetric {
    T a2, a3, c1, c2, e1, e1b, e2;
};

template <typename T, int G>
__device__ __forceinline__ CellMetric<T> cell_metric(const KP<T>& p, int i, int j) {
    CellMetric<T> m;
    m.a2 = p.d2; m.a3 = p.d3; m.c1 = T(0); m.c2 = T(0); m.e1 = T(0); m.e1b = T(0); m.e2 = T(0);
    if (G == SPH) {
        T iR = p.geo.invRc[i], iS = p.geo.invSinC[j], ct = p.geo.cotC[j];
        m.a2 = p.d2 * iR; m.a3 = p.d3 * iR * iS;
        m.c1 = T(2) * iR; m.c2 = ct * iR; m.e1 = iR; m.e1b = iR; m.e2 = ct * iR;
    } else if (G == CYL) {
        T iR = p.geo.invRc[i];
        m.a2 = p.d2 * iR; m.c1 = iR; m.e1 = iR;
    }
    return m;
}

}  // namespace sph
