// Pseudo-transient kernels (one thread per grid point, direct global access).
//
// These are the building blocks of one PT iteration in the reference's order
// (SphericalStokes_diapir.jl:413-425):
//   k_maxloc   maxloc! + copy_BC!(ηSM)          :149-152, :102-124
//   k_stress   compute_P!                        :155-241
//   k_rheo_tau compute_TII! + copy_BC!(τII) + power_law!   :243-265
//   k_strain / k_edot_law   strain-rate power law (not in the reference)
//   k_velocity compute_V!                        :267-329
//   k_bc       BC_R! / BC_θ! / BC_φ! and the cyl/cart BC kernels
// All three coordinate systems share the kernels; the metric terms come from
// the template parameter G and the 1D tables in Geo.  The FP32 fused sweep in
// sph_fused.cuh implements the same arithmetic with shared-memory tiling.
#pragma once
#include "sph_core.cuh"

namespace sph {

// ---------------------------------------------------------------------------
// ηSM = 7-point maximum of η on interior cells; boundary cells take the value
// of the clamped interior cell (copy_bc_r!, copy_bc_θ!, copy_bc_φ! in that
// order leave exactly that).  faces_only: CartesianStokes_diapir.jl:97-105
// copies only face interiors and edges/corners keep η (ηSM .= η before maxloc!).
template <typename T>
__global__ void k_maxloc(KP<T> p, int faces_only) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int c = i + d.sy * j + d.sz * k;
    int nb = (i == 0 || i == d.n1 - 1) + (j == 0 || j == d.n2 - 1) + (k == 0 || k == d.n3 - 1);
    if (faces_only && nb >= 2) { p.etaSM[c] = p.eta[c]; return; }
    const int a = clampi(i, 1, d.n1 - 2), b = clampi(j, 1, d.n2 - 2), e = clampi(k, 1, d.n3 - 2);
    const int s = a + d.sy * b + d.sz * e;
    const T* E = p.eta;
    p.etaSM[c] = jmax(jmax(jmax(jmax(E[s - 1], E[s + 1]), E[s]), jmax(E[s - d.sy], E[s + d.sy])), jmax(E[s - d.sz], E[s + d.sz]));
}

// ---------------------------------------------------------------------------
// compute_P!: pressure, normal deviatoric stresses and DT_R at cells, shear
// stresses at edges.  RHS: continuity right-hand side rP (correction problem:
// P -= KBDT*(div δV + div V_fp64)).
template <typename T, int G, bool RHS>
__global__ void __launch_bounds__(256) k_stress(KP<T> p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    {
        const CellD<T> D = cell_strain<T, G>(p.geo, p.d1, p.d2, p.d3, i, j, p.V1[c], p.V1[c + 1], p.V2[c], p.V2[c + sy], p.V3[c], p.V3[c + sz]);
        const T sm = p.etaSM[c], e = p.eta[c];
        const T gs = p.gsc * sm, kb = p.kbc * sm;
        const T f = pdiv(e, e + gs);  // 1/(1 + GSDT/η)
        T dv = D.div;
        if (RHS) dv += p.rP[c];
        T Pn = p.P[c] - kb * dv;
        const T n11 = (p.t11[c] + T(2) * gs * D.D11) * f;
        const T n22 = (p.t22[c] + T(2) * gs * D.D22) * f, n33 = (p.t33[c] + T(2) * gs * D.D33) * f;
        if (p.traction) traction_pressure(j, k, d.n2, d.n3, n22, n33, p.sig2, p.sig3, Pn);
        if (p.fs && i == d.n1 - 1) Pn = fs_pressure(n11, p.top_load ? p.top_load[c] : T(0), p.fs_kappa, p.V1[c], p.V1[c + 1]);
        p.P[c] = Pn;
        p.t11[c] = n11;
        p.t22[c] = n22;
        p.t33[c] = n33;
        p.DT_R[c] = pdiv(p.vpdt2, kb + gs * f);
    }
    // τ12 at (i+1/2, j+1/2, k+1): cells (i|i+1, j|j+1, k+1)
    if (i < d.n1 - 1 && j < d.n2 - 1 && k < d.n3 - 2) {
        const int q = c + sz;
        const T D = edge12<T, G>(p.geo, p.d1, p.d2, i, p.V2[q + sy], p.V2[q + sy + 1], p.V1[q + 1], p.V1[q + 1 + sy]);
        p.t12[c] = edge_update(p.t12[c], p.gsc, p.etaSM[q] + p.etaSM[q + sy] + p.etaSM[q + 1] + p.etaSM[q + 1 + sy],
                               p.eta[q] + p.eta[q + sy] + p.eta[q + 1] + p.eta[q + 1 + sy], D);
    }
    // τ13 at (i+1/2, j+1, k+1/2): cells (i|i+1, j+1, k|k+1)
    if (i < d.n1 - 1 && j < d.n2 - 2 && k < d.n3 - 1) {
        const int q = c + sy;
        const T D = edge13<T, G>(p.geo, p.d1, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + 1], p.V1[q + 1], p.V1[q + 1 + sz]);
        p.t13[c] = edge_update(p.t13[c], p.gsc, p.etaSM[q] + p.etaSM[q + sz] + p.etaSM[q + 1] + p.etaSM[q + 1 + sz],
                               p.eta[q] + p.eta[q + sz] + p.eta[q + 1] + p.eta[q + 1 + sz], D);
    }
    // τ23 at (i+1, j+1/2, k+1/2): cells (i+1, j|j+1, k|k+1)
    if (i < d.n1 - 2 && j < d.n2 - 1 && k < d.n3 - 1) {
        const int q = c + 1;
        const T D = edge23<T, G>(p.geo, p.d2, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + sy], p.V2[q + sy], p.V2[q + sy + sz]);
        p.t23[c] = edge_update(p.t23[c], p.gsc, p.etaSM[q] + p.etaSM[q + sz] + p.etaSM[q + sy] + p.etaSM[q + sy + sz],
                               p.eta[q] + p.eta[q + sz] + p.eta[q + sy] + p.eta[q + sy + sz], D);
    }
}

// ---------------------------------------------------------------------------
// strain rates of the current velocities as separate fields (the DIVV and D_*
// arrays compute_P! fills in CylindricalStokes_diapir.jl:153-159): divergence
// and normal rates at cells, engineering shear rates at the three edge sets,
// in the layout of P and τ12, τ13, τ23.
template <typename T, int G>
__global__ void __launch_bounds__(256) k_strain_out(KP<T> p, T* __restrict__ dv, T* __restrict__ d11, T* __restrict__ d22,
                                                    T* __restrict__ d33, T* __restrict__ d12, T* __restrict__ d13, T* __restrict__ d23) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const CellD<T> D = cell_strain<T, G>(p.geo, p.d1, p.d2, p.d3, i, j, p.V1[c], p.V1[c + 1], p.V2[c], p.V2[c + sy], p.V3[c], p.V3[c + sz]);
    dv[c] = D.div; d11[c] = D.D11; d22[c] = D.D22; d33[c] = D.D33;
    if (i < d.n1 - 1 && j < d.n2 - 1 && k < d.n3 - 2) {
        const int q = c + sz;
        d12[c] = edge12<T, G>(p.geo, p.d1, p.d2, i, p.V2[q + sy], p.V2[q + sy + 1], p.V1[q + 1], p.V1[q + 1 + sy]);
    }
    if (i < d.n1 - 1 && j < d.n2 - 2 && k < d.n3 - 1) {
        const int q = c + sy;
        d13[c] = edge13<T, G>(p.geo, p.d1, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + 1], p.V1[q + 1], p.V1[q + 1 + sz]);
    }
    if (i < d.n1 - 2 && j < d.n2 - 1 && k < d.n3 - 1) {
        const int q = c + 1;
        d23[c] = edge23<T, G>(p.geo, p.d2, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + sy], p.V2[q + sy], p.V2[q + sy + sz]);
    }
}

// ---------------------------------------------------------------------------
// second invariant of τ at an interior cell s (compute_TII!, :246-255)
template <typename T>
__device__ __forceinline__ T tau_II(const KP<T>& p, int s) {
    const int sy = p.d.sy, sz = p.d.sz;
    const T q4 = T(0.25);
    const int e = s - 1 - sy - sz;  // edge (I-1, J-1, K-1)
    const T a = (p.t12[e] + p.t12[e + sy] + p.t12[e + 1] + p.t12[e + 1 + sy]) * q4;
    const T b = (p.t13[e] + p.t13[e + sz] + p.t13[e + 1] + p.t13[e + 1 + sz]) * q4;
    const T c = (p.t23[e] + p.t23[e + sz] + p.t23[e + sy] + p.t23[e + sy + sz]) * q4;
    const T x = p.t11[s], y = p.t22[s], z = p.t33[s];
    return sqrt(T(0.5) * (x * x + y * y + z * z) + a * a + b * b + c * c);
}

// compute_TII! + copy_BC!(τII) + power_law! (RELAX: log-space relaxation of
// η_PL, CylindricalStokes_diapir.jl:185-192).  phase==1 cells are linear.
template <typename T, bool RELAX>
__global__ void k_rheo_tau(KP<T> p, int faces_only, T n_exp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int c = i + d.sy * j + d.sz * k;
    const int nb = (i == 0 || i == d.n1 - 1) + (j == 0 || j == d.n2 - 1) + (k == 0 || k == d.n3 - 1);
    T tii;
    if (faces_only && nb >= 2) {
        tii = p.tII[c];  // CartesianStokes_diapir.jl:97-105 never writes edges/corners of τII
    } else {
        const int s = clampi(i, 1, d.n1 - 2) + d.sy * clampi(j, 1, d.n2 - 2) + d.sz * clampi(k, 1, d.n3 - 2);
        tii = tau_II(p, s);
        p.tII[c] = tii;
    }
    const T ne = (p.phase && p.phase[c]) ? T(1) : n_exp;
    const T ei = p.eta_ini[c];
    if (!RELAX) {
        p.eta[c] = T(2) / (T(1) / ei + T(1) / (ei * pow(tii / p.tau_C, T(1) - ne)));
    } else {
        T pl = ei * pow(tii / p.tau_C, T(1) - ne);
        pl = exp(log(pl) * p.relax + log(p.eta_pl[c]) * (T(1) - p.relax));
        p.eta_pl[c] = pl;
        p.eta[c] = T(2) / (T(1) / ei + T(1) / pl);
    }
}

// ---------------------------------------------------------------------------
// strain rates of the current velocities (as compute_P! forms them):
// sDD = 0.5*(D11^2 + D22^2 + D33^2) at cells, s12/s13/s23 = engineering shear
// strain rates at the edges.
template <typename T, int G>
__global__ void __launch_bounds__(256) k_strain(KP<T> p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    {
        const CellD<T> D = cell_strain<T, G>(p.geo, p.d1, p.d2, p.d3, i, j, p.V1[c], p.V1[c + 1], p.V2[c], p.V2[c + sy], p.V3[c], p.V3[c + sz]);
        p.sDD[c] = T(0.5) * (D.D11 * D.D11 + D.D22 * D.D22 + D.D33 * D.D33);
    }
    if (i < d.n1 - 1 && j < d.n2 - 1 && k < d.n3 - 2) {
        const int q = c + sz;
        p.s12[c] = edge12<T, G>(p.geo, p.d1, p.d2, i, p.V2[q + sy], p.V2[q + sy + 1], p.V1[q + 1], p.V1[q + 1 + sy]);
    }
    if (i < d.n1 - 1 && j < d.n2 - 2 && k < d.n3 - 1) {
        const int q = c + sy;
        p.s13[c] = edge13<T, G>(p.geo, p.d1, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + 1], p.V1[q + 1], p.V1[q + 1 + sz]);
    }
    if (i < d.n1 - 2 && j < d.n2 - 1 && k < d.n3 - 1) {
        const int q = c + 1;
        p.s23[c] = edge23<T, G>(p.geo, p.d2, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + sy], p.V2[q + sy], p.V2[q + sy + sz]);
    }
}

// strain-rate power law (not in the reference): the invariant of the clamped
// interior cell (as copy_BC! does for τII), η_t = 2/(1/η_ini + 1/η_PL),
// η_PL = η_ini (edot_II/edot_bg)^((1-n)/n); RELAXED: η_out = η^(1-relax) η_t^relax.
template <typename T, bool RELAXED>
__global__ void k_edot_law(KP<T> p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const int s = clampi(i, 1, d.n1 - 2) + sy * clampi(j, 1, d.n2 - 2) + sz * clampi(k, 1, d.n3 - 2);
    const T q4 = T(0.25);
    const int e = s - 1 - sy - sz;
    const T a = (p.s12[e] + p.s12[e + sy] + p.s12[e + 1] + p.s12[e + 1 + sy]) * q4;
    const T b = (p.s13[e] + p.s13[e + sz] + p.s13[e + 1] + p.s13[e + 1 + sz]) * q4;
    const T cc = (p.s23[e] + p.s23[e + sz] + p.s23[e + sy] + p.s23[e + sy + sz]) * q4;
    const T ed = sqrt(p.sDD[s] + q4 * (a * a + b * b + cc * cc));
    const T ei = p.eta_ini[c];
    T et;
    if (p.phase && p.phase[c]) {
        et = ei;
    } else {
        const T pl = ei * pow(ed / p.edot_bg, (T(1) - p.n_exp) / p.n_exp);
        et = T(2) / (T(1) / ei + T(1) / pl);
    }
    p.eta_out[c] = RELAXED ? exp((T(1) - p.relax) * log(p.eta[c]) + p.relax * log(et)) : et;
}

// ---------------------------------------------------------------------------
// compute_V!: momentum residuals at interior velocity nodes (:267-307).
// GRAV: include the ρg body force; RHS: add the right-hand side rV instead.
// ok[f] tells whether (I,J,K) is an interior node of velocity component f.
template <typename T, int G, bool GRAV, bool RHS>
__device__ __forceinline__ void momentum(const KP<T>& p, int I, int J, int K, T dv[3], bool ok[3]) {
    const Dims& d = p.d;
    const int sy = d.sy, sz = d.sz;
    const int c = I + sy * J + sz * K;
    const T h = T(0.5);
    const T Pc = p.P[c];
    const T s11 = p.t11[c] - Pc, s22 = p.t22[c] - Pc, s33 = p.t33[c] - Pc;
    ok[0] = (J <= d.n2 - 2 && K <= d.n3 - 2);
    ok[1] = (I <= d.n1 - 2 && K <= d.n3 - 2);
    ok[2] = (I <= d.n1 - 2 && J <= d.n2 - 2);
    if (ok[0]) {  // V1 (I-1/2, J, K)
        const int m = c - 1;
        const T Pm = p.P[m];
        T r = mom1<T, G>(p.geo, p.d1, p.d2, p.d3, I, J, p.t11[m] - Pm, s11, p.t22[m] - Pm, s22, p.t33[m] - Pm, s33,
                         p.t12[m - sz], p.t12[m - sy - sz], p.t13[m - sy], p.t13[m - sy - sz]);
        if (G != CART && GRAV) r -= (p.rho[m] * p.g + p.rho[c] * p.g) * h;
        if (RHS) r += p.rV1[c];
        dv[0] = r;
    }
    if (ok[1]) {  // V2 (I, J-1/2, K)
        const int m = c - sy;
        const T Pm = p.P[m];
        T r = mom2<T, G>(p.geo, p.d1, p.d2, p.d3, I, J, p.t22[m] - Pm, s22, p.t33[m] - Pm, s33,
                         p.t12[c - sy - sz], p.t12[c - 1 - sy - sz], p.t23[c - 1 - sy], p.t23[c - 1 - sy - sz]);
        if (RHS) r += p.rV2[c];
        dv[1] = r;
    }
    if (ok[2]) {  // V3 (I, J, K-1/2)
        const int m = c - sz;
        T r = mom3<T, G>(p.geo, p.d1, p.d2, p.d3, I, J, p.t33[m] - p.P[m], s33, p.t13[c - sy - sz], p.t13[c - 1 - sy - sz],
                         p.t23[c - 1 - sz], p.t23[c - 1 - sy - sz]);
        if (G == CART && GRAV) r -= p.g * (h * (p.rho[m] + p.rho[c]));
        if (RHS) r += p.rV3[c];
        dv[2] = r;
    }
}

// MODE 0: V += dV*avg(DT_R) with the ρg body force (reference compute_V!)
// MODE 1: V += (dV + rV)*avg(DT_R), no gravity (correction problem)
// MODE 2: rV = dV with gravity (residual evaluation, V unchanged)
template <typename T, int G, int MODE>
__global__ void __launch_bounds__(256) k_velocity(KP<T> p) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1, K = blockIdx.z + 1;
    const Dims& d = p.d;
    if (I > d.n1 - 1 || J > d.n2 - 1 || K > d.n3 - 1) return;
    const int sy = d.sy, sz = d.sz;
    const int c = I + sy * J + sz * K;
    T dv[3];
    bool ok[3];
    momentum<T, G, MODE != 1, MODE == 1>(p, I, J, K, dv, ok);
    const T h = T(0.5);
    if (MODE == 2) {
        if (ok[0]) p.rV1[c] = dv[0];
        if (ok[1]) p.rV2[c] = dv[1];
        if (ok[2]) p.rV3[c] = dv[2];
    } else {
        if (ok[0]) p.V1[c] = p.V1[c] + dv[0] * ((p.DT_R[c - 1] + p.DT_R[c]) * h);
        if (ok[1]) p.V2[c] = p.V2[c] + dv[1] * ((p.DT_R[c - sy] + p.DT_R[c]) * h);
        if (ok[2]) p.V3[c] = p.V3[c] + dv[2] * ((p.DT_R[c - sz] + p.DT_R[c]) * h);
    }
}

// max |dV + rV| of the correction problem over the velocity nodes of block (bx, by, bz) into
// *red (inner stopping test); 32 x 8 threads, the body of k_velocity_norm and of its batched
// launch over many grids
template <typename T, int G>
__device__ __forceinline__ void velocity_norm_body(const KP<T>& p, int bx, int by, int bz, unsigned long long* red) {
    const int I = bx * blockDim.x + threadIdx.x + 1, J = by * blockDim.y + threadIdx.y + 1, K = bz + 1;
    const Dims& d = p.d;
    unsigned long long m = 0ULL;  // ordered bits of the running max (NaN propagates)
    if (I <= d.n1 - 1 && J <= d.n2 - 1 && K <= d.n3 - 1) {
        T dv[3];
        bool ok[3];
        momentum<T, G, false, true>(p, I, J, K, dv, ok);
        for (int f = 0; f < 3; ++f)
            if (ok[f]) m = umax64(m, ord_bits((double)dv[f]));
    }
    // block reduction over the 2D block
    for (int o = 16; o > 0; o >>= 1) m = umax64(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ unsigned long long sm[32];
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = t & 31, w = t >> 5, nw = (blockDim.x * blockDim.y) >> 5;
    if (lane == 0) sm[w] = m;
    __syncthreads();
    if (w == 0) {
        m = lane < nw ? sm[lane] : 0ULL;
        for (int o = 16; o > 0; o >>= 1) m = umax64(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) atomicMax(red, m);
    }
}

template <typename T, int G>
__global__ void __launch_bounds__(256) k_velocity_norm(KP<T> p) {
    velocity_norm_body<T, G>(p, blockIdx.x, blockIdx.y, blockIdx.z, p.red);
}

// viscous stresses of the current velocities: τ_ii = 2 η D_ii at cells,
// τ_ij = avg4(η) D_ij at edges (the PT stress update's fixed point), and
// rP = div V.  Used by the FP64 residual.
template <typename T, int G>
__global__ void __launch_bounds__(256) k_tau_visc(KP<T> p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const T q4 = T(0.25);
    {
        const CellD<T> D = cell_strain<T, G>(p.geo, p.d1, p.d2, p.d3, i, j, p.V1[c], p.V1[c + 1], p.V2[c], p.V2[c + sy], p.V3[c], p.V3[c + sz]);
        const T e2 = T(2) * p.eta[c];
        p.t11[c] = e2 * D.D11; p.t22[c] = e2 * D.D22; p.t33[c] = e2 * D.D33;
        p.rP[c] = D.div;
    }
    if (i < d.n1 - 1 && j < d.n2 - 1 && k < d.n3 - 2) {
        const int q = c + sz;
        const T aE = (p.eta[q] + p.eta[q + sy] + p.eta[q + 1] + p.eta[q + 1 + sy]) * q4;
        p.t12[c] = aE * edge12<T, G>(p.geo, p.d1, p.d2, i, p.V2[q + sy], p.V2[q + sy + 1], p.V1[q + 1], p.V1[q + 1 + sy]);
    }
    if (i < d.n1 - 1 && j < d.n2 - 2 && k < d.n3 - 1) {
        const int q = c + sy;
        const T aE = (p.eta[q] + p.eta[q + sz] + p.eta[q + 1] + p.eta[q + 1 + sz]) * q4;
        p.t13[c] = aE * edge13<T, G>(p.geo, p.d1, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + 1], p.V1[q + 1], p.V1[q + 1 + sz]);
    }
    if (i < d.n1 - 2 && j < d.n2 - 1 && k < d.n3 - 1) {
        const int q = c + 1;
        const T aE = (p.eta[q] + p.eta[q + sz] + p.eta[q + sy] + p.eta[q + sy + sz]) * q4;
        p.t23[c] = aE * edge23<T, G>(p.geo, p.d2, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + sy], p.V2[q + sy], p.V2[q + sy + sz]);
    }
}

// ---------------------------------------------------------------------------
// Boundary conditions.  A BC set is a list of stages run in order; the ops of
// one stage act on different fields across the faces normal to one axis, so
// they are independent.  Each op writes both faces of its field:
//   NEG     A[b] = -A[in]          COPY  A[b] = A[in]          ZERO  A[b] = 0
//   LIN     A[b] = (x_cd - c1)*c0  LIN2M A[b] = 2*(x_cd - c1)*c0 - A[in]
//   STRESS  normal-velocity ghost giving the boundary cell the total normal
//           stress sig (x2 or x3 faces; not in the reference)
// x_cd is the cell-centre coordinate of the node along axis cd.  In the
// homogeneous form (correction problem) constants vanish: LIN -> 0,
// LIN2M -> -A[in], sig -> 0.
// BC_STRESS_SRC: BC_STRESS in a stage that also copies the two tangential fields
// into their ghost layer; it reads those fields at the copies' source cells
// instead of at the ghosts the copies are writing (the same values)
enum BcKind { BC_NEG = 0, BC_COPY = 1, BC_ZERO = 2, BC_LIN = 3, BC_LIN2M = 4, BC_STRESS = 5, BC_STRESS_SRC = 6 };
struct BcOp { int field; int kind; int cd; double c0, c1; int side; };  // side: -1 both faces, 0 low, 1 high
struct BcStage { int dim; int nops; BcOp op[3]; };

template <typename T>
__device__ __forceinline__ T* vfield(const KP<T>& p, int f) { return f == 0 ? p.V1 : (f == 1 ? p.V2 : p.V3); }

// one BC stage at face point (u, v) of the stage's faces (both sides); the body of k_bc and of
// the batched BC launch over many grids
template <typename T, int G>
__device__ __forceinline__ void bc_body(const KP<T>& p, const BcStage& st, int homog, int u, int v) {
    const Dims& d = p.d;
    const int D = st.dim;
    const int sy = d.sy, sz = d.sz;
    for (int o = 0; o < st.nops; ++o) {
        const BcOp op = st.op[o];
        const int f = op.field;
        // extents of field f: V1 (n1+1,n2,n3), V2 (n1,n2+1,n3), V3 (n1,n2,n3+1)
        int ext[3] = {d.n1 + (f == 0), d.n2 + (f == 1), d.n3 + (f == 2)};
        const int du = D == 0 ? 1 : 0, dv = D == 2 ? 1 : 2;
        if (u >= ext[du] || v >= ext[dv]) continue;
        T* A = vfield(p, f);
        const int stride[3] = {1, sy, sz};
        const int base = u * stride[du] + v * stride[dv];
        for (int side = 0; side < 2; ++side) {
            if (op.side >= 0 && op.side != side) continue;
            const int b = side == 0 ? 0 : ext[D] - 1;
            const int in = side == 0 ? 1 : ext[D] - 2;
            const int cb = base + b * stride[D], ci = base + in * stride[D];
            T val;
            switch (op.kind) {
                case BC_NEG: val = -A[ci]; break;
                case BC_COPY: val = A[ci]; break;
                case BC_ZERO: val = T(0); break;
                case BC_LIN: {
                    if (homog) { val = T(0); break; }
                    const int idx = (op.cd == D) ? b : (op.cd == du ? u : v);
                    const T* xc = op.cd == 0 ? p.geo.x1c : (op.cd == 1 ? p.geo.x2c : p.geo.x3c);
                    val = (xc[idx] - T(op.c1)) * T(op.c0);
                    break;
                }
                case BC_LIN2M: {
                    if (homog) { val = -A[ci]; break; }
                    const int idx = (op.cd == D) ? b : (op.cd == du ? u : v);
                    const T* xc = op.cd == 0 ? p.geo.x1c : (op.cd == 1 ? p.geo.x2c : p.geo.x3c);
                    val = T(2) * (xc[idx] - T(op.c1)) * T(op.c0) - A[ci];
                    break;
                }
                default: {  // BC_STRESS: normal ghost of V1 (D == 0), V2 (D == 1) or V3 (D == 2) from div V = 0 in the boundary cell
                    const int cellb = side == 0 ? 0 : ext[D] - 2;        // boundary cell index along D
                    // boundary cell (its tangential velocities: at the ghost, or at the source of its copy)
                    const int cc = base + (op.kind == BC_STRESS_SRC ? cellb + (side == 0 ? 1 : -1) : cellb) * stride[D];
                    const int i = (D == 0) ? cellb : u;
                    const int j = (D == 1) ? cellb : (du == 1 ? u : v);
                    const CellMetric<T> m = cell_metric<T, G>(p, i, j);
                    const T sgn = side == 0 ? T(-1) : T(1);
                    const T avx = (p.V1[cc] + p.V1[cc + 1]) * T(0.5);
                    const T vin = A[ci];
                    T A0, B;
                    if (D == 0) {  // V1 ghost of the free-surface top (or bottom) face
                        const T avy = (p.V2[cc] + p.V2[cc + sy]) * T(0.5);
                        A0 = p.d1 * (-sgn) * vin + T(0.5) * m.c1 * vin + m.a2 * (p.V2[cc + sy] - p.V2[cc]) + m.a3 * (p.V3[cc + sz] - p.V3[cc]) +
                             m.c2 * avy;
                        B = p.d1 * sgn + T(0.5) * m.c1;
                    } else if (D == 1) {
                        A0 = p.d1 * (p.V1[cc + 1] - p.V1[cc]) + m.a3 * (p.V3[cc + sz] - p.V3[cc]) + m.c1 * avx + m.a2 * (-sgn) * vin + m.c2 * T(0.5) * vin;
                        B = m.a2 * sgn + T(0.5) * m.c2;
                    } else {
                        const T avy = (p.V2[cc] + p.V2[cc + sy]) * T(0.5);
                        A0 = p.d1 * (p.V1[cc + 1] - p.V1[cc]) + m.a2 * (p.V2[cc + sy] - p.V2[cc]) + m.c1 * avx + m.c2 * avy + m.a3 * (-sgn) * vin;
                        B = m.a3 * sgn;
                    }
                    val = -A0 / B;
                    break;
                }
            }
            A[cb] = val;
        }
    }
}

template <typename T, int G>
__global__ void k_bc(KP<T> p, BcStage st, int homog) {
    pdl_enter();
    bc_body<T, G>(p, st, homog, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

// ---------------------------------------------------------------------------
// P_out = P except on the boundary cells of the normal-stress BC, where
// P_out = τ_nn - σ_bc from the given stresses (residual evaluation)
template <typename T>
__global__ void k_traction_pressure(KP<T> p, T* __restrict__ Pout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int c = i + d.sy * j + d.sz * k;
    T P = p.P[c];
    if (p.traction) traction_pressure(j, k, d.n2, d.n3, p.t22[c], p.t33[c], p.sig2, p.sig3, P);
    if (p.fs && i == d.n1 - 1) P = fs_pressure(p.t11[c], p.top_load ? p.top_load[c] : T(0), p.fs_kappa, p.V1[c], p.V1[c + 1]);
    Pout[c] = P;
}

// ---------------------------------------------------------------------------
// reductions: max|a| (or max|a-b|) over n entries into red[slot], as the ordered
// bits of ord_bits (a NaN entry makes the result NaN, as Julia's maximum(abs.(.)))
// block-wide max of ordered bits, one atomicMax per block
__device__ __forceinline__ void block_max_to(unsigned long long v, unsigned long long* slot) {
    for (int o = 16; o > 0; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ unsigned long long sm[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0ULL;
        for (int o = 16; o > 0; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) atomicMax(slot, v);
    }
}

template <typename T>
__global__ void k_maxabs(const T* __restrict__ a, const T* __restrict__ b, long long n, unsigned long long* slot) {
    unsigned long long m = 0ULL;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        m = umax64(m, ord_bits(b ? (double)a[q] - (double)b[q] : (double)a[q]));
    block_max_to(m, slot);
}

// ---------------------------------------------------------------------------
// elementwise helpers over the whole box
template <typename TD, typename TS>
__global__ void k_convert(TD* __restrict__ dst, const TS* __restrict__ src, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) dst[q] = (TD)src[q];
}
// dst += (double)src
template <typename TS>
__global__ void k_add_widen(double* __restrict__ dst, const TS* __restrict__ src, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) dst[q] += (double)src[q];
}

// A field in the reference layout (dense e0 x e1 x e2 doubles, x1 fastest) <-> its
// entries in the padded box (strides 1, sy, sz).  Launch: grid (ceil(e0/blockDim.x),
// e1, e2); one entry per thread, consecutive threads on consecutive x1 entries on
// both sides.  The host copies whole dense fields in one transfer and these kernels
// do the re-pitching on the device.
template <typename T>
__device__ __forceinline__ T from_double(double v) { return (T)v; }
template <>
__device__ __forceinline__ uint8_t from_double<uint8_t>(double v) { return v != 0.0 ? 1 : 0; }

template <typename T>
__global__ void k_unpack(T* __restrict__ box, const double* __restrict__ dense, int e0, int e1, int sy, int sz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e0) return;
    const int j = blockIdx.y, k = blockIdx.z;
    box[i + (long long)sy * j + (long long)sz * k] = from_double<T>(dense[i + (long long)e0 * (j + (long long)e1 * k)]);
}
template <typename T>
__global__ void k_pack(double* __restrict__ dense, const T* __restrict__ box, int e0, int e1, int sy, int sz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e0) return;
    const int j = blockIdx.y, k = blockIdx.z;
    dense[i + (long long)e0 * (j + (long long)e1 * k)] = (double)box[i + (long long)sy * j + (long long)sz * k];
}

}  // namespace sph
