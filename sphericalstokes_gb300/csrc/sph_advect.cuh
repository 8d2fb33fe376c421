// Explicit advection of cell fields by the current velocities (diapir ascent
// between Stokes solves; not in the reference, whose scripts run one time step)
// and its transpose.
//
// φ_new(c) = φ(c) - dt Σ_d a_d [ v_d (Δb + Δf)/2 - s(v_d) (Δf - Δb)/2 ]
//   v_d   = mean of the two face velocities of component d around cell c
//   a_d   = metric factor of the derivative along d: d1, d2/r, d3/(r sinθ)
//           (cylindrical d1, d2/r, d3; Cartesian d1, d2, d3)
//   Δb, Δf = backward / forward differences of φ along d (zero where the
//           neighbour is outside the grid)
//   s(v)  = sqrt(v² + δ²)
// With s(v) = |v| this is first-order upwinding; the smoothed |v| makes the step
// differentiable where a velocity component changes sign (stagnation surfaces,
// free-slip walls), which the adjoint needs, and adds a diffusion of order δ h
// there.  Up to four fields per launch.
#pragma once
#include "sph_pt.cuh"

namespace sph {

struct AdvFields {
    int nf;
    const double* in[4];
    double* out[4];
};

template <int G>
__device__ __forceinline__ void adv_metric(const KP<double>& p, int i, int j, double a[3]) {
    a[0] = p.d1;
    a[1] = p.d2;
    a[2] = p.d3;
    if (G != CART) a[1] = p.d2 * p.geo.invRc[i];
    if (G == SPH) a[2] = p.d3 * p.geo.invRc[i] * p.geo.invSinC[j];
}

template <int G>
__global__ void __launch_bounds__(256) k_advect(KP<double> p, AdvFields F, double dt, double delta) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const double v[3] = {0.5 * (p.V1[c] + p.V1[c + 1]), 0.5 * (p.V2[c] + p.V2[c + sy]), 0.5 * (p.V3[c] + p.V3[c + sz])};
    double a[3];
    adv_metric<G>(p, i, j, a);
    const int idx[3] = {i, j, k}, ext[3] = {d.n1, d.n2, d.n3}, str[3] = {1, sy, sz};
    for (int f = 0; f < F.nf; ++f) {
        const double* q = F.in[f];
        double s = 0.0;
        for (int dd = 0; dd < 3; ++dd) {
            const double db = idx[dd] > 0 ? q[c] - q[c - str[dd]] : 0.0;
            const double df = idx[dd] < ext[dd] - 1 ? q[c + str[dd]] - q[c] : 0.0;
            const double av = sqrt(v[dd] * v[dd] + delta * delta);
            s += a[dd] * (v[dd] * (db + df) * 0.5 - av * (df - db) * 0.5);
        }
        F.out[f][c] = q[c] - dt * s;
    }
}

// transpose: F.in = φ (the fields the step read), M.in = adjoint of φ_new,
// M.out += adjoint of φ, aV* += velocity adjoint (all entries)
template <int G>
__global__ void __launch_bounds__(256) k_advect_vjp(KP<double> p, AdvFields F, AdvFields M, double* aV1, double* aV2, double* aV3,
                                                    double dt, double delta) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const double v[3] = {0.5 * (p.V1[c] + p.V1[c + 1]), 0.5 * (p.V2[c] + p.V2[c + sy]), 0.5 * (p.V3[c] + p.V3[c + sz])};
    double a[3];
    adv_metric<G>(p, i, j, a);
    const int idx[3] = {i, j, k}, ext[3] = {d.n1, d.n2, d.n3}, str[3] = {1, sy, sz};
    double* aV[3] = {aV1, aV2, aV3};
    for (int f = 0; f < F.nf; ++f) {
        const double* q = F.in[f];
        double* mu_old = M.out[f];
        const double m = M.in[f][c];
        if (m == 0.0) continue;
        atomicAdd(mu_old + c, m);
        for (int dd = 0; dd < 3; ++dd) {
            const bool hb = idx[dd] > 0, hf = idx[dd] < ext[dd] - 1;
            const double db = hb ? q[c] - q[c - str[dd]] : 0.0;
            const double df = hf ? q[c + str[dd]] - q[c] : 0.0;
            const double av = sqrt(v[dd] * v[dd] + delta * delta);
            const double w = -dt * a[dd] * m;  // adjoint of the bracket
            const double wb = w * (v[dd] + av) * 0.5, wf = w * (v[dd] - av) * 0.5;  // of Δb, Δf
            if (hb) { atomicAdd(mu_old + c, wb); atomicAdd(mu_old + c - str[dd], -wb); }
            if (hf) { atomicAdd(mu_old + c + str[dd], wf); atomicAdd(mu_old + c, -wf); }
            // v_d = (V_d(c) + V_d(c + str)) / 2
            const double gv = w * ((db + df) * 0.5 - (v[dd] / av) * (df - db) * 0.5) * 0.5;
            if (gv != 0.0) { atomicAdd(aV[dd] + c, gv); atomicAdd(aV[dd] + c + str[dd], gv); }
        }
    }
}

}  // namespace sph
