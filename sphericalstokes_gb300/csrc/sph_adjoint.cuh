// Adjoint (vector-Jacobian product) kernels of the FP64 Stokes residual with
// the viscosity frozen (the linear operator of one Picard step; the n = 1 law
// exactly).  Forward map (residual64 of sphstokes.cu):
//   V (all entries) --strain rates, 2ηD / avg4(η)D--> τ  (k_tau_visc)
//   σ_ii = τ_ii - P_eff, P_eff = P or τ_nn - σ_bc on far-field-stress boundary cells
//   R_V = momentum(σ, τ_edges) - ρg at interior nodes  (k_velocity MODE 2)
//   R_P = div V at every cell
// and, for the interior-unknown form, V = B(V_interior) by the homogeneous BC
// program.  Each kernel here is the transpose of one forward step, written as a
// scatter: a thread takes the adjoint of the outputs it owns and adds
// coefficient × adjoint to every input (FP64 atomics).  The coefficients are the
// forward stencil functions of sph_core.cuh evaluated on unit inputs (they are
// linear in the field values), so the transpose matches the forward arithmetic
// term by term.  Gradients with respect to η (per cell) and ρ (per cell) come
// out of the same pass.
#pragma once
#include "sph_pt.cuh"

namespace sph {

struct Adj {
    const double *lV1, *lV2, *lV3, *lP;  // adjoint of the residual rows (interior nodes / all cells)
    double *aS11, *aS22, *aS33;          // adjoint of σ_ii, then of τ_ii (cells)
    double *aT12, *aT13, *aT23;          // adjoint of the edge stresses
    double *aV1, *aV2, *aV3, *aP;        // output: adjoint of V (all entries), P
    double *gEta, *gRho;                 // output: λᵀ ∂R/∂η, λᵀ ∂R/∂ρ per cell
};

__device__ __forceinline__ void aadd(double* a, double v) {
    if (v != 0.0) atomicAdd(a, v);
}

// momentum rows -> σ_ii, edge stresses, ρ (one thread per interior node, like k_velocity)
template <int G>
__global__ void __launch_bounds__(256) k_vjp_momentum(KP<double> p, Adj a) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1, K = blockIdx.z + 1;
    const Dims& d = p.d;
    if (I > d.n1 - 1 || J > d.n2 - 1 || K > d.n3 - 1) return;
    const int sy = d.sy, sz = d.sz;
    const int c = I + sy * J + sz * K;
    const double h = 0.5;
    if (J <= d.n2 - 2 && K <= d.n3 - 2) {  // V1 (I-1/2, J, K)
        const double lam = a.lV1[c];
        if (lam != 0.0) {
            const int m = c - 1;
            double x[10];
            double* dst[10] = {a.aS11 + m, a.aS11 + c, a.aS22 + m, a.aS22 + c, a.aS33 + m, a.aS33 + c,
                               a.aT12 + (m - sz), a.aT12 + (m - sy - sz), a.aT13 + (m - sy), a.aT13 + (m - sy - sz)};
            for (int q = 0; q < 10; ++q) {
                for (int t = 0; t < 10; ++t) x[t] = (t == q) ? 1.0 : 0.0;
                const double cf = mom1<double, G>(p.geo, p.d1, p.d2, p.d3, I, J, x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8], x[9]);
                aadd(dst[q], lam * cf);
            }
            if (G != CART) { aadd(a.gRho + m, -lam * p.g * h); aadd(a.gRho + c, -lam * p.g * h); }
        }
    }
    if (I <= d.n1 - 2 && K <= d.n3 - 2) {  // V2 (I, J-1/2, K)
        const double lam = a.lV2[c];
        if (lam != 0.0) {
            const int m = c - sy;
            double x[8];
            double* dst[8] = {a.aS22 + m, a.aS22 + c, a.aS33 + m, a.aS33 + c,
                              a.aT12 + (c - sy - sz), a.aT12 + (c - 1 - sy - sz), a.aT23 + (c - 1 - sy), a.aT23 + (c - 1 - sy - sz)};
            for (int q = 0; q < 8; ++q) {
                for (int t = 0; t < 8; ++t) x[t] = (t == q) ? 1.0 : 0.0;
                const double cf = mom2<double, G>(p.geo, p.d1, p.d2, p.d3, I, J, x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7]);
                aadd(dst[q], lam * cf);
            }
        }
    }
    if (I <= d.n1 - 2 && J <= d.n2 - 2) {  // V3 (I, J, K-1/2)
        const double lam = a.lV3[c];
        if (lam != 0.0) {
            const int m = c - sz;
            double x[6];
            double* dst[6] = {a.aS33 + m, a.aS33 + c, a.aT13 + (c - sy - sz), a.aT13 + (c - 1 - sy - sz),
                              a.aT23 + (c - 1 - sz), a.aT23 + (c - 1 - sy - sz)};
            for (int q = 0; q < 6; ++q) {
                for (int t = 0; t < 6; ++t) x[t] = (t == q) ? 1.0 : 0.0;
                const double cf = mom3<double, G>(p.geo, p.d1, p.d2, p.d3, I, J, x[0], x[1], x[2], x[3], x[4], x[5]);
                aadd(dst[q], lam * cf);
            }
            if (G == CART) { aadd(a.gRho + m, -lam * p.g * h); aadd(a.gRho + c, -lam * p.g * h); }
        }
    }
}

// σ_ii = τ_ii - P_eff: adjoint of σ becomes the adjoint of τ (in place) and of P;
// on far-field-stress boundary cells P_eff is a function of τ22 / τ33 instead of P
__global__ void __launch_bounds__(256) k_vjp_pressure(KP<double> p, Adj a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int c = i + d.sy * j + d.sz * k;
    const double aPe = -(a.aS11[c] + a.aS22[c] + a.aS33[c]);
    const bool b2 = p.traction && (j == 0 || j == d.n2 - 1), b3 = p.traction && (k == 0 || k == d.n3 - 1);
    if (b2 && b3) {
        a.aS22[c] += aPe * 0.5;
        a.aS33[c] += aPe * 0.5;
        a.aP[c] = 0.0;
    } else if (b2) {
        a.aS22[c] += aPe;
        a.aP[c] = 0.0;
    } else if (b3) {
        a.aS33[c] += aPe;
        a.aP[c] = 0.0;
    } else {
        a.aP[c] = aPe;
    }
}

// τ (cells, edges) and the continuity rows -> V (all entries), η
template <int G>
__global__ void __launch_bounds__(256) k_vjp_strain(KP<double> p, Adj a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const double q4 = 0.25;
    {
        const double e2 = 2.0 * p.eta[c];
        const double t11 = a.aS11[c], t22 = a.aS22[c], t33 = a.aS33[c], lp = a.lP[c];
        const double aD11 = e2 * t11, aD22 = e2 * t22, aD33 = e2 * t33;
        double* dst[6] = {a.aV1 + c, a.aV1 + c + 1, a.aV2 + c, a.aV2 + c + sy, a.aV3 + c, a.aV3 + c + sz};
        double x[6];
        for (int q = 0; q < 6; ++q) {
            for (int t = 0; t < 6; ++t) x[t] = (t == q) ? 1.0 : 0.0;
            const CellD<double> D = cell_strain<double, G>(p.geo, p.d1, p.d2, p.d3, i, j, x[0], x[1], x[2], x[3], x[4], x[5]);
            aadd(dst[q], D.div * lp + D.D11 * aD11 + D.D22 * aD22 + D.D33 * aD33);
        }
        const CellD<double> D = cell_strain<double, G>(p.geo, p.d1, p.d2, p.d3, i, j, p.V1[c], p.V1[c + 1], p.V2[c], p.V2[c + sy], p.V3[c],
                                                       p.V3[c + sz]);
        aadd(a.gEta + c, 2.0 * (t11 * D.D11 + t22 * D.D22 + t33 * D.D33));
    }
    if (i < d.n1 - 1 && j < d.n2 - 1 && k < d.n3 - 2) {  // τ12 = avg4(η) D12
        const int q = c + sz;
        const double at = a.aT12[c];
        if (at != 0.0) {
            const double aE = (p.eta[q] + p.eta[q + sy] + p.eta[q + 1] + p.eta[q + 1 + sy]) * q4;
            double* dst[4] = {a.aV2 + q + sy, a.aV2 + q + sy + 1, a.aV1 + q + 1, a.aV1 + q + 1 + sy};
            for (int s = 0; s < 4; ++s) {
                const double cf = edge12<double, G>(p.geo, p.d1, p.d2, i, s == 0 ? 1.0 : 0.0, s == 1 ? 1.0 : 0.0, s == 2 ? 1.0 : 0.0, s == 3 ? 1.0 : 0.0);
                aadd(dst[s], aE * at * cf);
            }
            const double D = edge12<double, G>(p.geo, p.d1, p.d2, i, p.V2[q + sy], p.V2[q + sy + 1], p.V1[q + 1], p.V1[q + 1 + sy]);
            const double ge = q4 * at * D;
            aadd(a.gEta + q, ge); aadd(a.gEta + q + sy, ge); aadd(a.gEta + q + 1, ge); aadd(a.gEta + q + 1 + sy, ge);
        }
    }
    if (i < d.n1 - 1 && j < d.n2 - 2 && k < d.n3 - 1) {  // τ13
        const int q = c + sy;
        const double at = a.aT13[c];
        if (at != 0.0) {
            const double aE = (p.eta[q] + p.eta[q + sz] + p.eta[q + 1] + p.eta[q + 1 + sz]) * q4;
            double* dst[4] = {a.aV3 + q + sz, a.aV3 + q + sz + 1, a.aV1 + q + 1, a.aV1 + q + 1 + sz};
            for (int s = 0; s < 4; ++s) {
                const double cf = edge13<double, G>(p.geo, p.d1, p.d3, i, j, s == 0 ? 1.0 : 0.0, s == 1 ? 1.0 : 0.0, s == 2 ? 1.0 : 0.0, s == 3 ? 1.0 : 0.0);
                aadd(dst[s], aE * at * cf);
            }
            const double D = edge13<double, G>(p.geo, p.d1, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + 1], p.V1[q + 1], p.V1[q + 1 + sz]);
            const double ge = q4 * at * D;
            aadd(a.gEta + q, ge); aadd(a.gEta + q + sz, ge); aadd(a.gEta + q + 1, ge); aadd(a.gEta + q + 1 + sz, ge);
        }
    }
    if (i < d.n1 - 2 && j < d.n2 - 1 && k < d.n3 - 1) {  // τ23
        const int q = c + 1;
        const double at = a.aT23[c];
        if (at != 0.0) {
            const double aE = (p.eta[q] + p.eta[q + sz] + p.eta[q + sy] + p.eta[q + sy + sz]) * q4;
            double* dst[4] = {a.aV3 + q + sz, a.aV3 + q + sz + sy, a.aV2 + q + sy, a.aV2 + q + sy + sz};
            for (int s = 0; s < 4; ++s) {
                const double cf = edge23<double, G>(p.geo, p.d2, p.d3, i, j, s == 0 ? 1.0 : 0.0, s == 1 ? 1.0 : 0.0, s == 2 ? 1.0 : 0.0, s == 3 ? 1.0 : 0.0);
                aadd(dst[s], aE * at * cf);
            }
            const double D = edge23<double, G>(p.geo, p.d2, p.d3, i, j, p.V3[q + sz], p.V3[q + sz + sy], p.V2[q + sy], p.V2[q + sy + sz]);
            const double ge = q4 * at * D;
            aadd(a.gEta + q, ge); aadd(a.gEta + q + sz, ge); aadd(a.gEta + q + sy, ge); aadd(a.gEta + q + sy + sz, ge);
        }
    }
}

// normal-velocity ghost of the far-field-stress BC (k_bc, BC_STRESS) as a function of its
// inputs: V1 at the boundary cell's two r-faces, the other tangential component's two
// faces, and the normal component one node inside (vin)
template <int G>
__device__ __forceinline__ double stress_ghost(const KP<double>& p, int D, int side, int i, int j, double v1a, double v1b, double wa,
                                               double wb, double vin) {
    const CellMetric<double> m = cell_metric<double, G>(p, i, j);
    const double sgn = side == 0 ? -1.0 : 1.0;
    const double avx = (v1a + v1b) * 0.5;
    double A0, B;
    if (D == 1) {  // wa, wb = V3 at cc, cc + sz
        A0 = p.d1 * (v1b - v1a) + m.a3 * (wb - wa) + m.c1 * avx + m.a2 * (-sgn) * vin + m.c2 * 0.5 * vin;
        B = m.a2 * sgn + 0.5 * m.c2;
    } else {  // wa, wb = V2 at cc, cc + sy
        const double avy = (wa + wb) * 0.5;
        A0 = p.d1 * (v1b - v1a) + m.a2 * (wb - wa) + m.c1 * avx + m.c2 * avy + m.a3 * (-sgn) * vin;
        B = m.a3 * sgn;
    }
    return -A0 / B;
}

// transpose of one homogeneous BC stage on the velocity adjoints: each boundary entry's
// adjoint goes back to the entries its value was computed from, then is cleared
template <int G>
__global__ void k_bc_adjoint(KP<double> p, Adj a, BcStage st) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y * blockDim.y + threadIdx.y;
    const Dims& d = p.d;
    const int D = st.dim;
    const int sy = d.sy, sz = d.sz;
    for (int o = st.nops - 1; o >= 0; --o) {
        const BcOp op = st.op[o];
        const int f = op.field;
        int ext[3] = {d.n1 + (f == 0), d.n2 + (f == 1), d.n3 + (f == 2)};
        const int du = D == 0 ? 1 : 0, dv = D == 2 ? 1 : 2;
        if (u >= ext[du] || v >= ext[dv]) continue;
        double* A = f == 0 ? a.aV1 : (f == 1 ? a.aV2 : a.aV3);
        const int stride[3] = {1, sy, sz};
        const int base = u * stride[du] + v * stride[dv];
        for (int side = 1; side >= 0; --side) {
            const int b = side == 0 ? 0 : ext[D] - 1;
            const int in = side == 0 ? 1 : ext[D] - 2;
            const int cb = base + b * stride[D], ci = base + in * stride[D];
            const double g = A[cb];
            A[cb] = 0.0;
            if (g == 0.0) continue;
            switch (op.kind) {
                case BC_NEG: atomicAdd(A + ci, -g); break;
                case BC_COPY: atomicAdd(A + ci, g); break;
                case BC_LIN2M: atomicAdd(A + ci, -g); break;  // homogeneous form: -A[in]
                case BC_ZERO:
                case BC_LIN: break;                              // constants: no dependence
                default: {                                       // BC_STRESS
                    const int cellb = side == 0 ? 0 : ext[D] - 2;
                    const int cc = base + cellb * stride[D];
                    const int i = (D == 0) ? cellb : u;
                    const int j = (D == 1) ? cellb : (du == 1 ? u : v);
                    const int wstep = D == 1 ? sz : sy;
                    double* W = D == 1 ? a.aV3 : a.aV2;
                    double* dst[5] = {a.aV1 + cc, a.aV1 + cc + 1, W + cc, W + cc + wstep, A + ci};
                    for (int q = 0; q < 5; ++q) {
                        const double cf = stress_ghost<G>(p, D, side, i, j, q == 0 ? 1.0 : 0.0, q == 1 ? 1.0 : 0.0, q == 2 ? 1.0 : 0.0,
                                                          q == 3 ? 1.0 : 0.0, q == 4 ? 1.0 : 0.0);
                        atomicAdd(dst[q], g * cf);
                    }
                    break;
                }
            }
        }
    }
}

// The strain-rate law's part of the transposed Jacobian (k_edot_law, unrelaxed target
// η_t = 2/(1/η_ini + 1/η_PL), η_PL = η_ini (ε̇_II/ε̇_bg)^m, m = (1-n)/n, ε̇_II of the clamped
// interior cell s from sDD(s) and the 4-edge averages a, b, c of the shear rates):
//   dη_t/dε̇ = m η_t² / (2 η_PL ε̇),  dε̇/dsDD = 1/(2ε̇),  dε̇/da = a/(4ε̇),  da/ds12(edge) = 1/4,
//   sDD = ½ Σ D_ii²,  dη_t/dη_ini = η_t/η_ini,  dη_t/dn = -η_t² ln(ε̇/ε̇_bg) / (2 η_PL n²).
// With g = λᵀ ∂R/∂η per cell (k_vjp_strain), NEWTON adds (∂η/∂V)ᵀ g to the velocity adjoint;
// gEI and gN receive g dη_t/dη_ini and g dη_t/dn.  Phase cells (linear) have η = η_ini.
template <int G, bool NEWTON>
__global__ void __launch_bounds__(256) k_vjp_law(KP<double> p, Adj a, double* __restrict__ gEI, double* __restrict__ gN) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const double g = a.gEta[c];
    const double ei = p.eta_ini[c];
    if (p.phase && p.phase[c]) {
        gEI[c] = g;
        gN[c] = 0.0;
        return;
    }
    const int si = clampi(i, 1, d.n1 - 2), sj = clampi(j, 1, d.n2 - 2), sk = clampi(k, 1, d.n3 - 2);
    const int s = si + sy * sj + sz * sk;
    const double q4 = 0.25;
    const int e = s - 1 - sy - sz;
    const double av = (p.s12[e] + p.s12[e + sy] + p.s12[e + 1] + p.s12[e + 1 + sy]) * q4;
    const double bv = (p.s13[e] + p.s13[e + sz] + p.s13[e + 1] + p.s13[e + 1 + sz]) * q4;
    const double cv = (p.s23[e] + p.s23[e + sz] + p.s23[e + sy] + p.s23[e + sy + sz]) * q4;
    const double ed = sqrt(p.sDD[s] + q4 * (av * av + bv * bv + cv * cv));
    const double n = p.n_exp, m = (1.0 - n) / n;
    const double pl = ei * pow(ed / p.edot_bg, m);
    const double et = 2.0 / (1.0 / ei + 1.0 / pl);
    gEI[c] = g * et / ei;
    gN[c] = ed > 0.0 ? -g * et * et * log(ed / p.edot_bg) / (2.0 * pl * n * n) : 0.0;
    if (!NEWTON || g == 0.0 || !(ed > 0.0)) return;
    const double w = g * m * et * et / (2.0 * pl * ed);  // g dη_t/dε̇
    // ε̇ -> sDD(s) -> D_ii(s) -> V around s
    {
        const double ws = w / (2.0 * ed);
        const CellD<double> D = cell_strain<double, G>(p.geo, p.d1, p.d2, p.d3, si, sj, p.V1[s], p.V1[s + 1], p.V2[s], p.V2[s + sy],
                                                       p.V3[s], p.V3[s + sz]);
        double* dst[6] = {a.aV1 + s, a.aV1 + s + 1, a.aV2 + s, a.aV2 + s + sy, a.aV3 + s, a.aV3 + s + sz};
        for (int q = 0; q < 6; ++q) {
            const CellD<double> u = cell_strain<double, G>(p.geo, p.d1, p.d2, p.d3, si, sj, q == 0 ? 1.0 : 0.0, q == 1 ? 1.0 : 0.0,
                                                           q == 2 ? 1.0 : 0.0, q == 3 ? 1.0 : 0.0, q == 4 ? 1.0 : 0.0, q == 5 ? 1.0 : 0.0);
            aadd(dst[q], ws * (D.D11 * u.D11 + D.D22 * u.D22 + D.D33 * u.D33));
        }
    }
    // ε̇ -> the 4-edge averages -> each edge's shear rate -> its 4 velocities
    const double wa = w * av / (4.0 * ed) * q4, wb = w * bv / (4.0 * ed) * q4, wc = w * cv / (4.0 * ed) * q4;
    const int e12[4] = {e, e + sy, e + 1, e + 1 + sy};
    for (int t = 0; t < 4; ++t) {
        const int ec = e12[t];
        const int ii = ec % sy, q = ec + sz;
        double* dst[4] = {a.aV2 + q + sy, a.aV2 + q + sy + 1, a.aV1 + q + 1, a.aV1 + q + 1 + sy};
        for (int u = 0; u < 4; ++u)
            aadd(dst[u], wa * edge12<double, G>(p.geo, p.d1, p.d2, ii, u == 0 ? 1.0 : 0.0, u == 1 ? 1.0 : 0.0, u == 2 ? 1.0 : 0.0, u == 3 ? 1.0 : 0.0));
    }
    const int e13[4] = {e, e + sz, e + 1, e + 1 + sz};
    for (int t = 0; t < 4; ++t) {
        const int ec = e13[t];
        const int ii = ec % sy, jj = (ec / sy) % d.py, q = ec + sy;
        double* dst[4] = {a.aV3 + q + sz, a.aV3 + q + sz + 1, a.aV1 + q + 1, a.aV1 + q + 1 + sz};
        for (int u = 0; u < 4; ++u)
            aadd(dst[u], wb * edge13<double, G>(p.geo, p.d1, p.d3, ii, jj, u == 0 ? 1.0 : 0.0, u == 1 ? 1.0 : 0.0, u == 2 ? 1.0 : 0.0, u == 3 ? 1.0 : 0.0));
    }
    const int e23[4] = {e, e + sz, e + sy, e + sy + sz};
    for (int t = 0; t < 4; ++t) {
        const int ec = e23[t];
        const int ii = ec % sy, jj = (ec / sy) % d.py, q = ec + 1;
        double* dst[4] = {a.aV3 + q + sz, a.aV3 + q + sz + sy, a.aV2 + q + sy, a.aV2 + q + sy + sz};
        for (int u = 0; u < 4; ++u)
            aadd(dst[u], wc * edge23<double, G>(p.geo, p.d2, p.d3, ii, jj, u == 0 ? 1.0 : 0.0, u == 1 ? 1.0 : 0.0, u == 2 ? 1.0 : 0.0, u == 3 ? 1.0 : 0.0));
    }
}

// pseudo-steps of the current viscosity (k_stress's DT_R) for the adjoint iteration
__global__ void __launch_bounds__(256) k_pt_dtr(KP<double> p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int c = i + d.sy * j + d.sz * k;
    const double sm = p.etaSM[c], e = p.eta[c];
    const double gs = p.gsc * sm, kb = p.kbc * sm;
    p.DT_R[c] = p.vpdt2 / (kb + gs * (e / (e + gs)));
}

// Transposed PT with the forward scheme's stress memory.  The forward PT relaxes
// τ toward 2η E(V) at the rate 1 - f (f = η/(η + GSDT); edges: avg4 η, avg4 GSDT) and
// drives V with the momentum of τ.  The transposed iteration relaxes the memory μ toward
// 2η M_τᵀ λ_V (M_τᵀ λ_V = aτ from k_vjp_momentum + k_vjp_pressure) at the same rate and
// drives λ_V with Eᵀ μ: the coupling products are the transposes of the forward ones.
// Here μ is updated and handed to k_vjp_strain as aτ = μ / (2η) (edges μ / avg4 η),
// so that kernel forms Eᵀ μ.
__global__ void __launch_bounds__(256) k_adj_memory(KP<double> p, Adj a, double* __restrict__ m11, double* __restrict__ m22,
                                                    double* __restrict__ m33, double* __restrict__ m12, double* __restrict__ m13,
                                                    double* __restrict__ m23) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const double q4 = 0.25;
    {
        const double e = p.eta[c], gs = p.gsc * p.etaSM[c];
        const double w = gs / (e + gs);  // 1 - f
        const double e2 = 2.0 * e;
        double* m[3] = {m11, m22, m33};
        double* t[3] = {a.aS11, a.aS22, a.aS33};
        for (int q = 0; q < 3; ++q) {
            const double mu = m[q][c] + w * (e2 * t[q][c] - m[q][c]);
            m[q][c] = mu;
            t[q][c] = mu / e2;
        }
    }
    auto edge = [&](double* mu, double* at, int q, int o1, int o2, int o3) {
        const double aE = (p.eta[q] + p.eta[q + o1] + p.eta[q + o2] + p.eta[q + o3]) * q4;
        const double aG = p.gsc * ((p.etaSM[q] + p.etaSM[q + o1] + p.etaSM[q + o2] + p.etaSM[q + o3]) * q4);
        const double w = aG / (aE + aG);
        const double v = mu[c] + w * (aE * at[c] - mu[c]);
        mu[c] = v;
        at[c] = v / aE;
    };
    if (i < d.n1 - 1 && j < d.n2 - 1 && k < d.n3 - 2) edge(m12, a.aT12, c + sz, sy, 1, 1 + sy);
    if (i < d.n1 - 1 && j < d.n2 - 2 && k < d.n3 - 1) edge(m13, a.aT13, c + sy, sz, 1, 1 + sz);
    if (i < d.n1 - 2 && j < d.n2 - 1 && k < d.n3 - 1) edge(m23, a.aT23, c + 1, sz, sy, sy + sz);
}

// λ_P of the transposed PT: λ_P -= KBDT (M_Pᵀ λ_V - b_P), before the velocity rows use it
__global__ void __launch_bounds__(256) k_adj_pressure_update(KP<double> p, Adj a, double* __restrict__ lP, const double* __restrict__ bP) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i >= d.n1 || j >= d.n2 || k >= d.n3) return;
    const int c = i + d.sy * j + d.sz * k;
    lP[c] -= p.kbc * p.etaSM[c] * (a.aP[c] - bP[c]);
}

// λ_V of the transposed PT: λ_V += avg(DT_R) (Eᵀ μ + Dᵀ λ_P - b_V) at interior nodes
__global__ void __launch_bounds__(256) k_adj_velocity_update(KP<double> p, Adj a, double* lV1, double* lV2, double* lV3,
                                                             const double* bV1, const double* bV2, const double* bV3) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y * blockDim.y + threadIdx.y + 1, k = blockIdx.z + 1;
    const Dims& d = p.d;
    if (i > d.n1 - 1 || j > d.n2 - 1 || k > d.n3 - 1) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const double h = 0.5;
    if (j <= d.n2 - 2 && k <= d.n3 - 2) lV1[c] += (a.aV1[c] - bV1[c]) * ((p.DT_R[c - 1] + p.DT_R[c]) * h);
    if (i <= d.n1 - 2 && k <= d.n3 - 2) lV2[c] += (a.aV2[c] - bV2[c]) * ((p.DT_R[c - sy] + p.DT_R[c]) * h);
    if (i <= d.n1 - 2 && j <= d.n2 - 2) lV3[c] += (a.aV3[c] - bV3[c]) * ((p.DT_R[c - sz] + p.DT_R[c]) * h);
}

// residual of the transposed system, r = Aᵀλ - b (convergence check)
__global__ void __launch_bounds__(256) k_adj_residual(KP<double> p, Adj a, const double* bV1, const double* bV2, const double* bV3,
                                                      const double* bP, double* rV1, double* rV2, double* rV3, double* rP) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const Dims& d = p.d;
    if (i > d.n1 || j > d.n2 || k > d.n3) return;
    const int sy = d.sy, sz = d.sz;
    const int c = i + sy * j + sz * k;
    const bool in1 = i >= 1 && i <= d.n1 - 1, in2 = j >= 1 && j <= d.n2 - 1, in3 = k >= 1 && k <= d.n3 - 1;
    rV1[c] = (in1 && in2 && in3 && j <= d.n2 - 2 && k <= d.n3 - 2) ? a.aV1[c] - bV1[c] : 0.0;
    rV2[c] = (in1 && in2 && in3 && i <= d.n1 - 2 && k <= d.n3 - 2) ? a.aV2[c] - bV2[c] : 0.0;
    rV3[c] = (in1 && in2 && in3 && i <= d.n1 - 2 && j <= d.n2 - 2) ? a.aV3[c] - bV3[c] : 0.0;
    rP[c] = (i < d.n1 && j < d.n2 && k < d.n3) ? a.aP[c] - bP[c] : 0.0;
}

}  // namespace sph
