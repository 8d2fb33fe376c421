// ORACLE — test infrastructure only.
//
// CPU FP64 restatement of the cylindrical and Cartesian diapir scripts of
// PTsolvers/SphericalStokes:
//   scripts_diapir/CylindricalStokes_diapir.jl (FD-macro kernels :41-220, loop :328-366)
//   scripts_diapir/CartesianStokes_diapir.jl   (index kernels :41-260, loop :349-379)
// Layout and indexing as in oracle.cpp (1-based, column-major, the scripts'
// array sizes).  ParallelStencil.FiniteDifferences3D macros are written out
// as the small lambdas below (d_xa, av_xyi, ...), with their published
// definitions.  Pinned against tests/golden/{cyl,cart}_diapir*.npz.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

namespace {

const double PI = 3.141592653589793;

struct Arr {
    double* p;
    long n1, n2, n3;
    inline double& operator()(long i, long j, long k) const { return p[(i - 1) + n1 * ((j - 1) + n2 * (k - 1))]; }
};
inline Arr A(double* p, long a, long b, long c) { return Arr{p, a, b, c}; }
inline double sq(double x) { return x * x; }

void copy_bc_full(double* a, long n1, long n2, long n3) {  // copy_bc_r!, copy_bc_θ!, copy_bc_z! in order
    Arr X = A(a, n1, n2, n3);
    for (long k = 1; k <= n3; ++k) for (long j = 1; j <= n2; ++j) { X(1, j, k) = X(2, j, k); X(n1, j, k) = X(n1 - 1, j, k); }
    for (long k = 1; k <= n3; ++k) for (long i = 1; i <= n1; ++i) { X(i, 1, k) = X(i, 2, k); X(i, n2, k) = X(i, n2 - 1, k); }
    for (long j = 1; j <= n2; ++j) for (long i = 1; i <= n1; ++i) { X(i, j, 1) = X(i, j, 2); X(i, j, n3) = X(i, j, n3 - 1); }
}

void copy_boundary_faces(double* a, long n1, long n2, long n3) {  // CartesianStokes_diapir.jl:97-105
    Arr X = A(a, n1, n2, n3);
    for (long k = 2; k <= n3 - 1; ++k) for (long j = 2; j <= n2 - 1; ++j) { X(1, j, k) = X(2, j, k); X(n1, j, k) = X(n1 - 1, j, k); }
    for (long k = 2; k <= n3 - 1; ++k) for (long i = 2; i <= n1 - 1; ++i) { X(i, 1, k) = X(i, 2, k); X(i, n2, k) = X(i, n2 - 1, k); }
    for (long j = 2; j <= n2 - 1; ++j) for (long i = 2; i <= n1 - 1; ++i) { X(i, j, 1) = X(i, j, 2); X(i, j, n3) = X(i, j, n3 - 1); }
}

void maxloc_inn(double* sm, const double* e, long n1, long n2, long n3) {
    Arr S = A(sm, n1, n2, n3), E = A(const_cast<double*>(e), n1, n2, n3);
    for (long k = 1; k <= n3 - 2; ++k)
        for (long j = 1; j <= n2 - 2; ++j)
            for (long i = 1; i <= n1 - 2; ++i) {
                long a = i + 1, b = j + 1, c = k + 1;
                S(a, b, c) = std::max(std::max(std::max(std::max(E(a - 1, b, c), E(a + 1, b, c)), E(a, b, c)), std::max(E(a, b - 1, c), E(a, b + 1, c))),
                                      std::max(E(a, b, c - 1), E(a, b, c + 1)));
            }
}

}  // namespace

extern "C" {

// state carried across PT iterations (the temporaries of the scripts are internal)
struct orc_cc_state {
    int64_t n1, n2, n3;
    double *P, *V1, *V2, *V3, *t11, *t22, *t33, *t12, *t13, *t23;
    double *rho, *eta, *eta_ini, *eta_pl, *etaSM, *DT_R, *tII;
    double *x1, *x2, *x3;  // 1D node coordinates (R_i, θ_i, Z_i / X_i, Y_i, Z_i)
};
struct orc_cc_params {
    double d1, d2, d3;     // spacings dr, dθ, dz (cyl) / dx, dy, dz (cart)
    double dmp, vpdt, lr, g, tau_C, n_exp, relax, r, sh;
};

// right-hand sides of the correction problem of the mixed-precision solve (EXT): rP in the
// pressure array's layout, rV1..rV3 in the velocity arrays' layouts
struct orc_cc_rhs {
    const double *rP, *rV1, *rV2, *rV3;
};

// ---------------------------------------------------------------------------
// CylindricalStokes_diapir.jl: one PT iteration (:331-366), n_exp given.
// rhs (EXT, may be NULL): a correction sweep instead — η and ηSM frozen (no
// maxloc!, no power law), P -= KBDT (DIVV + rP), rV added to the momentum rows in
// place of -ρg, the BCs in their homogeneous form (sh = 0).
static void cyl_iterate_impl(orc_cc_state* s, const orc_cc_params* qin, int64_t niter, const orc_cc_rhs* rhs) {
    orc_cc_params qh = *qin;
    if (rhs) { qh.sh = 0.0; qh.g = 0.0; }
    const orc_cc_params* q = &qh;
    const long nr = s->n1, nt = s->n2, nz = s->n3;
    const long nc = nr * nt * nz;
    std::vector<double> KBDT(nc), GSDT(nc), DIVV(nc), D_RR(nc), D_tt(nc), D_ZZ(nc), s_RR(nc), s_tt(nc), s_ZZ(nc), eta_pl_old(nc);
    std::vector<double> D_Rt((nr - 1) * (nt - 1) * (nz - 2)), D_RZ((nr - 1) * (nt - 2) * (nz - 1)), D_tZ((nr - 2) * (nt - 1) * (nz - 1));
    std::vector<double> dVR((nr - 1) * (nt - 2) * (nz - 2)), dVt((nr - 2) * (nt - 1) * (nz - 2)), dVZ((nr - 2) * (nt - 2) * (nz - 1));
    Arr P = A(s->P, nr, nt, nz), VR = A(s->V1, nr + 1, nt, nz), Vt = A(s->V2, nr, nt + 1, nz), VZ = A(s->V3, nr, nt, nz + 1);
    Arr tRR = A(s->t11, nr, nt, nz), ttt = A(s->t22, nr, nt, nz), tZZ = A(s->t33, nr, nt, nz);
    Arr tRt = A(s->t12, nr - 1, nt - 1, nz - 2), tRZ = A(s->t13, nr - 1, nt - 2, nz - 1), ttZ = A(s->t23, nr - 2, nt - 1, nz - 1);
    Arr eta = A(s->eta, nr, nt, nz), eta_INI = A(s->eta_ini, nr, nt, nz), eta_PL = A(s->eta_pl, nr, nt, nz), etaSM = A(s->etaSM, nr, nt, nz);
    Arr DT_R = A(s->DT_R, nr, nt, nz), tII = A(s->tII, nr, nt, nz), rho = A(s->rho, nr, nt, nz);
    Arr Kb = A(KBDT.data(), nr, nt, nz), Gs = A(GSDT.data(), nr, nt, nz), Dv = A(DIVV.data(), nr, nt, nz);
    Arr DRR = A(D_RR.data(), nr, nt, nz), Dtt = A(D_tt.data(), nr, nt, nz), DZZ = A(D_ZZ.data(), nr, nt, nz);
    Arr sRR = A(s_RR.data(), nr, nt, nz), stt = A(s_tt.data(), nr, nt, nz), sZZ = A(s_ZZ.data(), nr, nt, nz);
    Arr DRt = A(D_Rt.data(), nr - 1, nt - 1, nz - 2), DRZ = A(D_RZ.data(), nr - 1, nt - 2, nz - 1), DtZ = A(D_tZ.data(), nr - 2, nt - 1, nz - 1);
    Arr dR = A(dVR.data(), nr - 1, nt - 2, nz - 2), dt_ = A(dVt.data(), nr - 2, nt - 1, nz - 2), dZ = A(dVZ.data(), nr - 2, nt - 2, nz - 1);
    Arr PLO = A(eta_pl_old.data(), nr, nt, nz);
    Arr rV1 = A(rhs ? const_cast<double*>(rhs->rV1) : nullptr, nr + 1, nt, nz), rV2 = A(rhs ? const_cast<double*>(rhs->rV2) : nullptr, nr, nt + 1, nz),
        rV3 = A(rhs ? const_cast<double*>(rhs->rV3) : nullptr, nr, nt, nz + 1);
    const double dr = q->d1, dth = q->d2, dz = q->d3, dmp = q->dmp, vpdt = q->vpdt, lr = q->lr;
    auto R = [&](long i, long, long) { return s->x1[i - 1]; };
    for (long it = 0; it < niter; ++it) {
        // equal!(ηSM, η); maxloc!; copy_bc_r/θ/z!(ηSM)                         :331-335
        if (!rhs) {
            std::memcpy(s->etaSM, s->eta, sizeof(double) * nc);
            maxloc_inn(s->etaSM, s->eta, nr, nt, nz);
            copy_bc_full(s->etaSM, nr, nt, nz);
        }
        // timesteps!, timesteps2!                                                :336-337, :131-142
        for (long c = 0; c < nc; ++c) {
            KBDT[c] = dmp * 2.0 * PI * vpdt / lr * s->etaSM[c];
            GSDT[c] = 4.0 * PI * vpdt / lr * s->etaSM[c];
        }
        for (long c = 0; c < nc; ++c) s->DT_R[c] = vpdt * vpdt / (KBDT[c] + GSDT[c] / (1.0 + GSDT[c] / s->eta[c]));
        // compute_P!                                                             :145-168
        for (long k = 1; k <= nz + 1; ++k)
            for (long j = 1; j <= nt + 1; ++j)
                for (long i = 1; i <= nr + 1; ++i) {
                    if (i <= nr && j <= nt && k <= nz) {
                        double avxa = ((VR(i, j, k) + VR(i + 1, j, k)) * 0.5);
                        Dv(i, j, k) = (VR(i + 1, j, k) - VR(i, j, k)) / dr + 1 / R(i, j, k) * (Vt(i, j + 1, k) - Vt(i, j, k)) / dth + avxa / R(i, j, k) +
                                      (VZ(i, j, k + 1) - VZ(i, j, k)) / dz;
                        DRR(i, j, k) = (VR(i + 1, j, k) - VR(i, j, k)) / dr - 1.0 / 3.0 * Dv(i, j, k);
                        Dtt(i, j, k) = 1 / R(i, j, k) * (Vt(i, j + 1, k) - Vt(i, j, k)) / dth + avxa / R(i, j, k) - 1.0 / 3.0 * Dv(i, j, k);
                        DZZ(i, j, k) = (VZ(i, j, k + 1) - VZ(i, j, k)) / dz - 1.0 / 3.0 * Dv(i, j, k);
                    }
                    if (i <= nr - 1 && j <= nt - 1 && k <= nz - 2) {
                        double avR = ((R(i, j, k + 1) + R(i + 1, j, k + 1) + R(i, j + 1, k + 1) + R(i + 1, j + 1, k + 1)) * 0.25);
                        DRt(i, j, k) = (Vt(i + 1, j + 1, k + 1) - Vt(i, j + 1, k + 1)) / dr + 1 / avR * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j, k + 1)) / dth -
                                       ((Vt(i, j + 1, k + 1) + Vt(i + 1, j + 1, k + 1)) * 0.5) / avR;
                    }
                    if (i <= nr - 1 && j <= nt - 2 && k <= nz - 1)
                        DRZ(i, j, k) = (VZ(i + 1, j + 1, k + 1) - VZ(i, j + 1, k + 1)) / dr + (VR(i + 1, j + 1, k + 1) - VR(i + 1, j + 1, k)) / dz;
                    if (i <= nr - 2 && j <= nt - 1 && k <= nz - 1) {
                        double avR = ((R(i + 1, j, k) + R(i + 1, j + 1, k) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k + 1)) * 0.25);
                        DtZ(i, j, k) = 1 / avR * (VZ(i + 1, j + 1, k + 1) - VZ(i + 1, j, k + 1)) / dth + (Vt(i + 1, j + 1, k + 1) - Vt(i + 1, j + 1, k)) / dz;
                    }
                    if (i <= nr && j <= nt && k <= nz) {
                        const double dv = rhs ? Dv(i, j, k) + rhs->rP[(i - 1) + nr * ((j - 1) + nt * (k - 1))] : Dv(i, j, k);
                        P(i, j, k) = P(i, j, k) - Kb(i, j, k) * dv;
                        tRR(i, j, k) = (tRR(i, j, k) + Gs(i, j, k) * 2.0 * DRR(i, j, k)) / (1.0 + Gs(i, j, k) / eta(i, j, k));
                        ttt(i, j, k) = (ttt(i, j, k) + Gs(i, j, k) * 2.0 * Dtt(i, j, k)) / (1.0 + Gs(i, j, k) / eta(i, j, k));
                        tZZ(i, j, k) = (tZZ(i, j, k) + Gs(i, j, k) * 2.0 * DZZ(i, j, k)) / (1.0 + Gs(i, j, k) / eta(i, j, k));
                    }
                    if (i <= nr - 1 && j <= nt - 1 && k <= nz - 2) {
                        double aG = ((Gs(i, j, k + 1) + Gs(i + 1, j, k + 1) + Gs(i, j + 1, k + 1) + Gs(i + 1, j + 1, k + 1)) * 0.25);
                        double aE = ((eta(i, j, k + 1) + eta(i + 1, j, k + 1) + eta(i, j + 1, k + 1) + eta(i + 1, j + 1, k + 1)) * 0.25);
                        tRt(i, j, k) = (tRt(i, j, k) + aG * DRt(i, j, k)) / (1.0 + aG / aE);
                    }
                    if (i <= nr - 1 && j <= nt - 2 && k <= nz - 1) {
                        double aG = ((Gs(i, j + 1, k) + Gs(i + 1, j + 1, k) + Gs(i, j + 1, k + 1) + Gs(i + 1, j + 1, k + 1)) * 0.25);
                        double aE = ((eta(i, j + 1, k) + eta(i + 1, j + 1, k) + eta(i, j + 1, k + 1) + eta(i + 1, j + 1, k + 1)) * 0.25);
                        tRZ(i, j, k) = (tRZ(i, j, k) + aG * DRZ(i, j, k)) / (1.0 + aG / aE);
                    }
                    if (i <= nr - 2 && j <= nt - 1 && k <= nz - 1) {
                        double aG = ((Gs(i + 1, j, k) + Gs(i + 1, j + 1, k) + Gs(i + 1, j, k + 1) + Gs(i + 1, j + 1, k + 1)) * 0.25);
                        double aE = ((eta(i + 1, j, k) + eta(i + 1, j + 1, k) + eta(i + 1, j, k + 1) + eta(i + 1, j + 1, k + 1)) * 0.25);
                        ttZ(i, j, k) = (ttZ(i, j, k) + aG * DtZ(i, j, k)) / (1.0 + aG / aE);
                    }
                }
        // compute_sigma!                                                         :170-176
        for (long c = 0; c < nc; ++c) { s_RR[c] = -s->P[c] + s->t11[c]; s_tt[c] = -s->P[c] + s->t22[c]; s_ZZ[c] = -s->P[c] + s->t33[c]; }
        // power law block (n_exp > 1)                                            :345-352
        if (!rhs && q->n_exp > 1) {
            for (long k = 1; k <= nz - 2; ++k)
                for (long j = 1; j <= nt - 2; ++j)
                    for (long i = 1; i <= nr - 2; ++i)
                        tII(i + 1, j + 1, k + 1) = std::sqrt(1.0 / 2.0 * (sq(tRR(i + 1, j + 1, k + 1)) + sq(ttt(i + 1, j + 1, k + 1)) + sq(tZZ(i + 1, j + 1, k + 1))) +
                                                             sq((tRt(i, j, k) + tRt(i + 1, j, k) + tRt(i, j + 1, k) + tRt(i + 1, j + 1, k)) * 0.25) +
                                                             sq((tRZ(i, j, k) + tRZ(i + 1, j, k) + tRZ(i, j, k + 1) + tRZ(i + 1, j, k + 1)) * 0.25) +
                                                             sq((ttZ(i, j, k) + ttZ(i, j + 1, k) + ttZ(i, j, k + 1) + ttZ(i, j + 1, k + 1)) * 0.25));
            copy_bc_full(s->tII, nr, nt, nz);
            std::memcpy(eta_pl_old.data(), s->eta_pl, sizeof(double) * nc);
            for (long c = 0; c < nc; ++c) {
                s->eta_pl[c] = s->eta_ini[c] * std::pow(s->tII[c] / q->tau_C, 1.0 - q->n_exp);
                s->eta_pl[c] = std::exp(std::log(s->eta_pl[c]) * q->relax + std::log(eta_pl_old[c]) * (1.0 - q->relax));
                s->eta[c] = 2.0 / (1.0 / s->eta_ini[c] + 1.0 / s->eta_pl[c]);
            }
        }
        (void)PLO; (void)eta_PL; (void)eta_INI; (void)etaSM; (void)DT_R;
        // compute_dV!                                                            :194-206
        for (long k = 1; k <= nz - 1; ++k)
            for (long j = 1; j <= nt - 1; ++j)
                for (long i = 1; i <= nr - 1; ++i) {
                    if (j <= nt - 2 && k <= nz - 2) {
                        double aR = ((R(i, j + 1, k + 1) + R(i + 1, j + 1, k + 1)) * 0.5);
                        dR(i, j, k) = (sRR(i + 1, j + 1, k + 1) - sRR(i, j + 1, k + 1)) / dr + 1 / aR * (tRt(i, j + 1, k) - tRt(i, j, k)) / dth +
                                      (tRZ(i, j, k + 1) - tRZ(i, j, k)) / dz + ((sRR(i, j + 1, k + 1) + sRR(i + 1, j + 1, k + 1)) * 0.5) / aR -
                                      ((stt(i, j + 1, k + 1) + stt(i + 1, j + 1, k + 1)) * 0.5) / aR -
                                      ((rho(i, j + 1, k + 1) * q->g + rho(i + 1, j + 1, k + 1) * q->g) * 0.5);
                    }
                    if (i <= nr - 2 && k <= nz - 2) {
                        double aR = ((R(i + 1, j, k + 1) + R(i + 1, j + 1, k + 1)) * 0.5);
                        dt_(i, j, k) = (tRt(i + 1, j, k) - tRt(i, j, k)) / dr + 1 / aR * (stt(i + 1, j + 1, k + 1) - stt(i + 1, j, k + 1)) / dth +
                                       (ttZ(i, j, k + 1) - ttZ(i, j, k)) / dz + 2 * ((tRt(i, j, k) + tRt(i + 1, j, k)) * 0.5) / aR;
                    }
                    if (i <= nr - 2 && j <= nt - 2) {
                        double aR = ((R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.5);
                        dZ(i, j, k) = (tRZ(i + 1, j, k) - tRZ(i, j, k)) / dr + 1 / aR * (ttZ(i, j + 1, k) - ttZ(i, j, k)) / dth +
                                      (sZZ(i + 1, j + 1, k + 1) - sZZ(i + 1, j + 1, k)) / dz + ((tRZ(i, j, k) + tRZ(i + 1, j, k)) * 0.5) / aR;
                    }
                }
        // compute_V!                                                             :208-214
        for (long k = 1; k <= nz - 1; ++k)
            for (long j = 1; j <= nt - 1; ++j)
                for (long i = 1; i <= nr - 1; ++i) {
                    if (j <= nt - 2 && k <= nz - 2) {
                        double r = dR(i, j, k);
                        if (rhs) r += rV1(i + 1, j + 1, k + 1);
                        VR(i + 1, j + 1, k + 1) = VR(i + 1, j + 1, k + 1) + r * ((DT_R(i, j + 1, k + 1) + DT_R(i + 1, j + 1, k + 1)) * 0.5);
                    }
                    if (i <= nr - 2 && k <= nz - 2) {
                        double r = dt_(i, j, k);
                        if (rhs) r += rV2(i + 1, j + 1, k + 1);
                        Vt(i + 1, j + 1, k + 1) = Vt(i + 1, j + 1, k + 1) + r * ((DT_R(i + 1, j, k + 1) + DT_R(i + 1, j + 1, k + 1)) * 0.5);
                    }
                    if (i <= nr - 2 && j <= nt - 2) {
                        double r = dZ(i, j, k);
                        if (rhs) r += rV3(i + 1, j + 1, k + 1);
                        VZ(i + 1, j + 1, k + 1) = VZ(i + 1, j + 1, k + 1) + r * ((DT_R(i + 1, j + 1, k) + DT_R(i + 1, j + 1, k + 1)) * 0.5);
                    }
                }
        // boundary conditions                                                    :358-366
        const double r = q->r, sh = q->sh;
        for (long k = 1; k <= nz + 1; ++k) for (long j = 1; j <= nt; ++j) { VZ(1, j, k) = VZ(2, j, k); VZ(nr, j, k) = VZ(nr - 1, j, k); }     // copy_bc_r!(VZ)
        for (long k = 1; k <= nz; ++k) for (long j = 1; j <= nt + 1; ++j) { Vt(1, j, k) = Vt(2, j, k); Vt(nr, j, k) = Vt(nr - 1, j, k); }     // copy_bc_r!(Vθ)
        for (long k = 1; k <= nz; ++k) for (long j = 1; j <= nt; ++j) { VR(1, j, k) = -VR(2, j, k); VR(nr + 1, j, k) = -VR(nr, j, k); }       // bc_r_0!(VR)
        for (long k = 1; k <= nz + 1; ++k) for (long i = 1; i <= nr; ++i) { VZ(i, 1, k) = sh * s->x2[0] * r; VZ(i, nt, k) = sh * s->x2[nt - 1] * r; }  // bc_θ_fact!(VZ)
        for (long k = 1; k <= nz; ++k) for (long i = 1; i <= nr + 1; ++i) { VR(i, 1, k) = 0.0 * s->x2[0] * r; VR(i, nt, k) = 0.0 * s->x2[nt - 1] * r; } // bc_θ_fact!(VR, 0)
        for (long k = 1; k <= nz; ++k) for (long i = 1; i <= nr; ++i) { Vt(i, 1, k) = -Vt(i, 2, k); Vt(i, nt + 1, k) = -Vt(i, nt, k); }        // bc_θ_0!(Vθ)
        for (long j = 1; j <= nt + 1; ++j) for (long i = 1; i <= nr; ++i) { Vt(i, j, 1) = 0.0; Vt(i, j, nz) = 0.0; }                           // bc_z_0!(Vθ)
        for (long j = 1; j <= nt; ++j) for (long i = 1; i <= nr + 1; ++i) { VR(i, j, 1) = 0.0; VR(i, j, nz) = 0.0; }                           // bc_z_0!(VR)
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i) {                                                                                                  // bc_z_lin!(VZ)
                VZ(i, j, 1) = 2 * s->x2[j - 1] * r * sh - VZ(i, j, 2);
                VZ(i, j, nz + 1) = 2 * s->x2[j - 1] * r * sh - VZ(i, j, nz);
            }
    }
}

void orc_cyl_iterate(orc_cc_state* s, const orc_cc_params* q, int64_t niter) { cyl_iterate_impl(s, q, niter, nullptr); }

// ---------------------------------------------------------------------------
// CartesianStokes_diapir.jl: one PT iteration (:351-379); rhs as for the cylindrical script
static void cart_iterate_impl(orc_cc_state* s, const orc_cc_params* qin, int64_t niter, const orc_cc_rhs* rhs) {
    orc_cc_params qh = *qin;
    if (rhs) { qh.sh = 0.0; qh.g = 0.0; }
    const orc_cc_params* q = &qh;
    const long nx = s->n1, ny = s->n2, nz = s->n3;
    const long nc = nx * ny * nz;
    std::vector<double> eta_pl_old(nc);
    Arr P = A(s->P, nx, ny, nz), VX = A(s->V1, nx + 1, ny, nz), VY = A(s->V2, nx, ny + 1, nz), VZ = A(s->V3, nx, ny, nz + 1);
    Arr tXX = A(s->t11, nx, ny, nz), tYY = A(s->t22, nx, ny, nz), tZZ = A(s->t33, nx, ny, nz);
    Arr tXY = A(s->t12, nx - 1, ny - 1, nz - 2), tXZ = A(s->t13, nx - 1, ny - 2, nz - 1), tYZ = A(s->t23, nx - 2, ny - 1, nz - 1);
    Arr eta = A(s->eta, nx, ny, nz), etaSM = A(s->etaSM, nx, ny, nz), DT_R = A(s->DT_R, nx, ny, nz), tII = A(s->tII, nx, ny, nz), rho = A(s->rho, nx, ny, nz);
    const double _dx = 1.0 / q->d1, _dy = 1.0 / q->d2, _dz = 1.0 / q->d3, dmp = q->dmp, vpdt = q->vpdt, lx = q->lr, g = q->g;
    Arr rV1 = A(rhs ? const_cast<double*>(rhs->rV1) : nullptr, nx + 1, ny, nz), rV2 = A(rhs ? const_cast<double*>(rhs->rV2) : nullptr, nx, ny + 1, nz),
        rV3 = A(rhs ? const_cast<double*>(rhs->rV3) : nullptr, nx, ny, nz + 1);
    for (long it = 0; it < niter; ++it) {
        if (!rhs) {
            std::memcpy(s->etaSM, s->eta, sizeof(double) * nc);             // equal!(ηSM, η)
            maxloc_inn(s->etaSM, s->eta, nx, ny, nz);                       // maxloc!
            copy_boundary_faces(s->etaSM, nx, ny, nz);                      // copy_boundary!(ηSM)
        }
        auto KB = [&](long i, long j, long k) { return dmp * 2.0 * PI * vpdt / lx * etaSM(i, j, k); };
        auto GS = [&](long i, long j, long k) { return 4.0 * PI * vpdt / lx * etaSM(i, j, k); };
        for (long k = 1; k <= nz; ++k)                                      // timesteps!  :132-138
            for (long j = 1; j <= ny; ++j)
                for (long i = 1; i <= nx; ++i) DT_R(i, j, k) = vpdt * vpdt / (KB(i, j, k) + GS(i, j, k) / (1.0 + GS(i, j, k) / eta(i, j, k)));
        for (long k = 1; k <= nz; ++k)                                      // compute_P!  :165-193
            for (long j = 1; j <= ny; ++j)
                for (long i = 1; i <= nx; ++i) {
                    double Dxx = (VX(i + 1, j, k) - VX(i, j, k)) * _dx, Dyy = (VY(i, j + 1, k) - VY(i, j, k)) * _dy, Dzz = (VZ(i, j, k + 1) - VZ(i, j, k)) * _dz;
                    const double dv = rhs ? (Dxx + Dyy + Dzz) + rhs->rP[(i - 1) + nx * ((j - 1) + ny * (k - 1))] : (Dxx + Dyy + Dzz);
                    P(i, j, k) = P(i, j, k) - KB(i, j, k) * dv;
                    tXX(i, j, k) = (tXX(i, j, k) + GS(i, j, k) * 2.0 * Dxx) / (1.0 + GS(i, j, k) / eta(i, j, k));
                    tYY(i, j, k) = (tYY(i, j, k) + GS(i, j, k) * 2.0 * Dyy) / (1.0 + GS(i, j, k) / eta(i, j, k));
                    tZZ(i, j, k) = (tZZ(i, j, k) + GS(i, j, k) * 2.0 * Dzz) / (1.0 + GS(i, j, k) / eta(i, j, k));
                    if (i <= nx - 1 && j <= ny - 1 && k <= nz - 2) {
                        double aS = 0.25 * (etaSM(i, j, k + 1) + etaSM(i, j + 1, k + 1) + etaSM(i + 1, j, k + 1) + etaSM(i + 1, j + 1, k + 1));
                        double aE = 0.25 * (eta(i, j, k + 1) + eta(i, j + 1, k + 1) + eta(i + 1, j, k + 1) + eta(i + 1, j + 1, k + 1));
                        double aG = 4.0 * PI * vpdt / lx * aS;
                        double D = (VX(i + 1, j + 1, k + 1) - VX(i + 1, j, k + 1)) * _dy + (VY(i + 1, j + 1, k + 1) - VY(i, j + 1, k + 1)) * _dx;
                        tXY(i, j, k) = (tXY(i, j, k) + aG * D) / (1.0 + aG / aE);
                    }
                    if (i <= nx - 1 && j <= ny - 2 && k <= nz - 1) {
                        double aS = 0.25 * (etaSM(i, j + 1, k) + etaSM(i, j + 1, k + 1) + etaSM(i + 1, j + 1, k) + etaSM(i + 1, j + 1, k + 1));
                        double aE = 0.25 * (eta(i, j + 1, k) + eta(i, j + 1, k + 1) + eta(i + 1, j + 1, k) + eta(i + 1, j + 1, k + 1));
                        double aG = 4.0 * PI * vpdt / lx * aS;
                        double D = (VX(i + 1, j + 1, k + 1) - VX(i + 1, j + 1, k)) * _dz + (VZ(i + 1, j + 1, k + 1) - VZ(i, j + 1, k + 1)) * _dx;
                        tXZ(i, j, k) = (tXZ(i, j, k) + aG * D) / (1.0 + aG / aE);
                    }
                    if (i <= nx - 2 && j <= ny - 1 && k <= nz - 1) {
                        double aS = 0.25 * (etaSM(i + 1, j, k) + etaSM(i + 1, j, k + 1) + etaSM(i + 1, j + 1, k) + etaSM(i + 1, j + 1, k + 1));
                        double aE = 0.25 * (eta(i + 1, j, k) + eta(i + 1, j, k + 1) + eta(i + 1, j + 1, k) + eta(i + 1, j + 1, k + 1));
                        double aG = 4.0 * PI * vpdt / lx * aS;
                        double D = (VY(i + 1, j + 1, k + 1) - VY(i + 1, j + 1, k)) * _dz + (VZ(i + 1, j + 1, k + 1) - VZ(i + 1, j, k + 1)) * _dy;
                        tYZ(i, j, k) = (tYZ(i, j, k) + aG * D) / (1.0 + aG / aE);
                    }
                }
        if (!rhs && q->n_exp > 1) {                                         // :358-363
            for (long k = 1; k <= nz - 2; ++k)
                for (long j = 1; j <= ny - 2; ++j)
                    for (long i = 1; i <= nx - 2; ++i)
                        tII(i + 1, j + 1, k + 1) = std::sqrt(1.0 / 2.0 * (sq(tXX(i + 1, j + 1, k + 1)) + sq(tYY(i + 1, j + 1, k + 1)) + sq(tZZ(i + 1, j + 1, k + 1))) +
                                                             sq(0.25 * (tXY(i, j, k) + tXY(i, j + 1, k) + tXY(i + 1, j, k) + tXY(i + 1, j + 1, k))) +
                                                             sq(0.25 * (tXZ(i, j, k) + tXZ(i, j, k + 1) + tXZ(i + 1, j, k) + tXZ(i + 1, j, k + 1))) +
                                                             sq(0.25 * (tYZ(i, j, k) + tYZ(i, j, k + 1) + tYZ(i, j + 1, k) + tYZ(i, j + 1, k + 1))));
            copy_boundary_faces(s->tII, nx, ny, nz);
            std::memcpy(eta_pl_old.data(), s->eta_pl, sizeof(double) * nc);
            for (long c = 0; c < nc; ++c) {
                s->eta_pl[c] = s->eta_ini[c] * std::pow(s->tII[c] / q->tau_C, 1.0 - q->n_exp);
                s->eta_pl[c] = std::exp(std::log(s->eta_pl[c]) * q->relax + std::log(eta_pl_old[c]) * (1.0 - q->relax));
                s->eta[c] = 2.0 / (1.0 / s->eta_ini[c] + 1.0 / s->eta_pl[c]);
            }
        }
        for (long k = 1; k <= nz - 1; ++k)                                  // compute_V!  :223-254
            for (long j = 1; j <= ny - 1; ++j)
                for (long i = 1; i <= nx - 1; ++i) {
                    if (j <= ny - 2 && k <= nz - 2) {
                        double dV = -(P(i + 1, j + 1, k + 1) - P(i, j + 1, k + 1)) * _dx + (tXX(i + 1, j + 1, k + 1) - tXX(i, j + 1, k + 1)) * _dx +
                                    (tXY(i, j + 1, k) - tXY(i, j, k)) * _dy + (tXZ(i, j, k + 1) - tXZ(i, j, k)) * _dz;
                        if (rhs) dV += rV1(i + 1, j + 1, k + 1);
                        VX(i + 1, j + 1, k + 1) = VX(i + 1, j + 1, k + 1) + dV * 0.5 * (DT_R(i, j + 1, k + 1) + DT_R(i + 1, j + 1, k + 1));
                    }
                    if (i <= nx - 2 && k <= nz - 2) {
                        double dV = (tXY(i + 1, j, k) - tXY(i, j, k)) * _dx - (P(i + 1, j + 1, k + 1) - P(i + 1, j, k + 1)) * _dy +
                                    (tYY(i + 1, j + 1, k + 1) - tYY(i + 1, j, k + 1)) * _dy + (tYZ(i, j, k + 1) - tYZ(i, j, k)) * _dz;
                        if (rhs) dV += rV2(i + 1, j + 1, k + 1);
                        VY(i + 1, j + 1, k + 1) = VY(i + 1, j + 1, k + 1) + dV * 0.5 * (DT_R(i + 1, j, k + 1) + DT_R(i + 1, j + 1, k + 1));
                    }
                    if (i <= nx - 2 && j <= ny - 2) {
                        double dV = (tXZ(i + 1, j, k) - tXZ(i, j, k)) * _dx + (tYZ(i, j + 1, k) - tYZ(i, j, k)) * _dy -
                                    (P(i + 1, j + 1, k + 1) - P(i + 1, j + 1, k)) * _dz + (tZZ(i + 1, j + 1, k + 1) - tZZ(i + 1, j + 1, k)) * _dz -
                                    g * (0.5 * (rho(i + 1, j + 1, k) + rho(i + 1, j + 1, k + 1)));
                        if (rhs) dV += rV3(i + 1, j + 1, k + 1);
                        VZ(i + 1, j + 1, k + 1) = VZ(i + 1, j + 1, k + 1) + dV * 0.5 * (DT_R(i + 1, j + 1, k) + DT_R(i + 1, j + 1, k + 1));
                    }
                }
        const double sh = q->sh;                                            // BCs :371-379
        for (long k = 1; k <= nz; ++k)
            for (long j = 1; j <= ny; ++j) {                                // bc_x_lin!(VX, Y_VX, sh)
                VX(1, j, k) = 2 * s->x2[j - 1] * sh - VX(2, j, k);
                VX(nx + 1, j, k) = 2 * s->x2[j - 1] * sh - VX(nx, j, k);
            }
        for (long k = 1; k <= nz; ++k) for (long j = 1; j <= ny + 1; ++j) { VY(1, j, k) = 0.0; VY(nx, j, k) = 0.0; }          // bc_x_0!(VY)
        for (long k = 1; k <= nz + 1; ++k) for (long j = 1; j <= ny; ++j) { VZ(1, j, k) = 0.0; VZ(nx, j, k) = 0.0; }          // bc_x_0!(VZ)
        for (long k = 1; k <= nz; ++k) for (long i = 1; i <= nx + 1; ++i) { VX(i, 1, k) = sh * s->x2[0]; VX(i, ny, k) = sh * s->x2[ny - 1]; }  // bc_y_fact!(VX)
        for (long k = 1; k <= nz; ++k) for (long i = 1; i <= nx; ++i) { VY(i, 1, k) = -VY(i, 2, k); VY(i, ny + 1, k) = -VY(i, ny, k); }       // bc_y_0!(VY)
        for (long k = 1; k <= nz + 1; ++k) for (long i = 1; i <= nx; ++i) { VZ(i, 1, k) = 0.0 * s->x2[0]; VZ(i, ny, k) = 0.0 * s->x2[ny - 1]; } // bc_y_fact!(VZ, 0)
        for (long j = 1; j <= ny; ++j) for (long i = 1; i <= nx + 1; ++i) { VX(i, j, 1) = VX(i, j, 2); VX(i, j, nz) = VX(i, j, nz - 1); }     // copy_bc_z!(VX)
        for (long j = 1; j <= ny + 1; ++j) for (long i = 1; i <= nx; ++i) { VY(i, j, 1) = VY(i, j, 2); VY(i, j, nz) = VY(i, j, nz - 1); }     // copy_bc_z!(VY)
        for (long j = 1; j <= ny; ++j) for (long i = 1; i <= nx; ++i) { VZ(i, j, 1) = -VZ(i, j, 2); VZ(i, j, nz + 1) = -VZ(i, j, nz); }       // bc_z_0!(VZ)
    }
}

void orc_cart_iterate(orc_cc_state* s, const orc_cc_params* q, int64_t niter) { cart_iterate_impl(s, q, niter, nullptr); }

// EXT: nsweeps correction sweeps of the mixed-precision solve (geometry 1 cylindrical, 2 Cartesian);
// s holds the correction state, η and ηSM frozen
void orc_cc_corr_sweep(int32_t geometry, orc_cc_state* s, const orc_cc_params* q, const double* rP, const double* rV1,
                       const double* rV2, const double* rV3, int64_t nsweeps) {
    const orc_cc_rhs rhs{rP, rV1, rV2, rV3};
    if (geometry == 1) cyl_iterate_impl(s, q, nsweeps, &rhs);
    else cart_iterate_impl(s, q, nsweeps, &rhs);
}

}  // extern "C"
