// ORACLE — test infrastructure only.
//
// CPU FP64 restatement of the pseudo-transient (PT) Stokes kernels of
// PTsolvers/SphericalStokes (Julia + ParallelStencil).  Only tests/, the
// smoke check and bench.py's cpu_baseline / reference arm load this file;
// the product library never links or calls it.
//
// Indexing follows the reference exactly: 1-based (ix,iy,iz), column-major
// arrays with ix fastest, every array with the size the scripts allocate.
// Each function names the reference kernel (file:line) it restates.  Kernels
// write only their own point, so sequential loops reproduce the GPU
// semantics; the boundary-condition kernels are applied in the scripts' call
// order.  Loops are OpenMP-parallel over iz (the oracle doubles as the CPU
// baseline timed on the host cores).
//
// Parity pin: the reference has no tests or golden vectors and Julia is not
// available here, so this restatement is pinned against golden vectors that
// tests/golden/make_golden.py generates by mechanically transliterating the
// reference's own kernel source (macros expanded, launch ranges inferred as
// ParallelStencil does) — an executable check independent of this file.
//
// Extensions not in the reference (strain-rate power law with relaxation,
// far-field normal-stress boundary condition, FP64 Stokes residual) are marked
// EXT; for those this file IS the specification the CUDA path must match.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

#if defined(_OPENMP)
#include <omp.h>
#endif

namespace {

const double PI = 3.141592653589793;  // Float64(π) in Julia

struct Arr {
    double* p;
    long n1, n2, n3;
    inline double& operator()(long i, long j, long k) const {
        return p[(i - 1) + n1 * ((j - 1) + n2 * (k - 1))];
    }
};

inline double cot(double x) { return 1.0 / std::tan(x); }  // Base.cot = inv(tan(x))
// max of |x| that propagates NaN (a norm of a diverged state must not read 0)
inline double nmax(double m, double x) { x = std::fabs(x); return (x != x || m != m) ? NAN : (x > m ? x : m); }
inline double sq(double x) { return x * x; }

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Spherical state: every array the diapir/plateau scripts allocate
// (SphericalStokes_diapir.jl:381-399), plus the full 3D coordinate arrays
// (:374-378).  nr, nt, np are the cell counts (P is nr x nt x np).
// ---------------------------------------------------------------------------
struct orc_sph_state {
    int64_t nr, nt, np;
    double *P, *VR, *Vt, *Vp, *VR_err, *Vt_err, *Vp_err;
    double *tRR, *ttt, *tpp, *tRt, *tRp, *ttp;
    double *rho, *eta, *eta_ini, *etaSM, *DT_R, *tII;
    double *R, *th, *ph;
    uint8_t* phase;      // EXT: 1 = linear cell (n = 1); may be NULL (all power law)
    double* eta_tmp;     // EXT: scratch for the strain-rate law (nr x nt x np); may be NULL
};

struct orc_sph_params {
    double _dr, _dt, _dp;  // inverse spacings (SphericalStokes_diapir.jl:370)
    double dmp, vpdt, lr;  // PT numerics (:10, :400, :358)
    double g, tau_C, n_exp, r, sh;
    int32_t bc;            // 0 diapir simple shear (:61-99), 1 free slip (SphericalStokes_plateau.jl:64-92), 2 EXT stress
    int32_t rheo;          // 0 stress power law (:259-265), 1 EXT strain-rate power law, 2 linear (skip)
    double relax, edot_bg; // EXT
    double sig_t, sig_p;   // EXT far-field normal stresses on the theta / phi faces
    int32_t passes;        // EXT applications of the 7-point max filter giving ηSM (reference: 1)
    int32_t pad_;
    double fs_kappa;          // EXT bc 3: stabilisation coefficient of the free surface (θ Δt Δρ g)
    const double* top_load;   // EXT bc 3: surface load q per top cell (cell layout, top layer read; NULL: 0)
};

static inline Arr A(double* p, long n1, long n2, long n3) { return Arr{p, n1, n2, n3}; }

// equal3!  SphericalStokes_diapir.jl:46-58
void orc_sph_equal3(orc_sph_state* s) {
    long nr = s->nr, nt = s->nt, np = s->np;
    std::memcpy(s->VR_err, s->VR, sizeof(double) * (nr + 1) * nt * np);
    std::memcpy(s->Vt_err, s->Vt, sizeof(double) * nr * (nt + 1) * np);
    std::memcpy(s->Vp_err, s->Vp, sizeof(double) * nr * nt * (np + 1));
}

// copy_bc_r! / copy_bc_θ! / copy_bc_φ! / copy_BC!  SphericalStokes_diapir.jl:102-124
void orc_copy_BC(double* a, int64_t n1, int64_t n2, int64_t n3) {
    Arr X = A(a, n1, n2, n3);
    for (long k = 1; k <= n3; ++k)
        for (long j = 1; j <= n2; ++j) { X(1, j, k) = X(2, j, k); X(n1, j, k) = X(n1 - 1, j, k); }
    for (long k = 1; k <= n3; ++k)
        for (long i = 1; i <= n1; ++i) { X(i, 1, k) = X(i, 2, k); X(i, n2, k) = X(i, n2 - 1, k); }
    for (long j = 1; j <= n2; ++j)
        for (long i = 1; i <= n1; ++i) { X(i, j, 1) = X(i, j, 2); X(i, j, n3) = X(i, j, n3 - 1); }
}

// copy_boundary!  CartesianStokes_diapir.jl:97-105 (faces only; edges and
// corners keep their previous values)
void orc_copy_boundary_faces(double* a, int64_t n1, int64_t n2, int64_t n3) {
    Arr X = A(a, n1, n2, n3);
    for (long k = 2; k <= n3 - 1; ++k)
        for (long j = 2; j <= n2 - 1; ++j) { X(1, j, k) = X(2, j, k); X(n1, j, k) = X(n1 - 1, j, k); }
    for (long k = 2; k <= n3 - 1; ++k)
        for (long i = 2; i <= n1 - 1; ++i) { X(i, 1, k) = X(i, 2, k); X(i, n2, k) = X(i, n2 - 1, k); }
    for (long j = 2; j <= n2 - 1; ++j)
        for (long i = 2; i <= n1 - 1; ++i) { X(i, j, 1) = X(i, j, 2); X(i, j, n3) = X(i, j, n3 - 1); }
}

// maxloc!  @inn(ηSM) = @maxloc(η)  SphericalStokes_diapir.jl:149-152
// (explicit form of @maxloc: SphericalStokes_mxpu.jl:295-297)
void orc_maxloc(double* etaSM, const double* eta, int64_t n1, int64_t n2, int64_t n3) {
    Arr S = A(etaSM, n1, n2, n3);
    Arr E = A(const_cast<double*>(eta), n1, n2, n3);
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= n3 - 2; ++k)
        for (long j = 1; j <= n2 - 2; ++j)
            for (long i = 1; i <= n1 - 2; ++i) {
                long a = i + 1, b = j + 1, c = k + 1;
                S(a, b, c) = std::max(std::max(std::max(std::max(E(a - 1, b, c), E(a + 1, b, c)), E(a, b, c)),
                                               std::max(E(a, b - 1, c), E(a, b + 1, c))),
                                      std::max(E(a, b, c - 1), E(a, b, c + 1)));
            }
}

// initialize_inclusion!  SphericalStokes_diapir.jl:127-137 (squared distance
// compared with `radius`, as in the reference)
void orc_sph_init_inclusion(double* a, const double* R, const double* th, const double* ph,
                            int64_t nr, int64_t nt, int64_t np, double r, double radius, double in) {
    long n = nr * nt * np;
    for (long q = 0; q < n; ++q)
        if ((sq(R[q] - r) + sq((th[q] - PI / 2.0) * r) + sq(ph[q] * r)) < radius) a[q] = in;
}

// initialize_velocity!  SphericalStokes_diapir.jl:139-146
void orc_sph_init_velocity(double* Vp, const double* th, int64_t nr, int64_t nt, int64_t np, double fact, double r) {
    Arr V = A(Vp, nr, nt, np + 1);
    Arr T = A(const_cast<double*>(th), nr, nt, np);
    for (long k = 1; k <= np + 1; ++k)
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i)
                V(i, j, k) = (k <= np) ? (T(i, j, k) - PI / 2.0) * r * fact : (T(i, j, k - 1) - PI / 2.0) * r * fact;
}

// compute_P!  SphericalStokes_diapir.jl:155-241 (macros :155-208).  rP (EXT, may be NULL):
// right-hand side of the continuity row of the correction problem, P -= KBDT (DIVV + rP);
// the deviatoric strain rates use DIVV alone.
static void sph_compute_P_impl(orc_sph_state* s, const orc_sph_params* q, const double* rP) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr P = A(s->P, nr, nt, np), DT_R = A(s->DT_R, nr, nt, np);
    Arr tRR = A(s->tRR, nr, nt, np), ttt = A(s->ttt, nr, nt, np), tpp = A(s->tpp, nr, nt, np);
    Arr tRt = A(s->tRt, nr - 1, nt - 1, np - 2), tRp = A(s->tRp, nr - 1, nt - 2, np - 1), ttp = A(s->ttp, nr - 2, nt - 1, np - 1);
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np), eta = A(s->eta, nr, nt, np), etaSM = A(s->etaSM, nr, nt, np);
    const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp, dmp = q->dmp, vpdt = q->vpdt, lr = q->lr;
    auto KBDT = [&](long i, long j, long k) { return dmp * 2.0 * PI * vpdt / lr * etaSM(i, j, k); };
    auto GSDT = [&](long i, long j, long k) { return 4.0 * PI * vpdt / lr * etaSM(i, j, k); };
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= np; ++k)
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i) {
                double avxa_VR = ((VR(i, j, k) + VR(i + 1, j, k)) * 0.5);
                double avya_Vt = ((Vt(i, j, k) + Vt(i, j + 1, k)) * 0.5);
                double Rc = R(i, j, k), tc = th(i, j, k);
                double DIVV = (VR(i + 1, j, k) - VR(i, j, k)) * _dr + 1.0 / Rc * (Vt(i, j + 1, k) - Vt(i, j, k)) * _dt +
                              1.0 / Rc / std::sin(tc) * (Vp(i, j, k + 1) - Vp(i, j, k)) * _dp + 2.0 * avxa_VR / Rc +
                              avya_Vt / Rc * cot(tc);
                double DRR = (VR(i + 1, j, k) - VR(i, j, k)) * _dr - 1.0 / 3.0 * DIVV;
                double Dtt = 1.0 / Rc * (Vt(i, j + 1, k) - Vt(i, j, k)) * _dt + avxa_VR / Rc - 1.0 / 3.0 * DIVV;
                double Dpp = 1.0 / Rc / std::sin(tc) * (Vp(i, j, k + 1) - Vp(i, j, k)) * _dp + avxa_VR / Rc +
                             avya_Vt / Rc * cot(tc) - 1.0 / 3.0 * DIVV;
                double kb = KBDT(i, j, k), gs = GSDT(i, j, k), e = eta(i, j, k);
                const double dv = rP ? DIVV + rP[(i - 1) + nr * ((j - 1) + nt * (k - 1))] : DIVV;
                P(i, j, k) = P(i, j, k) - kb * dv;
                tRR(i, j, k) = (tRR(i, j, k) + gs * 2.0 * DRR) / (1.0 + gs / e);
                ttt(i, j, k) = (ttt(i, j, k) + gs * 2.0 * Dtt) / (1.0 + gs / e);
                tpp(i, j, k) = (tpp(i, j, k) + gs * 2.0 * Dpp) / (1.0 + gs / e);
                DT_R(i, j, k) = vpdt * vpdt / (kb + gs / (1.0 + gs / e));
                if (i <= nr - 1 && j <= nt - 1 && k <= np - 2) {
                    double aR = ((R(i, j, k + 1) + R(i, j + 1, k + 1) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k + 1)) * 0.25);
                    double avxi_Vt = ((Vt(i, j + 1, k + 1) + Vt(i + 1, j + 1, k + 1)) * 0.5);
                    double D = (Vt(i + 1, j + 1, k + 1) - Vt(i, j + 1, k + 1)) * _dr +
                               1.0 / aR * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j, k + 1)) * _dt - avxi_Vt / aR;
                    double aG = ((GSDT(i, j, k + 1) + GSDT(i, j + 1, k + 1) + GSDT(i + 1, j, k + 1) + GSDT(i + 1, j + 1, k + 1)) * 0.25);
                    double aE = ((eta(i, j, k + 1) + eta(i, j + 1, k + 1) + eta(i + 1, j, k + 1) + eta(i + 1, j + 1, k + 1)) * 0.25);
                    tRt(i, j, k) = (tRt(i, j, k) + aG * D) / (1.0 + aG / aE);
                }
                if (i <= nr - 1 && j <= nt - 2 && k <= np - 1) {
                    double aR = ((R(i, j + 1, k) + R(i, j + 1, k + 1) + R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.25);
                    double aT = ((th(i, j + 1, k) + th(i, j + 1, k + 1) + th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.25);
                    double avxi_Vp = ((Vp(i, j + 1, k + 1) + Vp(i + 1, j + 1, k + 1)) * 0.5);
                    double D = (Vp(i + 1, j + 1, k + 1) - Vp(i, j + 1, k + 1)) * _dr +
                               1.0 / aR / std::sin(aT) * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j + 1, k)) * _dp - avxi_Vp / aR;
                    double aG = ((GSDT(i, j + 1, k) + GSDT(i, j + 1, k + 1) + GSDT(i + 1, j + 1, k) + GSDT(i + 1, j + 1, k + 1)) * 0.25);
                    double aE = ((eta(i, j + 1, k) + eta(i, j + 1, k + 1) + eta(i + 1, j + 1, k) + eta(i + 1, j + 1, k + 1)) * 0.25);
                    tRp(i, j, k) = (tRp(i, j, k) + aG * D) / (1.0 + aG / aE);
                }
                if (i <= nr - 2 && j <= nt - 1 && k <= np - 1) {
                    double aR = ((R(i + 1, j, k) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.25);
                    double aT = ((th(i + 1, j, k) + th(i + 1, j, k + 1) + th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.25);
                    double avyi_Vp = ((Vp(i + 1, j, k + 1) + Vp(i + 1, j + 1, k + 1)) * 0.5);
                    double D = 1.0 / aR * (Vp(i + 1, j + 1, k + 1) - Vp(i + 1, j, k + 1)) * _dt +
                               1.0 / aR / std::sin(aT) * (Vt(i + 1, j + 1, k + 1) - Vt(i + 1, j + 1, k)) * _dp -
                               avyi_Vp / aR * cot(aT);
                    double aG = ((GSDT(i + 1, j, k) + GSDT(i + 1, j, k + 1) + GSDT(i + 1, j + 1, k) + GSDT(i + 1, j + 1, k + 1)) * 0.25);
                    double aE = ((eta(i + 1, j, k) + eta(i + 1, j, k + 1) + eta(i + 1, j + 1, k) + eta(i + 1, j + 1, k + 1)) * 0.25);
                    ttp(i, j, k) = (ttp(i, j, k) + aG * D) / (1.0 + aG / aE);
                }
            }
}

void orc_sph_compute_P(orc_sph_state* s, const orc_sph_params* q) { sph_compute_P_impl(s, q, nullptr); }

// compute_TII!  SphericalStokes_diapir.jl:243-257 (interior only; faces via copy_BC!)
void orc_sph_compute_TII(orc_sph_state* s) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr tII = A(s->tII, nr, nt, np), tRR = A(s->tRR, nr, nt, np), ttt = A(s->ttt, nr, nt, np), tpp = A(s->tpp, nr, nt, np);
    Arr tRt = A(s->tRt, nr - 1, nt - 1, np - 2), tRp = A(s->tRp, nr - 1, nt - 2, np - 1), ttp = A(s->ttp, nr - 2, nt - 1, np - 1);
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= np - 2; ++k)
        for (long j = 1; j <= nt - 2; ++j)
            for (long i = 1; i <= nr - 2; ++i)
                tII(i + 1, j + 1, k + 1) =
                    std::sqrt(1.0 / 2.0 * (sq(tRR(i + 1, j + 1, k + 1)) + sq(ttt(i + 1, j + 1, k + 1)) + sq(tpp(i + 1, j + 1, k + 1))) +
                              sq((tRt(i, j, k) + tRt(i, j + 1, k) + tRt(i + 1, j, k) + tRt(i + 1, j + 1, k)) * 0.25) +
                              sq((tRp(i, j, k) + tRp(i, j, k + 1) + tRp(i + 1, j, k) + tRp(i + 1, j, k + 1)) * 0.25) +
                              sq((ttp(i, j, k) + ttp(i, j, k + 1) + ttp(i, j + 1, k) + ttp(i, j + 1, k + 1)) * 0.25));
}

// power_law!  SphericalStokes_diapir.jl:259-265 (EXT: phase==1 cells are linear)
void orc_sph_power_law(orc_sph_state* s, const orc_sph_params* q) {
    long n = s->nr * s->nt * s->np;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < n; ++c) {
        double ne = (s->phase && s->phase[c]) ? 1.0 : q->n_exp;
        s->eta[c] = 2.0 / (1.0 / s->eta_ini[c] + 1.0 / (s->eta_ini[c] * std::pow(s->tII[c] / q->tau_C, 1.0 - ne)));
    }
}

// compute_V!  SphericalStokes_diapir.jl:267-329 (macros :267-307).  rV (EXT, may be NULL):
// right-hand sides of the momentum rows of the correction problem (velocity-array
// layouts), added to dV; the caller passes g = 0 with them.
static void sph_compute_V_impl(orc_sph_state* s, const orc_sph_params* q, const double* const* rV) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr P = A(s->P, nr, nt, np), DT_R = A(s->DT_R, nr, nt, np), rho = A(s->rho, nr, nt, np);
    Arr tRR = A(s->tRR, nr, nt, np), ttt = A(s->ttt, nr, nt, np), tpp = A(s->tpp, nr, nt, np);
    Arr tRt = A(s->tRt, nr - 1, nt - 1, np - 2), tRp = A(s->tRp, nr - 1, nt - 2, np - 1), ttp = A(s->ttp, nr - 2, nt - 1, np - 1);
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np);
    const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp, g = q->g;
    auto sRR = [&](long i, long j, long k) { return -P(i, j, k) + tRR(i, j, k); };
    auto stt = [&](long i, long j, long k) { return -P(i, j, k) + ttt(i, j, k); };
    auto spp = [&](long i, long j, long k) { return -P(i, j, k) + tpp(i, j, k); };
    auto rG = [&](long i, long j, long k) { return rho(i, j, k) * g; };
    Arr rV1 = A(rV ? const_cast<double*>(rV[0]) : nullptr, nr + 1, nt, np), rV2 = A(rV ? const_cast<double*>(rV[1]) : nullptr, nr, nt + 1, np),
        rV3 = A(rV ? const_cast<double*>(rV[2]) : nullptr, nr, nt, np + 1);
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= np - 1; ++k)
        for (long j = 1; j <= nt - 1; ++j)
            for (long i = 1; i <= nr - 1; ++i) {
                if (i <= nr + 1 - 2 && j <= nt - 2 && k <= np - 2) {
                    double aR = ((R(i, j + 1, k + 1) + R(i + 1, j + 1, k + 1)) * 0.5);
                    double aT = ((th(i, j + 1, k + 1) + th(i + 1, j + 1, k + 1)) * 0.5);
                    double dV = (sRR(i + 1, j + 1, k + 1) - sRR(i, j + 1, k + 1)) * _dr +
                                1.0 / aR * (tRt(i, j + 1, k) - tRt(i, j, k)) * _dt +
                                1.0 / aR / std::sin(aT) * (tRp(i, j, k + 1) - tRp(i, j, k)) * _dp +
                                2.0 * ((sRR(i, j + 1, k + 1) + sRR(i + 1, j + 1, k + 1)) * 0.5) / aR -
                                (((stt(i, j + 1, k + 1) + stt(i + 1, j + 1, k + 1)) * 0.5) + ((spp(i, j + 1, k + 1) + spp(i + 1, j + 1, k + 1)) * 0.5)) / aR +
                                ((tRt(i, j, k) + tRt(i, j + 1, k)) * 0.5) / aR * cot(aT) -
                                ((rG(i, j + 1, k + 1) + rG(i + 1, j + 1, k + 1)) * 0.5);
                    if (rV) dV += rV1(i + 1, j + 1, k + 1);
                    VR(i + 1, j + 1, k + 1) = VR(i + 1, j + 1, k + 1) + dV * ((DT_R(i, j + 1, k + 1) + DT_R(i + 1, j + 1, k + 1)) * 0.5);
                }
                if (i <= nr - 2 && j <= nt + 1 - 2 && k <= np - 2) {
                    double aR = ((R(i + 1, j, k + 1) + R(i + 1, j + 1, k + 1)) * 0.5);
                    double aT = ((th(i + 1, j, k + 1) + th(i + 1, j + 1, k + 1)) * 0.5);
                    double dV = (tRt(i + 1, j, k) - tRt(i, j, k)) * _dr +
                                1.0 / aR * (stt(i + 1, j + 1, k + 1) - stt(i + 1, j, k + 1)) * _dt +
                                1.0 / aR / std::sin(aT) * (ttp(i, j, k + 1) - ttp(i, j, k)) * _dp +
                                3.0 * ((tRt(i, j, k) + tRt(i + 1, j, k)) * 0.5) / aR +
                                (((stt(i + 1, j, k + 1) + stt(i + 1, j + 1, k + 1)) * 0.5) - ((spp(i + 1, j, k + 1) + spp(i + 1, j + 1, k + 1)) * 0.5)) / aR * cot(aT);
                    if (rV) dV += rV2(i + 1, j + 1, k + 1);
                    Vt(i + 1, j + 1, k + 1) = Vt(i + 1, j + 1, k + 1) + dV * ((DT_R(i + 1, j, k + 1) + DT_R(i + 1, j + 1, k + 1)) * 0.5);
                }
                if (i <= nr - 2 && j <= nt - 2 && k <= np + 1 - 2) {
                    double aR = ((R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.5);
                    double aT = ((th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.5);
                    double dV = (tRp(i + 1, j, k) - tRp(i, j, k)) * _dr +
                                1.0 / aR * (ttp(i, j + 1, k) - ttp(i, j, k)) * _dt +
                                1.0 / aR / std::sin(aT) * (spp(i + 1, j + 1, k + 1) - spp(i + 1, j + 1, k)) * _dp +
                                3.0 * ((tRp(i, j, k) + tRp(i + 1, j, k)) * 0.5) / aR +
                                2.0 * ((ttp(i, j, k) + ttp(i, j + 1, k)) * 0.5) / aR * cot(aT);
                    if (rV) dV += rV3(i + 1, j + 1, k + 1);
                    Vp(i + 1, j + 1, k + 1) = Vp(i + 1, j + 1, k + 1) + dV * ((DT_R(i + 1, j + 1, k) + DT_R(i + 1, j + 1, k + 1)) * 0.5);
                }
            }
}

void orc_sph_compute_V(orc_sph_state* s, const orc_sph_params* q) { sph_compute_V_impl(s, q, nullptr); }

// ---- boundary conditions ---------------------------------------------------
// BC_R!  SphericalStokes_diapir.jl:61-69 (identical in SphericalStokes_plateau.jl:64-72)
static void sph_bc_R(orc_sph_state* s) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    for (long k = 1; k <= np; ++k) for (long j = 1; j <= nt; ++j) { VR(1, j, k) = -VR(2, j, k); VR(nr + 1, j, k) = -VR(nr, j, k); }
    for (long k = 1; k <= np; ++k) for (long j = 1; j <= nt + 1; ++j) { Vt(1, j, k) = Vt(2, j, k); Vt(nr, j, k) = Vt(nr - 1, j, k); }
    for (long k = 1; k <= np + 1; ++k) for (long j = 1; j <= nt; ++j) { Vp(1, j, k) = Vp(2, j, k); Vp(nr, j, k) = Vp(nr - 1, j, k); }
}

// BC_θ! (diapir simple shear)  SphericalStokes_diapir.jl:71-86
static void sph_bc_t_diapir(orc_sph_state* s, const orc_sph_params* q) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr th = A(s->th, nr, nt, np);
    const double r = q->r, sh = q->sh;
    for (long k = 1; k <= np; ++k) for (long i = 1; i <= nr + 1; ++i) { VR(i, 1, k) = 0.0; VR(i, nt, k) = 0.0; }
    for (long k = 1; k <= np; ++k) for (long i = 1; i <= nr; ++i) { Vt(i, 1, k) = -Vt(i, 2, k); Vt(i, nt + 1, k) = -Vt(i, nt, k); }
    for (long k = 1; k <= np + 1; ++k)
        for (long i = 1; i <= nr; ++i) {
            long kk = (k <= np) ? k : k - 1;
            Vp(i, 1, k) = (th(i, 1, kk) - PI / 2.0) * r * sh;
            Vp(i, nt, k) = (th(i, nt, kk) - PI / 2.0) * r * sh;
        }
}

// BC_φ! (diapir simple shear)  SphericalStokes_diapir.jl:88-99
static void sph_bc_p_diapir(orc_sph_state* s, const orc_sph_params* q) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr th = A(s->th, nr, nt, np);
    const double r = q->r, sh = q->sh;
    for (long j = 1; j <= nt; ++j) for (long i = 1; i <= nr + 1; ++i) { VR(i, j, 1) = 0.0; VR(i, j, np) = 0.0; }
    for (long j = 1; j <= nt + 1; ++j) for (long i = 1; i <= nr; ++i) { Vt(i, j, 1) = 0.0; Vt(i, j, np) = 0.0; }
    for (long j = 1; j <= nt; ++j)
        for (long i = 1; i <= nr; ++i) {
            Vp(i, j, 1) = 2 * (th(i, j, 1) - PI / 2.0) * r * sh - Vp(i, j, 2);
            Vp(i, j, np + 1) = 2 * (th(i, j, np) - PI / 2.0) * r * sh - Vp(i, j, np);
        }
}

// BC_θ! / BC_φ! (free slip)  SphericalStokes_plateau.jl:74-92
static void sph_bc_t_free(orc_sph_state* s, bool copy_normal_ghost = true) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    for (long k = 1; k <= np; ++k) for (long i = 1; i <= nr + 1; ++i) { VR(i, 1, k) = VR(i, 2, k); VR(i, nt, k) = VR(i, nt - 1, k); }
    if (copy_normal_ghost)
        for (long k = 1; k <= np; ++k) for (long i = 1; i <= nr; ++i) { Vt(i, 1, k) = -Vt(i, 2, k); Vt(i, nt + 1, k) = -Vt(i, nt, k); }
    for (long k = 1; k <= np + 1; ++k) for (long i = 1; i <= nr; ++i) { Vp(i, 1, k) = Vp(i, 2, k); Vp(i, nt, k) = Vp(i, nt - 1, k); }
}
static void sph_bc_p_free(orc_sph_state* s, bool copy_normal_ghost = true) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    for (long j = 1; j <= nt; ++j) for (long i = 1; i <= nr + 1; ++i) { VR(i, j, 1) = VR(i, j, 2); VR(i, j, np) = VR(i, j, np - 1); }
    for (long j = 1; j <= nt + 1; ++j) for (long i = 1; i <= nr; ++i) { Vt(i, j, 1) = Vt(i, j, 2); Vt(i, j, np) = Vt(i, j, np - 1); }
    if (copy_normal_ghost)
        for (long j = 1; j <= nt; ++j) for (long i = 1; i <= nr; ++i) { Vp(i, j, 1) = -Vp(i, j, 2); Vp(i, j, np + 1) = -Vp(i, j, np); }
}

// EXT far-field normal stress (classic free-surface treatment of a grid whose
// boundary cells are centred on the wall): the ghost normal velocity makes the
// boundary cell divergence-free, and the boundary cell's pressure is slaved to
// the traction, P = τ_nn - σ_bc (sph_stress_pressure, after compute_P!; the
// average of the two conditions at cells on both a θ and a φ face).
// Tangential components: free slip.
static void sph_bc_stress_t(orc_sph_state* s, const orc_sph_params* q) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np);
    const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp;
    for (int side = 0; side < 2; ++side) {
        long jb = side == 0 ? 1 : nt;          // boundary cell row
        long jg = side == 0 ? 1 : nt + 1;      // ghost Vt row
        long jv = side == 0 ? 2 : nt;          // interior Vt row
        double sgn = side == 0 ? -1.0 : 1.0;   // d(Vt[j+1]-Vt[j])/d(ghost)
        for (long k = 1; k <= np; ++k)
            for (long i = 1; i <= nr; ++i) {
                double Rc = R(i, jb, k), tc = th(i, jb, k);
                double a2 = _dt / Rc, a3 = _dp / (Rc * std::sin(tc)), c1 = 2.0 / Rc, c2 = cot(tc) / Rc;
                double avx = 0.5 * (VR(i, jb, k) + VR(i + 1, jb, k));
                double v = Vt(i, jv, k);
                // DIVV = A0 + B*ghost = 0
                double A0 = _dr * (VR(i + 1, jb, k) - VR(i, jb, k)) + a3 * (Vp(i, jb, k + 1) - Vp(i, jb, k)) + c1 * avx + a2 * (-sgn) * v + c2 * 0.5 * v;
                double B = a2 * sgn + 0.5 * c2;
                Vt(i, jg, k) = -A0 / B;
            }
    }
    (void)q;
}
static void sph_bc_stress_p(orc_sph_state* s, const orc_sph_params* q) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np);
    const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp;
    for (int side = 0; side < 2; ++side) {
        long kb = side == 0 ? 1 : np, kg = side == 0 ? 1 : np + 1, kv = side == 0 ? 2 : np;
        double sgn = side == 0 ? -1.0 : 1.0;
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i) {
                double Rc = R(i, j, kb), tc = th(i, j, kb);
                double a2 = _dt / Rc, a3 = _dp / (Rc * std::sin(tc)), c1 = 2.0 / Rc, c2 = cot(tc) / Rc;
                double avx = 0.5 * (VR(i, j, kb) + VR(i + 1, j, kb));
                double avy = 0.5 * (Vt(i, j, kb) + Vt(i, j + 1, kb));
                double v = Vp(i, j, kv);
                double A0 = _dr * (VR(i + 1, j, kb) - VR(i, j, kb)) + a2 * (Vt(i, j + 1, kb) - Vt(i, j, kb)) + c1 * avx + c2 * avy + a3 * (-sgn) * v;
                double B = a3 * sgn;
                Vp(i, j, kg) = -A0 / B;
            }
    }
}

// EXT: boundary-cell pressure of the stress BC, P = τ_nn - σ_bc on the θ and φ faces
void orc_sph_stress_pressure(double* Pa, const double* ttt, const double* tpp, int64_t nr, int64_t nt, int64_t np,
                             double sig_t, double sig_p) {
    Arr P = A(Pa, nr, nt, np), T2 = A(const_cast<double*>(ttt), nr, nt, np), T3 = A(const_cast<double*>(tpp), nr, nt, np);
    for (long k = 1; k <= np; ++k)
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i) {
                bool bt = (j == 1 || j == nt), bp = (k == 1 || k == np);
                if (!bt && !bp) continue;
                double acc = 0.0, cnt = 0.0;
                if (bt) { acc += T2(i, j, k) - sig_t; cnt += 1.0; }
                if (bp) { acc += T3(i, j, k) - sig_p; cnt += 1.0; }
                P(i, j, k) = acc / cnt;
            }
}

// EXT free-surface top boundary (bc 3, the plateau's topography load without sticky air): the
// top radial face carries the traction of a surface load q(θ,φ) plus the stabilisation term
// κ V_r of the free-surface stabilisation algorithm (the load of the surface's rise over a time
// step, κ = θ Δt Δρ g), with zero shear traction; the bottom face and the θ, φ faces are free
// slip.  As for the far-field stress BC, the boundary passes through the top cells' centres:
// the ghost VR(nr+1) makes the top cell divergence-free and the top cell's pressure is slaved
// to the traction (orc_sph_fs_pressure).  BC_R's copies of Vθ, Vφ come first, the ghost uses them.
static void sph_bc_R_fs(orc_sph_state* s, const orc_sph_params* q) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np);
    for (long k = 1; k <= np; ++k) for (long j = 1; j <= nt; ++j) VR(1, j, k) = -VR(2, j, k);
    for (long k = 1; k <= np; ++k) for (long j = 1; j <= nt + 1; ++j) { Vt(1, j, k) = Vt(2, j, k); Vt(nr, j, k) = Vt(nr - 1, j, k); }
    for (long k = 1; k <= np + 1; ++k) for (long j = 1; j <= nt; ++j) { Vp(1, j, k) = Vp(2, j, k); Vp(nr, j, k) = Vp(nr - 1, j, k); }
    const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp;
    for (long k = 1; k <= np; ++k)
        for (long j = 1; j <= nt; ++j) {
            double Rc = R(nr, j, k), tc = th(nr, j, k);
            double a2 = _dt / Rc, a3 = _dp / (Rc * std::sin(tc)), c1 = 2.0 / Rc, c2 = cot(tc) / Rc;
            double v = VR(nr, j, k);
            double avy = 0.5 * (Vt(nr, j, k) + Vt(nr, j + 1, k));
            // DIVV of cell nr = A0 + B * ghost = 0
            double A0 = -_dr * v + 0.5 * c1 * v + a2 * (Vt(nr, j + 1, k) - Vt(nr, j, k)) + a3 * (Vp(nr, j, k + 1) - Vp(nr, j, k)) + c2 * avy;
            double B = _dr + 0.5 * c1;
            VR(nr + 1, j, k) = -A0 / B;
        }
}

// EXT: top-cell pressure of the free-surface BC, P = τ_RR + q + κ V_r (V_r at the cell centre:
// the mean of the top cell's inner face and ghost); load NULL: q = 0
void orc_sph_fs_pressure(double* Pa, const double* tRR, const double* VRa, const double* load, int64_t nr, int64_t nt, int64_t np,
                         double kappa) {
    Arr P = A(Pa, nr, nt, np), T1 = A(const_cast<double*>(tRR), nr, nt, np), VR = A(const_cast<double*>(VRa), nr + 1, nt, np);
    Arr L = A(const_cast<double*>(load), nr, nt, np);
    for (long k = 1; k <= np; ++k)
        for (long j = 1; j <= nt; ++j)
            P(nr, j, k) = T1(nr, j, k) + (load ? L(nr, j, k) : 0.0) + kappa * 0.5 * (VR(nr, j, k) + VR(nr + 1, j, k));
}

void orc_sph_apply_bc(orc_sph_state* s, const orc_sph_params* q) {
    if (q->bc == 3) sph_bc_R_fs(s, q);
    else sph_bc_R(s);
    if (q->bc == 0) { sph_bc_t_diapir(s, q); sph_bc_p_diapir(s, q); }
    else if (q->bc == 1 || q->bc == 3) { sph_bc_t_free(s); sph_bc_p_free(s); }
    else { sph_bc_t_free(s, false); sph_bc_stress_t(s, q); sph_bc_p_free(s, false); sph_bc_stress_p(s, q); }
}

// ---- EXT: strain rates at centres and edges (as in compute_P!), the strain-rate
// invariant at (clamped) cells, and the strain-rate power law ------------------
static void sph_strain(orc_sph_state* s, const orc_sph_params* q, double* Dd, double* Ert, double* Erp, double* Etp) {
    // Dd: 0.5*(DRR^2+Dtt^2+Dpp^2) at centres; E**: engineering shear strain rates at edges
    const long nr = s->nr, nt = s->nt, np = s->np;
    Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
    Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np);
    Arr DD = A(Dd, nr, nt, np), Ert_ = A(Ert, nr - 1, nt - 1, np - 2), Erp_ = A(Erp, nr - 1, nt - 2, np - 1), Etp_ = A(Etp, nr - 2, nt - 1, np - 1);
    const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp;
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= np; ++k)
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i) {
                double avxa_VR = ((VR(i, j, k) + VR(i + 1, j, k)) * 0.5);
                double avya_Vt = ((Vt(i, j, k) + Vt(i, j + 1, k)) * 0.5);
                double Rc = R(i, j, k), tc = th(i, j, k);
                double DIVV = (VR(i + 1, j, k) - VR(i, j, k)) * _dr + 1.0 / Rc * (Vt(i, j + 1, k) - Vt(i, j, k)) * _dt +
                              1.0 / Rc / std::sin(tc) * (Vp(i, j, k + 1) - Vp(i, j, k)) * _dp + 2.0 * avxa_VR / Rc + avya_Vt / Rc * cot(tc);
                double DRR = (VR(i + 1, j, k) - VR(i, j, k)) * _dr - 1.0 / 3.0 * DIVV;
                double Dtt = 1.0 / Rc * (Vt(i, j + 1, k) - Vt(i, j, k)) * _dt + avxa_VR / Rc - 1.0 / 3.0 * DIVV;
                double Dpp = 1.0 / Rc / std::sin(tc) * (Vp(i, j, k + 1) - Vp(i, j, k)) * _dp + avxa_VR / Rc + avya_Vt / Rc * cot(tc) - 1.0 / 3.0 * DIVV;
                DD(i, j, k) = 0.5 * (DRR * DRR + Dtt * Dtt + Dpp * Dpp);
                if (i <= nr - 1 && j <= nt - 1 && k <= np - 2) {
                    double aR = ((R(i, j, k + 1) + R(i, j + 1, k + 1) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k + 1)) * 0.25);
                    Ert_(i, j, k) = (Vt(i + 1, j + 1, k + 1) - Vt(i, j + 1, k + 1)) * _dr + 1.0 / aR * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j, k + 1)) * _dt -
                                    ((Vt(i, j + 1, k + 1) + Vt(i + 1, j + 1, k + 1)) * 0.5) / aR;
                }
                if (i <= nr - 1 && j <= nt - 2 && k <= np - 1) {
                    double aR = ((R(i, j + 1, k) + R(i, j + 1, k + 1) + R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.25);
                    double aT = ((th(i, j + 1, k) + th(i, j + 1, k + 1) + th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.25);
                    Erp_(i, j, k) = (Vp(i + 1, j + 1, k + 1) - Vp(i, j + 1, k + 1)) * _dr + 1.0 / aR / std::sin(aT) * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j + 1, k)) * _dp -
                                    ((Vp(i, j + 1, k + 1) + Vp(i + 1, j + 1, k + 1)) * 0.5) / aR;
                }
                if (i <= nr - 2 && j <= nt - 1 && k <= np - 1) {
                    double aR = ((R(i + 1, j, k) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.25);
                    double aT = ((th(i + 1, j, k) + th(i + 1, j, k + 1) + th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.25);
                    Etp_(i, j, k) = 1.0 / aR * (Vp(i + 1, j + 1, k + 1) - Vp(i + 1, j, k + 1)) * _dt + 1.0 / aR / std::sin(aT) * (Vt(i + 1, j + 1, k + 1) - Vt(i + 1, j + 1, k)) * _dp -
                                    ((Vp(i + 1, j, k + 1) + Vp(i + 1, j + 1, k + 1)) * 0.5) / aR * cot(aT);
                }
            }
}

// second invariant of the strain rate at cell (i,j,k) of the interior, with the
// edge components averaged 4->1 exactly as compute_TII! averages the stresses
static inline double sph_edot_II(const Arr& DD, const Arr& Ert, const Arr& Erp, const Arr& Etp, long i, long j, long k) {
    // (i,j,k) is an interior cell: 2 <= i <= nr-1 etc.; edge indices as compute_TII! with (i-1,j-1,k-1)
    long a = i - 1, b = j - 1, c = k - 1;
    double ert = (Ert(a, b, c) + Ert(a, b + 1, c) + Ert(a + 1, b, c) + Ert(a + 1, b + 1, c)) * 0.25;
    double erp = (Erp(a, b, c) + Erp(a, b, c + 1) + Erp(a + 1, b, c) + Erp(a + 1, b, c + 1)) * 0.25;
    double etp = (Etp(a, b, c) + Etp(a, b, c + 1) + Etp(a, b + 1, c) + Etp(a, b + 1, c + 1)) * 0.25;
    return std::sqrt(DD(i, j, k) + 0.25 * (ert * ert + erp * erp + etp * etp));
}

static inline long clampi(long i, long n) { return i < 2 ? 2 : (i > n - 1 ? n - 1 : i); }

// EXT strain-rate power law: eta_t = 2/(1/eta_ini + 1/(eta_ini (edot_II/edot_bg)^((1-n)/n)));
// relaxed in log space: eta <- eta^(1-relax) * eta_t^relax.  Boundary cells use
// the invariant of the clamped interior cell (as copy_BC! does for τII).
// relax_on == 0 returns the unrelaxed target (used by the residual).
void orc_sph_edot_law(orc_sph_state* s, const orc_sph_params* q, double* eta_out, int32_t relax_on, double* scratch) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    long nc = nr * nt * np;
    double* Dd = scratch;
    double* Ert = Dd + nc;
    double* Erp = Ert + (nr - 1) * (nt - 1) * (np - 2);
    double* Etp = Erp + (nr - 1) * (nt - 2) * (np - 1);
    sph_strain(s, q, Dd, Ert, Erp, Etp);
    Arr DD = A(Dd, nr, nt, np), E1 = A(Ert, nr - 1, nt - 1, np - 2), E2 = A(Erp, nr - 1, nt - 2, np - 1), E3 = A(Etp, nr - 2, nt - 1, np - 1);
    Arr eta = A(s->eta, nr, nt, np), ei = A(s->eta_ini, nr, nt, np), out = A(eta_out, nr, nt, np);
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= np; ++k)
        for (long j = 1; j <= nt; ++j)
            for (long i = 1; i <= nr; ++i) {
                double ed = sph_edot_II(DD, E1, E2, E3, clampi(i, nr), clampi(j, nt), clampi(k, np));
                long c = (i - 1) + nr * ((j - 1) + nt * (k - 1));
                bool lin = s->phase && s->phase[c];
                double ne = lin ? 1.0 : q->n_exp;
                double e0 = ei(i, j, k);
                double ept = e0 * std::pow(ed / q->edot_bg, (1.0 - ne) / ne);
                double et = lin ? e0 : 2.0 / (1.0 / e0 + 1.0 / ept);
                out(i, j, k) = relax_on ? std::exp((1.0 - q->relax) * std::log(eta(i, j, k)) + q->relax * std::log(et)) : et;
            }
}

// scratch size (doubles) needed by orc_sph_edot_law / orc_sph_residual
int64_t orc_sph_scratch_size(int64_t nr, int64_t nt, int64_t np) {
    return nr * nt * np + (nr - 1) * (nt - 1) * (np - 2) + (nr - 1) * (nt - 2) * (np - 1) + (nr - 2) * (nt - 1) * (np - 1);
}

// ---- one PT iteration in the scripts' call order ----------------------------
// SphericalStokes_diapir.jl:413-425 (plateau: SphericalStokes_plateau.jl:526-538)
void orc_sph_iterate(orc_sph_state* s, const orc_sph_params* q, int64_t niter) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    for (long it = 0; it < niter; ++it) {
        orc_sph_equal3(s);
        orc_maxloc(s->etaSM, s->eta, nr, nt, np);
        orc_copy_BC(s->etaSM, nr, nt, np);
        for (int pass = 1; pass < q->passes; ++pass) {  // EXT wider max filter
            std::vector<double> tmp(s->etaSM, s->etaSM + nr * nt * np);
            orc_maxloc(s->etaSM, tmp.data(), nr, nt, np);
            orc_copy_BC(s->etaSM, nr, nt, np);
        }
        orc_sph_compute_P(s, q);
        if (q->bc == 2) orc_sph_stress_pressure(s->P, s->ttt, s->tpp, nr, nt, np, q->sig_t, q->sig_p);
        if (q->bc == 3) orc_sph_fs_pressure(s->P, s->tRR, s->VR, q->top_load, nr, nt, np, q->fs_kappa);
        if (q->rheo == 0) {
            orc_sph_compute_TII(s);
            orc_copy_BC(s->tII, nr, nt, np);
            orc_sph_power_law(s, q);
        } else if (q->rheo == 1) {
            // EXT: the strain rates of the same velocities compute_P! used
            // (velocities are not modified by compute_P!)
            orc_sph_compute_TII(s);
            orc_copy_BC(s->tII, nr, nt, np);
            orc_sph_edot_law(s, q, s->eta_tmp, 1, s->eta_tmp + nr * nt * np);
            std::memcpy(s->eta, s->eta_tmp, sizeof(double) * nr * nt * np);
        }
        orc_sph_compute_V(s, q);
        orc_sph_apply_bc(s, q);
    }
}

// check_err! + the reference's stopping norm  SphericalStokes_diapir.jl:332-344, 428-432:
// max over the three velocity arrays of max|V - V_err| / max|V|, NaN propagating as
// Julia's maximum / max do.  skip_nan_phi: the plateau script's rule
// (SphericalStokes_plateau.jl:540-552), a NaN Vφ ratio is left out.
static double check_err_impl(orc_sph_state* s, bool skip_nan_phi) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    long n[3] = {(nr + 1) * nt * np, nr * (nt + 1) * np, nr * nt * (np + 1)};
    double* V[3] = {s->VR, s->Vt, s->Vp};
    double* E[3] = {s->VR_err, s->Vt_err, s->Vp_err};
    double err = 0.0;
    for (int f = 0; f < 3; ++f) {
        double md = 0.0, mv = 0.0;
        for (long c = 0; c < n[f]; ++c) {
            E[f][c] = V[f][c] - E[f][c];
            md = nmax(md, E[f][c]);
            mv = nmax(mv, V[f][c]);
        }
        const double r = md / mv;
        if (r != r && skip_nan_phi && f == 2) continue;
        err = (r != r || err != err) ? NAN : std::max(err, r);
    }
    return err;
}
double orc_sph_check_err(orc_sph_state* s) { return check_err_impl(s, false); }
double orc_sph_check_err_plateau(orc_sph_state* s) { return check_err_impl(s, true); }

// ---- EXT: FP64 Stokes residual ---------------------------------------------
// Momentum residual at interior velocity nodes (the compute_V! increments with
// tau = 2 eta D(V) at centres and avg4(eta) D at edges, eta = the strain-rate
// law target when rheo == 1, else the stored eta) and continuity (DIVV) at all
// cells.  out[0..2] = max|dVR|,|dVt|,|dVp|; out[3] = max|DIVV|; out[4] = max|V|
// over the three arrays.  Optional fields (may be NULL) receive dV and DIVV in
// the velocity / centre array layouts (boundary entries zero).
void orc_sph_residual(orc_sph_state* s, const orc_sph_params* q, double* out, double* scratch,
                      double* rVR, double* rVt, double* rVp, double* rDiv) {
    const long nr = s->nr, nt = s->nt, np = s->np;
    long nc = nr * nt * np;
    long ne1 = (nr - 1) * (nt - 1) * (np - 2), ne2 = (nr - 1) * (nt - 2) * (np - 1), ne3 = (nr - 2) * (nt - 1) * (np - 1);
    // layout of scratch: eta_eff | edot scratch (for the law) | tau (6) | P copy
    double* eta_eff = scratch;
    double* lawscr = eta_eff + nc;
    double* t6 = lawscr + orc_sph_scratch_size(nr, nt, np);
    double *tRR = t6, *ttt = tRR + nc, *tpp = ttt + nc, *tRt = tpp + nc, *tRp = tRt + ne1, *ttp = tRp + ne2;
    double* DT_R = ttp + ne3;   // holds zeros (unused by the residual)
    if (q->rheo == 1) orc_sph_edot_law(s, q, eta_eff, 0, lawscr);
    else std::memcpy(eta_eff, s->eta, sizeof(double) * nc);
    // tau = 2 eta D : run compute_P! with GSDT -> infinity is not representable,
    // so evaluate the strain rates directly
    {
        Arr VR = A(s->VR, nr + 1, nt, np), Vt = A(s->Vt, nr, nt + 1, np), Vp = A(s->Vp, nr, nt, np + 1);
        Arr R = A(s->R, nr, nt, np), th = A(s->th, nr, nt, np), E = A(eta_eff, nr, nt, np);
        Arr TRR = A(tRR, nr, nt, np), TTT = A(ttt, nr, nt, np), TPP = A(tpp, nr, nt, np);
        Arr TRt = A(tRt, nr - 1, nt - 1, np - 2), TRp = A(tRp, nr - 1, nt - 2, np - 1), Ttp = A(ttp, nr - 2, nt - 1, np - 1);
        Arr DIV = A(rDiv ? rDiv : DT_R, nr, nt, np);
        const double _dr = q->_dr, _dt = q->_dt, _dp = q->_dp;
        double mdiv = 0.0;
#pragma omp parallel for schedule(static)
        for (long k = 1; k <= np; ++k)
            for (long j = 1; j <= nt; ++j)
                for (long i = 1; i <= nr; ++i) {
                    double avxa_VR = ((VR(i, j, k) + VR(i + 1, j, k)) * 0.5);
                    double avya_Vt = ((Vt(i, j, k) + Vt(i, j + 1, k)) * 0.5);
                    double Rc = R(i, j, k), tc = th(i, j, k);
                    double DIVV = (VR(i + 1, j, k) - VR(i, j, k)) * _dr + 1.0 / Rc * (Vt(i, j + 1, k) - Vt(i, j, k)) * _dt +
                                  1.0 / Rc / std::sin(tc) * (Vp(i, j, k + 1) - Vp(i, j, k)) * _dp + 2.0 * avxa_VR / Rc + avya_Vt / Rc * cot(tc);
                    double DRR = (VR(i + 1, j, k) - VR(i, j, k)) * _dr - 1.0 / 3.0 * DIVV;
                    double Dtt = 1.0 / Rc * (Vt(i, j + 1, k) - Vt(i, j, k)) * _dt + avxa_VR / Rc - 1.0 / 3.0 * DIVV;
                    double Dpp = 1.0 / Rc / std::sin(tc) * (Vp(i, j, k + 1) - Vp(i, j, k)) * _dp + avxa_VR / Rc + avya_Vt / Rc * cot(tc) - 1.0 / 3.0 * DIVV;
                    double e = E(i, j, k);
                    TRR(i, j, k) = 2.0 * e * DRR; TTT(i, j, k) = 2.0 * e * Dtt; TPP(i, j, k) = 2.0 * e * Dpp;
                    DIV(i, j, k) = DIVV;
                    if (i <= nr - 1 && j <= nt - 1 && k <= np - 2) {
                        double aR = ((R(i, j, k + 1) + R(i, j + 1, k + 1) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k + 1)) * 0.25);
                        double D = (Vt(i + 1, j + 1, k + 1) - Vt(i, j + 1, k + 1)) * _dr + 1.0 / aR * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j, k + 1)) * _dt -
                                   ((Vt(i, j + 1, k + 1) + Vt(i + 1, j + 1, k + 1)) * 0.5) / aR;
                        double aE = ((E(i, j, k + 1) + E(i, j + 1, k + 1) + E(i + 1, j, k + 1) + E(i + 1, j + 1, k + 1)) * 0.25);
                        TRt(i, j, k) = aE * D;
                    }
                    if (i <= nr - 1 && j <= nt - 2 && k <= np - 1) {
                        double aR = ((R(i, j + 1, k) + R(i, j + 1, k + 1) + R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.25);
                        double aT = ((th(i, j + 1, k) + th(i, j + 1, k + 1) + th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.25);
                        double D = (Vp(i + 1, j + 1, k + 1) - Vp(i, j + 1, k + 1)) * _dr + 1.0 / aR / std::sin(aT) * (VR(i + 1, j + 1, k + 1) - VR(i + 1, j + 1, k)) * _dp -
                                   ((Vp(i, j + 1, k + 1) + Vp(i + 1, j + 1, k + 1)) * 0.5) / aR;
                        double aE = ((E(i, j + 1, k) + E(i, j + 1, k + 1) + E(i + 1, j + 1, k) + E(i + 1, j + 1, k + 1)) * 0.25);
                        TRp(i, j, k) = aE * D;
                    }
                    if (i <= nr - 2 && j <= nt - 1 && k <= np - 1) {
                        double aR = ((R(i + 1, j, k) + R(i + 1, j, k + 1) + R(i + 1, j + 1, k) + R(i + 1, j + 1, k + 1)) * 0.25);
                        double aT = ((th(i + 1, j, k) + th(i + 1, j, k + 1) + th(i + 1, j + 1, k) + th(i + 1, j + 1, k + 1)) * 0.25);
                        double D = 1.0 / aR * (Vp(i + 1, j + 1, k + 1) - Vp(i + 1, j, k + 1)) * _dt + 1.0 / aR / std::sin(aT) * (Vt(i + 1, j + 1, k + 1) - Vt(i + 1, j + 1, k)) * _dp -
                                   ((Vp(i + 1, j, k + 1) + Vp(i + 1, j + 1, k + 1)) * 0.5) / aR * cot(aT);
                        double aE = ((E(i + 1, j, k) + E(i + 1, j, k + 1) + E(i + 1, j + 1, k) + E(i + 1, j + 1, k + 1)) * 0.25);
                        Ttp(i, j, k) = aE * D;
                    }
                }
        const double* dv = rDiv ? rDiv : DT_R;
        for (long c = 0; c < nc; ++c) mdiv = nmax(mdiv, dv[c]);
        out[3] = mdiv;
    }
    // momentum residual: compute_V! increments with DT_R = 1 into zeroed arrays
    orc_sph_state t = *s;
    t.tRR = tRR; t.ttt = ttt; t.tpp = tpp; t.tRt = tRt; t.tRp = tRp; t.ttp = ttp;
    std::vector<double> Pres;
    if (q->bc == 2) {  // boundary-cell pressure of the stress BC from the viscous stresses
        Pres.assign(s->P, s->P + nc);
        orc_sph_stress_pressure(Pres.data(), ttt, tpp, nr, nt, np, q->sig_t, q->sig_p);
        t.P = Pres.data();
    }
    if (q->bc == 3) {  // top-cell pressure of the free surface from the viscous stress
        Pres.assign(s->P, s->P + nc);
        orc_sph_fs_pressure(Pres.data(), tRR, s->VR, q->top_load, nr, nt, np, q->fs_kappa);
        t.P = Pres.data();
    }
    long nv[3] = {(nr + 1) * nt * np, nr * (nt + 1) * np, nr * nt * (np + 1)};
    double* own[3] = {rVR, rVt, rVp};
    double* tmp[3];
    for (int f = 0; f < 3; ++f) {
        tmp[f] = own[f] ? own[f] : new double[nv[f]];
        std::memset(tmp[f], 0, sizeof(double) * nv[f]);
    }
    for (long c = 0; c < nc; ++c) DT_R[c] = 1.0;
    t.VR = tmp[0]; t.Vt = tmp[1]; t.Vp = tmp[2]; t.DT_R = DT_R;
    orc_sph_compute_V(&t, q);
    for (int f = 0; f < 3; ++f) {
        double m = 0.0, mv = 0.0;
        double* V = f == 0 ? s->VR : (f == 1 ? s->Vt : s->Vp);
        for (long c = 0; c < nv[f]; ++c) { m = nmax(m, tmp[f][c]); mv = nmax(mv, V[c]); }
        out[f] = m;
        out[4] = f == 0 ? mv : std::max(out[4], mv);
        if (!own[f]) delete[] tmp[f];
    }
}

// scratch size (doubles) for orc_sph_residual
int64_t orc_sph_residual_scratch_size(int64_t nr, int64_t nt, int64_t np) {
    int64_t nc = nr * nt * np;
    return nc + orc_sph_scratch_size(nr, nt, np) + 4 * nc + (nr - 1) * (nt - 1) * (np - 2) + (nr - 1) * (nt - 2) * (np - 1) +
           (nr - 2) * (nt - 1) * (np - 1);
}

// ---- EXT: correction sweeps of the mixed-precision solve ---------------------
// One PT iteration of the correction problem per sweep: the state (P, V, τ) holds
// the correction (δP, δV, δτ); η and ηSM are frozen (no maxloc!, no viscosity
// update); rP is added to the divergence in the pressure update and rV (velocity
// layouts) to the momentum rows in place of -ρg; the boundary conditions are the
// homogeneous form of the BC set (diapir shear sh = 0, prescribed stresses 0).
// The steps are those of the reference iteration (compute_P! :209-241, compute_V!
// :308-329, BC_R!/BC_θ!/BC_φ! :61-99) with these right-hand sides.
void orc_sph_corr_sweep(orc_sph_state* s, const orc_sph_params* q, const double* rP, const double* rVR, const double* rVt,
                        const double* rVp, int64_t nsweeps) {
    orc_sph_params h = *q;
    h.sh = 0.0;
    h.g = 0.0;
    h.sig_t = 0.0;
    h.sig_p = 0.0;
    const double* rV[3] = {rVR, rVt, rVp};
    for (int64_t it = 0; it < nsweeps; ++it) {
        sph_compute_P_impl(s, &h, rP);
        if (h.bc == 2) orc_sph_stress_pressure(s->P, s->ttt, s->tpp, s->nr, s->nt, s->np, 0.0, 0.0);
        if (h.bc == 3) orc_sph_fs_pressure(s->P, s->tRR, s->VR, nullptr, s->nr, s->nt, s->np, h.fs_kappa);
        sph_compute_V_impl(s, &h, rV);
        orc_sph_apply_bc(s, &h);
    }
}

int32_t orc_num_threads(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int32_t n) {
#if defined(_OPENMP)
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // extern "C"
