// libsphstokes — C ABI over the sm_103a pseudo-transient Stokes kernels.
//
// The context owns the device arrays of one grid (FP64 master state, plus an
// FP32 state for the FP32 / mixed-precision paths), the metric tables and the
// boundary-condition program, and drives the PT loop of the reference scripts
// (SphericalStokes_diapir.jl:409-443) on one CUDA stream.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <new>
#include <string>
#include <vector>

#include "sph_pt.cuh"
#include "sph_fused.cuh"
#include "sph_sweep_x2.cuh"
#include "sph_adjoint.cuh"
#include "sph_advect.cuh"
#include "sph_batch.cuh"
#include "sphstokes.h"

using namespace sph;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            return fail(SPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));        \
        }                                                                                         \
    } while (0)

const double kPi = 3.141592653589793;

enum FieldSlot {
    F_P, F_V1, F_V2, F_V3, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23,
    F_ETA, F_ETA_INI, F_ETA_SM, F_DT_R, F_TII, F_RHO, F_ETA_PL, F_ETA_OUT,
    F_V1E, F_V2E, F_V3E, F_RP, F_RV1, F_RV2, F_RV3, F_SDD, F_S12, F_S13, F_S23,
    F_Q11, F_Q22, F_Q33, F_Q12, F_Q13, F_Q23,
    // second copy of the PT state (ping-pong of the fused sweep)
    F_A_P, F_A_V1, F_A_V2, F_A_V3, F_A_T11, F_A_T22, F_A_T33, F_A_T12, F_A_T13, F_A_T23,
    F_PRES,  // pressure of the residual evaluation (traction-slaved boundary cells)
    F_LOAD,  // free-surface load on the top cells
    F_NSLOTS
};

template <typename T>
struct State {
    T* f[F_NSLOTS] = {};
    T* slab = nullptr;
    T* tab = nullptr;  // metric tables
    Geo<T> geo{};
};

struct Ctx {
    sph_params prm;
    Dims d;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    State<double> s64;
    State<float> s32;
    bool has32 = false;
    bool stale32 = true;   // FP32 state must be refreshed from FP64 before use
    bool stale64 = false;  // FP64 state must be refreshed from FP32 before use
    uint8_t* phase = nullptr;
    unsigned long long* red = nullptr;   // device reduction slots
    unsigned long long* hred = nullptr;  // pinned host copy
    std::vector<BcStage> bc;      // BC program: ghost-velocity stages in the reference order (the adjoint transposes these)
    std::vector<BcStage> bc_run;  // the program launched by launch_bc: bc, or an equivalent one with fewer stages
    // the first stage of bc_run in the homogeneous case as factors of the interior neighbour
    // (ghost = xg[f] x neighbour on both x1 faces, field f in bit f of xg_mask); 0: not of that form
    int xg_mask = 0;
    float xg[3] = {0.f, 0.f, 0.f};
    bool xg_fuse = true;  // the correction sweep writes those ghosts (SPH_NO_XGHOST=1: the BC stage does)
    double cur_n = 1.0;
    double f_scale = 1.0;
    double last_ms = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr, ev4 = nullptr;
    double sweep_ms = 0.0, outer_ms = 0.0;  // device time split of the last solve (MIXED)
    std::vector<double> hx1, hx2, hx3;  // node coordinates (host)
    bool corr_ready = false;  // a correction problem is prepared in the FP32 state (MIXED)
    double corr_r0 = 0.0;     // max|r_V| of the prepared correction problem
    // CUDA graphs of `graph_len` correction sweeps, one per ping-pong arrangement
    cudaGraphExec_t corr_graph[2] = {nullptr, nullptr};
    float* corr_graph_key[2] = {nullptr, nullptr};   // F_P pointer at capture time
    int graph_len = 0;
    // CUDA graphs of `warm_len` FP32 nonlinear iterations (mixed solve warm start), one per
    // arrangement of the ping-pong and η buffers, keyed by the P and η pointers at capture
    cudaGraphExec_t warm_graph[2] = {nullptr, nullptr};
    float* warm_key[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int warm_len = 0;
    bool use_graphs = true;
    // TMA tensor maps of the correction sweep, one set per ping-pong arrangement
    CUtensorMap* d_maps = nullptr;       // [2][TM_COUNT] in device memory
    float* map_key[2] = {nullptr, nullptr};  // V1 buffer of the arrangement a set was built for
    int* d_err = nullptr;                // set by a kernel whose bounded wait ran out
    bool use_tma = true;
    bool use_x2 = false;  // TMA sweep with two points per thread (k_sweep_x2) instead of k_fused_tma
    bool use_pdl = true;  // sweep and BC kernels launched with a programmatic dependency (pdl_enter)
    bool fused = true;   // FP32 sweeps use the fused kernel
    int fused_chunk = 0; // planes per block of the fused sweep (0: chosen by fused_chunk())
    int fused_slots = 0; // resident blocks of the fused TMA sweep on the device (SMs x blocks per SM)
    double* adj = nullptr;  // adjoint arrays (AJ_COUNT slots of the box), allocated on first use
    // per-launch timing of the fused sweep kernel (sph_sweep_profile): event pairs
    // recorded around each launch while prof_next < prof_ev.size()/2
    std::vector<cudaEvent_t> prof_ev;
    size_t prof_next = 0;
    bool prof_on = false;
    double* stage = nullptr;  // dense staging field of the host copies (vol doubles), allocated on first use
    // wall-clock ms from the start of the last sph_solve to each of its history entries
    std::vector<double> hist_ms;
    std::chrono::steady_clock::time_point solve_t0;
    bool broken = false;      // a bounded wait of a sweep kernel ran out: the context's state is suspect
    bool warm_abandoned = false;  // the last mixed solve's FP32 warm start produced a NaN and was abandoned
};

constexpr int kRedSlots = 16;

int field_extent(const Dims& d, int f, int e[3]) {
    e[0] = d.n1; e[1] = d.n2; e[2] = d.n3;
    switch (f) {
        case SPH_FIELD_V1: e[0] += 1; break;
        case SPH_FIELD_V2: e[1] += 1; break;
        case SPH_FIELD_V3: e[2] += 1; break;
        case SPH_FIELD_TAU12: e[0] -= 1; e[1] -= 1; e[2] -= 2; break;
        case SPH_FIELD_TAU13: e[0] -= 1; e[1] -= 2; e[2] -= 1; break;
        case SPH_FIELD_TAU23: e[0] -= 2; e[1] -= 1; e[2] -= 1; break;
        default: break;
    }
    return 0;
}

int slot_of(int field) {
    switch (field) {
        case SPH_FIELD_P: return F_P;
        case SPH_FIELD_V1: return F_V1;
        case SPH_FIELD_V2: return F_V2;
        case SPH_FIELD_V3: return F_V3;
        case SPH_FIELD_TAU11: return F_T11;
        case SPH_FIELD_TAU22: return F_T22;
        case SPH_FIELD_TAU33: return F_T33;
        case SPH_FIELD_TAU12: return F_T12;
        case SPH_FIELD_TAU13: return F_T13;
        case SPH_FIELD_TAU23: return F_T23;
        case SPH_FIELD_ETA: return F_ETA;
        case SPH_FIELD_ETA_INI: return F_ETA_INI;
        case SPH_FIELD_ETA_SM: return F_ETA_SM;
        case SPH_FIELD_DT_R: return F_DT_R;
        case SPH_FIELD_TII: return F_TII;
        case SPH_FIELD_RHO: return F_RHO;
        case SPH_FIELD_ETA_PL: return F_ETA_PL;
        case SPH_FIELD_TOP_LOAD: return F_LOAD;
        default: return -1;
    }
}

// ---------------------------------------------------------------------------
template <typename T>
KP<T> make_kp(Ctx& c, State<T>& s) {
    KP<T> p;
    std::memset(&p, 0, sizeof(p));
    const sph_params& q = c.prm;
    p.d = c.d;
    p.geo = s.geo;
    p.P = s.f[F_P]; p.V1 = s.f[F_V1]; p.V2 = s.f[F_V2]; p.V3 = s.f[F_V3];
    p.t11 = s.f[F_T11]; p.t22 = s.f[F_T22]; p.t33 = s.f[F_T33]; p.t12 = s.f[F_T12]; p.t13 = s.f[F_T13]; p.t23 = s.f[F_T23];
    p.eta = s.f[F_ETA]; p.eta_ini = s.f[F_ETA_INI]; p.etaSM = s.f[F_ETA_SM]; p.DT_R = s.f[F_DT_R]; p.tII = s.f[F_TII];
    p.rho = s.f[F_RHO]; p.eta_pl = s.f[F_ETA_PL]; p.eta_out = s.f[F_ETA_OUT];
    p.phase = c.phase;
    p.rP = s.f[F_RP]; p.rV1 = s.f[F_RV1]; p.rV2 = s.f[F_RV2]; p.rV3 = s.f[F_RV3];
    p.sDD = s.f[F_SDD]; p.s12 = s.f[F_S12]; p.s13 = s.f[F_S13]; p.s23 = s.f[F_S23];
    p.d1 = T((q.n1 - 1) / q.l1); p.d2 = T((q.n2 - 1) / q.l2); p.d3 = T((q.n3 - 1) / q.l3);
    p.kbc = T(q.dmp * 2.0 * kPi * q.vpdt / q.l_ref);
    p.gsc = T(4.0 * kPi * q.vpdt / q.l_ref);
    p.vpdt2 = T(q.vpdt * q.vpdt);
    p.g = T(q.g);
    p.tau_C = T(q.tau_C); p.n_exp = T(c.cur_n); p.relax = T(q.relax); p.edot_bg = T(q.edot_bg);
    p.sig2 = T(q.sig_bc[1]); p.sig3 = T(q.sig_bc[2]);
    p.traction = q.bc == SPH_BC_STRESS ? 1 : 0;
    p.fs = q.bc == SPH_BC_FREE_SURFACE ? 1 : 0;
    p.fs_kappa = T(q.fs_kappa);
    p.top_load = s.f[F_LOAD];
    p.red = c.red;
    return p;
}

dim3 blk2d() { return dim3(32, 8, 1); }

// launch with a programmatic dependency on the preceding grid of the stream (the
// kernel starts with pdl_enter()); a plain launch when PDL is switched off
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(bool pdl, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}
dim3 grid_cells(const Dims& d) { return dim3((d.n1 + 31) / 32, (d.n2 + 7) / 8, d.n3); }
dim3 grid_vel(const Dims& d) { return dim3((d.n1 - 1 + 31) / 32, (d.n2 - 1 + 7) / 8, d.n3 - 1); }

int ew_blocks(long long n) { return (int)std::min<long long>((n + 255) / 256, 152LL * 16); }

// ---------------------------------------------------------------------------
// boundary-condition programs (the reference's BC kernels in call order)
BcOp op(int field, int kind, int cd = 0, double c0 = 0.0, double c1 = 0.0, int side = -1) {
    BcOp o; o.field = field; o.kind = kind; o.cd = cd; o.c0 = c0; o.c1 = c1; o.side = side;
    return o;
}
BcStage stage(int dim, std::initializer_list<BcOp> ops) {
    BcStage s; std::memset(&s, 0, sizeof(s));
    s.dim = dim; s.nops = 0;
    for (const BcOp& o : ops) s.op[s.nops++] = o;
    return s;
}

int build_bc_program(Ctx& c);
int build_bc(Ctx& c) {
    const int rc = build_bc_program(c);
    if (rc != SPH_OK) return rc;
    if (c.bc_run.empty()) c.bc_run = c.bc;
    // homogeneous x1-face stage as factors (NEG -1, COPY +1, ZERO / LIN 0, LIN2M -1)
    c.xg_mask = 0;
    const BcStage& s0 = c.bc_run[0];
    int mask = 0;
    float xg[3] = {0.f, 0.f, 0.f};
    bool ok = s0.dim == 0 && c.xg_fuse;
    for (int i = 0; ok && i < s0.nops; ++i) {
        const BcOp& op = s0.op[i];
        if (op.field < 0 || op.field > 2 || (mask >> op.field & 1) || op.side >= 0) { ok = false; break; }
        switch (op.kind) {
            case BC_NEG: case BC_LIN2M: xg[op.field] = -1.f; break;
            case BC_COPY: xg[op.field] = 1.f; break;
            case BC_ZERO: case BC_LIN: xg[op.field] = 0.f; break;
            default: ok = false;
        }
        mask |= 1 << op.field;
    }
    if (ok && mask) {
        c.xg_mask = mask;
        for (int i = 0; i < 3; ++i) c.xg[i] = xg[i];
    }
    return SPH_OK;
}

// the ghost-velocity stages of the BC set (Julia reference order), in c.bc; a
// shorter equivalent program for the launches goes to c.bc_run where one exists
int build_bc_program(Ctx& c) {
    const sph_params& q = c.prm;
    c.bc.clear();
    c.bc_run.clear();
    const double rsh = q.r * q.sh;
    if (q.bc == SPH_BC_FREE_SLIP) {  // SphericalStokes_plateau.jl:64-92
        c.bc.push_back(stage(0, {op(0, BC_NEG), op(1, BC_COPY), op(2, BC_COPY)}));
        c.bc.push_back(stage(1, {op(0, BC_COPY), op(1, BC_NEG), op(2, BC_COPY)}));
        c.bc.push_back(stage(2, {op(0, BC_COPY), op(1, BC_COPY), op(2, BC_NEG)}));
        return SPH_OK;
    }
    if (q.bc == SPH_BC_STRESS) {
        if (q.geometry == SPH_GEOM_CARTESIAN) return fail(SPH_ERR_UNSUPPORTED, "SPH_BC_STRESS needs a deviatoric (spherical or cylindrical) scheme");
        c.bc.push_back(stage(0, {op(0, BC_NEG), op(1, BC_COPY), op(2, BC_COPY)}));
        c.bc.push_back(stage(1, {op(0, BC_COPY), op(2, BC_COPY)}));
        c.bc.push_back(stage(1, {op(1, BC_STRESS)}));
        c.bc.push_back(stage(2, {op(0, BC_COPY), op(1, BC_COPY)}));
        c.bc.push_back(stage(2, {op(2, BC_STRESS)}));
        // the launched program: each copy stage merged with the stress stage after it,
        // whose op then reads the copies' sources (same values, three launches)
        c.bc_run.clear();
        c.bc_run.push_back(c.bc[0]);
        c.bc_run.push_back(stage(1, {op(0, BC_COPY), op(2, BC_COPY), op(1, BC_STRESS_SRC)}));
        c.bc_run.push_back(stage(2, {op(0, BC_COPY), op(1, BC_COPY), op(2, BC_STRESS_SRC)}));
        return SPH_OK;
    }
    if (q.bc == SPH_BC_FREE_SURFACE) {  // free slip but at the top x1 face; its ghost after the copies
        if (q.geometry != SPH_GEOM_SPHERICAL) return fail(SPH_ERR_UNSUPPORTED, "SPH_BC_FREE_SURFACE is spherical only");
        c.bc.push_back(stage(0, {op(0, BC_NEG, 0, 0.0, 0.0, 0), op(1, BC_COPY), op(2, BC_COPY)}));
        c.bc.push_back(stage(0, {op(0, BC_STRESS, 0, 0.0, 0.0, 1)}));
        c.bc.push_back(stage(1, {op(0, BC_COPY), op(1, BC_NEG), op(2, BC_COPY)}));
        c.bc.push_back(stage(2, {op(0, BC_COPY), op(1, BC_COPY), op(2, BC_NEG)}));
        return SPH_OK;
    }
    if (q.bc != SPH_BC_DIAPIR) return fail(SPH_ERR_INVALID, "unknown bc");
    switch (q.geometry) {
        case SPH_GEOM_SPHERICAL:  // SphericalStokes_diapir.jl:61-99
            c.bc.push_back(stage(0, {op(0, BC_NEG), op(1, BC_COPY), op(2, BC_COPY)}));
            c.bc.push_back(stage(1, {op(0, BC_ZERO), op(1, BC_NEG), op(2, BC_LIN, 1, rsh, kPi / 2.0)}));
            c.bc.push_back(stage(2, {op(0, BC_ZERO), op(1, BC_ZERO), op(2, BC_LIN2M, 1, rsh, kPi / 2.0)}));
            break;
        case SPH_GEOM_CYLINDRICAL:  // CylindricalStokes_diapir.jl:358-366
            c.bc.push_back(stage(0, {op(2, BC_COPY), op(1, BC_COPY), op(0, BC_NEG)}));
            c.bc.push_back(stage(1, {op(2, BC_LIN, 1, rsh, 0.0), op(0, BC_ZERO), op(1, BC_NEG)}));
            c.bc.push_back(stage(2, {op(1, BC_ZERO), op(0, BC_ZERO), op(2, BC_LIN2M, 1, rsh, 0.0)}));
            break;
        case SPH_GEOM_CARTESIAN:  // CartesianStokes_diapir.jl:371-379
            c.bc.push_back(stage(0, {op(0, BC_LIN2M, 1, q.sh, 0.0), op(1, BC_ZERO), op(2, BC_ZERO)}));
            c.bc.push_back(stage(1, {op(0, BC_LIN, 1, q.sh, 0.0), op(1, BC_NEG), op(2, BC_ZERO)}));
            c.bc.push_back(stage(2, {op(0, BC_COPY), op(1, BC_COPY), op(2, BC_NEG)}));
            break;
        default: return fail(SPH_ERR_INVALID, "unknown geometry");
    }
    return SPH_OK;
}

template <typename T, int G>
void launch_bc(Ctx& c, KP<T>& p, int homog, int first = 0) {
    for (size_t i = first; i < c.bc_run.size(); ++i) {
        const BcStage& st = c.bc_run[i];
        int eu = st.dim == 0 ? c.d.n2 + 1 : c.d.n1 + 1;
        int ev = st.dim == 2 ? c.d.n2 + 1 : c.d.n3 + 1;
        dim3 g((eu + 31) / 32, (ev + 7) / 8, 1);
        launch_pdl(c.use_pdl, k_bc<T, G>, g, blk2d(), 0, c.stream, p, st, homog);
    }
}

// ---------------------------------------------------------------------------
// allocation and set-up
template <typename T>
int alloc_state(Ctx& c, State<T>& s) {
    const long long vol = c.d.vol;
    CK(cudaMalloc((void**)&s.slab, sizeof(T) * vol * F_NSLOTS));
    CK(cudaMemsetAsync(s.slab, 0, sizeof(T) * vol * F_NSLOTS, c.stream));
    for (int i = 0; i < F_NSLOTS; ++i) s.f[i] = s.slab + (long long)i * vol;
    // tables: invRc[n1] invRh[n1] invSinC[n2] invSinH[n2] cotC[n2] cotH[n2] x1c[n1] x2c[n2] x3c[n3]
    const int n1 = c.d.n1, n2 = c.d.n2, n3 = c.d.n3;
    size_t nt = 3 * (size_t)n1 + 4 * (size_t)n2 + (size_t)n2 + (size_t)n3;
    std::vector<T> h(nt, T(1));
    T* w = h.data();
    T* invRc = w; w += n1;
    T* invRh = w; w += n1;
    T* invSinC = w; w += n2;
    T* invSinH = w; w += n2;
    T* cotC = w; w += n2;
    T* cotH = w; w += n2;
    T* x1c = w; w += n1;
    T* x2c = w; w += n2;
    T* x3c = w; w += n3;
    for (int i = 0; i < n1; ++i) {
        x1c[i] = T(c.hx1[i]);
        invRc[i] = T(1.0 / c.hx1[i]);
        if (i < n1 - 1) invRh[i] = T(1.0 / (0.5 * (c.hx1[i] + c.hx1[i + 1])));
    }
    for (int j = 0; j < n2; ++j) {
        x2c[j] = T(c.hx2[j]);
        invSinC[j] = T(1.0 / std::sin(c.hx2[j]));
        cotC[j] = T(1.0 / std::tan(c.hx2[j]));
        if (j < n2 - 1) {
            double th = 0.5 * (c.hx2[j] + c.hx2[j + 1]);
            invSinH[j] = T(1.0 / std::sin(th));
            cotH[j] = T(1.0 / std::tan(th));
        }
    }
    for (int k = 0; k < n3; ++k) x3c[k] = T(c.hx3[k]);
    CK(cudaMalloc((void**)&s.tab, sizeof(T) * nt));
    CK(cudaMemcpyAsync(s.tab, h.data(), sizeof(T) * nt, cudaMemcpyHostToDevice, c.stream));
    T* t = s.tab;
    s.geo.invRc = t; t += n1;
    s.geo.invRh = t; t += n1;
    s.geo.invSinC = t; t += n2;
    s.geo.invSinH = t; t += n2;
    s.geo.cotC = t; t += n2;
    s.geo.cotH = t; t += n2;
    s.geo.x1c = t; t += n1;
    s.geo.x2c = t; t += n2;
    s.geo.x3c = t; t += n3;
    CK(cudaStreamSynchronize(c.stream));
    return SPH_OK;
}

template <typename T>
void free_state(State<T>& s) {
    if (s.slab) cudaFree(s.slab);
    if (s.tab) cudaFree(s.tab);
    s.slab = nullptr; s.tab = nullptr;
}

std::vector<double> linspace(double c, double l, int n) {
    // node coordinates spanning c - l/2 .. c + l/2 (Julia range(a, b, length=n))
    std::vector<double> x(n);
    const double lo = c - l / 2.0, hi = c + l / 2.0;
    for (int i = 0; i < n; ++i) x[i] = (i == n - 1) ? hi : lo + (hi - lo) * (double)i / (double)(n - 1);
    return x;
}

// host-side initial fields in the box layout (initialize_inclusion!, initialize_velocity!)
int init_fields(Ctx& c) {
    const sph_params& q = c.prm;
    const Dims& d = c.d;
    const long long vol = d.vol;
    std::vector<double> rho(vol, 0.0), eta(vol, 0.0), V(vol, 0.0);
    std::vector<uint8_t> ph(vol, 0);
    for (int k = 0; k < d.n3; ++k)
        for (int j = 0; j < d.n2; ++j)
            for (int i = 0; i < d.n1; ++i) {
                long long ci = i + (long long)d.sy * j + (long long)d.sz * k;
                rho[ci] = q.rho0;
                eta[ci] = q.eta0;
                if (q.init == SPH_INIT_INCLUSION) {
                    double x = c.hx1[i], y = c.hx2[j], z = c.hx3[k], r2;
                    if (q.geometry == SPH_GEOM_SPHERICAL)
                        r2 = (x - q.r) * (x - q.r) + ((y - kPi / 2.0) * q.r) * ((y - kPi / 2.0) * q.r) + (z * q.r) * (z * q.r);
                    else if (q.geometry == SPH_GEOM_CYLINDRICAL)
                        r2 = (x - q.r) * (x - q.r) + (y * q.r) * (y * q.r) + z * z;
                    else
                        r2 = x * x + y * y + z * z;
                    if (r2 < q.radius) {
                        rho[ci] = q.rho_in;
                        eta[ci] = q.eta0 / q.vr;
                        ph[ci] = q.incl_linear ? 1 : 0;
                    }
                }
            }
    State<double>& s = c.s64;
    CK(cudaMemcpyAsync(s.f[F_RHO], rho.data(), sizeof(double) * vol, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.f[F_ETA], eta.data(), sizeof(double) * vol, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.f[F_ETA_INI], eta.data(), sizeof(double) * vol, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(s.f[F_ETA_PL], eta.data(), sizeof(double) * vol, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phase, ph.data(), vol, cudaMemcpyHostToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (q.init == SPH_INIT_INCLUSION) {
        int vf = F_V3;
        if (q.geometry == SPH_GEOM_SPHERICAL) {  // Vφ = (θ - π/2) r sh everywhere
            for (int k = 0; k <= d.n3; ++k)
                for (int j = 0; j < d.n2; ++j)
                    for (int i = 0; i < d.n1; ++i) V[i + (long long)d.sy * j + (long long)d.sz * k] = (c.hx2[j] - kPi / 2.0) * q.r * q.sh;
        } else if (q.geometry == SPH_GEOM_CYLINDRICAL) {  // VZ = θ r sh on the θ and z faces
            for (int k = 0; k <= d.n3; ++k)
                for (int j = 0; j < d.n2; ++j)
                    for (int i = 0; i < d.n1; ++i)
                        if (j == 0 || j == d.n2 - 1 || k == 0 || k == d.n3) V[i + (long long)d.sy * j + (long long)d.sz * k] = c.hx2[j] * q.r * q.sh;
        } else {  // VX = Y sh everywhere
            vf = F_V1;
            for (int k = 0; k < d.n3; ++k)
                for (int j = 0; j < d.n2; ++j)
                    for (int i = 0; i <= d.n1; ++i) V[i + (long long)d.sy * j + (long long)d.sz * k] = c.hx2[j] * q.sh;
        }
        CK(cudaMemcpyAsync(s.f[vf], V.data(), sizeof(double) * vol, cudaMemcpyHostToDevice, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    }
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// precision bookkeeping: the FP64 state is the master copy for the ABI
int sync32(Ctx& c) {
    if (!c.has32 || !c.stale32) return SPH_OK;
    const long long vol = c.d.vol;
    const int slots[] = {F_P, F_V1, F_V2, F_V3, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23, F_ETA, F_ETA_INI, F_ETA_SM, F_DT_R, F_TII, F_RHO, F_ETA_PL, F_LOAD};
    for (int sl : slots) k_convert<float, double><<<ew_blocks(vol), 256, 0, c.stream>>>(c.s32.f[sl], c.s64.f[sl], vol);
    CK(cudaGetLastError());
    c.stale32 = false;
    return SPH_OK;
}
int sync64(Ctx& c) {
    if (!c.stale64) return SPH_OK;
    const long long vol = c.d.vol;
    const int slots[] = {F_P, F_V1, F_V2, F_V3, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23, F_ETA, F_ETA_SM, F_DT_R, F_TII, F_ETA_PL};
    for (int sl : slots) k_convert<double, float><<<ew_blocks(vol), 256, 0, c.stream>>>(c.s64.f[sl], c.s32.f[sl], vol);
    CK(cudaGetLastError());
    c.stale64 = false;
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// one reference PT iteration on state s
// ηSM: `etasm_passes` applications of the 7-point max filter (maxloc! + copy_BC!);
// intermediate passes go through the η_out scratch field, the last one into ηSM
template <typename T, int G>
void launch_maxloc(Ctx& c, KP<T>& p) {
    const int passes = c.prm.etasm_passes > 1 ? c.prm.etasm_passes : 1;
    KP<T> q = p;
    T* src = p.eta;
    for (int i = 0; i < passes; ++i) {
        const bool last = i == passes - 1;
        T* dst = last ? p.etaSM : (((passes - 1 - i) & 1) ? p.eta_out : p.etaSM);
        q.eta = src;
        q.etaSM = dst;
        k_maxloc<T><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(q, G == CART);
        src = dst;
    }
}

template <typename T, int G>
void launch_rheology(Ctx& c, State<T>& s, KP<T>& p) {
    const int rh = c.prm.rheology;
    const int faces_only = (G == CART);
    if (rh == SPH_RHEO_TAU_POWER) {
        k_rheo_tau<T, 0><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p, faces_only, T(c.cur_n));
    } else if (rh == SPH_RHEO_TAU_POWER_RELAX) {
        if (c.cur_n > 1.0) k_rheo_tau<T, 1><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p, faces_only, T(c.cur_n));
    } else if (rh == SPH_RHEO_EDOT_POWER_RELAX) {
        k_strain<T, G><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
        k_edot_law<T, true><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
        std::swap(s.f[F_ETA], s.f[F_ETA_OUT]);
        p.eta = s.f[F_ETA]; p.eta_out = s.f[F_ETA_OUT];
    }
}

template <typename T, int G>
void iterate_one(Ctx& c, State<T>& s) {
    KP<T> p = make_kp<T>(c, s);
    launch_maxloc<T, G>(c, p);
    k_stress<T, G, false><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
    launch_rheology<T, G>(c, s, p);
    k_velocity<T, G, 0><<<grid_vel(c.d), blk2d(), 0, c.stream>>>(p);
    launch_bc<T, G>(c, p, 0);
}

// the fused FP32 sweep: new state into the second buffer set, then swap sets
void swap_state(State<float>& s) {
    const int a[10] = {F_P, F_V1, F_V2, F_V3, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23};
    const int b[10] = {F_A_P, F_A_V1, F_A_V2, F_A_V3, F_A_T11, F_A_T22, F_A_T33, F_A_T12, F_A_T13, F_A_T23};
    for (int i = 0; i < 10; ++i) std::swap(s.f[a[i]], s.f[b[i]]);
}

// x3 chunk lengths picked by sph_autotune, per (geometry, n1, n2, n3), shared by every context
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int> g_tuned_chunk;

// x3 chunk length of the fused sweep.  Each block marches over one chunk of
// planes and pays about two planes more than it owns (the halo plane below the
// chunk and the pipeline fill), while the hardware scheduler balances the SMs
// only to within one block at the end of the launch.  The time model
// (k + 2.5) * (blocks / slots + 0.7), slots = resident blocks on the device, picks
// the chunk among 4..24 planes.  Measured on a GB300, its pick is the fastest
// chunk at 63^3 and within 1 % of it at 255^3 and 5 % at 127^3, where wave
// quantisation makes the ranking irregular (sph_autotune measures instead).
int fused_chunk(const Ctx& c) {
    if (c.fused_chunk > 0) return c.fused_chunk;
    const double xy = (double)((c.d.n1 + FTX - 1) / FTX) * ((c.d.n2 + FTY - 1) / FTY);
    const double slots = c.fused_slots > 0 ? c.fused_slots : 456.0;
    int best = 4;
    double best_t = 1e300;
    for (int k : {4, 6, 8, 12, 16, 24}) {
        const double blocks = xy * ((c.d.n3 + k - 1) / k);
        const double t = (k + 2.5) * (blocks / slots + 0.7);
        if (t < best_t) { best_t = t; best = k; }
        if (k >= c.d.n3) break;
    }
    return best;
}

template <int G, int MODE>
void set_tma_attr() {
    cudaFuncSetAttribute(k_fused_tma<G, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_tma_smem_bytes());
}

template <int G, int MODE>
void set_fused_attr() {
    cudaFuncSetAttribute(k_fused<G, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_smem_bytes());
}
int set_fused_attrs() {
    set_fused_attr<SPH, 0>(); set_fused_attr<SPH, 1>();
    set_fused_attr<CYL, 0>(); set_fused_attr<CYL, 1>();
    set_fused_attr<CART, 0>(); set_fused_attr<CART, 1>();
    set_tma_attr<SPH, 1>(); set_tma_attr<CYL, 1>(); set_tma_attr<CART, 1>();
    cudaFuncSetAttribute(k_fused_tma_batch<SPH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_tma_smem_bytes());
    cudaFuncSetAttribute(k_fused_tma_batch<CYL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_tma_smem_bytes());
    cudaFuncSetAttribute(k_fused_tma_batch<CART>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_tma_smem_bytes());
    cudaFuncSetAttribute(k_sweep_x2<SPH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_x2_smem_bytes());
    cudaFuncSetAttribute(k_sweep_x2<CYL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_x2_smem_bytes());
    cudaFuncSetAttribute(k_sweep_x2<CART>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_x2_smem_bytes());
    CK(cudaGetLastError());
    return SPH_OK;
}

template <int G, int MODE>
void launch_fused(Ctx& c, KP<float>& p, State<float>& s) {
    FusedOut<float> o;
    o.P = s.f[F_A_P]; o.V1 = s.f[F_A_V1]; o.V2 = s.f[F_A_V2]; o.V3 = s.f[F_A_V3];
    o.t11 = s.f[F_A_T11]; o.t22 = s.f[F_A_T22]; o.t33 = s.f[F_A_T33]; o.t12 = s.f[F_A_T12]; o.t13 = s.f[F_A_T13]; o.t23 = s.f[F_A_T23];
    const int kc = fused_chunk(c);
    dim3 grid((c.d.n1 + FTX - 1) / FTX, (c.d.n2 + FTY - 1) / FTY, (c.d.n3 + kc - 1) / kc);
    k_fused<G, MODE><<<grid, dim3(FNT, 1, 1), fused_smem_bytes(), c.stream>>>(p, o, kc);
}

// one reference iteration with the fused sweep (FP32)
template <int G>
void iterate_fused(Ctx& c, State<float>& s) {
    KP<float> p = make_kp<float>(c, s);
    launch_maxloc<float, G>(c, p);
    launch_fused<G, 0>(c, p, s);
    swap_state(s);
    KP<float> q = make_kp<float>(c, s);
    if (c.prm.rheology == SPH_RHEO_EDOT_POWER_RELAX) {
        // the law uses the velocities the stress update used (the previous set)
        KP<float> r = q;
        r.V1 = s.f[F_A_V1]; r.V2 = s.f[F_A_V2]; r.V3 = s.f[F_A_V3];
        launch_rheology<float, G>(c, s, r);
        q.eta = s.f[F_ETA]; q.eta_out = s.f[F_ETA_OUT];
    } else {
        launch_rheology<float, G>(c, s, q);
    }
    launch_bc<float, G>(c, q, 0);
}

template <typename T>
void iterate_dispatch(Ctx& c, State<T>& s) {
    switch (c.prm.geometry) {
        case SPH_GEOM_SPHERICAL: iterate_one<T, SPH>(c, s); break;
        case SPH_GEOM_CYLINDRICAL: iterate_one<T, CYL>(c, s); break;
        default: iterate_one<T, CART>(c, s); break;
    }
}
template <>
void iterate_dispatch<float>(Ctx& c, State<float>& s) {
    if (c.fused) {
        switch (c.prm.geometry) {
            case SPH_GEOM_SPHERICAL: iterate_fused<SPH>(c, s); break;
            case SPH_GEOM_CYLINDRICAL: iterate_fused<CYL>(c, s); break;
            default: iterate_fused<CART>(c, s); break;
        }
        return;
    }
    switch (c.prm.geometry) {
        case SPH_GEOM_SPHERICAL: iterate_one<float, SPH>(c, s); break;
        case SPH_GEOM_CYLINDRICAL: iterate_one<float, CYL>(c, s); break;
        default: iterate_one<float, CART>(c, s); break;
    }
}

// ---------------------------------------------------------------------------
// reductions
template <typename T>
void launch_maxabs(Ctx& c, const T* a, const T* b, int slot) {
    k_maxabs<T><<<ew_blocks(c.d.vol), 256, 0, c.stream>>>(a, b, c.d.vol, c.red + slot);
}
inline double slot_val(Ctx& c, int i) {
    double v;
    std::memcpy(&v, &c.hred[i], sizeof(double));
    return v;
}
int fetch_red(Ctx& c) {
    CK(cudaMemcpyAsync(c.hred, c.red, sizeof(unsigned long long) * kRedSlots, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return SPH_OK;
}

// relative velocity change of the last iteration (the reference's err)
template <typename T>
int ref_err(Ctx& c, State<T>& s, double* err, bool skip_nan_v3) {
    CK(cudaMemsetAsync(c.red, 0, sizeof(unsigned long long) * kRedSlots, c.stream));
    launch_maxabs<T>(c, s.f[F_V1], s.f[F_V1E], 0);
    launch_maxabs<T>(c, s.f[F_V2], s.f[F_V2E], 1);
    launch_maxabs<T>(c, s.f[F_V3], s.f[F_V3E], 2);
    launch_maxabs<T>(c, s.f[F_V1], nullptr, 3);
    launch_maxabs<T>(c, s.f[F_V2], nullptr, 4);
    launch_maxabs<T>(c, s.f[F_V3], nullptr, 5);
    CK(cudaGetLastError());
    int rc = fetch_red(c);
    if (rc) return rc;
    double e = 0.0;
    for (int f = 0; f < 3; ++f) {
        double dv = slot_val(c, f), vv = slot_val(c, 3 + f);
        double r = dv / vv;
        if (!(r == r) && skip_nan_v3 && f == 2) continue;
        if (!(r == r)) { e = r; break; }
        e = std::max(e, r);
    }
    *err = e;
    return SPH_OK;
}

template <typename T>
int snapshot(Ctx& c, State<T>& s) {
    const size_t b = sizeof(T) * c.d.vol;
    CK(cudaMemcpyAsync(s.f[F_V1E], s.f[F_V1], b, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(s.f[F_V2E], s.f[F_V2], b, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(s.f[F_V3E], s.f[F_V3], b, cudaMemcpyDeviceToDevice, c.stream));
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// FP64 residual of the FP64 state (see sph_residual in sphstokes.h)
template <int G>
int residual64_g(Ctx& c, double out[7], bool eta_from_law) {
    State<double>& s = c.s64;
    KP<double> p = make_kp<double>(c, s);
    const double* eta_eff = s.f[F_ETA];
    if (eta_from_law) {
        k_strain<double, G><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
        k_edot_law<double, false><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
        eta_eff = s.f[F_ETA_OUT];
    }
    KP<double> r = p;
    r.eta = const_cast<double*>(eta_eff);
    r.t11 = s.f[F_Q11]; r.t22 = s.f[F_Q22]; r.t33 = s.f[F_Q33]; r.t12 = s.f[F_Q12]; r.t13 = s.f[F_Q13]; r.t23 = s.f[F_Q23];
    k_tau_visc<double, G><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(r);
    if (r.traction || r.fs) {
        k_traction_pressure<double><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(r, s.f[F_PRES]);
        r.P = s.f[F_PRES];
    }
    k_velocity<double, G, 2><<<grid_vel(c.d), blk2d(), 0, c.stream>>>(r);
    CK(cudaMemsetAsync(c.red, 0, sizeof(unsigned long long) * kRedSlots, c.stream));
    launch_maxabs<double>(c, s.f[F_RV1], nullptr, 0);
    launch_maxabs<double>(c, s.f[F_RV2], nullptr, 1);
    launch_maxabs<double>(c, s.f[F_RV3], nullptr, 2);
    launch_maxabs<double>(c, s.f[F_RP], nullptr, 3);
    launch_maxabs<double>(c, s.f[F_V1], nullptr, 4);
    launch_maxabs<double>(c, s.f[F_V2], nullptr, 5);
    launch_maxabs<double>(c, s.f[F_V3], nullptr, 6);
    CK(cudaGetLastError());
    int rc = fetch_red(c);
    if (rc) return rc;
    for (int i = 0; i < 4; ++i) out[i] = slot_val(c, i);
    out[4] = std::max(slot_val(c, 4), std::max(slot_val(c, 5), slot_val(c, 6)));
    out[5] = c.f_scale;
    const double mom = std::max(out[0], std::max(out[1], out[2])) / c.f_scale;
    const double vs = out[4] > 0.0 ? out[4] : 1.0;
    const double cont = out[3] * c.prm.l1 / vs;
    out[6] = (mom != mom || cont != cont) ? NAN : std::max(mom, cont);
    return SPH_OK;
}

int residual64(Ctx& c, double out[7]) {
    const bool law = c.prm.rheology == SPH_RHEO_EDOT_POWER_RELAX;
    switch (c.prm.geometry) {
        case SPH_GEOM_SPHERICAL: return residual64_g<SPH>(c, out, law);
        case SPH_GEOM_CYLINDRICAL: return residual64_g<CYL>(c, out, law);
        default: return residual64_g<CART>(c, out, law);
    }
}

int compute_f_scale(Ctx& c) {
    CK(cudaMemsetAsync(c.red, 0, sizeof(unsigned long long) * kRedSlots, c.stream));
    launch_maxabs<double>(c, c.s64.f[F_RHO], nullptr, 0);
    int rc = fetch_red(c);
    if (rc) return rc;
    const sph_params& q = c.prm;
    double f = slot_val(c, 0) * std::fabs(q.g);
    if (q.bc == SPH_BC_STRESS) f = std::max(f, std::max(std::fabs(q.sig_bc[1]), std::fabs(q.sig_bc[2])) / q.l1);
    if (q.bc == SPH_BC_FREE_SURFACE) {  // the surface load's force scale, max|q| / l1
        CK(cudaMemsetAsync(c.red, 0, sizeof(unsigned long long) * kRedSlots, c.stream));
        launch_maxabs<double>(c, c.s64.f[F_LOAD], nullptr, 0);
        if ((rc = fetch_red(c))) return rc;
        f = std::max(f, slot_val(c, 0) / q.l1);
    }
    c.f_scale = f > 0.0 ? f : 1.0;
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// host <-> device copies of one field: one contiguous transfer of the dense field
// (the reference layout, e0 x e1 x e2 doubles) to or from a staging buffer, and a
// re-pitching kernel between the staging buffer and the padded box, so the copy engine
// moves a single large block instead of e1*e2 short rows
int ensure_stage(Ctx& c) {
    if (c.stage) return SPH_OK;
    if (cudaMalloc((void**)&c.stage, sizeof(double) * c.d.vol) != cudaSuccess) {
        cudaGetLastError();
        return fail(SPH_ERR_NOMEM, "staging buffer of the host copies");
    }
    return SPH_OK;
}
inline dim3 pack_grid(const int e[3]) { return dim3((e[0] + 127) / 128, e[1], e[2]); }

// host (dense doubles) -> box (converted to T); returns after the host buffer has been read
template <typename T>
int upload_box(Ctx& c, T* box, const int e[3], const double* host) {
    int rc = ensure_stage(c);
    if (rc) return rc;
    const size_t n = (size_t)e[0] * e[1] * e[2];
    CK(cudaMemcpyAsync(c.stage, host, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    k_unpack<T><<<pack_grid(e), 128, 0, c.stream>>>(box, c.stage, e[0], e[1], c.d.sy, c.d.sz);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c.stream));
    return SPH_OK;
}
// box (T) -> host (dense doubles); returns after the host buffer is written
template <typename T>
int download_box(Ctx& c, const T* box, const int e[3], double* host) {
    int rc = ensure_stage(c);
    if (rc) return rc;
    const size_t n = (size_t)e[0] * e[1] * e[2];
    k_pack<T><<<pack_grid(e), 128, 0, c.stream>>>(c.stage, box, e[0], e[1], c.d.sy, c.d.sz);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host, c.stage, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// plain PT solve (FP64 or FP32 state)
template <typename T>
int solve_plain(Ctx& c, State<T>& s, bool is32, const sph_solve_opts& o, sph_solve_info* info, int64_t* hi, double* he, int64_t cap) {
    const int nout = o.nout > 0 ? o.nout : 100;
    int64_t it = 0;
    double err = 1.0;
    int status = SPH_ERR_NOT_CONVERGED;
    const bool ref = o.criterion == SPH_CRIT_REFERENCE || o.criterion == SPH_CRIT_REFERENCE_PLATEAU;
    while (it < o.maxiter) {
        ++it;
        const bool check = (it % nout) == 0;
        if (check && ref) {
            int rc = snapshot<T>(c, s);
            if (rc) return rc;
        }
        iterate_dispatch<T>(c, s);
        if (!check) continue;
        CK(cudaGetLastError());
        if (ref) {
            int rc = ref_err<T>(c, s, &err, o.criterion == SPH_CRIT_REFERENCE_PLATEAU);
            if (rc) return rc;
        } else {
            if (is32) { c.stale64 = true; int rc = sync64(c); if (rc) return rc; }
            double out[7];
            int rc = residual64(c, out);
            if (rc) return rc;
            err = out[6];
        }
        if (info && info->nhist < cap) {
            if (hi) hi[info->nhist] = it;
            if (he) he[info->nhist] = err;
            info->nhist++;
            c.hist_ms.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - c.solve_t0).count());
        }
        if (!(err == err) || std::isinf(err)) { status = SPH_ERR_DIVERGED; break; }
        if (c.prm.switch_err > 0.0 && err < c.prm.switch_err) c.cur_n = c.prm.n_exp_late;
        if (err < o.tol && (!ref || it > 20)) { status = SPH_OK; break; }
    }
    if (info) { info->iters = it; info->err = err; info->status = status; }
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// mixed precision: FP32 PT sweeps on the correction problem inside an FP64
// defect-correction loop.
//   r_V = momentum residual of (V, P) with η = η_eff(V) (FP64), r_P = div V (FP64)
//   inner: PT on (δV, δP, δτ) with η frozen at η_eff, homogeneous BCs,
//          δP -= KBDT (div δV + r_P), δV += DT_R (div(-δP + δτ) + r_V)
//   V += δV, P += δP (FP64)
// FP64 viscosity η_eff(V), the full BC program and the residual of the FP64 state
template <int G>
int outer_residual(Ctx& c, double out[7]) {
    State<double>& s = c.s64;
    KP<double> p = make_kp<double>(c, s);
    const long long vol = c.d.vol;
    if (c.prm.rheology == SPH_RHEO_EDOT_POWER_RELAX) {
        k_strain<double, G><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
        k_edot_law<double, false><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(p);
        CK(cudaMemcpyAsync(s.f[F_ETA], s.f[F_ETA_OUT], sizeof(double) * vol, cudaMemcpyDeviceToDevice, c.stream));
    }
    launch_bc<double, G>(c, p, 0);
    return residual64_g<G>(c, out, false);
}

// freeze η_eff, ηSM and the FP64 residual into the FP32 correction problem, zero δ
template <int G>
int prepare_correction(Ctx& c, const double out[7]) {
    State<double>& s = c.s64;
    State<float>& t = c.s32;
    const long long vol = c.d.vol;
    k_convert<float, double><<<ew_blocks(vol), 256, 0, c.stream>>>(t.f[F_ETA], s.f[F_ETA], vol);
    k_convert<float, double><<<ew_blocks(vol), 256, 0, c.stream>>>(t.f[F_RV1], s.f[F_RV1], vol);
    k_convert<float, double><<<ew_blocks(vol), 256, 0, c.stream>>>(t.f[F_RV2], s.f[F_RV2], vol);
    k_convert<float, double><<<ew_blocks(vol), 256, 0, c.stream>>>(t.f[F_RV3], s.f[F_RV3], vol);
    k_convert<float, double><<<ew_blocks(vol), 256, 0, c.stream>>>(t.f[F_RP], s.f[F_RP], vol);
    const int zero[] = {F_P, F_V1, F_V2, F_V3, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23,
                        F_A_P, F_A_V1, F_A_V2, F_A_V3, F_A_T11, F_A_T22, F_A_T33, F_A_T12, F_A_T13, F_A_T23};
    for (int z : zero) CK(cudaMemsetAsync(t.f[z], 0, sizeof(float) * vol, c.stream));
    KP<float> q = make_kp<float>(c, t);
    launch_maxloc<float, G>(c, q);
    CK(cudaGetLastError());
    c.corr_r0 = std::max(out[0], std::max(out[1], out[2]));
    c.corr_ready = true;
    c.stale32 = true;  // the FP32 state no longer mirrors the FP64 state
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// TMA tensor maps over the padded box of FP32 fields
PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {  // looked up once, thread-safe
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

bool encode_map(const Ctx& c, CUtensorMap* m, const float* base, unsigned bx, unsigned by) {
    auto enc = tma_encoder();
    if (!enc) return false;
    cuuint64_t gdim[3] = {(cuuint64_t)c.d.px, (cuuint64_t)c.d.py, (cuuint64_t)c.d.pz};
    cuuint64_t gstr[2] = {(cuuint64_t)c.d.px * 4, (cuuint64_t)c.d.px * c.d.py * 4};
    cuuint32_t box[3] = {bx, by, 1};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), gdim, gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// maps of the current buffer arrangement; returns the device pointer of the set or nullptr
const CUtensorMap* tma_maps(Ctx& c) {
    if (!c.use_tma) return nullptr;
    State<float>& t = c.s32;
    for (int i = 0; i < 2; ++i)
        if (c.map_key[i] == t.f[F_V1]) return c.d_maps + i * TM_COUNT;
    if (!c.d_maps) {
        if (cudaMalloc((void**)&c.d_maps, sizeof(CUtensorMap) * 2 * TM_COUNT) != cudaSuccess) { c.use_tma = false; return nullptr; }
    }
    if (!c.d_err) {
        if (cudaMalloc((void**)&c.d_err, sizeof(int)) != cudaSuccess) { c.use_tma = false; return nullptr; }
        cudaMemsetAsync(c.d_err, 0, sizeof(int), c.stream);
    }
    const int slot = c.map_key[0] ? 1 : 0;
    CUtensorMap h[TM_COUNT];
    const int in_f[5] = {F_V1, F_V2, F_V3, F_ETA, F_ETA_SM};
    const int old_f[7] = {F_P, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23};
    bool ok = true;
    for (int i = 0; i < 5; ++i) ok &= encode_map(c, &h[TM_V1 + i], t.f[in_f[i]], TIN_X, TIN_Y);
    for (int i = 0; i < 7; ++i) ok &= encode_map(c, &h[TM_P + i], t.f[old_f[i]], TOLD_X, TOLD_Y);
    ok &= encode_map(c, &h[TM_RP], t.f[F_RP], TOLD_X, TOLD_Y);
    ok &= encode_map(c, &h[TM_RHO], t.f[F_RHO], TOLD_X, TOLD_Y);
    ok &= encode_map(c, &h[TM_RV1], t.f[F_RV1], FTX, FTY);
    ok &= encode_map(c, &h[TM_RV2], t.f[F_RV2], FTX, FTY);
    ok &= encode_map(c, &h[TM_RV3], t.f[F_RV3], FTX, FTY);
    if (!ok || cudaMemcpy(c.d_maps + slot * TM_COUNT, h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess) {
        c.use_tma = false;
        return nullptr;
    }
    c.map_key[slot] = t.f[F_V1];
    return c.d_maps + slot * TM_COUNT;
}

// build the tensor-map sets of both ping-pong arrangements (never inside a graph capture)
void ensure_tma_maps(Ctx& c) {
    if (!c.use_tma || !c.fused) return;
    tma_maps(c);
    swap_state(c.s32);
    tma_maps(c);
    swap_state(c.s32);
}

// The error word of the TMA sweep kernels: set when a bounded wait on a copy barrier ran
// out.  The kernel then stopped issuing copies and finished its march on whatever its
// tiles held, so the FP32 state is suspect and copies may have been in flight when its
// blocks exited: the context is marked unusable (every later call that would launch work
// on it fails) and the caller destroys it.
int check_kernel_flag(Ctx& c) {
    if (!c.d_err) return SPH_OK;
    int h = 0;
    CK(cudaMemcpyAsync(&h, c.d_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (h) {
        c.broken = true;
        return fail(SPH_ERR_CUDA, "a bounded wait on a TMA barrier ran out in the fused sweep; the context is unusable");
    }
    return SPH_OK;
}

// SPH_OK, or the failure every entry point that launches work returns on a context
// marked unusable by check_kernel_flag
int usable(const Ctx& c) {
    if (c.broken) return fail(SPH_ERR_CUDA, "context unusable: a bounded wait of a sweep kernel ran out earlier; destroy it");
    return SPH_OK;
}

// KP of the correction problem: homogeneous boundary data
KP<float> make_kp_corr(Ctx& c) {
    KP<float> q = make_kp<float>(c, c.s32);
    q.sig2 = 0.f;
    q.top_load = nullptr;
    q.sig3 = 0.f;
    return q;
}

// one FP32 sweep of the correction problem (fused or one kernel per step) + homogeneous BCs
template <int G>
void correction_sweep(Ctx& c) {
    State<float>& t = c.s32;
    KP<float> q = make_kp_corr(c);
    int first_bc = 0;
    if (c.fused) {
        const CUtensorMap* maps = tma_maps(c);
        if (maps) {
            FusedOut<float> o;
            o.P = t.f[F_A_P]; o.V1 = t.f[F_A_V1]; o.V2 = t.f[F_A_V2]; o.V3 = t.f[F_A_V3];
            o.t11 = t.f[F_A_T11]; o.t22 = t.f[F_A_T22]; o.t33 = t.f[F_A_T33]; o.t12 = t.f[F_A_T12]; o.t13 = t.f[F_A_T13]; o.t23 = t.f[F_A_T23];
            o.xg_mask = 0;
            o.xg[0] = o.xg[1] = o.xg[2] = 0.f;
            if (!c.use_x2 && c.xg_mask) {  // the sweep writes the x1-face ghosts: the BC launch skips its first stage
                o.xg_mask = c.xg_mask;
                for (int i = 0; i < 3; ++i) o.xg[i] = c.xg[i];
                first_bc = 1;
            }
            const int kc = fused_chunk(c);
            dim3 grid((c.d.n1 + FTX - 1) / FTX, (c.d.n2 + FTY - 1) / FTY, (c.d.n3 + kc - 1) / kc);
            const bool prof = c.prof_on && 2 * c.prof_next + 1 < c.prof_ev.size();
            if (prof) cudaEventRecord(c.prof_ev[2 * c.prof_next], c.stream);
            if (c.use_x2)
                k_sweep_x2<G><<<grid, dim3(X2_NT, 1, 1), sweep_x2_smem_bytes(), c.stream>>>(q, o, kc, maps, c.d_err);
            else
                launch_pdl(c.use_pdl, k_fused_tma<G, 1>, grid, dim3(FNT, 1, 1), fused_tma_smem_bytes(), c.stream, q, o, kc, maps, c.d_err);
            if (prof) cudaEventRecord(c.prof_ev[2 * c.prof_next++ + 1], c.stream);
        } else {
            const bool prof = c.prof_on && 2 * c.prof_next + 1 < c.prof_ev.size();
            if (prof) cudaEventRecord(c.prof_ev[2 * c.prof_next], c.stream);
            launch_fused<G, 1>(c, q, t);
            if (prof) cudaEventRecord(c.prof_ev[2 * c.prof_next++ + 1], c.stream);
        }
        swap_state(t);
        q = make_kp_corr(c);
    } else {
        k_stress<float, G, true><<<grid_cells(c.d), blk2d(), 0, c.stream>>>(q);
        k_velocity<float, G, 1><<<grid_vel(c.d), blk2d(), 0, c.stream>>>(q);
    }
    launch_bc<float, G>(c, q, 1, first_bc);
}

// run `n` correction sweeps; with graphs enabled and n even, replays a captured
// graph of n sweeps (after an even count the ping-pong arrangement of the
// buffers is back where it started, so the graph stays valid)
template <int G>
int run_correction_sweeps(Ctx& c, int n) {
    if (n <= 0) return SPH_OK;
    if (!c.use_graphs || (n & 1) || n < 8) {
        for (int i = 0; i < n; ++i) correction_sweep<G>(c);
        CK(cudaGetLastError());
        return SPH_OK;
    }
    if (n != c.graph_len) {
        for (int i = 0; i < 2; ++i) {
            if (c.corr_graph[i]) cudaGraphExecDestroy(c.corr_graph[i]);
            c.corr_graph[i] = nullptr;
            c.corr_graph_key[i] = nullptr;
        }
        c.graph_len = n;
    }
    float* key = c.s32.f[F_P];
    int slot = -1;
    for (int i = 0; i < 2; ++i)
        if (c.corr_graph[i] && c.corr_graph_key[i] == key) slot = i;
    if (slot < 0) {
        slot = c.corr_graph[0] ? 1 : 0;
        if (c.corr_graph[slot]) { cudaGraphExecDestroy(c.corr_graph[slot]); c.corr_graph[slot] = nullptr; }
        ensure_tma_maps(c);
        CK(cudaStreamSynchronize(c.stream));
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < n; ++i) correction_sweep<G>(c);  // recorded, not run
        cudaError_t e = cudaStreamEndCapture(c.stream, &g);
        if (e != cudaSuccess) return fail(SPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c.corr_graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(SPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        c.corr_graph_key[slot] = key;
    }
    CK(cudaGraphLaunch(c.corr_graph[slot], c.stream));
    return SPH_OK;
}

// V += δV, P += δP (FP64)
int apply_correction(Ctx& c) {
    State<double>& s = c.s64;
    State<float>& t = c.s32;
    const long long vol = c.d.vol;
    k_add_widen<float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_V1], t.f[F_V1], vol);
    k_add_widen<float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_V2], t.f[F_V2], vol);
    k_add_widen<float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_V3], t.f[F_V3], vol);
    k_add_widen<float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_P], t.f[F_P], vol);
    CK(cudaGetLastError());
    c.corr_ready = false;
    return SPH_OK;
}

// the correction problem of the current FP64 state, prepared unless one is (MIXED)
int ensure_correction(Ctx& c) {
    if (c.corr_ready) return SPH_OK;
    int rc = sync64(c);
    if (rc) return rc;
    double out[7];
    const int G = c.prm.geometry;
    rc = G == SPH ? outer_residual<SPH>(c, out) : (G == CYL ? outer_residual<CYL>(c, out) : outer_residual<CART>(c, out));
    if (rc) return rc;
    return G == SPH ? prepare_correction<SPH>(c, out) : (G == CYL ? prepare_correction<CYL>(c, out) : prepare_correction<CART>(c, out));
}

// the captured launches of a context (correction sweeps, warm-start iterations): dropped
// when the launch parameters they hold change
void drop_graphs(Ctx& c) {
    for (int i = 0; i < 2; ++i) {
        if (c.corr_graph[i]) cudaGraphExecDestroy(c.corr_graph[i]);
        c.corr_graph[i] = nullptr;
        c.corr_graph_key[i] = nullptr;
        if (c.warm_graph[i]) cudaGraphExecDestroy(c.warm_graph[i]);
        c.warm_graph[i] = nullptr;
        c.warm_key[i][0] = c.warm_key[i][1] = nullptr;
    }
    c.graph_len = 0;
    c.warm_len = 0;
}

// n (even, >= 8) FP32 nonlinear iterations of the warm start as one graph launch; after an
// even count the ping-pong and η buffers are back in the arrangement the graph was captured in
template <int G>
int run_warm_iterations(Ctx& c, int n) {
    if (n != c.warm_len) {
        for (int i = 0; i < 2; ++i) {
            if (c.warm_graph[i]) cudaGraphExecDestroy(c.warm_graph[i]);
            c.warm_graph[i] = nullptr;
            c.warm_key[i][0] = c.warm_key[i][1] = nullptr;
        }
        c.warm_len = n;
    }
    float* kp = c.s32.f[F_P];
    float* ke = c.s32.f[F_ETA];
    int slot = -1;
    for (int i = 0; i < 2; ++i)
        if (c.warm_graph[i] && c.warm_key[i][0] == kp && c.warm_key[i][1] == ke) slot = i;
    if (slot < 0) {
        slot = c.warm_graph[0] ? 1 : 0;
        if (c.warm_graph[slot]) { cudaGraphExecDestroy(c.warm_graph[slot]); c.warm_graph[slot] = nullptr; }
        CK(cudaStreamSynchronize(c.stream));
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < n; ++i) iterate_dispatch<float>(c, c.s32);  // recorded, not run
        cudaError_t e = cudaStreamEndCapture(c.stream, &g);
        if (e != cudaSuccess) return fail(SPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c.warm_graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(SPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        c.warm_key[slot][0] = kp;
        c.warm_key[slot][1] = ke;
        if (c.s32.f[F_P] != kp || c.s32.f[F_ETA] != ke) return fail(SPH_ERR_UNSUPPORTED, "warm-start graph: buffer arrangement not restored");
    }
    CK(cudaGraphLaunch(c.warm_graph[slot], c.stream));
    return SPH_OK;
}

template <int G>
int solve_mixed_g(Ctx& c, const sph_solve_opts& o, sph_solve_info* info, int64_t* hi, double* he, int64_t cap) {
    State<double>& s = c.s64;
    State<float>& t = c.s32;
    const long long vol = c.d.vol;
    const int nout = o.nout > 0 ? o.nout : 100;
    const bool law = c.prm.rheology == SPH_RHEO_EDOT_POWER_RELAX;
    if (c.prm.rheology == SPH_RHEO_TAU_POWER || c.prm.rheology == SPH_RHEO_TAU_POWER_RELAX)
        return fail(SPH_ERR_UNSUPPORTED, "mixed precision needs an explicit viscosity law (linear or strain-rate power law)");
    int64_t iters = 0;
    int status = SPH_ERR_NOT_CONVERGED;
    double err = 1.0;
    c.warm_abandoned = false;
    // optional FP32 nonlinear warm start on the full variables.  The FP64 state is only
    // overwritten once it succeeds: a warm start whose FP32 iteration produces a NaN is
    // abandoned and the correction loop starts from the FP64 state as it was.
    if (o.warm_tol > 0.0) {
        int rc = sync32(c);
        if (rc) return rc;
        double werr = 1.0;
        bool warm_ok = true;
        while (iters < o.maxiter) {
            // the plain iterations up to the next check, replayed from a graph
            const int64_t before = nout - 1 - (iters % nout);
            if (c.use_graphs && before >= 8 && iters + before < o.maxiter) {
                const int n = (int)(before & ~int64_t(1));
                rc = run_warm_iterations<G>(c, n);
                if (rc) return rc;
                iters += n;
                continue;
            }
            ++iters;
            const bool check = (iters % nout) == 0;
            if (check) { rc = snapshot<float>(c, t); if (rc) return rc; }
            iterate_dispatch<float>(c, t);
            if (!check) continue;
            rc = ref_err<float>(c, t, &werr, false);
            if (rc) return rc;
            if (!(werr == werr) || std::isinf(werr)) { warm_ok = false; break; }
            if (werr < o.warm_tol && iters > 20) break;
        }
        if (warm_ok) {  // widen V, P (η is recomputed from the law)
            k_convert<double, float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_V1], t.f[F_V1], vol);
            k_convert<double, float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_V2], t.f[F_V2], vol);
            k_convert<double, float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_V3], t.f[F_V3], vol);
            k_convert<double, float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_P], t.f[F_P], vol);
            if (!law) k_convert<double, float><<<ew_blocks(vol), 256, 0, c.stream>>>(s.f[F_ETA], t.f[F_ETA], vol);
            CK(cudaGetLastError());
        }
        c.warm_abandoned = !warm_ok;
        c.stale32 = true;  // the FP32 state holds the warm start's iterate, not the FP64 state
    }
    float ms = 0.f;
    for (int outer = 0; outer <= o.max_outer; ++outer) {
        double out[7];
        CK(cudaEventRecord(c.ev2, c.stream));
        int rc = outer_residual<G>(c, out);
        if (rc) return rc;
        err = out[6];
        if (info) {
            if (info->nhist < cap) {
                if (hi) hi[info->nhist] = iters;
                if (he) he[info->nhist] = err;
                info->nhist++;
                c.hist_ms.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - c.solve_t0).count());
            }
            info->outer = outer;
            info->residual = err;
        }
        if (!(err == err) || std::isinf(err)) { status = SPH_ERR_DIVERGED; break; }
        if (err < o.tol) { status = SPH_OK; break; }
        if (outer == o.max_outer || iters >= o.maxiter) break;
        rc = prepare_correction<G>(c, out);
        if (rc) return rc;
        CK(cudaEventRecord(c.ev3, c.stream));
        const int inner_max = o.inner_max > 0 ? o.inner_max : 100000;
        int inner = 0;
        while (inner < inner_max && iters < o.maxiter) {
            const int chunk = (int)std::min<int64_t>(std::min<int64_t>(nout, inner_max - inner), o.maxiter - iters);
            rc = run_correction_sweeps<G>(c, chunk);
            if (rc) return rc;
            inner += chunk; iters += chunk;
            if (chunk < nout) break;
            // momentum residual of the correction problem with the current δ state
            KP<float> q = make_kp_corr(c);
            CK(cudaMemsetAsync(c.red, 0, sizeof(unsigned long long) * kRedSlots, c.stream));
            k_velocity_norm<float, G><<<grid_vel(c.d), blk2d(), 0, c.stream>>>(q);
            CK(cudaGetLastError());
            rc = fetch_red(c);
            if (rc) return rc;
            const double ri = slot_val(c, 0);
            if (!(ri == ri) || std::isinf(ri)) { status = SPH_ERR_DIVERGED; break; }
            if (ri <= o.inner_rtol * c.corr_r0) break;
        }
        CK(cudaEventRecord(c.ev4, c.stream));
        rc = check_kernel_flag(c);
        if (rc) return rc;
        if (status == SPH_ERR_DIVERGED) break;
        rc = apply_correction(c);
        if (rc) return rc;
        CK(cudaEventSynchronize(c.ev4));
        CK(cudaEventElapsedTime(&ms, c.ev3, c.ev4));
        c.sweep_ms += ms;
        CK(cudaEventElapsedTime(&ms, c.ev2, c.ev3));
        c.outer_ms += ms;
    }
    // final τ = 2 η_eff D(V) of the FP64 state as the stress output (and the traction pressure)
    if (c.prm.bc == SPH_BC_STRESS) CK(cudaMemcpyAsync(s.f[F_P], s.f[F_PRES], sizeof(double) * vol, cudaMemcpyDeviceToDevice, c.stream));
    {
        const int q[6] = {F_Q11, F_Q22, F_Q33, F_Q12, F_Q13, F_Q23};
        const int d[6] = {F_T11, F_T22, F_T33, F_T12, F_T13, F_T23};
        for (int i = 0; i < 6; ++i) CK(cudaMemcpyAsync(s.f[d[i]], s.f[q[i]], sizeof(double) * vol, cudaMemcpyDeviceToDevice, c.stream));
    }
    c.stale32 = true;
    c.stale64 = false;
    if (info) {
        info->iters = iters; info->err = err; info->status = status;
        if (c.warm_abandoned) info->flags |= SPH_SOLVE_WARM_ABANDONED;
    }
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// Batched mixed-precision solves in lockstep (sph_batch.cuh): the per-solve sequence of
// solve_mixed_g (FP64 outer step, preparation, correction sweeps in chunks of nout with the
// inner test after each full chunk, FP64 update), with every full chunk of every solve run
// as one round of batched sweeps replayed from a CUDA graph.  All work is queued on one
// stream, so each solve's operations keep their order; results equal the solves run alone.
struct BatchSolve {
    Ctx* c = nullptr;
    const sph_solve_opts* o = nullptr;
    sph_solve_info* info = nullptr;
    enum { OUTER, INNER, DONE } st = OUTER;
    int64_t iters = 0;
    int outer = 0;
    int64_t inner = 0;
    int status = SPH_ERR_NOT_CONVERGED;
    double err = 1.0;
    cudaStream_t own = nullptr;  // the context's stream, restored at the end
};

int batch_nout(const sph_solve_opts& o) { return o.nout > 0 ? o.nout : 100; }

// whether a solve can run in the lockstep batch (else the batch falls back to host threads)
bool batch_eligible(const Ctx& c, const sph_solve_opts& o) {
    const int first = c.xg_mask ? 1 : 0;
    return c.prm.precision == SPH_PREC_MIXED && o.criterion == SPH_CRIT_RESIDUAL && !(o.warm_tol > 0.0) &&
           (c.prm.rheology == SPH_RHEO_LINEAR || c.prm.rheology == SPH_RHEO_EDOT_POWER_RELAX) && c.fused && c.use_tma && !c.use_x2 &&
           !c.broken && (batch_nout(o) % 2) == 0 && o.tol > 0.0 && o.maxiter > 0 && (int)c.bc_run.size() - first <= kBatchMaxBc;
}

// the device entry of a solve whose correction problem has just been prepared
int batch_entry(Ctx& c, BatchSweep& e) {
    std::memset(&e, 0, sizeof(e));
    ensure_tma_maps(c);
    State<float>& t = c.s32;
    for (int a = 0; a < 2; ++a) {
        const CUtensorMap* maps = tma_maps(c);
        if (!maps || !c.d_err) return fail(SPH_ERR_UNSUPPORTED, "batched sweeps need the TMA sweep");
        e.p[a] = make_kp_corr(c);
        FusedOut<float>& o = e.o[a];
        o.P = t.f[F_A_P]; o.V1 = t.f[F_A_V1]; o.V2 = t.f[F_A_V2]; o.V3 = t.f[F_A_V3];
        o.t11 = t.f[F_A_T11]; o.t22 = t.f[F_A_T22]; o.t33 = t.f[F_A_T33]; o.t12 = t.f[F_A_T12]; o.t13 = t.f[F_A_T13]; o.t23 = t.f[F_A_T23];
        o.xg_mask = c.xg_mask;
        for (int i = 0; i < 3; ++i) o.xg[i] = c.xg[i];
        e.maps[a] = maps;
        swap_state(t);
    }
    e.err = c.d_err;
    e.kchunk = fused_chunk(c);
    const int first = c.xg_mask ? 1 : 0;
    e.nbc = (int)c.bc_run.size() - first;
    for (int i = 0; i < e.nbc; ++i) e.bc[i] = c.bc_run[first + i];
    return SPH_OK;
}

template <int G>
int batch_outer_step(BatchSolve& b, BatchSweep& e) {
    Ctx& c = *b.c;
    const sph_solve_opts& o = *b.o;
    double out[7];
    int rc = outer_residual<G>(c, out);
    if (rc) return rc;
    b.err = out[6];
    b.info->outer = b.outer;
    b.info->residual = b.err;
    if (!(b.err == b.err) || std::isinf(b.err)) { b.status = SPH_ERR_DIVERGED; b.st = BatchSolve::DONE; return SPH_OK; }
    if (b.err < o.tol) { b.status = SPH_OK; b.st = BatchSolve::DONE; return SPH_OK; }
    if (b.outer == o.max_outer || b.iters >= o.maxiter) { b.st = BatchSolve::DONE; return SPH_OK; }
    if ((rc = prepare_correction<G>(c, out))) return rc;
    b.inner = 0;
    b.st = BatchSolve::INNER;
    return batch_entry(c, e);
}

// end of a solve's correction phase: the bounded-wait flag, then the FP64 update
int batch_end_inner(BatchSolve& b) {
    Ctx& c = *b.c;
    int rc = check_kernel_flag(c);
    if (rc) return rc;
    if (b.status == SPH_ERR_DIVERGED) { b.st = BatchSolve::DONE; return SPH_OK; }
    if ((rc = apply_correction(c))) return rc;
    ++b.outer;
    b.st = BatchSolve::OUTER;
    return SPH_OK;
}

// the final copies of solve_mixed_g and the solve's record
int batch_finish(BatchSolve& b) {
    Ctx& c = *b.c;
    State<double>& s = c.s64;
    const long long vol = c.d.vol;
    if (c.prm.bc == SPH_BC_STRESS) CK(cudaMemcpyAsync(s.f[F_P], s.f[F_PRES], sizeof(double) * vol, cudaMemcpyDeviceToDevice, c.stream));
    const int q[6] = {F_Q11, F_Q22, F_Q33, F_Q12, F_Q13, F_Q23};
    const int d[6] = {F_T11, F_T22, F_T33, F_T12, F_T13, F_T23};
    for (int i = 0; i < 6; ++i) CK(cudaMemcpyAsync(s.f[d[i]], s.f[q[i]], sizeof(double) * vol, cudaMemcpyDeviceToDevice, c.stream));
    c.stale32 = true;
    c.stale64 = false;
    b.info->iters = b.iters;
    b.info->err = b.err;
    b.info->status = b.status;
    return SPH_OK;
}

int batch_run_partial(Ctx& c, int n) {
    switch (c.prm.geometry) {
        case SPH_GEOM_SPHERICAL: return run_correction_sweeps<SPH>(c, n);
        case SPH_GEOM_CYLINDRICAL: return run_correction_sweeps<CYL>(c, n);
        default: return run_correction_sweeps<CART>(c, n);
    }
}

int batch_outer(BatchSolve& b, BatchSweep& e) {
    switch (b.c->prm.geometry) {
        case SPH_GEOM_SPHERICAL: return batch_outer_step<SPH>(b, e);
        case SPH_GEOM_CYLINDRICAL: return batch_outer_step<CYL>(b, e);
        default: return batch_outer_step<CART>(b, e);
    }
}

// device buffers of one lockstep batch (freed on every return path)
struct BatchDev {
    BatchSweep* entries = nullptr;
    int* active = nullptr;
    unsigned long long* red = nullptr;
    int4* items = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~BatchDev() {
        if (stream) cudaStreamSynchronize(stream);
        if (graph) cudaGraphExecDestroy(graph);
        if (entries) cudaFree(entries);
        if (active) cudaFree(active);
        if (red) cudaFree(red);
        if (items) cudaFree(items);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
    }
};

int batch_lockstep(void* const* ctxs, int32_t n, const sph_solve_opts* opts, sph_solve_info* infos) {
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<BatchSolve> bs((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        BatchSolve& b = bs[i];
        b.c = static_cast<Ctx*>(ctxs[i]);
        b.o = &opts[i];
        b.info = &infos[i];
        std::memset(b.info, 0, sizeof(*b.info));
        b.c->sweep_ms = b.c->outer_ms = 0.0;
        b.c->hist_ms.clear();
        b.c->corr_ready = false;
        CK(cudaStreamSynchronize(b.c->stream));
    }
    const int nout = batch_nout(opts[0]);
    bool pdl = true;  // programmatic dependent launches inside the round's graph (off if any solve has them off)
    for (int32_t i = 0; i < n; ++i) pdl = pdl && static_cast<Ctx*>(ctxs[i])->use_pdl;
    BatchDev dev;
    struct Restore {  // every context back on its own stream, on every return path
        std::vector<BatchSolve>& bs;
        ~Restore() { for (BatchSolve& b : bs) if (b.own) b.c->stream = b.own; }
    } restore{bs};
    CK(cudaStreamCreateWithFlags(&dev.stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&dev.e0));
    CK(cudaEventCreate(&dev.e1));
    for (BatchSolve& b : bs) { b.own = b.c->stream; b.c->stream = dev.stream; }
    CK(cudaEventRecord(dev.e0, dev.stream));
    for (BatchSolve& b : bs) { int rc = sync64(*b.c); if (rc) return rc; }

    // work lists: blocks of the member solves' fused sweeps, BC stages and inner tests, per geometry
    std::vector<BatchSweep> host((size_t)n);
    std::vector<int4> items;
    size_t fz_off[3], fz_n[3], nm_off[3], nm_n[3], bc_off[3][kBatchMaxBc], bc_n[3][kBatchMaxBc];
    size_t items_cap = 0, members = 0;
    auto build_lists = [&]() -> int {
        items.clear();
        members = 0;
        std::vector<int> mem;
        for (int32_t i = 0; i < n; ++i)
            if (bs[i].st != BatchSolve::DONE) mem.push_back(i);
        members = mem.size();
        for (int g = 0; g < 3; ++g) {
            fz_off[g] = items.size();
            for (int i : mem) {
                Ctx& c = *bs[i].c;
                if (c.prm.geometry != g) continue;
                const int kc = fused_chunk(c);
                const int gx = (c.d.n1 + FTX - 1) / FTX, gy = (c.d.n2 + FTY - 1) / FTY, gz = (c.d.n3 + kc - 1) / kc;
                for (int z = 0; z < gz; ++z) for (int y = 0; y < gy; ++y) for (int x = 0; x < gx; ++x) items.push_back(make_int4(i, x, y, z));
            }
            fz_n[g] = items.size() - fz_off[g];
            for (int t = 0; t < kBatchMaxBc; ++t) {
                bc_off[g][t] = items.size();
                for (int i : mem) {
                    Ctx& c = *bs[i].c;
                    const int first = c.xg_mask ? 1 : 0;
                    if (c.prm.geometry != g || first + t >= (int)c.bc_run.size()) continue;
                    const BcStage& st = c.bc_run[first + t];
                    const int eu = st.dim == 0 ? c.d.n2 + 1 : c.d.n1 + 1, ev = st.dim == 2 ? c.d.n2 + 1 : c.d.n3 + 1;
                    for (int v = 0; v < (ev + 7) / 8; ++v) for (int u = 0; u < (eu + 31) / 32; ++u) items.push_back(make_int4(i, u, v, 0));
                }
                bc_n[g][t] = items.size() - bc_off[g][t];
            }
            nm_off[g] = items.size();
            for (int i : mem) {
                Ctx& c = *bs[i].c;
                if (c.prm.geometry != g) continue;
                const dim3 gv = grid_vel(c.d);
                for (unsigned z = 0; z < gv.z; ++z) for (unsigned y = 0; y < gv.y; ++y) for (unsigned x = 0; x < gv.x; ++x)
                    items.push_back(make_int4(i, (int)x, (int)y, (int)z));
            }
            nm_n[g] = items.size() - nm_off[g];
        }
        if (items.size() > items_cap) {
            CK(cudaStreamSynchronize(dev.stream));
            if (dev.items) cudaFree(dev.items);
            dev.items = nullptr;
            if (cudaMalloc((void**)&dev.items, sizeof(int4) * std::max<size_t>(items.size(), 1)) != cudaSuccess) {
                cudaGetLastError();
                return fail(SPH_ERR_NOMEM, "batched solve: device work lists");
            }
            items_cap = items.size();
        }
        CK(cudaMemcpyAsync(dev.items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, dev.stream));
        CK(cudaStreamSynchronize(dev.stream));  // the host list is rebuilt in place next time
        return SPH_OK;
    };
    if (cudaMalloc((void**)&dev.entries, sizeof(BatchSweep) * n) != cudaSuccess || cudaMalloc((void**)&dev.active, sizeof(int) * n) != cudaSuccess ||
        cudaMalloc((void**)&dev.red, sizeof(unsigned long long) * n) != cudaSuccess) {
        cudaGetLastError();
        return fail(SPH_ERR_NOMEM, "batched solve: device work lists");
    }
    CK(cudaMemsetAsync(dev.entries, 0, sizeof(BatchSweep) * n, dev.stream));
    if (int rc = build_lists()) return rc;
    std::vector<int> act((size_t)n, 0);

    // one round: nout sweeps of every active solve (arrangement a = s & 1 read by sweep s)
    auto capture = [&]() -> int {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(dev.stream, cudaStreamCaptureModeThreadLocal));
        for (int sw = 0; sw < nout; ++sw) {
            const int a = sw & 1;
            // programmatic dependent launches, as the single-grid sweep: each launch overlaps the
            // tail of the one before (the kernels wait on it before touching memory)
            const BatchSweep* E = dev.entries;
            const int* act_d = dev.active;
            if (fz_n[SPH]) launch_pdl(pdl, k_fused_tma_batch<SPH>, dim3((unsigned)fz_n[SPH]), dim3(FNT), fused_tma_smem_bytes(), dev.stream, E, dev.items + fz_off[SPH], act_d, a);
            if (fz_n[CYL]) launch_pdl(pdl, k_fused_tma_batch<CYL>, dim3((unsigned)fz_n[CYL]), dim3(FNT), fused_tma_smem_bytes(), dev.stream, E, dev.items + fz_off[CYL], act_d, a);
            if (fz_n[CART]) launch_pdl(pdl, k_fused_tma_batch<CART>, dim3((unsigned)fz_n[CART]), dim3(FNT), fused_tma_smem_bytes(), dev.stream, E, dev.items + fz_off[CART], act_d, a);
            for (int t = 0; t < kBatchMaxBc; ++t) {
                if (bc_n[SPH][t]) launch_pdl(pdl, k_bc_batch<SPH>, dim3((unsigned)bc_n[SPH][t]), blk2d(), 0, dev.stream, E, dev.items + bc_off[SPH][t], act_d, a, t);
                if (bc_n[CYL][t]) launch_pdl(pdl, k_bc_batch<CYL>, dim3((unsigned)bc_n[CYL][t]), blk2d(), 0, dev.stream, E, dev.items + bc_off[CYL][t], act_d, a, t);
                if (bc_n[CART][t]) launch_pdl(pdl, k_bc_batch<CART>, dim3((unsigned)bc_n[CART][t]), blk2d(), 0, dev.stream, E, dev.items + bc_off[CART][t], act_d, a, t);
            }
        }
        cudaError_t e = cudaStreamEndCapture(dev.stream, &g);
        if (e != cudaSuccess) return fail(SPH_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&dev.graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(SPH_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
        return SPH_OK;
    };

    for (;;) {
        int rc;
        // FP64 outer steps of the solves between correction phases
        for (int32_t i = 0; i < n; ++i)
            if (bs[i].st == BatchSolve::OUTER) {
                if ((rc = batch_outer(bs[i], host[i]))) return rc;
                if (bs[i].st == BatchSolve::INNER)
                    CK(cudaMemcpyAsync(dev.entries + i, &host[i], sizeof(BatchSweep), cudaMemcpyHostToDevice, dev.stream));
            }
        // the next chunk of every solve in its correction phase: full chunks go into the round
        bool any = false, pending = false;
        for (int32_t i = 0; i < n; ++i) {
            BatchSolve& b = bs[i];
            act[i] = 0;
            if (b.st != BatchSolve::INNER) continue;
            const int64_t inner_max = b.o->inner_max > 0 ? b.o->inner_max : 100000;
            const int64_t chunk = std::min<int64_t>(std::min<int64_t>(nout, inner_max - b.inner), b.o->maxiter - b.iters);
            if (chunk <= 0) {  // the inner loop's condition fails before a sweep
                if ((rc = batch_end_inner(b))) return rc;
            } else if (chunk < nout) {  // a last, shorter chunk: this solve alone, no inner test after it
                if ((rc = batch_run_partial(*b.c, (int)chunk))) return rc;
                b.inner += chunk;
                b.iters += chunk;
                if ((rc = batch_end_inner(b))) return rc;
            } else {
                act[i] = 1;
                any = true;
            }
        }
        size_t open_solves = 0;
        for (const BatchSolve& b : bs) open_solves += b.st != BatchSolve::DONE;
        pending = open_solves > 0;
        if (!any) {
            if (!pending) break;
            continue;
        }
        // finished solves leave the work list once they are half of it (a new list, a new graph)
        if (2 * open_solves <= members && open_solves < members) {
            if (dev.graph) { CK(cudaStreamSynchronize(dev.stream)); cudaGraphExecDestroy(dev.graph); dev.graph = nullptr; }
            if ((rc = build_lists())) return rc;
        }
        if (!dev.graph && (rc = capture())) return rc;
        CK(cudaMemcpyAsync(dev.active, act.data(), sizeof(int) * n, cudaMemcpyHostToDevice, dev.stream));
        CK(cudaGraphLaunch(dev.graph, dev.stream));
        CK(cudaMemsetAsync(dev.red, 0, sizeof(unsigned long long) * n, dev.stream));
        if (nm_n[SPH]) k_velocity_norm_batch<SPH><<<(unsigned)nm_n[SPH], blk2d(), 0, dev.stream>>>(dev.entries, dev.items + nm_off[SPH], dev.active, dev.red);
        if (nm_n[CYL]) k_velocity_norm_batch<CYL><<<(unsigned)nm_n[CYL], blk2d(), 0, dev.stream>>>(dev.entries, dev.items + nm_off[CYL], dev.active, dev.red);
        if (nm_n[CART]) k_velocity_norm_batch<CART><<<(unsigned)nm_n[CART], blk2d(), 0, dev.stream>>>(dev.entries, dev.items + nm_off[CART], dev.active, dev.red);
        CK(cudaGetLastError());
        std::vector<unsigned long long> red((size_t)n);
        CK(cudaMemcpyAsync(red.data(), dev.red, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, dev.stream));
        CK(cudaStreamSynchronize(dev.stream));
        for (int32_t i = 0; i < n; ++i) {
            if (!act[i]) continue;
            BatchSolve& b = bs[i];
            b.inner += nout;
            b.iters += nout;
            double ri;
            std::memcpy(&ri, &red[i], sizeof(double));
            bool end = false;
            if (!(ri == ri) || std::isinf(ri)) { b.status = SPH_ERR_DIVERGED; end = true; }
            else if (ri <= b.o->inner_rtol * b.c->corr_r0) end = true;
            if (end && (rc = batch_end_inner(b))) return rc;
        }
    }
    for (BatchSolve& b : bs) { int rc = batch_finish(b); if (rc) return rc; }
    CK(cudaEventRecord(dev.e1, dev.stream));
    CK(cudaEventSynchronize(dev.e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, dev.e0, dev.e1));
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (BatchSolve& b : bs) { b.info->seconds = wall; b.info->device_ms = ms; b.c->last_ms = ms; }
    return SPH_OK;
}

// ---------------------------------------------------------------------------
int check_params(const sph_params* p) {
    if (!p) return fail(SPH_ERR_INVALID, "params is NULL");
    if (p->abi_version != SPH_ABI_VERSION) return fail(SPH_ERR_INVALID, "abi_version mismatch");
    if (p->geometry < 0 || p->geometry > 2) return fail(SPH_ERR_INVALID, "geometry");
    if (p->precision < 0 || p->precision > 2) return fail(SPH_ERR_INVALID, "precision");
    if (p->rheology < 0 || p->rheology > 3) return fail(SPH_ERR_INVALID, "rheology");
    if (p->bc < 0 || p->bc > 3) return fail(SPH_ERR_INVALID, "bc");
    if (p->bc == SPH_BC_FREE_SURFACE && p->geometry != SPH_GEOM_SPHERICAL) return fail(SPH_ERR_UNSUPPORTED, "SPH_BC_FREE_SURFACE is spherical only");
    if (p->n1 < 5 || p->n2 < 5 || p->n3 < 5) return fail(SPH_ERR_INVALID, "grid needs at least 5 cells per axis");
    // x2 and x3 index the launch grids' y and z dimensions (at most 65535 blocks each)
    if (p->n2 >= 65535 || p->n3 >= 65535) return fail(SPH_ERR_INVALID, "n2 and n3 must be below 65535");
    if (!(p->l1 > 0 && p->l2 > 0 && p->l3 > 0 && p->l_ref > 0)) return fail(SPH_ERR_INVALID, "lengths must be positive");
    long long px = ((p->n1 + 1 + 31) / 32) * 32LL;
    if (px * (p->n2 + 1LL) * (p->n3 + 1LL) >= (1LL << 31)) return fail(SPH_ERR_INVALID, "grid too large for 32-bit indexing");
    // the fused FP32 sweep stores at 32-bit byte offsets (4 bytes x box index < 2^32)
    if (p->precision != SPH_PREC_FP64 && px * (p->n2 + 1LL) * (p->n3 + 1LL) >= (1LL << 30))
        return fail(SPH_ERR_INVALID, "grid too large for the FP32 sweep (box of 2^30 points or more)");
    if (p->geometry == SPH_GEOM_SPHERICAL) {
        if (p->c1 - p->l1 / 2 <= 0) return fail(SPH_ERR_INVALID, "spherical radius range must be positive");
        if (p->c2 - p->l2 / 2 <= 0 || p->c2 + p->l2 / 2 >= kPi) return fail(SPH_ERR_INVALID, "colatitude range must be inside (0, pi)");
    }
    if (p->geometry == SPH_GEOM_CYLINDRICAL && p->c1 - p->l1 / 2 <= 0) return fail(SPH_ERR_INVALID, "cylindrical radius range must be positive");
    return SPH_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }

const char* sph_last_error(void) { return g_err.c_str(); }

const char* sph_strerror(int code) {
    switch (code) {
        case SPH_OK: return "ok";
        case SPH_ERR_INVALID: return "invalid argument";
        case SPH_ERR_CUDA: return "CUDA error";
        case SPH_ERR_NOT_CONVERGED: return "not converged";
        case SPH_ERR_DIVERGED: return "diverged (NaN/Inf)";
        case SPH_ERR_NOMEM: return "out of memory";
        case SPH_ERR_UNSUPPORTED: return "unsupported option combination";
        case SPH_ERR_NO_DEVICE: return "no usable CUDA device";
        default: return "unknown status";
    }
}

int sph_params_default(sph_params* p, int32_t geometry) {
    if (!p) return fail(SPH_ERR_INVALID, "params is NULL");
    std::memset(p, 0, sizeof(*p));
    p->abi_version = SPH_ABI_VERSION;
    p->geometry = geometry;
    p->precision = SPH_PREC_FP64;
    p->bc = SPH_BC_DIAPIR;
    p->init = SPH_INIT_INCLUSION;
    p->n1 = p->n2 = p->n3 = 208 - 1;
    p->eta0 = 1.0; p->vr = 1e2; p->rho0 = 0.0; p->rho_in = -10.0; p->g = 1.0;
    p->tau_C = 1.0; p->radius = 1.0; p->sh = 1.0; p->dmp = 4.5;
    p->relax = 1e-3; p->edot_bg = 1.0;
    const double lr = 6.0;
    switch (geometry) {
        case SPH_GEOM_SPHERICAL:  // SphericalStokes_diapir.jl:348-367
            p->rheology = SPH_RHEO_TAU_POWER; p->n_exp = 5.0; p->r = 1000.0;
            p->c1 = p->r; p->c2 = kPi / 2.0; p->c3 = 0.0;
            p->l1 = lr; p->l2 = lr / p->r; p->l3 = lr / p->r; p->l_ref = lr;
            break;
        case SPH_GEOM_CYLINDRICAL:  // CylindricalStokes_diapir.jl:227-251
            p->rheology = SPH_RHEO_TAU_POWER_RELAX; p->n_exp = 1.0; p->n_exp_late = 5.0; p->switch_err = 1e-5; p->r = 1000.0;
            p->c1 = p->r; p->c2 = 0.0; p->c3 = 0.0;
            p->l1 = lr; p->l2 = lr / p->r; p->l3 = lr; p->l_ref = lr;
            break;
        case SPH_GEOM_CARTESIAN:  // CartesianStokes_diapir.jl:267-289
            p->rheology = SPH_RHEO_TAU_POWER_RELAX; p->n_exp = 5.0; p->r = 0.0;
            p->c1 = p->c2 = p->c3 = 0.0;
            p->l1 = p->l2 = p->l3 = lr; p->l_ref = lr;
            break;
        default: return fail(SPH_ERR_INVALID, "geometry");
    }
    p->vpdt = 0.0;  // 0: dx1 * CFL with CFL = 1/(2 + 4.5 log10(vr)), set at sph_create
    p->etasm_passes = 1;
    return SPH_OK;
}

int sph_field_dims(const sph_params* p, int32_t field, int64_t dims[3]) {
    if (!p || !dims) return fail(SPH_ERR_INVALID, "NULL argument");
    if (field < 0 || field >= SPH_FIELD_COUNT) return fail(SPH_ERR_INVALID, "field");
    Dims d{}; d.n1 = p->n1; d.n2 = p->n2; d.n3 = p->n3;
    int e[3];
    field_extent(d, field, e);
    dims[0] = e[0]; dims[1] = e[1]; dims[2] = e[2];
    return SPH_OK;
}

int sph_create(const sph_params* prm, void** out) {
    if (!out) return fail(SPH_ERR_INVALID, "ctx out pointer is NULL");
    *out = nullptr;
    int rc = check_params(prm);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(SPH_ERR_NO_DEVICE, "no CUDA device");
    Ctx* c = new (std::nothrow) Ctx();
    if (!c) return fail(SPH_ERR_NOMEM, "host allocation");
    c->prm = *prm;
    sph_params& q = c->prm;
    if (q.vpdt <= 0.0) q.vpdt = q.l1 / (q.n1 - 1) * (1.0 / (2.0 + 4.5 * std::log10(q.vr)));
    c->cur_n = q.n_exp;
    c->fused = q.kernels != SPH_KERNELS_SIMPLE;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned_chunk.find(std::make_tuple(q.geometry, q.n1, q.n2, q.n3));
        if (it != g_tuned_chunk.end()) c->fused_chunk = it->second;
    }
    if (const char* e = std::getenv("SPH_FUSED_CHUNK")) c->fused_chunk = std::atoi(e);
    Dims& d = c->d;
    d.n1 = q.n1; d.n2 = q.n2; d.n3 = q.n3;
    d.px = ((q.n1 + 1 + 31) / 32) * 32; d.py = q.n2 + 1; d.pz = q.n3 + 1;
    d.sy = d.px; d.sz = d.px * d.py;
    d.vol = (long long)d.px * d.py * d.pz;
    c->hx1 = linspace(q.c1, q.l1, q.n1);
    c->hx2 = linspace(q.c2, q.l2, q.n2);
    c->hx3 = linspace(q.c3, q.l3, q.n3);
    auto cleanup = [&](int code) { sph_destroy(c); return code; };
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) return cleanup(fail(SPH_ERR_CUDA, "stream create"));
    c->stream = c->own_stream;
    if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess || cudaEventCreate(&c->ev2) != cudaSuccess ||
        cudaEventCreate(&c->ev3) != cudaSuccess || cudaEventCreate(&c->ev4) != cudaSuccess)
        return cleanup(fail(SPH_ERR_CUDA, "event create"));
    if (cudaMalloc((void**)&c->red, sizeof(unsigned long long) * kRedSlots) != cudaSuccess) return cleanup(fail(SPH_ERR_NOMEM, "reduction slots"));
    if (cudaMallocHost((void**)&c->hred, sizeof(unsigned long long) * kRedSlots) != cudaSuccess) return cleanup(fail(SPH_ERR_NOMEM, "pinned slots"));
    if (cudaMalloc((void**)&c->phase, d.vol) != cudaSuccess) return cleanup(fail(SPH_ERR_NOMEM, "phase"));
    if ((rc = alloc_state<double>(*c, c->s64))) return cleanup(rc == SPH_ERR_CUDA ? SPH_ERR_NOMEM : rc);
    if (q.precision != SPH_PREC_FP64) {
        if ((rc = alloc_state<float>(*c, c->s32))) return cleanup(rc == SPH_ERR_CUDA ? SPH_ERR_NOMEM : rc);
        c->has32 = true;
    }
    if ((rc = set_fused_attrs())) return cleanup(rc);
    {
        int dev = 0, sms = 0, per_sm = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_tma<SPH, 1>, FNT, fused_tma_smem_bytes()) == cudaSuccess)
            c->fused_slots = sms * per_sm;
        cudaGetLastError();
    }
    if (const char* e = std::getenv("SPH_NO_GRAPHS")) c->use_graphs = std::atoi(e) == 0;
    if (const char* e = std::getenv("SPH_NO_TMA")) c->use_tma = std::atoi(e) == 0;
    if (const char* e = std::getenv("SPH_SWEEP_X2")) c->use_x2 = std::atoi(e) != 0;
    if (q.bc == SPH_BC_FREE_SURFACE) c->use_x2 = false;  // the paired-FP32 sweep has no free-surface top cell
    if (const char* e = std::getenv("SPH_NO_PDL")) c->use_pdl = std::atoi(e) == 0;
    if (const char* e = std::getenv("SPH_NO_XGHOST")) c->xg_fuse = std::atoi(e) == 0;
    if ((rc = build_bc(*c))) return cleanup(rc);
    if ((rc = init_fields(*c))) return cleanup(rc);
    if ((rc = compute_f_scale(*c))) return cleanup(rc);
    c->stale32 = true;
    *out = c;
    return SPH_OK;
}

int sph_batch_solve(void* const* ctxs, int32_t n, const sph_solve_opts* opts, sph_solve_info* infos, int32_t threads) {
    if (n < 0 || (n > 0 && (!ctxs || !opts || !infos))) return fail(SPH_ERR_INVALID, "sph_batch_solve: NULL argument");
    for (int32_t i = 0; i < n; ++i) {
        if (!ctxs[i]) return fail(SPH_ERR_INVALID, "sph_batch_solve: NULL context");
        for (int32_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(SPH_ERR_INVALID, "sph_batch_solve: a context appears twice");
    }
    if (n == 0) return SPH_OK;
    // lockstep batch: every solve mixed-precision on the FP64 residual, no warm start, the TMA
    // sweep, one nout for all (the common case of a parameter sweep); else one host thread per
    // solve at a time, each on its own stream
    bool lockstep = true;
    for (int32_t i = 0; i < n && lockstep; ++i)
        lockstep = batch_eligible(*static_cast<Ctx*>(ctxs[i]), opts[i]) && batch_nout(opts[i]) == batch_nout(opts[0]);
    if (lockstep) return batch_lockstep(ctxs, n, opts, infos);
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    nt = std::max(1, std::min(nt, (int)n));
    int dev = 0;
    CK(cudaGetDevice(&dev));
    std::atomic<int32_t> next(0);
    std::vector<std::string> errs(n);
    auto worker = [&]() {
        cudaSetDevice(dev);  // the caller's device in every worker
        for (int32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
            const int rc = sph_solve(ctxs[i], &opts[i], &infos[i], nullptr, nullptr, 0);
            if (rc != SPH_OK && rc != SPH_ERR_NOT_CONVERGED && rc != SPH_ERR_DIVERGED) {
                infos[i].status = rc;
                errs[i] = g_err;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    for (int32_t i = 0; i < n; ++i)
        if (!errs[i].empty()) return fail(infos[i].status, "solve " + std::to_string(i) + ": " + errs[i]);
    return SPH_OK;
}

int sph_autotune(void* h, int32_t sweeps, int32_t* best_chunk, double* best_ms) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (c->prm.precision != SPH_PREC_MIXED || !c->fused) return fail(SPH_ERR_UNSUPPORTED, "sph_autotune tunes the fused FP32 sweep (MIXED, SPH_KERNELS_AUTO)");
    if (sweeps < 2) sweeps = 2;
    int rc = sph_sweep(h, 0);  // prepares a correction problem (FP64 state unchanged)
    if (rc) return rc;
    const int G = c->prm.geometry;
    const int n3 = c->d.n3;
    const int cand[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256};
    struct Restore {
        Ctx* c;
        bool graphs;
        ~Restore() { c->use_graphs = graphs; c->corr_ready = false; }
    } restore{c, c->use_graphs};
    c->use_graphs = false;
    double bms = 1e300;
    int bk = 0;
    for (int kc : cand) {
        if (kc > n3 && bk) break;
        c->fused_chunk = std::min(kc, n3);
        rc = G == SPH ? run_correction_sweeps<SPH>(*c, 1) : (G == CYL ? run_correction_sweeps<CYL>(*c, 1) : run_correction_sweeps<CART>(*c, 1));
        if (rc) return rc;
        CK(cudaEventRecord(c->ev0, c->stream));
        rc = G == SPH ? run_correction_sweeps<SPH>(*c, sweeps) : (G == CYL ? run_correction_sweeps<CYL>(*c, sweeps) : run_correction_sweeps<CART>(*c, sweeps));
        if (rc) return rc;
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaEventSynchronize(c->ev1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        if (ms < bms) { bms = ms; bk = c->fused_chunk; }
        if (kc >= n3) break;
    }
    if ((rc = check_kernel_flag(*c))) return rc;
    c->fused_chunk = bk;
    drop_graphs(*c);  // graphs were captured with the previous chunk length
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tuned_chunk[std::make_tuple(c->prm.geometry, c->d.n1, c->d.n2, c->d.n3)] = bk;
    }
    if (best_chunk) *best_chunk = bk;
    if (best_ms) *best_ms = bms / sweeps;
    return SPH_OK;
}

int sph_update_params(void* h, const sph_params* p) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    int rc = check_params(p);
    if (rc) return rc;
    const sph_params& q = c->prm;
    if (p->geometry != q.geometry || p->precision != q.precision || p->bc != q.bc || p->rheology != q.rheology ||
        p->kernels != q.kernels || p->n1 != q.n1 || p->n2 != q.n2 || p->n3 != q.n3 || p->c1 != q.c1 || p->c2 != q.c2 ||
        p->c3 != q.c3 || p->l1 != q.l1 || p->l2 != q.l2 || p->l3 != q.l3)
        return fail(SPH_ERR_INVALID, "sph_update_params: geometry, precision, bc, rheology, kernels, n1..n3, c1..c3 and l1..l3 "
                                     "are fixed at sph_create");
    if ((rc = sync64(*c))) return rc;
    sph_params n = *p;
    if (n.vpdt <= 0.0) n.vpdt = n.l1 / (n.n1 - 1) * (1.0 / (2.0 + 4.5 * std::log10(n.vr)));
    c->prm = n;
    c->cur_n = n.n_exp;
    // captured launches and the prepared correction problem hold the old scalars
    drop_graphs(*c);
    c->corr_ready = false;
    if ((rc = build_bc(*c))) return rc;
    return compute_f_scale(*c);
}

int sph_destroy(void* h) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return SPH_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_state(c->s64);
    free_state(c->s32);
    if (c->phase) cudaFree(c->phase);
    if (c->d_maps) cudaFree(c->d_maps);
    if (c->d_err) cudaFree(c->d_err);
    if (c->red) cudaFree(c->red);
    if (c->hred) cudaFreeHost(c->hred);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    drop_graphs(*c);
    if (c->ev2) cudaEventDestroy(c->ev2);
    if (c->ev3) cudaEventDestroy(c->ev3);
    if (c->ev4) cudaEventDestroy(c->ev4);
    for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
    if (c->adj) cudaFree(c->adj);
    if (c->stage) cudaFree(c->stage);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return SPH_OK;
}

int sph_set_stream(void* h, void* stream) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    CK(cudaStreamSynchronize(c->stream));
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    return SPH_OK;
}

static int copy_field(Ctx* c, int32_t field, double* host, const double* src_host, int64_t count) {
    if (field < 0 || field >= SPH_FIELD_COUNT) return fail(SPH_ERR_INVALID, "field");
    int e[3];
    field_extent(c->d, field, e);
    const int64_t need = (int64_t)e[0] * e[1] * e[2];
    if (count != need) return fail(SPH_ERR_INVALID, "count does not match the field size");
    if (!host && !src_host) return fail(SPH_ERR_INVALID, "host pointer is NULL");
    const bool get = host != nullptr;
    int rc = usable(*c);
    if (rc) return rc;
    if (get && (rc = sync64(*c))) return rc;
    if (field == SPH_FIELD_PHASE) {  // stored as one byte per entry (1 = linear cell)
        rc = get ? download_box<uint8_t>(*c, c->phase, e, host) : upload_box<uint8_t>(*c, c->phase, e, src_host);
    } else {
        double* dev = c->s64.f[slot_of(field)];
        rc = get ? download_box<double>(*c, dev, e, host) : upload_box<double>(*c, dev, e, src_host);
    }
    if (rc) return rc;
    if (!get) c->stale32 = true;
    return SPH_OK;
}

// one FP64 state slot with the extent e, in the reference's column-major layout
static int copy_slot_out(Ctx* c, int slot, const int e[3], double* host) {
    return download_box<double>(*c, c->s64.f[slot], e, host);
}

static std::string strf(const char* f, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, f);
    std::vsnprintf(buf, sizeof(buf), f, ap);
    va_end(ap);
    return std::string(buf);
}

static int write_file(const std::string& path, const void* data, size_t bytes) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail(SPH_ERR_INVALID, "sph_save: cannot open " + path + " for writing");
    const size_t w = bytes ? std::fwrite(data, 1, bytes, f) : 0;
    const int cl = std::fclose(f);
    if (w != bytes || cl != 0) return fail(SPH_ERR_INVALID, "sph_save: short write to " + path);
    return SPH_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// adjoint of the FP64 residual (sph_adjoint.cuh)
enum AdjSlot {
    AJ_LV1, AJ_LV2, AJ_LV3, AJ_LP, AJ_S11, AJ_S22, AJ_S33, AJ_T12, AJ_T13, AJ_T23,
    AJ_V1, AJ_V2, AJ_V3, AJ_P, AJ_GETA, AJ_GRHO, AJ_B1, AJ_B2, AJ_B3, AJ_BP, AJ_R1, AJ_R2, AJ_R3, AJ_RP, AJ_ETA,
    AJ_GEI, AJ_GN, AJ_M11, AJ_M22, AJ_M33, AJ_M12, AJ_M13, AJ_M23, AJ_COUNT
};

static int adj_alloc(Ctx* c) {
    if (c->prm.bc == SPH_BC_FREE_SURFACE)  // no transposed free-surface BC or top-cell pressure
        return fail(SPH_ERR_UNSUPPORTED, "the adjoint is not built for SPH_BC_FREE_SURFACE");
    if (c->adj) return SPH_OK;
    const size_t b = sizeof(double) * (size_t)c->d.vol * AJ_COUNT;
    if (cudaMalloc((void**)&c->adj, b) != cudaSuccess) return fail(SPH_ERR_NOMEM, "adjoint arrays");
    CK(cudaMemsetAsync(c->adj, 0, b, c->stream));
    return SPH_OK;
}
static double* adj_slot(Ctx* c, int s) { return c->adj + (size_t)s * c->d.vol; }

// host array with a field's extent (reference layout) <-> an adjoint slot; NULL host: zero
static int adj_upload(Ctx* c, int slot, int field, const double* host) {
    double* dev = adj_slot(c, slot);
    CK(cudaMemsetAsync(dev, 0, sizeof(double) * c->d.vol, c->stream));
    if (!host) return SPH_OK;
    int e[3];
    field_extent(c->d, field, e);
    return upload_box<double>(*c, dev, e, host);
}
static int adj_download(Ctx* c, int slot, int field, double* host) {
    if (!host) return SPH_OK;
    int e[3];
    field_extent(c->d, field, e);
    return download_box<double>(*c, adj_slot(c, slot), e, host);
}

// KP of the adjoint: the FP64 state with η = the residual's viscosity (the law's target for
// the strain-rate law, frozen at the current V), ηSM and DT_R recomputed from it
template <int G>
static KP<double> adj_kp(Ctx* c) {
    State<double>& s = c->s64;
    KP<double> p = make_kp<double>(*c, s);
    double* eta = adj_slot(c, AJ_ETA);
    if (c->prm.rheology == SPH_RHEO_EDOT_POWER_RELAX) {
        k_strain<double, G><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p);
        k_edot_law<double, false><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p);
        cudaMemcpyAsync(eta, s.f[F_ETA_OUT], sizeof(double) * c->d.vol, cudaMemcpyDeviceToDevice, c->stream);
    } else {
        cudaMemcpyAsync(eta, s.f[F_ETA], sizeof(double) * c->d.vol, cudaMemcpyDeviceToDevice, c->stream);
    }
    p.eta = eta;
    KP<double> q = p;
    q.etaSM = s.f[F_ETA_SM];
    k_maxloc<double><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(q, G == CART);
    k_pt_dtr<<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p);
    return p;
}

static Adj adj_ptrs(Ctx* c) {
    Adj a;
    a.lV1 = adj_slot(c, AJ_LV1); a.lV2 = adj_slot(c, AJ_LV2); a.lV3 = adj_slot(c, AJ_LV3); a.lP = adj_slot(c, AJ_LP);
    a.aS11 = adj_slot(c, AJ_S11); a.aS22 = adj_slot(c, AJ_S22); a.aS33 = adj_slot(c, AJ_S33);
    a.aT12 = adj_slot(c, AJ_T12); a.aT13 = adj_slot(c, AJ_T13); a.aT23 = adj_slot(c, AJ_T23);
    a.aV1 = adj_slot(c, AJ_V1); a.aV2 = adj_slot(c, AJ_V2); a.aV3 = adj_slot(c, AJ_V3); a.aP = adj_slot(c, AJ_P);
    a.gEta = adj_slot(c, AJ_GETA); a.gRho = adj_slot(c, AJ_GRHO);
    return a;
}

// Aᵀ λ (λ in the AJ_L* slots) into AJ_V*, AJ_P, with ∂R/∂η, ∂R/∂ρ contractions; with_bc: the
// transposed homogeneous BC program (interior-unknown form)
template <int G>
static int adj_apply(Ctx* c, KP<double>& p, bool with_bc) {
    Adj a = adj_ptrs(c);
    CK(cudaMemsetAsync(adj_slot(c, AJ_S11), 0, sizeof(double) * c->d.vol * (AJ_GRHO - AJ_S11 + 1), c->stream));
    k_vjp_momentum<G><<<grid_vel(c->d), blk2d(), 0, c->stream>>>(p, a);
    k_vjp_pressure<<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a);
    k_vjp_strain<G><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a);
    if (c->prm.rheology == SPH_RHEO_EDOT_POWER_RELAX)  // the law's dependence on V (Newton form) and its η_ini, n chain
        k_vjp_law<G, true><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a, adj_slot(c, AJ_GEI), adj_slot(c, AJ_GN));
    else
        CK(cudaMemcpyAsync(adj_slot(c, AJ_GEI), adj_slot(c, AJ_GETA), sizeof(double) * c->d.vol, cudaMemcpyDeviceToDevice, c->stream));
    if (with_bc) {
        KP<double> hp = p;
        hp.sig2 = 0.0; hp.sig3 = 0.0;
        for (auto it = c->bc.rbegin(); it != c->bc.rend(); ++it) {
            const BcStage& st = *it;
            int eu = st.dim == 0 ? c->d.n2 + 1 : c->d.n1 + 1;
            int ev = st.dim == 2 ? c->d.n2 + 1 : c->d.n3 + 1;
            dim3 g((eu + 31) / 32, (ev + 7) / 8, 1);
            k_bc_adjoint<G><<<g, blk2d(), 0, c->stream>>>(hp, a, st);
        }
    }
    CK(cudaGetLastError());
    return SPH_OK;
}

template <int G>
static int adjoint_solve_g(Ctx* c, const sph_solve_opts& o, sph_solve_info* inf) {
    KP<double> p = adj_kp<G>(c);
    Adj a = adj_ptrs(c);
    const int nout = o.nout > 0 ? o.nout : 100;
    // max|b|
    CK(cudaMemsetAsync(c->red, 0, sizeof(unsigned long long) * kRedSlots, c->stream));
    for (int s = 0; s < 4; ++s) launch_maxabs<double>(*c, adj_slot(c, AJ_B1 + s), nullptr, s);
    int rc = fetch_red(*c);
    if (rc) return rc;
    double bmax = 0.0;
    for (int s = 0; s < 4; ++s) bmax = std::max(bmax, slot_val(*c, s));
    if (bmax == 0.0) bmax = 1.0;
    for (int s = AJ_M11; s <= AJ_M23; ++s) CK(cudaMemsetAsync(adj_slot(c, s), 0, sizeof(double) * c->d.vol, c->stream));
    const bool law = c->prm.rheology == SPH_RHEO_EDOT_POWER_RELAX;
    dim3 gu((c->d.n1 + 1 + 31) / 32, (c->d.n2 + 1 + 7) / 8, c->d.n3 + 1);
    int64_t it = 0;
    double err = 1.0;
    int status = SPH_ERR_NOT_CONVERGED;
    while (it < o.maxiter) {
        ++it;
        // M_τᵀ λ_V (σ adjoints -> τ adjoints) and M_Pᵀ λ_V
        CK(cudaMemsetAsync(adj_slot(c, AJ_S11), 0, sizeof(double) * c->d.vol * (AJ_GRHO - AJ_S11 + 1), c->stream));
        k_vjp_momentum<G><<<grid_vel(c->d), blk2d(), 0, c->stream>>>(p, a);
        k_vjp_pressure<<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a);
        k_adj_pressure_update<<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a, adj_slot(c, AJ_LP), adj_slot(c, AJ_BP));
        k_adj_memory<<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a, adj_slot(c, AJ_M11), adj_slot(c, AJ_M22), adj_slot(c, AJ_M33),
                                                                  adj_slot(c, AJ_M12), adj_slot(c, AJ_M13), adj_slot(c, AJ_M23));
        k_vjp_strain<G><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a);  // Eᵀ μ + Dᵀ λ_P
        if (law) k_vjp_law<G, true><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, a, adj_slot(c, AJ_GEI), adj_slot(c, AJ_GN));
        {
            KP<double> hp = p;
            hp.sig2 = 0.0; hp.sig3 = 0.0;
            for (auto st = c->bc.rbegin(); st != c->bc.rend(); ++st) {
                int eu = st->dim == 0 ? c->d.n2 + 1 : c->d.n1 + 1;
                int ev = st->dim == 2 ? c->d.n2 + 1 : c->d.n3 + 1;
                dim3 g((eu + 31) / 32, (ev + 7) / 8, 1);
                k_bc_adjoint<G><<<g, blk2d(), 0, c->stream>>>(hp, a, *st);
            }
        }
        k_adj_velocity_update<<<grid_vel(c->d), blk2d(), 0, c->stream>>>(p, a, adj_slot(c, AJ_LV1), adj_slot(c, AJ_LV2), adj_slot(c, AJ_LV3),
                                                                         adj_slot(c, AJ_B1), adj_slot(c, AJ_B2), adj_slot(c, AJ_B3));
        if (it % nout) continue;
        // convergence: the transposed residual Aᵀλ - b of the current λ
        if ((rc = adj_apply<G>(c, p, true))) return rc;
        k_adj_residual<<<gu, blk2d(), 0, c->stream>>>(p, a, adj_slot(c, AJ_B1), adj_slot(c, AJ_B2), adj_slot(c, AJ_B3), adj_slot(c, AJ_BP),
                                                      adj_slot(c, AJ_R1), adj_slot(c, AJ_R2), adj_slot(c, AJ_R3), adj_slot(c, AJ_RP));
        CK(cudaMemsetAsync(c->red, 0, sizeof(unsigned long long) * kRedSlots, c->stream));
        for (int s = 0; s < 4; ++s) launch_maxabs<double>(*c, adj_slot(c, AJ_R1 + s), nullptr, s);
        if ((rc = fetch_red(*c))) return rc;
        double r = 0.0;
        for (int s = 0; s < 4; ++s) r = std::max(r, slot_val(*c, s));
        err = r / bmax;
        if (!(err == err) || std::isinf(err)) { status = SPH_ERR_DIVERGED; break; }
        if (err < o.tol) { status = SPH_OK; break; }
    }
    inf->iters = it;
    inf->err = err;
    inf->residual = err;
    inf->status = status;
    return SPH_OK;
}

extern "C" {

int sph_set_field(void* h, int32_t field, const double* host, int64_t count) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (!host) return fail(SPH_ERR_INVALID, "host pointer is NULL");
    int rc = sync64(*c);
    if (rc) return rc;
    rc = copy_field(c, field, nullptr, host, count);
    if (rc) return rc;
    if (field == SPH_FIELD_RHO || field == SPH_FIELD_TOP_LOAD) return compute_f_scale(*c);
    return SPH_OK;
}

int sph_get_field(void* h, int32_t field, double* host, int64_t count) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (!host) return fail(SPH_ERR_INVALID, "host pointer is NULL");
    return copy_field(c, field, host, nullptr, count);
}

int sph_step(void* h, int64_t k) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (k < 0) return fail(SPH_ERR_INVALID, "k < 0");
    const bool use32 = c->prm.precision != SPH_PREC_FP64;
    int rc = use32 ? sync32(*c) : sync64(*c);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev0, c->stream));
    for (int64_t i = 0; i < k; ++i) {
        if (use32) iterate_dispatch<float>(*c, c->s32);
        else iterate_dispatch<double>(*c, c->s64);
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    if (use32) c->stale64 = true;
    return SPH_OK;
}

int sph_solve(void* h, const sph_solve_opts* o, sph_solve_info* info, int64_t* hist_iter, double* hist_err, int64_t hist_cap) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !o) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    if (o->tol <= 0.0 || o->maxiter <= 0) return fail(SPH_ERR_INVALID, "tol and maxiter must be positive");
    if (o->criterion < SPH_CRIT_REFERENCE || o->criterion > SPH_CRIT_REFERENCE_PLATEAU) return fail(SPH_ERR_INVALID, "criterion");
    sph_solve_info local;
    std::memset(&local, 0, sizeof(local));
    sph_solve_info* inf = info ? info : &local;
    std::memset(inf, 0, sizeof(*inf));
    auto t0 = std::chrono::steady_clock::now();
    c->solve_t0 = t0;
    c->hist_ms.clear();
    c->sweep_ms = c->outer_ms = 0.0;
    CK(cudaEventRecord(c->ev0, c->stream));
    int rc;
    const int prec = c->prm.precision;
    if (prec == SPH_PREC_MIXED) {
        if (o->criterion != SPH_CRIT_RESIDUAL) return fail(SPH_ERR_UNSUPPORTED, "mixed precision stops on the FP64 residual (SPH_CRIT_RESIDUAL)");
        rc = sync64(*c);
        if (rc) return rc;
        switch (c->prm.geometry) {
            case SPH_GEOM_SPHERICAL: rc = solve_mixed_g<SPH>(*c, *o, inf, hist_iter, hist_err, hist_cap); break;
            case SPH_GEOM_CYLINDRICAL: rc = solve_mixed_g<CYL>(*c, *o, inf, hist_iter, hist_err, hist_cap); break;
            default: rc = solve_mixed_g<CART>(*c, *o, inf, hist_iter, hist_err, hist_cap); break;
        }
    } else if (prec == SPH_PREC_FP32) {
        rc = sync32(*c);
        if (!rc) rc = solve_plain<float>(*c, c->s32, true, *o, inf, hist_iter, hist_err, hist_cap);
        c->stale64 = true;
    } else {
        rc = sync64(*c);
        if (!rc) rc = solve_plain<double>(*c, c->s64, false, *o, inf, hist_iter, hist_err, hist_cap);
        c->stale32 = true;
    }
    if (rc) return rc;
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    inf->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    inf->device_ms = ms;
    inf->sweep_ms = prec == SPH_PREC_MIXED ? c->sweep_ms : ms;
    inf->outer_ms = c->outer_ms;
    // the FP64 residual of the final state: the mixed solve's last outer step evaluated it (its
    // loop ends right after a residual evaluation; the final P and τ copies leave it unchanged)
    if (prec != SPH_PREC_MIXED) {
        rc = sync64(*c);
        if (rc) return rc;
        double out[7];
        rc = residual64(*c, out);
        if (rc) return rc;
        inf->residual = out[6];
    }
    return inf->status;
}

int sph_sweep(void* h, int64_t k) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (c->prm.precision != SPH_PREC_MIXED) return fail(SPH_ERR_UNSUPPORTED, "sph_sweep needs SPH_PREC_MIXED");
    if (k < 0) return fail(SPH_ERR_INVALID, "k < 0");
    if (c->prm.rheology == SPH_RHEO_TAU_POWER || c->prm.rheology == SPH_RHEO_TAU_POWER_RELAX)
        return fail(SPH_ERR_UNSUPPORTED, "mixed precision needs an explicit viscosity law (linear or strain-rate power law)");
    const int G = c->prm.geometry;
    int rc = ensure_correction(*c);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev0, c->stream));
    const int chunk = 100;
    for (int64_t done = 0; done < k;) {
        const int m = (int)std::min<int64_t>(chunk, k - done);
        rc = G == SPH ? run_correction_sweeps<SPH>(*c, m) : (G == CYL ? run_correction_sweeps<CYL>(*c, m) : run_correction_sweeps<CART>(*c, m));
        if (rc) return rc;
        done += m;
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    return check_kernel_flag(*c);
}

int sph_residual_fields(void* h, double* rV1, double* rV2, double* rV3, double* rP) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    int rc = sync64(*c);
    if (rc) return rc;
    double out[7];
    if ((rc = residual64(*c, out))) return rc;
    const int slots[4] = {F_RV1, F_RV2, F_RV3, F_RP};
    const int fields[4] = {SPH_FIELD_V1, SPH_FIELD_V2, SPH_FIELD_V3, SPH_FIELD_P};
    double* hs[4] = {rV1, rV2, rV3, rP};
    for (int i = 0; i < 4; ++i) {
        if (!hs[i]) continue;
        int e[3];
        field_extent(c->d, fields[i], e);
        if ((rc = copy_slot_out(c, slots[i], e, hs[i]))) return rc;
    }
    return SPH_OK;
}

int sph_residual_vjp(void* h, const double* lV1, const double* lV2, const double* lV3, const double* lP, double* aV1, double* aV2,
                     double* aV3, double* aP, double* g_eta, double* g_rho, int32_t flags) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    int rc = sync64(*c);
    if (rc || (rc = adj_alloc(c))) return rc;
    if ((rc = adj_upload(c, AJ_LV1, SPH_FIELD_V1, lV1)) || (rc = adj_upload(c, AJ_LV2, SPH_FIELD_V2, lV2)) ||
        (rc = adj_upload(c, AJ_LV3, SPH_FIELD_V3, lV3)) || (rc = adj_upload(c, AJ_LP, SPH_FIELD_P, lP)))
        return rc;
    const int G = c->prm.geometry;
    const bool bc = (flags & 1) != 0;
    if (G == SPH) { KP<double> p = adj_kp<SPH>(c); rc = adj_apply<SPH>(c, p, bc); }
    else if (G == CYL) { KP<double> p = adj_kp<CYL>(c); rc = adj_apply<CYL>(c, p, bc); }
    else { KP<double> p = adj_kp<CART>(c); rc = adj_apply<CART>(c, p, bc); }
    if (rc) return rc;
    if ((rc = adj_download(c, AJ_V1, SPH_FIELD_V1, aV1)) || (rc = adj_download(c, AJ_V2, SPH_FIELD_V2, aV2)) ||
        (rc = adj_download(c, AJ_V3, SPH_FIELD_V3, aV3)) || (rc = adj_download(c, AJ_P, SPH_FIELD_P, aP)) ||
        (rc = adj_download(c, AJ_GETA, SPH_FIELD_P, g_eta)) || (rc = adj_download(c, AJ_GRHO, SPH_FIELD_P, g_rho)))
        return rc;
    CK(cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

int sph_advect(void* h, double dt, double delta, int32_t nf, const double* const* phi, double* const* phi_new) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || (nf > 0 && (!phi || !phi_new))) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    if (nf < 1 || nf > 4) return fail(SPH_ERR_INVALID, "sph_advect: 1 to 4 fields");
    int rc = sync64(*c);
    if (rc || (rc = adj_alloc(c))) return rc;
    AdvFields F;
    F.nf = nf;
    for (int f = 0; f < nf; ++f) {
        if ((rc = adj_upload(c, AJ_B1 + f, SPH_FIELD_P, phi[f]))) return rc;
        F.in[f] = adj_slot(c, AJ_B1 + f);
        F.out[f] = adj_slot(c, AJ_R1 + f);
    }
    KP<double> p = make_kp<double>(*c, c->s64);
    const int G = c->prm.geometry;
    if (G == SPH) k_advect<SPH><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, F, dt, delta);
    else if (G == CYL) k_advect<CYL><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, F, dt, delta);
    else k_advect<CART><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, F, dt, delta);
    CK(cudaGetLastError());
    for (int f = 0; f < nf; ++f)
        if ((rc = adj_download(c, AJ_R1 + f, SPH_FIELD_P, phi_new[f]))) return rc;
    return SPH_OK;
}

int sph_advect_vjp(void* h, double dt, double delta, int32_t nf, const double* const* phi, const double* const* mu_new, double* const* mu,
                   double* aV1, double* aV2, double* aV3) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !phi || !mu_new || !mu) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    if (nf < 1 || nf > 4) return fail(SPH_ERR_INVALID, "sph_advect_vjp: 1 to 4 fields");
    int rc = sync64(*c);
    if (rc || (rc = adj_alloc(c))) return rc;
    AdvFields F, M;
    F.nf = M.nf = nf;
    for (int f = 0; f < nf; ++f) {
        if ((rc = adj_upload(c, AJ_B1 + f, SPH_FIELD_P, phi[f])) || (rc = adj_upload(c, AJ_R1 + f, SPH_FIELD_P, mu_new[f])) ||
            (rc = adj_upload(c, AJ_M11 + f, SPH_FIELD_P, nullptr)))
            return rc;
        F.in[f] = adj_slot(c, AJ_B1 + f);
        M.in[f] = adj_slot(c, AJ_R1 + f);
        M.out[f] = adj_slot(c, AJ_M11 + f);
    }
    for (int s = AJ_V1; s <= AJ_V3; ++s) CK(cudaMemsetAsync(adj_slot(c, s), 0, sizeof(double) * c->d.vol, c->stream));
    KP<double> p = make_kp<double>(*c, c->s64);
    double *a1 = adj_slot(c, AJ_V1), *a2 = adj_slot(c, AJ_V2), *a3 = adj_slot(c, AJ_V3);
    const int G = c->prm.geometry;
    if (G == SPH) k_advect_vjp<SPH><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, F, M, a1, a2, a3, dt, delta);
    else if (G == CYL) k_advect_vjp<CYL><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, F, M, a1, a2, a3, dt, delta);
    else k_advect_vjp<CART><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, F, M, a1, a2, a3, dt, delta);
    CK(cudaGetLastError());
    for (int f = 0; f < nf; ++f)
        if ((rc = adj_download(c, AJ_M11 + f, SPH_FIELD_P, mu[f]))) return rc;
    if ((rc = adj_download(c, AJ_V1, SPH_FIELD_V1, aV1)) || (rc = adj_download(c, AJ_V2, SPH_FIELD_V2, aV2)) ||
        (rc = adj_download(c, AJ_V3, SPH_FIELD_V3, aV3)))
        return rc;
    return SPH_OK;
}

int sph_bc_vjp(void* h, double* aV1, double* aV2, double* aV3) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !aV1 || !aV2 || !aV3) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    int rc = sync64(*c);
    if (rc || (rc = adj_alloc(c))) return rc;
    if ((rc = adj_upload(c, AJ_V1, SPH_FIELD_V1, aV1)) || (rc = adj_upload(c, AJ_V2, SPH_FIELD_V2, aV2)) ||
        (rc = adj_upload(c, AJ_V3, SPH_FIELD_V3, aV3)))
        return rc;
    KP<double> p = make_kp<double>(*c, c->s64);
    p.sig2 = 0.0; p.sig3 = 0.0;
    Adj a = adj_ptrs(c);
    const int G = c->prm.geometry;
    for (auto st = c->bc.rbegin(); st != c->bc.rend(); ++st) {
        int eu = st->dim == 0 ? c->d.n2 + 1 : c->d.n1 + 1;
        int ev = st->dim == 2 ? c->d.n2 + 1 : c->d.n3 + 1;
        dim3 g((eu + 31) / 32, (ev + 7) / 8, 1);
        if (G == SPH) k_bc_adjoint<SPH><<<g, blk2d(), 0, c->stream>>>(p, a, *st);
        else if (G == CYL) k_bc_adjoint<CYL><<<g, blk2d(), 0, c->stream>>>(p, a, *st);
        else k_bc_adjoint<CART><<<g, blk2d(), 0, c->stream>>>(p, a, *st);
    }
    CK(cudaGetLastError());
    if ((rc = adj_download(c, AJ_V1, SPH_FIELD_V1, aV1)) || (rc = adj_download(c, AJ_V2, SPH_FIELD_V2, aV2)) ||
        (rc = adj_download(c, AJ_V3, SPH_FIELD_V3, aV3)))
        return rc;
    return SPH_OK;
}

int sph_residual_vjp_law(void* h, double* g_eta_ini, double* g_n) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (!c->adj) return fail(SPH_ERR_INVALID, "sph_residual_vjp_law: no sph_residual_vjp before");
    int rc = adj_download(c, AJ_GEI, SPH_FIELD_P, g_eta_ini);
    if (rc) return rc;
    if (g_n) {
        *g_n = 0.0;
        if (c->prm.rheology == SPH_RHEO_EDOT_POWER_RELAX) {
            std::vector<double> h((size_t)c->prm.n1 * c->prm.n2 * c->prm.n3);
            if ((rc = adj_download(c, AJ_GN, SPH_FIELD_P, h.data()))) return rc;
            for (double v : h) *g_n += v;
        }
    }
    return SPH_OK;
}

int sph_adjoint_solve(void* h, const double* bV1, const double* bV2, const double* bV3, const double* bP, double* lV1, double* lV2,
                      double* lV3, double* lP, const sph_solve_opts* o, sph_solve_info* info) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !o || !lV1 || !lV2 || !lV3 || !lP) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    if (o->tol <= 0.0 || o->maxiter <= 0) return fail(SPH_ERR_INVALID, "tol and maxiter must be positive");
    int rc = sync64(*c);
    if (rc || (rc = adj_alloc(c))) return rc;
    if ((rc = adj_upload(c, AJ_B1, SPH_FIELD_V1, bV1)) || (rc = adj_upload(c, AJ_B2, SPH_FIELD_V2, bV2)) ||
        (rc = adj_upload(c, AJ_B3, SPH_FIELD_V3, bV3)) || (rc = adj_upload(c, AJ_BP, SPH_FIELD_P, bP)) ||
        (rc = adj_upload(c, AJ_LV1, SPH_FIELD_V1, lV1)) || (rc = adj_upload(c, AJ_LV2, SPH_FIELD_V2, lV2)) ||
        (rc = adj_upload(c, AJ_LV3, SPH_FIELD_V3, lV3)) || (rc = adj_upload(c, AJ_LP, SPH_FIELD_P, lP)))
        return rc;
    for (int s = AJ_R1; s <= AJ_RP; ++s) CK(cudaMemsetAsync(adj_slot(c, s), 0, sizeof(double) * c->d.vol, c->stream));
    sph_solve_info local;
    std::memset(&local, 0, sizeof(local));
    sph_solve_info* inf = info ? info : &local;
    std::memset(inf, 0, sizeof(*inf));
    auto t0 = std::chrono::steady_clock::now();
    const int G = c->prm.geometry;
    rc = G == SPH ? adjoint_solve_g<SPH>(c, *o, inf) : (G == CYL ? adjoint_solve_g<CYL>(c, *o, inf) : adjoint_solve_g<CART>(c, *o, inf));
    if (rc) return rc;
    inf->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if ((rc = adj_download(c, AJ_LV1, SPH_FIELD_V1, lV1)) || (rc = adj_download(c, AJ_LV2, SPH_FIELD_V2, lV2)) ||
        (rc = adj_download(c, AJ_LV3, SPH_FIELD_V3, lV3)) || (rc = adj_download(c, AJ_LP, SPH_FIELD_P, lP)))
        return rc;
    return inf->status;
}

int sph_save(void* h, const char* dir, int32_t num, double tol, double runtime_s, const int64_t* hist_iter, const double* hist_err,
             int64_t nhist) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !dir) return fail(SPH_ERR_INVALID, "sph_save: NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    if (nhist < 0 || (nhist > 0 && (!hist_iter || !hist_err))) return fail(SPH_ERR_INVALID, "sph_save: history");
    int rc = sync64(*c);
    if (rc) return rc;
    if (mkdir(dir, 0777) != 0 && errno != EEXIST) return fail(SPH_ERR_INVALID, std::string("sph_save: cannot create ") + dir);
    const std::string out = std::string(dir) + "/";
    const sph_params& q = c->prm;
    const int G = q.geometry;
    // Save_infos: the scripts print εnonl and the run time with %d, which Julia's Printf
    // renders for a Float64 as %.0f
    std::string txt = strf("%d %f %f %f %d %d %d %.0f %.0f", num, q.l1, q.l2, q.l3, q.n1, q.n2, q.n3, tol, runtime_s);
    if ((rc = write_file(out + std::to_string(num) + "_infos.inf", txt.data(), txt.size()))) return rc;
    if (G == SPH_GEOM_SPHERICAL)
        txt = strf("%d   %f  %f  %f    %f     %f   %f  %f, %f, %f, %f    , %f", num, q.eta0, q.rho0, q.rho_in, q.n_exp, q.tau_C, q.vr, q.g,
                   q.sh, q.r, q.radius, q.dmp);
    else if (G == SPH_GEOM_CYLINDRICAL)
        txt = strf("%d  %f  %f  %f    %f     %f   %f  %f  %f  %f  %f      %f", num, q.eta0, q.rho0, q.rho_in, q.n_exp, q.tau_C, q.vr, q.g,
                   q.sh, q.r, q.radius, q.dmp);
    else
        txt = strf("%d   %f  %f  %f    %f     %f   %f  %f  %f  %f      %f", num, q.eta0, q.rho0, q.rho_in, q.n_exp, q.tau_C, q.vr, q.g, q.sh,
                   q.radius, q.dmp);
    if ((rc = write_file(out + std::to_string(num) + "_phys.inf", txt.data(), txt.size()))) return rc;

    auto save = [&](const char* name, const std::vector<double>& a) {
        return write_file(out + "A_" + name + ".bin", a.data(), a.size() * sizeof(double));
    };
    auto save_field = [&](const char* name, int field) {
        int e[3];
        field_extent(c->d, field, e);
        std::vector<double> a((size_t)e[0] * e[1] * e[2]);
        int r = copy_field(c, field, a.data(), nullptr, (int64_t)a.size());
        return r ? r : save(name, a);
    };
    const int n1 = q.n1, n2 = q.n2, n3 = q.n3;
    const size_t nc = (size_t)n1 * n2 * n3;
    // coordinate grids of the cell centres ([xc for xc = X_i, yc = Y_i, zc = Z_i])
    std::vector<double> X(nc), Y(nc), Z(nc);
    for (int k = 0; k < n3; ++k)
        for (int j = 0; j < n2; ++j)
            for (int i = 0; i < n1; ++i) {
                const size_t t = i + (size_t)n1 * (j + (size_t)n2 * k);
                X[t] = c->hx1[i]; Y[t] = c->hx2[j]; Z[t] = c->hx3[k];
            }
    static const char* const kSph[] = {"R", "TH", "PH", "VR", "VTH", "VPH", "TAU_RR", "TAU_THTH", "TAU_PHPH", "TAU_RTH", "TAU_RPH", "TAU_THPH"};
    static const char* const kCyl[] = {"R", "TH", "Z", "VR", "VTH", "VZ", "TAU_RR", "TAU_THTH", "TAU_ZZ", "TAU_RTH", "TAU_RZ", "TAU_THZ"};
    static const char* const kCart[] = {"X3D", "Y3D", "Z3D", "VX", "VY", "VZ", "TAU_XX", "TAU_YY", "TAU_ZZ", "TAU_XY", "TAU_XZ", "TAU_YZ"};
    const char* const* nm = G == SPH_GEOM_SPHERICAL ? kSph : (G == SPH_GEOM_CYLINDRICAL ? kCyl : kCart);
    if ((rc = save(nm[0], X)) || (rc = save(nm[1], Y)) || (rc = save(nm[2], Z))) return rc;
    if ((rc = save_field("ETAS", SPH_FIELD_ETA)) || (rc = save_field("RHO", SPH_FIELD_RHO)) || (rc = save_field("P", SPH_FIELD_P))) return rc;
    const int vf[9] = {SPH_FIELD_V1, SPH_FIELD_V2, SPH_FIELD_V3, SPH_FIELD_TAU11, SPH_FIELD_TAU22, SPH_FIELD_TAU33,
                       SPH_FIELD_TAU12, SPH_FIELD_TAU13, SPH_FIELD_TAU23};
    for (int i = 0; i < 9; ++i)
        if ((rc = save_field(nm[3 + i], vf[i]))) return rc;
    if ((rc = save_field("TII", SPH_FIELD_TII))) return rc;
    if (G == SPH_GEOM_CYLINDRICAL) {
        // ρG = ρ·g, DIVV and the strain rates D_* of the current velocities
        std::vector<double> rho(nc);
        if ((rc = copy_field(c, SPH_FIELD_RHO, rho.data(), nullptr, (int64_t)nc))) return rc;
        for (double& v : rho) v *= q.g;
        if ((rc = save("RHOG", rho))) return rc;
        State<double>& st = c->s64;
        KP<double> p = make_kp<double>(*c, st);
        k_strain_out<double, CYL><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p, st.f[F_SDD], st.f[F_Q11], st.f[F_Q22], st.f[F_Q33],
                                                                                st.f[F_Q12], st.f[F_Q13], st.f[F_Q23]);
        CK(cudaGetLastError());
        static const char* const dn[7] = {"DIVV", "D_RR", "D_THTH", "D_ZZ", "D_RTH", "D_RZ", "D_THZ"};
        const int ds[7] = {F_SDD, F_Q11, F_Q22, F_Q33, F_Q12, F_Q13, F_Q23};
        const int df[7] = {SPH_FIELD_P, SPH_FIELD_P, SPH_FIELD_P, SPH_FIELD_P, SPH_FIELD_TAU12, SPH_FIELD_TAU13, SPH_FIELD_TAU23};
        for (int i = 0; i < 7; ++i) {
            int e[3];
            field_extent(c->d, df[i], e);
            std::vector<double> a((size_t)e[0] * e[1] * e[2]);
            if ((rc = copy_slot_out(c, ds[i], e, a.data())) || (rc = save(dn[i], a))) return rc;
        }
    }
    // err_evo / iter_evo: Data.Array(...) of the scripts, i.e. Float64
    std::vector<double> ev((size_t)nhist), it((size_t)nhist);
    for (int64_t i = 0; i < nhist; ++i) { ev[i] = hist_err[i]; it[i] = (double)hist_iter[i]; }
    if ((rc = save("err_evo", ev)) || (rc = save("iter_evo", it))) return rc;
    return SPH_OK;
}

int sph_sweep_profile(void* h, int64_t k, double* sweep_ms, double* kernel_ms) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !sweep_ms || !kernel_ms) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    if (k < 0) return fail(SPH_ERR_INVALID, "k < 0");
    if (!c->fused) return fail(SPH_ERR_UNSUPPORTED, "sph_sweep_profile times the fused sweep kernel (SPH_KERNELS_AUTO)");
    *sweep_ms = 0.0;
    *kernel_ms = 0.0;
    if (k == 0) return SPH_OK;
    int rc = sph_sweep(h, 0);  // prepares the correction problem if needed
    if (rc) return rc;
    const size_t chunk = 256;  // launches timed between two host synchronisations
    while (c->prof_ev.size() < 2 * chunk) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        c->prof_ev.push_back(e);
    }
    const int G = c->prm.geometry;
    struct Restore {  // graphs back on and timing off on every return path
        Ctx* c;
        bool graphs;
        ~Restore() { c->use_graphs = graphs; c->prof_on = false; }
    } restore{c, c->use_graphs};
    c->use_graphs = false;  // one launch at a time, an event pair around each fused launch
    c->prof_on = true;
    for (int64_t done = 0; done < k;) {
        const int m = (int)std::min<int64_t>((int64_t)chunk, k - done);
        c->prof_next = 0;
        CK(cudaEventRecord(c->ev0, c->stream));
        rc = G == SPH ? run_correction_sweeps<SPH>(*c, m) : (G == CYL ? run_correction_sweeps<CYL>(*c, m) : run_correction_sweeps<CART>(*c, m));
        if (rc) break;
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaEventSynchronize(c->ev1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        *sweep_ms += ms;
        for (size_t i = 0; i < c->prof_next; ++i) {
            CK(cudaEventElapsedTime(&ms, c->prof_ev[2 * i], c->prof_ev[2 * i + 1]));
            *kernel_ms += ms;
        }
        done += m;
    }
    if (rc) return rc;
    c->last_ms = *sweep_ms;
    return check_kernel_flag(*c);
}

int sph_sweep_apply(void* h) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (!c->corr_ready) return SPH_OK;
    int rc = apply_correction(*c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

// FP32 slot and reference-layout extent of a correction-problem field (sph_corr_field)
static int corr_slot(const Ctx* c, int32_t field, int e[3]) {
    static const int slots[SPH_CORR_COUNT] = {F_P, F_V1, F_V2, F_V3, F_T11, F_T22, F_T33, F_T12, F_T13, F_T23,
                                              F_ETA, F_ETA_SM, F_RP, F_RV1, F_RV2, F_RV3};
    static const int shape[SPH_CORR_COUNT] = {SPH_FIELD_P, SPH_FIELD_V1, SPH_FIELD_V2, SPH_FIELD_V3, SPH_FIELD_TAU11,
                                              SPH_FIELD_TAU22, SPH_FIELD_TAU33, SPH_FIELD_TAU12, SPH_FIELD_TAU13, SPH_FIELD_TAU23,
                                              SPH_FIELD_P, SPH_FIELD_P, SPH_FIELD_P, SPH_FIELD_V1, SPH_FIELD_V2, SPH_FIELD_V3};
    if (field < 0 || field >= SPH_CORR_COUNT) return -1;
    field_extent(c->d, shape[field], e);
    return slots[field];
}

static int corr_access(void* h, int32_t field, double* host, const double* src, int64_t count) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (c->prm.precision != SPH_PREC_MIXED) return fail(SPH_ERR_UNSUPPORTED, "the correction problem exists in SPH_PREC_MIXED only");
    if (c->prm.rheology == SPH_RHEO_TAU_POWER || c->prm.rheology == SPH_RHEO_TAU_POWER_RELAX)
        return fail(SPH_ERR_UNSUPPORTED, "mixed precision needs an explicit viscosity law (linear or strain-rate power law)");
    if (!host && !src) return fail(SPH_ERR_INVALID, "host pointer is NULL");
    int e[3];
    const int slot = corr_slot(c, field, e);
    if (slot < 0) return fail(SPH_ERR_INVALID, "correction field");
    if (count != (int64_t)e[0] * e[1] * e[2]) return fail(SPH_ERR_INVALID, "count does not match the field size");
    int rc = ensure_correction(*c);
    if (rc) return rc;
    float* dev = c->s32.f[slot];
    return host ? download_box<float>(*c, dev, e, host) : upload_box<float>(*c, dev, e, src);
}

int sph_corr_get(void* h, int32_t field, double* host, int64_t count) {
    if (!host) return fail(SPH_ERR_INVALID, "host pointer is NULL");
    return corr_access(h, field, host, nullptr, count);
}

int sph_corr_set(void* h, int32_t field, const double* host, int64_t count) {
    if (!host) return fail(SPH_ERR_INVALID, "host pointer is NULL");
    return corr_access(h, field, nullptr, host, count);
}

int sph_selftest_wait_timeout(void* h) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (!c->d_err) {
        if (cudaMalloc((void**)&c->d_err, sizeof(int)) != cudaSuccess) return fail(SPH_ERR_NOMEM, "error word");
        CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    }
    // 1000 polls of at most 1 us each: the wait runs out within a few milliseconds
    k_wait_selftest<<<1, 32, 0, c->stream>>>(c->d_err, 1000, 1000u);
    CK(cudaGetLastError());
    return check_kernel_flag(*c);
}

int sph_residual(void* h, double out[7]) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !out) return fail(SPH_ERR_INVALID, "NULL argument");
    if (int rc_ = usable(*c)) return rc_;
    int rc = sync64(*c);
    if (rc) return rc;
    return residual64(*c, out);
}

int sph_run_kernel(void* h, int32_t kernel) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c) return fail(SPH_ERR_INVALID, "ctx is NULL");
    if (int rc_ = usable(*c)) return rc_;
    if (c->prm.precision != SPH_PREC_FP64) return fail(SPH_ERR_UNSUPPORTED, "single kernels run on the FP64 state");
    int rc = sync64(*c);
    if (rc) return rc;
    State<double>& s = c->s64;
    KP<double> p = make_kp<double>(*c, s);
    const int G = c->prm.geometry;
    switch (kernel) {
        case SPH_K_MAXLOC:
            if (G == SPH) launch_maxloc<double, SPH>(*c, p); else if (G == CYL) launch_maxloc<double, CYL>(*c, p); else launch_maxloc<double, CART>(*c, p);
            break;
        case SPH_K_COMPUTE_P:
            if (G == SPH) k_stress<double, SPH, false><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p);
            else if (G == CYL) k_stress<double, CYL, false><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p);
            else k_stress<double, CART, false><<<grid_cells(c->d), blk2d(), 0, c->stream>>>(p);
            break;
        case SPH_K_RHEOLOGY:
            if (G == SPH) launch_rheology<double, SPH>(*c, s, p); else if (G == CYL) launch_rheology<double, CYL>(*c, s, p); else launch_rheology<double, CART>(*c, s, p);
            break;
        case SPH_K_COMPUTE_V:
            if (G == SPH) k_velocity<double, SPH, 0><<<grid_vel(c->d), blk2d(), 0, c->stream>>>(p);
            else if (G == CYL) k_velocity<double, CYL, 0><<<grid_vel(c->d), blk2d(), 0, c->stream>>>(p);
            else k_velocity<double, CART, 0><<<grid_vel(c->d), blk2d(), 0, c->stream>>>(p);
            break;
        case SPH_K_BC:
            if (G == SPH) launch_bc<double, SPH>(*c, p, 0); else if (G == CYL) launch_bc<double, CYL>(*c, p, 0); else launch_bc<double, CART>(*c, p, 0);
            break;
        default: return fail(SPH_ERR_INVALID, "kernel id");
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

int sph_solve_history_ms(void* h, double* ms, int64_t cap, int64_t* n) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !n || (cap > 0 && !ms)) return fail(SPH_ERR_INVALID, "NULL argument");
    *n = (int64_t)c->hist_ms.size();
    for (int64_t i = 0; i < cap && i < *n; ++i) ms[i] = c->hist_ms[(size_t)i];
    return SPH_OK;
}

int sph_last_device_ms(void* h, double* ms) {
    Ctx* c = static_cast<Ctx*>(h);
    if (!c || !ms) return fail(SPH_ERR_INVALID, "NULL argument");
    *ms = c->last_ms;
    return SPH_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free exit check.  The scratch of k_maxabs (one reduction slot per
// array and quantity: [0, m) max|v - v_old|, [m, 2m) max|v|) is this static
// array instead of the context's cudaMalloc'd slots; every device that loads
// the library holds it (2 * SPH_NOALLOC_MAX_ARRAYS * 8 bytes) until exit.  All
// calls share it: each call clears the slots it uses before its reductions, so
// calls whose work overlaps on the GPU (other streams, other host threads) race.
static __device__ __align__(256) unsigned long long g_noalloc_red[2 * SPH_NOALLOC_MAX_ARRAYS];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_addr[kNoAllocMaxDevices] = {};  // device address of g_noalloc_red, per device

// once per device, with that device current: the device address of the static scratch
int noalloc_scratch(unsigned long long** out) {
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(SPH_ERR_UNSUPPORTED, "sph_check_err_noalloc: device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* a = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_red);
        if (e != cudaSuccess || !a)
            return fail(SPH_ERR_CUDA, std::string("sph_check_err_noalloc: cudaGetSymbolAddress of the static scratch: ") +
                                          cudaGetErrorString(e));
        g_noalloc_addr[dev] = static_cast<unsigned long long*>(a);
    }
    *out = g_noalloc_addr[dev];
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_check_err_noalloc(int32_t m, const double* const* v, const double* const* v_old, const int64_t* count, double* err,
                          void* stream) {
    if (!v || !v_old || !count || !err) return fail(SPH_ERR_INVALID, "sph_check_err_noalloc: NULL argument");
    if (m < 1 || m > SPH_NOALLOC_MAX_ARRAYS)
        return fail(SPH_ERR_INVALID, "sph_check_err_noalloc: m = " + std::to_string(m) + " arrays; its static scratch holds 1 to " +
                                         std::to_string(SPH_NOALLOC_MAX_ARRAYS));
    for (int i = 0; i < m; ++i) {
        if (!v[i] || !v_old[i]) return fail(SPH_ERR_INVALID, "sph_check_err_noalloc: NULL array pointer");
        if (count[i] < 1) return fail(SPH_ERR_INVALID, "sph_check_err_noalloc: count < 1");
    }
    unsigned long long* slots = nullptr;
    int rc = noalloc_scratch(&slots);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaMemsetAsync(slots, 0, sizeof(unsigned long long) * 2 * m, st));  // max-reductions start at 0
    for (int i = 0; i < m; ++i) {
        k_maxabs<double><<<ew_blocks(count[i]), 256, 0, st>>>(v[i], v_old[i], count[i], slots + i);
        k_maxabs<double><<<ew_blocks(count[i]), 256, 0, st>>>(v[i], nullptr, count[i], slots + m + i);
    }
    CK(cudaGetLastError());
    unsigned long long h[2 * SPH_NOALLOC_MAX_ARRAYS];
    CK(cudaMemcpyAsync(h, slots, sizeof(unsigned long long) * 2 * m, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // err = max_i max|v_i - v_old_i| / max|v_i| with NaN propagation (Julia's max)
    double e = 0.0;
    for (int i = 0; i < m; ++i) {
        double dv, vv;
        std::memcpy(&dv, &h[i], sizeof(double));
        std::memcpy(&vv, &h[m + i], sizeof(double));
        const double r = dv / vv;
        if (!(r == r)) { e = r; break; }
        e = std::max(e, r);
    }
    *err = e;
    return SPH_OK;
}

}  // extern "C"
