// swc_api.cu -- host orchestration and C ABI of the GB300 dual-particle SPH
// projection (see include/swc.h).  One context = one simulation on one GPU and
// one CUDA stream.  The CG loop runs from device-resident scalars; batches of
// iterations are replayed from captured CUDA graphs between host convergence
// checks.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <cstdio>
#include <cstring>
#include <numbers>
#include <string>
#include <vector>

#include "../../include/swc.h"
#include "swc_kernels.h"

using namespace swc;

namespace swc {
// allocations left before the armed failure (-1: none armed)
std::atomic<int64_t> g_fail_alloc_after{-1};

bool debug_alloc_should_fail() {
    int64_t k = g_fail_alloc_after.load();
    while (k >= 0) {
        if (g_fail_alloc_after.compare_exchange_weak(k, k - 1)) return k == 0;
    }
    return false;
}
}  // namespace swc

namespace {

constexpr int kPhases = 8;

struct HostCg {
    CgState st;
    int     nv;
    int     nbricks;
    int     mlp_err;
};

}  // namespace

struct swc_ctx {
    int             dim = 3;
    swc_scene       scene{};
    swc_solver_opts opts{};
    cudaStream_t    stream     = nullptr;
    bool            own_stream = false;
    int             device = 0, num_sms = 152;
    Lattice         L{};
    Phys            P{};
    Stencil         S{};
    StencilD        SD{};
    int             grid  = 1;  // grid of the 256-thread brick / streaming kernels
    int             sgrid = 1;  // resident grid of the CG SpMV (static brick striding, deterministic pq)
    int             rgrid = 1;  // grid of the other row-stencil kernels (one brick per block at a time)
    int             ggrid = 1;  // resident grid of the virtual gather (brick queue)
    int             pgrid = 1;  // resident grid of the pressure gradient (brick queue)
    int *           queues = nullptr;  // brick queues: gather [0, 2), gradient [2, 4)
    std::string     err;

    // real particles (sorted by cell)
    long long  n = 0;
    float4 *   pos = nullptr, *vel = nullptr, *vel2 = nullptr;
    int *      id = nullptr;
    float *    rho = nullptr;
    float *    vol_by_id = nullptr;
    double *   stage = nullptr;  // FP64 host-format staging (2 * n * dim)
    int *      pleft = nullptr;  // particle pairs left to the single-particle pass: [count, done, pair ids]
    int *      cellStart = nullptr;
    SortScratch sortR{};

    // boundary particles
    long long  nb = 0;
    float4 *   bpos = nullptr, *bvel = nullptr, *bnrm = nullptr;
    int *      bid = nullptr;
    float *    brho = nullptr;
    int *      bcellStart = nullptr;
    SortScratch sortB{};
    bool       has_motion = false;
    double     motion_c[3] = {0, 0, 0};
    double     motion_omega = 0;
    double *   bstage = nullptr;

    // lattice
    NodeArrays  N{};
    BrickArrays B{};
    unsigned char * pflag = nullptr;  // bricks holding real particles (own cell)
    int *           plist = nullptr;
    int *           pcount = nullptr;
    unsigned char * bnear = nullptr;  // bricks within reach of boundary particles
    unsigned char * bcell = nullptr;  // node cells within reach of boundary particles
    unsigned char * bcell_tmp = nullptr;
    // learned warm start / training-data logging
    float * mlp_params = nullptr;  // SWC_MLP_PARAMS
    float * mlp_norm   = nullptr;  // SWC_MLP_NORM
    bool    mlp_ready  = false;
    int *   mlp_err    = nullptr;
    int *   slot_of    = nullptr;  // compact index -> slot
    float * xprev      = nullptr;  // node-mapped previous pressure (brick layout)
    float * feat_buf   = nullptr;  // logged features (reference order, 6 per node)
    float * tgt_buf    = nullptr;  // logged targets
    bool    features_valid = false;
    // extrapolated warm start: consecutive advance steps whose solution history
    // (N.xm1, flags two steps back) is valid, and whether this step shifted the flags
    int     extrap_steps   = 0;
    bool    extrap_shifted = false;
    // learned-start gate: consecutive rejections by the residual test, steps left to skip
    int     gate_rejects = 0;
    int     gate_skip    = 0;
    int     gate_windows = 0;  // skip windows since the prediction was last kept
    float *     pcomp = nullptr;    // last solution in reference order (prefix warm start)
    int *       nv_prev = nullptr;
    bool        pcomp_stale = false;  // the last projection did not export pcomp (other warm-start modes)
    int *       scan_tiles = nullptr;
    CgState *   cg = nullptr;
    double *    partials = nullptr;
    HostCg *    hcg = nullptr;  // pinned
    unsigned long long * diag_bits = nullptr;
    unsigned long long * vmax_bits = nullptr;  // max |v|^2 (swc_get_time_step)
    int *       max_bits = nullptr;
    double *    res2 = nullptr;
    cudaGraphExec_t g1 = nullptr, g8 = nullptr;

    bool   initialized = false;
    double rho0 = 0, alpha0 = -1e6, kappa = 0;
    int    last_iters = 16;
    bool   profiling = false;
    cudaEvent_t ev[kPhases + 2] = {};
    cudaEvent_t evA = nullptr, evB = nullptr;
    double phase_ms[kPhases] = {};
};

namespace {

#define CK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            if (c) c->err = std::string(#call) + ": " + cudaGetErrorString(e_);                                        \
            return e_ == cudaErrorMemoryAllocation ? SWC_OUT_OF_MEMORY : SWC_CUDA_ERROR;                               \
        }                                                                                                              \
    } while (0)

template<class T> int dalloc(swc_ctx * c, T ** p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (count == 0) count = 1;
    if (debug_alloc_should_fail()) {
        c->err = "cudaMalloc: out of memory (injected)";
        return SWC_OUT_OF_MEMORY;
    }
    CK(cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * count));
    return SWC_OK;
}
template<class T> void dfree(T *& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

double kernelW(double dist, double h, int dim) {
    const double inv_h = 1 / h, inv_h2 = 1 / (h * h);
    const double c0 = std::numbers::inv_pi * inv_h2 * (dim == 2 ? 40.0 / 7 : 8 * inv_h);
    const double x  = dist * inv_h;
    if (x < .5) return c0 * (6 * x * x * (x - 1) + 1);
    if (x < 1) return c0 * 2 * (1 - x) * (1 - x) * (1 - x);
    return 0;
}
double kernelDW(double dist, double h, int dim) {
    const double inv_h = 1 / h, inv_h2 = 1 / (h * h);
    const double c0 = std::numbers::inv_pi * inv_h2 * (dim == 2 ? 40.0 / 7 : 8 * inv_h);
    const double c1 = 6 * inv_h * c0;
    const double x  = dist * inv_h;
    if (x < .5) return c1 * x * (3 * x - 2);
    if (x < 1) return c1 * (1 - x) * (x - 1);
    return 0;
}

int alloc_sort(swc_ctx * c, SortScratch & S, long long n, bool aux) {
    int rc;
    if ((rc = dalloc(c, &S.key, n))) return rc;
    if ((rc = dalloc(c, &S.rank, n))) return rc;
    if ((rc = dalloc(c, &S.perm, n))) return rc;
    if ((rc = dalloc(c, &S.count, c->L.ncells))) return rc;
    if ((rc = dalloc(c, &S.tiles, scan_tile_count(c->L.ncells + 1) + 2))) return rc;
    if ((rc = dalloc(c, &S.pos2, n))) return rc;
    if ((rc = dalloc(c, &S.vel2, n))) return rc;
    if (aux && (rc = dalloc(c, &S.aux2, n))) return rc;
    if ((rc = dalloc(c, &S.id2, n))) return rc;
    return SWC_OK;
}
void free_sort(SortScratch & S) {
    dfree(S.key);
    dfree(S.rank);
    dfree(S.perm);
    dfree(S.count);
    dfree(S.tiles);
    dfree(S.pos2);
    dfree(S.vel2);
    dfree(S.aux2);
    dfree(S.id2);
}

// Pressure history of the extrapolated and learned warm starts (allocated on
// demand, empty history).
int ensure_extrap_buffers(swc_ctx * c) {
    if (c->N.xm1) return SWC_OK;
    const size_t slots = size_t(c->L.nbricks) * (c->dim == 3 ? 512 : 256);
    int rc;
    if ((rc = dalloc(c, &c->N.flag_m2, slots)) || (rc = dalloc(c, &c->N.flag_m3, slots)) ||
        (rc = dalloc(c, &c->B.flag_m2, size_t(c->L.nbricks))) || (rc = dalloc(c, &c->B.flag_m3, size_t(c->L.nbricks))) ||
        (rc = dalloc(c, &c->N.xm2, slots)) || (rc = dalloc(c, &c->N.xm1, slots)))
        return rc;
    CK(cudaMemset(c->N.flag_m2, 0, slots));
    CK(cudaMemset(c->N.flag_m3, 0, slots));
    CK(cudaMemset(c->B.flag_m2, 0, size_t(c->L.nbricks)));
    CK(cudaMemset(c->B.flag_m3, 0, size_t(c->L.nbricks)));
    CK(cudaMemset(c->N.xm1, 0, sizeof(float) * slots));
    CK(cudaMemset(c->N.xm2, 0, sizeof(float) * slots));
    c->extrap_steps = 0;
    // the CG graphs captured the old NodeArrays: recapture
    if (c->g1) cudaGraphExecDestroy(c->g1);
    if (c->g8) cudaGraphExecDestroy(c->g8);
    c->g1 = c->g8 = nullptr;
    return SWC_OK;
}

// Buffers of the learned warm start and of training-data logging (allocated on demand).
int ensure_learn_buffers(swc_ctx * c) {
    if (c->slot_of) return SWC_OK;
    const size_t slots = size_t(c->L.nbricks) * (c->dim == 3 ? 512 : 256);
    int rc;
    if ((rc = dalloc(c, &c->mlp_err, 1)) || (rc = dalloc(c, &c->slot_of, size_t(c->L.ncells))) ||
        (rc = dalloc(c, &c->xprev, slots)) || (rc = dalloc(c, &c->feat_buf, size_t(c->L.ncells) * SWC_MLP_IN)) ||
        (rc = dalloc(c, &c->tgt_buf, size_t(c->L.ncells))))
        return rc;
    if (!c->N.nreal && (rc = dalloc(c, &c->N.nreal, slots))) return rc;
    if ((rc = ensure_extrap_buffers(c))) return rc;
    if (!c->N.d2p && (rc = dalloc(c, &c->N.d2p, slots))) return rc;
    CK(cudaMemset(c->N.d2p, 0, sizeof(float) * slots));
    CK(cudaMemset(c->mlp_err, 0, sizeof(int)));
    // the CG graphs captured the old NodeArrays (feature pointers): recapture
    if (c->g1) cudaGraphExecDestroy(c->g1);
    if (c->g8) cudaGraphExecDestroy(c->g8);
    c->g1 = c->g8 = nullptr;
    return SWC_OK;
}

void setup_phys(swc_ctx * c) {
    const swc_scene & s = c->scene;
    const int dim       = s.dim;
    Phys & P            = c->P;
    const double h = s.particle_radius * 4, H = s.grid_spacing * 4;
    auto coeffs = [&](double kr, float & inv, float & c0, float & c1) {
        const double ih = 1 / kr, ih2 = 1 / (kr * kr);
        const double k0 = std::numbers::inv_pi * ih2 * (dim == 2 ? 40.0 / 7 : 8 * ih);
        inv = float(ih);
        c0  = float(k0);
        c1  = float(6 * ih * k0);
    };
    P.h  = float(h);
    P.h2 = float(h * h);
    coeffs(h, P.inv_h, P.c0h, P.c1h);
    P.H  = float(H);
    P.H2 = float(H * H);
    coeffs(H, P.inv_H, P.c0H, P.c1H);
    P.h_d     = h;
    P.inv_h_d = 1 / h;
    // |d|^2 within tie2 of h^2 is re-decided in FP64 where a jump at h matters
    // (rho_I sums W_H cut at h): a few relative roundings of the FP32 square,
    // whose offsets come from float-float node positions
    P.tie2 = float(8e-6 * h * h);
    P.c0h_d   = std::numbers::inv_pi * (1 / (h * h)) * (dim == 2 ? 40.0 / 7 : 8 * (1 / h));
    P.mass    = float(s.mass);
    P.inv_mass = float(1.0 / s.mass);
    P.bmass   = float(s.boundary_mass);
    P.rho0    = float(c->rho0 > 0 ? c->rho0 : 1.0);
    P.kappa   = float(c->kappa);
    P.alpha0  = float(c->alpha0);
    double ratio = h / s.grid_spacing;
    if (std::fabs(ratio - std::round(ratio)) < 1e-9) ratio = std::round(ratio);
    P.cell_lo    = int(std::floor(-ratio));
    P.cell_hi    = int(std::ceil(ratio)) - 1;
    P.gx         = float(s.gravity[0]);
    P.gy         = float(s.gravity[1]);
    P.gz         = float(s.gravity[2]);
    P.viscosity  = float(s.viscosity);
    P.gravity_on = s.enable_gravity ? 1 : 0;
    // virtual stencil: c(|k|^2) = 2 W'_H(r) / (r + 1e-6), r = |k| * spacing
    // (alpha_IJ / V_J of VirtualParticle::calculateCoef, VirtualParticle.cpp:157)
    for (int r2 = 0; r2 < 16; r2++) {
        const double r = std::sqrt(double(r2)) * s.grid_spacing;
        const double v = r2 == 0 ? 0.0 : 2.0 * kernelDW(r, H, dim) / (r + 1e-6);
        c->SD.c[r2]    = v;
        c->S.c[r2]     = float(v);
    }
}

// advect_dt != 0: the particles move by v dt first (advection fused into the count pass)
template<int DIM> int run_bin_real(swc_ctx * c, float advect_dt = 0.f) {
    float4 * no_aux = nullptr;
    launch_bin<DIM>(c->L, c->n, c->pos, c->vel, no_aux, c->id, c->sortR, c->cellStart, advect_dt, c->stream);
    return SWC_OK;
}
template<int DIM> int run_bin_boundary(swc_ctx * c) {
    launch_bin<DIM>(c->L, c->nb, c->bpos, c->bvel, c->bnrm, c->bid, c->sortB, c->bcellStart, 0.f, c->stream);
    launch_mark_bricks<DIM>(c->bcellStart, c->nb, c->L, c->P, c->bnear, nullptr, c->stream);
    launch_near_cells<DIM>(c->bcellStart, c->nb, c->L, c->P, c->bcell, c->bcell_tmp, c->stream);
    return SWC_OK;
}

inline void mark(swc_ctx * c, int k) {
    if (c->profiling) cudaEventRecord(c->ev[k], c->stream);
}

// Virtual generation: active bricks, fused gather, reference-order compaction,
// alpha_hat (VirtualParticle::generateParticles + calculateCoef diagonal).
// `features`: the step needs the learned warm start's per-node features (the
// real-neighbour counts of the gather); without them the gather skips the count.
template<int DIM> void run_generate(swc_ctx * c, bool with_ahat, bool features = true) {
    launch_mark_bricks<DIM>(c->cellStart, c->n, c->L, c->P, c->B.flag, c->pflag, c->stream);
    launch_brick_list(c->B.flag, c->L.nbricks, c->B.list, c->B.count, c->stream);
    launch_brick_list(c->pflag, c->L.nbricks, c->plist, c->pcount, c->stream);
    NodeArrays N = c->N;
    if (!features) N.nreal = nullptr;
    launch_node_gather<DIM>(c->L, c->P, c->B, N, c->pos, c->vel, c->cellStart, c->bpos, c->bvel, c->bcellStart,
                            c->bnear, c->bcell, c->ggrid, c->queues, c->stream);
    launch_segments<DIM>(c->L, c->B, c->N, c->scan_tiles, c->grid, c->stream);
    if (with_ahat) launch_ahat<DIM>(c->L, c->P, c->B, c->N, c->S, c->sgrid, c->stream);
}

int capture_graphs(swc_ctx * c) {
    for (int k = 0; k < 2; k++) {
        const int reps = k == 0 ? 1 : 8;
        cudaGraph_t g  = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < reps; i++) {
            if (c->dim == 2)
                launch_cg_iteration<2>(c->L, c->B, c->N, c->S, c->cg, c->partials, c->sgrid, c->grid, c->stream);
            else launch_cg_iteration<3>(c->L, c->B, c->N, c->S, c->cg, c->partials, c->sgrid, c->grid, c->stream);
        }
        CK(cudaStreamEndCapture(c->stream, &g));
        cudaGraphExec_t ge = nullptr;
        CK(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
        if (k == 0) c->g1 = ge;
        else c->g8 = ge;
    }
    return SWC_OK;
}

// CG solve from the warm start in N.x; fills stats.
// CG start from the current N.x; the device state is mirrored into hcg.
// CG start state on entry of run_cg: none (run_cg launches the initialisation),
// on the device only (launched by the caller), or also copied to the host.
enum { kInitNone = 0, kInitDevice = 1, kInitHost = 2 };

template<int DIM> int run_cg(swc_ctx * c, swc_stats * st, int init_mode) {
    if (!c->g1) {
        CK(cudaStreamSynchronize(c->stream));
        int rc = capture_graphs(c);
        if (rc) return rc;
    }
    if (init_mode != kInitHost) {
        // initial residual on the device; its state comes back with the first
        // convergence check (the iteration kernels are no-ops once CG is done)
        const int * nv = c->B.seg_off + c->B.nseg;
        if (init_mode == kInitNone)
            launch_cg_init<DIM>(c->L, c->B, c->N, c->S, c->cg, c->partials, c->opts.tolerance, c->opts.max_iterations,
                                nv, c->sgrid, c->grid, c->stream);
        c->hcg->st.done     = 0;
        c->hcg->st.iter     = 0;
        c->hcg->st.max_iter = c->opts.max_iterations >= 0 ? c->opts.max_iterations : std::numeric_limits<int>::max();
    }
    // first batch: the last solve's count and one more (one convergence check in
    // the common case; the iteration kernels are no-ops past convergence)
    int first   = c->opts.check_interval > 0 ? c->opts.check_interval : std::max(4, c->last_iters + 1);
    bool counts = init_mode == kInitHost;
    while (!c->hcg->st.done) {
        const int room = c->hcg->st.max_iter - c->hcg->st.iter;
        int m          = std::min(first, std::max(room, 1));
        for (; m >= 8; m -= 8) CK(cudaGraphLaunch(c->g8, c->stream));
        for (; m > 0; m--) CK(cudaGraphLaunch(c->g1, c->stream));
        CK(cudaMemcpyAsync(&c->hcg->st, c->cg, sizeof(CgState), cudaMemcpyDeviceToHost, c->stream));
        if (!counts) {
            CK(cudaMemcpyAsync(&c->hcg->nv, c->B.seg_off + c->B.nseg, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaMemcpyAsync(&c->hcg->nbricks, c->B.count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            counts = true;
        }
        CK(cudaStreamSynchronize(c->stream));
        first = c->opts.check_interval > 0 ? c->opts.check_interval : 8;
    }
    const double rr0 = c->hcg->st.rr0, bb = c->hcg->st.bb;
    const CgState & h = c->hcg->st;
    int status        = SWC_OK;
    if (h.done == 4) launch_zero_active<DIM>(c->L, c->B, c->N.x, c->grid, c->stream);  // b = 0 -> x = 0
    if (h.done == 2) status = SWC_CG_NOT_CONVERGED;
    if (h.done == 3) status = SWC_NAN_DETECTED;
    c->last_iters = std::max(1, h.iter);
    if (st) {
        st->n_virtual            = c->hcg->nv;
        st->active_bricks        = c->hcg->nbricks;
        st->cg_iterations        = h.iter;
        st->rhs_norm             = std::sqrt(bb);
        st->rel_residual         = bb > 0 ? std::sqrt(h.rr / bb) : 0.0;
        st->initial_rel_residual = bb > 0 ? std::sqrt(rr0 / bb) : 0.0;
        st->true_rel_residual    = -1;
        st->status               = status;
    }
    if (c->opts.compute_true_residual && st) {
        launch_true_residual<DIM>(c->L, c->B, c->N, c->S, c->cg, c->partials, c->res2, c->rgrid, c->stream);
        double r2[2];
        CK(cudaMemcpyAsync(r2, c->res2, sizeof(r2), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        st->true_rel_residual = r2[1] > 0 ? std::sqrt(r2[0] / r2[1]) : 0.0;
    }
    return status;
}

// p in reference order into pcomp and N_v into nv_prev (the prefix warm start's
// previous pressure vector, ParticlesBasedData.h:25-29).
template<int DIM> int export_prefix(swc_ctx * c) {
    launch_compact_export<DIM>(c->L, c->B, c->N, c->pcomp, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                               nullptr, nullptr, c->grid, c->stream);
    CK(cudaMemcpyAsync(c->nv_prev, c->B.seg_off + c->B.nseg, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
    c->pcomp_stale = false;
    return SWC_OK;
}

// The projection keeps a pressure history (extrapolated or learned warm start,
// training-data logging).
bool history_on(const swc_ctx * c) {
    const int mode = c->opts.warm_start;
    return c->N.xm1 && (mode == SWC_WARM_EXTRAPOLATE || (mode == SWC_WARM_LEARNED && c->mlp_ready) ||
                        (c->opts.keep_features && c->feat_buf));
}

// The shared tail of advance / project: virtual generation, projection, G_i.
template<int DIM> int run_projection(swc_ctx * c, swc_stats * st) {
    const int mode     = c->opts.warm_start;
    // the gate skips the network (base start) while it keeps losing the residual test
    const bool gated   = mode == SWC_WARM_LEARNED && c->mlp_ready && c->opts.learned_gate > 0 &&
                       !c->opts.learned_no_fallback && c->gate_skip > 0;
    if (gated) c->gate_skip--;
    const bool learned = mode == SWC_WARM_LEARNED && c->mlp_ready && !gated;
    const bool logging = c->opts.keep_features != 0 && c->feat_buf;
    mark(c, 3);
    // a step that runs neither the network nor the feature logging needs no features
    run_generate<DIM>(c, true, learned || logging);
    mark(c, 4);
    const int * nv     = c->B.seg_off + c->B.nseg;
    const size_t slots = size_t(c->L.nbricks) * BrickGeom<DIM>::BN;
    int used           = mode;
    int init_mode      = kInitNone;
    bool mlp_checked   = false, picked = false;
    // Pressure history (extrapolated and learned warm starts, logged features):
    // the base start is 3 p1 - 3 p2 + p3 with three steps of history, 2 p1 - p2
    // with two, p1 (node-mapped) with fewer; the history spans consecutive
    // advance calls.
    const bool hist_on  = history_on(c);
    const int history   = (hist_on && c->extrap_shifted) ? std::min(c->extrap_steps, 2) : 0;
    const int base_used = history >= 1 ? SWC_WARM_EXTRAPOLATE : SWC_WARM_NODE;
    if (mode == SWC_WARM_EXTRAPOLATE || mode == SWC_WARM_LEARNED) used = base_used;
    if (learned || logging) {
        // base start (and history shift): the fallback, the network's base and the target reference
        launch_warm_start<DIM>(c->L, c->B, c->N, kWarmExtrap, c->pcomp, c->nv_prev, nullptr, c->grid, c->stream,
                               history);
        const bool no_fallback = learned && c->opts.learned_no_fallback && !logging;
        const bool pick        = learned && !no_fallback;
        if (!no_fallback)
            CK(cudaMemcpyAsync(c->xprev, c->N.x, sizeof(float) * slots, cudaMemcpyDeviceToDevice, c->stream));
        if (logging) launch_slot_of<DIM>(c->L, c->B, c->N, c->slot_of, c->grid, c->stream);
        // |b|^2 for sD: from the base start's residual pass when the residual test
        // needs that pass anyway, else a reduction of its own
        const double * bb = &c->cg->bb;
        if (pick) {
            launch_cg_residual<DIM>(c->L, c->B, c->N, c->S, c->N.x, c->N.q, nullptr, c->cg->sums + 2, c->cg, c->partials,
                                    c->sgrid, c->grid, c->stream);
            bb = c->cg->sums + 3;
        }
        if (!pick || logging) launch_rhs_norm<DIM>(c->B, c->N, c->cg, c->partials, c->grid, c->stream);
        const float inv_a0 = float(1.0 / c->alpha0), inv_r0 = float(1.0 / c->rho0), inv_nr = 1.f / 32.f;
        if (logging)
            launch_node_features(c->N, c->slot_of, nv, c->L.ncells, c->cg, inv_a0, inv_r0, inv_nr, c->feat_buf,
                                 c->stream);
        if (learned) {
            launch_mlp_forward_nodes(c->mlp_params, c->mlp_norm, c->N, c->B, DIM == 3 ? 9 : 8, (long long) slots, bb,
                                     inv_a0, inv_r0, inv_nr, c->mlp_err, c->stream);
            CK(cudaMemcpyAsync(&c->hcg->mlp_err, c->mlp_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            mlp_checked = true;  // the error flag is read with CG's first check
            if (no_fallback) {
                used = SWC_WARM_LEARNED;  // CG initialises from the prediction
            } else {
                // residual test on the device: the prediction's residual against the
                // base start's (computed above), the smaller kept
                launch_cg_residual<DIM>(c->L, c->B, c->N, c->S, c->N.x, c->N.r, c->N.d, c->cg->sums, c->cg,
                                        c->partials, c->sgrid, c->grid, c->stream);
                launch_cg_pick<DIM>(c->B, c->N, c->xprev, c->N.q, c->mlp_err, false, c->cg, c->opts.tolerance,
                                    c->opts.max_iterations, nv, c->grid, c->stream);
                init_mode = kInitDevice;
                picked    = true;
            }
        } else if (mode == SWC_WARM_NODE) {
            // node-mapped previous pressure, kept in xm1 by the history shift
            CK(cudaMemcpyAsync(c->N.x, c->N.xm1, sizeof(float) * slots, cudaMemcpyDeviceToDevice, c->stream));
        } else if (mode != SWC_WARM_EXTRAPOLATE && mode != SWC_WARM_LEARNED) {
            launch_warm_start<DIM>(c->L, c->B, c->N, mode, c->pcomp, c->nv_prev, nullptr, c->grid, c->stream);
        }
    } else if (hist_on) {
        // the second differences are a feature: not written on a step without the network
        NodeArrays N = c->N;
        N.d2p        = nullptr;
        launch_warm_start<DIM>(c->L, c->B, N, kWarmExtrap, c->pcomp, c->nv_prev, nullptr, c->grid, c->stream, history);
    } else {
        launch_warm_start<DIM>(c->L, c->B, c->N, mode == SWC_WARM_LEARNED || mode == SWC_WARM_EXTRAPOLATE ? kWarmNode : mode,
                               c->pcomp, c->nv_prev, nullptr, c->grid, c->stream);
    }
    mark(c, 5);
    int rc = run_cg<DIM>(c, st, init_mode);
    if (picked) {
        used = c->hcg->st.start == 0 ? SWC_WARM_LEARNED : base_used;
        if (c->opts.learned_gate > 0) {
            c->gate_rejects = used == SWC_WARM_LEARNED ? 0 : c->gate_rejects + 1;
            if (used == SWC_WARM_LEARNED) c->gate_windows = 0;
            // after a window, the re-test's rejection alone starts the next one
            if (c->gate_rejects >= c->opts.learned_gate || (c->gate_windows > 0 && c->gate_rejects > 0)) {
                // the window doubles with every window since the prediction was last kept
                c->gate_skip    = (4 * c->opts.learned_gate) << std::min(c->gate_windows, 4);
                c->gate_windows++;
                c->gate_rejects = 0;
            }
        }
    }
    if (mlp_checked && c->hcg->mlp_err) {
        c->err = picked ? "learned warm start: the tensor-core pass timed out; CG ran from the base start"
                        : "learned warm start: the tensor-core pass timed out; CG ran from its output";
        used   = base_used;
    }
    c->extrap_steps   = (hist_on && c->extrap_shifted && (rc == SWC_OK || rc == SWC_CG_NOT_CONVERGED)) ? c->extrap_steps + 1 : 0;
    c->extrap_shifted = false;
    if (st) st->warm_start_used = used;
    if (logging && (rc == SWC_OK || rc == SWC_CG_NOT_CONVERGED)) {
        launch_mlp_targets(c->L.ncells, nv, c->slot_of, c->N.x, c->xprev, c->N.xm1, c->N.d2p, c->N.ahat, c->cg,
                           c->tgt_buf, c->stream);
        c->features_valid = true;
    }
    if (rc != SWC_OK && rc != SWC_CG_NOT_CONVERGED && rc != SWC_NAN_DETECTED) return rc;
    const int cg_status = rc;
    if (cg_status == SWC_NAN_DETECTED) {
        // report, leave the velocities unprojected and drop the poisoned warm start
        launch_zero_active<DIM>(c->L, c->B, c->N.x, c->grid, c->stream);
        CK(cudaMemsetAsync(c->nv_prev, 0, sizeof(int), c->stream));
        c->pcomp_stale = false;
        for (int k = 6; k <= 8; k++) mark(c, k);
        return cg_status;
    }
    mark(c, 6);
    launch_pressure_gradient<DIM>(c->L, c->P, c->B, c->N, c->plist, c->pcount, c->bnear, c->pos, c->vel,
                                  c->cellStart, c->bpos, c->bvel, c->bnrm, c->bcellStart, c->bcell, c->pgrid, c->queues + 2,
                                  c->stream);
    mark(c, 7);
    // p in reference order (the next step's prefix warm start) and N_v for it;
    // other modes skip it (a switch to the prefix mode exports the last solution)
    if (mode == SWC_WARM_PREFIX) {
        if ((rc = export_prefix<DIM>(c))) return rc;
    } else c->pcomp_stale = true;
    mark(c, 8);
    if (st) {
        st->n_particles     = c->n;
        st->n_boundary      = c->nb;
    }
    return cg_status;
}

// Activity flags of the previous step (and, for the extrapolated warm start on
// an advance, of the step before).  A projection without motion (swc_project)
// ends the extrapolation history.
void save_prev_flags(swc_ctx * c, bool move) {
    using namespace swc;
    const size_t bn = c->dim == 3 ? BrickGeom<3>::BN : BrickGeom<2>::BN;
    c->extrap_shifted = false;
    if (move && history_on(c)) {
        // rotate the history buffers (no kernel reads them inside the captured CG graphs)
        std::swap(c->N.flag_m3, c->N.flag_m2);
        std::swap(c->N.flag_m2, c->N.flag_prev);
        std::swap(c->B.flag_m3, c->B.flag_m2);
        std::swap(c->B.flag_m2, c->B.flag_prev);
        c->extrap_shifted = true;
    }
    cudaMemcpyAsync(c->N.flag_prev, c->N.flag, size_t(c->L.nbricks) * bn, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->B.flag_prev, c->B.flag, size_t(c->L.nbricks), cudaMemcpyDeviceToDevice, c->stream);
}

template<int DIM> int do_advance(swc_ctx * c, double dt, swc_stats * st, bool move) {
    CK(cudaEventRecord(c->evA, c->stream));
    mark(c, 0);
    save_prev_flags(c, move);
    if (move) {
        if (c->has_motion && c->nb > 0) {
            launch_rotate_boundary(c->bpos, c->bvel, c->bnrm, c->nb, float(c->motion_c[0]), float(c->motion_c[2]),
                                   float(c->motion_omega), float(dt), c->stream);
        }
    }
    if (move && c->has_motion && c->nb > 0) {
        // moving solids: rebin the boundary (the motion flag travels in bnrm.w)
        run_bin_boundary<DIM>(c);
    }
    run_bin_real<DIM>(c, move ? float(dt) : 0.f);
    mark(c, 1);
    launch_density<DIM>(c->pos, c->vel, c->rho, c->n, c->L, c->P, c->cellStart, c->pleft, c->stream);
    mark(c, 2);
    if (move) {
        launch_forces<DIM>(c->pos, c->vel, c->vel2, c->n, c->L, c->P, c->cellStart, float(dt), c->pleft, c->stream);
        std::swap(c->vel, c->vel2);
    }
    int rc = run_projection<DIM>(c, st);
    if (rc != SWC_OK && rc != SWC_CG_NOT_CONVERGED && rc != SWC_NAN_DETECTED) return rc;
    const int status = rc;
    CK(cudaEventRecord(c->evB, c->stream));
    CK(cudaEventSynchronize(c->evB));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->evA, c->evB);
    if (st) st->device_ms = ms;
    if (c->profiling) {
        for (int k = 0; k < kPhases; k++) {
            float t = 0;
            cudaEventElapsedTime(&t, c->ev[k], c->ev[k + 1]);
            c->phase_ms[k] = t;
        }
    }
    CK(cudaGetLastError());
    return status;
}

template<int DIM> int do_initialize(swc_ctx * c) {
    if (c->n <= 0) {
        c->err = "no particles";
        return SWC_BAD_ARG;
    }
    run_bin_real<DIM>(c);
    launch_density<DIM>(c->pos, c->vel, c->rho, c->n, c->L, c->P, c->cellStart, c->pleft, c->stream);
    launch_set_volume(c->pos, c->rho, c->n, float(c->scene.mass), c->stream);
    // V_i per particle id (travels with the particle)
    launch_scatter_w_to_id(c->pos, c->id, c->n, c->vol_by_id, c->stream);
    // rho0 = max rho_i (DualParticleSphLiquid.cpp:91)
    launch_max_positive(c->rho, c->n, c->max_bits, c->stream);
    int bits = 0;
    CK(cudaMemcpyAsync(&bits, c->max_bits, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    // boundary
    if (c->nb > 0) {
        run_bin_boundary<DIM>(c);
        launch_boundary_density<DIM>(c->bpos, c->bvel, c->brho, c->nb, c->L, c->P, c->bcellStart, c->stream);
    }
    CK(cudaStreamSynchronize(c->stream));
    float rmax = 0;
    std::memcpy(&rmax, &bits, sizeof(float));
    c->rho0   = c->scene.target_density > 0 ? c->scene.target_density : double(rmax);
    c->kappa  = c->scene.kappa >= 0 ? c->scene.kappa : 0.0;
    if (c->scene.kappa < 0) {
        const double r = c->scene.particle_radius, h = 4 * r;
        const int d    = c->dim;
        const double packed = d == 2 ? kernelW(0, h, d) + kernelW(r * 2, h, d) * 6 +
                                           kernelW(r * 2 * std::numbers::sqrt3, h, d) * 6
                                     : kernelW(0, h, d) + kernelW(r * 2, h, d) * 12 +
                                           kernelW(r * 2 * std::numbers::sqrt2, h, d) * 6 +
                                           kernelW(r * 2 * std::numbers::sqrt3, h, d) * 24;
        c->kappa = 1.0 / packed;
    }
    setup_phys(c);
    // alpha0 = max diagonal with the clamp off, in FP64 (VirtualParticle::setAlpha)
    run_generate<DIM>(c, false);
    launch_diag_max_f64<DIM>(c->L, c->B, c->N, c->SD, c->diag_bits, c->grid, c->stream);
    unsigned long long dbits = 0;
    CK(cudaMemcpyAsync(&dbits, c->diag_bits, sizeof(dbits), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double a0 = 0;
    std::memcpy(&a0, &dbits, sizeof(double));
    c->alpha0 = dbits ? a0 : -1e6;
    setup_phys(c);
    // no previous pressure: empty prefix, no extrapolation history
    c->extrap_steps = 0;
    c->pcomp_stale  = false;
    c->gate_rejects = c->gate_skip = c->gate_windows = 0;
    CK(cudaMemsetAsync(c->nv_prev, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->N.x, 0, sizeof(float) * size_t(c->L.nbricks) * (DIM == 3 ? 512 : 256), c->stream));
    CK(cudaMemsetAsync(c->N.flag, 0, size_t(c->L.nbricks) * (DIM == 3 ? 512 : 256), c->stream));
    CK(cudaMemsetAsync(c->B.flag, 0, size_t(c->L.nbricks), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    c->initialized = true;
    return SWC_OK;
}

bool valid_ctx(const swc_ctx * c) { return c != nullptr; }

}  // namespace

extern "C" {

void swc_default_solver_opts(swc_solver_opts * o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->tolerance      = 1e-6;
    o->max_iterations = -1;
    o->warm_start     = SWC_WARM_PREFIX;
}

const char * swc_status_str(int s) {
    switch (s) {
    case SWC_OK: return "ok";
    case SWC_CG_NOT_CONVERGED: return "CG did not converge";
    case SWC_NAN_DETECTED: return "NaN or breakdown detected";
    case SWC_BAD_ARG: return "bad argument";
    case SWC_CUDA_ERROR: return "CUDA error";
    case SWC_NOT_INITIALIZED: return "not initialized";
    case SWC_OUT_OF_MEMORY: return "out of device memory";
    default: return "unknown status";
    }
}

const char * swc_last_error(const swc_ctx * c) { return c ? c->err.c_str() : "null context"; }

int swc_create(const swc_scene * s, const swc_solver_opts * o, swc_ctx ** out) {
    if (!s || !out) return SWC_BAD_ARG;
    *out = nullptr;
    if ((s->dim != 2 && s->dim != 3) || !(s->particle_radius > 0) || !(s->grid_spacing > 0) || !(s->mass > 0) ||
        s->grid_size[0] < 1 || s->grid_size[1] < 1 || (s->dim == 3 && s->grid_size[2] < 1))
        return SWC_BAD_ARG;
    if (o && (o->warm_start < SWC_WARM_PREFIX || o->warm_start > SWC_WARM_EXTRAPOLATE)) return SWC_BAD_ARG;
    auto * c  = new swc_ctx();
    c->dim    = s->dim;
    c->scene  = *s;
    if (s->boundary_mass <= 0) c->scene.boundary_mass = s->mass;
    if (o) c->opts = *o;
    else swc_default_solver_opts(&c->opts);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        c->err = "no CUDA device";
        delete c;
        return SWC_CUDA_ERROR;
    }
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    Lattice & L = c->L;
    L.ox = float(s->grid_origin[0]);
    L.oy = float(s->grid_origin[1]);
    L.oz = float(s->dim == 3 ? s->grid_origin[2] : 0.0);
    L.ox_d = s->grid_origin[0];
    L.oy_d = s->grid_origin[1];
    L.oz_d = s->dim == 3 ? s->grid_origin[2] : 0.0;
    L.dx   = float(s->grid_spacing);
    L.dx_d = s->grid_spacing;
    L.inv_dx = float(1.0 / s->grid_spacing);
    L.nx = s->grid_size[0];
    L.ny = s->grid_size[1];
    L.nz = s->dim == 3 ? s->grid_size[2] : 1;
    const int bx = s->dim == 3 ? 8 : 16, by = s->dim == 3 ? 8 : 16, bz = s->dim == 3 ? 8 : 1;
    L.bnx = (L.nx + bx - 1) / bx;
    L.bny = (L.ny + by - 1) / by;
    L.bnz = (L.nz + bz - 1) / bz;
    L.nbricks = L.bnx * L.bny * L.bnz;
    L.ncells  = (long long) L.nx * L.ny * L.nz;
    if ((long long) L.nbricks * bx * by * bz > (1LL << 31) - 1 || L.ncells > (1LL << 31) - 2) {
        c->err = "node grid too large";
        delete c;
        return SWC_BAD_ARG;
    }
    c->grid  = std::max(1, std::min(L.nbricks, c->num_sms * 8));
    c->rgrid = std::max(1, std::min(L.nbricks, c->num_sms * 10));
    {
        const bool d3 = s->dim == 3;
        const int so  = d3 ? cg_spmv_blocks_per_sm<3>() : cg_spmv_blocks_per_sm<2>();
        const int go  = d3 ? node_gather_blocks_per_sm<3>() : node_gather_blocks_per_sm<2>();
        const int po  = d3 ? pressure_gradient_blocks_per_sm<3>() : pressure_gradient_blocks_per_sm<2>();
        c->sgrid      = std::max(1, std::min(L.nbricks, c->num_sms * so));
        c->ggrid      = std::max(1, std::min(L.nbricks, c->num_sms * go));
        c->pgrid      = std::max(1, std::min(L.nbricks, c->num_sms * po));
    }
    const size_t npart = 3 * size_t(std::max({c->grid, c->sgrid, c->rgrid})) + 8;
    setup_phys(c);
    int rc = SWC_OK;
    const size_t slots = size_t(L.nbricks) * bx * by * bz;
    auto fail = [&](int r) {
        swc_destroy(c);
        return r;
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SWC_CUDA_ERROR);
    c->own_stream = true;
    if ((rc = dalloc(c, &c->N.flag, slots)) || (rc = dalloc(c, &c->N.flag_prev, slots)) ||
        (rc = dalloc(c, &c->N.V, slots)) || (rc = dalloc(c, &c->N.D, slots)) || (rc = dalloc(c, &c->N.rho, slots)) ||
        (rc = dalloc(c, &c->N.ahat, slots)) || (rc = dalloc(c, &c->N.x, slots)) || (rc = dalloc(c, &c->N.r, slots)) ||
        (rc = dalloc(c, &c->N.q, slots)) || (rc = dalloc(c, &c->N.d, slots)) || (rc = dalloc(c, &c->N.u, slots)))
        return fail(rc);
    if (c->opts.keep_virtual_velocity && (rc = dalloc(c, &c->N.vbar, slots))) return fail(rc);
    if (c->opts.keep_features && (rc = ensure_learn_buffers(c))) return fail(rc);
    if (c->opts.warm_start == SWC_WARM_EXTRAPOLATE && (rc = ensure_extrap_buffers(c))) return fail(rc);
    c->B.nseg = (long long) L.ny * L.nz * L.bnx;
    if ((rc = dalloc(c, &c->B.flag, L.nbricks)) || (rc = dalloc(c, &c->B.flag_prev, L.nbricks)) ||
        (rc = dalloc(c, &c->B.list, L.nbricks)) || (rc = dalloc(c, &c->B.count, 1)) ||
        (rc = dalloc(c, &c->B.seg, c->B.nseg)) || (rc = dalloc(c, &c->B.seg_off, c->B.nseg + 1)) ||
        (rc = dalloc(c, &c->pflag, L.nbricks)) || (rc = dalloc(c, &c->plist, L.nbricks)) ||
        (rc = dalloc(c, &c->pcount, 1)) || (rc = dalloc(c, &c->bnear, L.nbricks)))
        return fail(rc);
    if ((rc = dalloc(c, &c->pcomp, size_t(L.ncells))) || (rc = dalloc(c, &c->nv_prev, 1)) ||
        (rc = dalloc(c, &c->scan_tiles, scan_tile_count(std::max<long long>(c->B.nseg, L.ncells) + 1) + 2)) ||
        (rc = dalloc(c, &c->cg, 1)) || (rc = dalloc(c, &c->partials, npart)) || (rc = dalloc(c, &c->queues, 4)) ||
        (rc = dalloc(c, &c->diag_bits, 1)) || (rc = dalloc(c, &c->max_bits, 1)) || (rc = dalloc(c, &c->res2, 2)) ||
        (rc = dalloc(c, &c->cellStart, L.ncells + 1)) || (rc = dalloc(c, &c->bcellStart, L.ncells + 1)) ||
        (rc = dalloc(c, &c->bcell, L.ncells)) || (rc = dalloc(c, &c->bcell_tmp, L.ncells)))
        return fail(rc);
    if (cudaMallocHost(reinterpret_cast<void **>(&c->hcg), sizeof(HostCg)) != cudaSuccess) return fail(SWC_OUT_OF_MEMORY);
    cudaMemsetAsync(c->cg, 0, sizeof(CgState), c->stream);
    cudaMemsetAsync(c->partials, 0, sizeof(double) * npart, c->stream);
    cudaMemsetAsync(c->queues, 0, sizeof(int) * 4, c->stream);
    cudaMemsetAsync(c->B.flag, 0, L.nbricks, c->stream);
    cudaMemsetAsync(c->B.flag_prev, 0, L.nbricks, c->stream);
    cudaMemsetAsync(c->N.flag, 0, slots, c->stream);
    cudaMemsetAsync(c->N.x, 0, slots * sizeof(float), c->stream);
    cudaMemsetAsync(c->nv_prev, 0, sizeof(int), c->stream);
    cudaMemsetAsync(c->bcellStart, 0, sizeof(int) * (L.ncells + 1), c->stream);
    cudaMemsetAsync(c->bnear, 0, L.nbricks, c->stream);
    cudaMemsetAsync(c->bcell, 0, L.ncells, c->stream);
    for (auto & e : c->ev) cudaEventCreate(&e);
    cudaEventCreate(&c->evA);
    cudaEventCreate(&c->evB);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(SWC_CUDA_ERROR);
    *out = c;
    return SWC_OK;
}

void swc_destroy(swc_ctx * c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->g1) cudaGraphExecDestroy(c->g1);
    if (c->g8) cudaGraphExecDestroy(c->g8);
    dfree(c->pos);
    dfree(c->vel);
    dfree(c->vel2);
    dfree(c->id);
    dfree(c->rho);
    dfree(c->vol_by_id);
    dfree(c->pleft);
    dfree(c->stage);
    dfree(c->cellStart);
    free_sort(c->sortR);
    dfree(c->bpos);
    dfree(c->bvel);
    dfree(c->bnrm);
    dfree(c->bid);
    dfree(c->brho);
    dfree(c->bcellStart);
    dfree(c->bstage);
    free_sort(c->sortB);
    dfree(c->N.flag);
    dfree(c->N.flag_prev);
    dfree(c->N.flag_m2);
    dfree(c->N.flag_m3);
    dfree(c->N.xm1);
    dfree(c->N.xm2);
    dfree(c->N.d2p);
    dfree(c->B.flag_m2);
    dfree(c->B.flag_m3);
    dfree(c->N.V);
    dfree(c->N.D);
    dfree(c->N.rho);
    dfree(c->N.ahat);
    dfree(c->N.x);
    dfree(c->N.r);
    dfree(c->N.q);
    dfree(c->N.d);
    dfree(c->N.u);
    dfree(c->N.vbar);
    dfree(c->N.nreal);
    dfree(c->mlp_params);
    dfree(c->mlp_norm);
    dfree(c->mlp_err);
    dfree(c->slot_of);
    dfree(c->xprev);
    dfree(c->feat_buf);
    dfree(c->tgt_buf);
    dfree(c->B.flag);
    dfree(c->B.flag_prev);
    dfree(c->B.list);
    dfree(c->B.count);
    dfree(c->B.seg);
    dfree(c->B.seg_off);
    dfree(c->pflag);
    dfree(c->plist);
    dfree(c->pcount);
    dfree(c->bnear);
    dfree(c->bcell);
    dfree(c->bcell_tmp);
    dfree(c->pcomp);
    dfree(c->nv_prev);
    dfree(c->scan_tiles);
    dfree(c->cg);
    dfree(c->partials);
    dfree(c->queues);
    dfree(c->diag_bits);
    dfree(c->vmax_bits);
    dfree(c->max_bits);
    dfree(c->res2);
    if (c->hcg) cudaFreeHost(c->hcg);
    for (auto & e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->evA) cudaEventDestroy(c->evA);
    if (c->evB) cudaEventDestroy(c->evB);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int swc_set_stream(swc_ctx * c, void * stream) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    CK(cudaStreamSynchronize(c->stream));
    if (c->g1) cudaGraphExecDestroy(c->g1);
    if (c->g8) cudaGraphExecDestroy(c->g8);
    c->g1 = c->g8 = nullptr;
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (stream) {
        c->stream     = static_cast<cudaStream_t>(stream);
        c->own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    return SWC_OK;
}

int swc_set_solver_opts(swc_ctx * c, const swc_solver_opts * o) {
    if (!valid_ctx(c) || !o || o->warm_start < SWC_WARM_PREFIX || o->warm_start > SWC_WARM_EXTRAPOLATE)
        return SWC_BAD_ARG;
    if (o->warm_start == SWC_WARM_PREFIX && c->pcomp_stale) {
        // the last solution (still in the lattice slots) as the next prefix start
        const int rc0 = c->dim == 2 ? export_prefix<2>(c) : export_prefix<3>(c);
        if (rc0) return rc0;
    }
    const bool need_vbar = o->keep_virtual_velocity && !c->N.vbar;
    const bool need_feat = o->keep_features && !c->N.nreal;
    c->opts         = *o;
    c->gate_rejects = c->gate_skip = c->gate_windows = 0;
    const size_t slots = size_t(c->L.nbricks) * (c->dim == 3 ? 512 : 256);
    int rc;
    if (need_vbar || need_feat) {
        CK(cudaStreamSynchronize(c->stream));
        if (c->g1) cudaGraphExecDestroy(c->g1);
        if (c->g8) cudaGraphExecDestroy(c->g8);
        c->g1 = c->g8 = nullptr;
    }
    if (need_vbar && (rc = dalloc(c, &c->N.vbar, slots))) return rc;
    if (need_feat && (rc = ensure_learn_buffers(c))) return rc;
    if (o->warm_start == SWC_WARM_EXTRAPOLATE && !c->N.xm1) {
        CK(cudaStreamSynchronize(c->stream));
        if ((rc = ensure_extrap_buffers(c))) return rc;
    }
    return SWC_OK;
}

int swc_set_particles(swc_ctx * c, const double * x, const double * v, int64_t n) {
    if (!valid_ctx(c) || n < 0 || (n > 0 && !x)) return SWC_BAD_ARG;
    if (n > (1LL << 30)) return SWC_BAD_ARG;
    int rc;
    if (n != c->n || !c->pos) {
        if (c->initialized && n != c->n) {
            c->err = "particle count changed after initialize";
            return SWC_BAD_ARG;
        }
        CK(cudaStreamSynchronize(c->stream));
        if ((rc = dalloc(c, &c->pos, n)) || (rc = dalloc(c, &c->vel, n)) || (rc = dalloc(c, &c->vel2, n)) ||
            (rc = dalloc(c, &c->id, n)) || (rc = dalloc(c, &c->rho, n)) || (rc = dalloc(c, &c->vol_by_id, n)) ||
            (rc = dalloc(c, &c->stage, size_t(2) * std::max<int64_t>(n, 1) * c->dim)) ||
            (rc = dalloc(c, &c->pleft, size_t(n) / 2 + 3)) || (rc = alloc_sort(c, c->sortR, n, false))) {
            c->n           = 0;
            c->initialized = false;
            return rc;
        }
        CK(cudaMemsetAsync(c->pleft, 0, sizeof(int) * 2, c->stream));
        c->n = n;
    }
    const size_t bytes = sizeof(double) * size_t(n) * c->dim;
    CK(cudaMemcpyAsync(c->stage, x, bytes, cudaMemcpyHostToDevice, c->stream));
    if (v) CK(cudaMemcpyAsync(c->stage + size_t(n) * c->dim, v, bytes, cudaMemcpyHostToDevice, c->stream));
    launch_import(c->stage, v ? c->stage + size_t(n) * c->dim : nullptr, c->dim, n, c->pos, c->vel, c->id, c->stream);
    if (c->initialized) launch_fill_w_by_id(c->pos, c->vol_by_id, nullptr, n, c->stream);  // ids are 0..n-1 here
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_get_particles(swc_ctx * c, double * x, double * v, int64_t n) {
    if (!valid_ctx(c) || n != c->n) return SWC_BAD_ARG;
    double * sx = c->stage;
    double * sv = c->stage + size_t(n) * c->dim;
    launch_export(c->pos, c->vel, c->id, c->dim, n, x ? sx : nullptr, v ? sv : nullptr, c->stream);
    const size_t bytes = sizeof(double) * size_t(n) * c->dim;
    if (x) CK(cudaMemcpyAsync(x, sx, bytes, cudaMemcpyDeviceToHost, c->stream));
    if (v) CK(cudaMemcpyAsync(v, sv, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SWC_OK;
}

int swc_set_boundary(swc_ctx * c, const double * x, const double * nrm, const double * v, int64_t nb) {
    if (!valid_ctx(c) || nb < 0 || (nb > 0 && (!x || !nrm))) return SWC_BAD_ARG;
    int rc;
    CK(cudaStreamSynchronize(c->stream));
    // a failed allocation leaves no boundary and an uninitialized context, so a later
    // advance returns SWC_NOT_INITIALIZED instead of reaching freed buffers
    if ((rc = dalloc(c, &c->bpos, nb)) || (rc = dalloc(c, &c->bvel, nb)) || (rc = dalloc(c, &c->bnrm, nb)) ||
        (rc = dalloc(c, &c->bid, nb)) || (rc = dalloc(c, &c->brho, nb)) ||
        (rc = dalloc(c, &c->bstage, size_t(3) * std::max<int64_t>(nb, 1) * c->dim)) ||
        (rc = alloc_sort(c, c->sortB, nb, true))) {
        c->nb          = 0;
        c->initialized = false;
        return rc;
    }
    c->nb = nb;
    const size_t bytes = sizeof(double) * size_t(nb) * c->dim;
    double * sx = c->bstage;
    double * sn = c->bstage + size_t(nb) * c->dim;
    double * sv = c->bstage + 2 * size_t(nb) * c->dim;
    if (nb > 0) {
        CK(cudaMemcpyAsync(sx, x, bytes, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(sn, nrm, bytes, cudaMemcpyHostToDevice, c->stream));
        if (v) CK(cudaMemcpyAsync(sv, v, bytes, cudaMemcpyHostToDevice, c->stream));
    }
    launch_import(sx, v ? sv : nullptr, c->dim, nb, c->bpos, c->bvel, c->bid, c->stream);
    launch_import(sn, nullptr, c->dim, nb, c->bnrm, c->sortB.vel2, nullptr, c->stream);
    if (c->dim == 2) run_bin_boundary<2>(c);
    else run_bin_boundary<3>(c);
    c->has_motion = false;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_set_boundary_motion(swc_ctx * c, const uint8_t * moving, const double center[3], double omega) {
    if (!valid_ctx(c) || !moving || !center || c->nb <= 0) return SWC_BAD_ARG;
    unsigned char * d = nullptr;
    CK(cudaMalloc(&d, c->nb));
    CK(cudaMemcpy(d, moving, c->nb, cudaMemcpyHostToDevice));
    launch_set_moving(c->bnrm, d, c->bid, c->nb, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(d);
    c->has_motion   = true;
    c->motion_omega = omega;
    for (int a = 0; a < 3; a++) c->motion_c[a] = center[a];
    return SWC_OK;
}

int swc_initialize(swc_ctx * c) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    int rc = c->dim == 2 ? do_initialize<2>(c) : do_initialize<3>(c);
    return rc;
}

int swc_advance(swc_ctx * c, double dt, swc_stats * st) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    if (!c->initialized) return SWC_NOT_INITIALIZED;
    if (!(dt >= 0) || !std::isfinite(dt)) return SWC_BAD_ARG;
    if (st) std::memset(st, 0, sizeof(*st));
    return c->dim == 2 ? do_advance<2>(c, dt, st, true) : do_advance<3>(c, dt, st, true);
}

int swc_project(swc_ctx * c, swc_stats * st) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    if (!c->initialized) return SWC_NOT_INITIALIZED;
    if (st) std::memset(st, 0, sizeof(*st));
    return c->dim == 2 ? do_advance<2>(c, 0.0, st, false) : do_advance<3>(c, 0.0, st, false);
}

int swc_get_time_step(swc_ctx * c, double step_rate, double * dt) {
    if (!valid_ctx(c) || !dt) return SWC_BAD_ARG;
    unsigned long long bits = 0;
    if (c->n > 0) {
        int rc;
        if (!c->vmax_bits && (rc = dalloc(c, &c->vmax_bits, 1))) return rc;
        CK(cudaMemsetAsync(c->vmax_bits, 0, sizeof(unsigned long long), c->stream));
        launch_max_speed2(c->vel, c->n, c->dim, c->vmax_bits, c->stream);
        CK(cudaMemcpyAsync(&bits, c->vmax_bits, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    double m2;
    std::memcpy(&m2, &bits, sizeof(m2));
    // at rest max |v| = 0 and the step is unbounded (+inf), as in the reference
    *dt = step_rate * c->scene.particle_radius * 2 / std::sqrt(m2);
    return SWC_OK;
}

int swc_get_boundary(swc_ctx * c, double * pos, double * normals, double * vel, int64_t nb) {
    if (!valid_ctx(c) || nb != c->nb) return SWC_BAD_ARG;
    if (nb == 0) return SWC_OK;
    double * sx = c->bstage;
    double * sn = c->bstage + size_t(nb) * c->dim;
    double * sv = c->bstage + 2 * size_t(nb) * c->dim;
    launch_export(c->bpos, c->bvel, c->bid, c->dim, nb, pos ? sx : nullptr, vel ? sv : nullptr, c->stream);
    if (normals) launch_export(c->bnrm, nullptr, c->bid, c->dim, nb, sn, nullptr, c->stream);
    const size_t bytes = sizeof(double) * size_t(nb) * c->dim;
    if (pos) CK(cudaMemcpyAsync(pos, sx, bytes, cudaMemcpyDeviceToHost, c->stream));
    if (normals) CK(cudaMemcpyAsync(normals, sn, bytes, cudaMemcpyDeviceToHost, c->stream));
    if (vel) CK(cudaMemcpyAsync(vel, sv, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SWC_OK;
}

int swc_get_real_info(swc_ctx * c, double * rho, double * vol, int64_t n) {
    if (!valid_ctx(c) || n != c->n) return SWC_BAD_ARG;
    double * s0 = c->stage;
    double * s1 = c->stage + size_t(n) * c->dim;
    if (rho) launch_export_scalar(c->rho, 1, 0, c->id, n, s0, c->stream);
    if (vol) launch_export_scalar(reinterpret_cast<const float *>(c->pos), 4, 3, c->id, n, s1, c->stream);
    if (rho) CK(cudaMemcpyAsync(rho, s0, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (vol) CK(cudaMemcpyAsync(vol, s1, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SWC_OK;
}

int swc_set_volumes(swc_ctx * c, const double * vol, int64_t n) {
    if (!valid_ctx(c) || n != c->n || !vol) return SWC_BAD_ARG;
    std::vector<float> vf(vol, vol + n);
    CK(cudaMemcpy(c->vol_by_id, vf.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    launch_fill_w_by_id(c->pos, c->vol_by_id, c->id, n, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    return SWC_OK;
}

int swc_get_boundary_info(swc_ctx * c, double * rho, double * vol, int64_t nb) {
    if (!valid_ctx(c) || nb != c->nb) return SWC_BAD_ARG;
    if (nb == 0) return SWC_OK;
    double * s0 = c->bstage;
    double * s1 = c->bstage + size_t(nb) * c->dim;
    // rho_b = m_b / (m_b / rho_b): bvel.w travels through the boundary re-sorts of
    // moving solids, a separate per-slot rho array would not
    if (rho)
        launch_export_ratio(reinterpret_cast<const float *>(c->bvel), 4, 3, c->P.bmass, c->bid, nb, s0, c->stream);
    if (vol) launch_export_scalar(reinterpret_cast<const float *>(c->bpos), 4, 3, c->bid, nb, s1, c->stream);
    if (rho) CK(cudaMemcpyAsync(rho, s0, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
    if (vol) CK(cudaMemcpyAsync(vol, s1, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SWC_OK;
}

int swc_set_boundary_info(swc_ctx * c, const double * rho, const double * vol, int64_t nb) {
    if (!valid_ctx(c) || nb != c->nb || !rho || !vol) return SWC_BAD_ARG;
    if (nb == 0) return SWC_OK;
    std::vector<float> r(rho, rho + nb), v(vol, vol + nb);
    float * tmp = nullptr;
    CK(cudaMalloc(&tmp, sizeof(float) * 2 * nb));
    cudaMemcpy(tmp, r.data(), sizeof(float) * nb, cudaMemcpyHostToDevice);
    cudaMemcpy(tmp + nb, v.data(), sizeof(float) * nb, cudaMemcpyHostToDevice);
    launch_set_boundary_info(c->bpos, c->bvel, c->brho, tmp, tmp + nb, c->bid, nb, float(c->scene.boundary_mass),
                             c->stream);
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_get_scalars(swc_ctx * c, double * rho0, double * alpha0, double * kappa) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    if (rho0) *rho0 = c->rho0;
    if (alpha0) *alpha0 = c->alpha0;
    if (kappa) *kappa = c->kappa;
    return SWC_OK;
}

int swc_set_scalars(swc_ctx * c, double rho0, double alpha0, double kappa) {
    if (!valid_ctx(c) || !(rho0 > 0)) return SWC_BAD_ARG;
    c->rho0   = rho0;
    c->alpha0 = alpha0;
    c->kappa  = kappa;
    setup_phys(c);
    return SWC_OK;
}

int64_t swc_num_virtual(swc_ctx * c) {
    if (!valid_ctx(c)) return -1;
    int nv = 0;
    if (cudaMemcpy(&nv, c->B.seg_off + c->B.nseg, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return nv;
}

int swc_get_virtual(swc_ctx * c, int64_t * node_id, double * rho, double * vol, double * vbar, double * div,
                    double * ahat, double * p, int64_t capacity) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    const int64_t nv = swc_num_virtual(c);
    if (nv < 0) return SWC_CUDA_ERROR;
    if (capacity < nv) return SWC_BAD_ARG;
    if (vbar && !c->N.vbar) {
        c->err = "vbar not kept (keep_virtual_velocity = 0)";
        return SWC_BAD_ARG;
    }
    const size_t n1 = std::max<int64_t>(nv, 1);
    long long * d_id = nullptr;
    double * d_buf   = nullptr;
    CK(cudaMalloc(&d_id, sizeof(long long) * n1));
    CK(cudaMalloc(&d_buf, sizeof(double) * n1 * (5 + c->dim)));
    double *dr = d_buf, *dv = d_buf + n1, *dd = d_buf + 2 * n1, *da = d_buf + 3 * n1, *dp = d_buf + 4 * n1,
           *dvb = d_buf + 5 * n1;
    if (c->dim == 2)
        launch_compact_export<2>(c->L, c->B, c->N, nullptr, d_id, dr, dv, vbar ? dvb : nullptr, dd, da, dp, nullptr,
                                 c->grid, c->stream);
    else
        launch_compact_export<3>(c->L, c->B, c->N, nullptr, d_id, dr, dv, vbar ? dvb : nullptr, dd, da, dp, nullptr,
                                 c->grid, c->stream);
    cudaStreamSynchronize(c->stream);
    if (nv > 0) {
        if (node_id) cudaMemcpy(node_id, d_id, sizeof(long long) * nv, cudaMemcpyDeviceToHost);
        if (rho) cudaMemcpy(rho, dr, sizeof(double) * nv, cudaMemcpyDeviceToHost);
        if (vol) cudaMemcpy(vol, dv, sizeof(double) * nv, cudaMemcpyDeviceToHost);
        if (div) cudaMemcpy(div, dd, sizeof(double) * nv, cudaMemcpyDeviceToHost);
        if (ahat) cudaMemcpy(ahat, da, sizeof(double) * nv, cudaMemcpyDeviceToHost);
        if (p) cudaMemcpy(p, dp, sizeof(double) * nv, cudaMemcpyDeviceToHost);
        if (vbar) cudaMemcpy(vbar, dvb, sizeof(double) * nv * c->dim, cudaMemcpyDeviceToHost);
    }
    cudaFree(d_id);
    cudaFree(d_buf);
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_set_pressure(swc_ctx * c, const double * p, int64_t n) {
    if (!valid_ctx(c) || n < 0 || (n > 0 && !p) || n > c->L.ncells) return SWC_BAD_ARG;
    std::vector<float> f(p, p + n);
    if (n > 0) CK(cudaMemcpy(c->pcomp, f.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    int ni = int(n);
    CK(cudaMemcpy(c->nv_prev, &ni, sizeof(int), cudaMemcpyHostToDevice));
    c->pcomp_stale = false;
    return SWC_OK;
}

int swc_set_mlp(swc_ctx * c, const float * params, const float * norm) {
    if (!valid_ctx(c) || !params || !norm) return SWC_BAD_ARG;
    for (int k = SWC_MLP_IN; k < 2 * SWC_MLP_IN; k++)
        if (!(norm[k] > 0)) return SWC_BAD_ARG;
    if (!(norm[2 * SWC_MLP_IN + 1] > 0)) return SWC_BAD_ARG;
    int rc;
    CK(cudaStreamSynchronize(c->stream));
    if ((rc = ensure_learn_buffers(c))) return rc;
    if (!c->mlp_params && ((rc = dalloc(c, &c->mlp_params, SWC_MLP_PARAMS)) || (rc = dalloc(c, &c->mlp_norm, SWC_MLP_NORM))))
        return rc;
    CK(cudaMemcpy(c->mlp_params, params, sizeof(float) * SWC_MLP_PARAMS, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->mlp_norm, norm, sizeof(float) * SWC_MLP_NORM, cudaMemcpyHostToDevice));
    c->mlp_ready = true;
    return SWC_OK;
}

int swc_get_features(swc_ctx * c, float * features, float * targets, int64_t capacity, int64_t * n) {
    if (!valid_ctx(c) || !n) return SWC_BAD_ARG;
    if (!c->features_valid) {
        c->err = "no features logged (keep_features off or no projection yet)";
        return SWC_BAD_ARG;
    }
    const int64_t nv = swc_num_virtual(c);
    if (nv < 0) return SWC_CUDA_ERROR;
    *n = nv;
    if (capacity < nv) return SWC_BAD_ARG;
    if (nv > 0 && features) CK(cudaMemcpy(features, c->feat_buf, sizeof(float) * SWC_MLP_IN * nv, cudaMemcpyDeviceToHost));
    if (nv > 0 && targets) CK(cudaMemcpy(targets, c->tgt_buf, sizeof(float) * nv, cudaMemcpyDeviceToHost));
    return SWC_OK;
}

int swc_apply_operator(swc_ctx * c, const double * x, double * y, int64_t n) {
    if (!valid_ctx(c) || !x || !y) return SWC_BAD_ARG;
    const int64_t nv = swc_num_virtual(c);
    if (n != nv) return SWC_BAD_ARG;
    const size_t slots = size_t(c->L.nbricks) * (c->dim == 3 ? 512 : 256);
    double * d_in = nullptr;
    double * d_out = nullptr;
    float * t_in = nullptr;
    float * t_out = nullptr;
    CK(cudaMalloc(&d_in, sizeof(double) * std::max<int64_t>(n, 1)));
    CK(cudaMalloc(&d_out, sizeof(double) * std::max<int64_t>(n, 1)));
    CK(cudaMalloc(&t_in, sizeof(float) * slots));
    CK(cudaMalloc(&t_out, sizeof(float) * slots));
    cudaMemcpy(d_in, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    // brick-layout vector: reuse compact export machinery through a temporary NodeArrays view
    if (c->dim == 2) {
        launch_compact_import<2>(c->L, c->B, c->N, d_in, t_in, c->grid, c->stream);
        launch_apply_operator<2>(c->L, c->B, c->N, c->S, t_in, t_out, c->rgrid, c->stream);
        NodeArrays T = c->N;
        T.x          = t_out;
        launch_compact_export<2>(c->L, c->B, T, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, d_out,
                                 nullptr, c->grid, c->stream);
    } else {
        launch_compact_import<3>(c->L, c->B, c->N, d_in, t_in, c->grid, c->stream);
        launch_apply_operator<3>(c->L, c->B, c->N, c->S, t_in, t_out, c->rgrid, c->stream);
        NodeArrays T = c->N;
        T.x          = t_out;
        launch_compact_export<3>(c->L, c->B, T, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, d_out,
                                 nullptr, c->grid, c->stream);
    }
    cudaStreamSynchronize(c->stream);
    cudaMemcpy(y, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    cudaFree(t_in);
    cudaFree(t_out);
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_debug_neighbors(swc_ctx * c, int which, int64_t nq, const double * q, int64_t * counts,
                        const int64_t * offsets, int64_t * ids) {
    if (!valid_ctx(c) || which < 0 || which > 2 || nq < 0 || (nq > 0 && (!q || !counts))) return SWC_BAD_ARG;
    if (ids && !offsets) return SWC_BAD_ARG;
    if (nq == 0) return SWC_OK;
    int64_t total = 0;
    if (ids) total = offsets[nq - 1] + counts[nq - 1];
    double * dq = nullptr;
    long long *dc = nullptr, *doff = nullptr, *dids = nullptr;
    CK(cudaMalloc(&dq, sizeof(double) * nq * c->dim));
    CK(cudaMalloc(&dc, sizeof(long long) * nq));
    if (ids) {
        CK(cudaMalloc(&doff, sizeof(long long) * nq));
        CK(cudaMalloc(&dids, sizeof(long long) * std::max<int64_t>(total, 1)));
        cudaMemcpy(doff, offsets, sizeof(long long) * nq, cudaMemcpyHostToDevice);
    }
    cudaMemcpy(dq, q, sizeof(double) * nq * c->dim, cudaMemcpyHostToDevice);
    const float4 * P  = which == 0 ? c->pos : c->bpos;
    const int * ID    = which == 0 ? c->id : c->bid;
    const int * CS    = which == 0 ? c->cellStart : c->bcellStart;
    if (c->dim == 2)
        launch_debug_neighbors<2>(which, nq, dq, c->L, c->P, P, ID, CS, c->B.flag, c->N.flag, dc, doff, dids, c->stream);
    else
        launch_debug_neighbors<3>(which, nq, dq, c->L, c->P, P, ID, CS, c->B.flag, c->N.flag, dc, doff, dids, c->stream);
    cudaStreamSynchronize(c->stream);
    cudaMemcpy(counts, dc, sizeof(long long) * nq, cudaMemcpyDeviceToHost);
    if (ids && total > 0) cudaMemcpy(ids, dids, sizeof(long long) * total, cudaMemcpyDeviceToHost);
    cudaFree(dq);
    cudaFree(dc);
    cudaFree(doff);
    cudaFree(dids);
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_set_profiling(swc_ctx * c, int on) {
    if (!valid_ctx(c)) return SWC_BAD_ARG;
    c->profiling = on != 0;
    return SWC_OK;
}

int swc_get_phase_times(swc_ctx * c, double * ms, int n) {
    if (!valid_ctx(c) || !ms) return SWC_BAD_ARG;
    for (int k = 0; k < n && k < kPhases; k++) ms[k] = c->phase_ms[k];
    return SWC_OK;
}

int swc_time_kernel(swc_ctx * c, int which, int reps, double * mean_ms) {
    if (!valid_ctx(c) || !mean_ms || reps <= 0 || !c->initialized || which < 0 || which > 7) return SWC_BAD_ARG;
    if (which == 7 && !c->mlp_ready) return SWC_BAD_ARG;  // needs a network (swc_set_mlp)
    CK(cudaStreamSynchronize(c->stream));
    // keep the solver state: run the CG kernels against a scratch copy of the scalars
    CgState saved{};
    CK(cudaMemcpy(&saved, c->cg, sizeof(CgState), cudaMemcpyDeviceToHost));
    CgState run = saved;
    run.done      = 0;
    run.iter      = 2;  // beta path of the SpMV
    run.threshold = 0;  // never converge while timing
    run.max_iter  = 0x7fffffff;
    if (!(run.rr_prev > 0)) run.rr_prev = 1, run.rr = 1;
    if (!(run.pq != 0)) run.pq = 1;
    CK(cudaMemcpy(c->cg, &run, sizeof(CgState), cudaMemcpyHostToDevice));
    float * x_save = nullptr;
    const size_t slots = size_t(c->L.nbricks) * (c->dim == 3 ? 512 : 256);
    if (which == 1 || which == 7) {
        CK(cudaMalloc(&x_save, sizeof(float) * slots * 2));
        cudaMemcpy(x_save, c->N.x, sizeof(float) * slots, cudaMemcpyDeviceToDevice);
        cudaMemcpy(x_save + slots, c->N.r, sizeof(float) * slots, cudaMemcpyDeviceToDevice);
    }
    float4 * vel_save = nullptr;
    if (which == 3) {
        CK(cudaMalloc(&vel_save, sizeof(float4) * std::max<long long>(c->n, 1)));
        cudaMemcpy(vel_save, c->vel, sizeof(float4) * c->n, cudaMemcpyDeviceToDevice);
    }
    auto launch = [&]() {
        if (which == 7) {
            launch_mlp_forward_nodes(c->mlp_params, c->mlp_norm, c->N, c->B, c->dim == 3 ? 9 : 8, (long long) slots,
                                     &c->cg->bb, float(1.0 / c->alpha0), float(1.0 / c->rho0), 1.f / 32.f, c->mlp_err,
                                     c->stream);
            return;
        }
        if (c->dim == 3) {
            switch (which) {
            case 0: launch_cg_spmv<3>(c->L, c->B, c->N, c->S, c->cg, c->partials, c->sgrid, c->stream); break;
            case 1: launch_cg_update<3>(c->B, c->N, c->cg, c->partials, c->grid, c->stream); break;
            case 6: launch_cg_direction<3>(c->B, c->N, c->cg, c->grid, c->stream); break;
            case 2:
                launch_node_gather<3>(c->L, c->P, c->B, c->N, c->pos, c->vel, c->cellStart, c->bpos, c->bvel,
                                      c->bcellStart, c->bnear, c->bcell, c->ggrid, c->queues, c->stream);
                break;
            case 3:
                launch_pressure_gradient<3>(c->L, c->P, c->B, c->N, c->plist, c->pcount, c->bnear, c->pos, c->vel,
                                            c->cellStart, c->bpos, c->bvel, c->bnrm, c->bcellStart, c->bcell, c->pgrid,
                                            c->queues + 2, c->stream);
                break;
            case 4: launch_density<3>(c->pos, c->vel, c->rho, c->n, c->L, c->P, c->cellStart, c->pleft, c->stream); break;
            case 5: launch_forces<3>(c->pos, c->vel, c->vel2, c->n, c->L, c->P, c->cellStart, 0.f, c->pleft, c->stream); break;
            }
        } else {
            switch (which) {
            case 2:
                launch_node_gather<2>(c->L, c->P, c->B, c->N, c->pos, c->vel, c->cellStart, c->bpos, c->bvel,
                                      c->bcellStart, c->bnear, c->bcell, c->ggrid, c->queues, c->stream);
                break;
            case 4: launch_density<2>(c->pos, c->vel, c->rho, c->n, c->L, c->P, c->cellStart, c->pleft, c->stream); break;
            default: break;
            }
        }
    };
    launch();  // warm
    CK(cudaEventRecord(c->evA, c->stream));
    for (int k = 0; k < reps; k++) launch();
    CK(cudaEventRecord(c->evB, c->stream));
    CK(cudaEventSynchronize(c->evB));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->evA, c->evB);
    *mean_ms = ms / reps;
    CK(cudaMemcpy(c->cg, &saved, sizeof(CgState), cudaMemcpyHostToDevice));
    if (x_save) {
        cudaMemcpy(c->N.x, x_save, sizeof(float) * slots, cudaMemcpyDeviceToDevice);
        cudaMemcpy(c->N.r, x_save + slots, sizeof(float) * slots, cudaMemcpyDeviceToDevice);
        cudaFree(x_save);
    }
    if (vel_save) {
        cudaMemcpy(c->vel, vel_save, sizeof(float4) * c->n, cudaMemcpyDeviceToDevice);
        cudaFree(vel_save);
    }
    CK(cudaGetLastError());
    return SWC_OK;
}

int swc_debug_fail_alloc(int64_t after) {
    swc::g_fail_alloc_after.store(after < 0 ? -1 : after);
    return SWC_OK;
}

void * swc_host_alloc(size_t bytes) {
    void * p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}
void swc_host_free(void * p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
