// swc_kernels.h -- launcher declarations shared by the translation units of
// the GB300 dual-particle SPH projection (internal; not part of the C ABI).
#pragma once

#include "swc_common.cuh"

namespace swc {

// Scratch for the counting sort of one particle set.
struct SortScratch {
    int *    key = nullptr, *rank = nullptr, *perm = nullptr, *count = nullptr, *tiles = nullptr;
    float4 * pos2 = nullptr, *vel2 = nullptr, *aux2 = nullptr;
    int *    id2 = nullptr;
};

// Radial stencil coefficients of the virtual Laplacian, indexed by |offset|^2
// (0..15): c = 2 W'_H(r) / (r + 1e-6) with r = |offset| * grid spacing.
struct Stencil {
    float c[16];
};
struct StencilD {
    double c[16];
};

// Node-lattice arrays (brick layout, indexed by brick * BN + local).
struct NodeArrays {
    unsigned char * flag      = nullptr;  // active this step
    unsigned char * flag_prev = nullptr;  // active in the previous step
    float *         V         = nullptr;  // virtual volume V_I (0 when inactive)
    float *         D         = nullptr;  // divergence D_I (CG right-hand side)
    float *         rho       = nullptr;  // virtual density rho_I
    float *         ahat      = nullptr;  // clamped diagonal alpha_hat_I (1 when inactive)
    float *         x         = nullptr;  // pressure (CG solution), kept across steps
    float *         r         = nullptr;
    float *         q         = nullptr;
    float *         d         = nullptr;  // CG search direction
    float *         u         = nullptr;  // V * d, the halo source of the SpMV
    float4 *        vbar      = nullptr;  // optional: virtual velocity (debug / export)
    unsigned short * nreal    = nullptr;  // optional: real neighbours within h
    // pressure history of the extrapolated / learned warm starts (see k_warm_start)
    float *         xm1       = nullptr;  // p one step back (0 where inactive then)
    float *         xm2       = nullptr;  // p two steps back
    float *         d2p       = nullptr;  // optional: second difference p1 - 2 p2 + p3 (learned features)
    unsigned char * flag_m2   = nullptr;  // active two steps back
    unsigned char * flag_m3   = nullptr;  // active three steps back
};

struct BrickArrays {
    unsigned char * flag      = nullptr;  // active this step
    unsigned char * flag_prev = nullptr;
    unsigned char * flag_m2   = nullptr;  // active two / three steps back (pressure history)
    unsigned char * flag_m3   = nullptr;
    int *           list      = nullptr;  // active brick ids, ascending
    int *           count     = nullptr;  // device: number of active bricks
    int *           seg       = nullptr;  // per (row, brick column) active-node counts
    int *           seg_off   = nullptr;  // exclusive scan of seg (+ total at the end)
    long long       nseg      = 0;
};

// ---- k_particles.cu ----
void launch_import(const double * x, const double * v, int dim, long long n, float4 * pos, float4 * vel, int * id,
                   cudaStream_t st);
void launch_export(const float4 * pos, const float4 * vel, const int * id, int dim, long long n, double * x,
                   double * v, cudaStream_t st);
void launch_export_scalar(const float * a, int stride, int comp, const int * id, long long n, double * out,
                          cudaStream_t st);
void launch_max_speed2(const float4 * vel, long long n, int dim, unsigned long long * out, cudaStream_t st);
void launch_export_ratio(const float * a, int stride, int comp, float num, const int * id, long long n, double * out,
                         cudaStream_t st);
void launch_scan(const int * in, long long n, int * out, int * tile_buf, cudaStream_t st,
                 const Lattice * Ld = nullptr);
long long scan_tile_count(long long n);
void launch_set_volume(float4 * pos, const float * rho, long long n, float mass, cudaStream_t st);
void launch_rotate_boundary(float4 * bpos, float4 * bvel, float4 * bnrm, long long nb, float cx, float cz,
                            float omega, float dt, cudaStream_t st);
void launch_fill_w_by_id(float4 * pos, const float * vol, const int * id, long long n, cudaStream_t st);
void launch_scatter_w_to_id(const float4 * pos, const int * id, long long n, float * vol, cudaStream_t st);
void launch_set_boundary_info(float4 * bpos, float4 * bvel, float * brho, const float * rho, const float * vol,
                              const int * bid, long long nb, float bmass, cudaStream_t st);
void launch_set_moving(float4 * bnrm, const unsigned char * moving, const int * bid, long long nb, cudaStream_t st);
void launch_max_positive(const float * a, long long n, int * out_bits, cudaStream_t st);
// counting sort into cells; the sorted arrays are swapped in (pos, vel, aux, id
// then point at what were the scratch targets); advect_dt != 0 first moves the
// particles by vel * advect_dt; with aux_lo, aux holds the low parts of
// float-float positions (pos + aux) and the move uses dt = advect_dt + advect_dt_lo;
// with Ld (device memory) the cell keys come from that lattice and L.ncells only
// gives the length of the cell arrays (at least Ld->ncells)
template<int DIM>
void launch_bin(const Lattice & L, long long n, float4 *& pos, float4 *& vel, float4 *& aux, int *& id, SortScratch & S,
                int * cellStart, float advect_dt, cudaStream_t st, float advect_dt_lo = 0.f, bool aux_lo = false,
                const Lattice * Ld = nullptr);
// Density and forces run one thread per pair of consecutive sorted particles;
// `left` (n/2 + 3 ints, zeroed once at allocation) collects the pairs that are
// not in one cell row for a second, single-particle pass.
template<int DIM>
void launch_density(const float4 * pos, float4 * vel, float * rho, long long n, const Lattice & L, const Phys & P,
                    const int * cellStart, int * left, cudaStream_t st);
template<int DIM>
void launch_forces(const float4 * pos, const float4 * vel, float4 * vel_out, long long n, const Lattice & L,
                   const Phys & P, const int * cellStart, float dt, int * left, cudaStream_t st);
template<int DIM>
void launch_boundary_density(float4 * bpos, float4 * bvel, float * rho, long long nb, const Lattice & L,
                             const Phys & P, const int * bcellStart, cudaStream_t st);
template<int DIM>
// bricks within reach of the particles binned in cellStart (and, with pflag, the
// bricks holding their cells); n = 0 clears the flags
void launch_mark_bricks(const int * cellStart, long long n, const Lattice & L, const Phys & P, unsigned char * bflag,
                        unsigned char * pflag, cudaStream_t st);
// cells within reach (h) of the particles binned in cellStart, one byte per node
// cell (a box dilation by ceil(h / dx) + 1 cells; tmp: scratch of the same size)
template<int DIM>
void launch_near_cells(const int * cellStart, long long n, const Lattice & L, const Phys & P, unsigned char * near,
                       unsigned char * tmp, cudaStream_t st);
template<int DIM>
void launch_debug_neighbors(int which, long long nq, const double * q, const Lattice & L, const Phys & P,
                            const float4 * pos, const int * id, const int * cellStart, const unsigned char * bflag,
                            const unsigned char * nflag, long long * counts, const long long * offsets, long long * ids,
                            cudaStream_t st);

// ---- k_nodes.cu ----
void launch_brick_list(const unsigned char * bflag, int nbricks, int * list, int * count, cudaStream_t st);
template<int DIM>
void launch_node_gather(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                        const float4 * pos, const float4 * vel, const int * cellStart, const float4 * bpos,
                        const float4 * bvel, const int * bcellStart, const unsigned char * bnear,
                        const unsigned char * bcell, int grid, int * queue, cudaStream_t st);
// Pressure-gradient update over the bricks that hold particles (plist / pcount),
// node field staged per brick in shared memory; bnear flags bricks near walls.
template<int DIM>
void launch_pressure_gradient(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N,
                              const int * plist, const int * pcount, const unsigned char * bnear, const float4 * pos,
                              float4 * vel, const int * cellStart, const float4 * bpos, const float4 * bvel,
                              const float4 * bnrm, const int * bcellStart, const unsigned char * bcell, int grid,
                              int * queue, cudaStream_t st);
// Resident blocks per SM of the persistent brick kernels (their grids are
// SMs x this; gather and gradient take bricks from a zero-initialised queue of
// two ints).
template<int DIM> int node_gather_blocks_per_sm();
template<int DIM> int pressure_gradient_blocks_per_sm();
template<int DIM> int cg_spmv_blocks_per_sm();
template<int DIM>
void launch_segments(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int * tiles, int grid,
                     cudaStream_t st);
template<int DIM>
void launch_ahat(const Lattice & L, const Phys & P, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                 int sgrid, cudaStream_t st);
template<int DIM>
void launch_diag_max_f64(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const StencilD & S,
                         unsigned long long * out_bits, int grid, cudaStream_t st);
// warm-start modes
enum { kWarmPrefix = 0, kWarmNode = 1, kWarmZero = 2, kWarmGiven = 3, kWarmExtrap = 4 };
// history (kWarmExtrap): steps of valid pressure history before this one (0, 1 or 2)
template<int DIM>
void launch_warm_start(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int mode, const float * pcomp,
                       const int * nv_prev, const float * given, int grid, cudaStream_t st, int history = 0);
template<int DIM>
void launch_compact_export(const Lattice & L, const BrickArrays & B, const NodeArrays & N, float * pcomp,
                           long long * node_id, double * rho, double * vol, double * vbar, double * div,
                           double * ahat, double * p, unsigned short * nreal_out, int grid, cudaStream_t st);
// CG
template<int DIM>
void launch_cg_init(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S, CgState * cg,
                    double * partials, double tol, int max_iterations, const int * nv, int sgrid, int ugrid,
                    cudaStream_t st);
// Residual r = b - A x of one candidate CG start (r, and d when non-null;
// |r|^2, |b|^2 into sums[0..1]).
template<int DIM>
void launch_cg_residual(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                        const float * x, float * r, float * d, double * sums, CgState * cg, double * partials,
                        int sgrid, int ugrid, cudaStream_t st);
// CG start from the better of the prediction (N.x, residual sums in cg->sums[0..1])
// and the base start xb (cg->sums[2..3], residual rb), decided on the device
// (cg->start: 0 prediction, 1 base); keep_prediction skips the comparison.
template<int DIM>
void launch_cg_pick(const BrickArrays & B, const NodeArrays & N, const float * xb, const float * rb,
                    const int * mlp_err, bool keep_prediction, CgState * cg, double tol, int max_iterations,
                    const int * nv, int ugrid, cudaStream_t st);
template<int DIM>
void launch_cg_iteration(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                         CgState * cg, double * partials, int sgrid, int ugrid, cudaStream_t st);
template<int DIM>
void launch_cg_direction(const BrickArrays & B, const NodeArrays & N, const CgState * cg, int ugrid, cudaStream_t st);
template<int DIM>
void launch_cg_spmv(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S, CgState * cg,
                    double * partials, int sgrid, cudaStream_t st);
template<int DIM>
void launch_cg_update(const BrickArrays & B, const NodeArrays & N, CgState * cg, double * partials, int ugrid,
                      cudaStream_t st);
template<int DIM>
void launch_apply_operator(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                           const float * in, float * out, int sgrid, cudaStream_t st);
template<int DIM>
void launch_zero_active(const Lattice & L, const BrickArrays & B, float * a, int grid, cudaStream_t st);
template<int DIM>
void launch_compact_import(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const double * in,
                           float * out, int grid, cudaStream_t st);
template<int DIM>
void launch_rhs_norm(const BrickArrays & B, const NodeArrays & N, CgState * cg, double * partials, int ugrid,
                     cudaStream_t st);
template<int DIM>
void launch_true_residual(const Lattice & L, const BrickArrays & B, const NodeArrays & N, const Stencil & S,
                          CgState * cg, double * partials, double * out2, int sgrid, cudaStream_t st);

// ---- k_mlp.cu (learned warm start) ----
void launch_mlp_forward_array(long long n, const float * params, const float * norm, const float * feat, float * out,
                              int * err, cudaStream_t st);
// node mode: every slot of the active bricks (inactive slots are skipped), the
// active-node count at B.seg_off[B.nseg]
void launch_mlp_forward_nodes(const float * params, const float * norm, const NodeArrays & N, const BrickArrays & B,
                              int bn_log2, long long slots_max, const double * bb, float inv_alpha0, float inv_rho0,
                              float inv_nreal, int * err, cudaStream_t st);
void launch_node_features(const NodeArrays & N, const int * slot_of, const int * nv, long long rows_max,
                          const CgState * cg, float inv_alpha0, float inv_rho0, float inv_nreal, float * feat_out,
                          cudaStream_t st);
// Loss gradient of one batch on the tensor cores (k_mlp_train.cu): `ctas` CTAs
// (mlp_train_ctas(n)) write their shares into share (mlp_train_share_floats(ctas)
// floats), a second kernel adds them in order into grad[SWC_MLP_PARAMS] and the
// mean squared error into *loss (NaN with *err set on a tensor-core timeout).
// Returns nonzero when a launch failed.
constexpr int kMlpTrainShare = 128 * 80 + 64 + 2;  // floats of one CTA's share (D, dw3, db3, loss)
int    mlp_train_ctas(long long n);
size_t mlp_train_share_floats(int ctas);
int    launch_mlp_train_grad(long long n, const float * params, const float * norm, const float * feat,
                             const float * target, float * share, int ctas, int * err, float * grad, float * loss,
                             cudaStream_t st);
void launch_adam(float * p, const float * g, float * m, float * v, int count, float lr, float b1, float b2, float eps,
                 float bc1, float bc2, cudaStream_t st);
template<int DIM>
void launch_slot_of(const Lattice & L, const BrickArrays & B, const NodeArrays & N, int * slot_of, int grid,
                    cudaStream_t st);
void launch_mlp_targets(long long rows_max, const int * nv, const int * slot_of, const float * x, const float * prev,
                        const float * xm1, const float * d2p, const float * ahat, const CgState * cg, float * target,
                        cudaStream_t st);
// Rows b0 .. b0 + nb - 1 of a pseudo-random permutation of the n rows (a Feistel
// network on 2 x half bits, 2^(2 half) >= n, keyed by key[4]) into dst / dst_t.
void launch_gather_shuffled(const float * src, const float * src_t, long long n, long long b0, long long nb, int half,
                            const unsigned * key, float * dst, float * dst_t, cudaStream_t st);
// Per-block FP64 sums of ((pred - tgt) * inv_tstd)^2 over n rows into part[blocks].
void launch_sq_err(const float * pred, const float * tgt, long long n, float inv_tstd, double * part, int blocks,
                   cudaStream_t st);

// ---- host-side allocation fault injection (tests of the failure paths) ----
// True when the device allocation about to be made is the one armed by
// swc_debug_fail_alloc; that allocation then reports out-of-memory.
bool debug_alloc_should_fail();

}  // namespace swc
