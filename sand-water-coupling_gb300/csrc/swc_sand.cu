// swc_sand.cu -- the DEM sand step on the GPU and its C ABI (include/swc_sand.h).
//
// One step (DEMParticleSand<Dim>::advance, Cores/Physics/DEMParticleSand.cpp:90-94):
//   1. move x += v dt in float-float arithmetic, fused into the count pass of the
//      counting sort into cells of 2r (moveParticles + resetNearbySearcher,
//      DEMParticleSand.cpp:98-109);
//   2. one thread per sorted particle: contact forces of the particles within 2r
//      (DEMParticle::getForceSum, Cores/Structures/DEMParticle.cpp:126-134), the
//      friction of the boundary particles within 4r (DEMParticleSand.cpp:130-151)
//      and gravity (DEMParticleSand.cpp:111-115), written to a second velocity
//      buffer so every particle reads the velocities from the start of the pass.
// Positions are float-float (hi in pos, lo in plo): the pair distance, the test
// |d|^2 < (2r)^2 and the penetration 2r - |d| are evaluated from the exact
// difference of the pairs; everything after the penetration depth is FP32.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numbers>
#include <string>

#include "../../include/swc_sand.h"
#include "swc_kernels.h"

using namespace swc;

namespace swc {

// Constants of the contact model (DEMParticle.cpp:15-33) and the boundary kernel.
struct SandPhys {
    float R, R2;              // contact reach 2r and (2r)^2, FP32 (cell windows)
    float Rh, Rl, R2h, R2l;   // 2r and (2r)^2 as float-float (exact tests)
    float Rb, Rb2;            // boundary reach 4r and (4r)^2
    float c0b, inv_hb;        // W_4r: normalisation and 1 / 4r
    float rclamp;             // 1e-4 r, the distance clamp of the normal
    float Kn, Kt, tanf;       // K_norm, K_tang, tan(friction angle)
    float drup, cap_a, cap_b; // d_rupture, V_bridge / (pi r), 2 / r
    float cap_neck, cap_surf; // -2 pi c r cos(theta), -2 pi c r sin(theta)
    float dt, gdt;            // step and 9.8 dt (0 without gravity)
};

namespace {

constexpr int kSandNT   = 256;
constexpr int kSandList = 16;  // candidates per thread gathered before their pair terms run

inline int sand_grid(long long n, int threads, int cap = 152 * 16) {
    const long long g = (n + threads - 1) / threads;
    return int(std::max<long long>(1, std::min<long long>(g, cap)));
}

// W_4r (SmoothedParticles::kernel, Cores/Structures/SmoothedParticles.h:60-65).
__device__ __forceinline__ float sand_wb(const SandPhys & P, float dist) {
    const float x = dist * P.inv_hb;
    if (x < .5f) return P.c0b * (6.f * x * x * (x - 1.f) + 1.f);
    if (x < 1.f) {
        const float y = 1.f - x;
        return P.c0b * 2.f * y * y * y;
    }
    return 0.f;
}

// FP64 host values -> float-float device pairs; velocities rounded to FP32.
__global__ void k_sand_import(const double * __restrict__ x, const double * __restrict__ v, int dim, long long n,
                              float4 * __restrict__ hi, float4 * __restrict__ lo, float4 * __restrict__ vel,
                              int * __restrict__ id) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f}, u[3] = {0.f, 0.f, 0.f};
        for (int a = 0; a < dim; a++) {
            const double d = x[i * dim + a];
            h[a]           = float(d);
            l[a]           = float(d - double(h[a]));
            if (v) u[a] = float(v[i * dim + a]);
        }
        hi[i] = make_float4(h[0], h[1], h[2], 0.f);
        lo[i] = make_float4(l[0], l[1], l[2], 0.f);
        if (vel) vel[i] = make_float4(u[0], u[1], u[2], 0.f);
        if (id) id[i] = int(i);
    }
}

__global__ void k_sand_import_vec(const double * __restrict__ x, int dim, long long n, float4 * __restrict__ out) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        float u[3] = {0.f, 0.f, 0.f};
        for (int a = 0; a < dim; a++) u[a] = float(x[i * dim + a]);
        out[i] = make_float4(u[0], u[1], u[2], 0.f);
    }
}

__global__ void k_sand_export(const float4 * __restrict__ hi, const float4 * __restrict__ lo,
                              const float4 * __restrict__ vel, const int * __restrict__ id, int dim, long long n,
                              double * __restrict__ x, double * __restrict__ v) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x) {
        const long long i = id[s];
        const float4 h = hi[s], l = lo[s], u = vel[s];
        const float hh[3] = {h.x, h.y, h.z}, ll[3] = {l.x, l.y, l.z}, uu[3] = {u.x, u.y, u.z};
        for (int a = 0; a < dim; a++) {
            if (x) x[i * dim + a] = double(hh[a]) + double(ll[a]);
            if (v) v[i * dim + a] = double(uu[a]);
        }
    }
}

__global__ void k_sand_boundary_out(const float * __restrict__ brho, const float4 * __restrict__ bpos,
                                    const int * __restrict__ bid, long long nb, double * __restrict__ rho,
                                    double * __restrict__ vol) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < nb; s += (long long) gridDim.x * blockDim.x) {
        const int i = bid[s];
        if (rho) rho[i] = brho[s];
        if (vol) vol[i] = bpos[s].w;
    }
}

// rho_b = m sum_{b'} W_4r(x_b - x_b') over the boundary particles within 4r
// (SmoothedParticles::computeDensities / computeVolumes, SmoothedParticles.cpp:25-36).
template<int DIM>
__global__ void __launch_bounds__(kSandNT) k_sand_boundary_density(Lattice L, SandPhys P, const int * __restrict__ bcellStart,
                                                                  const float4 * __restrict__ bpos,
                                                                  const float4 * __restrict__ blo, long long nb,
                                                                  float mass, float * __restrict__ brho) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < nb; i += (long long) gridDim.x * blockDim.x) {
        const float4 q = bpos[i], ql = blo[i];
        float s = 0.f;
        for_each_in_radius<DIM>(L, bcellStart, q.x, q.y, q.z, P.Rb * 1.0001f, P.Rb2 * 1.0002f, [&](int j) {
            const float4 p = bpos[j], pl = blo[j];
            const float dx = (q.x - p.x) + (ql.x - pl.x), dy = (q.y - p.y) + (ql.y - pl.y);
            const float dz = DIM == 3 ? (q.z - p.z) + (ql.z - pl.z) : 0.f;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < P.Rb2) s += sand_wb(P, sqrtf(r2));
        });
        brho[i] = mass * s;
    }
}
__global__ void k_sand_set_volume(float4 * __restrict__ bpos, const float * __restrict__ brho, long long nb, float mass) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < nb; i += (long long) gridDim.x * blockDim.x)
        bpos[i].w = mass / brho[i];
}

// Cells that hold boundary particles, then dilated along each axis by k cells:
// a sand particle whose cell is unmarked has no boundary particle within 4r.
__global__ void k_sand_occupied(const int * __restrict__ bcellStart, long long ncells, unsigned char * __restrict__ out) {
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < ncells; c += (long long) gridDim.x * blockDim.x)
        out[c] = bcellStart[c + 1] > bcellStart[c] ? 1 : 0;
}
__global__ void k_sand_dilate(Lattice L, int axis, int k, const unsigned char * __restrict__ in,
                              unsigned char * __restrict__ out) {
    const long long stride = axis == 0 ? 1 : (axis == 1 ? L.nx : (long long) L.nx * L.ny);
    const int len          = axis == 0 ? L.nx : (axis == 1 ? L.ny : L.nz);
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < L.ncells; c += (long long) gridDim.x * blockDim.x) {
        const int t = int((c / stride) % len);
        unsigned char m = 0;
        for (int o = -k; o <= k && !m; o++) {
            const int u = t + o;
            if (u >= 0 && u < len) m = in[c + (long long) o * stride];
        }
        out[c] = m;
    }
}

// max |v| as the bits of a non-negative float (their order is the integer order).
__global__ void k_sand_vmax(const float4 * __restrict__ vel, long long n, unsigned * __restrict__ bits) {
    float m = 0.f;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const float4 u = vel[i];
        m              = fmaxf(m, sqrtf(u.x * u.x + u.y * u.y + u.z * u.z));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(bits, __float_as_uint(m));
}

// Order-preserving map of floats to unsigned integers (for atomic min / max).
__device__ __forceinline__ unsigned f2ord(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

// Box of the positions after this step's move, x + v dt (FP32; the lattice pads
// it and clamps whatever falls outside): box[0..2] minima, box[3..5] maxima.
template<int DIM>
__global__ void k_sand_bbox(const float4 * __restrict__ pos, const float4 * __restrict__ vel, long long n, float dt,
                            unsigned * __restrict__ box) {
    pdl_wait_and_release();
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const float4 p = pos[i], u = vel[i];
        const float q[3] = {fmaf(u.x, dt, p.x), fmaf(u.y, dt, p.y), fmaf(u.z, dt, p.z)};
        for (int a = 0; a < DIM; a++)
            if (fabsf(q[a]) < 3.0e38f) {
                lo[a] = fminf(lo[a], q[a]);
                hi[a] = fmaxf(hi[a], q[a]);
            }
    }
    // warp, then block (256 threads), then one atomic per block and bound
    __shared__ float sl[3][8], sh[3][8];
    for (int a = 0; a < DIM; a++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
        if ((threadIdx.x & 31) == 0) {
            sl[a][threadIdx.x >> 5] = lo[a];
            sh[a][threadIdx.x >> 5] = hi[a];
        }
    }
    __syncthreads();
    if (threadIdx.x < DIM) {
        const int a = threadIdx.x;
        float l = sl[a][0], h = sh[a][0];
        for (int w = 1; w < int(blockDim.x >> 5); w++) {
            l = fminf(l, sl[a][w]);
            h = fmaxf(h, sh[a][w]);
        }
        if (l <= h) {
            atomicMin(box + a, f2ord(l));
            atomicMax(box + 3 + a, f2ord(h));
        }
    }
}

// One thread: the step's cell lattice over the box (clipped to the home box),
// cells of 2r doubled until the lattice fits `cap` cells, two cells of margin;
// then the box accumulators are reset for the next step.
__global__ void k_sand_lattice(unsigned * __restrict__ box, float3 home_lo, float3 home_hi, float cell0, long long cap,
                               int dim, Lattice * __restrict__ Ld) {
    pdl_wait_and_release();
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float hl[3] = {home_lo.x, home_lo.y, home_lo.z}, hh[3] = {home_hi.x, home_hi.y, home_hi.z};
    float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
    for (int a = 0; a < dim; a++) {
        if (box[a] != 0xffffffffu) {
            lo[a] = fmaxf(ord2f(box[a]), hl[a]);
            hi[a] = fminf(ord2f(box[3 + a]), hh[a]);
            if (lo[a] > hi[a]) lo[a] = hi[a] = fminf(fmaxf(lo[a], hl[a]), hh[a]);
        }
        box[a]     = 0xffffffffu;
        box[3 + a] = 0u;
    }
    // the cell grows by at least 2x (or the factor the cell count asks for) until it fits
    double cell = cell0, dims[3] = {1, 1, 1};
    for (int it = 0; it < 64; it++) {
        double total = 1;
        for (int a = 0; a < dim; a++) {
            dims[a] = floor((double(hi[a]) - double(lo[a])) / cell) + 5;
            total *= dims[a];
        }
        if (total <= double(cap)) break;
        cell *= fmax(2.0, 1.01 * pow(total / double(cap), 1.0 / dim));
    }
    cell = fmin(cell, 1e37);
    Lattice L{};
    L.ox     = float(lo[0] - 2 * cell);
    L.oy     = float(lo[1] - 2 * cell);
    L.oz     = dim == 3 ? float(lo[2] - 2 * cell) : 0.f;
    L.dx     = float(cell);
    L.inv_dx = float(1 / cell);
    L.nx     = int(dims[0]);
    L.ny     = int(dims[1]);
    L.nz     = dim == 3 ? int(dims[2]) : 1;
    L.bnx = L.bny = L.bnz = L.nbricks = 1;
    L.ncells = (long long) L.nx * L.ny * L.nz;
    *Ld      = L;
}

// The contact pass.  d = x_j - x_i, w = v_j - v_i as in DEMParticle::getForce
// (DEMParticle.cpp:62-67).
template<int DIM>
__global__ void __launch_bounds__(kSandNT, 5) k_sand_forces(const Lattice * __restrict__ Ld, Lattice Lb, SandPhys P,
                                                        const int * __restrict__ cellStart,
                                                        const float4 * __restrict__ pos, const float4 * __restrict__ plo,
                                                        const float4 * __restrict__ vel, float4 * __restrict__ vel_out,
                                                        long long n, const int * __restrict__ bcellStart,
                                                        const float4 * __restrict__ bpos,
                                                        const float4 * __restrict__ blo,
                                                        const float4 * __restrict__ bnrm,
                                                        const unsigned char * __restrict__ bnear) {
    pdl_wait_and_release();
    __shared__ int clist[kSandList * kSandNT];  // per-thread candidate lists, slot-major
    const Lattice L = *Ld;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const float4 qi = pos[i], li = plo[i], vi = vel[i];
        // The FP32 window and pre-test ignore the low parts (|lo| <= 2^-24 |x|) and
        // round the difference once: widen the reach by 2^-21 (|x|_max + 2r).
        const float ax  = fmaxf(fabsf(qi.x), fmaxf(fabsf(qi.y), DIM == 3 ? fabsf(qi.z) : 0.f));
        const float Rq  = P.R + ldexpf(ax + P.R, -21);
        const float Rq2 = Rq * Rq * 1.000001f;
        float fx = 0.f, fy = 0.f, fz = 0.f;
        // the pair terms of the candidates that pass the FP32 pre-test; run from the
        // per-thread list below so the lanes of a warp take this path together
        auto contact = [&](int j) {
            const float4 qj = pos[j];
            const float4 lj = plo[j];
            float hx, lx, hy, ly, hz = 0.f, lz = 0.f;
            ff_diff(qj.x, lj.x, qi.x, li.x, hx, lx);
            ff_diff(qj.y, lj.y, qi.y, li.y, hy, ly);
            if (DIM == 3) ff_diff(qj.z, lj.z, qi.z, li.z, hz, lz);
            float Dh = 0.f, Dl = 0.f;
            ff_sqr_add(hx, lx, Dh, Dl);
            ff_sqr_add(hy, ly, Dh, Dl);
            if (DIM == 3) ff_sqr_add(hz, lz, Dh, Dl);
            // the searcher's strict test |d|^2 < (2r)^2
            // (Cores/Structures/ParticlesNearbySearcher.cpp:27-33)
            if (!(Dh < P.R2h || (Dh == P.R2h && Dl < P.R2l))) return;
            // |d| = s0 + sl: one Newton correction of the rounded square root
            const float s0 = __fsqrt_rn(Dh);
            const float sl = s0 > 0.f ? __fmul_rn(__fadd_rn(__fmaf_rn(-s0, s0, Dh), Dl), __fdividef(0.5f, s0)) : 0.f;
            // penetration 2r - |d| (DEMParticle.cpp:72-73); Rh - s0 is exact for |d| >= r
            const float pen = __fadd_rn(__fsub_rn(P.Rh, s0), __fsub_rn(P.Rl, sl));
            if (pen > 0.f) {
                // DEMParticle::ComputeDemForces (DEMParticle.cpp:74-94)
                const float dist = __fadd_rn(s0, sl);
                const bool clamp = dist <= P.rclamp;
                const float inv  = __frcp_rn(clamp ? P.rclamp : dist);
                const float nx = __fadd_rn(hx, lx) * inv, ny = __fadd_rn(hy, ly) * inv;
                const float nz = DIM == 3 ? __fadd_rn(hz, lz) * inv : 0.f;
                const float4 vj = vel[j];
                const float wx = vj.x - vi.x, wy = vj.y - vi.y, wz = DIM == 3 ? vj.z - vi.z : 0.f;
                const float dn = wx * nx + wy * ny + wz * nz;
                float tx = wx - dn * nx, ty = wy - dn * ny, tz = wz - dn * nz;
                if (tx * tx + ty * ty + tz * tz < 1e-4f * (wx * wx + wy * wy + wz * wz)) {
                    // |w_t| < |w| / 100: the FP32 difference w - (w.n) n keeps few digits
                    // and the capped shear takes its direction; redo it in FP64 (rare)
                    const double inv_d = 1.0 / fmax(double(s0) + double(sl), double(P.rclamp));
                    const double mx = (double(hx) + double(lx)) * inv_d, my = (double(hy) + double(ly)) * inv_d;
                    const double mz = DIM == 3 ? (double(hz) + double(lz)) * inv_d : 0.0;
                    const double Wx = double(vj.x) - double(vi.x), Wy = double(vj.y) - double(vi.y);
                    const double Wz = DIM == 3 ? double(vj.z) - double(vi.z) : 0.0;
                    const double dd = Wx * mx + Wy * my + Wz * mz;
                    tx = float(Wx - dd * mx);
                    ty = float(Wy - dd * my);
                    tz = float(Wz - dd * mz);
                }
                const float kp = P.Kn * pen;
                const float Nx = kp * nx, Ny = kp * ny, Nz = kp * nz;
                float Sx = -P.Kt * tx, Sy = -P.Kt * ty, Sz = -P.Kt * tz;
                // |normal| = K_n pen |n|, |n| = 1 unless the distance was clamped
                const float max_fs = kp * (clamp ? dist * inv : 1.f) * P.tanf;
                const float sn2    = Sx * Sx + Sy * Sy + Sz * Sz;
                if (sn2 > max_fs * max_fs) {
                    const float k = max_fs * rsqrtf(sn2);
                    Sx *= k;
                    Sy *= k;
                    Sz *= k;
                }
                fx -= Nx + Sx;
                fy -= Ny + Sy;
                fz -= Nz + Sz;
            }
            // DEMParticle::ComputeDemCapillaryForces (DEMParticle.cpp:98-124).  Every pair
            // that gets here has |d| < 2r, so H = |d| - 2r < 0 fails H > 1e-6: the
            // liquid bridge never acts between neighbours found within 2r.
            const float H = -pen;
            if (H < P.drup && H > 1e-6f) {
                const float dist = __fadd_rn(s0, sl);
                const float dd   = -H + sqrtf(H * H + P.cap_a);
                const float phi  = sqrtf(P.cap_b * H * (-1.f + sqrtf(1.f + P.cap_a / (H * H))));
                const float s    = P.cap_neck / (1.f + H / (2.f * dd)) + P.cap_surf * phi;
                const float inv  = 1.f / dist;
                fx -= __fadd_rn(hx, lx) * inv * s;
                fy -= __fadd_rn(hy, ly) * inv * s;
                fz -= __fadd_rn(hz, lz) * inv * s;
            }
        };
        int cnt = 0;
        for_each_in_radius<DIM>(L, cellStart, qi.x, qi.y, qi.z, Rq, Rq2, [&](int j) {
            if (j == int(i)) return;  // d = 0, w = 0: the reference's self term is zero
            const float4 qj = pos[j];
            const float ex = qj.x - qi.x, ey = qj.y - qi.y, ez = DIM == 3 ? qj.z - qi.z : 0.f;
            if (ex * ex + ey * ey + ez * ez >= Rq2) return;
            clist[cnt * kSandNT + threadIdx.x] = j;
            if (++cnt == kSandList) {
                for (int k = 0; k < cnt; k++) contact(clist[k * kSandNT + threadIdx.x]);
                cnt = 0;
            }
        });
        for (int k = 0; k < cnt; k++) contact(clist[k * kSandNT + threadIdx.x]);
        // force = dt * sum_j F_ij, then the boundary terms without dt (DEMParticleSand.cpp:133-150)
        float Fx = fx * P.dt, Fy = fy * P.dt, Fz = fz * P.dt;
        if (bnear[cell_linear(Lb, cell_of<DIM>(Lb, qi.x, qi.y, qi.z))]) {
            for_each_in_radius<DIM>(Lb, bcellStart, qi.x, qi.y, qi.z, P.Rb * 1.0001f, P.Rb2 * 1.0002f, [&](int j) {
                const float4 pb = bpos[j], lb = blo[j];
                const float dx = (qi.x - pb.x) + (li.x - lb.x), dy = (qi.y - pb.y) + (li.y - lb.y);
                const float dz = DIM == 3 ? (qi.z - pb.z) + (li.z - lb.z) : 0.f;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 >= P.Rb2) return;
                const float w   = sand_wb(P, sqrtf(r2));
                const float4 nb = bnrm[j];
                // dv = v_i - v_b with v_b = 0 (the reference's _boundary_velocity is never set)
                const float dvn = nb.x * vi.x + nb.y * vi.y + nb.z * vi.z;
                const float m   = -pb.w * fminf(dvn, 0.f);
                const float Nx = m * nb.x * w, Ny = m * nb.y * w, Nz = m * nb.z * w;
                float ux = vi.x - dvn * nb.x, uy = vi.y - dvn * nb.y, uz = DIM == 3 ? vi.z - dvn * nb.z : 0.f;
                if (ux * ux + uy * uy + uz * uz < 1e-4f * (vi.x * vi.x + vi.y * vi.y + vi.z * vi.z)) {
                    // nearly normal motion: the tangential part in FP64, as in the contacts
                    const double e = double(nb.x) * vi.x + double(nb.y) * vi.y + (DIM == 3 ? double(nb.z) * vi.z : 0.0);
                    ux = float(double(vi.x) - e * nb.x);
                    uy = float(double(vi.y) - e * nb.y);
                    uz = DIM == 3 ? float(double(vi.z) - e * nb.z) : 0.f;
                }
                const float Tx = -P.Kt * ux, Ty = -P.Kt * uy, Tz = -P.Kt * uz;
                const float nt = sqrtf(Tx * Tx + Ty * Ty + Tz * Tz);
                float k        = 1.f;
                if (nt > 0.000001f) {
                    const float cap = sqrtf(Nx * Nx + Ny * Ny + Nz * Nz) * P.tanf;
                    if (!(cap > nt)) k = cap / nt;
                }
                Fx += Nx + k * Tx;
                Fy += Ny + k * Ty;
                Fz += Nz + k * Tz;
            });
        }
        float4 o = vi;
        o.x += Fx;
        o.y += Fy;
        if (DIM == 3) o.z += Fz;
        o.y -= P.gdt;
        vel_out[i] = o;
    }
}

}  // namespace
}  // namespace swc

// ---------------------------------------------------------------------------
// Host context and C ABI
// ---------------------------------------------------------------------------
struct swc_sand {
    swc_sand_params p{};
    int dim = 2;
    std::string err;
    cudaStream_t stream = nullptr;
    bool own_stream     = false;
    Lattice Lb{};             // boundary lattice (static, host copy)
    Lattice Lcap{};           // sizes the sand cell arrays: ncells = capacity
    Lattice * dL     = nullptr;  // the sand lattice of the current step (device)
    unsigned * dbox  = nullptr;  // box accumulators of the next step (device)
    float home_lo[3] = {0, 0, 0}, home_hi[3] = {0, 0, 0};
    SandPhys P{};
    long long n = 0, nb = 0;
    float4 *pos = nullptr, *plo = nullptr, *vel = nullptr, *vel2 = nullptr;
    int * id = nullptr;
    SortScratch S{};
    float4 *bpos = nullptr, *blo = nullptr, *bnrm = nullptr;
    int * bid     = nullptr;
    float * brho  = nullptr;
    int *cellStart = nullptr, *bcellStart = nullptr;
    unsigned char *bnear = nullptr, *btmp = nullptr;
    double * stage    = nullptr;
    size_t stage_cap  = 0;
    unsigned * vbits  = nullptr;
    double bb_lo[3] = {0, 0, 0}, bb_hi[3] = {0, 0, 0};    // every particle set so far
    double bbb_lo[3] = {0, 0, 0}, bbb_hi[3] = {0, 0, 0};  // boundary particles
    bool has_bb = false, has_bbb = false;
    bool initialized = false;
    bool sorted      = false;  // the particle arrays follow the cells of the current lattice
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace {

#define SK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            if (s) s->err = std::string(#call) + ": " + cudaGetErrorString(e_);                                        \
            return e_ == cudaErrorMemoryAllocation ? SWC_OUT_OF_MEMORY : SWC_CUDA_ERROR;                               \
        }                                                                                                              \
    } while (0)

template<class T> int salloc(swc_sand * s, T ** p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (count == 0) count = 1;
    if (swc::debug_alloc_should_fail()) {
        s->err = "cudaMalloc: out of memory (injected)";
        return SWC_OUT_OF_MEMORY;
    }
    SK(cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * count));
    return SWC_OK;
}
template<class T> void sfree(T *& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

int ensure_stage(swc_sand * s, size_t doubles) {
    if (doubles <= s->stage_cap && s->stage) return SWC_OK;
    SK(cudaStreamSynchronize(s->stream));
    int rc = salloc(s, &s->stage, doubles);
    if (rc) return rc;
    s->stage_cap = doubles;
    return SWC_OK;
}

void grow_box(int dim, const double * x, long long n, double * lo, double * hi, bool & has) {
    for (long long i = 0; i < n; i++)
        for (int a = 0; a < dim; a++) {
            const double v = x[i * dim + a];
            if (!std::isfinite(v)) continue;
            if (!has) {
                for (int b = 0; b < 3; b++) lo[b] = hi[b] = 0;
                for (int b = 0; b < dim; b++) lo[b] = hi[b] = std::isfinite(x[i * dim + b]) ? x[i * dim + b] : 0.0;
                has = true;
            }
            lo[a] = std::min(lo[a], v);
            hi[a] = std::max(hi[a], v);
        }
}

void setup_phys(swc_sand * s) {
    const double r = s->p.radius, R = 2 * r, Rb = 4 * r;
    SandPhys & P   = s->P;
    P.R            = float(R);
    P.R2           = float(R * R);
    P.Rh           = float(R);
    P.Rl           = float(R - double(P.Rh));
    P.R2h          = float(R * R);
    P.R2l          = float(R * R - double(P.R2h));
    P.Rb           = float(Rb);
    P.Rb2          = float(Rb * Rb);
    P.inv_hb       = float(1 / Rb);
    P.c0b          = float(std::numbers::inv_pi / (Rb * Rb) * (s->dim == 2 ? 40.0 / 7 : 8 / Rb));
    P.rclamp       = float(0.0001 * r);
    const double Kn = s->p.young * r, Kt = Kn * s->p.poisson;
    P.Kn           = float(Kn);
    P.Kt           = float(Kt);
    P.tanf         = float(std::tan(s->p.fric_angle));
    // capillary constants (DEMParticle.cpp:20-31); coefficient G.calculate(0.1) = 1
    const double theta = 30. / 180. * std::numbers::pi;
    const double vlb   = 4. / 3. * std::numbers::pi * std::pow(r, 3.) * 0.01 * 0.01;
    P.drup     = float((1.f + 0.5f * theta) * (std::pow(vlb, 1. / 3.) + 0.1 * std::pow(vlb, 2. / 3.)));
    P.cap_a    = float(vlb / (std::numbers::pi * r));
    P.cap_b    = float(2. / r);
    P.cap_neck = float(-2. * std::numbers::pi * r * std::cos(theta));
    P.cap_surf = float(-2. * std::numbers::pi * r * std::sin(theta));
    P.dt = P.gdt = 0.f;
}

// A static lattice of cells of 2r over [lo, hi] plus two cells; the cell
// doubles while it would exceed `cap` cells.
Lattice box_lattice(int dim, const double * lo, const double * hi, double cell, long long cap) {
    Lattice L{};
    long long dims[3] = {1, 1, 1};
    for (int it = 0; it < 64; it++) {
        double total = 1;
        for (int a = 0; a < dim; a++) {
            dims[a] = (long long) std::floor((hi[a] - lo[a]) / cell) + 5;
            total *= double(dims[a]);
        }
        if (total <= double(cap)) break;
        cell *= 2;
    }
    L.ox_d   = lo[0] - 2 * cell;
    L.oy_d   = lo[1] - 2 * cell;
    L.oz_d   = dim == 3 ? lo[2] - 2 * cell : 0.0;
    L.ox     = float(L.ox_d);
    L.oy     = float(L.oy_d);
    L.oz     = float(L.oz_d);
    L.dx_d   = cell;
    L.dx     = float(cell);
    L.inv_dx = float(1 / cell);
    L.nx     = int(dims[0]);
    L.ny     = int(dims[1]);
    L.nz     = dim == 3 ? int(dims[2]) : 1;
    L.bnx = L.bny = L.bnz = L.nbricks = 1;
    L.ncells = (long long) L.nx * L.ny * L.nz;
    return L;
}

int alloc_particle_sort(swc_sand * s) {
    int rc;
    SortScratch & S = s->S;
    if ((rc = salloc(s, &S.key, s->n)) || (rc = salloc(s, &S.rank, s->n)) || (rc = salloc(s, &S.perm, s->n)) ||
        (rc = salloc(s, &S.pos2, s->n)) || (rc = salloc(s, &S.vel2, s->n)) || (rc = salloc(s, &S.aux2, s->n)) ||
        (rc = salloc(s, &S.id2, s->n)))
        return rc;
    return SWC_OK;
}

// Sand cell arrays sized for max(2^20, 4 n) cells: a packed block needs about
// 0.7 n cells of 2r; a spread-out one gets coarser cells instead of more.
int ensure_sand_cells(swc_sand * s) {
    const long long cap = std::min<long long>((1LL << 31) - 2, std::max<long long>(1LL << 20, 4 * s->n));
    if (s->cellStart && s->Lcap.ncells == cap) return SWC_OK;
    SK(cudaStreamSynchronize(s->stream));
    s->Lcap        = Lattice{};
    s->Lcap.ncells = cap;
    int rc;
    if ((rc = salloc(s, &s->cellStart, cap + 1)) || (rc = salloc(s, &s->S.count, cap)) ||
        (rc = salloc(s, &s->S.tiles, scan_tile_count(cap + 1) + 2)))
        return rc;
    return SWC_OK;
}

// The step's lattice from the box of x + v dt (dt = 0: the current positions),
// then the counting sort (with the float-float move when dt != 0).
template<int DIM> void bin_sand(swc_sand * s, float dth, float dtl) {
    cudaStream_t st = s->stream;
    if (s->n > 0)
        launch_pdl(k_sand_bbox<DIM>, sand_grid(s->n, 256, 152 * 8), 256, 0, st, (const float4 *) s->pos,
                   (const float4 *) s->vel, s->n, dth, s->dbox);
    launch_pdl(k_sand_lattice, 1, 32, 0, st, s->dbox, make_float3(s->home_lo[0], s->home_lo[1], s->home_lo[2]),
               make_float3(s->home_hi[0], s->home_hi[1], s->home_hi[2]), s->P.R, s->Lcap.ncells, s->dim, s->dL);
    launch_bin<DIM>(s->Lcap, s->n, s->pos, s->vel, s->plo, s->id, s->S, s->cellStart, dth, st, dtl, true, s->dL);
    s->sorted = true;
}

template<int DIM> int do_initialize(swc_sand * s) {
    SK(cudaStreamSynchronize(s->stream));
    int rc;
    cudaStream_t st = s->stream;
    const double cell = 2 * s->p.radius;
    // home box: every particle's box widened by its own extent (at least 8r) on each
    // side; the step lattices stay inside it, whatever leaves it is clamped in
    for (int a = 0; a < 3; a++) {
        const double lo = s->has_bb ? s->bb_lo[a] : 0.0, hi = s->has_bb ? s->bb_hi[a] : 0.0;
        const double ext = std::max(hi - lo, 4 * cell);
        s->home_lo[a]    = float(lo - ext);
        s->home_hi[a]    = float(hi + ext);
    }
    // boundary: one static lattice, sorted once, densities and volumes
    {
        double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        if (s->has_bbb)
            for (int a = 0; a < 3; a++) lo[a] = s->bbb_lo[a], hi[a] = s->bbb_hi[a];
        const long long cap = std::min<long long>((1LL << 31) - 2, std::max<long long>(1LL << 22, 8 * s->nb));
        s->Lb = box_lattice(s->dim, lo, hi, cell, cap);
    }
    const Lattice & Lb = s->Lb;
    if ((rc = salloc(s, &s->bcellStart, Lb.ncells + 1)) || (rc = salloc(s, &s->bnear, Lb.ncells)) ||
        (rc = salloc(s, &s->btmp, Lb.ncells)))
        return rc;
    SortScratch B{};
    if ((rc = salloc(s, &B.key, s->nb)) || (rc = salloc(s, &B.rank, s->nb)) || (rc = salloc(s, &B.perm, s->nb)) ||
        (rc = salloc(s, &B.pos2, s->nb)) || (rc = salloc(s, &B.vel2, s->nb)) || (rc = salloc(s, &B.aux2, s->nb)) ||
        (rc = salloc(s, &B.id2, s->nb)) || (rc = salloc(s, &B.count, Lb.ncells)) ||
        (rc = salloc(s, &B.tiles, scan_tile_count(Lb.ncells + 1) + 2)))
        return rc;
    launch_bin<DIM>(Lb, s->nb, s->bpos, s->bnrm, s->blo, s->bid, B, s->bcellStart, 0.f, st);
    SK(cudaGetLastError());
    SK(cudaStreamSynchronize(st));
    sfree(B.key);
    sfree(B.rank);
    sfree(B.perm);
    sfree(B.pos2);
    sfree(B.vel2);
    sfree(B.aux2);
    sfree(B.id2);
    sfree(B.count);
    sfree(B.tiles);
    if (s->nb > 0) {
        k_sand_boundary_density<DIM><<<sand_grid(s->nb, kSandNT), kSandNT, 0, st>>>(
            Lb, s->P, s->bcellStart, s->bpos, s->blo, s->nb, float(s->p.mass), s->brho);
        k_sand_set_volume<<<sand_grid(s->nb, 256), 256, 0, st>>>(s->bpos, s->brho, s->nb, float(s->p.mass));
    }
    // boundary cells dilated by the reach 4r (at most two cells) plus one
    const int k = int(std::ceil(4 * s->p.radius / Lb.dx_d)) + 1;
    k_sand_occupied<<<sand_grid(Lb.ncells, 256), 256, 0, st>>>(s->bcellStart, Lb.ncells, s->btmp);
    unsigned char *a = s->btmp, *b = s->bnear;
    for (int axis = 0; axis < DIM; axis++) {
        k_sand_dilate<<<sand_grid(Lb.ncells, 256), 256, 0, st>>>(Lb, axis, k, a, b);
        std::swap(a, b);
    }
    if (a != s->bnear) SK(cudaMemcpyAsync(s->bnear, a, Lb.ncells, cudaMemcpyDeviceToDevice, st));
    // sand: cell arrays, box accumulators (min = all ones, max = 0), first binning
    if ((rc = ensure_sand_cells(s))) return rc;
    SK(cudaMemsetAsync(s->dbox, 0xff, 3 * sizeof(unsigned), st));
    SK(cudaMemsetAsync(s->dbox + 3, 0, 3 * sizeof(unsigned), st));
    bin_sand<DIM>(s, 0.f, 0.f);
    SK(cudaGetLastError());
    SK(cudaStreamSynchronize(st));
    s->initialized = true;
    return SWC_OK;
}

template<int DIM> void launch_forces(swc_sand * s, float4 * out) {
    if (s->n == 0) return;
    launch_pdl(k_sand_forces<DIM>, sand_grid(s->n, kSandNT, 152 * 64), kSandNT, 0, s->stream, (const Lattice *) s->dL,
               s->Lb, s->P, (const int *) s->cellStart, (const float4 *) s->pos, (const float4 *) s->plo,
               (const float4 *) s->vel, out, s->n, (const int *) s->bcellStart, (const float4 *) s->bpos,
               (const float4 *) s->blo, (const float4 *) s->bnrm, (const unsigned char *) s->bnear);
}

template<int DIM> int do_advance(swc_sand * s, double dt) {
    const float dth = float(dt), dtl = float(dt - double(dth));
    s->P.dt  = dth;
    s->P.gdt = s->p.enable_gravity ? float(9.8 * dt) : 0.f;  // kGravity, Cores/Utilities/Constants.h:7
    bin_sand<DIM>(s, dth, dtl);
    launch_forces<DIM>(s, s->vel2);
    std::swap(s->vel, s->vel2);
    SK(cudaGetLastError());
    return SWC_OK;
}

bool valid(const swc_sand * s) { return s != nullptr; }

}  // namespace

extern "C" {

void swc_sand_default_params(swc_sand_params * p) {
    if (!p) return;
    *p                = swc_sand_params{};
    p->dim            = 2;
    p->enable_gravity = 1;
    p->radius         = 1.0 / 120;  // DEMParticleSandBuilder case 0 at its default scale 30
    p->mass           = 1;
    p->young          = 1e9;
    p->poisson        = 0.3;
    p->fric_angle     = 0.5;
}

const char * swc_sand_last_error(const swc_sand * s) { return s ? s->err.c_str() : "null context"; }

int swc_sand_create(const swc_sand_params * p, swc_sand ** out) {
    if (!p || !out) return SWC_BAD_ARG;
    *out = nullptr;
    if ((p->dim != 2 && p->dim != 3) || !(p->radius > 0) || !(p->mass > 0) || !(p->young >= 0) || !(p->poisson >= 0))
        return SWC_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SWC_CUDA_ERROR;
    auto * s = new swc_sand();
    s->p     = *p;
    s->dim   = p->dim;
    setup_phys(s);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return SWC_CUDA_ERROR;
    }
    s->own_stream = true;
    int rc;
    if ((rc = salloc(s, &s->vbits, 1)) || (rc = salloc(s, &s->dL, 1)) || (rc = salloc(s, &s->dbox, 6))) {
        swc_sand_destroy(s);
        return rc;
    }
    cudaEventCreate(&s->e0);
    cudaEventCreate(&s->e1);
    *out = s;
    return SWC_OK;
}

void swc_sand_destroy(swc_sand * s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    sfree(s->pos);
    sfree(s->plo);
    sfree(s->vel);
    sfree(s->vel2);
    sfree(s->id);
    sfree(s->S.key);
    sfree(s->S.rank);
    sfree(s->S.perm);
    sfree(s->S.count);
    sfree(s->S.tiles);
    sfree(s->S.pos2);
    sfree(s->S.vel2);
    sfree(s->S.aux2);
    sfree(s->S.id2);
    sfree(s->bpos);
    sfree(s->blo);
    sfree(s->bnrm);
    sfree(s->bid);
    sfree(s->brho);
    sfree(s->cellStart);
    sfree(s->bcellStart);
    sfree(s->bnear);
    sfree(s->btmp);
    sfree(s->stage);
    sfree(s->vbits);
    sfree(s->dL);
    sfree(s->dbox);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int swc_sand_set_stream(swc_sand * s, void * stream) {
    if (!valid(s)) return SWC_BAD_ARG;
    SK(cudaStreamSynchronize(s->stream));
    if (s->own_stream) cudaStreamDestroy(s->stream);
    if (stream) {
        s->stream     = static_cast<cudaStream_t>(stream);
        s->own_stream = false;
    } else {
        SK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    return SWC_OK;
}

int swc_sand_set_particles(swc_sand * s, const double * x, const double * v, int64_t n) {
    if (!valid(s) || n < 0 || (n > 0 && !x) || n > (1LL << 30)) return SWC_BAD_ARG;
    int rc;
    // a failed allocation leaves no particles and an uninitialized context, so a
    // later advance returns SWC_NOT_INITIALIZED instead of reaching freed buffers
    auto fail = [s](int code) {
        s->n           = 0;
        s->initialized = false;
        s->sorted      = false;
        return code;
    };
    if (n != s->n || !s->pos) {
        SK(cudaStreamSynchronize(s->stream));
        s->n = n;
        if ((rc = salloc(s, &s->pos, n)) || (rc = salloc(s, &s->plo, n)) || (rc = salloc(s, &s->vel, n)) ||
            (rc = salloc(s, &s->vel2, n)) || (rc = salloc(s, &s->id, n)) || (rc = alloc_particle_sort(s)))
            return fail(rc);
    }
    // the box only places the home box at initialize; later states need no host pass
    if (!s->initialized) grow_box(s->dim, x, n, s->bb_lo, s->bb_hi, s->has_bb);
    if ((rc = ensure_stage(s, size_t(2) * std::max<int64_t>(n, 1) * s->dim))) return fail(rc);
    const size_t bytes = sizeof(double) * size_t(n) * s->dim;
    if (n > 0) {
        SK(cudaMemcpyAsync(s->stage, x, bytes, cudaMemcpyHostToDevice, s->stream));
        if (v) SK(cudaMemcpyAsync(s->stage + size_t(n) * s->dim, v, bytes, cudaMemcpyHostToDevice, s->stream));
        k_sand_import<<<sand_grid(n, 256), 256, 0, s->stream>>>(s->stage, v ? s->stage + size_t(n) * s->dim : nullptr,
                                                               s->dim, n, s->pos, s->plo, s->vel, s->id);
    }
    SK(cudaGetLastError());
    // cell arrays for a new count; the next advance sorts the particles into them
    if (s->initialized && (rc = ensure_sand_cells(s))) return fail(rc);
    s->sorted = false;
    return SWC_OK;
}

int swc_sand_get_particles(swc_sand * s, double * x, double * v, int64_t n) {
    if (!valid(s) || n != s->n) return SWC_BAD_ARG;
    if (n == 0) return SWC_OK;
    int rc;
    if ((rc = ensure_stage(s, size_t(2) * n * s->dim))) return rc;
    double * sx = s->stage;
    double * sv = s->stage + size_t(n) * s->dim;
    k_sand_export<<<sand_grid(n, 256), 256, 0, s->stream>>>(s->pos, s->plo, s->vel, s->id, s->dim, n,
                                                           x ? sx : nullptr, v ? sv : nullptr);
    const size_t bytes = sizeof(double) * size_t(n) * s->dim;
    if (x) SK(cudaMemcpyAsync(x, sx, bytes, cudaMemcpyDeviceToHost, s->stream));
    if (v) SK(cudaMemcpyAsync(v, sv, bytes, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    return SWC_OK;
}

int swc_sand_set_boundary(swc_sand * s, const double * x, const double * normals, int64_t nb) {
    if (!valid(s) || nb < 0 || (nb > 0 && (!x || !normals)) || nb > (1LL << 30)) return SWC_BAD_ARG;
    SK(cudaStreamSynchronize(s->stream));
    int rc;
    // the boundary changes: volumes and lattice wait for the next initialize, also
    // when an allocation below fails (no boundary is left then)
    s->initialized = false;
    s->nb          = nb;
    if ((rc = salloc(s, &s->bpos, nb)) || (rc = salloc(s, &s->blo, nb)) || (rc = salloc(s, &s->bnrm, nb)) ||
        (rc = salloc(s, &s->bid, nb)) || (rc = salloc(s, &s->brho, nb))) {
        s->nb = 0;
        return rc;
    }
    grow_box(s->dim, x, nb, s->bb_lo, s->bb_hi, s->has_bb);
    s->has_bbb = false;
    grow_box(s->dim, x, nb, s->bbb_lo, s->bbb_hi, s->has_bbb);
    if ((rc = ensure_stage(s, size_t(2) * std::max<int64_t>(nb, 1) * s->dim))) {
        s->nb = 0;
        return rc;
    }
    if (nb > 0) {
        const size_t bytes = sizeof(double) * size_t(nb) * s->dim;
        SK(cudaMemcpyAsync(s->stage, x, bytes, cudaMemcpyHostToDevice, s->stream));
        SK(cudaMemcpyAsync(s->stage + size_t(nb) * s->dim, normals, bytes, cudaMemcpyHostToDevice, s->stream));
        // positions as float-float pairs, normals in FP32
        k_sand_import<<<sand_grid(nb, 256), 256, 0, s->stream>>>(s->stage, nullptr, s->dim, nb, s->bpos, s->blo,
                                                                nullptr, s->bid);
        k_sand_import_vec<<<sand_grid(nb, 256), 256, 0, s->stream>>>(s->stage + size_t(nb) * s->dim, s->dim, nb,
                                                                    s->bnrm);
    }
    SK(cudaGetLastError());
    SK(cudaStreamSynchronize(s->stream));
    return SWC_OK;
}

int swc_sand_initialize(swc_sand * s) {
    if (!valid(s)) return SWC_BAD_ARG;
    return s->dim == 2 ? do_initialize<2>(s) : do_initialize<3>(s);
}

int swc_sand_advance(swc_sand * s, double dt) {
    if (!valid(s) || !std::isfinite(dt)) return SWC_BAD_ARG;
    if (!s->initialized) return SWC_NOT_INITIALIZED;
    return s->dim == 2 ? do_advance<2>(s, dt) : do_advance<3>(s, dt);
}

int swc_sand_get_time_step(swc_sand * s, double step_rate, double * dt) {
    if (!valid(s) || !dt) return SWC_BAD_ARG;
    SK(cudaMemsetAsync(s->vbits, 0, sizeof(unsigned), s->stream));
    if (s->n > 0) k_sand_vmax<<<sand_grid(s->n, 256, 152 * 4), 256, 0, s->stream>>>(s->vel, s->n, s->vbits);
    unsigned bits = 0;
    SK(cudaMemcpyAsync(&bits, s->vbits, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    float vmax;
    std::memcpy(&vmax, &bits, sizeof(float));
    *dt = step_rate * s->p.radius * 2 / double(vmax);
    return SWC_OK;
}

int swc_sand_get_boundary_info(swc_sand * s, double * rho, double * vol, int64_t nb) {
    if (!valid(s) || nb != s->nb) return SWC_BAD_ARG;
    if (!s->initialized) return SWC_NOT_INITIALIZED;
    if (nb == 0) return SWC_OK;
    int rc;
    if ((rc = ensure_stage(s, size_t(2) * nb))) return rc;
    k_sand_boundary_out<<<sand_grid(nb, 256), 256, 0, s->stream>>>(s->brho, s->bpos, s->bid, nb, rho ? s->stage : nullptr,
                                                                  vol ? s->stage + nb : nullptr);
    if (rho) SK(cudaMemcpyAsync(rho, s->stage, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream));
    if (vol) SK(cudaMemcpyAsync(vol, s->stage + nb, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    return SWC_OK;
}

int swc_sand_time_kernel(swc_sand * s, int which, int reps, double * mean_ms) {
    if (!valid(s) || !mean_ms || reps < 1 || which < 0 || which > 1) return SWC_BAD_ARG;
    if (!s->initialized) return SWC_NOT_INITIALIZED;
    SK(cudaStreamSynchronize(s->stream));
    if (which == 0 && !s->sorted) {
        if (s->dim == 2) bin_sand<2>(s, 0.f, 0.f);
        else bin_sand<3>(s, 0.f, 0.f);
    }
    SK(cudaEventRecord(s->e0, s->stream));
    for (int r = 0; r < reps; r++) {
        if (which == 0) {
            if (s->dim == 2) launch_forces<2>(s, s->vel2);
            else launch_forces<3>(s, s->vel2);
        } else {
            if (s->dim == 2) bin_sand<2>(s, 0.f, 0.f);
            else bin_sand<3>(s, 0.f, 0.f);
        }
    }
    SK(cudaEventRecord(s->e1, s->stream));
    SK(cudaEventSynchronize(s->e1));
    SK(cudaGetLastError());
    float ms = 0.f;
    SK(cudaEventElapsedTime(&ms, s->e0, s->e1));
    *mean_ms = double(ms) / reps;
    return SWC_OK;
}

}  // extern "C"
