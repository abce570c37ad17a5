// k_particles.cu -- particle-side kernels of the dual-particle SPH projection:
// host-format conversion, advection, counting-sort binning into node cells,
// real and boundary densities, gravity + div-free viscosity, brick activation,
// the pressure-gradient update G_i and the export back to host order.
#include "swc_kernels.h"

namespace swc {

// ---------------------------------------------------------------------------
// Host FP64 AoS (dim components per particle, the .sav layout of
// Cores/Utilities/IO.h:19-26) <-> device float4.
// ---------------------------------------------------------------------------
__global__ void k_import(const double * __restrict__ x, const double * __restrict__ v, int dim, long long n,
                         float4 * __restrict__ pos, float4 * __restrict__ vel, int * __restrict__ id) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f), u = make_float4(0.f, 0.f, 0.f, 0.f);
        p.x = float(x[i * dim]);
        p.y = float(x[i * dim + 1]);
        if (dim == 3) p.z = float(x[i * dim + 2]);
        if (v) {
            u.x = float(v[i * dim]);
            u.y = float(v[i * dim + 1]);
            if (dim == 3) u.z = float(v[i * dim + 2]);
        }
        pos[i] = p;
        vel[i] = u;
        if (id) id[i] = int(i);
    }
}

__global__ void k_export(const float4 * __restrict__ pos, const float4 * __restrict__ vel, const int * __restrict__ id,
                         int dim, long long n, double * __restrict__ x, double * __restrict__ v) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x) {
        const long long i = id[s];
        const float4 p = pos[s], u = vel[s];
        if (x) {
            x[i * dim]     = p.x;
            x[i * dim + 1] = p.y;
            if (dim == 3) x[i * dim + 2] = p.z;
        }
        if (v) {
            v[i * dim]     = u.x;
            v[i * dim + 1] = u.y;
            if (dim == 3) v[i * dim + 2] = u.z;
        }
    }
}

// Scatter a per-slot float attribute to original-id order (FP64 out).
__global__ void k_export_scalar(const float * __restrict__ a, int stride, int comp, const int * __restrict__ id,
                                long long n, double * __restrict__ out) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x)
        out[id[s]] = a[s * stride + comp];
}

// out[id] = num / a[slot * stride + comp] (a density from a stored m / rho that
// travels with the particle through every re-sort).
__global__ void k_export_ratio(const float * __restrict__ a, int stride, int comp, float num,
                               const int * __restrict__ id, long long n, double * __restrict__ out) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x)
        out[id[s]] = double(num) / double(a[s * stride + comp]);
}

// max_i |v_i|^2 over the particles, squared norms in FP64 of the FP32 components
// (ParticlesAttribute::normMax, Cores/Structures/ParticlesAttribute.h:61-67; a NaN
// component is skipped as std::max skips it there).  Non-negative doubles order
// like their bit patterns, so block maxima combine with an integer atomicMax.
__global__ void k_max_speed2(const float4 * __restrict__ vel, long long n, int dim,
                             unsigned long long * __restrict__ out) {
    double m = 0;
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x) {
        const float4 u = vel[s];
        double q = double(u.x) * u.x + double(u.y) * u.y;
        if (dim == 3) q += double(u.z) * u.z;
        m = fmax(m, q);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double wm[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) wm[w] = m;
    __syncthreads();
    if (w == 0) {
        m = lane < (int) (blockDim.x >> 5) ? wm[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) atomicMax(out, (unsigned long long) __double_as_longlong(m));
    }
}

// ---------------------------------------------------------------------------
// Counting sort into cells.  Order within a cell is made deterministic by an
// insertion sort on the original id, so the final order is (cell, id).
// ---------------------------------------------------------------------------
// With vel non-null the particles are first moved, x += v dt
// (SmthParticleHydrodLiquid::moveParticles, Cores/Physics/SmthParticleHydrodLiquid.cpp:72-76,
// DEMParticleSand::moveParticles, Cores/Physics/DEMParticleSand.cpp:98-99), fused into
// the pass that reads them anyway.  With lo non-null the position is the
// float-float pair (pos, lo) and dt = dt + dt_lo: the move is done in
// float-float arithmetic.  With Ld non-null the lattice is read from device
// memory (written by an earlier kernel of the stream); L then only sizes the
// cell arrays.
template<int DIM>
__global__ void k_cell_count(float4 * __restrict__ pos, const float4 * __restrict__ vel, float dt, long long n,
                             Lattice L, int * __restrict__ key, int * __restrict__ rank, int * __restrict__ count,
                             float4 * __restrict__ lo, float dt_lo, const Lattice * __restrict__ Ld) {
    pdl_wait_and_release();
    if (Ld) L = *Ld;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        float4 p = pos[i];
        if (vel) {
            const float4 u = vel[i];
            if (lo) {
                float4 l = lo[i];
                ff_add_product(p.x, l.x, u.x, dt, dt_lo);
                ff_add_product(p.y, l.y, u.y, dt, dt_lo);
                if (DIM == 3) ff_add_product(p.z, l.z, u.z, dt, dt_lo);
                lo[i] = l;
            } else {
                p.x = fmaf(u.x, dt, p.x);
                p.y = fmaf(u.y, dt, p.y);
                p.z = fmaf(u.z, dt, p.z);
            }
            pos[i] = p;
        }
        const int3 c   = cell_of<DIM>(L, p.x, p.y, p.z);
        const int k    = int(cell_linear(L, c));
        key[i]         = k;
        rank[i]        = atomicAdd(count + k, 1);
    }
}

__global__ void k_cell_scatter(const int * __restrict__ key, const int * __restrict__ rank,
                               const int * __restrict__ start, long long n, int * __restrict__ perm) {
    pdl_wait_and_release();
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        perm[start[key[i]] + rank[i]] = int(i);
}

__global__ void k_cell_sort_segments(const int * __restrict__ start, long long ncells, const int * __restrict__ id,
                                     int * __restrict__ perm, const Lattice * __restrict__ Ld) {
    pdl_wait_and_release();
    if (Ld) ncells = min(ncells, Ld->ncells);
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < ncells; c += (long long) gridDim.x * blockDim.x) {
        const int b = start[c], e = start[c + 1];
        if (e - b < 2) continue;
        for (int i = b + 1; i < e; i++) {
            const int pi = perm[i];
            const int ki = id[pi];
            int j        = i - 1;
            while (j >= b && id[perm[j]] > ki) {
                perm[j + 1] = perm[j];
                j--;
            }
            perm[j + 1] = pi;
        }
    }
}

__global__ void k_permute(const int * __restrict__ perm, long long n, const float4 * __restrict__ a0,
                          const float4 * __restrict__ a1, const float4 * __restrict__ a2, const int * __restrict__ i0,
                          float4 * __restrict__ b0, float4 * __restrict__ b1, float4 * __restrict__ b2,
                          int * __restrict__ j0) {
    pdl_wait_and_release();
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x) {
        const int src = perm[s];
        b0[s]         = a0[src];
        b1[s]         = a1[src];
        if (a2) b2[s] = a2[src];
        j0[s] = i0[src];
    }
}

// Sum of w (W_h = 2 c0h w) over the neighbours within h of two particles a, b,
// visited once for both (packed FP32x2 arithmetic).
template<int DIM>
__device__ __forceinline__ float2 density_sum2(const Lattice & L, const Phys & P, const int * __restrict__ cellStart,
                                               const float4 * __restrict__ pos, float4 qa, float4 qb) {
    const float2 qx = make_float2(qa.x, qb.x), qy = make_float2(qa.y, qb.y), qz = make_float2(qa.z, qb.z);
    float2 s = f2(0.f);
    for_each_in_radius2<DIM>(L, cellStart, make_float3(qa.x, qa.y, qa.z), make_float3(qb.x, qb.y, qb.z), P.h, P.h2,
                             [&](int j) {
                                 const float4 p  = pos[j];
                                 const float2 dx = add2(qx, f2(-p.x)), dy = add2(qy, f2(-p.y));
                                 float2 r2       = fma2(dy, dy, mul2(dx, dx));
                                 if (DIM == 3) {
                                     const float2 dz = add2(qz, f2(-p.z));
                                     r2              = fma2(dz, dz, r2);
                                 }
                                 const bool m0 = r2.x < P.h2, m1 = r2.y < P.h2;
                                 if (m0 || m1) s = add2(s, spline2(r2, m0, m1, P.inv_h).w);
                             });
    return s;
}

// rho_i = m sum_j W_h(x_i - x_j)  (SmoothedParticles::computeDensities,
// Cores/Structures/SmoothedParticles.cpp:25-31); writes vel.w = m / rho_i and rho_i.
// One thread per pair of consecutive sorted particles.  A pair that is not in
// one cell row is appended to left (left[0] = count, ids from left[2]) and
// visited particle by particle by k_density_left, so no warp runs both paths.
template<int DIM>
__global__ void __launch_bounds__(256) k_density(const float4 * __restrict__ pos, float4 * __restrict__ vel,
                                                 float * __restrict__ rho_out, long long n, Lattice L, Phys P,
                                                 const int * __restrict__ cellStart, float mass, int * __restrict__ left) {
    pdl_wait_and_release();
    const long long npair = (n + 1) / 2;
    const float c         = 2.f * P.c0h * mass;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < npair;
         t += (long long) gridDim.x * blockDim.x) {
        const long long ia = 2 * t, ib = ia + 1 < n ? ia + 1 : ia;
        const float4 qa = pos[ia], qb = pos[ib];
        if (!near_pair<DIM>(L, qa, qb)) {
            left[2 + atomicAdd(left, 1)] = int(t);
            continue;
        }
        const float2 s  = density_sum2<DIM>(L, P, cellStart, pos, qa, qb);
        const float ra = c * s.x, rb = c * s.y;
        if (rho_out) rho_out[ia] = ra;
        vel[ia].w = mass / ra;
        if (ib != ia) {
            if (rho_out) rho_out[ib] = rb;
            vel[ib].w = mass / rb;
        }
    }
}
template<int DIM>
__global__ void __launch_bounds__(256) k_density_left(const float4 * __restrict__ pos, float4 * __restrict__ vel,
                                                      float * __restrict__ rho_out, long long n, Lattice L, Phys P,
                                                      const int * __restrict__ cellStart, float mass, int * left) {
    pdl_wait_and_release();
    // one warp per left-over particle, its neighbour rows spread over the lanes
    const long long cnt = 2LL * left[0];
    const float c       = 2.f * P.c0h * mass;
    const int lane      = threadIdx.x & 31;
    const long long nw  = (long long) gridDim.x * (blockDim.x >> 5);
    for (long long k = (blockIdx.x * (long long) blockDim.x + threadIdx.x) >> 5; k < cnt; k += nw) {
        const long long i = 2LL * left[2 + k / 2] + (k & 1);
        if (i >= n) continue;
        const float4 q = pos[i];
        float s        = 0.f;
        for_rows_in_radius<DIM>(L, cellStart, q.x, q.y, q.z, P.h, P.h2, lane, 32, [&](int j) {
            const float4 p = pos[j];
            const float dx = q.x - p.x, dy = q.y - p.y, dz = DIM == 3 ? q.z - p.z : 0.f;
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            s += spline2(f2(r2), r2 < P.h2, false, P.inv_h).w.x;
        });
        s = warp_sum(s);
        if (lane == 0) {
            const float r = c * s;
            if (rho_out) rho_out[i] = r;
            vel[i].w = mass / r;
        }
    }
    grid_done_reset(left);
}

// V_i = m / rho_i, stored in pos.w (initialize only; DualParticleSphLiquid.cpp:88-89).
__global__ void k_set_volume(float4 * __restrict__ pos, const float * __restrict__ rho, long long n, float mass) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        pos[i].w = mass / rho[i];
}

// Viscous sums of two particles a, b over their neighbours within h (packed;
// ParticlesBasedVectorField::divFreeLaplacianAtDataPoint,
// Cores/Structures/ParticlesBasedVectorField.cpp:56-69):
// l += g s (m/rho_j) / m (x_j - x_i) with s = (v_j - v_i).(x_j - x_i) / r^2 and
// gradientKernel(x_j - x_i) = -W'(r) (x_j - x_i) / r = c1h g (x_j - x_i)
// (c1h applied by the caller); the particle itself (r = 0) adds nothing.
template<int DIM>
__device__ __forceinline__ void viscous_sum2(const Lattice & L, const Phys & P, const int * __restrict__ cellStart,
                                             const float4 * __restrict__ pos, const float4 * __restrict__ vel,
                                             float4 qa, float4 va, float4 qb, float4 vb, float2 & lx, float2 & ly,
                                             float2 & lz) {
    const float2 qx = make_float2(qa.x, qb.x), qy = make_float2(qa.y, qb.y), qz = make_float2(qa.z, qb.z);
    const float2 vx = make_float2(va.x, vb.x), vy = make_float2(va.y, vb.y), vz = make_float2(va.z, vb.z);
    for_each_in_radius2<DIM>(
        L, cellStart, make_float3(qa.x, qa.y, qa.z), make_float3(qb.x, qb.y, qb.z), P.h, P.h2, [&](int j) {
            const float4 p = pos[j];
            // x_j - x_i and v_j - v_i
            const float2 dx = fma2(qx, f2(-1.f), f2(p.x)), dy = fma2(qy, f2(-1.f), f2(p.y));
            const float2 dz = DIM == 3 ? fma2(qz, f2(-1.f), f2(p.z)) : f2(0.f);
            float2 r2       = fma2(dy, dy, mul2(dx, dx));
            if (DIM == 3) r2 = fma2(dz, dz, r2);
            const bool m0 = r2.x < P.h2 && r2.x > 0.f, m1 = r2.y < P.h2 && r2.y > 0.f;
            if (!(m0 || m1)) return;
            const float4 vj = vel[j];
            float2 dot = fma2(fma2(vy, f2(-1.f), f2(vj.y)), dy, mul2(fma2(vx, f2(-1.f), f2(vj.x)), dx));
            if (DIM == 3) dot = fma2(fma2(vz, f2(-1.f), f2(vj.z)), dz, dot);
            const Spline2 k = spline2(r2, m0, m1, P.inv_h);
            const float2 gs = mul2(mul2(k.g, mul2(dot, mul2(k.ri, k.ri))), f2(vj.w * P.inv_mass));
            lx              = fma2(gs, dx, lx);
            ly              = fma2(gs, dy, ly);
            if (DIM == 3) lz = fma2(gs, dz, lz);
        });
}

// Gravity (applyExternalForces, SmthParticleHydrodLiquid.cpp:84-88) followed by
// the div-free Laplacian viscosity (applyViscosityForce :90-98).  Velocity
// differences are invariant under the uniform gravity increment, so both run
// in one pass; one thread per pair of consecutive sorted particles as in
// k_density.
__device__ __forceinline__ float4 forces_out(float4 v, float gx, float gy, float gz, float visc, float lx, float ly,
                                             float lz, bool d3) {
    v.x += gx;
    v.y += gy;
    v.z += gz;
    v.x += visc * lx;
    v.y += visc * ly;
    if (d3) v.z += visc * lz;
    return v;
}

template<int DIM>
__global__ void __launch_bounds__(256) k_forces(const float4 * __restrict__ pos, const float4 * __restrict__ vel,
                                                float4 * __restrict__ vel_out, long long n, Lattice L, Phys P,
                                                const int * __restrict__ cellStart, float dt, int * __restrict__ left) {
    pdl_wait_and_release();
    const float visc      = P.viscosity * 2.f * (DIM + 2.f) * P.mass * dt * P.c1h;
    const float gx = P.gravity_on ? P.gx * dt : 0.f, gy = P.gravity_on ? P.gy * dt : 0.f;
    const float gz = P.gravity_on && DIM == 3 ? P.gz * dt : 0.f;
    const long long npair = (n + 1) / 2;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < npair;
         t += (long long) gridDim.x * blockDim.x) {
        const long long ia = 2 * t, ib = ia + 1 < n ? ia + 1 : ia;
        const float4 qa = pos[ia], qb = pos[ib], va = vel[ia], vb = vel[ib];
        float2 lx = f2(0.f), ly = f2(0.f), lz = f2(0.f);
        if (P.viscosity != 0.f) {
            if (!near_pair<DIM>(L, qa, qb)) {
                left[2 + atomicAdd(left, 1)] = int(t);
                continue;
            }
            viscous_sum2<DIM>(L, P, cellStart, pos, vel, qa, va, qb, vb, lx, ly, lz);
        }
        vel_out[ia] = forces_out(va, gx, gy, gz, visc, lx.x, ly.x, lz.x, DIM == 3);
        if (ib != ia) vel_out[ib] = forces_out(vb, gx, gy, gz, visc, lx.y, ly.y, lz.y, DIM == 3);
    }
}
template<int DIM>
__global__ void __launch_bounds__(256) k_forces_left(const float4 * __restrict__ pos, const float4 * __restrict__ vel,
                                                     float4 * __restrict__ vel_out, long long n, Lattice L, Phys P,
                                                     const int * __restrict__ cellStart, float dt, int * left) {
    pdl_wait_and_release();
    const float visc = P.viscosity * 2.f * (DIM + 2.f) * P.mass * dt * P.c1h;
    const float gx = P.gravity_on ? P.gx * dt : 0.f, gy = P.gravity_on ? P.gy * dt : 0.f;
    const float gz = P.gravity_on && DIM == 3 ? P.gz * dt : 0.f;
    // one warp per left-over particle, its neighbour rows spread over the lanes
    const long long cnt = 2LL * left[0];
    const int lane      = threadIdx.x & 31;
    const long long nw  = (long long) gridDim.x * (blockDim.x >> 5);
    for (long long k = (blockIdx.x * (long long) blockDim.x + threadIdx.x) >> 5; k < cnt; k += nw) {
        const long long i = 2LL * left[2 + k / 2] + (k & 1);
        if (i >= n) continue;
        const float4 q = pos[i], v = vel[i];
        float lx = 0.f, ly = 0.f, lz = 0.f;
        if (P.viscosity != 0.f) {
            for_rows_in_radius<DIM>(L, cellStart, q.x, q.y, q.z, P.h, P.h2, lane, 32, [&](int j) {
                const float4 p = pos[j], vj = vel[j];
                const float dx = p.x - q.x, dy = p.y - q.y, dz = DIM == 3 ? p.z - q.z : 0.f;  // x_j - x_i
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float dot = fmaf(vj.z - v.z, dz, fmaf(vj.y - v.y, dy, (vj.x - v.x) * dx));
                const Spline2 k2 = spline2(f2(r2), r2 < P.h2 && r2 > 0.f, false, P.inv_h);
                const float gs   = k2.g.x * (dot * (k2.ri.x * k2.ri.x)) * (vj.w * P.inv_mass);
                lx = fmaf(gs, dx, lx);
                ly = fmaf(gs, dy, ly);
                lz = fmaf(gs, dz, lz);
            });
            lx = warp_sum(lx);
            ly = warp_sum(ly);
            lz = warp_sum(lz);
        }
        if (lane == 0) vel_out[i] = forces_out(v, gx, gy, gz, visc, lx, ly, lz, DIM == 3);
    }
    grid_done_reset(left);
}

// Boundary densities from boundary-boundary neighbours (initialize,
// DualParticleSphLiquid.cpp:93-94): rho_b = m_b sum W_h, V_b = m_b / rho_b.
template<int DIM>
__global__ void __launch_bounds__(256) k_boundary_density(float4 * __restrict__ bpos, float4 * __restrict__ bvel,
                                                          float * __restrict__ rho_out, long long nb, Lattice L,
                                                          Phys P, const int * __restrict__ bcellStart) {
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < nb; i += (long long) gridDim.x * blockDim.x) {
        const float4 q = bpos[i];
        float s        = 0.f;
        for_each_in_radius<DIM>(L, bcellStart, q.x, q.y, q.z, P.h, P.h2, [&](int j) {
            const float4 p = bpos[j];
            const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < P.h2) s += kW(r2 * rsqrt_n(fmaxf(r2, 1e-30f)), P.inv_h, P.c0h);
        });
        const float rho = P.bmass * s;
        if (rho_out) rho_out[i] = rho;
        bpos[i].w = P.bmass / rho;
        bvel[i].w = P.bmass / rho;
    }
}

// Bricks holding a node within reach of a particle (bflag: only nodes within h of
// a real particle can have a positive weight, VirtualParticle.cpp:50-56) and
// bricks holding a particle's own cell (pflag: the bricks the brick-tiled
// particle kernels visit), from the sorted cell ranges.  A particle in cell c
// reaches nodes c - ceil(h/dx) .. c + ceil(h/dx) along each axis; `reach` adds one
// for FP32 rounding, so a brick is flagged when a particle lies in its cells
// dilated by `reach` (particles outside the lattice sit in the border cells, so
// the dilation still covers the nodes they reach).  One warp per brick, lanes
// over the dilated cell rows; every brick's flag is written.
template<int DIM>
__global__ void __launch_bounds__(256) k_mark_bricks(Lattice L, const int * __restrict__ cellStart, int reach,
                                                     unsigned char * __restrict__ bflag,
                                                     unsigned char * __restrict__ pflag) {
    pdl_wait_and_release();
    using G               = BrickGeom<DIM>;
    const int lane        = threadIdx.x & 31;
    const long long warp  = (blockIdx.x * (long long) blockDim.x + threadIdx.x) >> 5;
    const long long warps = (gridDim.x * (long long) blockDim.x) >> 5;
    for (long long b = warp; b < L.nbricks; b += warps) {
        const int bx = int(b % L.bnx), by = int((b / L.bnx) % L.bny), bz = int(b / ((long long) L.bnx * L.bny));
        const int ox0 = bx * G::BX, ox1 = min(ox0 + G::BX - 1, L.nx - 1);
        const int oy0 = by * G::BY, oy1 = min(oy0 + G::BY - 1, L.ny - 1);
        const int oz0 = DIM == 3 ? bz * G::BZ : 0, oz1 = DIM == 3 ? min(oz0 + G::BZ - 1, L.nz - 1) : 0;
        const int x0 = max(ox0 - reach, 0), x1 = min(ox1 + reach, L.nx - 1);
        const int y0 = max(oy0 - reach, 0), y1 = min(oy1 + reach, L.ny - 1);
        const int z0 = DIM == 3 ? max(oz0 - reach, 0) : 0, z1 = DIM == 3 ? min(oz1 + reach, L.nz - 1) : 0;
        const int nyr = y1 - y0 + 1, rows = nyr * (z1 - z0 + 1);
        bool any = false, own = false;
        for (int r = lane; r < rows; r += 32) {
            const int y = y0 + r % nyr, z = z0 + r / nyr;
            const long long row = (long long) L.nx * (y + (long long) L.ny * z);
            any = any || cellStart[row + x1 + 1] > cellStart[row + x0];
            if (pflag && y >= oy0 && y <= oy1 && z >= oz0 && z <= oz1)
                own = own || cellStart[row + ox1 + 1] > cellStart[row + ox0];
        }
        any = __any_sync(0xffffffffu, any);
        own = __any_sync(0xffffffffu, own);
        if (lane == 0) {
            bflag[b] = any ? 1 : 0;
            if (pflag) pflag[b] = own ? 1 : 0;
        }
    }
}

// Cells within reach of the boundary: near[c] = 1 when some boundary particle is
// binned within R cells of cell c along every axis (a box dilation of the
// boundary's occupancy, done axis by axis).  The x pass reads the occupancy of
// the whole x-range from the row's prefix sums; the y / z passes OR R cells on
// either side.  With R = ceil(h / dx) + 1 a particle (or node) whose cell is not
// flagged has no boundary particle within h.
template<int DIM>
__global__ void __launch_bounds__(256) k_near_x(Lattice L, const int * __restrict__ cellStart, int R,
                                                unsigned char * __restrict__ out) {
    pdl_wait_and_release();
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < L.ncells;
         c += (long long) gridDim.x * blockDim.x) {
        const int x = int(c % L.nx);
        const long long row = c - x;
        out[c] = cellStart[row + min(x + R, L.nx - 1) + 1] > cellStart[row + max(x - R, 0)] ? 1 : 0;
    }
}
__global__ void __launch_bounds__(256) k_near_dilate(long long ncells, long long stride, int extent, int R,
                                                     const unsigned char * __restrict__ in,
                                                     unsigned char * __restrict__ out) {
    pdl_wait_and_release();
    for (long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x; c < ncells;
         c += (long long) gridDim.x * blockDim.x) {
        const int k = int((c / stride) % extent);
        unsigned char v = 0;
        for (int d = max(-R, -k); d <= min(R, extent - 1 - k); d++) v |= in[c + d * stride];
        out[c] = v;
    }
}

// Rigid motion of boundary particles flagged as moving (paddle): rotation about
// the y axis through c with angular velocity omega; v_b = omega x (x - c).
// The moving flag travels with the particle in bnrm.w (1 = moving).
__global__ void k_rotate_boundary(float4 * __restrict__ bpos, float4 * __restrict__ bvel, float4 * __restrict__ bnrm,
                                  long long nb, float cx, float cz, float omega, float dt) {
    const float ca = cosf(omega * dt), sa = sinf(omega * dt);
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < nb; i += (long long) gridDim.x * blockDim.x) {
        float4 p = bpos[i], v = bvel[i], nn = bnrm[i];
        if (nn.w == 0.f) continue;
        // rotation by -omega dt about +y (x' = x cos + z sin, z' = -x sin + z cos)
        const float rx = p.x - cx, rz = p.z - cz;
        const float nx = rx * ca + rz * sa, nz = -rx * sa + rz * ca;
        p.x = cx + nx;
        p.z = cz + nz;
        const float mx = nn.x * ca + nn.z * sa, mz = -nn.x * sa + nn.z * ca;
        nn.x = mx;
        nn.z = mz;
        v.x = omega * nz;
        v.z = -omega * nx;
        bpos[i] = p;
        bvel[i] = v;
        bnrm[i] = nn;
    }
}

// pos.w = vol_by_id[id[s]] (V_i travels with the particle id).
__global__ void k_fill_w_by_id(float4 * __restrict__ pos, const float * __restrict__ vol, const int * __restrict__ id,
                               long long n) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x)
        pos[s].w = vol[id ? id[s] : s];
}
// vol_by_id[id[s]] = pos[s].w
__global__ void k_scatter_w_to_id(const float4 * __restrict__ pos, const int * __restrict__ id, long long n,
                                  float * __restrict__ vol) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < n; s += (long long) gridDim.x * blockDim.x)
        vol[id[s]] = pos[s].w;
}
// Boundary rho_b / V_b given by original id (replay of another run's initialize).
__global__ void k_set_boundary_info(float4 * __restrict__ bpos, float4 * __restrict__ bvel, float * __restrict__ brho,
                                    const float * __restrict__ rho, const float * __restrict__ vol,
                                    const int * __restrict__ bid, long long nb, float bmass) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < nb; s += (long long) gridDim.x * blockDim.x) {
        const int i = bid[s];
        brho[s]     = rho[i];
        bpos[s].w   = vol[i];
        bvel[s].w   = bmass / rho[i];
    }
}
// bnrm.w = moving[bid[s]]
__global__ void k_set_moving(float4 * __restrict__ bnrm, const unsigned char * __restrict__ moving,
                             const int * __restrict__ bid, long long nb) {
    for (long long s = blockIdx.x * (long long) blockDim.x + threadIdx.x; s < nb; s += (long long) gridDim.x * blockDim.x)
        bnrm[s].w = moving[bid[s]] ? 1.f : 0.f;
}


// Neighbour ids of arbitrary query points with the product's cell search
// (parity checks): FP32 distances, FP64 re-test within 1e-5 h^2 of the support
// edge so the strict |d|^2 < R^2 test matches an FP64 evaluation.
// which: 0 real (original ids), 1 boundary (original ids), 2 active virtual
// nodes within H (node ids).  ids == nullptr: counts only.
template<int DIM>
__global__ void k_debug_neighbors(int which, long long nq, const double * __restrict__ q, Lattice L, Phys P,
                                  const float4 * __restrict__ pos, const int * __restrict__ id,
                                  const int * __restrict__ cellStart, const unsigned char * __restrict__ bflag,
                                  const unsigned char * __restrict__ nflag, long long * __restrict__ counts,
                                  const long long * __restrict__ offsets, long long * __restrict__ ids) {
    using G = BrickGeom<DIM>;
    for (long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x; t < nq; t += (long long) gridDim.x * blockDim.x) {
        const double qx = q[t * DIM], qy = q[t * DIM + 1], qz = DIM == 3 ? q[t * DIM + 2] : 0.0;
        const float fx = float(qx), fy = float(qy), fz = float(qz);
        long long c = 0;
        const long long o = offsets ? offsets[t] : 0;
        auto accept = [&](float px, float py, float pz, double R2d, float R2f) {
            const float dx = fx - px, dy = fy - py, dz = fz - pz;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (fabsf(r2 - R2f) > 1e-5f * R2f) return r2 < R2f;
            const double ex = qx - double(px), ey = qy - double(py), ez = DIM == 3 ? qz - double(pz) : 0.0;
            return ex * ex + ey * ey + ez * ez < R2d;
        };
        if (which < 2) {
            const double R2d = P.h_d * P.h_d;
            for_each_in_radius<DIM>(L, cellStart, fx, fy, fz, P.h * 1.0001f, P.h2 * 1.0002f, [&](int j) {
                const float4 p = pos[j];
                if (accept(p.x, p.y, p.z, R2d, P.h2)) {
                    if (ids) ids[o + c] = id[j];
                    c++;
                }
            });
        } else {
            const double Hd = 4.0 * L.dx_d, R2d = Hd * Hd;
            const float Hn = P.H * L.inv_dx * 1.0001f;
            const float ux = (fx - L.ox) * L.inv_dx, uy = (fy - L.oy) * L.inv_dx, uz = (fz - L.oz) * L.inv_dx;
            const int x0 = max(__float2int_rd(ux - Hn), 0), x1 = min(__float2int_ru(ux + Hn), L.nx - 1);
            const int y0 = max(__float2int_rd(uy - Hn), 0), y1 = min(__float2int_ru(uy + Hn), L.ny - 1);
            int z0 = 0, z1 = 0;
            if (DIM == 3) z0 = max(__float2int_rd(uz - Hn), 0), z1 = min(__float2int_ru(uz + Hn), L.nz - 1);
            for (int kz = z0; kz <= z1; kz++)
                for (int ky = y0; ky <= y1; ky++)
                    for (int kx = x0; kx <= x1; kx++) {
                        const int brick = kx / G::BX + L.bnx * (ky / G::BY + L.bny * (DIM == 3 ? kz / G::BZ : 0));
                        if (!bflag[brick] || !nflag[node_slot<DIM>(L, kx, ky, kz)]) continue;
                        // FP64 node position, as the reference computes it
                        const double nx = L.ox_d + kx * L.dx_d, ny = L.oy_d + ky * L.dx_d,
                                     nz = DIM == 3 ? L.oz_d + kz * L.dx_d : 0.0;
                        const double ex = qx - nx, ey = qy - ny, ez = qz - nz;
                        if (ex * ex + ey * ey + ez * ez < R2d) {
                            if (ids) ids[o + c] = (long long) kx + (long long) L.nx * (ky + (long long) L.ny * kz);
                            c++;
                        }
                    }
        }
        counts[t] = c;
    }
}

// Max over a positive float array (ordered as int bits).
__global__ void k_max_positive(const float * __restrict__ a, long long n, int * __restrict__ out_bits) {
    int m = 0;
    for (long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        m = max(m, __float_as_int(a[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out_bits, m);
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32 counts (three phases: tile sums, scan of tile sums,
// tile scan + offset).  out has n + 1 entries; out[n] = total.  With Ld (a
// lattice in device memory) only its first Ld->ncells <= n counts are scanned.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int * __restrict__ in, long long n,
                                                              int * __restrict__ tile_sum, const Lattice * __restrict__ Ld) {
    pdl_wait_and_release();
    if (Ld) n = min(n, Ld->ncells);
    __shared__ int sm[kScanThreads / 32];
    const long long base = (long long) blockIdx.x * kScanTile;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const long long i = base + threadIdx.x + (long long) k * kScanThreads;
        if (i < n) s += in[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += sm[w];
        tile_sum[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) k_scan_top(int * __restrict__ tile_sum, int ntiles) {
    pdl_wait_and_release();
    __shared__ int sm[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < ntiles ? tile_sum[i] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) sm[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int w = sm[threadIdx.x];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            sm[threadIdx.x] = w;
        }
        __syncthreads();
        const int warp_off = (threadIdx.x >> 5) ? sm[(threadIdx.x >> 5) - 1] : 0;
        const int incl     = x + warp_off + carry;
        if (i < ntiles) tile_sum[i] = incl - v;  // exclusive
        __syncthreads();
        if (threadIdx.x == 1023) carry = incl;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int * __restrict__ in, long long n,
                                                              const int * __restrict__ tile_off, int * __restrict__ out,
                                                              const Lattice * __restrict__ Ld) {
    pdl_wait_and_release();
    if (Ld) {
        n = min(n, Ld->ncells);
        if ((long long) blockIdx.x * kScanTile > n) return;  // past the lattice's cells (and past out[n])
    }
    __shared__ int sm[kScanThreads / 32];
    const long long base = (long long) blockIdx.x * kScanTile + (long long) threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const long long i = base + k;
        v[k]              = i < n ? in[i] : 0;
        s += v[k];
    }
    int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) sm[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = threadIdx.x < kScanThreads / 32 ? sm[threadIdx.x] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (threadIdx.x >= o) w += y;
        }
        if (threadIdx.x < kScanThreads / 32) sm[threadIdx.x] = w;
    }
    __syncthreads();
    int run = tile_off[blockIdx.x] + x - s + ((threadIdx.x >> 5) ? sm[(threadIdx.x >> 5) - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
        if (i == n - 1) out[n] = run;
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
constexpr int kLeftBlocks = 256;  // grid of the single-particle passes over left-over pairs (grid-stride)
static inline int grid_for(long long n, int threads, int cap = 152 * 16) {
    long long g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return int(g);
}

void launch_import(const double * x, const double * v, int dim, long long n, float4 * pos, float4 * vel, int * id,
                   cudaStream_t st) {
    if (n > 0) k_import<<<grid_for(n, 256), 256, 0, st>>>(x, v, dim, n, pos, vel, id);
}
void launch_export(const float4 * pos, const float4 * vel, const int * id, int dim, long long n, double * x,
                   double * v, cudaStream_t st) {
    if (n > 0) k_export<<<grid_for(n, 256), 256, 0, st>>>(pos, vel, id, dim, n, x, v);
}
void launch_max_speed2(const float4 * vel, long long n, int dim, unsigned long long * out, cudaStream_t st) {
    if (n > 0) k_max_speed2<<<grid_for(n, 256), 256, 0, st>>>(vel, n, dim, out);
}
void launch_export_scalar(const float * a, int stride, int comp, const int * id, long long n, double * out,
                          cudaStream_t st) {
    if (n > 0) k_export_scalar<<<grid_for(n, 256), 256, 0, st>>>(a, stride, comp, id, n, out);
}
void launch_export_ratio(const float * a, int stride, int comp, float num, const int * id, long long n, double * out,
                         cudaStream_t st) {
    if (n > 0) k_export_ratio<<<grid_for(n, 256), 256, 0, st>>>(a, stride, comp, num, id, n, out);
}

void launch_scan(const int * in, long long n, int * out, int * tile_buf, cudaStream_t st, const Lattice * Ld) {
    const long long ntiles = (n + kScanTile - 1) / kScanTile;
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int), st);
        return;
    }
    launch_pdl(k_scan_tiles, int(ntiles), kScanThreads, 0, st, in, n, tile_buf, Ld);
    launch_pdl(k_scan_top, 1, 1024, 0, st, tile_buf, int(ntiles));
    launch_pdl(k_scan_apply, int(ntiles), kScanThreads, 0, st, in, n, (const int *) tile_buf, out, Ld);
}
long long scan_tile_count(long long n) { return (n + kScanTile - 1) / kScanTile + 1; }

template<int DIM>
void launch_bin(const Lattice & L, long long n, float4 *& pos, float4 *& vel, float4 *& aux, int *& id,
                SortScratch & S, int * cellStart, float advect_dt, cudaStream_t st, float advect_dt_lo, bool aux_lo,
                const Lattice * Ld) {
    cudaMemsetAsync(S.count, 0, sizeof(int) * L.ncells, st);
    if (n > 0)
        launch_pdl(k_cell_count<DIM>, grid_for(n, 256), 256, 0, st, pos, advect_dt != 0.f ? vel : nullptr, advect_dt, n, L,
                   S.key, S.rank, S.count, aux_lo ? aux : nullptr, advect_dt_lo, Ld);
    launch_scan(S.count, L.ncells, cellStart, S.tiles, st, Ld);
    if (n == 0) return;
    launch_pdl(k_cell_scatter, grid_for(n, 256), 256, 0, st, S.key, S.rank, cellStart, n, S.perm);
    launch_pdl(k_cell_sort_segments, grid_for(L.ncells, 256), 256, 0, st, (const int *) cellStart, L.ncells,
               (const int *) id, S.perm, Ld);
    launch_pdl(k_permute, grid_for(n, 256), 256, 0, st, S.perm, n, pos, vel, aux, id, S.pos2, S.vel2, S.aux2, S.id2);
    // the sorted arrays become the state; the previous ones the next sort's targets
    std::swap(pos, S.pos2);
    std::swap(vel, S.vel2);
    if (aux) std::swap(aux, S.aux2);
    std::swap(id, S.id2);
}

template<int DIM>
void launch_density(const float4 * pos, float4 * vel, float * rho, long long n, const Lattice & L, const Phys & P,
                    const int * cellStart, int * left, cudaStream_t st) {
    if (n <= 0) return;
    launch_pdl(k_density<DIM>, grid_for((n + 1) / 2, 256, 1 << 20), 256, 0, st, pos, vel, rho, n, L, P, cellStart, P.mass,
                                                                         left);
    launch_pdl(k_density_left<DIM>, kLeftBlocks, 256, 0, st, pos, vel, rho, n, L, P, cellStart, P.mass, left);
}
void launch_set_volume(float4 * pos, const float * rho, long long n, float mass, cudaStream_t st) {
    if (n > 0) k_set_volume<<<grid_for(n, 256), 256, 0, st>>>(pos, rho, n, mass);
}
template<int DIM>
void launch_forces(const float4 * pos, const float4 * vel, float4 * vel_out, long long n, const Lattice & L,
                   const Phys & P, const int * cellStart, float dt, int * left, cudaStream_t st) {
    if (n <= 0) return;
    launch_pdl(k_forces<DIM>, grid_for((n + 1) / 2, 256, 1 << 20), 256, 0, st, pos, vel, vel_out, n, L, P, cellStart, dt,
                                                                       left);
    launch_pdl(k_forces_left<DIM>, kLeftBlocks, 256, 0, st, pos, vel, vel_out, n, L, P, cellStart, dt, left);
}
template<int DIM>
void launch_boundary_density(float4 * bpos, float4 * bvel, float * rho, long long nb, const Lattice & L,
                             const Phys & P, const int * bcellStart, cudaStream_t st) {
    if (nb > 0)
        k_boundary_density<DIM><<<grid_for(nb, 256, 1 << 20), 256, 0, st>>>(bpos, bvel, rho, nb, L, P, bcellStart);
}
template<int DIM>
void launch_mark_bricks(const int * cellStart, long long n, const Lattice & L, const Phys & P, unsigned char * bflag,
                        unsigned char * pflag, cudaStream_t st) {
    if (n <= 0 || L.nbricks <= 0) {
        cudaMemsetAsync(bflag, 0, L.nbricks, st);
        if (pflag) cudaMemsetAsync(pflag, 0, L.nbricks, st);
        return;
    }
    const int reach   = int(std::ceil(double(P.h) / double(L.dx))) + 1;
    const long long b = (L.nbricks + 7) / 8;  // eight warps per block, one warp per brick
    launch_pdl(k_mark_bricks<DIM>, int(std::min<long long>(b, 152LL * 64)), 256, 0, st, L, cellStart, reach, bflag, pflag);
}
template<int DIM>
void launch_near_cells(const int * cellStart, long long n, const Lattice & L, const Phys & P, unsigned char * near,
                       unsigned char * tmp, cudaStream_t st) {
    if (n <= 0 || L.ncells <= 0) {
        cudaMemsetAsync(near, 0, size_t(L.ncells), st);
        return;
    }
    const int R = int(std::ceil(double(P.h) / double(L.dx))) + 1;
    const int g = int(std::min<long long>((L.ncells + 255) / 256, 152LL * 16));
    // 3D: x -> near, y: near -> tmp, z: tmp -> near; 2D: x -> tmp, y: tmp -> near
    unsigned char * xo = DIM == 3 ? near : tmp;
    launch_pdl(k_near_x<DIM>, g, 256, 0, st, L, cellStart, R, xo);
    launch_pdl(k_near_dilate, g, 256, 0, st, L.ncells, (long long) L.nx, L.ny, R, (const unsigned char *) xo,
               DIM == 3 ? tmp : near);
    if (DIM == 3)
        launch_pdl(k_near_dilate, g, 256, 0, st, L.ncells, (long long) L.nx * L.ny, L.nz, R, (const unsigned char *) tmp,
                   near);
}
void launch_rotate_boundary(float4 * bpos, float4 * bvel, float4 * bnrm, long long nb, float cx, float cz,
                            float omega, float dt, cudaStream_t st) {
    if (nb > 0) k_rotate_boundary<<<grid_for(nb, 256), 256, 0, st>>>(bpos, bvel, bnrm, nb, cx, cz, omega, dt);
}
void launch_fill_w_by_id(float4 * pos, const float * vol, const int * id, long long n, cudaStream_t st) {
    if (n > 0) k_fill_w_by_id<<<grid_for(n, 256), 256, 0, st>>>(pos, vol, id, n);
}
void launch_scatter_w_to_id(const float4 * pos, const int * id, long long n, float * vol, cudaStream_t st) {
    if (n > 0) k_scatter_w_to_id<<<grid_for(n, 256), 256, 0, st>>>(pos, id, n, vol);
}
void launch_set_boundary_info(float4 * bpos, float4 * bvel, float * brho, const float * rho, const float * vol,
                              const int * bid, long long nb, float bmass, cudaStream_t st) {
    if (nb > 0) k_set_boundary_info<<<grid_for(nb, 256), 256, 0, st>>>(bpos, bvel, brho, rho, vol, bid, nb, bmass);
}
void launch_set_moving(float4 * bnrm, const unsigned char * moving, const int * bid, long long nb, cudaStream_t st) {
    if (nb > 0) k_set_moving<<<grid_for(nb, 256), 256, 0, st>>>(bnrm, moving, bid, nb);
}
void launch_max_positive(const float * a, long long n, int * out_bits, cudaStream_t st) {
    cudaMemsetAsync(out_bits, 0, sizeof(int), st);
    if (n > 0) k_max_positive<<<grid_for(n, 256), 256, 0, st>>>(a, n, out_bits);
}


template<int DIM>
void launch_debug_neighbors(int which, long long nq, const double * q, const Lattice & L, const Phys & P,
                            const float4 * pos, const int * id, const int * cellStart, const unsigned char * bflag,
                            const unsigned char * nflag, long long * counts, const long long * offsets, long long * ids,
                            cudaStream_t st) {
    if (nq > 0)
        k_debug_neighbors<DIM><<<grid_for(nq, 128), 128, 0, st>>>(which, nq, q, L, P, pos, id, cellStart, bflag, nflag,
                                                                   counts, offsets, ids);
}

#define SWC_INST(D)                                                                                                    \
    template void launch_bin<D>(const Lattice &, long long, float4 *&, float4 *&, float4 *&, int *&, SortScratch &,   \
                                int *, float, cudaStream_t, float, bool, const Lattice *);                             \
    template void launch_density<D>(const float4 *, float4 *, float *, long long, const Lattice &, const Phys &,       \
                                    const int *, int *, cudaStream_t);                                                 \
    template void launch_forces<D>(const float4 *, const float4 *, float4 *, long long, const Lattice &, const Phys &,  \
                                   const int *, float, int *, cudaStream_t);                                           \
    template void launch_boundary_density<D>(float4 *, float4 *, float *, long long, const Lattice &, const Phys &,    \
                                             const int *, cudaStream_t);                                               \
    template void launch_near_cells<D>(const int *, long long, const Lattice &, const Phys &, unsigned char *,         \
                                       unsigned char *, cudaStream_t);                                                 \
    template void launch_mark_bricks<D>(const int *, long long, const Lattice &, const Phys &, unsigned char *,        \
                                        unsigned char *,                                                               \
                                        cudaStream_t);                                                                 \
    template void launch_debug_neighbors<D>(int, long long, const double *, const Lattice &, const Phys &,            \
                                            const float4 *, const int *, const int *, const unsigned char *,           \
                                            const unsigned char *, long long *, const long long *, long long *,        \
                                            cudaStream_t);
SWC_INST(2)
SWC_INST(3)
#undef SWC_INST

}  // namespace swc
