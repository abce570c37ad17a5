// swc_tiles.cuh -- brick/tile helpers shared by the node-lattice kernels:
// brick coordinates, reference-order compact index, halo tile loading (scalar
// and 16-byte vectorised) and the radial virtual-Laplacian stencil.
#pragma once

#include "swc_kernels.h"

namespace swc {

constexpr int kNT = 256;  // threads per block of the brick kernels

// Brick coordinates of brick id b.
__device__ __forceinline__ int3 brick_coords(const Lattice & L, int b) {
    return make_int3(b % L.bnx, (b / L.bnx) % L.bny, b / (L.bnx * L.bny));
}

template<int DIM>
__device__ __forceinline__ long long compact_index(const Lattice & L, const int * __restrict__ seg_off,
                                                   const unsigned char * __restrict__ flag, int b, int bx, int x,
                                                   int y, int z, int l) {
    using G       = BrickGeom<DIM>;
    const int lx  = l % G::BX;
    long long I   = seg_off[((long long) z * L.ny + y) * L.bnx + bx];
    const unsigned char * f = flag + (long long) b * G::BN + (l - lx);
    for (int k = 0; k < lx; k++) I += f[k];
    return I;
}

// ---------------------------------------------------------------------------
// Halo tile loading and the radial stencil.
// ---------------------------------------------------------------------------
template<int DIM, class Get>
__device__ __forceinline__ void load_tile(const Lattice & L, const unsigned char * __restrict__ bflag, int3 bc,
                                          float * tile, Get get) {
    using G       = BrickGeom<DIM>;
    constexpr int NT = G::TX * G::TY * G::TZ;
    for (int t = threadIdx.x; t < NT; t += kNT) {
        const int tx = t % G::TX, ty = (t / G::TX) % G::TY, tz = t / (G::TX * G::TY);
        const int x = bc.x * G::BX + tx - G::HALO, y = bc.y * G::BY + ty - G::HALO;
        const int z = DIM == 3 ? bc.z * G::BZ + tz - G::HALO : 0;
        float v = 0.f;
        if (x >= 0 && x < L.nx && y >= 0 && y < L.ny && (DIM == 2 || (z >= 0 && z < L.nz))) {
            const int nbx = x / G::BX, nby = y / G::BY, nbz = DIM == 3 ? z / G::BZ : 0;
            const int nbk = nbx + L.bnx * (nby + L.bny * nbz);
            if (bflag[nbk])
                v = get((long long) nbk * G::BN + (x - nbx * G::BX) + G::BX * ((y - nby * G::BY) + G::BY * (z - nbz * G::BZ)));
        }
        tile[tx + G::PX * (ty + G::TY * tz)] = v;
    }
}

template<int DIM> __device__ __forceinline__ int tile_center(int l) {
    using G      = BrickGeom<DIM>;
    const int lx = l % G::BX, ly = (l / G::BX) % G::BY, lz = l / (G::BX * G::BY);
    return (lx + G::HALO) + G::PX * ((ly + G::HALO) + G::TY * (DIM == 3 ? lz + G::HALO : 0));
}

// sum over offsets 0 < |k|^2 < 16 of c(|k|^2) * tile[center + k]
template<int DIM> __device__ __forceinline__ float stencil_apply(const float * tile, int c, const Stencil & S) {
    using G   = BrickGeom<DIM>;
    float acc = 0.f;
    constexpr int ZR = DIM == 3 ? 3 : 0;
#pragma unroll
    for (int dz = -ZR; dz <= ZR; dz++)
#pragma unroll
        for (int dy = -3; dy <= 3; dy++)
#pragma unroll
            for (int dx = -3; dx <= 3; dx++) {
                const int r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > 0 && r2 < 16) acc = fmaf(S.c[r2], tile[c + dx + G::PX * (dy + G::TY * dz)], acc);
            }
    return acc;
}
template<int DIM> __device__ __forceinline__ double stencil_apply_d(const float * tile, int c, const StencilD & S) {
    using G    = BrickGeom<DIM>;
    double acc = 0.0;
    constexpr int ZR = DIM == 3 ? 3 : 0;
#pragma unroll
    for (int dz = -ZR; dz <= ZR; dz++)
#pragma unroll
        for (int dy = -3; dy <= 3; dy++)
#pragma unroll
            for (int dx = -3; dx <= 3; dx++) {
                const int r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > 0 && r2 < 16) acc += S.c[r2] * double(tile[c + dx + G::PX * (dy + G::TY * dz)]);
            }
    return acc;
}

// Threads of the row-stencil kernels: one thread per x-row of a brick.
template<int DIM> struct RowGeom {
    static constexpr int NT = BrickGeom<DIM>::BY * BrickGeom<DIM>::BZ;  // 64 (3D) or 16 (2D)
};

// Halo tile with 16-byte loads: the tile is read as 4-node x-segments, each of
// which lies inside one brick and is 16-byte aligned in the brick layout.
// get4(slot) returns the 4 values starting at `slot`; nodes outside the lattice
// or in inactive bricks read as zero.
template<int DIM, class Get4>
__device__ __forceinline__ void load_tile4(const Lattice & L, const unsigned char * __restrict__ bflag, int3 bc,
                                           float * tile, Get4 get4) {
    using G            = BrickGeom<DIM>;
    constexpr int SEGX = G::TX / 4;
    constexpr int NSEG = SEGX * G::TY * G::TZ;
    constexpr int NT   = RowGeom<DIM>::NT;
#pragma unroll 4
    for (int t = threadIdx.x; t < NSEG; t += NT) {
        const int sx = t % SEGX, ty = (t / SEGX) % G::TY, tz = t / (SEGX * G::TY);
        const int x = bc.x * G::BX - G::HALO + 4 * sx, y = bc.y * G::BY + ty - G::HALO;
        const int z = DIM == 3 ? bc.z * G::BZ + tz - G::HALO : 0;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (x >= 0 && x < L.nx && y >= 0 && y < L.ny && (DIM == 2 || (z >= 0 && z < L.nz))) {
            const int nbx = x / G::BX, nby = y / G::BY, nbz = DIM == 3 ? z / G::BZ : 0;
            const int nbk = nbx + L.bnx * (nby + L.bny * nbz);
            if (bflag[nbk])
                v = get4((long long) nbk * G::BN + (x - nbx * G::BX) + G::BX * ((y - nby * G::BY) + G::BY * (z - nbz * G::BZ)));
        }
        *reinterpret_cast<float4 *>(tile + 4 * sx + G::PX * (ty + G::TY * tz)) = v;
    }
}

// Row stencil: the BX outputs of brick row (ly, lz),
//   out[i] = sum_{0 < |k|^2 < 16} c(|k|^2) tile[node (i, ly, lz) + k],
// from one 16-byte-vectorised load of each of the 45 (dy, dz) tile rows.
template<int DIM>
__device__ __forceinline__ void stencil_row(const float * tile, int ly, int lz, const Stencil & S,
                                            float (&out)[BrickGeom<DIM>::BX]) {
    using G          = BrickGeom<DIM>;
    constexpr int BX = G::BX;
    constexpr int ZR = DIM == 3 ? 3 : 0;
#pragma unroll
    for (int i = 0; i < BX; i++) out[i] = 0.f;
#pragma unroll
    for (int dz = -ZR; dz <= ZR; dz++)
#pragma unroll
        for (int dy = -3; dy <= 3; dy++) {
            const int ryz = dy * dy + dz * dz;
            if (ryz >= 16) continue;
            const float * row = tile + G::PX * ((ly + G::HALO + dy) + G::TY * (DIM == 3 ? lz + G::HALO + dz : 0));
            float v[G::TX];
#pragma unroll
            for (int s = 0; s < G::TX / 4; s++) {
                const float4 t = reinterpret_cast<const float4 *>(row)[s];
                v[4 * s] = t.x;
                v[4 * s + 1] = t.y;
                v[4 * s + 2] = t.z;
                v[4 * s + 3] = t.w;
            }
#pragma unroll
            for (int dx = -3; dx <= 3; dx++) {
                const int r2 = dx * dx + ryz;
                if (r2 >= 16 || r2 == 0) continue;
                const float c = S.c[r2];
#pragma unroll
                for (int i = 0; i < BX; i++) out[i] = fmaf(c, v[i + G::HALO + dx], out[i]);
            }
        }
}


}  // namespace swc
