// swc_tiles.cuh -- brick/tile helpers shared by the node-lattice kernels:
// brick coordinates, reference-order compact index, halo tile loading (scalar
// and 16-byte vectorised) and the radial virtual-Laplacian stencil.
#pragma once

#include "swc_kernels.h"

namespace swc {

constexpr int kNT = 256;  // threads per block of the brick kernels

// Dynamic brick queue of the kernels without cross-block reductions (gather,
// pressure gradient): blocks take list indices from q[0] until they run out,
// and the last block to finish resets q[0] and its finish counter q[1] for the
// next launch, so a queue is zeroed once, at allocation.  Every thread of the
// block calls queue_take (it synchronises the block).
__device__ __forceinline__ int queue_take(int * q, int * slot) {
    __syncthreads();  // the previous *slot has been read by every thread
    if (threadIdx.x == 0) *slot = atomicAdd(q, 1);
    __syncthreads();
    return *slot;
}
__device__ __forceinline__ void queue_finish(int * q) {
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(q + 1, 1) == int(gridDim.x) - 1) {
            atomicExch(q, 0);
            atomicExch(q + 1, 0);
        }
    }
}

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
// or in inactive bricks read as zero.  PITCH: row pitch of the tile in floats
// (a multiple of 4).
template<int DIM, int NT = RowGeom<DIM>::NT, int PITCH = BrickGeom<DIM>::PX, class Get4>
__device__ __forceinline__ void load_tile4(const Lattice & L, const unsigned char * __restrict__ bflag, int3 bc,
                                           float * tile, Get4 get4) {
    using G            = BrickGeom<DIM>;
    constexpr int SEGX = G::TX / 4;
    constexpr int NSEG = SEGX * G::TY * G::TZ;
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
        *reinterpret_cast<float4 *>(tile + 4 * sx + PITCH * (ty + G::TY * tz)) = v;
    }
}

// Row stencil over a halo tile with row pitch PX, TY rows per z-plane, y/z
// halos HY/HZ and an x halo of 4 (rows start 16-byte aligned): the BX outputs
// of brick row (ly, lz),
//   out[i] = sum_{0 < |k|^2 < 16} c(|k|^2) tile[node (i, ly, lz) + k].
// The 45 (dy, dz) rows within reach (7 in 2D) fall into classes of equal
// m = dy^2 + dz^2 (9 in 3D: 0 1 2 4 5 8 9 10 13; 4 in 2D), and all rows of a
// class share the x-coefficients c(dx^2 + m).  The rows of a class are summed
// first (T_m) and the 1D x-convolution is applied once per class, so in 3D a
// row of 8 outputs costs 45 row loads, 450 adds and 416 FMAs instead of 2000
// FMAs.
template<int DIM, int PX, int TY, int M>
__device__ __forceinline__ void stencil_class(const float * centre, const Stencil & S,
                                              float (&out)[BrickGeom<DIM>::BX]) {
    constexpr int BX = BrickGeom<DIM>::BX, TX = BX + 8;
    constexpr int ZR = DIM == 3 ? 3 : 0;
    constexpr int R  = M <= 6 ? 3 : (M <= 11 ? 2 : 1);  // x reach: dx^2 + M <= 15
    float T[TX];
    bool have = false;
#pragma unroll
    for (int dz = -ZR; dz <= ZR; dz++)
#pragma unroll
        for (int dy = -3; dy <= 3; dy++) {
            if (dy * dy + dz * dz != M) continue;
            const float * row = centre + PX * (dy + TY * dz);
#pragma unroll
            for (int s = 0; s < TX / 4; s++) {
                const float4 t = reinterpret_cast<const float4 *>(row)[s];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int k = 4 * s + j;
                    if (k < 4 - R || k > BX + 3 + R) continue;
                    const float v = j == 0 ? t.x : (j == 1 ? t.y : (j == 2 ? t.z : t.w));
                    T[k]          = have ? T[k] + v : v;
                }
            }
            have = true;
        }
#pragma unroll
    for (int dx = -R; dx <= R; dx++) {
        if (dx == 0 && M == 0) continue;
        const float c = S.c[dx * dx + M];
#pragma unroll
        for (int i = 0; i < BX; i++) out[i] = fmaf(c, T[i + 4 + dx], out[i]);
    }
}

template<int DIM, int PX, int TY, int HY, int HZ>
__device__ __forceinline__ void stencil_row_t(const float * tile, int ly, int lz, const Stencil & S,
                                              float (&out)[BrickGeom<DIM>::BX]) {
    constexpr int BX     = BrickGeom<DIM>::BX;
    const float * centre = tile + PX * ((ly + HY) + TY * (DIM == 3 ? lz + HZ : 0));
#pragma unroll
    for (int i = 0; i < BX; i++) out[i] = 0.f;
    stencil_class<DIM, PX, TY, 0>(centre, S, out);
    stencil_class<DIM, PX, TY, 1>(centre, S, out);
    if constexpr (DIM == 3) stencil_class<DIM, PX, TY, 2>(centre, S, out);
    stencil_class<DIM, PX, TY, 4>(centre, S, out);
    if constexpr (DIM == 3) {
        stencil_class<DIM, PX, TY, 5>(centre, S, out);
        stencil_class<DIM, PX, TY, 8>(centre, S, out);
    }
    stencil_class<DIM, PX, TY, 9>(centre, S, out);
    if constexpr (DIM == 3) {
        stencil_class<DIM, PX, TY, 10>(centre, S, out);
        stencil_class<DIM, PX, TY, 13>(centre, S, out);
    }
}

// Row stencil over a brick-geometry tile (halo 4 on every side).
template<int DIM>
__device__ __forceinline__ void stencil_row(const float * tile, int ly, int lz, const Stencil & S,
                                            float (&out)[BrickGeom<DIM>::BX]) {
    using G = BrickGeom<DIM>;
    stencil_row_t<DIM, G::PX, G::TY, G::HALO, G::HALO>(tile, ly, lz, S, out);
}

// Halo tile of the CG SpMV: x halo 4 (16-byte aligned rows), y/z halo 3 (the
// stencil reach), pitch chosen so the 8 rows read by a quarter-warp's LDS.128
// hit distinct banks.
__device__ __forceinline__ void cp_async16(float * smem_dst, const float * gsrc, bool valid) {
    const unsigned sa = unsigned(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sa), "l"(gsrc), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// cp.async 16-byte copies (zero-filled when !valid) and their groups.
// Neighbour-brick table of brick b: tab[(k+1)*9 + (j+1)*3 + (i+1)] = id of brick
// (bx+i, by+j, bz+k) when it exists and is active, else -1.
template<int DIM>
__device__ __forceinline__ void neighbour_table(const Lattice & L, const unsigned char * __restrict__ bflag, int b,
                                                int * tab) {
    const int t = threadIdx.x;
    if (t < 27) {
        const int3 bc = brick_coords(L, b);
        const int i = t % 3 - 1, j = (t / 3) % 3 - 1, k = t / 9 - 1;
        const int x = bc.x + i, y = bc.y + j, z = bc.z + k;
        int id = -1;
        if (x >= 0 && x < L.bnx && y >= 0 && y < L.bny && z >= 0 && z < L.bnz && (DIM == 3 || k == 0)) {
            const int nb = x + L.bnx * (y + L.bny * z);
            if (bflag[nb]) id = nb;
        }
        tab[t] = id;
    }
}

template<int DIM> struct SpmvTile {
    using G = BrickGeom<DIM>;
    static constexpr int HX = 4, HY = 3, HZ = DIM == 3 ? 3 : 0;
    static constexpr int TX = G::BX + 2 * HX, TY = G::BY + 2 * HY, TZ = DIM == 3 ? G::BZ + 2 * HZ : 1;
    static constexpr int PX   = DIM == 3 ? 20 : 28;
    static constexpr int TILE = PX * TY * TZ;
};


}  // namespace swc
