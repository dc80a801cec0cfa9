// Internal (C++) interface shared by the sph103 translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "sph_common.cuh"

namespace sph {

constexpr int kBlock = 256;

// Uniform cell grid over the domain. Periodic axes are tiled by an integer number of
// cells (cell >= the requested size); non-periodic axes clamp out-of-range particles
// into the edge cells (clamping is 1-Lipschitz, so the 3x3 stencil stays a superset).
struct Grid {
    float mn[2];
    float inv_cell[2];
    int nc[2];
    int per[2];
    int rad;  // stencil radius in cells: (2 rad + 1)^2 cells cover the search radius
    // sorted slot range of the domain; periodic neighbor-list offsets are stored modulo
    // nslots so that neighbors across the wrap stay within a few cell rows of each other
    int slot0;
    int nslots;
};

__device__ __forceinline__ int cell_coord(float v, float mn, float inv, int nc) {
    int c = (int)floorf((v - mn) * inv);
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

constexpr int kMaxRad = 2;
constexpr int kMaxRows = 2 * kMaxRad + 1;
constexpr int kMaxRanges = 2 * kMaxRows;

// Rows (y cells) of the stencil around cy, each listed once.
__device__ __forceinline__ int stencil_rows(int cy, const Grid& g, int rows[kMaxRows]) {
    int nc = g.nc[1];
    if (g.per[1] && nc < 2 * g.rad + 1) {
        for (int k = 0; k < nc; ++k) rows[k] = k;
        return nc;
    }
    int n = 0;
    for (int dy = -g.rad; dy <= g.rad; ++dy) {
        int y = cy + dy;
        if (g.per[1]) y = (y + nc) % nc;
        else if (y < 0 || y >= nc) continue;
        rows[n++] = y;
    }
    return n;
}

// Column ranges [lo, hi] (inclusive) of the stencil around cx: one contiguous range, or
// two when a periodic axis wraps.
__device__ __forceinline__ int stencil_cols(int cx, const Grid& g, int lo[2], int hi[2]) {
    int nc = g.nc[0], R = g.rad;
    if (g.per[0]) {
        if (nc < 2 * R + 1) { lo[0] = 0; hi[0] = nc - 1; return 1; }
        if (cx - R < 0) { lo[0] = cx - R + nc; hi[0] = nc - 1; lo[1] = 0; hi[1] = cx + R; return 2; }
        if (cx + R > nc - 1) { lo[0] = cx - R; hi[0] = nc - 1; lo[1] = 0; hi[1] = cx + R - nc; return 2; }
    }
    lo[0] = cx - R > 0 ? cx - R : 0;
    hi[0] = cx + R < nc - 1 ? cx + R : nc - 1;
    return 1;
}

// Host helpers
Grid make_grid(const double mn[2], const double mx[2], const int per[2], double cell_min,
               int64_t* ncells_out, int rad = 1);
Geo make_geo(const double mn[2], const double mx[2], const int per[2]);

// Device-wide exclusive scans: out[0..n] with out[n] = total. tmp holds scan_tmp_elems(n).
int64_t scan_tmp_elems(int64_t n);
// With a gate (a device word), every launch returns at once when the word reads zero.
cudaError_t scan_exclusive(const int32_t* in, int32_t* out, int64_t n, int32_t* tmp, cudaStream_t s,
                           const uint32_t* gate = nullptr);
cudaError_t scan_exclusive(const int32_t* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t s,
                           const uint32_t* gate = nullptr);

// Counting sort of points (xy of a float2 or float4 array given by stride in floats) by
// cell, with ascending input index inside each cell (deterministic order).
// key[n], perm[n] (slot -> input index), count/fill[ncells], start[ncells+1].
cudaError_t cell_sort(const float* xy, int stride, int64_t n, const Grid& g, int64_t ncells,
                      int32_t* key, int32_t* perm, int32_t* count, int32_t* fill, int32_t* start,
                      int32_t* scan_tmp, cudaStream_t s);

// The same after the keys were computed and counted by the caller (count[key]++); with a
// gate, its kernels do nothing when the word reads zero (start and perm keep their values).
cudaError_t cell_sort_counted(int64_t n, int64_t ncells, const int32_t* key, int32_t* perm, int32_t* count,
                              int32_t* fill, int32_t* start, int32_t* scan_tmp, cudaStream_t s,
                              const uint32_t* gate = nullptr);

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Sequential carve-out of a caller workspace.
struct Carver {
    char* base;
    size_t off = 0;
    template <typename T>
    T* take(int64_t count) {
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += align256(sizeof(T) * (size_t)(count > 0 ? count : 1));
        return p;
    }
};

}  // namespace sph
