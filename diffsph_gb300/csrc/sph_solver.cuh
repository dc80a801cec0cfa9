// Solver internals shared by the step kernels (sph_solver.cu) and the implicit shifting
// solve (sph_ips.cu): scheme constants, the domain table, the cell-stencil neighbor loops
// and the solver handle.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <vector>

#include "../../include/sph103.h"
#include "sph_internal.cuh"

namespace sph {

// pass_a_gradient: pass A launches that filter the skin list; pass_a_scan: those that scan
// the cell stencil (the first pass A after a sort, and every pass A of a periodic domain)
// ips_setup / ips_spmv / ips_vector: the implicit shift's neighbor pass (b and its list), its
// matrix products, and its vector updates (with the final position update); free_surface:
// the surface detection passes of the shift
// density_sum: the summation density of simulation.densityScheme 'summation'
enum KernelClass {
    KC_SORT = 0, KC_GATHER, KC_MDBC, KC_PASS_A, KC_PASS_B, KC_SHIFT, KC_PASS_A_SCAN,
    KC_IPS_SETUP, KC_IPS_SPMV, KC_IPS_VECTOR, KC_SURFACE, KC_DENSITY, KC_COUNT
};

// The classes' names: sph_solver_kernel_name and the NVTX ranges around their launches
inline const char* kernel_class_name(int cls) {
    static const char* const names[KC_COUNT] = {"cell_sort", "gather", "mdbc_ghosts", "pass_a_gradient",
                                                 "pass_b_rates", "shift", "pass_a_scan", "ips_setup",
                                                 "ips_spmv", "ips_vector", "free_surface", "density_sum"};
    return (cls >= 0 && cls < KC_COUNT) ? names[cls] : nullptr;
}

// Launch shapes of the neighbor passes (warps per block, list entry width, grid), picked per
// pass and problem by sph_solver_autotune; shape 0 is the default. Shapes 0-3 launch one
// block per tile of 32 W slots. Shape 4 is persistent: as many blocks as the SMs hold at
// once, each looping over the tiles blockIdx.x, blockIdx.x + gridDim.x, ... (for a packed
// batch, the tiles of all domains in the offset-indexed slot order). The loop is a
// separate kernel instance: it costs the passes 6-15 registers per thread, which the
// one-tile kernels do not pay.
struct Shape {
    int warps;
    int list16;
    int persist;
};
constexpr int kNumShapes = 5;
static const Shape kShapes[kNumShapes] = {{4, 0, 0}, {4, 1, 0}, {8, 1, 0}, {16, 1, 0}, {8, 1, 1}};
// The passes the autotuner shapes separately: pass A scanning the stencil (and keeping the
// skin list), pass A filtering the skin list, pass B, the delta+ shift, the summation density
enum TunedPass { TP_A_SCAN = 0, TP_A_FILTER, TP_B, TP_SHIFT, TP_DENSITY, TP_COUNT };
constexpr int kCap = 64;  // exact neighbors held per lane before the pair terms are evaluated
constexpr int kUnroll = 4;  // stencil candidates tested per lane per step of the scan
constexpr unsigned kFull = 0xffffffffu;

struct Phys {
    Geo geo;
    float h;            // support
    float T;            // exact inclusion threshold: s <= T  <=>  fl(fl(sqrt(s)) / h) <= 1
    float inv_h;
    float m;            // particle mass
    float dt, dth;      // dt, dt/2
    KernelCoef kc;
    Eos eos;
    float rho0;
    float diff_coef;    // delta * h / kappa * cs
    float diff_eps;     // 1e-6 * h
    float v_eps;        // eps * h^2
    float v_num;        // viscid 8 nu rho0 ; inviscid alpha h cs rho0   (divided by rho_i)
    float dvnum_dnu;    // d v_num / d nu (viscid: 8 rho0; inviscid: 0)
    int bvisc;
    float bv_eps, bv_num;
    float gx, gy;
    int nF;
    float invW0;        // 1 / W(dx/h) for the shifting term
    float shR, shN, sh_thr;
    int shN4;           // n == 4
    float sh_scale;     // -CFL * (h/kappa*2)^2 (times Ma)
    float inv_cs;
    int compute_mach;
    int density_update;
    float verlet_lim;   // (skin - 1) * h: largest displacement since the sort
    float T_skin;       // squared radius of the skin list (1.1 h, with a rounding margin)
    float skin_lim;     // displacement since the sort up to which the skin list holds every pair
    float area;         // particle area dx^2 (the omega of the implicit shifting matrices)
};

struct RhsOut {
    float* dudt;
    float* drhodt;
    float* grad;
    float* L;
    float* pressure;
    float* rho_b;
    int32_t* nn;    // [nF][2]: fluid and boundary neighbors (incl. self) per fluid particle
};

// One independent domain: its scheme constants, its cell grid and the offset of its cells in
// the global cell table. A single simulation is a table of one; packed batches of domains
// with different particle counts (and hence different dx, h, dt) share every kernel launch.
struct Dom {
    Phys P;
    Grid g;
    int32_t cell0;
    int32_t pad;
};
static_assert(sizeof(Dom) % 4 == 0, "Dom is copied as 32-bit words");

__device__ __forceinline__ bool is_boundary(float rho_signed) { return __float_as_int(rho_signed) < 0; }

__device__ __forceinline__ int dom_of(const int32_t* __restrict__ did, int64_t i, int64_t n) {
    return (did && i < n) ? did[i] : 0;
}

// Packed batches: a block of consecutive slots spans at most two domains when every domain
// holds at least a block's worth of particles. Their constants are copied to shared memory
// once per block; slots of any other domain read the global table.
__device__ __forceinline__ void stage_doms(const Dom* __restrict__ doms, const int32_t* __restrict__ did,
                                           int64_t first, int64_t last, int64_t n, Dom* s_dom, int* s_id) {
    const int64_t a = first < n ? first : n - 1, b = last < n ? last : n - 1;
    const int d0 = dom_of(did, a, n), d1 = dom_of(did, b, n);
    constexpr int kWords = (int)(sizeof(Dom) / 4);
    const uint32_t* src0 = reinterpret_cast<const uint32_t*>(doms + d0);
    const uint32_t* src1 = reinterpret_cast<const uint32_t*>(doms + d1);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s_dom);
    for (int k = threadIdx.x; k < 2 * kWords; k += blockDim.x) dst[k] = k < kWords ? src0[k] : src1[k - kWords];
    if (threadIdx.x == 0) {
        s_id[0] = d0;
        s_id[1] = d1;
    }
    __syncthreads();
}

__device__ __forceinline__ const Dom& dom_ref(const Dom* __restrict__ doms, const Dom* s_dom, const int* s_id,
                                              int d) {
    return d == s_id[0] ? s_dom[0] : (d == s_id[1] ? s_dom[1] : doms[d]);
}


// ------------------------------------------------------------------------------------
// Neighbor loop: candidates from the 3x3 cell stencil of the sort, exact filter, per-warp
// shared-memory list of accepted slots, then f(j) for every exact neighbor j. Every lane of
// the warp must call it (it votes); lanes with active == false contribute no pairs.
// The cells are >= (h + largest displacement since the sort), so the stencil of the
// particle's current cell holds every particle within h.
// ------------------------------------------------------------------------------------
// Bit k of *wrap marks range k as one whose pairs may cross the periodic boundary. Every
// other range lies within rad cells of the particle's cell without wrapping and away from
// the edge cells (where a particle may have crossed the boundary since the sort; the skin
// check keeps that motion below one cell). On an axis of at least 2 (rad + 2) cells its
// pairs then have |x_ij| < (rad + 2) cells <= half the extent, where the reference's minimum
// image is the identity, so the scan may skip it there exactly.
__device__ __forceinline__ int stencil_ranges(float2 p, const Grid& g, const int32_t* __restrict__ start,
                                              int rs[kMaxRanges], int re[kMaxRanges], unsigned* wrap = nullptr) {
    int cx = cell_coord(p.x, g.mn[0], g.inv_cell[0], g.nc[0]);
    int cy = cell_coord(p.y, g.mn[1], g.inv_cell[1], g.nc[1]);
    int rows[kMaxRows], lo[2], hi[2];
    int nr = stencil_rows(cy, g, rows);
    int ncol = stencil_cols(cx, g, lo, hi);
    const bool smallx = g.per[0] && g.nc[0] < 2 * g.rad + 4;
    const bool smally = g.per[1] && g.nc[1] < 2 * g.rad + 4;
    unsigned w = 0;
    int n = 0;
    for (int a = 0; a < nr; ++a) {
        int base = rows[a] * g.nc[0];
        const int dy = rows[a] - cy;
        const bool wy =
            smally || (g.per[1] && (dy > g.rad || dy < -g.rad || rows[a] == 0 || rows[a] == g.nc[1] - 1));
        for (int b = 0; b < ncol; ++b) {
            int s0 = __ldg(&start[base + lo[b]]), s1 = __ldg(&start[base + hi[b] + 1]);
            if (s1 > s0) {
                const bool wx = smallx || (g.per[0] && (lo[b] > cx + g.rad || hi[b] < cx - g.rad || lo[b] == 0 ||
                                                        hi[b] == g.nc[0] - 1));
                if (wx || wy) w |= 1u << n;
                rs[n] = s0;
                re[n] = s1;
                ++n;
            }
        }
    }
    if (wrap) *wrap = w;
    return n;
}

// Each scan step takes up to kUnroll consecutive candidates of the lane's current range,
// so that several independent loads are in flight per lane. List entries are slot offsets
// relative to the particle's own slot: int16_t halves the shared memory (leaving more of
// the unified L1 for the neighbor data) and is used when the grid keeps every stencil
// within +-32767 slots; an entry that does not fit raises SPH_FLAG_CAPACITY.
// capacity of the neighbor list pass A stores for pass B (entries per particle)
constexpr int kStoreCap = 64;
// skin list: every candidate within (1 + kSkinFrac) h at the sort positions, kept by the
// first pass A of a step; the second pass A and the shift filter it instead of the stencil
constexpr double kSkinFrac = 0.1;
constexpr int kSkinCap = 80;
// A stored row count (skin list, exact list) carries kRowWraps when the row's stencil held a
// range whose pairs may cross the periodic boundary (stencil_ranges): only such rows need the
// minimum image. A row without it and its candidates lie away from the edge cells and within
// rad cells of each other, and stay so while they move less than a cell, so their raw
// differences are the minimum image exactly. Counts stay below kRowCount; -1 marks a row that
// was not stored.
constexpr int kRowWraps = 0x4000;
constexpr int kRowCount = 0x3fff;



// The count of a stored row (negative: not stored) and the warp's wrap flags as
// neighbor_loop sets them (bit 0 this row, bit 1 some row of the warp). Every lane calls it.
__device__ __forceinline__ int row_count(int raw, int& wrap) {
    const bool wl = raw > 0 && (raw & kRowWraps) != 0;
    wrap = (wl ? 1 : 0) | (__any_sync(kFull, wl) ? 2 : 0);
    return raw < 0 ? raw : (raw & kRowCount);
}

// The stored count of a row with its wrap flag (bit 0 of a neighbor_loop / row_count flag word)
__device__ __forceinline__ int16_t stored_count(int cnt, int wrap) {
    return (int16_t)(cnt | ((wrap & 1) ? kRowWraps : 0));
}

template <typename LT>
__device__ __forceinline__ bool fits(int d) {
    return sizeof(LT) >= 4 || (d >= -32768 && d <= 32767);
}

template <bool PER>
__device__ __forceinline__ int list_slot(int self, int d, const Grid& g) {
    int j = self + d;
    if (PER) {
        if (j < g.slot0) j += g.nslots;
        else if (j >= g.slot0 + g.nslots) j -= g.nslots;
    }
    return j;
}

// SKIN: keep every candidate within the skin radius (T_skin) instead of the exact neighbors
// wrap (optional): set before the first f call to bit 0 = this lane's stencil has a range
// that may wrap, bit 1 = some lane of the warp's has.
template <bool PER, typename LT, class F, bool SKIN = false>
__device__ __forceinline__ void neighbor_loop(bool active, int self, float2 pi, const float4* __restrict__ X4,
                                              const int32_t* __restrict__ start, const Grid& g, const Phys& P,
                                              LT* __restrict__ lst, uint32_t* __restrict__ words, F&& f,
                                              int* wrap = nullptr) {
    const float thr = SKIN ? P.T_skin : P.T;
    const int lane = threadIdx.x & 31;
    int rs[kMaxRanges], re[kMaxRanges];
    unsigned wmask = 0;
    int nrng = active ? stencil_ranges(pi, g, start, rs, re, PER ? &wmask : nullptr) : 0;
    if (wrap) {
        const bool wl = PER && wmask != 0u;
        *wrap = (wl ? 1 : 0) | (__any_sync(kFull, wl) ? 2 : 0);
    }
    int r = 0;
    int s = nrng > 0 ? rs[0] : 0, se = nrng > 0 ? re[0] : 0;
    int cnt = 0;
    bool overflow = false;
    while (__any_sync(kFull, r < nrng)) {
        if (r < nrng) {
            int m = se - s < kUnroll ? se - s : kUnroll;
            const bool wr = PER && ((wmask >> r) & 1u);
            float4 xj[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u)
                if (u < m) xj[u] = __ldg(&X4[s + u]);
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                if (u < m) {
                    float x0, x1;
                    if (wr)
                        pair_vec<true>(pi, make_float2(xj[u].x, xj[u].y), P.geo, x0, x1);
                    else
                        pair_vec<false>(pi, make_float2(xj[u].x, xj[u].y), P.geo, x0, x1);
                    if (sq_norm_ref(x0, x1) <= thr) {
                        int d = s + u - self;
                        if (PER) {  // shortest offset modulo the domain's slots
                            const int h2 = g.nslots >> 1;
                            if (d > h2) d -= g.nslots;
                            else if (d < -h2) d += g.nslots;
                        }
                        if (fits<LT>(d)) lst[(cnt++) * 32 + lane] = (LT)d;
                        else overflow = true;
                    }
                }
            }
            s += m;
            if (s == se) {
                ++r;
                if (r < nrng) {
                    s = rs[r];
                    se = re[r];
                }
            }
        }
        if (__any_sync(kFull, cnt > kCap - kUnroll)) {
            int mc = (int)__reduce_max_sync(kFull, (unsigned)cnt);
            for (int k = 0; k < mc; ++k)
                if (k < cnt) f(list_slot<PER>(self, (int)lst[k * 32 + lane], g));
            cnt = 0;
        }
    }
    int mc = (int)__reduce_max_sync(kFull, (unsigned)cnt);
    for (int k = 0; k < mc; ++k)
        if (k < cnt) f(list_slot<PER>(self, (int)lst[k * 32 + lane], g));
    if (overflow) atomicOr(&words[0], SPH_FLAG_CAPACITY);
}

// The stored lists (skin list, exact list) are warp-tile-major: the cap entries of the 32
// slots of a warp form one block, entry k of every lane contiguous, so a lane walks its row
// at a fixed 64-byte stride (no index arithmetic per entry) and the warp's k-th loads
// coalesce. Row of slot i: list + tile_row(i, cap), entry k at [k * 32].
__host__ __device__ __forceinline__ int64_t tile_row(int64_t i, int cap) {
    return (i >> 5) * (int64_t)(cap * 32) + (i & 31);
}
// elements of a list of cap entries per slot for n slots (rounded up to whole warps)
inline int64_t tile_elems(int64_t n, int cap) { return ((n + 31) & ~(int64_t)31) * cap; }

// The xy of a stored state entry (an 8-byte load of the float4)
__device__ __forceinline__ float2 ldg_xy(const float4* __restrict__ X4, int j) {
    return __ldg(reinterpret_cast<const float2*>(X4) + 2 * (int64_t)j);
}

// The exact neighbors of the stored skin list (scan order of the first pass A of the step,
// so the same order a scan at the same cells gives), filtered at the current positions.
template <bool PER, class F>
__device__ __forceinline__ void skin_loop(int self, float2 pi, const float4* __restrict__ X4, const Grid& g,
                                          const Phys& P, const int16_t* __restrict__ sl, int cnt, F&& f) {
    const int16_t* __restrict__ row = sl + tile_row(self, kSkinCap);
    int k = 0;
    for (; k + 4 <= cnt; k += 4) {
        int j[4];
        float2 xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) j[u] = list_slot<PER>(self, (int)row[(k + u) * 32], g);
#pragma unroll
        for (int u = 0; u < 4; ++u) xj[u] = ldg_xy(X4, j[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            float x0, x1;
            pair_vec<PER>(pi, xj[u], P.geo, x0, x1);
            if (sq_norm_ref(x0, x1) <= P.T) f(j[u]);
        }
    }
    for (; k < cnt; ++k) {
        const int j = list_slot<PER>(self, (int)row[k * 32], g);
        float x0, x1;
        pair_vec<PER>(pi, ldg_xy(X4, j), P.geo, x0, x1);
        if (sq_norm_ref(x0, x1) <= P.T) f(j);
    }
}

// The same neighbors in two steps, for pair terms that cost more than the test: the filter
// (list entry, neighbor position, the reference's exact test) fills the warp's shared-memory
// list lst, then f(j) runs over the accepted entries with every lane busy, in the skin
// list's order. Every lane of the warp must call it (it votes); lanes with cnt = 0 add no
// pairs. WR: some row of the warp carries kRowWraps, so the filter takes the minimum image
// and the slots the modular form (the offsets of the other rows are direct). PF: load the next
// group's entries ahead (measured faster on single domains, slower in packed batches).
template <bool PER, bool WR, typename LT, class F, bool PF = true>
__device__ __forceinline__ void skin_list_loop(int self, float2 pi, const float4* __restrict__ X4, const Grid& g,
                                               const Phys& P, const int16_t* __restrict__ sl, int cnt,
                                               LT* __restrict__ lst, F&& f) {
    const int lane = threadIdx.x & 31;
    const int kmax = (int)__reduce_max_sync(kFull, (unsigned)cnt);
    const int16_t* __restrict__ row = sl + tile_row(self, kSkinCap);
    int m = 0;
    // PF: the next group's entries are loaded before this group's tests, so their latency
    // (the list is read from DRAM) hides behind the work of this group
    int dn[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) dn[u] = (PF && u < cnt) ? (int)row[u * 32] : 0;
    for (int k = 0; k < kmax; k += 4) {
        int d[4];
        float2 xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) d[u] = PF ? dn[u] : ((k + u < cnt) ? (int)row[(k + u) * 32] : 0);
        if (PF) {
#pragma unroll
            for (int u = 0; u < 4; ++u) dn[u] = (k + 4 + u < cnt) ? (int)row[(k + 4 + u) * 32] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k + u < cnt) xj[u] = ldg_xy(X4, list_slot<WR>(self, d[u], g));
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (k + u < cnt) {
                float x0, x1;
                pair_vec<WR>(pi, xj[u], P.geo, x0, x1);
                if (sq_norm_ref(x0, x1) <= P.T) lst[(m++) * 32 + lane] = (LT)d[u];
            }
        }
        if (__any_sync(kFull, m > kCap - 4)) {
            const int mc = (int)__reduce_max_sync(kFull, (unsigned)m);
            for (int q = 0; q < mc; ++q)
                if (q < m) f(list_slot<WR>(self, (int)lst[q * 32 + lane], g));
            m = 0;
        }
    }
    const int mc = (int)__reduce_max_sync(kFull, (unsigned)m);
    for (int q = 0; q < mc; ++q)
        if (q < m) f(list_slot<WR>(self, (int)lst[q * 32 + lane], g));
}

// Geometry of a pair that already passed the exact test: r, q = r / h and the reference's
// unit-vector factor inv = 1 / (r + 1e-7) (tolerance-checked sums: fast reciprocal square
// root and reciprocal). 1e-30 enters the squared norm so that the self pair (sq = 0) gives
// r = 0 rather than 0 * inf; it changes no realistic sq.
struct PairR {
    float sq, r, q, inv;
};

__device__ __forceinline__ PairR pair_r(float x0, float x1, float inv_h) {
    PairR p;
    p.sq = fmaf(x1, x1, fmaf(x0, x0, 1e-30f));
    p.r = p.sq * rsqrtf(p.sq);
    p.q = p.r * inv_h;
    p.inv = __fdividef(1.0f, p.r + 1e-7f);
    return p;
}

// The Wendland C2 gradient as gradW = x_ij * wendland_gf(...): with om = (1 - q)_+,
// dW/dr = -20 q om^3 C_d/h^3 and xhat = x_ij inv, so the factor is q om^3 (-20 C_d/h^3) inv.
__device__ __forceinline__ float wendland_gf(const PairR& p, float om, float cg20) {
    return (p.q * (om * om * om)) * cg20 * p.inv;
}

// Free-surface fields of the shift (solveShifting with shifting.freeSurface), per slot;
// fs == nullptr when the handling is off.
struct SurfaceView {
    const uint8_t* fs;    // on the surface (detectFreeSurfaceBarecasco)
    const uint8_t* fsm;   // expanded mask (expandFreeSurfaceMask)
    const float* lam;     // Lambdas: the smaller singular value of the normalization matrix
    const float2* nrm;    // normalised lambda gradient
    float scaling;        // shifting.surfaceScaling
};

// The projection of solveShifting (shifting.py:972-982, projectionScheme 'mat') applied to
// the update before its clamp: (I - n n^T) u on the expanded mask, zero where Lambdas < 0.4,
// times surfaceScaling on the surface.
__device__ __forceinline__ void surface_project(const SurfaceView& sv, int64_t i, float& u0, float& u1) {
    if (!sv.fs) return;
    if (sv.fsm[i]) {
        const float2 nn = sv.nrm[i];
        const float m00 = 1.f - nn.x * nn.x, m01 = 0.f - nn.x * nn.y;
        const float m10 = 0.f - nn.y * nn.x, m11 = 1.f - nn.y * nn.y;
        const float r0 = m00 * u0 + m01 * u1, r1 = m10 * u0 + m11 * u1;
        u0 = r0;
        u1 = r1;
    }
    if (sv.lam[i] < 0.4f) {
        u0 = 0.f;
        u1 = 0.f;
    }
    if (sv.fs[i]) {
        u0 *= sv.scaling;
        u1 *= sv.scaling;
    }
}

}  // namespace sph

using namespace sph;

// ------------------------------------------------------------------------------------
// Solver handle (one domain, or a packed batch of independent fluid domains)
// ------------------------------------------------------------------------------------
struct sph_solver {
    sph_params_t prm;            // parameters of domain 0 (mDBC, shifting switch)
    int nd = 1;
    std::vector<Dom> doms_host;
    std::vector<int64_t> off_host;  // fluid particle offsets of the domains [nd + 1]
    int64_t nF, nB, n;
    int64_t ncells;
    bool periodic;
    float2 *Xr, *Xr_t;
    float2* Xs;                  // raw positions at the last cell sort (displacement checks)
    float4 *Xc, *Xh, *Xf, *Xt;
    float4 *Vc, *Vh, *Vf, *Vt;
    int32_t *uid, *uid_t, *did, *did_t;
    int32_t* slot;  // slot of each particle (original order): the inverse of uid
    int32_t *key, *perm, *count, *fill, *start, *scan32;
    int32_t* bidx;
    // [0] flags, [2] boundary count, [3] skin list invalid, [4] sort this step, [5] sorts done
    uint32_t* words;
    int16_t* nl;      // exact neighbor list of the last pass A: slot offsets, [kStoreCap][n]
    int16_t* nlc;     // its length per slot (-1: not stored)
    int16_t* sl;      // skin list of the step's first pass A, [kSkinCap][n]
    int16_t* slc;     // its length per slot (-1: not stored)
    float* msums;     // mDBC ghost moments, [nB][kMdbcSums]
    uint32_t* maxv;   // per-domain max |u| (float bits)
    Dom* doms;
    int64_t* dom_off;
    float2* bnormal;
    float* bdist;
    bool list16 = false;
    int shape_of[TP_COUNT] = {0, 0, 0, 0, 0};  // launch shape per tuned pass
    int grid_cap[TP_COUNT][kNumShapes] = {};   // persistent grid per pass and shape (0: not yet known)
    bool attrs_set = false;
    bool tables_uploaded = false;
    // Verlet reuse of the cell sort and the skin list across steps: a step sorts again only
    // when a particle moved farther than its domain's limit since the last sort (reuse_lim
    // for one domain; min(reuse_half h, 0.7 skin_lim) per domain of a batch), or the skin
    // list of that sort went invalid
    bool reuse = false;
    bool uploaded = false;  // a state was loaded (uid holds the slot order)
    float reuse_lim = 0.f;
    float reuse_half = 1e30f;  // (verletScale - 1) / 2: the reference's limit over h
    // captured step graph
    // captured step graphs, keyed by step count and buffer assignment (two slots: eager
    // steps between replays alternate the assignment)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_n[2] = {0, 0};
    const void* graph_key[2][14] = {};
    int graph_next = 0;

    // timing
    uint32_t timing_mask = 0;
    struct Ev {
        cudaEvent_t a, b;
        int cls;
    };
    std::vector<Ev> pool;
    size_t used = 0;

    // implicit particle shifting (shifting.scheme 'IPS'), replacing delta+ once configured
    bool ips = false;
    float ips_rtol = 1e-4f;
    int ips_maxiter = 64;
    float ips_thr = 0.f;             // per-particle |x| limit of the solve (solverThreshold)
    float2* ips_vec = nullptr;       // x, r, r0, p, ap, s, as: [7][n] in the caller's workspace
    float* ips_H = nullptr;          // blocks of the stored exact list (warp-tile-major)
    int16_t* ips_nl = nullptr;       // that list: slot offsets (warp-tile-major)
    int16_t* ips_nlc = nullptr;      // its length per slot (-1: not stored)
    int ips_sms = 0;                 // SM count of the device (grid caps)

    // free-surface handling of the shift (shifting.freeSurface), off unless set
    bool fs_on = false;
    float fs_cos_half = 0.f;         // cos(surfaceDetection.BarecascoThreshold / 2)
    int fs_expand = 2;               // surfaceDetection.expansionIterations
    float fs_scaling = 0.1f;         // shifting.surfaceScaling
    uint8_t *fs = nullptr, *fsm = nullptr, *fsm_t = nullptr;
    float* fs_lam = nullptr;
    float4* fs_L = nullptr;
    float2* fs_nrm = nullptr;
    int16_t *fs_nl = nullptr, *fs_nlc = nullptr;
    double* ips_part = nullptr;      // per-block partial sums
    void* ips_state = nullptr;       // scalars of the solve (device)
};

// The implicit shift on the sorted state Xin/Vin (integrated positions) into Xout/Vout, with
// the fluid increments in the original order in dx_out when non-NULL (sph_ips.cu).
int ips_shift(sph_solver* S, float4* Xin, float4* Vin, float4* Xout, float4* Vout, float* dx_out, int use_skin,
              cudaStream_t st);
size_t ips_workspace_bytes(int64_t n);
// The free-surface fields at the sorted state X4 (sph_surface.cu); a view of them for the
// shift kernels (fs == nullptr when the handling is off).
int surface_detect(sph_solver* S, const float4* X4, int use_skin, cudaStream_t st);
SurfaceView surface_view(const sph_solver* S);

inline unsigned blocks_for(int64_t n, int threads = kBlock) { return (unsigned)((n + threads - 1) / threads); }

// Blocks of a neighbor-pass launch: one per tile of 32 W slots, or for a persistent shape
// the blocks the SMs hold at once (capped by the tiles). kern is the kernel instance,
// smem its dynamic shared memory; the occupancy query runs once per pass and shape.
template <class K>
inline unsigned pass_grid(sph_solver* S, int pass, int shape, K kern, int threads, size_t smem) {
    const unsigned tiles = blocks_for(S->n, threads);
    if (!kShapes[shape].persist) return tiles;
    int& cap = S->grid_cap[pass][shape];
    if (cap == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        cap = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    }
    return tiles < (unsigned)cap ? tiles : (unsigned)cap;
}

// The tiles of a neighbor-pass block: body(first) for the first slot of each tile the block
// owns, one tile (PERSIST false) or every gridDim.x-th tile from blockIdx.x on. For packed
// batches the domain constants of the tile are staged in shared memory first (after a
// barrier between tiles, so no warp still reads the previous tile's).
template <bool BATCH, int W, bool PERSIST, class F>
__device__ __forceinline__ void run_tiles(int64_t n, const Dom* __restrict__ doms, const int32_t* __restrict__ did,
                                          Dom* s_dom, int* s_id, F&& body) {
    const int64_t first0 = (int64_t)blockIdx.x * (32 * W);
    if (!PERSIST) {
        if (BATCH) stage_doms(doms, did, first0, first0 + 32 * W - 1, n, s_dom, s_id);
        body(first0);
        return;
    }
    const int64_t step = (int64_t)gridDim.x * (32 * W);
#pragma unroll 1
    for (int64_t first = first0; first < n; first += step) {
        if (BATCH) {
            if (first != first0) __syncthreads();
            stage_doms(doms, did, first, first + 32 * W - 1, n, s_dom, s_id);
        }
        body(first);
    }
}

template <typename LT, int W>
constexpr size_t list_bytes() { return (size_t)W * kCap * 32 * sizeof(LT); }

// brackets of each launch group: an NVTX range named after its class (host-side, so a
// profiler can select the group's kernels by range), and CUDA events for the classes in the
// timing mask
inline void tbeg(sph_solver* S, int cls, cudaStream_t st) {
    nvtxRangePushA(kernel_class_name(cls));
    if (!(S->timing_mask & (1u << cls))) return;
    if (S->used == S->pool.size()) {
        sph_solver::Ev e;
        cudaEventCreate(&e.a);
        cudaEventCreate(&e.b);
        S->pool.push_back(e);
    }
    S->pool[S->used].cls = cls;
    cudaEventRecord(S->pool[S->used].a, st);
}
inline void tend(sph_solver* S, int cls, cudaStream_t st) {
    nvtxRangePop();
    if (!(S->timing_mask & (1u << cls))) return;
    cudaEventRecord(S->pool[S->used].b, st);
    S->used++;
}
