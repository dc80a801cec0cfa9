// Cell grid, device-wide scans, counting sort by cell, and the exact neighbor search
// exported for the neighborSearch drop-in (src/diffSPH/v2/modules/neighborhood.py:491-593).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <math.h>

#include <mutex>

#include "../../include/sph103.h"
#include "sph_internal.cuh"

namespace sph {

Geo make_geo(const double mn[2], const double mx[2], const int per[2]) {
    Geo g;
    for (int a = 0; a < 2; ++a) {
        g.mn[a] = (float)mn[a];
        g.ext[a] = (float)(mx[a] - mn[a]);
        g.half[a] = (float)((mx[a] - mn[a]) / 2.0);
        g.per[a] = per[a] ? 1 : 0;
    }
    return g;
}

Grid make_grid(const double mn[2], const double mx[2], const int per[2], double cell_min,
               int64_t* ncells_out, int rad) {
    Grid g;
    g.rad = rad;
    g.slot0 = 0;
    g.nslots = 0;
    int64_t total = 1;
    for (int a = 0; a < 2; ++a) {
        double ext = mx[a] - mn[a];
        int nc;
        double cell;
        if (per[a]) {
            nc = (int)floor(ext / cell_min);
            if (nc < 1) nc = 1;
            cell = ext / nc;
        } else {
            nc = (int)ceil(ext / cell_min);
            if (nc < 1) nc = 1;
            cell = cell_min;
        }
        g.mn[a] = (float)mn[a];
        g.inv_cell[a] = (float)(1.0 / cell);
        g.nc[a] = nc;
        g.per[a] = per[a] ? 1 : 0;
        total *= nc;
    }
    if (ncells_out) *ncells_out = total;
    return g;
}

// ------------------------------------------------------------------------------------
// Exclusive scan: 256 threads x 8 items per block, block totals scanned by one block.
// ------------------------------------------------------------------------------------
constexpr int kScanItems = 8;
constexpr int kScanTile = kBlock * kScanItems;

int64_t scan_tmp_elems(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

template <typename O>
__device__ __forceinline__ O block_exclusive(O v, O* total) {
    __shared__ O warp_tot[kBlock / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    O x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        O y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        O w = lane < kBlock / 32 ? warp_tot[lane] : O(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            O y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kBlock / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    O base = wid > 0 ? warp_tot[wid - 1] : O(0);
    if (total) *total = warp_tot[kBlock / 32 - 1];
    O res = base + x - v;
    __syncthreads();
    return res;
}

// gate: a device word read at entry; when it is given and zero the launch does nothing
// (the solver skips the cell sort of a step that reuses the previous one)
__device__ __forceinline__ bool gated_off(const uint32_t* gate) { return gate && *gate == 0u; }

template <typename I, typename O>
__global__ void k_scan_local(const I* __restrict__ in, O* __restrict__ out, O* __restrict__ sums, int64_t n,
                             const uint32_t* gate) {
    if (gated_off(gate)) return;
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    O v[kScanItems];
    O t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? (O)in[i] : O(0);
        t += v[k];
    }
    O tot;
    O ex = block_exclusive<O>(t, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename O>
__global__ void k_scan_sums(O* sums, int64_t nb, const uint32_t* gate) {
    if (gated_off(gate)) return;
    O carry = 0;
    for (int64_t c0 = 0; c0 < nb; c0 += kBlock) {
        int64_t i = c0 + threadIdx.x;
        O v = i < nb ? sums[i] : O(0);
        O tot;
        O ex = block_exclusive<O>(v, &tot);
        if (i < nb) sums[i] = ex + carry;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

template <typename O>
__global__ void k_scan_add(O* __restrict__ out, const O* __restrict__ sums, int64_t n, int64_t nb,
                           const uint32_t* gate) {
    if (gated_off(gate)) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / kScanTile];
    if (i == 0) out[n] = sums[nb];
}

template <typename I, typename O>
static cudaError_t scan_impl(const I* in, O* out, int64_t n, O* tmp, cudaStream_t s, const uint32_t* gate) {
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) {
        return cudaMemsetAsync(out, 0, sizeof(O), s);
    }
    k_scan_local<I, O><<<(unsigned)nb, kBlock, 0, s>>>(in, out, tmp, n, gate);
    k_scan_sums<O><<<1, kBlock, 0, s>>>(tmp, nb, gate);
    k_scan_add<O><<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(out, tmp, n, nb, gate);
    return cudaGetLastError();
}

cudaError_t scan_exclusive(const int32_t* in, int32_t* out, int64_t n, int32_t* tmp, cudaStream_t s,
                           const uint32_t* gate) {
    return scan_impl<int32_t, int32_t>(in, out, n, tmp, s, gate);
}
cudaError_t scan_exclusive(const int32_t* in, int64_t* out, int64_t n, int64_t* tmp, cudaStream_t s,
                           const uint32_t* gate) {
    return scan_impl<int32_t, int64_t>(in, out, n, tmp, s, gate);
}

// ------------------------------------------------------------------------------------
// Counting sort by cell
// ------------------------------------------------------------------------------------
__global__ void k_cell_keys(const float* __restrict__ xy, int stride, int64_t n, Grid g,
                            int32_t* __restrict__ key, int32_t* __restrict__ count) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = xy[i * stride], y = xy[i * stride + 1];
    int cx = cell_coord(x, g.mn[0], g.inv_cell[0], g.nc[0]);
    int cy = cell_coord(y, g.mn[1], g.inv_cell[1], g.nc[1]);
    int k = cy * g.nc[0] + cx;
    key[i] = k;
    atomicAdd(&count[k], 1);
}

__global__ void k_cell_scatter(int64_t n, const int32_t* __restrict__ key, const int32_t* __restrict__ start,
                               int32_t* __restrict__ fill, int32_t* __restrict__ perm, const uint32_t* gate) {
    if (gated_off(gate)) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = key[i];
    int slot = start[k] + atomicAdd(&fill[k], 1);
    perm[slot] = (int32_t)i;
}

// Cells hold a few tens of particles: one thread sorts its cell's slots by input index.
__global__ void k_cell_order(int64_t ncells, const int32_t* __restrict__ start, int32_t* __restrict__ perm,
                             const uint32_t* gate) {
    if (gated_off(gate)) return;
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = start[c], e = start[c + 1];
    for (int a = b + 1; a < e; ++a) {
        int v = perm[a];
        int k = a - 1;
        while (k >= b && perm[k] > v) {
            perm[k + 1] = perm[k];
            --k;
        }
        perm[k + 1] = v;
    }
}

cudaError_t cell_sort_counted(int64_t n, int64_t ncells, const int32_t* key, int32_t* perm, int32_t* count,
                              int32_t* fill, int32_t* start, int32_t* scan_tmp, cudaStream_t s,
                              const uint32_t* gate) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(fill, 0, sizeof(int32_t) * ncells, s)) != cudaSuccess) return e;
    if ((e = scan_exclusive(count, start, ncells, scan_tmp, s, gate)) != cudaSuccess) return e;
    unsigned gb = (unsigned)((n + kBlock - 1) / kBlock);
    if (n > 0) k_cell_scatter<<<gb, kBlock, 0, s>>>(n, key, start, fill, perm, gate);
    k_cell_order<<<(unsigned)((ncells + kBlock - 1) / kBlock), kBlock, 0, s>>>(ncells, start, perm, gate);
    return cudaGetLastError();
}

cudaError_t cell_sort(const float* xy, int stride, int64_t n, const Grid& g, int64_t ncells,
                      int32_t* key, int32_t* perm, int32_t* count, int32_t* fill, int32_t* start,
                      int32_t* scan_tmp, cudaStream_t s) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(count, 0, sizeof(int32_t) * ncells, s)) != cudaSuccess) return e;
    unsigned gb = (unsigned)((n + kBlock - 1) / kBlock);
    if (n > 0) k_cell_keys<<<gb, kBlock, 0, s>>>(xy, stride, n, g, key, count);
    return cell_sort_counted(n, ncells, key, perm, count, fill, start, scan_tmp, s);
}

// ------------------------------------------------------------------------------------
// Exact neighbor search, separate query and reference sets, per-particle h_j.
// ------------------------------------------------------------------------------------
// The largest fp32 s with fl(fl(sqrt(s)) / h) <= 1 (IEEE round-to-nearest): both steps are
// monotone in s, so exact_in(s, h) holds exactly for s <= T. The searches reject most
// stencil candidates (about two in three) by this one comparison and take the square root
// and the division only for the accepted ones. -1 for a support that admits no pair.
__device__ float exact_T(float h) {
    if (!(h > 0.f) || !isfinite(h)) return -1.f;
    auto ok = [&](float s) { return __fdiv_rn(__fsqrt_rn(s), h) <= 1.f; };
    float s = __fmul_rn(h, h);
    for (int k = 0; k < 64 && !ok(s); ++k) s = nextafterf(s, 0.f);
    for (int k = 0; k < 64 && ok(nextafterf(s, INFINITY)); ++k) s = nextafterf(s, INFINITY);
    return s;
}

struct NbWork {
    Grid grid;
    Geo geo;
    int64_t ncells;
    int32_t *key, *perm, *count, *fill, *start, *scan32;
    int64_t* scan64;
    float2* ref_tmp;    // wrapped reference positions, input order
    float2* ref_xy;     // sorted, wrapped reference positions
    // per sorted reference slot s: [2 s] = (h, T) with T the exact threshold
    // (s <= T <=> fl(fl(sqrt(s)) / h) <= 1), [2 s + 1] = the kernel's (C_d / h^2, C_d / h^3)
    float2* ref_hT;
    int32_t* ref_idx;   // sorted -> original index
    float2* qry_xy;     // wrapped query positions
};

static int nb_layout(int64_t nq, int64_t nr, const sph_domain_t* d, double hmax, void* ws, NbWork* w,
                     size_t* bytes) {
    if (!d || hmax <= 0 || nq < 0 || nr < 0) return SPH_ERR_ARGUMENT;
    int per[2] = {d->periodic[0], d->periodic[1]};
    w->grid = make_grid(d->min, d->max, per, hmax * (1.0 + 1e-4), &w->ncells);
    w->geo = make_geo(d->min, d->max, per);
    if (w->ncells > (int64_t)1 << 30) return SPH_ERR_ARGUMENT;
    Carver c{(char*)ws};
    w->key = c.take<int32_t>(nr);
    w->perm = c.take<int32_t>(nr);
    w->count = c.take<int32_t>(w->ncells);
    w->fill = c.take<int32_t>(w->ncells);
    w->start = c.take<int32_t>(w->ncells + 1);
    w->scan32 = c.take<int32_t>(scan_tmp_elems(w->ncells > nq ? w->ncells : nq));
    w->scan64 = c.take<int64_t>(scan_tmp_elems(nq));
    w->ref_tmp = c.take<float2>(nr);
    w->ref_xy = c.take<float2>(nr);
    w->ref_hT = c.take<float2>(2 * nr);
    w->ref_idx = c.take<int32_t>(nr);
    w->qry_xy = c.take<float2>(nq);
    *bytes = c.off;
    return SPH_OK;
}

__global__ void k_wrap_copy(const float* __restrict__ x, int64_t n, Geo geo, float2* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = wrap_pos(make_float2(x[2 * i], x[2 * i + 1]), geo);
}

__global__ void k_ref_gather(int64_t n, const int32_t* __restrict__ perm, const float2* __restrict__ wrapped,
                             const float* __restrict__ h, float2* __restrict__ sxy, float2* __restrict__ shT,
                             int32_t* __restrict__ sidx) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int o = perm[s];
    sxy[s] = wrapped[o];
    const float hh = h[o];
    shT[2 * s] = make_float2(hh, exact_T(hh));
    shT[2 * s + 1] = make_float2(kCd / (hh * hh), kCd / (hh * hh * hh));
    sidx[s] = o;
}

// One query row by one thread: the count (FILL = false), or the row's pairs written and then
// put in the reference's column order by an insertion sort in place (FILL = true; the fill of
// rows longer than the warp fill's shared buffer).
template <bool FILL>
__device__ void nb_row(int64_t i, const float2* __restrict__ qxy, const float2* __restrict__ rxy,
                       const float2* __restrict__ rhT, const int32_t* __restrict__ ridx,
                       const int32_t* __restrict__ start, const Grid& g, const Geo& geo, int32_t* __restrict__ counts,
                       const int64_t* __restrict__ offsets, int64_t* __restrict__ pi, int64_t* __restrict__ pj,
                       float* __restrict__ pq, float* __restrict__ px, float* __restrict__ ph) {
    float2 p = qxy[i];
    int cx = cell_coord(p.x, g.mn[0], g.inv_cell[0], g.nc[0]);
    int cy = cell_coord(p.y, g.mn[1], g.inv_cell[1], g.nc[1]);
    int rows[kMaxRows], lo[2], hi[2];
    int nr = stencil_rows(cy, g, rows);
    int ncr = stencil_cols(cx, g, lo, hi);
    int64_t w = FILL ? offsets[i] : 0;
    int cnt = 0;
    for (int a = 0; a < nr; ++a) {
        for (int b = 0; b < ncr; ++b) {
            int c0 = rows[a] * g.nc[0] + lo[b], c1 = rows[a] * g.nc[0] + hi[b];
            int s0 = start[c0], s1 = start[c1 + 1];
            for (int s = s0; s < s1; ++s) {
                float x0, x1;
                pair_vec<true>(p, rxy[s], geo, x0, x1);
                const float sq = sq_norm_ref(x0, x1);
                const float2 hT = rhT[2 * s];
                if (!(sq <= hT.y)) continue;  // exactly the reference's q <= 1 (exact_T)
                if (FILL) {
                    float r, q;
                    exact_in(sq, hT.x, r, q);
                    float den = __fadd_rn(r, 1e-7f);
                    int64_t o = w + cnt;
                    pi[o] = i;
                    pj[o] = ridx[s];
                    pq[o] = q;
                    px[2 * o] = __fdiv_rn(x0, den);
                    px[2 * o + 1] = __fdiv_rn(x1, den);
                    ph[o] = hT.x;
                }
                ++cnt;
            }
        }
    }
    if (!FILL) counts[i] = cnt;
    if (FILL) {
        // canonical order: ascending reference index inside the row
        int64_t b0 = w, e0 = w + cnt;
        for (int64_t a2 = b0 + 1; a2 < e0; ++a2) {
            int64_t vj = pj[a2];
            float vq = pq[a2], vx0 = px[2 * a2], vx1 = px[2 * a2 + 1], vh = ph[a2];
            int64_t k = a2 - 1;
            while (k >= b0 && pj[k] > vj) {
                pj[k + 1] = pj[k];
                pq[k + 1] = pq[k];
                px[2 * (k + 1)] = px[2 * k];
                px[2 * (k + 1) + 1] = px[2 * k + 1];
                ph[k + 1] = ph[k];
                --k;
            }
            pj[k + 1] = vj;
            pq[k + 1] = vq;
            px[2 * (k + 1)] = vx0;
            px[2 * (k + 1) + 1] = vx1;
            ph[k + 1] = vh;
        }
    }
}

template <bool FILL>
__global__ void k_nb_query(int64_t nq, const float2* __restrict__ qxy, const float2* __restrict__ rxy,
                           const float2* __restrict__ rhT, const int32_t* __restrict__ ridx,
                           const int32_t* __restrict__ start, Grid g, Geo geo, int32_t* __restrict__ counts,
                           const int64_t* __restrict__ offsets, int64_t* __restrict__ pi, int64_t* __restrict__ pj,
                           float* __restrict__ pq, float* __restrict__ px, float* __restrict__ ph) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    nb_row<FILL>(i, qxy, rxy, rhT, ridx, start, g, geo, counts, offsets, pi, pj, pq, px, ph);
}

// The Wendland C2 kernel and gradient of one pair from its stored q, unit vector and support
__device__ __forceinline__ void pair_kernel(float qq, float x0h, float x1h, KernelCoef kc, float* W, float* G,
                                            int64_t k) {
    if (W) W[k] = wendland_w(qq, kc);
    if (G) {
        const float d = wendland_dw(qq, kc);
        G[2 * k] = x0h * d;
        G[2 * k + 1] = x1h * d;
    }
}

// The pair list by one warp per query row. The lanes test the row's stencil candidates 32 at
// a time (the exact test of the count pass, so the same pairs), the accepted ones are packed
// into the warp's shared buffer in candidate order (ballot + prefix count), each entry's rank
// among the row's reference indices gives its slot (the reference's column order, ascending
// reference index; indices are distinct within a row), and the row leaves with stores that
// cover its contiguous range of every output array, the kernel values fused in. Rows with
// more than kFillCap pairs take the one-thread path (nb_row) instead.
constexpr int kFillWarps = 8;
constexpr int kFillCap = 128;

__global__ void __launch_bounds__(32 * kFillWarps)
    k_nb_fill_warp(int64_t nq, const float2* __restrict__ qxy, const float2* __restrict__ rxy,
                   const float2* __restrict__ rhT, const int32_t* __restrict__ ridx, const int32_t* __restrict__ start,
                   Grid g, Geo geo, const int64_t* __restrict__ offsets, int64_t* __restrict__ pi,
                   int64_t* __restrict__ pj, float* __restrict__ pq, float* __restrict__ px, float* __restrict__ ph,
                   float* __restrict__ W, float* __restrict__ G) {
    __shared__ int32_t s_j[kFillWarps][kFillCap];
    __shared__ float s_q[kFillWarps][kFillCap], s_x0[kFillWarps][kFillCap], s_x1[kFillWarps][kFillCap];
    __shared__ int32_t s_sl[kFillWarps][kFillCap];  // the pair's reference slot
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t i = (int64_t)blockIdx.x * kFillWarps + wid;
    if (i >= nq) return;  // warp-uniform
    const int64_t w0 = offsets[i];
    const int cnt_row = (int)(offsets[i + 1] - w0);
    if (cnt_row > kFillCap) {
        if (lane == 0) nb_row<true>(i, qxy, rxy, rhT, ridx, start, g, geo, nullptr, offsets, pi, pj, pq, px, ph);
        __syncwarp();
        if (W || G)
            for (int e = lane; e < cnt_row; e += 32) {
                const int64_t o = w0 + e;
                const float hh = ph[o];
                pair_kernel(pq[o], px[2 * o], px[2 * o + 1], KernelCoef{kCd / (hh * hh), kCd / (hh * hh * hh)}, W,
                            G, o);
            }
        return;
    }
    const float2 p = qxy[i];
    const int cx = cell_coord(p.x, g.mn[0], g.inv_cell[0], g.nc[0]);
    const int cy = cell_coord(p.y, g.mn[1], g.inv_cell[1], g.nc[1]);
    int rows[kMaxRows], lo[2], hi[2];
    const int nr = stencil_rows(cy, g, rows);
    const int ncr = stencil_cols(cx, g, lo, hi);
    int rs[kMaxRanges], len[kMaxRanges];
    int nrg = 0, total = 0;
    for (int a = 0; a < nr; ++a)
        for (int b = 0; b < ncr; ++b) {
            const int s0 = start[rows[a] * g.nc[0] + lo[b]], s1 = start[rows[a] * g.nc[0] + hi[b] + 1];
            if (s1 > s0) {
                rs[nrg] = s0;
                len[nrg] = s1 - s0;
                total += s1 - s0;
                ++nrg;
            }
        }
    // phase 1: the exact test of every candidate is one comparison with the reference's
    // threshold (exact_T); the accepted pairs are packed with their squared distance
    int base = 0;
    int cr = 0, cbase = 0;  // the lane's current range and its first flat index (only advance)
    for (int t0 = 0; t0 < total; t0 += 32) {
        const int t = t0 + lane;
        bool acc = false;
        int jo = 0, sl = 0;
        float sq = 0.f, x0 = 0.f, x1 = 0.f;
        if (t < total) {
            while (t >= cbase + len[cr]) {
                cbase += len[cr];
                ++cr;
            }
            sl = rs[cr] + (t - cbase);
            pair_vec<true>(p, rxy[sl], geo, x0, x1);
            sq = sq_norm_ref(x0, x1);
            if (sq <= rhT[2 * sl].y) {
                acc = true;
                jo = ridx[sl];
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        if (acc && pos < kFillCap) {
            s_j[wid][pos] = jo;
            s_q[wid][pos] = sq;
            s_x0[wid][pos] = x0;
            s_x1[wid][pos] = x1;
            s_sl[wid][pos] = sl;
        }
        base += __popc(m);
    }
    __syncwarp();
    // phase 2: the accepted pairs' q and unit vector (the reference's IEEE square root and
    // divisions), every lane busy
    for (int e = lane; e < base && e < kFillCap; e += 32) {
        float rr, qq;
        exact_in(s_q[wid][e], rhT[2 * s_sl[wid][e]].x, rr, qq);
        const float den = __fadd_rn(rr, 1e-7f);
        s_q[wid][e] = qq;
        s_x0[wid][e] = __fdiv_rn(s_x0[wid][e], den);
        s_x1[wid][e] = __fdiv_rn(s_x1[wid][e], den);
    }
    __syncwarp();
    // the count pass found the same pairs (same candidates, same test); the bound only
    // keeps an inconsistent row inside its own range
    const int n_e = base < cnt_row ? base : cnt_row;
    auto put = [&](int e, int je, int rank) {
        const int64_t o = w0 + rank;
        const float q = s_q[wid][e], x0h = s_x0[wid][e], x1h = s_x1[wid][e];
        const int sl = s_sl[wid][e];
        pi[o] = i;
        pj[o] = je;
        pq[o] = q;
        px[2 * o] = x0h;
        px[2 * o + 1] = x1h;
        ph[o] = rhT[2 * sl].x;
        if (W || G) {
            const float2 c = rhT[2 * sl + 1];
            pair_kernel(q, x0h, x1h, KernelCoef{c.x, c.y}, W, G, o);
        }
    };
    // each lane ranks two entries (lane and lane + 32) in one sweep over the row's keys (rows
    // over 64 pairs take a second sweep for entries 64 on)
    for (int e0 = lane; e0 < n_e; e0 += 64) {
        const int e1 = e0 + 32;
        const int j0 = s_j[wid][e0];
        const int j1 = e1 < n_e ? s_j[wid][e1] : 0x7fffffff;
        int r0 = 0, r1 = 0;
#pragma unroll 4
        for (int k = 0; k < n_e; ++k) {
            const int v = s_j[wid][k];
            r0 += v < j0 ? 1 : 0;
            r1 += v < j1 ? 1 : 0;
        }
        put(e0, j0, r0);
        if (e1 < n_e) put(e1, j1, r1);
    }
}

// CSR only: original reference indices of each query's exact neighbors, in cell order
__global__ void k_nb_csr(int64_t nq, const float2* __restrict__ qxy, const float2* __restrict__ rxy,
                         const float2* __restrict__ rhT, const int32_t* __restrict__ ridx,
                         const int32_t* __restrict__ start, Grid g, Geo geo, const int64_t* __restrict__ offsets,
                         int32_t* __restrict__ nbr) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    float2 p = qxy[i];
    int cx = cell_coord(p.x, g.mn[0], g.inv_cell[0], g.nc[0]);
    int cy = cell_coord(p.y, g.mn[1], g.inv_cell[1], g.nc[1]);
    int rows[kMaxRows], lo[2], hi[2];
    int nr = stencil_rows(cy, g, rows);
    int ncr = stencil_cols(cx, g, lo, hi);
    int64_t w = offsets[i];
    const int64_t wend = offsets[i + 1];
    for (int a = 0; a < nr; ++a) {
        for (int b = 0; b < ncr; ++b) {
            int c0 = rows[a] * g.nc[0] + lo[b], c1 = rows[a] * g.nc[0] + hi[b];
            int s0 = start[c0], s1 = start[c1 + 1];
            for (int s = s0; s < s1; ++s) {
                float x0, x1;
                pair_vec<true>(p, rxy[s], geo, x0, x1);
                const float sq = sq_norm_ref(x0, x1);
                if (!(sq <= rhT[2 * s].y)) continue;  // exactly the reference's q <= 1 (exact_T)
                if (w < wend) nbr[w] = ridx[s];
                ++w;
            }
        }
    }
}

}  // namespace sph

using namespace sph;

extern "C" int sph_neighbor_workspace_bytes(int64_t n_query, int64_t n_ref, const sph_domain_t* domain,
                                            double max_support, size_t* bytes) {
    if (!bytes) return SPH_ERR_ARGUMENT;
    NbWork w;
    return nb_layout(n_query, n_ref, domain, max_support, nullptr, &w, bytes);
}

static int nb_prepare(const float* xq, int64_t nq, const float* xr, const float* hr, int64_t nr,
                      const sph_domain_t* d, double hmax, void* ws, size_t wsb, NbWork* w, cudaStream_t s) {
    size_t need;
    int st = nb_layout(nq, nr, d, hmax, ws, w, &need);
    if (st) return st;
    if (!ws || wsb < need) return SPH_ERR_WORKSPACE;
    if ((nq > 0 && !xq) || (nr > 0 && (!xr || !hr))) return SPH_ERR_ARGUMENT;
    unsigned gr = (unsigned)((nr + kBlock - 1) / kBlock), gq = (unsigned)((nq + kBlock - 1) / kBlock);
    if (nr > 0) k_wrap_copy<<<gr, kBlock, 0, s>>>(xr, nr, w->geo, w->ref_tmp);
    if (cell_sort((const float*)w->ref_tmp, 2, nr, w->grid, w->ncells, w->key, w->perm, w->count, w->fill,
                  w->start, w->scan32, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (nr > 0) k_ref_gather<<<gr, kBlock, 0, s>>>(nr, w->perm, w->ref_tmp, hr, w->ref_xy, w->ref_hT, w->ref_idx);
    if (nq > 0) k_wrap_copy<<<gq, kBlock, 0, s>>>(xq, nq, w->geo, w->qry_xy);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_neighbor_count(const float* x_query, int64_t n_query, const float* x_ref, const float* h_ref,
                                  int64_t n_ref, const sph_domain_t* domain, double max_support, void* workspace,
                                  size_t workspace_bytes, int32_t* counts, int64_t* offsets, sph_stream_t stream) {
    cudaStream_t s = (cudaStream_t)stream;
    NbWork w;
    int st = nb_prepare(x_query, n_query, x_ref, h_ref, n_ref, domain, max_support, workspace, workspace_bytes, &w, s);
    if (st) return st;
    if (!offsets || (n_query > 0 && !counts)) return SPH_ERR_ARGUMENT;
    if (n_query > 0)
        k_nb_query<false><<<(unsigned)((n_query + kBlock - 1) / kBlock), kBlock, 0, s>>>(
            n_query, w.qry_xy, w.ref_xy, w.ref_hT, w.ref_idx, w.start, w.grid, w.geo, counts, nullptr, nullptr,
            nullptr, nullptr, nullptr, nullptr);
    if (scan_exclusive(counts, offsets, n_query, w.scan64, s) != cudaSuccess) return SPH_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_neighbor_fill(const float* x_query, int64_t n_query, const float* x_ref, const float* h_ref,
                                 int64_t n_ref, const sph_domain_t* domain, double max_support, void* workspace,
                                 size_t workspace_bytes, const int64_t* offsets, int64_t n_pairs,
                                 int64_t* pair_i, int64_t* pair_j,
                                 float* q, float* xhat, float* h_pair, float* kernels, float* gradients,
                                 sph_stream_t stream) {
    cudaStream_t s = (cudaStream_t)stream;
    NbWork w;
    size_t need;
    int st = nb_layout(n_query, n_ref, domain, max_support, workspace, &w, &need);
    if (st) return st;
    if (!workspace || workspace_bytes < need) return SPH_ERR_WORKSPACE;
    if (!offsets || (n_pairs > 0 && (!pair_i || !pair_j || !q || !xhat || !h_pair))) return SPH_ERR_ARGUMENT;
    // the sorted reference set from sph_neighbor_count is still in the workspace
    if (n_query > 0)
        k_nb_fill_warp<<<(unsigned)((n_query + kFillWarps - 1) / kFillWarps), 32 * kFillWarps, 0, s>>>(
            n_query, w.qry_xy, w.ref_xy, w.ref_hT, w.ref_idx, w.start, w.grid, w.geo, offsets, pair_i, pair_j, q, xhat,
            h_pair, kernels, gradients);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_neighbor_fill_csr(const float* x_query, int64_t n_query, const float* x_ref, const float* h_ref,
                                     int64_t n_ref, const sph_domain_t* domain, double max_support, void* workspace,
                                     size_t workspace_bytes, const int64_t* offsets, int32_t* neighbors,
                                     sph_stream_t stream) {
    cudaStream_t s = (cudaStream_t)stream;
    NbWork w;
    size_t need;
    int st = nb_layout(n_query, n_ref, domain, max_support, workspace, &w, &need);
    if (st) return st;
    if (!workspace || workspace_bytes < need) return SPH_ERR_WORKSPACE;
    if (!offsets || (n_query > 0 && !neighbors)) return SPH_ERR_ARGUMENT;
    if (n_query > 0)
        k_nb_csr<<<(unsigned)((n_query + kBlock - 1) / kBlock), kBlock, 0, s>>>(
            n_query, w.qry_xy, w.ref_xy, w.ref_hT, w.ref_idx, w.start, w.grid, w.geo, offsets, neighbors);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// ------------------------------------------------------------------------------------
// Neighbor count without caller workspace. The scratch is one file-scope device array per
// device (the module's global, created with the module in each context); its device address
// is looked up once per device and context and cached: a new context on the device (after a
// cudaDeviceReset, the module loaded again) is noticed and the address looked up again.
// Nothing here allocates. Of the scratch, only the per-cell counters must start at zero, and
// cell_sort clears them (cudaMemsetAsync) on every call; every other region is written before
// it is read.
// ------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_nb_static_scratch[SPH_NEIGHBOR_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kStaticMaxDevices];      // device address of g_nb_static_scratch, per device
CUcontext g_static_ctx[kStaticMaxDevices];  // the context that address belongs to

PFN_cuCtxGetCurrent_v4000 ctx_get_current() {
    static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    });
    return fn;
}

int static_scratch(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return SPH_ERR_CUDA;
    if (dev < 0 || dev >= kStaticMaxDevices) return SPH_ERR_ARGUMENT;
    PFN_cuCtxGetCurrent_v4000 get = ctx_get_current();
    if (!get) return SPH_ERR_CUDA;
    CUcontext ctx = nullptr;
    void* fresh = nullptr;
    if (get(&ctx) != CUDA_SUCCESS) return SPH_ERR_CUDA;
    if (!ctx) {
        // no context current on this thread yet: the lookup binds the device's primary context
        if (cudaGetSymbolAddress(&fresh, g_nb_static_scratch) != cudaSuccess || !fresh) return SPH_ERR_CUDA;
        if (get(&ctx) != CUDA_SUCCESS || !ctx) return SPH_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev] || g_static_ctx[dev] != ctx) {
        void* p = fresh;
        if (!p && (cudaGetSymbolAddress(&p, g_nb_static_scratch) != cudaSuccess || !p)) return SPH_ERR_CUDA;
        g_static_ptr[dev] = p;
        g_static_ctx[dev] = ctx;
    }
    *out = g_static_ptr[dev];
    return SPH_OK;
}
}  // namespace

extern "C" int sph_neighbor_count_static(const float* x_query, int64_t n_query, const float* x_ref,
                                         const float* h_ref, int64_t n_ref, const sph_domain_t* domain,
                                         double max_support, int32_t* counts, int64_t* offsets,
                                         sph_stream_t stream) {
    NbWork w;
    size_t need = 0;
    int st = nb_layout(n_query, n_ref, domain, max_support, nullptr, &w, &need);
    if (st) return st;
    if (need > SPH_NEIGHBOR_STATIC_SCRATCH_BYTES) return SPH_ERR_STATIC_LIMIT;
    void* scratch = nullptr;
    if ((st = static_scratch(&scratch))) return st;
    return sph_neighbor_count(x_query, n_query, x_ref, h_ref, n_ref, domain, max_support, scratch,
                              SPH_NEIGHBOR_STATIC_SCRATCH_BYTES, counts, offsets, stream);
}
