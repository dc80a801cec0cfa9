// Fused delta-SPH time step for sm_103a.
//
// One step reproduces the reference runner (src/diffSPH/v2/runner.py:37-42):
//   integrate(simulationStep) with scheme symplecticEuler (modules/integration.py:357-392),
//   then solveShifting (modules/shifting.py:882-1019, delta+ branch, one iteration).
//
// Data layout (structure of arrays, particles in cell-sorted order, re-sorted every step or,
// under Verlet reuse, when a particle moved 0.034 h since the last sort):
//   Xr[n]  float2  raw positions (never wrapped, like the reference state)
//   Xs[n]  float2  raw positions at the last sort
//   X4[n]  float4  (wrapped x, wrapped y, rho, p); rho carries the sign bit for boundary
//                  particles (-rho), so a neighbor's kind costs no extra load
//   V4[n]  float4  (u, v, gradRho^L x, gradRho^L y)
// Neighbor passes walk the 5x5 half-cell stencil of every particle over the sorted arrays,
// keep the exact neighbors (the reference's fp32 test) in a per-warp shared-memory list and
// evaluate the pair terms over it. The first pass A after a sort also stores the skin list
// (candidates within 1.1 h) that the later passes filter until the next sort, and every
// pass A stores its exact list for the pass B that follows. Per step:
//   displacement check -> sort by cell -> gather (the last two only when sorting)
//   stage 1: mDBC ghosts -> pass A -> pass B (+ half-step update)
//   stage 2: mDBC ghosts -> pass A -> pass B (+ final update, max |u|)
//   shift pass (+ position update)
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/sph103.h"
#include "sph_internal.cuh"
#include "sph_solver.cuh"

namespace sph {


// ------------------------------------------------------------------------------------
// upload / download / gather
// ------------------------------------------------------------------------------------
__global__ void k_upload(int64_t nF, int64_t nB, const float* __restrict__ xf, const float* __restrict__ uf,
                         const float* __restrict__ rf, const float* __restrict__ xb, const float* __restrict__ nb,
                         const float* __restrict__ db, const float* __restrict__ rb, const Dom* __restrict__ doms,
                         const int64_t* __restrict__ dom_off, int nd, float2* Xr, float4* X4, float4* V4,
                         int32_t* uid, int32_t* slot, int32_t* did, float2* bnormal, float* bdist) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nF + nB) return;
    // domain of fluid particle i: dom_off[d] <= i < dom_off[d + 1]; boundaries belong to domain 0
    int d = 0;
    if (i < nF) {
        int lo = 0, hi = nd - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (dom_off[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        d = lo;
    }
    did[i] = d;
    const Phys& P = doms[d].P;
    float2 x;
    float2 u = make_float2(0.f, 0.f);
    float rho, rho_s;
    if (i < nF) {
        x = make_float2(xf[2 * i], xf[2 * i + 1]);
        u = make_float2(uf[2 * i], uf[2 * i + 1]);
        rho = rf[i];
        rho_s = rho;
    } else {
        int64_t b = i - nF;
        x = make_float2(xb[2 * b], xb[2 * b + 1]);
        rho = rb ? rb[b] : P.rho0;
        rho_s = -rho;
        bnormal[b] = make_float2(nb[2 * b], nb[2 * b + 1]);
        bdist[b] = db[b];
    }
    Xr[i] = x;
    float2 w = wrap_pos(x, P.geo);
    X4[i] = make_float4(w.x, w.y, rho_s, eos_p(rho, P.eos));
    V4[i] = make_float4(u.x, u.y, 0.f, 0.f);
    uid[i] = (int32_t)i;
    slot[i] = (int32_t)i;
}

// Element o of a caller's [n][2] float array: one 8-byte access when the array is 8-byte
// aligned (the same for every thread), so a warp's accesses fill whole lines of host memory
__device__ __forceinline__ float2 ld_pair(const float* a, int64_t o) {
    if ((reinterpret_cast<uintptr_t>(a) & 7u) == 0) return reinterpret_cast<const float2*>(a)[o];
    return make_float2(a[2 * o], a[2 * o + 1]);
}
__device__ __forceinline__ void st_pair(float* a, int64_t o, float2 v) {
    if ((reinterpret_cast<uintptr_t>(a) & 7u) == 0) {
        reinterpret_cast<float2*>(a)[o] = v;
    } else {
        a[2 * o] = v.x;
        a[2 * o + 1] = v.y;
    }
}

// Upload into the current slot order (Verlet reuse): particle o's state goes to its slot
// slot[o]; the sort words are left as they are, so the next step's displacement check decides.
// The threads run over the original order, so the caller's arrays are read contiguously: they
// may be page-locked host memory, which the kernel then reads over the host link itself.
__global__ void k_upload_keep(int64_t n, int64_t nF, const int32_t* __restrict__ slot, const float* __restrict__ xf,
                              const float* __restrict__ uf, const float* __restrict__ rf,
                              const float* __restrict__ xb, const float* __restrict__ nb,
                              const float* __restrict__ db, const float* __restrict__ rb, Phys P, float2* Xr,
                              float4* X4, float4* V4, float2* bnormal, float* bdist) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int64_t s = slot[o];
    float2 x, u = make_float2(0.f, 0.f);
    float rho, rho_s;
    if (o < nF) {
        x = ld_pair(xf, o);
        u = ld_pair(uf, o);
        rho = rf[o];
        rho_s = rho;
    } else {
        const int64_t b = o - nF;
        x = make_float2(xb[2 * b], xb[2 * b + 1]);
        rho = rb ? rb[b] : P.rho0;
        rho_s = -rho;
        bnormal[b] = make_float2(nb[2 * b], nb[2 * b + 1]);
        bdist[b] = db[b];
    }
    Xr[s] = x;
    const float2 w = wrap_pos(x, P.geo);
    X4[s] = make_float4(w.x, w.y, rho_s, eos_p(rho, P.eos));
    V4[s] = make_float4(u.x, u.y, 0.f, 0.f);
}

// The state in the original order (particle o from its slot): the threads run over the
// original order, so the caller's arrays are written contiguously (page-locked host memory
// included, written over the host link by the kernel itself)
__global__ void k_download(int64_t n, int nF, const int32_t* __restrict__ slot, const float2* __restrict__ Xr,
                           const float4* __restrict__ X4, const float4* __restrict__ V4, float* xf, float* uf,
                           float* rf, float* rb) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int s = slot[o];
    if (o < nF) {
        const float4 v = V4[s];
        if (xf) st_pair(xf, o, Xr[s]);
        if (uf) st_pair(uf, o, make_float2(v.x, v.y));
        if (rf) rf[o] = X4[s].z;
    } else if (rb) {
        rb[o - nF] = fabsf(X4[s].z);
    }
}

__global__ void k_gather(int64_t n, int nF, const int32_t* __restrict__ perm, const float2* __restrict__ Xr_in,
                         const float4* __restrict__ X4_in, const float4* __restrict__ V4_in,
                         const int32_t* __restrict__ uid_in, const int32_t* __restrict__ did_in,
                         float2* __restrict__ Xr_out, float4* __restrict__ X4_out, float4* __restrict__ V4_out,
                         int32_t* __restrict__ uid_out, int32_t* __restrict__ did_out, int32_t* __restrict__ bidx,
                         uint32_t* __restrict__ words, float2* __restrict__ Xs, int32_t* __restrict__ slot,
                         const uint32_t* __restrict__ gate) {
    if (gate && *gate == 0u) return;
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int o = perm[s];
    const float2 xo = Xr_in[o];
    Xr_out[s] = xo;
    Xs[s] = xo;
    X4_out[s] = X4_in[o];
    V4_out[s] = V4_in[o];
    did_out[s] = did_in[o];
    int u = uid_in[o];
    uid_out[s] = u;
    slot[u] = (int32_t)s;
    if (u >= nF) bidx[atomicAdd(&words[2], 1u)] = (int32_t)s;
}

// Verlet reuse: the gathered state goes back into the current buffers (the assignment of
// buffers stays fixed, so steps that keep the sort need no copy at all)
__global__ void k_copy_back(int64_t n, const float2* __restrict__ Xr_t, const float4* __restrict__ Xt,
                            const float4* __restrict__ Vt, const int32_t* __restrict__ uid_t,
                            const int32_t* __restrict__ did_t, float2* __restrict__ Xr, float4* __restrict__ Xc,
                            float4* __restrict__ Vc, int32_t* __restrict__ uid, int32_t* __restrict__ did,
                            const uint32_t* __restrict__ gate) {
    if (*gate == 0u) return;
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    Xr[s] = Xr_t[s];
    Xc[s] = Xt[s];
    Vc[s] = Vt[s];
    uid[s] = uid_t[s];
    did[s] = did_t[s];
}

// Verlet reuse: words[4] (sort this step) is set when a particle moved farther than lim since
// the last sort, or when the skin list of that sort went invalid (words[3]). In a packed
// batch (did != nullptr) the limit is each domain's: min(half h, 0.7 skin_lim).
__global__ void k_verlet_check(int64_t n, const float2* __restrict__ Xr, const float2* __restrict__ Xs,
                               uint32_t* __restrict__ words, float lim2, const Dom* __restrict__ doms,
                               const int32_t* __restrict__ did, float half) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool far = false;
    if (i < n) {
        const float2 a = Xr[i], b = Xs[i];
        const float e0 = a.x - b.x, e1 = a.y - b.y;
        float l2 = lim2;
        if (did) {
            const Phys& P = doms[did[i]].P;
            const float lim = fminf(half * P.h, 0.7f * P.skin_lim);
            l2 = lim * lim;
        }
        far = e0 * e0 + e1 * e1 > l2;
    }
    if (i == 0 && words[3] != 0u) far = true;
    if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicOr(&words[4], 1u);
}

// start of a sort: reset the gather's boundary count, count the sort, and mark the skin list
// valid when the caller's first pass A rebuilds it for this sort (invalid otherwise: it
// belongs to an earlier order)
__global__ void k_sort_begin(uint32_t* words, int skin_rebuilt) {
    if (threadIdx.x == 0 && words[4] != 0u) {
        words[2] = 0u;
        words[3] = skin_rebuilt ? 0u : 1u;
        words[5] += 1u;
    }
}

// ------------------------------------------------------------------------------------
// mDBC boundary density (src/diffSPH/v2/modules/mDBC.py:9-36 ghosts, :50-163 density)
// ------------------------------------------------------------------------------------
// Two kernels: one warp per wall particle sums the 13 moments of its ghost, its lanes
// striding over the candidates of all stencil ranges (a fixed shuffle tree combines them);
// then one thread per wall particle solves the fp64 3x3 system, 32 wall particles per warp.
constexpr int kMdbcSolveBlock = 64;  // threads per block of the fp64 solve (one wall each)
constexpr int kMdbcSums = 16;  // 13 used: num, den, gs0, gs1, vg0, vg1, ps0, ps1, pm00, pm01, pm10, pm11, count

__device__ __forceinline__ float2 mdbc_ghost(const Phys& P, float2 xb, float2 nrm, float d) {
    // mappingDistance = d + max(d, -h); ghost = x_b + mappingDistance * n
    float mapd = __fadd_rn(d, fmaxf(d, -P.h));
    return make_float2(__fadd_rn(xb.x, __fmul_rn(mapd, nrm.x)), __fadd_rn(xb.y, __fmul_rn(mapd, nrm.y)));
}

// The 13 moments of one ghost over the fluid candidates of its cell stencil, lane-strided
// over the flat candidate index with a fixed xor-shuffle tree: every lane of the warp ends
// with the totals (k_mdbc_sums and its adjoint k_mdbc_vjp sum in exactly this order).
template <bool PER>
__device__ __forceinline__ void mdbc_moments(const Phys& P, float2 gw, const int* rs, const int* re, int nr,
                                             const float4* __restrict__ X4, int lane, float acc[13]) {
    int total = 0;
    for (int a = 0; a < nr; ++a) total += re[a] - rs[a];
#pragma unroll
    for (int q = 0; q < 13; ++q) acc[q] = 0.f;
    int r = 0, base = 0;  // range of the lane's current flat index and the flat start of that range
    for (int t = lane; t < total; t += 32) {
        while (t >= base + (re[r] - rs[r])) {
            base += re[r] - rs[r];
            ++r;
        }
        const int j = rs[r] + (t - base);
        const float4 xj = __ldg(&X4[j]);
        if (is_boundary(xj.z)) continue;
        float x0, x1;
        pair_vec<PER>(gw, make_float2(xj.x, xj.y), P.geo, x0, x1);
        const float sq = sq_norm_ref(x0, x1);
        if (sq > P.T) continue;
        const PairG pg = pair_fast(x0, x1, sq, P.inv_h);
        const float W = wendland_w(pg.q, P.kc);
        const float dW = wendland_dw(pg.q, P.kc);
        const float g0 = pg.xh0 * dW, g1 = pg.xh1 * dW;
        const float V = P.m / xj.z;
        const float k0 = V * g0, k1 = V * g1;
        const float xr = -pg.q * P.h;
        const float xi0 = pg.xh0 * xr, xi1 = pg.xh1 * xr;
        const float vw = V * W;
        acc[0] += P.m * W;
        acc[1] += vw;
        acc[2] += xj.z * k0;
        acc[3] += xj.z * k1;
        acc[4] += k0;
        acc[5] += k1;
        acc[6] += xi0 * vw;
        acc[7] += xi1 * vw;
        acc[8] += xi0 * k0;
        acc[9] += xi0 * k1;
        acc[10] += xi1 * k0;
        acc[11] += xi1 * k1;
        acc[12] += 1.f;
    }
#pragma unroll
    for (int q = 0; q < 13; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(kFull, acc[q], o);
    }
}

template <bool PER>
__global__ void __launch_bounds__(128) k_mdbc_sums(int nB, const int32_t* __restrict__ bidx,
                                                   const int32_t* __restrict__ uid, const float2* __restrict__ Xr,
                                                   const float4* __restrict__ X4, const float2* __restrict__ bnormal,
                                                   const float* __restrict__ bdist,
                                                   const int32_t* __restrict__ start, Grid g, Phys P,
                                                   float* __restrict__ sums) {
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= nB) return;  // warp-uniform
    const int s = bidx[k];
    const int b = uid[s] - P.nF;
    const float2 gp = mdbc_ghost(P, Xr[s], bnormal[b], bdist[b]);
    const float2 gw = wrap_pos(gp, P.geo);
    int rs[kMaxRanges], re[kMaxRanges];
    const int nr = stencil_ranges(gw, g, start, rs, re);
    float acc[13];
    mdbc_moments<PER>(P, gw, rs, re, nr, X4, lane, acc);
    if (lane < 13) {
        float v = acc[0];
#pragma unroll
        for (int q = 1; q < 13; ++q)
            if (lane == q) v = acc[q];
        sums[(int64_t)k * kMdbcSums + lane] = v;
    }
}

__global__ void k_mdbc_solve(int nB, const int32_t* __restrict__ bidx, const int32_t* __restrict__ uid,
                             const float2* __restrict__ Xr, float4* X4, const float2* __restrict__ bnormal,
                             const float* __restrict__ bdist, Phys P, const float* __restrict__ sums,
                             float* __restrict__ rho_b_out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nB) return;
    const int s = bidx[k];
    const int b = uid[s] - P.nF;
    const float2 xb = Xr[s];
    const float2 gp = mdbc_ghost(P, xb, bnormal[b], bdist[b]);
    const float* a = sums + (int64_t)k * kMdbcSums;
    const float num = a[0], den = a[1], gs0 = a[2], gs1 = a[3];
    const int cnt = (int)a[12];
    float rho;
    if (cnt > 5) {
        double A[9] = {den, a[6], a[7], a[4], a[8], a[9], a[5], a[10], a[11]};
        double Pi[9];
        pinv3_f64(A, Pi, 3.0 * 1.1920928955078125e-07);
        double r0 = Pi[0] * num + Pi[1] * gs0 + Pi[2] * gs1;
        double r1 = Pi[3] * num + Pi[4] * gs0 + Pi[5] * gs1;
        double r2 = Pi[6] * num + Pi[7] * gs0 + Pi[8] * gs1;
        float rel0 = __fsub_rn(xb.x, gp.x), rel1 = __fsub_rn(xb.y, gp.y);
        rho = (float)(r0 + (double)rel0 * r1 + (double)rel1 * r2);
    } else if (cnt > 0) {
        rho = num / (den + 1e-7f);
    } else {
        rho = P.rho0;
    }
    X4[s].z = -rho;  // boundary particles carry the sign bit
    X4[s].w = eos_p(rho, P.eos);
    if (rho_b_out) rho_b_out[b] = rho;
}

// ------------------------------------------------------------------------------------
// Pass A: normalisation matrix, its pseudo-inverse and the renormalised density gradient
//   M_i = sum_j (-r x_ij) (m_j/rho_j gradW)       (normalizationMatrices.py:18-23, fluid + boundary)
//   M_i = I where the fluid neighbor count < 4; L_i = pinv2x2(M_i)  (deltaPlus.py:240-252)
//   gradRho^L_i = L_i sum_fluid (rho_i - rho_j) V_j gradW + sum_boundary (rho_i - rho_j) V_j gradW
//                                                 (densityDiffusion.py:7-46, deltaPlus.py:256-262)
// The uniform mass m is factored out of the sums.
// ------------------------------------------------------------------------------------
template <bool PER, bool BATCH, typename LT, bool BUILD>
__device__ __forceinline__ void pass_a_tile(const Dom& D0, int64_t i, int64_t n, const float4* __restrict__ X4,
                                            float4* __restrict__ V4, const int32_t* __restrict__ start_all,
                                            const Dom* __restrict__ doms, const Dom* s_dom, const int* s_id,
                                            const int32_t* __restrict__ did,
                                            const int32_t* __restrict__ uid, const RhsOut& out,
                                            LT* __restrict__ lst, uint32_t* __restrict__ words,
                                            int16_t* __restrict__ nl, int16_t* __restrict__ nlc,
                                            int skin_mode, int16_t* __restrict__ sl, int16_t* __restrict__ slc) {
    const Dom& D = BATCH ? dom_ref(doms, s_dom, s_id, dom_of(did, i, n)) : D0;
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int32_t* __restrict__ start = start_all + D.cell0;
    bool inb = i < n;
    float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, -1.f, 0.f);
    bool active = inb && !is_boundary(xi.z);
    float2 pi = make_float2(xi.x, xi.y);
    float rhoi = xi.z;
    float2 M0 = make_float2(0.f, 0.f);  // (M00, M01)
    float M11 = 0.f;
    float2 gfv = make_float2(0.f, 0.f), gbv = make_float2(0.f, 0.f);
    int nf = 0, nbnd = 0;
    int nstored = 0;
    bool unstored = false;
    const float cg20 = -20.0f * P.kc.cg;
    int16_t* __restrict__ nrow = nl + tile_row(i, kStoreCap);
    // wrap flags of the row (neighbor_loop / row_count): the pairs take the minimum image only
    // in a warp with a row whose stencil may wrap (set before the first pair)
    int wf = 3;
    auto pair_a = [&](int j) {
        {  // keep the exact list (scan order) for pass B at the same positions (offsets of a
           // row that may wrap modulo the domain's slots, of any other row direct)
            int d = j - (int)i;
            if (PER && (wf & 1)) {
                const int h2 = g.nslots >> 1;
                if (d > h2) d -= g.nslots;
                else if (d < -h2) d += g.nslots;
            }
            if (nstored < kStoreCap && d >= -32768 && d <= 32767)
                nrow[nstored * 32] = (int16_t)d;
            else
                unstored = true;
            ++nstored;
        }
        const float4 xj = __ldg(&X4[j]);
        float2 xv;
        if (PER && (wf & 2)) {
            pair_vec<true>(pi, make_float2(xj.x, xj.y), P.geo, xv.x, xv.y);
        } else {
            xv = __ffma2_rn(make_float2(xj.x, xj.y), make_float2(-1.f, -1.f), pi);
        }
        const float x0 = xv.x, x1 = xv.y;
        const PairR pr = pair_r(x0, x1, P.inv_h);
        const float om = fmaxf(1.0f - pr.q, 0.0f);
        const float rj = fabsf(xj.z);
        // gradW / rho_j = x w
        const float w = wendland_gf(pr, om, cg20) * __fdividef(1.0f, rj);
        // (-r xhat) (x) (gradW / rho_j) = c x x^T: the matrix is symmetric
        const float c = -(pr.r * pr.inv) * w;
        const float t0 = c * x0;
        M0 = __ffma2_rn(make_float2(t0, t0), xv, M0);
        M11 = fmaf(c * x1, x1, M11);
        const float dw = (rhoi - rj) * w;
        if (is_boundary(xj.z)) {
            gbv = __ffma2_rn(make_float2(dw, dw), xv, gbv);
            ++nbnd;
        } else {
            gfv = __ffma2_rn(make_float2(dw, dw), xv, gfv);
            ++nf;
        }
    };
    // BUILD (first pass A after a sort): scan the stencil and keep every candidate within
    // the skin radius. Otherwise skin_mode 1 filters the skin list when it is complete for
    // every lane of the warp (no overflow, displacements within skin_lim) and skin_mode 2
    // scans.
    if (BUILD) {
        // the scan's list holds the skin candidates; each flush stores them (lanes flush their
        // k-th entries together, so the stores coalesce) and passes the exact ones on, in
        // scan order. The offsets of a row that may wrap are stored modulo the domain's slots
        // (its count carries kRowWraps), those of any other row direct.
        int ns = 0;
        bool sbad = false;
        int16_t* __restrict__ srow = sl + tile_row(i, kSkinCap);
        auto skin_then_exact = [&](int j) {
            int d = j - (int)i;
            if (PER && (wf & 1)) {
                const int h2 = g.nslots >> 1;
                if (d > h2) d -= g.nslots;
                else if (d < -h2) d += g.nslots;
            }
            if (ns < kSkinCap && d >= -32768 && d <= 32767)
                srow[ns * 32] = (int16_t)d;
            else
                sbad = true;
            ++ns;
            float x0, x1;
            if (PER && (wf & 2))
                pair_vec<true>(pi, ldg_xy(X4, j), P.geo, x0, x1);
            else
                pair_vec<false>(pi, ldg_xy(X4, j), P.geo, x0, x1);
            if (sq_norm_ref(x0, x1) <= P.T) pair_a(j);
        };
        neighbor_loop<PER, LT, decltype(skin_then_exact)&, true>(active, (int)i, pi, X4, start, g, P, lst, words,
                                                                 skin_then_exact, &wf);
        if (inb) slc[i] = active ? (sbad ? (int16_t)-1 : stored_count(ns, wf)) : (int16_t)0;
    } else {
        const int sraw = (skin_mode == 1 && active) ? (int)slc[i] : 0;
        const int sk = row_count(sraw, wf);
        const bool use_skin = skin_mode == 1 && __all_sync(kFull, sk >= 0) && words[3] == 0u;
        if (use_skin) {
            if (PER && (wf & 2))
                skin_list_loop<PER, PER, LT, decltype(pair_a)&, !BATCH>((int)i, pi, X4, g, P, sl, sk, lst, pair_a);
            else
                skin_list_loop<PER, false, LT, decltype(pair_a)&, !BATCH>((int)i, pi, X4, g, P, sl, sk, lst, pair_a);
        } else {
            neighbor_loop<PER, LT>(active, (int)i, pi, X4, start, g, P, lst, words, pair_a, &wf);
        }
    }
    if (inb) nlc[i] = active ? (unstored ? (int16_t)-1 : stored_count(nstored, wf)) : (int16_t)0;
    if (!active) return;
    float M00 = M0.x, M01 = M0.y;
    const float gf0 = gfv.x, gf1 = gfv.y, gb0 = gbv.x, gb1 = gbv.y;
    float m = P.m;
    if (nf < 4) {
        M00 = 1.f; M01 = 0.f; M11 = 1.f;
    } else {
        M00 *= m; M01 *= m; M11 *= m;
    }
    M2 L = pinv2x2_ref(M00, M01, M01, M11);
    float g0 = m * (L.a * gf0 + L.b * gf1 + gb0);
    float g1 = m * (L.c * gf0 + L.d * gf1 + gb1);
    *reinterpret_cast<float2*>(&V4[i].z) = make_float2(g0, g1);
    if (out.grad || out.L || out.nn) {
        int o = uid[i];
        if (out.nn) { out.nn[2 * o] = nf; out.nn[2 * o + 1] = nbnd; }
        if (out.grad) { out.grad[2 * o] = g0; out.grad[2 * o + 1] = g1; }
        if (out.L) { out.L[4 * o] = L.a; out.L[4 * o + 1] = L.b; out.L[4 * o + 2] = L.c; out.L[4 * o + 3] = L.d; }
    }
}

// One block handles 32 W consecutive slots: its warps sit in neighboring cells and share
// most of their stencil data in L1.

template <bool PER, bool BATCH, typename LT, int W, bool BUILD, bool PERSIST>
__global__ void __launch_bounds__(32 * W) k_pass_a(const Dom D0, int64_t n, const float4* __restrict__ X4,
                                                   float4* __restrict__ V4, const int32_t* __restrict__ start,
                                                   const Dom* __restrict__ doms, const int32_t* __restrict__ did,
                                                   const int32_t* __restrict__ uid, RhsOut out,
                                                   uint32_t* __restrict__ words, int16_t* __restrict__ nl,
                                                   int16_t* __restrict__ nlc, int skin_mode, int16_t* __restrict__ sl,
                                                   int16_t* __restrict__ slc) {
    // skin_mode 3 / 4: the first pass A of a step under Verlet reuse, launched both ways; 3
    // runs (as 0: scan, keep the skin list) after a sort, 4 (as 1: filter it) otherwise
    if (skin_mode >= 3) {
        if ((words[4] != 0u) != (skin_mode == 3)) return;
        skin_mode -= 3;
    }
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ Dom s_dom[BATCH ? 2 : 1];
    __shared__ int s_id[2];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    run_tiles<BATCH, W, PERSIST>(n, doms, did, s_dom, s_id, [&](int64_t first) {
        pass_a_tile<PER, BATCH, LT, BUILD>(D0, first + threadIdx.x, n, X4, V4, start, doms, s_dom, s_id, did, uid,
                                           out, lst, words, nl, nlc, skin_mode, sl, slc);
    });
}

// ------------------------------------------------------------------------------------
// Pass B: rates of one right-hand side and the fused integrator stage.
//   continuity   -sum m_j (u_j - u_i).gradW rho_i/rho_j          (momentumEquation.py:6-39)
//   diffusion    delta h/kappa cs sum psi_ij . V_j gradW (fluid)   (densityDiffusion.py:49-73)
//   pressure     -(1/rho_i) sum (p_i + p_j) V_j gradW              (pressureForce.py:10-12)
//   viscosity    c/rho_i sum V_j pi_ij gradW                       (viscosity.py:123-218,
//                                                                   boundaryViscosity.py:123-219)
//   gravity                                                        (gravity.py:8-29)
// MODE 0: write the rates (original order); 1: half step (integration.py:23-32);
// MODE 2: final symplectic Euler update (integration.py:381-392, 439-513).
// ------------------------------------------------------------------------------------
template <bool PER, bool BATCH, int MODE, typename LT>
__device__ __forceinline__ void pass_b_tile(const Dom& D0, int64_t i, int64_t n, const float4* __restrict__ X4,
                                            const float4* __restrict__ V4, const int32_t* __restrict__ start_all,
                                            const Dom* __restrict__ doms, const Dom* s_dom, const int* s_id,
                                            const int32_t* __restrict__ did,
                                            const int32_t* __restrict__ uid, const RhsOut& out,
                                            float2* __restrict__ Xr, const float4* __restrict__ X4n,
                                            const float4* __restrict__ V4n, float4* __restrict__ X4o,
                                            float4* __restrict__ V4o, uint32_t* __restrict__ words,
                                            uint32_t* __restrict__ maxv, LT* __restrict__ lst,
                                            const int16_t* __restrict__ nl, const int16_t* __restrict__ nlc,
                                            const float2* __restrict__ Xs) {
    const int dom = BATCH ? dom_of(did, i, n) : 0;
    const Dom& D = BATCH ? dom_ref(doms, s_dom, s_id, dom) : D0;
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int32_t* __restrict__ start = start_all + D.cell0;
    bool inb = i < n;
    float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, -1.f, 0.f);
    float4 vi = inb ? V4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    bool active = inb && !is_boundary(xi.z);
    float2 pi = make_float2(xi.x, xi.y);
    float rhoi = xi.z, pri = xi.w;
    float ac = 0.f, ad = 0.f;
    float2 apv = make_float2(0.f, 0.f), avv = make_float2(0.f, 0.f), abv = make_float2(0.f, 0.f);
    const float cg20 = -20.0f * P.kc.cg;
    int wf = 3;  // wrap flags of the row (pass A's stored count, or the fallback scan)
    // gradW = gf x_ij with gf = dW/dr / (r + 1e-7) (wendland_gf); xhat = x_ij inv. The
    // x/y pairs use sm_100's packed fp32 operations (__ffma2_rn, __fadd2_rn; a - b as
    // fma(b, -1, a)): each component rounds exactly as the scalar operation, so the sums are
    // bit-identical to scalar code, with 7 % fewer instructions in this pass.
    auto pair_b = [&](int j) {
        const float4 xj = __ldg(&X4[j]);
        const float4 vj = __ldg(&V4[j]);
        float2 xv;
        if (PER && (wf & 2)) {
            pair_vec<true>(pi, make_float2(xj.x, xj.y), P.geo, xv.x, xv.y);
        } else {
            xv = __ffma2_rn(make_float2(xj.x, xj.y), make_float2(-1.f, -1.f), pi);
        }
        const float x0 = xv.x, x1 = xv.y;
        const PairR pr = pair_r(x0, x1, P.inv_h);
        const float om = fmaxf(1.0f - pr.q, 0.0f);
        const float gf = wendland_gf(pr, om, cg20);
        const float rj = fabsf(xj.z);
        const float irj = __fdividef(1.0f, rj);
        // (u_j - u_i) . x_ij
        const float2 dv = __ffma2_rn(make_float2(vi.x, vi.y), make_float2(-1.f, -1.f), make_float2(vj.x, vj.y));
        const float dux = fmaf(dv.y, x1, dv.x * x0);
        // continuity: sum (u_j - u_i).gradW / rho_j          (x -m rho_i below)
        ac = fmaf(gf * dux, irj, ac);
        // pressure: sum (p_i + p_j) / rho_j gradW            (x -m / rho_i below)
        const float pp = (pri + xj.w) * irj * gf;
        apv = __ffma2_rn(make_float2(pp, pp), xv, apv);
        // viscosity: pi_ij = (u_i - u_j).xhat / (r + eps h^2) = -dux inv / (r + eps h^2)
        const float vr = -dux * pr.inv;
        if (is_boundary(xj.z)) {
            const float piv = __fdividef(vr, pr.r + P.bv_eps);
            const float w = (P.bvisc ? __fdividef(piv, rhoi + rj) : piv * irj) * gf;
            abv = __ffma2_rn(make_float2(w, w), xv, abv);
        } else {
            const float w = __fdividef(vr, pr.r + P.v_eps) * irj * gf;
            avv = __ffma2_rn(make_float2(w, w), xv, avv);
            // delta-SPH density diffusion: psi = -2 (rho_j - rho_i)/(r + 1e-6 h) xhat + (gradRho_i + gradRho_j);
            // psi . gradW = gf (-2 (rho_j - rho_i)/(r + 1e-6 h) inv sq + (G_i + G_j) . x_ij)
            const float rij = __fdividef(2.f * (rj - rhoi), pr.r + P.diff_eps);
            const float2 gs = __fadd2_rn(make_float2(vi.z, vi.w), make_float2(vj.z, vj.w));
            const float gx = fmaf(gs.y, x1, gs.x * x0);
            ad = fmaf(gf * fmaf(-rij * pr.inv, pr.sq, gx), irj, ad);
        }
    };
    // the exact list pass A stored at these positions (same scan order, so the same sums);
    // a warp with a row that could not be stored scans the stencil itself
    const int nst = row_count(active ? (int)nlc[i] : 0, wf);
    if (__any_sync(kFull, nst < 0)) {
        neighbor_loop<PER, LT>(active, (int)i, pi, X4, start, g, P, lst, words, pair_b, &wf);
    } else {
        const int16_t* __restrict__ row = nl + tile_row(i, kStoreCap);
        // the modular slot arithmetic only in a warp with a row that may wrap (the other rows'
        // offsets are direct: the modular form leaves them as they are)
        // the next group's entries are loaded before this group's pairs, so their latency
        // (the list is read once, mostly from DRAM) hides behind the pair terms
        auto walk = [&](auto wr) {
            constexpr bool WR = decltype(wr)::value;
            int k = 0;
            int n0 = 0, n1 = 0, n2 = 0, n3 = 0;
            if (nst >= 4) {
                n0 = row[0];
                n1 = row[32];
                n2 = row[64];
                n3 = row[96];
            }
            for (; k + 4 <= nst; k += 4) {
                const int d0 = n0, d1 = n1, d2 = n2, d3 = n3;
                if (k + 8 <= nst) {
                    n0 = row[(k + 4) * 32];
                    n1 = row[(k + 5) * 32];
                    n2 = row[(k + 6) * 32];
                    n3 = row[(k + 7) * 32];
                }
                pair_b(list_slot<WR>((int)i, d0, g));
                pair_b(list_slot<WR>((int)i, d1, g));
                pair_b(list_slot<WR>((int)i, d2, g));
                pair_b(list_slot<WR>((int)i, d3, g));
            }
            for (; k < nst; ++k) pair_b(list_slot<WR>((int)i, (int)row[k * 32], g));
        };
        if (PER && (wf & 2))
            walk(std::integral_constant<bool, PER>{});
        else
            walk(std::integral_constant<bool, false>{});
    }
    if (!inb) return;
    if (!active) {  // boundary rows: static, carried over to the next stage
        if (MODE != 0) {
            X4o[i] = xi;
            V4o[i] = vi;
        }
        return;
    }
    const float ap0 = apv.x, ap1 = apv.y, av0 = avv.x, av1 = avv.y, ab0 = abv.x, ab1 = abv.y;
    float m = P.m;
    float irhoi = 1.0f / rhoi;
    float du0 = (-m * ap0 * irhoi + P.gx) + (P.v_num * irhoi * m * av0 + P.bv_num * irhoi * m * ab0);
    float du1 = (-m * ap1 * irhoi + P.gy) + (P.v_num * irhoi * m * av1 + P.bv_num * irhoi * m * ab1);
    float drho = -m * rhoi * ac + P.diff_coef * m * ad;
    if (MODE == 0) {
        int o = uid[i];
        out.dudt[2 * o] = du0;
        out.dudt[2 * o + 1] = du1;
        out.drhodt[o] = drho;
        if (out.pressure) out.pressure[o] = pri;
        return;
    }
    float2 x = Xr[i];
    if (MODE == 1) {
        // updateStates(dt/2): x += u dt/2, u += dudt dt/2, rho += drhodt dt/2
        float2 xh = make_float2(__fadd_rn(x.x, __fmul_rn(vi.x, P.dth)), __fadd_rn(x.y, __fmul_rn(vi.y, P.dth)));
        float u0 = __fadd_rn(vi.x, __fmul_rn(du0, P.dth)), u1 = __fadd_rn(vi.y, __fmul_rn(du1, P.dth));
        float rh = __fadd_rn(rhoi, __fmul_rn(drho, P.dth));
        float2 w = wrap_pos(xh, P.geo);
        X4o[i] = make_float4(w.x, w.y, rh, eos_p(rh, P.eos));
        V4o[i] = make_float4(u0, u1, 0.f, 0.f);
        {  // the second pass A filters the skin list at these positions
            const float2 xs = Xs[i];
            const float e0 = xh.x - xs.x, e1 = xh.y - xs.y;
            if (e0 * e0 + e1 * e1 > P.skin_lim * P.skin_lim) atomicOr(&words[3], 1u);
        }
    } else {
        // v' = v + dudt dt; x' = x + 0.5 (v + v') dt; rho' per density_update
        float4 vn = V4n[i];
        float4 xn = X4n[i];
        float u0 = __fadd_rn(vn.x, __fmul_rn(du0, P.dt)), u1 = __fadd_rn(vn.y, __fmul_rn(du1, P.dt));
        float d0 = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(vn.x, u0)), P.dt);
        float d1 = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(vn.y, u1)), P.dt);
        float2 xp = make_float2(__fadd_rn(x.x, d0), __fadd_rn(x.y, d1));
        float rnew;
        if (P.density_update == 0) {
            rnew = rhoi;  // the half-step density (the reference's observable update)
        } else {
            float eps = __fdiv_rn(__fmul_rn(-P.dt, drho), rhoi);
            rnew = __fdiv_rn(__fmul_rn(xn.z, __fsub_rn(2.f, eps)), __fadd_rn(2.f, eps));
        }
        Xr[i] = xp;
        float2 w = wrap_pos(xp, P.geo);
        X4o[i] = make_float4(w.x, w.y, rnew, eos_p(rnew, P.eos));
        V4o[i] = make_float4(u0, u1, 0.f, 0.f);
        float sp = __fsqrt_rn(__fmaf_rn(u1, u1, __fmul_rn(u0, u0)));
        {  // one atomic per warp and domain (speeds are non-negative: their bits order as uints)
            const unsigned act = __activemask();
            const unsigned grp = BATCH ? __match_any_sync(act, dom) : act;
            const unsigned vmax = __reduce_max_sync(grp, __float_as_uint(sp));
            if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(&maxv[dom], vmax);
        }
        if (!isfinite(u0) || !isfinite(u1) || !isfinite(rnew) || !isfinite(xp.x) || !isfinite(xp.y))
            atomicOr(&words[0], SPH_FLAG_NONFINITE);
        // the cells of the last sort must still cover h + the displacement at the shift pass
        // (the shift clamp adds at most sqrt(2) thr dx, covered by the margin of verlet_lim)
        const float2 xs = Xs[i];
        float e0 = xp.x - xs.x, e1 = xp.y - xs.y;
        if (sqrtf(e0 * e0 + e1 * e1) > P.verlet_lim) atomicOr(&words[0], SPH_FLAG_VERLET);
        // the shift filters the skin list at these positions
        if (e0 * e0 + e1 * e1 > P.skin_lim * P.skin_lim) atomicOr(&words[3], 1u);
    }
}

template <bool PER, bool BATCH, int MODE, typename LT, int W, bool PERSIST>
__global__ void __launch_bounds__(32 * W) k_pass_b(const Dom D0, int64_t n, const float4* __restrict__ X4,
                                                   const float4* __restrict__ V4, const int32_t* __restrict__ start,
                                                   const Dom* __restrict__ doms, const int32_t* __restrict__ did,
                                                   const int32_t* __restrict__ uid, RhsOut out,
                                                   float2* __restrict__ Xr, const float4* __restrict__ X4n,
                                                   const float4* __restrict__ V4n, float4* __restrict__ X4o,
                                                   float4* __restrict__ V4o, uint32_t* __restrict__ words,
                                                   uint32_t* __restrict__ maxv, const int16_t* __restrict__ nl,
                                                   const int16_t* __restrict__ nlc, const float2* __restrict__ Xs) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ Dom s_dom[BATCH ? 2 : 1];
    __shared__ int s_id[2];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    run_tiles<BATCH, W, PERSIST>(n, doms, did, s_dom, s_id, [&](int64_t first) {
        pass_b_tile<PER, BATCH, MODE, LT>(D0, first + threadIdx.x, n, X4, V4, start, doms, s_dom, s_id, did, uid,
                                          out, Xr, X4n, V4n, X4o, V4o, words, maxv, lst, nl, nlc, Xs);
    });
}

// ------------------------------------------------------------------------------------
// delta+ shifting (shifting.py:119-147, applied as in solveShifting :990-1005)
//   dx_i = clamp(-CFL Ma (2h/kappa)^2 sum (1 + R (W/W0)^n) m_j/(rho_i+rho_j) gradW, +-thr dx)
// ------------------------------------------------------------------------------------
template <bool PER, bool BATCH, typename LT>
__device__ __forceinline__ void shift_tile(const Dom& D0, int64_t i, int64_t n, const float4* __restrict__ X4,
                                           const float4* __restrict__ V4, const int32_t* __restrict__ start_all,
                                           const Dom* __restrict__ doms, const Dom* s_dom, const int* s_id,
                                           const int32_t* __restrict__ did,
                                           float2* __restrict__ Xr, float4* __restrict__ X4o,
                                           float4* __restrict__ V4o, uint32_t* __restrict__ words,
                                           const uint32_t* __restrict__ maxv, int enabled,
                                           const int32_t* __restrict__ uid, float* __restrict__ dx_out,
                                           LT* __restrict__ lst, int use_skin, const int16_t* __restrict__ sl,
                                           const int16_t* __restrict__ slc, const SurfaceView& sv) {
    const int dom = BATCH ? dom_of(did, i, n) : 0;
    const Dom& D = BATCH ? dom_ref(doms, s_dom, s_id, dom) : D0;
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int32_t* __restrict__ start = start_all + D.cell0;
    bool inb = i < n;
    float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, -1.f, 0.f);
    bool active = inb && !is_boundary(xi.z) && enabled;
    float2 pi = make_float2(xi.x, xi.y);
    float rhoi = xi.z;
    float2 sacc = make_float2(0.f, 0.f);
    const float cg20 = -20.0f * P.kc.cg;
    int wf = 3;  // wrap flags of the row (the skin list's count, or the scan)
    auto pair_s = [&](int j) {
        const float4 xj = __ldg(&X4[j]);
        float2 xv;
        if (PER && (wf & 2)) {
            pair_vec<true>(pi, make_float2(xj.x, xj.y), P.geo, xv.x, xv.y);
        } else {
            xv = __ffma2_rn(make_float2(xj.x, xj.y), make_float2(-1.f, -1.f), pi);
        }
        const float x0 = xv.x, x1 = xv.y;
        const PairR pr = pair_r(x0, x1, P.inv_h);
        const float om = fmaxf(1.0f - pr.q, 0.0f);
        const float om2 = om * om;
        const float W = om2 * om2 * (1.0f + 4.0f * pr.q) * P.kc.cw;
        const float kk = W * P.invW0;
        const float kn = P.shN4 ? (kk * kk) * (kk * kk) : powf(kk, P.shN);
        // (1 + R (W/W0)^n) m_j/(rho_i + rho_j) gradW without m (applied below), gradW = gf x_ij
        const float c = (1.f + P.shR * kn) * __fdividef(1.0f, rhoi + fabsf(xj.z)) * wendland_gf(pr, om, cg20);
        sacc = __ffma2_rn(make_float2(c, c), xv, sacc);
    };
    // the skin list of the step's first pass A holds every pair of the integrated positions
    // unless a particle moved farther than skin_lim (flag set by the integrator)
    const int sk = row_count((use_skin && active) ? (int)slc[i] : 0, wf);
    if (use_skin && __all_sync(kFull, sk >= 0) && words[3] == 0u) {
        if (PER && (wf & 2))
            skin_list_loop<PER, PER, LT, decltype(pair_s)&, !BATCH>((int)i, pi, X4, g, P, sl, sk, lst, pair_s);
        else
            skin_list_loop<PER, false, LT, decltype(pair_s)&, !BATCH>((int)i, pi, X4, g, P, sl, sk, lst, pair_s);
    } else {
        neighbor_loop<PER, LT>(active, (int)i, pi, X4, start, g, P, lst, words, pair_s, &wf);
    }
    if (!inb) return;
    const float s0 = sacc.x, s1 = sacc.y;
    float4 vi = V4[i];
    if (!active) {
        X4o[i] = xi;
        V4o[i] = vi;
        if (dx_out && !is_boundary(xi.z)) {
            int o = uid[i];
            dx_out[2 * o] = 0.f;
            dx_out[2 * o + 1] = 0.f;
        }
        return;
    }
    float Ma = P.compute_mach ? __uint_as_float(maxv[dom]) * P.inv_cs : 0.1f;
    float sc = P.sh_scale * Ma * P.m;
    // update = clamp(-(sc * s)) (after the free-surface projection when that is on);
    // x_new = x - update; the reference then adds (x_new - x) to x
    float u0 = -(sc * s0), u1 = -(sc * s1);
    surface_project(sv, i, u0, u1);
    float up0 = fminf(fmaxf(u0, -P.sh_thr), P.sh_thr);
    float up1 = fminf(fmaxf(u1, -P.sh_thr), P.sh_thr);
    float2 x = Xr[i];
    float y0 = __fsub_rn(x.x, up0), y1 = __fsub_rn(x.y, up1);
    float2 xn = make_float2(__fadd_rn(x.x, __fsub_rn(y0, x.x)), __fadd_rn(x.y, __fsub_rn(y1, x.y)));
    Xr[i] = xn;
    float2 w = wrap_pos(xn, P.geo);
    X4o[i] = make_float4(w.x, w.y, xi.z, xi.w);
    V4o[i] = vi;
    if (dx_out) {
        int o = uid[i];
        dx_out[2 * o] = __fsub_rn(y0, x.x);
        dx_out[2 * o + 1] = __fsub_rn(y1, x.y);
    }
}

template <bool PER, bool BATCH, typename LT, int W, bool PERSIST>
__global__ void __launch_bounds__(32 * W) k_shift(const Dom D0, int64_t n, const float4* __restrict__ X4,
                                                  const float4* __restrict__ V4, const int32_t* __restrict__ start,
                                                  const Dom* __restrict__ doms, const int32_t* __restrict__ did,
                                                  float2* __restrict__ Xr, float4* __restrict__ X4o,
                                                  float4* __restrict__ V4o, uint32_t* __restrict__ words,
                                                  const uint32_t* __restrict__ maxv, int enabled,
                                                  const int32_t* __restrict__ uid, float* __restrict__ dx_out,
                                                  int use_skin, const int16_t* __restrict__ sl,
                                                  const int16_t* __restrict__ slc, const SurfaceView sv) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ Dom s_dom[BATCH ? 2 : 1];
    __shared__ int s_id[2];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    run_tiles<BATCH, W, PERSIST>(n, doms, did, s_dom, s_id, [&](int64_t first) {
        shift_tile<PER, BATCH, LT>(D0, first + threadIdx.x, n, X4, V4, start, doms, s_dom, s_id, did, Xr, X4o, V4o,
                                   words, maxv, enabled, uid, dx_out, lst, use_skin, sl, slc, sv);
    });
}

// ------------------------------------------------------------------------------------
// Summation density (simulation.densityScheme 'summation', deltaPlus.py:193-198):
//   rho_i = sum_fluid m_j W_ij + sum_walls m_j W_ij   (computeDensity, density.py:6-15 ->
//   sphDensityInterpolation, sphOps.py:20-29; direction 'all': ftf + btf for the fluid rows)
// It runs first in every right-hand side, before the mDBC extrapolation that reads the
// fluid densities. The state is written out of place (X4 -> X4o, walls copied), so no
// thread reads a density another thread of the launch writes. The wall rows' own
// summation is not kept: the mDBC extrapolation replaces it (deltaPlus.py:200-202).
// ------------------------------------------------------------------------------------
template <bool PER, bool BATCH, typename LT>
__device__ __forceinline__ void density_sum_tile(const Dom& D0, int64_t i, int64_t n, const float4* __restrict__ X4,
                                                 float4* __restrict__ X4o, const int32_t* __restrict__ start_all,
                                                 const Dom* __restrict__ doms, const Dom* s_dom, const int* s_id,
                                                 const int32_t* __restrict__ did, uint32_t* __restrict__ words,
                                                 int skin_mode, const int16_t* __restrict__ sl,
                                                 const int16_t* __restrict__ slc, LT* __restrict__ lst) {
    const Dom& D = BATCH ? dom_ref(doms, s_dom, s_id, dom_of(did, i, n)) : D0;
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int32_t* __restrict__ start = start_all + D.cell0;
    const bool inb = i < n;
    const float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, -1.f, 0.f);
    const bool active = inb && !is_boundary(xi.z);
    const float2 pi = make_float2(xi.x, xi.y);
    float sf = 0.f, sb = 0.f;
    auto pair_d = [&](int j) {
        const float4 xj = __ldg(&X4[j]);
        float x0, x1;
        pair_vec<PER>(pi, make_float2(xj.x, xj.y), P.geo, x0, x1);
        const PairG pg = pair_fast(x0, x1, sq_norm_ref(x0, x1), P.inv_h);
        const float w = P.m * wendland_w(pg.q, P.kc);
        if (is_boundary(xj.z)) sb += w;
        else sf += w;
    };
    // skin_mode 1 filters the skin list (complete for every lane of the warp, still valid);
    // 4 does the same when this step kept its sort (words[4] == 0) and scans otherwise; 2 scans
    // (the pairs here always take the minimum image on periodic domains)
    const bool try_skin = skin_mode == 1 || (skin_mode == 4 && words[4] == 0u);
    int wf;
    const int sk = row_count((try_skin && active) ? (int)slc[i] : 0, wf);
    if (try_skin && __all_sync(kFull, sk >= 0) && words[3] == 0u)
        skin_list_loop<PER, PER, LT>((int)i, pi, X4, g, P, sl, sk, lst, pair_d);
    else
        neighbor_loop<PER, LT>(active, (int)i, pi, X4, start, g, P, lst, words, pair_d);
    if (!inb) return;
    float4 o = xi;
    if (active) {
        o.z = sf + sb;
        o.w = eos_p(o.z, P.eos);
    }
    X4o[i] = o;
}

template <bool PER, bool BATCH, typename LT, int W, bool PERSIST>
__global__ void __launch_bounds__(32 * W) k_density_sum(const Dom D0, int64_t n, const float4* __restrict__ X4,
                                                        float4* __restrict__ X4o, const int32_t* __restrict__ start_all,
                                                        const Dom* __restrict__ doms, const int32_t* __restrict__ did,
                                                        uint32_t* __restrict__ words, int skin_mode,
                                                        const int16_t* __restrict__ sl,
                                                        const int16_t* __restrict__ slc) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ Dom s_dom[BATCH ? 2 : 1];
    __shared__ int s_id[2];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    run_tiles<BATCH, W, PERSIST>(n, doms, did, s_dom, s_id, [&](int64_t first) {
        density_sum_tile<PER, BATCH, LT>(D0, first + threadIdx.x, n, X4, X4o, start_all, doms, s_dom, s_id, did,
                                         words, skin_mode, sl, slc, lst);
    });
}

// Caller-given wall densities (sph_solver_rhs_walls): rho_b[b] in the original order of the
// walls, its EOS pressure; the sign bit of the stored density marks the wall
__global__ void k_set_walls(int nB, const int32_t* __restrict__ bidx, const int32_t* __restrict__ uid,
                            float4* __restrict__ X4, Phys P, const float* __restrict__ rho_b) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nB) return;
    const int s = bidx[k];
    const float rho = rho_b[uid[s] - P.nF];
    X4[s].z = -rho;
    X4[s].w = eos_p(rho, P.eos);
}

// max |u| over all particles (the Mach number of shifting.py:139-142)
__global__ void k_maxvel(int64_t n, const float4* __restrict__ V4, const int32_t* __restrict__ did,
                         uint32_t* __restrict__ maxv) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = V4[i];
    float sp = __fsqrt_rn(__fmaf_rn(v.y, v.y, __fmul_rn(v.x, v.x)));
    atomicMax(&maxv[dom_of(did, i, n)], __float_as_uint(sp));
}

// global cell key = first cell of the particle's domain + its cell in the domain grid
__global__ void k_dom_keys(int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ did,
                           const Dom* __restrict__ doms, int32_t* __restrict__ key, int32_t* __restrict__ count,
                           const uint32_t* __restrict__ gate) {
    if (gate && *gate == 0u) return;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Dom& D = doms[dom_of(did, i, n)];
    float4 x = X4[i];
    int cx = cell_coord(x.x, D.g.mn[0], D.g.inv_cell[0], D.g.nc[0]);
    int cy = cell_coord(x.y, D.g.mn[1], D.g.inv_cell[1], D.g.nc[1]);
    int k = D.cell0 + cy * D.g.nc[0] + cx;
    key[i] = k;
    atomicAdd(&count[k], 1);
}


// ======================================================================================
// Adjoint of the delta-SPH step: vector-Jacobian products of pass A, pass B and the shift,
// in gather form. With a uniform support the exact neighbor relation is symmetric, so
// particle k collects, over its neighbors j, the derivative of its own pair terms T_kj
// (with its own multipliers) and of the neighbors' terms T_jk with respect to k's
// variables (with the neighbors' multipliers): the transpose of the neighbor list is walked
// without atomics. Wall particles (mDBC) have no terms of their own; they collect the
// derivatives of their fluid neighbors' terms with respect to the wall density and
// pressure, which k_mdbc_vjp then pulls back to the fluid state the densities were
// extrapolated from. Derivatives are those of the exact expressions with
// grad W_ij = f(r) x_ij, f = -20 C/h^4 (1-q)^3, f' = 60 C/h^5 (1-q)^2.
// ======================================================================================
// Each particle's pairs are spread over kAdjL lanes: lane sub of the group scans candidates
// sub, sub + kAdjL, ... of every stencil range, and the group's partial sums are combined by a
// butterfly of shuffles (a fixed order) before the group's first lane writes the results. At
// the adjoint's sizes (tens of thousands of particles) one lane per particle leaves most of
// the GPU idle, and each lane's pair chain is then a quarter as long.
constexpr int kAdjL = 4;

template <bool PER, class F>
__device__ __forceinline__ void neighbor_loop_split(bool active, float2 pi, const float4* __restrict__ X4,
                                                    const int32_t* __restrict__ start, const Grid& g, const Phys& P,
                                                    int32_t* __restrict__ lst, F&& f) {
    const int lane = threadIdx.x & 31, sub = lane % kAdjL;
    int rs[kMaxRanges], re[kMaxRanges];
    unsigned wmask = 0;
    const int nrng = active ? stencil_ranges(pi, g, start, rs, re, PER ? &wmask : nullptr) : 0;
    int r = 0;
    int s = nrng > 0 ? rs[0] + sub : 0, se = nrng > 0 ? re[0] : 0;
    auto advance = [&]() {  // to the next range this lane has a candidate in
        while (r < nrng && s >= se) {
            ++r;
            if (r < nrng) {
                s = rs[r] + sub;
                se = re[r];
            }
        }
    };
    advance();
    int cnt = 0;
    while (__any_sync(kFull, r < nrng)) {
        if (r < nrng) {
            const int left = (se - s + kAdjL - 1) / kAdjL;
            const int m = left < kUnroll ? left : kUnroll;
            const bool wr = PER && ((wmask >> r) & 1u);
            float4 xj[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u)
                if (u < m) xj[u] = __ldg(&X4[s + u * kAdjL]);
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                if (u < m) {
                    float x0, x1;
                    if (wr)
                        pair_vec<true>(pi, make_float2(xj[u].x, xj[u].y), P.geo, x0, x1);
                    else
                        pair_vec<false>(pi, make_float2(xj[u].x, xj[u].y), P.geo, x0, x1);
                    if (sq_norm_ref(x0, x1) <= P.T) lst[(cnt++) * 32 + lane] = s + u * kAdjL;
                }
            }
            s += m * kAdjL;
            advance();
        }
        if (__any_sync(kFull, cnt > kCap - kUnroll)) {
            const int mc = (int)__reduce_max_sync(kFull, (unsigned)cnt);
            for (int k = 0; k < mc; ++k)
                if (k < cnt) f(lst[k * 32 + lane]);
            cnt = 0;
        }
    }
    const int mc = (int)__reduce_max_sync(kFull, (unsigned)cnt);
    for (int k = 0; k < mc; ++k)
        if (k < cnt) f(lst[k * 32 + lane]);
}

__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = kAdjL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

struct KD {
    float f, fp;
};

__device__ __forceinline__ KD kern_fd(float r, const Phys& P) {
    float q = r * P.inv_h;
    float om = fmaxf(1.f - q, 0.f);
    float c4 = P.kc.cg * P.inv_h;
    KD k;
    k.f = -20.f * c4 * om * om * om;
    k.fp = 60.f * c4 * P.inv_h * om * om;
    return k;
}

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }

// gradients of lam . T_ij for the four pass-B pair terms (pressure, viscosity, continuity,
// diffusion) with respect to the pair vector and the variables of i and j
struct BVjp {
    float2 gx, gui, guj, gGi, gGj;
    float gri, grj, gpi, gpj;
};

__device__ __forceinline__ BVjp pairB_vjp(float2 x, float r, float2 ui, float2 uj, float ri, float rj, float pi,
                                          float pj, float2 Gi, float2 Gj, float2 lP, float2 lV, float lC, float lD,
                                          const Phys& P) {
    BVjp o;
    KD k = kern_fd(r, P);
    float ir = 1.f / r, irj = 1.f / rj;
    float2 xh = f2(x.x * ir, x.y * ir);
    // pressure: (p_i + p_j)/rho_j f x
    float lPx = dot2(lP, x);
    float sP = (pi + pj) * irj;
    o.gx = f2(sP * (k.f * lP.x + lPx * k.fp * xh.x), sP * (k.f * lP.y + lPx * k.fp * xh.y));
    o.gpi = o.gpj = k.f * lPx * irj;
    o.grj = -sP * k.f * lPx * irj;
    // viscosity: (u_ij . x) phi f x / rho_j, phi = 1 / (r (r + eps h^2))
    float2 uij = f2(ui.x - uj.x, ui.y - uj.y);
    float ux = dot2(uij, x), lVx = dot2(lV, x);
    float phi = 1.f / (r * (r + P.v_eps));
    float phip = -(2.f * r + P.v_eps) * phi * phi;
    float pf = phi * k.f, pfp = phip * k.f + phi * k.fp;
    float cV = pf * irj;
    o.gx.x += (uij.x * lVx + lV.x * ux) * cV + ux * lVx * irj * pfp * xh.x;
    o.gx.y += (uij.y * lVx + lV.y * ux) * cV + ux * lVx * irj * pfp * xh.y;
    o.gui = f2(x.x * lVx * cV, x.y * lVx * cV);
    o.guj = f2(-o.gui.x, -o.gui.y);
    o.grj += -(ux * lVx * cV) * irj;
    // continuity: (u_j - u_i) . x f / rho_j
    float cx = -ux;
    o.gx.x += lC * irj * (-uij.x * k.f + cx * k.fp * xh.x);
    o.gx.y += lC * irj * (-uij.y * k.f + cx * k.fp * xh.y);
    float cC = lC * k.f * irj;
    o.guj.x += cC * x.x;
    o.guj.y += cC * x.y;
    o.gui.x -= cC * x.x;
    o.gui.y -= cC * x.y;
    o.grj += -lC * cx * k.f * irj * irj;
    // diffusion: [-2 (rho_j - rho_i) f psi + (G_i + G_j) . x f] / rho_j, psi = r / (r + 1e-6 h)
    float psi = r / (r + P.diff_eps);
    float psip = P.diff_eps / ((r + P.diff_eps) * (r + P.diff_eps));
    float fpsi = k.f * psi, fpsip = k.fp * psi + k.f * psip;
    float2 Gs = f2(Gi.x + Gj.x, Gi.y + Gj.y);
    float Gx = dot2(Gs, x);
    float dr = rj - ri;
    float TD = (-2.f * dr * fpsi + Gx * k.f) * irj;
    o.gx.x += lD * irj * (-2.f * dr * fpsip * xh.x + Gs.x * k.f + Gx * k.fp * xh.x);
    o.gx.y += lD * irj * (-2.f * dr * fpsip * xh.y + Gs.y * k.f + Gx * k.fp * xh.y);
    o.gri = lD * irj * 2.f * fpsi;
    o.grj += lD * irj * (-2.f * fpsi) - lD * TD * irj;
    o.gGi = o.gGj = f2(lD * k.f * x.x * irj, lD * k.f * x.y * irj);
    return o;
}

// gradients of lam . T_ib for the pair terms of fluid particle i with wall particle b (wall
// velocity 0): pressure, continuity and the boundary viscosity (no density diffusion)
struct BWVjp {
    float2 gx, gui;
    float gri, grb, gpi, gpb;
};

__device__ __forceinline__ BWVjp pairBW_vjp(float2 x, float r, float2 ui, float ri, float rb, float pi, float pb,
                                            float2 lP, float2 lB, float lC, const Phys& P) {
    BWVjp o;
    KD k = kern_fd(r, P);
    float ir = 1.f / r, irb = 1.f / rb;
    float2 xh = f2(x.x * ir, x.y * ir);
    // pressure: (p_i + p_b)/rho_b f x
    float lPx = dot2(lP, x);
    float sP = (pi + pb) * irb;
    o.gx = f2(sP * (k.f * lP.x + lPx * k.fp * xh.x), sP * (k.f * lP.y + lPx * k.fp * xh.y));
    o.gpi = o.gpb = k.f * lPx * irb;
    o.grb = -sP * k.f * lPx * irb;
    o.gri = 0.f;
    // continuity: (u_b - u_i) . x f / rho_b = -(u_i . x) f / rho_b
    float ux = dot2(ui, x);
    o.gx.x += lC * irb * (-ui.x * k.f - ux * k.fp * xh.x);
    o.gx.y += lC * irb * (-ui.y * k.f - ux * k.fp * xh.y);
    o.gui = f2(-lC * k.f * irb * x.x, -lC * k.f * irb * x.y);
    o.grb += lC * ux * k.f * irb * irb;
    // boundary viscosity: (u_i . x) phi f D x, phi = 1 / (r (r + eps_b h^2)),
    // D = 1 / (rho_i + rho_b) (boundaryViscosity) or 1 / rho_b
    float D = P.bvisc ? 1.f / (ri + rb) : irb;
    float lBx = dot2(lB, x);
    float phi = 1.f / (r * (r + P.bv_eps));
    float phip = -(2.f * r + P.bv_eps) * phi * phi;
    float pf = phi * k.f, pfp = phip * k.f + phi * k.fp;
    float cB = pf * D;
    o.gx.x += (ui.x * lBx + lB.x * ux) * cB + ux * lBx * D * pfp * xh.x;
    o.gx.y += (ui.y * lBx + lB.y * ux) * cB + ux * lBx * D * pfp * xh.y;
    o.gui.x += x.x * lBx * cB;
    o.gui.y += x.y * lBx * cB;
    float EB = ux * lBx * cB;
    o.grb -= EB * D;
    if (P.bvisc) o.gri -= EB * D;
    return o;
}

__device__ __forceinline__ float eos_dpdr(float rho, const Phys& P) {
    // p = B ((rho/rho0)^gamma - 1): dp/drho = B gamma (rho/rho0)^(gamma-1) / rho0
    return P.eos.B * P.eos.gamma * powf(rho / P.eos.rho0, P.eos.gamma - 1.f) / P.eos.rho0;
}

// multipliers of pass B from the adjoints of the rates (original order in, sorted order out);
// wall particles have no rates and carry none
__global__ void k_lam_rates(int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ uid, Dom D,
                            const float* __restrict__ abar, const float* __restrict__ drbar,
                            float4* __restrict__ L4, float4* __restrict__ L2) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const Phys& P = D.P;
    float rho = X4[s].z;
    if (is_boundary(rho)) {
        L4[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        L2[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    int o = uid[s];
    float2 a = f2(abar[2 * o], abar[2 * o + 1]);
    float dr = drbar ? drbar[o] : 0.f;
    float mr = P.m / rho;
    L4[s] = make_float4(-mr * a.x, -mr * a.y, P.v_num * mr * a.x, P.v_num * mr * a.y);
    L2[s] = make_float4(-P.m * rho * dr, P.diff_coef * P.m * dr, P.bv_num * mr * a.x, P.bv_num * mr * a.y);
}

// Fluid particle k: its own pair terms and its fluid neighbors' terms, as for a fluid-only
// domain, plus its own terms with wall neighbors. Wall particle k: the derivatives of its
// fluid neighbors' terms with respect to its density and pressure, folded into the wall
// density's adjoint rbbar (original wall order).
template <bool PER>
__global__ void __launch_bounds__(128) k_vjp_rates(int64_t n, const float4* __restrict__ X4,
                                                   const float4* __restrict__ V4, const int32_t* __restrict__ start,
                                                   Dom D, const int32_t* __restrict__ uid,
                                                   const float4* __restrict__ L4, const float4* __restrict__ L2,
                                                   uint32_t* __restrict__ words, float* __restrict__ xbar,
                                                   float* __restrict__ ubar, float* __restrict__ rbar,
                                                   float* __restrict__ Gbar, float* __restrict__ nup,
                                                   float* __restrict__ rbbar) {
    __shared__ int32_t s_list[4][kCap * 32];
    const Phys& P = D.P;
    const Grid& g = D.g;
    int64_t k = ((int64_t)blockIdx.x * 128 + threadIdx.x) / kAdjL;
    bool inb = k < n;
    float4 xk = inb ? X4[k] : make_float4(0.f, 0.f, 1.f, 0.f);
    float4 vk = inb ? V4[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 lk4 = inb ? L4[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 lk2 = inb ? L2[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool kb = is_boundary(xk.z);
    const float rk = fabsf(xk.z);
    float2 pk = f2(xk.x, xk.y);
    float2 gx = f2(0.f, 0.f), gu = f2(0.f, 0.f), gG = f2(0.f, 0.f);
    float gr = 0.f, gp = 0.f;
    float2 Ps = f2(0.f, 0.f), Vs = f2(0.f, 0.f), Bs = f2(0.f, 0.f);
    float Cs = 0.f;
    neighbor_loop_split<PER>(inb, pk, X4, start + D.cell0, g, P, s_list[threadIdx.x >> 5], [&](int j) {
        if (j == (int)k) return;
        float4 xj = __ldg(&X4[j]);
        const bool jb = is_boundary(xj.z);
        if (kb && jb) return;
        float x0, x1;
        pair_vec<PER>(pk, make_float2(xj.x, xj.y), P.geo, x0, x1);
        float sq = sq_norm_ref(x0, x1);
        float r = sqrtf(sq);
        if (r <= 0.f) return;
        const float rj = fabsf(xj.z);
        float2 x = f2(x0, x1);
        float2 uk = f2(vk.x, vk.y);
        if (!kb && !jb) {
            float4 vj = __ldg(&V4[j]);
            float4 lj4 = __ldg(&L4[j]);
            float4 lj2 = __ldg(&L2[j]);
            float2 uj = f2(vj.x, vj.y);
            float2 Gk = f2(vk.z, vk.w), Gj = f2(vj.z, vj.w);
            // k's own pair term T_kj
            BVjp a = pairB_vjp(x, r, uk, uj, rk, rj, xk.w, xj.w, Gk, Gj, f2(lk4.x, lk4.y), f2(lk4.z, lk4.w), lk2.x,
                               lk2.y, P);
            // the neighbor's pair term T_jk (pair vector x_j - x_k = -x)
            BVjp b = pairB_vjp(f2(-x0, -x1), r, uj, uk, rj, rk, xj.w, xk.w, Gj, Gk, f2(lj4.x, lj4.y),
                               f2(lj4.z, lj4.w), lj2.x, lj2.y, P);
            gx.x += a.gx.x - b.gx.x;
            gx.y += a.gx.y - b.gx.y;
            gu.x += a.gui.x + b.guj.x;
            gu.y += a.gui.y + b.guj.y;
            gr += a.gri + b.grj;
            gp += a.gpi + b.gpj;
            gG.x += a.gGi.x + b.gGj.x;
            gG.y += a.gGi.y + b.gGj.y;
            // forward sums of k (for the derivatives of the 1/rho_k and rho_k prefactors)
            KD kd = kern_fd(r, P);
            float irj = 1.f / rj;
            float sP = (xk.w + xj.w) * irj * kd.f;
            Ps.x += sP * x0;
            Ps.y += sP * x1;
            float ux = (uk.x - uj.x) * x0 + (uk.y - uj.y) * x1;
            float sV = ux / (r * (r + P.v_eps)) * kd.f * irj;
            Vs.x += sV * x0;
            Vs.y += sV * x1;
            Cs += -ux * kd.f * irj;
        } else if (!kb) {  // fluid k, wall j: k's own term
            BWVjp a = pairBW_vjp(x, r, uk, rk, rj, xk.w, xj.w, f2(lk4.x, lk4.y), f2(lk2.z, lk2.w), lk2.x, P);
            gx.x += a.gx.x;
            gx.y += a.gx.y;
            gu.x += a.gui.x;
            gu.y += a.gui.y;
            gr += a.gri;
            gp += a.gpi;
            KD kd = kern_fd(r, P);
            float irj = 1.f / rj;
            float sP = (xk.w + xj.w) * irj * kd.f;
            Ps.x += sP * x0;
            Ps.y += sP * x1;
            float ux = uk.x * x0 + uk.y * x1;
            Cs += -ux * kd.f * irj;
            float sB = ux / (r * (r + P.bv_eps)) * kd.f * (P.bvisc ? 1.f / (rk + rj) : irj);
            Bs.x += sB * x0;
            Bs.y += sB * x1;
        } else {  // wall k, fluid j: j's term with respect to the wall's density and pressure
            float4 vj = __ldg(&V4[j]);
            float4 lj4 = __ldg(&L4[j]);
            float4 lj2 = __ldg(&L2[j]);
            BWVjp b = pairBW_vjp(f2(-x0, -x1), r, f2(vj.x, vj.y), rj, rk, xj.w, xk.w, f2(lj4.x, lj4.y),
                                 f2(lj2.z, lj2.w), lj2.x, P);
            gr += b.grb;
            gp += b.gpb;
        }
    });
    gx.x = group_sum(gx.x);
    gx.y = group_sum(gx.y);
    gu.x = group_sum(gu.x);
    gu.y = group_sum(gu.y);
    gG.x = group_sum(gG.x);
    gG.y = group_sum(gG.y);
    gr = group_sum(gr);
    gp = group_sum(gp);
    Ps.x = group_sum(Ps.x);
    Ps.y = group_sum(Ps.y);
    Vs.x = group_sum(Vs.x);
    Vs.y = group_sum(Vs.y);
    Bs.x = group_sum(Bs.x);
    Bs.y = group_sum(Bs.y);
    Cs = group_sum(Cs);
    if (!inb || (threadIdx.x & (kAdjL - 1)) != 0) return;
    int o = uid[k];
    if (kb) {
        if (rbbar) rbbar[o - P.nF] += gr + gp * eos_dpdr(rk, P);
        return;
    }
    float rho = rk;
    gr += gp * eos_dpdr(rho, P) - (lk4.x * Ps.x + lk4.y * Ps.y) / rho - (lk4.z * Vs.x + lk4.w * Vs.y) / rho -
          (lk2.z * Bs.x + lk2.w * Bs.y) / rho + lk2.x * Cs / rho;
    xbar[2 * o] += gx.x;
    xbar[2 * o + 1] += gx.y;
    ubar[2 * o] += gu.x;
    ubar[2 * o + 1] += gu.y;
    rbar[o] += gr;
    if (Gbar) {
        Gbar[2 * o] += gG.x;
        Gbar[2 * o + 1] += gG.y;
    }
    // d du_k / d nu = dvnum_dnu (m / rho_k) Vs, and (m / rho_k) abar_k = -lambda_P
    if (nup) nup[o] = -P.dvnum_dnu * (lk4.x * Vs.x + lk4.y * Vs.y);
}

// pass A: per-particle multipliers of g_f = sum_fluid (rho_i - rho_j)/rho_j f x, of
// g_b = sum_walls (rho_i - rho_b)/rho_b f x and of M = -sum_all f/rho_j x x^T from the
// adjoint of gradRho^L = m (L g_f + g_b), L = (m M)^-1: Lg.xy = m L^T G (fluid pairs),
// Lg.zw = m G (wall pairs); walls carry none
template <bool PER>
__global__ void __launch_bounds__(128) k_lam_grad(int64_t n, const float4* __restrict__ X4,
                                                  const int32_t* __restrict__ start, Dom D,
                                                  const int32_t* __restrict__ uid, const float* __restrict__ Gbar,
                                                  uint32_t* __restrict__ words, float4* __restrict__ LM,
                                                  float4* __restrict__ Lg) {
    __shared__ int32_t s_list[4][kCap * 32];
    const Phys& P = D.P;
    int64_t k = ((int64_t)blockIdx.x * 128 + threadIdx.x) / kAdjL;
    bool inb = k < n;
    float4 xk = inb ? X4[k] : make_float4(0.f, 0.f, 1.f, 0.f);
    const bool kb = is_boundary(xk.z);
    float2 pk = f2(xk.x, xk.y);
    float M00 = 0.f, M01 = 0.f, M10 = 0.f, M11 = 0.f, g0 = 0.f, g1 = 0.f;
    int nf = 0;
    neighbor_loop_split<PER>(inb && !kb, pk, X4, start + D.cell0, D.g, P, s_list[threadIdx.x >> 5], [&](int j) {
        float4 xj = __ldg(&X4[j]);
        const bool jb = is_boundary(xj.z);
        float x0, x1;
        pair_vec<PER>(pk, make_float2(xj.x, xj.y), P.geo, x0, x1);
        if (!jb) ++nf;
        if (j == (int)k) return;
        float r = sqrtf(sq_norm_ref(x0, x1));
        KD kd = kern_fd(r, P);
        const float rj = fabsf(xj.z);
        float w = kd.f / rj;
        M00 -= w * x0 * x0;
        M01 -= w * x0 * x1;
        M10 -= w * x1 * x0;
        M11 -= w * x1 * x1;
        if (!jb) {
            float c = (xk.z - rj) * w;
            g0 += c * x0;
            g1 += c * x1;
        }
    });
    M00 = group_sum(M00);
    M01 = group_sum(M01);
    M10 = group_sum(M10);
    M11 = group_sum(M11);
    g0 = group_sum(g0);
    g1 = group_sum(g1);
    nf = (int)group_sum((float)nf);
    if (!inb || (threadIdx.x & (kAdjL - 1)) != 0) return;
    if (kb) {
        LM[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        Lg[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    int o = uid[k];
    float m = P.m;
    float G0 = Gbar[2 * o], G1 = Gbar[2 * o + 1];
    M2 L;
    if (nf < 4) {
        L.a = 1.f; L.b = 0.f; L.c = 0.f; L.d = 1.f;
    } else {
        L = pinv2x2_ref(m * M00, m * M01, m * M10, m * M11);
    }
    // gbar = m L^T G; Lbar = m G g^T; Mbar = -L^T Lbar L^T (the multiplier of M carries m)
    float gb0 = m * (L.a * G0 + L.c * G1), gb1 = m * (L.b * G0 + L.d * G1);
    float mb00 = 0.f, mb01 = 0.f, mb10 = 0.f, mb11 = 0.f;
    if (nf >= 4) {
        float Lb00 = m * G0 * g0, Lb01 = m * G0 * g1, Lb10 = m * G1 * g0, Lb11 = m * G1 * g1;
        // T = L^T Lbar
        float t00 = L.a * Lb00 + L.c * Lb10, t01 = L.a * Lb01 + L.c * Lb11;
        float t10 = L.b * Lb00 + L.d * Lb10, t11 = L.b * Lb01 + L.d * Lb11;
        // Mbar = -T L^T
        mb00 = -(t00 * L.a + t01 * L.b);
        mb01 = -(t00 * L.c + t01 * L.d);
        mb10 = -(t10 * L.a + t11 * L.b);
        mb11 = -(t10 * L.c + t11 * L.d);
    }
    LM[k] = make_float4(m * mb00, m * mb01, m * mb10, m * mb11);
    Lg[k] = make_float4(gb0, gb1, m * G0, m * G1);
}

__device__ __forceinline__ void pairA_vjp(float2 x, float r, float ri, float rj, float2 lg, float4 lM, const Phys& P,
                                          float2& gx, float& gri, float& grj) {
    KD k = kern_fd(r, P);
    float irj = 1.f / rj;
    float2 xh = f2(x.x / r, x.y / r);
    // g term: (rho_i - rho_j)/rho_j f (lg . x)
    float lgx = dot2(lg, x);
    float c = (ri - rj) * irj;
    gx = f2(c * (k.f * lg.x + lgx * k.fp * xh.x), c * (k.f * lg.y + lgx * k.fp * xh.y));
    gri = irj * k.f * lgx;
    grj = -k.f * lgx * ri * irj * irj;
    // M term: -f/rho_j x^T Mbar x
    float Mx0 = (lM.x + lM.x) * x.x + (lM.y + lM.z) * x.y;
    float Mx1 = (lM.z + lM.y) * x.x + (lM.w + lM.w) * x.y;
    float xMx = x.x * (lM.x * x.x + lM.y * x.y) + x.y * (lM.z * x.x + lM.w * x.y);
    gx.x += -irj * (k.f * Mx0 + xMx * k.fp * xh.x);
    gx.y += -irj * (k.f * Mx1 + xMx * k.fp * xh.y);
    grj += k.f * irj * irj * xMx;
}

template <bool PER>
__global__ void __launch_bounds__(128) k_vjp_grad(int64_t n, const float4* __restrict__ X4,
                                                  const int32_t* __restrict__ start, Dom D,
                                                  const int32_t* __restrict__ uid, const float4* __restrict__ LM,
                                                  const float4* __restrict__ Lg, uint32_t* __restrict__ words,
                                                  float* __restrict__ xbar, float* __restrict__ rbar,
                                                  float* __restrict__ rbbar) {
    __shared__ int32_t s_list[4][kCap * 32];
    const Phys& P = D.P;
    int64_t k = ((int64_t)blockIdx.x * 128 + threadIdx.x) / kAdjL;
    bool inb = k < n;
    float4 xk = inb ? X4[k] : make_float4(0.f, 0.f, 1.f, 0.f);
    float4 lMk = inb ? LM[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 lgk = inb ? Lg[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool kb = is_boundary(xk.z);
    const float rk = fabsf(xk.z);
    float2 pk = f2(xk.x, xk.y);
    float2 gx = f2(0.f, 0.f);
    float gr = 0.f;
    neighbor_loop_split<PER>(inb, pk, X4, start + D.cell0, D.g, P, s_list[threadIdx.x >> 5], [&](int j) {
        if (j == (int)k) return;
        float4 xj = __ldg(&X4[j]);
        const bool jb = is_boundary(xj.z);
        if (kb && jb) return;
        float x0, x1;
        pair_vec<PER>(pk, make_float2(xj.x, xj.y), P.geo, x0, x1);
        float r = sqrtf(sq_norm_ref(x0, x1));
        if (r <= 0.f) return;
        const float rj = fabsf(xj.z);
        float2 ga, gb;
        float ari, arj, bri, brj;
        if (!kb && !jb) {
            float4 lMj = __ldg(&LM[j]);
            float4 lgj = __ldg(&Lg[j]);
            pairA_vjp(f2(x0, x1), r, rk, rj, f2(lgk.x, lgk.y), lMk, P, ga, ari, arj);
            pairA_vjp(f2(-x0, -x1), r, rj, rk, f2(lgj.x, lgj.y), lMj, P, gb, bri, brj);
            gx.x += ga.x - gb.x;
            gx.y += ga.y - gb.y;
            gr += ari + brj;
        } else if (!kb) {  // fluid k, wall j: k's own term (the boundary part of the gradient)
            pairA_vjp(f2(x0, x1), r, rk, rj, f2(lgk.z, lgk.w), lMk, P, ga, ari, arj);
            gx.x += ga.x;
            gx.y += ga.y;
            gr += ari;
        } else {  // wall k, fluid j: j's term with respect to the wall's density
            float4 lMj = __ldg(&LM[j]);
            float4 lgj = __ldg(&Lg[j]);
            pairA_vjp(f2(-x0, -x1), r, rj, rk, f2(lgj.z, lgj.w), lMj, P, gb, bri, brj);
            gr += brj;
        }
    });
    gx.x = group_sum(gx.x);
    gx.y = group_sum(gx.y);
    gr = group_sum(gr);
    if (!inb || (threadIdx.x & (kAdjL - 1)) != 0) return;
    int o = uid[k];
    if (kb) {
        if (rbbar) rbbar[o - P.nF] += gr;
        return;
    }
    xbar[2 * o] += gx.x;
    xbar[2 * o + 1] += gx.y;
    rbar[o] += gr;
}

// shift: multipliers from the adjoint of the shifted positions (clamped components carry
// none); walls are not shifted and carry none
template <bool PER>
__global__ void __launch_bounds__(128) k_lam_shift(int64_t n, const float4* __restrict__ X4,
                                                   const int32_t* __restrict__ start, Dom D,
                                                   const int32_t* __restrict__ uid, const uint32_t* __restrict__ maxv,
                                                   const float* __restrict__ xbar_new, uint32_t* __restrict__ words,
                                                   float4* __restrict__ LS, float* __restrict__ mapart) {
    __shared__ int32_t s_list[4][kCap * 32];
    const Phys& P = D.P;
    int64_t k = ((int64_t)blockIdx.x * 128 + threadIdx.x) / kAdjL;
    bool inb = k < n;
    float4 xk = inb ? X4[k] : make_float4(0.f, 0.f, 1.f, 0.f);
    const bool kb = is_boundary(xk.z);
    float2 pk = f2(xk.x, xk.y);
    float s0 = 0.f, s1 = 0.f;
    neighbor_loop_split<PER>(inb && !kb, pk, X4, start + D.cell0, D.g, P, s_list[threadIdx.x >> 5], [&](int j) {
        if (j == (int)k) return;
        float4 xj = __ldg(&X4[j]);
        float x0, x1;
        pair_vec<PER>(pk, make_float2(xj.x, xj.y), P.geo, x0, x1);
        float r = sqrtf(sq_norm_ref(x0, x1));
        KD kd = kern_fd(r, P);
        float W = wendland_w(r * P.inv_h, P.kc);
        float kk = W * P.invW0;
        float w = 1.f + P.shR * (kk * kk) * (kk * kk);
        float c = w * kd.f / (xk.z + fabsf(xj.z));
        s0 += c * x0;
        s1 += c * x1;
    });
    s0 = group_sum(s0);
    s1 = group_sum(s1);
    if (!inb || (threadIdx.x & (kAdjL - 1)) != 0) return;
    if (kb) {
        LS[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    int o = uid[k];
    float Ma = P.compute_mach ? __uint_as_float(maxv[0]) * P.inv_cs : 0.1f;
    float sc = P.sh_scale * P.m;
    float d0 = sc * Ma * s0, d1 = sc * Ma * s1;
    float a0 = fabsf(d0) < P.sh_thr ? 1.f : 0.f, a1 = fabsf(d1) < P.sh_thr ? 1.f : 0.f;
    float xb0 = xbar_new[2 * o] * a0, xb1 = xbar_new[2 * o + 1] * a1;
    LS[k] = make_float4(sc * Ma * xb0, sc * Ma * xb1, 0.f, 0.f);
    mapart[o] = P.compute_mach ? sc * (xb0 * s0 + xb1 * s1) : 0.f;
}

__device__ __forceinline__ void pairS_vjp(float2 x, float r, float ri, float rj, float2 lS, const Phys& P, float2& gx,
                                          float& gri, float& grj) {
    KD k = kern_fd(r, P);
    float W = wendland_w(r * P.inv_h, P.kc);
    float kk = W * P.invW0;
    float kk3 = kk * kk * kk;
    float w = 1.f + P.shR * kk3 * kk;
    float Wp = k.f * r;
    float wp = 4.f * P.shR * kk3 * Wp * P.invW0;
    float ir = 1.f / r, den = 1.f / (ri + rj);
    float2 xh = f2(x.x * ir, x.y * ir);
    float lx = dot2(lS, x);
    float wf = w * k.f, wfp = wp * k.f + w * k.fp;
    gx = f2(den * (wf * lS.x + lx * wfp * xh.x), den * (wf * lS.y + lx * wfp * xh.y));
    gri = grj = -wf * lx * den * den;
}

template <bool PER>
__global__ void __launch_bounds__(128) k_vjp_shift(int64_t n, const float4* __restrict__ X4,
                                                   const int32_t* __restrict__ start, Dom D,
                                                   const int32_t* __restrict__ uid, const float4* __restrict__ LS,
                                                   const float* __restrict__ xbar_new, uint32_t* __restrict__ words,
                                                   float* __restrict__ xbar, float* __restrict__ rbar,
                                                   float* __restrict__ rbbar) {
    __shared__ int32_t s_list[4][kCap * 32];
    const Phys& P = D.P;
    int64_t k = ((int64_t)blockIdx.x * 128 + threadIdx.x) / kAdjL;
    bool inb = k < n;
    float4 xk = inb ? X4[k] : make_float4(0.f, 0.f, 1.f, 0.f);
    float4 lk = inb ? LS[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool kb = is_boundary(xk.z);
    const float rk = fabsf(xk.z);
    float2 pk = f2(xk.x, xk.y);
    float2 gx = f2(0.f, 0.f);
    float gr = 0.f;
    neighbor_loop_split<PER>(inb, pk, X4, start + D.cell0, D.g, P, s_list[threadIdx.x >> 5], [&](int j) {
        if (j == (int)k) return;
        float4 xj = __ldg(&X4[j]);
        const bool jb = is_boundary(xj.z);
        if (kb && jb) return;
        float x0, x1;
        pair_vec<PER>(pk, make_float2(xj.x, xj.y), P.geo, x0, x1);
        float r = sqrtf(sq_norm_ref(x0, x1));
        if (r <= 0.f) return;
        const float rj = fabsf(xj.z);
        float2 ga, gb;
        float ari, arj, bri, brj;
        if (!kb) {
            pairS_vjp(f2(x0, x1), r, rk, rj, f2(lk.x, lk.y), P, ga, ari, arj);
            gx.x += ga.x;
            gx.y += ga.y;
            gr += ari;
        }
        if (!jb) {  // the fluid neighbor's term
            float4 lj = __ldg(&LS[j]);
            pairS_vjp(f2(-x0, -x1), r, rj, rk, f2(lj.x, lj.y), P, gb, bri, brj);
            if (!kb) {
                gx.x -= gb.x;
                gx.y -= gb.y;
            }
            gr += brj;
        }
    });
    gx.x = group_sum(gx.x);
    gx.y = group_sum(gx.y);
    gr = group_sum(gr);
    if (!inb || (threadIdx.x & (kAdjL - 1)) != 0) return;
    int o = uid[k];
    if (kb) {
        if (rbbar) rbbar[o - P.nF] += gr;
        return;
    }
    // x'' = x' + delta(x'): the identity part plus the shift's Jacobian
    xbar[2 * o] += xbar_new[2 * o] + gx.x;
    xbar[2 * o + 1] += xbar_new[2 * o + 1] + gx.y;
    rbar[o] += gr;
}

// The 13 ghost moments of mdbc_moments in fp64 (the adjoint's solve: near free edges the
// moment matrix reaches condition numbers of ~1e4, where fp32 moments would cost the
// derivative ~1e-3 of its accuracy)
template <bool PER>
__device__ __forceinline__ void mdbc_moments_f64(const Phys& P, float2 gw, const int* rs, const int* re, int nr,
                                                 const float4* __restrict__ X4, int lane, double acc[13]) {
    int total = 0;
    for (int a = 0; a < nr; ++a) total += re[a] - rs[a];
#pragma unroll
    for (int q = 0; q < 13; ++q) acc[q] = 0.0;
    int r = 0, base = 0;
    for (int t = lane; t < total; t += 32) {
        while (t >= base + (re[r] - rs[r])) {
            base += re[r] - rs[r];
            ++r;
        }
        const int j = rs[r] + (t - base);
        const float4 xj = __ldg(&X4[j]);
        if (is_boundary(xj.z)) continue;
        float x0, x1;
        pair_vec<PER>(gw, make_float2(xj.x, xj.y), P.geo, x0, x1);
        const float sq = sq_norm_ref(x0, x1);
        if (sq > P.T) continue;
        const double dr = sqrt((double)sq);
        const double q = dr * P.inv_h;
        const double om = 1.0 - q;
        const double W = om * om * om * om * (1.0 + 4.0 * q) * P.kc.cw;
        const double W1 = -20.0 * q * om * om * om * P.kc.cg;
        const double e0 = dr > 0.0 ? x0 / dr : 0.0, e1 = dr > 0.0 ? x1 / dr : 0.0;
        const double g0 = W1 * e0, g1 = W1 * e1;
        const double V = (double)P.m / xj.z;
        const double xi0 = -(double)x0, xi1 = -(double)x1;
        acc[0] += P.m * W;
        acc[1] += V * W;
        acc[2] += P.m * g0;
        acc[3] += P.m * g1;
        acc[4] += V * g0;
        acc[5] += V * g1;
        acc[6] += xi0 * V * W;
        acc[7] += xi1 * V * W;
        acc[8] += xi0 * V * g0;
        acc[9] += xi0 * V * g1;
        acc[10] += xi1 * V * g0;
        acc[11] += xi1 * V * g1;
        acc[12] += 1.0;
    }
#pragma unroll
    for (int q = 0; q < 13; ++q) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(kFull, acc[q], o);
    }
}

// mDBC adjoint: the wall densities' adjoint rbbar (original wall order) pulled back to the
// fluid positions and densities the ghost moments read (mDBC.py:50-163 as k_mdbc_sums /
// k_mdbc_solve evaluate it). One warp per wall particle recomputes its ghost's moments (in
// fp64); every lane then forms the adjoints of the 13 moments from the fp64 solve
// (y = A^+ b, rho_b = c . y with c = (1, x_b - x_ghost): bbar = A^+T c rhobar,
// Abar = -bbar y^T; the Shepard branch rho_b = num / (den + 1e-7)) and adds its fluid
// candidates' derivatives into fp64 accumulators by slot (the sums are rounded to fp32
// once, by k_wall_adjoint_fin). With d = x_ghost - x_j, V = m / rho_j, g = W'(r) d/r and
// xi = -d, the moments of one fluid particle are m W, V W, m g, V g, xi V W and xi (x) V g.
template <bool PER>
__global__ void __launch_bounds__(128) k_mdbc_vjp(int nB, const int32_t* __restrict__ bidx,
                                                  const int32_t* __restrict__ uid, const float2* __restrict__ Xr,
                                                  const float4* __restrict__ X4, const float2* __restrict__ bnormal,
                                                  const float* __restrict__ bdist, const int32_t* __restrict__ start,
                                                  Grid g, Phys P, const float* __restrict__ rbbar,
                                                  double* __restrict__ xacc, double* __restrict__ racc) {
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= nB) return;  // warp-uniform
    const int s = bidx[k];
    const int b = uid[s] - P.nF;
    const float rhobar = rbbar[b];
    if (rhobar == 0.f) return;  // warp-uniform
    const float2 xb = Xr[s];
    const float2 gp = mdbc_ghost(P, xb, bnormal[b], bdist[b]);
    const float2 gw = wrap_pos(gp, P.geo);
    int rs[kMaxRanges], re[kMaxRanges];
    const int nr = stencil_ranges(gw, g, start, rs, re);
    double a[13];
    mdbc_moments_f64<PER>(P, gw, rs, re, nr, X4, lane, a);
    const int cnt = (int)a[12];
    double sb[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) sb[q] = 0.0;
    if (cnt > 5) {
        double A[9] = {a[1], a[6], a[7], a[4], a[8], a[9], a[5], a[10], a[11]};
        double Pi[9];
        pinv3_f64(A, Pi, 3.0 * 1.1920928955078125e-07);
        const double bv[3] = {a[0], a[2], a[3]};
        double y[3];
        for (int r = 0; r < 3; ++r) y[r] = Pi[3 * r] * bv[0] + Pi[3 * r + 1] * bv[1] + Pi[3 * r + 2] * bv[2];
        const float rel0 = __fsub_rn(xb.x, gp.x), rel1 = __fsub_rn(xb.y, gp.y);
        const double yb[3] = {(double)rhobar, (double)rel0 * rhobar, (double)rel1 * rhobar};
        double bb[3];
        for (int c = 0; c < 3; ++c) bb[c] = Pi[c] * yb[0] + Pi[3 + c] * yb[1] + Pi[6 + c] * yb[2];
        sb[0] = bb[0];
        sb[2] = bb[1];
        sb[3] = bb[2];
        // A's entries and the moments they hold: (den, xi0 VW, xi1 VW; V g0, xi0 V g0, xi0 V g1;
        // V g1, xi1 V g0, xi1 V g1)
        const int mom[9] = {1, 6, 7, 4, 8, 9, 5, 10, 11};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) sb[mom[3 * r + c]] = -bb[r] * y[c];
    } else if (cnt > 0) {
        const double dd = a[1] + 1e-7;
        sb[0] = rhobar / dd;
        sb[1] = -rhobar * a[0] / (dd * dd);
    } else {
        return;
    }
    int total = 0;
    for (int q = 0; q < nr; ++q) total += re[q] - rs[q];
    const float cg20 = -20.f * P.kc.cg * P.inv_h;
    int r = 0, base = 0;
    for (int t = lane; t < total; t += 32) {
        while (t >= base + (re[r] - rs[r])) {
            base += re[r] - rs[r];
            ++r;
        }
        const int j = rs[r] + (t - base);
        const float4 xj = __ldg(&X4[j]);
        if (is_boundary(xj.z)) continue;
        float d0, d1;
        pair_vec<PER>(gw, make_float2(xj.x, xj.y), P.geo, d0, d1);
        const float sq = sq_norm_ref(d0, d1);
        if (sq > P.T) continue;
        const double dr = sqrt((double)sq);
        const double q = dr * P.inv_h;
        const double om = 1.0 - q;
        const double Wv = om * om * om * om * (1.0 + 4.0 * q) * P.kc.cw;
        const double W1 = -20.0 * q * om * om * om * P.kc.cg;   // dW/dr
        const double Wr = (double)cg20 * om * om * om;           // W'/r
        const double W2 = (double)cg20 * om * om * (1.0 - 4.0 * q);  // d2W/dr2
        const double e0 = dr > 0.0 ? d0 / dr : 0.0, e1 = dr > 0.0 ? d1 / dr : 0.0;
        const double g0 = W1 * e0, g1 = W1 * e1;
        const double V = (double)P.m / xj.z;
        const double xi0 = -(double)d0, xi1 = -(double)d1;
        // E = cW W + cg . g (+ the xi dependence below)
        const double cW = sb[0] * P.m + sb[1] * V + V * (sb[6] * xi0 + sb[7] * xi1);
        const double cg0 = sb[2] * P.m + sb[4] * V + V * (sb[8] * xi0 + sb[10] * xi1);
        const double cg1 = sb[3] * P.m + sb[5] * V + V * (sb[9] * xi0 + sb[11] * xi1);
        // Jg cg, Jg = W2 e e^T + Wr (I - e e^T)
        const double ec = e0 * cg0 + e1 * cg1;
        const double J0 = W2 * ec * e0 + Wr * (cg0 - ec * e0), J1 = W2 * ec * e1 + Wr * (cg1 - ec * e1);
        const double Gd0 = cW * W1 * e0 + J0 - V * Wv * sb[6] - V * (sb[8] * g0 + sb[9] * g1);
        const double Gd1 = cW * W1 * e1 + J1 - V * Wv * sb[7] - V * (sb[10] * g0 + sb[11] * g1);
        // the V-proportional moments, for d/d rho_j (V = m / rho_j)
        const double VE = V * (sb[1] * Wv + sb[4] * g0 + sb[5] * g1 + Wv * (sb[6] * xi0 + sb[7] * xi1) +
                               sb[8] * xi0 * g0 + sb[9] * xi0 * g1 + sb[10] * xi1 * g0 + sb[11] * xi1 * g1);
        atomicAdd(&xacc[2 * (int64_t)j], -Gd0);
        atomicAdd(&xacc[2 * (int64_t)j + 1], -Gd1);
        atomicAdd(&racc[j], -VE / xj.z);
    }
}

__global__ void k_wall_adjoint_fin(int64_t n, int nF, const int32_t* __restrict__ uid,
                                   const double* __restrict__ xacc, const double* __restrict__ racc,
                                   float* __restrict__ xbar, float* __restrict__ rbar) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = uid[s];
    if (o >= nF) return;
    xbar[2 * o] += (float)xacc[2 * s];
    xbar[2 * o + 1] += (float)xacc[2 * s + 1];
    rbar[o] += (float)racc[s];
}

}  // namespace sph

using namespace sph;


// Cells of half the search radius with a 5x5 stencil: the stencil covers skin * h around
// the cell, with fewer candidates than a 3x3 stencil of full-radius cells.
constexpr int kSolverRad = 2;
static double cell_size(const sph_params_t* p) { return p->support * p->skin * (1.0 + 1e-4) / kSolverRad; }

static Grid dom_grid(const sph_params_t* p, int64_t* ncells) {
    int per[2] = {p->domain.periodic[0], p->domain.periodic[1]};
    return make_grid(p->domain.min, p->domain.max, per, cell_size(p), ncells, kSolverRad);
}

static size_t solver_layout(const sph_params_t* p, const int64_t* nF_d, int nd, int64_t nB, void* ws,
                            sph_solver* S) {
    int64_t nF = 0, ncells = 0;
    for (int d = 0; d < nd; ++d) {
        nF += nF_d[d];
        int64_t nc = 0;
        dom_grid(&p[d], &nc);
        ncells += nc;
    }
    int64_t n = nF + nB;
    Carver c{(char*)ws};
    float2* Xr = c.take<float2>(n);
    float2* Xr_t = c.take<float2>(n);
    float2* Xs = c.take<float2>(n);
    float4* X[4];
    float4* V[4];
    for (int k = 0; k < 4; ++k) X[k] = c.take<float4>(n);
    for (int k = 0; k < 4; ++k) V[k] = c.take<float4>(n);
    int32_t* uid = c.take<int32_t>(n);
    int32_t* uid_t = c.take<int32_t>(n);
    int32_t* did = c.take<int32_t>(n);
    int32_t* did_t = c.take<int32_t>(n);
    int32_t* key = c.take<int32_t>(n);
    int32_t* perm = c.take<int32_t>(n);
    int32_t* slot = c.take<int32_t>(n);
    int32_t* count = c.take<int32_t>(ncells);
    int32_t* fill = c.take<int32_t>(ncells);
    int32_t* start = c.take<int32_t>(ncells + 1);
    int32_t* scan32 = c.take<int32_t>(scan_tmp_elems(ncells));
    int32_t* bidx = c.take<int32_t>(nB);
    uint32_t* words = c.take<uint32_t>(8);
    uint32_t* maxv = c.take<uint32_t>(nd);
    Dom* doms = c.take<Dom>(nd);
    int64_t* dom_off = c.take<int64_t>(nd + 1);
    float2* bnormal = c.take<float2>(nB);
    float* bdist = c.take<float>(nB);
    int16_t* nl = c.take<int16_t>(tile_elems(n, kStoreCap));
    int16_t* nlc = c.take<int16_t>(n);
    int16_t* sl = c.take<int16_t>(tile_elems(n, kSkinCap));
    int16_t* slc = c.take<int16_t>(n);
    float* msums = c.take<float>(nB * kMdbcSums);
    if (S) {
        S->msums = msums;
        S->nl = nl;
        S->nlc = nlc;
        S->sl = sl;
        S->slc = slc;
        S->n = n;
        S->nF = nF;
        S->nB = nB;
        S->ncells = ncells;
        S->Xr = Xr; S->Xr_t = Xr_t; S->Xs = Xs;
        S->Xc = X[0]; S->Xh = X[1]; S->Xf = X[2]; S->Xt = X[3];
        S->Vc = V[0]; S->Vh = V[1]; S->Vf = V[2]; S->Vt = V[3];
        S->uid = uid; S->uid_t = uid_t; S->did = did; S->did_t = did_t; S->slot = slot;
        S->key = key; S->perm = perm; S->count = count; S->fill = fill; S->start = start; S->scan32 = scan32;
        S->bidx = bidx; S->words = words; S->maxv = maxv; S->doms = doms; S->dom_off = dom_off;
        S->bnormal = bnormal; S->bdist = bdist;
    }
    return c.off;
}

static int check_params(const sph_params_t* p, int64_t nF, int64_t nB) {
    if (!p || nF < 1 || nB < 0 || nF + nB >= ((int64_t)1 << 31) - 1) return SPH_ERR_ARGUMENT;
    if (!(p->support > 0) || !(p->dx > 0) || !(p->mass > 0) || !(p->rho0 > 0) || !(p->cs > 0)) return SPH_ERR_ARGUMENT;
    if (!(p->skin >= 1.0) || !(p->kernel_scale > 0)) return SPH_ERR_ARGUMENT;
    // the summation density replaces the integrated one: the rational density update (an
    // option of this library, not the reference's observable update) does not apply to it
    if (p->density_scheme < 0 || p->density_scheme > 1 || (p->density_scheme == 1 && p->density_update != 0))
        return SPH_ERR_ARGUMENT;
    for (int a = 0; a < 2; ++a)
        if (!(p->domain.max[a] > p->domain.min[a])) return SPH_ERR_ARGUMENT;
    int64_t ncells = 0;
    dom_grid(p, &ncells);
    if (ncells > ((int64_t)1 << 28)) return SPH_ERR_ARGUMENT;
    return SPH_OK;
}

// Largest fp32 s with fl(fl(sqrt(s)) / h) <= 1 under IEEE round-to-nearest. Both steps are
// monotone in s, so the reference's test q <= 1 is exactly s <= T for a uniform h.
static float exact_threshold(float h) {
    volatile float hv = h;
    auto ok = [&](float s) {
        volatile float r = sqrtf(s);
        volatile float q = r / hv;
        return q <= 1.0f;
    };
    float s = h * h;
    for (int k = 0; k < 64 && !ok(s); ++k) s = nextafterf(s, 0.0f);
    for (int k = 0; k < 64 && ok(nextafterf(s, INFINITY)); ++k) s = nextafterf(s, INFINITY);
    return s;
}

static Phys make_phys(const sph_params_t* p, int64_t nF) {
    Phys P;
    int per[2] = {p->domain.periodic[0], p->domain.periodic[1]};
    P.geo = make_geo(p->domain.min, p->domain.max, per);
    double h = p->support;
    P.h = (float)h;
    P.T = exact_threshold((float)h);
    P.inv_h = (float)(1.0 / h);
    P.m = (float)p->mass;
    P.dt = (float)p->dt;
    P.dth = (float)(p->dt / 2.0);
    P.kc.cw = (float)(kCd / (h * h));
    P.kc.cg = (float)(kCd / (h * h * h));
    P.eos.B = (float)(p->rho0 * p->cs * p->cs / p->gamma);
    P.eos.rho0 = (float)p->rho0;
    P.eos.gamma = (float)p->gamma;
    P.rho0 = (float)p->rho0;
    P.diff_coef = (float)((float)((float)p->delta * (float)h) / (float)p->kernel_scale * (float)p->cs);
    P.diff_eps = (float)(1e-6f * (float)h);
    P.v_eps = (float)p->eps * (float)(h * h);
    P.v_num = p->visc_scheme ? (float)((float)((float)p->alpha * (float)h) * (float)p->cs * (float)p->rho0)
                             : (float)(2.0 * (2 + 2) * p->nu * p->rho0);
    P.dvnum_dnu = p->visc_scheme ? 0.f : (float)(2.0 * (2 + 2) * p->rho0);
    P.bvisc = p->bvisc_scheme;
    P.bv_eps = (float)p->b_eps * (float)(h * h);
    P.bv_num = p->bvisc_scheme ? (float)((float)((float)p->b_alpha * (float)h) * (float)p->cs * (float)p->rho0)
                               : (float)(2.0 * (2 + 2) * p->b_nu * p->rho0);
    P.gx = p->gravity_on ? (float)p->gravity[0] : 0.f;
    P.gy = p->gravity_on ? (float)p->gravity[1] : 0.f;
    P.nF = (int)nF;
    {  // W0 = W(dx/h, h) evaluated in fp32 like the reference (shifting.py:122)
        float q0 = (float)(p->dx / h);  // torch.tensor(dx / support): the double quotient, rounded
        float om = 1.f - q0;
        float hh = (float)h;
        float W0 = (om * om) * (om * om) * (1.f + 4.f * q0) * (float)(7.0 / M_PI) / (hh * hh);
        P.invW0 = 1.0f / W0;
    }
    P.shR = (float)p->shift_R;
    P.shN = (float)p->shift_n;
    P.shN4 = p->shift_n == 4.0;
    P.sh_thr = (float)(p->shift_threshold * p->dx);
    {
        float t = (float)h / (float)p->kernel_scale * 2.f;
        P.sh_scale = -(float)p->shift_CFL * (t * t);
    }
    P.inv_cs = (float)(1.0 / p->cs);
    P.compute_mach = p->compute_mach;
    P.density_update = p->density_update;
    // displacement allowed between the sort and the last pass of the step; the shift clamp
    // (at most sqrt(2) threshold dx) is reserved out of the cell margin
    P.verlet_lim = (float)((p->skin - 1.0) * h - 1.5 * p->shift_threshold * p->dx);
    // pairs within h later were within h + 2 D at the sort for displacements D <= skin_lim
    P.T_skin = (float)((h * (1.0 + kSkinFrac)) * (h * (1.0 + kSkinFrac)) * (1.0 + 1e-4));
    P.skin_lim = (float)(0.5 * kSkinFrac * h * 0.98);
    P.area = (float)(p->dx * p->dx);  // areas = full(n, dx * dx) in fp32
    return P;
}

static int check_batch(const sph_params_t* params, const int64_t* n_fluid, int nd, int64_t nB) {
    if (!params || !n_fluid || nd < 1) return SPH_ERR_ARGUMENT;
    if (nd > 1 && nB != 0) return SPH_ERR_ARGUMENT;  // packed batches are fluid-only
    int64_t tot = 0, cells = 0;
    for (int d = 0; d < nd; ++d) {
        int st = check_params(&params[d], n_fluid[d], d == 0 ? nB : 0);
        if (st) return st;
        if (params[d].density_scheme != params[0].density_scheme) return SPH_ERR_ARGUMENT;
        tot += n_fluid[d];
        int64_t nc = 0;
        dom_grid(&params[d], &nc);
        cells += nc;
    }
    if (tot + nB >= ((int64_t)1 << 31) - 1 || cells >= ((int64_t)1 << 30)) return SPH_ERR_ARGUMENT;
    return SPH_OK;
}

static int create_impl(const sph_params_t* params, const int64_t* n_fluid, int nd, int64_t n_boundary,
                       void* workspace, size_t workspace_bytes, sph_solver_t** out) {
    int st = check_batch(params, n_fluid, nd, n_boundary);
    if (st) return st;
    if (!out) return SPH_ERR_ARGUMENT;
    size_t need = solver_layout(params, n_fluid, nd, n_boundary, nullptr, nullptr);
    if (!workspace || workspace_bytes < need) return SPH_ERR_WORKSPACE;
    if (((uintptr_t)workspace & 255) != 0) return SPH_ERR_ARGUMENT;
    sph_solver* S = new sph_solver();
    S->prm = params[0];
    S->nd = nd;
    solver_layout(params, n_fluid, nd, n_boundary, workspace, S);
    S->periodic = false;
    S->doms_host.resize(nd);
    S->off_host.resize(nd + 1);
    int64_t off = 0, cell0 = 0;
    double span_max = 0.0;
    for (int d = 0; d < nd; ++d) {
        Dom& D = S->doms_host[d];
        memset(&D, 0, sizeof(Dom));
        D.P = make_phys(&params[d], S->nF);
        int64_t nc = 0;
        D.g = dom_grid(&params[d], &nc);
        D.g.slot0 = (int)off;
        D.g.nslots = (int)(n_fluid[d] + (nd == 1 ? n_boundary : 0));
        D.cell0 = (int32_t)cell0;
        cell0 += nc;
        S->off_host[d] = off;
        off += n_fluid[d];
        S->periodic = S->periodic || params[d].domain.periodic[0] || params[d].domain.periodic[1];
        // one-sided slot span of a stencil: rad rows of cells plus rad + 1 cells, at the rest
        // density (cell/dx)^2 per cell with a 1.5x compression margin
        double ppc = (cell_size(&params[d]) / params[d].dx) * (cell_size(&params[d]) / params[d].dx);
        // (periodic offsets are stored modulo the domain's slots: the same bound holds across
        // the wrap)
        double span = ((double)kSolverRad * D.g.nc[0] + kSolverRad + 1) * ppc * 1.5;
        span_max = span > span_max ? span : span_max;
    }
    S->off_host[nd] = off;
    S->list16 = span_max < 32767.0;
    *out = S;
    return SPH_OK;
}

extern "C" int sph_solver_workspace_bytes(const sph_params_t* params, int64_t n_fluid, int64_t n_boundary,
                                          size_t* bytes) {
    int st = check_batch(params, &n_fluid, 1, n_boundary);
    if (st) return st;
    if (!bytes) return SPH_ERR_ARGUMENT;
    *bytes = solver_layout(params, &n_fluid, 1, n_boundary, nullptr, nullptr);
    return SPH_OK;
}

extern "C" int sph_solver_create(const sph_params_t* params, int64_t n_fluid, int64_t n_boundary, void* workspace,
                                 size_t workspace_bytes, sph_solver_t** out) {
    return create_impl(params, &n_fluid, 1, n_boundary, workspace, workspace_bytes, out);
}

extern "C" int sph_batch_workspace_bytes(const sph_params_t* params, const int64_t* n_fluid, int32_t n_domains,
                                         size_t* bytes) {
    int st = check_batch(params, n_fluid, n_domains, 0);
    if (st) return st;
    if (!bytes) return SPH_ERR_ARGUMENT;
    *bytes = solver_layout(params, n_fluid, n_domains, 0, nullptr, nullptr);
    return SPH_OK;
}

extern "C" int sph_batch_create(const sph_params_t* params, const int64_t* n_fluid, int32_t n_domains,
                                void* workspace, size_t workspace_bytes, sph_solver_t** out) {
    return create_impl(params, n_fluid, n_domains, 0, workspace, workspace_bytes, out);
}

extern "C" void sph_solver_destroy(sph_solver_t* s) {
    if (!s) return;
    for (int k = 0; k < 2; ++k)
        if (s->graph[k]) cudaGraphExecDestroy(s->graph[k]);
    for (auto& e : s->pool) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    delete s;
}



extern "C" int sph_solver_upload(sph_solver_t* S, const float* x_fluid, const float* u_fluid, const float* rho_fluid,
                                 const float* x_boundary, const float* normal_boundary, const float* dist_boundary,
                                 const float* rho_boundary, sph_stream_t stream) {
    if (!S || !x_fluid || !u_fluid || !rho_fluid) return SPH_ERR_ARGUMENT;
    if (S->nB > 0 && (!x_boundary || !normal_boundary || !dist_boundary)) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (!S->tables_uploaded) {
        if (cudaMemcpyAsync(S->doms, S->doms_host.data(), sizeof(Dom) * S->nd, cudaMemcpyHostToDevice, st) != cudaSuccess)
            return SPH_ERR_CUDA;
        if (cudaMemcpyAsync(S->dom_off, S->off_host.data(), sizeof(int64_t) * (S->nd + 1), cudaMemcpyHostToDevice,
                            st) != cudaSuccess)
            return SPH_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return SPH_ERR_CUDA;
        S->tables_uploaded = true;
    }
    if (S->reuse && S->uploaded && S->nd == 1) {
        // keep the current order (and the pending-sort and skin-list words): the next step's
        // displacement check sorts when the new positions are too far from the last sort's
        k_upload_keep<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->nF, S->slot, x_fluid, u_fluid, rho_fluid,
                                                             x_boundary, normal_boundary, dist_boundary,
                                                             rho_boundary, S->doms_host[0].P, S->Xr, S->Xc, S->Vc,
                                                             S->bnormal, S->bdist);
        if (cudaMemsetAsync(S->words, 0, sizeof(uint32_t), st) != cudaSuccess) return SPH_ERR_CUDA;
        if (cudaMemsetAsync(S->words + 5, 0, sizeof(uint32_t), st) != cudaSuccess) return SPH_ERR_CUDA;
        return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
    }
    k_upload<<<blocks_for(S->n), kBlock, 0, st>>>(S->nF, S->nB, x_fluid, u_fluid, rho_fluid, x_boundary,
                                                    normal_boundary, dist_boundary, rho_boundary, S->doms, S->dom_off,
                                                    S->nd, S->Xr, S->Xc, S->Vc, S->uid, S->slot, S->did, S->bnormal,
                                                    S->bdist);
    if (cudaMemsetAsync(S->words, 0, sizeof(uint32_t) * 8, st) != cudaSuccess) return SPH_ERR_CUDA;
    // a new state is always sorted first
    if (cudaMemsetAsync(S->words + 4, 1, sizeof(uint32_t), st) != cudaSuccess) return SPH_ERR_CUDA;
    S->uploaded = true;
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// sort by cell and gather the state into the new order
// With Verlet reuse the sort runs only when k_verlet_check asks for it (words[4]); its kernels
// are launched every step and return at once otherwise, so a captured graph covers both
// cases. in_step: the caller is a step, whose first pass A branches on words[4] too (it is
// left set) and rebuilds the skin list after a sort.
static int rebuild(sph_solver* S, cudaStream_t st, bool in_step = false) {
    const uint32_t* gate = S->reuse ? S->words + 4 : nullptr;
    if (S->reuse)
        k_verlet_check<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->Xr, S->Xs, S->words,
                                                            S->reuse_lim * S->reuse_lim, S->doms,
                                                            S->nd > 1 ? S->did : nullptr, S->reuse_half);
    else if (cudaMemsetAsync(S->words + 4, 1, sizeof(uint32_t), st) != cudaSuccess)
        return SPH_ERR_CUDA;
    k_sort_begin<<<1, 32, 0, st>>>(S->words, in_step ? 1 : 0);
    tbeg(S, KC_SORT, st);
    if (cudaMemsetAsync(S->count, 0, sizeof(int32_t) * S->ncells, st) != cudaSuccess) return SPH_ERR_CUDA;
    k_dom_keys<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->Xc, S->nd > 1 ? S->did : nullptr, S->doms, S->key,
                                                      S->count, gate);
    if (cell_sort_counted(S->n, S->ncells, S->key, S->perm, S->count, S->fill, S->start, S->scan32, st, gate) !=
        cudaSuccess)
        return SPH_ERR_CUDA;
    tend(S, KC_SORT, st);
    tbeg(S, KC_GATHER, st);
    k_gather<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, (int)S->nF, S->perm, S->Xr, S->Xc, S->Vc, S->uid, S->did,
                                                    S->Xr_t, S->Xt, S->Vt, S->uid_t, S->did_t, S->bidx, S->words,
                                                    S->Xs, S->slot, gate);
    if (S->reuse)
        k_copy_back<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->Xr_t, S->Xt, S->Vt, S->uid_t, S->did_t, S->Xr,
                                                          S->Xc, S->Vc, S->uid, S->did, gate);
    tend(S, KC_GATHER, st);
    if (!S->reuse) {
        std::swap(S->Xr, S->Xr_t);
        std::swap(S->Xc, S->Xt);
        std::swap(S->Vc, S->Vt);
        std::swap(S->uid, S->uid_t);
        std::swap(S->did, S->did_t);
    } else if (!in_step && cudaMemsetAsync(S->words + 4, 0, sizeof(uint32_t), st) != cudaSuccess) {
        return SPH_ERR_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

static const int32_t* dids(sph_solver* S) { return S->nd > 1 ? S->did : nullptr; }

static void launch_mdbc(sph_solver* S, float4* X4, float* rho_b_out, cudaStream_t st) {
    if (S->nB == 0) return;
    tbeg(S, KC_MDBC, st);
    const Dom& D = S->doms_host[0];
    const unsigned gw = (unsigned)((S->nB + 3) / 4);
    if (S->periodic)
        k_mdbc_sums<true><<<gw, 128, 0, st>>>((int)S->nB, S->bidx, S->uid, S->Xr, X4, S->bnormal, S->bdist, S->start,
                                              D.g, D.P, S->msums);
    else
        k_mdbc_sums<false><<<gw, 128, 0, st>>>((int)S->nB, S->bidx, S->uid, S->Xr, X4, S->bnormal, S->bdist, S->start,
                                               D.g, D.P, S->msums);
    // 64-thread blocks: the solve is bound by each SM's FP64 rate, so its warps are spread
    // over every SM (24.6 k walls in 256-thread blocks filled 96 of the 152)
    k_mdbc_solve<<<blocks_for(S->nB, kMdbcSolveBlock), kMdbcSolveBlock, 0, st>>>((int)S->nB, S->bidx, S->uid, S->Xr, X4, S->bnormal, S->bdist,
                                                       D.P, S->msums, rho_b_out);
    tend(S, KC_MDBC, st);
}


template <bool PER, bool BATCH, typename LT, int W, bool PS>
static void allow_lists_k(int b) {
    cudaFuncSetAttribute(k_pass_a<PER, BATCH, LT, W, false, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(k_pass_a<PER, BATCH, LT, W, true, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(k_pass_b<PER, BATCH, 0, LT, W, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(k_pass_b<PER, BATCH, 1, LT, W, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(k_pass_b<PER, BATCH, 2, LT, W, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(k_shift<PER, BATCH, LT, W, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(k_density_sum<PER, BATCH, LT, W, PS>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
}

template <typename LT, int W, bool PS>
static void allow_lists_s() {
    const int b = (int)list_bytes<LT, W>();
    allow_lists_k<true, false, LT, W, PS>(b);
    allow_lists_k<false, false, LT, W, PS>(b);
    allow_lists_k<true, true, LT, W, PS>(b);
    allow_lists_k<false, true, LT, W, PS>(b);
}

static void set_attrs(sph_solver* S) {
    if (S->attrs_set) return;
    allow_lists_s<int32_t, 4, false>();
    allow_lists_s<int16_t, 4, false>();
    allow_lists_s<int16_t, 8, false>();
    allow_lists_s<int16_t, 16, false>();
    allow_lists_s<int16_t, 8, true>();
    S->attrs_set = true;
}

// dispatch a launcher template over the shape table
#define SPH_SHAPE_DISPATCH(SH, CALL)                  \
    switch (SH) {                                     \
        case 1: CALL(int16_t, 4, false); break;       \
        case 2: CALL(int16_t, 8, false); break;       \
        case 3: CALL(int16_t, 16, false); break;      \
        case 4: CALL(int16_t, 8, true); break;        \
        default: CALL(int32_t, 4, false); break;      \
    }

// skin_mode: 0 keeps the skin list (first pass A after a sort), 1 filters it (second pass A
// of the same step), 2 neither; 3 and 4 are 0 and 1 decided on the device by words[4]
static int pass_a_tuned(int skin_mode) { return (skin_mode == 1 || skin_mode == 4) ? TP_A_FILTER : TP_A_SCAN; }

template <bool PER, bool BATCH, typename LT, int W, bool PS>
static void launch_a_k(sph_solver* S, float4* X4, float4* V4, RhsOut o, int skin_mode, cudaStream_t st) {
    const int tp = pass_a_tuned(skin_mode), sh = S->shape_of[tp];
    const size_t sm = list_bytes<LT, W>();
    if (skin_mode == 0 || skin_mode == 3) {
        auto kern = k_pass_a<PER, BATCH, LT, W, true, PS>;
        kern<<<pass_grid(S, tp, sh, kern, 32 * W, sm), 32 * W, sm, st>>>(
            S->doms_host[0], S->n, X4, V4, S->start, S->doms, dids(S), S->uid, o, S->words, S->nl, S->nlc, skin_mode,
            S->sl, S->slc);
    } else {
        auto kern = k_pass_a<PER, BATCH, LT, W, false, PS>;
        kern<<<pass_grid(S, tp, sh, kern, 32 * W, sm), 32 * W, sm, st>>>(
            S->doms_host[0], S->n, X4, V4, S->start, S->doms, dids(S), S->uid, o, S->words, S->nl, S->nlc, skin_mode,
            S->sl, S->slc);
    }
}

template <typename LT, int W, bool PS>
static void launch_a_t(sph_solver* S, float4* X4, float4* V4, RhsOut o, int skin_mode, cudaStream_t st) {
    if (S->nd > 1) {
        if (S->periodic) launch_a_k<true, true, LT, W, PS>(S, X4, V4, o, skin_mode, st);
        else launch_a_k<false, true, LT, W, PS>(S, X4, V4, o, skin_mode, st);
    } else {
        if (S->periodic) launch_a_k<true, false, LT, W, PS>(S, X4, V4, o, skin_mode, st);
        else launch_a_k<false, false, LT, W, PS>(S, X4, V4, o, skin_mode, st);
    }
}

static void launch_a(sph_solver* S, float4* X4, float4* V4, RhsOut o, cudaStream_t st, int skin_mode = 2) {
    set_attrs(S);
    const int cls = (skin_mode == 1 || skin_mode == 4) ? KC_PASS_A : KC_PASS_A_SCAN;
    tbeg(S, cls, st);
#define SPH_CALL_A(LT, W, PS) launch_a_t<LT, W, PS>(S, X4, V4, o, skin_mode, st)
    SPH_SHAPE_DISPATCH(S->shape_of[pass_a_tuned(skin_mode)], SPH_CALL_A)
#undef SPH_CALL_A
    tend(S, cls, st);
}

template <bool PER, bool BATCH, int MODE, typename LT, int W, bool PS>
static void launch_b_k(sph_solver* S, float4* X4, float4* V4, RhsOut o, float4* X4o, float4* V4o, cudaStream_t st) {
    const size_t sm = list_bytes<LT, W>();
    auto kern = k_pass_b<PER, BATCH, MODE, LT, W, PS>;
    kern<<<pass_grid(S, TP_B, S->shape_of[TP_B], kern, 32 * W, sm), 32 * W, sm, st>>>(
        S->doms_host[0], S->n, X4, V4, S->start, S->doms, dids(S), S->uid, o, S->Xr, S->Xc, S->Vc, X4o, V4o,
        S->words, S->maxv, S->nl, S->nlc, S->Xs);
}

template <int MODE, typename LT, int W, bool PS>
static void launch_b_t(sph_solver* S, float4* X4, float4* V4, RhsOut o, float4* X4o, float4* V4o, cudaStream_t st) {
    if (S->nd > 1) {
        if (S->periodic) launch_b_k<true, true, MODE, LT, W, PS>(S, X4, V4, o, X4o, V4o, st);
        else launch_b_k<false, true, MODE, LT, W, PS>(S, X4, V4, o, X4o, V4o, st);
    } else {
        if (S->periodic) launch_b_k<true, false, MODE, LT, W, PS>(S, X4, V4, o, X4o, V4o, st);
        else launch_b_k<false, false, MODE, LT, W, PS>(S, X4, V4, o, X4o, V4o, st);
    }
}

template <int MODE>
static void launch_b(sph_solver* S, float4* X4, float4* V4, RhsOut o, float4* X4o, float4* V4o, cudaStream_t st) {
    set_attrs(S);
    tbeg(S, KC_PASS_B, st);
#define SPH_CALL_B(LT, W, PS) launch_b_t<MODE, LT, W, PS>(S, X4, V4, o, X4o, V4o, st)
    SPH_SHAPE_DISPATCH(S->shape_of[TP_B], SPH_CALL_B)
#undef SPH_CALL_B
    tend(S, KC_PASS_B, st);
}

template <bool PER, bool BATCH, typename LT, int W, bool PS>
static void launch_dsum_k(sph_solver* S, const float4* Xin, float4* Xout, int skin_mode, cudaStream_t st) {
    const size_t sm = list_bytes<LT, W>();
    auto kern = k_density_sum<PER, BATCH, LT, W, PS>;
    kern<<<pass_grid(S, TP_DENSITY, S->shape_of[TP_DENSITY], kern, 32 * W, sm), 32 * W, sm, st>>>(
        S->doms_host[0], S->n, Xin, Xout, S->start, S->doms, dids(S), S->words, skin_mode, S->sl, S->slc);
}

template <typename LT, int W, bool PS>
static void launch_dsum_t(sph_solver* S, const float4* Xin, float4* Xout, int skin_mode, cudaStream_t st) {
    if (S->nd > 1) {
        if (S->periodic) launch_dsum_k<true, true, LT, W, PS>(S, Xin, Xout, skin_mode, st);
        else launch_dsum_k<false, true, LT, W, PS>(S, Xin, Xout, skin_mode, st);
    } else {
        if (S->periodic) launch_dsum_k<true, false, LT, W, PS>(S, Xin, Xout, skin_mode, st);
        else launch_dsum_k<false, false, LT, W, PS>(S, Xin, Xout, skin_mode, st);
    }
}

// Summation density of the state Xin into Xout (skin_mode as k_density_sum)
static void launch_dsum(sph_solver* S, const float4* Xin, float4* Xout, cudaStream_t st, int skin_mode) {
    set_attrs(S);
    tbeg(S, KC_DENSITY, st);
#define SPH_CALL_D(LT, W, PS) launch_dsum_t<LT, W, PS>(S, Xin, Xout, skin_mode, st)
    SPH_SHAPE_DISPATCH(S->shape_of[TP_DENSITY], SPH_CALL_D)
#undef SPH_CALL_D
    tend(S, KC_DENSITY, st);
}

static bool summation(const sph_solver* S) { return S->prm.density_scheme == 1; }

// the step keeps a skin list for its later passes (walled domains always; periodic ones
// under Verlet reuse)
static bool uses_skin(const sph_solver* S) { return !S->periodic || S->reuse; }

static int run_stages(sph_solver* S, cudaStream_t st) {
    RhsOut none = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int rc = rebuild(S, st, true);
    if (rc) return rc;
    // skin list: kept by the first pass A after a sort and filtered by the later passes;
    // periodic domains keep it only under Verlet reuse (sorting every step, the cost of
    // keeping it is not won back: the stencil scan skips the minimum image on most ranges)
    const int skin = uses_skin(S) ? 0 : 2;
    // stage 1 at t^n. With the summation density the stage reads the state with the summed
    // densities from the spare buffer Xt (free between the sort and the next step)
    float4* X1 = S->Xc;
    if (summation(S)) {
        launch_dsum(S, S->Xc, S->Xt, st, S->reuse ? 4 : 2);
        X1 = S->Xt;
    }
    launch_mdbc(S, X1, nullptr, st);
    if (S->reuse) {
        // after a sort: scan and keep the skin list; otherwise filter the one kept
        launch_a(S, X1, S->Vc, none, st, 3);
        launch_a(S, X1, S->Vc, none, st, 4);
        if (cudaMemsetAsync(S->words + 4, 0, sizeof(uint32_t), st) != cudaSuccess) return SPH_ERR_CUDA;
    } else {
        launch_a(S, X1, S->Vc, none, st, skin);
    }
    launch_b<1>(S, X1, S->Vc, none, S->Xh, S->Vh, st);
    // stage 2 at the half step; the epilogue also reduces max |u'| for the shifting Mach number.
    // With the summation density the half-step densities are replaced by the sums at the
    // half-step positions, which the final update keeps (the reference's state sync,
    // integration.py:439-513, takes the temporary state's densities)
    float4* X2 = S->Xh;
    if (summation(S)) {
        launch_dsum(S, S->Xh, S->Xt, st, skin == 0 ? 1 : 2);
        X2 = S->Xt;
    }
    launch_mdbc(S, X2, nullptr, st);
    launch_a(S, X2, S->Vh, none, st, skin == 0 ? 1 : 2);
    if (cudaMemsetAsync(S->maxv, 0, sizeof(uint32_t) * S->nd, st) != cudaSuccess) return SPH_ERR_CUDA;
    launch_b<2>(S, X2, S->Vh, none, S->Xf, S->Vf, st);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

template <bool PER, bool BATCH, typename LT, int W, bool PS>
static void launch_shift_k(sph_solver* S, float4* Xin, float4* Vin, float4* Xout, float4* Vout, float* dx_out,
                           int use_skin, cudaStream_t st) {
    const size_t sm = list_bytes<LT, W>();
    auto kern = k_shift<PER, BATCH, LT, W, PS>;
    kern<<<pass_grid(S, TP_SHIFT, S->shape_of[TP_SHIFT], kern, 32 * W, sm), 32 * W, sm, st>>>(
        S->doms_host[0], S->n, Xin, Vin, S->start, S->doms, dids(S), S->Xr, Xout, Vout, S->words, S->maxv,
        S->prm.shift_on, S->uid, dx_out, use_skin, S->sl, S->slc, surface_view(S));
}

template <typename LT, int W, bool PS>
static void launch_shift_t(sph_solver* S, float4* Xin, float4* Vin, float4* Xout, float4* Vout, float* dx_out,
                           int use_skin, cudaStream_t st) {
    if (S->nd > 1) {
        if (S->periodic) launch_shift_k<true, true, LT, W, PS>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st);
        else launch_shift_k<false, true, LT, W, PS>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st);
    } else {
        if (S->periodic) launch_shift_k<true, false, LT, W, PS>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st);
        else launch_shift_k<false, false, LT, W, PS>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st);
    }
}

// use_skin: the skin list of this step's first pass A is valid for this sort (same step)
static void launch_shift(sph_solver* S, float4* Xin, float4* Vin, float4* Xout, float4* Vout, float* dx_out,
                         cudaStream_t st, int use_skin = 0) {
    set_attrs(S);
    tbeg(S, KC_SHIFT, st);
#define SPH_CALL_S(LT, W, PS) launch_shift_t<LT, W, PS>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st)
    SPH_SHAPE_DISPATCH(S->shape_of[TP_SHIFT], SPH_CALL_S)
#undef SPH_CALL_S
    tend(S, KC_SHIFT, st);
}

static int step_impl(sph_solver* S, int32_t n_steps, cudaStream_t st) {
    for (int it = 0; it < n_steps; ++it) {
        int rc = run_stages(S, st);
        if (rc) return rc;
        // shifting at the integrated positions, on the same cell sort and skin list
        rc = surface_detect(S, S->Xf, S->periodic ? 0 : 1, st);
        if (rc) return rc;
        if (S->ips) {
            rc = ips_shift(S, S->Xf, S->Vf, S->Xc, S->Vc, nullptr, S->periodic ? 0 : 1, st);
            if (rc) return rc;
        } else {
            launch_shift(S, S->Xf, S->Vf, S->Xc, S->Vc, nullptr, st, uses_skin(S) ? 1 : 0);
        }
        if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
    }
    return SPH_OK;
}

extern "C" int sph_solver_step(sph_solver_t* S, int32_t n_steps, sph_stream_t stream) {
    if (!S || n_steps < 0) return SPH_ERR_ARGUMENT;
    return step_impl(S, n_steps, (cudaStream_t)stream);
}

// The step sequence is static, so a fixed number of steps can be captured once into a CUDA
// graph and replayed. Every step swaps the sorted/gather buffers, so an even number of steps
// returns the handle to the buffer assignment it was captured with; under Verlet reuse the
// assignment never changes and any number of steps can be captured.
extern "C" int sph_solver_graph_step(sph_solver_t* S, int32_t n_steps, sph_stream_t stream) {
    if (!S || n_steps < 1 || (!S->reuse && (n_steps & 1))) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (st == nullptr) return SPH_ERR_ARGUMENT;  // the legacy default stream cannot be captured
    // a graph bakes in which buffer holds the current state; eager steps, integrate and
    // shift rotate the assignment, so graphs are keyed by it as well as by the step count
    const void* bufs[14] = {S->Xr, S->Xr_t, S->Xc, S->Xh, S->Xf, S->Xt, S->Vc,
                            S->Vh, S->Vf, S->Vt, S->uid, S->uid_t, S->did, S->did_t};
    for (int k = 0; k < 2; ++k)
        if (S->graph[k] && S->graph_n[k] == n_steps && memcmp(bufs, S->graph_key[k], sizeof(bufs)) == 0)
            return cudaGraphLaunch(S->graph[k], st) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
    const int slot = S->graph_next;
    if (S->graph[slot]) {
        cudaGraphExecDestroy(S->graph[slot]);
        S->graph[slot] = nullptr;
    }
    set_attrs(S);
    uint32_t mask = S->timing_mask;
    S->timing_mask = 0;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return SPH_ERR_CUDA;
    int rc = step_impl(S, n_steps, st);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    S->timing_mask = mask;
    if (rc || e != cudaSuccess || !g) {  // the capture is invalid: drop what it recorded
        if (g) cudaGraphDestroy(g);
        return rc ? rc : SPH_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&S->graph[slot], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return SPH_ERR_CUDA;
    S->graph_n[slot] = n_steps;
    memcpy(S->graph_key[slot], bufs, sizeof(bufs));
    S->graph_next = 1 - slot;
    return cudaGraphLaunch(S->graph[slot], st) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_integrate(sph_solver_t* S, sph_stream_t stream) {
    if (!S) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = run_stages(S, st);
    if (rc) return rc;
    std::swap(S->Xc, S->Xf);
    std::swap(S->Vc, S->Vf);
    return SPH_OK;
}

extern "C" int sph_solver_shift(sph_solver_t* S, float* dx_out, sph_stream_t stream) {
    if (!S) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = rebuild(S, st);
    if (rc) return rc;
    if (cudaMemsetAsync(S->maxv, 0, sizeof(uint32_t) * S->nd, st) != cudaSuccess) return SPH_ERR_CUDA;
    k_maxvel<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->Vc, dids(S), S->maxv);
    rc = surface_detect(S, S->Xc, 0, st);
    if (rc) return rc;
    if (S->ips) {
        rc = ips_shift(S, S->Xc, S->Vc, S->Xt, S->Vt, dx_out, 0, st);
        if (rc) return rc;
    } else {
        launch_shift(S, S->Xc, S->Vc, S->Xt, S->Vt, dx_out, st);
    }
    std::swap(S->Xc, S->Xt);
    std::swap(S->Vc, S->Vt);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// The autotuner times every pass it shapes separately, on the current state, under each
// shape: a fresh sort at the current positions first (so that the skin list the timed
// scanning pass A keeps belongs to it), then pass A scanning, pass A filtering that list,
// the shift (into the spare buffers, with the raw positions it moves saved and restored),
// the summation density and pass B (half-step update into the spare stage buffers). The
// skin list is marked invalid at the end, so a Verlet-reuse step sorts again first.
extern "C" int sph_solver_autotune(sph_solver_t* S, int32_t* shapes_out, float* ms_out, sph_stream_t stream) {
    if (!S) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(S->words + 3, 1, sizeof(uint32_t), st) != cudaSuccess) return SPH_ERR_CUDA;
    int rc = rebuild(S, st);
    if (rc) return rc;
    set_attrs(S);
    RhsOut none = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return SPH_ERR_CUDA;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return SPH_ERR_CUDA;
    }
    const uint32_t saved_mask = S->timing_mask;
    const bool saved_fs = S->fs_on;
    S->timing_mask = 0;
    S->fs_on = false;
    const bool skin = uses_skin(S);
    const int order[TP_COUNT] = {TP_A_SCAN, TP_A_FILTER, TP_SHIFT, TP_DENSITY, TP_B};
    rc = SPH_OK;
    for (int oi = 0; oi < TP_COUNT && rc == SPH_OK; ++oi) {
        const int tp = order[oi];
        const bool applies = tp == TP_A_SCAN || tp == TP_B || (tp == TP_A_FILTER && skin) ||
                             (tp == TP_SHIFT && !S->ips) || (tp == TP_DENSITY && summation(S));
        auto run = [&]() {
            switch (tp) {
                case TP_A_SCAN: launch_a(S, S->Xc, S->Vc, none, st, skin ? 0 : 2); break;
                case TP_A_FILTER: launch_a(S, S->Xc, S->Vc, none, st, 1); break;
                case TP_B: launch_b<1>(S, S->Xc, S->Vc, none, S->Xh, S->Vh, st); break;
                case TP_SHIFT: launch_shift(S, S->Xc, S->Vc, S->Xt, S->Vt, nullptr, st, skin ? 1 : 0); break;
                default: launch_dsum(S, S->Xc, S->Xt, st, skin ? 1 : 2); break;
            }
        };
        if (tp == TP_SHIFT && applies &&
            cudaMemcpyAsync(S->Xr_t, S->Xr, sizeof(float2) * S->n, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
            rc = SPH_ERR_CUDA;
            break;
        }
        float best = 1e30f;
        int best_shape = 0;
        for (int k = 0; k < kNumShapes; ++k) {
            float ms = -1.f;
            if (applies && (!kShapes[k].list16 || S->list16)) {
                S->shape_of[tp] = k;
                run();  // warm-up
                cudaEventRecord(a, st);
                for (int r = 0; r < 3; ++r) run();
                cudaEventRecord(b, st);
                if (cudaEventSynchronize(b) != cudaSuccess) {
                    rc = SPH_ERR_CUDA;
                    break;
                }
                cudaEventElapsedTime(&ms, a, b);
                ms /= 3.f;
                if (ms < best) {
                    best = ms;
                    best_shape = k;
                }
            }
            if (ms_out) ms_out[tp * kNumShapes + k] = ms;
        }
        S->shape_of[tp] = best_shape;
        // the scanning pass A kept the skin list at the sort positions: valid for the filters
        if (tp == TP_A_SCAN && !S->periodic &&
            cudaMemsetAsync(S->words + 3, 0, sizeof(uint32_t), st) != cudaSuccess)
            rc = SPH_ERR_CUDA;
        if (tp == TP_SHIFT && applies &&
            cudaMemcpyAsync(S->Xr, S->Xr_t, sizeof(float2) * S->n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            rc = SPH_ERR_CUDA;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    S->timing_mask = saved_mask;
    S->fs_on = saved_fs;
    if (cudaMemsetAsync(S->words + 3, 1, sizeof(uint32_t), st) != cudaSuccess) rc = rc ? rc : SPH_ERR_CUDA;
    for (int k = 0; k < 2; ++k) {  // a captured graph holds the old shapes' kernels
        if (S->graph[k]) cudaGraphExecDestroy(S->graph[k]);
        S->graph[k] = nullptr;
    }
    if (shapes_out)
        for (int p = 0; p < TP_COUNT; ++p) shapes_out[p] = S->shape_of[p];
    if (rc) return rc;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SPH_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}


// ------------------------------------------------------------------------------------
// Adjoint entry points (single domain, delta+ shift without the free-surface handling,
// continuity density), evaluated at the current state; gradients accumulate (+=) into the
// caller's arrays (original order). With walls the wall-density adjoint accumulates into
// rhob_bar (original wall order), which sph_solver_vjp_walls pulls back to the fluid.
// ------------------------------------------------------------------------------------
static int adjoint_ok(sph_solver* S) {
    if (!S || S->nd != 1 || summation(S) || S->ips || S->fs_on) return SPH_ERR_ARGUMENT;
    return SPH_OK;
}

extern "C" int sph_solver_vjp_rates(sph_solver_t* S, const float* abar, const float* drbar, float* xbar, float* ubar,
                                    float* rbar, float* Gbar, float* nu_part, float* rhob_bar, sph_stream_t stream) {
    int rc = adjoint_ok(S);
    if (rc) return rc;
    if (!abar || !xbar || !ubar || !rbar || (S->nB > 0 && !rhob_bar)) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = rebuild(S, st))) return rc;
    RhsOut none = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    launch_mdbc(S, S->Xc, nullptr, st);   // the wall densities of the current state
    launch_a(S, S->Xc, S->Vc, none, st);  // gradRho^L of the current state (pass-B inputs)
    const Dom& D = S->doms_host[0];
    k_lam_rates<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->Xc, S->uid, D, abar, drbar, S->Xh, S->Xf);
    unsigned gb = blocks_for(S->n * kAdjL, 128);  // kAdjL lanes per particle
    if (S->periodic)
        k_vjp_rates<true><<<gb, 128, 0, st>>>(S->n, S->Xc, S->Vc, S->start, D, S->uid, S->Xh, S->Xf, S->words, xbar,
                                              ubar, rbar, Gbar, nu_part, rhob_bar);
    else
        k_vjp_rates<false><<<gb, 128, 0, st>>>(S->n, S->Xc, S->Vc, S->start, D, S->uid, S->Xh, S->Xf, S->words, xbar,
                                               ubar, rbar, Gbar, nu_part, rhob_bar);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_vjp_gradient(sph_solver_t* S, const float* Gbar, float* xbar, float* rbar, float* rhob_bar,
                                       sph_stream_t stream) {
    int rc = adjoint_ok(S);
    if (rc) return rc;
    if (!Gbar || !xbar || !rbar || (S->nB > 0 && !rhob_bar)) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = rebuild(S, st))) return rc;
    launch_mdbc(S, S->Xc, nullptr, st);  // the wall densities of the current state
    const Dom& D = S->doms_host[0];
    unsigned gb = blocks_for(S->n * kAdjL, 128);  // kAdjL lanes per particle
    if (S->periodic) {
        k_lam_grad<true><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, Gbar, S->words, S->Xh, S->Xf);
        k_vjp_grad<true><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, S->Xh, S->Xf, S->words, xbar, rbar,
                                             rhob_bar);
    } else {
        k_lam_grad<false><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, Gbar, S->words, S->Xh, S->Xf);
        k_vjp_grad<false><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, S->Xh, S->Xf, S->words, xbar, rbar,
                                              rhob_bar);
    }
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_vjp_shift(sph_solver_t* S, const float* xbar_new, float* xbar, float* rbar,
                                    float* mach_part, float* rhob_bar, sph_stream_t stream) {
    int rc = adjoint_ok(S);
    if (rc) return rc;
    if (!xbar_new || !xbar || !rbar || !mach_part || (S->nB > 0 && !rhob_bar)) return SPH_ERR_ARGUMENT;
    if (!S->prm.shift_on) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = rebuild(S, st))) return rc;
    if (cudaMemsetAsync(S->maxv, 0, sizeof(uint32_t), st) != cudaSuccess) return SPH_ERR_CUDA;
    k_maxvel<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->Vc, nullptr, S->maxv);
    const Dom& D = S->doms_host[0];
    unsigned gb = blocks_for(S->n * kAdjL, 128);  // kAdjL lanes per particle
    if (S->periodic) {
        k_lam_shift<true><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, S->maxv, xbar_new, S->words, S->Xh,
                                              mach_part);
        k_vjp_shift<true><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, S->Xh, xbar_new, S->words, xbar,
                                              rbar, rhob_bar);
    } else {
        k_lam_shift<false><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, S->maxv, xbar_new, S->words,
                                               S->Xh, mach_part);
        k_vjp_shift<false><<<gb, 128, 0, st>>>(S->n, S->Xc, S->start, D, S->uid, S->Xh, xbar_new, S->words, xbar,
                                               rbar, rhob_bar);
    }
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_vjp_walls(sph_solver_t* S, const float* rhob_bar, float* xbar, float* rbar,
                                    sph_stream_t stream) {
    int rc = adjoint_ok(S);
    if (rc) return rc;
    if (S->nB == 0) return SPH_OK;
    if (!rhob_bar || !xbar || !rbar) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = rebuild(S, st))) return rc;
    // fp64 accumulators by slot in the spare state buffers (free between a sort and a step)
    double* xacc = reinterpret_cast<double*>(S->Xt);
    double* racc = reinterpret_cast<double*>(S->Vt);
    if (cudaMemsetAsync(xacc, 0, sizeof(double) * 2 * S->n, st) != cudaSuccess) return SPH_ERR_CUDA;
    if (cudaMemsetAsync(racc, 0, sizeof(double) * S->n, st) != cudaSuccess) return SPH_ERR_CUDA;
    const Dom& D = S->doms_host[0];
    const unsigned gw = (unsigned)((S->nB + 3) / 4);
    if (S->periodic)
        k_mdbc_vjp<true><<<gw, 128, 0, st>>>((int)S->nB, S->bidx, S->uid, S->Xr, S->Xc, S->bnormal, S->bdist,
                                             S->start, D.g, D.P, rhob_bar, xacc, racc);
    else
        k_mdbc_vjp<false><<<gw, 128, 0, st>>>((int)S->nB, S->bidx, S->uid, S->Xr, S->Xc, S->bnormal, S->bdist,
                                              S->start, D.g, D.P, rhob_bar, xacc, racc);
    k_wall_adjoint_fin<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, (int)S->nF, S->uid, xacc, racc, xbar, rbar);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// One right-hand side at the current state: the summation density (when configured), the
// wall densities (mDBC, or the caller's rho_b_in), pass A and pass B with the rates written
static int rhs_impl(sph_solver* S, const float* rho_b_in, float* dudt, float* drhodt, float* grad_rho, float* L,
                    float* pressure, float* rho_boundary, int32_t* num_neighbors, cudaStream_t st) {
    int rc = rebuild(S, st);
    if (rc) return rc;
    RhsOut o = {dudt, drhodt, grad_rho, L, pressure, rho_boundary, num_neighbors};
    float4* X = S->Xc;
    if (summation(S)) {
        launch_dsum(S, S->Xc, S->Xt, st, 2);
        X = S->Xt;
    }
    if (rho_b_in) {
        if (S->nB > 0)
            k_set_walls<<<blocks_for(S->nB), kBlock, 0, st>>>((int)S->nB, S->bidx, S->uid, X, S->doms_host[0].P,
                                                              rho_b_in);
    } else {
        launch_mdbc(S, X, rho_boundary, st);
    }
    launch_a(S, X, S->Vc, o, st);
    launch_b<0>(S, X, S->Vc, o, nullptr, nullptr, st);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_rhs(sph_solver_t* S, float* dudt, float* drhodt, float* grad_rho, float* L, float* pressure,
                              float* rho_boundary, int32_t* num_neighbors, sph_stream_t stream) {
    if (!S || !dudt || !drhodt) return SPH_ERR_ARGUMENT;
    return rhs_impl(S, nullptr, dudt, drhodt, grad_rho, L, pressure, rho_boundary, num_neighbors,
                    (cudaStream_t)stream);
}

extern "C" int sph_solver_rhs_walls(sph_solver_t* S, const float* rho_boundary_in, float* dudt, float* drhodt,
                                    float* grad_rho, float* L, float* pressure, int32_t* num_neighbors,
                                    sph_stream_t stream) {
    if (!S || !dudt || !drhodt || (S->nB > 0 && !rho_boundary_in)) return SPH_ERR_ARGUMENT;
    return rhs_impl(S, rho_boundary_in, dudt, drhodt, grad_rho, L, pressure, nullptr, num_neighbors,
                    (cudaStream_t)stream);
}

extern "C" int sph_solver_download(sph_solver_t* S, float* x_fluid, float* u_fluid, float* rho_fluid,
                                   float* rho_boundary, sph_stream_t stream) {
    if (!S) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    k_download<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, (int)S->nF, S->slot, S->Xr, S->Xc, S->Vc, x_fluid,
                                                      u_fluid, rho_fluid, rho_boundary);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_flags(sph_solver_t* S, uint32_t* flags_host, sph_stream_t stream) {
    if (!S || !flags_host) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(flags_host, S->words, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SPH_ERR_CUDA;
    return SPH_OK;
}

extern "C" int sph_solver_launches_per_step(const sph_solver_t* S) {
    if (!S) return -1;
    // cell keys, scan (3), scatter, cell order, gather, 2 x (mdbc moments and solve?, pass A, pass B), shift;
    // the free-surface passes (detection, normals, expansions) when on. An implicit shift adds
    // its solve's launches (1 + 5 per iteration + 1 in place of the shift), which depend on
    // how many iterations it runs.
    // Verlet reuse launches the displacement check, the copy back of a sort and the first
    // pass A both ways (one returns at once), every step
    // The summation density adds one launch per right-hand side.
    const int fs = (S->fs_on && S->prm.shift_on) ? 2 + S->fs_expand : 0;
    return 8 + 2 * ((S->nB > 0 ? 2 : 0) + 2 + (summation(S) ? 1 : 0)) + 1 + fs + (S->reuse ? 3 : 0);
}

extern "C" int sph_solver_set_verlet_reuse(sph_solver_t* S, int32_t on) {
    if (!S || on < 0 || on > 1) return SPH_ERR_ARGUMENT;
    if (S->reuse != (on == 1)) {
        // the captured sequences differ (and so does the buffer rotation of a sort)
        for (int k = 0; k < 2; ++k) {
            if (S->graph[k]) cudaGraphExecDestroy(S->graph[k]);
            S->graph[k] = nullptr;
        }
    }
    S->reuse = on == 1;
    // a sort ahead of the skin list's limit (0.049 h): a step moves particles up to about
    // 0.013 h in the first steps of a dam break, so the list keeps holding every pair through
    // the step that crosses 0.034 h
    S->reuse_lim = 0.7f * S->doms_host[0].P.skin_lim;
    return SPH_OK;
}

extern "C" int sph_solver_set_verlet_scale(sph_solver_t* S, double verlet_scale) {
    if (!S || !(verlet_scale > 1.0)) return SPH_ERR_ARGUMENT;
    // the reference rebuilds once 2 max|dx| > (verletScale - 1) h; the skin list of this solver
    // holds every pair up to 0.049 h of displacement, and sorting at 0.7 of that keeps it
    // complete through the step that crosses the limit: the stricter of the two applies
    const float ref_lim = (float)((verlet_scale - 1.0) * S->doms_host[0].P.h * 0.5);
    const float own_lim = 0.7f * S->doms_host[0].P.skin_lim;
    S->reuse_lim = ref_lim < own_lim ? ref_lim : own_lim;
    S->reuse_half = (float)((verlet_scale - 1.0) * 0.5);
    return SPH_OK;
}

extern "C" int sph_solver_sort_count(sph_solver_t* S, uint32_t* sorts, sph_stream_t stream) {
    if (!S || !sorts) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(sorts, S->words + 5, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return SPH_ERR_CUDA;
    return cudaStreamSynchronize(st) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_kernel_classes(void) { return KC_COUNT; }

extern "C" int sph_solver_shapes(void) { return kNumShapes; }
extern "C" int sph_solver_tuned_passes(void) { return TP_COUNT; }

extern "C" int sph_solver_set_pass_shape(sph_solver_t* S, int32_t pass, int32_t shape) {
    if (!S || shape < 0 || shape >= kNumShapes || pass < -1 || pass >= TP_COUNT) return SPH_ERR_ARGUMENT;
    if (kShapes[shape].list16 && !S->list16) return SPH_ERR_ARGUMENT;
    for (int p = 0; p < TP_COUNT; ++p)
        if (pass < 0 || p == pass) S->shape_of[p] = shape;
    for (int k = 0; k < 2; ++k) {  // a captured graph holds the old shapes' kernels
        if (S->graph[k]) cudaGraphExecDestroy(S->graph[k]);
        S->graph[k] = nullptr;
    }
    return SPH_OK;
}

extern "C" int sph_solver_set_shape(sph_solver_t* S, int32_t shape) { return sph_solver_set_pass_shape(S, -1, shape); }

extern "C" int sph_solver_pass_shapes(const sph_solver_t* S, int32_t* shapes_out) {
    if (!S || !shapes_out) return SPH_ERR_ARGUMENT;
    for (int p = 0; p < TP_COUNT; ++p) shapes_out[p] = S->shape_of[p];
    return SPH_OK;
}

extern "C" const char* sph_solver_kernel_name(int cls) {
    return kernel_class_name(cls);
}

extern "C" int sph_solver_set_timing(sph_solver_t* S, int32_t enabled) {
    if (!S) return SPH_ERR_ARGUMENT;
    S->timing_mask = (uint32_t)enabled;
    return SPH_OK;
}

extern "C" int sph_solver_kernel_times(sph_solver_t* S, float* ms_host, int32_t* launches_host, sph_stream_t stream) {
    if (!S || !ms_host || !launches_host) return SPH_ERR_ARGUMENT;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return SPH_ERR_CUDA;
    for (int c = 0; c < KC_COUNT; ++c) {
        ms_host[c] = 0.f;
        launches_host[c] = 0;
    }
    for (size_t k = 0; k < S->used; ++k) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, S->pool[k].a, S->pool[k].b) != cudaSuccess) return SPH_ERR_CUDA;
        ms_host[S->pool[k].cls] += ms;
        launches_host[S->pool[k].cls] += 1;
    }
    S->used = 0;
    return SPH_OK;
}
