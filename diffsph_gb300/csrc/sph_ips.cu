// Implicit particle shifting (shifting.scheme = 'IPS') for sm_103a.
//
// Follows computeShifting (src/diffSPH/v2/modules/shifting.py:780-880) as solveShifting
// (:882-1019) calls it with the default parameters: no free-surface handling,
// shifting.summationDensity off (omega_j = the particle area dx^2), initialization 'zero'.
// The system (getShiftingMatrices, :611-705) has one 2x2 block per pair,
//   H_ij = Hessian W(x_ij) omega_j          (KernelWrapper.Hessian2D, src/diffSPH/kernels.py:263-303)
//   b_i  = sum_j grad W(x_ij) omega_j        (kernelGradient, kernelFunctions/Wendland2.py:32-34)
// with wall rows removed (b_i = 0, no H row), and is solved by bicgstab_shifting (:322-493):
// unpreconditioned BiCGStab (the Jacobi matrix it receives is never applied) from x = 0,
// returning at |r| < rtol |b|, at |s| < rtol |b| mid-iteration, on the rho / rv / omega
// breakdowns and as soon as any particle's |x_i| exceeds solverThreshold. The shift is then
// clamp(x_i, +-threshold dx) on fluid particles, applied as the delta+ update is.
//
// Layout: the solve runs on the cell-sorted slots of the step. The first kernel walks the
// exact neighbors once (the step's skin list, or the cell stencil), accumulates b and keeps
// the exact list (int16 slot offsets) with the three distinct entries of each pair's block
// (12 B per pair), both warp-tile-major, which the matrix products then stream; a row longer
// than the stored list is rescanned with H recomputed from the positions. Vectors are float2
// per slot; dot products take exact fp64 products of the fp32 entries, summed per block and
// then over blocks in block order by the last block to finish, so the scalars are
// deterministic; they are rounded to fp32, the precision of the reference's 0-dim tensors.
// A solve is 1 + 5 launches per iteration + 1: the iteration kernels return at once after the
// solve has returned, and the host stops launching at the next check.
#include <math.h>
#include <string.h>

#include "sph_solver.cuh"

namespace sph {

struct IpsState {
    float rho;          // r . r0 of the current iteration
    float alpha, omega, beta;
    float atol;         // rtol |b|
    int iter;           // current iteration; the iteration count once done
    int done;           // the solve has returned
    int code;           // bicgstab_shifting's second return value
    int final_alpha;    // |s| < atol: x += alpha p, then return
    unsigned count;     // blocks finished (last-block reduction)
    unsigned xmax;      // max |x_i| of the iteration (float bits)
    unsigned pad[5];
};

constexpr int kIpsBlock = 256;   // elementwise kernels
constexpr int kIpsW = 4;         // warps per block of the neighbor kernels
constexpr int kIpsSums = 3;      // partial sums per block
constexpr size_t kIpsMaxBlocks = 8 * 1024;  // the grids are capped at 8 blocks per SM
constexpr float kRhoTol = 1.4210854715202004e-14f;  // float32 eps^2 (rhotol = omegatol)

// Sums of K values over the block in a fixed order; the result is valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sums(const double (&v)[K], double (&out)[K]) {
    __shared__ double sh[K][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    double w[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        w[k] = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w[k] += __shfl_down_sync(kFull, w[k], o);
    }
    __syncthreads();  // sh may still be read by a previous call
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) sh[k][warp] = w[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0.0;
            for (int q = 0; q < nw; ++q) s += sh[k][q];
            out[k] = s;
        }
}

// Every block stores its sums; the block that finishes last adds them up in block order
// (the same order whichever block that is) and calls fin(totals) in its thread 0. Every
// thread of every block must call it.
template <int K, class Fin>
__device__ __forceinline__ void grid_sums(const double (&v)[K], double* __restrict__ part, IpsState* st, Fin&& fin) {
    __shared__ bool last;
    double b[K];
    block_sums<K>(v, b);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) part[(size_t)blockIdx.x * K + k] = b[k];
        __threadfence();
        last = atomicAdd(&st->count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += __ldcg(&part[(size_t)q * K + k]);
    double tot[K];
    block_sums<K>(acc, tot);
    if (threadIdx.x == 0) {
        st->count = 0u;
        fin(tot);
    }
}

// Largest value over the block (valid in thread 0); every thread must call it.
__device__ __forceinline__ unsigned block_max(unsigned v) {
    __shared__ unsigned shm[32];
    v = __reduce_max_sync(kFull, v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned m = 0u;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) m = shm[q] > m ? shm[q] : m;
    return m;
}

__device__ __forceinline__ double dot2(float2 a, float2 b) { return (double)a.x * b.x + (double)a.y * b.y; }

__device__ __forceinline__ void finish(IpsState* st, int iters, int code) {
    st->iter = iters;
    st->code = code;
    st->done = 1;
}

// Kernel Hessian of one pair in the reference's closed form (src/diffSPH/kernels.py:263-303):
//   d2W/dx2 = C/h^2 (x^2 k''/(h^2 r^2 + 1e-5 h) + y^2 k'/(h r^3 + 1e-10 h) + [q < 1e-5] k''(0)/h^2)
//   d2W/dxdy = C h^-2 x y/(h r^2 + 1e-5 h) (k''/h - k'/(r + 1e-3 h))
// with k' = -20 q (1-q)^3, k'' = 20 (4q - 1)(1-q)^2 (Wendland2.py:12-22) and x = xhat r.
struct HessK {
    float h, h2, inv_h, fac, cdh2, e5h, e10h, e3h, self_term;
};

__device__ __forceinline__ HessK hess_k(float h) {
    HessK K;
    K.h = h;
    K.h2 = h * h;
    K.inv_h = 1.0f / h;
    K.fac = kCd / K.h2;
    K.cdh2 = kCd * (1.0f / K.h2);
    K.e5h = 1e-5f * h;
    K.e10h = 1e-10f * h;
    K.e3h = 1e-3f * h;
    K.self_term = (1.0f / K.h2) * -20.0f;  // d2kdq2(0) = -20
    return K;
}

__device__ __forceinline__ void pair_hessian(float q, float xh0, float xh1, const HessK& K, float& hxx, float& hxy,
                                             float& hyy) {
    const float r = q * K.h;
    const float x0 = xh0 * r, x1 = xh1 * r;
    const float om = fminf(fmaxf(1.f - q, 0.f), 1.f);
    const float k2 = 20.f * (4.f * q - 1.f) * (om * om);
    const float k1 = -20.f * q * (om * om * om);
    const float r2 = r * r;
    const float iA = __fdividef(1.f, K.h2 * r2 + K.e5h);
    const float iB = __fdividef(1.f, K.h * (r2 * r) + K.e10h);
    const float st = q < 1e-5f ? K.self_term : 0.f;
    const float ax = x0 * x0, ay = x1 * x1;
    hxx = K.fac * (ax * iA * k2 + ay * iB * k1 + st);
    hyy = K.fac * (ay * iA * k2 + ax * iB * k1 + st);
    hxy = K.cdh2 * ((x0 * x1) * __fdividef(1.f, K.h * r2 + K.e5h) *
                    (K.inv_h * k2 - __fdividef(1.f, r + K.e3h) * k1));
}

// The exact list and its blocks are stored warp-tile-major: for the 32 slots of a warp, list
// position k, component c at ((tile * kStoreCap + k) * 3 + c) * 32 + lane, so that one warp's
// data is one contiguous run (the products stream it with full DRAM pages). Vectors are float2
// per slot.
struct IpsVec {
    float2 *x, *r, *r0, *p, *ap, *s, *as;
    float* H;        // [tiles][kStoreCap][3][32]: xx, xy, yy
    int16_t* nl;     // [tiles][kStoreCap][32]: slot offsets
    int16_t* nlc;    // [n]: list length (-1: not stored)
};

__host__ __device__ inline int64_t tile_pad(int64_t n) { return (n + 31) & ~(int64_t)31; }

__device__ __forceinline__ int64_t nl_at(int64_t i, int k) { return ((i >> 5) * kStoreCap + k) * 32 + (i & 31); }
__device__ __forceinline__ int64_t h_at(int64_t i, int k, int c) {
    return (((i >> 5) * kStoreCap + k) * 3 + c) * 32 + (i & 31);
}

// ---- b, the exact list with its blocks, and the initial vectors ---------------------------
template <bool PER, typename LT, int W>
__global__ void __launch_bounds__(32 * W)
    k_ips_setup(const Dom D, int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ start,
                uint32_t* __restrict__ words, int use_skin, const int16_t* __restrict__ sl,
                const int16_t* __restrict__ slc, IpsVec V, double* __restrict__ part, IpsState* st, float rtol,
                int maxiter, const SurfaceView sv) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    const Phys& P = D.P;
    const Grid& g = D.g;
    const HessK K = hess_k(P.h);
    const int64_t ntiles = (n + 32 * W - 1) / (32 * W);
    double bb = 0.0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {  // block-uniform
        const int64_t i = tile * (32 * W) + threadIdx.x;
        const bool inb = i < n;
        const float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, -1.f, 0.f);
        // surface rows leave the system like wall rows (getShiftingMatrices :657-678)
        const bool active = inb && !is_boundary(xi.z) && !(sv.fs && sv.fs[i]);
        const float2 pi = make_float2(xi.x, xi.y);
        float b0 = 0.f, b1 = 0.f;
        int nst = 0;
        bool unstored = false;
        auto pair_j = [&](int j) {
            int d = j - (int)i;
            if (PER) {
                const int h2 = g.nslots >> 1;
                if (d > h2) d -= g.nslots;
                else if (d < -h2) d += g.nslots;
            }
            const bool store = nst < kStoreCap && d >= -32768 && d <= 32767;
            const float4 xj = __ldg(&X4[j]);
            float x0, x1;
            pair_vec<PER>(pi, make_float2(xj.x, xj.y), P.geo, x0, x1);
            const PairG pg = pair_fast(x0, x1, sq_norm_ref(x0, x1), P.inv_h);
            if (store) {
                V.nl[nl_at(i, nst)] = (int16_t)d;
                float hxx, hxy, hyy;
                pair_hessian(pg.q, pg.xh0, pg.xh1, K, hxx, hxy, hyy);
                V.H[h_at(i, nst, 0)] = hxx;
                V.H[h_at(i, nst, 1)] = hxy;
                V.H[h_at(i, nst, 2)] = hyy;
            } else {
                unstored = true;
            }
            ++nst;
            const float dW = wendland_dw(pg.q, P.kc);
            b0 = fmaf(pg.xh0 * dW, P.area, b0);
            b1 = fmaf(pg.xh1 * dW, P.area, b1);
        };
        const int sk = (!PER && use_skin && active) ? (int)slc[i] : 0;
        if (!PER && use_skin && __all_sync(kFull, sk >= 0) && words[3] == 0u)
            skin_loop<PER>((int)i, pi, X4, g, P, sl, sk, pair_j);
        else
            neighbor_loop<PER, LT>(active, (int)i, pi, X4, start, g, P, lst, words, pair_j);
        const float2 b = make_float2(b0, b1);  // zero on wall rows
        if (inb) {
            V.nlc[i] = active ? (unstored ? (int16_t)-1 : (int16_t)nst) : (int16_t)0;
            V.x[i] = make_float2(0.f, 0.f);
            V.r[i] = b;
            V.r0[i] = b;
            V.p[i] = b;
            bb += dot2(b, b);
        }
    }
    const double v[1] = {bb};
    grid_sums<1>(v, part, st, [&](const double (&t)[1]) {
        const float bnrm = (float)sqrt(t[0]);
        st->atol = (float)fmax(0.0, (double)rtol * (double)bnrm);
        st->rho = (float)t[0];  // r . r0 = b . b
        st->final_alpha = 0;
        st->iter = 0;
        st->done = 0;
        st->code = 0;
        if (bnrm == 0.f) finish(st, 0, 0);  // returns b (= 0)
        else if (maxiter <= 0) finish(st, 0, 0);
        else if (bnrm < st->atol) finish(st, 0, 0);
        else if (fabsf(st->rho) < kRhoTol) finish(st, 0, -10);
    });
}

// ---- y = A v over the stored exact list (scan fallback), with its dot products ------------
// WHICH 0: ap = A p and ap . r0 -> alpha; WHICH 1: as = A s, as . s and as . as -> omega
// (or, when |s| already converged, x += alpha p and return).
template <bool PER, typename LT, int W, int WHICH>
__global__ void __launch_bounds__(32 * W)
    k_ips_spmv(const Dom D, int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ start,
               uint32_t* __restrict__ words, IpsVec V, double* __restrict__ part, IpsState* st) {
    if (st->done) return;
    extern __shared__ __align__(16) unsigned char s_dyn[];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    const int64_t ntiles = (n + 32 * W - 1) / (32 * W);
    if (WHICH == 1 && st->final_alpha) {
        const float alpha = st->alpha;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x) {
            const float2 x = V.x[i], p = V.p[i];
            V.x[i] = make_float2(x.x + alpha * p.x, x.y + alpha * p.y);
        }
        const double z[1] = {0.0};
        grid_sums<1>(z, part, st, [&](const double (&)[1]) { finish(st, st->iter + 1, 0); });
        return;
    }
    const Phys& P = D.P;
    const Grid& g = D.g;
    const float2* __restrict__ vin = WHICH == 0 ? V.p : V.s;
    const HessK K = hess_k(P.h);
    double acc0 = 0.0, acc1 = 0.0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {  // block-uniform
        const int64_t i = tile * (32 * W) + threadIdx.x;
        const bool inb = i < n;
        const float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, -1.f, 0.f);
        const bool active = inb && !is_boundary(xi.z);
        const float2 pi = make_float2(xi.x, xi.y);
        float y0 = 0.f, y1 = 0.f;
        auto pair_h = [&](int j) {  // a row the setup could not store: the same blocks, recomputed
            const float4 xj = __ldg(&X4[j]);
            if (is_boundary(xj.z)) return;  // wall entries of v are zero
            const float2 vj = vin[j];
            float x0, x1;
            pair_vec<PER>(pi, make_float2(xj.x, xj.y), P.geo, x0, x1);
            const PairG pg = pair_fast(x0, x1, sq_norm_ref(x0, x1), P.inv_h);
            float hxx, hxy, hyy;
            pair_hessian(pg.q, pg.xh0, pg.xh1, K, hxx, hxy, hyy);
            y0 = fmaf(hxx, vj.x, fmaf(hxy, vj.y, y0));
            y1 = fmaf(hxy, vj.x, fmaf(hyy, vj.y, y1));
        };
        const int nst = active ? (int)V.nlc[i] : 0;
        if (__any_sync(kFull, nst < 0)) {
            neighbor_loop<PER, LT>(active, (int)i, pi, X4, start, g, P, lst, words, pair_h);
        } else {
            // the blocks stored by the setup pass, in list order (wall entries of v are zero and
            // add nothing); four list positions in flight per step
            constexpr int U = 4;
            int k = 0;
            for (; k + U <= nst; k += U) {
                int j[U];
                float a[U], b[U], c[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    j[u] = list_slot<PER>((int)i, (int)V.nl[nl_at(i, k + u)], g);
                    a[u] = V.H[h_at(i, k + u, 0)];
                    b[u] = V.H[h_at(i, k + u, 1)];
                    c[u] = V.H[h_at(i, k + u, 2)];
                }
                float2 vj[U];
#pragma unroll
                for (int u = 0; u < U; ++u) vj[u] = vin[j[u]];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    y0 = fmaf(a[u], vj[u].x, fmaf(b[u], vj[u].y, y0));
                    y1 = fmaf(b[u], vj[u].x, fmaf(c[u], vj[u].y, y1));
                }
            }
            for (; k < nst; ++k) {
                const float2 vj = vin[list_slot<PER>((int)i, (int)V.nl[nl_at(i, k)], g)];
                const float a = V.H[h_at(i, k, 0)], b = V.H[h_at(i, k, 1)], c = V.H[h_at(i, k, 2)];
                y0 = fmaf(a, vj.x, fmaf(b, vj.y, y0));
                y1 = fmaf(b, vj.x, fmaf(c, vj.y, y1));
            }
        }
        const float2 y = make_float2(y0 * P.area, y1 * P.area);
        if (inb) {
            if (WHICH == 0) {
                V.ap[i] = y;
                acc0 += dot2(y, V.r0[i]);
            } else {
                V.as[i] = y;
                const float2 si = V.s[i];
                acc0 += dot2(y, si);
                acc1 += dot2(y, y);
            }
        }
    }
    if (WHICH == 0) {
        const double v[1] = {acc0};
        grid_sums<1>(v, part, st, [&](const double (&t)[1]) {
            const float rv = (float)t[0];
            if (rv == 0.f) finish(st, st->iter, -11);
            else st->alpha = st->rho / rv;
        });
    } else {
        const double v[2] = {acc0, acc1};
        grid_sums<2>(v, part, st, [&](const double (&t)[2]) { st->omega = (float)t[0] / (float)t[1]; });
    }
}

// s = r - alpha ap; |s| < atol -> final step
__global__ void __launch_bounds__(kIpsBlock) k_ips_s(int64_t n, IpsVec V, double* __restrict__ part, IpsState* st) {
    if (st->done) return;
    const float alpha = st->alpha;
    double ss = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 r = V.r[i], ap = V.ap[i];
        const float2 s = make_float2(r.x - alpha * ap.x, r.y - alpha * ap.y);
        V.s[i] = s;
        ss += dot2(s, s);
    }
    const double v[1] = {ss};
    grid_sums<1>(v, part, st, [&](const double (&t)[1]) {
        if ((float)sqrt(t[0]) < st->atol) st->final_alpha = 1;
        st->xmax = 0u;
    });
}

// x += alpha p + omega s; r = s - omega as; then the end-of-iteration and next-iteration checks
__global__ void __launch_bounds__(kIpsBlock)
    k_ips_xr(int64_t n, IpsVec V, double* __restrict__ part, IpsState* st, float threshold, int maxiter) {
    if (st->done || st->final_alpha) return;
    const float alpha = st->alpha, omega = st->omega;
    double v[2] = {0.0, 0.0};
    unsigned d = 0u;  // largest |x_i| of the thread (float bits; non-negative values order as unsigned)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 x = V.x[i], p = V.p[i], s = V.s[i], as = V.as[i];
        const float2 xn = make_float2((x.x + alpha * p.x) + omega * s.x, (x.y + alpha * p.y) + omega * s.y);
        const float2 r = make_float2(s.x - omega * as.x, s.y - omega * as.y);
        V.x[i] = xn;
        V.r[i] = r;
        v[0] += dot2(r, V.r0[i]);
        v[1] += dot2(r, r);
        const unsigned di = __float_as_uint(sqrtf(xn.x * xn.x + xn.y * xn.y));
        d = di > d ? di : d;
    }
    // the block's largest |x_i|, published by thread 0 before its fence in grid_sums
    const unsigned bm = block_max(d);
    if (threadIdx.x == 0) atomicMax(&st->xmax, bm);
    grid_sums<2>(v, part, st, [&](const double (&t)[2]) {
        const float rho_new = (float)t[0];
        st->beta = (rho_new / st->rho) * (st->alpha / st->omega);
        const int it = st->iter;
        if (it > 0 && fabsf(st->omega) < kRhoTol) {
            finish(st, it + 1, -11);
        } else if (__uint_as_float(st->xmax) > threshold) {
            finish(st, it + 1, -12);
        } else if (it + 1 >= maxiter) {
            finish(st, maxiter, maxiter);
        } else if ((float)sqrt(t[1]) < st->atol) {
            finish(st, it + 1, it + 1);
        } else if (fabsf(rho_new) < kRhoTol) {
            finish(st, it + 1, -10);
        } else {
            st->rho = rho_new;
            st->iter = it + 1;
        }
    });
}

// p = r + beta (p - omega ap)
__global__ void __launch_bounds__(kIpsBlock) k_ips_p(int64_t n, IpsVec V, const IpsState* st) {
    if (st->done) return;
    const float beta = st->beta, omega = st->omega;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 r = V.r[i], p = V.p[i], ap = V.ap[i];
        V.p[i] = make_float2(r.x + beta * (p.x - omega * ap.x), r.y + beta * (p.y - omega * ap.y));
    }
}

// update = clamp(-x, +-threshold dx) (wall rows zero); positions - update, as the delta+ path
__global__ void __launch_bounds__(kIpsBlock)
    k_ips_apply(const Dom D, int64_t n, const float4* __restrict__ X4, const float4* __restrict__ V4,
                float2* __restrict__ Xr, float4* __restrict__ X4o, float4* __restrict__ V4o, const float2* __restrict__ x,
                int enabled, const int32_t* __restrict__ uid, float* __restrict__ dx_out, const SurfaceView sv) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Phys& P = D.P;
    const float4 xi = X4[i], vi = V4[i];
    if (is_boundary(xi.z) || !enabled) {
        X4o[i] = xi;
        V4o[i] = vi;
        if (dx_out && !is_boundary(xi.z)) {
            const int o = uid[i];
            dx_out[2 * o] = 0.f;
            dx_out[2 * o + 1] = 0.f;
        }
        return;
    }
    const float2 s = x[i];
    float u0 = -s.x, u1 = -s.y;
    surface_project(sv, i, u0, u1);
    const float up0 = fminf(fmaxf(u0, -P.sh_thr), P.sh_thr);
    const float up1 = fminf(fmaxf(u1, -P.sh_thr), P.sh_thr);
    const float2 xr = Xr[i];
    const float y0 = __fsub_rn(xr.x, up0), y1 = __fsub_rn(xr.y, up1);
    const float2 xn = make_float2(__fadd_rn(xr.x, __fsub_rn(y0, xr.x)), __fadd_rn(xr.y, __fsub_rn(y1, xr.y)));
    Xr[i] = xn;
    const float2 w = wrap_pos(xn, P.geo);
    X4o[i] = make_float4(w.x, w.y, xi.z, xi.w);
    V4o[i] = vi;
    if (dx_out) {
        const int o = uid[i];
        dx_out[2 * o] = __fsub_rn(y0, xr.x);
        dx_out[2 * o + 1] = __fsub_rn(y1, xr.y);
    }
}

static unsigned ips_grid_neighbor(const sph_solver* S, int64_t n) {
    const int64_t tiles = (n + 32 * kIpsW - 1) / (32 * kIpsW);
    const int64_t cap = 8 * (int64_t)S->ips_sms;
    return (unsigned)(tiles < cap ? tiles : cap);
}

static unsigned ips_grid_vector(const sph_solver* S, int64_t n) {
    const int64_t blocks = (n + kIpsBlock - 1) / kIpsBlock;
    const int64_t cap = 4 * (int64_t)S->ips_sms;
    return (unsigned)(blocks < cap ? blocks : cap);
}

static IpsVec ips_vectors(const sph_solver* S, int64_t n) {
    IpsVec v;
    float2* base = S->ips_vec;
    v.x = base;
    v.r = base + n;
    v.r0 = base + 2 * n;
    v.p = base + 3 * n;
    v.ap = base + 4 * n;
    v.s = base + 5 * n;
    v.as = base + 6 * n;
    v.H = S->ips_H;
    v.nl = S->ips_nl;
    v.nlc = S->ips_nlc;
    return v;
}

template <bool PER, typename LT>
static void ips_launch(sph_solver* S, float4* Xin, float4* Vin, float4* Xout, float4* Vout, float* dx_out,
                       int use_skin, cudaStream_t st) {
    const int64_t n = S->n;
    const IpsVec V = ips_vectors(S, n);
    IpsState* ist = reinterpret_cast<IpsState*>(S->ips_state);
    const Dom& D = S->doms_host[0];
    // grids of a few blocks per SM: the blocks loop over the particles, and the last block's
    // sum over the per-block partials stays short
    const unsigned gn = ips_grid_neighbor(S, n), ge = ips_grid_vector(S, n);
    const size_t smem = list_bytes<LT, kIpsW>();
    cudaMemsetAsync(ist, 0, sizeof(IpsState), st);
    tbeg(S, KC_IPS_SETUP, st);
    k_ips_setup<PER, LT, kIpsW><<<gn, 32 * kIpsW, smem, st>>>(D, n, Xin, S->start, S->words, use_skin, S->sl, S->slc,
                                                               V, S->ips_part, ist, S->ips_rtol, S->ips_maxiter,
                                                               surface_view(S));
    tend(S, KC_IPS_SETUP, st);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cap);
    for (int it = 0; it < S->ips_maxiter; ++it) {
        tbeg(S, KC_IPS_SPMV, st);
        k_ips_spmv<PER, LT, kIpsW, 0><<<gn, 32 * kIpsW, smem, st>>>(D, n, Xin, S->start, S->words, V, S->ips_part, ist);
        tend(S, KC_IPS_SPMV, st);
        tbeg(S, KC_IPS_VECTOR, st);
        k_ips_s<<<ge, kIpsBlock, 0, st>>>(n, V, S->ips_part, ist);
        tend(S, KC_IPS_VECTOR, st);
        tbeg(S, KC_IPS_SPMV, st);
        k_ips_spmv<PER, LT, kIpsW, 1><<<gn, 32 * kIpsW, smem, st>>>(D, n, Xin, S->start, S->words, V, S->ips_part, ist);
        tend(S, KC_IPS_SPMV, st);
        tbeg(S, KC_IPS_VECTOR, st);
        k_ips_xr<<<ge, kIpsBlock, 0, st>>>(n, V, S->ips_part, ist, S->ips_thr, S->ips_maxiter);
        tend(S, KC_IPS_VECTOR, st);
        tbeg(S, KC_IPS_VECTOR, st);
        k_ips_p<<<ge, kIpsBlock, 0, st>>>(n, V, ist);
        tend(S, KC_IPS_VECTOR, st);
        // outside a graph capture, stop launching once the solve has returned (checked every
        // 4 iterations: one host round trip per check)
        if (cap == cudaStreamCaptureStatusNone && (it & 3) == 3 && it + 1 < S->ips_maxiter) {
            int done = 0;
            if (cudaMemcpyAsync(&done, &ist->done, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) break;
            if (cudaStreamSynchronize(st) != cudaSuccess || done) break;
        }
    }
    tbeg(S, KC_IPS_VECTOR, st);
    k_ips_apply<<<blocks_for(n, kIpsBlock), kIpsBlock, 0, st>>>(D, n, Xin, Vin, S->Xr, Xout, Vout, V.x,
                                                                S->prm.shift_on, S->uid, dx_out, surface_view(S));
    tend(S, KC_IPS_VECTOR, st);
}

}  // namespace sph


// IPS workspace: vectors [7][n] float2, blocks [tiles][kStoreCap][3][32] float, list
// [tiles][kStoreCap][32] int16, lengths [n] int16, partial sums, the solve's scalars
static size_t ips_layout(int64_t n, char* base, sph_solver* S) {
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t np = (size_t)tile_pad(n);
    const size_t sz[6] = {up(7 * (size_t)n * sizeof(float2)), up(3 * (size_t)kStoreCap * np * sizeof(float)),
                          up((size_t)kStoreCap * np * sizeof(int16_t)), up((size_t)n * sizeof(int16_t)),
                          up(kIpsMaxBlocks * kIpsSums * sizeof(double)), up(sizeof(IpsState))};
    if (S && base) {
        char* w = base;
        S->ips_vec = reinterpret_cast<float2*>(w);
        w += sz[0];
        S->ips_H = reinterpret_cast<float*>(w);
        w += sz[1];
        S->ips_nl = reinterpret_cast<int16_t*>(w);
        w += sz[2];
        S->ips_nlc = reinterpret_cast<int16_t*>(w);
        w += sz[3];
        S->ips_part = reinterpret_cast<double*>(w);
        w += sz[4];
        S->ips_state = w;
    }
    return sz[0] + sz[1] + sz[2] + sz[3] + sz[4] + sz[5];
}

size_t ips_workspace_bytes(int64_t n) { return ips_layout(n, nullptr, nullptr); }

int ips_shift(sph_solver* S, float4* Xin, float4* Vin, float4* Xout, float4* Vout, float* dx_out, int use_skin,
              cudaStream_t st) {
    if (!S->ips || S->nd != 1) return SPH_ERR_ARGUMENT;
    if (S->periodic) {
        if (S->list16) ips_launch<true, int16_t>(S, Xin, Vin, Xout, Vout, dx_out, 0, st);
        else ips_launch<true, int32_t>(S, Xin, Vin, Xout, Vout, dx_out, 0, st);
    } else {
        if (S->list16) ips_launch<false, int16_t>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st);
        else ips_launch<false, int32_t>(S, Xin, Vin, Xout, Vout, dx_out, use_skin, st);
    }
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_solver_ips_workspace_bytes(const sph_solver_t* S, size_t* bytes) {
    if (!S || !bytes) return SPH_ERR_ARGUMENT;
    *bytes = ips_workspace_bytes(S->n);
    return SPH_OK;
}

extern "C" int sph_solver_set_ips(sph_solver_t* S, const sph_ips_params_t* p, void* workspace,
                                  size_t workspace_bytes) {
    if (!S) return SPH_ERR_ARGUMENT;
    // captured graphs hold the other shifting scheme's launches
    for (int k = 0; k < 2; ++k)
        if (S->graph[k]) {
            cudaGraphExecDestroy(S->graph[k]);
            S->graph[k] = nullptr;
            S->graph_n[k] = 0;
        }
    if (!p) {
        S->ips = false;
        return SPH_OK;
    }
    if (S->nd != 1 || !workspace || !(p->rtol >= 0.0) || p->max_iter < 0 || !(p->solver_threshold > 0.0))
        return SPH_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return SPH_ERR_ARGUMENT;
    if (workspace_bytes < ips_workspace_bytes(S->n)) return SPH_ERR_WORKSPACE;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms <= 0 || sms > 1024)
        return SPH_ERR_CUDA;
    S->ips_sms = sms;
    ips_layout(S->n, static_cast<char*>(workspace), S);
    S->ips_rtol = (float)p->rtol;
    S->ips_maxiter = p->max_iter;
    S->ips_thr = (float)p->solver_threshold;
    S->ips = true;
    return SPH_OK;
}

extern "C" int sph_solver_ips_result(sph_solver_t* S, int32_t* iterations, int32_t* code, sph_stream_t stream) {
    if (!S || !S->ips) return SPH_ERR_ARGUMENT;
    IpsState h;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(&h, S->ips_state, sizeof(IpsState), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (iterations) *iterations = h.iter;
    if (code) *code = h.code;
    return SPH_OK;
}
