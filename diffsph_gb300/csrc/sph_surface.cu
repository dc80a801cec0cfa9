// Free-surface handling of the shift (shifting.freeSurface = True) for sm_103a.
//
// solveShifting (src/diffSPH/v2/modules/shifting.py:882-1019) with the reference's defaults
// for this branch (surfaceDetection 'Barcasco', normalScheme 'lambda', projectionScheme
// 'mat', useExtendedMask off) works on the merged fluid + wall particle set:
//   fs  = detectFreeSurfaceBarecasco   (src/diffSPH/v2/modules/surfaceDetection.py:95-107)
//         no neighbor j != i within the cone of half-angle threshold / 2 around the
//         normalised cover vector sum_j -xhat_ij (a vanishing cover vector: interior)
//   fsm = expandFreeSurfaceMask        (surfaceDetection.py:54-63), OR over the neighbors,
//         expansionIterations times
//   L, Lambdas = pinv2x2 of the normalization matrix and its smaller singular value
//         (normalizationMatrices.py:7-16, math.py:11-57, surfaceDetection.py:41-52)
//   n   = normalize(sum_j V_j (Lambda_i - Lambda_j) L_i gradW_ij)   (computeLambdaGrad,
//         shifting.py:151-171)
// and the shift kernels then project their update (surface_project). For the implicit
// scheme the surface rows leave the system like wall rows (getShiftingMatrices :657-678).
//
// Three kinds of pass over the sorted slots, one thread per slot, every slot a row (walls
// included: their flags feed the mask expansion of the fluid):
//   k_fs_detect  the step's skin list (warps of fluid rows) or the stencil: cover vector,
//                normalization matrix -> L, Lambdas; keeps the exact list (int16 offsets,
//                edge-major); then the cone test over that list
//   k_fs_scatter each mask expansion, written from the (sparse) flagged particles
//   k_fs_normals the lambda gradient -> n, on the rows of the final mask
// The cone test uses the reference's unit vectors bit for bit (correctly rounded sqrt and
// division) and tests acos(d) <= threshold / 2 as d >= cos(threshold / 2); the cover vector's
// summation order differs from the reference's, so a flag can differ only for a pair within
// rounding of the cone's edge.
#include <math.h>
#include <string.h>

#include "sph_solver.cuh"

namespace sph {

constexpr int kFsW = 4;  // warps per block

// the reference's unit vector x_ij / (|x_ij| + 1e-7) (neighborhood.py:433-460)
__device__ __forceinline__ void unit_ref(float x0, float x1, float& u0, float& u1) {
    const float r = __fsqrt_rn(sq_norm_ref(x0, x1));
    const float d = __fadd_rn(r, 1e-7f);
    u0 = __fdiv_rn(x0, d);
    u1 = __fdiv_rn(x1, d);
}

// torch.nn.functional.normalize: v / max(|v|, 1e-12)
__device__ __forceinline__ float2 normalize_ref(float v0, float v1) {
    const float nrm = fmaxf(sqrtf(v0 * v0 + v1 * v1), 1e-12f);
    return make_float2(v0 / nrm, v1 / nrm);
}

template <bool PER, typename LT, int W>
__global__ void __launch_bounds__(32 * W)
    k_fs_detect(const Dom D, int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ start,
                uint32_t* __restrict__ words, int16_t* __restrict__ fnl, int16_t* __restrict__ fnlc,
                uint8_t* __restrict__ fs, float* __restrict__ lam, float4* __restrict__ Lout, float cos_half,
                int use_skin, const int16_t* __restrict__ sl, const int16_t* __restrict__ slc) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int64_t i = (int64_t)blockIdx.x * (32 * W) + threadIdx.x;
    const bool inb = i < n;
    const float4 xi = inb ? X4[i] : make_float4(0.f, 0.f, 1.f, 0.f);
    const float2 pi = make_float2(xi.x, xi.y);
    // fluid rows hold the step's skin list (wall rows do not): a warp of fluid rows with
    // complete lists filters them, any other warp scans the stencil (same pairs, same order)
    const int sk = (!PER && use_skin && inb && !is_boundary(xi.z)) ? (int)slc[i] : (inb ? -1 : 0);
    const bool skin = !PER && use_skin && __all_sync(kFull, sk >= 0) && words[3] == 0u;
    float c0 = 0.f, c1 = 0.f;                          // cover vector
    float M00 = 0.f, M01 = 0.f, M10 = 0.f, M11 = 0.f;  // normalization matrix
    int nst = 0;
    bool unstored = false;
    auto pair_m = [&](int j) {
        int d = j - (int)i;
        if (PER) {
            const int h2 = g.nslots >> 1;
            if (d > h2) d -= g.nslots;
            else if (d < -h2) d += g.nslots;
        }
        if (nst < kStoreCap && d >= -32768 && d <= 32767)
            fnl[(int64_t)nst * n + i] = (int16_t)d;
        else
            unstored = true;
        ++nst;
        const float4 xj = __ldg(&X4[j]);
        float x0, x1;
        pair_vec<PER>(pi, make_float2(xj.x, xj.y), P.geo, x0, x1);
        const PairG pg = pair_fast(x0, x1, sq_norm_ref(x0, x1), P.inv_h);
        c0 -= pg.xh0;  // the cover vector only sets the cone's axis: its summation order already
        c1 -= pg.xh1;  // differs from the reference's, so the unit vectors need no exact rounding
        const float dW = wendland_dw(pg.q, P.kc);
        const float V = __fdividef(P.m, fabsf(xj.z));
        const float k0 = pg.xh0 * dW * V, k1 = pg.xh1 * dW * V;
        const float d0 = -pg.r * pg.xh0, d1 = -pg.r * pg.xh1;  // -(q h) xhat
        M00 = fmaf(d0, k0, M00);
        M01 = fmaf(d0, k1, M01);
        M10 = fmaf(d1, k0, M10);
        M11 = fmaf(d1, k1, M11);
    };
    if (skin)
        skin_loop<PER>((int)i, pi, X4, g, P, sl, sk, pair_m);
    else
        neighbor_loop<PER, LT>(inb, (int)i, pi, X4, start, g, P, lst, words, pair_m);
    if (inb) fnlc[i] = unstored ? (int16_t)-1 : (int16_t)nst;
    // the cone test over the same neighbors (the stored list, or a second scan)
    const float2 cn = normalize_ref(c0, c1);
    const bool interior = sqrtf(cn.x * cn.x + cn.y * cn.y) <= 1e-5f;
    bool inside = false;  // some neighbor within the cone
    auto pair_c = [&](int j) {
        if (j == (int)i || inside) return;
        const float4 xj = __ldg(&X4[j]);
        float x0, x1;
        pair_vec<PER>(pi, make_float2(xj.x, xj.y), P.geo, x0, x1);
        float u0, u1;
        unit_ref(x0, x1, u0, u1);
        const float dot = __fadd_rn(__fmul_rn(u0, cn.x), __fmul_rn(u1, cn.y));
        // acos(dot) <= half_angle, tested as dot >= cos(half_angle) (acos is decreasing)
        if (dot >= cos_half) inside = true;
    };
    const int cnt = inb ? (int)fnlc[i] : 0;
    if (__any_sync(kFull, cnt < 0)) {
        neighbor_loop<PER, LT>(inb && !interior, (int)i, pi, X4, start, g, P, lst, words, pair_c);
    } else if (!interior) {
        // stops at the first neighbor inside the cone (most rows find one within a few)
        for (int k = 0; k < cnt && !inside; ++k) pair_c(list_slot<PER>((int)i, (int)fnl[(int64_t)k * n + i], g));
    }
    if (!inb) return;
    fs[i] = (uint8_t)(!interior && !inside);
    float o1, o2;
    const M2 L = pinv2x2_ref(M00, M01, M10, M11, &o1, &o2);
    lam[i] = fminf(fabsf(o1), fabsf(o2));
    Lout[i] = make_float4(L.a, L.b, L.c, L.d);
}

// the normalised lambda gradient, on the rows of the final mask (the only ones that use it)
template <bool PER, typename LT, int W>
__global__ void __launch_bounds__(32 * W)
    k_fs_normals(const Dom D, int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ start,
                 uint32_t* __restrict__ words, const int16_t* __restrict__ fnl, const int16_t* __restrict__ fnlc,
                 const uint8_t* __restrict__ fsm, const float* __restrict__ lam, const float4* __restrict__ Lin,
                 float2* __restrict__ nrm) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int64_t i = (int64_t)blockIdx.x * (32 * W) + threadIdx.x;
    const bool row = i < n && fsm[i];
    if (!__any_sync(kFull, row)) return;
    const float4 xi = row ? X4[i] : make_float4(0.f, 0.f, 1.f, 0.f);
    const float2 pi = make_float2(xi.x, xi.y);
    const float4 L = row ? Lin[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float li = row ? lam[i] : 0.f;
    float g0 = 0.f, g1 = 0.f;
    auto pair_n = [&](int j) {
        const float4 xj = __ldg(&X4[j]);
        float x0, x1;
        pair_vec<PER>(pi, make_float2(xj.x, xj.y), P.geo, x0, x1);
        const PairG pg = pair_fast(x0, x1, sq_norm_ref(x0, x1), P.inv_h);
        const float dW = wendland_dw(pg.q, P.kc);
        const float gw0 = pg.xh0 * dW, gw1 = pg.xh1 * dW;
        const float ng0 = L.x * gw0 + L.y * gw1, ng1 = L.z * gw0 + L.w * gw1;  // L_i gradW
        const float w = __fdividef(P.m, fabsf(xj.z)) * (li - lam[j]);
        g0 = fmaf(w, ng0, g0);
        g1 = fmaf(w, ng1, g1);
    };
    const int cnt = row ? (int)fnlc[i] : 0;
    if (__any_sync(kFull, cnt < 0)) {
        neighbor_loop<PER, LT>(row, (int)i, pi, X4, start, g, P, lst, words, pair_n);
    } else {
        for (int k = 0; k < cnt; ++k) pair_n(list_slot<PER>((int)i, (int)fnl[(int64_t)k * n + i], g));
    }
    if (row) nrm[i] = normalize_ref(g0, g1);
}

// one mask expansion, out_k = OR over the neighbors j of k of in_j, written from the flagged
// particles: every flagged j marks its neighbors (the neighbor relation is symmetric with one
// support). The flags are sparse, and equal stores of 1 make the result independent of order.
template <bool PER, typename LT, int W>
__global__ void __launch_bounds__(32 * W)
    k_fs_scatter(const Dom D, int64_t n, const float4* __restrict__ X4, const int32_t* __restrict__ start,
                 uint32_t* __restrict__ words, const int16_t* __restrict__ fnl, const int16_t* __restrict__ fnlc,
                 const uint8_t* __restrict__ in, uint8_t* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    LT* lst = reinterpret_cast<LT*>(s_dyn) + (threadIdx.x >> 5) * (kCap * 32);
    const Phys& P = D.P;
    const Grid& g = D.g;
    const int64_t i = (int64_t)blockIdx.x * (32 * W) + threadIdx.x;
    const bool row = i < n && in[i];
    if (!__any_sync(kFull, row)) return;
    const float4 xi = row ? X4[i] : make_float4(0.f, 0.f, 1.f, 0.f);
    const float2 pi = make_float2(xi.x, xi.y);
    auto mark = [&](int j) { out[j] = 1; };
    const int cnt = row ? (int)fnlc[i] : 0;
    if (__any_sync(kFull, cnt < 0)) {
        neighbor_loop<PER, LT>(row, (int)i, pi, X4, start, g, P, lst, words, mark);
    } else {
        for (int k = 0; k < cnt; ++k) mark(list_slot<PER>((int)i, (int)fnl[(int64_t)k * n + i], g));
    }
}

// the fields in the original particle order (fluid first, then walls)
__global__ void k_fs_download(int64_t n, const int32_t* __restrict__ uid, const uint8_t* __restrict__ fs,
                              const uint8_t* __restrict__ fsm, const float* __restrict__ lam,
                              const float2* __restrict__ nrm, uint8_t* fs_out, uint8_t* fsm_out, float* lam_out,
                              float* nrm_out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = uid[s];
    if (fs_out) fs_out[o] = fs[s];
    if (fsm_out) fsm_out[o] = fsm[s];
    if (lam_out) lam_out[o] = lam[s];
    if (nrm_out) {
        nrm_out[2 * o] = nrm[s].x;
        nrm_out[2 * o + 1] = nrm[s].y;
    }
}

// computePressureAccelSwitch (src/diffSPH/v2/modules/pressureForce.py:15-33) on a
// neighborhood in the reference's format: rows sorted by the query index, one thread per row,
// its pairs in the stored order, each fp32 step in the reference's order (so the sums are
// the reference's bit for bit when the inputs are).
__global__ void k_pressure_switch(int64_t n, const int32_t* __restrict__ off, const int32_t* __restrict__ cnt,
                                  const int64_t* __restrict__ pj, const float* __restrict__ grad,
                                  const float* __restrict__ pA, const float* __restrict__ rhoA,
                                  const float* __restrict__ maskA, const float* __restrict__ pB,
                                  const float* __restrict__ rhoB, const float* __restrict__ mB, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float p_i = pA[i], r_i = rhoA[i];
    const bool sum = p_i >= 0.f || (maskA && maskA[i] > 0.5f);
    float a0 = 0.f, a1 = 0.f;
    const int64_t e0 = off[i], e1 = e0 + cnt[i];
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = pj[e];
        const float pij = sum ? __fadd_rn(pB[j], p_i) : __fsub_rn(pB[j], p_i);
        const float k = __fdiv_rn(mB[j], __fmul_rn(r_i, rhoB[j]));
        a0 = __fadd_rn(a0, __fmul_rn(pij, __fmul_rn(k, grad[2 * e])));
        a1 = __fadd_rn(a1, __fmul_rn(pij, __fmul_rn(k, grad[2 * e + 1])));
    }
    out[2 * i] = -a0;
    out[2 * i + 1] = -a1;
}

// LiuLiuConsistent (src/diffSPH/v2/sphOps.py:313-341) on a neighborhood in the reference's
// format: per query (ghost) row, the moment sums of b and M in the pair order with each fp32
// step in the reference's order, then Cramer's rule in fp64 (the reference divides
// determinants of fp32 LU factorisations; fp64 keeps the ill-conditioned rows accurate).
__device__ __forceinline__ double det3(const double m[9]) {
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
           m[2] * (m[3] * m[7] - m[4] * m[6]);
}

__global__ void k_liuliu(int64_t n, const int32_t* __restrict__ off, const int32_t* __restrict__ cnt,
                         const int64_t* __restrict__ pj, const float* __restrict__ qd, const float* __restrict__ xh,
                         const float* __restrict__ hp, const float* __restrict__ W, const float* __restrict__ G,
                         const float* __restrict__ m, const float* __restrict__ rho, const float* __restrict__ q,
                         float* __restrict__ sol, float* __restrict__ Mout, float* __restrict__ bout) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float b0 = 0.f, b1 = 0.f, b2 = 0.f;
    float M0 = 0.f, Mg0 = 0.f, Mg1 = 0.f, Mx0 = 0.f, Mx1 = 0.f, Mxg00 = 0.f, Mxg01 = 0.f, Mxg10 = 0.f, Mxg11 = 0.f;
    const int64_t e0 = off[i], e1 = e0 + cnt[i];
    for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = pj[e];
        const float V = __fdiv_rn(m[j], rho[j]);
        const float vw = __fmul_rn(V, W[e]);
        const float vg0 = __fmul_rn(V, G[2 * e]), vg1 = __fmul_rn(V, G[2 * e + 1]);
        const float x0 = __fmul_rn(__fmul_rn(-xh[2 * e], qd[e]), hp[e]);
        const float x1 = __fmul_rn(__fmul_rn(-xh[2 * e + 1], qd[e]), hp[e]);
        const float qj = q[j];
        b0 = __fadd_rn(b0, __fmul_rn(qj, vw));
        b1 = __fadd_rn(b1, __fmul_rn(qj, vg0));
        b2 = __fadd_rn(b2, __fmul_rn(qj, vg1));
        M0 = __fadd_rn(M0, vw);
        Mg0 = __fadd_rn(Mg0, vg0);
        Mg1 = __fadd_rn(Mg1, vg1);
        Mx0 = __fadd_rn(Mx0, __fmul_rn(x0, vw));
        Mx1 = __fadd_rn(Mx1, __fmul_rn(x1, vw));
        Mxg00 = __fadd_rn(Mxg00, __fmul_rn(x0, vg0));
        Mxg01 = __fadd_rn(Mxg01, __fmul_rn(x0, vg1));
        Mxg10 = __fadd_rn(Mxg10, __fmul_rn(x1, vg0));
        Mxg11 = __fadd_rn(Mxg11, __fmul_rn(x1, vg1));
    }
    const float Mf[9] = {M0, Mx0, Mx1, Mg0, Mxg00, Mxg01, Mg1, Mxg10, Mxg11};
    const float bf[3] = {b0, b1, b2};
    double Md[9];
    for (int k = 0; k < 9; ++k) Md[k] = Mf[k];
    const double d0 = det3(Md) + 1e-7;
    for (int c = 0; c < 3; ++c) {
        double Mk[9];
        for (int k = 0; k < 9; ++k) Mk[k] = (k % 3 == c) ? (double)bf[k / 3] : Md[k];
        sol[3 * i + c] = (float)(det3(Mk) / d0);
    }
    if (Mout)
        for (int k = 0; k < 9; ++k) Mout[9 * i + k] = Mf[k];
    if (bout)
        for (int k = 0; k < 3; ++k) bout[3 * i + k] = bf[k];
}

template <bool PER, typename LT>
static void fs_launch(sph_solver* S, const float4* X4, int use_skin, cudaStream_t st) {
    const int64_t n = S->n;
    const Dom& D = S->doms_host[0];
    const unsigned gb = (unsigned)((n + 32 * kFsW - 1) / (32 * kFsW));
    const size_t smem = list_bytes<LT, kFsW>();
    k_fs_detect<PER, LT, kFsW><<<gb, 32 * kFsW, smem, st>>>(D, n, X4, S->start, S->words, S->fs_nl, S->fs_nlc, S->fs,
                                                            S->fs_lam, S->fs_L, S->fs_cos_half, use_skin, S->sl,
                                                            S->slc);
    const uint8_t* in = S->fs;
    for (int k = 0; k < S->fs_expand; ++k) {
        uint8_t* out = ((S->fs_expand - 1 - k) & 1) ? S->fsm_t : S->fsm;  // the last one into fsm
        cudaMemsetAsync(out, 0, (size_t)n, st);
        k_fs_scatter<PER, LT, kFsW><<<gb, 32 * kFsW, smem, st>>>(D, n, X4, S->start, S->words, S->fs_nl, S->fs_nlc,
                                                                 in, out);
        in = out;
    }
    cudaMemsetAsync(S->fs_nrm, 0, (size_t)n * sizeof(float2), st);  // zero off the mask
    k_fs_normals<PER, LT, kFsW><<<gb, 32 * kFsW, smem, st>>>(D, n, X4, S->start, S->words, S->fs_nl, S->fs_nlc,
                                                             S->fsm, S->fs_lam, S->fs_L, S->fs_nrm);
}

}  // namespace sph

int surface_detect(sph_solver* S, const float4* X4, int use_skin, cudaStream_t st) {
    if (!S->fs_on || !S->prm.shift_on) return SPH_OK;
    tbeg(S, KC_SURFACE, st);
    if (S->periodic) {
        if (S->list16) fs_launch<true, int16_t>(S, X4, 0, st);
        else fs_launch<true, int32_t>(S, X4, 0, st);
    } else {
        if (S->list16) fs_launch<false, int16_t>(S, X4, use_skin, st);
        else fs_launch<false, int32_t>(S, X4, use_skin, st);
    }
    tend(S, KC_SURFACE, st);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

SurfaceView surface_view(const sph_solver* S) {
    SurfaceView v;
    const bool on = S->fs_on && S->prm.shift_on;
    v.fs = on ? S->fs : nullptr;
    v.fsm = on ? S->fsm : nullptr;
    v.lam = on ? S->fs_lam : nullptr;
    v.nrm = on ? S->fs_nrm : nullptr;
    v.scaling = S->fs_scaling;
    return v;
}

// workspace: list [kStoreCap][n] + length [n] (int16), fs, fsm, fsm_t [n] (uint8), Lambdas [n],
// L [n] (float4), normals [n] (float2)
static size_t fs_layout(int64_t n, char* base, sph_solver* S) {
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t N = (size_t)n;
    const size_t sz[8] = {up((size_t)kStoreCap * N * sizeof(int16_t)), up(N * sizeof(int16_t)), up(N), up(N), up(N),
                          up(N * sizeof(float)), up(N * sizeof(float4)), up(N * sizeof(float2))};
    if (S && base) {
        char* w = base;
        S->fs_nl = reinterpret_cast<int16_t*>(w);
        w += sz[0];
        S->fs_nlc = reinterpret_cast<int16_t*>(w);
        w += sz[1];
        S->fs = reinterpret_cast<uint8_t*>(w);
        w += sz[2];
        S->fsm = reinterpret_cast<uint8_t*>(w);
        w += sz[3];
        S->fsm_t = reinterpret_cast<uint8_t*>(w);
        w += sz[4];
        S->fs_lam = reinterpret_cast<float*>(w);
        w += sz[5];
        S->fs_L = reinterpret_cast<float4*>(w);
        w += sz[6];
        S->fs_nrm = reinterpret_cast<float2*>(w);
    }
    size_t t = 0;
    for (size_t b : sz) t += b;
    return t;
}

extern "C" int sph_solver_free_surface_workspace_bytes(const sph_solver_t* S, size_t* bytes) {
    if (!S || !bytes) return SPH_ERR_ARGUMENT;
    *bytes = fs_layout(S->n, nullptr, nullptr);
    return SPH_OK;
}

extern "C" int sph_solver_set_free_surface(sph_solver_t* S, const sph_free_surface_params_t* p, void* workspace,
                                           size_t workspace_bytes) {
    if (!S) return SPH_ERR_ARGUMENT;
    for (int k = 0; k < 2; ++k)  // captured graphs hold the launches without the handling
        if (S->graph[k]) {
            cudaGraphExecDestroy(S->graph[k]);
            S->graph[k] = nullptr;
            S->graph_n[k] = 0;
        }
    if (!p) {
        S->fs_on = false;
        return SPH_OK;
    }
    if (S->nd != 1 || !workspace || p->expansion_iterations < 1 || !(p->barecasco_threshold >= 0.0))
        return SPH_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(workspace) & 255u) != 0) return SPH_ERR_ARGUMENT;
    if (workspace_bytes < fs_layout(S->n, nullptr, nullptr)) return SPH_ERR_WORKSPACE;
    fs_layout(S->n, static_cast<char*>(workspace), S);
    S->fs_cos_half = (float)cos((double)(float)(p->barecasco_threshold / 2.0));
    S->fs_expand = p->expansion_iterations;
    S->fs_scaling = (float)p->surface_scaling;
    S->fs_on = true;
    return SPH_OK;
}

extern "C" int sph_solver_free_surface_fields(sph_solver_t* S, uint8_t* fs, uint8_t* fsm, float* lambdas,
                                              float* normals, sph_stream_t stream) {
    if (!S || !S->fs_on) return SPH_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    k_fs_download<<<blocks_for(S->n), kBlock, 0, st>>>(S->n, S->uid, S->fs, S->fsm, S->fs_lam, S->fs_nrm, fs, fsm,
                                                        lambdas, normals);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_pressure_switch(int64_t n_query, const int32_t* offsets, const int32_t* counts,
                                   const int64_t* pair_j, const float* gradients, const float* p_query,
                                   const float* rho_query, const float* surface_mask, const float* p_ref,
                                   const float* rho_ref, const float* m_ref, float* accel, sph_stream_t stream) {
    if (n_query < 0 || (n_query > 0 && (!offsets || !counts || !p_query || !rho_query || !p_ref || !rho_ref ||
                                        !m_ref || !accel)))
        return SPH_ERR_ARGUMENT;
    if (n_query == 0) return SPH_OK;
    cudaStream_t st = (cudaStream_t)stream;
    k_pressure_switch<<<blocks_for(n_query), kBlock, 0, st>>>(n_query, offsets, counts, pair_j, gradients, p_query,
                                                               rho_query, surface_mask, p_ref, rho_ref, m_ref, accel);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_liuliu_consistent(int64_t n_query, const int32_t* offsets, const int32_t* counts,
                                     const int64_t* pair_j, const float* distances, const float* vectors,
                                     const float* supports, const float* kernels, const float* gradients,
                                     const float* m_ref, const float* rho_ref, const float* quantity,
                                     float* solution, float* M, float* b, sph_stream_t stream) {
    if (n_query < 0 || (n_query > 0 && (!offsets || !counts || !m_ref || !rho_ref || !quantity || !solution)))
        return SPH_ERR_ARGUMENT;
    if (n_query == 0) return SPH_OK;
    cudaStream_t st = (cudaStream_t)stream;
    k_liuliu<<<blocks_for(n_query), kBlock, 0, st>>>(n_query, offsets, counts, pair_j, distances, vectors, supports,
                                                      kernels, gradients, m_ref, rho_ref, quantity, solution, M, b);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
