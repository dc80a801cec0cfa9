// Device helpers shared by the sph103 kernels (sm_103a).
//
// Pair geometry follows the reference's fp32 operation order exactly, so that the
// inclusion test q <= 1 selects the same pairs as the reference:
//   periodic position  rem(x - min, ext) + min       src/diffSPH/v2/modules/neighborhood.py:431
//   minimum image      where(|x| > ext/2, sgn(x) ((|x| + min) % ext + min), x)   src/diffSPH/v2/math.py:5-6
//   r = sqrt(fma(y, y, x*x))  (torch's CPU 2-norm of a 2-vector), q = r / h_j,
//   xhat = x_ij / (r + 1e-7)                         neighborhood.py:433-460
// The __f*_rn intrinsics keep nvcc from contracting or reassociating these steps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sph {

constexpr float kCd = 2.2281692032865347f;  // 7 / pi, Wendland C2 in 2D (kernelFunctions/Wendland2.py:24-27)

struct Geo {
    float mn[2];    // domain min (fp32, as the reference casts its python floats)
    float ext[2];   // max - min
    float half[2];  // (max - min) / 2
    int per[2];     // periodic axes
};

__device__ __forceinline__ float rem_f(float a, float b) {
    // torch's float remainder: fmod with a sign fix-up (fmodf is exact)
    float m = fmodf(a, b);
    if (m != 0.0f && ((b < 0.0f) != (m < 0.0f))) m = __fadd_rn(m, b);
    return m;
}

__device__ __forceinline__ float wrap_axis(float x, float mn, float ext) {
    return __fadd_rn(rem_f(__fsub_rn(x, mn), ext), mn);
}

__device__ __forceinline__ float2 wrap_pos(float2 p, const Geo& g) {
    if (g.per[0]) p.x = wrap_axis(p.x, g.mn[0], g.ext[0]);
    if (g.per[1]) p.y = wrap_axis(p.y, g.mn[1], g.ext[1]);
    return p;
}

__device__ __forceinline__ float mod_axis(float x, float mn, float ext, float half) {
    float a = fabsf(x);
    if (a > half) {
        float s = (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f);
        return __fmul_rn(s, __fadd_rn(rem_f(__fadd_rn(a, mn), ext), mn));
    }
    return x;
}

// x_ij = mod(p_i - p_j) on periodic axes (p already wrapped)
template <bool PER>
__device__ __forceinline__ void pair_vec(float2 pi, float2 pj, const Geo& g, float& x0, float& x1) {
    x0 = __fsub_rn(pi.x, pj.x);
    x1 = __fsub_rn(pi.y, pj.y);
    if (PER) {
        if (g.per[0]) x0 = mod_axis(x0, g.mn[0], g.ext[0], g.half[0]);
        if (g.per[1]) x1 = mod_axis(x1, g.mn[1], g.ext[1], g.half[1]);
    }
}

__device__ __forceinline__ float sq_norm_ref(float x0, float x1) {
    return __fmaf_rn(x1, x1, __fmul_rn(x0, x0));
}

// Geometry of a pair that passed the exact inclusion test. r, q and the unit vector feed
// tolerance-checked sums only, so they use the fast reciprocal square root / reciprocal.
struct PairG {
    float r, q, xh0, xh1;
};

__device__ __forceinline__ PairG pair_fast(float x0, float x1, float sq, float inv_h) {
    PairG g;
    g.r = sq > 0.0f ? sq * rsqrtf(sq) : 0.0f;
    g.q = g.r * inv_h;
    float inv = __fdividef(1.0f, g.r + 1e-7f);
    g.xh0 = x0 * inv;
    g.xh1 = x1 * inv;
    return g;
}

// Exact reference test: q = sqrt(s) / h <= 1. Returns q, r.
__device__ __forceinline__ bool exact_in(float s, float h, float& r, float& q) {
    r = __fsqrt_rn(s);
    q = __fdiv_rn(r, h);
    return q <= 1.0f;
}

// Wendland C2 (2D): W = (1-q)^4 (1+4q) C_d/h^2, dW/dr factor = -20 q (1-q)^3 C_d/h^3
struct KernelCoef {
    float cw;  // C_d / h^2
    float cg;  // C_d / h^3
};

__device__ __forceinline__ float wendland_w(float q, const KernelCoef& k) {
    float om = fminf(fmaxf(1.0f - q, 0.0f), 1.0f);
    float om2 = om * om;
    return om2 * om2 * (1.0f + 4.0f * q) * k.cw;
}

__device__ __forceinline__ float wendland_dw(float q, const KernelCoef& k) {
    float om = fminf(fmaxf(1.0f - q, 0.0f), 1.0f);
    return -20.0f * q * (om * om * om) * k.cg;
}

__device__ __forceinline__ float sgnf(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }

// The reference's closed-form 2x2 pseudo-inverse (src/diffSPH/v2/math.py:11-57): an SVD
// assembled from two half-angle rotations, the smaller singular value regularised by
// 1e-7 under the square root, singular values <= 1e-5 dropped.
struct M2 {
    float a, b, c, d;
};

__device__ __forceinline__ M2 pinv2x2_ref(float a, float b, float c, float d, float* sv1 = nullptr,
                                          float* sv2 = nullptr) {
    float aa = a * a, bb = b * b, cc = c * c, dd = d * d;
    float theta = 0.5f * atan2f(2.0f * a * c + 2.0f * b * d, aa + bb - cc - dd);
    float ct, st;
    sincosf(theta, &st, &ct);
    float S1 = aa + bb + cc + dd;
    float t = aa + bb - cc - dd;
    float u = a * c + b * d;
    float S2 = sqrtf(t * t + 4.0f * u * u);
    float o1 = sqrtf((S1 + S2) * 0.5f);
    float o2 = sqrtf(fmaxf(S1 - S2 + 1e-7f, 1e-7f) * 0.5f);
    if (sv1) *sv1 = o1;  // the singular values (math.py:53-54 orders them by magnitude)
    if (sv2) *sv2 = o2;
    float phi = 0.5f * atan2f(2.0f * a * b + 2.0f * c * d, aa - bb + cc - dd);
    float cp, sp;
    sincosf(phi, &sp, &cp);
    float s11 = sgnf((a * ct + c * st) * cp + (b * ct + d * st) * sp);
    float s22 = sgnf((a * st - c * ct) * sp + (-b * st + d * ct) * cp);
    float i1 = fabsf(o1) > 1e-5f ? 1.0f / o1 : 0.0f;
    float i2 = fabsf(o2) > 1e-5f ? 1.0f / o2 : 0.0f;
    // pinv = V diag(i1, i2) U^T with U = [[ct,-st],[st,ct]], V = [[cp s11, -sp s22],[sp s11, cp s22]]
    float v00 = cp * s11 * i1, v01 = -sp * s22 * i2;
    float v10 = sp * s11 * i1, v11 = cp * s22 * i2;
    M2 L;
    L.a = v00 * ct - v01 * st;
    L.b = v00 * st + v01 * ct;
    L.c = v10 * ct - v11 * st;
    L.d = v10 * st + v11 * ct;
    return L;
}

// 3x3 pseudo-inverse in fp64 with torch.linalg.pinv's truncation rule (singular values
// below rtol * sigma_max dropped). Well-conditioned matrices take the adjugate inverse;
// the rest an eigen-decomposition of A^T A by cyclic Jacobi rotations (bounded sweeps).
__device__ inline void pinv3_f64(const double A[9], double P[9], double rtol) {
    double c00 = A[4] * A[8] - A[5] * A[7];
    double c01 = A[5] * A[6] - A[3] * A[8];
    double c02 = A[3] * A[7] - A[4] * A[6];
    double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    double fa = 0.0;
    for (int k = 0; k < 9; ++k) fa += A[k] * A[k];
    if (det != 0.0 && isfinite(det)) {
        double id = 1.0 / det;
        double I[9];
        I[0] = c00 * id;
        I[1] = (A[2] * A[7] - A[1] * A[8]) * id;
        I[2] = (A[1] * A[5] - A[2] * A[4]) * id;
        I[3] = c01 * id;
        I[4] = (A[0] * A[8] - A[2] * A[6]) * id;
        I[5] = (A[2] * A[3] - A[0] * A[5]) * id;
        I[6] = c02 * id;
        I[7] = (A[1] * A[6] - A[0] * A[7]) * id;
        I[8] = (A[0] * A[4] - A[1] * A[3]) * id;
        double fi = 0.0;
        for (int k = 0; k < 9; ++k) fi += I[k] * I[k];
        // ||A||_F ||A^-1||_F >= cond_2(A) = sigma_max / sigma_min: below 0.9 / rtol every
        // singular value exceeds rtol sigma_max, nothing is truncated and A^+ = A^-1
        if (sqrt(fa * fi) < 0.9 / rtol) {
            for (int k = 0; k < 9; ++k) P[k] = I[k];
            return;
        }
    }
    // B = A^T A (symmetric), V accumulates rotations
    double B[9], V[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) B[3 * r + c] = A[r] * A[c] + A[3 + r] * A[3 + c] + A[6 + r] * A[6 + c];
    for (int sweep = 0; sweep < 24; ++sweep) {
        double off = B[1] * B[1] + B[2] * B[2] + B[5] * B[5];
        double dg = B[0] * B[0] + B[4] * B[4] + B[8] * B[8];
        if (off <= 1e-30 * dg) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = (pq == 2) ? 1 : 0;
            const int q = (pq == 0) ? 1 : 2;
            const int r = 3 - p - q;
            const double bpq = B[3 * p + q];
            if (bpq == 0.0) continue;
            // t = tan(theta) of the rotation that zeroes b_pq (the smaller root):
            // sgn(d) e / (|d| + sqrt(d^2 + e^2)), d = b_qq - b_pp, e = 2 b_pq; one square root,
            // one division and one reciprocal square root (FP64 is slow on this part)
            const double d = B[3 * q + q] - B[3 * p + p], e = 2.0 * bpq;
            const double t = (d >= 0.0 ? e : -e) / (fabs(d) + sqrt(d * d + e * e));
            const double c = rsqrt(1.0 + t * t), s = t * c;
            // B <- J^T B J in closed form: the (p, q) block becomes diagonal, row/column r rotates
            const double tb = t * bpq;
            B[3 * p + p] -= tb;
            B[3 * q + q] += tb;
            B[3 * p + q] = B[3 * q + p] = 0.0;
            const double brp = B[3 * r + p], brq = B[3 * r + q];
            const double nrp = c * brp - s * brq, nrq = s * brp + c * brq;
            B[3 * r + p] = B[3 * p + r] = nrp;
            B[3 * r + q] = B[3 * q + r] = nrq;
            for (int k = 0; k < 3; ++k) {
                double vkp = V[3 * k + p], vkq = V[3 * k + q];
                V[3 * k + p] = c * vkp - s * vkq;
                V[3 * k + q] = s * vkp + c * vkq;
            }
        }
    }
    double lam[3] = {fmax(B[0], 0.0), fmax(B[4], 0.0), fmax(B[8], 0.0)};
    double smax = sqrt(fmax(lam[0], fmax(lam[1], lam[2])));
    for (int k = 0; k < 9; ++k) P[k] = 0.0;
    for (int m = 0; m < 3; ++m) {
        double sg = sqrt(lam[m]);
        if (!(sg > rtol * smax) || sg == 0.0) continue;
        // pinv += v_m (A v_m)^T / sigma_m^2
        double v0 = V[m], v1 = V[3 + m], v2 = V[6 + m];
        double w0 = A[0] * v0 + A[1] * v1 + A[2] * v2;
        double w1 = A[3] * v0 + A[4] * v1 + A[5] * v2;
        double w2 = A[6] * v0 + A[7] * v1 + A[8] * v2;
        double inv = 1.0 / lam[m];
        double vv[3] = {v0, v1, v2}, ww[3] = {w0, w1, w2};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) P[3 * r + c] += vv[r] * ww[c] * inv;
    }
}

// stiff Tait EOS (src/diffSPH/v2/modules/pressureEOS.py:5-11): B ((rho/rho0)^gamma - 1)
struct Eos {
    float B;       // rho0 cs^2 / gamma
    float rho0;
    float gamma;
};

__device__ __forceinline__ float eos_p(float rho, const Eos& e) {
    return e.B * (powf(rho / e.rho0, e.gamma) - 1.0f);
}

}  // namespace sph
