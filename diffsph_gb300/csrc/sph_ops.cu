// Pair-sum operators on a neighborhood in the reference's format, for sm_103a.
//
// The reference's module functions (src/diffSPH/v2/modules/*.py) and its operator family
// (sphOperation, src/diffSPH/v2/sphOps.py:6-303) evaluate per-pair tensors and reduce them
// with scatter_sum (src/diffSPH/v2/math.py:77-93) over pairs sorted by query index. Here one
// thread walks one query row: the pairs [offsets[i], offsets[i] + counts[i]) in their stored
// order, so each row's sum has the reference's order (its CPU scatter_add adds the pairs in
// index order). Every per-pair expression keeps the reference's fp32 operation order with
// round-to-nearest intrinsics (no contraction into fused multiply-adds), so the results
// follow the reference's own arithmetic.
//
// These operators serve callers that keep the reference's own simulationStep (or a scheme
// the fused solver does not implement); the fused solver's passes are the fast path.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/sph103.h"

namespace {

constexpr int kOpBlock = 128;

struct Pairs {
    const int32_t* off;
    const int32_t* cnt;
    const int64_t* j;
    const float* q;   // r / h_j
    const float* v;   // unit x_ij [P][2]
    const float* h;   // h_j
    const float* W;
    const float* G;   // gradW [P][2]
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

inline unsigned grid_for(int64_t n) { return (unsigned)((n + kOpBlock - 1) / kOpBlock); }

bool pairs_ok(const sph_pairs_t* nb) { return nb && nb->n_query >= 0 && (nb->n_query == 0 || (nb->offsets && nb->counts && nb->pair_j)); }

Pairs view(const sph_pairs_t* nb) {
    return Pairs{nb->offsets, nb->counts, nb->pair_j, nb->distances, nb->vectors, nb->supports, nb->kernels, nb->gradients};
}

// ------------------------------------------------------------------------------------
// sphOperation (sphOps.py:243-275): density, interpolate, gradient, divergence, curl and
// laplacian, for scalar (C = 1), vector (C = 2) and 2x2 matrix (C = 4, row-major) quantities,
// given per particle as the tuple (q_a, q_b) or per pair (q_pair: the reference's
// non-tuple argument, used as is in every mode).
// ------------------------------------------------------------------------------------
template <int C>
__device__ __forceinline__ void load_q(const float* q, int64_t k, float (&o)[C]) {
#pragma unroll
    for (int c = 0; c < C; ++c) o[c] = q[k * C + c];
}

template <int C>
__global__ void k_operation(Pairs nb, int64_t n, int op, int mode, int dmode, const float* __restrict__ m_b,
                            const float* __restrict__ rho_a, const float* __restrict__ rho_b,
                            const float* __restrict__ q_a, const float* __restrict__ q_b,
                            const float* __restrict__ q_pair, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    float acc[2 * C];
#pragma unroll
    for (int c = 0; c < 2 * C; ++c) acc[c] = 0.f;
    float qi[C];
#pragma unroll
    for (int c = 0; c < C; ++c) qi[c] = 0.f;
    if (q_a) load_q<C>(q_a, i, qi);
    // the symmetric forms (sphGradient / sphDivergence / sphCurl 'symmetric'): m_j gradW and
    // q_i / rho_i^2 + q_j / rho_j^2, the sum times rho_i; the laplacian's type only picks its
    // formula (its pair quantity is always q_i - q_j)
    const bool sym = mode == SPH_MODE_SYMMETRIC && !q_pair &&
                     (op == SPH_OP_GRADIENT || op == SPH_OP_DIVERGENCE || op == SPH_OP_CURL);
    float inv2_i = 0.f;
    if (sym) {  // 1.0 / densities[0][i]**2
        const float r = rho_a[i];
        inv2_i = fd(1.0f, fm(r, r));
#pragma unroll
        for (int c = 0; c < C; ++c) qi[c] = fm(qi[c], inv2_i);
    }
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float mj = m_b[j];
        if (op == SPH_OP_DENSITY) {  // sphDensityInterpolation: m_j W
            acc[0] = fa(acc[0], fm(mj, nb.W[p]));
            continue;
        }
        // the pair's quantity in the operation's mode
        float qj[C], qq[C];
        if (q_pair) {
            load_q<C>(q_pair, p, qq);
        } else {
            load_q<C>(q_b, j, qj);
            if (sym) {
                const float r = rho_b[j];
                const float inv2 = fd(1.0f, fm(r, r));
#pragma unroll
                for (int c = 0; c < C; ++c) qq[c] = fa(qi[c], fm(qj[c], inv2));
            } else if (op == SPH_OP_LAPLACIAN) {  // q_i - q_j
#pragma unroll
                for (int c = 0; c < C; ++c) qq[c] = fs(qi[c], qj[c]);
            } else if (mode == SPH_MODE_NAIVE || op == SPH_OP_INTERPOLATE) {
#pragma unroll
                for (int c = 0; c < C; ++c) qq[c] = qj[c];
            } else if (mode == SPH_MODE_SUMMATION) {
#pragma unroll
                for (int c = 0; c < C; ++c) qq[c] = fa(qj[c], qi[c]);
            } else if (op == SPH_OP_GRADIENT) {  // q_i - q_j
#pragma unroll
                for (int c = 0; c < C; ++c) qq[c] = fs(qi[c], qj[c]);
            } else {  // divergence, curl: q_j - q_i
#pragma unroll
                for (int c = 0; c < C; ++c) qq[c] = fs(qj[c], qi[c]);
            }
        }
        if (op == SPH_OP_INTERPOLATE) {  // (m_j / rho_j) W q
            const float k = fm(fd(mj, rho_b[j]), nb.W[p]);
#pragma unroll
            for (int c = 0; c < C; ++c) acc[c] = fa(acc[c], fm(qq[c], k));
            continue;
        }
        const float g0 = nb.G[2 * p], g1 = nb.G[2 * p + 1];
        // k = (m_j / rho_j) gradW, or m_j gradW in the symmetric form
        const float V = sym ? mj : fd(mj, rho_b[j]);
        const float k0 = fm(V, g0), k1 = fm(V, g1);
        if (op == SPH_OP_GRADIENT) {  // q (x) k
#pragma unroll
            for (int c = 0; c < C; ++c) {
                acc[2 * c] = fa(acc[2 * c], fm(qq[c], k0));
                acc[2 * c + 1] = fa(acc[2 * c + 1], fm(qq[c], k1));
            }
        } else if (op == SPH_OP_DIVERGENCE) {
            if (C == 2) {
                acc[0] = fa(acc[0], fa(fm(qq[0], k0), fm(qq[1], k1)));
            } else if (C == 4) {
                if (dmode == 0) {  // 'div': contract the last index
                    acc[0] = fa(acc[0], fa(fm(qq[0], k0), fm(qq[1], k1)));
                    acc[1] = fa(acc[1], fa(fm(qq[2], k0), fm(qq[3], k1)));
                } else {  // 'dot': contract the first index
                    acc[0] = fa(acc[0], fa(fm(qq[0], k0), fm(qq[2], k1)));
                    acc[1] = fa(acc[1], fa(fm(qq[1], k0), fm(qq[3], k1)));
                }
            }
        } else if (op == SPH_OP_CURL) {  // 2D: q_1 k_0 - q_0 k_1
            if (C == 2) acc[0] = fa(acc[0], fs(fm(qq[1], k0), fm(qq[0], k1)));
        } else if (op == SPH_OP_LAPLACIAN) {  // sphLaplacian sphOps.py:197-240 (not 'naive')
            const float x0 = nb.v[2 * p], x1 = nb.v[2 * p + 1];
            const float hh = nb.h[p];
            const float quot = fa(fm(nb.q[p], hh), fm(1e-7f, hh));
            // kernelApproximation = einsum(gradW, -x_ij) / quotient
            const float kA = fd(fa(fm(g0, -x0), fm(g1, -x1)), quot);
            const float Vj = fd(mj, rho_b[j]);
            if (C == 1) {
                acc[0] = fa(acc[0], fm(fm(fm(-qq[0], Vj), 2.0f), kA));
            } else if (C == 2) {
                const float dot = fa(fm(qq[0], x0), fm(qq[1], x1));
                if (mode == SPH_MODE_CONSERVING) {
                    const float s = fm(fm(Vj, kA), dot);
                    acc[0] = fa(acc[0], fm(-s, x0));
                    acc[1] = fa(acc[1], fm(-s, x1));
                } else if (mode == SPH_MODE_DIVERGENCE_FREE) {
                    const float s = fm(fm(8.0f, Vj), fd(dot, quot));
                    acc[0] = fa(acc[0], fm(s, g0));
                    acc[1] = fa(acc[1], fm(s, g1));
                } else if (mode == SPH_MODE_DOT) {
                    const float vk = fm(Vj, kA);
                    const float t0 = fs(fm(fm(-4.0f, dot), x0), qq[0]);
                    const float t1 = fs(fm(fm(-4.0f, dot), x1), qq[1]);
                    acc[0] = fa(acc[0], fm(t0, vk));
                    acc[1] = fa(acc[1], fm(t1, vk));
                } else {
                    const float s = fm(fm(-2.0f, Vj), kA);
                    acc[0] = fa(acc[0], fm(qq[0], s));
                    acc[1] = fa(acc[1], fm(qq[1], s));
                }
            }
        }
    }
    int nout;
    switch (op) {
        case SPH_OP_DENSITY: nout = 1; break;
        case SPH_OP_INTERPOLATE: case SPH_OP_LAPLACIAN: nout = C; break;
        case SPH_OP_GRADIENT: nout = 2 * C; break;
        case SPH_OP_DIVERGENCE: nout = C / 2; break;
        default: nout = 1; break;
    }
    const float scale = sym ? rho_a[i] : 1.0f;  // the symmetric forms multiply by rho_i
#pragma unroll
    for (int c = 0; c < 2 * C; ++c)
        if (c < nout) out[i * nout + c] = sym ? fm(scale, acc[c]) : acc[c];
}

// ------------------------------------------------------------------------------------
// Module functions
// ------------------------------------------------------------------------------------
// computeCovarianceMatrices (normalizationMatrices.py:18-23): the gradient ('difference') of
// the pair quantity -(q h) xhat:  M_i = sum (-(q h) xhat) (x) ((m_j / rho_j) gradW)
__global__ void k_covariance(Pairs nb, int64_t n, const float* __restrict__ m_b, const float* __restrict__ rho_b,
                             float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a00 = 0.f, a01 = 0.f, a10 = 0.f, a11 = 0.f;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float rh = -fm(nb.q[p], nb.h[p]);
        const float d0 = fm(rh, nb.v[2 * p]), d1 = fm(rh, nb.v[2 * p + 1]);
        const float V = fd(m_b[j], rho_b[j]);
        const float k0 = fm(V, nb.G[2 * p]), k1 = fm(V, nb.G[2 * p + 1]);
        a00 = fa(a00, fm(d0, k0));
        a01 = fa(a01, fm(d0, k1));
        a10 = fa(a10, fm(d1, k0));
        a11 = fa(a11, fm(d1, k1));
    }
    out[4 * i] = a00;
    out[4 * i + 1] = a01;
    out[4 * i + 2] = a10;
    out[4 * i + 3] = a11;
}

// renormalizedDensityGradient (densityDiffusion.py:7-26) when L != NULL: the gradient
// ('difference') of the densities with the normalised kernel gradient L_i gradW;
// densityGradient (:28-46) with gradW itself.
__global__ void k_density_gradient(Pairs nb, int64_t n, const float* __restrict__ m_b, const float* __restrict__ rho_a,
                                   const float* __restrict__ rho_b, const float* __restrict__ L,
                                   float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float L00 = 1.f, L01 = 0.f, L10 = 0.f, L11 = 1.f;
    if (L) {
        L00 = L[4 * i];
        L01 = L[4 * i + 1];
        L10 = L[4 * i + 2];
        L11 = L[4 * i + 3];
    }
    const float ri = rho_a[i];
    float a0 = 0.f, a1 = 0.f;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        float g0 = nb.G[2 * p], g1 = nb.G[2 * p + 1];
        if (L) {  // einsum('ijk,ik->ij', L_i, gradW)
            const float n0 = fa(fm(L00, g0), fm(L01, g1));
            const float n1 = fa(fm(L10, g0), fm(L11, g1));
            g0 = n0;
            g1 = n1;
        }
        const float V = fd(m_b[j], rho_b[j]);
        const float dq = fs(ri, rho_b[j]);
        a0 = fa(a0, fm(dq, fm(V, g0)));
        a1 = fa(a1, fm(dq, fm(V, g1)));
    }
    out[2 * i] = a0;
    out[2 * i + 1] = a1;
}

// computeDensityDeltaTerm (densityDiffusion.py:49-73), scheme 'deltaSPH': the divergence
// ('difference', pair quantity) of psi_ij = -2 (rho_j - rho_i)/(r_ij + 1e-6 h) xhat +
// (gradRho^L_i + gradRho^L_j), times delta h_i / kappa cs (coef = delta, kappa, cs)
__global__ void k_delta_term(Pairs nb, int64_t n, const float* __restrict__ m_b, const float* __restrict__ rho_a,
                             const float* __restrict__ rho_b, const float* __restrict__ grad_a,
                             const float* __restrict__ grad_b, const float* __restrict__ h_a, float delta,
                             float kappa, float cs, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ri = rho_a[i], gi0 = grad_a[2 * i], gi1 = grad_a[2 * i + 1];
    float acc = 0.f;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float hh = nb.h[p];
        const float rij = fm(nb.q[p], hh);
        const float gr0 = fa(gi0, grad_b[2 * j]), gr1 = fa(gi1, grad_b[2 * j + 1]);
        const float rho_ij = fd(fm(2.0f, fs(rho_b[j], ri)), fa(rij, fm(1e-6f, hh)));
        const float psi0 = fa(fm(-rho_ij, nb.v[2 * p]), gr0);
        const float psi1 = fa(fm(-rho_ij, nb.v[2 * p + 1]), gr1);
        const float V = fd(m_b[j], rho_b[j]);
        const float k0 = fm(V, nb.G[2 * p]), k1 = fm(V, nb.G[2 * p + 1]);
        acc = fa(acc, fa(fm(psi0, k0), fm(psi1, k1)));
    }
    out[i] = fm(fm(fd(fm(delta, h_a[i]), kappa), cs), acc);
}

// computeMomentumEquation (momentumEquation.py:6-39): -sum ((u_j - u_i) m_j).gradW rho_i / rho_j
__global__ void k_momentum(Pairs nb, int64_t n, const float* __restrict__ m_b, const float* __restrict__ rho_a,
                           const float* __restrict__ rho_b, const float* __restrict__ u_a,
                           const float* __restrict__ u_b, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ri = rho_a[i], ui0 = u_a[2 * i], ui1 = u_a[2 * i + 1];
    float acc = 0.f;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float mj = m_b[j];
        const float q0 = fm(fs(u_b[2 * j], ui0), mj), q1 = fm(fs(u_b[2 * j + 1], ui1), mj);
        const float kq = fa(fm(q0, nb.G[2 * p]), fm(q1, nb.G[2 * p + 1]));
        acc = fa(acc, fd(fm(kq, ri), rho_b[j]));
    }
    out[i] = -acc;
}

// computePressureAccel (pressureForce.py:10-12): -(sum (p_i + p_j) (m_j / rho_j) gradW) / rho_i
__global__ void k_pressure_accel(Pairs nb, int64_t n, const float* __restrict__ m_b, const float* __restrict__ rho_a,
                                 const float* __restrict__ rho_b, const float* __restrict__ p_a,
                                 const float* __restrict__ p_b, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float pi = p_a[i];
    float a0 = 0.f, a1 = 0.f;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float V = fd(m_b[j], rho_b[j]);
        const float q = fa(pi, p_b[j]);
        a0 = fa(a0, fm(q, fm(V, nb.G[2 * p])));
        a1 = fa(a1, fm(q, fm(V, nb.G[2 * p + 1])));
    }
    out[2 * i] = fd(-a0, rho_a[i]);
    out[2 * i + 1] = fd(-a1, rho_a[i]);
}

// computeViscosity (viscosity.py:222-241), schemes deltaSPH_viscid (:200-218) and
// deltaSPH_inviscid (:123-170); the wall versions of boundaryViscosity.py:199-219 and :123-173
// (inviscid: V_j = m_j / (rho_i + rho_j)). pi_ij = (u_i - u_j).xhat / (r_ij + eps h^2), zero
// where (u_i - u_j).xhat >= 0 with the pi-switch. The per-row factor is
// fl(2 (d + 2) nu rho0) / rho_i (viscid, c1 = that product) or alpha h_i cs rho0 / rho_i
// (inviscid: c1 = alpha, c2 = cs, c3 = rho0), in the reference's operation order.
__global__ void k_viscosity(Pairs nb, int64_t n, const float* __restrict__ m_b, const float* __restrict__ rho_a,
                            const float* __restrict__ rho_b, const float* __restrict__ u_a,
                            const float* __restrict__ u_b, const float* __restrict__ h_a, int inviscid,
                            int wall_volume, int pi_switch, float eps, float c1, float c2, float c3,
                            float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ri = rho_a[i], ui0 = u_a[2 * i], ui1 = u_a[2 * i + 1];
    float a0 = 0.f, a1 = 0.f;
    const int64_t p0 = nb.off[i], p1 = p0 + nb.cnt[i];
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float hh = nb.h[p];
        const float v0 = fs(ui0, u_b[2 * j]), v1 = fs(ui1, u_b[2 * j + 1]);
        const float rij = fm(nb.q[p], hh);
        const float vr = fa(fm(v0, nb.v[2 * p]), fm(v1, nb.v[2 * p + 1]));
        float piv = fd(vr, fa(rij, fm(eps, fm(hh, hh))));
        if (pi_switch && !(vr < 0.f)) piv = 0.f;
        const float V = wall_volume ? fd(m_b[j], fa(ri, rho_b[j])) : fd(m_b[j], rho_b[j]);
        const float s = fm(V, piv);
        a0 = fa(a0, fm(s, nb.G[2 * p]));
        a1 = fa(a1, fm(s, nb.G[2 * p + 1]));
    }
    const float f = inviscid ? fd(fm(fm(fm(c1, h_a[i]), c2), c3), ri) : fd(c1, ri);
    out[2 * i] = fm(f, a0);
    out[2 * i + 1] = fm(f, a1);
}

// mDBCDensity (mDBC.py:50-163) on the ghost -> fluid neighborhood: the Shepard sums, the 3x3
// moment system and the first-order extrapolation to the wall particle, in the reference's
// pair order; the pseudo-inverse of the moment matrix (where a ghost has more than four
// neighbors) in fp64 with torch.linalg.pinv's truncation rule (the reference's fp32 LAPACK
// solve carries ~1e-4 relative rounding on the ill-conditioned matrices near free edges).
__device__ void pinv3_64(const double A[9], double P[9], double rtol);

__global__ void k_mdbc_pairs(Pairs nb, int64_t n, const float* __restrict__ m_f, const float* __restrict__ rho_f,
                             const float* __restrict__ x_wall, const float* __restrict__ x_ghost, float support,
                             float rho0, float* __restrict__ rho_out, float* __restrict__ shepard_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // num = sum m W; den = sum V W; gs = sum rho V gradW; vg = sum V gradW; ps = sum x V W;
    // pm[c][d] = sum x_c V gradW_d, with x_ij = -xhat q h (h = particle.support)
    float num = 0.f, den = 0.f, gs0 = 0.f, gs1 = 0.f, vg0 = 0.f, vg1 = 0.f, ps0 = 0.f, ps1 = 0.f;
    float pm00 = 0.f, pm01 = 0.f, pm10 = 0.f, pm11 = 0.f;
    const int cnt = nb.cnt[i];
    const int64_t p0 = nb.off[i], p1 = p0 + cnt;
    for (int64_t p = p0; p < p1; ++p) {
        const int64_t j = nb.j[p];
        const float W = nb.W[p], g0 = nb.G[2 * p], g1 = nb.G[2 * p + 1];
        const float mj = m_f[j], rj = rho_f[j];
        const float V = fd(mj, rj);
        num = fa(num, fm(mj, W));
        const float vw = fm(V, W);
        den = fa(den, fm(1.0f, vw));
        const float k0 = fm(V, g0), k1 = fm(V, g1);
        gs0 = fa(gs0, fm(rj, k0));
        gs1 = fa(gs1, fm(rj, k1));
        vg0 = fa(vg0, fm(1.0f, k0));
        vg1 = fa(vg1, fm(1.0f, k1));
        const float qh = nb.q[p];
        const float x0 = fm(fm(-nb.v[2 * p], qh), support), x1 = fm(fm(-nb.v[2 * p + 1], qh), support);
        ps0 = fa(ps0, fm(x0, vw));
        ps1 = fa(ps1, fm(x1, vw));
        pm00 = fa(pm00, fm(x0, k0));
        pm01 = fa(pm01, fm(x0, k1));
        pm10 = fa(pm10, fm(x1, k0));
        pm11 = fa(pm11, fm(x1, k1));
    }
    const float shep = fd(num, fa(den, 1e-7f));
    float rho = rho0;
    if (cnt > 0) rho = shep;
    if (cnt > 5) {
        const double A[9] = {den, ps0, ps1, vg0, pm00, pm01, vg1, pm10, pm11};
        double P[9];
        pinv3_64(A, P, 3.0 * 1.1920928955078125e-07);
        const double r0 = P[0] * num + P[1] * gs0 + P[2] * gs1;
        const double r1 = P[3] * num + P[4] * gs0 + P[5] * gs1;
        const double r2 = P[6] * num + P[7] * gs0 + P[8] * gs1;
        const float rel0 = fs(x_wall[2 * i], x_ghost[2 * i]), rel1 = fs(x_wall[2 * i + 1], x_ghost[2 * i + 1]);
        rho = (float)(r0 + (double)rel0 * r1 + (double)rel1 * r2);
    }
    rho_out[i] = rho;
    if (shepard_out) shepard_out[i] = shep;
}

}  // namespace

#include "sph_common.cuh"

namespace {
__device__ void pinv3_64(const double A[9], double P[9], double rtol) { sph::pinv3_f64(A, P, rtol); }
}  // namespace

// ------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------
extern "C" int sph_operation(const sph_pairs_t* nb, int32_t operation, int32_t mode, int32_t divergence_mode,
                             int32_t components, const float* m_b, const float* rho_a, const float* rho_b,
                             const float* q_a, const float* q_b, const float* q_pair, float* out,
                             sph_stream_t stream) {
    if (!pairs_ok(nb) || !out || !m_b) return SPH_ERR_ARGUMENT;
    if (operation < SPH_OP_DENSITY || operation > SPH_OP_LAPLACIAN) return SPH_ERR_ARGUMENT;
    if (components != 1 && components != 2 && components != 4) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->kernels && (operation == SPH_OP_DENSITY || operation == SPH_OP_INTERPOLATE)) return SPH_ERR_ARGUMENT;
    if (operation != SPH_OP_DENSITY) {
        if (!rho_b) return SPH_ERR_ARGUMENT;
        if (!q_pair && !q_b) return SPH_ERR_ARGUMENT;
        const bool needs_a = !q_pair && operation != SPH_OP_INTERPOLATE &&
                             (mode != SPH_MODE_NAIVE || operation == SPH_OP_LAPLACIAN);
        if (needs_a && !q_a) return SPH_ERR_ARGUMENT;
        if (mode == SPH_MODE_SYMMETRIC && !q_pair && !rho_a) return SPH_ERR_ARGUMENT;
    }
    if (operation >= SPH_OP_GRADIENT && !nb->gradients) return SPH_ERR_ARGUMENT;
    if (operation == SPH_OP_DIVERGENCE && components == 1) return SPH_ERR_ARGUMENT;
    if (operation == SPH_OP_CURL && components != 2) return SPH_ERR_ARGUMENT;
    if (operation == SPH_OP_LAPLACIAN) {
        if (components == 4 || mode == SPH_MODE_NAIVE || !nb->distances || !nb->vectors || !nb->supports)
            return SPH_ERR_ARGUMENT;
    }
    const Pairs p = view(nb);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = nb->n_query;
    switch (components) {
        case 1:
            k_operation<1><<<grid_for(n), kOpBlock, 0, st>>>(p, n, operation, mode, divergence_mode, m_b, rho_a, rho_b,
                                                             q_a, q_b, q_pair, out);
            break;
        case 2:
            k_operation<2><<<grid_for(n), kOpBlock, 0, st>>>(p, n, operation, mode, divergence_mode, m_b, rho_a, rho_b,
                                                             q_a, q_b, q_pair, out);
            break;
        default:
            k_operation<4><<<grid_for(n), kOpBlock, 0, st>>>(p, n, operation, mode, divergence_mode, m_b, rho_a, rho_b,
                                                             q_a, q_b, q_pair, out);
            break;
    }
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_covariance(const sph_pairs_t* nb, const float* m_b, const float* rho_b, float* out,
                              sph_stream_t stream) {
    if (!pairs_ok(nb) || !m_b || !rho_b || !out) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->distances || !nb->supports || !nb->vectors || !nb->gradients) return SPH_ERR_ARGUMENT;
    k_covariance<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(view(nb), nb->n_query, m_b, rho_b, out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_density_gradient(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                                    const float* L, float* out, sph_stream_t stream) {
    if (!pairs_ok(nb) || !m_b || !rho_a || !rho_b || !out) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->gradients) return SPH_ERR_ARGUMENT;
    k_density_gradient<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(view(nb), nb->n_query, m_b, rho_a,
                                                                                     rho_b, L, out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_delta_term(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                              const float* grad_a, const float* grad_b, const float* h_a, double delta, double kappa,
                              double cs, float* out, sph_stream_t stream) {
    if (!pairs_ok(nb) || !m_b || !rho_a || !rho_b || !grad_a || !grad_b || !h_a || !out) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->distances || !nb->supports || !nb->vectors || !nb->gradients) return SPH_ERR_ARGUMENT;
    k_delta_term<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(
        view(nb), nb->n_query, m_b, rho_a, rho_b, grad_a, grad_b, h_a, (float)delta, (float)kappa, (float)cs, out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_momentum(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                            const float* u_a, const float* u_b, float* out, sph_stream_t stream) {
    if (!pairs_ok(nb) || !m_b || !rho_a || !rho_b || !u_a || !u_b || !out) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->gradients) return SPH_ERR_ARGUMENT;
    k_momentum<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(view(nb), nb->n_query, m_b, rho_a, rho_b,
                                                                             u_a, u_b, out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_pressure_accel(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                                  const float* p_a, const float* p_b, float* out, sph_stream_t stream) {
    if (!pairs_ok(nb) || !m_b || !rho_a || !rho_b || !p_a || !p_b || !out) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->gradients) return SPH_ERR_ARGUMENT;
    k_pressure_accel<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(view(nb), nb->n_query, m_b, rho_a,
                                                                                   rho_b, p_a, p_b, out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_viscosity(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                             const float* u_a, const float* u_b, const float* h_a, const sph_viscosity_params_t* prm,
                             float* out, sph_stream_t stream) {
    if (!pairs_ok(nb) || !prm || !m_b || !rho_a || !rho_b || !u_a || !u_b || !out) return SPH_ERR_ARGUMENT;
    if (prm->scheme != 0 && prm->scheme != 1) return SPH_ERR_ARGUMENT;
    if (prm->scheme == 1 && !h_a) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->distances || !nb->supports || !nb->vectors || !nb->gradients) return SPH_ERR_ARGUMENT;
    // viscid: the python-side product 2 (d + 2) nu rho0 in double, rounded once (the reference
    // divides that python float by the fp32 densities); inviscid: alpha, cs, rho0 each enter
    // its fp32 product chain
    float c1, c2 = 0.f, c3 = 0.f;
    if (prm->scheme == 0) {
        c1 = (float)(2.0 * (2 + 2) * prm->nu * prm->rho0);
    } else {
        c1 = (float)prm->alpha;
        c2 = (float)prm->cs;
        c3 = (float)prm->rho0;
    }
    const int wall_volume = prm->scheme == 1 && prm->wall_volume;
    k_viscosity<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(
        view(nb), nb->n_query, m_b, rho_a, rho_b, u_a, u_b, h_a, prm->scheme, wall_volume, prm->pi_switch,
        (float)prm->eps, c1, c2, c3, out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_mdbc_density(const sph_pairs_t* nb, const float* m_f, const float* rho_f, const float* x_wall,
                                const float* x_ghost, double support, double rho0, float* rho_out, float* shepard_out,
                                sph_stream_t stream) {
    if (!pairs_ok(nb) || !m_f || !rho_f || !x_wall || !x_ghost || !rho_out) return SPH_ERR_ARGUMENT;
    if (nb->n_query == 0) return SPH_OK;
    if (!nb->distances || !nb->vectors || !nb->kernels || !nb->gradients) return SPH_ERR_ARGUMENT;
    k_mdbc_pairs<<<grid_for(nb->n_query), kOpBlock, 0, (cudaStream_t)stream>>>(
        view(nb), nb->n_query, m_f, rho_f, x_wall, x_ghost, (float)support, (float)rho0, rho_out, shepard_out);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
