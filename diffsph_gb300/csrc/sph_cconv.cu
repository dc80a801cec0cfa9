// Learned continuous-convolution step: the edge-basis aggregation over the exact neighbor
// lists and the basis-weight contraction as a tcgen05 BF16 GEMM (TMA-fed shared-memory
// tiles, FP32 accumulator in tensor memory).
//
// Layer (per particle i, neighbors j within the support H, self included):
//   E_i[b, c] = inv_norm * sum_j phi_b(x_i - x_j) h_j[c]              (aggregation)
//   or, in the relative (difference) form, h_j[c] - h_i[c] in place of h_j[c]
//   y_i[o]    = sum_{b, c} E_i[b, c] W[b C + c, o]                     (contraction, GEMM)
// Basis phi_{8a + m}(x) = w(q) T_a(2q - 1) F_m(theta), q = |x| / H, w(q) = (1 - q^2)^2,
// T_a Chebyshev polynomials (a < 8), F_m the angular Fourier terms of z = x / |x|:
// 1, Re z, Im z, Re z^2, Im z^2, Re z^3, Im z^3, Re z^4 (all but F_0 vanish at x = 0).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <math.h>

#include <mutex>

#include "../../include/sph103.h"
#include "sph_internal.cuh"

namespace sph {
namespace cconv {

// ------------------------------------------------------------------------------------
// tcgen05 GEMM  D[M x N] (fp32, row-major) (+)= A[M x K] (bf16, row-major) * Bt[N x K]^T
// One CTA computes a 128 x BN tile. Warp 0 lane 0 feeds a 4-stage ring of shared-memory
// tiles with TMA (128-byte swizzle, the canonical K-major layout of the MMA); warp 1
// lane 0 issues the MMAs (K = 16 per instruction) into a TMEM accumulator of BN columns
// and releases each stage with tcgen05.commit; all four warps then drain the accumulator
// (warp w owns TMEM lanes 32w..32w+31 = rows) to global memory.
// ------------------------------------------------------------------------------------
constexpr int kBM = 128, kBK = 64, kStages = 4, kThreads = 128;
constexpr uint32_t kSpinLimit = 1u << 22;  // bounded mbarrier polls (seconds at most)
// the poll limit of the GEMM's waits (sph_set_gemm_wait_limit); read at each launch
static uint32_t g_gemm_polls = kSpinLimit;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// false when the phase did not complete within `polls` polls (kSpinLimit by default)
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, uint32_t polls = kSpinLimit) {
    for (uint32_t it = 0; it < polls; ++it)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 B
// apart (stride byte offset), leading byte offset unused for swizzled K-major layouts.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>(1) << 16;
    d |= static_cast<uint64_t>(1024 >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;  // descriptor version of sm_100 and later
    d |= static_cast<uint64_t>(2) << 61;  // SWIZZLE_128B
    return d;
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
struct GemmCfg {
    static constexpr uint32_t kA = kBM * kBK * 2;
    static constexpr uint32_t kB = BN * kBK * 2;
    static constexpr uint32_t kStage = kA + kB;
    static constexpr size_t kSmem = static_cast<size_t>(kStage) * kStages + 1024;
};

// Every mbarrier wait polls at most `polls` times. A wait that runs out sets a bit of *err:
// 1 the producer's wait for a free stage (it then issues no further load), 2 the MMA
// issuer's wait for a loaded stage (it issues no further MMA), 4 the wait for the MMAs to
// complete (the accumulator is then not read), 32 the final wait for loads still in flight.
// Before the TMEM is released the producer waits (bounded) for the last loads it issued, so
// no bulk copy lands in the shared memory of an exited CTA. polls = 0 makes every wait fail
// at once: no load and no MMA is issued.
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb, float* __restrict__ D,
              int64_t ldd, int K, int accumulate, uint32_t* __restrict__ err, uint32_t polls) {
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t full[kStages], empty[kStages], done;
    __shared__ uint32_t tmem_slot;
    using C = GemmCfg<BN>;
    uint8_t* tiles = dsm + ((1024u - (smem_u32(dsm) & 1023u)) & 1023u);  // SW128 tiles: 1024-aligned
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = static_cast<int64_t>(blockIdx.y) * kBM;
    const int n0 = blockIdx.x * BN;
    const int nk = K / kBK;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;

    int issued = 0;  // loads issued by the producer (its lane only)
    if (warp == 0 && lane == 0) {  // TMA producer
        for (int k = 0; k < nk; ++k) {
            const int s = k % kStages;
            const uint32_t ph = (k / kStages) & 1;
            if (!mbar_wait(&empty[s], ph ^ 1, polls)) {
                atomicOr(err, 1u);
                break;
            }
            uint8_t* sa = tiles + s * C::kStage;
            mbar_expect_tx(&full[s], C::kStage);
            tma_load_2d(sa, &ma, &full[s], k * kBK, static_cast<int>(m0));
            tma_load_2d(sa + C::kA, &mb, &full[s], k * kBK, n0);
            issued = k + 1;
        }
    } else if (warp == 1 && lane == 0) {  // MMA issuer
        constexpr uint32_t idesc = idesc_bf16(kBM, BN);
        int mmas = 0;
        for (int k = 0; k < nk; ++k) {
            const int s = k % kStages;
            const uint32_t ph = (k / kStages) & 1;
            if (!mbar_wait(&full[s], ph, polls)) {  // every load issued before this one has landed
                atomicOr(err, 2u);
                break;
            }
            ++mmas;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint64_t da = sw128_desc(smem_u32(tiles + s * C::kStage));
            const uint64_t db = sw128_desc(smem_u32(tiles + s * C::kStage + C::kA));
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk)  // +32 bytes along K inside the swizzle atom
                mma_bf16(tmem, da + 2 * kk, db + 2 * kk, idesc, (k > 0 || kk > 0) ? 1u : 0u);
            mma_commit(&empty[s]);
        }
        // arrives once every MMA issued above has completed; with none issued (a timed-out
        // first wait) a plain arrive, so that no asynchronous arrive outlives the CTA
        if (mmas > 0) mma_commit(&done);
        else mbar_arrive(&done);
    }
    __syncwarp();
    // warp-uniform so that the .sync.aligned TMEM loads below run converged
    const bool ready = __all_sync(0xffffffffu, mbar_wait(&done, 0, polls));
    if (!ready && lane == 0) atomicOr(err, 4u);
    if (warp == 0 && lane == 0) {
        // the last loads issued (one per stage at most) have landed, whether or not the MMA
        // issuer consumed them: each stage's full barrier has at most that one phase pending
        for (int k = issued > kStages ? issued - kStages : 0; k < issued; ++k)
            if (!mbar_wait(&full[k % kStages], (k / kStages) & 1, polls)) atomicOr(err, 32u);
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ready) {
        const int64_t row = m0 + warp * 32 + lane;
        float* drow = D + row * ldd + n0;
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c), v);
            float4* dst = reinterpret_cast<float4*>(drow + c);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float4 o = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                       __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
                if (accumulate) {
                    const float4 p = dst[q];
                    o.x += p.x;
                    o.y += p.y;
                    o.z += p.z;
                    o.w += p.w;
                }
                dst[q] = o;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
}

// ------------------------------------------------------------------------------------
// Edge basis and aggregation (CUDA cores, FP32 accumulation)
// ------------------------------------------------------------------------------------
constexpr int kBasis = 64;
constexpr int kAggThreads = 128;
constexpr int kEdgeChunk = 16;

struct BasisGeo {
    Geo geo;
    float inv_H;
    float eps;  // added to |x| in z = x / (|x| + eps) so that the self pair has z = 0
};

// the 8 values phi_{8a + m}, m = 0..7, of radial order a for the pair vector x
__device__ __forceinline__ void basis_row(float x0, float x1, int a, const BasisGeo& bg, float* out) {
    const float r = sqrtf(x0 * x0 + x1 * x1);
    const float q = fminf(r * bg.inv_H, 1.f);
    const float om = 1.f - q * q;
    const float w = om * om;
    const float s = 2.f * q - 1.f;
    float t0 = 1.f, t1 = s, ta = (a == 0) ? 1.f : s;
    for (int k = 2; k <= a; ++k) {
        const float t2 = 2.f * s * t1 - t0;
        t0 = t1;
        t1 = t2;
        ta = t2;
    }
    const float R = w * ta;
    const float inv = 1.f / (r + bg.eps);
    const float zr = x0 * inv, zi = x1 * inv;
    const float z2r = zr * zr - zi * zi, z2i = 2.f * zr * zi;
    const float z3r = z2r * zr - z2i * zi, z3i = z2r * zi + z2i * zr;
    const float z4r = z3r * zr - z3i * zi;
    out[0] = R;
    out[1] = R * zr;
    out[2] = R * zi;
    out[3] = R * z2r;
    out[4] = R * z2i;
    out[5] = R * z3r;
    out[6] = R * z3i;
    out[7] = R * z4r;
}

// phi for up to kEdgeChunk edges of the row [e0, e1) into s_phi[edge][64]; sign = +1 for
// x_i - x_j (row of i lists j), -1 for the transposed use (row of j lists i)
__device__ __forceinline__ void chunk_basis(const float* __restrict__ x, float2 pi, const int32_t* __restrict__ nbr,
                                            int64_t e0, int64_t e1, const BasisGeo& bg, float sign,
                                            float (*s_phi)[kBasis], int32_t* s_j) {
    const int t = threadIdx.x;
    const int e = t >> 3, a = t & 7;
    const int64_t ge = e0 + e;
    float vals[8];
    int j = -1;
    if (ge < e1) {
        j = nbr[ge];
        float x0, x1;
        pair_vec<true>(pi, make_float2(x[2 * j], x[2 * j + 1]), bg.geo, x0, x1);
        basis_row(sign * x0, sign * x1, a, bg, vals);
    } else {
#pragma unroll
        for (int m = 0; m < 8; ++m) vals[m] = 0.f;
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) s_phi[e][a * 8 + m] = vals[m];
    if (a == 0) s_j[e] = j;
}

template <int C, bool REL>
__global__ void __launch_bounds__(kAggThreads) k_aggregate(int64_t n, const float* __restrict__ x,
                                                           const int64_t* __restrict__ off,
                                                           const int32_t* __restrict__ nbr, BasisGeo bg,
                                                           float inv_norm, const __nv_bfloat16* __restrict__ h,
                                                           __nv_bfloat16* __restrict__ E) {
    constexpr int kPer = kBasis * C / kAggThreads;  // outputs per thread
    constexpr int kStride = kAggThreads / C;        // basis stride between them
    __shared__ float s_phi[kEdgeChunk][kBasis];
    __shared__ int32_t s_j[kEdgeChunk];
    const int64_t i = blockIdx.x;
    const int t = threadIdx.x;
    const int c = t % C, b0 = t / C;
    const float2 pi = make_float2(x[2 * i], x[2 * i + 1]);
    const float hi = REL ? __bfloat162float(h[i * C + c]) : 0.f;
    float acc[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) acc[k] = 0.f;
    const int64_t e1 = off[i + 1];
    for (int64_t e0 = off[i]; e0 < e1; e0 += kEdgeChunk) {
        chunk_basis(x, pi, nbr, e0, e1, bg, 1.f, s_phi, s_j);
        __syncthreads();
        const int ne = static_cast<int>(e1 - e0 < kEdgeChunk ? e1 - e0 : kEdgeChunk);
        for (int e = 0; e < ne; ++e) {
            const float hv = __bfloat162float(h[static_cast<int64_t>(s_j[e]) * C + c]) - hi;
#pragma unroll
            for (int k = 0; k < kPer; ++k) acc[k] = fmaf(s_phi[e][b0 + k * kStride], hv, acc[k]);
        }
        __syncthreads();
    }
    __nv_bfloat16* Ei = E + i * (kBasis * C);
#pragma unroll
    for (int k = 0; k < kPer; ++k) Ei[(b0 + k * kStride) * C + c] = __float2bfloat16_rn(acc[k] * inv_norm);
}

// ------------------------------------------------------------------------------------
// Aggregation on the tensor cores. Per particle, E_i = Phi_i^T G_i with Phi_i [edges x 64]
// the basis values and G_i [edges x C] the neighbor features (or their differences to h_i in
// the relative form), edges zero-padded to 64. Two particles share one M = 128 MMA group in
// block-diagonal form: K atom 0 holds particle A (rows 0..63 of the A tile = Phi_A^T, rows
// 64..127 zero) and K atom 1 particle B (rows 0..63 zero, rows 64..127 = Phi_B^T); the B
// tile holds G_A^T and G_B^T in the two atoms. The accumulator rows 0..63 are then E_A and
// rows 64..127 E_B, drained by warps 0-1 and 2-3. Operands are K-major with the 128-byte
// swizzle; the zero quadrants are written once. One stage of 48 KB (C = 64) lets four CTAs
// share an SM, which hides the gather latency of one another's operand builds.
// ------------------------------------------------------------------------------------
constexpr int kTcMaxEdges = 64;             // neighbors per particle (row), self included
constexpr int kTcPairsPerCta = 32;          // 64 particles per CTA
constexpr uint32_t kTcAtomA = 128u * 128u;  // 128 rows x 64 bf16

template <int C>
struct TcCfg {
    static constexpr uint32_t kAtomB = C * 128u;
    static constexpr uint32_t kTileA = 2 * kTcAtomA;
    static constexpr uint32_t kTileB = 2 * kAtomB;
    static constexpr size_t kSmem = static_cast<size_t>(kTileA + kTileB) + 1024;
    static constexpr int kCols = C < 32 ? 32 : C;
};

// byte offset of element (row r, column k) in a K-major atom of 64 bf16 columns with the
// 128-byte swizzle (16-byte chunk index XOR row mod 8), as TMA writes it
__device__ __forceinline__ uint32_t sw128_off(int r, int k) {
    return static_cast<uint32_t>(r) * 128u +
           ((((static_cast<uint32_t>(k) >> 3) ^ (static_cast<uint32_t>(r) & 7u))) << 4) +
           (static_cast<uint32_t>(k) & 7u) * 2u;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

template <int C, bool REL>
__global__ void __launch_bounds__(128, 4)
    k_aggregate_tc(int64_t n, const float* __restrict__ x, const int64_t* __restrict__ off,
                   const int32_t* __restrict__ nbr, BasisGeo bg, float inv_norm,
                   const __nv_bfloat16* __restrict__ h, __nv_bfloat16* __restrict__ E, uint32_t* __restrict__ err) {
    using Cf = TcCfg<C>;
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t mma_done;
    __shared__ uint32_t tmem_slot;
    uint8_t* tiles = dsm + ((1024u - (smem_u32(dsm) & 1023u)) & 1023u);
    uint8_t* A = tiles;
    uint8_t* B = tiles + Cf::kTileA;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = static_cast<int64_t>(blockIdx.x) * (2 * kTcPairsPerCta);
    for (uint32_t o = static_cast<uint32_t>(tid) * 16u; o < Cf::kTileA + Cf::kTileB; o += 128u * 16u)
        *reinterpret_cast<uint4*>(tiles + o) = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        mbar_init(&mma_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(Cf::kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = idesc_bf16(128, C);
    for (int it = 0; it < kTcPairsPerCta; ++it) {
        const int64_t ia = q0 + 2 * it;
        if (ia >= n) break;  // uniform across the CTA
        // one thread per (particle p, edge e): the 64 basis values go to rows 64 p + b of A atom
        // p and the neighbor's C features to rows c of B atom p, both at column e; lanes of a
        // warp hold consecutive edges, so every store hits distinct banks
        {
            const int p = tid >> 6, e = tid & 63;
            const int64_t i = ia + p;
            int ne = 0;
            int64_t e0 = 0;
            if (i < n) {
                e0 = off[i];
                ne = static_cast<int>(off[i + 1] - e0);
                if (ne > kTcMaxEdges) {
                    if (e == 0) atomicOr(err, 8u);
                    ne = kTcMaxEdges;
                }
            }
            const bool valid = e < ne;
            const int64_t j = valid ? static_cast<int64_t>(nbr[e0 + e]) : 0;
            float x0 = 0.f, x1 = 0.f;
            if (valid)
                pair_vec<true>(make_float2(x[2 * i], x[2 * i + 1]), make_float2(x[2 * j], x[2 * j + 1]), bg.geo, x0,
                               x1);
            // basis: w(q) T_a(2q - 1) F_m(z), z = x / (|x| + eps)
            const float r = sqrtf(x0 * x0 + x1 * x1);
            const float q = fminf(r * bg.inv_H, 1.f);
            const float om = 1.f - q * q;
            const float w = valid ? om * om : 0.f;
            const float sc = 2.f * q - 1.f;
            const float inv = 1.f / (r + bg.eps);
            const float zr = x0 * inv, zi = x1 * inv;
            const float z2r = zr * zr - zi * zi, z2i = 2.f * zr * zi;
            const float z3r = z2r * zr - z2i * zi, z3i = z2r * zi + z2i * zr;
            const float z4r = z3r * zr - z3i * zi;
            uint8_t* atomA = A + p * kTcAtomA;
            float tm1 = 1.f, t0 = sc;
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                float ta;
                if (a == 0) {
                    ta = 1.f;
                } else if (a == 1) {
                    ta = sc;
                } else {
                    ta = 2.f * sc * t0 - tm1;
                    tm1 = t0;
                    t0 = ta;
                }
                const float R = w * ta;
                const int row = 64 * p + 8 * a;
                __nv_bfloat16* const bp = reinterpret_cast<__nv_bfloat16*>(atomA);
                bp[sw128_off(row + 0, e) >> 1] = __float2bfloat16_rn(R);
                bp[sw128_off(row + 1, e) >> 1] = __float2bfloat16_rn(R * zr);
                bp[sw128_off(row + 2, e) >> 1] = __float2bfloat16_rn(R * zi);
                bp[sw128_off(row + 3, e) >> 1] = __float2bfloat16_rn(R * z2r);
                bp[sw128_off(row + 4, e) >> 1] = __float2bfloat16_rn(R * z2i);
                bp[sw128_off(row + 5, e) >> 1] = __float2bfloat16_rn(R * z3r);
                bp[sw128_off(row + 6, e) >> 1] = __float2bfloat16_rn(R * z3i);
                bp[sw128_off(row + 7, e) >> 1] = __float2bfloat16_rn(R * z4r);
            }
            __nv_bfloat16* const bq = reinterpret_cast<__nv_bfloat16*>(B + p * Cf::kAtomB);
            const uint4* hj = reinterpret_cast<const uint4*>(h + j * C);
            const uint4* hi = reinterpret_cast<const uint4*>(h + (i < n ? i : 0) * C);
#pragma unroll
            for (int c8 = 0; c8 < C / 8; ++c8) {
                uint4 vj = valid ? hj[c8] : make_uint4(0u, 0u, 0u, 0u);
                const __nv_bfloat162* pj = reinterpret_cast<const __nv_bfloat162*>(&vj);
                float f[8];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float2 g = __bfloat1622float2(pj[t]);
                    f[2 * t] = g.x;
                    f[2 * t + 1] = g.y;
                }
                if (REL && valid) {
                    uint4 vi = hi[c8];
                    const __nv_bfloat162* pi2 = reinterpret_cast<const __nv_bfloat162*>(&vi);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const float2 g = __bfloat1622float2(pi2[t]);
                        f[2 * t] -= g.x;
                        f[2 * t + 1] -= g.y;
                    }
                }
#pragma unroll
                for (int t = 0; t < 8; ++t) bq[sw128_off(8 * c8 + t, e) >> 1] = __float2bfloat16_rn(f[t]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor core
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int at = 0; at < 2; ++at) {
                const uint64_t da = sw128_desc(smem_u32(A + at * kTcAtomA));
                const uint64_t db = sw128_desc(smem_u32(B + at * Cf::kAtomB));
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    mma_bf16(tmem, da + 2 * kk, db + 2 * kk, idesc, (at > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&mma_done);
        }
        __syncwarp();
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&mma_done, static_cast<uint32_t>(it) & 1u));
        if (!ok && lane == 0) atomicOr(err, 16u);
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int p = warp >> 1;  // warps 0-1: particle A (rows 0..63), 2-3: particle B
        const int64_t i = ia + p;
        if (ok && i < n) {
            const int b = (warp & 1) * 32 + lane;
            __nv_bfloat16* dst = E + i * (64 * C) + b * C;
#pragma unroll 1
            for (int c = 0; c < C; c += 16) {
                uint32_t v[16];
                tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c), v);
                uint4 o0, o1;
                o0.x = pack_bf16x2(__uint_as_float(v[0]) * inv_norm, __uint_as_float(v[1]) * inv_norm);
                o0.y = pack_bf16x2(__uint_as_float(v[2]) * inv_norm, __uint_as_float(v[3]) * inv_norm);
                o0.z = pack_bf16x2(__uint_as_float(v[4]) * inv_norm, __uint_as_float(v[5]) * inv_norm);
                o0.w = pack_bf16x2(__uint_as_float(v[6]) * inv_norm, __uint_as_float(v[7]) * inv_norm);
                o1.x = pack_bf16x2(__uint_as_float(v[8]) * inv_norm, __uint_as_float(v[9]) * inv_norm);
                o1.y = pack_bf16x2(__uint_as_float(v[10]) * inv_norm, __uint_as_float(v[11]) * inv_norm);
                o1.z = pack_bf16x2(__uint_as_float(v[12]) * inv_norm, __uint_as_float(v[13]) * inv_norm);
                o1.w = pack_bf16x2(__uint_as_float(v[14]) * inv_norm, __uint_as_float(v[15]) * inv_norm);
                *reinterpret_cast<uint4*>(dst + c) = o0;
                *reinterpret_cast<uint4*>(dst + c + 8) = o1;
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cf::kCols));
}

// dh_j[c] = inv_norm * sum_{i in N(j)} sum_b phi_b(x_i - x_j) dE_i[b C + c]; the relative
// form adds the own term -inv_norm * sum_b dE_j[b C + c] sum_{i in N(j)} phi_b(x_j - x_i)
template <int C, bool REL>
__global__ void __launch_bounds__(kAggThreads) k_aggregate_t(int64_t n, const float* __restrict__ x,
                                                             const int64_t* __restrict__ off,
                                                             const int32_t* __restrict__ nbr, BasisGeo bg,
                                                             float inv_norm, const float* __restrict__ dE,
                                                             int64_t ldE, float* __restrict__ dh) {
    constexpr int kPer = kBasis * C / kAggThreads;
    constexpr int kStride = kAggThreads / C;
    __shared__ float s_phi[kEdgeChunk][kBasis];
    __shared__ int32_t s_j[kEdgeChunk];
    __shared__ float s_red[kAggThreads];
    const int64_t jrow = blockIdx.x;
    const int t = threadIdx.x;
    const int c = t % C, b0 = t / C;
    const float2 pj = make_float2(x[2 * jrow], x[2 * jrow + 1]);
    float acc = 0.f;
    float own[REL ? kPer : 1];
#pragma unroll
    for (int k = 0; k < (REL ? kPer : 1); ++k) own[k] = 0.f;
    const int64_t e1 = off[jrow + 1];
    for (int64_t e0 = off[jrow]; e0 < e1; e0 += kEdgeChunk) {
        chunk_basis(x, pj, nbr, e0, e1, bg, -1.f, s_phi, s_j);
        __syncthreads();
        const int ne = static_cast<int>(e1 - e0 < kEdgeChunk ? e1 - e0 : kEdgeChunk);
        for (int e = 0; e < ne; ++e) {
            const float* dEi = dE + static_cast<int64_t>(s_j[e]) * ldE + c;
#pragma unroll
            for (int k = 0; k < kPer; ++k) acc = fmaf(s_phi[e][b0 + k * kStride], dEi[(b0 + k * kStride) * C], acc);
            if (REL) {
                // phi_b(x_j - x_i) = (-1)^(angular order of b) phi_b(x_i - x_j): F_1, F_2, F_5, F_6 are odd
#pragma unroll
                for (int k = 0; k < (REL ? kPer : 1); ++k) {
                    const int b = b0 + k * kStride;
                    const int m = b & 7;
                    const float sg = (m == 1 || m == 2 || m == 5 || m == 6) ? -1.f : 1.f;
                    own[k] = fmaf(sg, s_phi[e][b], own[k]);
                }
            }
        }
        __syncthreads();
    }
    if (REL) {
        const float* dEj = dE + jrow * ldE + c;
#pragma unroll
        for (int k = 0; k < (REL ? kPer : 1); ++k) acc = fmaf(-own[k], dEj[(b0 + k * kStride) * C], acc);
    }
    s_red[t] = acc;
    __syncthreads();
    if (t < C) {
        float s = 0.f;
        for (int k = 0; k < kStride; ++k) s += s_red[t + k * C];
        dh[jrow * C + t] = s * inv_norm;
    }
}

// ------------------------------------------------------------------------------------
// host
// ------------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// row-major bf16 matrix [rows x cols] (leading dimension ld elements), box 64 x box_rows
int make_map(CUtensorMap* m, const void* ptr, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return SPH_ERR_CUDA;
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(kBK), static_cast<cuuint32_t>(box_rows)};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? SPH_OK : SPH_ERR_ARGUMENT;
}

template <int BN>
int launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, float* D, int64_t M, int64_t N, int64_t K, int64_t ldd,
                int acc, uint32_t* err, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_gemm_tn<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(GemmCfg<BN>::kSmem));
    });
    if (attr != cudaSuccess) return SPH_ERR_CUDA;
    dim3 grid(static_cast<unsigned>(N / BN), static_cast<unsigned>(M / kBM));
    k_gemm_tn<BN><<<grid, kThreads, GemmCfg<BN>::kSmem, s>>>(ma, mb, D, ldd, static_cast<int>(K), acc, err,
                                                              g_gemm_polls);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

BasisGeo make_basis_geo(const sph_domain_t* d, double support) {
    BasisGeo bg;
    int per[2] = {d->periodic[0], d->periodic[1]};
    bg.geo = make_geo(d->min, d->max, per);
    bg.inv_H = static_cast<float>(1.0 / support);
    bg.eps = static_cast<float>(1e-6 * support);
    return bg;
}

}  // namespace cconv
}  // namespace sph

using namespace sph;
using namespace sph::cconv;

extern "C" int sph_set_gemm_wait_limit(uint32_t polls, uint32_t* previous) {
    if (previous) *previous = g_gemm_polls;
    g_gemm_polls = polls;
    return SPH_OK;
}

extern "C" int sph_gemm_bf16_tn(const void* A, const void* Bt, float* D, int64_t M, int64_t N, int64_t K, int64_t lda,
                                int64_t ldb, int64_t ldd, int32_t accumulate, uint32_t* err, sph_stream_t stream) {
    if (!A || !Bt || !D || !err) return SPH_ERR_ARGUMENT;
    if (M <= 0 || N <= 0 || K <= 0 || M % kBM || N % 64 || K % kBK) return SPH_ERR_ARGUMENT;
    if (M / kBM > 65535 || lda < K || ldb < K || ldd < N || lda % 8 || ldb % 8 || ldd % 4) return SPH_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(Bt) | reinterpret_cast<uintptr_t>(D)) & 15)
        return SPH_ERR_ARGUMENT;
    const int bn = (N % 256 == 0) ? 256 : (N % 128 == 0) ? 128 : 64;
    CUtensorMap ma, mb;
    int rc = make_map(&ma, A, M, K, lda, kBM);
    if (!rc) rc = make_map(&mb, Bt, N, K, ldb, bn);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (bn == 256) return launch_gemm<256>(ma, mb, D, M, N, K, ldd, accumulate, err, s);
    if (bn == 128) return launch_gemm<128>(ma, mb, D, M, N, K, ldd, accumulate, err, s);
    return launch_gemm<64>(ma, mb, D, M, N, K, ldd, accumulate, err, s);
}

static int check_agg(int64_t n, const float* x, const int64_t* off, const sph_domain_t* d, double support,
                     int32_t channels) {
    if (n < 0 || !d || support <= 0) return SPH_ERR_ARGUMENT;
    if (n > 0 && (!x || !off)) return SPH_ERR_ARGUMENT;
    if (channels != 16 && channels != 32 && channels != 64) return SPH_ERR_ARGUMENT;
    return SPH_OK;
}

extern "C" int sph_cconv_aggregate(const float* x, int64_t n, const int64_t* offsets, const int32_t* neighbors,
                                   const sph_domain_t* domain, double support, double inv_norm, const void* h,
                                   int32_t channels, int32_t relative, void* E, sph_stream_t stream) {
    int rc = check_agg(n, x, offsets, domain, support, channels);
    if (rc) return rc;
    if (n == 0) return SPH_OK;
    if (!h || !E || !neighbors) return SPH_ERR_ARGUMENT;
    BasisGeo bg = make_basis_geo(domain, support);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto* hb = static_cast<const __nv_bfloat16*>(h);
    auto* Eb = static_cast<__nv_bfloat16*>(E);
    const float nz = static_cast<float>(inv_norm);
    const unsigned g = static_cast<unsigned>(n);
#define SPH_AGG(CC, RR) k_aggregate<CC, RR><<<g, kAggThreads, 0, s>>>(n, x, offsets, neighbors, bg, nz, hb, Eb)
    if (channels == 16) {
        if (relative) SPH_AGG(16, true); else SPH_AGG(16, false);
    } else if (channels == 32) {
        if (relative) SPH_AGG(32, true); else SPH_AGG(32, false);
    } else {
        if (relative) SPH_AGG(64, true); else SPH_AGG(64, false);
    }
#undef SPH_AGG
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_cconv_aggregate_t(const float* x, int64_t n, const int64_t* offsets, const int32_t* neighbors,
                                     const sph_domain_t* domain, double support, double inv_norm, const float* dE,
                                     int64_t ldE, int32_t channels, int32_t relative, float* dh,
                                     sph_stream_t stream) {
    int rc = check_agg(n, x, offsets, domain, support, channels);
    if (rc) return rc;
    if (n == 0) return SPH_OK;
    if (!dE || !dh || !neighbors || ldE < 64 * channels) return SPH_ERR_ARGUMENT;
    BasisGeo bg = make_basis_geo(domain, support);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const float nz = static_cast<float>(inv_norm);
    const unsigned g = static_cast<unsigned>(n);
#define SPH_AGGT(CC, RR) k_aggregate_t<CC, RR><<<g, kAggThreads, 0, s>>>(n, x, offsets, neighbors, bg, nz, dE, ldE, dh)
    if (channels == 16) {
        if (relative) SPH_AGGT(16, true); else SPH_AGGT(16, false);
    } else if (channels == 32) {
        if (relative) SPH_AGGT(32, true); else SPH_AGGT(32, false);
    } else {
        if (relative) SPH_AGGT(64, true); else SPH_AGGT(64, false);
    }
#undef SPH_AGGT
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// ------------------------------------------------------------------------------------
// The same aggregation for C = 64 with both operands MN-major (128-byte swizzle): a K row
// (one edge) of A is a particle's 64 basis values, of B the neighbor's 64 features, 128
// contiguous bytes each. A thread per edge and operand (256 threads: the basis rows and the
// feature rows are built by different halves of the CTA) therefore writes eight 16-byte
// chunks, the features copied as they sit in global memory, instead of one 2-byte value per
// basis row and feature; all eight warps then drain TMEM, two per lane quarter. A holds, per group of 8 K rows, the two particles' 64-row atoms
// side by side (1 KB each; LBO 1 KB between them, SBO 2 KB between K groups); B holds one
// 64-wide atom per K group (SBO 1 KB). Block-diagonal as above: K rows 0..63 are particle
// A's edges (its atom), 64..127 particle B's; the other atom's rows stay zero.
// ------------------------------------------------------------------------------------
constexpr uint32_t kMnA = 16u * 2048u;  // 16 K groups x (2 atoms x 8 rows x 128 B)
constexpr uint32_t kMnB = 16u * 1024u;  // 16 K groups x 8 rows x 128 B
constexpr size_t kMnSmem = static_cast<size_t>(kMnA + kMnB) + 1024;

__device__ __forceinline__ uint64_t mn128_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;  // descriptor version of sm_100 and later
    d |= static_cast<uint64_t>(2) << 61;  // SWIZZLE_128B
    return d;
}

// kind::f16 instruction descriptor with A and B MN-major (bits 15 and 16)
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) {
    return idesc_bf16(m, n) | (1u << 15) | (1u << 16);
}

template <bool REL>
__global__ void __launch_bounds__(256, 4)
    k_aggregate_tc_mn(int64_t n, const float* __restrict__ x, const int64_t* __restrict__ off,
                      const int32_t* __restrict__ nbr, BasisGeo bg, float inv_norm,
                      const __nv_bfloat16* __restrict__ h, __nv_bfloat16* __restrict__ E, uint32_t* __restrict__ err) {
    constexpr int C = 64;
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t mma_done;
    __shared__ uint32_t tmem_slot;
    uint8_t* tiles = dsm + ((1024u - (smem_u32(dsm) & 1023u)) & 1023u);
    uint8_t* A = tiles;
    uint8_t* B = tiles + kMnA;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t q0 = static_cast<int64_t>(blockIdx.x) * (2 * kTcPairsPerCta);
    for (uint32_t o = static_cast<uint32_t>(tid) * 16u; o < kMnA + kMnB; o += 256u * 16u)
        *reinterpret_cast<uint4*>(tiles + o) = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        mbar_init(&mma_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(64));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = idesc_bf16_mn(128, C);
    // threads 0..127 build the basis rows (A), 128..255 the feature rows (B), one K row
    // (edge e of particle p of the pair) each
    const int role = tid >> 7, t = tid & 127;
    const int p = t >> 6, e = t & 63;
    const int k = 64 * p + e, grp = k >> 3, r = k & 7;
    uint8_t* row = role == 0 ? A + grp * 2048 + p * 1024 + r * 128 : B + grp * 1024 + r * 128;
    for (int it = 0; it < kTcPairsPerCta; ++it) {
        const int64_t ia = q0 + 2 * it;
        if (ia >= n) break;  // uniform across the CTA
        {
            const int64_t i = ia + p;
            int ne = 0;
            int64_t e0 = 0;
            if (i < n) {
                e0 = off[i];
                ne = static_cast<int>(off[i + 1] - e0);
                if (ne > kTcMaxEdges) {
                    if (e == 0 && role == 0) atomicOr(err, 8u);
                    ne = kTcMaxEdges;
                }
            }
            const bool valid = e < ne;
            const int64_t j = valid ? static_cast<int64_t>(nbr[e0 + e]) : 0;
            if (role == 0) {
                float x0 = 0.f, x1 = 0.f;
                if (valid)
                    pair_vec<true>(make_float2(x[2 * i], x[2 * i + 1]), make_float2(x[2 * j], x[2 * j + 1]), bg.geo,
                                   x0, x1);
                // basis: w(q) T_a(2q - 1) F_m(z); chunk a of the row holds phi_{8a..8a+7}
                const float rr = sqrtf(x0 * x0 + x1 * x1);
                const float q = fminf(rr * bg.inv_H, 1.f);
                const float om = 1.f - q * q;
                const float w = valid ? om * om : 0.f;
                const float sc = 2.f * q - 1.f;
                const float inv = 1.f / (rr + bg.eps);
                const float zr = x0 * inv, zi = x1 * inv;
                const float z2r = zr * zr - zi * zi, z2i = 2.f * zr * zi;
                const float z3r = z2r * zr - z2i * zi, z3i = z2r * zi + z2i * zr;
                const float z4r = z3r * zr - z3i * zi;
                float tm1 = 1.f, t0 = sc;
#pragma unroll
                for (int a = 0; a < 8; ++a) {
                    float ta;
                    if (a == 0) {
                        ta = 1.f;
                    } else if (a == 1) {
                        ta = sc;
                    } else {
                        ta = 2.f * sc * t0 - tm1;
                        tm1 = t0;
                        t0 = ta;
                    }
                    const float R = w * ta;
                    uint4 v;
                    v.x = pack_bf16x2(R, R * zr);
                    v.y = pack_bf16x2(R * zi, R * z2r);
                    v.z = pack_bf16x2(R * z2i, R * z3r);
                    v.w = pack_bf16x2(R * z3i, R * z4r);
                    *reinterpret_cast<uint4*>(row + ((a ^ r) << 4)) = v;
                }
            } else if (!REL) {
                // the neighbor's feature row, copied global -> shared in eight asynchronous
                // 16-byte pieces (zeros for a padding edge)
                const __nv_bfloat16* hj = h + j * C;
#pragma unroll
                for (int c8 = 0; c8 < C / 8; ++c8) {
                    uint8_t* dst = row + ((c8 ^ r) << 4);
                    if (valid)
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(hj + 8 * c8)
                                     : "memory");
                    else
                        *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
                }
                asm volatile("cp.async.wait_all;" ::: "memory");
            } else {
                // the differences of the neighbor's features to particle i's, 16 B per chunk
                const uint4* hj = reinterpret_cast<const uint4*>(h + j * C);
                const uint4* hi = reinterpret_cast<const uint4*>(h + (i < n ? i : 0) * C);
                uint4 vj[C / 8];
#pragma unroll
                for (int c8 = 0; c8 < C / 8; ++c8) vj[c8] = valid ? hj[c8] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (int c8 = 0; c8 < C / 8; ++c8) {
                    if (REL && valid) {
                        const uint4 vi = hi[c8];
                        __nv_bfloat162* pj = reinterpret_cast<__nv_bfloat162*>(&vj[c8]);
                        const __nv_bfloat162* pi2 = reinterpret_cast<const __nv_bfloat162*>(&vi);
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const float2 a2 = __bfloat1622float2(pj[u]), b2 = __bfloat1622float2(pi2[u]);
                            pj[u] = __floats2bfloat162_rn(a2.x - b2.x, a2.y - b2.y);
                        }
                    }
                    *reinterpret_cast<uint4*>(row + ((c8 ^ r) << 4)) = vj[c8];
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor core
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)  // 16 K rows (2 groups) per MMA
                mma_bf16(tmem, mn128_desc(smem_u32(A + kk * 4096), 1024u, 2048u),
                         mn128_desc(smem_u32(B + kk * 2048), 1024u, 1024u), idesc, kk > 0 ? 1u : 0u);
            mma_commit(&mma_done);
        }
        __syncwarp();
        const bool ok_w = __all_sync(0xffffffffu, mbar_wait(&mma_done, static_cast<uint32_t>(it) & 1u));
        if (!ok_w && lane == 0) atomicOr(err, 16u);
        const bool ok = __syncthreads_and(ok_w) != 0;  // the staging below needs every warp's rows
        asm volatile("tcgen05.fence::after_thread_sync;");
        // warp w drains TMEM lanes 32 (w % 4) .. + 31 (its quarter), columns 32 (w / 4) .. + 31,
        // into the B tile (free once the MMA has completed) as the pair's E rows: row 64 p + b,
        // 128 B, its 16-byte chunks XOR-swizzled by the row so that the lanes' stores spread
        // over the banks. Then the CTA copies the two particles' E (16 KB, contiguous in
        // global memory) out with coalesced 16-byte stores.
        const int qd = warp & 3, half = warp >> 2;
        if (ok) {
            const int erow = qd * 32 + lane;  // = 64 pd + b
#pragma unroll
            for (int c = 32 * half; c < 32 * half + 32; c += 16) {
                uint32_t v[16];
                tmem_ld16(tmem + (static_cast<uint32_t>(qd * 32) << 16) + static_cast<uint32_t>(c), v);
                uint4 o0, o1;
                o0.x = pack_bf16x2(__uint_as_float(v[0]) * inv_norm, __uint_as_float(v[1]) * inv_norm);
                o0.y = pack_bf16x2(__uint_as_float(v[2]) * inv_norm, __uint_as_float(v[3]) * inv_norm);
                o0.z = pack_bf16x2(__uint_as_float(v[4]) * inv_norm, __uint_as_float(v[5]) * inv_norm);
                o0.w = pack_bf16x2(__uint_as_float(v[6]) * inv_norm, __uint_as_float(v[7]) * inv_norm);
                o1.x = pack_bf16x2(__uint_as_float(v[8]) * inv_norm, __uint_as_float(v[9]) * inv_norm);
                o1.y = pack_bf16x2(__uint_as_float(v[10]) * inv_norm, __uint_as_float(v[11]) * inv_norm);
                o1.z = pack_bf16x2(__uint_as_float(v[12]) * inv_norm, __uint_as_float(v[13]) * inv_norm);
                o1.w = pack_bf16x2(__uint_as_float(v[14]) * inv_norm, __uint_as_float(v[15]) * inv_norm);
                const int ch = c >> 3;  // 16-byte chunk of the row
                *reinterpret_cast<uint4*>(B + erow * 128 + (((ch) ^ (erow & 7)) << 4)) = o0;
                *reinterpret_cast<uint4*>(B + erow * 128 + (((ch + 1) ^ (erow & 7)) << 4)) = o1;
            }
        }
        __syncthreads();
        if (ok) {
            const int64_t rows = (ia + 1 < n) ? 128 : 64;  // E rows of the pair that exist
            uint4* dst = reinterpret_cast<uint4*>(E + ia * (64 * C));
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int idx = u * 256 + tid;  // 16-byte unit of the pair's E
                const int erow = idx >> 3, ch = idx & 7;
                if (erow < rows) dst[idx] = *reinterpret_cast<const uint4*>(B + erow * 128 + ((ch ^ (erow & 7)) << 4));
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(64));
}

template <bool REL>
static int launch_agg_tc_mn(int64_t n, const float* x, const int64_t* off, const int32_t* nbr, const BasisGeo& bg,
                            float nz, const __nv_bfloat16* h, __nv_bfloat16* E, uint32_t* err, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_aggregate_tc_mn<REL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(kMnSmem));
    });
    if (attr != cudaSuccess) return SPH_ERR_CUDA;
    const unsigned grid = static_cast<unsigned>((n + 2 * kTcPairsPerCta - 1) / (2 * kTcPairsPerCta));
    k_aggregate_tc_mn<REL><<<grid, 256, kMnSmem, s>>>(n, x, off, nbr, bg, nz, h, E, err);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

template <int C, bool REL>
static int launch_agg_tc(int64_t n, const float* x, const int64_t* off, const int32_t* nbr, const BasisGeo& bg,
                         float nz, const __nv_bfloat16* h, __nv_bfloat16* E, uint32_t* err, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_aggregate_tc<C, REL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(TcCfg<C>::kSmem));
    });
    if (attr != cudaSuccess) return SPH_ERR_CUDA;
    const unsigned grid = static_cast<unsigned>((n + 2 * kTcPairsPerCta - 1) / (2 * kTcPairsPerCta));
    k_aggregate_tc<C, REL><<<grid, 128, TcCfg<C>::kSmem, s>>>(n, x, off, nbr, bg, nz, h, E, err);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_cconv_aggregate_tc(const float* x, int64_t n, const int64_t* offsets, const int32_t* neighbors,
                                      const sph_domain_t* domain, double support, double inv_norm, const void* h,
                                      int32_t channels, int32_t relative, void* E, uint32_t* err,
                                      sph_stream_t stream) {
    int rc = check_agg(n, x, offsets, domain, support, channels);
    if (rc) return rc;
    if (n == 0) return SPH_OK;
    if (!h || !E || !neighbors || !err) return SPH_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(E) | reinterpret_cast<uintptr_t>(h)) & 15) return SPH_ERR_ARGUMENT;
    BasisGeo bg = make_basis_geo(domain, support);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto* hb = static_cast<const __nv_bfloat16*>(h);
    auto* Eb = static_cast<__nv_bfloat16*>(E);
    const float nz = static_cast<float>(inv_norm);
    if (channels == 16)
        return relative ? launch_agg_tc<16, true>(n, x, offsets, neighbors, bg, nz, hb, Eb, err, s)
                        : launch_agg_tc<16, false>(n, x, offsets, neighbors, bg, nz, hb, Eb, err, s);
    if (channels == 32)
        return relative ? launch_agg_tc<32, true>(n, x, offsets, neighbors, bg, nz, hb, Eb, err, s)
                        : launch_agg_tc<32, false>(n, x, offsets, neighbors, bg, nz, hb, Eb, err, s);
    return relative ? launch_agg_tc_mn<true>(n, x, offsets, neighbors, bg, nz, hb, Eb, err, s)
                    : launch_agg_tc_mn<false>(n, x, offsets, neighbors, bg, nz, hb, Eb, err, s);
}
