/*
 * sph103 — C ABI of the GB300 (sm_103a) delta-SPH particle path.
 *
 * All pointers are device pointers unless named *_host. All sizes are element counts.
 * Every entry point returns an int status (SPH_OK = 0) and launches its work on the
 * given stream; none of them allocates device memory: callers query a workspace size
 * and pass the memory in. Nothing here synchronises the stream unless stated.
 *
 * Float arithmetic is fp32 (the reference's default precision). The neighbor filter
 * reproduces the reference's fp32 operation order bit for bit, so neighbor sets are
 * identical to the reference's on the same inputs.
 */
#ifndef SPH103_H
#define SPH103_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* sph_stream_t; /* a cudaStream_t */

enum sph_status {
    SPH_OK = 0,
    SPH_ERR_ARGUMENT = 1,       /* invalid size, pointer or parameter */
    SPH_ERR_WORKSPACE = 2,      /* workspace smaller than the queried size */
    SPH_ERR_CAPACITY = 3,       /* a neighbor row exceeded the list capacity */
    SPH_ERR_CUDA = 4,           /* a CUDA launch or copy failed */
    SPH_ERR_VERLET = 5,         /* particles moved farther than the list skin allows */
    SPH_ERR_NONFINITE = 6,      /* a NaN / Inf appeared in the state */
    SPH_ERR_STATIC_LIMIT = 7    /* the problem needs more scratch than the fixed static
                                   array of sph_neighbor_count_static holds */
};

/* Error flag bits accumulated on the device (sph_solver_flags). */
#define SPH_FLAG_CAPACITY 1u
#define SPH_FLAG_VERLET 2u
#define SPH_FLAG_NONFINITE 4u

typedef struct sph_domain {
    double min[2];   /* config['domain']['minExtent'] */
    double max[2];   /* config['domain']['maxExtent'] */
    int32_t periodic[2];
} sph_domain_t;

/* Scheme constants; names follow the reference's config keys. */
typedef struct sph_params {
    sph_domain_t domain;
    double support;          /* particle.support  (H, uniform) */
    double dx;               /* particle.dx */
    double mass;             /* uniform particle mass (fluid and boundary) */
    double rho0;             /* fluid.rho0 */
    double cs;               /* fluid.cs */
    double gamma;            /* EOS.polytropicExponent (stiff Tait) */
    double kernel_scale;     /* kernel.kernelScale */
    double delta;            /* diffusion.delta (density diffusion, deltaSPH scheme) */
    int32_t visc_scheme;     /* 0 deltaSPH_viscid, 1 deltaSPH_inviscid (diffusion.velocityScheme) */
    double nu, alpha, eps;   /* diffusion.nu / alpha / eps */
    int32_t bvisc_scheme;    /* boundaryDiffusion.velocityScheme (0 viscid, 1 inviscid) */
    double b_nu, b_alpha, b_eps;
    int32_t gravity_on;      /* gravity.active (constant mode) */
    double gravity[2];       /* direction * magnitude */
    double dt;               /* timestep.dt */
    int32_t shift_on;        /* shifting active (delta+ scheme, one iteration) */
    double shift_R, shift_n, shift_CFL, shift_threshold;
    int32_t compute_mach;    /* shifting.computeMach */
    int32_t density_update;  /* 0: the reference's observable update (half-step density),
                                1: rational symplectic update rho (2-eps)/(2+eps) */
    double skin;             /* cell margin factor (>= 1): the displacement since the last sort
                                that the cells still cover is (skin - 1) h, less the shift clamp */
    int32_t capacity;        /* candidate slots per particle */
    int32_t density_scheme;  /* simulation.densityScheme: 0 'continuity' (the density is
                                integrated), 1 'summation' (deltaPlus.py:193-198: every
                                right-hand side first sets the fluid densities to
                                sum_j m_j W_ij over fluid and wall neighbors; needs
                                density_update 0) */
} sph_params_t;

/* ------------------------------------------------------------------------------------
 * Neighbor search (drop-in for neighborSearch, src/diffSPH/v2/modules/neighborhood.py:491-593,
 * whose candidate stage is the external torchCompactRadius package and whose exact filter is
 * computeNeighborhood, neighborhood.py:433-460). Scatter mode: pairs with |x_i - x_j| <= h_j.
 * Rows ordered by query index, columns by reference index (original indices).
 * ------------------------------------------------------------------------------------ */

/* Workspace bytes for sph_neighbor_count / sph_neighbor_fill. */
int sph_neighbor_workspace_bytes(int64_t n_query, int64_t n_ref, const sph_domain_t* domain,
                                 double max_support, size_t* bytes);

/* Pass 1: sorts the reference particles into cells (inside the workspace) and writes the
 * exact per-query counts to counts[n_query] and the CSR row offsets to offsets[n_query+1]
 * (offsets[n_query] = total pairs). The caller reads offsets[n_query] to size the outputs. */
int sph_neighbor_count(const float* x_query, int64_t n_query, const float* x_ref,
                       const float* h_ref, int64_t n_ref, const sph_domain_t* domain,
                       double max_support, void* workspace, size_t workspace_bytes,
                       int32_t* counts, int64_t* offsets, sph_stream_t stream);

/* Pass 2 (same workspace, after pass 1): per pair i, j (int64), q = r/h_j, unit x_ij (2),
 * h_j, and when kernels / gradients != NULL the Wendland C2 kernel W and gradient grad W (2).
 * n_pairs = offsets[n_query] as read back by the caller. */
int sph_neighbor_fill(const float* x_query, int64_t n_query, const float* x_ref,
                      const float* h_ref, int64_t n_ref, const sph_domain_t* domain,
                      double max_support, void* workspace, size_t workspace_bytes,
                      const int64_t* offsets, int64_t n_pairs, int64_t* pair_i, int64_t* pair_j,
                      float* q, float* xhat, float* h_pair, float* kernels, float* gradients,
                      sph_stream_t stream);

/* Pass 2, indices only (same workspace, after pass 1): the original reference index of each
 * exact neighbor as int32, rows in the search's cell order rather than sorted by index.
 * For callers that need the neighbor lists but not the pair fields (the learned step);
 * no counterpart in the reference. */
int sph_neighbor_fill_csr(const float* x_query, int64_t n_query, const float* x_ref,
                          const float* h_ref, int64_t n_ref, const sph_domain_t* domain,
                          double max_support, void* workspace, size_t workspace_bytes,
                          const int64_t* offsets, int32_t* neighbors, sph_stream_t stream);

/* Pass 1 without caller workspace; no counterpart in the reference (its neighborSearch
 * allocates through torch). Same inputs, outputs and results as sph_neighbor_count, but the
 * scratch is a file-scope device array of SPH_NEIGHBOR_STATIC_SCRATCH_BYTES per device, so
 * the call allocates nothing. Returns SPH_ERR_STATIC_LIMIT, before any device work, when
 * sph_neighbor_workspace_bytes for the same sizes exceeds that limit (about 400k particles
 * in a square domain). The first call on a device, with that device current, looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before any stream
 * capture. The address is cached per device and CUDA context: after a cudaDeviceReset the
 * next call (again outside any capture) looks it up in the new context. The per-cell counters that must start at zero are cleared on every call. All
 * calls on one device share the one array: calls that overlap on the GPU (other streams, or
 * another thread before the previous call's work has finished) race on it. Pass 2
 * (sph_neighbor_fill) needs the caller workspace of sph_neighbor_count, not this call. */
#define SPH_NEIGHBOR_STATIC_SCRATCH_BYTES ((size_t)24 << 20)
int sph_neighbor_count_static(const float* x_query, int64_t n_query, const float* x_ref,
                              const float* h_ref, int64_t n_ref, const sph_domain_t* domain,
                              double max_support, int32_t* counts, int64_t* offsets,
                              sph_stream_t stream);

/* ------------------------------------------------------------------------------------
 * Fused solver: one time step of the reference runner (src/diffSPH/v2/runner.py:37-42):
 * integrate(simulationStep) with scheme symplecticEuler (integration.py:357-392), whose two
 * right-hand sides are simulationStep (deltaPlus.py:176-422) with mDBC walls (mDBC.py:9-163),
 * followed by solveShifting (shifting.py:882-1019, delta+ branch).
 * Fluid particles come first in the original order (0..n_fluid-1), boundary particles after.
 * ------------------------------------------------------------------------------------ */
typedef struct sph_solver sph_solver_t;

int sph_solver_workspace_bytes(const sph_params_t* params, int64_t n_fluid, int64_t n_boundary,
                               size_t* bytes);

/* Packed batch of independent fluid-only domains (no walls): domain d has its own
 * parameters (params[d]: extent, dx, support, dt, ...) and n_fluid[d] particles; the
 * state arrays of sph_solver_upload / _download are the domains' arrays concatenated in
 * domain order. Every kernel launch covers all domains (a per-particle domain id selects
 * the constants and the cell grid); results equal those of one solver per domain. */
int sph_batch_workspace_bytes(const sph_params_t* params, const int64_t* n_fluid, int32_t n_domains,
                              size_t* bytes);
int sph_batch_create(const sph_params_t* params, const int64_t* n_fluid, int32_t n_domains,
                     void* workspace, size_t workspace_bytes, sph_solver_t** out);

/* Creates a host-side handle over the caller's workspace (no device allocation). */
int sph_solver_create(const sph_params_t* params, int64_t n_fluid, int64_t n_boundary,
                      void* workspace, size_t workspace_bytes, sph_solver_t** out);
void sph_solver_destroy(sph_solver_t* solver);

/* Loads the state (original order; float2 arrays as [n][2]). Boundary arrays may be NULL
 * when n_boundary == 0. normals point into the wall, distances are negative depths.
 * Under Verlet reuse (sph_solver_set_verlet_reuse) an upload after the first keeps the
 * particles' current order (one domain; a packed batch is loaded in the original order): each particle's state is written into the slot it occupies, so
 * the next step sorts again only if a particle is farther than the reuse limit from its
 * position at the last sort (a state read back by sph_solver_download and uploaded again
 * costs no sort). Otherwise the particles are loaded in the original order and the next
 * step sorts. The arrays may be device memory or page-locked host memory (mapped into the
 * device's address space, as sph_solver_download): the kernel reads host arrays itself
 * over the host link, in the original order. */
int sph_solver_upload(sph_solver_t* s, const float* x_fluid, const float* u_fluid,
                      const float* rho_fluid, const float* x_boundary, const float* normal_boundary,
                      const float* dist_boundary, const float* rho_boundary, sph_stream_t stream);

/* Advances n_steps full time steps (integrate + shifting, fused). */
int sph_solver_step(sph_solver_t* s, int32_t n_steps, sph_stream_t stream);

/* Same as sph_solver_step, replayed from a CUDA graph captured on first use. The solver
 * keeps two graphs, keyed by n_steps and by which internal buffers hold the current state
 * (eager steps, integrate and shift rotate them); other calls capture again. n_steps must
 * be even, or at least 1 under Verlet reuse (whose sorts copy back and never rotate the
 * buffers), and stream must not be the legacy default stream. */
int sph_solver_graph_step(sph_solver_t* s, int32_t n_steps, sph_stream_t stream);

/* The two halves of a step as the reference runner calls them: integrate (both
 * right-hand sides and the symplectic Euler update; integration.py:92-513) ... */
int sph_solver_integrate(sph_solver_t* s, sph_stream_t stream);

/* ... and solveShifting (shifting.py:882-1019): rebuilds the lists at the current
 * positions, applies the delta+ shift and writes the fluid increments dx[nF][2] in the
 * original order when dx != NULL. */
int sph_solver_shift(sph_solver_t* s, float* dx, sph_stream_t stream);

/* Evaluates one right-hand side at the current state (simulationStep, deltaPlus.py:176-422)
 * and writes, in the original order, dudt[nF][2], drhodt[nF], and optionally (NULL to
 * skip) gradRho^L[nF][2], L[nF][4], pressures[nF], boundary densities[nB], and the number
 * of fluid and of boundary neighbors (self included) of every fluid particle nn[nF][2]. */
int sph_solver_rhs(sph_solver_t* s, float* dudt, float* drhodt, float* grad_rho, float* L,
                   float* pressure, float* rho_boundary, int32_t* num_neighbors, sph_stream_t stream);

/* sph_solver_rhs with the wall densities rho_boundary_in[nB] (original order) given by the
 * caller in place of the mDBC extrapolation: the rest of simulationStep (deltaPlus.py:240-422)
 * after its mDBCDensity call (deltaPlus.py:200-202), e.g. for a caller that keeps the
 * reference's own wall model. The walls' pressures are the EOS of the given densities.
 * Outputs as sph_solver_rhs. */
int sph_solver_rhs_walls(sph_solver_t* s, const float* rho_boundary_in, float* dudt, float* drhodt,
                         float* grad_rho, float* L, float* pressure, int32_t* num_neighbors,
                         sph_stream_t stream);

/* ------------------------------------------------------------------------------------
 * Adjoint (vector-Jacobian products) of the step's operators at the current state, for a
 * single domain (periodic or walled with mDBC), either viscosity scheme (deltaSPH_viscid
 * or _inviscid, with the boundary viscosity), gravity, the continuity density and the
 * delta+ shift without the free-surface handling. No reference entry point has these: the
 * reference differentiates its torch operators with autograd (simulationStep,
 * deltaPlus.py:176-422, per step). Every VJP walks the exact neighbor lists in gather form
 * (each particle collects its own pair terms and its neighbors' terms through the
 * symmetric neighbor relation), so no atomics are used except in sph_solver_vjp_walls.
 * Inputs and outputs are in the original particle order; gradients ACCUMULATE (+=) into
 * xbar[nF][2], ubar[nF][2], rbar[nF], gbar[nF][2] and, with walls, into the adjoint of
 * the wall densities rhob_bar[nB] (their pressures' adjoint folded in through the EOS;
 * required when the solver has walls, ignored otherwise). Positions are differentiated
 * through the periodic wrap as the identity. Other configurations (summation density,
 * implicit shifting, free-surface handling, packed batches) return SPH_ERR_ARGUMENT.
 * ------------------------------------------------------------------------------------ */

/* Right-hand side (pass B: continuity, delta-diffusion, pressure with the Tait EOS,
 * viscosity, boundary viscosity): given the adjoints abar[nF][2] of dudt and drbar[nF] of
 * drhodt (NULL = 0), accumulates the adjoints of positions, velocities, densities, of
 * gradRho^L (gbar, NULL to drop) and of the wall densities the mDBC extrapolation gives at
 * this state, and writes per particle nu_part[nF] (NULL to skip) whose sum is the adjoint
 * of diffusion.nu (0 for the inviscid scheme). gradRho^L is an input here; its own
 * dependence on the state is sph_solver_vjp_gradient. */
int sph_solver_vjp_rates(sph_solver_t* s, const float* abar, const float* drbar, float* xbar,
                         float* ubar, float* rbar, float* gbar, float* nu_part, float* rhob_bar,
                         sph_stream_t stream);

/* Renormalised density gradient (pass A: M, L = pinv(M), gradRho^L = m (L g_fluid +
 * g_walls)): given gbar[nF][2], accumulates the adjoints of positions, densities and the
 * wall densities (mDBC at this state). */
int sph_solver_vjp_gradient(sph_solver_t* s, const float* gbar, float* xbar, float* rbar,
                            float* rhob_bar, sph_stream_t stream);

/* delta+ shift x'' = x' + clamp(dx(x', rho', Ma)): given xbar_new[nF][2] (the adjoint of
 * x''), accumulates xbar (identity part included), rbar and the adjoint of the wall
 * densities as uploaded (the fused step shifts with the second stage's mDBC densities), and
 * writes mach_part[nF] whose sum is the adjoint of Ma = max|u| / cs (0 when
 * shifting.computeMach is off). Clamped components carry no gradient. */
int sph_solver_vjp_shift(sph_solver_t* s, const float* xbar_new, float* xbar, float* rbar,
                         float* mach_part, float* rhob_bar, sph_stream_t stream);

/* mDBC wall densities (mDBC.py:50-163; the fp64 moment solve of sph_solver_rhs): given
 * the adjoint rhob_bar[nB] of the wall densities extrapolated from the current fluid state,
 * accumulates the adjoints of the fluid positions and densities. The derivatives are summed
 * per fluid particle in fp64 with atomics and rounded to fp32 once. No-op without walls. */
int sph_solver_vjp_walls(sph_solver_t* s, const float* rhob_bar, float* xbar, float* rbar,
                         sph_stream_t stream);

/* ------------------------------------------------------------------------------------
 * Implicit particle shifting (shifting.scheme = 'IPS'): computeShifting,
 * src/diffSPH/v2/modules/shifting.py:780-880, as solveShifting (:882-1019) calls it, with
 * the system of getShiftingMatrices (:611-705; no free-surface handling, shifting.
 * summationDensity off so omega = the particle area dx^2, initialization 'zero') solved by
 * bicgstab_shifting (:322-493). Once set, it replaces the delta+ shift of sph_solver_step,
 * sph_solver_graph_step and sph_solver_shift (single-domain solvers only). Outside a graph
 * capture a solve synchronises the stream every 4 iterations to stop once it has returned;
 * a captured step holds all max_iter iterations (those after the return do nothing).
 * ------------------------------------------------------------------------------------ */
typedef struct sph_ips_params {
    double rtol;              /* shifting.rtol (reference default 1e-4) */
    int32_t max_iter;         /* shifting.maxSolveIter (64) */
    double solver_threshold;  /* shifting.solverThreshold as parsed: dx / 2 when negative
                                 (parameters.py:238); the solve returns once any |x_i| exceeds it */
} sph_ips_params_t;

/* Bytes of the IPS workspace: 7 float2 vectors and the stored 2x2 blocks of up to 64 exact
 * neighbors (12 B each) per particle, and the reduction scratch. */
int sph_solver_ips_workspace_bytes(const sph_solver_t* s, size_t* bytes);
/* Switches the solver to IPS (params != NULL; workspace 256-byte aligned, at least
 * sph_solver_ips_workspace_bytes) or back to delta+ (params == NULL). Drops captured graphs. */
int sph_solver_set_ips(sph_solver_t* s, const sph_ips_params_t* params, void* workspace,
                       size_t workspace_bytes);
/* Iteration count and bicgstab_shifting's second return value (the count when |r|
 * converged, 0 when |s| converged, -10 / -11 breakdowns, -12 threshold, max_iter when the
 * loop ran out) of the last solve. Synchronises the stream. */
int sph_solver_ips_result(sph_solver_t* s, int32_t* iterations, int32_t* code, sph_stream_t stream);

/* ------------------------------------------------------------------------------------
 * Free-surface handling of the shift (shifting.freeSurface = True): solveShifting
 * (src/diffSPH/v2/modules/shifting.py:882-1019) with surface detection 'Barcasco'
 * (detectFreeSurfaceBarecasco, surfaceDetection.py:95-107), the mask expansion
 * (expandFreeSurfaceMask, :54-63), normals 'lambda' (computeNormalsMaronne :41-52 and
 * computeLambdaGrad, shifting.py:151-171) and projection 'mat' (shifting.py:972-982), on the
 * merged fluid and wall particles. Applies to the delta+ and the IPS shift (whose system
 * then drops the surface rows, getShiftingMatrices :657-678). Single-domain solvers only.
 * ------------------------------------------------------------------------------------ */
typedef struct sph_free_surface_params {
    double barecasco_threshold;    /* surfaceDetection.BarecascoThreshold (pi / 3) */
    int32_t expansion_iterations;  /* surfaceDetection.expansionIterations (2) */
    double surface_scaling;        /* shifting.surfaceScaling (0.1) */
} sph_free_surface_params_t;

/* Bytes of the free-surface workspace (about 160 B per particle, walls included). */
int sph_solver_free_surface_workspace_bytes(const sph_solver_t* s, size_t* bytes);
/* Switches the handling on (params != NULL; workspace 256-byte aligned) or off (NULL).
 * Drops captured graphs. */
int sph_solver_set_free_surface(sph_solver_t* s, const sph_free_surface_params_t* params,
                                void* workspace, size_t workspace_bytes);
/* The fields of the last shift's detection, in the original order of the merged set (fluid
 * particles, then walls; NULL entries are skipped): surface flags fs[n] and expanded mask
 * fsm[n] (uint8), Lambdas[n], normals[n][2] (computed on the rows of the expanded mask, the
 * only ones the projection uses; zero elsewhere). */
int sph_solver_free_surface_fields(sph_solver_t* s, uint8_t* fs, uint8_t* fsm, float* lambdas,
                                   float* normals, sph_stream_t stream);

/* computePressureAccelSwitch (src/diffSPH/v2/modules/pressureForce.py:15-33), Antuono's
 * switch: a_i = -sum_j m_j / (rho_i rho_j) p_ij gradW_ij with p_ij = p_j + p_i where p_i >= 0
 * or surface_mask_i > 0.5, else p_j - p_i. Works on a neighborhood in the reference's format
 * (neighborSearch, or sph_neighbor_fill): pairs sorted by query index, offsets[n_query] and
 * counts[n_query] (neighborOffsets, numNeighbors), reference indices pair_j and gradients
 * [pairs][2]. surface_mask may be NULL (no particle on the surface). Writes accel[n][2]. */
int sph_pressure_switch(int64_t n_query, const int32_t* offsets, const int32_t* counts,
                        const int64_t* pair_j, const float* gradients, const float* p_query,
                        const float* rho_query, const float* surface_mask, const float* p_ref,
                        const float* rho_ref, const float* m_ref, float* accel, sph_stream_t stream);

/* LiuLiuConsistent (src/diffSPH/v2/sphOps.py:313-341), the first-order consistent
 * interpolation the open-boundary (mirror outlet) ghosts use (deltaPlus.py:210-235): per
 * query row of a neighborhood in the reference's format (offsets, counts, pair_j, and the pair
 * distances q = r/h, unit vectors [pairs][2], supports, kernels, gradients [pairs][2]), the
 * moments b[3] and M[3][3] of the fluid quantity (m_ref / rho_ref volumes) and the solution
 * [value, d/dx, d/dy] by Cramer's rule. M and b may be NULL. */
int sph_liuliu_consistent(int64_t n_query, const int32_t* offsets, const int32_t* counts,
                          const int64_t* pair_j, const float* distances, const float* vectors,
                          const float* supports, const float* kernels, const float* gradients,
                          const float* m_ref, const float* rho_ref, const float* quantity,
                          float* solution, float* M, float* b, sph_stream_t stream);

/* ------------------------------------------------------------------------------------
 * Pair-sum operators on a neighborhood in the reference's format (what neighborSearch,
 * src/diffSPH/v2/modules/neighborhood.py:491-593, or sph_neighbor_fill returns), for callers
 * that keep the reference's own simulationStep. Each query row i sums its pairs
 * [offsets[i], offsets[i] + counts[i]) in their stored order, with the reference's fp32
 * operation order per pair, as its scatter_sum (src/diffSPH/v2/math.py:77-93) adds them on
 * the CPU. Per-pair arrays: pair_j (int64), distances (q = r / h_j), vectors (unit x_ij,
 * [P][2]), supports (h_j), kernels (W), gradients (grad W, [P][2]); an operator that does
 * not read one of them accepts NULL there. "a" arrays are per query particle, "b" arrays
 * per reference particle; vectors are [n][2], 2x2 matrices [n][4] row-major.
 * ------------------------------------------------------------------------------------ */
typedef struct sph_pairs {
    int64_t n_query;
    const int32_t* offsets;   /* neighborOffsets [n_query] */
    const int32_t* counts;    /* numNeighbors [n_query] */
    const int64_t* pair_j;    /* indices[1] [P] */
    const float* distances;
    const float* vectors;
    const float* supports;
    const float* kernels;
    const float* gradients;
} sph_pairs_t;

/* sphOperation / sphOperationStates (src/diffSPH/v2/sphOps.py:243-303) */
enum sph_operation_kind {
    SPH_OP_DENSITY = 0,       /* sphDensityInterpolation (:20-29): sum m_j W */
    SPH_OP_INTERPOLATE = 1,   /* sphInterpolation (:6-18): sum (m_j / rho_j) W q */
    SPH_OP_GRADIENT = 2,      /* sphGradient (:32-60): sum q (x) (m_j / rho_j) grad W */
    SPH_OP_DIVERGENCE = 3,    /* sphDivergence (:63-98): sum q . (m_j / rho_j) grad W */
    SPH_OP_CURL = 4,          /* sphCurl (:139-171), 2D */
    SPH_OP_LAPLACIAN = 5      /* sphLaplacian (:174-240), every type but 'naive' */
};
/* gradientMode (and the laplacian's type): the pair quantity q_j (naive), q_i - q_j
 * (gradient 'difference'; q_j - q_i for divergence and curl), q_i + q_j (summation), or the
 * symmetric form rho_i sum m_j (q_i / rho_i^2 + q_j / rho_j^2) grad W; the laplacian types
 * 'conserving', 'divergenceFree', 'dot' and its default formula (any other value) */
enum sph_operation_mode {
    SPH_MODE_NAIVE = 0,
    SPH_MODE_DIFFERENCE = 1,
    SPH_MODE_SUMMATION = 2,
    SPH_MODE_SYMMETRIC = 3,
    SPH_MODE_CONSERVING = 4,
    SPH_MODE_DIVERGENCE_FREE = 5,
    SPH_MODE_DOT = 6
};

/* One sphOperation over quantities with `components` values per particle (1 scalar, 2
 * vector, 4 2x2 matrix): per particle as the tuple (q_a, q_b), or per pair (q_pair != NULL,
 * the reference's non-tuple argument, used as is in every mode). divergence_mode 0 is 'div'
 * (the last index contracted), 1 'dot' (the first). Output per query row: 1 value (density,
 * curl, divergence of a vector), components (interpolate, laplacian), 2 components
 * (gradient: q_c grad W_d at [c][d]), 2 (divergence of a matrix). */
int sph_operation(const sph_pairs_t* nb, int32_t operation, int32_t mode, int32_t divergence_mode,
                  int32_t components, const float* m_b, const float* rho_a, const float* rho_b,
                  const float* q_a, const float* q_b, const float* q_pair, float* out,
                  sph_stream_t stream);

/* computeCovarianceMatrices (src/diffSPH/v2/modules/normalizationMatrices.py:18-23):
 * out[n][4] = sum (-(q h) xhat) (x) (m_j / rho_j) grad W. */
int sph_covariance(const sph_pairs_t* nb, const float* m_b, const float* rho_b, float* out,
                   sph_stream_t stream);

/* renormalizedDensityGradient (src/diffSPH/v2/modules/densityDiffusion.py:7-26) with L[n][4]
 * (the normalised kernel gradient L_i grad W), or densityGradient (:28-46) with L == NULL:
 * out[n][2] = sum (rho_i - rho_j) (m_j / rho_j) grad W. */
int sph_density_gradient(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                         const float* L, float* out, sph_stream_t stream);

/* computeDensityDeltaTerm (densityDiffusion.py:49-73), scheme 'deltaSPH': out[n] =
 * delta h_i / kappa cs sum psi_ij . (m_j / rho_j) grad W with psi_ij = -2 (rho_j - rho_i) /
 * (r_ij + 1e-6 h) xhat + (gradRho^L_i + gradRho^L_j); h_a are the query supports. */
int sph_delta_term(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                   const float* grad_a, const float* grad_b, const float* h_a, double delta, double kappa,
                   double cs, float* out, sph_stream_t stream);

/* computeMomentumEquation (src/diffSPH/v2/modules/momentumEquation.py:6-39): out[n] =
 * -sum ((u_j - u_i) m_j) . grad W rho_i / rho_j. */
int sph_momentum(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                 const float* u_a, const float* u_b, float* out, sph_stream_t stream);

/* computePressureAccel (src/diffSPH/v2/modules/pressureForce.py:10-12): out[n][2] =
 * -(sum (p_i + p_j) (m_j / rho_j) grad W) / rho_i. */
int sph_pressure_accel(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                       const float* p_a, const float* p_b, float* out, sph_stream_t stream);

/* computeViscosity (src/diffSPH/v2/modules/viscosity.py:222-241) for the deltaSPH schemes
 * (:123-170 inviscid, :200-218 viscid) and computeViscosity_Boundary
 * (boundaryViscosity.py:123-173, 199-219; wall_volume = 1 gives the inviscid wall scheme's
 * m_j / (rho_i + rho_j)). The values are the config section's (diffusion or
 * boundaryDiffusion). h_a (query supports) is read by the inviscid scheme. */
typedef struct sph_viscosity_params {
    int32_t scheme;        /* 0 deltaSPH_viscid, 1 deltaSPH_inviscid */
    int32_t wall_volume;   /* inviscid wall scheme: V_j = m_j / (rho_i + rho_j) */
    int32_t pi_switch;     /* pi-switch: only approaching pairs ((u_i - u_j).xhat < 0) */
    double nu, alpha, eps;
    double cs, rho0;       /* fluid.cs, fluid.rho0 */
} sph_viscosity_params_t;
int sph_viscosity(const sph_pairs_t* nb, const float* m_b, const float* rho_a, const float* rho_b,
                  const float* u_a, const float* u_b, const float* h_a, const sph_viscosity_params_t* params,
                  float* out, sph_stream_t stream);

/* mDBCDensity (src/diffSPH/v2/modules/mDBC.py:50-163) on the ghost -> fluid neighborhood
 * (query = the wall particles' ghosts, x_ghost[n][2]; reference = the fluid): the Shepard
 * density, the 3x3 moment system solved where a ghost has more than five neighbors and the
 * first-order extrapolation to the wall particle x_wall[n][2]; the rest density rho0 where a
 * ghost has none. The sums follow the reference's order; the pseudo-inverse is fp64 with
 * torch.linalg.pinv's truncation rule (the reference's fp32 solve carries ~1e-4 relative
 * rounding on the ill-conditioned matrices near free edges). support is particle.support.
 * Writes rho_out[n] and, when non-NULL, shepard_out[n]. */
int sph_mdbc_density(const sph_pairs_t* nb, const float* m_f, const float* rho_f, const float* x_wall,
                     const float* x_ghost, double support, double rho0, float* rho_out, float* shepard_out,
                     sph_stream_t stream);

/* Writes the current state back in the original order (NULL entries are skipped). The arrays
 * may be device memory or page-locked host memory (cudaHostAlloc / cudaHostRegister; mapped
 * into the device's address space): the kernel then writes the host arrays itself over the
 * host link, one pass in the original order, with no staging copy. Host arrays are complete
 * once the stream has reached this call. */
int sph_solver_download(sph_solver_t* s, float* x_fluid, float* u_fluid, float* rho_fluid,
                        float* rho_boundary, sph_stream_t stream);

/* Copies the device error flags (SPH_FLAG_*) to *flags_host; synchronises the stream. */
int sph_solver_flags(sph_solver_t* s, uint32_t* flags_host, sph_stream_t stream);

/* Verlet reuse of the neighbor structure across steps, as the reference's neighborSearch
 * does with neighborhood.verletScale > 1 (src/diffSPH/v2/modules/neighborhood.py:505-518,
 * the default scale 1.5 at :603): a step sorts the particles by cell again, and rebuilds the
 * skin list of candidates within 1.1 h, only when a particle moved farther than 0.034 h
 * since the last sort (or the list went invalid); otherwise it keeps that order and filters
 * the kept list. Walled, periodic and packed batches of domains (each domain's particles
 * against its own limit; any domain past it sorts the batch); off after sph_solver_create.
 * The decision is taken on the device, so captured step graphs replay both cases. Results
 * differ from the sort-every-step ones only in the order of each particle's pair sums. */
int sph_solver_set_verlet_reuse(sph_solver_t* s, int32_t on);
/* The reference's rebuild rule for that reuse (neighborhood.py:509-513): a rebuild once
 * 2 max |x - x_sort| > (verletScale - 1) h. The solver sorts at the stricter of
 * (verletScale - 1) h / 2 and its own 0.034 h (the skin list's limit with a margin);
 * verlet_scale must exceed 1. With the default verletScale 1.5 the solver's limit applies.
 * In a batch each domain's limit follows from its own h. */
int sph_solver_set_verlet_scale(sph_solver_t* s, double verlet_scale);
/* Number of cell sorts since the last upload (device counter); synchronises the stream. */
int sph_solver_sort_count(sph_solver_t* s, uint32_t* sorts, sph_stream_t stream);

/* Launch shapes of the neighbor passes: warps per block, width of the per-warp neighbor
 * list and grid. Shapes 0-3 launch one block per tile of 32 x warps slots (0: 4 warps with
 * 32-bit entries; 1, 2, 3: 4, 8, 16 warps with 16-bit entries); shape 4 is shape 2 under a
 * persistent grid (as many blocks as the SMs hold at once, each looping over the tiles, for
 * a packed batch over the tiles of every domain). Each of the sph_solver_tuned_passes() passes has its own shape, in this
 * order: 0 pass A scanning the cell stencil (and keeping the skin list), 1 pass A filtering
 * the skin list, 2 pass B, 3 the delta+ shift, 4 the summation density. No shape changes a
 * result: every shape evaluates the same pairs in the same order.
 *
 * Autotuner: times every pass under every shape on the current state (after a cell sort
 * at the current positions; the state itself is left unchanged) and keeps the fastest per
 * pass. Writes the chosen shapes to shapes_out[sph_solver_tuned_passes()] and the time of
 * each pass and shape (ms; -1 when the shape or the pass does not apply) to
 * ms_out[pass * sph_solver_shapes() + shape] when non-NULL. Synchronises the stream. */
int sph_solver_autotune(sph_solver_t* s, int32_t* shapes_out, float* ms_out, sph_stream_t stream);
int sph_solver_shapes(void);
int sph_solver_tuned_passes(void);
/* Forces a launch shape (0 <= shape < sph_solver_shapes()) on every pass, or on one
 * (0 <= pass < sph_solver_tuned_passes(); -1: all); rejects shapes whose 16-bit list
 * entries cannot address the grid's stencils. */
int sph_solver_set_shape(sph_solver_t* s, int32_t shape);
int sph_solver_set_pass_shape(sph_solver_t* s, int32_t pass, int32_t shape);
/* The shape of each pass, shapes_out[sph_solver_tuned_passes()]. */
int sph_solver_pass_shapes(const sph_solver_t* s, int32_t* shapes_out);

/* Number of kernel launches one sph_solver_step(s, 1, ...) issues (with the delta+ shift;
 * an implicit shift replaces its one launch by 2 + 5 per iteration of its solve). */
int sph_solver_launches_per_step(const sph_solver_t* s);

/* Kernel timing: when enabled, sph_solver_step brackets every launch with CUDA events on
 * its stream and accumulates per-kernel-class device time. Classes are listed by
 * sph_solver_kernel_name (index < sph_solver_kernel_classes()). */
int sph_solver_kernel_classes(void);
const char* sph_solver_kernel_name(int cls);
int sph_solver_set_timing(sph_solver_t* s, int32_t enabled);
/* Synchronises the stream, writes per-class total ms and launch counts, and resets them. */
int sph_solver_kernel_times(sph_solver_t* s, float* ms_host, int32_t* launches_host,
                            sph_stream_t stream);

/* ------------------------------------------------------------------------------------
 * Learned continuous-convolution step (no reference implementation: the network is a
 * stand-in for 4 solver steps). One layer is E = aggregate(h) followed by the basis-weight
 * contraction y = E W on the tensor cores.
 * ------------------------------------------------------------------------------------ */

/* D[M x N] (fp32, row-major, leading dimension ldd) = A[M x K] * Bt[N x K]^T, or += when
 * accumulate != 0. A and Bt are row-major bf16 (leading dimensions lda, ldb in elements).
 * tcgen05 MMA (BF16 inputs, FP32 accumulation in tensor memory) fed by TMA. Requires
 * M % 128 == 0, N % 64 == 0, K % 64 == 0, 16-byte aligned pointers, lda, ldb multiples of
 * 8 and ldd a multiple of 4. A wait that does not complete sets a bit in *err (device
 * word, caller-cleared) instead of hanging. */
int sph_gemm_bf16_tn(const void* A, const void* Bt, float* D, int64_t M, int64_t N, int64_t K,
                     int64_t lda, int64_t ldb, int64_t ldd, int32_t accumulate, uint32_t* err,
                     sph_stream_t stream);

/* The poll limit of sph_gemm_bf16_tn's mbarrier waits (default 2^22 polls, about a
 * second): a wait that runs out sets a bit of *err (1: a free stage, 2: a loaded stage,
 * 4: the MMAs' completion, 32: loads still in flight at the end) and the CTA stops issuing
 * work, waits (bounded) for the loads it issued and releases its tensor memory. 0 makes every
 * wait fail at once, so that no load or MMA is issued: the error path can be exercised without
 * a stuck wait. Applies to launches after the call (process-wide); *previous (when non-NULL)
 * gets the old limit. */
int sph_set_gemm_wait_limit(uint32_t polls, uint32_t* previous);

/* E_i[b C + c] = inv_norm * sum_j phi_b(x_i - x_j) h_j[c] over the CSR neighbor rows
 * (offsets[n+1] int64, neighbors int32, e.g. the exact lists of sph_neighbor_fill), with
 * the 64 basis functions phi_{8a+m} = (1-q^2)^2 T_a(2q-1) F_m(angle), q = |x| / support.
 * relative != 0 aggregates h_j[c] - h_i[c] instead (the difference form of SPH operators).
 * h: bf16 [n][C], E: bf16 [n][64 C], C in {16, 32, 64}. */
int sph_cconv_aggregate(const float* x, int64_t n, const int64_t* offsets, const int32_t* neighbors,
                        const sph_domain_t* domain, double support, double inv_norm, const void* h,
                        int32_t channels, int32_t relative, void* E, sph_stream_t stream);

/* sph_cconv_aggregate on the tensor cores: per particle E_i = Phi_i^T G_i as a tcgen05 MMA
 * (BF16 basis values and features, FP32 accumulation in tensor memory), up to 128
 * neighbors per row. Same layout and arguments; *err (device word, caller-cleared) gets
 * bit 8 when a row had more than 128 neighbors (the rest are dropped) and bit 16 when a
 * wait did not complete. */
int sph_cconv_aggregate_tc(const float* x, int64_t n, const int64_t* offsets, const int32_t* neighbors,
                           const sph_domain_t* domain, double support, double inv_norm, const void* h,
                           int32_t channels, int32_t relative, void* E, uint32_t* err, sph_stream_t stream);

/* Transpose of sph_cconv_aggregate (for the backward pass, symmetric neighbor relation):
 * dh_j[c] = inv_norm * sum_{i in N(j)} sum_b phi_b(x_i - x_j) dE_i[b C + c]; dE fp32 rows of
 * leading dimension ldE, dh fp32 [n][C]. */
int sph_cconv_aggregate_t(const float* x, int64_t n, const int64_t* offsets, const int32_t* neighbors,
                          const sph_domain_t* domain, double support, double inv_norm, const float* dE,
                          int64_t ldE, int32_t channels, int32_t relative, float* dh, sph_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SPH103_H */
