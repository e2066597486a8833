/*
 * fdadi.h -- C ABI of libfdadi.so, the GB300 (sm_103a) FP64 ADI pricer.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*; NULL = legacy default stream) and returns 0 on success or
 * a nonzero FDADI_E* code; fdadi_last_error() gives the message of the last
 * failure on the calling thread. Nothing here allocates device memory:
 * scratch is passed in by the caller (workspace pointers sized by the
 * *_workspace_bytes queries). All arithmetic is IEEE binary64.
 *
 * Grid layout: a 2-D state V[n0][n1] is row-major (n1 contiguous), the
 * reference domain layout V[iS, iv] (FiniteDifference/Grid.py:35-40). A 1-D
 * state uses n1 = 1.
 *
 * Operator layout: an operator along `axis` acts on `blocks` independent
 * lines of `block_len = operator_rows / blocks` points. Its diagonals are
 * row-aligned (sup[r] = A[r, r+1], mid[r] = A[r, r], sub[r] = A[r, r-1]) and
 * indexed in the reference's flattened block-major order r = b * block_len + k
 * (the order after the operator axis is rolled last,
 * FiniteDifference/BandedOperator.pyx:335-337; the GPU reference keeps the same
 * "cublas" layout, FiniteDifference/BandedOperatorGPU.pyx:651-676). For axis 0
 * line b is grid column j = b and element k is row i; for axis 1 line b is
 * grid row i = b and element k is column j.
 */
#ifndef FDADI_H
#define FDADI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDADI_OK 0
#define FDADI_E_ARG 1        /* bad argument: sizes, pointers, shapes ("Dimension mismatch") */
#define FDADI_E_CUDA 2       /* a CUDA runtime call failed */
#define FDADI_E_WORKSPACE 3  /* workspace too small */
#define FDADI_E_STATE 4      /* operation not valid in the operator's fold state */

/* fold status codes: the reference's "CANNOT_FOLD", "CAN_FOLD", "FOLDED"
 * strings (FiniteDifference/BandedOperator.pyx:15-17) */
#define FDADI_CANNOT_FOLD 0
#define FDADI_CAN_FOLD 1
#define FDADI_FOLDED 2

#define FDADI_SCHEME_IMPLICIT 0
#define FDADI_SCHEME_DOUGLAS 1
#define FDADI_SCHEME_HV 2
#define FDADI_SCHEME_CS 3     /* Craig-Sneyd, FiniteDifferenceEngine.pyx:843-898 */
#define FDADI_SCHEME_MCS 4    /* modified Craig-Sneyd, FiniteDifferenceEngine.pyx:779-841 */

/* library version (major*10000 + minor*100 + patch) */
int fdadi_version(void);

/* Copies the message of the last failed call on this thread into buf
 * (NUL-terminated, truncated to len); returns its length. Replaces the
 * reference's DIE()/std::domain_error text (FiniteDifference/common.h:17-27). */
int fdadi_last_error(char *buf, size_t len);

/* ------------------------------------------------------------------------ */
/* Host-side meshes (no device work).                                       */
/* ------------------------------------------------------------------------ */

/* utils.exponential_space (FiniteDifference/utils.py:161-190) on the host:
 * out[i] = l + (i*dv)**ex on [low, ~high], the upper end stretched so that
 * `exact` lands on a point when force_exact is nonzero. Same operations and
 * order as the reference's Python floats (C pow(), no contraction), so the
 * mesh is bit-identical. FDADI_E_ARG with the reference's message "Did not
 * find suitable value." when no point lies below `exact`. */
int fdadi_exponential_space(double low, double exact, double high, double ex, int32_t size,
                            int32_t force_exact, double *out);

/* The variance meshes of n Heston engines, as HestonFiniteDifferenceEngine
 * builds them (FiniteDifference/heston.py:384-389: exponential_space(0, v0[k],
 * var_max, varexp, nv[k])), concatenated in option order into out
 * (sum(nv) doubles), spread over `threads` host threads (0: all cores). */
int fdadi_heston_var_meshes(int32_t n, const double *v0, const int32_t *nv, double var_max,
                            double varexp, int32_t force_exact, int32_t threads, double *out);

/* ------------------------------------------------------------------------ */
/* Tridiagonal operator: replaces the C++ class _TriBandedOperator          */
/* (FiniteDifference/_TriBandedOperatorGPU.cuh:21-85) behind                */
/* BandedOperatorGPU.BandedOperator (FiniteDifference/BandedOperatorGPU.pxd).*/
/* ------------------------------------------------------------------------ */
typedef struct fdadi_tri {
    int64_t operator_rows;        /* N = blocks * block_len */
    int64_t blocks;
    int32_t axis;                 /* 0 or 1 */
    int32_t has_residual;         /* enable_residual() state */
    int32_t has_low_dirichlet;
    int32_t has_high_dirichlet;
    int32_t top_fold_status;      /* FDADI_CANNOT_FOLD / CAN_FOLD / FOLDED */
    int32_t bottom_fold_status;
    double *sup, *mid, *sub;      /* [N] row-aligned diagonals */
    double *R;                    /* [N] residual */
    double *low_dirichlet;        /* [blocks] values forced on row 0 of each line */
    double *high_dirichlet;       /* [blocks] values forced on the last row */
    double *top_factors;          /* [blocks] CAN_FOLD: A[0,2]; FOLDED: fold factor */
    double *bottom_factors;       /* [blocks] CAN_FOLD: A[L-1,L-3]; FOLDED: fold factor */
    double *sup2, *sub2;          /* [N] A[r, r+2] and A[r, r-2] inside the lines, or NULL:
                                   * the rows a spliced upwind scheme gives a second
                                   * off-diagonal (splice_with, BandedOperator.pyx:527-591).
                                   * The corner entries A[0,2], A[L-1,L-3] stay in the fold
                                   * slots (sup2[row 0], sub2[row L-1] unused). Not allowed on
                                   * a FOLDED operator: diagonalize drops them, as the
                                   * reference's does (BandedOperator.pyx:181-198). */
} fdadi_tri_t;

/* y = A x (+ R if has_residual), x with its Dirichlet entries forced first;
 * a folded operator is unfolded after the product. y may alias x.
 * Replaces _TriBandedOperator::apply (_TriBandedOperatorGPU.cu:463-553). */
int fdadi_tri_apply(const fdadi_tri_t *op, const double *x, double *y,
                    int64_t n0, int64_t n1, void *stream);

/* x <- A^-1 (x_forced - R): Dirichlet entries forced, residual subtracted if
 * enabled, right-hand side folded, then one Thomas solve per line. A CAN_FOLD
 * operator is folded on the fly (same linear system). With sup2/sub2 the line
 * is solved as a band of width 2 + 2 by LU without row exchanges (the system
 * scipy's solve_banded solves in the reference CPU engine, BandedOperator.pyx:
 * 364-394). scratch: [N] doubles, [3N] with sup2/sub2.
 * Replaces _TriBandedOperator::solve (_TriBandedOperatorGPU.cu:719-770). */
int fdadi_tri_solve(const fdadi_tri_t *op, double *x, int64_t n0, int64_t n1,
                    double *scratch, void *stream);

/* Same solve as fdadi_tri_solve for callers that cannot allocate device
 * memory (a host that owns all device memory in its own pool, or a latency-
 * critical loop that must not let cudaMalloc/cudaFree synchronize the
 * device). No counterpart in the reference. The scratch is the library's own
 * static device array of FDADI_NOALLOC_MAX_ROWS doubles (8 MiB), held by
 * every device that loads the library until the process exits; operators with
 * more rows are rejected (FDADI_E_ARG). Every call looks up the array's
 * device address on the current device (cudaGetSymbolAddress), so the call
 * stays valid after cudaDeviceReset; the first call on a device also loads the
 * library's module there, so make it before any stream capture. All calls
 * share the array, so calls
 * whose kernels overlap on the GPU race: order them. */
#define FDADI_NOALLOC_MAX_ROWS (1 << 20)
int fdadi_tri_solve_noalloc(const fdadi_tri_t *op, double *x, int64_t n0, int64_t n1,
                            void *stream);

/* Row r of every diagonal, R and the fold extras scaled by vec[r]; Dirichlet
 * rows are left alone. Replaces vectorized_scale
 * (_TriBandedOperatorGPU.cu:1012-1105). If vec is NULL, `scalar` is used for
 * every row (mul_scalar_from_host, BandedOperatorGPU.pyx:488-501). */
int fdadi_tri_scale(fdadi_tri_t *op, const double *vec, double scalar, void *stream);

/* mid[r] += value on all rows but Dirichlet rows (residual untouched).
 * Replaces add_scalar_from_host / add_scalar (_TriBandedOperatorGPU.cu:674-711). */
int fdadi_tri_add_scalar(fdadi_tri_t *op, double value, void *stream);

/* self += other (same axis, rows, blocks; neither folded): off-diagonals and
 * R everywhere, main diagonal skipping self's Dirichlet rows, CAN_FOLD
 * extras added. Replaces add_operator (_TriBandedOperatorGPU.cu:577-671). */
int fdadi_tri_add_operator(fdadi_tri_t *self, const fdadi_tri_t *other, void *stream);

/* Fold (unfold = 0) or unfold (unfold = 1) the top and/or bottom rows of
 * every line: one Gaussian-elimination step that removes A[0,2] / A[L-1,L-3].
 * Updates the status fields of *op. Replaces diagonalize/undiagonalize and
 * fold_top/fold_bottom (_TriBandedOperatorGPU.cu:836-1009). */
int fdadi_tri_fold(fdadi_tri_t *op, int32_t top, int32_t bottom, int32_t unfold, void *stream);

/* ------------------------------------------------------------------------ */
/* Mixed d2/dx0dx1 operator: replaces _CSRBandedOperator                    */
/* (FiniteDifference/_CSRBandedOperatorGPU.cuh:15-82) and its cuSPARSE csrmv.*/
/* The reference's 9-point CSR stencil (_CSRBandedOperatorGPU.cu:505-774) is */
/* the product of two centred first-derivative stencils times a per-point   */
/* coefficient; it is stored here in that factored form.                   */
/* ------------------------------------------------------------------------ */
typedef struct fdadi_mixed {
    int64_t n0, n1;
    int32_t has_residual;
    int32_t reserved;
    double *coeff;   /* [n0*n1] per-point coefficient (grid order) */
    double *w0;      /* [3][n0]: A_0[i,i-1], A_0[i,i], A_0[i,i+1] (rows 0, n0-1 zero) */
    double *w1;      /* [3][n1]: same along axis 1 */
    double *R;       /* [n0*n1] */
} fdadi_mixed_t;

/* y = coeff .* (D0 (x) D1) x (+ R). y must not alias x. */
int fdadi_mixed_apply(const fdadi_mixed_t *op, const double *x, double *y, void *stream);

/* coeff[p] *= vec[p] (or *= scalar if vec is NULL); R scaled too. */
int fdadi_mixed_scale(fdadi_mixed_t *op, const double *vec, double scalar, void *stream);

/* y = a*y + b*x over n doubles: the SizedArray pluseq/minuseq/minuseq_over2/
 * timeseq used by the reference GPU loops (FiniteDifference/VecArray.cu:32-116). */
int fdadi_axpby(double *y, const double *x, double a, double b, int64_t n, void *stream);

/* ------------------------------------------------------------------------ */
/* Fused batched Heston engine: replaces the per-step call chains of        */
/* FiniteDifferenceEngineGPU.solve_{implicit,douglas,hundsdorferverwer,     */
/* smooth}_ (FiniteDifference/FiniteDifferenceEngineGPU.pyx:379-593) with    */
/* operators built on the device as HestonFiniteDifferenceEngine builds     */
/* them (FiniteDifferenceEngineGPU.pyx:596-724, heston.py:302-359).         */
/* ------------------------------------------------------------------------ */
/* Launch plan of the batched engine's line solves (chosen by
 * fdadi_heston_tune, or by a size heuristic when a batch has none). */
typedef struct fdadi_heston_plan {
    int32_t spot_kind;   /* 0: one thread per spot line; 1: partitioned lines */
    int32_t spot_a;      /* kind 0: rows prefetched ahead (1, 2, 4 or 8); kind 1: lines per block */
    int32_t spot_b;      /* kind 0: threads per block; kind 1: segments per line */
    int32_t var_kind;    /* 0: one shared tile per warp; 1: two tiles, copies pipelined,
                          * factors by shuffle; 2: one tile, factors by shuffle;
                          * 3: partitioned lines (one 32-row task per block, its warps
                          * splitting the columns) */
    int32_t var_warps;   /* warps per variance-solve block (kind 3: 4, 8 or 16 segments) */
    int32_t groups;      /* option groups whose explicit stages and solves overlap
                          * (1..4; 0 counts as 1) */
    int32_t expl_per_sm; /* explicit stage: 0 = one block per tile; n = n blocks per SM
                          * looping over tiles (leaves room for another group's solves) */
    int32_t reserved[1];
} fdadi_heston_plan_t;

typedef struct fdadi_heston_batch {
    int32_t n_options;
    int32_t scheme;          /* FDADI_SCHEME_DOUGLAS, _HV, _CS or _MCS (main segment) */
    int32_t n_steps;         /* main-segment steps */
    int32_t implicit_steps;  /* fully implicit steps run before the main segment */
    double theta;            /* main-segment theta */
    double implicit_dt_factor; /* implicit step = dt * factor (0.5: Rannacher half-steps) */
    int32_t flags;           /* FDADI_HESTON_* bits */
    int32_t reserved;
    const int32_t *n0;       /* HOST [n_options] spot points */
    const int32_t *n1;       /* HOST [n_options] variance points */
    const double *spots;     /* DEVICE [sum n0] spot meshes, packed */
    const double *vars;      /* DEVICE [sum n1] variance meshes, packed */
    const double *params;    /* DEVICE [n_options][5]: r, kappa, theta, sigma, rho */
    const double *dt;        /* DEVICE [n_options] main-segment step */
    const int32_t *barrier;  /* DEVICE [n_options] nonzero: up-and-out (Dirichlet 0 at S_max), or NULL */
    const fdadi_heston_plan_t *plan; /* HOST launch plan of the line solves, or NULL (heuristic) */
    const double *rates;     /* DEVICE [n_options][implicit_steps + n_steps] interest rate of
                              * every step (time-dependent coefficients), or NULL: params' r.
                              * Step k (the implicit steps first) uses rates[o][k] wherever r
                              * enters the operators (the drift r S, the -r/2 split, the S_max
                              * residual); the operators and line-solve factors are rebuilt
                              * before every step, as preprocess_operators is documented to be
                              * run per step for time-dependent parameters
                              * (FiniteDifferenceEngineGPU.pyx:163-167). */
} fdadi_heston_batch_t;

/* drop the mixed operator of options with rho == 0, as the GPU reference
 * does (FiniteDifferenceEngineGPU.pyx:118-126, 720-724) */
#define FDADI_HESTON_DROP_ZERO_MIXED 1
/* capture the time loop in a CUDA graph and launch that */
#define FDADI_HESTON_GRAPH 2

/* Bytes of device workspace fdadi_heston_prepare/run need for this batch
 * (operator plans, line tables and stage buffers). */
int64_t fdadi_heston_workspace_bytes(const fdadi_heston_batch_t *batch);

/* Build every option's operators and line-solve factors into the workspace.
 * Meshes/params must be on the device. */
int fdadi_heston_prepare(const fdadi_heston_batch_t *batch, void *workspace,
                         int64_t workspace_bytes, void *stream);

/* Run the schedule (implicit_steps fully implicit steps of dt*implicit_dt_factor,
 * then n_steps of the scheme; solve_smooth's Rannacher start is
 * implicit_steps = 2*s with factor 0.5, FiniteDifferenceEngine.pyx:1010-1016) on
 * the packed state V (DEVICE [sum n0*n1], option k at offset sum_{m<k} n0*n1),
 * in place. Requires a prepared workspace. */
int fdadi_heston_run(const fdadi_heston_batch_t *batch, void *workspace,
                     int64_t workspace_bytes, double *V, void *stream);

/* out[k] = V[flat_index[k]] for k < n (DEVICE arrays): price read-out. */
int fdadi_gather(const double *V, const int64_t *flat_index, double *out, int64_t n,
                 void *stream);

/* Number of kernel launches fdadi_heston_run issues for this batch (each
 * stage is launched once per option group of the plan). */
int64_t fdadi_heston_launch_count(const fdadi_heston_batch_t *batch);

/* Launch one stage kernel of the time loop (for per-kernel timing; a run is
 * the sequence these make up). stage: FDADI_STAGE_*. */
#define FDADI_STAGE_EXPLICIT_DOUGLAS 0
#define FDADI_STAGE_EXPLICIT_HV0 1
#define FDADI_STAGE_EXPLICIT_HV3 2
#define FDADI_STAGE_EXPLICIT_IMPLICIT 3
#define FDADI_STAGE_SPOT_SOLVE 4        /* W -> W - T (main plan) */
#define FDADI_STAGE_VAR_SOLVE_TO_Y2 5   /* W -> Y2 (main plan) */
#define FDADI_STAGE_VAR_SOLVE_TO_V 6    /* W -> V (main plan) */
#define FDADI_STAGE_VAR_SOLVE_IMPLICIT 7 /* W -> W (implicit plan) */
#define FDADI_STAGE_SPOT_SOLVE_IMPLICIT 8 /* W -> V (implicit plan) */
int fdadi_heston_stage(const fdadi_heston_batch_t *batch, void *workspace,
                       int64_t workspace_bytes, double *V, int32_t stage, void *stream);

/* Autotuner: time every launch shape of the spot and variance line solves on
 * this prepared batch (reps launches each, in place on the stage buffer W),
 * then the number of option groups and the explicit stage's blocks per SM
 * (two time steps per choice on a scratch state), and write the fastest plan
 * to *plan. The state is untouched; the
 * stage buffers hold garbage afterwards, which every step overwrites.
 * Allocates the scratch state for the call and synchronises the stream. Pass
 * the plan back in batch->plan for fdadi_heston_run. */
int fdadi_heston_tune(const fdadi_heston_batch_t *batch, void *workspace,
                      int64_t workspace_bytes, int32_t reps, fdadi_heston_plan_t *plan,
                      void *stream);

/* Initial state of every option on its mesh, built on the device (the
 * reference initializes the grid on the host, heston.py:402): V = max(S - K, 0)
 * for calls (put == 0) or max(K - S, 0) for puts, with strikes DEVICE
 * double [n_options] and V the packed arena. Requires a prepared workspace. */
int fdadi_heston_payoff(const fdadi_heston_batch_t *batch, void *workspace,
                        int64_t workspace_bytes, const double *strikes, int32_t put, double *V,
                        void *stream);

/* Per-option status words (the reference raises from DIE() on a failed solve,
 * common.h:17-27; a batch reports per option instead). */
#define FDADI_STATUS_PIVOT 1      /* a line-solve pivot of the option was zero or non-finite */
#define FDADI_STATUS_NONFINITE 2  /* the option's state grid holds a NaN or infinity */
/* status[k] (DEVICE, int32 [n_options]) = the FDADI_STATUS_* bits of option k:
 * pivot flags recorded by fdadi_heston_prepare, plus a scan of the state V
 * (DEVICE, the packed arena) for non-finite values. */
int fdadi_heston_status(const fdadi_heston_batch_t *batch, void *workspace,
                        int64_t workspace_bytes, const double *V, int32_t *status, void *stream);

/* Price, delta and gamma of every option at its grid point flat_index[k]
 * (DEVICE int64 [n_options], an index into the packed arena inside option k's
 * grid): V there and the centred non-uniform first and second derivatives in
 * S along the spot line (the reference's centercoeffs stencils,
 * BandedOperator.pyx:970-1017). Greeks are NaN on the first and last spot rows.
 * Outputs are DEVICE double [n_options]. */
int fdadi_heston_greeks(const fdadi_heston_batch_t *batch, void *workspace,
                        int64_t workspace_bytes, const double *V, const int64_t *flat_index,
                        double *price, double *delta, double *gamma, void *stream);

/* The plan fdadi_heston_run uses for this batch when batch->plan is NULL. */
int fdadi_heston_default_plan(const fdadi_heston_batch_t *batch, fdadi_heston_plan_t *plan);

/* ------------------------------------------------------------------------ */
/* Fused batched Black-Scholes engine: the 1-D counterpart of the Heston    */
/* batch. Replaces FiniteDifferenceEngineGPU's solve_* loops on the engine  */
/* from_host_FiniteDifferenceEngine makes of a BlackScholesFiniteDifference */
/* Engine (FiniteDifferenceEngineGPU.pyx:100-128, blackscholes.py:144-239): */
/* A = r S D_S + 1/2 sigma^2 S^2 D_SS - r with U = 0 at the first mesh point */
/* and dU/dS = 1 at S_max. Lines are independent, so one launch runs every  */
/* option's whole schedule.                                                 */
/* ------------------------------------------------------------------------ */
typedef struct fdadi_bs_batch {
    int32_t n_options;
    int32_t scheme;          /* FDADI_SCHEME_DOUGLAS, _HV, _CS or _MCS (main segment) */
    int32_t n_steps;         /* main-segment steps (0: implicit steps only) */
    int32_t implicit_steps;  /* fully implicit steps run before the main segment */
    double theta;            /* main-segment theta */
    double implicit_dt_factor; /* implicit step = dt * factor (0.5: Rannacher half-steps) */
    const int32_t *n;        /* HOST [n_options] spot points (>= 4) */
    const double *spots;     /* DEVICE [sum n] spot meshes, packed */
    const double *params;    /* DEVICE [n_options][2]: r, variance sigma^2 */
    const double *dt;        /* DEVICE [n_options] main-segment step */
    int32_t prefetch;        /* rows each thread keeps in flight in its forward sweeps
                              * (2, 4 or 8; four times as many in the back
                              * substitutions), copied asynchronously into shared
                              * memory; 0: chosen by batch size. Results are identical. */
    int32_t reserved;
} fdadi_bs_batch_t;

/* Bytes of device workspace fdadi_bs_prepare/run need for this batch. */
int64_t fdadi_bs_workspace_bytes(const fdadi_bs_batch_t *batch);

/* Build every option's operators (F = dt A, Le = theta dt A) and the Thomas
 * factors of 1 - theta dt A and of the implicit 1 - dt' A into the workspace. */
int fdadi_bs_prepare(const fdadi_bs_batch_t *batch, void *workspace, int64_t workspace_bytes,
                     void *stream);

/* Run the schedule (implicit_steps fully implicit steps of dt*implicit_dt_factor,
 * then n_steps of the scheme) on the packed state V (DEVICE [sum n], option k
 * at offset sum_{m<k} n_m), in place: one kernel launch. */
int fdadi_bs_run(const fdadi_bs_batch_t *batch, void *workspace, int64_t workspace_bytes,
                 double *V, void *stream);

/* Initial state: V = max(S - K, 0) (put == 0) or max(K - S, 0), strikes DEVICE
 * double [n_options], V the packed state. */
int fdadi_bs_payoff(const fdadi_bs_batch_t *batch, void *workspace, int64_t workspace_bytes,
                    const double *strikes, int32_t put, double *V, void *stream);

/* status[k] (DEVICE int32 [n_options]): FDADI_STATUS_PIVOT if a pivot of
 * option k's line solves was zero or non-finite at prepare, FDADI_STATUS_NONFINITE
 * if its state in V holds a NaN or infinity. */
int fdadi_bs_status(const fdadi_bs_batch_t *batch, void *workspace, int64_t workspace_bytes,
                    const double *V, int32_t *status, void *stream);

/* FP64 throughput probe: every thread runs `chains` (1, 2, 4, 8 or 16)
 * independent DFMA chains for `iters` iterations; writes one value per thread
 * to out (>= blocks*threads doubles) and returns the number of floating-point
 * operations it issues (2 per DFMA) in *flops. Used by the benchmark to
 * measure the FP64 roofline on the device. No reference counterpart. */
int fdadi_fp64_probe(double *out, int32_t blocks, int32_t threads, int32_t iters,
                     int32_t chains, double *flops, void *stream);

/* ------------------------------------------------------------------------ */
/* Pricing surrogate: BF16 tensor-core MLP kernels (no reference            */
/* counterpart; the reference prices every option with ADI).                */
/* ------------------------------------------------------------------------ */

/* C[M,N] = A[M,K] * B[N,K]^T on 5th-generation tensor cores (tcgen05.mma,
 * accumulator in tensor memory), FP32 accumulation, for `problems`
 * independent problems (operand p at base + p * stride). A and B are bf16 with
 * K contiguous; M % 128 == 0, N in 16..256 step 16, K % 16 == 0, leading
 * dimensions multiples of 8 elements, 16-byte aligned bases. Epilogue per
 * element: x = acc (+ bias[n]); out_f32 = x; act 1: x = SiLU(x), act 2:
 * x *= SiLU'(aux[m][n]); out_bf16 = bf16(x). *status is set to 1 if a
 * tensor-core completion wait timed out (the kernel then returns without
 * writing). */
typedef struct fdadi_gemm {
    const void *A; int64_t lda, strideA;
    const void *B; int64_t ldb, strideB;
    const float *bias; int64_t strideBias;
    const float *aux; int64_t ldaux, strideAux;
    float *out_f32; int64_t ldo, strideO;
    void *out_bf16; int64_t ldh, strideH;
    int32_t M, N, K, act, problems;
    int32_t variant;   /* 0: persistent warp-specialised kernel (TMA producer warp, MMA warp,
                        * epilogue warps, two tensor-memory accumulators; K split with fp32
                        * atomic adds when there are few output tiles and no epilogue);
                        * 1: one CTA per tile, two cp.async stages */
    int32_t *status;
    int64_t wait_cycles;  /* variant 0: clock cycles after which a wait on a copy,
                           * an MMA or an epilogue gives up (0: about 2 s). The
                           * kernel then drains the copies and MMAs it issued,
                           * frees its tensor memory, sets *status and returns.
                           * Negative: a test of that path; the MMA warp first
                           * waits -wait_cycles cycles on a barrier that nothing
                           * completes, so the launch always aborts. */
} fdadi_gemm_t;
int fdadi_mlp_gemm(const fdadi_gemm_t *gemm, void *stream);

/* The surrogate network for fused inference: per layer l, weights W[l] (bf16
 * [members][N[l]][K[l]], K contiguous) and bias b[l] (fp32 [members][N[l]]).
 * Supported shape: K = 16, 256, 256, 256, 256; N = 256 for the hidden layers,
 * 16..256 for the last (its first two outputs are produced). */
typedef struct fdadi_mlp_net {
    const void *W[5];
    const float *b[5];
    int32_t K[5], N[5];
    int32_t members;
    int32_t reserved;
} fdadi_mlp_net_t;

/* Ensemble inference with every hidden activation kept on chip: one
 * persistent kernel runs all five layers (tcgen05 MMAs into tensor memory,
 * bias + SiLU epilogue writing the next layer's bf16 operand in shared memory,
 * weights streamed by TMA). X: bf16 [M][16] shared by the members, M a
 * multiple of 128; out: fp32 [members][M][2] (the last layer's first two
 * outputs, bias included). status: set to 1 if a bounded wait timed out. */
int fdadi_mlp_infer(const fdadi_mlp_net_t *net, const void *X, int32_t M, float *out,
                    int32_t *status, void *stream);

/* out[c][r] = in[r][c] (bf16), per problem. */
int fdadi_transpose_bf16(const void *in, int64_t ldi, int64_t stride_in, void *out, int64_t ldo,
                         int64_t stride_out, int32_t rows, int32_t cols, int32_t problems,
                         void *stream);

/* Weighted mean squared error of pred[:, :nout] (fp32) against target
 * [M][nout]; writes the bf16 gradient into grad[M][ncols] (zero beyond nout)
 * and adds the loss of problem p to loss[p]. */
int fdadi_mlp_mse(const float *pred, int64_t ldp, int64_t stride_p, const float *target,
                  const float *weights, int32_t nout, void *grad, int64_t ldg, int64_t stride_g,
                  int32_t M, int32_t ncols, int32_t problems, double *loss, void *stream);

/* db[n] = sum_m dy[m][n] (bf16 dy, fp32 db), per problem. */
int fdadi_mlp_colsum(const void *dy, int64_t ld, int64_t stride, float *db, int64_t stride_db,
                     int32_t M, int32_t N, int32_t problems, void *stream);

/* One Adam step on FP32 master parameters p (n values; a rows x cols matrix
 * when w/wt are given) with gradient g and moments m1, m2; refreshes the bf16
 * copies w (same layout) and wt (transposed) when non-NULL. */
int fdadi_mlp_adam(float *p, const float *g, float *m1, float *m2, int64_t n, int32_t rows,
                   int32_t cols, float lr, float b1, float b2, float eps, int32_t step, void *w,
                   void *wt, void *stream);

/* Surrogate front end: queries [M][9] = (S0, K, T, r, kappa, theta, sigma,
 * rho, v0) -> bf16 network inputs X [M][16] (features S0/K, T, r, kappa,
 * theta, sigma, rho, v0 mapped to [-1, 1] by the box lo/hi [8], then derived
 * inputs), the control variate base [M][4] = (price/K, delta, price-residual
 * scale, delta-residual scale), and inbox [M]. cv = 0: Black-Scholes at the
 * expected mean variance, scales 1. cv = 1 or 2: that price plus the first-
 * or second-order expansion in the volatility of variance, price scale
 * sigma sqrt(T) + 0.1 (the delta keeps the Black-Scholes variate). */
int fdadi_mlp_featurize(const double *queries, int32_t M, const double *lo, const double *hi,
                        int32_t cv, void *X, double *base, int32_t *inbox, void *stream);

/* Ensemble read-out: y [problems][M][ldy] scaled residual outputs ->
 * price = K (base0 + base2 mean y0 / s0), delta = base1 + base3 mean y1 / s1, spread =
 * max - min of the members' prices, fallback = out of box or spread > tol*K;
 * *count += number of fallbacks. */
int fdadi_mlp_combine(const float *y, int64_t ldy, int64_t stride, int32_t problems, int32_t M,
                      const double *queries, const double *base, const int32_t *inbox, double s0,
                      double s1, double tol, double *price, double *delta, double *spread,
                      int32_t *fallback, int32_t *count, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FDADI_H */
