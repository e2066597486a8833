// Fused, batched Heston ADI engine.
//
// A batch of options with independent (uneven) grids lives in one packed
// arena: option k owns points [p_off[k], p_off[k] + n0*n1) of every per-point
// array (row-major, variance contiguous), rows [s_off[k], s_off[k] + n0) of
// every per-spot-index array and columns [v_off[k], v_off[k] + n1) of every
// per-variance-index array. Each time step is a short chain of launches over
// the whole batch:
//
//   explicit stage  -- 16x32-point tiles staged in shared memory with a halo:
//                      the spot, variance and mixed applies of F(V) fused
//                      with the scheme's combination; the mixed stencil's
//                      row sums are formed once per tile row and shared;
//   spot solve      -- one thread per grid column walking the strided
//                      direction; adjacent threads read adjacent columns, so
//                      every access is coalesced without a transpose;
//   variance solve  -- one warp per 32 grid rows: 32x32 chunks pass through
//                      a padded shared tile so global loads and stores are
//                      coalesced while each lane runs its row's recurrence.
//
// GB300 executes FP64 at ~1 TFLOP/s against ~6.8 TB/s of HBM, so the kernels
// are built to minimise FP64 instructions first: Thomas factors are
// precomputed once per (dt, theta) (the operators are time independent,
// FiniteDifferenceEngineGPU.pyx:163-167), each solve costs two FMAs and a
// multiply per point, the HV corrector reuses F(V) from the predictor, and the
// mixed stencil is factored. The variance operator of the Heston PDE is the
// same on every spot row with S > 0 (its coefficients kappa(theta - v) and
// sigma^2 v / 2 do not depend on S, heston.py:309-322), so its coefficients
// and Thomas factors are stored once per option as 1-D arrays.
//
// Operators are built on the device with the reference's arithmetic order
// (explicitly rounded intrinsics, no FMA contraction), so they equal the
// reference CPU engine's bit for bit.
#include <algorithm>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "fdadi_internal.cuh"
#include "fdadi_rows.cuh"

namespace fdadi {

enum : int { OPT_S_LOW_DIR = 1, OPT_S_HIGH_DIR = 2, OPT_MIXED = 4, OPT_ROW0_ZERO = 8 };

constexpr int TI = 16;                // explicit tile rows
constexpr int TJ = 32;                // explicit tile columns
constexpr int EXPL_THREADS = TI * TJ;
constexpr int XR = TI + 2;            // staged rows (one-row halo above and below)
constexpr int XC = TJ + 3;            // staged columns (two on the left, one on the right)
constexpr int XCP = 36;               // padded row pitch of the staged tile
constexpr int SPOT_MAX_THREADS = 256; // largest block of the line-per-thread spot solve
constexpr int VS_PITCH = 33;          // padded pitch of the 32x32 variance tile

// Half-open index range of tiles, spot lines or variance tasks: a stage
// kernel works on one option group's range.
struct Span {
    int64_t lo, hi;
};

// Device view of a prepared workspace.
struct Arena {
    int n_opt;
    int64_t P, SS, SV;         // total points, total spot indices, total variance indices
    // tables
    const int *n0, *n1, *oflags;
    const int64_t *p_off, *s_off, *v_off;
    const int *lineS;          // option of each spot line (grid column)
    const int4 *tiles;         // explicit tiles: (option, i0, j0, -)
    const int4 *vtasks;        // variance-solve tasks: (option, i0, rows, -)
    // main plan (dt, theta)
    double *F0;                // [3P] spot operator rows (sub, mid, sup) * dt; Dirichlet rows identity
    double *w0;                // [3 SS] spot first-derivative weights * rho sigma S_i dt
    double *w1;                // [3 SV] variance first-derivative weights * v_j
    double *LS;                // [3P] Thomas factors (a, 1/m, c') of 1 - theta dt A0
    double *R0top;             // [SV] spot residual on the S_max row * dt
    double *F1v;               // [3 SV] variance operator rows on S > 0 * dt
    double *F1x;               // [n_opt] its A[n1-1, n1-3] * dt
    double *F1z;               // [n_opt] variance operator on S = 0 (diagonal) * dt
    double *LVv;               // [3 SV] factors of 1 - theta dt A1 on S > 0, bottom folded
    double *foldV;             // [n_opt] bottom fold factor of that operator
    double *LVz;               // [n_opt] 1/diagonal of 1 - theta dt A1 on S = 0
    double *dirS;              // [2 SV] Dirichlet values of the spot lines (low, high)
    // implicit plan (dt * factor, theta = 1, residual kept)
    double *w0i, *RSi, *LSi, *LVvi, *foldVi, *LVzi;
    // HV corrector: (1/2 - theta) * F0 [3P] and w0 / 2 [3 SS]
    double *F0h, *w0h;
    // HV corrector: the variance operator times theta dt rounded as the
    // reference's Les are, (A1 * theta) * dt ([3 SV] rows on S > 0, its
    // A[n1-1, n1-3], the S = 0 diagonal), and a per-option 1 (the corrector's
    // spot solve subtracts that product as it stands)
    double *LE1v, *LE1x, *LE1z, *one;
    double *F1h;               // [3 SV] F1v / 2 (exact): the corrector's 1/2 F1 Y2 in its chain
    double *sw;                // [6 SS] spot stencil weights for the builders
    // stage buffers
    double *FV, *W, *T, *Y2;
    const double *theta;       // [n_opt]
    int *ostat;                // [n_opt] FDADI_STATUS_* bits found while building
};

// Combined variance operator A1 = kappa(theta - v) D_v + 1/2 sigma^2 v D_vv - r/2
// at element j of the variance line through S_i (coefficients zero at S = 0,
// heston.py:309-322); boundaries heston.py:344-358: first derivative
// one-sided at both ends, second derivative Neumann 0 at v = 0 and
// second-order backward at v_max (the A[n-1, n-3] entry that is folded).
__device__ Row3 var_row(const double *v, int n, int j, double Si, double r, float half_r,
                        double kappa, double theta, double sigma) {
    Row3 o{0.0, 0.0, 0.0, 0.0, 0.0, false};
    const double f = (double)half_r;
    double c1 = 0.0, c11 = 0.0;
    if (Si != 0.0) {
        c1 = MUL(kappa, SUB(theta, v[j]));
        c11 = MUL(MUL(0.5, MUL(sigma, sigma)), v[j]);
    }
    if (j == 0) {
        const double d1 = SUB(v[1], v[0]);
        const double p1 = DIV(1.0, d1), m1 = DIV(-1.0, d1);
        o.sup = ADD(MUL(p1, c1), MUL(0.0, c11));
        o.mid = ADD(ADD(MUL(m1, c1), f), MUL(0.0, c11));
        o.sub = 0.0;
        return o;
    }
    if (j == n - 1) {
        const double dm1 = SUB(v[n - 1], v[n - 2]), dm2 = SUB(v[n - 2], v[n - 3]);
        const double m1 = DIV(1.0, dm1), s1 = DIV(-1.0, dm1);
        const double rd = DIV(1.0, MUL(MUL(MUL(0.5, ADD(dm2, dm1)), dm2), dm1));
        const double e2 = MUL(dm1, rd), s2 = MUL(-ADD(dm2, dm1), rd), m2 = MUL(dm2, rd);
        o.mid = ADD(ADD(MUL(m1, c1), f), MUL(m2, c11));
        o.sub = ADD(MUL(s1, c1), MUL(s2, c11));
        o.ext = ADD(0.0, MUL(e2, c11));
        o.sup = 0.0;
        return o;
    }
    double s1, m1, p1, s2, m2, p2;
    centre(v, j, 1, s1, m1, p1);
    centre(v, j, 2, s2, m2, p2);
    o.sup = ADD(MUL(p1, c1), MUL(p2, c11));
    o.mid = ADD(ADD(MUL(m1, c1), f), MUL(m2, c11));
    o.sub = ADD(MUL(s1, c1), MUL(s2, c11));
    return o;
}

struct BuildArgs {
    const double *spots, *vars, *params, *dt;
    const int *barrier;
    double theta;
    double dt_factor;  // implicit step = dt * dt_factor
    int smoothing;     // nonzero: build the implicit plan too
    int drop_zero_mixed;
    int hv;            // nonzero: build the HV corrector's scaled copies too
    const double *rates = nullptr;  // per-step r ([n_opt][rate_stride]) or null
    int64_t rate_stride = 0;
    int rate_step = 0;              // the step whose r the build uses
};

__device__ __forceinline__ void opt_params(const BuildArgs &a, int o, double &r, double &kappa,
                                           double &th, double &sigma, double &rho) {
    const double *p = a.params + 5 * (int64_t)o;
    r = a.rates ? a.rates[(int64_t)o * a.rate_stride + a.rate_step] : p[0];
    kappa = p[1]; th = p[2]; sigma = p[3]; rho = p[4];
}

// Per option: flags, the 1-D variance operator on S > 0 and S = 0 and the
// Thomas factors of 1 - theta dt A1 (bottom folded, BandedOperator.pyx:223-256)
// for the main and implicit plans.
__device__ void var_factors(const Arena &A, int o, const double *v, int n1, double r, float half_r,
                            double kappa, double th, double sigma, double scale, double *L,
                            double *fold, double *zinv) {
    const int64_t vo = A.v_off[o];
    const Row3 a2 = var_row(v, n1, n1 - 2, 1.0, r, half_r, kappa, th, sigma);
    const Row3 a1 = var_row(v, n1, n1 - 1, 1.0, r, half_r, kappa, th, sigma);
    const double an1 = MUL(a2.sub, scale), bn1 = ADD(MUL(a2.mid, scale), 1.0),
                 cn1 = MUL(a2.sup, scale);
    const double zn = MUL(a1.ext, scale);
    double an = MUL(a1.sub, scale), bn = ADD(MUL(a1.mid, scale), 1.0);
    const double f = an1 != 0.0 ? DIV(-zn, an1) : 0.0;
    an = ADD(an, MUL(bn1, f));
    bn = ADD(bn, MUL(cn1, f));
    fold[o] = f;
    Thomas t;
    for (int j = 0; j < n1 - 1; ++j) {
        const Row3 w = var_row(v, n1, j, 1.0, r, half_r, kappa, th, sigma);
        t.row(L, A.SV, vo + j, MUL(w.sub, scale), ADD(MUL(w.mid, scale), 1.0), MUL(w.sup, scale),
              j == 0);
    }
    t.row(L, A.SV, vo + n1 - 1, an, bn, 0.0, false);
    // S = 0: A1 is (-r/2) I (both variance coefficients vanish there)
    const Row3 z = var_row(v, n1, 0, 0.0, r, half_r, kappa, th, sigma);
    *zinv = 1.0 / ADD(MUL(z.mid, scale), 1.0);
    if (t.bad || !isfinite(*zinv) || !isfinite(f)) atomicOr(&A.ostat[o], FDADI_STATUS_PIVOT);
}

// One block per option: the spot-index weights of spot_row_w.
__global__ void build_spot_weights_kernel(Arena A, BuildArgs a) {
    const int o = blockIdx.x;
    const int n0 = A.n0[o];
    const int64_t so = A.s_off[o];
    const double *S = a.spots + so;
    for (int i = threadIdx.x; i < n0; i += blockDim.x) spot_weights(S, n0, i, A.sw + so + i, A.SS);
}

__global__ void build_options_kernel(Arena A, BuildArgs a) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= A.n_opt) return;
    const int n1 = A.n1[o];
    const double *S = a.spots + A.s_off[o], *v = a.vars + A.v_off[o];
    double r, kappa, th, sigma, rho;
    opt_params(a, o, r, kappa, th, sigma, rho);
    const float half_r = (float)(-r / 2.0);   // add_scalar takes a C float (BandedOperator.pxd:32)
    const double dt = a.dt[o];
    const bool barrier = a.barrier && a.barrier[o];
    int fl = OPT_S_LOW_DIR;
    if (barrier) fl |= OPT_S_HIGH_DIR;
    if (!(a.drop_zero_mixed && rho == 0.0)) fl |= OPT_MIXED;
    if (S[0] == 0.0) fl |= OPT_ROW0_ZERO;
    const_cast<int *>(A.oflags)[o] = fl;
    const Row3 xb = var_row(v, n1, n1 - 1, 1.0, r, half_r, kappa, th, sigma);
    A.F1x[o] = MUL(xb.ext, dt);
    const Row3 z = var_row(v, n1, 0, 0.0, r, half_r, kappa, th, sigma);
    A.F1z[o] = MUL(z.mid, dt);
    if (a.hv) {
        A.LE1x[o] = MUL(MUL(xb.ext, a.theta), dt);
        A.LE1z[o] = MUL(MUL(z.mid, a.theta), dt);
        A.one[o] = 1.0;
    }
    var_factors(A, o, v, n1, r, half_r, kappa, th, sigma, MUL(a.theta, -dt), A.LVv, A.foldV,
                &A.LVz[o]);
    if (a.smoothing)
        var_factors(A, o, v, n1, r, half_r, kappa, th, sigma, -MUL(dt, a.dt_factor), A.LVvi,
                    A.foldVi, &A.LVzi[o]);
}

// Per point: scaled spot operator rows (Firsts = A0 * dt, Dirichlet rows
// unscaled, BandedOperator.pyx:771-779) and mixed coefficients; per spot
// index: stencil weights; per variance index: stencil weights, the variance
// operator rows, the S_max residual and the Dirichlet values.
__global__ void build_points_kernel(Arena A, BuildArgs a) {
    const int4 t = A.tiles[blockIdx.x];
    const int o = t.x, n0 = A.n0[o], n1 = A.n1[o];
    const int i = t.y + threadIdx.x / TJ, j = t.z + threadIdx.x % TJ;
    if (i >= n0 || j >= n1) return;
    const int64_t p = A.p_off[o] + (int64_t)i * n1 + j, P = A.P;
    const double *S = a.spots + A.s_off[o], *v = a.vars + A.v_off[o];
    double r, kappa, th, sigma, rho;
    opt_params(a, o, r, kappa, th, sigma, rho);
    const float half_r = (float)(-r / 2.0);
    const bool barrier = a.barrier && a.barrier[o];
    const double dt = a.dt[o];
    const double dti = MUL(dt, a.dt_factor);

    const double *swo = A.sw + A.s_off[o];
    const Row3 s = spot_row_w(swo + i, A.SS, S, n0, i, v[j], r, half_r, barrier);
    double f0[3];
    if (s.dirichlet) {
        f0[0] = 0.0; f0[1] = 1.0; f0[2] = 0.0;
    } else {
        f0[0] = MUL(s.sub, dt); f0[1] = MUL(s.mid, dt); f0[2] = MUL(s.sup, dt);
    }
    A.F0[p] = f0[0]; A.F0[P + p] = f0[1]; A.F0[2 * P + p] = f0[2];
    if (a.hv) {
        const double h = SUB(0.5, a.theta);
        A.F0h[p] = MUL(f0[0], h); A.F0h[P + p] = MUL(f0[1], h); A.F0h[2 * P + p] = MUL(f0[2], h);
    }
    // mixed term rho sigma S_i v_j (D_S (x) D_v): the coefficient is
    // separable, so it is folded into the two stencils' weights
    if (j == 0) {
        double sb = 0.0, md = 0.0, sp = 0.0;
        if (i > 0 && i < n0 - 1) centre(S, i, 1, sb, md, sp);
        const int64_t q = A.s_off[o] + i;
        const double cs = MUL(MUL(rho, sigma), S[i]);
        const double cm = MUL(cs, dt);
        A.w0[q] = sb * cm; A.w0[A.SS + q] = md * cm; A.w0[2 * A.SS + q] = sp * cm;
        if (a.hv) {
            A.w0h[q] = 0.5 * A.w0[q]; A.w0h[A.SS + q] = 0.5 * A.w0[A.SS + q];
            A.w0h[2 * A.SS + q] = 0.5 * A.w0[2 * A.SS + q];
        }
        if (a.smoothing) {
            const double ci = MUL(cs, dti);
            A.w0i[q] = sb * ci; A.w0i[A.SS + q] = md * ci; A.w0i[2 * A.SS + q] = sp * ci;
        }
    }
    if (i == 0) {
        const int64_t q = A.v_off[o] + j;
        double sb = 0.0, md = 0.0, sp = 0.0;
        if (j > 0 && j < n1 - 1) centre(v, j, 1, sb, md, sp);
        A.w1[q] = sb * v[j]; A.w1[A.SV + q] = md * v[j]; A.w1[2 * A.SV + q] = sp * v[j];
        A.dirS[q] = 0.0;
        A.dirS[A.SV + q] = 0.0;
        const Row3 top = spot_row_w(swo + n0 - 1, A.SS, S, n0, n0 - 1, v[j], r, half_r, barrier);
        A.R0top[q] = top.dirichlet ? top.R : MUL(top.R, dt);
        if (a.smoothing) A.RSi[q] = top.dirichlet ? top.R : MUL(top.R, -dti);
        const Row3 w = var_row(v, n1, j, 1.0, r, half_r, kappa, th, sigma);
        A.F1v[q] = MUL(w.sub, dt); A.F1v[A.SV + q] = MUL(w.mid, dt);
        A.F1v[2 * A.SV + q] = MUL(w.sup, dt);
        if (a.hv) {
            A.LE1v[q] = MUL(MUL(w.sub, a.theta), dt);
            A.LE1v[A.SV + q] = MUL(MUL(w.mid, a.theta), dt);
            A.LE1v[2 * A.SV + q] = MUL(MUL(w.sup, a.theta), dt);
            A.F1h[q] = 0.5 * A.F1v[q];
            A.F1h[A.SV + q] = 0.5 * A.F1v[A.SV + q];
            A.F1h[2 * A.SV + q] = 0.5 * A.F1v[2 * A.SV + q];
        }
    }
}

// Spot lines: factors of Li0 = 1 - theta dt A0 (main) and 1 - dt f A0 (implicit).
__global__ void build_spot_lines_kernel(Arena A, BuildArgs a) {
    const int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= A.SV) return;
    const int o = A.lineS[line];
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int j = (int)(line - A.v_off[o]);
    const double *S = a.spots + A.s_off[o], *v = a.vars + A.v_off[o];
    double r, kappa, th, sigma, rho;
    opt_params(a, o, r, kappa, th, sigma, rho);
    const float half_r = (float)(-r / 2.0);
    const bool barrier = a.barrier && a.barrier[o];
    const double dt = a.dt[o];
    const double sm = MUL(a.theta, -dt), si = -MUL(dt, a.dt_factor);
    const double *swo = A.sw + A.s_off[o];
    Thomas tm, ti;
    for (int i = 0; i < n0; ++i) {
        const int64_t p = A.p_off[o] + (int64_t)i * n1 + j;
        const Row3 s = spot_row_w(swo + i, A.SS, S, n0, i, v[j], r, half_r, barrier);
        double sb = 0.0, md = 1.0, sp = 0.0;
        if (!s.dirichlet) { sb = MUL(s.sub, sm); md = ADD(MUL(s.mid, sm), 1.0); sp = MUL(s.sup, sm); }
        tm.row(A.LS, A.P, p, sb, md, sp, i == 0);
        if (a.smoothing) {
            sb = 0.0; md = 1.0; sp = 0.0;
            if (!s.dirichlet) { sb = MUL(s.sub, si); md = ADD(MUL(s.mid, si), 1.0); sp = MUL(s.sup, si); }
            ti.row(A.LSi, A.P, p, sb, md, sp, i == 0);
        }
    }
    if (tm.bad || ti.bad) atomicOr(&A.ostat[o], FDADI_STATUS_PIVOT);
}

// ---- stage kernels --------------------------------------------------------

enum : int { ST_DOUGLAS = 0, ST_HV0 = 1, ST_HV3 = 2, ST_IMPLICIT = 3, ST_CS3 = 4, ST_MCS3 = 5 };

// One 16x32 tile of one option. X (the operand of the applies: V, or Y2 in
// the HV corrector) is staged with a halo of one row above and below, two
// columns on the left (the A[n1-1, n1-3] corner) and one on the right.
template <int MODE>
__device__ __forceinline__ void explicit_tile(const Arena &A, const double *__restrict__ V,
                                              int64_t tile, double (*sX)[XCP], double (*sT)[TJ],
                                              double (*sD)[XCP]) {
    constexpr bool CS = MODE == ST_CS3 || MODE == ST_MCS3;
    const int4 t = A.tiles[tile];
    const int o = t.x, i0 = t.y, j0 = t.z;
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int fl = A.oflags[o];
    const int64_t P = A.P, p0 = A.p_off[o];
    const double *X = (MODE == ST_HV3 ? A.Y2 : V) + p0;
    const int tid = threadIdx.x;
    for (int e = tid; e < XR * XC; e += EXPL_THREADS) {
        const int rr = e / XC, cc = e - rr * XC;
        const int ii = i0 - 1 + rr, jj = j0 - 2 + cc;
        const bool in = ii >= 0 && ii < n0 && jj >= 0 && jj < n1;
        const double x = in ? X[(int64_t)ii * n1 + jj] : 0.0;
        sX[rr][cc] = x;
        // Craig-Sneyd correctors: D = Y2 - V beside V
        if constexpr (CS) sD[rr][cc] = in ? A.Y2[p0 + (int64_t)ii * n1 + jj] - x : 0.0;
    }
    __syncthreads();
    const bool mixed = fl & OPT_MIXED;
    const int64_t vo = A.v_off[o], so = A.s_off[o];
    if (mixed) {
        // mixed stencil row sums t(r, j) = sum_b w1[b](j) X(r, j + b) (of D in
        // the Craig-Sneyd correctors)
        double(*sM)[XCP] = CS ? sD : sX;
        for (int e = tid; e < XR * TJ; e += EXPL_THREADS) {
            const int rr = e / TJ, cc = e - rr * TJ;
            const int jj = j0 + cc;
            double s = 0.0;
            if (jj > 0 && jj < n1 - 1)
                s = A.w1[vo + jj] * sM[rr][cc + 1] + A.w1[A.SV + vo + jj] * sM[rr][cc + 2] +
                    A.w1[2 * A.SV + vo + jj] * sM[rr][cc + 3];
            sT[rr][cc] = s;
        }
        __syncthreads();
    }
    const int ty = tid / TJ, tx = tid - ty * TJ;
    const int i = i0 + ty, j = j0 + tx;
    if (i >= n0 || j >= n1) return;
    const int64_t pl = (int64_t)i * n1 + j, p = p0 + pl;
    const int64_t js = vo + j;
    const bool slow = fl & OPT_S_LOW_DIR, shigh = fl & OPT_S_HIGH_DIR;

    const bool mix_pt = mixed && i > 0 && i < n0 - 1 && j > 0 && j < n1 - 1;
    const double xc = sX[ty + 1][tx + 2];
    if constexpr (CS) {
        // Craig-Sneyd corrector (FiniteDifferenceEngine.pyx:843-898): right-hand
        // side of the second sweep, Y0 + (dt/2) M D - theta dt A0 V with
        // Y0 = V + R + F(V) and D = Y2 - V. Modified (:779-841): theta dt M D +
        // (1/2 - theta) sum_k F_k.apply(D) in place of (dt/2) M D, which is
        // (dt/2) M D + (1/2 - theta)(dt A0 D + dt A1 D + dt R): the reference
        // applies F_k with its residual. T = dt A1 V for the variance sweep.
        const double th = A.theta[o];
        const double gl = A.dirS[js], gh = A.dirS[A.SV + js];
        const bool dlo = i == 0 && slow, dhi = i == n0 - 1 && shigh;
        auto spot_apply = [&](double (*sY)[XCP], const double *F) {
            if (dlo) return gl;
            if (dhi) return gh;
            const double ym = (i == 1 && slow) ? gl : sY[ty][tx + 2];
            const double yp = (i == n0 - 2 && shigh) ? gh : sY[ty + 2][tx + 2];
            return F[p] * ym + F[P + p] * sY[ty + 1][tx + 2] + F[2 * P + p] * yp;
        };
        auto var_apply = [&](double (*sY)[XCP]) {
            const double yc = sY[ty + 1][tx + 2];
            if (i == 0 && (fl & OPT_ROW0_ZERO)) return A.F1z[o] * yc;
            double r = A.F1v[js] * sY[ty + 1][tx + 1] + A.F1v[A.SV + js] * yc +
                       A.F1v[2 * A.SV + js] * sY[ty + 1][tx + 3];
            if (j == n1 - 1) r += A.F1x[o] * sY[ty + 1][tx];
            return r;
        };
        const double a0v = spot_apply(sX, A.F0), a1v = var_apply(sX);
        double acc = xc + A.FV[p];
        if (i == n0 - 1) acc = fma(MODE == ST_CS3 ? 1.0 : 1.5 - th, A.R0top[js], acc);
        acc = fma(-th, a0v, acc);
        if (mix_pt) {
            acc = fma(A.w0h[so + i], sT[ty][tx], acc);
            acc = fma(A.w0h[A.SS + so + i], sT[ty + 1][tx], acc);
            acc = fma(A.w0h[2 * A.SS + so + i], sT[ty + 2][tx], acc);
        }
        if constexpr (MODE == ST_MCS3) {
            // (1/2 - theta) dt A0 D through the (1/2 - theta) F0 copy; Dirichlet
            // rows give the boundary value, as apply does
            const double a0d = (dlo || dhi) ? (0.5 - th) * (dlo ? gl : gh) : spot_apply(sD, A.F0h);
            acc += a0d;
            acc = fma(0.5 - th, var_apply(sD), acc);
        }
        A.W[p] = acc;
        A.T[p] = a1v;
        return;
    }
    if constexpr (MODE == ST_HV3) {
        // Y0 - F(V - Y2)/2 - theta F0 Y2 = V + R + F(V)/2 + (1/2 - theta) F0 Y2
        //   + F1 Y2 / 2 + M Y2 / 2, accumulated in one FMA chain with the
        // (1/2 - theta) F0, F1 / 2 and w0 / 2 copies built for this stage (the
        // halvings are exact)
        double acc = V[p];
        if (i == n0 - 1) acc += A.R0top[js];
        acc = fma(0.5, A.FV[p], acc);
        if ((i == 0 && slow) || (i == n0 - 1 && shigh)) {
            acc = fma(0.5 - A.theta[o], i == 0 ? A.dirS[js] : A.dirS[A.SV + js], acc);
        } else {
            const double xm = (i == 1 && slow) ? A.dirS[js] : sX[ty][tx + 2];
            const double xp = (i == n0 - 2 && shigh) ? A.dirS[A.SV + js] : sX[ty + 2][tx + 2];
            acc = fma(A.F0h[p], xm, acc);
            acc = fma(A.F0h[P + p], xc, acc);
            acc = fma(A.F0h[2 * P + p], xp, acc);
        }
        if (mix_pt) {
            acc = fma(A.w0h[so + i], sT[ty][tx], acc);
            acc = fma(A.w0h[A.SS + so + i], sT[ty + 1][tx], acc);
            acc = fma(A.w0h[2 * A.SS + so + i], sT[ty + 2][tx], acc);
        }
        // The corrector's variance term theta dt A1 Y2 is formed beside the
        // chain's 1/2 F1 Y2 (same neighbours), with the reference's
        // (A1 theta) dt coefficients: these operators are built once, so a
        // coefficient rounded otherwise (theta times dt A1, or 1/2 F1 taken
        // from it) would bias every step alike, and over a run the price
        // drifts by up to ~1e-10.
        double le;
        if (i == 0 && (fl & OPT_ROW0_ZERO)) {
            acc = fma(0.5 * A.F1z[o], xc, acc);
            le = A.LE1z[o] * xc;
        } else {
            acc = fma(A.F1h[js], sX[ty + 1][tx + 1], acc);
            acc = fma(A.F1h[A.SV + js], xc, acc);
            acc = fma(A.F1h[2 * A.SV + js], sX[ty + 1][tx + 3], acc);
            le = A.LE1v[js] * sX[ty + 1][tx + 1] + A.LE1v[A.SV + js] * xc +
                 A.LE1v[2 * A.SV + js] * sX[ty + 1][tx + 3];
            if (j == n1 - 1) {
                acc = fma(0.5 * A.F1x[o], sX[ty + 1][tx], acc);
                le += A.LE1x[o] * sX[ty + 1][tx];
            }
        }
        A.T[p] = le;
        A.W[p] = acc;
        return;
    }
    if constexpr (MODE == ST_IMPLICIT) {
        // x + M x, the mixed term chained onto x
        double acc = xc;
        if (mix_pt) {
            acc = fma(A.w0i[so + i], sT[ty][tx], acc);
            acc = fma(A.w0i[A.SS + so + i], sT[ty + 1][tx], acc);
            acc = fma(A.w0i[2 * A.SS + so + i], sT[ty + 2][tx], acc);
        }
        A.W[p] = acc;
        return;
    }
    // spot operator with the Dirichlet rows forced (BandedOperator.pyx:339-344)
    const double gl = A.dirS[js], gh = A.dirS[A.SV + js];
    double a0;
    if (i == 0 && slow) a0 = gl;
    else if (i == n0 - 1 && shigh) a0 = gh;
    else {
        const double xm = (i == 1 && slow) ? gl : sX[ty][tx + 2];
        const double xp = (i == n0 - 2 && shigh) ? gh : sX[ty + 2][tx + 2];
        a0 = A.F0[p] * xm + A.F0[P + p] * xc + A.F0[2 * P + p] * xp;
    }
    // variance operator (1-D on S > 0, diagonal on S = 0)
    double a1;
    if (i == 0 && (fl & OPT_ROW0_ZERO)) {
        a1 = A.F1z[o] * xc;
    } else {
        a1 = A.F1v[js] * sX[ty + 1][tx + 1] + A.F1v[A.SV + js] * xc +
             A.F1v[2 * A.SV + js] * sX[ty + 1][tx + 3];
        if (j == n1 - 1) a1 += A.F1x[o] * sX[ty + 1][tx];
    }
    // F1 x + M x, the mixed term chained onto F1 x
    double s = a1;
    if (mix_pt) {
        s = fma(A.w0[so + i], sT[ty][tx], s);
        s = fma(A.w0[A.SS + so + i], sT[ty + 1][tx], s);
        s = fma(A.w0[2 * A.SS + so + i], sT[ty + 2][tx], s);
    }
    // Y0 = V + F(V) + R; right-hand side of the spot solve Y0 - theta F0 V.
    // T holds F1 x; the spot solve subtracts theta T from its result.
    const double fv = s + a0;
    if (MODE == ST_HV0) A.FV[p] = fv;
    double base = xc + fv;
    if (i == n0 - 1) base += A.R0top[js];
    A.W[p] = fma(-A.theta[o], a0, base);
    A.T[p] = a1;
}

// Explicit stage over tiles [tile0, tile1): one block per tile, or (with
// fewer blocks) each block loops over tiles, so the stage can be held to a
// share of every SM while line solves of another option group run beside it.
template <int MODE>
__global__ void __launch_bounds__(EXPL_THREADS, 4) explicit_kernel(Arena A, const double *__restrict__ V,
                                                                  int64_t tile0, int64_t tile1) {
    __shared__ double sX[XR][XCP];
    __shared__ double sT[XR][TJ];
    __shared__ double sD[(MODE == ST_CS3 || MODE == ST_MCS3) ? XR : 1][XCP];
    for (int64_t t = tile0 + blockIdx.x; t < tile1; t += gridDim.x) {
        explicit_tile<MODE>(A, V, t, sX, sT, sD);
        __syncthreads();  // the next tile reuses the shared tiles
    }
}

// Spot-line solve, one thread per grid column. src -> dst (may alias).
// IMPLICIT: implicit-plan factors and residual. SUBT: write x - T (the next
// stage's right-hand side) instead of x.
template <bool IMPLICIT, bool SUBT, int PF>
__global__ void __launch_bounds__(SPOT_MAX_THREADS) spot_solve_kernel(Arena A, const double *src,
                                                                      double *dst, Span lines) {
    const int64_t line = lines.lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= lines.hi) return;
    const int o = A.lineS[line];
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int64_t js = line, j = line - A.v_off[o];
    const int fl = A.oflags[o];
    const bool slow = fl & OPT_S_LOW_DIR, shigh = fl & OPT_S_HIGH_DIR;
    const int64_t P = A.P, b = A.p_off[o] + j;
    const double *L = IMPLICIT ? A.LSi : A.LS;
    const double gl = A.dirS[js], gh = A.dirS[A.SV + js];
    if constexpr (PF == 1) {
        double dp = 0.0;
        for (int i = 0; i < n0; ++i) {
            const int64_t p = b + (int64_t)i * n1;
            double rk;
            if (i == 0 && slow) rk = gl;
            else if (i == n0 - 1 && shigh) rk = gh;
            else rk = src[p];
            if (IMPLICIT && i == n0 - 1) rk = rk - A.RSi[js];
            dp = (i == 0) ? rk * L[P + p] : (rk - L[p] * dp) * L[P + p];
            dst[p] = dp;
        }
        const double th = SUBT ? A.theta[o] : 0.0;
        double x = dp;
        {
            const int64_t p = b + (int64_t)(n0 - 1) * n1;
            if (SUBT) dst[p] = fma(-th, A.T[p], x);
        }
        for (int i = n0 - 2; i >= 0; --i) {
            const int64_t p = b + (int64_t)i * n1;
            x = dst[p] - L[2 * P + p] * x;
            dst[p] = SUBT ? fma(-th, A.T[p], x) : x;
        }
    } else {
        // Rows i+1 .. i+PF are loaded while row i is eliminated: each row's
        // loads are independent of the recurrence, so PF of them stay in flight
        // (src and dst may alias, so the compiler would not hoist them itself).
        // PF = 1 is the plain loop, for batches with enough lines to hide latency.
        double rs[PF], la[PF], li[PF];
    #pragma unroll
        for (int d = 0; d < PF; ++d) {
            if (d < n0) {
                const int64_t p = b + (int64_t)d * n1;
                rs[d] = src[p]; la[d] = L[p]; li[d] = L[P + p];
            }
        }
        double dp = 0.0;
        for (int i0 = 0; i0 < n0; i0 += PF) {
    #pragma unroll
            for (int d = 0; d < PF; ++d) {
                const int i = i0 + d;
                if (i < n0) {
                    const int64_t p = b + (int64_t)i * n1;
                    double rk = rs[d];
                    if (i == 0 && slow) rk = gl;
                    else if (i == n0 - 1 && shigh) rk = gh;
                    if (IMPLICIT && i == n0 - 1) rk = rk - A.RSi[js];
                    dp = (i == 0) ? rk * li[d] : (rk - la[d] * dp) * li[d];
                    dst[p] = dp;
                    if (i + PF < n0) {
                        const int64_t q = p + (int64_t)PF * n1;
                        rs[d] = src[q]; la[d] = L[q]; li[d] = L[P + q];
                    }
                }
            }
        }
        // back substitution, bottom to top, with the same prefetch ring
        const double th = SUBT ? A.theta[o] : 0.0;
        double ds[PF], cs[PF], ts[PF];
    #pragma unroll
        for (int d = 0; d < PF; ++d) {
            const int i = n0 - 2 - d;
            if (i >= 0) {
                const int64_t p = b + (int64_t)i * n1;
                ds[d] = dst[p]; cs[d] = L[2 * P + p]; ts[d] = SUBT ? A.T[p] : 0.0;
            }
        }
        double x = dp;
        if (SUBT) {
            const int64_t p = b + (int64_t)(n0 - 1) * n1;
            dst[p] = fma(-th, A.T[p], x);
        }
        for (int k0 = 0; k0 < n0 - 1; k0 += PF) {
    #pragma unroll
            for (int d = 0; d < PF; ++d) {
                const int i = n0 - 2 - (k0 + d);
                if (i >= 0) {
                    const int64_t p = b + (int64_t)i * n1;
                    x = ds[d] - cs[d] * x;
                    dst[p] = SUBT ? fma(-th, ts[d], x) : x;
                    if (i - PF >= 0) {
                        const int64_t q = p - (int64_t)PF * n1;
                        ds[d] = dst[q]; cs[d] = L[2 * P + q]; ts[d] = SUBT ? A.T[q] : 0.0;
                    }
                }
            }
        }
    }
}

// Variance-line solve: one warp per task of up to 32 consecutive grid rows of
// one option (lane = row). Chunks of 32 columns are loaded row by row
// (coalesced) into a padded shared tile, each lane runs its row's recurrence
// over the chunk, and the chunk is stored back row by row. The bottom row of
// the right-hand side is folded with the option's fold factor.
template <bool IMPLICIT, int NW>
__global__ void __launch_bounds__(NW * 32) var_solve_kernel(Arena A, Span tasks,
                                                            const double *src, double *dst) {
    __shared__ double tile[NW][32][VS_PITCH];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = tasks.lo + (int64_t)blockIdx.x * NW + warp;
    if (task >= tasks.hi) return;
    const int4 tk = A.vtasks[task];
    const int o = tk.x, i0 = tk.y, rows = tk.z;
    const int n1 = A.n1[o];
    const int64_t base = A.p_off[o] + (int64_t)i0 * n1;
    const int64_t vo = A.v_off[o], SV = A.SV;
    const double *L = IMPLICIT ? A.LVvi : A.LVv;
    const double f = IMPLICIT ? A.foldVi[o] : A.foldV[o];
    const double z = IMPLICIT ? A.LVzi[o] : A.LVz[o];
    const bool special = (i0 + lane == 0) && (A.oflags[o] & OPT_ROW0_ZERO);
    double(*tl)[VS_PITCH] = tile[warp];
    const int nch = (n1 + 31) >> 5;
    double dp = 0.0, rprev = 0.0;
    for (int ch = 0; ch < nch; ++ch) {
        const int c0 = ch << 5, w = min(32, n1 - c0);
        for (int rr = 0; rr < rows; ++rr)
            tl[rr][lane] = lane < w ? src[base + (int64_t)rr * n1 + c0 + lane] : 0.0;
        __syncwarp();
        if (lane < rows) {
            for (int c = 0; c < w; ++c) {
                const int col = c0 + c;
                double rk = tl[lane][c];
                const double raw = rk;
                if (special) {
                    dp = rk * z;
                } else {
                    if (col == n1 - 1) rk += 1.0 * rprev * f;
                    const double inv = L[SV + vo + col];
                    dp = (col == 0) ? rk * inv : (rk - L[vo + col] * dp) * inv;
                }
                tl[lane][c] = dp;
                rprev = raw;
            }
        }
        __syncwarp();
        for (int rr = 0; rr < rows; ++rr)
            if (lane < w) dst[base + (int64_t)rr * n1 + c0 + lane] = tl[rr][lane];
        __syncwarp();
    }
    double x = 0.0;
    for (int ch = nch - 1; ch >= 0; --ch) {
        const int c0 = ch << 5, w = min(32, n1 - c0);
        for (int rr = 0; rr < rows; ++rr)
            tl[rr][lane] = lane < w ? dst[base + (int64_t)rr * n1 + c0 + lane] : 0.0;
        __syncwarp();
        if (lane < rows) {
            for (int c = w - 1; c >= 0; --c) {
                const int col = c0 + c;
                const double d = tl[lane][c];
                x = (col == n1 - 1 || special) ? d : d - L[2 * SV + vo + col] * x;
                tl[lane][c] = x;
            }
        }
        __syncwarp();
        for (int rr = 0; rr < rows; ++rr)
            if (lane < w) dst[base + (int64_t)rr * n1 + c0 + lane] = tl[rr][lane];
        __syncwarp();
    }
}

// Partitioned spot solve, for batches with few, long spot lines (one large
// grid, small batches), where one thread per line leaves most of the GPU idle.
// A block holds LPB adjacent lines (thread t: line t % LPB) and cuts each line
// into NSEG contiguous row segments (segment t / LPB), so accesses stay
// coalesced across the block's lines. Both Thomas sweeps are first-order
// linear recurrences on the precomputed factors,
//   d_i = (r_i - a_i d_{i-1}) / m_i,   x_i = d_i - c'_i x_{i+1},
// so each segment runs them from a zero carry while tracking the product of
// the multipliers (the carry's weight), one thread per line combines the
// segment carries in order, and a second pass adds weight * carry: four
// passes of a segment instead of two passes of the whole line.
template <bool IMPLICIT, bool SUBT, int LPB, int NSEG>
__global__ void __launch_bounds__(LPB * NSEG) spot_seg_kernel(Arena A, const double *src,
                                                              double *dst, Span lines) {
    __shared__ double cval[NSEG][LPB], cwt[NSEG][LPB];
    const int t = threadIdx.x, ls = t % LPB, sg = t / LPB;
    const int64_t line = lines.lo + (int64_t)blockIdx.x * LPB + ls;
    const bool valid = line < lines.hi;
    const double *L = IMPLICIT ? A.LSi : A.LS;
    const int64_t P = A.P;
    int o = 0, n0 = 0, n1 = 1, lo = 0, hi = 0;
    int64_t b = 0;
    if (valid) {
        o = A.lineS[line];
        n0 = A.n0[o];
        n1 = A.n1[o];
        b = A.p_off[o] + (line - A.v_off[o]);
        const int seg = (n0 + NSEG - 1) / NSEG;
        lo = min(n0, sg * seg);
        hi = min(n0, lo + seg);
    }
    // pass 1: forward sweep from a zero carry; g = d(d_i)/d(d_{lo-1})
    {
        const int fl = valid ? A.oflags[o] : 0;
        const bool slow = fl & OPT_S_LOW_DIR, shigh = fl & OPT_S_HIGH_DIR;
        const double gl = valid ? A.dirS[line] : 0.0, gh = valid ? A.dirS[A.SV + line] : 0.0;
        double d = 0.0, g = 1.0;
        for (int i = lo; i < hi; ++i) {
            const int64_t p = b + (int64_t)i * n1;
            double rk;
            if (i == 0 && slow) rk = gl;
            else if (i == n0 - 1 && shigh) rk = gh;
            else rk = src[p];
            if (IMPLICIT && i == n0 - 1) rk = rk - A.RSi[line];
            const double inv = L[P + p];
            if (i == 0) {
                d = rk * inv;
                g = 0.0;
            } else {
                const double a = L[p];
                d = (rk - a * d) * inv;
                g = (-a * g) * inv;
            }
            dst[p] = d;
        }
        cval[sg][ls] = d;
        cwt[sg][ls] = g;
    }
    __syncthreads();
    if (sg == 0) {
        double D = 0.0;  // d at the row before segment s
        for (int s = 0; s < NSEG; ++s) {
            const double v = cval[s][ls], w = cwt[s][ls];
            cval[s][ls] = D;
            D = fma(w, D, v);
        }
    }
    __syncthreads();
    // pass 2: d_i += g_i * carry (segment 0 starts at row 0 and is exact)
    if (sg > 0) {
        const double C = cval[sg][ls];
        double g = 1.0;
        for (int i = lo; i < hi; ++i) {
            const int64_t p = b + (int64_t)i * n1;
            g = (-L[p] * g) * L[P + p];
            dst[p] = fma(g, C, dst[p]);
        }
    }
    __syncthreads();
    // pass 3: back substitution from a zero carry; h = d(x_i)/d(x_{hi})
    {
        double x = 0.0, h = 1.0;
        for (int i = hi - 1; i >= lo; --i) {
            const int64_t p = b + (int64_t)i * n1;
            if (i == n0 - 1) {
                x = dst[p];
                h = 0.0;
            } else {
                const double c = L[2 * P + p];
                x = dst[p] - c * x;
                h = -c * h;
            }
            dst[p] = x;
        }
        cval[sg][ls] = x;
        cwt[sg][ls] = h;
    }
    __syncthreads();
    if (sg == 0) {
        double X = 0.0;  // x at the row after segment s
        for (int s = NSEG - 1; s >= 0; --s) {
            const double v = cval[s][ls], w = cwt[s][ls];
            cval[s][ls] = X;
            X = fma(w, X, v);
        }
    }
    __syncthreads();
    // pass 4: x_i += h_i * carry, then the stage's output
    {
        const double C = cval[sg][ls];
        const double th = (SUBT && valid) ? A.theta[o] : 0.0;
        double h = 1.0;
        for (int i = hi - 1; i >= lo; --i) {
            const int64_t p = b + (int64_t)i * n1;
            h = (i == n0 - 1) ? 0.0 : -L[2 * P + p] * h;
            const double x = fma(h, C, dst[p]);
            dst[p] = SUBT ? fma(-th, A.T[p], x) : x;
        }
    }
}

__device__ __forceinline__ void cp_async8(void *sdst, const void *gsrc) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gsrc));
}

// Variance-line solve with the Thomas factors in registers: as
// var_solve_kernel (one warp per task of up to 32 grid rows, 32x32 chunks
// through a padded shared tile), with each chunk's factors held one per lane
// and broadcast by shuffle, so no global load sits on the recurrence's path.
// DB: two tiles per warp, the cp.async copies of the next chunk in flight
// while the lanes run the current chunk; without DB one tile (half the shared
// memory, twice the resident warps). The back substitution starts from the
// forward sweep's last chunk, still in shared memory. Dynamic shared memory:
// NW * (DB ? 2 : 1) * 32 * VS_PITCH doubles.
template <bool IMPLICIT, int NW, bool DB>
__global__ void __launch_bounds__(NW * 32) var_solve_pipe_kernel(Arena A, Span tasks,
                                                                 const double *src, double *dst) {
    constexpr int NB = DB ? 2 : 1;
    extern __shared__ double vsm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = tasks.lo + (int64_t)blockIdx.x * NW + warp;
    if (task >= tasks.hi) return;
    double(*tl)[32][VS_PITCH] =
        reinterpret_cast<double(*)[32][VS_PITCH]>(vsm + (size_t)warp * NB * 32 * VS_PITCH);
    const int4 tk = A.vtasks[task];
    const int o = tk.x, i0 = tk.y, rows = tk.z;
    const int n1 = A.n1[o];
    const int64_t base = A.p_off[o] + (int64_t)i0 * n1;
    const int64_t vo = A.v_off[o], SV = A.SV;
    const double *L = IMPLICIT ? A.LVvi : A.LVv;
    const double f = IMPLICIT ? A.foldVi[o] : A.foldV[o];
    const double z = IMPLICIT ? A.LVzi[o] : A.LVz[o];
    const bool special = (i0 + lane == 0) && (A.oflags[o] & OPT_ROW0_ZERO);
    const int nch = (n1 + 31) >> 5;
    const unsigned FULL = 0xffffffffu;
    auto issue = [&](const double *from, int ch, int buf) {
        const int c0 = ch << 5, w = min(32, n1 - c0);
        if (lane < w)
            for (int rr = 0; rr < rows; ++rr)
                cp_async8(&tl[buf][rr][lane], from + base + (int64_t)rr * n1 + c0 + lane);
        asm volatile("cp.async.commit_group;");
    };
    // forward sweep
    issue(src, 0, 0);
    double fa = 0.0, fi = 0.0;
    if (lane < min(32, n1)) { fa = L[vo + lane]; fi = L[SV + vo + lane]; }
    double dp = 0.0, rprev = 0.0;
    for (int ch = 0; ch < nch; ++ch) {
        const int buf = DB ? (ch & 1) : 0, c0 = ch << 5, w = min(32, n1 - c0);
        double na = 0.0, ni = 0.0;
        if (ch + 1 < nch) {
            const int c1 = c0 + 32;
            if (DB) issue(src, ch + 1, buf ^ 1);
            if (lane < min(32, n1 - c1)) { na = L[vo + c1 + lane]; ni = L[SV + vo + c1 + lane]; }
        }
        if (DB && ch + 1 < nch) asm volatile("cp.async.wait_group 1;");
        else asm volatile("cp.async.wait_group 0;");
        __syncwarp();
        for (int c = 0; c < w; ++c) {
            const double ac = __shfl_sync(FULL, fa, c), ic = __shfl_sync(FULL, fi, c);
            if (lane < rows) {
                const int col = c0 + c;
                double rk = tl[buf][lane][c];
                const double raw = rk;
                if (special) {
                    dp = rk * z;
                } else {
                    if (col == n1 - 1) rk += 1.0 * rprev * f;
                    dp = (col == 0) ? rk * ic : (rk - ac * dp) * ic;
                }
                tl[buf][lane][c] = dp;
                rprev = raw;
            }
        }
        __syncwarp();
        if (lane < w)
            for (int rr = 0; rr < rows; ++rr)
                dst[base + (int64_t)rr * n1 + c0 + lane] = tl[buf][rr][lane];
        __syncwarp();
        fa = na;
        fi = ni;
        if (!DB && ch + 1 < nch) issue(src, ch + 1, 0);
    }
    // the next copies read dst back: order this lane's stores before them
    __threadfence_block();
    // back substitution, last chunk first (its forward results are still in
    // the tile the forward sweep ended on)
    double fc = 0.0;
    {
        const int c0 = (nch - 1) << 5;
        if (lane < n1 - c0) fc = L[2 * SV + vo + c0 + lane];
    }
    double x = 0.0;
    for (int ch = nch - 1; ch >= 0; --ch) {
        const int buf = DB ? (ch & 1) : 0, c0 = ch << 5, w = min(32, n1 - c0);
        double nc = 0.0;
        if (ch > 0) {
            if (DB) issue(dst, ch - 1, buf ^ 1);
            nc = L[2 * SV + vo + c0 - 32 + lane];
        }
        if (DB && ch > 0) asm volatile("cp.async.wait_group 1;");
        else asm volatile("cp.async.wait_group 0;");
        __syncwarp();
        for (int c = w - 1; c >= 0; --c) {
            const double cc = __shfl_sync(FULL, fc, c);
            if (lane < rows) {
                const int col = c0 + c;
                const double d = tl[buf][lane][c];
                x = (col == n1 - 1 || special) ? d : d - cc * x;
                tl[buf][lane][c] = x;
            }
        }
        __syncwarp();
        if (lane < w)
            for (int rr = 0; rr < rows; ++rr)
                dst[base + (int64_t)rr * n1 + c0 + lane] = tl[buf][rr][lane];
        __syncwarp();
        fc = nc;
        if (!DB && ch > 0) issue(dst, ch - 1, 0);
    }
}

// Partitioned variance solve, for few long variance lines (one large grid):
// one block per task of up to 32 grid rows, its NSEG warps each taking a
// contiguous range of 32-column chunks. As in spot_seg_kernel, each segment
// runs both Thomas recurrences from a zero carry while tracking the product
// of the multipliers, warp 0 combines the segment carries per row, and a
// second pass adds product x carry; every pass streams its chunks through the
// warp's padded shared tile (coalesced rows, lane = grid row in the
// recurrence) with the factors broadcast by shuffle. Dynamic shared memory:
// NSEG * 32 * VS_PITCH doubles.
template <bool IMPLICIT, int NSEG>
__global__ void __launch_bounds__(NSEG * 32) var_seg_kernel(Arena A, Span tasks,
                                                            const double *src, double *dst) {
    extern __shared__ double vsm[];
    __shared__ double cval[NSEG][32], cwt[NSEG][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t task = tasks.lo + blockIdx.x;   // grid = tasks.hi - tasks.lo
    double(*tl)[VS_PITCH] = reinterpret_cast<double(*)[VS_PITCH]>(vsm + (size_t)warp * 32 * VS_PITCH);
    const int4 tk = A.vtasks[task];
    const int o = tk.x, i0 = tk.y, rows = tk.z;
    const int n1 = A.n1[o];
    const int64_t base = A.p_off[o] + (int64_t)i0 * n1;
    const int64_t vo = A.v_off[o], SV = A.SV;
    const double *L = IMPLICIT ? A.LVvi : A.LVv;
    const double f = IMPLICIT ? A.foldVi[o] : A.foldV[o];
    const double z = IMPLICIT ? A.LVzi[o] : A.LVz[o];
    const bool special = (i0 + lane == 0) && (A.oflags[o] & OPT_ROW0_ZERO);
    const unsigned FULL = 0xffffffffu;
    const int nch = (n1 + 31) >> 5;
    const int cps = (nch + NSEG - 1) / NSEG;
    const int ch_lo = min(nch, warp * cps), ch_hi = min(nch, ch_lo + cps);
    // raw right-hand side at column n1 - 2 (the bottom fold adds it to the last
    // column), read before any write since src and dst may alias
    double rfold = 0.0;
    if (lane < rows) rfold = src[base + (int64_t)lane * n1 + n1 - 2];
    __syncthreads();
    auto load = [&](const double *from, int ch) {
        const int c0 = ch << 5, w = min(32, n1 - c0);
        if (lane < w)
            for (int rr = 0; rr < rows; ++rr) tl[rr][lane] = from[base + (int64_t)rr * n1 + c0 + lane];
        __syncwarp();
    };
    auto store = [&](int ch) {
        __syncwarp();
        const int c0 = ch << 5, w = min(32, n1 - c0);
        if (lane < w)
            for (int rr = 0; rr < rows; ++rr) dst[base + (int64_t)rr * n1 + c0 + lane] = tl[rr][lane];
        __syncwarp();
    };
    // pass 1: forward sweep from a zero carry; g = d(d_j)/d(d_{first column - 1})
    double d = 0.0, g = 1.0;
    for (int ch = ch_lo; ch < ch_hi; ++ch) {
        load(src, ch);
        const int c0 = ch << 5, w = min(32, n1 - c0);
        double ca = 0.0, ci = 0.0;
        if (lane < w) { ca = L[vo + c0 + lane]; ci = L[SV + vo + c0 + lane]; }
        for (int c = 0; c < w; ++c) {
            const double a = __shfl_sync(FULL, ca, c), inv = __shfl_sync(FULL, ci, c);
            if (lane < rows) {
                const int col = c0 + c;
                double rk = tl[lane][c];
                if (special) {
                    d = rk * z;
                    g = 0.0;
                } else {
                    if (col == n1 - 1) rk += 1.0 * rfold * f;
                    if (col == 0) {
                        d = rk * inv;
                        g = 0.0;
                    } else {
                        d = (rk - a * d) * inv;
                        g = (-a * g) * inv;
                    }
                }
                tl[lane][c] = d;
            }
        }
        store(ch);
    }
    cval[warp][lane] = d;
    cwt[warp][lane] = g;
    __syncthreads();
    if (warp == 0) {
        double D = 0.0;   // d at the column before segment s
        for (int s = 0; s < NSEG; ++s) {
            const double v = cval[s][lane], wt = cwt[s][lane];
            cval[s][lane] = D;
            D = fma(wt, D, v);
        }
    }
    __syncthreads();
    // pass 2: d_j += g_j * carry (the first segment starts at column 0 and is exact)
    if (ch_lo > 0) {
        const double C = cval[warp][lane];
        double gg = 1.0;
        for (int ch = ch_lo; ch < ch_hi; ++ch) {
            load(dst, ch);
            const int c0 = ch << 5, w = min(32, n1 - c0);
            double ca = 0.0, ci = 0.0;
            if (lane < w) { ca = L[vo + c0 + lane]; ci = L[SV + vo + c0 + lane]; }
            for (int c = 0; c < w; ++c) {
                const double a = __shfl_sync(FULL, ca, c), inv = __shfl_sync(FULL, ci, c);
                if (lane < rows) {
                    gg = special ? 0.0 : (-a * gg) * inv;
                    tl[lane][c] = fma(gg, C, tl[lane][c]);
                }
            }
            store(ch);
        }
    }
    __syncthreads();
    // pass 3: back substitution from a zero carry; h = d(x_j)/d(x_{last column + 1})
    double x = 0.0, h = 1.0;
    for (int ch = ch_hi - 1; ch >= ch_lo; --ch) {
        load(dst, ch);
        const int c0 = ch << 5, w = min(32, n1 - c0);
        const double cc0 = lane < w ? L[2 * SV + vo + c0 + lane] : 0.0;
        for (int c = w - 1; c >= 0; --c) {
            const double cc = __shfl_sync(FULL, cc0, c);
            if (lane < rows) {
                const int col = c0 + c;
                const double dd = tl[lane][c];
                if (col == n1 - 1 || special) {
                    x = dd;
                    h = 0.0;
                } else {
                    x = dd - cc * x;
                    h = -cc * h;
                }
                tl[lane][c] = x;
            }
        }
        store(ch);
    }
    cval[warp][lane] = x;
    cwt[warp][lane] = h;
    __syncthreads();
    if (warp == 0) {
        double X = 0.0;   // x at the column after segment s
        for (int s = NSEG - 1; s >= 0; --s) {
            const double v = cval[s][lane], wt = cwt[s][lane];
            cval[s][lane] = X;
            X = fma(wt, X, v);
        }
    }
    __syncthreads();
    // pass 4: x_j += h_j * carry (the last segment ends at column n1 - 1 and is exact)
    if (ch_hi < nch && ch_lo < ch_hi) {
        const double C = cval[warp][lane];
        double hh = 1.0;
        for (int ch = ch_hi - 1; ch >= ch_lo; --ch) {
            load(dst, ch);
            const int c0 = ch << 5, w = min(32, n1 - c0);
            const double cc0 = lane < w ? L[2 * SV + vo + c0 + lane] : 0.0;
            for (int c = w - 1; c >= 0; --c) {
                const double cc = __shfl_sync(FULL, cc0, c);
                if (lane < rows) {
                    hh = special ? 0.0 : -cc * hh;
                    tl[lane][c] = fma(hh, C, tl[lane][c]);
                }
            }
            store(ch);
        }
    }
}

// Initial grid of a European call or put on every option's mesh (the
// reference's grid initializer, heston.py:402): V = max(S_i - K, 0) (call) or
// max(K - S_i, 0) (put) on every variance point; one block per tile.
__global__ void payoff_kernel(Arena A, const double *spots, const double *strikes, int put,
                              double *V) {
    const int4 t = A.tiles[blockIdx.x];
    const int o = t.x, n0 = A.n0[o], n1 = A.n1[o];
    const int i = t.y + threadIdx.x / TJ, j = t.z + threadIdx.x % TJ;
    if (i >= n0 || j >= n1) return;
    const double S = spots[A.s_off[o] + i], K = strikes[o];
    V[A.p_off[o] + (int64_t)i * n1 + j] = put ? fmax(K - S, 0.0) : fmax(S - K, 0.0);
}

// Per-option status: the build's pivot flags, plus FDADI_STATUS_NONFINITE if
// any value of the option's state grid is NaN or infinite (one block per option).
__global__ void status_kernel(Arena A, const double *V, int *out) {
    const int o = blockIdx.x;
    const int64_t p0 = A.p_off[o], n = (int64_t)A.n0[o] * A.n1[o];
    int bad = 0;
    for (int64_t k = threadIdx.x; k < n && !bad; k += blockDim.x)
        if (!isfinite(V[p0 + k])) bad = 1;
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) out[o] = A.ostat[o] | (bad ? FDADI_STATUS_NONFINITE : 0);
}

// Price, delta and gamma of option o at the grid point idx[o] (an index into
// the packed arena on its spot line): V there and the centred non-uniform first
// and second derivative stencils in S (centercoeffs, BandedOperator.pyx:970-1017)
// applied along the spot line; NaN greeks at the first or last spot row.
__global__ void greeks_kernel(Arena A, const double *spots, const double *V, const int64_t *idx,
                              double *price, double *delta, double *gamma) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= A.n_opt) return;
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int64_t q = idx[o];
    const int i = (int)((q - A.p_off[o]) / n1);
    const double vc = V[q];
    price[o] = vc;
    if (i <= 0 || i >= n0 - 1) {
        delta[o] = gamma[o] = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    const double *S = spots + A.s_off[o];
    const double vm = V[q - n1], vp = V[q + n1];
    double sb, md, sp;
    centre(S, i, 1, sb, md, sp);
    delta[o] = sb * vm + md * vc + sp * vp;
    centre(S, i, 2, sb, md, sp);
    gamma[o] = sb * vm + md * vc + sp * vp;
}

// Eight independent DFMA chains per thread: measures the FP64 pipe, not latency.
template <int CHAINS>
__global__ void fp64_probe_kernel(double *out, int iters) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = 1.0 + 1e-3 * (t + k);
    const double b = 0.999999999, c = 1e-9;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    out[t] = s;
}

__global__ void gather_kernel(const double *V, const int64_t *idx, double *out, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        out[k] = V[idx[k]];
}

// ---- host side ------------------------------------------------------------

static inline int64_t align256(int64_t x) { return (x + 255) & ~(int64_t)255; }

struct Layout {
    int n_opt = 0;
    int64_t P = 0, SS = 0, SV = 0, n_tiles = 0, n_vtasks = 0;
    bool smoothing = false, hv = false;
    // byte offsets into the workspace (-1: absent)
    int64_t o_n0, o_n1, o_flags, o_p, o_s, o_v, o_lineS, o_tiles, o_vtasks, o_theta, o_ostat;
    int64_t o_F0, o_w0, o_w1, o_LS, o_R0top, o_F1v, o_F1x, o_F1z, o_LVv, o_foldV, o_LVz,
        o_dirS;
    int64_t o_w0i, o_RSi, o_LSi, o_LVvi, o_foldVi, o_LVzi;
    int64_t o_FV, o_W, o_T, o_Y2, o_F0h, o_w0h, o_sw;
    int64_t o_LE1v, o_LE1x, o_LE1z, o_one, o_F1h;
    int64_t bytes = 0;
    std::vector<int64_t> p_off, s_off, v_off, tile_off, task_off;
};

static int make_layout(const fdadi_heston_batch_t *b, Layout &L) {
    FDADI_REQUIRE(b != nullptr, "null batch");
    FDADI_REQUIRE(b->n_options > 0, "empty batch");
    FDADI_REQUIRE(b->n0 && b->n1, "batch needs host size arrays n0, n1");
    FDADI_REQUIRE(b->scheme == FDADI_SCHEME_DOUGLAS || b->scheme == FDADI_SCHEME_HV ||
                      b->scheme == FDADI_SCHEME_CS || b->scheme == FDADI_SCHEME_MCS,
                  "main scheme must be Douglas, Hundsdorfer-Verwer or (modified) Craig-Sneyd");
    FDADI_REQUIRE(b->n_steps >= 0 && b->implicit_steps >= 0, "negative step count");
    FDADI_REQUIRE(b->implicit_steps == 0 || b->implicit_dt_factor > 0.0,
                  "implicit_dt_factor must be positive");
    L.n_opt = b->n_options;
    L.smoothing = b->implicit_steps > 0;
    // predictor/corrector schemes (HV, CS, MCS) keep F(V) and Y2
    L.hv = b->scheme != FDADI_SCHEME_DOUGLAS;
    L.p_off.resize(L.n_opt + 1);
    L.s_off.resize(L.n_opt + 1);
    L.v_off.resize(L.n_opt + 1);
    L.tile_off.resize(L.n_opt + 1);
    L.task_off.resize(L.n_opt + 1);
    L.p_off[0] = L.s_off[0] = L.v_off[0] = L.tile_off[0] = L.task_off[0] = 0;
    for (int k = 0; k < L.n_opt; ++k) {
        FDADI_REQUIRE(b->n0[k] >= 4 && b->n1[k] >= 4,
                      "Vector too short to use finite differencing (option %d: %d x %d)", k,
                      b->n0[k], b->n1[k]);
        const int64_t N = (int64_t)b->n0[k] * b->n1[k];
        L.p_off[k + 1] = L.p_off[k] + N;
        L.s_off[k + 1] = L.s_off[k] + b->n0[k];
        L.v_off[k + 1] = L.v_off[k] + b->n1[k];
        L.n_tiles += (int64_t)((b->n0[k] + TI - 1) / TI) * ((b->n1[k] + TJ - 1) / TJ);
        L.n_vtasks += (b->n0[k] + 31) / 32;
        L.tile_off[k + 1] = L.n_tiles;
        L.task_off[k + 1] = L.n_vtasks;
    }
    L.P = L.p_off[L.n_opt];
    L.SS = L.s_off[L.n_opt];
    L.SV = L.v_off[L.n_opt];
    FDADI_REQUIRE(L.n_tiles < ((int64_t)1 << 31) && L.n_vtasks < ((int64_t)1 << 31),
                  "batch too large");
    int64_t off = 0;
    auto take = [&](int64_t bytes) { int64_t o = off; off = align256(off + bytes); return o; };
    const int64_t D = sizeof(double), N = L.n_opt;
    L.o_n0 = take(4 * N); L.o_n1 = take(4 * N); L.o_flags = take(4 * N);
    L.o_p = take(8 * N); L.o_s = take(8 * N); L.o_v = take(8 * N);
    L.o_lineS = take(4 * L.SV); L.o_tiles = take(16 * L.n_tiles);
    L.o_vtasks = take(16 * L.n_vtasks); L.o_theta = take(D * N);
    L.o_ostat = take(4 * N);
    L.o_F0 = take(3 * D * L.P);
    L.o_sw = take(6 * D * L.SS);
    L.o_w0 = take(3 * D * L.SS); L.o_w1 = take(3 * D * L.SV);
    L.o_LS = take(3 * D * L.P); L.o_R0top = take(D * L.SV); L.o_F1v = take(3 * D * L.SV);
    L.o_F1x = take(D * N); L.o_F1z = take(D * N); L.o_LVv = take(3 * D * L.SV);
    L.o_foldV = take(D * N); L.o_LVz = take(D * N); L.o_dirS = take(2 * D * L.SV);
    if (L.smoothing) {
        L.o_w0i = take(3 * D * L.SS); L.o_RSi = take(D * L.SV); L.o_LSi = take(3 * D * L.P);
        L.o_LVvi = take(3 * D * L.SV); L.o_foldVi = take(D * N); L.o_LVzi = take(D * N);
    } else {
        L.o_w0i = L.o_RSi = L.o_LSi = L.o_LVvi = L.o_foldVi = L.o_LVzi = -1;
    }
    L.o_W = take(D * L.P); L.o_T = take(D * L.P);
    if (L.hv) {
        L.o_FV = take(D * L.P); L.o_Y2 = take(D * L.P);
        L.o_F0h = take(3 * D * L.P); L.o_w0h = take(3 * D * L.SS);
        L.o_LE1v = take(3 * D * L.SV); L.o_LE1x = take(D * N); L.o_LE1z = take(D * N);
        L.o_one = take(D * N); L.o_F1h = take(3 * D * L.SV);
    } else {
        L.o_FV = L.o_Y2 = L.o_F0h = L.o_w0h = -1;
        L.o_LE1v = L.o_LE1x = L.o_LE1z = L.o_one = L.o_F1h = -1;
    }
    L.bytes = off;
    return FDADI_OK;
}

static Arena arena_view(const Layout &L, char *ws) {
    Arena A;
    auto ptr = [&](int64_t o) -> double * { return o < 0 ? nullptr : (double *)(ws + o); };
    A.n_opt = L.n_opt; A.P = L.P; A.SS = L.SS; A.SV = L.SV;
    A.n0 = (const int *)(ws + L.o_n0); A.n1 = (const int *)(ws + L.o_n1);
    A.oflags = (const int *)(ws + L.o_flags);
    A.p_off = (const int64_t *)(ws + L.o_p); A.s_off = (const int64_t *)(ws + L.o_s);
    A.v_off = (const int64_t *)(ws + L.o_v);
    A.lineS = (const int *)(ws + L.o_lineS);
    A.tiles = (const int4 *)(ws + L.o_tiles);
    A.vtasks = (const int4 *)(ws + L.o_vtasks);
    A.theta = ptr(L.o_theta);
    A.ostat = (int *)(ws + L.o_ostat);
    A.F0 = ptr(L.o_F0); A.w0 = ptr(L.o_w0); A.w1 = ptr(L.o_w1);
    A.LS = ptr(L.o_LS); A.R0top = ptr(L.o_R0top); A.F1v = ptr(L.o_F1v); A.F1x = ptr(L.o_F1x);
    A.F1z = ptr(L.o_F1z); A.LVv = ptr(L.o_LVv); A.foldV = ptr(L.o_foldV); A.LVz = ptr(L.o_LVz);
    A.dirS = ptr(L.o_dirS);
    A.w0i = ptr(L.o_w0i); A.RSi = ptr(L.o_RSi); A.LSi = ptr(L.o_LSi); A.LVvi = ptr(L.o_LVvi);
    A.foldVi = ptr(L.o_foldVi); A.LVzi = ptr(L.o_LVzi);
    A.FV = ptr(L.o_FV); A.W = ptr(L.o_W); A.T = ptr(L.o_T); A.Y2 = ptr(L.o_Y2);
    A.F0h = ptr(L.o_F0h); A.w0h = ptr(L.o_w0h); A.sw = ptr(L.o_sw);
    A.LE1v = ptr(L.o_LE1v); A.LE1x = ptr(L.o_LE1x); A.LE1z = ptr(L.o_LE1z);
    A.one = ptr(L.o_one); A.F1h = ptr(L.o_F1h);
    return A;
}

// ---- launch plans ----------------------------------------------------------
//
// The spot and variance solves come in several launch shapes; which is
// fastest depends on the batch (number and length of lines, grid sizes), so a
// plan names one shape of each and fdadi_heston_tune measures them on the
// prepared batch. Without a plan a size heuristic picks: with many spot lines,
// thread parallelism hides memory latency and the plain loop (fewer registers,
// more resident threads) wins; with few lines the prefetching loop in 32-thread
// blocks spreads them over more SMs.
//
// A plan also splits the batch into option groups. The explicit stages are
// bound by the FP64 pipe and the line solves by HBM, so with two or more
// groups one group's solves run beside another group's explicit stage: each
// group's launches form their own chain (own stream, or own graph branch),
// the explicit stages of all groups are chained one after another so they do
// not compete for the FP64 pipe, and the solves are launched at the device's
// highest priority so their blocks take SM slots as explicit blocks retire.

using SpotFn = void (*)(Arena, const double *, double *, Span);
using VarFn = void (*)(Arena, Span, const double *, double *);

struct SpotVariant {
    int kind, a, b;   // plan fields
    int threads;      // block size
    int lines;        // spot lines per block
    SpotFn main;      // main plan, writes x - theta T
    SpotFn impl;      // implicit plan
};
struct VarVariant {
    int kind, warps;
    int smem;         // dynamic shared memory bytes
    VarFn main, impl;
    int tasks;        // tasks per block (kind 3: one task shared by all warps)
};

#define SPOT_T(PF, TH)                                                                  \
    SpotVariant{0, PF, TH, TH, TH, spot_solve_kernel<false, true, PF>,                  \
                spot_solve_kernel<true, false, PF>}
#define SPOT_S(LPB, NS)                                                                 \
    SpotVariant{1, LPB, NS, LPB * NS, LPB, spot_seg_kernel<false, true, LPB, NS>,       \
                spot_seg_kernel<true, false, LPB, NS>}
static const SpotVariant SPOT_VARIANTS[] = {
    SPOT_T(1, 128), SPOT_T(1, 64),  SPOT_T(1, 256), SPOT_T(4, 32),  SPOT_T(8, 32),
    SPOT_T(8, 64),  SPOT_S(32, 4),  SPOT_S(32, 8),  SPOT_S(32, 16), SPOT_S(32, 32),
    SPOT_S(16, 16), SPOT_S(16, 32), SPOT_S(16, 64), SPOT_S(8, 32),  SPOT_S(8, 64),
    SPOT_S(8, 128), SPOT_T(2, 64),  SPOT_T(2, 128), SPOT_T(4, 64),  SPOT_T(4, 128)};
#undef SPOT_T
#undef SPOT_S

constexpr int VAR_TILE_BYTES = 32 * VS_PITCH * (int)sizeof(double);
#define VAR_P(NW, DB)                                                                   \
    VarVariant{DB ? 1 : 2, NW, NW * (DB ? 2 : 1) * VAR_TILE_BYTES,                     \
               var_solve_pipe_kernel<false, NW, DB>, var_solve_pipe_kernel<true, NW, DB>, NW}
#define VAR_S(NS)                                                                       \
    VarVariant{3, NS, NS * VAR_TILE_BYTES, var_seg_kernel<false, NS>, var_seg_kernel<true, NS>, 1}
static const VarVariant VAR_VARIANTS[] = {
    {0, 4, 0, var_solve_kernel<false, 4>, var_solve_kernel<true, 4>, 4},
    {0, 2, 0, var_solve_kernel<false, 2>, var_solve_kernel<true, 2>, 2},
    VAR_P(1, true), VAR_P(2, true), VAR_P(4, true),
    VAR_P(1, false), VAR_P(2, false), VAR_P(4, false),
    VAR_S(4), VAR_S(8), VAR_S(16)};
#undef VAR_P
#undef VAR_S

constexpr int N_SPOT_VARIANTS = sizeof(SPOT_VARIANTS) / sizeof(SPOT_VARIANTS[0]);
constexpr int N_VAR_VARIANTS = sizeof(VAR_VARIANTS) / sizeof(VAR_VARIANTS[0]);
constexpr int64_t SPOT_MANY_LINES = 150000;
constexpr int MAX_GROUPS = 4;

static int find_spot(int kind, int a, int b) {
    for (int k = 0; k < N_SPOT_VARIANTS; ++k)
        if (SPOT_VARIANTS[k].kind == kind && SPOT_VARIANTS[k].a == a && SPOT_VARIANTS[k].b == b)
            return k;
    return -1;
}
static int find_var(int kind, int warps) {
    for (int k = 0; k < N_VAR_VARIANTS; ++k)
        if (VAR_VARIANTS[k].kind == kind && VAR_VARIANTS[k].warps == warps) return k;
    return -1;
}

// Per-device launch resources, made once: the dynamic shared memory opt-in of
// the kernels above 48 KB, the priority range and the side streams of the
// option groups.
struct DeviceRes {
    bool ready = false;
    int prio_high = 0;
    cudaStream_t side[MAX_GROUPS] = {};
};
static std::mutex g_dev_mu;
static DeviceRes g_dev[64];

static int device_res(DeviceRes *&out) {
    int dev = 0;
    FDADI_CUDA(cudaGetDevice(&dev));
    FDADI_REQUIRE(dev >= 0 && dev < 64, "device ordinal out of range");
    std::lock_guard<std::mutex> g(g_dev_mu);
    DeviceRes &r = g_dev[dev];
    if (!r.ready) {
        for (int k = 0; k < N_VAR_VARIANTS; ++k) {
            const VarVariant &v = VAR_VARIANTS[k];
            if (v.smem > 48 * 1024) {
                FDADI_CUDA(cudaFuncSetAttribute(v.main, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem));
                FDADI_CUDA(cudaFuncSetAttribute(v.impl, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem));
            }
        }
        int lo = 0, hi = 0;
        FDADI_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        r.prio_high = hi;
        for (int g = 0; g < MAX_GROUPS; ++g)
            FDADI_CUDA(cudaStreamCreateWithPriority(&r.side[g], cudaStreamNonBlocking, lo));
        r.ready = true;
    }
    out = &r;
    return FDADI_OK;
}

static fdadi_heston_plan_t default_plan(const Layout &L) {
    fdadi_heston_plan_t p{};
    p.spot_kind = 0;
    p.spot_a = L.SV >= SPOT_MANY_LINES ? 1 : 8;
    p.spot_b = L.SV >= SPOT_MANY_LINES ? 128 : 32;
    p.var_kind = 0;
    p.var_warps = 4;
    p.groups = 1;
    p.expl_per_sm = 0;
    return p;
}

// The index ranges of one option group.
struct GroupSpan {
    Span tiles, lines, tasks;
};

struct Grids {
    int si, vi;       // variant indices
    int corr;         // explicit mode of the corrector stage (ST_HV3, ST_CS3, ST_MCS3)
    int groups;
    int64_t expl_ctas; // explicit-stage blocks (0: one per tile)
    GroupSpan all;
    GroupSpan part[MAX_GROUPS];
    int prio_high;
    cudaStream_t side[MAX_GROUPS];
};

// Options are packed in order, so a group is a contiguous option range and
// its tiles, lines and tasks are contiguous too; groups are cut at the option
// boundaries nearest to equal shares of the grid points.
static GroupSpan span_of(const Layout &L, int o0, int o1) {
    return GroupSpan{{L.tile_off[o0], L.tile_off[o1]}, {L.v_off[o0], L.v_off[o1]},
                     {L.task_off[o0], L.task_off[o1]}};
}

static int grids(const fdadi_heston_batch_t *b, const Layout &L, Grids &g) {
    const fdadi_heston_plan_t p = b->plan ? *b->plan : default_plan(L);
    g.si = find_spot(p.spot_kind, p.spot_a, p.spot_b);
    g.vi = find_var(p.var_kind, p.var_warps);
    FDADI_REQUIRE(g.si >= 0, "unknown spot-solve plan (%d, %d, %d)", p.spot_kind, p.spot_a,
                  p.spot_b);
    FDADI_REQUIRE(g.vi >= 0, "unknown variance-solve plan (%d, %d)", p.var_kind, p.var_warps);
    FDADI_REQUIRE(p.groups >= 0 && p.groups <= MAX_GROUPS, "plan groups must be 0..%d (%d)",
                  MAX_GROUPS, p.groups);
    g.groups = std::max(1, std::min<int>(p.groups, L.n_opt));
    // per-step rebuilds run on the batch's stream between whole steps
    if (b->rates) g.groups = 1;
    g.corr = b->scheme == FDADI_SCHEME_CS ? ST_CS3 : b->scheme == FDADI_SCHEME_MCS ? ST_MCS3 : ST_HV3;
    FDADI_REQUIRE(p.expl_per_sm >= 0 && p.expl_per_sm <= 4,
                  "plan expl_per_sm must be 0..4 (%d)", p.expl_per_sm);
    g.expl_ctas = (int64_t)p.expl_per_sm * sm_count();
    g.all = span_of(L, 0, L.n_opt);
    int o = 0;
    for (int k = 0; k < g.groups; ++k) {
        int o1 = L.n_opt;
        if (k + 1 < g.groups) {
            const int64_t target = L.P * (k + 1) / g.groups;
            o1 = o + 1;
            while (o1 < L.n_opt - (g.groups - 1 - k) && L.p_off[o1] < target) ++o1;
            if (o1 > o + 1 && target - L.p_off[o1 - 1] < L.p_off[o1] - target) --o1;
        }
        g.part[k] = span_of(L, o, o1);
        o = o1;
    }
    DeviceRes *r = nullptr;
    const int rc = device_res(r);
    if (rc) return rc;
    g.prio_high = r->prio_high;
    for (int k = 0; k < MAX_GROUPS; ++k) g.side[k] = r->side[k];
    return FDADI_OK;
}

template <typename... Args>
static void launch_ex(void (*kern)(Args...), unsigned grid, unsigned block, size_t smem,
                      cudaStream_t st, int prio, Args... args) {
    if (grid == 0) return;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = prio;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

// ctas: blocks of the explicit stage (0: one per tile).
static void launch_explicit(int mode, const Span &t, int64_t ctas, const Arena &A, double *V,
                            cudaStream_t st) {
    int64_t n64 = t.hi - t.lo;
    if (ctas > 0) n64 = std::min(n64, ctas);
    const unsigned n = (unsigned)n64;
    if (n == 0) return;
    switch (mode) {
    case ST_DOUGLAS: explicit_kernel<ST_DOUGLAS><<<n, EXPL_THREADS, 0, st>>>(A, V, t.lo, t.hi); break;
    case ST_HV0: explicit_kernel<ST_HV0><<<n, EXPL_THREADS, 0, st>>>(A, V, t.lo, t.hi); break;
    case ST_HV3: explicit_kernel<ST_HV3><<<n, EXPL_THREADS, 0, st>>>(A, V, t.lo, t.hi); break;
    case ST_CS3: explicit_kernel<ST_CS3><<<n, EXPL_THREADS, 0, st>>>(A, V, t.lo, t.hi); break;
    case ST_MCS3: explicit_kernel<ST_MCS3><<<n, EXPL_THREADS, 0, st>>>(A, V, t.lo, t.hi); break;
    default: explicit_kernel<ST_IMPLICIT><<<n, EXPL_THREADS, 0, st>>>(A, V, t.lo, t.hi); break;
    }
}
static void launch_spot(int si, bool implicit, const Span &lines, const Arena &A,
                        const double *src, double *dst, cudaStream_t st, int prio) {
    const SpotVariant &v = SPOT_VARIANTS[si];
    const unsigned grid = (unsigned)((lines.hi - lines.lo + v.lines - 1) / v.lines);
    launch_ex(implicit ? v.impl : v.main, grid, v.threads, 0, st, prio, A, src, dst, lines);
}
static void launch_var(int vi, bool implicit, const Span &tasks, const Arena &A,
                       const double *src, double *dst, cudaStream_t st, int prio) {
    const VarVariant &v = VAR_VARIANTS[vi];
    const unsigned grid = (unsigned)((tasks.hi - tasks.lo + v.tasks - 1) / v.tasks);
    launch_ex(implicit ? v.impl : v.main, grid, v.warps * 32, (size_t)v.smem, st, prio, A, tasks,
              src, dst);
}

// One stage kernel over the whole batch (fdadi_heston_stage).
static void launch_stage(int stage, const Grids &g, const Arena &A, double *V, cudaStream_t st) {
    const GroupSpan &a = g.all;
    switch (stage) {
    case FDADI_STAGE_EXPLICIT_DOUGLAS: launch_explicit(ST_DOUGLAS, a.tiles, g.expl_ctas, A, V, st); break;
    case FDADI_STAGE_EXPLICIT_HV0: launch_explicit(ST_HV0, a.tiles, g.expl_ctas, A, V, st); break;
    case FDADI_STAGE_EXPLICIT_HV3: launch_explicit(g.corr, a.tiles, g.expl_ctas, A, V, st); break;
    case FDADI_STAGE_EXPLICIT_IMPLICIT: launch_explicit(ST_IMPLICIT, a.tiles, g.expl_ctas, A, V, st); break;
    case FDADI_STAGE_SPOT_SOLVE: launch_spot(g.si, false, a.lines, A, A.W, A.W, st, 0); break;
    case FDADI_STAGE_VAR_SOLVE_TO_Y2: launch_var(g.vi, false, a.tasks, A, A.W, A.Y2, st, 0); break;
    case FDADI_STAGE_VAR_SOLVE_TO_V: launch_var(g.vi, false, a.tasks, A, A.W, V, st, 0); break;
    case FDADI_STAGE_VAR_SOLVE_IMPLICIT: launch_var(g.vi, true, a.tasks, A, A.W, A.W, st, 0); break;
    case FDADI_STAGE_SPOT_SOLVE_IMPLICIT: launch_spot(g.si, true, a.lines, A, A.W, V, st, 0); break;
    default: break;
    }
}

// One phase of a time step: an explicit stage and the two line solves after it.
enum PhaseKind : int { PH_IMPLICIT, PH_DOUGLAS, PH_HV_PREDICT, PH_HV_CORRECT };

// The HV corrector's T already holds theta dt A1 Y2 (reference rounding), so
// its spot solve subtracts T with a factor of 1.
static Arena corrector_solve_view(const Grids &g, const Arena &A) {
    Arena B = A;
    if (g.corr == ST_HV3) B.theta = A.one;
    return B;
}

static void launch_phase(int kind, const Grids &g, const GroupSpan &s, const Arena &A, double *V,
                         cudaStream_t st, int prio) {
    switch (kind) {
    case PH_IMPLICIT:
        launch_explicit(ST_IMPLICIT, s.tiles, g.expl_ctas, A, V, st);
        launch_var(g.vi, true, s.tasks, A, A.W, A.W, st, prio);
        launch_spot(g.si, true, s.lines, A, A.W, V, st, prio);
        break;
    case PH_DOUGLAS:
        launch_explicit(ST_DOUGLAS, s.tiles, g.expl_ctas, A, V, st);
        launch_spot(g.si, false, s.lines, A, A.W, A.W, st, prio);
        launch_var(g.vi, false, s.tasks, A, A.W, V, st, prio);
        break;
    case PH_HV_PREDICT:
        launch_explicit(ST_HV0, s.tiles, g.expl_ctas, A, V, st);
        launch_spot(g.si, false, s.lines, A, A.W, A.W, st, prio);
        launch_var(g.vi, false, s.tasks, A, A.W, A.Y2, st, prio);
        break;
    default:
        launch_explicit(g.corr, s.tiles, g.expl_ctas, A, V, st);
        launch_spot(g.si, false, s.lines, corrector_solve_view(g, A), A.W, A.W, st, prio);
        launch_var(g.vi, false, s.tasks, A, A.W, V, st, prio);
        break;
    }
}

// Events of one grouped launch sequence, destroyed with it (after a graph
// capture has ended).
struct EventSet {
    std::vector<cudaEvent_t> ev;
    ~EventSet() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    int make(int n) {
        for (int k = 0; k < n; ++k) {
            cudaEvent_t e;
            FDADI_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ev.push_back(e);
        }
        return FDADI_OK;
    }
};

// The per-option scalars, the per-point operator rows and the spot-line
// factors (everything that depends on r; the spot stencil weights do not).
static int launch_build(const Layout &L, const Arena &A, const BuildArgs &a, cudaStream_t st) {
    build_options_kernel<<<(unsigned)((L.n_opt + 127) / 128), 128, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    build_points_kernel<<<(unsigned)L.n_tiles, EXPL_THREADS, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    build_spot_lines_kernel<<<(unsigned)((L.SV + 127) / 128), 128, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

// Build arguments of this batch; with per-step rates, the builds of `step`.
static BuildArgs build_args(const fdadi_heston_batch_t *b, const Layout &L, int step) {
    BuildArgs a{b->spots, b->vars, b->params, b->dt, b->barrier, b->theta, b->implicit_dt_factor,
                L.smoothing ? 1 : 0, (b->flags & FDADI_HESTON_DROP_ZERO_MIXED) ? 1 : 0,
                L.hv ? 1 : 0};
    if (b->rates) {
        a.rates = b->rates;
        a.rate_stride = (int64_t)b->implicit_steps + b->n_steps;
        a.rate_step = step;
    }
    return a;
}


static void phases_of(const fdadi_heston_batch_t *b, std::vector<int> &ph) {
    for (int s = 0; s < b->implicit_steps; ++s) ph.push_back(PH_IMPLICIT);
    for (int s = 0; s < b->n_steps; ++s) {
        if (b->scheme == FDADI_SCHEME_DOUGLAS) {
            ph.push_back(PH_DOUGLAS);
        } else {
            ph.push_back(PH_HV_PREDICT);
            ph.push_back(PH_HV_CORRECT);
        }
    }
}

// Launch sequence of the time loop (shared by the direct path and the graph
// capture). With one group every launch goes to st in order. With G groups
// the work forks from st onto G side streams and joins back: group k's phases
// run in order on side stream k, and each explicit stage also waits for the
// previous explicit stage of any group, so the FP64-bound stages run one at a
// time while the solves of the group before run beside them.
static int launch_steps(const fdadi_heston_batch_t *b, const Layout &L, const Arena &A, double *V,
                        cudaStream_t st, EventSet &es) {
    Grids g;
    int rc = grids(b, L, g);
    if (rc) return rc;
    std::vector<int> ph;
    phases_of(b, ph);
    if (g.groups == 1) {
        int step = 0;
        for (int kind : ph) {
            // time-dependent coefficients: rebuild before the step's first phase
            if (b->rates && kind != PH_HV_CORRECT) {
                rc = launch_build(L, A, build_args(b, L, step), st);
                if (rc) return rc;
                ++step;
            }
            launch_phase(kind, g, g.all, A, V, st, 0);
        }
        FDADI_CHECK_LAUNCH();
        return FDADI_OK;
    }
    rc = es.make(2 + g.groups);
    if (rc) return rc;
    cudaEvent_t fork = es.ev[0], chain = es.ev[1];
    FDADI_CUDA(cudaEventRecord(fork, st));
    for (int k = 0; k < g.groups; ++k) FDADI_CUDA(cudaStreamWaitEvent(g.side[k], fork, 0));
    bool first = true;
    for (int kind : ph) {
        for (int k = 0; k < g.groups; ++k) {
            cudaStream_t sk = g.side[k];
            if (!first) FDADI_CUDA(cudaStreamWaitEvent(sk, chain, 0));
            // the explicit stage, then (at high priority) the solves
            const GroupSpan &s = g.part[k];
            switch (kind) {
            case PH_IMPLICIT: launch_explicit(ST_IMPLICIT, s.tiles, g.expl_ctas, A, V, sk); break;
            case PH_DOUGLAS: launch_explicit(ST_DOUGLAS, s.tiles, g.expl_ctas, A, V, sk); break;
            case PH_HV_PREDICT: launch_explicit(ST_HV0, s.tiles, g.expl_ctas, A, V, sk); break;
            default: launch_explicit(g.corr, s.tiles, g.expl_ctas, A, V, sk); break;
            }
            FDADI_CUDA(cudaEventRecord(chain, sk));
            first = false;
            switch (kind) {
            case PH_IMPLICIT:
                launch_var(g.vi, true, s.tasks, A, A.W, A.W, sk, g.prio_high);
                launch_spot(g.si, true, s.lines, A, A.W, V, sk, g.prio_high);
                break;
            case PH_DOUGLAS:
                launch_spot(g.si, false, s.lines, A, A.W, A.W, sk, g.prio_high);
                launch_var(g.vi, false, s.tasks, A, A.W, V, sk, g.prio_high);
                break;
            case PH_HV_PREDICT:
                launch_spot(g.si, false, s.lines, A, A.W, A.W, sk, g.prio_high);
                launch_var(g.vi, false, s.tasks, A, A.W, A.Y2, sk, g.prio_high);
                break;
            default:
                launch_spot(g.si, false, s.lines, corrector_solve_view(g, A), A.W, A.W, sk,
                            g.prio_high);
                launch_var(g.vi, false, s.tasks, A, A.W, V, sk, g.prio_high);
                break;
            }
        }
    }
    for (int k = 0; k < g.groups; ++k) {
        FDADI_CUDA(cudaEventRecord(es.ev[2 + k], g.side[k]));
        FDADI_CUDA(cudaStreamWaitEvent(st, es.ev[2 + k], 0));
    }
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

// Instantiated graphs of the time loop, keyed by everything the launches
// capture (workspace, state pointer, schedule, launch geometry, plan).
struct GraphKey {
    const void *ws; const void *V; int n_opt, scheme, n_steps, smoothing;
    int64_t P, SS, SV, n_tiles, n_vtasks;
    int si, vi, groups;
    const void *rates;
    bool operator==(const GraphKey &o) const {
        return ws == o.ws && V == o.V && n_opt == o.n_opt && scheme == o.scheme && rates == o.rates &&
               n_steps == o.n_steps && smoothing == o.smoothing && P == o.P && SS == o.SS &&
               SV == o.SV && n_tiles == o.n_tiles && n_vtasks == o.n_vtasks && si == o.si &&
               vi == o.vi && groups == o.groups;
    }
};
struct GraphKeyHash {
    size_t operator()(const GraphKey &k) const {
        return std::hash<const void *>()(k.ws) ^ (std::hash<const void *>()(k.V) << 1) ^
               ((size_t)k.n_steps << 7) ^ ((size_t)k.n_opt << 19) ^ ((size_t)k.P << 3) ^
               ((size_t)(k.si * 8 + k.vi) << 11) ^ ((size_t)k.groups << 13);
    }
};
static std::mutex g_graph_mu;
static std::unordered_map<GraphKey, cudaGraphExec_t, GraphKeyHash> g_graphs;

static int check_ws(const Layout &L, void *ws, int64_t bytes) {
    FDADI_REQUIRE(ws != nullptr, "null workspace");
    if (bytes < L.bytes) {
        set_error("workspace too small: %lld < %lld bytes", (long long)bytes, (long long)L.bytes);
        return FDADI_E_WORKSPACE;
    }
    return FDADI_OK;
}

}  // namespace fdadi

using namespace fdadi;

extern "C" {

int64_t fdadi_heston_workspace_bytes(const fdadi_heston_batch_t *batch) {
    Layout L;
    if (make_layout(batch, L)) return -1;
    return L.bytes;
}

int64_t fdadi_heston_launch_count(const fdadi_heston_batch_t *b) {
    if (!b) return -1;
    int64_t groups = 1;
    if (b->plan && b->plan->groups > 1 && !b->rates)
        groups = std::min<int64_t>(std::min(b->plan->groups, MAX_GROUPS), b->n_options);
    // time-dependent coefficients: three build launches before every step
    const int64_t rebuild = b->rates ? (int64_t)3 * (b->implicit_steps + b->n_steps) : 0;
    return rebuild + groups * ((int64_t)3 * b->implicit_steps +
                               (int64_t)b->n_steps * (b->scheme == FDADI_SCHEME_DOUGLAS ? 3 : 6));
}

int fdadi_heston_prepare(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes,
                         void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(b->spots && b->vars && b->params && b->dt, "null mesh/params/dt pointer");
    cudaStream_t st = as_stream(stream);
    char *ws = (char *)workspace;
    // host tables (flags are completed on the device)
    std::vector<int> n0(L.n_opt), n1(L.n_opt), flags(L.n_opt, 0), lineS(L.SV);
    std::vector<int4> tiles, vtasks;
    tiles.reserve(L.n_tiles);
    vtasks.reserve(L.n_vtasks);
    std::vector<double> theta(L.n_opt, b->theta);
    for (int k = 0; k < L.n_opt; ++k) {
        n0[k] = b->n0[k];
        n1[k] = b->n1[k];
        for (int64_t j = L.v_off[k]; j < L.v_off[k + 1]; ++j) lineS[j] = k;
        for (int i0 = 0; i0 < n0[k]; i0 += TI)
            for (int j0 = 0; j0 < n1[k]; j0 += TJ) tiles.push_back(make_int4(k, i0, j0, 0));
        for (int i0 = 0; i0 < n0[k]; i0 += 32)
            vtasks.push_back(make_int4(k, i0, std::min(32, n0[k] - i0), 0));
    }
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_n0, n0.data(), 4 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_n1, n1.data(), 4 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_flags, flags.data(), 4 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_p, L.p_off.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_s, L.s_off.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_v, L.v_off.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_lineS, lineS.data(), 4 * L.SV, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_tiles, tiles.data(), 16 * tiles.size(), cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_vtasks, vtasks.data(), 16 * vtasks.size(), cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_theta, theta.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemsetAsync(ws + L.o_ostat, 0, 4 * L.n_opt, st));
    Arena A = arena_view(L, ws);
    const BuildArgs a = build_args(b, L, 0);
    build_spot_weights_kernel<<<(unsigned)L.n_opt, 128, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    rc = launch_build(L, A, a, st);
    if (rc) return rc;
    // the host tables must outlive the copies
    FDADI_CUDA(cudaStreamSynchronize(st));
    return FDADI_OK;
}

int fdadi_heston_run(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes, double *V,
                     void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(V != nullptr, "null state");
    cudaStream_t st = as_stream(stream);
    Arena A = arena_view(L, (char *)workspace);
    if (!(b->flags & FDADI_HESTON_GRAPH)) {
        EventSet es;
        return launch_steps(b, L, A, V, st, es);
    }
    FDADI_REQUIRE(st != nullptr, "graph mode needs a non-default stream");
    Grids g;
    rc = grids(b, L, g);
    if (rc) return rc;
    GraphKey key{workspace, V, b->n_options, b->scheme, b->n_steps, b->implicit_steps,
                 L.P, L.SS, L.SV, L.n_tiles, L.n_vtasks, g.si, g.vi, g.groups, b->rates};
    cudaGraphExec_t exec = nullptr;
    {
        std::lock_guard<std::mutex> g(g_graph_mu);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) exec = it->second;
    }
    if (!exec) {
        cudaGraph_t graph;
        EventSet es;
        FDADI_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int lrc = launch_steps(b, L, A, V, st, es);
        cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (lrc) return lrc;
        FDADI_CUDA(ec);
        FDADI_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        cudaGraphDestroy(graph);
        std::lock_guard<std::mutex> g(g_graph_mu);
        g_graphs[key] = exec;
    }
    FDADI_CUDA(cudaGraphLaunch(exec, st));
    return FDADI_OK;
}

int fdadi_heston_stage(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes, double *V,
                       int32_t stage, void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(V != nullptr, "null state");
    FDADI_REQUIRE(stage >= FDADI_STAGE_EXPLICIT_DOUGLAS && stage <= FDADI_STAGE_SPOT_SOLVE_IMPLICIT,
                  "unknown stage %d", stage);
    FDADI_REQUIRE(!(stage == FDADI_STAGE_EXPLICIT_HV0 || stage == FDADI_STAGE_EXPLICIT_HV3 ||
                    stage == FDADI_STAGE_VAR_SOLVE_TO_Y2) || L.hv,
                  "stage %d needs a predictor-corrector (HV or Craig-Sneyd) batch", stage);
    FDADI_REQUIRE(!(stage == FDADI_STAGE_EXPLICIT_IMPLICIT ||
                    stage == FDADI_STAGE_VAR_SOLVE_IMPLICIT ||
                    stage == FDADI_STAGE_SPOT_SOLVE_IMPLICIT) || L.smoothing,
                  "stage %d needs a batch with implicit steps", stage);
    Arena A = arena_view(L, (char *)workspace);
    Grids g;
    rc = grids(b, L, g);
    if (rc) return rc;
    launch_stage(stage, g, A, V, as_stream(stream));
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_heston_payoff(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes,
                        const double *strikes, int32_t put, double *V, void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(strikes && V && b->spots, "null payoff argument");
    Arena A = arena_view(L, (char *)workspace);
    payoff_kernel<<<(unsigned)L.n_tiles, EXPL_THREADS, 0, as_stream(stream)>>>(A, b->spots, strikes,
                                                                               put ? 1 : 0, V);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_heston_status(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes,
                        const double *V, int32_t *status, void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(V != nullptr && status != nullptr, "null state or status array");
    Arena A = arena_view(L, (char *)workspace);
    status_kernel<<<(unsigned)L.n_opt, 256, 0, as_stream(stream)>>>(A, V, status);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_heston_greeks(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes,
                        const double *V, const int64_t *flat_index, double *price, double *delta,
                        double *gamma, void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(V && flat_index && price && delta && gamma && b->spots,
                  "null greeks argument");
    Arena A = arena_view(L, (char *)workspace);
    greeks_kernel<<<(unsigned)((L.n_opt + 127) / 128), 128, 0, as_stream(stream)>>>(
        A, b->spots, V, flat_index, price, delta, gamma);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_heston_default_plan(const fdadi_heston_batch_t *b, fdadi_heston_plan_t *plan) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    FDADI_REQUIRE(plan != nullptr, "null plan");
    *plan = default_plan(L);
    return FDADI_OK;
}

int fdadi_heston_tune(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes,
                      int32_t reps, fdadi_heston_plan_t *plan, void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    rc = check_ws(L, workspace, ws_bytes);
    if (rc) return rc;
    FDADI_REQUIRE(plan != nullptr, "null plan");
    FDADI_REQUIRE(reps >= 1 && reps <= 1000, "reps must be 1..1000 (%d)", reps);
    DeviceRes *res = nullptr;
    rc = device_res(res);
    if (rc) return rc;
    cudaStream_t st = as_stream(stream);
    Arena A = arena_view(L, (char *)workspace);
    cudaEvent_t e0, e1;
    FDADI_CUDA(cudaEventCreate(&e0));
    FDADI_CUDA(cudaEventCreate(&e1));
    // time one variant: a warm-up launch, then reps launches between events
    auto time_it = [&](auto launch, float &ms) -> int {
        launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { ms = -1.0f; return FDADI_OK; }  // shape not launchable here
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps; ++r) launch();
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            set_error("CUDA error while tuning: %s", cudaGetErrorString(e));
            return FDADI_E_CUDA;
        }
        cudaEventElapsedTime(&ms, e0, e1);
        return FDADI_OK;
    };
    fdadi_heston_plan_t best = default_plan(L);
    float best_spot = 1e30f, best_var = 1e30f;
    for (int k = 0; k < N_SPOT_VARIANTS && !rc; ++k) {
        const SpotVariant &v = SPOT_VARIANTS[k];
        const unsigned grid = (unsigned)((L.SV + v.lines - 1) / v.lines);
        float ms = 0.0f;
        const Span lines{0, L.SV};
        rc = time_it([&] { v.main<<<grid, v.threads, 0, st>>>(A, A.W, A.W, lines); }, ms);
        if (!rc && ms >= 0.0f && ms < best_spot) {
            best_spot = ms;
            best.spot_kind = v.kind; best.spot_a = v.a; best.spot_b = v.b;
        }
    }
    for (int k = 0; k < N_VAR_VARIANTS && !rc; ++k) {
        const VarVariant &v = VAR_VARIANTS[k];
        const unsigned grid = (unsigned)((L.n_vtasks + v.tasks - 1) / v.tasks);
        const Span tasks{0, L.n_vtasks};
        float ms = 0.0f;
        rc = time_it([&] { v.main<<<grid, v.warps * 32, v.smem, st>>>(A, tasks, A.W, A.W); }, ms);
        if (!rc && ms >= 0.0f && ms < best_var) {
            best_var = ms;
            best.var_kind = v.kind; best.var_warps = v.warps;
        }
    }
    if (!rc && (best_spot >= 1e30f || best_var >= 1e30f)) {
        set_error("no launch plan could be launched");
        rc = FDADI_E_CUDA;
    }
    // option groups: two main steps per choice on a zeroed scratch state (the
    // stages' cost does not depend on the values)
    double *scratch = nullptr;
    if (!rc && L.n_opt > 1) {
        cudaError_t e = cudaMallocAsync((void **)&scratch, (size_t)L.P * sizeof(double), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, (size_t)L.P * sizeof(double), st);
        if (e != cudaSuccess) {
            set_error("tune scratch: %s", cudaGetErrorString(e));
            rc = FDADI_E_CUDA;
        }
        fdadi_heston_batch_t tb = *b;
        tb.n_steps = 2;
        tb.implicit_steps = 0;
        tb.flags &= ~FDADI_HESTON_GRAPH;
        float best_g = 1e30f;
        const fdadi_heston_plan_t base = best;
        for (int c = 0; c < 4 * 3 && !rc; ++c) {
            const int G = 1 + c / 3, X = (c % 3 == 0) ? 0 : 1 + c % 3;  // X: 0, 2, 3 per SM
            if (G > L.n_opt) break;
            fdadi_heston_plan_t cand = base;
            cand.groups = G;
            cand.expl_per_sm = X;
            tb.plan = &cand;
            float ms = 0.0f;
            int lrc = FDADI_OK;
            rc = time_it([&] {
                EventSet es;
                const int r2 = launch_steps(&tb, L, A, scratch, st, es);
                if (r2) lrc = r2;
            }, ms);
            if (!rc && lrc) rc = lrc;
            // anything but the plain schedule must win by 2%
            if (!rc && ms >= 0.0f && (c == 0 ? ms < best_g : ms < best_g * 0.98f)) {
                best_g = ms;
                best.groups = G;
                best.expl_per_sm = X;
            }
        }
        if (scratch) cudaFreeAsync(scratch, st);
        cudaError_t e2 = cudaStreamSynchronize(st);
        if (!rc && e2 != cudaSuccess) {
            set_error("CUDA error while tuning: %s", cudaGetErrorString(e2));
            rc = FDADI_E_CUDA;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *plan = best;
    return FDADI_OK;
}

int fdadi_fp64_probe(double *out, int32_t blocks, int32_t threads, int32_t iters,
                     int32_t chains, double *flops, void *stream) {
    FDADI_REQUIRE(out && blocks > 0 && threads > 0 && threads <= 1024 && iters > 0,
                  "bad probe arguments");
    cudaStream_t st = as_stream(stream);
    switch (chains) {
    case 1: fp64_probe_kernel<1><<<blocks, threads, 0, st>>>(out, iters); break;
    case 2: fp64_probe_kernel<2><<<blocks, threads, 0, st>>>(out, iters); break;
    case 4: fp64_probe_kernel<4><<<blocks, threads, 0, st>>>(out, iters); break;
    case 8: fp64_probe_kernel<8><<<blocks, threads, 0, st>>>(out, iters); break;
    case 16: fp64_probe_kernel<16><<<blocks, threads, 0, st>>>(out, iters); break;
    default: FDADI_REQUIRE(false, "probe chains must be 1, 2, 4, 8 or 16 (got %d)", (int)chains);
    }
    FDADI_CHECK_LAUNCH();
    if (flops) *flops = 2.0 * (double)chains * (double)blocks * threads * (double)iters;
    return FDADI_OK;
}

int fdadi_gather(const double *V, const int64_t *idx, double *out, int64_t n, void *stream) {
    FDADI_REQUIRE(V && idx && out && n >= 0, "bad gather arguments");
    if (n == 0) return FDADI_OK;
    gather_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(V, idx, out, n);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

}  // extern "C"
