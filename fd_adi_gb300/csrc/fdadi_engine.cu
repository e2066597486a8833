// Fused, batched Heston ADI engine.
//
// A batch of options with independent (uneven) grids lives in one packed
// arena: option k owns points [p_off[k], p_off[k] + n0*n1) of every per-point
// array, rows [s_off[k], s_off[k] + n0) of every per-spot-index array and
// columns [v_off[k], v_off[k] + n1) of every per-variance-index array. Each
// time step is a short chain of launches over the whole batch:
//
//   explicit stage  -- one thread per grid point: the three operator applies
//                      of F(V) (spot, variance, mixed) fused with the scheme's
//                      combination, writing the next right-hand side;
//   spot solve      -- one thread per spot line (grid column); adjacent
//                      threads read adjacent columns, so the strided
//                      direction is coalesced without a transpose;
//   variance solve  -- one thread per variance line (grid row).
//
// Line solves use Thomas factors precomputed once per (dt, theta): the
// operators are time independent (FiniteDifferenceEngineGPU.pyx:163-167), so
// every step costs two FMAs and a multiply per point per solve and no
// division. Operators are built on the device with the reference's
// arithmetic order (explicitly rounded intrinsics, no FMA contraction), so
// they equal the reference CPU engine's bit for bit.
#include <algorithm>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "fdadi_internal.cuh"

namespace fdadi {

#define MUL(a, b) __dmul_rn((a), (b))
#define ADD(a, b) __dadd_rn((a), (b))
#define SUB(a, b) __dsub_rn((a), (b))
#define DIV(a, b) __ddiv_rn((a), (b))

enum : int { OPT_S_LOW_DIR = 1, OPT_S_HIGH_DIR = 2, OPT_MIXED = 4 };

constexpr int EXPL_TILE = 256;
constexpr int SOLVE_THREADS = 128;

// Device view of a prepared workspace.
struct Arena {
    int n_opt;
    int64_t P, SS, SV;        // total points, total spot indices, total variance indices
    // tables
    const int *n0, *n1, *oflags;
    const int64_t *p_off, *s_off, *v_off;
    const int *lineS, *lineV;  // option of each spot line (grid column) / variance line (grid row)
    const int2 *tiles;         // (option, first point) of each explicit tile
    // main plan (dt, theta)
    double *F0, *R0, *F1, *R1, *F1x, *cM, *w0, *w1, *LS, *LV, *foldV, *dirS;
    // implicit plan (dt/2, theta = 1, residual kept)
    double *cMi, *RSi, *RVi, *LSi, *LVi, *foldVi;
    // stage buffers
    double *Y0, *W, *T, *Y2;
    const double *theta;       // [n_opt]
};

// ---- operator rows (reference construction) ------------------------------

struct Row3 {
    double sub, mid, sup, R, ext;  // ext: A[n-1, n-3] on the last row of a variance line
    bool dirichlet;
};

// Centred non-uniform stencil of row i (1 <= i <= n-2), centercoeffs
// (BandedOperator.pyx:970-1017).
__device__ __forceinline__ void centre(const double *x, int i, int derivative, double &sub,
                                       double &mid, double &sup) {
    const double di = SUB(x[i], x[i - 1]), dn = SUB(x[i + 1], x[i]);
    const double s = ADD(di, dn);
    if (derivative == 1) {
        sup = DIV(di, MUL(dn, s));
        mid = DIV(ADD(-di, dn), MUL(di, dn));
        sub = DIV(-dn, MUL(di, s));
    } else {
        sup = DIV(2.0, MUL(dn, s));
        mid = DIV(-2.0, MUL(di, dn));
        sub = DIV(2.0, MUL(di, s));
    }
}

// Combined spot operator A0 = r S D_S + 1/2 v S^2 D_SS - r/2 at row i of the
// spot line through variance v_j: boundaries heston.py:337-342 (Dirichlet
// U = 0 at S = 0, dU/dS = 1 at S_max) or the up-and-out Dirichlet row at S_max
// (heston.py:361-370); combination FiniteDifferenceEngine.pyx:563-592.
__device__ Row3 spot_row(const double *S, int n, int i, double vj, double r, float half_r,
                         bool barrier) {
    Row3 o{0.0, 0.0, 0.0, 0.0, 0.0, false};
    if (i == 0 || (i == n - 1 && barrier)) {
        o.mid = 1.0;
        o.dirichlet = true;
        return o;
    }
    const double f = (double)half_r;
    const double c0 = MUL(r, S[i]);
    const double c00 = MUL(MUL(0.5, vj), MUL(S[i], S[i]));
    if (i == n - 1) {
        const double dm1 = SUB(S[n - 1], S[n - 2]);
        const double xx = MUL(dm1, dm1);
        const double mid2 = DIV(-2.0, xx), sub2 = DIV(2.0, xx);
        const double R2 = DIV(MUL(1.0, 2.0), dm1);
        o.mid = ADD(ADD(MUL(0.0, c0), f), MUL(mid2, c00));
        o.sub = ADD(MUL(0.0, c0), MUL(sub2, c00));
        o.sup = 0.0;
        o.R = ADD(MUL(1.0, c0), MUL(R2, c00));
        return o;
    }
    double s1, m1, p1, s2, m2, p2;
    centre(S, i, 1, s1, m1, p1);
    centre(S, i, 2, s2, m2, p2);
    o.sup = ADD(MUL(p1, c0), MUL(p2, c00));
    o.mid = ADD(ADD(MUL(m1, c0), f), MUL(m2, c00));
    o.sub = ADD(MUL(s1, c0), MUL(s2, c00));
    return o;
}

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
};

__device__ __forceinline__ void opt_params(const BuildArgs &a, int o, double &r, double &kappa,
                                           double &th, double &sigma, double &rho) {
    const double *p = a.params + 5 * (int64_t)o;
    r = p[0]; kappa = p[1]; th = p[2]; sigma = p[3]; rho = p[4];
}

// Per point: scaled explicit operators (Firsts = A * dt), mixed coefficient,
// residuals of the implicit plan; per line/index: stencil weights, extras,
// Dirichlet values.
__global__ void build_points_kernel(Arena A, BuildArgs a) {
    const int2 t = A.tiles[blockIdx.x];
    const int o = t.x;
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int64_t N = (int64_t)n0 * n1;
    const int64_t pl = (int64_t)t.y + threadIdx.x;
    if (pl >= N) return;
    const int i = (int)(pl / n1), j = (int)(pl - (int64_t)i * n1);
    const int64_t p = A.p_off[o] + pl, P = A.P;
    const double *S = a.spots + A.s_off[o], *v = a.vars + A.v_off[o];
    double r, kappa, th, sigma, rho;
    opt_params(a, o, r, kappa, th, sigma, rho);
    const float half_r = (float)(-r / 2.0);   // add_scalar takes a C float (BandedOperator.pxd:32)
    const bool barrier = a.barrier && a.barrier[o];
    const double dt = a.dt[o];

    const Row3 s = spot_row(S, n0, i, v[j], r, half_r, barrier);
    if (s.dirichlet) {  // Dirichlet rows are not scaled (BandedOperator.pyx:771-779)
        A.F0[p] = 0.0; A.F0[P + p] = 1.0; A.F0[2 * P + p] = 0.0; A.R0[p] = s.R;
    } else {
        A.F0[p] = MUL(s.sub, dt); A.F0[P + p] = MUL(s.mid, dt); A.F0[2 * P + p] = MUL(s.sup, dt);
        A.R0[p] = MUL(s.R, dt);
    }
    const Row3 w = var_row(v, n1, j, S[i], r, half_r, kappa, th, sigma);
    A.F1[p] = MUL(w.sub, dt); A.F1[P + p] = MUL(w.mid, dt); A.F1[2 * P + p] = MUL(w.sup, dt);
    A.R1[p] = MUL(w.R, dt);
    if (j == n1 - 1) A.F1x[A.s_off[o] + i] = MUL(w.ext, dt);
    const double c = MUL(MUL(MUL(rho, sigma), S[i]), v[j]);
    A.cM[p] = MUL(c, dt);
    if (a.smoothing) {
        const double dti = MUL(dt, a.dt_factor);
        A.cMi[p] = MUL(c, dti);
        A.RSi[p] = s.dirichlet ? s.R : MUL(s.R, -dti);
        A.RVi[p] = MUL(w.R, -dti);
    }
    if (j == 0) {  // spot stencil weights (centred first derivative, rows 0 and n0-1 zero)
        double sb = 0.0, md = 0.0, sp = 0.0;
        if (i > 0 && i < n0 - 1) centre(S, i, 1, sb, md, sp);
        const int64_t q = A.s_off[o] + i;
        A.w0[q] = sb; A.w0[A.SS + q] = md; A.w0[2 * A.SS + q] = sp;
    }
    if (i == 0) {  // variance stencil weights; Dirichlet values of the spot lines (U = 0)
        double sb = 0.0, md = 0.0, sp = 0.0;
        if (j > 0 && j < n1 - 1) centre(v, j, 1, sb, md, sp);
        const int64_t q = A.v_off[o] + j;
        A.w1[q] = sb; A.w1[A.SV + q] = md; A.w1[2 * A.SV + q] = sp;
        A.dirS[q] = 0.0;
        A.dirS[A.SV + q] = 0.0;
    }
}

// Thomas factors (a_k, 1/m_k, c'_k) of one line with rows (sub, mid, sup):
// m_0 = mid_0, m_k = mid_k - sub_k c'_{k-1}, c'_k = sup_k / m_k.
struct Thomas {
    double cp = 0.0;
    __device__ __forceinline__ void row(double *L, int64_t P, int64_t p, double sub, double mid,
                                        double sup, bool first) {
        const double m = first ? mid : mid - sub * cp;
        const double inv = 1.0 / m;
        cp = sup * inv;
        L[p] = sub;
        L[P + p] = inv;
        L[2 * P + p] = cp;
    }
};

// Spot lines: factors of Li0 = 1 - theta dt A0 (main) and 1 - dt/2 A0 (implicit).
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
    Thomas tm, ti;
    for (int i = 0; i < n0; ++i) {
        const int64_t p = A.p_off[o] + (int64_t)i * n1 + j;
        const Row3 s = spot_row(S, n0, i, v[j], r, half_r, barrier);
        double sb = 0.0, md = 1.0, sp = 0.0;
        if (!s.dirichlet) { sb = MUL(s.sub, sm); md = ADD(MUL(s.mid, sm), 1.0); sp = MUL(s.sup, sm); }
        tm.row(A.LS, A.P, p, sb, md, sp, i == 0);
        if (a.smoothing) {
            sb = 0.0; md = 1.0; sp = 0.0;
            if (!s.dirichlet) { sb = MUL(s.sub, si); md = ADD(MUL(s.mid, si), 1.0); sp = MUL(s.sup, si); }
            ti.row(A.LSi, A.P, p, sb, md, sp, i == 0);
        }
    }
}

// Variance lines: Li1 folded at the bottom (BandedOperator.pyx:223-256) and
// factorised; the fold factor is kept for the right-hand side.
__device__ void var_line_factor(const Arena &A, int o, int i, const double *v, int n1, double Si,
                                double r, float half_r, double kappa, double th, double sigma,
                                double scale, double *L, double *fold) {
    const int64_t base = A.p_off[o] + (int64_t)i * n1;
    // rows n1-2 and n1-1 are needed before the last row is factorised
    const Row3 a2 = var_row(v, n1, n1 - 2, Si, r, half_r, kappa, th, sigma);
    const Row3 a1 = var_row(v, n1, n1 - 1, Si, r, half_r, kappa, th, sigma);
    const double an1 = MUL(a2.sub, scale), bn1 = ADD(MUL(a2.mid, scale), 1.0),
                 cn1 = MUL(a2.sup, scale);
    const double zn = MUL(a1.ext, scale);
    double an = MUL(a1.sub, scale), bn = ADD(MUL(a1.mid, scale), 1.0);
    const double f = an1 != 0.0 ? DIV(-zn, an1) : 0.0;
    an = ADD(an, MUL(bn1, f));
    bn = ADD(bn, MUL(cn1, f));
    fold[A.s_off[o] + i] = f;
    Thomas t;
    for (int j = 0; j < n1 - 1; ++j) {
        const Row3 w = var_row(v, n1, j, Si, r, half_r, kappa, th, sigma);
        t.row(L, A.P, base + j, MUL(w.sub, scale), ADD(MUL(w.mid, scale), 1.0), MUL(w.sup, scale),
              j == 0);
    }
    t.row(L, A.P, base + n1 - 1, an, bn, 0.0, false);
}

__global__ void build_var_lines_kernel(Arena A, BuildArgs a) {
    const int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= A.SS) return;
    const int o = A.lineV[line];
    const int n1 = A.n1[o];
    const int i = (int)(line - A.s_off[o]);
    const double *S = a.spots + A.s_off[o], *v = a.vars + A.v_off[o];
    double r, kappa, th, sigma, rho;
    opt_params(a, o, r, kappa, th, sigma, rho);
    const float half_r = (float)(-r / 2.0);
    const double dt = a.dt[o];
    var_line_factor(A, o, i, v, n1, S[i], r, half_r, kappa, th, sigma, MUL(a.theta, -dt), A.LV,
                    A.foldV);
    if (a.smoothing)
        var_line_factor(A, o, i, v, n1, S[i], r, half_r, kappa, th, sigma, -MUL(dt, a.dt_factor),
                        A.LVi, A.foldVi);
}

// ---- stage kernels --------------------------------------------------------

enum : int { ST_DOUGLAS = 0, ST_HV0 = 1, ST_HV3 = 2, ST_IMPLICIT = 3 };

// Grid-point accessor with the spot operator's forced Dirichlet rows.
struct OptView {
    int n0, n1, flags;
    int64_t p0;      // first point of the option
    int64_t sv;      // v_off: first spot-line index
    int64_t ss;      // s_off
};

template <int MODE>
__global__ void __launch_bounds__(EXPL_TILE) explicit_kernel(Arena A, const double *__restrict__ V) {
    const int2 t = A.tiles[blockIdx.x];
    const int o = t.x;
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int64_t N = (int64_t)n0 * n1;
    const int64_t pl = (int64_t)t.y + threadIdx.x;
    if (pl >= N) return;
    const int i = (int)(pl / n1), j = (int)(pl - (int64_t)i * n1);
    const int64_t P = A.P, p0 = A.p_off[o], p = p0 + pl;
    const int fl = A.oflags[o];
    const bool slow = fl & OPT_S_LOW_DIR, shigh = fl & OPT_S_HIGH_DIR, mixed = fl & OPT_MIXED;
    const int64_t js = A.v_off[o] + j;
    const double gl = A.dirS[js], gh = A.dirS[A.SV + js];
    const double *Vo = V + p0;

    // F0 x: spot operator along the column through (i, j), forced Dirichlet rows
    auto spot_apply = [&](auto X) -> double {
        if (i == 0 && slow) return gl;
        if (i == n0 - 1 && shigh) return gh;
        auto xs = [&](int ii) -> double {
            if (ii == 0 && slow) return gl;
            if (ii == n0 - 1 && shigh) return gh;
            return X((int64_t)ii * n1 + j);
        };
        double acc = 0.0;
        if (i + 1 < n0) acc += A.F0[2 * P + p] * xs(i + 1);
        acc += A.F0[P + p] * xs(i);
        if (i > 0) acc += A.F0[p] * xs(i - 1);
        return acc;
    };
    // F1 x: variance operator along the row through (i, j)
    auto var_apply = [&](auto X) -> double {
        const int64_t b = (int64_t)i * n1;
        double acc = 0.0;
        if (j + 1 < n1) acc += A.F1[2 * P + p] * X(b + j + 1);
        acc += A.F1[P + p] * X(b + j);
        if (j > 0) acc += A.F1[p] * X(b + j - 1);
        if (j == n1 - 1) acc += A.F1x[A.s_off[o] + i] * X(b + n1 - 3);
        return acc;
    };
    // M x: c * sum_a w0[a](i) sum_b w1[b](j) x(i+a, j+b), zero on the edges
    auto mixed_apply = [&](auto X, const double *c) -> double {
        if (!mixed || i == 0 || i == n0 - 1 || j == 0 || j == n1 - 1) return 0.0;
        const int64_t si = A.s_off[o] + i, vj = A.v_off[o] + j;
        const double b0 = A.w1[vj], b1 = A.w1[A.SV + vj], b2 = A.w1[2 * A.SV + vj];
        const int64_t q = (int64_t)i * n1 + j;
        const double tm = b0 * X(q - n1 - 1) + b1 * X(q - n1) + b2 * X(q - n1 + 1);
        const double tc = b0 * X(q - 1) + b1 * X(q) + b2 * X(q + 1);
        const double tp = b0 * X(q + n1 - 1) + b1 * X(q + n1) + b2 * X(q + n1 + 1);
        return c[p] * (A.w0[si] * tm + A.w0[A.SS + si] * tc + A.w0[2 * A.SS + si] * tp);
    };
    auto Xv = [&](int64_t q) -> double { return __ldg(Vo + q); };

    if (MODE == ST_IMPLICIT) {
        A.W[p] = Vo[pl] + mixed_apply(Xv, A.cMi);
        return;
    }
    const double theta = A.theta[o];
    if (MODE == ST_DOUGLAS || MODE == ST_HV0) {
        const double a0 = spot_apply(Xv), a1 = var_apply(Xv), m = mixed_apply(Xv, A.cM);
        const double y = Vo[pl] + (a0 + A.R0[p]) + (a1 + A.R1[p]) + m;
        if (MODE == ST_HV0) A.Y0[p] = y;
        A.W[p] = y - theta * a0;
        A.T[p] = theta * a1;
        return;
    }
    // ST_HV3: W = Y0 - F(V - Y2)/2 (no residual) - theta F0 Y2; T = theta F1 Y2
    const double *Y2o = A.Y2 + p0;
    auto Xd = [&](int64_t q) -> double { return __ldg(Vo + q) - __ldg(Y2o + q); };
    auto Xy = [&](int64_t q) -> double { return __ldg(Y2o + q); };
    const double d = spot_apply(Xd) + var_apply(Xd) + mixed_apply(Xd, A.cM);
    const double ay0 = spot_apply(Xy), ay1 = var_apply(Xy);
    A.W[p] = A.Y0[p] - 0.5 * d - theta * ay0;
    A.T[p] = theta * ay1;
}

// Spot-line solve, one thread per grid column. src -> dst (may alias).
// RESID: subtract the implicit plan's residual. SUBT: write x - T (the next
// stage's right-hand side) instead of x.
template <bool IMPLICIT, bool SUBT>
__global__ void __launch_bounds__(SOLVE_THREADS) spot_solve_kernel(Arena A, const double *src,
                                                                   double *dst) {
    const int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= A.SV) return;
    const int o = A.lineS[line];
    const int n0 = A.n0[o], n1 = A.n1[o];
    const int64_t js = line, j = line - A.v_off[o];
    const int fl = A.oflags[o];
    const bool slow = fl & OPT_S_LOW_DIR, shigh = fl & OPT_S_HIGH_DIR;
    const int64_t P = A.P, b = A.p_off[o] + j;
    const double *L = IMPLICIT ? A.LSi : A.LS;
    const double gl = A.dirS[js], gh = A.dirS[A.SV + js];
    double dp = 0.0;
    for (int i = 0; i < n0; ++i) {
        const int64_t p = b + (int64_t)i * n1;
        double rk;
        if (i == 0 && slow) rk = gl;
        else if (i == n0 - 1 && shigh) rk = gh;
        else rk = src[p];
        if (IMPLICIT) rk = rk - A.RSi[p];
        dp = (i == 0) ? rk * L[P + p] : (rk - L[p] * dp) * L[P + p];
        dst[p] = dp;
    }
    double x = dp;
    {
        const int64_t p = b + (int64_t)(n0 - 1) * n1;
        if (SUBT) dst[p] = x - A.T[p];
    }
    for (int i = n0 - 2; i >= 0; --i) {
        const int64_t p = b + (int64_t)i * n1;
        x = dst[p] - L[2 * P + p] * x;
        dst[p] = SUBT ? x - A.T[p] : x;
    }
}

// Variance-line solve, one thread per grid row; the bottom row of the
// right-hand side is folded with the line's fold factor.
template <bool IMPLICIT>
__global__ void __launch_bounds__(SOLVE_THREADS) var_solve_kernel(Arena A, const double *src,
                                                                  double *dst) {
    const int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= A.SS) return;
    const int o = A.lineV[line];
    const int n1 = A.n1[o];
    const int64_t i = line - A.s_off[o];
    const int64_t P = A.P, b = A.p_off[o] + i * n1;
    const double *L = IMPLICIT ? A.LVi : A.LV;
    const double f = IMPLICIT ? A.foldVi[line] : A.foldV[line];
    double dp = 0.0, rprev = 0.0;
    for (int j = 0; j < n1; ++j) {
        const int64_t p = b + j;
        double rk = src[p];
        if (IMPLICIT) rk = rk - A.RVi[p];
        const double raw = rk;
        if (j == n1 - 1) rk += 1.0 * rprev * f;
        dp = (j == 0) ? rk * L[P + p] : (rk - L[p] * dp) * L[P + p];
        dst[p] = dp;
        rprev = raw;
    }
    double x = dp;
    for (int j = n1 - 2; j >= 0; --j) {
        const int64_t p = b + j;
        x = dst[p] - L[2 * P + p] * x;
        dst[p] = x;
    }
}

// Eight independent DFMA chains per thread: measures the FP64 pipe, not latency.
__global__ void fp64_probe_kernel(double *out, int iters) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * (t + k);
    const double b = 0.999999999, c = 1e-9;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
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
    int64_t P = 0, SS = 0, SV = 0, n_tiles = 0;
    bool smoothing = false;
    // byte offsets into the workspace
    int64_t o_n0, o_n1, o_flags, o_p, o_s, o_v, o_lineS, o_lineV, o_tiles, o_theta;
    int64_t o_F0, o_R0, o_F1, o_R1, o_F1x, o_cM, o_w0, o_w1, o_LS, o_LV, o_foldV, o_dirS;
    int64_t o_cMi, o_RSi, o_RVi, o_LSi, o_LVi, o_foldVi;
    int64_t o_Y0, o_W, o_T, o_Y2;
    int64_t bytes = 0;
    std::vector<int64_t> p_off, s_off, v_off;
};

static int make_layout(const fdadi_heston_batch_t *b, Layout &L) {
    FDADI_REQUIRE(b != nullptr, "null batch");
    FDADI_REQUIRE(b->n_options > 0, "empty batch");
    FDADI_REQUIRE(b->n0 && b->n1, "batch needs host size arrays n0, n1");
    FDADI_REQUIRE(b->scheme == FDADI_SCHEME_DOUGLAS || b->scheme == FDADI_SCHEME_HV,
                  "main scheme must be Douglas or Hundsdorfer-Verwer");
    FDADI_REQUIRE(b->n_steps >= 0 && b->implicit_steps >= 0, "negative step count");
    FDADI_REQUIRE(b->implicit_steps == 0 || b->implicit_dt_factor > 0.0,
                  "implicit_dt_factor must be positive");
    L.n_opt = b->n_options;
    L.smoothing = b->implicit_steps > 0;
    L.p_off.resize(L.n_opt + 1);
    L.s_off.resize(L.n_opt + 1);
    L.v_off.resize(L.n_opt + 1);
    L.p_off[0] = L.s_off[0] = L.v_off[0] = 0;
    for (int k = 0; k < L.n_opt; ++k) {
        FDADI_REQUIRE(b->n0[k] >= 4 && b->n1[k] >= 4,
                      "Vector too short to use finite differencing (option %d: %d x %d)", k,
                      b->n0[k], b->n1[k]);
        const int64_t N = (int64_t)b->n0[k] * b->n1[k];
        L.p_off[k + 1] = L.p_off[k] + N;
        L.s_off[k + 1] = L.s_off[k] + b->n0[k];
        L.v_off[k + 1] = L.v_off[k] + b->n1[k];
        L.n_tiles += (N + EXPL_TILE - 1) / EXPL_TILE;
    }
    L.P = L.p_off[L.n_opt];
    L.SS = L.s_off[L.n_opt];
    L.SV = L.v_off[L.n_opt];
    FDADI_REQUIRE(L.n_tiles < (int64_t)1 << 31, "batch too large");
    int64_t off = 0;
    auto take = [&](int64_t bytes) { int64_t o = off; off = align256(off + bytes); return o; };
    const int64_t D = sizeof(double);
    L.o_n0 = take(4 * L.n_opt); L.o_n1 = take(4 * L.n_opt); L.o_flags = take(4 * L.n_opt);
    L.o_p = take(8 * L.n_opt); L.o_s = take(8 * L.n_opt); L.o_v = take(8 * L.n_opt);
    L.o_lineS = take(4 * L.SV); L.o_lineV = take(4 * L.SS); L.o_tiles = take(8 * L.n_tiles);
    L.o_theta = take(D * L.n_opt);
    L.o_F0 = take(3 * D * L.P); L.o_R0 = take(D * L.P); L.o_F1 = take(3 * D * L.P);
    L.o_R1 = take(D * L.P); L.o_F1x = take(D * L.SS); L.o_cM = take(D * L.P);
    L.o_w0 = take(3 * D * L.SS); L.o_w1 = take(3 * D * L.SV);
    L.o_LS = take(3 * D * L.P); L.o_LV = take(3 * D * L.P); L.o_foldV = take(D * L.SS);
    L.o_dirS = take(2 * D * L.SV);
    if (L.smoothing) {
        L.o_cMi = take(D * L.P); L.o_RSi = take(D * L.P); L.o_RVi = take(D * L.P);
        L.o_LSi = take(3 * D * L.P); L.o_LVi = take(3 * D * L.P); L.o_foldVi = take(D * L.SS);
    } else {
        L.o_cMi = L.o_RSi = L.o_RVi = L.o_LSi = L.o_LVi = L.o_foldVi = -1;
    }
    L.o_W = take(D * L.P); L.o_T = take(D * L.P);
    if (b->scheme == FDADI_SCHEME_HV) { L.o_Y0 = take(D * L.P); L.o_Y2 = take(D * L.P); }
    else L.o_Y0 = L.o_Y2 = -1;
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
    A.lineS = (const int *)(ws + L.o_lineS); A.lineV = (const int *)(ws + L.o_lineV);
    A.tiles = (const int2 *)(ws + L.o_tiles);
    A.theta = ptr(L.o_theta);
    A.F0 = ptr(L.o_F0); A.R0 = ptr(L.o_R0); A.F1 = ptr(L.o_F1); A.R1 = ptr(L.o_R1);
    A.F1x = ptr(L.o_F1x); A.cM = ptr(L.o_cM); A.w0 = ptr(L.o_w0); A.w1 = ptr(L.o_w1);
    A.LS = ptr(L.o_LS); A.LV = ptr(L.o_LV); A.foldV = ptr(L.o_foldV); A.dirS = ptr(L.o_dirS);
    A.cMi = ptr(L.o_cMi); A.RSi = ptr(L.o_RSi); A.RVi = ptr(L.o_RVi); A.LSi = ptr(L.o_LSi);
    A.LVi = ptr(L.o_LVi); A.foldVi = ptr(L.o_foldVi);
    A.Y0 = ptr(L.o_Y0); A.W = ptr(L.o_W); A.T = ptr(L.o_T); A.Y2 = ptr(L.o_Y2);
    return A;
}

// Launch sequence of the time loop (shared by the direct path and the graph
// capture).
static int launch_steps(const fdadi_heston_batch_t *b, const Layout &L, const Arena &A, double *V,
                        cudaStream_t st, int64_t *count) {
    const unsigned tiles = (unsigned)L.n_tiles;
    const unsigned gS = (unsigned)((L.SV + SOLVE_THREADS - 1) / SOLVE_THREADS);
    const unsigned gV = (unsigned)((L.SS + SOLVE_THREADS - 1) / SOLVE_THREADS);
    int64_t n = 0;
    for (int s = 0; s < b->implicit_steps; ++s) {
        explicit_kernel<ST_IMPLICIT><<<tiles, EXPL_TILE, 0, st>>>(A, V);
        var_solve_kernel<true><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, A.W);
        spot_solve_kernel<true, false><<<gS, SOLVE_THREADS, 0, st>>>(A, A.W, V);
        n += 3;
    }
    for (int s = 0; s < b->n_steps; ++s) {
        if (b->scheme == FDADI_SCHEME_DOUGLAS) {
            explicit_kernel<ST_DOUGLAS><<<tiles, EXPL_TILE, 0, st>>>(A, V);
            spot_solve_kernel<false, true><<<gS, SOLVE_THREADS, 0, st>>>(A, A.W, A.W);
            var_solve_kernel<false><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, V);
            n += 3;
        } else {
            explicit_kernel<ST_HV0><<<tiles, EXPL_TILE, 0, st>>>(A, V);
            spot_solve_kernel<false, true><<<gS, SOLVE_THREADS, 0, st>>>(A, A.W, A.W);
            var_solve_kernel<false><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, A.Y2);
            explicit_kernel<ST_HV3><<<tiles, EXPL_TILE, 0, st>>>(A, V);
            spot_solve_kernel<false, true><<<gS, SOLVE_THREADS, 0, st>>>(A, A.W, A.W);
            var_solve_kernel<false><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, V);
            n += 6;
        }
    }
    if (count) *count = n;
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

// Instantiated graphs of the time loop, keyed by everything the launches
// capture (workspace, state pointer, schedule).
struct GraphKey {
    const void *ws; const void *V; int n_opt, scheme, n_steps, smoothing;
    double factor, theta;
    int64_t P, SS, SV, n_tiles;
    bool operator==(const GraphKey &o) const {
        return ws == o.ws && V == o.V && n_opt == o.n_opt && scheme == o.scheme &&
               n_steps == o.n_steps && smoothing == o.smoothing && P == o.P && SS == o.SS &&
               factor == o.factor && theta == o.theta &&
               SV == o.SV && n_tiles == o.n_tiles;
    }
};
struct GraphKeyHash {
    size_t operator()(const GraphKey &k) const {
        return std::hash<const void *>()(k.ws) ^ (std::hash<const void *>()(k.V) << 1) ^
               ((size_t)k.n_steps << 7) ^ ((size_t)k.n_opt << 19);
    }
};
static std::mutex g_graph_mu;
static std::unordered_map<GraphKey, cudaGraphExec_t, GraphKeyHash> g_graphs;

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
    return (int64_t)3 * b->implicit_steps +
           (int64_t)b->n_steps * (b->scheme == FDADI_SCHEME_HV ? 6 : 3);
}

int fdadi_heston_prepare(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes,
                         void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    FDADI_REQUIRE(workspace != nullptr, "null workspace");
    if (ws_bytes < L.bytes) {
        set_error("workspace too small: %lld < %lld bytes", (long long)ws_bytes, (long long)L.bytes);
        return FDADI_E_WORKSPACE;
    }
    FDADI_REQUIRE(b->spots && b->vars && b->params && b->dt, "null mesh/params/dt pointer");
    cudaStream_t st = as_stream(stream);
    char *ws = (char *)workspace;
    // host tables
    std::vector<int> n0(L.n_opt), n1(L.n_opt), flags(L.n_opt), lineS(L.SV), lineV(L.SS);
    std::vector<int2> tiles;
    tiles.reserve(L.n_tiles);
    std::vector<double> theta(L.n_opt, b->theta);
    std::vector<int> barrier(L.n_opt, 0);
    if (b->barrier)
        FDADI_CUDA(cudaMemcpyAsync(barrier.data(), b->barrier, 4 * L.n_opt, cudaMemcpyDeviceToHost, st));
    // rho per option decides whether the mixed operator runs
    std::vector<double> params(5 * (size_t)L.n_opt);
    FDADI_CUDA(cudaMemcpyAsync(params.data(), b->params, 8 * params.size(), cudaMemcpyDeviceToHost, st));
    FDADI_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < L.n_opt; ++k) {
        n0[k] = b->n0[k];
        n1[k] = b->n1[k];
        const double rho = params[5 * (size_t)k + 4];
        const bool mixed = !((b->flags & FDADI_HESTON_DROP_ZERO_MIXED) && rho == 0.0);
        flags[k] = OPT_S_LOW_DIR | (barrier[k] ? OPT_S_HIGH_DIR : 0) | (mixed ? OPT_MIXED : 0);
        for (int64_t j = L.v_off[k]; j < L.v_off[k + 1]; ++j) lineS[j] = k;
        for (int64_t i = L.s_off[k]; i < L.s_off[k + 1]; ++i) lineV[i] = k;
        const int64_t N = L.p_off[k + 1] - L.p_off[k];
        for (int64_t t = 0; t < N; t += EXPL_TILE) tiles.push_back(make_int2(k, (int)t));
    }
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_n0, n0.data(), 4 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_n1, n1.data(), 4 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_flags, flags.data(), 4 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_p, L.p_off.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_s, L.s_off.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_v, L.v_off.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_lineS, lineS.data(), 4 * L.SV, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_lineV, lineV.data(), 4 * L.SS, cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_tiles, tiles.data(), 8 * tiles.size(), cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(ws + L.o_theta, theta.data(), 8 * L.n_opt, cudaMemcpyHostToDevice, st));
    Arena A = arena_view(L, ws);
    BuildArgs a{b->spots, b->vars, b->params, b->dt, b->barrier, b->theta, b->implicit_dt_factor,
                L.smoothing ? 1 : 0};
    build_points_kernel<<<(unsigned)L.n_tiles, EXPL_TILE, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    build_spot_lines_kernel<<<(unsigned)((L.SV + 127) / 128), 128, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    build_var_lines_kernel<<<(unsigned)((L.SS + 127) / 128), 128, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    // the host tables must outlive the copies
    FDADI_CUDA(cudaStreamSynchronize(st));
    return FDADI_OK;
}

int fdadi_heston_run(const fdadi_heston_batch_t *b, void *workspace, int64_t ws_bytes, double *V,
                     void *stream) {
    Layout L;
    int rc = make_layout(b, L);
    if (rc) return rc;
    FDADI_REQUIRE(workspace && V, "null workspace or state");
    if (ws_bytes < L.bytes) {
        set_error("workspace too small: %lld < %lld bytes", (long long)ws_bytes, (long long)L.bytes);
        return FDADI_E_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    Arena A = arena_view(L, (char *)workspace);
    if (!(b->flags & FDADI_HESTON_GRAPH)) return launch_steps(b, L, A, V, st, nullptr);
    FDADI_REQUIRE(st != nullptr, "graph mode needs a non-default stream");
    GraphKey key{workspace, V, b->n_options, b->scheme, b->n_steps, b->implicit_steps,
                 b->implicit_dt_factor, b->theta, L.P, L.SS, L.SV, L.n_tiles};
    cudaGraphExec_t exec = nullptr;
    {
        std::lock_guard<std::mutex> g(g_graph_mu);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) exec = it->second;
    }
    if (!exec) {
        cudaGraph_t graph;
        FDADI_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int lrc = launch_steps(b, L, A, V, st, nullptr);
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
    FDADI_REQUIRE(workspace && V, "null workspace or state");
    if (ws_bytes < L.bytes) {
        set_error("workspace too small: %lld < %lld bytes", (long long)ws_bytes, (long long)L.bytes);
        return FDADI_E_WORKSPACE;
    }
    const bool hv = b->scheme == FDADI_SCHEME_HV;
    FDADI_REQUIRE(!(stage == FDADI_STAGE_EXPLICIT_HV0 || stage == FDADI_STAGE_EXPLICIT_HV3 ||
                    stage == FDADI_STAGE_VAR_SOLVE_TO_Y2) || hv,
                  "stage %d needs a Hundsdorfer-Verwer batch", stage);
    FDADI_REQUIRE(stage < FDADI_STAGE_EXPLICIT_IMPLICIT || stage > FDADI_STAGE_SPOT_SOLVE_IMPLICIT ||
                      stage == FDADI_STAGE_SPOT_SOLVE || stage == FDADI_STAGE_VAR_SOLVE_TO_Y2 ||
                      stage == FDADI_STAGE_VAR_SOLVE_TO_V || L.smoothing,
                  "stage %d needs a batch with implicit steps", stage);
    cudaStream_t st = as_stream(stream);
    Arena A = arena_view(L, (char *)workspace);
    const unsigned tiles = (unsigned)L.n_tiles;
    const unsigned gS = (unsigned)((L.SV + SOLVE_THREADS - 1) / SOLVE_THREADS);
    const unsigned gV = (unsigned)((L.SS + SOLVE_THREADS - 1) / SOLVE_THREADS);
    switch (stage) {
    case FDADI_STAGE_EXPLICIT_DOUGLAS: explicit_kernel<ST_DOUGLAS><<<tiles, EXPL_TILE, 0, st>>>(A, V); break;
    case FDADI_STAGE_EXPLICIT_HV0: explicit_kernel<ST_HV0><<<tiles, EXPL_TILE, 0, st>>>(A, V); break;
    case FDADI_STAGE_EXPLICIT_HV3: explicit_kernel<ST_HV3><<<tiles, EXPL_TILE, 0, st>>>(A, V); break;
    case FDADI_STAGE_EXPLICIT_IMPLICIT: explicit_kernel<ST_IMPLICIT><<<tiles, EXPL_TILE, 0, st>>>(A, V); break;
    case FDADI_STAGE_SPOT_SOLVE: spot_solve_kernel<false, true><<<gS, SOLVE_THREADS, 0, st>>>(A, A.W, A.W); break;
    case FDADI_STAGE_VAR_SOLVE_TO_Y2: var_solve_kernel<false><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, A.Y2); break;
    case FDADI_STAGE_VAR_SOLVE_TO_V: var_solve_kernel<false><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, V); break;
    case FDADI_STAGE_VAR_SOLVE_IMPLICIT: var_solve_kernel<true><<<gV, SOLVE_THREADS, 0, st>>>(A, A.W, A.W); break;
    case FDADI_STAGE_SPOT_SOLVE_IMPLICIT: spot_solve_kernel<true, false><<<gS, SOLVE_THREADS, 0, st>>>(A, A.W, V); break;
    default:
        set_error("unknown stage %d", stage);
        return FDADI_E_ARG;
    }
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_fp64_probe(double *out, int32_t blocks, int32_t threads, int32_t iters, double *flops,
                     void *stream) {
    FDADI_REQUIRE(out && blocks > 0 && threads > 0 && threads <= 1024 && iters > 0,
                  "bad probe arguments");
    fp64_probe_kernel<<<blocks, threads, 0, as_stream(stream)>>>(out, iters);
    FDADI_CHECK_LAUNCH();
    if (flops) *flops = 2.0 * 8.0 * (double)blocks * threads * (double)iters;
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
