/*
 * fdadi_oracle.c -- CPU restatement of the reference ADI engine.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: the GPU kernels under
 * fd_adi_gb300/csrc are compared against it, and bench.py times it as the CPU
 * baseline. Nothing in the product links or calls it.
 *
 * It restates, in plain C, the algorithm of the reference CPU engine
 * (FiniteDifference/BandedOperator.pyx + FiniteDifference/FiniteDifferenceEngine.pyx)
 * for the Heston and Black-Scholes problems of FiniteDifference/heston.py and
 * FiniteDifference/blackscholes.py. Each function names the reference lines it
 * follows. Floating-point expressions keep the reference's evaluation order and
 * the file is compiled with -ffp-contract=off, so operator construction matches
 * the reference bit for bit; the line solves use Thomas elimination on the
 * folded tridiagonal system where the reference calls LAPACK gbsv, which agrees
 * to rounding (about 1e-16 per solve).
 *
 * Storage: an operator over `blocks` independent lines of length L holds five
 * row-aligned diagonals d[0..4] = A[i,i+2], A[i,i+1], A[i,i], A[i,i-1],
 * A[i,i-2] for every flat row i = b*L + k (block-major, the reference's
 * flattened order after rolling the operator's axis last,
 * BandedOperator.pyx:335-337).
 */
#include <malloc.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Every apply and solve takes grid-sized scratch from malloc; keep those
 * blocks on the heap (glibc would map and unmap each one, paying page faults
 * on every call). */
__attribute__((constructor)) static void oracle_malloc_tuning(void) {
    mallopt(M_MMAP_THRESHOLD, 256 << 20);
    mallopt(M_TRIM_THRESHOLD, 512 << 20);
}

enum { CANNOT_FOLD = 0, CAN_FOLD = 1, FOLDED = 2 };
enum { BND_NONE = -1, BND_DIRICHLET = 0, BND_NEUMANN = 1 };

typedef struct {
    int N, blocks, L, axis;
    double *d[5];
    double *R;
    int has_R;
    int has_low, has_high;
    double *low, *high;      /* Dirichlet values, one per block */
    int top_status, bot_status;
    double *top_f, *bot_f;   /* fold factors, one per block (FOLDED only) */
    /* mixed d2/dx0dx1 operator (FiniteDifferenceEngine.pyx:502-545) */
    int mixed, n0, n1;
    double *m9;              /* 9 coefficients per point, [N][9], (a,b) = (-1..1,-1..1) */
} op_t;

static op_t *op_new(int blocks, int L, int axis) {
    op_t *o = (op_t *)calloc(1, sizeof(op_t));
    o->N = blocks * L; o->blocks = blocks; o->L = L; o->axis = axis;
    for (int k = 0; k < 5; ++k) o->d[k] = (double *)calloc((size_t)o->N, sizeof(double));
    o->R = (double *)calloc((size_t)o->N, sizeof(double));
    o->has_R = 1;
    o->low = (double *)calloc((size_t)blocks, sizeof(double));
    o->high = (double *)calloc((size_t)blocks, sizeof(double));
    o->top_f = (double *)calloc((size_t)blocks, sizeof(double));
    o->bot_f = (double *)calloc((size_t)blocks, sizeof(double));
    return o;
}

static void op_free(op_t *o) {
    if (!o) return;
    for (int k = 0; k < 5; ++k) free(o->d[k]);
    free(o->R); free(o->low); free(o->high); free(o->top_f); free(o->bot_f); free(o->m9);
    free(o);
}

static op_t *op_copy(const op_t *s) {
    op_t *o = op_new(s->blocks, s->L, s->axis);
    size_t nb = (size_t)s->N * sizeof(double), bb = (size_t)s->blocks * sizeof(double);
    for (int k = 0; k < 5; ++k) memcpy(o->d[k], s->d[k], nb);
    memcpy(o->R, s->R, nb);
    o->has_R = s->has_R; o->has_low = s->has_low; o->has_high = s->has_high;
    memcpy(o->low, s->low, bb); memcpy(o->high, s->high, bb);
    o->top_status = s->top_status; o->bot_status = s->bot_status;
    memcpy(o->top_f, s->top_f, bb); memcpy(o->bot_f, s->bot_f, bb);
    o->mixed = s->mixed; o->n0 = s->n0; o->n1 = s->n1;
    if (s->m9) {
        o->m9 = (double *)malloc((size_t)s->N * 9 * sizeof(double));
        memcpy(o->m9, s->m9, (size_t)s->N * 9 * sizeof(double));
    }
    return o;
}

/* ---- construction ------------------------------------------------------ */

/* centercoeffs, BandedOperator.pyx:970-1017: non-uniform 3-point stencil on
 * inner rows 1..n-2 of one line; deltas d[i] = x[i] - x[i-1]. */
static void center_line(const double *x, int n, int derivative,
                        double *sup, double *mid, double *sub) {
    for (int i = 1; i < n - 1; ++i) {
        double di = x[i] - x[i - 1], dn = x[i + 1] - x[i];
        double s = di + dn;
        if (derivative == 1) {
            sup[i] = di / (dn * s);
            mid[i] = (-di + dn) / (di * dn);
            sub[i] = -dn / (di * s);
        } else {
            sup[i] = 2 / (dn * s);
            mid[i] = -2 / (di * dn);
            sub[i] = 2 / (di * s);
        }
    }
}

/* applyboundary, BandedOperator.pyx:398-524, for one line whose rows start
 * at flat index `o0`. `lval`/`hval` may be NAN to mean "None". */
static void boundary_line(op_t *B, int o0, const double *x, int n, int derivative,
                          int ltype, double lval, int htype, double hval, int blk) {
    double d1 = x[1] - x[0], d2 = x[2] - x[1];
    double dm1 = x[n - 1] - x[n - 2], dm2 = x[n - 2] - x[n - 3];
    double *e2 = B->d[0] + o0, *e1 = B->d[1] + o0, *e0 = B->d[2] + o0,
           *f1 = B->d[3] + o0, *f2 = B->d[4] + o0, *R = B->R + o0;
    (void)e2; (void)f2;
    if (ltype == BND_DIRICHLET) {
        e0[0] = 1; B->has_low = 1; B->low[blk] = lval;
    } else if (ltype == BND_NEUMANN) {
        R[0] = lval;
    } else if (derivative == 1) {
        e1[0] = 1 / d1;
        e0[0] = -1 / d1;
    } else if (!isnan(lval)) {
        double xx = d1 * d1;
        e1[0] = 2 / xx;
        e0[0] = -2 / xx;
        R[0] = -lval * 2 / d1;
    } else {
        double rd = 1.0 / (0.5 * (d2 + d1) * d2 * d1);
        e2[0] = d1 * rd;
        e1[0] = -(d2 + d1) * rd;
        e0[0] = d2 * rd;
    }
    if (htype == BND_DIRICHLET) {
        e0[n - 1] = 1; B->has_high = 1; B->high[blk] = hval;
    } else if (htype == BND_NEUMANN) {
        R[n - 1] = hval;
    } else if (derivative == 1) {
        e0[n - 1] = 1.0 / dm1;
        f1[n - 1] = -1.0 / dm1;
    } else if (!isnan(hval)) {
        double xx = dm1 * dm1;
        e0[n - 1] = -2 / xx;
        f1[n - 1] = 2 / xx;
        R[n - 1] = (hval * 2) / dm1;
    } else {
        double rd = 1.0 / (0.5 * (dm2 + dm1) * dm2 * dm1);
        f2[n - 1] = dm1 * rd;
        f1[n - 1] = -(dm2 + dm1) * rd;
        e0[n - 1] = dm2 * rd;
    }
}

/* forwardcoeffs (BandedOperator.pyx:917-967), first derivative, order 2, for
 * the rows a spliced 'forward' scheme takes (rows >= at): rows 1..n-3 use the
 * 3-point forward stencil (i, i+1, i+2), row n-2 the centred one. Rows are
 * written into the 5 diagonals at line offset o0 (offsets 2, 1, 0, -1, -2). */
static void forward_rows(op_t *B, int o0, const double *x, int n, int at) {
    double *e2 = B->d[0] + o0, *e1 = B->d[1] + o0, *e0 = B->d[2] + o0,
           *f1 = B->d[3] + o0, *f2 = B->d[4] + o0;
    for (int i = at; i < n; ++i) { e2[i] = e1[i] = e0[i] = f1[i] = f2[i] = 0; }
    for (int i = at > 1 ? at : 1; i < n - 2; ++i) {
        double d1 = x[i + 1] - x[i], d2 = x[i + 2] - x[i + 1];
        e1[i] = (d1 + d2) / (d1 * d2);
        e2[i] = -d1 / (d2 * (d1 + d2));
        e0[i] = (-2 * d1 - d2) / (d1 * (d1 + d2));
    }
    if (n - 2 >= at) {
        double dl = x[n - 1] - x[n - 2], dm = x[n - 2] - x[n - 3];
        e1[n - 2] = dm / (dl * (dm + dl));
        e0[n - 2] = (-dm + dl) / (dm * dl);
        f1[n - 2] = -dl / (dm * (dm + dl));
    }
}

/* backwardcoeffs (BandedOperator.pyx:1020-1067), first derivative, order 2,
 * for rows >= at: rows 2..n-2 use the 3-point backward stencil (i-2, i-1, i),
 * row 1 the centred one. */
static void backward_rows(op_t *B, int o0, const double *x, int n, int at) {
    double *e2 = B->d[0] + o0, *e1 = B->d[1] + o0, *e0 = B->d[2] + o0,
           *f1 = B->d[3] + o0, *f2 = B->d[4] + o0;
    for (int i = at; i < n; ++i) { e2[i] = e1[i] = e0[i] = f1[i] = f2[i] = 0; }
    for (int i = at > 2 ? at : 2; i < n - 1; ++i) {
        double dp = x[i - 1] - x[i - 2], di = x[i] - x[i - 1];
        e0[i] = (dp + 2 * di) / (di * (dp + di));
        f1[i] = (-dp - di) / (dp * di);
        f2[i] = di / (dp * (dp + di));
    }
    if (at <= 1) {
        double d1 = x[1] - x[0], d2 = x[2] - x[1];
        double xx = d1 + d2;
        e1[1] = d1 / (d2 * xx);
        e0[1] = (-d1 + d2) / (d1 * d2);
        f1[1] = -d2 / (d1 * xx);
    }
}

/* for_vector + applyboundary + _replicate/_flatten_tensor_aligned
 * (FiniteDifferenceEngine.pyx:446-497): one derivative operator along `axis`
 * replicated over `blocks` lines, same boundary on every line. `splice`: 0
 * none, 1 a 'forward' scheme from row `at` on, 2 a 'backward' scheme from row
 * `at` on (first derivatives; make_operator_template and splice_with,
 * FiniteDifferenceEngine.pyx:267-289, BandedOperator.pyx:527-591: every row
 * >= at comes from the second scheme's operator). */
static op_t *derivative_op_spliced(const double *x, int n, int blocks, int axis, int derivative,
                                   int ltype, double lval, int htype, double hval, int pentadiag,
                                   int splice, int at) {
    op_t *B = op_new(blocks, n, axis);
    for (int b = 0; b < blocks; ++b) {
        int o0 = b * n;
        center_line(x, n, derivative, B->d[1] + o0, B->d[2] + o0, B->d[3] + o0);
        if (splice == 1) forward_rows(B, o0, x, n, at);
        else if (splice == 2) backward_rows(B, o0, x, n, at);
        boundary_line(B, o0, x, n, derivative, ltype, lval, htype, hval, b);
    }
    /* the operator's offsets include +2 (forward) or -2 (backward), so it can
     * fold there (BandedOperator.pyx:64-65) */
    B->bot_status = (pentadiag || splice == 2) ? CAN_FOLD : CANNOT_FOLD;
    B->top_status = splice == 1 ? CAN_FOLD : CANNOT_FOLD;
    return B;
}

static op_t *derivative_op(const double *x, int n, int blocks, int axis, int derivative,
                           int ltype, double lval, int htype, double hval, int pentadiag) {
    op_t *B = op_new(blocks, n, axis);
    for (int b = 0; b < blocks; ++b) {
        int o0 = b * n;
        center_line(x, n, derivative, B->d[1] + o0, B->d[2] + o0, B->d[3] + o0);
        boundary_line(B, o0, x, n, derivative, ltype, lval, htype, hval, b);
    }
    /* fold status from the offsets (BandedOperator.pyx:64-65); the offsets are
     * chosen by _min_possible_bandwidth (FiniteDifferenceEngine.pyx:295-351). */
    B->bot_status = pentadiag ? CAN_FOLD : CANNOT_FOLD;
    B->top_status = CANNOT_FOLD;
    return B;
}

/* vectorized_scale, BandedOperator.pyx:749-792: row i scaled by vec[i], except
 * Dirichlet rows (vec forced to 1 there); R scaled too. */
static void op_vscale(op_t *o, const double *vec_in) {
    double *vec = (double *)malloc((size_t)o->N * sizeof(double));
    memcpy(vec, vec_in, (size_t)o->N * sizeof(double));
    for (int b = 0; b < o->blocks; ++b) {
        if (o->has_low) vec[b * o->L] = 1;
        if (o->has_high) vec[(b + 1) * o->L - 1] = 1;
    }
    if (o->mixed) {
        for (int i = 0; i < o->N; ++i)
            for (int k = 0; k < 9; ++k) o->m9[i * 9 + k] *= vec[i];
    } else {
        for (int k = 0; k < 5; ++k)
            for (int i = 0; i < o->N; ++i) o->d[k][i] *= vec[i];
    }
    for (int i = 0; i < o->N; ++i) o->R[i] *= vec[i];
    free(vec);
}

/* __imul__ (BandedOperator.pyx:599-601) */
static op_t *op_mul(const op_t *s, double val) {
    op_t *o = op_copy(s);
    double *v = (double *)malloc((size_t)o->N * sizeof(double));
    for (int i = 0; i < o->N; ++i) v[i] = val;
    op_vscale(o, v);
    free(v);
    return o;
}

/* add_scalar, BandedOperator.pyx:713-745. The argument is declared as a C
 * `float` in BandedOperator.pxd:32, so the scalar is rounded to binary32. */
static void op_add_scalar_f32(op_t *o, double val) {
    double v = (double)(float)val;
    for (int b = 0; b < o->blocks; ++b) {
        int end = b * o->L + (o->has_low ? 1 : 0);
        int begin = b * o->L + o->L - (o->has_high ? 1 : 0);
        for (int i = end; i < begin; ++i) o->d[2][i] += v;
    }
}

/* add_operator, BandedOperator.pyx:618-710: off-diagonals added everywhere,
 * the main diagonal blockwise skipping this operator's Dirichlet rows. */
static void op_add(op_t *B, const op_t *other) {
    for (int k = 0; k < 5; ++k) {
        if (k == 2) continue;
        for (int i = 0; i < B->N; ++i) B->d[k][i] += other->d[k][i];
    }
    for (int b = 0; b < B->blocks; ++b) {
        int end = b * B->L + (B->has_low ? 1 : 0);
        int begin = b * B->L + B->L - (B->has_high ? 1 : 0);
        for (int i = end; i < begin; ++i) B->d[2][i] += other->d[2][i];
    }
    for (int i = 0; i < B->N; ++i) B->R[i] += other->R[i];
    if (other->top_status == CAN_FOLD) B->top_status = CAN_FOLD;
    if (other->bot_status == CAN_FOLD) B->bot_status = CAN_FOLD;
}

/* fold_bottom / fold_top / diagonalize, BandedOperator.pyx:181-290 */
static void op_diagonalize(op_t *o) {
    int L = o->L;
    if (o->top_status == CAN_FOLD) {
        for (int b = 0; b < o->blocks; ++b) {
            int r0 = b * L, r1 = r0 + 1;
            double c1 = o->d[1][r1], d0 = o->d[0][r0];
            double f = c1 != 0 ? -d0 / c1 : 0;
            o->top_f[b] = f;
            o->d[0][r0] += c1 * f;
            o->d[1][r0] += o->d[2][r1] * f;
            o->d[2][r0] += o->d[3][r1] * f;
        }
        o->top_status = FOLDED;
    }
    if (o->bot_status == CAN_FOLD) {
        for (int b = 0; b < o->blocks; ++b) {
            int rn = (b + 1) * L - 1, rn1 = rn - 1;
            double an1 = o->d[3][rn1], zn = o->d[4][rn];
            double f = an1 != 0 ? -zn / an1 : 0;
            o->bot_f[b] = f;
            o->d[4][rn] += an1 * f;
            o->d[3][rn] += o->d[2][rn1] * f;
            o->d[2][rn] += o->d[1][rn1] * f;
        }
        o->bot_status = FOLDED;
    }
    /* the +-2 diagonals are dropped (BandedOperator.pyx:195-198) */
    memset(o->d[0], 0, (size_t)o->N * sizeof(double));
    memset(o->d[4], 0, (size_t)o->N * sizeof(double));
}

static int op_folded(const op_t *o) { return o->top_status == FOLDED || o->bot_status == FOLDED; }
static int op_foldable(const op_t *o) { return o->top_status == CAN_FOLD || o->bot_status == CAN_FOLD; }

/* fold_vector, BandedOperator.pyx:293-311 */
static void fold_vector(const op_t *o, double *v, int unfold) {
    double dir = unfold ? -1 : 1;
    for (int b = 0; b < o->blocks; ++b) {
        int u0 = b * o->L, u1 = u0 + 1, un = (b + 1) * o->L - 1, un1 = un - 1;
        if (o->top_status == FOLDED) v[u0] += dir * v[u1] * o->top_f[b];
        if (o->bot_status == FOLDED) v[un] += dir * v[un1] * o->bot_f[b];
    }
}

/* ---- apply / solve on a grid ------------------------------------------- */

/* Grid V has shape [n0][n1] row-major (n1 = 1 for one dimension). An axis-0
 * operator sees line b = column j, element k = row i; an axis-1 operator sees
 * line b = row i, element k = column j (BandedOperator.pyx:335-337). */
/* Lines are independent within every loop below, so large grids spread them
 * over threads (each element's arithmetic is unchanged, and so are the bits);
 * inside oracle_heston_batch's per-option threads these run single-threaded. */
#define PAR_MIN 65536
static void gather(const op_t *o, const double *V, int n0, int n1, double *flat) {
    if (o->axis == 0) {
#pragma omp parallel for if ((long)n0 * n1 >= PAR_MIN)
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n0; ++i) flat[j * n0 + i] = V[i * n1 + j];
    } else {
        memcpy(flat, V, (size_t)n0 * n1 * sizeof(double));
    }
}

static void scatter(const op_t *o, const double *flat, int n0, int n1, double *V) {
    if (o->axis == 0) {
#pragma omp parallel for if ((long)n0 * n1 >= PAR_MIN)
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n0; ++i) V[i * n1 + j] = flat[j * n0 + i];
    } else {
        memcpy(V, flat, (size_t)n0 * n1 * sizeof(double));
    }
}

static void force_dirichlet(const op_t *o, double *flat) {
    for (int b = 0; b < o->blocks; ++b) {
        if (o->has_low) flat[b * o->L] = o->low[b];
        if (o->has_high) flat[(b + 1) * o->L - 1] = o->high[b];
    }
}

/* apply, BandedOperator.pyx:331-361 (mixed: the flattened 9-offset DIA built
 * at FiniteDifferenceEngine.pyx:502-545). out may alias nothing. */
static void op_apply(const op_t *o, const double *V, int n0, int n1, double *out) {
    int N = o->N;
    double *x = (double *)malloc((size_t)N * sizeof(double));
    double *y = (double *)malloc((size_t)N * sizeof(double));
    if (o->mixed) {
        memcpy(x, V, (size_t)N * sizeof(double));
#pragma omp parallel for if (N >= PAR_MIN)
        for (int i = 0; i < n0; ++i)
            for (int j = 0; j < n1; ++j) {
                const double *c = o->m9 + (size_t)(i * n1 + j) * 9;
                double acc = 0;
                /* stored offset order n1+1, n1, n1-1, 1, 0, -1, -n1+1, -n1, -n1-1 */
                for (int a = 1; a >= -1; --a)
                    for (int bb = 1; bb >= -1; --bb) {
                        int ii = i + a, jj = j + bb;
                        double w = c[(a + 1) * 3 + (bb + 1)];
                        if (ii < 0 || ii >= n0 || jj < 0 || jj >= n1) continue;
                        acc += w * x[ii * n1 + jj];
                    }
                y[i * n1 + j] = acc;
            }
        if (o->has_R) for (int i = 0; i < N; ++i) y[i] += o->R[i];
        memcpy(out, y, (size_t)N * sizeof(double));
        free(x); free(y);
        return;
    }
    gather(o, V, n0, n1, x);
    force_dirichlet(o, x);
    int L = o->L;
#pragma omp parallel for if (N >= PAR_MIN)
    for (int b = 0; b < o->blocks; ++b) {
        for (int k = 0; k < L; ++k) {
            int i = b * L + k;
            /* scipy's DIA matvec accumulates diagonal by diagonal in the
             * stored offset order (2, 1, 0, -1, -2). */
            double acc = 0;
            if (k + 2 < L) acc += o->d[0][i] * x[i + 2];
            if (k + 1 < L) acc += o->d[1][i] * x[i + 1];
            acc += o->d[2][i] * x[i];
            if (k >= 1) acc += o->d[3][i] * x[i - 1];
            if (k >= 2) acc += o->d[4][i] * x[i - 2];
            y[i] = acc;
        }
    }
    if (op_folded(o)) fold_vector(o, y, 1);
    if (o->has_R) for (int i = 0; i < N; ++i) y[i] += o->R[i];
    scatter(o, y, n0, n1, out);
    free(x); free(y);
}

/* solve, BandedOperator.pyx:364-394: Dirichlet values forced, R subtracted,
 * RHS folded, then a tridiagonal solve per line. Operators that still carry a
 * +-2 diagonal (the unfolded implicit operator) are folded on a private copy
 * first, which is the same linear system. */
/* True if the +2 (-2) diagonal holds entries beyond the first (last) row of a
 * line: a spliced forward (backward) scheme, which folding cannot remove. */
static int op_interior_band(const op_t *o) {
    for (int b = 0; b < o->blocks; ++b)
        for (int k = 0; k < o->L; ++k) {
            int i = b * o->L + k;
            if (k != 0 && o->d[0][i] != 0) return 1;
            if (k != o->L - 1 && o->d[4][i] != 0) return 1;
        }
    return 0;
}

/* Banded LU without pivoting on every line (offsets 2..-2), the system
 * scipy's solve_banded solves (LAPACK gbsv; no row exchange happens on these
 * diagonally dominant systems, so they agree to rounding). x: right-hand
 * sides in, solutions out, block-major. */
static void band_solve(const op_t *o, double *x) {
    int L = o->L;
#pragma omp parallel if (o->N >= PAR_MIN)
    {
    double *a2 = (double *)malloc((size_t)L * sizeof(double));
    double *a1 = (double *)malloc((size_t)L * sizeof(double));
    double *a0 = (double *)malloc((size_t)L * sizeof(double));
    double *b1 = (double *)malloc((size_t)L * sizeof(double));
    double *b2 = (double *)malloc((size_t)L * sizeof(double));
#pragma omp for
    for (int b = 0; b < o->blocks; ++b) {
        int r0 = b * L;
        double *r = x + (size_t)r0;
        memcpy(a2, o->d[0] + r0, (size_t)L * sizeof(double));
        memcpy(a1, o->d[1] + r0, (size_t)L * sizeof(double));
        memcpy(a0, o->d[2] + r0, (size_t)L * sizeof(double));
        memcpy(b1, o->d[3] + r0, (size_t)L * sizeof(double));
        memcpy(b2, o->d[4] + r0, (size_t)L * sizeof(double));
        for (int k = 0; k < L; ++k) {
            double p = a0[k];
            if (k + 1 < L) {
                double l = b1[k + 1] / p;
                a0[k + 1] = a0[k + 1] - l * a1[k];
                a1[k + 1] = a1[k + 1] - l * a2[k];
                r[k + 1] = r[k + 1] - l * r[k];
            }
            if (k + 2 < L) {
                double l = b2[k + 2] / p;
                b1[k + 2] = b1[k + 2] - l * a1[k];
                a0[k + 2] = a0[k + 2] - l * a2[k];
                r[k + 2] = r[k + 2] - l * r[k];
            }
        }
        for (int k = L - 1; k >= 0; --k) {
            double acc = r[k];
            if (k + 1 < L) acc = acc - a1[k] * r[k + 1];
            if (k + 2 < L) acc = acc - a2[k] * r[k + 2];
            r[k] = acc / a0[k];
        }
    }
    free(a2); free(a1); free(a0); free(b1); free(b2);
    }
}

static void op_solve(const op_t *o_in, double *V, int n0, int n1) {
    const op_t *o = o_in;
    op_t *tmp = NULL;
    int N = o->N, L = o->L;
    double *x = (double *)malloc((size_t)N * sizeof(double));
    gather(o, V, n0, n1, x);
    force_dirichlet(o, x);
    if (o->has_R) for (int i = 0; i < N; ++i) x[i] = x[i] - o->R[i];
    if (!op_folded(o) && op_interior_band(o)) {
        band_solve(o, x);
        scatter(o, x, n0, n1, V);
        free(x);
        return;
    }
    if (op_foldable(o)) {
        tmp = op_copy(o);
        op_diagonalize(tmp);
        o = tmp;
    }
    if (op_folded(o)) fold_vector(o, x, 0);
#pragma omp parallel if (N >= PAR_MIN)
    {
    double *cp = (double *)malloc((size_t)L * sizeof(double));
#pragma omp for
    for (int b = 0; b < o->blocks; ++b) {
        double *r = x + (size_t)b * L;
        const double *sup = o->d[1] + (size_t)b * L, *mid = o->d[2] + (size_t)b * L,
                     *sub = o->d[3] + (size_t)b * L;
        cp[0] = sup[0] / mid[0];
        r[0] = r[0] / mid[0];
        for (int k = 1; k < L; ++k) {
            double m = mid[k] - sub[k] * cp[k - 1];
            cp[k] = sup[k] / m;
            r[k] = (r[k] - sub[k] * r[k - 1]) / m;
        }
        for (int k = L - 2; k >= 0; --k) r[k] = r[k] - cp[k] * r[k + 1];
    }
    free(cp);
    }
    scatter(o, x, n0, n1, V);
    free(x);
    if (tmp) op_free(tmp);
}

/* ---- engines ----------------------------------------------------------- */

typedef struct {
    int ndim, n0, n1;
    op_t *A[2];    /* combined per-dimension operators */
    op_t *M;       /* mixed operator, NULL if absent */
} engine_t;

static void engine_free(engine_t *E) {
    op_free(E->A[0]); op_free(E->A[1]); op_free(E->M);
}

/* Heston operators: coefficients heston.py:303-333, boundaries heston.py:335-359,
 * built as in make_discrete_operators and scale_and_combine_operators
 * (FiniteDifferenceEngine.pyx:423-592). An up-and-out barrier at the top of
 * the spot mesh makes the high boundary of both spot operators Dirichlet 0,
 * and (0,0) takes (0,)'s boundaries (heston.py:361-370). */
static void heston_engine(engine_t *E, const double *S, int nS, const double *v, int nv,
                          double r, double kappa, double theta, double sigma, double rho,
                          int barrier, int flip_spot, int flip_var) {
    int N = nS * nv;
    E->ndim = 2; E->n0 = nS; E->n1 = nv;
    double *vec = (double *)malloc((size_t)N * sizeof(double));
    /* (0,): D U=0 / Neumann dU/dS = 1 (barrier: D U=0); from flip_spot on
     * (>= 0), forward differences (heston.py:432-433) */
    op_t *d0 = derivative_op_spliced(S, nS, nv, 0, 1, BND_DIRICHLET, 0.0,
                                     barrier ? BND_DIRICHLET : BND_NEUMANN, barrier ? 0.0 : 1.0,
                                     0, flip_spot >= 0 ? 1 : 0, flip_spot);
    /* (0,0): D U=0 / free, first derivative 1 (barrier: D U=0) */
    op_t *d00 = barrier
        ? derivative_op(S, nS, nv, 0, 2, BND_DIRICHLET, 0.0, BND_DIRICHLET, 0.0, 0)
        : derivative_op(S, nS, nv, 0, 2, BND_DIRICHLET, 0.0, BND_NONE, 1.0, 0);
    /* (1,): free / free; from flip_var on (>= 0), backward differences
     * (heston.py:436-437) */
    op_t *d1 = derivative_op_spliced(v, nv, nS, 1, 1, BND_NONE, NAN, BND_NONE, NAN, 0,
                                     flip_var >= 0 ? 2 : 0, flip_var);
    /* (1,1): Neumann 0 / free second order (offset -2) */
    op_t *d11 = derivative_op(v, nv, nS, 1, 2, BND_NEUMANN, 0.0, BND_NONE, NAN, 1);

    /* coefficient_vector(f, t, dim): dim is the fastest varying index */
    for (int j = 0; j < nv; ++j) for (int i = 0; i < nS; ++i) vec[j * nS + i] = r * S[i];
    op_vscale(d0, vec);
    for (int j = 0; j < nv; ++j) for (int i = 0; i < nS; ++i)
        vec[j * nS + i] = 0.5 * v[j] * (S[i] * S[i]);
    op_vscale(d00, vec);
    for (int i = 0; i < nS; ++i) for (int j = 0; j < nv; ++j)
        vec[i * nv + j] = S[i] == 0 ? 0.0 : kappa * (theta - v[j]);
    op_vscale(d1, vec);
    for (int i = 0; i < nS; ++i) for (int j = 0; j < nv; ++j)
        vec[i * nv + j] = S[i] == 0 ? 0.0 : 0.5 * (sigma * sigma) * v[j];
    op_vscale(d11, vec);

    /* sorted keys (0,), (0,0), (0,1), (1,), (1,1): dim 0 = (0,) - r/2, += (0,0) */
    op_add_scalar_f32(d0, -r / 2.0);
    op_add(d0, d00);
    op_add_scalar_f32(d1, -r / 2.0);
    op_add(d1, d11);
    op_free(d00); op_free(d11);
    E->A[0] = d0; E->A[1] = d1;

    /* mixed: centred first-derivative weights in S and v, products, edges 0 */
    op_t *M = op_new(nS, nv, 1);
    M->mixed = 1; M->n0 = nS; M->n1 = nv;
    M->m9 = (double *)calloc((size_t)N * 9, sizeof(double));
    double *ws[3], *wv[3];
    for (int k = 0; k < 3; ++k) {
        ws[k] = (double *)calloc((size_t)nS, sizeof(double));
        wv[k] = (double *)calloc((size_t)nv, sizeof(double));
    }
    center_line(S, nS, 1, ws[2], ws[1], ws[0]);   /* ws[a+1][i] = A_S[i, i+a] */
    center_line(v, nv, 1, wv[2], wv[1], wv[0]);
    for (int i = 1; i < nS - 1; ++i)
        for (int j = 1; j < nv - 1; ++j)
            for (int a = -1; a <= 1; ++a)
                for (int b = -1; b <= 1; ++b)
                    M->m9[(size_t)(i * nv + j) * 9 + (a + 1) * 3 + (b + 1)] =
                        wv[b + 1][j] * ws[a + 1][i];
    for (int i = 0; i < nS; ++i) for (int j = 0; j < nv; ++j)
        vec[i * nv + j] = rho * sigma * S[i] * v[j];
    op_vscale(M, vec);
    E->M = M;
    for (int k = 0; k < 3; ++k) { free(ws[k]); free(wv[k]); }
    free(vec);
}

/* Black-Scholes, blackscholes.py:144-239 (non-log mesh) */
static void bs_engine(engine_t *E, const double *S, int nS, double r, double var) {
    E->ndim = 1; E->n0 = nS; E->n1 = 1;
    double *vec = (double *)malloc((size_t)nS * sizeof(double));
    op_t *d0 = derivative_op(S, nS, 1, 0, 1, BND_DIRICHLET, 0.0, BND_NEUMANN, 1.0, 0);
    op_t *d00 = derivative_op(S, nS, 1, 0, 2, BND_DIRICHLET, 0.0, BND_NONE, 1.0, 0);
    for (int i = 0; i < nS; ++i) vec[i] = r * S[i];
    op_vscale(d0, vec);
    for (int i = 0; i < nS; ++i) vec[i] = 0.5 * var * (S[i] * S[i]);
    op_vscale(d00, vec);
    op_add_scalar_f32(d0, -r / 1.0);
    op_add(d0, d00);
    op_free(d00);
    E->A[0] = d0; E->A[1] = NULL; E->M = NULL;
    free(vec);
}

static void vadd(double *a, const double *b, size_t n) {
#pragma omp parallel for if (n >= PAR_MIN)
    for (size_t i = 0; i < n; ++i) a[i] += b[i];
}
static void vsub(double *a, const double *b, size_t n) {
#pragma omp parallel for if (n >= PAR_MIN)
    for (size_t i = 0; i < n; ++i) a[i] -= b[i];
}

/* solve_douglas, FiniteDifferenceEngine.pyx:945-1006 */
static void run_douglas(const engine_t *E, int n, double dt, double theta, double *V) {
    int nd = E->ndim;
    size_t N = (size_t)E->n0 * E->n1;
    op_t *F[3], *Le[2], *Li[2];
    int nf = 0;
    for (int d = 0; d < nd; ++d) F[nf++] = op_mul(E->A[d], dt);
    if (E->M) F[nf++] = op_mul(E->M, dt);
    for (int d = 0; d < nd; ++d) {
        op_t *t = op_mul(E->A[d], theta);
        Le[d] = op_mul(t, dt);
        op_free(t);
        Li[d] = op_mul(E->A[d], theta * -dt);
        op_add_scalar_f32(Li[d], 1.0);
        Le[d]->has_R = 0; Li[d]->has_R = 0;
    }
    for (int k = 0; k < nf; ++k) if (op_foldable(F[k]) && !F[k]->mixed) op_diagonalize(F[k]);
    for (int d = 0; d < nd; ++d) {
        if (op_foldable(Le[d])) op_diagonalize(Le[d]);
        if (op_foldable(Li[d])) op_diagonalize(Li[d]);
    }
    double *Y = (double *)malloc(N * sizeof(double)), *T = (double *)malloc(N * sizeof(double));
    for (int s = 0; s < n; ++s) {
        memcpy(Y, V, N * sizeof(double));
        for (int k = 0; k < nf; ++k) { op_apply(F[k], V, E->n0, E->n1, T); vadd(Y, T, N); }
        for (int d = 0; d < nd; ++d) {
            op_apply(Le[d], V, E->n0, E->n1, T);
            vsub(Y, T, N);
            op_solve(Li[d], Y, E->n0, E->n1);
        }
        memcpy(V, Y, N * sizeof(double));
    }
    free(Y); free(T);
    for (int k = 0; k < nf; ++k) op_free(F[k]);
    for (int d = 0; d < nd; ++d) { op_free(Le[d]); op_free(Li[d]); }
}

/* solve_hundsdorferverwer, FiniteDifferenceEngine.pyx:700-775 */
static void run_hv(const engine_t *E, int n, double dt, double theta, double *V) {
    int nd = E->ndim;
    size_t N = (size_t)E->n0 * E->n1;
    op_t *F[3], *Le[2], *Li[2];
    int nf = 0;
    for (int d = 0; d < nd; ++d) F[nf++] = op_mul(E->A[d], dt);
    if (E->M) F[nf++] = op_mul(E->M, dt);
    for (int d = 0; d < nd; ++d) {
        op_t *t = op_mul(E->A[d], theta);
        Le[d] = op_mul(t, dt);
        op_free(t);
        Li[d] = op_mul(E->A[d], theta * -dt);
        op_add_scalar_f32(Li[d], 1.0);
        Le[d]->has_R = 0; Li[d]->has_R = 0;
    }
    for (int d = 0; d < nd; ++d) {
        if (op_foldable(Le[d])) op_diagonalize(Le[d]);
        if (op_foldable(Li[d])) op_diagonalize(Li[d]);
    }
    for (int k = 0; k < nf; ++k) if (op_foldable(F[k]) && !F[k]->mixed) op_diagonalize(F[k]);
    double *Y = (double *)malloc(N * sizeof(double)), *Z = (double *)malloc(N * sizeof(double)),
           *T = (double *)malloc(N * sizeof(double));
    for (int s = 0; s < n; ++s) {
        memcpy(Y, V, N * sizeof(double));
        for (int k = 0; k < nf; ++k) { op_apply(F[k], Y, E->n0, E->n1, T); vadd(V, T, N); }
        memcpy(Z, V, N * sizeof(double));
        for (int d = 0; d < nd; ++d) {
            op_apply(Le[d], Y, E->n0, E->n1, T);
            vsub(Z, T, N);
            op_solve(Li[d], Z, E->n0, E->n1);
        }
        vsub(Y, Z, N);
        for (int k = 0; k < nf; ++k) {
            int keep = F[k]->has_R;
            F[k]->has_R = 0;
            op_apply(F[k], Y, E->n0, E->n1, T);
            F[k]->has_R = keep;
#pragma omp parallel for if (N >= PAR_MIN)
            for (size_t i = 0; i < N; ++i) V[i] -= 0.5 * T[i];
        }
        for (int d = 0; d < nd; ++d) {
            op_apply(Le[d], Z, E->n0, E->n1, T);
            vsub(V, T, N);
            op_solve(Li[d], V, E->n0, E->n1);
        }
    }
    free(Y); free(Z); free(T);
    for (int k = 0; k < nf; ++k) op_free(F[k]);
    for (int d = 0; d < nd; ++d) { op_free(Le[d]); op_free(Li[d]); }
}

/* solve_implicit, FiniteDifferenceEngine.pyx:617-659: Lis = 1 - dt*A_d with the
 * residual kept, solved in the order dim 1 then dim 0 (np.roll(Lis, -1)),
 * after an explicit mixed step V += dt*A01 V. */
static void run_implicit(const engine_t *E, int n, double dt, double *V) {
    int nd = E->ndim;
    size_t N = (size_t)E->n0 * E->n1;
    op_t *Li[2];
    for (int d = 0; d < nd; ++d) {
        Li[d] = op_mul(E->A[d], -dt);
        op_add_scalar_f32(Li[d], 1.0);
    }
    op_t *C = E->M ? op_mul(E->M, dt) : NULL;
    double *T = (double *)malloc(N * sizeof(double));
    for (int s = 0; s < n; ++s) {
        if (C) { op_apply(C, V, E->n0, E->n1, T); vadd(V, T, N); }
        for (int q = 0; q < nd; ++q) {
            int d = (q + 1) % nd;
            op_solve(Li[d], V, E->n0, E->n1);
        }
    }
    free(T);
    if (C) op_free(C);
    for (int d = 0; d < nd; ++d) op_free(Li[d]);
}

/* Craig-Sneyd, FiniteDifferenceEngine.pyx:843-898 (modified = 0), and the
 * modified Craig-Sneyd scheme, :779-841 (modified = 1). Per step:
 *   Y0 = V + sum_k F_k V (F_k = dt A_k with their residuals, and dt M),
 *   Y2 = the Douglas sweep from Y0 (Y <- Li_d^-1 (Y - Le_d V), d = 0, 1),
 *   CS:  Z = Y0 + (dt/2) M (Y2 - V);
 *   MCS: Z = Y0 + theta dt M (Y2 - V) + (1/2 - theta) sum_k F_k.apply(Y2 - V)
 *        (the reference applies F_k with its residual here, so it is added),
 *   then the same sweep from Z, and V <- the result. The reference solves the
 *   unfolded banded systems with LAPACK; the folded Thomas solve here is the
 *   same linear system. */
static void run_cs(const engine_t *E, int n, double dt, double theta, double *V, int modified) {
    int nd = E->ndim;
    size_t N = (size_t)E->n0 * E->n1;
    op_t *F[3], *Le[2], *Li[2];
    int nf = 0;
    for (int d = 0; d < nd; ++d) F[nf++] = op_mul(E->A[d], dt);
    if (E->M) F[nf++] = op_mul(E->M, dt);
    for (int d = 0; d < nd; ++d) {
        op_t *t = op_mul(E->A[d], theta);
        Le[d] = op_mul(t, dt);
        op_free(t);
        Li[d] = op_mul(E->A[d], theta * -dt);
        op_add_scalar_f32(Li[d], 1.0);
        Le[d]->has_R = 0; Li[d]->has_R = 0;
    }
    /* Craig-Sneyd keeps every operator at full bandwidth (the reference does
     * not diagonalize here): applies use all five diagonals and solves the
     * whole band, which matters once a spliced scheme puts +-2 entries inside
     * the lines. */
    double *Y = (double *)malloc(N * sizeof(double)), *Y0 = (double *)malloc(N * sizeof(double)),
           *D = (double *)malloc(N * sizeof(double)), *T = (double *)malloc(N * sizeof(double));
    for (int s = 0; s < n; ++s) {
        memcpy(Y, V, N * sizeof(double));
        for (int k = 0; k < nf; ++k) { op_apply(F[k], V, E->n0, E->n1, T); vadd(Y, T, N); }
        memcpy(Y0, Y, N * sizeof(double));
        for (int d = 0; d < nd; ++d) {
            op_apply(Le[d], V, E->n0, E->n1, T);
            vsub(Y, T, N);
            op_solve(Li[d], Y, E->n0, E->n1);
        }
        for (size_t i = 0; i < N; ++i) D[i] = Y[i] - V[i];
        if (E->M) {
            op_apply(E->M, D, E->n0, E->n1, T);
            const double c = modified ? theta * dt : 0.5 * dt;
            for (size_t i = 0; i < N; ++i) Y[i] = Y0[i] + c * T[i];
        } else {
            memcpy(Y, Y0, N * sizeof(double));
        }
        if (modified) {
            for (int k = 0; k < nf; ++k) {
                op_apply(F[k], D, E->n0, E->n1, T);
                for (size_t i = 0; i < N; ++i) Y[i] += (0.5 - theta) * T[i];
            }
        }
        for (int d = 0; d < nd; ++d) {
            op_apply(Le[d], V, E->n0, E->n1, T);
            vsub(Y, T, N);
            op_solve(Li[d], Y, E->n0, E->n1);
        }
        memcpy(V, Y, N * sizeof(double));
    }
    free(Y); free(Y0); free(D); free(T);
    for (int k = 0; k < nf; ++k) op_free(F[k]);
    for (int d = 0; d < nd; ++d) { op_free(Le[d]); op_free(Li[d]); }
}

enum { SCHEME_IMPLICIT = 0, SCHEME_DOUGLAS = 1, SCHEME_HV = 2, SCHEME_CS = 3, SCHEME_MCS = 4 };

static void run_schedule(const engine_t *E, int nseg, const int *scheme, const int *nsteps,
                         const double *dt, const double *theta, double *V) {
    for (int s = 0; s < nseg; ++s) {
        if (scheme[s] == SCHEME_IMPLICIT) run_implicit(E, nsteps[s], dt[s], V);
        else if (scheme[s] == SCHEME_DOUGLAS) run_douglas(E, nsteps[s], dt[s], theta[s], V);
        else if (scheme[s] == SCHEME_CS) run_cs(E, nsteps[s], dt[s], theta[s], V, 0);
        else if (scheme[s] == SCHEME_MCS) run_cs(E, nsteps[s], dt[s], theta[s], V, 1);
        else run_hv(E, nsteps[s], dt[s], theta[s], V);
    }
}

/* ---- exported entry points (ctypes) ------------------------------------ */

/* One Heston solve on a given mesh. V: [nS*nv] initial grid in, final out.
 * Segments run in order: scheme 0 implicit, 1 Douglas, 2 Hundsdorfer-Verwer,
 * 3 Craig-Sneyd, 4 modified Craig-Sneyd. flags: bit 0 drops the mixed
 * operator when rho = 0, bit 1 makes the top of the spot mesh an up-and-out
 * barrier. */
int oracle_heston_solve(const double *S, int nS, const double *v, int nv,
                        double r, double kappa, double theta, double sigma, double rho,
                        int flags,
                        int nseg, const int *scheme, const int *nsteps,
                        const double *dt, const double *th, double *V, const double *rates) {
    if (nS < 4 || nv < 4) return 1;
    /* flags bits 8..19: flip_idx_spot + 1, bits 20..30: flip_idx_var + 1 (0: none) */
    const int flip_spot = ((flags >> 8) & 0xFFF) - 1, flip_var = ((flags >> 20) & 0x7FF) - 1;
    if (flip_spot >= nS - 1 || flip_var >= nv - 1) return 1;
    engine_t E;
    if (!rates) {
        heston_engine(&E, S, nS, v, nv, r, kappa, theta, sigma, rho, (flags & 2) != 0,
                      flip_spot, flip_var);
        if ((flags & 1) && rho == 0) { op_free(E.M); E.M = NULL; }
        run_schedule(&E, nseg, scheme, nsteps, dt, th, V);
        engine_free(&E);
        return 0;
    }
    /* time-dependent coefficients: step k of the schedule (segments in order)
     * runs on operators built with r = rates[k], the operators rebuilt before
     * every step (what preprocess_operators is documented to do per step,
     * FiniteDifferenceEngineGPU.pyx:163-167). */
    int k = 0;
    for (int sg = 0; sg < nseg; ++sg) {
        for (int s = 0; s < nsteps[sg]; ++s, ++k) {
            heston_engine(&E, S, nS, v, nv, rates[k], kappa, theta, sigma, rho, (flags & 2) != 0,
                          flip_spot, flip_var);
            if ((flags & 1) && rho == 0) { op_free(E.M); E.M = NULL; }
            const int one = 1;
            run_schedule(&E, 1, scheme + sg, &one, dt + sg, th + sg, V);
            engine_free(&E);
        }
    }
    return 0;
}

/* Black-Scholes on a 1-D spot mesh. */
int oracle_bs_solve(const double *S, int nS, double r, double var,
                    int nseg, const int *scheme, const int *nsteps,
                    const double *dt, const double *th, double *V) {
    if (nS < 4) return 1;
    engine_t E;
    bs_engine(&E, S, nS, r, var);
    run_schedule(&E, nseg, scheme, nsteps, dt, th, V);
    engine_free(&E);
    return 0;
}

/* Export the combined Heston operators for structural checks:
 * A0, A1: [5][N] row-aligned diagonals (offsets 2,1,0,-1,-2) in each
 * operator's own block-major order, R0, R1: [N], M9: [N][9] (may be NULL),
 * status: bottom fold status of A1. */
int oracle_heston_operators(const double *S, int nS, const double *v, int nv,
                            double r, double kappa, double theta, double sigma, double rho,
                            double *A0, double *R0, double *A1, double *R1, double *M9,
                            int *status) {
    if (nS < 4 || nv < 4) return 1;
    engine_t E;
    heston_engine(&E, S, nS, v, nv, r, kappa, theta, sigma, rho, 0, -1, -1);
    size_t N = (size_t)nS * nv;
    for (int k = 0; k < 5; ++k) {
        memcpy(A0 + k * N, E.A[0]->d[k], N * sizeof(double));
        memcpy(A1 + k * N, E.A[1]->d[k], N * sizeof(double));
    }
    memcpy(R0, E.A[0]->R, N * sizeof(double));
    memcpy(R1, E.A[1]->R, N * sizeof(double));
    if (M9) memcpy(M9, E.M->m9, N * 9 * sizeof(double));
    status[0] = E.A[0]->top_status; status[1] = E.A[0]->bot_status;
    status[2] = E.A[1]->top_status; status[3] = E.A[1]->bot_status;
    engine_free(&E);
    return 0;
}

/* A batch of independent Heston solves, one OpenMP thread per option. The
 * meshes and grids of option k start at S_off[k], v_off[k], V_off[k]; every
 * option runs the same segment list; barrier (may be NULL) marks up-and-out
 * options. */
int oracle_heston_batch(int n_opt, const double *S, const int64_t *S_off, const int *nS,
                        const double *v, const int64_t *v_off, const int *nv,
                        const double *params /* [n_opt][5]: r kappa theta sigma rho */,
                        int nseg, const int *scheme, const int *nsteps,
                        const double *dt /* [n_opt][nseg] */, const double *th,
                        double *V, const int64_t *V_off, int nthreads, const int *barrier,
                        const double *rates /* [n_opt][total steps] or NULL */) {
    int bad = 0;
    int total = 0;
    for (int sg = 0; sg < nseg; ++sg) total += nsteps[sg];
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
    for (int k = 0; k < n_opt; ++k) {
        const double *p = params + 5 * k;
        bad += oracle_heston_solve(S + S_off[k], nS[k], v + v_off[k], nv[k],
                                   p[0], p[1], p[2], p[3], p[4],
                                   1 | ((barrier && barrier[k]) ? 2 : 0),
                                   nseg, scheme, nsteps, dt + (size_t)k * nseg, th,
                                   V + V_off[k], rates ? rates + (size_t)k * total : NULL);
    }
    return bad;
}
