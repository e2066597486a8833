// Operator rows and Thomas factors built with the reference's arithmetic:
// shared by the batched Heston and Black-Scholes engines. Every operation is
// an explicitly rounded intrinsic (no contraction), so rows built here equal
// the reference CPU engine's bit for bit.
#pragma once

#include <cuda_runtime.h>

namespace fdadi {

#define MUL(a, b) __dmul_rn((a), (b))
#define ADD(a, b) __dadd_rn((a), (b))
#define SUB(a, b) __dsub_rn((a), (b))
#define DIV(a, b) __ddiv_rn((a), (b))

// ---- operator rows (reference construction) ------------------------------

struct Row3 {
    double sub, mid, sup, R, ext;  // ext: A[n-1, n-3] on the last row of a variance line
    bool dirichlet;
};

// Centred non-uniform stencil of row i (1 <= i <= n-2), centercoeffs
// (BandedOperator.pyx:970-1017).
static __device__ __forceinline__ void centre(const double *x, int i, int derivative,
                                              double &sub, double &mid, double &sup) {
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


// The spot-index parts of a spot operator row, computed once per (option, i)
// so that the per-point builders do no division: w[0..5] = centred first and second
// derivative weights (sub, mid, sup) at an interior row; on the last row
// w[0..2] = the "first derivative = 1" row's mid2, sub2 and R2. Stored at
// w[k * SS + s_off + i].
static __device__ void spot_weights(const double *S, int n, int i, double *w, int64_t SS) {
    if (i == 0) return;
    if (i == n - 1) {
        const double dm1 = SUB(S[n - 1], S[n - 2]);
        const double xx = MUL(dm1, dm1);
        w[0] = DIV(-2.0, xx);
        w[SS] = DIV(2.0, xx);
        w[2 * SS] = DIV(MUL(1.0, 2.0), dm1);
        return;
    }
    double s1, m1, p1, s2, m2, p2;
    centre(S, i, 1, s1, m1, p1);
    centre(S, i, 2, s2, m2, p2);
    w[0] = s1; w[SS] = m1; w[2 * SS] = p1;
    w[3 * SS] = s2; w[4 * SS] = m2; w[5 * SS] = p2;
}

// Combined spot operator A0 = r S D_S + 1/2 v S^2 D_SS - r/2 at row i of the
// spot line through variance v_j: boundaries heston.py:337-342 (Dirichlet
// U = 0 at S = 0, dU/dS = 1 at S_max) or the up-and-out Dirichlet row at S_max
// (heston.py:361-370); combination FiniteDifferenceEngine.pyx:563-592.
// The stencil weights come precomputed per spot index (spot_weights); every
// per-point operation is the reference's, in its order, so the rows are
// bit-identical to building them from the mesh directly.
static __device__ Row3 spot_row_w(const double *w, int64_t SS, const double *S, int n, int i,
                                  double vj, double r, float half_r, bool barrier) {
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
        const double mid2 = w[0], sub2 = w[SS], R2 = w[2 * SS];
        o.mid = ADD(ADD(MUL(0.0, c0), f), MUL(mid2, c00));
        o.sub = ADD(MUL(0.0, c0), MUL(sub2, c00));
        o.sup = 0.0;
        o.R = ADD(MUL(1.0, c0), MUL(R2, c00));
        return o;
    }
    const double s1 = w[0], m1 = w[SS], p1 = w[2 * SS], s2 = w[3 * SS], m2 = w[4 * SS],
                 p2 = w[5 * SS];
    o.sup = ADD(MUL(p1, c0), MUL(p2, c00));
    o.mid = ADD(ADD(MUL(m1, c0), f), MUL(m2, c00));
    o.sub = ADD(MUL(s1, c0), MUL(s2, c00));
    return o;
}

// Thomas factors (a_k, 1/m_k, c'_k) of one line with rows (sub, mid, sup):
// m_0 = mid_0, m_k = mid_k - sub_k c'_{k-1}, c'_k = sup_k / m_k; stored at
// L[q], L[stride + q], L[2 stride + q].
// bad: some pivot m_k was zero or non-finite.
// The factors are formed with the elimination's own operations, each rounded
// once (m = mid - sub c' without a fused multiply-add, c' = sup / m by true
// division), as the reference's banded solve forms them. They are built once
// and reused by every solve of the run, so a factor rounded differently (c' as
// sup times the rounded 1/m) would bias every step the same way: over 1000
// steps of the 1024 x 512 grid that drift reached 1.4e-10 of the price. The
// time loop multiplies by the stored 1/m, whose rounding does not accumulate
// that way.
struct Thomas {
    double cp = 0.0;
    bool bad = false;
    __device__ __forceinline__ void row(double *L, int64_t stride, int64_t q, double sub,
                                        double mid, double sup, bool first) {
        const double m = first ? mid : SUB(mid, MUL(sub, cp));
        const double inv = DIV(1.0, m);
        if (!isfinite(inv)) bad = true;
        cp = DIV(sup, m);
        L[q] = sub;
        L[stride + q] = inv;
        L[2 * stride + q] = cp;
    }
};

}  // namespace fdadi
