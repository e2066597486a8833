// Per-operator kernels of the BandedOperator API (the unfused path).
//
// One thread owns one line of an operator and walks it sequentially, so the
// strided direction (axis 0: lines are grid columns) is read with adjacent
// threads on adjacent columns -- coalesced, with no transpose -- and the
// contiguous direction is read through L1. These kernels reproduce the
// reference operator semantics exactly (Dirichlet forcing, folding, residual);
// the fused engine in fdadi_engine.cu is the fast path.
#include <stdarg.h>
#include <string.h>



#include "fdadi_internal.cuh"

namespace fdadi {

static thread_local char g_err[512];

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

// Address of element k of line b in a [n0][n1] grid for an operator on `axis`.
struct LineMap {
    int64_t base, stride;
    __device__ __forceinline__ LineMap(int axis, int64_t b, int64_t n1) {
        if (axis == 0) { base = b; stride = n1; }
        else { base = b * n1; stride = 1; }
    }
    __device__ __forceinline__ int64_t operator()(int64_t k) const { return base + k * stride; }
};

__global__ void tri_apply_kernel(fdadi_tri_t op, const double *__restrict__ x, double *y,
                                 int64_t n1) {
    const int64_t L = op.operator_rows / op.blocks;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < op.blocks;
         b += (int64_t)gridDim.x * blockDim.x) {
        LineMap at(op.axis, b, n1);
        const int64_t r0 = b * L;
        const bool lowd = op.has_low_dirichlet, highd = op.has_high_dirichlet;
        auto xin = [&](int64_t k) -> double {
            if (k == 0 && lowd) return op.low_dirichlet[b];
            if (k == L - 1 && highd) return op.high_dirichlet[b];
            return x[at(k)];
        };
        double xm2 = 0.0, xm1 = 0.0, x0 = xin(0), x1 = xin(1);
        const double x2 = L > 2 ? xin(2) : 0.0;
        const double x_l3 = L > 2 ? xin(L - 3) : 0.0;
        double xp2 = x2;   // x[k + 2]
        const bool band = op.sup2 != nullptr;
        double yprev = 0.0, y0 = 0.0;
        for (int64_t k = 0; k < L; ++k) {
            const int64_t r = r0 + k;
            double acc = 0.0;
            if (band && k >= 1 && k + 2 < L) acc += op.sup2[r] * xp2;
            if (k + 1 < L) acc += op.sup[r] * x1;
            acc += op.mid[r] * x0;
            if (k >= 1) acc += op.sub[r] * xm1;
            if (band && k >= 2 && k < L - 1) acc += op.sub2[r] * xm2;
            if (k == 0 && op.top_fold_status == FDADI_CAN_FOLD) acc += op.top_factors[b] * x2;
            if (k == L - 1 && op.bottom_fold_status == FDADI_CAN_FOLD)
                acc += op.bottom_factors[b] * x_l3;
            double yk = acc;
            // the residual is added after unfolding; unfolding needs the
            // neighbouring product, so row 0 is finished once row 1 is known
            if (k == L - 1 && op.bottom_fold_status == FDADI_FOLDED)
                yk += -1.0 * yprev * op.bottom_factors[b];
            if (k >= 1) {
                double ywrite = yprev;
                if (k == 1) {
                    ywrite = y0;
                    if (op.top_fold_status == FDADI_FOLDED) ywrite += -1.0 * acc * op.top_factors[b];
                }
                if (op.has_residual) ywrite += op.R[r - 1];
                y[at(k - 1)] = ywrite;
            } else {
                y0 = acc;
            }
            yprev = acc;
            if (k == L - 1) {
                if (op.has_residual) yk += op.R[r];
                y[at(k)] = yk;
            }
            xm2 = xm1;
            xm1 = x0;
            x0 = x1;
            if (k + 2 < L) x1 = xin(k + 2);
            if (band && k + 3 < L) xp2 = xin(k + 3);
        }
    }
}

__global__ void tri_solve_kernel(fdadi_tri_t op, double *x, int64_t n1, double *scratch) {
    const int64_t L = op.operator_rows / op.blocks;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < op.blocks;
         b += (int64_t)gridDim.x * blockDim.x) {
        LineMap at(op.axis, b, n1);
        const int64_t r0 = b * L;
        const bool lowd = op.has_low_dirichlet, highd = op.has_high_dirichlet;
        auto rhs = [&](int64_t k) -> double {
            double v;
            if (k == 0 && lowd) v = op.low_dirichlet[b];
            else if (k == L - 1 && highd) v = op.high_dirichlet[b];
            else v = x[at(k)];
            if (op.has_residual) v = v - op.R[r0 + k];
            return v;
        };
        // row 0 and row L-1 after folding
        double sup0 = op.sup[r0], mid0 = op.mid[r0];
        double midn = op.mid[r0 + L - 1], subn = op.sub[r0 + L - 1];
        double ftop = 0.0, fbot = 0.0;
        bool top = false, bot = false;
        if (op.top_fold_status == FDADI_FOLDED) { ftop = op.top_factors[b]; top = true; }
        else if (op.top_fold_status == FDADI_CAN_FOLD) {
            const double d0 = op.top_factors[b], c1 = op.sup[r0 + 1];
            ftop = c1 != 0.0 ? -d0 / c1 : 0.0;
            sup0 += op.mid[r0 + 1] * ftop;
            mid0 += op.sub[r0 + 1] * ftop;
            top = true;
        }
        if (op.bottom_fold_status == FDADI_FOLDED) { fbot = op.bottom_factors[b]; bot = true; }
        else if (op.bottom_fold_status == FDADI_CAN_FOLD) {
            const double zn = op.bottom_factors[b], an1 = op.sub[r0 + L - 2];
            fbot = an1 != 0.0 ? -zn / an1 : 0.0;
            subn += op.mid[r0 + L - 2] * fbot;
            midn += op.sup[r0 + L - 2] * fbot;
            bot = true;
        }
        // forward elimination: scratch holds c', x holds d'
        double r_0 = rhs(0), r_1 = rhs(1);
        if (top) r_0 += 1.0 * r_1 * ftop;
        double cp = sup0 / mid0, dp = r_0 / mid0;
        scratch[r0] = cp;
        x[at(0)] = dp;
        double rprev = r_1;  // raw right-hand side of row k-1 (for the bottom fold)
        double rk = r_1;
        for (int64_t k = 1; k < L; ++k) {
            const int64_t r = r0 + k;
            const double rnext = (k + 1 < L) ? rhs(k + 1) : 0.0;
            double sub = op.sub[r], mid = op.mid[r], sup = (k + 1 < L) ? op.sup[r] : 0.0;
            double rr = rk;
            if (k == L - 1) {
                sub = subn;
                mid = midn;
                if (bot) rr += 1.0 * rprev * fbot;
            }
            const double m = mid - sub * cp;
            cp = sup / m;
            dp = (rr - sub * dp) / m;
            scratch[r] = cp;
            x[at(k)] = dp;
            rprev = rk;
            rk = rnext;
        }
        double xn = dp;
        for (int64_t k = L - 2; k >= 0; --k) {
            xn = x[at(k)] - scratch[r0 + k] * xn;
            x[at(k)] = xn;
        }
    }
}

// Banded solve of one line per thread: rows (A[k,k-2] .. A[k,k+2]), the
// corner entries from the CAN_FOLD slots, eliminated top to bottom without row
// exchanges, each row update rounded as written (no fused multiply-add), in
// the order of a plain band elimination. The factored upper band (u0, u1, u2)
// goes to scratch [3N], the forward-eliminated right-hand side to x; then back
// substitution.
struct BandRow {
    double b2, b1, a0, a1, a2, r;
};

__global__ void band_solve_kernel(fdadi_tri_t op, double *x, int64_t n1, double *scratch) {
    const int64_t N = op.operator_rows, L = op.operator_rows / op.blocks;
    double *U0 = scratch, *U1 = scratch + N, *U2 = scratch + 2 * N;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < op.blocks;
         b += (int64_t)gridDim.x * blockDim.x) {
        LineMap at(op.axis, b, n1);
        const int64_t r0 = b * L;
        const bool lowd = op.has_low_dirichlet, highd = op.has_high_dirichlet;
        auto row = [&](int64_t k) -> BandRow {
            BandRow w{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            if (k >= L) return w;
            const int64_t r = r0 + k;
            double v;
            if (k == 0 && lowd) v = op.low_dirichlet[b];
            else if (k == L - 1 && highd) v = op.high_dirichlet[b];
            else v = x[at(k)];
            if (op.has_residual) v = v - op.R[r];
            w.r = v;
            w.a0 = op.mid[r];
            if (k + 1 < L) w.a1 = op.sup[r];
            if (k >= 1) w.b1 = op.sub[r];
            if (k + 2 < L)
                w.a2 = k == 0 ? (op.top_fold_status == FDADI_CAN_FOLD ? op.top_factors[b] : 0.0)
                              : op.sup2[r];
            if (k >= 2)
                w.b2 = k == L - 1
                           ? (op.bottom_fold_status == FDADI_CAN_FOLD ? op.bottom_factors[b] : 0.0)
                           : op.sub2[r];
            return w;
        };
        BandRow c0 = row(0), c1 = row(1), c2 = row(2);
        for (int64_t k = 0; k < L; ++k) {
            const double p = c0.a0;
            if (k + 1 < L) {
                const double l = __ddiv_rn(c1.b1, p);
                c1.a0 = __dsub_rn(c1.a0, __dmul_rn(l, c0.a1));
                c1.a1 = __dsub_rn(c1.a1, __dmul_rn(l, c0.a2));
                c1.r = __dsub_rn(c1.r, __dmul_rn(l, c0.r));
            }
            if (k + 2 < L) {
                const double l = __ddiv_rn(c2.b2, p);
                c2.b1 = __dsub_rn(c2.b1, __dmul_rn(l, c0.a1));
                c2.a0 = __dsub_rn(c2.a0, __dmul_rn(l, c0.a2));
                c2.r = __dsub_rn(c2.r, __dmul_rn(l, c0.r));
            }
            const int64_t r = r0 + k;
            U0[r] = c0.a0; U1[r] = c0.a1; U2[r] = c0.a2;
            x[at(k)] = c0.r;
            c0 = c1;
            c1 = c2;
            c2 = row(k + 3);
        }
        double xk1 = 0.0, xk2 = 0.0;
        for (int64_t k = L - 1; k >= 0; --k) {
            const int64_t r = r0 + k;
            double acc = x[at(k)];
            if (k + 1 < L) acc = __dsub_rn(acc, __dmul_rn(U1[r], xk1));
            if (k + 2 < L) acc = __dsub_rn(acc, __dmul_rn(U2[r], xk2));
            const double xk = __ddiv_rn(acc, U0[r]);
            x[at(k)] = xk;
            xk2 = xk1;
            xk1 = xk;
        }
    }
}

__global__ void tri_scale_kernel(fdadi_tri_t op, const double *__restrict__ vec, double scalar) {
    const int64_t N = op.operator_rows, L = op.operator_rows / op.blocks;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = r % L, b = r / L;
        double v = vec ? vec[r] : scalar;
        if ((k == 0 && op.has_low_dirichlet) || (k == L - 1 && op.has_high_dirichlet)) v = 1.0;
        op.sup[r] *= v;
        op.mid[r] *= v;
        op.sub[r] *= v;
        op.R[r] *= v;
        if (op.sup2) { op.sup2[r] *= v; op.sub2[r] *= v; }
        if (k == 0 && op.top_fold_status == FDADI_CAN_FOLD) op.top_factors[b] *= v;
        if (k == L - 1 && op.bottom_fold_status == FDADI_CAN_FOLD) op.bottom_factors[b] *= v;
    }
}

__global__ void tri_add_scalar_kernel(fdadi_tri_t op, double value) {
    const int64_t N = op.operator_rows, L = op.operator_rows / op.blocks;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = r % L;
        if ((k == 0 && op.has_low_dirichlet) || (k == L - 1 && op.has_high_dirichlet)) continue;
        op.mid[r] += value;
    }
}

__global__ void tri_add_operator_kernel(fdadi_tri_t a, fdadi_tri_t o) {
    const int64_t N = a.operator_rows, L = a.operator_rows / a.blocks;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = r % L, b = r / L;
        a.sup[r] += o.sup[r];
        a.sub[r] += o.sub[r];
        if (o.sup2) { a.sup2[r] += o.sup2[r]; a.sub2[r] += o.sub2[r]; }
        if (!((k == 0 && a.has_low_dirichlet) || (k == L - 1 && a.has_high_dirichlet)))
            a.mid[r] += o.mid[r];
        a.R[r] += o.R[r];
        if (k == 0 && o.top_fold_status == FDADI_CAN_FOLD) {
            a.top_factors[b] = (a.top_fold_status == FDADI_CAN_FOLD ? a.top_factors[b] : 0.0) +
                               o.top_factors[b];
        }
        if (k == L - 1 && o.bottom_fold_status == FDADI_CAN_FOLD) {
            a.bottom_factors[b] =
                (a.bottom_fold_status == FDADI_CAN_FOLD ? a.bottom_factors[b] : 0.0) +
                o.bottom_factors[b];
        }
    }
}

__global__ void tri_fold_kernel(fdadi_tri_t op, int top, int bottom, int unfold) {
    const int64_t L = op.operator_rows / op.blocks;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < op.blocks;
         b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r0 = b * L, rn = r0 + L - 1;
        if (top) {
            if (!unfold) {
                const double d0 = op.top_factors[b], c1 = op.sup[r0 + 1];
                const double f = c1 != 0.0 ? -d0 / c1 : 0.0;
                op.sup[r0] += op.mid[r0 + 1] * f;
                op.mid[r0] += op.sub[r0 + 1] * f;
                op.top_factors[b] = f;
            } else {
                const double f = op.top_factors[b];
                op.top_factors[b] = 0.0 - op.sup[r0 + 1] * f;
                op.sup[r0] -= op.mid[r0 + 1] * f;
                op.mid[r0] -= op.sub[r0 + 1] * f;
            }
        }
        if (bottom) {
            if (!unfold) {
                const double zn = op.bottom_factors[b], an1 = op.sub[rn - 1];
                const double f = an1 != 0.0 ? -zn / an1 : 0.0;
                op.sub[rn] += op.mid[rn - 1] * f;
                op.mid[rn] += op.sup[rn - 1] * f;
                op.bottom_factors[b] = f;
            } else {
                const double f = op.bottom_factors[b];
                op.bottom_factors[b] = 0.0 - op.sub[rn - 1] * f;
                op.sub[rn] -= op.mid[rn - 1] * f;
                op.mid[rn] -= op.sup[rn - 1] * f;
            }
        }
    }
}

__global__ void mixed_apply_kernel(fdadi_mixed_t op, const double *__restrict__ x,
                                   double *__restrict__ y) {
    const int64_t n0 = op.n0, n1 = op.n1, N = n0 * n1;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = p / n1, j = p - i * n1;
        double acc = 0.0;
        if (i > 0 && i < n0 - 1 && j > 0 && j < n1 - 1) {
            const double b0 = op.w1[j], b1 = op.w1[n1 + j], b2 = op.w1[2 * n1 + j];
            const double *xm = x + p - n1, *xc = x + p, *xp = x + p + n1;
            const double tm = b0 * xm[-1] + b1 * xm[0] + b2 * xm[1];
            const double tc = b0 * xc[-1] + b1 * xc[0] + b2 * xc[1];
            const double tp = b0 * xp[-1] + b1 * xp[0] + b2 * xp[1];
            acc = op.coeff[p] * (op.w0[i] * tm + op.w0[n0 + i] * tc + op.w0[2 * n0 + i] * tp);
        }
        if (op.has_residual) acc += op.R[p];
        y[p] = acc;
    }
}

__global__ void mixed_scale_kernel(fdadi_mixed_t op, const double *__restrict__ vec, double scalar) {
    const int64_t N = op.n0 * op.n1;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < N;
         p += (int64_t)gridDim.x * blockDim.x) {
        const double v = vec ? vec[p] : scalar;
        op.coeff[p] *= v;
        op.R[p] *= v;
    }
}

__global__ void axpby_kernel(double *y, const double *__restrict__ x, double a, double b, int64_t n) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x)
        y[p] = a * y[p] + b * x[p];
}

static int check_tri(const fdadi_tri_t *op, int64_t n0, int64_t n1, bool grid) {
    FDADI_REQUIRE(op != nullptr, "null operator");
    FDADI_REQUIRE(op->blocks > 0 && op->operator_rows > 0 && op->operator_rows % op->blocks == 0,
                  "Vector length does not divide into blocks (%lld rows, %lld blocks)",
                  (long long)op->operator_rows, (long long)op->blocks);
    FDADI_REQUIRE(op->operator_rows / op->blocks >= 4,
                  "Vector too short to use finite differencing.");
    FDADI_REQUIRE(op->axis == 0 || op->axis == 1, "axis must be 0 or 1");
    FDADI_REQUIRE(op->sup && op->mid && op->sub && op->R && op->low_dirichlet &&
                      op->high_dirichlet && op->top_factors && op->bottom_factors,
                  "operator has a null array");
    FDADI_REQUIRE((op->sup2 == nullptr) == (op->sub2 == nullptr),
                  "sup2 and sub2 must both be set or both be NULL");
    FDADI_REQUIRE(!op->sup2 || (op->top_fold_status != FDADI_FOLDED &&
                                op->bottom_fold_status != FDADI_FOLDED),
                  "a folded operator has no second off-diagonals (diagonalize drops them)");
    if (grid) {
        FDADI_REQUIRE(n0 > 0 && n1 > 0 && n0 * n1 == op->operator_rows,
                      "Dimension mismatch: grid %lld x %lld vs %lld operator rows",
                      (long long)n0, (long long)n1, (long long)op->operator_rows);
        FDADI_REQUIRE((op->axis == 0 ? n1 : n0) == op->blocks,
                      "Dimension mismatch: %lld blocks on axis %d of a %lld x %lld grid",
                      (long long)op->blocks, op->axis, (long long)n0, (long long)n1);
    }
    return FDADI_OK;
}

}  // namespace fdadi

using namespace fdadi;

extern "C" {

int fdadi_version(void) { return 10000; }

int fdadi_last_error(char *buf, size_t len) {
    size_t n = strlen(g_err);
    if (buf && len) {
        size_t m = n < len - 1 ? n : len - 1;
        memcpy(buf, g_err, m);
        buf[m] = 0;
    }
    return (int)n;
}

int fdadi_tri_apply(const fdadi_tri_t *op, const double *x, double *y, int64_t n0, int64_t n1,
                    void *stream) {
    int rc = check_tri(op, n0, n1, true);
    if (rc) return rc;
    FDADI_REQUIRE(x && y, "null grid pointer");
    const int threads = 128;
    tri_apply_kernel<<<grid_for(op->blocks, threads), threads, 0, as_stream(stream)>>>(*op, x, y, n1);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_tri_solve(const fdadi_tri_t *op, double *x, int64_t n0, int64_t n1, double *scratch,
                    void *stream) {
    int rc = check_tri(op, n0, n1, true);
    if (rc) return rc;
    FDADI_REQUIRE(x && scratch, "null grid or scratch pointer");
    const int threads = 128;
    if (op->sup2)
        band_solve_kernel<<<grid_for(op->blocks, threads), threads, 0, as_stream(stream)>>>(
            *op, x, n1, scratch);
    else
        tri_solve_kernel<<<grid_for(op->blocks, threads), threads, 0, as_stream(stream)>>>(
            *op, x, n1, scratch);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_tri_scale(fdadi_tri_t *op, const double *vec, double scalar, void *stream) {
    int rc = check_tri(op, 0, 0, false);
    if (rc) return rc;
    if (op->top_fold_status == FDADI_FOLDED || op->bottom_fold_status == FDADI_FOLDED) {
        set_error("Cannot scale a diagonalized (folded) operator.");
        return FDADI_E_STATE;
    }
    const int threads = 256;
    tri_scale_kernel<<<grid_for(op->operator_rows, threads), threads, 0, as_stream(stream)>>>(
        *op, vec, scalar);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_tri_add_scalar(fdadi_tri_t *op, double value, void *stream) {
    int rc = check_tri(op, 0, 0, false);
    if (rc) return rc;
    const int threads = 256;
    tri_add_scalar_kernel<<<grid_for(op->operator_rows, threads), threads, 0,
                            as_stream(stream)>>>(*op, value);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_tri_add_operator(fdadi_tri_t *self, const fdadi_tri_t *other, void *stream) {
    int rc = check_tri(self, 0, 0, false);
    if (rc) return rc;
    rc = check_tri(other, 0, 0, false);
    if (rc) return rc;
    FDADI_REQUIRE(self->axis == other->axis,
                  "Both operators must operate on the same axis. (%d != %d)", self->axis,
                  other->axis);
    FDADI_REQUIRE(self->operator_rows == other->operator_rows && self->blocks == other->blocks,
                  "Both operators must have the same length");
    FDADI_REQUIRE(!other->sup2 || self->sup2,
                  "add_operator: the operator added to must carry second off-diagonals too");
    if (self->top_fold_status == FDADI_FOLDED || self->bottom_fold_status == FDADI_FOLDED ||
        other->top_fold_status == FDADI_FOLDED || other->bottom_fold_status == FDADI_FOLDED) {
        set_error("Cannot add diagonalized operators.");
        return FDADI_E_STATE;
    }
    const int threads = 256;
    tri_add_operator_kernel<<<grid_for(self->operator_rows, threads), threads, 0,
                              as_stream(stream)>>>(*self, *other);
    FDADI_CHECK_LAUNCH();
    if (other->top_fold_status == FDADI_CAN_FOLD) self->top_fold_status = FDADI_CAN_FOLD;
    if (other->bottom_fold_status == FDADI_CAN_FOLD) self->bottom_fold_status = FDADI_CAN_FOLD;
    return FDADI_OK;
}

int fdadi_tri_fold(fdadi_tri_t *op, int32_t top, int32_t bottom, int32_t unfold, void *stream) {
    int rc = check_tri(op, 0, 0, false);
    if (rc) return rc;
    const int want = unfold ? FDADI_FOLDED : FDADI_CAN_FOLD;
    int t = top && op->top_fold_status == want;
    int b = bottom && op->bottom_fold_status == want;
    if (!t && !b) return FDADI_OK;
    const int threads = 128;
    tri_fold_kernel<<<grid_for(op->blocks, threads), threads, 0, as_stream(stream)>>>(*op, t, b,
                                                                                     unfold);
    FDADI_CHECK_LAUNCH();
    const int to = unfold ? FDADI_CAN_FOLD : FDADI_FOLDED;
    if (t) op->top_fold_status = to;
    if (b) op->bottom_fold_status = to;
    return FDADI_OK;
}

int fdadi_mixed_apply(const fdadi_mixed_t *op, const double *x, double *y, void *stream) {
    FDADI_REQUIRE(op && op->coeff && op->w0 && op->w1 && op->R, "mixed operator has a null array");
    FDADI_REQUIRE(op->n0 >= 3 && op->n1 >= 3, "mixed operator needs a 3x3 grid at least");
    FDADI_REQUIRE(x && y && x != y, "mixed apply needs distinct input and output grids");
    const int threads = 256;
    mixed_apply_kernel<<<grid_for(op->n0 * op->n1, threads), threads, 0, as_stream(stream)>>>(
        *op, x, y);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_mixed_scale(fdadi_mixed_t *op, const double *vec, double scalar, void *stream) {
    FDADI_REQUIRE(op && op->coeff && op->R, "mixed operator has a null array");
    const int threads = 256;
    mixed_scale_kernel<<<grid_for(op->n0 * op->n1, threads), threads, 0, as_stream(stream)>>>(
        *op, vec, scalar);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_axpby(double *y, const double *x, double a, double b, int64_t n, void *stream) {
    FDADI_REQUIRE(y && x && n >= 0, "bad axpby arguments");
    if (n == 0) return FDADI_OK;
    const int threads = 256;
    axpby_kernel<<<grid_for(n, threads), threads, 0, as_stream(stream)>>>(y, x, a, b, n);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

}  // extern "C"

// ---- tridiagonal solve without caller scratch -----------------------------
//
// Some callers cannot allocate device memory themselves: a host application
// that hands out every byte of device memory from its own fixed pool and
// forbids components to call cudaMalloc, or a latency-critical pricing loop
// where cudaMalloc/cudaFree would synchronize the whole device between
// requests. fdadi_tri_solve asks them for an operator-sized scratch buffer;
// fdadi_tri_solve_noalloc instead uses the library's own scratch below, a
// fixed array that every device which loads the library holds until the
// process exits.
//
// The array is one per device and shared by every call: calls whose kernels
// overlap on the GPU (different streams, different host threads) race on it,
// so the caller must order them. The solve writes every scratch element it
// reads before reading it, so the contents a previous call left behind never
// matter and nothing needs clearing.

namespace fdadi {

// FDADI_NOALLOC_MAX_ROWS doubles (8 MiB) per device.
static __device__ __align__(256) double g_noalloc_scratch[FDADI_NOALLOC_MAX_ROWS];

// Device address of g_noalloc_scratch on the current device (host code cannot
// use the symbol itself as a pointer). It is looked up on every call rather
// than cached: after cudaDeviceReset the module is loaded again and the array
// may sit at a new address, so a cached pointer could go stale. Once the
// module is loaded on the device the lookup does not synchronize or allocate.
static int noalloc_scratch(double **out) {
    void *p = nullptr;
    FDADI_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    *out = static_cast<double *>(p);
    return FDADI_OK;
}

}  // namespace fdadi

extern "C" int fdadi_tri_solve_noalloc(const fdadi_tri_t *op, double *x, int64_t n0, int64_t n1,
                                       void *stream) {
    int rc = check_tri(op, n0, n1, true);
    if (rc) return rc;
    FDADI_REQUIRE(x, "null grid pointer");
    FDADI_REQUIRE(!op->sup2, "fdadi_tri_solve_noalloc: tridiagonal operators only (this one has "
                             "second off-diagonals); use fdadi_tri_solve");
    FDADI_REQUIRE(op->operator_rows <= FDADI_NOALLOC_MAX_ROWS,
                  "fdadi_tri_solve_noalloc: %lld operator rows exceed the library scratch of %d "
                  "rows; use fdadi_tri_solve with caller scratch",
                  (long long)op->operator_rows, (int)FDADI_NOALLOC_MAX_ROWS);
    double *scratch = nullptr;
    rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    const int threads = 128;
    tri_solve_kernel<<<grid_for(op->blocks, threads), threads, 0, as_stream(stream)>>>(*op, x, n1,
                                                                                      scratch);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}
