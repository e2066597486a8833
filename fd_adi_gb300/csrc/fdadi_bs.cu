// Fused, batched Black-Scholes ADI engine (one spatial dimension).
//
// The reference prices Black-Scholes on the GPU by converting the CPU engine
// (FiniteDifferenceEngineGPU.pyx:100-128) and running the same per-step loops
// as for Heston, one option at a time. In one dimension every option is a
// single line and lines are independent, so here one thread owns one option
// for the whole schedule: a single launch runs every option's every step,
// with no synchronisation between steps.
//
// Layout: options are sorted by line length and dealt to slots of 32 (one
// warp). A slot group's arrays are interleaved, element i of lane l at
// base_g + 32 i + l, so every load and store of a warp covers 256 contiguous
// bytes even though each lane walks its own line. The per-point operators
// F = dt A, Le = theta dt A and the Thomas factors of 1 - theta dt A (and of
// the implicit 1 - dt' A) are built once, with the reference's arithmetic
// (fdadi_rows.cuh), so they equal the reference CPU engine's rows bit for bit.
//
// Per step and point: Douglas 11 FP64 instructions, HV 23, MCS 24; the
// stored operator rows keep the per-step work free of the multiplications
// that building F and Le would cost, and the rows' own rounding (a
// coefficient rounded differently would bias every step the same way).
#include <algorithm>
#include <vector>

#include "fdadi_internal.cuh"
#include "fdadi_rows.cuh"

namespace fdadi {
namespace {

constexpr int BS_LANES = 32;
constexpr int BS_THREADS = 128;

// Interleaved per-point arrays, in units of NI doubles.
enum : int {
    BA_V = 0,    // state
    BA_D = 1,    // forward-sweep results d'
    BA_Y0 = 2,   // HV / MCS predictor Y0
    BA_Y1 = 3,   // HV / MCS first solve Y1
    BA_F = 4,    // F = dt A rows: sub, mid, sup (4, 5, 6)
    BA_LE = 7,   // Le = (A theta) dt rows (7, 8, 9)
    BA_LM = 10,  // main Thomas factors: sub, 1/m, c' (10, 11, 12)
    BA_LI = 13,  // implicit Thomas factors (13, 14, 15)
    BA_COUNT = 16
};

struct BsArena {
    int64_t NI;                 // doubles per interleaved array
    int S;                      // slots (32 per group)
    const int *slot_opt;        // [S] option of the slot, -1 if empty
    const int *slot_n;          // [S] line length
    const int64_t *slot_base;   // [S] index of element 0 (group base + lane)
    const int64_t *slot_soff;   // [S] offset of the option in the packed arrays
    double *RF;                 // [S] F's S_max residual: R dt
    double *RI;                 // [S] implicit operator's S_max residual: R (-dt')
    int *ostat;                 // [n_opt] status bits found at prepare
    double *arr;                // [BA_COUNT][NI]
};

struct BsLayout {
    int n_opt = 0, n_groups = 0, S = 0;
    int64_t NI = 0;
    std::vector<int> slot_opt, slot_n;
    std::vector<int64_t> slot_base, slot_soff;
    int64_t o_opt = 0, o_n = 0, o_base = 0, o_soff = 0, o_RF = 0, o_RI = 0, o_stat = 0,
            o_arr = 0, bytes = 0;
};

int bs_layout(const fdadi_bs_batch_t *b, BsLayout &L) {
    FDADI_REQUIRE(b != nullptr, "null batch");
    FDADI_REQUIRE(b->n_options > 0 && b->n, "batch needs options and their sizes");
    FDADI_REQUIRE(b->n_steps >= 0 && b->implicit_steps >= 0, "negative step count");
    FDADI_REQUIRE(b->scheme == FDADI_SCHEME_DOUGLAS || b->scheme == FDADI_SCHEME_HV ||
                      b->scheme == FDADI_SCHEME_CS || b->scheme == FDADI_SCHEME_MCS,
                  "unknown scheme %d", b->scheme);
    const int n = b->n_options;
    L.n_opt = n;
    int nmax = 0;
    for (int k = 0; k < n; ++k) {
        FDADI_REQUIRE(b->n[k] >= 4, "option %d: need >= 4 spot points", k);
        nmax = std::max(nmax, (int)b->n[k]);
    }
    // longest lines first (a stable counting sort), so each warp's lanes walk
    // lines of similar length
    std::vector<int> order(n), start(nmax + 2, 0);
    for (int k = 0; k < n; ++k) ++start[nmax - b->n[k] + 1];
    for (int v = 1; v <= nmax + 1; ++v) start[v] += start[v - 1];
    for (int k = 0; k < n; ++k) order[start[nmax - b->n[k]]++] = k;
    L.n_groups = (n + BS_LANES - 1) / BS_LANES;
    L.S = L.n_groups * BS_LANES;
    L.slot_opt.assign(L.S, -1);
    L.slot_n.assign(L.S, 0);
    L.slot_base.assign(L.S, 0);
    L.slot_soff.assign(L.S, 0);
    std::vector<int64_t> soff(n + 1, 0);
    for (int k = 0; k < n; ++k) soff[k + 1] = soff[k] + b->n[k];
    int64_t base = 0;
    for (int g = 0; g < L.n_groups; ++g) {
        const int len = b->n[order[g * BS_LANES]];
        for (int l = 0; l < BS_LANES; ++l) {
            const int s = g * BS_LANES + l;
            L.slot_base[s] = base + l;
            if (s < n) {
                const int o = order[s];
                L.slot_opt[s] = o;
                L.slot_n[s] = b->n[o];
                L.slot_soff[s] = soff[o];
            }
        }
        base += (int64_t)BS_LANES * len;
    }
    L.NI = base;
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t o = off;
        off += (bytes + 255) & ~(int64_t)255;
        return o;
    };
    L.o_opt = take(4 * (int64_t)L.S);
    L.o_n = take(4 * (int64_t)L.S);
    L.o_base = take(8 * (int64_t)L.S);
    L.o_soff = take(8 * (int64_t)L.S);
    L.o_RF = take(8 * (int64_t)L.S);
    L.o_RI = take(8 * (int64_t)L.S);
    L.o_stat = take(4 * (int64_t)n);
    L.o_arr = take(8 * (int64_t)BA_COUNT * L.NI);
    L.bytes = off;
    return FDADI_OK;
}

BsArena bs_view(const BsLayout &L, char *ws) {
    BsArena A;
    A.NI = L.NI;
    A.S = L.S;
    A.slot_opt = (const int *)(ws + L.o_opt);
    A.slot_n = (const int *)(ws + L.o_n);
    A.slot_base = (const int64_t *)(ws + L.o_base);
    A.slot_soff = (const int64_t *)(ws + L.o_soff);
    A.RF = (double *)(ws + L.o_RF);
    A.RI = (double *)(ws + L.o_RI);
    A.ostat = (int *)(ws + L.o_stat);
    A.arr = (double *)(ws + L.o_arr);
    return A;
}

int bs_check_ws(const BsLayout &L, void *ws, int64_t bytes) {
    FDADI_REQUIRE(ws != nullptr, "null workspace");
    if (bytes < L.bytes) {
        set_error("workspace too small: %lld bytes, need %lld", (long long)bytes,
                  (long long)L.bytes);
        return FDADI_E_WORKSPACE;
    }
    FDADI_REQUIRE(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
    return FDADI_OK;
}

struct BsBuild {
    const double *spots, *params, *dt;
    double theta, dt_factor;
};

// One thread per slot: the operator rows of blackscholes.py:144-239 as
// FiniteDifferenceEngine.pyx:563-592 combines them (r S D_S + 1/2 var S^2
// D_SS, then add_scalar(-r) with the scalar rounded to binary32,
// BandedOperator.pxd:32), scaled for the schemes as the reference's solve_*
// loops scale them (FiniteDifferenceEngine.pyx:617-659, 700-775, 945-1006):
// F = A dt, Le = (A theta) dt, Li = A (theta (-dt)) + 1, implicit
// A (-dt') + 1 with dt' = dt * factor and its residual kept. The Dirichlet
// row at the first mesh point is never scaled (vectorized_scale,
// BandedOperator.pyx:749-792), so it stays (0, 1, 0) in every operator.
__global__ void bs_build_kernel(BsArena A, BsBuild a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= A.S) return;
    const int o = A.slot_opt[s];
    if (o < 0) return;
    const int n = A.slot_n[s];
    const double *S = a.spots + A.slot_soff[s];
    const double r = a.params[2 * (int64_t)o], var = a.params[2 * (int64_t)o + 1];
    const double dt = a.dt[o];
    const float minus_r = (float)(-r / 1.0);
    const double sm = MUL(a.theta, -dt), si = -MUL(dt, a.dt_factor);
    const int64_t NI = A.NI, b = A.slot_base[s];
    double *arr = A.arr;
    Thomas tm, ti;
    for (int i = 0; i < n; ++i) {
        double w[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        spot_weights(S, n, i, w, 1);
        const Row3 row = spot_row_w(w, 1, S, n, i, var, r, minus_r, false);
        const int64_t q = b + (int64_t)BS_LANES * i;
        double f[3], e[3], m[3], im[3];
        if (row.dirichlet) {
            f[0] = e[0] = m[0] = im[0] = 0.0;
            f[1] = e[1] = m[1] = im[1] = 1.0;
            f[2] = e[2] = m[2] = im[2] = 0.0;
        } else {
            const double c[3] = {row.sub, row.mid, row.sup};
            for (int k = 0; k < 3; ++k) {
                f[k] = MUL(c[k], dt);
                e[k] = MUL(MUL(c[k], a.theta), dt);
                m[k] = MUL(c[k], sm);
                im[k] = MUL(c[k], si);
            }
            m[1] = ADD(m[1], 1.0);
            im[1] = ADD(im[1], 1.0);
        }
        for (int k = 0; k < 3; ++k) {
            arr[(BA_F + k) * NI + q] = f[k];
            arr[(BA_LE + k) * NI + q] = e[k];
        }
        tm.row(arr + BA_LM * NI, NI, q, m[0], m[1], m[2], i == 0);
        ti.row(arr + BA_LI * NI, NI, q, im[0], im[1], im[2], i == 0);
        if (i == n - 1) {
            A.RF[s] = MUL(row.R, dt);
            A.RI[s] = MUL(row.R, si);
        }
    }
    A.ostat[o] = (tm.bad || ti.bad) ? FDADI_STATUS_PIVOT : 0;
}

// One lane's line: element i of array k at arr[k NI + base + 32 i].
struct BsLine {
    double *arr;
    int64_t NI, base;
    int n;
    __device__ __forceinline__ double *at(int k) const { return arr + k * NI + base; }
};

constexpr int64_t ST = BS_LANES;  // element stride of a line

// y = F x on row i (1 <= i <= n-1) with x[-1] forced to the Dirichlet value 0
// (apply, BandedOperator.pyx:331-361: force_dirichlet, then the DIA
// matvec's diagonal order +1, 0, -1).
__device__ __forceinline__ double row_apply(const double *c, int64_t NI, int64_t q, bool top,
                                            double xm, double x0, double xp) {
    const double sub = c[q], mid = c[NI + q];
    double acc = top ? mid * x0 : fma(mid, x0, c[2 * NI + q] * xp);
    return fma(sub, xm, acc);
}

// Thomas forward sweep of the rows 1..n-1 given their right-hand sides; row
// 0 is the Dirichlet row (forced to 0, so d'_0 = 0).
// Douglas (and Craig-Sneyd, which in one dimension without a mixed term
// repeats the Douglas sweep and keeps its result): V <- Li^-1 (V + F V - Le V).
__device__ void bs_douglas(const BsLine &l, double rf) {
    const int n = l.n;
    const double *V = l.at(BA_V);
    double *D = l.at(BA_D);
    const double *F = l.at(BA_F), *E = l.at(BA_LE), *M = l.at(BA_LM);
    const int64_t NI = l.NI;
    double xm = 0.0, x0 = V[ST], dp = 0.0;
    D[0] = 0.0;
    for (int i = 1; i < n; ++i) {
        const int64_t q = i * ST;
        const bool top = i == n - 1;
        const double xp = top ? 0.0 : V[q + ST];
        double y = x0 + (row_apply(F, NI, q, top, xm, x0, xp) + (top ? rf : 0.0));
        y = y - row_apply(E, NI, q, top, xm, x0, xp);
        dp = (y - M[q] * dp) * M[NI + q];
        D[q] = dp;
        xm = x0;
        x0 = xp;
    }
    double *Vw = l.at(BA_V);
    double x = dp;
    Vw[(n - 1) * ST] = x;
    for (int i = n - 2; i >= 0; --i) {
        const int64_t q = i * ST;
        x = D[q] - M[2 * NI + q] * x;
        Vw[q] = x;
    }
}

// Implicit step: V <- (1 - dt' A)^-1 (V - R_i) with the residual on the
// S_max row (solve, BandedOperator.pyx:364-394).
__device__ void bs_implicit(const BsLine &l, double ri) {
    const int n = l.n;
    double *V = l.at(BA_V), *D = l.at(BA_D);
    const double *M = l.at(BA_LI);
    const int64_t NI = l.NI;
    double dp = 0.0;
    D[0] = 0.0;
    for (int i = 1; i < n; ++i) {
        const int64_t q = i * ST;
        double y = V[q];
        if (i == n - 1) y = y - ri;
        dp = (y - M[q] * dp) * M[NI + q];
        D[q] = dp;
    }
    double x = dp;
    V[(n - 1) * ST] = x;
    for (int i = n - 2; i >= 0; --i) {
        const int64_t q = i * ST;
        x = D[q] - M[2 * NI + q] * x;
        V[q] = x;
    }
}

// Backward sweep into array k from the forward results in D.
__device__ __forceinline__ void back_into(const BsLine &l, double dp, int k) {
    const int n = l.n;
    const double *D = l.at(BA_D), *M = l.at(BA_LM);
    double *Y = l.at(k);
    double x = dp;
    Y[(n - 1) * ST] = x;
    for (int i = n - 2; i >= 0; --i) {
        const int64_t q = i * ST;
        x = D[q] - M[2 * l.NI + q] * x;
        Y[q] = x;
    }
}

// HV in one dimension (FiniteDifferenceEngine.pyx:700-775):
//   Y0 = V + F V, Y1 = Li^-1 (Y0 - Le V),
//   V <- Li^-1 (Y0 - 1/2 F (V - Y1) - Le Y1), F without its residual there.
// Modified Craig-Sneyd (FiniteDifferenceEngine.pyx:779-841), one dimension,
// no mixed term:
//   Y0 = V + F V, Y1 = Li^-1 (Y0 - Le V),
//   V <- Li^-1 (Y0 + (1/2 - theta) F (Y1 - V) - Le V), F with its residual.
template <bool MCS>
__device__ void bs_two_sweeps(const BsLine &l, double rf, double c) {
    const int n = l.n;
    const int64_t NI = l.NI;
    const double *V = l.at(BA_V), *F = l.at(BA_F), *E = l.at(BA_LE), *M = l.at(BA_LM);
    double *D = l.at(BA_D), *Y0 = l.at(BA_Y0);
    double xm = 0.0, x0 = V[ST], dp = 0.0;
    D[0] = 0.0;
    for (int i = 1; i < n; ++i) {
        const int64_t q = i * ST;
        const bool top = i == n - 1;
        const double xp = top ? 0.0 : V[q + ST];
        const double y0 = x0 + (row_apply(F, NI, q, top, xm, x0, xp) + (top ? rf : 0.0));
        Y0[q] = y0;
        const double z = y0 - row_apply(E, NI, q, top, xm, x0, xp);
        dp = (z - M[q] * dp) * M[NI + q];
        D[q] = dp;
        xm = x0;
        x0 = xp;
    }
    back_into(l, dp, BA_Y1);
    const double *Y1 = l.at(BA_Y1);
    // second sweep: differences D = V - Y1 (HV) or Y1 - V (MCS), each formed
    // once and carried along the window; the Dirichlet row's is forced to 0
    double vm = 0.0, v0 = V[ST], ym = 0.0, y0r = Y1[ST];
    double dm = 0.0, d0 = MCS ? y0r - v0 : v0 - y0r;
    dp = 0.0;
    for (int i = 1; i < n; ++i) {
        const int64_t q = i * ST;
        const bool top = i == n - 1;
        const double vp = top ? 0.0 : V[q + ST], yp = top ? 0.0 : Y1[q + ST];
        const double dpn = top ? 0.0 : (MCS ? yp - vp : vp - yp);
        const double fd = row_apply(F, NI, q, top, dm, d0, dpn);
        double w;
        if (MCS) {
            w = fma(c, fd + (top ? rf : 0.0), Y0[q]);
            w = w - row_apply(E, NI, q, top, vm, v0, vp);
        } else {
            w = fma(-0.5, fd, Y0[q]);
            w = w - row_apply(E, NI, q, top, ym, y0r, yp);
        }
        dp = (w - M[q] * dp) * M[NI + q];
        D[q] = dp;
        vm = v0; v0 = vp;
        ym = y0r; y0r = yp;
        dm = d0; d0 = dpn;
    }
    back_into(l, dp, BA_V);
}

struct BsSched {
    int scheme, n_steps, implicit_steps;
    double theta;
};

// One thread per slot: copy the option's packed state into its interleaved
// line, run the whole schedule, copy the result back.
__global__ void __launch_bounds__(BS_THREADS) bs_run_kernel(BsArena A, double *Vp, BsSched sc) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= A.S) return;
    if (A.slot_opt[s] < 0) return;
    BsLine l{A.arr, A.NI, A.slot_base[s], A.slot_n[s]};
    double *V = l.at(BA_V);
    double *src = Vp + A.slot_soff[s];
    for (int i = 0; i < l.n; ++i) V[i * ST] = src[i];
    const double rf = A.RF[s], ri = A.RI[s];
    for (int k = 0; k < sc.implicit_steps; ++k) bs_implicit(l, ri);
    const double c = 0.5 - sc.theta;
    for (int k = 0; k < sc.n_steps; ++k) {
        if (sc.scheme == FDADI_SCHEME_HV) bs_two_sweeps<false>(l, rf, c);
        else if (sc.scheme == FDADI_SCHEME_MCS) bs_two_sweeps<true>(l, rf, c);
        else bs_douglas(l, rf);
    }
    for (int i = 0; i < l.n; ++i) src[i] = V[i * ST];
}

// One block per option: V = max(S - K, 0) or max(K - S, 0).
__global__ void bs_payoff_kernel(BsArena A, const double *spots, const double *K, int put,
                                 double *Vp) {
    const int s = blockIdx.x;
    const int o = A.slot_opt[s];
    if (o < 0) return;
    const int64_t off = A.slot_soff[s];
    const double k = K[o];
    for (int i = threadIdx.x; i < A.slot_n[s]; i += blockDim.x) {
        const double x = spots[off + i];
        Vp[off + i] = put ? fmax(k - x, 0.0) : fmax(x - k, 0.0);
    }
}

__global__ void bs_status_kernel(BsArena A, const double *Vp, int *status) {
    const int s = blockIdx.x;
    const int o = A.slot_opt[s];
    if (o < 0) return;
    const int64_t off = A.slot_soff[s];
    int bad = 0;
    for (int i = threadIdx.x; i < A.slot_n[s]; i += blockDim.x)
        if (!isfinite(Vp[off + i])) bad = 1;
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) status[o] = A.ostat[o] | (bad ? FDADI_STATUS_NONFINITE : 0);
}

int bs_begin(const fdadi_bs_batch_t *b, void *ws, int64_t bytes, BsLayout &L) {
    int rc = bs_layout(b, L);
    if (rc) return rc;
    return bs_check_ws(L, ws, bytes);
}

}  // namespace
}  // namespace fdadi

using namespace fdadi;

extern "C" {

int64_t fdadi_bs_workspace_bytes(const fdadi_bs_batch_t *b) {
    BsLayout L;
    if (bs_layout(b, L)) return -1;
    return L.bytes;
}

int fdadi_bs_prepare(const fdadi_bs_batch_t *b, void *ws, int64_t bytes, void *stream) {
    BsLayout L;
    int rc = bs_begin(b, ws, bytes, L);
    if (rc) return rc;
    FDADI_REQUIRE(b->spots && b->params && b->dt, "null mesh/params/dt pointer");
    cudaStream_t st = as_stream(stream);
    char *w = (char *)ws;
    FDADI_CUDA(cudaMemcpyAsync(w + L.o_opt, L.slot_opt.data(), 4 * (size_t)L.S,
                               cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(w + L.o_n, L.slot_n.data(), 4 * (size_t)L.S,
                               cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(w + L.o_base, L.slot_base.data(), 8 * (size_t)L.S,
                               cudaMemcpyHostToDevice, st));
    FDADI_CUDA(cudaMemcpyAsync(w + L.o_soff, L.slot_soff.data(), 8 * (size_t)L.S,
                               cudaMemcpyHostToDevice, st));
    // the host tables are locals: wait for their copies before returning
    BsArena A = bs_view(L, w);
    BsBuild a{b->spots, b->params, b->dt, b->theta, b->implicit_dt_factor};
    bs_build_kernel<<<(L.S + BS_THREADS - 1) / BS_THREADS, BS_THREADS, 0, st>>>(A, a);
    FDADI_CHECK_LAUNCH();
    FDADI_CUDA(cudaStreamSynchronize(st));
    return FDADI_OK;
}

int fdadi_bs_run(const fdadi_bs_batch_t *b, void *ws, int64_t bytes, double *V, void *stream) {
    BsLayout L;
    int rc = bs_begin(b, ws, bytes, L);
    if (rc) return rc;
    FDADI_REQUIRE(V != nullptr, "null state");
    BsSched sc{b->scheme, b->n_steps, b->implicit_steps, b->theta};
    bs_run_kernel<<<(L.S + BS_THREADS - 1) / BS_THREADS, BS_THREADS, 0, as_stream(stream)>>>(
        bs_view(L, (char *)ws), V, sc);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_bs_payoff(const fdadi_bs_batch_t *b, void *ws, int64_t bytes, const double *strikes,
                    int32_t put, double *V, void *stream) {
    BsLayout L;
    int rc = bs_begin(b, ws, bytes, L);
    if (rc) return rc;
    FDADI_REQUIRE(strikes && V && b->spots, "null payoff argument");
    bs_payoff_kernel<<<L.S, 128, 0, as_stream(stream)>>>(bs_view(L, (char *)ws), b->spots,
                                                         strikes, put ? 1 : 0, V);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

int fdadi_bs_status(const fdadi_bs_batch_t *b, void *ws, int64_t bytes, const double *V,
                    int32_t *status, void *stream) {
    BsLayout L;
    int rc = bs_begin(b, ws, bytes, L);
    if (rc) return rc;
    FDADI_REQUIRE(V && status, "null state or status array");
    bs_status_kernel<<<L.S, 128, 0, as_stream(stream)>>>(bs_view(L, (char *)ws), V, status);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
}

}  // extern "C"
