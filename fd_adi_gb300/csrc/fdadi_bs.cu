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
// warp). A slot group's arrays are interleaved by row: array k of row i of
// lane l sits at base_g + (16 i + k) 32 + l. Every load and store of a warp
// covers 256 contiguous bytes even though each lane walks its own line, and
// all 16 values of a row lie within 4 KB of one address register (the array
// index is an immediate offset). The per-point operators
// F = dt A, Le = theta dt A and the Thomas factors of 1 - theta dt A (and of
// the implicit 1 - dt' A) are built once, with the reference's arithmetic
// (fdadi_rows.cuh), so they equal the reference CPU engine's rows bit for bit.
//
// Per step and point: Douglas 11 FP64 instructions, HV 23, MCS 24; the
// stored operator rows keep the per-step work free of the multiplications
// that building F and Le would cost, and the rows' own rounding (a
// coefficient rounded differently would bias every step the same way).
//
// A thread's rows stream from HBM (a large batch's rows do not fit in L2)
// and each row's arithmetic is short, so the sweeps keep several rows in
// flight: cp.async copies into a per-thread ring in shared memory.
#include <algorithm>
#include <vector>

#include "fdadi_internal.cuh"
#include "fdadi_rows.cuh"

namespace fdadi {
namespace {

constexpr int BS_LANES = 32;
constexpr int BS_THREADS = 128;

// Per-point arrays of a row (array k at offset 32 k within the row).
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

constexpr int64_t ST = BS_LANES;             // stride between a row's arrays
constexpr int64_t RS = BS_LANES * BA_COUNT;  // stride between rows of a line

struct BsArena {
    int S;                      // slots (32 per group)
    const int *slot_opt;        // [S] option of the slot, -1 if empty
    const int *slot_n;          // [S] line length
    const int64_t *slot_base;   // [S] index of row 0, array 0 (group base + lane)
    const int64_t *slot_soff;   // [S] offset of the option in the packed arrays
    double *RF;                 // [S] F's S_max residual: R dt
    double *RI;                 // [S] implicit operator's S_max residual: R (-dt')
    int *ostat;                 // [n_opt] status bits found at prepare
    double *arr;                // [rows][BA_COUNT][32] per group
};

struct BsLayout {
    int n_opt = 0, n_groups = 0, S = 0;
    int64_t NI = 0;             // doubles of all groups' arrays
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
        base += (int64_t)BS_LANES * BA_COUNT * len;
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
    L.o_arr = take(8 * L.NI);
    L.bytes = off;
    return FDADI_OK;
}

BsArena bs_view(const BsLayout &L, char *ws) {
    BsArena A;
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
    double *p = A.arr + A.slot_base[s];
    Thomas tm, ti;
    for (int i = 0; i < n; ++i) {
        double w[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        spot_weights(S, n, i, w, 1);
        const Row3 row = spot_row_w(w, 1, S, n, i, var, r, minus_r, false);
        const int64_t q = (int64_t)i * RS;
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
            p[q + (BA_F + k) * ST] = f[k];
            p[q + (BA_LE + k) * ST] = e[k];
        }
        tm.row(p, ST, q + BA_LM * ST, m[0], m[1], m[2], i == 0);
        ti.row(p, ST, q + BA_LI * ST, im[0], im[1], im[2], i == 0);
        if (i == n - 1) {
            A.RF[s] = MUL(row.R, dt);
            A.RI[s] = MUL(row.R, si);
        }
    }
    A.ostat[o] = (tm.bad || ti.bad) ? FDADI_STATUS_PIVOT : 0;
}

// One lane's line: array k of row i at p[RS i + ST k].
struct BsLine {
    double *p;
    int n;
    __device__ __forceinline__ double &at(int i, int k) const {
        return p[(int64_t)i * RS + k * ST];
    }
};

// ---- asynchronous row ring -------------------------------------------------
//
// Every row's operands are independent of the recurrence, so they can be
// fetched long before the row is eliminated. Each thread keeps a ring of
// rows in shared memory, filled by cp.async (8-byte copies, no registers
// held while they fly): value v of ring slot s of lane l at
// ring[(s * NV + v) * 32 + l], NV the values a row of that sweep needs
// (the ring holds RING_W of them a slot). PF rows are in flight in the forward
// sweeps, PFB in the back substitutions (two values a row, one FP64
// instruction: the same latency needs more rows). A thread reads only what
// its own copies wrote, after waiting for them, so no barrier is needed.
constexpr int RING_W = 11;  // values a forward-sweep row needs (second HV sweep)

__device__ __forceinline__ void cp_async8(double *dst, const double *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Runs body(i, slot) for i = lo, lo + dir, ... (count rows), slot holding
// row i as issue(i, slot) requested it (NV values, stride 32). PF: power of 2.
template <int PF, int NV, class Issue, class Body>
__device__ __forceinline__ void ring_sweep(double *ring, int lo, int count, int dir, Issue issue,
                                           Body body) {
#pragma unroll
    for (int d = 0; d < PF; ++d) {
        if (d < count) issue(lo + d * dir, ring + d * NV * 32);
        cp_commit();
    }
    for (int k = 0; k < count; ++k) {
        cp_wait<PF - 1>();
        double *slot = ring + (k & (PF - 1)) * NV * 32;
        body(lo + k * dir, slot);
        if (k + PF < count) issue(lo + (k + PF) * dir, slot);
        cp_commit();
    }
}

// y = c x on row i (1 <= i <= n-1) with x[-1] forced to the Dirichlet value 0
// (apply, BandedOperator.pyx:331-361: force_dirichlet, then the DIA
// matvec's diagonal order +1, 0, -1); the last row has no +1 entry.
__device__ __forceinline__ double row_apply(double sub, double mid, double sup, bool top,
                                            double xm, double x0, double xp) {
    const double acc = top ? mid * x0 : fma(mid, x0, sup * xp);
    return fma(sub, xm, acc);
}

// Forward-sweep row operands: slot values 0..8 = V[i+1], F (3), Le (3),
// elimination factors (sub, 1/m); the second HV sweep adds Y1[i+1] and Y0[i]
// at 9 and 10. On the last row the "next" values are fetched from the row
// itself (always inside the line) and ignored.
template <bool WITH_Y>
__device__ __forceinline__ void issue_sweep(const BsLine &l, int i, double *slot) {
    const double *q = l.p + (int64_t)i * RS;
    const double *nx = i == l.n - 1 ? q : q + RS;
    cp_async8(slot, nx + BA_V * ST);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        cp_async8(slot + (1 + k) * 32, q + (BA_F + k) * ST);
        cp_async8(slot + (4 + k) * 32, q + (BA_LE + k) * ST);
    }
    cp_async8(slot + 7 * 32, q + BA_LM * ST);
    cp_async8(slot + 8 * 32, q + (BA_LM + 1) * ST);
    if (WITH_Y) {
        cp_async8(slot + 9 * 32, nx + BA_Y1 * ST);
        cp_async8(slot + 10 * 32, q + BA_Y0 * ST);
    }
}

// Back substitution x_i = d'_i - c'_i x_{i+1} into array k (factors of
// array fac), from x_{n-1} = d'_{n-1} = dp.
template <int PFB>
__device__ __forceinline__ void back_into(const BsLine &l, double *ring, double dp, int k,
                                          int fac) {
    const int n = l.n;
    l.at(n - 1, k) = dp;
    double x = dp;
    ring_sweep<PFB, 2>(
        ring, n - 2, n - 1, -1,
        [&](int i, double *slot) {
            const double *q = l.p + (int64_t)i * RS;
            cp_async8(slot, q + BA_D * ST);
            cp_async8(slot + 32, q + (fac + 2) * ST);
        },
        [&](int i, const double *slot) {
            x = slot[0] - slot[32] * x;
            l.at(i, k) = x;
        });
}

// Douglas (and Craig-Sneyd, which in one dimension without a mixed term
// repeats the Douglas sweep and keeps its result): V <- Li^-1 (V + F V - Le V).
// Row 0 is the Dirichlet row, forced to 0 (d'_0 = 0).
template <int PF, int PFB>
__device__ void bs_douglas(const BsLine &l, double *ring, double rf) {
    const int n = l.n;
    double xm = 0.0, x0 = l.at(1, BA_V), dp = 0.0;
    l.at(0, BA_D) = 0.0;
    ring_sweep<PF, RING_W>(
        ring, 1, n - 1, 1, [&](int i, double *slot) { issue_sweep<false>(l, i, slot); },
        [&](int i, const double *r) {
            const bool top = i == n - 1;
            const double xp = top ? 0.0 : r[0];
            double y = x0 + (row_apply(r[32], r[64], r[96], top, xm, x0, xp) + (top ? rf : 0.0));
            y = y - row_apply(r[128], r[160], r[192], top, xm, x0, xp);
            dp = (y - r[224] * dp) * r[256];
            l.at(i, BA_D) = dp;
            xm = x0;
            x0 = xp;
        });
    back_into<PFB>(l, ring, dp, BA_V, BA_LM);
}

// Implicit step: V <- (1 - dt' A)^-1 (V - R_i) with the residual on the
// S_max row (solve, BandedOperator.pyx:364-394).
template <int PF, int PFB>
__device__ void bs_implicit(const BsLine &l, double *ring, double ri) {
    const int n = l.n;
    double dp = 0.0;
    l.at(0, BA_D) = 0.0;
    ring_sweep<PF, 3>(
        ring, 1, n - 1, 1,
        [&](int i, double *slot) {
            const double *q = l.p + (int64_t)i * RS;
            cp_async8(slot, q + BA_V * ST);
            cp_async8(slot + 32, q + BA_LI * ST);
            cp_async8(slot + 64, q + (BA_LI + 1) * ST);
        },
        [&](int i, const double *r) {
            const double y = i == n - 1 ? r[0] - ri : r[0];
            dp = (y - r[32] * dp) * r[64];
            l.at(i, BA_D) = dp;
        });
    back_into<PFB>(l, ring, dp, BA_V, BA_LI);
}

// HV in one dimension (FiniteDifferenceEngine.pyx:700-775):
//   Y0 = V + F V, Y1 = Li^-1 (Y0 - Le V),
//   V <- Li^-1 (Y0 - 1/2 F (V - Y1) - Le Y1), F without its residual there.
// Modified Craig-Sneyd (FiniteDifferenceEngine.pyx:779-841), one dimension,
// no mixed term:
//   Y0 = V + F V, Y1 = Li^-1 (Y0 - Le V),
//   V <- Li^-1 (Y0 + (1/2 - theta) F (Y1 - V) - Le V), F with its residual.
template <bool MCS, int PF, int PFB>
__device__ void bs_two_sweeps(const BsLine &l, double *ring, double rf, double c) {
    const int n = l.n;
    const double v1 = l.at(1, BA_V);
    double xm = 0.0, x0 = v1, dp = 0.0;
    l.at(0, BA_D) = 0.0;
    ring_sweep<PF, RING_W>(
        ring, 1, n - 1, 1, [&](int i, double *slot) { issue_sweep<false>(l, i, slot); },
        [&](int i, const double *r) {
            const bool top = i == n - 1;
            const double xp = top ? 0.0 : r[0];
            const double y0 =
                x0 + (row_apply(r[32], r[64], r[96], top, xm, x0, xp) + (top ? rf : 0.0));
            l.at(i, BA_Y0) = y0;
            const double z = y0 - row_apply(r[128], r[160], r[192], top, xm, x0, xp);
            dp = (z - r[224] * dp) * r[256];
            l.at(i, BA_D) = dp;
            xm = x0;
            x0 = xp;
        });
    back_into<PFB>(l, ring, dp, BA_Y1, BA_LM);
    // second sweep: differences D = V - Y1 (HV) or Y1 - V (MCS), each formed
    // once and carried along the window; the Dirichlet row's is forced to 0
    const double y1 = l.at(1, BA_Y1);
    double vm = 0.0, v0 = v1, ym = 0.0, y0r = y1;
    double dm = 0.0, d0 = MCS ? y0r - v0 : v0 - y0r;
    dp = 0.0;
    ring_sweep<PF, RING_W>(
        ring, 1, n - 1, 1, [&](int i, double *slot) { issue_sweep<true>(l, i, slot); },
        [&](int i, const double *r) {
            const bool top = i == n - 1;
            const double vp = top ? 0.0 : r[0], yp = top ? 0.0 : r[288];
            const double dpn = top ? 0.0 : (MCS ? yp - vp : vp - yp);
            const double fd = row_apply(r[32], r[64], r[96], top, dm, d0, dpn);
            double w;
            if (MCS) {
                w = fma(c, fd + (top ? rf : 0.0), r[320]);
                w = w - row_apply(r[128], r[160], r[192], top, vm, v0, vp);
            } else {
                w = fma(-0.5, fd, r[320]);
                w = w - row_apply(r[128], r[160], r[192], top, ym, y0r, yp);
            }
            dp = (w - r[224] * dp) * r[256];
            l.at(i, BA_D) = dp;
            vm = v0; v0 = vp;
            ym = y0r; y0r = yp;
            dm = d0; d0 = dpn;
        });
    back_into<PFB>(l, ring, dp, BA_V, BA_LM);
}

struct BsSched {
    int scheme, n_steps, implicit_steps;
    double theta;
};

// One thread per slot: copy the option's packed state into its interleaved
// line, run the whole schedule, copy the result back.
// PF rows in flight in the forward sweeps, PFB in the back substitutions,
// held in a shared-memory ring of PF * RING_W values per thread. MINB: the
// blocks per SM the registers must allow (the ring's shared memory allows
// four blocks at PF 4, two at PF 8).
template <int PF, int PFB, int MINB>
__global__ void __launch_bounds__(BS_THREADS, MINB) bs_run_kernel(BsArena A, double *Vp,
                                                                  BsSched sc) {
    static_assert(PFB * 2 <= PF * RING_W, "back ring must fit the forward ring");
    extern __shared__ double bs_ring[];
    double *ring = bs_ring + (threadIdx.x / 32) * (PF * RING_W * 32) + (threadIdx.x & 31);
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= A.S) return;
    if (A.slot_opt[s] < 0) return;
    const BsLine l{A.arr + A.slot_base[s], A.slot_n[s]};
    double *src = Vp + A.slot_soff[s];
    for (int i = 0; i < l.n; ++i) l.at(i, BA_V) = src[i];
    const double rf = A.RF[s], ri = A.RI[s];
    for (int k = 0; k < sc.implicit_steps; ++k) bs_implicit<PF, PFB>(l, ring, ri);
    const double c = 0.5 - sc.theta;
    for (int k = 0; k < sc.n_steps; ++k) {
        if (sc.scheme == FDADI_SCHEME_HV) bs_two_sweeps<false, PF, PFB>(l, ring, rf, c);
        else if (sc.scheme == FDADI_SCHEME_MCS) bs_two_sweeps<true, PF, PFB>(l, ring, rf, c);
        else bs_douglas<PF, PFB>(l, ring, rf);
    }
    for (int i = 0; i < l.n; ++i) src[i] = l.at(i, BA_V);
}

template <int PF, int PFB, int MINB>
int launch_run(const BsArena &A, double *V, const BsSched &sc, unsigned grid, cudaStream_t st) {
    const size_t smem = (size_t)BS_THREADS * PF * RING_W * sizeof(double);
    if (smem > 48 * 1024)
        FDADI_CUDA(cudaFuncSetAttribute(bs_run_kernel<PF, PFB, MINB>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    bs_run_kernel<PF, PFB, MINB><<<grid, BS_THREADS, smem, st>>>(A, V, sc);
    FDADI_CHECK_LAUNCH();
    return FDADI_OK;
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
    FDADI_REQUIRE(b->prefetch == 0 || b->prefetch == 2 || b->prefetch == 4 || b->prefetch == 8,
                  "prefetch must be 0 (by batch size), 2, 4 or 8");
    BsSched sc{b->scheme, b->n_steps, b->implicit_steps, b->theta};
    // rows in flight: 8 (32 in the back substitutions; 88 KB of ring a block)
    // measured fastest at 65,536 options (199 ms against 266 ms with 4 and
    // 265 ms with 2, although it allows two blocks an SM instead of four) and
    // level with the others at 4096 and 16,384
    const int pf = b->prefetch == 0 ? 8 : b->prefetch;
    const unsigned grid = (L.S + BS_THREADS - 1) / BS_THREADS;
    cudaStream_t st = as_stream(stream);
    const BsArena A = bs_view(L, (char *)ws);
    if (pf == 2) return launch_run<2, 8, 4>(A, V, sc, grid, st);
    if (pf == 4) return launch_run<4, 16, 4>(A, V, sc, grid, st);
    return launch_run<8, 32, 2>(A, V, sc, grid, st);
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
