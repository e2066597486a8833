// Host-side variance meshes for many options at once.
//
// The reference builds every engine's variance mesh on the host with
// utils.exponential_space (FiniteDifference/utils.py:161-190), in Python
// float arithmetic: v_i = l + (i*dv)**ex, with the upper end stretched so that
// the last point below v0 (in ex-th-root coordinates) lands on it. Python's
// float ** calls the C library's pow() for finite positive operands, so the
// same operations in the same order, compiled without floating-point
// contraction (-ffp-contract=off, no fused multiply-add), give the reference's
// meshes bit for bit. Options are spread over host threads.
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "fdadi_internal.cuh"

namespace {

// utils.py:161-190 for one option; returns 0, or FDADI_E_ARG when no point
// lies below `exact` (the reference's "Did not find suitable value.").
int exponential_space_one(double low, double exact, double high, double ex, int size,
                          int force_exact, double *v) {
    if (size == 1) {
        v[0] = exact;
        return 0;
    }
    const double l = std::pow(low, 1.0 / ex);
    double h = std::pow(high, 1.0 / ex);
    const double x = std::pow(exact, 1.0 / ex);
    double dv = (h - l) / (double)(size - 1);
    if (force_exact) {
        int j = 0;
        for (int i = 0; i < size; ++i) {
            if (l + (double)i * dv > x) {
                j = i - 1;
                break;
            }
        }
        if (j == 0) return FDADI_E_ARG;
        const double dx = x - (l + (double)j * dv);
        h += ((double)(size - 1) * dx) / (double)j;
    }
    dv = (h - l) / (double)(size - 1);
    for (int i = 0; i < size; ++i) v[i] = l + std::pow((double)i * dv, ex);
    return 0;
}

}  // namespace

extern "C" int fdadi_exponential_space(double low, double exact, double high, double ex,
                                       int32_t size, int32_t force_exact, double *out) {
    FDADI_REQUIRE(out && size >= 1, "exponential_space: bad arguments");
    FDADI_REQUIRE(exponential_space_one(low, exact, high, ex, size, force_exact, out) == 0,
                  "Did not find suitable value.");
    return FDADI_OK;
}

extern "C" int fdadi_heston_var_meshes(int32_t n, const double *v0, const int32_t *nv,
                                       double var_max, double varexp, int32_t force_exact,
                                       int32_t threads, double *out) {
    FDADI_REQUIRE(n >= 0 && (n == 0 || (v0 && nv && out)), "var_meshes: bad arguments");
    std::vector<int64_t> off(n + 1, 0);
    for (int32_t k = 0; k < n; ++k) {
        FDADI_REQUIRE(nv[k] >= 1, "var_meshes: option %d has %d variance points", (int)k,
                      (int)nv[k]);
        off[k + 1] = off[k] + nv[k];
    }
    unsigned hw = std::thread::hardware_concurrency();
    int nt = threads > 0 ? threads : (int)(hw ? hw : 1);
    if (nt > 64) nt = 64;
    if (nt > n) nt = n > 0 ? n : 1;
    std::vector<int> bad(nt, -1);
    auto work = [&](int t) {
        for (int32_t k = t; k < n; k += nt)
            if (exponential_space_one(0.0, v0[k], var_max, varexp, nv[k], force_exact,
                                      out + off[k]) != 0 && bad[t] < 0)
                bad[t] = k;
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(work, t);
        for (auto &th : pool) th.join();
    }
    for (int t = 0; t < nt; ++t)
        FDADI_REQUIRE(bad[t] < 0, "Did not find suitable value. (option %d)", bad[t]);
    return FDADI_OK;
}
