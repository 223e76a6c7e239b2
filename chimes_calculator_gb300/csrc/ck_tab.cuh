// Tabulated 2-body and 3-body terms (the reference's TABULATION build, used by
// its LAMMPS pair style): table look-up instead of the Chebyshev expansion.
//
//   2-body: get_tab_2B (chimesFF/src/chimesFF.cpp:1869-1922) -- the grid
//           interval from a binary search (std::lower_bound semantics), then a
//           local cubic whose coefficients the host precomputed per interval;
//   3-body: interpolateTricubic / get_tab_3B (:2353-2463) -- 4x4x4 grid points
//           around the cluster's (rij, rik, rjk), Catmull-Rom along rjk, rik,
//           rij in turn, for the energy and the three force scalars at once.
//
// tab2_lookup and tab3_lookup round every multiply and add separately
// (__dmul_rn / __dadd_rn), in the reference's order, so their results are the
// reference's bit for bit (the per-cluster entry uses them).  The pair-style
// kernel uses tab3_lookup_sep, the same interpolant as one separable weighted
// sum with fused multiply-adds (FP64-pipe bound: a quarter of the operations).
#pragma once
#include <cuda_runtime.h>

#include "ck_common.h"

namespace ck {

// Status of a look-up (also the bit the kernels raise in flags[5]).
enum TabStatus : int {
    kTabOk = 0,
    kTabBelow2 = 1,   // 2-body distance at or below the first usable grid point (the reference exits)
    kTabPast3 = 2,    // 3-body grid index past the table's rows (the reference reads past its vectors)
};

__device__ __forceinline__ double tab_cubic_eval(const double* q, double dx) {
    // a + b*dx + c*dx*dx + d*dx*dx*dx, left to right
    double v = __dadd_rn(q[0], __dmul_rn(q[1], dx));
    v = __dadd_rn(v, __dmul_rn(__dmul_rn(q[2], dx), dx));
    return __dadd_rn(v, __dmul_rn(__dmul_rn(__dmul_rn(q[3], dx), dx), dx));
}

// Energy and force scalar of a tabulated pair type at distance r.  Zero past
// the last interval, as the reference returns 0 there.
__device__ __forceinline__ int tab2_lookup(const DevParamSet& P, int pair, double r, double& E, double& F) {
    E = 0.0;
    F = 0.0;
    const Tab2Rec T = P.t2rec[pair];
    const double* x = P.tab2r + T.off;
    // first grid point not below r
    int lo = 0, len = T.n;
    while (len > 0) {
        const int half = len >> 1;
        if (x[lo + half] < r) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    int i = lo;
    if (i == T.n) return kTabOk;
    if (i == 0) return kTabBelow2;
    if (r == x[i] && i > 0) i--;
    if (i >= T.n - 1) return kTabOk;
    if (i <= 0) return kTabBelow2;
    const double dx = __dsub_rn(r, x[i]);
    const double* q = P.tab2c + 8 * (T.off + i);
    E = tab_cubic_eval(q, dx);
    F = tab_cubic_eval(q + 4, dx);
    return kTabOk;
}

// cubicInterpolate (:2339-2342): p1 + 0.5*x*(p2 - p0 + x*(2*p0 - 5*p1 + 4*p2 - p3 + x*(3*(p1 - p2) + p3 - p0)))
__device__ __forceinline__ double tab_catmull(double p0, double p1, double p2, double p3, double x) {
    const double i3 = __dsub_rn(__dadd_rn(__dmul_rn(3.0, __dsub_rn(p1, p2)), p3), p0);
    const double i2 = __dadd_rn(
        __dsub_rn(__dadd_rn(__dsub_rn(__dmul_rn(2.0, p0), __dmul_rn(5.0, p1)), __dmul_rn(4.0, p2)), p3),
        __dmul_rn(x, i3));
    const double i1 = __dadd_rn(__dsub_rn(p2, p0), __dmul_rn(x, i2));
    return __dadd_rn(p1, __dmul_rn(__dmul_rn(0.5, x), i1));
}

// Energy and force scalars (ij, ik, jk) of tabulated triplet type t at the
// cluster's distances; out = {E, F_ij, F_ik, F_jk}.
__device__ __forceinline__ int tab3_lookup(const DevParamSet& P, int t, double rij, double rik, double rjk,
                                           double* out) {
    const Tab3Rec T = P.t3rec[t];
    const double* cij = P.tab3r + 3 * T.off;
    const double* cik = cij + T.nrows;
    const double* cjk = cik + T.nrows;
    const double* val = P.tab3v + 4 * T.off;
    const int n = T.size;
    const long long nn = (long long)n * n;
    int i = __double2int_rz(__dmul_rn(__dsub_rn(rij, cij[0]), T.inv));
    int j = __double2int_rz(__dmul_rn(__dsub_rn(rik, cik[0]), T.inv));
    int k = __double2int_rz(__dmul_rn(__dsub_rn(rjk, cjk[0]), T.inv));
    i = max(1, i);
    j = max(1, j);
    k = max(1, k);
    // the fractional offsets read the grid rows at (i, j, k), (0, j, k), (0, 0, k)
    const long long ri = nn * i + (long long)n * j + k, rj = (long long)n * j + k, rk = k;
    if (ri >= T.nrows || rj >= T.nrows || rk >= T.nrows) {
        for (int w = 0; w < 4; w++) out[w] = 0.0;
        return kTabPast3;
    }
    const double xi = __dmul_rn(__dsub_rn(rij, cij[ri]), T.inv);
    const double yi = __dmul_rn(__dsub_rn(rik, cik[rj]), T.inv);
    const double zi = __dmul_rn(__dsub_rn(rjk, cjk[rk]), T.inv);
    // grid points outside the table (index >= size along any axis) count as zero
    double a_di[4][4];   // [value][di]
    for (int di = 0; di < 4; di++) {
        double a_dj[4][4];   // [value][dj]
        for (int dj = 0; dj < 4; dj++) {
            double p[4][4];   // [value][dk]
            for (int dk = 0; dk < 4; dk++) {
                const int ti = i + di - 1, tj = j + dj - 1, tk = k + dk - 1;
                if (ti < n && tj < n && tk < n) {
                    const double* v = val + 4 * (nn * ti + (long long)n * tj + tk);
                    for (int w = 0; w < 4; w++) p[w][dk] = v[w];
                } else {
                    for (int w = 0; w < 4; w++) p[w][dk] = 0.0;
                }
            }
            for (int w = 0; w < 4; w++) a_dj[w][dj] = tab_catmull(p[w][0], p[w][1], p[w][2], p[w][3], zi);
        }
        for (int w = 0; w < 4; w++) a_di[w][di] = tab_catmull(a_dj[w][0], a_dj[w][1], a_dj[w][2], a_dj[w][3], yi);
    }
    for (int w = 0; w < 4; w++) out[w] = tab_catmull(a_di[w][0], a_di[w][1], a_di[w][2], a_di[w][3], xi);
    return kTabOk;
}

// Catmull-Rom weights of offset x for the points at -1, 0, 1, 2:
// cubicInterpolate(p0, p1, p2, p3, x) = sum_k w[k] p[k].
__device__ __forceinline__ void tab_catmull_weights(double x, double* w) {
    const double x2 = x * x, x3 = x2 * x;
    w[0] = 0.5 * (-x + 2.0 * x2 - x3);
    w[1] = 0.5 * (2.0 - 5.0 * x2 + 3.0 * x3);
    w[2] = 0.5 * (x + 4.0 * x2 - 3.0 * x3);
    w[3] = 0.5 * (-x2 + x3);
}

// The same tricubic look-up as tab3_lookup, evaluated as the separable sum
// sum_{di,dj,dk} wx[di] wy[dj] wz[dk] v(i+di-1, j+dj-1, k+dk-1) with fused
// multiply-adds: the reference's interpolant up to rounding (about 1e-16
// relative), with a quarter of its FP64 operations (the FP64 pipe bounds this
// look-up).  Grid indices, range rules and out-of-table zeros as in tab3_lookup.
__device__ __forceinline__ int tab3_lookup_sep(const DevParamSet& P, int t, double rij, double rik, double rjk,
                                               double* out) {
    const Tab3Rec T = P.t3rec[t];
    const double* cij = P.tab3r + 3 * T.off;
    const double* cik = cij + T.nrows;
    const double* cjk = cik + T.nrows;
    const double* val = P.tab3v + 4 * T.off;
    const int n = T.size;
    const long long nn = (long long)n * n;
    int i = __double2int_rz(__dmul_rn(__dsub_rn(rij, cij[0]), T.inv));
    int j = __double2int_rz(__dmul_rn(__dsub_rn(rik, cik[0]), T.inv));
    int k = __double2int_rz(__dmul_rn(__dsub_rn(rjk, cjk[0]), T.inv));
    i = max(1, i);
    j = max(1, j);
    k = max(1, k);
    const long long ri = nn * i + (long long)n * j + k, rj = (long long)n * j + k, rk = k;
    for (int w = 0; w < 4; w++) out[w] = 0.0;
    if (ri >= T.nrows || rj >= T.nrows || rk >= T.nrows) return kTabPast3;
    double wx[4], wy[4], wz[4];
    tab_catmull_weights(__dmul_rn(__dsub_rn(rij, cij[ri]), T.inv), wx);
    tab_catmull_weights(__dmul_rn(__dsub_rn(rik, cik[rj]), T.inv), wy);
    tab_catmull_weights(__dmul_rn(__dsub_rn(rjk, cjk[rk]), T.inv), wz);
    for (int di = 0; di < 4; di++) {
        const int ti = i + di - 1;
        if (ti >= n) break;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int dj = 0; dj < 4; dj++) {
            const int tj = j + dj - 1;
            if (tj >= n) break;
            // a grid row's values are 32 bytes (E, F_ij, F_ik, F_jk): two 16-byte loads
            const double2* row = reinterpret_cast<const double2*>(val + 4 * (nn * ti + (long long)n * tj));
            double r4[4] = {0.0, 0.0, 0.0, 0.0};
            for (int dk = 0; dk < 4; dk++) {
                const int tk = k + dk - 1;
                if (tk >= n) break;
                const double2 a = row[2 * tk], b = row[2 * tk + 1];
                r4[0] = fma(wz[dk], a.x, r4[0]);
                r4[1] = fma(wz[dk], a.y, r4[1]);
                r4[2] = fma(wz[dk], b.x, r4[2]);
                r4[3] = fma(wz[dk], b.y, r4[3]);
            }
            for (int w = 0; w < 4; w++) acc[w] = fma(wy[dj], r4[w], acc[w]);
        }
        for (int w = 0; w < 4; w++) out[w] = fma(wx[di], acc[w], out[w]);
    }
    return kTabOk;
}

}  // namespace ck
