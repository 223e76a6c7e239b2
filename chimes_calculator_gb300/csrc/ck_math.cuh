// Device math shared by the cluster kernels: Morse coordinate, Chebyshev
// tables, smoothing cutoff, cluster pair topology and the per-precision
// coefficient accessors.  Restated from chimesFF (chimesFF/src/chimesFF.h:347-386
// get_fcut, :542-628 set_cheby_polys; chimesFF/src/chimesFF.cpp:1572-1613
// set_polys_out_of_range).
#pragma once
#include <cuda_runtime.h>

#include "ck_common.h"

namespace ck {
namespace {

constexpr double kPi = 3.14159265359;   // the reference's `pi` macro (chimesFF.h:22)

template <typename CT> __device__ __forceinline__ void csincos(CT x, CT* s, CT* c);
template <> __device__ __forceinline__ void csincos<double>(double x, double* s, double* c) { sincos(x, s, c); }
template <> __device__ __forceinline__ void csincos<float>(float x, float* s, float* c) { sincosf(x, s, c); }

template <typename CT> __device__ __forceinline__ const CT* coef2(const DevParamSet& P);
template <> __device__ __forceinline__ const double* coef2<double>(const DevParamSet& P) { return P.c2d; }
template <> __device__ __forceinline__ const float* coef2<float>(const DevParamSet& P) { return P.c2f; }
template <typename CT, int NB> __device__ __forceinline__ const CT* coefn(const DevParamSet& P);
template <> __device__ __forceinline__ const double* coefn<double, 3>(const DevParamSet& P) { return P.c3d; }
template <> __device__ __forceinline__ const float* coefn<float, 3>(const DevParamSet& P) { return P.c3f; }
template <> __device__ __forceinline__ const double* coefn<double, 4>(const DevParamSet& P) { return P.c4d; }
template <> __device__ __forceinline__ const float* coefn<float, 4>(const DevParamSet& P) { return P.c4f; }

// get_fcut (chimesFF.h:347-386), evaluated in CT
template <typename CT>
__device__ __forceinline__ void fcut_eval(const DevParamSet& P, double r, double rc, CT& fc, CT& fcd) {
    if (!P.tersoff) {
        CT f0 = CT(1.0) - CT(r) / CT(rc);
        fc = f0 * f0 * f0;
        fcd = f0 * f0 * (CT(-3.0) / CT(rc));
    } else {
        const double th = rc - P.fcut_var * rc;
        if (r < th) { fc = CT(1); fcd = CT(0); }
        else if (r > rc) { fc = CT(0); fcd = CT(0); }
        else {
            const CT inv = CT(1.0) / CT(rc - th);
            const CT f0 = CT(r - th) * inv * CT(kPi) + CT(kPi / 2.0);
            CT sn, cs;
            csincos<CT>(f0, &sn, &cs);
            fc = CT(0.5) + CT(0.5) * sn;
            fcd = CT(0.5) * cs * (CT(kPi) * inv);
        }
    }
}

// Morse coordinate: x and dx/dr at r (clamped to rin below the inner cutoff).
// The exponential and the map are taken in FP64 in both precision modes: the
// polynomial recursion magnifies an error in x by up to n^2.
__device__ __forceinline__ void morse_x(double r, double rin, double lam, double xavg, double xdiff,
                                        double& x, double& dxdr, bool& oor) {
    oor = r < rin;
    const double rr = oor ? rin : r;
    const double e = exp(-rr / lam);
    x = (e - xavg) / xdiff;
    dxdr = (-e / lam) / xdiff;
}

// Chebyshev table T[0..o], dT/dr[0..o] (set_cheby_polys and
// set_polys_out_of_range, chimesFF.cpp:1572-1613) into a strided array.
template <typename CT>
__device__ __forceinline__ void cheby_table(CT* T, CT* D, double r, double rin, double lam, double xavg,
                                            double xdiff, int order, double inner_smooth, int* flags) {
    double xd, dxdr;
    bool oor;
    morse_x(r, rin, lam, xavg, xdiff, xd, dxdr, oor);
    const CT x = CT(xd), tx = CT(2) * x, g = CT(dxdr);
    CT t0 = CT(1), t1 = x, u0 = CT(1), u1 = tx;
    T[0] = t0; D[0] = CT(0);
    if (order >= 1) { T[1] = t1; D[1] = g * u0; }
    for (int n = 2; n <= order; n++) {
        const CT t2 = tx * t1 - t0;
        const CT u2 = tx * u1 - u0;
        T[n] = t2;
        D[n] = CT(n) * g * u1;
        t0 = t1; t1 = t2; u0 = u1; u1 = u2;
    }
    if (oor) {
        if (flags) atomicAdd(&flags[4], 1);   // global device flags, or null
        const double damp = exp((r - rin) / inner_smooth);
        const CT k = CT(inner_smooth * (damp - 1.0)), dm = CT(damp);
        for (int n = 0; n <= order; n++) {
            T[n] = T[n] + k * D[n];
            D[n] = D[n] * dm;
        }
    }
}

// The same table from a precomputed Morse coordinate (x, dx/dr, r below the
// inner cutoff), entries n = 0..nT-1 only, at T[n*stride], D[n*stride]
// (interleaved per-cluster tables of the factored contraction).
template <typename CT>
__device__ __forceinline__ void cheby_fill_strided(CT* T, CT* D, int stride, int nT, double xd, double dxdr, bool oor,
                                                   double r, double rin, double inner_smooth, int* flags) {
    const CT x = CT(xd), tx = CT(2) * x, g = CT(dxdr);
    CT k = CT(0), dm = CT(1);
    if (oor) {
        if (flags) atomicAdd(&flags[4], 1);
        const double damp = exp((r - rin) / inner_smooth);
        k = CT(inner_smooth * (damp - 1.0));
        dm = CT(damp);
    }
    // n = 0: T = 1, dT = 0
    T[0] = CT(1);
    D[0] = CT(0);
    CT t0 = CT(1), t1 = x, u0 = CT(1), u1 = tx;
    if (nT > 1) {
        const CT d1 = g * u0;
        T[stride] = oor ? t1 + k * d1 : t1;
        D[stride] = oor ? d1 * dm : d1;
    }
    for (int n = 2; n < nT; n++) {
        const CT t2 = tx * t1 - t0;
        const CT u2 = tx * u1 - u0;
        const CT dn = CT(n) * g * u1;
        T[n * stride] = oor ? t2 + k * dn : t2;
        D[n * stride] = oor ? dn * dm : dn;
        t0 = t1; t1 = t2; u0 = u1; u1 = u2;
    }
}

template <int NB>
struct Topo;
template <>
struct Topo<3> {
    static constexpr int NP = 3;
    __device__ static int a(int p) { return p == 2 ? 1 : 0; }
    __device__ static int b(int p) { return p == 0 ? 1 : 2; }
};
template <>
struct Topo<4> {
    static constexpr int NP = 6;
    __device__ static int a(int p) { return p < 3 ? 0 : (p < 5 ? 1 : 2); }
    __device__ static int b(int p) { return p < 3 ? p + 1 : (p == 3 ? 2 : 3); }
};


}  // namespace
}  // namespace ck
