// Per-system cell algebra on the host.
//
// These O(1)-per-system steps restate, operation for operation, the cell
// handling of the reference's simulation_system
// (serial_interface/src/serial_chimes_interface.cpp): set_hmat (:85-113), the
// replication count and volume of init (:150-341), the LAMMPS-convention
// rotation of reorient (:342-476) and the ghost-layer count and box checks of
// build_layered_system (:477-534) and run_checks (:866-905).  This file is
// compiled with -ffp-contract=off so every product is rounded before it is
// summed, as in the reference's x86-64 build; the per-atom and per-ghost work
// that uses these matrices runs on the GPU with the same rounding.
#include <cmath>
#include <string>

#include "ck_common.h"
#include "ck_geom.h"

namespace ck {

static double mag3(const double* a) {
    double m = 0;
    for (int i = 0; i < 3; i++) m += a[i] * a[i];
    return std::sqrt(m);
}
static double dot3(const double* a, const double* b) {
    double d = 0;
    for (int i = 0; i < 3; i++) d += a[i] * b[i];
    return d;
}
static double angle3(const double* a, const double* b) {
    double g = dot3(a, b);
    g /= mag3(a);
    g /= mag3(b);
    return std::acos(g);
}

void set_hmat(const double* ca, const double* cb, const double* cc, double* h, double* hi, int rep) {
    h[0] = ca[0] * (rep + 1); h[3] = ca[1] * (rep + 1); h[6] = ca[2] * (rep + 1);
    h[1] = cb[0] * (rep + 1); h[4] = cb[1] * (rep + 1); h[7] = cb[2] * (rep + 1);
    h[2] = cc[0] * (rep + 1); h[5] = cc[1] * (rep + 1); h[8] = cc[2] * (rep + 1);
    double det = h[0] * (h[4] * h[8] - h[5] * h[7]) - h[1] * (h[3] * h[8] - h[5] * h[6]) +
                 h[2] * (h[3] * h[7] - h[4] * h[6]);
    double t[9];
    t[0] = (h[4] * h[8] - h[5] * h[7]);      t[3] = -1 * (h[1] * h[8] - h[2] * h[7]); t[6] = (h[1] * h[5] - h[2] * h[4]);
    t[1] = -1 * (h[3] * h[8] - h[5] * h[6]); t[4] = (h[0] * h[8] - h[2] * h[6]);      t[7] = -1 * (h[0] * h[5] - h[2] * h[3]);
    t[2] = (h[3] * h[7] - h[4] * h[6]);      t[5] = -1 * (h[0] * h[7] - h[1] * h[6]); t[8] = (h[0] * h[4] - h[1] * h[3]);
    hi[0] = t[0]; hi[3] = t[1]; hi[6] = t[2];
    hi[1] = t[3]; hi[4] = t[4]; hi[7] = t[5];
    hi[2] = t[6]; hi[5] = t[7]; hi[8] = t[8];
    for (int i = 0; i < 9; i++) hi[i] /= det;
}

static void lattice(const double* h, double& la, double& lb, double& lc) {
    double A[3] = {h[0], h[3], h[6]}, B[3] = {h[1], h[4], h[7]}, C[3] = {h[2], h[5], h[8]};
    la = mag3(A); lb = mag3(B); lc = mag3(C);
}

static Status layer_check(double la, double lb, double lc, double c2, double c3, double c4, bool has3, bool has4,
                          int& n_layers, std::string& err) {
    double mn = la;
    if (lb < mn) mn = lb;
    if (lc < mn) mn = lc;
    n_layers = (int)std::ceil(c2 * 2.0 / mn + 1);
    int n = n_layers;
    double ex = la * (2 * n + 1), ey = lb * (2 * n + 1), ez = lc * (2 * n + 1);
    if (c2 > 0.5 * ex || c2 > 0.5 * ey || c2 > 0.5 * ez) {
        err = "maximum 2b cutoff is greater than half at least one box length";
        return kErrGeometry;
    }
    if (has3 && (c3 > 0.5 * ex || c3 > 0.5 * ey || c3 > 0.5 * ez)) {
        err = "maximum 3b cutoff is greater than half at least one box length";
        return kErrGeometry;
    }
    if (has4 && (c4 > 0.5 * ex || c4 > 0.5 * ey || c4 > 0.5 * ez)) {
        err = "maximum 4b cutoff is greater than half at least one box length";
        return kErrGeometry;
    }
    return kOk;
}

Status system_geometry(const double* ca, const double* cb, const double* cc, int n_in, bool small,
                       double c2, double c3, double c4, bool has3, bool has4, SysDesc& d, double& vol,
                       std::string& err) {
    if (n_in <= 0) {
        err = "a configuration needs at least one atom";
        return kErrInput;
    }
    // init: replication count from the input cell lengths
    double la = mag3(ca), lb = mag3(cb), lc = mag3(cc);
    double mn = la;
    if (lb < mn) mn = lb;
    if (lc < mn) mn = lc;
    if (!(mn > 0.0) || !std::isfinite(la) || !std::isfinite(lb) || !std::isfinite(lc)) {
        err = "cell vectors must be finite and nonzero";
        return kErrInput;
    }
    {
        double h[9], hi[9];
        set_hmat(ca, cb, cc, h, hi, 0);
        for (double v : hi)
            if (!std::isfinite(v)) {
                err = "cell vectors are linearly dependent";
                return kErrInput;
            }
    }
    if (c2 * 2.0 / mn + 1 > 1000.0) {
        err = "cell is too small for the cutoffs (more than 1000 ghost layers)";
        return kErrInput;
    }
    int n_rep = small ? (int)std::ceil(c2 / mn) - 1 : 0;
    if (n_rep < 0) n_rep = 0;
    set_hmat(ca, cb, cc, d.h0, d.h0i, 0);
    set_hmat(ca, cb, cc, d.h, d.hi, n_rep);
    // init: volume of the (replicated) cell
    {
        double A[3] = {d.h[0], d.h[3], d.h[6]}, B[3] = {d.h[1], d.h[4], d.h[7]}, C[3] = {d.h[2], d.h[5], d.h[8]};
        double sla = mag3(A), slb = mag3(B), slc = mag3(C);
        double al = angle3(B, C), be = angle3(C, A), ga = angle3(A, B);
        double v = 1;
        v += 2 * std::cos(al) * std::cos(be) * std::cos(ga);
        v -= std::cos(al) * std::cos(al);
        v -= std::cos(be) * std::cos(be);
        v -= std::cos(ga) * std::cos(ga);
        vol = sla * slb * slc * std::sqrt(v);
    }
    // reorient: rotated cell (a along x, b in the xy plane)
    {
        double A[3] = {d.h[0], d.h[3], d.h[6]}, B[3] = {d.h[1], d.h[4], d.h[7]}, C[3] = {d.h[2], d.h[5], d.h[8]};
        double ma = mag3(A);
        double u[3] = {0.0 + A[0] / ma, 0.0 + A[1] / ma, 0.0 + A[2] / ma};
        double cr[3] = {(u[1] * B[2] - u[2] * B[1]), -1 * (u[0] * B[2] - u[2] * B[0]), (u[0] * B[1] - u[1] * B[0])};
        double ta[3] = {mag3(A), 0, 0};
        double tb[3] = {dot3(B, u), mag3(cr), 0};
        double tc[3];
        tc[0] = dot3(C, u);
        tc[1] = (dot3(B, C) - tb[0] * tc[0]) / tb[1];
        tc[2] = std::sqrt(mag3(C) * mag3(C) - tc[0] * tc[0] - tc[1] * tc[1]);
        set_hmat(ta, tb, tc, d.hn, d.hni, 0);
    }
    int nl_sys, nl_neigh;
    double sa, sb, sc;
    lattice(d.h, sa, sb, sc);
    Status st = layer_check(sa, sb, sc, c2, c3, c4, has3, has4, nl_sys, err);
    if (st != kOk) return st;
    lattice(d.hn, sa, sb, sc);
    st = layer_check(sa, sb, sc, c2, c3, c4, has3, has4, nl_neigh, err);
    if (st != kOk) return st;
    if (nl_sys != nl_neigh) {
        err = "ghost-layer count differs between the input cell and its reoriented copy";
        return kErrGeometry;
    }
    const int side = 2 * nl_sys + 1;
    const int n_atoms = n_in * (n_rep + 1) * (n_rep + 1) * (n_rep + 1);
    long long n_ghost = (long long)n_atoms * side * side * side;
    int body = 2 + (has3 ? 1 : 0) + (has4 ? 1 : 0);
    if (body > n_ghost) {
        err = "layered system contains too few atoms";
        return kErrGeometry;
    }
    if (n_ghost > 2000000000LL) {
        err = "layered system exceeds 2^31 ghost atoms";
        return kErrInput;
    }
    d.search = c2;
    if (c3 > d.search) d.search = c3;
    if (c4 > d.search) d.search = c4;
    d.c3 = has3 ? c3 : 0.0;
    d.c4 = has4 ? c4 : 0.0;
    d.n_in = n_in;
    d.n_rep = n_rep;
    d.n_atoms = n_atoms;
    d.n_layers = nl_sys;
    d.side = side;
    d.has3 = has3 ? 1 : 0;
    d.has4 = has4 ? 1 : 0;
    // Kept images.  Every list member lies within `search` of a real atom, and
    // real atoms have reoriented fractional coordinates in [0,1).  Along axis k
    // the distance between points whose fractional coordinates differ by du is
    // at least |du| * h_k, h_k the cell height normal to the other two axes, so
    // an image whose coordinate falls outside [-search/h_k, 1 + search/h_k] is
    // never a neighbour.  The 1e-6 slack covers rounding of the stored coordinates.
    {
        const double* H = d.hn;
        const double A[3] = {H[0], H[3], H[6]}, B[3] = {H[1], H[4], H[7]}, C[3] = {H[2], H[5], H[8]};
        auto cross = [](const double* x, const double* y, double* o) {
            o[0] = x[1] * y[2] - x[2] * y[1];
            o[1] = x[2] * y[0] - x[0] * y[2];
            o[2] = x[0] * y[1] - x[1] * y[0];
        };
        double bc[3], ca[3], ab[3];
        cross(B, C, bc);
        cross(C, A, ca);
        cross(A, B, ab);
        const double V = std::fabs(A[0] * bc[0] + A[1] * bc[1] + A[2] * bc[2]);
        const double hgt[3] = {V / mag3(bc), V / mag3(ca), V / mag3(ab)};
        int stride = 1;
        double ext = 0.0;
        for (int k = 0; k < 3; k++) {
            const double w = d.search / hgt[k];
            d.ulo[k] = -w - 1e-6;
            d.uhi[k] = 1.0 + w + 1e-6;
            int cnt = (int)std::floor(d.uhi[k] - d.ulo[k] + 1e-9) + 1;
            if (cnt > side) cnt = side;
            stride *= cnt;
            for (int j = 0; j < 3; j++) ext += std::fabs(H[3 * k + j]) * (d.n_layers + 1);
        }
        d.gstride = stride;
        // FP32 copies of coordinates up to `ext` carry errors below 2e-7 * ext
        d.eps = 2e-3 + 1e-6 * ext;
    }
    if ((long long)n_atoms * d.gstride > 2000000000LL) {
        err = "ghost slots exceed 2^31";
        return kErrInput;
    }
    // Bin-grid capacity: the ghost cloud spans at most (2n+1) * sum_j |hn_ij| per axis.
    long long cap = 1;
    for (int i = 0; i < 3; i++) {
        double ext = 0;
        for (int j = 0; j < 3; j++) ext += std::fabs(d.hn[3 * i + j]);
        ext *= side;
        long long nb = (long long)std::ceil(ext / d.search) + 2;
        cap *= nb;
    }
    if (cap > 1000000000LL) {
        err = "bin grid too large";
        return kErrInput;
    }
    d.bin_cap = (int)cap;
    // FP32 thresholds of the enumeration's pair tests (c -/+ eps), rounded outward
    auto down = [](double v) {
        float f = (float)v;
        if ((double)f > v) f = std::nextafter(f, -INFINITY);
        return f;
    };
    auto up = [](double v) {
        float f = (float)v;
        if ((double)f < v) f = std::nextafter(f, INFINITY);
        return f;
    };
    d.c3lo = down(d.c3 - d.eps);
    d.c3hi = up(d.c3 + d.eps);
    d.c4lo = down(d.c4 - d.eps);
    d.c4hi = up(d.c4 + d.eps);
    auto sq_down = [&](float v) { return v > 0.0f ? down((double)v * v) : -1.0f; };
    auto sq_up = [&](float v) { return up((double)v * v); };
    d.c3lo2 = sq_down(d.c3lo);
    d.c3hi2 = sq_up(d.c3hi);
    d.c4lo2 = sq_down(d.c4lo);
    d.c4hi2 = sq_up(d.c4hi);
    d.far2 = (float)((d.search + d.eps) * (d.search + d.eps));
    d.near2 = d.search > d.eps ? (float)((d.search - d.eps) * (d.search - d.eps)) : 0.0f;
    return kOk;
}

}  // namespace ck
