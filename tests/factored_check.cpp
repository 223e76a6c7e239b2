// Host check of the factored coefficient tables (pack_params): for every valid
// 3-/4-body tuple of a parameter file, random Chebyshev tables T_p, dT_p give
// the same S = sum a prod T and G_p = sum a dT_p prod_{q!=p} T through the
// per-coefficient packed powers and through the row/column factored lists
// (whose last entry per record carries the record-end bit).
// The tensor-core images of the tuples (3-body at its own width, 4-body) hold
// the same coefficient matrix: X . A . Y reproduces S, and the padding is zero.
// With a second argument (a binary parameter cache of the same file) it also
// checks that the cache packs into the same device image as the text file.
// Usage: factored_check <params> [cache]; prints "ok <tuples checked>" or a mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "ck_params.h"

using namespace ck;

template <class T>
static const T* at(const std::vector<unsigned char>& img, const T* off) {
    return reinterpret_cast<const T*>(img.data() + reinterpret_cast<uintptr_t>(off));
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    HostParams P;
    std::string err;
    if (parse_parameter_file(argv[1], P, err) != kOk) {
        std::printf("parse error: %s\n", err.c_str());
        return 1;
    }
    ParamImage img = pack_params(P);
    const DevParamSet& H = img.header;
    if (argc > 2) {
        HostParams Q;
        if (parse_parameter_file(argv[2], Q, err) != kOk) {
            std::printf("cache parse error: %s\n", err.c_str());
            return 1;
        }
        ParamImage img2 = pack_params(Q);
        if (img2.bytes != img.bytes || img2.header_off != img.header_off) {
            std::printf("cache packs differently\n");
            return 1;
        }
    }
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    int checked = 0, tc_checked = 0;
    for (int nb = 3; nb <= 4; nb++) {
        const int order = nb == 3 ? H.o3 : H.o4;
        const int Rp = nb == 3 ? H.R3 : H.R4;
        if (order <= 0) continue;
        if (Rp <= 0) {
            std::printf("no factored tables for %d-body\n", nb);
            continue;
        }
        const int np = nb == 3 ? 3 : 6, K = nb == 3 ? 1 : 3;
        int ntup = 1;
        for (int k = 0; k < nb; k++) ntup *= H.ntypes;
        const TupleRec* tr = at(img.bytes, nb == 3 ? H.t3 : H.t4);
        const double* cd = at(img.bytes, nb == 3 ? H.c3d : H.c4d);
        const uint32_t* pw = at(img.bytes, nb == 3 ? H.p3 : H.p4);
        const FactRow* fr = at(img.bytes, nb == 3 ? H.fr3 : H.fr4);
        const FactEntD* fe = at(img.bytes, nb == 3 ? H.fe3d : H.fe4d);
        const FactEntF* ff = at(img.bytes, nb == 3 ? H.fe3f : H.fe4f);
        for (int u = 0; u < ntup; u++) {
            const TupleRec& R = tr[u];
            if (!R.valid) continue;
            std::vector<double> T(np * Rp), D(np * Rp);
            for (auto& v : T) v = U(rng);
            for (auto& v : D) v = U(rng);
            // per coefficient
            double S0 = 0, G0[6] = {0, 0, 0, 0, 0, 0};
            for (int c = 0; c < R.ncoef; c++) {
                const uint32_t pk = pw[R.coef_off + c];
                double prod = cd[R.coef_off + c];
                int q[6];
                for (int p = 0; p < np; p++) {
                    q[p] = (pk >> (kPowBits * p)) & 31u;
                    if (q[p] >= Rp) { std::printf("power %d >= R %d\n", q[p], Rp); return 1; }
                    prod *= T[p * Rp + q[p]];
                }
                S0 += prod;
                for (int p = 0; p < np; p++) {
                    double g = cd[R.coef_off + c] * D[p * Rp + q[p]];
                    for (int o = 0; o < np; o++)
                        if (o != p) g *= T[o * Rp + q[o]];
                    G0[p] += g;
                }
            }
            // factored
            int ny = 1, nx = 1;
            for (int p = K; p < np; p++) ny *= Rp;
            for (int p = 0; p < K; p++) nx *= Rp;
            auto prod_of = [&](int idx, int lo, int hi, int dpair) {
                double v = 1.0;
                for (int p = hi - 1; p >= lo; p--) {
                    const int q = idx % Rp;
                    idx /= Rp;
                    v *= (p == dpair ? D : T)[p * Rp + q];
                }
                return v;
            };
            // record powers packed kPowBits per pair from the side's first pair
            auto prod_packed = [&](int pows, int lo, int hi, int dpair) {
                double v = 1.0;
                for (int p = lo; p < hi; p++) {
                    const int q = (pows >> (kPowBits * (p - lo))) & 31;
                    v *= (p == dpair ? D : T)[p * Rp + q];
                }
                return v;
            };
            // packed powers of n pairs (first pair lowest) -> linear index (first pair most significant)
            auto packed_lin = [&](int pows, int n) {
                int lin = 0;
                for (int p = 0; p < n; p++) lin = lin * Rp + ((pows >> (kPowBits * p)) & 31);
                return lin;
            };
            double S1 = 0, G1[6] = {0, 0, 0, 0, 0, 0};
            int e = R.f_ent;
            if (R.f_nrow <= 0 || R.f_ncol <= 0) { std::printf("tuple %d without rows\n", u); return 1; }
            for (int r = 0; r < R.f_nrow; r++) {
                const FactRow rw = fr[R.f_row + r];
                double z = 0;
                for (int k = e; k < rw.end; k++) {
                    const int lin = fe[k].idx & 0xffff;
                    if (lin >= ny || ff[k].idx != fe[k].idx || ff[k].a != (float)fe[k].a ||
                        packed_lin(fe[k].idx >> 16, np - K) != lin || (fe[k].idx < 0) != (k + 1 == rw.end)) {
                        std::printf("bad row entry\n");
                        return 1;
                    }
                    z += fe[k].a * prod_of(lin, K, np, -1);
                }
                e = rw.end;
                S1 += prod_packed(rw.pows, 0, K, -1) * z;
                for (int p = 0; p < K; p++) G1[p] += prod_packed(rw.pows, 0, K, p) * z;
            }
            if (e != R.f_ent + R.ncoef) { std::printf("row entries %d != %d\n", e - R.f_ent, R.ncoef); return 1; }
            for (int c = 0; c < R.f_ncol; c++) {
                const FactRow cl = fr[R.f_row + R.f_nrow + c];
                double w = 0;
                for (int k = e; k < cl.end; k++) {
                    const int lin = fe[k].idx & 0xffff;
                    if (lin >= nx || ff[k].idx != fe[k].idx ||
                        packed_lin(fe[k].idx >> 16, K) != lin || (fe[k].idx < 0) != (k + 1 == cl.end)) {
                        std::printf("bad column entry\n");
                        return 1;
                    }
                    w += fe[k].a * prod_of(lin, 0, K, -1);
                }
                e = cl.end;
                for (int p = K; p < np; p++) G1[p] += prod_packed(cl.pows, K, np, p) * w;
            }
            if (e != R.f_ent + 2 * R.ncoef) { std::printf("column entries mismatch\n"); return 1; }
            double scale = std::fabs(S0);
            for (int p = 0; p < np; p++) scale = std::fmax(scale, std::fabs(G0[p]));
            scale = std::fmax(scale, 1e-300);
            bool bad = std::fabs(S1 - S0) > 1e-12 * scale;
            for (int p = 0; p < np; p++) bad = bad || std::fabs(G1[p] - G0[p]) > 1e-12 * scale;
            if (bad) {
                std::printf("mismatch %d-body tuple %d: S %.17g vs %.17g\n", nb, u, S1, S0);
                return 1;
            }
            // tensor-core image (the B operand: N rows of K values, core-matrix
            // layout, kTc3Parts parts): the parts' sum is the coefficient matrix
            // (rows = the first K pairs' powers, columns = the rest), zero in
            // the padding, and S = X . A . Y reproduces the per-coefficient sum
            const float* tcimg = nb == 3 ? (H.tc3 ? at(img.bytes, H.tc3) : nullptr)
                                         : (H.tc4 ? at(img.bytes, H.tc4) : nullptr);
            const long long ntc = nb == 3 ? H.n_tc3 : H.n_tc4;
            if (tcimg && R.tc_off >= 0) {
                const int nrow = nx, ncol = ny;   // R^K rows (I), R^(P-K) columns (J)
                const int kpad = nb == 3 ? tc3_kpad(Rp) : tc4_kpad(nrow);
                const int npad = nb == 3 ? tc3_npad(Rp) : tc4_npad(ncol);
                const long long part = (long long)kpad * npad;
                if (R.tc_off + kTc3Parts * part > ntc) { std::printf("tensor-core image out of range\n"); return 1; }
                double S2 = 0, pad = 0;
                for (int n = 0; n < npad; n++)
                    for (int k = 0; k < kpad; k++) {
                        const long long off = ((long long)(n / 8) * (kpad / 4) + k / 4) * 32 + (n % 8) * 4 + (k % 4);
                        double a = 0;
                        for (int t = 0; t < kTc3Parts; t++) a += (double)tcimg[R.tc_off + t * part + off];
                        // 3-body columns at Rw = R are q1 * R + q2, i.e. J itself
                        if (n >= ncol || k >= nrow) { pad += std::fabs(a); continue; }
                        S2 += prod_of(k, 0, K, -1) * a * prod_of(n, K, np, -1);
                    }
                if (pad != 0.0 || std::fabs(S2 - S0) > 1e-6 * scale) {
                    std::printf("tensor-core image mismatch %d-body tuple %d: S %.17g vs %.17g (padding %g)\n", nb, u,
                                S2, S0, pad);
                    return 1;
                }
                tc_checked++;
            }
            checked++;
        }
    }
    std::printf("ok %d (tensor-core images %d)\n", checked, tc_checked);
    return 0;
}
