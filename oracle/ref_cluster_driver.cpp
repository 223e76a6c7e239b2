// Test-infrastructure driver for the UNMODIFIED reference's per-cluster API.
//
// Part of the oracle: linked against the reference's own
// chimesFF/src/chimesFF.cpp (default build, no TABULATION) by oracle/Makefile
// into oracle/_ref/.  Nothing in the product links or runs it.
//
// It evaluates chimesFF::compute_1B / compute_2B / compute_3B / compute_4B
// (chimesFF.cpp:1636-1775, 1931-2176, 2496-2872), the overloads with
// force_scalar_in, on the clusters of a query file, one per line:
//   1 t
//   2 t0 t1 dx drx dry drz
//   3 t0 t1 t2 dx[3] dr[9]            (pairs ij, ik, jk)
//   4 t0 t1 t2 t3 dx[6] dr[18]        (pairs ij, ik, il, jk, jl, kl)
// Each query starts from zero energy, forces and stress and writes one line:
// energy, force (3 x atoms), stress (6), force_scalar_in (0, 1, 3 or 6
// values) at 17 significant digits, then get_badness() after the call (reset
// before each query).
//
// Usage: ref_cluster_driver <params> <queries> <out>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "chimesFF.h"

int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: ref_cluster_driver params queries out\n"); return 2; }
    std::ofstream devnull("/dev/null");
    std::streambuf* saved = std::cout.rdbuf(devnull.rdbuf());
    chimesFF ff;
    ff.init(0);
    ff.read_parameters(argv[1]);
    ff.build_pair_int_trip_map();
    ff.build_pair_int_quad_map();

    std::ifstream q(argv[2]);
    FILE* fo = fopen(argv[3], "w");
    std::string line;
    while (std::getline(q, line)) {
        std::istringstream ls(line);
        int nb;
        if (!(ls >> nb)) continue;
        ff.reset_badness();
        const int np = nb * (nb - 1) / 2;
        std::vector<int> t(nb);
        for (auto& v : t) ls >> v;
        std::vector<double> dx(np > 0 ? np : 1), dr(3 * (np > 0 ? np : 1));
        for (int p = 0; p < np; p++) ls >> dx[p];
        for (int p = 0; p < 3 * np; p++) ls >> dr[p];
        double e = 0.0;
        std::vector<double> force(3 * nb, 0.0), stress(6, 0.0), fs;
        if (nb == 1) {
            ff.compute_1B(t[0], e);
        } else if (nb == 2) {
            double f1 = 0.0;
            chimes2BTmp tmp(ff.poly_orders[0]);
            ff.compute_2B(dx[0], dr, t, force, stress, e, tmp, f1);
            fs.push_back(f1);
        } else if (nb == 3) {
            fs.assign(3, 0.0);
            chimes3BTmp tmp(ff.poly_orders[1]);
            ff.compute_3B(dx, dr, t, force, stress, e, tmp, fs);
        } else {
            fs.assign(6, 0.0);
            chimes4BTmp tmp(ff.poly_orders[2]);
            ff.compute_4B(dx, dr, t, force, stress, e, tmp, fs);
        }
        fprintf(fo, "%.17g", e);
        for (double v : force) fprintf(fo, " %.17g", v);
        for (double v : stress) fprintf(fo, " %.17g", v);
        for (double v : fs) fprintf(fo, " %.17g", v);
        fprintf(fo, " %d\n", ff.get_badness());
    }
    fclose(fo);
    std::cout.rdbuf(saved);
    return 0;
}
