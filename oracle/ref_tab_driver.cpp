// Test-infrastructure driver for the UNMODIFIED reference's tabulated terms.
//
// Part of the oracle: linked against the reference's own
// chimesFF/src/chimesFF.cpp compiled with -DTABULATION (the option its LAMMPS
// build uses) by oracle/Makefile into oracle/_ref/.  Nothing in the product
// links or runs it.
//
// It reads a parameter file whose 2-body and/or 3-body terms are tabulated and
// evaluates chimesFF::compute_2B_tab / compute_3B_tab (chimesFF.cpp:1776-2322)
// on the clusters listed in a query file, one per line:
//   2 t0 t1 dx drx dry drz
//   3 t0 t1 t2 dx_ij dx_ik dx_jk dr_ij[3] dr_ik[3] dr_jk[3]
// and writes, per query, energy, force (6 or 9), stress (6) and the
// force_scalar_in values (1 or 3) at 17 significant digits.
//
// Usage: ref_tab_driver <params> <queries> <out>

#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "chimesFF.h"

int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: ref_tab_driver params queries out\n"); return 2; }
    std::ofstream devnull("/dev/null");
    std::streambuf* saved = std::cout.rdbuf(devnull.rdbuf());
    chimesFF ff;
    ff.init(0);
    ff.read_parameters(argv[1]);
    ff.build_pair_int_trip_map();
    ff.build_pair_int_quad_map();
    std::cout.rdbuf(saved);

    std::ifstream q(argv[2]);
    FILE* fo = fopen(argv[3], "w");
    std::string line;
    while (std::getline(q, line)) {
        std::istringstream ls(line);
        int nb;
        if (!(ls >> nb)) continue;
        if (nb == 2) {
            std::vector<int> t(2);
            double dx;
            std::vector<double> dr(3), force(6, 0.0), stress(6, 0.0);
            ls >> t[0] >> t[1] >> dx >> dr[0] >> dr[1] >> dr[2];
            double e = 0.0, fs = 0.0;
            chimes2BTmp tmp(ff.poly_orders[0]);
            ff.compute_2B_tab(dx, dr, t, force, stress, e, tmp, fs);
            fprintf(fo, "%.17g", e);
            for (double v : force) fprintf(fo, " %.17g", v);
            for (double v : stress) fprintf(fo, " %.17g", v);
            fprintf(fo, " %.17g\n", fs);
        } else {
            std::vector<int> t(3);
            std::vector<double> dx(3), dr(9), force(9, 0.0), stress(6, 0.0), fs(3, 0.0);
            ls >> t[0] >> t[1] >> t[2];
            for (auto& v : dx) ls >> v;
            for (auto& v : dr) ls >> v;
            double e = 0.0;
            chimes3BTmp tmp(ff.poly_orders[1]);
            ff.compute_3B_tab(dx, dr, t, force, stress, e, tmp, fs);
            fprintf(fo, "%.17g", e);
            for (double v : force) fprintf(fo, " %.17g", v);
            for (double v : stress) fprintf(fo, " %.17g", v);
            for (double v : fs) fprintf(fo, " %.17g", v);
            fprintf(fo, "\n");
        }
    }
    fclose(fo);
    return 0;
}
