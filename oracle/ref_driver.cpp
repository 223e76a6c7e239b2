// Test-infrastructure driver for the UNMODIFIED reference ChIMES calculator.
//
// This file is part of the oracle: it is linked against the reference's own
// chimesFF/src/chimesFF.cpp and serial_interface/src/serial_chimes_interface.cpp,
// compiled from the read-only reference tree by oracle/Makefile into
// oracle/_ref/.  Nothing in the product links or runs it.
//
// It runs serial_chimes_interface::calculate (serial_chimes_interface.cpp:960-1124)
// on one configuration and writes energy, stress[9] and forces at 17 significant
// digits.  With --lists it also writes the private cluster lists
// (neighlist_2b/3b/4b, built by simulation_system::build_neigh_lists,
// serial_chimes_interface.cpp:588-864), reached with the access-specifier
// override below.  With --time K it times K calls of calculate() with
// steady_clock (parameters pre-loaded, reference stdout muted).
//
// Usage: ref_driver <params> <xyz> <small 0|1> <out_prefix> [--lists] [--time K]

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <map>
#include <algorithm>
#include <cmath>
#include <iomanip>

#define private public
#include "serial_chimes_interface.h"
#undef private

static void read_xyz(const std::string& path, std::vector<std::string>& types, std::vector<double>& x,
                     std::vector<double>& y, std::vector<double>& z, std::vector<double>& ca,
                     std::vector<double>& cb, std::vector<double>& cc) {
    std::ifstream f(path);
    if (!f.good()) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
    std::string line;
    std::getline(f, line);
    int n = std::stoi(line);
    std::getline(f, line);
    std::istringstream cs(line);
    ca.assign(3, 0.0); cb.assign(3, 0.0); cc.assign(3, 0.0);
    cs >> ca[0] >> ca[1] >> ca[2] >> cb[0] >> cb[1] >> cb[2] >> cc[0] >> cc[1] >> cc[2];
    for (int i = 0; i < n; i++) {
        std::getline(f, line);
        std::istringstream ls(line);
        std::string t; double a, b, c;
        ls >> t >> a >> b >> c;
        types.push_back(t); x.push_back(a); y.push_back(b); z.push_back(c);
    }
}

int main(int argc, char** argv) {
    if (argc < 5) { fprintf(stderr, "usage: ref_driver params xyz small out [--lists] [--time K]\n"); return 2; }
    std::string params = argv[1], xyz = argv[2], out = argv[4];
    bool small = atoi(argv[3]) != 0;
    bool lists = false;
    int time_reps = 0;
    for (int a = 5; a < argc; a++) {
        if (!strcmp(argv[a], "--lists")) lists = true;
        else if (!strcmp(argv[a], "--time") && a + 1 < argc) time_reps = atoi(argv[++a]);
    }
    std::vector<std::string> types; std::vector<double> x, y, z, ca, cb, cc;
    read_xyz(xyz, types, x, y, z, ca, cb, cc);
    int n = (int)x.size();

    std::ofstream devnull("/dev/null");
    std::streambuf* saved = std::cout.rdbuf(devnull.rdbuf());

    serial_chimes_interface chimes(small);
    chimes.init_chimesFF(params, 0);

    double energy = 0.0;
    std::vector<double> stress(9, 0.0);
    std::vector<std::vector<double> > force(n, std::vector<double>(3, 0.0));
    std::vector<std::string> types_in = types;
    chimes.calculate(x, y, z, ca, cb, cc, types_in, energy, force, stress);

    double best = 1e300, total = 0.0;
    for (int r = 0; r < time_reps; r++) {
        double e2 = 0.0; std::vector<double> s2(9, 0.0);
        std::vector<std::vector<double> > f2(n, std::vector<double>(3, 0.0));
        std::vector<std::string> t2 = types;
        auto t0 = std::chrono::steady_clock::now();
        chimes.calculate(x, y, z, ca, cb, cc, t2, e2, f2, s2);
        auto t1 = std::chrono::steady_clock::now();
        double dt = std::chrono::duration<double>(t1 - t0).count();
        best = std::min(best, dt); total += dt;
    }
    std::cout.rdbuf(saved);

    FILE* fo = fopen((out + ".res").c_str(), "w");
    fprintf(fo, "%.17g\n", energy);
    for (int k = 0; k < 9; k++) fprintf(fo, "%.17g%c", stress[k], k == 8 ? '\n' : ' ');
    for (int i = 0; i < n; i++) fprintf(fo, "%.17g %.17g %.17g\n", force[i][0], force[i][1], force[i][2]);
    fclose(fo);

    if (lists) {
        FILE* fl = fopen((out + ".lists").c_str(), "w");
        size_t n2 = 0;
        for (int i = 0; i < chimes.neigh.n_atoms; i++) n2 += chimes.neighlist_2b[i].size();
        fprintf(fl, "%d %d %zu %zu %zu\n", chimes.neigh.n_atoms, chimes.neigh.n_ghost, n2,
                chimes.neighlist_3b.size(), chimes.neighlist_4b.size());
        for (int i = 0; i < chimes.neigh.n_atoms; i++)
            for (size_t j = 0; j < chimes.neighlist_2b[i].size(); j++) fprintf(fl, "%d %d\n", i, chimes.neighlist_2b[i][j]);
        for (auto& t : chimes.neighlist_3b) fprintf(fl, "%d %d %d\n", t[0], t[1], t[2]);
        for (auto& q : chimes.neighlist_4b) fprintf(fl, "%d %d %d %d\n", q[0], q[1], q[2], q[3]);
        fclose(fl);
    }
    if (time_reps > 0) printf("{\"best_s\": %.9g, \"mean_s\": %.9g, \"reps\": %d}\n", best, total / time_reps, time_reps);
    return 0;
}
