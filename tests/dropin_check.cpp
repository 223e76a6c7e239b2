// A program written against the reference's C++ and per-cluster C interfaces
// (serial_chimes_interface, chimesFF, chimescalc_C.h), compiled unchanged
// against this library's headers and linked with libchimescalc.so.  The GPU
// tests build and run it and compare its output with the reference-made
// fixtures.
//
//   dropin_check serial   <params> <xyz> <small> <out>
//       serial_chimes_interface(small).calculate on one configuration, with
//       energy 2.0, forces 0.1 and stress 7.0 passed in (energy and forces
//       accumulate, stress is overwritten); writes energy, stress[9], forces,
//       then get_badness().
//   dropin_check clusters <params> <queries> <out>
//       chimesFF::compute_1B/2B/3B/4B on every query (format of
//       oracle/ref_cluster_driver.cpp), the overloads with force_scalar_in
//       from zero; writes energy, forces, stress[6], force_scalar_in,
//       get_badness() (reset before each query) and a 0/1 flag telling whether
//       the overload without force_scalar_in gave identical results.
//   dropin_check capi     <params> <queries> <out>
//       chimes_compute_{2,3,4}b_props (and the _fromf90 forms) on the 2-4 atom
//       queries, type names looked up in the parameter file's order, with
//       energy 1.0, forces 0.25 and stress 0.5 (all nine) passed in; writes
//       energy, forces, stress[9] of the C form, then of the _fromf90 form.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "chimescalc_C.h"
#include "serial_chimes_interface.h"

static void read_xyz(const char* path, std::vector<std::string>& types, std::vector<double>& x,
                     std::vector<double>& y, std::vector<double>& z, std::vector<double>& a, std::vector<double>& b,
                     std::vector<double>& c) {
    std::ifstream f(path);
    std::string line;
    std::getline(f, line);
    const int n = std::atoi(line.c_str());
    std::getline(f, line);
    std::istringstream cs(line);
    a.assign(3, 0.0), b.assign(3, 0.0), c.assign(3, 0.0);
    cs >> a[0] >> a[1] >> a[2] >> b[0] >> b[1] >> b[2] >> c[0] >> c[1] >> c[2];
    for (int i = 0; i < n; i++) {
        std::getline(f, line);
        std::istringstream ls(line);
        std::string t;
        double p, q, r;
        ls >> t >> p >> q >> r;
        types.push_back(t), x.push_back(p), y.push_back(q), z.push_back(r);
    }
}

static void put(FILE* fo, const std::vector<double>& v) {
    for (double d : v) fprintf(fo, " %.17g", d);
}

struct Query {
    int nb = 0;
    std::vector<int> t;
    std::vector<double> dx, dr;
};

static std::vector<Query> read_queries(const char* path) {
    std::vector<Query> out;
    std::ifstream q(path);
    std::string line;
    while (std::getline(q, line)) {
        std::istringstream ls(line);
        Query Q;
        if (!(ls >> Q.nb)) continue;
        const int np = Q.nb * (Q.nb - 1) / 2;
        Q.t.resize(Q.nb);
        for (auto& v : Q.t) ls >> v;
        Q.dx.resize(np > 0 ? np : 1);
        Q.dr.resize(3 * (np > 0 ? np : 1));
        for (int p = 0; p < np; p++) ls >> Q.dx[p];
        for (int p = 0; p < 3 * np; p++) ls >> Q.dr[p];
        out.push_back(Q);
    }
    return out;
}

static int run_serial(int argc, char** argv) {
    if (argc < 6) return 2;
    std::vector<std::string> types;
    std::vector<double> x, y, z, a, b, c;
    read_xyz(argv[3], types, x, y, z, a, b, c);
    serial_chimes_interface chimes(std::atoi(argv[4]) != 0);
    chimes.init_chimesFF(argv[2], 0);
    const size_t n = x.size();
    double energy = 2.0;
    std::vector<std::vector<double> > force(n, std::vector<double>(3, 0.1));
    std::vector<double> stress(9, 7.0);
    chimes.calculate(x, y, z, a, b, c, types, energy, force, stress);
    FILE* fo = std::fopen(argv[5], "w");
    fprintf(fo, "%.17g\n", energy);
    put(fo, stress);
    fprintf(fo, "\n");
    for (size_t i = 0; i < n; i++) {
        put(fo, force[i]);
        fprintf(fo, "\n");
    }
    fprintf(fo, "%d\n", chimes.get_badness());
    std::fclose(fo);
    return 0;
}

static int run_clusters(int argc, char** argv) {
    if (argc < 5) return 2;
    chimesFF ff;
    ff.init(0);
    ff.read_parameters(argv[2]);
    ff.build_pair_int_trip_map();
    ff.build_pair_int_quad_map();
    FILE* fo = std::fopen(argv[4], "w");
    for (const Query& Q : read_queries(argv[3])) {
        ff.reset_badness();
        double e = 0.0, e2 = 0.0;
        std::vector<double> f(3 * Q.nb, 0.0), s(6, 0.0), fs, f2(3 * Q.nb, 0.0), s2(6, 0.0);
        if (Q.nb == 1) {
            ff.compute_1B(Q.t[0], e);
            ff.compute_1B(Q.t[0], e2);
        } else if (Q.nb == 2) {
            chimes2BTmp tmp(ff.poly_orders[0]);
            double f1 = 0.0;
            ff.compute_2B(Q.dx[0], Q.dr, Q.t, f, s, e, tmp, f1);
            fs.push_back(f1);
            ff.compute_2B(Q.dx[0], Q.dr, Q.t, f2, s2, e2, tmp);
        } else if (Q.nb == 3) {
            chimes3BTmp tmp(ff.poly_orders[1]);
            fs.assign(3, 0.0);
            ff.compute_3B(Q.dx, Q.dr, Q.t, f, s, e, tmp, fs);
            ff.compute_3B(Q.dx, Q.dr, Q.t, f2, s2, e2, tmp);
        } else {
            chimes4BTmp tmp(ff.poly_orders[2]);
            fs.assign(6, 0.0);
            ff.compute_4B(Q.dx, Q.dr, Q.t, f, s, e, tmp, fs);
            ff.compute_4B(Q.dx, Q.dr, Q.t, f2, s2, e2, tmp);
        }
        const int badness = ff.get_badness();
        const bool same = e == e2 && f == f2 && s == s2;
        fprintf(fo, "%.17g", e);
        put(fo, f);
        put(fo, s);
        put(fo, fs);
        fprintf(fo, " %d %d\n", badness, same ? 1 : 0);
    }
    std::fclose(fo);
    return 0;
}

static int run_capi(int argc, char** argv) {
    if (argc < 5) return 2;
    chimesFF names;   // the parameter file's type order, for name look-up
    names.init(0);
    names.read_parameters(argv[2]);
    set_chimes();
    init_chimes(0);
    chimes_read_params(argv[2]);
    chimes_build_pair_int_trip_map();
    chimes_build_pair_int_quad_map();
    FILE* fo = std::fopen(argv[4], "w");
    for (const Query& Q : read_queries(argv[3])) {
        if (Q.nb < 2) continue;
        std::vector<std::string> tn;
        for (int t : Q.t) tn.push_back(names.atmtyps[t]);
        std::vector<char*> tp;
        for (auto& s : tn) tp.push_back(const_cast<char*>(s.c_str()));
        for (int form = 0; form < 2; form++) {
            double e = 1.0;
            double f[4][3], s[9];
            for (auto& row : f)
                for (double& v : row) v = 0.25;
            for (double& v : s) v = 0.5;
            double dx[6], dr[6][3];
            for (int p = 0; p < (int)Q.dx.size(); p++) dx[p] = Q.dx[p];
            for (int p = 0; p < (int)Q.dx.size(); p++)
                for (int k = 0; k < 3; k++) dr[p][k] = Q.dr[3 * p + k];
            if (Q.nb == 2) {
                double fo2[2][3];
                std::memcpy(fo2, f, sizeof(fo2));
                if (form == 0) chimes_compute_2b_props(dx[0], dr[0], tp.data(), fo2, s, &e);
                else chimes_compute_2b_props_fromf90(&dx[0], dr[0], tp[0], tp[1], fo2, s, &e);
                std::memcpy(f, fo2, sizeof(fo2));
            } else if (Q.nb == 3) {
                double fo3[3][3], d3[3][3];
                std::memcpy(fo3, f, sizeof(fo3));
                std::memcpy(d3, dr, sizeof(d3));
                if (form == 0) chimes_compute_3b_props(dx, d3, tp.data(), fo3, s, &e);
                else chimes_compute_3b_props_fromf90(dx, d3, tp[0], tp[1], tp[2], fo3, s, &e);
                std::memcpy(f, fo3, sizeof(fo3));
            } else {
                if (form == 0) chimes_compute_4b_props(dx, dr, tp.data(), f, s, &e);
                else chimes_compute_4b_props_fromf90(dx, dr, tp[0], tp[1], tp[2], tp[3], f, s, &e);
            }
            fprintf(fo, "%s%.17g", form ? " " : "", e);
            for (int a = 0; a < Q.nb; a++)
                for (int k = 0; k < 3; k++) fprintf(fo, " %.17g", f[a][k]);
            for (double v : s) fprintf(fo, " %.17g", v);
        }
        fprintf(fo, "\n");
    }
    std::fclose(fo);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    if (!std::strcmp(argv[1], "serial")) return run_serial(argc, argv);
    if (!std::strcmp(argv[1], "clusters")) return run_clusters(argc, argv);
    if (!std::strcmp(argv[1], "capi")) return run_capi(argc, argv);
    return 2;
}
