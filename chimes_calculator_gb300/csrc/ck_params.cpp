// Parsing of the ChIMES parameter-file format and packing of the device tables.
//
// The parse follows chimesFF::read_parameters (chimesFF/src/chimesFF.cpp:354-1570)
// pass for pass: the same keywords, token positions, rewinds and defaults, so
// a file reads into the same tables.  Differences: errors are returned as
// status codes with a message instead of printing and calling exit(0), the
// per-coefficient echo to stdout is not reproduced, and inputs that would make
// the reference read outside its polynomial tables (a power larger than the
// order) are rejected.
#include "ck_params.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <sstream>

namespace ck {

namespace {

// chimesFF::split_line (chimesFF.cpp:148-180): strip '!' and '##' comments,
// split on whitespace.
std::vector<std::string> tokens(const std::string& raw) {
    std::string line = raw;
    size_t p = line.find('!');
    if (p != std::string::npos) line.erase(p);
    p = line.find("##");
    if (p != std::string::npos) line.erase(p);
    std::vector<std::string> out;
    std::istringstream ss(line);
    std::string t;
    while (ss >> t) out.push_back(t);
    return out;
}

bool has(const std::string& line, const char* key) { return line.find(key) != std::string::npos; }

struct Lines {
    std::vector<std::string> v;
    size_t i = 0;
    bool next(std::string& out) {
        if (i >= v.size()) return false;
        out = v[i++];
        return true;
    }
    void rewind() { i = 0; }
};

struct ParseError {
    std::string msg;
};

[[noreturn]] void fail(const std::string& m) { throw ParseError{m}; }

int to_int(const std::vector<std::string>& t, size_t k, const char* what) {
    if (k >= t.size()) fail(std::string("missing integer field in ") + what);
    try {
        return std::stoi(t[k]);
    } catch (...) {
        fail(std::string("bad integer '") + t[k] + "' in " + what);
    }
}

double to_dbl(const std::vector<std::string>& t, size_t k, const char* what) {
    if (k >= t.size()) fail(std::string("missing number field in ") + what);
    try {
        return std::stod(t[k]);
    } catch (...) {
        fail(std::string("bad number '") + t[k] + "' in " + what);
    }
}

const std::string& tok(const std::vector<std::string>& t, size_t k, const char* what) {
    if (k >= t.size()) fail(std::string("missing field in ") + what);
    return t[k];
}

// get_proper_pair (chimesFF.cpp:69-84)
// Tabulated-term files (read_2B_tab / read_3B_tab, chimesFF.cpp:199-351):
// <name>.energy and <name>.force, a row count on the first line, then rows of
// "r value" (2-body) or "rij rik rjk value[s]" (3-body).  The reference
// concatenates the parameter file's directory and the table name without a
// separator; here the name is taken relative to the parameter file's directory
// (identical when the parameter file is named without a directory).
std::vector<std::vector<double>> read_table_rows(const std::string& path, const char* what,
                                                 const std::vector<size_t>& widths) {
    std::ifstream f(path);
    if (!f.is_open()) fail("could not open file: " + path);
    std::string line;
    if (!std::getline(f, line)) fail("error reading line in " + path);
    auto t = tokens(line);
    const long long n = to_int(t, 0, what);
    if (n < 0) fail(std::string("negative row count in ") + path);
    std::vector<std::vector<double>> rows;
    rows.reserve((size_t)n);
    for (long long i = 0; i < n; i++) {
        if (!std::getline(f, line)) fail("error reading line in " + path + " (fewer rows than announced)");
        auto u = tokens(line);
        if (std::find(widths.begin(), widths.end(), u.size()) == widths.end())
            fail(std::string("unexpected number of items in ") + what + " row: " + line);
        std::vector<double> v(u.size());
        for (size_t k = 0; k < u.size(); k++) v[k] = to_dbl(u, k, what);
        rows.push_back(std::move(v));
    }
    return rows;
}

void read_tab2(const std::string& dir, const std::string& name, HostParams& P) {
    auto e = read_table_rows(dir + name + ".energy", "2-body energy table", {2});
    auto f = read_table_rows(dir + name + ".force", "2-body force table", {2});
    if (e.size() != f.size()) fail("2-body energy and force tables of " + name + " differ in length");
    HostParams::Tab2 T;
    for (size_t i = 0; i < e.size(); i++) {
        T.r.push_back(e[i][0]);
        T.e.push_back(e[i][1]);
        T.f.push_back(f[i][1]);
        // the interval search (std::lower_bound in get_tab_2B) needs ascending distances
        if (i > 0 && !(T.r[i] > T.r[i - 1])) fail("2-body table " + name + ": distances must be strictly ascending");
    }
    P.t2tab.push_back(std::move(T));
}

void read_tab3(const std::string& dir, const std::string& name, HostParams& P) {
    auto e = read_table_rows(dir + name + ".energy", "3-body energy table", {4, 6});
    auto f = read_table_rows(dir + name + ".force", "3-body force table", {6});
    if (e.size() != f.size()) fail("3-body energy and force tables of " + name + " differ in length");
    HostParams::Tab3 T;
    for (size_t i = 0; i < e.size(); i++) {
        T.rij.push_back(e[i][0]);
        T.rik.push_back(e[i][1]);
        T.rjk.push_back(e[i][2]);
        T.e.push_back(e[i][3]);
        T.fij.push_back(f[i][3]);
        T.fik.push_back(f[i][4]);
        T.fjk.push_back(f[i][5]);
    }
    // interpolateTricubic reads the rjk column at row size^2 + size + 1 for the grid step
    const int size = (int)std::cbrt((double)T.rik.size());
    if (size < 2) fail("3-body table " + name + " needs at least 2 grid points per distance (8 rows)");
    P.t3tab.push_back(std::move(T));
}

int proper_pair(const HostParams& P, const std::string& a, const std::string& b) {
    for (int i = 0; i < P.npairs; i++) {
        if (a == P.pa1[i] && b == P.pa2[i]) return i;
        if (b == P.pa1[i] && a == P.pa2[i]) return i;
    }
    fail("no proper pair name found for atom types " + a + ", " + b);
}

// build_atom_and_pair_mappers (chimesFF/src/chimesFF.h:438-539): the first
// permutation (std::next_permutation order) of the cluster's atom slots whose
// runtime pair names equal the parameter type's pair names gives, for each
// cluster pair j, the parameter pair index mapped[j].  `mapped` keeps its
// previous contents when no permutation matches, like the reference's reused
// vector.
void atom_pair_mapper(const HostParams& P, int natoms, const int* typ,
                      const std::vector<std::string>& clu_pairs, std::vector<int>& mapped) {
    const int npairs = natoms * (natoms - 1) / 2;
    std::vector<int> perm(natoms);
    for (int i = 0; i < natoms; i++) perm[i] = i;
    std::vector<std::pair<int, int>> slots, run(npairs, {0, 0});
    for (int i = 0; i < natoms; i++)
        for (int j = i + 1; j < natoms; j++) slots.push_back({i, j});
    do {
        bool match = true;
        for (int p = 0; p < npairs && match; p++) {
            int a = typ[perm[slots[p].first]], b = typ[perm[slots[p].second]];
            if (clu_pairs[p] != P.pair_name(P.prpr[a * P.ntypes + b])) match = false;
        }
        if (match) {
            for (int p = 0; p < npairs; p++) run[p] = {perm[slots[p].first], perm[slots[p].second]};
            break;
        }
    } while (std::next_permutation(perm.begin(), perm.end()));
    for (int i = 0; i < npairs; i++)
        for (int j = 0; j < npairs; j++)
            if ((run[i].first == slots[j].first && run[i].second == slots[j].second) ||
                (run[i].first == slots[j].second && run[i].second == slots[j].first))
                mapped[j] = i;
}

void parse_lines(Lines& L, HostParams& P, const std::string& dir) {
    std::string line;
    // pass 1: PAIRTYP: CHEBYSHEV o2 [o3 [o4]]  (chimesFF.cpp:390-437)
    bool found = false;
    while (L.next(line)) {
        if (has(line, "ENDFILE")) fail("could not find line containing \"PAIRTYP: CHEBYSHEV\"");
        if (has(line, "PAIRTYP: CHEBYSHEV")) {
            auto t = tokens(line);
            if (t.size() < 3) fail("\"PAIRTYP: CHEBYSHEV\" line must at least contain the 2-body order");
            P.o2 = to_int(t, 2, "PAIRTYP");
            P.o3 = t.size() >= 4 ? to_int(t, 3, "PAIRTYP") : 0;
            P.o4 = t.size() >= 5 ? to_int(t, 4, "PAIRTYP") : 0;
            found = true;
            break;
        }
    }
    if (!found) fail("error reading line: no ENDFILE and no PAIRTYP line");
    if (P.o2 < 1 || P.o2 > kMaxOrder || P.o3 < 0 || P.o3 > kMaxOrder || P.o4 < 0 || P.o4 > kMaxOrder)
        fail("polynomial orders must lie in [1,31] (2B) and [0,31] (3B, 4B)");

    // pass 2: types, pairs, cutoff style, penalty, energy offsets (chimesFF.cpp:445-686)
    L.rewind();
    int no_pairs = 0;
    while (true) {
        if (!L.next(line)) fail("error reading line: missing ENDFILE");
        if (has(line, "ENDFILE")) break;
        if (has(line, "ATOM TYPES:")) {
            auto t = tokens(line);
            P.ntypes = to_int(t, 2, "ATOM TYPES");
            if (P.ntypes < 1 || P.ntypes > kMaxTypes) fail("number of atom types must lie in [1,8]");
            P.eoff.assign(P.ntypes, 0.0);
        }
        if (has(line, "# TYPEIDX #")) {
            P.atm.assign(P.ntypes, "");
            P.mass.assign(P.ntypes, 0.0);
            for (int i = 0; i < P.ntypes; i++) {
                if (!L.next(line)) fail("error reading line: truncated TYPEIDX block");
                auto t = tokens(line);
                P.atm[i] = tok(t, 1, "TYPEIDX row");
                P.mass[i] = to_dbl(t, 3, "TYPEIDX row");
            }
        }
        if (has(line, "ATOM PAIRS:")) {
            auto t = tokens(line);
            no_pairs = to_int(t, 2, "ATOM PAIRS");
        }
        if (has(line, "# PAIRIDX #")) {
            if (has(line, "# USEOVRP #")) continue;
            if (no_pairs <= 0) fail("PAIRIDX block before ATOM PAIRS");
            P.npairs = no_pairs;
            P.pa1.assign(no_pairs, ""); P.pa2.assign(no_pairs, "");
            P.rin.assign(no_pairs, 0.0); P.rout.assign(no_pairs, 0.0); P.lam.assign(no_pairs, 0.0);
            std::string style;
            for (int i = 0; i < no_pairs; i++) {
                if (!L.next(line)) fail("error reading line: truncated PAIRIDX block");
                auto t = tokens(line);
                int xf, mo;
                if (t.size() == 8) { xf = 6; mo = 7; }
                else if (t.size() == 7) { xf = 5; mo = 6; }
                else fail("incorrect input in pair line (expect 7 or 8 entries): " + line);
                P.pa1[i] = t[1]; P.pa2[i] = t[2];
                P.rin[i] = to_dbl(t, 3, "pair line");
                P.rout[i] = to_dbl(t, 4, "pair line");
                if (i == 0) style = t[xf];
                else if (t[xf] != style) fail("distance transformation style must be the same for all pair types");
                if (style != "MORSE") fail("only the MORSE distance transformation is supported: " + style);
                P.lam[i] = to_dbl(t, mo, "pair line (MORSE lambda)");
            }
        }
        if (has(line, "FCUT TYPE:")) {
            auto t = tokens(line);
            const std::string& s = tok(t, 2, "FCUT TYPE");
            if (s == "CUBIC") P.tersoff = false;
            else if (s == "TERSOFF") { P.tersoff = true; P.fcut_var = to_dbl(t, 3, "FCUT TYPE"); }
            else fail("unknown FCUT TYPE: " + s);
        }
        if (has(line, "PAIR CHEBYSHEV PENALTY DIST:")) P.pen_dist = to_dbl(tokens(line), 4, "PENALTY DIST");
        if (has(line, "PAIR CHEBYSHEV PENALTY SCALING:")) P.pen_scale = to_dbl(tokens(line), 4, "PENALTY SCALING");
        if (has(line, "NO ENERGY OFFSETS:")) {
            auto t = tokens(line);
            if (t.empty() || to_int(t, t.size() - 1, "NO ENERGY OFFSETS") != P.ntypes)
                fail("number of energy offsets does not match number of atom types");
            for (int i = 0; i < P.ntypes; i++) {
                if (!L.next(line)) fail("error reading line: truncated energy offsets");
                auto u = tokens(line);
                int k = to_int(u, 2, "ENERGY OFFSET");
                if (k < 1 || k > P.ntypes) fail("energy offset index out of range");
                P.eoff[k - 1] = to_dbl(u, 3, "ENERGY OFFSET");
            }
        }
    }
    if (P.ntypes < 1 || (int)P.atm.size() != P.ntypes) fail("missing ATOM TYPES / TYPEIDX block");
    if (P.npairs < 1) fail("missing ATOM PAIRS / PAIRIDX block");
    const int nt = P.ntypes;

    // pass 3: 2B coefficients and PAIRMAPS (chimesFF.cpp:694-830)
    L.rewind();
    P.pows2.assign(P.npairs, {});
    P.coef2.assign(P.npairs, {});
    bool have_pmap = false;
    int n_plain2 = 0;
    while (true) {
        if (!L.next(line)) fail("error reading line: missing ENDFILE");
        if (has(line, "ENDFILE")) break;
        if (has(line, "PAIRTYPE PARAMS:")) {
            auto t = tokens(line);
            if (t.size() == 7) {   // PAIRTYPE PARAMS: <i> <a> <b> TABULATED <table> (chimesFF.cpp:719-735)
                if (n_plain2 > 0)
                    fail("All parameters of a given bodiedness must either be tabulated or not tabulated, but not "
                         "a mixture of each");
                read_tab2(dir, t[6], P);
                P.tab2 = true;
                continue;
            }
            if (P.tab2)
                fail("All parameters of a given bodiedness must either be tabulated or not tabulated, but not a "
                     "mixture of each");
            n_plain2++;
            int p = to_int(t, 2, "PAIRTYPE PARAMS");
            if (p < 0 || p >= P.npairs) fail("PAIRTYPE PARAMS index out of range");
            if (!L.next(line)) fail("error reading line");
            P.pows2[p].clear(); P.coef2[p].clear();
            for (int i = 0; i < P.o2; i++) {
                if (!L.next(line)) fail("error reading line: truncated 2B parameters");
                auto u = tokens(line);
                int pw = to_int(u, 0, "2B parameter");
                if (pw < 0 || pw + 1 > P.o2) fail("2B power out of range for the 2B order");
                P.pows2[p].push_back(pw);
                P.coef2[p].push_back(to_dbl(u, 1, "2B parameter"));
            }
        }
        if (has(line, "PAIRMAPS:")) {
            auto t = tokens(line);
            int nm = to_int(t, 1, "PAIRMAPS");
            std::map<std::string, int> m;
            std::vector<std::string> order;
            for (int i = 0; i < nm; i++) {
                if (!L.next(line)) fail("error reading line: truncated PAIRMAPS");
                auto u = tokens(line);
                const std::string& key = tok(u, 1, "PAIRMAPS row");
                const int idx = to_int(u, 0, "PAIRMAPS row");
                P.pair_map_file_idx.push_back(idx);
                if (!m.count(key)) m[key] = idx;
            }
            P.pair_map.assign(nt * nt, 0);
            P.prpr.assign(nt * nt, 0);
            for (int i = 0; i < nt; i++)
                for (int j = 0; j < nt; j++) {
                    auto it = m.find(P.atm[i] + P.atm[j]);
                    if (it == m.end()) fail("could not find element in vector: " + P.atm[i] + P.atm[j]);
                    if (it->second < 0 || it->second >= P.npairs) fail("PAIRMAPS index out of range");
                    P.pair_map[i * nt + j] = it->second;
                    P.prpr[i * nt + j] = proper_pair(P, P.atm[i], P.atm[j]);
                }
            have_pmap = true;
        }
    }
    if (!have_pmap) fail("missing PAIRMAPS block");
    if (P.tab2) {
        // get_tab_2B indexes the tables by pair type
        if ((int)P.t2tab.size() < P.npairs) fail("fewer tabulated 2-body tables than pair types");
    } else {
        for (int p = 0; p < P.npairs; p++)
            if ((int)P.coef2[p].size() != P.o2) fail("missing PAIRTYPE PARAMS block for a pair type");
    }

    // passes 4-7: 3B and 4B blocks (chimesFF.cpp:834-1567)
    for (int nb = 3; nb <= 4; nb++) {
        HostParams::Body& B = nb == 3 ? P.b3 : P.b4;
        const int order = nb == 3 ? P.o3 : P.o4;
        B.nbody = nb;
        B.npair = nb * (nb - 1) / 2;
        if (order <= 0) continue;
        const int np = B.npair;
        const char* h_count = nb == 3 ? "ATOM PAIR TRIPLETS:" : "ATOM PAIR QUADRUPLETS:";
        const char* h_type = nb == 3 ? "TRIPLETTYPE PARAMS:" : "QUADRUPLETYPE PARAMS:";
        const char* h_maps = nb == 3 ? "TRIPMAPS:" : "QUADMAPS:";
        std::map<std::string, int> keys;   // map key -> type index
        int ntup = 1;
        for (int k = 0; k < nb; k++) ntup *= nt;
        L.rewind();
        bool have_map = false;
        while (true) {
            if (!L.next(line)) fail("error reading line: missing ENDFILE");
            if (has(line, "ENDFILE")) break;
            if (has(line, h_count)) {
                auto t = tokens(line);
                B.ntyp = to_int(t, 3, h_count);
                if (B.ntyp < 0) fail("negative cluster type count");
                B.ncoef.assign(B.ntyp, 0);
                B.pows.assign(B.ntyp, {});
                B.coef.assign(B.ntyp, {});
                B.cut_in.assign(B.ntyp, std::vector<double>(np, 0.0));
                B.cut_out.assign(B.ntyp, std::vector<double>(np, 0.0));
                B.atoms.assign(B.ntyp, {});
                B.pairs.assign(B.ntyp, {});
            }
            if (has(line, h_type)) {
                if (!L.next(line)) fail("error reading line");
                auto t = tokens(line);
                int ti = to_int(t, 1, h_type);
                if (ti < 0 || ti >= B.ntyp) fail("cluster type index out of range");
                B.atoms[ti].clear();
                for (int a = 0; a < nb; a++) B.atoms[ti].push_back(tok(t, 3 + a, h_type));
                if (nb == 3 && t.size() == 8) {   // INDEX: i ATOMS: a b c TABULATED <table> (:882-896)
                    read_tab3(dir, t[7], P);
                    P.tab3 = true;
                }
                if (!L.next(line)) fail("error reading line");
                auto u = tokens(line);
                B.pairs[ti].clear();
                for (int p = 0; p < np; p++) B.pairs[ti].push_back(tok(u, 1 + p, "PAIRS line"));
                // once a triplet is tabulated no later triplet's coefficients are read (:912-918)
                if (tok(u, 1 + np, "PAIRS line") != "EXCLUDED:" && !(nb == 3 && P.tab3)) {
                    int nc = to_int(u, nb == 3 ? 7 : 10, "PAIRS line (TOTAL)");
                    if (nc < 0) fail("negative coefficient count");
                    B.ncoef[ti] = nc;
                    if (!L.next(line) || !L.next(line)) fail("error reading line");
                    B.pows[ti].assign((size_t)nc * np, 0);
                    B.coef[ti].assign(nc, 0.0);
                    for (int c = 0; c < nc; c++) {
                        if (!L.next(line)) fail("error reading line: truncated coefficient list");
                        auto w = tokens(line);
                        for (int p = 0; p < np; p++) {
                            int pw = to_int(w, 1 + p, "coefficient row");
                            if (pw < 0 || pw > order) fail("many-body power larger than its order");
                            B.pows[ti][(size_t)c * np + p] = pw;
                        }
                        B.coef[ti][c] = to_dbl(w, nb == 3 ? 6 : 9, "coefficient row");
                    }
                }
            }
            if (has(line, h_maps)) {
                auto t = tokens(line);
                int nm = to_int(t, 1, h_maps);
                for (int i = 0; i < nm; i++) {
                    if (!L.next(line)) fail("error reading line: truncated map block");
                    auto u = tokens(line);
                    const std::string& key = tok(u, 1, "map row");
                    if (!keys.count(key)) keys[key] = to_int(u, 0, "map row");
                }
                B.map.assign(ntup, 0);
                for (int uidx = 0; uidx < ntup; uidx++) {
                    int a[4], r = uidx;
                    for (int k = nb - 1; k >= 0; k--) { a[k] = r % nt; r /= nt; }
                    std::string key;
                    for (int i = 0; i < nb; i++)
                        for (int j = i + 1; j < nb; j++) key += P.pair_name(proper_pair(P, P.atm[a[i]], P.atm[a[j]]));
                    auto it = keys.find(key);
                    if (it == keys.end()) fail("could not find element in vector: " + key);
                    if (it->second >= B.ntyp) fail("cluster map index out of range");
                    B.map[uidx] = it->second;
                }
                have_map = true;
            }
        }
        if (!have_map) fail(std::string("missing ") + h_maps + " block");
        if (nb == 3 && P.tab3)   // get_tab_3B indexes the tables by triplet type
            for (int v : B.map)
                if (v >= (int)P.t3tab.size()) fail("no tabulated 3-body table for triplet type " + std::to_string(v));
        for (int ti = 0; ti < B.ntyp; ti++)
            if ((int)B.atoms[ti].size() != nb || (int)B.pairs[ti].size() != np) fail("missing cluster type block");
        // default cutoffs from the 2B pair types of the type's atoms (chimesFF.cpp:947-980, 1280-1325)
        for (int ti = 0; ti < B.ntyp; ti++) {
            int a[4];
            for (int k = 0; k < nb; k++) {
                a[k] = P.type_index(B.atoms[ti][k]);
                if (a[k] < 0) fail("cluster type names an unknown atom type: " + B.atoms[ti][k]);
            }
            int p = 0;
            for (int i = 0; i < nb; i++)
                for (int j = i + 1; j < nb; j++, p++) {
                    int pt = P.pair_map[a[i] * nt + a[j]];
                    B.cut_in[ti][p] = P.rin[pt];
                    B.cut_out[ti][p] = P.rout[pt];
                }
        }
        // SPECIAL nB S_MAXIM / S_MINIM: ALL v | SPECIFIC n (chimesFF.cpp:1009-1168, 1353-1566)
        const std::string smax = nb == 3 ? "SPECIAL 3B S_MAXIM:" : "SPECIAL 4B S_MAXIM:";
        const std::string smin = nb == 3 ? "SPECIAL 3B S_MINIM:" : "SPECIAL 4B S_MINIM:";
        L.rewind();
        while (true) {
            if (!L.next(line)) fail("error reading line: missing ENDFILE");
            if (has(line, "ENDFILE")) break;
            int which = has(line, smax.c_str()) ? 1 : (has(line, smin.c_str()) ? 0 : -1);
            if (which < 0) continue;
            auto t = tokens(line);
            auto& dst = which ? B.cut_out : B.cut_in;
            if (tok(t, 3, "SPECIAL") == "ALL") {
                double v = to_dbl(t, 4, "SPECIAL ALL");
                for (auto& row : dst) std::fill(row.begin(), row.end(), v);
            } else {
                int ne = to_int(t, 4, "SPECIAL SPECIFIC");
                if (which == 0 && nb == 4)
                    for (auto& row : dst) std::fill(row.begin(), row.end(), -1.0);
                for (int e = 0; e < ne; e++) {
                    if (!L.next(line)) fail("error reading line: truncated SPECIAL block");
                    auto u = tokens(line);
                    auto it = keys.find(tok(u, 0, "SPECIAL row"));
                    if (it == keys.end() || it->second < 0 || it->second >= B.ntyp)
                        fail("SPECIAL row names an unknown cluster type");
                    int ti = it->second;
                    std::vector<bool> disq(np, false);
                    for (int q = 0; q < np; q++) {
                        const std::string& nm = tok(u, 1 + q, "SPECIAL row");
                        int slot = -1;
                        for (int p = 0; p < np; p++)
                            if (B.pairs[ti][p] == nm && !disq[p]) { disq[p] = true; slot = p; break; }
                        if (slot < 0) fail("could not find element in vector: " + nm);
                        dst[ti][slot] = to_dbl(u, 1 + np + q, "SPECIAL row");
                    }
                }
            }
        }
        // pair_int_{trip,quad}_map
        B.perm.assign(ntup, std::vector<int>(np, 0));
        std::vector<int> pm(np, 0);
        for (int uidx = 0; uidx < ntup; uidx++) {
            int a[4], r = uidx;
            for (int k = nb - 1; k >= 0; k--) { a[k] = r % nt; r /= nt; }
            int ti = B.map[uidx];
            if (ti < 0) continue;
            atom_pair_mapper(P, nb, a, B.pairs[ti], pm);
            B.perm[uidx] = pm;
        }
    }
}

}  // namespace

double HostParams::max_cut2() const {
    double m = rout[0];
    for (double v : rout) if (v > m) m = v;
    return m;
}

static double max_cut_body(const HostParams::Body& B, int order) {
    if (order == 0 || B.ntyp == 0) return 0.0;
    double m = B.cut_out[0][0];
    for (auto& row : B.cut_out) for (double v : row) if (v > m) m = v;
    return m;
}
double HostParams::max_cut3() const { return max_cut_body(b3, o3); }
double HostParams::max_cut4() const { return max_cut_body(b4, o4); }

int HostParams::type_index(const std::string& name) const {
    for (int i = 0; i < ntypes; i++) if (atm[i] == name) return i;
    return -1;
}

// ---------------------------------------------------------------------------
// Binary parameter cache: the parsed tables in a flat little-endian stream
// ("CKPC" magic, format version, then every HostParams field in declaration
// order; strings and vectors carry their lengths).  Loading it skips the text
// parse; packing it gives the same device image as the text file.
// ---------------------------------------------------------------------------
namespace {
constexpr char kCacheMagic[4] = {'C', 'K', 'P', 'C'};
constexpr int kCacheVersion = 2;

struct Writer {
    std::string b;
    void raw(const void* p, size_t n) { b.append(static_cast<const char*>(p), n); }
    void i(long long v) { raw(&v, sizeof(v)); }
    void d(double v) { raw(&v, sizeof(v)); }
    void str(const std::string& v) { i((long long)v.size()); raw(v.data(), v.size()); }
    void vi(const std::vector<int>& v) { i((long long)v.size()); for (int x : v) i(x); }
    void vd(const std::vector<double>& v) { i((long long)v.size()); raw(v.data(), v.size() * sizeof(double)); }
    void vs(const std::vector<std::string>& v) { i((long long)v.size()); for (auto& x : v) str(x); }
    void vvi(const std::vector<std::vector<int>>& v) { i((long long)v.size()); for (auto& x : v) vi(x); }
    void vvd(const std::vector<std::vector<double>>& v) { i((long long)v.size()); for (auto& x : v) vd(x); }
    void vvs(const std::vector<std::vector<std::string>>& v) { i((long long)v.size()); for (auto& x : v) vs(x); }
};

struct Reader {
    const std::string& b;
    size_t pos = 0;
    explicit Reader(const std::string& s) : b(s) {}
    void raw(void* p, size_t n) {
        if (pos + n > b.size()) throw ParseError{"truncated parameter cache"};
        std::memcpy(p, b.data() + pos, n);
        pos += n;
    }
    long long i() { long long v; raw(&v, sizeof(v)); return v; }
    double d() { double v; raw(&v, sizeof(v)); return v; }
    size_t len() {
        const long long n = i();
        if (n < 0 || (size_t)n > b.size()) throw ParseError{"corrupt parameter cache"};
        return (size_t)n;
    }
    std::string str() { std::string v(len(), '\0'); raw(&v[0], v.size()); return v; }
    std::vector<int> vi() { std::vector<int> v(len()); for (auto& x : v) x = (int)i(); return v; }
    std::vector<double> vd() { std::vector<double> v(len()); raw(v.data(), v.size() * sizeof(double)); return v; }
    std::vector<std::string> vs() { std::vector<std::string> v(len()); for (auto& x : v) x = str(); return v; }
    std::vector<std::vector<int>> vvi() { std::vector<std::vector<int>> v(len()); for (auto& x : v) x = vi(); return v; }
    std::vector<std::vector<double>> vvd() { std::vector<std::vector<double>> v(len()); for (auto& x : v) x = vd(); return v; }
    std::vector<std::vector<std::string>> vvs() {
        std::vector<std::vector<std::string>> v(len());
        for (auto& x : v) x = vs();
        return v;
    }
};

void put_body(Writer& w, const HostParams::Body& B) {
    w.i(B.nbody); w.i(B.npair); w.i(B.ntyp);
    w.vi(B.ncoef); w.vvi(B.pows); w.vvd(B.coef); w.vvd(B.cut_in); w.vvd(B.cut_out);
    w.vvs(B.atoms); w.vvs(B.pairs); w.vi(B.map); w.vvi(B.perm);
}

void get_body(Reader& r, HostParams::Body& B) {
    B.nbody = (int)r.i(); B.npair = (int)r.i(); B.ntyp = (int)r.i();
    B.ncoef = r.vi(); B.pows = r.vvi(); B.coef = r.vvd(); B.cut_in = r.vvd(); B.cut_out = r.vvd();
    B.atoms = r.vvs(); B.pairs = r.vvs(); B.map = r.vi(); B.perm = r.vvi();
}

void get_params(Reader& r, HostParams& P) {
    P.ntypes = (int)r.i(); P.npairs = (int)r.i();
    P.o2 = (int)r.i(); P.o3 = (int)r.i(); P.o4 = (int)r.i();
    P.atm = r.vs(); P.mass = r.vd(); P.pa1 = r.vs(); P.pa2 = r.vs();
    P.rin = r.vd(); P.rout = r.vd(); P.lam = r.vd();
    P.tersoff = r.i() != 0;
    P.fcut_var = r.d(); P.pen_dist = r.d(); P.pen_scale = r.d(); P.inner_smooth = r.d();
    P.eoff = r.vd(); P.pows2 = r.vvi(); P.coef2 = r.vvd();
    P.pair_map = r.vi(); P.prpr = r.vi(); P.pair_map_file_idx = r.vi();
    get_body(r, P.b3);
    get_body(r, P.b4);
    P.tab2 = r.i() != 0;
    P.t2tab.resize(r.len());
    for (auto& T : P.t2tab) { T.r = r.vd(); T.e = r.vd(); T.f = r.vd(); }
    P.tab3 = r.i() != 0;
    P.t3tab.resize(r.len());
    for (auto& T : P.t3tab) {
        T.rij = r.vd(); T.rik = r.vd(); T.rjk = r.vd();
        T.e = r.vd(); T.fij = r.vd(); T.fik = r.vd(); T.fjk = r.vd();
    }
    // the kernels index these tables without further checks
    const int nt = P.ntypes;
    if (nt <= 0 || nt > kMaxTypes || P.npairs != nt * (nt + 1) / 2 || (int)P.pair_map.size() != nt * nt ||
        (int)P.rin.size() != P.npairs || (int)P.coef2.size() != P.npairs || (int)P.eoff.size() != nt ||
        P.o2 < 0 || P.o2 > kMaxOrder || P.o3 < 0 || P.o3 > kMaxOrder || P.o4 < 0 || P.o4 > kMaxOrder)
        throw ParseError{"inconsistent parameter cache"};
    for (int v : P.pair_map)
        if (v < 0 || v >= P.npairs) throw ParseError{"inconsistent parameter cache"};
    if (P.tab2 && (int)P.t2tab.size() < P.npairs) throw ParseError{"inconsistent parameter cache"};
    for (auto& T : P.t2tab) {
        if (T.e.size() != T.r.size() || T.f.size() != T.r.size()) throw ParseError{"inconsistent parameter cache"};
        for (size_t i = 1; i < T.r.size(); i++)
            if (!(T.r[i] > T.r[i - 1])) throw ParseError{"inconsistent parameter cache"};
    }
    for (auto& T : P.t3tab) {
        const size_t n = T.rij.size();
        if (T.rik.size() != n || T.rjk.size() != n || T.e.size() != n || T.fij.size() != n || T.fik.size() != n ||
            T.fjk.size() != n || (int)std::cbrt((double)n) < 2)
            throw ParseError{"inconsistent parameter cache"};
    }
    if (P.tab3 && P.o3 > 0)
        for (int v : P.b3.map)
            if (v >= (int)P.t3tab.size()) throw ParseError{"inconsistent parameter cache"};
    for (int nb = 3; nb <= 4; nb++) {
        const HostParams::Body& B = nb == 3 ? P.b3 : P.b4;
        if ((nb == 3 ? P.o3 : P.o4) == 0) continue;
        int ntup = 1;
        for (int k = 0; k < nb; k++) ntup *= nt;
        if ((int)B.map.size() != ntup || (int)B.perm.size() != ntup) throw ParseError{"inconsistent parameter cache"};
        for (int u = 0; u < ntup; u++) {
            const int ti = B.map[u];
            if (ti < 0) continue;
            if (ti >= (int)B.ncoef.size() || ti >= (int)B.pows.size() || ti >= (int)B.coef.size() ||
                ti >= (int)B.cut_in.size() || ti >= (int)B.cut_out.size() || (int)B.perm[u].size() != B.npair ||
                (long long)B.pows[ti].size() != (long long)B.ncoef[ti] * B.npair ||
                (int)B.coef[ti].size() != B.ncoef[ti])
                throw ParseError{"inconsistent parameter cache"};
            for (int m : B.perm[u])
                if (m < 0 || m >= B.npair || m >= (int)B.cut_in[ti].size() || m >= (int)B.cut_out[ti].size())
                    throw ParseError{"inconsistent parameter cache"};
            for (int v : B.pows[ti])
                if (v < 0 || v > kMaxOrder) throw ParseError{"inconsistent parameter cache"};
        }
    }
}
}  // namespace

Status save_parameter_cache(const HostParams& P, const std::string& path, std::string& err) {
    Writer w;
    w.raw(kCacheMagic, 4);
    w.i(kCacheVersion);
    w.i(P.ntypes); w.i(P.npairs); w.i(P.o2); w.i(P.o3); w.i(P.o4);
    w.vs(P.atm); w.vd(P.mass); w.vs(P.pa1); w.vs(P.pa2);
    w.vd(P.rin); w.vd(P.rout); w.vd(P.lam);
    w.i(P.tersoff ? 1 : 0);
    w.d(P.fcut_var); w.d(P.pen_dist); w.d(P.pen_scale); w.d(P.inner_smooth);
    w.vd(P.eoff); w.vvi(P.pows2); w.vvd(P.coef2);
    w.vi(P.pair_map); w.vi(P.prpr); w.vi(P.pair_map_file_idx);
    put_body(w, P.b3);
    put_body(w, P.b4);
    w.i(P.tab2 ? 1 : 0);
    w.i((long long)P.t2tab.size());
    for (auto& T : P.t2tab) { w.vd(T.r); w.vd(T.e); w.vd(T.f); }
    w.i(P.tab3 ? 1 : 0);
    w.i((long long)P.t3tab.size());
    for (auto& T : P.t3tab) {
        w.vd(T.rij); w.vd(T.rik); w.vd(T.rjk);
        w.vd(T.e); w.vd(T.fij); w.vd(T.fik); w.vd(T.fjk);
    }
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f.is_open()) {
        err = "cannot write parameter cache: " + path;
        return kErrParam;
    }
    f.write(w.b.data(), (std::streamsize)w.b.size());
    if (!f) {
        err = "error writing parameter cache: " + path;
        return kErrParam;
    }
    return kOk;
}

Status parse_parameter_file(const std::string& path, HostParams& P, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) {
        err = "cannot open parameter file: " + path;
        return kErrParam;
    }
    char head[4] = {0, 0, 0, 0};
    f.read(head, 4);
    if (f.gcount() == 4 && std::memcmp(head, kCacheMagic, 4) == 0) {
        std::string all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        P = HostParams();
        try {
            Reader r(all);
            if (r.i() != kCacheVersion) throw ParseError{"parameter cache of another format version"};
            get_params(r, P);
        } catch (const ParseError& e) {
            err = e.msg + ": " + path;
            return kErrParam;
        }
        return kOk;
    }
    f.clear();
    f.seekg(0);
    Lines L;
    std::string line;
    while (std::getline(f, line)) L.v.push_back(line);
    P = HostParams();
    const size_t slash = path.find_last_of("/\\");
    const std::string dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
    try {
        parse_lines(L, P, dir);
    } catch (const ParseError& e) {
        err = e.msg;
        return kErrParam;
    }
    return kOk;
}

// ---------------------------------------------------------------------------
// Device image
// ---------------------------------------------------------------------------
namespace {
struct Blob {
    std::vector<unsigned char> b;
    template <class T>
    size_t add(const T* p, size_t n) {
        size_t off = (b.size() + 255) & ~size_t(255);
        b.resize(off + n * sizeof(T));
        if (n) std::memcpy(b.data() + off, p, n * sizeof(T));
        return off;
    }
};
template <class T>
T* as_off(size_t off) { return reinterpret_cast<T*>(off); }

// TF32 rounding for the tensor-core contraction's operand split: x rounded to
// 10 explicit mantissa bits, ties away from zero.
float tf32_hi_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xffffe000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// Tensor-core image of one 3-body tuple's dense coefficient matrix
// A[q0][q1*Rw + q2] (q0 the ij power, q1 ik, q2 jk; the tuple's R powers per
// pair, zero above) for a kernel working with Rw >= R powers: the B operand
// of W = X . A with X = T_ij, stored as N = tc3_npad(Rw) rows (J) of
// K = tc3_kpad(Rw) values (q0), K-major, no swizzle: the core matrix of rows
// 8i..8i+7 and k = 4j..4j+3 (8 x 16 bytes) at byte (i * K/4 + j) * 128, row
// n % 8 at +16 * (n % 8).  kTc3Parts parts follow each other: the TF32
// rounding of the coefficient, of what it leaves, and so on (the last part
// is the FP32 remainder, which the tensor core truncates to TF32).
void tc3_image(const std::vector<double>& dense, int R, int Rw, std::vector<float>& out) {
    const int kpad = tc3_kpad(Rw), npad = tc3_npad(Rw);
    const size_t base = out.size();
    const size_t part = (size_t)kpad * npad;
    out.resize(base + kTc3Parts * part, 0.0f);
    for (int q1 = 0; q1 < R; q1++)
        for (int q2 = 0; q2 < R; q2++)
            for (int k = 0; k < R; k++) {
                double rest = dense[(size_t)k * R * R + q1 * R + q2];
                const int n = q1 * Rw + q2;
                const size_t off = ((size_t)(n / 8) * (kpad / 4) + k / 4) * 32 + (n % 8) * 4 + (k % 4);
                for (int t = 0; t < kTc3Parts; t++) {
                    const float v = t + 1 < kTc3Parts ? tf32_hi_host((float)rest) : (float)rest;
                    out[base + t * part + off] = v;
                    rest -= (double)v;
                }
            }
}

// Tensor-core image of one 4-body tuple's dense coefficient matrix
// A[I][J] (I = (q_ij, q_ik, q_il), J = (q_jk, q_jl, q_kl), n3 = R^3 each):
// the B operand of W = X . A, N = tc4_npad(n3) rows (J) of K = tc4_kpad(n3)
// values (I), in tc3_image's layout and parts.
void tc4_image(const std::vector<double>& dense, int n3, std::vector<float>& out) {
    const int kpad = tc4_kpad(n3), npad = tc4_npad(n3);
    const size_t base = out.size();
    const size_t part = (size_t)kpad * npad;
    out.resize(base + kTc3Parts * part, 0.0f);
    for (int n = 0; n < n3; n++)
        for (int k = 0; k < n3; k++) {
            double rest = dense[(size_t)k * n3 + n];
            const size_t off = ((size_t)(n / 8) * (kpad / 4) + k / 4) * 32 + (n % 8) * 4 + (k % 4);
            for (int t = 0; t < kTc3Parts; t++) {
                const float v = t + 1 < kTc3Parts ? tf32_hi_host((float)rest) : (float)rest;
                out[base + t * part + off] = v;
                rest -= (double)v;
            }
        }
}

// set_cheby_polys' Morse-map constants (chimesFF.h:553-559)
void morse_consts(double rin, double rout, double lam, double& xavg, double& xdiff) {
    double x_min = std::exp(-1 * rin / lam);
    double x_max = std::exp(-1 * rout / lam);
    xavg = 0.5 * (x_max + x_min);
    xdiff = 0.5 * (x_max - x_min);
    xdiff *= -1.0;
}
// Local cubic of get_tab_2B (chimesFF.cpp:1898-1916) on the interval that
// starts at grid point i (1 <= i <= n-2), for table y: q = {a, b, c, d}.
// The expressions keep the reference's operation order (the host code is
// compiled without contraction), so the coefficients are bit-identical.
void tab2_interval(const std::vector<double>& r, const std::vector<double>& y, int i, double* q) {
    const double h = r[i + 1] - r[i];
    const double alpha = (3 * (y[i + 1] - y[i]) / h) - (3 * (y[i] - y[i - 1]) / (r[i] - r[i - 1]));
    const double l = 2 * (r[i + 1] - r[i - 1]) - h;
    const double mu = h / l;
    const double z = alpha / l;
    const double c_prev = 0.0;   // natural-spline end condition of the reference
    const double c = z - mu * c_prev;
    const double b = (y[i + 1] - y[i]) / h - h * (c + 2 * c_prev) / 3.0;
    const double d = (c - c_prev) / (3.0 * h);
    q[0] = y[i];
    q[1] = b;
    q[2] = c;
    q[3] = d;
}
}  // namespace

ParamImage pack_params(const HostParams& P) {
    ParamImage img;
    Blob B;
    B.b.resize(256);   // no array at offset 0, so a zero offset can mean "absent"
    DevParamSet& H = img.header;
    const int nt = P.ntypes;
    H.ntypes = nt; H.npairs = P.npairs; H.o2 = P.o2; H.o3 = P.o3; H.o4 = P.o4;
    H.tersoff = P.tersoff ? 1 : 0;
    H.fcut_var = P.fcut_var; H.pen_dist = P.pen_dist; H.pen_scale = P.pen_scale; H.inner_smooth = P.inner_smooth;
    H.maxcut2 = P.max_cut2(); H.maxcut3 = P.max_cut3(); H.maxcut4 = P.max_cut4();
    H.search = H.maxcut2;
    if (H.maxcut3 > H.search) H.search = H.maxcut3;
    if (H.maxcut4 > H.search) H.search = H.maxcut4;

    H.eoff = as_off<const double>(B.add(P.eoff.data(), P.eoff.size()));
    H.pair_map = as_off<const int>(B.add(P.pair_map.data(), P.pair_map.size()));
    std::vector<PairRec> pr(P.npairs);
    std::vector<double> c2d;
    std::vector<float> c2f;
    std::vector<int> p2;
    for (int p = 0; p < P.npairs; p++) {
        pr[p].rin = P.rin[p]; pr[p].rout = P.rout[p]; pr[p].lam = P.lam[p];
        morse_consts(P.rin[p], P.rout[p], P.lam[p], pr[p].xavg, pr[p].xdiff);
        pr[p].inv_lam = 1.0 / pr[p].lam;
        pr[p].inv_xdiff = 1.0 / pr[p].xdiff;
        if (P.tersoff) {
            pr[p].fc_th = pr[p].rout - P.fcut_var * pr[p].rout;
            pr[p].fc_inv = 1.0 / (pr[p].rout - pr[p].fc_th);
        } else {
            pr[p].fc_th = 0.0;
            pr[p].fc_inv = 1.0 / pr[p].rout;
        }
        // dense table a_n (n = 0..o2) with a_{pow+1} = sum of the coefficients of
        // that power: the 2B kernel sums along the Chebyshev recursion
        pr[p].ncoef = P.o2 + 1;
        pr[p].coef_off = (int)c2d.size();
        std::vector<double> dense(P.o2 + 1, 0.0);
        for (int c = 0; c < (int)P.coef2[p].size(); c++) {   // none when the 2-body term is tabulated
            dense[P.pows2[p][c] + 1] += P.coef2[p][c];
            p2.push_back(P.pows2[p][c]);
        }
        for (int n = 0; n <= P.o2; n++) {
            c2d.push_back(dense[n]);
            c2f.push_back((float)dense[n]);
        }
    }
    H.pairs = as_off<const PairRec>(B.add(pr.data(), pr.size()));
    H.c2d = as_off<const double>(B.add(c2d.data(), c2d.size()));
    H.c2f = as_off<const float>(B.add(c2f.data(), c2f.size()));
    H.p2 = as_off<const int>(B.add(p2.data(), p2.size()));

    for (int nb = 3; nb <= 4; nb++) {
        const HostParams::Body& Bd = nb == 3 ? P.b3 : P.b4;
        const int order = nb == 3 ? P.o3 : P.o4;
        if (order <= 0) continue;
        const int np = Bd.npair;
        int ntup = 1;
        for (int k = 0; k < nb; k++) ntup *= nt;
        std::vector<TupleRec> tr(ntup);
        std::vector<double> cd;
        std::vector<float> cf;
        std::vector<uint32_t> pw;
        // factored tables: R powers per pair; kept when R^K and R^(P-K) fit
        const int K = nb == 3 ? 1 : 3;
        int R_pow = 1;
        for (size_t ti = 0; ti < Bd.pows.size(); ti++)
            for (int v : Bd.pows[ti]) R_pow = std::max(R_pow, v + 1);
        long long rk = 1, rc = 1;
        for (int k = 0; k < K; k++) rk *= R_pow;
        for (int k = K; k < np; k++) rc *= R_pow;
        const bool fact = rk <= kFactMaxDim && rc <= kFactMaxDim;
        std::vector<FactRow> fr;
        std::vector<FactEntD> fed;
        std::vector<FactEntF> fef;
        // tensor-core images (3-body, R <= kTc3MaxR: N = R^2 <= 128 TMEM columns
        // per accumulator), one per working width Rw = R .. kTc3MaxR so that a
        // batch mixing sets of different orders runs at its largest R
        const bool tc = nb == 3 ? fact && R_pow >= 2 && R_pow <= kTc3MaxR
                                : fact && R_pow >= 2 && R_pow <= kTc4MaxR;
        std::vector<float> tcimg;
        struct Shared { int coef_off, f_row, f_nrow, f_ncol, f_ent, tc_off; };
        std::map<std::pair<int, std::vector<int>>, Shared> shared;  // (type, mapping) -> tables
        for (int u = 0; u < ntup; u++) {
            TupleRec& R = tr[u];
            std::memset(&R, 0, sizeof(R));
            int a[4], r = u;
            for (int k = nb - 1; k >= 0; k--) { a[k] = r % nt; r /= nt; }
            int ti = Bd.map[u];
            R.type_id = ti;
            if (ti < 0) continue;
            const std::vector<int>& m = Bd.perm[u];
            int p = 0;
            for (int i = 0; i < nb; i++)
                for (int j = i + 1; j < nb; j++, p++) {
                    R.rin[p] = Bd.cut_in[ti][m[p]];
                    R.rout[p] = Bd.cut_out[ti][m[p]];
                    R.rout_f[p] = (float)R.rout[p];
                    R.lam[p] = P.lam[P.pair_map[a[i] * nt + a[j]]];
                    morse_consts(R.rin[p], R.rout[p], R.lam[p], R.xavg[p], R.xdiff[p]);
                    R.inv_lam[p] = 1.0 / R.lam[p];
                    R.inv_xdiff[p] = 1.0 / R.xdiff[p];
                    if (P.tersoff) {
                        R.fc_th[p] = R.rout[p] - P.fcut_var * R.rout[p];
                        R.fc_inv[p] = 1.0 / (R.rout[p] - R.fc_th[p]);
                    } else {
                        R.fc_th[p] = 0.0;
                        R.fc_inv[p] = 1.0 / R.rout[p];
                    }
                }
            R.ncoef = Bd.ncoef[ti];
            R.valid = R.ncoef > 0 ? 1 : 0;
            R.tc_off = -1;
            auto key = std::make_pair(ti, m);
            auto it = shared.find(key);
            if (it != shared.end()) {
                R.coef_off = it->second.coef_off;
                R.f_row = it->second.f_row; R.f_nrow = it->second.f_nrow;
                R.f_ncol = it->second.f_ncol; R.f_ent = it->second.f_ent;
                R.tc_off = it->second.tc_off;
                continue;
            }
            R.coef_off = (int)cd.size();
            const int Rp = R_pow;
            std::vector<int> rowi(R.ncoef), coli(R.ncoef), rowp(R.ncoef), colp(R.ncoef);
            for (int c = 0; c < R.ncoef; c++) {
                cd.push_back(Bd.coef[ti][c]);
                cf.push_back((float)Bd.coef[ti][c]);
                uint32_t packed = 0;
                int I = 0, J = 0, Ip = 0, Jp = 0;
                for (int q = 0; q < np; q++) {
                    const int v = Bd.pows[ti][(size_t)c * np + m[q]];
                    packed |= uint32_t(v) << (kPowBits * q);
                    if (q < K) { I = I * Rp + v; Ip |= v << (kPowBits * q); }
                    else { J = J * Rp + v; Jp |= v << (kPowBits * (q - K)); }
                }
                pw.push_back(packed);
                rowi[c] = I;
                coli[c] = J;
                rowp[c] = Ip;
                colp[c] = Jp;
            }
            if (fact) {
                R.f_row = (int)fr.size();
                R.f_ent = (int)fed.size();
                // rows: entries by (I, J) holding (a, J); then columns: by (J, I) holding (a, I)
                for (int pass = 0; pass < 2; pass++) {
                    const std::vector<int>& major = pass == 0 ? rowi : coli;
                    const std::vector<int>& minor = pass == 0 ? coli : rowi;
                    const std::vector<int>& mpows = pass == 0 ? rowp : colp;
                    const std::vector<int>& opows = pass == 0 ? colp : rowp;   // the other side's powers
                    std::vector<int> ord(R.ncoef);
                    for (int c = 0; c < R.ncoef; c++) ord[c] = c;
                    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
                        return major[x] != major[y] ? major[x] < major[y] : minor[x] < minor[y];
                    });
                    int nrec = 0;
                    for (int k = 0; k < R.ncoef; k++) {
                        const int c = ord[k];
                        const bool last = k + 1 == R.ncoef || major[ord[k + 1]] != major[c];
                        const int code = (int)((uint32_t)minor[c] | ((uint32_t)opows[c] << 16) | (last ? 0x80000000u : 0u));
                        fed.push_back(FactEntD{Bd.coef[ti][c], code, 0});
                        fef.push_back(FactEntF{(float)Bd.coef[ti][c], code});
                        if (k + 1 == R.ncoef || major[ord[k + 1]] != major[c]) {
                            fr.push_back(FactRow{mpows[c], (int)fed.size()});
                            nrec++;
                        }
                    }
                    if (pass == 0) R.f_nrow = nrec; else R.f_ncol = nrec;
                }
            }
            if (tc && R.ncoef > 0 && nb == 3) {
                std::vector<double> dense((size_t)R_pow * R_pow * R_pow, 0.0);
                for (int c = 0; c < R.ncoef; c++) dense[(size_t)rowi[c] * R_pow * R_pow + coli[c]] += Bd.coef[ti][c];
                R.tc_off = (int)tcimg.size();
                for (int Rw = R_pow; Rw <= kTc3MaxR; Rw++) tc3_image(dense, R_pow, Rw, tcimg);
            }
            if (tc && R.ncoef > 0 && nb == 4) {
                const int n3 = R_pow * R_pow * R_pow;
                std::vector<double> dense((size_t)n3 * n3, 0.0);
                for (int c = 0; c < R.ncoef; c++) dense[(size_t)rowi[c] * n3 + coli[c]] += Bd.coef[ti][c];
                R.tc_off = (int)tcimg.size();
                tc4_image(dense, n3, tcimg);
            }
            shared[key] = Shared{R.coef_off, R.f_row, R.f_nrow, R.f_ncol, R.f_ent, R.tc_off};
        }
        // per-pair-type tables when no tuple overrides a pair type's cutoffs
        std::vector<PairTab> ptab(P.npairs);
        std::vector<int> seen(P.npairs, 0);
        bool uniform = true;
        for (int u = 0; u < ntup && uniform; u++) {
            const TupleRec& R = tr[u];
            if (!R.valid) continue;
            int a[4], r = u;
            for (int k = nb - 1; k >= 0; k--) { a[k] = r % nt; r /= nt; }
            int p = 0;
            for (int i = 0; i < nb; i++)
                for (int j = i + 1; j < nb; j++, p++) {
                    const int pt = P.pair_map[a[i] * nt + a[j]];
                    PairTab t{R.rin[p], R.rout[p], R.xavg[p], R.xdiff[p], R.inv_lam[p], R.inv_xdiff[p], R.fc_th[p],
                              R.fc_inv[p]};
                    if (!seen[pt]) { ptab[pt] = t; seen[pt] = 1; }
                    else if (std::memcmp(&ptab[pt], &t, sizeof(t)) != 0) uniform = false;
                }
        }
        size_t pto = uniform ? B.add(ptab.data(), ptab.size()) : 0;
        size_t tro = B.add(tr.data(), tr.size());
        size_t cdo = B.add(cd.data(), cd.size());
        size_t cfo = B.add(cf.data(), cf.size());
        size_t pwo = B.add(pw.data(), pw.size());
        size_t fro = 0, fdo = 0, ffo = 0;
        if (fact && !fed.empty()) {
            fro = B.add(fr.data(), fr.size());
            fdo = B.add(fed.data(), fed.size());
            ffo = B.add(fef.data(), fef.size());
        }
        const int Rf = (fact && !fed.empty()) ? R_pow : 0;
        if (nb == 3 && tc && Rf > 0 && !tcimg.empty()) {
            H.tc3_k = tc3_kpad(R_pow);
            H.tc3_n = tc3_npad(R_pow);
            H.tc3 = as_off<const float>(B.add(tcimg.data(), tcimg.size()));
            H.n_tc3 = (long long)tcimg.size();
        }
        if (nb == 4 && tc && Rf > 0 && !tcimg.empty()) {
            H.tc4_r = R_pow;
            H.tc4 = as_off<const float>(B.add(tcimg.data(), tcimg.size()));
            H.n_tc4 = (long long)tcimg.size();
        }
        if (nb == 3) {
            H.n_c3 = (long long)cd.size();
            H.n_fe3 = (long long)fed.size();
            H.t3 = as_off<const TupleRec>(tro); H.c3d = as_off<const double>(cdo);
            H.c3f = as_off<const float>(cfo); H.p3 = as_off<const uint32_t>(pwo);
            H.R3 = Rf;
            H.pt3 = as_off<const PairTab>(pto);
            H.fr3 = as_off<const FactRow>(fro); H.fe3d = as_off<const FactEntD>(fdo);
            H.fe3f = as_off<const FactEntF>(ffo);
        } else {
            H.n_c4 = (long long)cd.size();
            H.n_fe4 = (long long)fed.size();
            H.t4 = as_off<const TupleRec>(tro); H.c4d = as_off<const double>(cdo);
            H.c4f = as_off<const float>(cfo); H.p4 = as_off<const uint32_t>(pwo);
            H.R4 = Rf;
            H.pt4 = as_off<const PairTab>(pto);
            H.fr4 = as_off<const FactRow>(fro); H.fe4d = as_off<const FactEntD>(fdo);
            H.fe4f = as_off<const FactEntF>(ffo);
        }
    }
    // tabulated terms
    H.tab2 = P.tab2 ? 1 : 0;
    H.tab3 = P.tab3 ? 1 : 0;
    if (!P.t2tab.empty()) {
        std::vector<Tab2Rec> rec;
        std::vector<double> r, cf;
        for (const auto& T : P.t2tab) {
            const int n = (int)T.r.size();
            rec.push_back(Tab2Rec{(long long)r.size(), n, 0});
            r.insert(r.end(), T.r.begin(), T.r.end());
            for (int i = 0; i < n; i++) {
                double q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                if (i >= 1 && i <= n - 2)
                    for (int w = 0; w < 2; w++) tab2_interval(T.r, w == 0 ? T.e : T.f, i, &q[4 * w]);
                cf.insert(cf.end(), q, q + 8);
            }
        }
        H.n_tab2 = (int)rec.size();
        H.t2rec = as_off<const Tab2Rec>(B.add(rec.data(), rec.size()));
        H.tab2r = as_off<const double>(B.add(r.data(), r.size()));
        H.tab2c = as_off<const double>(B.add(cf.data(), cf.size()));
    }
    if (!P.t3tab.empty()) {
        std::vector<Tab3Rec> rec;
        std::vector<double> cols, vals;
        long long off = 0;
        for (const auto& T : P.t3tab) {
            const long long n = (long long)T.rij.size();
            Tab3Rec R{};
            R.off = off;
            R.nrows = n;
            // interpolateTricubic (chimesFF.cpp:2386-2389): rows per rij value, grid step
            R.size = (int)std::cbrt((double)T.rik.size());
            const long long sij = (long long)R.size * R.size;
            R.inv = 1 / (T.rjk[sij + R.size + 1] - T.rjk[0]);
            rec.push_back(R);
            cols.insert(cols.end(), T.rij.begin(), T.rij.end());
            cols.insert(cols.end(), T.rik.begin(), T.rik.end());
            cols.insert(cols.end(), T.rjk.begin(), T.rjk.end());
            for (long long k = 0; k < n; k++) {
                vals.push_back(T.e[k]);
                vals.push_back(T.fij[k]);
                vals.push_back(T.fik[k]);
                vals.push_back(T.fjk[k]);
            }
            off += n;
        }
        H.n_tab3 = (int)rec.size();
        H.t3rec = as_off<const Tab3Rec>(B.add(rec.data(), rec.size()));
        H.tab3r = as_off<const double>(B.add(cols.data(), cols.size()));
        H.tab3v = as_off<const double>(B.add(vals.data(), vals.size()));
    }
    img.header_off = B.add(&H, 1);
    img.bytes = std::move(B.b);
    return img;
}

}  // namespace ck
