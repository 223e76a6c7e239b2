// Parameter sets: parsing of the ChIMES text format and packing into the
// device-resident tables the kernels read.
#pragma once
#include <string>
#include <vector>

#include "ck_common.h"

namespace ck {

// A parsed parameter file: the tables chimesFF builds in read_parameters
// (chimesFF/src/chimesFF.cpp:354-1570) and build_pair_int_{trip,quad}_map
// (chimesFF.cpp:2958-3080).
struct HostParams {
    int ntypes = 0, npairs = 0;
    int o2 = 0, o3 = 0, o4 = 0;
    std::vector<std::string> atm;       // atmtyps
    std::vector<double> mass;
    std::vector<std::string> pa1, pa2;  // pair_params_atm_chem_1/2
    std::vector<double> rin, rout, lam; // chimes_2b_cutoff[.][0/1], morse_var
    bool tersoff = false;
    double fcut_var = 0.0;
    double pen_dist = 0.01, pen_scale = 1.0e4, inner_smooth = 0.01;  // chimesFF.cpp:104-116
    std::vector<double> eoff;           // energy_offsets
    std::vector<std::vector<int>> pows2;
    std::vector<std::vector<double>> coef2;
    std::vector<int> pair_map;          // atom_int_pair_map [nt*nt]
    std::vector<int> prpr;              // proper pair index [nt*nt] (atom_int_prpr_map)
    std::vector<int> pair_map_file_idx; // PAIRMAPS indices in file order (atom_idx_pair_map)

    struct Body {
        int nbody = 0, npair = 0, ntyp = 0;
        std::vector<int> ncoef;                     // ncoeffs_{3,4}b
        std::vector<std::vector<int>> pows;         // [type][c*npair + p]
        std::vector<std::vector<double>> coef;      // [type][c]
        std::vector<std::vector<double>> cut_in, cut_out;  // [type][p] in parameter pair order
        std::vector<std::vector<std::string>> atoms, pairs;
        std::vector<int> map;                       // atom_int_{trip,quad}_map [nt^nbody]
        std::vector<std::vector<int>> perm;         // pair_int_{trip,quad}_map [nt^nbody][npair]
    };
    Body b3, b4;

    // Tabulated 2-/3-body terms (a PAIRTYPE PARAMS line with a table name, or
    // an INDEX line of a triplet with one: chimesFF.cpp:719-769, 882-934):
    // the tables in the order the file names them; the 2-body ones are looked
    // up by pair type index, the 3-body ones by triplet type index.
    struct Tab2 { std::vector<double> r, e, f; };
    struct Tab3 { std::vector<double> rij, rik, rjk, e, fij, fik, fjk; };
    bool tab2 = false, tab3 = false;
    std::vector<Tab2> t2tab;
    std::vector<Tab3> t3tab;

    double max_cut2() const;
    double max_cut3() const;
    double max_cut4() const;
    int type_index(const std::string& name) const;
    std::string pair_name(int p) const { return pa1[p] + pa2[p]; }
};

// Reads a ChIMES parameter file, or a binary parameter cache written by
// save_parameter_cache (recognised by its magic bytes).
Status parse_parameter_file(const std::string& path, HostParams& P, std::string& err);
Status save_parameter_cache(const HostParams& P, const std::string& path, std::string& err);

// Contiguous host image of one DevParamSet: the struct followed by its arrays.
// Pointers inside `header` are offsets until relocated to a device base.
struct ParamImage {
    std::vector<unsigned char> bytes;
    DevParamSet header{};
    size_t header_off = 0;
};
ParamImage pack_params(const HostParams& P);

}  // namespace ck
