// Pair-style evaluation on a caller's neighbour list (LAMMPS layout): the
// host side of ck_neigh.cu, sharing an Engine's parameter sets, stream,
// precision and launch tuning.
#pragma once
#include <string>
#include <vector>

#include "ck_engine.h"

namespace ck {

class NeighCompute {
public:
    explicit NeighCompute(Engine& eng) : eng_(eng) {}

    // x[nall][3], type[nall] (type indices of the slot's set), tag[nall];
    // ilist[inum]; numneigh[inum] and neigh[] concatenated in ilist order.
    // rebuild = 1 builds the 3-/4-body cluster lists from this neighbour
    // list (also done on the first call and whenever nall, inum or the entry
    // count change); 0 reuses them with the new positions.  Accumulates
    // f[nall][3], *energy and virial[6] (xx yy zz xy xz yz).
    // eatom[nall] / vatom[nall][6] (may be null): per-atom energy and virial,
    // each interaction shared equally by its atoms, accumulated.
    Status compute(int slot, int nall, const double* x, const int* type, const long long* tag, int inum,
                   const int* ilist, const int* numneigh, const int* neigh, double skin, bool rebuild, double* f,
                   double* energy, double* virial, double* eatom, double* vatom, std::string& err);

    long long n3() const { return n3_; }
    // worst 2-body penalty region entered by the last call (chimesFF badness: 0, 1, 2)
    int badness() const { return badness_; }
    long long n4() const { return n4_; }
    // cluster lists of the last build (atom indices), for checks
    Status lists(std::vector<int>& l3, std::vector<int>& l4, std::string& err);
    // Fingerprint records of the last compute (FINGERPRINT build of the pair
    // style): the clusters of body order nbody that compute_nB evaluates and
    // whose atoms are in recording order (2-body i < j, 3-/4-body strictly
    // increasing tags), as distances d[n][P] and type indices t[n][nbody], in
    // the pair style's loop order.
    Status fp_records(int nbody, std::vector<double>& d, std::vector<int>& t, std::string& err);

private:
    Engine& eng_;
    int slot_ = -1, nall_ = -1, inum_ = -1, badness_ = 0;
    long long nent_ = -1, n3_ = 0, n4_ = 0, cap3_ = 0, cap4_ = 0;
    double skin_ = -1.0;
    bool built_ = false;
    int fact3_ = -1, fact4_ = -1, nbk3_ = -1, nbk4_ = -1;   // state the clusters were bucketed for
    BatchView B_{};
    NeighView N_{};
    DevBuf<SysDesc> d_sys_;
    DevBuf<double> d_x_, d_force_, d_ev_, d_eatom_, d_vatom_;
    DevBuf<int> d_type_, d_atom_sys_, d_atom_orig_, d_parent_, d_ilist_, d_neigh_, d_owner_;
    DevBuf<long long> d_tag_, d_off_;
    DevBuf<int> d_e_cnt3_, d_e_cnt4_, d_c3_, d_c4_;
    DevBuf<long long> d_e_off3_, d_e_off4_;
    DevBuf<int> d_flags_, d_bk_count_, d_bk_fill_, d_perm3_, d_perm4_, d_bk_key3_, d_bk_key4_;
    DevBuf<long long> d_bk_start_;
    DevBuf<unsigned long long> d_queue_, d_minmax_;
    DevBuf<unsigned char> d_scan_tmp_, d_fp_tmp_;
    DevBuf<int> d_fp_flag_, d_fp_t_;
    DevBuf<long long> d_fp_off_;
    DevBuf<double> d_fp_d_, d_tselr_;
    DevBuf<float> d_xf_;
    DevBuf<int> d_tsel_;
    DevBuf<unsigned long long> d_tcount_;
    std::vector<double> h_force_, h_eatom_, h_vatom_;
};

}  // namespace ck
