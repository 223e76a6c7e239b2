// Host side of the pair-style path (see ck_neigh.cu and ck_nl.h).
#include "ck_nl.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "ck_kernels.h"

namespace ck {

#define NL_TRY(call)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call; \
            return kErrCuda;                                                          \
        }                                                                             \
    } while (0)

Status NeighCompute::compute(int slot, int nall, const double* x, const int* type, const long long* tag, int inum,
                             const int* ilist, const int* numneigh, const int* neigh, double skin, bool rebuild,
                             double* f, double* energy, double* virial, double* eatom, double* vatom,
                             std::string& err) {
    Status st = eng_.init_device(err);
    if (st != kOk) return st;
    if (slot < 0 || slot >= eng_.n_param_sets()) {
        err = "parameter set not loaded";
        return kErrState;
    }
    if (nall <= 0 || inum < 0 || inum > nall || !x || !type || !tag || (inum > 0 && (!ilist || !numneigh))) {
        err = "neighbour-list call: need nall > 0, 0 <= inum <= nall and non-null arrays";
        return kErrInput;
    }
    if (!(skin >= 0.0) || !std::isfinite(skin)) {
        err = "skin must be a finite non-negative distance";
        return kErrInput;
    }
    const HostParams& P = eng_.params(slot);
    long long nent = 0;
    for (int ii = 0; ii < inum; ii++) {
        if (ilist[ii] < 0 || ilist[ii] >= nall || numneigh[ii] < 0) {
            err = "ilist / numneigh entry out of range at position " + std::to_string(ii);
            return kErrInput;
        }
        nent += numneigh[ii];
    }
    if (nent > 0 && !neigh) {
        err = "neighbour array is null";
        return kErrInput;
    }
    for (long long e = 0; e < nent; e++)
        if (neigh[e] < 0 || neigh[e] >= nall) {
            err = "neighbour index out of range at entry " + std::to_string(e) + " (strip the LAMMPS NEIGHMASK bits)";
            return kErrInput;
        }
    double maxabs = 0.0;
    for (int a = 0; a < nall; a++) {
        for (int c = 0; c < 3; c++) maxabs = std::max(maxabs, std::fabs(x[3 * a + c]));
        if (type[a] < 0 || type[a] >= P.ntypes) {
            err = "atom type index out of range for the parameter set at atom " + std::to_string(a);
            return kErrInput;
        }
        if (!std::isfinite(x[3 * a]) || !std::isfinite(x[3 * a + 1]) || !std::isfinite(x[3 * a + 2])) {
            err = "atom coordinates must be finite";
            return kErrInput;
        }
    }
    const cudaStream_t s = eng_.stream();
    const DevParamSet& V = eng_.param_view(slot);
    ForceLaunch L = eng_.tuning;
    L.precision = eng_.precision;
    L.stride3 = P.o3 > 0 ? P.o3 + 1 : 0;
    L.stride4 = P.o4 > 0 ? P.o4 + 1 : 0;
    L.fact3 = (eng_.factored && V.R3 > 0 && L.want_fact3) ? 1 : 0;
    L.fact4 = (eng_.factored && V.R4 > 0 && L.want_fact4) ? 1 : 0;
    L.rf3 = V.R3;
    L.rf4 = V.R4;
    const int nbk3 = eng_.n_buckets(3), nbk4 = eng_.n_buckets(4);
    // the cluster buckets depend on the contraction form and on the sets loaded
    const bool build = rebuild || !built_ || nall != nall_ || inum != inum_ || nent != nent_ || slot != slot_ ||
                       skin != skin_ || L.fact3 != fact3_ || L.fact4 != fact4_ || nbk3 != nbk3_ || nbk4 != nbk4_;

    NL_TRY(d_x_.reserve(3 * (long long)nall));
    NL_TRY(d_type_.reserve(nall));
    NL_TRY(d_atom_sys_.reserve(nall));
    NL_TRY(d_atom_orig_.reserve(nall));
    NL_TRY(d_parent_.reserve(nall));
    NL_TRY(d_tag_.reserve(nall));
    NL_TRY(d_force_.reserve(3 * (long long)nall));
    NL_TRY(d_ev_.reserve(8));
    NL_TRY(d_flags_.reserve(8));
    NL_TRY(d_queue_.reserve(2));
    NL_TRY(d_minmax_.reserve(6));
    NL_TRY(d_sys_.reserve(1));
    NL_TRY(d_xf_.reserve(3 * (long long)nall));
    NL_TRY(cudaMemcpyAsync(d_x_.p, x, sizeof(double) * 3 * nall, cudaMemcpyHostToDevice, s));
    NL_TRY(cudaMemcpyAsync(d_type_.p, type, sizeof(int) * nall, cudaMemcpyHostToDevice, s));
    launch_nl_xf(d_x_.p, d_xf_.p, 3 * (long long)nall, s);
    // FP32 distances of coordinates up to maxabs are within 1e-6 * maxabs + 1e-5 of
    // the FP64 ones (several times the rounding of the coordinates and the arithmetic)
    const double feps = 1e-5 + 1e-6 * maxabs;

    if (build) {
        NL_TRY(d_ilist_.reserve(std::max(1, inum)));
        NL_TRY(d_off_.reserve(inum + 1));
        NL_TRY(d_neigh_.reserve(std::max(1LL, nent)));
        NL_TRY(d_owner_.reserve(std::max(1LL, nent)));
        NL_TRY(d_e_cnt3_.reserve(std::max(1LL, nent)));
        NL_TRY(d_e_cnt4_.reserve(std::max(1LL, nent)));
        NL_TRY(d_e_off3_.reserve(nent + 1));
        NL_TRY(d_e_off4_.reserve(nent + 1));
        NL_TRY(d_scan_tmp_.reserve(scan_tmp_bytes(std::max(1LL, nent))));
        std::vector<long long> off(inum + 1, 0);
        for (int ii = 0; ii < inum; ii++) off[ii + 1] = off[ii] + numneigh[ii];
        NL_TRY(cudaMemcpyAsync(d_tag_.p, tag, sizeof(long long) * nall, cudaMemcpyHostToDevice, s));
        if (inum > 0) NL_TRY(cudaMemcpyAsync(d_ilist_.p, ilist, sizeof(int) * inum, cudaMemcpyHostToDevice, s));
        NL_TRY(cudaMemcpyAsync(d_off_.p, off.data(), sizeof(long long) * (inum + 1), cudaMemcpyHostToDevice, s));
        if (nent > 0) NL_TRY(cudaMemcpyAsync(d_neigh_.p, neigh, sizeof(int) * nent, cudaMemcpyHostToDevice, s));
        // identity cell: the batch kernels' pair geometry becomes x_b - x_a
        SysDesc d;
        std::memset(&d, 0, sizeof(d));
        for (int k = 0; k < 9; k++) d.h[k] = d.hi[k] = d.hn[k] = d.hni[k] = d.h0[k] = d.h0i[k] = (k % 4 == 0) ? 1.0 : 0.0;
        d.pset = slot;
        d.has3 = P.o3 > 0;
        d.has4 = P.o4 > 0;
        d.n_in = d.n_atoms = nall;
        NL_TRY(cudaMemcpyAsync(d_sys_.p, &d, sizeof(d), cudaMemcpyHostToDevice, s));
    }

    BatchView& B = B_;
    B = BatchView();
    B.n_sys = 1;
    B.n_in_total = B.n_atoms_total = B.n_ghost_total = nall;
    B.sys = d_sys_.p;
    B.psets = eng_.device_params();
    B.in_pos = d_x_.p;
    B.in_type = d_type_.p;
    B.atom_sys = d_atom_sys_.p;
    B.atom_type = d_type_.p;
    B.atom_orig = d_atom_orig_.p;
    B.ghost_parent = d_parent_.p;
    B.ghost_fs = d_x_.p;
    B.minmax = d_minmax_.p;
    B.n2_cap = nent;
    B.e_cnt3 = d_e_cnt3_.p; B.e_cnt4 = d_e_cnt4_.p; B.e_off3 = d_e_off3_.p; B.e_off4 = d_e_off4_.p;
    B.force = d_force_.p; B.ev = d_ev_.p; B.flags = d_flags_.p; B.queue = d_queue_.p;
    B.enum_serial = 0;
    NeighView& N = N_;
    N.inum = inum;
    N.nent = nent;
    N.ilist = d_ilist_.p;
    N.off = d_off_.p;
    N.neigh = d_neigh_.p;
    N.owner = d_owner_.p;
    N.tag = d_tag_.p;
    // padded cutoffs of build_mb_neighlists: max_cutoff_nB (0 for an absent order) + skin
    N.c3p = (P.o3 > 0 ? P.max_cut3() : 0.0) + skin;
    N.c4p = (P.o4 > 0 ? P.max_cut4() : 0.0) + skin;
    N.has3 = P.o3 > 0;
    N.has4 = P.o4 > 0;
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
    N.xf = d_xf_.p;
    N.c3lo = down(N.c3p - feps);
    N.c3hi = up(N.c3p + feps);
    N.c4lo = down(N.c4p - feps);
    N.c4hi = up(N.c4p + feps);
    B.pos_f = d_xf_.p;
    B.float_eps = up(feps);

    if (build) {
        launch_nl_setup(B, N, s);
        long long tot[2] = {0, 0};
        if (nent > 0) {
            launch_nl_enum(B, N, false, s);
            exclusive_scan2(d_e_cnt3_.p, d_e_off3_.p, d_e_cnt4_.p, d_e_off4_.p, nent, d_scan_tmp_.p, s);
            NL_TRY(cudaMemcpyAsync(&tot[0], d_e_off3_.p + nent, sizeof(long long), cudaMemcpyDeviceToHost, s));
            NL_TRY(cudaMemcpyAsync(&tot[1], d_e_off4_.p + nent, sizeof(long long), cudaMemcpyDeviceToHost, s));
            NL_TRY(cudaStreamSynchronize(s));
        } else {
            NL_TRY(cudaMemsetAsync(d_e_off3_.p, 0, sizeof(long long), s));
            NL_TRY(cudaMemsetAsync(d_e_off4_.p, 0, sizeof(long long), s));
        }
        n3_ = tot[0];
        n4_ = tot[1];
        if (n3_ > cap3_ || !d_c3_.p) { NL_TRY(d_c3_.reserve(3 * std::max(1LL, n3_))); cap3_ = std::max(1LL, n3_); }
        if (n4_ > cap4_ || !d_c4_.p) { NL_TRY(d_c4_.reserve(4 * std::max(1LL, n4_))); cap4_ = std::max(1LL, n4_); }
        NL_TRY(d_perm3_.reserve(std::max(1LL, n3_ + 32LL * nbk3)));
        NL_TRY(d_perm4_.reserve(std::max(1LL, n4_ + 32LL * nbk4)));
        NL_TRY(d_bk_key3_.reserve(std::max(1LL, n3_)));
        NL_TRY(d_bk_key4_.reserve(std::max(1LL, n4_)));
        NL_TRY(d_bk_count_.reserve(nbk3 + nbk4 + 1));
        NL_TRY(d_bk_fill_.reserve(nbk3 + nbk4 + 1));
        NL_TRY(d_bk_start_.reserve(nbk3 + nbk4 + 2));
    }
    B.c3 = d_c3_.p; B.c4 = d_c4_.p;
    B.n3_cap = cap3_; B.n4_cap = cap4_;
    B.nbk3 = nbk3; B.nbk4 = nbk4;
    B.bk_count = d_bk_count_.p; B.bk_fill = d_bk_fill_.p; B.bk_start = d_bk_start_.p;
    // the count pass keeps each cluster's key (its cutoff test takes FP64 distances) for the scatter pass
    B.bk_key3 = d_bk_key3_.p; B.bk_key4 = d_bk_key4_.p;
    B.perm3 = d_perm3_.p; B.perm4 = d_perm4_.p;
    B.perm3_cap = nbk3 > 0 ? n3_ + 32LL * nbk3 : 0;
    B.perm4_cap = nbk4 > 0 ? n4_ + 32LL * nbk4 : 0;
    if (build) {
        if (nent > 0) launch_nl_enum(B, N, true, s);
        built_ = true;
        slot_ = slot;
        nall_ = nall;
        inum_ = inum;
        nent_ = nent;
        skin_ = skin;
        fact3_ = L.fact3;
        fact4_ = L.fact4;
        nbk3_ = nbk3;
        nbk4_ = nbk4;
    }

    // evaluation with the current positions
    if (eatom) {
        NL_TRY(d_eatom_.reserve(nall));
        NL_TRY(cudaMemsetAsync(d_eatom_.p, 0, sizeof(double) * nall, s));
        B.eatom = d_eatom_.p;
    }
    if (vatom) {
        NL_TRY(d_vatom_.reserve(6 * (long long)nall));
        NL_TRY(cudaMemsetAsync(d_vatom_.p, 0, sizeof(double) * 6 * nall, s));
        B.vatom = d_vatom_.p;
    }
    launch_reset(B, s);
    // The lists hold every cluster within the padded cutoffs; the factored
    // kernels get only those within their tuple's cutoffs at the current
    // positions (rebucketed every call, as atoms move between rebuilds).
    B.bucket_cut = 1;
    // a tabulated 3-body term is looked up per listed triplet (no buckets)
    const bool tab3 = P.tab3 && L.stride3 > 0;
    const bool bk3 = L.stride3 > 0 && L.fact3 && n3_ > 0 && !tab3;
    if (bk3 || (L.stride4 > 0 && L.fact4 && n4_ > 0)) {
        NL_TRY(cudaMemsetAsync(B.bk_count, 0, sizeof(int) * (nbk3 + nbk4), s));
        NL_TRY(cudaMemsetAsync(B.bk_fill, 0, sizeof(int) * (nbk3 + nbk4), s));
        if (bk3) launch_bucket(B, 3, s);
        if (L.stride4 > 0 && L.fact4 && n4_ > 0) launch_bucket(B, 4, s);
    }
    launch_nl_pairs(B, N, L.precision, s);
    if (L.stride3 > 0 && n3_ > 0) {
        if (tab3) {
            NL_TRY(d_tsel_.reserve(n3_));
            NL_TRY(d_tselr_.reserve(3 * n3_));
            NL_TRY(d_tcount_.reserve(1));
            launch_nl_tab3(B, n3_, d_tsel_.p, d_tselr_.p, d_tcount_.p, s);
        }
        else if (L.fact3) launch_force3f(B, L, s);
        else launch_force3(B, L, s);
    }
    if (L.stride4 > 0 && n4_ > 0) {
        if (L.fact4) launch_force4f(B, L, s);
        else launch_force4(B, L, s);
    }
    NL_TRY(cudaGetLastError());
    h_force_.resize(3 * (size_t)nall);
    double ev[8];
    int flags[8];
    NL_TRY(cudaMemcpyAsync(h_force_.data(), d_force_.p, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, s));
    NL_TRY(cudaMemcpyAsync(ev, d_ev_.p, sizeof(double) * 8, cudaMemcpyDeviceToHost, s));
    NL_TRY(cudaMemcpyAsync(flags, d_flags_.p, sizeof(int) * 8, cudaMemcpyDeviceToHost, s));
    if (eatom) {
        h_eatom_.resize(nall);
        NL_TRY(cudaMemcpyAsync(h_eatom_.data(), d_eatom_.p, sizeof(double) * nall, cudaMemcpyDeviceToHost, s));
    }
    if (vatom) {
        h_vatom_.resize(6 * (size_t)nall);
        NL_TRY(cudaMemcpyAsync(h_vatom_.data(), d_vatom_.p, sizeof(double) * 6 * nall, cudaMemcpyDeviceToHost, s));
    }
    NL_TRY(cudaStreamSynchronize(s));
    badness_ = flags[2];
    if (flags[5] & 1) {   // get_tab_2B prints and exits here
        err = "Distance is outside the tabulated range (a 2-body distance at or below the table's first usable "
              "grid point)";
        return kErrGeometry;
    }
    if (flags[5] & 2) {
        err = "a 3-body distance lies past the tabulated grid (the table does not cover the 3-body cutoffs)";
        return kErrGeometry;
    }
    for (size_t k = 0; k < h_force_.size(); k++) f[k] += h_force_[k];
    if (eatom)
        for (int a = 0; a < nall; a++) eatom[a] += h_eatom_[a];
    if (vatom)
        for (size_t k = 0; k < h_vatom_.size(); k++) vatom[k] += h_vatom_[k];
    if (energy) *energy += ev[0];
    if (virial) {   // Pair::ev_tally_mb order: xx yy zz xy xz yz
        virial[0] += ev[1];
        virial[1] += ev[4];
        virial[2] += ev[6];
        virial[3] += ev[2];
        virial[4] += ev[3];
        virial[5] += ev[5];
    }
    return kOk;
}

Status NeighCompute::lists(std::vector<int>& l3, std::vector<int>& l4, std::string& err) {
    l3.assign(3 * (size_t)n3_, 0);
    l4.assign(4 * (size_t)n4_, 0);
    if (n3_) NL_TRY(cudaMemcpy(l3.data(), d_c3_.p, sizeof(int) * l3.size(), cudaMemcpyDeviceToHost));
    if (n4_) NL_TRY(cudaMemcpy(l4.data(), d_c4_.p, sizeof(int) * l4.size(), cudaMemcpyDeviceToHost));
    return kOk;
}

Status NeighCompute::fp_records(int nbody, std::vector<double>& d, std::vector<int>& t, std::string& err) {
    d.clear();
    t.clear();
    if (!built_) {
        err = "no neighbour-list evaluation yet";
        return kErrState;
    }
    if (nbody < 2 || nbody > 4) {
        err = "fingerprint records exist for 2-, 3- and 4-body clusters";
        return kErrInput;
    }
    const HostParams& P = eng_.params(slot_);
    if ((nbody == 3 && P.o3 <= 0) || (nbody == 4 && P.o4 <= 0)) {
        err = "the parameter set has no " + std::to_string(nbody) + "-body terms";
        return kErrInput;
    }
    const long long n = nbody == 2 ? nent_ : (nbody == 3 ? n3_ : n4_);
    if (n <= 0) return kOk;
    const int np = nbody * (nbody - 1) / 2;
    const cudaStream_t s = eng_.stream();
    NL_TRY(d_fp_flag_.reserve(n));
    NL_TRY(d_fp_off_.reserve(n + 1));
    NL_TRY(d_fp_tmp_.reserve(scan_tmp_bytes(n)));
    launch_nl_fp(B_, N_, nbody, n, false, d_fp_flag_.p, nullptr, nullptr, nullptr, s);
    exclusive_scan(d_fp_flag_.p, d_fp_off_.p, n, d_fp_tmp_.p, s);
    long long total = 0;
    NL_TRY(cudaMemcpyAsync(&total, d_fp_off_.p + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
    NL_TRY(cudaStreamSynchronize(s));
    if (total <= 0) return kOk;
    NL_TRY(d_fp_d_.reserve(total * np));
    NL_TRY(d_fp_t_.reserve(total * nbody));
    launch_nl_fp(B_, N_, nbody, n, true, d_fp_flag_.p, d_fp_off_.p, d_fp_d_.p, d_fp_t_.p, s);
    NL_TRY(cudaGetLastError());
    d.resize((size_t)total * np);
    t.resize((size_t)total * nbody);
    NL_TRY(cudaMemcpyAsync(d.data(), d_fp_d_.p, sizeof(double) * d.size(), cudaMemcpyDeviceToHost, s));
    NL_TRY(cudaMemcpyAsync(t.data(), d_fp_t_.p, sizeof(int) * t.size(), cudaMemcpyDeviceToHost, s));
    NL_TRY(cudaStreamSynchronize(s));
    return kOk;
}

}  // namespace ck
