// The reference's C++ classes (chimesFF, serial_chimes_interface) and its
// per-cluster C interface (chimesFF/api/chimescalc_C.h), implemented on the
// GPU engine.  Declarations: include/chimesFF.h, include/serial_chimes_interface.h,
// include/chimescalc_C.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "ck_engine.h"
#include "chimesFF.h"
#include "serial_chimes_interface.h"

struct chimesFF::Impl {
    ck::Engine eng;
    int slot = -1;
    int badness = 0;
    Impl() { eng.use_graph = true; }   // repeated calculate() calls replay one CUDA graph
};

namespace {

void die(const std::string& msg) { ck::report_error(ck::kErrInput, msg); }

const ck::HostParams* params_of(chimesFF::Impl* im) {
    if (im->slot < 0) {
        ck::report_error(ck::kErrState, "chimesFF: parameters have not been read");
        return nullptr;
    }
    return &im->eng.params(im->slot);
}

// One cluster through the per-cluster kernel; adds into the caller's buffers.
bool one_cluster(chimesFF::Impl* im, int nbody, const double* dx, const double* dr, const int* typ, double* force,
                 double* stress, double& energy, double* fscal_out, bool tab = false) {
    const int np = nbody * (nbody - 1) / 2;
    double f[12], s[6], e, fs[6];
    int status = 0;
    std::string err;
    ck::Status st = im->eng.compute_clusters(im->slot, nbody, 1, dx, dr, typ, f, s, &e, fs, &status, err, tab);
    if (st != ck::kOk) {
        ck::report_error(st, err);
        return false;
    }
    if (!(status & 1)) return true;   // excluded type or beyond a cutoff: nothing added
    if (status & 16) {   // get_tab_2B prints this and exits; a 3-body grid index past the table
        ck::report_error(ck::kErrGeometry, nbody == 2 ? "Distance is outside the tabulated range"
                                                      : "3-body distance past the tabulated grid");
        return false;
    }
    for (int k = 0; k < 3 * nbody; k++) force[k] += f[k];
    for (int k = 0; k < 6; k++) stress[k] += s[k];
    energy += e;
    if (status & 4) im->badness = 2;
    else if ((status & 2) && im->badness < 1) im->badness = 1;
    if (fscal_out)
        for (int p = 0; p < np; p++) fscal_out[p] = fs[p];
    return true;
}

}  // namespace

// ---------------------------------------------------------------------------
// chimesFF
// ---------------------------------------------------------------------------
chimesFF::chimesFF() : rank(0), natmtyps(0), tabulate_2B(false), tabulate_3B(false), impl_(new Impl()) {}
chimesFF::~chimesFF() { delete impl_; }

void chimesFF::init(int mpi_rank) { rank = mpi_rank; }

void chimesFF::read_parameters(std::string paramfile) {
    std::string err;
    int slot = impl_->eng.load_params(paramfile, err);
    if (slot < 0) {
        ck::report_error(slot, "chimesFF: " + err);
        return;
    }
    impl_->slot = slot;
    const ck::HostParams& P = impl_->eng.params(slot);
    natmtyps = P.ntypes;
    poly_orders = {P.o2, P.o3, P.o4};
    atmtyps = P.atm;
    masses = P.mass;
    tabulate_2B = P.tab2;
    tabulate_3B = P.tab3;
}

void chimesFF::compute_1B(const int typ_idx, double& energy) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return;
    if (typ_idx < 0 || typ_idx >= P->ntypes) return die("compute_1B: atom type index out of range");
    energy += P->eoff[typ_idx];
}

void chimesFF::compute_2B(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                          std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp& tmp) {
    double fs = 0.0;
    compute_2B(dx, dr, typ_idxs, force, stress, energy, tmp, fs);
}

void chimesFF::compute_2B(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                          std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp&,
                          double& force_scalar_in) {
    if (!params_of(impl_)) return;
    if (dr.size() < 3 || typ_idxs.size() < 2 || force.size() < 6 || stress.size() < 6)
        return die("compute_2B: dr needs 3, typ_idxs 2, force 6 and stress 6 entries");
    one_cluster(impl_, 2, &dx, dr.data(), typ_idxs.data(), force.data(), stress.data(), energy, &force_scalar_in);
}

void chimesFF::compute_3B(const std::vector<double>& dx, const std::vector<double>& dr,
                          const std::vector<int>& typ_idxs, std::vector<double>& force, std::vector<double>& stress,
                          double& energy, chimes3BTmp& tmp) {
    std::vector<double> fs(3);
    compute_3B(dx, dr, typ_idxs, force, stress, energy, tmp, fs);
}

void chimesFF::compute_3B(const std::vector<double>& dx, const std::vector<double>& dr,
                          const std::vector<int>& typ_idxs, std::vector<double>& force, std::vector<double>& stress,
                          double& energy, chimes3BTmp&, std::vector<double>& force_scalar_in) {
    if (!params_of(impl_)) return;
    if (dx.size() < 3 || dr.size() < 9 || typ_idxs.size() < 3 || force.size() < 9 || stress.size() < 6)
        return die("compute_3B: dx needs 3, dr 9, typ_idxs 3, force 9 and stress 6 entries");
    if (force_scalar_in.size() < 3) force_scalar_in.resize(3);
    one_cluster(impl_, 3, dx.data(), dr.data(), typ_idxs.data(), force.data(), stress.data(), energy,
                force_scalar_in.data());
}

void chimesFF::compute_2B_tab(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                              std::vector<double>& force, std::vector<double>& stress, double& energy,
                              chimes2BTmp& tmp) {
    double fs = 0.0;
    compute_2B_tab(dx, dr, typ_idxs, force, stress, energy, tmp, fs);
}

void chimesFF::compute_2B_tab(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                              std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp&,
                              double& force_scalar_in) {
    if (!params_of(impl_)) return;
    if (dr.size() < 3 || typ_idxs.size() < 2 || force.size() < 6 || stress.size() < 6)
        return die("compute_2B_tab: dr needs 3, typ_idxs 2, force 6 and stress 6 entries");
    one_cluster(impl_, 2, &dx, dr.data(), typ_idxs.data(), force.data(), stress.data(), energy, &force_scalar_in,
                true);
}

void chimesFF::compute_3B_tab(const std::vector<double>& dx, const std::vector<double>& dr,
                              const std::vector<int>& typ_idxs, std::vector<double>& force,
                              std::vector<double>& stress, double& energy, chimes3BTmp& tmp) {
    std::vector<double> fs(3);
    compute_3B_tab(dx, dr, typ_idxs, force, stress, energy, tmp, fs);
}

void chimesFF::compute_3B_tab(const std::vector<double>& dx, const std::vector<double>& dr,
                              const std::vector<int>& typ_idxs, std::vector<double>& force,
                              std::vector<double>& stress, double& energy, chimes3BTmp&,
                              std::vector<double>& force_scalar_in) {
    if (!params_of(impl_)) return;
    if (dx.size() < 3 || dr.size() < 9 || typ_idxs.size() < 3 || force.size() < 9 || stress.size() < 6)
        return die("compute_3B_tab: dx needs 3, dr 9, typ_idxs 3, force 9 and stress 6 entries");
    if (force_scalar_in.size() < 3) force_scalar_in.resize(3);
    one_cluster(impl_, 3, dx.data(), dr.data(), typ_idxs.data(), force.data(), stress.data(), energy,
                force_scalar_in.data(), true);
}

void chimesFF::compute_4B(const std::vector<double>& dx, const std::vector<double>& dr,
                          const std::vector<int>& typ_idxs, std::vector<double>& force, std::vector<double>& stress,
                          double& energy, chimes4BTmp& tmp) {
    std::vector<double> fs(6);
    compute_4B(dx, dr, typ_idxs, force, stress, energy, tmp, fs);
}

void chimesFF::compute_4B(const std::vector<double>& dx, const std::vector<double>& dr,
                          const std::vector<int>& typ_idxs, std::vector<double>& force, std::vector<double>& stress,
                          double& energy, chimes4BTmp&, std::vector<double>& force_scalar_in) {
    if (!params_of(impl_)) return;
    if (dx.size() < 6 || dr.size() < 18 || typ_idxs.size() < 4 || force.size() < 12 || stress.size() < 6)
        return die("compute_4B: dx needs 6, dr 18, typ_idxs 4, force 12 and stress 6 entries");
    if (force_scalar_in.size() < 6) force_scalar_in.resize(6);
    one_cluster(impl_, 4, dx.data(), dr.data(), typ_idxs.data(), force.data(), stress.data(), energy,
                force_scalar_in.data());
}

void chimesFF::compute_clusters(int nbody, int n, const double* dx, const double* dr, const int* typ, double* force,
                                double* stress, double& energy) {
    if (!params_of(impl_) || n <= 0) return;
    const int np = nbody * (nbody - 1) / 2;
    std::vector<double> f((size_t)n * 3 * nbody), s((size_t)n * 6), e(n), fs((size_t)n * np);
    std::vector<int> status(n);
    std::string err;
    ck::Status st = impl_->eng.compute_clusters(impl_->slot, nbody, n, dx, dr, typ, f.data(), s.data(), e.data(),
                                                fs.data(), status.data(), err);
    if (st != ck::kOk) {
        ck::report_error(st, err);
        return;
    }
    for (int c = 0; c < n; c++) {
        if (!(status[c] & 1)) continue;
        for (int k = 0; k < 3 * nbody; k++) force[(size_t)c * 3 * nbody + k] += f[(size_t)c * 3 * nbody + k];
        for (int k = 0; k < 6; k++) stress[k] += s[(size_t)c * 6 + k];
        energy += e[c];
        if (status[c] & 4) impl_->badness = 2;
        else if ((status[c] & 2) && impl_->badness < 1) impl_->badness = 1;
    }
}

void chimesFF::get_cutoff_2B(std::vector<std::vector<double> >& cutoff_2b) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return;
    cutoff_2b.assign(P->npairs, std::vector<double>(2));
    for (int i = 0; i < P->npairs; i++) { cutoff_2b[i][0] = P->rin[i]; cutoff_2b[i][1] = P->rout[i]; }
}

double chimesFF::max_cutoff_2B(bool silent) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return 0.0;
    double m = P->max_cut2();
    if (rank == 0 && !silent) std::cout << "chimesFF: \tSetting 2-body max cutoff to: " << m << std::endl;
    return m;
}
double chimesFF::max_cutoff_3B(bool silent) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return 0.0;
    double m = P->max_cut3();
    if (P->o3 > 0 && rank == 0 && !silent) std::cout << "chimesFF: \tSetting 3-body max cutoff to: " << m << std::endl;
    return m;
}
double chimesFF::max_cutoff_4B(bool silent) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return 0.0;
    double m = P->max_cut4();
    if (P->o4 > 0 && rank == 0 && !silent) std::cout << "chimesFF: \tSetting 4-body max cutoff to: " << m << std::endl;
    return m;
}

void chimesFF::set_atomtypes(std::vector<std::string>& type_list) { type_list = atmtyps; }

int chimesFF::get_atom_pair_index(int pair_id) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return -1;
    if (pair_id < 0 || pair_id >= (int)P->pair_map_file_idx.size()) {
        die("get_atom_pair_index: index out of range");
        return -1;
    }
    return P->pair_map_file_idx[pair_id];
}

// The pair permutation maps are built when the parameters are read; these
// calls are kept for source compatibility.
void chimesFF::build_pair_int_trip_map() {}
void chimesFF::build_pair_int_quad_map() {}

int chimesFF::get_badness() { return impl_->badness; }
void chimesFF::reset_badness() { impl_->badness = 0; }

// ---------------------------------------------------------------------------
// serial_chimes_interface
// ---------------------------------------------------------------------------
serial_chimes_interface::serial_chimes_interface(bool small) : allow_replication(small) {}
serial_chimes_interface::~serial_chimes_interface() {}

void serial_chimes_interface::init_chimesFF(std::string paramfile, int rank_in) {
    init(rank_in);
    read_parameters(paramfile);
}

void serial_chimes_interface::calculate(std::vector<double>& x_in, std::vector<double>& y_in,
                                        std::vector<double>& z_in, std::vector<double>& cella_in,
                                        std::vector<double>& cellb_in, std::vector<double>& cellc_in,
                                        std::vector<std::string>& atmtyps_in, double& energy,
                                        std::vector<std::vector<double> >& force, std::vector<double>& stress) {
    const ck::HostParams* P = params_of(impl_);
    if (!P) return;
    const int n = (int)x_in.size();
    if ((int)y_in.size() != n) return die("x and y coordinate vector lengths do not match!");
    if ((int)z_in.size() != n) return die("x and z coordinate vector lengths do not match!");
    if ((int)atmtyps_in.size() < n || (int)force.size() < n || stress.size() < 9 || cella_in.size() < 3 ||
        cellb_in.size() < 3 || cellc_in.size() < 3)
        return die("calculate: atom types, forces (n x 3), stress (9) and cell vectors (3) must be sized");
    atmtyps_in.erase(atmtyps_in.begin() + n, atmtyps_in.end());
    std::vector<int> types(n);
    for (int i = 0; i < n; i++) {
        types[i] = P->type_index(atmtyps_in[i]);
        if (types[i] < 0) return die("Couldn't assign an atom type index for (index/type) " + std::to_string(i) + " " +
                                     atmtyps_in[i]);
    }
    std::vector<double> pos(3 * (size_t)n), f(3 * (size_t)n);
    for (int i = 0; i < n; i++) { pos[3 * i] = x_in[i]; pos[3 * i + 1] = y_in[i]; pos[3 * i + 2] = z_in[i]; }
    ck::SystemSpec s;
    s.n = n;
    s.pos = pos.data();
    s.types = types.data();
    for (int k = 0; k < 3; k++) { s.cell[k] = cella_in[k]; s.cell[3 + k] = cellb_in[k]; s.cell[6 + k] = cellc_in[k]; }
    s.small = allow_replication;
    s.pset = impl_->slot;
    std::vector<ck::SystemResult> res;
    std::string err;
    ck::Status st = impl_->eng.run({s}, f.data(), res, err);
    if (st != ck::kOk) {
        ck::report_error(st, err);
        return;
    }
    const ck::SystemResult& r = res[0];
    // replicas' types are appended to the caller's list (serial_chimes_interface.cpp:187,257)
    const int nrep = (r.n_rep + 1) * (r.n_rep + 1) * (r.n_rep + 1);
    for (int b = 1; b < nrep; b++)
        for (int a = 0; a < n; a++) atmtyps_in.push_back(atmtyps_in[a]);
    energy = energy / std::pow(r.n_rep + 1.0, 3.0) + r.energy;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) force[i][k] += f[3 * i + k];
    const double* v = r.virial;
    const double full[9] = {v[0], v[1], v[2], v[1], v[3], v[4], v[2], v[4], v[5]};
    for (int k = 0; k < 9; k++) stress[k] = full[k] / r.vol;
    impl_->badness = std::max(impl_->badness, impl_->eng.last.badness);
}

// ---------------------------------------------------------------------------
// Per-cluster C interface (chimesFF/api/chimescalc_C.h:11-28)
// ---------------------------------------------------------------------------
namespace {
chimesFF* g_ff = nullptr;   // chimes_ptr of chimescalc_C.cpp:23

chimesFF* ff() {
    if (!g_ff) ck::report_error(ck::kErrState, "set_chimes() must be called first");
    return g_ff;
}

bool type_idx(chimesFF* F, char* names[], int n, int* out) {
    for (int i = 0; i < n; i++) {
        auto it = std::find(F->atmtyps.begin(), F->atmtyps.end(), std::string(names[i]));
        if (it == F->atmtyps.end()) {
            ck::report_error(ck::kErrInput, std::string("input atom type not in parameter file: ") + names[i]);
            return false;
        }
        out[i] = (int)(it - F->atmtyps.begin());
    }
    return true;
}
}  // namespace

extern "C" {

double get_chimes_max_2b_cutoff() { return ff() ? g_ff->max_cutoff_2B() : 0.0; }
double get_chimes_max_3b_cutoff() { return ff() ? g_ff->max_cutoff_3B() : 0.0; }
double get_chimes_max_4b_cutoff() { return ff() ? g_ff->max_cutoff_4B() : 0.0; }
int get_chimes_2b_order() { return ff() && !g_ff->poly_orders.empty() ? g_ff->poly_orders[0] : 0; }
int get_chimes_3b_order() { return ff() && g_ff->poly_orders.size() > 1 ? g_ff->poly_orders[1] : 0; }
int get_chimes_4b_order() { return ff() && g_ff->poly_orders.size() > 2 ? g_ff->poly_orders[2] : 0; }

void set_chimes() {
    static chimesFF instance;
    g_ff = &instance;
}

void init_chimes(int rank) {
    if (ff()) g_ff->init(rank);
}

void chimes_read_params(char* param_file) {
    if (ff()) g_ff->read_parameters(param_file ? param_file : "");
}

void chimes_build_pair_int_trip_map() {}
void chimes_build_pair_int_quad_map() {}

void chimes_compute_2b_props(double rij, double dr[3], char* atype2b[2], double force[2][3], double stress[9],
                             double* epot) {
    chimesFF* F = ff();
    if (!F) return;
    int t[2];
    if (!type_idx(F, atype2b, 2, t)) return;
    std::vector<double> drv(dr, dr + 3), fv(6, 0.0), sv(9, 0.0);
    chimes2BTmp tmp(0);
    F->compute_2B(rij, drv, std::vector<int>(t, t + 2), fv, sv, *epot, tmp);
    for (int a = 0; a < 2; a++)
        for (int k = 0; k < 3; k++) force[a][k] += fv[3 * a + k];
    for (int k = 0; k < 9; k++) stress[k] += sv[k];
}

void chimes_compute_3b_props(double dr_3b[3], double dist_3b[3][3], char* atype3b[3], double f3b[3][3],
                             double stress[9], double* epot) {
    chimesFF* F = ff();
    if (!F) return;
    int t[3];
    if (!type_idx(F, atype3b, 3, t)) return;
    std::vector<double> dx(dr_3b, dr_3b + 3), drv(9), fv(9, 0.0), sv(9, 0.0);
    for (int p = 0; p < 3; p++)
        for (int k = 0; k < 3; k++) drv[3 * p + k] = dist_3b[p][k];
    chimes3BTmp tmp(0);
    F->compute_3B(dx, drv, std::vector<int>(t, t + 3), fv, sv, *epot, tmp);
    for (int a = 0; a < 3; a++)
        for (int k = 0; k < 3; k++) f3b[a][k] += fv[3 * a + k];
    for (int k = 0; k < 9; k++) stress[k] += sv[k];
}

void chimes_compute_4b_props(double dr_4b[6], double dist_4b[6][3], char* atype4b[4], double f4b[4][3],
                             double stress[9], double* epot) {
    chimesFF* F = ff();
    if (!F) return;
    int t[4];
    if (!type_idx(F, atype4b, 4, t)) return;
    std::vector<double> dx(dr_4b, dr_4b + 6), drv(18), fv(12, 0.0), sv(stress, stress + 9);
    for (int p = 0; p < 6; p++)
        for (int k = 0; k < 3; k++) drv[3 * p + k] = dist_4b[p][k];
    chimes4BTmp tmp(0);
    F->compute_4B(dx, drv, std::vector<int>(t, t + 4), fv, sv, *epot, tmp);
    for (int a = 0; a < 4; a++)
        for (int k = 0; k < 3; k++) f4b[a][k] += fv[3 * a + k];
    for (int k = 0; k < 9; k++) stress[k] = sv[k];   // the reference assigns the accumulated copy back
}

void chimes_compute_2b_props_fromf90(double* rij, double dr[3], char* type1, char* type2, double force[2][3],
                                     double stress[9], double* epot) {
    char* t[2] = {type1, type2};
    chimes_compute_2b_props(*rij, dr, t, force, stress, epot);
}

void chimes_compute_3b_props_fromf90(double dr_3b[3], double dist_3b[3][3], char* type1, char* type2, char* type3,
                                     double f3b[3][3], double stress[9], double* epot) {
    char* t[3] = {type1, type2, type3};
    chimes_compute_3b_props(dr_3b, dist_3b, t, f3b, stress, epot);
}

void chimes_compute_4b_props_fromf90(double dr_4b[6], double dist_4b[6][3], char* type1, char* type2, char* type3,
                                     char* type4, double f4b[4][3], double stress[9], double* epot) {
    char* t[4] = {type1, type2, type3, type4};
    chimes_compute_4b_props(dr_4b, dist_4b, t, f4b, stress, epot);
}

}  // extern "C"
