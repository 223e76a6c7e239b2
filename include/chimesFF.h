/*
 * chimesFF -- source-compatible C++ class of the GB300 ChIMES library.
 *
 * Same class, public members and method signatures as the reference's
 * chimesFF (chimesFF/src/chimesFF.h:125-227), so code written against the
 * reference compiles against this header and links against libchimescalc.so.
 * Every compute_nB call runs on the GPU (per-cluster kernels); the *_batch
 * methods evaluate many clusters in one launch for callers that own the
 * cluster loop (the LAMMPS pattern).
 *
 * Semantics kept from the reference:
 *   - force, stress and energy are accumulated into the caller's buffers;
 *   - dr holds atom2 - atom1 for each pair, pairs ordered ij / ij,ik,jk /
 *     ij,ik,il,jk,jl,kl; force is packed [atom][xyz]; stress is packed
 *     xx,xy,xz,yy,yz,zz;
 *   - force_scalar_in receives the reference's force_scalar values (see
 *     chimesFF.cpp:1771-1774, 2171-2173, 2866-2871);
 *   - errors print a message on stdout and call exit(0), like the reference.
 */
#ifndef CHIMES_GB300_CHIMESFF_H
#define CHIMES_GB300_CHIMESFF_H

#include <string>
#include <vector>

#ifndef CHDIM
#define CHDIM 3
#endif

/* Scratch objects of the reference API (chimesFF.h:37-117).  The GPU kernels
 * keep their Chebyshev tables on chip, so these only carry the polynomial
 * vectors for source compatibility. */
class chimes2BTmp {
public:
    explicit chimes2BTmp(int poly_order) : Tn(poly_order + 1), Tnd(poly_order + 1) {}
    void resize(int poly_order) {
        if ((int)Tn.size() < poly_order + 1) Tn.resize(poly_order + 1);
        if ((int)Tnd.size() < poly_order + 1) Tnd.resize(poly_order + 1);
    }
    std::vector<double> Tn, Tnd;
};

class chimes3BTmp {
public:
    explicit chimes3BTmp(int poly_order)
        : Tn_ij(poly_order + 1), Tn_ik(poly_order + 1), Tn_jk(poly_order + 1),
          Tnd_ij(poly_order + 1), Tnd_ik(poly_order + 1), Tnd_jk(poly_order + 1) {}
    void resize(int poly_order) {
        for (auto* v : {&Tn_ij, &Tn_ik, &Tn_jk, &Tnd_ij, &Tnd_ik, &Tnd_jk})
            if ((int)v->size() < poly_order + 1) v->resize(poly_order + 1);
    }
    std::vector<double> Tn_ij, Tn_ik, Tn_jk;
    std::vector<double> Tnd_ij, Tnd_ik, Tnd_jk;
};

class chimes4BTmp {
public:
    explicit chimes4BTmp(int poly_order)
        : Tn_ij(poly_order + 1), Tn_ik(poly_order + 1), Tn_il(poly_order + 1), Tn_jk(poly_order + 1),
          Tn_jl(poly_order + 1), Tn_kl(poly_order + 1), Tnd_ij(poly_order + 1), Tnd_ik(poly_order + 1),
          Tnd_il(poly_order + 1), Tnd_jk(poly_order + 1), Tnd_jl(poly_order + 1), Tnd_kl(poly_order + 1) {}
    void resize(int poly_order) {
        for (auto* v : {&Tn_ij, &Tn_ik, &Tn_il, &Tn_jk, &Tn_jl, &Tn_kl, &Tnd_ij, &Tnd_ik, &Tnd_il, &Tnd_jk,
                        &Tnd_jl, &Tnd_kl})
            if ((int)v->size() < poly_order + 1) v->resize(poly_order + 1);
    }
    std::vector<double> Tn_ij, Tn_ik, Tn_il, Tn_jk, Tn_jl, Tn_kl;
    std::vector<double> Tnd_ij, Tnd_ik, Tnd_il, Tnd_jk, Tnd_jl, Tnd_kl;
};

class chimesFF {
public:
    int rank;                          /* only gates printing */
    int natmtyps;                      /* number of atom types of the parameter set */
    std::vector<int> poly_orders;      /* [2B order, 3B order, 4B order] */
    std::vector<std::string> atmtyps;  /* atom type names in parameter-file order */
    std::vector<double> masses;
    /* Tabulated 2-/3-body terms (chimesFF.h:196-227; the reference declares
     * these only when built with TABULATION, as its LAMMPS pair style is).
     * Set by read_parameters when the file names tables; declared in every
     * build here so that the class layout does not depend on the option. */
    bool tabulate_2B;
    bool tabulate_3B;

    chimesFF();
    virtual ~chimesFF();
    chimesFF(const chimesFF&) = delete;
    chimesFF& operator=(const chimesFF&) = delete;

    void init(int mpi_rank);                         /* chimesFF.h:148 */
    void read_parameters(std::string paramfile);     /* chimesFF.h:150 */

    void compute_1B(const int typ_idx, double& energy);   /* chimesFF.h:152 */

    /* chimesFF.h:156-161 */
    void compute_2B(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                    std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp& tmp);
    void compute_2B(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                    std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp& tmp,
                    double& force_scalar_in);
    /* chimesFF.h:163-168 */
    void compute_3B(const std::vector<double>& dx, const std::vector<double>& dr, const std::vector<int>& typ_idxs,
                    std::vector<double>& force, std::vector<double>& stress, double& energy, chimes3BTmp& tmp);
    void compute_3B(const std::vector<double>& dx, const std::vector<double>& dr, const std::vector<int>& typ_idxs,
                    std::vector<double>& force, std::vector<double>& stress, double& energy, chimes3BTmp& tmp,
                    std::vector<double>& force_scalar_in);
    /* chimesFF.h:170-175 */
    void compute_4B(const std::vector<double>& dx, const std::vector<double>& dr, const std::vector<int>& typ_idxs,
                    std::vector<double>& force, std::vector<double>& stress, double& energy, chimes4BTmp& tmp);
    void compute_4B(const std::vector<double>& dx, const std::vector<double>& dr, const std::vector<int>& typ_idxs,
                    std::vector<double>& force, std::vector<double>& stress, double& energy, chimes4BTmp& tmp,
                    std::vector<double>& force_scalar_in);

    /* chimesFF.h:204-205, 224-225: the tabulated forms (table look-up instead
     * of the Chebyshev sum; 2-body spline of get_tab_2B, 3-body tricubic
     * interpolation of interpolateTricubic).  Same argument conventions and
     * accumulation as compute_2B/3B; force_scalar_in receives get_penalty's
     * value (2B) or the three table force scalars (3B).  A distance outside
     * the table prints the reference's message and exits (error mode 0). */
    void compute_2B_tab(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                        std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp& tmp);
    void compute_2B_tab(const double dx, const std::vector<double>& dr, const std::vector<int> typ_idxs,
                        std::vector<double>& force, std::vector<double>& stress, double& energy, chimes2BTmp& tmp,
                        double& force_scalar_in);
    void compute_3B_tab(const std::vector<double>& dx, const std::vector<double>& dr, const std::vector<int>& typ_idxs,
                        std::vector<double>& force, std::vector<double>& stress, double& energy, chimes3BTmp& tmp);
    void compute_3B_tab(const std::vector<double>& dx, const std::vector<double>& dr, const std::vector<int>& typ_idxs,
                        std::vector<double>& force, std::vector<double>& stress, double& energy, chimes3BTmp& tmp,
                        std::vector<double>& force_scalar_in);

    /* Batched per-cluster evaluation: n clusters of nbody atoms in one launch.
     * dx[n][P], dr[n][P][3], typ[n][nbody]; force[n][nbody][3] (accumulated per
     * cluster), stress[6] and energy accumulated over all clusters. */
    void compute_clusters(int nbody, int n, const double* dx, const double* dr, const int* typ, double* force,
                          double* stress, double& energy);

    void get_cutoff_2B(std::vector<std::vector<double> >& cutoff_2b);   /* chimesFF.h:177 */
    double max_cutoff_2B(bool silent = false);                          /* chimesFF.h:179-181 */
    double max_cutoff_3B(bool silent = false);
    double max_cutoff_4B(bool silent = false);
    void set_atomtypes(std::vector<std::string>& type_list);            /* chimesFF.h:183 */
    int get_atom_pair_index(int pair_id);                               /* chimesFF.h:185 */
    void build_pair_int_trip_map();                                     /* chimesFF.h:186-187 */
    void build_pair_int_quad_map();
    int get_badness();                                                  /* chimesFF.h:191-192 */
    void reset_badness();

    struct Impl;   /* opaque: GPU engine and parameter slot */

protected:
    Impl* impl_;
    friend class serial_chimes_interface;
};

#endif
