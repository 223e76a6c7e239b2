/*
 * Per-cluster C interface of the GB300 ChIMES library -- drop-in for the
 * reference's chimesFF/api/chimescalc_C.h (lines 11-28).
 *
 * The caller owns the cluster loop and passes distances, displacement vectors
 * (atom2 - atom1) and atom type names; every call evaluates its cluster on the
 * GPU (per-cluster kernel).  Energy and forces are added into the caller's
 * values; the packed stress (xx xy xz yy yz zz) is added into stress[0..5],
 * as the reference's wrappers do (chimescalc_C.cpp:114-318; the 4-body
 * wrapper assigns back its accumulated copy, which has the same effect).
 * The 3B/4B wrappers take the distances in the argument named dr_3b/dr_4b and
 * the vectors in dist_3b/dist_4b, as in the reference.
 * For many clusters per call use ck_compute_cluster_batch (chimes_gb300.h) or
 * chimesFF::compute_clusters (chimesFF.h).
 */
#ifndef CHIMES_GB300_CHIMESCALC_C_H
#define CHIMES_GB300_CHIMESCALC_C_H

#ifdef __cplusplus
extern "C" {
#endif

/* replace chimescalc_C.h:11-13 (chimescalc_C.cpp:24-37) */
double get_chimes_max_2b_cutoff();
double get_chimes_max_3b_cutoff();
double get_chimes_max_4b_cutoff();
/* replace chimescalc_C.h:14-16 (chimescalc_C.cpp:43-66) */
int get_chimes_2b_order();
int get_chimes_3b_order();
int get_chimes_4b_order();
/* replaces chimescalc_C.h:17 (chimescalc_C.cpp:39-41) */
void set_chimes();
/* replaces chimescalc_C.h:18 (chimescalc_C.cpp:68-70) */
void init_chimes(int rank);
/* replaces chimescalc_C.h:19 (chimescalc_C.cpp:72-76); also builds the pair maps */
void chimes_read_params(char *param_file);
/* replace chimescalc_C.h:20-21 (chimescalc_C.cpp:78-84); the maps are built by chimes_read_params */
void chimes_build_pair_int_trip_map();
void chimes_build_pair_int_quad_map();
/* replaces chimescalc_C.h:22 (chimescalc_C.cpp:114-163) */
void chimes_compute_2b_props(double rij, double dr[3], char *atype2b[2], double force[2][3], double stress[9],
                             double *epot);
/* replaces chimescalc_C.h:23 (chimescalc_C.cpp:165-230) */
void chimes_compute_3b_props(double dr_3b[3], double dist_3b[3][3], char *atype3b[3], double f3b[3][3],
                             double stress[9], double *epot);
/* replaces chimescalc_C.h:24 (chimescalc_C.cpp:232-318) */
void chimes_compute_4b_props(double dr_4b[6], double dist_4b[6][3], char *atype4b[4], double f4b[4][3],
                             double stress[9], double *epot);
/* replace chimescalc_C.h:26-28 (chimescalc_C.cpp:86-112): Fortran-callable variants */
void chimes_compute_2b_props_fromf90(double *rij, double dr[3], char *type1, char *type2, double force[2][3],
                                     double stress[9], double *epot);
void chimes_compute_3b_props_fromf90(double dr_3b[3], double dist_3b[3][3], char *type1, char *type2, char *type3,
                                     double f3b[3][3], double stress[9], double *epot);
void chimes_compute_4b_props_fromf90(double dr_4b[6], double dist_4b[6][3], char *type1, char *type2, char *type3,
                                     char *type4, double f4b[4][3], double stress[9], double *epot);

#ifdef __cplusplus
}
#endif

#endif
