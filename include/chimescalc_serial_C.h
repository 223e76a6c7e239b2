/*
 * C interface of the GB300 ChIMES serial calculator -- drop-in for the
 * reference's serial_interface/api/chimescalc_serial_C.h (lines 11-18).
 *
 * Same symbols, arguments and semantics as the reference (implementation of
 * the reference: serial_interface/api/chimescalc_serial_C.cpp:24-124):
 *   - set_chimes_serial(small) selects the library's static instance and must
 *     be called before init_chimes_serial;
 *   - calculate_chimes adds the energy and forces into *energy and fx/fy/fz
 *     (the energy sum is divided by (n_replicates+1)^3 when a small cell is
 *     replicated) and overwrites stress[9] (xx xy xz yx yy yz zx zy zz, the
 *     virial over the cell volume);
 *   - the *_instance variants work on handles from chimes_open_instance;
 *     init_chimes_serial_instance ignores rank, like the reference;
 *   - on an error the message goes to stdout and the process exits with status
 *     0, like the reference; ck_set_error_mode(1) (chimes_gb300.h) switches to
 *     returned status codes instead.
 * Units: kcal/mol, Angstrom, kcal/mol/Angstrom, kcal/mol/Angstrom^3.
 * Every calculation runs on the GPU; there is no CPU path.
 */
#ifndef CHIMES_GB300_CHIMESCALC_SERIAL_C_H
#define CHIMES_GB300_CHIMESCALC_SERIAL_C_H

#ifdef __cplusplus
extern "C" {
#endif

/* replaces chimescalc_serial_C.h:11 (chimescalc_serial_C.cpp:24-29) */
void *chimes_open_instance();
/* replaces chimescalc_serial_C.h:12 (chimescalc_serial_C.cpp:30-34) */
void chimes_close_instance(void *handle);
/* replaces chimescalc_serial_C.h:13 (chimescalc_serial_C.cpp:35-46) */
void set_chimes_serial(int small);
/* replaces chimescalc_serial_C.h:14 (chimescalc_serial_C.cpp:47-57) */
void set_chimes_serial_instance(void *handle, int small);
/* replaces chimescalc_serial_C.h:15 (chimescalc_serial_C.cpp:59-63) */
void init_chimes_serial(char *param_file, int *rank);
/* replaces chimescalc_serial_C.h:16 (chimescalc_serial_C.cpp:64-69) */
void init_chimes_serial_instance(void *handle, char *param_file, int rank);
/* replaces chimescalc_serial_C.h:17 (chimescalc_serial_C.cpp:70-73) */
void calculate_chimes(int natom, double *xc, double *yc, double *zc, char *atom_types[], double ca[3], double cb[3],
                      double cc[3], double *energy, double fx[], double fy[], double fz[], double stress[9]);
/* replaces chimescalc_serial_C.h:18 (chimescalc_serial_C.cpp:74-124) */
void calculate_chimes_instance(void *handle, int natom, double *xc, double *yc, double *zc, char *atom_types[],
                               double ca[3], double cb[3], double cc[3], double *energy, double fx[], double fy[],
                               double fz[], double stress[9]);

#ifdef __cplusplus
}
#endif

#endif
