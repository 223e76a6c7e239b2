/*
 * GB300 extension of the ChIMES C interface (libchimescalc.so).
 *
 * These entry points have no counterpart in the reference, whose serial
 * interface evaluates one configuration per call on one CPU core
 * (serial_interface/api/chimescalc_serial_C.h).  They add: returned status
 * codes, several device-resident parameter sets per handle, batched
 * evaluation of many configurations in one set of launches, the mixed
 * FP32/FP64 precision mode, launch tuning, CUDA-graph replay, a split
 * stage/launch/collect form for device timing, diagnostics, cluster-list
 * export and batched per-cluster evaluation.
 *
 * Status codes: 0 ok; -1 parameter file; -2 input; -3 geometry (cutoff vs box,
 * bins); -4 CUDA; -5 capacity (retried internally); -6 call order; -7 device
 * wait timed out.  ck_last_error() returns the message of the last failure on
 * the calling thread.
 *
 * Layouts: positions and forces are [atom][xyz] doubles, concatenated over the
 * configurations of a batch; cells are [config][a,b,c][xyz] (rows are the
 * lattice vectors); types are indices into the parameter set's atom types;
 * stress is [config][9] (xx xy xz yx yy yz zx zy zz) divided by the volume.
 * Batched results are written, not accumulated.
 */
#ifndef CHIMES_GB300_H
#define CHIMES_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* 0 (default): print + exit(0) on errors like the reference; 1: return status. Returns the old mode. */
int ck_set_error_mode(int mode);
const char *ck_last_error(void);

/* Handles (same object as chimes_open_instance / chimes_close_instance). */
void *ck_open(void);
void ck_close(void *h);

/* Parses and uploads a parameter file into a new slot; returns the slot (>= 0)
 * or a negative status.  The first slot loaded becomes the handle's current one. */
int ck_load_params(void *h, const char *path);
int ck_select_params(void *h, int slot);
/* Parses a parameter file on the host only (no device needed): validation and
 * inspection.  Same outputs as ck_param_info. */
int ck_check_params(const char *path, int *orders, int *ntypes, double *maxcuts);
/* orders[3] = 2B/3B/4B orders, *ntypes, maxcuts[3] = max outer cutoffs. */
/* Binary parameter cache (no counterpart in the reference, whose
 * read_parameters parses the text file, chimesFF.cpp:354-1570, on every start):
 * the parsed tables of a slot, or of a text file (host only, no device), in a
 * flat binary file.  ck_load_params / ck_check_params / init_chimes_serial
 * accept either form (the cache is recognised by its magic bytes) and give the
 * same device tables; loading the cache skips the text parse. */
int ck_save_params_cache(void *h, int slot, const char *path);
int ck_convert_params(const char *text_path, const char *cache_path);
int ck_param_info(void *h, int slot, int *orders, int *ntypes, double *maxcuts);
/* Per ordered atom-type tuple u (nbody = 3: nt^3 entries, 4: nt^4) of a slot:
 * valid[u] (an included type with coefficients), ncoef[u] and rout[u][6], the
 * outer cutoffs in the cluster's own pair order. */
int ck_tuple_table(void *h, int slot, int nbody, int *valid, int *ncoef, double *rout);
/* Factored coefficient lists per ordered tuple u (see ck_set_contraction):
 * nrow[u], ncol[u] row and column records (0 for tuples without coefficients)
 * and *R, the powers per pair (0 when the set has no factored tables). */
int ck_tuple_factored(void *h, int slot, int nbody, int *nrow, int *ncol, int *R);
/* out[11] = tpc3, tpc4, blocks_per_sm (per-coefficient kernels), factored 3B and
 * 4B in use for the staged batch (0/1), their threads per cluster and one-warp
 * blocks per SM (ftpc3, ftpc4, fbps3, fbps4), whether the factored 3-body
 * kernel forms its column products per coefficient instead of keeping a table
 * of them (noy3), and which contractions run on the tensor cores (mixed
 * form): bit 0 the 3-body one, bit 1 the 4-body one */
int ck_get_tuning(void *h, int *out);
/* index of an atom type name in a slot, or -1 */
int ck_type_index(void *h, int slot, const char *name);

/* 0: FP64 throughout (default); 1: FP32 Chebyshev/cutoff/contraction with FP64
 * distances and FP64 energy/force/virial accumulation. */
int ck_set_precision(void *h, int precision);
/* threads per 3-body and 4-body cluster (1,2,4,8,16,32) and resident 4-warp
 * blocks per SM of the per-coefficient kernels; the factored kernels take
 * min(tpc, 4) threads per cluster and 4 * blocks_per_sm one-warp blocks
 * (capped by their shared-memory occupancy). */
int ck_set_tuning(void *h, int tpc3, int tpc4, int blocks_per_sm);
/* 3-/4-body contraction kernels: 1 (default) = factored (coefficients grouped
 * by row and column products, two multiply-adds per coefficient) wherever every
 * parameter set of the batch has factored tables (powers per pair R with R^K and
 * R^(P-K) <= 128, K = 1 for 3-body and 3 for 4-body), 0 = per-coefficient
 * kernels everywhere; 2 = factored without the per-entry pair-table cache
 * (the factored kernels otherwise take the Chebyshev tables of a cluster's
 * pairs ij, ik[, il] from one evaluation per neighbour-list entry, when every
 * tuple uses the same cutoffs for a given pair type); 3 = factored with the
 * 3-body kernel forming its column products per coefficient instead of
 * keeping a table of them (ck_autotune also tries this); 4 = factored with
 * the 3-body and 4-body contractions on the tensor cores (tcgen05 TF32 MMAs
 * with a three-part split of both operands) in the mixed form, where every
 * parameter set of the batch has 2-11 powers per pair (3-body) and one
 * count of 2-4 powers per pair (4-body) (ck_autotune also tries these in the
 * mixed form).  All give the same sums in another rounding
 * order. */
int ck_set_contraction(void *h, int factored);
/* Autotuner for the batch staged with ck_stage_batch: times the 3-body and
 * 4-body force kernels (CUDA events) for threads per cluster 1..32 and then
 * 1, 2, 4, 8 resident blocks per SM, keeps the fastest and caches it by the
 * batch's shape (precision, parameter orders, atom and configuration counts
 * rounded to powers of two).  chosen[3] = tpc3, tpc4, blocks_per_sm. */
int ck_autotune(void *h, int *chosen);
/* replay the whole list-build + force sequence as one CUDA graph (1) or launch
 * it stream-ordered (0).  Instances of the serial interface start with 1. */
int ck_use_graph(void *h, int on);
/* Serial-interface instances (calculate_chimes*) autotune once on the third
 * consecutive call with the same atom count (on = 1, the default); 0 keeps the
 * default launch shape. */
int ck_autotune_repeats(void *h, int on);

/* Evaluates nsys configurations in one set of launches.  small[s] (or NULL for
 * all 0) allows replication of small cells, pset[s] (or NULL for the current
 * slot) picks each configuration's parameter set.  energy[nsys], force[sum
 * natoms][3], stress[nsys][9] are written. */
int ck_calculate_batch(void *h, int nsys, const int *natoms, const double *pos, const int *types,
                       const double *cells, const int *small, const int *pset, double *energy, double *force,
                       double *stress);

/* Split form of ck_calculate_batch: stage copies the inputs to the device,
 * launch enqueues the list build and force kernels on the handle's stream
 * (no host synchronisation), collect waits and writes the results.  A
 * capacity overflow is reported by collect as -5 (call launch again). */
int ck_stage_batch(void *h, int nsys, const int *natoms, const double *pos, const int *types, const double *cells,
                   const int *small, const int *pset);
int ck_launch(void *h);
int ck_collect(void *h, double *energy, double *force, double *stress);
/* the handle's cudaStream_t */
void *ck_stream(void *h);

/* Stage timing with CUDA events recorded on the handle's stream around the
 * list build, the 1B+2B, 3B and 4B force kernels.  ck_set_profiling(h, 1)
 * enables and resets it; after each launch ck_read_stage_times waits for the
 * events and adds the intervals: ms[4] (accumulated milliseconds), the number
 * of launches accumulated, and the kernels one launch enqueues. */
int ck_set_profiling(void *h, int on);
/* Measured CUDA-core FMA throughput of this GPU in TFLOP/s, FP64 (precision 0)
 * or FP32 (1): the roofline denominator of the force kernels. */
int ck_fma_peak(int precision, double *tflops);
int ck_read_stage_times(void *h, double *ms, long long *launches, int *kernels_per_launch);

/* out[5] = pairs, triplets, quadruplets, ghost atoms, atoms of the last evaluation */
int ck_last_counts(void *h, long long *out);
/* out[3] = badness (0 good, 1 penalty region, 2 below the inner cutoff), penalty hits, pairs below rin */
int ck_last_diagnostics(void *h, int *out);
/* Cluster lists of the last evaluation in each configuration's ghost numbering
 * (the reference's neighlist_2b/3b/4b order and indices): l2[n2][2] = (atom,
 * neighbour), l3[n3][3], l4[n4][4].  Sizes from ck_last_counts. */
int ck_export_lists(void *h, int *l2, int *l3, int *l4);

/* Evaluation of one periodic configuration that allocates no device memory.
 * No counterpart in the reference (which has no device memory at all).  For
 * callers that cannot call cudaMalloc while they compute forces -- an MD code
 * or framework that reserves the GPU's memory up front and hands out only its
 * own buffers, or a step loop where an allocation could fail or stall.
 * Inputs and outputs are the caller's DEVICE buffers: d_pos[natom][3]
 * Cartesian positions, d_types[natom] type indices of the handle's current
 * parameter set; cell[9] (host) = lattice vectors a, b, c; small allows
 * replication.  Written (not accumulated): *d_energy (divided by
 * (n_replicates+1)^3 as in serial_chimes_interface::calculate),
 * d_force[natom][3], d_stress[9] (virial over volume).  Work is enqueued on
 * `stream` (a cudaStream_t, 0 = legacy default) and the call waits for it.
 * Every intermediate array lives in one static device array of about 13.4 MiB
 * that each GPU loading the library holds until the process exits; limits per
 * call: 2048 atoms after replication, 65536 ghost-image slots, 65536 bin cells,
 * 65536 pairs, 131072 triplets, 65536 quadruplets.  Larger inputs return -2
 * (sizes known before the launch) or -5 (list sizes found on the device; the
 * outputs are then invalid), with the message in ck_last_error().  The first
 * call on each device looks up the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  Calls share the array and
 * each clears what must start at zero; calls whose GPU work overlaps (other
 * streams, threads or handles) race on it and corrupt each other's results. */
int ck_calculate_noalloc(void *h, int natom, const double *d_pos, const int *d_types, const double *cell,
                         int small, double *d_energy, double *d_force, double *d_stress, void *stream);

/* Continuous-batching request server (no counterpart in the reference).
 * n_workers threads each own an engine (CUDA stream, device-resident
 * parameter sets, workspace); each takes the oldest waiting requests while the
 * batch stays under max_batch_atoms and the estimated device memory of all
 * batches in flight stays under hbm_budget_gb, evaluates them in one set of
 * launches and publishes the results.  Requests submitted while batches run
 * join the next batch a worker forms; batches of different workers overlap on
 * the GPU.  precision: 0 FP64, 1 mixed.  Returns NULL on failure. */
void *ck_server_open(int n_workers, double hbm_budget_gb, long long max_batch_atoms, int precision);
void ck_server_close(void *server);
/* loads a parameter file into every worker; returns its slot */
int ck_server_load_params(void *server, const char *path);
/* queues one configuration (host arrays are copied); returns a request id > 0 */
long long ck_server_submit(void *server, int slot, int natom, const double *pos, const int *types,
                           const double *cell, int small);
/* Results of a request: returns 1 when done (outputs written: energy, force[natom][3],
 * stress[9], latency from submit to completion in seconds; the request is
 * released), 0 while pending (wait = 1 blocks up to timeout_s), or a negative
 * status if the request failed (released; message in ck_last_error). */
int ck_server_take(void *server, long long id, int wait, double timeout_s, double *energy, double *force,
                   double *stress, double *latency_s);
/* Tunes the contraction kernels of every worker on a representative batch
 * (arrays as for ck_calculate_batch; small and pset may be NULL): worker 0
 * times the contraction forms and launch shapes on it and every worker takes
 * its choices.  Call it after loading the parameter sets and before
 * submitting requests.  chosen[3] (may be NULL) = lanes per 3-body and
 * 4-body cluster, resident blocks per SM. */
int ck_server_autotune(void *server, int nsys, const int *natoms, const double *pos, const int *types,
                       const double *cells, const int *small, const int *pset, int *chosen);
/* Offers a trace of nreq requests (arrays as for ck_calculate_batch, plus
 * their parameter slots) at arrival_s[q] seconds after the call starts, from
 * a native submitting thread, and takes the results in order on the calling
 * thread: latency_s[q] (submit to result) and energy[q] (either may be NULL),
 * wall_s = first submission to last result.  Measures the server without a
 * client's per-request overhead. */
int ck_server_replay(void *server, int nreq, const int *slots, const int *natoms, const double *pos,
                     const int *types, const double *cells, const int *small, const double *arrival_s,
                     double *latency_s, double *energy, double *wall_s);
/* out[6] = submitted, completed, batches, largest batch, bytes in flight, peak bytes in flight */
int ck_server_stats(void *server, long long *out);
/* out[11] = worker's launch preferences, in ck_get_tuning's order with the
 * factored and tensor-core entries as preferences (want_fact3, want_fact4;
 * out[10] bit 0 the 3-body, bit 1 the 4-body tensor-core preference): after
 * ck_server_autotune every worker holds worker 0's. */
int ck_server_worker_tuning(void *server, int worker, int *out);

/* Pair-style evaluation on a caller's full neighbour list with ghost atoms:
 * the GPU form of LAMMPS pair_style chimesFF (etc/lmp/src/pair_chimes.cpp:
 * build_mb_neighlists :321-478, compute :480-884), newton on.  Arrays are the
 * caller's host arrays: x[nall][3] (local then ghost atoms), type[nall] (type
 * indices of the handle's current parameter set, i.e. chimes_type[type-1]),
 * tag[nall] (global atom ids; a ghost carries its owner's id); ilist[inum]
 * (atoms with lists), numneigh[inum] and neigh[] (each list's neighbour
 * indices with the NEIGHMASK bits stripped, concatenated in ilist order).
 * 1-body for ilist atoms and 2-body for listed pairs with tag[j] > tag[i] use
 * this call's list; 3-/4-body clusters are built from it when rebuild != 0
 * (LAMMPS: neighbor->ago == 0; also on the first call and whenever nall, inum
 * or the entry count change) with the cutoffs max_cutoff_3B/4B + skin, and
 * evaluated every call with the current positions.  Accumulates f[nall][3]
 * (forces on ghosts included, for the reverse communication), *energy and
 * virial[6] (xx yy zz xy xz yz, as Pair::ev_tally_mb) and, when not NULL,
 * per-atom eatom[nall] and vatom[nall][6] (each interaction's energy and
 * virial shared equally by its atoms, as ev_tally_mb's eflag_atom and
 * vflag_atom branches).  A parameter set with tabulated 2-/3-body terms (the
 * reference's TABULATION build, pair_chimes.cpp:620-622, 697-699) is evaluated
 * with the table look-ups of compute_2B_tab / compute_3B_tab; a distance
 * outside a table returns an error. */
int ck_nl_compute(void *h, int nall, const double *x, const int *type, const long long *tag, int inum,
                  const int *ilist, const int *numneigh, const int *neigh, double skin, int rebuild, double *f,
                  double *energy, double *virial, double *eatom, double *vatom);
/* counts[2] = triplets, quadruplets of the last cluster build; l3[n3][3] and
 * l4[n4][4] (atom indices, may be NULL) */
int ck_nl_lists(void *h, long long *counts, int *l3, int *l4);

/* Cluster fingerprints (the reference's FINGERPRINT build,
 * etc/lmp/src/pair_chimes.cpp:525-536, 620-662, 700-741, 775-810 and
 * chimesFF/src/chimesFF.cpp:1694-1702, 2013-2021, 2603-2612): the records the
 * pair style writes to "<step>.<rank>.<n>b_clusters.txt" for the last
 * ck_nl_compute call -- the nbody-atom clusters compute_nB evaluated whose
 * atoms are in recording order (2-body: i < j; 3-/4-body: strictly increasing
 * tags), in the pair style's loop order.  *n receives the count; dist[n][P]
 * (distances ij / ij,ik,jk / ij,ik,il,jk,jl,kl) and types[n][nbody] (type
 * indices) are filled when not NULL (call once with NULLs to size them). */
int ck_nl_fingerprint(void *h, int nbody, long long *n, double *dist, int *types);

/* Cluster-distance histogram of the reference's fingerprint tool
 * (chimesFF/src/FP/multi_calc_histogram.cpp, gen_flat_hists with one process)
 * for records of one body order, with the handle's parameter set: each
 * record's distances are mapped with the Morse transform of its own cutoffs
 * and sorted; every pair (i of set 1, j of set 2, or j > i within set 1 when
 * same != 0) adds its Euclidean distance to counts[nbin] over [0, maxd), maxd
 * = 3, sqrt(12)+1, sqrt(24)+1 for nbody = 2, 3, 4 (the reference uses nbin =
 * 100).  *nsamples receives the number of counted pairs; the normalised
 * histogram is counts / nsamples at bin centres (k + 1/2) * maxd / nbin.  As in
 * the reference, a first set of fewer than two records counts nothing.  A
 * distance past the last bin is an error (the reference exits there). */
int ck_fp_histogram(void *h, int nbody, long long n1, const double *d1, const int *t1, long long n2,
                    const double *d2, const int *t2, int same, int nbin, long long *counts, long long *nsamples);

/* Batched per-cluster evaluation (chimesFF::compute_nB semantics, FP64) with
 * the handle's current parameter set: n clusters of nbody = 2, 3 or 4 atoms,
 * dx[n][P] distances, dr[n][P][3] vectors (atom2 - atom1, pairs ij / ij,ik,jk /
 * ij,ik,il,jk,jl,kl), typ[n][nbody].  Writes force[n][nbody][3], packed
 * stress[n][6], energy[n] and the reference's force scalars fscal[n][P]
 * (may be NULL); clusters of excluded types or beyond a cutoff get zeros. */
int ck_compute_cluster_batch(void *h, int nbody, int n, const double *dx, const double *dr, const int *typ,
                             double *force, double *stress, double *energy, double *fscal);
/* The same for tabulated terms (chimesFF::compute_2B_tab / compute_3B_tab,
 * chimesFF/src/chimesFF.cpp:1776-1867, 2177-2322, the reference's TABULATION
 * build): nbody = 2 or 3, the set's terms of that order must be tabulated.
 * fscal[n][P] receives force_scalar_in (2B: get_penalty's value, 3B: the table
 * force scalars).  A distance outside a table is an error (the reference prints
 * "Distance is outside the tabulated range" and exits). */
int ck_compute_cluster_batch_tab(void *h, int nbody, int n, const double *dx, const double *dr, const int *typ,
                                 double *force, double *stress, double *energy, double *fscal);
/* tab[2] = 1 when the handle's 2-body / 3-body terms are tabulated */
int ck_tabulated(void *h, int *tab);

#ifdef __cplusplus
}
#endif

#endif
