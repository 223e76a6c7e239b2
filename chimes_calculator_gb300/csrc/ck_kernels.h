// Kernel launchers of the GB300 ChIMES force path.
#pragma once
#include <cuda_runtime.h>

#include "ck_common.h"

namespace ck {

// ---- cluster-list build (ck_lists.cu) -------------------------------------
void launch_atoms(const BatchView& B, cudaStream_t st);
void launch_ghosts(const BatchView& B, cudaStream_t st);
void launch_bin_setup(const BatchView& B, cudaStream_t st);
void launch_bin_count(const BatchView& B, cudaStream_t st);
void launch_bin_scatter(const BatchView& B, cudaStream_t st);
void launch_bin_sort(const BatchView& B, cudaStream_t st);
void launch_l2(const BatchView& B, int* l2_owner, bool fill, cudaStream_t st);
// Runs over the list capacity B.n2_cap; the live count is read on the device.
void launch_enum(const BatchView& B, const int* l2_owner, bool fill, cudaStream_t st);
// Sets capacity flags when a live count exceeds its buffer.
void launch_check(const BatchView& B, cudaStream_t st);
// Clears bounding boxes, accumulators and flags.
void launch_reset(const BatchView& B, cudaStream_t st);

// Exclusive scan of n ints into n+1 int64 (out[n] = total).  `tmp` must hold
// scan_tmp_bytes(n) bytes.
size_t scan_tmp_bytes(long long n);
void exclusive_scan(const int* in, long long* out, long long n, void* tmp, cudaStream_t st);
// two scans of the same length in the same launches (tmp as for one)
void exclusive_scan2(const int* in_a, long long* out_a, const int* in_b, long long* out_b, long long n, void* tmp,
                     cudaStream_t st);

// ---- forces (ck_force.cu) ------------------------------------------------
enum Precision : int { kFP64 = 0, kMixed = 1 };

struct ForceLaunch {
    int precision = kFP64;
    int tpc3 = 4;          // threads per 3-body cluster
    int tpc4 = 8;          // threads per 4-body cluster
    int block = 256;
    int blocks_per_sm = 4;
    int stride3 = 0;       // polynomial table stride (max 3B order + 1 over the batch's sets)
    int stride4 = 0;
    // factored contraction (ck_factored.cu), used per body order when every
    // parameter set of the batch has its tables
    int fact3 = 0, fact4 = 0;
    int want_fact3 = 1, want_fact4 = 1;   // preference (autotuner); fact = want && tables present
    int rf3 = 0, rf4 = 0;  // powers per pair (max over the batch's sets)
    // threads per cluster: 1, 2 or 4 (the 4-body default 4: what the autotuner
    // picks on the FP64 workloads; untuned paths such as ck_nl_compute use it)
    int ftpc3 = 1, ftpc4 = 4;
    int fbps3 = 8, fbps4 = 8;      // resident one-warp blocks per SM (capped by occupancy)
    int noy3 = 0;                  // factored 3-body without the Y table (products per entry)
    // tensor-core 3-body contraction (mixed form only; ck_tensor.cu): tc3 = in
    // use for this launch, want_tc3 = preference (autotuner or forced)
    int tc3 = 0, want_tc3 = 0;
    // tensor-core 4-body contraction (mixed form, one R <= kTc4MaxR over the batch)
    int tc4 = 0, want_tc4 = 0;
};

// Cluster counts are read on the device (l2_off[n_atoms], e_off3/4[n2_cap]) and
// clamped to the capacities, so launches need no host round trip.
void launch_force2(const BatchView& B, const int* l2_owner, const ForceLaunch& L, cudaStream_t st);
void launch_force3(const BatchView& B, const ForceLaunch& L, cudaStream_t st);
void launch_force4(const BatchView& B, const ForceLaunch& L, cudaStream_t st);

// Factored contraction (ck_factored.cu): bucket the clusters of one body
// order by (parameter set, type tuple), then contract.  Both read their
// counts on the device.
void launch_bucket(const BatchView& B, int nbody, cudaStream_t st);
// Pair-table cache of body order nbody (when B.use_pc3 / use_pc4): one pass over the list entries.
void launch_pair_tables(const BatchView& B, const int* l2_owner, int nbody, const ForceLaunch& L, cudaStream_t st);
void launch_force3f(const BatchView& B, const ForceLaunch& L, cudaStream_t st);
void launch_force4f(const BatchView& B, const ForceLaunch& L, cudaStream_t st);
// Tensor-core 3-body contraction (ck_tensor.cu): mixed form, R3 powers per
// pair in [2, kTc3MaxR]; clusters bucketed with 128-slot padding (bk_pad3).
bool tc3_supported(int rf3);
void launch_force3tc(const BatchView& B, const ForceLaunch& L, cudaStream_t st);
// Tensor-core 4-body contraction (ck_tensor.cu): mixed form, R4 powers per
// pair in [2, kTc4MaxR]; tiles of 32 clusters (the 4-body buckets' padding).
bool tc4_supported(int rf4);
void launch_force4tc(const BatchView& B, const ForceLaunch& L, cudaStream_t st);
// dynamic shared memory of one factored-kernel block (one warp)
size_t factored_smem_bytes(int nbody, int precision, int tpc, int rs);

// Pair-style path on a caller's neighbour list (ck_neigh.cu): list-entry
// owners and the identity atom/slot mapping; cluster counting / filling; 1B+2B.
void launch_nl_setup(const BatchView& B, const NeighView& N, cudaStream_t st);
void launch_nl_enum(const BatchView& B, const NeighView& N, bool fill, cudaStream_t st);
void launch_nl_pairs(const BatchView& B, const NeighView& N, int precision, cudaStream_t st);
// FP32 copy of the positions (n = 3 * atoms values) for the cutoff tests
void launch_nl_xf(const double* x, float* xf, long long n, cudaStream_t st);
// tabulated 3-body term: selection of the evaluated triplets (sel[n3], selr[3*n3],
// *count on the device) and their look-ups
void launch_nl_tab3(const BatchView& B, long long n3, int* sel, double* selr, unsigned long long* count,
                    cudaStream_t st);
// Fingerprint records of body order nbody over n candidates (list entries for
// 2-body, listed clusters for 3-/4-body): count pass (flag[n]) or fill pass
// (records at the scanned offsets off[n]) (ck_fingerprint.cu).
void launch_nl_fp(const BatchView& B, const NeighView& N, int nbody, long long n, bool fill, int* flag,
                  const long long* off, double* d, int* t, cudaStream_t st);

// Per-cluster evaluation (caller-owned cluster loop), FP64; order = the body
// order's polynomial order of the set (sizes the 3-/4-body kernels' tables).
void launch_direct(const DevParamSet* P, int nbody, int order, int n, const double* dx, const double* dr,
                   const int* typ, double* force, double* stress, double* energy, double* fscal, int* status,
                   cudaStream_t st, bool tab = false);

int sm_count();

// Measured CUDA-core FMA throughput (TFLOP/s) in FP64 (precision 0) or FP32 (1).
double fma_peak_tflops(int precision);

// Host-side count of kernel launches enqueued by the launchers above (for
// reporting how many of the library's kernels one evaluation runs).
void count_launch();
long long launch_counter();

}  // namespace ck
