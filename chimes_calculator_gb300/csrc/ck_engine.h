// Host engine of the GB300 ChIMES force path: owns one CUDA stream, the
// device-resident parameter sets and a grow-only batch workspace, and runs the
// list build and force kernels for a batch of periodic systems.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "ck_common.h"
#include "ck_kernels.h"
#include "ck_params.h"

namespace ck {

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { if (p) cudaFree(p); }
    // grows (never shrinks); contents are not preserved
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        size_t want = n + n / 4 + 64;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        cap = e == cudaSuccess ? want : 0;
        return e;
    }
};

template <class T>
struct PinnedBuf {
    T* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        size_t want = n + n / 4 + 64;
        cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
        cap = e == cudaSuccess ? want : 0;
        return e;
    }
};

// One periodic configuration as the caller passes it.
struct SystemSpec {
    int n = 0;
    const double* pos = nullptr;   // [n][3] Cartesian (x,y,z interleaved)
    const int* types = nullptr;    // [n] atom type index of the parameter set
    double cell[9] = {0};          // rows: lattice vectors a, b, c
    bool small = false;            // allow replication of small cells (reference `small`)
    int pset = 0;                  // parameter-set slot
};

struct SystemResult {
    double energy = 0.0;           // 1B+2B+3B+4B energy divided by (n_rep+1)^3
    double virial[6] = {0, 0, 0, 0, 0, 0};   // packed xx xy xz yy yz zz, not divided by the volume
    double vol = 0.0;
    int n_rep = 0;
};

struct RunStats {
    long long n2 = 0, n3 = 0, n4 = 0;
    long long n_atoms = 0, n_ghost = 0;
    int badness = 0;
    int penalty_hits = 0, below_rin = 0;
};

class Engine {
public:
    Engine();
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    Status init_device(std::string& err);
    // CUDA device current when the engine was set up (its stream, parameter sets, workspace)
    int device() const { return device_; }
    // Parses a parameter file into a new device-resident slot; returns the slot (>= 0).
    int load_params(const std::string& path, std::string& err);
    const HostParams& params(int slot) const { return *sets_[slot].host; }
    int n_param_sets() const { return (int)sets_.size(); }
    const DevParamSet* device_params() const { return dsets_.p; }   // device array, by slot
    const DevParamSet& param_view(int slot) const { return sets_[slot].view; }
    int n_buckets(int nbody) const { return nbody == 3 ? nbk3_ : nbk4_; }
    const std::vector<TupleRec>& tuples(int slot, int nbody) const {
        return nbody == 3 ? sets_[slot].t3 : sets_[slot].t4;
    }

    // Full evaluation of a batch: stage + launch + collect, retrying on capacity growth.
    // force_out: [sum n][3], zeroed and filled (not accumulated).
    Status run(const std::vector<SystemSpec>& sys, double* force_out, std::vector<SystemResult>& res,
               std::string& err);

    // Split form (the bench times launch() on device-resident inputs):
    Status stage(const std::vector<SystemSpec>& sys, std::string& err);   // host geometry + async H2D
    Status launch(std::string& err);                                       // list build + forces, async
    Status collect(double* force_out, std::vector<SystemResult>& res, std::string& err);  // D2H + sync

    cudaStream_t stream() const { return stream_; }
    ForceLaunch tuning;
    // 3-/4-body contraction: true = factored kernels wherever every parameter
    // set of the batch has factored tables, false = per-coefficient kernels
    bool factored = true;
    // run the 4-body branch on a second stream beside 1B+2B and 3-body (not while profiling)
    bool concurrent = true;
    // factored kernels take the pairs of a cluster's first atom from a per-entry table cache
    bool pair_cache = true;
    int precision = kFP64;
    bool use_graph = false;
    RunStats last;

    // Stage timing: CUDA events recorded on the engine's stream between the
    // list build, the 1B+2B, 3B and 4B force kernels, accumulated over launches.
    bool profile = false;
    double stage_ms[4] = {0, 0, 0, 0};   // list build, 2B, 3B, 4B
    long long stage_launches = 0;
    int kernels_per_launch = 0;          // kernels one launch() enqueues
    Status read_stage_times(std::string& err);   // adds the last launch's event intervals

    // Autotuner for the staged batch: times the 3-body and 4-body force stages
    // (CUDA events on the engine's stream) for each threads-per-cluster value
    // and then each resident-blocks value, keeps the fastest, and caches the
    // choice by the batch's shape (precision, parameter orders, atom and system
    // counts in powers of two).  chosen = {tpc3, tpc4, blocks_per_sm}.
    Status autotune(int* chosen, std::string& err);

    // Per-cluster evaluation (the chimesFF::compute_nB entry points): n
    // clusters of `nbody` atoms given as distances dx[n][P], displacement
    // vectors dr[n][P][3] (atom2 - atom1) and type indices typ[n][nbody].
    // Writes per-cluster force[n][nbody][3], packed stress[n][6], energy[n],
    // force scalars fscal[n][P] and status[n] (see ck_direct.cu).
    Status compute_clusters(int slot, int nbody, int n, const double* dx, const double* dr, const int* typ,
                            double* force, double* stress, double* energy, double* fscal, int* status,
                            std::string& err, bool tab = false);

    // Cluster lists of the last run in system-local ghost numbering (the
    // reference's sys_parent/ghost indices), for set comparisons.
    Status export_lists(std::vector<int>& l2, std::vector<int>& l3, std::vector<int>& l4, std::string& err);

private:
    struct PSet {
        std::unique_ptr<HostParams> host;
        void* dev = nullptr;
        DevParamSet view{};
        std::vector<TupleRec> t3, t4;   // host copies of the tuple records
    };
    std::vector<PSet> sets_;
    DevBuf<DevParamSet> dsets_;
    cudaStream_t stream_ = nullptr;
    cudaStream_t stream2_ = nullptr;              // the 4-body branch
    cudaEvent_t fork_ = nullptr, fork2_ = nullptr, join_ = nullptr;
    bool ready_ = false;
    int device_ = -1;

    // batch layout of the staged batch
    std::vector<SysDesc> hsys_;
    std::vector<double> vols_;
    BatchView V_{};
    long long n2_cap_ = 0, n3_cap_ = 0, n4_cap_ = 0;
    bool staged_ = false;

    DevBuf<SysDesc> d_sys_;
    DevBuf<double> d_in_pos_;
    DevBuf<int> d_in_type_;
    DevBuf<int> d_atom_sys_, d_atom_type_, d_atom_orig_;
    DevBuf<int> d_atom_self_, d_ghost_id_;
    DevBuf<float> d_ghost_xf_, d_l2_vec_, d_bin_xp_;
    DevBuf<int> d_ghost_parent_, d_ghost_bin_;
    DevBuf<double> d_ghost_fs_, d_ghost_xn_, d_ghost_fn_;
    DevBuf<unsigned long long> d_minmax_;
    DevBuf<int> d_bin_count_, d_bin_fill_, d_bin_items_;
    DevBuf<long long> d_bin_start_;
    DevBuf<int> d_l2_count_, d_l2_ghost_, d_l2_owner_;
    DevBuf<long long> d_l2_off_;
    DevBuf<double> d_l2_dist_;
    DevBuf<int> d_e_cnt3_, d_e_cnt4_;
    DevBuf<long long> d_e_off3_, d_e_off4_;
    DevBuf<int> d_c3_, d_c4_;
    int nbk3_ = 0, nbk4_ = 0;     // cluster buckets over all loaded parameter sets
    bool avail_fact3_ = false, avail_fact4_ = false;   // staged batch has factored tables
    bool avail_tc3_ = false;                           // ... and tensor-core 3-body images (mixed form)
    bool avail_tc4_ = false;                           // ... and tensor-core 4-body images at one R
    bool enum_serial_ = false;                         // staged batch needs the sequential enumeration
    bool avail_pc3_ = false, avail_pc4_ = false;       // pair-table cache usable for the staged batch
    bool pc_small_ = false;                            // list small enough for the cache to stay near L2
    DevBuf<int> d_c3e_, d_c4e_;
    DevBuf<double> d_pcd3_, d_pcd4_;
    DevBuf<unsigned char> d_pct3_, d_pct4_;
    DevBuf<int> d_bk_count_, d_bk_fill_, d_perm3_, d_perm4_;
    DevBuf<long long> d_bk_start_;
    DevBuf<double> d_force_, d_ev_;
    DevBuf<int> d_flags_;
    DevBuf<unsigned long long> d_queue_;
    DevBuf<unsigned char> d_scan_tmp_;
    DevBuf<double> d_dir_d_;      // per-cluster inputs and outputs (doubles)
    DevBuf<int> d_dir_i_;         // per-cluster types and status

    PinnedBuf<double> h_in_pos_;
    PinnedBuf<int> h_in_type_;
    PinnedBuf<double> h_force_;
    PinnedBuf<double> h_ev_;
    PinnedBuf<int> h_flags_;
    PinnedBuf<long long> h_counts_;

    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    std::vector<long long> graph_key_;
    std::vector<long long> seen_key_;   // shape of the last launch (a graph is captured on a repeat)
    cudaEvent_t ev_[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool ev_recorded_ = false;

    Status ensure_lists(std::string& err);
    Status enqueue(std::string& err);
    void drop_graph();
    std::string tune_key() const;
    std::vector<std::pair<std::string, ForceLaunch>> tune_cache_;
};

const char* status_name(int s);

// One configuration evaluated with every intermediate array in a static
// device array instead of allocated memory (ck_noalloc.cu); inputs and
// outputs are the caller's device buffers.  Synchronises `st` before returning.
Status calculate_noalloc(Engine& eng, int slot, int natom, const double* d_pos, const int* d_types,
                         const double* cell, bool small, double* d_energy, double* d_force, double* d_stress,
                         cudaStream_t st, std::string& err);

// Error reporting of the public interfaces: records the message for
// ck_last_error() and, in the default (reference) mode, prints it on stdout
// and calls exit(0); in return mode it only returns `status`.
int report_error(int status, const std::string& msg);
void clear_error();

}  // namespace ck
