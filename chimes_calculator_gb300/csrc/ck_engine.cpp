// Host engine: staging, the launch sequence of the list build and force
// kernels (optionally replayed as one CUDA graph), capacity growth and result
// collection.  See ck_engine.h.
#include "ck_engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "ck_geom.h"
#include "nvtx3/nvToolsExt.h"

namespace ck {

#define CK_TRY(call)                                                              \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call; \
            return kErrCuda;                                                      \
        }                                                                         \
    } while (0)

const char* status_name(int s) {
    switch (s) {
        case kOk: return "ok";
        case kErrParam: return "parameter file error";
        case kErrInput: return "input error";
        case kErrGeometry: return "geometry error";
        case kErrCuda: return "CUDA error";
        case kErrCapacity: return "capacity exceeded";
        case kErrState: return "call-order error";
        case kErrTimeout: return "device wait timed out";
        default: return "error";
    }
}

Engine::Engine() {}

Engine::~Engine() {
    drop_graph();
    for (auto& e : ev_)
        if (e) cudaEventDestroy(e);
    for (auto& s : sets_)
        if (s.dev) cudaFree(s.dev);
    if (fork_) cudaEventDestroy(fork_);
    if (fork2_) cudaEventDestroy(fork2_);
    if (join_) cudaEventDestroy(join_);
    if (stream2_) cudaStreamDestroy(stream2_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Engine::drop_graph() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    graph_exec_ = nullptr;
    graph_ = nullptr;
    graph_key_.clear();
}

Status Engine::init_device(std::string& err) {
    if (ready_) return kOk;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        err = std::string("no CUDA device available: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        return kErrCuda;
    }
    CK_TRY(cudaGetDevice(&device_));
    CK_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    CK_TRY(cudaStreamCreateWithFlags(&stream2_, cudaStreamNonBlocking));
    CK_TRY(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    CK_TRY(cudaEventCreateWithFlags(&fork2_, cudaEventDisableTiming));
    CK_TRY(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
    CK_TRY(h_flags_.reserve(8));
    CK_TRY(h_counts_.reserve(4));
    CK_TRY(d_flags_.reserve(8));
    CK_TRY(d_queue_.reserve(2));
    ready_ = true;
    return kOk;
}

int Engine::load_params(const std::string& path, std::string& err) {
    Status st = init_device(err);
    if (st != kOk) return st;
    PSet ps;
    ps.host.reset(new HostParams());
    st = parse_parameter_file(path, *ps.host, err);
    if (st != kOk) return st;
    ParamImage img = pack_params(*ps.host);
    cudaError_t e = cudaMalloc(&ps.dev, img.bytes.size());
    if (e == cudaSuccess) e = cudaMemcpy(ps.dev, img.bytes.data(), img.bytes.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        err = std::string("CUDA error uploading parameters: ") + cudaGetErrorString(e);
        if (ps.dev) cudaFree(ps.dev);
        return kErrCuda;
    }
    // host copies of the tuple records (inspection, work models)
    {
        const int nt = img.header.ntypes;
        if (img.header.t3)
            ps.t3.assign(reinterpret_cast<const TupleRec*>(img.bytes.data() + (uintptr_t)img.header.t3),
                         reinterpret_cast<const TupleRec*>(img.bytes.data() + (uintptr_t)img.header.t3) + nt * nt * nt);
        if (img.header.t4)
            ps.t4.assign(reinterpret_cast<const TupleRec*>(img.bytes.data() + (uintptr_t)img.header.t4),
                         reinterpret_cast<const TupleRec*>(img.bytes.data() + (uintptr_t)img.header.t4) +
                             nt * nt * nt * nt);
    }
    // relocate the offsets of the header to device pointers
    DevParamSet h = img.header;
    const uintptr_t base = (uintptr_t)ps.dev;
    auto rel = [&](auto& ptr) {
        if (ptr) ptr = reinterpret_cast<std::remove_reference_t<decltype(ptr)>>(base + (uintptr_t)ptr);
    };
    rel(h.eoff); rel(h.pair_map); rel(h.pairs); rel(h.c2d); rel(h.c2f); rel(h.p2);
    rel(h.t3); rel(h.c3d); rel(h.c3f); rel(h.p3);
    rel(h.t4); rel(h.c4d); rel(h.c4f); rel(h.p4);
    rel(h.fr3); rel(h.fe3d); rel(h.fe3f);
    rel(h.fr4); rel(h.fe4d); rel(h.fe4f);
    rel(h.pt3); rel(h.pt4);
    rel(h.tc3);
    rel(h.tc4);
    rel(h.t2rec); rel(h.tab2r); rel(h.tab2c);
    rel(h.t3rec); rel(h.tab3r); rel(h.tab3v);
    // this set's cluster buckets follow those of the sets loaded before it
    int nt3 = h.ntypes * h.ntypes * h.ntypes;
    h.bk3 = nbk3_;
    h.bk4 = nbk4_;
    if (h.o3 > 0) nbk3_ += nt3;
    if (h.o4 > 0) nbk4_ += nt3 * h.ntypes;
    ps.view = h;
    sets_.push_back(std::move(ps));
    std::vector<DevParamSet> all;
    for (auto& s : sets_) all.push_back(s.view);
    drop_graph();
    e = dsets_.reserve(all.size());
    if (e == cudaSuccess) e = cudaMemcpy(dsets_.p, all.data(), all.size() * sizeof(DevParamSet), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        err = std::string("CUDA error uploading parameter table: ") + cudaGetErrorString(e);
        return kErrCuda;
    }
    return (int)sets_.size() - 1;
}

Status Engine::stage(const std::vector<SystemSpec>& sys, std::string& err) {
    Status st = init_device(err);
    if (st != kOk) return st;
    if (sys.empty()) {
        err = "empty batch";
        return kErrInput;
    }
    CK_TRY(cudaStreamSynchronize(stream_));   // pinned staging may still feed a previous launch
    const int S = (int)sys.size();
    hsys_.assign(S, SysDesc());
    vols_.assign(S, 0.0);
    long long in_off = 0, atom_off = 0, ghost_off = 0, bin_off = 0;
    int stride3 = 0, stride4 = 0;
    bool fact3 = factored, fact4 = factored;
    bool pc3 = pair_cache, pc4 = pair_cache;
    int rf3 = 0, rf4 = 0;
    bool tc3 = precision == kMixed, tc4 = precision == kMixed;
    int r4_lo = 1 << 30;   // the 4-body tensor-core kernel needs one R over the batch's sets
    bool enum_serial = false;
    double n2_est = 0.0, n3_est = 0.0, n4_est = 0.0;
    for (int s = 0; s < S; s++) {
        const SystemSpec& in = sys[s];
        if (in.pset < 0 || in.pset >= (int)sets_.size()) {
            err = "configuration " + std::to_string(s) + ": parameter set not loaded";
            return kErrState;
        }
        const HostParams& P = *sets_[in.pset].host;
        if (P.tab2 || P.tab3) {
            // the reference evaluates tabulated terms only in its LAMMPS pair
            // style; its serial interface has no coefficients to expand for them
            err = "tabulated parameter sets are evaluated on a neighbour list (ck_nl_compute) or per cluster "
                  "(chimesFF::compute_2B_tab / compute_3B_tab), not by the serial interface";
            return kErrParam;
        }
        SysDesc& d = hsys_[s];
        std::memset(&d, 0, sizeof(d));
        std::string gerr;
        st = system_geometry(&in.cell[0], &in.cell[3], &in.cell[6], in.n, in.small, P.max_cut2(), P.max_cut3(),
                             P.max_cut4(), P.o3 > 0, P.o4 > 0, d, vols_[s], gerr);
        if (st != kOk) {
            err = (S > 1 ? "configuration " + std::to_string(s) + ": " : std::string()) + gerr;
            return st;
        }
        for (int a = 0; a < in.n; a++) {
            if (in.types[a] < 0 || in.types[a] >= P.ntypes) {
                err = "atom type index out of range for the parameter set";
                return kErrInput;
            }
            if (!std::isfinite(in.pos[3 * a]) || !std::isfinite(in.pos[3 * a + 1]) ||
                !std::isfinite(in.pos[3 * a + 2])) {
                err = "atom coordinates must be finite";
                return kErrInput;
            }
        }
        d.pset = in.pset;
        if (d.has3 && d.has4 && d.c4 > d.c3) enum_serial = true;
        d.in_off = in_off; d.atom_off = atom_off; d.ghost_off = ghost_off; d.bin_off = bin_off;
        in_off += in.n;
        atom_off += d.n_atoms;
        ghost_off += (long long)d.n_atoms * d.gstride;
        bin_off += d.bin_cap;
        stride3 = std::max(stride3, P.o3 > 0 ? P.o3 + 1 : 0);
        stride4 = std::max(stride4, P.o4 > 0 ? P.o4 + 1 : 0);
        const DevParamSet& V = sets_[in.pset].view;
        if (P.o3 > 0) {
            fact3 = fact3 && V.R3 > 0;
            rf3 = std::max(rf3, V.R3);
            pc3 = pc3 && V.pt3;
            tc3 = tc3 && V.tc3 != nullptr;
        }
        if (P.o4 > 0) {
            fact4 = fact4 && V.R4 > 0;
            rf4 = std::max(rf4, V.R4);
            r4_lo = std::min(r4_lo, V.R4);
            pc4 = pc4 && V.pt4;
            tc4 = tc4 && V.tc4 != nullptr;
        }
        // list-size estimates for the first capacity guess
        const double rho = d.n_atoms / (vols_[s] > 0 ? vols_[s] : 1.0);
        const double m = rho * 4.18879 * d.search * d.search * d.search;
        n2_est += d.n_atoms * (0.55 * m + 4);
        if (d.has3) n3_est += d.n_atoms * (0.3 * m * m * std::pow(d.c3 / d.search, 6.0) + 4);
        if (d.has4) n4_est += d.n_atoms * (0.1 * m * m * m * std::pow(d.c4 / d.search, 9.0) + 4);
    }
    if (ghost_off > 2000000000LL) {
        err = "batch exceeds 2^31 ghost slots";
        return kErrInput;
    }
    tuning.stride3 = stride3;
    tuning.stride4 = stride4;
    tuning.fact3 = fact3 && rf3 > 0 && tuning.want_fact3 ? 1 : 0;
    tuning.fact4 = fact4 && rf4 > 0 && tuning.want_fact4 ? 1 : 0;
    avail_fact3_ = fact3 && rf3 > 0;
    avail_fact4_ = fact4 && rf4 > 0;
    avail_tc3_ = avail_fact3_ && tc3 && tc3_supported(rf3);
    tuning.tc3 = tuning.fact3 && avail_tc3_ && tuning.want_tc3 ? 1 : 0;
    avail_tc4_ = avail_fact4_ && tc4 && r4_lo == rf4 && tc4_supported(rf4);
    tuning.tc4 = tuning.fact4 && avail_tc4_ && tuning.want_tc4 ? 1 : 0;
    // the pair-table cache needs the enumeration that records entry indices;
    // it pays for itself while its tables stay near L2 (measured: ~10% on the
    // 3-body kernel for 25k list entries, nothing for 11M), so large batches
    // compute every pair in the cluster kernel
    // The tensor-core 3-body kernel reads its ij and ik tables from the cache
    // at every size: there the cache replaces FP64 work (geometry and Morse
    // exponential of two of the three pairs, the kernel's bound) with loads
    // that stay far below the memory bandwidth.
    const bool pc_size = n2_est <= 2.0e6;
    pc_small_ = pc_size;
    avail_pc3_ = avail_fact3_ && pc3 && !enum_serial && (pc_size || avail_tc3_);
    avail_pc4_ = avail_fact4_ && pc4 && !enum_serial && pc_size;
    tuning.rf3 = rf3;
    tuning.rf4 = rf4;
    V_ = BatchView();
    V_.n_sys = S;
    V_.n_in_total = in_off;
    V_.n_atoms_total = atom_off;
    V_.n_ghost_total = ghost_off;
    V_.n_bins_total = bin_off;
    enum_serial_ = enum_serial;
    n2_cap_ = std::max(n2_cap_, (long long)n2_est + 1024);
    n3_cap_ = std::max(n3_cap_, (long long)n3_est + 1024);
    n4_cap_ = std::max(n4_cap_, (long long)n4_est + 1024);

    CK_TRY(d_sys_.reserve(S));
    CK_TRY(d_in_pos_.reserve(3 * in_off));
    CK_TRY(d_in_type_.reserve(in_off));
    CK_TRY(d_atom_sys_.reserve(atom_off));
    CK_TRY(d_atom_type_.reserve(atom_off));
    CK_TRY(d_atom_orig_.reserve(atom_off));
    CK_TRY(d_atom_self_.reserve(atom_off));
    CK_TRY(d_ghost_id_.reserve(ghost_off));
    CK_TRY(d_ghost_xf_.reserve(3 * ghost_off));
    CK_TRY(d_ghost_parent_.reserve(ghost_off));
    CK_TRY(d_ghost_bin_.reserve(ghost_off));
    CK_TRY(d_ghost_fs_.reserve(3 * ghost_off));
    CK_TRY(d_ghost_xn_.reserve(3 * ghost_off));
    CK_TRY(d_ghost_fn_.reserve(3 * ghost_off));
    CK_TRY(d_bin_items_.reserve(ghost_off));
    CK_TRY(d_bin_xp_.reserve(4 * ghost_off));
    CK_TRY(d_minmax_.reserve(6 * S));
    CK_TRY(d_bin_count_.reserve(bin_off));
    CK_TRY(d_bin_fill_.reserve(bin_off));
    CK_TRY(d_bin_start_.reserve(bin_off + 1));
    CK_TRY(d_l2_count_.reserve(atom_off));
    CK_TRY(d_l2_off_.reserve(atom_off + 1));
    CK_TRY(d_force_.reserve(3 * in_off));
    CK_TRY(d_ev_.reserve(8 * S));
    CK_TRY(h_in_pos_.reserve(3 * in_off));
    CK_TRY(h_in_type_.reserve(in_off));
    CK_TRY(h_force_.reserve(3 * in_off));
    CK_TRY(h_ev_.reserve(8 * S));
    st = ensure_lists(err);
    if (st != kOk) return st;

    for (int s = 0; s < S; s++) {
        const SystemSpec& in = sys[s];
        std::memcpy(h_in_pos_.p + 3 * hsys_[s].in_off, in.pos, sizeof(double) * 3 * in.n);
        std::memcpy(h_in_type_.p + hsys_[s].in_off, in.types, sizeof(int) * in.n);
    }
    CK_TRY(cudaMemcpyAsync(d_sys_.p, hsys_.data(), sizeof(SysDesc) * S, cudaMemcpyHostToDevice, stream_));
    CK_TRY(cudaMemcpyAsync(d_in_pos_.p, h_in_pos_.p, sizeof(double) * 3 * in_off, cudaMemcpyHostToDevice, stream_));
    CK_TRY(cudaMemcpyAsync(d_in_type_.p, h_in_type_.p, sizeof(int) * in_off, cudaMemcpyHostToDevice, stream_));
    staged_ = true;
    return kOk;
}

Status Engine::ensure_lists(std::string& err) {
    CK_TRY(d_l2_ghost_.reserve(n2_cap_));
    CK_TRY(d_l2_owner_.reserve(n2_cap_));
    CK_TRY(d_l2_dist_.reserve(n2_cap_));
    CK_TRY(d_l2_vec_.reserve(4 * n2_cap_));
    CK_TRY(d_e_cnt3_.reserve(n2_cap_));
    CK_TRY(d_e_cnt4_.reserve(n2_cap_));
    CK_TRY(d_e_off3_.reserve(n2_cap_ + 1));
    CK_TRY(d_e_off4_.reserve(n2_cap_ + 1));
    CK_TRY(d_c3_.reserve(3 * n3_cap_));
    CK_TRY(d_c4_.reserve(4 * n4_cap_));
    // buckets pad each (set, tuple) to 32 slots (3-body: 128 for the tensor-core form)
    const long long p3cap = nbk3_ > 0 ? n3_cap_ + 128LL * nbk3_ : 0;
    const long long p4cap = nbk4_ > 0 ? n4_cap_ + 32LL * nbk4_ : 0;
    CK_TRY(d_perm3_.reserve(std::max(1LL, p3cap)));
    CK_TRY(d_perm4_.reserve(std::max(1LL, p4cap)));
    CK_TRY(d_bk_count_.reserve(nbk3_ + nbk4_ + 1));
    CK_TRY(d_bk_fill_.reserve(nbk3_ + nbk4_ + 1));
    CK_TRY(d_bk_start_.reserve(nbk3_ + nbk4_ + 2));
    if (avail_pc3_) {
        CK_TRY(d_c3e_.reserve(2 * n3_cap_));
        CK_TRY(d_pcd3_.reserve(8 * n2_cap_));
        CK_TRY(d_pct3_.reserve((long long)sizeof(double) * 2 * tuning.rf3 * n2_cap_));
    }
    if (avail_pc4_) {
        CK_TRY(d_c4e_.reserve(3 * n4_cap_));
        CK_TRY(d_pcd4_.reserve(8 * n2_cap_));
        CK_TRY(d_pct4_.reserve((long long)sizeof(double) * 2 * tuning.rf4 * n2_cap_));
    }
    long long scan_n = std::max(std::max(V_.n_bins_total, V_.n_atoms_total), n2_cap_);
    CK_TRY(d_scan_tmp_.reserve(scan_tmp_bytes(scan_n)));
    BatchView& B = V_;
    B.sys = d_sys_.p;
    B.psets = dsets_.p;
    B.in_pos = d_in_pos_.p;
    B.in_type = d_in_type_.p;
    B.atom_sys = d_atom_sys_.p; B.atom_type = d_atom_type_.p; B.atom_orig = d_atom_orig_.p;
    B.atom_self = d_atom_self_.p;
    B.ghost_id = d_ghost_id_.p;
    B.ghost_xf = d_ghost_xf_.p;
    B.ghost_parent = d_ghost_parent_.p;
    B.ghost_fs = d_ghost_fs_.p; B.ghost_xn = d_ghost_xn_.p; B.ghost_fn = d_ghost_fn_.p;
    B.minmax = d_minmax_.p;
    B.ghost_bin = d_ghost_bin_.p;
    B.bin_count = d_bin_count_.p; B.bin_start = d_bin_start_.p; B.bin_fill = d_bin_fill_.p;
    B.bin_items = d_bin_items_.p;
    B.bin_xp = d_bin_xp_.p;
    B.l2_count = d_l2_count_.p; B.l2_off = d_l2_off_.p; B.l2_ghost = d_l2_ghost_.p; B.l2_dist = d_l2_dist_.p;
    B.l2_vec = d_l2_vec_.p;
    B.n2_cap = n2_cap_;
    B.e_cnt3 = d_e_cnt3_.p; B.e_cnt4 = d_e_cnt4_.p; B.e_off3 = d_e_off3_.p; B.e_off4 = d_e_off4_.p;
    B.c3 = d_c3_.p; B.c4 = d_c4_.p;
    B.n3_cap = n3_cap_; B.n4_cap = n4_cap_;
    B.force = d_force_.p; B.ev = d_ev_.p; B.flags = d_flags_.p; B.queue = d_queue_.p;
    B.enum_serial = enum_serial_ ? 1 : 0;
    B.c3e = avail_pc3_ ? d_c3e_.p : nullptr;
    B.c4e = avail_pc4_ ? d_c4e_.p : nullptr;
    B.pcd3 = d_pcd3_.p; B.pcd4 = d_pcd4_.p;
    B.pct3 = d_pct3_.p; B.pct4 = d_pct4_.p;
    B.use_pc3 = B.use_pc4 = 0;   // set per launch from the contraction form
    B.nbk3 = nbk3_; B.nbk4 = nbk4_;
    B.bk_count = d_bk_count_.p; B.bk_fill = d_bk_fill_.p; B.bk_start = d_bk_start_.p;
    B.perm3 = d_perm3_.p; B.perm4 = d_perm4_.p;
    B.perm3_cap = p3cap; B.perm4_cap = p4cap;
    return kOk;
}

// Stage events: inside a stream capture they become external event-record
// nodes of the graph (so each replay records them); outside a capture the
// external flag is refused, and a plain record is used.
static cudaError_t record_stage_event(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    if (cs == cudaStreamCaptureStatusActive) return cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
    return cudaEventRecord(ev, st);
}

// NVTX range over the enqueue of one stage: a profiler that records NVTX
// (Nsight Systems) shows the stage's kernels under its name; without one
// attached the calls return at once.
namespace {
struct NvtxRange {
    bool open = true;
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    void end() {
        if (open) nvtxRangePop();
        open = false;
    }
    ~NvtxRange() { end(); }
};
}  // namespace

Status Engine::enqueue(std::string& err) {
    BatchView B = V_;
    B.use_pc3 = avail_pc3_ && tuning.fact3 && (tuning.tc3 || pc_small_) ? 1 : 0;
    B.bk_pad3 = tuning.tc3 ? 128 : 32;
    B.use_pc4 = avail_pc4_ && tuning.fact4 && !tuning.tc4 ? 1 : 0;
    cudaStream_t st = stream_;
    const long long k0 = launch_counter();
    if (profile) {
        for (auto& e : ev_)
            if (!e) CK_TRY(cudaEventCreate(&e));
        CK_TRY(record_stage_event(ev_[0], st));
    }
    NvtxRange lists_range("chimes: list build");
    CK_TRY(cudaMemsetAsync(B.bin_count, 0, sizeof(int) * B.n_bins_total, st));
    CK_TRY(cudaMemsetAsync(B.bin_fill, 0, sizeof(int) * B.n_bins_total, st));
    launch_reset(B, st);
    launch_atoms(B, st);
    launch_ghosts(B, st);
    launch_bin_setup(B, st);
    launch_bin_count(B, st);
    exclusive_scan(B.bin_count, B.bin_start, B.n_bins_total, d_scan_tmp_.p, st);
    launch_bin_scatter(B, st);
    launch_bin_sort(B, st);
    launch_l2(B, d_l2_owner_.p, false, st);
    exclusive_scan(B.l2_count, B.l2_off, B.n_atoms_total, d_scan_tmp_.p, st);
    launch_l2(B, d_l2_owner_.p, true, st);
    ForceLaunch L = tuning;
    L.precision = precision;
    // Concurrent form: the second stream takes 1B+2B (it needs only the pair
    // lists) while the first enumerates the clusters, then the 4-body branch
    // while the first runs the 3-body one; both join before the copies out.
    // Not while profiling (the stage events time the stages one after another).
    const bool conc = !profile && concurrent;
    if (conc) {
        CK_TRY(cudaEventRecord(fork_, st));
        CK_TRY(cudaStreamWaitEvent(stream2_, fork_, 0));
        NvtxRange r("chimes: 1B+2B");
        launch_force2(B, d_l2_owner_.p, L, stream2_);
    }
    launch_enum(B, d_l2_owner_.p, false, st);
    exclusive_scan2(B.e_cnt3, B.e_off3, B.e_cnt4, B.e_off4, B.n2_cap, d_scan_tmp_.p, st);
    launch_enum(B, d_l2_owner_.p, true, st);
    launch_check(B, st);
    lists_range.end();
    if (profile) CK_TRY(record_stage_event(ev_[1], st));
    if ((L.stride3 > 0 && L.fact3) || (L.stride4 > 0 && L.fact4)) {
        CK_TRY(cudaMemsetAsync(B.bk_count, 0, sizeof(int) * (B.nbk3 + B.nbk4), st));
        CK_TRY(cudaMemsetAsync(B.bk_fill, 0, sizeof(int) * (B.nbk3 + B.nbk4), st));
    }
    auto body3 = [&](cudaStream_t q) {
        if (L.stride3 <= 0) return;
        NvtxRange r("chimes: 3B");
        if (L.fact3 && L.tc3) {
            launch_pair_tables(B, d_l2_owner_.p, 3, L, q);
            launch_bucket(B, 3, q);
            launch_force3tc(B, L, q);
        } else if (L.fact3) {
            launch_pair_tables(B, d_l2_owner_.p, 3, L, q);
            launch_bucket(B, 3, q);
            launch_force3f(B, L, q);
        } else {
            launch_force3(B, L, q);
        }
    };
    auto body4 = [&](cudaStream_t q) {
        if (L.stride4 <= 0) return;
        NvtxRange r("chimes: 4B");
        if (L.fact4 && L.tc4) {
            launch_bucket(B, 4, q);
            launch_force4tc(B, L, q);
        } else if (L.fact4) {
            launch_pair_tables(B, d_l2_owner_.p, 4, L, q);
            launch_bucket(B, 4, q);
            launch_force4f(B, L, q);
        } else {
            launch_force4(B, L, q);
        }
    };
    if (conc) {
        // separate work queues; forces and energies meet in atomics; captured
        // as parallel graph branches
        CK_TRY(cudaEventRecord(fork2_, st));
        CK_TRY(cudaStreamWaitEvent(stream2_, fork2_, 0));
        body4(stream2_);
        CK_TRY(cudaEventRecord(join_, stream2_));
        body3(st);
        CK_TRY(cudaStreamWaitEvent(st, join_, 0));
    } else {
        {
            NvtxRange r("chimes: 1B+2B");
            launch_force2(B, d_l2_owner_.p, L, st);
        }
        if (profile) CK_TRY(record_stage_event(ev_[2], st));
        body3(st);
        if (profile) CK_TRY(record_stage_event(ev_[3], st));
        body4(st);
    }
    if (profile) CK_TRY(record_stage_event(ev_[4], st));
    ev_recorded_ = profile;
    kernels_per_launch = (int)(launch_counter() - k0);
    CK_TRY(cudaMemcpyAsync(h_force_.p, B.force, sizeof(double) * 3 * B.n_in_total, cudaMemcpyDeviceToHost, st));
    CK_TRY(cudaMemcpyAsync(h_ev_.p, B.ev, sizeof(double) * 8 * B.n_sys, cudaMemcpyDeviceToHost, st));
    CK_TRY(cudaMemcpyAsync(h_flags_.p, B.flags, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
    CK_TRY(cudaMemcpyAsync(h_counts_.p + 0, B.l2_off + B.n_atoms_total, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK_TRY(cudaMemcpyAsync(h_counts_.p + 1, B.e_off3 + B.n2_cap, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK_TRY(cudaMemcpyAsync(h_counts_.p + 2, B.e_off4 + B.n2_cap, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK_TRY(cudaGetLastError());
    return kOk;
}

Status Engine::read_stage_times(std::string& err) {
    if (!ev_recorded_) return kOk;
    CK_TRY(cudaEventSynchronize(ev_[4]));
    for (int k = 0; k < 4; k++) {
        float ms = 0.f;
        CK_TRY(cudaEventElapsedTime(&ms, ev_[k], ev_[k + 1]));
        stage_ms[k] += ms;
    }
    stage_launches++;
    return kOk;
}

Status Engine::launch(std::string& err) {
    if (!staged_) {
        err = "launch before stage";
        return kErrState;
    }
    if (!use_graph) return enqueue(err);
    std::vector<long long> key = {(long long)V_.n_sys, V_.n_in_total, V_.n_atoms_total, V_.n_ghost_total,
                                  V_.n_bins_total, n2_cap_, n3_cap_, n4_cap_, precision, tuning.tpc3, tuning.tpc4,
                                  tuning.stride3, tuning.stride4, tuning.blocks_per_sm, profile ? 1 : 0,
                                  tuning.fact3, tuning.fact4, tuning.rf3, tuning.rf4, tuning.ftpc3, tuning.ftpc4,
                                  tuning.fbps3, tuning.fbps4, nbk3_, nbk4_, concurrent ? 1 : 0, tuning.noy3,
                                  tuning.tc3, tuning.tc4};
    for (const void* p : {(const void*)V_.sys, (const void*)V_.in_pos, (const void*)V_.ghost_fs,
                          (const void*)V_.bin_items, (const void*)V_.l2_ghost, (const void*)V_.c3,
                          (const void*)V_.c4, (const void*)V_.force, (const void*)d_scan_tmp_.p,
                          (const void*)h_force_.p, (const void*)h_ev_.p, (const void*)V_.bin_count,
                          (const void*)V_.e_off3, (const void*)V_.psets, (const void*)V_.perm3,
                          (const void*)V_.perm4, (const void*)V_.bk_count, (const void*)V_.bk_fill,
                          (const void*)V_.bk_start, (const void*)V_.c3e, (const void*)V_.c4e,
                          (const void*)V_.pcd3, (const void*)V_.pcd4, (const void*)V_.pct3, (const void*)V_.pct4})
        key.push_back((long long)(uintptr_t)p);
    if (key != graph_key_) {
        // capture only when the same shape launches twice in a row: a batch
        // seen once (a one-off call, or sizes that change every call) runs
        // stream-ordered without paying for a capture
        if (key != seen_key_) {
            seen_key_ = key;
            return enqueue(err);
        }
        drop_graph();
        CK_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        Status st = enqueue(err);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(stream_, &g);
        if (st != kOk) { if (g) cudaGraphDestroy(g); return st; }
        if (e != cudaSuccess) {
            err = std::string("CUDA graph capture failed: ") + cudaGetErrorString(e);
            return kErrCuda;
        }
        graph_ = g;
        CK_TRY(cudaGraphInstantiate(&graph_exec_, graph_, 0));
        graph_key_ = key;
    }
    CK_TRY(cudaGraphLaunch(graph_exec_, stream_));
    return kOk;
}

Status Engine::collect(double* force_out, std::vector<SystemResult>& res, std::string& err) {
    CK_TRY(cudaStreamSynchronize(stream_));
    const int* f = h_flags_.p;
    const long long* c = h_counts_.p;
    last.n2 = c[0]; last.n3 = c[1]; last.n4 = c[2];
    last.n_atoms = V_.n_atoms_total;
    last.n_ghost = V_.n_ghost_total;
    if (f[0] & 1) {
        err = "bin grid larger than its reserved capacity";
        return kErrGeometry;
    }
    if ((f[0] & (2 | 4 | 8)) || c[0] > n2_cap_ || c[1] > n3_cap_ || c[2] > n4_cap_) {
        if (c[0] > n2_cap_) n2_cap_ = c[0] + c[0] / 8 + 1024;
        else {
            if (c[1] > n3_cap_) n3_cap_ = c[1] + c[1] / 8 + 1024;
            if (c[2] > n4_cap_) n4_cap_ = c[2] + c[2] / 8 + 1024;
        }
        err = "list capacity exceeded";
        return kErrCapacity;
    }
    if (f[7] & 1) {
        err = "tensor-core contraction: a bounded wait for the matrix units expired";
        return kErrTimeout;
    }
    if (f[7] & 2) {
        err = "checked build: an index outside its array was found and the access skipped";
        return kErrState;
    }
    if (f[1]) {
        err = f[1] == 1 ? "negative bin computed (check box lengths and atom coordinates)"
                        : f[1] == 3 ? "bad bin computed for a real atom (check box lengths and atom coordinates)"
                                    : "bin index out of range";
        return kErrGeometry;
    }
    last.badness = f[2];
    last.penalty_hits = f[3];
    last.below_rin = f[4];
    res.assign(V_.n_sys, SystemResult());
    for (int s = 0; s < V_.n_sys; s++) {
        const double* ev = h_ev_.p + 8 * s;
        SystemResult& r = res[s];
        r.n_rep = hsys_[s].n_rep;
        r.energy = ev[0] / std::pow(hsys_[s].n_rep + 1.0, 3.0);
        for (int k = 0; k < 6; k++) r.virial[k] = ev[1 + k];
        r.vol = vols_[s];
    }
    if (force_out) std::memcpy(force_out, h_force_.p, sizeof(double) * 3 * V_.n_in_total);
    return kOk;
}

Status Engine::run(const std::vector<SystemSpec>& sys, double* force_out, std::vector<SystemResult>& res,
                   std::string& err) {
    Status st = stage(sys, err);
    if (st != kOk) return st;
    for (int attempt = 0; attempt < 6; attempt++) {
        st = launch(err);
        if (st != kOk) return st;
        st = collect(force_out, res, err);
        if (st != kErrCapacity) return st;
        st = ensure_lists(err);
        if (st != kOk) return st;
    }
    err = "list capacity did not converge";
    return kErrCapacity;
}

std::string Engine::tune_key() const {
    std::string k = "p" + std::to_string(precision) + (factored ? "f" : "c");
    std::vector<int> seen;
    for (const SysDesc& d : hsys_)
        if (std::find(seen.begin(), seen.end(), d.pset) == seen.end()) seen.push_back(d.pset);
    for (int s : seen) {
        const HostParams& P = *sets_[s].host;
        k += "|" + std::to_string(P.ntypes) + ":" + std::to_string(P.o2) + "/" + std::to_string(P.o3) + "/" +
             std::to_string(P.o4);
    }
    auto lg = [](long long v) { int b = 0; while (v > 1) { v >>= 1; b++; } return b; };
    k += "|a" + std::to_string(lg(V_.n_atoms_total)) + "|s" + std::to_string(lg(V_.n_sys));
    return k;
}

Status Engine::autotune(int* chosen, std::string& err) {
    if (!staged_) {
        err = "autotune needs a staged batch";
        return kErrState;
    }
    const std::string key = tune_key();
    auto report = [&]() {
        if (chosen) {
            chosen[0] = tuning.fact3 ? tuning.ftpc3 : tuning.tpc3;
            chosen[1] = tuning.fact4 ? tuning.ftpc4 : tuning.tpc4;
            chosen[2] = tuning.blocks_per_sm;
        }
    };
    for (auto& kv : tune_cache_)
        if (kv.first == key) {
            tuning.tpc3 = kv.second.tpc3;
            tuning.tpc4 = kv.second.tpc4;
            tuning.blocks_per_sm = kv.second.blocks_per_sm;
            tuning.ftpc3 = kv.second.ftpc3;
            tuning.ftpc4 = kv.second.ftpc4;
            tuning.fbps3 = kv.second.fbps3;
            tuning.fbps4 = kv.second.fbps4;
            tuning.want_fact3 = kv.second.want_fact3;
            tuning.want_fact4 = kv.second.want_fact4;
            tuning.noy3 = kv.second.noy3;
            tuning.want_tc3 = kv.second.want_tc3;
            tuning.want_tc4 = kv.second.want_tc4;
            tuning.fact3 = avail_fact3_ && tuning.want_fact3;
            tuning.fact4 = avail_fact4_ && tuning.want_fact4;
            tuning.tc3 = tuning.fact3 && avail_tc3_ && tuning.want_tc3;
            tuning.tc4 = tuning.fact4 && avail_tc4_ && tuning.want_tc4;
            report();
            return kOk;
        }
    const bool save_profile = profile, save_graph = use_graph;
    const ForceLaunch save_tuning = tuning;
    profile = true;
    use_graph = false;
    std::vector<SystemResult> res;
    auto run_once = [&](double& ms3, double& ms4) -> Status {
        for (int attempt = 0; attempt < 6; attempt++) {
            for (double& v : stage_ms) v = 0.0;
            stage_launches = 0;
            Status st = launch(err);
            if (st != kOk) return st;
            st = collect(nullptr, res, err);
            if (st == kErrCapacity) {
                st = ensure_lists(err);
                if (st != kOk) return st;
                continue;
            }
            if (st != kOk) return st;
            st = read_stage_times(err);
            if (st != kOk) return st;
            ms3 = stage_ms[2];
            ms4 = stage_ms[3];
            return kOk;
        }
        err = "list capacity did not converge";
        return kErrCapacity;
    };
    double a, b;
    Status st = run_once(a, b);   // warm-up and list sizing
    const bool do3 = tuning.stride3 > 0, do4 = tuning.stride4 > 0;
    // candidates per body order: factored kernels (1, 2, 4 lanes per cluster)
    // where the tables exist, then the per-coefficient kernels (1..32 lanes)
    // (3-body factored also without its Y table).  The factored forms differ
    // in shared memory per cluster, so each is tried at 8 and at up to 16
    // resident one-warp blocks per SM (capped by its occupancy); the per-SM
    // count is refined below.
    // (in the mixed form also the tensor-core contractions)
    struct Cand { int fact, tpc, noy, fbps, tc; };
    auto cands = [](bool can_fact, bool with_noy, bool with_tc) {
        std::vector<Cand> v;
        if (with_tc) v.push_back({1, 1, 0, 0, 1});
        if (can_fact)
            for (int t : {1, 2, 4})
                for (int nf : {0, 1}) {
                    if (nf && !with_noy) continue;
                    v.push_back({1, t, nf, 8, 0});
                    v.push_back({1, t, nf, 16, 0});
                }
        for (int t : {1, 2, 4, 8, 16, 32}) v.push_back({0, t, 0, 0, 0});
        return v;
    };
    const std::vector<Cand> c3 = cands(avail_fact3_, true, avail_tc3_), c4 = cands(avail_fact4_, false, avail_tc4_);
    auto apply = [&](int nb, const Cand& c) {
        if (nb == 3) {
            tuning.fact3 = c.fact;
            (c.fact ? tuning.ftpc3 : tuning.tpc3) = c.tpc;
            tuning.noy3 = c.noy;
            tuning.tc3 = c.tc;
            if (c.fbps > 0) tuning.fbps3 = c.fbps;
        } else {
            tuning.fact4 = c.fact;
            (c.fact ? tuning.ftpc4 : tuning.tpc4) = c.tpc;
            tuning.tc4 = c.tc;
            if (c.fbps > 0) tuning.fbps4 = c.fbps;
        }
    };
    double best3 = 1e300, best4 = 1e300;
    Cand b3 = {tuning.fact3, tuning.fact3 ? tuning.ftpc3 : tuning.tpc3, tuning.noy3, tuning.fbps3, tuning.tc3};
    Cand b4 = {tuning.fact4, tuning.fact4 ? tuning.ftpc4 : tuning.tpc4, 0, tuning.fbps4, tuning.tc4};
    const size_t nc = std::max(c3.size(), c4.size());
    for (size_t i = 0; i < nc && st == kOk; i++) {
        const bool need3 = do3 && i < c3.size(), need4 = do4 && i < c4.size();
        if (!need3 && !need4) break;
        apply(3, c3[std::min(i, c3.size() - 1)]);
        apply(4, c4[std::min(i, c4.size() - 1)]);
        double m3 = 1e300, m4 = 1e300;
        for (int rep = 0; rep < 2 && st == kOk; rep++) {
            st = run_once(a, b);
            m3 = std::min(m3, a);
            m4 = std::min(m4, b);
        }
        if (need3 && m3 < best3) { best3 = m3; b3 = c3[i]; }
        if (need4 && m4 < best4) { best4 = m4; b4 = c4[i]; }
    }
    apply(3, b3);
    apply(4, b4);
    tuning.want_fact3 = b3.fact;
    tuning.want_fact4 = b4.fact;
    tuning.want_tc3 = b3.tc;
    tuning.want_tc4 = b4.tc;
    // (the tensor-core forms' occupancy is fixed by their shared memory)
    const bool f3 = tuning.fact3 != 0 && !tuning.tc3, f4 = tuning.fact4 != 0 && !tuning.tc4;
    // resident blocks per SM: 4-warp blocks for the per-coefficient kernels,
    // one-warp blocks for the factored ones (capped by their occupancy)
    const int bps[] = {1, 2, 4, 8};
    const int fbps[] = {2, 4, 8, 16};
    double bestb = 1e300, bestf3 = 1e300, bestf4 = 1e300;
    int bb = tuning.blocks_per_sm, bf3 = tuning.fbps3, bf4 = tuning.fbps4;
    for (int i = 0; i < 4 && st == kOk; i++) {
        tuning.blocks_per_sm = bps[i];
        tuning.fbps3 = tuning.fbps4 = fbps[i];
        double m3 = 1e300, m4 = 1e300;
        for (int rep = 0; rep < 2 && st == kOk; rep++) {
            st = run_once(a, b);
            m3 = std::min(m3, a);
            m4 = std::min(m4, b);
        }
        const double mold = (do3 && !f3 ? m3 : 0.0) + (do4 && !f4 ? m4 : 0.0);
        if (mold < bestb) { bestb = mold; bb = bps[i]; }
        if (f3 && m3 < bestf3) { bestf3 = m3; bf3 = fbps[i]; }
        if (f4 && m4 < bestf4) { bestf4 = m4; bf4 = fbps[i]; }
    }
    tuning.blocks_per_sm = bb;
    tuning.fbps3 = bf3;
    tuning.fbps4 = bf4;
    profile = save_profile;
    use_graph = save_graph;
    for (double& v : stage_ms) v = 0.0;
    stage_launches = 0;
    if (st != kOk) {
        tuning = save_tuning;
        return st;
    }
    tune_cache_.push_back({key, tuning});
    report();
    return kOk;
}

Status Engine::compute_clusters(int slot, int nbody, int n, const double* dx, const double* dr, const int* typ,
                                double* force, double* stress, double* energy, double* fscal, int* status,
                                std::string& err, bool tab) {
    Status st = init_device(err);
    if (st != kOk) return st;
    if (slot < 0 || slot >= (int)sets_.size()) {
        err = "parameters not initialised";
        return kErrState;
    }
    if (nbody < 2 || nbody > 4) {
        err = "clusters have 2, 3 or 4 atoms";
        return kErrInput;
    }
    if (n <= 0) return kOk;
    const HostParams& P = *sets_[slot].host;
    if ((nbody == 3 && P.o3 <= 0) || (nbody == 4 && P.o4 <= 0)) {
        err = "the parameter set has no " + std::to_string(nbody) + "-body terms";
        return kErrInput;
    }
    const bool tabbed = (nbody == 2 && P.tab2) || (nbody == 3 && P.tab3);
    if (tab && !tabbed) {
        err = "the parameter set's " + std::to_string(nbody) + "-body terms are not tabulated";
        return kErrInput;
    }
    if (!tab && tabbed) {
        err = "the parameter set's " + std::to_string(nbody) + "-body terms are tabulated (use compute_" +
              std::to_string(nbody) + "B_tab)";
        return kErrInput;
    }
    for (long long i = 0; i < (long long)n * nbody; i++)
        if (typ[i] < 0 || typ[i] >= P.ntypes) {
            err = "atom type index out of range for the parameter set";
            return kErrInput;
        }
    const int np = nbody * (nbody - 1) / 2;
    const size_t nd_in = (size_t)n * np * 4;                       // dx + dr
    const size_t nd_out = (size_t)n * (3 * nbody + 6 + 1 + np);    // force, stress, energy, fscal
    CK_TRY(d_dir_d_.reserve(nd_in + nd_out));
    CK_TRY(d_dir_i_.reserve((size_t)n * (nbody + 1)));
    double* ddx = d_dir_d_.p;
    double* ddr = ddx + (size_t)n * np;
    double* dforce = ddr + (size_t)n * np * 3;
    double* dstress = dforce + (size_t)n * 3 * nbody;
    double* denergy = dstress + (size_t)n * 6;
    double* dfscal = denergy + n;
    int* dtyp = d_dir_i_.p;
    int* dstatus = dtyp + (size_t)n * nbody;
    CK_TRY(cudaMemcpyAsync(ddx, dx, sizeof(double) * n * np, cudaMemcpyHostToDevice, stream_));
    CK_TRY(cudaMemcpyAsync(ddr, dr, sizeof(double) * n * np * 3, cudaMemcpyHostToDevice, stream_));
    CK_TRY(cudaMemcpyAsync(dtyp, typ, sizeof(int) * n * nbody, cudaMemcpyHostToDevice, stream_));
    launch_direct(dsets_.p + slot, nbody, nbody == 2 ? P.o2 : nbody == 3 ? P.o3 : P.o4, n, ddx, ddr, dtyp, dforce,
                  dstress, denergy, dfscal, dstatus, stream_, tab);
    CK_TRY(cudaGetLastError());
    CK_TRY(cudaMemcpyAsync(force, dforce, sizeof(double) * n * 3 * nbody, cudaMemcpyDeviceToHost, stream_));
    CK_TRY(cudaMemcpyAsync(stress, dstress, sizeof(double) * n * 6, cudaMemcpyDeviceToHost, stream_));
    CK_TRY(cudaMemcpyAsync(energy, denergy, sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    if (fscal) CK_TRY(cudaMemcpyAsync(fscal, dfscal, sizeof(double) * n * np, cudaMemcpyDeviceToHost, stream_));
    if (status) CK_TRY(cudaMemcpyAsync(status, dstatus, sizeof(int) * n, cudaMemcpyDeviceToHost, stream_));
    CK_TRY(cudaStreamSynchronize(stream_));
    return kOk;
}

Status Engine::export_lists(std::vector<int>& l2, std::vector<int>& l3, std::vector<int>& l4, std::string& err) {
    if (!staged_) {
        err = "no evaluation to export";
        return kErrState;
    }
    CK_TRY(cudaStreamSynchronize(stream_));
    const long long n2 = last.n2, n3 = last.n3, n4 = last.n4;
    std::vector<int> g2(n2), own(n2), g3(3 * n3), g4(4 * n4), asys(V_.n_atoms_total);
    if (n2) {
        CK_TRY(cudaMemcpy(g2.data(), V_.l2_ghost, sizeof(int) * n2, cudaMemcpyDeviceToHost));
        CK_TRY(cudaMemcpy(own.data(), d_l2_owner_.p, sizeof(int) * n2, cudaMemcpyDeviceToHost));
    }
    if (n3) CK_TRY(cudaMemcpy(g3.data(), V_.c3, sizeof(int) * 3 * n3, cudaMemcpyDeviceToHost));
    if (n4) CK_TRY(cudaMemcpy(g4.data(), V_.c4, sizeof(int) * 4 * n4, cudaMemcpyDeviceToHost));
    if (V_.n_atoms_total)
        CK_TRY(cudaMemcpy(asys.data(), V_.atom_sys, sizeof(int) * V_.n_atoms_total, cudaMemcpyDeviceToHost));
    // slots -> the reference's ghost numbering within each system
    std::vector<int> gid(V_.n_ghost_total);
    if (V_.n_ghost_total)
        CK_TRY(cudaMemcpy(gid.data(), V_.ghost_id, sizeof(int) * V_.n_ghost_total, cudaMemcpyDeviceToHost));
    l2.resize(2 * n2);
    for (long long e = 0; e < n2; e++) {
        const SysDesc& d = hsys_[asys[own[e]]];
        l2[2 * e] = (int)(own[e] - d.atom_off);
        l2[2 * e + 1] = gid[g2[e]];
    }
    l3.resize(3 * n3);
    for (long long q = 0; q < 3 * n3; q++) l3[q] = gid[g3[q]];
    l4.resize(4 * n4);
    for (long long q = 0; q < 4 * n4; q++) l4[q] = gid[g4[q]];
    return kOk;
}

}  // namespace ck
