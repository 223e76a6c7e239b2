// Evaluation of one periodic configuration that allocates no device memory.
//
// Some callers cannot call cudaMalloc while they compute forces: an MD code
// or a framework that reserves the GPU's memory up front and hands out only
// its own buffers (a caching allocator, a fixed pool), or a tight step loop
// where an allocation could fail or stall the step.  For them the library
// offers ck_calculate_noalloc: the caller passes device pointers for the
// inputs and outputs, and every intermediate array of the evaluation -- ghost
// images, bin grid, neighbour and cluster lists, scan workspace, accumulators
// -- lives in one file-scope device array of fixed size (kScratchBytes, about
// 13.4 MiB), which every GPU that loads the library holds until the process
// exits.  The list-build and force kernels are the allocating path's own, in
// one fixed launch shape: the thread-per-entry cluster enumeration and the
// per-coefficient contraction (k_forcen) with the handle's tuning, never the
// bucketed factored contraction, which needs per-batch bucket arrays the
// static layout does not hold.  Because the inputs are already on the device,
// their check (type index inside the parameter set, finite coordinates) runs
// on the device too; a bad value is replaced in the scratch copy before any
// table is indexed with it and the call returns an input error.
//
// The array is shared by all calls on a device and keeps the previous call's
// contents; everything that must start at zero is cleared by each call.  Two
// calls whose work overlaps on the GPU (different streams, threads or
// handles) race on the array and corrupt each other's results.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "ck_engine.h"
#include "ck_geom.h"
#include "ck_kernels.h"

namespace ck {

namespace {

// Maximum sizes of one call (after replication of small cells).
constexpr long long kNaAtoms = 2048;      // atoms
constexpr long long kNaGhosts = 65536;    // ghost-image slots (atoms x kept images per atom)
constexpr long long kNaBins = 65536;      // bin-grid cells
constexpr long long kNaPairs = 65536;     // 2-body list entries
constexpr long long kNaTrip = 131072;     // triplets
constexpr long long kNaQuad = 65536;      // quadruplets

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte layout of the scratch array
struct Layout {
    size_t sys, minmax, ev, flags, queue, in_pos, in_type, atom_sys, atom_type, atom_orig, atom_self;
    size_t ghost_id, ghost_parent, ghost_bin, ghost_fs, ghost_xn, ghost_fn, ghost_xf, bin_items;
    size_t bin_count, bin_fill, bin_start, l2_count, l2_off;
    size_t l2_ghost, l2_owner, l2_dist, l2_vec, e_cnt3, e_cnt4, e_off3, e_off4, c3, c4, force, scan, total;
};

constexpr size_t kScanBytes = 8192;   // >= scan_tmp_bytes of the largest scan below (65536 entries)

constexpr Layout make_layout() {
    Layout L{};
    size_t o = 0;
    auto take = [&o](size_t bytes) { size_t at = o; o = align256(o + bytes); return at; };
    L.sys = take(sizeof(SysDesc));
    L.minmax = take(6 * sizeof(unsigned long long));
    L.ev = take(8 * sizeof(double));
    L.flags = take(8 * sizeof(int));
    L.queue = take(2 * sizeof(unsigned long long));
    L.in_pos = take(3 * kNaAtoms * sizeof(double));
    L.in_type = take(kNaAtoms * sizeof(int));
    L.atom_sys = take(kNaAtoms * sizeof(int));
    L.atom_type = take(kNaAtoms * sizeof(int));
    L.atom_orig = take(kNaAtoms * sizeof(int));
    L.atom_self = take(kNaAtoms * sizeof(int));
    L.ghost_id = take(kNaGhosts * sizeof(int));
    L.ghost_parent = take(kNaGhosts * sizeof(int));
    L.ghost_bin = take(kNaGhosts * sizeof(int));
    L.ghost_fs = take(3 * kNaGhosts * sizeof(double));
    L.ghost_xn = take(3 * kNaGhosts * sizeof(double));
    L.ghost_fn = take(3 * kNaGhosts * sizeof(double));
    L.ghost_xf = take(3 * kNaGhosts * sizeof(float));
    L.bin_items = take(kNaGhosts * sizeof(int));
    L.bin_count = take(kNaBins * sizeof(int));
    L.bin_fill = take(kNaBins * sizeof(int));
    L.bin_start = take((kNaBins + 1) * sizeof(long long));
    L.l2_count = take(kNaAtoms * sizeof(int));
    L.l2_off = take((kNaAtoms + 1) * sizeof(long long));
    L.l2_ghost = take(kNaPairs * sizeof(int));
    L.l2_owner = take(kNaPairs * sizeof(int));
    L.l2_dist = take(kNaPairs * sizeof(double));
    L.l2_vec = take(4 * kNaPairs * sizeof(float));
    L.e_cnt3 = take(kNaPairs * sizeof(int));
    L.e_cnt4 = take(kNaPairs * sizeof(int));
    L.e_off3 = take((kNaPairs + 1) * sizeof(long long));
    L.e_off4 = take((kNaPairs + 1) * sizeof(long long));
    L.c3 = take(3 * kNaTrip * sizeof(int));
    L.c4 = take(4 * kNaQuad * sizeof(int));
    L.force = take(3 * kNaAtoms * sizeof(double));
    L.scan = take(kScanBytes);
    L.total = o;
    return L;
}

constexpr Layout kLayout = make_layout();
constexpr size_t kScratchBytes = kLayout.total;

// The scratch array.  Host code must not use `g_noalloc_scratch` as an
// address: it is a host-side stand-in for the device symbol.  The device
// address comes from cudaGetSymbolAddress (see scratch_base).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
unsigned char* g_base[kMaxDevices] = {nullptr};
std::mutex g_base_mu;

// Once per device, with that device (`dev`, current) : the device address of the array.
Status scratch_base(int dev, unsigned char** out, std::string& err) {
    if (dev < 0 || dev >= kMaxDevices) {
        err = "no usable CUDA device";
        return kErrCuda;
    }
    std::lock_guard<std::mutex> lock(g_base_mu);
    cudaError_t e = cudaSuccess;
    if (!g_base[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress of the scratch array failed: ") + cudaGetErrorString(e);
            return kErrCuda;
        }
        g_base[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_base[dev];
    return kOk;
}

// Device-side input check (Engine::stage does the same on host arrays): a type
// index outside [0, ntypes) becomes 0 and a non-finite coordinate 0.0 in the
// scratch copies, so no later kernel indexes a table with a bad value;
// flags[6] bit 1 / bit 2 records it and the call reports an input error.
__global__ void k_noalloc_check_inputs(double* pos, int* type, int n, int ntypes, int* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int bad = 0;
    const int t = type[i];
    if (t < 0 || t >= ntypes) {
        type[i] = 0;
        bad |= 1;
    }
    for (int k = 0; k < 3; k++) {
        if (!isfinite(pos[3 * i + k])) {
            pos[3 * i + k] = 0.0;
            bad |= 2;
        }
    }
    if (bad) atomicOr(&flags[6], bad);
}

// energy / (n_rep+1)^3, forces copied out, stress = virial / volume
__global__ void k_noalloc_finish(const double* ev, const double* force, int n, double scale, double vol,
                                 double* energy_out, double* force_out, double* stress_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * n) force_out[i] = force[i];
    if (i == 0) {
        *energy_out = ev[0] * scale;
        const double v[9] = {ev[1], ev[2], ev[3], ev[2], ev[4], ev[5], ev[3], ev[5], ev[6]};
        for (int k = 0; k < 9; k++) stress_out[k] = v[k] / vol;
    }
}

}  // namespace

Status calculate_noalloc(Engine& eng, int slot, int natom, const double* d_pos, const int* d_types,
                         const double* cell, bool small, double* d_energy, double* d_force, double* d_stress,
                         cudaStream_t st, std::string& err) {
    if (scan_tmp_bytes(kNaGhosts) > kScanBytes) {   // the largest scan is no longer than kNaGhosts
        err = "ck_calculate_noalloc: scan workspace too small";
        return kErrState;
    }
    if (slot < 0 || slot >= eng.n_param_sets()) {
        err = "parameters not initialised";
        return kErrState;
    }
    if (natom <= 0 || natom > kNaAtoms) {
        err = "ck_calculate_noalloc: natom must lie in [1, " + std::to_string(kNaAtoms) + "]";
        return kErrInput;
    }
    if (!d_pos || !d_types || !d_energy || !d_force || !d_stress || !cell) {
        err = "ck_calculate_noalloc: null input or output pointer";
        return kErrInput;
    }
    const HostParams& P = eng.params(slot);
    if (P.tab2 || P.tab3) {
        err = "ck_calculate_noalloc: tabulated parameter sets are evaluated on a neighbour list only";
        return kErrParam;
    }
    SysDesc d;
    std::memset(&d, 0, sizeof(d));
    double vol = 0.0;
    Status s = system_geometry(&cell[0], &cell[3], &cell[6], natom, small, P.max_cut2(), P.max_cut3(),
                               P.max_cut4(), P.o3 > 0, P.o4 > 0, d, vol, err);
    if (s != kOk) return s;
    const long long n_ghost = (long long)d.n_atoms * d.gstride;
    if (d.n_atoms > kNaAtoms || n_ghost > kNaGhosts || d.bin_cap > kNaBins) {
        err = "ck_calculate_noalloc: configuration exceeds the static maximum (" + std::to_string(d.n_atoms) +
              " atoms, " + std::to_string(n_ghost) + " ghost slots, " + std::to_string(d.bin_cap) +
              " bins; limits " + std::to_string(kNaAtoms) + ", " + std::to_string(kNaGhosts) + ", " +
              std::to_string(kNaBins) + ")";
        return kErrInput;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != eng.device()) {
        err = "ck_calculate_noalloc: the current CUDA device (" + std::to_string(dev) +
              ") is not the one the handle's parameters were loaded on (" + std::to_string(eng.device()) + ")";
        return kErrState;
    }
    unsigned char* base = nullptr;
    s = scratch_base(dev, &base, err);
    if (s != kOk) return s;
    d.pset = slot;
    d.in_off = d.atom_off = d.ghost_off = d.bin_off = 0;

    BatchView B;
    std::memset(&B, 0, sizeof(B));
    B.enum_serial = 1;   // one thread per list entry: the enumeration this entry point was validated with
    B.n_sys = 1;
    B.n_in_total = natom;
    B.n_atoms_total = d.n_atoms;
    B.n_ghost_total = n_ghost;
    B.n_bins_total = d.bin_cap;
    B.sys = reinterpret_cast<SysDesc*>(base + kLayout.sys);
    B.psets = eng.device_params();
    B.in_pos = reinterpret_cast<double*>(base + kLayout.in_pos);
    B.in_type = reinterpret_cast<int*>(base + kLayout.in_type);
    B.atom_sys = reinterpret_cast<int*>(base + kLayout.atom_sys);
    B.atom_type = reinterpret_cast<int*>(base + kLayout.atom_type);
    B.atom_orig = reinterpret_cast<int*>(base + kLayout.atom_orig);
    B.atom_self = reinterpret_cast<int*>(base + kLayout.atom_self);
    B.ghost_id = reinterpret_cast<int*>(base + kLayout.ghost_id);
    B.ghost_xf = reinterpret_cast<float*>(base + kLayout.ghost_xf);
    B.ghost_parent = reinterpret_cast<int*>(base + kLayout.ghost_parent);
    B.ghost_fs = reinterpret_cast<double*>(base + kLayout.ghost_fs);
    B.ghost_xn = reinterpret_cast<double*>(base + kLayout.ghost_xn);
    B.ghost_fn = reinterpret_cast<double*>(base + kLayout.ghost_fn);
    B.minmax = reinterpret_cast<unsigned long long*>(base + kLayout.minmax);
    B.ghost_bin = reinterpret_cast<int*>(base + kLayout.ghost_bin);
    B.bin_count = reinterpret_cast<int*>(base + kLayout.bin_count);
    B.bin_start = reinterpret_cast<long long*>(base + kLayout.bin_start);
    B.bin_fill = reinterpret_cast<int*>(base + kLayout.bin_fill);
    B.bin_items = reinterpret_cast<int*>(base + kLayout.bin_items);
    B.l2_count = reinterpret_cast<int*>(base + kLayout.l2_count);
    B.l2_off = reinterpret_cast<long long*>(base + kLayout.l2_off);
    B.l2_ghost = reinterpret_cast<int*>(base + kLayout.l2_ghost);
    B.l2_dist = reinterpret_cast<double*>(base + kLayout.l2_dist);
    B.l2_vec = reinterpret_cast<float*>(base + kLayout.l2_vec);
    B.n2_cap = kNaPairs;
    B.e_cnt3 = reinterpret_cast<int*>(base + kLayout.e_cnt3);
    B.e_cnt4 = reinterpret_cast<int*>(base + kLayout.e_cnt4);
    B.e_off3 = reinterpret_cast<long long*>(base + kLayout.e_off3);
    B.e_off4 = reinterpret_cast<long long*>(base + kLayout.e_off4);
    B.c3 = reinterpret_cast<int*>(base + kLayout.c3);
    B.c4 = reinterpret_cast<int*>(base + kLayout.c4);
    B.n3_cap = kNaTrip;
    B.n4_cap = kNaQuad;
    B.force = reinterpret_cast<double*>(base + kLayout.force);
    B.ev = reinterpret_cast<double*>(base + kLayout.ev);
    B.flags = reinterpret_cast<int*>(base + kLayout.flags);
    B.queue = reinterpret_cast<unsigned long long*>(base + kLayout.queue);
    int* l2_owner = reinterpret_cast<int*>(base + kLayout.l2_owner);
    void* scan = base + kLayout.scan;

#define NA_TRY(call)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call; \
            return kErrCuda;                                                          \
        }                                                                             \
    } while (0)

    // inputs into the scratch array (copies, no allocation)
    NA_TRY(cudaMemcpyAsync(B.sys, &d, sizeof(SysDesc), cudaMemcpyHostToDevice, st));
    NA_TRY(cudaMemcpyAsync((void*)B.in_pos, d_pos, sizeof(double) * 3 * natom, cudaMemcpyDeviceToDevice, st));
    NA_TRY(cudaMemcpyAsync((void*)B.in_type, d_types, sizeof(int) * natom, cudaMemcpyDeviceToDevice, st));
    // what must start at zero (the array keeps the previous call's contents)
    NA_TRY(cudaMemsetAsync(B.bin_count, 0, sizeof(int) * B.n_bins_total, st));
    NA_TRY(cudaMemsetAsync(B.bin_fill, 0, sizeof(int) * B.n_bins_total, st));
    launch_reset(B, st);   // bounding box, energy/virial, forces, flags, system error word
    count_launch(), k_noalloc_check_inputs<<<(natom + 255) / 256, 256, 0, st>>>(
        reinterpret_cast<double*>(base + kLayout.in_pos), reinterpret_cast<int*>(base + kLayout.in_type), natom,
        P.ntypes, B.flags);
    launch_atoms(B, st);
    launch_ghosts(B, st);
    launch_bin_setup(B, st);
    launch_bin_count(B, st);
    exclusive_scan(B.bin_count, B.bin_start, B.n_bins_total, scan, st);
    launch_bin_scatter(B, st);
    launch_bin_sort(B, st);
    launch_l2(B, l2_owner, false, st);
    exclusive_scan(B.l2_count, B.l2_off, B.n_atoms_total, scan, st);
    launch_l2(B, l2_owner, true, st);
    launch_enum(B, l2_owner, false, st);
    exclusive_scan(B.e_cnt3, B.e_off3, B.n2_cap, scan, st);
    exclusive_scan(B.e_cnt4, B.e_off4, B.n2_cap, scan, st);
    launch_enum(B, l2_owner, true, st);
    launch_check(B, st);
    ForceLaunch L = eng.tuning;
    L.precision = eng.precision;
    L.stride3 = P.o3 > 0 ? P.o3 + 1 : 0;
    L.stride4 = P.o4 > 0 ? P.o4 + 1 : 0;
    launch_force2(B, l2_owner, L, st);
    if (L.stride3 > 0) launch_force3(B, L, st);
    if (L.stride4 > 0) launch_force4(B, L, st);
    const double scale = 1.0 / std::pow(d.n_rep + 1.0, 3.0);
    count_launch(), k_noalloc_finish<<<(3 * natom + 255) / 256, 256, 0, st>>>(B.ev, B.force, natom, scale, vol,
                                                                            d_energy, d_force, d_stress);
    NA_TRY(cudaGetLastError());
    int flags[8];
    long long counts[3];
    NA_TRY(cudaMemcpyAsync(flags, B.flags, sizeof(flags), cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaMemcpyAsync(&counts[0], B.l2_off + B.n_atoms_total, sizeof(long long), cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaMemcpyAsync(&counts[1], B.e_off3 + B.n2_cap, sizeof(long long), cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaMemcpyAsync(&counts[2], B.e_off4 + B.n2_cap, sizeof(long long), cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaStreamSynchronize(st));
#undef NA_TRY
    eng.last.n2 = counts[0];
    eng.last.n3 = counts[1];
    eng.last.n4 = counts[2];
    eng.last.n_atoms = d.n_atoms;
    eng.last.n_ghost = n_ghost;
    eng.last.badness = flags[2];
    eng.last.penalty_hits = flags[3];
    eng.last.below_rin = flags[4];
    if (flags[6]) {
        err = std::string("ck_calculate_noalloc: ") +
              ((flags[6] & 1) ? "atom type index outside the parameter set" : "") +
              ((flags[6] & 3) == 3 ? " and " : "") + ((flags[6] & 2) ? "non-finite atom coordinate" : "") +
              "; the outputs are not valid";
        return kErrInput;
    }
    if (flags[7] & 2) {
        err = "ck_calculate_noalloc: checked build: an index outside its array was found and the access skipped";
        return kErrState;
    }
    if (flags[0] & 1) {
        err = "ck_calculate_noalloc: the bin grid exceeds its capacity (" + std::to_string(kNaBins) +
              " bins); the outputs are not valid";
        return kErrCapacity;
    }
    if ((flags[0] & ~1) || counts[0] > kNaPairs || counts[1] > kNaTrip || counts[2] > kNaQuad) {
        err = "ck_calculate_noalloc: cluster lists exceed the static maximum (" + std::to_string(counts[0]) +
              " pairs, " + std::to_string(counts[1]) + " triplets, " + std::to_string(counts[2]) +
              " quadruplets; limits " + std::to_string(kNaPairs) + ", " + std::to_string(kNaTrip) + ", " +
              std::to_string(kNaQuad) + "); the outputs are not valid";
        return kErrCapacity;
    }
    if (flags[1]) {
        err = "ck_calculate_noalloc: bad bin computed (check box lengths and atom coordinates)";
        return kErrGeometry;
    }
    return kOk;
}

}  // namespace ck
