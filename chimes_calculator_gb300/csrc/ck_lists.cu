// Cluster-list build on the GPU: periodic ghost images, the bin grid, the 2B
// neighbour lists and the 3B/4B cluster enumeration.
//
// The lists must be the reference's lists exactly (same members, same order),
// because cluster membership is decided by floating-point distance tests.
// Every floating-point step whose result decides membership therefore uses
// explicit round-to-nearest intrinsics (__dmul_rn/__dadd_rn/__dsub_rn/
// __ddiv_rn/__dsqrt_rn), which the compiler never fuses, in the reference's
// evaluation order:
//   set-up, wrap, reorient, ghosts ... serial_interface/src/serial_chimes_interface.cpp:150-587
//   bins and lists ................... serial_chimes_interface.cpp:588-864
//   get_dist ......................... serial_interface/src/serial_chimes_interface.h:141-215
//
// Two shortcuts keep the result exact while doing less work than the
// reference:
//  * only the ghost images that can lie within the search radius of the
//    primary cell are generated (host bound in ck_geom.cpp); the bin grid still
//    spans the bounding box of ALL images, which is exact from the corner
//    images alone: a ghost coordinate is a composition of IEEE-rounded sums and
//    products, each monotone in the image shift, so over the shift box its
//    extremes sit at the corners;
//  * distances are first tested in FP32 with a margin (SysDesc::eps) far above
//    the FP32 error; only a distance within the margin of a cutoff, and every
//    distance that is stored, is evaluated exactly in FP64.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "ck_common.h"
#include "ck_kernels.h"

namespace ck {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// o = m * (x,y,z) with the reference's association ((m0 x + m1 y) + m2 z)
__device__ __forceinline__ void mv(const double* m, double x, double y, double z, double* o) {
    o[0] = add(add(mul(m[0], x), mul(m[1], y)), mul(m[2], z));
    o[1] = add(add(mul(m[3], x), mul(m[4], y)), mul(m[5], z));
    o[2] = add(add(mul(m[6], x), mul(m[7], y)), mul(m[8], z));
}

// get_dist on stored fractional coordinates: |H (f_j - f_i)|; r = H (f_j - f_i)
__device__ __forceinline__ double dist_frac(const double* H, const double* fi, const double* fj, double* r = nullptr) {
    double dx = sub(fj[0], fi[0]), dy = sub(fj[1], fi[1]), dz = sub(fj[2], fi[2]);
    double r0 = add(add(mul(H[0], dx), mul(H[1], dy)), mul(H[2], dz));
    double r1 = add(add(mul(H[3], dx), mul(H[4], dy)), mul(H[5], dz));
    double r2 = add(add(mul(H[6], dx), mul(H[7], dy)), mul(H[8], dz));
    if (r) { r[0] = r0; r[1] = r1; r[2] = r2; }
    return __dsqrt_rn(add(add(mul(r0, r0), mul(r1, r1)), mul(r2, r2)));
}

__device__ __forceinline__ int find_sys_atom(const SysDesc* sys, int n, long long a) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sys[mid].atom_off <= a) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int find_sys_ghost(const SysDesc* sys, int n, long long g) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sys[mid].ghost_off <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// order-preserving unsigned key of a double (for atomicMin/atomicMax)
__device__ __forceinline__ unsigned long long okey(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_inv(unsigned long long k) {
    unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}

// reference ghost image number of shift (i,j,k): 1.. for the images of
// build_layered_system's (i,j,k) loop, skipping (0,0,0)
__device__ __forceinline__ int image_index(int i, int j, int k, int n, int side) {
    const int full = ((i + n) * side + (j + n)) * side + (k + n);
    const int center = (n * side + n) * side + n;
    return full < center ? full + 1 : full;
}

// kept image shifts of an atom with reoriented fractional coordinates fn:
// s_k in [lo_k, lo_k + cnt_k), shift 0 (the atom itself) always included
struct ShiftBox {
    int lo[3], cnt[3], count;
};
__device__ __forceinline__ void shift_box(const SysDesc& d, const double* fn, ShiftBox& b) {
    const int n = d.n_layers;
    b.count = 1;
    for (int k = 0; k < 3; k++) {
        int lo = (int)ceil(d.ulo[k] - fn[k]), hi = (int)floor(d.uhi[k] - fn[k]);
        lo = lo < -n ? -n : lo;
        hi = hi > n ? n : hi;
        lo = lo > 0 ? 0 : lo;
        hi = hi < 0 ? 0 : hi;
        b.lo[k] = lo;
        b.cnt[k] = hi - lo + 1;
        b.count *= b.cnt[k];
    }
}

// --- 1. atoms: replicate (small=true), wrap, reorient, bounding box --------
// simulation_system::init (:196-322) and reorient (:352-405).  The bounding box
// of all ghost images (build_neigh_lists :590-610) comes from each atom, its
// two corner images per axis, reduced per system.
__global__ void k_atoms(BatchView B) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = r < B.n_atoms_total;
    int s = -1;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (valid) {
        s = find_sys_atom(B.sys, B.n_sys, r);
        const SysDesc& d = B.sys[s];
        const int rl = (int)(r - d.atom_off);
        const int a = rl % d.n_in, blk = rl / d.n_in;
        const double* xin = B.in_pos + 3 * (d.in_off + a);
        double x[3] = {xin[0], xin[1], xin[2]};
        if (blk > 0) {
            const int nr1 = d.n_rep + 1;
            const int i = blk / (nr1 * nr1), j = (blk / nr1) % nr1, k = blk % nr1;
            double t[3];
            mv(d.h0i, x[0], x[1], x[2], t);
            t[0] = add(t[0], (double)i); t[1] = add(t[1], (double)j); t[2] = add(t[2], (double)k);
            mv(d.h0, t[0], t[1], t[2], x);
        }
        double f[3], xw[3], fa[3], xn[3], fn[3];
        mv(d.hi, x[0], x[1], x[2], f);
        f[0] = sub(f[0], floor(f[0])); f[1] = sub(f[1], floor(f[1])); f[2] = sub(f[2], floor(f[2]));
        mv(d.h, f[0], f[1], f[2], xw);
        mv(d.hi, xw[0], xw[1], xw[2], fa);
        mv(d.hn, fa[0], fa[1], fa[2], xn);
        mv(d.hni, xn[0], xn[1], xn[2], fn);
        ShiftBox sb;
        shift_box(d, fn, sb);
        if (sb.count > d.gstride) atomicOr(&B.flags[0], 16);   // slot bound violated (cannot happen)
        const int j0 = ((0 - sb.lo[0]) * sb.cnt[1] + (0 - sb.lo[1])) * sb.cnt[2] + (0 - sb.lo[2]);
        const long long q = d.ghost_off + (long long)rl * d.gstride + (j0 < d.gstride ? j0 : 0);
        for (int c = 0; c < 3; c++) {
            B.ghost_fs[3 * q + c] = fa[c];
            B.ghost_xn[3 * q + c] = xn[c];
            B.ghost_fn[3 * q + c] = fn[c];
            B.ghost_xf[3 * q + c] = (float)xn[c];
        }
        B.ghost_parent[q] = (int)r;
        B.ghost_id[q] = rl;
        B.atom_self[r] = (int)q;
        B.atom_sys[r] = s;
        B.atom_type[r] = B.in_type[d.in_off + a];
        B.atom_orig[r] = (int)(d.in_off + a);
        const int n = d.n_layers;
        for (int c = 0; c < 3; c++) {
            double tl[3], th[3];
            for (int k = 0; k < 3; k++) {
                const bool up = d.hn[3 * c + k] >= 0.0;
                tl[k] = add(fn[k], (double)(up ? -n : n));
                th[k] = add(fn[k], (double)(up ? n : -n));
            }
            const double vl = add(add(mul(d.hn[3 * c], tl[0]), mul(d.hn[3 * c + 1], tl[1])), mul(d.hn[3 * c + 2], tl[2]));
            const double vh = add(add(mul(d.hn[3 * c], th[0]), mul(d.hn[3 * c + 1], th[1])), mul(d.hn[3 * c + 2], th[2]));
            lo[c] = vl < xn[c] ? vl : xn[c];
            hi[c] = vh > xn[c] ? vh : xn[c];
        }
    }
    const int lane = threadIdx.x & 31;
    const int s0 = __shfl_sync(kFull, s, 0);
    if (s0 < 0) return;   // whole warp out of range (valid lanes form a prefix)
    const bool uniform = __all_sync(kFull, !valid || s == s0);
    unsigned long long kmin[3], kmax[3];
    for (int c = 0; c < 3; c++) {
        kmin[c] = valid ? okey(lo[c]) : ~0ull;
        kmax[c] = valid ? okey(hi[c]) : 0ull;
    }
    if (uniform) {
        for (int off = 16; off; off >>= 1)
            for (int c = 0; c < 3; c++) {
                unsigned long long a = __shfl_xor_sync(kFull, kmin[c], off);
                unsigned long long b = __shfl_xor_sync(kFull, kmax[c], off);
                kmin[c] = a < kmin[c] ? a : kmin[c];
                kmax[c] = b > kmax[c] ? b : kmax[c];
            }
        if (lane == 0)
            for (int c = 0; c < 3; c++) {
                atomicMin(&B.minmax[6 * s0 + c], kmin[c]);
                atomicMax(&B.minmax[6 * s0 + 3 + c], kmax[c]);
            }
    } else if (valid) {
        for (int c = 0; c < 3; c++) {
            atomicMin(&B.minmax[6 * s + c], kmin[c]);
            atomicMax(&B.minmax[6 * s + 3 + c], kmax[c]);
        }
    }
}

// --- 2. kept ghost images, one thread per slot -----------------------------
// build_layered_system (:546-585) for both the input-cell system (fractional
// coordinates for the force evaluation) and the reoriented system (Cartesian
// and fractional coordinates for the lists).
__global__ void k_ghosts(BatchView B) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= B.n_ghost_total) return;
    const int s = find_sys_ghost(B.sys, B.n_sys, q);
    const SysDesc& d = B.sys[s];
    const long long ql = q - d.ghost_off;
    const int rl = (int)(ql / d.gstride), j = (int)(ql % d.gstride);
    const long long r = d.atom_off + rl;
    const long long qs = B.atom_self[r];
    if (q == qs) return;   // the atom itself, written by k_atoms
    const double fa[3] = {B.ghost_fs[3 * qs], B.ghost_fs[3 * qs + 1], B.ghost_fs[3 * qs + 2]};
    const double fn[3] = {B.ghost_fn[3 * qs], B.ghost_fn[3 * qs + 1], B.ghost_fn[3 * qs + 2]};
    ShiftBox sb;
    shift_box(d, fn, sb);
    if (j >= sb.count) {
        B.ghost_id[q] = -1;
        return;
    }
    const int i0 = sb.lo[0] + j / (sb.cnt[1] * sb.cnt[2]);
    const int i1 = sb.lo[1] + (j / sb.cnt[2]) % sb.cnt[1];
    const int i2 = sb.lo[2] + j % sb.cnt[2];
    double t[3], p[3], o[3], xn[3];
    t[0] = add(fa[0], (double)i0); t[1] = add(fa[1], (double)i1); t[2] = add(fa[2], (double)i2);
    mv(d.h, t[0], t[1], t[2], p);
    mv(d.hi, p[0], p[1], p[2], o);
    B.ghost_fs[3 * q] = o[0]; B.ghost_fs[3 * q + 1] = o[1]; B.ghost_fs[3 * q + 2] = o[2];
    t[0] = add(fn[0], (double)i0); t[1] = add(fn[1], (double)i1); t[2] = add(fn[2], (double)i2);
    mv(d.hn, t[0], t[1], t[2], xn);
    mv(d.hni, xn[0], xn[1], xn[2], o);
    for (int c = 0; c < 3; c++) {
        B.ghost_xn[3 * q + c] = xn[c];
        B.ghost_fn[3 * q + c] = o[c];
        B.ghost_xf[3 * q + c] = (float)xn[c];
    }
    B.ghost_parent[q] = (int)r;
    B.ghost_id[q] = image_index(i0, i1, i2, d.n_layers, d.side) * d.n_atoms + rl;
}

// --- 3. bin grid per system (build_neigh_lists :622-642) -------------------
__global__ void k_bin_setup(BatchView B) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.n_sys) return;
    SysDesc& d = B.sys[s];
    long long total = 1;
    for (int c = 0; c < 3; c++) {
        const double mn = okey_inv(B.minmax[6 * s + c]), mx = okey_inv(B.minmax[6 * s + 3 + c]);
        d.minpos[c] = mn;
        int nb = (int)ceil(__ddiv_rn(sub(mx, mn), d.search));
        if (nb < 1) nb = 1;
        d.nb[c] = nb;
        total *= nb;
    }
    if (total > d.bin_cap) {
        d.err = kErrCapacity;
        atomicOr(&B.flags[0], 1);
    }
}

__device__ __forceinline__ void bin_of(const SysDesc& d, const double* x, int& bx, int& by, int& bz) {
    bx = (int)floor(__ddiv_rn(sub(x[0], d.minpos[0]), d.search));
    by = (int)floor(__ddiv_rn(sub(x[1], d.minpos[1]), d.search));
    bz = (int)floor(__ddiv_rn(sub(x[2], d.minpos[2]), d.search));
}

// --- 4. bin population (:644-678) -------------------------------------------
__global__ void k_bin_count(BatchView B) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= B.n_ghost_total) return;
    if (B.ghost_id[q] < 0) { B.ghost_bin[q] = -1; return; }
    const int s = find_sys_ghost(B.sys, B.n_sys, q);
    const SysDesc& d = B.sys[s];
    if (d.err) { B.ghost_bin[q] = -1; return; }
    int bx, by, bz;
    bin_of(d, &B.ghost_xn[3 * q], bx, by, bz);
    const long long total = (long long)d.nb[0] * d.nb[1] * d.nb[2];
    if (bx < 0 || by < 0 || bz < 0) { atomicExch(&B.flags[1], 1); B.ghost_bin[q] = -1; return; }
    const long long ib = bx + (long long)by * d.nb[0] + (long long)bz * d.nb[0] * d.nb[1];
    if (ib >= total) { atomicExch(&B.flags[1], 2); B.ghost_bin[q] = -1; return; }
    B.ghost_bin[q] = (int)ib;
    atomicAdd(&B.bin_count[d.bin_off + ib], 1);
}

__global__ void k_bin_scatter(BatchView B, const long long* bin_start) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= B.n_ghost_total) return;
    const int ib = B.ghost_bin[q];
    if (ib < 0) return;
    const int s = find_sys_ghost(B.sys, B.n_sys, q);
    const long long b = B.sys[s].bin_off + ib;
    const long long pos = bin_start[b] + atomicAdd(&B.bin_fill[b], 1);
    B.bin_items[pos] = (int)q;
}

// FP32 coordinates and parent atom of ghost q at bin position pos (read by
// the pair-list kernel in bin order instead of gathered by ghost id)
__device__ __forceinline__ void put_xp(const BatchView& B, long long pos, int q) {
    const float* x = &B.ghost_xf[3 * (long long)q];
    reinterpret_cast<float4*>(B.bin_xp)[pos] = make_float4(x[0], x[1], x[2], __int_as_float(B.ghost_parent[q]));
}

// each bin's members in ascending ghost id (the reference pushes ghosts into
// bins in index order): a warp takes one bin, or 32 in a large batch (most of
// the reserved bins are empty); a bin of one member needs no sort, larger
// ones are ranked by the whole warp in turn: a member's place is the number of members with a
// smaller id (ids are unique), counted over the warp's registers up to 64
// members, over a shared-memory copy of the ids up to kRankSmem; larger
// bins (none in practice) fall back to an insertion sort by one lane
constexpr int kRankSmem = 256;
__device__ __forceinline__ void rank_bin(const BatchView& B, long long s0, int n, int lane, int* key, int* val) {
    int* v = B.bin_items + s0;
    if (n > 64 && n <= kRankSmem) {
        for (int i = lane; i < n; i += 32) {
            val[i] = v[i];
            key[i] = B.ghost_id[val[i]];
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            const int k = key[i];
            int r = 0;
            for (int j = 0; j < n; j++) r += key[j] < k;
            v[r] = val[i];
            if (B.bin_xp) put_xp(B, s0 + r, val[i]);
        }
        __syncwarp();
        return;
    }
    if (n > 64) {
        if (lane == 0)
            for (int i = 1; i < n; i++) {
                const int k2 = v[i], kid = B.ghost_id[k2];
                int j = i - 1;
                while (j >= 0 && B.ghost_id[v[j]] > kid) { v[j + 1] = v[j]; j--; }
                v[j + 1] = k2;
            }
        __syncwarp();
        if (B.bin_xp)
            for (int i = lane; i < n; i += 32) put_xp(B, s0 + i, v[i]);
        __syncwarp();
        return;
    }
    const int big = 0x7fffffff;
    const int q0 = lane < n ? v[lane] : -1, q1 = lane + 32 < n ? v[lane + 32] : -1;
    const int k0 = q0 >= 0 ? B.ghost_id[q0] : big, k1 = q1 >= 0 ? B.ghost_id[q1] : big;
    int r0 = 0, r1 = 0;
    for (int src = 0; src < 32; src++) {
        const int o0 = __shfl_sync(kFull, k0, src), o1 = __shfl_sync(kFull, k1, src);
        r0 += (o0 < k0) + (o1 < k0);
        r1 += (o0 < k1) + (o1 < k1);
    }
    __syncwarp();
    if (q0 >= 0) {
        v[r0] = q0;
        if (B.bin_xp) put_xp(B, s0 + r0, q0);
    }
    if (q1 >= 0) {
        v[r1] = q1;
        if (B.bin_xp) put_xp(B, s0 + r1, q1);
    }
    __syncwarp();
}

__global__ void __launch_bounds__(256) k_bin_rank(BatchView B, const long long* bin_start, int per) {
    __shared__ int s_key[8][kRankSmem], s_val[8][kRankSmem];
    const long long b0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * per;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (b0 >= B.n_bins_total) return;   // whole warp
    const long long b = b0 + lane;
    int n = 0;
    long long st = 0;
    if (lane < per && b < B.n_bins_total) {
        n = B.bin_count[b];
        if (n > 0) st = bin_start[b];
    }
    if (n == 1 && B.bin_xp) put_xp(B, st, B.bin_items[st]);
    unsigned many = __ballot_sync(kFull, n > 1);
    while (many) {
        const int src = __ffs(many) - 1;
        many &= many - 1;
        rank_bin(B, __shfl_sync(kFull, st, src), __shfl_sync(kFull, n, src), lane, s_key[wib], s_val[wib]);
    }
}

// --- 5. 2B neighbour lists (:680-731): one warp per atom --------------------
// Lane b < 27 owns neighbour bin b in the reference's loop order (x bins
// outermost, z innermost); the candidates of all 27 bins are numbered bin by
// bin and the warp walks them 32 at a time, so the emitted order is the
// reference's and short bins leave no lanes idle.  The FP32 displacement
// decides most candidates; the exact FP64 distance (which the list keeps) is
// taken only for the candidates that survive it, queued in candidate order in
// shared memory and evaluated 32 at a time, so the FP64 pipe (1/64 of the
// FP32 rate) runs full warps instead of one or two live lanes per chunk.  The
// count pass counts the candidates the FP32 test places inside the cutoff by
// more than the margin without an FP64 distance.
constexpr int kL2Block = 256;
// bits of l2_vec.w above the parent atom index (atom indices are below 2^30)
constexpr unsigned kL2Parent = 0x3FFFFFFFu, kL2In3 = 1u << 30, kL2In4 = 1u << 31;
template <bool FILL>
__global__ void __launch_bounds__(kL2Block) k_l2(BatchView B, const long long* bin_start, int* l2_owner) {
    __shared__ int queue[kL2Block / 32][64];
    __shared__ int qpar[kL2Block / 32][64];
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    if (warp >= B.n_atoms_total) return;
    const long long r = warp;
    const int s = B.atom_sys[r];
    const SysDesc& d = B.sys[s];
    if (d.err) { if (!FILL && lane == 0) B.l2_count[r] = 0; return; }
    const long long gi = B.atom_self[r];
    const double fi[3] = {B.ghost_fn[3 * gi], B.ghost_fn[3 * gi + 1], B.ghost_fn[3 * gi + 2]};
    const float xi[3] = {B.ghost_xf[3 * gi], B.ghost_xf[3 * gi + 1], B.ghost_xf[3 * gi + 2]};
    double hn[9];
    for (int c = 0; c < 9; c++) hn[c] = d.hn[c];
    const double sd = d.search;
    const float far2 = d.far2, near2 = d.near2;
    // the atom's bin, as k_bin_count placed it (bin_of of the same coordinates;
    // recomputing it would cost three FP64 divisions per atom)
    const int ib0 = B.ghost_bin[gi];
    int bx = -1, by = -1, bz = -1;
    if (ib0 >= 0) {
        bx = ib0 % d.nb[0];
        by = (ib0 / d.nb[0]) % d.nb[1];
        bz = ib0 / (d.nb[0] * d.nb[1]);
    }
    if (bx < 1 || by < 1 || bz < 1) {
        if (lane == 0) { atomicExch(&B.flags[1], 3); if (!FILL) B.l2_count[r] = 0; }
        return;
    }
    const long long total = (long long)d.nb[0] * d.nb[1] * d.nb[2];
    long long base = FILL ? B.l2_off[r] : 0;
    int count = 0;
    long long bst = 0;
    int nbin = 0;
    if (lane < 27) {
        const int i = bx - 1 + lane / 9, j = by - 1 + (lane / 3) % 3, k = bz - 1 + lane % 3;
        const long long ib = i + (long long)j * d.nb[0] + (long long)k * d.nb[0] * d.nb[1];
        if (ib >= total) {
            atomicExch(&B.flags[1], 4);
        } else {
            const long long b = d.bin_off + ib;
            bst = bin_start[b];
            nbin = B.bin_count[b];
        }
    }
    int incl = nbin;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    const int excl = incl - nbin;
    const int ncand = __shfl_sync(kFull, incl, 31);
    int* q = queue[wib];
    int* qp = qpar[wib];
    int qn = 0;   // queued candidates (warp-uniform)
    // exact distances of the first n queued candidates; members counted / written in order
    auto drain = [&](int n) {
        bool pred = false;
        int ajj = -1, par = -1;
        double dd = 0.0, rv[3] = {0, 0, 0};
        if (lane < n) {
            ajj = q[lane];
            par = qp[lane];
            dd = dist_frac(hn, fi, &B.ghost_fn[3 * (long long)ajj], rv);
            pred = dd < sd;
        }
        const unsigned bal = __ballot_sync(kFull, pred);
        if (FILL && pred) {
            const long long pos = base + count + __popc(bal & lt);
            if (pos < B.n2_cap) {
                B.l2_ghost[pos] = ajj;
                B.l2_dist[pos] = dd;
                l2_owner[pos] = (int)r;
                // x, y, z: FP32 displacement for the enumeration's prefilter;
                // w: the neighbour's parent atom (int bits; saves the
                // enumeration a dependent load per candidate) with the exact
                // tests dd < c3 and dd < c4 in bits 30 and 31, so the
                // enumeration compares no FP64 distances
                const unsigned w = (unsigned)par | (dd < d.c3 ? kL2In3 : 0u) | (dd < d.c4 ? kL2In4 : 0u);
                float4 v = make_float4((float)rv[0], (float)rv[1], (float)rv[2], __uint_as_float(w));
                reinterpret_cast<float4*>(B.l2_vec)[pos] = v;
            }
        }
        count += __popc(bal);
        // move the rest of the queue to its front
        __syncwarp();
        const int rest = qn - n;
        int mv = -1, mp = -1;
        if (lane < rest) { mv = q[n + lane]; mp = qp[n + lane]; }
        __syncwarp();
        if (lane < rest) { q[lane] = mv; qp[lane] = mp; }
        __syncwarp();
        qn = rest;
    };
    for (int t0 = 0; t0 < ncand; t0 += 32) {
        const int t = t0 + lane;
        // bin of candidate t: the last bin whose first candidate is <= t
        int lo = 0;
        for (int step = 16; step >= 1; step >>= 1) {
            const int cand = lo + step;
            const int ex = __shfl_sync(kFull, excl, cand & 31);
            if (cand < 27 && ex <= t) lo = cand;
        }
        const long long st = __shfl_sync(kFull, bst, lo);
        const int first = __shfl_sync(kFull, excl, lo);
        bool exact = false, sure = false;
        int ajj = -1, par = -1;
        if (t < ncand) {
            const long long it = st + (t - first);
            ajj = B.bin_items[it];
            float xj[3];
            if (B.bin_xp) {   // the candidate's coordinates and parent stored in bin order
                const float4 p = reinterpret_cast<const float4*>(B.bin_xp)[it];
                xj[0] = p.x; xj[1] = p.y; xj[2] = p.z;
                par = __float_as_int(p.w);
            } else {
                par = B.ghost_parent[ajj];
                xj[0] = B.ghost_xf[3 * (long long)ajj];
                xj[1] = B.ghost_xf[3 * (long long)ajj + 1];
                xj[2] = B.ghost_xf[3 * (long long)ajj + 2];
            }
            if (ajj != gi && r <= par) {
                const float ex = xj[0] - xi[0], ey = xj[1] - xi[1], ez = xj[2] - xi[2];
                const float e2 = ex * ex + ey * ey + ez * ez;
                if (e2 < far2) {   // else certainly >= sd
                    if (!FILL && e2 < near2) sure = true;   // certainly < sd
                    else exact = true;
                }
            }
        }
        if (!FILL) count += __popc(__ballot_sync(kFull, sure));
        const unsigned m = __ballot_sync(kFull, exact);
        if (exact) {
            const int pos = qn + __popc(m & lt);
            q[pos] = ajj;
            qp[pos] = par;
        }
        qn += __popc(m);
        __syncwarp();
        if (qn >= 32) drain(32);
    }
    if (qn > 0) drain(qn);
    if (!FILL && lane == 0) B.l2_count[r] = count;
}

// Exact test "distance >= c" for a ghost pair of one atom's list, deciding
// from the FP32 displacement difference when it is farther than eps from c.
struct PairDist {
    const double* hn;
    const double* fa;
    const double* fb;
    float df;
    double exact;
    bool have;
    __device__ bool ge(double c, double eps) {
        if ((double)df < c - eps) return false;
        if ((double)df >= c + eps) return true;
        if (!have) { exact = dist_frac(hn, fa, fb); have = true; }
        return exact >= c;
    }
};

// The same test with the margins as FP32 thresholds (lo <= c - eps, hi >=
// c + eps, rounded outward), so the decided cases take no FP64 instruction.
struct PairDistF {
    const double* hn;
    const double* fa;
    const double* fb;
    float df;
    __device__ bool ge(double c, float lo, float hi) const {
        if (df < lo) return false;
        if (df >= hi) return true;
        return dist_frac(hn, fa, fb) >= c;
    }
};

__device__ __forceinline__ float vdist(const float4& a, const float4& b) {
    const float x = b.x - a.x, y = b.y - a.y, z = b.z - a.z;
    return sqrtf(x * x + y * y + z * z);
}

// --- 6. 3B/4B enumeration (:735-855): one thread per (i, j) list entry -----
// The valid_3mer / valid_4mer flags carry over between k iterations exactly as
// in the reference, so the emitted sets and their order match it.
template <bool FILL>
__device__ void enum_entry(const BatchView& B, const int* l2_owner, long long e) {
    const int r = l2_owner[e];
    const SysDesc& d = B.sys[B.atom_sys[r]];
    int n3 = 0, n4 = 0;
    long long o3 = 0, o4 = 0;
    if (FILL) { o3 = B.e_off3[e]; o4 = B.e_off4[e]; }
    const double c3 = d.c3, c4 = d.c4, eps = d.eps;
    if (d.has3 || d.has4) {
        double hn[9];
        for (int c = 0; c < 9; c++) hn[c] = d.hn[c];
        const int gi = B.atom_self[r];
        const long long b0 = min(B.l2_off[r], B.n2_cap), b1 = min(B.l2_off[r + 1], B.n2_cap);
        const float4* vec = reinterpret_cast<const float4*>(B.l2_vec);
        const int jj = B.l2_ghost[e];
        const double dij = B.l2_dist[e];
        bool v3 = true, v4 = true;
        if (dij >= c3) v3 = false;
        if (dij >= c4) v4 = false;
        if (v3 || v4) {
            const double* fj = &B.ghost_fn[3 * (long long)jj];
            const float4 vj = vec[e];
            const int pj = B.ghost_parent[jj];
            for (long long k = b0; k < b1; k++) {
                const int kk = B.l2_ghost[k];
                if (jj == kk) continue;
                const int pk = B.ghost_parent[kk];
                if (pj > pk) continue;
                const double dik = B.l2_dist[k];
                if (dik >= c3) v3 = false;
                if (dik >= c4) v4 = false;
                const float4 vk = vec[k];
                const double* fk = &B.ghost_fn[3 * (long long)kk];
                PairDist jk{hn, fj, fk, vdist(vj, vk), 0.0, false};
                if (jk.ge(c3, eps)) v3 = false;
                if (jk.ge(c4, eps)) v4 = false;
                if (!v3 && !v4) {
                    if (dij < c3) v3 = true;
                    if (dij < c4) v4 = true;
                    continue;
                }
                if (v3) {
                    if (FILL && o3 + n3 < B.n3_cap) {
                        int* out = B.c3 + 3 * (o3 + n3);
                        out[0] = gi; out[1] = jj; out[2] = kk;
                    }
                    n3++;
                }
                if (!d.has4) continue;
                if (!v4) {
                    if (dij < c4) v4 = true;
                    continue;
                }
                for (long long l = b0; l < b1; l++) {
                    const int ll = B.l2_ghost[l];
                    if (jj == ll || kk == ll) continue;
                    const int pl = B.ghost_parent[ll];
                    if (pj > pl) continue;
                    if (pk > pl) continue;
                    if (B.l2_dist[l] >= c4) continue;
                    const float4 vl = vec[l];
                    const double* fl = &B.ghost_fn[3 * (long long)ll];
                    PairDist jl{hn, fj, fl, vdist(vj, vl), 0.0, false};
                    if (jl.ge(c4, eps)) continue;
                    PairDist kl{hn, fk, fl, vdist(vk, vl), 0.0, false};
                    if (kl.ge(c4, eps)) continue;
                    if (v4) {
                        if (FILL && o4 + n4 < B.n4_cap) {
                            int* out = B.c4 + 4 * (o4 + n4);
                            out[0] = gi; out[1] = jj; out[2] = kk; out[3] = ll;
                        }
                        n4++;
                    }
                }
            }
        }
    }
    if (!FILL) { B.e_cnt3[e] = n3; B.e_cnt4[e] = n4; }
}

template <bool FILL>
__global__ void k_enum(BatchView B, const int* l2_owner) {
    const long long n2 = min(B.l2_off[B.n_atoms_total], B.n2_cap);
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < B.n2_cap;
         e += (long long)gridDim.x * blockDim.x) {
        if (e >= n2) {
            if (!FILL) { B.e_cnt3[e] = 0; B.e_cnt4[e] = 0; }
            continue;
        }
        enum_entry<FILL>(B, l2_owner, e);
    }
}

// Per-entry warp form of the same enumeration.  When the 4-body outer cutoff
// does not exceed the 3-body one (or a system lacks one of the two), the
// valid_3mer / valid_4mer flags are restored before every k (the reference's
// reset branch), so each k -- and each l -- is decided on its own: lanes take
// consecutive k (then l) of the atom's list and a ballot plus prefix count
// emits the clusters in the reference's (k, l) order.  Systems with 3- and
// 4-body terms and rc4 > rc3 keep the sequential carry-over (k_enum).  Used
// by k_enuma for atoms whose list is longer than its bit matrices hold.
template <bool FILL>
__device__ void enumw_entry(const BatchView& B, long long e, int r, const SysDesc& d, int lane, unsigned lt) {
    const float4* vec = reinterpret_cast<const float4*>(B.l2_vec);
    const double c3 = d.c3, c4 = d.c4;
    const float4 vj = vec[e];
    const unsigned wj = __float_as_uint(vj.w);
    const bool want3 = d.has3 && (wj & kL2In3), want4 = d.has4 && (wj & kL2In4);
    long long n3 = 0, n4 = 0;
    long long o3 = 0, o4 = 0;
    if (FILL) { o3 = B.e_off3[e]; o4 = B.e_off4[e]; }
    if (want3 || want4) {
        const double* hn = d.hn;   // read in place: the exact distances are rare
        const float c3lo = d.c3lo, c3hi = d.c3hi, c4lo = d.c4lo, c4hi = d.c4hi;
        const int gi = B.atom_self[r];
        const long long b0 = min(B.l2_off[r], B.n2_cap), b1 = min(B.l2_off[r + 1], B.n2_cap);
        const int jj = B.l2_ghost[e];
        const double* fj = &B.ghost_fn[3 * (long long)jj];
        const int pj = (int)(wj & kL2Parent);
        for (long long kb = b0; kb < b1; kb += 32) {
            const long long k = kb + lane;
            bool ok3 = false, ok4 = false;
            int kk = -1, pk = 0;
            float4 vk = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < b1) {
                kk = B.l2_ghost[k];
                vk = vec[k];
                const unsigned wk = __float_as_uint(vk.w);
                pk = (int)(wk & kL2Parent);
                if (kk != jj && pj <= pk) {
                    const PairDistF jk{hn, fj, &B.ghost_fn[3 * (long long)kk], vdist(vj, vk)};
                    ok3 = want3 && (wk & kL2In3) && !jk.ge(c3, c3lo, c3hi);
                    ok4 = want4 && (wk & kL2In4) && !jk.ge(c4, c4lo, c4hi);
                }
            }
            const unsigned m3 = __ballot_sync(kFull, ok3);
            if (FILL && ok3) {
                const long long q = o3 + n3 + __popc(m3 & lt);
                if (q < B.n3_cap) {
                    int* out = B.c3 + 3 * q;
                    out[0] = gi; out[1] = jj; out[2] = kk;
                    if (B.c3e) { B.c3e[2 * q] = (int)e; B.c3e[2 * q + 1] = (int)k; }
                }
            }
            n3 += __popc(m3);
            unsigned m4 = __ballot_sync(kFull, ok4);
            while (m4) {
                const int src = __ffs(m4) - 1;
                m4 &= m4 - 1;
                const int ks = __shfl_sync(kFull, kk, src);
                const int pks = __shfl_sync(kFull, pk, src);
                float4 vks;
                vks.x = __shfl_sync(kFull, vk.x, src);
                vks.y = __shfl_sync(kFull, vk.y, src);
                vks.z = __shfl_sync(kFull, vk.z, src);
                vks.w = 0.f;
                const double* fk = &B.ghost_fn[3 * (long long)ks];
                for (long long lb = b0; lb < b1; lb += 32) {
                    const long long l = lb + lane;
                    bool okl = false;
                    int ll = -1;
                    if (l < b1) {
                        ll = B.l2_ghost[l];
                        const float4 vl = vec[l];
                        if (ll != jj && ll != ks) {
                            const unsigned wl = __float_as_uint(vl.w);
                            const int pl = (int)(wl & kL2Parent);
                            if (pj <= pl && pks <= pl && (wl & kL2In4)) {
                                const double* fl = &B.ghost_fn[3 * (long long)ll];
                                const PairDistF jl{hn, fj, fl, vdist(vj, vl)};
                                if (!jl.ge(c4, c4lo, c4hi)) {
                                    const PairDistF kl{hn, fk, fl, vdist(vks, vl)};
                                    okl = !kl.ge(c4, c4lo, c4hi);
                                }
                            }
                        }
                    }
                    const unsigned ml = __ballot_sync(kFull, okl);
                    if (FILL && okl) {
                        const long long q = o4 + n4 + __popc(ml & lt);
                        if (q < B.n4_cap) {
                            int* out = B.c4 + 4 * q;
                            out[0] = gi; out[1] = jj; out[2] = ks; out[3] = ll;
                            if (B.c4e) {
                                B.c4e[3 * q] = (int)e;
                                B.c4e[3 * q + 1] = (int)(kb + src);
                                B.c4e[3 * q + 2] = (int)l;
                            }
                        }
                    }
                    n4 += __popc(ml);
                }
            }
        }
    }
    if (!FILL && lane == 0) { B.e_cnt3[e] = (int)n3; B.e_cnt4[e] = (int)n4; }
}

// Bit-matrix form (G warps per atom i, atoms with at most kEnumRows list
// entries).  With the reset semantics above, membership depends only on pair
// tests among the entries of i's list:
//   T[j][k] = want3(j) && in3(k) && j != k && parent(j) <= parent(k) && |r_jk| < rc3
//   Q[j][k] = want4(j) && in4(k) && j != k && parent(j) <= parent(k) && |r_jk| < rc4
// (i, j, k) is a triplet iff T[j][k]; (i, j, k, l) a quadruplet iff Q[j][k]
// && Q[j][l] && Q[k][l] (Q[j][k] implies want4(k), which Q[k][l] carries).
// The warps test every ordered pair of entries once -- the FP32 distance with
// the same thresholds and, inside the margin, the same exact FP64 distance as
// the per-entry form -- and keep the rows T[j], Q[j] as bit masks in shared
// memory.  The count pass then takes n3(j) = popc T[j] and n4(j) = sum over
// k in Q[j] of popc(Q[j] & Q[k]); the fill pass emits the clusters from the
// masks in the same order (k ascending, then l ascending), each entry at the
// offset of the atom's first entry plus the counts of the entries before it
// (which the masks give).  The per-entry form walks k and, for every 4-body
// k, all l again, once per pass; here both passes cost one test per ordered
// pair.  G = 1 for batches with many atoms; small ones spread an atom over
// up to a whole block so that the launch still fills the GPU.
constexpr int kEnumRows = 96;
constexpr int kEnumWords = kEnumRows / 32;   // odd: column reads of the masks hit distinct banks
constexpr int kEnumWarps = 8;

template <int G>
__device__ __forceinline__ void group_sync(int grp) {
    if (G == 1) __syncwarp();
    else if (G == kEnumWarps) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(32 * G) : "memory");
}

// position of the k-th (from 0) set bit of m
__device__ __forceinline__ int select_bit(unsigned m, int k) {
    int pos = 0;
    for (int sh = 16; sh; sh >>= 1) {
        const int c = __popc(m & ((1u << sh) - 1u));
        if (k >= c) { k -= c; m >>= sh; pos += sh; }
    }
    return pos;
}

// n3 and n4 of entry a from the masks
__device__ __forceinline__ void mask_counts(const unsigned* rt, const unsigned* rq, int a, int nw, int& n3, int& n4) {
    n3 = 0;
    n4 = 0;
    for (int c = 0; c < nw; c++) n3 += __popc(rt[a * kEnumWords + c]);
    for (int c = 0; c < nw; c++) {
        unsigned m = rq[a * kEnumWords + c];
        while (m) {
            const int b = 32 * c + __ffs(m) - 1;
            m &= m - 1;
            for (int c2 = 0; c2 < nw; c2++) n4 += __popc(rq[a * kEnumWords + c2] & rq[b * kEnumWords + c2]);
        }
    }
}

template <bool FILL, int G>
__global__ void __launch_bounds__(32 * kEnumWarps, 4) k_enuma(BatchView B) {
    constexpr int NG = kEnumWarps / G;   // atoms a block works on at a time
    __shared__ float4 s_v[NG][kEnumRows];
    __shared__ int s_g[NG][kEnumRows];
    __shared__ unsigned s_t[NG][kEnumRows * kEnumWords];
    __shared__ unsigned s_q[NG][kEnumRows * kEnumWords];
    __shared__ int s_o[FILL ? NG : 1][FILL ? 2 * kEnumRows + 2 : 1];   // per-entry offsets, then the totals
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int grp = wib / G, w = wib % G;
    const unsigned lt = (1u << lane) - 1u;
    const long long n2 = min(B.l2_off[B.n_atoms_total], B.n2_cap);
    if (!FILL) {
        for (long long e = n2 + (long long)blockIdx.x * blockDim.x + threadIdx.x; e < B.n2_cap;
             e += (long long)gridDim.x * blockDim.x) {
            B.e_cnt3[e] = 0;
            B.e_cnt4[e] = 0;
        }
    }
    const float4* vec = reinterpret_cast<const float4*>(B.l2_vec);
    float4* sv = s_v[grp];
    int* sg = s_g[grp];
    unsigned* rt = s_t[grp];
    unsigned* rq = s_q[grp];
    const long long ngroups = (long long)gridDim.x * NG;
    for (long long r = (long long)blockIdx.x * NG + grp; r < B.n_atoms_total; r += ngroups) {
        const long long b0 = min(B.l2_off[r], B.n2_cap), b1 = min(B.l2_off[r + 1], B.n2_cap);
        const int L = (int)(b1 - b0);
        if (L <= 0) continue;
        const SysDesc& d = B.sys[B.atom_sys[r]];
        if (!d.has3 && !d.has4) {
            if (!FILL)
                for (int a = 32 * w + lane; a < L; a += 32 * G) { B.e_cnt3[b0 + a] = 0; B.e_cnt4[b0 + a] = 0; }
            continue;
        }
        if (L > kEnumRows) {
            for (long long e = b0 + w; e < b1; e += G) enumw_entry<FILL>(B, e, (int)r, d, lane, lt);
            continue;
        }
        long long o3 = 0, o4 = 0;
        if (FILL) { o3 = B.e_off3[b0]; o4 = B.e_off4[b0]; }
        group_sync<G>(grp);   // the previous atom's masks are no longer read
        for (int a = 32 * w + lane; a < L; a += 32 * G) {
            sv[a] = vec[b0 + a];
            sg[a] = B.l2_ghost[b0 + a];
        }
        group_sync<G>(grp);
        const int nw = (L + 31) >> 5;
        {
            const double* hn = d.hn;   // read in place: the exact distances are rare
            const double c3 = d.c3, c4 = d.c4;
            // squared FP32 thresholds: the prefilter needs no square root
            const float c3lo2 = d.c3lo2, c3hi2 = d.c3hi2, c4lo2 = d.c4lo2, c4hi2 = d.c4hi2;
            const bool has3 = d.has3, has4 = d.has4;
            for (int c = 0; c < nw; c++) {
                // this lane's candidate k (column b of every row) stays in registers
                const int b = 32 * c + lane;
                float4 vb = make_float4(0.f, 0.f, 0.f, 0.f);
                int gb = -1;
                if (b < L) { vb = sv[b]; gb = sg[b]; }
                const unsigned wb = __float_as_uint(vb.w);
                const int pb = (int)(wb & kL2Parent);
                const bool in3 = has3 && (wb & kL2In3), in4 = has4 && (wb & kL2In4);
                for (int a = w; a < L; a += G) {
                    const float4 va = sv[a];
                    const unsigned wa = __float_as_uint(va.w);
                    const int ga = sg[a];
                    const bool t0 = in3 && (wa & kL2In3) && b < L && gb != ga && (int)(wa & kL2Parent) <= pb;
                    const bool q0 = in4 && (wa & kL2In4) && b < L && gb != ga && (int)(wa & kL2Parent) <= pb;
                    bool t = false, q = false;
                    if (t0 || q0) {
                        const float ex = vb.x - va.x, ey = vb.y - va.y, ez = vb.z - va.z;
                        const float e2 = ex * ex + ey * ey + ez * ez;
                        // inside the margin of a cutoff: decided by the exact distance
                        // (FP64 only on that rare branch: GB300 issues FP64 at a small
                        // fraction of the FP32 rate)
                        const bool x3 = t0 && !(e2 < c3lo2) && !(e2 >= c3hi2);
                        const bool x4 = q0 && !(e2 < c4lo2) && !(e2 >= c4hi2);
                        t = t0 && e2 < c3lo2;
                        q = q0 && e2 < c4lo2;
                        if (x3 || x4) {
                            const double dx = dist_frac(hn, &B.ghost_fn[3 * (long long)ga], &B.ghost_fn[3 * (long long)gb]);
                            if (x3) t = dx < c3;
                            if (x4) q = dx < c4;
                        }
                    }
                    const unsigned bt = __ballot_sync(kFull, t), bq = __ballot_sync(kFull, q);
                    if (lane == 0) { rt[a * kEnumWords + c] = bt; rq[a * kEnumWords + c] = bq; }
                }
            }
        }
        group_sync<G>(grp);
        if (!FILL) {
            for (int a = 32 * w + lane; a < L; a += 32 * G) {
                int n3, n4;
                mask_counts(rt, rq, a, nw, n3, n4);
                B.e_cnt3[b0 + a] = n3;
                B.e_cnt4[b0 + a] = n4;
            }
            continue;
        }
        // offsets of the entries within the atom (triplets, quadruplets) and
        // the atom's totals
        int* so = s_o[FILL ? grp : 0];
        if (w == 0) {
            int c3 = 0, c4 = 0;
            for (int a0 = 0; a0 < L; a0 += 32) {
                const int a = a0 + lane;
                int n3 = 0, n4 = 0;
                if (a < L) mask_counts(rt, rq, a, nw, n3, n4);
                int i3 = n3, i4 = n4;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y3 = __shfl_up_sync(kFull, i3, o), y4 = __shfl_up_sync(kFull, i4, o);
                    if (lane >= o) { i3 += y3; i4 += y4; }
                }
                if (a < L) { so[2 * a] = c3 + i3 - n3; so[2 * a + 1] = c4 + i4 - n4; }
                c3 += __shfl_sync(kFull, i3, 31);
                c4 += __shfl_sync(kFull, i4, 31);
            }
            if (lane == 0) { so[2 * L] = c3; so[2 * L + 1] = c4; }
        }
        group_sync<G>(grp);
        // the atom's clusters in the reference's order, one per lane: the t-th
        // triplet belongs to the last entry whose offset is <= t and is that
        // entry's (t - offset)-th set bit of T; the t-th quadruplet likewise,
        // walking the entry's k in Q and the set bits of Q[j] & Q[k]
        const int gi = B.atom_self[r];
        const long long base3 = B.e_off3[b0], base4 = B.e_off4[b0];
        const int t3 = so[2 * L], t4 = so[2 * L + 1];
        for (int t = 32 * w + lane; t < t3; t += 32 * G) {
            int lo = 0, hi = L - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (so[2 * mid] <= t) lo = mid; else hi = mid - 1;
            }
            const int a = lo;
            int rk = t - so[2 * a], bk = 0;
            for (int c = 0; c < nw; c++) {
                const unsigned m = rt[a * kEnumWords + c];
                const int pc = __popc(m);
                if (rk < pc) { bk = 32 * c + select_bit(m, rk); break; }
                rk -= pc;
            }
            const long long q = base3 + t;
            if (q < B.n3_cap) {
                int* out = B.c3 + 3 * q;
                out[0] = gi; out[1] = sg[a]; out[2] = sg[bk];
                if (B.c3e) { B.c3e[2 * q] = (int)(b0 + a); B.c3e[2 * q + 1] = (int)(b0 + bk); }
            }
        }
        for (int t = 32 * w + lane; t < t4; t += 32 * G) {
            int lo = 0, hi = L - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (so[2 * mid + 1] <= t) lo = mid; else hi = mid - 1;
            }
            const int a = lo;
            int rk = t - so[2 * a + 1], bk = 0, lk = 0;
            bool found = false;
            for (int c = 0; c < nw && !found; c++) {
                unsigned mb = rq[a * kEnumWords + c];
                while (mb && !found) {
                    const int bb = 32 * c + __ffs(mb) - 1;
                    mb &= mb - 1;
                    for (int c2 = 0; c2 < nw; c2++) {
                        const unsigned x = rq[a * kEnumWords + c2] & rq[bb * kEnumWords + c2];
                        const int pc = __popc(x);
                        if (rk < pc) { bk = bb; lk = 32 * c2 + select_bit(x, rk); found = true; break; }
                        rk -= pc;
                    }
                }
            }
            const long long q = base4 + t;
            if (q < B.n4_cap) {
                int* out = B.c4 + 4 * q;
                out[0] = gi; out[1] = sg[a]; out[2] = sg[bk]; out[3] = sg[lk];
                if (B.c4e) {
                    B.c4e[3 * q] = (int)(b0 + a);
                    B.c4e[3 * q + 1] = (int)(b0 + bk);
                    B.c4e[3 * q + 2] = (int)(b0 + lk);
                }
            }
        }
    }
}

template <bool FILL, int G>
void launch_enuma(const BatchView& B, cudaStream_t st) {
    constexpr int NG = kEnumWarps / G;
    const long long want = (long long)sm_count() * 4;   // 4 blocks of 8 warps per SM
    const long long need = (B.n_atoms_total + NG - 1) / NG;
    const unsigned grid = (unsigned)(want < need ? want : need);
    count_launch(), k_enuma<FILL, G><<<grid, 32 * kEnumWarps, 0, st>>>(B);
}

// --- capacity checks and accumulator reset ---------------------------------
__global__ void k_check(BatchView B) {
    if (B.l2_off[B.n_atoms_total] > B.n2_cap) atomicOr(&B.flags[0], 2);
    if (B.e_off3[B.n2_cap] > B.n3_cap) atomicOr(&B.flags[0], 4);
    if (B.e_off4[B.n2_cap] > B.n4_cap) atomicOr(&B.flags[0], 8);
}

__global__ void k_reset(BatchView B) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6LL * B.n_sys) B.minmax[i] = (i % 6) < 3 ? ~0ull : 0ull;
    if (i < 8LL * B.n_sys) B.ev[i] = 0.0;
    if (i < 3 * B.n_in_total) B.force[i] = 0.0;
    if (i < 8) B.flags[i] = 0;
    if (i < 2) B.queue[i] = 0ull;
    if (i < B.n_sys) B.sys[i].err = 0;
}

// --- exclusive scan (three phases, recursive on block sums) -----------------
constexpr int kScanBlock = 1024;

__global__ void k_scan_block(const int* in, const long long* in64, long long* out, long long n, long long* sums) {
    __shared__ long long wsum[32];
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    long long v = 0;
    if (i < n) v = in ? (long long)in[i] : in64[i];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
    for (int off = 1; off < 32; off <<= 1) {
        long long y = __shfl_up_sync(kFull, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        long long t = wsum[lane];
        for (int off = 1; off < 32; off <<= 1) {
            long long y = __shfl_up_sync(kFull, t, off);
            if (lane >= off) t += y;
        }
        wsum[lane] = t;
    }
    __syncthreads();
    const long long incl = x + (w ? wsum[w - 1] : 0);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = incl;
}

__global__ void k_scan_add(long long* out, long long n, const long long* offs) {
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += offs[blockIdx.x];
}

__global__ void k_scan_total(long long* out, long long n, const int* in, const long long* in64) {
    // out[n] = out[n-1] + in[n-1]
    if (n == 0) { out[0] = 0; return; }
    out[n] = out[n - 1] + (in ? (long long)in[n - 1] : in64[n - 1]);
}

void scan_rec(const int* in, const long long* in64, long long* out, long long n, long long* tmp, cudaStream_t st) {
    if (n == 0) return;
    const long long nb = (n + kScanBlock - 1) / kScanBlock;
    long long* sums = tmp;
    long long* sums_scan = tmp + nb;
    count_launch(), k_scan_block<<<(unsigned)nb, kScanBlock, 0, st>>>(in, in64, out, n, sums);
    if (nb > 1) {
        scan_rec(nullptr, sums, sums_scan, nb, tmp + 2 * nb, st);
        count_launch(), k_scan_add<<<(unsigned)nb, kScanBlock, 0, st>>>(out, n, sums_scan);
    }
}

unsigned grid_for(long long n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

// Kernel launches enqueued by this library (all threads; a per-engine count
// is the difference across one enqueue sequence on that engine's thread).
static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launch_counter() { return g_launches.load(std::memory_order_relaxed); }

size_t scan_tmp_bytes(long long n) {
    size_t total = 0;
    long long m = n;
    while (m > 1) {
        long long nb = (m + kScanBlock - 1) / kScanBlock;
        total += 2 * nb;
        m = nb;
    }
    return (total + 16) * sizeof(long long);
}

namespace {

// Up to two scans side by side (blockIdx.y): tiles of kScanBlock scanned in
// place with the tile sums recorded; a single tile also writes the total.
struct ScanPair {
    const int* in[2];
    long long* out[2];
    long long* sums[2];
};

__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(ScanPair a, long long n) {
    const int y = blockIdx.y;
    __shared__ long long wsum[32];
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    const long long v = i < n ? (long long)a.in[y][i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
    for (int off = 1; off < 32; off <<= 1) {
        const long long t = __shfl_up_sync(kFull, x, off);
        if (lane >= off) x += t;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        long long t = wsum[lane];
        for (int off = 1; off < 32; off <<= 1) {
            const long long u = __shfl_up_sync(kFull, t, off);
            if (lane >= off) t += u;
        }
        wsum[lane] = t;
    }
    __syncthreads();
    const long long incl = x + (w ? wsum[w - 1] : 0);
    if (i < n) a.out[y][i] = incl - v;
    if (threadIdx.x == kScanBlock - 1) {
        a.sums[y][blockIdx.x] = incl;
        if (gridDim.x == 1) a.out[y][n] = incl;
    }
}

// tile b adds the sum of tiles 0..b-1 (reduced by the block itself, at most
// kScanBlock tiles); the last tile writes the total at out[n]
__global__ void __launch_bounds__(kScanBlock) k_scan_offsets(ScanPair a, long long n) {
    const int y = blockIdx.y;
    const int b = blockIdx.x;
    __shared__ long long wsum[32];
    long long v = threadIdx.x < b ? a.sums[y][threadIdx.x] : 0;
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    long long offs = 0;
    for (int k = 0; k < kScanBlock / 32; k++) offs += wsum[k];
    const long long i = (long long)b * kScanBlock + threadIdx.x;
    if (i < n) a.out[y][i] += offs;
    if (b == (int)gridDim.x - 1 && threadIdx.x == 0) a.out[y][n] = offs + a.sums[y][b];
}

// nb <= kScanBlock tiles: two launches for one or two arrays
void scan_small(int m, const int* ia, long long* oa, const int* ib, long long* ob, long long n, long long* tmp,
                cudaStream_t st) {
    const long long nb = (n + kScanBlock - 1) / kScanBlock;
    ScanPair a;
    a.in[0] = ia; a.out[0] = oa; a.sums[0] = tmp;
    a.in[1] = ib; a.out[1] = ob; a.sums[1] = tmp + nb;
    const dim3 grid((unsigned)nb, (unsigned)m);
    count_launch(), k_scan_tiles<<<grid, kScanBlock, 0, st>>>(a, n);
    if (nb > 1) count_launch(), k_scan_offsets<<<grid, kScanBlock, 0, st>>>(a, n);
}

}  // namespace

void exclusive_scan(const int* in, long long* out, long long n, void* tmp, cudaStream_t st) {
    if (n > 0 && n <= (long long)kScanBlock * kScanBlock) {
        scan_small(1, in, out, in, out, n, (long long*)tmp, st);
        return;
    }
    scan_rec(in, nullptr, out, n, (long long*)tmp, st);
    count_launch(), k_scan_total<<<1, 1, 0, st>>>(out, n, in, nullptr);
}

void exclusive_scan2(const int* in_a, long long* out_a, const int* in_b, long long* out_b, long long n, void* tmp,
                     cudaStream_t st) {
    if (n > 0 && n <= (long long)kScanBlock * kScanBlock) {
        scan_small(2, in_a, out_a, in_b, out_b, n, (long long*)tmp, st);
        return;
    }
    exclusive_scan(in_a, out_a, n, tmp, st);
    exclusive_scan(in_b, out_b, n, tmp, st);
}

void launch_atoms(const BatchView& B, cudaStream_t st) {
    // small blocks: the per-atom cell algebra is FP64 work, spread over as many SMs as possible
    if (B.n_atoms_total) count_launch(), k_atoms<<<grid_for(B.n_atoms_total, 32), 32, 0, st>>>(B);
}
void launch_ghosts(const BatchView& B, cudaStream_t st) {
    if (B.n_ghost_total) count_launch(), k_ghosts<<<grid_for(B.n_ghost_total, 64), 64, 0, st>>>(B);
}
void launch_bin_setup(const BatchView& B, cudaStream_t st) {
    count_launch(), k_bin_setup<<<grid_for(B.n_sys, 128), 128, 0, st>>>(B);
}
void launch_bin_count(const BatchView& B, cudaStream_t st) {
    if (B.n_ghost_total) count_launch(), k_bin_count<<<grid_for(B.n_ghost_total, 256), 256, 0, st>>>(B);
}
void launch_bin_scatter(const BatchView& B, cudaStream_t st) {
    if (B.n_ghost_total) count_launch(), k_bin_scatter<<<grid_for(B.n_ghost_total, 256), 256, 0, st>>>(B, B.bin_start);
}
void launch_bin_sort(const BatchView& B, cudaStream_t st) {
    if (!B.n_bins_total) return;
    // bins per warp: one while that still gives a few warps per resident slot
    // (a small batch's bins are few and mostly occupied), else 32 (a large
    // batch reserves many times the bins its ghost clouds occupy)
    const int per = B.n_bins_total > 64LL * 32 * sm_count() ? 32 : 1;
    const long long warps = (B.n_bins_total + per - 1) / per;
    count_launch(), k_bin_rank<<<grid_for(warps * 32, 256), 256, 0, st>>>(B, B.bin_start, per);
}
void launch_l2(const BatchView& B, int* l2_owner, bool fill, cudaStream_t st) {
    if (!B.n_atoms_total) return;
    const unsigned grid = grid_for(B.n_atoms_total * 32, kL2Block);
    if (fill) count_launch(), k_l2<true><<<grid, kL2Block, 0, st>>>(B, B.bin_start, l2_owner);
    else count_launch(), k_l2<false><<<grid, kL2Block, 0, st>>>(B, B.bin_start, l2_owner);
}
void launch_enum(const BatchView& B, const int* l2_owner, bool fill, cudaStream_t st) {
    if (!B.n2_cap) return;
    if (B.enum_serial) {
        long long want = (long long)sm_count() * 16;
        long long need = (B.n2_cap + 127) / 128;
        const unsigned grid = (unsigned)(want < need ? want : need);
        if (fill) count_launch(), k_enum<true><<<grid, 128, 0, st>>>(B, l2_owner);
        else count_launch(), k_enum<false><<<grid, 128, 0, st>>>(B, l2_owner);
        return;
    }
    // warps per atom: the fewest that still give about two warps per
    // resident warp slot (32 per SM)
    const long long target = 64LL * sm_count();
    const long long n = B.n_atoms_total;
    const int G = n >= target ? 1 : 2 * n >= target ? 2 : 4 * n >= target ? 4 : 8;
    switch (G) {
    case 1: fill ? launch_enuma<true, 1>(B, st) : launch_enuma<false, 1>(B, st); break;
    case 2: fill ? launch_enuma<true, 2>(B, st) : launch_enuma<false, 2>(B, st); break;
    case 4: fill ? launch_enuma<true, 4>(B, st) : launch_enuma<false, 4>(B, st); break;
    default: fill ? launch_enuma<true, 8>(B, st) : launch_enuma<false, 8>(B, st); break;
    }
}
void launch_check(const BatchView& B, cudaStream_t st) { count_launch(), k_check<<<1, 1, 0, st>>>(B); }
void launch_reset(const BatchView& B, cudaStream_t st) {
    long long n = 8LL * B.n_sys;
    if (3 * B.n_in_total > n) n = 3 * B.n_in_total;
    if (n < 8) n = 8;
    count_launch(), k_reset<<<grid_for(n, 256), 256, 0, st>>>(B);
}

}  // namespace ck
