// Cluster-list build on the GPU: periodic ghost images, the bin grid, the 2B
// neighbour lists and the 3B/4B cluster enumeration.
//
// The lists must be the reference's lists exactly (same members, same order),
// because cluster membership is decided by floating-point distance tests.
// Every floating-point step here therefore uses explicit round-to-nearest
// intrinsics (__dmul_rn/__dadd_rn/__dsub_rn/__ddiv_rn/__dsqrt_rn), which the
// compiler never fuses, in the reference's evaluation order:
//   set-up, wrap, reorient, ghosts ... serial_interface/src/serial_chimes_interface.cpp:150-587
//   bins and lists ................... serial_chimes_interface.cpp:588-864
//   get_dist ......................... serial_interface/src/serial_chimes_interface.h:141-215
#include <cuda_runtime.h>

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

// get_dist on stored fractional coordinates: |H (f_j - f_i)|
__device__ __forceinline__ double dist_frac(const double* H, const double* fi, const double* fj) {
    double dx = sub(fj[0], fi[0]), dy = sub(fj[1], fi[1]), dz = sub(fj[2], fi[2]);
    double r0 = add(add(mul(H[0], dx), mul(H[1], dy)), mul(H[2], dz));
    double r1 = add(add(mul(H[3], dx), mul(H[4], dy)), mul(H[5], dz));
    double r2 = add(add(mul(H[6], dx), mul(H[7], dy)), mul(H[8], dz));
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

__device__ __forceinline__ void ghost_shift(int img, int n, int side, int& i, int& j, int& k) {
    int full = img - 1;
    int center = (n * side + n) * side + n;
    if (full >= center) full++;
    i = full / (side * side) - n;
    j = (full / side) % side - n;
    k = full % side - n;
}

// --- 1. atoms: replicate (small=true), wrap, reorient -----------------------
// simulation_system::init (:196-322) and reorient (:352-405)
__global__ void k_atoms(BatchView B) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B.n_atoms_total) return;
    const int s = find_sys_atom(B.sys, B.n_sys, r);
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
    const long long g = d.ghost_off + rl;
    for (int c = 0; c < 3; c++) {
        B.ghost_fs[3 * g + c] = fa[c];
        B.ghost_xn[3 * g + c] = xn[c];
        B.ghost_fn[3 * g + c] = fn[c];
    }
    B.ghost_parent[g] = (int)r;
    B.atom_sys[r] = s;
    B.atom_type[r] = B.in_type[d.in_off + a];
    B.atom_orig[r] = (int)(d.in_off + a);
}

// --- 2. ghosts + bounding box ------------------------------------------------
// build_layered_system (:546-585) for both the input-cell system (fractional
// coordinates for the force evaluation) and the reoriented system (Cartesian and
// fractional coordinates for the lists); the min/max of the reoriented cloud
// (build_neigh_lists :590-610) is reduced on the fly.
__global__ void k_ghosts(BatchView B) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = g < B.n_ghost_total;
    int s = -1;
    double xn[3] = {0, 0, 0};
    if (valid) {
        s = find_sys_ghost(B.sys, B.n_sys, g);
        const SysDesc& d = B.sys[s];
        const long long gl = g - d.ghost_off;
        const int img = (int)(gl / d.n_atoms), a = (int)(gl % d.n_atoms);
        if (img == 0) {
            xn[0] = B.ghost_xn[3 * g]; xn[1] = B.ghost_xn[3 * g + 1]; xn[2] = B.ghost_xn[3 * g + 2];
        } else {
            int i, j, k;
            ghost_shift(img, d.n_layers, d.side, i, j, k);
            const long long src = d.ghost_off + a;
            double t[3], p[3], o[3];
            t[0] = add(B.ghost_fs[3 * src], (double)i);
            t[1] = add(B.ghost_fs[3 * src + 1], (double)j);
            t[2] = add(B.ghost_fs[3 * src + 2], (double)k);
            mv(d.h, t[0], t[1], t[2], p);
            mv(d.hi, p[0], p[1], p[2], o);
            B.ghost_fs[3 * g] = o[0]; B.ghost_fs[3 * g + 1] = o[1]; B.ghost_fs[3 * g + 2] = o[2];
            t[0] = add(B.ghost_fn[3 * src], (double)i);
            t[1] = add(B.ghost_fn[3 * src + 1], (double)j);
            t[2] = add(B.ghost_fn[3 * src + 2], (double)k);
            mv(d.hn, t[0], t[1], t[2], xn);
            mv(d.hni, xn[0], xn[1], xn[2], o);
            B.ghost_xn[3 * g] = xn[0]; B.ghost_xn[3 * g + 1] = xn[1]; B.ghost_xn[3 * g + 2] = xn[2];
            B.ghost_fn[3 * g] = o[0]; B.ghost_fn[3 * g + 1] = o[1]; B.ghost_fn[3 * g + 2] = o[2];
            B.ghost_parent[g] = (int)(d.atom_off + a);
        }
    }
    const int lane = threadIdx.x & 31;
    const int s0 = __shfl_sync(kFull, s, 0);
    if (s0 < 0) return;   // whole warp out of range (valid lanes form a prefix)
    const bool uniform = __all_sync(kFull, !valid || s == s0);
    unsigned long long kmin[3], kmax[3];
    for (int c = 0; c < 3; c++) {
        kmin[c] = valid ? okey(xn[c]) : ~0ull;
        kmax[c] = valid ? okey(xn[c]) : 0ull;
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
        atomicExch(&B.flags[0], 1);
    }
}

__device__ __forceinline__ bool bin_of(const SysDesc& d, const double* x, int& bx, int& by, int& bz) {
    bx = (int)floor(__ddiv_rn(sub(x[0], d.minpos[0]), d.search));
    by = (int)floor(__ddiv_rn(sub(x[1], d.minpos[1]), d.search));
    bz = (int)floor(__ddiv_rn(sub(x[2], d.minpos[2]), d.search));
    return true;
}

// --- 4. bin population (:644-678) -------------------------------------------
__global__ void k_bin_count(BatchView B) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= B.n_ghost_total) return;
    const int s = find_sys_ghost(B.sys, B.n_sys, g);
    const SysDesc& d = B.sys[s];
    if (d.err) { B.ghost_bin[g] = -1; return; }
    int bx, by, bz;
    bin_of(d, &B.ghost_xn[3 * g], bx, by, bz);
    const long long total = (long long)d.nb[0] * d.nb[1] * d.nb[2];
    if (bx < 0 || by < 0 || bz < 0) { atomicExch(&B.flags[1], 1); B.ghost_bin[g] = -1; return; }
    const long long ib = bx + (long long)by * d.nb[0] + (long long)bz * d.nb[0] * d.nb[1];
    if (ib >= total) { atomicExch(&B.flags[1], 2); B.ghost_bin[g] = -1; return; }
    B.ghost_bin[g] = (int)ib;
    atomicAdd(&B.bin_count[d.bin_off + ib], 1);
}

__global__ void k_bin_scatter(BatchView B, const long long* bin_start) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= B.n_ghost_total) return;
    const int ib = B.ghost_bin[g];
    if (ib < 0) return;
    const int s = find_sys_ghost(B.sys, B.n_sys, g);
    const long long b = B.sys[s].bin_off + ib;
    const long long pos = bin_start[b] + atomicAdd(&B.bin_fill[b], 1);
    B.bin_items[pos] = (int)g;
}

// each bin's members in ascending ghost order (the reference pushes ghosts
// into bins in index order)
__global__ void k_bin_sort(BatchView B, const long long* bin_start) {
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B.n_bins_total) return;
    const long long s0 = bin_start[b];
    const int n = B.bin_count[b];
    int* v = B.bin_items + s0;
    for (int i = 1; i < n; i++) {
        int key = v[i], j = i - 1;
        while (j >= 0 && v[j] > key) { v[j + 1] = v[j]; j--; }
        v[j + 1] = key;
    }
}

// --- 5. 2B neighbour lists (:680-731): one warp per atom --------------------
template <bool FILL>
__global__ void k_l2(BatchView B, const long long* bin_start, int* l2_owner) {
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B.n_atoms_total) return;
    const long long r = warp;
    const int s = B.atom_sys[r];
    const SysDesc& d = B.sys[s];
    if (d.err) { if (!FILL && lane == 0) B.l2_count[r] = 0; return; }
    const long long gi = d.ghost_off + (r - d.atom_off);
    const double fi[3] = {B.ghost_fn[3 * gi], B.ghost_fn[3 * gi + 1], B.ghost_fn[3 * gi + 2]};
    double hn[9];
    for (int c = 0; c < 9; c++) hn[c] = d.hn[c];
    const double sd = d.search;
    int bx, by, bz;
    bin_of(d, &B.ghost_xn[3 * gi], bx, by, bz);
    if (bx < 1 || by < 1 || bz < 1) {
        if (lane == 0) { atomicExch(&B.flags[1], 3); if (!FILL) B.l2_count[r] = 0; }
        return;
    }
    const long long total = (long long)d.nb[0] * d.nb[1] * d.nb[2];
    long long base = FILL ? B.l2_off[r] : 0;
    int count = 0;
    for (int i = bx - 1; i <= bx + 1; i++)
        for (int j = by - 1; j <= by + 1; j++)
            for (int k = bz - 1; k <= bz + 1; k++) {
                const long long ib = i + (long long)j * d.nb[0] + (long long)k * d.nb[0] * d.nb[1];
                if (ib >= total) {
                    if (lane == 0) atomicExch(&B.flags[1], 4);
                    continue;
                }
                const long long b = d.bin_off + ib;
                const long long st = bin_start[b];
                const int nb = B.bin_count[b];
                for (int q0 = 0; q0 < nb; q0 += 32) {
                    const int q = q0 + lane;
                    bool pred = false;
                    int ajj = -1;
                    double dd = 0.0;
                    if (q < nb) {
                        ajj = B.bin_items[st + q];
                        if (ajj != gi && r <= B.ghost_parent[ajj]) {
                            dd = dist_frac(hn, fi, &B.ghost_fn[3 * (long long)ajj]);
                            pred = dd < sd;
                        }
                    }
                    const unsigned bal = __ballot_sync(kFull, pred);
                    if (FILL && pred) {
                        const long long pos = base + count + __popc(bal & ((1u << lane) - 1u));
                        if (pos < B.n2_cap) {
                            B.l2_ghost[pos] = ajj;
                            B.l2_dist[pos] = dd;
                            l2_owner[pos] = (int)r;
                        }
                    }
                    count += __popc(bal);
                }
            }
    if (!FILL && lane == 0) B.l2_count[r] = count;
}

// --- 6. 3B/4B enumeration (:735-855): one thread per (i, j) list entry -----
// The valid_3mer / valid_4mer flags carry over between k iterations exactly as
// in the reference, so the emitted sets and their order match it.
template <bool FILL>
__device__ void enum_entry(const BatchView& B, const int* l2_owner, long long e);

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

template <bool FILL>
__device__ void enum_entry(const BatchView& B, const int* l2_owner, long long e) {
    const int r = l2_owner[e];
    const SysDesc& d = B.sys[B.atom_sys[r]];
    int n3 = 0, n4 = 0;
    long long o3 = 0, o4 = 0;
    if (FILL) { o3 = B.e_off3[e]; o4 = B.e_off4[e]; }
    const double c3 = d.c3, c4 = d.c4;
    if (d.has3 || d.has4) {
        double hn[9];
        for (int c = 0; c < 9; c++) hn[c] = d.hn[c];
        const int gi = (int)(d.ghost_off + (r - d.atom_off));
        const long long b0 = min(B.l2_off[r], B.n2_cap), b1 = min(B.l2_off[r + 1], B.n2_cap);
        const int jj = B.l2_ghost[e];
        const double dij = B.l2_dist[e];
        bool v3 = true, v4 = true;
        if (dij >= c3) v3 = false;
        if (dij >= c4) v4 = false;
        if (v3 || v4) {
            const double fj[3] = {B.ghost_fn[3 * (long long)jj], B.ghost_fn[3 * (long long)jj + 1],
                                  B.ghost_fn[3 * (long long)jj + 2]};
            const int pj = B.ghost_parent[jj];
            for (long long k = b0; k < b1; k++) {
                const int kk = B.l2_ghost[k];
                if (jj == kk) continue;
                const int pk = B.ghost_parent[kk];
                if (pj > pk) continue;
                const double dik = B.l2_dist[k];
                if (dik >= c3) v3 = false;
                if (dik >= c4) v4 = false;
                const double* fk = &B.ghost_fn[3 * (long long)kk];
                const double djk = dist_frac(hn, fj, fk);
                if (djk >= c3) v3 = false;
                if (djk >= c4) v4 = false;
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
                const double fkk[3] = {fk[0], fk[1], fk[2]};
                for (long long l = b0; l < b1; l++) {
                    const int ll = B.l2_ghost[l];
                    if (jj == ll || kk == ll) continue;
                    const int pl = B.ghost_parent[ll];
                    if (pj > pl) continue;
                    if (pk > pl) continue;
                    if (B.l2_dist[l] >= c4) continue;
                    const double* fl = &B.ghost_fn[3 * (long long)ll];
                    if (dist_frac(hn, fj, fl) >= c4) continue;
                    if (dist_frac(hn, fkk, fl) >= c4) continue;
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

static long long g_launches = 0;
void count_launch() { g_launches++; }
long long launch_counter() { return g_launches; }

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

void exclusive_scan(const int* in, long long* out, long long n, void* tmp, cudaStream_t st) {
    scan_rec(in, nullptr, out, n, (long long*)tmp, st);
    count_launch(), k_scan_total<<<1, 1, 0, st>>>(out, n, in, nullptr);
}

void launch_atoms(const BatchView& B, cudaStream_t st) {
    if (B.n_atoms_total) count_launch(), k_atoms<<<grid_for(B.n_atoms_total, 256), 256, 0, st>>>(B);
}
void launch_ghosts(const BatchView& B, cudaStream_t st) {
    if (B.n_ghost_total) count_launch(), k_ghosts<<<grid_for(B.n_ghost_total, 256), 256, 0, st>>>(B);
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
    if (B.n_bins_total) count_launch(), k_bin_sort<<<grid_for(B.n_bins_total, 128), 128, 0, st>>>(B, B.bin_start);
}
void launch_l2(const BatchView& B, int* l2_owner, bool fill, cudaStream_t st) {
    if (!B.n_atoms_total) return;
    const unsigned grid = grid_for(B.n_atoms_total * 32, 256);
    if (fill) count_launch(), k_l2<true><<<grid, 256, 0, st>>>(B, B.bin_start, l2_owner);
    else count_launch(), k_l2<false><<<grid, 256, 0, st>>>(B, B.bin_start, l2_owner);
}
void launch_enum(const BatchView& B, const int* l2_owner, bool fill, cudaStream_t st) {
    if (!B.n2_cap) return;
    long long want = (long long)sm_count() * 16;
    long long need = (B.n2_cap + 127) / 128;
    const unsigned grid = (unsigned)(want < need ? want : need);
    if (fill) count_launch(), k_enum<true><<<grid, 128, 0, st>>>(B, l2_owner);
    else count_launch(), k_enum<false><<<grid, 128, 0, st>>>(B, l2_owner);
}
void launch_check(const BatchView& B, cudaStream_t st) { count_launch(), k_check<<<1, 1, 0, st>>>(B); }
void launch_reset(const BatchView& B, cudaStream_t st) {
    long long n = 8LL * B.n_sys;
    if (3 * B.n_in_total > n) n = 3 * B.n_in_total;
    if (n < 8) n = 8;
    count_launch(), k_reset<<<grid_for(n, 256), 256, 0, st>>>(B);
}

}  // namespace ck
