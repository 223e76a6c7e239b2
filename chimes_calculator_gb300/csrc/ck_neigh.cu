// LAMMPS pair-style path: ChIMES on a caller's full neighbour list with ghost
// atoms, as pair_style chimesFF computes it (etc/lmp/src/pair_chimes.cpp).
//
//   * 1-body for every atom of ilist, 2-body for every listed (i, j) with
//     tag[j] > tag[i] (compute, :572-655);
//   * 3-/4-body clusters built from the list of i only (build_mb_neighlists,
//     :321-478): j, k, l with tags not below the earlier members', every
//     distance below the padded cutoff max_cutoff_nB + skin; the clusters are
//     rebuilt only when the caller says so (LAMMPS: neighbor->ago == 0) and
//     evaluated every call with the current positions by the batch force
//     kernels, which apply the per-tuple cutoffs of compute_3B/4B.
//
// The batch kernels see the atoms through an identity mapping: atom index =
// ghost slot = force slot, positions as "fractional" coordinates of a unit
// cell, so their pair geometry is x_b - x_a (PairCHIMES::get_dist, :303-312).
// Distances that decide list membership are taken in FP64 with separate
// roundings (no fused multiply-add), as the reference computes them.
#include <cuda_runtime.h>

#include <cstdint>

#include "ck_common.h"
#include "ck_force_common.cuh"
#include "ck_kernels.h"
#include "ck_math.cuh"
#include "ck_tab.cuh"

namespace ck {

namespace {

__device__ __forceinline__ double nl_dist(const double* x, int i, int j, double* dr) {
    const double d0 = __dsub_rn(x[3 * (long long)j + 0], x[3 * (long long)i + 0]);
    const double d1 = __dsub_rn(x[3 * (long long)j + 1], x[3 * (long long)i + 1]);
    const double d2 = __dsub_rn(x[3 * (long long)j + 2], x[3 * (long long)i + 2]);
    if (dr) { dr[0] = d0; dr[1] = d1; dr[2] = d2; }
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
}

// Distance of one pair for cutoff tests: the FP32 distance first, the FP64
// one (as nl_dist computes it) only when the FP32 value is within the margin
// of the cutoff; the FP64 value is kept for further tests of the same pair.
struct NlDist {
    const double* x;
    int i, j;
    float df;
    double exact;
    bool have;
    __device__ NlDist(const double* x_, const float* xf, int i_, int j_) : x(x_), i(i_), j(j_), exact(0.0), have(false) {
        const float* a = xf + 3 * (long long)i;
        const float* b = xf + 3 * (long long)j;
        const float ex = b[0] - a[0], ey = b[1] - a[1], ez = b[2] - a[2];
        df = sqrtf(ex * ex + ey * ey + ez * ez);
    }
    __device__ bool lt(double c, float lo, float hi) {
        if (df < lo) return true;
        if (df >= hi) return false;
        if (!have) {
            exact = nl_dist(x, i, j, nullptr);
            have = true;
        }
        return exact < c;
    }
};

__global__ void k_nl_xf(const double* x, float* xf, long long n) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) xf[k] = (float)x[k];
}

// list entry -> position of its atom in ilist
__global__ void k_nl_owner(NeighView N) {
    const long long ii = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= N.inum) return;
    for (long long e = N.off[ii]; e < N.off[ii + 1]; e++) N.owner[e] = (int)ii;
}

// identity atom <-> slot mapping of the batch kernels
__global__ void k_nl_identity(BatchView B) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= B.n_atoms_total) return;
    B.atom_sys[q] = 0;
    B.atom_orig[q] = (int)q;
    B.ghost_parent[q] = (int)q;
}

// 1-body over ilist and 2-body over the list entries (compute, :572-655)
template <typename CT>
__global__ void __launch_bounds__(256) k_nl_pairs(BatchView B, NeighView N) {
    const DevParamSet& P = B.psets[B.sys[0].pset];
    const double* x = B.ghost_fs;
    EVAcc acc;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long ntot = N.nent > N.inum ? N.nent : N.inum;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < ntot; e += stride) {
        double vir[6] = {0, 0, 0, 0, 0, 0};
        if (e < N.inum) {
            const int a = N.ilist[e];
            acc.add(B, 0, P.eoff[B.atom_type[a]], vir);
            tally_atoms(B, &a, 1, P.eoff[B.atom_type[a]], vir);
        }
        if (e >= N.nent) continue;
        const int i = N.ilist[N.owner[e]];
        const int j = N.neigh[e];
        if (N.tag[j] <= N.tag[i]) continue;
        double dr[3];
        const double dist = nl_dist(x, i, j, dr);
        const int pt = P.pair_map[B.atom_type[i] * P.ntypes + B.atom_type[j]];
        const PairRec pr = P.pairs[pt];
        if (dist >= pr.rout) continue;
        double E, fs;
        if (P.tab2) {
            // compute_2B_tab (chimesFF.cpp:1782-1867): table energy and force
            // scalar; the penalty only records badness (the table includes it)
            const int ts = tab2_lookup(P, pt, dist, E, fs);
            if (ts) atomicOr(&B.flags[5], ts);
            if (dist - P.pen_dist < pr.rin) {
                atomicMax(&B.flags[2], dist < pr.rin ? 2 : 1);
                if (pr.rin + P.pen_dist - dist > 0.0) atomicAdd(&B.flags[3], 1);
            }
        } else {
            pair_2b<CT>(P, pr, dist, B.flags, E, fs);
        }
        add_force(B, i, fs * dr[0], fs * dr[1], fs * dr[2]);
        add_force(B, j, -fs * dr[0], -fs * dr[1], -fs * dr[2]);
        virial_add(vir, fs, dr);
        acc.add(B, 0, E, vir);
        const int pair[2] = {i, j};
        tally_atoms(B, pair, 2, E, vir);
    }
    acc.flush_warp(B);
}

// Cluster lists (build_mb_neighlists, :321-478): one warp per list entry
// (i, j); lanes take consecutive k of i's list, a ballot and prefix count
// emit triplets in list order; for each k that can start a quadruplet, lanes
// take consecutive l.  Count pass (FILL = false) and fill pass.
template <bool FILL>
__global__ void __launch_bounds__(256) k_nl_enum(BatchView B, NeighView N) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const double* x = B.ghost_fs;
    const double c3p = N.c3p, c4p = N.c4p;
    for (long long e = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < N.nent; e += nwarps) {
        long long n3 = 0, n4 = 0, o3 = 0, o4 = 0;
        if (FILL) { o3 = B.e_off3[e]; o4 = B.e_off4[e]; }
        const int ii = N.owner[e];
        const int i = N.ilist[ii];
        const int j = N.neigh[e];
        const long long ti = N.tag[i], tj = N.tag[j];
        bool go = j != i && tj >= ti;
        bool ij3 = false, ij4 = false;
        if (go) {
            NlDist Dij(x, N.xf, i, j);
            ij3 = Dij.lt(c3p, N.c3lo, N.c3hi);
            ij4 = Dij.lt(c4p, N.c4lo, N.c4hi);
            go = ij3 || ij4;
        }
        if (go) {
            const long long b0 = N.off[ii], b1 = N.off[ii + 1];
            for (long long kb = b0; kb < b1; kb += 32) {
                const long long kk = kb + lane;
                bool ok3 = false, ok4 = false;
                int k = -1;
                long long tk = 0;
                if (kk < b1) {
                    k = N.neigh[kk];
                    tk = N.tag[k];
                    if (k != i && k != j && tk >= ti && tk >= tj) {
                        NlDist Dik(x, N.xf, i, k);
                        const bool ik3 = Dik.lt(c3p, N.c3lo, N.c3hi), ik4 = Dik.lt(c4p, N.c4lo, N.c4hi);
                        if (ik3 || ik4) {
                            NlDist Djk(x, N.xf, j, k);
                            ok3 = N.has3 && ij3 && ik3 && Djk.lt(c3p, N.c3lo, N.c3hi);
                            ok4 = N.has4 && ij4 && ik4 && Djk.lt(c4p, N.c4lo, N.c4hi);
                        }
                    }
                }
                const unsigned m3 = __ballot_sync(kFull, ok3);
                if (FILL && ok3) {
                    const long long q = o3 + n3 + __popc(m3 & lt);
                    if (q < B.n3_cap) {
                        int* out = B.c3 + 3 * q;
                        out[0] = i; out[1] = j; out[2] = k;
                    }
                }
                n3 += __popc(m3);
                unsigned m4 = __ballot_sync(kFull, ok4);
                while (m4) {
                    const int src = __ffs(m4) - 1;
                    m4 &= m4 - 1;
                    const int ks = __shfl_sync(kFull, k, src);
                    const long long tks = __shfl_sync(kFull, tk, src);
                    for (long long lb = b0; lb < b1; lb += 32) {
                        const long long ll = lb + lane;
                        bool okl = false;
                        int l = -1;
                        if (ll < b1) {
                            l = N.neigh[ll];
                            const long long tl = N.tag[l];
                            if (l != i && l != j && l != ks && tl >= ti && tl >= tj && tl >= tks)
                                okl = NlDist(x, N.xf, i, l).lt(c4p, N.c4lo, N.c4hi) &&
                                      NlDist(x, N.xf, j, l).lt(c4p, N.c4lo, N.c4hi) &&
                                      NlDist(x, N.xf, ks, l).lt(c4p, N.c4lo, N.c4hi);
                        }
                        const unsigned ml = __ballot_sync(kFull, okl);
                        if (FILL && okl) {
                            const long long q = o4 + n4 + __popc(ml & lt);
                            if (q < B.n4_cap) {
                                int* out = B.c4 + 4 * q;
                                out[0] = i; out[1] = j; out[2] = ks; out[3] = l;
                            }
                        }
                        n4 += __popc(ml);
                    }
                }
            }
        }
        if (!FILL && lane == 0) { B.e_cnt3[e] = (int)n3; B.e_cnt4[e] = (int)n4; }
    }
}

// Tabulated 3-body term (compute_3B_tab, chimesFF.cpp:2183-2322) in two
// passes.  Selection: one thread per listed triplet applies compute_3B's type
// and per-pair outer-cutoff checks (the lists hold every triplet within the
// padded cutoffs, most of them outside the table's cutoffs) and appends the
// evaluated ones with their distances (warp-aggregated atomics).  Evaluation:
// one thread per selected triplet, so no lane idles in the FP64-bound look-up.
__global__ void __launch_bounds__(256) k_nl_tab3_sel(BatchView B, long long n3, int* sel, double* selr,
                                                     unsigned long long* count) {
    const DevParamSet& P = B.psets[B.sys[0].pset];
    const double* x = B.ghost_fs;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n3; base += stride) {
        const long long q = base + lane;
        bool pass = false;
        double r[3] = {0.0, 0.0, 0.0};
        if (q < n3) {
            const int id[3] = {B.c3[3 * q], B.c3[3 * q + 1], B.c3[3 * q + 2]};
            const int u = (B.atom_type[id[0]] * P.ntypes + B.atom_type[id[1]]) * P.ntypes + B.atom_type[id[2]];
            const TupleRec& R = P.t3[u];
            if (R.type_id >= 0) {
                pass = true;
                for (int p = 0; p < 3 && pass; p++) {
                    const int a = id[p == 2 ? 1 : 0], b = id[p == 0 ? 1 : 2];   // ij, ik, jk
                    NlDist D(x, B.pos_f, a, b);
                    const float m = B.float_eps + 1e-6f * R.rout_f[p];
                    pass = D.lt(R.rout[p], R.rout_f[p] - m, R.rout_f[p] + m);
                    if (pass) r[p] = D.have ? D.exact : nl_dist(x, a, b, nullptr);
                }
            }
        }
        const unsigned m = __ballot_sync(kFull, pass);
        if (!m) continue;
        const int leader = __ffs(m) - 1;
        unsigned long long b0 = 0;
        if (lane == leader) b0 = atomicAdd(count, (unsigned long long)__popc(m));
        b0 = __shfl_sync(kFull, b0, leader);
        if (pass) {
            const unsigned long long s = b0 + __popc(m & ((1u << lane) - 1u));
            sel[s] = (int)q;
            selr[3 * s] = r[0];
            selr[3 * s + 1] = r[1];
            selr[3 * s + 2] = r[2];
        }
    }
}

__global__ void __launch_bounds__(128) k_nl_tab3(BatchView B, const int* sel, const double* selr,
                                                 const unsigned long long* count) {
    const DevParamSet& P = B.psets[B.sys[0].pset];
    const double* x = B.ghost_fs;
    const long long n = (long long)*count;
    EVAcc acc;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += stride) {
        const long long q = sel[s];
        const int id[3] = {B.c3[3 * q], B.c3[3 * q + 1], B.c3[3 * q + 2]};
        const int u = (B.atom_type[id[0]] * P.ntypes + B.atom_type[id[1]]) * P.ntypes + B.atom_type[id[2]];
        const int type_id = P.t3[u].type_id;
        double dr[3][3];
        nl_dist(x, id[0], id[1], dr[0]);   // ij
        nl_dist(x, id[0], id[2], dr[1]);   // ik
        nl_dist(x, id[1], id[2], dr[2]);   // jk
        double v[4];
        const int ts = tab3_lookup_sep(P, type_id, selr[3 * s], selr[3 * s + 1], selr[3 * s + 2], v);
        if (ts) atomicOr(&B.flags[5], ts);
        // forces in the reference's order: ij on (i, j), ik on (i, k), jk on (j, k)
        double f[3][3];
        for (int c = 0; c < 3; c++) {
            const double a = v[1] * dr[0][c], b = v[2] * dr[1][c], g = v[3] * dr[2][c];
            f[0][c] = a + b;
            f[1][c] = g - a;
            f[2][c] = -b - g;
        }
        // stress -= fs_p * (dr_p (x) dr_p), pair by pair (distance-tensor form)
        double vir[6] = {0, 0, 0, 0, 0, 0};
        for (int p = 0; p < 3; p++) {
            const double* d = dr[p];
            const double fsp = v[1 + p];
            vir[0] -= fsp * (d[0] * d[0]);
            vir[1] -= fsp * (d[0] * d[1]);
            vir[2] -= fsp * (d[0] * d[2]);
            vir[3] -= fsp * (d[1] * d[1]);
            vir[4] -= fsp * (d[1] * d[2]);
            vir[5] -= fsp * (d[2] * d[2]);
        }
        for (int a = 0; a < 3; a++) add_force(B, id[a], f[a][0], f[a][1], f[a][2]);
        acc.add(B, 0, v[0], vir);
        tally_atoms(B, id, 3, v[0], vir);
    }
    acc.flush_warp(B);
}

unsigned grid_of(long long n, int block, long long cap_blocks) {
    long long need = (n + block - 1) / block;
    if (need < 1) need = 1;
    return (unsigned)(need < cap_blocks ? need : cap_blocks);
}

}  // namespace

void launch_nl_setup(const BatchView& B, const NeighView& N, cudaStream_t st) {
    if (N.inum > 0) count_launch(), k_nl_owner<<<grid_of(N.inum, 128, 1LL << 30), 128, 0, st>>>(N);
    if (B.n_atoms_total > 0)
        count_launch(), k_nl_identity<<<grid_of(B.n_atoms_total, 256, 1LL << 30), 256, 0, st>>>(B);
}

void launch_nl_enum(const BatchView& B, const NeighView& N, bool fill, cudaStream_t st) {
    if (N.nent <= 0) return;
    const unsigned grid = grid_of(N.nent * 32, 256, (long long)sm_count() * 8);
    if (fill) count_launch(), k_nl_enum<true><<<grid, 256, 0, st>>>(B, N);
    else count_launch(), k_nl_enum<false><<<grid, 256, 0, st>>>(B, N);
}

void launch_nl_pairs(const BatchView& B, const NeighView& N, int precision, cudaStream_t st) {
    const long long ntot = N.nent > N.inum ? N.nent : N.inum;
    if (ntot <= 0) return;
    const unsigned grid = grid_of(ntot, 256, (long long)sm_count() * 8);
    // FP64 in both precision forms, as the batch path's 1-/2-body stage
    // (alternating 2-body series of fitted force fields cancel in FP32)
    (void)precision;
    count_launch(), k_nl_pairs<double><<<grid, 256, 0, st>>>(B, N);
}

void launch_nl_tab3(const BatchView& B, long long n3, int* sel, double* selr, unsigned long long* count,
                    cudaStream_t st) {
    if (n3 <= 0) return;
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
    count_launch(), k_nl_tab3_sel<<<grid_of(n3, 256, (long long)sm_count() * 8), 256, 0, st>>>(B, n3, sel, selr,
                                                                                                count);
    // the selected count stays on the device: the grid covers the listed triplets
    count_launch(), k_nl_tab3<<<grid_of(n3, 128, (long long)sm_count() * 8), 128, 0, st>>>(B, sel, selr, count);
}

void launch_nl_xf(const double* x, float* xf, long long n, cudaStream_t st) {
    if (n <= 0) return;
    count_launch(), k_nl_xf<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, xf, n);
}

}  // namespace ck
