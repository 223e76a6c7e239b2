// Factored 3-body and 4-body contraction.
//
// The per-coefficient form (k_forcen in ck_force.cu) spends about 2P+P FP64
// operations on every coefficient term: the product of P Chebyshev values and
// P gradient terms.  Here a cluster's pairs are split into row pairs (the
// first K) and column pairs (the rest), and the coefficient list of each
// ordered type tuple is stored twice, grouped by row and grouped by column
// (FactRow, ck_common.h).  With X_I = prod_{p<K} T_p, Y_J = prod_{p>=K} T_p:
//   S        = sum_I X_I z_I,            z_I = sum_J a_IJ Y_J     (row pass)
//   G_p, p<K = sum_I dX_I/dT_p.dT_p z_I                           (row pass)
//   G_p, p>=K= sum_J dY_J/dT_p.dT_p w_J, w_J = sum_I a_IJ X_I     (column pass)
// so a coefficient costs two multiply-adds, and the products are formed once
// per row or column.  The sums are the reference's (compute_3B/4B,
// chimesFF.cpp:1931-2176, 2496-2872) in another association order.
//
// Clusters are first bucketed by (parameter set, ordered type tuple), each
// bucket padded with -1 to a multiple of 32 slots, so every warp works on one
// tuple: loop bounds and coefficient loads are uniform across the warp (the
// loads are broadcasts).  TPC lanes share a cluster (TPC = 1, 2 or 4): one
// lane streams both passes' entries; two lanes (FP64) take one pass each;
// otherwise the lanes take whole records round robin.  Per-cluster tables
// (T, dT/dr per pair, Y and X) sit in shared memory interleaved by cluster,
// [entry][cluster].
#include <cuda_runtime.h>

#include <cstdint>

#include "ck_common.h"
#include "ck_force_common.cuh"
#include "ck_kernels.h"
#include "ck_math.cuh"

namespace ck {

namespace {

template <int NB>
struct Split;
template <>
struct Split<3> {
    static constexpr int K = 1;
};
template <>
struct Split<4> {
    static constexpr int K = 3;
};

template <typename CT>
struct EntOf;
template <>
struct EntOf<double> {
    using type = FactEntD;
};
template <>
struct EntOf<float> {
    using type = FactEntF;
};

template <typename CT, int NB>
__device__ __forceinline__ const typename EntOf<CT>::type* fact_ent(const DevParamSet& P);
template <> __device__ __forceinline__ const FactEntD* fact_ent<double, 3>(const DevParamSet& P) { return P.fe3d; }
template <> __device__ __forceinline__ const FactEntF* fact_ent<float, 3>(const DevParamSet& P) { return P.fe3f; }
template <> __device__ __forceinline__ const FactEntD* fact_ent<double, 4>(const DevParamSet& P) { return P.fe4d; }
template <> __device__ __forceinline__ const FactEntF* fact_ent<float, 4>(const DevParamSet& P) { return P.fe4f; }

// sum over entries [e0, e1) taken by lane gl of TPC: a * V[idx]; eight
// entries per round in two partial sums, so their loads overlap
template <typename CT, int TPC, int G, typename E>
__device__ __forceinline__ CT entry_sum(const E* __restrict__ ent, int e0, int e1, int gl, const CT* V, int grp) {
    CT z0 = CT(0), z1 = CT(0);
    int k = e0 + gl;
    for (; k + 7 * TPC < e1; k += 8 * TPC) {
        E q[8];
#pragma unroll
        for (int u = 0; u < 8; u++) q[u] = ent[k + u * TPC];
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
            z0 += CT(q[u].a) * V[(q[u].idx & 0xffff) * G + grp];
            z1 += CT(q[u + 1].a) * V[(q[u + 1].idx & 0xffff) * G + grp];
        }
    }
    for (; k < e1; k += TPC) {
        const E q = ent[k];
        z0 += CT(q.a) * V[(q.idx & 0xffff) * G + grp];
    }
    return z0 + z1;
}

// One pass over the entries [e0, e1) of nrec consecutive records (TPC = 1):
// z += a * V[idx] per entry; at an entry with the record-end bit (idx < 0)
// flush(record powers, z) and start the next record.  Entries are loaded
// eight (NOY: four) at a time regardless of where records end, so a short
// record does not pay its own load latency.
// The entry's multiplier is V[idx] (a table), or with NOY the product of the
// two column pairs' values T1[q1] T2[q2] (powers in the entry's high bits).
template <typename CT, int G, bool NOY, typename E>
__device__ __forceinline__ CT entry_value(const E& q, const CT* V, const CT* T2, int grp) {
    if constexpr (NOY) {
        const int c = q.idx >> 16;
        return V[(c & 31) * G + grp] * T2[((c >> kPowBits) & 31) * G + grp];
    } else {
        return V[(q.idx & 0xffff) * G + grp];
    }
}

template <typename CT, int G, bool NOY = false, typename E, typename F>
__device__ __forceinline__ void flat_pass(const E* __restrict__ ent, int e0, int e1, const FactRow* rec, int nrec,
                                          const CT* V, const CT* T2, int grp, F&& flush) {
    constexpr int NBAT = NOY ? 4 : 8;   // the NOY form keeps fewer entries in flight (registers)
    CT z = CT(0);
    int r = 0;
    int pw = nrec > 0 ? rec[0].pows : 0;
    for (int k = e0; k < e1; k += NBAT) {
        E q[NBAT];
        CT x[NBAT];
#pragma unroll
        for (int u = 0; u < NBAT; u++)
            if (k + u < e1) q[u] = ent[k + u];
#pragma unroll
        for (int u = 0; u < NBAT; u++)
            if (k + u < e1) x[u] = entry_value<CT, G, NOY>(q[u], V, T2, grp);
#pragma unroll
        for (int u = 0; u < NBAT; u++)
            if (k + u < e1) {
                z += CT(q[u].a) * x[u];
                if (q[u].idx < 0) {   // uniform: all lanes read the same entries
                    flush(pw, z);
                    z = CT(0);
                    r++;
                    pw = r < nrec ? rec[r].pows : 0;
                }
            }
    }
}

// The 3-body row sum without a Y table: sum over [e0, e1) of a * T1[q1] T2[q2],
// the column's powers q1, q2 taken from the entry's high bits.
template <typename CT, int G, typename E>
__device__ __forceinline__ CT entry_sum_noy(const E* __restrict__ ent, int e0, int e1, const CT* T1, const CT* T2,
                                            int grp) {
    CT z0 = CT(0), z1 = CT(0);
    int k = e0;
    for (; k + 3 < e1; k += 4) {
        E q[4];
#pragma unroll
        for (int u = 0; u < 4; u++) q[u] = ent[k + u];
#pragma unroll
        for (int u = 0; u < 4; u += 2) {
            const int c0 = q[u].idx >> 16, c1 = q[u + 1].idx >> 16;
            z0 += CT(q[u].a) * (T1[(c0 & 31) * G + grp] * T2[((c0 >> kPowBits) & 31) * G + grp]);
            z1 += CT(q[u + 1].a) * (T1[(c1 & 31) * G + grp] * T2[((c1 >> kPowBits) & 31) * G + grp]);
        }
    }
    for (; k < e1; k++) {
        const E q = ent[k];
        const int c = q.idx >> 16;
        z0 += CT(q.a) * (T1[(c & 31) * G + grp] * T2[((c >> kPowBits) & 31) * G + grp]);
    }
    return z0 + z1;
}

// Chebyshev tables and cutoff of pair p of a tuple (set_cheby_polys,
// chimesFF.h:542-628; get_fcut, chimesFF.h:347-386) with the tuple's
// precomputed reciprocals in place of the divisions.
__device__ __forceinline__ PairTab tuple_pair(const TupleRec& R, int p) {
    return PairTab{R.rin[p], R.rout[p], R.xavg[p], R.xdiff[p], R.inv_lam[p], R.inv_xdiff[p], R.fc_th[p], R.fc_inv[p]};
}

template <typename CT>
__device__ __forceinline__ void pair_setup(const DevParamSet& P, const PairTab& Q, double r, CT* T, CT* D,
                                           int stride, int nT, CT& fc, CT& fcd, int* flags) {
    const double rin = Q.rin;
    const bool oor = r < rin;
    const double rr = oor ? rin : r;
    const double e = exp(-rr * Q.inv_lam);
    const double xd = (e - Q.xavg) * Q.inv_xdiff;
    const double dxdr = -e * Q.inv_lam * Q.inv_xdiff;
    cheby_fill_strided<CT>(T, D, stride, nT, xd, dxdr, oor, r, rin, P.inner_smooth, flags);
    const double finv = Q.fc_inv;
    if (!P.tersoff) {
        const CT f0 = CT(1.0) - CT(r) * CT(finv);
        fc = f0 * f0 * f0;
        fcd = f0 * f0 * (CT(-3.0) * CT(finv));
    } else {
        const double th = Q.fc_th;
        if (r < th) { fc = CT(1); fcd = CT(0); }
        else if (r > Q.rout) { fc = CT(0); fcd = CT(0); }
        else {
            const CT f0 = CT(r - th) * CT(finv) * CT(kPi) + CT(kPi / 2.0);
            CT sn, cs;
            csincos<CT>(f0, &sn, &cs);
            fc = CT(0.5) + CT(0.5) * sn;
            fcd = CT(0.5) * cs * (CT(kPi) * CT(finv));
        }
    }
}

// Bucket key of cluster c, or -1 when its tuple has no coefficients.
template <int NB>
__device__ __forceinline__ int bucket_key(const BatchView& B, const int* clusters, long long c) {
    int id[NB], s, u;
    const DevParamSet* P;
    const TupleRec* R = cluster_tuple<NB>(B, clusters, c, id, s, P, u);
    if (!R->valid || (NB == 3 ? P->R3 : P->R4) <= 0) return -1;
    if (B.bucket_cut) {   // compute_3B/4B would return at once: leave the cluster out
        const double* h = B.sys[s].h;
        for (int p = 0; p < Topo<NB>::NP; p++) {
            const int a = id[Topo<NB>::a(p)], b = id[Topo<NB>::b(p)];
            if (B.pos_f) {   // decided by the FP32 distance unless within the margin
                const float* xa = B.pos_f + 3 * (long long)a;
                const float* xb = B.pos_f + 3 * (long long)b;
                const float ex = xb[0] - xa[0], ey = xb[1] - xa[1], ez = xb[2] - xa[2];
                const float df = sqrtf(ex * ex + ey * ey + ez * ez);
                const float m = B.float_eps + 1e-6f * R->rout_f[p];
                if (df < R->rout_f[p] - m) continue;
                if (df >= R->rout_f[p] + m) return -1;
            }
            double dr[3], r;
            pair_geom(B, h, a, b, dr, r);
            if (r >= R->rout[p]) return -1;
        }
    }
    return (NB == 3 ? P->bk3 : P->bk4) + u;
}

template <int NB>
__global__ void __launch_bounds__(256) k_bucket_count(BatchView B, const int* clusters, const long long* n_ptr,
                                                      long long cap) {
    const long long n = min(*n_ptr, cap);
    int* count = B.bk_count + (NB == 3 ? 0 : B.nbk3);
    int* keys = NB == 3 ? B.bk_key3 : B.bk_key4;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    // base is uniform over the block, so whole warps take part in the match
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long c = base + threadIdx.x;
        const int key = c < n ? bucket_key<NB>(B, clusters, c) : -1;
        if (keys && c < n) keys[c] = key;
        const unsigned peers = __match_any_sync(kFull, key);
        if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&count[key], __popc(peers));
    }
}

// Exclusive scan of the bucket sizes rounded up to 32 (3-body: bk_pad3); the total goes to
// start[nbk] and the padding slots of every bucket are set to -1.  One block.
__global__ void __launch_bounds__(1024) k_bucket_scan(BatchView B, int nb) {
    const int nbk = nb == 3 ? B.nbk3 : B.nbk4;
    const int* count = B.bk_count + (nb == 3 ? 0 : B.nbk3);
    long long* start = B.bk_start + (nb == 3 ? 0 : B.nbk3 + 1);
    int* perm = nb == 3 ? B.perm3 : B.perm4;
    const long long pcap = nb == 3 ? B.perm3_cap : B.perm4_cap;
    const int pad = nb == 3 && B.bk_pad3 > 0 ? B.bk_pad3 : 32;   // a power of two
    __shared__ long long wsum[32];
    __shared__ long long carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nbk; base += blockDim.x) {
        const int k = base + threadIdx.x;
        const long long v = k < nbk ? (long long)((count[k] + pad - 1) & ~(pad - 1)) : 0;
        long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long w = lane < nwarps ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(kFull, w, o);
                if (lane >= o) w += y;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const long long incl = x + (warp > 0 ? wsum[warp - 1] : 0);
        if (k < nbk) start[k] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[nwarps - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) start[nbk] = carry;
    __syncthreads();
    for (int k = threadIdx.x; k < nbk; k += blockDim.x) {
        const long long s1 = k + 1 < nbk ? start[k + 1] : carry;
        for (long long q = start[k] + count[k]; q < s1 && q < pcap; q++) perm[q] = -1;
    }
}

template <int NB>
__global__ void __launch_bounds__(256) k_bucket_scatter(BatchView B, const int* clusters, const long long* n_ptr,
                                                        long long cap) {
    const long long n = min(*n_ptr, cap);
    int* fill = B.bk_fill + (NB == 3 ? 0 : B.nbk3);
    const long long* start = B.bk_start + (NB == 3 ? 0 : B.nbk3 + 1);
    int* perm = NB == 3 ? B.perm3 : B.perm4;
    const long long pcap = NB == 3 ? B.perm3_cap : B.perm4_cap;
    const int* keys = NB == 3 ? B.bk_key3 : B.bk_key4;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long c = base + threadIdx.x;
        const int key = c < n ? (keys ? keys[c] : bucket_key<NB>(B, clusters, c)) : -1;
        const unsigned peers = __match_any_sync(kFull, key);
        const int leader = __ffs(peers) - 1;
        int b = 0;
        if (key >= 0 && lane == leader) b = atomicAdd(&fill[key], __popc(peers));
        b = __shfl_sync(kFull, b, leader);
        if (key >= 0) {
            const long long slot = start[key] + b + __popc(peers & ((1u << lane) - 1u));
            if (slot < pcap) perm[slot] = (int)c;
        }
    }
}

// Pair-table cache: for every list entry (i, j) closer than the body order's
// largest outer cutoff, the pair's geometry (dr, r), cutoff (fc, fc') and
// Chebyshev tables T, dT/dr with the pair type's constants -- the same values
// the cluster kernel would compute for a cluster pair ij, ik (or il), once per
// entry instead of once per cluster.  pcd[e][8] = dr0 dr1 dr2 r fc fc' oor -;
// pct[e][2*rs] = T[0..R), then dT/dr at offset rs.
template <int NB, typename CT>
__global__ void __launch_bounds__(256) k_pair_tables(BatchView B, const int* l2_owner, int rs) {
    const long long n2 = min(B.l2_off[B.n_atoms_total], B.n2_cap);
    double* pcd = NB == 3 ? B.pcd3 : B.pcd4;
    CT* pct = reinterpret_cast<CT*>(NB == 3 ? B.pct3 : B.pct4);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n2; e += stride) {
        const int r = l2_owner[e];
        const SysDesc& d = B.sys[B.atom_sys[r]];
        if (!(NB == 3 ? d.has3 : d.has4) || B.l2_dist[e] >= (NB == 3 ? d.c3 : d.c4)) continue;
        const DevParamSet& P = B.psets[d.pset];
        const int gi = B.atom_self[r], gj = B.l2_ghost[e];
        double dr[3], rr;
        pair_geom(B, d.h, gi, gj, dr, rr);
        const int pt = P.pair_map[B.atom_type[r] * P.ntypes + B.atom_type[B.ghost_parent[gj]]];
        const PairTab& Q = (NB == 3 ? P.pt3 : P.pt4)[pt];
        CT fc, fcd;
        CT* T = pct + (size_t)e * 2 * rs;
        pair_setup<CT>(P, Q, rr, T, T + rs, 1, NB == 3 ? P.R3 : P.R4, fc, fcd, nullptr);
        double* g = pcd + 8 * e;
        g[0] = dr[0]; g[1] = dr[1]; g[2] = dr[2]; g[3] = rr;
        g[4] = double(fc); g[5] = double(fcd); g[6] = rr < Q.rin ? 1.0 : 0.0; g[7] = 0.0;
    }
}

// Shared-memory layout of one warp (one block), G = 32/TPC clusters,
// interleaved [entry][cluster]:
//   double geo[NP*4][G] (dr, r), fc[NP][G], fcd[NP][G]
//   CT     T[NP*rs][G], D[NP*rs][G], Y[ys][G], X[xs][G]
// NOY (3-body only): no Y table in shared memory; the row sums multiply the
// two column pairs' Chebyshev values per entry instead (one more multiply per
// coefficient, half the shared memory, so twice the resident warps).
template <int NB, typename CT, int TPC, bool NOY = false>
__global__ void __launch_bounds__(32) k_forcef(BatchView B, const int* clusters, const int* perm,
                                               const long long* perm_n, long long perm_cap, int rs, int ys,
                                               int xs) {
    constexpr int NP = Topo<NB>::NP;
    constexpr int K = Split<NB>::K;
    constexpr int G = 32 / TPC;
    const long long n = min(*perm_n, perm_cap);
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int grp = lane / TPC, gl = lane % TPC;
    double* geo = reinterpret_cast<double*>(smem);
    double* fcs = geo + NP * 4 * G;
    double* fcds = fcs + NP * G;
    CT* Tt = reinterpret_cast<CT*>(fcds + NP * G);
    CT* Dt = Tt + NP * rs * G;
    CT* Y = Dt + NP * rs * G;
    CT* X = Y + ys * G;
    CT* const Xv = K > 1 ? X : Tt;   // the row-side products (3-body: pair 0's T itself)

    const long long steps = n / G;
    unsigned long long* head = &B.queue[NB - 3];
    EVAcc acc;

    for (;;) {
        long long step = 0;
        if (lane == 0) step = (long long)atomicAdd(head, 1ull);
        step = __shfl_sync(kFull, step, 0);
        if (step >= steps) break;
        const long long base = step * G;
        const int c0 = perm[base];
        if (c0 < 0) continue;   // uniform: a chunk never starts in a bucket's padding
        // the warp's tuple (shared by all its clusters)
        int id0[NB], s0, u0;
        const DevParamSet* P;
        const TupleRec* R = cluster_tuple<NB>(B, clusters, c0, id0, s0, P, u0);
        const int Rp = NB == 3 ? P->R3 : P->R4;
        const int c = perm[base + grp];
        bool active = c >= 0;
        int id[NB];
        int s = 0;
        // pairs 0 .. KC-1 (ij, ik[, il]) are list entries of the first atom:
        // with the pair-table cache their geometry and tables are loaded
        constexpr int KC = NB - 1;
        const bool use_pc = NB == 3 ? B.use_pc3 : B.use_pc4;
        const int* ce = NB == 3 ? B.c3e : B.c4e;
        const double* pcd = NB == 3 ? B.pcd3 : B.pcd4;
        const CT* pct = reinterpret_cast<const CT*>(NB == 3 ? B.pct3 : B.pct4);
        if (active) {
            for (int k = 0; k < NB; k++) id[k] = clusters[(long long)NB * c + k];
            s = B.atom_sys[B.ghost_parent[id[0]]];
            const double* h = B.sys[s].h;
            for (int sl = gl; sl < NP; sl += TPC) {
                // with the cache the evaluated pairs come first, spread over the lanes
                const int p = use_pc ? (sl < NP - KC ? KC + sl : sl - (NP - KC)) : sl;
                double dr[3], r;
                if (use_pc && p < KC) {
                    const double* g = pcd + 8 * (long long)ce[(long long)KC * c + p];
                    dr[0] = g[0]; dr[1] = g[1]; dr[2] = g[2]; r = g[3];
                } else {
                    pair_geom(B, h, id[Topo<NB>::a(p)], id[Topo<NB>::b(p)], dr, r);
                }
                geo[(4 * p + 0) * G + grp] = dr[0];
                geo[(4 * p + 1) * G + grp] = dr[1];
                geo[(4 * p + 2) * G + grp] = dr[2];
                geo[(4 * p + 3) * G + grp] = r;
            }
        }
        __syncwarp();
        if (active)   // compute_3B/4B early-outs on the per-pair outer cutoffs
            for (int p = 0; p < NP; p++)
                if (geo[(4 * p + 3) * G + grp] >= R->rout[p]) active = false;
        if (active)
            for (int sl = gl; sl < NP; sl += TPC) {
                const int p = use_pc ? (sl < NP - KC ? KC + sl : sl - (NP - KC)) : sl;
                if (use_pc && p < KC) {
                    const long long ent = ce[(long long)KC * c + p];
                    const double* g = pcd + 8 * ent;
                    const CT* tab = pct + ent * 2 * rs;
                    for (int n = 0; n < Rp; n++) {
                        Tt[(p * rs + n) * G + grp] = tab[n];
                        Dt[(p * rs + n) * G + grp] = tab[rs + n];
                    }
                    fcs[p * G + grp] = g[4];
                    fcds[p * G + grp] = g[5];
                    if (g[6] != 0.0) atomicAdd(&B.flags[4], 1);
                } else {
                    CT fc, fcd;
                    pair_setup<CT>(*P, tuple_pair(*R, p), geo[(4 * p + 3) * G + grp], Tt + p * rs * G + grp,
                                   Dt + p * rs * G + grp, G, Rp, fc, fcd, B.flags);
                    fcs[p * G + grp] = double(fc);
                    fcds[p * G + grp] = double(fcd);
                }
            }
        __syncwarp();
        // column-side products Y_J (and row-side X_I for 4-body); the mixed-radix
        // digits of the running index advance by TPC with carries (no division)
        {
            constexpr int C = NP - K;
            int ny = 1;
            for (int p = K; p < NP; p++) ny *= Rp;
            if (NOY) ny = 0;   // the row sums form the products themselves
            int q[C];
#pragma unroll
            for (int p = 0; p < C; p++) q[p] = 0;
            q[C - 1] = gl;
            for (int j = gl; j < ny; j += TPC) {
#pragma unroll
                for (int p = C - 1; p > 0; p--)
                    while (q[p] >= Rp) { q[p] -= Rp; q[p - 1]++; }
                CT y = CT(1);
#pragma unroll
                for (int p = 0; p < C; p++) y *= Tt[((K + p) * rs + q[p]) * G + grp];
                Y[j * G + grp] = y;
                q[C - 1] += TPC;
            }
            if constexpr (K > 1) {
                int nx = 1;
                for (int p = 0; p < K; p++) nx *= Rp;
                int v[K];
#pragma unroll
                for (int p = 0; p < K; p++) v[p] = 0;
                v[K - 1] = gl;
                for (int i = gl; i < nx; i += TPC) {
#pragma unroll
                    for (int p = K - 1; p > 0; p--)
                        while (v[p] >= Rp) { v[p] -= Rp; v[p - 1]++; }
                    CT x = CT(1);
#pragma unroll
                    for (int p = 0; p < K; p++) x *= Tt[(p * rs + v[p]) * G + grp];
                    X[i * G + grp] = x;
                    v[K - 1] += TPC;
                }
            }
        }
        __syncwarp();

        const auto* ent = fact_ent<CT, NB>(*P);
        const FactRow* rows = (NB == 3 ? P->fr3 : P->fr4) + R->f_row;
        int nrow = R->f_nrow, ncol = R->f_ncol;
        if (!ck_bound(B, R->f_ent >= 0 && R->f_ent + 2LL * R->ncoef <= (NB == 3 ? P->n_fe3 : P->n_fe4)))
            nrow = ncol = 0;
        CT S = CT(0), Gp[NP];
#pragma unroll
        for (int p = 0; p < NP; p++) Gp[p] = CT(0);
        // A record's entries start where the previous record's end; its last
        // entry carries the record-end bit.  Records are sorted by their powers
        // (first pair most significant), so the products of a record's pairs
        // are factored out level by level: the flushes sum over the last pair's
        // power within a run of equal leading powers and multiply by the
        // leading pairs' values once per run (nested sums instead of full
        // products per record); the saving is largest with one lane per
        // cluster, where runs stay whole.
        const int e_col0 = R->f_ent + R->ncoef;
        // Row records: z_I = sum_J a Y_J; S += X_I z_I, G_p += dX_I/dr_p z_I (p < K).
        // With K = 3, I = (q0, q1, q2): inner sums over q2, then q1, then q0.
        int rc0 = -1, rc1 = -1;
        CT ra = CT(0), rb = CT(0), rP = CT(0), rQ = CT(0), rR = CT(0);
        auto row_flush = [&](int pows, CT z) {
            if constexpr (K == 1) {
                const int q = pows & 31;
                S += Tt[q * G + grp] * z;
                Gp[0] += Dt[q * G + grp] * z;
            } else {
                const int q0 = pows & 31, q1 = (pows >> kPowBits) & 31, q2 = (pows >> (2 * kPowBits)) & 31;
                if (q0 != rc0 || q1 != rc1) {
                    if (rc1 >= 0) {
                        const CT t1 = Tt[(1 * rs + rc1) * G + grp];
                        rP += t1 * ra;
                        rQ += Dt[(1 * rs + rc1) * G + grp] * ra;
                        rR += t1 * rb;
                    }
                    ra = CT(0);
                    rb = CT(0);
                    if (q0 != rc0) {
                        if (rc0 >= 0) {
                            const CT t0 = Tt[rc0 * G + grp];
                            S += t0 * rP;
                            Gp[0] += Dt[rc0 * G + grp] * rP;
                            Gp[1] += t0 * rQ;
                            Gp[2] += t0 * rR;
                        }
                        rP = CT(0);
                        rQ = CT(0);
                        rR = CT(0);
                        rc0 = q0;
                    }
                    rc1 = q1;
                }
                ra += Tt[(2 * rs + q2) * G + grp] * z;
                rb += Dt[(2 * rs + q2) * G + grp] * z;
            }
        };
        auto row_end = [&]() {
            if constexpr (K == 3) {
                if (rc1 >= 0) {
                    const CT t1 = Tt[(1 * rs + rc1) * G + grp];
                    rP += t1 * ra;
                    rQ += Dt[(1 * rs + rc1) * G + grp] * ra;
                    rR += t1 * rb;
                    const CT t0 = Tt[rc0 * G + grp];
                    S += t0 * rP;
                    Gp[0] += Dt[rc0 * G + grp] * rP;
                    Gp[1] += t0 * rQ;
                    Gp[2] += t0 * rR;
                }
            }
        };
        // Column records: w_J = sum_I a X_I; G_p += dY_J/dr_p w_J (p >= K), summed
        // over the last column pair within runs of equal leading powers.
        constexpr int C = NP - K;
        int cc0 = -1, cc1 = -1;
        CT ca = CT(0), cb = CT(0), cP = CT(0), cQ = CT(0), cR = CT(0);
        auto col_flush = [&](int pows, CT w) {
            const int q0 = pows & 31, q1 = (pows >> kPowBits) & 31;
            if constexpr (C == 2) {
                // J = (q0, q1) of pairs K, K+1: sums over q1 within a run of q0
                if (q0 != cc0) {
                    if (cc0 >= 0) {
                        Gp[K] += Dt[(K * rs + cc0) * G + grp] * ca;
                        Gp[K + 1] += Tt[(K * rs + cc0) * G + grp] * cb;
                    }
                    ca = CT(0);
                    cb = CT(0);
                    cc0 = q0;
                }
                ca += Tt[((K + 1) * rs + q1) * G + grp] * w;
                cb += Dt[((K + 1) * rs + q1) * G + grp] * w;
            } else {
                // J = (q0, q1, q2) of pairs K .. K+2
                const int q2 = (pows >> (2 * kPowBits)) & 31;
                if (q0 != cc0 || q1 != cc1) {
                    if (cc1 >= 0) {
                        const CT t1 = Tt[((K + 1) * rs + cc1) * G + grp];
                        cP += t1 * ca;
                        cQ += Dt[((K + 1) * rs + cc1) * G + grp] * ca;
                        cR += t1 * cb;
                    }
                    ca = CT(0);
                    cb = CT(0);
                    if (q0 != cc0) {
                        if (cc0 >= 0) {
                            const CT t0 = Tt[(K * rs + cc0) * G + grp];
                            Gp[K] += Dt[(K * rs + cc0) * G + grp] * cP;
                            Gp[K + 1] += t0 * cQ;
                            Gp[K + 2] += t0 * cR;
                        }
                        cP = CT(0);
                        cQ = CT(0);
                        cR = CT(0);
                        cc0 = q0;
                    }
                    cc1 = q1;
                }
                ca += Tt[((K + 2) * rs + q2) * G + grp] * w;
                cb += Dt[((K + 2) * rs + q2) * G + grp] * w;
            }
        };
        auto col_end = [&]() {
            if constexpr (C == 2) {
                if (cc0 >= 0) {
                    Gp[K] += Dt[(K * rs + cc0) * G + grp] * ca;
                    Gp[K + 1] += Tt[(K * rs + cc0) * G + grp] * cb;
                }
            } else {
                if (cc1 >= 0) {
                    const CT t1 = Tt[((K + 1) * rs + cc1) * G + grp];
                    cP += t1 * ca;
                    cQ += Dt[((K + 1) * rs + cc1) * G + grp] * ca;
                    cR += t1 * cb;
                    const CT t0 = Tt[(K * rs + cc0) * G + grp];
                    Gp[K] += Dt[(K * rs + cc0) * G + grp] * cP;
                    Gp[K + 1] += t0 * cQ;
                    Gp[K + 2] += t0 * cR;
                }
            }
        };
        // (in FP32 the NOY form keeps its per-record loop: the one-stream form's
        // registers cost it more resident warps than the batched loads save)
        if constexpr (TPC == 1 && !(NOY && sizeof(CT) == 4)) {
            // one lane per cluster: each pass is one stream of entries across
            // its records (loads batched across record ends)
            if constexpr (NOY && NB == 3)
                flat_pass<CT, G, true>(ent, R->f_ent, e_col0, rows, nrow, Tt + 1 * rs * G, Tt + 2 * rs * G, grp,
                                       row_flush);
            else
                flat_pass<CT, G>(ent, R->f_ent, e_col0, rows, nrow, Y, nullptr, grp, row_flush);
            flat_pass<CT, G>(ent, e_col0, e_col0 + R->ncoef, rows + nrow, ncol, Xv, nullptr, grp, col_flush);
        } else if constexpr (TPC == 2 && !NOY && sizeof(CT) == 8) {
            // two lanes per cluster (FP64): lane 0 streams the row entries, lane
            // 1 the column entries (as many), each flushing its own records
            // (4096-configuration batch, 4-body: 34.0 -> 31.7 ms; in FP32 the
            // extra registers cost more than the whole runs save)
            const bool colp = gl == 1;
            flat_pass<CT, G>(ent, colp ? e_col0 : R->f_ent, colp ? e_col0 + R->ncoef : e_col0, colp ? rows + nrow : rows,
                             colp ? ncol : nrow, colp ? Xv : Y, nullptr, grp, [&](int pw, CT z) {
                                 if (colp) col_flush(pw, z);
                                 else row_flush(pw, z);
                             });
        } else {
            // The TPC lanes of a cluster take whole records round robin
            // (adjacent records, adjacent loads), each flushing its own.  A
            // lane's share is a sorted subsequence, so the nested sums apply.
            for (int r0 = 0; r0 < nrow; r0 += TPC) {
                const int r = r0 + gl;
                if (r < nrow) {
                    const FactRow rw = rows[r];
                    const int e0 = r == 0 ? R->f_ent : rows[r - 1].end;
                    CT z;
                    if constexpr (NOY && NB == 3)
                        z = entry_sum_noy<CT, G>(ent, e0, rw.end, Tt + 1 * rs * G, Tt + 2 * rs * G, grp);
                    else
                        z = entry_sum<CT, 1, G>(ent, e0, rw.end, 0, Y, grp);
                    row_flush(rw.pows, z);
                }
            }
            for (int cb0 = 0; cb0 < ncol; cb0 += TPC) {
                const int cc = cb0 + gl;
                if (cc < ncol) {
                    const FactRow cl = rows[nrow + cc];
                    const int e0 = cc == 0 ? e_col0 : rows[nrow + cc - 1].end;
                    col_flush(cl.pows, entry_sum<CT, 1, G>(ent, e0, cl.end, 0, Xv, grp));
                }
            }
        }
        row_end();
        col_end();
        // combine the TPC partial sums of each cluster
#pragma unroll
        for (int off = TPC / 2; off > 0; off >>= 1) {
            S += __shfl_xor_sync(kFull, S, off);
#pragma unroll
            for (int p = 0; p < NP; p++) Gp[p] += __shfl_xor_sync(kFull, Gp[p], off);
        }
        if (sizeof(CT) == 4 && active && gl == 0) {   // mixed form: the epilogue in FP32
            float drf[NP][3], rinv[NP], fcf[NP], fcdf[NP], Gf[NP];
            for (int p = 0; p < NP; p++) {
                for (int k = 0; k < 3; k++) drf[p][k] = float(geo[(4 * p + k) * G + grp]);
                rinv[p] = 1.0f / float(geo[(4 * p + 3) * G + grp]);
                fcf[p] = float(fcs[p * G + grp]);
                fcdf[p] = float(fcds[p * G + grp]);
                Gf[p] = float(Gp[p]);
            }
            double e_c, vir_c[6];
            cluster_epilogue_f32<NB>(B, id, drf, rinv, fcf, fcdf, float(S), Gf, e_c, vir_c);
            acc.add(B, s, e_c, vir_c);
        } else if (active && gl == 0) {
            double dr[NP][4], fc[NP], fcd[NP], Gd[NP];
            for (int p = 0; p < NP; p++) {
                for (int k = 0; k < 4; k++) dr[p][k] = geo[(4 * p + k) * G + grp];
                fc[p] = fcs[p * G + grp];
                fcd[p] = fcds[p * G + grp];
                Gd[p] = double(Gp[p]);
            }
            cluster_epilogue<NB>(B, id, s, dr, fc, fcd, double(S), Gd, acc);
        }
        __syncwarp();
    }
    acc.flush_warp(B);
}

template <int NB, typename CT>
size_t smem_bytes(int tpc, int rs, bool noy = false) {
    constexpr int NP = Topo<NB>::NP;
    constexpr int K = Split<NB>::K;
    const int G = 32 / tpc;
    long long ys = 1, xs = 1;
    for (int p = K; p < NP; p++) ys *= rs;
    for (int p = 0; p < K; p++) xs *= rs;
    if (K == 1) xs = 0;
    if (noy) ys = 0;
    return sizeof(double) * (size_t)NP * 6 * G + sizeof(CT) * (size_t)(2 * NP * rs + ys + xs) * G;
}

template <int NB, typename CT>
void launch_f(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    constexpr int NP = Topo<NB>::NP;
    constexpr int K = Split<NB>::K;
    const int tpc = NB == 3 ? L.ftpc3 : L.ftpc4;
    const int rs = NB == 3 ? L.rf3 : L.rf4;
    const long long pcap = NB == 3 ? B.perm3_cap : B.perm4_cap;
    const int nbk = NB == 3 ? B.nbk3 : B.nbk4;
    if (pcap <= 0 || nbk <= 0 || rs <= 0) return;
    const bool noy = NB == 3 && L.noy3;
    int ys = 1, xs = 1;
    for (int p = K; p < NP; p++) ys *= rs;
    for (int p = 0; p < K; p++) xs *= rs;
    if (K == 1) xs = 0;
    if (noy) ys = 0;
    const size_t smem = smem_bytes<NB, CT>(tpc, rs, noy);
    const long long* pn = B.bk_start + (NB == 3 ? 0 : B.nbk3 + 1) + nbk;
    const int* clusters = NB == 3 ? B.c3 : B.c4;
    const int* perm = NB == 3 ? B.perm3 : B.perm4;
    const int want_bps = NB == 3 ? L.fbps3 : L.fbps4;
#define CK_LAUNCH_F(T_, NOY_)                                                                            \
    do {                                                                                                 \
        auto kern = k_forcef<NB, CT, T_, NOY_>;                                                          \
        allow_max_smem((const void*)kern);                                                              \
        int occ = 0;                                                                                     \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32, smem);                             \
        if (occ < 1) occ = 1;                                                                            \
        const long long steps = (pcap + (32 / T_) - 1) / (32 / T_);                                      \
        long long want = (long long)sm_count() * (want_bps < occ ? want_bps : occ);                       \
        const unsigned grid = (unsigned)(want < steps ? want : steps);                                   \
        count_launch(), kern<<<grid, 32, smem, st>>>(B, clusters, perm, pn, pcap, rs, ys, xs);            \
    } while (0)
    if (noy) {
        switch (tpc) {
            case 1: CK_LAUNCH_F(1, NB == 3); break;
            case 2: CK_LAUNCH_F(2, NB == 3); break;
            default: CK_LAUNCH_F(4, NB == 3); break;
        }
    } else {
        switch (tpc) {
            case 1: CK_LAUNCH_F(1, false); break;
            case 2: CK_LAUNCH_F(2, false); break;
            default: CK_LAUNCH_F(4, false); break;
        }
    }
#undef CK_LAUNCH_F
}

template <int NB>
void launch_bucket_n(const BatchView& B, cudaStream_t st) {
    const int nbk = NB == 3 ? B.nbk3 : B.nbk4;
    const long long cap = NB == 3 ? B.n3_cap : B.n4_cap;
    if (nbk <= 0 || cap <= 0) return;
    const long long* n_ptr = (NB == 3 ? B.e_off3 : B.e_off4) + B.n2_cap;
    const int* clusters = NB == 3 ? B.c3 : B.c4;
    long long want = (long long)sm_count() * 8;
    long long need = (cap + 255) / 256;
    const unsigned grid = (unsigned)(want < need ? want : need);
    count_launch(), k_bucket_count<NB><<<grid, 256, 0, st>>>(B, clusters, n_ptr, cap);
    count_launch(), k_bucket_scan<<<1, 1024, 0, st>>>(B, NB);
    count_launch(), k_bucket_scatter<NB><<<grid, 256, 0, st>>>(B, clusters, n_ptr, cap);
}

}  // namespace

size_t factored_smem_bytes(int nbody, int precision, int tpc, int rs) {
    if (nbody == 3)
        return precision == kMixed ? smem_bytes<3, float>(tpc, rs) : smem_bytes<3, double>(tpc, rs);
    return precision == kMixed ? smem_bytes<4, float>(tpc, rs) : smem_bytes<4, double>(tpc, rs);
}

void launch_bucket(const BatchView& B, int nbody, cudaStream_t st) {
    if (nbody == 3) launch_bucket_n<3>(B, st);
    else launch_bucket_n<4>(B, st);
}

void launch_pair_tables(const BatchView& B, const int* l2_owner, int nbody, const ForceLaunch& L, cudaStream_t st) {
    if (!(nbody == 3 ? B.use_pc3 : B.use_pc4) || B.n2_cap <= 0) return;
    const int rs = nbody == 3 ? L.rf3 : L.rf4;
    long long want = (long long)sm_count() * 8;
    long long need = (B.n2_cap + 255) / 256;
    const unsigned grid = (unsigned)(want < need ? want : need);
    if (nbody == 3) {
        if (L.precision == kMixed) count_launch(), k_pair_tables<3, float><<<grid, 256, 0, st>>>(B, l2_owner, rs);
        else count_launch(), k_pair_tables<3, double><<<grid, 256, 0, st>>>(B, l2_owner, rs);
    } else {
        if (L.precision == kMixed) count_launch(), k_pair_tables<4, float><<<grid, 256, 0, st>>>(B, l2_owner, rs);
        else count_launch(), k_pair_tables<4, double><<<grid, 256, 0, st>>>(B, l2_owner, rs);
    }
}

void launch_force3f(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    if (L.precision == kMixed) launch_f<3, float>(B, L, st);
    else launch_f<3, double>(B, L, st);
}

void launch_force4f(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    if (L.precision == kMixed) launch_f<4, float>(B, L, st);
    else launch_f<4, double>(B, L, st);
}

}  // namespace ck
