// Cluster fingerprints: the FINGERPRINT build of the reference (records of
// the clusters its LAMMPS pair style evaluates, etc/lmp/src/pair_chimes.cpp:
// 525-536, 620-662, 700-741, 775-810, chimesFF.cpp:1694-1702, 2013-2021,
// 2603-2612) and its cluster-distance histograms
// (chimesFF/src/FP/multi_calc_histogram.cpp).
//
// Records: after a pair-style evaluation, the clusters of one body order that
// pass compute_nB's type and cutoff checks and the recording order rule
// (2-body: i < j, 3-/4-body: strictly increasing tags), as distances and type
// indices, compacted in the pair style's loop order (flag, scan, fill).
//
// Histogram: each record's distances go through the Morse map of its own
// cutoffs (read_flat_clusters) and are sorted; every pair of records (i from
// set 1, j from set 2; j > i when both are the same set) contributes its
// Euclidean distance to a histogram of nbin bins over [0, maxd).  The pair
// loop is O(n1*n2) and runs here as tiles of 256 x 256 records: set-2 tiles
// staged in shared memory (broadcast reads), each thread owning two set-1
// records and a private histogram column in shared memory (bin-major, so a
// warp's 32 columns sit on 32 different banks and increments never collide).
// Distances are computed in FP32 with a rigorous bound on the error of the
// squared distance; a pair whose bin the bound certifies is counted directly,
// the rest (those within ~1e-6 of a bin edge) are recomputed in FP64 with the
// reference's operations, so the counts equal the FP64 histogram's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ck_common.h"
#include "ck_engine.h"
#include "ck_force_common.cuh"
#include "ck_fingerprint.h"
#include "ck_kernels.h"

namespace ck {

namespace {

constexpr int kFpTileJ = 256;   // set-2 records per shared-memory tile
constexpr int kFpRows = 2;      // set-1 records per thread

template <int P>
struct __align__(P == 1 ? 8 : 16) FpRec {   // one staged set-2 record: edges and squared norm
    float e[P];
    float q;
};

__device__ __forceinline__ float fp_sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Exact FP64 bin of one pair, with the tool's operations (dist_struct +=
// pow(a - b, 2) in order, sqrt, floor(dist / binw), the dist == maxd rule);
// -1 when the distance falls past the last bin.
template <int P>
__device__ __forceinline__ int fp_exact_bin(const double* a, const double* b, double binw, double maxd, int nbin,
                                            int cand) {
    double ds = 0.0;
    for (int p = 0; p < P; p++) {
        const double d = __dsub_rn(a[p], b[p]);
        ds = __dadd_rn(ds, __dmul_rn(d, d));
    }
    // the FP32 candidate bin, confirmed in FP64 when ds lies inside its
    // squared edges by far more than the roundings of sqrt and the division
    if (cand >= 0 && cand < nbin) {
        const double lo = cand * binw, hi = lo + binw;
        if (ds >= lo * lo * (1.0 + 1e-12) && ds <= hi * hi * (1.0 - 1e-12)) return cand;
    }
    const double dist = __dadd_rn(__dsqrt_rn(ds), 0.0);
    int bin = (int)floor(__ddiv_rn(dist, binw));
    if (dist == maxd) bin = bin - 1;
    return (bin < 0 || bin >= nbin) ? -1 : bin;
}

// One thread owns kFpRows set-1 records (i0 + tid + r*T) and loops over the
// staged set-2 tile.  Per pair: the FP32 squared distance s, its error bound
// eps, a candidate bin k from an approximate square root (floor by a
// round-down add at 1.5*2^23: no conversion instructions), and the test
// (k w)^2 (1+d) <= s - eps, s + eps <= ((k+1) w)^2 (1-d) written as fused
// multiply-adds; a pair that fails it (near an edge, ~1e-4 of them) takes the
// exact FP64 path.
template <int P>
__global__ void __launch_bounds__(128) k_fp_hist(const float* __restrict__ e1, const float* __restrict__ q1,
                                                 const double* __restrict__ d1, long long n1,
                                                 const float* __restrict__ e2, const float* __restrict__ q2,
                                                 const double* __restrict__ d2, long long n2, int same, int nbin,
                                                 double binw, double maxd, long long n_itile, long long n_jtile,
                                                 unsigned long long* counts, int* flags) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int T = blockDim.x;
    const int tid = threadIdx.x;
    unsigned int* hist = reinterpret_cast<unsigned int*>(smem);                  // [nbin][T]
    FpRec<P>* tile = reinterpret_cast<FpRec<P>*>(smem + sizeof(unsigned int) * (size_t)nbin * T);
    for (int b = 0; b < nbin; b++) hist[b * T + tid] = 0u;
    // |s32 - s| <= (4 + P) u sum_k (|a_k| + |b_k|)^2 <= 2 (4 + P) u (qa + qb), u = 2^-24;
    // the staged norms carry kEps (a margin of 3x over that bound)
    const float kEps = 6.0f * (4 + P) * 5.9604645e-8f;
    const float inv_wf = (float)(1.0 / binw);
    const float wlo = (float)(binw * (1.0 + 1.0e-6)), whi = (float)(binw * (1.0 - 1.0e-6));
    const float kMagic = 12582912.0f;                // 1.5 * 2^23: adding it rounds to an integer
    const int kMagicBits = 0x4B400000;
    const int rows = T * kFpRows;
    const long long ntiles = n_itile * n_jtile;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long it = t / n_jtile, jt = t % n_jtile;
        const long long i0 = it * rows, j0 = jt * kFpTileJ;
        // a tile whose every j is <= every i holds no pair j > i
        if (same && j0 + kFpTileJ - 1 <= i0) continue;
        const int jn = (int)min((long long)kFpTileJ, n2 - j0);
        __syncthreads();
        for (int k = tid; k < jn; k += T) {
            FpRec<P> r;
            for (int p = 0; p < P; p++) r.e[p] = e2[(j0 + k) * P + p];
            r.q = kEps * q2[j0 + k];
            tile[k] = r;
        }
        __syncthreads();
        for (int rr = 0; rr < kFpRows; rr++) {
            const long long i = i0 + tid + (long long)rr * T;
            if (i >= n1) break;
            float a[P];
            for (int p = 0; p < P; p++) a[p] = e1[i * P + p];
            const float qa = kEps * q1[i];
            const int jstart = same ? (int)max(0LL, min((long long)jn, i + 1 - j0)) : 0;
#pragma unroll 2
            for (int k = jstart; k < jn; k++) {
                const FpRec<P> r = tile[k];
                float s = 0.0f;
#pragma unroll
                for (int p = 0; p < P; p++) {
                    const float d = a[p] - r.e[p];
                    s = fmaf(d, d, s);
                }
                const float eps = qa + r.q;
                // rounded down at magnitude 1.5*2^23 (unit spacing): kMagic + floor(sqrt(s) / w)
                const float mag = __fmaf_rd(fp_sqrt_approx(s), inv_wf, kMagic);
                const float kf = mag - kMagic;                 // candidate bin, an exact float integer
                const int bin = __float_as_int(mag) - kMagicBits;
                const float lo = kf * wlo, hi = fmaf(kf, whi, whi);
                const bool ok = bin < nbin && fmaf(lo, lo, eps - s) <= 0.0f && fmaf(-hi, hi, s + eps) <= 0.0f;
                int b = bin;
                if (!ok) {
                    const long long j = j0 + k;
                    b = fp_exact_bin<P>(d1 + i * P, d2 + j * P, binw, maxd, nbin, bin);
                    if (b < 0) {
                        atomicOr(&flags[0], 1);
                        continue;
                    }
                }
                hist[b * T + tid] += 1u;
            }
        }
    }
    __syncthreads();
    for (int b = tid; b < nbin; b += T) {
        unsigned long long sum = 0;
        for (int t2 = 0; t2 < T; t2++) sum += hist[b * T + t2];
        if (sum) atomicAdd(&counts[b], sum);
    }
}

// ---- fingerprint records of the pair-style path ---------------------------
__device__ __forceinline__ double fp_dist(const double* x, int i, int j) {
    const double d0 = __dsub_rn(x[3 * (long long)j + 0], x[3 * (long long)i + 0]);
    const double d1 = __dsub_rn(x[3 * (long long)j + 1], x[3 * (long long)i + 1]);
    const double d2 = __dsub_rn(x[3 * (long long)j + 2], x[3 * (long long)i + 2]);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
}

// 2-body: list entries (i, j) with tag[j] > tag[i] (the pair loop), i < j
// (valid_order) and r below the pair type's outer cutoff (compute_2B).
template <bool FILL>
__global__ void k_nl_fp2(BatchView B, NeighView N, int* flag, const long long* off, double* d, int* t) {
    const DevParamSet& P = B.psets[B.sys[0].pset];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < N.nent; e += stride) {
        const int i = N.ilist[N.owner[e]];
        const int j = N.neigh[e];
        bool ok = N.tag[j] > N.tag[i] && i < j;
        double r = 0.0;
        if (ok) {
            r = fp_dist(B.ghost_fs, i, j);
            ok = r < P.pairs[P.pair_map[B.atom_type[i] * P.ntypes + B.atom_type[j]]].rout;
        }
        if (!FILL) {
            flag[e] = ok ? 1 : 0;
        } else if (ok) {
            const long long o = off[e];
            d[o] = r;
            t[2 * o] = B.atom_type[i];
            t[2 * o + 1] = B.atom_type[j];
        }
    }
}

// 3-/4-body: listed clusters with strictly increasing tags (valid_order),
// a type that is not excluded and every pair below its outer cutoff.
template <int NB, bool FILL>
__global__ void k_nl_fpn(BatchView B, NeighView N, long long n, int* flag, const long long* off, double* d, int* t) {
    constexpr int NP = NB * (NB - 1) / 2;
    const DevParamSet& P = B.psets[B.sys[0].pset];
    const int* cl = NB == 3 ? B.c3 : B.c4;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        int id[NB];
        for (int k = 0; k < NB; k++) id[k] = cl[(long long)NB * q + k];
        bool ok = true;
        if (NB == 3) ok = N.tag[id[0]] < N.tag[id[1]] && N.tag[id[0]] < N.tag[id[2]] && N.tag[id[1]] < N.tag[id[2]];
        else ok = N.tag[id[0]] < N.tag[id[1]] && N.tag[id[1]] < N.tag[id[2]] && N.tag[id[2]] < N.tag[id[3]];
        double r[NP];
        int u = 0;
        for (int k = 0; k < NB; k++) u = u * P.ntypes + B.atom_type[id[k]];
        const TupleRec& R = (NB == 3 ? P.t3 : P.t4)[u];
        if (ok) ok = R.type_id >= 0;
        if (ok)
            for (int p = 0; p < NP; p++) {
                r[p] = fp_dist(B.ghost_fs, id[Topo<NB>::a(p)], id[Topo<NB>::b(p)]);
                if (r[p] >= R.rout[p]) ok = false;
            }
        if (!FILL) {
            flag[q] = ok ? 1 : 0;
        } else if (ok) {
            const long long o = off[q];
            for (int p = 0; p < NP; p++) d[o * NP + p] = r[p];
            for (int k = 0; k < NB; k++) t[o * NB + k] = B.atom_type[id[k]];
        }
    }
}

unsigned fp_grid(long long n) {
    long long g = (n + 255) / 256;
    if (g < 1) g = 1;
    const long long cap = (long long)sm_count() * 8;
    return (unsigned)(g < cap ? g : cap);
}

}  // namespace

void launch_nl_fp(const BatchView& B, const NeighView& N, int nbody, long long n, bool fill, int* flag,
                  const long long* off, double* d, int* t, cudaStream_t st) {
    if (n <= 0) return;
    const unsigned g = fp_grid(n);
    if (nbody == 2) {
        if (fill) count_launch(), k_nl_fp2<true><<<g, 256, 0, st>>>(B, N, flag, off, d, t);
        else count_launch(), k_nl_fp2<false><<<g, 256, 0, st>>>(B, N, flag, off, d, t);
    } else if (nbody == 3) {
        if (fill) count_launch(), k_nl_fpn<3, true><<<g, 256, 0, st>>>(B, N, n, flag, off, d, t);
        else count_launch(), k_nl_fpn<3, false><<<g, 256, 0, st>>>(B, N, n, flag, off, d, t);
    } else {
        if (fill) count_launch(), k_nl_fpn<4, true><<<g, 256, 0, st>>>(B, N, n, flag, off, d, t);
        else count_launch(), k_nl_fpn<4, false><<<g, 256, 0, st>>>(B, N, n, flag, off, d, t);
    }
}

// ---------------------------------------------------------------------------
// Histogram driver
// ---------------------------------------------------------------------------
namespace {

// transform of read_flat_clusters (multi_calc_histogram.cpp:112-123), host FP64
double fp_transform(double rcin, double rcout, double lambda, double rij) {
    double x_min = std::exp(-1 * rcin / lambda);
    double x_max = std::exp(-1 * rcout / lambda);
    double x_avg = 0.5 * (x_max + x_min);
    double x_diff = 0.5 * (x_max - x_min);
    x_diff *= -1.0;
    return (std::exp(-1 * rij / lambda) - x_avg) / x_diff;
}

// sorted transformed edges of n records (the cluster's own cutoffs, pair
// lambdas by the atoms' pair type), read_flat_clusters (:26-107)
Status fp_edges(const Engine& eng, int slot, int nbody, long long n, const double* d, const int* t,
                std::vector<double>& out, std::string& err) {
    const HostParams& P = eng.params(slot);
    const int nt = P.ntypes, np = nbody * (nbody - 1) / 2;
    out.assign((size_t)n * np, 0.0);
    for (long long c = 0; c < n; c++) {
        const int* ty = t + c * nbody;
        for (int k = 0; k < nbody; k++)
            if (ty[k] < 0 || ty[k] >= nt) {
                err = "fingerprint record " + std::to_string(c) + ": type index out of range";
                return kErrInput;
            }
        double* e = &out[(size_t)c * np];
        if (nbody == 2) {
            const int p = P.pair_map[ty[0] * nt + ty[1]];
            e[0] = fp_transform(P.rin[p], P.rout[p], P.lam[p], d[c]);
        } else {
            int u = 0;
            for (int k = 0; k < nbody; k++) u = u * nt + ty[k];
            const TupleRec& R = eng.tuples(slot, nbody)[u];
            if (R.type_id < 0) {
                err = "fingerprint record " + std::to_string(c) + ": excluded cluster type";
                return kErrInput;
            }
            for (int p = 0; p < np; p++) e[p] = fp_transform(R.rin[p], R.rout[p], R.lam[p], d[c * np + p]);
        }
        std::sort(e, e + np);
    }
    return kOk;
}

}  // namespace

Status fp_histogram(Engine& eng, int slot, int nbody, long long n1, const double* d1, const int* t1, long long n2,
                    const double* d2, const int* t2, bool same, int nbin, long long* counts, long long* nsamples,
                    std::string& err) {
    Status st = eng.init_device(err);
    if (st != kOk) return st;
    if (slot < 0 || slot >= eng.n_param_sets()) {
        err = "parameter set not loaded";
        return kErrState;
    }
    if (nbody < 2 || nbody > 4 || nbin < 1 || n1 < 0 || n2 < 0) {
        err = "fingerprint histogram: nbody 2..4, nbin >= 1, non-negative record counts";
        return kErrInput;
    }
    const HostParams& P = eng.params(slot);
    if ((nbody == 3 && P.o3 <= 0) || (nbody == 4 && P.o4 <= 0)) {
        err = "the parameter set has no " + std::to_string(nbody) + "-body terms";
        return kErrInput;
    }
    for (int b = 0; b < nbin; b++) counts[b] = 0;
    *nsamples = 0;
    const int np = nbody * (nbody - 1) / 2;
    std::vector<double> e1, e2;
    if ((st = fp_edges(eng, slot, nbody, n1, d1, t1, e1, err)) != kOk) return st;
    if (same) {
        n2 = n1;
    } else if ((st = fp_edges(eng, slot, nbody, n2, d2, t2, e2, err)) != kOk) {
        return st;
    }
    // one process of gen_flat_hists: nothing is counted unless the first set
    // has at least two records (its task range must have end > start)
    if (n1 <= 1 || n2 <= 0) return kOk;
    const double maxd = nbody == 2 ? 3.0 : (nbody == 3 ? std::sqrt(12.0) + 1.0 : std::sqrt(24.0) + 1.0);
    const double binw = maxd / nbin;
    int T = 128;
    while (T > 32 && (size_t)nbin * T * 4 > 160 * 1024) T /= 2;
    const size_t rec = nbody == 2 ? sizeof(FpRec<1>) : nbody == 3 ? sizeof(FpRec<3>) : sizeof(FpRec<6>);
    const size_t smem = (size_t)nbin * T * 4 + rec * kFpTileJ;
    if (smem > 200 * 1024) {
        err = "fingerprint histogram: nbin too large for the shared-memory histogram (at most 1280 bins)";
        return kErrInput;
    }
    auto pack = [&](const std::vector<double>& e, long long n, std::vector<float>& ef, std::vector<float>& q) {
        ef.resize((size_t)n * np);
        q.resize((size_t)n);
        for (long long c = 0; c < n; c++) {
            double s = 0.0;
            for (int p = 0; p < np; p++) {
                ef[(size_t)c * np + p] = (float)e[(size_t)c * np + p];
                s += e[(size_t)c * np + p] * e[(size_t)c * np + p];
            }
            q[(size_t)c] = (float)(s * (1.0 + 1e-6));   // rounded up: the bound stays a bound
        }
    };
    std::vector<float> f1, q1, f2, q2;
    pack(e1, n1, f1, q1);
    if (!same) pack(e2, n2, f2, q2);
    const cudaStream_t s = eng.stream();
    DevBuf<double> dd1, dd2;
    DevBuf<float> df1, dq1, df2, dq2;
    DevBuf<unsigned long long> dcounts;
    DevBuf<int> dflags;
#define FP_TRY(call)                                                                   \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call; \
            return kErrCuda;                                                           \
        }                                                                              \
    } while (0)
    FP_TRY(dd1.reserve(e1.size()));
    FP_TRY(df1.reserve(f1.size()));
    FP_TRY(dq1.reserve(q1.size()));
    FP_TRY(cudaMemcpyAsync(dd1.p, e1.data(), sizeof(double) * e1.size(), cudaMemcpyHostToDevice, s));
    FP_TRY(cudaMemcpyAsync(df1.p, f1.data(), sizeof(float) * f1.size(), cudaMemcpyHostToDevice, s));
    FP_TRY(cudaMemcpyAsync(dq1.p, q1.data(), sizeof(float) * q1.size(), cudaMemcpyHostToDevice, s));
    const double* pd2 = dd1.p;
    const float *pf2 = df1.p, *pq2 = dq1.p;
    if (!same) {
        FP_TRY(dd2.reserve(e2.size()));
        FP_TRY(df2.reserve(f2.size()));
        FP_TRY(dq2.reserve(q2.size()));
        FP_TRY(cudaMemcpyAsync(dd2.p, e2.data(), sizeof(double) * e2.size(), cudaMemcpyHostToDevice, s));
        FP_TRY(cudaMemcpyAsync(df2.p, f2.data(), sizeof(float) * f2.size(), cudaMemcpyHostToDevice, s));
        FP_TRY(cudaMemcpyAsync(dq2.p, q2.data(), sizeof(float) * q2.size(), cudaMemcpyHostToDevice, s));
        pd2 = dd2.p;
        pf2 = df2.p;
        pq2 = dq2.p;
    }
    FP_TRY(dcounts.reserve(nbin));
    FP_TRY(dflags.reserve(1));
    FP_TRY(cudaMemsetAsync(dcounts.p, 0, sizeof(unsigned long long) * nbin, s));
    FP_TRY(cudaMemsetAsync(dflags.p, 0, sizeof(int), s));
    const long long n_it = (n1 + (long long)T * kFpRows - 1) / ((long long)T * kFpRows),
                    n_jt = (n2 + kFpTileJ - 1) / kFpTileJ;
    const void* kern = nbody == 2 ? (const void*)k_fp_hist<1> : nbody == 3 ? (const void*)k_fp_hist<3>
                                                                           : (const void*)k_fp_hist<6>;
    if (smem > 48 * 1024) allow_max_smem(kern);
    int per_sm = 1;
    FP_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem));
    long long grid = (long long)sm_count() * std::max(1, per_sm);
    if (grid > n_it * n_jt) grid = n_it * n_jt;
    const int sm = same ? 1 : 0;
    if (nbody == 2)
        count_launch(), k_fp_hist<1><<<(unsigned)grid, T, smem, s>>>(df1.p, dq1.p, dd1.p, n1, pf2, pq2, pd2, n2, sm,
                                                                    nbin, binw, maxd, n_it, n_jt, dcounts.p, dflags.p);
    else if (nbody == 3)
        count_launch(), k_fp_hist<3><<<(unsigned)grid, T, smem, s>>>(df1.p, dq1.p, dd1.p, n1, pf2, pq2, pd2, n2, sm,
                                                                    nbin, binw, maxd, n_it, n_jt, dcounts.p, dflags.p);
    else
        count_launch(), k_fp_hist<6><<<(unsigned)grid, T, smem, s>>>(df1.p, dq1.p, dd1.p, n1, pf2, pq2, pd2, n2, sm,
                                                                    nbin, binw, maxd, n_it, n_jt, dcounts.p, dflags.p);
    FP_TRY(cudaGetLastError());
    std::vector<unsigned long long> hc(nbin);
    int hflag = 0;
    FP_TRY(cudaMemcpyAsync(hc.data(), dcounts.p, sizeof(unsigned long long) * nbin, cudaMemcpyDeviceToHost, s));
    FP_TRY(cudaMemcpyAsync(&hflag, dflags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FP_TRY(cudaStreamSynchronize(s));
#undef FP_TRY
    if (hflag) {
        err = "ERROR: computed bin larger than nbins (a cluster distance lies past the histogram range)";
        return kErrInput;
    }
    long long tot = 0;
    for (int b = 0; b < nbin; b++) {
        counts[b] = (long long)hc[b];
        tot += counts[b];
    }
    *nsamples = tot;
    return kOk;
}

}  // namespace ck
