// Cluster force kernels: Morse/Chebyshev stage, coefficient contraction and
// energy / force / virial reduction for 2-, 3- and 4-body clusters.
//
// Math (restated from chimesFF, chimesFF/src/chimesFF.cpp:1644-1775 (2B),
// 1931-2176 (3B), 2496-2872 (4B); set_cheby_polys chimesFF.h:542-628; get_fcut
// chimesFF.h:347-386; get_penalty chimesFF.h:388-419):
//   s = exp(-r/lambda), x = (s - xavg)/xdiff, dx/dr = -s/(lambda*xdiff)
//   T_0 = 1, T_1 = x, T_n = 2x T_{n-1} - T_{n-2};  dT_n/dr = n U_{n-1}(x) dx/dr
//   2B:  E += fc * sum_c a_c T_{p_c+1};   many-body: E += fc_all * S,
//        S   = sum_c a_c prod_q T_q[p_cq]
//        G_p = sum_c a_c dT_p[p_cp] prod_{q!=p} T_q[p_cq]
//   force scalar of pair p = (prod_{q!=p} fc_q / r_p) (fc_p G_p + fc'_p S),
//   which equals the reference's per-coefficient sum of force_scalar[p];
//   F_i += f_p dr_p, F_j -= f_p dr_p, virial -= f_p dr_p (x) dr_p.
// Only the summation order differs from the reference (sums are formed per
// cluster first), which moves results by rounding only.
//
// Work mapping: a warp takes 32/TPC clusters per step, TPC lanes per cluster.
// Lanes of a cluster compute its pair geometry (FP64) and Chebyshev tables
// (compute type CT) into shared memory, then split the coefficient list
// (lane l takes coefficients l, l+TPC, ...) and combine S and G_p by xor
// shuffles.  The group leader turns them into forces (FP64 atomics on the
// caller's atoms) and accumulates energy and virial per system in FP64.
// CT = double is the plain FP64 path; CT = float is the mixed path (FP32
// Chebyshev recursion, cutoff and contraction; FP64 geometry and accumulation).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <set>

#include "ck_common.h"
#include "ck_kernels.h"
#include "ck_force_common.cuh"
#include "ck_math.cuh"

namespace ck {

namespace {

// ---------------------------------------------------------------------------
// 1-body + 2-body: one thread per neighbour-list entry (and per atom for 1B).
// The 2B coefficients are summed along the recursion with the dense
// per-pair-type table a_n = sum of coefficients whose power+1 is n.
// ---------------------------------------------------------------------------
template <typename CT>
__global__ void __launch_bounds__(256) k_force2(BatchView B, const int* l2_owner) {
    const long long n2 = min(B.l2_off[B.n_atoms_total], B.n2_cap);
    EVAcc acc;
    const long long ntot = n2 > B.n_atoms_total ? n2 : B.n_atoms_total;
    // each block takes one contiguous range of entries (threads striding by
    // the block size, so loads stay coalesced): a thread's entries then belong
    // to the same atom and system for long runs, and its energy/virial
    // accumulator reaches the system's totals with few atomics even when a
    // batch holds many systems
    const long long per = ((ntot + gridDim.x - 1) / gridDim.x + blockDim.x - 1) / blockDim.x * blockDim.x;
    const long long e_end = min(ntot, per * (blockIdx.x + 1));
    for (long long e = per * blockIdx.x + threadIdx.x; e < e_end; e += blockDim.x) {
        double vir[6] = {0, 0, 0, 0, 0, 0};
        if (e < B.n_atoms_total) {   // compute_1B (chimesFF.cpp:1636-1641)
            const int s = B.atom_sys[e];
            const DevParamSet& P = B.psets[B.sys[s].pset];
            acc.add(B, s, P.eoff[B.atom_type[e]], vir);
        }
        if (e >= n2) continue;
        const int r = l2_owner[e];
        const int s = B.atom_sys[r];
        const SysDesc& d = B.sys[s];
        const DevParamSet& P = B.psets[d.pset];
        const int gi = B.atom_self[r];
        const int gj = B.l2_ghost[e];
        const int t0 = B.atom_type[r], t1 = B.atom_type[B.ghost_parent[gj]];
        int pidx = P.pair_map[t0 * P.ntypes + t1];
        if (!ck_bound(B, pidx >= 0 && pidx < P.npairs)) continue;
        const PairRec pr = P.pairs[pidx];
        double dr[3], dist;
        pair_geom(B, d.h, gi, gj, dr, dist);
        if (dist >= pr.rout) continue;
        double E, fs;
        pair_2b<CT>(P, pr, dist, B.flags, E, fs);
        add_force(B, gi, fs * dr[0], fs * dr[1], fs * dr[2]);
        add_force(B, gj, -fs * dr[0], -fs * dr[1], -fs * dr[2]);
        virial_add(vir, fs, dr);
        acc.add(B, s, E, vir);
    }
    acc.flush_warp(B);
}

// ---------------------------------------------------------------------------
// 3-body and 4-body clusters
// ---------------------------------------------------------------------------
// Shared memory of one cluster group: its T and dT/dr tables (CT), then the
// pair geometry and cutoff values (double).  Lanes of different groups read
// the same table offsets of their own clusters at once, so the group stride is
// padded (in 8-byte steps) to spread the groups' first banks as far apart as
// possible within one access phase (32 four-byte banks for FP32; 16 lanes of
// eight-byte words for FP64).  Without it a 416-byte stride put every fourth
// FP32 group on the same bank.
__host__ __device__ inline size_t forcen_table_bytes(int np, int stride, size_t ct) {
    return ((size_t)2 * np * stride * ct + 7) & ~size_t(7);
}
__host__ __device__ inline size_t forcen_group_bytes(int np, int stride, size_t ct, int tpc) {
    const size_t base = forcen_table_bytes(np, stride, ct) + sizeof(double) * np * 6;
    const int nb = ct == 4 ? 32 : 16;                         // banks per phase, in CT words
    const int lanes = ct == 4 ? 32 : 16;                      // lanes per phase
    const int groups = lanes / tpc > 1 ? lanes / tpc : 1;     // groups per phase
    size_t best = base;
    int best_d = -1;
    for (int k = 0; k < 8; k++) {
        const size_t g = base + 8 * (size_t)k;
        const int S = (int)((g / ct) % (size_t)nb);
        int dmin = nb;
        for (int a = 1; a < groups; a++) {
            const int o = (a * S) % nb;
            const int d = o < nb - o ? o : nb - o;
            if (d < dmin) dmin = d;
        }
        if (dmin > best_d) {
            best_d = dmin;
            best = g;
        }
    }
    return best;
}

template <int NB, typename CT, int TPC>
__global__ void __launch_bounds__(128) k_forcen(BatchView B, const int* clusters, const long long* n_ptr,
                                                long long cap, int stride) {
    const long long n = min(*n_ptr, cap);
    constexpr int NP = Topo<NB>::NP;
    constexpr int G = 32 / TPC;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int warp_in_block = threadIdx.x >> 5;
    const int grp = lane / TPC, gl = lane % TPC;
    // per-group shared layout: T[NP*stride], D[NP*stride] (CT); geo[NP][4], fc[NP], fcd[NP] (double)
    const size_t tbytes = forcen_table_bytes(NP, stride, sizeof(CT));
    const size_t gbytes = forcen_group_bytes(NP, stride, sizeof(CT), TPC);
    unsigned char* gbase = smem + ((size_t)warp_in_block * G + grp) * gbytes;
    CT* T = reinterpret_cast<CT*>(gbase);
    CT* D = T + NP * stride;
    double* geo = reinterpret_cast<double*>(gbase + tbytes);
    double* fcs = geo + 4 * NP;
    double* fcds = fcs + NP;

    // work queue: each warp claims kChunk consecutive steps (G clusters each) at a
    // time, so warps that drew cheap clusters come back for more
    const long long steps = (n + G - 1) / G;
    constexpr long long kChunk = 2;
    unsigned long long* head = &B.queue[NB - 3];
    EVAcc acc;

    for (;;) {
    long long st0 = 0;
    if (lane == 0) st0 = (long long)atomicAdd(head, (unsigned long long)kChunk);
    st0 = __shfl_sync(kFull, st0, 0);
    if (st0 >= steps) break;
    const long long st1 = min(steps, st0 + kChunk);
    for (long long step = st0; step < st1; step++) {
        const long long c = step * G + grp;
        const bool have = c < n;
        int id[NB];
        int s = 0;
        const SysDesc* d = nullptr;
        const DevParamSet* P = nullptr;
        const TupleRec* R = nullptr;
        int nc = 0;
        if (have) {
            for (int k = 0; k < NB; k++) id[k] = clusters[(long long)NB * c + k];
            s = B.atom_sys[B.ghost_parent[id[0]]];
            d = &B.sys[s];
            P = &B.psets[d->pset];
            int u = 0;
            for (int k = 0; k < NB; k++) u = u * P->ntypes + B.atom_type[B.ghost_parent[id[k]]];
            R = (NB == 3 ? P->t3 : P->t4) + u;
            if (R->valid) nc = R->ncoef;
            // geometry of this lane's pairs
            for (int p = gl; p < NP; p += TPC) {
                double dr[3], r;
                pair_geom(B, d->h, id[Topo<NB>::a(p)], id[Topo<NB>::b(p)], dr, r);
                geo[4 * p + 0] = dr[0]; geo[4 * p + 1] = dr[1]; geo[4 * p + 2] = dr[2]; geo[4 * p + 3] = r;
            }
        }
        __syncwarp();
        if (nc > 0) {   // compute_3B/4B early-outs on the per-pair outer cutoffs
            for (int p = 0; p < NP; p++)
                if (geo[4 * p + 3] >= R->rout[p]) { nc = 0; break; }
        }
        const int order = NB == 3 ? (P ? P->o3 : 0) : (P ? P->o4 : 0);
        if (nc > 0) {
            for (int p = gl; p < NP; p += TPC) {
                const double r = geo[4 * p + 3];
                cheby_table<CT>(T + p * stride, D + p * stride, r, R->rin[p], R->lam[p], R->xavg[p], R->xdiff[p],
                                order, P->inner_smooth, B.flags);
                CT fc, fcd;
                fcut_eval<CT>(*P, r, R->rout[p], fc, fcd);
                fcs[p] = double(fc);
                fcds[p] = double(fcd);
            }
        }
        __syncwarp();
        // contraction
        CT S = CT(0), Gp[NP];
        for (int p = 0; p < NP; p++) Gp[p] = CT(0);
        if (nc > 0) {
            const CT* cf = coefn<CT, NB>(*P) + R->coef_off;
            const uint32_t* pw = (NB == 3 ? P->p3 : P->p4) + R->coef_off;
            if (!ck_bound(B, R->coef_off >= 0 && R->coef_off + (long long)nc <= (NB == 3 ? P->n_c3 : P->n_c4))) nc = 0;
            for (int k = gl; k < nc; k += TPC) {
                const CT a = cf[k];
                const uint32_t pk = pw[k];
                CT t[NP], dd[NP];
#pragma unroll
                for (int p = 0; p < NP; p++) {
                    int q = (pk >> (kPowBits * p)) & 31u;
                    if (!ck_bound(B, q < stride)) q = 0;
                    t[p] = T[p * stride + q];
                    dd[p] = D[p * stride + q];
                }
                // prefix/suffix products of the T's
                CT pre[NP + 1], suf[NP + 1];
                pre[0] = a;
#pragma unroll
                for (int p = 0; p < NP; p++) pre[p + 1] = pre[p] * t[p];
                suf[NP] = CT(1);
#pragma unroll
                for (int p = NP - 1; p >= 0; p--) suf[p] = suf[p + 1] * t[p];
                S += pre[NP];
#pragma unroll
                for (int p = 0; p < NP; p++) Gp[p] += pre[p] * dd[p] * suf[p + 1];
            }
        }
        // combine the TPC partial sums of each cluster
#pragma unroll
        for (int off = TPC / 2; off > 0; off >>= 1) {
            S += __shfl_xor_sync(kFull, S, off);
#pragma unroll
            for (int p = 0; p < NP; p++) Gp[p] += __shfl_xor_sync(kFull, Gp[p], off);
        }
        if constexpr (sizeof(CT) == 4) {   // mixed form: the epilogue in FP32 (cluster_epilogue_f32)
            if (nc > 0 && gl == 0) {
                float drf[NP][3], rinv[NP], fcf[NP], fcdf[NP], Gf[NP];
                for (int p = 0; p < NP; p++) {
                    for (int k = 0; k < 3; k++) drf[p][k] = float(geo[4 * p + k]);
                    rinv[p] = 1.0f / float(geo[4 * p + 3]);
                    fcf[p] = float(fcs[p]);
                    fcdf[p] = float(fcds[p]);
                    Gf[p] = float(Gp[p]);
                }
                double e_c, vir_c[6];
                cluster_epilogue_f32<NB>(B, id, drf, rinv, fcf, fcdf, float(S), Gf, e_c, vir_c);
                acc.add(B, s, e_c, vir_c);
            }
        } else if (nc > 0 && gl == 0) {
            double fc[NP], fcd[NP], pre[NP + 1], suf[NP + 1];
            for (int p = 0; p < NP; p++) { fc[p] = fcs[p]; fcd[p] = fcds[p]; }
            pre[0] = 1.0;
            for (int p = 0; p < NP; p++) pre[p + 1] = pre[p] * fc[p];
            suf[NP] = 1.0;
            for (int p = NP - 1; p >= 0; p--) suf[p] = suf[p + 1] * fc[p];
            const double Sd = double(S);
            double f[NB][3];
            for (int k = 0; k < NB; k++) f[k][0] = f[k][1] = f[k][2] = 0.0;
            double vir[6] = {0, 0, 0, 0, 0, 0};
            for (int p = 0; p < NP; p++) {
                const double* dr = &geo[4 * p];
                const double fsp = pre[p] * suf[p + 1] / dr[3] * (fc[p] * double(Gp[p]) + fcd[p] * Sd);
                const int a = Topo<NB>::a(p), b = Topo<NB>::b(p);
                for (int k = 0; k < 3; k++) {
                    f[a][k] += fsp * dr[k];
                    f[b][k] -= fsp * dr[k];
                }
                virial_add(vir, fsp, dr);
            }
            for (int k = 0; k < NB; k++) add_force(B, id[k], f[k][0], f[k][1], f[k][2]);
            acc.add(B, s, pre[NP] * Sd, vir);
        }
        __syncwarp();
    }
    }
    acc.flush_warp(B);
}

template <int NB, typename CT>
void launch_n(const BatchView& B, const int* clusters, const long long* n_ptr, long long n, int tpc, int stride,
              const ForceLaunch& L, cudaStream_t st) {
    if (n <= 0) return;
    constexpr int NP = NB * (NB - 1) / 2;
    const int block = 128;
    const size_t gbytes = forcen_group_bytes(NP, stride, sizeof(CT), tpc);
    const int G = 32 / tpc;
    const size_t smem = gbytes * G * (block / 32);
    const long long steps = (n + G - 1) / G;
    long long want = (long long)sm_count() * L.blocks_per_sm;
    long long need = (steps + (block / 32) - 1) / (block / 32);
    const unsigned grid = (unsigned)(want < need ? want : need);
#define CK_LAUNCH(T_)                                                                          \
    do {                                                                                       \
        auto kern = k_forcen<NB, CT, T_>;                                                      \
        if (smem > 48 * 1024) allow_max_smem((const void*)kern);                                \
        count_launch(), kern<<<grid, block, smem, st>>>(B, clusters, n_ptr, n, stride);                               \
    } while (0)
    switch (tpc) {
        case 1: CK_LAUNCH(1); break;
        case 2: CK_LAUNCH(2); break;
        case 4: CK_LAUNCH(4); break;
        case 8: CK_LAUNCH(8); break;
        case 16: CK_LAUNCH(16); break;
        default: CK_LAUNCH(32); break;
    }
#undef CK_LAUNCH
}

// Throughput probe for the roofline denominator: 8 independent FMA chains per
// thread over every SM; the result is only stored if it hits an impossible
// value, which keeps the chains live.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, int iters, T b, T c) {
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = T(threadIdx.x + k) * T(1e-3);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
    }
    T s = a[0] + a[1] + a[2] + a[3] + a[4] + a[5] + a[6] + a[7];
    if (s == T(-1.2345e-7)) out[0] = s;
}

}  // namespace

double fma_peak_tflops(int precision) {
    const int blocks = sm_count() * 8, threads = 256;
    const int iters = precision == kMixed ? 1 << 16 : 1 << 12;
    void* out = nullptr;
    if (cudaMalloc(&out, 16) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        if (precision == kMixed)
            count_launch(), k_fma_probe<float><<<blocks, threads>>>((float*)out, iters, 1.0000001f, 1e-7f);
        else
            count_launch(), k_fma_probe<double><<<blocks, threads>>>((double*)out, iters, 1.0000000001, 1e-12);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return -1.0;
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    return flops / (best * 1e-3) / 1e12;
}

cudaError_t allow_max_smem(const void* kernel) {
    static std::mutex mu;
    static std::set<const void*> done;
    std::lock_guard<std::mutex> g(mu);
    if (done.count(kernel)) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) done.insert(kernel);
    return e;
}

int sm_count() {
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

void launch_force2(const BatchView& B, const int* l2_owner, const ForceLaunch& L, cudaStream_t st) {
    const long long n2 = B.n2_cap;
    const long long ntot = n2 > B.n_atoms_total ? n2 : B.n_atoms_total;
    if (ntot <= 0) return;
    long long want = (long long)sm_count() * 8;
    long long need = (ntot + 255) / 256;
    const unsigned grid = (unsigned)(want < need ? want : need);
    // The 1-/2-body stage runs in FP64 in both precision forms.  Fitted force
    // fields' 2-body series alternate in sign with coefficients of 10-10^3
    // (the CHON and HN3 parameter files), so an FP32 sum cancels away ~1e-6 of
    // the energy; this stage is a few per cent of an evaluation.
    count_launch(), k_force2<double><<<grid, 256, 0, st>>>(B, l2_owner);
}

void launch_force3(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    const long long* np = B.e_off3 + B.n2_cap;
    if (L.precision == kMixed) launch_n<3, float>(B, B.c3, np, B.n3_cap, L.tpc3, L.stride3, L, st);
    else launch_n<3, double>(B, B.c3, np, B.n3_cap, L.tpc3, L.stride3, L, st);
}

void launch_force4(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    const long long* np = B.e_off4 + B.n2_cap;
    if (L.precision == kMixed) launch_n<4, float>(B, B.c4, np, B.n4_cap, L.tpc4, L.stride4, L, st);
    else launch_n<4, double>(B, B.c4, np, B.n4_cap, L.tpc4, L.stride4, L, st);
}

}  // namespace ck
