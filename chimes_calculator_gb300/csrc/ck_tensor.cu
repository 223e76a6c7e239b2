// Tensor-core 3-body contraction (mixed form) on the fifth-generation tensor
// cores: tcgen05.mma with TF32 operands in shared memory and FP32
// accumulators in tensor memory (TMEM).
//
// For the clusters of one ordered type tuple, with R powers per pair and the
// tuple's coefficients as a dense matrix A[q_ij][J], J = q_ik * R + q_jk
// (the factored form's row and column indices, ck_common.h FactRow):
//   W  = X  . A,   X[c][q]  = T_ij(c)[q]        (energy and column gradients)
//   W' = dX . A,   dX[c][q] = dT_ij/dr(c)[q]    (row gradient)
// one MMA pair per 128 clusters (M = 128, K = R padded to 8 or 16, N = R^2
// padded to 16).  Each cluster's thread then reduces its TMEM row:
//   V[b] = sum_c W[b,c] T_jk[c],  V2[b] = sum_c W[b,c] dT_jk[c],
//   V'[b] = sum_c W'[b,c] T_jk[c]
//   S = sum_b V[b] T_ik[b],   G_ij = sum_b V'[b] T_ik[b],
//   G_ik = sum_b V[b] dT_ik[b],   G_jk = sum_b V2[b] T_ik[b]
// which are the sums of compute_3B (chimesFF/src/chimesFF.cpp:2068-2169) in
// another association order.
//
// Precision: TF32 keeps 10 mantissa bits, so both operands are split into
// three TF32 parts (high h, middle m, low l: each the TF32 rounding of what
// the previous ones leave) and W = Xh.Ah + Xh.Am + Xm.Ah + Xh.Al + Xl.Ah +
// Xm.Am (six MMAs per product; the dropped terms are ~2^-33 relative), with
// FP32 accumulation: the FP32 contraction's accuracy.  (With two parts and
// three MMAs the error is ~2^-21 per product, 3e-6 of the stress of the
// reference's HN3 force field.)  Distances (minimum image) and the Morse
// exponential stay in FP64; the Chebyshev recursion, cutoff and the
// cluster's force scalars, forces and virial are FP32 (they derive from the
// FP32 sums); the per-atom force, energy and virial accumulation is FP64.
// GB300 issues one FP64 warp instruction per 16 cycles per SM, so FP64 work
// bounds this kernel: with the pair-table cache (k_pair_tables) the geometry,
// exponential and tables of the pairs ij and ik -- list entries of the
// cluster's first atom -- are read instead of recomputed per cluster.
//
// Work: persistent CTAs of 128 threads (one cluster per thread) take
// 128-cluster tiles from an atomic queue over the clusters bucketed by
// (parameter set, tuple) and padded to 128 slots, so a tile has one tuple.
// Per tile: the tuple's coefficient image (B operand) is copied to shared
// memory when the tuple changes; each thread builds its cluster's tables and
// writes its X / dX rows (K-major, no-swizzle core-matrix layout); one thread
// issues the MMAs and commits them to an mbarrier; every thread waits on it
// with a bounded poll, reads its TMEM row in 16-column chunks and finishes the
// cluster.  At most two CTAs per SM (their shared memory) hold 256 TMEM
// columns each.  A wait that runs out sets flags[7] and the CTA stops after
// freeing its TMEM.
#include <cuda_runtime.h>

#include <cstdint>

#include "ck_common.h"
#include "ck_force_common.cuh"
#include "ck_kernels.h"
#include "ck_math.cuh"

namespace ck {

namespace {

constexpr int kTcTile = 128;              // clusters per tile (MMA M)
constexpr uint32_t kTcCols = 256;         // TMEM columns per CTA: W at 0, W' at 128
constexpr int kTcSpin = 1 << 22;          // bounded mbarrier wait: polls (~0.15 s with the back-off)
constexpr size_t kTcMinSmem = 80 * 1024;  // keeps two CTAs per SM (TMEM: 2 x 256 of 512 columns)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05.mma: start address, leading
// byte offset (between core matrices adjacent in K), stride byte offset
// (between core matrices adjacent in M/N), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

// Chebyshev tables T[0..R), dT/dr[0..R) and cutoff of one pair, in registers
// (the arithmetic of pair_setup / cheby_fill_strided, ck_factored.cu and
// ck_math.cuh, unrolled for a compile-time R).
template <int R>
__device__ __forceinline__ void pair_regs(const DevParamSet& P, const TupleRec& Q, int p, double r, float (&T)[R],
                                          float (&D)[R], float& fc, float& fcd, int* flags) {
    const double rin = Q.rin[p];
    const bool oor = r < rin;
    const double rr = oor ? rin : r;
    const double e = exp(-rr * Q.inv_lam[p]);
    const double xd = (e - Q.xavg[p]) * Q.inv_xdiff[p];
    const double dxdr = -e * Q.inv_lam[p] * Q.inv_xdiff[p];
    const float x = float(xd), tx = 2.0f * x, g = float(dxdr);
    float k = 0.0f, dm = 1.0f;
    if (oor) {
        atomicAdd(&flags[4], 1);
        const double damp = exp((r - rin) / P.inner_smooth);
        k = float(P.inner_smooth * (damp - 1.0));
        dm = float(damp);
    }
    T[0] = 1.0f;
    D[0] = 0.0f;
    float t0 = 1.0f, t1 = x, u0 = 1.0f, u1 = tx;
    if (R > 1) {
        const float d1 = g * u0;
        T[1] = oor ? t1 + k * d1 : t1;
        D[1] = oor ? d1 * dm : d1;
    }
#pragma unroll
    for (int n = 2; n < R; n++) {
        const float t2 = tx * t1 - t0;
        const float u2 = tx * u1 - u0;
        const float dn = float(n) * g * u1;
        T[n] = oor ? t2 + k * dn : t2;
        D[n] = oor ? dn * dm : dn;
        t0 = t1; t1 = t2; u0 = u1; u1 = u2;
    }
    const double finv = Q.fc_inv[p];
    if (!P.tersoff) {
        const float f0 = 1.0f - float(r) * float(finv);
        fc = f0 * f0 * f0;
        fcd = f0 * f0 * (-3.0f * float(finv));
    } else {
        const double th = Q.fc_th[p];
        if (r < th) { fc = 1.0f; fcd = 0.0f; }
        else if (r > Q.rout[p]) { fc = 0.0f; fcd = 0.0f; }
        else {
            const float f0 = float(r - th) * float(finv) * float(kPi) + float(kPi / 2.0);
            float sn, cs;
            sincosf(f0, &sn, &cs);
            fc = 0.5f + 0.5f * sn;
            fcd = 0.5f * cs * (float(kPi) * float(finv));
        }
    }
}

// One row of an A operand's three part images (K-major, no swizzle; part t
// at img + t * AFL): row m's KP values at core-matrix rows, split into TF32
// high / middle / low parts (zero past R, or all zero).
template <int R, int KP>
__device__ __forceinline__ void put_row(float* img, int m, const float (&v)[R], bool on) {
    constexpr int SBOF = KP * 8;   // floats between row blocks (KP/4 core matrices of 32 floats)
    constexpr int AFL = 128 * KP;  // floats per part image
    float* r0 = img + (m >> 3) * SBOF + (m & 7) * 4;
#pragma unroll
    for (int j = 0; j < KP / 4; j++) {
        float h[4], md[4], l[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = 4 * j + q;
            const float x = (on && k < R) ? v[k < R ? k : 0] : 0.0f;
            h[q] = tf32_hi(x);
            const float rest = x - h[q];
            md[q] = tf32_hi(rest);
            l[q] = rest - md[q];
        }
        *reinterpret_cast<float4*>(r0 + j * 32) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(r0 + AFL + j * 32) = make_float4(md[0], md[1], md[2], md[3]);
        *reinterpret_cast<float4*>(r0 + 2 * AFL + j * 32) = make_float4(l[0], l[1], l[2], l[3]);
    }
}

template <int R>
__global__ void __launch_bounds__(128) k_forcetc3(BatchView B, const int* clusters, const int* perm,
                                                  const long long* perm_n, long long perm_cap) {
    constexpr int KP = tc3_kpad(R);                     // K padded to whole MMA steps (8 for TF32)
    constexpr int NP = tc3_npad(R);                     // N padded to 16
    constexpr int AFL = kTcTile * KP;                   // floats per A part image
    constexpr int BFL = NP * KP;                        // floats per B part image
    constexpr uint32_t LBO = 128, SBO = KP * 32;        // bytes: next core matrix in K; next 8 rows
    static_assert(kTc3Parts == 3, "the MMA sequence below pairs three parts");
    extern __shared__ __align__(1024) unsigned char smem[];
    float* Xs = reinterpret_cast<float*>(smem);         // T_ij parts h, m, l
    float* Ds = Xs + 3 * AFL;                           // dT_ij/dr parts
    float* Bs = Ds + 3 * AFL;                           // coefficient parts
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ long long s_tile, s_next;

    const int tid = threadIdx.x, warp = tid >> 5;
    const long long n = min(*perm_n, perm_cap);
    const long long ntiles = n / kTcTile;
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NP >> 3) << 17) |
                           ((uint32_t)(kTcTile >> 4) << 24);
    uint32_t phase = 0;
    int loaded = -1;                                    // tc_off of the B image in shared memory
    const DevParamSet* loaded_set = nullptr;
    EVAcc acc;

    // Tiles: first a contiguous block per CTA (consecutive tiles share the
    // tuple's coefficient image, so the image is seldom reloaded, and the
    // pair-cache entries and positions of the same atoms), then the last
    // eighth claimed one at a time so that the CTAs finish together.  Claimed
    // one ahead, so that each thread can prefetch its next cluster's data into
    // L2 while the current tile's MMAs run.
    const long long per = ntiles * 7 / 8 / gridDim.x;
    long long own = (long long)blockIdx.x * per;        // thread 0's next tile of its block
    const long long own_end = own + per, shared0 = per * gridDim.x;
    auto claim = [&]() -> long long {
        return own < own_end ? own++ : shared0 + (long long)atomicAdd(&B.queue[0], 1ull);
    };
    if (tid == 0) s_next = claim();
    for (;;) {
        if (tid == 0) {
            s_tile = s_next;
            s_next = s_next < ntiles ? claim() : ntiles;
        }
        __syncthreads();
        const long long tile = s_tile;
        const long long next = s_next;
        if (tile >= ntiles) break;
        const long long base = tile * kTcTile;
        const int c0 = perm[base];
        if (c0 < 0) {               // uniform: a tile never starts in a bucket's padding
            __syncthreads();
            continue;
        }
        int id0[3], s0, u0;
        const DevParamSet* P;
        const TupleRec* Rt = cluster_tuple<3>(B, clusters, c0, id0, s0, P, u0);
        // the tuple's coefficient image at this kernel's width, when it is not
        // the one in shared memory
        if (Rt->tc_off != loaded || P != loaded_set) {
            const long long img = Rt->tc_off + tc3_offset(P->R3, R);
            const bool img_ok = ck_bound(B, Rt->tc_off >= 0 && img + (long long)kTc3Parts * BFL <= P->n_tc3);
            const float4* src = reinterpret_cast<const float4*>(P->tc3 + (img_ok ? img : 0));
            float4* dst = reinterpret_cast<float4*>(Bs);
            for (int q = tid; q < kTc3Parts * BFL / 4; q += kTcTile) dst[q] = src[q];
            loaded = Rt->tc_off;
            loaded_set = P;
        }
        // this thread's cluster: geometry, cutoff early-outs, tables; with
        // the cache, pairs ij and ik (list entries of atom i) come from it
        const int c = perm[base + tid];
        bool active = c >= 0;
        int id[3] = {0, 0, 0};
        int s = 0;
        float drf[3][3], rinv[3] = {0, 0, 0}, fcf[3] = {0, 0, 0}, fcdf[3] = {0, 0, 0};
        double rr[3] = {0, 0, 0};
        long long ent[2] = {0, 0};
        float T0[R], D0[R], T1[R], D1[R], T2[R], D2[R];
#pragma unroll
        for (int q = 0; q < R; q++) T0[q] = D0[q] = T1[q] = D1[q] = T2[q] = D2[q] = 0.0f;
        const bool use_pc = B.use_pc3 != 0;
        if (active) {
            for (int k = 0; k < 3; k++) id[k] = clusters[3LL * c + k];
            s = B.atom_sys[B.ghost_parent[id[0]]];
#pragma unroll
            for (int p = 0; p < 3; p++) {
                double d[3], r;
                if (use_pc && p < 2) {
                    ent[p] = B.c3e[2LL * c + p];
                    const double* g = B.pcd3 + 8 * ent[p];
                    d[0] = g[0]; d[1] = g[1]; d[2] = g[2]; r = g[3];
                } else {
                    pair_geom(B, B.sys[s].h, id[Topo<3>::a(p)], id[Topo<3>::b(p)], d, r);
                }
                drf[p][0] = float(d[0]); drf[p][1] = float(d[1]); drf[p][2] = float(d[2]);
                rr[p] = r;
                if (r >= Rt->rout[p]) active = false;   // compute_3B's early-outs
            }
        }
        if (active) {
            const int R3 = P->R3;   // the set's own powers; entries above it multiply zero coefficients
            if (use_pc) {
                const float* pct = reinterpret_cast<const float*>(B.pct3);
#pragma unroll
                for (int p = 0; p < 2; p++) {
                    const double* g = B.pcd3 + 8 * ent[p];
                    const float* tab = pct + ent[p] * 2 * R;
                    float* T = p == 0 ? T0 : T1;
                    float* D = p == 0 ? D0 : D1;
#pragma unroll
                    for (int q = 0; q < R; q++) {
                        T[q] = q < R3 ? tab[q] : 0.0f;
                        D[q] = q < R3 ? tab[R + q] : 0.0f;
                    }
                    fcf[p] = float(g[4]);
                    fcdf[p] = float(g[5]);
                    if (g[6] != 0.0) atomicAdd(&B.flags[4], 1);
                }
            } else {
                pair_regs<R>(*P, *Rt, 0, rr[0], T0, D0, fcf[0], fcdf[0], B.flags);
                pair_regs<R>(*P, *Rt, 1, rr[1], T1, D1, fcf[1], fcdf[1], B.flags);
            }
            pair_regs<R>(*P, *Rt, 2, rr[2], T2, D2, fcf[2], fcdf[2], B.flags);
#pragma unroll
            for (int p = 0; p < 3; p++) rinv[p] = 1.0f / float(rr[p]);
        }
        put_row<R, KP>(Xs, tid, T0, active);
        put_row<R, KP>(Ds, tid, D0, active);
        // generic-proxy writes of the operands -> visible to the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t xs = smem_u32(Xs), ds = smem_u32(Ds), bs = smem_u32(Bs);
            constexpr uint32_t AB = AFL * 4, BB = BFL * 4;   // bytes per part image
            // part pairs (operand part, coefficient part), smallest first so
            // that the accumulator is small while the small terms go in (the
            // tensor core's accumulation rounds each addition at the
            // accumulator's magnitude): m.m, h.l, l.h, h.m, m.h, then h.h
            constexpr int pa[6] = {1, 0, 2, 0, 1, 0}, pb[6] = {1, 2, 0, 1, 0, 0};
#pragma unroll
            for (int t = 0; t < 6; t++) {
#pragma unroll
                for (int ks = 0; ks < KP / 8; ks++) {
                    const uint32_t o = ks * 256;   // two core matrices along K per step
                    const uint64_t bd = umma_desc(bs + pb[t] * BB + o, LBO, SBO);
                    const int accum = ks > 0 || t > 0;
                    mma_tf32(tmem, umma_desc(xs + pa[t] * AB + o, LBO, SBO), bd, idesc, accum);
                    mma_tf32(tmem + 128, umma_desc(ds + pa[t] * AB + o, LBO, SBO), bd, idesc, accum);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&s_bar))
                         : "memory");
        }
        // prefetch the next tile's cluster data (list, pair-table entries,
        // positions) into L2 while the MMAs run
        if (next < ntiles) {
            const int cn = perm[next * kTcTile + tid];
            if (cn >= 0) {
                const int* ids = clusters + 3LL * cn;
                const int g0 = ids[0], g2 = ids[2];
                asm volatile("prefetch.global.L2 [%0];" ::"l"(B.ghost_fs + 3LL * g0));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(B.ghost_fs + 3LL * ids[1]));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(B.ghost_fs + 3LL * g2));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(B.ghost_parent + g0));
                if (use_pc) {
                    const long long e0 = B.c3e[2LL * cn], e1 = B.c3e[2LL * cn + 1];
                    const float* pct = reinterpret_cast<const float*>(B.pct3);
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(B.pcd3 + 8 * e0));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(B.pcd3 + 8 * e1));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pct + e0 * 2 * R));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pct + e0 * 2 * R + R + R - 1));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pct + e1 * 2 * R));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pct + e1 * 2 * R + R + R - 1));
                }
            }
        }
        // bounded wait for the MMAs of this tile (non-blocking polls, then a back-off)
        uint32_t done = 0;
        for (int it = 0; it < kTcSpin && !done; it++) {
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                : "=r"(done)
                : "r"(smem_u32(&s_bar)), "r"(phase)
                : "memory");
            if (!done && it > 256) __nanosleep(32);
        }
        phase ^= 1u;
        if (!__syncthreads_and(done)) {
            if (tid == 0) atomicOr(&B.flags[7], 1);
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // this thread's TMEM row (lane = tid): W at columns [0, NP), W' at [128, 128 + NP)
        float V[R], V2[R], Vp[R];
#pragma unroll
        for (int b = 0; b < R; b++) V[b] = V2[b] = Vp[b] = 0.0f;
        const uint32_t row = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int q = 0; q < NP / 16; q++) {
            float w[16], wp[16];
            tmem_ld16(row + 16 * q, w);
            tmem_ld16(row + 128 + 16 * q, wp);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const int j = 16 * q + u;
                if (j < R * R) {
                    const int b = j / R, cc = j % R;
                    V[b] += w[u] * T2[cc];
                    V2[b] += w[u] * D2[cc];
                    Vp[b] += wp[u] * T2[cc];
                }
            }
        }
        double e_c = 0.0, vir_c[6] = {0, 0, 0, 0, 0, 0};
        if (active) {
            float S = 0.0f, G0 = 0.0f, G1 = 0.0f, G2 = 0.0f;
#pragma unroll
            for (int b = 0; b < R; b++) {
                S += V[b] * T1[b];
                G0 += Vp[b] * T1[b];
                G1 += V[b] * D1[b];
                G2 += V2[b] * T1[b];
            }
            const float G[3] = {G0, G1, G2};
            cluster_epilogue_f32<3>(B, id, drf, rinv, fcf, fcdf, S, G, e_c, vir_c);
        }
        acc.add_warp(B, s, e_c, vir_c, active);
        // TMEM and the operand images are rewritten by the next tile
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    acc.flush_warp(B);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
}

template <int R>
void launch_tc_r(const BatchView& B, cudaStream_t st) {
    constexpr int KP = tc3_kpad(R);
    constexpr int NP = tc3_npad(R);
    size_t smem = sizeof(float) * (6 * (size_t)kTcTile * KP + kTc3Parts * (size_t)NP * KP);
    if (smem < kTcMinSmem) smem = kTcMinSmem;
    auto kern = k_forcetc3<R>;
    // the kernel's own dynamic size (its static shared memory counts against
    // the opt-in maximum, so the largest value is not accepted here); every
    // launch of a width asks for the same size, so concurrent callers agree
    cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const long long tiles = B.perm3_cap / kTcTile;
    long long want = 2LL * sm_count();
    const unsigned grid = (unsigned)(want < tiles ? want : (tiles > 0 ? tiles : 1));
    const long long* pn = B.bk_start + B.nbk3;
    count_launch(), kern<<<grid, kTcTile, smem, st>>>(B, B.c3, B.perm3, pn, B.perm3_cap);
}

}  // namespace

bool tc3_supported(int rf3) { return rf3 >= 2 && rf3 <= kTc3MaxR; }

void launch_force3tc(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    if (B.perm3_cap <= 0 || B.nbk3 <= 0) return;
    switch (L.rf3) {
        case 2: launch_tc_r<2>(B, st); break;
        case 3: launch_tc_r<3>(B, st); break;
        case 4: launch_tc_r<4>(B, st); break;
        case 5: launch_tc_r<5>(B, st); break;
        case 6: launch_tc_r<6>(B, st); break;
        case 7: launch_tc_r<7>(B, st); break;
        case 8: launch_tc_r<8>(B, st); break;
        case 9: launch_tc_r<9>(B, st); break;
        case 10: launch_tc_r<10>(B, st); break;
        case 11: launch_tc_r<11>(B, st); break;
        default: break;
    }
}

}  // namespace ck
