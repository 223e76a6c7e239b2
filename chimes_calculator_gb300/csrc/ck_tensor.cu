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


// ---------------------------------------------------------------------------
// Tensor-core 4-body contraction (mixed form).  With R powers per pair a
// tuple's coefficients form a dense matrix A[I][J], I = (q_ij, q_ik, q_il) and
// J = (q_jk, q_jl, q_kl) (R^3 each).  For a cluster, X_I = T_ij T_ik T_il and
// Y_J = T_jk T_jl T_kl: S = X.A.Y, and the pair gradients are
//   G_ij = dX_ij.A.Y, G_ik = dX_ik.A.Y, G_il = dX_il.A.Y  (dX_p: T_p -> dT_p/dr)
//   G_jk, G_jl, G_kl = W.dY_p with W = X.A.
// A tile is 32 clusters of one tuple and the MMA's 128 rows are the four row
// vectors X, dX_ij, dX_ik, dX_il of each (row 32 v + c: warp v builds variant
// v of cluster c and reads its TMEM row back), so one M = 128, N = R^3 MMA
// chain gives W, W_ij, W_ik, W_il for all 32 clusters; each row is then
// contracted with the cluster's column tables, and warp 0 forms the forces.
// Operands in three TF32 parts as in the 3-body kernel: the five small part
// products (smallest first) and the large one go into two accumulators that
// are summed in FP32.  The A operand passes through one shared-memory buffer
// in K halves (R = 4: 2 x 32), which lets two CTAs share an SM.  Pair tables
// are computed by the four threads of a cluster (pairs v and v + 4), after
// the early-outs of all six pairs.
constexpr int kTc4Tile = 32;              // clusters per tile

template <int R>
__global__ void __launch_bounds__(128, 2) k_forcetc4(BatchView B, const int* clusters, const int* perm,
                                                     const long long* perm_n, long long perm_cap) {
    constexpr int N3 = R * R * R;
    constexpr int KP = tc4_kpad(N3);                    // K padded to whole MMA steps
    constexpr int NP = tc4_npad(N3);                    // N padded to 16
    // the A operand goes in K halves of KH through one buffer (two CTAs per
    // SM fit in shared memory that way)
    constexpr int KH = KP > 32 ? KP / 2 : KP;
    constexpr int NH = KP / KH;
    constexpr int AFL = 128 * KH;                       // floats per A part image (one K half)
    constexpr int BFL = NP * KP;                        // floats per B part image
    constexpr uint32_t LBO = 128, SBOA = KH * 32, SBOB = KP * 32;   // bytes: next core matrix in K; next 8 rows
    // TMEM: the large (h.h) and the small part products in separate
    // accumulators, summed in FP32 at the end (each accumulates its own terms
    // in order of size, whatever the K half)
    constexpr uint32_t DCOL = NP <= 32 ? 32 : (NP <= 64 ? 64 : 128);
    constexpr uint32_t COLS = 2 * DCOL;
    constexpr int C = kTc4Tile;
    static_assert(kTc3Parts == 3, "the MMA sequence below pairs three parts");
    extern __shared__ __align__(1024) unsigned char smem[];
    float* As = reinterpret_cast<float*>(smem);         // rows X / dX parts h, m, l
    float* Bs = As + 3 * AFL;                           // coefficient parts
    __shared__ float s_tab[6][2 * R][C];                // T, then dT/dr, per pair and cluster
    __shared__ float s_fc[6][C], s_fcd[6][C], s_rinv[6][C], s_dr[6][3][C];
    __shared__ double s_r[6][C];
    __shared__ int s_far[6][C];
    __shared__ float s_res[7][C];                       // S, G_0 .. G_5
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ long long s_tile, s_next;

    const int tid = threadIdx.x, warp = tid >> 5, c = tid & 31;
    const long long n = min(*perm_n, perm_cap);
    const long long ntiles = n / C;
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(COLS));
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
                           ((uint32_t)(128 >> 4) << 24);
    uint32_t phase = 0;
    int loaded = -1;                                    // tc_off of the B image in shared memory
    const DevParamSet* loaded_set = nullptr;
    EVAcc acc;

    // tiles: a contiguous block per CTA, then the last eighth one at a time
    // (as in the 3-body kernel), claimed one ahead
    const long long per = ntiles * 7 / 8 / gridDim.x;
    long long own = (long long)blockIdx.x * per;
    const long long own_end = own + per, shared0 = per * gridDim.x;
    auto claim = [&]() -> long long {
        return own < own_end ? own++ : shared0 + (long long)atomicAdd(&B.queue[1], 1ull);
    };
    if (tid == 0) s_next = claim();
    for (;;) {
        if (tid == 0) {
            s_tile = s_next;
            s_next = s_next < ntiles ? claim() : ntiles;
        }
        __syncthreads();
        const long long tile = s_tile;
        if (tile >= ntiles) break;
        const long long base = tile * C;
        const int c0 = perm[base];
        if (c0 < 0) {               // uniform: a tile never starts in a bucket's padding
            __syncthreads();
            continue;
        }
        int id0[4], s0, u0;
        const DevParamSet* P;
        const TupleRec* Rt = cluster_tuple<4>(B, clusters, c0, id0, s0, P, u0);
        if (Rt->tc_off != loaded || P != loaded_set) {
            const long long img = Rt->tc_off;
            const bool img_ok = ck_bound(B, img >= 0 && img + (long long)kTc3Parts * BFL <= P->n_tc4);
            const float4* src = reinterpret_cast<const float4*>(P->tc4 + (img_ok ? img : 0));
            float4* dst = reinterpret_cast<float4*>(Bs);
            for (int q = tid; q < kTc3Parts * BFL / 4; q += 128) dst[q] = src[q];
            loaded = Rt->tc_off;
            loaded_set = P;
        }
        // this cluster's geometry: pairs warp and warp + 4 (the four warps
        // cover the six pairs)
        const int cl = perm[base + c];
        int id[4] = {0, 0, 0, 0};
        int s = 0;
        if (cl >= 0) {
            for (int k = 0; k < 4; k++) id[k] = clusters[4LL * cl + k];
            s = B.atom_sys[B.ghost_parent[id[0]]];
        }
        for (int p = warp; p < 6; p += 4) {
            double d[3] = {0, 0, 0}, r = 1e300;
            if (cl >= 0) pair_geom(B, B.sys[s].h, id[Topo<4>::a(p)], id[Topo<4>::b(p)], d, r);
            s_far[p][c] = cl < 0 || r >= Rt->rout[p];   // compute_4B's early-outs
            s_r[p][c] = r;
            s_dr[p][0][c] = float(d[0]);
            s_dr[p][1][c] = float(d[1]);
            s_dr[p][2][c] = float(d[2]);
        }
        __syncthreads();
        bool active = true;
#pragma unroll
        for (int p = 0; p < 6; p++) active = active && !s_far[p][c];
        for (int p = warp; p < 6; p += 4) {
            float T[R], D[R], fc = 0.0f, fcd = 0.0f;
#pragma unroll
            for (int q = 0; q < R; q++) T[q] = D[q] = 0.0f;
            if (active) pair_regs<R>(*P, *Rt, p, s_r[p][c], T, D, fc, fcd, B.flags);
            const int R4 = P->R4;   // the set's own powers; entries above it multiply zero coefficients
#pragma unroll
            for (int q = 0; q < R; q++) {
                s_tab[p][q][c] = q < R4 ? T[q] : 0.0f;
                s_tab[p][R + q][c] = q < R4 ? D[q] : 0.0f;
            }
            s_fc[p][c] = fc;
            s_fcd[p][c] = fcd;
            s_rinv[p][c] = active ? 1.0f / float(s_r[p][c]) : 0.0f;
        }
        __syncthreads();
        // row 32 warp + c of the A operand: X (warp 0) or dX_ij, dX_ik, dX_il
        {
            float f0[R], f1[R], f2[R];
#pragma unroll
            for (int q = 0; q < R; q++) {
                f0[q] = s_tab[0][(warp == 1 ? R : 0) + q][c];
                f1[q] = s_tab[1][(warp == 2 ? R : 0) + q][c];
                f2[q] = s_tab[2][(warp == 3 ? R : 0) + q][c];
            }
            float* r0 = As + (tid >> 3) * (KH * 8) + (tid & 7) * 4;
            bool ok = true;
            for (int hf = 0; hf < NH && ok; hf++) {
                if (hf > 0) {
                    // the previous half's MMAs have read the buffer
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
                    ok = __syncthreads_and(done);
                    if (!ok) break;
                }
#pragma unroll
                for (int j = 0; j < KH / 4; j++) {
                    float h[4], md[4], l[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int k = hf * KH + 4 * j + u;
                        const int kk = k < N3 ? k : 0;
                        const float x = (active && k < N3) ? f0[kk / (R * R)] * f1[(kk / R) % R] * f2[kk % R] : 0.0f;
                        h[u] = tf32_hi(x);
                        const float rest = x - h[u];
                        md[u] = tf32_hi(rest);
                        l[u] = rest - md[u];
                    }
                    *reinterpret_cast<float4*>(r0 + j * 32) = make_float4(h[0], h[1], h[2], h[3]);
                    *reinterpret_cast<float4*>(r0 + AFL + j * 32) = make_float4(md[0], md[1], md[2], md[3]);
                    *reinterpret_cast<float4*>(r0 + 2 * AFL + j * 32) = make_float4(l[0], l[1], l[2], l[3]);
                }
                // generic-proxy writes of the operands -> visible to the tensor core
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncthreads();
                if (tid == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t as = smem_u32(As), bs = smem_u32(Bs);
                    constexpr uint32_t AB = AFL * 4, BB = BFL * 4;   // bytes per part image
                    // small part products smallest first (m.m, h.l, l.h, h.m, m.h) into
                    // the first accumulator, h.h into the second
                    constexpr int pa[6] = {1, 0, 2, 0, 1, 0}, pb[6] = {1, 2, 0, 1, 0, 0};
#pragma unroll
                    for (int t = 0; t < 6; t++) {
#pragma unroll
                        for (int ks = 0; ks < KH / 8; ks++) {
                            const uint32_t oa = ks * 256;                       // two core matrices along K per step
                            const uint32_t ob = (hf * (KH / 8) + ks) * 256;
                            const uint32_t d = t < 5 ? tmem : tmem + DCOL;
                            const int acc = hf > 0 || ks > 0 || (t > 0 && t < 5);
                            mma_tf32(d, umma_desc(as + pa[t] * AB + oa, LBO, SBOA),
                                     umma_desc(bs + pb[t] * BB + ob, LBO, SBOB), idesc, acc);
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(&s_bar))
                                 : "memory");
                }
            }
            // bounded wait for the last half's MMAs
            if (ok) {
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
                ok = __syncthreads_and(done);
            }
            if (!ok) {
                if (tid == 0) atomicOr(&B.flags[7], 1);
                break;
            }
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // this thread's TMEM row (small + large products), contracted with the
        // cluster's column tables (jk: d, jl: e, kl: f; J = (d R + e) R + f)
        float W[NP];
        const uint32_t row = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int q = 0; q < NP / 16; q++) {
            float big[16];
            tmem_ld16(row + 16 * q, W + 16 * q);
            tmem_ld16(row + DCOL + 16 * q, big);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int u = 0; u < 16; u++) W[16 * q + u] += big[u];
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        {
            float T3[R], D3[R], T4[R], D4[R], T5[R], D5[R];
#pragma unroll
            for (int q = 0; q < R; q++) {
                T3[q] = s_tab[3][q][c]; D3[q] = s_tab[3][R + q][c];
                T4[q] = s_tab[4][q][c]; D4[q] = s_tab[4][R + q][c];
                T5[q] = s_tab[5][q][c]; D5[q] = s_tab[5][R + q][c];
            }
            float S = 0.0f, G3 = 0.0f, G4 = 0.0f, G5 = 0.0f;
#pragma unroll
            for (int d = 0; d < R; d++) {
                float w = 0.0f, w1 = 0.0f, w2 = 0.0f;
#pragma unroll
                for (int e = 0; e < R; e++) {
                    float u = 0.0f, u1 = 0.0f;
#pragma unroll
                    for (int f = 0; f < R; f++) {
                        const float x = W[(d * R + e) * R + f];
                        u += x * T5[f];
                        u1 += x * D5[f];
                    }
                    w += u * T4[e];
                    w1 += u * D4[e];
                    w2 += u1 * T4[e];
                }
                S += w * T3[d];
                G3 += w * D3[d];
                G4 += w1 * T3[d];
                G5 += w2 * T3[d];
            }
            if (warp == 0) {
                s_res[0][c] = S;
                s_res[4][c] = G3;
                s_res[5][c] = G4;
                s_res[6][c] = G5;
            } else {
                s_res[warp][c] = S;   // G_ij, G_ik, G_il from the derivative rows
            }
        }
        __syncthreads();
        if (warp == 0) {
            double e_c = 0.0, vir_c[6] = {0, 0, 0, 0, 0, 0};
            if (active) {
                float dr[6][3], rinv[6], fc[6], fcd[6], G[6];
#pragma unroll
                for (int p = 0; p < 6; p++) {
                    dr[p][0] = s_dr[p][0][c]; dr[p][1] = s_dr[p][1][c]; dr[p][2] = s_dr[p][2][c];
                    rinv[p] = s_rinv[p][c];
                    fc[p] = s_fc[p][c];
                    fcd[p] = s_fcd[p][c];
                    G[p] = s_res[1 + p][c];
                }
                cluster_epilogue_f32<4>(B, id, dr, rinv, fc, fcd, s_res[0][c], G, e_c, vir_c);
            }
            acc.add_warp(B, s, e_c, vir_c, active);
        }
    }
    if (warp == 0) acc.flush_warp(B);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS));
}

template <int R>
void launch_tc4_r(const BatchView& B, cudaStream_t st) {
    constexpr int N3 = R * R * R;
    constexpr int KP = tc4_kpad(N3);
    constexpr int NP = tc4_npad(N3);
    constexpr int KH = KP > 32 ? KP / 2 : KP;
    const size_t smem = sizeof(float) * (3 * (size_t)128 * KH + kTc3Parts * (size_t)NP * KP);
    auto kern = k_forcetc4<R>;
    cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const long long tiles = B.perm4_cap / kTc4Tile;
    const long long want = 2LL * sm_count();   // two CTAs per SM (shared memory)
    const unsigned grid = (unsigned)(want < tiles ? want : (tiles > 0 ? tiles : 1));
    const long long* pn = B.bk_start + B.nbk3 + 1 + B.nbk4;
    count_launch(), kern<<<grid, 128, smem, st>>>(B, B.c4, B.perm4, pn, B.perm4_cap);
}

}  // namespace

bool tc3_supported(int rf3) { return rf3 >= 2 && rf3 <= kTc3MaxR; }
bool tc4_supported(int rf4) { return rf4 >= 2 && rf4 <= kTc4MaxR; }

void launch_force4tc(const BatchView& B, const ForceLaunch& L, cudaStream_t st) {
    if (B.perm4_cap <= 0 || B.nbk4 <= 0) return;
    switch (L.rf4) {
        case 2: launch_tc4_r<2>(B, st); break;
        case 3: launch_tc4_r<3>(B, st); break;
        case 4: launch_tc4_r<4>(B, st); break;
        default: break;
    }
}

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
