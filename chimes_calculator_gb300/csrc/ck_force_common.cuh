// Device helpers shared by the cluster force kernels (ck_force.cu,
// ck_factored.cu): pair geometry, force scatter to the caller's atoms, the
// per-system energy/virial accumulator and the per-cluster force epilogue.
#pragma once
#include <cuda_runtime.h>

#include "ck_common.h"
#include "ck_math.cuh"

namespace ck {

// Raises a kernel's dynamic shared-memory limit to the device's opt-in maximum,
// once per kernel.  The limit is a per-function attribute shared by every host
// thread, so it is never lowered: threads launching the same kernel with
// different shared-memory sizes (request-server workers) cannot race on it.
// The shared memory a launch actually gets is its own launch argument.
cudaError_t allow_max_smem(const void* kernel);

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Checked build (compiled with -DCK_BOUNDS, libchimescalc_bounds.so): index
// checks on the arrays the cluster kernels index with computed values --
// ghost slots, caller atoms, type tuples, coefficient and factored-entry
// ranges, Chebyshev powers, tensor-core images.  A failed check raises bit 2
// of flags[7] and the access is skipped (the call then returns an error); it
// never traps.  In the normal build the checks compile to nothing.
#ifdef CK_BOUNDS
__device__ __forceinline__ bool ck_bound(const BatchView& B, bool ok) {
    if (!ok) atomicOr(&B.flags[7], 2);
    return ok;
}
#else
__device__ __forceinline__ bool ck_bound(const BatchView&, bool) { return true; }
#endif
__device__ __forceinline__ void pair_geom(const BatchView& B, const double* h, int ga, int gb, double* dr, double& r) {
    if (!ck_bound(B, ga >= 0 && ga < B.n_ghost_total && gb >= 0 && gb < B.n_ghost_total)) {
        dr[0] = dr[1] = dr[2] = 0.0;
        r = 1e300;   // beyond every cutoff: the cluster is dropped
        return;
    }
    const double* fa = &B.ghost_fs[3 * (long long)ga];
    const double* fb = &B.ghost_fs[3 * (long long)gb];
    const double dx = fb[0] - fa[0], dy = fb[1] - fa[1], dz = fb[2] - fa[2];
    dr[0] = h[0] * dx + h[1] * dy + h[2] * dz;
    dr[1] = h[3] * dx + h[4] * dy + h[5] * dz;
    dr[2] = h[6] * dx + h[7] * dy + h[8] * dz;
    r = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
}

// Ordered type tuple of cluster c: its ghost slots, system, parameter set and tuple index.
template <int NB>
__device__ __forceinline__ const TupleRec* cluster_tuple(const BatchView& B, const int* clusters, long long c,
                                                         int* id, int& s, const DevParamSet*& P, int& u) {
    for (int k = 0; k < NB; k++) {
        id[k] = clusters[(long long)NB * c + k];
        if (!ck_bound(B, id[k] >= 0 && id[k] < B.n_ghost_total)) id[k] = 0;
    }
    s = B.atom_sys[B.ghost_parent[id[0]]];
    P = &B.psets[B.sys[s].pset];
    u = 0;
    for (int k = 0; k < NB; k++) u = u * P->ntypes + B.atom_type[B.ghost_parent[id[k]]];
    int ntup = 1;
    for (int k = 0; k < NB; k++) ntup *= P->ntypes;
    if (!ck_bound(B, u >= 0 && u < ntup)) u = 0;
    return (NB == 3 ? P->t3 : P->t4) + u;
}

__device__ __forceinline__ void add_force(const BatchView& B, int ghost, double fx, double fy, double fz) {
    const int o = B.atom_orig[B.ghost_parent[ghost]];
    if (!ck_bound(B, o >= 0 && o < B.n_in_total)) return;
    atomicAdd(&B.force[3 * (long long)o + 0], fx);
    atomicAdd(&B.force[3 * (long long)o + 1], fy);
    atomicAdd(&B.force[3 * (long long)o + 2], fz);
}

// Per-atom energy and virial of one n-atom interaction, shared equally by its
// atoms (Pair::ev_tally_mb, etc/lmp/etc/pair.cpp); vir in the order
// xx xy xz yy yz zz, stored as xx yy zz xy xz yz.  Only when requested.
__device__ __forceinline__ void tally_atoms(const BatchView& B, const int* ghosts, int n, double e, const double* vir) {
    if (!B.eatom && !B.vatom) return;
    const double w = 1.0 / n;
    for (int k = 0; k < n; k++) {
        const long long o = B.atom_orig[B.ghost_parent[ghosts[k]]];
        if (B.eatom) atomicAdd(&B.eatom[o], e * w);
        if (B.vatom) {
            double* v = &B.vatom[6 * o];
            atomicAdd(&v[0], vir[0] * w);
            atomicAdd(&v[1], vir[3] * w);
            atomicAdd(&v[2], vir[5] * w);
            atomicAdd(&v[3], vir[1] * w);
            atomicAdd(&v[4], vir[2] * w);
            atomicAdd(&v[5], vir[4] * w);
        }
    }
}

// Per-lane energy/virial accumulator for one system at a time.
struct EVAcc {
    int s = -1;
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    __device__ void flush(const BatchView& B) {
        if (s >= 0)
            for (int k = 0; k < 7; k++) atomicAdd(&B.ev[8 * s + k], v[k]);
        s = -1;
        for (int k = 0; k < 7; k++) v[k] = 0;
    }
    __device__ void add(const BatchView& B, int sys, double e, const double* vir) {
        if (sys != s) { flush(B); s = sys; }
        v[0] += e;
        for (int k = 0; k < 6; k++) v[1 + k] += vir[k];
    }
    // Warp-collective (all 32 lanes call it): one interaction's energy and
    // virial per lane (valid lanes), summed over the warp first when every
    // valid lane's interaction belongs to one system, so that one lane's
    // accumulator takes the sum (atomics only when that lane changes system);
    // otherwise each valid lane adds its own.  Keeps batches of many systems
    // from turning every interaction into seven atomics on a few addresses.
    __device__ void add_warp(const BatchView& B, int sys, double e, const double* vir, bool valid) {
        const int lane = threadIdx.x & 31;
        const unsigned have = __ballot_sync(kFull, valid);
        if (!have) return;
        const int s0 = __shfl_sync(kFull, sys, __ffs(have) - 1);
        if (__all_sync(kFull, !valid || sys == s0)) {
            double x[7];
            x[0] = valid ? e : 0.0;
            for (int k = 0; k < 6; k++) x[1 + k] = valid ? vir[k] : 0.0;
            for (int k = 0; k < 7; k++)
                for (int off = 16; off; off >>= 1) x[k] += __shfl_xor_sync(kFull, x[k], off);
            if (lane == 0) add(B, s0, x[0], x + 1);
        } else if (valid) {
            add(B, sys, e, vir);
        }
    }
    // end of kernel: one set of atomics per warp when the warp holds one system
    __device__ void flush_warp(const BatchView& B) {
        const int lane = threadIdx.x & 31;
        int key = s;
        int s0 = -1;
        for (int l = 0; l < 32; l++) {
            int t = __shfl_sync(kFull, key, l);
            if (t >= 0) { s0 = t; break; }
        }
        const bool uniform = __all_sync(kFull, s < 0 || s == s0);
        if (uniform) {
            for (int k = 0; k < 7; k++) {
                double x = v[k];
                for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(kFull, x, off);
                v[k] = x;
            }
            if (lane == 0 && s0 >= 0)
                for (int k = 0; k < 7; k++) atomicAdd(&B.ev[8 * s0 + k], v[k]);
        } else {
            flush(B);
        }
    }
};

__device__ __forceinline__ void virial_add(double* vir, double f, const double* d) {
    vir[0] -= f * d[0] * d[0];
    vir[1] -= f * d[0] * d[1];
    vir[2] -= f * d[0] * d[2];
    vir[3] -= f * d[1] * d[1];
    vir[4] -= f * d[1] * d[2];
    vir[5] -= f * d[2] * d[2];
}

// compute_2B (chimesFF.cpp:1644-1775) of one pair below its outer cutoff:
// energy E (Chebyshev sum with T_{pow+1}, cutoff, penalty) and the force
// scalar fs (F_i += fs dr, F_j -= fs dr, virial -= fs dr (x) dr).  flags:
// device diagnostics (badness max, penalty hits, below-rin count).
template <typename CT>
__device__ __forceinline__ void pair_2b(const DevParamSet& P, const PairRec& pr, double dist, int* flags, double& E,
                                        double& fs) {
    // the Morse map with the pair type's reciprocals (no FP64 divisions:
    // GB300 issues FP64 at a small fraction of the FP32 rate, and a division
    // is several FP64 instructions)
    const bool oor = dist < pr.rin;
    const double rr = oor ? pr.rin : dist;
    const double ex = exp(-rr * pr.inv_lam);
    const double xd = (ex - pr.xavg) * pr.inv_xdiff;
    const double dxdr = -ex * pr.inv_lam * pr.inv_xdiff;
    const CT* a = coef2<CT>(P) + pr.coef_off;   // dense a_n, n = 0..o2
    const CT x = CT(xd), tx = CT(2) * x;
    CT t0c = CT(1), t1c = x, u0 = CT(1), u1 = tx;
    CT S = a[0] * t0c + a[1] * t1c;
    CT GD = a[1] * u0;                     // sum a_n n U_{n-1}
    for (int n = 2; n <= P.o2; n++) {
        const CT t2 = tx * t1c - t0c;
        const CT u2 = tx * u1 - u0;
        S += a[n] * t2;
        GD += a[n] * CT(n) * u1;
        t0c = t1c; t1c = t2; u0 = u1; u1 = u2;
    }
    double Sd = double(S), Gd = double(GD) * dxdr;
    if (oor) {
        atomicAdd(&flags[4], 1);
        const double damp = exp((dist - pr.rin) / P.inner_smooth);
        Sd += P.inner_smooth * (damp - 1.0) * Gd;
        Gd *= damp;
    }
    double fc, fcd;
    if (!P.tersoff) {
        const double f0 = 1.0 - dist * pr.fc_inv;
        fc = f0 * f0 * f0;
        fcd = f0 * f0 * (-3.0 * pr.fc_inv);
    } else if (dist < pr.fc_th) {
        fc = 1.0;
        fcd = 0.0;
    } else if (dist > pr.rout) {
        fc = 0.0;
        fcd = 0.0;
    } else {
        const double f0 = (dist - pr.fc_th) * pr.fc_inv * kPi + kPi / 2.0;
        double sn, cs;
        sincos(f0, &sn, &cs);
        fc = 0.5 + 0.5 * sn;
        fcd = 0.5 * cs * (kPi * pr.fc_inv);
    }
    E = fc * Sd;
    const double dx_inv = dist > 0.0 ? 1.0 / dist : 1e20;
    fs = (fc * Gd + fcd * Sd) * dx_inv;
    // get_penalty (chimesFF.h:388-419)
    if (dist - P.pen_dist < pr.rin) {
        const double rp = pr.rin + P.pen_dist - dist;
        atomicMax(&flags[2], dist < pr.rin ? 2 : 1);
        if (rp > 0.0) {
            atomicAdd(&flags[3], 1);
            E += rp * rp * rp * P.pen_scale;
            fs += (-3.0 * rp * rp * P.pen_scale) / dist;
        }
    }
}

// Forces, virial and energy of one 3- or 4-body cluster from its contraction
// sums (compute_3B/4B, chimesFF.cpp:2068-2169 and the 4-body counterpart):
//   f_p = (prod_{q!=p} fc_q / r_p) (fc_p G_p + fc'_p S),  E = prod fc * S.
template <int NB>
__device__ __forceinline__ void cluster_epilogue(const BatchView& B, const int* id, int sys,
                                                 const double (*dr)[4], const double* fc, const double* fcd,
                                                 double S, const double* G, EVAcc& acc) {
    constexpr int NP = Topo<NB>::NP;
    double pre[NP + 1], suf[NP + 1];
    pre[0] = 1.0;
    for (int p = 0; p < NP; p++) pre[p + 1] = pre[p] * fc[p];
    suf[NP] = 1.0;
    for (int p = NP - 1; p >= 0; p--) suf[p] = suf[p + 1] * fc[p];
    double f[NB][3];
    for (int k = 0; k < NB; k++) f[k][0] = f[k][1] = f[k][2] = 0.0;
    double vir[6] = {0, 0, 0, 0, 0, 0};
    for (int p = 0; p < NP; p++) {
        const double fsp = pre[p] * suf[p + 1] / dr[p][3] * (fc[p] * G[p] + fcd[p] * S);
        const int a = Topo<NB>::a(p), b = Topo<NB>::b(p);
        for (int k = 0; k < 3; k++) {
            f[a][k] += fsp * dr[p][k];
            f[b][k] -= fsp * dr[p][k];
        }
        virial_add(vir, fsp, dr[p]);
    }
    for (int k = 0; k < NB; k++) add_force(B, id[k], f[k][0], f[k][1], f[k][2]);
    acc.add(B, sys, pre[NP] * S, vir);
    tally_atoms(B, id, NB, pre[NP] * S, vir);
}

// The same for the mixed form, in FP32: the cluster's force scalars, forces
// and virial derive from the FP32 contraction sums, so they are formed in
// FP32 (GB300's FP64 pipe issues one warp instruction per 16 cycles per SM,
// and this epilogue was most of a mixed cluster kernel's FP64 work); the
// per-atom forces (FP64 atomics) and the system's energy and virial (FP64)
// are accumulated in FP64.  dr: the pairs' vectors, rinv: 1 / distance.
// The cluster's energy and virial are returned for the caller's (warp-wide)
// accumulation.
template <int NB>
__device__ __forceinline__ void cluster_epilogue_f32(const BatchView& B, const int* id, const float (*dr)[3],
                                                     const float* rinv, const float* fc, const float* fcd, float S,
                                                     const float* G, double& e_out, double* vir_out) {
    constexpr int NP = Topo<NB>::NP;
    float pre[NP + 1], suf[NP + 1];
    pre[0] = 1.0f;
#pragma unroll
    for (int p = 0; p < NP; p++) pre[p + 1] = pre[p] * fc[p];
    suf[NP] = 1.0f;
#pragma unroll
    for (int p = NP - 1; p >= 0; p--) suf[p] = suf[p + 1] * fc[p];
    float f[NB][3];
#pragma unroll
    for (int k = 0; k < NB; k++) f[k][0] = f[k][1] = f[k][2] = 0.0f;
    float v[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int p = 0; p < NP; p++) {
        const float fsp = pre[p] * suf[p + 1] * rinv[p] * (fc[p] * G[p] + fcd[p] * S);
        const int a = Topo<NB>::a(p), b = Topo<NB>::b(p);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            f[a][k] += fsp * dr[p][k];
            f[b][k] -= fsp * dr[p][k];
        }
        v[0] -= fsp * dr[p][0] * dr[p][0];
        v[1] -= fsp * dr[p][0] * dr[p][1];
        v[2] -= fsp * dr[p][0] * dr[p][2];
        v[3] -= fsp * dr[p][1] * dr[p][1];
        v[4] -= fsp * dr[p][1] * dr[p][2];
        v[5] -= fsp * dr[p][2] * dr[p][2];
    }
#pragma unroll
    for (int k = 0; k < NB; k++) add_force(B, id[k], double(f[k][0]), double(f[k][1]), double(f[k][2]));
    for (int k = 0; k < 6; k++) vir_out[k] = double(v[k]);
    e_out = double(pre[NP] * S);
    tally_atoms(B, id, NB, e_out, vir_out);
}

}  // namespace
}  // namespace ck
