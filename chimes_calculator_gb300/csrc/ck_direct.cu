// Per-cluster kernels: the chimesFF::compute_2B/3B/4B entry points, where the
// caller owns the cluster loop and passes distances, displacement vectors and
// type indices (chimesFF/src/chimesFF.cpp:1644-1775, 1931-2176, 2496-2872).
// One thread (3-/4-body: one or more lanes) per cluster, FP64, any number of
// clusters per launch; outputs are per-cluster (the host adds them into the
// caller's accumulators).
//
// Besides energy, forces and the packed stress, each cluster reports the
// reference's `force_scalar_in` value: for 2B the penalty force scalar over r
// (1.0 without a penalty), for 3B/4B the per-pair force scalars of the LAST
// coefficient of the list, as the reference's loop leaves them.  status bits:
// 1 = the cluster passed the type and cutoff checks, 2 = penalty region
// (badness 1), 4 = below the inner cutoff (badness 2), 8 = a many-body pair below
// its inner cutoff (the reference prints a warning; badness is unchanged),
// 16 = a tabulated term's distance outside its table (the reference exits or
// reads past its table there).
#include <cuda_runtime.h>

#include "ck_common.h"
#include "ck_kernels.h"
#include "ck_math.cuh"
#include "ck_tab.cuh"

namespace ck {

cudaError_t allow_max_smem(const void* kernel);   // ck_force.cu

namespace {

__global__ void k_direct2(const DevParamSet* Pp, int n, const double* dx, const double* dr, const int* typ,
                          double* force, double* stress, double* energy, double* fscal, int* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const DevParamSet& P = *Pp;
    for (int k = 0; k < 6; k++) { force[6 * c + k] = 0.0; stress[6 * c + k] = 0.0; }
    energy[c] = 0.0;
    fscal[c] = 0.0;
    status[c] = 0;
    const int t0 = typ[2 * c], t1 = typ[2 * c + 1];
    const PairRec pr = P.pairs[P.pair_map[t0 * P.ntypes + t1]];
    const double r = dx[c];
    const double* d = &dr[3 * c];
    if (r >= pr.rout) return;
    int st = 1;
    double xd, dxdr;
    bool oor;
    morse_x(r, pr.rin, pr.lam, pr.xavg, pr.xdiff, xd, dxdr, oor);
    const double* a = P.c2d + pr.coef_off;
    const double tx = 2.0 * xd;
    double t0c = 1.0, t1c = xd, u0 = 1.0, u1 = tx;
    double S = a[0] * t0c + a[1] * t1c, GD = a[1] * u0;
    for (int k = 2; k <= P.o2; k++) {
        const double t2 = tx * t1c - t0c, u2 = tx * u1 - u0;
        S += a[k] * t2;
        GD += a[k] * k * u1;
        t0c = t1c; t1c = t2; u0 = u1; u1 = u2;
    }
    double G = GD * dxdr;
    if (oor) {
        const double damp = exp((r - pr.rin) / P.inner_smooth);
        S += P.inner_smooth * (damp - 1.0) * G;
        G *= damp;
    }
    double fc, fcd;
    fcut_eval<double>(P, r, pr.rout, fc, fcd);
    double E = fc * S;
    const double dx_inv = r > 0.0 ? 1.0 / r : 1e20;
    double fs = (fc * G + fcd * S) * dx_inv;
    double fs_out = 1.0;
    if (r - P.pen_dist < pr.rin) {
        st |= r < pr.rin ? 4 : 2;
        const double rp = pr.rin + P.pen_dist - r;
        if (rp > 0.0) {
            E += rp * rp * rp * P.pen_scale;
            fs_out = (-3.0 * rp * rp * P.pen_scale) / r;
            fs += fs_out;
        }
    }
    for (int k = 0; k < 3; k++) {
        force[6 * c + k] = fs * d[k];
        force[6 * c + 3 + k] = -fs * d[k];
    }
    stress[6 * c + 0] = -fs * d[0] * d[0];
    stress[6 * c + 1] = -fs * d[0] * d[1];
    stress[6 * c + 2] = -fs * d[0] * d[2];
    stress[6 * c + 3] = -fs * d[1] * d[1];
    stress[6 * c + 4] = -fs * d[1] * d[2];
    stress[6 * c + 5] = -fs * d[2] * d[2];
    energy[c] = E;
    fscal[c] = fs_out;
    status[c] = st;
}

// TPC lanes per cluster (a power of two up to 32): the lanes of a cluster
// fill its Chebyshev tables and cutoffs in shared memory (pair p by lane
// p mod TPC), each lane sums every TPC-th coefficient, the group reduces S and
// G with shuffles, and the lane holding the list's last coefficient supplies
// force_scalar_in.  With few clusters (a 4-body batch of a few thousand) one
// lane per cluster leaves most SMs idle; the launcher picks TPC from the
// cluster count.  One-warp blocks; shared memory per cluster
// NP * (2 * (order + 1) + 2) doubles.
template <int NB, int TPC>
__global__ void __launch_bounds__(32) k_directn(const DevParamSet* Pp, int n, const double* dx, const double* dr,
                                                const int* typ, double* force, double* stress, double* energy,
                                                double* fscal, int* status) {
    constexpr int NP = Topo<NB>::NP;
    constexpr unsigned kAll = 0xffffffffu;
    extern __shared__ __align__(16) double dsm[];
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = (int)(tid / TPC), gl = (int)(tid % TPC);
    const DevParamSet& P = *Pp;
    const int order = NB == 3 ? P.o3 : P.o4;
    const int op1 = order + 1;
    // this cluster's tables: T[p][0..order], D[p][0..order], then fc[p], fcd[p]
    double* tab = dsm + (long long)(threadIdx.x / TPC) * NP * (2 * op1 + 2);
    double* fcs = tab + 2 * NP * op1;
    double* fcds = fcs + NP;
    bool active = c < n;   // group-uniform; every lane reaches the syncs and shuffles below
    if (active && gl == 0) {
        for (int k = 0; k < 3 * NB; k++) force[3 * NB * c + k] = 0.0;
        for (int k = 0; k < 6; k++) stress[6 * c + k] = 0.0;
        for (int k = 0; k < NP; k++) fscal[NP * c + k] = 0.0;
        energy[c] = 0.0;
        status[c] = 0;
    }
    const TupleRec* R = nullptr;
    const double* r = nullptr;
    if (active) {
        int u = 0;
        for (int k = 0; k < NB; k++) u = u * P.ntypes + typ[NB * c + k];
        R = (NB == 3 ? P.t3 : P.t4) + u;
        r = &dx[NP * c];
        if (R->type_id < 0) active = false;   // excluded cluster type
        else
            for (int p = 0; p < NP; p++)
                if (r[p] >= R->rout[p]) active = false;
    }
    if (active)
        for (int p = gl; p < NP; p += TPC) {
            cheby_table<double>(tab + 2 * p * op1, tab + (2 * p + 1) * op1, r[p], R->rin[p], R->lam[p], R->xavg[p],
                                R->xdiff[p], order, P.inner_smooth, nullptr);
            fcut_eval<double>(P, r[p], R->rout[p], fcs[p], fcds[p]);
        }
    __syncwarp();
    double S = 0.0, G[NP], last[NP], pre[NP + 1], suf[NP + 1];
    for (int p = 0; p < NP; p++) G[p] = last[p] = 0.0;
    pre[NP] = 0.0;
    int st = 1;
    if (active) {
        for (int p = 0; p < NP; p++)
            if (r[p] < R->rin[p]) st |= 8;   // below-rin warning only (badness is a 2B notion)
        pre[0] = 1.0;
        for (int p = 0; p < NP; p++) pre[p + 1] = pre[p] * fcs[p];
        suf[NP] = 1.0;
        for (int p = NP - 1; p >= 0; p--) suf[p] = suf[p + 1] * fcs[p];
        const double* cf = (NB == 3 ? P.c3d : P.c4d) + R->coef_off;
        const uint32_t* pw = (NB == 3 ? P.p3 : P.p4) + R->coef_off;
        const int kl = R->ncoef - 1;
        for (int k = gl; k < R->ncoef; k += TPC) {
            double t[NP], dd[NP];
            for (int p = 0; p < NP; p++) {
                const int q = (pw[k] >> (kPowBits * p)) & 31u;
                t[p] = tab[2 * p * op1 + q];
                dd[p] = tab[(2 * p + 1) * op1 + q];
            }
            double tp[NP + 1], ts[NP + 1];
            tp[0] = 1.0;
            for (int p = 0; p < NP; p++) tp[p + 1] = tp[p] * t[p];
            ts[NP] = 1.0;
            for (int p = NP - 1; p >= 0; p--) ts[p] = ts[p + 1] * t[p];
            S += cf[k] * tp[NP];
            for (int p = 0; p < NP; p++) G[p] += cf[k] * dd[p] * tp[p] * ts[p + 1];
            if (k == kl)
                for (int p = 0; p < NP; p++)
                    last[p] = cf[k] * (fcs[p] * dd[p] + fcds[p] * t[p]) * (pre[p] * suf[p + 1] / r[p]) * tp[p] *
                              ts[p + 1];
        }
    }
    // combine the group's partial sums; the last coefficient's lane holds
    // force_scalar_in, the others hold zeros
#pragma unroll
    for (int off = TPC / 2; off > 0; off >>= 1) {
        S += __shfl_xor_sync(kAll, S, off);
#pragma unroll
        for (int p = 0; p < NP; p++) {
            G[p] += __shfl_xor_sync(kAll, G[p], off);
            last[p] += __shfl_xor_sync(kAll, last[p], off);
        }
    }
    if (!active || gl != 0) return;
    const double* d = &dr[3 * NP * c];
    double vir[6] = {0, 0, 0, 0, 0, 0};
    for (int p = 0; p < NP; p++) {
        const double fsp = pre[p] * suf[p + 1] / r[p] * (fcs[p] * G[p] + fcds[p] * S);
        const double* dp = &d[3 * p];
        const int a = Topo<NB>::a(p), b = Topo<NB>::b(p);
        for (int k = 0; k < 3; k++) {
            force[3 * NB * c + 3 * a + k] += fsp * dp[k];
            force[3 * NB * c + 3 * b + k] -= fsp * dp[k];
        }
        vir[0] -= fsp * dp[0] * dp[0];
        vir[1] -= fsp * dp[0] * dp[1];
        vir[2] -= fsp * dp[0] * dp[2];
        vir[3] -= fsp * dp[1] * dp[1];
        vir[4] -= fsp * dp[1] * dp[2];
        vir[5] -= fsp * dp[2] * dp[2];
    }
    for (int k = 0; k < 6; k++) stress[6 * c + k] = vir[k];
    for (int p = 0; p < NP; p++) fscal[NP * c + p] = last[p];
    energy[c] = pre[NP] * S;
    status[c] = st;
}

template <int NB>
void launch_directn(const DevParamSet* Pd, int order, int n, const double* dx, const double* dr, const int* typ,
                    double* force, double* stress, double* energy, double* fscal, int* status, cudaStream_t st) {
    constexpr int NP = Topo<NB>::NP;
    // lanes per cluster: enough threads for about 16 warps on each of ~152 SMs
    const long long want = 152LL * 16 * 32 / (n > 0 ? n : 1);
    int tpc = 1;
    while (tpc < 32 && 2LL * tpc <= want) tpc *= 2;
    const unsigned grid = (unsigned)(((long long)n * tpc + 31) / 32);
    const size_t smem = sizeof(double) * (size_t)(32 / tpc) * NP * (2 * (order + 1) + 2);
#define CK_DIRECTN(T_)                                                                                    \
    do {                                                                                                  \
        auto kern = k_directn<NB, T_>;                                                                    \
        if (smem > 48 * 1024) allow_max_smem((const void*)kern);                                          \
        count_launch(), kern<<<grid, 32, smem, st>>>(Pd, n, dx, dr, typ, force, stress, energy, fscal, status); \
    } while (0)
    switch (tpc) {
        case 1: CK_DIRECTN(1); break;
        case 2: CK_DIRECTN(2); break;
        case 4: CK_DIRECTN(4); break;
        case 8: CK_DIRECTN(8); break;
        case 16: CK_DIRECTN(16); break;
        default: CK_DIRECTN(32); break;
    }
#undef CK_DIRECTN
}

// compute_2B_tab (chimesFF.cpp:1782-1867): table energy and force scalar;
// force_scalar_in is get_penalty's value (1.0, or the penalty slope inside the
// penalty region), which overwrites the table's scalar at the end.
__global__ void k_direct2tab(const DevParamSet* Pp, int n, const double* dx, const double* dr, const int* typ,
                             double* force, double* stress, double* energy, double* fscal, int* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const DevParamSet& P = *Pp;
    for (int k = 0; k < 6; k++) { force[6 * c + k] = 0.0; stress[6 * c + k] = 0.0; }
    energy[c] = 0.0;
    fscal[c] = 0.0;
    status[c] = 0;
    const int pt = P.pair_map[typ[2 * c] * P.ntypes + typ[2 * c + 1]];
    const PairRec pr = P.pairs[pt];
    const double r = dx[c];
    const double* d = &dr[3 * c];
    if (r >= pr.rout) return;
    int st = 1;
    double E, fs;
    if (tab2_lookup(P, pt, r, E, fs) != kTabOk) st |= 16;
    for (int k = 0; k < 3; k++) {
        force[6 * c + k] = __dmul_rn(fs, d[k]);
        force[6 * c + 3 + k] = __dsub_rn(0.0, __dmul_rn(fs, d[k]));
    }
    stress[6 * c + 0] = __dsub_rn(0.0, __dmul_rn(__dmul_rn(fs, d[0]), d[0]));
    stress[6 * c + 1] = __dsub_rn(0.0, __dmul_rn(__dmul_rn(fs, d[0]), d[1]));
    stress[6 * c + 2] = __dsub_rn(0.0, __dmul_rn(__dmul_rn(fs, d[0]), d[2]));
    stress[6 * c + 3] = __dsub_rn(0.0, __dmul_rn(__dmul_rn(fs, d[1]), d[1]));
    stress[6 * c + 4] = __dsub_rn(0.0, __dmul_rn(__dmul_rn(fs, d[1]), d[2]));
    stress[6 * c + 5] = __dsub_rn(0.0, __dmul_rn(__dmul_rn(fs, d[2]), d[2]));
    double fs_out = 1.0;
    if (r - P.pen_dist < pr.rin) {
        st |= r < pr.rin ? 4 : 2;
        const double rp = pr.rin + P.pen_dist - r;
        if (rp > 0.0) fs_out = __dmul_rn(__dmul_rn(__dmul_rn(-3.0, rp), rp), P.pen_scale);
    }
    energy[c] = E;
    fscal[c] = fs_out;
    status[c] = st;
}

// compute_3B_tab (chimesFF.cpp:2183-2322): the type and per-pair outer-cutoff
// checks of compute_3B, then the tricubic look-up; force_scalar_in receives the
// three table force scalars.
__global__ void k_direct3tab(const DevParamSet* Pp, int n, const double* dx, const double* dr, const int* typ,
                             double* force, double* stress, double* energy, double* fscal, int* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const DevParamSet& P = *Pp;
    for (int k = 0; k < 9; k++) force[9 * c + k] = 0.0;
    for (int k = 0; k < 6; k++) stress[6 * c + k] = 0.0;
    for (int k = 0; k < 3; k++) fscal[3 * c + k] = 0.0;
    energy[c] = 0.0;
    status[c] = 0;
    const int u = (typ[3 * c] * P.ntypes + typ[3 * c + 1]) * P.ntypes + typ[3 * c + 2];
    const TupleRec& R = P.t3[u];
    if (R.type_id < 0) return;
    const double* r = &dx[3 * c];
    for (int p = 0; p < 3; p++)
        if (r[p] >= R.rout[p]) return;
    double v[4];
    int st = 1;
    if (tab3_lookup(P, R.type_id, r[0], r[1], r[2], v) != kTabOk) st |= 16;
    double f[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vir[6] = {0, 0, 0, 0, 0, 0};
    for (int p = 0; p < 3; p++) {
        const double fsp = v[1 + p];
        const double* d = &dr[9 * c + 3 * p];
        const int a = Topo<3>::a(p), b = Topo<3>::b(p);
        for (int k = 0; k < 3; k++) {
            f[3 * a + k] = __dadd_rn(f[3 * a + k], __dmul_rn(fsp, d[k]));
            f[3 * b + k] = __dsub_rn(f[3 * b + k], __dmul_rn(fsp, d[k]));
        }
        vir[0] = __dsub_rn(vir[0], __dmul_rn(fsp, __dmul_rn(d[0], d[0])));
        vir[1] = __dsub_rn(vir[1], __dmul_rn(fsp, __dmul_rn(d[0], d[1])));
        vir[2] = __dsub_rn(vir[2], __dmul_rn(fsp, __dmul_rn(d[0], d[2])));
        vir[3] = __dsub_rn(vir[3], __dmul_rn(fsp, __dmul_rn(d[1], d[1])));
        vir[4] = __dsub_rn(vir[4], __dmul_rn(fsp, __dmul_rn(d[1], d[2])));
        vir[5] = __dsub_rn(vir[5], __dmul_rn(fsp, __dmul_rn(d[2], d[2])));
    }
    for (int k = 0; k < 9; k++) force[9 * c + k] = f[k];
    for (int k = 0; k < 6; k++) stress[6 * c + k] = vir[k];
    for (int k = 0; k < 3; k++) fscal[3 * c + k] = v[1 + k];
    energy[c] = v[0];
    status[c] = st;
}

}  // namespace

void launch_direct(const DevParamSet* P, int nbody, int order, int n, const double* dx, const double* dr,
                   const int* typ, double* force, double* stress, double* energy, double* fscal, int* status,
                   cudaStream_t st, bool tab) {
    if (n <= 0) return;
    const unsigned grid = (unsigned)((n + 63) / 64);
    if (tab) {
        if (nbody == 2) count_launch(), k_direct2tab<<<grid, 64, 0, st>>>(P, n, dx, dr, typ, force, stress, energy, fscal, status);
        else count_launch(), k_direct3tab<<<grid, 64, 0, st>>>(P, n, dx, dr, typ, force, stress, energy, fscal, status);
        return;
    }
    if (nbody == 2) count_launch(), k_direct2<<<grid, 64, 0, st>>>(P, n, dx, dr, typ, force, stress, energy, fscal, status);
    else if (nbody == 3) launch_directn<3>(P, order, n, dx, dr, typ, force, stress, energy, fscal, status, st);
    else launch_directn<4>(P, order, n, dx, dr, typ, force, stress, energy, fscal, status, st);
}

}  // namespace ck
