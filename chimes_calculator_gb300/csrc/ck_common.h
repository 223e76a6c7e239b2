// Shared host/device data layout of the GB300 ChIMES force path.
//
// Everything the kernels read lives in two kinds of device buffers:
//   * one parameter-set image per loaded parameter file (DevParamSet and the
//     arrays it points to), built once by read_parameters;
//   * one batch workspace per instance (BatchView), holding every system of a
//     batch back to back: caller atoms, replicated atoms, ghost images, bins,
//     the 2B neighbour lists, the 3B/4B cluster lists and the accumulators.
//
// Index spaces (all int32 inside a batch; offsets are int64):
//   caller atom  c   : 0 .. sum(n_in)         positions/forces as the caller passed them
//   atom         a   : 0 .. sum(n_atoms)      after replication (small=true), wrapped
//   ghost slot   q   : 0 .. sum(n_atoms*gstride); atom a of a system owns the slots
//                      ghost_off + a*gstride + [0, gstride) and fills them with its
//                      images that can lie within the search radius of the primary
//                      cell (the atom itself included); unused slots carry id -1.
//   ghost id         : the reference's numbering of a system's ghost atoms,
//                      img*n_atoms + a, img 0 the primary cell and img>=1 walking
//                      (i,j,k) in [-n,n]^3\{0} with i slowest
//                      (simulation_system::build_layered_system,
//                      serial_interface/src/serial_chimes_interface.cpp:546-585).
//                      Images farther than the search radius from every atom of the
//                      cell never enter a list, so only the kept ones get slots;
//                      bins, lists and clusters hold slots and order them by id.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define CK_HD __host__ __device__
#else
#define CK_HD
#endif

namespace ck {

constexpr int kMaxOrder = 31;      // powers are packed 5 bits per pair
constexpr int kMaxTypes = 8;       // nt^4 4-body tuple records
constexpr int kPowBits = 5;

enum Status : int {
    kOk = 0,
    kErrParam = -1,       // malformed / unsupported parameter file
    kErrInput = -2,       // bad caller input (unknown atom type, sizes)
    kErrGeometry = -3,    // cutoff larger than half the layered box, bad bins
    kErrCuda = -4,        // CUDA runtime error
    kErrCapacity = -5,    // a device capacity was exceeded (internal; retried)
    kErrState = -6,       // call order (e.g. calculate before init)
    kErrTimeout = -7,     // a bounded device wait expired
};

// One 2-body pair type (chimes_2b_cutoff / morse_var, chimesFF.h:290-295).
struct PairRec {
    double rin, rout, lam;
    double xavg, xdiff;    // Morse-map constants 0.5*(xmax+xmin), -0.5*(xmax-xmin)
    int ncoef;             // = 2B order
    int coef_off;          // offset into c2d/c2f/p2
    // reciprocals for the 2-body kernels (as TupleRec): 1/lam, 1/xdiff, and the
    // cutoff's 1/rc (cubic) or Tersoff threshold rc - f*rc and 1/(rc - threshold)
    double inv_lam, inv_xdiff, fc_th, fc_inv;
};

// One ordered atom-type tuple of a 3- or 4-body cluster.  Cutoffs, lambdas and
// the packed powers are already permuted into the cluster's own pair order
// (ij,ik,jk / ij,ik,il,jk,jl,kl) by the tuple's pair_int_{trip,quad}_map entry.
struct TupleRec {
    int valid;             // atom_int_{trip,quad}_map >= 0 and the type has coefficients
    int ncoef;
    int coef_off;          // offset into the body's coefficient arrays
    int type_id;           // tripidx / quadidx (for diagnostics)
    // factored form (see FactRow): rows at fr[f_row .. f_row+f_nrow), columns
    // right after them (f_ncol); row entries at [f_ent, f_ent+ncoef), column
    // entries at [f_ent+ncoef, f_ent+2*ncoef)
    int f_row, f_nrow, f_ncol, f_ent;
    // tensor-core form: offset of the tuple's coefficient matrix images in
    // DevParamSet::tc3 (3-body tuples) or tc4 (4-body tuples), in floats; -1
    // when absent
    int tc_off, tc_pad;
    double rin[6], rout[6], lam[6], xavg[6], xdiff[6];
    // reciprocals for the factored kernels: 1/lam, 1/xdiff, and the cutoff's
    // 1/rc (cubic) or Tersoff threshold rc - f*rc and 1/(rc - threshold)
    double inv_lam[6], inv_xdiff[6], fc_th[6], fc_inv[6];
    float rout_f[6];       // rout rounded to FP32 (FP32 cutoff tests add a margin for the rounding)
};

// Factored coefficient lists of one tuple.  The cluster's pairs split into
// row pairs (the first K: K = 1 for 3-body, 3 for 4-body) and column pairs
// (the rest); with R powers per pair (0..R-1), a coefficient with powers
// (q_0..q_{P-1}) sits at row I = sum_{p<K} q_p R^{K-1-p} and column
// J = sum_{p>=K} q_p R^{P-1-p}, so that
//   E-sum S = sum_I X_I sum_J a_IJ Y_J,   X_I = prod_{p<K} T_p[q_p],  Y_J = prod_{p>=K} T_p[q_p].
// Row entries (sorted by I, then J) hold (a, J); column entries (sorted by J,
// then I) hold (a, I).  A record gives the row's powers (or the column's),
// packed kPowBits per pair from the first pair of its side up, and the end of
// its entries; each starts where the previous one ended.
struct FactRow {
    int pows;
    int end;
};
constexpr int kFactMaxDim = 128;   // largest R^K and R^(P-K) kept in shared memory per cluster

// Tensor-core 3-body images (DevParamSet::tc3): with Rw powers per pair the
// MMA's K is Rw padded to 8 or 16 and N = Rw^2 padded to 16; a tuple stores
// one image per Rw from its own R up to kTc3MaxR, consecutively, so the image
// for Rw starts tc3_offset floats in.  An image holds kTc3Parts TF32 parts of
// each coefficient (high, middle, low: each the TF32 rounding of what the
// previous parts leave), one after another.
constexpr int kTc3MaxR = 11;
constexpr int kTc3Parts = 3;
CK_HD constexpr int tc3_kpad(int Rw) { return Rw <= 8 ? 8 : 16; }
CK_HD constexpr int tc3_npad(int Rw) { return ((Rw * Rw + 15) / 16) * 16; }
// Tensor-core 4-body images (DevParamSet::tc4): with R powers per pair the
// rows I = (q_ij, q_ik, q_il) and columns J = (q_jk, q_jl, q_kl) number
// n3 = R^3 each; K = n3 padded to 8, N = n3 padded to 16 (shared memory keeps
// R <= kTc4MaxR); one image per tuple at the set's own R, kTc3Parts parts.
constexpr int kTc4MaxR = 4;
CK_HD constexpr int tc4_kpad(int n3) { return (n3 + 7) / 8 * 8; }
CK_HD constexpr int tc4_npad(int n3) { return (n3 + 15) / 16 * 16; }
CK_HD inline long long tc3_offset(int R, int Rw) {
    long long o = 0;
    for (int r = R; r < Rw; r++) o += (long long)kTc3Parts * tc3_kpad(r) * tc3_npad(r);
    return o;
}

// Per-pair-type constants of a body order's Chebyshev stage, when every tuple
// uses the same inner/outer cutoff for a given pair type (then a pair's
// tables depend only on its distance and type and can be computed once per
// neighbour-list entry instead of once per cluster).
struct PairTab {
    double rin, rout, xavg, xdiff, inv_lam, inv_xdiff, fc_th, fc_inv;
};

// One factored-list entry: coefficient and the other side's record, in one
// 16-byte (FP64) or 8-byte (FP32) load.  idx = linear index (bits 0-15) |
// the other side's powers packed kPowBits per pair (bits 16-30) | bit 31 set on
// the last entry of its record (idx < 0).
struct __attribute__((aligned(16))) FactEntD {
    double a;
    int idx;
    int pad;
};
struct __attribute__((aligned(8))) FactEntF {
    float a;
    int idx;
};

// Tabulated 2-body term of one pair type (TABULATION build of the reference:
// read_2B_tab and get_tab_2B, chimesFF/src/chimesFF.cpp:199-255, 1869-1922).
// Grid r[0..n) ascending at tab2r[off..]; for every interval start i
// (1 <= i <= n-2) the local cubic a + b*dx + c*dx^2 + d*dx^3 of the energy and
// of the force scalar at tab2c[8*(off+i) ..] (E a,b,c,d then F a,b,c,d),
// computed on the host with get_tab_2B's arithmetic.
struct Tab2Rec {
    long long off;
    int n;
    int pad;
};

// Tabulated 3-body term of one triplet type (read_3B_tab, interpolateTricubic,
// chimesFF.cpp:257-351, 2370-2440): nrows rows of (rij, rik, rjk) with rij the
// slowest and rjk the fastest coordinate, columns at tab3r[3*off ..] (rij
// column, then rik, then rjk, nrows each) and values (E, F_ij, F_ik, F_jk) at
// tab3v[4*(off+row) ..].  size = (int)cbrt(nrows); inv = 1 / (grid step),
// computed as interpolateTricubic does.
struct Tab3Rec {
    long long off;
    long long nrows;
    int size;
    int pad;
    double inv;
};

struct DevParamSet {
    int ntypes, npairs, o2, o3, o4;
    int tersoff;
    double fcut_var, pen_dist, pen_scale, inner_smooth;
    double maxcut2, maxcut3, maxcut4, search;
    const double* eoff;        // [nt]
    const int* pair_map;       // [nt*nt]  atom_int_pair_map
    const PairRec* pairs;      // [npairs]
    const double* c2d; const float* c2f; const int* p2;
    const TupleRec* t3;        // [nt^3] (null when o3 == 0)
    const double* c3d; const float* c3f; const uint32_t* p3;
    const TupleRec* t4;        // [nt^4] (null when o4 == 0)
    const double* c4d; const float* c4f; const uint32_t* p4;
    // factored lists (FactRow); R3/R4 = powers per pair, 0 when the tables are
    // absent (R^K or R^(P-K) above kFactMaxDim)
    int R3, R4;
    int bk3, bk4;              // first cluster bucket of this set (per engine; see BatchView)
    // tensor-core 3-body contraction (mixed form): per tuple, the dense
    // coefficient matrix A[q_ij][q_ik*Rw + q_jk] as the B operand of a
    // tcgen05 TF32 MMA, one image per working width Rw >= R3 (see tc3_offset);
    // tc3_k, tc3_n = K and N at Rw = R3; null when R3 is 0 or above kTc3MaxR
    int tc3_k, tc3_n;
    const float* tc3;
    // tensor-core 4-body contraction (mixed form): per tuple, A[I][J] with
    // I = (q_ij, q_ik, q_il), J = (q_jk, q_jl, q_kl) as the B operand, at
    // tc4_r = R4 powers per pair; null when R4 is below 2 or above kTc4MaxR
    int tc4_r, tc4_pad;
    const float* tc4;
    // table lengths, for the index checks of the checked build (CK_BOUNDS):
    // 3-/4-body coefficients, factored entries, tensor-core image floats
    long long n_c3, n_c4, n_fe3, n_fe4, n_tc3, n_tc4;
    const FactRow* fr3; const FactEntD* fe3d; const FactEntF* fe3f;
    const FactRow* fr4; const FactEntD* fe4d; const FactEntF* fe4f;
    // per-pair-type tables [npairs] (null when some tuple's cutoffs differ by tuple)
    const PairTab* pt3; const PairTab* pt4;
    // tabulated terms: 2-body tables looked up by pair type index, 3-body
    // tables by triplet type index (the reference's tab_*[pair_idx / tripidx])
    int tab2, tab3;            // 1 when the 2B / 3B terms are tabulated
    int n_tab2, n_tab3;        // tables present
    const Tab2Rec* t2rec; const double* tab2r; const double* tab2c;
    const Tab3Rec* t3rec; const double* tab3r; const double* tab3v;
};

// Per-system geometry, written by the host set-up (cell algebra) and
// completed on the device (bin grid).
struct SysDesc {
    double h[9], hi[9];        // cell of the (replicated) system and inverse: r = h * s
    double hn[9], hni[9];      // reoriented cell used for the neighbour lists
    double h0[9], h0i[9];      // unreplicated cell (replication step)
    double search;             // max(rc2, rc3, rc4)
    double c3, c4;             // max 3B / 4B outer cutoffs (0 when the order is 0)
    int n_in;                  // caller atoms
    int n_rep;                 // n_replicates
    int n_atoms;               // replicated atoms = n_in * (n_rep+1)^3
    int n_layers, side;        // ghost layers and 2n+1
    int pset;                  // parameter set slot
    int has3, has4;
    long long in_off, atom_off, ghost_off, bin_off;
    int bin_cap;               // bins reserved for this system
    int gstride;               // ghost slots per atom (upper bound of its kept images, itself included)
    double ulo[3], uhi[3];     // kept fractional range per axis of the reoriented cell
    double eps;                // margin of the FP32 distance prefilter (Angstrom)
    float c3lo, c3hi, c4lo, c4hi;   // c3 -/+ eps and c4 -/+ eps as FP32, rounded outward
    float far2, near2;         // (search +/- eps)^2 as FP32: the pair lists' squared-distance prefilter
    float c3lo2, c3hi2, c4lo2, c4hi2;   // the same thresholds squared, rounded outward (-1: none below)
    // device-completed
    double minpos[3];
    int nb[3];
    int err;
};

// Flat views of a batch workspace (all device pointers).
struct BatchView {
    int n_sys;
    long long n_in_total, n_atoms_total, n_ghost_total, n_bins_total;
    SysDesc* sys;
    const DevParamSet* psets;      // device array of parameter sets (by slot)
    // caller atoms
    const double* in_pos;          // [n_in_total][3]
    const int* in_type;            // [n_in_total]
    // replicated atoms
    int* atom_sys;                 // [n_atoms_total]
    int* atom_type;
    int* atom_orig;                // caller-atom index receiving the force
    // ghost slots (an atom's own slot holds the atom itself)
    int* atom_self;                // [n_atoms_total] slot of the atom itself
    int* ghost_id;                 // [q] ghost id within its system, -1 = unused slot
    int* ghost_parent;             // [q] atom index (global)
    double* ghost_fs;              // [q][3] fractional coords, input cell
    double* ghost_xn;              // [q][3] Cartesian coords, reoriented cell
    double* ghost_fn;              // [q][3] fractional coords, reoriented cell
    float* ghost_xf;               // [q][3] ghost_xn rounded to FP32 (distance prefilter)
    // bins (per system, offset bin_off)
    unsigned long long* minmax;    // [n_sys][6] order-preserving keys
    int* ghost_bin;                // [g] local bin id
    int* bin_count;                // [n_bins_total]
    long long* bin_start;          // [n_bins_total+1] positions in bin_items (global exclusive scan)
    int* bin_fill;
    int* bin_items;                // [g] global ghost ids sorted by (bin, id)
    float* bin_xp;                 // [g][4] ghost_xf and ghost_parent (int bits) of bin_items, same order; or null
    // 2B lists
    int* l2_count;                 // [n_atoms_total]
    long long* l2_off;             // [n_atoms_total+1]
    int* l2_ghost;                 // [n2] ghost slot of the neighbour
    double* l2_dist;               // [n2] distance in the reoriented frame
    float* l2_vec;                 // [n2][4] displacement from the list's atom (FP32), for the prefilter
    long long n2_cap;
    // 3B/4B enumeration
    int* e_cnt3; int* e_cnt4;      // [n2]
    long long* e_off3; long long* e_off4;   // [n2+1]
    int* c3;                       // [n3][3] ghost slots (i, j, k)
    int* c4;                       // [n4][4]
    long long n3_cap, n4_cap;
    int enum_serial;               // 1: some system has 3B and 4B terms with rc4 > rc3 (sequential enumeration)
    // Pair-table cache of the factored kernels: the list entries (i, j) of a
    // cluster's first atom, c3e[n3][2] = entries of ij, ik and c4e[n4][3] =
    // ij, ik, il (written by the enumeration when not null), and per entry
    // the Chebyshev tables of body order 3 / 4 (pcd: dr[3], r, fc, fcd as
    // doubles; pct: T[R], dT/dr[R] in the compute type)
    int* c3e; int* c4e;
    int use_pc3, use_pc4;
    // 1: bucketing drops clusters with a pair at or beyond its tuple's outer
    // cutoff (lists built with padded cutoffs; rebucketed every evaluation)
    int bucket_cut;
    // with bucket_cut on the pair-style path: FP32 copies of the positions and
    // the margin of an FP32 distance (float_eps); a cutoff test decided by more
    // than the margin takes no FP64 distance (null: always exact)
    const float* pos_f;
    float float_eps;
    double* pcd3; double* pcd4;    // [n2_cap][6]
    void* pct3; void* pct4;        // [n2_cap][2R]
    // results
    double* force;                 // [n_in_total][3]
    double* eatom;                 // [n_in_total] per-atom energy or null (pair-style path)
    double* vatom;                 // [n_in_total][6] per-atom virial (xx yy zz xy xz yz) or null
    double* ev;                    // [n_sys][8]: energy, virial xx xy xz yy yz zz, spare
    int* flags;                    // [8] device error flags: 0 capacity, 1 geometry, 2 badness max,
                                   //     3 penalty count, 4 below-rin count, 5 table look-ups,
                                   //     6 inputs (no-alloc entry), 7 bounded wait expired
    unsigned long long* queue;     // [2] work-queue heads of the 3-body and 4-body force kernels
    // cluster buckets by (parameter set, ordered type tuple), for the factored
    // contraction: bucket key = pset.bk{3,4} + tuple index; each bucket padded
    // to a multiple of 32 slots with -1, so a warp's clusters share one tuple
    // (3-body: of bk_pad3 slots, 128 for the tensor-core form's 128-cluster tiles)
    int nbk3, nbk4;
    int bk_pad3;
    int* bk_key3;                  // [n3_cap] / [n4_cap] or null: each cluster's bucket key,
    int* bk_key4;                  //   written by the count pass and read by the scatter pass
    int* bk_count;                 // [nbk3 + nbk4]
    int* bk_fill;                  // [nbk3 + nbk4]
    long long* bk_start;           // [nbk3 + 1] then [nbk4 + 1]; last = slots in use
    int* perm3; int* perm4;        // [perm*_cap] cluster index or -1
    long long perm3_cap, perm4_cap;
};

// A caller's full neighbour list with ghost atoms (LAMMPS layout), for the
// pair-style path (ck_neigh.cu): local atoms ilist[inum], entries of atom
// ilist[ii] at neigh[off[ii] .. off[ii+1]), owner[e] = ii.
struct NeighView {
    long long inum, nent;
    const int* ilist;
    const long long* off;
    const int* neigh;
    int* owner;
    const long long* tag;
    double c3p, c4p;               // max 3-/4-body outer cutoffs + skin (0 + skin for an absent order)
    int has3, has4;
    // FP32 positions and the padded cutoffs -/+ the FP32 distance margin,
    // rounded outward: a test with the FP32 distance below lo or at or above
    // hi is decided without the FP64 distance
    const float* xf;
    float c3lo, c3hi, c4lo, c4hi;
};

}  // namespace ck
