/*
 * ORACLE -- test infrastructure only.  Nothing in the product links, loads or
 * calls this file; only tests/, the smoke check and the bench's CPU-baseline
 * leg do, as the checker.
 *
 * A plain-C restatement of the reference ChIMES calculator's force-evaluation
 * path (rk-lindsey/chimes_calculator), single-threaded, with the reference's
 * floating-point operation order kept term by term so that, built with
 * -ffp-contract=off against the same libm, it reproduces the reference's
 * results bit for bit.  Each function names the reference code it restates.
 *
 *   parameters ....... chimesFF::read_parameters     chimesFF/src/chimesFF.cpp:354-1570
 *   pair permutations  chimesFF::build_atom_and_pair_mappers  chimesFF/src/chimesFF.h:438-539
 *                      build_pair_int_trip_map / quad_map     chimesFF.cpp:3023-3080, 2958-3021
 *   Chebyshev ........ set_cheby_polys               chimesFF.h:542-628
 *                      set_polys_out_of_range        chimesFF.cpp:1572-1613
 *   cutoff/penalty ... get_fcut / get_penalty        chimesFF.h:347-419
 *   cluster terms .... compute_1B/2B/3B/4B           chimesFF.cpp:1636-1775, 1931-2176, 2496-2872
 *   system set-up .... set_hmat, simulation_system::init, reorient, build_layered_system
 *                      serial_interface/src/serial_chimes_interface.cpp:85-587
 *   cluster lists .... simulation_system::build_neigh_lists  serial_chimes_interface.cpp:588-864
 *   driver ........... serial_chimes_interface::calculate    serial_chimes_interface.cpp:960-1124
 *   fingerprints ..... cluster records of the FINGERPRINT build  etc/lmp/src/pair_chimes.cpp:525-536,
 *                      620-662, 700-741, 775-810; chimesFF.cpp:1694-1702, 2013-2021, 2603-2612
 *                      cluster-distance histograms  chimesFF/src/FP/multi_calc_histogram.cpp
 *   tabulated terms .. read_2B_tab / read_3B_tab     chimesFF.cpp:199-351 (TABULATION build)
 *                      compute_2B_tab / get_tab_2B   chimesFF.cpp:1776-1922
 *                      compute_3B_tab / interpolateTricubic / get_tab_3B  chimesFF.cpp:2177-2463
 *
 * Errors are returned as negative status codes with a message (the reference
 * prints and calls exit(0)); the oracle never terminates its host process.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORA_PI 3.14159265359 /* chimesFF.h:22 */
#define MAXTOK 64

typedef struct {
    int ntypes, npairs, o2, o3, o4;
    char (*atm)[16];          /* [ntypes] element names                   */
    char (*pname)[40];        /* [npairs] proper pair name (atm1+atm2)     */
    char (*pa1)[16], (*pa2)[16];
    double *rin, *rout, *lam; /* [npairs]                                  */
    int fcut_tersoff; double fcut_var;
    double pen_dist, pen_scale, inner_smooth;
    double *eoff;             /* [ntypes]                                  */
    int *pows2; double *c2;   /* [npairs][o2]                              */
    int *pair_map;            /* [nt*nt] atom_int_pair_map                 */
    int *prpr;                /* [nt*nt] index of proper pair name         */
    /* 3B */
    int ntrips; int *n3; int **pw3; double **c3; double *cut3; /* cut3[t][2][3] */
    char (*t3atm)[3][16]; char (*t3pair)[3][40];
    int *trip_map; int *trip_perm; /* [nt^3], [nt^3][3] */
    /* 4B */
    int nquads; int *n4; int **pw4; double **c4; double *cut4; /* cut4[q][2][6] */
    char (*q4atm)[4][16]; char (*q4pair)[6][40];
    int *quad_map; int *quad_perm; /* [nt^4], [nt^4][6] */
    int badness;
    long n_penalty, n_below_rin;
    /* tabulated terms: tables in the order the file names them */
    int tab2, tab3, n_t2, n_t3;
    struct { long n; double *r, *e, *f; } *t2;
    struct { long n; double *rij, *rik, *rjk, *e, *fij, *fik, *fjk; } *t3;
    int tab_err;             /* 1: 2B distance below the table (the reference exits); 2: 3B grid index past the rows */
} ora_ff;

typedef struct {
    int n_atoms, n_ghost, n_repl, n_replicates, n_layers;
    double *x, *y, *z; int *parent, *rep_parent, *typ;
    double h[9], hi[9];
    double la, lb, lc, vol;
    long cap;
} ora_sys;

typedef struct {
    ora_ff ff;
    char err[512];
    /* last calculate() cluster lists (neigh/sys ghost indices) */
    long n2, n3, n4;
    int *l2, *l3, *l4;
    /* cluster lists of the LAMMPS pair-style restatement (atom indices) */
    int *lmp_l3, *lmp_l4;
    long lmp_n3, lmp_n4, lmp_c3, lmp_c4;
    int lmp_built;
    long cap2, cap3, cap4;
    /* fingerprint records of the last pair-style call (when lmp_fp is set):
     * [body-2] -> distances [n][P] and type indices [n][body] */
    int lmp_fp;
    double *fp_d[3]; int *fp_t[3]; long fp_n[3], fp_cap[3];
} ora_handle;

/* ------------------------------------------------------------------ */
/* text helpers (chimesFF::split_line, chimesFF.cpp:148-180)           */
/* ------------------------------------------------------------------ */
typedef struct { char **lines; int n; char *buf; } ora_text;

static int load_text(const char *path, ora_text *t) {
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END); long sz = ftell(f); fseek(f, 0, SEEK_SET);
    t->buf = (char *)malloc(sz + 1);
    if (fread(t->buf, 1, sz, f) != (size_t)sz) { fclose(f); return -1; }
    t->buf[sz] = 0; fclose(f);
    int cap = 1024; t->lines = (char **)malloc(cap * sizeof(char *)); t->n = 0;
    char *p = t->buf;
    while (*p) {
        if (t->n == cap) { cap *= 2; t->lines = (char **)realloc(t->lines, cap * sizeof(char *)); }
        t->lines[t->n++] = p;
        char *e = strchr(p, '\n');
        if (!e) break;
        *e = 0; p = e + 1;
    }
    return 0;
}

static int split(const char *line, char tok[][MAXTOK], int maxt) {
    char tmp[4096];
    strncpy(tmp, line, sizeof(tmp) - 1); tmp[sizeof(tmp) - 1] = 0;
    char *c = strchr(tmp, '!'); if (c) *c = 0;
    c = strstr(tmp, "##"); if (c) *c = 0;
    int n = 0; char *s = tmp;
    while (*s && n < maxt) {
        while (*s == ' ' || *s == '\t' || *s == '\r' || *s == '\n' || *s == '\v' || *s == '\f') s++;
        if (!*s) break;
        int k = 0;
        while (*s && !(*s == ' ' || *s == '\t' || *s == '\r' || *s == '\n' || *s == '\v' || *s == '\f')) {
            if (k < MAXTOK - 1) tok[n][k++] = *s;
            s++;
        }
        tok[n][k] = 0; n++;
    }
    return n;
}

#define FAIL(h, ...) do { snprintf((h)->err, sizeof((h)->err), __VA_ARGS__); return -1; } while (0)

/* get_proper_pair, chimesFF.cpp:69-84 */
static int proper_pair(ora_ff *ff, const char *a, const char *b) {
    for (int i = 0; i < ff->npairs; i++) {
        if (!strcmp(a, ff->pa1[i]) && !strcmp(b, ff->pa2[i])) return i;
        if (!strcmp(b, ff->pa1[i]) && !strcmp(a, ff->pa2[i])) return i;
    }
    return -1;
}

static int find_atm(ora_ff *ff, const char *name) {
    for (int i = 0; i < ff->ntypes; i++) if (!strcmp(ff->atm[i], name)) return i;
    return ff->ntypes;
}

/* std::next_permutation on a small int array */
static int next_perm(int *a, int n) {
    int i = n - 2;
    while (i >= 0 && a[i] >= a[i + 1]) i--;
    if (i < 0) { for (int l = 0, r = n - 1; l < r; l++, r--) { int t = a[l]; a[l] = a[r]; a[r] = t; } return 0; }
    int j = n - 1;
    while (a[j] <= a[i]) j--;
    int t = a[i]; a[i] = a[j]; a[j] = t;
    for (int l = i + 1, r = n - 1; l < r; l++, r--) { t = a[l]; a[l] = a[r]; a[r] = t; }
    return 1;
}

/* build_atom_and_pair_mappers, chimesFF.h:438-539.  pair_map carries over
 * between calls when no permutation matches, as the reference's reused
 * vector does. */
static void atom_pair_mapper(ora_ff *ff, int natoms, const int *typ, char (*clu_pairs)[40], int *pair_map) {
    int npairs = natoms * (natoms - 1) / 2;
    int perm[4], tmp_pairs[6][2], run_pairs[6][2];
    memset(run_pairs, 0, sizeof(run_pairs));
    for (int i = 0; i < natoms; i++) perm[i] = i;
    int idx = 0;
    for (int i = 0; i < natoms; i++) for (int j = i + 1; j < natoms; j++) { tmp_pairs[idx][0] = i; tmp_pairs[idx][1] = j; idx++; }
    do {
        int match = 1; idx = 0;
        for (int i = 0; i < natoms && match; i++)
            for (int j = i + 1; j < natoms; j++) {
                const char *rt = ff->pname[ff->prpr[typ[perm[i]] * ff->ntypes + typ[perm[j]]]];
                if (strcmp(clu_pairs[idx], rt)) { match = 0; break; }
                idx++;
            }
        if (match) {
            idx = 0;
            for (int i = 0; i < natoms; i++) for (int j = i + 1; j < natoms; j++) { run_pairs[idx][0] = perm[i]; run_pairs[idx][1] = perm[j]; idx++; }
            break;
        }
    } while (next_perm(perm, natoms));
    for (int i = 0; i < npairs; i++)
        for (int j = 0; j < npairs; j++)
            if ((run_pairs[i][0] == tmp_pairs[j][0] && run_pairs[i][1] == tmp_pairs[j][1]) ||
                (run_pairs[i][0] == tmp_pairs[j][1] && run_pairs[i][1] == tmp_pairs[j][0]))
                pair_map[j] = i;
}

/* ------------------------------------------------------------------ */
/* read_parameters, chimesFF.cpp:354-1570                              */
/* ------------------------------------------------------------------ */
/* read_2B_tab / read_3B_tab (chimesFF.cpp:199-351): "<name>.energy" and
 * "<name>.force", a row count, then rows of 2 (2B) or 4 / 6 (3B) numbers.  The
 * name is taken relative to the parameter file's directory. */
static long read_rows(const char *path, int *widths, int nw, double **cols, int ncols) {
    ora_text T;
    if (load_text(path, &T)) return -1;
    char tok[MAXTOK][MAXTOK];
    if (T.n < 1 || split(T.lines[0], tok, MAXTOK) < 1) { free(T.lines); free(T.buf); return -1; }
    long n = atol(tok[0]);
    if (n < 0 || n + 1 > T.n) { free(T.lines); free(T.buf); return -1; }
    for (int c = 0; c < ncols; c++) cols[c] = calloc(n + 1, sizeof(double));
    for (long i = 0; i < n; i++) {
        int k = split(T.lines[i + 1], tok, MAXTOK), ok = 0;
        for (int w = 0; w < nw; w++) ok |= k == widths[w];
        if (!ok || k < ncols) { free(T.lines); free(T.buf); return -1; }
        for (int c = 0; c < ncols; c++) cols[c][i] = strtod(tok[c], 0);
    }
    free(T.lines); free(T.buf);
    return n;
}

static int read_tab(ora_handle *h, const char *dir, const char *name, int body) {
    ora_ff *ff = &h->ff;
    char pe[1024], pf[1024];
    snprintf(pe, sizeof(pe), "%s%s.energy", dir, name);
    snprintf(pf, sizeof(pf), "%s%s.force", dir, name);
    if (body == 2) {
        double *e[2], *f[2];
        int w2[1] = {2};
        long ne = read_rows(pe, w2, 1, e, 2), nf = read_rows(pf, w2, 1, f, 2);
        if (ne < 0 || nf < 0 || ne != nf) FAIL(h, "cannot read 2-body table %s", name);
        ff->t2 = realloc(ff->t2, (size_t)(ff->n_t2 + 1) * sizeof(*ff->t2));
        ff->t2[ff->n_t2].n = ne; ff->t2[ff->n_t2].r = e[0]; ff->t2[ff->n_t2].e = e[1]; ff->t2[ff->n_t2].f = f[1];
        free(f[0]);
        ff->n_t2++;
    } else {
        double *e[4], *f[6];
        int w3[2] = {4, 6}, w6[1] = {6};
        long ne = read_rows(pe, w3, 2, e, 4), nf = read_rows(pf, w6, 1, f, 6);
        if (ne < 0 || nf < 0 || ne != nf) FAIL(h, "cannot read 3-body table %s", name);
        if ((int)cbrt((double)ne) < 2) FAIL(h, "3-body table %s has fewer than 8 rows", name);
        ff->t3 = realloc(ff->t3, (size_t)(ff->n_t3 + 1) * sizeof(*ff->t3));
        ff->t3[ff->n_t3].n = ne;
        ff->t3[ff->n_t3].rij = e[0]; ff->t3[ff->n_t3].rik = e[1]; ff->t3[ff->n_t3].rjk = e[2]; ff->t3[ff->n_t3].e = e[3];
        ff->t3[ff->n_t3].fij = f[3]; ff->t3[ff->n_t3].fik = f[4]; ff->t3[ff->n_t3].fjk = f[5];
        free(f[0]); free(f[1]); free(f[2]);
        ff->n_t3++;
    }
    return 0;
}

static int parse(ora_handle *h, const char *path) {
    ora_ff *ff = &h->ff;
    ora_text T;
    if (load_text(path, &T)) FAIL(h, "cannot open parameter file: %s", path);
    char tok[MAXTOK][MAXTOK];
    int L;
    char dir[1024] = "";
    const char *slash = strrchr(path, '/');
    if (slash && (size_t)(slash - path + 1) < sizeof(dir)) { memcpy(dir, path, slash - path + 1); dir[slash - path + 1] = 0; }
    int n_plain2 = 0;
    ff->pen_dist = 0.01; ff->pen_scale = 1.0e4; ff->inner_smooth = 0.01; /* chimesFF.cpp:104-116 */
    ff->fcut_tersoff = 0;
    /* pass 1: orders */
    int found = 0;
    for (L = 0; L < T.n; L++) {
        if (strstr(T.lines[L], "ENDFILE")) break;
        if (strstr(T.lines[L], "PAIRTYP: CHEBYSHEV")) {
            int n = split(T.lines[L], tok, MAXTOK);
            if (n < 3) FAIL(h, "PAIRTYP line must contain the 2-body order");
            ff->o2 = atoi(tok[2]); ff->o3 = n >= 4 ? atoi(tok[3]) : 0; ff->o4 = n >= 5 ? atoi(tok[4]) : 0;
            found = 1; break;
        }
    }
    if (!found) FAIL(h, "not a ChIMES Chebyshev parameter file");
    /* pass 2: general */
    int npairs = 0;
    for (L = 0; L < T.n; L++) {
        const char *ln = T.lines[L];
        if (strstr(ln, "ENDFILE")) break;
        if (strstr(ln, "ATOM TYPES:")) {
            split(ln, tok, MAXTOK); ff->ntypes = atoi(tok[2]);
            ff->eoff = (double *)calloc(ff->ntypes, sizeof(double));
            ff->atm = calloc(ff->ntypes, sizeof(*ff->atm));
        }
        if (strstr(ln, "# TYPEIDX #")) {
            for (int i = 0; i < ff->ntypes; i++) {
                if (++L >= T.n) FAIL(h, "truncated TYPEIDX block");
                split(T.lines[L], tok, MAXTOK); strncpy(ff->atm[i], tok[1], 15);
            }
        }
        if (strstr(ln, "ATOM PAIRS:")) { split(ln, tok, MAXTOK); npairs = atoi(tok[2]); }
        if (strstr(ln, "# PAIRIDX #")) {
            if (strstr(ln, "# USEOVRP #")) continue;
            ff->npairs = npairs;
            ff->pname = calloc(npairs, sizeof(*ff->pname)); ff->pa1 = calloc(npairs, sizeof(*ff->pa1));
            ff->pa2 = calloc(npairs, sizeof(*ff->pa2));
            ff->rin = calloc(npairs, sizeof(double)); ff->rout = calloc(npairs, sizeof(double));
            ff->lam = calloc(npairs, sizeof(double));
            for (int i = 0; i < npairs; i++) {
                if (++L >= T.n) FAIL(h, "truncated PAIRIDX block");
                int n = split(T.lines[L], tok, MAXTOK);
                int xf, mo;
                if (n == 8) { xf = 6; mo = 7; } else if (n == 7) { xf = 5; mo = 6; }
                else FAIL(h, "pair line: expect 7 or 8 entries");
                strncpy(ff->pa1[i], tok[1], 15); strncpy(ff->pa2[i], tok[2], 15);
                snprintf(ff->pname[i], 40, "%.19s%.19s", tok[1], tok[2]);
                ff->rin[i] = strtod(tok[3], 0); ff->rout[i] = strtod(tok[4], 0);
                if (strcmp(tok[xf], "MORSE")) FAIL(h, "only the MORSE distance transformation is supported");
                ff->lam[i] = strtod(tok[mo], 0);
            }
        }
        if (strstr(ln, "FCUT TYPE:")) {
            split(ln, tok, MAXTOK);
            if (!strcmp(tok[2], "CUBIC")) ff->fcut_tersoff = 0;
            else if (!strcmp(tok[2], "TERSOFF")) { ff->fcut_tersoff = 1; ff->fcut_var = strtod(tok[3], 0); }
            else FAIL(h, "unknown FCUT TYPE: %s", tok[2]);
        }
        if (strstr(ln, "PAIR CHEBYSHEV PENALTY DIST:")) { split(ln, tok, MAXTOK); ff->pen_dist = strtod(tok[4], 0); }
        if (strstr(ln, "PAIR CHEBYSHEV PENALTY SCALING:")) { split(ln, tok, MAXTOK); ff->pen_scale = strtod(tok[4], 0); }
        if (strstr(ln, "NO ENERGY OFFSETS:")) {
            int n = split(ln, tok, MAXTOK);
            if (atoi(tok[n - 1]) != ff->ntypes) FAIL(h, "number of energy offsets does not match atom types");
            for (int i = 0; i < ff->ntypes; i++) {
                if (++L >= T.n) FAIL(h, "truncated energy offsets");
                split(T.lines[L], tok, MAXTOK);
                ff->eoff[atoi(tok[2]) - 1] = strtod(tok[3], 0);
            }
        }
    }
    int nt = ff->ntypes;
    if (nt <= 0 || ff->npairs <= 0) FAIL(h, "missing ATOM TYPES or ATOM PAIRS");
    /* pass 3: 2B parameters and PAIRMAPS */
    ff->pows2 = calloc((size_t)ff->npairs * (ff->o2 > 0 ? ff->o2 : 1), sizeof(int));
    ff->c2 = calloc((size_t)ff->npairs * (ff->o2 > 0 ? ff->o2 : 1), sizeof(double));
    ff->pair_map = calloc(nt * nt, sizeof(int)); ff->prpr = calloc(nt * nt, sizeof(int));
    int have_pmap = 0;
    for (L = 0; L < T.n; L++) {
        const char *ln = T.lines[L];
        if (strstr(ln, "ENDFILE")) break;
        if (strstr(ln, "PAIRTYPE PARAMS:")) {
            int nt7 = split(ln, tok, MAXTOK);
            if (nt7 == 7) {   /* tabulated 2B (chimesFF.cpp:719-735) */
                if (n_plain2) FAIL(h, "All parameters of a given bodiedness must either be tabulated or not tabulated");
                if (read_tab(h, dir, tok[6], 2)) return -1;
                ff->tab2 = 1;
                continue;
            }
            if (ff->tab2) FAIL(h, "All parameters of a given bodiedness must either be tabulated or not tabulated");
            n_plain2++;
            int p = atoi(tok[2]);
            if (p < 0 || p >= ff->npairs) FAIL(h, "pair index out of range");
            L++;
            for (int i = 0; i < ff->o2; i++) {
                if (++L >= T.n) FAIL(h, "truncated 2B parameters");
                split(T.lines[L], tok, MAXTOK);
                ff->pows2[p * ff->o2 + i] = atoi(tok[0]); ff->c2[p * ff->o2 + i] = strtod(tok[1], 0);
            }
        }
        if (strstr(ln, "PAIRMAPS:")) {
            split(ln, tok, MAXTOK); int nm = atoi(tok[1]);
            int *mi = calloc(nm, sizeof(int)); char (*mk)[64] = calloc(nm, 64);
            for (int i = 0; i < nm; i++) {
                if (++L >= T.n) FAIL(h, "truncated PAIRMAPS");
                split(T.lines[L], tok, MAXTOK); mi[i] = atoi(tok[0]); strncpy(mk[i], tok[1], 63);
            }
            for (int i = 0; i < nt; i++)
                for (int j = 0; j < nt; j++) {
                    char key[64]; snprintf(key, 64, "%s%s", ff->atm[i], ff->atm[j]);
                    int k; for (k = 0; k < nm; k++) if (!strcmp(mk[k], key)) break;
                    if (k == nm) FAIL(h, "could not find element in vector: %s", key);
                    ff->pair_map[i * nt + j] = mi[k];
                    int pp = proper_pair(ff, ff->atm[i], ff->atm[j]);
                    if (pp < 0) FAIL(h, "no proper pair name for %s %s", ff->atm[i], ff->atm[j]);
                    ff->prpr[i * nt + j] = pp;
                }
            free(mi); free(mk); have_pmap = 1;
        }
    }
    if (!have_pmap) FAIL(h, "missing PAIRMAPS");
    if (ff->tab2 && ff->n_t2 < ff->npairs) FAIL(h, "fewer tabulated 2-body tables than pair types");
    /* passes 4-5: 3B, then 6-7: 4B (same structure) */
    for (int body = 3; body <= 4; body++) {
        int order = body == 3 ? ff->o3 : ff->o4;
        if (order <= 0) continue;
        int np = body == 3 ? 3 : 6;
        const char *hdr_count = body == 3 ? "ATOM PAIR TRIPLETS:" : "ATOM PAIR QUADRUPLETS:";
        const char *hdr_type = body == 3 ? "TRIPLETTYPE PARAMS:" : "QUADRUPLETYPE PARAMS:";
        const char *hdr_maps = body == 3 ? "TRIPMAPS:" : "QUADMAPS:";
        int ntyp = 0; int *ncoef = NULL; int **pw = NULL; double **cf = NULL; double *cut = NULL;
        char (*catm)[16] = NULL; char (*cpair)[40] = NULL; /* [ntyp*body], [ntyp*np] */
        int *tmap = NULL; int ntup = body == 3 ? nt * nt * nt : nt * nt * nt * nt;
        int *map_idx = NULL; char (*map_key)[256] = NULL; int nmaps = 0;
        for (L = 0; L < T.n; L++) {
            const char *ln = T.lines[L];
            if (strstr(ln, "ENDFILE")) break;
            if (strstr(ln, hdr_count)) {
                split(ln, tok, MAXTOK); ntyp = atoi(tok[3]);
                ncoef = calloc(ntyp, sizeof(int)); pw = calloc(ntyp, sizeof(int *)); cf = calloc(ntyp, sizeof(double *));
                cut = calloc((size_t)ntyp * 2 * np, sizeof(double));
                catm = calloc((size_t)ntyp * body, 16); cpair = calloc((size_t)ntyp * np, 40);
            }
            if (strstr(ln, hdr_type)) {
                if (!ncoef) FAIL(h, "%s before %s", hdr_type, hdr_count);
                if (++L >= T.n) FAIL(h, "truncated cluster block");
                int ntk = split(T.lines[L], tok, MAXTOK);
                int t = atoi(tok[1]);
                if (t < 0 || t >= ntyp) FAIL(h, "cluster type index out of range");
                for (int a = 0; a < body; a++) strncpy(catm[t * body + a], tok[3 + a], 15);
                if (body == 3 && ntk == 8) {   /* tabulated 3B (chimesFF.cpp:882-896) */
                    if (read_tab(h, dir, tok[7], 3)) return -1;
                    ff->tab3 = 1;
                }
                if (++L >= T.n) FAIL(h, "truncated cluster block");
                split(T.lines[L], tok, MAXTOK);
                for (int p = 0; p < np; p++) strncpy(cpair[t * np + p], tok[1 + p], 39);
                if (strcmp(tok[1 + np], "EXCLUDED:") && !(body == 3 && ff->tab3)) {   /* :912-918 */
                    int nc = atoi(tok[body == 3 ? 7 : 10]);
                    ncoef[t] = nc; pw[t] = calloc((size_t)nc * np + 1, sizeof(int)); cf[t] = calloc(nc + 1, sizeof(double));
                    L += 2;
                    for (int c = 0; c < nc; c++) {
                        if (++L >= T.n) FAIL(h, "truncated coefficient list");
                        split(T.lines[L], tok, MAXTOK);
                        for (int p = 0; p < np; p++) pw[t][c * np + p] = atoi(tok[1 + p]);
                        cf[t][c] = strtod(tok[body == 3 ? 6 : 9], 0);
                    }
                }
            }
            if (strstr(ln, hdr_maps)) {
                split(ln, tok, MAXTOK); nmaps = atoi(tok[1]);
                map_idx = calloc(nmaps, sizeof(int)); map_key = calloc(nmaps, 256);
                for (int i = 0; i < nmaps; i++) {
                    if (++L >= T.n) FAIL(h, "truncated map block");
                    split(T.lines[L], tok, MAXTOK); map_idx[i] = atoi(tok[0]); strncpy(map_key[i], tok[1], 255);
                }
                tmap = calloc(ntup, sizeof(int));
                for (int u = 0; u < ntup; u++) {
                    int a[4], r = u;
                    for (int k = body - 1; k >= 0; k--) { a[k] = r % nt; r /= nt; }
                    char key[256] = "";
                    for (int i = 0; i < body; i++)
                        for (int j = i + 1; j < body; j++) strcat(key, ff->pname[proper_pair(ff, ff->atm[a[i]], ff->atm[a[j]])]);
                    int k; for (k = 0; k < nmaps; k++) if (!strcmp(map_key[k], key)) break;
                    if (k == nmaps) FAIL(h, "could not find element in vector: %s", key);
                    tmap[u] = map_idx[k];
                }
            }
        }
        if (!tmap) FAIL(h, "missing %s", hdr_maps);
        if (body == 3 && ff->tab3)
            for (int u = 0; u < ntup; u++)
                if (tmap[u] >= ff->n_t3) FAIL(h, "no tabulated 3-body table for triplet type %d", tmap[u]);
        /* default cutoffs: 2B values of each pair of the type's atoms (chimesFF.cpp:947-980, 1280-1325) */
        for (int t = 0; t < ntyp; t++) {
            int a[4];
            for (int k = 0; k < body; k++) a[k] = find_atm(ff, catm[t * body + k]);
            int p = 0;
            for (int i = 0; i < body; i++)
                for (int j = i + 1; j < body; j++, p++) {
                    int pt = ff->pair_map[a[i] * nt + a[j]];
                    cut[(t * 2 + 0) * np + p] = ff->rin[pt];
                    cut[(t * 2 + 1) * np + p] = ff->rout[pt];
                }
        }
        /* SPECIAL S_MAXIM / S_MINIM (chimesFF.cpp:1009-1168, 1353-1566) */
        const char *smax = body == 3 ? "SPECIAL 3B S_MAXIM:" : "SPECIAL 4B S_MAXIM:";
        const char *smin = body == 3 ? "SPECIAL 3B S_MINIM:" : "SPECIAL 4B S_MINIM:";
        for (L = 0; L < T.n; L++) {
            const char *ln = T.lines[L];
            if (strstr(ln, "ENDFILE")) break;
            int which = strstr(ln, smax) ? 1 : (strstr(ln, smin) ? 0 : -1);
            if (which < 0) continue;
            split(ln, tok, MAXTOK);
            if (!strcmp(tok[3], "ALL")) {
                double v = strtod(tok[4], 0);
                for (int t = 0; t < ntyp; t++) for (int p = 0; p < np; p++) cut[(t * 2 + which) * np + p] = v;
            } else {
                int ne = atoi(tok[4]);
                if (which == 0 && body == 4)
                    for (int t = 0; t < ntyp; t++) for (int p = 0; p < np; p++) cut[(t * 2 + 0) * np + p] = -1.0;
                for (int e = 0; e < ne; e++) {
                    if (++L >= T.n) FAIL(h, "truncated SPECIAL block");
                    split(T.lines[L], tok, MAXTOK);
                    int k; for (k = 0; k < nmaps; k++) if (!strcmp(map_key[k], tok[0])) break;
                    if (k == nmaps) FAIL(h, "SPECIAL entry names an unknown cluster type: %s", tok[0]);
                    int t = map_idx[k];
                    if (t < 0 || t >= ntyp) FAIL(h, "SPECIAL entry maps outside the cluster types");
                    int disq[6] = {0, 0, 0, 0, 0, 0};
                    for (int q = 0; q < np; q++) {
                        int slot = -1;
                        for (int p = 0; p < np; p++)
                            if (!strcmp(cpair[t * np + p], tok[1 + q]) && !disq[p]) { disq[p] = 1; slot = p; break; }
                        if (slot < 0) FAIL(h, "could not find element in vector: %s", tok[1 + q]);
                        cut[(t * 2 + which) * np + slot] = strtod(tok[1 + np + q], 0);
                    }
                }
            }
        }
        /* build_pair_int_trip_map / quad_map */
        int *perm = calloc((size_t)ntup * np, sizeof(int));
        int pair_map[6] = {0, 0, 0, 0, 0, 0};
        for (int u = 0; u < ntup; u++) {
            int a[4], r = u;
            for (int k = body - 1; k >= 0; k--) { a[k] = r % nt; r /= nt; }
            int t = tmap[u];
            if (t < 0) continue;
            if (t >= ntyp) FAIL(h, "cluster map entry out of range");
            atom_pair_mapper(ff, body, a, &cpair[t * np], pair_map);
            memcpy(&perm[u * np], pair_map, np * sizeof(int));
        }
        if (body == 3) {
            ff->ntrips = ntyp; ff->n3 = ncoef; ff->pw3 = pw; ff->c3 = cf; ff->cut3 = cut;
            ff->trip_map = tmap; ff->trip_perm = perm;
        } else {
            ff->nquads = ntyp; ff->n4 = ncoef; ff->pw4 = pw; ff->c4 = cf; ff->cut4 = cut;
            ff->quad_map = tmap; ff->quad_perm = perm;
        }
        free(map_idx); free(map_key); free(catm); free(cpair);
    }
    free(T.lines); free(T.buf);
    return 0;
}

/* max_cutoff_2B/3B/4B, chimesFF.cpp:2890-2943 */
static double max_cut2(ora_ff *ff) {
    double m = ff->rout[0];
    for (int i = 0; i < ff->npairs; i++) if (ff->rout[i] > m) m = ff->rout[i];
    return m;
}
static double max_cutn(ora_ff *ff, int body) {
    int order = body == 3 ? ff->o3 : ff->o4;
    if (order == 0) return 0.0;
    int np = body == 3 ? 3 : 6, nty = body == 3 ? ff->ntrips : ff->nquads;
    double *cut = body == 3 ? ff->cut3 : ff->cut4;
    double m = cut[(0 * 2 + 1) * np + 0];
    for (int t = 0; t < nty; t++) for (int p = 0; p < np; p++) if (cut[(t * 2 + 1) * np + p] > m) m = cut[(t * 2 + 1) * np + p];
    return m;
}

/* ------------------------------------------------------------------ */
/* per-cluster math                                                    */
/* ------------------------------------------------------------------ */
static void cheby(ora_ff *ff, double *Tn, double *Tnd, double dx, double morse, double rin, double rout, int order) {
    double x_min = exp(-1 * rin / morse);
    double x_max = exp(-1 * rout / morse);
    double x_avg = 0.5 * (x_max + x_min);
    double x_diff = 0.5 * (x_max - x_min);
    x_diff *= -1.0;
    int oor = 0; double dx_orig = dx;
    if (dx < rin) { oor = 1; dx = rin; }
    double exprlen = exp(-1 * dx / morse);
    double x = (exprlen - x_avg) / x_diff;
    double dx_dr = (-exprlen / morse) / x_diff;
    Tn[0] = 1.0; Tn[1] = x; Tnd[0] = 1.0; Tnd[1] = 2.0 * x;
    for (int i = 2; i <= order; i++) {
        Tn[i] = 2.0 * x * Tn[i - 1] - Tn[i - 2];
        Tnd[i] = 2.0 * x * Tnd[i - 1] - Tnd[i - 2];
    }
    for (int i = order; i >= 1; i--) Tnd[i] = i * dx_dr * Tnd[i - 1];
    Tnd[0] = 0.0;
    if (oor) {
        ff->n_below_rin++;
        double damp = exp((dx_orig - rin) / ff->inner_smooth);
        for (int i = 0; i <= order; i++) {
            Tn[i] += ff->inner_smooth * (damp - 1.0) * Tnd[i];
            Tnd[i] *= damp;
        }
    }
}

static void fcut_fn(ora_ff *ff, double dx, double rc, double *fc, double *fcd) {
    if (!ff->fcut_tersoff) {
        double f0 = (1.0 - dx / rc);
        *fc = pow(f0, 3.0);
        *fcd = pow(f0, 2.0);
        *fcd *= -1.0 * 3.0 / rc;
    } else {
        double th = rc - ff->fcut_var * rc;
        if (dx < th) { *fc = 1.0; *fcd = 0.0; }
        else if (dx > rc) { *fc = 0.0; *fcd = 0.0; }
        else {
            double f0 = (dx - th) / (rc - th) * ORA_PI + ORA_PI / 2.0;
            double f0d = ORA_PI / (rc - th);
            *fc = 0.5 + 0.5 * sin(f0);
            *fcd = 0.5 * cos(f0) * f0d;
        }
    }
}

void ora_compute_1b(void *vh, int t, double *E) { ora_handle *h = vh; *E += h->ff.eoff[t]; }

void ora_compute_2b(void *vh, double dx, const double *dr, int t0, int t1, double *force, double *stress, double *E) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    int p = ff->pair_map[t0 * ff->ntypes + t1];
    if (dx >= ff->rout[p]) return;
    double Tn[64], Tnd[64], fc, fcd;
    cheby(ff, Tn, Tnd, dx, ff->lam[p], ff->rin[p], ff->rout[p], ff->o2);
    fcut_fn(ff, dx, ff->rout[p], &fc, &fcd);
    double dx_inv = (dx > 0.0) ? 1.0 / dx : 1e20;
    for (int c = 0; c < ff->o2; c++) {
        double cv = ff->c2[p * ff->o2 + c];
        int pw = ff->pows2[p * ff->o2 + c] + 1;
        *E += cv * fc * Tn[pw];
        double deriv = fc * Tnd[pw] + fcd * Tn[pw];
        double fs = cv * deriv * dx_inv;
        force[0] += fs * dr[0]; force[1] += fs * dr[1]; force[2] += fs * dr[2];
        force[3] -= fs * dr[0]; force[4] -= fs * dr[1]; force[5] -= fs * dr[2];
        stress[0] -= fs * dr[0] * dr[0]; stress[1] -= fs * dr[0] * dr[1]; stress[2] -= fs * dr[0] * dr[2];
        stress[3] -= fs * dr[1] * dr[1]; stress[4] -= fs * dr[1] * dr[2]; stress[5] -= fs * dr[2] * dr[2];
    }
    /* get_penalty, chimesFF.h:388-419 */
    double rpen = 0.0, Epen = 0.0, fs = 1.0;
    if (dx - ff->pen_dist < ff->rin[p]) {
        rpen = ff->rin[p] + ff->pen_dist - dx;
        if (dx < ff->rin[p]) ff->badness = 2;
        else if (1 > ff->badness) ff->badness = 1;
    }
    if (rpen > 0.0) {
        Epen = rpen * rpen * rpen * ff->pen_scale;
        fs = -3.0 * rpen * rpen * ff->pen_scale;
        ff->n_penalty++;
    }
    if (Epen > 0.0) {
        *E += Epen;
        fs /= dx;
        force[0] += fs * dr[0]; force[1] += fs * dr[1]; force[2] += fs * dr[2];
        force[3] -= fs * dr[0]; force[4] -= fs * dr[1]; force[5] -= fs * dr[2];
        stress[0] -= fs * dr[0] * dr[0]; stress[1] -= fs * dr[0] * dr[1]; stress[2] -= fs * dr[0] * dr[2];
        stress[3] -= fs * dr[1] * dr[1]; stress[4] -= fs * dr[1] * dr[2]; stress[5] -= fs * dr[2] * dr[2];
    }
}

/* force/stress update of one pair p joining cluster atoms a and b, with the
 * reference's dr2 distance-tensor product (fs * (dr_a * dr_b)) */
static inline void pair_update(double fs, const double *d, int a, int b, double *force, double *stress) {
    force[a * 3 + 0] += fs * d[0]; force[a * 3 + 1] += fs * d[1]; force[a * 3 + 2] += fs * d[2];
    force[b * 3 + 0] -= fs * d[0]; force[b * 3 + 1] -= fs * d[1]; force[b * 3 + 2] -= fs * d[2];
    stress[0] -= fs * (d[0] * d[0]); stress[1] -= fs * (d[0] * d[1]); stress[2] -= fs * (d[0] * d[2]);
    stress[3] -= fs * (d[1] * d[1]); stress[4] -= fs * (d[1] * d[2]); stress[5] -= fs * (d[2] * d[2]);
}

void ora_compute_3b(void *vh, const double *dx, const double *dr, const int *typ, double *force, double *stress, double *E) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    int nt = ff->ntypes;
    int u = typ[0] * nt * nt + typ[1] * nt + typ[2];
    int t = ff->trip_map[u];
    if (t < 0) return;
    const int *m = &ff->trip_perm[u * 3];
    double co[3], ci[3];
    for (int p = 0; p < 3; p++) {
        co[p] = ff->cut3[(t * 2 + 1) * 3 + m[p]];
        ci[p] = ff->cut3[(t * 2 + 0) * 3 + m[p]];
        if (dx[p] >= co[p]) return;
    }
    int pt[3] = {ff->pair_map[typ[0] * nt + typ[1]], ff->pair_map[typ[0] * nt + typ[2]], ff->pair_map[typ[1] * nt + typ[2]]};
    double Tn[3][64], Tnd[3][64], fc[3], fcd[3];
    for (int p = 0; p < 3; p++) cheby(ff, Tn[p], Tnd[p], dx[p], ff->lam[pt[p]], ci[p], co[p], ff->o3);
    for (int p = 0; p < 3; p++) fcut_fn(ff, dx[p], co[p], &fc[p], &fcd[p]);
    double fall = fc[0] * fc[1] * fc[2];
    double f2[3] = {fc[1] * fc[2] / dx[0], fc[0] * fc[2] / dx[1], fc[0] * fc[1] / dx[2]};
    for (int c = 0; c < ff->n3[t]; c++) {
        double cv = ff->c3[t][c];
        int p0 = ff->pw3[t][c * 3 + m[0]], p1 = ff->pw3[t][c * 3 + m[1]], p2 = ff->pw3[t][c * 3 + m[2]];
        *E += cv * fall * Tn[0][p0] * Tn[1][p1] * Tn[2][p2];
        double d0 = fc[0] * Tnd[0][p0] + fcd[0] * Tn[0][p0];
        double d1 = fc[1] * Tnd[1][p1] + fcd[1] * Tn[1][p1];
        double d2 = fc[2] * Tnd[2][p2] + fcd[2] * Tn[2][p2];
        double fs0 = cv * d0 * f2[0] * Tn[1][p1] * Tn[2][p2];
        double fs1 = cv * d1 * f2[1] * Tn[0][p0] * Tn[2][p2];
        double fs2 = cv * d2 * f2[2] * Tn[0][p0] * Tn[1][p1];
        pair_update(fs0, &dr[0], 0, 1, force, stress);
        pair_update(fs1, &dr[3], 0, 2, force, stress);
        pair_update(fs2, &dr[6], 1, 2, force, stress);
    }
}

void ora_compute_4b(void *vh, const double *dx, const double *dr, const int *typ, double *force, double *stress, double *E) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    int nt = ff->ntypes;
    int u = ((typ[0] * nt + typ[1]) * nt + typ[2]) * nt + typ[3];
    u = typ[0] * nt * nt * nt + typ[1] * nt * nt + typ[2] * nt + typ[3];
    int t = ff->quad_map[u];
    if (t < 0) return;
    const int *m = &ff->quad_perm[u * 6];
    double co[6], ci[6];
    for (int p = 0; p < 6; p++) {
        co[p] = ff->cut4[(t * 2 + 1) * 6 + m[p]];
        ci[p] = ff->cut4[(t * 2 + 0) * 6 + m[p]];
        if (dx[p] >= co[p]) return;
    }
    static const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {1, 2, 3, 2, 3, 3};
    int pt[6];
    for (int p = 0; p < 6; p++) pt[p] = ff->pair_map[typ[A[p]] * nt + typ[B[p]]];
    double Tn[6][64], Tnd[6][64], fc[6], fcd[6];
    for (int p = 0; p < 6; p++) cheby(ff, Tn[p], Tnd[p], dx[p], ff->lam[pt[p]], ci[p], co[p], ff->o4);
    for (int p = 0; p < 6; p++) fcut_fn(ff, dx[p], co[p], &fc[p], &fcd[p]);
    double fall = fc[0] * fc[1] * fc[2] * fc[3] * fc[4] * fc[5];
    double f5[6] = {fc[1] * fc[2] * fc[3] * fc[4] * fc[5] / dx[0], fc[0] * fc[2] * fc[3] * fc[4] * fc[5] / dx[1],
                    fc[0] * fc[1] * fc[3] * fc[4] * fc[5] / dx[2], fc[0] * fc[1] * fc[2] * fc[4] * fc[5] / dx[3],
                    fc[0] * fc[1] * fc[2] * fc[3] * fc[5] / dx[4], fc[0] * fc[1] * fc[2] * fc[3] * fc[4] / dx[5]};
    for (int c = 0; c < ff->n4[t]; c++) {
        double cv = ff->c4[t][c];
        int pw[6];
        for (int p = 0; p < 6; p++) pw[p] = ff->pw4[t][c * 6 + m[p]];
        double t012 = Tn[0][pw[0]] * Tn[1][pw[1]] * Tn[2][pw[2]];
        double t34 = Tn[3][pw[3]] * Tn[4][pw[4]];
        double t5 = Tn[5][pw[5]];
        *E += cv * fall * t012 * t34 * t5;
        double d[6];
        for (int p = 0; p < 6; p++) d[p] = fc[p] * Tnd[p][pw[p]] + fcd[p] * Tn[p][pw[p]];
        double fs0 = cv * d[0] * f5[0] * Tn[1][pw[1]] * Tn[2][pw[2]] * t34 * t5;
        double fs1 = cv * d[1] * f5[1] * Tn[0][pw[0]] * Tn[2][pw[2]] * t34 * t5;
        double fs2 = cv * d[2] * f5[2] * Tn[0][pw[0]] * Tn[1][pw[1]] * t34 * t5;
        double fs3 = cv * d[3] * f5[3] * t012 * Tn[4][pw[4]] * t5;
        double fs4 = cv * d[4] * f5[4] * t012 * Tn[3][pw[3]] * t5;
        double fs5 = cv * d[5] * f5[5] * t012 * t34;
        pair_update(fs0, &dr[0], 0, 1, force, stress);
        pair_update(fs1, &dr[3], 0, 2, force, stress);
        pair_update(fs2, &dr[6], 0, 3, force, stress);
        pair_update(fs3, &dr[9], 1, 2, force, stress);
        pair_update(fs4, &dr[12], 1, 3, force, stress);
        pair_update(fs5, &dr[15], 2, 3, force, stress);
    }
}

/* ------------------------------------------------------------------ */
/* periodic system (serial_chimes_interface.cpp:20-587)                */
/* ------------------------------------------------------------------ */
/* ------------------------------------------------------------------ */
/* tabulated terms (TABULATION build; used by the LAMMPS pair style)    */
/* ------------------------------------------------------------------ */
/* get_tab_2B, chimesFF.cpp:1869-1922: the interval from std::lower_bound,
 * then the local spline coefficients of that interval */
static double tab2_value(ora_ff *ff, int p, double rij, int for_energy) {
    long n = ff->t2[p].n;
    const double *r = ff->t2[p].r;
    long lo = 0, len = n;   /* lower_bound: first r >= rij */
    while (len > 0) {
        long half = len / 2;
        if (r[lo + half] < rij) { lo += half + 1; len -= half + 1; } else len = half;
    }
    long i = lo;
    if (i == n) return 0.0;
    if (i == 0) { ff->tab_err |= 1; return 0.0; }
    if (rij == r[i] && i > 0) i--;
    const double *y = for_energy ? ff->t2[p].e : ff->t2[p].f;
    if (i >= n - 1) return 0.0;
    if (i <= 0) { ff->tab_err |= 1; return 0.0; }
    double h = r[i + 1] - r[i];
    double alpha = (3 * (y[i + 1] - y[i]) / h) - (3 * (y[i] - y[i - 1]) / (r[i] - r[i - 1]));
    double l = 2 * (r[i + 1] - r[i - 1]) - h;
    double mu = h / l;
    double z = alpha / l;
    double c_prev = 0.0;
    double c = z - mu * c_prev;
    double b = (y[i + 1] - y[i]) / h - h * (c + 2 * c_prev) / 3.0;
    double d = (c - c_prev) / (3.0 * h);
    double a = y[i];
    double dx = rij - r[i];
    return a + b * dx + c * dx * dx + d * dx * dx * dx;
}

double ora_tab2(void *vh, int pair, double r, int for_energy) { return tab2_value(&((ora_handle *)vh)->ff, pair, r, for_energy); }

/* compute_2B_tab, chimesFF.cpp:1782-1867.  fscal receives force_scalar_in:
 * get_penalty overwrites the table's scalar with 1.0 or the penalty slope. */
void ora_compute_2b_tab(void *vh, double dx, const double *dr, int t0, int t1, double *force, double *stress, double *E,
                        double *fscal) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    int p = ff->pair_map[t0 * ff->ntypes + t1];
    if (dx >= ff->rout[p]) return;
    *E += tab2_value(ff, p, dx, 1);
    double fs = tab2_value(ff, p, dx, 0);
    force[0] += fs * dr[0]; force[1] += fs * dr[1]; force[2] += fs * dr[2];
    force[3] -= fs * dr[0]; force[4] -= fs * dr[1]; force[5] -= fs * dr[2];
    stress[0] -= fs * dr[0] * dr[0]; stress[1] -= fs * dr[0] * dr[1]; stress[2] -= fs * dr[0] * dr[2];
    stress[3] -= fs * dr[1] * dr[1]; stress[4] -= fs * dr[1] * dr[2]; stress[5] -= fs * dr[2] * dr[2];
    /* get_penalty (chimesFF.h:388-419): badness only, the table carries the penalty */
    double rpen = 0.0;
    fs = 1.0;
    if (dx - ff->pen_dist < ff->rin[p]) {
        rpen = ff->rin[p] + ff->pen_dist - dx;
        if (dx < ff->rin[p]) ff->badness = 2;
        else if (1 > ff->badness) ff->badness = 1;
    }
    if (rpen > 0.0) { fs = -3.0 * rpen * rpen * ff->pen_scale; ff->n_penalty++; }
    if (fscal) *fscal = fs;
}

/* cubicInterpolate / bicubicInterpolate / tricubicInterpolate, chimesFF.cpp:2339-2366 */
static double tab_cubic(double p0, double p1, double p2, double p3, double x) {
    return p1 + 0.5 * x * (p2 - p0 + x * (2 * p0 - 5 * p1 + 4 * p2 - p3 + x * (3 * (p1 - p2) + p3 - p0)));
}
static double tab_bicubic(const double *p, double x, double y) {
    double arr[4];
    for (int i = 0; i < 4; i++) arr[i] = tab_cubic(p[i * 4 + 0], p[i * 4 + 1], p[i * 4 + 2], p[i * 4 + 3], x);
    return tab_cubic(arr[0], arr[1], arr[2], arr[3], y);
}
static double tab_tricubic(const double *p, double x, double y, double z) {
    double arr[4];
    for (int i = 0; i < 4; i++) arr[i] = tab_bicubic(p + i * 16, x, y);
    return tab_cubic(arr[0], arr[1], arr[2], arr[3], z);
}

/* interpolateTricubic, chimesFF.cpp:2370-2440: out = {E, F_ij, F_ik, F_jk} */
static void tab3_value(ora_ff *ff, int t, double rij, double rik, double rjk, double *out) {
    long nrows = ff->t3[t].n;
    const double *tij = ff->t3[t].rij, *tik = ff->t3[t].rik, *tjk = ff->t3[t].rjk;
    const double *ys[4] = {ff->t3[t].e, ff->t3[t].fij, ff->t3[t].fik, ff->t3[t].fjk};
    int size_ik = (int)cbrt((double)nrows);
    int size_ij = size_ik * size_ik;
    double dr = 1 / (tjk[size_ij + size_ik + 1] - tjk[0]);
    int i = (int)((rij - tij[0]) * dr);
    int j = (int)((rik - tik[0]) * dr);
    int k = (int)((rjk - tjk[0]) * dr);
    if (i < 1) i = 1;
    if (j < 1) j = 1;
    if (k < 1) k = 1;
    long ri = (long)i * size_ij + (long)j * size_ik + k, rj = (long)j * size_ik + k, rk = k;
    if (ri >= nrows || rj >= nrows || rk >= nrows) {   /* the reference reads past its vectors here */
        ff->tab_err |= 2;
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    double v[4][64];
    memset(v, 0, sizeof(v));
    for (int di = -1; di <= 2; ++di)
        for (int dj = -1; dj <= 2; ++dj)
            for (int dk = -1; dk <= 2; ++dk) {
                int ti = i + di, tj = j + dj, tk = k + dk;
                if (ti < size_ik && tj < size_ik && tk < size_ik) {
                    long index = (long)size_ij * ti + (long)size_ik * tj + tk;
                    int idx = (di + 1) * 16 + (dj + 1) * 4 + (dk + 1);
                    for (int w = 0; w < 4; w++) v[w][idx] = ys[w][index];
                }
            }
    double xi = (rij - tij[ri]) * dr;
    double yi = (rik - tik[rj]) * dr;
    double zi = (rjk - tjk[rk]) * dr;
    for (int w = 0; w < 4; w++) out[w] = tab_tricubic(v[w], zi, yi, xi);
}

void ora_tab3(void *vh, int t, double rij, double rik, double rjk, double *out) {
    tab3_value(&((ora_handle *)vh)->ff, t, rij, rik, rjk, out);
}

/* compute_3B_tab, chimesFF.cpp:2183-2322 (distance-tensor stress form) */
void ora_compute_3b_tab(void *vh, const double *dx, const double *dr, const int *typ, double *force, double *stress,
                        double *E, double *fscal) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    int nt = ff->ntypes;
    int u = typ[0] * nt * nt + typ[1] * nt + typ[2];
    int t = ff->trip_map[u];
    if (t < 0) return;
    const int *m = &ff->trip_perm[u * 3];
    for (int p = 0; p < 3; p++)
        if (dx[p] >= ff->cut3[(t * 2 + 1) * 3 + m[p]]) return;
    double v[4];
    tab3_value(ff, t, dx[0], dx[1], dx[2], v);
    *E += v[0];
    static const int A[3] = {0, 0, 1}, B[3] = {1, 2, 2};
    for (int p = 0; p < 3; p++) {
        const double fs = v[1 + p], *d = &dr[3 * p];
        force[A[p] * 3 + 0] += fs * d[0]; force[A[p] * 3 + 1] += fs * d[1]; force[A[p] * 3 + 2] += fs * d[2];
        force[B[p] * 3 + 0] -= fs * d[0]; force[B[p] * 3 + 1] -= fs * d[1]; force[B[p] * 3 + 2] -= fs * d[2];
        stress[0] -= fs * (d[0] * d[0]); stress[1] -= fs * (d[0] * d[1]); stress[2] -= fs * (d[0] * d[2]);
        stress[3] -= fs * (d[1] * d[1]); stress[4] -= fs * (d[1] * d[2]); stress[5] -= fs * (d[2] * d[2]);
    }
    if (fscal) { fscal[0] = v[1]; fscal[1] = v[2]; fscal[2] = v[3]; }
}

int ora_tab_flags(void *vh, int *tab2, int *tab3) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    if (tab2) *tab2 = ff->tab2;
    if (tab3) *tab3 = ff->tab3;
    int e = ff->tab_err;
    ff->tab_err = 0;
    return e;
}

static double mag3(const double *a) { double m = 0; for (int i = 0; i < 3; i++) m += a[i] * a[i]; return sqrt(m); }
static double dot3(const double *a, const double *b) { double d = 0; for (int i = 0; i < 3; i++) d += a[i] * b[i]; return d; }
static double angle3(const double *a, const double *b) { double g = dot3(a, b); g /= mag3(a); g /= mag3(b); return acos(g); }

static void set_hmat(const double *ca, const double *cb, const double *cc, double *h, double *hi, int rep) {
    h[0] = ca[0] * (rep + 1); h[3] = ca[1] * (rep + 1); h[6] = ca[2] * (rep + 1);
    h[1] = cb[0] * (rep + 1); h[4] = cb[1] * (rep + 1); h[7] = cb[2] * (rep + 1);
    h[2] = cc[0] * (rep + 1); h[5] = cc[1] * (rep + 1); h[8] = cc[2] * (rep + 1);
    double det = h[0] * (h[4] * h[8] - h[5] * h[7]) - h[1] * (h[3] * h[8] - h[5] * h[6]) + h[2] * (h[3] * h[7] - h[4] * h[6]);
    double t[9];
    t[0] = (h[4] * h[8] - h[5] * h[7]); t[3] = -1 * (h[1] * h[8] - h[2] * h[7]); t[6] = (h[1] * h[5] - h[2] * h[4]);
    t[1] = -1 * (h[3] * h[8] - h[5] * h[6]); t[4] = (h[0] * h[8] - h[2] * h[6]); t[7] = -1 * (h[0] * h[5] - h[2] * h[3]);
    t[2] = (h[3] * h[7] - h[4] * h[6]); t[5] = -1 * (h[0] * h[7] - h[1] * h[6]); t[8] = (h[0] * h[4] - h[1] * h[3]);
    hi[0] = t[0]; hi[3] = t[1]; hi[6] = t[2];
    hi[1] = t[3]; hi[4] = t[4]; hi[7] = t[5];
    hi[2] = t[6]; hi[5] = t[7]; hi[8] = t[8];
    for (int i = 0; i < 9; i++) hi[i] /= det;
}

static void matvec(const double *m, double x, double y, double z, double *o) {
    o[0] = m[0] * x + m[1] * y + m[2] * z;
    o[1] = m[3] * x + m[4] * y + m[5] * z;
    o[2] = m[6] * x + m[7] * y + m[8] * z;
}

static void sys_reserve(ora_sys *s, long n) {
    if (n <= s->cap) return;
    s->cap = n;
    s->x = realloc(s->x, n * sizeof(double)); s->y = realloc(s->y, n * sizeof(double)); s->z = realloc(s->z, n * sizeof(double));
    s->parent = realloc(s->parent, n * sizeof(int)); s->rep_parent = realloc(s->rep_parent, n * sizeof(int));
    s->typ = realloc(s->typ, n * sizeof(int));
}
static void sys_free(ora_sys *s) { free(s->x); free(s->y); free(s->z); free(s->parent); free(s->rep_parent); free(s->typ); }

/* simulation_system::init, serial_chimes_interface.cpp:150-341 */
static void sys_init(ora_sys *s, int n, const int *typ, const double *x, const double *y, const double *z,
                     const double *ca, const double *cb, const double *cc, double max_cut, int small) {
    s->n_atoms = n; s->n_ghost = n; s->n_repl = n;
    double la = mag3(ca), lb = mag3(cb), lc = mag3(cc);
    double mn = la; if (lb < mn) mn = lb; if (lc < mn) mn = lc;
    s->n_replicates = small ? (int)ceil(max_cut / mn) - 1 : 0;
    int nr = s->n_replicates;
    sys_reserve(s, (long)n * (nr + 1) * (nr + 1) * (nr + 1));
    for (int a = 0; a < n; a++) { s->x[a] = x[a]; s->y[a] = y[a]; s->z[a] = z[a]; s->parent[a] = a; s->rep_parent[a] = a; s->typ[a] = typ[a]; }
    set_hmat(ca, cb, cc, s->h, s->hi, 0);
    for (int i = 0; i <= nr; i++)
        for (int j = 0; j <= nr; j++)
            for (int k = 0; k <= nr; k++) {
                if (i == 0 && j == 0 && k == 0) continue;
                for (int a = 0; a < n; a++) {
                    int g = s->n_ghost++; s->n_repl++;
                    double t[3]; matvec(s->hi, s->x[a], s->y[a], s->z[a], t);
                    t[0] += i; t[1] += j; t[2] += k;
                    double o[3]; matvec(s->h, t[0], t[1], t[2], o);
                    s->x[g] = o[0]; s->y[g] = o[1]; s->z[g] = o[2];
                    s->parent[g] = s->n_repl - 1; s->rep_parent[g] = a; s->typ[g] = typ[a];
                }
            }
    s->n_atoms = s->n_repl;
    set_hmat(ca, cb, cc, s->h, s->hi, nr);
    for (int i = 0; i < s->n_atoms; i++) {
        double f[3]; matvec(s->hi, s->x[i], s->y[i], s->z[i], f);
        f[0] -= floor(f[0]); f[1] -= floor(f[1]); f[2] -= floor(f[2]);
        double o[3]; matvec(s->h, f[0], f[1], f[2], o);
        s->x[i] = o[0]; s->y[i] = o[1]; s->z[i] = o[2];
    }
    double A[3] = {s->h[0], s->h[3], s->h[6]}, B[3] = {s->h[1], s->h[4], s->h[7]}, C[3] = {s->h[2], s->h[5], s->h[8]};
    s->la = mag3(A); s->lb = mag3(B); s->lc = mag3(C);
    double al = angle3(B, C), be = angle3(C, A), ga = angle3(A, B);
    double v = 1;
    v += 2 * cos(al) * cos(be) * cos(ga);
    v -= cos(al) * cos(al); v -= cos(be) * cos(be); v -= cos(ga) * cos(ga);
    s->vol = s->la * s->lb * s->lc * sqrt(v);
}

/* simulation_system::reorient, serial_chimes_interface.cpp:342-476 (the
 * extents it also computes are not used by the list build and are omitted) */
static void sys_reorient(ora_sys *s) {
    for (int i = 0; i < s->n_atoms; i++) {
        double f[3]; matvec(s->hi, s->x[i], s->y[i], s->z[i], f);
        s->x[i] = f[0]; s->y[i] = f[1]; s->z[i] = f[2];
    }
    double A[3] = {s->h[0], s->h[3], s->h[6]}, B[3] = {s->h[1], s->h[4], s->h[7]}, C[3] = {s->h[2], s->h[5], s->h[8]};
    double ma = mag3(A);
    double u[3] = {0.0 + A[0] / ma, 0.0 + A[1] / ma, 0.0 + A[2] / ma};
    double cr[3] = {(u[1] * B[2] - u[2] * B[1]), -1 * (u[0] * B[2] - u[2] * B[0]), (u[0] * B[1] - u[1] * B[0])};
    double ta[3] = {mag3(A), 0, 0};
    double tb[3] = {dot3(B, u), mag3(cr), 0};
    double tc[3];
    tc[0] = dot3(C, u);
    tc[1] = (dot3(B, C) - tb[0] * tc[0]) / tb[1];
    tc[2] = sqrt(mag3(C) * mag3(C) - tc[0] * tc[0] - tc[1] * tc[1]);
    set_hmat(ta, tb, tc, s->h, s->hi, 0);
    for (int i = 0; i < s->n_atoms; i++) {
        double o[3]; matvec(s->h, s->x[i], s->y[i], s->z[i], o);
        s->x[i] = o[0]; s->y[i] = o[1]; s->z[i] = o[2];
    }
    double A2[3] = {s->h[0], s->h[3], s->h[6]}, B2[3] = {s->h[1], s->h[4], s->h[7]}, C2[3] = {s->h[2], s->h[5], s->h[8]};
    s->la = mag3(A2); s->lb = mag3(B2); s->lc = mag3(C2);
}

/* simulation_system::build_layered_system, serial_chimes_interface.cpp:477-587 */
static int sys_layers(ora_handle *h, ora_sys *s, double c2, double c3, double c4) {
    double mn = s->la; if (s->lb < mn) mn = s->lb; if (s->lc < mn) mn = s->lc;
    s->n_layers = (int)ceil(c2 * 2.0 / mn + 1);
    int n = s->n_layers;
    double ex = s->la * (2 * n + 1), ey = s->lb * (2 * n + 1), ez = s->lc * (2 * n + 1);
    if (c2 > 0.5 * ex || c2 > 0.5 * ey || c2 > 0.5 * ez) FAIL(h, "maximum 2b cutoff is greater than half at least one box length");
    if (h->ff.o3 > 0 && (c3 > 0.5 * ex || c3 > 0.5 * ey || c3 > 0.5 * ez)) FAIL(h, "maximum 3b cutoff is greater than half at least one box length");
    if (h->ff.o4 > 0 && (c4 > 0.5 * ex || c4 > 0.5 * ey || c4 > 0.5 * ez)) FAIL(h, "maximum 4b cutoff is greater than half at least one box length");
    long side = 2 * n + 1;
    sys_reserve(s, (long)s->n_atoms * side * side * side);
    s->n_ghost = s->n_atoms;
    for (int i = -n; i <= n; i++)
        for (int j = -n; j <= n; j++)
            for (int k = -n; k <= n; k++) {
                if (i == 0 && j == 0 && k == 0) continue;
                for (int a = 0; a < s->n_atoms; a++) {
                    int g = s->n_ghost++;
                    double t[3]; matvec(s->hi, s->x[a], s->y[a], s->z[a], t);
                    t[0] += i; t[1] += j; t[2] += k;
                    double o[3]; matvec(s->h, t[0], t[1], t[2], o);
                    s->x[g] = o[0]; s->y[g] = o[1]; s->z[g] = o[2];
                    s->parent[g] = a; s->typ[g] = s->typ[a];
                }
            }
    return 0;
}

/* simulation_system::get_dist, serial_chimes_interface.h:141-215 */
static double sys_dist(const ora_sys *s, int i, int j, double *r) {
    const double *m = s->hi, *H = s->h;
    double ix = m[0] * s->x[i] + m[1] * s->y[i] + m[2] * s->z[i];
    double iy = m[3] * s->x[i] + m[4] * s->y[i] + m[5] * s->z[i];
    double iz = m[6] * s->x[i] + m[7] * s->y[i] + m[8] * s->z[i];
    double jx = m[0] * s->x[j] + m[1] * s->y[j] + m[2] * s->z[j];
    double jy = m[3] * s->x[j] + m[4] * s->y[j] + m[5] * s->z[j];
    double jz = m[6] * s->x[j] + m[7] * s->y[j] + m[8] * s->z[j];
    double dx = jx - ix, dy = jy - iy, dz = jz - iz;
    double rr[3];
    if (!r) r = rr;
    r[0] = H[0] * dx + H[1] * dy + H[2] * dz;
    r[1] = H[3] * dx + H[4] * dy + H[5] * dz;
    r[2] = H[6] * dx + H[7] * dy + H[8] * dz;
    return sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
}

static void push(int **v, long *n, long *cap, const int *vals, int k) {
    if (*n + k > *cap) { *cap = (*cap ? *cap * 2 : 4096) + k; *v = realloc(*v, *cap * sizeof(int)); }
    memcpy(*v + *n, vals, k * sizeof(int)); *n += k;
}

/* simulation_system::build_neigh_lists, serial_chimes_interface.cpp:588-864.
 * l2 holds (i, ghost) pairs; l2_start[i]..l2_start[i+1] is atom i's list. */
static int build_lists(ora_handle *h, ora_sys *s, double c2, double c3, double c4, long *l2_start) {
    double mx[3] = {-1.0e100, -1.0e100, -1.0e100}, mn[3] = {1.0e100, 1.0e100, 1.0e100};
    for (int i = 0; i < s->n_ghost; i++) {
        if (s->x[i] > mx[0]) mx[0] = s->x[i];
        if (s->y[i] > mx[1]) mx[1] = s->y[i];
        if (s->z[i] > mx[2]) mx[2] = s->z[i];
        if (s->x[i] < mn[0]) mn[0] = s->x[i];
        if (s->y[i] < mn[1]) mn[1] = s->y[i];
        if (s->z[i] < mn[2]) mn[2] = s->z[i];
    }
    double sd = c2; if (c3 > sd) sd = c3; if (c4 > sd) sd = c4;
    int nbx = (int)ceil((mx[0] - mn[0]) / sd), nby = (int)ceil((mx[1] - mn[1]) / sd), nbz = (int)ceil((mx[2] - mn[2]) / sd);
    long tb = (long)nbx * nby * nbz;
    long *bstart = calloc(tb + 1, sizeof(long));
    int *bid = malloc(s->n_ghost * sizeof(int));
    for (int i = 0; i < s->n_ghost; i++) {
        int bx = (int)floor((s->x[i] - mn[0]) / sd), by = (int)floor((s->y[i] - mn[1]) / sd), bz = (int)floor((s->z[i] - mn[2]) / sd);
        if (bx < 0 || by < 0 || bz < 0) { free(bstart); free(bid); FAIL(h, "negative bin computed"); }
        long ib = bx + (long)by * nbx + (long)bz * nbx * nby;
        if (ib >= tb) { free(bstart); free(bid); FAIL(h, "ibin out of range"); }
        bid[i] = (int)ib; bstart[ib + 1]++;
    }
    for (long b = 0; b < tb; b++) bstart[b + 1] += bstart[b];
    long *fill = malloc(tb * sizeof(long)); memcpy(fill, bstart, tb * sizeof(long));
    int *bins = malloc(s->n_ghost * sizeof(int));
    for (int i = 0; i < s->n_ghost; i++) bins[fill[bid[i]]++] = i;
    free(fill); free(bid);
    h->n2 = h->n3 = h->n4 = 0;
    for (int ai = 0; ai < s->n_atoms; ai++) {
        l2_start[ai] = h->n2 / 2;
        int bx = (int)floor((s->x[ai] - mn[0]) / sd), by = (int)floor((s->y[ai] - mn[1]) / sd), bz = (int)floor((s->z[ai] - mn[2]) / sd);
        if (bx < 1 || by < 1 || bz < 1) { free(bstart); free(bins); FAIL(h, "bad bin computed"); }
        for (int i = bx - 1; i <= bx + 1; i++)
            for (int j = by - 1; j <= by + 1; j++)
                for (int k = bz - 1; k <= bz + 1; k++) {
                    long ib = i + (long)j * nbx + (long)k * nbx * nby;
                    if (ib >= tb) { free(bstart); free(bins); FAIL(h, "binning index out of range"); }
                    for (long q = bstart[ib]; q < bstart[ib + 1]; q++) {
                        int ajj = bins[q];
                        if (ajj == ai) continue;
                        if (ai <= s->parent[ajj] && sys_dist(s, ai, ajj, NULL) < sd) {
                            int v[2] = {ai, ajj}; push(&h->l2, &h->n2, &h->cap2, v, 2);
                        }
                    }
                }
    }
    l2_start[s->n_atoms] = h->n2 / 2;
    free(bstart); free(bins);
    if (h->ff.o3 == 0 && h->ff.o4 == 0) { h->n2 /= 2; return 0; }
    for (int i = 0; i < s->n_atoms; i++) {
        long b0 = l2_start[i], b1 = l2_start[i + 1];
        for (long j = b0; j < b1; j++) {
            int v3 = 1, v4 = 1;
            int jj = h->l2[2 * j + 1];
            double dij = sys_dist(s, i, jj, NULL);
            if (dij >= c3) v3 = 0;
            if (dij >= c4) v4 = 0;
            if (!v3 && !v4) continue;
            for (long k = b0; k < b1; k++) {
                int kk = h->l2[2 * k + 1];
                if (jj == kk) continue;
                if (s->parent[jj] > s->parent[kk]) continue;
                double dik = sys_dist(s, i, kk, NULL);
                if (dik >= c3) v3 = 0;
                if (dik >= c4) v4 = 0;
                double djk = sys_dist(s, jj, kk, NULL);
                if (djk >= c3) v3 = 0;
                if (djk >= c4) v4 = 0;
                if (!v3 && !v4) {
                    if (dij < c3) v3 = 1;
                    if (dij < c4) v4 = 1;
                    continue;
                }
                if (v3) { int v[3] = {i, jj, kk}; push(&h->l3, &h->n3, &h->cap3, v, 3); }
                if (h->ff.o4 == 0) continue;
                if (!v4) { if (dij < c4) v4 = 1; continue; }
                for (long l = b0; l < b1; l++) {
                    int ll = h->l2[2 * l + 1];
                    if (jj == ll || kk == ll) continue;
                    if (s->parent[jj] > s->parent[ll]) continue;
                    if (s->parent[kk] > s->parent[ll]) continue;
                    if (sys_dist(s, i, ll, NULL) >= c4) continue;
                    if (sys_dist(s, jj, ll, NULL) >= c4) continue;
                    if (sys_dist(s, kk, ll, NULL) >= c4) continue;
                    if (v4) { int v[4] = {i, jj, kk, ll}; push(&h->l4, &h->n4, &h->cap4, v, 4); }
                }
            }
        }
    }
    h->n2 /= 2; h->n3 /= 3; h->n4 /= 4;
    return 0;
}

/* ------------------------------------------------------------------ */
/* public entry points (ctypes)                                        */
/* ------------------------------------------------------------------ */
void *ora_load(const char *path, char *err, int errlen) {
    ora_handle *h = calloc(1, sizeof(ora_handle));
    if (parse(h, path)) {
        if (err && errlen > 0) { strncpy(err, h->err, errlen - 1); err[errlen - 1] = 0; }
        free(h); return NULL;
    }
    return h;
}

void ora_free(void *vh) {
    ora_handle *h = vh; if (!h) return;
    free(h->l2); free(h->l3); free(h->l4);
    free(h->lmp_l3); free(h->lmp_l4);
    for (int b = 0; b < 3; b++) { free(h->fp_d[b]); free(h->fp_t[b]); }
    free(h);  /* parameter tables are left to process exit: test-only object */
}

const char *ora_error(void *vh) { return ((ora_handle *)vh)->err; }

void ora_info(void *vh, int *orders, int *ntypes, double *maxcuts) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    orders[0] = ff->o2; orders[1] = ff->o3; orders[2] = ff->o4; *ntypes = ff->ntypes;
    maxcuts[0] = max_cut2(ff); maxcuts[1] = max_cutn(ff, 3); maxcuts[2] = max_cutn(ff, 4);
}

int ora_type_index(void *vh, const char *name) {
    ora_ff *ff = &((ora_handle *)vh)->ff;
    for (int i = 0; i < ff->ntypes; i++) if (!strcmp(ff->atm[i], name)) return i;
    return -1;
}

int ora_badness(void *vh) { return ((ora_handle *)vh)->ff.badness; }

/* serial_chimes_interface::calculate.  energy/force accumulate into the
 * caller's values; stress[9] is overwritten.  Returns 0 or -1 (see ora_error). */
int ora_calculate(void *vh, int n, const double *x, const double *y, const double *z, const int *typ,
                  const double *ca, const double *cb, const double *cc, int small,
                  double *energy, double *fx, double *fy, double *fz, double *stress) {
    ora_handle *h = vh; ora_ff *ff = &h->ff;
    double c2 = max_cut2(ff), c3 = max_cutn(ff, 3), c4 = max_cutn(ff, 4);
    double st[6] = {0, 0, 0, 0, 0, 0};
    ora_sys S = {0}, N = {0};
    sys_init(&S, n, typ, x, y, z, ca, cb, cc, c2, small);
    if (sys_layers(h, &S, c2, c3, c4)) { sys_free(&S); return -1; }
    int body = 2 + (ff->o3 > 0) + (ff->o4 > 0);
    if (body > S.n_ghost) { sys_free(&S); FAIL(h, "layered system contains too few atoms"); }
    sys_init(&N, n, typ, x, y, z, ca, cb, cc, c2, small);
    sys_reorient(&N);
    if (sys_layers(h, &N, c2, c3, c4)) { sys_free(&S); sys_free(&N); return -1; }
    long *l2s = malloc((N.n_atoms + 1) * sizeof(long));
    if (build_lists(h, &N, c2, c3, c4, l2s)) { free(l2s); sys_free(&S); sys_free(&N); return -1; }
    double *E = energy;
    double f2[6], f3[9], f4[12], dr[18], dx[6];
    for (int i = 0; i < S.n_atoms; i++) {
        ora_compute_1b(h, S.typ[i], E);
        for (long q = l2s[i]; q < l2s[i + 1]; q++) {
            int jj = h->l2[2 * q + 1];
            double d = sys_dist(&S, i, jj, dr);
            memset(f2, 0, sizeof(f2));
            ora_compute_2b(h, d, dr, S.typ[i], S.typ[jj], f2, st, E);
            int a = S.rep_parent[i], b = S.rep_parent[S.parent[jj]];
            fx[a] += f2[0]; fy[a] += f2[1]; fz[a] += f2[2];
            fx[b] += f2[3]; fy[b] += f2[4]; fz[b] += f2[5];
        }
    }
    if (ff->o3 > 0)
        for (long q = 0; q < h->n3; q++) {
            int id[3] = {h->l3[3 * q], h->l3[3 * q + 1], h->l3[3 * q + 2]};
            dx[0] = sys_dist(&S, id[0], id[1], &dr[0]);
            dx[1] = sys_dist(&S, id[0], id[2], &dr[3]);
            dx[2] = sys_dist(&S, id[1], id[2], &dr[6]);
            int t[3] = {S.typ[id[0]], S.typ[id[1]], S.typ[id[2]]};
            memset(f3, 0, sizeof(f3));
            ora_compute_3b(h, dx, dr, t, f3, st, E);
            for (int a = 0; a < 3; a++) {
                int o = S.rep_parent[S.parent[id[a]]];
                fx[o] += f3[3 * a]; fy[o] += f3[3 * a + 1]; fz[o] += f3[3 * a + 2];
            }
        }
    if (ff->o4 > 0)
        for (long q = 0; q < h->n4; q++) {
            int id[4] = {h->l4[4 * q], h->l4[4 * q + 1], h->l4[4 * q + 2], h->l4[4 * q + 3]};
            static const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {1, 2, 3, 2, 3, 3};
            for (int p = 0; p < 6; p++) dx[p] = sys_dist(&S, id[A[p]], id[B[p]], &dr[3 * p]);
            int t[4] = {S.typ[id[0]], S.typ[id[1]], S.typ[id[2]], S.typ[id[3]]};
            memset(f4, 0, sizeof(f4));
            ora_compute_4b(h, dx, dr, t, f4, st, E);
            for (int a = 0; a < 4; a++) {
                int o = S.rep_parent[S.parent[id[a]]];
                fx[o] += f4[3 * a]; fy[o] += f4[3 * a + 1]; fz[o] += f4[3 * a + 2];
            }
        }
    *E /= pow(S.n_replicates + 1.0, 3.0);
    stress[0] = st[0]; stress[1] = st[1]; stress[2] = st[2];
    stress[3] = st[1]; stress[4] = st[3]; stress[5] = st[4];
    stress[6] = st[2]; stress[7] = st[4]; stress[8] = st[5];
    for (int k = 0; k < 9; k++) stress[k] /= S.vol;
    free(l2s); sys_free(&S); sys_free(&N);
    return 0;
}

void ora_list_sizes(void *vh, long *n2, long *n3, long *n4) {
    ora_handle *h = vh; *n2 = h->n2; *n3 = h->n3; *n4 = h->n4;
}

void ora_get_lists(void *vh, int *l2, int *l3, int *l4) {
    ora_handle *h = vh;
    if (l2) memcpy(l2, h->l2, h->n2 * 2 * sizeof(int));
    if (l3) memcpy(l3, h->l3, h->n3 * 3 * sizeof(int));
    if (l4) memcpy(l4, h->l4, h->n4 * 4 * sizeof(int));
}

/* ------------------------------------------------------------------------
 * LAMMPS pair style (etc/lmp/src/pair_chimes.cpp): build_mb_neighlists
 * (:321-478) and compute (:480-884) over a full neighbour list with ghost
 * atoms, newton on (forces on ghosts are kept for the reverse communication).
 * x[nall*3], typ[nall] (ChIMES type index), tag[nall]; ilist[inum];
 * numneigh[inum] and the concatenated lists neigh[] in ilist order.
 * Accumulates f[nall*3], *energy and virial[6] (LAMMPS order xx yy zz xy xz
 * yz, the stensor mapping of Pair::ev_tally_mb, etc/lmp/etc/pair.cpp).
 * rebuild = 0 reuses the previous cluster lists (the reference rebuilds them
 * only when neighbor->ago == 0).
 * ---------------------------------------------------------------------- */
static double lmp_dist(const double *x, int i, int j, double *dr) {   /* PairCHIMES::get_dist, :303-312 */
    double d[3];
    d[0] = x[3 * j + 0] - x[3 * i + 0];
    d[1] = x[3 * j + 1] - x[3 * i + 1];
    d[2] = x[3 * j + 2] - x[3 * i + 2];
    if (dr) { dr[0] = d[0]; dr[1] = d[1]; dr[2] = d[2]; }
    return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

static int push_cluster(int **buf, long *n, long *cap, const int *v, int k) {
    if (*n >= *cap) {
        long nc = *cap ? 2 * *cap : 1024;
        int *nb = realloc(*buf, (size_t)nc * k * sizeof(int));
        if (!nb) return -1;
        *buf = nb; *cap = nc;
    }
    memcpy(*buf + (*n) * k, v, k * sizeof(int));
    (*n)++;
    return 0;
}

/* Pair::ev_tally_mb (etc/lmp/etc/pair.cpp): an n-atom interaction's energy and
 * stress shared equally by its atoms (eatom, vatom in LAMMPS order) */
static void lmp_tally(const int *atoms, int n, double e, const double *st, double *eatom, double *vatom) {
    for (int a = 0; a < n; a++) {
        if (eatom) eatom[atoms[a]] += e / n;
        if (vatom && n > 1) {
            double *v = &vatom[6 * atoms[a]];
            v[0] += st[0] / n; v[1] += st[3] / n; v[2] += st[5] / n;
            v[3] += st[1] / n; v[4] += st[2] / n; v[5] += st[4] / n;
        }
    }
}

/* one fingerprint record: the cluster's distances and type indices (what
 * compute_nB appends to clusters_nb in the FINGERPRINT build) */
static int fp_push(ora_handle *h, int body, const double *d, const int *t) {
    const int b = body - 2, P = body * (body - 1) / 2;
    if (h->fp_n[b] >= h->fp_cap[b]) {
        long nc = h->fp_cap[b] ? 2 * h->fp_cap[b] : 1024;
        double *nd = realloc(h->fp_d[b], (size_t)nc * P * sizeof(double));
        if (!nd) return -1;
        h->fp_d[b] = nd;
        int *nt = realloc(h->fp_t[b], (size_t)nc * body * sizeof(int));
        if (!nt) return -1;
        h->fp_t[b] = nt;
        h->fp_cap[b] = nc;
    }
    memcpy(h->fp_d[b] + h->fp_n[b] * P, d, P * sizeof(double));
    memcpy(h->fp_t[b] + h->fp_n[b] * body, t, body * sizeof(int));
    h->fp_n[b]++;
    return 0;
}

/* cutoff checks of compute_nB: 1 when the cluster is evaluated (and recorded) */
static int fp_passes(ora_ff *ff, int body, const double *dx, const int *t) {
    int nt = ff->ntypes;
    if (body == 2) return dx[0] < ff->rout[ff->pair_map[t[0] * nt + t[1]]];
    int u = 0;
    for (int k = 0; k < body; k++) u = u * nt + t[k];
    if (body == 3) {
        int c = ff->trip_map[u];
        if (c < 0) return 0;
        for (int p = 0; p < 3; p++) if (dx[p] >= ff->cut3[(c * 2 + 1) * 3 + ff->trip_perm[u * 3 + p]]) return 0;
        return 1;
    }
    int c = ff->quad_map[u];
    if (c < 0) return 0;
    for (int p = 0; p < 6; p++) if (dx[p] >= ff->cut4[(c * 2 + 1) * 6 + ff->quad_perm[u * 6 + p]]) return 0;
    return 1;
}

void ora_lammps_fp(void *vh, int on) { ((ora_handle *)vh)->lmp_fp = on; }

void ora_lammps_fp_sizes(void *vh, long *n) {
    ora_handle *h = vh;
    for (int b = 0; b < 3; b++) n[b] = h->fp_n[b];
}

void ora_lammps_fp_records(void *vh, int body, double *d, int *t) {
    ora_handle *h = vh;
    const int b = body - 2, P = body * (body - 1) / 2;
    if (h->fp_n[b]) {
        memcpy(d, h->fp_d[b], (size_t)h->fp_n[b] * P * sizeof(double));
        memcpy(t, h->fp_t[b], (size_t)h->fp_n[b] * body * sizeof(int));
    }
}

int ora_lammps_compute(void *vh, int nall, const double *x, const int *typ, const long long *tag, int inum,
                       const int *ilist, const int *numneigh, const int *neigh, double skin, int rebuild, double *f,
                       double *energy, double *virial, double *eatom, double *vatom) {
    ora_handle *h = vh;
    ora_ff *ff = &h->ff;
    (void)nall;
    long *off = malloc((size_t)(inum + 1) * sizeof(long));
    if (!off) FAIL(h, "out of memory");
    off[0] = 0;
    for (int ii = 0; ii < inum; ii++) off[ii + 1] = off[ii] + numneigh[ii];
    double c3 = 0.0, c4 = 0.0;   /* chimesFF::max_cutoff_3B/4B: 0 when the order is 0 */
    if (ff->o3 > 0) c3 = max_cutn(ff, 3);
    if (ff->o4 > 0) c4 = max_cutn(ff, 4);
    const double c3p = c3 + skin, c4p = c4 + skin;   /* maxcut_nb + neighbor->skin */
    h->fp_n[0] = h->fp_n[1] = h->fp_n[2] = 0;
    if (rebuild || !h->lmp_built) {
        h->lmp_n3 = h->lmp_n4 = 0;
        h->lmp_built = 1;
        if (ff->o3 > 0 || ff->o4 > 0)
            for (int ii = 0; ii < inum; ii++) {
                const int i = ilist[ii];
                for (long jj = off[ii]; jj < off[ii + 1]; jj++) {
                    const int j = neigh[jj];
                    if (j == i || tag[j] < tag[i]) continue;
                    const double dij = lmp_dist(x, i, j, NULL);
                    if (dij >= c3p && dij >= c4p) continue;
                    for (long kk = off[ii]; kk < off[ii + 1]; kk++) {
                        const int k = neigh[kk];
                        if (k == i || k == j) continue;
                        if (tag[k] < tag[i] || tag[k] < tag[j]) continue;
                        const double dik = lmp_dist(x, i, k, NULL);
                        if (dik >= c3p && dik >= c4p) continue;
                        const double djk = lmp_dist(x, j, k, NULL);
                        if (ff->o3 > 0 && dij < c3p && dik < c3p && djk < c3p) {
                            const int v[3] = {i, j, k};
                            if (push_cluster(&h->lmp_l3, &h->lmp_n3, &h->lmp_c3, v, 3)) { free(off); FAIL(h, "out of memory"); }
                        }
                        if (dij >= c4p || dik >= c4p || djk >= c4p) continue;
                        if (ff->o4 == 0) continue;
                        for (long ll = off[ii]; ll < off[ii + 1]; ll++) {
                            const int l = neigh[ll];
                            if (l == i || l == j || l == k) continue;
                            if (tag[l] < tag[i] || tag[l] < tag[j] || tag[l] < tag[k]) continue;
                            if (lmp_dist(x, i, l, NULL) >= c4p) continue;
                            if (lmp_dist(x, j, l, NULL) >= c4p) continue;
                            if (lmp_dist(x, k, l, NULL) >= c4p) continue;
                            const int v[4] = {i, j, k, l};
                            if (push_cluster(&h->lmp_l4, &h->lmp_n4, &h->lmp_c4, v, 4)) { free(off); FAIL(h, "out of memory"); }
                        }
                    }
                }
            }
    }
    double st[6], f2[6], f3[9], f4[12], dr[18], dx[6];
    /* 1- and 2-body over the current neighbour list (:572-655) */
    for (int ii = 0; ii < inum; ii++) {
        const int i = ilist[ii];
        double e = 0.0;
        ora_compute_1b(h, typ[i], &e);
        *energy += e;
        lmp_tally(&i, 1, e, NULL, eatom, vatom);
        for (long jj = off[ii]; jj < off[ii + 1]; jj++) {
            const int j = neigh[jj];
            if (tag[j] <= tag[i]) continue;
            const double d = lmp_dist(x, i, j, dr);
            memset(f2, 0, sizeof(f2)); memset(st, 0, sizeof(st));
            e = 0.0;
            if (ff->tab2) ora_compute_2b_tab(h, d, dr, typ[i], typ[j], f2, st, &e, NULL);   /* :620-622 */
            else ora_compute_2b(h, d, dr, typ[i], typ[j], f2, st, &e);
            for (int c = 0; c < 3; c++) { f[3 * i + c] += f2[c]; f[3 * j + c] += f2[3 + c]; }
            *energy += e;
            const int pr[2] = {i, j};
            if (h->lmp_fp && i < j) {   /* valid_order = (i < j) (:626) */
                const int tt[2] = {typ[i], typ[j]};
                if (fp_passes(ff, 2, &d, tt) && fp_push(h, 2, &d, tt)) { free(off); FAIL(h, "out of memory"); }
            }
            lmp_tally(pr, 2, e, st, eatom, vatom);
            virial[0] += st[0]; virial[1] += st[3]; virial[2] += st[5];
            virial[3] += st[1]; virial[4] += st[2]; virial[5] += st[4];
        }
    }
    static const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {1, 2, 3, 2, 3, 3};
    if (ff->o3 > 0)   /* :660-735 */
        for (long q = 0; q < h->lmp_n3; q++) {
            const int *id = &h->lmp_l3[3 * q];
            static const int A3[3] = {0, 0, 1}, B3[3] = {1, 2, 2};   /* ij, ik, jk */
            for (int p = 0; p < 3; p++) dx[p] = lmp_dist(x, id[A3[p]], id[B3[p]], &dr[3 * p]);
            const int t[3] = {typ[id[0]], typ[id[1]], typ[id[2]]};
            memset(f3, 0, sizeof(f3)); memset(st, 0, sizeof(st));
            double e = 0.0;
            if (ff->tab3) ora_compute_3b_tab(h, dx, dr, t, f3, st, &e, NULL);   /* :697-699 */
            else ora_compute_3b(h, dx, dr, t, f3, st, &e);
            for (int a = 0; a < 3; a++)
                for (int c = 0; c < 3; c++) f[3 * id[a] + c] += f3[3 * a + c];
            if (h->lmp_fp && tag[id[0]] < tag[id[1]] && tag[id[0]] < tag[id[2]] && tag[id[1]] < tag[id[2]] &&
                fp_passes(ff, 3, dx, t) && fp_push(h, 3, dx, t)) { free(off); FAIL(h, "out of memory"); }
            *energy += e;
            lmp_tally(id, 3, e, st, eatom, vatom);
            virial[0] += st[0]; virial[1] += st[3]; virial[2] += st[5];
            virial[3] += st[1]; virial[4] += st[2]; virial[5] += st[4];
        }
    if (ff->o4 > 0)   /* :740-820 */
        for (long q = 0; q < h->lmp_n4; q++) {
            const int *id = &h->lmp_l4[4 * q];
            for (int p = 0; p < 6; p++) dx[p] = lmp_dist(x, id[A[p]], id[B[p]], &dr[3 * p]);
            const int t[4] = {typ[id[0]], typ[id[1]], typ[id[2]], typ[id[3]]};
            memset(f4, 0, sizeof(f4)); memset(st, 0, sizeof(st));
            double e = 0.0;
            ora_compute_4b(h, dx, dr, t, f4, st, &e);
            for (int a = 0; a < 4; a++)
                for (int c = 0; c < 3; c++) f[3 * id[a] + c] += f4[3 * a + c];
            if (h->lmp_fp && tag[id[0]] < tag[id[1]] && tag[id[1]] < tag[id[2]] && tag[id[2]] < tag[id[3]] &&
                fp_passes(ff, 4, dx, t) && fp_push(h, 4, dx, t)) { free(off); FAIL(h, "out of memory"); }
            *energy += e;
            lmp_tally(id, 4, e, st, eatom, vatom);
            virial[0] += st[0]; virial[1] += st[3]; virial[2] += st[5];
            virial[3] += st[1]; virial[4] += st[2]; virial[5] += st[4];
        }
    free(off);
    if (ff->tab_err) {
        int e = ff->tab_err;
        ff->tab_err = 0;
        FAIL(h, "%s", (e & 1) ? "Distance is outside the tabulated range" : "3-body distance past the tabulated grid");
    }
    return 0;
}

void ora_lammps_sizes(void *vh, long *n3, long *n4) { ora_handle *h = vh; *n3 = h->lmp_n3; *n4 = h->lmp_n4; }

void ora_lammps_lists(void *vh, int *l3, int *l4) {
    ora_handle *h = vh;
    if (l3 && h->lmp_n3) memcpy(l3, h->lmp_l3, h->lmp_n3 * 3 * sizeof(int));
    if (l4 && h->lmp_n4) memcpy(l4, h->lmp_l4, h->lmp_n4 * 4 * sizeof(int));
}

/* ------------------------------------------------------------------ */
/* cluster-distance histograms (chimesFF/src/FP/multi_calc_histogram.cpp,
 * one process)                                                         */
/* ------------------------------------------------------------------ */
/* transform (multi_calc_histogram.cpp:112-123): the Morse map of the cluster's own cutoffs */
static double fp_transform(double rcin, double rcout, double lambda, double rij) {
    double x_min = exp(-1 * rcin / lambda);
    double x_max = exp(-1 * rcout / lambda);
    double x_avg = 0.5 * (x_max + x_min);
    double x_diff = 0.5 * (x_max - x_min);
    x_diff *= -1.0;
    return (exp(-1 * rij / lambda) - x_avg) / x_diff;
}

static int cmp_dbl(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* read_flat_clusters (:26-107): transformed edge lengths of each record, ascending */
static int fp_edges(ora_handle *h, int body, long n, const double *d, const int *t, double *out) {
    ora_ff *ff = &h->ff;
    int nt = ff->ntypes, P = body * (body - 1) / 2;
    static const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {1, 2, 3, 2, 3, 3};
    static const int A3[3] = {0, 0, 1}, B3[3] = {1, 2, 2};
    for (long c = 0; c < n; c++) {
        const int *ty = t + c * body;
        for (int k = 0; k < body; k++)
            if (ty[k] < 0 || ty[k] >= nt) FAIL(h, "fingerprint record %ld: type index out of range", c);
        double *e = out + c * P;
        if (body == 2) {
            int p = ff->pair_map[ty[0] * nt + ty[1]];
            e[0] = fp_transform(ff->rin[p], ff->rout[p], ff->lam[p], d[c]);
        } else {
            int u = 0;
            for (int k = 0; k < body; k++) u = u * nt + ty[k];
            int tt = body == 3 ? ff->trip_map[u] : ff->quad_map[u];
            if (tt < 0) FAIL(h, "fingerprint record %ld: excluded cluster type", c);
            const int *m = body == 3 ? &ff->trip_perm[u * 3] : &ff->quad_perm[u * 6];
            const double *cut = body == 3 ? ff->cut3 : ff->cut4;
            for (int p = 0; p < P; p++) {
                int a = body == 3 ? A3[p] : A[p], b = body == 3 ? B3[p] : B[p];
                double lam = ff->lam[ff->pair_map[ty[a] * nt + ty[b]]];
                e[p] = fp_transform(cut[(tt * 2 + 0) * P + m[p]], cut[(tt * 2 + 1) * P + m[p]], lam, d[c * P + p]);
            }
        }
        qsort(e, P, sizeof(double), cmp_dbl);
    }
    return 0;
}

/* gen_flat_hists (:240-480) with one process: counts[nbin], *nsamples.  The
 * composition term is zero there (it reads the zero-filled front of vectors
 * that were sized before being appended to), so the distance is the Euclidean
 * distance of the sorted edge vectors.  Returns -1 with a message when a
 * distance falls past the last bin (the reference exits, or writes past its
 * histogram when it falls exactly one bin past). */
int ora_fp_histogram(void *vh, int body, long n1, const double *d1, const int *t1, long n2, const double *d2,
                     const int *t2, int same, int nbin, long long *counts, long long *nsamples) {
    ora_handle *h = vh;
    int P = body * (body - 1) / 2;
    double maxd = body == 2 ? 3.0 : (body == 3 ? sqrt(12.0) + 1.0 : sqrt(24.0) + 1.0);
    double binw = maxd / nbin;
    double *e1 = malloc((size_t)(n1 > 0 ? n1 : 1) * P * sizeof(double));
    double *e2 = malloc((size_t)(n2 > 0 ? n2 : 1) * P * sizeof(double));
    if (!e1 || !e2) { free(e1); free(e2); FAIL(h, "out of memory"); }
    if (fp_edges(h, body, n1, d1, t1, e1) || fp_edges(h, body, n2, d2, t2, e2)) { free(e1); free(e2); return -1; }
    memset(counts, 0, (size_t)nbin * sizeof(long long));
    *nsamples = 0;
    /* divide_task with one process: tasks 0..n1-1, and nothing at all unless
     * end - start > 0 (a single cluster in the first set counts nothing) */
    long start = n1 > 0 ? 0 : 1, end = n1 - 1;
    int bad = 0;
    if (end - start > 0)
        for (long i = start; i <= end; i++)
            for (long j = same ? i + 1 : 0; j < n2; j++) {
                double ds = 0;
                for (int k = 0; k < P; k++) ds += pow(e1[i * P + k] - e2[j * P + k], 2.0);
                double dist = sqrt(ds) + fabs(0.0 - 0.0);
                int bin = (int)floor(dist / binw);
                if (dist == maxd) bin = bin - 1;
                if (bin >= nbin || bin < 0) { bad = 1; continue; }
                counts[bin] += 1;
                *nsamples += 1;
            }
    free(e1); free(e2);
    if (bad) FAIL(h, "ERROR: computed bin larger than nbins");
    return 0;
}
