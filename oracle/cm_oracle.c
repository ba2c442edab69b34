/*
 * cm_oracle.c -- CPU restatement of ComplexMixtures.jl's per-frame MDDF path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the GPU
 * engine.  Only the test-suite, the smoke check and the CPU-baseline leg of the
 * benchmark load it; the product never links, calls or falls back to it.
 *
 * Everything here is plain FP64 scalar C, compiled with -ffp-contract=off so
 * that no multiply-add is fused.  Each function cites the reference code it
 * restates (paths are relative to the ComplexMixtures.jl repository):
 *
 *   frame loop, random branch, list save/restore   src/mddf.jl:361-429
 *   coordination-number frame                       src/mddf.jl:438-471
 *   bulk test and bulk-index list                    src/mddf.jl:55-57, 406-415
 *   solvent randomisation                            src/mddf.jl:65-88
 *   rigid-body move, Euler matrix                    src/rigid_body.jl:35-57, 73-80, 107-137
 *   argmin merge with tie rule                       src/minimum_distances.jl:30-39
 *   per-pair list update (cross / auto)              src/minimum_distances.jl:81-120
 *   cutoff used for pairs                            src/minimum_distances.jl:157-176 (:166)
 *   counters, groups, atom types                     src/update_counters.jl:9, 22-87
 *   histogram bin                                    src/results.jl:28
 *   cell volume                                      src/mddf.jl:350-352
 *
 * The pair search of the reference lives in CellListMap.jl 0.10.1 (Project.toml
 * compat, not vendored).  Its contract is restated as: a pair (i, j) is reported
 * iff the squared minimum-image distance between atoms i and j is <= cutoff^2.
 * Two backends produce the same pairs with the same FP64 distance:
 *   backend 0 ("brute"): every solute atom against every solvent atom;
 *   backend 1 ("cells"): a cell list over solvent molecule anchors selects the
 *                        candidate molecules of each solute atom, like the
 *                        x-against-y-cell-list traversal of CellListMap.
 * In both, the squared distance of a pair is the minimum over lattice images of
 * |y - x - H n|^2, with n searched around rint(Hinv (y - x)); the pair is
 * reported iff it is <= cutoff^2 and its distance is the square root.
 *
 * Random numbers.  The reference draws placements from Xoroshiro128Plus /
 * StableRNG streams (src/rigid_body.jl:8-19), which depend on the number of
 * threads.  Here the placements come from a seeded counter-based stream that
 * the GPU engine reproduces bit for bit; the distributions are those of the
 * reference (uniform bulk molecule, uniform centre in the cell, three Euler
 * angles uniform in [0, 2pi)), the stream is not.  The stream:
 *   mix64(z)   = SplitMix64 output function (Steele, Lea, Flood 2014)
 *   key(tag,a,b,c) = mix64(mix64(mix64(mix64(seed + G*(tag+1)) ^ a) ^ b) ^ c)
 *   next(s)    : s += G; return mix64(s)            G = 0x9E3779B97F4A7C15
 *   uniform    : (next >> 11) * 2^-53
 *   index(n)   : high 64 bits of next * n
 *   angle      : (u, v) = (2U-1, 2U-1) until 0 < u^2+v^2 < 1 (at most 64 tries);
 *                cos = (u*u - v*v)/r2, sin = (u*v + u*v)/r2.
 * Per frame, stream key(TAG_REF, frame, 0, 0) draws the n_random_samples
 * reference solute molecules.  Per (frame, solute s, repetition r, slot k),
 * stream key(TAG_SLOT, frame, s, r<<32|k) draws, in order: the bulk pick, the
 * three fractional coordinates of the new centre, and the angles beta, gamma,
 * theta.
 *
 * Counters are int64 in half units (2 per unit of frame weight) so that the
 * w/2 increments of the self-MDDF (src/update_counters.jl:276-277) are exact.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2

typedef struct {
    int32_t ms, aps, mv, apv;   /* solute / solvent molecules and atoms per molecule */
    int32_t autocorrelation;    /* 1: solute and solvent are the same selection */
    int32_t irefatom;           /* 1-based reference atom of the solvent molecule */
    double cutoff, binstep, dbulk;
    int32_t usecutoff;
    int32_t nbins;
    int32_t n_random_samples;
    int32_t coordination_number_only;
    uint64_t seed;
    /* solute-side credits: CSR over the aps atoms of a solute molecule (local index) */
    int32_t solute_ngroups;
    const int64_t *solute_grp_off;
    const int32_t *solute_grp;
    /* solvent-side credits: CSR over all solvent atoms (global index in the selection) */
    int32_t solvent_ngroups;
    const int64_t *solvent_grp_off;
    const int32_t *solvent_grp;
    int32_t backend;            /* 0 brute, 1 cells */
} orc_desc;

typedef struct {
    int64_t *md, *md_rand, *rdf, *rdf_rand;   /* [nbins] */
    int64_t *gs, *gs_rand;                    /* [solute_ngroups * nbins] */
    int64_t *gv, *gv_rand;                    /* [solvent_ngroups * nbins] (unused in self mode) */
    int64_t pairs_real, pairs_rand;           /* atom pairs within cutoff (work measure) */
} orc_counts;

/* ------------------------------------------------------------------ stream */
#define ORC_G 0x9E3779B97F4A7C15ULL
#define TAG_REF 1ULL
#define TAG_SLOT 2ULL

static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline uint64_t stream_key(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b, uint64_t c) {
    uint64_t k = mix64(seed + ORC_G * (tag + 1ULL));
    k = mix64(k ^ a);
    k = mix64(k ^ b);
    k = mix64(k ^ c);
    return k;
}
static inline uint64_t next64(uint64_t *s) { *s += ORC_G; return mix64(*s); }
static inline double uniform01(uint64_t *s) { return (double)(next64(s) >> 11) * 0x1.0p-53; }
static inline uint64_t index_below(uint64_t *s, uint64_t n) {
    return (uint64_t)(((unsigned __int128)next64(s) * (unsigned __int128)n) >> 64);
}
static void angle_cs(uint64_t *s, double *c, double *sn) {
    for (int t = 0; t < 64; ++t) {
        double u = 2.0 * uniform01(s) - 1.0;
        double v = 2.0 * uniform01(s) - 1.0;
        double uu = u * u, vv = v * v;
        double r2 = uu + vv;
        if (r2 > 0.0 && r2 < 1.0) {
            double uv = u * v;
            *c = (uu - vv) / r2;
            *sn = (uv + uv) / r2;
            return;
        }
    }
    *c = 1.0;
    *sn = 0.0;
}

/* Exposed for tests: the first `n` raw draws of a stream. */
void orc_stream_draws(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b, uint64_t c, int32_t n, uint64_t *out) {
    uint64_t s = stream_key(seed, tag, a, b, c);
    for (int32_t i = 0; i < n; ++i) out[i] = next64(&s);
}

/* ------------------------------------------------------------------- cell */
typedef struct {
    double H[9];      /* column-major: H[0..2] = a, H[3..5] = b, H[6..8] = c */
    double Hi[9];     /* row-major inverse: Hi[3*k + m] */
    double det;       /* dot(cross(a, b), c), src/mddf.jl:350-351 */
    double wmin;      /* smallest perpendicular width */
    double w[3];
    int ortho;        /* off-diagonal entries all zero */
} cellinfo;

static void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double *a, const double *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static void cell_setup(const double *H, cellinfo *ci) {
    memcpy(ci->H, H, 9 * sizeof(double));
    const double *a = H, *b = H + 3, *c = H + 6;
    double ab[3], bc[3], ca[3];
    cross3(a, b, ab);
    cross3(b, c, bc);
    cross3(c, a, ca);
    ci->det = dot3(ab, c);
    for (int m = 0; m < 3; ++m) {
        ci->Hi[0 + m] = bc[m] / ci->det;
        ci->Hi[3 + m] = ca[m] / ci->det;
        ci->Hi[6 + m] = ab[m] / ci->det;
    }
    double V = fabs(ci->det);
    ci->w[0] = V / sqrt(dot3(bc, bc));
    ci->w[1] = V / sqrt(dot3(ca, ca));
    ci->w[2] = V / sqrt(dot3(ab, ab));
    ci->wmin = fmin(ci->w[0], fmin(ci->w[1], ci->w[2]));
    ci->ortho = (H[1] == 0.0 && H[2] == 0.0 && H[3] == 0.0 && H[5] == 0.0 && H[6] == 0.0 && H[7] == 0.0);
}
/* f = Hinv * d */
static inline void to_frac(const cellinfo *ci, const double *d, double *f) {
    if (ci->ortho) {
        f[0] = d[0] * ci->Hi[0];
        f[1] = d[1] * ci->Hi[4];
        f[2] = d[2] * ci->Hi[8];
    } else {
        for (int k = 0; k < 3; ++k) f[k] = (ci->Hi[3 * k] * d[0] + ci->Hi[3 * k + 1] * d[1]) + ci->Hi[3 * k + 2] * d[2];
    }
}
/* v = H * n */
static inline void lat(const cellinfo *ci, const double *n, double *v) {
    if (ci->ortho) {
        v[0] = ci->H[0] * n[0];
        v[1] = ci->H[4] * n[1];
        v[2] = ci->H[8] * n[2];
    } else {
        for (int k = 0; k < 3; ++k) v[k] = (ci->H[k] * n[0] + ci->H[3 + k] * n[1]) + ci->H[6 + k] * n[2];
    }
}

/* Minimum-image squared distance between x and y (restated CellListMap
 * contract: the pair is reported iff this is <= cutoff^2, and d = sqrt of it). */
static double mindist2(const cellinfo *ci, const double *x, const double *y) {
    double d[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    double f[3], n0[3], s[3], e[3];
    to_frac(ci, d, f);
    for (int k = 0; k < 3; ++k) n0[k] = rint(f[k]);
    if (n0[0] != 0.0 || n0[1] != 0.0 || n0[2] != 0.0) {
        lat(ci, n0, s);
        for (int k = 0; k < 3; ++k) e[k] = d[k] - s[k];
    } else {
        e[0] = d[0]; e[1] = d[1]; e[2] = d[2];
    }
    double best = (e[0] * e[0] + e[1] * e[1]) + e[2] * e[2];
    /* an image no longer than half the smallest perpendicular width is the
     * minimum image; otherwise search the 26 neighbouring images */
    double h = 0.5 * ci->wmin;
    if (best <= h * h) return best;
    for (int i = -1; i <= 1; ++i)
        for (int j = -1; j <= 1; ++j)
            for (int l = -1; l <= 1; ++l) {
                if (i == 0 && j == 0 && l == 0) continue;
                double n[3] = {n0[0] + i, n0[1] + j, n0[2] + l};
                lat(ci, n, s);
                double t0 = d[0] - s[0], t1 = d[1] - s[1], t2 = d[2] - s[2];
                double q = (t0 * t0 + t1 * t1) + t2 * t2;
                if (q < best) best = q;
            }
    return best;
}

/* src/results.jl:28  setbin(d, step) = max(1, ceil(Int, d/step)) ; 0-based here */
static inline int setbin0(double d, double step) {
    double q = ceil(d / step);
    int b = (int)q;
    if (b < 1) b = 1;
    return b - 1;
}
int32_t orc_setbin(double d, double step) { return setbin0(d, step) + 1; }

/* ------------------------------------------------------------- list record */
typedef struct {
    int within;      /* within_cutoff */
    int i;           /* solute atom, local index in its molecule */
    int64_t j;       /* solvent atom, global index in the selection */
    double d;
    int ref;         /* ref_atom_within_cutoff */
    double dref;
} mdrec;

static inline void md_zero(mdrec *m) {
    m->within = 0; m->i = -1; m->j = -1; m->d = INFINITY; m->ref = 0; m->dref = INFINITY;
}
/* src/minimum_distances.jl:30-39 with md2 = the new pair (within=true).  The
 * new pair replaces the record unless the record is strictly closer, so among
 * equal distances the pair visited last wins; pairs are visited with the solute
 * atom index outer and the solvent atom index inner. */
static inline void md_update(mdrec *m, int i, int64_t j, double d, int isref) {
    int ref = m->ref || isref;
    double dref = ref ? fmin(m->dref, isref ? d : INFINITY) : INFINITY;
    if (!(m->d < d)) { m->within = 1; m->i = i; m->j = j; m->d = d; }
    m->ref = ref;
    m->dref = dref;
}

/* ----------------------------------------------------------------- context */
typedef struct {
    const orc_desc *D;
    cellinfo ci;
    /* cells backend over solvent molecule anchors */
    int n[3];
    int ncell;
    int *cstart, *cnext_mol, *cmol;   /* counting-sorted molecules per cell */
    double rmax;
    int64_t *stamp;
    int64_t stampc;
    mdrec *list, *list_save;
    int *bulk;
    double *placed;                     /* Nv*3 */
    double *work_u;                     /* apv*3 */
} ctx;

static int grp_credit(int64_t *tab, int nb, const int64_t *off, const int32_t *grp, int64_t atom, int bin, int64_t inc) {
    for (int64_t p = off[atom]; p < off[atom + 1]; ++p) tab[(int64_t)grp[p] * nb + bin] += inc;
    return 0;
}

static void cells_build(ctx *C, const double *y) {
    const orc_desc *D = C->D;
    const cellinfo *ci = &C->ci;
    double rmax = 0.0;
    for (int v = 0; v < D->mv; ++v) {
        const double *y0 = y + (int64_t)v * D->apv * 3;
        for (int b = 1; b < D->apv; ++b) {
            double r = sqrt(mindist2(ci, y0, y0 + 3 * b));
            if (r > rmax) rmax = r;
        }
    }
    C->rmax = rmax;
    double range = D->cutoff + rmax + 1e-6 * (1.0 + D->cutoff);
    for (int k = 0; k < 3; ++k) {
        int n = (int)floor(ci->w[k] / range);
        C->n[k] = n < 1 ? 1 : n;
    }
    C->ncell = C->n[0] * C->n[1] * C->n[2];
    C->cstart = (int *)realloc(C->cstart, (size_t)(C->ncell + 1) * sizeof(int));
    memset(C->cstart, 0, (size_t)(C->ncell + 1) * sizeof(int));
    for (int v = 0; v < D->mv; ++v) {
        const double *y0 = y + (int64_t)v * D->apv * 3;
        double f[3];
        to_frac(ci, y0, f);
        int c[3];
        for (int k = 0; k < 3; ++k) {
            double g = f[k] - floor(f[k]);
            int q = (int)floor(g * C->n[k]);
            if (q >= C->n[k]) q = C->n[k] - 1;
            if (q < 0) q = 0;
            c[k] = q;
        }
        int cell = (c[2] * C->n[1] + c[1]) * C->n[0] + c[0];
        C->cnext_mol[v] = cell;
        C->cstart[cell + 1]++;
    }
    for (int i = 0; i < C->ncell; ++i) C->cstart[i + 1] += C->cstart[i];
    int *fill = (int *)malloc((size_t)C->ncell * sizeof(int));
    memcpy(fill, C->cstart, (size_t)C->ncell * sizeof(int));
    for (int v = 0; v < D->mv; ++v) C->cmol[fill[C->cnext_mol[v]]++] = v;
    free(fill);
}

/* Minimum distances of one solute molecule (atoms xs) to all solvent molecules
 * (coordinates y): src/minimum_distances.jl:129-148 + :81-120. */
static int64_t min_distances(ctx *C, int s, const double *xs, const double *y, mdrec *list) {
    const orc_desc *D = C->D;
    const cellinfo *ci = &C->ci;
    double cut = D->usecutoff ? D->cutoff : D->dbulk;
    double cut2 = cut * cut;
    int jref = D->irefatom - 1;
    int64_t npairs = 0;
    for (int v = 0; v < D->mv; ++v) md_zero(&list[v]);
    if (D->backend == 0) {
        for (int a = 0; a < D->aps; ++a) {
            const double *x = xs + 3 * a;
            for (int v = 0; v < D->mv; ++v) {
                if (D->autocorrelation && v == s) continue;
                for (int b = 0; b < D->apv; ++b) {
                    int64_t j = (int64_t)v * D->apv + b;
                    double d2 = mindist2(ci, x, y + 3 * j);
                    if (d2 <= cut2) { md_update(&list[v], a, j, sqrt(d2), b == jref); npairs++; }
                }
            }
        }
        return npairs;
    }
    /* cells backend: the anchors of y are binned in C (cells_build must have run on y) */
    double pre = cut + C->rmax + 1e-6 * (1.0 + cut);
    double pre2 = pre * pre;
    for (int a = 0; a < D->aps; ++a) {
        const double *x = xs + 3 * a;
        double f[3];
        to_frac(ci, x, f);
        int c[3];
        for (int k = 0; k < 3; ++k) {
            double g = f[k] - floor(f[k]);
            int q = (int)floor(g * C->n[k]);
            if (q >= C->n[k]) q = C->n[k] - 1;
            if (q < 0) q = 0;
            c[k] = q;
        }
        C->stampc++;
        int lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            if (C->n[k] >= 3) { lo[k] = c[k] - 1; hi[k] = c[k] + 1; }
            else { lo[k] = 0; hi[k] = C->n[k] - 1; }
        }
        /* gather candidate molecules, then visit them in ascending order so that
         * the (a, b) visiting order per molecule is the same as in backend 0 */
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int yy = lo[1]; yy <= hi[1]; ++yy)
                for (int xx = lo[0]; xx <= hi[0]; ++xx) {
                    int cx = (xx % C->n[0] + C->n[0]) % C->n[0];
                    int cy = (yy % C->n[1] + C->n[1]) % C->n[1];
                    int cz = (z % C->n[2] + C->n[2]) % C->n[2];
                    int cell = (cz * C->n[1] + cy) * C->n[0] + cx;
                    for (int p = C->cstart[cell]; p < C->cstart[cell + 1]; ++p) {
                        int v = C->cmol[p];
                        if (D->autocorrelation && v == s) continue;
                        if (C->stamp[v] == C->stampc) continue;
                        C->stamp[v] = C->stampc;
                        /* no atom of v can be within the cutoff if its anchor is
                         * farther than cutoff + rmax (exact, conservative) */
                        if (mindist2(ci, x, y + (int64_t)v * D->apv * 3) > pre2) continue;
                        for (int b = 0; b < D->apv; ++b) {
                            int64_t j = (int64_t)v * D->apv + b;
                            double d2 = mindist2(ci, x, y + 3 * j);
                            if (d2 <= cut2) { md_update(&list[v], a, j, sqrt(d2), b == jref); npairs++; }
                        }
                    }
                }
    }
    return npairs;
}

/* src/update_counters.jl:43-64 (real) and :67-87 (random); src/results.jl:28 */
static void update_counters(ctx *C, const mdrec *list, orc_counts *o, int random) {
    const orc_desc *D = C->D;
    int nb = D->nbins;
    int64_t *md = random ? o->md_rand : o->md;
    int64_t *rdf = random ? o->rdf_rand : o->rdf;
    int64_t *gs = random ? o->gs_rand : o->gs;
    int64_t *gv = random ? o->gv_rand : o->gv;
    for (int v = 0; v < D->mv; ++v) {
        const mdrec *m = &list[v];
        if (!m->within) continue;
        int bin = setbin0(m->d, D->binstep);
        md[bin] += 2;
        if (D->autocorrelation) {
            /* both atoms credit the solute table with w/2: i is local to the
             * solute molecule, j is global in the (same) selection */
            grp_credit(gs, nb, D->solute_grp_off, D->solute_grp, m->i, bin, 1);
            grp_credit(gs, nb, D->solvent_grp_off, D->solvent_grp, m->j, bin, 1);
        } else {
            grp_credit(gs, nb, D->solute_grp_off, D->solute_grp, m->i, bin, 2);
            grp_credit(gv, nb, D->solvent_grp_off, D->solvent_grp, m->j, bin, 2);
        }
        if (m->ref) rdf[setbin0(m->dref, D->binstep)] += 2;
    }
}

/* src/rigid_body.jl:35-57 eulermat, with (cos, sin) of the three angles */
void orc_eulermat_cs(double c1, double s1, double c2, double s2, double c3, double s3, double *A /*row-major*/) {
    A[0] = c2 * c3;
    A[1] = -(c2 * s3);
    A[2] = s2;
    A[3] = c1 * s3 + (c3 * s1) * s2;
    A[4] = c1 * c3 - (s1 * s2) * s3;
    A[5] = -(c2 * s1);
    A[6] = s1 * s3 - (c1 * c3) * s2;
    A[7] = (c1 * s2) * s3 + c3 * s1;
    A[8] = c1 * c2;
}

/* src/rigid_body.jl:73-80 move!: x <- A (x - mean(x)) + newcm, in place on n atoms */
void orc_move(double *x, int32_t n, const double *newcm, const double *A) {
    double cm[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cm[k] += x[3 * i + k];
    for (int k = 0; k < 3; ++k) cm[k] = cm[k] / (double)n;
    for (int i = 0; i < n; ++i) {
        double u[3] = {x[3 * i] - cm[0], x[3 * i + 1] - cm[1], x[3 * i + 2] - cm[2]};
        for (int k = 0; k < 3; ++k) x[3 * i + k] = ((A[3 * k] * u[0] + A[3 * k + 1] * u[1]) + A[3 * k + 2] * u[2]) + newcm[k];
    }
}

/* src/mddf.jl:65-88 randomize_solvent! + src/rigid_body.jl:107-137 random_move! */
static void randomize_solvent(ctx *C, int64_t frame, int s, int rep, const double *yreal, int nbulk, double *out) {
    const orc_desc *D = C->D;
    const cellinfo *ci = &C->ci;
    int apv = D->apv;
    int iref = D->irefatom - 1;
    double *u = C->work_u;
    for (int k = 0; k < D->mv; ++k) {
        uint64_t st = stream_key(D->seed, TAG_SLOT, (uint64_t)frame, (uint64_t)s, ((uint64_t)rep << 32) | (uint64_t)k);
        int jmol = nbulk > 0 ? C->bulk[index_below(&st, (uint64_t)nbulk)] : (int)index_below(&st, (uint64_t)D->mv);
        double fc[3];
        for (int q = 0; q < 3; ++q) fc[q] = uniform01(&st);
        double cb, sb, cg, sg, ct, stt;
        angle_cs(&st, &cb, &sb);
        angle_cs(&st, &cg, &sg);
        angle_cs(&st, &ct, &stt);
        double A[9];
        orc_eulermat_cs(cb, sb, cg, sg, ct, stt, A);
        double newcm[3];
        lat(ci, fc, newcm);
        const double *src = yreal + (int64_t)jmol * apv * 3;
        const double *xr = src + 3 * iref;
        /* wrap_relative_to(x, x[irefatom], uc) */
        for (int b = 0; b < apv; ++b) {
            double d[3] = {src[3 * b] - xr[0], src[3 * b + 1] - xr[1], src[3 * b + 2] - xr[2]};
            double f[3], n[3];
            to_frac(ci, d, f);
            for (int q = 0; q < 3; ++q) n[q] = rint(f[q]);
            if (n[0] != 0.0 || n[1] != 0.0 || n[2] != 0.0) {
                double sh[3];
                lat(ci, n, sh);
                for (int q = 0; q < 3; ++q) u[3 * b + q] = src[3 * b + q] - sh[q];
            } else {
                for (int q = 0; q < 3; ++q) u[3 * b + q] = src[3 * b + q];
            }
        }
        orc_move(u, apv, newcm, A);
        memcpy(out + (int64_t)k * apv * 3, u, (size_t)apv * 3 * sizeof(double));
    }
}

/* src/mddf.jl:55-57 */
static inline int inbulk(const mdrec *m, const orc_desc *D) {
    return D->usecutoff ? (m->within && m->d > D->dbulk) : !m->within;
}

/* src/mddf.jl:361-429 (mddf_frame!) and :438-471 (coordination_number_frame!) */
static void frame_one(ctx *C, int64_t frame, const double *xsol, const double *ysol, orc_counts *o) {
    const orc_desc *D = C->D;
    int nrs = D->n_random_samples;
    int *ref_solutes = (int *)malloc((size_t)(nrs > 0 ? nrs : 1) * sizeof(int));
    if (!D->coordination_number_only) {
        uint64_t st = stream_key(D->seed, TAG_REF, (uint64_t)frame, 0, 0);
        for (int i = 0; i < nrs; ++i) ref_solutes[i] = (int)index_below(&st, (uint64_t)D->ms);
    }
    if (D->backend == 1) cells_build(C, ysol);
    for (int s = 0; s < D->ms; ++s) {
        const double *xs = xsol + (int64_t)s * D->aps * 3;
        o->pairs_real += min_distances(C, s, xs, ysol, C->list);
        update_counters(C, C->list, o, 0);
        if (D->coordination_number_only) continue;
        int nrand = 0;
        for (int i = 0; i < nrs; ++i) nrand += (ref_solutes[i] == s);
        if (nrand == 0) continue;
        memcpy(C->list_save, C->list, (size_t)D->mv * sizeof(mdrec));
        int nbulk = 0;
        for (int v = 0; v < D->mv; ++v) {
            if (D->autocorrelation && v == s) continue;
            if (inbulk(&C->list_save[v], D)) C->bulk[nbulk++] = v;
        }
        for (int r = 0; r < nrand; ++r) {
            randomize_solvent(C, frame, s, r, ysol, nbulk, C->placed);
            if (D->backend == 1) cells_build(C, C->placed);
            o->pairs_rand += min_distances(C, s, xs, C->placed, C->list);
            update_counters(C, C->list, o, 1);
        }
        if (D->backend == 1) cells_build(C, ysol);
    }
    free(ref_solutes);
}

static int counts_alloc(const orc_desc *D, orc_counts *o) {
    int nb = D->nbins;
    o->md = calloc((size_t)nb, 8); o->md_rand = calloc((size_t)nb, 8);
    o->rdf = calloc((size_t)nb, 8); o->rdf_rand = calloc((size_t)nb, 8);
    o->gs = calloc((size_t)D->solute_ngroups * nb, 8); o->gs_rand = calloc((size_t)D->solute_ngroups * nb, 8);
    o->gv = calloc((size_t)(D->solvent_ngroups > 0 ? D->solvent_ngroups : 1) * nb, 8);
    o->gv_rand = calloc((size_t)(D->solvent_ngroups > 0 ? D->solvent_ngroups : 1) * nb, 8);
    o->pairs_real = o->pairs_rand = 0;
    return (o->md && o->md_rand && o->rdf && o->rdf_rand && o->gs && o->gs_rand && o->gv && o->gv_rand) ? ORC_OK : ORC_ENOMEM;
}
static void counts_free(orc_counts *o) {
    free(o->md); free(o->md_rand); free(o->rdf); free(o->rdf_rand);
    free(o->gs); free(o->gs_rand); free(o->gv); free(o->gv_rand);
}
static void counts_add(const orc_desc *D, orc_counts *dst, const orc_counts *src) {
    int nb = D->nbins;
    for (int i = 0; i < nb; ++i) {
        dst->md[i] += src->md[i]; dst->md_rand[i] += src->md_rand[i];
        dst->rdf[i] += src->rdf[i]; dst->rdf_rand[i] += src->rdf_rand[i];
    }
    for (int64_t i = 0; i < (int64_t)D->solute_ngroups * nb; ++i) { dst->gs[i] += src->gs[i]; dst->gs_rand[i] += src->gs_rand[i]; }
    for (int64_t i = 0; i < (int64_t)D->solvent_ngroups * nb; ++i) { dst->gv[i] += src->gv[i]; dst->gv_rand[i] += src->gv_rand[i]; }
    dst->pairs_real += src->pairs_real;
    dst->pairs_rand += src->pairs_rand;
}

static int ctx_init(ctx *C, const orc_desc *D) {
    memset(C, 0, sizeof(*C));
    C->D = D;
    int64_t Nv = (int64_t)D->mv * D->apv;
    C->list = malloc((size_t)D->mv * sizeof(mdrec));
    C->list_save = malloc((size_t)D->mv * sizeof(mdrec));
    C->bulk = malloc((size_t)D->mv * sizeof(int));
    C->placed = malloc((size_t)Nv * 3 * sizeof(double));
    C->work_u = malloc((size_t)D->apv * 3 * sizeof(double));
    C->cnext_mol = malloc((size_t)D->mv * sizeof(int));
    C->cmol = malloc((size_t)D->mv * sizeof(int));
    C->stamp = calloc((size_t)D->mv, sizeof(int64_t));
    return (C->list && C->list_save && C->bulk && C->placed && C->work_u && C->cnext_mol && C->cmol && C->stamp) ? ORC_OK : ORC_ENOMEM;
}
static void ctx_free(ctx *C) {
    free(C->list); free(C->list_save); free(C->bulk); free(C->placed); free(C->work_u);
    free(C->cnext_mol); free(C->cmol); free(C->stamp); free(C->cstart);
}

static int desc_check(const orc_desc *D) {
    if (D->ms < 1 || D->aps < 1 || D->mv < 1 || D->apv < 1) return ORC_EINVAL;
    if (D->irefatom < 1 || D->irefatom > D->apv) return ORC_EINVAL;
    if (D->nbins < 1 || !(D->binstep > 0.0)) return ORC_EINVAL;
    if (D->autocorrelation && (D->ms != D->mv || D->aps != D->apv)) return ORC_EINVAL;
    if (!D->solute_grp_off || !D->solvent_grp_off) return ORC_EINVAL;
    double cut = D->usecutoff ? D->cutoff : D->dbulk;
    if (setbin0(cut, D->binstep) >= D->nbins) return ORC_EINVAL;
    if (D->solute_ngroups < 1 || D->solvent_ngroups < 1) return ORC_EINVAL;
    /* in self mode both credits go to the solute table */
    if (D->autocorrelation && D->solvent_ngroups != D->solute_ngroups) return ORC_EINVAL;
    for (int64_t a = 0; a < D->aps; ++a)
        for (int64_t p = D->solute_grp_off[a]; p < D->solute_grp_off[a + 1]; ++p)
            if (D->solute_grp[p] < 0 || D->solute_grp[p] >= D->solute_ngroups) return ORC_EINVAL;
    int64_t Nv = (int64_t)D->mv * D->apv;
    for (int64_t j = 0; j < Nv; ++j)
        for (int64_t p = D->solvent_grp_off[j]; p < D->solvent_grp_off[j + 1]; ++p)
            if (D->solvent_grp[p] < 0 || D->solvent_grp[p] >= D->solvent_ngroups) return ORC_EINVAL;
    return ORC_OK;
}

/*
 * Run frames [0, nframes) and add their half-unit counts to *out (the caller
 * zeroes *out).  Coordinates are FP64 xyz in selection order,
 * [nframes][natoms][3]; in self mode `solvent_xyz` may be NULL.  `cells` holds
 * [nframes][9] column-major unit cells; `frame_ids` the trajectory frame number
 * of each frame (it keys the random stream).  Frames run in parallel on
 * `nthreads` threads with private counters (src/mddf.jl:287-338).
 */
int orc_frames(const orc_desc *D, int32_t nframes, const double *solute_xyz, const double *solvent_xyz,
               const double *cells, const int64_t *frame_ids, int32_t nthreads, orc_counts *out) {
    int rc = desc_check(D);
    if (rc) return rc;
    if (nframes <= 0) return ORC_OK;
    if (!solvent_xyz) solvent_xyz = solute_xyz;
    int64_t Ns = (int64_t)D->ms * D->aps, Nv = (int64_t)D->mv * D->apv;
    int err = 0;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
    {
        ctx C;
        orc_counts loc;
        memset(&loc, 0, sizeof(loc));
        int ok = (ctx_init(&C, D) == ORC_OK) && (counts_alloc(D, &loc) == ORC_OK);
        if (!ok) err |= 1;
        else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int32_t f = 0; f < nframes; ++f) {
                cell_setup(cells + 9 * (int64_t)f, &C.ci);
                frame_one(&C, frame_ids[f], solute_xyz + (int64_t)f * Ns * 3, solvent_xyz + (int64_t)f * Nv * 3, &loc);
            }
#ifdef _OPENMP
#pragma omp critical
#endif
            counts_add(D, out, &loc);
        }
        counts_free(&loc);
        ctx_free(&C);
    }
    return err ? ORC_ENOMEM : ORC_OK;
}

/* Volume term of one frame: dot(cross(a, b), c) (src/mddf.jl:350-351). */
double orc_cell_volume(const double *H) {
    cellinfo ci;
    cell_setup(H, &ci);
    return ci.det;
}

/* Minimum-image squared distance (exposed for tests). */
double orc_mindist2(const double *H, const double *x, const double *y) {
    cellinfo ci;
    cell_setup(H, &ci);
    return mindist2(&ci, x, y);
}
