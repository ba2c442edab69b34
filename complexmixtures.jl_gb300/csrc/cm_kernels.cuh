// cm_kernels.cuh -- device code of the GB300 MDDF engine.
//
// Per frame the engine answers, for every (solute molecule s, solvent molecule v)
// pair, the question mddf_frame! asks through CellListMap (src/mddf.jl:382-396,
// src/minimum_distances.jl:81-148): the minimum-distance atom pair within the
// cutoff, its distance, and the shortest distance from s to v's reference atom;
// then it bins the answer into the MDDF / RDF / group histograms
// (src/update_counters.jl:43-87).  Only pairs that are within the cutoff touch
// the histograms, which replaces the reference's O(nsolute * nsolvent) scan of
// the whole list with the same counts.
//
// Two search layouts ("regimes"):
//   PAIRS  molecules of both selections are small.  Molecules are binned by
//          their centroid; a warp walks the stencil of one solute molecule,
//          queues candidate solvent molecules whose bounding spheres come within
//          the cutoff, and each lane evaluates all atom pairs of one candidate.
//          In self mode each unordered pair is evaluated once and credited in
//          both directions.
//   ATOMS  the solute molecule is large (a protein).  Its atoms are counting-
//          sorted into cells; one thread per solvent molecule scans the stencil
//          of each of its atoms.
//
// Precision.  In FP32 mode the search runs in single precision on cell-relative
// coordinates.  Every discrete decision -- within cutoff, which atom pair is the
// minimum, the histogram bin, the bulk test, the reference-atom distance -- is
// taken from the FP32 value only when the value is farther than the guard band
// `delta` from the decision boundary; otherwise the pair is re-evaluated in FP64
// with the same formula the FP64 mode uses, so both modes produce identical
// integer counts.  `delta` is a rigorous bound on the FP32 rounding error,
// computed per frame from the magnitudes that enter the FP32 displacement.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cm_geom.h"

namespace cmk {

using cmfeed::add;
using cmfeed::div;
using cmfeed::mul;
using cmfeed::sub;
using namespace cmgeom;

constexpr int kMaxSmallMol = 32;  // PAIRS regime: atoms per molecule on either side
constexpr int kWarps = 8;         // warps per CTA of the PAIRS real-pass kernels
constexpr int kQueue = 64;        // per-warp candidate queue
constexpr int kTileCells = 128;   // half-stencil cells the tiled real pass stages per home cell
constexpr int kAgridMaxStencil = 343;  // ATOMS stencil cells the candidate-grid build stages (half-widths up to 3)

enum : int { ERR_STENCIL = 1, ERR_BIN = 2, ERR_QUEUE = 4, ERR_SIZE = 8 };
enum : int {
    ST_MOLPAIRS = 0,
    ST_ATOMPAIRS,
    ST_HITS_REAL,
    ST_HITS_RAND,
    ST_GUARD,
    ST_GUARD_PAIRS,
    ST_MAXERR,  // bits of a non-negative double
    ST_AGRID_OVF,   // frames whose candidate-grid lists did not fit (they took the walk)
    ST_AGRID_NEED,  // the largest list entries of such a frame
    ST_N
};

struct DevSys {
    int ms, aps, mv, apv;
    int self;
    int iref;       // 0-based reference atom (solvent role)
    int nbins;
    int nrs;
    int fp32;
    int usecutoff;
    int Gs, Gv;
    int default_s, default_v;
    int smem_groups;
    double cut, cut2, binstep, dbulk;
    uint64_t seed;
    const int64_t *gs_off;
    const int32_t *gs_idx;
    const int64_t *gv_off;
    const int32_t *gv_idx;
    unsigned long long *hist;  // class accumulators, half units
    int64_t o_md, o_mdr, o_rdf, o_rdfr, o_gs, o_gsr, o_gv, o_gvr;
    unsigned long long *stats;
    int *err;
};

// Decision constants of one frame for a search in precision R (float: the
// FP32 search; double: the FP64 search).  A value computed in R is within
// delta of the exact distance (cm_geom.h, exact_d2), so a decision taken from
// it is the exact decision when the value lies farther than delta from the
// decision boundary.
template <typename R>
struct GuardT {
    double delta;     // Angstrom
    R cutp2;          // (cut + delta)^2, rounded up
    R cutm2;          // (cut - delta)^2, rounded down
    R two_delta;
    R inv_bs;         // 1 / binstep in R
    R bin_band;       // half-width of the bin-edge band in units of bins
    R dbulk_lo, dbulk_hi;
    float cut_pre;    // cutoff + margin of the bounding-sphere tests
};
using Guard = GuardT<float>;
using Guard64 = GuardT<double>;

// Geometry of the candidate grid's fine cells (K^3 per search cell) of a frame.
struct FineCells {
    int K, K3;
    float e[9];  // column-major edge vectors of a fine cell (column k = search-cell edge k / K)
    float h[3];  // orthogonal cells: half sides
    float R;     // bounding-sphere radius (half the longest diagonal), rounded up
    int ortho;
};

// Per-frame values found by the prep kernels and the constants derived from
// them by k_frame_consts (one block, before the search kernels).
struct FrameScratch {
    float rmax_s;   // largest solute molecule radius (PAIRS: about the centroid)
    float rmax_v;   // largest solvent molecule radius
    float rcmax;    // largest solvent centroid radius (ATOMS layout)
    float hin[9];   // n_k * (H^-1 row k): cell-relative position -> grid units in the cell (FP32)
    float cw[3];    // cell widths between opposite faces (FP32)
    int ortho;      // cell axes orthogonal (H/n diagonal)
    int ok;         // stencils fit the offset table
    int L[3];       // PAIRS stencil half-widths
    int multi;      // PAIRS axes with several images (bit k set for axis k)
    int La[3];      // ATOMS stencil half-widths
    float xmax;     // largest |coordinate component| of the frame's input atoms (rounded up)
    int tile;       // self mode, one image per pair, half stencil within kTileCells: the tiled real pass takes the frame
    int agrid;      // ATOMS, one solute molecule: the frame's candidate grid is complete (k_agrid_scan clears it on overflow)
    FineCells fcells;  // the candidate grid's fine cells (when agrid)
    int place32;    // ATOMS, FP32 search: random-insertion slots placed in FP32 (placed_store32), the band widened to match
    Guard g;        // FP32 search
    Guard64 g64;    // FP64 search
};

struct Sample {
    int s;     // solute molecule
    int rep;   // repetition index of s in this frame
    int d;     // distinct-sample index (flags / bulk list row)
    int pad;
};

__device__ __forceinline__ void raise_err(const DevSys &S, int code) { atomicOr(S.err, code); }

__device__ __forceinline__ int setbin0(double d, double step) {
    int b = (int)ceil(div(d, step));
    return (b < 1 ? 1 : b) - 1;
}

__device__ __forceinline__ float norm3f(float x, float y, float z) { return sqrtf(fmaf(z, z, fmaf(y, y, x * x))); }

// ------------------------------------------------------------------ histograms
struct SHist {
    unsigned int *md, *rdf, *gs, *gv;  // shared-memory privatised counters
};

__device__ __forceinline__ int hist_words(const DevSys &S) {
    return S.nbins * (2 + (S.smem_groups ? (S.Gs + (S.self ? 0 : S.Gv)) : 0));
}

__device__ __forceinline__ SHist shist_bind(const DevSys &S, unsigned int *base) {
    SHist h;
    h.md = base;
    h.rdf = base + S.nbins;
    h.gs = base + 2 * S.nbins;
    h.gv = h.gs + (int64_t)S.Gs * S.nbins;
    return h;
}

__device__ void shist_zero(const DevSys &S, unsigned int *base) {
    int n = hist_words(S);
    for (int i = threadIdx.x; i < n; i += blockDim.x) base[i] = 0u;
}

__device__ void shist_flush(const DevSys &S, const SHist &h, bool rnd) {
    unsigned long long *md = S.hist + (rnd ? S.o_mdr : S.o_md);
    unsigned long long *rdf = S.hist + (rnd ? S.o_rdfr : S.o_rdf);
    for (int i = threadIdx.x; i < S.nbins; i += blockDim.x) {
        if (h.md[i]) atomicAdd(md + i, (unsigned long long)h.md[i]);
        if (h.rdf[i]) atomicAdd(rdf + i, (unsigned long long)h.rdf[i]);
    }
    if (S.smem_groups) {
        unsigned long long *gs = S.hist + (rnd ? S.o_gsr : S.o_gs);
        int64_t n = (int64_t)S.Gs * S.nbins;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
            if (h.gs[i]) atomicAdd(gs + i, (unsigned long long)h.gs[i]);
        if (!S.self) {
            unsigned long long *gv = S.hist + (rnd ? S.o_gvr : S.o_gv);
            int64_t m = (int64_t)S.Gv * S.nbins;
            for (int64_t i = threadIdx.x; i < m; i += blockDim.x)
                if (h.gv[i]) atomicAdd(gv + i, (unsigned long long)h.gv[i]);
        }
    }
}

__device__ __forceinline__ void add_group(const DevSys &S, const SHist &h, bool rnd, bool solvent_table, int g, int bin,
                                          unsigned inc) {
    int64_t idx = (int64_t)g * S.nbins + bin;
    if (S.smem_groups) {
        atomicAdd((solvent_table ? h.gv : h.gs) + idx, inc);
    } else {
        int64_t o = solvent_table ? (rnd ? S.o_gvr : S.o_gv) : (rnd ? S.o_gsr : S.o_gs);
        atomicAdd(S.hist + o + idx, (unsigned long long)inc);
    }
}

// update_group_count! (src/update_counters.jl:22-36) for the solute-side atom,
// identified by its index inside the solute molecule.
__device__ __forceinline__ void credit_solute(const DevSys &S, const SHist &h, bool rnd, int i_local, int bin, unsigned inc) {
    if (S.default_s) {
        add_group(S, h, rnd, false, i_local, bin, inc);
    } else {
        for (int64_t p = S.gs_off[i_local]; p < S.gs_off[i_local + 1]; ++p) add_group(S, h, rnd, false, S.gs_idx[p], bin, inc);
    }
}

// The solvent-side atom, identified by its index in the whole selection; in
// self mode it credits the solute table (src/update_counters.jl:272-277).
// j_local is the atom's index within its molecule.
__device__ __forceinline__ void credit_solvent(const DevSys &S, const SHist &h, bool rnd, int64_t j, int j_local, int bin,
                                               unsigned inc) {
    bool to_solvent = !S.self;
    if (S.default_v) {
        add_group(S, h, rnd, to_solvent, j_local, bin, inc);
    } else {
        for (int64_t p = S.gv_off[j]; p < S.gv_off[j + 1]; ++p) add_group(S, h, rnd, to_solvent, S.gv_idx[p], bin, inc);
    }
}

// One within-cutoff record of the reference's list, binned (update_counters!).
// j is the solvent atom's index in the selection, j_local its index within
// its molecule.
__device__ __forceinline__ void apply_hit_local(const DevSys &S, const SHist &h, bool rnd, int bin, int i_local, int64_t j,
                                                int j_local, bool ref, int rbin) {
    if (bin < 0 || bin >= S.nbins || (ref && (rbin < 0 || rbin >= S.nbins))) {
        raise_err(S, ERR_BIN);
        return;
    }
    atomicAdd(h.md + bin, 2u);
    if (S.self) {
        credit_solute(S, h, rnd, i_local, bin, 1u);
        credit_solvent(S, h, rnd, j, j_local, bin, 1u);
    } else {
        credit_solute(S, h, rnd, i_local, bin, 2u);
        credit_solvent(S, h, rnd, j, j_local, bin, 2u);
    }
    if (ref) atomicAdd(h.rdf + rbin, 2u);
}

// Both directions of one unordered self-MDDF pair: the same md bin, the
// solute molecule's atom a and the solvent molecule's atom b each credited
// once per direction (both into the solute table), and each direction's
// reference-atom row.  Equals two apply_hit_local calls with fewer atomics.
__device__ __forceinline__ void apply_pair_self(const DevSys &S, const SHist &h, int bin, int a, int64_t ja, int b,
                                                int64_t jb, bool ref1, int rbin1, bool ref2, int rbin2) {
    if (bin < 0 || bin >= S.nbins || (ref1 && (rbin1 < 0 || rbin1 >= S.nbins)) ||
        (ref2 && (rbin2 < 0 || rbin2 >= S.nbins))) {
        raise_err(S, ERR_BIN);
        return;
    }
    atomicAdd(h.md + bin, 4u);
    if (S.default_s && S.default_v) {
        if (a == b) {
            add_group(S, h, false, false, a, bin, 4u);
        } else {
            add_group(S, h, false, false, a, bin, 2u);
            add_group(S, h, false, false, b, bin, 2u);
        }
    } else {
        // direction 1: solute atom a (local), solvent atom jb (global index);
        // direction 2: solute atom b, solvent atom ja
        credit_solute(S, h, false, a, bin, 1u);
        credit_solvent(S, h, false, jb, b, bin, 1u);
        credit_solute(S, h, false, b, bin, 1u);
        credit_solvent(S, h, false, ja, a, bin, 1u);
    }
    if (ref1) atomicAdd(h.rdf + rbin1, 2u);
    if (ref2) atomicAdd(h.rdf + rbin2, 2u);
}

__device__ __forceinline__ void apply_hit(const DevSys &S, const SHist &h, bool rnd, int bin, int i_local, int64_t j, bool ref,
                                          int rbin) {
    apply_hit_local(S, h, rnd, bin, i_local, j, (int)j % S.apv, ref, rbin);
}

// Warp-aggregated statistics counters.
struct LocalStats {
    unsigned long long molpairs = 0, atompairs = 0, hits = 0, guard = 0, guard_pairs = 0;
    double maxerr = 0.0;
};

__device__ void stats_flush(const DevSys &S, LocalStats &st, bool rnd) {
    unsigned long long v[5] = {st.molpairs, st.atompairs, st.hits, st.guard, st.guard_pairs};
#pragma unroll
    for (int k = 0; k < 5; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    double e = st.maxerr;
    for (int o = 16; o > 0; o >>= 1) e = fmax(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) {
        if (v[0]) atomicAdd(S.stats + ST_MOLPAIRS, v[0]);
        if (v[1]) atomicAdd(S.stats + ST_ATOMPAIRS, v[1]);
        if (v[2]) atomicAdd(S.stats + (rnd ? ST_HITS_RAND : ST_HITS_REAL), v[2]);
        if (v[3]) atomicAdd(S.stats + ST_GUARD, v[3]);
        if (v[4]) atomicAdd(S.stats + ST_GUARD_PAIRS, v[4]);
        if (e > 0.0) atomicMax(S.stats + ST_MAXERR, (unsigned long long)__double_as_longlong(e));
    }
}

// Images of a candidate pair: along axis k the stencil offsets
// Delta_k = base_k + t * step_k, t < cnt_k.  A single image (cnt = 1 on every
// axis) is the normal case; several images arise when the box is narrower
// than the search range along an axis, and then all images are searched and
// the minimum over them is kept, as the reference's cell list does.
struct Images {
    int base[3];
    int step[3];
    int cnt[3];
};

__device__ __forceinline__ int image_count(const Images &im) { return im.cnt[0] * im.cnt[1] * im.cnt[2]; }

// All Delta == t0 (mod n) inside [-L, L].
__device__ __forceinline__ void axis_images(int t0, int n, int L, int &base, int &cnt) {
    int r = ((t0 + L) % n + n) % n;
    base = -L + r;
    cnt = base > L ? 0 : (L - base) / n + 1;
}

#define CM_FOR_IMAGES(im, DX, DY, DZ)                                       \
    for (int _iz = 0; _iz < (im).cnt[2]; ++_iz)                            \
        for (int _iy = 0; _iy < (im).cnt[1]; ++_iy)                        \
            for (int _ix = 0; _ix < (im).cnt[0]; ++_ix)                    \
                if (int DX = (im).base[0] + _ix * (im).step[0], DY = (im).base[1] + _iy * (im).step[1], \
                    DZ = (im).base[2] + _iz * (im).step[2]; true)

// One direction of a (solute molecule, solvent molecule) result: the record the
// reference keeps in its list for the solvent molecule (src/minimum_distances.jl:12-19),
// already binned.
struct DirRec {
    int within;
    int i_local;   // solute-side atom, index inside its molecule
    int64_t j;     // solvent-side atom, index in the whole selection
    int bin;       // 0-based histogram bin of d
    int ref;       // reference atom within cutoff
    int rbin;      // 0-based bin of d_ref_atom
    int bulk;      // inbulk(...) of the solvent molecule for this solute molecule (src/mddf.jl:55-57)
};

// ------------------------------------------------------------------- buffers
// Frames are processed in chunks.  Every per-frame buffer holds the chunk's
// frames at a fixed stride, and each kernel finds the frame of its work item
// (grid y, or the item's own frame tag), so one launch per stage serves all
// frames of the chunk.
struct Bufs {
    int nf;                         // frames in the chunk
    int ndist;                      // rows per frame of flags / bulk
    int64_t ms, Ns, mv, Nv;
    const FrameGeom *G;             // [nf]
    FrameScratch *FS;               // [nf]
    // the chunk's input coordinates as the caller gave them ([nf][Ns][3] and
    // [nf][Nv][3] at the strides below, FP32 or FP64; xv_raw == xs_raw in self
    // mode): the exact distances are formed from these
    const void *xs_raw, *xv_raw;
    int64_t xs_stride, xv_stride;   // coordinate values from one frame's first atom to the next frame's
    int raw64;                      // 1: FP64 input coordinates
    d4 *off64;                      // [nf][kOffEntries]
    float4 *off32;
    // PAIRS molecules; in self mode the solvent pointers alias the solute ones
    int *scell;                     // [nf][ms]
    float4 *sq32;
    d4 *sq64;
    float4 *so32;                   // [nf][Ns]
    d4 *so64;
    int *vcell;                     // [nf][mv]
    float4 *vq32;
    d4 *vq64;
    float4 *vo32;                   // [nf][Nv]
    d4 *vo64;
    int *ccount, *cstart, *cfill;   // [nf][cs]
    int64_t cs;
    int *cmol;                      // [nf][mv]
    float4 *cq32;                   // [nf][mv] molecule table (FP32 centroid, radius) in cell order
    // random insertion
    int *slot;                      // [nf][ms], -1 where not sampled
    unsigned char *flags;           // [nf][ndist][mv]
    int *bulk;                      // [nf][ndist][mv]
    int *nbulk;                     // [nf][ndist]
    const Sample *samples;          // the chunk's samples; .pad = frame
    // queues of the chunk
    int4 *gq;                       // (s, v, packed delta, frame)
    int gq_cap;
    int2 *rq;                       // (sample, slot)
    int rq_cap;
    int4 *eq;                       // edge queue: 3 int4 per entry (s, v, code, frame), (a | b << 8, rb1, rb2, bin), (d32 bits)
    int eq_cap;
    int *counters;                  // [0] guard queue, [1] random queue, [2] ATOMS queue, [3] edge queue,
                                    // [4] the chunk's real pass is redone without queues (k_queue_check)
    // ATOMS
    int *akey;                      // [nf][Ns]
    float4 *atq32, *asq32;
    d4 *atq64, *asq64;
    int *acount, *astart, *afill;   // [nf][as]
    int64_t as;
    int *avcell;                    // [nf][Nv]
    float4 *avq32;
    d4 *avq64;
    d4 *u64;                        // [nf][Nv]
    float4 *u32;                    // [nf][Nv] FP32 copies of u64 (the FP32 placement)
    float *rc;                      // [nf][mv]
    int *pcell;                     // [placed samples][Nv]
    float4 *pq32;
    d4 *pq64;
    unsigned char *anear;           // [nf][as] cells within a stencil of a solute molecule's atoms
    int4 *aq;                       // ATOMS work queue; count in counters[2]
    int aq_cap;
    int *aslot;                     // random-insertion slots that can reach the solute (y * mv + slot); count in counters[5]
    int aslot_cap;
    // ATOMS candidate grid (one solute molecule, FP32 search): each search
    // cell split into agk^3 fine cells, each with the list of solute atoms
    // that can be the closest (or within the guard band of it) to a point of
    // the fine cell; agk = 0: no grid
    int agk;
    int64_t gfs;                    // fine cells per frame (ncell_cap * agk^3)
    int64_t gcap;                   // entries per frame
    int *gstart;                    // [nf][gfs][buckets + 1]: each fine cell's bucket starts and its end
    int *gpool;                     // [nf]: entries reserved in the frame's pool
    float2 *gedge;                  // [nf][gfs]: smallest distance of a listed atom to the fine cell, list threshold
    float4 *gent;                   // [nf][gcap]: position from the fine cell's search-cell origin, solute atom index
};

// ------------------------------------------------------------ exact distances
// Input coordinates of one atom of frame f (solute or solvent selection),
// widened to FP64 exactly.
__device__ __forceinline__ void raw_atom(const Bufs &B, bool solvent, int f, int64_t atom, double *x) {
    const int64_t i = (int64_t)f * (solvent ? B.xv_stride : B.xs_stride) + atom * 3;
    if (B.raw64) {
        const double *p = (const double *)(solvent ? B.xv_raw : B.xs_raw) + i;
        x[0] = p[0]; x[1] = p[1]; x[2] = p[2];
    } else {
        const float *p = (const float *)(solvent ? B.xv_raw : B.xs_raw) + i;
        x[0] = (double)p[0]; x[1] = (double)p[1]; x[2] = (double)p[2];
    }
}

// The two molecules of one evaluated pair, for the exact distances: the
// solute molecule's atoms and the solvent molecule's atoms from the input
// coordinates, or, for a random-insertion slot, the source molecule placed by
// the slot's draws exactly as the random insertion defines it
// (exact_unwrapped / exact_placed: src/rigid_body.jl:107-137).
struct ExactMol {
    int f;
    int apv, iref;
    int placed;
    int ready;         // placed: xr and cm computed
    int64_t sbase;     // selection index of the solute molecule's first atom
    int64_t vbase;     // selection index of the solvent molecule's (the placed source molecule's) first atom
    double A[9];       // placed: rotation (row-major)
    double ncm[3];     // placed: new centre H fc
    double xr[3];      // placed: the source molecule's reference atom
    double cm[3];      // placed: mean of the unwrapped source atoms
};

__device__ __forceinline__ ExactMol exact_mol(const DevSys &S, int f, int64_t s, int64_t v) {
    ExactMol X;
    X.f = f;
    X.apv = S.apv;
    X.iref = S.iref;
    X.placed = 0;
    X.ready = 1;
    X.sbase = s * S.aps;
    X.vbase = v * S.apv;
    return X;
}

__device__ __forceinline__ ExactMol exact_mol_placed(const DevSys &S, const FrameGeom &G, int f, int64_t s, int jmol,
                                                     const double *fc, const double *A) {
    ExactMol X = exact_mol(S, f, s, jmol);
    X.placed = 1;
    X.ready = 0;
    for (int k = 0; k < 9; ++k) X.A[k] = A[k];
    exact_lat(G, fc, X.ncm);
    return X;
}

__device__ __noinline__ void exact_mol_ready(const Bufs &B, const FrameGeom &G, ExactMol &X) {
    raw_atom(B, true, X.f, X.vbase + X.iref, X.xr);
    double cm[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < X.apv; ++b) {
        double x[3], u[3];
        raw_atom(B, true, X.f, X.vbase + b, x);
        exact_unwrapped(G, x, X.xr, u);
        for (int k = 0; k < 3; ++k) cm[k] = add(cm[k], u[k]);
    }
    for (int k = 0; k < 3; ++k) X.cm[k] = div(cm[k], (double)X.apv);
    X.ready = 1;
}

__device__ __forceinline__ void exact_solute_atom(const Bufs &B, const ExactMol &X, int a, double *x) {
    raw_atom(B, false, X.f, X.sbase + a, x);
}

__device__ __forceinline__ void exact_solvent_atom(const Bufs &B, const FrameGeom &G, ExactMol &X, int b, double *y) {
    raw_atom(B, true, X.f, X.vbase + b, y);
    if (!X.placed) return;
    if (!X.ready) exact_mol_ready(B, G, X);
    double u[3];
    exact_unwrapped(G, y, X.xr, u);
    exact_placed(u, X.cm, X.A, X.ncm, y);
}

// Exact squared distance of solute atom a and solvent atom b of a pair.
__device__ __forceinline__ double exact_pair_d2(const Bufs &B, const FrameGeom &G, ExactMol &X, int a, int b) {
    double x[3], y[3];
    exact_solute_atom(B, X, a, x);
    exact_solvent_atom(B, G, X, b, y);
    return exact_d2(G, x, y);
}

// A pair's molecules as the search kernels name them (a few words, so the
// search loops carry no ExactMol): frame, solute molecule, solvent molecule,
// and for a random-insertion slot the placed source molecule (v), its
// rotation and its fractional centre.
struct ExactRef {
    int f, s, v;
    const double *A;    // nullptr: a real pair
    const double *fc;
};

__device__ __forceinline__ ExactMol exact_mol_of(const DevSys &S, const FrameGeom &G, const ExactRef &r) {
    return r.A ? exact_mol_placed(S, G, r.f, r.s, r.v, r.fc, r.A) : exact_mol(S, r.f, r.s, r.v);
}

// exact_pair_d2 out of line, for the searches' rare exact decisions.
__device__ __noinline__ double exact_pair_ref(const DevSys &S, const Bufs &B, const FrameGeom &G, const ExactRef &r, int a,
                                              int b) {
    ExactMol X = exact_mol_of(S, G, r);
    return exact_pair_d2(B, G, X, a, b);
}

// ---------------------------------------------------------- PAIRS evaluation
// Search pass in precision R over cell-relative coordinates (float4 for the
// FP32 search, d4 for the FP64 search): smallest / second-smallest squared
// distance and the pair (a, b) of the smallest, plus the reference-atom row /
// column minima.
template <typename R>
struct Vec4T;
template <>
struct Vec4T<float> {
    using type = float4;
};
template <>
struct Vec4T<double> {
    using type = d4;
};

template <typename R>
struct PassT {
    R m1, m2;
    int k1;        // a * apv + b
    R r1, r2;
};
using Pass32 = PassT<float>;

__device__ __forceinline__ float sq3(float x, float y, float z) { return fmaf(z, z, fmaf(y, y, x * x)); }
__device__ __forceinline__ double sq3(double x, double y, double z) { return fma(z, z, fma(y, y, x * x)); }
__device__ __forceinline__ float r_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double r_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float r_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double r_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float r_abs(float a) { return fabsf(a); }
__device__ __forceinline__ double r_abs(double a) { return fabs(a); }

template <bool ROW, typename R, typename V>
__device__ __forceinline__ void inner_pass(const V *__restrict__ os, int aps, int apv, int b, R tx, R ty, R tz,
                                           PassT<R> &P) {
    R row = P.r1;
    for (int a = 0; a < aps; ++a) {
        const V oa = os[a];
        const R d2 = sq3(tx - (R)oa.x, ty - (R)oa.y, tz - (R)oa.z);
        P.m2 = r_min(P.m2, r_max(P.m1, d2));
        P.k1 = d2 < P.m1 ? a * apv + b : P.k1;
        P.m1 = r_min(P.m1, d2);
        if (ROW) row = r_min(row, d2);
    }
    if (ROW) P.r1 = row;
}

template <bool SELF, typename R, typename V>
__device__ __forceinline__ void pairs_pass(const DevSys &S, const V *__restrict__ off, const Images &im, V qs, V qv,
                                           const V *__restrict__ os, const V *ov, PassT<R> &P) {
    P.m1 = P.m2 = P.r1 = P.r2 = (R)INFINITY;
    P.k1 = 0;
    const int aps = S.aps, apv = S.apv, iref = S.iref;
    CM_FOR_IMAGES(im, dx, dy, dz) {
        const V o = off[off_index(dx, dy, dz)];
        const R Dx = ((R)qv.x - (R)qs.x) + (R)o.x, Dy = ((R)qv.y - (R)qs.y) + (R)o.y, Dz = ((R)qv.z - (R)qs.z) + (R)o.z;
        for (int b = 0; b < apv; ++b) {
            const V ob = ov[b];
            const R tx = Dx + (R)ob.x, ty = Dy + (R)ob.y, tz = Dz + (R)ob.z;
            if (b == iref) inner_pass<true>(os, aps, apv, b, tx, ty, tz, P);
            else inner_pass<false>(os, aps, apv, b, tx, ty, tz, P);
            if (SELF) {
                const V oa = os[iref];
                P.r2 = r_min(P.r2, sq3(tx - (R)oa.x, ty - (R)oa.y, tz - (R)oa.z));
            }
        }
    }
}

// Exact minimum search with the reference's tie rule: among equal distances
// the pair visited last wins (src/minimum_distances.jl:33-37, the new pair
// replaces the record unless the record is strictly closer), restated as the
// largest (solute atom, solvent atom) index pair.  Distances are compared as
// d = sqrt(d2) like the reference; d2 decides when it is far enough from the
// current best that the square roots cannot tie.
struct Best64 {
    double d2, d, lo, hi;
    int a, b;     // direction 1: key (a, b)
    int a2, b2;   // direction 2 (self mode): key (b, a)
};

__device__ __forceinline__ void best_init(Best64 &B) {
    B.d2 = INFINITY;
    B.d = -1.0;
    B.lo = INFINITY;
    B.hi = INFINITY;
    B.a = B.b = B.a2 = B.b2 = -1;
}

template <bool DIR2>
__device__ __forceinline__ void best_update(Best64 &B, double d2, int a, int b) {
    if (d2 < B.lo) {
        B.d2 = d2;
        B.d = -1.0;
        B.lo = mul(d2, 1.0 - 0x1.0p-50);
        B.hi = mul(d2, 1.0 + 0x1.0p-50);
        B.a = a; B.b = b; B.a2 = a; B.b2 = b;
    } else if (d2 <= B.hi) {
        double d = sqrt(d2);
        if (B.d < 0.0) B.d = sqrt(B.d2);
        if (d < B.d) {
            B.d2 = d2;
            B.d = d;
            B.lo = mul(d2, 1.0 - 0x1.0p-50);
            B.hi = mul(d2, 1.0 + 0x1.0p-50);
            B.a = a; B.b = b; B.a2 = a; B.b2 = b;
        } else if (d == B.d) {
            if (a > B.a || (a == B.a && b > B.b)) { B.a = a; B.b = b; }
            if (DIR2 && (b > B.b2 || (b == B.b2 && a > B.a2))) { B.a2 = a; B.b2 = b; }
        }
    }
}

__device__ __forceinline__ double best_d(Best64 &B) {
    if (B.d < 0.0) B.d = sqrt(B.d2);
    return B.d;
}

struct Exact64 {
    Best64 B;
    double rr1, rr2;   // exact squared minima (within cutoff) of the row / column
    long long evals;
};

// Exact scan of a molecule pair.  An atom pair is evaluated exactly
// (exact_d2 on the input coordinates, the smallest over the images) only if
// its squared distance in the search precision R, the smallest over the
// images, is at most the threshold of an accumulator it feeds (thr_arg: the
// minimum; thr_r1: row of v's reference atom; thr_r2: column of s's reference
// atom); each threshold keeps every pair that can hold the exact minimum of
// its accumulator.
template <bool SELF, typename R, typename V>
__device__ __noinline__ void pairs_exact(const DevSys &S, const FrameGeom &G, const Bufs &B, const ExactRef &xref,
                                         const V *__restrict__ off, const Images &im, V qs, V qv, const V *os, const V *ov,
                                         R thr_arg, R thr_r1, R thr_r2, Exact64 &E) {
    ExactMol X = exact_mol_of(S, G, xref);
    best_init(E.B);
    E.rr1 = INFINITY;
    E.rr2 = INFINITY;
    E.evals = 0;
    const int aps = S.aps, apv = S.apv, iref = S.iref;
    const double cut2 = S.cut2;
    for (int b = 0; b < apv; ++b) {
        const V ob = ov[b];
        double yb[3];
        bool have_y = false;
        for (int a = 0; a < aps; ++a) {
            const V oa = os[a];
            R m = (R)INFINITY;
            CM_FOR_IMAGES(im, ix, iy, iz) {
                const V o = off[off_index(ix, iy, iz)];
                const R tx = (((R)qv.x - (R)qs.x) + (R)o.x) + (R)ob.x;
                const R ty = (((R)qv.y - (R)qs.y) + (R)o.y) + (R)ob.y;
                const R tz = (((R)qv.z - (R)qs.z) + (R)o.z) + (R)ob.z;
                m = r_min(m, sq3(tx - (R)oa.x, ty - (R)oa.y, tz - (R)oa.z));
            }
            const bool need = m <= thr_arg || (b == iref && m <= thr_r1) || (SELF && a == iref && m <= thr_r2);
            if (!need) continue;
            if (!have_y) {
                exact_solvent_atom(B, G, X, b, yb);
                have_y = true;
            }
            double xa[3];
            exact_solute_atom(B, X, a, xa);
            const double d2 = exact_d2(G, xa, yb);
            E.evals++;
            if (d2 <= cut2) {
                if (b == iref) E.rr1 = fmin(E.rr1, d2);
                if (SELF && a == iref) E.rr2 = fmin(E.rr2, d2);
                best_update<SELF>(E.B, d2, a, b);
            }
        }
    }
}

__device__ __forceinline__ float r_rint(float x) { return rintf(x); }
__device__ __forceinline__ double r_rint(double x) { return rint(x); }
__device__ __forceinline__ float r_ceil(float x) { return ceilf(x); }
__device__ __forceinline__ double r_ceil(double x) { return ceil(x); }
__device__ __forceinline__ float r_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double r_sqrt(double x) { return sqrt(x); }
// a * a rounded up: thresholds that must not lose a pair to rounding
__device__ __forceinline__ float r_sq_ru(float x) { return __fmul_ru(x, x); }
__device__ __forceinline__ double r_sq_ru(double x) { return __dmul_ru(x, x); }

// Bin from a search-precision distance, or -1 when it lies in the band
// around a bin edge.
template <typename R>
__device__ __forceinline__ int bin_of(const GuardT<R> &g, R d) {
    const R k = d * g.inv_bs;
    const R r = r_rint(k);
    if (r_abs(k - r) <= g.bin_band) return -1;
    const int b = (int)r_ceil(k);
    return (b < 1 ? 1 : b) - 1;
}
__device__ __forceinline__ int bin32(const Guard &g, float d) { return bin_of<float>(g, d); }

__device__ __forceinline__ DirRec dir_none(const DevSys &S) {
    DirRec r;
    r.within = 0; r.i_local = -1; r.j = -1; r.bin = -1; r.ref = 0; r.rbin = -1;
    r.bulk = S.usecutoff ? 0 : 1;
    return r;
}

__device__ __forceinline__ int inbulk64(const DevSys &S, bool within, double d) {
    return S.usecutoff ? (within && d > S.dbulk) : !within;
}

// Records from an exact scan.
template <bool SELF>
__device__ __forceinline__ void records_from_exact(const DevSys &S, Exact64 &E, int s, int64_t v, DirRec &r1, DirRec &r2) {
    r1 = dir_none(S);
    r2 = dir_none(S);
    if (!(E.B.d2 <= S.cut2)) return;
    double d = best_d(E.B);
    int bin = setbin0(d, S.binstep);
    r1.within = 1;
    r1.i_local = E.B.a;
    r1.j = v * S.apv + E.B.b;
    r1.bin = bin;
    r1.bulk = inbulk64(S, true, d);
    if (E.rr1 <= S.cut2) { r1.ref = 1; r1.rbin = setbin0(sqrt(E.rr1), S.binstep); }
    if (SELF) {
        r2.within = 1;
        r2.i_local = E.B.b2;
        r2.j = (int64_t)s * S.aps + E.B.a2;
        r2.bin = bin;
        r2.bulk = r1.bulk;
        if (E.rr2 <= S.cut2) { r2.ref = 1; r2.rbin = setbin0(sqrt(E.rr2), S.binstep); }
    }
}

// Decide one molecule pair from its search pass (precision R), with the exact
// rules wherever a value lies within the guard band of its decision boundary.
// Produces exactly the records of an unfiltered exact scan.
template <bool SELF, typename R, typename V>
__device__ void pairs_decide(const DevSys &S, const FrameGeom &G, const Bufs &B, const ExactRef &X, const GuardT<R> &g,
                             const PassT<R> &P, const V *__restrict__ off, const Images &im, V qs, V qv, const V *os,
                             const V *ov, int s, int64_t v, DirRec &r1, DirRec &r2, LocalStats &st) {
    r1 = dir_none(S);
    r2 = dir_none(S);
    if (P.m1 > g.cutp2) return;  // every pair is beyond the cutoff
    const R d1 = r_sqrt(P.m1);
    const bool amb = P.m1 >= g.cutm2 || (r_sqrt(P.m2) - d1) <= g.two_delta;
    if (amb) {
        const R thr = r_sq_ru(d1 + g.two_delta);
        R thr1 = (R)-1, thr2 = (R)-1;
        if (P.r1 <= g.cutp2) thr1 = r_sq_ru(r_sqrt(P.r1) + g.two_delta);
        if (SELF && P.r2 <= g.cutp2) thr2 = r_sq_ru(r_sqrt(P.r2) + g.two_delta);
        Exact64 E;
        pairs_exact<SELF>(S, G, B, X, off, im, qs, qv, os, ov, thr, thr1, thr2, E);
        records_from_exact<SELF>(S, E, s, v, r1, r2);
        st.guard++;
        st.guard_pairs += E.evals;
        if (E.B.d2 <= S.cut2) st.maxerr = fmax(st.maxerr, fabs((double)d1 - best_d(E.B)));
        return;
    }
    // unambiguous: the search's minimum pair is the exact minimum pair, within cutoff
    const int a = P.k1 / S.apv, b = P.k1 - a * S.apv;
    int bin = bin_of(g, d1);
    double d64 = -1.0;
    if (bin < 0 || (S.usecutoff && d1 >= g.dbulk_lo && d1 <= g.dbulk_hi)) {
        d64 = sqrt(exact_pair_ref(S, B, G, X, a, b));
        bin = setbin0(d64, S.binstep);
        st.guard++;
        st.guard_pairs += 1;
        st.maxerr = fmax(st.maxerr, fabs((double)d1 - d64));
    }
    const int bulk = S.usecutoff ? (d64 >= 0.0 ? (d64 > S.dbulk) : (d1 > g.dbulk_hi)) : 0;
    r1.within = 1;
    r1.i_local = a;
    r1.j = v * S.apv + b;
    r1.bin = bin;
    r1.bulk = bulk;
    if (SELF) {
        r2.within = 1;
        r2.i_local = b;
        r2.j = (int64_t)s * S.aps + a;
        r2.bin = bin;
        r2.bulk = bulk;
    }
    // reference-atom rows (and columns in self mode)
    for (int dir = 0; dir < (SELF ? 2 : 1); ++dir) {
        const R rm = dir == 0 ? P.r1 : P.r2;
        DirRec &r = dir == 0 ? r1 : r2;
        if (rm > g.cutp2) continue;
        int rb = -1;
        if (rm < g.cutm2) rb = bin_of(g, r_sqrt(rm));
        if (rb >= 0) {
            r.ref = 1;
            r.rbin = rb;
            continue;
        }
        const R thr = r_sq_ru(r_sqrt(rm) + g.two_delta);
        Exact64 E;
        pairs_exact<SELF>(S, G, B, X, off, im, qs, qv, os, ov, (R)-1, dir == 0 ? thr : (R)-1, dir == 1 ? thr : (R)-1, E);
        const double rr = dir == 0 ? E.rr1 : E.rr2;
        st.guard++;
        st.guard_pairs += E.evals;
        if (rr <= S.cut2) {
            r.ref = 1;
            r.rbin = setbin0(sqrt(rr), S.binstep);
        }
    }
}

__device__ __forceinline__ unsigned char flag_code(const DirRec &r) { return r.within ? (unsigned char)(1 + (r.bulk ? 1 : 0)) : 0; }

__device__ __forceinline__ int pack_delta(int dx, int dy, int dz) { return (dx + 16) | ((dy + 16) << 5) | ((dz + 16) << 10); }
__device__ __forceinline__ void unpack_delta(int c, int &dx, int &dy, int &dz) {
    dx = (c & 31) - 16;
    dy = ((c >> 5) & 31) - 16;
    dz = ((c >> 10) & 31) - 16;
}

// ------------------------------------------------------------------ geometry
__device__ __forceinline__ double norm3d(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

// Largest |Hn v| over the 8 sign patterns of v = (+-l0, +-l1, +-l2).
__device__ double corner_norm(const FrameGeom &G, double l0, double l1, double l2) {
    double best = 0.0;
    for (int m = 0; m < 8; ++m) {
        double v[3];
        matvec_cm(G.Hn, (m & 1) ? -l0 : l0, (m & 2) ? -l1 : l1, (m & 4) ? -l2 : l2, v);
        best = fmax(best, norm3d(v[0], v[1], v[2]));
    }
    return best;
}

// Stencil half-widths for a search range; false if the offset table is too small.
__device__ bool stencil(const FrameGeom &G, double range, int *L) {
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
        int l = (int)ceil(range * (1.0 + 1e-9) / G.cw[k]);
        if (l < 1) l = 1;
        if (l > kLT) { ok = false; l = kLT; }
        L[k] = l;
    }
    return ok;
}

// ------------------------------------------------------------------- kernels
// Per-frame offset tables: off(Delta) = Hn Delta for Delta in [-kLT, kLT]^3.
__device__ __forceinline__ void k_offtable_body(const uint3 blockIdx, const dim3 gridDim, const Bufs &B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, f = blockIdx.y;
    if (i >= kOffEntries) return;
    const int dx = i % kLTW - kLT, dy = (i / kLTW) % kLTW - kLT, dz = i / (kLTW * kLTW) - kLT;
    double v[3];
    matvec_cm(B.G[f].Hn, (double)dx, (double)dy, (double)dz, v);
    B.off64[(int64_t)f * kOffEntries + i] = make_d4(v[0], v[1], v[2], 0.0);
    B.off32[(int64_t)f * kOffEntries + i] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
}

__global__ void k_offtable(Bufs B) {
    k_offtable_body(blockIdx, gridDim, B);
}

template <typename T>
__device__ __forceinline__ void load_xyz(const T *p, double *x) {
    x[0] = (double)p[0];
    x[1] = (double)p[1];
    x[2] = (double)p[2];
}

// Atomic maximum of a nonnegative float (its bits order as int) of the largest
// value over the calling warp's active lanes (one atomic per warp).
__device__ __forceinline__ void warp_max_pos(float *addr, float v) {
    const unsigned mask = __activemask();
    const int m = __reduce_max_sync(mask, __float_as_int(v));
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) atomicMax((int *)addr, m);
}

// PAIRS prep, one thread per molecule (grid y = frame).  The molecule is made
// whole around its first atom (minimum image of each atom's displacement), its
// centroid c = x_0 + mean(d) is binned, and its atoms are stored as FP64 and
// FP32 offsets from the centroid; the radius is the largest offset (rounded
// up).  Displacements shorter than 0.45 of the narrowest cell width are their
// own minimum image, so the FP64 unwrap runs only for longer ones.
template <typename T>
__global__ void k_prep_pairs(Bufs B, const T *__restrict__ xyz, int64_t xyz_stride, int solvent_side, int count_cells) {
    const int f = blockIdx.y;
    const int nmol = (int)(solvent_side ? B.mv : B.ms);
    const int64_t Nmol_atoms = solvent_side ? B.Nv : B.Ns;
    const int apm = (int)(Nmol_atoms / nmol);
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmol) return;
    const FrameGeom &G = B.G[f];
    int *mcell = (solvent_side ? B.vcell : B.scell) + (int64_t)f * nmol;
    float4 *mq32 = (solvent_side ? B.vq32 : B.sq32) + (int64_t)f * nmol;
    d4 *mq64 = (solvent_side ? B.vq64 : B.sq64) + (int64_t)f * nmol;
    float4 *mo32 = (solvent_side ? B.vo32 : B.so32) + (int64_t)f * Nmol_atoms;
    d4 *mo64 = (solvent_side ? B.vo64 : B.so64) + (int64_t)f * Nmol_atoms;
    FrameScratch &F = B.FS[f];
    const T *x = xyz + (int64_t)f * xyz_stride + (int64_t)m * apm * 3;
    const int64_t base = (int64_t)m * apm;
    double x0[3];
    load_xyz(x, x0);
    const float wlim = (float)(0.45 * fmin(G.w[0], fmin(G.w[1], G.w[2])));
    double sx = 0.0, sy = 0.0, sz = 0.0, xm = 0.0;
    for (int a = 0; a < apm; ++a) {
        double xa[3], d[3];
        load_xyz(x + 3 * a, xa);
        xm = fmax(xm, fmax(fabs(xa[0]), fmax(fabs(xa[1]), fabs(xa[2]))));
        for (int k = 0; k < 3; ++k) d[k] = sub(xa[k], x0[k]);
        const float fx = (float)d[0], fy = (float)d[1], fz = (float)d[2];
        if (fmaf(fz, fz, fmaf(fy, fy, fx * fx)) > wlim * wlim) unwrap(G, d);
        mo64[base + a] = make_d4(d[0], d[1], d[2], 0.0);
        sx = add(sx, d[0]);
        sy = add(sy, d[1]);
        sz = add(sz, d[2]);
    }
    const double n = (double)apm;
    const double mx = div(sx, n), my = div(sy, n), mz = div(sz, n);
    int c[3];
    double q[3];
    bin_position(G, add(x0[0], mx), add(x0[1], my), add(x0[2], mz), c, q);
    const int cell = cell_linear(G, c[0], c[1], c[2]);
    float r = 0.f;
    for (int a = 0; a < apm; ++a) {
        d4 w = mo64[base + a];
        w.x = sub(w.x, mx);
        w.y = sub(w.y, my);
        w.z = sub(w.z, mz);
        mo64[base + a] = w;
        const float fx = (float)w.x, fy = (float)w.y, fz = (float)w.z;
        mo32[base + a] = make_float4(fx, fy, fz, 0.f);
        r = fmaxf(r, norm3f(fx, fy, fz));
    }
    // radius bound: FP32 norm of the rounded offsets, enlarged to cover rounding
    const float rf = r * (1.0f + 0x1.0p-18f) + 1e-5f;
    mcell[m] = cell;
    mq64[m] = make_d4(q[0], q[1], q[2], 0.0);
    mq32[m] = make_float4((float)q[0], (float)q[1], (float)q[2], rf);
    if (count_cells) atomicAdd(B.ccount + (int64_t)f * B.cs + cell, 1);
    warp_max_pos(solvent_side ? &F.rmax_v : &F.rmax_s, rf);
    warp_max_pos(&F.xmax, __double2float_ru(xm));
}

// Exclusive scans of the chunk's per-frame count arrays (one CTA of 1024
// threads per frame): start[0..n] and a copy in fill for the scatter.  n is
// the frame's cell count times `mult` (1: molecule cells, ms: per-molecule
// atom cells).
__device__ __forceinline__ void k_scan_body(const uint3 blockIdx, const dim3 gridDim, const Bufs &B, int atoms_layout) {
    __shared__ int wsum[32];
    const int f = blockIdx.x;
    const int64_t stride = atoms_layout ? B.as : B.cs;
    const int *count = (atoms_layout ? B.acount : B.ccount) + (int64_t)f * stride;
    int *start = (atoms_layout ? B.astart : B.cstart) + (int64_t)f * stride;
    int *fill = (atoms_layout ? B.afill : B.cfill) + (int64_t)f * stride;
    const int n = B.G[f].ncell * (atoms_layout ? (int)B.ms : 1);
    const int t = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int lo = t * per, hi = min(n, lo + per);
    int local = 0;
    for (int i = lo; i < hi; ++i) local += count[i];
    const int lane = t & 31, w = t >> 5;
    int v = local;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
        int s = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    int excl = v - local + (w > 0 ? wsum[w - 1] : 0);
    for (int i = lo; i < hi; ++i) {
        start[i] = excl;
        fill[i] = excl;
        excl += count[i];
    }
    if (hi == n && lo < hi) start[n] = excl;
    if (n == 0 && t == 0) start[0] = 0;
}

__global__ void __launch_bounds__(1024) k_scan(Bufs B, int atoms_layout) {
    k_scan_body(blockIdx, gridDim, B, atoms_layout);
}

__global__ void k_scatter_mols(Bufs B, int self) {
    const int f = blockIdx.y;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= B.mv) return;
    const int *mcell = (self ? B.scell : B.vcell) + (int64_t)f * B.mv;
    const int p = atomicAdd(B.cfill + (int64_t)f * B.cs + mcell[m], 1);
    B.cmol[(int64_t)f * B.mv + p] = m;
    B.cq32[(int64_t)f * B.mv + p] = (self ? B.sq32 : B.vq32)[(int64_t)f * B.mv + m];
}

// Images of a PAIRS candidate from its packed stencil offset.
__device__ __forceinline__ Images images_of(const FrameGeom &G, const FrameScratch &F, int code) {
    int d[3];
    unpack_delta(code, d[0], d[1], d[2]);
    Images im;
    for (int k = 0; k < 3; ++k) {
        if (F.multi & (1 << k)) {
            axis_images(d[k], G.n[k], F.L[k], im.base[k], im.cnt[k]);
            im.step[k] = G.n[k];
        } else {
            im.base[k] = d[k];
            im.cnt[k] = 1;
            im.step[k] = 0;
        }
    }
    return im;
}

// Pointers of one frame of a PAIRS chunk.
struct PairsFrame {
    const FrameGeom *G;
    FrameScratch *F;
    const d4 *off64;
    const float4 *off32;
    const int *scell;
    const float4 *sq32;
    const d4 *sq64;
    const float4 *so32;
    const d4 *so64;
    const float4 *vq32;
    const d4 *vq64;
    const float4 *vo32;
    const d4 *vo64;
    const int *cstart;
    const int *cmol;
    int *slot;
    unsigned char *flags;
    int *bulk;
    int *nbulk;
};

__device__ __forceinline__ PairsFrame pairs_frame(const Bufs &B, int f, bool self) {
    PairsFrame P;
    P.G = B.G + f;
    P.F = B.FS + f;
    P.off64 = B.off64 + (int64_t)f * kOffEntries;
    P.off32 = B.off32 + (int64_t)f * kOffEntries;
    P.scell = B.scell + (int64_t)f * B.ms;
    P.sq32 = B.sq32 + (int64_t)f * B.ms;
    P.sq64 = B.sq64 + (int64_t)f * B.ms;
    P.so32 = B.so32 + (int64_t)f * B.Ns;
    P.so64 = B.so64 + (int64_t)f * B.Ns;
    P.vq32 = (self ? B.sq32 : B.vq32) + (int64_t)f * B.mv;
    P.vq64 = (self ? B.sq64 : B.vq64) + (int64_t)f * B.mv;
    P.vo32 = (self ? B.so32 : B.vo32) + (int64_t)f * B.Nv;
    P.vo64 = (self ? B.so64 : B.vo64) + (int64_t)f * B.Nv;
    P.cstart = B.cstart + (int64_t)f * B.cs;
    P.cmol = B.cmol + (int64_t)f * B.mv;
    P.slot = B.slot ? B.slot + (int64_t)f * B.ms : nullptr;
    P.flags = B.flags ? B.flags + (int64_t)f * B.ndist * B.mv : nullptr;
    P.bulk = B.bulk ? B.bulk + (int64_t)f * B.ndist * B.mv : nullptr;
    P.nbulk = B.nbulk ? B.nbulk + (int64_t)f * B.ndist : nullptr;
    return P;
}

// Stencil walk of one solute molecule by one warp: every solvent molecule
// whose bounding sphere reaches the solute's (cut_pre) is handed to
// process(v, code) one candidate per lane, 32 at a time, through a warp queue.
template <bool SELF, typename Proc>
__device__ __forceinline__ void walk_candidates(const FrameGeom &G, const FrameScratch &F, int s, int sc, float4 qs32,
                                                const float4 *__restrict__ off32, const float4 *__restrict__ vq32,
                                                const int *__restrict__ cstart, const int *__restrict__ cmol, int *qv,
                                                int *qi, int lane, Proc &&process) {
    const int n0 = G.n[0], n1 = G.n[1], n2 = G.n[2];
    const bool m0 = F.multi & 1, m1 = F.multi & 2, m2 = F.multi & 4;
    const bool anymulti = F.multi != 0;
    const int e0 = m0 ? n0 : 2 * F.L[0] + 1, e1 = m1 ? n1 : 2 * F.L[1] + 1, e2 = m2 ? n2 : 2 * F.L[2] + 1;
    const int cx = sc % n0, cy = (sc / n0) % n1, cz = sc / (n0 * n1);
    const float rsc = F.g.cut_pre + qs32.w;
    int cnt = 0;
    for (int iz = 0; iz < e2; ++iz) {
        const int dz = m2 ? iz - cz : iz - F.L[2];
        const int zc = m2 ? iz : wrap_cell(cz + dz, n2);
        for (int iy = 0; iy < e1; ++iy) {
            const int dy = m1 ? iy - cy : iy - F.L[1];
            const int yc = m1 ? iy : wrap_cell(cy + dy, n1);
            for (int ix = 0; ix < e0; ++ix) {
                const int dx = m0 ? ix - cx : ix - F.L[0];
                const int xc = m0 ? ix : wrap_cell(cx + dx, n0);
                const int cell = (zc * n1 + yc) * n0 + xc;
                const int beg = cstart[cell], end = cstart[cell + 1];
                if (beg == end) continue;
                const int code = pack_delta(dx, dy, dz);
                float4 of = make_float4(0.f, 0.f, 0.f, 0.f);
                if (!anymulti) of = off32[off_index(dx, dy, dz)];
                const float bx = of.x - qs32.x, by = of.y - qs32.y, bz = of.z - qs32.z;
                for (int p0 = beg; p0 < end; p0 += 32) {
                    const int p = p0 + lane;
                    bool cand = false;
                    int v = 0;
                    if (p < end) {
                        v = cmol[p];
                        cand = !SELF || v > s;
                        if (cand && !anymulti) {
                            const float4 q = vq32[v];
                            const float ex = q.x + bx, ey = q.y + by, ez = q.z + bz;
                            const float rr = rsc + q.w;
                            cand = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) <= rr * rr;
                        }
                    }
                    const unsigned mask = __ballot_sync(0xffffffffu, cand);
                    const int pos = cnt + __popc(mask & ((1u << lane) - 1u));
                    if (cand) { qv[pos] = v; qi[pos] = code; }
                    cnt += __popc(mask);
                    if (cnt >= 32) {
                        __syncwarp();
                        process(qv[lane], qi[lane]);
                        __syncwarp();
                        int rest = cnt - 32, tv = 0, ti = 0;
                        if (lane < rest) { tv = qv[32 + lane]; ti = qi[32 + lane]; }
                        __syncwarp();
                        if (lane < rest) { qv[lane] = tv; qi[lane] = ti; }
                        cnt = rest;
                        __syncwarp();
                    }
                }
            }
        }
    }
    __syncwarp();
    if (lane < cnt) process(qv[lane], qi[lane]);
    __syncwarp();
}

// Records of both directions written into the histograms and the bulk flags.
template <bool SELF>
__device__ __forceinline__ void emit(const DevSys &S, const SHist &h, const DirRec &r1, const DirRec &r2, int s, int v,
                                     const int *__restrict__ slot, unsigned char *__restrict__ flags, LocalStats &st) {
    if (r1.within) { apply_hit(S, h, false, r1.bin, r1.i_local, r1.j, r1.ref, r1.rbin); st.hits++; }
    if (SELF && r2.within) { apply_hit(S, h, false, r2.bin, r2.i_local, r2.j, r2.ref, r2.rbin); st.hits++; }
    if (slot) {
        const int sl = slot[s];
        if (sl >= 0) flags[(int64_t)sl * S.mv + v] = flag_code(r1);
        if (SELF) {
            const int vs = slot[v];
            if (vs >= 0) flags[(int64_t)vs * S.mv + s] = flag_code(r2);
        }
    }
}

// PAIRS real pass, generic (any molecule size, FP32 or FP64): one warp per
// (frame, solute molecule) work item, every record decided where it is found
// (no queues).  only_multi 0: every frame; 1: only the frames that need
// several images per molecule pair (the rest were done by the specialised
// FP32 kernel); 2: every frame, if k_queue_check raised the chunk's redo flag.
template <bool FP32, bool SELF>
__global__ void __launch_bounds__(kWarps * 32) k_pairs_real(DevSys S, Bufs B, int only_multi) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    const int hw = hist_words(S);
    float4 *os_all = (float4 *)(smem_raw + (((size_t)hw * 4 + 15) & ~(size_t)15));
    int *q_all = (int *)(os_all + kWarps * kMaxSmallMol);
    if (only_multi == 2) {
        if (B.counters[4] == 0) return;
    } else if (only_multi) {
        // nothing to do unless a frame of the chunk needs several images
        int any = 0;
        for (int f = threadIdx.x; f < B.nf; f += blockDim.x) any |= B.FS[f].multi;
        if (!__syncthreads_or(any)) return;
    }
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4 *os = os_all + warp * kMaxSmallMol;
    int *qv = q_all + warp * kQueue * 2;
    int *qi = qv + kQueue;
    LocalStats st;
    const int64_t items = (int64_t)B.nf * B.ms;
    for (int64_t t = (int64_t)blockIdx.x * kWarps + warp; t < items; t += (int64_t)gridDim.x * kWarps) {
        const int f = (int)(t / B.ms), s = (int)(t - (int64_t)f * B.ms);
        const PairsFrame Pf = pairs_frame(B, f, SELF);
        const FrameGeom &G = *Pf.G;
        const FrameScratch &F = *Pf.F;
        if (only_multi == 1 && !F.multi) continue;
        if (!F.ok) {
            if (lane == 0) raise_err(S, ERR_STENCIL);
            continue;
        }
        const float4 qs32 = Pf.sq32[s];
        const d4 qs64 = Pf.sq64[s];
        __syncwarp();
        for (int a = lane; a < S.aps; a += 32) os[a] = Pf.so32[(int64_t)s * S.aps + a];
        __syncwarp();
        auto process = [&](int v, int code) {
            const Images im = images_of(G, F, code);
            DirRec r1, r2;
            st.molpairs++;
            st.atompairs += (unsigned long long)S.aps * S.apv * image_count(im);
            const ExactRef X{f, s, v, nullptr, nullptr};
            if (FP32) {
                const float4 qv32 = Pf.vq32[v];
                const float4 *ov32 = Pf.vo32 + (int64_t)v * S.apv;
                Pass32 P;
                pairs_pass<SELF>(S, Pf.off32, im, qs32, qv32, os, ov32, P);
                pairs_decide<SELF>(S, G, B, X, F.g, P, Pf.off32, im, qs32, qv32, (const float4 *)os, ov32, s, v, r1, r2, st);
            } else {
                const d4 qv64 = Pf.vq64[v];
                const d4 *ov64 = Pf.vo64 + (int64_t)v * S.apv;
                const d4 *os64 = Pf.so64 + (int64_t)s * S.aps;
                PassT<double> P;
                pairs_pass<SELF>(S, Pf.off64, im, qs64, qv64, os64, ov64, P);
                pairs_decide<SELF>(S, G, B, X, F.g64, P, Pf.off64, im, qs64, qv64, os64, ov64, s, v, r1, r2, st);
            }
            emit<SELF>(S, h, r1, r2, s, v, Pf.slot, Pf.flags, st);
        };
        walk_candidates<SELF>(G, F, s, Pf.scell[s], qs32, Pf.off32, Pf.vq32, Pf.cstart, Pf.cmol, qv, qi, lane, process);
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// After the FP32 real pass, its guard and edge kernels: if a queue
// overflowed (records past the capacity were dropped), the accumulators and
// statistics go back to their values before the real pass and the chunk's
// redo flag is raised, so k_pairs_real (mode 2) decides every record of the
// chunk again without queues.  Any grid; returns at once without an overflow.
__global__ void k_queue_check(Bufs B, unsigned long long *__restrict__ hist, const unsigned long long *__restrict__ snap,
                              int64_t n, unsigned long long *__restrict__ stats,
                              const unsigned long long *__restrict__ stats_snap) {
    if (B.counters[0] <= B.gq_cap && B.counters[3] <= B.eq_cap) return;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t i = t0; i < n; i += (int64_t)gridDim.x * blockDim.x) hist[i] = snap[i];
    if (t0 < ST_N) stats[t0] = stats_snap[t0];
    if (t0 == 0) B.counters[4] = 1;
}

// Bulk-molecule list of each distinct sampled solute molecule of each frame,
// ascending (src/mddf.jl:406-415); one CTA per (frame, sampled molecule) entry
// of `tab` = (frame, distinct index, solute molecule).  Clears the molecule's
// entry of the slot table when done (it was set by k_frame_consts).
__device__ __forceinline__ void k_bulk_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B, const int4 *__restrict__ tab) {
    __shared__ int wsum[32];
    __shared__ int carry;
    const int4 e = tab[blockIdx.x];
    const int f = e.x, d = e.y, s = e.z;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned char *fl = B.flags + ((int64_t)f * B.ndist + d) * B.mv;
    int *out = B.bulk + ((int64_t)f * B.ndist + d) * B.mv;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < B.mv; base += blockDim.x) {
        const int v = base + threadIdx.x;
        int keep = 0;
        if (v < B.mv && !(S.self && v == s)) {
            const unsigned char c = fl[v];
            keep = S.usecutoff ? (c == 2) : (c == 0);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) wsum[w] = __popc(m);
        __syncthreads();
        if (w == 0) {
            int x = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            wsum[lane] = x;
        }
        __syncthreads();
        const int pos = carry + (w > 0 ? wsum[w - 1] : 0) + __popc(m & ((1u << lane) - 1u));
        if (keep) out[pos] = v;
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        B.nbulk[(int64_t)f * B.ndist + d] = carry;
        B.slot[(int64_t)f * B.ms + s] = -1;
    }
}

__global__ void __launch_bounds__(1024) k_bulk(const DevSys S, Bufs B, const int4 *__restrict__ tab) {
    k_bulk_body(blockIdx, gridDim, S, B, tab);
}

// Draws of one placement slot, in stream order: bulk pick, centre, angles.
struct Placement {
    int jmol;
    double fc[3];
    uint64_t st;  // stream state after the centre (angles follow)
};

__device__ __forceinline__ Placement draw_placement(const DevSys &S, int64_t frame_id, const Sample &sm, int k, const int *bulk,
                                                   const int *nbulk) {
    Placement P;
    uint64_t st = cmfeed::key(S.seed, cmfeed::kTagSlot, (uint64_t)frame_id, (uint64_t)sm.s,
                              ((uint64_t)(uint32_t)sm.rep << 32) | (uint64_t)(uint32_t)k);
    const int nb = nbulk[sm.d];
    if (nb > 0) P.jmol = bulk[(int64_t)sm.d * S.mv + (int64_t)cmfeed::below(st, (uint64_t)nb)];
    else P.jmol = (int)cmfeed::below(st, (uint64_t)S.mv);
    for (int q = 0; q < 3; ++q) P.fc[q] = cmfeed::uniform(st);
    P.st = st;
    return P;
}

__device__ __forceinline__ void draw_rotation(uint64_t &st, double *A) {
    double cb, sb, cg, sg, ct, stt;
    cmfeed::angle(st, cb, sb);
    cmfeed::angle(st, cg, sg);
    cmfeed::angle(st, ct, stt);
    cmfeed::eulermat(cb, sb, cg, sg, ct, stt, A);
}

// draw_rotation for the FP32 search: cmfeed::angle32's (cos, sin) (the same
// draws and acceptance as cmfeed::angle, within 3.01 u of its values, u =
// 2^-24) and eulermat's products in FP32: every entry within 20 u of the FP64
// matrix's (two-factor products 7.01 u, the three-factor sums 19.1 u).
__device__ __forceinline__ void draw_rotation32(uint64_t &st, float *A) {
    float c1, s1, c2, s2, c3, s3;
    cmfeed::angle32(st, c1, s1);
    cmfeed::angle32(st, c2, s2);
    cmfeed::angle32(st, c3, s3);
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

// draw_placement's draws as integers: the bulk pick and the centre's three
// 53-bit uniforms U_q = fk[q] 2^-53; returns the stream state after them
// (the angles follow).
__device__ __forceinline__ uint64_t draw_slot_bits(const DevSys &S, int64_t frame_id, const Sample &sm, int k,
                                                   const int *bulk, const int *nbulk, int &jmol, uint64_t *fk) {
    uint64_t st = cmfeed::key(S.seed, cmfeed::kTagSlot, (uint64_t)frame_id, (uint64_t)sm.s,
                              ((uint64_t)(uint32_t)sm.rep << 32) | (uint64_t)(uint32_t)k);
    const int nb = nbulk[sm.d];
    if (nb > 0) jmol = bulk[(int64_t)sm.d * S.mv + (int64_t)cmfeed::below(st, (uint64_t)nb)];
    else jmol = (int)cmfeed::below(st, (uint64_t)S.mv);
    for (int q = 0; q < 3; ++q) fk[q] = cmfeed::next(st) >> 11;
    return st;
}

// The centre's cell and its FP32 position from that cell's origin, from the
// 53-bit uniforms: c = floor(U n) and g = U n - c exactly (integer product
// fk n < 2^63), q0 = Hn g in FP64, rounded to FP32.
__device__ __forceinline__ void centre32(const FrameGeom &G, const uint64_t *fk, int *c0, float *q0) {
    double g[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const uint64_t kn = fk[q] * (uint64_t)G.n[q];
        c0[q] = (int)(kn >> 53);
        g[q] = (double)(kn & ((1ull << 53) - 1)) * 0x1.0p-53;
    }
    double v[3];
    matvec_cm(G.Hn, g[0], g[1], g[2], v);
    q0[0] = (float)v[0];
    q0[1] = (float)v[1];
    q0[2] = (float)v[2];
}

// Images of a placed molecule (centre in fractional coordinates fc) relative
// to solute molecule s, and its cell-relative position.
__device__ __forceinline__ Images placed_images(const FrameGeom &G, const FrameScratch &F, int sc, const double *fc,
                                                double *qp) {
    int cp[3];
    bin_fractional(G, fc, cp, qp);
    const int cs[3] = {sc % G.n[0], (sc / G.n[0]) % G.n[1], sc / (G.n[0] * G.n[1])};
    Images im;
    for (int q = 0; q < 3; ++q) {
        axis_images(cp[q] - cs[q], G.n[q], F.L[q], im.base[q], im.cnt[q]);
        im.step[q] = G.n[q];
    }
    return im;
}

// PAIRS random pass, stage 1: one thread per (sample, slot) of the chunk.
// Draws the bulk molecule and the new centre (src/mddf.jl:65-88,
// src/rigid_body.jl:115-120) and keeps the slot if the placed molecule's
// bounding sphere reaches the sampled solute molecule's.  The other slots
// cannot come within the cutoff and need no further work.
__global__ void __launch_bounds__(128) k_random_filter(DevSys S, Bufs B, int sample0, int nsamp) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nsamp * B.mv) return;
    const int i = sample0 + (int)(t / B.mv), k = (int)(t % B.mv);
    const Sample sm = B.samples[i];
    const int s = sm.s, f = sm.pad;
    if (S.self && k == s) return;
    const PairsFrame Pf = pairs_frame(B, f, S.self);
    const FrameGeom &G = *Pf.G;
    const FrameScratch &F = *Pf.F;
    if (!F.ok) return;
    const Placement P = draw_placement(S, G.frame_id, sm, k, Pf.bulk, Pf.nbulk);
    double qp[3];
    const Images im = placed_images(G, F, Pf.scell[s], P.fc, qp);
    const float4 qs = Pf.sq32[s];
    const float rr = F.g.cut_pre + qs.w + Pf.vq32[P.jmol].w;
    const float px = (float)qp[0] - qs.x, py = (float)qp[1] - qs.y, pz = (float)qp[2] - qs.z;
    bool any = false;
    CM_FOR_IMAGES(im, ix, iy, iz) {
        const float4 o = Pf.off32[off_index(ix, iy, iz)];
        const float Dx = px + o.x, Dy = py + o.y, Dz = pz + o.z;
        any |= fmaf(Dz, Dz, fmaf(Dy, Dy, Dx * Dx)) <= rr * rr;
    }
    if (!any) return;
    const int slotq = atomicAdd(B.counters + 1, 1);
    if (slotq < B.rq_cap) B.rq[slotq] = make_int2(i, k);
    else raise_err(S, ERR_QUEUE);
}

// PAIRS random pass, stage 2: one thread per kept slot.  Rotates the bulk
// molecule about its centroid (src/rigid_body.jl:73-80, 122-134) and evaluates
// it against the sampled solute molecule (one direction).
template <bool FP32>
__global__ void __launch_bounds__(128) k_random_eval(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    LocalStats st;
    const int n = min(B.counters[1], B.rq_cap);
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < n; it += gridDim.x * blockDim.x) {
        const int2 e = B.rq[it];
        const Sample sm = B.samples[e.x];
        const int s = sm.s, k = e.y, f = sm.pad;
        const PairsFrame Pf = pairs_frame(B, f, S.self);
        const FrameGeom &G = *Pf.G;
        const FrameScratch &F = *Pf.F;
        Placement P = draw_placement(S, G.frame_id, sm, k, Pf.bulk, Pf.nbulk);
        double qp[3];
        const Images im = placed_images(G, F, Pf.scell[s], P.fc, qp);
        double A[9];
        draw_rotation(P.st, A);
        // the search places the molecule's centroid-relative atom offsets;
        // the exact distances use the placement of the input coordinates
        const ExactRef X{f, s, P.jmol, A, P.fc};
        const d4 *o = Pf.vo64 + (int64_t)P.jmol * S.apv;
        DirRec r1, r2;
        st.molpairs++;
        st.atompairs += (unsigned long long)S.aps * S.apv * image_count(im);
        if (FP32) {
            float4 ov32[kMaxSmallMol];
            for (int b = 0; b < S.apv; ++b) {
                const d4 w = o[b];
                double r[3];
                matvec_rm(A, w.x, w.y, w.z, r);
                ov32[b] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.f);
            }
            const float4 qs32 = Pf.sq32[s];
            const float4 qp32 = make_float4((float)qp[0], (float)qp[1], (float)qp[2], 0.f);
            const float4 *os32 = Pf.so32 + (int64_t)s * S.aps;
            Pass32 Q;
            pairs_pass<false>(S, Pf.off32, im, qs32, qp32, os32, (const float4 *)ov32, Q);
            pairs_decide<false>(S, G, B, X, F.g, Q, Pf.off32, im, qs32, qp32, os32, (const float4 *)ov32, s, k, r1, r2, st);
        } else {
            d4 ov64[kMaxSmallMol];
            for (int b = 0; b < S.apv; ++b) {
                const d4 w = o[b];
                double r[3];
                matvec_rm(A, w.x, w.y, w.z, r);
                ov64[b] = make_d4(r[0], r[1], r[2], 0.0);
            }
            const d4 qs64 = Pf.sq64[s];
            const d4 qp64 = make_d4(qp[0], qp[1], qp[2], 0.0);
            const d4 *os64 = Pf.so64 + (int64_t)s * S.aps;
            PassT<double> Q;
            pairs_pass<false>(S, Pf.off64, im, qs64, qp64, os64, (const d4 *)ov64, Q);
            pairs_decide<false>(S, G, B, X, F.g64, Q, Pf.off64, im, qs64, qp64, os64, (const d4 *)ov64, s, k, r1, r2, st);
        }
        if (r1.within) { apply_hit(S, h, true, r1.bin, r1.i_local, r1.j, r1.ref, r1.rbin); st.hits++; }
    }
    stats_flush(S, st, true);
    __syncthreads();
    shist_flush(S, h, true);
}

// The fine cells of a frame's candidate grid (FP64, once per frame).
__device__ __forceinline__ FineCells fine_cells(const FrameGeom &G, const FrameScratch &F, int K) {
    FineCells fc;
    fc.K = K;
    fc.K3 = K * K * K;
    fc.ortho = F.ortho;
    for (int i = 0; i < 9; ++i) fc.e[i] = (float)(G.Hn[i] / (double)K);
    for (int k = 0; k < 3; ++k) fc.h[k] = (float)(0.5 * fabs(G.Hn[4 * k]) / (double)K) * (1.0f + 1e-6f);
    double R = 0.0;
    for (int m = 0; m < 4; ++m) {
        double v[3];
        matvec_cm(G.Hn, 1.0, (m & 1) ? -1.0 : 1.0, (m & 2) ? -1.0 : 1.0, v);
        R = fmax(R, 0.5 * norm3d(v[0], v[1], v[2]) / (double)K);
    }
    fc.R = __double2float_ru(R * (1.0 + 1e-6) + 1e-6);
    return fc;
}

// One block per frame computes the frame constants: stencils, the FP32 guard
// band, and the slot table of the frame's sampled solute molecules.
//
// Guard band.  In the FP32 displacement of an atom pair,
//   dx = ((q_v - q_s) + off) + o_b) - o_a,
// every input is the rounding of an FP64 value and every operation rounds, so
// with u = 2^-24 each component is within u times the sum of the magnitudes of
// the inputs and intermediate results of its exact value:
//   |q| <= Q (a site inside its cell), |off| <= OFF (stencil offsets),
//   |o| <= r (molecule radii), |q_v - q_s| <= Q, |off - q_s| <= Q + OFF,
//   |D| <= Q + OFF, |t| <= Q + OFF + r_v, |dx| <= cutoff,
// and D formed either as (q_v - q_s) + off or as q_v + (off - q_s), giving
// E = u (5Q + 4 OFF + 2 r_v + r_s + cutoff).  In the ATOMS layout a placed
// atom of the random insertion is no rounding of an FP64 value: placed_store32
// forms it in FP32 within u (5Q + 41 r_c) of the FP64 placement (r_c the
// largest centroid radius), and E adds u (5Q + 44 r_c) in the frames that
// place in FP32 (F.place32).  The distance is within
// sqrt(3) E plus 2.5 u d (three roundings of d^2, one of the square root).  The
// atom-cell layout's displacement (q_a - (q_b - off)) is bounded by the same
// expression with r = 0.  delta adds 25 % to the bound.
//
// The exact distance (exact_d2, on the input coordinates) and the FP64 values
// the searches start from (cell-relative positions, offsets, radii, placed
// atoms) are other roundings of the same real distance.  Each is a chain of
// at most a few dozen FP64 operations (plus a sum over a molecule's atoms for
// a centroid or a placement) whose operands are bounded by
//   M = X (1 + 3 |H| |H^-1|) + 16 |H| + cutoff + 2 (r_s + r_v + r_c) + 1,
// X the largest input coordinate, |H| and |H^-1| the largest entries of the
// cell matrix and of its inverse, r_c the largest molecule radius of the
// random insertion; so with u64 = 2^-53 both are within
//   eps = u64 (512 + 4 (apv + aps in the molecule layout)) M
// of the real distance.  The FP32 band is delta + eps; the FP64 search uses
// eps as its band, so both decide every count from the exact distance.
__device__ __forceinline__ void k_frame_consts_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B, int pairs) {
    const int f = blockIdx.x;
    const FrameGeom &G = B.G[f];
    FrameScratch &F = B.FS[f];
    if (B.slot)
        for (int i = threadIdx.x; i < G.nsamples; i += blockDim.x) {
            const Sample sm = B.samples[G.sample_off + i];
            B.slot[(int64_t)f * B.ms + sm.s] = sm.d;
        }
    // the two corner norms in parallel: lanes 0-7 and 8-15
    const int lane = threadIdx.x;
    __shared__ double cn[16];
    __shared__ int Ls[6];
    __shared__ double radii[2];
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) {
            for (int m = 0; m < 3; ++m) F.hin[3 * k + m] = (float)(G.Hi[3 * k + m] * (double)G.n[k]);
            F.cw[k] = (float)G.cw[k];
        }
        F.ortho = (G.Hn[1] == 0.0 && G.Hn[2] == 0.0 && G.Hn[3] == 0.0 && G.Hn[5] == 0.0 && G.Hn[6] == 0.0 &&
                   G.Hn[7] == 0.0) ? 1 : 0;
        double rs = F.rmax_s, rv = S.self ? F.rmax_s : F.rmax_v;
        if (!pairs) rs = rv = 0.0;
        radii[0] = rs;
        radii[1] = rv;
        const double range = S.cut + rs + rv;
        int L[3], La[3];
        bool ok = true;
        if (pairs) ok = stencil(G, range + 1e-6 * (1.0 + range), L) && ok;
        else L[0] = L[1] = L[2] = 1;
        ok = stencil(G, S.cut * (1.0 + 1e-7) + 1e-7, La) && ok;
        int multi = 0;
        for (int k = 0; k < 3; ++k) {
            F.L[k] = L[k];
            F.La[k] = La[k];
            // ATOMS: one cell beyond the stencil, for the grouped site walk
            Ls[k] = pairs ? max(L[k], La[k]) : La[k] + 1;
            if (2 * L[k] + 1 > G.n[k]) multi |= 1 << k;
        }
        F.multi = multi;
        // half-stencil cells: the home cell's row forward, the rest of its plane forward, the planes above
        const int K = (L[0] + 1) + (2 * L[0] + 1) * L[1] + (2 * L[0] + 1) * (2 * L[1] + 1) * L[2];
        F.tile = (pairs && S.self && multi == 0 && K <= kTileCells && S.mv < (1 << 24)) ? 1 : 0;
        F.ok = ok ? 1 : 0;
        F.agrid = (!pairs && B.agk > 0 && ok && (2 * La[0] + 1) * (2 * La[1] + 1) * (2 * La[2] + 1) <= kAgridMaxStencil) ? 1 : 0;
        if (F.agrid) F.fcells = fine_cells(G, F, B.agk);
    }
    __syncthreads();
    if (lane < 16) {
        const int m = lane & 7;
        const double l0 = lane < 8 ? 1.0 : (double)Ls[0], l1 = lane < 8 ? 1.0 : (double)Ls[1],
                     l2 = lane < 8 ? 1.0 : (double)Ls[2];
        double v[3];
        matvec_cm(G.Hn, (m & 1) ? -l0 : l0, (m & 2) ? -l1 : l1, (m & 4) ? -l2 : l2, v);
        cn[lane] = norm3d(v[0], v[1], v[2]);
    }
    __syncthreads();
    if (lane != 0) return;
    double Q = 0.0, OFF = 0.0;
    for (int k = 0; k < 8; ++k) {
        Q = fmax(Q, cn[k]);
        OFF = fmax(OFF, cn[8 + k]);
    }
    const double rs = radii[0], rv = radii[1];
    const double range = S.cut + rs + rv;
    // eps: the exact distance against the FP64 values the searches use
    double hmax = 0.0, himax = 0.0;
    for (int k = 0; k < 9; ++k) {
        hmax = fmax(hmax, fabs(G.H[k]));
        himax = fmax(himax, fabs(G.Hi[k]));
    }
    const double rc = S.self ? F.rmax_s : fmax((double)F.rmax_v, (double)F.rcmax);
    const double M = (double)F.xmax * (1.0 + 3.0 * hmax * himax) + 16.0 * hmax + S.cut +
                     2.0 * ((double)F.rmax_s + rc + (double)F.rcmax) + 1.0;
    const double eps = 0x1.0p-53 * (512.0 + 4.0 * (double)(S.apv + (pairs ? S.aps : 0))) * M;
    const double u = 0x1.0p-24;
    const double E0 = u * (5.0 * Q + 4.0 * OFF + 2.0 * rv + rs + S.cut + 1.0);
    // ATOMS frames: the random insertion's slots are placed in FP32 (placed_store32) when
    // that widens the band by at most 60 % (small molecules); larger molecules have few
    // slots per atom and more records per slot in a wider band, and keep the FP64 placement
    const double P = u * (5.0 * Q + 44.0 * (double)F.rcmax);
    const bool place32 = !pairs && S.fp32 && P <= 0.6 * E0;
    F.place32 = place32 ? 1 : 0;
    const double E = E0 + (place32 ? P : 0.0);
    const double delta = 1.25 * (1.7320508075688772 * E + 2.5 * u * (S.cut + 1.0)) + 1e-9 + eps;
    Guard g;
    g.delta = delta;
    const double cp = S.cut + delta, cm = S.cut - delta;
    g.cutp2 = __double2float_ru(cp * cp);
    g.cutm2 = cm > 0.0 ? __double2float_rd(cm * cm) : 0.0f;
    g.two_delta = __double2float_ru(2.0 * delta);
    g.inv_bs = (float)(1.0 / S.binstep);
    // |k - d/binstep| <= delta/binstep + (rounding of d * inv_bs and of inv_bs)
    g.bin_band = __double2float_ru(delta / S.binstep + (double)(S.nbins + 1) * 4.0 * u + 1e-6);
    g.dbulk_lo = __double2float_rd(S.dbulk - delta);
    g.dbulk_hi = __double2float_ru(S.dbulk + delta);
    g.cut_pre = __double2float_ru(S.cut + 1e-3 * (1.0 + range));
    F.g = g;
    // the FP64 search: the same rules with band eps
    Guard64 g64;
    g64.delta = eps;
    const double cp64 = __dadd_ru(S.cut, eps), cm64 = __dsub_rd(S.cut, eps);
    g64.cutp2 = __dmul_ru(cp64, cp64);
    g64.cutm2 = cm64 > 0.0 ? __dmul_rd(cm64, cm64) : 0.0;
    g64.two_delta = __dmul_ru(2.0, eps);
    g64.inv_bs = 1.0 / S.binstep;
    g64.bin_band = __dadd_ru(__ddiv_ru(eps, S.binstep), (double)(S.nbins + 2) * 8.0 * 0x1.0p-53);
    g64.dbulk_lo = __dsub_rd(S.dbulk, eps);
    g64.dbulk_hi = __dadd_ru(S.dbulk, eps);
    g64.cut_pre = g.cut_pre;
    F.g64 = g64;
}

__global__ void k_frame_consts(DevSys S, Bufs B, int pairs) {
    k_frame_consts_body(blockIdx, gridDim, S, B, pairs);
}

// Molecule-centred data for random insertion (src/rigid_body.jl:127-134):
// the molecule made whole around its reference atom, relative to its mean.
template <typename T>
__device__ void centroid_data(const FrameGeom &G, const T *x, int apm, int iref, d4 *u64, float &rc) {
    double xr[3];
    load_xyz(x + 3 * iref, xr);
    double cm[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < apm; ++b) {
        double xb[3], d[3];
        load_xyz(x + 3 * b, xb);
        for (int k = 0; k < 3; ++k) d[k] = sub(xb[k], xr[k]);
        double f[3];
        matvec_rm(G.Hi, d[0], d[1], d[2], f);
        double n0 = rint(f[0]), n1 = rint(f[1]), n2 = rint(f[2]);
        if (n0 != 0.0 || n1 != 0.0 || n2 != 0.0) {
            double sh[3];
            matvec_cm(G.H, n0, n1, n2, sh);
            for (int k = 0; k < 3; ++k) xb[k] = sub(xb[k], sh[k]);
        }
        u64[b] = make_d4(xb[0], xb[1], xb[2], 0.0);
        for (int k = 0; k < 3; ++k) cm[k] = add(cm[k], xb[k]);
    }
    for (int k = 0; k < 3; ++k) cm[k] = div(cm[k], (double)apm);
    double r = 0.0;
    for (int b = 0; b < apm; ++b) {
        d4 w = u64[b];
        w.x = sub(w.x, cm[0]);
        w.y = sub(w.y, cm[1]);
        w.z = sub(w.z, cm[2]);
        u64[b] = w;
        r = fmax(r, sqrt(w.x * w.x + w.y * w.y + w.z * w.z));
    }
    rc = __double2float_ru(r * (1.0 + 1e-12) + 1e-12);
}

// ----------------------------------------------------------- ATOMS regime
__device__ __forceinline__ int pack_cell(const int *c) { return c[0] | (c[1] << 10) | (c[2] << 20); }

// Solvent atoms binned individually (grid y = frame); molecule-centred data
// for random insertion.
template <typename T>
__device__ __forceinline__ void k_prep_atoms_solvent_body(const uint3 blockIdx, const dim3 gridDim, const Bufs &B, const T *__restrict__ xyz, int64_t xyz_stride, int iref, int centroids) {
    const int f = blockIdx.y;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= B.mv) return;
    const int apm = (int)(B.Nv / B.mv);
    const FrameGeom &G = B.G[f];
    const T *x = xyz + (int64_t)f * xyz_stride + (int64_t)m * apm * 3;
    const int64_t fo = (int64_t)f * B.Nv;
    double xm = 0.0;
    for (int b = 0; b < apm; ++b) {
        double xb[3];
        load_xyz(x + 3 * b, xb);
        xm = fmax(xm, fmax(fabs(xb[0]), fmax(fabs(xb[1]), fabs(xb[2]))));
        int c[3];
        double q[3];
        bin_position(G, xb[0], xb[1], xb[2], c, q);
        const int64_t i = fo + (int64_t)m * apm + b;
        B.avcell[i] = pack_cell(c);
        B.avq32[i] = make_float4((float)q[0], (float)q[1], (float)q[2], 0.f);
        B.avq64[i] = make_d4(q[0], q[1], q[2], 0.0);
    }
    warp_max_pos(&B.FS[f].xmax, __double2float_ru(xm));
    if (centroids) {
        float r;
        centroid_data(G, x, apm, iref, B.u64 + fo + (int64_t)m * apm, r);
        for (int b = 0; b < apm; ++b) {
            const d4 w = B.u64[fo + (int64_t)m * apm + b];
            B.u32[fo + (int64_t)m * apm + b] = make_float4((float)w.x, (float)w.y, (float)w.z, 0.f);
        }
        B.rc[(int64_t)f * B.mv + m] = r;
        warp_max_pos(&B.FS[f].rcmax, r);
    }
}

template <typename T>
__global__ void k_prep_atoms_solvent(Bufs B, const T *__restrict__ xyz, int64_t xyz_stride, int iref, int centroids) {
    k_prep_atoms_solvent_body<T>(blockIdx, gridDim, B, xyz, xyz_stride, iref, centroids);
}

// Solute atoms binned into per-molecule cell lists: key = s * ncell + cell.
template <typename T>
__device__ __forceinline__ void k_prep_atoms_solute_body(const uint3 blockIdx, const dim3 gridDim, const Bufs &B, const T *__restrict__ xyz, int64_t xyz_stride) {
    const int f = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.Ns) return;
    const int aps = (int)(B.Ns / B.ms);
    const FrameGeom &G = B.G[f];
    double x[3];
    load_xyz(xyz + (int64_t)f * xyz_stride + 3 * (int64_t)i, x);
    int c[3];
    double q[3];
    bin_position(G, x[0], x[1], x[2], c, q);
    const int s = i / aps, a = i - s * aps;
    const int k = s * G.ncell + cell_linear(G, c[0], c[1], c[2]);
    const int64_t fi = (int64_t)f * B.Ns + i;
    B.akey[fi] = k;
    B.atq32[fi] = make_float4((float)q[0], (float)q[1], (float)q[2], __int_as_float(a));
    B.atq64[fi] = make_d4(q[0], q[1], q[2], 0.0);
    atomicAdd(B.acount + (int64_t)f * B.as + k, 1);
    warp_max_pos(&B.FS[f].xmax, __double2float_ru(fmax(fabs(x[0]), fmax(fabs(x[1]), fabs(x[2])))));
}

template <typename T>
__global__ void k_prep_atoms_solute(Bufs B, const T *__restrict__ xyz, int64_t xyz_stride) {
    k_prep_atoms_solute_body<T>(blockIdx, gridDim, B, xyz, xyz_stride);
}

__device__ __forceinline__ void k_scatter_atoms_body(const uint3 blockIdx, const dim3 gridDim, const Bufs &B) {
    const int f = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.Ns) return;
    const int64_t fi = (int64_t)f * B.Ns + i;
    const int p = atomicAdd(B.afill + (int64_t)f * B.as + B.akey[fi], 1);
    B.asq32[(int64_t)f * B.Ns + p] = B.atq32[fi];
    B.asq64[(int64_t)f * B.Ns + p] = B.atq64[fi];
}

__global__ void k_scatter_atoms(Bufs B) {
    k_scatter_atoms_body(blockIdx, gridDim, B);
}

// Far-slot test of a placement: every atom lies within the molecule's radius
// rc of the centre, so its cell is in the box of cells that sphere touches;
// false if no cell of the box is near the solute molecule (nm: its near mask),
// and then no atom of the slot can be within the cutoff.
__device__ __forceinline__ bool placed_maybe_near(const FrameGeom &G, const FrameScratch &F, const unsigned char *nm,
                                                  const double *fc, const int *c0, float rc) {
    int lo[3], hi[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float g = (float)(fc[q] * (double)G.n[q]) - (float)c0[q];  // grid units inside the cell
        const float reach = rc / F.cw[q] + 1e-3f;
        lo[q] = (int)floorf(g - reach);
        hi[q] = (int)floorf(g + reach);
    }
    if (hi[0] - lo[0] >= G.n[0] || hi[1] - lo[1] >= G.n[1] || hi[2] - lo[2] >= G.n[2]) return true;
    for (int dz = lo[2]; dz <= hi[2]; ++dz)
        for (int dy = lo[1]; dy <= hi[1]; ++dy)
            for (int dx = lo[0]; dx <= hi[0]; ++dx)
                if (nm[(wrap_cell(c0[2] + dz, G.n[2]) * G.n[1] + wrap_cell(c0[1] + dy, G.n[1])) * G.n[0] +
                       wrap_cell(c0[0] + dx, G.n[0])]) return true;
    return false;
}

// Atom w (molecule-centred, FP64) of a slot rotated by A and moved to the
// centre (cell c0, position q0 from that cell's origin; fc its fractional
// coordinates): its cell c and its FP64 position q from that cell's origin.
// The cell is c0 shifted by the floor of the atom's FP32 grid coordinates;
// the FP64 offset is taken from the shifted cell's origin, so the two stay
// consistent.
__device__ __forceinline__ void placed_atom(const FrameGeom &G, const FrameScratch &F, const d4 *off64, const double *A,
                                            const d4 &w, const int *c0, const double *q0, const double *fc, int *c,
                                            double *q) {
    double o[3];
    matvec_rm(A, w.x, w.y, w.z, o);
    const double t[3] = {add(q0[0], o[0]), add(q0[1], o[1]), add(q0[2], o[2])};
    const float tx = (float)t[0], ty = (float)t[1], tz = (float)t[2];
    int dl[3];
    bool in_table = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        dl[k] = (int)floorf(fmaf(F.hin[3 * k + 2], tz, fmaf(F.hin[3 * k + 1], ty, F.hin[3 * k] * tx)));
        if (dl[k] < -kLT || dl[k] > kLT) in_table = false;
        c[k] = wrap_cell(c0[k] + dl[k], G.n[k]);
    }
    if (in_table) {
        const d4 ov = off64[off_index(dl[0], dl[1], dl[2])];
        q[0] = sub(t[0], ov.x);
        q[1] = sub(t[1], ov.y);
        q[2] = sub(t[2], ov.z);
    } else {
        // a molecule much larger than a cell: bin its absolute position
        double cm[3];
        matvec_cm(G.H, fc[0], fc[1], fc[2], cm);
        bin_position(G, add(o[0], cm[0]), add(o[1], cm[1]), add(o[2], cm[2]), c, q);
    }
}

// Every atom of a placed slot into the placement buffers at `base` (the FP64
// positions only for the FP64 search: the FP32 search and its exact scans
// read the FP32 ones and draw the exact placement again).
__device__ __forceinline__ void placed_store(const DevSys &S, const Bufs &B, const FrameGeom &G, const FrameScratch &F,
                                             const d4 *off64, const double *A, const d4 *u, const int *c0,
                                             const double *q0, const double *fc, int64_t base) {
    for (int b = 0; b < S.apv; ++b) {
        int c[3];
        double q[3];
        placed_atom(G, F, off64, A, u[b], c0, q0, fc, c, q);
        B.pcell[base + b] = pack_cell(c);
        B.pq32[base + b] = make_float4((float)q[0], (float)q[1], (float)q[2], 0.f);
        if (!S.fp32) B.pq64[base + b] = make_d4(q[0], q[1], q[2], 0.0);
    }
}

// The FP32 search's placement of a slot: the molecule-centred atom offsets
// (FP32 copies u32) rotated by the FP32 matrix of draw_rotation32 and moved to
// the centre (centre32), the cell chosen as in placed_atom and the FP32
// offset of the shift taken off.  Each coordinate is within P = u (5 Q + 41 r_c)
// of placed_atom's FP64 one (the guard band of k_frame_consts adds
// u (5 Q + 44 r_c)): u Q for q0, 39 u r_c for the rotated offset (entries of A
// within 20 u, the offsets' rounding, three roundings of the dot product),
// u (Q + r_c) for the sum t, u (2 Q + r_c) for the shift's offset and u Q for
// the difference.  False when an atom lands beyond the offset table; the
// caller then places the slot in FP64.
__device__ __forceinline__ bool placed_store32(const Bufs &B, const FrameScratch &F, const FrameGeom &G,
                                               const float4 *off32, const float *A, const float4 *u, const int *c0,
                                               const float *q0, int64_t base, int apv) {
    for (int b = 0; b < apv; ++b) {
        const float4 w = u[b];
        const float tx = q0[0] + fmaf(A[2], w.z, fmaf(A[1], w.y, A[0] * w.x));
        const float ty = q0[1] + fmaf(A[5], w.z, fmaf(A[4], w.y, A[3] * w.x));
        const float tz = q0[2] + fmaf(A[8], w.z, fmaf(A[7], w.y, A[6] * w.x));
        int dl[3], c[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            dl[k] = (int)floorf(fmaf(F.hin[3 * k + 2], tz, fmaf(F.hin[3 * k + 1], ty, F.hin[3 * k] * tx)));
            if (dl[k] < -kLT || dl[k] > kLT) return false;
            c[k] = wrap_cell(c0[k] + dl[k], G.n[k]);
        }
        const float4 ov = off32[off_index(dl[0], dl[1], dl[2])];
        B.pcell[base + b] = pack_cell(c);
        B.pq32[base + b] = make_float4(tx - ov.x, ty - ov.y, tz - ov.z, 0.f);
    }
    return true;
}

// Random-insertion slots of the ATOMS regime, first pass: one thread per
// slot of samples sample0 .. sample0 + gridDim.y - 1 of the chunk.  Only the
// slot's draws are taken (the bulk pick and the centre; integer and FP32
// work): a slot whose molecule cannot reach a cell near its solute molecule
// (placed_maybe_near on a box widened to cover the FP32 rounding of the
// centre's cell) can hold no pair within the cutoff and is dropped; the others
// go to the slot list (y * mv + slot, count in counters[5]), so that the FP64
// placement runs on full warps.
__device__ __forceinline__ void k_slot_filter_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B, int sample0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= S.mv) return;
    const int y = blockIdx.y;
    const Sample sm = B.samples[sample0 + y];
    if (S.self && k == sm.s) return;
    const int f = sm.pad;
    const FrameGeom &G = B.G[f];
    const FrameScratch &F = B.FS[f];
    int jmol;
    uint64_t fk[3];
    draw_slot_bits(S, G.frame_id, sm, k, B.bulk + (int64_t)f * B.ndist * B.mv, B.nbulk + (int64_t)f * B.ndist, jmol, fk);
    const unsigned char *nm = B.anear + (int64_t)f * B.as + (int64_t)sm.s * G.ncell;
    const float rc = B.rc[(int64_t)f * B.mv + jmol];
    int lo[3], hi[3];
    bool maybe = false;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        // U n in grid units from the grid's origin (FP32 of the exact product fk n 2^-53)
        const float g = cmfeed::u128_to_f32(0, fk[q] * (uint64_t)G.n[q]) * 0x1.0p-53f;
        const float reach = rc / F.cw[q] + 2e-3f;
        lo[q] = (int)floorf(g - reach);
        hi[q] = (int)floorf(g + reach);
        if (hi[q] - lo[q] >= G.n[q]) maybe = true;
    }
    for (int dz = lo[2]; dz <= hi[2] && !maybe; ++dz)
        for (int dy = lo[1]; dy <= hi[1] && !maybe; ++dy)
            for (int dx = lo[0]; dx <= hi[0] && !maybe; ++dx)
                maybe = nm[(wrap_cell(dz, G.n[2]) * G.n[1] + wrap_cell(dy, G.n[1])) * G.n[0] + wrap_cell(dx, G.n[0])] != 0;
    if (!maybe) return;
    const int at = atomicAdd(B.counters + 5, 1);
    if (at < B.aslot_cap) B.aslot[at] = y * S.mv + k;
    else raise_err(S, ERR_QUEUE);
}

__global__ void k_slot_filter(DevSys S, Bufs B, int sample0) {
    k_slot_filter_body(blockIdx, gridDim, S, B, sample0);
}

// Second pass: the listed slots placed (FP64, the same draws, on full warps),
// written to the placement buffers, and -- in frames without a candidate grid
// -- queued for k_atoms_eval when one of their atoms lies in a near cell of
// the solute molecule: (slot, placed sample, sample, 1).  The grid's frames
// are queried by k_agrid_random, which reads these positions.  Persistent
// grid over the list.
__device__ __forceinline__ void k_atoms_place_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B, int sample0) {
    const int n = min(B.counters[5], B.aslot_cap);
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < n; it += gridDim.x * blockDim.x) {
        const int e = B.aslot[it];
        const int y = e / S.mv, k = e - y * S.mv;
        const Sample sm = B.samples[sample0 + y];
        const int f = sm.pad;
        const FrameGeom &G = B.G[f];
        const FrameScratch &F = B.FS[f];
        const int64_t base = (int64_t)y * B.Nv + (int64_t)k * S.apv;
        const int *bulk = B.bulk + (int64_t)f * B.ndist * B.mv, *nbulk = B.nbulk + (int64_t)f * B.ndist;
        const unsigned char *nm = B.anear + (int64_t)f * B.as + (int64_t)sm.s * G.ncell;
        bool placed = false;
        if (F.place32) {
            int jmol;
            uint64_t fk[3];
            uint64_t rs = draw_slot_bits(S, G.frame_id, sm, k, bulk, nbulk, jmol, fk);
            int c0[3];
            float q0[3];
            centre32(G, fk, c0, q0);
            float A32[9];
            draw_rotation32(rs, A32);
            placed = placed_store32(B, F, G, B.off32 + (int64_t)f * kOffEntries, A32,
                                    B.u32 + (int64_t)f * B.Nv + (int64_t)jmol * S.apv, c0, q0, base, S.apv);
        }
        if (!placed) {
            const Placement P = draw_placement(S, G.frame_id, sm, k, bulk, nbulk);
            // the new centre's cell c0 and its position q0 from that cell's origin
            int c0[3];
            double q0[3];
            bin_fractional(G, P.fc, c0, q0);
            uint64_t rs = P.st;
            double A[9];
            draw_rotation(rs, A);
            placed_store(S, B, G, F, B.off64 + (int64_t)f * kOffEntries, A, B.u64 + (int64_t)f * B.Nv + (int64_t)P.jmol * S.apv,
                         c0, q0, P.fc, base);
        }
        if (F.agrid) continue;
        bool near = false;
        for (int b = 0; b < S.apv && !near; ++b) {
            const int pc = B.pcell[base + b];
            near = nm[((pc >> 20) * G.n[1] + ((pc >> 10) & 1023)) * G.n[0] + (pc & 1023)] != 0;
        }
        if (near) {
            const int slot = atomicAdd(B.counters + 2, 1);
            if (slot < B.aq_cap) B.aq[slot] = make_int4(k, y, sample0 + y, 1);
            else raise_err(S, ERR_QUEUE);
        }
    }
}

__global__ void k_atoms_place(DevSys S, Bufs B, int sample0) {
    k_atoms_place_body(blockIdx, gridDim, S, B, sample0);
}

// DCD decode (src/trajectory_formats/NamdDCD.jl:141-169): a frame of the file
// is its unit-cell record followed by three Fortran records holding the x, y
// and z float32 arrays of all atoms.  Raw frames go to the device as read
// from the file; this kernel gathers the selection's atoms (0-based indices
// into the frame) into the engine's [frame][atom][xyz] float32 staging
// layout, swapping bytes for big-endian files.  All offsets are multiples of
// four bytes (records of float32 with 4-byte markers), so the loads are
// aligned.
__global__ void k_dcd_gather(const unsigned char *__restrict__ raw, int64_t frame_bytes, int64_t xoff, int64_t yoff,
                             int64_t zoff, int swap, const int32_t *__restrict__ atoms, int64_t nsel,
                             float *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsel) return;
    const int f = blockIdx.y;
    const unsigned char *fr = raw + (int64_t)f * frame_bytes;
    const int64_t a = atoms[i];
    unsigned int w[3];
    w[0] = reinterpret_cast<const unsigned int *>(fr + xoff)[a];
    w[1] = reinterpret_cast<const unsigned int *>(fr + yoff)[a];
    w[2] = reinterpret_cast<const unsigned int *>(fr + zoff)[a];
    float *o = out + ((int64_t)f * nsel + i) * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = __uint_as_float(swap ? __byte_perm(w[k], 0, 0x0123) : w[k]);
}

// Weight change: fold the integer class accumulators into FP64 sums
// (acc += w * count / 2) and clear them.
__global__ void k_fold(unsigned long long *__restrict__ acc, double *__restrict__ sums, int64_t n, double w) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long c = acc[i];
    if (c) {
        sums[i] = add(sums[i], mul(w, div((double)c, 2.0)));
        acc[i] = 0ull;
    }
}

// FP32 throughput probe: kProbeChains independent multiply-add chains per
// thread kept in registers, so the loop is issue-bound on the FP32 pipes.
constexpr int kProbeChains = 8;
__global__ void __launch_bounds__(256) k_fma_probe(float *__restrict__ sink, int iters, float m) {
    float a[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    const float c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kProbeChains; ++k) a[k] = fmaf(a[k], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) s += a[k];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace cmk
