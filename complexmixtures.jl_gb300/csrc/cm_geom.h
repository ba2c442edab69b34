// cm_geom.h -- unit-cell geometry shared by the host planner and the kernels.
//
// Positions are binned on a grid in fractional coordinates: with f = Hinv x
// wrapped into [0, 1), the cell along axis k is c_k = floor(f_k n_k) and the
// position inside the cell is g_k = f_k n_k - c_k in [0, 1).  A site is then
// stored as its cell index and q = Hn g, its offset from the cell origin
// (Hn = H diag(1/n) holds the three cell edge vectors).  The displacement from
// a site in cell c to a site in cell c + Delta (Delta unwrapped, so it carries
// the periodic image) is q' - q + Hn Delta.  Hn Delta is tabulated per frame,
// so the single-precision search never works with coordinates larger than a
// few cells, whatever the size of the box.
#pragma once
#include <math.h>
#include <stdint.h>

#include "cm_feed.h"

namespace cmgeom {

// Four doubles, 32-byte aligned: one vector load per site.
struct alignas(32) d4 {
    double x, y, z, w;
};
CM_HD d4 make_d4(double x, double y, double z, double w) {
    d4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}

// Largest stencil half-width the per-frame offset table covers.
constexpr int kLT = 6;
constexpr int kLTW = 2 * kLT + 1;
constexpr int kOffEntries = kLTW * kLTW * kLTW;

struct FrameGeom {
    double H[9];      // column-major: H[0..2] = a, H[3..5] = b, H[6..8] = c
    double Hi[9];     // row-major inverse
    double Hn[9];     // column-major cell edge vectors: column k = H column k / n_k
    double det;       // dot(cross(a, b), c)  (src/mddf.jl:350-351)
    double w[3];      // perpendicular widths of the cell
    double cw[3];     // perpendicular widths of one grid cell (w / n)
    double weight;
    double hw;        // half the smallest perpendicular width: an image this close is the minimum image
    int64_t frame_id;
    int n[3];
    int ncell;
    int sample_off;   // offset of this frame's random samples
    int nsamples;     // random samples this frame (0 in coordination-number mode)
    int ndistinct;    // distinct sampled solute molecules
    int hortho;       // the off-diagonal entries of H are all zero
};

using cmfeed::add;
using cmfeed::mul;
using cmfeed::sub;

// v = M x for column-major M: v_k = (M[k] x0 + M[3+k] x1) + M[6+k] x2
CM_HD void matvec_cm(const double *M, double x0, double x1, double x2, double *v) {
    for (int k = 0; k < 3; ++k) v[k] = add(add(mul(M[k], x0), mul(M[3 + k], x1)), mul(M[6 + k], x2));
}
// v = M x for row-major M
CM_HD void matvec_rm(const double *M, double x0, double x1, double x2, double *v) {
    for (int k = 0; k < 3; ++k) v[k] = add(add(mul(M[3 * k], x0), mul(M[3 * k + 1], x1)), mul(M[3 * k + 2], x2));
}

// Bin a position: cell index per axis and FP64 offset from the cell origin.
CM_HD void bin_position(const FrameGeom &G, double x0, double x1, double x2, int *c, double *q) {
    double f[3], g[3];
    matvec_rm(G.Hi, x0, x1, x2, f);
    for (int k = 0; k < 3; ++k) {
        double fk = sub(f[k], floor(f[k]));
        if (!(fk < 1.0)) fk = 0.0;  // f just below an integer can round up to 1
        if (!(fk >= 0.0)) fk = 0.0; // NaN guard
        double fn = mul(fk, (double)G.n[k]);
        double ck = floor(fn);
        int ci = (int)ck;
        if (ci >= G.n[k]) ci = G.n[k] - 1;
        if (ci < 0) ci = 0;
        c[k] = ci;
        g[k] = sub(fn, (double)ci);
    }
    matvec_cm(G.Hn, g[0], g[1], g[2], q);
}

// Bin a fractional position already in [0, 1) (the centre of a placed molecule).
CM_HD void bin_fractional(const FrameGeom &G, const double *f, int *c, double *q) {
    double g[3];
    for (int k = 0; k < 3; ++k) {
        double fn = mul(f[k], (double)G.n[k]);
        int ci = (int)floor(fn);
        if (ci >= G.n[k]) ci = G.n[k] - 1;
        if (ci < 0) ci = 0;
        c[k] = ci;
        g[k] = sub(fn, (double)ci);
    }
    matvec_cm(G.Hn, g[0], g[1], g[2], q);
}

// Minimum-image displacement d -> d - H rint(Hinv d), the unwrap used to make
// molecules whole (CellListMap.wrap_relative_to, src/rigid_body.jl:129-131).
CM_HD void unwrap(const FrameGeom &G, double *d) {
    double f[3];
    matvec_rm(G.Hi, d[0], d[1], d[2], f);
    double n0 = rint(f[0]), n1 = rint(f[1]), n2 = rint(f[2]);
    if (n0 != 0.0 || n1 != 0.0 || n2 != 0.0) {
        double s[3];
        matvec_cm(G.H, n0, n1, n2, s);
        for (int k = 0; k < 3; ++k) d[k] = sub(d[k], s[k]);
    }
}

// ------------------------------------------------------------- exact distance
// The FP64 distance that defines every count.  CellListMap's pairwise!
// (src/minimum_distances.jl:129-148) reports a pair iff its minimum-image
// distance is within the cutoff; the engine and the oracle both evaluate it as
//   d = y - x,  n0 = rint(H^-1 d),  e = d - H n0,  |e|^2,
// keeping that image when |e| is at most half the smallest perpendicular
// width, else the smallest |d - H n|^2 over the 27 images n around n0.  Every
// operation below is one IEEE round-to-nearest step in the order written
// (no contraction), so the value is the same bit for bit on the host and on
// the device, for the same FP64 inputs x and y.

// f = H^-1 d (row-major inverse; diagonal cells use the diagonal only)
CM_HD void exact_frac(const FrameGeom &G, const double *d, double *f) {
    if (G.hortho) {
        f[0] = mul(d[0], G.Hi[0]);
        f[1] = mul(d[1], G.Hi[4]);
        f[2] = mul(d[2], G.Hi[8]);
    } else {
        for (int k = 0; k < 3; ++k) f[k] = add(add(mul(G.Hi[3 * k], d[0]), mul(G.Hi[3 * k + 1], d[1])), mul(G.Hi[3 * k + 2], d[2]));
    }
}

// v = H n (column-major H)
CM_HD void exact_lat(const FrameGeom &G, const double *n, double *v) {
    if (G.hortho) {
        v[0] = mul(G.H[0], n[0]);
        v[1] = mul(G.H[4], n[1]);
        v[2] = mul(G.H[8], n[2]);
    } else {
        for (int k = 0; k < 3; ++k) v[k] = add(add(mul(G.H[k], n[0]), mul(G.H[3 + k], n[1])), mul(G.H[6 + k], n[2]));
    }
}

CM_HD double exact_d2(const FrameGeom &G, const double *x, const double *y) {
    const double d[3] = {sub(y[0], x[0]), sub(y[1], x[1]), sub(y[2], x[2])};
    double f[3], n0[3], e[3];
    exact_frac(G, d, f);
    for (int k = 0; k < 3; ++k) n0[k] = rint(f[k]);
    if (n0[0] != 0.0 || n0[1] != 0.0 || n0[2] != 0.0) {
        double s[3];
        exact_lat(G, n0, s);
        for (int k = 0; k < 3; ++k) e[k] = sub(d[k], s[k]);
    } else {
        for (int k = 0; k < 3; ++k) e[k] = d[k];
    }
    double best = add(add(mul(e[0], e[0]), mul(e[1], e[1])), mul(e[2], e[2]));
    if (best <= mul(G.hw, G.hw)) return best;
    for (int i = -1; i <= 1; ++i)
        for (int j = -1; j <= 1; ++j)
            for (int l = -1; l <= 1; ++l) {
                if (i == 0 && j == 0 && l == 0) continue;
                const double n[3] = {add(n0[0], (double)i), add(n0[1], (double)j), add(n0[2], (double)l)};
                double s[3];
                exact_lat(G, n, s);
                const double t0 = sub(d[0], s[0]), t1 = sub(d[1], s[1]), t2 = sub(d[2], s[2]);
                const double q = add(add(mul(t0, t0), mul(t1, t1)), mul(t2, t2));
                if (q < best) best = q;
            }
    return best;
}

// Position of atom b of a randomly placed solvent molecule, as the random
// insertion defines it (src/rigid_body.jl:107-137, src/mddf.jl:65-88): the
// source molecule made whole around its reference atom xr,
// u_b = x_b - H rint(H^-1 (x_b - xr)); then rotated about the mean of the u
// (cm) by A (row-major) and moved to the new centre ncm:
// p_b = ((A0 w0 + A1 w1) + A2 w2) + ncm, w = u_b - cm.
CM_HD void exact_unwrapped(const FrameGeom &G, const double *xb, const double *xr, double *u) {
    const double d[3] = {sub(xb[0], xr[0]), sub(xb[1], xr[1]), sub(xb[2], xr[2])};
    double f[3], n[3];
    exact_frac(G, d, f);
    for (int k = 0; k < 3; ++k) n[k] = rint(f[k]);
    if (n[0] != 0.0 || n[1] != 0.0 || n[2] != 0.0) {
        double sh[3];
        exact_lat(G, n, sh);
        for (int k = 0; k < 3; ++k) u[k] = sub(xb[k], sh[k]);
    } else {
        for (int k = 0; k < 3; ++k) u[k] = xb[k];
    }
}

CM_HD void exact_placed(const double *u, const double *cm, const double *A, const double *ncm, double *p) {
    const double w[3] = {sub(u[0], cm[0]), sub(u[1], cm[1]), sub(u[2], cm[2])};
    for (int k = 0; k < 3; ++k) p[k] = add(add(add(mul(A[3 * k], w[0]), mul(A[3 * k + 1], w[1])), mul(A[3 * k + 2], w[2])), ncm[k]);
}

CM_HD int cell_linear(const FrameGeom &G, int cx, int cy, int cz) { return (cz * G.n[1] + cy) * G.n[0] + cx; }

CM_HD int off_index(int dx, int dy, int dz) { return ((dz + kLT) * kLTW + (dy + kLT)) * kLTW + (dx + kLT); }

CM_HD int wrapi(int c, int n) {
    int r = c % n;
    return r < 0 ? r + n : r;
}

// wrapi for cell coordinates that are almost always in range already (a
// stencil offset from an in-range cell): the modulo only when they are not.
CM_HD int wrap_cell(int c, int n) { return (unsigned)c < (unsigned)n ? c : wrapi(c, n); }

}  // namespace cmgeom
