// cm_atoms32.cuh -- ATOMS layout (molecules above 32 atoms): one warp per
// (solute molecule, solvent molecule) pair that can hold a pair within the
// cutoff.
//
// The solute atoms of each molecule are binned into a cell list; k_atoms_near
// marks every cell within one stencil of an occupied cell ("near").  A solvent
// molecule none of whose atoms sits in a near cell has every atom pair beyond
// the cutoff and is dropped by k_atoms_filter (real pass) or by the placement
// kernel (random insertion); the others go to a queue.  k_atoms_eval takes
// one queue entry per warp.  For dense solutes (many atoms per occupied cell),
// for each solvent atom and stencil cell, the lanes read consecutive solute
// atoms of the cell (coalesced); for sparse solutes the lanes run through the
// atoms of all stencil cells end to end, so no lane idles on a short cell.
// Each lane keeps its own top-2, and a shuffle reduction gives the molecule
// pair's closest pair, second-closest distance and reference-atom row (the
// FP64 engine path takes one thread per entry for sparse solutes).  Cells
// whose box is farther than the cutoff from the atom are skipped.  The
// decision follows the FP32 + guard rules; inside the guard band the exact
// FP64 scan (warp-cooperative in warp mode, reduced in the order of the
// reference's tie rule: distance, then the larger atom-index pair) decides.
// The FP64 engine path runs that exact scan directly.
#pragma once
#include "cm_kernels.cuh"

namespace cmk {

// One CTA of 16 warps per SM (the register budget allows 16 warps at 128
// registers); its warps share one privatised histogram, 1-2% faster than two
// CTAs of 8 warps on configs 1, 2 and 4.
#ifndef CM_ATOMS_WARPS
#define CM_ATOMS_WARPS 16
#endif
constexpr int kAtomsWarps = CM_ATOMS_WARPS;  // warps per CTA of k_atoms_eval
#ifndef CM_ATOMS_MIN_CTAS
#define CM_ATOMS_MIN_CTAS 1         // resident CTAs per SM that k_atoms_eval's register budget is sized for
#endif

// Dilated occupancy of each solute molecule's cell list: near = some cell
// within the ATOMS stencil half-widths La holds an atom of the molecule.
// Grid: x over ms * ncell, y = frame.
__device__ __forceinline__ void k_atoms_near_body(const uint3 blockIdx, const dim3 gridDim, const Bufs &B) {
    const int f = blockIdx.y;
    const FrameGeom &G = B.G[f];
    const FrameScratch &F = B.FS[f];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)B.ms * G.ncell) return;
    const int s = (int)(t / G.ncell), cell = (int)(t - (int64_t)s * G.ncell);
    const int *cs = B.astart + (int64_t)f * B.as + (int64_t)s * G.ncell;
    const int n0 = G.n[0], n1 = G.n[1], n2 = G.n[2];
    const int cx = cell % n0, cy = (cell / n0) % n1, cz = cell / (n0 * n1);
    unsigned char near = 0;
    for (int dz = -F.La[2]; dz <= F.La[2] && !near; ++dz)
        for (int dy = -F.La[1]; dy <= F.La[1] && !near; ++dy)
            for (int dx = -F.La[0]; dx <= F.La[0]; ++dx) {
                const int c = (wrap_cell(cz + dz, n2) * n1 + wrap_cell(cy + dy, n1)) * n0 + wrap_cell(cx + dx, n0);
                if (cs[c + 1] > cs[c]) {
                    near = 1;
                    break;
                }
            }
    B.anear[(int64_t)f * B.as + t] = near;
}

__global__ void k_atoms_near(Bufs B) {
    k_atoms_near_body(blockIdx, gridDim, B);
}

__device__ __forceinline__ int unpack_cell_linear(const FrameGeom &G, int c) {
    return ((c >> 20) * G.n[1] + ((c >> 10) & 1023)) * G.n[0] + (c & 1023);
}

// True if some atom of the solvent molecule at sites[0 .. apv) lies in a
// near cell of solute molecule s.
__device__ __forceinline__ bool atoms_near(const Bufs &B, const FrameGeom &G, int f, int s, const int *cells, int apv) {
    const unsigned char *nm = B.anear + (int64_t)f * B.as + (int64_t)s * G.ncell;
    for (int b = 0; b < apv; ++b)
        if (nm[unpack_cell_linear(G, cells[b])]) return true;
    return false;
}

__device__ __forceinline__ void atoms_push(const DevSys &S, const Bufs &B, int4 e) {
    const int slot = atomicAdd(B.counters + 2, 1);
    if (slot < B.aq_cap) B.aq[slot] = e;
    else raise_err(S, ERR_QUEUE);
}

// Real pass filter, thread per (frame, solute molecule, solvent molecule)
// item in [i0, i0 + n): queue entry (v, s, frame, 0).
__device__ __forceinline__ void k_atoms_filter_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B, int64_t i0, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int64_t it = i0 + t;
    const int64_t per_frame = B.ms * B.mv;
    const int f = (int)(it / per_frame);
    const int64_t r = it - (int64_t)f * per_frame;
    const int s = (int)(r / B.mv), v = (int)(r - (int64_t)s * B.mv);
    if (S.self && v == s) return;
    if (!B.FS[f].ok) {
        raise_err(S, ERR_STENCIL);
        return;
    }
    const FrameGeom &G = B.G[f];
    if (atoms_near(B, G, f, s, B.avcell + (int64_t)f * B.Nv + (int64_t)v * S.apv, S.apv)) atoms_push(S, B, make_int4(v, s, f, 0));
}

__global__ void k_atoms_filter(DevSys S, Bufs B, int64_t i0, int64_t n) {
    k_atoms_filter_body(blockIdx, gridDim, S, B, i0, n);
}

// Top-2 of one lane in the search precision R.
template <typename R>
struct Top2T {
    R m1, m2, r1;
    int p1, b1;
};
using Top2 = Top2T<float>;

template <typename R>
__device__ __forceinline__ void top2_init(Top2T<R> &T) {
    T.m1 = T.m2 = T.r1 = (R)INFINITY;
    T.p1 = 0x7fffffff;
    T.b1 = 0;
}

template <typename R>
__device__ __forceinline__ void top2_merge(Top2T<R> &A, const Top2T<R> &Bt) {
    const R m2 = r_min(r_max(A.m1, Bt.m1), r_min(A.m2, Bt.m2));
    const bool take = Bt.m1 < A.m1 || (Bt.m1 == A.m1 && (Bt.p1 < A.p1 || (Bt.p1 == A.p1 && Bt.b1 < A.b1)));
    if (take) {
        A.m1 = Bt.m1;
        A.p1 = Bt.p1;
        A.b1 = Bt.b1;
    }
    A.m2 = m2;
    A.r1 = r_min(A.r1, Bt.r1);
}

template <typename R>
__device__ __forceinline__ void top2_reduce(Top2T<R> &T) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Top2T<R> U;
        U.m1 = __shfl_xor_sync(0xffffffffu, T.m1, o);
        U.m2 = __shfl_xor_sync(0xffffffffu, T.m2, o);
        U.r1 = __shfl_xor_sync(0xffffffffu, T.r1, o);
        U.p1 = __shfl_xor_sync(0xffffffffu, T.p1, o);
        U.b1 = __shfl_xor_sync(0xffffffffu, T.b1, o);
        top2_merge(T, U);
    }
}

// Exact minimum of one lane, reduced in the reference's order: smaller
// distance first, then the larger (solute atom, solvent atom) index pair.
__device__ __forceinline__ void best_reduce(Best64 &Bst, double &rr1, long long &evals) {
    double d = Bst.d2 <= 1e300 ? best_d(Bst) : INFINITY;
    int a = Bst.a, b = Bst.b;
    double d2 = Bst.d2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xffffffffu, d, o);
        const double od2 = __shfl_xor_sync(0xffffffffu, d2, o);
        const int oa = __shfl_xor_sync(0xffffffffu, a, o), ob = __shfl_xor_sync(0xffffffffu, b, o);
        const bool take = od < d || (od == d && (oa > a || (oa == a && ob > b)));
        if (take) {
            d = od;
            d2 = od2;
            a = oa;
            b = ob;
        }
        rr1 = fmin(rr1, __shfl_xor_sync(0xffffffffu, rr1, o));
        evals += __shfl_xor_sync(0xffffffffu, evals, o);
    }
    Bst.d2 = d2;
    Bst.d = d;
    Bst.a = a;
    Bst.b = b;
}

// Geometry of one solvent site for the stencil walk: its cell, its FP32
// cell-relative position and its fractional position inside the cell.
struct Site {
    int cx, cy, cz;
    float4 q;
    float g[3];
};

__device__ __forceinline__ Site site_of(const FrameScratch &F, int packed, float4 q) {
    Site st;
    st.cx = packed & 1023;
    st.cy = (packed >> 10) & 1023;
    st.cz = (packed >> 20) & 1023;
    st.q = q;
    for (int k = 0; k < 3; ++k) st.g[k] = fmaf(F.hin[3 * k + 2], q.z, fmaf(F.hin[3 * k + 1], q.y, F.hin[3 * k] * q.x));
    return st;
}

// Lower bound of the squared distance from the site to every atom of the
// stencil cell image at offset d: per axis k the cell lies in a slab whose
// distance from the site is (grid units outside the slab) x (cell width
// between the faces).  Orthogonal cells: the slabs' distances add in
// quadrature (the exact box distance); other cells: the largest of them.
__device__ __forceinline__ float cell_d2(const FrameScratch &F, float g0, float g1, float g2, int dx, int dy, int dz) {
    const float ux = (fminf(fmaxf(g0, (float)dx), (float)dx + 1.f) - g0) * F.cw[0];
    const float uy = (fminf(fmaxf(g1, (float)dy), (float)dy + 1.f) - g1) * F.cw[1];
    const float uz = (fminf(fmaxf(g2, (float)dz), (float)dz + 1.f) - g2) * F.cw[2];
    if (F.ortho) return fmaf(uz, uz, fmaf(uy, uy, ux * ux));
    const float m = fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz)));
    return m * m;
}
__device__ __forceinline__ float cell_d2(const FrameScratch &F, const Site &st, int dx, int dy, int dz) {
    return cell_d2(F, st.g[0], st.g[1], st.g[2], dx, dy, dz);
}

// Walk the stencil cells of one site that can hold an atom within the
// cutoff; body(beg, end, oi) for each non-empty one.
template <typename Body>
__device__ __forceinline__ void atoms_walk(const FrameGeom &G, const FrameScratch &F, const int *cs, const Site &st,
                                           float prune2, Body &&body) {
    const int n0 = G.n[0], n1 = G.n[1], n2 = G.n[2];
    for (int dz = -F.La[2]; dz <= F.La[2]; ++dz) {
        const int zc = wrap_cell(st.cz + dz, n2);
        for (int dy = -F.La[1]; dy <= F.La[1]; ++dy) {
            const int row = (zc * n1 + wrap_cell(st.cy + dy, n1)) * n0;
            for (int dx = -F.La[0]; dx <= F.La[0]; ++dx) {
                const int cell = row + wrap_cell(st.cx + dx, n0);
                const int beg = cs[cell], end = cs[cell + 1];
                if (beg == end) continue;
                if (cell_d2(F, st, dx, dy, dz) > prune2) continue;
                body(beg, end, off_index(dx, dy, dz));
            }
        }
    }
}

// Warp-cooperative FP32 walk of a site's stencil, balanced over the lanes
// whatever the cells' sizes.  The lanes take the stencil's cells 32 at a time
// and prefix-sum their atom counts (cells beyond the cutoff count zero); the
// cells' atoms, end to end, are then run through 32 at a time, one pair per
// lane.  Lane l of the window of pairs [kb, kb + 32) belongs to the last cell
// that starts at or before kb + l: every cell with atoms in the window sets
// bit (start - kb, or 0 for the cell running into the window) of a mask and
// leaves its displacement base and atom base in win[that bit], and the lane
// takes the highest set bit at or below l.  body(p, tx, ty, tz) gets the
// solute atom and the site's position relative to that cell image.
template <typename Body>
__device__ __forceinline__ void atoms_walk_flat(const FrameGeom &G, const FrameScratch &F, const int *cs, const Site &st,
                                                float prune2, const float4 *off32, int lane, float4 *win, Body &&body) {
    constexpr unsigned kFull = 0xffffffffu;
    const int nx = 2 * F.La[0] + 1, ny = 2 * F.La[1] + 1;
    const int ncells = nx * ny * (2 * F.La[2] + 1);
    for (int c0 = 0; c0 < ncells; c0 += 32) {
        const int ci = c0 + lane;
        int cnt = 0, beg = 0;
        float tx = 0.f, ty = 0.f, tz = 0.f;
        if (ci < ncells) {
            const int dx = ci % nx - F.La[0], dy = (ci / nx) % ny - F.La[1], dz = ci / (nx * ny) - F.La[2];
            const int cell = (wrap_cell(st.cz + dz, G.n[2]) * G.n[1] + wrap_cell(st.cy + dy, G.n[1])) * G.n[0] +
                             wrap_cell(st.cx + dx, G.n[0]);
            beg = cs[cell];
            const int end = cs[cell + 1];
            if (end > beg && cell_d2(F, st, dx, dy, dz) <= prune2) {
                cnt = end - beg;
                const float4 of = off32[off_index(dx, dy, dz)];
                tx = st.q.x - of.x;
                ty = st.q.y - of.y;
                tz = st.q.z - of.z;
            }
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += u;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        const int excl = incl - cnt;
        for (int kb = 0; kb < total; kb += 32) {
            const bool in = cnt > 0 && excl < kb + 32 && incl > kb;
            const int pos = in ? max(excl - kb, 0) : 0;
            if (in) win[pos] = make_float4(tx, ty, tz, __int_as_float(beg - excl));
            const unsigned m = __reduce_or_sync(kFull, in ? (1u << pos) : 0u);
            __syncwarp();
            const int k = kb + lane;
            if (k < total) {
                const float4 w = win[31 - __clz(m & (kFull >> (31 - lane)))];
                body(__float_as_int(w.w) + k, w.x, w.y, w.z);
            }
            __syncwarp();
        }
    }
}

// Up to kSiteGroup sites of one solvent molecule walked together (FP32): the
// stencils of the sites are one box of cells around the cell of the group's
// first site (the reference cell), each solute atom is loaded once per walk
// and compared with every site of the group.  Sites are given relative to the
// reference cell's origin, q_j + off(d_j) with d_j the site's cell offset
// from the reference cell, so the displacement of a pair is
// (q_a + off(cell_a - ref)) - (q_j + off(d_j)); its FP32 error is within the
// frame's guard band, whose offset bound covers one cell beyond the ATOMS
// stencil for that reason.
constexpr int kSiteGroup = 4;

struct SiteGroup {
    int ns;                           // sites in the group
    int cx, cy, cz;                   // reference cell
    int lo[3], hi[3];                 // range of the sites' cell offsets d_j
    float qx[kSiteGroup], qy[kSiteGroup], qz[kSiteGroup];  // q_j + off(d_j)
    const float4 *site;               // per-warp shared table: (fractional position in the cell, packed d_j)
};

__device__ __forceinline__ int unpack_d(float w, int k) { return ((__float_as_int(w) >> (2 * k)) & 3) - 1; }

// Sets up the group of sites [b0, b0 + ns) of a molecule, lane j taking site
// j; false when a site's cell is more than one cell from the reference cell
// or the walk box would leave the offset table (the sites are then walked one
// by one).  `tab` is the warp's kSiteGroup-entry shared table.
__device__ __forceinline__ bool site_group(const FrameGeom &G, const FrameScratch &F, const float4 *off32,
                                           const int *cells, const float4 *q32, int b0, int ns, int lane, float4 *tab,
                                           SiteGroup &sg) {
    constexpr unsigned kFull = 0xffffffffu;
    const int pk0 = cells[b0];
    sg.ns = ns;
    sg.cx = pk0 & 1023;
    sg.cy = (pk0 >> 10) & 1023;
    sg.cz = (pk0 >> 20) & 1023;
    const int ref[3] = {sg.cx, sg.cy, sg.cz};
    bool bad = false;
    int d[3] = {0, 0, 0};
    float qx = 0.f, qy = 0.f, qz = 0.f;
    if (lane < ns) {
        const int pk = cells[b0 + lane];
        const int c[3] = {pk & 1023, (pk >> 10) & 1023, (pk >> 20) & 1023};
        const float4 q = q32[b0 + lane];
        float g[3];
        int code = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            int t = c[k] - ref[k];
            if (2 * t > G.n[k]) t -= G.n[k];
            else if (2 * t < -G.n[k]) t += G.n[k];
            if (t < -1 || t > 1) bad = true;
            d[k] = max(-1, min(1, t));
            code |= (d[k] + 1) << (2 * k);
            g[k] = fmaf(F.hin[3 * k + 2], q.z, fmaf(F.hin[3 * k + 1], q.y, F.hin[3 * k] * q.x));
        }
        const float4 of = off32[off_index(d[0], d[1], d[2])];
        qx = q.x + of.x;
        qy = q.y + of.y;
        qz = q.z + of.z;
        tab[lane] = make_float4(g[0], g[1], g[2], __int_as_float(code));
    }
#pragma unroll
    for (int j = 0; j < kSiteGroup; ++j) {
        sg.qx[j] = __shfl_sync(kFull, qx, j);
        sg.qy[j] = __shfl_sync(kFull, qy, j);
        sg.qz[j] = __shfl_sync(kFull, qz, j);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        sg.lo[k] = __reduce_min_sync(kFull, d[k]);
        sg.hi[k] = __reduce_max_sync(kFull, d[k]);
        if (sg.hi[k] + F.La[k] > kLT || sg.lo[k] - F.La[k] < -kLT) bad = true;
    }
    sg.site = tab;
    __syncwarp();
    return !__any_sync(kFull, bad);
}

// The group's walk box: cells at offsets [lo - La, hi + La] from the
// reference cell; a cell is kept if its box lies within the cutoff of some
// site.  The kept cells' atoms run end to end, 32 pairs of lanes at a time
// (as in atoms_walk_flat).  body(p, ox, oy, oz) gets the solute atom and
// off(cell - ref).
template <typename Body>
__device__ __forceinline__ void atoms_walk_group(const FrameGeom &G, const FrameScratch &F, const int *cs,
                                                 const SiteGroup &sg, float prune2, const float4 *off32, int lane,
                                                 float4 *win, Body &&body) {
    constexpr unsigned kFull = 0xffffffffu;
    const int x0 = sg.lo[0] - F.La[0], y0 = sg.lo[1] - F.La[1], z0 = sg.lo[2] - F.La[2];
    const int nx = sg.hi[0] - x0 + F.La[0] + 1, ny = sg.hi[1] - y0 + F.La[1] + 1, nz = sg.hi[2] - z0 + F.La[2] + 1;
    const int ncells = nx * ny * nz;
    auto probe = [&](int ci, int &beg, int &end, float4 &of) {
        const int dx = x0 + ci % nx, dy = y0 + (ci / nx) % ny, dz = z0 + ci / (nx * ny);
        const int cell = (wrap_cell(sg.cz + dz, G.n[2]) * G.n[1] + wrap_cell(sg.cy + dy, G.n[1])) * G.n[0] +
                         wrap_cell(sg.cx + dx, G.n[0]);
        beg = cs[cell];
        end = cs[cell + 1];
        bool near = false;
        for (int j = 0; j < sg.ns; ++j) {
            const float4 t = sg.site[j];
            near = near || cell_d2(F, t.x, t.y, t.z, dx - unpack_d(t.w, 0), dy - unpack_d(t.w, 1), dz - unpack_d(t.w, 2)) <= prune2;
        }
        if (!near) end = beg;
        if (end > beg) of = off32[off_index(dx, dy, dz)];
    };
    for (int c0 = 0; c0 < ncells; c0 += 32) {
        const int ci = c0 + lane;
        int cnt = 0, beg = 0;
        float4 of = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ci < ncells) {
            int end;
            probe(ci, beg, end, of);
            cnt = end - beg;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += u;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        const int excl = incl - cnt;
        for (int kb = 0; kb < total; kb += 32) {
            const bool in = cnt > 0 && excl < kb + 32 && incl > kb;
            const int pos = in ? max(excl - kb, 0) : 0;
            if (in) win[pos] = make_float4(of.x, of.y, of.z, __int_as_float(beg - excl));
            const unsigned m = __reduce_or_sync(kFull, in ? (1u << pos) : 0u);
            __syncwarp();
            const int k = kb + lane;
            if (k < total) {
                const float4 w = win[31 - __clz(m & (kFull >> (31 - lane)))];
                body(__float_as_int(w.w) + k, w.x, w.y, w.z);
            }
            __syncwarp();
        }
    }
}

// Dense solutes (cell schedule): the group's walk box with the lanes probing
// 32 cells at once; each kept cell carries the mask of the sites whose own
// stencil keeps it (its box within the cutoff of the site), so every site
// meets exactly the cells of its per-site walk, and the lanes then run over
// each kept cell's atoms.  body(p, ox, oy, oz, mask).
template <typename Body>
__device__ __forceinline__ void atoms_walk_group_cells(const FrameGeom &G, const FrameScratch &F, const int *cs,
                                                       const SiteGroup &sg, float prune2, const float4 *off32, int lane,
                                                       Body &&body) {
    constexpr unsigned kFull = 0xffffffffu;
    const int x0 = sg.lo[0] - F.La[0], y0 = sg.lo[1] - F.La[1], z0 = sg.lo[2] - F.La[2];
    const int nx = sg.hi[0] - x0 + F.La[0] + 1, ny = sg.hi[1] - y0 + F.La[1] + 1, nz = sg.hi[2] - z0 + F.La[2] + 1;
    const int ncells = nx * ny * nz;
    for (int c0 = 0; c0 < ncells; c0 += 32) {
        const int ci = c0 + lane;
        int beg = 0, end = 0;
        unsigned mask = 0;
        float4 of = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ci < ncells) {
            const int dx = x0 + ci % nx, dy = y0 + (ci / nx) % ny, dz = z0 + ci / (nx * ny);
            const int cell = (wrap_cell(sg.cz + dz, G.n[2]) * G.n[1] + wrap_cell(sg.cy + dy, G.n[1])) * G.n[0] +
                             wrap_cell(sg.cx + dx, G.n[0]);
            beg = cs[cell];
            end = cs[cell + 1];
            for (int j = 0; j < sg.ns; ++j) {
                const float4 t = sg.site[j];
                if (cell_d2(F, t.x, t.y, t.z, dx - unpack_d(t.w, 0), dy - unpack_d(t.w, 1), dz - unpack_d(t.w, 2)) <= prune2)
                    mask |= 1u << j;
            }
            if (end > beg && mask) of = off32[off_index(dx, dy, dz)];
        }
        unsigned todo = __ballot_sync(kFull, end > beg && mask != 0);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int b0 = __shfl_sync(kFull, beg, src), e0 = __shfl_sync(kFull, end, src);
            const unsigned m = __shfl_sync(kFull, mask, src);
            const float ox = __shfl_sync(kFull, of.x, src), oy = __shfl_sync(kFull, of.y, src),
                        oz = __shfl_sync(kFull, of.z, src);
            for (int p = b0 + lane; p < e0; p += 32) body(p, ox, oy, oz, m);
        }
    }
}

// What the exact scan of one queued molecule pair reads.
struct AtomsPair {
    const FrameGeom *G;
    const FrameScratch *F;
    const int *vcell;
    const float4 *vq32;
    const d4 *vq64;
    const d4 *off64;
    const float4 *off32;
    const float4 *sq32;
    const d4 *sq64;
    const int *cs;
    int64_t vb;
    float prune2;
    // the pair, for the exact distances: frame, solute molecule, solvent
    // molecule or slot, and for a random slot its sample
    int f, s, v, sample;
    bool random;
};

__device__ __forceinline__ const d4 *sq_of(const AtomsPair &A, double) { return A.sq64; }
__device__ __forceinline__ const float4 *sq_of(const AtomsPair &A, float) { return A.sq32; }
__device__ __forceinline__ const d4 *vq_of(const AtomsPair &A, double) { return A.vq64; }
__device__ __forceinline__ const float4 *vq_of(const AtomsPair &A, float) { return A.vq32; }
__device__ __forceinline__ const d4 *off_of(const AtomsPair &A, double) { return A.off64; }
__device__ __forceinline__ const float4 *off_of(const AtomsPair &A, float) { return A.off32; }

// The pair's molecules for the exact distances; a random slot's placement is
// drawn again from its stream (the same draws as k_atoms_place).
__device__ __noinline__ ExactMol atoms_exact_mol(const DevSys &S, const Bufs &B, const AtomsPair &A) {
    if (!A.random) return exact_mol(S, A.f, A.s, A.v);
    const Sample sm = B.samples[A.sample];
    const Placement P = draw_placement(S, A.G->frame_id, sm, A.v, B.bulk + (int64_t)A.f * B.ndist * B.mv,
                                       B.nbulk + (int64_t)A.f * B.ndist);
    uint64_t st = P.st;
    double R[9];
    draw_rotation(st, R);
    return exact_mol_placed(S, *A.G, A.f, A.s, P.jmol, P.fc, R);
}

// Exact scan of a molecule pair; STRIDE 32: lanes over the atoms of each cell
// (the whole warp calls it, the result is reduced over the lanes); STRIDE 1:
// one thread.  Only the pairs whose squared distance in the search precision
// R is within the thresholds are evaluated exactly (exact_d2 on the input
// coordinates).  Out of line: it runs only for records inside the guard band,
// and keeps its registers away from the search loops.
template <int STRIDE, typename R>
__device__ __noinline__ void atoms_exact(const DevSys &S, const Bufs &B, const AtomsPair &A, int lane, R thr_arg, R thr_r1,
                                         Best64 &Bst, double &rr1, long long &evals) {
    using V = typename Vec4T<R>::type;
    best_init(Bst);
    rr1 = INFINITY;
    evals = 0;
    const int apv = S.apv, iref = S.iref;
    const V *sq = sq_of(A, (R)0), *vq = vq_of(A, (R)0), *off = off_of(A, (R)0);
    ExactMol X = atoms_exact_mol(S, B, A);
    for (int b = 0; b < apv; ++b) {
        const Site sb = site_of(*A.F, A.vcell[A.vb + b], A.vq32[A.vb + b]);
        const V qb = vq[A.vb + b];
        double yb[3];
        bool have_y = false;
        atoms_walk(*A.G, *A.F, A.cs, sb, A.prune2, [&](int beg, int end, int oi) {
            const V o = off[oi];
            const R tx = (R)qb.x - (R)o.x, ty = (R)qb.y - (R)o.y, tz = (R)qb.z - (R)o.z;
            for (int p = beg + lane; p < end; p += STRIDE) {
                const V qa = sq[p];
                const R d2f = sq3((R)qa.x - tx, (R)qa.y - ty, (R)qa.z - tz);
                if (!(d2f <= thr_arg || (b == iref && d2f <= thr_r1))) continue;
                if (!have_y) {
                    exact_solvent_atom(B, *A.G, X, b, yb);
                    have_y = true;
                }
                const int a = __float_as_int(A.sq32[p].w);
                double xa[3];
                exact_solute_atom(B, X, a, xa);
                const double d2 = exact_d2(*A.G, xa, yb);
                evals++;
                if (d2 <= S.cut2) {
                    if (b == iref) rr1 = fmin(rr1, d2);
                    best_update<false>(Bst, d2, a, b);
                }
            }
        });
    }
    if (STRIDE == 32) best_reduce(Bst, rr1, evals);
}

// FP64 search of a molecule pair (the FP64 engine path): each site's stencil
// cells, every solute atom in them, squared distances from the FP64
// cell-relative positions; top-2 per lane, reduced over the warp for STRIDE 32.
template <int STRIDE>
__device__ __noinline__ Top2T<double> atoms_pass64(const DevSys &S, const AtomsPair &A, int lane, long long &evals) {
    Top2T<double> T;
    top2_init(T);
    const int apv = S.apv, iref = S.iref;
    for (int b = 0; b < apv; ++b) {
        const Site sb = site_of(*A.F, A.vcell[A.vb + b], A.vq32[A.vb + b]);
        const d4 qb = A.vq64[A.vb + b];
        const bool isref = b == iref;
        atoms_walk(*A.G, *A.F, A.cs, sb, A.prune2, [&](int beg, int end, int oi) {
            const d4 o = A.off64[oi];
            const double tx = qb.x - o.x, ty = qb.y - o.y, tz = qb.z - o.z;
            for (int p = beg + lane; p < end; p += STRIDE) {
                const d4 qa = A.sq64[p];
                const double d2 = sq3(qa.x - tx, qa.y - ty, qa.z - tz);
                evals++;
                T.m2 = fmin(T.m2, fmax(T.m1, d2));
                const bool lt = d2 < T.m1;
                T.p1 = lt ? p : T.p1;
                T.b1 = lt ? b : T.b1;
                T.m1 = fmin(T.m1, d2);
                if (isref) T.r1 = fmin(T.r1, d2);
            }
        });
    }
    if (STRIDE == 32) top2_reduce(T);
    return T;
}

// The record of a molecule pair from its search's top-2 (precision R): taken
// from the search where every value is farther than the band from its
// decision boundary, otherwise from exact distances.  With STRIDE 32 every
// lane holds the same T and takes the same branches.
template <int STRIDE, typename R>
__device__ __noinline__ DirRec atoms_decide(const DevSys &S, const Bufs &B, const AtomsPair &A, const GuardT<R> &g, const Top2T<R> &T,
                               int lane, LocalStats &st) {
    DirRec r = dir_none(S);
    if (!(T.m1 <= g.cutp2)) return r;
    auto from_exact = [&](Best64 &Bst, double rr1) {
        DirRec q = dir_none(S);
        if (Bst.d2 <= S.cut2) {
            const double d = best_d(Bst);
            q.within = 1;
            q.i_local = Bst.a;
            q.j = A.vb + Bst.b;
            q.bin = setbin0(d, S.binstep);
            q.bulk = inbulk64(S, true, d);
            if (rr1 <= S.cut2) { q.ref = 1; q.rbin = setbin0(sqrt(rr1), S.binstep); }
        }
        return q;
    };
    const R d1 = r_sqrt(T.m1);
    const bool amb = T.m1 >= g.cutm2 || (r_sqrt(T.m2) - d1) <= g.two_delta;
    if (amb) {
        R thr1 = (R)-1;
        if (T.r1 <= g.cutp2) thr1 = r_sq_ru(r_sqrt(T.r1) + g.two_delta);
        Best64 Bst;
        double rr1;
        long long ev;
        atoms_exact<STRIDE, R>(S, B, A, lane, r_sq_ru(d1 + g.two_delta), thr1, Bst, rr1, ev);
        r = from_exact(Bst, rr1);
        if (lane == 0) {
            st.guard++;
            st.guard_pairs += ev;
            if (Bst.d2 <= S.cut2) st.maxerr = fmax(st.maxerr, fabs((double)d1 - best_d(Bst)));
        }
        return r;
    }
    // unambiguous: the search's minimum pair is the exact minimum pair
    int bin = bin_of(g, d1);
    double d64 = -1.0;
    const int a1 = __float_as_int(A.sq32[T.p1].w);
    if (bin < 0 || (S.usecutoff && d1 >= g.dbulk_lo && d1 <= g.dbulk_hi)) {
        ExactMol X = atoms_exact_mol(S, B, A);
        d64 = sqrt(exact_pair_d2(B, *A.G, X, a1, T.b1));
        bin = setbin0(d64, S.binstep);
        if (lane == 0) {
            st.guard++;
            st.guard_pairs++;
            st.maxerr = fmax(st.maxerr, fabs((double)d1 - d64));
        }
    }
    r.within = 1;
    r.i_local = a1;
    r.j = A.vb + T.b1;
    r.bin = bin;
    r.bulk = S.usecutoff ? (d64 >= 0.0 ? (d64 > S.dbulk) : (d1 > g.dbulk_hi)) : 0;
    if (T.r1 <= g.cutp2) {
        const int rb = T.r1 < g.cutm2 ? bin_of(g, r_sqrt(T.r1)) : -1;
        if (rb >= 0) {
            r.ref = 1;
            r.rbin = rb;
        } else {
            Best64 Bst;
            double rr1;
            long long ev;
            atoms_exact<STRIDE, R>(S, B, A, lane, (R)-1, r_sq_ru(r_sqrt(T.r1) + g.two_delta), Bst, rr1, ev);
            if (lane == 0) {
                st.guard++;
                st.guard_pairs += ev;
            }
            if (rr1 <= S.cut2) { r.ref = 1; r.rbin = setbin0(sqrt(rr1), S.binstep); }
        }
    }
    return r;
}

// Schedules of k_atoms_eval.  CELL: one warp per queue entry, the lanes over
// the atoms of each stencil cell in turn (dense solutes: cells of a warp's
// worth of atoms or more).  BALANCED: one warp per entry, the lanes over the
// cells' atoms end to end (atoms_walk_flat; sparse solutes in FP32).  THREAD:
// one thread per entry (sparse solutes in the FP64 engine path).
enum AtomsSched { kSchedThread = 0, kSchedCell = 1, kSchedBalanced = 2 };

// ATOMS evaluation of the queue (persistent grid).
template <bool FP32, bool RANDOM, int SCHED>
__device__ __forceinline__ void k_atoms_eval_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B) {
    constexpr bool WARP = SCHED != kSchedThread;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float4 s_win[kAtomsWarps][32];  // atoms_walk_flat's window table, one per warp
    __shared__ float4 s_site[kAtomsWarps][kSiteGroup];  // site_group's table, one per warp
    // an empty queue (every frame of the chunk decided on its candidate grid): nothing to add
    if (B.counters[2] == 0) return;
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    LocalStats st;
    float4 *win = s_win[threadIdx.x >> 5];
    // WARP: one warp per queue entry, lanes over the atoms of each cell;
    // otherwise one thread per entry (lane 0 of a one-thread "warp")
    constexpr int STRIDE = WARP ? 32 : 1;
    const int lane = WARP ? (threadIdx.x & 31) : 0;
    const int worker = WARP ? (threadIdx.x >> 5) : threadIdx.x;
    const int per_block = WARP ? kAtomsWarps : kAtomsWarps * 32;
    const int n = min(B.counters[2], B.aq_cap);
    const int apv = S.apv, iref = S.iref;
    for (int it = blockIdx.x * per_block + worker; it < n; it += gridDim.x * per_block) {
        const int4 e = B.aq[it];
        int v, s, f;
        const int *vcell;
        const float4 *vq32;
        const d4 *vq64;
        if (RANDOM) {
            const Sample sm = B.samples[e.z];
            v = e.x;
            s = sm.s;
            f = sm.pad;
            vcell = B.pcell + (int64_t)e.y * B.Nv;
            vq32 = B.pq32 + (int64_t)e.y * B.Nv;
            vq64 = B.pq64 + (int64_t)e.y * B.Nv;
        } else {
            v = e.x;
            s = e.y;
            f = e.z;
            vcell = B.avcell + (int64_t)f * B.Nv;
            vq32 = B.avq32 + (int64_t)f * B.Nv;
            vq64 = B.avq64 + (int64_t)f * B.Nv;
        }
        const FrameGeom &G = B.G[f];
        const FrameScratch &F = B.FS[f];
        const Guard g = F.g;
        const d4 *off64 = B.off64 + (int64_t)f * kOffEntries;
        const float4 *off32 = B.off32 + (int64_t)f * kOffEntries;
        const float4 *sq32 = B.asq32 + (int64_t)f * B.Ns;
        const d4 *sq64 = B.asq64 + (int64_t)f * B.Ns;
        const int *cs = B.astart + (int64_t)f * B.as + (int64_t)s * G.ncell;
        const float prune2 = g.cut_pre * g.cut_pre;
        const int64_t vb = (int64_t)v * apv;

        AtomsPair A;
        A.G = &G;
        A.F = &F;
        A.vcell = vcell;
        A.vq32 = vq32;
        A.vq64 = vq64;
        A.off64 = off64;
        A.off32 = off32;
        A.sq32 = sq32;
        A.sq64 = sq64;
        A.cs = cs;
        A.vb = vb;
        A.prune2 = prune2;
        A.f = f;
        A.s = s;
        A.v = v;
        A.sample = RANDOM ? e.z : -1;
        A.random = RANDOM;
        DirRec r = dir_none(S);
        long long lane_evals = 0;
        if (!FP32) {
            const Top2T<double> T = atoms_pass64<STRIDE>(S, A, lane, lane_evals);
            r = atoms_decide<STRIDE, double>(S, B, A, F.g64, T, lane, st);
        } else {
            Top2 T;
            top2_init(T);
            // one site with its own stencil walk
            auto one_site = [&](int b) {
                const Site sb = site_of(F, vcell[vb + b], vq32[vb + b]);
                const bool isref = b == iref;
                auto pair = [&](int p, float tx, float ty, float tz) {
                    lane_evals++;
                    const float4 qa = sq32[p];
                    const float ex = qa.x - tx, ey = qa.y - ty, ez = qa.z - tz;
                    const float d2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                    T.m2 = fminf(T.m2, fmaxf(T.m1, d2));
                    const bool lt = d2 < T.m1;
                    T.p1 = lt ? p : T.p1;
                    T.b1 = lt ? b : T.b1;
                    T.m1 = fminf(T.m1, d2);
                    if (isref) T.r1 = fminf(T.r1, d2);
                };
                if (SCHED == kSchedBalanced) {
                    atoms_walk_flat(G, F, cs, sb, prune2, off32, lane, win, pair);
                } else {
                    atoms_walk(G, F, cs, sb, prune2, [&](int beg, int end, int oi) {
                        const float4 of = off32[oi];
                        const float tx = sb.q.x - of.x, ty = sb.q.y - of.y, tz = sb.q.z - of.z;
                        for (int p = beg + lane; p < end; p += STRIDE) pair(p, tx, ty, tz);
                    });
                }
            };
            if constexpr (SCHED == kSchedCell) {
                // dense solutes: the sites of a group probe their cells together and
                // share each solute-atom load; a site meets only its own stencil's cells
                for (int b0 = 0; b0 < apv; b0 += kSiteGroup) {
                    const int ns = min(kSiteGroup, apv - b0);
                    SiteGroup sg;
                    if (!site_group(G, F, off32, vcell + vb, vq32 + vb, b0, ns, lane, s_site[threadIdx.x >> 5], sg)) {
                        for (int b = b0; b < b0 + ns; ++b) one_site(b);
                        continue;
                    }
                    auto pairs = [&](int p, float ox, float oy, float oz, unsigned m) {
                        const float4 qa = sq32[p];
                        const float ux = qa.x + ox, uy = qa.y + oy, uz = qa.z + oz;
#pragma unroll
                        for (int j = 0; j < kSiteGroup; ++j) {
                            if (!((m >> j) & 1u)) continue;
                            lane_evals++;
                            const float ex = ux - sg.qx[j], ey = uy - sg.qy[j], ez = uz - sg.qz[j];
                            const float d2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                            T.m2 = fminf(T.m2, fmaxf(T.m1, d2));
                            const bool lt = d2 < T.m1;
                            T.p1 = lt ? p : T.p1;
                            T.b1 = lt ? b0 + j : T.b1;
                            T.m1 = fminf(T.m1, d2);
                            if (b0 + j == iref) T.r1 = fminf(T.r1, d2);
                        }
                    };
                    atoms_walk_group_cells(G, F, cs, sg, prune2, off32, lane, pairs);
                }
            } else if constexpr (SCHED == kSchedBalanced) {
                // sparse solutes: the sites of a group share one walk
                for (int b0 = 0; b0 < apv; b0 += kSiteGroup) {
                    const int ns = min(kSiteGroup, apv - b0);
                    SiteGroup sg;
                    if (!site_group(G, F, off32, vcell + vb, vq32 + vb, b0, ns, lane, s_site[threadIdx.x >> 5], sg)) {
                        for (int b = b0; b < b0 + ns; ++b) one_site(b);
                        continue;
                    }
                    // the group's sites against each solute atom of the walk box
                    auto pairs = [&](int p, float ox, float oy, float oz) {
                        lane_evals += ns;
                        const float4 qa = sq32[p];
                        const float ux = qa.x + ox, uy = qa.y + oy, uz = qa.z + oz;
#pragma unroll
                        for (int j = 0; j < kSiteGroup; ++j) {
                            if (j >= ns) break;
                            const float ex = ux - sg.qx[j], ey = uy - sg.qy[j], ez = uz - sg.qz[j];
                            const float d2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                            T.m2 = fminf(T.m2, fmaxf(T.m1, d2));
                            const bool lt = d2 < T.m1;
                            T.p1 = lt ? p : T.p1;
                            T.b1 = lt ? b0 + j : T.b1;
                            T.m1 = fminf(T.m1, d2);
                            if (b0 + j == iref) T.r1 = fminf(T.r1, d2);
                        }
                    };
                    atoms_walk_group(G, F, cs, sg, prune2, off32, lane, win, pairs);
                }
            } else {
                for (int b = 0; b < apv; ++b) one_site(b);
            }
            if (WARP) top2_reduce(T);
            r = atoms_decide<STRIDE, float>(S, B, A, g, T, lane, st);
        }
        st.atompairs += (unsigned long long)lane_evals;
        if (lane == 0) {
            st.molpairs++;
            if (r.within) {
                apply_hit(S, h, RANDOM, r.bin, r.i_local, r.j, r.ref, r.rbin);
                st.hits++;
                if (!RANDOM && B.slot) {
                    const int sl = B.slot[(int64_t)f * B.ms + s];
                    if (sl >= 0) B.flags[((int64_t)f * B.ndist + sl) * S.mv + v] = flag_code(r);
                }
            }
        }
        if (WARP) __syncwarp();
    }
    stats_flush(S, st, RANDOM);
    __syncthreads();
    shist_flush(S, h, RANDOM);
}

template <bool FP32, bool RANDOM, int SCHED>
__global__ void __launch_bounds__(kAtomsWarps * 32, CM_ATOMS_MIN_CTAS) k_atoms_eval(DevSys S, Bufs B) {
    k_atoms_eval_body<FP32, RANDOM, SCHED>(blockIdx, gridDim, S, B);
}

}  // namespace cmk
