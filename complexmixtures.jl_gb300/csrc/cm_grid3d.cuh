// cm_grid3d.cuh -- grid3D (src/tools/grid3D.jl:47-147) on the device: for
// every point of a grid around the solute, the closest solute atom and its
// contribution to the MDDF (or coordination number, md count) interpolated
// at that distance.
//
// One thread per grid point.  The solute atoms are binned on the host into
// cells of side above dmax over the grid's box, so the atoms within dmax of a
// point lie in the 3 x 3 x 3 cells around it; a point whose closest atom is
// farther than dmax is not kept, so the cell search decides the same points as
// the reference's search over all atoms.  Distances are FP64 formed as the
// reference's Euclidean norm, ties go to the lower atom index (the first atom
// at the minimum), and the interpolation keeps the reference's expression, so
// the kept points, atoms, distances and values equal the CPU restatement's.
#pragma once
#include "cm_kernels.cuh"

namespace cmk {

struct GridJob {
    int64_t n[3];            // grid points per axis
    double origin[3];        // xmin - dmax per axis
    double step, dmin, dmax;
    int64_t c[3];            // cells per axis of the atom cell list
    double cell;             // cell side (>= dmax)
    const int *cstart;       // [ncells + 1] atoms of each cell, sorted by cell
    const d4 *atoms;         // [natoms] FP64 position, original 0-based index in w (as a double)
    const int *type;         // [natoms] by original index: row of the table
    const double *table;     // [ntypes][nbins]
    const double *d;         // [nbins] bin distances, increasing
    int nbins;
    int64_t cap;
    unsigned long long *count;
    long long *out_point;
    int *out_atom;
    double *out_r, *out_v;
};

__global__ void k_grid3d(GridJob J) {
    const int64_t total = J.n[0] * J.n[1] * J.n[2];
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ix = g / (J.n[1] * J.n[2]), rem = g - ix * (J.n[1] * J.n[2]);
        const int64_t iy = rem / J.n[2], iz = rem - iy * J.n[2];
        const int64_t idx[3] = {ix, iy, iz};
        double p[3];
        int64_t pc[3];
        for (int k = 0; k < 3; ++k) {
            p[k] = add(J.origin[k], mul(J.step, (double)idx[k]));
            pc[k] = (int64_t)floor(div(sub(p[k], J.origin[k]), J.cell));
        }
        double best = INFINITY;
        int ba = -1;
        for (int64_t cz = pc[2] - 1; cz <= pc[2] + 1; ++cz) {
            if (cz < 0 || cz >= J.c[2]) continue;
            for (int64_t cy = pc[1] - 1; cy <= pc[1] + 1; ++cy) {
                if (cy < 0 || cy >= J.c[1]) continue;
                for (int64_t cx = pc[0] - 1; cx <= pc[0] + 1; ++cx) {
                    if (cx < 0 || cx >= J.c[0]) continue;
                    const int64_t cl = (cz * J.c[1] + cy) * J.c[0] + cx;
                    for (int a = J.cstart[cl]; a < J.cstart[cl + 1]; ++a) {
                        const d4 q = J.atoms[a];
                        const double dx = sub(p[0], q.x), dy = sub(p[1], q.y), dz = sub(p[2], q.z);
                        const double d2 = add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz));
                        const int ia = (int)q.w;
                        if (d2 < best || (d2 == best && ia < ba)) {
                            best = d2;
                            ba = ia;
                        }
                    }
                }
            }
        }
        if (ba < 0) continue;
        const double r = __dsqrt_rn(best);
        if (!(J.dmin < r && r < J.dmax)) continue;
        // first bin distance beyond r (the caller checks d[0] <= dmin and dmax < d[nbins - 1])
        int lo = 0, hi = J.nbins;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (J.d[mid] > r) hi = mid;
            else lo = mid + 1;
        }
        const int iright = lo, ileft = lo - 1;
        if (ileft < 0 || iright >= J.nbins) continue;
        const double *c = J.table + (int64_t)J.type[ba] * J.nbins;
        const double v = add(c[ileft], mul(div(sub(c[iright], c[ileft]), sub(J.d[iright], J.d[ileft])), sub(r, J.d[ileft])));
        if (!(v > 0.0)) continue;
        const unsigned long long slot = atomicAdd(J.count, 1ull);
        if ((int64_t)slot < J.cap) {
            J.out_point[slot] = g;
            J.out_atom[slot] = ba;
            J.out_r[slot] = r;
            J.out_v[slot] = v;
        }
    }
}

}  // namespace cmk
