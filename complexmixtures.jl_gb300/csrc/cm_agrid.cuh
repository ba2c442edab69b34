// cm_agrid.cuh -- candidate grid of the ATOMS layout for a single solute
// molecule (a protein or a long chain: configs 1, 2 and 4), FP32 search.
//
// The question the ATOMS search answers per solvent molecule is, site by
// site, "which solute atom is closest, how close is the second, and how close
// is the closest atom to the reference site" (src/minimum_distances.jl:30-39,
// 107-120).  With one solute molecule that is a nearest-neighbour query
// against one fixed point set per frame, asked once per real solvent molecule
// and n_random_samples times per slot of the random insertion
// (src/mddf.jl:65-88, 403-423).  So per frame each search cell is split into
// K^3 fine cells, and each fine cell g gets the list of solute atoms a with
//
//     dmin(a, g) <= min( min_a' dmax(a', g), cutoff ) + margin,
//
// dmin / dmax the smallest / largest distance from a to a point of g (exact
// box distances for orthogonal cells, the fine cell's bounding sphere
// otherwise) and margin = 2 delta + 1e-3 (1 + cutoff).  For a point y of g the
// nearest atom is within min_a' dmax(a', g), so the list holds every atom
// within (nearest distance + 2 delta) of y, and every atom within the cutoff
// when nothing is closer.  A query (one site) reads its fine cell's list and
// evaluates only those atoms: the smallest FP32 distance, its atom, the
// second-smallest value (exact whenever it is within 2 delta of the smallest;
// the guard test only asks that) and the reference site's smallest distance
// are then the values a walk over every stencil cell gives, and every decision
// follows the FP32 + guard rules of atoms_decide.  A query whose record lies
// inside the guard band is decided in place from exact distances
// (agrid_record), its exact scans reading the same lists, so the counts stay
// the oracle's.
//
// A list entry is the atom's FP32 position from the fine cell's search-cell
// origin, q_a + off(cell_a - cell), which is the displacement form of the
// ATOMS walks (the guard band's error bound covers it), and the atom's index
// in the molecule.
//
// Kernels: k_agrid_build (the lists of every frame, one CTA per search cell,
// space reserved in a per-frame pool; a frame whose pool runs out loses its
// grid), k_agrid_real (real pass) and k_agrid_random (random insertion: the
// queries of the slots k_slot_filter listed and k_atoms_place placed).
// Frames without a grid take the walk path: k_agrid_real queues their
// molecule pairs for k_atoms_eval as k_atoms_filter does, and k_atoms_place
// queues their slots.
#pragma once
#include "cm_atoms32.cuh"

namespace cmk {

constexpr int kAgridMaxK = 6;          // fine cells per search-cell axis
constexpr int kAgridBuckets = 8;       // each list ordered by bucket of the atom's smallest distance to the fine cell
constexpr int kAgridStage = 3072;      // stencil atoms staged in shared memory at a time (48 KB, dynamic)
constexpr int kAgridRound = 4;         // stencil atoms each thread loads per staging round
constexpr int kAgridBuildThreads = 256;

// The fine cells of a search cell: edge vectors and bounds, FP32.
// Largest distance from p to a point of the fine cell centred at c: squared
// for orthogonal cells, the distance to the centre squared otherwise (the
// bound is then that distance + R).
__device__ __forceinline__ float fine_far2(const FineCells &fc, const float *c, const float4 &p) {
    const float dx = fabsf(p.x - c[0]), dy = fabsf(p.y - c[1]), dz = fabsf(p.z - c[2]);
    if (fc.ortho) {
        const float vx = dx + fc.h[0], vy = dy + fc.h[1], vz = dz + fc.h[2];
        return fmaf(vz, vz, fmaf(vy, vy, vx * vx));
    }
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// Smallest distance from p to the fine cell, squared (orthogonal cells), or
// the squared distance to the centre (the bound is then that distance - R).
__device__ __forceinline__ float fine_near2(const FineCells &fc, const float *c, const float4 &p) {
    const float dx = fabsf(p.x - c[0]), dy = fabsf(p.y - c[1]), dz = fabsf(p.z - c[2]);
    if (fc.ortho) {
        const float ux = fmaxf(dx - fc.h[0], 0.f), uy = fmaxf(dy - fc.h[1], 0.f), uz = fmaxf(dz - fc.h[2], 0.f);
        return fmaf(uz, uz, fmaf(uy, uy, ux * ux));
    }
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// Lists of the fine cells of one search cell (grid: x = search cell, y =
// frame), in one pass.  The CTA stages the cell's stencil atoms in shared
// memory; each warp takes fine cells in turn and its lanes split the staged
// atoms (warp reductions, and ballots for the compacted writes).  The CTA
// counts its lists by bucket, reserves their room in the frame's entry pool
// with one atomic, writes each fine cell's bucket starts and end to gstart and
// its bucket edges to gedge, then the entries.  A frame whose pool runs out
// loses its grid (its queries take the walk).
__device__ __forceinline__ void k_agrid_build_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B) {
    extern __shared__ float4 s_at[];  // kAgridStage entries
    __shared__ int s_pre[kAgridMaxStencil + 1];
    __shared__ int s_beg[kAgridMaxStencil];
    __shared__ short s_oi[kAgridMaxStencil];
    __shared__ float s_far[kAgridMaxK * kAgridMaxK * kAgridMaxK], s_near[kAgridMaxK * kAgridMaxK * kAgridMaxK];
    __shared__ int s_pos[kAgridMaxK * kAgridMaxK * kAgridMaxK][kAgridBuckets];
    __shared__ int s_wsum[kAgridBuildThreads / 32];
    __shared__ int s_base;
    __shared__ float s_tmax;
    const int f = blockIdx.y;
    const int c = blockIdx.x;
    const FrameGeom &G = B.G[f];
    const FrameScratch &F = B.FS[f];
    if (c >= G.ncell) return;
    const int K = B.agk, K3 = K * K * K;
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5, nwarps = blockDim.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    const int64_t gbase = ((int64_t)f * B.gfs + (int64_t)c * K3) * (kAgridBuckets + 1);  // bucket starts and end
    const int64_t ebase = (int64_t)f * B.gfs + (int64_t)c * K3;                            // fine-cell bucket edges
    const bool active = F.agrid && B.anear[(int64_t)f * B.as + c];
    if (!active) {
        // no solute atom within a stencil of this cell: empty lists
        for (int g = t; g < K3 * (kAgridBuckets + 1); g += blockDim.x) B.gstart[gbase + g] = 0;
        for (int g = t; g < K3; g += blockDim.x) B.gedge[ebase + g] = make_float2(0.f, 0.f);
        return;
    }
    const int La0 = F.La[0], La1 = F.La[1], La2 = F.La[2];
    const int nx = 2 * La0 + 1, ny = 2 * La1 + 1, nst = nx * ny * (2 * La2 + 1);
    const int cx = c % G.n[0], cy = (c / G.n[0]) % G.n[1], cz = c / (G.n[0] * G.n[1]);
    const int *cs = B.astart + (int64_t)f * B.as;  // solute molecule 0
    for (int i = t; i < nst; i += blockDim.x) {
        const int dx = i % nx - La0, dy = (i / nx) % ny - La1, dz = i / (nx * ny) - La2;
        const int cell = (wrap_cell(cz + dz, G.n[2]) * G.n[1] + wrap_cell(cy + dy, G.n[1])) * G.n[0] +
                         wrap_cell(cx + dx, G.n[0]);
        s_beg[i] = cs[cell];
        s_pre[i] = cs[cell + 1] - cs[cell];
        s_oi[i] = (short)off_index(dx, dy, dz);
    }
    __syncthreads();
    if (t < 32) {
        // exclusive scan of the stencil cells' atom counts
        int run = 0;
        for (int i0 = 0; i0 < nst; i0 += 32) {
            const int i = i0 + t;
            const int v = i < nst ? s_pre[i] : 0;
            int incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if (t >= o) incl += u;
            }
            if (i < nst) s_pre[i] = run + incl - v;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (t == 0) s_pre[nst] = run;
    }
    __syncthreads();
    const int N = s_pre[nst];
    const float4 *aq = B.asq32 + (int64_t)f * B.Ns;
    const float4 *off = B.off32 + (int64_t)f * kOffEntries;
    // stencil atom kk: its position from this cell's origin
    auto atom_at = [&](int kk) {
        int lo = 0, hi = nst - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_pre[mid] <= kk) lo = mid;
            else hi = mid - 1;
        }
        const float4 q = aq[s_beg[lo] + (kk - s_pre[lo])];
        const float4 o = off[s_oi[lo]];
        return make_float4(q.x + o.x, q.y + o.y, q.z + o.z, q.w);
    };
    // the frame's fine-cell geometry (k_frame_consts), shared
    __shared__ FineCells s_fc;
    if (t == 0) s_fc = F.fcells;
    __syncthreads();
    const FineCells fc = s_fc;
    auto centre = [&](int g, float *cen) {
        const float u0 = ((float)(g % K) + 0.5f), u1 = ((float)((g / K) % K) + 0.5f), u2 = ((float)(g / (K * K)) + 0.5f);
        for (int r = 0; r < 3; ++r) cen[r] = fmaf(fc.e[6 + r], u2, fmaf(fc.e[3 + r], u1, fc.e[r] * u0));
    };
    // a lower bound of the distance from p to this search cell: its box for
    // orthogonal cells, its bounding sphere otherwise
    float blo[3], bhi[3], cc[3];
    const float Rc = fc.R * (float)K;
    for (int r = 0; r < 3; ++r) {
        const float e = fc.e[4 * r] * (float)K;
        blo[r] = fminf(0.f, e);
        bhi[r] = fmaxf(0.f, e);
        cc[r] = 0.5f * (float)K * (fc.e[r] + fc.e[3 + r] + fc.e[6 + r]);
    }
    auto cell_near = [&](const float4 &p) {
        if (fc.ortho) {
            const float dx = fmaxf(fmaxf(blo[0] - p.x, p.x - bhi[0]), 0.f);
            const float dy = fmaxf(fmaxf(blo[1] - p.y, p.y - bhi[1]), 0.f);
            const float dz = fmaxf(fmaxf(blo[2] - p.z, p.z - bhi[2]), 0.f);
            return sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
        }
        const float dx = p.x - cc[0], dy = p.y - cc[1], dz = p.z - cc[2];
        return fmaxf(sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx))) - Rc, 0.f);
    };
    // the next stencil atoms within `thr` of this cell, from atom `cursor` on,
    // compacted into s_at in stencil order (kAgridRound atoms per thread and
    // two barriers per round); returns how many
    auto stage_kept = [&](int &cursor, float thr) {
        int n = 0;
        const int round = kAgridRound * (int)blockDim.x;
        while (cursor < N && n + round <= kAgridStage) {
            float4 p[kAgridRound];
            unsigned m[kAgridRound];
            int mine_n = 0;
#pragma unroll
            for (int j = 0; j < kAgridRound; ++j) {
                const int kk = cursor + j * (int)blockDim.x + t;
                bool keep = false;
                p[j] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (kk < N) {
                    p[j] = atom_at(kk);
                    keep = cell_near(p[j]) <= thr;
                }
                m[j] = __ballot_sync(0xffffffffu, keep);
                mine_n += __popc(m[j]);
            }
            if (lane == 0) s_wsum[warp] = mine_n;
            __syncthreads();
            int before = 0, total = 0;
            for (int w = 0; w < nwarps; ++w) {
                const int cw = s_wsum[w];
                before += w < warp ? cw : 0;
                total += cw;
            }
            int at = n + before;
#pragma unroll
            for (int j = 0; j < kAgridRound; ++j) {
                if ((m[j] >> lane) & 1u) s_at[at + __popc(m[j] & below)] = p[j];
                at += __popc(m[j]);
            }
            n += total;
            cursor += round;
            __syncthreads();
        }
        return n;
    };
    auto warp_min = [&](float v) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        return v;
    };
    const float cut = (float)S.cut;
    const float slack = 1e-3f * (1.0f + cut);
    const float margin = F.g.two_delta + slack;
    // the list threshold and bucket edges of fine cell g from its bounds
    auto thresh = [&](int g) { return fminf(fc.ortho ? sqrtf(s_far[g]) : sqrtf(s_far[g]) + fc.R, cut) + margin; };
    auto lowest = [&](int g) { return fc.ortho ? sqrtf(s_near[g]) : fmaxf(sqrtf(s_near[g]) - fc.R, 0.f); };
    if (t == 0) s_tmax = 0.f;
    int kept = -1;  // atoms of pass 1 still staged (-1 none yet, -2 several stages)
    {
        for (int g = t; g < K3; g += blockDim.x) {
            s_far[g] = INFINITY;
            s_near[g] = INFINITY;
        }
        // the search cell's own atoms first: each fine cell's bound from them
        // limits the stencil atoms that can matter to those within the
        // largest bound of the cell (dense solutes: a few Angstrom)
        const int own = (La2 * ny + La1) * nx + La0;
        const int own_beg = s_pre[own], own_n = s_pre[own + 1] - s_pre[own];
        for (int k0 = 0; k0 < own_n; k0 += kAgridStage) {
            const int nb = min(kAgridStage, own_n - k0);
            __syncthreads();
            for (int k = t; k < nb; k += blockDim.x) s_at[k] = atom_at(own_beg + k0 + k);
            __syncthreads();
            for (int g = warp; g < K3; g += nwarps) {
                float cen[3];
                centre(g, cen);
                float far = INFINITY;
                for (int k = lane; k < nb; k += 32) far = fminf(far, fine_far2(fc, cen, s_at[k]));
                far = warp_min(far);
                if (lane == 0) s_far[g] = fminf(s_far[g], far);
            }
        }
        __syncthreads();
        for (int g = t; g < K3; g += blockDim.x) atomicMax((int *)&s_tmax, __float_as_int(thresh(g)));
        __syncthreads();
        const float thr1 = s_tmax + slack;
        // pass 1: an upper bound of the nearest atom's distance over each fine
        // cell, and the smallest distance of any atom to it
        int cursor = 0;
        while (cursor < N) {
            const int nb = stage_kept(cursor, thr1);
            kept = kept == -1 && cursor >= N ? nb : -2;  // one stage held every atom that passed
            for (int g = warp; g < K3; g += nwarps) {
                float cen[3];
                centre(g, cen);
                float far = INFINITY, near = INFINITY;
                for (int k = lane; k < nb; k += 32) {
                    const float4 p = s_at[k];
                    far = fminf(far, fine_far2(fc, cen, p));
                    near = fminf(near, fine_near2(fc, cen, p));
                }
                far = warp_min(far);
                near = warp_min(near);
                if (lane == 0) {
                    s_far[g] = fminf(s_far[g], far);
                    s_near[g] = fminf(s_near[g], near);
                }
            }
            __syncthreads();
        }
        for (int g = t; g < K3; g += blockDim.x) B.gedge[ebase + g] = make_float2(lowest(g), thresh(g));
        __syncthreads();
        if (t == 0) s_tmax = 0.f;
        __syncthreads();
    }
    // pass 2: the atoms whose smallest distance to the fine cell is within T,
    // by bucket of that distance: counted, then written
    auto LT = [&](int g, float &L, float &T) {
        L = lowest(g);
        T = thresh(g);
    };
    for (int g = t; g < K3; g += blockDim.x) {
        float L, T;
        LT(g, L, T);
        atomicMax((int *)&s_tmax, __float_as_int(T));
#pragma unroll
        for (int b = 0; b < kAgridBuckets; ++b) s_pos[g][b] = 0;
    }
    __syncthreads();
    const float thr2 = s_tmax + slack;
    float4 *ent = B.gent + (int64_t)f * B.gcap;
    // one stage of atoms through every fine cell: lane k of a group of 32
    // tests atom k; counting sums the buckets, filling writes each bucket's
    // atoms in stage order after its start
    auto pass2 = [&](int nb, bool fill) {
        for (int g = warp; g < K3; g += nwarps) {
            float cen[3];
            centre(g, cen);
            float L, T;
            LT(g, L, T);
            const float lim2 = fc.ortho ? T * T : (T + fc.R) * (T + fc.R);
            const float inv = T > L ? (float)kAgridBuckets / (T - L) : 0.f;
            for (int k0 = 0; k0 < nb; k0 += 32) {
                const int k = k0 + lane;
                int bk = -1;
                float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k < nb) {
                    p = s_at[k];
                    const float d2 = fine_near2(fc, cen, p);
                    if (d2 <= lim2) {
                        const float dmin = fc.ortho ? sqrtf(d2) : fmaxf(sqrtf(d2) - fc.R, 0.f);
                        bk = min(kAgridBuckets - 1, max(0, (int)((dmin - L) * inv)));
                    }
                }
                if (!__any_sync(0xffffffffu, bk >= 0)) continue;
                // the lanes of each bucket: the lowest one advances the
                // bucket's position, the others write after it in lane order
                const unsigned m = __match_any_sync(0xffffffffu, bk);
                const int leader = __ffs(m) - 1;
                int at = 0;
                if (bk >= 0 && lane == leader) {
                    at = s_pos[g][bk];
                    s_pos[g][bk] = at + __popc(m);
                }
                at = __shfl_sync(0xffffffffu, at, leader);
                if (fill && bk >= 0) ent[at + __popc(m & below)] = p;
                __syncwarp();
            }
        }
    };
    // pass 1's single stage holds every atom that passes thr2 (thr2 <= thr1),
    // and the others fail the bucket test: counting and filling reuse it
    auto sweep = [&](bool fill) {
        int cursor = 0;
        if (kept >= 0) {
            pass2(kept, fill);
            cursor = N;
        }
        while (cursor < N) {
            const int nb = stage_kept(cursor, thr2);
            pass2(nb, fill);
            __syncthreads();
        }
        __syncthreads();
    };
    sweep(false);
    // the CTA's lists: offsets by (fine cell, bucket), one reservation in the
    // frame's pool, the starts and each fine cell's end
    int tot = 0;
    if (t < K3) {
#pragma unroll
        for (int b = 0; b < kAgridBuckets; ++b) {
            const int n = s_pos[t][b];
            s_pos[t][b] = tot;
            tot += n;
        }
    }
    int incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    int wbefore = 0, all = 0;
    for (int w = 0; w < nwarps; ++w) {
        wbefore += w < warp ? s_wsum[w] : 0;
        all += s_wsum[w];
    }
    if (t == 0) {
        const int base = atomicAdd(B.gpool + f, all);
        if ((int64_t)base + all > B.gcap) {
            B.FS[f].agrid = 0;  // this frame's queries take the walk
            atomicAdd(S.stats + ST_AGRID_OVF, 1ull);
            atomicMax(S.stats + ST_AGRID_NEED, (unsigned long long)((int64_t)base + all));
            s_base = -1;
        } else {
            s_base = base;
        }
    }
    __syncthreads();
    if (s_base < 0) return;
    if (t < K3) {
        const int start = s_base + wbefore + incl - tot;
        int *st = B.gstart + gbase + (int64_t)t * (kAgridBuckets + 1);
#pragma unroll
        for (int b = 0; b < kAgridBuckets; ++b) {
            s_pos[t][b] += start;
            st[b] = s_pos[t][b];
        }
        st[kAgridBuckets] = start + tot;
    }
    __syncthreads();
    sweep(true);
}

__global__ void __launch_bounds__(kAgridBuildThreads) k_agrid_build(DevSys S, Bufs B) {
    k_agrid_build_body(blockIdx, gridDim, S, B);
}

// A site's fine cell (FP32 position q in search cell (cx, cy, cz)): its list's
// bucket starts and the smallest distance and width of its buckets.
struct AgridCell {
    const int *st;  // kAgridBuckets + 1 starts in the frame's entries
    float lo, w;
};

__device__ __forceinline__ AgridCell agrid_cell(const Bufs &B, const FrameGeom &G, const FrameScratch &F, int f, int packed,
                                                float4 q) {
    const int K = B.agk;
    const int cx = packed & 1023, cy = (packed >> 10) & 1023, cz = packed >> 20;
    int gi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float u = fmaf(F.hin[3 * k + 2], q.z, fmaf(F.hin[3 * k + 1], q.y, F.hin[3 * k] * q.x));
        gi[k] = min(max((int)floorf(u * (float)K), 0), K - 1);
    }
    const int64_t fine = (int64_t)((cz * G.n[1] + cy) * G.n[0] + cx) * (K * K * K) + (gi[2] * K + gi[1]) * K + gi[0];
    const float2 edge = B.gedge[(int64_t)f * B.gfs + fine];
    AgridCell c;
    c.st = B.gstart + ((int64_t)f * B.gfs + fine) * (kAgridBuckets + 1);
    c.lo = edge.x;
    c.w = (edge.y - edge.x) * (1.0f / (float)kAgridBuckets);
    return c;
}

// One site's query: the top-2 update over its fine cell's list (p1 holds the
// solute atom index in the molecule), bucket by bucket of the entries'
// smallest distance to the fine cell.  A bucket whose smallest distance
// exceeds the running minimum (for the reference site, also its own minimum)
// by more than `band` holds no atom that can be the minimum, be within the
// guard band of it or lower the reference row, and neither do the buckets
// after it.
__device__ __forceinline__ void agrid_query(const Bufs &B, const FrameGeom &G, const FrameScratch &F, int f, int packed,
                                            float4 q, int b, bool isref, float band, Top2 &T, long long &evals) {
    const AgridCell c = agrid_cell(B, G, F, f, packed, q);
    const float4 *e = B.gent + (int64_t)f * B.gcap;
    int i = c.st[0];
#pragma unroll 1
    for (int k = 0; k < kAgridBuckets; ++k) {
        const float thr = fmaxf(sqrtf(T.m1), isref ? sqrtf(T.r1) : 0.f) + band;
        if (fmaf(c.w, (float)k, c.lo) > thr) break;
        const int end = c.st[k + 1];
        evals += end - i;
        for (; i < end; ++i) {
            const float4 a = e[i];
            const float ex = a.x - q.x, ey = a.y - q.y, ez = a.z - q.z;
            const float d2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
            T.m2 = fminf(T.m2, fmaxf(T.m1, d2));
            const bool lt = d2 < T.m1;
            T.p1 = lt ? __float_as_int(a.w) : T.p1;
            T.b1 = lt ? b : T.b1;
            T.m1 = fminf(T.m1, d2);
            if (isref) T.r1 = fminf(T.r1, d2);
        }
    }
}

// Exact scan of a slot's or molecule's sites over their lists: every list
// entry whose FP32 squared distance is within thr_arg (or, for the reference
// site, thr_r1) is evaluated exactly (exact_d2 on the input coordinates) and
// kept by the reference's tie rule -- the pairs of atoms_exact's stencil walk
// for the same thresholds.  The thresholds come from the query's minima plus
// 2 delta, so each such atom lies within (nearest distance + 3 delta) of its
// site, which the list's margin covers, and the buckets past sqrt(thr) + band
// hold none of them.
__device__ __noinline__ void agrid_exact(const DevSys &S, const Bufs &B, const FrameGeom &G, const FrameScratch &F, int f,
                                         ExactMol &X, const int *vc, const float4 *vq, float band, float thr_arg,
                                         float thr_r1, Best64 &Bst, double &rr1, long long &evals) {
    best_init(Bst);
    rr1 = INFINITY;
    evals = 0;
    const float4 *e = B.gent + (int64_t)f * B.gcap;
    for (int b = 0; b < S.apv; ++b) {
        const bool isref = b == S.iref;
        const float thr = isref ? fmaxf(thr_arg, thr_r1) : thr_arg;
        if (!(thr >= 0.f)) continue;
        const float4 q = vq[b];
        const AgridCell c = agrid_cell(B, G, F, f, vc[b], q);
        const float lim = sqrtf(thr) + band;
        double yb[3];
        bool have_y = false;
        int i = c.st[0];
        for (int k = 0; k < kAgridBuckets; ++k) {
            if (fmaf(c.w, (float)k, c.lo) > lim) break;
            const int end = c.st[k + 1];
            for (; i < end; ++i) {
                const float4 a = e[i];
                const float ex = a.x - q.x, ey = a.y - q.y, ez = a.z - q.z;
                const float d2f = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                if (!(d2f <= thr_arg || (isref && d2f <= thr_r1))) continue;
                if (!have_y) {
                    exact_solvent_atom(B, G, X, b, yb);
                    have_y = true;
                }
                const int ai = __float_as_int(a.w);
                double xa[3];
                exact_solute_atom(B, X, ai, xa);
                const double d2 = exact_d2(G, xa, yb);
                evals++;
                if (d2 <= S.cut2) {
                    if (isref) rr1 = fmin(rr1, d2);
                    best_update<false>(Bst, d2, ai, b);
                }
            }
        }
    }
}

// The record of a query's top-2 when every value is farther than the band
// from its decision boundary (the unambiguous branch of atoms_decide):
// 0 = no record within the cutoff, 1 = record r, 2 = inside the band (the
// record is then agrid_record's).
__device__ __forceinline__ int agrid_decide(const DevSys &S, const Guard &g, const Top2 &T, int64_t vb, DirRec &r) {
    r = dir_none(S);
    if (!(T.m1 <= g.cutp2)) return 0;
    const float d1 = sqrtf(T.m1);
    if (T.m1 >= g.cutm2 || (sqrtf(T.m2) - d1) <= g.two_delta) return 2;
    const int bin = bin_of(g, d1);
    if (bin < 0 || (S.usecutoff && d1 >= g.dbulk_lo && d1 <= g.dbulk_hi)) return 2;
    r.within = 1;
    r.i_local = T.p1;
    r.j = vb + T.b1;
    r.bin = bin;
    r.bulk = S.usecutoff ? (d1 > g.dbulk_hi) : 0;
    if (T.r1 <= g.cutp2) {
        const int rb = T.r1 < g.cutm2 ? bin_of(g, sqrtf(T.r1)) : -1;
        if (rb < 0) return 2;
        r.ref = 1;
        r.rbin = rb;
    }
    return 1;
}

// The record of a query inside the band (agrid_decide's 2), decided by
// atoms_decide's rules with the exact scans over the sites' lists (agrid_exact)
// instead of the stencil walk: v the solvent molecule (sample < 0) or the
// slot of sample `sample`, whose placement is drawn again in FP64.
__device__ __noinline__ DirRec agrid_record(const DevSys &S, const Bufs &B, const FrameGeom &G, const FrameScratch &F,
                                            int f, int v, int sample, const int *vc, const float4 *vq, const Top2 &T,
                                            LocalStats &st) {
    const Guard &g = F.g;
    const float band = g.two_delta + 1e-3f * (1.0f + (float)S.cut);
    const int64_t vb = (int64_t)v * S.apv;
    ExactMol X;
    if (sample < 0) {
        X = exact_mol(S, f, 0, v);
    } else {
        const Sample sm = B.samples[sample];
        const Placement P = draw_placement(S, G.frame_id, sm, v, B.bulk + (int64_t)f * B.ndist * B.mv,
                                           B.nbulk + (int64_t)f * B.ndist);
        uint64_t rs = P.st;
        double R[9];
        draw_rotation(rs, R);
        X = exact_mol_placed(S, G, f, sm.s, P.jmol, P.fc, R);
    }
    DirRec r = dir_none(S);
    if (!(T.m1 <= g.cutp2)) return r;
    const float d1 = sqrtf(T.m1);
    if (T.m1 >= g.cutm2 || (sqrtf(T.m2) - d1) <= g.two_delta) {
        const float thr1 = T.r1 <= g.cutp2 ? r_sq_ru(sqrtf(T.r1) + g.two_delta) : -1.f;
        Best64 Bst;
        double rr1;
        long long ev;
        agrid_exact(S, B, G, F, f, X, vc, vq, band, r_sq_ru(d1 + g.two_delta), thr1, Bst, rr1, ev);
        st.guard++;
        st.guard_pairs += ev;
        if (Bst.d2 <= S.cut2) {
            const double d = best_d(Bst);
            st.maxerr = fmax(st.maxerr, fabs((double)d1 - d));
            r.within = 1;
            r.i_local = Bst.a;
            r.j = vb + Bst.b;
            r.bin = setbin0(d, S.binstep);
            r.bulk = inbulk64(S, true, d);
            if (rr1 <= S.cut2) {
                r.ref = 1;
                r.rbin = setbin0(sqrt(rr1), S.binstep);
            }
        }
        return r;
    }
    // the search's minimum pair is the exact minimum pair
    int bin = bin_of(g, d1);
    double d64 = -1.0;
    if (bin < 0 || (S.usecutoff && d1 >= g.dbulk_lo && d1 <= g.dbulk_hi)) {
        d64 = sqrt(exact_pair_d2(B, G, X, T.p1, T.b1));
        bin = setbin0(d64, S.binstep);
        st.guard++;
        st.guard_pairs++;
        st.maxerr = fmax(st.maxerr, fabs((double)d1 - d64));
    }
    r.within = 1;
    r.i_local = T.p1;
    r.j = vb + T.b1;
    r.bin = bin;
    r.bulk = S.usecutoff ? (d64 >= 0.0 ? (d64 > S.dbulk) : (d1 > g.dbulk_hi)) : 0;
    if (T.r1 <= g.cutp2) {
        const int rb = T.r1 < g.cutm2 ? bin_of(g, sqrtf(T.r1)) : -1;
        if (rb >= 0) {
            r.ref = 1;
            r.rbin = rb;
        } else {
            Best64 Bst;
            double rr1;
            long long ev;
            agrid_exact(S, B, G, F, f, X, vc, vq, band, -1.f, r_sq_ru(sqrtf(T.r1) + g.two_delta), Bst, rr1, ev);
            st.guard++;
            st.guard_pairs += ev;
            if (rr1 <= S.cut2) {
                r.ref = 1;
                r.rbin = setbin0(sqrt(rr1), S.binstep);
            }
        }
    }
    return r;
}

// Real pass of a single solute molecule, one thread per (frame, solvent
// molecule), persistent grid; frames without a grid queue their near pairs
// for k_atoms_eval (k_atoms_filter's rule).
__device__ __forceinline__ void k_agrid_real_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    const SHist h = shist_bind(S, hbase);
    LocalStats st;
    const int apv = S.apv, iref = S.iref;
    const int64_t n = (int64_t)B.nf * S.mv;
    auto one_molecule = [&](int64_t it) {
        const int f = (int)(it / S.mv), v = (int)(it - (int64_t)f * S.mv);
        const FrameScratch &F = B.FS[f];
        const FrameGeom &G = B.G[f];
        const int *vc = B.avcell + (int64_t)f * B.Nv + (int64_t)v * apv;
        if (!F.agrid) {
            if (!F.ok) {
                raise_err(S, ERR_STENCIL);
                return;
            }
            if (atoms_near(B, G, f, 0, vc, apv)) atoms_push(S, B, make_int4(v, 0, f, 0));
            return;
        }
        const float4 *vq = B.avq32 + (int64_t)f * B.Nv + (int64_t)v * apv;
        Top2 T;
        top2_init(T);
        long long ev = 0;
        const float band = F.g.two_delta + 1e-3f * (1.0f + (float)S.cut);
        for (int b = 0; b < apv; ++b) agrid_query(B, G, F, f, vc[b], vq[b], b, b == iref, band, T, ev);
        if (ev == 0) return;
        st.atompairs += (unsigned long long)ev;
        DirRec r;
        if (agrid_decide(S, F.g, T, (int64_t)v * apv, r) == 2) r = agrid_record(S, B, G, F, f, v, -1, vc, vq, T, st);
        st.molpairs++;
        if (r.within) {
            apply_hit(S, h, false, r.bin, r.i_local, r.j, r.ref, r.rbin);
            st.hits++;
            if (B.slot) {
                const int sl = B.slot[(int64_t)f * B.ms];
                if (sl >= 0) B.flags[((int64_t)f * B.ndist + sl) * S.mv + v] = flag_code(r);
            }
        }
    };
    // warps take 32 molecules at a time from counters[6] (zeroed with the
    // chunk's counters), as k_agrid_random takes its slots
    const int lane = threadIdx.x & 31;
    for (;;) {
        long long at = 0;
        if (lane == 0) at = (long long)atomicAdd((unsigned long long *)(B.counters + 6), 32ull);
        at = __shfl_sync(0xffffffffu, at, 0);
        if (at >= n) break;
        if (at + lane < n) one_molecule(at + lane);
        __syncwarp();
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// four resident CTAs per SM: the queries wait on their list entries (agrid_record is out of line)
__global__ void __launch_bounds__(256, 4) k_agrid_real(DevSys S, Bufs B) {
    k_agrid_real_body(blockIdx, gridDim, S, B);
}

// Random insertion of a single solute molecule, third pass: one thread per
// slot of the list k_slot_filter made, after k_atoms_place has placed them
// into the placement buffers; persistent grid.  In a frame with a grid the
// slot's sites are queried and the record is decided at once (agrid_record
// inside the band); k_atoms_place has queued the near slots of the other
// frames for k_atoms_eval.
__device__ __forceinline__ void k_agrid_random_body(const uint3 blockIdx, const dim3 gridDim, const DevSys &S, const Bufs &B, int sample0, int ny) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    const SHist h = shist_bind(S, hbase);
    LocalStats st;
    const int apv = S.apv, iref = S.iref;
    (void)ny;
    const int n = min(B.counters[5], B.aslot_cap);
    auto one_slot = [&](int it) {
        const int e = B.aslot[it];
        const int y = e / S.mv, k = e - y * S.mv;
        const int f = B.samples[sample0 + y].pad;
        const FrameScratch &F = B.FS[f];
        if (!F.agrid) return;
        const FrameGeom &G = B.G[f];
        const int64_t base = (int64_t)y * B.Nv + (int64_t)k * apv;
        Top2 T;
        top2_init(T);
        long long ev = 0;
        const float band = F.g.two_delta + 1e-3f * (1.0f + (float)S.cut);
        for (int b = 0; b < apv; ++b)
            agrid_query(B, G, F, f, B.pcell[base + b], B.pq32[base + b], b, b == iref, band, T, ev);
        if (ev == 0) return;
        st.atompairs += (unsigned long long)ev;
        DirRec r;
        if (agrid_decide(S, F.g, T, (int64_t)k * apv, r) == 2)
            r = agrid_record(S, B, G, F, f, k, sample0 + y, B.pcell + base, B.pq32 + base, T, st);
        st.molpairs++;
        if (r.within) {
            apply_hit(S, h, true, r.bin, r.i_local, r.j, r.ref, r.rbin);
            st.hits++;
        }
    };
    // warps take 32 listed slots at a time from counters[6] (zeroed with the
    // slot list): the slots' costs vary with their lists, and a fixed share per
    // thread left the CTAs' warps waiting for their slowest one
    const int lane = threadIdx.x & 31;
    for (;;) {
        int at = 0;
        if (lane == 0) at = atomicAdd(B.counters + 6, 32);
        at = __shfl_sync(0xffffffffu, at, 0);
        if (at >= n) break;
        if (at + lane < n) one_slot(at + lane);
        __syncwarp();
    }
    stats_flush(S, st, true);
    __syncthreads();
    shist_flush(S, h, true);
}

__global__ void __launch_bounds__(256, 4) k_agrid_random(DevSys S, Bufs B, int sample0, int ny) {
    k_agrid_random_body(blockIdx, gridDim, S, B, sample0, ny);
}

}  // namespace cmk
