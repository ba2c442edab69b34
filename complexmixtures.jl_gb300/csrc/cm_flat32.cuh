// cm_flat32.cuh -- FP32 real pass of the PAIRS layout with one lane per
// solvent atom.
//
// One warp per (frame, solute molecule) work item.  The warp walks the cell
// stencil row by row; in self mode only the forward half (the own cell with
// v > s, then the cells whose offset is positive in (z, y, x) order), so every
// unordered molecule pair is met once.  The cells of a stencil row are
// consecutive in the cell-sorted molecule table, so a row is one or two
// contiguous ranges of it; a lane finds the x offset of its molecule's cell by
// comparing its position with the row's cell starts.  A solvent molecule is a
// candidate if its bounding sphere reaches the solute's.
//
// Each batch of up to 32 candidates is expanded into its atoms; an atom
// farther than cutoff + solute radius from the solute centroid cannot hold a
// pair within the cutoff and is dropped.  The remaining atoms are evaluated 32
// at a time, one per lane, against the solute atoms in shared memory, and the
// lanes fold their results into per-candidate slots with shared-memory atomics:
//   k1  (d^2 bits << 32 | a << 8 | b): the closest pair and its atoms,
//   m2  the second-smallest d^2 over all pairs (top-2 by displacement:
//       old = atomicMin(k1, key); atomicMin(m2, max(old, d^2)), together with
//       each lane's own second-smallest),
//   r1  d^2 of the solvent molecule's reference atom to the closest solute atom,
//   r2  (self) d^2 of the solute molecule's reference atom to the closest atom
//       of the solvent molecule.
// Lane c then decides candidate c: records inside the guard band of the
// cutoff, of a bin edge or of dbulk, or with a second-closest pair within
// 2 delta of the closest, go to the guard queue for the exact FP64 rules.
#pragma once
#include "cm_kernels.cuh"

namespace cmk {

// One CTA of 32 warps per SM at 64 registers: the SM's 32 warps share one
// privatised histogram (measured 3.8% faster on config 3 than 2 CTAs of 16
// warps, each zeroing and flushing its own histogram).
#ifndef CM_FLAT_WARPS
#define CM_FLAT_WARPS 32
#endif
#ifndef CM_FLAT_MIN_CTAS
#define CM_FLAT_MIN_CTAS 1
#endif
constexpr int kFlatWarps = CM_FLAT_WARPS;  // warps per CTA
constexpr int kAtomQueue = 64;   // per-warp atom queue (float4: t, tag)

// The 32 candidates' fold slots, one array per field: the lanes of a flush
// hold different candidates, and their atomics then fall on distinct banks.
struct CandSlots {
    unsigned long long k1[32];
    unsigned int m2[32], r1[32], r2[32];
};

constexpr unsigned long long kNoPair = (0x7f800000ull << 32) | 0xffffffffull;  // +inf, largest index

// Shared memory of one warp after the histograms.
struct FlatWarpSmem {
    float4 os[kMaxSmallMol];      // solute atom offsets (x, y, z)
    float4 aq[kAtomQueue];        // atom queue: t = position relative to the solute centroid, w = tag c << 8 | b
    float4 cq[kQueue];            // candidate queue: D = centroid displacement, w = molecule index
    int cc[kQueue];               // candidate queue: packed cell offset
    CandSlots cand;
};

__host__ __device__ constexpr size_t flat_warp_smem() { return sizeof(FlatWarpSmem); }

// Top-2 of the squared distances of one solvent atom t to solute atoms
// [a0, a1) with step 2 (two independent chains per lane).
__device__ __forceinline__ void top2_step(const float4 &e, const float4 &oa, int a, float &m1, float &m2, int &k1) {
    const float dx = e.x - oa.x, dy = e.y - oa.y, dz = e.z - oa.z;
    const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    m2 = fminf(m2, fmaxf(m1, d2));
    k1 = d2 < m1 ? a : k1;
    m1 = fminf(m1, d2);
}

// Evaluate the first n queued atoms (one per lane) and fold them into the
// candidate slots.  APS > 0 is the compile-time solute molecule size.
template <bool SELF, int APS>
__device__ __forceinline__ void flat_flush(const DevSys &S, FlatWarpSmem &W, int n, int lane, LocalStats &st) {
    if (lane < n) {
        const float4 e = W.aq[lane];
        const int tag = __float_as_int(e.w);
        const int c = tag >> 8, b = tag & 0xff;
        float m1a = INFINITY, m2a = INFINITY, m1b = INFINITY, m2b = INFINITY;
        int k1a = 0, k1b = 0;
        const int aps = APS > 0 ? APS : S.aps;
        if (APS > 0) {
            // fully unrolled for small molecules; two pairs of steps per
            // iteration otherwise, so the solute atoms are not all held live
#pragma unroll(APS <= 6 ? 3 : 2)
            for (int a = 0; a + 1 < APS; a += 2) {
                top2_step(e, W.os[a], a, m1a, m2a, k1a);
                top2_step(e, W.os[a + 1], a + 1, m1b, m2b, k1b);
            }
            if (APS & 1) top2_step(e, W.os[APS - 1], APS - 1, m1a, m2a, k1a);
        } else {
            int a = 0;
#pragma unroll 1
            for (; a + 1 < aps; a += 2) {
                top2_step(e, W.os[a], a, m1a, m2a, k1a);
                top2_step(e, W.os[a + 1], a + 1, m1b, m2b, k1b);
            }
            if (a < aps) top2_step(e, W.os[a], a, m1a, m2a, k1a);
        }
        // merge the two chains (equal minima leave m2 == m1, which the guard catches)
        const float m1 = fminf(m1a, m1b);
        const float m2 = fminf(fmaxf(m1a, m1b), fminf(m2a, m2b));
        const int k1 = m1b < m1a ? k1b : k1a;
        st.atompairs += (unsigned long long)aps;
        CandSlots &C = W.cand;
        const unsigned long long key = ((unsigned long long)__float_as_uint(m1) << 32) | (unsigned)(k1 << 8 | b);
        const unsigned long long old = atomicMin(&C.k1[c], key);
        const float displaced = fmaxf(m1, __uint_as_float((unsigned)(old >> 32)));
        atomicMin(&C.m2[c], __float_as_uint(fminf(displaced, m2)));
        if (b == S.iref) C.r1[c] = __float_as_uint(m1);
        if (SELF) {
            const float4 oi = W.os[S.iref];
            const float dx = e.x - oi.x, dy = e.y - oi.y, dz = e.z - oi.z;
            atomicMin(&C.r2[c], __float_as_uint(fmaf(dz, dz, fmaf(dy, dy, dx * dx))));
        }
    }
    __syncwarp();
}

// One batch: the first nc (<= 32) entries of the warp's candidate queue.
// Expansion runs one lane per (candidate, atom) in atom-major order, so the
// lanes of one flush hold atoms of different candidates and their
// shared-memory atomics rarely meet on one slot; then lane c decides
// candidate c.
template <bool SELF, int APS>
__device__ __forceinline__ void flat_batch(const DevSys &S, const Bufs &B, const SHist &h, FlatWarpSmem &W,
                                           const PairsFrame &Pf, const Guard &g, int f, int s, int sslot, float rs2,
                                           int lane, int nc, LocalStats &st) {
    if (lane < nc) {
        CandSlots &C = W.cand;
        C.k1[lane] = kNoPair;
        C.m2[lane] = 0x7f800000u;
        C.r1[lane] = 0x7f800000u;
        C.r2[lane] = 0x7f800000u;
    }
    __syncwarp();
    const int apv = S.apv;
    const float inv_nc = 1.0f / (float)nc;
    const int total = nc * apv;
    int nq = 0;
    for (int base = 0; base < total; base += 64) {
        // two rounds of 32 (candidate, atom) entries; their loads are independent
        bool keep[2];
        float4 t[2];
        int tag[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int i = base + 32 * r + lane;
            const bool in = i < total;
            // b = i / nc, exact for i < 2^16: (i + 0.5) / nc stays within half of 1/nc of the quotient
            const int b = in ? (int)((float(i) + 0.5f) * inv_nc) : 0;
            const int c = in ? i - b * nc : 0;
            const float4 D = W.cq[c];
            float4 ob = make_float4(0.f, 0.f, 0.f, 0.f);
            if (in) ob = Pf.vo32[(int64_t)__float_as_int(D.w) * apv + b];
            t[r] = make_float4(D.x + ob.x, D.y + ob.y, D.z + ob.z, 0.f);
            keep[r] = in && fmaf(t[r].z, t[r].z, fmaf(t[r].y, t[r].y, t[r].x * t[r].x)) <= rs2;
            tag[r] = c << 8 | b;
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const unsigned mask = __ballot_sync(0xffffffffu, keep[r]);
            if (keep[r]) W.aq[nq + __popc(mask & ((1u << lane) - 1u))] = make_float4(t[r].x, t[r].y, t[r].z, __int_as_float(tag[r]));
            nq += __popc(mask);
            if (nq >= 32) {
                __syncwarp();
                flat_flush<SELF, APS>(S, W, 32, lane, st);
                float4 rest = make_float4(0.f, 0.f, 0.f, 0.f);
                if (lane < nq - 32) rest = W.aq[32 + lane];
                __syncwarp();
                if (lane < nq - 32) W.aq[lane] = rest;
                nq -= 32;
                __syncwarp();
            }
        }
    }
    __syncwarp();
    if (nq > 0) flat_flush<SELF, APS>(S, W, nq, lane, st);
    if (lane >= nc) return;
    st.molpairs++;
    const CandSlots &C = W.cand;
    const unsigned long long k1 = C.k1[lane];
    if (k1 == kNoPair) return;
    const float m1 = __uint_as_float((unsigned)(k1 >> 32));
    if (m1 > g.cutp2) return;  // no atom pair within the cutoff
    const int v = __float_as_int(W.cq[lane].w), code = W.cc[lane];
    const int a1 = (int)((unsigned)k1 >> 8) & 0xff, b1 = (int)(k1 & 0xff);
    const float m2 = __uint_as_float(C.m2[lane]), r1 = __uint_as_float(C.r1[lane]), r2 = __uint_as_float(C.r2[lane]);
    const float dmin = sqrtf(m1);
    // hard: the closest pair, or the cutoff or dbulk decision, needs the full
    // FP64 rules (guard queue)
    bool hard = m1 >= g.cutm2 || (sqrtf(m2) - dmin) <= g.two_delta;
    if (S.usecutoff) hard = hard || (dmin >= g.dbulk_lo && dmin <= g.dbulk_hi);
    if (hard) {
        // past the capacity the record is dropped and k_queue_check has the
        // chunk redone without queues
        const int slot = atomicAdd(B.counters + 0, 1);
        if (slot < B.gq_cap) B.gq[slot] = make_int4(s, v, code, f);
        return;
    }
    // otherwise each of the md bin, the solvent reference-atom row and (self)
    // the solute reference-atom column is decided here, or marked -2 when it
    // lies within the guard band of a bin edge or of the cutoff: the edge
    // kernel then computes it from FP64 pair distances
    int bin = bin32(g, dmin);
    if (bin < 0) bin = -2;
    int rb1 = -1, rb2 = -1;
    if (r1 <= g.cutp2) {
        rb1 = r1 < g.cutm2 ? bin32(g, sqrtf(r1)) : -1;
        if (rb1 < 0) rb1 = -2;
    }
    if (SELF && r2 <= g.cutp2) {
        rb2 = r2 < g.cutm2 ? bin32(g, sqrtf(r2)) : -1;
        if (rb2 < 0) rb2 = -2;
    }
    if (bin == -2 || rb1 == -2 || rb2 == -2) {
        const int slot = atomicAdd(B.counters + 3, 1);
        if (slot < B.eq_cap) {
            B.eq[3 * slot] = make_int4(s, v, code, f);
            B.eq[3 * slot + 1] = make_int4(a1 | b1 << 8, rb1, rb2, bin);
            B.eq[3 * slot + 2] = make_int4(__float_as_int(dmin), 0, 0, 0);
        }
        return;
    }
    const int bulk = S.usecutoff ? (dmin > g.dbulk_hi) : 0;
    if (SELF) {
        apply_pair_self(S, h, bin, a1, (int64_t)s * S.aps + a1, b1, (int64_t)v * apv + b1, rb1 >= 0, rb1, rb2 >= 0, rb2);
        st.hits += 2;
    } else {
        apply_hit_local(S, h, false, bin, a1, (int64_t)v * apv + b1, b1, rb1 >= 0, rb1);
        st.hits++;
    }
    if (Pf.slot) {
        const unsigned char code1 = (unsigned char)(1 + bulk);
        if (sslot >= 0) Pf.flags[(int64_t)sslot * S.mv + v] = code1;
        if (SELF) {
            const int vs = Pf.slot[v];
            if (vs >= 0) Pf.flags[(int64_t)vs * S.mv + s] = code1;
        }
    }
}

// skip_tile: the frames the tiled kernel took (FrameScratch::tile) are
// skipped, and the kernel returns at once when that is every frame.
template <bool SELF, int APS>
__global__ void __launch_bounds__(kFlatWarps * 32, CM_FLAT_MIN_CTAS) k_pairs_flat32(DevSys S, Bufs B, int skip_tile) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    const int hw = hist_words(S);
    FlatWarpSmem *wsm = (FlatWarpSmem *)(smem_raw + (((size_t)hw * 4 + 15) & ~(size_t)15));
    if (skip_tile) {
        int any = 0;
        for (int f = threadIdx.x; f < B.nf; f += blockDim.x) any |= (B.FS[f].tile == 0);
        if (!__syncthreads_or(any)) return;
    }
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    FlatWarpSmem &W = wsm[warp];
    LocalStats st;
    const int aps = S.aps;
    const int64_t items = (int64_t)B.nf * B.ms;
    for (int64_t t = (int64_t)blockIdx.x * kFlatWarps + warp; t < items; t += (int64_t)gridDim.x * kFlatWarps) {
        const int f = (int)(t / B.ms), s = (int)(t - (int64_t)f * B.ms);
        const PairsFrame Pf = pairs_frame(B, f, SELF);
        const FrameScratch &F = *Pf.F;
        if (!F.ok) {
            if (lane == 0) raise_err(S, ERR_STENCIL);
            continue;
        }
        if (F.multi) continue;  // several images per pair: the generic kernel takes the frame
        if (skip_tile && F.tile) continue;
        const FrameGeom &G = *Pf.G;
        const Guard g = F.g;
        const float4 qs = Pf.sq32[s];
        const int sc = Pf.scell[s];
        const int sslot = Pf.slot ? Pf.slot[s] : -1;
        __syncwarp();
        for (int a = lane; a < aps; a += 32) W.os[a] = Pf.so32[(int64_t)s * aps + a];
        __syncwarp();
        const float rsc = g.cut_pre + qs.w;     // candidate molecules: centroid within rsc + r_v
        const float rs2 = rsc * rsc;            // candidate atoms: within rsc of the solute centroid
        const float4 *cq32 = B.cq32 + (int64_t)f * B.mv;
        const int *cmol = Pf.cmol;
        const int *cstart = Pf.cstart;
        const int n0 = G.n[0], n1 = G.n[1], n2 = G.n[2];
        const int cx = sc % n0, cyz = sc / n0, cy = cyz % n1, cz = cyz / n1;
        const int L0 = F.L[0], L1 = F.L[1], L2 = F.L[2];
        int cnt = 0;
        for (int dz = SELF ? 0 : -L2; dz <= L2; ++dz) {
            int zc = cz + dz;
            zc = zc < 0 ? zc + n2 : (zc >= n2 ? zc - n2 : zc);
            for (int dy = (SELF && dz == 0) ? 0 : -L1; dy <= L1; ++dy) {
                int yc = cy + dy;
                yc = yc < 0 ? yc + n1 : (yc >= n1 ? yc - n1 : yc);
                const int row = (zc * n1 + yc) * n0;
                const bool own_row = SELF && dz == 0 && dy == 0;
                // the row's stencil offsets, lane j holding dx = j - L0
                float4 rowoff = make_float4(0.f, 0.f, 0.f, 0.f);
                if (lane <= 2 * L0) rowoff = Pf.off32[off_index(lane - L0, dy, dz)];
                // unwrapped x range of the row, split at the box edges into
                // contiguous pieces of the cell-sorted table
                const int ulo = cx + (own_row ? 0 : -L0), uhi = cx + L0;
                for (int piece = 0; piece < 3; ++piece) {
                    const int plo = piece == 0 ? ulo : (piece == 1 ? max(ulo, 0) : max(ulo, n0));
                    const int phi = piece == 0 ? min(uhi, -1) : (piece == 1 ? min(uhi, n0 - 1) : uhi);
                    if (plo > phi) continue;
                    const int shift = piece == 0 ? n0 : (piece == 1 ? 0 : -n0);
                    const int first = row + plo + shift;          // first cell of the piece
                    const int ncell = phi - plo + 1;
                    const int beg = cstart[first], end = cstart[first + ncell];
                    if (beg == end) continue;
                    // cell starts inside the piece, one per lane
                    const int bnd = lane + 1 < ncell ? cstart[first + lane + 1] : 0x7fffffff;
                    for (int p0 = beg; p0 < end; p0 += 32) {
                        const int p = p0 + lane;
                        const bool in = p < end;
                        const int pc = in ? p : end - 1;
                        const float4 q = cq32[pc];
                        const int v = cmol[pc];
                        int k = 0;  // cells of the piece that start at or before p
                        for (int j = 0; j + 1 < ncell; ++j) k += p >= __shfl_sync(0xffffffffu, bnd, j) ? 1 : 0;
                        const int dx = plo + k - cx;
                        const int src = dx + L0;
                        const float ox = __shfl_sync(0xffffffffu, rowoff.x, src);
                        const float oy = __shfl_sync(0xffffffffu, rowoff.y, src);
                        const float oz = __shfl_sync(0xffffffffu, rowoff.z, src);
                        float4 Dv;
                        Dv.x = (q.x - qs.x) + ox;
                        Dv.y = (q.y - qs.y) + oy;
                        Dv.z = (q.z - qs.z) + oz;
                        Dv.w = __int_as_float(v);
                        const float rr = rsc + q.w;
                        const bool cand = in && fmaf(Dv.z, Dv.z, fmaf(Dv.y, Dv.y, Dv.x * Dv.x)) <= rr * rr &&
                                          !(own_row && dx == 0 && v <= s);
                        const unsigned mask = __ballot_sync(0xffffffffu, cand);
                        const int pos = cnt + __popc(mask & ((1u << lane) - 1u));
                        if (cand) {
                            W.cq[pos] = Dv;
                            W.cc[pos] = pack_delta(dx, dy, dz);
                        }
                        cnt += __popc(mask);
                        if (cnt >= 32) {
                            __syncwarp();
                            flat_batch<SELF, APS>(S, B, h, W, Pf, g, f, s, sslot, rs2, lane, 32, st);
                            __syncwarp();
                            float4 rq = make_float4(0.f, 0.f, 0.f, 0.f);
                            int rc = 0;
                            if (lane < cnt - 32) {
                                rq = W.cq[32 + lane];
                                rc = W.cc[32 + lane];
                            }
                            __syncwarp();
                            if (lane < cnt - 32) {
                                W.cq[lane] = rq;
                                W.cc[lane] = rc;
                            }
                            cnt -= 32;
                            __syncwarp();
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (cnt > 0) flat_batch<SELF, APS>(S, B, h, W, Pf, g, f, s, sslot, rs2, lane, cnt, st);
        __syncwarp();
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// ------------------------------------------------------------ tiled real pass
// Self mode.  The stencil walk of k_pairs_flat32 gathers each neighbour
// cell's molecule table from L2 once per solute molecule, one warp per
// molecule, and was most of that kernel's time.  Here a CTA takes one home
// cell: it stages the molecules of the cell's half stencil (the home cell,
// its row forward, the rest of its plane forward, the planes above) in
// shared memory once -- each as its cell-relative centroid plus the cell's
// stencil offset, with its radius and, packed with its index, the staged
// cell -- and its warps then claim the home cell's molecules one by one and
// test each against the whole staged table, 32 candidates per round.  The
// candidates then go through flat_batch exactly as in k_pairs_flat32 (the
// displacement is formed as (q_v + off) - q_s, an order the guard band
// covers), so the records, and the guard and edge queues, are the same.
#ifndef CM_TILE_WARPS
#define CM_TILE_WARPS 12
#endif
#ifndef CM_TILE_MIN_CTAS
#define CM_TILE_MIN_CTAS 2
#endif
constexpr int kTileWarps = CM_TILE_WARPS;
constexpr int kTileStage = 1024;  // staged neighbour molecules per pass

struct TileSmem {
    float4 w[kTileStage];       // staged molecule: centroid + stencil offset (x, y, z), radius
    int v[kTileStage];          // molecule index | staged cell << 24
    int nbeg[kTileCells + 1];   // first staged position of each cell (prefix of the cells' molecule counts)
    int cbeg[kTileCells];       // the cell's first position in the cell-sorted molecule table
    int code[kTileCells];       // the cell's packed stencil offset
    int next;                   // next home molecule to claim
    int item;                   // the CTA's current (frame, home cell) item
};

__host__ __device__ constexpr size_t tile_smem_extra() { return sizeof(TileSmem) + 16; }

// Stencil offset of half-stencil cell k: the home cell's row forward
// (k <= L0), the rest of its plane forward, then the planes above.
__device__ __forceinline__ void half_stencil_cell(int k, const int *L, int &dx, int &dy, int &dz) {
    const int wx = 2 * L[0] + 1;
    if (k <= L[0]) {
        dx = k; dy = 0; dz = 0;
        return;
    }
    k -= L[0] + 1;
    if (k < wx * L[1]) {
        dy = 1 + k / wx; dx = k % wx - L[0]; dz = 0;
        return;
    }
    k -= wx * L[1];
    const int wxy = wx * (2 * L[1] + 1);
    dz = 1 + k / wxy;
    const int r = k % wxy;
    dy = r / wx - L[1];
    dx = r % wx - L[0];
}

template <int APS>
__global__ void __launch_bounds__(kTileWarps * 32, CM_TILE_MIN_CTAS) k_pairs_tile32(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    const int hw = hist_words(S);
    FlatWarpSmem *wsm = (FlatWarpSmem *)(smem_raw + (((size_t)hw * 4 + 15) & ~(size_t)15));
    TileSmem &T = *(TileSmem *)(((uintptr_t)(wsm + kTileWarps) + 15) & ~(uintptr_t)15);
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
    FlatWarpSmem &W = wsm[warp];
    LocalStats st;
    const int aps = S.aps;
    const int64_t ncap = B.cs - 1;
    const int64_t items = (int64_t)B.nf * ncap;
    // CTAs claim (frame, home cell) items from counters[6] (zeroed with the
    // chunk's counters): the items' costs vary with the cells' occupancy
    for (;;) {
        __syncthreads();  // the previous item's staged table and claim are no longer read
        if (tid == 0) T.item = atomicAdd(B.counters + 6, 1);
        __syncthreads();
        const int64_t t = T.item;
        if (t >= items) break;
        const int f = (int)(t / ncap), H = (int)(t - (int64_t)f * ncap);
        const PairsFrame Pf = pairs_frame(B, f, true);
        const FrameScratch &F = *Pf.F;
        const FrameGeom &G = *Pf.G;
        // every thread takes the same branches: the conditions depend on the item only
        if (!F.ok || !F.tile || H >= G.ncell) continue;
        const int hbeg = Pf.cstart[H], nH = Pf.cstart[H + 1] - hbeg;
        if (nH == 0) continue;
        const int n0 = G.n[0], n1 = G.n[1], n2 = G.n[2];
        const int cx = H % n0, cy = (H / n0) % n1, cz = H / (n0 * n1);
        const int K = (F.L[0] + 1) + (2 * F.L[0] + 1) * F.L[1] + (2 * F.L[0] + 1) * (2 * F.L[1] + 1) * F.L[2];
        const Guard g = F.g;
        const float4 *cq32 = B.cq32 + (int64_t)f * B.mv;
        if (tid < K) {
            int dx, dy, dz;
            half_stencil_cell(tid, F.L, dx, dy, dz);
            const int c = (wrap_cell(cz + dz, n2) * n1 + wrap_cell(cy + dy, n1)) * n0 + wrap_cell(cx + dx, n0);
            T.cbeg[tid] = Pf.cstart[c];
            T.nbeg[tid + 1] = Pf.cstart[c + 1] - Pf.cstart[c];
            T.code[tid] = pack_delta(dx, dy, dz);
        }
        if (tid == 0) T.nbeg[0] = 0;
        __syncthreads();
        if (warp == 0) {
            // inclusive prefix of the K <= kTileCells counts, four per lane
            int c[4], sum = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = 4 * lane + j;
                c[j] = k < K ? T.nbeg[k + 1] : 0;
                sum += c[j];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += u;
            }
            int run = incl - sum;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = 4 * lane + j;
                run += c[j];
                if (k < K) T.nbeg[k + 1] = run;
            }
        }
        __syncthreads();
        const int M = T.nbeg[K];
        for (int m0 = 0; m0 < M; m0 += kTileStage) {
            const int n = min(kTileStage, M - m0);
            if (m0 > 0) __syncthreads();  // the previous pass's table is no longer read
            for (int i = tid; i < n; i += blockDim.x) {
                const int m = m0 + i;
                int lo = 0, hi = K;  // the cell k with nbeg[k] <= m < nbeg[k + 1]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (T.nbeg[mid] <= m) lo = mid;
                    else hi = mid;
                }
                int dx, dy, dz;
                half_stencil_cell(lo, F.L, dx, dy, dz);
                const float4 of = Pf.off32[off_index(dx, dy, dz)];
                const int p = T.cbeg[lo] + (m - T.nbeg[lo]);
                const float4 q = cq32[p];
                T.w[i] = make_float4(q.x + of.x, q.y + of.y, q.z + of.z, q.w);
                T.v[i] = Pf.cmol[p] | (lo << 24);
            }
            if (tid == 0) T.next = 0;
            __syncthreads();
            // the home molecules, claimed one at a time
            const int own_end = T.nbeg[1] - m0;  // staged positions below this are the home cell (pass 0)
            for (;;) {
                int sl = 0;
                if (lane == 0) sl = atomicAdd(&T.next, 1);
                sl = __shfl_sync(0xffffffffu, sl, 0);
                if (sl >= nH) break;
                const int s = Pf.cmol[hbeg + sl];
                const float4 qs = Pf.sq32[s];
                const int sslot = Pf.slot ? Pf.slot[s] : -1;
                __syncwarp();
                for (int a = lane; a < aps; a += 32) W.os[a] = Pf.so32[(int64_t)s * aps + a];
                __syncwarp();
                const float rsc = g.cut_pre + qs.w;
                const float rs2 = rsc * rsc;
                int cnt = 0;
                for (int p0 = 0; p0 < n; p0 += 32) {
                    const int p = p0 + lane;
                    const bool in = p < n;
                    const int pc = in ? p : n - 1;
                    const float4 w = T.w[pc];
                    const int vk = T.v[pc];
                    const int v = vk & 0xffffff;
                    float4 Dv;
                    Dv.x = w.x - qs.x;
                    Dv.y = w.y - qs.y;
                    Dv.z = w.z - qs.z;
                    Dv.w = __int_as_float(v);
                    const float rr = rsc + w.w;
                    const bool cand = in && fmaf(Dv.z, Dv.z, fmaf(Dv.y, Dv.y, Dv.x * Dv.x)) <= rr * rr &&
                                      !(p < own_end && v <= s);
                    const unsigned mask = __ballot_sync(0xffffffffu, cand);
                    const int pos = cnt + __popc(mask & ((1u << lane) - 1u));
                    if (cand) {
                        W.cq[pos] = Dv;
                        W.cc[pos] = T.code[vk >> 24];
                    }
                    cnt += __popc(mask);
                    if (cnt >= 32) {
                        __syncwarp();
                        flat_batch<true, APS>(S, B, h, W, Pf, g, f, s, sslot, rs2, lane, 32, st);
                        __syncwarp();
                        float4 rq = make_float4(0.f, 0.f, 0.f, 0.f);
                        int rc = 0;
                        if (lane < cnt - 32) {
                            rq = W.cq[32 + lane];
                            rc = W.cc[32 + lane];
                        }
                        __syncwarp();
                        if (lane < cnt - 32) {
                            W.cq[lane] = rq;
                            W.cc[lane] = rc;
                        }
                        cnt -= 32;
                        __syncwarp();
                    }
                }
                __syncwarp();
                if (cnt > 0) flat_batch<true, APS>(S, B, h, W, Pf, g, f, s, sslot, rs2, lane, cnt, st);
                __syncwarp();
            }
        }
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// ------------------------------------------------------------ guard kernel
// Exact processing of the candidates deferred by the FP32 real pass, one warp
// per queued molecule pair: the lanes split the pair's atom pairs (over its
// images), for the FP32 pass and for the filtered FP64 scan, and the lanes'
// results are merged.  The FP64 minimum is merged by the reference's tie rule
// (distance, then the larger (solute atom, solvent atom) pair; in self mode the
// second direction's key is (solvent atom, solute atom)), which does not
// depend on the order in which pairs are visited, so the records are those of
// pairs_decide.

// Atom pair i of a molecule pair: image i / (aps apv), then solvent atom b and
// solute atom a; the quotients from FP32 reciprocals are exact for i < 2^16.
struct PairIndex {
    float inv_pi, inv_aps;
    int per_img, aps;
    __device__ __forceinline__ void at(int i, int &img, int &b, int &a) const {
        img = (int)((float(i) + 0.5f) * inv_pi);
        const int r = i - img * per_img;
        b = (int)((float(r) + 0.5f) * inv_aps);
        a = r - b * aps;
    }
};

__device__ __forceinline__ void image_at(const Images &im, int img, int &dx, int &dy, int &dz) {
    const int ix = img % im.cnt[0], iy = (img / im.cnt[0]) % im.cnt[1], iz = img / (im.cnt[0] * im.cnt[1]);
    dx = im.base[0] + ix * im.step[0];
    dy = im.base[1] + iy * im.step[1];
    dz = im.base[2] + iz * im.step[2];
}

// FP32 pass of pairs_pass32 with the pairs split over the lanes; every lane
// ends with the merged result (second-smallest over the union: the smaller of
// the larger minimum and the smaller second minima).
template <bool SELF>
__device__ __forceinline__ void pass32_warp(const DevSys &S, const float4 *__restrict__ off32, const Images &im, float4 qs,
                                            float4 qv, const float4 *os, const float4 *ov, const PairIndex &pi, int total,
                                            int lane, Pass32 &P) {
    constexpr unsigned kFull = 0xffffffffu;
    P.m1 = P.m2 = P.r1 = P.r2 = INFINITY;
    P.k1 = 0x7fffffff;
    const int apv = S.apv, iref = S.iref;
    int cur = -1;
    float Dx = 0.f, Dy = 0.f, Dz = 0.f;
    for (int i = lane; i < total; i += 32) {
        int img, b, a;
        pi.at(i, img, b, a);
        if (img != cur) {
            int dx, dy, dz;
            image_at(im, img, dx, dy, dz);
            const float4 o = off32[off_index(dx, dy, dz)];
            Dx = (qv.x - qs.x) + o.x;
            Dy = (qv.y - qs.y) + o.y;
            Dz = (qv.z - qs.z) + o.z;
            cur = img;
        }
        const float4 ob = ov[b], oa = os[a];
        const float tx = Dx + ob.x, ty = Dy + ob.y, tz = Dz + ob.z;
        const float ex = tx - oa.x, ey = ty - oa.y, ez = tz - oa.z;
        const float d2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
        const int k = a * apv + b;
        P.m2 = fminf(P.m2, fmaxf(P.m1, d2));
        P.k1 = d2 < P.m1 ? k : P.k1;
        P.m1 = fminf(P.m1, d2);
        if (b == iref) P.r1 = fminf(P.r1, d2);
        if (SELF && a == iref) P.r2 = fminf(P.r2, d2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float m1 = __shfl_xor_sync(kFull, P.m1, o), m2 = __shfl_xor_sync(kFull, P.m2, o);
        const int k1 = __shfl_xor_sync(kFull, P.k1, o);
        P.m2 = fminf(fmaxf(P.m1, m1), fminf(P.m2, m2));
        if (m1 < P.m1 || (m1 == P.m1 && k1 < P.k1)) {
            P.m1 = m1;
            P.k1 = k1;
        }
        P.r1 = fminf(P.r1, __shfl_xor_sync(kFull, P.r1, o));
        if (SELF) P.r2 = fminf(P.r2, __shfl_xor_sync(kFull, P.r2, o));
    }
}

// pairs_exact with the pairs split over the lanes (FP32 filter), merged over
// the warp; every lane ends with the result.
template <bool SELF>
__device__ void exact_warp(const DevSys &S, const FrameGeom &G, const Bufs &B, ExactMol &X,
                           const float4 *__restrict__ off32, const Images &im, float4 qs32, float4 qv32,
                           const float4 *os32, const float4 *ov32, float thr_arg, float thr_r1, float thr_r2,
                           const PairIndex &pi, int total, int lane, Exact64 &E) {
    constexpr unsigned kFull = 0xffffffffu;
    best_init(E.B);
    E.rr1 = INFINITY;
    E.rr2 = INFINITY;
    E.evals = 0;
    const int iref = S.iref;
    const double cut2 = S.cut2;
    int cur = -1;
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    for (int i = lane; i < total; i += 32) {
        int img, b, a;
        pi.at(i, img, b, a);
        if (img != cur) {
            int dx, dy, dz;
            image_at(im, img, dx, dy, dz);
            const float4 of = off32[off_index(dx, dy, dz)];
            Fx = (qv32.x - qs32.x) + of.x;
            Fy = (qv32.y - qs32.y) + of.y;
            Fz = (qv32.z - qs32.z) + of.z;
            cur = img;
        }
        const float4 ob32 = ov32[b], oa32 = os32[a];
        const float ex = (Fx + ob32.x) - oa32.x, ey = (Fy + ob32.y) - oa32.y, ez = (Fz + ob32.z) - oa32.z;
        const float d2f = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
        if (!(d2f <= thr_arg || (b == iref && d2f <= thr_r1) || (SELF && a == iref && d2f <= thr_r2))) continue;
        const double d2 = exact_pair_d2(B, G, X, a, b);
        E.evals++;
        if (d2 <= cut2) {
            if (b == iref) E.rr1 = fmin(E.rr1, d2);
            if (SELF && a == iref) E.rr2 = fmin(E.rr2, d2);
            best_update<SELF>(E.B, d2, a, b);
        }
    }
    // merge: smallest d = sqrt(d2); among equal d the larger (a, b), and in
    // self mode separately the larger (b, a)
    double d = E.B.d2 <= cut2 ? best_d(E.B) : INFINITY;
    double d2 = E.B.d2;
    int a1 = E.B.a, b1 = E.B.b, a2 = E.B.a2, b2 = E.B.b2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(kFull, d, o), od2 = __shfl_xor_sync(kFull, d2, o);
        const int oa1 = __shfl_xor_sync(kFull, a1, o), ob1 = __shfl_xor_sync(kFull, b1, o);
        const int oa2 = __shfl_xor_sync(kFull, a2, o), ob2 = __shfl_xor_sync(kFull, b2, o);
        if (od < d) {
            d = od;
            d2 = od2;
            a1 = oa1; b1 = ob1; a2 = oa2; b2 = ob2;
        } else if (od == d) {
            if (oa1 > a1 || (oa1 == a1 && ob1 > b1)) { a1 = oa1; b1 = ob1; }
            if (SELF && (ob2 > b2 || (ob2 == b2 && oa2 > a2))) { a2 = oa2; b2 = ob2; }
        }
        E.rr1 = fmin(E.rr1, __shfl_xor_sync(kFull, E.rr1, o));
        if (SELF) E.rr2 = fmin(E.rr2, __shfl_xor_sync(kFull, E.rr2, o));
        E.evals += __shfl_xor_sync(kFull, E.evals, o);
    }
    E.B.d2 = d2;
    E.B.d = d <= 1e300 ? d : -1.0;
    E.B.a = a1; E.B.b = b1; E.B.a2 = a2; E.B.b2 = b2;
}

// pairs_decide with the warp-parallel pass and scans; the statistics are
// counted on lane 0.
template <bool SELF>
__device__ void decide_warp(const DevSys &S, const FrameGeom &G, const Bufs &B, ExactMol &X, const Guard &g,
                            const Pass32 &P, const float4 *__restrict__ off32, const Images &im, float4 qs32, float4 qv32,
                            const float4 *os32, const float4 *ov32, int s, int64_t v, const PairIndex &pi, int total,
                            int lane, DirRec &r1, DirRec &r2, LocalStats &st) {
    r1 = dir_none(S);
    r2 = dir_none(S);
    if (P.m1 > g.cutp2) return;
    const float d1 = sqrtf(P.m1);
    const bool amb = P.m1 >= g.cutm2 || (sqrtf(P.m2) - d1) <= g.two_delta;
    if (amb) {
        const float t = d1 + g.two_delta;
        const float thr = __fmul_ru(t, t);
        float thr1 = -1.f, thr2 = -1.f;
        if (P.r1 <= g.cutp2) { const float u = sqrtf(P.r1) + g.two_delta; thr1 = __fmul_ru(u, u); }
        if (SELF && P.r2 <= g.cutp2) { const float u = sqrtf(P.r2) + g.two_delta; thr2 = __fmul_ru(u, u); }
        if (!SELF) thr2 = INFINITY;
        Exact64 E;
        exact_warp<SELF>(S, G, B, X, off32, im, qs32, qv32, os32, ov32, thr, thr1, thr2, pi, total, lane, E);
        records_from_exact<SELF>(S, E, s, v, r1, r2);
        if (lane == 0) {
            st.guard++;
            st.guard_pairs += E.evals;
            if (E.B.d2 <= S.cut2) st.maxerr = fmax(st.maxerr, fabs((double)d1 - best_d(E.B)));
        }
        return;
    }
    // unambiguous: the FP32 minimum pair is the exact minimum pair, within cutoff
    const int a = P.k1 / S.apv, b = P.k1 - a * S.apv;
    int bin = bin32(g, d1);
    double d64 = -1.0;
    if (bin < 0 || (S.usecutoff && d1 >= g.dbulk_lo && d1 <= g.dbulk_hi)) {
        d64 = sqrt(exact_pair_d2(B, G, X, a, b));
        bin = setbin0(d64, S.binstep);
        if (lane == 0) {
            st.guard++;
            st.guard_pairs += 1;
            st.maxerr = fmax(st.maxerr, fabs((double)d1 - d64));
        }
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
        const float rm = dir == 0 ? P.r1 : P.r2;
        DirRec &r = dir == 0 ? r1 : r2;
        if (rm > g.cutp2) continue;
        const int rb = rm < g.cutm2 ? bin32(g, sqrtf(rm)) : -1;
        if (rb >= 0) {
            r.ref = 1;
            r.rbin = rb;
            continue;
        }
        const float u = sqrtf(rm) + g.two_delta;
        const float thr = __fmul_ru(u, u);
        Exact64 E;
        exact_warp<SELF>(S, G, B, X, off32, im, qs32, qv32, os32, ov32, -1.f, dir == 0 ? thr : -1.f, dir == 1 ? thr : -1.f,
                         pi, total, lane, E);
        const double rr = dir == 0 ? E.rr1 : E.rr2;
        if (lane == 0) {
            st.guard++;
            st.guard_pairs += E.evals;
        }
        if (rr <= S.cut2) {
            r.ref = 1;
            r.rbin = setbin0(sqrt(rr), S.binstep);
        }
    }
}

constexpr int kGuardWarps = 4;  // warps per CTA of k_pairs_guard

template <bool SELF>
__global__ void __launch_bounds__(kGuardWarps * 32) k_pairs_guard(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float4 s_os[kGuardWarps][kMaxSmallMol], s_ov[kGuardWarps][kMaxSmallMol];
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    LocalStats st;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int aps = S.aps, apv = S.apv;
    PairIndex pi;
    pi.per_img = aps * apv;
    pi.aps = aps;
    pi.inv_pi = 1.0f / (float)pi.per_img;
    pi.inv_aps = 1.0f / (float)aps;
    const int n = min(B.counters[0], B.gq_cap);
    // warps claim records from counters[7] (zeroed with the chunk's
    // counters): a record's cost varies with its exact scan
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(B.counters + 7, 1);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= n) break;
        const int4 it = B.gq[i];
        const int s = it.x, v = it.y, f = it.w;
        const PairsFrame Pf = pairs_frame(B, f, SELF);
        const FrameScratch &F = *Pf.F;
        const Images im = images_of(*Pf.G, F, it.z);
        const int total = pi.per_img * image_count(im);
        const float4 qs32 = Pf.sq32[s], qv32 = Pf.vq32[v];
        __syncwarp();
        if (lane < aps) s_os[warp][lane] = Pf.so32[(int64_t)s * aps + lane];
        if (lane < apv) s_ov[warp][lane] = Pf.vo32[(int64_t)v * apv + lane];
        __syncwarp();
        Pass32 P;
        pass32_warp<SELF>(S, Pf.off32, im, qs32, qv32, s_os[warp], s_ov[warp], pi, total, lane, P);
        DirRec r1, r2;
        ExactMol X = exact_mol(S, f, s, v);
        decide_warp<SELF>(S, *Pf.G, B, X, F.g, P, Pf.off32, im, qs32, qv32, s_os[warp], s_ov[warp], s, v, pi, total, lane, r1,
                          r2, st);
        if (lane == 0) emit<SELF>(S, h, r1, r2, s, v, Pf.slot, Pf.flags, st);
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// FP32 squared distance of one atom pair, the smallest over the images,
// formed as in the FP32 passes ((q_v - q_s) + off + offset of b - offset of a).
__device__ __forceinline__ float edge_d2(const PairsFrame &Pf, const Images &im, int s, int v, float4 oa, float4 ob) {
    const float4 qs = Pf.sq32[s], qv = Pf.vq32[v];
    float best = INFINITY;
    CM_FOR_IMAGES(im, dx, dy, dz) {
        const float4 o = Pf.off32[off_index(dx, dy, dz)];
        const float ex = (((qv.x - qs.x) + o.x) + ob.x) - oa.x;
        const float ey = (((qv.y - qs.y) + o.y) + ob.y) - oa.y;
        const float ez = (((qv.z - qs.z) + o.z) + ob.z) - oa.z;
        best = fminf(best, fmaf(ez, ez, fmaf(ey, ey, ex * ex)));
    }
    return best;
}

// Edge kernel: records whose closest atom pair is known from the FP32 pass
// (second-closest pair beyond 2 delta, cutoff and dbulk clear) but whose md
// bin, solvent reference-atom row or solute reference-atom column (marked -2)
// lies within the guard band of a bin edge or of the cutoff.  Each marked
// value comes from exact pair distances (exact_d2): the closest pair for the
// md bin, the aps pairs of the solvent molecule's reference atom for the row,
// the apv pairs of the solute molecule's reference atom for the column.
template <bool SELF>
__global__ void __launch_bounds__(128) k_pairs_edge(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    LocalStats st;
    const int n = min(B.counters[3], B.eq_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 e = B.eq[3 * i], x = B.eq[3 * i + 1], y = B.eq[3 * i + 2];
        const int s = e.x, v = e.y, f = e.w;
        const int a1 = x.x & 0xff, b1 = (x.x >> 8) & 0xff;
        int rb1 = x.y, rb2 = x.z, bin = x.w;
        const float d32 = __int_as_float(y.x);
        const PairsFrame Pf = pairs_frame(B, f, SELF);
        const Images im = images_of(*Pf.G, *Pf.F, e.z);
        const FrameGeom &G = *Pf.G;
        ExactMol X = exact_mol(S, f, s, v);
        st.guard++;
        int bulk = S.usecutoff ? (d32 > Pf.F->g.dbulk_hi) : 0;
        if (bin == -2) {
            const double d64 = sqrt(exact_pair_d2(B, G, X, a1, b1));
            bin = setbin0(d64, S.binstep);
            bulk = S.usecutoff ? (d64 > S.dbulk) : 0;
            st.guard_pairs += 1;
            st.maxerr = fmax(st.maxerr, fabs((double)d32 - d64));
        }
        // a row or column minimum in the band: its FP32 pass picks the pairs
        // within 2 delta of the FP32 minimum (the exact minimum is among them),
        // which are then evaluated exactly
        const Guard &g = Pf.F->g;
        if (rb1 == -2) {
            const float4 ob = Pf.vo32[(int64_t)v * S.apv + S.iref];
            const float4 *os32 = Pf.so32 + (int64_t)s * S.aps;
            float m = INFINITY;
            for (int a = 0; a < S.aps; ++a) m = fminf(m, edge_d2(Pf, im, s, v, os32[a], ob));
            const float t = sqrtf(m) + g.two_delta, thr = __fmul_ru(t, t);
            double rr = INFINITY;
            for (int a = 0; a < S.aps; ++a) {
                if (!(edge_d2(Pf, im, s, v, os32[a], ob) <= thr)) continue;
                rr = fmin(rr, exact_pair_d2(B, G, X, a, S.iref));
                st.guard_pairs += 1;
            }
            rb1 = rr <= S.cut2 ? setbin0(sqrt(rr), S.binstep) : -1;
        }
        if (SELF && rb2 == -2) {
            const float4 oa = Pf.so32[(int64_t)s * S.aps + S.iref];
            const float4 *ov32 = Pf.vo32 + (int64_t)v * S.apv;
            float m = INFINITY;
            for (int b = 0; b < S.apv; ++b) m = fminf(m, edge_d2(Pf, im, s, v, oa, ov32[b]));
            const float t = sqrtf(m) + g.two_delta, thr = __fmul_ru(t, t);
            double rr = INFINITY;
            for (int b = 0; b < S.apv; ++b) {
                if (!(edge_d2(Pf, im, s, v, oa, ov32[b]) <= thr)) continue;
                rr = fmin(rr, exact_pair_d2(B, G, X, S.iref, b));
                st.guard_pairs += 1;
            }
            rb2 = rr <= S.cut2 ? setbin0(sqrt(rr), S.binstep) : -1;
        }
        apply_hit_local(S, h, false, bin, a1, (int64_t)v * S.apv + b1, b1, rb1 >= 0, rb1);
        st.hits++;
        if (SELF) {
            apply_hit_local(S, h, false, bin, b1, (int64_t)s * S.aps + a1, a1, rb2 >= 0, rb2);
            st.hits++;
        }
        if (Pf.slot) {
            const unsigned char code1 = (unsigned char)(1 + bulk);
            const int sl = Pf.slot[s];
            if (sl >= 0) Pf.flags[(int64_t)sl * S.mv + v] = code1;
            if (SELF) {
                const int vs = Pf.slot[v];
                if (vs >= 0) Pf.flags[(int64_t)vs * S.mv + s] = code1;
            }
        }
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

}  // namespace cmk
