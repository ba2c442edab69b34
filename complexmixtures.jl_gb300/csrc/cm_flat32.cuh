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

constexpr int kFlatWarps = 16;   // warps per CTA (2 CTAs per SM at 64 registers)
constexpr int kAtomQueue = 64;   // per-warp atom queue (float4: t, tag)

struct CandSlot {
    unsigned long long k1;
    unsigned int m2, r1, r2, pad;
};

constexpr unsigned long long kNoPair = (0x7f800000ull << 32) | 0xffffffffull;  // +inf, largest index

// Shared memory of one warp after the histograms.
struct FlatWarpSmem {
    float4 os[kMaxSmallMol];      // solute atom offsets (x, y, z)
    float4 aq[kAtomQueue];        // atom queue: t = position relative to the solute centroid, w = tag c << 8 | b
    float4 cq[kQueue];            // candidate queue: D = centroid displacement, w = molecule index
    int cc[kQueue];               // candidate queue: packed cell offset
    CandSlot cand[32];
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
        CandSlot &C = W.cand[c];
        const unsigned long long key = ((unsigned long long)__float_as_uint(m1) << 32) | (unsigned)(k1 << 8 | b);
        const unsigned long long old = atomicMin(&C.k1, key);
        const float displaced = fmaxf(m1, __uint_as_float((unsigned)(old >> 32)));
        atomicMin(&C.m2, __float_as_uint(fminf(displaced, m2)));
        if (b == S.iref) C.r1 = __float_as_uint(m1);
        if (SELF) {
            const float4 oi = W.os[S.iref];
            const float dx = e.x - oi.x, dy = e.y - oi.y, dz = e.z - oi.z;
            atomicMin(&C.r2, __float_as_uint(fmaf(dz, dz, fmaf(dy, dy, dx * dx))));
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
        CandSlot &C = W.cand[lane];
        C.k1 = kNoPair;
        C.m2 = 0x7f800000u;
        C.r1 = 0x7f800000u;
        C.r2 = 0x7f800000u;
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
    const CandSlot &C = W.cand[lane];
    const unsigned long long k1 = C.k1;
    if (k1 == kNoPair) return;
    const float m1 = __uint_as_float((unsigned)(k1 >> 32));
    if (m1 > g.cutp2) return;  // no atom pair within the cutoff
    const int v = __float_as_int(W.cq[lane].w), code = W.cc[lane];
    const int a1 = (int)((unsigned)k1 >> 8) & 0xff, b1 = (int)(k1 & 0xff);
    const float m2 = __uint_as_float(C.m2), r1 = __uint_as_float(C.r1), r2 = __uint_as_float(C.r2);
    const float dmin = sqrtf(m1);
    // hard: the closest pair, or the cutoff or dbulk decision, needs the full
    // FP64 rules (guard queue)
    bool hard = m1 >= g.cutm2 || (sqrtf(m2) - dmin) <= g.two_delta;
    if (S.usecutoff) hard = hard || (dmin >= g.dbulk_lo && dmin <= g.dbulk_hi);
    if (hard) {
        const int slot = atomicAdd(B.counters + 0, 1);
        if (slot < B.gq_cap) B.gq[slot] = make_int4(s, v, code, f);
        else raise_err(S, ERR_QUEUE);
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
        } else {
            raise_err(S, ERR_QUEUE);
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

template <bool SELF, int APS>
__global__ void __launch_bounds__(kFlatWarps * 32, 2) k_pairs_flat32(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    const int hw = hist_words(S);
    FlatWarpSmem *wsm = (FlatWarpSmem *)(smem_raw + (((size_t)hw * 4 + 15) & ~(size_t)15));
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

// Guard kernel: exact processing of the candidates deferred by the FP32 real
// pass (the FP32 pass of the molecule pair is recomputed and pairs_decide
// takes every decision with the FP64 rules).
template <bool SELF>
__global__ void __launch_bounds__(128) k_pairs_guard(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    LocalStats st;
    const int n = min(B.counters[0], B.gq_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 it = B.gq[i];
        const int s = it.x, v = it.y, f = it.w;
        const PairsFrame Pf = pairs_frame(B, f, SELF);
        const FrameScratch &F = *Pf.F;
        const Images im = images_of(*Pf.G, F, it.z);
        const float4 qs32 = Pf.sq32[s], qv32 = Pf.vq32[v];
        const d4 qs64 = Pf.sq64[s], qv64 = Pf.vq64[v];
        const float4 *os = Pf.so32 + (int64_t)s * S.aps;
        const float4 *ov = Pf.vo32 + (int64_t)v * S.apv;
        Pass32 P;
        pairs_pass32<SELF>(S, Pf.off32, im, qs32, qv32, os, ov, P);
        DirRec r1, r2;
        pairs_decide<SELF>(S, F.g, P, Pf.off64, Pf.off32, im, qs64, qs32, qv64, qv32, Pf.so64 + (int64_t)s * S.aps, os,
                           Pf.vo64 + (int64_t)v * S.apv, ov, s, v, r1, r2, st);
        emit<SELF>(S, h, r1, r2, s, v, Pf.slot, Pf.flags, st);
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// Edge kernel: records whose closest atom pair is known from the FP32 pass
// (second-closest pair beyond 2 delta, cutoff and dbulk clear) but whose md
// bin, solvent reference-atom row or solute reference-atom column (marked -2)
// lies within the guard band of a bin edge or of the cutoff.  Each marked
// value comes from FP64 pair distances formed as in the exact scan: the
// closest pair for the md bin, the aps pairs of the solvent molecule's
// reference atom for the row, the apv pairs of the solute molecule's
// reference atom for the column.
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
        const d4 qs = Pf.sq64[s], qv = Pf.vq64[v];
        const d4 *os = Pf.so64 + (int64_t)s * S.aps;
        const d4 *ov = Pf.vo64 + (int64_t)v * S.apv;
        const int nimg = image_count(im);
        st.guard++;
        int bulk = S.usecutoff ? (d32 > Pf.F->g.dbulk_hi) : 0;
        if (bin == -2) {
            const double d64 = sqrt(pairs_one64(Pf.off64, im, qs, qv, os[a1], ov[b1]));
            bin = setbin0(d64, S.binstep);
            bulk = S.usecutoff ? (d64 > S.dbulk) : 0;
            st.guard_pairs += nimg;
            st.maxerr = fmax(st.maxerr, fabs((double)d32 - d64));
        }
        if (rb1 == -2) {
            double rr = INFINITY;
            for (int a = 0; a < S.aps; ++a) rr = fmin(rr, pairs_one64(Pf.off64, im, qs, qv, os[a], ov[S.iref]));
            rb1 = rr <= S.cut2 ? setbin0(sqrt(rr), S.binstep) : -1;
            st.guard_pairs += (unsigned long long)S.aps * nimg;
        }
        if (SELF && rb2 == -2) {
            double rr = INFINITY;
            for (int b = 0; b < S.apv; ++b) rr = fmin(rr, pairs_one64(Pf.off64, im, qs, qv, os[S.iref], ov[b]));
            rb2 = rr <= S.cut2 ? setbin0(sqrt(rr), S.binstep) : -1;
            st.guard_pairs += (unsigned long long)S.apv * nimg;
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
