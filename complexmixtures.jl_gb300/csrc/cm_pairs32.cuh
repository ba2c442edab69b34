// cm_pairs32.cuh -- FP32 real pass of the PAIRS layout, specialised on the
// number of atoms of the solvent molecule.
//
// The hot loop runs in single precision only.  Per candidate molecule pair the
// lane keeps the solvent molecule's atoms, shifted by the pair displacement, in
// registers and streams the solute molecule's atoms from shared memory.  A
// candidate whose result cannot be decided from the FP32 values (inside the
// guard band of the cutoff, of a bin edge, of dbulk, or with a second-closest
// pair within 2 delta of the closest) is appended to a guard queue; the guard
// kernel re-evaluates those candidates with the exact FP64 rules, so the hot
// loop executes no FP64 instruction and its warps do not diverge into them.
// The records produced here are exactly those of pairs_decide.
#pragma once
#include "cm_kernels.cuh"

namespace cmk {

// One row (solute atom a) against the APV solvent atoms held in registers.
template <int APV, bool COL>
__device__ __forceinline__ void row32(const float (&tx)[APV], const float (&ty)[APV], const float (&tz)[APV], float4 oa,
                                      int a, float &m1, float &m2, int &k1, float &col) {
#pragma unroll
    for (int b = 0; b < APV; ++b) {
        float dx = tx[b] - oa.x, dy = ty[b] - oa.y, dz = tz[b] - oa.z;
        float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        m2 = fminf(m2, fmaxf(m1, d2));
        k1 = d2 < m1 ? a * APV + b : k1;
        m1 = fminf(m1, d2);
        if (COL) col = fminf(col, d2);
    }
}

// Occupancy: 3 CTAs per SM when the register-resident solvent molecule is small,
// 2 for larger molecules (14 atoms keep 42 coordinates live).  One warp per
// (frame, solute molecule) work item of the chunk.  Frames whose boxes need
// several images per molecule pair are left to k_pairs_real (only_multi).
template <int APV, bool SELF>
__global__ void __launch_bounds__(kWarps * 32, (APV <= 5 ? 3 : 2)) k_pairs_real32(DevSys S, Bufs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hbase = (unsigned int *)smem_raw;
    const int hw = hist_words(S);
    float4 *os_all = (float4 *)(smem_raw + (((size_t)hw * 4 + 15) & ~(size_t)15));
    int *q_all = (int *)(os_all + kWarps * kMaxSmallMol);
    shist_zero(S, hbase);
    __syncthreads();
    SHist h = shist_bind(S, hbase);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4 *os = os_all + warp * kMaxSmallMol;
    int *qv = q_all + warp * kQueue * 2;
    int *qi = qv + kQueue;
    LocalStats st;
    const int aps = S.aps, iref = S.iref;
    const int64_t items = (int64_t)B.nf * B.ms;
    for (int64_t t = (int64_t)blockIdx.x * kWarps + warp; t < items; t += (int64_t)gridDim.x * kWarps) {
        const int f = (int)(t / B.ms), s = (int)(t - (int64_t)f * B.ms);
        const PairsFrame Pf = pairs_frame(B, f, SELF);
        const FrameScratch &F = *Pf.F;
        if (!F.ok) {
            if (lane == 0) raise_err(S, ERR_STENCIL);
            continue;
        }
        if (F.multi) continue;  // several images per pair: the generic kernel takes the frame
        const Guard g = F.g;
        const float4 qs32 = Pf.sq32[s];
        __syncwarp();
        for (int a = lane; a < aps; a += 32) os[a] = Pf.so32[(int64_t)s * aps + a];
        __syncwarp();
        const int sslot = Pf.slot ? Pf.slot[s] : -1;
        auto defer = [&](int v, int code) {
            const int slot = atomicAdd(B.counters + 0, 1);
            if (slot < B.gq_cap) B.gq[slot] = make_int4(s, v, code, f);
            else raise_err(S, ERR_QUEUE);
        };
        auto process = [&](int v, int code) {
            st.molpairs++;
            st.atompairs += (unsigned long long)aps * APV;
            int d0, d1, d2;
            unpack_delta(code, d0, d1, d2);
            const float4 o = Pf.off32[off_index(d0, d1, d2)];
            const float4 qv = Pf.vq32[v];
            const float Dx = (qv.x - qs32.x) + o.x, Dy = (qv.y - qs32.y) + o.y, Dz = (qv.z - qs32.z) + o.z;
            float tx[APV], ty[APV], tz[APV];
            const float4 *ov = Pf.vo32 + (int64_t)v * APV;
#pragma unroll
            for (int b = 0; b < APV; ++b) {
                const float4 ob = ov[b];
                tx[b] = Dx + ob.x;
                ty[b] = Dy + ob.y;
                tz[b] = Dz + ob.z;
            }
            float m1 = INFINITY, m2 = INFINITY, r2 = INFINITY, unused = 0.f;
            int k1 = 0;
#pragma unroll 1
            for (int a = 0; a < aps; ++a) {
                const float4 oa = os[a];
                if (SELF && a == iref) row32<APV, true>(tx, ty, tz, oa, a, m1, m2, k1, r2);
                else row32<APV, false>(tx, ty, tz, oa, a, m1, m2, k1, unused);
            }
            if (m1 > g.cutp2) return;  // no atom pair within the cutoff
            // column of v's reference atom
            float cxr = 0.f, cyr = 0.f, czr = 0.f;
#pragma unroll
            for (int b = 0; b < APV; ++b)
                if (b == iref) { cxr = tx[b]; cyr = ty[b]; czr = tz[b]; }
            float r1 = INFINITY;
#pragma unroll 1
            for (int a = 0; a < aps; ++a) {
                const float4 oa = os[a];
                const float dx = cxr - oa.x, dy = cyr - oa.y, dz = czr - oa.z;
                r1 = fminf(r1, fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
            }
            const float dmin = sqrtf(m1);
            bool hard = m1 >= g.cutm2 || (sqrtf(m2) - dmin) <= g.two_delta;
            const int bin = hard ? -1 : bin32(g, dmin);
            hard = hard || bin < 0;
            if (S.usecutoff) hard = hard || (dmin >= g.dbulk_lo && dmin <= g.dbulk_hi);
            int rb1 = -1, rb2 = -1;
            if (!hard && r1 <= g.cutp2) {
                rb1 = r1 < g.cutm2 ? bin32(g, sqrtf(r1)) : -1;
                hard = rb1 < 0;
            }
            if (SELF && !hard && r2 <= g.cutp2) {
                rb2 = r2 < g.cutm2 ? bin32(g, sqrtf(r2)) : -1;
                hard = rb2 < 0;
            }
            if (hard) {
                defer(v, code);
                return;
            }
            const int a1 = k1 / APV, b1 = k1 - a1 * APV;
            const int bulk = S.usecutoff ? (dmin > g.dbulk_hi) : 0;
            apply_hit(S, h, false, bin, a1, (int64_t)v * APV + b1, rb1 >= 0, rb1);
            st.hits++;
            if (SELF) {
                apply_hit(S, h, false, bin, b1, (int64_t)s * aps + a1, rb2 >= 0, rb2);
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
        };
        walk_candidates<SELF>(*Pf.G, F, s, Pf.scell[s], qs32, Pf.off32, Pf.vq32, Pf.cstart, Pf.cmol, qv, qi, lane, process);
    }
    stats_flush(S, st, false);
    __syncthreads();
    shist_flush(S, h, false);
}

// Guard kernel: exact processing of the candidates deferred by k_pairs_real32
// (the FP32 pass is recomputed and pairs_decide takes every decision).
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

}  // namespace cmk
