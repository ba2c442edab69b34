// cm_multi.cuh -- one launch per stage for many systems (cm_batch).
//
// A batch of independent systems of uneven size (config 4: 64 systems of
// 2,000-200,000 atoms) runs the same chain of stages per compute chunk.  Each
// stage of every system is one entry of a device work table: the system's own
// arguments (DevSys, Bufs, stage parameters), the grid it would have been
// launched with, and the first block it takes in the fused grid.  k_multi<KID>
// runs all entries of a stage in one launch: CTA b takes fused blocks
// b, b + gridDim.x, ...; a block finds its entry by binary search over the
// entries' first blocks and runs the stage's kernel body with the entry's
// arguments and its block index inside the entry's grid.  The persistent
// kernels (the ATOMS evaluation and the candidate-grid queries) get a small
// grid per system sized by its work and grid-stride inside it as they do in a
// launch of their own, each CTA privatising the histogram of its system.  A
// stage's zero-fills of every system are one k_multi_zero launch over a table
// of (pointer, bytes).
#pragma once
#include "cm_agrid.cuh"

namespace cmk {

// Arguments of one system's stage (the union of what the stage bodies take).
struct __align__(16) MArgs {
    DevSys S;
    Bufs B;
    const void *p;   // coordinates (prep), bulk table (k_bulk)
    int64_t i0, i1;  // coordinate stride (prep); item range (k_atoms_filter)
    int a0, a1;      // iref, centroids (prep solvent); pairs (frame consts); atoms_layout (scan); sample0, ny (random)
};

struct MTask {
    MArgs a;
    uint3 grid;          // the system's grid of this stage
    long long first;     // its first block in the fused grid
};

enum MKid : int {
    MK_OFFTABLE = 0,
    MK_PREP_SOLVENT_F32,
    MK_PREP_SOLVENT_F64,
    MK_PREP_SOLUTE_F32,
    MK_PREP_SOLUTE_F64,
    MK_FRAME_CONSTS,
    MK_SCAN,
    MK_SCATTER_ATOMS,
    MK_ATOMS_NEAR,
    MK_AGRID_BUILD,
    MK_AGRID_REAL,
    MK_AGRID_RANDOM,
    MK_ATOMS_FILTER,
    MK_ATOMS_PLACE,
    MK_SLOT_FILTER,
    MK_BULK,
    MK_EVAL_REAL_CELL,
    MK_EVAL_RANDOM_CELL,
    MK_EVAL_REAL_BALANCED,
    MK_EVAL_RANDOM_BALANCED,
    // the FP64 evaluations: stand-alone launches only (the plain FP64 path is not fused)
    MK_EVAL64_REAL_CELL,
    MK_EVAL64_RANDOM_CELL,
    MK_EVAL64_REAL_THREAD,
    MK_EVAL64_RANDOM_THREAD,
    MK_NKIDS
};

// Threads per CTA of each stage (the stand-alone launch's block size).
__host__ __device__ constexpr int mk_threads(int kid) {
    return kid == MK_OFFTABLE ? 256
         : (kid == MK_PREP_SOLVENT_F32 || kid == MK_PREP_SOLVENT_F64) ? 128
         : (kid == MK_PREP_SOLUTE_F32 || kid == MK_PREP_SOLUTE_F64) ? 256
         : kid == MK_FRAME_CONSTS ? 128
         : kid == MK_SCAN ? 1024
         : (kid == MK_SCATTER_ATOMS || kid == MK_ATOMS_NEAR) ? 256
         : kid == MK_AGRID_BUILD ? kAgridBuildThreads
         : (kid == MK_AGRID_REAL || kid == MK_AGRID_RANDOM || kid == MK_ATOMS_FILTER) ? 256
         : (kid == MK_ATOMS_PLACE || kid == MK_SLOT_FILTER) ? 128
         : kid == MK_BULK ? 1024
         : kAtomsWarps * 32;
}

template <int KID>
__device__ __forceinline__ void mk_body(const uint3 vb, const dim3 vg, const MArgs &a) {
    if constexpr (KID == MK_OFFTABLE) k_offtable_body(vb, vg, a.B);
    else if constexpr (KID == MK_PREP_SOLVENT_F32)
        k_prep_atoms_solvent_body<float>(vb, vg, a.B, (const float *)a.p, a.i0, a.a0, a.a1);
    else if constexpr (KID == MK_PREP_SOLVENT_F64)
        k_prep_atoms_solvent_body<double>(vb, vg, a.B, (const double *)a.p, a.i0, a.a0, a.a1);
    else if constexpr (KID == MK_PREP_SOLUTE_F32) k_prep_atoms_solute_body<float>(vb, vg, a.B, (const float *)a.p, a.i0);
    else if constexpr (KID == MK_PREP_SOLUTE_F64) k_prep_atoms_solute_body<double>(vb, vg, a.B, (const double *)a.p, a.i0);
    else if constexpr (KID == MK_FRAME_CONSTS) k_frame_consts_body(vb, vg, a.S, a.B, a.a0);
    else if constexpr (KID == MK_SCAN) k_scan_body(vb, vg, a.B, a.a0);
    else if constexpr (KID == MK_SCATTER_ATOMS) k_scatter_atoms_body(vb, vg, a.B);
    else if constexpr (KID == MK_ATOMS_NEAR) k_atoms_near_body(vb, vg, a.B);
    else if constexpr (KID == MK_AGRID_BUILD) k_agrid_build_body(vb, vg, a.S, a.B);
    else if constexpr (KID == MK_AGRID_REAL) k_agrid_real_body(vb, vg, a.S, a.B);
    else if constexpr (KID == MK_AGRID_RANDOM) k_agrid_random_body(vb, vg, a.S, a.B, a.a0, a.a1);
    else if constexpr (KID == MK_ATOMS_FILTER) k_atoms_filter_body(vb, vg, a.S, a.B, a.i0, a.i1);
    else if constexpr (KID == MK_ATOMS_PLACE) k_atoms_place_body(vb, vg, a.S, a.B, a.a0);
    else if constexpr (KID == MK_SLOT_FILTER) k_slot_filter_body(vb, vg, a.S, a.B, a.a0);
    else if constexpr (KID == MK_BULK) k_bulk_body(vb, vg, a.S, a.B, (const int4 *)a.p);
    else if constexpr (KID == MK_EVAL_REAL_CELL) k_atoms_eval_body<true, false, kSchedCell>(vb, vg, a.S, a.B);
    else if constexpr (KID == MK_EVAL_RANDOM_CELL) k_atoms_eval_body<true, true, kSchedCell>(vb, vg, a.S, a.B);
    else if constexpr (KID == MK_EVAL_REAL_BALANCED) k_atoms_eval_body<true, false, kSchedBalanced>(vb, vg, a.S, a.B);
    else if constexpr (KID == MK_EVAL_RANDOM_BALANCED) k_atoms_eval_body<true, true, kSchedBalanced>(vb, vg, a.S, a.B);
}

// Two resident CTAs per SM for the stages of up to 256 threads (four for the
// candidate-grid queries, as their stand-alone kernels): the arguments now
// come from the work table instead of the parameter space, and the register
// budget of the stand-alone kernels is kept.
__host__ __device__ constexpr int mk_min_ctas(int kid) {
    return (kid == MK_AGRID_REAL || kid == MK_AGRID_RANDOM) ? 4 : mk_threads(kid) <= 256 ? 2 : 1;
}

template <int KID>
__global__ void __launch_bounds__(mk_threads(KID), mk_min_ctas(KID))
    k_multi(const MTask *__restrict__ tasks, int ntasks, long long nblocks) {
    // the entry's arguments in shared memory: the bodies read them from there
    // as they need them instead of holding copies in registers
    __shared__ __align__(16) MArgs s_args;
    static_assert(sizeof(MArgs) % 16 == 0, "MArgs is copied as 16-byte words");
    for (long long vbk = blockIdx.x; vbk < nblocks; vbk += gridDim.x) {
        int lo = 0, hi = ntasks - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tasks[mid].first <= vbk) lo = mid;
            else hi = mid - 1;
        }
        const MTask &t = tasks[lo];
        for (int w = threadIdx.x; w < (int)(sizeof(MArgs) / 16); w += blockDim.x)
            reinterpret_cast<int4 *>(&s_args)[w] = reinterpret_cast<const int4 *>(&t.a)[w];
        const long long local = vbk - t.first;
        const uint3 g = t.grid;
        const uint3 vb = make_uint3((unsigned)(local % g.x), (unsigned)((local / g.x) % g.y),
                                    (unsigned)(local / ((long long)g.x * g.y)));
        __syncthreads();
        mk_body<KID>(vb, dim3(g.x, g.y, g.z), s_args);
        __syncthreads();  // the next block of this CTA reuses its shared memory
    }
}

// Zero-fill of (pointer, bytes) ranges: CTA r takes range r, r + gridDim.x, ...
struct MZero {
    void *p;
    long long bytes;
};

__global__ void __launch_bounds__(256) k_multi_zero(const MZero *__restrict__ z, int n) {
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        unsigned char *p = (unsigned char *)z[r].p;
        const long long nb = z[r].bytes;
        // the engine's buffers are 256-byte aligned blocks; word-sized fill, then the tail
        const long long nw = (((uintptr_t)p & 15) == 0) ? nb / 16 : 0;
        for (long long i = threadIdx.x; i < nw; i += blockDim.x) ((uint4 *)p)[i] = make_uint4(0u, 0u, 0u, 0u);
        for (long long i = nw * 16 + threadIdx.x; i < nb; i += blockDim.x) p[i] = 0;
    }
}

}  // namespace cmk
