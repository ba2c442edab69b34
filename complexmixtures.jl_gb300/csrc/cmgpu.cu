// cmgpu.cu -- C ABI and host orchestration of the GB300 MDDF engine.
//
// One handle = one system (solute and solvent selections, options) on one
// device.  Frames are staged into HBM in chunks (double-buffered against the
// compute stream when they come from host memory) and each frame runs a fixed
// chain of kernels on the handle's stream.  Counts accumulate in int64 half
// units per frame-weight class; a change of weight folds the class into FP64
// sums (sum += w * count / 2), so runs with one weight are exact integers.
//
// Replaces (ComplexMixtures.jl): the frame loop of mddf (src/mddf.jl:287-338),
// mddf_frame! (src/mddf.jl:361-429), coordination_number_frame!
// (src/mddf.jl:438-471) and sum! (src/results.jl:629-649).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cmgpu.h"
#include "cm_kernels.cuh"
#include "cm_atoms32.cuh"
#include "cm_agrid.cuh"
#include "cm_multi.cuh"
#include "cm_flat32.cuh"
#include "cm_final.cuh"
#include "cm_grid3d.cuh"

namespace {
// NVTX range over a host scope (header-only NVTX v3: a no-op unless a
// profiler is attached), named after the stage of the reference's frame loop
// it covers; the reference reports the same stages as progress
// (src/mddf.jl:251, 279-282).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
}  // namespace

using namespace cmk;
using cmgeom::FrameGeom;

namespace {

thread_local std::string g_create_error;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;    // size of the block
    size_t charged = 0;  // what the handle's memory budget counts: the request rounded to the allocation step
};

struct cm_error : std::exception {
    int code;
    std::string msg;
    cm_error(int c, std::string m) : code(c), msg(std::move(m)) {}
};

#define CM_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t _e = (call);                                                                       \
        if (_e != cudaSuccess)                                                                         \
            throw cm_error(CM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(_e));              \
    } while (0)

// Process-wide cache of device and pinned host blocks.  cudaFree and
// cudaFreeHost wait for the whole device, so a handle that closed (or grew a
// buffer) while other handles had work queued stalled all of them: a request
// server that opens and closes a handle per request then runs its requests
// one after the other.  Handles return their blocks here instead, and a later
// handle takes the smallest free block within 12.5 % of its request (rounded
// to the allocation step).  Blocks go back to the driver only on an
// allocation failure (then the device's free blocks are released and the
// allocation retried once) or through cm_release_cached_memory.
class BlockCache {
  public:
    static constexpr int kMaxDevices = 64;

    static size_t round_up(size_t bytes) {
        const size_t step = bytes >= (size_t(1) << 20) ? (size_t(2) << 20) : 4096;
        return (std::max<size_t>(bytes, 16) + step - 1) / step * step;
    }

    // A block of at least `bytes` (its size in *got).  `host` selects pinned
    // host memory (cudaMallocHost) instead of device memory.
    void *get(int device, bool host, size_t bytes, size_t *got) {
        const size_t want = round_up(bytes);
        {
            std::lock_guard<std::mutex> lock(mu_);
            auto &fl = list(device, host);
            auto it = fl.lower_bound(want);
            if (it != fl.end() && it->first <= want + want / 8) {
                void *p = it->second;
                *got = it->first;
                cached_[host][device] -= it->first;
                fl.erase(it);
                return p;
            }
        }
        void *p = nullptr;
        cudaError_t e = host ? cudaMallocHost(&p, want) : cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            release(device, host);
            e = host ? cudaMallocHost(&p, want) : cudaMalloc(&p, want);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                *got = 0;
                return nullptr;
            }
        }
        *got = want;
        return p;
    }

    void put(int device, bool host, void *p, size_t bytes) {
        if (!p) return;
        std::lock_guard<std::mutex> lock(mu_);
        list(device, host).emplace(bytes, p);
        cached_[host][device] += bytes;
    }

    // Return the free blocks of one device (or all devices for -1) to the driver.
    void release(int device, bool host) {
        std::multimap<size_t, void *> drop;
        {
            std::lock_guard<std::mutex> lock(mu_);
            for (int dv = 0; dv < kMaxDevices; ++dv) {
                if (device >= 0 && dv != device) continue;
                drop.insert(free_[host][dv].begin(), free_[host][dv].end());
                free_[host][dv].clear();
                cached_[host][dv] = 0;
            }
        }
        for (auto &kv : drop) {
            if (host) cudaFreeHost(kv.second);
            else cudaFree(kv.second);
        }
    }

    size_t cached(int device, bool host) {
        std::lock_guard<std::mutex> lock(mu_);
        return device >= 0 && device < kMaxDevices ? cached_[host][device] : 0;
    }

  private:
    std::multimap<size_t, void *> &list(int device, bool host) {
        if (device < 0 || device >= kMaxDevices) throw cm_error(CM_EINVAL, "device index out of range");
        return free_[host][device];
    }
    std::mutex mu_;
    std::multimap<size_t, void *> free_[2][kMaxDevices];
    size_t cached_[2][kMaxDevices] = {};
};

BlockCache &blocks() {
    static BlockCache *c = new BlockCache();  // never destroyed: blocks outlive static destructors
    return *c;
}

constexpr int kChunkSamples = 32;  // random samples placed per launch in the ATOMS regime

}  // namespace

struct cm_handle {
    // configuration
    cm_system_desc d{};
    std::vector<int64_t> gs_off, gv_off;
    std::vector<int32_t> gs_idx, gv_idx;
    int regime = CM_REGIME_PAIRS;
    int Gs = 0, Gv = 0;
    int64_t Ns = 0, Nv = 0;
    int ndist_max = 0;
    bool mddf = true;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr, copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr};
    std::string err;

    // plan
    bool planned = false;
    double pair_cell = 0.0;
    int64_t ncell_cap = 0;
    int max_frames = 64;  // frames staged per submit chunk
    int fc = 32;          // frames per compute chunk (one launch per stage)
    int coord_elem = 0;   // bytes per coordinate of the staging buffers

    // device memory
    int64_t device_bytes = 0;
    DevBuf geoms, samples, tabs, fscratch, off64, off32, hist, sums, stats, errflag, counters, slot, flags, bulk, nbulk;
    DevBuf hist_snap, stats_snap;  // accumulators before a chunk's real pass (restored if its queues overflow)
    DevBuf stage_s[2], stage_v[2];
    // PAIRS
    DevBuf scell, sq32, sq64, so32, so64, vcell, vq32, vq64, vo32, vo64, ccount, cstart, cfill, cmol, cq32, gq, rq, eq;
    int gq_cap = 0, rq_cap = 0;
    int flat_ctas = 0;  // resident CTAs per SM of k_pairs_flat32
    int tile_ctas = 0;  // resident CTAs per SM of k_pairs_tile32 (self mode)
    int guard_ctas = 1, edge_ctas = 1, rand_ctas = 1, real_ctas = 1;  // ... of the guard, edge, random and generic kernels
    // group tables
    DevBuf g_soff, g_sidx, g_voff, g_vidx;
    // ATOMS
    DevBuf akey, atq32, atq64, asq32, asq64, acount, astart, afill, avcell, avq32, avq64, u64, u32, rc, pcell, pq32, pq64,
        anear, aq, aslot;
    int aq_cap = 0;
    int aslot_cap = 0;     // random-insertion slot list (slots of one placement piece)
    int atoms_ctas = 0;    // resident CTAs per SM of k_atoms_eval
    bool atoms_dense = true; // ATOMS evaluation schedule: dense solutes (many atoms per occupied cell) or sparse
    int atoms_piece = 0;   // samples placed per random-insertion launch
    // candidate grid of a single solute molecule (FP32): agk fine cells per
    // search-cell axis (0: none), gcap entries per frame
    DevBuf gstart, gedge, gpool, gent;
    int agk = 0;
    int64_t gcap = 0;
    int agrid_real_ctas = 1, agrid_rand_ctas = 1;  // resident CTAs per SM of k_agrid_real / k_agrid_random
    // pinned host staging
    FrameGeom *h_geoms[2] = {nullptr, nullptr};
    Sample *h_samples[2] = {nullptr, nullptr};
    int4 *h_tabs[2] = {nullptr, nullptr};
    int64_t h_samples_cap = 0;
    std::vector<DevBuf> host_blocks;  // the pinned blocks above, as taken from the block cache

    // accumulation state
    bool class_open = false;
    double class_w = 1.0;
    int64_t folds = 0;
    double volume_total = 0.0, weight_total = 0.0;
    int64_t frames = 0;
    int64_t hist_n = 0;
    int64_t o_md, o_mdr, o_rdf, o_rdfr, o_gs, o_gsr, o_gv, o_gvr;
    int smem_groups = 0;
    double last_guard = 0.0;
    int kernels_per_frame = 0;
    int chunk_parity = 0;

    // raw DCD frames (cm_set_dcd_layout)
    bool dcd = false;
    int64_t dcd_natoms = 0, dcd_frame_bytes = 0, dcd_off[3] = {0, 0, 0};
    int dcd_swap = 0;
    std::vector<int32_t> dcd_s, dcd_v;  // host copies of the selections' atom indices
    DevBuf dcd_sidx, dcd_vidx, dcd_raw[2];
    DevBuf final_out, final_job;  // cm_read_results
    DevBuf contrib_q, contrib_g, contrib_out;  // cm_contributions

    // CUDA-graph launch of compute chunks
    bool graphs = false;
    cudaGraphExec_t gexec = nullptr;
    int64_t graph_launches = 0, graph_instantiations = 0;

    // launch accounting and optional per-launch event timing
    int64_t launches_total = 0;
    int64_t class_launches[CM_K_NCLASSES] = {};
    double class_ms[CM_K_NCLASSES] = {};
    bool timing = false;
    std::vector<cudaEvent_t> ev_free;
    struct Pending {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    cudaEvent_t cur_start = nullptr;
    int cur_class = 0;
};

namespace {

// Wait for the handle's own queued work (not the device's), so that its
// blocks can go back to the cache.
void quiesce(cm_handle *h) {
    if (h->stream) CM_CUDA(cudaStreamSynchronize(h->stream));
    if (h->copy_stream) CM_CUDA(cudaStreamSynchronize(h->copy_stream));
}

void dev_alloc(cm_handle *h, DevBuf &b, size_t bytes) {
    if (b.bytes >= bytes && b.p) return;
    if (b.p) {
        quiesce(h);  // queued kernels of this handle may still read the old block
        blocks().put(h->device, false, b.p, b.bytes);
        h->device_bytes -= (int64_t)b.charged;
        b.p = nullptr;
        b.bytes = b.charged = 0;
    }
    const size_t want = BlockCache::round_up(bytes);
    if (h->d.hbm_budget_bytes > 0 && h->device_bytes + (int64_t)want > h->d.hbm_budget_bytes)
        throw cm_error(CM_ENOMEM, "device memory budget exceeded (" + std::to_string(h->device_bytes + (int64_t)want) +
                                      " > " + std::to_string(h->d.hbm_budget_bytes) + " bytes)");
    size_t got = 0;
    b.p = blocks().get(h->device, false, bytes, &got);
    if (!b.p) throw cm_error(CM_ENOMEM, "cudaMalloc(" + std::to_string(want) + "): out of device memory");
    b.bytes = got;
    b.charged = want;  // independent of which cached block was reused
    h->device_bytes += (int64_t)want;
}

// Pinned host staging from the block cache.
template <typename T>
void host_alloc(cm_handle *h, T *&p, size_t bytes) {
    size_t got = 0;
    p = static_cast<T *>(blocks().get(h->device, true, bytes, &got));
    if (!p) throw cm_error(CM_ENOMEM, "cudaMallocHost(" + std::to_string(bytes) + "): out of pinned host memory");
    h->host_blocks.push_back({(void *)p, got});
}

template <typename T>
T *P(DevBuf &b) {
    return reinterpret_cast<T *>(b.p);
}

// ----------------------------------------------------------------- geometry
void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
double dot3(const double *a, const double *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

// Geometry of one frame with a grid of target cell side `cs`.
void frame_geometry(const double *H, double cs, int ncap_axis, FrameGeom &G) {
    memcpy(G.H, H, 9 * sizeof(double));
    const double *a = H, *b = H + 3, *c = H + 6;
    double ab[3], bc[3], ca[3];
    cross3(a, b, ab);
    cross3(b, c, bc);
    cross3(c, a, ca);
    G.det = dot3(ab, c);
    if (!(std::fabs(G.det) > 0.0) || !std::isfinite(G.det)) throw cm_error(CM_EINVAL, "degenerate unit cell (zero volume)");
    for (int m = 0; m < 3; ++m) {
        G.Hi[0 + m] = bc[m] / G.det;
        G.Hi[3 + m] = ca[m] / G.det;
        G.Hi[6 + m] = ab[m] / G.det;
    }
    double V = std::fabs(G.det);
    G.w[0] = V / std::sqrt(dot3(bc, bc));
    G.w[1] = V / std::sqrt(dot3(ca, ca));
    G.w[2] = V / std::sqrt(dot3(ab, ab));
    G.hw = 0.5 * std::fmin(G.w[0], std::fmin(G.w[1], G.w[2]));
    G.hortho = (H[1] == 0.0 && H[2] == 0.0 && H[3] == 0.0 && H[5] == 0.0 && H[6] == 0.0 && H[7] == 0.0) ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
        int n = (int)std::floor(G.w[k] / cs);
        if (n < 1) n = 1;
        if (n > ncap_axis) n = ncap_axis;
        G.n[k] = n;
        G.cw[k] = G.w[k] / n;
        for (int m = 0; m < 3; ++m) G.Hn[3 * k + m] = H[3 * k + m] / (double)n;
    }
    G.ncell = G.n[0] * G.n[1] * G.n[2];
}

// Largest distance of an atom to its molecule's centroid (molecule made whole
// around its first atom by minimum image); sizes the PAIRS cells on the host.
double centroid_radius(const double *xyz, int nmol, int apm, const double *H) {
    FrameGeom G;
    frame_geometry(H, 1e30, 1, G);
    double r = 0.0;
    std::vector<double> d(3 * (size_t)apm);
    for (int m = 0; m < nmol; ++m) {
        const double *x0 = xyz + (int64_t)m * apm * 3;
        double c[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < apm; ++a) {
            double *e = &d[3 * (size_t)a];
            for (int k = 0; k < 3; ++k) e[k] = x0[3 * a + k] - x0[k];
            cmgeom::unwrap(G, e);
            for (int k = 0; k < 3; ++k) c[k] += e[k];
        }
        for (int a = 0; a < apm; ++a) {
            double *e = &d[3 * (size_t)a];
            double dx = e[0] - c[0] / apm, dy = e[1] - c[1] / apm, dz = e[2] - c[2] / apm;
            r = std::max(r, std::sqrt(dx * dx + dy * dy + dz * dz));
        }
    }
    return r;
}

void check_desc(const cm_system_desc *d) {
    auto bad = [](const std::string &m) { throw cm_error(CM_EINVAL, m); };
    if (!d) bad("NULL system description");
    if (d->api_version != CM_API_VERSION) bad("api_version mismatch");
    if (d->launch < CM_LAUNCH_AUTO || d->launch > CM_LAUNCH_GRAPH) bad("unknown launch mode");
    if (d->atoms_schedule < CM_SCHED_AUTO || d->atoms_schedule > CM_SCHED_BALANCED) bad("unknown atoms_schedule");
    if (d->guard_queue_capacity < 0) bad("guard_queue_capacity must be >= 0");
    if (d->real_pass < CM_REAL_AUTO || d->real_pass > CM_REAL_TILE) bad("unknown real_pass");
    if (d->atoms_grid < -1 || d->atoms_grid > kAgridMaxK) bad("atoms_grid must be -1, 0 or 1-" + std::to_string(kAgridMaxK));
    if (d->atoms_grid_capacity < 0) bad("atoms_grid_capacity must be >= 0");
    if (d->solute_nmols < 1 || d->solute_natomspermol < 1 || d->solvent_nmols < 1 || d->solvent_natomspermol < 1)
        bad("selections must have at least one molecule of at least one atom");
    if (d->autocorrelation && (d->solute_nmols != d->solvent_nmols || d->solute_natomspermol != d->solvent_natomspermol))
        bad("autocorrelation requires identical solute and solvent selections");
    if (d->irefatom < 1 || d->irefatom > d->solvent_natomspermol)
        bad("Reference atom index " + std::to_string(d->irefatom) + " is greater than number of atoms of the solvent molecule.");
    if (!(d->binstep > 0.0) || !(d->cutoff > 0.0) || !(d->dbulk > 0.0)) bad("cutoff, dbulk and binstep must be positive");
    if (d->usecutoff && d->dbulk >= d->cutoff) bad("The bulk volume is zero (dbulk must be smaller than cutoff).");
    double cut = d->usecutoff ? d->cutoff : d->dbulk;
    int need = std::max(1, (int)std::ceil(cut / d->binstep));
    if (d->nbins < need) bad("nbins is smaller than setbin(cutoff, binstep)");
    if (d->n_random_samples < 0) bad("n_random_samples must be >= 0");
    if (d->mode == CM_MODE_MDDF && d->n_random_samples < 1) bad("n_random_samples must be greater than 0.");
    if (d->mode != CM_MODE_MDDF && d->mode != CM_MODE_COORDINATION_NUMBER) bad("unknown mode");
    if (d->precision != CM_PRECISION_FP64 && d->precision != CM_PRECISION_FP32_GUARD) bad("unknown precision");
    if (d->regime < CM_REGIME_AUTO || d->regime > CM_REGIME_ATOMS) bad("unknown regime");
    if (d->lcell < 1) bad("lcell must be >= 1");
    if (d->cell_scale_pct != 0 && (d->cell_scale_pct < 30 || d->cell_scale_pct > 300))
        bad("cell_scale_pct must be 0 or within 30-300");
    int64_t Nv = (int64_t)d->solvent_nmols * d->solvent_natomspermol;
    int64_t Ns = (int64_t)d->solute_nmols * d->solute_natomspermol;
    if (Ns >= (1LL << 31) || Nv >= (1LL << 31)) bad("selections above 2^31 atoms are not supported");
    if ((d->solute_group_offsets == nullptr) != (d->solute_groups == nullptr) ||
        (d->solvent_group_offsets == nullptr) != (d->solvent_groups == nullptr))
        bad("group CSR needs both offsets and indices");
    if (d->solute_group_offsets && d->solute_ngroups < 1) bad("solute_ngroups must be >= 1 with custom groups");
    if (d->solvent_group_offsets && d->solvent_ngroups < 1) bad("solvent_ngroups must be >= 1 with custom groups");
}

void copy_csr(int64_t natoms, int ngroups, const int64_t *off, const int32_t *idx, std::vector<int64_t> &o,
              std::vector<int32_t> &ix, const char *what) {
    o.assign(off, off + natoms + 1);
    if (o[0] != 0) throw cm_error(CM_EINVAL, std::string(what) + " group offsets must start at 0");
    for (int64_t i = 0; i < natoms; ++i)
        if (o[i + 1] < o[i]) throw cm_error(CM_EINVAL, std::string(what) + " group offsets must be non-decreasing");
    ix.assign(idx, idx + o[natoms]);
    for (int32_t g : ix)
        if (g < 0 || g >= ngroups) throw cm_error(CM_EINVAL, std::string(what) + " group index out of range");
}

DevSys make_devsys(cm_handle *h) {
    DevSys S{};
    const cm_system_desc &d = h->d;
    S.ms = d.solute_nmols;
    S.aps = d.solute_natomspermol;
    S.mv = d.solvent_nmols;
    S.apv = d.solvent_natomspermol;
    S.self = d.autocorrelation ? 1 : 0;
    S.iref = d.irefatom - 1;
    S.nbins = d.nbins;
    S.nrs = h->mddf ? d.n_random_samples : 0;
    S.fp32 = d.precision == CM_PRECISION_FP32_GUARD;
    S.usecutoff = d.usecutoff ? 1 : 0;
    S.Gs = h->Gs;
    S.Gv = h->Gv;
    S.default_s = h->gs_off.empty() ? 1 : 0;
    S.default_v = h->gv_off.empty() ? 1 : 0;
    S.smem_groups = h->smem_groups;
    S.cut = d.usecutoff ? d.cutoff : d.dbulk;  // src/minimum_distances.jl:166
    S.cut2 = S.cut * S.cut;
    S.binstep = d.binstep;
    S.dbulk = d.dbulk;
    S.seed = d.seed;
    S.gs_off = nullptr;
    S.gs_idx = nullptr;
    S.gv_off = nullptr;
    S.gv_idx = nullptr;
    S.hist = P<unsigned long long>(h->hist);
    S.o_md = h->o_md; S.o_mdr = h->o_mdr; S.o_rdf = h->o_rdf; S.o_rdfr = h->o_rdfr;
    S.o_gs = h->o_gs; S.o_gsr = h->o_gsr; S.o_gv = h->o_gv; S.o_gvr = h->o_gvr;
    S.stats = P<unsigned long long>(h->stats);
    S.err = P<int>(h->errflag);
    return S;
}

size_t hist_smem_bytes(const cm_handle *h, int smem_groups) {
    int words = h->d.nbins * (2 + (smem_groups ? (h->Gs + (h->d.autocorrelation ? 0 : h->Gv)) : 0));
    return ((size_t)words * 4 + 15) & ~(size_t)15;
}

}  // namespace

namespace {

DevSys devsys_full(cm_handle *h) {
    DevSys S = make_devsys(h);
    if (!h->gs_off.empty()) {
        S.gs_off = P<int64_t>(h->g_soff);
        S.gs_idx = P<int32_t>(h->g_sidx);
    }
    if (!h->gv_off.empty()) {
        S.gv_off = P<int64_t>(h->g_voff);
        S.gv_idx = P<int32_t>(h->g_vidx);
    }
    return S;
}

void upload_groups(cm_handle *h) {
    auto up = [&](DevBuf &b, const void *src, size_t bytes) {
        dev_alloc(h, b, bytes);
        // on the handle's stream: the caller's next stream sync covers the copy
        if (bytes) CM_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, h->stream));
    };
    if (!h->gs_off.empty()) {
        up(h->g_soff, h->gs_off.data(), h->gs_off.size() * 8);
        up(h->g_sidx, h->gs_idx.data(), std::max<size_t>(h->gs_idx.size() * 4, 4));
    }
    if (!h->gv_off.empty()) {
        up(h->g_voff, h->gv_off.data(), h->gv_off.size() * 8);
        up(h->g_vidx, h->gv_idx.data(), std::max<size_t>(h->gv_idx.size() * 4, 4));
    }
}

// Search-cell side: PAIRS the molecule cell (cutoff + both radii, with a
// margin), ATOMS cutoff / lcell; both scaled by cell_scale_pct.
double target_cell(const cm_handle *h) {
    double cut = h->d.usecutoff ? h->d.cutoff : h->d.dbulk;
    const double scale = (h->d.cell_scale_pct > 0 ? h->d.cell_scale_pct : 100) / 100.0;
    if (h->regime == CM_REGIME_ATOMS) return cut / h->d.lcell * (1.0 + 1e-6) * scale;
    return h->pair_cell * scale;
}

// Per-CTA shared memory of the PAIRS real-pass kernels beyond the histograms.
size_t pairs_extra_smem() {
    const size_t real = (size_t)kWarps * kMaxSmallMol * 16 + (size_t)kWarps * kQueue * 8;
    const size_t flat = (size_t)kFlatWarps * flat_warp_smem();
    const size_t tile = (size_t)kTileWarps * flat_warp_smem() + tile_smem_extra();
    return std::max(real, std::max(flat, tile));
}

// The FP32 real-pass kernel for a system: specialised on the solute molecule
// size for the common sizes, generic otherwise.
// The tiled kernel (self mode) is launched first; the per-molecule kernel then
// takes the frames it did not (skip = 1), or every frame (skip = 0).
using FlatLaunch = void (*)(int, size_t, cudaStream_t, const DevSys &, const Bufs &, int);
using TileLaunch = void (*)(int, size_t, cudaStream_t, const DevSys &, const Bufs &);
struct FlatKernel {
    const void *fn;
    FlatLaunch launch;
    const void *tile_fn;  // nullptr in cross mode
    TileLaunch tile_launch;
};

template <bool SELF, int APS>
void launch_flat(int grid, size_t smem, cudaStream_t st, const DevSys &S, const Bufs &B, int skip_tile) {
    k_pairs_flat32<SELF, APS><<<grid, kFlatWarps * 32, smem, st>>>(S, B, skip_tile);
}

template <int APS>
void launch_tile(int grid, size_t smem, cudaStream_t st, const DevSys &S, const Bufs &B) {
    k_pairs_tile32<APS><<<grid, kTileWarps * 32, smem, st>>>(S, B);
}

template <bool SELF, int APS>
FlatKernel flat_kernel_for() {
    if (SELF)
        return {(const void *)k_pairs_flat32<SELF, APS>, launch_flat<SELF, APS>, (const void *)k_pairs_tile32<APS>,
                launch_tile<APS>};
    return {(const void *)k_pairs_flat32<SELF, APS>, launch_flat<SELF, APS>, nullptr, nullptr};
}

template <bool SELF>
FlatKernel flat_kernel_of(int aps) {
    switch (aps) {
        case 1: return flat_kernel_for<SELF, 1>();
        case 3: return flat_kernel_for<SELF, 3>();
        case 4: return flat_kernel_for<SELF, 4>();
        case 5: return flat_kernel_for<SELF, 5>();
        case 14: return flat_kernel_for<SELF, 14>();
        default: return flat_kernel_for<SELF, 0>();
    }
}

FlatKernel flat_kernel(const cm_handle *h) {
    return h->d.autocorrelation ? flat_kernel_of<true>(h->d.solute_natomspermol)
                                : flat_kernel_of<false>(h->d.solute_natomspermol);
}

// Shared memory one CTA of the system's kernels needs at most; fails when
// it is beyond the device's opt-in limit (very many histogram bins).
void check_smem(const cm_handle *h, size_t need) {
    int optin = 0;
    CM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
    if (need > (size_t)optin)
        throw cm_error(CM_EINVAL, "the histograms need " + std::to_string(need) +
                                      " bytes of shared memory per block, more than the device's " +
                                      std::to_string(optin) + " (use fewer bins)");
}

// Resident CTAs per SM of a kernel at a launch shape: the persistent
// (grid-stride) kernels launch that many per SM, so they run in one wave.
int resident_ctas(const void *fn, int threads, size_t smem) {
    int n = 0;
    CM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem));
    return std::max(1, n);
}

// Resident CTAs per SM of the PAIRS kernels: the FP32 real pass (returned)
// and the guard, edge, random-evaluation and generic kernels (kept in h).
int flat_setup(cm_handle *h) {
    const size_t hsm = hist_smem_bytes(h, h->smem_groups);
    const bool self = h->d.autocorrelation, fp32 = h->d.precision == CM_PRECISION_FP32_GUARD;
    h->guard_ctas = resident_ctas(self ? (const void *)k_pairs_guard<true> : (const void *)k_pairs_guard<false>,
                                  kGuardWarps * 32, hsm);
    h->edge_ctas = resident_ctas(self ? (const void *)k_pairs_edge<true> : (const void *)k_pairs_edge<false>, 128, hsm);
    h->rand_ctas = resident_ctas(fp32 ? (const void *)k_random_eval<true> : (const void *)k_random_eval<false>, 128, hsm);
    const void *real = fp32 ? (self ? (const void *)k_pairs_real<true, true> : (const void *)k_pairs_real<true, false>)
                            : (self ? (const void *)k_pairs_real<false, true> : (const void *)k_pairs_real<false, false>);
    h->real_ctas = resident_ctas(real, kWarps * 32, hsm + (size_t)kWarps * kMaxSmallMol * 16 + (size_t)kWarps * kQueue * 8);
    const FlatKernel fk = flat_kernel(h);
    h->tile_ctas = fk.tile_fn ? resident_ctas(fk.tile_fn, kTileWarps * 32,
                                              hsm + (size_t)kTileWarps * flat_warp_smem() + tile_smem_extra())
                              : 0;
    return resident_ctas(fk.fn, kFlatWarps * 32, hsm + (size_t)kFlatWarps * flat_warp_smem());
}

// The ATOMS evaluation kernels of a system (precision x schedule).
using AtomsLaunch = void (*)(int, size_t, cudaStream_t, const DevSys &, const Bufs &);
struct AtomsKernels {
    const void *fn, *fn_random;
    AtomsLaunch real, random;
};

template <bool FP32, bool RANDOM, int SCHED>
void launch_atoms(int grid, size_t smem, cudaStream_t st, const DevSys &S, const Bufs &B) {
    k_atoms_eval<FP32, RANDOM, SCHED><<<grid, kAtomsWarps * 32, smem, st>>>(S, B);
}

template <bool FP32, int SCHED>
AtomsKernels atoms_kernels_of() {
    return {(const void *)k_atoms_eval<FP32, false, SCHED>, (const void *)k_atoms_eval<FP32, true, SCHED>,
            launch_atoms<FP32, false, SCHED>, launch_atoms<FP32, true, SCHED>};
}

// Dense solutes: a warp over each cell's atoms; sparse: the balanced warp
// walk in FP32, a thread per entry in FP64.
AtomsKernels atoms_kernels(const cm_handle *h) {
    const bool fp32 = h->d.precision == CM_PRECISION_FP32_GUARD;
    if (fp32) return h->atoms_dense ? atoms_kernels_of<true, kSchedCell>() : atoms_kernels_of<true, kSchedBalanced>();
    return h->atoms_dense ? atoms_kernels_of<false, kSchedCell>() : atoms_kernels_of<false, kSchedThread>();
}

// The dynamic shared-memory limit of a kernel is a property of the function
// shared by every handle of the process, so it is raised once per device to
// the opt-in maximum (less the kernel's static shared memory) for every kernel
// that takes dynamic shared memory; each launch then asks for what its system
// needs, and handles with different needs never lower one another's limit.
std::mutex g_smem_mu;
bool g_smem_done[64] = {};

void kernel_smem_limits(int device) {
    std::lock_guard<std::mutex> lock(g_smem_mu);
    if (device < 0 || device >= 64) throw cm_error(CM_EINVAL, "device index out of range");
    if (g_smem_done[device]) return;
    int optin = 0;
    CM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    auto raise = [&](const void *fn) {
        cudaFuncAttributes fa;
        CM_CUDA(cudaFuncGetAttributes(&fa, fn));
        CM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    };
    raise((const void *)k_pairs_real<true, true>);
    raise((const void *)k_pairs_real<true, false>);
    raise((const void *)k_pairs_real<false, true>);
    raise((const void *)k_pairs_real<false, false>);
    raise((const void *)k_random_eval<true>);
    raise((const void *)k_random_eval<false>);
    for (const AtomsKernels &k : {atoms_kernels_of<true, kSchedCell>(), atoms_kernels_of<true, kSchedBalanced>(),
                                  atoms_kernels_of<false, kSchedCell>(), atoms_kernels_of<false, kSchedThread>()}) {
        raise(k.fn);
        raise(k.fn_random);
    }
    raise((const void *)k_pairs_guard<true>);
    raise((const void *)k_pairs_guard<false>);
    raise((const void *)k_pairs_edge<true>);
    raise((const void *)k_pairs_edge<false>);
    raise((const void *)k_agrid_real);
    raise((const void *)k_agrid_random);
    raise((const void *)k_agrid_build);
    raise((const void *)k_multi<MK_AGRID_BUILD>);
    raise((const void *)k_multi<MK_AGRID_REAL>);
    raise((const void *)k_multi<MK_AGRID_RANDOM>);
    raise((const void *)k_multi<MK_EVAL_REAL_CELL>);
    raise((const void *)k_multi<MK_EVAL_RANDOM_CELL>);
    raise((const void *)k_multi<MK_EVAL_REAL_BALANCED>);
    raise((const void *)k_multi<MK_EVAL_RANDOM_BALANCED>);
    for (int aps : {0, 1, 3, 4, 5, 14}) {
        raise(flat_kernel_of<true>(aps).fn);
        raise(flat_kernel_of<true>(aps).tile_fn);
        raise(flat_kernel_of<false>(aps).fn);
    }
    g_smem_done[device] = true;
}

// Resident CTAs per SM of the ATOMS evaluation kernel.
int atoms_setup(cm_handle *h) {
    const size_t smem = hist_smem_bytes(h, h->smem_groups);
    int n = 0;
    CM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, atoms_kernels(h).fn, kAtomsWarps * 32, smem));
    return std::max(1, n);
}

// Mean solute atoms per occupied search cell in the first frame: lanes over
// each cell's atoms pay off when the cells hold about a warp's worth of atoms
// or more; sparse solutes (chains spread through the box) take the balanced
// walk (FP32) or a thread per queued pair (FP64).
bool atoms_dense(const cm_handle *h, const cm_frames *f) {
    const int64_t n = h->Ns;
    std::vector<double> x(n * 3);
    std::vector<char> raw(n * 3 * h->coord_elem);
    if (f->memory == CM_MEM_DEVICE) CM_CUDA(cudaMemcpy(raw.data(), f->solute_xyz, raw.size(), cudaMemcpyDeviceToHost));
    else memcpy(raw.data(), f->solute_xyz, raw.size());
    for (int64_t i = 0; i < n * 3; ++i)
        x[i] = h->coord_elem == 4 ? (double)reinterpret_cast<float *>(raw.data())[i] : reinterpret_cast<double *>(raw.data())[i];
    FrameGeom G;
    memset(&G, 0, sizeof(G));
    frame_geometry(f->cells, target_cell(h), 1023, G);
    const int aps = h->d.solute_natomspermol;
    std::vector<int64_t> keys(n);
    for (int64_t i = 0; i < n; ++i) {
        int c[3];
        double q[3];
        cmgeom::bin_position(G, x[3 * i], x[3 * i + 1], x[3 * i + 2], c, q);
        keys[i] = (i / aps) * (int64_t)G.ncell + cmgeom::cell_linear(G, c[0], c[1], c[2]);
    }
    std::sort(keys.begin(), keys.end());
    const int64_t occupied = std::unique(keys.begin(), keys.end()) - keys.begin();
    return (double)n / (double)std::max<int64_t>(1, occupied) >= 64.0;
}

// Reallocate the per-frame cell arrays of a compute chunk if a frame needs
// more cells than planned.
void ensure_cells(cm_handle *h, int64_t ncell) {
    if (ncell <= h->ncell_cap) return;
    h->ncell_cap = ncell;
    if (h->regime == CM_REGIME_PAIRS) {
        const size_t n = (size_t)h->fc * (ncell + 1) * 4;
        dev_alloc(h, h->ccount, n);
        dev_alloc(h, h->cstart, n);
        dev_alloc(h, h->cfill, n);
    } else {
        const size_t n = (size_t)h->fc * ((int64_t)h->d.solute_nmols * ncell + 1);
        dev_alloc(h, h->acount, n * 4);
        dev_alloc(h, h->astart, n * 4);
        dev_alloc(h, h->afill, n * 4);
        dev_alloc(h, h->anear, n);
        if (h->agk > 0) {
            const int64_t k3 = (int64_t)h->agk * h->agk * h->agk;
            dev_alloc(h, h->gstart, (size_t)h->fc * ncell * k3 * (kAgridBuckets + 1) * 4);
            dev_alloc(h, h->gedge, (size_t)h->fc * ncell * k3 * sizeof(float2));
            dev_alloc(h, h->gpool, (size_t)h->fc * 4);
        }
    }
}

void plan(cm_handle *h, const cm_frames *f) {
    const cm_system_desc &d = h->d;
    h->coord_elem = f->coord_type == CM_COORD_F32 ? 4 : 8;
    CM_CUDA(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device));
    // molecule radii of the first frame size the PAIRS cells
    if (h->regime == CM_REGIME_PAIRS) {
        std::vector<double> xs, xv;
        auto fetch = [&](const void *src, int64_t n, std::vector<double> &out) {
            out.resize(n * 3);
            std::vector<char> raw(n * 3 * h->coord_elem);
            if (f->memory == CM_MEM_DEVICE) CM_CUDA(cudaMemcpy(raw.data(), src, raw.size(), cudaMemcpyDeviceToHost));
            else memcpy(raw.data(), src, raw.size());
            for (int64_t i = 0; i < n * 3; ++i)
                out[i] = h->coord_elem == 4 ? (double)reinterpret_cast<float *>(raw.data())[i] : reinterpret_cast<double *>(raw.data())[i];
        };
        fetch(f->solute_xyz, h->Ns, xs);
        double rs = centroid_radius(xs.data(), d.solute_nmols, d.solute_natomspermol, f->cells);
        double rv = rs;
        if (!d.autocorrelation) {
            fetch(f->solvent_xyz, h->Nv, xv);
            rv = centroid_radius(xv.data(), d.solvent_nmols, d.solvent_natomspermol, f->cells);
        }
        const double cut = d.usecutoff ? d.cutoff : d.dbulk;
        h->pair_cell = (cut + rs + rv) * 1.05 + 0.25;
    }
    h->max_frames = d.max_frames_per_batch > 0 ? d.max_frames_per_batch : 64;
    // keep the per-chunk sample table bounded (n_random_samples can be 10^5)
    if (h->mddf && (int64_t)h->max_frames * d.n_random_samples > (1 << 22))
        h->max_frames = (int)std::max<int64_t>(1, (1 << 22) / std::max(1, d.n_random_samples));
    h->fc = std::min(h->max_frames, 32);
    const int fc = h->fc;
    const int64_t ms = d.solute_nmols, mv = d.solvent_nmols;

    // staging of geometries, samples and bulk tables (two chunks in flight)
    dev_alloc(h, h->geoms, sizeof(FrameGeom) * h->max_frames * 2);
    for (int i = 0; i < 2; ++i) host_alloc(h, h->h_geoms[i], sizeof(FrameGeom) * h->max_frames);
    if (h->mddf) {
        h->h_samples_cap = (int64_t)h->max_frames * d.n_random_samples;
        dev_alloc(h, h->samples, sizeof(Sample) * h->h_samples_cap * 2);
        dev_alloc(h, h->tabs, sizeof(int4) * (size_t)h->max_frames * h->ndist_max * 2);
        for (int i = 0; i < 2; ++i) {
            host_alloc(h, h->h_samples[i], sizeof(Sample) * h->h_samples_cap);
            host_alloc(h, h->h_tabs[i], sizeof(int4) * (size_t)h->max_frames * h->ndist_max);
        }
    }
    if (f->memory == CM_MEM_HOST) {
        for (int i = 0; i < 2; ++i) {
            dev_alloc(h, h->stage_s[i], (size_t)h->max_frames * h->Ns * 3 * h->coord_elem);
            if (!d.autocorrelation) dev_alloc(h, h->stage_v[i], (size_t)h->max_frames * h->Nv * 3 * h->coord_elem);
        }
    }
    // per-frame buffers of one compute chunk
    dev_alloc(h, h->fscratch, sizeof(FrameScratch) * fc);
    dev_alloc(h, h->off64, sizeof(d4) * cmgeom::kOffEntries * fc);
    dev_alloc(h, h->off32, sizeof(float4) * cmgeom::kOffEntries * fc);
    dev_alloc(h, h->counters, 8 * sizeof(int));
    if (h->mddf) {
        const int nd = h->ndist_max;
        dev_alloc(h, h->slot, (size_t)fc * ms * 4);
        CM_CUDA(cudaMemsetAsync(h->slot.p, 0xff, (size_t)fc * ms * 4, h->stream));
        dev_alloc(h, h->flags, (size_t)fc * nd * mv);
        dev_alloc(h, h->bulk, (size_t)fc * nd * mv * 4);
        dev_alloc(h, h->nbulk, (size_t)fc * nd * 4);
    }
    if (h->regime == CM_REGIME_PAIRS) {
        dev_alloc(h, h->scell, fc * ms * 4);
        dev_alloc(h, h->sq32, fc * ms * 16);
        dev_alloc(h, h->sq64, fc * ms * 32);
        dev_alloc(h, h->so32, fc * h->Ns * 16);
        dev_alloc(h, h->so64, fc * h->Ns * 32);
        if (!d.autocorrelation) {
            dev_alloc(h, h->vcell, fc * mv * 4);
            dev_alloc(h, h->vq32, fc * mv * 16);
            dev_alloc(h, h->vq64, fc * mv * 32);
            dev_alloc(h, h->vo32, fc * h->Nv * 16);
            dev_alloc(h, h->vo64, fc * h->Nv * 32);
        }
        dev_alloc(h, h->cmol, fc * mv * 4);
        dev_alloc(h, h->cq32, fc * mv * 16);
        // guard queue of a chunk: every candidate fits when the system is small
        // (candidates <= ms * mv per frame); otherwise 64 per solute molecule and
        // frame, far above the guard-band rate
        const int64_t bound = ms * mv * fc;
        h->gq_cap = (int)(bound <= (1LL << 24) ? std::max<int64_t>(bound, 1024)
                                               : std::min<int64_t>(std::max<int64_t>(1 << 20, 64 * ms * fc), 1LL << 25));
        if (d.guard_queue_capacity > 0) h->gq_cap = d.guard_queue_capacity;
        dev_alloc(h, h->gq, (size_t)h->gq_cap * sizeof(int4));
        dev_alloc(h, h->eq, (size_t)h->gq_cap * 3 * sizeof(int4));
        if (h->mddf) {
            // random-insertion queue: every slot of `chunk` samples fits
            const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>((int64_t)fc * d.n_random_samples, (1 << 23) / mv));
            h->rq_cap = (int)(chunk * mv);
            dev_alloc(h, h->rq, (size_t)h->rq_cap * sizeof(int2));
        }
    } else {
        dev_alloc(h, h->akey, fc * h->Ns * 4);
        dev_alloc(h, h->atq32, fc * h->Ns * 16);
        dev_alloc(h, h->atq64, fc * h->Ns * 32);
        dev_alloc(h, h->asq32, fc * h->Ns * 16);
        dev_alloc(h, h->asq64, fc * h->Ns * 32);
        dev_alloc(h, h->avcell, fc * h->Nv * 4);
        dev_alloc(h, h->avq32, fc * h->Nv * 16);
        dev_alloc(h, h->avq64, fc * h->Nv * 32);
        if (h->mddf) {
            dev_alloc(h, h->u64, fc * h->Nv * 32);
            dev_alloc(h, h->u32, fc * h->Nv * 16);
            dev_alloc(h, h->rc, fc * mv * 4);
            // the work queue holds every slot of the samples placed in one launch
            const int64_t want = std::min<int64_t>((int64_t)kChunkSamples * mv, std::max<int64_t>(1 << 22, mv));
            h->atoms_piece = (int)std::max<int64_t>(1, std::min<int64_t>(kChunkSamples, want / mv));
            const int chunk = std::min(h->atoms_piece, std::max(1, fc * d.n_random_samples));
            dev_alloc(h, h->pcell, (size_t)chunk * h->Nv * 4);
            h->aslot_cap = (int)std::min<int64_t>((int64_t)chunk * mv, (int64_t)INT32_MAX);
            dev_alloc(h, h->aslot, (size_t)h->aslot_cap * 4);
            dev_alloc(h, h->pq32, (size_t)chunk * h->Nv * 16);
            dev_alloc(h, h->pq64, (size_t)chunk * h->Nv * 32);
        }
    }
    if (h->regime == CM_REGIME_ATOMS) {
        // real pass: (frame, solute molecule, solvent molecule) items in
        // pieces of the queue's capacity
        const int64_t items = (int64_t)fc * ms * mv;
        h->aq_cap = (int)std::max<int64_t>(std::min<int64_t>(std::max<int64_t>(items, (int64_t)h->atoms_piece * mv), 1 << 25),
                                           (int64_t)h->atoms_piece * mv);
        dev_alloc(h, h->aq, (size_t)h->aq_cap * sizeof(int4));
    }
    // histogram shared-memory plan
    // (the ATOMS evaluation's window tables are static shared memory)
    const size_t extra = h->regime == CM_REGIME_PAIRS ? pairs_extra_smem() : sizeof(float4) * 32 * kAtomsWarps;
    h->smem_groups = hist_smem_bytes(h, 1) + extra + 2048 <= 160 * 1024 ? 1 : 0;
    kernel_smem_limits(h->device);
    check_smem(h, hist_smem_bytes(h, h->smem_groups) + extra);
    if (h->regime == CM_REGIME_PAIRS) h->flat_ctas = flat_setup(h);
    else {
        const bool dense = atoms_dense(h, f);
        h->atoms_dense = h->d.atoms_schedule == CM_SCHED_AUTO ? dense : h->d.atoms_schedule == CM_SCHED_CELL;
        h->atoms_ctas = atoms_setup(h);
        // candidate grid of a single solute molecule in the FP32 search (the
        // plain FP64 path keeps the walk): by default for dense solutes, whose
        // stencils hold many atoms per query, with fine cells of about 2.5 A.
        // The fallback of a frame whose lists overflow queues its near pairs,
        // so every item of a chunk must fit the queue.
        h->agk = 0;
        const bool fp32 = d.precision == CM_PRECISION_FP32_GUARD;
        // a query is one thread per solvent molecule over its sites, so the
        // grid pays off for small solvent molecules queried many times per
        // frame (each real molecule and every random-insertion slot)
        const bool pays = d.solvent_natomspermol <= 4 &&
                          mv * (1 + (h->mddf ? (int64_t)d.n_random_samples : 0)) >= 4 * h->Ns;
        (void)dense;
        const bool want = d.atoms_grid > 0 || (d.atoms_grid == 0 && pays);
        if (want && fp32 && ms == 1 && !d.autocorrelation && (int64_t)fc * mv <= h->aq_cap) {
            int K = d.atoms_grid > 0 ? d.atoms_grid : (int)std::ceil(target_cell(h) / 4.5);
            K = std::max(1, std::min(K, kAgridMaxK));
            const int64_t gcap = d.atoms_grid_capacity > 0 ? (int64_t)d.atoms_grid_capacity
                                                           : std::min<int64_t>(h->Ns * 128 + 131072, (int64_t)INT32_MAX);
            const int64_t bytes = (int64_t)fc * gcap * 16;
            // under an HBM budget the grid takes at most a quarter of it
            if (d.hbm_budget_bytes <= 0 || h->device_bytes + bytes <= d.hbm_budget_bytes / 4) {
                h->agk = K;
                h->gcap = gcap;
                dev_alloc(h, h->gent, (size_t)bytes);
            }
        }
        if (h->agk > 0) {
            const size_t hsm = hist_smem_bytes(h, h->smem_groups);
            h->agrid_real_ctas = resident_ctas((const void *)k_agrid_real, 256, hsm);
            h->agrid_rand_ctas = resident_ctas((const void *)k_agrid_random, 256, hsm);
        }
    }
    h->planned = true;
}

// Reference solute molecules of one frame (src/mddf.jl:374-376), sorted, with
// their repetition number and distinct index.
int draw_samples(const cm_handle *h, int64_t frame_id, Sample *out, int &ndistinct) {
    const cm_system_desc &d = h->d;
    int nrs = d.n_random_samples;
    uint64_t st = cmfeed::key(d.seed, cmfeed::kTagRef, (uint64_t)frame_id, 0, 0);
    std::vector<int> s(nrs);
    for (int i = 0; i < nrs; ++i) s[i] = (int)cmfeed::below(st, (uint64_t)d.solute_nmols);
    std::sort(s.begin(), s.end());
    ndistinct = 0;
    for (int i = 0; i < nrs; ++i) {
        if (i == 0 || s[i] != s[i - 1]) {
            out[i].rep = 0;
            out[i].d = ndistinct++;
        } else {
            out[i].rep = out[i - 1].rep + 1;
            out[i].d = out[i - 1].d;
        }
        out[i].s = s[i];
        out[i].pad = 0;
    }
    return nrs;
}

int grid_for(int64_t n, int block) { return (int)std::max<int64_t>(1, (n + block - 1) / block); }

cudaEvent_t ev_get(cm_handle *h) {
    if (!h->ev_free.empty()) {
        cudaEvent_t e = h->ev_free.back();
        h->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    CM_CUDA(cudaEventCreate(&e));
    return e;
}

// Fold finished timing events into the per-class totals (synchronises).
void timing_drain(cm_handle *h) {
    if (h->pending.empty()) return;
    CM_CUDA(cudaStreamSynchronize(h->stream));
    for (auto &p : h->pending) {
        float ms = 0.f;
        CM_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
        h->class_ms[p.cls] += ms;
        h->ev_free.push_back(p.a);
        h->ev_free.push_back(p.b);
    }
    h->pending.clear();
}

void kbegin(cm_handle *h, int cls) {
    h->cur_class = cls;
    if (!h->timing) return;
    if (h->pending.size() > 65536) timing_drain(h);
    h->cur_start = ev_get(h);
    CM_CUDA(cudaEventRecord(h->cur_start, h->stream));
}

void kend(cm_handle *h) {
    h->launches_total++;
    h->class_launches[h->cur_class]++;
    if (!h->timing) return;
    cudaEvent_t e = ev_get(h);
    CM_CUDA(cudaEventRecord(e, h->stream));
    h->pending.push_back({h->cur_class, h->cur_start, e});
}

#define CM_LAUNCH(cls, ...)   \
    do {                      \
        kbegin(h, cls);       \
        __VA_ARGS__;          \
        kend(h);              \
        launches++;           \
    } while (0)

// One compute chunk: consecutive frames of one staging batch that carry the
// same non-zero weight.  Every stage of the chain is one launch per chunk.
struct Chunk {
    int c0 = 0, nf = 0;       // first frame (in the staging batch) and count
    int smp0 = 0, nsmp = 0;   // the chunk's samples in the staging sample table
    int tab0 = 0, ntab = 0;   // its (frame, distinct, molecule) bulk-table rows
    int ncell_max = 0;
    double weight = 1.0;
};

Bufs chunk_bufs(cm_handle *h, const Chunk &c, const FrameGeom *dG, const Sample *dS) {
    const cm_system_desc &d = h->d;
    Bufs B{};
    B.nf = c.nf;
    B.ndist = h->ndist_max;
    B.ms = d.solute_nmols;
    B.Ns = h->Ns;
    B.mv = d.solvent_nmols;
    B.Nv = h->Nv;
    B.G = dG + c.c0;
    B.FS = P<FrameScratch>(h->fscratch);
    B.off64 = P<d4>(h->off64);
    B.off32 = P<float4>(h->off32);
    B.counters = P<int>(h->counters);
    B.samples = dS;
    if (h->mddf) {
        B.slot = P<int>(h->slot);
        B.flags = P<unsigned char>(h->flags);
        B.bulk = P<int>(h->bulk);
        B.nbulk = P<int>(h->nbulk);
    }
    if (h->regime == CM_REGIME_PAIRS) {
        B.scell = P<int>(h->scell);
        B.sq32 = P<float4>(h->sq32);
        B.sq64 = P<d4>(h->sq64);
        B.so32 = P<float4>(h->so32);
        B.so64 = P<d4>(h->so64);
        if (!d.autocorrelation) {
            B.vcell = P<int>(h->vcell);
            B.vq32 = P<float4>(h->vq32);
            B.vq64 = P<d4>(h->vq64);
            B.vo32 = P<float4>(h->vo32);
            B.vo64 = P<d4>(h->vo64);
        }
        B.ccount = P<int>(h->ccount);
        B.cstart = P<int>(h->cstart);
        B.cfill = P<int>(h->cfill);
        B.cs = h->ncell_cap + 1;
        B.cmol = P<int>(h->cmol);
        B.cq32 = P<float4>(h->cq32);
        B.gq = P<int4>(h->gq);
        B.gq_cap = h->gq_cap;
        B.eq = P<int4>(h->eq);
        B.eq_cap = h->gq_cap;
        B.rq = P<int2>(h->rq);
        B.rq_cap = h->rq_cap;
    } else {
        B.akey = P<int>(h->akey);
        B.atq32 = P<float4>(h->atq32);
        B.asq32 = P<float4>(h->asq32);
        B.atq64 = P<d4>(h->atq64);
        B.asq64 = P<d4>(h->asq64);
        B.acount = P<int>(h->acount);
        B.astart = P<int>(h->astart);
        B.afill = P<int>(h->afill);
        B.as = (int64_t)d.solute_nmols * h->ncell_cap + 1;
        B.avcell = P<int>(h->avcell);
        B.avq32 = P<float4>(h->avq32);
        B.avq64 = P<d4>(h->avq64);
        B.anear = P<unsigned char>(h->anear);
        B.aq = P<int4>(h->aq);
        B.aq_cap = h->aq_cap;
        if (h->mddf) {
            B.aslot = P<int>(h->aslot);
            B.aslot_cap = h->aslot_cap;
        }
        B.agk = h->agk;
        if (h->agk > 0) {
            B.gfs = h->ncell_cap * (int64_t)h->agk * h->agk * h->agk;
            B.gcap = h->gcap;
            B.gstart = P<int>(h->gstart);
            B.gpool = P<int>(h->gpool);
            B.gedge = P<float2>(h->gedge);
            B.gent = P<float4>(h->gent);
        }
        if (h->mddf) {
            B.u64 = P<d4>(h->u64);
            B.u32 = P<float4>(h->u32);
            B.rc = P<float>(h->rc);
            B.pcell = P<int>(h->pcell);
            B.pq32 = P<float4>(h->pq32);
            B.pq64 = P<d4>(h->pq64);
        }
    }
    return B;
}

// One launch of a chain stage with its arguments, as a stand-alone kernel.
void launch_one(int kid, dim3 g, size_t smem, cudaStream_t st, const MArgs &a) {
    const int t = mk_threads(kid);
    switch (kid) {
    case MK_OFFTABLE: k_offtable<<<g, t, smem, st>>>(a.B); break;
    case MK_PREP_SOLVENT_F32:
        k_prep_atoms_solvent<float><<<g, t, smem, st>>>(a.B, (const float *)a.p, a.i0, a.a0, a.a1);
        break;
    case MK_PREP_SOLVENT_F64:
        k_prep_atoms_solvent<double><<<g, t, smem, st>>>(a.B, (const double *)a.p, a.i0, a.a0, a.a1);
        break;
    case MK_PREP_SOLUTE_F32: k_prep_atoms_solute<float><<<g, t, smem, st>>>(a.B, (const float *)a.p, a.i0); break;
    case MK_PREP_SOLUTE_F64: k_prep_atoms_solute<double><<<g, t, smem, st>>>(a.B, (const double *)a.p, a.i0); break;
    case MK_FRAME_CONSTS: k_frame_consts<<<g, t, smem, st>>>(a.S, a.B, a.a0); break;
    case MK_SCAN: k_scan<<<g, t, smem, st>>>(a.B, a.a0); break;
    case MK_SCATTER_ATOMS: k_scatter_atoms<<<g, t, smem, st>>>(a.B); break;
    case MK_ATOMS_NEAR: k_atoms_near<<<g, t, smem, st>>>(a.B); break;
    case MK_AGRID_BUILD: k_agrid_build<<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_AGRID_REAL: k_agrid_real<<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_AGRID_RANDOM: k_agrid_random<<<g, t, smem, st>>>(a.S, a.B, a.a0, a.a1); break;
    case MK_ATOMS_FILTER: k_atoms_filter<<<g, t, smem, st>>>(a.S, a.B, a.i0, a.i1); break;
    case MK_ATOMS_PLACE: k_atoms_place<<<g, t, smem, st>>>(a.S, a.B, a.a0); break;
    case MK_SLOT_FILTER: k_slot_filter<<<g, t, smem, st>>>(a.S, a.B, a.a0); break;
    case MK_BULK: k_bulk<<<g, t, smem, st>>>(a.S, a.B, (const int4 *)a.p); break;
    case MK_EVAL_REAL_CELL: k_atoms_eval<true, false, kSchedCell><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL_RANDOM_CELL: k_atoms_eval<true, true, kSchedCell><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL_REAL_BALANCED: k_atoms_eval<true, false, kSchedBalanced><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL_RANDOM_BALANCED: k_atoms_eval<true, true, kSchedBalanced><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL64_REAL_CELL: k_atoms_eval<false, false, kSchedCell><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL64_RANDOM_CELL: k_atoms_eval<false, true, kSchedCell><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL64_REAL_THREAD: k_atoms_eval<false, false, kSchedThread><<<g, t, smem, st>>>(a.S, a.B); break;
    case MK_EVAL64_RANDOM_THREAD: k_atoms_eval<false, true, kSchedThread><<<g, t, smem, st>>>(a.S, a.B); break;
    default: throw cm_error(CM_ECUDA, "unknown chain stage");
    }
}

// A stage of a compute chunk's chain: a zero-fill or a kernel with its grid
// and arguments.
struct Step {
    int kernel = 0;  // 0: zero-fill of (zp, zbytes); 1: kernel kid
    int kid = 0;
    dim3 grid;
    size_t smem = 0;
    int cls = 0;
    MArgs a{};
    void *zp = nullptr;
    size_t zbytes = 0;
};

// Where a chain goes: launched on the handle's stream (rec == nullptr), or
// recorded for cm_batch, which launches each stage once for all its systems.
struct Emitter {
    cm_handle *h;
    std::vector<Step> *rec;
    int launches = 0;
    void zero(void *p, size_t bytes) {
        if (rec) {
            Step s;
            s.zp = p;
            s.zbytes = bytes;
            rec->push_back(s);
            return;
        }
        CM_CUDA(cudaMemsetAsync(p, 0, bytes, h->stream));
    }
    void kernel(int kid, dim3 grid, size_t smem, int cls, const MArgs &a) {
        if (rec) {
            Step s;
            s.kernel = 1;
            s.kid = kid;
            s.grid = grid;
            s.smem = smem;
            s.cls = cls;
            s.a = a;
            rec->push_back(s);
            return;
        }
        kbegin(h, cls);
        launch_one(kid, grid, smem, h->stream, a);
        kend(h);
        launches++;
    }
};

// The ATOMS-layout evaluation stage of a handle (precision x schedule).
int eval_kid(const cm_handle *h, bool random) {
    if (h->d.precision == CM_PRECISION_FP32_GUARD)
        return h->atoms_dense ? (random ? MK_EVAL_RANDOM_CELL : MK_EVAL_REAL_CELL)
                              : (random ? MK_EVAL_RANDOM_BALANCED : MK_EVAL_REAL_BALANCED);
    return h->atoms_dense ? (random ? MK_EVAL64_RANDOM_CELL : MK_EVAL64_REAL_CELL)
                          : (random ? MK_EVAL64_RANDOM_THREAD : MK_EVAL64_REAL_THREAD);
}

// The chain of one ATOMS-layout compute chunk (solute atoms binned per
// molecule; see cm_atoms32.cuh and cm_agrid.cuh).
template <typename T>
void atoms_chain(cm_handle *h, const Chunk &c, const DevSys &S, const Bufs &B, const int4 *dtab, const T *xs,
                 const T *xv, int64_t xs_stride, int64_t xv_stride, Emitter &em) {
    const cm_system_desc &d = h->d;
    const bool self = d.autocorrelation;
    const int nf = c.nf;
    const int64_t ms = d.solute_nmols, mv = d.solvent_nmols;
    const int iref = d.irefatom - 1;
    const bool rnd = h->mddf && c.nsmp > 0;
    const size_t hsm = hist_smem_bytes(h, h->smem_groups);
    const int sms = h->sms;
    const bool f32 = sizeof(T) == 4;
    MArgs base{};
    base.S = S;
    base.B = B;
    auto args = [&](const void *p, int64_t i0, int64_t i1, int a0, int a1) {
        MArgs a = base;
        a.p = p;
        a.i0 = i0;
        a.i1 = i1;
        a.a0 = a0;
        a.a1 = a1;
        return a;
    };
    em.zero(B.FS, sizeof(FrameScratch) * nf);
    em.zero(B.counters, 8 * sizeof(int));
    em.kernel(MK_OFFTABLE, dim3(grid_for(cmgeom::kOffEntries, 256), nf), 0, CM_K_PREP, base);
    const T *xsolv = self ? xs : xv;
    em.kernel(f32 ? MK_PREP_SOLVENT_F32 : MK_PREP_SOLVENT_F64, dim3(grid_for(mv, 128), nf), 0, CM_K_PREP,
              args(xsolv, self ? xs_stride : xv_stride, 0, iref, h->mddf ? 1 : 0));
    em.zero(B.acount, (size_t)nf * B.as * 4);
    em.kernel(f32 ? MK_PREP_SOLUTE_F32 : MK_PREP_SOLUTE_F64, dim3(grid_for(h->Ns, 256), nf), 0, CM_K_PREP,
              args(xs, xs_stride, 0, 0, 0));
    em.kernel(MK_FRAME_CONSTS, dim3(nf), 0, CM_K_PREP, args(nullptr, 0, 0, 0, 0));
    em.kernel(MK_SCAN, dim3(nf), 0, CM_K_CELLS, args(nullptr, 0, 0, 1, 0));
    em.kernel(MK_SCATTER_ATOMS, dim3(grid_for(h->Ns, 256), nf), 0, CM_K_CELLS, base);
    if (rnd) em.zero(B.flags, (size_t)nf * B.ndist * mv);
    em.kernel(MK_ATOMS_NEAR, dim3(grid_for(ms * h->ncell_cap, 256), nf), 0, CM_K_CELLS, base);
    // the evaluation's persistent grid: one wave, or fewer CTAs when its
    // queue (at most `items` entries, one per warp at a time) cannot fill them
    auto wgrid_for = [&](int64_t items) {
        return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * h->atoms_ctas, grid_for(items, kAtomsWarps)));
    };
    const bool agrid = h->agk > 0;
    auto agrid_grid = [&](int64_t n, int ctas) {
        return (int)std::min<int64_t>(grid_for(n, 256), (int64_t)sms * ctas);
    };
    if (agrid) {
        // the single solute molecule's candidate lists of every frame
        em.zero(B.gpool, (size_t)nf * sizeof(int));
        em.kernel(MK_AGRID_BUILD, dim3(c.ncell_max, nf), (size_t)kAgridStage * sizeof(float4), CM_K_CELLS, base);
        // real pass: every solvent molecule queried (records inside the band
        // decided in place); frames without a grid go to the evaluation queue.
        // counters[6 .. 7]: the queries' next molecule (zeroed with the chunk's counters)
        em.zero(B.counters + 2, sizeof(int));
        em.kernel(MK_AGRID_REAL, dim3(agrid_grid((int64_t)nf * mv, h->agrid_real_ctas)), hsm, CM_K_REAL, base);
        // the queue is empty unless a frame lost its grid: a grid for one
        // entry per 32 molecules
        em.kernel(eval_kid(h, false), dim3(wgrid_for((int64_t)nf * mv / 32)), hsm, CM_K_REAL, base);
    } else {
        // real pass: molecule pairs that can hold a pair within the cutoff,
        // in pieces of the queue's capacity
        const int64_t items = (int64_t)nf * ms * mv;
        for (int64_t i0 = 0; i0 < items; i0 += h->aq_cap) {
            const int64_t n = std::min<int64_t>(h->aq_cap, items - i0);
            em.zero(B.counters + 2, sizeof(int));
            em.kernel(MK_ATOMS_FILTER, dim3(grid_for(n, 256)), 0, CM_K_REAL, args(nullptr, i0, n, 0, 0));
            em.kernel(eval_kid(h, false), dim3(wgrid_for(n)), hsm, CM_K_REAL, base);
        }
    }
    if (rnd) {
        em.kernel(MK_BULK, dim3(c.ntab), 0, CM_K_BULK, args(dtab + c.tab0, 0, 0, 0, 0));
        for (int s0 = 0; s0 < c.nsmp; s0 += h->atoms_piece) {
            const int ny = std::min(h->atoms_piece, c.nsmp - s0);
            // the evaluation queue, the slot list and the queries' next slot (counters 2 .. 6)
            em.zero(B.counters + 2, 5 * sizeof(int));
            // slots that can reach the solute, their FP64 placement on full
            // warps, then (candidate grid) their queries
            em.kernel(MK_SLOT_FILTER, dim3(grid_for(mv, 128), ny), 0, CM_K_RANDOM, args(nullptr, 0, 0, c.smp0 + s0, 0));
            em.kernel(MK_ATOMS_PLACE, dim3((unsigned)std::min<int64_t>(grid_for((int64_t)ny * mv, 128), (int64_t)sms * 16)),
                      0, CM_K_RANDOM, args(nullptr, 0, 0, c.smp0 + s0, 0));
            if (agrid)
                em.kernel(MK_AGRID_RANDOM, dim3(agrid_grid((int64_t)ny * mv, h->agrid_rand_ctas)), hsm, CM_K_RANDOM,
                          args(nullptr, 0, 0, c.smp0 + s0, ny));
            em.kernel(eval_kid(h, true), dim3(wgrid_for((int64_t)ny * mv / (agrid ? 32 : 1))), hsm, CM_K_RANDOM, base);
        }
    }
}

template <typename T>
void run_chunk(cm_handle *h, const Chunk &c, const FrameGeom *dG, const Sample *dS, const int4 *dtab, const T *xs,
               const T *xv, int64_t xs_stride, int64_t xv_stride) {
    const cm_system_desc &d = h->d;
    cudaStream_t st = h->stream;
    NvtxRange range("cm: chunk (mddf_frame! of each frame)");
    ensure_cells(h, c.ncell_max);
    DevSys S = devsys_full(h);
    Bufs B = chunk_bufs(h, c, dG, dS);
    const bool self = d.autocorrelation;
    B.xs_raw = xs;
    B.xv_raw = self ? (const void *)xs : (const void *)xv;
    B.xs_stride = xs_stride;
    B.xv_stride = self ? xs_stride : xv_stride;
    B.raw64 = sizeof(T) == 8 ? 1 : 0;
    const bool fp32 = d.precision == CM_PRECISION_FP32_GUARD;
    const int nf = c.nf;
    const int64_t ms = d.solute_nmols, mv = d.solvent_nmols, apv = d.solvent_natomspermol;
    const int iref = d.irefatom - 1;
    const bool rnd = h->mddf && c.nsmp > 0;
    const size_t hsm = hist_smem_bytes(h, h->smem_groups);
    const int sms = h->sms;
    int launches = 0;
    if (h->regime == CM_REGIME_PAIRS) {
        CM_CUDA(cudaMemsetAsync(B.FS, 0, sizeof(FrameScratch) * nf, st));
        CM_CUDA(cudaMemsetAsync(B.counters, 0, 8 * sizeof(int), st));
        CM_LAUNCH(CM_K_PREP, k_offtable<<<dim3(grid_for(cmgeom::kOffEntries, 256), nf), 256, 0, st>>>(B));
        if (rnd) CM_CUDA(cudaMemsetAsync(B.flags, 0, (size_t)nf * B.ndist * mv, st));
        CM_CUDA(cudaMemsetAsync(B.ccount, 0, (size_t)nf * B.cs * 4, st));
        // solute molecules (in self mode they also fill the cell counts)
        CM_LAUNCH(CM_K_PREP, k_prep_pairs<T><<<dim3(grid_for(ms, 128), nf), 128, 0, st>>>(B, xs, xs_stride, 0, self ? 1 : 0));
        if (!self)
            CM_LAUNCH(CM_K_PREP, k_prep_pairs<T><<<dim3(grid_for(mv, 128), nf), 128, 0, st>>>(B, xv, xv_stride, 1, 1));
        CM_LAUNCH(CM_K_PREP, k_frame_consts<<<nf, 128, 0, st>>>(S, B, 1));
        CM_LAUNCH(CM_K_CELLS, k_scan<<<nf, 1024, 0, st>>>(B, 0));
        CM_LAUNCH(CM_K_CELLS, k_scatter_mols<<<dim3(grid_for(mv, 256), nf), 256, 0, st>>>(B, self ? 1 : 0));
        const size_t smem = hsm + (size_t)kWarps * kMaxSmallMol * 16 + (size_t)kWarps * kQueue * 8;
        const int grid = (int)std::min<int64_t>(((int64_t)nf * ms + kWarps - 1) / kWarps, (int64_t)sms * h->real_ctas);
        // FP32: one lane per solvent atom; the frames that need several images
        // per molecule pair are left to the generic kernel below
        const bool special = fp32;
        if (fp32) {
            // the accumulators before the real pass, for a redo after a queue overflow
            CM_CUDA(cudaMemcpyAsync(h->hist_snap.p, h->hist.p, (size_t)h->hist_n * 8, cudaMemcpyDeviceToDevice, st));
            CM_CUDA(cudaMemcpyAsync(h->stats_snap.p, h->stats.p, ST_N * 8, cudaMemcpyDeviceToDevice, st));
            const size_t fsm = hsm + (size_t)kFlatWarps * flat_warp_smem();
            const int fgrid = (int)std::min<int64_t>(((int64_t)nf * ms + kFlatWarps - 1) / kFlatWarps,
                                                     (int64_t)sms * h->flat_ctas);
            const FlatKernel fk = flat_kernel(h);
            const bool tile = fk.tile_fn && d.real_pass != CM_REAL_WARP;
            if (tile) {
                // one CTA per home cell; the per-molecule kernel returns at once
                // unless a frame's stencil is beyond the tiled kernel's table
                const size_t tsm = hsm + (size_t)kTileWarps * flat_warp_smem() + tile_smem_extra();
                CM_LAUNCH(CM_K_REAL, fk.tile_launch(sms * h->tile_ctas, tsm, st, S, B));
            }
            CM_LAUNCH(CM_K_REAL, fk.launch(fgrid, fsm, st, S, B, tile ? 1 : 0));
        }
        // the generic kernel takes every frame, or after the specialised one
        // only the frames that need several images per molecule pair
        const int only_multi = special ? 1 : 0;
        if (fp32 && self) CM_LAUNCH(CM_K_REAL, k_pairs_real<true, true><<<grid, kWarps * 32, smem, st>>>(S, B, only_multi));
        else if (fp32) CM_LAUNCH(CM_K_REAL, k_pairs_real<true, false><<<grid, kWarps * 32, smem, st>>>(S, B, only_multi));
        else if (self) CM_LAUNCH(CM_K_REAL, k_pairs_real<false, true><<<grid, kWarps * 32, smem, st>>>(S, B, only_multi));
        else CM_LAUNCH(CM_K_REAL, k_pairs_real<false, false><<<grid, kWarps * 32, smem, st>>>(S, B, only_multi));
        if (special) {
            const int ggrid = sms * h->guard_ctas, egrid = sms * h->edge_ctas;
            if (self) CM_LAUNCH(CM_K_GUARD, k_pairs_guard<true><<<ggrid, kGuardWarps * 32, hsm, st>>>(S, B));
            else CM_LAUNCH(CM_K_GUARD, k_pairs_guard<false><<<ggrid, kGuardWarps * 32, hsm, st>>>(S, B));
            if (self) CM_LAUNCH(CM_K_GUARD, k_pairs_edge<true><<<egrid, 128, hsm, st>>>(S, B));
            else CM_LAUNCH(CM_K_GUARD, k_pairs_edge<false><<<egrid, 128, hsm, st>>>(S, B));
            // a guard or edge queue overflow: the accumulators go back to the
            // snapshot and the generic kernel redoes every frame of the chunk,
            // deciding each record where it is found (both launches return at
            // once otherwise)
            const int64_t nrest = std::max<int64_t>(h->hist_n, ST_N);
            CM_LAUNCH(CM_K_GUARD, k_queue_check<<<(int)std::min<int64_t>(grid_for(nrest, 256), (int64_t)sms * 4), 256, 0, st>>>(
                                      B, P<unsigned long long>(h->hist), P<unsigned long long>(h->hist_snap), h->hist_n,
                                      P<unsigned long long>(h->stats), P<unsigned long long>(h->stats_snap)));
            if (self) CM_LAUNCH(CM_K_REAL, k_pairs_real<true, true><<<grid, kWarps * 32, smem, st>>>(S, B, 2));
            else CM_LAUNCH(CM_K_REAL, k_pairs_real<true, false><<<grid, kWarps * 32, smem, st>>>(S, B, 2));
        }
        if (rnd) {
            CM_LAUNCH(CM_K_BULK, k_bulk<<<c.ntab, 1024, 0, st>>>(S, B, dtab + c.tab0));
            // the random queue holds every slot of `piece` samples
            const int piece = (int)std::max<int64_t>(1, h->rq_cap / mv);
            for (int s0 = 0; s0 < c.nsmp; s0 += piece) {
                const int ny = std::min(piece, c.nsmp - s0);
                if (s0 > 0) CM_CUDA(cudaMemsetAsync(B.counters + 1, 0, sizeof(int), st));
                CM_LAUNCH(CM_K_RANDOM, k_random_filter<<<grid_for((int64_t)ny * mv, 128), 128, 0, st>>>(S, B, c.smp0 + s0, ny));
                if (fp32) CM_LAUNCH(CM_K_RANDOM, k_random_eval<true><<<sms * h->rand_ctas, 128, hsm, st>>>(S, B));
                else CM_LAUNCH(CM_K_RANDOM, k_random_eval<false><<<sms * h->rand_ctas, 128, hsm, st>>>(S, B));
            }
        }
    } else {
        Emitter em{h, nullptr};
        atoms_chain<T>(h, c, S, B, dtab, xs, xv, xs_stride, xv_stride, em);
        launches += em.launches;
    }
    CM_CUDA(cudaGetLastError());
    h->kernels_per_frame = (launches + nf - 1) / nf;
}

void fold_class(cm_handle *h) {
    if (!h->class_open) return;
    int launches = 0;
    CM_LAUNCH(CM_K_OTHER, k_fold<<<grid_for(h->hist_n, 256), 256, 0, h->stream>>>(P<unsigned long long>(h->hist), P<double>(h->sums), h->hist_n, h->class_w));
    (void)launches;
    CM_CUDA(cudaGetLastError());
    h->folds++;
    h->class_open = false;
}

// Frames per compute chunk.
int chunk_frames(const cm_handle *h) { return h->fc; }

// Capture one compute chunk's chain (memsets and kernels on the handle's
// stream) as a CUDA graph and replay it through the handle's executable graph.
// Consecutive chunks of a system have the same chain with other arguments and
// grid sizes, so the executable graph is updated in place; a chain of another
// shape (fewer frames, another number of queue pieces) instantiates it anew.
// Launches already queued are not affected by the update.
template <typename Fn>
void launch_captured(cm_handle *h, Fn &&chain) {
    CM_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t g = nullptr;
    try {
        chain();
    } catch (...) {
        cudaStreamEndCapture(h->stream, &g);
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        throw;
    }
    CM_CUDA(cudaStreamEndCapture(h->stream, &g));
    bool updated = false;
    if (h->gexec) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(h->gexec, g, &info) == cudaSuccess;
        if (!updated) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(h->gexec);  // freed once its queued launches finish
            h->gexec = nullptr;
        }
    }
    if (!updated) {
        const cudaError_t e = cudaGraphInstantiate(&h->gexec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            h->gexec = nullptr;
            throw cm_error(CM_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        h->graph_instantiations++;
    }
    cudaGraphDestroy(g);
    CM_CUDA(cudaGraphLaunch(h->gexec, h->stream));
    h->graph_launches++;
}

// One staging batch of a submit: frames [f0, f0 + nf) of the caller's batch,
// copied into the handle's staging buffers of parity b and split into chunks.
struct Staged {
    int b = 0, f0 = 0, nf = 0, elem = 0;
    const FrameGeom *hg = nullptr;
    FrameGeom *dG = nullptr;
    Sample *dS = nullptr;
    int4 *dT = nullptr;
    const char *xs_base = nullptr, *xv_base = nullptr;
    int64_t sbytes = 0, vbytes = 0;  // bytes from one frame to the next as the kernels read them
    std::vector<Chunk> chunks;
};

// Frame 0 of a raw DCD batch gathered on the host (float32, selection order):
// the planner sizes the cells from one frame's coordinates.
struct DcdFirstFrame {
    std::vector<float> xs, xv;
    cm_frames f{};
};

void dcd_first_frame(cm_handle *h, const cm_frames *f, DcdFirstFrame &out) {
    std::vector<unsigned char> raw((size_t)h->dcd_frame_bytes);
    if (f->memory == CM_MEM_DEVICE) CM_CUDA(cudaMemcpy(raw.data(), f->solute_xyz, raw.size(), cudaMemcpyDeviceToHost));
    else memcpy(raw.data(), f->solute_xyz, raw.size());
    auto gather = [&](const std::vector<int32_t> &idx, std::vector<float> &xyz) {
        xyz.resize(idx.size() * 3);
        for (size_t i = 0; i < idx.size(); ++i)
            for (int k = 0; k < 3; ++k) {
                uint32_t w;
                memcpy(&w, raw.data() + h->dcd_off[k] + 4 * (int64_t)idx[i], 4);
                if (h->dcd_swap) w = (w >> 24) | ((w >> 8) & 0xff00u) | ((w << 8) & 0xff0000u) | (w << 24);
                memcpy(&xyz[3 * i + k], &w, 4);
            }
    };
    gather(h->dcd_s, out.xs);
    if (!h->d.autocorrelation) gather(h->dcd_v, out.xv);
    out.f = *f;
    out.f.nframes = 1;
    out.f.coord_type = CM_COORD_F32;
    out.f.memory = CM_MEM_HOST;
    out.f.solute_xyz = out.xs.data();
    out.f.solvent_xyz = h->d.autocorrelation ? nullptr : out.xv.data();
}

void check_frames(cm_handle *h, const cm_frames *f) {
    const cm_system_desc &d = h->d;
    if (!f || f->nframes < 0) throw cm_error(CM_EINVAL, "invalid frame batch");
    if (f->nframes == 0) return;
    if (!f->solute_xyz || !f->cells || !f->frame_ids) throw cm_error(CM_EINVAL, "solute_xyz, cells and frame_ids are required");
    if (f->coord_type != CM_COORD_F32 && f->coord_type != CM_COORD_F64 && f->coord_type != CM_COORD_DCD)
        throw cm_error(CM_EINVAL, "unknown coord_type");
    if (f->memory != CM_MEM_HOST && f->memory != CM_MEM_DEVICE) throw cm_error(CM_EINVAL, "unknown memory kind");
    const bool dcd = f->coord_type == CM_COORD_DCD;
    if (dcd && !h->dcd) throw cm_error(CM_ESTATE, "raw DCD frames need cm_set_dcd_layout first");
    if (dcd && f->solvent_xyz) throw cm_error(CM_EINVAL, "raw DCD frames hold both selections: solvent_xyz must be NULL");
    if (dcd && (f->solute_frame_stride || f->solvent_frame_stride))
        throw cm_error(CM_EINVAL, "raw DCD frames take no frame strides (the layout gives them)");
    if (f->solute_frame_stride < 0 || (f->solute_frame_stride > 0 && f->solute_frame_stride < h->Ns * 3))
        throw cm_error(CM_EINVAL, "solute_frame_stride must be 0 or at least solute atoms x 3");
    if (!d.autocorrelation &&
        (f->solvent_frame_stride < 0 || (f->solvent_frame_stride > 0 && f->solvent_frame_stride < h->Nv * 3)))
        throw cm_error(CM_EINVAL, "solvent_frame_stride must be 0 or at least solvent atoms x 3");
    if (!dcd && !d.autocorrelation && !f->solvent_xyz) throw cm_error(CM_EINVAL, "solvent_xyz is required unless autocorrelation");
    if (!h->planned) {
        if (dcd) {
            DcdFirstFrame ff;
            dcd_first_frame(h, f, ff);
            plan(h, &ff.f);
        } else {
            plan(h, f);
        }
    }
    if (dcd && h->coord_elem != 4) throw cm_error(CM_EINVAL, "raw DCD frames are float32: this handle was planned for float64");
    const int elem = (f->coord_type == CM_COORD_F32 || dcd) ? 4 : 8;
    if (elem != h->coord_elem && (f->memory == CM_MEM_HOST || dcd))
        throw cm_error(CM_EINVAL, "coordinate type differs from the first batch of this handle");
    for (int i = 0; i < f->nframes; ++i) {
        double w = f->weights ? f->weights[i] : 1.0;
        if (!std::isfinite(w) || w < 0.0) throw cm_error(CM_EINVAL, "frame weights must be finite and non-negative");
    }
}

// Host preparation (geometries, random samples, chunking) and the copies of
// one staging batch; the copies end with ev_copied[b] on the copy stream.
Staged stage(cm_handle *h, const cm_frames *f, int f0) {
    NvtxRange range("cm: stage batch (geometry, samples, copies)");
    const cm_system_desc &d = h->d;
    Staged S;
    const bool dcd = f->coord_type == CM_COORD_DCD;
    S.elem = (f->coord_type == CM_COORD_F32 || dcd) ? 4 : 8;
    S.f0 = f0;
    S.sbytes = h->Ns * 3 * S.elem;
    S.vbytes = h->Nv * 3 * S.elem;
    // the caller's frame strides (bytes)
    const int64_t src_s = (f->solute_frame_stride > 0 ? f->solute_frame_stride : h->Ns * 3) * S.elem;
    const int64_t src_v = (f->solvent_frame_stride > 0 ? f->solvent_frame_stride : h->Nv * 3) * S.elem;
    const double cs = target_cell(h);
    const int fce = chunk_frames(h);
    const int nf = S.nf = std::min(h->max_frames, f->nframes - f0);
    const int b = S.b = h->chunk_parity;
    h->chunk_parity ^= 1;
    // host staging of this batch may be reused only after its previous copy finished
    CM_CUDA(cudaEventSynchronize(h->ev_copied[b]));
    FrameGeom *hg = h->h_geoms[b];
    Sample *hs = h->h_samples[b];
    int4 *ht = h->h_tabs[b];
    S.hg = hg;
    int soff = 0;
    for (int i = 0; i < nf; ++i) {
        FrameGeom &G = hg[i];
        memset(&G, 0, sizeof(G));
        frame_geometry(f->cells + 9 * (int64_t)(f0 + i), cs, 1023, G);
        G.weight = f->weights ? f->weights[f0 + i] : 1.0;
        G.frame_id = f->frame_ids[f0 + i];
        G.sample_off = soff;
        if (h->mddf) {
            int nd = 0;
            G.nsamples = draw_samples(h, G.frame_id, hs + soff, nd);
            G.ndistinct = nd;
            soff += G.nsamples;
        }
    }
    // compute chunks: runs of equal non-zero weight (zero-weight frames are
    // skipped, src/mddf.jl:102), at most fce frames each
    int ntab = 0;
    for (int i = 0; i < nf;) {
        if (hg[i].weight == 0.0) {
            ++i;
            continue;
        }
        Chunk c;
        c.c0 = i;
        c.weight = hg[i].weight;
        c.smp0 = hg[i].sample_off;
        c.tab0 = ntab;
        int j = i;
        while (j < nf && j - i < fce && hg[j].weight == c.weight) {
            const FrameGeom &G = hg[j];
            c.ncell_max = std::max(c.ncell_max, G.ncell);
            for (int k = 0; k < G.nsamples; ++k) {
                Sample &sm = hs[G.sample_off + k];
                sm.pad = j - i;
                if (sm.rep == 0) ht[ntab++] = make_int4(j - i, sm.d, sm.s, 0);
            }
            ++j;
        }
        c.nf = j - i;
        c.nsmp = hg[j - 1].sample_off + hg[j - 1].nsamples - c.smp0;
        c.ntab = ntab - c.tab0;
        S.chunks.push_back(c);
        i = j;
    }
    cudaStream_t cp = f->memory == CM_MEM_HOST ? h->copy_stream : h->stream;
    CM_CUDA(cudaStreamWaitEvent(cp, h->ev_done[b], 0));
    S.dG = P<FrameGeom>(h->geoms) + (size_t)b * h->max_frames;
    S.dS = h->mddf ? P<Sample>(h->samples) + (size_t)b * h->h_samples_cap : nullptr;
    S.dT = h->mddf ? P<int4>(h->tabs) + (size_t)b * h->max_frames * h->ndist_max : nullptr;
    CM_CUDA(cudaMemcpyAsync(S.dG, hg, sizeof(FrameGeom) * nf, cudaMemcpyHostToDevice, cp));
    if (h->mddf && soff > 0) CM_CUDA(cudaMemcpyAsync(S.dS, hs, sizeof(Sample) * soff, cudaMemcpyHostToDevice, cp));
    if (h->mddf && ntab > 0) CM_CUDA(cudaMemcpyAsync(S.dT, ht, sizeof(int4) * ntab, cudaMemcpyHostToDevice, cp));
    if (dcd) {
        // raw frames to the device (unless they are there already), then the
        // selections gathered into the staging buffers, on the copy stream
        const unsigned char *raw = (const unsigned char *)f->solute_xyz + h->dcd_frame_bytes * f0;
        dev_alloc(h, h->stage_s[b], (size_t)h->max_frames * h->Ns * 3 * 4);
        if (!d.autocorrelation) dev_alloc(h, h->stage_v[b], (size_t)h->max_frames * h->Nv * 3 * 4);
        if (f->memory == CM_MEM_HOST) {
            dev_alloc(h, h->dcd_raw[b], (size_t)h->dcd_frame_bytes * h->max_frames);
            CM_CUDA(cudaMemcpyAsync(h->dcd_raw[b].p, raw, (size_t)h->dcd_frame_bytes * nf, cudaMemcpyHostToDevice, cp));
            raw = (const unsigned char *)h->dcd_raw[b].p;
        }
        auto gather = [&](DevBuf &idx, int64_t n, DevBuf &out) {
            k_dcd_gather<<<dim3(grid_for(n, 256), nf), 256, 0, cp>>>(raw, h->dcd_frame_bytes, h->dcd_off[0], h->dcd_off[1],
                                                                      h->dcd_off[2], h->dcd_swap, P<int32_t>(idx), n,
                                                                      P<float>(out));
        };
        gather(h->dcd_sidx, h->Ns, h->stage_s[b]);
        S.xs_base = (const char *)h->stage_s[b].p;
        if (!d.autocorrelation) {
            gather(h->dcd_vidx, h->Nv, h->stage_v[b]);
            S.xv_base = (const char *)h->stage_v[b].p;
        }
        CM_CUDA(cudaGetLastError());
        h->launches_total += d.autocorrelation ? 1 : 2;
    } else if (f->memory == CM_MEM_HOST) {
        // the staging buffers exist already unless the handle's first frames came from device memory
        dev_alloc(h, h->stage_s[b], (size_t)h->max_frames * h->Ns * 3 * h->coord_elem);
        if (!d.autocorrelation) dev_alloc(h, h->stage_v[b], (size_t)h->max_frames * h->Nv * 3 * h->coord_elem);
        // consecutive frames in one copy, frames of a larger array row by row
        auto copy = [&](void *dst, const void *src, int64_t width, int64_t src_stride) {
            if (src_stride == width)
                CM_CUDA(cudaMemcpyAsync(dst, (const char *)src + width * f0, (size_t)width * nf, cudaMemcpyHostToDevice, cp));
            else
                CM_CUDA(cudaMemcpy2DAsync(dst, (size_t)width, (const char *)src + src_stride * f0, (size_t)src_stride,
                                          (size_t)width, (size_t)nf, cudaMemcpyHostToDevice, cp));
        };
        copy(h->stage_s[b].p, f->solute_xyz, S.sbytes, src_s);
        S.xs_base = (const char *)h->stage_s[b].p;
        if (!d.autocorrelation) {
            copy(h->stage_v[b].p, f->solvent_xyz, S.vbytes, src_v);
            S.xv_base = (const char *)h->stage_v[b].p;
        }
    } else {
        // device frames are read in place, at the caller's strides
        S.sbytes = src_s;
        S.vbytes = src_v;
        S.xs_base = (const char *)f->solute_xyz + S.sbytes * f0;
        if (!d.autocorrelation) S.xv_base = (const char *)f->solvent_xyz + S.vbytes * f0;
    }
    CM_CUDA(cudaEventRecord(h->ev_copied[b], cp));
    for (const Chunk &c : S.chunks) ensure_cells(h, c.ncell_max);  // may wait for this handle's stream: never inside a capture
    return S;
}

// The kernels of one chunk of a staged batch on the handle's stream.
void run_staged_chunk(cm_handle *h, const Staged &S, const Chunk &c) {
    const char *xs = S.xs_base + S.sbytes * c.c0;
    const char *xv = S.xv_base ? S.xv_base + S.vbytes * c.c0 : nullptr;
    const int64_t ss = S.sbytes / S.elem, vs = S.vbytes / S.elem;
    if (S.elem == 4) run_chunk<float>(h, c, S.dG, S.dS, S.dT, (const float *)xs, (const float *)xv, ss, vs);
    else run_chunk<double>(h, c, S.dG, S.dS, S.dT, (const double *)xs, (const double *)xv, ss, vs);
}

// Host accumulators of a chunk's frames (src/mddf.jl:352).
void account_chunk(cm_handle *h, const Staged &S, const Chunk &c) {
    for (int i = c.c0; i < c.c0 + c.nf; ++i) {
        h->volume_total += S.hg[i].weight * S.hg[i].det;
        h->weight_total += S.hg[i].weight;
        h->frames++;
    }
}

// Weight classes: a chunk of another weight first folds the open class.
void open_class(cm_handle *h, double w) {
    if (h->class_open && w != h->class_w) fold_class(h);
    h->class_open = true;
    h->class_w = w;
}

// Candidate-grid lists that did not fit in earlier submits (those frames took
// the walk): once the handle's queued work is done, grow the entries per
// frame to a quarter above the largest frame's need, at least doubling them
// (within the HBM budget), so that later chunks use the grid.
void agrid_grow(cm_handle *h) {
    if (h->agk <= 0 || h->d.atoms_grid_capacity > 0 || h->gcap >= INT32_MAX) return;
    if (cudaStreamQuery(h->stream) != cudaSuccess) {
        (void)cudaGetLastError();  // still running (cudaErrorNotReady): look again at the next submit
        return;
    }
    unsigned long long ovf[2] = {0, 0};
    CM_CUDA(cudaMemcpy(ovf, P<unsigned long long>(h->stats) + ST_AGRID_OVF, sizeof(ovf), cudaMemcpyDeviceToHost));
    if (ovf[0] == 0) return;
    const int64_t gcap = std::min<int64_t>(std::max<int64_t>(h->gcap * 2, (int64_t)(ovf[1] + ovf[1] / 4)), (int64_t)INT32_MAX);
    const int64_t bytes = (int64_t)h->fc * gcap * 16;
    const int64_t now = (int64_t)h->gent.charged;
    if (h->d.hbm_budget_bytes > 0 && h->device_bytes - now + bytes > h->d.hbm_budget_bytes / 4) return;
    dev_alloc(h, h->gent, (size_t)bytes);
    h->gcap = gcap;
    CM_CUDA(cudaMemsetAsync(P<unsigned long long>(h->stats) + ST_AGRID_OVF, 0, sizeof(ovf), h->stream));
}

void submit(cm_handle *h, const cm_frames *f) {
    check_frames(h, f);
    if (h->planned) agrid_grow(h);
    for (int f0 = 0; f0 < f->nframes; f0 += h->max_frames) {
        const Staged S = stage(h, f, f0);
        CM_CUDA(cudaStreamWaitEvent(h->stream, h->ev_copied[S.b], 0));
        for (const Chunk &c : S.chunks) {
            open_class(h, c.weight);
            if (h->graphs) launch_captured(h, [&] { run_staged_chunk(h, S, c); });
            else run_staged_chunk(h, S, c);
            account_chunk(h, S, c);
        }
        CM_CUDA(cudaEventRecord(h->ev_done[S.b], h->stream));
    }
}

void check_device_error(cm_handle *h) {
    CM_CUDA(cudaStreamSynchronize(h->stream));
    int e = 0;
    CM_CUDA(cudaMemcpy(&e, h->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        std::string m = "device-side check failed:";
        if (e & ERR_STENCIL) m += " search range wider than the offset table (box too small for the cutoff);";
        if (e & ERR_BIN) m += " histogram bin out of range;";
        if (e & ERR_QUEUE) m += " random-insertion or molecule-pair queue overflow;";
        if (e & ERR_SIZE) m += " molecule too large for the PAIRS layout;";
        throw cm_error(CM_EDEVICE, m);
    }
}

template <typename F>
int guarded(cm_handle *h, F &&fn) {
    if (!h) {
        g_create_error = "NULL handle";
        return CM_EINVAL;
    }
    try {
        CM_CUDA(cudaSetDevice(h->device));
        fn();
        return CM_OK;
    } catch (const cm_error &e) {
        h->err = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        h->err = "host allocation failed";
        return CM_ENOMEM;
    } catch (const std::exception &e) {
        h->err = e.what();
        return CM_ECUDA;
    }
}

void free_all(cm_handle *h) {
    // the blocks go back to the cache: nothing of this handle may still use them
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    DevBuf *all[] = {&h->geoms, &h->samples, &h->fscratch, &h->off64, &h->off32, &h->hist, &h->sums, &h->stats, &h->errflag, &h->hist_snap, &h->stats_snap,
                     &h->slot, &h->flags, &h->bulk, &h->nbulk, &h->tabs, &h->counters, &h->stage_s[0], &h->stage_s[1], &h->stage_v[0],
                     &h->stage_v[1], &h->scell, &h->sq32, &h->sq64, &h->so32, &h->so64, &h->vcell, &h->vq32, &h->vq64,
                     &h->vo32, &h->vo64, &h->u64, &h->u32, &h->rc, &h->ccount, &h->cstart, &h->cfill, &h->cmol, &h->cq32, &h->gq, &h->eq, &h->rq, &h->akey, &h->atq32,
                     &h->atq64, &h->asq32, &h->asq64, &h->acount, &h->astart, &h->afill, &h->avcell, &h->avq32, &h->avq64,
                     &h->pcell, &h->pq32, &h->pq64, &h->anear, &h->aq, &h->g_soff, &h->g_sidx, &h->g_voff, &h->g_vidx,
                     &h->dcd_sidx, &h->dcd_vidx, &h->dcd_raw[0], &h->dcd_raw[1], &h->final_out, &h->final_job,
                     &h->contrib_q, &h->contrib_g, &h->contrib_out};
    for (DevBuf *b : all) {
        blocks().put(h->device, false, b->p, b->bytes);
        b->p = nullptr;
        b->bytes = b->charged = 0;
    }
    h->device_bytes = 0;
    for (const DevBuf &b : h->host_blocks) blocks().put(h->device, true, b.p, b.bytes);
    h->host_blocks.clear();
    for (int i = 0; i < 2; ++i) {
        h->h_geoms[i] = nullptr;
        h->h_samples[i] = nullptr;
        h->h_tabs[i] = nullptr;
        if (h->ev_copied[i]) cudaEventDestroy(h->ev_copied[i]);
        if (h->ev_done[i]) cudaEventDestroy(h->ev_done[i]);
    }
    for (auto &p : h->pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    h->pending.clear();
    for (cudaEvent_t e : h->ev_free) cudaEventDestroy(e);
    h->ev_free.clear();
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
}

}  // namespace

// ---------------------------------------------------------------------------
// Allocation-free one-frame entry point (cm_frame_counts_noalloc).
//
// Every device buffer the frame needs beyond the caller's coordinates and
// output lives in g_noalloc_scratch, a file-scope array of
// CM_NOALLOC_SCRATCH_BYTES.  Each call looks up its address with the call's
// device current (cudaGetSymbolAddress).  All calls share the
// array and find the previous call's contents in it: each call clears what
// must start at zero (frame scratch, queue counters, cell counts, bulk flags,
// the slot table, statistics, the error flag and the output), and calls whose
// GPU work overlaps race on it.
namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[CM_NOALLOC_SCRATCH_BYTES];

constexpr int kNoAllocMaxDevices = 64;

// The array's device address in the current context, looked up on every call
// (a driver query, no stream work): a caller that runs calls in another
// context of the same device, or after cudaDeviceReset, gets the address that
// is valid there, never a stale one.
unsigned char *noalloc_scratch() {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) throw cm_error(CM_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    return (unsigned char *)p;
}

// Bump allocator over the scratch array, 256-byte aligned pieces.  With a
// null base it only adds up the sizes.
struct Carve {
    unsigned char *base = nullptr;
    size_t off = 0;
    void take(DevBuf &b, size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        b.p = base ? base + off : nullptr;
        b.bytes = bytes;
        off += std::max<size_t>(bytes, 16);
    }
};

void noalloc_fits(size_t bytes) {
    if (bytes > (size_t)CM_NOALLOC_SCRATCH_BYTES)
        throw cm_error(CM_EINVAL, "the system needs " + std::to_string(bytes) +
                                      " bytes of scratch; the allocation-free entry point has " +
                                      std::to_string((size_t)CM_NOALLOC_SCRATCH_BYTES) + " (use cm_create / cm_submit_frames)");
}

// Buffers of one frame that do not depend on the cell grid.
void noalloc_fixed(cm_handle *h, Carve &c) {
    const cm_system_desc &d = h->d;
    const int64_t ms = d.solute_nmols, mv = d.solvent_nmols;
    c.take(h->geoms, sizeof(FrameGeom));
    c.take(h->fscratch, sizeof(FrameScratch));
    c.take(h->off64, sizeof(d4) * cmgeom::kOffEntries);
    c.take(h->off32, sizeof(float4) * cmgeom::kOffEntries);
    c.take(h->counters, 8 * sizeof(int));
    c.take(h->stats, ST_N * 8);
    if (d.precision == CM_PRECISION_FP32_GUARD) {
        c.take(h->hist_snap, (size_t)h->hist_n * 8);
        c.take(h->stats_snap, ST_N * 8);
    }
    c.take(h->errflag, 8);
    if (h->mddf) {
        const int nd = h->ndist_max;
        c.take(h->samples, sizeof(Sample) * d.n_random_samples);
        c.take(h->tabs, sizeof(int4) * nd);
        c.take(h->slot, ms * 4);
        c.take(h->flags, (size_t)nd * mv);
        c.take(h->bulk, (size_t)nd * mv * 4);
        c.take(h->nbulk, (size_t)nd * 4);
    }
    c.take(h->scell, ms * 4);
    c.take(h->sq32, ms * 16);
    c.take(h->sq64, ms * 32);
    c.take(h->so32, h->Ns * 16);
    c.take(h->so64, h->Ns * 32);
    if (!d.autocorrelation) {
        c.take(h->vcell, mv * 4);
        c.take(h->vq32, mv * 16);
        c.take(h->vq64, mv * 32);
        c.take(h->vo32, h->Nv * 16);
        c.take(h->vo64, h->Nv * 32);
    }
    c.take(h->cmol, mv * 4);
    c.take(h->cq32, mv * 16);
    h->gq_cap = (int)std::min<int64_t>(std::max<int64_t>(ms * mv, 1024), 1 << 17);
    if (d.guard_queue_capacity > 0) h->gq_cap = std::min(h->gq_cap, d.guard_queue_capacity);
    c.take(h->gq, (size_t)h->gq_cap * sizeof(int4));
    c.take(h->eq, (size_t)h->gq_cap * 3 * sizeof(int4));
    if (h->mddf) {
        h->rq_cap = (int)std::min<int64_t>(std::max<int64_t>((int64_t)d.n_random_samples * mv, mv), std::max<int64_t>(mv, 1 << 18));
        c.take(h->rq, (size_t)h->rq_cap * sizeof(int2));
    }
}

// Reference solute molecules of one frame into a caller-provided array
// (same draws and order as draw_samples, without a temporary vector).
int noalloc_samples(const cm_system_desc &d, int64_t frame_id, Sample *out, int4 *tab, int &ntab) {
    const int nrs = d.n_random_samples;
    uint64_t st = cmfeed::key(d.seed, cmfeed::kTagRef, (uint64_t)frame_id, 0, 0);
    for (int i = 0; i < nrs; ++i) {
        out[i].s = (int)cmfeed::below(st, (uint64_t)d.solute_nmols);
        out[i].pad = 0;
    }
    std::sort(out, out + nrs, [](const Sample &a, const Sample &b) { return a.s < b.s; });
    int nd = 0;
    ntab = 0;
    for (int i = 0; i < nrs; ++i) {
        if (i == 0 || out[i].s != out[i - 1].s) {
            out[i].rep = 0;
            out[i].d = nd++;
            tab[ntab++] = make_int4(0, out[i].d, out[i].s, 0);
        } else {
            out[i].rep = out[i - 1].rep + 1;
            out[i].d = out[i - 1].d;
        }
    }
    return nd;
}

void noalloc_smem_attributes(cm_handle *h) {
    kernel_smem_limits(h->device);
    check_smem(h, hist_smem_bytes(h, h->smem_groups) + pairs_extra_smem());
    h->flat_ctas = flat_setup(h);
}

thread_local Sample t_noalloc_samples[CM_NOALLOC_MAX_SAMPLES];
thread_local int4 t_noalloc_tab[CM_NOALLOC_MAX_SAMPLES];

template <typename T>
void noalloc_run(cm_handle *h, const cm_frames *f, cudaStream_t stream) {
    const cm_system_desc &d = h->d;
    Carve c{noalloc_scratch(), 0};
    noalloc_fixed(h, c);
    const T *xs = (const T *)f->solute_xyz;
    const T *xv = d.autocorrelation ? nullptr : (const T *)f->solvent_xyz;
    FrameGeom *dG = P<FrameGeom>(h->geoms);

    // molecule radii on a one-cell grid of the box size the PAIRS cells
    FrameGeom G;
    memset(&G, 0, sizeof(G));
    frame_geometry(f->cells, 1e30, 1, G);
    G.weight = 1.0;
    G.frame_id = f->frame_ids[0];
    h->ncell_cap = 0;
    CM_CUDA(cudaMemcpyAsync(dG, &G, sizeof(G), cudaMemcpyHostToDevice, stream));
    CM_CUDA(cudaMemsetAsync(h->fscratch.p, 0, sizeof(FrameScratch), stream));
    {
        Chunk one;
        one.nf = 1;
        const Bufs B = chunk_bufs(h, one, dG, nullptr);
        k_prep_pairs<T><<<grid_for(d.solute_nmols, 128), 128, 0, stream>>>(B, xs, h->Ns * 3, 0, 0);
        if (!d.autocorrelation) k_prep_pairs<T><<<grid_for(d.solvent_nmols, 128), 128, 0, stream>>>(B, xv, h->Nv * 3, 1, 0);
        CM_CUDA(cudaGetLastError());
    }
    FrameScratch F;
    CM_CUDA(cudaMemcpyAsync(&F, h->fscratch.p, sizeof(F), cudaMemcpyDeviceToHost, stream));
    CM_CUDA(cudaStreamSynchronize(stream));
    const double rs = F.rmax_s, rv = d.autocorrelation ? F.rmax_s : F.rmax_v;
    const double cut = d.usecutoff ? d.cutoff : d.dbulk;
    h->pair_cell = (cut + rs + rv) * 1.05 + 0.25;

    // the frame on its cell grid
    memset(&G, 0, sizeof(G));
    frame_geometry(f->cells, target_cell(h), 1023, G);
    G.weight = 1.0;
    G.frame_id = f->frame_ids[0];
    Chunk one;
    one.nf = 1;
    one.ncell_max = G.ncell;
    if (h->mddf) {
        int ntab = 0;
        G.nsamples = d.n_random_samples;
        G.ndistinct = noalloc_samples(d, G.frame_id, t_noalloc_samples, t_noalloc_tab, ntab);
        one.nsmp = G.nsamples;
        one.ntab = ntab;
    }
    c.take(h->ccount, (size_t)(G.ncell + 1) * 4);
    c.take(h->cstart, (size_t)(G.ncell + 1) * 4);
    c.take(h->cfill, (size_t)(G.ncell + 1) * 4);
    noalloc_fits(c.off);
    h->ncell_cap = G.ncell;
    CM_CUDA(cudaMemcpyAsync(dG, &G, sizeof(G), cudaMemcpyHostToDevice, stream));
    if (h->mddf) {
        CM_CUDA(cudaMemcpyAsync(h->samples.p, t_noalloc_samples, sizeof(Sample) * one.nsmp, cudaMemcpyHostToDevice, stream));
        CM_CUDA(cudaMemcpyAsync(h->tabs.p, t_noalloc_tab, sizeof(int4) * one.ntab, cudaMemcpyHostToDevice, stream));
        CM_CUDA(cudaMemsetAsync(h->slot.p, 0xff, (size_t)d.solute_nmols * 4, stream));
    }
    CM_CUDA(cudaMemsetAsync(h->stats.p, 0, ST_N * 8, stream));
    CM_CUDA(cudaMemsetAsync(h->errflag.p, 0, 8, stream));
    CM_CUDA(cudaMemsetAsync(h->hist.p, 0, h->hist_n * 8, stream));
    run_chunk<T>(h, one, dG, P<Sample>(h->samples), P<int4>(h->tabs), xs, xv, h->Ns * 3, h->Nv * 3);
    int e = 0;
    CM_CUDA(cudaMemcpyAsync(&e, h->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CM_CUDA(cudaStreamSynchronize(stream));
    if (e) {
        std::string m = "device-side check failed:";
        if (e & ERR_STENCIL) m += " search range wider than the offset table (box too small for the cutoff);";
        if (e & ERR_BIN) m += " histogram bin out of range;";
        if (e & ERR_QUEUE) m += " random-insertion queue overflow;";
        if (e & ERR_SIZE) m += " molecule too large for the PAIRS layout;";
        throw cm_error(CM_EDEVICE, m);
    }
}

int noalloc_frame(const cm_system_desc *desc, const cm_frames *f, int64_t *counts, int64_t counts_len, void *stream) {
    NvtxRange range("cm: allocation-free frame");
    int prev = -1;
    try {
        check_desc(desc);
        if (desc->solute_group_offsets || desc->solvent_group_offsets)
            throw cm_error(CM_EINVAL, "the allocation-free entry point uses the default per-atom groups (no group tables)");
        if (desc->regime == CM_REGIME_ATOMS || desc->solute_natomspermol > kMaxSmallMol || desc->solvent_natomspermol > kMaxSmallMol)
            throw cm_error(CM_EINVAL, "the allocation-free entry point runs the PAIRS layout only (at most 32 atoms per molecule)");
        if (desc->mode == CM_MODE_MDDF && desc->n_random_samples > CM_NOALLOC_MAX_SAMPLES)
            throw cm_error(CM_EINVAL, "the allocation-free entry point takes at most " + std::to_string(CM_NOALLOC_MAX_SAMPLES) +
                                          " random samples per frame");
        if (desc->device < 0 || desc->device >= kNoAllocMaxDevices) throw cm_error(CM_EINVAL, "device index out of range");
        if (!f || f->nframes != 1) throw cm_error(CM_EINVAL, "the allocation-free entry point takes exactly one frame");
        if (f->memory != CM_MEM_DEVICE) throw cm_error(CM_EINVAL, "the allocation-free entry point takes coordinates in device memory");
        if (f->coord_type != CM_COORD_F32 && f->coord_type != CM_COORD_F64) throw cm_error(CM_EINVAL, "unknown coord_type");
        if (!f->solute_xyz || !f->cells || !f->frame_ids) throw cm_error(CM_EINVAL, "solute_xyz, cells and frame_ids are required");
        if (!desc->autocorrelation && !f->solvent_xyz) throw cm_error(CM_EINVAL, "solvent_xyz is required unless autocorrelation");
        if (f->weights) throw cm_error(CM_EINVAL, "the allocation-free entry point counts one unweighted frame (weights must be NULL)");
        if (!counts) throw cm_error(CM_EINVAL, "NULL counts");

        cm_handle h;
        h.d = *desc;
        h.device = desc->device;
        h.Ns = (int64_t)desc->solute_nmols * desc->solute_natomspermol;
        h.Nv = (int64_t)desc->solvent_nmols * desc->solvent_natomspermol;
        h.mddf = desc->mode == CM_MODE_MDDF;
        h.regime = CM_REGIME_PAIRS;
        h.Gs = desc->solute_natomspermol;
        h.Gv = desc->solvent_natomspermol;
        h.ndist_max = h.mddf ? std::max(1, std::min(desc->solute_nmols, desc->n_random_samples)) : 0;
        h.fc = h.max_frames = 1;
        h.coord_elem = f->coord_type == CM_COORD_F32 ? 4 : 8;
        // histogram layout of cm_raw_counts, concatenated
        const int64_t nb = desc->nbins, Gv = desc->autocorrelation ? 0 : h.Gv;
        h.o_md = 0;
        h.o_mdr = nb;
        h.o_rdf = 2 * nb;
        h.o_rdfr = 3 * nb;
        h.o_gs = 4 * nb;
        h.o_gsr = h.o_gs + h.Gs * nb;
        h.o_gv = h.o_gsr + h.Gs * nb;
        h.o_gvr = h.o_gv + Gv * nb;
        h.hist_n = h.o_gvr + Gv * nb;
        if (counts_len != h.hist_n)
            throw cm_error(CM_EINVAL, "counts must hold " + std::to_string(h.hist_n) + " int64 values");
        h.hist.p = counts;
        h.hist.bytes = (size_t)h.hist_n * 8;
        const size_t extra = pairs_extra_smem();
        h.smem_groups = hist_smem_bytes(&h, 1) + extra + 2048 <= 160 * 1024 ? 1 : 0;
        {
            Carve dry;
            noalloc_fixed(&h, dry);
            noalloc_fits(dry.off);
        }
        CM_CUDA(cudaGetDevice(&prev));
        CM_CUDA(cudaSetDevice(h.device));
        CM_CUDA(cudaDeviceGetAttribute(&h.sms, cudaDevAttrMultiProcessorCount, h.device));
        h.stream = (cudaStream_t)stream;
        noalloc_smem_attributes(&h);
        if (h.coord_elem == 4) noalloc_run<float>(&h, f, h.stream);
        else noalloc_run<double>(&h, f, h.stream);
        h.stream = nullptr;
        cudaSetDevice(prev);
        return CM_OK;
    } catch (const cm_error &e) {
        g_create_error = e.msg;
        if (prev >= 0) cudaSetDevice(prev);
        return e.code;
    } catch (const std::exception &e) {
        g_create_error = e.what();
        if (prev >= 0) cudaSetDevice(prev);
        return CM_ECUDA;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Batches of systems in one CUDA graph.

struct cm_batch {
    std::vector<cm_handle *> hs;
    int device = 0;
    int mode = CM_BATCH_FUSED;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, after = nullptr;
    std::vector<cudaEvent_t> pre, join;
    cudaGraphExec_t gexec = nullptr, gexec_fused = nullptr;
    int64_t launches = 0, instantiations = 0;
    // fused rounds: one launch per stage for every system, from work tables
    // staged in pinned host memory and copied to the device before the graph
    int64_t fused_rounds = 0, stage_launches = 0, fused_systems = 0;
    void *h_tab = nullptr, *d_tab = nullptr;
    size_t tab_cap = 0;
    cudaEvent_t tab_copied = nullptr;
    std::string err;
};

namespace {

void batch_free(cm_batch *b) {
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->gexec_fused) cudaGraphExecDestroy(b->gexec_fused);
    if (b->tab_copied) cudaEventDestroy(b->tab_copied);
    if (b->h_tab) cudaFreeHost(b->h_tab);
    if (b->d_tab) cudaFree(b->d_tab);
    for (cudaEvent_t e : b->pre) cudaEventDestroy(e);
    for (cudaEvent_t e : b->join) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->after) cudaEventDestroy(b->after);
    if (b->stream) cudaStreamDestroy(b->stream);
}

// One fused launch of a chain stage: k_multi<kid> over every system's work-table
// entry.
void launch_multi(int kid, unsigned grid, size_t smem, cudaStream_t st, const MTask *t, int n, long long nb) {
    const int th = mk_threads(kid);
    switch (kid) {
#define CM_MK(K)                                          \
    case K:                                               \
        k_multi<K><<<grid, th, smem, st>>>(t, n, nb); \
        break;
        CM_MK(MK_OFFTABLE)
        CM_MK(MK_PREP_SOLVENT_F32)
        CM_MK(MK_PREP_SOLVENT_F64)
        CM_MK(MK_PREP_SOLUTE_F32)
        CM_MK(MK_PREP_SOLUTE_F64)
        CM_MK(MK_FRAME_CONSTS)
        CM_MK(MK_SCAN)
        CM_MK(MK_SCATTER_ATOMS)
        CM_MK(MK_ATOMS_NEAR)
        CM_MK(MK_AGRID_BUILD)
        CM_MK(MK_AGRID_REAL)
        CM_MK(MK_AGRID_RANDOM)
        CM_MK(MK_ATOMS_FILTER)
        CM_MK(MK_ATOMS_PLACE)
        CM_MK(MK_SLOT_FILTER)
        CM_MK(MK_BULK)
        CM_MK(MK_EVAL_REAL_CELL)
        CM_MK(MK_EVAL_RANDOM_CELL)
        CM_MK(MK_EVAL_REAL_BALANCED)
        CM_MK(MK_EVAL_RANDOM_BALANCED)
#undef CM_MK
    default: throw cm_error(CM_ECUDA, "stage without a fused kernel");
    }
}

// Systems whose chains a batch fuses: the ATOMS layout in FP32 (the plain FP64
// path keeps one launch per system), stream launches without per-launch timing.
bool fusable(const cm_handle *h) {
    return h->regime == CM_REGIME_ATOMS && h->d.precision == CM_PRECISION_FP32_GUARD && !h->timing;
}

// The stages of one staged chunk, recorded instead of launched.
void record_chunk(cm_handle *h, const Staged &S, const Chunk &c, std::vector<Step> &out) {
    Emitter em{h, &out};
    const char *xs = S.xs_base + S.sbytes * c.c0;
    const char *xv = S.xv_base ? S.xv_base + S.vbytes * c.c0 : nullptr;
    const int64_t ss = S.sbytes / S.elem, vs = S.vbytes / S.elem;
    DevSys D = devsys_full(h);
    Bufs B = chunk_bufs(h, c, S.dG, S.dS);
    const bool self = h->d.autocorrelation;
    B.xs_raw = xs;
    B.xv_raw = self ? (const void *)xs : (const void *)xv;
    B.xs_stride = ss;
    B.xv_stride = self ? ss : vs;
    B.raw64 = S.elem == 8 ? 1 : 0;
    if (S.elem == 4) atoms_chain<float>(h, c, D, B, S.dT, (const float *)xs, (const float *)xv, ss, vs, em);
    else atoms_chain<double>(h, c, D, B, S.dT, (const double *)xs, (const double *)xv, ss, vs, em);
}

// A fused staging round: every system's chunk j goes through the same chain
// of stages, and each stage runs once for all of them (k_multi, k_multi_zero)
// in one captured graph on the batch stream; where the systems' kernels of a
// stage differ (the ATOMS evaluation schedule follows each solute's density)
// the stage takes one launch per kernel.  False (nothing launched) when the
// systems cannot share the launches: another layout or precision, a weight
// class change inside the round, or chains of different lengths.
bool batch_round_fused(cm_batch *bt, std::vector<Staged> &st, const std::vector<char> &active) {
    const size_t n = bt->hs.size();
    size_t nchunks = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!active[i]) continue;
        cm_handle *h = bt->hs[i];
        if (!fusable(h)) return false;
        for (const Chunk &c : st[i].chunks)
            if ((h->class_open && c.weight != h->class_w) || c.weight != st[i].chunks[0].weight) return false;
        nchunks = std::max(nchunks, st[i].chunks.size());
    }
    // one shared-memory size for every system's stage: the group histograms go
    // to global memory (their credits are a few per record), the privatised
    // MDDF and RDF rows stay in shared memory, so the systems' launches of a
    // stage need not be split by shared-memory class
    for (size_t i = 0; i < n; ++i)
        if (active[i]) bt->hs[i]->smem_groups = 0;
    // rec[j][i]: the stages of system i's chunk j
    std::vector<std::vector<std::vector<Step>>> rec(nchunks, std::vector<std::vector<Step>>(n));
    for (size_t j = 0; j < nchunks; ++j) {
        const std::vector<Step> *shape = nullptr;
        for (size_t i = 0; i < n; ++i) {
            if (!active[i] || j >= st[i].chunks.size()) continue;
            record_chunk(bt->hs[i], st[i], st[i].chunks[j], rec[j][i]);
            const std::vector<Step> &r = rec[j][i];
            if (!shape) shape = &r;
            else {
                if (r.size() != shape->size()) return false;
                for (size_t k = 0; k < r.size(); ++k)
                    if (r[k].kernel != (*shape)[k].kernel) return false;
            }
        }
    }
    // the systems in order of decreasing size: a fused launch dispatches its
    // blocks roughly in table order, so the largest systems' work starts
    // first and the smaller ones fill the SMs as it drains
    std::vector<size_t> order;
    for (size_t i = 0; i < n; ++i)
        if (active[i]) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return bt->hs[a]->Ns + bt->hs[a]->Nv > bt->hs[b]->Ns + bt->hs[b]->Nv;
    });
    // the work tables of the round, laid out in one pinned buffer
    struct Launch {
        int kernel, kid;
        size_t off;
        int n;
        long long blocks;
        size_t smem;
    };
    std::vector<Launch> plan;
    std::vector<unsigned char> host;
    auto put = [&](const void *p, size_t bytes) {
        const size_t off = (host.size() + 255) & ~(size_t)255;
        host.resize(off + bytes);
        memcpy(host.data() + off, p, bytes);
        return off;
    };
    for (size_t j = 0; j < nchunks; ++j) {
        size_t nsteps = 0;
        for (size_t i = 0; i < n; ++i) nsteps = std::max(nsteps, rec[j][i].size());
        for (size_t k = 0; k < nsteps; ++k) {
            // the kernels of this stage across the systems, in order of first
            // appearance, each with the systems' shared memory in 32 KB classes:
            // a launch asks for its largest class, and a system with a small
            // histogram does not lower the occupancy of those with none
            auto smem_class = [](size_t b) { return (int)((b + 32767) / 32768); };
            std::vector<std::pair<int, int>> kids;
            bool zero = false;
            for (size_t i = 0; i < n; ++i) {
                if (rec[j][i].size() <= k) continue;
                const Step &s = rec[j][i][k];
                if (!s.kernel) zero = true;
                else {
                    const std::pair<int, int> key(s.kid, smem_class(s.smem));
                    if (std::find(kids.begin(), kids.end(), key) == kids.end()) kids.push_back(key);
                }
            }
            if (zero) {
                std::vector<MZero> zs;
                for (size_t i : order)
                    if (rec[j][i].size() > k) zs.push_back({rec[j][i][k].zp, (long long)rec[j][i][k].zbytes});
                Launch L{};
                L.n = (int)zs.size();
                L.off = put(zs.data(), zs.size() * sizeof(MZero));
                plan.push_back(L);
                continue;
            }
            for (const auto &key : kids) {
                Launch L{};
                L.kernel = 1;
                L.kid = key.first;
                std::vector<MTask> ts;
                long long blocks = 0;
                for (size_t i : order) {
                    if (rec[j][i].size() <= k || rec[j][i][k].kid != key.first ||
                        smem_class(rec[j][i][k].smem) != key.second)
                        continue;
                    const Step &s = rec[j][i][k];
                    MTask t;
                    t.a = s.a;
                    t.grid = make_uint3(s.grid.x, s.grid.y, s.grid.z);
                    t.first = blocks;
                    blocks += (long long)s.grid.x * s.grid.y * s.grid.z;
                    ts.push_back(t);
                    L.smem = std::max(L.smem, s.smem);
                }
                L.n = (int)ts.size();
                L.blocks = blocks;
                L.off = put(ts.data(), ts.size() * sizeof(MTask));
                plan.push_back(L);
            }
        }
    }
    // the tables to the device, ahead of the graph on the batch stream
    if (host.size() > bt->tab_cap) {
        CM_CUDA(cudaStreamSynchronize(bt->stream));
        if (bt->h_tab) cudaFreeHost(bt->h_tab);
        if (bt->d_tab) cudaFree(bt->d_tab);
        bt->h_tab = bt->d_tab = nullptr;
        bt->tab_cap = 0;
        const size_t cap = host.size() * 3 / 2 + 4096;
        CM_CUDA(cudaMallocHost(&bt->h_tab, cap));
        CM_CUDA(cudaMalloc(&bt->d_tab, cap));
        bt->tab_cap = cap;
    }
    CM_CUDA(cudaEventSynchronize(bt->tab_copied));  // the previous round's copy has read the host table
    memcpy(bt->h_tab, host.data(), host.size());
    CM_CUDA(cudaMemcpyAsync(bt->d_tab, bt->h_tab, host.size(), cudaMemcpyHostToDevice, bt->stream));
    CM_CUDA(cudaEventRecord(bt->tab_copied, bt->stream));
    for (size_t i = 0; i < n; ++i)
        if (active[i])
            for (const Chunk &c : st[i].chunks) open_class(bt->hs[i], c.weight);
    CM_CUDA(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t g = nullptr;
    try {
        unsigned char *base = (unsigned char *)bt->d_tab;
        for (const Launch &L : plan) {
            if (L.kernel && L.blocks == 0) continue;
            if (!L.kernel) {
                k_multi_zero<<<(unsigned)std::min(L.n, 4096), 256, 0, bt->stream>>>((const MZero *)(base + L.off), L.n);
            } else {
                const unsigned grid = (unsigned)std::min<long long>(L.blocks, (1LL << 31) - 1);
                launch_multi(L.kid, grid, L.smem, bt->stream, (const MTask *)(base + L.off), L.n, L.blocks);
            }
            CM_CUDA(cudaGetLastError());
        }
    } catch (...) {
        cudaStreamEndCapture(bt->stream, &g);
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        throw;
    }
    CM_CUDA(cudaStreamEndCapture(bt->stream, &g));
    bool updated = false;
    if (bt->gexec_fused) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(bt->gexec_fused, g, &info) == cudaSuccess;
        if (!updated) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(bt->gexec_fused);
            bt->gexec_fused = nullptr;
        }
    }
    if (!updated) {
        const cudaError_t e = cudaGraphInstantiate(&bt->gexec_fused, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            bt->gexec_fused = nullptr;
            throw cm_error(CM_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        bt->instantiations++;
    }
    cudaGraphDestroy(g);
    CM_CUDA(cudaGraphLaunch(bt->gexec_fused, bt->stream));
    bt->launches++;
    bt->fused_rounds++;
    bt->stage_launches += (int64_t)plan.size();
    int64_t nsys = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!active[i]) continue;
        ++nsys;
        cm_handle *h = bt->hs[i];
        for (const Chunk &c : st[i].chunks) account_chunk(h, st[i], c);
        h->launches_total += (int64_t)rec[0][i].size();
    }
    bt->fused_systems = nsys;
    return true;
}

// One staging round: frames [r * max_frames, ...) of every system that has
// them, captured as one graph on the batch stream and launched once.
void batch_round(cm_batch *bt, const cm_frames *frames, int r) {
    const size_t n = bt->hs.size();
    std::vector<Staged> st(n);
    std::vector<char> active(n, 0);
    for (size_t i = 0; i < n; ++i) {
        cm_handle *h = bt->hs[i];
        const int64_t f0 = (int64_t)r * h->max_frames;
        if (frames[i].nframes == 0 || f0 >= frames[i].nframes) continue;
        if (h->planned) agrid_grow(h);
        st[i] = stage(h, &frames[i], (int)f0);
        active[i] = 1;
    }
    // outside the capture: each system's stream after its copies and its
    // earlier work, and the batch stream after all of them
    for (size_t i = 0; i < n; ++i) {
        if (!active[i]) continue;
        cm_handle *h = bt->hs[i];
        CM_CUDA(cudaStreamWaitEvent(h->stream, h->ev_copied[st[i].b], 0));
        CM_CUDA(cudaEventRecord(bt->pre[i], h->stream));
        CM_CUDA(cudaStreamWaitEvent(bt->stream, bt->pre[i], 0));
    }
    if (bt->mode == CM_BATCH_FUSED && batch_round_fused(bt, st, active)) {
        CM_CUDA(cudaEventRecord(bt->after, bt->stream));
        for (size_t i = 0; i < n; ++i) {
            if (!active[i]) continue;
            cm_handle *h = bt->hs[i];
            CM_CUDA(cudaStreamWaitEvent(h->stream, bt->after, 0));
            CM_CUDA(cudaEventRecord(h->ev_done[st[i].b], h->stream));
        }
        return;
    }
    CM_CUDA(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t g = nullptr;
    try {
        CM_CUDA(cudaEventRecord(bt->fork, bt->stream));
        for (size_t i = 0; i < n; ++i) {
            if (!active[i]) continue;
            cm_handle *h = bt->hs[i];
            CM_CUDA(cudaStreamWaitEvent(h->stream, bt->fork, 0));
            for (const Chunk &c : st[i].chunks) {
                open_class(h, c.weight);
                run_staged_chunk(h, st[i], c);
                account_chunk(h, st[i], c);
            }
            CM_CUDA(cudaEventRecord(bt->join[i], h->stream));
            CM_CUDA(cudaStreamWaitEvent(bt->stream, bt->join[i], 0));
        }
    } catch (...) {
        cudaStreamEndCapture(bt->stream, &g);
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        throw;
    }
    CM_CUDA(cudaStreamEndCapture(bt->stream, &g));
    bool updated = false;
    if (bt->gexec) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(bt->gexec, g, &info) == cudaSuccess;
        if (!updated) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(bt->gexec);
            bt->gexec = nullptr;
        }
    }
    if (!updated) {
        const cudaError_t e = cudaGraphInstantiate(&bt->gexec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            bt->gexec = nullptr;
            throw cm_error(CM_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        bt->instantiations++;
    }
    cudaGraphDestroy(g);
    CM_CUDA(cudaGraphLaunch(bt->gexec, bt->stream));
    bt->launches++;
    CM_CUDA(cudaEventRecord(bt->after, bt->stream));
    for (size_t i = 0; i < n; ++i) {
        if (!active[i]) continue;
        cm_handle *h = bt->hs[i];
        CM_CUDA(cudaStreamWaitEvent(h->stream, bt->after, 0));
        CM_CUDA(cudaEventRecord(h->ev_done[st[i].b], h->stream));
    }
}

template <typename F>
int batch_guarded(cm_batch *b, F &&fn) {
    if (!b) {
        g_create_error = "NULL batch";
        return CM_EINVAL;
    }
    try {
        CM_CUDA(cudaSetDevice(b->device));
        fn();
        return CM_OK;
    } catch (const cm_error &e) {
        b->err = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        b->err = "host allocation failed";
        return CM_ENOMEM;
    } catch (const std::exception &e) {
        b->err = e.what();
        return CM_ECUDA;
    }
}

}  // namespace

extern "C" {

int cm_create(const cm_system_desc *desc, cm_handle **out) {
    if (!out) {
        g_create_error = "NULL output pointer";
        return CM_EINVAL;
    }
    *out = nullptr;
    cm_handle *h = nullptr;
    try {
        check_desc(desc);
        h = new cm_handle();
        h->d = *desc;
        h->device = desc->device;
        h->Ns = (int64_t)desc->solute_nmols * desc->solute_natomspermol;
        h->Nv = (int64_t)desc->solvent_nmols * desc->solvent_natomspermol;
        h->mddf = desc->mode == CM_MODE_MDDF;
        h->timing = desc->kernel_timing != 0;
        // per-launch timing events cannot sit inside a captured chain
        h->graphs = desc->launch == CM_LAUNCH_GRAPH || (desc->launch == CM_LAUNCH_AUTO && !h->timing);
        if (desc->launch == CM_LAUNCH_GRAPH && h->timing)
            throw cm_error(CM_EINVAL, "kernel_timing needs stream launches (launch = CM_LAUNCH_STREAM or AUTO)");
        if (desc->solute_group_offsets) {
            copy_csr(desc->solute_natomspermol, desc->solute_ngroups, desc->solute_group_offsets, desc->solute_groups, h->gs_off,
                     h->gs_idx, "solute");
            h->Gs = desc->solute_ngroups;
        } else {
            h->Gs = desc->solute_natomspermol;
        }
        if (desc->solvent_group_offsets) {
            copy_csr(h->Nv, desc->solvent_ngroups, desc->solvent_group_offsets, desc->solvent_groups, h->gv_off, h->gv_idx, "solvent");
            h->Gv = desc->solvent_ngroups;
        } else {
            h->Gv = desc->solvent_natomspermol;
        }
        if (desc->autocorrelation && h->Gv != h->Gs)
            throw cm_error(CM_EINVAL, "in self mode the solvent groups must describe the solute selection");
        int rg = desc->regime;
        if (rg == CM_REGIME_AUTO)
            rg = (desc->solute_natomspermol <= kMaxSmallMol && desc->solvent_natomspermol <= kMaxSmallMol) ? CM_REGIME_PAIRS : CM_REGIME_ATOMS;
        if (rg == CM_REGIME_PAIRS && (desc->solute_natomspermol > kMaxSmallMol || desc->solvent_natomspermol > kMaxSmallMol))
            throw cm_error(CM_EINVAL, "the PAIRS layout supports at most 32 atoms per molecule");
        h->regime = rg;
        h->ndist_max = h->mddf ? std::max(1, std::min(desc->solute_nmols, desc->n_random_samples)) : 0;
        CM_CUDA(cudaSetDevice(h->device));
        CM_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        CM_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; ++i) {
            CM_CUDA(cudaEventCreateWithFlags(&h->ev_copied[i], cudaEventDisableTiming));
            CM_CUDA(cudaEventCreateWithFlags(&h->ev_done[i], cudaEventDisableTiming));
            CM_CUDA(cudaEventRecord(h->ev_copied[i], h->stream));
            CM_CUDA(cudaEventRecord(h->ev_done[i], h->stream));
        }
        // histogram layout
        int64_t nb = desc->nbins;
        int64_t Gv = desc->autocorrelation ? 0 : h->Gv;
        h->o_md = 0;
        h->o_mdr = nb;
        h->o_rdf = 2 * nb;
        h->o_rdfr = 3 * nb;
        h->o_gs = 4 * nb;
        h->o_gsr = h->o_gs + h->Gs * nb;
        h->o_gv = h->o_gsr + h->Gs * nb;
        h->o_gvr = h->o_gv + Gv * nb;
        h->hist_n = h->o_gvr + Gv * nb;
        dev_alloc(h, h->hist, h->hist_n * 8);
        dev_alloc(h, h->sums, h->hist_n * 8);
        dev_alloc(h, h->stats, ST_N * 8);
        dev_alloc(h, h->errflag, 8);
        if (desc->precision == CM_PRECISION_FP32_GUARD) {
            dev_alloc(h, h->hist_snap, h->hist_n * 8);
            dev_alloc(h, h->stats_snap, ST_N * 8);
        }
        CM_CUDA(cudaMemsetAsync(h->hist.p, 0, h->hist_n * 8, h->stream));
        CM_CUDA(cudaMemsetAsync(h->sums.p, 0, h->hist_n * 8, h->stream));
        CM_CUDA(cudaMemsetAsync(h->stats.p, 0, ST_N * 8, h->stream));
        CM_CUDA(cudaMemsetAsync(h->errflag.p, 0, 8, h->stream));
        upload_groups(h);
        CM_CUDA(cudaStreamSynchronize(h->stream));  // this handle only: other handles keep running
        *out = h;
        return CM_OK;
    } catch (const cm_error &e) {
        g_create_error = e.msg;
        if (h) { free_all(h); delete h; }
        return e.code;
    } catch (const std::bad_alloc &) {
        g_create_error = "host allocation failed";
        if (h) { free_all(h); delete h; }
        return CM_ENOMEM;
    }
}

int cm_submit_frames(cm_handle *h, const cm_frames *frames) {
    return guarded(h, [&] { submit(h, frames); });
}

int cm_synchronize(cm_handle *h) {
    return guarded(h, [&] { check_device_error(h); });
}

int cm_set_dcd_layout(cm_handle *h, const cm_dcd_layout *L) {
    return guarded(h, [&] {
        if (!L) throw cm_error(CM_EINVAL, "NULL layout");
        if (L->natoms < 1 || L->natoms >= (1LL << 31)) throw cm_error(CM_EINVAL, "natoms out of range");
        if (L->frame_bytes < 12 * L->natoms || L->frame_bytes % 4) throw cm_error(CM_EINVAL, "frame_bytes must hold three float32 arrays and be a multiple of 4");
        const int64_t off[3] = {L->x_offset, L->y_offset, L->z_offset};
        for (int k = 0; k < 3; ++k)
            if (off[k] < 0 || off[k] % 4 || off[k] + 4 * L->natoms > L->frame_bytes)
                throw cm_error(CM_EINVAL, "x/y/z offsets must be multiples of 4 with the arrays inside the frame");
        if (!L->solute_atoms) throw cm_error(CM_EINVAL, "solute_atoms is required");
        if (h->d.autocorrelation != (L->solvent_atoms == nullptr))
            throw cm_error(CM_EINVAL, "solvent_atoms is required for a cross MDDF and must be NULL in self mode");
        if (h->planned && h->coord_elem != 4) throw cm_error(CM_ESTATE, "this handle was planned for float64 frames");
        auto take = [&](const int32_t *src, int64_t n, std::vector<int32_t> &dst, DevBuf &dev) {
            dst.assign(src, src + n);
            for (int32_t a : dst)
                if (a < 0 || a >= L->natoms) throw cm_error(CM_EINVAL, "selection atom index outside the DCD frame");
            dev_alloc(h, dev, (size_t)n * 4);
            CM_CUDA(cudaMemcpyAsync(dev.p, dst.data(), (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
        };
        take(L->solute_atoms, h->Ns, h->dcd_s, h->dcd_sidx);
        if (!h->d.autocorrelation) take(L->solvent_atoms, h->Nv, h->dcd_v, h->dcd_vidx);
        CM_CUDA(cudaStreamSynchronize(h->stream));
        h->dcd_natoms = L->natoms;
        h->dcd_frame_bytes = L->frame_bytes;
        for (int k = 0; k < 3; ++k) h->dcd_off[k] = off[k];
        h->dcd_swap = L->big_endian ? 1 : 0;
        h->dcd = true;
    });
}

int cm_batch_create(cm_handle *const *handles, int32_t nhandles, cm_batch **out) {
    if (!out || !handles || nhandles < 1) {
        g_create_error = "cm_batch_create needs an output pointer and at least one handle";
        return CM_EINVAL;
    }
    *out = nullptr;
    cm_batch *b = nullptr;
    try {
        for (int i = 0; i < nhandles; ++i) {
            if (!handles[i]) throw cm_error(CM_EINVAL, "NULL handle in the batch");
            if (handles[i]->device != handles[0]->device) throw cm_error(CM_EINVAL, "the handles of a batch share one device");
            if (handles[i]->timing) throw cm_error(CM_EINVAL, "handles with kernel_timing cannot be batched");
            for (int j = 0; j < i; ++j)
                if (handles[j] == handles[i]) throw cm_error(CM_EINVAL, "a handle appears twice in the batch");
        }
        b = new cm_batch();
        b->hs.assign(handles, handles + nhandles);
        b->device = handles[0]->device;
        CM_CUDA(cudaSetDevice(b->device));
        CM_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        CM_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        CM_CUDA(cudaEventCreateWithFlags(&b->after, cudaEventDisableTiming));
        CM_CUDA(cudaEventCreateWithFlags(&b->tab_copied, cudaEventDisableTiming));
        b->pre.assign(nhandles, nullptr);
        b->join.assign(nhandles, nullptr);
        for (int i = 0; i < nhandles; ++i) {
            CM_CUDA(cudaEventCreateWithFlags(&b->pre[i], cudaEventDisableTiming));
            CM_CUDA(cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming));
        }
        *out = b;
        return CM_OK;
    } catch (const cm_error &e) {
        g_create_error = e.msg;
        if (b) { batch_free(b); delete b; }
        return e.code;
    } catch (const std::bad_alloc &) {
        g_create_error = "host allocation failed";
        if (b) { batch_free(b); delete b; }
        return CM_ENOMEM;
    }
}

int cm_batch_submit(cm_batch *b, const cm_frames *frames) {
    NvtxRange range("cm: batch submit (all systems)");
    return batch_guarded(b, [&] {
        if (!frames) throw cm_error(CM_EINVAL, "NULL frames");
        int rounds = 0;
        for (size_t i = 0; i < b->hs.size(); ++i) {
            cm_handle *h = b->hs[i];
            try {
                check_frames(h, &frames[i]);
            } catch (const cm_error &e) {
                throw cm_error(e.code, "system " + std::to_string(i) + ": " + e.msg);
            }
            if (frames[i].nframes > 0)
                rounds = std::max<int>(rounds, (frames[i].nframes + h->max_frames - 1) / h->max_frames);
        }
        for (int r = 0; r < rounds; ++r) batch_round(b, frames, r);
    });
}

int cm_batch_set_mode(cm_batch *b, int32_t mode) {
    if (!b) return CM_EINVAL;
    if (mode != CM_BATCH_FUSED && mode != CM_BATCH_STREAMS) {
        b->err = "unknown batch mode";
        return CM_EINVAL;
    }
    b->mode = mode;
    return CM_OK;
}

int cm_batch_fused_stats(const cm_batch *b, int64_t *fused_rounds, int64_t *stage_launches, int64_t *systems) {
    if (!b) return CM_EINVAL;
    if (fused_rounds) *fused_rounds = b->fused_rounds;
    if (stage_launches) *stage_launches = b->stage_launches;
    if (systems) *systems = b->fused_systems;
    return CM_OK;
}

int cm_batch_graph_stats(const cm_batch *b, int64_t *graph_launches, int64_t *graph_instantiations) {
    if (!b) return CM_EINVAL;
    if (graph_launches) *graph_launches = b->launches;
    if (graph_instantiations) *graph_instantiations = b->instantiations;
    return CM_OK;
}

int cm_batch_destroy(cm_batch *b) {
    if (!b) return CM_OK;
    cudaSetDevice(b->device);
    batch_free(b);
    delete b;
    return CM_OK;
}

const char *cm_batch_last_error(const cm_batch *b) {
    if (!b) return g_create_error.c_str();
    return b->err.c_str();
}

int cm_read_counts(cm_handle *h, cm_counts *out) {
    return guarded(h, [&] {
        NvtxRange range("cm: read counts");
        if (!out) throw cm_error(CM_EINVAL, "NULL output");
        check_device_error(h);
        std::vector<unsigned long long> acc(h->hist_n);
        std::vector<double> sums(h->hist_n);
        CM_CUDA(cudaMemcpy(acc.data(), h->hist.p, h->hist_n * 8, cudaMemcpyDeviceToHost));
        CM_CUDA(cudaMemcpy(sums.data(), h->sums.p, h->hist_n * 8, cudaMemcpyDeviceToHost));
        std::vector<double> tot(h->hist_n);
        for (int64_t i = 0; i < h->hist_n; ++i)
            tot[i] = (h->class_open && acc[i]) ? sums[i] + h->class_w * ((double)acc[i] / 2.0) : sums[i];
        const int64_t nb = h->d.nbins;
        auto put = [&](double *dst, int64_t off, int64_t n) {
            if (dst) memcpy(dst, tot.data() + off, n * 8);
        };
        put(out->md_count, h->o_md, nb);
        put(out->md_count_random, h->o_mdr, nb);
        put(out->rdf_count, h->o_rdf, nb);
        put(out->rdf_count_random, h->o_rdfr, nb);
        put(out->solute_group_count, h->o_gs, h->Gs * nb);
        put(out->solute_group_count_random, h->o_gsr, h->Gs * nb);
        if (h->d.autocorrelation) {
            if (out->solvent_group_count) memset(out->solvent_group_count, 0, h->Gv * nb * 8);
            if (out->solvent_group_count_random) memset(out->solvent_group_count_random, 0, h->Gv * nb * 8);
        } else {
            put(out->solvent_group_count, h->o_gv, h->Gv * nb);
            put(out->solvent_group_count_random, h->o_gvr, h->Gv * nb);
        }
        out->volume_total = h->volume_total;
        out->weight_total = h->weight_total;
        out->frames = h->frames;
    });
}

// Launch k_finalize on the handle's accumulators into h->final_out (packed
// FinalVec vectors, group blocks, FinalScalar scalars); returns its length in
// doubles.  Asynchronous on the handle's stream.
static int64_t launch_finalize(cm_handle *h, double frame_weight_sum) {
    NvtxRange range("cm: finalresults (k_finalize)");
    if (!(frame_weight_sum >= 0.0) || !std::isfinite(frame_weight_sum))
        throw cm_error(CM_EINVAL, "frame_weight_sum must be finite and non-negative");
    check_device_error(h);
    const cm_system_desc &d = h->d;
    const int64_t nb = d.nbins, Gs = h->Gs, Gv = d.autocorrelation ? h->Gs : h->Gv;
    const int64_t n = FV_NVEC * nb + 2 * Gs * nb + 2 * Gv * nb + FS_NSCALAR;
    FinalJob J{};
    J.acc = P<unsigned long long>(h->hist);
    J.sums = P<double>(h->sums);
    J.class_w = h->class_w;
    J.class_open = h->class_open ? 1 : 0;
    J.nbins = d.nbins;
    J.Gs = h->Gs;
    J.Gv = d.autocorrelation ? 0 : h->Gv;
    J.autocorrelation = d.autocorrelation;
    J.mddf_mode = h->mddf ? 1 : 0;
    J.usecutoff = d.usecutoff;
    J.o_md = h->o_md; J.o_mdr = h->o_mdr; J.o_rdf = h->o_rdf; J.o_rdfr = h->o_rdfr;
    J.o_gs = h->o_gs; J.o_gsr = h->o_gsr; J.o_gv = h->o_gv; J.o_gvr = h->o_gvr;
    J.binstep = d.binstep;
    J.dbulk = d.dbulk;
    J.Q = frame_weight_sum > 0.0 ? frame_weight_sum : h->weight_total;
    J.volume_sum = h->volume_total;
    J.solute_nmols = d.solute_nmols;
    J.solvent_nmols = d.solvent_nmols;
    J.solvent_nmols_samples = d.autocorrelation ? d.solvent_nmols - 1 : d.solvent_nmols;  // src/results.jl:230-237
    J.nrandom = d.n_random_samples;
    J.units_f = 6.022140857e23 / 1e24;  // units.Angs3tocm3permol = mole / Angs3tocm3 (src/io.jl:6-14)
    J.ibulk = std::max(1, (int)std::ceil((d.dbulk + 0.5 * d.binstep) / d.binstep));  // setbin (src/results.jl:28)
    dev_alloc(h, h->final_out, (size_t)n * 8);
    dev_alloc(h, h->final_job, sizeof(FinalJob));
    J.out = P<double>(h->final_out);
    CM_CUDA(cudaMemcpyAsync(h->final_job.p, &J, sizeof(J), cudaMemcpyHostToDevice, h->stream));
    k_finalize<<<1, 256, 0, h->stream>>>(P<FinalJob>(h->final_job));
    CM_CUDA(cudaGetLastError());
    return n;
}

int cm_read_results(cm_handle *h, double frame_weight_sum, cm_results *out) {
    return guarded(h, [&] {
        if (!out) throw cm_error(CM_EINVAL, "NULL output");
        const int64_t n = launch_finalize(h, frame_weight_sum);
        const int64_t nb = h->d.nbins, Gs = h->Gs, Gv = h->d.autocorrelation ? h->Gs : h->Gv;
        std::vector<double> v(n);
        CM_CUDA(cudaMemcpyAsync(v.data(), h->final_out.p, (size_t)n * 8, cudaMemcpyDeviceToHost, h->stream));
        CM_CUDA(cudaStreamSynchronize(h->stream));
        auto put = [&](double *dst, int64_t off, int64_t len) {
            if (dst) memcpy(dst, v.data() + off, len * 8);
        };
        double *arr[FV_NVEC] = {out->d, out->md_count, out->md_count_random, out->coordination_number,
                                out->coordination_number_random, out->mddf, out->kb, out->rdf_count, out->rdf_count_random,
                                out->sum_rdf_count, out->sum_rdf_count_random, out->rdf, out->kb_rdf, out->volume_shell};
        for (int k = 0; k < FV_NVEC; ++k) put(arr[k], k * nb, nb);
        int64_t o = FV_NVEC * nb;
        put(out->solute_group_count, o, Gs * nb);
        put(out->solute_group_count_random, o + Gs * nb, Gs * nb);
        put(out->solvent_group_count, o + 2 * Gs * nb, Gv * nb);
        put(out->solvent_group_count_random, o + 2 * Gs * nb + Gv * nb, Gv * nb);
        const double *sc = v.data() + o + 2 * Gs * nb + 2 * Gv * nb;
        out->volume_total = sc[FS_TOTAL];
        out->volume_bulk = sc[FS_BULK];
        out->volume_domain = sc[FS_DOMAIN];
        out->density_solute = sc[FS_DSOLUTE];
        out->density_solvent = sc[FS_DSOLVENT];
        out->density_solvent_bulk = sc[FS_DSOLVENT_BULK];
        out->density_fix = sc[FS_DENSITY_FIX];
        out->zero_random_bins = (int64_t)sc[FS_ZERO_RANDOM_BINS];
    });
}

int cm_contributions(cm_handle *h, double frame_weight_sum, int32_t nqueries, const cm_contrib_query *queries,
                     double *out) {
    NvtxRange range("cm: contributions (k_contrib)");
    return guarded(h, [&] {
        if (nqueries < 1 || !queries || !out) throw cm_error(CM_EINVAL, "contributions need at least one query and an output");
        if (nqueries > 65535) throw cm_error(CM_EINVAL, "at most 65535 queries per call");
        const cm_system_desc &d = h->d;
        const int Gs = (int)h->Gs, Gv = d.autocorrelation ? (int)h->Gs : (int)h->Gv;
        std::vector<ContribQuery> q(nqueries);
        std::vector<int> groups;
        for (int k = 0; k < nqueries; ++k) {
            const cm_contrib_query &c = queries[k];
            if (c.side != CM_GROUP_SOLUTE && c.side != CM_GROUP_SOLVENT)
                throw cm_error(CM_EINVAL, "query " + std::to_string(k) + ": side must be CM_GROUP_SOLUTE or CM_GROUP_SOLVENT");
            if (c.type < CM_CONTRIB_MDDF || c.type > CM_CONTRIB_KBI)
                throw cm_error(CM_EINVAL, "query " + std::to_string(k) + ": type must be :mddf (default), :coordination_number, :md_count, :kbi");
            if (c.nterms < 1 || !c.groups)
                throw cm_error(CM_EINVAL, "query " + std::to_string(k) + ": a query sums at least one group");
            const int G = c.side == CM_GROUP_SOLUTE ? Gs : Gv;
            q[k].side = c.side;
            q[k].type = c.type;
            q[k].divide = c.divide ? 1 : 0;
            q[k].nmols = c.side == CM_GROUP_SOLUTE ? (double)d.solute_nmols : (double)d.solvent_nmols;
            q[k].t0 = (int)groups.size();
            for (int t = 0; t < c.nterms; ++t) {
                const int g = c.groups[t];
                if (g < 0 || g >= G)
                    throw cm_error(CM_EINVAL, "query " + std::to_string(k) + ": group " + std::to_string(g + 1) +
                                                  " greater than number of groups (" + std::to_string(G) + ")");
                groups.push_back(g);
            }
            q[k].t1 = (int)groups.size();
        }
        launch_finalize(h, frame_weight_sum);
        const int64_t nb = d.nbins;
        dev_alloc(h, h->contrib_q, q.size() * sizeof(ContribQuery));
        dev_alloc(h, h->contrib_g, groups.size() * sizeof(int));
        dev_alloc(h, h->contrib_out, (size_t)2 * nqueries * nb * 8);
        CM_CUDA(cudaMemcpyAsync(h->contrib_q.p, q.data(), q.size() * sizeof(ContribQuery), cudaMemcpyHostToDevice, h->stream));
        CM_CUDA(cudaMemcpyAsync(h->contrib_g.p, groups.data(), groups.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        ContribJob J{};
        J.fin = P<double>(h->final_out);
        J.nbins = d.nbins;
        J.Gs = Gs;
        J.Gv = Gv;
        J.units_f = 6.022140857e23 / 1e24;  // units.Angs3tocm3permol (src/io.jl:6-14)
        J.q = P<ContribQuery>(h->contrib_q);
        J.groups = P<int>(h->contrib_g);
        J.out = P<double>(h->contrib_out);
        J.scratch = J.out + (int64_t)nqueries * nb;
        k_contrib<<<nqueries, 128, 0, h->stream>>>(J);
        CM_CUDA(cudaGetLastError());
        CM_CUDA(cudaMemcpyAsync(out, h->contrib_out.p, (size_t)nqueries * nb * 8, cudaMemcpyDeviceToHost, h->stream));
        CM_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int cm_read_raw_counts(cm_handle *h, cm_raw_counts *out) {
    return guarded(h, [&] {
        if (!out) throw cm_error(CM_EINVAL, "NULL output");
        if (h->folds > 0) throw cm_error(CM_ESTATE, "raw counts are defined only while all frames carry one weight");
        check_device_error(h);
        std::vector<int64_t> acc(h->hist_n);
        CM_CUDA(cudaMemcpy(acc.data(), h->hist.p, h->hist_n * 8, cudaMemcpyDeviceToHost));
        const int64_t nb = h->d.nbins;
        auto put = [&](int64_t *dst, int64_t off, int64_t n) {
            if (dst) memcpy(dst, acc.data() + off, n * 8);
        };
        put(out->md, h->o_md, nb);
        put(out->md_random, h->o_mdr, nb);
        put(out->rdf, h->o_rdf, nb);
        put(out->rdf_random, h->o_rdfr, nb);
        put(out->solute_group, h->o_gs, h->Gs * nb);
        put(out->solute_group_random, h->o_gsr, h->Gs * nb);
        if (h->d.autocorrelation) {
            if (out->solvent_group) memset(out->solvent_group, 0, h->Gv * nb * 8);
            if (out->solvent_group_random) memset(out->solvent_group_random, 0, h->Gv * nb * 8);
        } else {
            put(out->solvent_group, h->o_gv, h->Gv * nb);
            put(out->solvent_group_random, h->o_gvr, h->Gv * nb);
        }
    });
}

int cm_get_stats(cm_handle *h, cm_stats *out) {
    return guarded(h, [&] {
        if (!out) throw cm_error(CM_EINVAL, "NULL output");
        CM_CUDA(cudaStreamSynchronize(h->stream));
        unsigned long long s[ST_N];
        CM_CUDA(cudaMemcpy(s, h->stats.p, sizeof(s), cudaMemcpyDeviceToHost));
        memset(out, 0, sizeof(*out));
        out->frames = h->frames;
        out->molecule_pairs_evaluated = (int64_t)s[ST_MOLPAIRS];
        out->atom_pairs_evaluated = (int64_t)s[ST_ATOMPAIRS];
        out->hits_real = (int64_t)s[ST_HITS_REAL];
        out->hits_random = (int64_t)s[ST_HITS_RAND];
        out->guard_reevaluations = (int64_t)s[ST_GUARD];
        out->guard_pair_evaluations = (int64_t)s[ST_GUARD_PAIRS];
        double e;
        memcpy(&e, &s[ST_MAXERR], 8);
        out->max_guard_error = e;
        if (h->planned && h->frames > 0) {
            FrameScratch F0;
            CM_CUDA(cudaMemcpy(&F0, h->fscratch.p, sizeof(F0), cudaMemcpyDeviceToHost));
            h->last_guard = F0.g.delta;  // guard band of the last chunk's first frame
        }
        out->guard_band = h->last_guard;
        out->regime = h->regime;
        out->kernels_per_frame = h->kernels_per_frame;
        out->kernel_launches = h->launches_total;
        out->graph_launches = h->graph_launches;
        out->graph_instantiations = h->graph_instantiations;
    });
}

int cm_get_kernel_times(cm_handle *h, cm_kernel_times *out) {
    return guarded(h, [&] {
        if (!out) throw cm_error(CM_EINVAL, "NULL output");
        if (!h->timing) throw cm_error(CM_ESTATE, "kernel timing was not enabled at cm_create");
        timing_drain(h);
        for (int i = 0; i < CM_K_NCLASSES; ++i) {
            out->ms[i] = h->class_ms[i];
            out->launches[i] = h->class_launches[i];
        }
    });
}

int cm_reset(cm_handle *h) {
    return guarded(h, [&] {
        CM_CUDA(cudaMemsetAsync(h->hist.p, 0, h->hist_n * 8, h->stream));
        CM_CUDA(cudaMemsetAsync(h->sums.p, 0, h->hist_n * 8, h->stream));
        CM_CUDA(cudaMemsetAsync(h->stats.p, 0, ST_N * 8, h->stream));
        CM_CUDA(cudaMemsetAsync(h->errflag.p, 0, 8, h->stream));
        CM_CUDA(cudaStreamSynchronize(h->stream));
        h->class_open = false;
        h->class_w = 1.0;
        h->folds = 0;
        h->volume_total = h->weight_total = 0.0;
        h->frames = 0;
        timing_drain(h);
        h->launches_total = 0;
        h->graph_launches = h->graph_instantiations = 0;
        for (int i = 0; i < CM_K_NCLASSES; ++i) {
            h->class_ms[i] = 0.0;
            h->class_launches[i] = 0;
        }
    });
}

int cm_raw_counts_weight(cm_handle *h, double *frame_weight) {
    return guarded(h, [&] {
        if (!frame_weight) throw cm_error(CM_EINVAL, "NULL output");
        if (h->folds > 0) throw cm_error(CM_ESTATE, "raw counts are defined only while all frames carry one weight");
        *frame_weight = h->class_open ? h->class_w : 1.0;
    });
}

int cm_load_raw_counts(cm_handle *h, const cm_raw_counts *in, double frame_weight, int64_t frames, double volume_total) {
    return guarded(h, [&] {
        if (!in || !in->md || !in->md_random || !in->rdf || !in->rdf_random || !in->solute_group ||
            !in->solute_group_random)
            throw cm_error(CM_EINVAL, "md, md_random, rdf, rdf_random, solute_group and solute_group_random are required");
        if (!h->d.autocorrelation && (!in->solvent_group || !in->solvent_group_random))
            throw cm_error(CM_EINVAL, "solvent_group and solvent_group_random are required unless autocorrelation");
        if (!(frame_weight > 0.0) || !std::isfinite(frame_weight)) throw cm_error(CM_EINVAL, "frame_weight must be finite and positive");
        if (frames < 0) throw cm_error(CM_EINVAL, "frames must be >= 0");
        if (!std::isfinite(volume_total)) throw cm_error(CM_EINVAL, "volume_total must be finite");
        const int64_t nb = h->d.nbins;
        std::vector<int64_t> acc(h->hist_n, 0);
        auto get = [&](const int64_t *src, int64_t off, int64_t n) {
            for (int64_t i = 0; i < n; ++i) {
                if (src[i] < 0) throw cm_error(CM_EINVAL, "counts must be non-negative");
                acc[off + i] = src[i];
            }
        };
        get(in->md, h->o_md, nb);
        get(in->md_random, h->o_mdr, nb);
        get(in->rdf, h->o_rdf, nb);
        get(in->rdf_random, h->o_rdfr, nb);
        get(in->solute_group, h->o_gs, h->Gs * nb);
        get(in->solute_group_random, h->o_gsr, h->Gs * nb);
        if (!h->d.autocorrelation) {
            get(in->solvent_group, h->o_gv, h->Gv * nb);
            get(in->solvent_group_random, h->o_gvr, h->Gv * nb);
        }
        check_device_error(h);  // the handle's earlier work is done (synchronised)
        CM_CUDA(cudaMemcpy(h->hist.p, acc.data(), h->hist_n * 8, cudaMemcpyHostToDevice));
        CM_CUDA(cudaMemset(h->sums.p, 0, h->hist_n * 8));
        h->class_open = true;
        h->class_w = frame_weight;
        h->folds = 0;
        h->frames = frames;
        h->weight_total = frame_weight * (double)frames;
        h->volume_total = volume_total;
    });
}

int cm_destroy(cm_handle *h) {
    if (!h) return CM_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return CM_OK;
}

const char *cm_last_error(const cm_handle *h) {
    if (!h) return g_create_error.c_str();
    return h->err.c_str();
}

const char *cm_status_string(int status) {
    switch (status) {
        case CM_OK: return "ok";
        case CM_EINVAL: return "invalid argument";
        case CM_ENOMEM: return "out of memory or over the device memory budget";
        case CM_ECUDA: return "CUDA runtime error";
        case CM_EDEVICE: return "device-side check failed";
        case CM_ESTATE: return "invalid state";
        default: return "unknown status";
    }
}

int64_t cm_device_bytes(const cm_handle *h) { return h ? h->device_bytes : 0; }

int cm_grid3d(const cm_grid3d_desc *D, cm_grid3d_out *out) {
    NvtxRange range("cm: grid3D (k_grid3d)");
    if (!D || !out) {
        g_create_error = "NULL argument";
        return CM_EINVAL;
    }
    std::vector<std::pair<void *, size_t>> taken;  // device blocks from the cache, returned at the end
    cudaStream_t st = nullptr;
    int prev = -1;
    auto release = [&] {
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        for (auto &b : taken) blocks().put(D->device, false, b.first, b.second);
        if (prev >= 0) cudaSetDevice(prev);
    };
    try {
        if (D->natoms < 1 || D->natoms >= (1LL << 31) || !D->xyz || !D->atom_type || !D->table || !D->d)
            throw cm_error(CM_EINVAL, "natoms, xyz, atom_type, table and d are required");
        if (D->nbins < 2 || D->ntypes < 1) throw cm_error(CM_EINVAL, "nbins must be >= 2 and ntypes >= 1");
        if (!(D->step > 0.0) || !(D->dmax > D->dmin) || !(D->dmin >= 0.0))
            throw cm_error(CM_EINVAL, "need step > 0 and 0 <= dmin < dmax");
        if (!(D->d[0] <= D->dmin) || !(D->dmax < D->d[D->nbins - 1]))
            throw cm_error(CM_EINVAL, "dmin and dmax must lie within the bin distances (d[0] <= dmin, dmax < d[end])");
        for (int64_t i = 0; i < D->natoms; ++i)
            if (D->atom_type[i] < 0 || D->atom_type[i] >= D->ntypes) throw cm_error(CM_EINVAL, "atom_type out of range");
        // grid (PDBTools.maxmin and the point count of src/tools/grid3D.jl:76-77)
        double xmin[3], xmax[3];
        for (int k = 0; k < 3; ++k) xmin[k] = xmax[k] = D->xyz[k];
        for (int64_t i = 1; i < D->natoms; ++i)
            for (int k = 0; k < 3; ++k) {
                xmin[k] = std::min(xmin[k], D->xyz[3 * i + k]);
                xmax[k] = std::max(xmax[k], D->xyz[3 * i + k]);
            }
        GridJob J{};
        for (int k = 0; k < 3; ++k) {
            J.n[k] = (int64_t)std::ceil((xmax[k] - xmin[k] + 2 * D->dmax) / D->step + 1);
            J.origin[k] = xmin[k] - D->dmax;
            out->n[k] = J.n[k];
            out->origin[k] = J.origin[k];
        }
        J.step = D->step;
        J.dmin = D->dmin;
        J.dmax = D->dmax;
        J.nbins = D->nbins;
        // atoms binned into cells a little wider than dmax
        J.cell = D->dmax * 1.001;
        for (int k = 0; k < 3; ++k) J.c[k] = (int64_t)std::floor((xmax[k] - J.origin[k]) / J.cell) + 2;
        const int64_t ncell = J.c[0] * J.c[1] * J.c[2];
        if (ncell > (1LL << 28)) throw cm_error(CM_EINVAL, "grid box too large for its cell list");
        std::vector<int64_t> acell(D->natoms);
        std::vector<int> cstart(ncell + 1, 0);
        for (int64_t i = 0; i < D->natoms; ++i) {
            int64_t ci[3];
            for (int k = 0; k < 3; ++k)
                ci[k] = std::min<int64_t>(J.c[k] - 1, std::max<int64_t>(0, (int64_t)std::floor((D->xyz[3 * i + k] - J.origin[k]) / J.cell)));
            acell[i] = (ci[2] * J.c[1] + ci[1]) * J.c[0] + ci[0];
            cstart[acell[i] + 1]++;
        }
        for (int64_t c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
        std::vector<int> fill(cstart.begin(), cstart.end() - 1);
        std::vector<d4> sorted(D->natoms);
        for (int64_t i = 0; i < D->natoms; ++i)
            sorted[fill[acell[i]]++] = cmgeom::make_d4(D->xyz[3 * i], D->xyz[3 * i + 1], D->xyz[3 * i + 2], (double)i);
        const int64_t total = J.n[0] * J.n[1] * J.n[2];
        CM_CUDA(cudaGetDevice(&prev));
        CM_CUDA(cudaSetDevice(D->device));
        CM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        auto take = [&](size_t bytes) {
            size_t got = 0;
            void *p = blocks().get(D->device, false, bytes, &got);
            if (!p) throw cm_error(CM_ENOMEM, "out of device memory");
            taken.push_back({p, got});
            return p;
        };
        auto up = [&](const void *src, size_t bytes) {
            void *p = take(bytes);
            CM_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, st));
            return p;
        };
        J.cstart = (const int *)up(cstart.data(), cstart.size() * 4);
        J.atoms = (const d4 *)up(sorted.data(), sorted.size() * sizeof(d4));
        J.type = (const int *)up(D->atom_type, (size_t)D->natoms * 4);
        J.table = (const double *)up(D->table, (size_t)D->ntypes * D->nbins * 8);
        J.d = (const double *)up(D->d, (size_t)D->nbins * 8);
        J.cap = total;
        J.count = (unsigned long long *)take(8);
        CM_CUDA(cudaMemsetAsync(J.count, 0, 8, st));
        J.out_point = (long long *)take((size_t)total * 8);
        J.out_atom = (int *)take((size_t)total * 4);
        J.out_r = (double *)take((size_t)total * 8);
        J.out_v = (double *)take((size_t)total * 8);
        int sms = 0;
        CM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device));
        const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sms * 16);
        k_grid3d<<<grid, 256, 0, st>>>(J);
        CM_CUDA(cudaGetLastError());
        unsigned long long cnt = 0;
        CM_CUDA(cudaMemcpyAsync(&cnt, J.count, 8, cudaMemcpyDeviceToHost, st));
        CM_CUDA(cudaStreamSynchronize(st));
        out->count = (int64_t)cnt;
        if ((int64_t)cnt > out->capacity) throw cm_error(CM_ENOMEM, "cm_grid3d_out.capacity below the kept points (see count)");
        std::vector<long long> pt(cnt);
        std::vector<int> at(cnt);
        std::vector<double> rr(cnt), vv(cnt);
        if (cnt) {
            CM_CUDA(cudaMemcpyAsync(pt.data(), J.out_point, cnt * 8, cudaMemcpyDeviceToHost, st));
            CM_CUDA(cudaMemcpyAsync(at.data(), J.out_atom, cnt * 4, cudaMemcpyDeviceToHost, st));
            CM_CUDA(cudaMemcpyAsync(rr.data(), J.out_r, cnt * 8, cudaMemcpyDeviceToHost, st));
            CM_CUDA(cudaMemcpyAsync(vv.data(), J.out_v, cnt * 8, cudaMemcpyDeviceToHost, st));
            CM_CUDA(cudaStreamSynchronize(st));
        }
        std::vector<int64_t> order(cnt);
        for (int64_t i = 0; i < (int64_t)cnt; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return pt[a] < pt[b]; });
        for (int64_t i = 0; i < (int64_t)cnt; ++i) {
            const int64_t j = order[i];
            if (out->point) out->point[i] = pt[j];
            if (out->atom) out->atom[i] = at[j];
            if (out->distance) out->distance[i] = rr[j];
            if (out->value) out->value[i] = vv[j];
        }
        release();
        return CM_OK;
    } catch (const cm_error &e) {
        g_create_error = e.msg;
        release();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_create_error = "host allocation failed";
        release();
        return CM_ENOMEM;
    }
}

int cm_memory_cache(int32_t device, int32_t release, int64_t *cached_device_bytes, int64_t *cached_host_bytes) {
    if (device < 0 || device >= BlockCache::kMaxDevices) {
        g_create_error = "device index out of range";
        return CM_EINVAL;
    }
    if (release) {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        blocks().release(device, false);
        blocks().release(device, true);
        if (prev >= 0) cudaSetDevice(prev);
    }
    if (cached_device_bytes) *cached_device_bytes = (int64_t)blocks().cached(device, false);
    if (cached_host_bytes) *cached_host_bytes = (int64_t)blocks().cached(device, true);
    return CM_OK;
}

int cm_measure_fp32_peak(int32_t device, double ms_target, double *tflops) {
    if (!tflops) return CM_EINVAL;
    try {
        CM_CUDA(cudaSetDevice(device));
        int sms = 0;
        CM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        const int block = 256, blocks = sms * 8;
        float *sink = nullptr;
        CM_CUDA(cudaMalloc(&sink, sizeof(float) * block * blocks));
        cudaStream_t st;
        CM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        cudaEvent_t a, b;
        CM_CUDA(cudaEventCreate(&a));
        CM_CUDA(cudaEventCreate(&b));
        int iters = 1 << 12;
        double best = 0.0;
        for (int rep = 0; rep < 6; ++rep) {
            CM_CUDA(cudaEventRecord(a, st));
            k_fma_probe<<<blocks, block, 0, st>>>(sink, iters, 1.0000001f);
            CM_CUDA(cudaEventRecord(b, st));
            CM_CUDA(cudaEventSynchronize(b));
            float ms = 0.f;
            CM_CUDA(cudaEventElapsedTime(&ms, a, b));
            double flops = (double)blocks * block * iters * kProbeChains * 2.0;
            best = std::max(best, flops / (ms * 1e-3) / 1e12);
            if (ms < ms_target / 6.0 && iters < (1 << 24)) iters *= 2;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaStreamDestroy(st);
        cudaFree(sink);
        *tflops = best;
        return CM_OK;
    } catch (const cm_error &e) {
        g_create_error = e.msg;
        return e.code;
    }
}

void *cm_stream(cm_handle *h) { return h ? (void *)h->stream : nullptr; }

int cm_frame_counts_noalloc(const cm_system_desc *desc, const cm_frames *frame, int64_t *counts, int64_t counts_len,
                            void *stream) {
    return noalloc_frame(desc, frame, counts, counts_len, stream);
}

int cm_autotune(const cm_system_desc *desc, const cm_frames *sample, cm_tuning *out) {
    if (!desc || !sample || !out) {
        g_create_error = "NULL argument";
        return CM_EINVAL;
    }
    memset(out, 0, sizeof(*out));
    const bool atoms = desc->regime == CM_REGIME_ATOMS ||
                       (desc->regime == CM_REGIME_AUTO &&
                        (desc->solute_natomspermol > kMaxSmallMol || desc->solvent_natomspermol > kMaxSmallMol));
    // ATOMS: cutoff / (lcell k), each with both evaluation schedules;
    // PAIRS: the molecule cell and smaller ones, in self mode each with both
    // real-pass schedules (home-cell tiles, warps per molecule)
    const int cand_atoms[] = {100, 80, 50, 34};
    const int cand_pairs[] = {100, 75, 60, 50};
    const int *cand = atoms ? cand_atoms : cand_pairs;
    const bool two_real = !atoms && desc->autocorrelation && desc->precision == CM_PRECISION_FP32_GUARD;
    // a single solute molecule in the FP32 search: the walk with both
    // schedules at two cell sizes, and the candidate grid at several fine-cell
    // counts (the walk schedule then only serves the records inside the band)
    const bool grid = atoms && desc->solute_nmols == 1 && !desc->autocorrelation &&
                      desc->precision == CM_PRECISION_FP32_GUARD && desc->atoms_grid >= 0;
    const int cand_grid_pct[] = {100, 100, 80, 80, 100, 100, 100, 100};
    const int cand_grid_k[] = {-1, -1, -1, -1, 2, 3, 4, 5};
    const int ncand = (atoms || two_real) ? 8 : 4;
    double best = 0.0;
    for (int c = 0; c < ncand; ++c) {
        cm_system_desc d = *desc;
        d.cell_scale_pct = grid ? cand_grid_pct[c] : cand[c % 4];
        d.atoms_schedule = atoms ? (grid ? (c < 4 ? (c % 2 == 0 ? CM_SCHED_CELL : CM_SCHED_BALANCED) : desc->atoms_schedule)
                                         : (c < 4 ? CM_SCHED_CELL : CM_SCHED_BALANCED))
                                 : CM_SCHED_AUTO;
        if (grid) d.atoms_grid = cand_grid_k[c];
        if (!atoms) d.real_pass = two_real ? (c < 4 ? CM_REAL_TILE : CM_REAL_WARP) : desc->real_pass;
        d.kernel_timing = 1;
        d.launch = CM_LAUNCH_STREAM;
        cm_handle *h = nullptr;
        int st = cm_create(&d, &h);
        if (st != CM_OK) return st;
        double ms = 0.0;
        st = guarded(h, [&] {
            submit(h, sample);  // warm-up: allocations, first launches
            check_device_error(h);
            timing_drain(h);
            for (int k = 0; k < CM_K_NCLASSES; ++k) h->class_ms[k] = 0.0;
            submit(h, sample);
            check_device_error(h);
            timing_drain(h);
            for (int k = 0; k < CM_K_NCLASSES; ++k) ms += h->class_ms[k];
        });
        if (st != CM_OK) {
            g_create_error = h->err;
            cm_destroy(h);
            return st;
        }
        cm_destroy(h);
        out->candidates[c] = d.cell_scale_pct;
        out->schedules[c] = atoms ? d.atoms_schedule : d.real_pass;
        out->grids[c] = grid ? d.atoms_grid : 0;
        out->ms_per_frame[c] = ms / std::max(1, sample->nframes);
        if (c == 0 || out->ms_per_frame[c] < best) {
            best = out->ms_per_frame[c];
            out->cell_scale_pct = d.cell_scale_pct;
            out->atoms_schedule = atoms ? d.atoms_schedule : 0;
            out->real_pass = atoms ? 0 : d.real_pass;
            out->atoms_grid = grid ? d.atoms_grid : 0;
        }
    }
    out->ncandidates = ncand;
    return CM_OK;
}

}  // extern "C"
