/*
 * cmgpu.h -- C ABI of the GB300 MDDF engine (libcmgpu.so).
 *
 * The engine computes, on one GPU, the per-frame hot path of ComplexMixtures.jl:
 * minimum distances between solute and solvent molecules under periodic
 * boundary conditions (orthorhombic and triclinic cells), the MDDF / RDF /
 * group-contribution histograms, and the random-insertion ideal-gas reference
 * counts.  Everything before the path (trajectory file parsing, selections,
 * options) stays in the host language.  The steps after it can run on the
 * device or stay on the host: normalisation (cm_read_results) and the group and
 * residue contributions (cm_contributions).
 *
 * Reference interfaces replaced (paths relative to ComplexMixtures.jl):
 *   mddf_frame!(r_chunk, system, buff, options, frame_weight, RNG)  src/mddf.jl:361-429
 *   coordination_number_frame!(r_chunk, system, buff, frame_weight) src/mddf.jl:438-471
 *   the per-chunk frame loop and sum!(R, r_chunk)                     src/mddf.jl:287-338,
 *                                                                     src/results.jl:629-649
 *   build_particle_system(trajectory, unitcell, options, ...)         src/minimum_distances.jl:157-176
 *
 * Conventions
 *   - Coordinates are xyz triplets in selection order (the order of
 *     AtomSelection.indices); molecules are contiguous blocks of
 *     natomspermol atoms (src/viewmol.jl:8-23).
 *   - A unit cell is 9 doubles, column-major: cell[0..2] is the first lattice
 *     vector, cell[3..5] the second, cell[6..8] the third (the columns of the
 *     reference's unit-cell matrix, src/mddf.jl:350-351).  An orthorhombic box
 *     is the diagonal matrix.
 *   - All entry points return a cm_status; nothing aborts or throws across
 *     the ABI.  cm_last_error() gives the message of the last failure.
 *   - A handle is used by one host thread at a time.  Different handles may
 *     run concurrently; each owns a CUDA stream on its device.
 *   - Host arrays passed in are read during the call only.
 */
#ifndef CMGPU_H
#define CMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CM_API_VERSION 4

typedef enum cm_status {
    CM_OK = 0,
    CM_EINVAL = 1,    /* invalid argument (ArgumentError in the reference) */
    CM_ENOMEM = 2,    /* device or host allocation failed, or over the HBM budget */
    CM_ECUDA = 3,     /* a CUDA runtime call failed */
    CM_EDEVICE = 4,   /* a device-side consistency check failed (error flag set by a kernel) */
    CM_ESTATE = 5     /* call not valid in the handle's current state */
} cm_status;

enum { CM_MODE_MDDF = 0, CM_MODE_COORDINATION_NUMBER = 1 };
enum { CM_PRECISION_FP64 = 0, CM_PRECISION_FP32_GUARD = 1 };
enum { CM_REGIME_AUTO = 0, CM_REGIME_PAIRS = 1, CM_REGIME_ATOMS = 2 };
/* How a compute chunk's chain of kernels is launched: one launch per kernel on
 * the handle's stream, or captured as a CUDA graph and replayed through one
 * executable graph per handle (updated in place while the chain keeps its
 * shape).  AUTO takes GRAPH unless kernel_timing is set. */
enum { CM_LAUNCH_AUTO = 0, CM_LAUNCH_STREAM = 1, CM_LAUNCH_GRAPH = 2 };
/* ATOMS-layout evaluation schedule: CELL = a warp per queued molecule pair,
 * lanes over each stencil cell's solute atoms in turn (dense solutes);
 * BALANCED = lanes over the atoms of all stencil cells end to end in FP32 (a
 * thread per pair in the FP64 path) for sparse solutes.  AUTO picks by the
 * solute atoms per occupied cell of the first frame (64 or more: CELL). */
enum { CM_SCHED_AUTO = 0, CM_SCHED_CELL = 1, CM_SCHED_BALANCED = 2 };
/* FP32 real pass of the PAIRS layout: WARP = one warp per solute molecule
 * walking its stencil; TILE (self-MDDF) = one CTA per home cell, the cell's
 * half-stencil molecules staged in shared memory and shared by its warps.
 * AUTO takes TILE in self mode. */
enum { CM_REAL_AUTO = 0, CM_REAL_WARP = 1, CM_REAL_TILE = 2 };
/* CM_COORD_DCD: solute_xyz points at nframes raw DCD frames (frame_bytes each,
 * laid out as cm_set_dcd_layout declared) and solvent_xyz is NULL; the
 * engine gathers the selections on the device. */
enum { CM_COORD_F64 = 0, CM_COORD_F32 = 1, CM_COORD_DCD = 2 };
enum { CM_MEM_HOST = 0, CM_MEM_DEVICE = 1 };

/*
 * System description.  Field meanings follow Options (src/Options.jl:6-42),
 * AtomSelection (src/AtomSelection.jl:48-59) and Result (src/results.jl:61-118).
 *
 * Groups.  Histogram credits follow update_group_count! (src/update_counters.jl:22-36):
 *   - the solute-side atom of a minimum-distance pair is identified by its index
 *     *within its molecule* (0..solute_natomspermol-1), so solute credits are a
 *     CSR over those local indices: solute_group_offsets[natomspermol+1],
 *     solute_groups[...] (group numbers, 0-based);
 *   - the solvent-side atom is identified by its index in the whole selection
 *     (0..solvent_nmols*solvent_natomspermol-1): solvent_group_offsets[N+1],
 *     solvent_groups[...].
 *   For default groups (custom_groups == false) pass NULL CSRs: the group of an
 *   atom is then its atom type (src/update_counters.jl:9) and the group count
 *   equals natomspermol.  In self mode (autocorrelation) both credits go to the
 *   solute table (src/update_counters.jl:272-277) and the solvent CSR must
 *   describe the same selection.
 */
typedef struct cm_system_desc {
    int32_t api_version;              /* CM_API_VERSION */
    int32_t solute_nmols;
    int32_t solute_natomspermol;
    int32_t solvent_nmols;
    int32_t solvent_natomspermol;
    int32_t autocorrelation;          /* 1: solute and solvent are the same selection */
    int32_t irefatom;                 /* 1-based reference atom of the solvent molecule */
    double cutoff;
    double binstep;
    double dbulk;
    int32_t usecutoff;
    int32_t nbins;                    /* setbin(cutoff, binstep) */
    int32_t n_random_samples;
    int32_t lcell;                    /* cell side = cutoff / lcell for atom cell lists */
    int32_t mode;                     /* CM_MODE_* */
    int32_t precision;                /* CM_PRECISION_* */
    int32_t regime;                   /* CM_REGIME_*: search layout, AUTO picks by molecule size */
    uint64_t seed;                    /* seed of the random-insertion stream */
    int32_t solute_ngroups;           /* 0 with NULL CSR = default groups */
    const int64_t *solute_group_offsets;
    const int32_t *solute_groups;
    int32_t solvent_ngroups;
    const int64_t *solvent_group_offsets;
    const int32_t *solvent_groups;
    int32_t device;                   /* CUDA device ordinal */
    int32_t max_frames_per_batch;     /* frames staged on the device per submit chunk; 0 = 64 */
    int64_t hbm_budget_bytes;         /* 0 = no limit; cm_create fails with CM_ENOMEM above it */
    int32_t kernel_timing;            /* 1: time every launch with CUDA events (cm_get_kernel_times) */
    int32_t cell_scale_pct;           /* search-cell size in percent of the default (0 = 100, range 30-300);
                                         the counts do not depend on it, only the speed (cm_autotune) */
    int32_t launch;                   /* CM_LAUNCH_*; the counts do not depend on it */
    int32_t atoms_schedule;           /* CM_SCHED_*; the counts do not depend on it */
    int32_t guard_queue_capacity;     /* records per compute chunk of the FP32 real pass's guard and edge
                                         queues; 0 = sized by the engine.  A chunk whose deferred records
                                         do not fit is redone on the device without queues, so the counts
                                         do not depend on it (a small value only exercises that path) */
    int32_t real_pass;                /* CM_REAL_*: FP32 real-pass schedule of the PAIRS layout; the counts do
                                         not depend on it */
    int32_t atoms_grid;               /* ATOMS layout with one solute molecule, FP32 search: fine cells per
                                         search-cell axis of the per-frame candidate grid (1-6; 0 = a grid of
                                         fine cells of about 2.5 A for dense solutes, the stencil walk for
                                         sparse ones; -1 = no grid, every query walks the stencil).  The
                                         counts do not depend on it */
    int32_t atoms_grid_capacity;      /* list entries per frame of that grid; 0 = sized by the engine.  A frame
                                         whose lists do not fit walks the stencil instead, so the counts do
                                         not depend on it (a small value only exercises that path) */
} cm_system_desc;

/*
 * A batch of frames.  Counts of all frames are added to the handle's
 * accumulators, as sum!(R, r_chunk) does (src/results.jl:629-649).
 */
typedef struct cm_frames {
    int32_t nframes;
    int32_t coord_type;               /* CM_COORD_F64, CM_COORD_F32 or CM_COORD_DCD */
    int32_t memory;                   /* where solute_xyz / solvent_xyz live: CM_MEM_HOST / CM_MEM_DEVICE */
    int32_t reserved;
    const void *solute_xyz;           /* [nframes][solute atoms][3] */
    const void *solvent_xyz;          /* [nframes][solvent atoms][3]; NULL in self mode */
    const double *cells;              /* host [nframes][9] */
    const double *weights;            /* host [nframes]; NULL = all 1.0 (frame_weights) */
    const int64_t *frame_ids;         /* host [nframes]; 1-based trajectory frame numbers,
                                         they key the random-insertion stream */
    int64_t solute_frame_stride;      /* coordinate values from one frame's first solute atom to the next
                                         frame's (>= solute atoms x 3); 0 = consecutive frames.  A frame
                                         may thus be a slice of a larger array, e.g. a contiguous
                                         selection of a trajectory's frames, with no gather */
    int64_t solvent_frame_stride;     /* the same for solvent_xyz; ignored in self mode */
} cm_frames;

/*
 * Accumulated counts in the units of the reference's Result fields before
 * finalresults! (src/results.jl:311-376): frame-weighted sums.  All arrays are
 * caller-owned host buffers; NULL pointers are skipped.
 */
typedef struct cm_counts {
    double *md_count;                     /* [nbins] */
    double *md_count_random;              /* [nbins] */
    double *rdf_count;                    /* [nbins] */
    double *rdf_count_random;             /* [nbins] */
    double *solute_group_count;           /* [solute_ngroups][nbins] */
    double *solute_group_count_random;    /* [solute_ngroups][nbins] */
    double *solvent_group_count;          /* [solvent_ngroups][nbins]; zero in self mode */
    double *solvent_group_count_random;   /* [solvent_ngroups][nbins]; zero in self mode */
    double volume_total;                  /* sum of w * det(cell) (src/mddf.jl:350-352) */
    double weight_total;                  /* sum of w over computed frames */
    int64_t frames;                       /* frames computed */
} cm_counts;

/*
 * Exact integer counts in half units (2 per unit of frame weight), valid while
 * every frame submitted since the last reset carried the same weight.
 * Array layout as in cm_counts.
 */
typedef struct cm_raw_counts {
    int64_t *md, *md_random, *rdf, *rdf_random;
    int64_t *solute_group, *solute_group_random;
    int64_t *solvent_group, *solvent_group_random;
} cm_raw_counts;

typedef struct cm_stats {
    int64_t frames;
    int64_t molecule_pairs_evaluated;     /* candidate molecule pairs whose atom pairs were evaluated */
    int64_t atom_pairs_evaluated;         /* atom-pair distance evaluations (FP32 or FP64) */
    int64_t hits_real;                    /* minimum-distance records within cutoff, real pass */
    int64_t hits_random;                  /* same, random-insertion passes */
    int64_t guard_reevaluations;          /* records re-evaluated in FP64 inside the guard band */
    int64_t guard_pair_evaluations;       /* FP64 atom-pair evaluations done by those re-evaluations */
    double max_guard_error;               /* max |d_fp32 - d_fp64| seen in re-evaluated pairs (Angstrom) */
    double guard_band;                    /* guard half-width used in the last frame (Angstrom) */
    int32_t regime;                       /* CM_REGIME_PAIRS or CM_REGIME_ATOMS actually used */
    int32_t kernels_per_frame;            /* kernel launches of the last frame */
    int64_t kernel_launches;              /* kernel launches since create / reset */
    int64_t graph_launches;               /* chunks replayed as a CUDA graph since create / reset */
    int64_t graph_instantiations;         /* of those, chunks whose chain changed shape (graph built anew) */
} cm_stats;

/* Kernel classes of cm_get_kernel_times. */
enum {
    CM_K_PREP = 0,        /* binning, offsets, centroid data, offset table */
    CM_K_CELLS = 1,       /* counting sort: scan + scatter */
    CM_K_REAL = 2,        /* real-frame minimum distances + histograms */
    CM_K_BULK = 3,        /* bulk-molecule lists */
    CM_K_RANDOM = 4,      /* random-insertion placement + minimum distances */
    CM_K_OTHER = 5,       /* weight folds */
    CM_K_GUARD = 6,       /* FP64 re-evaluation of the candidates deferred by the FP32 real pass */
    CM_K_NCLASSES = 7
};

/* Per-class GPU time (ms, from CUDA events around each launch on the handle's
 * stream) and launch counts since create / reset; needs kernel_timing = 1. */
typedef struct cm_kernel_times {
    double ms[CM_K_NCLASSES];
    int64_t launches[CM_K_NCLASSES];
} cm_kernel_times;

typedef struct cm_handle cm_handle;

/* Validate the description, allocate device state.  *out is set on success. */
int cm_create(const cm_system_desc *desc, cm_handle **out);

/* Enqueue a batch of frames (asynchronous on the handle's stream for device
 * memory; host memory is staged through pinned buffers before return). */
int cm_submit_frames(cm_handle *h, const cm_frames *frames);

/* Wait for all submitted work; returns CM_EDEVICE if a kernel raised its error flag. */
int cm_synchronize(cm_handle *h);

/*
 * Raw DCD frames (replaces the host-side read and gather of
 * src/trajectory_formats/NamdDCD.jl:141-169 and the selection copy of
 * src/Trajectory.jl's nextframe!): frames are given to cm_submit_frames with
 * coord_type CM_COORD_DCD as the bytes read from the file, from the first byte
 * of a frame's unit-cell record to the last byte of its z record, and the
 * engine gathers the selected atoms on the device.  The unit cells still come
 * through cm_frames.cells (parsed on the host: the frame geometry is host
 * work).  Set once per handle, before the first DCD submit.
 */
typedef struct cm_dcd_layout {
    int64_t natoms;                   /* atoms per frame in the file */
    int64_t frame_bytes;              /* bytes per frame (a multiple of 4) */
    int64_t x_offset;                 /* byte offset, within a frame, of the first x value (past its record marker) */
    int64_t y_offset;
    int64_t z_offset;
    int32_t big_endian;               /* 1: the file's floats are big-endian */
    int32_t reserved;
    const int32_t *solute_atoms;      /* host [solute atoms]: 0-based atom index in the frame, selection order */
    const int32_t *solvent_atoms;     /* host [solvent atoms]; NULL in self mode */
} cm_dcd_layout;
int cm_set_dcd_layout(cm_handle *h, const cm_dcd_layout *layout);

/*
 * Batches of systems (no counterpart in the reference, which runs one system
 * per mddf call).  cm_batch_submit gives frames[i] to handles[i] like
 * cm_submit_frames, but the kernels of all systems are captured into one CUDA
 * graph -- each system's chain on its own stream, forked from and joined to the
 * batch's stream -- and launched once, so systems of uneven size run side by
 * side with one launch per staging round.  The executable graph is updated in
 * place while the systems and their chunk shapes repeat.  Counts are those of
 * cm_submit_frames on each handle.  All handles live on one device, have
 * kernel_timing off, and are used by no other thread during a call; destroy
 * the batch before its handles.  After a failed cm_batch_submit the handles'
 * counts are undefined until cm_reset.
 */
typedef struct cm_batch cm_batch;
int cm_batch_create(cm_handle *const *handles, int32_t nhandles, cm_batch **out);
int cm_batch_submit(cm_batch *b, const cm_frames *frames);  /* frames[nhandles]; nframes 0 skips a system */
int cm_batch_graph_stats(const cm_batch *b, int64_t *graph_launches, int64_t *graph_instantiations);

/* How a staging round runs (the counts do not depend on it).  FUSED (the
 * default): when every system of the round is in the ATOMS layout with the
 * FP32 search and their chunks have the same chain of stages, each stage runs
 * once for all systems -- one kernel launch drains a device work table of
 * (system, block) entries, each entry the system's own arguments and grid --
 * so a round is one graph of about 15 launches plus 3 per random-insertion
 * piece whatever the number of systems; other rounds fall back to STREAMS.
 * STREAMS: each system's chain on its own stream of the graph, as above. */
enum { CM_BATCH_FUSED = 0, CM_BATCH_STREAMS = 1 };
int cm_batch_set_mode(cm_batch *b, int32_t mode);
/* Rounds run fused, their stage launches in total, and the systems of the last fused round. */
int cm_batch_fused_stats(const cm_batch *b, int64_t *fused_rounds, int64_t *stage_launches, int64_t *systems);
int cm_batch_destroy(cm_batch *b);
const char *cm_batch_last_error(const cm_batch *b);

/* Synchronise and copy the weighted accumulators out. */
int cm_read_counts(cm_handle *h, cm_counts *out);

/*
 * Finalised results (finalresults!, src/results.jl:311-469) computed on the
 * device in FP64 from the handle's accumulators: the normalisation by frames
 * and molecules, the shell and bulk volumes, the bulk density and its
 * correction of the random counts, coordination numbers, MDDF, RDF and KB
 * integrals, in the reference's order of operations.  frame_weight_sum is
 * sum_frame_weights of the Result (0: the sum of the weights submitted).
 * Caller-owned host arrays; NULL pointers are skipped.  In self mode the
 * solvent group arrays receive the solute's (src/results.jl:335-337).
 */
typedef struct cm_results {
    double *d, *md_count, *md_count_random, *coordination_number, *coordination_number_random, *mddf, *kb;  /* [nbins] */
    double *rdf_count, *rdf_count_random, *sum_rdf_count, *sum_rdf_count_random, *rdf, *kb_rdf;         /* [nbins] */
    double *volume_shell;                                                                                /* [nbins] */
    double *solute_group_count, *solute_group_count_random;      /* [solute groups][nbins] */
    double *solvent_group_count, *solvent_group_count_random;    /* [solvent groups][nbins] */
    double volume_total, volume_bulk, volume_domain;
    double density_solute, density_solvent, density_solvent_bulk, density_fix;
    int64_t zero_random_bins;         /* bins with no random-insertion count (the reference warns about them) */
} cm_results;
int cm_read_results(cm_handle *h, double frame_weight_sum, cm_results *out);

/*
 * Group contributions on the device, many queries per call.  Replaces
 * contributions(R, SoluteGroup|SolventGroup; type) (src/tools/contributions.jl:70-248)
 * and the per-residue loop of ResidueContributions
 * (src/tools/residue_contributions.jl:157-215), which calls it once per residue.
 * The handle's accumulators are finalised as cm_read_results does
 * (frame_weight_sum has the same meaning).  Then each query sums the finalised
 * group-count rows `groups[0..nterms-1]` of its side, in that order,
 * bin by bin.  With `divide` set, each term is group_count[g] / nmols, the
 * reference's rule for atom indices of a selection with more than one molecule.
 * The sum is then converted by `type`, in FP64 and in the reference's order of
 * operations:
 *   - MDDF: sum / md_count_random, or 0 where md_count_random is 0;
 *   - COORDINATION_NUMBER: its cumulative sum;
 *   - MD_COUNT: the sum itself;
 *   - KBI: Angs3tocm3permol * (1 / density.solvent_bulk) * (cumsum(sum) - cumsum(random sum)).
 * The host resolves group names, atom names and atom indices into
 * 0-based group rows, which is where the reference raises its argument errors.
 * out: caller-owned [nqueries][nbins] doubles.  In self mode the solvent rows
 * are the solute's.
 */
enum { CM_GROUP_SOLUTE = 0, CM_GROUP_SOLVENT = 1 };
enum { CM_CONTRIB_MDDF = 0, CM_CONTRIB_COORDINATION_NUMBER = 1, CM_CONTRIB_MD_COUNT = 2, CM_CONTRIB_KBI = 3 };
typedef struct cm_contrib_query {
    int32_t side;            /* CM_GROUP_SOLUTE or CM_GROUP_SOLVENT */
    int32_t type;            /* CM_CONTRIB_* */
    int32_t divide;          /* nonzero: each term is divided by the side's number of molecules */
    int32_t nterms;          /* >= 1 */
    const int32_t *groups;   /* host [nterms]: 0-based group rows, summed in this order */
} cm_contrib_query;
int cm_contributions(cm_handle *h, double frame_weight_sum, int32_t nqueries, const cm_contrib_query *queries,
                     double *out);

/* Synchronise and copy the exact half-unit counts (single-weight runs only). */
int cm_read_raw_counts(cm_handle *h, cm_raw_counts *out);

/* The weight of the frames behind cm_read_raw_counts (1.0 before any frame);
 * CM_ESTATE once frames of different weights were submitted. */
int cm_raw_counts_weight(cm_handle *h, double *frame_weight);

/*
 * Resume (src/results.jl:533-588 save/load, src/tools/merge.jl:10 merge):
 * replace the handle's accumulators with saved half-unit counts -- what
 * cm_read_raw_counts and cm_raw_counts_weight gave for `frames` frames of
 * weight `frame_weight`, with volume_total the sum of weight x cell volume
 * over them (cm_counts volume_total) -- so that frames submitted afterwards
 * add to them.  With the same frame weight the handle then holds exactly the counts
 * of one run over all the frames.  The solvent arrays may be NULL with
 * autocorrelation.  Synchronises the handle's stream; keeps its statistics.
 */
int cm_load_raw_counts(cm_handle *h, const cm_raw_counts *in, double frame_weight, int64_t frames, double volume_total);

/* Engine statistics (synchronises). */
int cm_get_stats(cm_handle *h, cm_stats *out);

/* Kernel times per class (synchronises). */
int cm_get_kernel_times(cm_handle *h, cm_kernel_times *out);

/* Zero the accumulators and statistics; keeps device allocations. */
int cm_reset(cm_handle *h);

/* Release everything owned by the handle.  NULL is accepted. */
int cm_destroy(cm_handle *h);

/* Message of the last failure on this handle (or of the last cm_create failure
 * on this thread when h is NULL).  Never NULL. */
const char *cm_last_error(const cm_handle *h);

/* Static description of a status code. */
const char *cm_status_string(int status);

/* Measure the FP32 CUDA-core throughput of a device (TFLOP/s, FMA = 2 flops)
 * with a register-resident multiply-add loop over all SMs; the denominator of
 * the engine's compute roofline.  Runs for about `ms_target` milliseconds. */
int cm_measure_fp32_peak(int32_t device, double ms_target, double *tflops);

/* Device memory the handle holds, in bytes. */
int64_t cm_device_bytes(const cm_handle *h);

/*
 * grid3D (src/tools/grid3D.jl:47-147) on the device.  For every point of the
 * grid spanning the solute's bounding box widened by dmax (n = ceil((length +
 * 2 dmax) / step + 1) points per axis, point (ix, iy, iz) at xmin - dmax +
 * step * ix, 0-based), the closest solute atom (Euclidean, no periodic images,
 * ties to the lower index) is found; the point is kept when dmin < r < dmax
 * and the atom's contribution curve, linearly interpolated at r over the bin
 * distances d, is positive.  Kept points come back in ascending point order.
 * The reference's ArgumentErrors (custom groups) and the beta scaling and PDB
 * output are host-side.
 */
typedef struct cm_grid3d_desc {
    int32_t device;
    int32_t nbins;
    int64_t natoms;                   /* solute atoms */
    const double *xyz;                /* host [natoms][3] */
    const int32_t *atom_type;         /* host [natoms]: row of `table` (the atom's position in its molecule) */
    int32_t ntypes;
    int32_t reserved;
    const double *table;              /* host [ntypes][nbins]: contribution curve of each atom type */
    const double *d;                  /* host [nbins]: bin distances (Result.d), increasing; d[0] <= dmin, dmax < d[nbins-1] */
    double dmin, dmax, step;
} cm_grid3d_desc;

typedef struct cm_grid3d_out {
    int64_t capacity;                 /* entries the arrays below hold */
    int64_t count;                    /* kept points (when above capacity: CM_ENOMEM, arrays untouched) */
    int64_t n[3];                     /* grid points per axis */
    double origin[3];                 /* position of point (0, 0, 0) */
    int64_t *point;                   /* [capacity] (ix * n[1] + iy) * n[2] + iz, ascending */
    int32_t *atom;                    /* [capacity] 0-based solute atom closest to the point */
    double *distance;                 /* [capacity] */
    double *value;                    /* [capacity] interpolated contribution */
} cm_grid3d_out;

int cm_grid3d(const cm_grid3d_desc *desc, cm_grid3d_out *out);

/* Process-wide block cache (no counterpart in the reference, whose arrays
 * are garbage-collected Julia memory).  A destroyed handle returns its device
 * and pinned host blocks to a per-device cache that later handles draw from,
 * because freeing them waits for every stream of the device.  Report the
 * cached (free) bytes of `device` and, when `release` is nonzero, return them
 * to the driver first (that waits for the device).  Either output may be
 * NULL. */
int cm_memory_cache(int32_t device, int32_t release, int64_t *cached_device_bytes, int64_t *cached_host_bytes);

/* The CUDA stream of the handle (as cudaStream_t), for callers that order
 * their own device work against the engine. */
void *cm_stream(cm_handle *h);

/* ---------------------------------------------------------------------------
 * Autotuner.  No counterpart in the reference (its cell size is
 * cutoff / lcell).  Times the real and random-insertion passes of a sample
 * of frames for each candidate search-cell size, with temporary handles and
 * CUDA events, and returns the fastest as cell_scale_pct (and, in the ATOMS
 * layout, atoms_schedule) for cm_create.  The candidates are the default cell
 * (100 %) and smaller cells (more, finer stencil cells: less volume searched
 * per molecule, more cells to walk), in the ATOMS layout each with both
 * evaluation schedules. */
#define CM_TUNE_MAX 8
typedef struct cm_tuning {
    int32_t cell_scale_pct;           /* the fastest candidate */
    int32_t ncandidates;
    int32_t candidates[CM_TUNE_MAX];  /* cell_scale_pct of each candidate */
    double ms_per_frame[CM_TUNE_MAX]; /* measured GPU time per frame of each candidate */
    int32_t atoms_schedule;           /* the fastest candidate's CM_SCHED_* (ATOMS layout; 0 otherwise) */
    int32_t schedules[CM_TUNE_MAX];   /* each candidate's CM_SCHED_* (ATOMS layout) or CM_REAL_* (molecule
                                         layout) */
    int32_t real_pass;                /* the fastest candidate's CM_REAL_* (molecule layout; 0 otherwise) */
    int32_t atoms_grid;               /* the fastest candidate's atoms_grid (one solute molecule in the ATOMS
                                         layout, FP32; 0 otherwise) */
    int32_t grids[CM_TUNE_MAX];       /* each candidate's atoms_grid */
} cm_tuning;

int cm_autotune(const cm_system_desc *desc, const cm_frames *sample, cm_tuning *out);

/* ---------------------------------------------------------------------------
 * Request server: continuous batching of MDDF jobs on one device.  No
 * counterpart in the reference (it runs one mddf call at a time); each
 * request's counts are those of cm_create + cm_submit_frames +
 * cm_read_counts for its system and frames alone.
 *
 * Requests queue in arrival order.  The server admits one when fewer than
 * max_active requests are on the device and its handle fits in what is left
 * of hbm_budget_bytes (0: no budget, only the device's memory); a request that
 * does not fit waits while smaller ones behind it may be admitted.  Admitted
 * requests keep their coordinates, cell lists and accumulators on the device,
 * run on their own streams (their work overlaps on the GPU) and take turns of
 * frames_per_turn frames.  A request's counts are read back as soon as its
 * last frame is done and its device memory goes back to the budget.  The
 * caller keeps the request's coordinate arrays alive until it is finished
 * (cells, weights and frame ids are copied at submit). */
enum {
    CM_REQ_QUEUED = 0,
    CM_REQ_RUNNING = 1,
    CM_REQ_DONE = 2,
    CM_REQ_FAILED = 3,
    CM_REQ_CANCELLED = 4
};

typedef struct cm_server_desc {
    int32_t device;
    int32_t max_active;             /* requests on the device at once, 0: no limit */
    int64_t hbm_budget_bytes;       /* device memory for admitted requests, 0: no budget */
    int32_t frames_per_turn;        /* frames a request submits per turn, 0: 32 */
    int32_t reserved;
} cm_server_desc;

typedef struct cm_request_info {
    int32_t state;                  /* CM_REQ_* */
    int32_t status;                 /* cm_status of a failed request */
    double t_submit, t_admit, t_done; /* seconds since cm_server_create (host clock) */
    int64_t frames_submitted;
    int64_t device_bytes;           /* device memory of the request's handle */
} cm_request_info;

typedef struct cm_server cm_server;

/* Start a server (and its scheduler thread) on one device. */
int cm_server_create(const cm_server_desc *desc, cm_server **out);

/* Queue a request: a system and its frames, in host memory or in device memory
 * that stays valid (and unchanged) until the request is done. */
int cm_server_submit(cm_server *s, const cm_system_desc *desc, const cm_frames *frames, int64_t *request_id);

/* State of a request. */
int cm_server_poll(cm_server *s, int64_t request_id, cm_request_info *out);

/* Wait until a request is done, failed or cancelled (timeout_s < 0: no
 * timeout); CM_ESTATE if it is still running at the timeout. */
int cm_server_wait(cm_server *s, int64_t request_id, double timeout_s, cm_request_info *out);

/* Results of a finished request (weighted FP64, and exact half units). */
int cm_server_read_counts(cm_server *s, int64_t request_id, cm_counts *out);
int cm_server_read_raw_counts(cm_server *s, int64_t request_id, cm_raw_counts *out);

/* Cancel a queued or running request. */
int cm_server_cancel(cm_server *s, int64_t request_id);

/* Forget a finished request and its results. */
int cm_server_release(cm_server *s, int64_t request_id);

/* Stop the scheduler and free every request. */
int cm_server_destroy(cm_server *s);

/* Message of the last failure of a server call (s NULL: of cm_server_create). */
const char *cm_server_last_error(const cm_server *s);

/* ---------------------------------------------------------------------------
 * Allocation-free entry point.  No counterpart in the reference: it serves
 * callers that cannot allocate device memory (an in-situ analysis callback
 * inside a simulation engine that owns the device memory, a host program whose
 * memory pool must not grow while its streams are captured).
 *
 * Computes the exact half-unit counts of ONE frame -- the values
 * cm_read_raw_counts gives for a handle that was given only that frame -- into
 * `counts` (device memory, int64, overwritten), laid out as
 *   md[nbins] md_random[nbins] rdf[nbins] rdf_random[nbins]
 *   solute_group[Gs][nbins] solute_group_random[Gs][nbins]
 *   solvent_group[Gv][nbins] solvent_group_random[Gv][nbins]
 * with Gs, Gv the atoms per solute / solvent molecule (the two solvent blocks
 * are absent with autocorrelation); counts_len must equal that total.
 *
 * It calls no device allocator: every buffer beyond the caller's coordinates
 * and `counts` is carved from one file-scope device array of
 * CM_NOALLOC_SCRATCH_BYTES.  Limits, refused with CM_EINVAL and a message:
 * the PAIRS layout (at most 32 atoms per molecule), default per-atom groups,
 * frame->nframes == 1 with coordinates in device memory and weights NULL,
 * n_random_samples <= CM_NOALLOC_MAX_SAMPLES, and the frame's buffers within
 * the scratch array (the message gives the size needed).  Of the tuning
 * fields, cell_scale_pct and guard_queue_capacity are honoured; launch,
 * atoms_schedule, max_frames_per_batch, hbm_budget_bytes and kernel_timing
 * are ignored.  The guard and edge queues hold at most 131,072 records: a
 * frame that defers more is redone on the device without queues (slower,
 * the same counts).
 *
 * Every call looks up the scratch array's address in the current context
 * (cudaGetSymbolAddress, with desc->device current), so calls from another
 * context of the device, or after cudaDeviceReset, use the address valid
 * there.  The first call in a context may load the library's device code:
 * make it before any stream capture.  Every call shares the array and finds the
 * previous call's contents in it; each call clears what must start at zero.
 * Calls whose GPU work overlaps (several streams or host threads) race on the
 * array.  Work is ordered on `stream` (NULL: the legacy default stream) and
 * the call synchronises it before returning (it reads the molecule radii and
 * the device error flag back).  Errors: cm_last_error(NULL). */
#define CM_NOALLOC_SCRATCH_BYTES (32ull << 20)
#define CM_NOALLOC_MAX_SAMPLES 4096
int cm_frame_counts_noalloc(const cm_system_desc *desc, const cm_frames *frame, int64_t *counts, int64_t counts_len,
                            void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CMGPU_H */
