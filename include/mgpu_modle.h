/*
 * mgpu_modle.h - C ABI of the GB300 loop-extrusion epoch engine.
 *
 * The library replaces MoDLE's per-cell epoch loop
 *   void Simulation::simulate_one_cell(State& s) const
 *   (src/libmodle/cpu/include/modle/simulation.hpp:199,
 *    src/libmodle/cpu/simulation.cpp:1056-1152)
 * which the reference calls once per (chromosome, cell) task from
 *   Simulation::simulate_worker (src/libmodle/cpu/scheduler_simulate.cpp:255).
 *
 * Design rules of this boundary:
 *   - plain C types only: pointers, sizes, doubles and fixed-width integers;
 *   - no exception crosses it: every call returns an int status (MGPU_OK == 0, negative on
 *     error) and mgpu_last_error_string() describes the last failure of the calling thread;
 *   - the caller owns every input and output buffer; buffers may live in host or device
 *     memory (the library checks with cudaPointerGetAttributes);
 *   - one context per device; a context is safe to call from several host threads (calls
 *     are serialised by a per-context mutex), and contexts are independent.
 *
 * Positions are base pairs.  The reference stores them as 64-bit integers (bp_t,
 * src/common/include/modle/common/common.hpp:72); the device stores them as 32-bit
 * integers, which is exact because every chromosome must be shorter than 2^32 - 1 bp
 * (the library rejects longer ones).  Contacts are 32-bit counters (contacts_t, common.hpp:73).
 */
#ifndef MGPU_MODLE_H
#define MGPU_MODLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGPU_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------------------- */
#define MGPU_OK 0
#define MGPU_ERR_INVALID_ARG (-1)   /* bad pointer, size or parameter                       */
#define MGPU_ERR_CUDA (-2)          /* a CUDA runtime call failed                           */
#define MGPU_ERR_TIMEOUT (-3)       /* a device loop hit its iteration limit                */
#define MGPU_ERR_OVERFLOW (-4)      /* a device counter or buffer would overflow            */
#define MGPU_ERR_UNSUPPORTED (-5)   /* valid input outside what this build supports         */
#define MGPU_ERR_NO_DEVICE (-6)     /* no usable CUDA device                                */
#define MGPU_ERR_OUT_OF_MEMORY (-7) /* device allocation failed                             */
#define MGPU_ERR_INTERNAL (-8)      /* device code detected an inconsistent state           */

/* Contact sampling strategy bits (Config::ContactSamplingStrategy,
 * src/common/include/modle/common/simulation_config.hpp:32-37). */
#define MGPU_CS_NOISIFY 1u
#define MGPU_CS_TAD 2u
#define MGPU_CS_LOOP 4u

/* Barrier blocking direction (dna::Direction, src/common/include/modle/common/dna.hpp:75-78). */
#define MGPU_DIR_REV 1u
#define MGPU_DIR_FWD 2u

/* Collision event bits (Collision<I>, src/libmodle/cpu/include/modle/collision_encoding.hpp:91-96).
 * Trace and phase outputs use the reference's 64-bit word: index | (event << 56). */
#define MGPU_COLL_COLLISION 0x10u
#define MGPU_COLL_CHROM_BOUNDARY 0x08u
#define MGPU_COLL_LEF_BAR 0x04u
#define MGPU_COLL_LEF_LEF_PRIMARY 0x02u
#define MGPU_COLL_LEF_LEF_SECONDARY 0x01u
#define MGPU_COLL_INDEX_BITS 56

/*
 * Simulation parameters: the fields of modle::Config that the epoch loop reads
 * (src/common/include/modle/common/simulation_config.hpp:60-124).  mgpu_config_defaults()
 * fills the reference defaults; mgpu_config_transform() applies the CLI derivations of
 * Cli::transform_args (src/modle/cli.cpp:1086-1215).  mgpu_create() expects a transformed
 * config, exactly like Simulation's constructor receives one.
 */
typedef struct mgpu_config {
  /* stopping criterion (simulation_config.hpp:61-63) */
  uint64_t target_simulation_epochs;
  double target_contact_density; /* < 0 selects the epoch criterion */
  uint32_t stop_on_epochs;       /* StoppingCriterion::simulation_epochs */
  /* contact matrix and sampling (simulation_config.hpp:66-74) */
  uint64_t bin_size;
  uint64_t diagonal_width;
  uint32_t contact_sampling_strategy; /* MGPU_CS_* bits */
  double tad_to_loop_contact_ratio;
  double genextreme_mu;
  double genextreme_sigma;
  double genextreme_xi;
  /* LEFs (simulation_config.hpp:77-86) */
  uint64_t fwd_extrusion_speed;
  uint64_t rev_extrusion_speed;
  double fwd_extrusion_speed_std;
  double rev_extrusion_speed_std;
  double number_of_lefs_per_mbp;
  double prob_of_lef_release;
  double prob_of_lef_release_burnin;
  uint64_t avg_lef_processivity;
  uint64_t contact_sampling_interval;
  /* barriers (simulation_config.hpp:89-93) */
  double extrusion_barrier_occupancy;
  double barrier_occupied_stp;
  double barrier_not_occupied_stp;
  /* collisions and stalls (simulation_config.hpp:96-100) */
  double hard_stall_lef_stability_multiplier;
  double soft_stall_lef_stability_multiplier;
  double probability_of_extrusion_unit_bypass;
  double lef_bar_major_collision_pblock;
  double lef_bar_minor_collision_pblock;
  /* miscellaneous (simulation_config.hpp:104-108) */
  uint64_t num_cells;
  uint64_t seed;
  uint64_t probability_normalization_factor;
  uint32_t normalize_probabilities;
  /* burn-in (simulation_config.hpp:116-124) */
  uint32_t skip_burnin;
  uint64_t burnin_history_length;
  uint64_t burnin_smoothing_window_size;
  uint64_t min_burnin_epochs;
  uint64_t max_burnin_epochs;
  uint64_t burnin_target_epochs_for_lef_activation;
  double burnin_speed_coefficient;
  uint64_t fwd_extrusion_speed_burnin;
  uint64_t rev_extrusion_speed_burnin;
  /* which options the user set explicitly: Cli::transform_args branches on these */
  uint32_t rev_speed_set;
  uint32_t fwd_speed_set;
  uint32_t occupancy_set;
  /* optional outputs that change what a cell computes (simulation_config.hpp:86, :111) */
  uint32_t track_1d_lef_position;    /* sample the 1D LEF occupancy after the contacts */
  uint32_t log_model_internal_state; /* per-epoch model-state records (dump_stats) */
} mgpu_config;

/* One chromosome (the simulated range of modle::Chromosome, src/libmodle/internal/genome.cpp). */
typedef struct mgpu_chrom {
  const char* name; /* hashed into the per-cell seed (Chromosome::hash, genome.cpp:317-335) */
  uint64_t name_len;
  uint64_t size;  /* full chromosome size (Chromosome::size) */
  uint64_t start; /* first simulated bp (Chromosome::start_pos) */
  uint64_t end;   /* one past the last simulated bp (Chromosome::end_pos) */
} mgpu_chrom;

/* One extrusion barrier after BED import (ExtrusionBarrier,
 * src/libmodle/internal/include/modle/extrusion_barriers.hpp:104-127). */
typedef struct mgpu_barrier {
  uint64_t pos;
  double stp_active;   /* P(occupied -> occupied) */
  double stp_inactive; /* P(free -> free) */
  uint32_t blocking_dir; /* MGPU_DIR_REV or MGPU_DIR_FWD */
  uint32_t reserved;
} mgpu_barrier;

/* Per-cell outcome (fields of Simulation::State after simulate_one_cell, simulation.hpp:95-101). */
typedef struct mgpu_cell_stats {
  uint64_t epochs;          /* State::epoch at exit */
  uint64_t burnin_epochs;   /* State::num_burnin_epochs */
  uint64_t contacts;        /* State::num_contacts (missed updates included) */
  uint64_t missed_updates;  /* contacts that fell outside the band */
  uint64_t lef_epochs;      /* sum over epochs of active LEFs (burn-in included) */
  uint64_t rng_draws;       /* 64-bit draws taken from the cell's Xoshiro256++ stream */
  uint64_t sort_fallbacks;  /* epochs whose ranking needed the exact sequential sort */
  uint64_t status;          /* 0 or a positive device error code */
} mgpu_cell_stats;

typedef struct mgpu_ctx mgpu_ctx;

/* ---- configuration and host-side helpers ---------------------------------------------- */

/* Reference defaults of modle::Config (simulation_config.hpp:24-135). */
void mgpu_config_defaults(mgpu_config* cfg);

/* Cli::transform_args (src/modle/cli.cpp:1194-1215): extrusion speeds and their std
 * (:1086-1110), release probability (:1113-1119), stp/occupancy (:1122-1135), contact
 * sampling ratio (:1169-1182), burn-in activation epochs (:1184-1190) and probability
 * normalisation (:1138-1167). */
int mgpu_config_transform(mgpu_config* cfg);

/* Chromosome::hash (src/libmodle/internal/genome.cpp:317-335): XXH3-64 with seed
 * cfg.seed over name bytes | size (u64 LE) | cell_id (u64 LE). */
uint64_t mgpu_cell_seed(const char* name, uint64_t name_len, uint64_t chrom_size, uint64_t seed,
                        uint64_t cell_id);

/* XXH3_64bits_withSeed over an arbitrary buffer (inputs up to 240 bytes; longer inputs
 * return 0 and set the last error). */
uint64_t mgpu_xxh3_64(const void* data, uint64_t len, uint64_t seed);

/* Simulation::compute_num_lefs (simulation.cpp:1253-1257). */
uint64_t mgpu_num_lefs(const mgpu_config* cfg, uint64_t simulated_size);
/* Simulation::compute_contacts_per_epoch (simulation.cpp:1243-1251). */
uint64_t mgpu_contacts_per_epoch(const mgpu_config* cfg, uint64_t num_lefs);
/* Chromosome::npixels (src/libmodle/internal/genome_impl.hpp:20-25). */
uint64_t mgpu_npixels(const mgpu_config* cfg, uint64_t simulated_size);
/* Band shape of ContactMatrixDense(length, diagonal_width, bin_size)
 * (src/contact_matrix/contact_matrix_dense_impl.hpp:40-51). */
void mgpu_band_shape(const mgpu_config* cfg, uint64_t simulated_size, uint64_t* nrows,
                     uint64_t* ncols);

/* Per-cell task targets of Simulation::run_simulate (scheduler_simulate.cpp:129-153):
 * fills target_contacts[ncells] and returns the per-task target epochs in *target_epochs. */
int mgpu_task_targets(const mgpu_config* cfg, uint64_t simulated_size, uint64_t num_lefs,
                      uint64_t ncells, uint64_t* target_contacts, uint64_t* target_epochs);

/* Chromosome::add_extrusion_barrier (genome.cpp:194-210) with compute_barrier_stp
 * (genome.cpp:181-192): a BED record [chrom_start, chrom_end) with strand '+'/'-' and score
 * (occupancy, 0 = use the defaults) becomes one barrier at the interval midpoint.  Returns 0
 * when the midpoint lies outside [start, end), 1 otherwise. */
int mgpu_barrier_from_bed(const mgpu_chrom* chrom, uint64_t chrom_start, uint64_t chrom_end,
                          char strand, double score, double default_stp_active,
                          double default_stp_inactive, mgpu_barrier* out);

/* ExtrusionBarriers::sort (src/libmodle/internal/extrusion_barriers.cpp:234-259): orders the
 * barriers by position with the same pattern-defeating quicksort the reference uses. */
int mgpu_sort_barriers(mgpu_barrier* barriers, uint64_t nbarriers);

/* ---- device context ------------------------------------------------------------------- */

const char* mgpu_last_error_string(void);
int mgpu_abi_version(void);

/* Create a context on `device` for a transformed config (Simulation::Simulation,
 * simulation.cpp:58-105).  The config is copied. */
int mgpu_create(int device, const mgpu_config* cfg, mgpu_ctx** out);
int mgpu_destroy(mgpu_ctx* ctx);
/* Wait for every call issued on the context's stream (and on the caller's stream set with
 * mgpu_set_stream). */
int mgpu_sync(mgpu_ctx* ctx);

/* Instrumentation (no counterpart in the reference): launch on the caller's CUDA stream
 * (a cudaStream_t, NULL = the context's own stream), and read the device time of the last
 * simulation kernel measured with CUDA events around its launch. */
int mgpu_set_stream(mgpu_ctx* ctx, void* cuda_stream);
int mgpu_last_kernel_ms(mgpu_ctx* ctx, double* ms);

/* Test and tuning switches (no counterpart in the reference).  flags: bit 0 ranks, bit 1
 * move adjustment, bit 2 collision processing, bit 3 contact sampling use the exact serial
 * restatement instead of the warp-parallel form (results are identical either way); bit 4
 * collects the per-step cycle counters of mgpu_last_profile;
 * smem_budget caps the shared memory one cell may use (0 = device limit), placing the
 * remaining per-LEF arrays in global scratch.  Flags bits 8-15 give the shared-memory carveout
 * preference in percent and bits 16-23 cap the cells per SM (0 = the CUDA driver's default and the
 * occupancy limit). */
int mgpu_set_debug_flags(mgpu_ctx* ctx, uint32_t flags, uint64_t smem_budget);

/* Tuned settings of large batched launches (no counterpart in the reference): entries in
 * increasing max_lefs; a batch of at least 8 tasks per SM, on a context without explicit
 * mgpu_set_debug_flags budget or carveout, takes the first entry whose max_lefs is at least the
 * LEF count of its LEF-weighted median task (the last entry beyond).  smem_budget is the shared
 * memory per cell (0 = the device limit), carveout_pct the shared-memory carveout preference
 * (0 = the CUDA driver's default), max_cells_per_sm a cap on resident cells per SM (0 = the
 * occupancy limit).  The settings move arrays between shared memory and global slots; results
 * do not depend on them.  modlefork_gb300/autotune.py measures a table per device; n = 0 clears. */
typedef struct mgpu_launch_setting {
  uint64_t max_lefs;
  uint64_t smem_budget;
  uint32_t carveout_pct;
  uint32_t max_cells_per_sm;
} mgpu_launch_setting;
int mgpu_set_launch_table(mgpu_ctx* ctx, const mgpu_launch_setting* table, uint64_t n);

/* Profile of the last mgpu_simulate_cells or mgpu_simulate_batch launch made with debug flag
 * bit 4 (all zero otherwise; no counterpart in the reference): SM cycles
 * spent in each step of the epoch summed over cells (entries 0-15: burn-in, bind, rank,
 * contacts, moves, adjust, barriers, boundaries, LEF-BAR, primary, corrections, secondary,
 * fix, extrude+release, trace, total) and event counts (16: rank fallbacks, 17: adjust
 * fallbacks, 18: serial chain walks, 19: serial contact attempts, 20: fix fallbacks,
 * 21: PRNG refills, 22: refills after serial draws, 23: epochs). */
int mgpu_last_profile(mgpu_ctx* ctx, uint64_t counters[32]);

/* Upload one chromosome and its barriers (sorted with mgpu_sort_barriers order); returns a
 * handle in *chrom_id.  Barriers are shared by every cell of the chromosome. */
int mgpu_upload_chrom(mgpu_ctx* ctx, const mgpu_chrom* chrom, const mgpu_barrier* barriers,
                      uint64_t nbarriers, int* chrom_id);

/* A window of a chromosome for modle perturbate (Simulation::simulate_window,
 * scheduler_perturbate.cpp:429-480): cells bind LEFs and sample contacts inside
 * [window_start, window_end), their band covers the window (band shape of its length), while
 * moves are still clamped by the chromosome's own range [start, end); pass the window's
 * barriers (map_barriers_to_window, deleted ones with stp_active 0 and stp_inactive 1). */
int mgpu_upload_window(mgpu_ctx* ctx, const mgpu_chrom* chrom, uint64_t window_start,
                       uint64_t window_end, const mgpu_barrier* barriers, uint64_t nbarriers,
                       int* chrom_id);

/* Give one uploaded chromosome (or window) its own configuration, used instead of the
 * context's for every later launch that simulates it; NULL restores the context's.  The
 * reference runs one Config per process (simulation.hpp); with this a single
 * mgpu_simulate_batch launch advances windows of different bin sizes, LEF densities, lifetimes
 * and speeds, each cell exactly as a context created with that configuration would simulate
 * it.  The configuration is validated like mgpu_create's and must already be transformed
 * (mgpu_config_transform). */
int mgpu_set_chrom_config(mgpu_ctx* ctx, int chrom_id, const mgpu_config* cfg);

/*
 * Simulate `ncells` cells of one chromosome: the drop-in for calling
 * Simulation::simulate_one_cell once per task (scheduler_simulate.cpp:229-256).
 *   cell_seeds[i]       per-cell seed (mgpu_cell_seed);
 *   target_contacts[i]  State::num_target_contacts (0 = nothing to do in contact mode);
 *   target_epochs       State::num_target_epochs (epoch criterion);
 *   num_lefs            State::num_lefs;
 *   band                nrows*ncols uint32 band of ContactMatrixDense, column-major
 *                       (index = col*nrows + row, contact_matrix_internal_impl.hpp:40-42);
 *                       contacts are ADDED to it, like the reference's shared matrix;
 *   missed_updates      incremented by the contacts that fall outside the band (may be NULL);
 *   stats               optional per-cell results (ncells entries, may be NULL).
 * Host or device pointers are accepted for every buffer.  The call returns after the work
 * completes.
 */
int mgpu_simulate_cells(mgpu_ctx* ctx, int chrom_id, const uint64_t* cell_seeds,
                        const uint64_t* target_contacts, uint64_t target_epochs,
                        uint64_t num_lefs, uint64_t ncells, uint32_t* band,
                        uint64_t* missed_updates, mgpu_cell_stats* stats);

/*
 * mgpu_simulate_cells without any memory allocation (no counterpart in the reference, whose
 * worker threads allocate their State buffers once and reuse them).
 *
 * For callers that must not allocate device memory while they run: a process whose GPU memory
 * is all held by another allocator (a framework's caching pool, say), a loop with a fixed
 * memory budget, or a loop that cannot afford the device-wide synchronisation a cudaFree
 * implies.  The call needs a little scratch space (the per-cell task list, the work counter
 * and, for chromosomes whose per-LEF arrays do not fit in one block's shared memory, one
 * global slot per concurrently simulated cell); it takes it from one fixed array of
 * MGPU_NOALLOC_SCRATCH_BYTES that is part of the loaded library, one per device.
 *
 *   - Every buffer must be device memory of the context's device (or managed memory):
 *     cell_seeds, target_contacts and band are required,
 *     missed_updates (added to, like mgpu_simulate_cells) and stats may be NULL.
 *   - ncells may be at most MGPU_NOALLOC_MAX_CELLS; larger batches, host pointers and
 *     chromosomes whose global slot does not fit the scratch are rejected with
 *     MGPU_ERR_INVALID_ARG / MGPU_ERR_UNSUPPORTED and a message, before any work is issued.
 *   - The work counter in the scratch is cleared on the stream before each launch.
 *   - The call only enqueues work on the context's stream and returns; the results are ready
 *     after mgpu_sync (or when the stream completes).  Errors detected on the device (the
 *     per-cell status) are reported through stats[i].status, not through the return value.
 *   - The first call on a context looks up the scratch's address (cudaGetSymbolAddress) with
 *     the context's device current and keeps it with the context; make that first call before
 *     capturing the stream.  Like every buffer of a context, the address does not survive a
 *     cudaDeviceReset: destroy the context first and create a new one after the reset.
 *   - The scratch is shared by every context of the process on that device, so calls that
 *     overlap in time (two streams, two contexts, two threads) race on it and give wrong
 *     results: issue them on one stream, or synchronise between them.
 */
#define MGPU_NOALLOC_SCRATCH_BYTES (8u << 20)
#define MGPU_NOALLOC_MAX_CELLS 16384u
int mgpu_simulate_cells_noalloc(mgpu_ctx* ctx, int chrom_id, const uint64_t* cell_seeds,
                                const uint64_t* target_contacts, uint64_t target_epochs,
                                uint64_t num_lefs, uint64_t ncells, uint32_t* band,
                                uint64_t* missed_updates, mgpu_cell_stats* stats);

/*
 * Pixel table of a band, for writing a cooler (Cooler::write_or_append_cmatrix_to_file,
 * src/libmodle_io/cooler_write_impl.hpp:275-316): for bin1 row i = 0..ncols-1 and bin2
 * j = i..min(i + nrows, ncols) - 1, every non-zero count, in that order, as
 * (bin_offset + i, bin_offset + j, count).  bin_offset is the genome-wide id of the band's
 * first bin.  bin1_offset[i] receives the number of pixels before row i (ncols + 1 entries; the
 * last is the total).  bin1, bin2 and count may be NULL to query the size; otherwise they need
 * `capacity` entries, and a capacity below the total returns MGPU_ERR_OVERFLOW with *nnz set
 * and no pixel written.  Buffers may be host or device pointers.
 */
int mgpu_band_to_pixels(mgpu_ctx* ctx, const uint32_t* band, uint64_t nrows, uint64_t ncols,
                        uint64_t bin_offset, uint64_t* bin1_offset, int64_t* bin1, int64_t* bin2,
                        uint32_t* count, uint64_t capacity, uint64_t* nnz);

/*
 * One epoch of one cell as Simulation::dump_stats logs it (simulation.cpp:1166-1224), taken
 * after extrude and before release_lefs when log_model_internal_state is set.  The effective
 * barrier occupancy is barriers_occupied / nbarriers; collision counts add the rev and fwd
 * units whose word holds that event as a collision.
 */
typedef struct mgpu_epoch_record {
  uint64_t epoch;
  uint64_t cell;              /* index of the cell in the call */
  uint64_t burnin;            /* 1 while the burn-in is running */
  uint64_t barriers_occupied;
  uint64_t nbarriers;
  uint64_t num_lefs;          /* active LEFs */
  uint64_t stalled_rev;       /* rev units with a collision */
  uint64_t stalled_fwd;
  uint64_t stalled_both;      /* LEFs with both units stalled */
  uint64_t lef_bar;           /* LEF-BAR collisions (rev + fwd) */
  uint64_t lef_lef_primary;
  uint64_t lef_lef_secondary;
  double avg_loop_size;       /* stats::mean of fwd - rev over the active LEFs */
} mgpu_epoch_record;

/* Outputs beyond the band (all optional, device or host pointers). */
typedef struct mgpu_extra_outputs {
  /* with track_1d_lef_position: Chromosome::lef_1d_occupancy, ceil(chrom size / bin size)
   * counters, ADDED to (register_1d_lef_occupancy, register_contacts.cpp:200-232).  When the
   * config flag is set the sampling happens (and draws from the cell's stream) even if this
   * pointer is NULL. */
  uint64_t* lef_1d_occupancy;
  /* with log_model_internal_state: records of cell i go to epoch_records[i * max_epoch_records
   * + k] for its first max_epoch_records epochs; records_written[i] receives the number of
   * records kept (ncells entries). */
  mgpu_epoch_record* epoch_records;
  uint64_t max_epoch_records;
  uint64_t* records_written;
} mgpu_extra_outputs;

/* mgpu_simulate_cells with the optional outputs of mgpu_extra_outputs (extra may be NULL). */
int mgpu_simulate_cells_ex(mgpu_ctx* ctx, int chrom_id, const uint64_t* cell_seeds,
                           const uint64_t* target_contacts, uint64_t target_epochs,
                           uint64_t num_lefs, uint64_t ncells, uint32_t* band,
                           uint64_t* missed_updates, mgpu_cell_stats* stats,
                           const mgpu_extra_outputs* extra);

/*
 * Batched launch (no counterpart in the reference, whose worker threads pop one (chromosome,
 * cell) task at a time, scheduler_simulate.cpp:229-256): the cells of many chromosomes or
 * windows advance in one persistent kernel with a work queue, largest first.  Task i is one
 * simulate_one_cell call on chromosome handle chrom_id with its own seed, targets and LEF
 * count.  bands[chrom_id] (nbands entries, host or device pointers, NULL where no task uses the
 * chromosome) receives the contacts, added to; missed[chrom_id] is incremented (may be NULL);
 * stats[i] is task i's outcome (may be NULL).  Results equal one mgpu_simulate_cells call per
 * chromosome.  A shared-memory budget set with mgpu_set_debug_flags applies to every cell;
 * without one, large batches use 16 KiB per cell and a 60 % shared-memory carveout, so that
 * nine cells share an SM and keep an 88 KB L1 for their arrays in global slots.
 */
typedef struct mgpu_batch_task {
  uint64_t seed;
  uint64_t target_contacts;
  uint64_t target_epochs;
  uint64_t num_lefs;
  int32_t chrom_id;
  uint32_t reserved;
} mgpu_batch_task;

int mgpu_simulate_batch(mgpu_ctx* ctx, const mgpu_batch_task* tasks, uint64_t ntasks,
                        uint32_t* const* bands, uint64_t nbands, uint64_t* missed,
                        mgpu_cell_stats* stats);

/* ---- parity and debugging entry points (used by the test-suite) ------------------------ */

/*
 * Per-epoch record of one traced cell.  Arrays have num_lefs entries each and hold the
 * reference's own encodings: 64-bit positions with UINT64_MAX for unbound units,
 * 64-bit binding epochs (UINT64_MAX when unbound), 64-bit collision words
 * (index | event << 56).  A record is written at the end of every completed epoch, after
 * release_lefs (simulation.cpp:1143-1145).
 */
typedef struct mgpu_trace_header {
  uint64_t epoch;
  uint64_t num_active_lefs;
  uint64_t burnin_completed;
  uint64_t num_burnin_epochs;
  uint64_t num_contacts;
  uint64_t rng_draws;
  uint64_t n5prime; /* rev units at the 5' end (process_collisions return value) */
  uint64_t n3prime; /* fwd units at the 3' end */
  uint64_t digest;  /* mgpu_state_digest of the arrays below */
} mgpu_trace_header;

/*
 * Trace one cell.  `max_records` epochs are recorded in full into the caller's arrays
 * (headers[max_records]; each array pointer has max_records*num_lefs entries, any may be
 * NULL); every epoch's header (with the digest) goes to all_headers[max_epochs] when given.
 * `band` receives the cell's own contacts (host or device pointer, nrows*ncols entries).
 */
typedef struct mgpu_trace_request {
  uint64_t max_records;
  mgpu_trace_header* headers;
  uint64_t* rev_pos;
  uint64_t* fwd_pos;
  uint64_t* binding_epoch;
  uint64_t* rev_rank;
  uint64_t* fwd_rank;
  uint64_t* rev_move;
  uint64_t* fwd_move;
  uint64_t* rev_collision;
  uint64_t* fwd_collision;
  uint64_t max_epochs;
  mgpu_trace_header* all_headers;
  uint64_t num_epochs_recorded; /* out: epochs written to all_headers */
} mgpu_trace_request;

int mgpu_trace_cell(mgpu_ctx* ctx, int chrom_id, uint64_t cell_seed, uint64_t target_contacts,
                    uint64_t target_epochs, uint64_t num_lefs, uint32_t* band,
                    mgpu_cell_stats* stats, mgpu_trace_request* trace);

/* Order-independent 64-bit digest of one epoch's state (the same formula is computed on
 * the device): sum over i of mix(i, rev_pos[i], fwd_pos[i], binding_epoch[i], rev_rank[i],
 * fwd_rank[i], rev_move[i], fwd_move[i], rev_collision[i], fwd_collision[i]). */
uint64_t mgpu_state_digest(uint64_t num_lefs, const uint64_t* rev_pos, const uint64_t* fwd_pos,
                           const uint64_t* binding_epoch, const uint64_t* rev_rank,
                           const uint64_t* fwd_rank, const uint64_t* rev_move,
                           const uint64_t* fwd_move, const uint64_t* rev_collision,
                           const uint64_t* fwd_collision);

/*
 * Run one step of the epoch loop on the device on caller-provided state, in the reference's
 * encodings; this is how the reference's own step-level unit tests run against the kernels.
 * All arrays have num_lefs entries and are read and written in place (host memory).
 */
enum mgpu_phase {
  /* one entry per test hook of the reference (simulation.hpp:499-651) */
  MGPU_PHASE_BIND = 1,               /* test_bind_lefs: bind_lefs (simulation_impl.hpp:28-67) */
  MGPU_PHASE_RANK = 2,               /* test_rank_lefs: rank_lefs (simulation.cpp:402-487) */
  MGPU_PHASE_ADJUST_AND_CLAMP = 3,   /* test_adjust_and_clamp_moves (simulation.cpp:325-399) */
  MGPU_PHASE_GENERATE_MOVES = 4,     /* test_generate_moves: generate_moves (simulation.cpp:292-323) */
  MGPU_PHASE_PROCESS_COLLISIONS = 5, /* test_process_collisions: process_collisions without fix */
  MGPU_PHASE_FIX_SECONDARY = 6,      /* test_fix_secondary_lef_lef_collisions (n5 = n3 = 0) */
  MGPU_PHASE_DETECT_LEF_BAR = 7,     /* test_detect_lef_bar_collisions (n5 = n3 = 0) */
  MGPU_PHASE_LEF_LEF = 8,            /* test_process_lef_lef_collisions (n5 = n3 = 0) */
  MGPU_PHASE_DETECT_PRIMARY = 9,     /* test_detect_primary_lef_lef_collisions (n5 = n3 = 0) */
  MGPU_PHASE_EXTRUDE = 10,           /* extrude (simulation.cpp:489-512) */
  MGPU_PHASE_RELEASE = 11,           /* release_lefs (simulation.cpp:544-592) */
  MGPU_PHASE_BARRIER_NEXT = 12,      /* ExtrusionBarriers::next_state (extrusion_barriers.cpp:145-161) */
  MGPU_PHASE_BARRIER_INIT = 13,      /* ExtrusionBarriers::init_states (extrusion_barriers.cpp:220-231) */
  MGPU_PHASE_DETECT_BOUNDARIES = 14, /* test_detect_units_at_chrom_boundaries */
  MGPU_PHASE_CORRECT_LEF_BAR = 15,   /* test_correct_moves_for_lef_bar_collisions */
  MGPU_PHASE_CORRECT_PRIMARY = 16    /* test_adjust_moves_for_primary_lef_lef_collisions */
};

typedef struct mgpu_phase_io {
  uint64_t num_lefs;
  uint64_t* rev_pos;
  uint64_t* fwd_pos;
  uint64_t* binding_epoch;
  uint64_t* rev_rank;
  uint64_t* fwd_rank;
  uint64_t* rev_move;
  uint64_t* fwd_move;
  uint64_t* rev_collision;
  uint64_t* fwd_collision;
  uint64_t* bind_mask;      /* MGPU_PHASE_BIND: nonzero = bind this LEF; NULL = bind all */
  uint8_t* barrier_state;   /* nbarriers entries, 1 = occupied; read and written */
  uint64_t epoch;           /* current epoch (bind, rank) */
  uint32_t burnin_completed;
  uint32_t ranks_partially_sorted; /* rank: 1 = split_sort, 0 = pdq_sort */
  uint32_t init_ranks;      /* rank: iota the rank buffers first */
  uint32_t adjust_moves;    /* generate_moves: also adjust consecutive units */
  uint64_t prng_state[4];   /* Xoshiro256++ state, read and written */
  uint64_t n5prime;         /* out */
  uint64_t n3prime;         /* out */
  uint64_t lefs_released;   /* out (release) */
} mgpu_phase_io;

int mgpu_run_phase(mgpu_ctx* ctx, int chrom_id, int phase, mgpu_phase_io* io);

/* Xoshiro256++ seeded through SplitMix64 (random::PRNG, random.hpp:26-30): writes the state. */
void mgpu_prng_seed(uint64_t seed, uint64_t state[4]);

/*
 * Probes of the device's floating-point arithmetic (test hooks, no counterpart in the
 * reference).  The reference computes its transcendentals with the host's libm (glibc); the
 * device uses CUDA's.  These run the epoch loop's own device code so that the test-suite can
 * compare it with the host, bit for bit, on the argument streams the loop feeds it.
 *
 * mgpu_probe_samplers: per_stream samples from each of nstreams seeded streams (seed as for
 * mgpu_prng_seed) through the serial samplers the epoch loop uses; out[s * per_stream + i] is
 * sample i of stream s and draws[s] the raw 64-bit draws stream s consumed (UINT64_MAX if a
 * sampler hit its iteration limit).  Kinds and parameters:
 *   MGPU_PROBE_NORMAL              normal(a0, a1): move lengths (simulation.cpp:264-290)
 *   MGPU_PROBE_EXPONENTIAL         unit exponential (the normal's tail)
 *   MGPU_PROBE_POISSON             Poisson(a0): burn-in activations (simulation.cpp:1031-1032)
 *   MGPU_PROBE_BINOMIAL            binomial(a0, a1): loop/TAD split (register_contacts.cpp:73-92)
 *                                  with (1 - p)^t taken from the host, as in a full epoch
 *   MGPU_PROBE_BINOMIAL_DEVICE_POW the same with (1 - p)^t evaluated on the device (last epoch)
 *   MGPU_PROBE_GEV                 genextreme(0, a0, a1) noise (genextreme_value_distribution.hpp:87-105)
 * mgpu_probe_libm: out[i] = f(x[i], y[i]) on the device for
 *   MGPU_PROBE_LOG log x, MGPU_PROBE_EXP exp x, MGPU_PROBE_POW pow(x, y),
 *   MGPU_PROBE_GEV_NOISE the GEV noise of a uniform x with (mu, sigma, xi),
 *   MGPU_PROBE_BELOW_EXP 1.0 if x < exp(y) as the ziggurat decides it, else 0.0.
 * Host buffers; the calls allocate and synchronise the device.
 */
#define MGPU_PROBE_NORMAL 0
#define MGPU_PROBE_EXPONENTIAL 1
#define MGPU_PROBE_POISSON 2
#define MGPU_PROBE_BINOMIAL 3
#define MGPU_PROBE_BINOMIAL_DEVICE_POW 4
#define MGPU_PROBE_GEV 5
#define MGPU_PROBE_LOG 0
#define MGPU_PROBE_EXP 1
#define MGPU_PROBE_POW 2
#define MGPU_PROBE_GEV_NOISE 3
#define MGPU_PROBE_BELOW_EXP 4
int mgpu_probe_samplers(int device, int kind, const uint64_t* seeds, uint64_t nstreams, uint64_t per_stream,
                        double a0, double a1, double* out, uint64_t* draws);
int mgpu_probe_libm(int device, int kind, const double* x, const double* y, uint64_t n, double mu,
                    double sigma, double xi, double* out);

#ifdef __cplusplus
}
#endif

#endif /* MGPU_MODLE_H */
