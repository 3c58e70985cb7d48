// Internal declarations shared by the host library (mgpu_host.cpp) and the device code
// (mgpu_device.cu).  Nothing here is part of the C ABI.
#pragma once
#include <stdint.h>

#include "../../include/mgpu_modle.h"

#if defined(__CUDACC__)
#define MGPU_HD __host__ __device__
#else
#define MGPU_HD
#endif

namespace mgpu {

typedef uint32_t u32;
typedef uint64_t u64;
typedef int64_t i64;

// Unbound unit / LEF sentinel for the 32-bit device encodings.
constexpr u32 UNBOUND = 0xFFFFFFFFu;

// PRNG ring: each of the 32 lanes of a cell's warp generates RNG_S consecutive draws of the
// cell's single Xoshiro256++ stream per refill; RING is a power of two holding two blocks.
constexpr int RNG_S = 16;
constexpr int RNG_BLOCK = 32 * RNG_S;
constexpr int RING = 2 * RNG_BLOCK;
constexpr int JUMP_DISTANCE = 31 * RNG_S;  // lane state advance between two refills
constexpr int JUMP_TABLE_ENTRIES = 64 * 16;  // 4-bit chunks of the 256-bit state

// Compact 32-bit collision word: event bits (collision_encoding.hpp:91-96) in bits 27..31,
// index in bits 0..26.
constexpr u32 CW_SHIFT = 27;
constexpr u32 CW_IDX_MASK = (1u << CW_SHIFT) - 1;
constexpr u32 EV_COLLISION = 0x10, EV_CHROM_BOUNDARY = 0x08, EV_LEF_BAR = 0x04,
              EV_PRIMARY = 0x02, EV_SECONDARY = 0x01;

MGPU_HD inline u32 cw_make(u32 idx, u32 ev) { return (idx & CW_IDX_MASK) | (ev << CW_SHIFT); }
MGPU_HD inline u32 cw_idx(u32 w) { return w & CW_IDX_MASK; }
MGPU_HD inline u32 cw_event(u32 w) { return w >> CW_SHIFT; }
MGPU_HD inline bool cw_occurred(u32 w) { return (w >> CW_SHIFT) & EV_COLLISION; }
MGPU_HD inline bool cw_occurred_as(u32 w, u32 c) { return (w >> CW_SHIFT) == (c | EV_COLLISION); }
MGPU_HD inline bool cw_avoided_as(u32 w, u32 c) { return !cw_occurred(w) && (w >> CW_SHIFT) == c; }
// reference 64-bit word: idx | event << 56
MGPU_HD inline u64 cw_to_ref(u32 w) { return (u64)(w & CW_IDX_MASK) | ((u64)(w >> CW_SHIFT) << 56); }
MGPU_HD inline u32 cw_from_ref(u64 w) {
  return (u32)(w & CW_IDX_MASK) | ((u32)((w >> 56) & 0x1F) << CW_SHIFT);
}

// Barrier as seen by the kernels: integer thresholds replace the floating-point tests of
// init_states (bernoulli), next_state (generate_canonical > stp).
enum : u32 {
  BF_DIR_MASK = 3u,        // MGPU_DIR_REV / MGPU_DIR_FWD
  BF_OCC_DRAWS = 1u << 2,  // occupancy != 0: init_states draws for this barrier
  BF_INA_NEVER = 1u << 3,  // no draw can make a free barrier occupied
  BF_ACT_NEVER = 1u << 4,  // no draw can make an occupied barrier free
};
struct DevBarrier {
  u64 t_occ;  // init: occupied iff draw <= t_occ
  u64 t_ina;  // free -> occupied iff draw >= t_ina
  u64 t_act;  // occupied -> free iff draw >= t_act
  u32 pos;
  u32 flags;
};

// Bernoulli trial with integer threshold: success iff draw <= thr; no draw when !draws.
struct Trial {
  u64 thr;
  u32 draws;  // 0: p == 0, the reference returns false without drawing
  u32 always; // 1: the reference short-circuits to true without drawing
};

struct KParams {
  u32 start, end;    // chromosome range [start, end): move clamps, boundary collisions
  u32 wstart, wend;  // simulated window: binding, contacts and the band (= start, end for a chromosome)
  u32 bin, nrows, ncols;
  u32 nlefs, nbarriers;
  u32 hist_cap, smooth_w;
  u32 skip_burnin;
  u64 min_burnin, max_burnin;
  // moves: [0] = burn-in speeds, [1] = after burn-in
  double rev_speed[2], fwd_speed[2];
  double rev_std, fwd_std;
  u64 rev_move_int[2], fwd_move_int[2];
  // release_lefs: [burnin_completed][number of hard LEF-BAR collisions 0..2]
  Trial release[2][3];
  Trial lef_lef;      // run_lef_lef_collision_trial
  Trial lef_bar[2];   // run_lef_bar_collision_trial: [0] major pblock, [1] minor pblock
  // burn-in Poisson(nlefs / burnin_target_epochs) (constants computed on the host)
  double pois_mean, pois_exp_mean, pois_smu, pois_b, pois_a, pois_inv_alpha, pois_v_r;
  // contacts
  u64 spe;               // sampling events per epoch
  u32 contact_mode;      // target_contact_density >= 0
  u32 density_positive;  // target_contact_density > 0
  u32 ratio_mode;        // 0: all loop, 1: all TAD, 2: binomial split
  u32 noisify;
  double p_loop;         // 1 / (ratio + 1)
  double gev_mu, gev_sigma, gev_xi;
  // binomial(spe, p_loop) constants computed on the host
  double bin_q_n;
  // binding positions: uniform_int[start, end - 1]
  u64 pos_bucket;
  u64 pos_range;
  // per-LEF array layout (planned on the host): byte offset of each array inside the shared
  // memory of the cell or inside its global scratch slot
  u32 arr_off[12];
  u32 arr_smem;    // bit k set: array k lives in shared memory
  u32 smem_bytes;  // dynamic shared memory of one cell
  u64 slot_bytes;  // global scratch of one resident cell (arrays that do not fit on chip)
  u32 debug_flags; // DBG_* bits: force the exact serial implementation of a step
  u64* prof;       // per-launch profile counters (32 entries, device memory) or null
  // optional outputs (mgpu_extra_outputs)
  u32 track_occ;               // sample the 1D LEF occupancy (draws even without a buffer)
  u32 log_state;               // write per-epoch model-state records
  unsigned long long* occ;     // occupancy counters (occ_bins entries) or null
  u64 occ_bins;
  mgpu_epoch_record* records;  // records of cell i at records + i * rec_max, or null
  u64 rec_max;
  u64* rec_count;              // per cell number of records written, or null
};

// Per-LEF arrays of a cell, in on-chip placement priority order.  SR and SF are adjacent:
// together they also serve as a double-precision scratch of nlefs entries.
enum : u32 {
  ARR_REV = 0, ARR_FWD, ARR_RR, ARR_FR, ARR_RM, ARR_FM, ARR_RC, ARR_FC, ARR_SR, ARR_SF,
  ARR_TMP, ARR_BEP, NARR
};
constexpr u32 CELL_HEADER_BYTES = 256;  // per-cell scalars at the start of shared memory

enum : u32 {
  DBG_SERIAL_RANK = 1u << 0,
  DBG_SERIAL_ADJUST = 1u << 1,
  DBG_SERIAL_COLLISIONS = 1u << 2,
  DBG_SERIAL_CONTACTS = 1u << 3,
  DBG_PROFILE = 1u << 4,  // collect per-step cycle counters (mgpu_last_profile)
};

struct CellTask {
  u64 seed;
  u64 target_contacts;
};

// Per-cell trace output (device pointers; all NULL when tracing is off).
struct DevTrace {
  u64 max_records;
  mgpu_trace_header* headers;
  u64 *rev_pos, *fwd_pos, *binding_epoch, *rev_rank, *fwd_rank, *rev_move, *fwd_move,
      *rev_collision, *fwd_collision;
  u64 max_epochs;
  mgpu_trace_header* all_headers;
  u64* num_recorded;
};

// Device error codes reported through mgpu_cell_stats::status (0 = OK).
enum : u32 {
  DEV_OK = 0,
  DEV_ERR_ITER_LIMIT = 1,    // a rejection loop hit its iteration limit
  DEV_ERR_MOVE_RANGE = 2,    // a move does not fit the 32-bit encoding
  DEV_ERR_BAD_STATE = 3,     // the reference would read out of bounds here
  DEV_ERR_NO_BOUND_LEF = 4,  // contact sampling found no bound LEF within bounds
};

// Fixed part of a cell's shared memory: scalars, PRNG ring, burn-in history, barrier bits.
MGPU_HD inline u64 cell_header_bytes(u64 nbarriers, u64 hist_cap) {
  const u64 ring = (u64)RING * 8;
  const u64 hist = 2 * hist_cap * 8;
  const u64 bars = (((nbarriers + 31) / 32) * 4 + 15) & ~15ull;
  return CELL_HEADER_BYTES + ring + hist + bars;
}

// Host side helpers implemented in mgpu_host.cpp, device launchers in mgpu_device.cu.
struct DevChrom {
  const DevBarrier* barriers;
  const uint2* pos_flags;  // {pos, flags} of each barrier: the compact copy the sweeps read
  u32 nbarriers;
};

int launch_simulate(const KParams& P, const DevChrom& ch, const CellTask* tasks, u64 ncells,
                    u64 target_epochs, u32* band, u64* missed, mgpu_cell_stats* stats,
                    const DevTrace* trace, const void* jump_table, u32* work_counter,
                    char* gscratch, u64 gscratch_bytes, void* stream, char* errbuf, int errlen);
// Number of cells resident at once for a launch (grid size of the persistent kernel).
u64 resident_cells(const KParams& P, u64 ncells);
int launch_phase(const KParams& P, const DevChrom& ch, int phase, u64 n, u64* arrays,
                 u64* bind_mask, uint8_t* barrier_state, u64 epoch, u32 burnin_completed,
                 u32 partially_sorted, u32 init_ranks, u32 adjust, u64* prng_state, u64* outs,
                 const void* jump_table, char* gscratch, void* stream, char* errbuf, int errlen);
u64 max_smem_per_block();

// Fixed scratch of mgpu_simulate_cells_noalloc: [0, 256) work counter, then the task list of
// up to MGPU_NOALLOC_MAX_CELLS cells, then global cell slots in what is left.
constexpr u64 NOALLOC_TASKS_OFFSET = 256;
constexpr u64 NOALLOC_SLOTS_OFFSET =
    (NOALLOC_TASKS_OFFSET + (u64)MGPU_NOALLOC_MAX_CELLS * sizeof(CellTask) + 255) & ~255ull;
static_assert(NOALLOC_SLOTS_OFFSET < MGPU_NOALLOC_SCRATCH_BYTES, "task list larger than the scratch");
// Batched launch: many (chromosome or window, LEF count) plans, one work queue of cells.
struct BatchPlan {
  KParams P;  // layout planned under the launch's common shared-memory size
  DevChrom ch;
  u32* band;
  unsigned long long* missed;  // this plan's missed updates (device)
  u64 target_epochs;
};
struct BatchTask {
  u64 seed;
  u64 target_contacts;
  u32 plan;
  u32 pad;
};
int launch_simulate_batch(const BatchPlan* plans, const BatchTask* tasks, u64 ntasks, u32 smem_bytes,
                          u64 slot_bytes, mgpu_cell_stats* stats, const void* jump_table, u32* work_counter,
                          char* gscratch, u64 gscratch_bytes, u32 carveout_pct, u32 max_per_sm, void* stream,
                          char* errbuf, int errlen);
// Grid of a batched launch with the given per-cell shared memory (optionally capped per SM, with
// a shared-memory carveout preference in percent, 0 = driver default).
u64 resident_batch_cells(u32 smem_bytes, u64 ntasks, u32 carveout_pct = 0, u32 max_per_sm = 0);

// Pixel table of a band (mgpu_pixels.cu): counts[i] = non-zero pixels of bin1 row i,
// offsets[0..ncols] their exclusive scan; then the (bin1, bin2, count) pixels.
int launch_band_counts(const u32* band, u64 nrows, u64 ncols, u32* counts, u64* offsets, void* stream,
                       char* errbuf, int errlen);
int launch_band_pixels(const u32* band, u64 nrows, u64 ncols, u64 bin_offset, const u64* offsets,
                       int64_t* bin1, int64_t* bin2, u32* count, void* stream, char* errbuf, int errlen);

// Test hooks: the epoch loop's serial samplers on seeded streams (kind 0 normal(a0, a1),
// 1 unit exponential, 2 Poisson(P.pois_*), 3 binomial(a0, a1) with P.spe / P.bin_q_n, 4 GEV
// with P.gev_*) and the device's log / exp / pow / GEV noise / below_exp on arguments.
int launch_sampler_probe(const KParams& P, int kind, const u64* states, u64 nstreams, u64 per, double a0,
                         double a1, double* out, u64* draws, void* stream, char* errbuf, int errlen);
int launch_libm_probe(int kind, const double* x, const double* y, u64 n, double mu, double sigma, double xi,
                      double* out, void* stream, char* errbuf, int errlen);

// Address of the scratch on the current device.
int noalloc_scratch_address(void** ptr, char* errbuf, int errlen);
// tasks[i] = {seeds[i], targets[i]} on the stream.
int launch_pack_tasks(const u64* seeds, const u64* targets, u64 n, CellTask* tasks, void* stream,
                      char* errbuf, int errlen);

}  // namespace mgpu
