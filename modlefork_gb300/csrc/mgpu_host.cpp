// mgpu_host.cpp - host side of the C ABI declared in include/mgpu_modle.h.
//
// Responsibilities: the Config derivations of the reference CLI, per-cell seeds (XXH3),
// conversion of every floating-point random test of the epoch loop into an exact integer
// threshold on the raw 64-bit draw, the GF(2) jump table of the per-warp PRNG, device buffer
// management and kernel launches.

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "cppsort_emul.h"
#include "mgpu_internal.h"

using namespace mgpu;

static thread_local std::string g_last_error;

static int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

static int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return MGPU_OK;
  if (e == cudaErrorMemoryAllocation) return fail(MGPU_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(MGPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr)                                  \
  do {                                            \
    const int rc_ = cuda_check((expr), #expr);    \
    if (rc_ != MGPU_OK) return rc_;               \
  } while (0)

// ===========================================================================================
// Config (simulation_config.hpp:60-124) and Cli::transform_args (cli.cpp:1086-1215)
// ===========================================================================================
extern "C" void mgpu_config_defaults(mgpu_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->target_simulation_epochs = 2000;
  c->target_contact_density = 1.0;
  c->bin_size = 5000;
  c->diagonal_width = 3000000;
  c->contact_sampling_strategy = MGPU_CS_TAD | MGPU_CS_LOOP | MGPU_CS_NOISIFY;
  c->tad_to_loop_contact_ratio = 5.0;
  c->genextreme_mu = 0.0;
  c->genextreme_sigma = 5000.0;
  c->genextreme_xi = 0.001;
  c->fwd_extrusion_speed = c->bin_size * 8 / 10;
  c->rev_extrusion_speed = c->fwd_extrusion_speed;
  c->fwd_extrusion_speed_std = 0.05;
  c->rev_extrusion_speed_std = 0.05;
  c->number_of_lefs_per_mbp = 20.0;
  c->avg_lef_processivity = 300000;
  c->contact_sampling_interval = 50000;
  c->extrusion_barrier_occupancy = 0.825;
  c->barrier_occupied_stp = 0.0;
  c->barrier_not_occupied_stp = 0.70;
  c->hard_stall_lef_stability_multiplier = 5.0;
  c->soft_stall_lef_stability_multiplier = 1.0;
  c->probability_of_extrusion_unit_bypass = 0.1;
  c->lef_bar_major_collision_pblock = 1.0;
  c->lef_bar_minor_collision_pblock = 0.0;
  c->num_cells = 512;
  c->seed = 0;
  c->probability_normalization_factor = c->rev_extrusion_speed + c->fwd_extrusion_speed;
  c->normalize_probabilities = 1;
  c->burnin_history_length = 100;
  c->burnin_smoothing_window_size = 5;
  c->min_burnin_epochs = 0;
  c->max_burnin_epochs = std::numeric_limits<uint64_t>::max();
  c->burnin_target_epochs_for_lef_activation = 320;
  c->burnin_speed_coefficient = 1.0;
  c->fwd_extrusion_speed_burnin = (uint64_t)((double)c->fwd_extrusion_speed * 1.0);
  c->rev_extrusion_speed_burnin = c->fwd_extrusion_speed_burnin;
}

// ExtrusionBarrier::compute_stp_active_from_occupancy (extrusion_barriers_impl.hpp:106-116)
static double stp_active_from_occupancy(double stp_inactive, double occupancy) {
  if (occupancy == 0) return 0.0;
  const double ia = 1.0 - stp_inactive;
  const double ai = (ia - (occupancy * ia)) / occupancy;
  return std::clamp(1.0 - ai, 0.0, 1.0);
}

// ExtrusionBarrier::compute_occupancy_from_stp (extrusion_barriers_impl.hpp:118-128)
static double occupancy_from_stp(double stp_active, double stp_inactive) {
  if (stp_active + stp_inactive == 0) return 0.0;
  const double ia = 1.0 - stp_inactive;
  const double ai = 1.0 - stp_active;
  return std::clamp(ia / (ia + ai), 0.0, 1.0);
}

extern "C" int mgpu_config_transform(mgpu_config* c) {
  if (!c) return fail(MGPU_ERR_INVALID_ARG, "mgpu_config_transform: null config");
  if (c->bin_size == 0) return fail(MGPU_ERR_INVALID_ARG, "bin_size must be positive");
  // cli_update_extr_speed (:1086-1110)
  if (!c->rev_speed_set) c->rev_extrusion_speed = c->bin_size * 8 / 10;
  if (!c->fwd_speed_set) c->fwd_extrusion_speed = c->bin_size * 8 / 10;
  if (c->fwd_extrusion_speed_std > 0 && c->fwd_extrusion_speed_std < 1)
    c->fwd_extrusion_speed_std *= (double)c->fwd_extrusion_speed;
  if (c->rev_extrusion_speed_std > 0 && c->rev_extrusion_speed_std < 1)
    c->rev_extrusion_speed_std *= (double)c->rev_extrusion_speed;
  c->rev_extrusion_speed_burnin =
      (uint64_t)std::round(c->burnin_speed_coefficient * (double)c->rev_extrusion_speed);
  c->fwd_extrusion_speed_burnin =
      (uint64_t)std::round(c->burnin_speed_coefficient * (double)c->fwd_extrusion_speed);
  // cli_compute_prob_of_lef_release (:1113-1119)
  if (c->avg_lef_processivity == 0) return fail(MGPU_ERR_INVALID_ARG, "avg_lef_processivity must be positive");
  c->prob_of_lef_release =
      (double)(c->rev_extrusion_speed + c->fwd_extrusion_speed) / (double)c->avg_lef_processivity;
  c->prob_of_lef_release_burnin =
      (double)(c->rev_extrusion_speed_burnin + c->fwd_extrusion_speed_burnin) /
      (double)c->avg_lef_processivity;
  // cli_update_barrier_stp_and_occupancy (:1122-1135)
  if (c->occupancy_set) {
    c->barrier_occupied_stp =
        stp_active_from_occupancy(c->barrier_not_occupied_stp, c->extrusion_barrier_occupancy);
  } else {
    c->extrusion_barrier_occupancy =
        occupancy_from_stp(c->barrier_occupied_stp, c->barrier_not_occupied_stp);
  }
  // cli_update_tad_to_loop_contact_ratio (:1169-1182)
  const bool loop = (c->contact_sampling_strategy & MGPU_CS_LOOP) != 0;
  const bool tad = (c->contact_sampling_strategy & MGPU_CS_TAD) != 0;
  if (!loop && !tad) return fail(MGPU_ERR_INVALID_ARG, "contact sampling needs loop or tad");
  if (loop && !tad) c->tad_to_loop_contact_ratio = 0;
  if (!loop && tad) c->tad_to_loop_contact_ratio = std::numeric_limits<double>::infinity();
  // cli_update_burnin_params (:1184-1190)
  const uint64_t speeds = c->rev_extrusion_speed_burnin + c->fwd_extrusion_speed_burnin;
  if (speeds == 0) return fail(MGPU_ERR_INVALID_ARG, "burn-in extrusion speeds sum to zero");
  c->burnin_target_epochs_for_lef_activation =
      std::min(c->max_burnin_epochs, (5 * c->avg_lef_processivity) / speeds);
  // cli_normalize_probabilities (:1138-1167)
  if (c->normalize_probabilities) {
    if (c->probability_normalization_factor == 0)
      return fail(MGPU_ERR_INVALID_ARG, "probability_normalization_factor must be positive");
    const double ratio = (double)(c->rev_extrusion_speed + c->fwd_extrusion_speed) /
                         (double)c->probability_normalization_factor;
    if (ratio != 1.0) {
      auto stable_pow = [](double base, double e) {
        if (base == 0.0) return 0.0;
        if (base == 1.0) return 1.0;
        return std::exp(std::log(base) * e);
      };
      c->barrier_not_occupied_stp = stable_pow(c->barrier_not_occupied_stp, ratio);
      c->barrier_occupied_stp =
          stp_active_from_occupancy(c->barrier_not_occupied_stp, c->extrusion_barrier_occupancy);
      const double p = c->probability_of_extrusion_unit_bypass;
      if (p != 0.0 && p != 1.0) c->probability_of_extrusion_unit_bypass = std::min(p * ratio, 1.0);
      c->lef_bar_major_collision_pblock = stable_pow(c->lef_bar_major_collision_pblock, ratio);
      c->lef_bar_minor_collision_pblock = stable_pow(c->lef_bar_minor_collision_pblock, ratio);
    }
  }
  if (c->stop_on_epochs) c->target_contact_density = -1;
  return MGPU_OK;
}

extern "C" uint64_t mgpu_num_lefs(const mgpu_config* c, uint64_t size_bp) {
  const double mbp = (double)size_bp / 1.0e6;
  return std::max<uint64_t>(1, (uint64_t)std::round(c->number_of_lefs_per_mbp * mbp));
}

extern "C" uint64_t mgpu_contacts_per_epoch(const mgpu_config* c, uint64_t nlefs) {
  const double speed = (double)(c->rev_extrusion_speed + c->fwd_extrusion_speed);
  const double p = speed / (double)c->contact_sampling_interval;
  return (uint64_t)std::max(1.0, std::round((double)nlefs * p));
}

extern "C" uint64_t mgpu_npixels(const mgpu_config* c, uint64_t size_bp) {
  const uint64_t npix1 = (c->diagonal_width + c->bin_size - 1) / c->bin_size;
  const uint64_t npix2 = (size_bp + c->bin_size - 1) / c->bin_size;
  return std::min(npix1, npix2) * npix2;
}

extern "C" void mgpu_band_shape(const mgpu_config* c, uint64_t size_bp, uint64_t* nrows,
                                uint64_t* ncols) {
  const uint64_t r = (c->diagonal_width + c->bin_size - 1) / c->bin_size;
  const uint64_t cc = (size_bp + c->bin_size - 1) / c->bin_size;
  if (nrows) *nrows = std::min(r, cc);
  if (ncols) *ncols = cc;
}

extern "C" int mgpu_task_targets(const mgpu_config* c, uint64_t size_bp, uint64_t nlefs,
                                 uint64_t ncells, uint64_t* targets, uint64_t* target_epochs) {
  if (!c || (ncells && !targets)) return fail(MGPU_ERR_INVALID_ARG, "mgpu_task_targets: null argument");
  if (c->num_cells == 0) return fail(MGPU_ERR_INVALID_ARG, "num_cells must be positive");
  const uint64_t npixels = mgpu_npixels(c, size_bp);
  const uint64_t tot = (uint64_t)std::round((double)npixels * c->target_contact_density);
  uint64_t epochs;
  if (c->stop_on_epochs) {
    epochs = c->num_cells * c->target_simulation_epochs;
  } else {
    const double tt = std::max(1.0, std::round(c->target_contact_density * (double)npixels));
    epochs = (uint64_t)std::round(tt / (double)mgpu_contacts_per_epoch(c, nlefs));
  }
  if (target_epochs) *target_epochs = epochs;
  const uint64_t per_cell = (tot + c->num_cells - 1) / c->num_cells;
  uint64_t rolling = 0;
  for (uint64_t i = 0; i < ncells; ++i) {
    const uint64_t eff = std::min(per_cell, tot - rolling);
    rolling += eff;
    targets[i] = eff;
  }
  return MGPU_OK;
}

extern "C" int mgpu_barrier_from_bed(const mgpu_chrom* chrom, uint64_t chrom_start,
                                     uint64_t chrom_end, char strand, double score,
                                     double default_stp_active, double default_stp_inactive,
                                     mgpu_barrier* out) {
  if (!chrom || !out) return fail(MGPU_ERR_INVALID_ARG, "mgpu_barrier_from_bed: null argument");
  if (strand != '+' && strand != '-') return fail(MGPU_ERR_INVALID_ARG, "strand must be '+' or '-'");
  const uint64_t pos = (chrom_start + chrom_end + 1) / 2;  // genome.cpp:199
  if (pos < chrom->start || pos >= chrom->end) return 0;
  double sa = default_stp_active, si = default_stp_inactive;
  if (score != 0.0) sa = stp_active_from_occupancy(default_stp_inactive, score);  // genome.cpp:181-192
  std::memset(out, 0, sizeof(*out));
  out->pos = pos;
  out->stp_active = sa;
  out->stp_inactive = si;
  out->blocking_dir = strand == '+' ? MGPU_DIR_REV : MGPU_DIR_FWD;  // extrusion_barriers_impl.hpp:67
  return 1;
}

extern "C" int mgpu_sort_barriers(mgpu_barrier* b, uint64_t n) {
  if (n == 0) return MGPU_OK;
  if (!b) return fail(MGPU_ERR_INVALID_ARG, "mgpu_sort_barriers: null barriers");
  std::vector<u32> key(n), idx(n);
  for (uint64_t i = 0; i < n; ++i) {
    if (b[i].pos >= 0xFFFFFFFFull) return fail(MGPU_ERR_UNSUPPORTED, "barrier position beyond 2^32 - 2");
    key[i] = (u32)b[i].pos;
    idx[i] = (u32)i;
  }
  pdq_sort(idx.data(), 0, (i64)n, KeyCmp{key.data()});
  std::vector<mgpu_barrier> tmp(b, b + n);
  for (uint64_t k = 0; k < n; ++k) b[k] = tmp[idx[k]];
  return MGPU_OK;
}

// ===========================================================================================
// XXH3-64 with seed (xxHash 0.8 spec, inputs up to 240 bytes), for Chromosome::hash
// ===========================================================================================
namespace xxh {
static const uint8_t kSecret[192] = {
    0xb8, 0xfe, 0x6c, 0x39, 0x23, 0xa4, 0x4b, 0xbe, 0x7c, 0x01, 0x81, 0x2c, 0xf7, 0x21, 0xad, 0x1c,
    0xde, 0xd4, 0x6d, 0xe9, 0x83, 0x90, 0x97, 0xdb, 0x72, 0x40, 0xa4, 0xa4, 0xb7, 0xb3, 0x67, 0x1f,
    0xcb, 0x79, 0xe6, 0x4e, 0xcc, 0xc0, 0xe5, 0x78, 0x82, 0x5a, 0xd0, 0x7d, 0xcc, 0xff, 0x72, 0x21,
    0xb8, 0x08, 0x46, 0x74, 0xf7, 0x43, 0x24, 0x8e, 0xe0, 0x35, 0x90, 0xe6, 0x81, 0x3a, 0x26, 0x4c,
    0x3c, 0x28, 0x52, 0xbb, 0x91, 0xc3, 0x00, 0xcb, 0x88, 0xd0, 0x65, 0x8b, 0x1b, 0x53, 0x2e, 0xa3,
    0x71, 0x64, 0x48, 0x97, 0xa2, 0x0d, 0xf9, 0x4e, 0x38, 0x19, 0xef, 0x46, 0xa9, 0xde, 0xac, 0xd8,
    0xa8, 0xfa, 0x76, 0x3f, 0xe3, 0x9c, 0x34, 0x3f, 0xf9, 0xdc, 0xbb, 0xc7, 0xc7, 0x0b, 0x4f, 0x1d,
    0x8a, 0x51, 0xe0, 0x4b, 0xcd, 0xb4, 0x59, 0x31, 0xc8, 0x9f, 0x7e, 0xc9, 0xd9, 0x78, 0x73, 0x64,
    0xea, 0xc5, 0xac, 0x83, 0x34, 0xd3, 0xeb, 0xc3, 0xc5, 0x81, 0xa0, 0xff, 0xfa, 0x13, 0x63, 0xeb,
    0x17, 0x0d, 0xdd, 0x51, 0xb7, 0xf0, 0xda, 0x49, 0xd3, 0x16, 0x55, 0x26, 0x29, 0xd4, 0x68, 0x9e,
    0x2b, 0x16, 0xbe, 0x58, 0x7d, 0x47, 0xa1, 0xfc, 0x8f, 0xf8, 0xb8, 0xd1, 0x7a, 0xd0, 0x31, 0xce,
    0x45, 0xcb, 0x3a, 0x8f, 0x95, 0x16, 0x04, 0x28, 0xaf, 0xd7, 0xfb, 0xca, 0xbb, 0x4b, 0x40, 0x7e,
};
constexpr uint64_t P32_1 = 0x9E3779B1u, P32_2 = 0x85EBCA77u, P32_3 = 0xC2B2AE3Du;
constexpr uint64_t P64_1 = 0x9E3779B185EBCA87ull, P64_2 = 0xC2B2AE3D27D4EB4Full,
                   P64_3 = 0x165667B19E3779F9ull, P64_4 = 0x85EBCA77C2B2AE63ull,
                   P64_5 = 0x27D4EB2F165667C5ull;
constexpr uint64_t PRIME_MX1 = 0x165667919E3779F9ull, PRIME_MX2 = 0x9FB21C651E98DF25ull;

static inline uint64_t rd64(const uint8_t* p) {
  uint64_t v = 0;
  for (int k = 7; k >= 0; --k) v = (v << 8) | p[k];
  return v;
}
static inline uint32_t rd32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
static inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
static inline uint64_t bswap64(uint64_t x) {
  uint64_t r = 0;
  for (int k = 0; k < 8; ++k) r = (r << 8) | ((x >> (8 * k)) & 0xFF);
  return r;
}
static inline uint32_t bswap32(uint32_t x) {
  return ((x & 0xFF) << 24) | ((x & 0xFF00) << 8) | ((x >> 8) & 0xFF00) | (x >> 24);
}
static inline uint64_t mul128_fold64(uint64_t a, uint64_t b) {
  const unsigned __int128 p = (unsigned __int128)a * b;
  return (uint64_t)p ^ (uint64_t)(p >> 64);
}
static inline uint64_t xxh64_avalanche(uint64_t h) {
  h ^= h >> 33;
  h *= P64_2;
  h ^= h >> 29;
  h *= P64_3;
  h ^= h >> 32;
  return h;
}
static inline uint64_t xxh3_avalanche(uint64_t h) {
  h ^= h >> 37;
  h *= PRIME_MX1;
  h ^= h >> 32;
  return h;
}
static inline uint64_t rrmxmx(uint64_t h, uint64_t len) {
  h ^= rotl64(h, 49) ^ rotl64(h, 24);
  h *= PRIME_MX2;
  h ^= (h >> 35) + len;
  h *= PRIME_MX2;
  h ^= h >> 28;
  return h;
}
static inline uint64_t mix16(const uint8_t* in, const uint8_t* sec, uint64_t seed) {
  return mul128_fold64(rd64(in) ^ (rd64(sec) + seed), rd64(in + 8) ^ (rd64(sec + 8) - seed));
}

static uint64_t hash(const uint8_t* in, uint64_t len, uint64_t seed, bool* ok) {
  const uint8_t* s = kSecret;
  *ok = true;
  if (len == 0) return xxh64_avalanche(seed ^ (rd64(s + 56) ^ rd64(s + 64)));
  if (len <= 3) {
    const uint32_t c1 = in[0], c2 = in[len >> 1], c3 = in[len - 1];
    const uint32_t combined = (c1 << 16) | (c2 << 24) | (c3 << 0) | ((uint32_t)len << 8);
    const uint64_t bitflip = (rd32(s) ^ rd32(s + 4)) + seed;
    return xxh64_avalanche((uint64_t)combined ^ bitflip);
  }
  if (len <= 8) {
    seed ^= (uint64_t)bswap32((uint32_t)seed) << 32;
    const uint32_t in1 = rd32(in), in2 = rd32(in + len - 4);
    const uint64_t bitflip = (rd64(s + 8) ^ rd64(s + 16)) - seed;
    const uint64_t in64 = in2 + ((uint64_t)in1 << 32);
    return rrmxmx(in64 ^ bitflip, len);
  }
  if (len <= 16) {
    const uint64_t bf1 = (rd64(s + 24) ^ rd64(s + 32)) + seed;
    const uint64_t bf2 = (rd64(s + 40) ^ rd64(s + 48)) - seed;
    const uint64_t lo = rd64(in) ^ bf1;
    const uint64_t hi = rd64(in + len - 8) ^ bf2;
    const uint64_t acc = len + bswap64(lo) + hi + mul128_fold64(lo, hi);
    return xxh3_avalanche(acc);
  }
  if (len <= 128) {
    uint64_t acc = len * P64_1;
    if (len > 32) {
      if (len > 64) {
        if (len > 96) {
          acc += mix16(in + 48, s + 96, seed);
          acc += mix16(in + len - 64, s + 112, seed);
        }
        acc += mix16(in + 32, s + 64, seed);
        acc += mix16(in + len - 48, s + 80, seed);
      }
      acc += mix16(in + 16, s + 32, seed);
      acc += mix16(in + len - 32, s + 48, seed);
    }
    acc += mix16(in + 0, s + 0, seed);
    acc += mix16(in + len - 16, s + 16, seed);
    return xxh3_avalanche(acc);
  }
  if (len <= 240) {
    uint64_t acc = len * P64_1;
    const int nb_rounds = (int)len / 16;
    for (int i = 0; i < 8; ++i) acc += mix16(in + 16 * i, s + 16 * i, seed);
    acc = xxh3_avalanche(acc);
    for (int i = 8; i < nb_rounds; ++i) acc += mix16(in + 16 * i, s + 16 * (i - 8) + 3, seed);
    acc += mix16(in + len - 16, s + 136 - 17, seed);
    return xxh3_avalanche(acc);
  }
  *ok = false;
  return 0;
}
}  // namespace xxh

extern "C" uint64_t mgpu_xxh3_64(const void* data, uint64_t len, uint64_t seed) {
  bool ok = true;
  const uint64_t h = xxh::hash((const uint8_t*)data, len, seed, &ok);
  if (!ok) fail(MGPU_ERR_UNSUPPORTED, "mgpu_xxh3_64: inputs longer than 240 bytes are not supported");
  return h;
}

extern "C" uint64_t mgpu_cell_seed(const char* name, uint64_t name_len, uint64_t chrom_size,
                                   uint64_t seed, uint64_t cell_id) {
  std::vector<uint8_t> buf(name_len + 16);
  if (name_len) std::memcpy(buf.data(), name, name_len);
  for (int k = 0; k < 8; ++k) buf[name_len + k] = (uint8_t)(chrom_size >> (8 * k));
  for (int k = 0; k < 8; ++k) buf[name_len + 8 + k] = (uint8_t)(cell_id >> (8 * k));
  return mgpu_xxh3_64(buf.data(), buf.size(), seed);
}

// ===========================================================================================
// Exact integer thresholds for the random tests of the epoch loop
// ===========================================================================================
static const double TWO64 = 18446744073709551616.0;

// bernoulli_distribution: true iff (double)u <= p * 2^64, i.e. iff u <= max{u : (double)u <= P}.
static Trial bernoulli_trial(double p) {
  Trial t{0, 0, 0};
  if (p == 0.0) return t;  // no draw
  t.draws = 1;
  const double P = p * TWO64;
  if ((double)UINT64_MAX <= P) {
    t.thr = UINT64_MAX;
    return t;
  }
  uint64_t lo = 0, hi = UINT64_MAX;  // (double)lo <= P < (double)hi
  if (!((double)lo <= P)) {          // p < 0 or NaN: never true (still one draw)
    t.thr = 0;
    t.draws = 1;
    return t;
  }
  while (hi - lo > 1) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if ((double)mid <= P) lo = mid; else hi = mid;
  }
  t.thr = lo;
  return t;
}

// generate_canonical<double, 53> of one draw (Boost): (double)u / 2^64, 1.0 mapped to 1 - eps/2.
static double canonical_of(uint64_t u) {
  double r = (double)u / TWO64;
  if (r == 1.0) r -= DBL_EPSILON / 2;
  return r;
}

// smallest u with canonical_of(u) > s; false when no draw satisfies it.
static bool min_draw_above(double s, uint64_t* out) {
  if (!(canonical_of(UINT64_MAX) > s)) return false;
  if (canonical_of(0) > s) {
    *out = 0;
    return true;
  }
  uint64_t lo = 0, hi = UINT64_MAX;
  while (hi - lo > 1) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (canonical_of(mid) > s) hi = mid; else lo = mid;
  }
  *out = hi;
  return true;
}

static DevBarrier make_dev_barrier(const mgpu_barrier& b) {
  DevBarrier d{};
  d.pos = (u32)b.pos;
  d.flags = b.blocking_dir & BF_DIR_MASK;
  const Trial occ = bernoulli_trial(occupancy_from_stp(b.stp_active, b.stp_inactive));
  if (occ.draws) d.flags |= BF_OCC_DRAWS;
  d.t_occ = occ.thr;
  if (!min_draw_above(b.stp_inactive, &d.t_ina)) d.flags |= BF_INA_NEVER;
  if (!min_draw_above(b.stp_active, &d.t_act)) d.flags |= BF_ACT_NEVER;
  return d;
}

// ===========================================================================================
// Jump table of the per-lane PRNG: T^JUMP_DISTANCE on the 256-bit state, 4-bit chunks.
// ===========================================================================================
static void xo_linear_step(uint64_t* s) {
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = (s[3] << 45) | (s[3] >> 19);
}

static std::vector<uint64_t> build_jump_table() {
  std::vector<uint64_t> col(256 * 4);
  for (int b = 0; b < 256; ++b) {
    uint64_t s[4] = {0, 0, 0, 0};
    s[b / 64] = 1ull << (b % 64);
    for (int k = 0; k < JUMP_DISTANCE; ++k) xo_linear_step(s);
    for (int w = 0; w < 4; ++w) col[b * 4 + w] = s[w];
  }
  std::vector<uint64_t> table(JUMP_TABLE_ENTRIES * 4, 0);
  for (int c = 0; c < 64; ++c) {
    for (int v = 0; v < 16; ++v) {
      uint64_t* e = &table[(c * 16 + v) * 4];
      for (int bit = 0; bit < 4; ++bit) {
        if (!((v >> bit) & 1)) continue;
        const int b = 4 * c + bit;
        for (int w = 0; w < 4; ++w) e[w] ^= col[b * 4 + w];
      }
    }
  }
  return table;
}

extern "C" void mgpu_prng_seed(uint64_t seed, uint64_t state[4]) {
  uint64_t st = seed;
  for (int k = 0; k < 4; ++k) {
    uint64_t z = (st += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    state[k] = z ^ (z >> 31);
  }
}

static inline uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ull;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebull;
  z ^= z >> 31;
  return z;
}

extern "C" uint64_t mgpu_state_digest(uint64_t n, const uint64_t* rev, const uint64_t* fwd,
                                      const uint64_t* ep, const uint64_t* rr, const uint64_t* fr,
                                      const uint64_t* rm, const uint64_t* fm, const uint64_t* rc,
                                      const uint64_t* fc) {
  uint64_t d = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t v[9] = {rev[i], fwd[i], ep[i], rr[i], fr[i], rm[i], fm[i], rc[i], fc[i]};
    uint64_t h = mix64(i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull);
    for (int k = 0; k < 9; ++k) h = mix64(h ^ v[k]);
    d += h;
  }
  return d;
}

// ===========================================================================================
// Context
// ===========================================================================================
struct ChromEntry {
  mgpu_chrom chrom{};
  uint64_t ws = 0, we = 0;  // simulated window (the whole range unless uploaded as a window)
  bool own_cfg = false;     // cfg overrides the context's configuration
  mgpu_config cfg{};
  std::string name;
  DevBarrier* d_bars = nullptr;
  uint2* d_pos_flags = nullptr;  // inside the d_bars allocation
  u32 nb = 0;
};

struct mgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // the context's own stream
  cudaStream_t user_stream = nullptr;  // caller's stream set by mgpu_set_stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_kernel_ms = 0.0;
  mgpu_config cfg{};
  void* d_jump = nullptr;
  u32* d_work = nullptr;
  std::vector<ChromEntry> chroms;
  std::mutex mu;
  u64 smem_limit = 0;
  u64 smem_budget = 0;     // per-cell shared memory the layout planner may use (0 = limit)
  uint32_t debug_flags = 0;
  char* d_scratch = nullptr;  // per-cell global slots for arrays that do not fit on chip
  u64 scratch_bytes = 0;
  uint64_t* d_prof = nullptr;  // profile counters of the last launch
  uint64_t h_prof[32] = {0};
  void* noalloc_scratch = nullptr;  // device address of the fixed scratch, looked up by this context
  std::vector<mgpu_launch_setting> launch_table;  // tuned settings of large batched launches
};

extern "C" const char* mgpu_last_error_string(void) { return g_last_error.c_str(); }
extern "C" int mgpu_abi_version(void) { return MGPU_ABI_VERSION; }

static int validate_config(const mgpu_config* c) {
  if (c->bin_size == 0) return fail(MGPU_ERR_INVALID_ARG, "bin_size must be positive");
  if (c->contact_sampling_interval == 0) return fail(MGPU_ERR_INVALID_ARG, "contact_sampling_interval must be positive");
  if (c->burnin_target_epochs_for_lef_activation == 0)
    return fail(MGPU_ERR_INVALID_ARG, "burnin_target_epochs_for_lef_activation must be positive");
  if (c->burnin_history_length == 0 || c->burnin_smoothing_window_size >= c->burnin_history_length)
    return fail(MGPU_ERR_INVALID_ARG, "burn-in history must be longer than its smoothing window");
  if (c->burnin_history_length > 100000) return fail(MGPU_ERR_UNSUPPORTED, "burn-in history longer than 100000");
  if (!(c->rev_extrusion_speed_std >= 0) || !(c->fwd_extrusion_speed_std >= 0))
    return fail(MGPU_ERR_INVALID_ARG, "extrusion speed std must be non-negative");
  if (!(c->genextreme_sigma > 0)) return fail(MGPU_ERR_INVALID_ARG, "genextreme_sigma must be positive");
  return MGPU_OK;
}

extern "C" int mgpu_create(int device, const mgpu_config* cfg, mgpu_ctx** out) {
  if (!cfg || !out) return fail(MGPU_ERR_INVALID_ARG, "mgpu_create: null argument");
  *out = nullptr;
  int rc = validate_config(cfg);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(MGPU_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= ndev) return fail(MGPU_ERR_INVALID_ARG, "device %d out of range", device);
  CK(cudaSetDevice(device));
  auto* ctx = new mgpu_ctx();
  ctx->device = device;
  ctx->cfg = *cfg;
  rc = cuda_check(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  const std::vector<uint64_t> jt = build_jump_table();
  if (!rc) rc = cuda_check(cudaMalloc(&ctx->d_jump, jt.size() * 8), "cudaMalloc(jump table)");
  if (!rc) rc = cuda_check(cudaMemcpy(ctx->d_jump, jt.data(), jt.size() * 8, cudaMemcpyHostToDevice), "copy jump table");
  if (!rc) rc = cuda_check(cudaMalloc(&ctx->d_work, sizeof(u32)), "cudaMalloc(work counter)");
  if (!rc) rc = cuda_check(cudaMalloc(&ctx->d_prof, 32 * sizeof(uint64_t)), "cudaMalloc(profile)");
  if (!rc) rc = cuda_check(cudaEventCreate(&ctx->ev0), "cudaEventCreate");
  if (!rc) rc = cuda_check(cudaEventCreate(&ctx->ev1), "cudaEventCreate");
  if (rc) {
    mgpu_destroy(ctx);
    return rc;
  }
  ctx->smem_limit = max_smem_per_block();
  *out = ctx;
  return MGPU_OK;
}

extern "C" int mgpu_destroy(mgpu_ctx* ctx) {
  if (!ctx) return MGPU_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& c : ctx->chroms) cudaFree(c.d_bars);
  cudaFree(ctx->d_jump);
  cudaFree(ctx->d_work);
  cudaFree(ctx->d_scratch);
  cudaFree(ctx->d_prof);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MGPU_OK;
}

extern "C" int mgpu_sync(mgpu_ctx* ctx) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_sync: null context");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->user_stream) CK(cudaStreamSynchronize(ctx->user_stream));
  return MGPU_OK;
}

extern "C" int mgpu_set_stream(mgpu_ctx* ctx, void* cuda_stream) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_set_stream: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->user_stream = (cudaStream_t)cuda_stream;
  return MGPU_OK;
}

extern "C" int mgpu_last_kernel_ms(mgpu_ctx* ctx, double* ms) {
  if (!ctx || !ms) return fail(MGPU_ERR_INVALID_ARG, "mgpu_last_kernel_ms: null argument");
  *ms = ctx->last_kernel_ms;
  return MGPU_OK;
}

static cudaStream_t active_stream(const mgpu_ctx* ctx) {
  return ctx->user_stream ? ctx->user_stream : ctx->stream;
}

extern "C" int mgpu_upload_chrom(mgpu_ctx* ctx, const mgpu_chrom* chrom, const mgpu_barrier* barriers,
                                 uint64_t nb, int* chrom_id) {
  if (!ctx || !chrom || !chrom_id || (nb && !barriers))
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_upload_chrom: null argument");
  if (chrom->end <= chrom->start || chrom->end - chrom->start < 3)
    return fail(MGPU_ERR_INVALID_ARG, "chromosome range must span at least 3 bp");
  if (chrom->end >= 0xFFFFFFFFull) return fail(MGPU_ERR_UNSUPPORTED, "chromosome end beyond 2^32 - 2");
  if (nb >= (1ull << 27)) return fail(MGPU_ERR_UNSUPPORTED, "too many barriers");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  // State::operator= builds ExtrusionBarriers{first, last} with sort = true (simulation.cpp:860)
  std::vector<mgpu_barrier> sorted(barriers, barriers + nb);
  int rc = mgpu_sort_barriers(sorted.data(), nb);
  if (rc) return rc;
  std::vector<DevBarrier> dev(nb);
  for (uint64_t i = 0; i < nb; ++i) {
    if (sorted[i].blocking_dir != MGPU_DIR_REV && sorted[i].blocking_dir != MGPU_DIR_FWD)
      return fail(MGPU_ERR_INVALID_ARG, "barrier %llu: blocking_dir must be REV or FWD", (unsigned long long)i);
    dev[i] = make_dev_barrier(sorted[i]);
  }
  ChromEntry e;
  e.name.assign(chrom->name ? chrom->name : "", chrom->name ? chrom->name_len : 0);
  e.chrom = *chrom;
  e.ws = chrom->start;
  e.we = chrom->end;
  e.nb = (u32)nb;
  if (nb) {
    // one allocation: the DevBarrier records, then the compact {pos, flags} pairs
    std::vector<uint2> pf(nb);
    for (uint64_t i = 0; i < nb; ++i) pf[i] = make_uint2(dev[i].pos, dev[i].flags);
    const size_t rec_bytes = (nb * sizeof(DevBarrier) + 15) & ~size_t(15);
    CK(cudaMalloc(&e.d_bars, rec_bytes + nb * sizeof(uint2)));
    CK(cudaMemcpy(e.d_bars, dev.data(), nb * sizeof(DevBarrier), cudaMemcpyHostToDevice));
    e.d_pos_flags = reinterpret_cast<uint2*>(reinterpret_cast<char*>(e.d_bars) + rec_bytes);
    CK(cudaMemcpy(e.d_pos_flags, pf.data(), nb * sizeof(uint2), cudaMemcpyHostToDevice));
  }
  ctx->chroms.push_back(e);
  *chrom_id = (int)ctx->chroms.size() - 1;
  return MGPU_OK;
}

extern "C" int mgpu_upload_window(mgpu_ctx* ctx, const mgpu_chrom* chrom, uint64_t window_start,
                                  uint64_t window_end, const mgpu_barrier* barriers, uint64_t nb,
                                  int* chrom_id) {
  if (!ctx || !chrom || !chrom_id) return fail(MGPU_ERR_INVALID_ARG, "mgpu_upload_window: null argument");
  if (window_start < chrom->start || window_end > chrom->end || window_end <= window_start ||
      window_end - window_start < 3)
    return fail(MGPU_ERR_INVALID_ARG, "window [%llu, %llu) must span at least 3 bp inside [%llu, %llu)",
                (unsigned long long)window_start, (unsigned long long)window_end,
                (unsigned long long)chrom->start, (unsigned long long)chrom->end);
  const int rc = mgpu_upload_chrom(ctx, chrom, barriers, nb, chrom_id);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->chroms[*chrom_id].ws = window_start;
  ctx->chroms[*chrom_id].we = window_end;
  return MGPU_OK;
}

extern "C" int mgpu_set_chrom_config(mgpu_ctx* ctx, int chrom_id, const mgpu_config* cfg) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_set_chrom_config: null context");
  if (cfg) {
    const int rc = validate_config(cfg);
    if (rc) return rc;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (chrom_id < 0 || chrom_id >= (int)ctx->chroms.size())
    return fail(MGPU_ERR_INVALID_ARG, "unknown chromosome handle %d", chrom_id);
  ChromEntry& e = ctx->chroms[chrom_id];
  e.own_cfg = cfg != nullptr;
  if (cfg) e.cfg = *cfg;
  return MGPU_OK;
}

static int make_kparams(const mgpu_ctx* ctx, const ChromEntry& ch, uint64_t nlefs, KParams* P,
                        uint64_t budget_override = 0) {
  const mgpu_config& c = ch.own_cfg ? ch.cfg : ctx->cfg;
  std::memset(P, 0, sizeof(*P));
  if (nlefs == 0) return fail(MGPU_ERR_INVALID_ARG, "num_lefs must be positive");
  if (nlefs >= (1ull << 27)) return fail(MGPU_ERR_UNSUPPORTED, "too many LEFs");
  P->start = (u32)ch.chrom.start;
  P->end = (u32)ch.chrom.end;
  P->wstart = (u32)ch.ws;
  P->wend = (u32)ch.we;
  const uint64_t len = ch.we - ch.ws;
  uint64_t nrows, ncols;
  mgpu_band_shape(&c, len, &nrows, &ncols);
  P->bin = (u32)c.bin_size;
  P->nrows = (u32)nrows;
  P->ncols = (u32)ncols;
  P->nlefs = (u32)nlefs;
  P->nbarriers = ch.nb;
  P->hist_cap = (u32)c.burnin_history_length;
  P->smooth_w = (u32)c.burnin_smoothing_window_size;
  P->skip_burnin = c.skip_burnin ? 1 : 0;
  P->min_burnin = c.min_burnin_epochs;
  P->max_burnin = c.max_burnin_epochs;
  P->rev_speed[0] = (double)c.rev_extrusion_speed_burnin;
  P->rev_speed[1] = (double)c.rev_extrusion_speed;
  P->fwd_speed[0] = (double)c.fwd_extrusion_speed_burnin;
  P->fwd_speed[1] = (double)c.fwd_extrusion_speed;
  P->rev_std = c.rev_extrusion_speed_std;
  P->fwd_std = c.fwd_extrusion_speed_std;
  for (int k = 0; k < 2; ++k) {
    P->rev_move_int[k] = (uint64_t)std::round(P->rev_speed[k]);
    P->fwd_move_int[k] = (uint64_t)std::round(P->fwd_speed[k]);
  }
  const double aff[3] = {1.0, 1.0 / c.soft_stall_lef_stability_multiplier,
                         1.0 / c.hard_stall_lef_stability_multiplier};
  for (int nh = 0; nh < 3; ++nh) {
    P->release[0][nh] = bernoulli_trial(aff[nh] * c.prob_of_lef_release_burnin);
    P->release[1][nh] = bernoulli_trial(aff[nh] * c.prob_of_lef_release);
  }
  if (c.probability_of_extrusion_unit_bypass == 0.0) {
    P->lef_lef = Trial{0, 0, 1};
  } else {
    P->lef_lef = bernoulli_trial(1.0 - c.probability_of_extrusion_unit_bypass);
  }
  const double pb[2] = {c.lef_bar_major_collision_pblock, c.lef_bar_minor_collision_pblock};
  for (int k = 0; k < 2; ++k) P->lef_bar[k] = pb[k] == 1.0 ? Trial{0, 0, 1} : bernoulli_trial(pb[k]);
  // Poisson(nlefs / burnin_target_epochs), Boost constants (poisson_distribution::init)
  const double mean = (double)nlefs / (double)c.burnin_target_epochs_for_lef_activation;
  P->pois_mean = mean;
  P->pois_exp_mean = std::exp(-mean);
  P->pois_smu = std::sqrt(mean);
  P->pois_b = 0.931 + 2.53 * P->pois_smu;
  P->pois_a = -0.059 + 0.02483 * P->pois_b;
  P->pois_inv_alpha = 1.1239 + 1.1328 / (P->pois_b - 3.4);
  P->pois_v_r = 0.9277 - 3.6224 / (P->pois_b - 2);
  // contacts
  P->spe = mgpu_contacts_per_epoch(&c, nlefs);
  P->contact_mode = c.target_contact_density >= 0 ? 1 : 0;
  P->density_positive = c.target_contact_density > 0.0 ? 1 : 0;
  const double ratio = c.tad_to_loop_contact_ratio;
  P->ratio_mode = ratio == 0 ? 0 : (!std::isfinite(ratio) ? 1 : 2);
  P->p_loop = 1.0 / (ratio + 1.0);
  P->noisify = (c.contact_sampling_strategy & MGPU_CS_NOISIFY) ? 1 : 0;
  P->gev_mu = c.genextreme_mu;
  P->gev_sigma = c.genextreme_sigma;
  P->gev_xi = c.genextreme_xi;
  {
    const double p = (0.5 < P->p_loop) ? (1 - P->p_loop) : P->p_loop;
    P->bin_q_n = std::pow((1 - p), (double)(int64_t)P->spe);
  }
  const uint64_t range = (uint64_t)P->wend - 1 - P->wstart;  // bind positions: uniform_int[ws, we - 1]
  uint64_t bucket = UINT64_MAX / (range + 1);
  if (UINT64_MAX % (range + 1) == range) ++bucket;
  P->pos_bucket = bucket;
  P->pos_range = range;
  P->debug_flags = ctx->debug_flags;
  P->track_occ = c.track_1d_lef_position ? 1u : 0u;
  P->log_state = c.log_model_internal_state ? 1u : 0u;
  P->occ_bins = (ch.chrom.size + c.bin_size - 1) / c.bin_size;
  // Layout: the header (scalars, PRNG ring, burn-in history, barrier bits) is always on chip;
  // per-LEF arrays go on chip in priority order while they fit, the rest into a global slot.
  const u64 header = cell_header_bytes(ch.nb, P->hist_cap);
  const u64 budget = budget_override ? budget_override : ctx->smem_budget;
  const u64 limit = std::min<u64>(ctx->smem_limit, budget ? budget : ctx->smem_limit);
  if (header > limit)
    return fail(MGPU_ERR_UNSUPPORTED, "%u barriers need %llu B of shared memory (limit %llu)", ch.nb,
                (unsigned long long)header, (unsigned long long)limit);
  const u64 arr_bytes = ((u64)nlefs * 4 + 15) & ~15ull;
  u64 smem_used = header, slot_used = 0;
  P->arr_smem = 0;
  const int groups[][2] = {{ARR_REV, -1}, {ARR_FWD, -1}, {ARR_RR, -1}, {ARR_FR, -1}, {ARR_RM, -1},
                           {ARR_FM, -1},  {ARR_RC, -1},  {ARR_FC, -1}, {ARR_SR, ARR_SF}, {ARR_TMP, -1},
                           {ARR_BEP, -1}};
  for (const auto& g : groups) {
    const u64 bytes = g[1] < 0 ? arr_bytes : (((u64)nlefs * 8 + 15) & ~15ull);
    const bool on_chip = smem_used + bytes <= limit;
    u64& used = on_chip ? smem_used : slot_used;
    P->arr_off[g[0]] = (u32)used;
    if (g[1] >= 0) P->arr_off[g[1]] = (u32)(used + (u64)nlefs * 4);  // SF right after SR
    if (on_chip) {
      P->arr_smem |= 1u << g[0];
      if (g[1] >= 0) P->arr_smem |= 1u << g[1];
    }
    used += bytes;
  }
  P->smem_bytes = (u32)smem_used;
  P->slot_bytes = slot_used;
  return MGPU_OK;
}

// Make sure the context's global scratch holds `cells` slots of the plan's size.
static int ensure_scratch(mgpu_ctx* ctx, const KParams& P, u64 cells) {
  const u64 need = P.slot_bytes * cells;
  if (need <= ctx->scratch_bytes) return MGPU_OK;
  // stream-ordered: the old slots are released after the launches already issued on the stream
  cudaStream_t st = ctx->user_stream ? ctx->user_stream : ctx->stream;
  if (ctx->d_scratch) CK(cudaFreeAsync(ctx->d_scratch, st));
  ctx->d_scratch = nullptr;
  ctx->scratch_bytes = 0;
  CK(cudaMallocAsync((void**)&ctx->d_scratch, need, st));
  ctx->scratch_bytes = need;
  return MGPU_OK;
}

extern "C" int mgpu_last_profile(mgpu_ctx* ctx, uint64_t counters[32]) {
  if (!ctx || !counters) return fail(MGPU_ERR_INVALID_ARG, "mgpu_last_profile: null argument");
  std::memcpy(counters, ctx->h_prof, sizeof(ctx->h_prof));
  return MGPU_OK;
}

extern "C" int mgpu_set_launch_table(mgpu_ctx* ctx, const mgpu_launch_setting* table, uint64_t n) {
  if (!ctx || (n && !table)) return fail(MGPU_ERR_INVALID_ARG, "mgpu_set_launch_table: null argument");
  std::vector<mgpu_launch_setting> t(table, table + n);
  for (uint64_t i = 0; i < n; ++i) {
    if (t[i].carveout_pct > 100 || t[i].max_cells_per_sm > 255)
      return fail(MGPU_ERR_INVALID_ARG, "mgpu_set_launch_table: entry %llu: carveout above 100 %% or cap above 255",
                  (unsigned long long)i);
    if (i && t[i].max_lefs <= t[i - 1].max_lefs)
      return fail(MGPU_ERR_INVALID_ARG, "mgpu_set_launch_table: max_lefs must increase");
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->launch_table = std::move(t);
  return MGPU_OK;
}

extern "C" int mgpu_set_debug_flags(mgpu_ctx* ctx, uint32_t flags, uint64_t smem_budget) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_set_debug_flags: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->debug_flags = flags;
  ctx->smem_budget = smem_budget;
  return MGPU_OK;
}

static bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device memory that a kernel on `device` may touch: managed memory, or device memory owned by
// that device.  Memory of another GPU is refused (its kernels would need peer access).
static bool is_device_ptr_on(const void* p, int device) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

// Device buffer (RAII).  Buffers allocated with a stream are stream-ordered
// (cudaMallocAsync / cudaFreeAsync), so a call never synchronises the whole device and calls
// of independent contexts overlap.
struct DevBuf {
  void* p = nullptr;
  bool owned = false;
  cudaStream_t st = nullptr;
  bool ordered = false;
  ~DevBuf() {
    if (!owned) return;
    if (ordered) {
      cudaFreeAsync(p, st);
    } else {
      cudaFree(p);
    }
  }
};

static int alloc_on_stream(DevBuf& d, size_t bytes, cudaStream_t st) {
  CK(cudaMallocAsync(&d.p, bytes, st));
  d.owned = true;
  d.ordered = true;
  d.st = st;
  return MGPU_OK;
}

static int to_device(const void* src, size_t bytes, DevBuf& d, cudaStream_t st, bool copy) {
  if (!src || bytes == 0) return MGPU_OK;
  if (is_device_ptr(src)) {
    d.p = const_cast<void*>(src);
    return MGPU_OK;
  }
  int rc = alloc_on_stream(d, bytes, st);
  if (rc) return rc;
  if (copy) CK(cudaMemcpyAsync(d.p, src, bytes, cudaMemcpyHostToDevice, st));
  return MGPU_OK;
}

static int status_from_stats(const mgpu_cell_stats* st, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    switch (st[i].status) {
      case DEV_OK:
        break;
      case DEV_ERR_ITER_LIMIT:
        return fail(MGPU_ERR_TIMEOUT, "cell %llu: a device loop hit its iteration limit", (unsigned long long)i);
      case DEV_ERR_MOVE_RANGE:
        return fail(MGPU_ERR_OVERFLOW, "cell %llu: a move exceeded 2^32 - 1 bp", (unsigned long long)i);
      case DEV_ERR_BAD_STATE:
        return fail(MGPU_ERR_INTERNAL, "cell %llu: the reference would read out of bounds", (unsigned long long)i);
      case DEV_ERR_NO_BOUND_LEF:
        return fail(MGPU_ERR_TIMEOUT, "cell %llu: no LEF could register a contact", (unsigned long long)i);
      default:
        return fail(MGPU_ERR_INTERNAL, "cell %llu: device status %llu", (unsigned long long)i,
                    (unsigned long long)st[i].status);
    }
  }
  return MGPU_OK;
}

static int run_cells(mgpu_ctx* ctx, int chrom_id, const uint64_t* seeds, const uint64_t* targets,
                     uint64_t target_epochs, uint64_t nlefs, uint64_t ncells, uint32_t* band,
                     uint64_t* missed, mgpu_cell_stats* stats, const DevTrace* trace,
                     const mgpu_extra_outputs* extra = nullptr) {
  if (chrom_id < 0 || chrom_id >= (int)ctx->chroms.size())
    return fail(MGPU_ERR_INVALID_ARG, "unknown chromosome handle %d", chrom_id);
  if (ncells == 0) return MGPU_OK;
  if (!seeds || !targets) return fail(MGPU_ERR_INVALID_ARG, "cell seeds and targets are required");
  const ChromEntry& ch = ctx->chroms[chrom_id];
  KParams P;
  int rc = make_kparams(ctx, ch, nlefs, &P);
  if (rc) return rc;
  cudaStream_t st = active_stream(ctx);
  // tasks
  std::vector<CellTask> tasks(ncells);
  std::vector<uint64_t> hs(ncells), ht(ncells);
  const bool seeds_dev = is_device_ptr(seeds), targets_dev = is_device_ptr(targets);
  if (seeds_dev) CK(cudaMemcpyAsync(hs.data(), seeds, ncells * 8, cudaMemcpyDeviceToHost, st));
  if (targets_dev) CK(cudaMemcpyAsync(ht.data(), targets, ncells * 8, cudaMemcpyDeviceToHost, st));
  if (seeds_dev || targets_dev) CK(cudaStreamSynchronize(st));
  for (uint64_t i = 0; i < ncells; ++i) {
    tasks[i].seed = seeds_dev ? hs[i] : seeds[i];
    tasks[i].target_contacts = targets_dev ? ht[i] : targets[i];
  }
  DevBuf d_tasks;
  rc = alloc_on_stream(d_tasks, ncells * sizeof(CellTask), st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(d_tasks.p, tasks.data(), ncells * sizeof(CellTask), cudaMemcpyHostToDevice, st));
  const size_t band_bytes = (size_t)P.nrows * P.ncols * sizeof(uint32_t);
  DevBuf d_band, d_missed, d_stats;
  rc = to_device(band, band_bytes, d_band, st, true);
  if (rc) return rc;
  rc = alloc_on_stream(d_missed, 8, st);
  if (rc) return rc;
  CK(cudaMemsetAsync(d_missed.p, 0, 8, st));
  rc = alloc_on_stream(d_stats, ncells * sizeof(mgpu_cell_stats), st);
  if (rc) return rc;
  char err[256] = {0};
  DevChrom dc{ch.d_bars, ch.d_pos_flags, ch.nb};
  if (P.slot_bytes) {
    rc = ensure_scratch(ctx, P, resident_cells(P, ncells));
    if (rc) return rc;
  }
  // optional outputs: occupancy counters are added to; records land where the caller wants them
  DevBuf d_occ, d_rec, d_recn;
  if (extra && extra->lef_1d_occupancy && P.track_occ) {
    rc = to_device(extra->lef_1d_occupancy, P.occ_bins * sizeof(uint64_t), d_occ, st, true);
    if (rc) return rc;
    P.occ = (unsigned long long*)d_occ.p;
  }
  const uint64_t rec_max = extra ? extra->max_epoch_records : 0;
  if (extra && extra->epoch_records && rec_max && P.log_state) {
    if (ncells > UINT64_MAX / rec_max / sizeof(mgpu_epoch_record))
      return fail(MGPU_ERR_INVALID_ARG, "too many epoch records requested");
    rc = to_device(extra->epoch_records, ncells * rec_max * sizeof(mgpu_epoch_record), d_rec, st, false);
    if (rc) return rc;
    rc = alloc_on_stream(d_recn, ncells * sizeof(uint64_t), st);
    if (rc) return rc;
    CK(cudaMemsetAsync(d_recn.p, 0, ncells * sizeof(uint64_t), st));
    P.records = (mgpu_epoch_record*)d_rec.p;
    P.rec_max = rec_max;
    P.rec_count = (u64*)d_recn.p;
  }
  P.prof = (ctx->debug_flags & DBG_PROFILE) ? ctx->d_prof : nullptr;
  CK(cudaMemsetAsync(ctx->d_prof, 0, 32 * sizeof(uint64_t), st));
  CK(cudaEventRecord(ctx->ev0, st));
  rc = launch_simulate(P, dc, (const CellTask*)d_tasks.p, ncells, target_epochs, (u32*)d_band.p,
                       (u64*)d_missed.p, (mgpu_cell_stats*)d_stats.p, trace, ctx->d_jump,
                       ctx->d_work, ctx->d_scratch, ctx->scratch_bytes, st, err, sizeof(err));
  if (rc) return fail(rc, "%s", err);
  CK(cudaEventRecord(ctx->ev1, st));
  if (band && d_band.owned) CK(cudaMemcpyAsync(band, d_band.p, band_bytes, cudaMemcpyDeviceToHost, st));
  if (P.occ && d_occ.owned)
    CK(cudaMemcpyAsync(extra->lef_1d_occupancy, d_occ.p, P.occ_bins * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  if (P.records) {
    if (d_rec.owned)
      CK(cudaMemcpyAsync(extra->epoch_records, d_rec.p, ncells * rec_max * sizeof(mgpu_epoch_record),
                         cudaMemcpyDeviceToHost, st));
    if (extra->records_written)
      CK(cudaMemcpyAsync(extra->records_written, d_recn.p, ncells * sizeof(uint64_t), cudaMemcpyDefault, st));
  }
  uint64_t h_missed = 0;
  CK(cudaMemcpyAsync(&h_missed, d_missed.p, 8, cudaMemcpyDeviceToHost, st));
  std::vector<mgpu_cell_stats> h_stats(ncells);
  CK(cudaMemcpyAsync(h_stats.data(), d_stats.p, ncells * sizeof(mgpu_cell_stats), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(ctx->h_prof, ctx->d_prof, 32 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_kernel_ms = ms;
  }
  if (missed) {
    if (is_device_ptr(missed)) {
      uint64_t cur = 0;
      CK(cudaMemcpyAsync(&cur, missed, 8, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      cur += h_missed;
      CK(cudaMemcpyAsync(missed, &cur, 8, cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    } else {
      *missed += h_missed;
    }
  }
  if (stats) {
    if (is_device_ptr(stats)) {
      CK(cudaMemcpyAsync(stats, h_stats.data(), ncells * sizeof(mgpu_cell_stats), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    } else {
      std::memcpy(stats, h_stats.data(), ncells * sizeof(mgpu_cell_stats));
    }
  }
  return status_from_stats(h_stats.data(), ncells);
}

extern "C" int mgpu_simulate_cells(mgpu_ctx* ctx, int chrom_id, const uint64_t* cell_seeds,
                                   const uint64_t* target_contacts, uint64_t target_epochs,
                                   uint64_t num_lefs, uint64_t ncells, uint32_t* band,
                                   uint64_t* missed_updates, mgpu_cell_stats* stats) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_cells: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  return run_cells(ctx, chrom_id, cell_seeds, target_contacts, target_epochs, num_lefs, ncells,
                   band, missed_updates, stats, nullptr);
}

extern "C" int mgpu_simulate_batch(mgpu_ctx* ctx, const mgpu_batch_task* tasks, uint64_t ntasks,
                                   uint32_t* const* bands, uint64_t nbands, uint64_t* missed,
                                   mgpu_cell_stats* stats) {
  if (!ctx || (ntasks && !tasks)) return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_batch: null argument");
  if (ntasks == 0) return MGPU_OK;
  if (ntasks >= 0xFFFFFFFFull) return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_batch: too many tasks");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = active_stream(ctx);
  // plans: one per (chromosome, LEF count, target epochs)
  struct Key {
    int chrom;
    uint64_t nlefs, te;
    bool operator<(const Key& o) const {
      return chrom != o.chrom ? chrom < o.chrom : (nlefs != o.nlefs ? nlefs < o.nlefs : te < o.te);
    }
  };
  std::map<Key, u32> plan_of;
  std::vector<Key> keys;
  for (uint64_t i = 0; i < ntasks; ++i) {
    const mgpu_batch_task& t = tasks[i];
    if (t.chrom_id < 0 || t.chrom_id >= (int)ctx->chroms.size())
      return fail(MGPU_ERR_INVALID_ARG, "task %llu: unknown chromosome handle %d", (unsigned long long)i, t.chrom_id);
    if ((uint64_t)t.chrom_id >= nbands || !bands || !bands[t.chrom_id])
      return fail(MGPU_ERR_INVALID_ARG, "task %llu: no band for chromosome handle %d", (unsigned long long)i,
                  t.chrom_id);
    const Key k{t.chrom_id, t.num_lefs, t.target_epochs};
    if (!plan_of.count(k)) {
      plan_of[k] = (u32)keys.size();
      keys.push_back(k);
    }
  }
  int dev_sms = 0;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
  // Large batches: 16 KiB per cell and a 60 % shared-memory carveout, so that nine cells share
  // an SM and the per-LEF arrays that live in global slots keep an 88 KB L1 (measured best on the
  // genome workload).
  const bool large = ntasks >= 8ull * (uint64_t)dev_sms;
  uint64_t budget = ctx->smem_budget ? ctx->smem_budget : (large ? 16384ull : 0ull);
  // a tuned table (mgpu_set_launch_table) replaces those defaults for large batches without
  // explicit switches: the entry of the LEF-weighted median cell's LEF count
  const mgpu_launch_setting* tuned = nullptr;
  if (large && !ctx->smem_budget && !(ctx->debug_flags & 0xFFFF00u) && !ctx->launch_table.empty()) {
    std::vector<uint64_t> nl(ntasks);
    uint64_t total = 0;
    for (uint64_t i = 0; i < ntasks; ++i) total += (nl[i] = tasks[i].num_lefs);
    std::sort(nl.begin(), nl.end());
    uint64_t acc = 0, median = nl.back();
    for (uint64_t v : nl) {
      acc += v;
      if (2 * acc >= total) {
        median = v;
        break;
      }
    }
    tuned = &ctx->launch_table.back();
    for (const mgpu_launch_setting& e : ctx->launch_table) {
      if (median <= e.max_lefs) {
        tuned = &e;
        break;
      }
    }
    budget = tuned->smem_budget;
  }
  std::vector<BatchPlan> plans(keys.size());
  u32 smem_bytes = 0;
  u64 slot_bytes = 0;
  for (size_t p = 0; p < keys.size(); ++p) {
    const ChromEntry& ch = ctx->chroms[keys[p].chrom];
    int rc = make_kparams(ctx, ch, keys[p].nlefs, &plans[p].P, budget);
    if (rc) return rc;
    plans[p].ch = DevChrom{ch.d_bars, ch.d_pos_flags, ch.nb};
    plans[p].target_epochs = keys[p].te;
    smem_bytes = std::max(smem_bytes, plans[p].P.smem_bytes);
    slot_bytes = std::max<u64>(slot_bytes, plans[p].P.slot_bytes);
  }
  // bands of the chromosomes in use
  std::map<int, DevBuf> dband;
  for (const Key& k : keys) {
    if (dband.count(k.chrom)) continue;
    const KParams& P0 = plans[plan_of[k]].P;
    const size_t bytes = (size_t)P0.nrows * P0.ncols * sizeof(uint32_t);
    int rc = to_device(bands[k.chrom], bytes, dband[k.chrom], st, true);
    if (rc) return rc;
  }
  DevBuf d_missed;
  int rc = alloc_on_stream(d_missed, keys.size() * sizeof(uint64_t), st);
  if (rc) return rc;
  CK(cudaMemsetAsync(d_missed.p, 0, keys.size() * sizeof(uint64_t), st));
  for (size_t p = 0; p < keys.size(); ++p) {
    plans[p].band = (u32*)dband[keys[p].chrom].p;
    plans[p].missed = (unsigned long long*)d_missed.p + p;
    plans[p].P.prof = (ctx->debug_flags & DBG_PROFILE) ? ctx->d_prof : nullptr;
  }
  CK(cudaMemsetAsync(ctx->d_prof, 0, 32 * sizeof(uint64_t), st));
  // work queue: largest LEF count first, cells of one plan together
  std::vector<uint64_t> order(ntasks);
  for (uint64_t i = 0; i < ntasks; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) {
    const uint64_t na = tasks[a].num_lefs, nb = tasks[b].num_lefs;
    if (na != nb) return na > nb;
    return plan_of[Key{tasks[a].chrom_id, tasks[a].num_lefs, tasks[a].target_epochs}] <
           plan_of[Key{tasks[b].chrom_id, tasks[b].num_lefs, tasks[b].target_epochs}];
  });
  std::vector<BatchTask> bt(ntasks);
  for (uint64_t k = 0; k < ntasks; ++k) {
    const mgpu_batch_task& t = tasks[order[k]];
    bt[k] = BatchTask{t.seed, t.target_contacts, plan_of[Key{t.chrom_id, t.num_lefs, t.target_epochs}], 0};
  }
  DevBuf d_plans, d_tasks, d_stats;
  rc = alloc_on_stream(d_plans, plans.size() * sizeof(BatchPlan), st);
  if (!rc) rc = alloc_on_stream(d_tasks, ntasks * sizeof(BatchTask), st);
  if (!rc) rc = alloc_on_stream(d_stats, ntasks * sizeof(mgpu_cell_stats), st);
  if (rc) return rc;
  CK(cudaMemcpyAsync(d_plans.p, plans.data(), plans.size() * sizeof(BatchPlan), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d_tasks.p, bt.data(), ntasks * sizeof(BatchTask), cudaMemcpyHostToDevice, st));
  // tuning switches (mgpu_set_debug_flags bits 8-15: carveout percent, 16-23: blocks per SM cap)
  u32 carveout = (ctx->debug_flags >> 8) & 0xFFu;
  u32 max_per_sm = (ctx->debug_flags >> 16) & 0xFFu;
  if (!carveout && large && !ctx->smem_budget) carveout = 60;
  if (tuned) {
    carveout = tuned->carveout_pct;
    max_per_sm = tuned->max_cells_per_sm;
  }
  if (slot_bytes) {
    KParams Pslot = plans[0].P;
    Pslot.slot_bytes = slot_bytes;
    rc = ensure_scratch(ctx, Pslot, resident_batch_cells(smem_bytes, ntasks, carveout, max_per_sm));
    if (rc) return rc;
  }
  char err[256] = {0};
  CK(cudaEventRecord(ctx->ev0, st));
  rc = launch_simulate_batch((const BatchPlan*)d_plans.p, (const BatchTask*)d_tasks.p, ntasks, smem_bytes,
                             slot_bytes, (mgpu_cell_stats*)d_stats.p, ctx->d_jump, ctx->d_work, ctx->d_scratch,
                             ctx->scratch_bytes, carveout, max_per_sm, st, err, sizeof(err));
  if (rc) return fail(rc, "%s", err);
  CK(cudaEventRecord(ctx->ev1, st));
  for (auto& kv : dband) {
    if (kv.second.owned) {
      const KParams* P0 = nullptr;
      for (size_t p = 0; p < keys.size(); ++p)
        if (keys[p].chrom == kv.first) P0 = &plans[p].P;
      CK(cudaMemcpyAsync(bands[kv.first], kv.second.p, (size_t)P0->nrows * P0->ncols * sizeof(uint32_t),
                         cudaMemcpyDeviceToHost, st));
    }
  }
  std::vector<uint64_t> h_missed(keys.size());
  std::vector<mgpu_cell_stats> h_stats(ntasks);
  CK(cudaMemcpyAsync(h_missed.data(), d_missed.p, keys.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h_stats.data(), d_stats.p, ntasks * sizeof(mgpu_cell_stats), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(ctx->h_prof, ctx->d_prof, 32 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_kernel_ms = ms;
  }
  if (missed) {
    std::vector<uint64_t> add(nbands, 0);
    for (size_t p = 0; p < keys.size(); ++p) add[keys[p].chrom] += h_missed[p];
    if (is_device_ptr(missed)) {
      std::vector<uint64_t> cur(nbands);
      CK(cudaMemcpyAsync(cur.data(), missed, nbands * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (uint64_t c = 0; c < nbands; ++c) cur[c] += add[c];
      CK(cudaMemcpyAsync(missed, cur.data(), nbands * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    } else {
      for (uint64_t c = 0; c < nbands; ++c) missed[c] += add[c];
    }
  }
  std::vector<mgpu_cell_stats> out(ntasks);
  for (uint64_t k = 0; k < ntasks; ++k) out[order[k]] = h_stats[k];
  if (stats) {
    if (is_device_ptr(stats)) {
      CK(cudaMemcpyAsync(stats, out.data(), ntasks * sizeof(mgpu_cell_stats), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    } else {
      std::memcpy(stats, out.data(), ntasks * sizeof(mgpu_cell_stats));
    }
  }
  return status_from_stats(out.data(), ntasks);
}

// Copy a device result to the caller's buffer (host or device).
static int copy_out(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (!dst || bytes == 0 || dst == src) return MGPU_OK;
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st));
  return MGPU_OK;
}

extern "C" int mgpu_band_to_pixels(mgpu_ctx* ctx, const uint32_t* band, uint64_t nrows, uint64_t ncols,
                                   uint64_t bin_offset, uint64_t* bin1_offset, int64_t* bin1,
                                   int64_t* bin2, uint32_t* count, uint64_t capacity, uint64_t* nnz) {
  if (!ctx || !nnz || !bin1_offset || (ncols && nrows && !band))
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_band_to_pixels: null argument");
  const bool want_pixels = bin1 || bin2 || count;
  if (want_pixels && !(bin1 && bin2 && count))
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_band_to_pixels: bin1, bin2 and count go together");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = active_stream(ctx);
  const size_t band_bytes = (size_t)nrows * ncols * sizeof(uint32_t);
  DevBuf d_band, d_counts, d_off;
  int rc = to_device(band, band_bytes, d_band, st, true);
  if (rc) return rc;
  rc = alloc_on_stream(d_counts, (ncols ? ncols : 1) * sizeof(uint32_t), st);
  if (rc) return rc;
  rc = to_device(bin1_offset, (ncols + 1) * sizeof(uint64_t), d_off, st, false);
  if (rc) return rc;
  char err[256] = {0};
  rc = launch_band_counts((const u32*)d_band.p, nrows, ncols, (u32*)d_counts.p, (u64*)d_off.p, st, err,
                          sizeof(err));
  if (rc) return fail(rc, "%s", err);
  uint64_t total = 0;
  CK(cudaMemcpyAsync(&total, (u64*)d_off.p + ncols, sizeof(total), cudaMemcpyDeviceToHost, st));
  rc = copy_out(bin1_offset, d_off.p, (ncols + 1) * sizeof(uint64_t), st);
  if (rc) return rc;
  CK(cudaStreamSynchronize(st));
  *nnz = total;
  if (!want_pixels) return MGPU_OK;
  if (capacity < total)
    return fail(MGPU_ERR_OVERFLOW, "mgpu_band_to_pixels: capacity %llu < %llu non-zero pixels",
                (unsigned long long)capacity, (unsigned long long)total);
  DevBuf d_b1, d_b2, d_c;
  rc = to_device(bin1, total * sizeof(int64_t), d_b1, st, false);
  if (!rc) rc = to_device(bin2, total * sizeof(int64_t), d_b2, st, false);
  if (!rc) rc = to_device(count, total * sizeof(uint32_t), d_c, st, false);
  if (rc) return rc;
  if (total) {
    rc = launch_band_pixels((const u32*)d_band.p, nrows, ncols, bin_offset, (const u64*)d_off.p,
                            (int64_t*)d_b1.p, (int64_t*)d_b2.p, (u32*)d_c.p, st, err, sizeof(err));
    if (rc) return fail(rc, "%s", err);
    rc = copy_out(bin1, d_b1.p, total * sizeof(int64_t), st);
    if (!rc) rc = copy_out(bin2, d_b2.p, total * sizeof(int64_t), st);
    if (!rc) rc = copy_out(count, d_c.p, total * sizeof(uint32_t), st);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(st));
  return MGPU_OK;
}


extern "C" int mgpu_simulate_cells_noalloc(mgpu_ctx* ctx, int chrom_id, const uint64_t* cell_seeds,
                                           const uint64_t* target_contacts, uint64_t target_epochs,
                                           uint64_t num_lefs, uint64_t ncells, uint32_t* band,
                                           uint64_t* missed_updates, mgpu_cell_stats* stats) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_cells_noalloc: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  if (chrom_id < 0 || chrom_id >= (int)ctx->chroms.size())
    return fail(MGPU_ERR_INVALID_ARG, "unknown chromosome handle %d", chrom_id);
  if (ncells > MGPU_NOALLOC_MAX_CELLS)
    return fail(MGPU_ERR_INVALID_ARG,
                "mgpu_simulate_cells_noalloc: %llu cells requested, the fixed scratch holds at most %u "
                "(split the batch or use mgpu_simulate_cells)",
                (unsigned long long)ncells, MGPU_NOALLOC_MAX_CELLS);
  if (ncells == 0) return MGPU_OK;
  const void* need_dev[3] = {cell_seeds, target_contacts, band};
  const char* names[5] = {"cell_seeds", "target_contacts", "band", "missed_updates", "stats"};
  for (int k = 0; k < 3; ++k) {
    if (!is_device_ptr_on(need_dev[k], ctx->device))
      return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_cells_noalloc: %s must be a device pointer of device %d",
                  names[k], ctx->device);
  }
  if (missed_updates && !is_device_ptr_on(missed_updates, ctx->device))
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_cells_noalloc: %s must be a device pointer of device %d or NULL",
                names[3], ctx->device);
  if (stats && !is_device_ptr_on(stats, ctx->device))
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_cells_noalloc: %s must be a device pointer of device %d or NULL",
                names[4], ctx->device);
  const ChromEntry& ch = ctx->chroms[chrom_id];
  KParams P;
  int rc = make_kparams(ctx, ch, num_lefs, &P);
  if (rc) return rc;
  char err[256] = {0};
  // The array's address in the CUDA context current on ctx->device, looked up on this mgpu
  // context's first call and kept with the context (whose own device buffers belong to the same
  // CUDA context and die with it).
  if (!ctx->noalloc_scratch) {
    void* addr = nullptr;
    rc = noalloc_scratch_address(&addr, err, sizeof(err));
    if (rc) return fail(rc, "%s", err);
    ctx->noalloc_scratch = addr;
  }
  char* scratch = (char*)ctx->noalloc_scratch;
  const u64 slot_room = MGPU_NOALLOC_SCRATCH_BYTES - NOALLOC_SLOTS_OFFSET;
  if (P.slot_bytes > slot_room)
    return fail(MGPU_ERR_UNSUPPORTED,
                "mgpu_simulate_cells_noalloc: %llu LEFs need %llu B of global scratch per cell, the fixed "
                "scratch has %llu B for cell slots",
                (unsigned long long)num_lefs, (unsigned long long)P.slot_bytes, (unsigned long long)slot_room);
  P.prof = nullptr;
  cudaStream_t st = active_stream(ctx);
  CellTask* tasks = (CellTask*)(scratch + NOALLOC_TASKS_OFFSET);
  rc = launch_pack_tasks(cell_seeds, target_contacts, ncells, tasks, st, err, sizeof(err));
  if (rc) return fail(rc, "%s", err);
  DevChrom dc{ch.d_bars, ch.d_pos_flags, ch.nb};
  rc = launch_simulate(P, dc, tasks, ncells, target_epochs, band, missed_updates, stats, nullptr,
                       ctx->d_jump, (u32*)scratch, scratch + NOALLOC_SLOTS_OFFSET, slot_room, st, err,
                       sizeof(err));
  if (rc) return fail(rc, "%s", err);
  return MGPU_OK;
}

extern "C" int mgpu_simulate_cells_ex(mgpu_ctx* ctx, int chrom_id, const uint64_t* cell_seeds,
                                      const uint64_t* target_contacts, uint64_t target_epochs,
                                      uint64_t num_lefs, uint64_t ncells, uint32_t* band,
                                      uint64_t* missed_updates, mgpu_cell_stats* stats,
                                      const mgpu_extra_outputs* extra) {
  if (!ctx) return fail(MGPU_ERR_INVALID_ARG, "mgpu_simulate_cells_ex: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  return run_cells(ctx, chrom_id, cell_seeds, target_contacts, target_epochs, num_lefs, ncells,
                   band, missed_updates, stats, nullptr, extra);
}

extern "C" int mgpu_trace_cell(mgpu_ctx* ctx, int chrom_id, uint64_t cell_seed,
                               uint64_t target_contacts, uint64_t target_epochs, uint64_t num_lefs,
                               uint32_t* band, mgpu_cell_stats* stats, mgpu_trace_request* tr) {
  if (!ctx || !tr) return fail(MGPU_ERR_INVALID_ARG, "mgpu_trace_cell: null argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  const uint64_t n = num_lefs;
  const uint64_t recs = tr->max_records;
  std::vector<DevBuf> arrs(9);
  uint64_t* host_arrays[9] = {tr->rev_pos, tr->fwd_pos, tr->binding_epoch, tr->rev_rank, tr->fwd_rank,
                              tr->rev_move, tr->fwd_move, tr->rev_collision, tr->fwd_collision};
  DevTrace T{};
  T.max_records = recs;
  uint64_t* dev_arrays[9] = {nullptr};
  for (int k = 0; k < 9; ++k) {
    if (host_arrays[k] && recs) {
      CK(cudaMalloc(&arrs[k].p, recs * n * 8));
      arrs[k].owned = true;
      dev_arrays[k] = (uint64_t*)arrs[k].p;
    }
  }
  T.rev_pos = dev_arrays[0];
  T.fwd_pos = dev_arrays[1];
  T.binding_epoch = dev_arrays[2];
  T.rev_rank = dev_arrays[3];
  T.fwd_rank = dev_arrays[4];
  T.rev_move = dev_arrays[5];
  T.fwd_move = dev_arrays[6];
  T.rev_collision = dev_arrays[7];
  T.fwd_collision = dev_arrays[8];
  DevBuf d_headers, d_all, d_num;
  if (tr->headers && recs) {
    CK(cudaMalloc(&d_headers.p, recs * sizeof(mgpu_trace_header)));
    d_headers.owned = true;
    T.headers = (mgpu_trace_header*)d_headers.p;
  }
  if (tr->all_headers && tr->max_epochs) {
    CK(cudaMalloc(&d_all.p, tr->max_epochs * sizeof(mgpu_trace_header)));
    d_all.owned = true;
    T.all_headers = (mgpu_trace_header*)d_all.p;
    T.max_epochs = tr->max_epochs;
  }
  CK(cudaMalloc(&d_num.p, 8));
  d_num.owned = true;
  CK(cudaMemset(d_num.p, 0, 8));
  T.num_recorded = (uint64_t*)d_num.p;
  mgpu_cell_stats local{};
  int rc = run_cells(ctx, chrom_id, &cell_seed, &target_contacts, target_epochs, num_lefs, 1, band,
                     nullptr, &local, &T);
  if (stats) *stats = local;
  uint64_t nrec = 0;
  CK(cudaMemcpy(&nrec, d_num.p, 8, cudaMemcpyDeviceToHost));
  tr->num_epochs_recorded = std::min(nrec, tr->max_epochs);
  const uint64_t have = std::min(nrec, recs);
  for (int k = 0; k < 9; ++k) {
    if (dev_arrays[k] && have) CK(cudaMemcpy(host_arrays[k], dev_arrays[k], have * n * 8, cudaMemcpyDeviceToHost));
  }
  if (T.headers && have) CK(cudaMemcpy(tr->headers, T.headers, have * sizeof(mgpu_trace_header), cudaMemcpyDeviceToHost));
  if (T.all_headers && tr->num_epochs_recorded)
    CK(cudaMemcpy(tr->all_headers, T.all_headers, tr->num_epochs_recorded * sizeof(mgpu_trace_header),
                  cudaMemcpyDeviceToHost));
  return rc;
}

extern "C" int mgpu_run_phase(mgpu_ctx* ctx, int chrom_id, int phase, mgpu_phase_io* io) {
  if (!ctx || !io) return fail(MGPU_ERR_INVALID_ARG, "mgpu_run_phase: null argument");
  std::lock_guard<std::mutex> lk(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  if (chrom_id < 0 || chrom_id >= (int)ctx->chroms.size())
    return fail(MGPU_ERR_INVALID_ARG, "unknown chromosome handle %d", chrom_id);
  const ChromEntry& ch = ctx->chroms[chrom_id];
  const uint64_t n = io->num_lefs;
  if (n == 0) return fail(MGPU_ERR_INVALID_ARG, "num_lefs must be positive");
  KParams P;
  int rc = make_kparams(ctx, ch, n, &P);
  if (rc) return rc;
  uint64_t* host_arrays[9] = {io->rev_pos, io->fwd_pos, io->binding_epoch, io->rev_rank, io->fwd_rank,
                              io->rev_move, io->fwd_move, io->rev_collision, io->fwd_collision};
  for (int k = 0; k < 9; ++k)
    if (!host_arrays[k]) return fail(MGPU_ERR_INVALID_ARG, "mgpu_run_phase: state array %d is null", k);
  // the kernel indexes shared memory with these values: reject what the reference's own
  // invariants exclude (ranks are permutations of [0, n); collision indices point at
  // barriers or LEFs that exist)
  {
    std::vector<uint8_t> seen_r(n, 0), seen_f(n, 0);
    for (uint64_t i = 0; i < n; ++i) {
      const uint64_t r = io->rev_rank[i], f = io->fwd_rank[i];
      if (r >= n || f >= n || seen_r[r]++ || seen_f[f]++)
        return fail(MGPU_ERR_INVALID_ARG, "rank buffers must be permutations of [0, num_lefs)");
      for (const uint64_t w : {io->rev_collision[i], io->fwd_collision[i]}) {
        const uint64_t ev = w >> 56, idx = w & ((1ull << 55) - 1);
        if (ev & ~0x1Full) return fail(MGPU_ERR_INVALID_ARG, "invalid collision event bits");
        if ((ev & MGPU_COLL_LEF_BAR) && idx >= ch.nb)
          return fail(MGPU_ERR_INVALID_ARG, "LEF-BAR collision points past the barriers");
        if ((ev & (MGPU_COLL_LEF_LEF_PRIMARY | MGPU_COLL_LEF_LEF_SECONDARY)) && idx >= n)
          return fail(MGPU_ERR_INVALID_ARG, "LEF-LEF collision points past the LEFs");
        if (idx > CW_IDX_MASK) return fail(MGPU_ERR_UNSUPPORTED, "collision index beyond 2^27");
      }
      const uint64_t rp = io->rev_pos[i], fp = io->fwd_pos[i];
      if ((rp != UINT64_MAX && rp >= 0xFFFFFFFFull) || (fp != UINT64_MAX && fp >= 0xFFFFFFFFull))
        return fail(MGPU_ERR_UNSUPPORTED, "positions beyond 2^32 - 2");
      if (io->rev_move[i] > 0xFFFFFFFFull || io->fwd_move[i] > 0xFFFFFFFFull)
        return fail(MGPU_ERR_UNSUPPORTED, "moves beyond 2^32 - 1");
    }
  }
  DevBuf d_arr, d_mask, d_bst, d_prng, d_outs;
  CK(cudaMalloc(&d_arr.p, 9 * n * 8));
  d_arr.owned = true;
  for (int k = 0; k < 9; ++k)
    CK(cudaMemcpy((uint64_t*)d_arr.p + k * n, host_arrays[k], n * 8, cudaMemcpyHostToDevice));
  if (io->bind_mask) {
    CK(cudaMalloc(&d_mask.p, n * 8));
    d_mask.owned = true;
    CK(cudaMemcpy(d_mask.p, io->bind_mask, n * 8, cudaMemcpyHostToDevice));
  }
  if (io->barrier_state && ch.nb) {
    CK(cudaMalloc(&d_bst.p, ch.nb));
    d_bst.owned = true;
    CK(cudaMemcpy(d_bst.p, io->barrier_state, ch.nb, cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&d_prng.p, 32));
  d_prng.owned = true;
  CK(cudaMemcpy(d_prng.p, io->prng_state, 32, cudaMemcpyHostToDevice));
  CK(cudaMalloc(&d_outs.p, 32));
  d_outs.owned = true;
  CK(cudaMemset(d_outs.p, 0, 32));
  char err[256] = {0};
  DevChrom dc{ch.d_bars, ch.d_pos_flags, ch.nb};
  if (P.slot_bytes) {
    rc = ensure_scratch(ctx, P, 1);
    if (rc) return rc;
  }
  rc = launch_phase(P, dc, phase, n, (uint64_t*)d_arr.p, (uint64_t*)d_mask.p, (uint8_t*)d_bst.p,
                    io->epoch, io->burnin_completed, io->ranks_partially_sorted, io->init_ranks,
                    io->adjust_moves, (uint64_t*)d_prng.p, (uint64_t*)d_outs.p, ctx->d_jump,
                    ctx->d_scratch, active_stream(ctx), err, sizeof(err));
  if (rc) return fail(rc, "%s", err);
  CK(cudaStreamSynchronize(active_stream(ctx)));
  for (int k = 0; k < 9; ++k)
    CK(cudaMemcpy(host_arrays[k], (uint64_t*)d_arr.p + k * n, n * 8, cudaMemcpyDeviceToHost));
  if (io->barrier_state && ch.nb) CK(cudaMemcpy(io->barrier_state, d_bst.p, ch.nb, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(io->prng_state, d_prng.p, 32, cudaMemcpyDeviceToHost));
  uint64_t outs[4];
  CK(cudaMemcpy(outs, d_outs.p, 32, cudaMemcpyDeviceToHost));
  io->n5prime = outs[0];
  io->n3prime = outs[1];
  io->lefs_released = outs[2];
  if (outs[3] != DEV_OK) {
    mgpu_cell_stats s{};
    s.status = outs[3];
    return status_from_stats(&s, 1);
  }
  return MGPU_OK;
}

// ===========================================================================================
// Probes of the device's floating-point library (test hooks, no reference counterpart)
// ===========================================================================================
extern "C" int mgpu_probe_samplers(int device, int kind, const uint64_t* seeds, uint64_t nstreams,
                                   uint64_t per_stream, double a0, double a1, double* out, uint64_t* draws) {
  if ((nstreams && (!seeds || !out || !draws)) || kind < 0 || kind > MGPU_PROBE_GEV)
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_probe_samplers: bad argument");
  if (nstreams == 0 || per_stream == 0) return MGPU_OK;
  CK(cudaSetDevice(device));
  KParams P{};
  int dev_kind = 0;
  switch (kind) {
    case MGPU_PROBE_NORMAL: dev_kind = 0; break;
    case MGPU_PROBE_EXPONENTIAL: dev_kind = 1; break;
    case MGPU_PROBE_POISSON: {
      // constants as the epoch loop's burn-in Poisson has them (make_kparams)
      dev_kind = 2;
      const double mean = a0;
      P.pois_mean = mean;
      P.pois_exp_mean = std::exp(-mean);
      P.pois_smu = std::sqrt(mean);
      P.pois_b = 0.931 + 2.53 * P.pois_smu;
      P.pois_a = -0.059 + 0.02483 * P.pois_b;
      P.pois_inv_alpha = 1.1239 + 1.1328 / (P.pois_b - 3.4);
      P.pois_v_r = 0.9277 - 3.6224 / (P.pois_b - 2);
      break;
    }
    case MGPU_PROBE_BINOMIAL:
    case MGPU_PROBE_BINOMIAL_DEVICE_POW: {
      dev_kind = 3;
      const double p = (0.5 < a1) ? (1 - a1) : a1;
      // the epoch loop's full epochs take (1 - p)^t from the host; a last, shorter epoch
      // evaluates it on the device
      P.spe = kind == MGPU_PROBE_BINOMIAL ? (uint64_t)(int64_t)a0 : ~0ull;
      P.bin_q_n = std::pow((1 - p), (double)(int64_t)a0);
      break;
    }
    case MGPU_PROBE_GEV:
      dev_kind = 4;
      P.gev_mu = 0.0;
      P.gev_sigma = a0;
      P.gev_xi = a1;
      break;
  }
  std::vector<uint64_t> states(4 * nstreams);
  for (uint64_t s = 0; s < nstreams; ++s) mgpu_prng_seed(seeds[s], &states[4 * s]);
  u64 *d_states = nullptr, *d_draws = nullptr;
  double* d_out = nullptr;
  const size_t nout = (size_t)nstreams * per_stream;
  int rc = cuda_check(cudaMalloc(&d_states, states.size() * 8), "cudaMalloc(states)");
  if (!rc) rc = cuda_check(cudaMalloc(&d_out, nout * 8), "cudaMalloc(samples)");
  if (!rc) rc = cuda_check(cudaMalloc(&d_draws, nstreams * 8), "cudaMalloc(draws)");
  if (!rc) rc = cuda_check(cudaMemcpy(d_states, states.data(), states.size() * 8, cudaMemcpyHostToDevice), "copy");
  char err[256] = {0};
  if (!rc) {
    rc = launch_sampler_probe(P, dev_kind, d_states, nstreams, per_stream, a0, a1, d_out, d_draws, nullptr, err,
                              sizeof(err));
    if (rc) rc = fail(rc, "%s", err);
  }
  if (!rc) rc = cuda_check(cudaDeviceSynchronize(), "sampler probe");
  if (!rc) rc = cuda_check(cudaMemcpy(out, d_out, nout * 8, cudaMemcpyDeviceToHost), "copy samples");
  if (!rc) rc = cuda_check(cudaMemcpy(draws, d_draws, nstreams * 8, cudaMemcpyDeviceToHost), "copy draws");
  cudaFree(d_states);
  cudaFree(d_out);
  cudaFree(d_draws);
  return rc;
}

extern "C" int mgpu_probe_libm(int device, int kind, const double* x, const double* y, uint64_t n, double mu,
                               double sigma, double xi, double* out) {
  const bool needs_y = kind == MGPU_PROBE_POW || kind == MGPU_PROBE_BELOW_EXP;
  if ((n && (!x || !out || (needs_y && !y))) || kind < 0 || kind > MGPU_PROBE_BELOW_EXP)
    return fail(MGPU_ERR_INVALID_ARG, "mgpu_probe_libm: bad argument");
  if (n == 0) return MGPU_OK;
  CK(cudaSetDevice(device));
  double *d_x = nullptr, *d_y = nullptr, *d_out = nullptr;
  int rc = cuda_check(cudaMalloc(&d_x, n * 8), "cudaMalloc(x)");
  if (!rc && needs_y) rc = cuda_check(cudaMalloc(&d_y, n * 8), "cudaMalloc(y)");
  if (!rc) rc = cuda_check(cudaMalloc(&d_out, n * 8), "cudaMalloc(out)");
  if (!rc) rc = cuda_check(cudaMemcpy(d_x, x, n * 8, cudaMemcpyHostToDevice), "copy x");
  if (!rc && needs_y) rc = cuda_check(cudaMemcpy(d_y, y, n * 8, cudaMemcpyHostToDevice), "copy y");
  char err[256] = {0};
  if (!rc) {
    rc = launch_libm_probe(kind, d_x, d_y, n, mu, sigma, xi, d_out, nullptr, err, sizeof(err));
    if (rc) rc = fail(rc, "%s", err);
  }
  if (!rc) rc = cuda_check(cudaDeviceSynchronize(), "libm probe");
  if (!rc) rc = cuda_check(cudaMemcpy(out, d_out, n * 8, cudaMemcpyDeviceToHost), "copy out");
  cudaFree(d_x);
  cudaFree(d_y);
  cudaFree(d_out);
  return rc;
}
