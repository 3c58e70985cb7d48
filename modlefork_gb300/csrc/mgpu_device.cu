// mgpu_device.cu - sm_103a kernels of the loop-extrusion epoch engine.
//
// One warp simulates one cell (Simulation::simulate_one_cell, src/libmodle/cpu/
// simulation.cpp:1056-1152).  The cell's state is structure-of-arrays of 32-bit words; the
// host plans which per-LEF arrays fit in the cell's shared memory and places the rest in a
// per-cell global scratch slot (large chromosomes).  The barrier track and its integer
// thresholds are read-only in global memory and shared by every cell of the chromosome.
// The kernel is persistent: each warp pulls cell indices from a global work counter.
//
// Draw order.  Every random number of the reference comes from one sequential
// Xoshiro256++ stream per cell, consumed in a data-dependent order.  The warp keeps a ring of
// pre-generated draws in shared memory: all 32 lanes generate RNG_S consecutive draws each per
// refill and then advance their private state by 31 * RNG_S steps with a GF(2) jump table (the
// state transition of xoshiro is linear), so the ring always holds the exact stream.
//
// Every step of the epoch runs warp-parallel with the exact draw order:
//  * steps whose items take one draw each (binding, barrier steps, moves, release, LEF-BAR
//    and LEF-LEF trials) give lane k the draw at offset popc(ballot & lanemask_lt);
//  * items that may take more draws (ziggurat wedges and tails, rejected contact attempts,
//    failed bypass trials in a chain of secondary collisions) are evaluated speculatively at
//    the offsets they would have if every earlier item took its usual count; the first item
//    that deviates is resolved exactly and the warp resumes after it;
//  * sequential sweeps are replaced by closed forms: rank_lefs by a merge of the units bound
//    this epoch into the still-sorted order of the others, adjust_moves by segmented min/max
//    scans, the LEF-BAR and primary LEF-LEF sweeps by binary searches over the ranked
//    positions.
// Where a closed form's precondition does not hold (full ties in the ranking, a chain that
// reaches a chromosome end, unsorted caller input), the step falls back to a line-by-line
// serial restatement run by lane 0, so results never depend on the fast path.
//
// Floating point.  The file is compiled with --fmad=false so every double multiply and add
// is rounded separately, like the reference's x86-64 build; bernoulli and
// generate_canonical comparisons are exact integer thresholds computed on the host.

#include <cuda_runtime.h>

#include <cstdio>

#include "cppsort_emul.h"
#include "mgpu_internal.h"
#define MGPU_ZIG_TABLE_QUAL __device__ const
#include "ziggurat_tables.h"

namespace mgpu {

#define MGPU_ITER_LIMIT 100000000ull
#define FULL 0xFFFFFFFFu

// Items per lane in the chunked sweeps: the per-LEF arrays of large cells live in global
// memory, where every dependent load waits for L2; a lane that carries MLP independent items
// through each stage of a sweep keeps MLP loads in flight instead of one.
#ifndef MGPU_MLP
#define MGPU_MLP 2
#endif
constexpr unsigned MLP = MGPU_MLP;


__device__ __forceinline__ u64 rotl64(u64 x, int k) { return (x << k) | (x >> (64 - k)); }

__device__ __forceinline__ u64 xo_next(u64* s) {
  const u64 result = rotl64(s[0] + s[3], 23) + s[0];
  const u64 t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return result;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ u32 ln() { return threadIdx.x & 31u; }

__device__ __forceinline__ u64 pos64(u32 v) { return v == UNBOUND ? ~0ull : (u64)v; }

// exclusive prefix sum over the warp; *total receives the sum of all lanes
__device__ __forceinline__ u32 warp_excl_scan(u32 v, u32* total) {
  u32 x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const u32 y = __shfl_up_sync(FULL, x, d);
    if ((int)ln() >= d) x += y;
  }
  if (total) *total = __shfl_sync(FULL, x, 31);
  return x - v;
}

// Cell scalars (warp-uniform, kept in shared memory so lane 0's serial code can update them).
// Per-launch profile counters (cycles per step and fallback counts), summed over cells.
enum : u32 {
  PF_BURNIN = 0, PF_BIND, PF_RANK, PF_CONTACTS, PF_MOVES, PF_ADJUST, PF_BARRIERS, PF_BOUNDARIES,
  PF_LEF_BAR, PF_PRIMARY, PF_CORRECT, PF_SECONDARY, PF_FIX, PF_EXTRUDE_RELEASE, PF_TRACE, PF_TOTAL,
  PF_RANK_FALLBACK, PF_ADJUST_FALLBACK, PF_CHAIN_SERIAL, PF_CONTACT_SERIAL, PF_FIX_FALLBACK,
  PF_REFILLS, PF_STALE_REFILLS, PF_EPOCHS, PF_RANK_PDQ, PF_RANK_PASS, PF_RANK_BLOCK, PF_RANK_MERGE,
  PF_RANK_SERIAL, PF_COUNT = 32
};

struct Scalars {
  u64 rpos, gpos;  // next draw to consume / to generate (stream indices)
  u64 canon[4];    // xoshiro state at gpos
  u32 lanes_stale; // lanes must re-derive their states from canon before the next refill
  u32 status;
  u64 epoch, num_burnin_epochs, num_active, num_contacts;
  u32 burnin_completed, flag;
  u64 missed, lef_epochs, sort_fallbacks;
  u64 n5, n3;
  u32 hist_size, hist_head;
  u64 bc0, bc1, bc2;  // broadcast slots for lane 0 results
  u64 nrec;           // model-state records written for this cell
  u64* prof;          // profile counters of the launch (device memory) or null
};
static_assert(sizeof(Scalars) <= CELL_HEADER_BYTES, "scalars do not fit the cell header");

// Pointers of one cell (lives in shared memory; identical for every lane).
struct Cell {
  Scalars* sc;
  u64* ring;
  u32 *rev, *fwd, *rr, *fr, *rm, *fm, *rc, *fc, *sr, *sf, *tmp, *bep;
  u32* bst;
  double *hcfx, *havg;
  const DevBarrier* bar;
  const uint2* bpf;  // {pos, flags}
  u32 nb;
  u32 nl;
  const ulonglong2* jt;
  u32* band;
};

// Position and flags of barrier i through the read-only data path (8 bytes per barrier, so the
// sweeps over the barrier track stay in cache).
__device__ __forceinline__ u32 bar_pos(const Cell& c, u32 i) { return __ldg(&c.bpf[i].x); }
__device__ __forceinline__ u32 bar_flags(const Cell& c, u32 i) { return __ldg(&c.bpf[i].y); }

// ---------------------------------------------------------------------------------------
// PRNG ring
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void xo_jump(u64* s, const ulonglong2* jt) {
  u64 n0 = 0, n1 = 0, n2 = 0, n3 = 0;
#pragma unroll 8
  for (int c = 0; c < 64; ++c) {
    const u32 v = (u32)(s[c >> 4] >> ((c & 15) * 4)) & 15u;
    const ulonglong2* e = jt + 2 * (c * 16 + v);
    const ulonglong2 e0 = __ldg(e), e1 = __ldg(e + 1);
    n0 ^= e0.x;
    n1 ^= e0.y;
    n2 ^= e1.x;
    n3 ^= e1.y;
  }
  s[0] = n0;
  s[1] = n1;
  s[2] = n2;
  s[3] = n3;
}

// Collective: append RNG_BLOCK draws to the ring.  s is this lane's private stream state.
__device__ __noinline__ void rng_refill(Cell& c, u64* s) {
  Scalars* sc = c.sc;
  const u32 lane = ln();
  const bool stale = sc->lanes_stale != 0;
  if (stale) {
    for (int k = 0; k < 4; ++k) s[k] = sc->canon[k];
    for (u32 t = 0; t < lane * RNG_S; ++t) xo_next(s);
  }
  if (lane == 0 && sc->prof) {
    atomicAdd((unsigned long long*)&sc->prof[PF_REFILLS], 1ull);
    if (stale) atomicAdd((unsigned long long*)&sc->prof[PF_STALE_REFILLS], 1ull);
  }
  const u64 g = sc->gpos;
#pragma unroll 4
  for (int k = 0; k < RNG_S; ++k) c.ring[(g + (u64)lane * RNG_S + k) & (RING - 1)] = xo_next(s);
  xo_jump(s, c.jt);
  __syncwarp();
  if (lane == 0) {
    sc->gpos = g + RNG_BLOCK;
    for (int k = 0; k < 4; ++k) sc->canon[k] = s[k];
    sc->lanes_stale = 0;
  }
  __syncwarp();
}

// Collective: make at least n (<= RNG_BLOCK) unconsumed draws available.
__device__ __forceinline__ void rng_ensure(Cell& c, u64* s, u32 n) {
  while (c.sc->gpos - c.sc->rpos < n) rng_refill(c, s);
}

__device__ __forceinline__ u64 ring_at(const Cell& c, u64 k) { return c.ring[k & (RING - 1)]; }

// Lane 0 only: next draw of the stream, generated serially when the ring is dry.
__device__ __noinline__ u64 rng_serial(Cell& c) {
  Scalars* sc = c.sc;
  if (sc->rpos == sc->gpos) {
    const u64 v = xo_next(sc->canon);
    c.ring[sc->gpos & (RING - 1)] = v;
    sc->gpos++;
    sc->lanes_stale = 1;
  }
  const u64 v = c.ring[sc->rpos & (RING - 1)];
  sc->rpos++;
  return v;
}

__device__ __forceinline__ void prof_add(Cell& c, u32 k, u64 v) {
  if (ln() == 0 && c.sc->prof) atomicAdd((unsigned long long*)&c.sc->prof[k], (unsigned long long)v);
}

__device__ __forceinline__ void set_status(Cell& c, u32 st) {
  if (c.sc->status == DEV_OK) c.sc->status = st;
}

// ---------------------------------------------------------------------------------------
// Serial distributions (lane 0).  Boost.Random 1.79 semantics, see the oracle for the
// line-by-line restatement; thresholds replace bernoulli / canonical comparisons.
// ---------------------------------------------------------------------------------------

__device__ u64 s_uniform_int(Cell& c, u64 a, u64 b) {
  const u64 range = b - a;
  if (range == 0) return a;
  if (range == ~0ull) return rng_serial(c) + a;
  u64 bucket = ~0ull / (range + 1);
  if (~0ull % (range + 1) == range) ++bucket;
  for (u64 it = 0; it < 1000; ++it) {
    const u64 r = rng_serial(c) / bucket;
    if (r <= range) return a + r;
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
  return a;
}

__device__ __forceinline__ bool s_trial(Cell& c, const Trial& t) {
  if (t.always) return true;
  if (!t.draws) return false;
  return rng_serial(c) <= t.thr;
}

__device__ __forceinline__ double u01_of(u64 u) { return (double)u * (1.0 / 18446744073709551616.0); }

__device__ double s_uniform01(Cell& c) {
  for (int it = 0; it < 1000; ++it) {
    const double r = u01_of(rng_serial(c));
    if (r < 1.0) return r;
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
  return 0.0;
}

__device__ __forceinline__ double canonical_of(u64 u) {
  double r = (double)u / 18446744073709551616.0;
  if (r == 1.0) r -= 1.1102230246251565e-16;  // DBL_EPSILON / 2
  return r;
}

// generate_int_float_pair<double, 8>
__device__ __forceinline__ double ifp_fraction(u64 u) {
  u &= ~(1ull << 11);
  return (double)(u >> 8) * (1.0 / 72057594037927936.0);
}

// Draw sources of the samplers below.  SerialSrc is lane 0's view of the cell's stream; RingSrc
// is one lane's view of the pre-generated ring starting at a given stream position, which
// reports exhaustion instead of generating.
struct SerialSrc {
  Cell& c;
  u32 n;
  __device__ bool next(u64& u) {
    u = rng_serial(c);
    ++n;
    return true;
  }
};

struct RingSrc {
  const u64* ring;
  u64 pos, end;
  u32 n;
  __device__ bool next(u64& u) {
    if (pos >= end) return false;
    u = ring[pos & (RING - 1)];
    ++pos;
    ++n;
    return true;
  }
};

// Sampler results: 0 = value produced, 1 = the source ran dry, 2 = iteration limit.
enum { SMP_OK = 0, SMP_DRY = 1, SMP_LIMIT = 2 };

// y < exp(a) for a <= 0, decided exactly: a float estimate of exp(a) settles it unless y lies
// within 1e-5 (relative) of the estimate, whose error is below 1e-6; only then is the double
// exp evaluated.
__device__ __forceinline__ bool below_exp(double y, double a) {
  const float ef = expf((float)a);
  const double d = y - (double)ef;
  if (fabs(d) > 1e-5 * (double)ef) return d < 0;
  return y < exp(a);
}

// uniform_01<double> on one draw per attempt (values equal to 1 are rejected)
template <class Src>
__device__ int uniform01_t(Src& g, double& r) {
  for (int it = 0; it < 1000; ++it) {
    u64 u;
    if (!g.next(u)) return SMP_DRY;
    r = u01_of(u);
    if (r < 1.0) return SMP_OK;
  }
  return SMP_LIMIT;
}

// unit_exponential_distribution: 256-layer ziggurat with the shift-on-layer-0 tail
template <class Src>
__device__ int unit_exponential_t(Src& g, double& out) {
  double shift = 0;
  for (int it = 0; it < 100000; ++it) {
    u64 u;
    if (!g.next(u)) return SMP_DRY;
    const int i = (int)(u & 0xFF);
    const double x = ifp_fraction(u) * mgpu_zig_exp_x[i];
    if (x < mgpu_zig_exp_x[i + 1]) {
      out = shift + x;
      return SMP_OK;
    }
    if (i == 0) {
      shift += mgpu_zig_exp_x[1];
    } else {
      double y01;
      const int r = uniform01_t(g, y01);
      if (r) return r;
      const double y = mgpu_zig_exp_y[i] + y01 * (mgpu_zig_exp_y[i + 1] - mgpu_zig_exp_y[i]);
      if (below_exp(y, -x)) {
        out = x + shift;
        return SMP_OK;
      }
    }
  }
  return SMP_LIMIT;
}

// tail of the normal ziggurat (Marsaglia's method with two exponentials)
template <class Src>
__device__ int normal_tail_t(Src& g, double& out) {
  const double tail_start = mgpu_zig_normal_x[1];
  for (int it = 0; it < 100000; ++it) {
    double e1, e2;
    int r = unit_exponential_t(g, e1);
    if (r) return r;
    r = unit_exponential_t(g, e2);
    if (r) return r;
    const double x = e1 / tail_start;
    const double y = e2 / 1.0;
    if (2 * y > x * x) {
      out = x + tail_start;
      return SMP_OK;
    }
  }
  return SMP_LIMIT;
}

// unit_normal_distribution: 128-layer ziggurat, sign from bit 0 of the layer byte
template <class Src>
__device__ int unit_normal_t(Src& g, double& out) {
  for (int it = 0; it < 100000; ++it) {
    u64 u;
    if (!g.next(u)) return SMP_DRY;
    const int ii = (int)(u & 0xFF);
    const int sign = (ii & 1) * 2 - 1;
    const int i = ii >> 1;
    const double x = ifp_fraction(u) * mgpu_zig_normal_x[i];
    if (x < mgpu_zig_normal_x[i + 1]) {
      out = x * sign;
      return SMP_OK;
    }
    if (i == 0) {
      double t;
      const int r = normal_tail_t(g, t);
      if (r) return r;
      out = t * sign;
      return SMP_OK;
    }
    double y01;
    const int r = uniform01_t(g, y01);
    if (r) return r;
    const double y = mgpu_zig_normal_y[i] + y01 * (mgpu_zig_normal_y[i + 1] - mgpu_zig_normal_y[i]);
    if (below_exp(y, -(x * x / 2))) {
      out = x * sign;
      return SMP_OK;
    }
  }
  return SMP_LIMIT;
}

__device__ __noinline__ double s_unit_exponential(Cell& c) {
  SerialSrc g{c, 0};
  double v = 0.0;
  if (unit_exponential_t(g, v) != SMP_OK) set_status(c, DEV_ERR_ITER_LIMIT);
  return v;
}

__device__ __noinline__ double s_unit_normal(Cell& c) {
  SerialSrc g{c, 0};
  double v = 0.0;
  if (unit_normal_t(g, v) != SMP_OK) set_status(c, DEV_ERR_ITER_LIMIT);
  return v;
}

__device__ const double kLogFactorial[10] = {0.0,
                                             0.0,
                                             0.69314718055994529,
                                             1.7917594692280550,
                                             3.1780538303479458,
                                             4.7874917427820458,
                                             6.5792512120101012,
                                             8.5251613610654147,
                                             10.604602902745251,
                                             12.801827480081469};

__device__ __noinline__ u64 s_poisson(Cell& c, const KParams& P) {
  const double mean = P.pois_mean;
  if (mean < 10) {
    double p = P.pois_exp_mean;
    u64 x = 0;
    double u = s_uniform01(c);
    while (u > p) {
      u = u - p;
      ++x;
      p = mean * p / (double)x;
      if (x > MGPU_ITER_LIMIT) {
        set_status(c, DEV_ERR_ITER_LIMIT);
        break;
      }
    }
    return x;
  }
  const double smu = P.pois_smu, b = P.pois_b, a = P.pois_a, inv_alpha = P.pois_inv_alpha,
               v_r = P.pois_v_r;
  for (int it = 0; it < 100000; ++it) {
    double u;
    double v = s_uniform01(c);
    if (v <= 0.86 * v_r) {
      u = v / v_r - 0.43;
      return (u64)floor((2 * a / (0.5 - fabs(u)) + b) * u + mean + 0.445);
    }
    if (v >= v_r) {
      u = s_uniform01(c) - 0.5;
    } else {
      u = v / v_r - 0.93;
      u = ((u < 0) ? -0.5 : 0.5) - u;
      v = s_uniform01(c) * v_r;
    }
    const double us = 0.5 - fabs(u);
    if (us < 0.013 && v > us) continue;
    const double k = floor((2 * a / us + b) * u + mean + 0.43);
    v = v * inv_alpha / (a / (us * us) + b);
    const double log_sqrt_2pi = 0.91893853320467267;
    if (k >= 10) {
      if (log(v * smu) <= (k + 0.5) * log(mean / k) - mean - log_sqrt_2pi + k -
                              (1 / 12. - (1 / 360. - 1 / (1260. * k * k)) / (k * k)) / k) {
        return (u64)k;
      }
    } else if (k >= 0) {
      if (log(v) <= k * log(mean) - mean - kLogFactorial[(int)k]) return (u64)k;
    }
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
  return 0;
}

__device__ const double kBinomialFc[10] = {0.08106146679532726, 0.04134069595540929,
                                           0.02767792568499834, 0.02079067210376509,
                                           0.01664469118982119, 0.01387612882307075,
                                           0.01189670994589177, 0.01041126526197209,
                                           0.009255462182712733, 0.008330563433362871};

__device__ double binomial_fc(i64 k) {
  if (k < 10) return kBinomialFc[k];
  const double ikp1 = 1.0 / (double)(k + 1);
  return (1.0 / 12 - (1.0 / 360 - (1.0 / 1260) * (ikp1 * ikp1)) * (ikp1 * ikp1)) * ikp1;
}

__device__ __noinline__ i64 s_binomial(Cell& c, const KParams& P, i64 t_, double p_) {
  const double p = (0.5 < p_) ? (1 - p_) : p_;
  const i64 t = t_;
  const i64 m = (i64)((t + 1) * p);
  if (m < 11) {
    const double q_n = ((u64)t == P.spe) ? P.bin_q_n : pow((1 - p), (double)t);
    const double pp = (0.5 < p_) ? (1 - p_) : p_;
    const double q = 1 - pp;
    const double s = pp / q;
    const double a = (t + 1) * s;
    double r = q_n;
    double u = s_uniform01(c);
    i64 x = 0;
    while (u > r) {
      u = u - r;
      ++x;
      const double r1 = ((a / x) - s) * r;
      if (r1 < 2.220446049250313e-16 && r1 < r) break;
      r = r1;
    }
    return (0.5 < p_) ? t_ - x : x;
  }
  const double r = p / (1 - p);
  const double nr = (t + 1) * r;
  const double npq = t * p * (1 - p);
  const double sqrt_npq = sqrt(npq);
  const double b = 1.15 + 2.53 * sqrt_npq;
  const double a = -0.0873 + 0.0248 * b + 0.01 * p;
  const double cc = t * p + 0.5;
  const double alpha = (2.83 + 5.1 / b) * sqrt_npq;
  const double v_r = 0.92 - 4.2 / b;
  const double u_rv_r = 0.86 * v_r;
  i64 res = 0;
  bool done = false;
  for (int it = 0; it < 100000 && !done; ++it) {
    double u;
    double v = s_uniform01(c);
    if (v <= u_rv_r) {
      u = v / v_r - 0.43;
      res = (i64)floor((2 * a / (0.5 - fabs(u)) + b) * u + cc);
      done = true;
      break;
    }
    if (v >= v_r) {
      u = s_uniform01(c) - 0.5;
    } else {
      u = v / v_r - 0.93;
      u = ((u < 0) ? -0.5 : 0.5) - u;
      v = s_uniform01(c) * v_r;
    }
    const double us = 0.5 - fabs(u);
    const i64 k = (i64)floor((2 * a / us + b) * u + cc);
    if (k < 0 || k > t) continue;
    v = v * alpha / (a / (us * us) + b);
    const double km = fabs((double)(k - m));
    if (km <= 15) {
      double f = 1;
      if (m < k) {
        i64 i = m;
        do {
          ++i;
          f = f * (nr / i - r);
        } while (i != k);
      } else if (m > k) {
        i64 i = k;
        do {
          ++i;
          v = v * (nr / i - r);
        } while (i != m);
      }
      if (v <= f) {
        res = k;
        done = true;
      }
      continue;
    }
    v = log(v);
    const double rho = (km / npq) * (((km / 3. + 0.625) * km + 1. / 6) / npq + 0.5);
    const double tt = -km * km / (2 * npq);
    if (v < tt - rho) {
      res = k;
      done = true;
      continue;
    }
    if (v > tt + rho) continue;
    const i64 nm = t - m + 1;
    const double h = (m + 0.5) * log((m + 1) / (r * nm)) + binomial_fc(m) + binomial_fc(t - m);
    const i64 nk = t - k + 1;
    if (v <= h + (t + 1) * log((double)nm / nk) + (k + 0.5) * log(nk * r / (k + 1)) -
                 binomial_fc(k) - binomial_fc(t - k)) {
      res = k;
      done = true;
    }
  }
  if (!done) set_status(c, DEV_ERR_ITER_LIMIT);
  return (0.5 < p_) ? t_ - res : res;
}

__device__ __noinline__ double s_gev(Cell& c, const KParams& P) {
  const double u = canonical_of(rng_serial(c));
  if (P.gev_xi == 0.0) return (P.gev_mu - P.gev_sigma) * log(-log(u));
  return P.gev_mu + (P.gev_sigma * (1.0 - pow(-log(u), P.gev_xi))) / P.gev_xi;
}


// ---------------------------------------------------------------------------------------
// Serial restatements (lane 0): the exact fallbacks of the warp-parallel steps.  They and the
// serial samplers are kept out of line: the epoch loop's code is large enough that, with eight
// or more cells per SM, instruction fetch stalls grow with its size.
// ---------------------------------------------------------------------------------------

// rank_lefs for one direction (simulation.cpp:402-487): split_sort (or pdq_sort at epoch 0)
// by position, then runs of equal positions insertion-sorted by binding epoch (ascending
// for rev units, descending for fwd units).
__device__ __noinline__ void rank_dir_serial(Cell& c, u32 dir, u32 n, bool partially_sorted) {
  u32* R = dir ? c.fr : c.rr;
  const u32* pos = dir ? c.fwd : c.rev;
  const KeyCmp cmp{pos};
  if (partially_sorted) {
    split_sort(R, n, c.tmp, cmp);
  } else {
    pdq_sort(R, 0, n, cmp);
  }
  for (u32 i = 1; i < n; ++i) {
    if (pos[R[i - 1]] == pos[R[i]]) {
      const u32 begin = i - 1;
      for (; i < n; ++i) {
        if (pos[R[i - 1]] != pos[R[i]]) break;
      }
      if (dir) {
        ins_sort(R, begin, i, KeyCmpRev{c.bep});
      } else {
        ins_sort(R, begin, i, KeyCmp{c.bep});
      }
    }
  }
}

// adjust_moves_of_consecutive_extr_units (simulation.cpp:343-399), one direction; lane 0
__device__ __noinline__ void adjust_dir_serial(Cell& c, const KParams& P, u32 dir, u32 n) {
  if (n == 0) return;
  const u64 start = P.start, end = P.end;
  if (dir == 0) {
    for (u32 i = n - 1; i > 0; --i) {
      const u32 i1 = c.rr[i - 1], i2 = c.rr[i];
      if (c.bep[i1] != UNBOUND && c.bep[i2] != UNBOUND) {
        const u64 r1 = pos64(c.rev[i1]), r2 = pos64(c.rev[i2]);
        const u64 m1 = c.rm[i1], m2 = c.rm[i2];
        if (r1 <= start + m1 || r2 <= start + m2) continue;
        const u64 pos1 = r1 - m1, pos2 = r2 - m2;
        if (pos2 <= pos1) c.rm[i1] = (u32)(m1 + (pos1 - pos2) + 1);
      }
    }
  } else {
    for (u32 i = 1; i < n; ++i) {
      const u32 i1 = c.fr[i - 1], i2 = c.fr[i];
      if (c.bep[i1] != UNBOUND && c.bep[i2] != UNBOUND) {
        const u64 f1 = pos64(c.fwd[i1]), f2 = pos64(c.fwd[i2]);
        const u64 m1 = c.fm[i1], m2 = c.fm[i2];
        if (f1 + m1 > end - 1 || f2 + m2 > end - 1) continue;
        const u64 pos1 = f1 + m1, pos2 = f2 + m2;
        if (pos1 >= pos2) c.fm[i2] = (u32)(m2 + (pos1 - pos2) + 1);
      }
    }
  }
}

// compute_lef_lef_collision_pos (simulation.cpp:514-542)
__device__ __forceinline__ void lef_lef_collision_pos(u64 rev_pos, u64 fwd_pos, u64 rev_move,
                                                      u64 fwd_move, u64& p_rev, u64& p_fwd) {
  const u64 rel = rev_move + fwd_move;
  const double t = (double)(rev_pos - fwd_pos) / (double)rel;
  const u64 cp = fwd_pos + (u64)round((double)fwd_move * t);
  if (cp == fwd_pos) {
    p_rev = cp + 1;
    p_fwd = cp;
  } else {
    p_rev = cp;
    p_fwd = cp - 1;
  }
}


// detect_units_at_chrom_boundaries (simulation_detect_collisions.cpp:30-125); lane 0.  The
// loops stop at the first unit that is neither at nor about to reach a chromosome end.
__device__ void detect_boundaries_serial(Cell& c, const KParams& P, u32 n, u64& n5, u64& n3) {
  n5 = 0;
  n3 = 0;
  const u64 start = P.start, end = P.end;
  const u64 first_fwd_pos = pos64(c.fwd[c.fr[0]]);
  u32 last_rev = UNBOUND;
  for (u32 k = n; k > 0; --k) {
    if (c.bep[c.rr[k - 1]] != UNBOUND) {
      last_rev = c.rr[k - 1];
      break;
    }
  }
  if (last_rev == UNBOUND) {
    set_status(c, DEV_ERR_BAD_STATE);
    last_rev = c.rr[0];
  }
  const u64 last_rev_pos = pos64(c.rev[last_rev]);
  for (u32 i = 0; i < n; ++i) {
    const u32 idx = c.rr[i];
    const u64 pos = pos64(c.rev[idx]);
    const u64 mv = c.rm[idx];
    if (pos == start) {
      ++n5;
      c.rc[idx] = cw_make(5, EV_COLLISION | EV_CHROM_BOUNDARY);
    } else if (pos > first_fwd_pos) {
      break;
    } else if (pos - mv == start) {
      c.rc[idx] = cw_make(5, EV_COLLISION | EV_CHROM_BOUNDARY);
      ++n5;
      break;
    }
  }
  for (u32 i = n - 1; i > 0; --i) {
    const u32 idx = c.fr[i];
    const u64 pos = pos64(c.fwd[idx]);
    const u64 mv = c.fm[idx];
    if (c.bep[idx] == UNBOUND) {
      ++n3;
      continue;
    }
    if (pos == end - 1) {
      ++n3;
      c.fc[idx] = cw_make(3, EV_COLLISION | EV_CHROM_BOUNDARY);
    } else if (pos < last_rev_pos) {
      break;
    } else if (pos + mv == end - 1) {
      c.fc[idx] = cw_make(3, EV_COLLISION | EV_CHROM_BOUNDARY);
      ++n3;
      break;
    }
  }
}

__device__ __forceinline__ bool bar_active(const Cell& c, u32 i) { return (c.bst[i >> 5] >> (i & 31)) & 1u; }

// detect_lef_bar_collisions (simulation_detect_collisions.cpp:128-252); lane 0
__device__ __noinline__ void detect_lef_bar_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  u64 j = min(n5, n5 - 1);
  u32 unit_idx = c.rr[j];
  u64 unit_pos = pos64(c.rev[unit_idx]);
  bool rev_done = false;
  for (u32 i = 0; i < c.nb && !rev_done; ++i) {
    if (!bar_active(c, i)) continue;
    const u32 dir = bar_flags(c, i) & BF_DIR_MASK;
    const Trial& tr = P.lef_bar[dir == MGPU_DIR_REV ? 0 : 1];
    const u64 bpos = bar_pos(c, i);
    while (unit_pos <= bpos) {
      if (++j == n) {
        rev_done = true;
        break;
      }
      unit_idx = c.rr[j];
      unit_pos = pos64(c.rev[unit_idx]);
    }
    if (rev_done) break;
    if (c.bep[unit_idx] != UNBOUND) {
      const u64 delta = unit_pos - bpos;
      if (delta > 0 && delta <= c.rm[unit_idx] && s_trial(c, tr)) {
        c.rc[unit_idx] = cw_make(i, EV_COLLISION | EV_LEF_BAR);
      }
    }
  }
  j = n - min(n3, n3 - 1);
  unit_idx = c.fr[--j];
  unit_pos = pos64(c.fwd[unit_idx]);
  for (u64 i = (u64)c.nb - 1; i != ~0ull; --i) {
    if (!bar_active(c, (u32)i)) continue;
    const u32 dir = bar_flags(c, i) & BF_DIR_MASK;
    const Trial& tr = P.lef_bar[dir == MGPU_DIR_FWD ? 0 : 1];
    const u64 bpos = bar_pos(c, i);
    while (unit_pos >= bpos) {
      if (--j == ~0ull) return;
      unit_idx = c.fr[j];
      unit_pos = pos64(c.fwd[unit_idx]);
    }
    if (c.bep[unit_idx] != UNBOUND) {
      const u64 delta = bpos - unit_pos;
      if (delta > 0 && delta <= c.fm[unit_idx] && s_trial(c, tr)) {
        c.fc[unit_idx] = cw_make((u32)i, EV_COLLISION | EV_LEF_BAR);
      }
    }
  }
}

__device__ __forceinline__ u64 barrier_pos_checked(Cell& c, u32 idx) {
  if (idx >= c.nb) {
    set_status(c, DEV_ERR_BAD_STATE);
    return 0;
  }
  return bar_pos(c, idx);
}

// The collision words of one tested primary pair (simulation_detect_collisions.cpp:344-399).
__device__ __forceinline__ void primary_pair_update(Cell& c, u32 rev_idx, u32 fwd_idx, u64 rev_pos,
                                                    u64 fwd_pos, u64 rmv, u64 fmv) {
  u64 cpr, cpf;
  lef_lef_collision_pos(rev_pos, fwd_pos, rmv, fmv, cpr, cpf);
  const u32 rcol = c.rc[rev_idx], fcol = c.fc[fwd_idx];
  if (!cw_occurred(rcol) && !cw_occurred(fcol)) {
    c.rc[rev_idx] = cw_make(fwd_idx, EV_COLLISION | EV_PRIMARY);
    c.fc[fwd_idx] = cw_make(rev_idx, EV_COLLISION | EV_PRIMARY);
  } else if (cw_occurred(rcol) && !cw_occurred(fcol)) {
    const u64 bpos = barrier_pos_checked(c, cw_idx(rcol));
    if (cpf > bpos) {
      c.rc[rev_idx] = cw_make(fwd_idx, EV_COLLISION | EV_PRIMARY);
      c.fc[fwd_idx] = cw_make(rev_idx, EV_COLLISION | EV_PRIMARY);
    } else {
      c.fc[fwd_idx] = cw_make(rev_idx, EV_COLLISION | EV_PRIMARY);
    }
  } else if (!cw_occurred(rcol) && cw_occurred(fcol)) {
    const u64 bpos = barrier_pos_checked(c, cw_idx(fcol));
    c.rc[rev_idx] = cw_make(fwd_idx, EV_COLLISION | EV_PRIMARY);
    if (cpr < bpos) c.fc[fwd_idx] = cw_make(rev_idx, EV_COLLISION | EV_PRIMARY);
  }
}

// detect_primary_lef_lef_collisions (simulation_detect_collisions.cpp:255-401); lane 0
__device__ __noinline__ void detect_primary_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  if (n5 == n || n3 == n) return;
  u64 i1 = 0, j1 = n5;
  const u64 i2 = n - min(n3, n3 - 1);
  const u64 j2 = n;
  for (u64 it = 0; it < 4ull * n + 16; ++it) {
    u32 rev_idx = c.rr[j1];
    u64 rev_pos = pos64(c.rev[rev_idx]);
    u32 fwd_idx = c.fr[i1];
    u64 fwd_pos = pos64(c.fwd[fwd_idx]);
    while (rev_pos <= fwd_pos) {
      if (++j1 == j2) return;
      rev_idx = c.rr[j1];
      rev_pos = pos64(c.rev[rev_idx]);
    }
    while (fwd_pos < rev_pos) {
      if (++i1 == i2) return;
      fwd_idx = c.fr[i1];
      fwd_pos = pos64(c.fwd[fwd_idx]);
    }
    fwd_idx = c.fr[min(i1, i1 - 1)];
    fwd_pos = pos64(c.fwd[fwd_idx]);
    const u64 delta = rev_pos - fwd_pos;
    const u64 rmv = c.rm[rev_idx], fmv = c.fm[fwd_idx];
    if (delta > 0 && delta < rmv + fmv && s_trial(c, P.lef_lef)) {
      primary_pair_update(c, rev_idx, fwd_idx, rev_pos, fwd_pos, rmv, fmv);
    }
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
}

// process_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:404-518); lane 0
__device__ __noinline__ void process_secondary_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  for (u64 i = max((u64)1, n5); i < n; ++i) {
    const u32 idx1 = c.rr[i - 1];
    if (!cw_occurred(c.rc[idx1])) continue;
    const u32 idx2 = c.rr[i];
    if (cw_occurred(c.rc[idx2])) continue;
    const u64 pos1 = pos64(c.rev[idx1]), pos2 = pos64(c.rev[idx2]);
    const u64 move1 = c.rm[idx1], move2 = c.rm[idx2];
    if (pos2 - move2 <= pos1 - move1) {
      if (s_trial(c, P.lef_lef)) {
        c.rc[idx2] = cw_make(idx1, EV_COLLISION | EV_SECONDARY);
        const u64 mv = pos2 - (pos1 - move1);
        c.rm[idx2] = (u32)min(mv, mv - 1);
      } else {
        c.rc[idx2] = cw_make(idx1, EV_SECONDARY);
      }
    }
  }
  u64 i = n - min(n3, n3 - 1) - 1;
  for (; i > 0 && i != ~0ull; --i) {
    const u32 idx2 = c.fr[i];
    if (!cw_occurred(c.fc[idx2])) continue;
    const u32 idx1 = c.fr[i - 1];
    if (cw_occurred(c.fc[idx1])) continue;
    const u64 pos1 = pos64(c.fwd[idx1]), pos2 = pos64(c.fwd[idx2]);
    const u64 move1 = c.fm[idx1], move2 = c.fm[idx2];
    if (pos1 + move1 >= pos2 + move2) {
      if (s_trial(c, P.lef_lef)) {
        c.fc[idx1] = cw_make(idx2, EV_COLLISION | EV_SECONDARY);
        const u64 mv = (pos2 + move2) - pos1;
        c.fm[idx1] = (u32)min(mv, mv - 1);
      } else {
        c.fc[idx1] = cw_make(idx2, EV_SECONDARY);
      }
    }
  }
}

// One rev candidate of fix_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:556-605).
__device__ __forceinline__ void fix_rev_at(Cell& c, u64 start, u64 i) {
  const u32 idx2 = c.rr[i];
  const u32 idx1 = c.rr[i - 1];
  const u64 pos1 = pos64(c.rev[idx1]) - c.rm[idx1];
  const u64 r2 = pos64(c.rev[idx2]);
  c.rm[idx2] = (r2 > pos1 + 1) ? (u32)(r2 - (pos1 + 1)) : 0u;
  c.rc[idx2] = cw_make(idx1, EV_COLLISION | EV_SECONDARY);
  const u64 p1 = pos64(c.rev[idx1]), p2 = r2;
  c.rev[idx1] = (u32)min(pos64(c.fwd[idx1]), p2);
  c.rev[idx2] = (u32)min(pos64(c.fwd[idx2]), p1);
  u32 t = c.rc[idx1];
  c.rc[idx1] = c.rc[idx2];
  c.rc[idx2] = t;
  t = c.rm[idx1];
  c.rm[idx1] = c.rm[idx2];
  c.rm[idx2] = t;
  c.rr[i - 1] = idx2;
  c.rr[i] = idx1;
  c.rm[idx2] = (u32)min(pos64(c.rev[idx2]) - start, (u64)c.rm[idx2]);
  c.rm[idx1] = (u32)min(pos64(c.rev[idx1]) - start, (u64)c.rm[idx1]);
}

// One fwd candidate (simulation_detect_collisions.cpp:608-646).
__device__ __forceinline__ void fix_fwd_at(Cell& c, u64 end, u64 i) {
  const u32 idx1 = c.fr[i];
  const u32 idx2 = c.fr[i + 1];
  const u64 f1 = pos64(c.fwd[idx1]);
  const u64 pos2 = pos64(c.fwd[idx2]) + c.fm[idx2];
  c.fm[idx1] = (pos2 > f1 + 1) ? (u32)(pos2 - (f1 + 1)) : 0u;
  c.fc[idx1] = cw_make(idx2, EV_COLLISION | EV_SECONDARY);
  const u64 p1 = f1, p2 = pos64(c.fwd[idx2]);
  c.fwd[idx1] = (u32)max(pos64(c.rev[idx1]), p2);
  c.fwd[idx2] = (u32)max(pos64(c.rev[idx2]), p1);
  u32 t = c.fc[idx1];
  c.fc[idx1] = c.fc[idx2];
  c.fc[idx2] = t;
  t = c.fm[idx1];
  c.fm[idx1] = c.fm[idx2];
  c.fm[idx2] = t;
  c.fr[i] = idx2;
  c.fr[i + 1] = idx1;
  c.fm[idx2] = (u32)min(end - 1 - pos64(c.fwd[idx2]), (u64)c.fm[idx2]);
  c.fm[idx1] = (u32)min(end - 1 - pos64(c.fwd[idx1]), (u64)c.fm[idx1]);
}

// fix_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:520-647); lane 0
__device__ __noinline__ void fix_secondary_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  const u64 num_active_fwd = n - min(n3, n3 - 1);
  for (u64 i = max((u64)1, n5); i < n; ++i) {
    if (cw_avoided_as(c.rc[c.rr[i]], EV_SECONDARY)) fix_rev_at(c, P.start, i);
  }
  for (u64 i = 0; i + 1 < num_active_fwd; ++i) {
    if (cw_avoided_as(c.fc[c.fr[i]], EV_SECONDARY)) fix_fwd_at(c, P.end, i);
  }
}


// ---------------------------------------------------------------------------------------
// Warp-parallel steps (all 32 lanes, uniform control flow)
// ---------------------------------------------------------------------------------------

// ExtrusionBarriers::init_states (extrusion_barriers.cpp:220-231)
__device__ void barriers_init(Cell& c, u64* s) {
  for (u32 base = 0; base < c.nb; base += 32) {
    rng_ensure(c, s, 32);
    const u32 i = base + ln();
    const bool need = i < c.nb && (bar_flags(c, i) & BF_OCC_DRAWS);
    const unsigned m = __ballot_sync(FULL, need);
    const u32 off = __popc(m & lanemask_lt());
    bool occ = false;
    if (need) occ = ring_at(c, c.sc->rpos + off) <= c.bar[i].t_occ;
    const unsigned om = __ballot_sync(FULL, occ);
    __syncwarp();
    if (ln() == 0) {
      c.bst[base >> 5] = om;
      c.sc->rpos += __popc(m);
    }
    __syncwarp();
  }
}

// ExtrusionBarriers::next_state (extrusion_barriers.cpp:145-161): one draw per barrier.
__device__ void barriers_next(Cell& c, u64* s) {
  const u32 nwords = (c.nb + 31) / 32;
  for (u32 base = 0; base < c.nb; base += 32 * MLP) {
    rng_ensure(c, s, 32 * MLP);
    const u64 r0 = c.sc->rpos;
    u32 word[MLP], f[MLP];
    u64 thr[MLP], u[MLP];
    bool st[MLP], valid[MLP];
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) {
      const u32 i = base + 32 * h + ln();
      valid[h] = i < c.nb;
      const u32 w = (base >> 5) + h;
      word[h] = w < nwords ? c.bst[w] : 0u;
      st[h] = (word[h] >> ln()) & 1u;
      const u32 ic = valid[h] ? i : 0u;
      f[h] = bar_flags(c, ic);
      thr[h] = st[h] ? c.bar[ic].t_act : c.bar[ic].t_ina;
      u[h] = ring_at(c, r0 + 32 * h + ln());
    }
    unsigned nm[MLP];
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) {
      bool nst = st[h];
      if (valid[h]) {
        if (!st[h]) {
          nst = !(f[h] & BF_INA_NEVER) && u[h] >= thr[h];
        } else {
          nst = !(!(f[h] & BF_ACT_NEVER) && u[h] >= thr[h]);
        }
      }
      nm[h] = __ballot_sync(FULL, valid[h] && nst);
    }
    __syncwarp();
    if (ln() == 0) {
#pragma unroll
      for (u32 h = 0; h < MLP; ++h)
        if ((base >> 5) + h < nwords) c.bst[(base >> 5) + h] = nm[h];
      c.sc->rpos = r0 + min(32u * MLP, c.nb - base);
    }
    __syncwarp();
  }
}

// select_lefs_to_bind + bind_lefs (simulation_impl.hpp:28-89): one uniform_int draw per
// selected LEF in index order.  Selection: mode 0 = unbound LEFs (the epoch loop), 1 =
// nonzero entries of mask, 2 = every LEF (an empty mask in the reference).
__device__ __forceinline__ bool bind_selected(const Cell& c, u32 i, int mode, const u64* mask) {
  return mode == 0 ? c.bep[i] == UNBOUND : (mode == 1 ? mask[i] != 0 : true);
}

__device__ void bind_lefs(Cell& c, u64* s, const KParams& P, u32 n, u32 epoch, int mode,
                          const u64* mask) {
  for (u32 i0 = 0; i0 < n; i0 += 32) {
    rng_ensure(c, s, 32);
    const u32 i = i0 + ln();
    const bool need = i < n && bind_selected(c, i, mode, mask);
    const unsigned m = __ballot_sync(FULL, need);
    const u32 off = __popc(m & lanemask_lt());
    u64 r = 0;
    bool ok = true;
    if (need) {
      r = ring_at(c, c.sc->rpos + off) / P.pos_bucket;
      ok = r <= P.pos_range;
    }
    const unsigned bad = __ballot_sync(FULL, need && !ok);
    const u32 f = bad ? (u32)(__ffs(bad) - 1) : 32u;
    if (need && ln() < f) {
      const u32 pos = (u32)(P.wstart + r);
      c.rev[i] = pos;
      c.fwd[i] = pos;
      c.bep[i] = epoch;
    }
    __syncwarp();
    if (ln() == 0) {
      c.sc->rpos += __popc(m & (f == 32 ? FULL : ((1u << f) - 1)));
      if (f < 32) {  // finish this chunk serially from the rejecting LEF
        for (u32 k = i0 + f; k < min(i0 + 32, n); ++k) {
          if (!bind_selected(c, k, mode, mask)) continue;
          const u64 pos = s_uniform_int(c, P.wstart, (u64)P.wend - 1);
          c.rev[k] = (u32)pos;
          c.fwd[k] = (u32)pos;
          c.bep[k] = epoch;
        }
      }
    }
    __syncwarp();
  }
}

// Ranking key of a unit: position, then binding epoch ascending (rev) or descending (fwd).
__device__ __forceinline__ u64 rank_key(const Cell& c, u32 dir, u32 idx) {
  const u32 p = dir ? c.fwd[idx] : c.rev[idx];
  const u32 e = dir ? ~c.bep[idx] : c.bep[idx];
  return ((u64)p << 32) | e;
}

// Warp bitonic sort of the index block a[0..m) by the 64-bit keys hi[k] << 32 | lo[k] stored
// beside it (a, hi and lo move together).  Only ascending comparators are used (each merge
// starts by comparing mirror pairs), so the virtual +inf padding up to a power of two never
// moves and needs no storage.  Block sizes and strides are powers of two, so the comparator
// indexes are shifts and masks.
__device__ void bitonic_keyed(u32* a, u32* hi, u32* lo, u32 m) {
  u32 lg = 0;
  while ((1u << lg) < m) ++lg;
  const u32 ncmp = (1u << lg) >> 1;  // comparators per stage
  auto cmpx = [&](u32 i, u32 j) {
    if (j >= m) return;
    const u64 ki = ((u64)hi[i] << 32) | lo[i], kj = ((u64)hi[j] << 32) | lo[j];
    if (ki > kj) {
      hi[i] = (u32)(kj >> 32);
      lo[i] = (u32)kj;
      hi[j] = (u32)(ki >> 32);
      lo[j] = (u32)ki;
      const u32 x = a[i];
      a[i] = a[j];
      a[j] = x;
    }
  };
  for (u32 s = 1; s <= lg; ++s) {
    // merge into sorted blocks of 2^s: mirror pairs, then strides 2^(s-2) .. 1
    for (u32 t = ln(); t < ncmp; t += 32) {
      const u32 base = (t >> (s - 1)) << s, off = t & ((1u << (s - 1)) - 1u);
      cmpx(base + off, base + (1u << s) - 1u - off);
    }
    __syncwarp();
    for (int q = (int)s - 2; q >= 0; --q) {
      for (u32 t = ln(); t < ncmp; t += 32) {
        const u32 i = ((t >> q) << (q + 1)) | (t & ((1u << q) - 1u));
        cmpx(i, i + (1u << q));
      }
      __syncwarp();
    }
  }
}

// Lane 0: insertion-sort the run of equal positions around a[t-1], a[t] by binding epoch
// (ascending for rev units, descending for fwd units), as the tie fix of rank_lefs does
// (simulation.cpp:446-485).  Returns the end of the run.
__device__ __noinline__ u32 tie_fix_run(const Cell& c, u32 dir, u32* a, u32 t, u32 len) {
  const u32* pos = dir ? c.fwd : c.rev;
  const u32 p = pos[a[t]];
  u32 lo = t - 1, hi = t + 1;
  while (lo > 0 && pos[a[lo - 1]] == p) --lo;
  while (hi < len && pos[a[hi]] == p) ++hi;
  if (dir) {
    ins_sort(a, lo, hi, KeyCmpRev{c.bep});
  } else {
    ins_sort(a, lo, hi, KeyCmp{c.bep});
  }
  return hi;
}

// rank_lefs for one direction when the previous order is reused (split_sort,
// simulation.cpp:427-435, then the tie fix :446-485), warp-parallel and exact.
//
// split_sort makes one pass that keeps a non-decreasing stack K of the input (a smaller
// element pops the stack top and both leave), pdq-sorts the removed elements B in the order the
// pass's swaps leave them, and merges K and B stably.  The tie fix then orders runs of equal
// positions by binding epoch.  The result is the stable sort of K followed by B by the key
// (position, epoch): the order is unique except among full ties (equal position and epoch),
// which keep K's order, then B's order after pdq_sort.
//
// Here the pass runs 32 elements at a time: the lanes up to the first one below its
// predecessor (or below the stack top) are pushed together, and each pop is an event.  The
// removed block only changes by events (top prepended, reader appended) and by pushes (each
// rotates it left by one), so every removed element's final slot follows from the event list.
// B is sorted by key with a warp bitonic sort; only if B holds full ties is it pdq-sorted
// exactly on lane 0.  Returns false (R untouched) for n < 2 or n > 65535.
//
// Scratch: the stack K in sr, the input positions and later B in tmp, and the event lists in
// rm, fm and sf.  The move arrays are dead from binding until the moves are generated (the
// callers that keep them restore them), and every event removes one input element, so n
// entries per list always suffice.
__device__ bool rank_dir_split(Cell& c, u32 dir, u32 n) {
  if (n < 2 || n > 0xFFFFu) return false;
  u32* R = dir ? c.fr : c.rr;
  const u32* pos = dir ? c.fwd : c.rev;
  u32* K = c.sr;
  const u32 EMAX = n;
  u32* ev_q = c.rm;  // pushes since the previous event; later (q mod k_prev) | k_prev << 16
  u32* ev_top = c.fm;
  u32* ev_rd = c.sf;
  u32* B = c.tmp;
  const u32 lane = ln();
  u64 tprof = clock64();
  // positions in input order, gathered up front with independent loads (B is written to tmp
  // only after the pass)
  {
    const u32* __restrict__ Rr = R;
    const u32* __restrict__ pr = pos;
    u32* __restrict__ V = c.tmp;
#pragma unroll 4
    for (u32 r = lane; r < n; r += 32) V[r] = pr[Rr[r]];
  }
  __syncwarp();
  const u32* V = c.tmp;
  const u32 first = R[0];
  if (lane == 0) K[0] = first;
  u32 m = 0, T = V[0], E = 0, q = 0;
  for (u32 base = 1; base < n; base += 32) {
    const u32 r = base + lane;
    const u32 nvalid = min(32u, n - base);
    const bool valid = lane < nvalid;
    const u32 idx = valid ? R[r] : 0;
    const u32 v = valid ? V[r] : 0;
    const u32 vprev = __shfl_up_sync(FULL, v, 1);
    const bool pre_ok = lane == 0 || v >= vprev;
    u32 start = 0;
    while (start < nvalid) {
      const bool ok = lane == start ? v >= T : pre_ok;
      const unsigned fail = __ballot_sync(FULL, !ok && lane >= start && valid);
      const u32 f = fail ? (u32)(__ffs(fail) - 1) : nvalid;
      if (lane >= start && lane < f) K[m + 1 + lane - start] = idx;
      if (f > start) {
        m += f - start;
        if (E) q += f - start;
        T = __shfl_sync(FULL, v, f - 1);
      }
      if (f == nvalid) break;
      const u32 rd = __shfl_sync(FULL, idx, f);
      if (E >= EMAX) return false;
      __syncwarp();
      u32 top = UNBOUND;
      if (m > 0) {
        top = K[m];
        --m;
        T = pos[K[m]];
      }
      if (lane == 0) {
        ev_q[E] = q;
        ev_top[E] = top;
        ev_rd[E] = rd;
      }
      ++E;
      q = 0;
      start = f + 1;
    }
  }
  __syncwarp();
  {
    const u64 t = clock64();
    prof_add(c, PF_RANK_PASS, t - tprof);
    tprof = t;
  }
  const u32 ns = m + 1;
  // block size before each event, and the rotation it saw since the previous event
  u32 kacc = 0;
  for (u32 b = 0; b < E; b += 32) {
    const u32 j = b + lane;
    const bool vj = j < E;
    const u32 sz = vj ? (ev_top[j] != UNBOUND ? 2u : 1u) : 0u;
    u32 tot;
    const u32 ex = warp_excl_scan(sz, &tot);
    if (vj) {
      const u32 kprev = kacc + ex;
      const u32 qm = kprev ? ev_q[j] % kprev : 0u;
      ev_q[j] = qm | (kprev << 16);
    }
    kacc += tot;
  }
  const u32 kE = kacc;
  __syncwarp();
  // final slot of every removed element
  const u32 qfm = kE ? q % kE : 0u;
  for (u32 b = 0; b < E; b += 32) {
    const u32 j = b + lane;
    const bool vj = j < E;
    const u32 top = vj ? ev_top[j] : UNBOUND;
    const u32 rd = vj ? ev_rd[j] : 0u;
    const u32 kj = vj ? (ev_q[j] >> 16) + (top != UNBOUND ? 2u : 1u) : 1u;
    u32 it = 0, ir = kj - 1;
    for (u32 jj = b + 1; jj < E; ++jj) {
      const u32 w = ev_q[jj];
      const bool pop = ev_top[jj] != UNBOUND;
      if (jj > j) {
        const u32 qm = w & 0xFFFFu, kk = w >> 16;
        it = it >= qm ? it - qm : it + kk - qm;
        ir = ir >= qm ? ir - qm : ir + kk - qm;
        if (pop) {
          ++it;
          ++ir;
        }
      }
    }
    it = it >= qfm ? it - qfm : it + kE - qfm;
    ir = ir >= qfm ? ir - qfm : ir + kE - qfm;
    if (vj) {
      if (top != UNBOUND) B[it] = top;
      B[ir] = rd;
    }
  }
  __syncwarp();
  // sort B by key (the events are dead: sf, rm and fm are free); the keys are loaded once and
  // sorted alongside the indices, so the network compares values already in memory.  Measured
  // on the genome workload, sorting every block this way beats handing large blocks (or, as
  // split_sort's event list once had to, whole ranks) to lane 0's serial sorts.
  u32* Bs = c.sf;
  u32* Kh = c.rm;  // position
  u32* Kl = c.fm;  // binding epoch (complemented for fwd units)
  bool full_tie = false;
  for (u32 t = lane; t < kE; t += 32) {
    const u32 idx = B[t];
    const u64 k = rank_key(c, dir, idx);
    Bs[t] = idx;
    Kh[t] = (u32)(k >> 32);
    Kl[t] = (u32)k;
  }
  __syncwarp();
  bitonic_keyed(Bs, Kh, Kl, kE);
  for (u32 t = lane + 1; t < kE; t += 32) full_tie |= Kh[t - 1] == Kh[t] && Kl[t - 1] == Kl[t];
  const u32* Bf = Bs;
  if (__any_sync(FULL, full_tie)) {
    prof_add(c, PF_RANK_PDQ, 1);
    if (lane == 0) {
      pdq_sort(B, 0, kE, KeyCmp{pos});
      for (u32 t = 1; t < kE; ++t) {
        if (pos[B[t - 1]] == pos[B[t]]) t = tie_fix_run(c, dir, B, t, kE);
      }
    }
    __syncwarp();
    Bf = B;
  }
  {
    const u64 t = clock64();
    prof_add(c, PF_RANK_BLOCK, t - tprof);
    tprof = t;
  }
  // tie fix of K: runs of equal positions whose epochs are out of order (each element's key is
  // read once; the previous element's comes from the adjacent lane or the previous chunk)
  u64 kprev = ns ? rank_key(c, dir, K[0]) : 0;
  for (u32 base = 1; base < ns; base += 32) {
    const u32 t = base + lane;
    const u64 kt = t < ns ? rank_key(c, dir, K[t]) : ~0ull;
    u64 k0 = __shfl_up_sync(FULL, kt, 1);
    if (lane == 0) k0 = kprev;
    kprev = __shfl_sync(FULL, kt, 31);
    const bool bad = t < ns && (k0 >> 32) == (kt >> 32) && k0 > kt;
    unsigned bm = __ballot_sync(FULL, bad);
    if (bm) {
      if (lane == 0) {
        while (bm) {
          const u32 t0 = base + (u32)(__ffs(bm) - 1);
          const u32 hi = tie_fix_run(c, dir, K, t0, ns);
          const u32 last = hi - 1 - base;  // bits up to the run's end are done
          bm = last >= 31 ? 0u : bm & ~((2u << last) - 1u);
        }
      }
      __syncwarp();
      // a fixed run may reach the chunk's end: carry the key now at its last slot
      const u32 tl = min(base + 31, ns - 1);
      kprev = rank_key(c, dir, K[tl]);
    }
  }
  // merge, K first among equal keys.  u_j = #K with key <= key(B_j) (binary search; K is
  // sorted by key), so B_j lands at j + u_j and K_i at i + #{j : u_j <= i}; u is
  // non-decreasing in j, so one pass over K with a pointer into u counts the latter.
  u32* U = Bf == Bs ? B : Bs;  // the dead one of the two B buffers
  for (u32 j = lane; j < kE; j += 32) {
    const u32 idx = Bf[j];
    const u64 key = rank_key(c, dir, idx);
    u32 lo = 0, hi = ns;
    while (lo < hi) {
      const u32 mid = (lo + hi) >> 1;
      if (rank_key(c, dir, K[mid]) <= key) lo = mid + 1; else hi = mid;
    }
    U[j] = lo;
    R[j + lo] = idx;
  }
  __syncwarp();
  u32 jb = 0;  // B elements with u_j below the chunk
  for (u32 base = 0; base < ns; base += 32) {
    const u32 i = base + lane;
    u32 cnt = jb, j = jb;
    for (; j < kE; ++j) {
      const u32 uj = U[j];
      if (uj >= base + 32) break;
      cnt += uj <= i ? 1u : 0u;
    }
    if (i < ns) R[i + cnt] = K[i];
    jb = j;
  }
  __syncwarp();
  prof_add(c, PF_RANK_MERGE, clock64() - tprof);
  return true;
}

__device__ void rank_lefs(Cell& c, const KParams& P, u32 n, u32 epoch, bool partially_sorted) {
  for (u32 dir = 0; dir < 2; ++dir) {
    const bool ok = partially_sorted && !(P.debug_flags & DBG_SERIAL_RANK) && rank_dir_split(c, dir, n);
    if (!ok) {
      const u64 t0 = clock64();
      prof_add(c, PF_RANK_FALLBACK, 1);
      if (ln() == 0) {
        rank_dir_serial(c, dir, n, partially_sorted);
        c.sc->sort_fallbacks++;
      }
      __syncwarp();
      prof_add(c, PF_RANK_SERIAL, clock64() - t0);
    }
  }
}

// positions in rank order: sr[k] = rev[rr[k]], sf[k] = fwd[fr[k]]
__device__ void gather_ranked(Cell& c, u32 n) {
  const u32* __restrict__ rr = c.rr;
  const u32* __restrict__ fr = c.fr;
  const u32* __restrict__ rev = c.rev;
  const u32* __restrict__ fwd = c.fwd;
  u32* __restrict__ sr = c.sr;
  u32* __restrict__ sf = c.sf;
#pragma unroll 4
  for (u32 k = ln(); k < n; k += 32) {
    sr[k] = rev[rr[k]];
    sf[k] = fwd[fr[k]];
  }
  __syncwarp();
}

// generate_moves_helper (simulation.cpp:264-290) for one direction: move = round(max(0,
// normal(mean, sd))) for every bound LEF in index order, unbound ones get 0.
//
// The normals are variable-length (a ziggurat wedge takes a second draw, the tail takes
// exponentials), so the warp evaluates a window of 32 candidate starts at once: lane k runs the
// whole sampler as if a normal started at stream position rpos + k.  The real starts form the
// chain s0 = 0, s(j+1) = s(j) + len(s(j)); lane j finds s(j) by binary lifting over the
// lanes' next-start pointers.  A window serves the normals whose start lies inside it (31 or
// 32 of them in the common case), in stream order, to the next LEFs in index order.
// Kept out of line: inlined into the epoch loop it shares the kernel's register allocation,
// and the batched genome launch took 13 % longer that way.
__device__ __noinline__ void gen_moves_dir(Cell& c, u64* s, u32* mv, u32 n, double mean, double sd, u64 move_int) {
  if (sd == 0.0) {
    for (u32 i = ln(); i < n; i += 32) mv[i] = c.bep[i] == UNBOUND ? 0u : (u32)move_int;
    __syncwarp();
    return;
  }
  // items: the bound LEFs in index order (a compacted list only when some are unbound)
  u32 nb = 0;
  for (u32 base = 0; base < n; base += 32) {
    const u32 i = base + ln();
    const bool need = i < n && c.bep[i] != UNBOUND;
    const unsigned m = __ballot_sync(FULL, need);
    if (i < n && !need) mv[i] = 0;
    if (need) c.tmp[nb + __popc(m & lanemask_lt())] = i;
    nb += __popc(m);
  }
  const bool all = nb == n;
  __syncwarp();
  u32 t0 = 0;
  while (t0 < nb) {
    rng_ensure(c, s, 96);
    const u64 r0 = c.sc->rpos;
    RingSrc g{c.ring, r0 + ln(), c.sc->gpos, 0};
    double z = 0.0;
    const int st = unit_normal_t(g, z);
    const u32 len = g.n;
    // next-start pointers: 32 = beyond the window, 33 = unknown (the sampler ran dry)
    u32 J[5];
    J[0] = st == SMP_OK ? min(ln() + len, 32u) : 33u;
#pragma unroll
    for (int b = 1; b < 5; ++b) {
      const u32 prev = J[b - 1];
      const u32 v = __shfl_sync(FULL, prev, prev < 32 ? prev : 0);
      J[b] = prev < 32 ? v : prev;
    }
    u32 p = 0;  // start of the ln()-th normal of the window
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      const u32 v = __shfl_sync(FULL, J[b], p < 32 ? p : 0);
      if (((ln() >> b) & 1) && p < 32) p = v;
    }
    // the ln()-th normal is usable when it starts inside the window and its sampler finished
    const u32 jn = __shfl_sync(FULL, J[0], p < 32 ? p : 0);
    const u32 m = __popc(__ballot_sync(FULL, p < 32 && jn != 33u));
    const u32 served = min(m, nb - t0);
    if (served == 0) {
      // the first normal needs more draws than the ring holds: take it serially
      if (ln() == 0) {
        const double zz = s_unit_normal(c);
        const double v = round(fmax(0.0, zz * sd + mean));
        if (v > 4294967295.0) set_status(c, DEV_ERR_MOVE_RANGE);
        mv[all ? t0 : c.tmp[t0]] = (u32)(u64)v;
      }
      __syncwarp();
      ++t0;
      continue;
    }
    const double zj = __shfl_sync(FULL, z, p < 32 ? p : 0);
    if (ln() < served) {
      const double v = round(fmax(0.0, zj * sd + mean));
      if (v > 4294967295.0) set_status(c, DEV_ERR_MOVE_RANGE);
      mv[all ? t0 + ln() : c.tmp[t0 + ln()]] = (u32)(u64)v;
    }
    const u32 plast = __shfl_sync(FULL, p, served - 1);
    const u32 llast = __shfl_sync(FULL, len, plast);
    __syncwarp();
    if (ln() == 0) c.sc->rpos = r0 + plast + llast;
    __syncwarp();
    t0 += served;
  }
}

// adjust_moves_of_consecutive_extr_units, rev units: pairs (k, k+1) from the top rank down.
// With t_k = pos_k - move_k the reference computes T_k = min(t_k, T_{k+1} - 1) when the pair
// links (both bound, t_k > start, T_{k+1} > start), else T_k = t_k.  In U_k = T_k - k this is
// a segmented suffix minimum.  The scan takes the static part of the link condition; the
// dynamic part (T_{k+1} > start) is checked afterwards and a failure anywhere rejects the
// result (serial fallback).  New moves go to tmp first and are copied only on success.
__device__ bool adjust_rev_fast(Cell& c, const KParams& P, u32 n) {
  const i64 start = P.start;
  u32* out = c.tmp;
  i64 carry_u = 0;       // U of element kb + 32
  bool carry_b = false;  // bound flag of element kb + 32
  bool bad = false;
  {
  // the chunk below is loaded while this one is scanned (the scan writes only tmp)
  const u32* __restrict__ rr = c.rr;
  const u32* __restrict__ sr = c.sr;
  const u32* __restrict__ bep = c.bep;
  const u32* __restrict__ rm = c.rm;
  i64 kb = ((i64)n - 1) / 32 * 32;
  u32 idx_n = 0, sp_n = 0, be_n = UNBOUND, m_n = 0;
  {
    const i64 k = kb + ln();
    const bool valid = k < (i64)n;
    idx_n = valid ? rr[k] : 0u;
    sp_n = valid ? sr[k] : 0u;
    be_n = valid ? bep[idx_n] : UNBOUND;
    m_n = valid ? rm[idx_n] : 0u;
  }
  for (; kb >= 0; kb -= 32) {
    const i64 k = kb + ln();
    const bool valid = k < (i64)n;
    const bool b = valid && be_n != UNBOUND;
    const i64 p = valid ? (i64)sp_n : 0;
    const i64 t = valid ? p - (i64)m_n : 0;
    if (kb >= 32) {
      const i64 k2 = kb - 32 + ln();
      idx_n = rr[k2];
      sp_n = sr[k2];
      be_n = bep[idx_n];
      m_n = rm[idx_n];
    }
    bool b_next = __shfl_down_sync(FULL, b, 1);
    if (ln() == 31) b_next = carry_b;
    const bool link_next = valid && k + 1 < (i64)n && b && b_next && t > start;
    i64 v = t - k;
    bool stop = !link_next;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const i64 vr = __shfl_down_sync(FULL, v, d);
      const bool sr_ = __shfl_down_sync(FULL, stop, d);
      if ((int)ln() + d < 32 && !stop) {
        v = min(v, vr);
        stop = sr_;
      }
    }
    if (valid && !stop) v = min(v, carry_u);  // linked through lane 31 to element kb + 32
    const i64 T = v + k;
    i64 T_next = __shfl_down_sync(FULL, T, 1);
    if (ln() == 31) T_next = carry_u + kb + 32;
    if (link_next && T_next <= start) bad = true;  // the reference would skip this pair
    if (valid) out[k] = (u32)(p - T);
    carry_u = __shfl_sync(FULL, v, 0);
    carry_b = __shfl_sync(FULL, b, 0);
  }
  }
  if (__any_sync(FULL, bad)) return false;
  __syncwarp();
#pragma unroll 4
  for (u32 k = ln(); k < n; k += 32) c.rm[c.rr[k]] = out[k];
  __syncwarp();
  return true;
}

// fwd units: pairs (k-1, k) from the bottom rank up; T_k = max(t_k, T_{k-1} + 1) when linked
// (both bound, t_k <= end - 1, T_{k-1} <= end - 1); V_k = T_k - k is a segmented prefix max.
__device__ bool adjust_fwd_fast(Cell& c, const KParams& P, u32 n) {
  const i64 endm1 = (i64)P.end - 1;
  u32* out = c.tmp;
  i64 carry_v = 0;       // V of element kb - 1
  bool carry_b = false;  // bound flag of element kb - 1
  bool bad = false;
  {
  // the next chunk is loaded while this one is scanned (the scan writes only tmp)
  const u32* __restrict__ fr = c.fr;
  const u32* __restrict__ sf = c.sf;
  const u32* __restrict__ bep = c.bep;
  const u32* __restrict__ fm = c.fm;
  u32 idx_n = 0, sp_n = 0, be_n = UNBOUND, m_n = 0;
  if (ln() < n) {
    idx_n = fr[ln()];
    sp_n = sf[ln()];
    be_n = bep[idx_n];
    m_n = fm[idx_n];
  }
  for (u32 kb = 0; kb < n; kb += 32) {
    const i64 k = (i64)kb + ln();
    const bool valid = k < (i64)n;
    const bool b = valid && be_n != UNBOUND;
    const i64 p = valid ? (i64)sp_n : 0;
    const i64 t = valid ? p + (i64)m_n : 0;
    {
      const u32 k2 = kb + 32 + ln();
      if (k2 < n) {
        idx_n = fr[k2];
        sp_n = sf[k2];
        be_n = bep[idx_n];
        m_n = fm[idx_n];
      }
    }
    bool b_prev = __shfl_up_sync(FULL, b, 1);
    if (ln() == 0) b_prev = carry_b;
    const bool link_prev = valid && k > 0 && b && b_prev && t <= endm1;
    i64 v = t - k;
    bool stop = !link_prev;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const i64 vl = __shfl_up_sync(FULL, v, d);
      const bool sl = __shfl_up_sync(FULL, stop, d);
      if ((int)ln() >= d && !stop) {
        v = max(v, vl);
        stop = sl;
      }
    }
    if (valid && !stop) v = max(v, carry_v);  // linked through lane 0 to element kb - 1
    const i64 T = v + k;
    i64 T_prev = __shfl_up_sync(FULL, T, 1);
    if (ln() == 0) T_prev = carry_v + (i64)kb - 1;
    if (link_prev && T_prev > endm1) bad = true;
    if (valid) out[k] = (u32)(T - p);
    carry_v = __shfl_sync(FULL, v, 31);
    carry_b = __shfl_sync(FULL, b, 31);
  }
  }
  if (__any_sync(FULL, bad)) return false;
  __syncwarp();
#pragma unroll 4
  for (u32 k = ln(); k < n; k += 32) c.fm[c.fr[k]] = out[k];
  __syncwarp();
  return true;
}

__device__ void adjust_moves(Cell& c, const KParams& P, u32 n) {
  const bool serial = P.debug_flags & DBG_SERIAL_ADJUST;
  if (serial || !adjust_rev_fast(c, P, n)) {
    prof_add(c, PF_ADJUST_FALLBACK, 1);
    if (ln() == 0) adjust_dir_serial(c, P, 0, n);
    __syncwarp();
  }
  if (serial || !adjust_fwd_fast(c, P, n)) {
    prof_add(c, PF_ADJUST_FALLBACK, 1);
    if (ln() == 0) adjust_dir_serial(c, P, 1, n);
    __syncwarp();
  }
}

// clamp_moves (simulation.cpp:325-340)
__device__ void clamp_moves(Cell& c, const KParams& P, u32 n) {
  const u32* __restrict__ bep = c.bep;
  const u32* __restrict__ rev = c.rev;
  const u32* __restrict__ fwd = c.fwd;
  u32* __restrict__ rm = c.rm;
  u32* __restrict__ fm = c.fm;
  const u64 start = P.start, end = P.end;
#pragma unroll 4
  for (u32 i = ln(); i < n; i += 32) {
    if (bep[i] == UNBOUND) continue;
    const u64 rmv = min((u64)rm[i], pos64(rev[i]) - start);
    const u64 fmv = min((u64)fm[i], end - pos64(fwd[i]) - 1);
    rm[i] = (u32)rmv;
    fm[i] = (u32)fmv;
  }
  __syncwarp();
}

// ranked positions sorted (non-decreasing)?  Needed by the closed forms below; the epoch loop
// always satisfies it, caller-provided ranks may not.
__device__ bool ranked_sorted(const Cell& c, u32 n) {
  bool bad = false;
  u32 pr = 0, pf = 0;  // last values of the previous chunk
  for (u32 base = 0; base < n; base += 32) {
    const u32 k = base + ln();
    const u32 r = k < n ? c.sr[k] : UNBOUND, f = k < n ? c.sf[k] : UNBOUND;
    u32 r0 = __shfl_up_sync(FULL, r, 1), f0 = __shfl_up_sync(FULL, f, 1);
    if (ln() == 0) {
      r0 = pr;
      f0 = pf;
    }
    if (k < n && k > 0 && (r0 > r || f0 > f)) bad = true;
    pr = __shfl_sync(FULL, r, 31);
    pf = __shfl_sync(FULL, f, 31);
  }
  return !__any_sync(FULL, bad);
}

// Bucket index over a sorted array of ranked positions (unbound units, UNBOUND, at the tail):
// T[b] = #{k : key[k] < start + (b << shift)} for b in [0, nbk], with shift chosen so that
// nbk + 1 <= n (about one key per bucket).  lower_bound(x) then starts from T[b(x)] and scans a
// few keys instead of a binary search over the whole array.
struct BucketIndex {
  const u32* key;
  const u32* T;
  u32 n, start, shift, nbk;
  __device__ u32 lower_bound(u32 x) const {
    if (x <= start) return 0;
    u32 b = (x - start) >> shift;
    if (b > nbk) b = nbk;
    u32 k = T[b];
    while (k < n && key[k] < x) ++k;
    return k;
  }
};

// Collective; T needs n entries.  Returns an index with T == nullptr (binary-search fallback)
// when n is too small for a table.
__device__ BucketIndex build_bucket_index(const u32* key, u32 n, u32 start, u32 end, u32* T) {
  BucketIndex ix{key, nullptr, n, start, 0, 0};
  if (n < 8 || end <= start) return ix;
  const u32 range = end - start;
  u32 shift = 0;
  while ((range >> shift) + 2 > n) ++shift;
  const u32 nbk = range >> shift;
  for (u32 k = ln(); k <= n; k += 32) {
    u32 bmin = 0, bmax = nbk;
    if (k > 0) {
      const u32 lo = key[k - 1];
      bmin = lo == UNBOUND ? nbk + 1 : ((lo - start) >> shift) + 1;
    }
    if (k < n) {
      const u32 hi = key[k];
      if (hi != UNBOUND) bmax = min(nbk, (hi - start) >> shift);
    }
    for (u32 b = bmin; b <= bmax; ++b) T[b] = k;
  }
  __syncwarp();
  ix.T = T;
  ix.shift = shift;
  ix.nbk = nbk;
  return ix;
}

// first k in [0, n) with key[k] >= x
__device__ __forceinline__ u32 ranked_lower_bound(const BucketIndex& ix, u32 x) {
  if (ix.T) return ix.lower_bound(x);
  u32 lo = 0, hi = ix.n;
  while (lo < hi) {
    const u32 mid = (lo + hi) >> 1;
    if (ix.key[mid] >= x) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Bernoulli trial of one lane with the draw at its offset (or none).
__device__ __forceinline__ bool trial_needs_draw(const Trial& t) { return !t.always && t.draws; }
__device__ __forceinline__ bool trial_outcome(const Trial& t, u64 u) {
  if (t.always) return true;
  if (!t.draws) return false;
  return u <= t.thr;
}

// ranked_lower_bound of MLP queries at once: the bucket loads and the scans of all queries are
// issued together.
__device__ __forceinline__ void ranked_lower_bounds(const BucketIndex& ix, const u32* x, u32* out) {
  if (!ix.T) {
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) out[h] = ranked_lower_bound(ix, x[h]);
    return;
  }
#pragma unroll
  for (u32 h = 0; h < MLP; ++h) {
    const u32 b = x[h] <= ix.start ? 0u : min((x[h] - ix.start) >> ix.shift, ix.nbk);
    out[h] = x[h] <= ix.start ? 0u : ix.T[b];
  }
  for (;;) {
    bool more = false;
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) {
      const bool a = out[h] < ix.n && ix.key[out[h]] < x[h];
      out[h] += a ? 1u : 0u;
      more |= a;
    }
    if (!more) break;
  }
}

// detect_lef_bar_collisions (simulation_detect_collisions.cpp:128-252), warp-parallel.  For
// an occupied barrier the reference's sweep tests the first rev unit (in rank order, from
// index max(n5 - 1, 0)) strictly downstream of it and the last fwd unit strictly upstream of
// it (up to index n - max(n3 - 1, 0) - 1): binary searches over the ranked positions.
// Trials draw in barrier order (ascending for rev units, descending for fwd units); a unit
// hit by several barriers keeps the last successful one in that order.
__device__ void detect_lef_bar_fast(Cell& c, u64* s, const KParams& P, u32 n, u64 n5, u64 n3) {
  const u32* __restrict__ rr = c.rr;
  const u32* __restrict__ fr = c.fr;
  const u32* __restrict__ sr = c.sr;
  const u32* __restrict__ sf = c.sf;
  const u32* __restrict__ bep = c.bep;
  const u32* __restrict__ rm = c.rm;
  const u32* __restrict__ fm = c.fm;
  for (u32 dir = 0; dir < 2; ++dir) {
    // rev: first k >= j0 with sr[k] > bpos; fwd: last k <= jtop with sf[k] < bpos
    const u32 j0 = (u32)min(n5, n5 - 1);
    const u32 jtop = (u32)(n - min(n3, n3 - 1)) - 1;
    const BucketIndex ix = build_bucket_index(dir ? sf : sr, n, (u32)P.start, (u32)P.end, c.tmp);
    const u32 nchunks = (c.nb + 32 * MLP - 1) / (32 * MLP);
    for (u32 ch = 0; ch < nchunks; ++ch) {
      rng_ensure(c, s, 32 * MLP);
      u32 bi[MLP], bpos[MLP], x[MLP], lo[MLP], k[MLP], unit[MLP], kpos[MLP], be[MLP], mv[MLP];
      bool act[MLP];
      int ti[MLP];
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) {
        const i64 i = dir ? (i64)c.nb - 1 - (i64)(ch * 32 * MLP + 32 * h + ln()) : (i64)(ch * 32 * MLP + 32 * h + ln());
        act[h] = i >= 0 && i < (i64)c.nb && bar_active(c, (u32)i);
        bi[h] = act[h] ? (u32)i : 0u;
        const uint2 pf = act[h] ? __ldg(&c.bpf[bi[h]]) : make_uint2(0u, 0u);
        bpos[h] = pf.x;
        const u32 bdir = pf.y & BF_DIR_MASK;
        ti[h] = dir ? (bdir == MGPU_DIR_FWD ? 0 : 1) : (bdir == MGPU_DIR_REV ? 0 : 1);
        x[h] = act[h] ? (dir ? pf.x : pf.x + 1) : 0u;
      }
      ranked_lower_bounds(ix, x, lo);
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) {
        bool ok;
        if (dir == 0) {
          lo[h] = max(j0, lo[h]);
          ok = lo[h] < n;
          k[h] = ok ? lo[h] : 0u;
        } else {
          lo[h] = min(jtop + 1, lo[h]);
          ok = lo[h] > 0;
          k[h] = ok ? lo[h] - 1 : 0u;
        }
        act[h] = act[h] && ok;
        unit[h] = dir ? fr[k[h]] : rr[k[h]];
        kpos[h] = dir ? sf[k[h]] : sr[k[h]];
      }
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) {
        be[h] = bep[unit[h]];
        mv[h] = dir ? fm[unit[h]] : rm[unit[h]];
      }
      u32 used = 0;
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) {
        bool cand = false, drawn = false;
        if (act[h] && be[h] != UNBOUND) {
          const u64 delta = dir ? (u64)bpos[h] - kpos[h] : (u64)kpos[h] - bpos[h];
          if (delta > 0 && delta <= mv[h]) {
            cand = true;
            drawn = trial_needs_draw(P.lef_bar[ti[h]]);
          }
        }
        const unsigned dm = __ballot_sync(FULL, drawn);
        bool hit = false;
        if (cand) {
          const u64 u = drawn ? ring_at(c, c.sc->rpos + used + __popc(dm & lanemask_lt())) : 0;
          hit = trial_outcome(P.lef_bar[ti[h]], u);
        }
        used += __popc(dm);
        // within an item the highest lane is the last barrier in sweep order; later items
        // overwrite earlier ones
        const unsigned hm = __ballot_sync(FULL, hit);
        const unsigned same = __match_any_sync(FULL, hit ? unit[h] : 0xFFFFFFFFu);
        if (hit && (31 - __clz(same & hm)) == (int)ln()) {
          const u32 w = cw_make(bi[h], EV_COLLISION | EV_LEF_BAR);
          if (dir) c.fc[unit[h]] = w; else c.rc[unit[h]] = w;
        }
        __syncwarp();
      }
      if (ln() == 0) c.sc->rpos += used;
      __syncwarp();
    }
  }
}

// detect_primary_lef_lef_collisions (simulation_detect_collisions.cpp:255-401), warp-parallel.
// With cnt(j) = number of fwd units (rank < i2) strictly before rev unit j, the sweep tests
// exactly the rev units j >= n5 with cnt(j) > cnt(j - 1) (cnt(n5 - 1) := 0) and cnt(j) < i2,
// each against the fwd unit of rank cnt(j) - 1.  Tested pairs are disjoint, so their
// collision words are updated independently; trials draw in ascending j.
__device__ void detect_primary_fast(Cell& c, u64* s, const KParams& P, u32 n, u64 n5, u64 n3) {
  if (n5 == n || n3 == n) return;
  const u32 i2 = (u32)(n - min(n3, n3 - 1));
  // bucket index over the fwd ranked positions (this step can also run on its own)
  const BucketIndex ixf = build_bucket_index(c.sf, n, (u32)P.start, (u32)P.end, c.tmp);
  u32 carry = 0;  // cnt of the element before the chunk
  for (u32 base = (u32)n5; base < n; base += 32) {
    rng_ensure(c, s, 32);
    const u32 j = base + ln();
    const bool valid = j < n;
    u32 cnt = 0;
    if (valid) cnt = min(i2, ranked_lower_bound(ixf, c.sr[j]));  // first i < i2 with sf[i] >= rp
    u32 prev = __shfl_up_sync(FULL, cnt, 1);
    if (ln() == 0) prev = carry;
    const bool tested = valid && cnt > prev && cnt < i2;
    u32 rev_idx = 0, fwd_idx = 0;
    u64 rmv = 0, fmv = 0, rp = 0, fp = 0;
    bool cand = false;
    if (tested) {
      rev_idx = c.rr[j];
      fwd_idx = c.fr[cnt - 1];
      rp = pos64(c.sr[j]);
      fp = pos64(c.sf[cnt - 1]);
      rmv = c.rm[rev_idx];
      fmv = c.fm[fwd_idx];
      const u64 delta = rp - fp;
      cand = delta > 0 && delta < rmv + fmv;
    }
    const bool drawn = cand && trial_needs_draw(P.lef_lef);
    const unsigned dm = __ballot_sync(FULL, drawn);
    bool hit = false;
    if (cand) hit = trial_outcome(P.lef_lef, drawn ? ring_at(c, c.sc->rpos + __popc(dm & lanemask_lt())) : 0);
    if (hit) primary_pair_update(c, rev_idx, fwd_idx, rp, fp, rmv, fmv);
    carry = __shfl_sync(FULL, cnt, 31);
    __syncwarp();
    if (ln() == 0) c.sc->rpos += __popc(dm);
    __syncwarp();
  }
}

// correct_moves_for_lef_bar_collisions (simulation_correct_moves.cpp:20-51)
__device__ void correct_lef_bar(Cell& c, u32 n) {
  const u32* __restrict__ rc = c.rc;
  const u32* __restrict__ fc = c.fc;
  const u32* __restrict__ rev = c.rev;
  const u32* __restrict__ fwd = c.fwd;
  u32* __restrict__ rm = c.rm;
  u32* __restrict__ fm = c.fm;
#pragma unroll 4
  for (u32 i = ln(); i < n; i += 32) {
    const u32 r = rc[i], f = fc[i];
    if (cw_occurred_as(r, EV_LEF_BAR)) rm[i] = (u32)(pos64(rev[i]) - bar_pos(c, cw_idx(r)) - 1);
    if (cw_occurred_as(f, EV_LEF_BAR)) fm[i] = (u32)(bar_pos(c, cw_idx(f)) - pos64(fwd[i]) - 1);
  }
  __syncwarp();
}

// correct_moves_for_primary_lef_lef_collisions (simulation_correct_moves.cpp:54-122): the
// pairs it visits are disjoint, so both passes are warp-parallel.
__device__ void correct_primary(Cell& c, u32 n) {
  // detect_primary pairs each fwd unit with at most one rev unit, so visiting the units in
  // index order instead of rank order changes nothing
  for (u32 rev_idx = ln(); rev_idx < n; rev_idx += 32) {
    const u32 r = c.rc[rev_idx];
    if (!cw_occurred_as(r, EV_PRIMARY)) continue;
    const u32 fwd_idx = cw_idx(r);
    const u32 f = c.fc[fwd_idx];
    if (cw_occurred_as(f, EV_PRIMARY)) {
      const u64 rp = pos64(c.rev[rev_idx]), fp = pos64(c.fwd[fwd_idx]);
      u64 p1, p2;
      lef_lef_collision_pos(rp, fp, c.rm[rev_idx], c.fm[fwd_idx], p1, p2);
      c.rm[rev_idx] = (u32)(rp - p1);
      c.fm[fwd_idx] = (u32)(p2 - fp);
    } else if (cw_occurred_as(f, EV_LEF_BAR)) {
      c.rm[rev_idx] = (u32)(pos64(c.rev[rev_idx]) - (pos64(c.fwd[fwd_idx]) + c.fm[fwd_idx]) - 1);
    }
  }
  __syncwarp();
  for (u32 fwd_idx = ln(); fwd_idx < n; fwd_idx += 32) {
    const u32 f = c.fc[fwd_idx];
    if (!cw_occurred_as(f, EV_PRIMARY)) continue;
    const u32 rev_idx = cw_idx(f);
    if (cw_occurred_as(c.rc[rev_idx], EV_LEF_BAR)) {
      c.fm[fwd_idx] = (u32)((pos64(c.rev[rev_idx]) - c.rm[rev_idx]) - pos64(c.fwd[fwd_idx]) - 1);
    }
  }
  __syncwarp();
}

// process_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:404-518), warp-parallel.
// A stalled unit followed (rev: in rank order; fwd: in reverse rank order) by free units
// starts a chain: each free unit whose target passes its stalled predecessor's target draws a
// bypass trial; success stalls it one bp behind (extending the chain), failure marks it
// avoided and ends the chain.  Chains lie between units that were stalled on entry, so they
// are disjoint and one lane walks one chain.  Draw offsets assume every trial succeeds; the
// first chain whose trial fails shifts the later ones, so the warp commits up to it and
// resumes after it.  dir 0: rev units (chains ascend), dir 1: fwd units (chains descend).
enum ChainMode { CHAIN_COUNT = 0, CHAIN_RING = 1, CHAIN_SERIAL = 2 };

template <int MODE>
__device__ __forceinline__ u32 chain_walk(Cell& c, const KParams& P, u32 dir, u32 n, i64 k,
                                          u64 off, u32* used_out) {
  const Trial& tr = P.lef_lef;
  const u32* R = dir ? c.fr : c.rr;
  u32* M = dir ? c.fm : c.rm;
  u32* C = dir ? c.fc : c.rc;
  const u32* S = dir ? c.sf : c.sr;
  const i64 step = dir ? -1 : 1;
  const i64 stop = dir ? -1 : (i64)n;
  u32 idx_prev = R[k - step];
  u64 tprev = dir ? pos64(S[k - step]) + M[idx_prev] : pos64(S[k - step]) - M[idx_prev];
  u32 used = 0, trials = 0;
  for (; k != stop; k += step) {
    const u32 idx = R[k];
    if (cw_occurred(C[idx])) break;  // stalled on entry: the next chain starts after it
    const u64 p = pos64(S[k]);
    const u64 m = M[idx];
    if (!(dir ? (p + m >= tprev) : (p - m <= tprev))) break;
    bool ok;
    if (tr.always) {
      ok = true;
    } else if (!tr.draws) {
      ok = false;
    } else {
      u64 u = 0;
      if (MODE == CHAIN_RING) u = ring_at(c, c.sc->rpos + off + used);
      if (MODE == CHAIN_SERIAL) u = rng_serial(c);
      ok = MODE == CHAIN_COUNT || u <= tr.thr;
      ++used;
    }
    ++trials;
    if (!ok) {
      if (MODE != CHAIN_COUNT) C[idx] = cw_make(idx_prev, EV_SECONDARY);
      break;
    }
    const u64 mv = dir ? (tprev - p) : (p - tprev);
    const u64 m2 = min(mv, mv - 1);
    if (MODE != CHAIN_COUNT) {
      C[idx] = cw_make(idx_prev, EV_COLLISION | EV_SECONDARY);
      M[idx] = (u32)m2;
    }
    tprev = dir ? p + m2 : p - m2;
    idx_prev = idx;
  }
  *used_out = used;
  return trials;
}

__device__ void secondary_dir_fast(Cell& c, u64* s, const KParams& P, u32 dir, u32 n, u64 n5, u64 n3) {
  const u32* R = dir ? c.fr : c.rr;
  const u32* C = dir ? c.fc : c.rc;
  // chain starts (index of the first free unit): rev: k in [max(1, n5), n) with R[k-1]
  // stalled and R[k] free, ascending; fwd: k = i - 1 for i in [1, itop] with R[i] stalled
  // and R[k] free, in descending i
  u32* starts = c.tmp;
  u32 nst = 0;
  // stalled(k) = the unit of rank k collided; each unit's word is read once and its neighbour's
  // flag comes from the adjacent lane (or the previous chunk)
  if (dir == 0) {
    const u32 k0 = (u32)max((u64)1, n5);
    bool prev = k0 - 1 < n && cw_occurred(C[R[k0 - 1]]);
    for (u32 base = k0; base < n; base += 32) {
      const u32 k = base + ln();
      const bool cur = k < n && cw_occurred(C[R[k]]);
      bool before = __shfl_up_sync(FULL, cur, 1);
      if (ln() == 0) before = prev;
      const bool st = k < n && before && !cur;
      const unsigned m = __ballot_sync(FULL, st);
      if (st) starts[nst + __popc(m & lanemask_lt())] = k;
      nst += __popc(m);
      prev = __shfl_sync(FULL, cur, 31);
    }
  } else {
    const i64 itop = (i64)(n - min(n3, n3 - 1)) - 1;
    for (i64 top = itop; top >= 1; top -= 32) {
      // lane l holds i = top - l and needs stalled(i) and stalled(i - 1): the latter is the
      // next lane's flag, read directly by lane 31
      const i64 i = top - (i64)ln();
      const bool stalled = i >= 0 && cw_occurred(C[R[i]]);
      bool below = __shfl_down_sync(FULL, stalled, 1);
      if (ln() == 31) below = i - 1 >= 0 && cw_occurred(C[R[i - 1]]);
      const bool st = i >= 1 && stalled && !below;
      const unsigned m = __ballot_sync(FULL, st);
      if (st) starts[nst + __popc(m & lanemask_lt())] = (u32)(i - 1);
      nst += __popc(m);
    }
  }
  __syncwarp();
  const bool draws = trial_needs_draw(P.lef_lef);
  u32 q = 0;
  while (q < nst) {
    rng_ensure(c, s, RNG_BLOCK);
    const u32 ci = q + ln();
    u32 L = 0, unused;
    if (ci < nst) L = chain_walk<CHAIN_COUNT>(c, P, dir, n, starts[ci], 0, &unused);
    const u32 Ld = draws ? L : 0;
    u32 tot;
    const u32 off = warp_excl_scan(Ld, &tot);
    // lanes whose speculative window would run past the draws known to be in the ring
    const unsigned over = __ballot_sync(FULL, ci < nst && off + Ld > RNG_BLOCK);
    const u32 fb = over ? (u32)(__ffs(over) - 1) : 32u;
    if (fb == 0) {  // a single chain longer than the ring window: walk it serially
      prof_add(c, PF_CHAIN_SERIAL, 1);
      if (ln() == 0) {
        u32 used;
        chain_walk<CHAIN_SERIAL>(c, P, dir, n, starts[q], 0, &used);
      }
      __syncwarp();
      q += 1;
      continue;
    }
    // evaluate each chain's trials at its speculative offset
    u32 used = 0;
    bool fails = false;
    if (ci < nst && ln() < fb && Ld > 0) {
      u32 k = 0;
      while (k < Ld && ring_at(c, c.sc->rpos + off + k) <= P.lef_lef.thr) ++k;
      fails = k < Ld;
      used = fails ? k + 1 : Ld;
    } else {
      used = Ld;
    }
    const unsigned fm_ = __ballot_sync(FULL, fails);
    const u32 f = fm_ ? (u32)(__ffs(fm_) - 1) : 32u;  // first chain whose trial fails
    const u32 last = min(f == 32 ? 31u : f, fb - 1);   // commit chains q .. q + last
    if (ci < nst && ln() <= last) {
      u32 u2;
      chain_walk<CHAIN_RING>(c, P, dir, n, starts[ci], off, &u2);
    }
    const u32 consumed = __shfl_sync(FULL, off + used, last);
    __syncwarp();
    if (ln() == 0) c.sc->rpos += consumed;
    __syncwarp();
    q += last + 1;
  }
}

// fix_secondary_lef_lef_collisions, warp-parallel: candidates (units marked avoided) are never
// adjacent in rank order (the unit before a rev candidate, after a fwd candidate, is stalled),
// so each is an independent swap of two neighbours.
__device__ bool fix_secondary_fast(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  const u32 k0 = (u32)max((u64)1, n5);
  const u32 naf = (u32)(n - min(n3, n3 - 1));
  u32* list = c.tmp;
  u32 nr = 0, nf = 0;
  bool adj = false;
  for (u32 dir = 0; dir < 2; ++dir) {
    const u32* __restrict__ R = dir ? c.fr : c.rr;
    const u32* __restrict__ W = dir ? c.fc : c.rc;
    // candidate ranks: rev [k0, n), fwd [0, naf - 1)
    const u32 lo = dir ? 0u : k0, hi = dir ? (naf > 0 ? naf - 1 : 0u) : n;
    bool prev = false;  // avoided flag of the rank before the item
    u32& cnt = dir ? nf : nr;
    for (u32 base = lo; base < hi; base += 32 * MLP) {
      u32 idx[MLP], w[MLP];
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) {
        const u32 k = base + 32 * h + ln();
        idx[h] = k < hi ? R[k] : 0u;
      }
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) w[h] = W[idx[h]];
#pragma unroll
      for (u32 h = 0; h < MLP; ++h) {
        const u32 k = base + 32 * h + ln();
        const bool av = k < hi && cw_avoided_as(w[h], EV_SECONDARY);
        bool before = __shfl_up_sync(FULL, av, 1);
        if (ln() == 0) before = prev;
        if (av && before) adj = true;
        const unsigned m = __ballot_sync(FULL, av);
        const u32 slot = (dir ? nr + nf : nr) + __popc(m & lanemask_lt());
        if (av && slot < n) list[slot] = k;
        cnt += __popc(m);
        prev = __shfl_sync(FULL, av, 31);
      }
    }
  }
  if (__any_sync(FULL, adj) || nr + nf > n) return false;
  __syncwarp();
  for (u32 t = ln(); t < nr; t += 32) fix_rev_at(c, P.start, list[t]);
  __syncwarp();
  for (u32 t = ln(); t < nf; t += 32) fix_fwd_at(c, P.end, list[nr + t]);
  __syncwarp();
  return true;
}

// process_collisions (simulation.cpp:925-955) in the reference's order.
// sorted_ranks: the ranked positions are known to be sorted (the epoch loop ranks them itself);
// otherwise (caller state) they are checked and unsorted ones take the serial restatement.
__device__ void process_collisions(Cell& c, u64* s, const KParams& P, u32 n, bool fix,
                                   bool sorted_ranks = false) {
  Scalars* sc = c.sc;
  u64 t0 = clock64();
  const bool serial = (P.debug_flags & DBG_SERIAL_COLLISIONS) || !(sorted_ranks || ranked_sorted(c, n));
  __syncwarp();
  if (ln() == 0) {
    u64 n5, n3;
    detect_boundaries_serial(c, P, n, n5, n3);
    sc->n5 = n5;
    sc->n3 = n3;
  }
  __syncwarp();
  u64 t1 = clock64();
  prof_add(c, PF_BOUNDARIES, t1 - t0);
  const u64 n5 = sc->n5, n3 = sc->n3;
  if (serial) {
    rng_ensure(c, s, RNG_BLOCK);
    if (ln() == 0) {
      detect_lef_bar_serial(c, P, n, n5, n3);
      detect_primary_serial(c, P, n, n5, n3);
    }
    __syncwarp();
  } else {
    detect_lef_bar_fast(c, s, P, n, n5, n3);
    t0 = clock64();
    prof_add(c, PF_LEF_BAR, t0 - t1);
    t1 = t0;
    detect_primary_fast(c, s, P, n, n5, n3);
  }
  t0 = clock64();
  prof_add(c, PF_PRIMARY, t0 - t1);
  correct_lef_bar(c, n);
  correct_primary(c, n);
  t1 = clock64();
  prof_add(c, PF_CORRECT, t1 - t0);
  if (serial) {
    rng_ensure(c, s, RNG_BLOCK);
    if (ln() == 0) process_secondary_serial(c, P, n, n5, n3);
    __syncwarp();
  } else {
    // chains read ranked positions; secondary moves only change moves and words
    secondary_dir_fast(c, s, P, 0, n, n5, n3);
    secondary_dir_fast(c, s, P, 1, n, n5, n3);
  }
  t0 = clock64();
  prof_add(c, PF_SECONDARY, t0 - t1);
  if (fix) {
    if (serial || !fix_secondary_fast(c, P, n, n5, n3)) {
      prof_add(c, PF_FIX_FALLBACK, 1);
      if (ln() == 0) fix_secondary_serial(c, P, n, n5, n3);
      __syncwarp();
    }
  }
  prof_add(c, PF_FIX, clock64() - t0);
}

// extrude (simulation.cpp:489-512)
__device__ void extrude(Cell& c, u32 n) {
  const u32* __restrict__ bep = c.bep;
  const u32* __restrict__ rm = c.rm;
  const u32* __restrict__ fm = c.fm;
  u32* __restrict__ rev = c.rev;
  u32* __restrict__ fwd = c.fwd;
#pragma unroll 4
  for (u32 i = ln(); i < n; i += 32) {
    if (bep[i] == UNBOUND) continue;
    rev[i] -= rm[i];
    fwd[i] += fm[i];
  }
  __syncwarp();
}

// release_lefs (simulation.cpp:544-592): one draw per bound LEF with p > 0.
__device__ u32 release_lefs(Cell& c, u64* s, const KParams& P, u32 n, bool completed) {
  u32 released = 0;
  for (u32 base = 0; base < n; base += 32 * MLP) {
    rng_ensure(c, s, 32 * MLP);
    u32 r[MLP], f[MLP], be[MLP], fr_[MLP], ff[MLP];
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) {
      const u32 i = base + 32 * h + ln();
      const u32 ic = i < n ? i : 0u;
      be[h] = i < n ? c.bep[ic] : UNBOUND;
      r[h] = c.rc[ic];
      f[h] = c.fc[ic];
    }
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) {
      const bool rb = be[h] != UNBOUND && cw_occurred_as(r[h], EV_LEF_BAR);
      const bool fb = be[h] != UNBOUND && cw_occurred_as(f[h], EV_LEF_BAR);
      fr_[h] = rb ? bar_flags(c, cw_idx(r[h])) : 0u;
      ff[h] = fb ? bar_flags(c, cw_idx(f[h])) : 0u;
    }
    u32 used = 0;
#pragma unroll
    for (u32 h = 0; h < MLP; ++h) {
      const u32 i = base + 32 * h + ln();
      const bool bound = be[h] != UNBOUND;
      Trial tr{0, 0, 0};
      if (bound) {
        u32 nh = 0;
        if (cw_occurred_as(r[h], EV_LEF_BAR) && (fr_[h] & BF_DIR_MASK) == MGPU_DIR_REV) ++nh;
        if (cw_occurred_as(f[h], EV_LEF_BAR) && (ff[h] & BF_DIR_MASK) == MGPU_DIR_FWD) ++nh;
        tr = P.release[completed ? 1 : 0][nh];
      }
      const bool need = bound && tr.draws;
      const unsigned m = __ballot_sync(FULL, need);
      const bool rel = need && ring_at(c, c.sc->rpos + used + __popc(m & lanemask_lt())) <= tr.thr;
      used += __popc(m);
      if (rel) {
        c.rev[i] = UNBOUND;
        c.fwd[i] = UNBOUND;
        c.bep[i] = UNBOUND;
      }
      released += __popc(__ballot_sync(FULL, rel));
    }
    __syncwarp();
    if (ln() == 0) c.sc->rpos += used;
    __syncwarp();
  }
  return released;
}

// compute_loop_size_stats + evaluate_burnin (simulation.cpp:957-1025).  Loop sizes are
// integers below 2^32, so the reference's double sum is exact and the mean is computed from a
// warp sum; the sum of squared deviations keeps the reference's left-to-right rounding (the
// terms are computed by all lanes, the accumulation by lane 0).
__device__ bool burnin_stats(Cell& c, const KParams& P, u32 n) {
  Scalars* sc = c.sc;
  const u32 cap = P.hist_cap;
  if (n == 0) {
    if (ln() == 0) {
      sc->hist_size = 0;
      sc->hist_head = 0;
    }
    __syncwarp();
    return false;
  }
  u64 part = 0;
#pragma unroll 4
  for (u32 i = ln(); i < n; i += 32) part += pos64(c.fwd[i]) - pos64(c.rev[i]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) part += __shfl_xor_sync(FULL, part, d);
  const double mean = (double)part / (double)n;
  double* terms = reinterpret_cast<double*>(c.sr);  // sr and sf are adjacent: n doubles
  for (u32 i = ln(); i < n; i += 32) {
    const double d = (double)(pos64(c.fwd[i]) - pos64(c.rev[i])) - mean;
    terms[i] = d * d;
  }
  __syncwarp();
  if (ln() == 0) {
    double ssd = 0.0;
    for (u32 i = 0; i < n; ++i) ssd = ssd + terms[i];
    const double sd = sqrt(ssd / (double)n);
    if (sc->hist_size == cap) {
      sc->hist_head = (sc->hist_head + 1) % cap;
      sc->hist_size--;
    }
    const u32 slot = (sc->hist_head + sc->hist_size) % cap;
    c.havg[slot] = mean;
    c.hcfx[slot] = sd / mean;
    sc->hist_size++;
  }
  __syncwarp();
  bool done = false;
  if (sc->hist_size == cap) {
    // evaluate_burnin's smoothed-dip ratio: window pairs (i1, i2) = (k + 1, k + 1 + w) for
    // k < cap - w - 1, one window per lane, each window summed in the reference's order
    const u32 w = P.smooth_w;
    const u32 head = sc->hist_head;
    auto ratio = [&](const double* d) {
      u32 nd = 0;
      for (u32 i1 = 1 + ln(); i1 + w < cap; i1 += 32) {
        const u32 i2 = i1 + w;
        double a1 = 0.0, a2 = 0.0;
        u32 k = head + i1 - 1;
        if (k >= cap) k -= cap;
        for (u32 t = 0; t < w; ++t) {
          a1 = a1 + d[k];
          if (++k == cap) k = 0;
        }
        k = head + i1;
        if (k >= cap) k -= cap;
        for (u32 t = 0; t < w; ++t) {
          a2 = a2 + d[k];
          if (++k == cap) k = 0;
        }
        const double n1 = a1 / (double)(i2 - i1), n2 = a2 / (double)(i2 - i1);
        nd += (n1 > n2) ? 1u : 0u;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) nd += __shfl_xor_sync(FULL, nd, o);
      return (double)nd / (double)((u64)cap - w - nd);
    };
    const double r1 = ratio(c.hcfx);
    if (r1 >= 0.95 && r1 <= 1.05) {
      const double r2 = ratio(c.havg);
      done = r2 >= 0.95 && r2 <= 1.05;
    }
  }
  return done;
}

// run_burnin (simulation.cpp:1027-1054)
__device__ void run_burnin(Cell& c, u64* s, const KParams& P) {
  Scalars* sc = c.sc;
  for (u64 it = 0; it < MGPU_ITER_LIMIT; ++it) {
    if (ln() == 0) ++sc->num_burnin_epochs;
    __syncwarp();
    if (sc->num_active != P.nlefs) {
      rng_ensure(c, s, 64);
      if (ln() == 0) {
        const u64 k = s_poisson(c, P);
        sc->num_active = min(sc->num_active + k, (u64)P.nlefs);
      }
      __syncwarp();
    } else {
      bool done = burnin_stats(c, P, (u32)sc->num_active);
      done = done && (sc->epoch > P.min_burnin);
      if (!done && sc->epoch >= P.max_burnin) done = true;
      if (ln() == 0) sc->burnin_completed = done ? 1 : 0;
      __syncwarp();
    }
    if (sc->num_active != 0) return;
  }
  if (ln() == 0) set_status(c, DEV_ERR_ITER_LIMIT);
  __syncwarp();
}

// ContactMatrixDense::increment (contact_matrix_dense_safe_impl.hpp:52-87); returns whether
// the contact fell outside the band (missed update).
__device__ __forceinline__ bool band_increment(Cell& c, const KParams& P, u64 row, u64 col) {
  u64 i, j;
  if (row > col) {
    i = row - col;
    j = row;
  } else {
    i = col - row;
    j = col;
  }
  if (i >= P.nrows) return true;
  if (c.band) atomicAdd(&c.band[j * P.nrows + i], 1u);
  return false;
}

__device__ u64 s_uniform_int(Cell& c, u64 a, u64 b);
__device__ double s_gev(Cell& c, const KParams& P);
__device__ i64 s_binomial(Cell& c, const KParams& P, i64 t_, double p_);
__device__ __forceinline__ double canonical_of(u64 u);

// One contact attempt read from draws at `off` (register_contacts.cpp:129-198).  Returns the
// draws it takes; *ok tells whether it registers a contact; *regular is false when the attempt
// hit a bucket rejection (exact handling needs the serial path).
__device__ __forceinline__ u32 contact_attempt(const Cell& c, const KParams& P, u64 off, bool tad,
                                               u64 na, u64 lbucket, bool* ok, bool* regular,
                                               u64* row, u64* col) {
  *ok = false;
  *regular = true;
  const u64 start = (u64)P.wstart + 1, end = (u64)P.wend - 1;
  u32 used = 0;
  const u64 li = ring_at(c, c.sc->rpos + off + used++) / lbucket;
  if (li > na - 1) {
    *regular = false;
    return used;
  }
  if (c.bep[li] == UNBOUND) return used;
  const u64 rp = pos64(c.rev[li]), fp = pos64(c.fwd[li]);
  if (!(rp > start && rp < end && fp > start && fp < end)) return used;
  double n1 = 0.0, n2 = 0.0;
  if (P.noisify) {
    const double u1 = canonical_of(ring_at(c, c.sc->rpos + off + used++));
    n1 = (P.gev_xi == 0.0) ? (P.gev_mu - P.gev_sigma) * log(-log(u1))
                           : P.gev_mu + (P.gev_sigma * (1.0 - pow(-log(u1), P.gev_xi))) / P.gev_xi;
  }
  const double a = (double)rp - n1;
  if (P.noisify) {
    const double u2 = canonical_of(ring_at(c, c.sc->rpos + off + used++));
    n2 = (P.gev_xi == 0.0) ? (P.gev_mu - P.gev_sigma) * log(-log(u2))
                           : P.gev_mu + (P.gev_sigma * (1.0 - pow(-log(u2), P.gev_xi))) / P.gev_xi;
  }
  const double b = (double)fp + n2;
  const double p1 = fmin(a, b), p2 = fmax(a, b);
  const double ds = (double)start, de = (double)end;
  if (!(p1 >= ds && p2 >= ds && p1 < de && p2 < de)) return used;
  if (!tad) {
    *row = ((u64)p1 - start) / P.bin;
    *col = ((u64)p2 - start) / P.bin;
    *ok = true;
    return used;
  }
  const u64 q1 = (u64)p1, q2 = (u64)p2;
  const u64 range = q2 - q1;
  u64 p11 = q1, p22 = q1;
  if (range != 0) {
    u64 bucket = ~0ull / (range + 1);
    if (~0ull % (range + 1) == range) ++bucket;
    const u64 r1 = ring_at(c, c.sc->rpos + off + used++) / bucket;
    if (r1 > range) {
      *regular = false;
      return used;
    }
    const u64 r2 = ring_at(c, c.sc->rpos + off + used++) / bucket;
    if (r2 > range) {
      *regular = false;
      return used;
    }
    p11 = q1 + r1;
    p22 = q1 + r2;
  }
  *row = (p11 - start) / P.bin;
  *col = (p22 - start) / P.bin;
  *ok = true;
  return used;
}

// Lane 0: one contact attempt with serial draws (the exact path for rejections).
// register_1d_lef_occupancy (register_contacts.cpp:200-232): one count in each of the two bins
__device__ __forceinline__ void occ_increment(const KParams& P, u64 i1, u64 i2) {
  if (!P.occ) return;
  if (i1 < P.occ_bins) atomicAdd(&P.occ[i1], 1ull);
  if (i2 < P.occ_bins) atomicAdd(&P.occ[i2], 1ull);
}

// One attempt of register_contacts_loop / _tad (register_contacts.cpp:129-198) or, with occ, of
// register_1d_lef_occupancy (the loop attempt with the 1D counters as its sink); lane 0.
__device__ __noinline__ void contact_attempt_serial(Cell& c, const KParams& P, bool tad, u64 na, bool* ok, bool* miss,
                                       bool occ = false) {
  *ok = false;
  *miss = false;
  const u64 start = (u64)P.wstart + 1, end = (u64)P.wend - 1;
  const u64 li = s_uniform_int(c, 0, na - 1);
  if (c.bep[li] == UNBOUND) return;
  const u64 rp = pos64(c.rev[li]), fp = pos64(c.fwd[li]);
  if (!(rp > start && rp < end && fp > start && fp < end)) return;
  const double n1 = P.noisify ? s_gev(c, P) : 0.0;
  const double a = (double)rp - n1;
  const double n2 = P.noisify ? s_gev(c, P) : 0.0;
  const double b = (double)fp + n2;
  const double p1 = fmin(a, b), p2 = fmax(a, b);
  if (!(p1 >= (double)start && p2 >= (double)start && p1 < (double)end && p2 < (double)end)) return;
  if (occ) {
    occ_increment(P, ((u64)p1 - start) / P.bin, ((u64)p2 - start) / P.bin);
  } else if (!tad) {
    *miss = band_increment(c, P, ((u64)p1 - start) / P.bin, ((u64)p2 - start) / P.bin);
  } else {
    const u64 p11 = s_uniform_int(c, (u64)p1, (u64)p2);
    const u64 p22 = s_uniform_int(c, (u64)p1, (u64)p2);
    *miss = band_increment(c, P, (p11 - start) / P.bin, (p22 - start) / P.bin);
  }
  *ok = true;
}

// sample_and_register_contacts (register_contacts.cpp:94-198): attempts are evaluated 32 at a
// time at the offsets they would have if each took the usual number of draws (1 for the LEF,
// 2 for the noise, 2 more for a TAD contact).  The warp commits up to the first attempt that
// took a different number (a LEF or position outside the bounds, a zero-width TAD range) and
// resumes after it; an attempt that hit a uniform_int bucket rejection is redone serially.
__device__ void sample_contacts(Cell& c, u64* s, const KParams& P, u64 target) {
  Scalars* sc = c.sc;
  u64 num = P.spe;
  if (P.density_positive) num = min(num, target - sc->num_contacts);
  if (num == 0) return;
  rng_ensure(c, s, 64);
  if (ln() == 0) {
    u64 n_loop;
    if (P.ratio_mode == 0) {
      n_loop = num;
    } else if (P.ratio_mode == 1) {
      n_loop = 0;
    } else {
      n_loop = (u64)s_binomial(c, P, (i64)num, P.p_loop);
    }
    sc->bc0 = n_loop;
  }
  __syncwarp();
  const u64 n_loop = sc->bc0;
  const u64 na = sc->num_active;
  u64 lbucket;
  {
    const u64 range = na - 1;
    lbucket = ~0ull / (range + 1);
    if (~0ull % (range + 1) == range) ++lbucket;
  }
  const bool serial = P.debug_flags & DBG_SERIAL_CONTACTS;
  u64 budget = 1000 * num + 1000000;  // attempts before giving up (see DEV_ERR_NO_BOUND_LEF)
  u32 missed = 0;
  const int passes = P.track_occ ? 3 : 2;  // loop, TAD, then the 1D occupancy
  for (int pass = 0; pass < passes; ++pass) {
    const bool tad = pass == 1, occ = pass == 2;
    u64 todo = occ ? num : (tad ? num - n_loop : n_loop);
    const u32 nominal = 1 + (P.noisify ? 2 : 0) + (tad ? 2 : 0);
    while (todo != 0) {
      if (budget < 32) {
        if (ln() == 0) set_status(c, DEV_ERR_NO_BOUND_LEF);
        __syncwarp();
        return;
      }
      budget -= 32;
      rng_ensure(c, s, 32 * 5);
      bool ok = false, regular = true;
      u64 row = 0, col = 0;
      u32 used = nominal;
      if (!serial) used = contact_attempt(c, P, (u64)ln() * nominal, tad, na, lbucket, &ok, &regular, &row, &col);
      const bool deviates = serial || !regular || used != nominal;
      const unsigned dm = __ballot_sync(FULL, deviates);
      const u32 f = dm ? (u32)(__ffs(dm) - 1) : 32u;
      const bool f_regular = f < 32 && __shfl_sync(FULL, regular && !serial, f);
      u32 lim = (f == 32) ? 32u : (f_regular ? f + 1 : f);  // lanes [0, lim) are exact
      const unsigned okm = __ballot_sync(FULL, ok && ln() < lim);
      if ((u64)__popc(okm) >= todo) {  // the todo-th success ends the pass
        unsigned mm = okm;
        for (u64 t = 1; t < todo; ++t) mm &= mm - 1;
        lim = (u32)__ffs(mm);
      }
      const unsigned lanes = lim >= 32 ? FULL : ((1u << lim) - 1);
      if (ok && ((lanes >> ln()) & 1u)) {
        if (occ) {
          occ_increment(P, row, col);
        } else if (band_increment(c, P, row, col)) {
          ++missed;
        }
      }
      const u32 draws = lim == 0 ? 0 : (lim - 1) * nominal + __shfl_sync(FULL, used, lim == 0 ? 0 : lim - 1);
      todo -= __popc(okm & lanes);
      __syncwarp();
      if (ln() == 0) sc->rpos += draws;
      __syncwarp();
      if (todo != 0 && lim == f && f < 32) {
        // attempt f could not be evaluated from the ring: run it serially
        prof_add(c, PF_CONTACT_SERIAL, 1);
        if (ln() == 0) {
          bool sok, smiss;
          contact_attempt_serial(c, P, tad, na, &sok, &smiss, occ);
          sc->bc1 = sok ? 1 : 0;
          if (smiss) sc->missed++;
        }
        __syncwarp();
        if (sc->bc1) todo -= 1;
        __syncwarp();
        if (sc->status != DEV_OK) return;
      }
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) missed += __shfl_xor_sync(FULL, missed, d);
  if (ln() == 0) {
    sc->missed += missed;
    sc->num_contacts += num;
  }
  __syncwarp();
}

// sample_and_register_contacts with serial draws (lane 0): the exact path behind the
// DBG_SERIAL_CONTACTS switch.
__device__ __noinline__ void sample_contacts_serial(Cell& c, const KParams& P, u64 target) {
  Scalars* sc = c.sc;
  u64 num = P.spe;
  if (P.density_positive) num = min(num, target - sc->num_contacts);
  if (num == 0) return;
  u64 n_loop;
  if (P.ratio_mode == 0) {
    n_loop = num;
  } else if (P.ratio_mode == 1) {
    n_loop = 0;
  } else {
    n_loop = (u64)s_binomial(c, P, (i64)num, P.p_loop);
  }
  u64 budget = 1000 * num + 1000000;
  const int passes = P.track_occ ? 3 : 2;  // loop, TAD, then the 1D occupancy
  for (int pass = 0; pass < passes; ++pass) {
    u64 todo = pass == 0 ? n_loop : (pass == 1 ? num - n_loop : num);
    while (todo != 0) {
      if (--budget == 0 || sc->status != DEV_OK) {
        set_status(c, DEV_ERR_NO_BOUND_LEF);
        return;
      }
      bool ok, miss;
      contact_attempt_serial(c, P, pass == 1, sc->num_active, &ok, &miss, pass == 2);
      if (miss) sc->missed++;
      if (ok) --todo;
    }
  }
  sc->num_contacts += num;
}

// ---------------------------------------------------------------------------------------
// Trace, cell setup and the epoch loop (simulation.cpp:1056-1152)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ u64 mix64(u64 z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ull;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebull;
  z ^= z >> 31;
  return z;
}

// mgpu_state_digest of the cell's state, and the full arrays when requested.
__device__ __noinline__ void trace_record(Cell& c, const KParams& P, const DevTrace& T, u64 rec) {
  const u32 nl = P.nlefs;
  const bool full = rec < T.max_records;
  u64 part = 0;
  for (u32 i = ln(); i < nl; i += 32) {
    const u64 v[9] = {pos64(c.rev[i]), pos64(c.fwd[i]), pos64(c.bep[i]), c.rr[i], c.fr[i],
                      c.rm[i], c.fm[i], cw_to_ref(c.rc[i]), cw_to_ref(c.fc[i])};
    u64 h = mix64((u64)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull);
    for (int k = 0; k < 9; ++k) h = mix64(h ^ v[k]);
    part += h;
    if (full) {
      const u64 o = rec * nl + i;
      if (T.rev_pos) T.rev_pos[o] = v[0];
      if (T.fwd_pos) T.fwd_pos[o] = v[1];
      if (T.binding_epoch) T.binding_epoch[o] = v[2];
      if (T.rev_rank) T.rev_rank[o] = v[3];
      if (T.fwd_rank) T.fwd_rank[o] = v[4];
      if (T.rev_move) T.rev_move[o] = v[5];
      if (T.fwd_move) T.fwd_move[o] = v[6];
      if (T.rev_collision) T.rev_collision[o] = v[7];
      if (T.fwd_collision) T.fwd_collision[o] = v[8];
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(FULL, part, off);
  if (ln() == 0) {
    const Scalars* sc = c.sc;
    mgpu_trace_header h;
    h.epoch = sc->epoch;
    h.num_active_lefs = sc->num_active;
    h.burnin_completed = sc->burnin_completed;
    h.num_burnin_epochs = sc->num_burnin_epochs;
    h.num_contacts = sc->num_contacts;
    h.rng_draws = sc->rpos;
    h.n5prime = sc->n5;
    h.n3prime = sc->n3;
    h.digest = part;
    if (T.all_headers && rec < T.max_epochs) T.all_headers[rec] = h;
    if (full && T.headers) T.headers[rec] = h;
  }
  __syncwarp();
}

// Lay out one cell: the header in shared memory, then each per-LEF array either in shared
// memory or in the block's global scratch slot, as planned by the host.
__device__ void carve(Cell& c, char* smem, char* gslot, const KParams& P, u32 nl, const DevChrom& ch,
                      const ulonglong2* jt, u32* band) {
  if (ln() == 0) {
    char* p = smem;
    c.sc = reinterpret_cast<Scalars*>(p);
    p += CELL_HEADER_BYTES;
    c.ring = reinterpret_cast<u64*>(p);
    p += (u64)RING * 8;
    c.hcfx = reinterpret_cast<double*>(p);
    p += (u64)P.hist_cap * 8;
    c.havg = reinterpret_cast<double*>(p);
    p += (u64)P.hist_cap * 8;
    c.bst = reinterpret_cast<u32*>(p);
    u32** arr[NARR] = {&c.rev, &c.fwd, &c.rr, &c.fr, &c.rm, &c.fm, &c.rc, &c.fc, &c.sr, &c.sf, &c.tmp, &c.bep};
    for (u32 k = 0; k < NARR; ++k) {
      char* base = ((P.arr_smem >> k) & 1u) ? smem : gslot;
      *arr[k] = reinterpret_cast<u32*>(base + P.arr_off[k]);
    }
    c.bar = ch.barriers;
    c.bpf = ch.pos_flags;
    c.nb = ch.nbarriers;
    c.nl = nl;
    c.jt = jt;
    c.band = band;
  }
  __syncwarp();
}

__device__ void cell_reset(Cell& c, u32 nl, u64 seed) {
  for (u32 i = ln(); i < nl; i += 32) {
    c.rev[i] = UNBOUND;
    c.fwd[i] = UNBOUND;
    c.bep[i] = UNBOUND;
    c.rr[i] = i;
    c.fr[i] = i;
    c.rm[i] = 0;
    c.fm[i] = 0;
    c.rc[i] = 0;
    c.fc[i] = 0;
  }
  for (u32 w = ln(); w < (c.nb + 31) / 32; w += 32) c.bst[w] = 0;
  if (ln() == 0) {
    Scalars* sc = c.sc;
    u64 st = seed;  // SplitMix64 seeding (random.hpp:26-30)
    for (int k = 0; k < 4; ++k) {
      u64 z = (st += 0x9e3779b97f4a7c15ull);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      sc->canon[k] = z ^ (z >> 31);
    }
    sc->rpos = 0;
    sc->gpos = 0;
    sc->nrec = 0;
    sc->lanes_stale = 1;
    sc->status = DEV_OK;
    sc->epoch = 0;
    sc->num_burnin_epochs = 0;
    sc->num_active = 0;
    sc->num_contacts = 0;
    sc->burnin_completed = 0;
    sc->missed = 0;
    sc->lef_epochs = 0;
    sc->sort_fallbacks = 0;
    sc->n5 = sc->n3 = 0;
    sc->hist_size = 0;
    sc->hist_head = 0;
    sc->bc0 = sc->bc1 = sc->bc2 = 0;
    sc->flag = 0;
  }
  __syncwarp();
}

// Simulation::dump_stats (simulation.cpp:1166-1224): the epoch's model-state record, taken after
// extrude and before release_lefs; the loop-size mean is exact (an integer sum below 2^53).
__device__ __noinline__ void log_model_state(Cell& c, const KParams& P, u32 n, u64 cell) {
  Scalars* sc = c.sc;
  if (!P.records || sc->nrec >= P.rec_max) return;
  u32 st_rev = 0, st_fwd = 0, st_both = 0, lb = 0, pri = 0, sec = 0;
  u64 loop = 0;
  for (u32 i = ln(); i < n; i += 32) {
    const u32 r = c.rc[i], f = c.fc[i];
    const bool sr = cw_occurred(r), sf = cw_occurred(f);
    st_rev += sr;
    st_fwd += sf;
    st_both += sr && sf;
    lb += cw_occurred_as(r, EV_LEF_BAR) + cw_occurred_as(f, EV_LEF_BAR);
    pri += cw_occurred_as(r, EV_PRIMARY) + cw_occurred_as(f, EV_PRIMARY);
    sec += cw_occurred_as(r, EV_SECONDARY) + cw_occurred_as(f, EV_SECONDARY);
    loop += pos64(c.fwd[i]) - pos64(c.rev[i]);
  }
  u32 occ = 0;
  for (u32 w = ln(); w < (c.nb + 31) / 32; w += 32) occ += __popc(c.bst[w]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    st_rev += __shfl_xor_sync(FULL, st_rev, d);
    st_fwd += __shfl_xor_sync(FULL, st_fwd, d);
    st_both += __shfl_xor_sync(FULL, st_both, d);
    lb += __shfl_xor_sync(FULL, lb, d);
    pri += __shfl_xor_sync(FULL, pri, d);
    sec += __shfl_xor_sync(FULL, sec, d);
    loop += __shfl_xor_sync(FULL, loop, d);
    occ += __shfl_xor_sync(FULL, occ, d);
  }
  if (ln() == 0) {
    mgpu_epoch_record* r = P.records + cell * P.rec_max + sc->nrec;
    r->epoch = sc->epoch;
    r->cell = cell;
    r->burnin = sc->burnin_completed ? 0 : 1;
    r->barriers_occupied = occ;
    r->nbarriers = c.nb;
    r->num_lefs = n;
    r->stalled_rev = st_rev;
    r->stalled_fwd = st_fwd;
    r->stalled_both = st_both;
    r->lef_bar = lb;
    r->lef_lef_primary = pri;
    r->lef_lef_secondary = sec;
    r->avg_loop_size = n ? (double)loop / (double)n : 0.0;
    sc->nrec++;
  }
  __syncwarp();
}

__device__ void run_cell(Cell& c, u64* s, const KParams& P, const CellTask& task, u64 target_epochs,
                         const DevTrace* trace, mgpu_cell_stats* stats, u64 cell) {
  Scalars* sc = c.sc;
  const u32 nl = P.nlefs;
  cell_reset(c, nl, task.seed);
  if (ln() == 0) sc->prof = P.prof;
  __syncwarp();
  barriers_init(c, s);
  if (P.skip_burnin && ln() == 0) {
    sc->num_active = nl;
    sc->burnin_completed = 1;
  }
  __syncwarp();
  const u64 target = task.target_contacts;
  for (u64 guard = 0; guard < MGPU_ITER_LIMIT; ++guard) {
    const bool go = P.contact_mode ? (sc->num_contacts < target)
                                   : (sc->epoch - sc->num_burnin_epochs < target_epochs);
    if (!go) break;
    const u64 te0 = clock64();
    if (!sc->burnin_completed) run_burnin(c, s, P);
    u64 ta = clock64();
    prof_add(c, PF_BURNIN, ta - te0);
    const u32 n = (u32)sc->num_active;
    const u32 epoch = (u32)sc->epoch;
    const bool completed = sc->burnin_completed != 0;
    if (ln() == 0) sc->lef_epochs += n;
    bind_lefs(c, s, P, n, epoch, 0, nullptr);
    u64 tb = clock64();
    prof_add(c, PF_BIND, tb - ta);
    rank_lefs(c, P, n, epoch, epoch != 0);
    ta = clock64();
    prof_add(c, PF_RANK, ta - tb);
    if (completed) {
      if (P.debug_flags & DBG_SERIAL_CONTACTS) {
        rng_ensure(c, s, RNG_BLOCK);
        if (ln() == 0) sample_contacts_serial(c, P, target);
        __syncwarp();
      } else {
        sample_contacts(c, s, P, target);
      }
      tb = clock64();
      prof_add(c, PF_CONTACTS, tb - ta);
      ta = tb;
      if (target != 0 && sc->num_contacts >= target) {
        prof_add(c, PF_TOTAL, clock64() - te0);
        break;
      }
      if (sc->status != DEV_OK) break;
    }
    gen_moves_dir(c, s, c.rm, n, P.rev_speed[completed], P.rev_std, P.rev_move_int[completed]);
    gen_moves_dir(c, s, c.fm, n, P.fwd_speed[completed], P.fwd_std, P.fwd_move_int[completed]);
    tb = clock64();
    prof_add(c, PF_MOVES, tb - ta);
    gather_ranked(c, n);
    adjust_moves(c, P, n);
    clamp_moves(c, P, n);
    ta = clock64();
    prof_add(c, PF_ADJUST, ta - tb);
    barriers_next(c, s);
#pragma unroll 4
    for (u32 i = ln(); i < n; i += 32) {
      c.rc[i] = 0;
      c.fc[i] = 0;
    }
    __syncwarp();
    tb = clock64();
    prof_add(c, PF_BARRIERS, tb - ta);
    process_collisions(c, s, P, n, true, true);
    ta = clock64();
    extrude(c, n);
    if (P.log_state) log_model_state(c, P, n, cell);
    release_lefs(c, s, P, n, completed);
    tb = clock64();
    prof_add(c, PF_EXTRUDE_RELEASE, tb - ta);
    if (trace) trace_record(c, P, *trace, sc->epoch);
    if (ln() == 0) sc->epoch++;
    __syncwarp();
    prof_add(c, PF_TRACE, clock64() - tb);
    prof_add(c, PF_TOTAL, clock64() - te0);
    prof_add(c, PF_EPOCHS, 1);
    if (sc->status != DEV_OK) break;
  }
  if (ln() == 0) {
    if (P.rec_count) P.rec_count[cell] = sc->nrec;
    if (trace && trace->num_recorded) *trace->num_recorded = sc->epoch;
    if (stats) {
      stats->epochs = sc->epoch;
      stats->burnin_epochs = sc->num_burnin_epochs;
      stats->contacts = sc->num_contacts;
      stats->missed_updates = sc->missed;
      stats->lef_epochs = sc->lef_epochs;
      stats->rng_draws = sc->rpos;
      stats->sort_fallbacks = sc->sort_fallbacks;
      stats->status = sc->status;
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(32) simulate_kernel(const __grid_constant__ KParams P, DevChrom ch,
                                                      const CellTask* tasks, u64 ncells,
                                                      u64 target_epochs, u32* band, u64* missed,
                                                      mgpu_cell_stats* stats, DevTrace trace,
                                                      u32 tracing, const ulonglong2* jt, u32* work,
                                                      char* gscratch) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Cell c;
  u64 s[4] = {0, 0, 0, 0};
  carve(c, smem, gscratch + (u64)blockIdx.x * P.slot_bytes, P, P.nlefs, ch, jt, band);
  for (;;) {
    u32 cell = 0;
    if (ln() == 0) cell = atomicAdd(work, 1u);
    cell = __shfl_sync(FULL, cell, 0);
    if (cell >= ncells) break;
    run_cell(c, s, P, tasks[cell], target_epochs, tracing ? &trace : nullptr, stats ? stats + cell : nullptr, cell);
    if (ln() == 0 && missed) atomicAdd((unsigned long long*)missed, (unsigned long long)c.sc->missed);
    __syncwarp();
  }
}

// Batched persistent kernel: cells of many chromosomes or windows in one work queue.  Each
// task names its plan (parameters, layout, barrier track, band); a warp copies the plan's
// parameters into shared memory when its next cell belongs to another plan than the last.
__global__ void __launch_bounds__(32) simulate_batch_kernel(const BatchPlan* plans, const BatchTask* tasks,
                                                            u64 ntasks, u64 slot_bytes,
                                                            mgpu_cell_stats* stats, const ulonglong2* jt,
                                                            u32* work, char* gscratch) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Cell c;
  __shared__ __align__(16) KParams Psh;
  u64 s[4] = {0, 0, 0, 0};
  char* gslot = gscratch + (u64)blockIdx.x * slot_bytes;
  u32 cur = 0xFFFFFFFFu;
  for (;;) {
    u32 cell = 0;
    if (ln() == 0) cell = atomicAdd(work, 1u);
    cell = __shfl_sync(FULL, cell, 0);
    if (cell >= ntasks) break;
    const BatchTask t = tasks[cell];
    const BatchPlan& pl = plans[t.plan];
    if (t.plan != cur) {
      const u32* src = reinterpret_cast<const u32*>(&pl.P);
      u32* dst = reinterpret_cast<u32*>(&Psh);
      for (u32 w = ln(); w < sizeof(KParams) / 4; w += 32) dst[w] = src[w];
      __syncwarp();
      carve(c, smem, gslot, Psh, Psh.nlefs, pl.ch, jt, pl.band);
      cur = t.plan;
    }
    const CellTask ct{t.seed, t.target_contacts};
    run_cell(c, s, Psh, ct, pl.target_epochs, nullptr, stats ? stats + cell : nullptr, cell);
    if (ln() == 0 && pl.missed) atomicAdd(pl.missed, (unsigned long long)c.sc->missed);
    __syncwarp();
  }
}

// One step of the epoch loop on caller state (mgpu_run_phase).
__global__ void __launch_bounds__(32) phase_kernel(const __grid_constant__ KParams P, DevChrom ch, int phase,
                                                   u32 n, u64* arrays, u64* bind_mask,
                                                   uint8_t* barrier_state, u64 epoch,
                                                   u32 burnin_completed, u32 partially_sorted,
                                                   u32 init_ranks, u32 adjust, u64* prng,
                                                   u64* outs, const ulonglong2* jt, char* gslot) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Cell c;
  u64 s[4] = {0, 0, 0, 0};
  carve(c, smem, gslot, P, n, ch, jt, nullptr);
  u64* A[9];
  for (int k = 0; k < 9; ++k) A[k] = arrays + (u64)k * n;
  for (u32 i = ln(); i < n; i += 32) {
    c.rev[i] = A[0][i] == ~0ull ? UNBOUND : (u32)A[0][i];
    c.fwd[i] = A[1][i] == ~0ull ? UNBOUND : (u32)A[1][i];
    c.bep[i] = A[2][i] == ~0ull ? UNBOUND : (u32)A[2][i];
    c.rr[i] = (u32)A[3][i];
    c.fr[i] = (u32)A[4][i];
    c.rm[i] = (u32)A[5][i];
    c.fm[i] = (u32)A[6][i];
    c.rc[i] = cw_from_ref(A[7][i]);
    c.fc[i] = cw_from_ref(A[8][i]);
  }
  for (u32 w = ln(); w < (c.nb + 31) / 32; w += 32) {
    u32 bits = 0;
    for (u32 b = 0; b < 32; ++b) {
      const u32 i = w * 32 + b;
      if (i < c.nb && barrier_state && barrier_state[i]) bits |= 1u << b;
    }
    c.bst[w] = bits;
  }
  u64 init_state[4];
  for (int k = 0; k < 4; ++k) init_state[k] = prng[k];
  if (ln() == 0) {
    Scalars* sc = c.sc;
    for (int k = 0; k < 4; ++k) sc->canon[k] = prng[k];
    sc->rpos = sc->gpos = 0;
    sc->lanes_stale = 1;
    sc->status = DEV_OK;
    sc->epoch = epoch;
    sc->num_active = n;
    sc->burnin_completed = burnin_completed;
    sc->sort_fallbacks = 0;
    sc->prof = nullptr;
  }
  __syncwarp();
  const bool completed = burnin_completed != 0;
  u64 released = 0;
  switch (phase) {
    case MGPU_PHASE_BIND:
      bind_lefs(c, s, P, n, (u32)epoch, bind_mask ? 1 : 2, bind_mask);
      rank_lefs(c, P, n, (u32)epoch, epoch != 0);
      break;
    case MGPU_PHASE_RANK:
      if (init_ranks) {
        for (u32 i = ln(); i < n; i += 32) {
          c.rr[i] = i;
          c.fr[i] = i;
        }
        __syncwarp();
      }
      rank_lefs(c, P, n, (u32)epoch, partially_sorted != 0);
      break;
    case MGPU_PHASE_ADJUST_AND_CLAMP:
      gather_ranked(c, n);
      adjust_moves(c, P, n);
      clamp_moves(c, P, n);
      break;
    case MGPU_PHASE_GENERATE_MOVES:
      gen_moves_dir(c, s, c.rm, n, P.rev_speed[completed], P.rev_std, P.rev_move_int[completed]);
      gen_moves_dir(c, s, c.fm, n, P.fwd_speed[completed], P.fwd_std, P.fwd_move_int[completed]);
      if (adjust) {
        gather_ranked(c, n);
        adjust_moves(c, P, n);
      }
      clamp_moves(c, P, n);
      break;
    case MGPU_PHASE_PROCESS_COLLISIONS:
      gather_ranked(c, n);
      process_collisions(c, s, P, n, false);
      break;
    case MGPU_PHASE_FIX_SECONDARY:
      if (ln() == 0) fix_secondary_serial(c, P, n, 0, 0);
      break;
    case MGPU_PHASE_DETECT_LEF_BAR:
      gather_ranked(c, n);
      if (ranked_sorted(c, n) && !(P.debug_flags & DBG_SERIAL_COLLISIONS)) {
        detect_lef_bar_fast(c, s, P, n, 0, 0);
      } else {
        rng_ensure(c, s, RNG_BLOCK);
        if (ln() == 0) detect_lef_bar_serial(c, P, n, 0, 0);
      }
      break;
    case MGPU_PHASE_LEF_LEF:
      gather_ranked(c, n);
      if (ranked_sorted(c, n) && !(P.debug_flags & DBG_SERIAL_COLLISIONS)) {
        detect_primary_fast(c, s, P, n, 0, 0);
        correct_primary(c, n);
        secondary_dir_fast(c, s, P, 0, n, 0, 0);
        secondary_dir_fast(c, s, P, 1, n, 0, 0);
      } else {
        rng_ensure(c, s, RNG_BLOCK);
        if (ln() == 0) detect_primary_serial(c, P, n, 0, 0);
        __syncwarp();
        correct_primary(c, n);
        if (ln() == 0) process_secondary_serial(c, P, n, 0, 0);
      }
      break;
    case MGPU_PHASE_DETECT_PRIMARY:
      gather_ranked(c, n);
      if (ranked_sorted(c, n) && !(P.debug_flags & DBG_SERIAL_COLLISIONS)) {
        detect_primary_fast(c, s, P, n, 0, 0);
      } else {
        rng_ensure(c, s, RNG_BLOCK);
        if (ln() == 0) detect_primary_serial(c, P, n, 0, 0);
      }
      break;
    case MGPU_PHASE_DETECT_BOUNDARIES:
      if (ln() == 0) {
        u64 n5, n3;
        detect_boundaries_serial(c, P, n, n5, n3);
        c.sc->n5 = n5;
        c.sc->n3 = n3;
      }
      break;
    case MGPU_PHASE_CORRECT_LEF_BAR:
      correct_lef_bar(c, n);
      break;
    case MGPU_PHASE_CORRECT_PRIMARY:
      correct_primary(c, n);
      break;
    case MGPU_PHASE_EXTRUDE:
      extrude(c, n);
      break;
    case MGPU_PHASE_RELEASE:
      released = release_lefs(c, s, P, n, completed);
      break;
    case MGPU_PHASE_BARRIER_NEXT:
      barriers_next(c, s);
      break;
    case MGPU_PHASE_BARRIER_INIT:
      barriers_init(c, s);
      break;
    default:
      break;
  }
  __syncwarp();
  // rank_lefs uses the move arrays as scratch: the caller's moves stay as they were
  const bool moves_kept = phase == MGPU_PHASE_BIND || phase == MGPU_PHASE_RANK;
  for (u32 i = ln(); i < n; i += 32) {
    A[0][i] = pos64(c.rev[i]);
    A[1][i] = pos64(c.fwd[i]);
    A[2][i] = pos64(c.bep[i]);
    A[3][i] = c.rr[i];
    A[4][i] = c.fr[i];
    if (!moves_kept) {
      A[5][i] = c.rm[i];
      A[6][i] = c.fm[i];
    }
    A[7][i] = cw_to_ref(c.rc[i]);
    A[8][i] = cw_to_ref(c.fc[i]);
  }
  for (u32 i = ln(); i < c.nb; i += 32) {
    if (barrier_state) barrier_state[i] = bar_active(c, i) ? 1 : 0;
  }
  if (ln() == 0) {
    // the caller's PRNG advanced by exactly the number of draws consumed
    u64 st[4] = {init_state[0], init_state[1], init_state[2], init_state[3]};
    for (u64 k = 0; k < c.sc->rpos; ++k) xo_next(st);
    for (int k = 0; k < 4; ++k) prng[k] = st[k];
    outs[0] = c.sc->n5;
    outs[1] = c.sc->n3;
    outs[2] = released;
    outs[3] = c.sc->status;
  }
}

// ---------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------
static int cuda_fail(cudaError_t e, const char* what, char* errbuf, int errlen) {
  if (e == cudaSuccess) return MGPU_OK;
  if (errbuf) snprintf(errbuf, errlen, "%s: %s", what, cudaGetErrorString(e));
  return MGPU_ERR_CUDA;
}

// Largest dynamic shared memory a block of either kernel may request: the device's opt-in
// limit minus the kernels' static shared memory.
u64 max_smem_per_block() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  u64 stat = 0;
  cudaFuncAttributes a{};
  if (cudaFuncGetAttributes(&a, simulate_kernel) == cudaSuccess) stat = a.sharedSizeBytes;
  if (cudaFuncGetAttributes(&a, phase_kernel) == cudaSuccess && a.sharedSizeBytes > stat) stat = a.sharedSizeBytes;
  if (cudaFuncGetAttributes(&a, simulate_batch_kernel) == cudaSuccess && a.sharedSizeBytes > stat)
    stat = a.sharedSizeBytes;
  cudaGetLastError();
  return (u64)v > stat ? (u64)v - stat : 0;
}

u64 resident_cells(const KParams& P, u64 ncells) {
  // tuning switches carried in the debug flags: bits 8-15 carveout percent, 16-23 cells per SM
  const u32 carveout = (P.debug_flags >> 8) & 0xFFu, max_per_sm = (P.debug_flags >> 16) & 0xFFu;
  cudaFuncSetAttribute(simulate_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                       carveout ? (int)carveout : -1);
  cudaGetLastError();
  // The attribute is a per-function permission shared by every thread and context of the
  // process, so it is always set to the device limit: lowering it for one launch would make a
  // concurrent launch with a larger plan fail.
  if (cudaFuncSetAttribute(simulate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)max_smem_per_block()) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, simulate_kernel, 32, P.smem_bytes) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (max_per_sm && per_sm > (int)max_per_sm) per_sm = (int)max_per_sm;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  u64 grid = (u64)sms * (u64)(per_sm > 0 ? per_sm : 1);
  return grid < ncells ? grid : ncells;
}

int launch_simulate(const KParams& P, const DevChrom& ch, const CellTask* tasks, u64 ncells,
                    u64 target_epochs, u32* band, u64* missed, mgpu_cell_stats* stats,
                    const DevTrace* trace, const void* jump_table, u32* work_counter,
                    char* gscratch, u64 gscratch_bytes, void* stream, char* errbuf, int errlen) {
  int rc = cuda_fail(cudaFuncSetAttribute(simulate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)max_smem_per_block()),
                     "cudaFuncSetAttribute", errbuf, errlen);
  if (rc) return rc;
  u64 grid = resident_cells(P, ncells);
  if (grid == 0) return MGPU_OK;
  if (P.slot_bytes && gscratch_bytes / P.slot_bytes < grid) grid = gscratch_bytes / P.slot_bytes;
  if (grid == 0) {
    if (errbuf) snprintf(errbuf, errlen, "global scratch too small for one cell");
    return MGPU_ERR_INTERNAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  rc = cuda_fail(cudaMemsetAsync(work_counter, 0, sizeof(u32), st), "memset", errbuf, errlen);
  if (rc) return rc;
  DevTrace tr{};
  u32 tracing = 0;
  if (trace) {
    tr = *trace;
    tracing = 1;
  }
  simulate_kernel<<<(unsigned)grid, 32, P.smem_bytes, st>>>(P, ch, tasks, ncells, target_epochs, band,
                                                             missed, stats, tr, tracing,
                                                             (const ulonglong2*)jump_table, work_counter,
                                                             gscratch);
  return cuda_fail(cudaGetLastError(), "simulate_kernel launch", errbuf, errlen);
}

u64 resident_batch_cells(u32 smem_bytes, u64 ntasks, u32 carveout_pct, u32 max_per_sm) {
  if (cudaFuncSetAttribute(simulate_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)max_smem_per_block()) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  // shared memory / L1 split preference (a tuning switch; -1 lets the CUDA driver choose)
  cudaFuncSetAttribute(simulate_batch_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                       carveout_pct ? (int)carveout_pct : -1);
  cudaGetLastError();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, simulate_batch_kernel, 32, smem_bytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (max_per_sm && per_sm > (int)max_per_sm) per_sm = (int)max_per_sm;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (max_per_sm && per_sm > (int)max_per_sm) per_sm = (int)max_per_sm;
  const u64 grid = (u64)sms * (u64)(per_sm > 0 ? per_sm : 1);
  return grid < ntasks ? grid : ntasks;
}

int launch_simulate_batch(const BatchPlan* plans, const BatchTask* tasks, u64 ntasks, u32 smem_bytes,
                          u64 slot_bytes, mgpu_cell_stats* stats, const void* jump_table, u32* work_counter,
                          char* gscratch, u64 gscratch_bytes, u32 carveout_pct, u32 max_per_sm, void* stream,
                          char* errbuf, int errlen) {
  u64 grid = resident_batch_cells(smem_bytes, ntasks, carveout_pct, max_per_sm);
  if (grid == 0) return ntasks ? MGPU_ERR_CUDA : MGPU_OK;
  if (slot_bytes && gscratch_bytes / slot_bytes < grid) grid = gscratch_bytes / slot_bytes;
  if (grid == 0) {
    if (errbuf) snprintf(errbuf, errlen, "global scratch too small for one cell");
    return MGPU_ERR_INTERNAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int rc = cuda_fail(cudaMemsetAsync(work_counter, 0, sizeof(u32), st), "memset", errbuf, errlen);
  if (rc) return rc;
  simulate_batch_kernel<<<(unsigned)grid, 32, smem_bytes, st>>>(plans, tasks, ntasks, slot_bytes, stats,
                                                                 (const ulonglong2*)jump_table, work_counter,
                                                                 gscratch);
  return cuda_fail(cudaGetLastError(), "simulate_batch_kernel launch", errbuf, errlen);
}

int launch_phase(const KParams& P, const DevChrom& ch, int phase, u64 n, u64* arrays,
                 u64* bind_mask, uint8_t* barrier_state, u64 epoch, u32 burnin_completed,
                 u32 partially_sorted, u32 init_ranks, u32 adjust, u64* prng_state, u64* outs,
                 const void* jump_table, char* gscratch, void* stream, char* errbuf, int errlen) {
  int rc = cuda_fail(cudaFuncSetAttribute(phase_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)max_smem_per_block()),
                     "cudaFuncSetAttribute", errbuf, errlen);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  phase_kernel<<<1, 32, P.smem_bytes, st>>>(P, ch, phase, (u32)n, arrays, bind_mask, barrier_state, epoch,
                                            burnin_completed, partially_sorted, init_ranks, adjust,
                                            prng_state, outs, (const ulonglong2*)jump_table, gscratch);
  return cuda_fail(cudaGetLastError(), "phase_kernel launch", errbuf, errlen);
}

// ---------------------------------------------------------------------------------------
// Probes of the device's floating-point library (test hooks): the samplers of the epoch loop
// run on whole seeded streams, and the transcendental functions on caller arguments, so that
// the test-suite can compare them with the host's libm (glibc, the reference's) bit for bit.
// ---------------------------------------------------------------------------------------

// One block per stream (grid-stride): lane 0 draws `per` samples of one distribution from the
// Xoshiro256++ state states[4 s .. 4 s + 3] through the same serial samplers the epoch loop
// uses, writes them to out[s * per ..] and the number of raw draws taken to draws[s].
__global__ void __launch_bounds__(32) sampler_probe_kernel(const __grid_constant__ KParams P, int kind,
                                                           const u64* states, u64 nstreams, u64 per,
                                                           double a0, double a1, double* out, u64* draws) {
  __shared__ Scalars sc;
  __shared__ u64 ring[RING];
  if (threadIdx.x != 0) return;
  for (u64 s = blockIdx.x; s < nstreams; s += gridDim.x) {
    Cell c{};
    c.sc = &sc;
    c.ring = ring;
    sc.rpos = sc.gpos = 0;
    sc.status = DEV_OK;
    sc.lanes_stale = 0;
    sc.prof = nullptr;
    for (int k = 0; k < 4; ++k) sc.canon[k] = states[4 * s + k];
    for (u64 i = 0; i < per; ++i) {
      double v = 0.0;
      switch (kind) {
        case 0: v = s_unit_normal(c) * a1 + a0; break;
        case 1: v = s_unit_exponential(c); break;
        case 2: v = (double)s_poisson(c, P); break;
        case 3: v = (double)s_binomial(c, P, (i64)a0, a1); break;
        case 4: v = s_gev(c, P); break;
        default: break;
      }
      out[s * per + i] = v;
    }
    draws[s] = sc.status == DEV_OK ? sc.rpos : ~0ull;
  }
}

// out[i] = f(x[i], y[i]) for f = 0: log x, 1: exp x, 2: pow(x, y), 3: the GEV noise of
// register_contacts.cpp:48-64 from u = x (mu, sigma, xi), 4: below_exp(x, y) as 0 or 1.
__global__ void libm_probe_kernel(int kind, const double* x, const double* y, u64 n, double mu, double sigma,
                                  double xi, double* out) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const double a = x[i];
    double r = 0.0;
    switch (kind) {
      case 0: r = log(a); break;
      case 1: r = exp(a); break;
      case 2: r = pow(a, y[i]); break;
      case 3: r = xi == 0.0 ? (mu - sigma) * log(-log(a)) : mu + (sigma * (1.0 - pow(-log(a), xi))) / xi; break;
      case 4: r = below_exp(a, y[i]) ? 1.0 : 0.0; break;
      default: break;
    }
    out[i] = r;
  }
}

int launch_sampler_probe(const KParams& P, int kind, const u64* states, u64 nstreams, u64 per, double a0,
                         double a1, double* out, u64* draws, void* stream, char* errbuf, int errlen) {
  if (nstreams == 0) return MGPU_OK;
  const u64 blocks = nstreams < 65535 ? nstreams : 65535;
  sampler_probe_kernel<<<(unsigned)blocks, 32, 0, (cudaStream_t)stream>>>(P, kind, states, nstreams, per, a0, a1,
                                                                          out, draws);
  return cuda_fail(cudaGetLastError(), "sampler_probe_kernel launch", errbuf, errlen);
}

int launch_libm_probe(int kind, const double* x, const double* y, u64 n, double mu, double sigma, double xi,
                      double* out, void* stream, char* errbuf, int errlen) {
  if (n == 0) return MGPU_OK;
  const u64 blocks = (n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16;
  libm_probe_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(kind, x, y, n, mu, sigma, xi, out);
  return cuda_fail(cudaGetLastError(), "libm_probe_kernel launch", errbuf, errlen);
}

// ---------------------------------------------------------------------------------------
// Fixed scratch of the allocation-free entry point (one array per device, part of the module)
// ---------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[MGPU_NOALLOC_SCRATCH_BYTES];

__global__ void pack_tasks_kernel(const u64* seeds, const u64* targets, u64 n, CellTask* tasks) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    tasks[i].seed = seeds[i];
    tasks[i].target_contacts = targets[i];
  }
}

int noalloc_scratch_address(void** ptr, char* errbuf, int errlen) {
  return cuda_fail(cudaGetSymbolAddress(ptr, g_noalloc_scratch), "cudaGetSymbolAddress", errbuf, errlen);
}

int launch_pack_tasks(const u64* seeds, const u64* targets, u64 n, CellTask* tasks, void* stream,
                      char* errbuf, int errlen) {
  if (n == 0) return MGPU_OK;
  const u64 blocks = (n + 255) / 256;
  pack_tasks_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(seeds, targets, n, tasks);
  return cuda_fail(cudaGetLastError(), "pack_tasks_kernel launch", errbuf, errlen);
}

}  // namespace mgpu
