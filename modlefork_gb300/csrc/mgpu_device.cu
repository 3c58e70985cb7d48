// mgpu_device.cu - sm_103a kernels of the loop-extrusion epoch engine.
//
// One warp simulates one cell (Simulation::simulate_one_cell, src/libmodle/cpu/
// simulation.cpp:1056-1152).  The cell's whole state lives in shared memory as 32-bit
// structure-of-arrays; the barrier track and its integer thresholds are read-only in global
// memory and shared by every cell of the chromosome.  The kernel is persistent: each warp
// pulls cell indices from a global work counter until the batch is drained.
//
// Draw order.  Every random number of the reference comes from one sequential
// Xoshiro256++ stream per cell, consumed in a data-dependent order.  The warp keeps a ring of
// pre-generated draws in shared memory: all 32 lanes generate RNG_S consecutive draws each
// per refill, and then advance their private state by 31 * RNG_S steps with a GF(2) jump
// table (the state transition of xoshiro is linear), so the ring always holds the exact
// stream.  Phases whose items take one draw each (binding, barrier steps, moves, release)
// give lane k the draw at offset popc(ballot & lanemask_lt); the rare item that needs more
// draws (a ziggurat wedge or tail, a bucket rejection) is finished by lane 0 from its exact
// offset and the warp resumes after it.  Sequential sweeps (collision detection, chains of
// secondary collisions, the exact split_sort) run on lane 0 and read draws serially.
//
// Floating point.  The file is compiled with --fmad=false so every double multiply and add
// is rounded separately, like the reference's x86-64 build; bernoulli and
// generate_canonical comparisons are replaced by exact integer thresholds computed on the
// host.

#include <cuda_runtime.h>

#include <cstdio>

#include "cppsort_emul.h"
#include "mgpu_internal.h"
#define MGPU_ZIG_TABLE_QUAL __device__ const
#include "ziggurat_tables.h"

namespace mgpu {

#define MGPU_ITER_LIMIT 100000000ull

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

__device__ __forceinline__ u64 pos64(u32 v) { return v == UNBOUND ? ~0ull : (u64)v; }

// Cell scalars (warp-uniform, kept in shared memory so lane 0's serial code can update them).
struct Scalars {
  u64 rpos, gpos;  // next draw to consume / to generate (stream indices)
  u64 canon[4];    // xoshiro state at gpos
  u32 lanes_stale; // lanes must re-derive their states from canon before the next refill
  u32 status;
  u64 epoch, num_burnin_epochs, num_active, num_contacts;
  u32 burnin_completed, pad0;
  u64 missed, lef_epochs, sort_fallbacks;
  u64 n5, n3;
  u32 hist_size, hist_head;
  u64 records;
};

struct Cell {
  Scalars* sc;
  u64* ring;
  u32 *rev, *fwd, *bep, *rr, *fr, *rm, *fm, *rc, *fc, *tmp;
  u32* bst;
  double *hcfx, *havg;
  const DevBarrier* bar;
  u32 nb;
  const ulonglong2* jt;
  int lane;
  u64 s[4];
  u32* band;
};

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

// Collective: append RNG_BLOCK draws to the ring.
__device__ __noinline__ void rng_refill(Cell& c) {
  Scalars* sc = c.sc;
  if (sc->lanes_stale) {
    for (int k = 0; k < 4; ++k) c.s[k] = sc->canon[k];
    for (int t = 0; t < c.lane * RNG_S; ++t) xo_next(c.s);
  }
  const u64 g = sc->gpos;
  for (int k = 0; k < RNG_S; ++k) c.ring[(g + (u64)c.lane * RNG_S + k) & (RING - 1)] = xo_next(c.s);
  xo_jump(c.s, c.jt);
  __syncwarp();
  if (c.lane == 0) {
    sc->gpos = g + RNG_BLOCK;
    for (int k = 0; k < 4; ++k) sc->canon[k] = c.s[k];
    sc->lanes_stale = 0;
  }
  __syncwarp();
}

// Collective: make at least n (<= RNG_BLOCK) unconsumed draws available.
__device__ __forceinline__ void rng_ensure(Cell& c, u32 n) {
  while (c.sc->gpos - c.sc->rpos < n) rng_refill(c);
}

__device__ __forceinline__ u64 ring_at(const Cell& c, u64 k) { return c.ring[k & (RING - 1)]; }

// Lane 0 only: next draw of the stream, generated serially when the ring is dry.
__device__ u64 rng_serial(Cell& c) {
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

// ---------------------------------------------------------------------------------------
// Serial distributions (lane 0).  Boost.Random 1.79 semantics, see the oracle for the
// line-by-line restatement; thresholds replace bernoulli / canonical comparisons.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void set_status(Cell& c, u32 st) {
  if (c.sc->status == DEV_OK) c.sc->status = st;
}

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

__device__ double s_unit_exponential(Cell& c) {
  double shift = 0;
  for (int it = 0; it < 100000; ++it) {
    const u64 u = rng_serial(c);
    const int i = (int)(u & 0xFF);
    const double x = ifp_fraction(u) * mgpu_zig_exp_x[i];
    if (x < mgpu_zig_exp_x[i + 1]) return shift + x;
    if (i == 0) {
      shift += mgpu_zig_exp_x[1];
    } else {
      const double y01 = s_uniform01(c);
      const double y = mgpu_zig_exp_y[i] + y01 * (mgpu_zig_exp_y[i + 1] - mgpu_zig_exp_y[i]);
      if (y < exp(-x)) return x + shift;
    }
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
  return 0.0;
}

__device__ double s_normal_tail(Cell& c) {
  const double tail_start = mgpu_zig_normal_x[1];
  for (int it = 0; it < 100000; ++it) {
    const double x = s_unit_exponential(c) / tail_start;
    const double y = s_unit_exponential(c) / 1.0;
    if (2 * y > x * x) return x + tail_start;
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
  return 0.0;
}

// Fast path of unit_normal_distribution for one draw: returns false when the draw falls in a
// wedge or the tail (the full algorithm is then needed).
__device__ __forceinline__ bool normal_fast(u64 u, double& z) {
  const int ii = (int)(u & 0xFF);
  const double sign = (double)((ii & 1) * 2 - 1);
  const int i = ii >> 1;
  const double x = ifp_fraction(u) * mgpu_zig_normal_x[i];
  z = x * sign;
  return x < mgpu_zig_normal_x[i + 1];
}

__device__ double s_unit_normal(Cell& c) {
  for (int it = 0; it < 100000; ++it) {
    const u64 u = rng_serial(c);
    const int ii = (int)(u & 0xFF);
    const int sign = (ii & 1) * 2 - 1;
    const int i = ii >> 1;
    const double x = ifp_fraction(u) * mgpu_zig_normal_x[i];
    if (x < mgpu_zig_normal_x[i + 1]) return x * sign;
    if (i == 0) return s_normal_tail(c) * sign;
    const double y01 = s_uniform01(c);
    const double y =
        mgpu_zig_normal_y[i] + y01 * (mgpu_zig_normal_y[i + 1] - mgpu_zig_normal_y[i]);
    if (y < exp(-(x * x / 2))) return x * sign;
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
  return 0.0;
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

__device__ u64 s_poisson(Cell& c, const KParams& P) {
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

__device__ i64 s_binomial(Cell& c, const KParams& P, i64 t_, double p_) {
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

__device__ double s_gev(Cell& c, const KParams& P) {
  const double u = canonical_of(rng_serial(c));
  if (P.gev_xi == 0.0) return (P.gev_mu - P.gev_sigma) * log(-log(u));
  return P.gev_mu + (P.gev_sigma * (1.0 - pow(-log(u), P.gev_xi))) / P.gev_xi;
}

// rank_lefs (simulation.cpp:402-487); lane 0
__device__ void rank_lefs_serial(Cell& c, u32 n, bool partially_sorted, bool init) {
  if (init) {
    for (u32 i = 0; i < n; ++i) {
      c.rr[i] = i;
      c.fr[i] = i;
    }
  }
  const KeyCmp rcmp{c.rev}, fcmp{c.fwd};
  if (partially_sorted) {
    split_sort(c.rr, n, c.tmp, rcmp);
    split_sort(c.fr, n, c.tmp, fcmp);
  } else {
    pdq_sort(c.rr, 0, n, rcmp);
    pdq_sort(c.fr, 0, n, fcmp);
  }
  for (u32 i = 1; i < n; ++i) {
    if (c.rev[c.rr[i - 1]] == c.rev[c.rr[i]]) {
      const u32 begin = i - 1;
      for (; i < n; ++i) {
        if (c.rev[c.rr[i - 1]] != c.rev[c.rr[i]]) break;
      }
      ins_sort(c.rr, begin, i, KeyCmp{c.bep});
    }
  }
  for (u32 i = 1; i < n; ++i) {
    if (c.fwd[c.fr[i - 1]] == c.fwd[c.fr[i]]) {
      const u32 begin = i - 1;
      for (; i < n; ++i) {
        if (c.fwd[c.fr[i - 1]] != c.fwd[c.fr[i]]) break;
      }
      ins_sort(c.fr, begin, i, KeyCmpRev{c.bep});
    }
  }
}

// ---------------------------------------------------------------------------------------
// Epoch steps
// ---------------------------------------------------------------------------------------

// ExtrusionBarriers::init_states (extrusion_barriers.cpp:220-231): warp-parallel.
__device__ void barriers_init(Cell& c) {
  for (u32 base = 0; base < c.nb; base += 32) {
    rng_ensure(c, 32);
    const u32 i = base + c.lane;
    const bool need = i < c.nb && (c.bar[i].flags & BF_OCC_DRAWS);
    const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    const u32 off = __popc(m & lanemask_lt());
    bool occ = false;
    if (need) occ = ring_at(c, c.sc->rpos + off) <= c.bar[i].t_occ;
    const unsigned om = __ballot_sync(0xFFFFFFFFu, occ);
    __syncwarp();
    if (c.lane == 0) {
      c.bst[base >> 5] = om;
      c.sc->rpos += __popc(m);
    }
    __syncwarp();
  }
}

// ExtrusionBarriers::next_state (extrusion_barriers.cpp:145-161): one draw per barrier.
__device__ void barriers_next(Cell& c) {
  for (u32 base = 0; base < c.nb; base += 32) {
    rng_ensure(c, 32);
    const u32 i = base + c.lane;
    const bool valid = i < c.nb;
    bool st = (c.bst[base >> 5] >> c.lane) & 1u;
    if (valid) {
      const u64 u = ring_at(c, c.sc->rpos + c.lane);
      const u32 f = c.bar[i].flags;
      if (!st) {
        st = !(f & BF_INA_NEVER) && u >= c.bar[i].t_ina;
      } else {
        st = !(!(f & BF_ACT_NEVER) && u >= c.bar[i].t_act);
      }
    }
    const unsigned nm = __ballot_sync(0xFFFFFFFFu, valid && st);
    __syncwarp();
    if (c.lane == 0) {
      c.bst[base >> 5] = nm;
      c.sc->rpos += min(32u, c.nb - base);
    }
    __syncwarp();
  }
}

__device__ __forceinline__ bool bar_active(const Cell& c, u32 i) { return (c.bst[i >> 5] >> (i & 31)) & 1u; }

// select_lefs_to_bind + bind_lefs (simulation_impl.hpp:28-89): warp-parallel, one
// uniform_int draw per selected LEF in index order.  Selection: mode 0 = unbound LEFs (the
// epoch loop), 1 = nonzero entries of mask, 2 = every LEF (an empty mask in the reference).
__device__ __forceinline__ bool bind_selected(const Cell& c, u32 i, int mode, const u64* mask) {
  return mode == 0 ? c.bep[i] == UNBOUND : (mode == 1 ? mask[i] != 0 : true);
}

__device__ void bind_lefs(Cell& c, const KParams& P, u32 n, u32 epoch, int mode, const u64* mask) {
  u32 i0 = 0;
  while (i0 < n) {
    rng_ensure(c, 32);
    const u32 i = i0 + c.lane;
    const bool need = i < n && bind_selected(c, i, mode, mask);
    const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    const u32 off = __popc(m & lanemask_lt());
    u64 r = 0;
    bool ok = true;
    if (need) {
      r = ring_at(c, c.sc->rpos + off) / P.pos_bucket;
      ok = r <= P.pos_range;
    }
    const unsigned bad = __ballot_sync(0xFFFFFFFFu, need && !ok);
    const u32 f = bad ? (u32)(__ffs(bad) - 1) : 32u;
    if (need && c.lane < f) {
      const u32 pos = (u32)(P.start + r);
      c.rev[i] = pos;
      c.fwd[i] = pos;
      c.bep[i] = epoch;
    }
    __syncwarp();
    if (c.lane == 0) {
      c.sc->rpos += __popc(m & (f == 32 ? 0xFFFFFFFFu : ((1u << f) - 1)));
      if (f < 32) {  // finish this chunk serially from the rejecting LEF
        for (u32 k = i0 + f; k < min(i0 + 32, n); ++k) {
          const bool nk = bind_selected(c, k, mode, mask);
          if (!nk) continue;
          const u64 pos = s_uniform_int(c, P.start, (u64)P.end - 1);
          c.rev[k] = (u32)pos;
          c.fwd[k] = (u32)pos;
          c.bep[k] = epoch;
        }
      }
    }
    __syncwarp();
    i0 += 32;
  }
}

// generate_moves_helper (simulation.cpp:264-290): warp-parallel speculation on the ziggurat
// fast path; the first item that needs more draws is finished serially by lane 0.
__device__ void gen_moves_dir(Cell& c, u32* mv, u32 n, double mean, double sd, u64 move_int) {
  if (sd == 0.0) {
    for (u32 i = c.lane; i < n; i += 32) mv[i] = c.bep[i] == UNBOUND ? 0u : (u32)move_int;
    __syncwarp();
    return;
  }
  u32 i0 = 0;
  while (i0 < n) {
    rng_ensure(c, 64);
    const u32 i = i0 + c.lane;
    const bool need = i < n && c.bep[i] != UNBOUND;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    const u32 off = __popc(m & lanemask_lt());
    double z = 0;
    bool ok = true;
    if (need) ok = normal_fast(ring_at(c, c.sc->rpos + off), z);
    const unsigned bad = __ballot_sync(0xFFFFFFFFu, need && !ok);
    const u32 f = bad ? (u32)(__ffs(bad) - 1) : 32u;
    if (i < n && c.lane < f) {
      if (need) {
        const double v = round(fmax(0.0, z * sd + mean));
        if (v > 4294967295.0) set_status(c, DEV_ERR_MOVE_RANGE);
        mv[i] = (u32)(u64)v;
      } else {
        mv[i] = 0;
      }
    }
    __syncwarp();
    if (c.lane == 0) {
      c.sc->rpos += __popc(m & (f == 32 ? 0xFFFFFFFFu : ((1u << f) - 1)));
      if (f < 32) {
        const double zz = s_unit_normal(c);
        const double v = round(fmax(0.0, zz * sd + mean));
        if (v > 4294967295.0) set_status(c, DEV_ERR_MOVE_RANGE);
        mv[i0 + f] = (u32)(u64)v;
      }
    }
    __syncwarp();
    i0 += (f == 32) ? 32 : f + 1;
  }
}

// adjust_moves_of_consecutive_extr_units (simulation.cpp:343-399); lane 0
__device__ void adjust_moves_serial(Cell& c, const KParams& P, u32 n) {
  if (n == 0) return;
  const u64 start = P.start, end = P.end;
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

// clamp_moves (simulation.cpp:325-340): warp-parallel
__device__ void clamp_moves(Cell& c, const KParams& P, u32 n) {
  for (u32 i = c.lane; i < n; i += 32) {
    if (c.bep[i] == UNBOUND) continue;
    const u64 rmv = min((u64)c.rm[i], pos64(c.rev[i]) - P.start);
    const u64 fmv = min((u64)c.fm[i], (u64)P.end - pos64(c.fwd[i]) - 1);
    c.rm[i] = (u32)rmv;
    c.fm[i] = (u32)fmv;
  }
  __syncwarp();
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

// detect_units_at_chrom_boundaries (simulation_detect_collisions.cpp:30-125); lane 0
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

// detect_lef_bar_collisions (simulation_detect_collisions.cpp:128-252); lane 0
__device__ void detect_lef_bar_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  u64 j = min(n5, n5 - 1);
  u32 unit_idx = c.rr[j];
  u64 unit_pos = pos64(c.rev[unit_idx]);
  bool rev_done = false;
  for (u32 i = 0; i < c.nb && !rev_done; ++i) {
    if (!bar_active(c, i)) continue;
    const u32 dir = c.bar[i].flags & BF_DIR_MASK;
    const Trial& tr = P.lef_bar[dir == MGPU_DIR_REV ? 0 : 1];
    const u64 bpos = c.bar[i].pos;
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
    const u32 dir = c.bar[i].flags & BF_DIR_MASK;
    const Trial& tr = P.lef_bar[dir == MGPU_DIR_FWD ? 0 : 1];
    const u64 bpos = c.bar[i].pos;
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
  return c.bar[idx].pos;
}

// detect_primary_lef_lef_collisions (simulation_detect_collisions.cpp:255-401); lane 0
__device__ void detect_primary_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
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
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
}

// correct_moves_for_lef_bar_collisions (simulation_correct_moves.cpp:20-51): warp-parallel
__device__ void correct_lef_bar(Cell& c, u32 n) {
  for (u32 i = c.lane; i < n; i += 32) {
    const u32 r = c.rc[i], f = c.fc[i];
    if (cw_occurred_as(r, EV_LEF_BAR)) c.rm[i] = (u32)(pos64(c.rev[i]) - c.bar[cw_idx(r)].pos - 1);
    if (cw_occurred_as(f, EV_LEF_BAR)) c.fm[i] = (u32)(c.bar[cw_idx(f)].pos - pos64(c.fwd[i]) - 1);
  }
  __syncwarp();
}

// correct_moves_for_primary_lef_lef_collisions (simulation_correct_moves.cpp:54-122):
// the pairs it visits are disjoint, so both passes are warp-parallel.
__device__ void correct_primary(Cell& c, u32 n) {
  for (u32 k = c.lane; k < n; k += 32) {
    const u32 rev_idx = c.rr[k];
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
  for (u32 k = c.lane; k < n; k += 32) {
    const u32 fwd_idx = c.fr[k];
    const u32 f = c.fc[fwd_idx];
    if (!cw_occurred_as(f, EV_PRIMARY)) continue;
    const u32 rev_idx = cw_idx(f);
    if (cw_occurred_as(c.rc[rev_idx], EV_LEF_BAR)) {
      c.fm[fwd_idx] = (u32)((pos64(c.rev[rev_idx]) - c.rm[rev_idx]) - pos64(c.fwd[fwd_idx]) - 1);
    }
  }
  __syncwarp();
}

// process_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:404-518); lane 0
__device__ void process_secondary_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
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

// fix_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:520-647); lane 0
__device__ void fix_secondary_serial(Cell& c, const KParams& P, u32 n, u64 n5, u64 n3) {
  const u64 start = P.start, end = P.end;
  const u64 num_active_fwd = n - min(n3, n3 - 1);
  for (u64 i = max((u64)1, n5); i < n; ++i) {
    const u32 idx2 = c.rr[i];
    if (!cw_avoided_as(c.rc[idx2], EV_SECONDARY)) continue;
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
    const u32 a = c.rr[i - 1], b = c.rr[i];
    c.rm[a] = (u32)min(pos64(c.rev[a]) - start, (u64)c.rm[a]);
    c.rm[b] = (u32)min(pos64(c.rev[b]) - start, (u64)c.rm[b]);
  }
  for (u64 i = 0; i + 1 < num_active_fwd; ++i) {
    const u32 idx1 = c.fr[i];
    if (!cw_avoided_as(c.fc[idx1], EV_SECONDARY)) continue;
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
    const u32 a = c.fr[i], b = c.fr[i + 1];
    c.fm[a] = (u32)min(end - 1 - pos64(c.fwd[a]), (u64)c.fm[a]);
    c.fm[b] = (u32)min(end - 1 - pos64(c.fwd[b]), (u64)c.fm[b]);
  }
}

// extrude (simulation.cpp:489-512): warp-parallel
__device__ void extrude(Cell& c, u32 n) {
  for (u32 i = c.lane; i < n; i += 32) {
    if (c.bep[i] == UNBOUND) continue;
    c.rev[i] -= c.rm[i];
    c.fwd[i] += c.fm[i];
  }
  __syncwarp();
}

// release_lefs (simulation.cpp:544-592): warp-parallel, one draw per bound LEF with p > 0.
__device__ u32 release_lefs(Cell& c, const KParams& P, u32 n, bool completed) {
  u32 released = 0;
  for (u32 base = 0; base < n; base += 32) {
    rng_ensure(c, 32);
    const u32 i = base + c.lane;
    const bool bound = i < n && c.bep[i] != UNBOUND;
    Trial tr{0, 0, 0};
    if (bound) {
      const u32 r = c.rc[i], f = c.fc[i];
      u32 nh = 0;
      if (cw_occurred_as(r, EV_LEF_BAR) && (c.bar[cw_idx(r)].flags & BF_DIR_MASK) == MGPU_DIR_REV) ++nh;
      if (cw_occurred_as(f, EV_LEF_BAR) && (c.bar[cw_idx(f)].flags & BF_DIR_MASK) == MGPU_DIR_FWD) ++nh;
      tr = P.release[completed ? 1 : 0][nh];
    }
    const bool need = bound && tr.draws;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
    const u32 off = __popc(m & lanemask_lt());
    const bool rel = need && ring_at(c, c.sc->rpos + off) <= tr.thr;
    if (rel) {
      c.rev[i] = UNBOUND;
      c.fwd[i] = UNBOUND;
      c.bep[i] = UNBOUND;
    }
    released += __popc(__ballot_sync(0xFFFFFFFFu, rel));
    __syncwarp();
    if (c.lane == 0) c.sc->rpos += __popc(m);
    __syncwarp();
  }
  return released;
}

// compute_loop_size_stats + evaluate_burnin (simulation.cpp:957-1025); lane 0.
__device__ bool burnin_stats_serial(Cell& c, const KParams& P, u32 n) {
  Scalars* sc = c.sc;
  const u32 cap = P.hist_cap;
  if (n == 0) {
    sc->hist_size = 0;
    sc->hist_head = 0;
  } else {
    u64 sum = 0;  // loop sizes are integers < 2^32: the double sum of the reference is exact
    for (u32 i = 0; i < n; ++i) sum += pos64(c.fwd[i]) - pos64(c.rev[i]);
    const double mean = (double)sum / (double)n;
    double ssd = 0.0;
    for (u32 i = 0; i < n; ++i) {
      const double d = (double)(pos64(c.fwd[i]) - pos64(c.rev[i])) - mean;
      ssd = ssd + (d * d);
    }
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
  if (sc->hist_size != cap) return false;
  const u32 w = P.smooth_w;
  auto ratio = [&](const double* d) {
    u64 nd = 0;
    for (u32 i1 = 1, i2 = w + 1; i2 != cap; ++i1, ++i2) {
      double a1 = 0.0, a2 = 0.0;
      for (u32 k = i1 - 1; k < i2 - 1; ++k) a1 = a1 + d[(sc->hist_head + k) % cap];
      for (u32 k = i1; k < i2; ++k) a2 = a2 + d[(sc->hist_head + k) % cap];
      const double n1 = a1 / (double)(i2 - i1), n2 = a2 / (double)(i2 - i1);
      nd += (n1 > n2) ? 1u : 0u;
    }
    return (double)nd / (double)((u64)cap - w - nd);
  };
  const double r1 = ratio(c.hcfx);
  if (!(r1 >= 0.95 && r1 <= 1.05)) return false;
  const double r2 = ratio(c.havg);
  return r2 >= 0.95 && r2 <= 1.05;
}

// run_burnin (simulation.cpp:1027-1054); lane 0
__device__ void run_burnin_serial(Cell& c, const KParams& P) {
  Scalars* sc = c.sc;
  for (u64 it = 0; it < MGPU_ITER_LIMIT; ++it) {
    ++sc->num_burnin_epochs;
    if (sc->num_active != P.nlefs) {
      const u64 k = s_poisson(c, P);
      sc->num_active = min(sc->num_active + k, (u64)P.nlefs);
    } else {
      bool done = burnin_stats_serial(c, P, (u32)sc->num_active);
      done = done && (sc->epoch > P.min_burnin);
      if (!done && sc->epoch >= P.max_burnin) done = true;
      sc->burnin_completed = done ? 1 : 0;
    }
    if (sc->num_active != 0) return;
  }
  set_status(c, DEV_ERR_ITER_LIMIT);
}

// ContactMatrixDense::increment (contact_matrix_dense_safe_impl.hpp:52-87)
__device__ __forceinline__ void band_increment(Cell& c, const KParams& P, u64 row, u64 col) {
  u64 i, j;
  if (row > col) {
    i = row - col;
    j = row;
  } else {
    i = col - row;
    j = col;
  }
  if (i >= P.nrows) {
    c.sc->missed++;
    return;
  }
  if (c.band) atomicAdd(&c.band[j * P.nrows + i], 1u);
}

// sample_and_register_contacts (register_contacts.cpp:94-198); lane 0
__device__ void sample_contacts_serial(Cell& c, const KParams& P, u64 target) {
  Scalars* sc = c.sc;
  u64 num = P.spe;
  if (P.density_positive) num = min(num, target - sc->num_contacts);
  if (num == 0) return;
  const u64 start = (u64)P.start + 1, end = (u64)P.end - 1;
  u64 n_loop;
  if (P.ratio_mode == 0) {
    n_loop = num;
  } else if (P.ratio_mode == 1) {
    n_loop = 0;
  } else {
    n_loop = (u64)s_binomial(c, P, (i64)num, P.p_loop);
  }
  const u64 n_tad = num - n_loop;
  const double ds = (double)start, de = (double)end;
  const u64 na = sc->num_active;
  // attempts budget: rejections are rare in a valid run (units at the chromosome ends, noise
  // outside the range); a chromosome where no LEF can register a contact ends with an error
  // instead of looping forever
  u64 budget = 1000 * num + 1000000;
  for (int pass = 0; pass < 2; ++pass) {
    u64 todo = pass == 0 ? n_loop : n_tad;
    while (todo != 0) {
      if (--budget == 0 || sc->status != DEV_OK) {
        set_status(c, DEV_ERR_NO_BOUND_LEF);
        return;
      }
      const u64 li = s_uniform_int(c, 0, na - 1);
      if (c.bep[li] == UNBOUND) continue;
      const u64 rp = pos64(c.rev[li]), fp = pos64(c.fwd[li]);
      if (!(rp > start && rp < end && fp > start && fp < end)) continue;
      const double n1 = P.noisify ? s_gev(c, P) : 0.0;
      const double a = (double)rp - n1;
      const double n2 = P.noisify ? s_gev(c, P) : 0.0;
      const double b = (double)fp + n2;
      const double p1 = fmin(a, b), p2 = fmax(a, b);
      if (!(p1 >= ds && p2 >= ds && p1 < de && p2 < de)) continue;
      if (pass == 0) {
        band_increment(c, P, ((u64)p1 - start) / P.bin, ((u64)p2 - start) / P.bin);
      } else {
        const u64 q1 = (u64)p1, q2 = (u64)p2;
        const u64 p11 = s_uniform_int(c, q1, q2);
        const u64 p22 = s_uniform_int(c, q1, q2);
        band_increment(c, P, (p11 - start) / P.bin, (p22 - start) / P.bin);
      }
      --todo;
    }
  }
  sc->num_contacts += num;
}

// mgpu_state_digest / trace record of one epoch: warp-parallel.
__device__ __forceinline__ u64 mix64(u64 z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ull;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebull;
  z ^= z >> 31;
  return z;
}

__device__ void trace_record(Cell& c, const KParams& P, const DevTrace& T, u64 rec) {
  const u32 nl = P.nlefs;
  const bool full = rec < T.max_records;
  u64 part = 0;
  for (u32 i = c.lane; i < nl; i += 32) {
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
  for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, off);
  if (c.lane == 0) {
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

// ---------------------------------------------------------------------------------------
// Cell setup and the epoch loop (simulation.cpp:1056-1152)
// ---------------------------------------------------------------------------------------
__device__ void carve(Cell& c, char* smem, const KParams& P, u32 nl) {
  char* p = smem;
  c.sc = reinterpret_cast<Scalars*>(p);
  p += 512;
  c.ring = reinterpret_cast<u64*>(p);
  p += (u64)RING * 8;
  c.hcfx = reinterpret_cast<double*>(p);
  p += (u64)P.hist_cap * 8;
  c.havg = reinterpret_cast<double*>(p);
  p += (u64)P.hist_cap * 8;
  c.bst = reinterpret_cast<u32*>(p);
  p += ((((u64)c.nb + 31) / 32) * 4 + 15) & ~15ull;
  u32* a = reinterpret_cast<u32*>(p);
  c.rev = a;
  c.fwd = a + nl;
  c.bep = a + 2 * (u64)nl;
  c.rr = a + 3 * (u64)nl;
  c.fr = a + 4 * (u64)nl;
  c.rm = a + 5 * (u64)nl;
  c.fm = a + 6 * (u64)nl;
  c.rc = a + 7 * (u64)nl;
  c.fc = a + 8 * (u64)nl;
  c.tmp = a + 9 * (u64)nl;
}

__device__ void cell_reset(Cell& c, u32 nl, u64 seed) {
  for (u32 i = c.lane; i < nl; i += 32) {
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
  for (u32 w = c.lane; w < (c.nb + 31) / 32; w += 32) c.bst[w] = 0;
  if (c.lane == 0) {
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
    sc->records = 0;
  }
  __syncwarp();
}

__device__ void run_cell(Cell& c, const KParams& P, const CellTask& task, u64 target_epochs,
                         const DevTrace* trace, mgpu_cell_stats* stats) {
  Scalars* sc = c.sc;
  const u32 nl = P.nlefs;
  cell_reset(c, nl, task.seed);
  barriers_init(c);
  if (P.skip_burnin && c.lane == 0) {
    sc->num_active = nl;
    sc->burnin_completed = 1;
  }
  __syncwarp();
  const u64 target = task.target_contacts;
  for (u64 guard = 0; guard < MGPU_ITER_LIMIT; ++guard) {
    const bool go = P.contact_mode ? (sc->num_contacts < target)
                                   : (sc->epoch - sc->num_burnin_epochs < target_epochs);
    if (!go) break;
    if (!sc->burnin_completed) {
      rng_ensure(c, RNG_BLOCK);
      if (c.lane == 0) run_burnin_serial(c, P);
      __syncwarp();
    }
    const u32 n = (u32)sc->num_active;
    const u32 epoch = (u32)sc->epoch;
    const bool completed = sc->burnin_completed != 0;
    if (c.lane == 0) sc->lef_epochs += n;
    bind_lefs(c, P, n, epoch, 0, nullptr);
    if (c.lane == 0) rank_lefs_serial(c, n, epoch != 0, false);
    __syncwarp();
    if (completed) {
      rng_ensure(c, RNG_BLOCK);
      if (c.lane == 0) sample_contacts_serial(c, P, target);
      __syncwarp();
      if (target != 0 && sc->num_contacts >= target) break;
      if (sc->status != DEV_OK) break;
    }
    gen_moves_dir(c, c.rm, n, P.rev_speed[completed], P.rev_std, P.rev_move_int[completed]);
    gen_moves_dir(c, c.fm, n, P.fwd_speed[completed], P.fwd_std, P.fwd_move_int[completed]);
    if (c.lane == 0) adjust_moves_serial(c, P, n);
    __syncwarp();
    clamp_moves(c, P, n);
    barriers_next(c);
    for (u32 i = c.lane; i < n; i += 32) {
      c.rc[i] = 0;
      c.fc[i] = 0;
    }
    __syncwarp();
    rng_ensure(c, RNG_BLOCK);
    if (c.lane == 0) {
      u64 n5, n3;
      detect_boundaries_serial(c, P, n, n5, n3);
      detect_lef_bar_serial(c, P, n, n5, n3);
      detect_primary_serial(c, P, n, n5, n3);
      sc->n5 = n5;
      sc->n3 = n3;
    }
    __syncwarp();
    correct_lef_bar(c, n);
    correct_primary(c, n);
    rng_ensure(c, RNG_BLOCK);
    if (c.lane == 0) {
      process_secondary_serial(c, P, n, sc->n5, sc->n3);
      fix_secondary_serial(c, P, n, sc->n5, sc->n3);
    }
    __syncwarp();
    extrude(c, n);
    release_lefs(c, P, n, completed);
    if (trace) trace_record(c, P, *trace, sc->epoch);
    if (c.lane == 0) sc->epoch++;
    __syncwarp();
    if (sc->status != DEV_OK) break;
  }
  if (c.lane == 0) {
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
                                                      u32 tracing, const ulonglong2* jt,
                                                      u32* work) {
  extern __shared__ __align__(16) char smem[];
  Cell c;
  c.lane = threadIdx.x & 31;
  c.bar = ch.barriers;
  c.nb = ch.nbarriers;
  c.jt = jt;
  c.band = band;
  carve(c, smem, P, P.nlefs);
  for (;;) {
    u32 cell = 0;
    if (c.lane == 0) cell = atomicAdd(work, 1u);
    cell = __shfl_sync(0xFFFFFFFFu, cell, 0);
    if (cell >= ncells) break;
    run_cell(c, P, tasks[cell], target_epochs, tracing ? &trace : nullptr,
             stats ? stats + cell : nullptr);
    if (c.lane == 0 && missed) atomicAdd((unsigned long long*)missed, (unsigned long long)c.sc->missed);
    __syncwarp();
  }
}

// One step of the epoch loop on caller state (mgpu_run_phase).
__global__ void __launch_bounds__(32) phase_kernel(const __grid_constant__ KParams P, DevChrom ch, int phase,
                                                   u32 n, u64* arrays, u64* bind_mask,
                                                   uint8_t* barrier_state, u64 epoch,
                                                   u32 burnin_completed, u32 partially_sorted,
                                                   u32 init_ranks, u32 adjust, u64* prng,
                                                   u64* outs, const ulonglong2* jt) {
  extern __shared__ __align__(16) char smem[];
  Cell c;
  c.lane = threadIdx.x & 31;
  c.bar = ch.barriers;
  c.nb = ch.nbarriers;
  c.jt = jt;
  c.band = nullptr;
  carve(c, smem, P, n);
  u64* A[9];
  for (int k = 0; k < 9; ++k) A[k] = arrays + (u64)k * n;
  for (u32 i = c.lane; i < n; i += 32) {
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
  for (u32 w = c.lane; w < (c.nb + 31) / 32; w += 32) {
    u32 bits = 0;
    for (u32 b = 0; b < 32; ++b) {
      const u32 i = w * 32 + b;
      if (i < c.nb && barrier_state && barrier_state[i]) bits |= 1u << b;
    }
    c.bst[w] = bits;
  }
  u64 init_state[4];
  for (int k = 0; k < 4; ++k) init_state[k] = prng[k];
  if (c.lane == 0) {
    Scalars* sc = c.sc;
    for (int k = 0; k < 4; ++k) sc->canon[k] = prng[k];
    sc->rpos = sc->gpos = 0;
    sc->lanes_stale = 1;
    sc->status = DEV_OK;
    sc->epoch = epoch;
    sc->num_active = n;
    sc->burnin_completed = burnin_completed;
  }
  __syncwarp();
  const bool completed = burnin_completed != 0;
  u64 n5 = 0, n3 = 0, released = 0;
  switch (phase) {
    case MGPU_PHASE_BIND:
      bind_lefs(c, P, n, (u32)epoch, bind_mask ? 1 : 2, bind_mask);
      if (c.lane == 0) rank_lefs_serial(c, n, epoch != 0, false);
      break;
    case MGPU_PHASE_RANK:
      if (c.lane == 0) rank_lefs_serial(c, n, partially_sorted != 0, init_ranks != 0);
      break;
    case MGPU_PHASE_ADJUST_AND_CLAMP:
      if (c.lane == 0) adjust_moves_serial(c, P, n);
      __syncwarp();
      clamp_moves(c, P, n);
      break;
    case MGPU_PHASE_GENERATE_MOVES:
      gen_moves_dir(c, c.rm, n, P.rev_speed[completed], P.rev_std, P.rev_move_int[completed]);
      gen_moves_dir(c, c.fm, n, P.fwd_speed[completed], P.fwd_std, P.fwd_move_int[completed]);
      if (adjust && c.lane == 0) adjust_moves_serial(c, P, n);
      __syncwarp();
      clamp_moves(c, P, n);
      break;
    case MGPU_PHASE_PROCESS_COLLISIONS:
      rng_ensure(c, RNG_BLOCK);
      if (c.lane == 0) {
        detect_boundaries_serial(c, P, n, n5, n3);
        detect_lef_bar_serial(c, P, n, n5, n3);
        detect_primary_serial(c, P, n, n5, n3);
        c.sc->n5 = n5;
        c.sc->n3 = n3;
      }
      __syncwarp();
      correct_lef_bar(c, n);
      correct_primary(c, n);
      if (c.lane == 0) process_secondary_serial(c, P, n, c.sc->n5, c.sc->n3);
      n5 = c.sc->n5;
      n3 = c.sc->n3;
      break;
    case MGPU_PHASE_FIX_SECONDARY:
      if (c.lane == 0) fix_secondary_serial(c, P, n, 0, 0);
      break;
    case MGPU_PHASE_DETECT_LEF_BAR:
      if (c.lane == 0) detect_lef_bar_serial(c, P, n, 0, 0);
      break;
    case MGPU_PHASE_LEF_LEF:
      if (c.lane == 0) detect_primary_serial(c, P, n, 0, 0);
      __syncwarp();
      correct_primary(c, n);
      if (c.lane == 0) process_secondary_serial(c, P, n, 0, 0);
      break;
    case MGPU_PHASE_DETECT_PRIMARY:
      if (c.lane == 0) detect_primary_serial(c, P, n, 0, 0);
      break;
    case MGPU_PHASE_DETECT_BOUNDARIES:
      if (c.lane == 0) {
        detect_boundaries_serial(c, P, n, n5, n3);
        c.sc->n5 = n5;
        c.sc->n3 = n3;
      }
      __syncwarp();
      n5 = c.sc->n5;
      n3 = c.sc->n3;
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
      released = release_lefs(c, P, n, completed);
      break;
    case MGPU_PHASE_BARRIER_NEXT:
      barriers_next(c);
      break;
    case MGPU_PHASE_BARRIER_INIT:
      barriers_init(c);
      break;
    default:
      break;
  }
  __syncwarp();
  for (u32 i = c.lane; i < n; i += 32) {
    A[0][i] = pos64(c.rev[i]);
    A[1][i] = pos64(c.fwd[i]);
    A[2][i] = pos64(c.bep[i]);
    A[3][i] = c.rr[i];
    A[4][i] = c.fr[i];
    A[5][i] = c.rm[i];
    A[6][i] = c.fm[i];
    A[7][i] = cw_to_ref(c.rc[i]);
    A[8][i] = cw_to_ref(c.fc[i]);
  }
  for (u32 i = c.lane; i < c.nb; i += 32) {
    if (barrier_state) barrier_state[i] = bar_active(c, i) ? 1 : 0;
  }
  if (c.lane == 0) {
    // the caller's PRNG advanced by exactly the number of draws consumed
    u64 s[4] = {init_state[0], init_state[1], init_state[2], init_state[3]};
    for (u64 k = 0; k < c.sc->rpos; ++k) xo_next(s);
    for (int k = 0; k < 4; ++k) prng[k] = s[k];
    outs[0] = n5;
    outs[1] = n3;
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

u64 max_smem_per_block() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return (u64)v;
}

int launch_simulate(const KParams& P, const DevChrom& ch, const CellTask* tasks, u64 ncells,
                    u64 target_epochs, u32* band, u64* missed, mgpu_cell_stats* stats,
                    const DevTrace* trace, const void* jump_table, u32* work_counter,
                    void* stream, char* errbuf, int errlen) {
  const u64 smem = cell_smem_bytes(P.nlefs, ch.nbarriers, P.hist_cap);
  int rc = cuda_fail(cudaFuncSetAttribute(simulate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem),
                     "cudaFuncSetAttribute", errbuf, errlen);
  if (rc) return rc;
  int per_sm = 0;
  rc = cuda_fail(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, simulate_kernel, 32, smem),
                 "occupancy", errbuf, errlen);
  if (rc) return rc;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  u64 grid = (u64)sms * (u64)(per_sm > 0 ? per_sm : 1);
  if (grid > ncells) grid = ncells;
  if (grid == 0) return MGPU_OK;
  cudaStream_t st = (cudaStream_t)stream;
  rc = cuda_fail(cudaMemsetAsync(work_counter, 0, sizeof(u32), st), "memset", errbuf, errlen);
  if (rc) return rc;
  DevTrace tr{};
  u32 tracing = 0;
  if (trace) {
    tr = *trace;
    tracing = 1;
  }
  simulate_kernel<<<(unsigned)grid, 32, smem, st>>>(P, ch, tasks, ncells, target_epochs, band,
                                                    missed, stats,
                                                    tr, tracing,
                                                    (const ulonglong2*)jump_table, work_counter);
  return cuda_fail(cudaGetLastError(), "simulate_kernel launch", errbuf, errlen);
}

int launch_phase(const KParams& P, const DevChrom& ch, int phase, u64 n, u64* arrays,
                 u64* bind_mask, uint8_t* barrier_state, u64 epoch, u32 burnin_completed,
                 u32 partially_sorted, u32 init_ranks, u32 adjust, u64* prng_state, u64* outs,
                 const void* jump_table, void* stream, char* errbuf, int errlen) {
  const u64 smem = cell_smem_bytes(n, ch.nbarriers, P.hist_cap);
  int rc = cuda_fail(cudaFuncSetAttribute(phase_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem),
                     "cudaFuncSetAttribute", errbuf, errlen);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  phase_kernel<<<1, 32, smem, st>>>(P, ch, phase, (u32)n, arrays, bind_mask, barrier_state,
                                     epoch, burnin_completed, partially_sorted, init_ranks, adjust,
                                     prng_state, outs, (const ulonglong2*)jump_table);
  return cuda_fail(cudaGetLastError(), "phase_kernel launch", errbuf, errlen);
}

}  // namespace mgpu
