// modle_oracle.cpp - CPU ORACLE FOR THE TEST-SUITE. NOT PART OF THE PRODUCT.
//
// A line-by-line C++17 restatement of MoDLE's per-cell epoch loop
// (Simulation::simulate_one_cell, src/libmodle/cpu/simulation.cpp:1056-1152) and of every
// step it calls.  Only the test-suite, __graft_entry__.smoke() and the CPU-baseline leg of
// bench.py load this library, and only to check or time the reference algorithm; the
// product (modlefork_gb300/) never links or calls it.
//
// The reference itself cannot be compiled here: its third-party dependencies
// (conanfile.py:17-40) are absent.  The parts of the algorithm that live in those
// dependencies are restated from their published definitions:
//   * xoshiro-cpp 1.1: SplitMix64 seeding and Xoshiro256++ (Vigna & Blackman, 2018);
//   * Boost.Random 1.79 (WITH_BOOST_RANDOM=ON, CMakeLists.txt:107): uniform_int_distribution
//     (bucket rejection), bernoulli_distribution, generate_canonical, uniform_01,
//     normal_distribution and exponential_distribution (128/256-layer ziggurat, Marsaglia &
//     Tsang 2000, tables from ziggurat_tables.h), poisson_distribution (inversion below mean
//     10, PTRS transformed rejection of Hoermann 1993 above), binomial_distribution
//     (inversion for m < 11, BTRD of Hoermann 1993 above);
//   * cpp-sort 1.13: split_sort, pdq_sort (Peters' pattern-defeating quicksort) and
//     insertion_sort, used by rank_lefs and ExtrusionBarriers::sort.
// glibc libm supplies log, exp, pow and sqrt, as in the reference.
//
// Build: see oracle/Makefile (g++ -O3 -std=c++17 -ffp-contract=off).

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <numeric>
#include <thread>
#include <utility>
#include <vector>

#include "../include/mgpu_modle.h"
#include "../modlefork_gb300/csrc/ziggurat_tables.h"

namespace orc {

using u8 = uint8_t;
using u32 = uint32_t;
using u64 = uint64_t;
using i64 = int64_t;
using usize = uint64_t;
using isize = int64_t;
using bp_t = uint64_t;
static constexpr u64 U64MAX = std::numeric_limits<u64>::max();
static constexpr double TWO64 = 18446744073709551616.0;

// Full-tie counters of rank_lefs (off unless orc_tie_counters enables them, so that the timed
// CPU baseline runs the reference's work only).
static std::atomic<bool> g_count_ties{false};
static std::atomic<u64> g_tie_rank_calls{0}, g_tie_calls{0}, g_tie_pairs{0}, g_tie_interior{0};

// ---------------------------------------------------------------------------------------
// PRNG: random::PRNG (src/common/include/modle/common/random.hpp:26-30)
// ---------------------------------------------------------------------------------------
struct SplitMix64 {
  u64 state;
  u64 next() {
    u64 z = (state += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  }
};

static inline u64 rotl(u64 x, int k) { return (x << k) | (x >> (64 - k)); }

struct Rng {
  u64 s[4];
  u64 ndraws = 0;
  u64 operator()() {
    const u64 result = rotl(s[0] + s[3], 23) + s[0];
    const u64 t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    ++ndraws;
    return result;
  }
};

static Rng make_prng(u64 seed) {
  SplitMix64 sm{seed};
  Rng r;
  for (auto& w : r.s) w = sm.next();
  return r;
}

// ---------------------------------------------------------------------------------------
// Distributions (Boost.Random 1.79, aliases in random.hpp:34-53)
// ---------------------------------------------------------------------------------------

// uniform_int_distribution<u64>{a, b}: generate_uniform_int for a 64-bit engine.
static u64 uniform_int(Rng& g, u64 a, u64 b) {
  const u64 range = b - a;
  if (range == 0) return a;
  const u64 brange = U64MAX;
  if (range == brange) return g() + a;
  u64 bucket = brange / (range + 1);
  if (brange % (range + 1) == range) ++bucket;
  for (;;) {
    const u64 r = g() / bucket;
    if (r <= range) return a + r;
  }
}

// bernoulli_distribution<double>{p}: no draw when p == 0.
static bool bernoulli(Rng& g, double p) {
  if (p == 0.0) return false;
  return static_cast<double>(g()) <= p * TWO64;
}

// generate_canonical<double, 53>: one draw scaled by 2^-64, 1.0 mapped to 1 - eps/2.
static double canonical53(Rng& g) {
  const double S = static_cast<double>(g());
  double r = S / TWO64;
  if (r == 1.0) r -= DBL_EPSILON / 2;
  return r;
}

// uniform_01<double>: draw * 2^-64, retried while the result rounds to 1.
static double uniform01(Rng& g) {
  for (;;) {
    const double r = static_cast<double>(g()) * (1.0 / TWO64);
    if (r < 1.0) return r;
  }
}

// generate_int_float_pair<double, 8>: low 8 bits give the layer, the high 56 bits the
// fraction; bit 11 is cleared before the 56-bit value is converted ("zero out unused bits").
static std::pair<double, int> int_float_pair8(Rng& g) {
  u64 u = g();
  const int bucket = static_cast<int>(u & 0xFFu);
  u &= ~(u64(1) << 11);
  const double r = static_cast<double>(u >> 8) * (1.0 / 72057594037927936.0);
  return {r, bucket};
}

// unit_exponential_distribution: 256-layer ziggurat; the tail repeats the body shifted by x_1.
static double unit_exponential(Rng& g) {
  double shift = 0;
  for (;;) {
    const auto [r, i] = int_float_pair8(g);
    const double x = r * mgpu_zig_exp_x[i];
    if (x < mgpu_zig_exp_x[i + 1]) return shift + x;
    if (i == 0) {
      shift += mgpu_zig_exp_x[1];
    } else {
      const double y01 = uniform01(g);
      const double y = mgpu_zig_exp_y[i] + y01 * (mgpu_zig_exp_y[i + 1] - mgpu_zig_exp_y[i]);
      if (y < std::exp(-x)) return x + shift;
    }
  }
}

// unit_normal_distribution::generate_tail: exponential(x_1) offsets accepted when 2y > x^2.
static double normal_tail(Rng& g) {
  const double tail_start = mgpu_zig_normal_x[1];
  for (;;) {
    const double x = unit_exponential(g) / tail_start;
    const double y = unit_exponential(g) / 1.0;
    if (2 * y > x * x) return x + tail_start;
  }
}

// unit_normal_distribution: 128 layers, bit 0 of the layer byte is the sign.
static double unit_normal(Rng& g) {
  for (;;) {
    const auto [r, ii] = int_float_pair8(g);
    const int sign = (ii & 1) * 2 - 1;
    const int i = ii >> 1;
    const double x = r * mgpu_zig_normal_x[i];
    if (x < mgpu_zig_normal_x[i + 1]) return x * sign;
    if (i == 0) return normal_tail(g) * sign;
    const double y01 = uniform01(g);
    const double y =
        mgpu_zig_normal_y[i] + y01 * (mgpu_zig_normal_y[i + 1] - mgpu_zig_normal_y[i]);
    if (y < std::exp(-(x * x / 2))) return x * sign;
  }
}

// normal_distribution<double>{mean, sigma}
static double normal(Rng& g, double mean, double sigma) { return unit_normal(g) * sigma + mean; }

// poisson_distribution<usize>{mean}
static const double kLogFactorial[10] = {0.0,
                                         0.0,
                                         0.69314718055994529,
                                         1.7917594692280550,
                                         3.1780538303479458,
                                         4.7874917427820458,
                                         6.5792512120101012,
                                         8.5251613610654147,
                                         10.604602902745251,
                                         12.801827480081469};

static u64 poisson(Rng& g, double mean) {
  if (mean < 10) {  // inversion
    double p = std::exp(-mean);
    u64 x = 0;
    double u = uniform01(g);
    while (u > p) {
      u = u - p;
      ++x;
      p = mean * p / static_cast<double>(x);
    }
    return x;
  }
  // PTRS
  const double smu = std::sqrt(mean);
  const double b = 0.931 + 2.53 * smu;
  const double a = -0.059 + 0.02483 * b;
  const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
  const double v_r = 0.9277 - 3.6224 / (b - 2);
  for (;;) {
    double u;
    double v = uniform01(g);
    if (v <= 0.86 * v_r) {
      u = v / v_r - 0.43;
      return static_cast<u64>(std::floor((2 * a / (0.5 - std::abs(u)) + b) * u + mean + 0.445));
    }
    if (v >= v_r) {
      u = uniform01(g) - 0.5;
    } else {
      u = v / v_r - 0.93;
      u = ((u < 0) ? -0.5 : 0.5) - u;
      v = uniform01(g) * v_r;
    }
    const double us = 0.5 - std::abs(u);
    if (us < 0.013 && v > us) continue;
    const double k = std::floor((2 * a / us + b) * u + mean + 0.43);
    v = v * inv_alpha / (a / (us * us) + b);
    const double log_sqrt_2pi = 0.91893853320467267;
    if (k >= 10) {
      if (std::log(v * smu) <= (k + 0.5) * std::log(mean / k) - mean - log_sqrt_2pi + k -
                                   (1 / 12. - (1 / 360. - 1 / (1260. * k * k)) / (k * k)) / k) {
        return static_cast<u64>(k);
      }
    } else if (k >= 0) {
      if (std::log(v) <= k * std::log(mean) - mean - kLogFactorial[static_cast<int>(k)]) {
        return static_cast<u64>(k);
      }
    }
  }
}

// binomial_distribution<isize>{t, p}
static const double kBinomialFc[10] = {0.08106146679532726, 0.04134069595540929,
                                       0.02767792568499834, 0.02079067210376509,
                                       0.01664469118982119, 0.01387612882307075,
                                       0.01189670994589177, 0.01041126526197209,
                                       0.009255462182712733, 0.008330563433362871};

static double binomial_fc(i64 k) {
  if (k < 10) return kBinomialFc[k];
  const double ikp1 = 1.0 / static_cast<double>(k + 1);
  return (1.0 / 12 - (1.0 / 360 - (1.0 / 1260) * (ikp1 * ikp1)) * (ikp1 * ikp1)) * ikp1;
}

static i64 binomial(Rng& g, i64 t_, double p_) {
  const double p = (0.5 < p_) ? (1 - p_) : p_;
  const i64 t = t_;
  const i64 m = static_cast<i64>((t + 1) * p);
  const bool inversion = m < 11;
  if (inversion) {
    const double q_n = std::pow((1 - p), static_cast<double>(t));
    auto invert = [&](i64 tt, double pp) -> i64 {
      const double q = 1 - pp;
      const double s = pp / q;
      const double a = (tt + 1) * s;
      double r = q_n;
      double u = uniform01(g);
      i64 x = 0;
      while (u > r) {
        u = u - r;
        ++x;
        const double r1 = ((a / x) - s) * r;
        if (r1 < std::numeric_limits<double>::epsilon() && r1 < r) break;
        r = r1;
      }
      return x;
    };
    if (0.5 < p_) return t_ - invert(t_, 1 - p_);
    return invert(t_, p_);
  }
  // BTRD
  const double r = p / (1 - p);
  const double nr = (t + 1) * r;
  const double npq = t * p * (1 - p);
  const double sqrt_npq = std::sqrt(npq);
  const double b = 1.15 + 2.53 * sqrt_npq;
  const double a = -0.0873 + 0.0248 * b + 0.01 * p;
  const double c = t * p + 0.5;
  const double alpha = (2.83 + 5.1 / b) * sqrt_npq;
  const double v_r = 0.92 - 4.2 / b;
  const double u_rv_r = 0.86 * v_r;
  auto generate = [&]() -> i64 {
    for (;;) {
      double u;
      double v = uniform01(g);
      if (v <= u_rv_r) {
        u = v / v_r - 0.43;
        return static_cast<i64>(std::floor((2 * a / (0.5 - std::abs(u)) + b) * u + c));
      }
      if (v >= v_r) {
        u = uniform01(g) - 0.5;
      } else {
        u = v / v_r - 0.93;
        u = ((u < 0) ? -0.5 : 0.5) - u;
        v = uniform01(g) * v_r;
      }
      const double us = 0.5 - std::abs(u);
      const i64 k = static_cast<i64>(std::floor((2 * a / us + b) * u + c));
      if (k < 0 || k > t) continue;
      v = v * alpha / (a / (us * us) + b);
      const double km = std::abs(static_cast<double>(k - m));
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
        if (v <= f) return k;
        continue;
      }
      v = std::log(v);
      const double rho = (km / npq) * (((km / 3. + 0.625) * km + 1. / 6) / npq + 0.5);
      const double tt = -km * km / (2 * npq);
      if (v < tt - rho) return k;
      if (v > tt + rho) continue;
      const i64 nm = t - m + 1;
      const double h = (m + 0.5) * std::log((m + 1) / (r * nm)) + binomial_fc(m) + binomial_fc(t - m);
      const i64 nk = t - k + 1;
      if (v <= h + (t + 1) * std::log(static_cast<double>(nm) / nk) +
                   (k + 0.5) * std::log(nk * r / (k + 1)) - binomial_fc(k) - binomial_fc(t - k)) {
        return k;
      }
    }
  };
  if (0.5 < p_) return t_ - generate();
  return generate();
}

// genextreme_value_distribution<double> (genextreme_value_distribution.hpp:87-105)
static double gev(Rng& g, double mu, double sigma, double xi) {
  if (xi == 0.0) return (mu - sigma) * std::log(-std::log(canonical53(g)));
  return mu + (sigma * (1.0 - std::pow(-std::log(canonical53(g)), xi))) / xi;
}

// ---------------------------------------------------------------------------------------
// Collision word: Collision<u32f> (collision_encoding.hpp:54-108, impl :74-240).
// u32f is uint_fast32_t, a 64-bit word on LP64 Linux, so INDEX_BITS = 64 - 8 = 56.
// ---------------------------------------------------------------------------------------
static constexpr u8 NO_COLLISION = 0, COLLISION = 0x10, CHROM_BOUNDARY = 0x08, LEF_BAR = 0x04,
                    LEF_LEF_PRIMARY = 0x02, LEF_LEF_SECONDARY = 0x01;

struct Coll {
  static constexpr unsigned IB = 56;
  static constexpr u64 EVENT_MASK = (~u64(0)) << (IB - 1);
  static constexpr u64 INDEX_MASK = ~EVENT_MASK;
  u64 w = 0;
  void clear() { w = 0; }
  void set(u64 idx, u8 event) {
    w = 0;
    w |= idx & INDEX_MASK;
    w |= u64(event) << IB;
  }
  u64 idx() const { return w & INDEX_MASK; }
  u8 event() const { return static_cast<u8>(w >> IB); }
  bool occurred() const { return (w & (u64(COLLISION) << IB)) != 0; }
  bool occurred(u8 c) const { return event() == (c | COLLISION); }
  bool avoided(u8 c) const { return !occurred() && event() == c; }
};

// Lef / ExtrusionUnit (extrusion_factors.hpp:55-66, impl :94-122)
struct Lef {
  u64 binding_epoch = U64MAX;
  bp_t rev = U64MAX;
  bp_t fwd = U64MAX;
  bool bound() const { return binding_epoch != U64MAX; }
  void bind(u64 epoch, bp_t pos) {
    rev = pos;
    fwd = pos;
    binding_epoch = epoch;
  }
  void release() {
    rev = U64MAX;
    fwd = U64MAX;
    binding_epoch = U64MAX;
  }
  bp_t loop_size() const { return fwd - rev; }
};

// ---------------------------------------------------------------------------------------
// cpp-sort 1.13 emulation: insertion_sort, pdq_sort, split_sort
// ---------------------------------------------------------------------------------------
namespace sorting {

template <class It, class Cmp>
void insertion_sort(It first, It last, Cmp comp) {
  if (first == last) return;
  for (It cur = first + 1; cur != last; ++cur) {
    It sift = cur;
    It sift_1 = cur - 1;
    if (comp(*sift, *sift_1)) {
      auto tmp = *sift;
      do {
        *sift-- = *sift_1;
      } while (sift != first && comp(tmp, *--sift_1));
      *sift = tmp;
    }
  }
}

template <class It, class Cmp>
void unguarded_insertion_sort(It first, It last, Cmp comp) {
  if (first == last) return;
  for (It cur = first + 1; cur != last; ++cur) {
    It sift = cur;
    It sift_1 = cur - 1;
    if (comp(*sift, *sift_1)) {
      auto tmp = *sift;
      do {
        *sift-- = *sift_1;
      } while (comp(tmp, *--sift_1));
      *sift = tmp;
    }
  }
}

template <class It, class Cmp>
bool partial_insertion_sort(It first, It last, Cmp comp) {
  if (first == last) return true;
  std::size_t limit = 0;
  for (It cur = first + 1; cur != last; ++cur) {
    It sift = cur;
    It sift_1 = cur - 1;
    if (comp(*sift, *sift_1)) {
      auto tmp = *sift;
      do {
        *sift-- = *sift_1;
      } while (sift != first && comp(tmp, *--sift_1));
      *sift = tmp;
      limit += static_cast<std::size_t>(cur - sift);
    }
    if (limit > 8) return false;
  }
  return true;
}

template <class It, class Cmp>
void sort2(It a, It b, Cmp comp) {
  if (comp(*b, *a)) std::iter_swap(a, b);
}

template <class It, class Cmp>
void sort3(It a, It b, It c, Cmp comp) {
  sort2(a, b, comp);
  sort2(b, c, comp);
  sort2(a, b, comp);
}

template <class It, class Cmp>
std::pair<It, bool> partition_right(It begin, It end, Cmp comp) {
  auto pivot = *begin;
  It first = begin;
  It last = end;
  while (comp(*++first, pivot)) {
  }
  if (first - 1 == begin) {
    while (first < last && !comp(*--last, pivot)) {
    }
  } else {
    while (!comp(*--last, pivot)) {
    }
  }
  const bool already_partitioned = first >= last;
  while (first < last) {
    std::iter_swap(first, last);
    while (comp(*++first, pivot)) {
    }
    while (!comp(*--last, pivot)) {
    }
  }
  It pivot_pos = first - 1;
  *begin = *pivot_pos;
  *pivot_pos = pivot;
  return {pivot_pos, already_partitioned};
}

template <class It, class Cmp>
It partition_left(It begin, It end, Cmp comp) {
  auto pivot = *begin;
  It first = begin;
  It last = end;
  while (comp(pivot, *--last)) {
  }
  if (last + 1 == end) {
    while (first < last && !comp(pivot, *++first)) {
    }
  } else {
    while (!comp(pivot, *++first)) {
    }
  }
  while (first < last) {
    std::iter_swap(first, last);
    while (comp(pivot, *--last)) {
    }
    while (!comp(pivot, *++first)) {
    }
  }
  It pivot_pos = last;
  *begin = *pivot_pos;
  *pivot_pos = pivot;
  return pivot_pos;
}

// Heap fallback with the sift-down-to-leaf then push-up scheme of libstdc++.
template <class It, class Cmp, class T>
void push_heap_(It first, isize hole, isize top, T value, Cmp comp) {
  isize parent = (hole - 1) / 2;
  while (hole > top && comp(*(first + parent), value)) {
    *(first + hole) = *(first + parent);
    hole = parent;
    parent = (hole - 1) / 2;
  }
  *(first + hole) = value;
}

template <class It, class Cmp, class T>
void adjust_heap_(It first, isize hole, isize len, T value, Cmp comp) {
  const isize top = hole;
  isize child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (comp(*(first + child), *(first + (child - 1)))) child--;
    *(first + hole) = *(first + child);
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    *(first + hole) = *(first + (child - 1));
    hole = child - 1;
  }
  push_heap_(first, hole, top, value, comp);
}

template <class It, class Cmp>
void heap_sort(It first, It last, Cmp comp) {
  const isize len = last - first;
  if (len < 2) return;
  for (isize parent = (len - 2) / 2;; --parent) {
    auto v = *(first + parent);
    adjust_heap_(first, parent, len, v, comp);
    if (parent == 0) break;
  }
  while (last - first > 1) {
    --last;
    auto v = *last;
    *last = *first;
    adjust_heap_(first, isize(0), isize(last - first), v, comp);
  }
}

template <class It, class Cmp>
void pdqsort_loop(It begin, It end, Cmp comp, int bad_allowed, bool leftmost = true) {
  for (;;) {
    const isize size = end - begin;
    if (size < 24) {
      if (leftmost) {
        insertion_sort(begin, end, comp);
      } else {
        unguarded_insertion_sort(begin, end, comp);
      }
      return;
    }
    const isize s2 = size / 2;
    if (size > 128) {
      sort3(begin, begin + s2, end - 1, comp);
      sort3(begin + 1, begin + (s2 - 1), end - 2, comp);
      sort3(begin + 2, begin + (s2 + 1), end - 3, comp);
      sort3(begin + (s2 - 1), begin + s2, begin + (s2 + 1), comp);
      std::iter_swap(begin, begin + s2);
    } else {
      sort3(begin + s2, begin, end - 1, comp);
    }
    if (!leftmost && !comp(*(begin - 1), *begin)) {
      begin = partition_left(begin, end, comp) + 1;
      continue;
    }
    const auto [pivot_pos, already_partitioned] = partition_right(begin, end, comp);
    const isize l_size = pivot_pos - begin;
    const isize r_size = end - (pivot_pos + 1);
    const bool highly_unbalanced = l_size < size / 8 || r_size < size / 8;
    if (highly_unbalanced) {
      if (--bad_allowed == 0) {
        heap_sort(begin, end, comp);
        return;
      }
      if (l_size >= 24) {
        std::iter_swap(begin, begin + l_size / 4);
        std::iter_swap(pivot_pos - 1, pivot_pos - l_size / 4);
        if (l_size > 128) {
          std::iter_swap(begin + 1, begin + (l_size / 4 + 1));
          std::iter_swap(begin + 2, begin + (l_size / 4 + 2));
          std::iter_swap(pivot_pos - 2, pivot_pos - (l_size / 4 + 1));
          std::iter_swap(pivot_pos - 3, pivot_pos - (l_size / 4 + 2));
        }
      }
      if (r_size >= 24) {
        std::iter_swap(pivot_pos + 1, pivot_pos + (1 + r_size / 4));
        std::iter_swap(end - 1, end - r_size / 4);
        if (r_size > 128) {
          std::iter_swap(pivot_pos + 2, pivot_pos + (2 + r_size / 4));
          std::iter_swap(pivot_pos + 3, pivot_pos + (3 + r_size / 4));
          std::iter_swap(end - 2, end - (1 + r_size / 4));
          std::iter_swap(end - 3, end - (2 + r_size / 4));
        }
      }
    } else {
      if (already_partitioned && partial_insertion_sort(begin, pivot_pos, comp) &&
          partial_insertion_sort(pivot_pos + 1, end, comp)) {
        return;
      }
    }
    pdqsort_loop(begin, pivot_pos, comp, bad_allowed, leftmost);
    begin = pivot_pos + 1;
    leftmost = false;
  }
}

template <class It, class Cmp>
void pdq_sort(It begin, It end, Cmp comp) {
  if (begin == end) return;
  isize n = end - begin;
  int log = 0;
  while (n >>= 1) ++log;
  pdqsort_loop(begin, end, comp, log);
}

// Stable merge of [first, middle) and [middle, last); equal keys keep left-then-right order.
template <class It, class Cmp>
void stable_merge(It first, It middle, It last, Cmp comp) {
  std::vector<typename std::iterator_traits<It>::value_type> buf(first, middle);
  auto l = buf.begin();
  auto r = middle;
  auto out = first;
  while (l != buf.end() && r != last) {
    if (comp(*r, *l)) {
      *out++ = *r++;
    } else {
      *out++ = *l++;
    }
  }
  while (l != buf.end()) *out++ = *l++;
}

// split_sort: keep an approximate longest ascending subsequence on the left, move the other
// elements right, sort them with pdq_sort and merge.
template <class It, class Cmp>
void split_sort(It first, It last, Cmp comp) {
  if (last - first < 2) return;
  It middle = first;
  for (It reader = first + 1; reader != last; ++reader) {
    if (comp(*reader, *middle)) {
      if (middle != first) --middle;
    } else {
      ++middle;
      std::iter_swap(middle, reader);
    }
  }
  pdq_sort(middle + 1, last, comp);
  stable_merge(first, middle + 1, last, comp);
}

}  // namespace sorting

// ---------------------------------------------------------------------------------------
// Barriers: ExtrusionBarriers SoA (extrusion_barriers.hpp:32-102, .cpp:145-259)
// ---------------------------------------------------------------------------------------
struct Barriers {
  std::vector<bp_t> pos;
  std::vector<u32> dir;
  std::vector<double> stp_active, stp_inactive;
  std::vector<u8> state;  // 1 = ACTIVE (occupied)
  usize size() const { return pos.size(); }
  bool is_active(usize i) const { return state[i] == 1; }
  bool is_not_active(usize i) const { return state[i] == 0; }

  // compute_occupancy_from_stp (extrusion_barriers_impl.hpp:118-128)
  static double occupancy_from_stp(double sa, double si) {
    if (sa + si == 0) return 0.0;
    const double tp_inactive_to_active = 1.0 - si;
    const double tp_active_to_inactive = 1.0 - sa;
    const double occ = tp_inactive_to_active / (tp_inactive_to_active + tp_active_to_inactive);
    return std::clamp(occ, 0.0, 1.0);
  }
  // init_states (extrusion_barriers.cpp:220-231)
  void init_states(Rng& g) {
    for (usize i = 0; i < size(); ++i) {
      state[i] = bernoulli(g, occupancy_from_stp(stp_active[i], stp_inactive[i])) ? 1 : 0;
    }
  }
  // next_state (extrusion_barriers.cpp:145-161)
  void next_state(Rng& g) {
    for (usize i = 0; i < size(); ++i) {
      const double p = canonical53(g);
      if (is_not_active(i) && p > stp_inactive[i]) {
        state[i] = 1;
      } else if (is_active(i) && p > stp_active[i]) {
        state[i] = 0;
      }
    }
  }
  // sort (extrusion_barriers.cpp:234-259): pdq_sort of indices by position, then apply.
  void sort() {
    std::vector<usize> idx(size());
    std::iota(idx.begin(), idx.end(), usize(0));
    sorting::pdq_sort(idx.begin(), idx.end(), [&](usize a, usize b) { return pos[a] < pos[b]; });
    for (usize i = 0; i < size(); ++i) {
      while (idx[i] != i) {
        const usize j = idx[i];
        const usize k = idx[j];
        std::swap(pos[j], pos[k]);
        std::swap(dir[j], dir[k]);
        std::swap(stp_active[j], stp_active[k]);
        std::swap(stp_inactive[j], stp_inactive[k]);
        std::swap(state[j], state[k]);
        std::swap(idx[i], idx[j]);
      }
    }
  }
};

// ContactMatrixDense<u32> band (contact_matrix_dense_impl.hpp:40-51, safe_impl.hpp:52-87)
struct Band {
  usize nrows = 0, ncols = 0;
  u32* data = nullptr;  // nrows*ncols, column-major; may be null (contacts only counted)
  bool atomic = false;
  u64 missed = 0;
  u64 in_band = 0;
  void increment(usize row, usize col) {
    usize i, j;  // transpose_coords (contact_matrix_internal_impl.hpp:19-24)
    if (row > col) {
      i = row - col;
      j = row;
    } else {
      i = col - row;
      j = col;
    }
    if (i >= nrows) {
      ++missed;
      return;
    }
    ++in_band;
    if (!data) return;
    u32* px = data + (j * nrows + i);  // encode_idx (contact_matrix_internal_impl.hpp:40-42)
    if (atomic) {
      __atomic_fetch_add(px, 1u, __ATOMIC_RELAXED);
    } else {
      ++*px;
    }
  }
};

// Chromosome range (move clamps, boundary collisions) and the simulated window (binding,
// contacts, band): the window is the whole range for modle simulate and a part of it for the
// windows of modle perturbate (Simulation::select_and_bind_lefs and
// sample_and_register_contacts, simulation.cpp:1154-1164, register_contacts.cpp:107-108).
struct Chrom {
  bp_t start, end;
  bp_t ws, we;
};

// Post-transform Config fields read by the epoch loop.
struct Cfg {
  mgpu_config c;
};

// ---------------------------------------------------------------------------------------
// Simulation steps (src/libmodle/cpu/simulation*.cpp)
// ---------------------------------------------------------------------------------------
struct Sim {
  const mgpu_config& c;
  explicit Sim(const mgpu_config& cfg) : c(cfg) {}

  // bind_lefs (simulation_impl.hpp:28-67) with mask from select_lefs_to_bind (:79-89)
  void bind_lefs(bp_t start, bp_t end, std::vector<Lef>& lefs, usize n, std::vector<usize>& rr,
                 std::vector<usize>& fr, const u64* mask, Rng& g, usize epoch) const {
    for (usize i = 0; i < n; ++i) {
      if (!mask || mask[i]) lefs[i].bind(epoch, uniform_int(g, start, end - 1));
    }
    rank_lefs(lefs, n, rr, fr, epoch != 0, false);
    if (g_count_ties.load(std::memory_order_relaxed)) count_full_ties(lefs, n, rr, fr, start, end);
  }

  // rank_lefs (simulation.cpp:402-487)
  static void rank_lefs(const std::vector<Lef>& lefs, usize n, std::vector<usize>& rr,
                        std::vector<usize>& fr, bool partially_sorted, bool init) {
    auto rev_cmp = [&](usize a, usize b) { return lefs[a].rev < lefs[b].rev; };
    auto fwd_cmp = [&](usize a, usize b) { return lefs[a].fwd < lefs[b].fwd; };
    if (init) {
      std::iota(fr.begin(), fr.begin() + n, 0);
      std::iota(rr.begin(), rr.begin() + n, 0);
    }
    if (partially_sorted) {
      sorting::split_sort(rr.begin(), rr.begin() + n, rev_cmp);
      sorting::split_sort(fr.begin(), fr.begin() + n, fwd_cmp);
    } else {
      sorting::pdq_sort(rr.begin(), rr.begin() + n, rev_cmp);
      sorting::pdq_sort(fr.begin(), fr.begin() + n, fwd_cmp);
    }
    usize begin = 0, end = 0;
    for (usize i = 1; i < n; ++i) {
      if (lefs[rr[i - 1]].rev == lefs[rr[i]].rev) {
        begin = i - 1;
        for (; i < n; ++i) {
          if (lefs[rr[i - 1]].rev != lefs[rr[i]].rev) break;
        }
        end = i;
        sorting::insertion_sort(rr.begin() + begin, rr.begin() + end, [&](usize a, usize b) {
          return lefs[a].binding_epoch < lefs[b].binding_epoch;
        });
      }
    }
    for (usize i = 1; i < n; ++i) {
      if (lefs[fr[i - 1]].fwd == lefs[fr[i]].fwd) {
        begin = i - 1;
        for (; i < n; ++i) {
          if (lefs[fr[i - 1]].fwd != lefs[fr[i]].fwd) break;
        }
        end = i;
        sorting::insertion_sort(fr.begin() + begin, fr.begin() + end, [&](usize a, usize b) {
          return lefs[b].binding_epoch < lefs[a].binding_epoch;
        });
      }
    }
  }

  // Full ties: neighbours in a rank order that are bound and share both the position and the
  // binding epoch.  Their relative order is whatever the sort's element moves leave, the one
  // part of the ranking the reference's tests do not pin (cpp-sort's unstable sorts).  Ties of
  // units parked at a chromosome end (rev at start, fwd at end - 1) are counted apart from
  // interior ones.
  static void count_full_ties(const std::vector<Lef>& lefs, usize n, const std::vector<usize>& rr,
                              const std::vector<usize>& fr, bp_t start, bp_t end) {
    u64 pairs = 0, interior = 0;
    for (usize i = 1; i < n; ++i) {
      const Lef& a = lefs[rr[i - 1]];
      const Lef& b = lefs[rr[i]];
      if (a.bound() && b.bound() && a.rev == b.rev && a.binding_epoch == b.binding_epoch) {
        ++pairs;
        interior += a.rev != start;
      }
      const Lef& c = lefs[fr[i - 1]];
      const Lef& d = lefs[fr[i]];
      if (c.bound() && d.bound() && c.fwd == d.fwd && c.binding_epoch == d.binding_epoch) {
        ++pairs;
        interior += c.fwd != end - 1;
      }
    }
    g_tie_rank_calls.fetch_add(1, std::memory_order_relaxed);
    if (pairs) {
      g_tie_calls.fetch_add(1, std::memory_order_relaxed);
      g_tie_pairs.fetch_add(pairs, std::memory_order_relaxed);
      g_tie_interior.fetch_add(interior, std::memory_order_relaxed);
    }
  }

  // generate_moves_helper + generate_moves (simulation.cpp:264-323)
  void generate_moves(const Chrom& ch, const std::vector<Lef>& lefs, usize n,
                      const std::vector<usize>& rr, const std::vector<usize>& fr,
                      std::vector<bp_t>& rm, std::vector<bp_t>& fm, bool burnin_completed, Rng& g,
                      bool adjust = true) const {
    const double rev_speed = static_cast<double>(burnin_completed ? c.rev_extrusion_speed
                                                                  : c.rev_extrusion_speed_burnin);
    const double fwd_speed = static_cast<double>(burnin_completed ? c.fwd_extrusion_speed
                                                                  : c.fwd_extrusion_speed_burnin);
    auto helper = [&](std::vector<bp_t>& moves, double avg, double sd) {
      const bp_t move_int = static_cast<bp_t>(std::round(avg));
      for (usize i = 0; i < n; ++i) {
        if (!lefs[i].bound()) {
          moves[i] = 0;
        } else if (sd == 0.0) {
          moves[i] = move_int;
        } else {
          moves[i] = static_cast<bp_t>(std::round(std::max(0.0, normal(g, avg, sd))));
        }
      }
    };
    helper(rm, rev_speed, c.rev_extrusion_speed_std);
    helper(fm, fwd_speed, c.fwd_extrusion_speed_std);
    if (adjust) adjust_moves(ch, lefs, n, rr, fr, rm, fm);
    clamp_moves(ch, lefs, n, rm, fm);
  }

  // clamp_moves (simulation.cpp:325-340)
  static void clamp_moves(const Chrom& ch, const std::vector<Lef>& lefs, usize n,
                          std::vector<bp_t>& rm, std::vector<bp_t>& fm) {
    for (usize i = 0; i < n; ++i) {
      if (!lefs[i].bound()) continue;
      rm[i] = std::min(rm[i], lefs[i].rev - ch.start);
      fm[i] = std::min(fm[i], ch.end - lefs[i].fwd - 1);
    }
  }

  // adjust_moves_of_consecutive_extr_units (simulation.cpp:343-399)
  static void adjust_moves(const Chrom& ch, const std::vector<Lef>& lefs, usize n,
                           const std::vector<usize>& rr, const std::vector<usize>& fr,
                           std::vector<bp_t>& rm, std::vector<bp_t>& fm) {
    for (usize i = n - 1; i > 0; --i) {
      const usize i1 = rr[i - 1];
      const usize i2 = rr[i];
      if (lefs[i1].bound() && lefs[i2].bound()) {
        if (lefs[i1].rev <= ch.start + rm[i1] || lefs[i2].rev <= ch.start + rm[i2]) continue;
        const bp_t pos1 = lefs[i1].rev - rm[i1];
        const bp_t pos2 = lefs[i2].rev - rm[i2];
        if (pos2 <= pos1) rm[i1] += (pos1 - pos2) + 1;
      }
    }
    for (usize i = 1; i < n; ++i) {
      const usize i1 = fr[i - 1];
      const usize i2 = fr[i];
      if (lefs[i1].bound() && lefs[i2].bound()) {
        if (lefs[i1].fwd + fm[i1] > ch.end - 1 || lefs[i2].fwd + fm[i2] > ch.end - 1) continue;
        const bp_t pos1 = lefs[i1].fwd + fm[i1];
        const bp_t pos2 = lefs[i2].fwd + fm[i2];
        if (pos1 >= pos2) fm[i2] += (pos1 - pos2) + 1;
      }
    }
  }

  // extrude (simulation.cpp:489-512)
  static void extrude(std::vector<Lef>& lefs, usize n, const std::vector<bp_t>& rm,
                      const std::vector<bp_t>& fm) {
    for (usize i = 0; i < n; ++i) {
      if (!lefs[i].bound()) continue;
      lefs[i].rev -= rm[i];
      lefs[i].fwd += fm[i];
    }
  }

  // compute_lef_lef_collision_pos (simulation.cpp:514-542)
  static std::pair<bp_t, bp_t> lef_lef_collision_pos(bp_t rev_pos, bp_t fwd_pos, bp_t rev_move,
                                                      bp_t fwd_move) {
    const bp_t relative_speed = rev_move + fwd_move;
    const double time_to_collision =
        static_cast<double>(rev_pos - fwd_pos) / static_cast<double>(relative_speed);
    const bp_t collision_pos =
        fwd_pos + static_cast<bp_t>(std::round(static_cast<double>(fwd_move) * time_to_collision));
    if (collision_pos == fwd_pos) return {collision_pos + 1, collision_pos};
    return {collision_pos, collision_pos - 1};
  }

  // release_lefs (simulation.cpp:544-592)
  usize release_lefs(std::vector<Lef>& lefs, usize n, const Barriers& b,
                     const std::vector<Coll>& rc, const std::vector<Coll>& fc, Rng& g,
                     bool burnin_completed) const {
    const double base = burnin_completed ? c.prob_of_lef_release : c.prob_of_lef_release_burnin;
    auto hard = [&](const Coll& col, u32 d) {
      if (col.occurred(LEF_BAR)) return b.dir[col.idx()] == d;
      return false;
    };
    usize released = 0;
    for (usize i = 0; i < n; ++i) {
      if (!lefs[i].bound()) continue;
      const unsigned nh = unsigned(hard(rc[i], MGPU_DIR_REV)) + unsigned(hard(fc[i], MGPU_DIR_FWD));
      const double aff = nh == 0 ? 1.0
                         : nh == 1 ? 1.0 / c.soft_stall_lef_stability_multiplier
                                   : 1.0 / c.hard_stall_lef_stability_multiplier;
      const double p = aff * base;
      if (bernoulli(g, p)) {
        ++released;
        lefs[i].release();
      }
    }
    return released;
  }

  // run_lef_lef_collision_trial / run_lef_bar_collision_trial (simulation_impl.hpp:123-131)
  bool lef_lef_trial(Rng& g) const {
    return c.probability_of_extrusion_unit_bypass == 0.0 ||
           bernoulli(g, 1.0 - c.probability_of_extrusion_unit_bypass);
  }
  static bool lef_bar_trial(double pblock, Rng& g) { return pblock == 1.0 || bernoulli(g, pblock); }

  // detect_units_at_chrom_boundaries (simulation_detect_collisions.cpp:30-125)
  static std::pair<usize, usize> detect_boundaries(const Chrom& ch, const std::vector<Lef>& lefs,
                                                    usize n, const std::vector<usize>& rr,
                                                    const std::vector<usize>& fr,
                                                    const std::vector<bp_t>& rm,
                                                    const std::vector<bp_t>& fm,
                                                    std::vector<Coll>& rc, std::vector<Coll>& fc,
                                                    bool* ub) {
    usize n5 = 0, n3 = 0;
    const bp_t first_fwd_pos = lefs[fr[0]].fwd;
    usize last_rev = U64MAX;
    for (usize k = n; k > 0; --k) {
      if (lefs[rr[k - 1]].bound()) {
        last_rev = rr[k - 1];
        break;
      }
    }
    if (last_rev == U64MAX) {  // no bound LEF: the reference dereferences rend() here
      if (ub) *ub = true;
      last_rev = rr[0];
    }
    const bp_t last_rev_pos = lefs[last_rev].rev;
    for (usize i = 0; i < n; ++i) {
      const usize idx = rr[i];
      const bp_t pos = lefs[idx].rev;
      const bp_t mv = rm[idx];
      if (pos == ch.start) {
        ++n5;
        rc[idx].set(5, COLLISION | CHROM_BOUNDARY);
      } else if (pos > first_fwd_pos) {
        break;
      } else if (pos - mv == ch.start) {
        rc[idx].set(5, COLLISION | CHROM_BOUNDARY);
        ++n5;
        break;
      }
    }
    for (usize i = n - 1; i > 0; --i) {
      const usize idx = fr[i];
      const bp_t pos = lefs[idx].fwd;
      const bp_t mv = fm[idx];
      if (!lefs[idx].bound()) {
        ++n3;
        continue;
      }
      if (pos == ch.end - 1) {
        ++n3;
        fc[idx].set(3, COLLISION | CHROM_BOUNDARY);
      } else if (pos < last_rev_pos) {
        break;
      } else if (pos + mv == ch.end - 1) {
        fc[idx].set(3, COLLISION | CHROM_BOUNDARY);
        ++n3;
        break;
      }
    }
    return {n5, n3};
  }

  // detect_lef_bar_collisions (simulation_detect_collisions.cpp:128-252)
  void detect_lef_bar(const std::vector<Lef>& lefs, usize n, const std::vector<usize>& rr,
                      const std::vector<usize>& fr, const std::vector<bp_t>& rm,
                      const std::vector<bp_t>& fm, const Barriers& b, std::vector<Coll>& rc,
                      std::vector<Coll>& fc, Rng& g, usize n5, usize n3) const {
    usize j = std::min(n5, n5 - 1);
    usize unit_idx = rr[j];
    bp_t unit_pos = lefs[unit_idx].rev;
    bool rev_done = false;
    for (usize i = 0; i < b.size() && !rev_done; ++i) {
      if (b.is_not_active(i)) continue;
      const double pblock = b.dir[i] == MGPU_DIR_REV ? c.lef_bar_major_collision_pblock
                                                     : c.lef_bar_minor_collision_pblock;
      while (unit_pos <= b.pos[i]) {
        if (++j == n) {
          rev_done = true;
          break;
        }
        unit_idx = rr[j];
        unit_pos = lefs[unit_idx].rev;
      }
      if (rev_done) break;
      if (lefs[unit_idx].bound()) {
        const bp_t delta = unit_pos - b.pos[i];
        if (delta > 0 && delta <= rm[unit_idx] && lef_bar_trial(pblock, g)) {
          rc[unit_idx].set(i, COLLISION | LEF_BAR);
        }
      }
    }
    j = n - std::min(n3, n3 - 1);
    unit_idx = fr[--j];
    unit_pos = lefs[unit_idx].fwd;
    for (usize i = b.size() - 1; i != U64MAX; --i) {
      if (b.is_not_active(i)) continue;
      const double pblock = b.dir[i] == MGPU_DIR_FWD ? c.lef_bar_major_collision_pblock
                                                     : c.lef_bar_minor_collision_pblock;
      while (unit_pos >= b.pos[i]) {
        if (--j == U64MAX) return;
        unit_idx = fr[j];
        unit_pos = lefs[unit_idx].fwd;
      }
      if (lefs[unit_idx].bound()) {
        const bp_t delta = b.pos[i] - unit_pos;
        if (delta > 0 && delta <= fm[unit_idx] && lef_bar_trial(pblock, g)) {
          fc[unit_idx].set(i, COLLISION | LEF_BAR);
        }
      }
    }
  }

  // detect_primary_lef_lef_collisions (simulation_detect_collisions.cpp:255-401)
  void detect_primary(const std::vector<Lef>& lefs, usize n, const Barriers& b,
                      const std::vector<usize>& rr, const std::vector<usize>& fr,
                      const std::vector<bp_t>& rm, const std::vector<bp_t>& fm,
                      std::vector<Coll>& rc, std::vector<Coll>& fc, Rng& g, usize n5, usize n3,
                      bool* ub) const {
    if (n5 == n || n3 == n) return;
    usize i1 = 0;
    usize j1 = n5;
    const usize i2 = n - std::min(n3, n3 - 1);
    const usize j2 = n;
    auto barrier_pos = [&](usize idx) -> bp_t {
      if (idx >= b.size()) {  // the reference reads past the barrier vector here
        if (ub) *ub = true;
        return 0;
      }
      return b.pos[idx];
    };
    for (;;) {
      usize rev_idx = rr[j1];
      bp_t rev_pos = lefs[rev_idx].rev;
      usize fwd_idx = fr[i1];
      bp_t fwd_pos = lefs[fwd_idx].fwd;
      while (rev_pos <= fwd_pos) {
        if (++j1 == j2) return;
        rev_idx = rr[j1];
        rev_pos = lefs[rev_idx].rev;
      }
      while (fwd_pos < rev_pos) {
        if (++i1 == i2) return;
        fwd_idx = fr[i1];
        fwd_pos = lefs[fwd_idx].fwd;
      }
      fwd_idx = fr[std::min(i1, i1 - 1)];
      fwd_pos = lefs[fwd_idx].fwd;
      const bp_t delta = rev_pos - fwd_pos;
      if (delta > 0 && delta < rm[rev_idx] + fm[fwd_idx] && lef_lef_trial(g)) {
        const bp_t rev_move = rm[rev_idx];
        const bp_t fwd_move = fm[fwd_idx];
        Coll& rcol = rc[rev_idx];
        Coll& fcol = fc[fwd_idx];
        const auto [cpos_rev, cpos_fwd] =
            lef_lef_collision_pos(lefs[rev_idx].rev, lefs[fwd_idx].fwd, rev_move, fwd_move);
        if (!rcol.occurred() && !fcol.occurred()) {
          rcol.set(fwd_idx, COLLISION | LEF_LEF_PRIMARY);
          fcol.set(rev_idx, COLLISION | LEF_LEF_PRIMARY);
        } else if (rcol.occurred() && !fcol.occurred()) {
          const bp_t bpos = barrier_pos(rcol.idx());
          if (cpos_fwd > bpos) {
            rcol.set(fwd_idx, COLLISION | LEF_LEF_PRIMARY);
            fcol.set(rev_idx, COLLISION | LEF_LEF_PRIMARY);
          } else {
            fcol.set(rev_idx, COLLISION | LEF_LEF_PRIMARY);
          }
        } else if (!rcol.occurred() && fcol.occurred()) {
          const bp_t bpos = barrier_pos(fcol.idx());
          rcol.set(fwd_idx, COLLISION | LEF_LEF_PRIMARY);
          if (cpos_rev < bpos) fcol.set(rev_idx, COLLISION | LEF_LEF_PRIMARY);
        }
      }
    }
  }

  // correct_moves_for_lef_bar_collisions (simulation_correct_moves.cpp:20-51)
  static void correct_lef_bar(const std::vector<Lef>& lefs, usize n, const Barriers& b,
                              std::vector<bp_t>& rm, std::vector<bp_t>& fm,
                              const std::vector<Coll>& rc, const std::vector<Coll>& fc) {
    for (usize i = 0; i < n; ++i) {
      if (rc[i].occurred(LEF_BAR)) rm[i] = lefs[i].rev - b.pos[rc[i].idx()] - 1;
      if (fc[i].occurred(LEF_BAR)) fm[i] = b.pos[fc[i].idx()] - lefs[i].fwd - 1;
    }
  }

  // correct_moves_for_primary_lef_lef_collisions (simulation_correct_moves.cpp:54-122)
  static void correct_primary(const std::vector<Lef>& lefs, usize n, const std::vector<usize>& rr,
                              const std::vector<usize>& fr, std::vector<bp_t>& rm,
                              std::vector<bp_t>& fm, const std::vector<Coll>& rc,
                              const std::vector<Coll>& fc) {
    for (usize k = 0; k < n; ++k) {
      const usize rev_idx = rr[k];
      if (!rc[rev_idx].occurred(LEF_LEF_PRIMARY)) continue;
      const usize fwd_idx = rc[rev_idx].idx();
      if (fc[fwd_idx].occurred(LEF_LEF_PRIMARY)) {
        const bp_t rp = lefs[rev_idx].rev;
        const bp_t fp = lefs[fwd_idx].fwd;
        const auto [p1, p2] = lef_lef_collision_pos(rp, fp, rm[rev_idx], fm[fwd_idx]);
        rm[rev_idx] = rp - p1;
        fm[fwd_idx] = p2 - fp;
      } else if (fc[fwd_idx].occurred(LEF_BAR)) {
        rm[rev_idx] = lefs[rev_idx].rev - (lefs[fwd_idx].fwd + fm[fwd_idx]) - 1;
      }
    }
    for (usize k = 0; k < n; ++k) {
      const usize fwd_idx = fr[k];
      if (!fc[fwd_idx].occurred(LEF_LEF_PRIMARY)) continue;
      const usize rev_idx = fc[fwd_idx].idx();
      if (rc[rev_idx].occurred(LEF_BAR)) {
        fm[fwd_idx] = (lefs[rev_idx].rev - rm[rev_idx]) - lefs[fwd_idx].fwd - 1;
      }
    }
  }

  // process_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:404-518)
  void process_secondary(const std::vector<Lef>& lefs, usize n, const std::vector<usize>& rr,
                         const std::vector<usize>& fr, std::vector<bp_t>& rm,
                         std::vector<bp_t>& fm, std::vector<Coll>& rc, std::vector<Coll>& fc,
                         Rng& g, usize n5, usize n3) const {
    for (usize i = std::max(usize(1), n5); i < n; ++i) {
      const usize idx1 = rr[i - 1];
      const bp_t pos1 = lefs[idx1].rev;
      if (!rc[idx1].occurred()) continue;
      const usize idx2 = rr[i];
      const bp_t pos2 = lefs[idx2].rev;
      if (rc[idx2].occurred()) continue;
      bp_t& move1 = rm[idx1];
      bp_t& move2 = rm[idx2];
      if (pos2 - move2 <= pos1 - move1) {
        if (lef_lef_trial(g)) {
          rc[idx2].set(idx1, COLLISION | LEF_LEF_SECONDARY);
          const bp_t mv = pos2 - (pos1 - move1);
          move2 = std::min(mv, mv - 1);
        } else {
          rc[idx2].set(idx1, LEF_LEF_SECONDARY);
        }
      }
    }
    usize i = n - std::min(n3, n3 - 1) - 1;
    for (; i > 0; --i) {
      const usize idx2 = fr[i];
      const bp_t pos2 = lefs[idx2].fwd;
      if (!fc[idx2].occurred()) continue;
      const usize idx1 = fr[i - 1];
      const bp_t pos1 = lefs[idx1].fwd;
      if (fc[idx1].occurred()) continue;
      bp_t& move1 = fm[idx1];
      bp_t& move2 = fm[idx2];
      if (pos1 + move1 >= pos2 + move2) {
        if (lef_lef_trial(g)) {
          fc[idx1].set(idx2, COLLISION | LEF_LEF_SECONDARY);
          const bp_t mv = (pos2 + move2) - pos1;
          move1 = std::min(mv, mv - 1);
        } else {
          fc[idx1].set(idx2, LEF_LEF_SECONDARY);
        }
      }
    }
  }

  // fix_secondary_lef_lef_collisions (simulation_detect_collisions.cpp:520-647)
  static void fix_secondary(const Chrom& ch, std::vector<Lef>& lefs, usize n,
                            std::vector<usize>& rr, std::vector<usize>& fr, std::vector<bp_t>& rm,
                            std::vector<bp_t>& fm, std::vector<Coll>& rc, std::vector<Coll>& fc,
                            usize n5, usize n3) {
    const usize num_active_fwd = n - std::min(n3, n3 - 1);
    for (usize i = std::max(usize(1), n5); i < n; ++i) {
      const usize idx2 = rr[i];
      if (!rc[idx2].avoided(LEF_LEF_SECONDARY)) continue;
      const usize idx1 = rr[i - 1];
      Lef& lef1 = lefs[idx1];
      Lef& lef2 = lefs[idx2];
      const bp_t pos1 = lef1.rev - rm[idx1];
      if (lef2.rev > pos1 + 1) {
        rm[idx2] = lef2.rev - (pos1 + 1);
      } else {
        rm[idx2] = 0;
      }
      rc[idx2].set(idx1, COLLISION | LEF_LEF_SECONDARY);
      const bp_t p1 = lef1.rev;
      const bp_t p2 = lef2.rev;
      lef1.rev = std::min(lef1.fwd, p2);
      lef2.rev = std::min(lef2.fwd, p1);
      std::swap(rc[idx1], rc[idx2]);
      std::swap(rm[idx1], rm[idx2]);
      std::swap(rr[i - 1], rr[i]);
      rm[rr[i - 1]] = std::min(lefs[rr[i - 1]].rev - ch.start, rm[rr[i - 1]]);
      rm[rr[i]] = std::min(lefs[rr[i]].rev - ch.start, rm[rr[i]]);
    }
    for (usize i = 0; i < num_active_fwd - 1; ++i) {
      const usize idx1 = fr[i];
      if (!fc[idx1].avoided(LEF_LEF_SECONDARY)) continue;
      const usize idx2 = fr[i + 1];
      Lef& lef1 = lefs[idx1];
      Lef& lef2 = lefs[idx2];
      const bp_t pos2 = lef2.fwd + fm[idx2];
      if (pos2 > lef1.fwd + 1) {
        fm[idx1] = pos2 - (lef1.fwd + 1);
      } else {
        fm[idx1] = 0;
      }
      fc[idx1].set(idx2, COLLISION | LEF_LEF_SECONDARY);
      const bp_t p1 = lef1.fwd;
      const bp_t p2 = lef2.fwd;
      lef1.fwd = std::max(lef1.rev, p2);
      lef2.fwd = std::max(lef2.rev, p1);
      std::swap(fc[idx1], fc[idx2]);
      std::swap(fm[idx1], fm[idx2]);
      std::swap(fr[i], fr[i + 1]);
      fm[fr[i]] = std::min(ch.end - 1 - lefs[fr[i]].fwd, fm[fr[i]]);
      fm[fr[i + 1]] = std::min(ch.end - 1 - lefs[fr[i + 1]].fwd, fm[fr[i + 1]]);
    }
  }

  // process_collisions (simulation.cpp:925-955)
  std::pair<usize, usize> process_collisions(const Chrom& ch, std::vector<Lef>& lefs, usize n,
                                             const Barriers& b, std::vector<usize>& rr,
                                             std::vector<usize>& fr, std::vector<bp_t>& rm,
                                             std::vector<bp_t>& fm, std::vector<Coll>& rc,
                                             std::vector<Coll>& fc, Rng& g, bool fix,
                                             bool* ub) const {
    const auto [n5, n3] = detect_boundaries(ch, lefs, n, rr, fr, rm, fm, rc, fc, ub);
    detect_lef_bar(lefs, n, rr, fr, rm, fm, b, rc, fc, g, n5, n3);
    detect_primary(lefs, n, b, rr, fr, rm, fm, rc, fc, g, n5, n3, ub);
    correct_lef_bar(lefs, n, b, rm, fm, rc, fc);
    correct_primary(lefs, n, rr, fr, rm, fm, rc, fc);
    process_secondary(lefs, n, rr, fr, rm, fm, rc, fc, g, n5, n3);
    if (fix) fix_secondary(ch, lefs, n, rr, fr, rm, fm, rc, fc, n5, n3);
    return {n5, n3};
  }

  // Simulation::compute_contacts_per_epoch (simulation.cpp:1243-1251)
  usize contacts_per_epoch(usize nlefs) const {
    const double speed = static_cast<double>(c.rev_extrusion_speed + c.fwd_extrusion_speed);
    const double p = speed / static_cast<double>(c.contact_sampling_interval);
    return static_cast<usize>(std::max(1.0, std::round(static_cast<double>(nlefs) * p)));
  }
};

// compute_num_contacts_loop (register_contacts.cpp:73-92)
static usize num_contacts_loop(usize num, double ratio, Rng& g) {
  if (ratio == 0) return num;
  if (!std::isfinite(ratio)) return 0;
  const double p = 1.0 / (ratio + 1.0);
  return static_cast<usize>(binomial(g, static_cast<i64>(num), p));
}

// ---------------------------------------------------------------------------------------
// One cell: Simulation::simulate_one_cell (simulation.cpp:1056-1152)
// ---------------------------------------------------------------------------------------
static inline u64 mix64(u64 z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}

// The trace digest of one epoch; the same formula is documented in mgpu_state_digest.
static u64 digest_entry(u64 i, const u64 v[9]) {
  u64 h = mix64(i * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL);
  for (int k = 0; k < 9; ++k) h = mix64(h ^ v[k]);
  return h;
}

struct CellResult {
  u64 epochs = 0, burnin_epochs = 0, contacts = 0, missed = 0, lef_epochs = 0, draws = 0;
  int status = MGPU_OK;
};

class Cell {
 public:
  Cell(const mgpu_config& cfg, const Chrom& ch, const Barriers& barriers, usize nlefs)
      : sim(cfg), c(cfg), ch(ch), b(barriers), nlefs(nlefs) {
    lefs.assign(nlefs, Lef{});
    rr.resize(nlefs);
    fr.resize(nlefs);
    std::iota(rr.begin(), rr.end(), 0);
    std::copy(rr.begin(), rr.end(), fr.begin());
    rm.assign(nlefs, 0);
    fm.assign(nlefs, 0);
    idx.assign(nlefs, 0);
    rc.assign(nlefs, Coll{});
    fc.assign(nlefs, Coll{});
  }

  // compute_loop_size_stats (simulation.cpp:957-981) with stats::mean / standard_dev
  // (src/stats/descriptive_impl.hpp): left-to-right double accumulation.
  void loop_size_stats(usize n) {
    if (n == 0) {
      cfx.clear();
      avg.clear();
      return;
    }
    double acc = 0.0;
    for (usize i = 0; i < n; ++i) acc = acc + double(lefs[i].loop_size());
    const double mean = acc / static_cast<double>(n);
    double ssd = 0.0;
    for (usize i = 0; i < n; ++i) {
      const double d = double(lefs[i].loop_size()) - mean;
      ssd = ssd + (d * d);
    }
    const double sd = std::sqrt(ssd / static_cast<double>(n));
    if (avg.size() == c.burnin_history_length) {
      avg.pop_front();
      cfx.pop_front();
    }
    avg.push_back(mean);
    cfx.push_back(sd / avg.back());
  }

  // evaluate_burnin (simulation.cpp:983-1025)
  static bool evaluate_burnin(const std::deque<double>& cfx, const std::deque<double>& avg,
                              usize cap, usize w) {
    if (cfx.size() != cap) return false;
    auto window_mean = [](const std::deque<double>& d, usize from, usize to) {
      double acc = 0.0;
      for (usize k = from; k < to; ++k) acc = acc + d[k];
      return acc / static_cast<double>(to - from);
    };
    auto ratio = [&](const std::deque<double>& d) {
      usize nd = 0;
      for (usize i1 = 1, i2 = w + 1; i2 != d.size(); ++i1, ++i2) {
        const double n1 = window_mean(d, i1 - 1, i2 - 1);
        const double n2 = window_mean(d, i1, i2);
        nd += static_cast<usize>(n1 > n2);
      }
      return static_cast<double>(nd) / static_cast<double>(cap - w - nd);
    };
    const double r1 = ratio(cfx);
    if (!(r1 >= 0.95 && r1 <= 1.05)) return false;
    const double r2 = ratio(avg);
    return r2 >= 0.95 && r2 <= 1.05;
  }

  // run_burnin (simulation.cpp:1027-1054)
  void run_burnin(double rate) {
    do {
      ++num_burnin_epochs;
      if (num_active != nlefs) {
        const usize k = poisson(g, rate);
        num_active = std::min(num_active + k, nlefs);
      } else {
        loop_size_stats(num_active);
        burnin_completed = evaluate_burnin(cfx, avg, c.burnin_history_length,
                                           c.burnin_smoothing_window_size);
        burnin_completed = burnin_completed && (epoch > c.min_burnin_epochs);
        if (!burnin_completed && epoch >= c.max_burnin_epochs) burnin_completed = true;
      }
    } while (num_active == 0);
  }

  // sample_and_register_contacts (register_contacts.cpp:94-198)
  void sample_contacts(usize num_events, Band& band, u64 target) {
    if (c.target_contact_density > 0.0) num_events = std::min(num_events, target - num_contacts);
    if (num_events == 0) return;
    const bp_t start = ch.ws + 1;
    const bp_t end = ch.we - 1;
    const usize n_loop = num_contacts_loop(num_events, c.tad_to_loop_contact_ratio, g);
    const usize n_tad = num_events - n_loop;
    const bool noisify = (c.contact_sampling_strategy & MGPU_CS_NOISIFY) != 0;
    auto within = [&](const Lef& l) {
      return l.rev > start && l.rev < end && l.fwd > start && l.fwd < end;
    };
    auto noise_pair = [&](const Lef& l) {
      const double n1 = noisify ? gev(g, c.genextreme_mu, c.genextreme_sigma, c.genextreme_xi) : 0.0;
      const double a = static_cast<double>(l.rev) - n1;
      const double n2 = noisify ? gev(g, c.genextreme_mu, c.genextreme_sigma, c.genextreme_xi) : 0.0;
      const double bb = static_cast<double>(l.fwd) + n2;
      return std::pair<double, double>{std::min(a, bb), std::max(a, bb)};
    };
    auto pos_ok = [&](double p1, double p2) {
      const double s = static_cast<double>(start), e = static_cast<double>(end);
      return p1 >= s && p2 >= s && p1 < e && p2 < e;
    };
    usize todo = n_loop;
    while (todo != 0) {
      const Lef& l = lefs[uniform_int(g, 0, num_active - 1)];
      if (l.bound() && within(l)) {
        const auto [p1, p2] = noise_pair(l);
        if (!pos_ok(p1, p2)) continue;
        const bp_t q1 = static_cast<bp_t>(p1) - start;
        const bp_t q2 = static_cast<bp_t>(p2) - start;
        band.increment(q1 / c.bin_size, q2 / c.bin_size);
        --todo;
      }
    }
    todo = n_tad;
    while (todo != 0) {
      const Lef& l = lefs[uniform_int(g, 0, num_active - 1)];
      if (l.bound() && within(l)) {
        const auto [p1, p2] = noise_pair(l);
        if (!pos_ok(p1, p2)) continue;
        const bp_t a = static_cast<bp_t>(p1), bb = static_cast<bp_t>(p2);
        const bp_t p11 = uniform_int(g, a, bb);
        const bp_t p22 = uniform_int(g, a, bb);
        band.increment((p11 - start) / c.bin_size, (p22 - start) / c.bin_size);
        --todo;
      }
    }
    // register_1d_lef_occupancy (register_contacts.cpp:200-232): the loop attempt again, with
    // one count in each of the two bins of Chromosome::lef_1d_occupancy as its sink
    if (c.track_1d_lef_position) {
      todo = num_events;
      while (todo != 0) {
        const Lef& l = lefs[uniform_int(g, 0, num_active - 1)];
        if (l.bound() && within(l)) {
          const auto [p1, p2] = noise_pair(l);
          if (!pos_ok(p1, p2)) continue;
          const bp_t i1 = (static_cast<bp_t>(p1) - start) / c.bin_size;
          const bp_t i2 = (static_cast<bp_t>(p2) - start) / c.bin_size;
          if (occ) {
            occ[i1]++;
            occ[i2]++;
          }
          --todo;
        }
      }
    }
    num_contacts += num_events;
  }

  // Simulation::dump_stats (simulation.cpp:1166-1224) as a record
  void dump_stats() {
    if (!recs || nrec >= rec_max) return;
    mgpu_epoch_record r{};
    r.epoch = epoch;
    r.cell = cell_index;
    r.burnin = burnin_completed ? 0 : 1;
    for (usize i = 0; i < b.size(); ++i) r.barriers_occupied += b.is_active(i) ? 1 : 0;
    r.nbarriers = b.size();
    r.num_lefs = num_active;
    double acc = 0.0;
    for (usize i = 0; i < num_active; ++i) {
      const bool sr = rc[i].occurred(), sf = fc[i].occurred();
      r.stalled_rev += sr;
      r.stalled_fwd += sf;
      r.stalled_both += sr && sf;
      r.lef_bar += rc[i].occurred(LEF_BAR) + fc[i].occurred(LEF_BAR);
      r.lef_lef_primary += rc[i].occurred(LEF_LEF_PRIMARY) + fc[i].occurred(LEF_LEF_PRIMARY);
      r.lef_lef_secondary += rc[i].occurred(LEF_LEF_SECONDARY) + fc[i].occurred(LEF_LEF_SECONDARY);
      acc = acc + static_cast<double>(lefs[i].fwd - lefs[i].rev);
    }
    r.avg_loop_size = num_active ? acc / static_cast<double>(num_active) : 0.0;
    recs[nrec++] = r;
  }

  void record(mgpu_trace_request* tr, u64 rec_idx, usize n5, usize n3) {
    mgpu_trace_header h{};
    h.epoch = epoch;
    h.num_active_lefs = num_active;
    h.burnin_completed = burnin_completed;
    h.num_burnin_epochs = num_burnin_epochs;
    h.num_contacts = num_contacts;
    h.rng_draws = g.ndraws;
    h.n5prime = n5;
    h.n3prime = n3;
    u64 dig = 0;
    for (usize i = 0; i < nlefs; ++i) {
      const u64 v[9] = {lefs[i].rev, lefs[i].fwd, lefs[i].binding_epoch, rr[i], fr[i],
                        rm[i],       fm[i],       rc[i].w,             fc[i].w};
      dig += digest_entry(i, v);
    }
    h.digest = dig;
    if (tr->all_headers && rec_idx < tr->max_epochs) tr->all_headers[rec_idx] = h;
    if (rec_idx < tr->max_records) {
      if (tr->headers) tr->headers[rec_idx] = h;
      const usize o = rec_idx * nlefs;
      for (usize i = 0; i < nlefs; ++i) {
        if (tr->rev_pos) tr->rev_pos[o + i] = lefs[i].rev;
        if (tr->fwd_pos) tr->fwd_pos[o + i] = lefs[i].fwd;
        if (tr->binding_epoch) tr->binding_epoch[o + i] = lefs[i].binding_epoch;
        if (tr->rev_rank) tr->rev_rank[o + i] = rr[i];
        if (tr->fwd_rank) tr->fwd_rank[o + i] = fr[i];
        if (tr->rev_move) tr->rev_move[o + i] = rm[i];
        if (tr->fwd_move) tr->fwd_move[o + i] = fm[i];
        if (tr->rev_collision) tr->rev_collision[o + i] = rc[i].w;
        if (tr->fwd_collision) tr->fwd_collision[o + i] = fc[i].w;
      }
    }
  }

  // optional outputs: 1D occupancy counters and model-state records
  u64* occ = nullptr;
  mgpu_epoch_record* recs = nullptr;
  u64 rec_max = 0, nrec = 0, cell_index = 0;

  CellResult run(u64 seed, u64 target_contacts, u64 target_epochs, Band& band,
                 mgpu_trace_request* tr) {
    CellResult res;
    g = make_prng(seed);
    const double rate = static_cast<double>(nlefs) /
                        static_cast<double>(c.burnin_target_epochs_for_lef_activation);
    const usize spe = sim.contacts_per_epoch(nlefs);
    num_contacts = 0;
    b.init_states(g);
    if (c.skip_burnin) {
      num_active = nlefs;
      burnin_completed = true;
    }
    const bool contact_mode = c.target_contact_density >= 0;
    auto stop = [&]() {
      if (contact_mode) return num_contacts < target_contacts;
      return epoch - num_burnin_epochs < target_epochs;
    };
    u64 rec = 0;
    bool ub = false;
    for (; stop(); ++epoch) {
      if (!burnin_completed) run_burnin(rate);
      res.lef_epochs += num_active;
      const usize n = num_active;
      for (usize i = 0; i < n; ++i) idx[i] = lefs[i].bound() ? 0 : 1;
      sim.bind_lefs(ch.ws, ch.we, lefs, n, rr, fr, idx.data(), g, epoch);
      if (burnin_completed) {
        sample_contacts(spe, band, target_contacts);
        if (target_contacts != 0 && num_contacts >= target_contacts) break;
      }
      sim.generate_moves(ch, lefs, n, rr, fr, rm, fm, burnin_completed, g);
      b.next_state(g);
      for (usize i = 0; i < n; ++i) {
        rc[i].clear();
        fc[i].clear();
      }
      const auto [n5, n3] =
          sim.process_collisions(ch, lefs, n, b, rr, fr, rm, fm, rc, fc, g, true, &ub);
      Sim::extrude(lefs, n, rm, fm);
      if (c.log_model_internal_state) dump_stats();
      sim.release_lefs(lefs, n, b, rc, fc, g, burnin_completed);
      if (tr) record(tr, rec, n5, n3);
      ++rec;
    }
    if (tr) tr->num_epochs_recorded = std::min<u64>(rec, tr->max_epochs);
    res.epochs = epoch;
    res.burnin_epochs = num_burnin_epochs;
    res.contacts = num_contacts;
    res.draws = g.ndraws;
    if (ub) res.status = MGPU_ERR_INTERNAL;
    return res;
  }

  Sim sim;
  const mgpu_config& c;
  Chrom ch;
  Barriers b;
  usize nlefs;
  std::vector<Lef> lefs;
  std::vector<usize> rr, fr, idx;
  std::vector<bp_t> rm, fm;
  std::vector<Coll> rc, fc;
  std::deque<double> cfx, avg;
  Rng g{};
  usize epoch = 0, num_burnin_epochs = 0, num_active = 0, num_contacts = 0;
  bool burnin_completed = false;
};

static Barriers make_barriers(const mgpu_barrier* bs, u64 nb) {
  Barriers b;
  for (u64 i = 0; i < nb; ++i) {
    b.pos.push_back(bs[i].pos);
    b.dir.push_back(bs[i].blocking_dir);
    b.stp_active.push_back(bs[i].stp_active);
    b.stp_inactive.push_back(bs[i].stp_inactive);
    b.state.push_back(0);
  }
  b.sort();  // State::operator= builds ExtrusionBarriers{first, last} with sort = true
  return b;
}

}  // namespace orc

// =========================================================================================
// C API used by the Python test-suite (ctypes)
// =========================================================================================
using namespace orc;

static int simulate_cell_on(const mgpu_config* cfg, const Chrom& ch, const mgpu_barrier* bs, uint64_t nb,
                            uint64_t seed, uint64_t target_contacts, uint64_t target_epochs, uint64_t nlefs,
                            uint32_t* band, mgpu_cell_stats* stats, mgpu_trace_request* trace,
                            uint64_t* occupancy, mgpu_epoch_record* records, uint64_t max_records,
                            uint64_t cell_index, uint64_t* records_written);

extern "C" {

// Config defaults (simulation_config.hpp:60-124)
void orc_config_defaults(mgpu_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->target_simulation_epochs = 2000;
  c->target_contact_density = 1.0;
  c->stop_on_epochs = 0;
  c->bin_size = 5000;
  c->diagonal_width = 3000000;
  c->contact_sampling_strategy = MGPU_CS_TAD | MGPU_CS_LOOP | MGPU_CS_NOISIFY;
  c->tad_to_loop_contact_ratio = 5.0;
  c->genextreme_mu = 0;
  c->genextreme_sigma = 5000;
  c->genextreme_xi = 0.001;
  c->fwd_extrusion_speed = c->bin_size * 8 / 10;
  c->rev_extrusion_speed = c->fwd_extrusion_speed;
  c->fwd_extrusion_speed_std = 0.05;
  c->rev_extrusion_speed_std = c->fwd_extrusion_speed_std;
  c->number_of_lefs_per_mbp = 20;
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
  c->skip_burnin = 0;
  c->burnin_history_length = 100;
  c->burnin_smoothing_window_size = 5;
  c->min_burnin_epochs = 0;
  c->max_burnin_epochs = U64MAX;
  c->burnin_target_epochs_for_lef_activation = 320;
  c->burnin_speed_coefficient = 1.0;
  c->fwd_extrusion_speed_burnin =
      static_cast<u64>(double(c->fwd_extrusion_speed) * c->burnin_speed_coefficient);
  c->rev_extrusion_speed_burnin = c->fwd_extrusion_speed_burnin;
}

// Cli::transform_args (src/modle/cli.cpp:1086-1215)
int orc_config_transform(mgpu_config* c) {
  // cli_update_extr_speed (:1086-1110)
  if (!c->rev_speed_set) c->rev_extrusion_speed = c->bin_size * 8 / 10;
  if (!c->fwd_speed_set) c->fwd_extrusion_speed = c->bin_size * 8 / 10;
  if (c->fwd_extrusion_speed_std > 0 && c->fwd_extrusion_speed_std < 1)
    c->fwd_extrusion_speed_std *= static_cast<double>(c->fwd_extrusion_speed);
  if (c->rev_extrusion_speed_std > 0 && c->rev_extrusion_speed_std < 1)
    c->rev_extrusion_speed_std *= static_cast<double>(c->rev_extrusion_speed);
  c->rev_extrusion_speed_burnin = static_cast<u64>(
      std::round(c->burnin_speed_coefficient * static_cast<double>(c->rev_extrusion_speed)));
  c->fwd_extrusion_speed_burnin = static_cast<u64>(
      std::round(c->burnin_speed_coefficient * static_cast<double>(c->fwd_extrusion_speed)));
  // cli_compute_prob_of_lef_release (:1113-1119)
  c->prob_of_lef_release = static_cast<double>(c->rev_extrusion_speed + c->fwd_extrusion_speed) /
                           static_cast<double>(c->avg_lef_processivity);
  c->prob_of_lef_release_burnin =
      static_cast<double>(c->rev_extrusion_speed_burnin + c->fwd_extrusion_speed_burnin) /
      static_cast<double>(c->avg_lef_processivity);
  // cli_update_barrier_stp_and_occupancy (:1122-1135)
  auto stp_from_occ = [](double stp_inactive, double occ) {
    if (occ == 0) return 0.0;
    const double ia = 1.0 - stp_inactive;
    const double ai = (ia - (occ * ia)) / occ;
    return std::clamp(1.0 - ai, 0.0, 1.0);
  };
  if (c->occupancy_set) {
    c->barrier_occupied_stp = stp_from_occ(c->barrier_not_occupied_stp, c->extrusion_barrier_occupancy);
  } else {
    c->extrusion_barrier_occupancy =
        Barriers::occupancy_from_stp(c->barrier_occupied_stp, c->barrier_not_occupied_stp);
  }
  // cli_update_tad_to_loop_contact_ratio (:1169-1182)
  const bool loop = (c->contact_sampling_strategy & MGPU_CS_LOOP) != 0;
  const bool tad = (c->contact_sampling_strategy & MGPU_CS_TAD) != 0;
  if (!loop && !tad) return MGPU_ERR_INVALID_ARG;
  if (loop && !tad) c->tad_to_loop_contact_ratio = 0;
  if (!loop && tad) c->tad_to_loop_contact_ratio = std::numeric_limits<double>::infinity();
  // cli_update_burnin_params (:1184-1190)
  const u64 act_bp = 5 * c->avg_lef_processivity;
  const u64 sp = c->rev_extrusion_speed_burnin + c->fwd_extrusion_speed_burnin;
  if (sp == 0) return MGPU_ERR_INVALID_ARG;
  c->burnin_target_epochs_for_lef_activation = std::min(c->max_burnin_epochs, act_bp / sp);
  // cli_normalize_probabilities (:1138-1167)
  if (c->normalize_probabilities) {
    const double ratio = static_cast<double>(c->rev_extrusion_speed + c->fwd_extrusion_speed) /
                         static_cast<double>(c->probability_normalization_factor);
    if (ratio != 1.0) {
      auto stable_pow = [](double base, double e) {
        if (base == 0.0) return 0.0;
        if (base == 1.0) return 1.0;
        return std::exp(std::log(base) * e);
      };
      c->barrier_not_occupied_stp = stable_pow(c->barrier_not_occupied_stp, ratio);
      c->barrier_occupied_stp =
          stp_from_occ(c->barrier_not_occupied_stp, c->extrusion_barrier_occupancy);
      const double p = c->probability_of_extrusion_unit_bypass;
      if (p != 0.0 && p != 1.0) c->probability_of_extrusion_unit_bypass = std::min(p * ratio, 1.0);
      c->lef_bar_major_collision_pblock = stable_pow(c->lef_bar_major_collision_pblock, ratio);
      c->lef_bar_minor_collision_pblock = stable_pow(c->lef_bar_minor_collision_pblock, ratio);
    }
  }
  if (c->stop_on_epochs) c->target_contact_density = -1;
  return MGPU_OK;
}

uint64_t orc_num_lefs(const mgpu_config* c, uint64_t size_bp) {
  const double mbp = static_cast<double>(size_bp) / 1.0e6;
  return std::max(u64(1), static_cast<u64>(std::round(c->number_of_lefs_per_mbp * mbp)));
}

uint64_t orc_contacts_per_epoch(const mgpu_config* c, uint64_t nlefs) {
  return Sim(*c).contacts_per_epoch(nlefs);
}

// Simulation::run_simulate task targets (scheduler_simulate.cpp:129-153) and
// compute_tot_target_epochs (simulation.cpp:1226-1241)
int orc_task_targets(const mgpu_config* c, uint64_t size_bp, uint64_t nlefs, uint64_t ncells,
                     uint64_t* targets, uint64_t* target_epochs) {
  const u64 npix1 = (c->diagonal_width + c->bin_size - 1) / c->bin_size;
  const u64 npix2 = (size_bp + c->bin_size - 1) / c->bin_size;
  const u64 npixels = std::min(npix1, npix2) * npix2;
  const u64 tot = static_cast<u64>(std::round(static_cast<double>(npixels) * c->target_contact_density));
  u64 epochs;
  if (c->stop_on_epochs) {
    epochs = c->num_cells * c->target_simulation_epochs;
  } else {
    const double tt = std::max(1.0, std::round(c->target_contact_density * static_cast<double>(npixels)));
    epochs = static_cast<u64>(std::round(tt / static_cast<double>(orc_contacts_per_epoch(c, nlefs))));
  }
  *target_epochs = epochs;
  const u64 per_cell = (tot + c->num_cells - 1) / c->num_cells;
  u64 rolling = 0;
  for (u64 i = 0; i < ncells; ++i) {
    const u64 eff = std::min(per_cell, tot - rolling);
    rolling += eff;
    targets[i] = eff;
  }
  return MGPU_OK;
}

void orc_prng_seed(uint64_t seed, uint64_t state[4]) {
  const Rng r = make_prng(seed);
  for (int i = 0; i < 4; ++i) state[i] = r.s[i];
}

// Raw draws of the stream (for PRNG golden tests).
void orc_prng_draws(uint64_t seed, uint64_t n, uint64_t* out) {
  Rng r = make_prng(seed);
  for (u64 i = 0; i < n; ++i) out[i] = r();
}

// Samples of each distribution from a fresh stream: kind 0 uniform_int[a,b], 1 bernoulli(p),
// 2 canonical, 3 uniform01, 4 normal(a=mean bits, p=sigma), 5 poisson(p), 6 binomial(t=a,p),
// 7 gev(mu=0, sigma=p, xi=0.001), 8 unit exponential.  Writes doubles; returns draws used.
uint64_t orc_sample(uint64_t seed, int kind, uint64_t a, uint64_t b, double p, double q,
                    uint64_t n, double* out) {
  Rng g = make_prng(seed);
  for (u64 i = 0; i < n; ++i) {
    switch (kind) {
      case 0: out[i] = static_cast<double>(uniform_int(g, a, b)); break;
      case 1: out[i] = bernoulli(g, p) ? 1.0 : 0.0; break;
      case 2: out[i] = canonical53(g); break;
      case 3: out[i] = uniform01(g); break;
      case 4: out[i] = normal(g, p, q); break;
      case 5: out[i] = static_cast<double>(poisson(g, p)); break;
      case 6: out[i] = static_cast<double>(binomial(g, static_cast<i64>(a), p)); break;
      case 7: out[i] = gev(g, 0.0, p, q); break;
      case 8: out[i] = unit_exponential(g); break;
      default: return 0;
    }
  }
  return g.ndraws;
}

int orc_simulate_cell_ex(const mgpu_config* cfg, const mgpu_chrom* chrom, const mgpu_barrier* bs,
                         uint64_t nb, uint64_t seed, uint64_t target_contacts,
                         uint64_t target_epochs, uint64_t nlefs, uint32_t* band,
                         mgpu_cell_stats* stats, mgpu_trace_request* trace, uint64_t* occupancy,
                         mgpu_epoch_record* records, uint64_t max_records, uint64_t cell_index,
                         uint64_t* records_written);

int orc_simulate_cell(const mgpu_config* cfg, const mgpu_chrom* chrom, const mgpu_barrier* bs,
                      uint64_t nb, uint64_t seed, uint64_t target_contacts,
                      uint64_t target_epochs, uint64_t nlefs, uint32_t* band,
                      mgpu_cell_stats* stats, mgpu_trace_request* trace) {
  return orc_simulate_cell_ex(cfg, chrom, bs, nb, seed, target_contacts, target_epochs, nlefs, band,
                              stats, trace, nullptr, nullptr, 0, 0, nullptr);
}

// orc_simulate_cell with the optional outputs: occupancy has ceil(chrom size / bin) counters
// (added to), records receives the cell's first max_records model-state records.
int orc_simulate_cell_ex(const mgpu_config* cfg, const mgpu_chrom* chrom, const mgpu_barrier* bs,
                         uint64_t nb, uint64_t seed, uint64_t target_contacts,
                         uint64_t target_epochs, uint64_t nlefs, uint32_t* band,
                         mgpu_cell_stats* stats, mgpu_trace_request* trace, uint64_t* occupancy,
                         mgpu_epoch_record* records, uint64_t max_records, uint64_t cell_index,
                         uint64_t* records_written) {
  if (!cfg || !chrom || nlefs == 0) return MGPU_ERR_INVALID_ARG;
  const Chrom ch{chrom->start, chrom->end, chrom->start, chrom->end};
  return simulate_cell_on(cfg, ch, bs, nb, seed, target_contacts, target_epochs, nlefs, band, stats, trace,
                          occupancy, records, max_records, cell_index, records_written);
}

// One cell of a modle perturbate window (Simulation::simulate_window,
// scheduler_perturbate.cpp:429-480): LEFs bind and contacts are sampled in [ws, we), the band
// covers the window, and moves are clamped by the chromosome's own range.
int orc_simulate_window_cell(const mgpu_config* cfg, const mgpu_chrom* chrom, uint64_t ws, uint64_t we,
                             const mgpu_barrier* bs, uint64_t nb, uint64_t seed, uint64_t target_contacts,
                             uint64_t target_epochs, uint64_t nlefs, uint32_t* band, mgpu_cell_stats* stats) {
  if (!cfg || !chrom || nlefs == 0 || ws < chrom->start || we > chrom->end || we <= ws)
    return MGPU_ERR_INVALID_ARG;
  const Chrom ch{chrom->start, chrom->end, ws, we};
  return simulate_cell_on(cfg, ch, bs, nb, seed, target_contacts, target_epochs, nlefs, band, stats, nullptr,
                          nullptr, nullptr, 0, 0, nullptr);
}

}  // extern "C"

static int simulate_cell_on(const mgpu_config* cfg, const Chrom& ch, const mgpu_barrier* bs, uint64_t nb,
                            uint64_t seed, uint64_t target_contacts, uint64_t target_epochs, uint64_t nlefs,
                            uint32_t* band, mgpu_cell_stats* stats, mgpu_trace_request* trace,
                            uint64_t* occupancy, mgpu_epoch_record* records, uint64_t max_records,
                            uint64_t cell_index, uint64_t* records_written) {
  Barriers b = make_barriers(bs, nb);
  Band bd;
  bd.nrows = std::min((cfg->diagonal_width + cfg->bin_size - 1) / cfg->bin_size,
                      (ch.we - ch.ws + cfg->bin_size - 1) / cfg->bin_size);
  bd.ncols = (ch.we - ch.ws + cfg->bin_size - 1) / cfg->bin_size;
  bd.data = band;
  Cell cell(*cfg, ch, b, nlefs);
  cell.occ = occupancy;
  cell.recs = records;
  cell.rec_max = max_records;
  cell.cell_index = cell_index;
  const CellResult r = cell.run(seed, target_contacts, target_epochs, bd, trace);
  if (records_written) *records_written = cell.nrec;
  if (stats) {
    stats->epochs = r.epochs;
    stats->burnin_epochs = r.burnin_epochs;
    stats->contacts = r.contacts;
    stats->missed_updates = bd.missed;
    stats->lef_epochs = r.lef_epochs;
    stats->rng_draws = r.draws;
    stats->sort_fallbacks = 0;
    stats->status = static_cast<u64>(r.status == MGPU_OK ? 0 : 1);
  }
  return r.status;
}

extern "C" {

// Multi-threaded driver: one worker per thread, each simulating whole cells, like the
// reference's simulate_worker pool (scheduler_simulate.cpp:96-101, 186-284).  Contacts go to
// one shared band with atomic increments.  Returns the wall time in seconds via *seconds.
int orc_simulate_cells_mt(const mgpu_config* cfg, const mgpu_chrom* chrom, const mgpu_barrier* bs,
                          uint64_t nb, const uint64_t* seeds, const uint64_t* targets,
                          uint64_t target_epochs, uint64_t nlefs, uint64_t ncells,
                          uint64_t nthreads, uint32_t* band, uint64_t* missed,
                          mgpu_cell_stats* stats) {
  if (!cfg || !chrom || nlefs == 0) return MGPU_ERR_INVALID_ARG;
  const Chrom ch{chrom->start, chrom->end, chrom->start, chrom->end};
  const Barriers b = make_barriers(bs, nb);
  const u64 nrows = std::min((cfg->diagonal_width + cfg->bin_size - 1) / cfg->bin_size,
                             (ch.end - ch.start + cfg->bin_size - 1) / cfg->bin_size);
  const u64 ncols = (ch.end - ch.start + cfg->bin_size - 1) / cfg->bin_size;
  std::atomic<u64> next{0};
  std::atomic<u64> missed_total{0};
  std::atomic<int> status{MGPU_OK};
  auto worker = [&]() {
    for (;;) {
      const u64 i = next.fetch_add(1);
      if (i >= ncells) return;
      Band bd;
      bd.nrows = nrows;
      bd.ncols = ncols;
      bd.data = band;
      bd.atomic = true;
      Cell cell(*cfg, ch, b, nlefs);
      const CellResult r = cell.run(seeds[i], targets[i], target_epochs, bd, nullptr);
      missed_total += bd.missed;
      if (r.status != MGPU_OK) status = r.status;
      if (stats) {
        stats[i].epochs = r.epochs;
        stats[i].burnin_epochs = r.burnin_epochs;
        stats[i].contacts = r.contacts;
        stats[i].missed_updates = bd.missed;
        stats[i].lef_epochs = r.lef_epochs;
        stats[i].rng_draws = r.draws;
        stats[i].sort_fallbacks = 0;
        stats[i].status = static_cast<u64>(r.status == MGPU_OK ? 0 : 1);
      }
    }
  };
  std::vector<std::thread> pool;
  const u64 nt = std::max<u64>(1, nthreads);
  for (u64 t = 0; t < nt; ++t) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  if (missed) *missed += missed_total.load();
  return status.load();
}

uint64_t orc_state_digest(uint64_t n, const uint64_t* rev, const uint64_t* fwd,
                          const uint64_t* ep, const uint64_t* rr, const uint64_t* fr,
                          const uint64_t* rm, const uint64_t* fm, const uint64_t* rc,
                          const uint64_t* fc) {
  u64 d = 0;
  for (u64 i = 0; i < n; ++i) {
    const u64 v[9] = {rev[i], fwd[i], ep[i], rr[i], fr[i], rm[i], fm[i], rc[i], fc[i]};
    d += digest_entry(i, v);
  }
  return d;
}

// One step of the epoch loop on caller-provided state (same contract as mgpu_run_phase).
int orc_run_phase(const mgpu_config* cfg, const mgpu_chrom* chrom, const mgpu_barrier* bs,
                  uint64_t nb, int phase, mgpu_phase_io* io) {
  if (!cfg || !chrom || !io) return MGPU_ERR_INVALID_ARG;
  const usize n = io->num_lefs;
  const Chrom ch{chrom->start, chrom->end, chrom->start, chrom->end};
  Barriers b;
  for (u64 i = 0; i < nb; ++i) {
    b.pos.push_back(bs[i].pos);
    b.dir.push_back(bs[i].blocking_dir);
    b.stp_active.push_back(bs[i].stp_active);
    b.stp_inactive.push_back(bs[i].stp_inactive);
    b.state.push_back(io->barrier_state ? io->barrier_state[i] : 1);
  }
  std::vector<Lef> lefs(n);
  std::vector<usize> rr(n), fr(n);
  std::vector<bp_t> rm(n), fm(n);
  std::vector<Coll> rc(n), fc(n);
  for (usize i = 0; i < n; ++i) {
    lefs[i].rev = io->rev_pos[i];
    lefs[i].fwd = io->fwd_pos[i];
    lefs[i].binding_epoch = io->binding_epoch[i];
    rr[i] = io->rev_rank[i];
    fr[i] = io->fwd_rank[i];
    rm[i] = io->rev_move[i];
    fm[i] = io->fwd_move[i];
    rc[i].w = io->rev_collision[i];
    fc[i].w = io->fwd_collision[i];
  }
  Rng g;
  for (int k = 0; k < 4; ++k) g.s[k] = io->prng_state[k];
  Sim sim(*cfg);
  bool ub = false;
  switch (phase) {
    case MGPU_PHASE_BIND: {
      std::vector<u64> mask(n, 1);
      if (io->bind_mask)
        for (usize i = 0; i < n; ++i) mask[i] = io->bind_mask[i];
      sim.bind_lefs(ch.start, ch.end, lefs, n, rr, fr, io->bind_mask ? mask.data() : nullptr, g,
                    io->epoch);
      break;
    }
    case MGPU_PHASE_RANK:
      Sim::rank_lefs(lefs, n, rr, fr, io->ranks_partially_sorted != 0, io->init_ranks != 0);
      break;
    case MGPU_PHASE_ADJUST_AND_CLAMP:
      Sim::adjust_moves(ch, lefs, n, rr, fr, rm, fm);
      Sim::clamp_moves(ch, lefs, n, rm, fm);
      break;
    case MGPU_PHASE_GENERATE_MOVES:
      sim.generate_moves(ch, lefs, n, rr, fr, rm, fm, io->burnin_completed != 0, g,
                         io->adjust_moves != 0);
      break;
    case MGPU_PHASE_PROCESS_COLLISIONS: {
      const auto [n5, n3] =
          sim.process_collisions(ch, lefs, n, b, rr, fr, rm, fm, rc, fc, g, false, &ub);
      io->n5prime = n5;
      io->n3prime = n3;
      break;
    }
    case MGPU_PHASE_FIX_SECONDARY:
      Sim::fix_secondary(ch, lefs, n, rr, fr, rm, fm, rc, fc, 0, 0);
      break;
    case MGPU_PHASE_DETECT_LEF_BAR:
      sim.detect_lef_bar(lefs, n, rr, fr, rm, fm, b, rc, fc, g, 0, 0);
      break;
    case MGPU_PHASE_LEF_LEF:
      sim.detect_primary(lefs, n, b, rr, fr, rm, fm, rc, fc, g, 0, 0, &ub);
      Sim::correct_primary(lefs, n, rr, fr, rm, fm, rc, fc);
      sim.process_secondary(lefs, n, rr, fr, rm, fm, rc, fc, g, 0, 0);
      break;
    case MGPU_PHASE_DETECT_PRIMARY:
      sim.detect_primary(lefs, n, b, rr, fr, rm, fm, rc, fc, g, 0, 0, &ub);
      break;
    case MGPU_PHASE_DETECT_BOUNDARIES: {
      const auto [n5, n3] = Sim::detect_boundaries(ch, lefs, n, rr, fr, rm, fm, rc, fc, &ub);
      io->n5prime = n5;
      io->n3prime = n3;
      break;
    }
    case MGPU_PHASE_CORRECT_LEF_BAR:
      Sim::correct_lef_bar(lefs, n, b, rm, fm, rc, fc);
      break;
    case MGPU_PHASE_CORRECT_PRIMARY:
      Sim::correct_primary(lefs, n, rr, fr, rm, fm, rc, fc);
      break;
    case MGPU_PHASE_EXTRUDE:
      Sim::extrude(lefs, n, rm, fm);
      break;
    case MGPU_PHASE_RELEASE:
      io->lefs_released = sim.release_lefs(lefs, n, b, rc, fc, g, io->burnin_completed != 0);
      break;
    case MGPU_PHASE_BARRIER_NEXT:
      b.next_state(g);
      break;
    case MGPU_PHASE_BARRIER_INIT:
      b.init_states(g);
      break;
    default:
      return MGPU_ERR_INVALID_ARG;
  }
  for (usize i = 0; i < n; ++i) {
    io->rev_pos[i] = lefs[i].rev;
    io->fwd_pos[i] = lefs[i].fwd;
    io->binding_epoch[i] = lefs[i].binding_epoch;
    io->rev_rank[i] = rr[i];
    io->fwd_rank[i] = fr[i];
    io->rev_move[i] = rm[i];
    io->fwd_move[i] = fm[i];
    io->rev_collision[i] = rc[i].w;
    io->fwd_collision[i] = fc[i].w;
  }
  if (io->barrier_state)
    for (u64 i = 0; i < nb; ++i) io->barrier_state[i] = b.state[i];
  for (int k = 0; k < 4; ++k) io->prng_state[k] = g.s[k];
    return ub ? MGPU_ERR_INTERNAL : MGPU_OK;
}

// Pixel table of one chromosome's band, in the order Cooler::write_or_append_cmatrix_to_file
// emits it (src/libmodle_io/cooler_write_impl.hpp:275-316): bin1 i over the columns, bin2 j from i
// to min(i + nrows, ncols) - 1, non-zero counts only, where the count of (i, j) is the band
// entry at column j, row j - i (transpose_coords / encode_idx,
// src/contact_matrix/contact_matrix_internal_impl.hpp:19-42).  bin1_offset[i] is the number of
// pixels before row i (ncols + 1 entries).  Pixels are written only when capacity suffices.
int orc_band_to_pixels(const uint32_t* band, uint64_t nrows, uint64_t ncols, uint64_t bin_offset,
                       uint64_t* bin1_offset, int64_t* bin1, int64_t* bin2, uint32_t* count,
                       uint64_t capacity, uint64_t* nnz) {
  uint64_t k = 0;
  for (uint64_t i = 0; i < ncols; ++i) {
    bin1_offset[i] = k;
    for (uint64_t j = i; j < i + nrows && j < ncols; ++j) {
      const uint32_t m = band[j * nrows + (j - i)];
      if (m == 0) continue;
      if (k < capacity) {
        bin1[k] = (int64_t)(bin_offset + i);
        bin2[k] = (int64_t)(bin_offset + j);
        count[k] = m;
      }
      ++k;
    }
  }
  bin1_offset[ncols] = k;
  *nnz = k;
  return k <= capacity ? MGPU_OK : MGPU_ERR_OVERFLOW;
}


// Full-tie counters of the epoch loop's rank_lefs calls: enable (1) or disable (0) counting,
// optionally reset, and read out[0] = rank_lefs calls counted, out[1] = calls with at least one
// full tie, out[2] = adjacent full-tie pairs (rev and fwd orders together), out[3] = those of
// out[2] away from the chromosome ends.
void orc_tie_counters(int enable, int reset, uint64_t out[4]) {
  if (reset) {
    g_tie_rank_calls = 0;
    g_tie_calls = 0;
    g_tie_pairs = 0;
    g_tie_interior = 0;
  }
  g_count_ties = enable != 0;
  if (out) {
    out[0] = g_tie_rank_calls.load();
    out[1] = g_tie_calls.load();
    out[2] = g_tie_pairs.load();
    out[3] = g_tie_interior.load();
  }
}

// Band shape of ContactMatrixDense(length, diagonal_width, bin_size)
// (src/contact_matrix/contact_matrix_dense_impl.hpp:40-51) and Chromosome::npixels
// (src/libmodle/internal/genome_impl.hpp:20-25).
void orc_band_shape(const mgpu_config* c, uint64_t size_bp, uint64_t* nrows, uint64_t* ncols) {
  const u64 bins = (size_bp + c->bin_size - 1) / c->bin_size;
  const u64 diag = (c->diagonal_width + c->bin_size - 1) / c->bin_size;
  *nrows = diag < bins ? diag : bins;
  *ncols = bins;
}

// Chromosome::add_extrusion_barrier (src/libmodle/internal/genome.cpp:194-210) with
// compute_barrier_stp (genome.cpp:181-192) and ExtrusionBarrier's motif-to-blocking-direction
// rule (extrusion_barriers_impl.hpp:48-72): the barrier sits at the BED interval's midpoint
// (start + end + 1) / 2; a non-zero score is the occupancy, from which stp_active follows
// (compute_stp_active_from_occupancy, extrusion_barriers_impl.hpp:106-116); strand '+' blocks
// reverse units.  Returns 1 and fills *out for a barrier inside [chrom->start, chrom->end),
// 0 for one outside it, MGPU_ERR_INVALID_ARG for a bad strand.
int orc_barrier_from_bed(const mgpu_chrom* chrom, uint64_t bed_start, uint64_t bed_end, char strand,
                         double score, double stp_active_default, double stp_inactive_default,
                         mgpu_barrier* out) {
  if (strand != '+' && strand != '-') return MGPU_ERR_INVALID_ARG;
  const u64 mid = (bed_start + bed_end + 1) / 2;
  if (mid < chrom->start || mid >= chrom->end) return 0;
  double active = stp_active_default;
  if (score != 0.0) {
    const double free_to_bound = 1.0 - stp_inactive_default;
    const double bound_to_free = (free_to_bound - (score * free_to_bound)) / score;
    active = std::clamp(1.0 - bound_to_free, 0.0, 1.0);
  }
  *out = mgpu_barrier{};
  out->pos = mid;
  out->stp_active = active;
  out->stp_inactive = stp_inactive_default;
  out->blocking_dir = strand == '+' ? MGPU_DIR_REV : MGPU_DIR_FWD;
  return 1;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// XXH3-64 with a seed, for Chromosome::hash (src/libmodle/internal/genome.cpp:317-335).
// xxHash 0.8.1 is a dependency the reference does not vendor; this restates the published
// XXH3 specification (doc/xxhash_spec.md of the xxHash project) for inputs of at most 240
// bytes, the only lengths a chromosome name plus two 64-bit words reach.  It is written
// independently of the product's own hash so that the CPU arm derives its seeds without the
// product library.
// ---------------------------------------------------------------------------------------
namespace orc_xxh3 {
// The 192-byte default secret of the specification.
static const u8 kDefaultSecret[192] = {
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
static const u64 kPrime32[3] = {0x9E3779B1ull, 0x85EBCA77ull, 0xC2B2AE3Dull};
static const u64 kPrime64[5] = {0x9E3779B185EBCA87ull, 0xC2B2AE3D27D4EB4Full, 0x165667B19E3779F9ull,
                                0x85EBCA77C2B2AE63ull, 0x27D4EB2F165667C5ull};

// Little-endian reads of k bytes, independent of the host's byte order.
static u64 le(const u8* p, int k) {
  u64 v = 0;
  for (int i = 0; i < k; ++i) v |= static_cast<u64>(p[i]) << (8 * i);
  return v;
}
static u64 rotl64(u64 x, unsigned r) { return (x << r) | (x >> (64 - r)); }
// Byte reversal of the low 32 bits.
static u64 swap32(u64 x) {
  return ((x & 0xffu) << 24) | ((x & 0xff00u) << 8) | ((x >> 8) & 0xff00u) | ((x >> 24) & 0xffu);
}
static u64 swap64(u64 x) {
  u64 r = 0;
  for (int i = 0; i < 8; ++i, x >>= 8) r = (r << 8) | (x & 0xffu);
  return r;
}
// 64x64 -> 128-bit product, folded by xor of its halves.
static u64 fold_mul(u64 a, u64 b) {
  const unsigned __int128 m = static_cast<unsigned __int128>(a) * b;
  return static_cast<u64>(m) ^ static_cast<u64>(m >> 64);
}
static u64 avalanche_xxh64(u64 h) {
  h = (h ^ (h >> 33)) * kPrime64[1];
  h = (h ^ (h >> 29)) * kPrime64[2];
  return h ^ (h >> 32);
}
static u64 avalanche_xxh3(u64 h) {
  h = (h ^ (h >> 37)) * 0x165667919E3779F9ull;
  return h ^ (h >> 32);
}
// One 16-byte lane of input against 16 bytes of secret.
static u64 lane16(const u8* in, const u8* sec, u64 seed) {
  const u64 lo = le(in, 8) ^ (le(sec, 8) + seed);
  const u64 hi = le(in + 8, 8) ^ (le(sec + 8, 8) - seed);
  return fold_mul(lo, hi);
}

static bool hash64(const u8* in, u64 n, u64 seed, u64* out) {
  const u8* sec = kDefaultSecret;
  if (n == 0) {
    *out = avalanche_xxh64(seed ^ le(sec + 56, 8) ^ le(sec + 64, 8));
  } else if (n < 4) {
    const u64 word = (static_cast<u64>(in[0]) << 16) | (static_cast<u64>(in[n / 2]) << 24) |
                     static_cast<u64>(in[n - 1]) | (n << 8);
    const u64 key = (le(sec, 4) ^ le(sec + 4, 4)) + seed;
    *out = avalanche_xxh64(word ^ key);
  } else if (n <= 8) {
    const u64 s2 = seed ^ (swap32(seed & 0xffffffffu) << 32);
    const u64 key = (le(sec + 8, 8) ^ le(sec + 16, 8)) - s2;
    const u64 v = le(in + n - 4, 4) + (le(in, 4) << 32);
    u64 h = v ^ key;
    h ^= rotl64(h, 49) ^ rotl64(h, 24);
    h *= 0x9FB21C651E98DF25ull;
    h ^= (h >> 35) + n;
    h *= 0x9FB21C651E98DF25ull;
    *out = h ^ (h >> 28);
  } else if (n <= 16) {
    const u64 lo = le(in, 8) ^ ((le(sec + 24, 8) ^ le(sec + 32, 8)) + seed);
    const u64 hi = le(in + n - 8, 8) ^ ((le(sec + 40, 8) ^ le(sec + 48, 8)) - seed);
    *out = avalanche_xxh3(n + swap64(lo) + hi + fold_mul(lo, hi));
  } else if (n <= 128) {
    // Pairs of lanes taken from both ends inwards: pair k reads bytes [16k, 16k + 16) and
    // [n - 16(k + 1), n - 16k) against secret bytes [32k, 32k + 32).
    u64 acc = n * kPrime64[0];
    const u64 pairs = (n - 1) / 32 + 1;
    for (u64 k = 0; k < pairs; ++k) {
      acc += lane16(in + 16 * k, sec + 32 * k, seed);
      acc += lane16(in + n - 16 * (k + 1), sec + 32 * k + 16, seed);
    }
    *out = avalanche_xxh3(acc);
  } else if (n <= 240) {
    u64 acc = n * kPrime64[0];
    for (u64 k = 0; k < 8; ++k) acc += lane16(in + 16 * k, sec + 16 * k, seed);
    acc = avalanche_xxh3(acc);
    for (u64 k = 8; k < n / 16; ++k) acc += lane16(in + 16 * k, sec + 16 * (k - 8) + 3, seed);
    acc += lane16(in + n - 16, sec + 136 - 17, seed);
    *out = avalanche_xxh3(acc);
  } else {
    return false;
  }
  return true;
}
}  // namespace orc_xxh3

extern "C" {

// The host libm (glibc, as the reference links it) on arguments: out[i] = f(x[i], y[i]) with
// the kinds of the device probe: 0 log x, 1 exp x, 2 pow(x, y), 3 the GEV noise of a uniform x
// (genextreme_value_distribution.hpp:87-105) with (mu, sigma, xi), 4 x < exp(y) as 1.0 / 0.0.
// Threads split the range.
int orc_libm_eval(int kind, const double* x, const double* y, uint64_t n, double mu, double sigma, double xi,
                  double* out, uint64_t nthreads) {
  if (kind < 0 || kind > 4) return MGPU_ERR_INVALID_ARG;
  auto work = [&](u64 lo, u64 hi) {
    for (u64 i = lo; i < hi; ++i) {
      const double a = x[i];
      double r = 0.0;
      switch (kind) {
        case 0: r = std::log(a); break;
        case 1: r = std::exp(a); break;
        case 2: r = std::pow(a, y[i]); break;
        case 3:
          r = xi == 0.0 ? (mu - sigma) * std::log(-std::log(a))
                        : mu + (sigma * (1.0 - std::pow(-std::log(a), xi))) / xi;
          break;
        case 4: r = a < std::exp(y[i]) ? 1.0 : 0.0; break;
      }
      out[i] = r;
    }
  };
  const u64 nt = std::max<u64>(1, std::min<u64>(nthreads, n / 4096 + 1));
  std::vector<std::thread> pool;
  for (u64 t = 0; t < nt; ++t) pool.emplace_back(work, n * t / nt, n * (t + 1) / nt);
  for (auto& t : pool) t.join();
  return MGPU_OK;
}

// orc_sample over many streams in parallel: per_stream samples of one kind from each seed
// (out[s * per_stream + i]), draws[s] = raw draws stream s took.
int orc_sample_streams(const uint64_t* seeds, uint64_t nstreams, uint64_t per_stream, int kind, uint64_t a,
                       uint64_t b, double p, double q, double* out, uint64_t* draws, uint64_t nthreads) {
  std::atomic<u64> next{0};
  auto work = [&]() {
    for (;;) {
      const u64 s = next.fetch_add(1);
      if (s >= nstreams) return;
      draws[s] = orc_sample(seeds[s], kind, a, b, p, q, per_stream, out + s * per_stream);
    }
  };
  std::vector<std::thread> pool;
  for (u64 t = 0; t < std::max<u64>(1, nthreads); ++t) pool.emplace_back(work);
  for (auto& t : pool) t.join();
  return MGPU_OK;
}

// XXH3_64bits_withSeed for inputs of at most 240 bytes (0 with *ok = 0 beyond).
uint64_t orc_xxh3_64(const void* data, uint64_t len, uint64_t seed, int* ok) {
  u64 h = 0;
  const bool good = orc_xxh3::hash64(static_cast<const u8*>(data), len, seed, &h);
  if (ok) *ok = good ? 1 : 0;
  return h;
}

// Chromosome::hash (genome.cpp:317-335): XXH3 with Config::seed over the name's bytes, the
// chromosome size and the cell id (both 64-bit little-endian).
uint64_t orc_cell_seed(const char* name, uint64_t name_len, uint64_t chrom_size, uint64_t seed,
                       uint64_t cell_id) {
  std::vector<u8> msg(name_len + 16);
  std::memcpy(msg.data(), name, name_len);
  for (int i = 0; i < 8; ++i) {
    msg[name_len + i] = static_cast<u8>(chrom_size >> (8 * i));
    msg[name_len + 8 + i] = static_cast<u8>(cell_id >> (8 * i));
  }
  u64 h = 0;
  orc_xxh3::hash64(msg.data(), msg.size(), seed, &h);
  return h;
}

}  // extern "C"
