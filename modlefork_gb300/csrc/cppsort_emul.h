// cppsort_emul.h - pattern-defeating quicksort, split sort and insertion sort on index
// arrays, with the exact element movements of cpp-sort 1.13 (split_sort, pdq_sort,
// insertion_sort), which MoDLE uses in rank_lefs (src/libmodle/cpu/simulation.cpp:427-483)
// and ExtrusionBarriers::sort (src/libmodle/internal/extrusion_barriers.cpp:239-244).
// Orders of equal keys depend on those movements, so they are reproduced step by step:
// Peters' pdqsort (insertion below 24 elements, median-of-3 / pseudo-median-of-9 pivots,
// partition_right / partition_left, partial insertion sort, heap sort fallback after log2(n)
// unbalanced partitions) and split_sort (approximate longest ascending subsequence kept on the
// left, the rest pdq-sorted and merged stably).
// Algorithms: pdqsort by Orson Peters (zlib licence), as adopted by cpp-sort 1.13 by Morwenn
// (MIT licence); split_sort of cpp-sort 1.13.  This file restates their published steps.
#pragma once
#include "mgpu_internal.h"

namespace mgpu {

struct KeyCmp {
  const u32* key;
  MGPU_HD bool operator()(u32 a, u32 b) const { return key[a] < key[b]; }
};
struct KeyCmpRev {  // b < a on the key (descending)
  const u32* key;
  MGPU_HD bool operator()(u32 a, u32 b) const { return key[b] < key[a]; }
};

template <class Cmp>
MGPU_HD void ins_sort(u32* a, i64 lo, i64 hi, Cmp comp) {
  if (lo == hi) return;
  for (i64 cur = lo + 1; cur != hi; ++cur) {
    i64 sift = cur, sift_1 = cur - 1;
    if (comp(a[sift], a[sift_1])) {
      const u32 tmp = a[sift];
      do {
        a[sift--] = a[sift_1];
      } while (sift != lo && comp(tmp, a[--sift_1]));
      a[sift] = tmp;
    }
  }
}

template <class Cmp>
MGPU_HD void unguarded_ins_sort(u32* a, i64 lo, i64 hi, Cmp comp) {
  if (lo == hi) return;
  for (i64 cur = lo + 1; cur != hi; ++cur) {
    i64 sift = cur, sift_1 = cur - 1;
    if (comp(a[sift], a[sift_1])) {
      const u32 tmp = a[sift];
      do {
        a[sift--] = a[sift_1];
      } while (comp(tmp, a[--sift_1]));
      a[sift] = tmp;
    }
  }
}

template <class Cmp>
MGPU_HD bool partial_ins_sort(u32* a, i64 lo, i64 hi, Cmp comp) {
  if (lo == hi) return true;
  u64 limit = 0;
  for (i64 cur = lo + 1; cur != hi; ++cur) {
    i64 sift = cur, sift_1 = cur - 1;
    if (comp(a[sift], a[sift_1])) {
      const u32 tmp = a[sift];
      do {
        a[sift--] = a[sift_1];
      } while (sift != lo && comp(tmp, a[--sift_1]));
      a[sift] = tmp;
      limit += (u64)(cur - sift);
    }
    if (limit > 8) return false;
  }
  return true;
}

MGPU_HD inline void swp(u32* a, i64 i, i64 j) {
  const u32 t = a[i];
  a[i] = a[j];
  a[j] = t;
}

template <class Cmp>
MGPU_HD inline void sort2(u32* a, i64 i, i64 j, Cmp comp) {
  if (comp(a[j], a[i])) swp(a, i, j);
}

template <class Cmp>
MGPU_HD inline void sort3(u32* a, i64 i, i64 j, i64 k, Cmp comp) {
  sort2(a, i, j, comp);
  sort2(a, j, k, comp);
  sort2(a, i, j, comp);
}

template <class Cmp>
MGPU_HD i64 partition_right(u32* a, i64 begin, i64 end, Cmp comp, bool& already) {
  const u32 pivot = a[begin];
  i64 first = begin, last = end;
  while (comp(a[++first], pivot)) {
  }
  if (first - 1 == begin) {
    while (first < last && !comp(a[--last], pivot)) {
    }
  } else {
    while (!comp(a[--last], pivot)) {
    }
  }
  already = first >= last;
  while (first < last) {
    swp(a, first, last);
    while (comp(a[++first], pivot)) {
    }
    while (!comp(a[--last], pivot)) {
    }
  }
  const i64 pivot_pos = first - 1;
  a[begin] = a[pivot_pos];
  a[pivot_pos] = pivot;
  return pivot_pos;
}

template <class Cmp>
MGPU_HD i64 partition_left(u32* a, i64 begin, i64 end, Cmp comp) {
  const u32 pivot = a[begin];
  i64 first = begin, last = end;
  while (comp(pivot, a[--last])) {
  }
  if (last + 1 == end) {
    while (first < last && !comp(pivot, a[++first])) {
    }
  } else {
    while (!comp(pivot, a[++first])) {
    }
  }
  while (first < last) {
    swp(a, first, last);
    while (comp(pivot, a[--last])) {
    }
    while (!comp(pivot, a[++first])) {
    }
  }
  const i64 pivot_pos = last;
  a[begin] = a[pivot_pos];
  a[pivot_pos] = pivot;
  return pivot_pos;
}

template <class Cmp>
MGPU_HD void adjust_heap(u32* a, i64 base, i64 hole, i64 len, u32 value, Cmp comp) {
  const i64 top = hole;
  i64 child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (comp(a[base + child], a[base + child - 1])) child--;
    a[base + hole] = a[base + child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    a[base + hole] = a[base + child - 1];
    hole = child - 1;
  }
  i64 parent = (hole - 1) / 2;
  while (hole > top && comp(a[base + parent], value)) {
    a[base + hole] = a[base + parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  a[base + hole] = value;
}

template <class Cmp>
MGPU_HD void heap_sort(u32* a, i64 lo, i64 hi, Cmp comp) {
  const i64 len = hi - lo;
  if (len < 2) return;
  for (i64 parent = (len - 2) / 2;; --parent) {
    adjust_heap(a, lo, parent, len, a[lo + parent], comp);
    if (parent == 0) break;
  }
  for (i64 last = hi; last - lo > 1;) {
    --last;
    const u32 v = a[last];
    a[last] = a[lo];
    adjust_heap(a, lo, 0, last - lo, v, comp);
  }
}

template <class Cmp>
MGPU_HD void pdq_sort(u32* a, i64 lo, i64 hi, Cmp comp) {
  if (lo == hi) return;
  i64 n = hi - lo;
  int log2n = 0;
  while (n >>= 1) ++log2n;
  struct Task {
    i64 begin, end;
    int bad;
    bool leftmost;
  };
  Task stack[64];  // depth <= log2(n) + 1 < 64 for 32-bit sizes
  int sp = 0;
  stack[sp++] = {lo, hi, log2n, true};
  while (sp > 0) {
    Task t = stack[--sp];
    i64 begin = t.begin, end = t.end;
    int bad_allowed = t.bad;
    bool leftmost = t.leftmost;
    for (;;) {
      const i64 size = end - begin;
      if (size < 24) {
        if (leftmost) {
          ins_sort(a, begin, end, comp);
        } else {
          unguarded_ins_sort(a, begin, end, comp);
        }
        break;
      }
      const i64 s2 = size / 2;
      if (size > 128) {
        sort3(a, begin, begin + s2, end - 1, comp);
        sort3(a, begin + 1, begin + (s2 - 1), end - 2, comp);
        sort3(a, begin + 2, begin + (s2 + 1), end - 3, comp);
        sort3(a, begin + (s2 - 1), begin + s2, begin + (s2 + 1), comp);
        swp(a, begin, begin + s2);
      } else {
        sort3(a, begin + s2, begin, end - 1, comp);
      }
      if (!leftmost && !comp(a[begin - 1], a[begin])) {
        begin = partition_left(a, begin, end, comp) + 1;
        continue;
      }
      bool already = false;
      const i64 pivot_pos = partition_right(a, begin, end, comp, already);
      const i64 l_size = pivot_pos - begin;
      const i64 r_size = end - (pivot_pos + 1);
      const bool highly_unbalanced = l_size < size / 8 || r_size < size / 8;
      if (highly_unbalanced) {
        if (--bad_allowed == 0) {
          heap_sort(a, begin, end, comp);
          break;
        }
        if (l_size >= 24) {
          swp(a, begin, begin + l_size / 4);
          swp(a, pivot_pos - 1, pivot_pos - l_size / 4);
          if (l_size > 128) {
            swp(a, begin + 1, begin + (l_size / 4 + 1));
            swp(a, begin + 2, begin + (l_size / 4 + 2));
            swp(a, pivot_pos - 2, pivot_pos - (l_size / 4 + 1));
            swp(a, pivot_pos - 3, pivot_pos - (l_size / 4 + 2));
          }
        }
        if (r_size >= 24) {
          swp(a, pivot_pos + 1, pivot_pos + (1 + r_size / 4));
          swp(a, end - 1, end - r_size / 4);
          if (r_size > 128) {
            swp(a, pivot_pos + 2, pivot_pos + (2 + r_size / 4));
            swp(a, pivot_pos + 3, pivot_pos + (3 + r_size / 4));
            swp(a, end - 2, end - (1 + r_size / 4));
            swp(a, end - 3, end - (2 + r_size / 4));
          }
        }
      } else {
        if (already && partial_ins_sort(a, begin, pivot_pos, comp) &&
            partial_ins_sort(a, pivot_pos + 1, end, comp)) {
          break;
        }
      }
      // The two parts are disjoint and each only reads its own range plus the final pivot
      // before it, so the order they are sorted in does not change the result; deferring the
      // larger one bounds the stack by log2(n).
      if (pivot_pos - begin < end - (pivot_pos + 1)) {
        stack[sp++] = {pivot_pos + 1, end, bad_allowed, false};
        end = pivot_pos;
      } else {
        stack[sp++] = {begin, pivot_pos, bad_allowed, leftmost};
        begin = pivot_pos + 1;
        leftmost = false;
      }
    }
  }
}

template <class Cmp>
MGPU_HD void split_sort(u32* a, i64 n, u32* tmp, Cmp comp) {
  if (n < 2) return;
  i64 middle = 0;
  for (i64 reader = 1; reader != n; ++reader) {
    if (comp(a[reader], a[middle])) {
      if (middle != 0) --middle;
    } else {
      ++middle;
      swp(a, middle, reader);
    }
  }
  pdq_sort(a, middle + 1, n, comp);
  // stable merge of [0, middle] and (middle, n)
  const i64 nl = middle + 1;
  for (i64 k = 0; k < nl; ++k) tmp[k] = a[k];
  i64 l = 0, r = nl, out = 0;
  while (l < nl && r < n) {
    if (comp(a[r], tmp[l])) {
      a[out++] = a[r++];
    } else {
      a[out++] = tmp[l++];
    }
  }
  while (l < nl) a[out++] = tmp[l++];
}

}  // namespace mgpu
