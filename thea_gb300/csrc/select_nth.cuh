// Selection of the nth smallest of a short array in place, leaving the array permuted exactly as GCC's libstdc++
// std::nth_element leaves it (host and device; compiles with nvcc and with a plain C++ compiler).
//
// The reference's ShapeDiameter (SurfaceFeatures/Local/ShapeDiameter.hpp:199-217) calls std::nth_element on its hit
// distances but not on the parallel array of weights, then pairs values[i] with weights[i]: its result depends on the
// permutation the standard library's selection leaves behind, not only on the selected value. The permutation here is
// that of the introselect algorithm (D. R. Musser, "Introspective Sorting and Selection Algorithms", 1997) with the
// choices libstdc++ makes: ranges of more than 3 elements are partitioned around the median of the second, middle and
// last elements (moved to the front first) by an unguarded Hoare partition; after 2 floor(log2 n) partitions without
// reaching a short range, heap selection (a binary max-heap of the first nth + 1 elements, sift-down to a leaf then
// sift-up, J. W. J. Williams / R. W. Floyd) finishes; short ranges are finished by insertion sort. The test suite checks
// the permutation against the C++ library's own std::nth_element on random and adversarial arrays.
#pragma once

#if defined(__CUDACC__)
#define THEA_SELECT_HD __host__ __device__ __forceinline__
#else
#define THEA_SELECT_HD inline
#endif

namespace thea {
namespace select_detail {

template <class T> THEA_SELECT_HD void swap_at(T * a, int i, int j) {
  T t = a[i];
  a[i] = a[j];
  a[j] = t;
}

// Moves the median of a[x], a[y], a[z] to a[to]
template <class T> THEA_SELECT_HD void median_to(T * a, int to, int x, int y, int z) {
  if (a[x] < a[y]) {
    if (a[y] < a[z]) swap_at(a, to, y);
    else if (a[x] < a[z]) swap_at(a, to, z);
    else swap_at(a, to, x);
  } else if (a[x] < a[z]) {
    swap_at(a, to, x);
  } else if (a[y] < a[z]) {
    swap_at(a, to, z);
  } else {
    swap_at(a, to, y);
  }
}

// Hoare partition of a[lo, hi) around the value at a[pivot] (pivot < lo); the scans rely on sentinels, none checks a
// bound. Returns the first position of the upper part.
template <class T> THEA_SELECT_HD int partition_unguarded(T * a, int lo, int hi, int pivot) {
  for (;;) {
    while (a[lo] < a[pivot]) ++lo;
    --hi;
    while (a[pivot] < a[hi]) --hi;
    if (!(lo < hi)) return lo;
    swap_at(a, lo, hi);
    ++lo;
  }
}

// Max-heap on a[base, base + len): places `value` starting from the hole at `hole` by moving the larger child up until
// a leaf is reached, then sifting the value up no higher than `top`
template <class T> THEA_SELECT_HD void heap_fill_hole(T * a, int base, int hole, int len, T value) {
  int top = hole, child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);                              // right child
    if (a[base + child] < a[base + child - 1]) --child;   // the larger child, left on ties
    a[base + hole] = a[base + child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {         // a last node with a left child only
    child = 2 * (child + 1);
    a[base + hole] = a[base + child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && a[base + parent] < value) {
    a[base + hole] = a[base + parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  a[base + hole] = value;
}

// Heap selection: the smallest (mid - first) elements of a[first, last) end up in a[first, mid) as a max-heap
template <class T> THEA_SELECT_HD void heap_select(T * a, int first, int mid, int last) {
  int len = mid - first;
  if (len >= 2)
    for (int parent = (len - 2) / 2;; --parent) {
      heap_fill_hole(a, first, parent, len, a[first + parent]);
      if (parent == 0) break;
    }
  for (int i = mid; i < last; ++i)
    if (a[i] < a[first]) {  // replace the heap's maximum
      T value = a[i];
      a[i] = a[first];
      heap_fill_hole(a, first, 0, len, value);
    }
}

template <class T> THEA_SELECT_HD void insertion_sort(T * a, int first, int last) {
  if (first == last) return;
  for (int i = first + 1; i < last; ++i) {
    T value = a[i];
    if (value < a[first]) {
      for (int j = i; j > first; --j) a[j] = a[j - 1];
      a[first] = value;
    } else {
      int j = i;
      while (value < a[j - 1]) {
        a[j] = a[j - 1];
        --j;
      }
      a[j] = value;
    }
  }
}

THEA_SELECT_HD int floor_log2(int n) {
  int k = 0;
  while (n > 1) {
    n >>= 1;
    ++k;
  }
  return k;
}

}  // namespace select_detail

// a[nth] becomes the element a sorted a[0, n) would hold there, with no larger element before it and no smaller one
// after; the rest of the permutation is libstdc++'s.
template <class T> THEA_SELECT_HD void select_nth(T * a, int n, int nth) {
  using namespace select_detail;
  if (n <= 0 || nth >= n) return;
  int first = 0, last = n;
  int depth = 2 * floor_log2(n);
  while (last - first > 3) {
    if (depth == 0) {
      heap_select(a, first, nth + 1, last);
      swap_at(a, first, nth);
      return;
    }
    --depth;
    median_to(a, first, first + 1, first + (last - first) / 2, last - 1);
    int cut = partition_unguarded(a, first + 1, last, first);
    if (cut <= nth) first = cut;
    else last = cut;
  }
  insertion_sort(a, first, last);
}

}  // namespace thea
