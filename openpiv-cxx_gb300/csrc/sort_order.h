// sort_order.h -- which element std::sort puts first, among equal keys.
//
// find_peaks (openpiv/core/detail/image_utils.impl.h:67-71) orders its
// candidates with std::sort and a "value greater than" comparator, then
// keeps the first two.  std::sort is not stable: when several candidates
// share the top value (planes of periodic or symmetric windows), which one
// ends up first depends on the sorting algorithm.  GCC's library (the
// toolchain of the reference build) implements std::sort as introsort
// (Musser, 1997) with these parameters:
//   * partition while a range holds more than 16 elements; the pivot is the
//     median of elements first+1, mid = first + n/2 and last-1, moved to
//     `first`; Hoare-style unguarded partition of [first+1, last) around it;
//     recurse on the right part, loop on the left part;
//   * depth limit 2*floor(log2 n); when it is exhausted the range is heap
//     sorted (make_heap + sort_heap, the classic sift-down/sift-up heap);
//   * finally insertion sort (stable).
// Every partition leaves the left part >= pivot >= the right part, so no
// element crosses a partition boundary later: the first positions of the
// sorted sequence are decided by the leftmost chain of partitions alone,
// then by heap sort or by the stable insertion sort of the first block.
// This routine replays exactly that chain, O(n) on average, and works in
// place on the caller's arrays.  It is host/device code; the exact kernel
// runs it single-threaded on the (rare) windows it re-decides, and a host
// test replays it against std::sort.
#pragma once

#ifdef __CUDACC__
#define OPIV_HD __host__ __device__
#else
#define OPIV_HD
#endif

namespace opiv {

struct peak_cand {
    double v;    // centre value
    int key;     // row-major scan index
};

OPIV_HD inline bool cand_before(const peak_cand& a, const peak_cand& b) { return a.v > b.v; }

OPIV_HD inline void cand_swap(peak_cand* a, peak_cand* b)
{
    const peak_cand t = *a;
    *a = *b;
    *b = t;
}

// Sift `value` down from `hole` in the heap c[0..len) (max element first
// under cand_before), then back up towards `top`.
OPIV_HD inline void heap_adjust(peak_cand* c, int hole, int len, peak_cand value)
{
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (cand_before(c[child], c[child - 1])) --child;
        c[hole] = c[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        c[hole] = c[child - 1];
        hole = child - 1;
    }
    int parent = (hole - 1) / 2;
    while (hole > top && cand_before(c[parent], value)) {
        c[hole] = c[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    c[hole] = value;
}

OPIV_HD inline void heap_sort(peak_cand* c, int len)
{
    if (len < 2) return;
    for (int parent = (len - 2) / 2;; --parent) {
        heap_adjust(c, parent, len, c[parent]);
        if (parent == 0) break;
    }
    for (int last = len - 1; last > 0; --last) {
        const peak_cand v = c[last];
        c[last] = c[0];
        heap_adjust(c, 0, last, v);
    }
}

// Stable insertion sort of c[0..len).
OPIV_HD inline void insertion_sort(peak_cand* c, int len)
{
    for (int i = 1; i < len; ++i) {
        const peak_cand v = c[i];
        if (cand_before(v, c[0])) {
            for (int j = i; j > 0; --j) c[j] = c[j - 1];
            c[0] = v;
        } else {
            int j = i;
            while (cand_before(v, c[j - 1])) {
                c[j] = c[j - 1];
                --j;
            }
            c[j] = v;
        }
    }
}

// Reorders c[0..n) so that its first k elements (k returned, 1 <= k <= 16
// for n >= 1) are the first k of std::sort(c, c + n, cand_before), in the
// same order; in particular c[0] is the element std::sort puts first.  The
// rest of c is left in an unspecified order.
OPIV_HD inline int sort_order_head(peak_cand* c, int n)
{
    if (n < 2) return n;
    int lg = 0;
    while ((2 << lg) <= n) ++lg;
    int depth = 2 * lg;
    int last = n;
    while (last > 16) {
        if (depth == 0) {
            heap_sort(c, last);
            return last < 16 ? last : 16;
        }
        --depth;
        // median of c[1], c[mid], c[last-1] moved to c[0]
        const int mid = last / 2;
        peak_cand *a = c + 1, *b = c + mid, *z = c + last - 1;
        if (cand_before(*a, *b)) {
            if (cand_before(*b, *z)) cand_swap(c, b);
            else if (cand_before(*a, *z)) cand_swap(c, z);
            else cand_swap(c, a);
        } else if (cand_before(*a, *z)) {
            cand_swap(c, a);
        } else if (cand_before(*b, *z)) {
            cand_swap(c, z);
        } else {
            cand_swap(c, b);
        }
        // unguarded partition of [1, last) around c[0]
        int lo = 1, hi = last;
        for (;;) {
            while (cand_before(c[lo], c[0])) ++lo;
            --hi;
            while (cand_before(c[0], c[hi])) --hi;
            if (!(lo < hi)) break;
            cand_swap(c + lo, c + hi);
            ++lo;
        }
        last = lo;   // keep the left part; the right part never comes back
    }
    insertion_sort(c, last);
    return last;
}

}  // namespace opiv
