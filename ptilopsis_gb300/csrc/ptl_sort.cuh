// Emulation of the order libstdc++'s std::sort leaves when it sorts iota(n) by depth --
// the reference's isn_gen sort, src/codegen/rv_generator_avx.cpp:539-541.  That order
// decides which of two same-depth nodes writes a shared instruction slot last, so the
// GPU must reproduce it exactly, not merely sort.
//
// std::sort is introsort (the published algorithm, Musser 1997, as libstdc++ writes
// it): while a range holds more than 16 elements, move the median of (first+1, mid,
// last-1) to first, partition [first+1, last) around it with the unguarded Hoare scan,
// and recurse; a range whose depth budget (2*floor(log2 n)) runs out is heap-sorted;
// a final insertion sort finishes the small ranges.
//
// The Hoare scan is sequential, but its result has a closed form that parallelises:
// call an element an L-stop when its key >= pivot and an R-stop when key <= pivot.  Let
// A[k] be the k-th L-stop from the left and B[k] the k-th R-stop from the right.  The
// scan swaps A[k] with B[k] exactly for k < K, where K counts the k with A[k] < B[k],
// and returns cut = A[0] when K == 0, else min(A[K], B[K-1]).  (An element equal to the
// pivot is both kinds of stop but is swapped at most once.)  The insertion sort is
// stable and never moves an element across a partition boundary, so it amounts to a
// stable sort of each final range of <= 16 elements.
#pragma once

#include "ptl_common.cuh"

namespace ptl {

struct SortSeg {
    uint32_t first, last;  // [first, last) in the array
    uint32_t dl;           // remaining depth budget
    int32_t pivot;         // pivot key after the median move
    uint32_t tbase, tcount;  // tiles of [first+1, last)
    uint32_t nL, nR;       // stop counts
    uint32_t K, cut;
    int32_t kmin, kmax;    // least and greatest key in [first, last)
};

constexpr uint32_t kSortThreshold = 16;   // libstdc++ _S_threshold
constexpr uint32_t kSortTile = 2048;      // elements per partition tile

PTL_HD int32_t skey(unsigned long long e) { return static_cast<int32_t>(static_cast<uint32_t>(e >> 32)); }
PTL_HD uint32_t sidx(unsigned long long e) { return static_cast<uint32_t>(e); }

PTL_HD uint32_t floor_log2(uint32_t n) {
    uint32_t r = 0;
    while (n > 1) { n >>= 1; ++r; }
    return r;
}

template <class Arr>
PTL_HD void sswap(Arr a, uint32_t i, uint32_t j) {
    const unsigned long long t = a[i];
    a[i] = a[j];
    a[j] = t;
}

// std::__move_median_to_first(result = first, a = first+1, b = mid, c = last-1)
template <class Arr>
PTL_HD void median_to_first(Arr a, uint32_t first, uint32_t last) {
    const uint32_t ia = first + 1, ib = first + (last - first) / 2, ic = last - 1;
    const int32_t ka = skey(a[ia]), kb = skey(a[ib]), kc = skey(a[ic]);
    uint32_t pick;
    if (ka < kb) {
        if (kb < kc) pick = ib;
        else if (ka < kc) pick = ic;
        else pick = ia;
    } else if (ka < kc) {
        pick = ia;
    } else if (kb < kc) {
        pick = ic;
    } else {
        pick = ib;
    }
    sswap(a, first, pick);
}

PTL_HD bool is_lstop(int32_t key, int32_t pivot) { return !(key < pivot); }
PTL_HD bool is_rstop(int32_t key, int32_t pivot) { return !(pivot < key); }

// K = #{k : A[k] < B[k]}; the predicate is true for a prefix of k.
PTL_HD uint32_t partition_k(const uint32_t* apos, const uint32_t* bpos, uint32_t nL, uint32_t nR) {
    uint32_t lo = 0, hi = nL < nR ? nL : nR;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (apos[mid] < bpos[mid]) lo = mid + 1; else hi = mid;
    }
    return lo;
}

PTL_HD uint32_t partition_cut(const uint32_t* apos, const uint32_t* bpos, uint32_t nL, uint32_t K) {
    if (K == 0) return apos[0];
    const uint32_t b = bpos[K - 1];
    if (K < nL && apos[K] < b) return apos[K];
    return b;
}

// libstdc++ __adjust_heap / __push_heap / make_heap / sort_heap on a[first, first+len).
template <class Arr>
PTL_HD void heap_push(Arr a, int64_t hole, int64_t top, unsigned long long v) {
    int64_t parent = (hole - 1) / 2;
    while (hole > top && skey(a[parent]) < skey(v)) {
        a[hole] = a[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[hole] = v;
}

template <class Arr>
PTL_HD void heap_adjust(Arr a, int64_t hole, int64_t len, unsigned long long v) {
    const int64_t top = hole;
    int64_t second = hole;
    while (second < (len - 1) / 2) {
        second = 2 * (second + 1);
        if (skey(a[second]) < skey(a[second - 1])) second--;
        a[hole] = a[second];
        hole = second;
    }
    if ((len & 1) == 0 && second == (len - 2) / 2) {
        second = 2 * (second + 1);
        a[hole] = a[second - 1];
        hole = second - 1;
    }
    heap_push(a, hole, top, v);
}

template <class Arr>
PTL_HD void heap_sort_range(Arr base, uint32_t len) {
    if (len < 2) return;
    const int64_t n = len;
    for (int64_t parent = (n - 2) / 2;; --parent) {
        heap_adjust(base, parent, n, base[parent]);
        if (parent == 0) break;
    }
    for (int64_t last = n; last > 1;) {
        --last;
        const unsigned long long v = base[last];
        base[last] = base[0];
        heap_adjust(base, 0, last, v);
    }
}

// ---- ranges of equal keys
// On a range whose keys are all equal every comparison is false, so introsort's steps
// depend on the range's length m alone: the median move swaps first with mid = m/2, the
// Hoare scan stops at every element and swaps positions 1+k and m-1-k for k < s =
// (m-1)/2, and the range splits at s+1; the final insertion sort moves nothing.  An
// element's final index follows by descending these splits, which replaces every round
// below such a range.

// Levels the descent takes: the larger part of a split holds ceil(m/2) keys.
PTL_HD uint32_t equal_levels(uint32_t m) {
    uint32_t l = 0;
    while (m > kSortThreshold) {
        m -= m / 2;
        ++l;
    }
    return l;
}

// Final index of the element at index i of an equal-key range of m elements, given a
// depth budget of at least equal_levels(m) (no heap sort on the way).
PTL_HD uint32_t equal_final_index(uint32_t i, uint32_t m) {
    uint32_t off = 0;
    while (m > kSortThreshold) {
        const uint32_t mid = m / 2, s = (m - 1u) / 2u;
        if (i == 0) i = mid;
        else if (i == mid) i = 0;
        if ((i >= 1u && i <= s) || i >= m - s) i = m - i;
        if (i <= s) {
            m = s + 1u;
        } else {
            i -= s + 1u;
            off += s + 1u;
            m -= s + 1u;
        }
    }
    return off + i;
}

// Stable insertion sort by key (what the final insertion sort does to one small range).
template <class Arr>
PTL_HD void leaf_sort(Arr a, uint32_t first, uint32_t last) {
    for (uint32_t i = first + 1; i < last; ++i) {
        const unsigned long long v = a[i];
        uint32_t j = i;
        while (j > first && skey(v) < skey(a[j - 1])) {
            a[j] = a[j - 1];
            --j;
        }
        a[j] = v;
    }
}

// ---- ranges that fit on chip
// Ranges of at most kSortBlock elements with depth budget left finish without further
// rounds (they touch only their own range): one block each on the device (k_sort_block,
// whose warps take the parts of at most kSortLocal elements), and local_introsort
// below, the same steps taken sequentially, in the host model.
constexpr uint32_t kSortBlock = 8192;
constexpr uint32_t kSortLocal = 256;

// An array view with a stride (element i at base[i * stride]).
struct Strided {
    unsigned long long* base;
    uint32_t stride;
    PTL_HD unsigned long long& operator[](int64_t i) const { return base[static_cast<uint64_t>(i) * stride]; }
    PTL_HD Strided operator+(uint32_t k) const { return Strided{base + static_cast<uint64_t>(k) * stride, stride}; }
};

// libstdc++ __unguarded_partition of [first+1, last) around the key at first; returns
// the cut.  The median move leaves an L-stop and an R-stop in range, so the scans stop
// inside it; the bounds only keep a broken invariant in range.
template <class Arr>
PTL_HD uint32_t seq_partition(Arr a, uint32_t first, uint32_t last) {
    const int32_t pivot = skey(a[first]);
    uint32_t lo = first + 1, hi = last;
    for (;;) {
        while (lo < last && skey(a[lo]) < pivot) ++lo;
        --hi;
        while (hi > first && pivot < skey(a[hi])) --hi;
        if (!(lo < hi)) return lo;
        sswap(a, lo, hi);
        ++lo;
    }
}

// The introsort loop on [first, last) with depth budget dl, leaves and heap-sorted
// ranges included (one thread).
template <class Arr>
PTL_HD void local_introsort(Arr a, uint32_t first, uint32_t last, uint32_t dl) {
    uint32_t st_f[64], st_l[64], st_d[64];  // at most one pending range per depth level
    int sp = 0;
    st_f[0] = first;
    st_l[0] = last;
    st_d[0] = dl;
    sp = 1;
    while (sp > 0) {
        --sp;
        uint32_t f = st_f[sp], l = st_l[sp], d = st_d[sp];
        for (;;) {
            const uint32_t len = l - f;
            if (len <= kSortThreshold) {
                if (len > 1) leaf_sort(a, f, l);
                break;
            }
            if (d == 0) {
                heap_sort_range(a + f, len);
                break;
            }
            median_to_first(a, f, l);
            const uint32_t cut = seq_partition(a, f, l);
            --d;
            if (sp < 64) {
                st_f[sp] = cut;
                st_l[sp] = l;
                st_d[sp] = d;
                ++sp;
            }
            l = cut;
        }
    }
}

}  // namespace ptl
