// Bit-exact replicas of the two sorts the reference applies to occurrence lists
// (src/cpu/sort.h:43-57 and 97-109): an insertion sort for lists of at most 20
// entries, and libstdc++'s std::sort above that.
//
// std::sort is GCC libstdc++ (the reference is built with g++; GCC 13 here). Its
// published algorithm is introsort: a quicksort loop with median-of-three pivot
// moved to the front and an unguarded Hoare partition, switching to heapsort
// after 2*floor(log2(n)) levels, stopping at ranges of 16 and finishing with one
// insertion-sort pass (first 16 guarded, the rest unguarded). With keys that
// compare equal, the final order depends on every one of those steps, so they are
// restated exactly; tests check the replica against std::sort permutation by
// permutation.
//
// Both functions work on any random-access array of T with a strict-weak-order
// comparator cmp(a, b) and are usable from host and device code.
#pragma once

#include "device.cuh"

namespace sigma {

template <class T>
HD void swap_t(T& a, T& b) { T t = a; a = b; b = t; }

struct LitLess {
    HD bool operator()(u32 a, u32 b) const { return a < b; }
};

// Reference insertionSort (src/cpu/sort.h:43-57).
template <class T, class Cmp>
HD void ref_insertion_sort(T* d, int sz, Cmp cmp) {
    if (sz == 2 && cmp(d[1], d[0])) swap_t(d[1], d[0]);
    else if (sz > 2) {
        for (int i = 1; i < sz; i++) {
            T tmp = d[i];
            int j = i;
            for (; j > 0 && cmp(tmp, d[j - 1]); j--) d[j] = d[j - 1];
            d[j] = tmp;
        }
    }
}

namespace stdsort {

constexpr int kThreshold = 16;

HD int lg(int n) {
    int r = 0;
    while (n > 1) { n >>= 1; r++; }
    return r;
}

template <class T, class Cmp>
HD void move_median_to_first(T* result, T* a, T* b, T* c, Cmp& cmp) {
    if (cmp(*a, *b)) {
        if (cmp(*b, *c)) swap_t(*result, *b);
        else if (cmp(*a, *c)) swap_t(*result, *c);
        else swap_t(*result, *a);
    } else if (cmp(*a, *c)) swap_t(*result, *a);
    else if (cmp(*b, *c)) swap_t(*result, *c);
    else swap_t(*result, *b);
}

template <class T, class Cmp>
HD T* unguarded_partition(T* first, T* last, T* pivot, Cmp& cmp) {
    while (true) {
        while (cmp(*first, *pivot)) ++first;
        --last;
        while (cmp(*pivot, *last)) --last;
        if (!(first < last)) return first;
        swap_t(*first, *last);
        ++first;
    }
}

template <class T, class Cmp>
HD void push_heap(T* first, int hole, int top, T value, Cmp& cmp) {
    int parent = (hole - 1) / 2;
    while (hole > top && cmp(first[parent], value)) {
        first[hole] = first[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    first[hole] = value;
}

template <class T, class Cmp>
HD void adjust_heap(T* first, int hole, int len, T value, Cmp& cmp) {
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (cmp(first[child], first[child - 1])) child--;
        first[hole] = first[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        first[hole] = first[child - 1];
        hole = child - 1;
    }
    push_heap(first, hole, top, value, cmp);
}

template <class T, class Cmp>
HD void heap_sort(T* first, T* last, Cmp& cmp) {
    const int len = (int)(last - first);
    if (len >= 2) {  // make_heap
        int parent = (len - 2) / 2;
        while (true) {
            T v = first[parent];
            adjust_heap(first, parent, len, v, cmp);
            if (parent == 0) break;
            parent--;
        }
    }
    while (last - first > 1) {  // sort_heap via pop_heap
        --last;
        T v = *last;
        *last = *first;
        adjust_heap(first, 0, (int)(last - first), v, cmp);
    }
}

template <class T, class Cmp>
HD void unguarded_linear_insert(T* last, Cmp& cmp) {
    T val = *last;
    T* next = last - 1;
    while (cmp(val, *next)) {
        *last = *next;
        last = next;
        --next;
    }
    *last = val;
}

template <class T, class Cmp>
HD void insertion_sort(T* first, T* last, Cmp& cmp) {
    if (first == last) return;
    for (T* i = first + 1; i != last; ++i) {
        if (cmp(*i, *first)) {
            T val = *i;
            for (T* k = i; k != first; --k) *k = *(k - 1);
            *first = val;
        } else {
            unguarded_linear_insert(i, cmp);
        }
    }
}

}  // namespace stdsort

// libstdc++ std::sort(first, last, cmp). The quicksort recursion (which sorts the
// right part first, then loops on the left) touches disjoint ranges, so an explicit
// stack gives the identical result.
template <class T, class Cmp>
HD void std_sort_replica(T* first, T* last, Cmp cmp) {
    using namespace stdsort;
    const int n = (int)(last - first);
    if (n <= 1) return;
    struct Range { T* f; T* l; int depth; };
    Range stack[64];
    int sp = 0;
    stack[sp++] = Range{first, last, 2 * lg(n)};
    while (sp) {
        Range r = stack[--sp];
        T* f = r.f;
        T* l = r.l;
        int depth = r.depth;
        while (l - f > kThreshold) {
            if (depth == 0) {
                heap_sort(f, l, cmp);
                break;
            }
            --depth;
            T* mid = f + (l - f) / 2;
            move_median_to_first(f, f + 1, mid, l - 1, cmp);
            T* cut = unguarded_partition(f + 1, l, f, cmp);
            stack[sp++] = Range{cut, l, depth};
            l = cut;
        }
    }
    if (n > kThreshold) {
        insertion_sort(first, first + kThreshold, cmp);
        for (T* i = first + kThreshold; i != last; ++i) unguarded_linear_insert(i, cmp);
    } else {
        insertion_sort(first, last, cmp);
    }
}

// Sort(Vec, CMP) of the reference (src/cpu/sort.h:97-109).
template <class T, class Cmp>
HD void reference_list_sort(T* d, int n, Cmp cmp) {
    if (n <= 0) return;
    if (n <= 20) ref_insertion_sort(d, n, cmp);
    else std_sort_replica(d, d + n, cmp);
}

}  // namespace sigma
