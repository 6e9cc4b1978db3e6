// introsort.h — restatement of the introsort that GCC's libstdc++ runs for std::sort
// (<bits/stl_algo.h>, unchanged in substance across GCC 9-14), for reproducing the order in which
// std::sort leaves elements that compare equivalent. Test infrastructure for the oracle: the
// reference's convexHull (polygonizer.cpp:51-59) sorts point indices with std::sort, and which of
// two points with the same (x, y) ends up on the hull depends on that order.
//
// The published algorithm (Musser 1997, as libstdc++ configures it):
//   - depth limit 2 * floor(log2 n); ranges of at most 16 elements are left to the final pass;
//   - pivot: median of (first + 1, middle, last - 1), swapped into `first`; Hoare-style unguarded
//     partition of [first + 1, last) around it; recurse on the right part, loop on the left;
//   - at the depth limit: heapsort of the range (make_heap, then pop one element at a time);
//   - final pass: insertion sort of the first 16 elements, unguarded insertion of the rest.
// Every comparison is made between the same elements in the same sequence as that implementation,
// so the result equals std::sort's for any comparator, including ones that are not strict weak
// orders. `less(a, b)` compares two element values.
//
// nth_element below restates libstdc++'s introselect (std::nth_element), which the reference's
// KDTree::rebuild (kdtree.hpp:186-188) calls once per tree node: the same pivot and partition
// steps, narrowed to the side holding the nth position until at most three elements remain
// (insertion sort), with depth limit 2 * floor(log2 n) after which a heap selection of the nth
// element takes over. Elements that compare equal to the nth one end up on either side in the
// order this sequence of swaps leaves them, which decides the tree's shape when coordinates tie.
#pragma once

#include <cstddef>
#include <utility>

namespace lpo_sort
{
template <class T, class Less>
void push_up(T* a, std::ptrdiff_t hole, std::ptrdiff_t top, T v, Less& less)
{
    std::ptrdiff_t parent = (hole - 1) / 2;
    while (hole > top && less(a[parent], v))
    {
        a[hole] = a[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[hole] = v;
}

// Sift the value v down from `hole` into a heap of len elements: the hole follows the larger child
// to the bottom, then v is pushed back up from there.
template <class T, class Less>
void sift(T* a, std::ptrdiff_t hole, std::ptrdiff_t len, T v, Less& less)
{
    const std::ptrdiff_t top = hole;
    std::ptrdiff_t child = hole;
    while (child < (len - 1) / 2)
    {
        child = 2 * (child + 1);
        if (less(a[child], a[child - 1]))
            --child;
        a[hole] = a[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2)
    {
        child = 2 * (child + 1);
        a[hole] = a[child - 1];
        hole = child - 1;
    }
    push_up(a, hole, top, v, less);
}

template <class T, class Less>
void heap_sort(T* a, std::ptrdiff_t len, Less& less)
{
    if (len < 2)
        return;
    for (std::ptrdiff_t parent = (len - 2) / 2;; --parent)
    {
        sift(a, parent, len, a[parent], less);
        if (parent == 0)
            break;
    }
    for (std::ptrdiff_t last = len - 1; last > 0; --last)
    {
        const T v = a[last];
        a[last] = a[0];
        sift(a, 0, last, v, less);
    }
}

// Pivot selection: the median of a[1], a[mid], a[len - 1] is swapped into a[0].
template <class T, class Less>
void median_to_front(T* a, std::ptrdiff_t len, Less& less)
{
    T* r = a;
    T* x = a + 1;
    T* y = a + len / 2;
    T* z = a + len - 1;
    T* m;
    if (less(*x, *y))
        m = less(*y, *z) ? y : (less(*x, *z) ? z : x);
    else
        m = less(*x, *z) ? x : (less(*y, *z) ? z : y);
    std::swap(*r, *m);
}

// Partition of [1, len) around a[0] without bounds checks (the pivot and the median's other
// candidates stop both scans); returns the start of the right part.
template <class T, class Less>
std::ptrdiff_t partition(T* a, std::ptrdiff_t len, Less& less)
{
    std::ptrdiff_t lo = 1, hi = len;
    for (;;)
    {
        while (less(a[lo], a[0]))
            ++lo;
        --hi;
        while (less(a[0], a[hi]))
            --hi;
        if (!(lo < hi))
            return lo;
        std::swap(a[lo], a[hi]);
        ++lo;
    }
}

template <class T, class Less>
void introsort_loop(T* a, std::ptrdiff_t len, int depth, Less& less)
{
    while (len > 16)
    {
        if (depth == 0)
        {
            heap_sort(a, len, less);
            return;
        }
        --depth;
        median_to_front(a, len, less);
        const std::ptrdiff_t cut = partition(a, len, less);
        introsort_loop(a + cut, len - cut, depth, less);
        len = cut;
    }
}

// a[i] moves left while it is less than its left neighbour; nothing stops it at the front, so the
// caller guarantees a smaller-or-equal element to its left.
template <class T, class Less>
void insert_unguarded(T* a, std::ptrdiff_t i, Less& less)
{
    const T v = a[i];
    while (less(v, a[i - 1]))
    {
        a[i] = a[i - 1];
        --i;
    }
    a[i] = v;
}

template <class T, class Less>
void insertion_sort(T* a, std::ptrdiff_t len, Less& less)
{
    for (std::ptrdiff_t i = 1; i < len; ++i)
    {
        if (less(a[i], a[0]))
        {
            const T v = a[i];
            for (std::ptrdiff_t j = i; j > 0; --j)
                a[j] = a[j - 1];
            a[0] = v;
        }
        else
            insert_unguarded(a, i, less);
    }
}

// Heap selection (the introselect's fallback at the depth limit): a max-heap of the first `mid`
// elements, then every later element smaller than the heap's top replaces it.
template <class T, class Less>
void heap_select(T* a, std::ptrdiff_t mid, std::ptrdiff_t len, Less& less)
{
    if (mid >= 2)
        for (std::ptrdiff_t parent = (mid - 2) / 2;; --parent)
        {
            sift(a, parent, mid, a[parent], less);
            if (parent == 0)
                break;
        }
    for (std::ptrdiff_t i = mid; i < len; ++i)
        if (less(a[i], a[0]))
        {
            const T v = a[i];
            a[i] = a[0];
            sift(a, 0, mid, v, less);
        }
}

inline int floor_log2(std::size_t n);

// std::nth_element(a, a + nth, a + n, less) as libstdc++ performs it.
template <class T, class Less>
void nth_element(T* a, std::size_t n, std::size_t nth, Less less, int depth_override = -1)
{
    if (n == 0 || nth >= n)
        return;
    std::ptrdiff_t first = 0, last = static_cast<std::ptrdiff_t>(n);
    const std::ptrdiff_t k = static_cast<std::ptrdiff_t>(nth);
    int depth = depth_override >= 0 ? depth_override : 2 * floor_log2(n);
    while (last - first > 3)
    {
        if (depth == 0)
        {
            heap_select(a + first, k - first + 1, last - first, less);
            std::swap(a[first], a[k]);
            return;
        }
        --depth;
        median_to_front(a + first, last - first, less);
        const std::ptrdiff_t cut = first + partition(a + first, last - first, less);
        if (cut <= k)
            first = cut;
        else
            last = cut;
    }
    insertion_sort(a + first, last - first, less);
}

inline int floor_log2(std::size_t n)
{
    int k = -1;
    while (n)
    {
        n >>= 1;
        ++k;
    }
    return k;
}

// std::sort(a, a + n, less) as libstdc++ performs it. depth_override >= 0 replaces the depth limit
// (0 takes the heapsort path at once; used to test that path).
template <class T, class Less>
void sort(T* a, std::size_t n, Less less, int depth_override = -1)
{
    if (n == 0)
        return;
    const std::ptrdiff_t len = static_cast<std::ptrdiff_t>(n);
    introsort_loop(a, len, depth_override >= 0 ? depth_override : 2 * floor_log2(n), less);
    if (len > 16)
    {
        insertion_sort(a, 16, less);
        for (std::ptrdiff_t i = 16; i < len; ++i)
            insert_unguarded(a, i, less);
    }
    else
        insertion_sort(a, len, less);
}
} // namespace lpo_sort
