// Shared device-side definitions of the GB300 motif-extraction engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mtx
{

constexpr int kMaxPlanes = 5;        // PROT has 27 symbols -> 5 bit planes
constexpr int kDPThreads = 128;      // threads per DP CTA
constexpr int kSortThreads = 256;    // threads per radix-sort CTA
constexpr int kSortItems = 16;       // keys per thread per radix-sort tile
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kScanThreads = 1024;

/*
 * One text chunk of a DP launch, in units of 32-position blocks of the
 * concatenated text.  Blocks [warm, begin) are processed but not counted
 * (edit-distance restart warm-up, >= l+e-1 positions); [begin, end) are
 * counted.  first_split / last_split: index into the split-sequence flag
 * rows for the sequence that is active at `begin` having started before it,
 * resp. active at `end` and continuing past it; -1 when there is none.
 */
struct ChunkInfo
{
    uint32_t warm;
    uint32_t begin;
    uint32_t end;
    int32_t  first_split;
    int32_t  last_split;
};

/*
 * Packed scan text.  Plane b holds bit b of every symbol code, one bit per
 * position: word k+1 of plane b = positions 32k..32k+31 (bit r = position
 * 32k+r); word 0 of every plane is zero.  vmask bit = a match may end here
 * (the position belongs to a searchable sequence and, for Hamming, ends a
 * full window inside it); emask bit = last position of a sequence.
 */
struct TextView
{
    const uint32_t * planes;
    uint32_t         plane_stride;
    const uint32_t * vmask;
    const uint32_t * emask;
    uint32_t         nblk;
};

/*
 * Arguments of the factor-search DP.  The U searched factors are given as
 * bit planes (plane b of factor w at wplanes[b * wstride + w * nw64 ...]).
 */
struct DPArgs
{
    TextView          text;
    const uint32_t *  wplanes32;     // fast kernels: plane b of factor w at [b * U + w]
    const uint64_t *  wplanes64;     // generic kernel: [(b * U + w) * nw64 + q]
    uint32_t          U;
    uint32_t          l;
    uint32_t          e;
    // 1, 2 and -1 as kernel data: the edit-distance step multiplies by them
    // (x * one + y, x * two, x * neg1 + y) so that its adds and shifts issue
    // as multiply-adds on the FMA pipe; the compiler cannot fold them back
    uint32_t          one, two, neg1;
    const ChunkInfo * chunks;
    uint32_t *        u_acc;
    uint32_t *        v_acc;
    uint8_t *         split_flags;   // n_split rows of U bytes
};

__device__ __forceinline__ uint32_t lanemask_lt ()
{
    uint32_t m;
    asm ( "mov.u32 %0, %%lanemask_lt;" : "=r"( m ) );
    return m;
}

} // namespace mtx
