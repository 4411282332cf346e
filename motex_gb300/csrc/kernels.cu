// Packing, factor deduplication (stable LSD radix sort), filter and
// compaction kernels of the GB300 motif-extraction engine.
#include "kernels.cuh"

namespace mtx
{

// ------------------------------------------------------------------ scans

// Exclusive scan of one value per thread across a CTA of kScanThreads.
__device__ __forceinline__ uint32_t block_exclusive_scan ( uint32_t v, uint32_t * total )
{
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for ( int o = 1; o < 32; o <<= 1 )
    {
        uint32_t y = __shfl_up_sync ( 0xffffffffu, x, o );
        if ( lane >= o ) x += y;
    }
    if ( lane == 31 ) warp_sums[warp] = x;
    __syncthreads ();
    if ( warp == 0 )
    {
        const int nw = blockDim.x >> 5;
        uint32_t s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            uint32_t y = __shfl_up_sync ( 0xffffffffu, s, o );
            if ( lane >= o ) s += y;
        }
        warp_sums[lane] = s;           // inclusive warp-sum prefix
    }
    __syncthreads ();
    const uint32_t before = warp ? warp_sums[warp - 1] : 0u;
    if ( total ) *total = warp_sums[( blockDim.x >> 5 ) - 1];
    __syncthreads ();
    return before + x - v;
}

// In-place exclusive scan of n words with a single CTA; *total = sum.
__global__ void __launch_bounds__ ( kScanThreads ) k_scan_single ( uint32_t * data, uint32_t n, uint32_t * total )
{
    const uint32_t seg = ( n + kScanThreads - 1 ) / kScanThreads;
    const uint32_t s0 = min ( n, threadIdx.x * seg ), s1 = min ( n, s0 + seg );
    uint32_t sum = 0;
    for ( uint32_t i = s0; i < s1; ++i ) sum += data[i];
    uint32_t tot;
    uint32_t run = block_exclusive_scan ( sum, &tot );
    for ( uint32_t i = s0; i < s1; ++i )
    {
        uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
    if ( threadIdx.x == 0 && total ) *total = tot;
}

template <typename T>
__global__ void __launch_bounds__ ( kScanThreads ) k_tile_reduce ( const T * in, uint32_t n, uint32_t * tile_sums )
{
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t s = 0;
#pragma unroll
    for ( int r = 0; r < kScanItems; ++r )
    {
        uint32_t i = base + r * kScanThreads + threadIdx.x;
        if ( i < n ) s += ( uint32_t ) in[i];
    }
    uint32_t tot;
    block_exclusive_scan ( s, &tot );
    if ( threadIdx.x == 0 ) tile_sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void __launch_bounds__ ( kScanThreads ) k_tile_scan ( const T * in, uint32_t n, const uint32_t * tile_off,
                                                                  uint32_t * out )
{
    // thread t owns kScanItems consecutive items so the output order is preserved
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for ( int r = 0; r < kScanItems; ++r )
    {
        uint32_t i = base + r;
        v[r] = i < n ? ( uint32_t ) in[i] : 0u;
        s += v[r];
    }
    uint32_t run = tile_off[blockIdx.x] + block_exclusive_scan ( s, nullptr );
#pragma unroll
    for ( int r = 0; r < kScanItems; ++r )
    {
        uint32_t i = base + r;
        if ( i < n ) out[i] = run;
        run += v[r];
    }
}

template <typename T>
static cudaError_t scan_exclusive_impl ( const T * in, uint32_t n, uint32_t * out, uint32_t * d_total,
                                         uint32_t * tile_sums, cudaStream_t st )
{
    const uint32_t tiles = ( n + kScanTile - 1 ) / kScanTile;
    k_tile_reduce<T><<<tiles ? tiles : 1, kScanThreads, 0, st>>> ( in, n, tile_sums );
    k_scan_single<<<1, kScanThreads, 0, st>>> ( tile_sums, tiles ? tiles : 1, d_total );
    k_tile_scan<T><<<tiles ? tiles : 1, kScanThreads, 0, st>>> ( in, n, tile_sums, out );
    return cudaGetLastError ();
}

// Byte flags: a thread owns 16 consecutive bytes, read as one 16-byte load
// (in is an allocation base), and writes their 16 prefix words as four
// 16-byte stores; a tile is 16 times the thread count.
constexpr int kScanItemsU8 = 16;
constexpr uint32_t kScanTileU8 = kScanThreads * kScanItemsU8;

__device__ __forceinline__ uint4 load16_u8 ( const uint8_t * __restrict__ in, uint32_t n, uint32_t base )
{
    if ( base + 16 <= n ) return *reinterpret_cast<const uint4 *> ( in + base );
    uint32_t w[4] = { 0, 0, 0, 0 };
    for ( uint32_t k = 0; base + k < n; ++k ) w[k >> 2] |= ( uint32_t ) in[base + k] << ( 8 * ( k & 3 ) );
    return make_uint4 ( w[0], w[1], w[2], w[3] );
}

__device__ __forceinline__ uint32_t byte_sum ( const uint4 & q )
{
    return __dp4a ( q.x, 0x01010101u, 0u ) + __dp4a ( q.y, 0x01010101u, 0u ) + __dp4a ( q.z, 0x01010101u, 0u ) +
           __dp4a ( q.w, 0x01010101u, 0u );
}

__global__ void __launch_bounds__ ( kScanThreads ) k_tile_reduce_u8 ( const uint8_t * __restrict__ in, uint32_t n,
                                                                      uint32_t * tile_sums )
{
    const uint32_t base = blockIdx.x * kScanTileU8 + threadIdx.x * kScanItemsU8;
    const uint32_t s = base < n ? byte_sum ( load16_u8 ( in, n, base ) ) : 0u;
    uint32_t tot;
    block_exclusive_scan ( s, &tot );
    if ( threadIdx.x == 0 ) tile_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__ ( kScanThreads ) k_tile_scan_u8 ( const uint8_t * __restrict__ in, uint32_t n,
                                                                    const uint32_t * tile_off, uint32_t * out )
{
    const uint32_t base = blockIdx.x * kScanTileU8 + threadIdx.x * kScanItemsU8;
    const uint4 q = base < n ? load16_u8 ( in, n, base ) : make_uint4 ( 0, 0, 0, 0 );
    uint32_t run = tile_off[blockIdx.x] + block_exclusive_scan ( byte_sum ( q ), nullptr );
    const uint32_t w[4] = { q.x, q.y, q.z, q.w };
    uint32_t o[16];
#pragma unroll
    for ( int r = 0; r < 16; ++r )
    {
        o[r] = run;
        run += ( w[r >> 2] >> ( 8 * ( r & 3 ) ) ) & 255u;
    }
    if ( base + 16 <= n )
    {
        uint4 * dst = reinterpret_cast<uint4 *> ( out + base );
#pragma unroll
        for ( int r = 0; r < 4; ++r ) dst[r] = make_uint4 ( o[4 * r], o[4 * r + 1], o[4 * r + 2], o[4 * r + 3] );
    }
    else
    {
#pragma unroll
        for ( int r = 0; r < 16; ++r )
            if ( base + r < n ) out[base + r] = o[r];
    }
}

// tile_sums holds at least ceil(n / kScanTileU8) words (ceil(n / kScanTile) is more)
cudaError_t scan_exclusive_u8 ( const uint8_t * in, uint32_t n, uint32_t * out, uint32_t * d_total,
                                uint32_t * tile_sums, cudaStream_t st )
{
    const uint32_t tiles = ( n + kScanTileU8 - 1 ) / kScanTileU8;
    k_tile_reduce_u8<<<tiles ? tiles : 1, kScanThreads, 0, st>>> ( in, n, tile_sums );
    k_scan_single<<<1, kScanThreads, 0, st>>> ( tile_sums, tiles ? tiles : 1, d_total );
    k_tile_scan_u8<<<tiles ? tiles : 1, kScanThreads, 0, st>>> ( in, n, tile_sums, out );
    return cudaGetLastError ();
}

cudaError_t scan_exclusive_u32 ( const uint32_t * in, uint32_t n, uint32_t * out, uint32_t * d_total,
                                 uint32_t * tile_sums, cudaStream_t st )
{
    return scan_exclusive_impl<uint32_t> ( in, n, out, d_total, tile_sums, st );
}

// ------------------------------------------------------------------ packing

// present[c] = 1 for every byte value c occurring in raw[0..total).
__global__ void k_presence ( const uint8_t * __restrict__ raw, uint64_t total, uint32_t * present )
{
    __shared__ uint32_t seen[256];
    for ( int i = threadIdx.x; i < 256; i += blockDim.x ) seen[i] = 0;
    __syncthreads ();
    const uint64_t stride = ( uint64_t ) gridDim.x * blockDim.x * 16;
    for ( uint64_t p = ( ( uint64_t ) blockIdx.x * blockDim.x + threadIdx.x ) * 16; p < total; p += stride )
    {
        if ( p + 16 <= total && ( ( ( uintptr_t ) ( raw + p ) ) & 15 ) == 0 )
        {
            uint4 q = *reinterpret_cast<const uint4 *> ( raw + p );
            uint32_t w[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
            for ( int j = 0; j < 4; ++j )
#pragma unroll
                for ( int b = 0; b < 4; ++b ) seen[( w[j] >> ( 8 * b ) ) & 255] = 1;
        }
        else
            for ( uint64_t i = p; i < min ( total, p + 16 ); ++i ) seen[raw[i]] = 1;
    }
    __syncthreads ();
    for ( int i = threadIdx.x; i < 256; i += blockDim.x )
        if ( seen[i] ) present[i] = 1;
}

// ------------------------------------------------------------ TMA staging

namespace
{

// try_wait polls before the drain of a failed CTA gives up.  A bulk copy of
// one tile from valid global memory lands within microseconds; each poll
// suspends the thread for at most the hardware's try_wait window.
constexpr uint32_t kDrainWaitPolls = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32 ( const void * p ) { return ( uint32_t ) __cvta_generic_to_shared ( p ); }

__device__ __forceinline__ void mbar_init ( uint64_t * bar, uint32_t count )
{
    asm volatile ( "mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"( smem_u32 ( bar ) ), "r"( count ) : "memory" );
}

__device__ __forceinline__ void mbar_expect_tx ( uint64_t * bar, uint32_t bytes )
{
    asm volatile ( "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"( smem_u32 ( bar ) ), "r"( bytes )
                   : "memory" );
}

__device__ __forceinline__ bool mbar_try_wait ( uint64_t * bar, uint32_t parity )
{
    uint32_t done;
    asm volatile ( "{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"( done )
                   : "r"( smem_u32 ( bar ) ), "r"( parity )
                   : "memory" );
    return done != 0;
}

// Wait of at most `polls` polls for the completion of phase `parity`;
// false if it gave up (at once for polls = 0).
__device__ __forceinline__ bool mbar_wait_bounded ( uint64_t * bar, uint32_t parity, uint32_t polls )
{
    for ( uint32_t it = 0; it < polls; ++it )
        if ( mbar_try_wait ( bar, parity ) ) return true;
    return false;
}

// One-dimensional TMA copy global -> shared, completing on `bar`.  Both
// addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s ( void * dst, const void * src, uint32_t bytes, uint64_t * bar )
{
    asm volatile ( "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_u32 ( dst ) ),
                   "l"( src ), "r"( bytes ), "r"( smem_u32 ( bar ) )
                   : "memory" );
}

} // namespace

/*
 * Packing.  A persistent grid walks tiles of kPackTile raw bytes; each tile
 * is staged into shared memory by one TMA bulk copy (double-buffered: the
 * copy of the CTA's next tile runs while this one is packed).  Warp w of
 * the CTA packs the tile's 32-position blocks 32w .. 32w+31, lane r block
 * 32w+r, its 32 positions in order: the lane reads its 32-byte row of the
 * staged tile, and its codes, bit planes, validity and end masks (and with
 * a.key0 set the first radix-sort key of every factor, a shift-or over the
 * codes) accumulate in registers, so the sort starts without a gather pass.
 * Codes, planes and masks leave as one store per lane and row (the rows of
 * a warp's lanes are consecutive).  Factor ends are written block by block
 * afterwards, lane L the factor ending at position L (the block's first
 * sequence comes from the lane that packed it), so each store covers 32
 * consecutive factors; the keys reach those lanes through a per-warp shared
 * buffer.
 *
 * Failure path: a staging wait that gives up (a.wait_polls polls) sets bit 0
 * of *a.err.  The CTA then issues no further copy and packs the rest of its
 * tiles from global memory with plain loads, so every output row is written
 * and later stages read well-formed data; the host reports the run as a
 * timed-out device wait.  Before the CTA exits it waits (kDrainWaitPolls,
 * bit 1 of *a.err if that gives up too) for the copies it had in flight, so
 * none lands in shared memory the CTA no longer owns.
 */
__global__ void __launch_bounds__ ( kPackThreads, kPackCtasPerSm ) k_pack ( PackArgs a )
{
    __shared__ __align__ ( 128 ) uint8_t stage[2][kPackTile];
    __shared__ __align__ ( 8 ) uint64_t bar[2];
    __shared__ uint8_t cmap[256];
    extern __shared__ uint32_t s_key[];             // kPackKeyWords per warp, with a.key0 only
    for ( int i = threadIdx.x; i < 256; i += blockDim.x ) cmap[i] = a.cmap[i];
    const uint64_t ntiles = ( a.total + kPackTile - 1 ) / kPackTile;
    if ( threadIdx.x == 0 )
    {
        mbar_init ( &bar[0], 1 );
        mbar_init ( &bar[1], 1 );
        asm volatile ( "fence.mbarrier_init.release.cluster;" ::: "memory" );
    }
    __syncthreads ();

    auto issue = [&] ( uint64_t t, int buf ) {       // thread 0 only
        const uint64_t start = t * kPackTile;
        const uint64_t left = ( a.total - start + 15 ) & ~15ull;
        const uint32_t bytes = left < kPackTile ? ( uint32_t ) left : kPackTile;
        mbar_expect_tx ( &bar[buf], bytes );
        bulk_copy_g2s ( stage[buf], a.raw + start, bytes, &bar[buf] );
    };
    // tile n of this CTA (n = 0, 1, ...) goes to buffer n & 1 and completes that
    // buffer's barrier phase n >> 1
    if ( blockIdx.x < ntiles && threadIdx.x == 0 ) issue ( blockIdx.x, 0 );
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t full = 0xffffffffu;
    bool failed = false, fail_next_issued = false;
    uint32_t n = 0, n_fail = 0;
    for ( uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++n )
    {
        const int buf = n & 1;
        if ( ! failed )
        {
            const uint64_t tn = t + gridDim.x;
            const bool next_issued = tn < ntiles;
            if ( next_issued && threadIdx.x == 0 )
            {
                // the other buffer was last read before the barrier that ended the previous tile
                asm volatile ( "fence.proxy.async.shared::cta;" ::: "memory" );
                issue ( tn, buf ^ 1 );
            }
            const bool ok = mbar_wait_bounded ( &bar[buf], ( n >> 1 ) & 1, a.wait_polls );
            if ( __syncthreads_or ( ! ok ) )
            {
                failed = true;
                n_fail = n;
                fail_next_issued = next_issued;
            }
        }

        // 32-bit positions: inputs are below 2^32 symbols (the host refuses more).
        // Lane r packs block k = k0 + r, its 32 positions in order: plane,
        // mask and key bits accumulate in the lane's registers (no ballot, no
        // shuffle per position), and every row leaves as one coalesced store.
        const uint32_t total = ( uint32_t ) a.total;
        const uint32_t k0 = ( uint32_t ) t * ( kPackTile / 32 ) + ( uint32_t ) warp * 32;     // first block of this warp
        const uint32_t k = k0 + lane;
        const uint32_t p0 = k * 32;
        const int B = a.B;
        // phase 1, in two halves of 16 positions (one 16-byte shared load of the
        // staged row each, or byte loads from global memory after a failed
        // wait): codes packed four per word and the planes
        uint32_t cw[8], pl[kMaxPlanes] = {};
#pragma unroll
        for ( int h = 0; h < 2; ++h )
        {
            uint32_t rw[4];
            if ( ! failed )
            {
                const uint4 q = reinterpret_cast<const uint4 *> ( stage[buf] + ( size_t ) warp * 1024 + lane * 32 )[h];
                rw[0] = q.x; rw[1] = q.y; rw[2] = q.z; rw[3] = q.w;
            }
            else
            {
#pragma unroll
                for ( int q = 0; q < 4; ++q ) rw[q] = 0;
#pragma unroll
                for ( int j = 0; j < 16; ++j )
                    if ( p0 + 16 * h + j < total ) rw[j >> 2] |= ( uint32_t ) a.raw[p0 + 16 * h + j] << ( 8 * ( j & 3 ) );
            }
#pragma unroll
            for ( int j = 0; j < 16; ++j )
            {
                const int jj = 16 * h + j;
                const uint32_t c = p0 + jj < total ? cmap[( rw[j >> 2] >> ( 8 * ( j & 3 ) ) ) & 255u] : 0u;
                if ( ( jj & 3 ) == 0 ) cw[jj >> 2] = c;
                else cw[jj >> 2] |= c << ( 8 * ( jj & 3 ) );
#pragma unroll
                for ( int b = 0; b < kMaxPlanes; ++b ) pl[b] |= ( ( c >> b ) & 1u ) << jj;
            }
        }
        if ( p0 < total )
        {
            uint4 * dst = reinterpret_cast<uint4 *> ( a.codes + p0 );          // codes hold total + 64 bytes
            dst[0] = make_uint4 ( cw[0], cw[1], cw[2], cw[3] );
            dst[1] = make_uint4 ( cw[4], cw[5], cw[6], cw[7] );
        }
        // the first sort key of each factor: its last kwin codes, B bits each,
        // the last lowest (32 bits kept); the key before the block comes from
        // the previous lane's block, or for lane 0 from the raw bytes
        const bool want_keys = a.key0 != nullptr;
        const uint32_t kwin = a.kwin;
        const uint32_t kmask = kwin * ( uint32_t ) B >= 32 ? 0xffffffffu : ( 1u << ( kwin * B ) ) - 1u;
        uint32_t key = 0;
        if ( want_keys )
        {
            uint32_t last = 0;                                   // key at the block's last position
#pragma unroll
            for ( int j = 0; j < 32; ++j )
                if ( j >= 32 - ( int ) kwin ) last = ( last << B ) | ( ( cw[j >> 2] >> ( 8 * ( j & 3 ) ) ) & 255u );
            key = __shfl_up_sync ( full, last & kmask, 1 );
            if ( lane == 0 )
            {
                key = 0;
                for ( uint32_t e = kwin - 1; e >= 1; --e )
                    if ( p0 >= e ) key = ( key << B ) | cmap[a.raw[p0 - e]];
            }
        }
        // phase 2: sequences, masks and keys of the lane's block in order; the
        // keys go to the warp's shared buffer (row per block, 33 words: conflict-free)
        uint32_t vm = 0, em = 0;
        uint32_t s = 0, start = 0, end = 0, ws = 0;
        if ( p0 < total )
        {
            // sequence of the block's first position: offs[s] <= p0 < offs[s + 1]
            uint32_t lo = 0, hi = a.nseq;
            while ( hi - lo > 1 )
            {
                const uint32_t mid = ( lo + hi ) >> 1;
                if ( a.offs[mid] <= p0 ) lo = mid; else hi = mid;
            }
            s = lo;
            start = a.offs[s];
            end = a.offs[s + 1];
            ws = a.wstart[s];
        }
        const uint32_t s0 = s, start0 = start, end0 = end, ws0 = ws;
        uint32_t * skey = s_key + warp * kPackKeyWords;
#pragma unroll
        for ( int j = 0; j < 32; ++j )
        {
            const uint32_t pos = p0 + j;
            const uint32_t c = ( cw[j >> 2] >> ( 8 * ( j & 3 ) ) ) & 255u;
            key = ( ( key << B ) | c ) & kmask;
            if ( want_keys ) skey[lane * 33 + j] = key;
            if ( pos < total )
            {
                while ( end <= pos )
                {
                    ++s;
                    start = end;
                    end = a.offs[s + 1];
                }
                const uint32_t rel = pos - start;
                const bool is_short = ( end - start ) < a.tml;
                // pattern mode: sequences below npat are patterns (factors
                // only), the rest are texts (searched only)
                vm |= ( uint32_t ) ( ! is_short && rel >= a.vstart && s >= a.npat ) << j;
                em |= ( uint32_t ) ( pos == end - 1 ) << j;
            }
        }
        __syncwarp ();
        // phase 3: factor ends and keys, block by block: lane L writes the
        // factor ending at position L of block k0 + i, so each store covers a
        // run of 32 consecutive factors; the block's first sequence comes from
        // the lane that packed it
#pragma unroll 4
        for ( int i = 0; i < 32; ++i )
        {
            const uint32_t pos = ( k0 + i ) * 32 + lane;
            uint32_t si = __shfl_sync ( full, s0, i ), st = __shfl_sync ( full, start0, i );
            uint32_t en = __shfl_sync ( full, end0, i ), w = __shfl_sync ( full, ws0, i );
            if ( pos < total )
            {
                while ( en <= pos )
                {
                    ++si;
                    st = en;
                    en = a.offs[si + 1];
                    w = a.wstart[si];
                }
                const uint32_t rel = pos - st;
                if ( ( en - st ) >= a.tml && rel + 1 >= a.l && ( a.npat == 0 || si < a.npat ) )
                {
                    const uint32_t idx = w + rel + 1 - a.l;
                    a.wpos[idx] = pos;
                    if ( want_keys ) a.key0[idx] = skey[i * 33 + lane];
                }
            }
        }
        __syncwarp ();
        if ( k < a.nblk )
        {
#pragma unroll
            for ( int b = 0; b < kMaxPlanes; ++b )
                if ( b < B ) a.planes[( size_t ) b * a.plane_stride + k + 1] = pl[b];
            a.vmask[k] = vm;
            a.emask[k] = em;
        }
        __syncthreads ();                            // this buffer may be refilled
    }
    if ( failed )
    {
        // let copies still in flight land before the CTA's shared memory goes away
        bool drained = mbar_wait_bounded ( &bar[n_fail & 1], ( n_fail >> 1 ) & 1, kDrainWaitPolls );
        if ( fail_next_issued )
            drained &= mbar_wait_bounded ( &bar[( n_fail + 1 ) & 1], ( ( n_fail + 1 ) >> 1 ) & 1, kDrainWaitPolls );
        if ( threadIdx.x == 0 ) atomicOr ( a.err, drained ? 1u : 3u );
    }
}

// ------------------------------------------------------------------ dedup

// key_out[i] = bits [lo, lo+32) of the packed factor ending at idx[i]
// (first symbol most significant, B bits per symbol).
__global__ void k_gather_key ( const uint32_t * __restrict__ idx, uint32_t n, const uint8_t * __restrict__ codes,
                               uint32_t l, uint32_t B, uint32_t lo, uint32_t * __restrict__ key_out )
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= n ) return;
    const uint32_t p = idx[i];
    const uint32_t e0 = lo / B, e1 = min ( l - 1, ( lo + 31 ) / B );
    uint64_t acc = 0;
    for ( uint32_t e = e0; e <= e1; ++e )
    {
        const uint64_t c = codes[p - e];
        const int sh = ( int ) ( e * B ) - ( int ) lo;
        acc |= sh >= 0 ? ( c << sh ) : ( c >> ( -sh ) );
    }
    key_out[i] = ( uint32_t ) acc;
}

// Per-tile digit histogram, digit-major: hist[d * ntiles + tile].  Keys are
// read as 16-byte vectors where the tile allows; each warp counts into its
// own copy of the 256 bins (shared atomics), summed at the end.
__global__ void __launch_bounds__ ( kSortThreads ) k_radix_hist ( const uint32_t * __restrict__ keys, uint32_t n,
                                                                   int shift, uint32_t * hist, uint32_t ntiles )
{
    constexpr int NW = kSortThreads / 32;
    __shared__ uint32_t cnt[NW][256];
    const int warp = threadIdx.x >> 5;
    for ( int d = threadIdx.x; d < NW * 256; d += kSortThreads ) ( &cnt[0][0] )[d] = 0;
    __syncthreads ();
    const uint32_t base = blockIdx.x * kSortTile;
    uint32_t * mine = cnt[warp];
    if ( base + kSortTile <= n )
    {
        const uint4 * k4 = reinterpret_cast<const uint4 *> ( keys + base );
#pragma unroll
        for ( int r = 0; r < kSortItems / 4; ++r )
        {
            const uint4 q = __ldg ( k4 + r * kSortThreads + threadIdx.x );
            atomicAdd ( &mine[( q.x >> shift ) & 255u], 1u );
            atomicAdd ( &mine[( q.y >> shift ) & 255u], 1u );
            atomicAdd ( &mine[( q.z >> shift ) & 255u], 1u );
            atomicAdd ( &mine[( q.w >> shift ) & 255u], 1u );
        }
    }
    else
    {
        for ( int r = 0; r < kSortItems; ++r )
        {
            const uint32_t i = base + r * kSortThreads + threadIdx.x;
            if ( i < n ) atomicAdd ( &mine[( keys[i] >> shift ) & 255u], 1u );
        }
    }
    __syncthreads ();
    for ( int d = threadIdx.x; d < 256; d += kSortThreads )
    {
        uint32_t t = 0;
#pragma unroll
        for ( int w = 0; w < NW; ++w ) t += cnt[w][d];
        hist[( size_t ) d * ntiles + blockIdx.x] = t;
    }
}

/*
 * Stable scatter of one 8-bit digit.  The CTA sorts its tile by the digit in
 * shared memory, then writes every digit's run of the tile as contiguous
 * stores.  Warp w owns the tile's items w*512 .. w*512+511 (16 rounds of 32,
 * kept in registers): in pass 1 each item gets its rank among the warp's
 * items of its digit so far (warp match masks and a per-warp running count
 * per digit); the per-warp counts then give each warp's offset within each
 * digit and the digits' tile-local starts (three CTA barriers per tile in
 * all); pass 2 stores every item at start[d] + warp offset + its rank.  The
 * tile's global base per digit comes from the digit-major scanned
 * histogram: offsets[d * ntiles + t] is the first output slot of digit d
 * from tile t.
 */
__global__ void __launch_bounds__ ( kSortThreads ) k_radix_scatter ( const uint32_t * __restrict__ keys_in,
                                                                      const uint32_t * __restrict__ vals_in,
                                                                      uint32_t * __restrict__ keys_out,
                                                                      uint32_t * __restrict__ vals_out,
                                                                      uint32_t n, int shift,
                                                                      const uint32_t * __restrict__ offsets,
                                                                      uint32_t ntiles )
{
    constexpr int NW = kSortThreads / 32;
    constexpr int PER_WARP = kSortTile / NW;                     // 512 items, 16 rounds of 32
    constexpr int ROUNDS = PER_WARP / 32;
    __shared__ uint32_t s_base[256];                 // global first slot of digit d from this tile
    __shared__ uint32_t s_start[256];                // tile-local first slot of digit d
    __shared__ uint32_t s_wh[NW][256];               // per warp: running count, then offset, of digit d
    __shared__ uint32_t s_wtot[NW];
    __shared__ uint32_t s_key[kSortTile];
    __shared__ uint32_t s_val[kSortTile];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t full = 0xffffffffu;
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * kSortTile;
    const uint32_t tn = min ( ( uint32_t ) kSortTile, n - base );
    for ( int i = threadIdx.x; i < NW * 256; i += kSortThreads ) ( &s_wh[0][0] )[i] = 0;
    {
        const uint32_t d = threadIdx.x;                          // kSortThreads == 256
        s_base[d] = offsets[( size_t ) d * ntiles + tile];
    }
    __syncthreads ();
    // pass 1: ranks within the warp's items of each digit, in input order
    // (keys and ranks in registers -- two 16-bit ranks per register; the
    // values are read in pass 2, so each is still read once)
    const uint32_t lt = lanemask_lt ();
    uint32_t key[ROUNDS], loc[ROUNDS / 2];
    uint32_t * wh = s_wh[warp];
#pragma unroll
    for ( int r = 0; r < ROUNDS; ++r )
    {
        const uint32_t li = warp * PER_WARP + r * 32 + lane;
        const bool valid = li < tn;
        key[r] = valid ? keys_in[base + li] : 0u;
        const uint32_t d = valid ? ( ( key[r] >> shift ) & 255u ) : ( 256u + lane );
        // lanes with this lane's digit: eight ballots over the digit bits
        // (and the invalid lanes, whose d >= 256, kept out by the valid vote)
        const uint32_t vb = __ballot_sync ( full, valid );
        uint32_t peers = valid ? vb : ( 1u << lane );
#pragma unroll
        for ( int b = 0; b < 8; ++b )
        {
            const uint32_t bal = __ballot_sync ( full, ( d >> b ) & 1u );
            peers &= ( ( d >> b ) & 1u ) ? bal : ~bal;
        }
        const uint32_t before = valid ? wh[d] : 0u;
        __syncwarp ();
        if ( valid && ( peers & lt ) == 0 ) wh[d] = before + __popc ( peers );
        __syncwarp ();
        const uint32_t rank = before + __popc ( peers & lt );            // < 512
        if ( r & 1 ) loc[r >> 1] |= rank << 16;
        else loc[r >> 1] = rank;
    }
    __syncthreads ();
    // per digit: warp offsets (exclusive over warps) and the tile count, then
    // the digits' exclusive scan (one digit per thread: warp scans + totals)
    {
        const uint32_t d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for ( int w = 0; w < NW; ++w )
        {
            const uint32_t t = s_wh[w][d];
            s_wh[w][d] = run;
            run += t;
        }
        const uint32_t c = run;
        uint32_t x = c;
#pragma unroll
        for ( int o = 1; o < 32; o <<= 1 )
        {
            const uint32_t y = __shfl_up_sync ( full, x, o );
            if ( lane >= o ) x += y;
        }
        if ( lane == 31 ) s_wtot[warp] = x;
        __syncthreads ();
        uint32_t add = 0;
        for ( int w = 0; w < warp; ++w ) add += s_wtot[w];
        s_start[d] = add + x - c;
    }
    __syncthreads ();
    // pass 2: the locally sorted tile in shared memory
#pragma unroll
    for ( int r = 0; r < ROUNDS; ++r )
    {
        const uint32_t li = warp * PER_WARP + r * 32 + lane;
        if ( li < tn )
        {
            const uint32_t d = ( key[r] >> shift ) & 255u;
            const uint32_t pos = s_start[d] + wh[d] + ( ( loc[r >> 1] >> ( ( r & 1 ) * 16 ) ) & 0xffffu );
            s_key[pos] = key[r];
            s_val[pos] = vals_in[base + li];
        }
    }
    __syncthreads ();
    // item i of digit d goes to s_base[d] + (i - s_start[d]): contiguous runs
    for ( uint32_t i = threadIdx.x; i < tn; i += kSortThreads )
    {
        const uint32_t k = s_key[i];
        const uint32_t d = ( k >> shift ) & 255u;
        keys_out[s_base[d] + ( i - s_start[d] )] = k;
        vals_out[s_base[d] + ( i - s_start[d] )] = s_val[i];
    }
}

// head[i] = 1 iff the factor at idx[i] differs from the one at idx[i-1].
// keys[i] is the most significant key chunk of factor idx[i] (sorted order,
// coalesced); when it is the whole factor (full_key) it decides alone,
// otherwise equal chunks fall back to comparing the symbols.
// Four flags per thread: one 16-byte load of their keys (keys and head are
// allocation bases, 16-byte aligned) and one 4-byte store of the flags.
__global__ void k_heads ( const uint32_t * __restrict__ idx, const uint32_t * __restrict__ keys, int full_key,
                          uint32_t n, const uint8_t * __restrict__ codes, uint32_t l, uint8_t * __restrict__ head )
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x, i0 = q * 4;
    if ( i0 >= n ) return;
    const bool whole = i0 + 4 <= n;
    uint32_t k[5];
    k[0] = i0 > 0 ? keys[i0 - 1] : 0u;
    if ( whole )
    {
        const uint4 v = reinterpret_cast<const uint4 *> ( keys )[q];
        k[1] = v.x; k[2] = v.y; k[3] = v.z; k[4] = v.w;
    }
    else
        for ( uint32_t t = 0; t < 4; ++t ) k[t + 1] = i0 + t < n ? keys[i0 + t] : 0u;
    uint32_t hw = 0;
#pragma unroll
    for ( uint32_t t = 0; t < 4; ++t )
    {
        const uint32_t i = i0 + t;
        if ( i >= n ) break;                    // the last group: no flag, no key, no factor past n
        uint32_t h = 1;
        if ( i > 0 && k[t + 1] == k[t] )
        {
            h = 0;
            if ( ! full_key )
            {
                const uint32_t p = idx[i], pq = idx[i - 1];
                for ( uint32_t e = 0; e < l; ++e )
                    if ( codes[p - e] != codes[pq - e] ) { h = 1; break; }
            }
        }
        hw |= h << ( 8 * t );
    }
    if ( whole ) reinterpret_cast<uint32_t *> ( head )[q] = hw;
    else
        for ( uint32_t t = 0; i0 + t < n; ++t ) head[i0 + t] = ( uint8_t ) ( hw >> ( 8 * t ) );
}

// A flag array's 16-byte chunk c as four words (the last, partial chunk from
// byte loads; flags is 16-byte aligned).
__device__ __forceinline__ uint4 flag_chunk ( const uint8_t * __restrict__ flags, uint32_t n, uint32_t c )
{
    const uint32_t base = c * 16;
    if ( base + 16 <= n ) return reinterpret_cast<const uint4 *> ( flags )[c];
    uint32_t w[4] = { 0, 0, 0, 0 };
    for ( uint32_t k = 0; base + k < n; ++k ) w[k >> 2] |= ( uint32_t ) flags[base + k] << ( 8 * ( k & 3 ) );
    return make_uint4 ( w[0], w[1], w[2], w[3] );
}

// Grid-stride (a few CTAs per SM) over 16-flag chunks read as one 16-byte
// load: heads are sparse on repetitive inputs, where one byte load per
// thread made the instruction count the cost.
__global__ void k_unique ( const uint32_t * __restrict__ idx, const uint8_t * __restrict__ head,
                           const uint32_t * __restrict__ pref, uint32_t n, uint32_t * __restrict__ uniq_pos )
{
    const uint32_t nc = ( n + 15 ) / 16;
    for ( uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x )
    {
        const uint4 q = flag_chunk ( head, n, c );
        const uint32_t w[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
        for ( int k = 0; k < 16; ++k )
            if ( ( w[k >> 2] >> ( 8 * ( k & 3 ) ) ) & 255u )
            {
                const uint32_t i = c * 16 + k;
                uniq_pos[pref[i]] = idx[i];
            }
    }
}

/*
 * Bit planes of each searched factor (factor ends at uniq_pos[w]).
 * Hamming fast kernel: symbol q at bit 32-l+q (top-aligned, matching text
 * windows whose newest symbol is bit 31).  Edit distance: symbol q at bit q.
 */
__global__ void k_wplanes32 ( const uint32_t * __restrict__ uniq_pos, uint32_t U, const uint8_t * __restrict__ codes,
                              uint32_t l, uint32_t B, int top_aligned, uint32_t * __restrict__ out )
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if ( w >= U ) return;
    const uint32_t first = uniq_pos[w] + 1 - l;
    uint32_t pl[kMaxPlanes] = { 0, 0, 0, 0, 0 };
    for ( uint32_t q = 0; q < l; ++q )
    {
        const uint32_t c = codes[first + q];
        const uint32_t bit = top_aligned ? ( 32 - l + q ) : q;
#pragma unroll
        for ( int b = 0; b < kMaxPlanes; ++b ) pl[b] |= ( ( c >> b ) & 1u ) << bit;
    }
    for ( uint32_t b = 0; b < B; ++b ) out[( size_t ) b * U + w] = pl[b];
}

/*
 * 64-bit multiword planes for the generic kernel (any l <= MOTEX_MAX_FACTOR).
 * Edit distance: symbol q at bit q.  Hamming: symbol q at bit l-1-q (the
 * newest text symbol enters the sliding window at bit 0).
 */
__global__ void k_wplanes64 ( const uint32_t * __restrict__ uniq_pos, uint32_t U, const uint8_t * __restrict__ codes,
                              uint32_t l, uint32_t B, uint32_t nw64, int reversed, uint64_t * __restrict__ out )
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if ( w >= U ) return;
    const uint32_t first = uniq_pos[w] + 1 - l;
    for ( uint32_t b = 0; b < B; ++b )
        for ( uint32_t j = 0; j < nw64; ++j )
        {
            uint64_t word = 0;
            for ( uint32_t bit = 0; bit < 64; ++bit )
            {
                const uint32_t g = j * 64 + bit;             // bit index inside the factor
                if ( g >= l ) break;
                const uint32_t q = reversed ? ( l - 1 - g ) : g;
                word |= ( uint64_t ) ( ( codes[first + q] >> b ) & 1u ) << bit;
            }
            out[( ( size_t ) b * U + w ) * nw64 + j] = word;
        }
}

// ------------------------------------------------------------------ filter

/*
 * Quorum filter of functions.cc:1105-1108 (qok[u] holds the reference's
 * double-precision quorum test for u sequences, computed on the host) and
 * first-occurrence marking: each searched factor passing the filter is
 * reported at its first occurrence.
 */
__global__ void k_finalize ( FinalizeArgs a )
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if ( w >= a.U ) return;
    uint32_t u = a.u_acc[w];
    for ( uint32_t s = 0; s < a.n_split; ++s ) u += a.split_flags[( size_t ) s * a.U + w];
    const uint32_t v = a.v_acc[w];
    if ( a.u_out ) { a.u_out[w] = u; a.v_out[w] = v; }
    if ( ! a.mark ) return;
    if ( u <= a.nseq && a.qok[u] && v >= a.nmin && v <= a.nmax )
    {
        const uint32_t p = a.uniq_pos[w];
        a.mark[p] = 1;
        a.rec_u[p] = u;
        a.rec_v[p] = v;
    }
}

// Grid-stride over 16-mark chunks like k_unique (marks are sparse).
__global__ void k_compact ( const uint8_t * __restrict__ mark, const uint32_t * __restrict__ pref, uint32_t n,
                            const uint32_t * __restrict__ rec_u, const uint32_t * __restrict__ rec_v,
                            uint32_t * __restrict__ out )
{
    const uint32_t nc = ( n + 15 ) / 16;
    for ( uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x )
    {
        const uint4 q = flag_chunk ( mark, n, c );
        const uint32_t w[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
        for ( int k = 0; k < 16; ++k )
            if ( ( w[k >> 2] >> ( 8 * ( k & 3 ) ) ) & 255u )
            {
                const uint32_t p = c * 16 + k, j = pref[p];
                out[3 * ( size_t ) j + 0] = p;
                out[3 * ( size_t ) j + 1] = rec_u[p];
                out[3 * ( size_t ) j + 2] = rec_v[p];
            }
    }
}

} // namespace mtx
