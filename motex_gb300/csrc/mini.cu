// Small-job pipeline: the stages around the DP of jobs of at most
// kMiniMaxSymbols symbols in six kernels whose grid holds every job of a
// batch (blockIdx.y = job, a few CTAs per job), so that a batch of many
// small jobs costs a handful of launches instead of ~40 per job, and a lone
// small job two host synchronisations.
//
//   k_mini_clear   empty hash slots, cleared marks and accumulators;
//   k_mini_pack    codes, bit planes, match-end and sequence-end masks (warp
//                  ballots); the key of every factor (its l codes packed, B
//                  bits each, from a shift-or doubling over the warp's lanes)
//                  inserted into an open-addressing hash table that keeps
//                  each key's least end position -- the factor's first
//                  occurrence, as the reference's first-passing rule needs;
//   k_mini_uniq    the table's entries become the distinct-factor list (any
//                  order: every factor's u and v are independent);
//   k_mini_planes  the distinct factors' bit planes;
//   (the DP kernels, unchanged: one launch for the batch)
//   k_mini_final   quorum filter of every distinct factor (the reference's
//                  double expression, as a host table), marks at first
//                  occurrences;
//   k_mini_count / k_mini_write   ordered compaction of the marks into
//                  (position, u, v) records.
//
// Limits: plain motifs (no boxes) of l <= 31 symbols whose key fits 63 bits
// (l * B <= 63, so the all-ones word marks an empty slot), whole-set runs.
#include "kernels.cuh"

namespace mtx
{

namespace
{

__device__ __forceinline__ uint32_t mini_slot ( unsigned long long key, uint32_t tbits )
{
    return ( uint32_t ) ( ( key * 0x9E3779B97F4A7C15ull ) >> ( 64 - tbits ) );
}

// Key of the factor ending at each lane's position: c = this block's codes,
// pk = the previous block's keys (its lanes' l-symbol windows).  Window sizes
// double per level; a lane below s takes the previous block's window.
__device__ __forceinline__ unsigned long long mini_keys ( uint32_t c, unsigned long long pk, uint32_t l, uint32_t B,
                                                          unsigned long long keymask, int lane )
{
    unsigned long long y = c;
    for ( uint32_t s = 1; s < l; s <<= 1 )
    {
        const unsigned long long cur = __shfl_up_sync ( 0xffffffffu, y, s );
        const unsigned long long old = __shfl_sync ( 0xffffffffu, pk, ( lane + 32 - ( int ) s ) & 31 );
        const unsigned long long low = ( 1ull << ( s * B ) ) - 1ull;             // s * B < l * B <= 63
        const unsigned long long src = lane >= ( int ) s ? cur : ( old & low );
        y = ( y | ( src << ( s * B ) ) ) & keymask;
    }
    return y & keymask;
}

} // namespace

// CTA x of job blockIdx.y takes share x of n items (n split in gridDim.x
// near-equal ranges); false when the job needs fewer CTAs than the grid has.
__device__ __forceinline__ bool mini_share ( uint32_t n, uint32_t ctas, uint32_t & a, uint32_t & b )
{
    if ( blockIdx.x >= ctas ) return false;
    a = ( uint32_t ) ( ( uint64_t ) n * blockIdx.x / ctas );
    b = ( uint32_t ) ( ( uint64_t ) n * ( blockIdx.x + 1 ) / ctas );
    return true;
}

// Empty hash slots, cleared marks, accumulators and split flags (for the
// largest distinct-factor count, nwords), the planes' leading zero word.
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_clear ( const MiniJob * __restrict__ jobs )
{
    const MiniJob & J = jobs[blockIdx.y];
    if ( blockIdx.x >= J.ctas ) return;
    const uint32_t t = blockIdx.x * kMiniThreads + threadIdx.x, step = J.ctas * kMiniThreads;
    const uint32_t tsize = 1u << J.tbits;
    for ( uint32_t i = t; i < tsize; i += step )
    {
        J.tkey[i] = ~0ull;
        J.tpos[i] = 0xffffffffu;
    }
    for ( uint32_t i = t; i < J.total; i += step ) J.mark[i] = 0;
    for ( uint32_t i = t; i < J.nwords; i += step )
    {
        J.u_acc[i] = 0;
        J.v_acc[i] = 0;
    }
    for ( uint32_t i = t; i < J.n_split * J.nwords; i += step ) J.flags[i] = 0;
    if ( t < J.B ) J.planes[( size_t ) t * J.plane_stride] = 0;
    if ( t == 0 ) J.result[1] = 0;
}

// Codes, bit planes, masks; every factor's key into the hash table.
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_pack ( const MiniJob * __restrict__ jobs )
{
    constexpr int NWARP = kMiniThreads / 32;
    const MiniJob & J = jobs[blockIdx.y];
    __shared__ uint8_t s_cmap[256];
    uint32_t c0, c1;
    if ( ! mini_share ( J.nblk, J.ctas, c0, c1 ) ) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for ( int i = tid; i < 256; i += kMiniThreads ) s_cmap[i] = J.cmap[i];
    __syncthreads ();
    // warp w takes a contiguous range of this CTA's 32-position blocks, so
    // the previous block's keys are in its registers
    const uint32_t total = J.total, l = J.l, B = J.B, tsize = 1u << J.tbits;
    const unsigned long long keymask = ( 1ull << ( l * B ) ) - 1ull;
    const uint32_t kb0 = c0 + ( uint32_t ) ( ( uint64_t ) ( c1 - c0 ) * warp / NWARP );
    const uint32_t kb1 = c0 + ( uint32_t ) ( ( uint64_t ) ( c1 - c0 ) * ( warp + 1 ) / NWARP );
    const uint32_t full = 0xffffffffu;
    if ( kb0 >= kb1 ) return;
    unsigned long long pk = 0;
    if ( kb0 > 0 )
    {
        // keys of the block before the range, from the raw bytes (their low
        // windows, the part the doubling reads, need no earlier block)
        const uint32_t c = s_cmap[J.raw[( kb0 - 1 ) * 32 + lane]];
        pk = mini_keys ( c, 0ull, l, B, keymask, lane );
    }
    uint32_t pos = kb0 * 32 + lane;
    uint32_t s = 0;
    {
        uint32_t lo = 0, hi = J.nseq;
        const uint32_t p = pos < total ? pos : total - 1;
        while ( hi - lo > 1 )
        {
            const uint32_t mid = ( lo + hi ) >> 1;
            if ( J.offs[mid] <= p ) lo = mid; else hi = mid;
        }
        s = lo;
    }
    uint32_t start = J.offs[s], end = J.offs[s + 1];
    for ( uint32_t k = kb0; k < kb1; ++k, pos += 32 )
    {
        const bool in = pos < total;
        uint32_t c = 0;
        bool valid = false, is_end = false, factor = false;
        if ( in )
        {
            while ( end <= pos )
            {
                ++s;
                start = end;
                end = J.offs[s + 1];
            }
            c = s_cmap[J.raw[pos]];
            J.codes[pos] = ( uint8_t ) c;
            const uint32_t rel = pos - start, len = end - start;
            valid = len >= J.tml && rel >= J.vstart;
            is_end = pos == end - 1;
            factor = len >= J.tml && len >= l && rel + 1 >= l;
        }
        for ( uint32_t b = 0; b < B; ++b )
        {
            const uint32_t pl = __ballot_sync ( full, ( c >> b ) & 1u );
            if ( lane == 0 ) J.planes[( size_t ) b * J.plane_stride + k + 1] = pl;
        }
        const uint32_t vm = __ballot_sync ( full, valid ), em = __ballot_sync ( full, is_end );
        if ( lane == 0 )
        {
            J.vmask[k] = vm;
            J.emask[k] = em;
        }
        const unsigned long long key = mini_keys ( c, pk, l, B, keymask, lane );
        pk = key;
        if ( factor )
        {
            // open addressing at load <= 1/2: the probe meets the key or an
            // empty slot long before it could visit every slot (bit 0 of
            // result[0] if it ever did)
            uint32_t h = mini_slot ( key, J.tbits );
            bool placed = false;
            for ( uint32_t probe = 0; probe < tsize && ! placed; ++probe )
            {
                const unsigned long long old = atomicCAS ( J.tkey + h, ~0ull, key );
                if ( old == ~0ull || old == key )
                {
                    atomicMin ( J.tpos + h, pos );
                    placed = true;
                }
                h = ( h + 1 ) & ( tsize - 1 );
            }
            if ( ! placed ) atomicOr ( J.result, 1u );
        }
    }
}

// The table's entries: the first end position of every distinct factor
// (any order); result[1] counts them.
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_uniq ( const MiniJob * __restrict__ jobs )
{
    const MiniJob & J = jobs[blockIdx.y];
    uint32_t a, b;
    if ( ! mini_share ( 1u << J.tbits, J.ctas, a, b ) ) return;
    const int lane = threadIdx.x & 31;
    const uint32_t full = 0xffffffffu;
    for ( uint32_t i0 = a; i0 < b; i0 += kMiniThreads )
    {
        const uint32_t i = i0 + threadIdx.x;
        const bool occ = i < b && J.tkey[i] != ~0ull;
        const uint32_t m = __ballot_sync ( full, occ );
        uint32_t base = 0;
        if ( lane == 0 && m ) base = atomicAdd ( J.result + 1, __popc ( m ) );
        base = __shfl_sync ( full, base, 0 );
        if ( occ ) J.uniq[base + __popc ( m & lanemask_lt () )] = J.tpos[i];
    }
}

// Bit planes of the distinct factors (top-aligned for Hamming), [b * U + w].
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_planes ( const MiniJob * __restrict__ jobs )
{
    const MiniJob & J = jobs[blockIdx.y];
    if ( blockIdx.x >= J.ctas ) return;
    const uint32_t U = J.result[1], l = J.l;
    for ( uint32_t w = blockIdx.x * kMiniThreads + threadIdx.x; w < U; w += J.ctas * kMiniThreads )
    {
        const uint32_t p = J.uniq[w];
        uint32_t pl[kMaxPlanes] = { 0, 0, 0, 0, 0 };
        for ( uint32_t q = 0; q < l; ++q )
        {
            const uint32_t cc = J.codes[p + 1 - l + q];
            const uint32_t bit = J.top_aligned ? ( 32 - l + q ) : q;
#pragma unroll
            for ( int b = 0; b < kMaxPlanes; ++b ) pl[b] |= ( ( cc >> b ) & 1u ) << bit;
        }
        for ( uint32_t b = 0; b < J.B; ++b ) J.wpl[( size_t ) b * U + w] = pl[b];
    }
}

// Quorum filter of every distinct factor; marks at first occurrences.
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_final ( const MiniJob * __restrict__ jobs )
{
    const MiniJob & J = jobs[blockIdx.y];
    if ( blockIdx.x >= J.ctas ) return;
    const uint32_t U = J.result[1];
    for ( uint32_t w = blockIdx.x * kMiniThreads + threadIdx.x; w < U; w += J.ctas * kMiniThreads )
    {
        uint32_t u = J.u_acc[w];
        for ( uint32_t s = 0; s < J.n_split; ++s ) u += J.flags[( size_t ) s * U + w];
        const uint32_t v = J.v_acc[w];
        if ( u <= J.nseq && J.qok[u] && v >= J.nmin && v <= J.nmax )
        {
            const uint32_t p = J.uniq[w];
            J.mark[p] = 1;
            J.rec_u[p] = u;
            J.rec_v[p] = v;
        }
    }
}

// Marks per CTA share of the positions.
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_count ( const MiniJob * __restrict__ jobs )
{
    constexpr int NWARP = kMiniThreads / 32;
    const MiniJob & J = jobs[blockIdx.y];
    __shared__ uint32_t s_wsum[NWARP];
    uint32_t a, b;
    if ( ! mini_share ( J.total, J.ctas, a, b ) ) return;
    uint32_t cnt = 0;
    for ( uint32_t p = a + threadIdx.x; p < b; p += kMiniThreads ) cnt += J.mark[p];
    cnt = __reduce_add_sync ( 0xffffffffu, cnt );
    if ( ( threadIdx.x & 31 ) == 0 ) s_wsum[threadIdx.x >> 5] = cnt;
    __syncthreads ();
    if ( threadIdx.x == 0 )
    {
        uint32_t t = 0;
        for ( int w = 0; w < NWARP; ++w ) t += s_wsum[w];
        J.part[blockIdx.x] = t;
    }
}

// Ordered compaction of the marks into (position, u, v) records: CTA x
// starts after the marks of the shares before it; within the CTA thread t
// takes consecutive positions.  CTA 0 writes the job's motif count.
__global__ void __launch_bounds__ ( kMiniThreads ) k_mini_write ( const MiniJob * __restrict__ jobs )
{
    constexpr int NWARP = kMiniThreads / 32;
    const MiniJob & J = jobs[blockIdx.y];
    __shared__ uint32_t s_wsum[NWARP];
    uint32_t a, b;
    if ( ! mini_share ( J.total, J.ctas, a, b ) ) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t base = 0;
    for ( uint32_t x = 0; x < blockIdx.x; ++x ) base += J.part[x];
    if ( blockIdx.x == 0 && tid == 0 )
    {
        uint32_t all = 0;
        for ( uint32_t x = 0; x < J.ctas; ++x ) all += J.part[x];
        J.result[2] = all;
    }
    const uint32_t C = ( b - a + kMiniThreads - 1 ) / kMiniThreads;
    const uint32_t p0 = min ( b, a + tid * C ), p1 = min ( b, p0 + C );
    uint32_t cnt = 0;
    for ( uint32_t p = p0; p < p1; ++p ) cnt += J.mark[p];
    uint32_t x = cnt;
#pragma unroll
    for ( int o = 1; o < 32; o <<= 1 )
    {
        const uint32_t y = __shfl_up_sync ( 0xffffffffu, x, o );
        if ( lane >= o ) x += y;
    }
    if ( lane == 31 ) s_wsum[warp] = x;
    __syncthreads ();
    uint32_t before = 0;
    for ( int w = 0; w < warp; ++w ) before += s_wsum[w];
    uint32_t at = base + before + x - cnt;
    for ( uint32_t p = p0; p < p1; ++p )
        if ( J.mark[p] )
        {
            J.recs[3 * ( size_t ) at + 0] = p;
            J.recs[3 * ( size_t ) at + 1] = J.rec_u[p];
            J.recs[3 * ( size_t ) at + 2] = J.rec_v[p];
            ++at;
        }
}

} // namespace mtx
