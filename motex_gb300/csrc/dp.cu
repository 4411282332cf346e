// All-factors x all-texts approximate-matching DP of the GB300 engine.
//
// Every CTA owns kDPThreads * W searched factors (W per thread, bit planes in
// registers) and one chunk of the concatenated text; all its threads walk the
// same text positions, so the text stream is a broadcast read and every
// per-position quantity is computed once per thread and reused by W factors.
//
//  Hamming (d = 0), flasm_hd contract: a hit ends at text position p when the
//    window t[p-l+1..p] lies inside one sequence and has <= e mismatches.
//    The 32 text symbols ending at p are one funnel shift of two plane words
//    per plane; mismatches = OR over planes of (factor ^ window), masked to
//    the top l bits; hit = popc <= e.
//  Edit distance (d = 1), flasm_ed contract: a hit ends at p when
//    min_s ED(factor, t[s..p]) <= e.  Myers/Hyyro bit-vector column recurrence
//    (one 32-bit word per factor, l <= 32), Eq built from the factor planes
//    and the broadcast text symbol bits; the score D[l][p] is tracked either
//    scaled by 2^(l-1) (l <= 28, two ANDs and one add) or shifted down.
//
// Per (factor, sequence): hits are counted; at the end of each sequence the
// count goes to v and (count > 0) to u.  A sequence cut by a chunk boundary
// records its presence in a per-split-sequence flag row instead, so u counts
// it once however many chunks saw it.
#include "kernels.cuh"

namespace mtx
{

namespace
{

template <int W>
__device__ __forceinline__ void flush_sequence ( const DPArgs & a, uint32_t base, int cur_split, uint32_t ( &cnt )[W],
                                                 uint32_t ( &uacc )[W], uint32_t ( &vacc )[W] )
{
#pragma unroll
    for ( int i = 0; i < W; ++i )
    {
        const uint32_t c = cnt[i];
        if ( cur_split < 0 )
            uacc[i] += c != 0u;
        else if ( c )
        {
            const uint32_t w = base + i * kDPThreads;
            if ( w < a.U ) a.split_flags[( size_t ) cur_split * a.U + w] = 1;
        }
        vacc[i] += c;
        cnt[i] = 0;
    }
}

template <int W>
__device__ __forceinline__ void finish_chunk ( const DPArgs & a, const ChunkInfo & ch, uint32_t base,
                                               uint32_t ( &cnt )[W], uint32_t ( &uacc )[W], uint32_t ( &vacc )[W] )
{
#pragma unroll
    for ( int i = 0; i < W; ++i )
    {
        const uint32_t w = base + i * kDPThreads;
        if ( w >= a.U ) continue;
        const uint32_t c = cnt[i];
        if ( c )
        {
            if ( ch.last_split >= 0 ) a.split_flags[( size_t ) ch.last_split * a.U + w] = 1;
            else uacc[i] += 1;
        }
        const uint32_t v = vacc[i] + c;
        if ( uacc[i] ) atomicAdd ( a.u_acc + w, uacc[i] );
        if ( v ) atomicAdd ( a.v_acc + w, v );
    }
}

} // namespace

template <int B, int W, bool ED, bool SCALED>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_fast ( const DPArgs a )
{
    const uint32_t base = blockIdx.x * ( kDPThreads * W ) + threadIdx.x;
    const uint32_t l = a.l;
    uint32_t wp[W][B];
    uint32_t cnt[W], uacc[W], vacc[W];
#pragma unroll
    for ( int i = 0; i < W; ++i )
    {
        const uint32_t w = base + i * kDPThreads;
        const bool ok = w < a.U;
#pragma unroll
        for ( int b = 0; b < B; ++b ) wp[i][b] = ok ? __ldg ( a.wplanes32 + ( size_t ) b * a.U + w ) : 0u;
        cnt[i] = uacc[i] = vacc[i] = 0;
    }
    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;

    if constexpr ( ! ED )
    {
        const uint32_t topmask = l >= 32 ? 0xffffffffu : ~( ( 1u << ( 32 - l ) ) - 1u );
        const uint32_t e = a.e;
        uint32_t prev[B], cur[B];
#pragma unroll
        for ( int b = 0; b < B; ++b ) prev[b] = __ldg ( planes + ( size_t ) b * stride + ch.begin );
        for ( uint32_t k = ch.begin; k < ch.end; ++k )
        {
#pragma unroll
            for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( planes + ( size_t ) b * stride + k + 1 );
            const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
            if ( vm == 0xffffffffu && em == 0u )
            {
#pragma unroll
                for ( int r = 0; r < 32; ++r )
                {
                    uint32_t y[B];
#pragma unroll
                    for ( int b = 0; b < B; ++b )
                        y[b] = ( r == 31 ? cur[b] : __funnelshift_r ( prev[b], cur[b], r + 1 ) ) & topmask;
#pragma unroll
                    for ( int i = 0; i < W; ++i )
                    {
                        uint32_t x = wp[i][0] ^ y[0];
#pragma unroll
                        for ( int b = 1; b < B; ++b ) x |= wp[i][b] ^ y[b];
                        cnt[i] += __popc ( x ) <= e;
                    }
                }
            }
            else
            {
                for ( int r = 0; r < 32; ++r )
                {
                    if ( ( vm >> r ) & 1u )
                    {
                        uint32_t y[B];
#pragma unroll
                        for ( int b = 0; b < B; ++b ) y[b] = __funnelshift_rc ( prev[b], cur[b], r + 1 ) & topmask;
#pragma unroll
                        for ( int i = 0; i < W; ++i )
                        {
                            uint32_t x = wp[i][0] ^ y[0];
#pragma unroll
                            for ( int b = 1; b < B; ++b ) x |= wp[i][b] ^ y[b];
                            cnt[i] += __popc ( x ) <= e;
                        }
                    }
                    if ( ( em >> r ) & 1u )
                    {
                        flush_sequence<W> ( a, base, cur_split, cnt, uacc, vacc );
                        cur_split = -1;
                    }
                }
            }
#pragma unroll
            for ( int b = 0; b < B; ++b ) prev[b] = cur[b];
        }
    }
    else
    {
        const uint32_t hb = 1u << ( l - 1 );
        const uint32_t sc0 = SCALED ? ( l << ( l - 1 ) ) : l;
        const uint32_t thr = SCALED ? ( ( a.e + 1 ) << ( l - 1 ) ) : ( a.e + 1 );
        const uint32_t sh = l - 1;
        uint32_t Pv[W], Mv[W], sc[W];
#pragma unroll
        for ( int i = 0; i < W; ++i ) { Pv[i] = 0xffffffffu; Mv[i] = 0; sc[i] = sc0; }

        auto step = [&] ( int i, const uint32_t ( &T )[B] ) {
            uint32_t x = wp[i][0] ^ T[0];
#pragma unroll
            for ( int b = 1; b < B; ++b ) x |= wp[i][b] ^ T[b];
            const uint32_t Eq = ~x;
            const uint32_t Xv = Eq | Mv[i];
            const uint32_t Xh = ( ( ( Eq & Pv[i] ) + Pv[i] ) ^ Pv[i] ) | Eq;
            uint32_t Ph = Mv[i] | ~( Xh | Pv[i] );
            uint32_t Mh = Pv[i] & Xh;
            if constexpr ( SCALED )
                sc[i] += ( Ph & hb ) - ( Mh & hb );
            else
                sc[i] += ( ( Ph >> sh ) & 1u ) - ( ( Mh >> sh ) & 1u );
            Ph <<= 1;
            Mh <<= 1;
            Pv[i] = Mh | ~( Xv | Ph );
            Mv[i] = Ph & Xv;
        };

        uint32_t cur[B];
        for ( uint32_t k = ch.warm; k < ch.end; ++k )
        {
#pragma unroll
            for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( planes + ( size_t ) b * stride + k + 1 );
            const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
            const bool counting = k >= ch.begin;
            if ( counting && vm == 0xffffffffu && em == 0u )
            {
#pragma unroll
                for ( int r = 0; r < 32; ++r )
                {
                    uint32_t T[B];
#pragma unroll
                    for ( int b = 0; b < B; ++b ) T[b] = 0u - ( ( cur[b] >> r ) & 1u );
#pragma unroll
                    for ( int i = 0; i < W; ++i )
                    {
                        step ( i, T );
                        cnt[i] += sc[i] < thr;
                    }
                }
            }
            else
            {
                for ( int r = 0; r < 32; ++r )
                {
                    uint32_t T[B];
#pragma unroll
                    for ( int b = 0; b < B; ++b ) T[b] = 0u - ( ( cur[b] >> r ) & 1u );
                    const bool count_here = counting && ( ( vm >> r ) & 1u );
#pragma unroll
                    for ( int i = 0; i < W; ++i )
                    {
                        step ( i, T );
                        if ( count_here ) cnt[i] += sc[i] < thr;
                    }
                    if ( ( em >> r ) & 1u )
                    {
                        if ( counting )
                        {
                            flush_sequence<W> ( a, base, cur_split, cnt, uacc, vacc );
                            cur_split = -1;
                        }
#pragma unroll
                        for ( int i = 0; i < W; ++i ) { Pv[i] = 0xffffffffu; Mv[i] = 0; sc[i] = sc0; }
                    }
                }
            }
        }
    }
    finish_chunk<W> ( a, ch, base, cnt, uacc, vacc );
}

/*
 * Generic kernel for any factor length up to 64 * NW (one factor per
 * thread, 64-bit multiword planes).  Hamming keeps a B-plane sliding window
 * as a multiword shift register (newest symbol at bit 0); edit distance runs
 * the multiword Myers recurrence with carries across words.
 */
template <int NW, bool ED>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_generic ( const DPArgs a, int B )
{
    const uint32_t base = blockIdx.x * kDPThreads + threadIdx.x;
    const uint32_t w = base;
    const bool ok = w < a.U;
    const uint32_t l = a.l;
    const uint32_t top = ( l - 1 ) / 64, topbit = ( l - 1 ) % 64;
    const uint64_t lastmask = ( l % 64 ) ? ( ( 1ull << ( l % 64 ) ) - 1 ) : ~0ull;
    uint64_t wp[kMaxPlanes][NW];
#pragma unroll
    for ( int b = 0; b < kMaxPlanes; ++b )
#pragma unroll
        for ( int q = 0; q < NW; ++q )
            wp[b][q] = ( ok && b < B ) ? a.wplanes64[( ( size_t ) b * a.U + w ) * NW + q] : 0ull;
    uint32_t cnt[1] = { 0 }, uacc[1] = { 0 }, vacc[1] = { 0 };
    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;

    uint64_t Y[kMaxPlanes][NW];                       // Hamming window
    uint64_t Pv[NW], Mv[NW];                          // edit distance state
    uint32_t sc = l;
#pragma unroll
    for ( int q = 0; q < NW; ++q )
    {
        Pv[q] = ~0ull;
        Mv[q] = 0;
#pragma unroll
        for ( int b = 0; b < kMaxPlanes; ++b ) Y[b][q] = 0;
    }

    for ( uint32_t k = ch.warm; k < ch.end; ++k )
    {
        uint32_t cur[kMaxPlanes];
#pragma unroll
        for ( int b = 0; b < kMaxPlanes; ++b ) cur[b] = b < B ? __ldg ( planes + ( size_t ) b * stride + k + 1 ) : 0u;
        const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
        const bool counting = k >= ch.begin;
        for ( int r = 0; r < 32; ++r )
        {
            bool hit;
            if constexpr ( ! ED )
            {
                uint32_t d = 0;
#pragma unroll
                for ( int q = NW - 1; q >= 0; --q )
                {
                    uint64_t x = 0;
#pragma unroll
                    for ( int b = 0; b < kMaxPlanes; ++b )
                    {
                        if ( b >= B ) break;
                        const uint64_t in = q ? ( Y[b][q - 1] >> 63 ) : ( uint64_t ) ( ( cur[b] >> r ) & 1u );
                        Y[b][q] = ( Y[b][q] << 1 ) | in;
                        x |= wp[b][q] ^ Y[b][q];
                    }
                    if ( q == ( int ) top ) x &= lastmask;
                    if ( q <= ( int ) top ) d += __popcll ( x );
                }
                hit = d <= a.e;
            }
            else
            {
                uint64_t T[kMaxPlanes];
#pragma unroll
                for ( int b = 0; b < kMaxPlanes; ++b ) T[b] = 0ull - ( uint64_t ) ( ( cur[b] >> r ) & 1u );
                uint64_t carry = 0, ph_in = 0, mh_in = 0;
#pragma unroll
                for ( int q = 0; q < NW; ++q )
                {
                    uint64_t x = 0;
#pragma unroll
                    for ( int b = 0; b < kMaxPlanes; ++b )
                        if ( b < B ) x |= wp[b][q] ^ T[b];
                    const uint64_t Eq = ~x;
                    const uint64_t Xv = Eq | Mv[q];
                    const uint64_t t = Eq & Pv[q];
                    const uint64_t s1 = t + Pv[q];
                    const uint64_t s = s1 + carry;
                    carry = ( s1 < t ) | ( s < s1 );
                    const uint64_t Xh = ( s ^ Pv[q] ) | Eq;
                    const uint64_t Ph = Mv[q] | ~( Xh | Pv[q] );
                    const uint64_t Mh = Pv[q] & Xh;
                    if ( q == ( int ) top )
                        sc += ( uint32_t ) ( ( Ph >> topbit ) & 1u ) - ( uint32_t ) ( ( Mh >> topbit ) & 1u );
                    const uint64_t Ph2 = ( Ph << 1 ) | ph_in, Mh2 = ( Mh << 1 ) | mh_in;
                    ph_in = Ph >> 63;
                    mh_in = Mh >> 63;
                    Pv[q] = Mh2 | ~( Xv | Ph2 );
                    Mv[q] = Ph2 & Xv;
                }
                hit = sc <= a.e;
            }
            if ( counting && ( ( vm >> r ) & 1u ) ) cnt[0] += hit;
            if ( ( em >> r ) & 1u )
            {
                if ( counting )
                {
                    flush_sequence<1> ( a, base, cur_split, cnt, uacc, vacc );
                    cur_split = -1;
                }
                if constexpr ( ED )
                {
#pragma unroll
                    for ( int q = 0; q < NW; ++q ) { Pv[q] = ~0ull; Mv[q] = 0; }
                    sc = l;
                }
            }
        }
    }
    finish_chunk<1> ( a, ch, base, cnt, uacc, vacc );
}

// ------------------------------------------------------------------ launchers

template <int B, int W>
static bool launch_fast_bw ( const DPArgs & a, bool ed, dim3 grid, cudaStream_t st )
{
    if ( ! ed )
        k_dp_fast<B, W, false, false><<<grid, kDPThreads, 0, st>>> ( a );
    else if ( a.l <= 28 )
        k_dp_fast<B, W, true, true><<<grid, kDPThreads, 0, st>>> ( a );
    else
        k_dp_fast<B, W, true, false><<<grid, kDPThreads, 0, st>>> ( a );
    return true;
}

template <int B>
static bool launch_fast_b ( const DPArgs & a, int W, bool ed, dim3 grid, cudaStream_t st )
{
    switch ( W )
    {
        case 4: return launch_fast_bw<B, 4> ( a, ed, grid, st );
        case 8: return launch_fast_bw<B, 8> ( a, ed, grid, st );
        default: return false;
    }
}

bool launch_dp_fast ( const DPArgs & a, int B, int W, bool ed, dim3 grid, cudaStream_t st )
{
    if ( a.l < 1 || a.l > 32 ) return false;
    switch ( B )
    {
        case 1: return launch_fast_b<1> ( a, W, ed, grid, st );
        case 2: return launch_fast_b<2> ( a, W, ed, grid, st );
        case 3: return launch_fast_b<3> ( a, W, ed, grid, st );
        case 4: return launch_fast_b<4> ( a, W, ed, grid, st );
        case 5: return launch_fast_b<5> ( a, W, ed, grid, st );
        default: return false;
    }
}

bool launch_dp_generic ( const DPArgs & a, int B, uint32_t nw64, bool ed, dim3 grid, cudaStream_t st )
{
    if ( B < 1 || B > kMaxPlanes ) return false;
#define MTX_GEN( NW )                                                                              \
    case NW:                                                                                       \
        if ( ed ) k_dp_generic<NW, true><<<grid, kDPThreads, 0, st>>> ( a, B );                   \
        else k_dp_generic<NW, false><<<grid, kDPThreads, 0, st>>> ( a, B );                       \
        return true;
    switch ( nw64 )
    {
        MTX_GEN ( 1 )
        MTX_GEN ( 2 )
        MTX_GEN ( 3 )
        MTX_GEN ( 4 )
        default: return false;
    }
#undef MTX_GEN
}

} // namespace mtx
