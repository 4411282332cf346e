// Device bodies of the all-factors x all-texts approximate-matching DP.
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
//    (one 32-bit word per factor, l <= 32, or 2-4 factors per word for
//    l <= 15); Eq is read from a per-thread table by the text symbol's code
//    (B <= 3; split into low and high code bits for B = 4, 5 in the packed
//    body) or built from the factor planes and the broadcast text symbol
//    bits; the score D[l][p] is tracked either scaled by 2^(l-1) (l <= 28,
//    two ANDs and one add) or shifted down.
//
// Per (factor, sequence): hits are counted; at the end of each sequence the
// count goes to v and (count > 0) to u.  A sequence cut by a chunk boundary
// records its presence in a per-split-sequence flag row instead, so u counts
// it once however many chunks saw it.
#pragma once

#include "kernels.cuh"

namespace mtx
{

namespace dp_detail
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

} // namespace dp_detail

using namespace dp_detail;

/*
 * Shared memory of the 1-lane body: none for Hamming; for edit distance with
 * B <= 3 the per-thread match table Eq[code][register][thread] (Myers Peq of
 * each of the thread's W factors against each symbol code).
 */
__host__ __device__ constexpr size_t fast_smem_bytes ( int B, int W, bool ed )
{
    return ( ed && B <= 3 ) ? ( size_t ) ( 1 << B ) * W * kDPThreads * sizeof ( uint32_t ) : 0;
}

template <int B, int W, bool ED, bool SCALED, int UR>
__device__ __forceinline__ void dp_fast_body ( const DPArgs & a, uint32_t tile, uint32_t chunk )
{
    const uint32_t base = tile * ( kDPThreads * W ) + threadIdx.x;
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
    const ChunkInfo ch = a.chunks[chunk];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;

    if constexpr ( ! ED )
    {
        const uint32_t topmask = l >= 32 ? 0xffffffffu : ~( ( 1u << ( 32 - l ) ) - 1u );
        const uint32_t e = a.e;
        // every thread of the CTA walks the same text positions: the windows
        // of a block (32 positions x B planes) are built once into shared
        // memory, double-buffered so that one barrier per block suffices
        __shared__ uint32_t s_win[2][32 * B];
        for ( uint32_t k = ch.begin; k < ch.end; ++k )
        {
            uint32_t * win = s_win[( k - ch.begin ) & 1];
            for ( uint32_t i = threadIdx.x; i < 32u * B; i += kDPThreads )
            {
                const uint32_t * pl = planes + ( size_t ) ( i >> 5 ) * stride;
                win[i] = __funnelshift_rc ( __ldg ( pl + k ), __ldg ( pl + k + 1 ), ( i & 31u ) + 1 ) & topmask;
            }
            __syncthreads ();
            const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
            if ( vm == 0xffffffffu && em == 0u )
            {
#pragma unroll 1
                for ( int g = 0; g < 32; g += UR )
                {
#pragma unroll
                    for ( int rr = 0; rr < UR; ++rr )
                    {
                        const int r = g + rr;
                        uint32_t y[B];
#pragma unroll
                        for ( int b = 0; b < B; ++b ) y[b] = win[b * 32 + r];
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
            }
            else
            {
                for ( int r = 0; r < 32; ++r )
                {
                    if ( ( vm >> r ) & 1u )
                    {
                        uint32_t y[B];
#pragma unroll
                        for ( int b = 0; b < B; ++b ) y[b] = win[b * 32 + r];
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
        constexpr bool TAB = B <= 3;
        extern __shared__ uint32_t smem[];
        uint32_t * s_eq = smem;                                  // [code][register][thread]
        if constexpr ( TAB )
            for ( int c = 0; c < ( 1 << B ); ++c )
#pragma unroll
                for ( int i = 0; i < W; ++i )
                {
                    uint32_t x = 0;
#pragma unroll
                    for ( int b = 0; b < B; ++b ) x |= wp[i][b] ^ ( ( ( c >> b ) & 1 ) ? 0xffffffffu : 0u );
                    s_eq[( c * W + i ) * kDPThreads + threadIdx.x] = ~x;
                }
        // adds and shifts as multiply-adds by 1, 2 and -1 held in kernel data:
        // they issue on the FMA pipe, which the step's logic ops leave idle
        const uint32_t one = a.one, two = a.two, neg1 = a.neg1;
        auto step_eq = [&] ( int i, const uint32_t Eq ) {
            const uint32_t Xv = Eq | Mv[i];
            const uint32_t Xh = ( ( ( Eq & Pv[i] ) * one + Pv[i] ) ^ Pv[i] ) | Eq;
            const uint32_t Ph = Mv[i] | ~( Xh | Pv[i] );
            const uint32_t Mh = Pv[i] & Xh;
            if constexpr ( SCALED )
            {
                sc[i] = ( Ph & hb ) * one + sc[i];
                sc[i] = ( Mh & hb ) * neg1 + sc[i];
            }
            else
            {
                sc[i] = ( ( Ph >> sh ) & 1u ) * one + sc[i];
                sc[i] = ( ( Mh >> sh ) & 1u ) * neg1 + sc[i];
            }
            const uint32_t Ph2 = Ph * two, Mh2 = Mh * two;
            Pv[i] = Mh2 | ~( Xv | Ph2 );
            Mv[i] = Ph2 & Xv;
        };
        auto step = [&] ( int i, const uint32_t ( &T )[B] ) {
            uint32_t x = wp[i][0] ^ T[0];
#pragma unroll
            for ( int b = 1; b < B; ++b ) x |= wp[i][b] ^ T[b];
            step_eq ( i, ~x );
        };
        // B <= 3: every thread walks the same text positions, so each warp
        // builds the table row of each position of a block once (lane r takes
        // position r) into its own shared buffer, double-buffered so that one
        // warp barrier per block suffices.  B = 4, 5 form the broadcast
        // symbol-bit masks per thread (kept: the shared form raised their
        // register count).
        __shared__ uint32_t s_row[kDPThreads / 32][2][32];
        const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
        const uint32_t * my_eq = s_eq + threadIdx.x;
        uint32_t cur[B];
        for ( uint32_t k = ch.warm; k < ch.end; ++k )
        {
            const uint32_t * pre = s_row[wid][( k - ch.warm ) & 1];
            if constexpr ( TAB )
            {
                uint32_t c = 0;
#pragma unroll
                for ( int b = 0; b < B; ++b ) c |= ( ( __ldg ( planes + ( size_t ) b * stride + k + 1 ) >> lane ) & 1u ) << b;
                s_row[wid][( k - ch.warm ) & 1][lane] = c * ( W * kDPThreads );
                __syncwarp ();
            }
            else
#pragma unroll
                for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( planes + ( size_t ) b * stride + k + 1 );
            const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
            const bool counting = k >= ch.begin;
            if ( counting && vm == 0xffffffffu && em == 0u )
            {
#pragma unroll 1
                for ( int g = 0; g < 32; g += UR )
                {
                    uint32_t cg[B];
#pragma unroll
                    for ( int b = 0; b < B; ++b ) cg[b] = TAB ? 0u : cur[b] >> g;
#pragma unroll
                    for ( int rr = 0; rr < UR; ++rr )
                    {
                        if constexpr ( TAB )
                        {
                            const uint32_t * row = my_eq + pre[g + rr];
#pragma unroll
                            for ( int i = 0; i < W; ++i )
                            {
                                step_eq ( i, row[i * kDPThreads] );
                                cnt[i] += sc[i] < thr;
                            }
                        }
                        else
                        {
                            uint32_t T[B];
#pragma unroll
                            for ( int b = 0; b < B; ++b ) T[b] = 0u - ( ( cg[b] >> rr ) & 1u );
#pragma unroll
                            for ( int i = 0; i < W; ++i )
                            {
                                step ( i, T );
                                cnt[i] += sc[i] < thr;
                            }
                        }
                    }
                }
            }
            else
            {
                for ( int r = 0; r < 32; ++r )
                {
                    const bool count_here = counting && ( ( vm >> r ) & 1u );
                    if constexpr ( TAB )
                    {
                        const uint32_t * row = my_eq + pre[r];
#pragma unroll
                        for ( int i = 0; i < W; ++i )
                        {
                            step_eq ( i, row[i * kDPThreads] );
                            if ( count_here ) cnt[i] += sc[i] < thr;
                        }
                    }
                    else
                    {
                        uint32_t T[B];
#pragma unroll
                        for ( int b = 0; b < B; ++b ) T[b] = 0u - ( ( cur[b] >> r ) & 1u );
#pragma unroll
                        for ( int i = 0; i < W; ++i )
                        {
                            step ( i, T );
                            if ( count_here ) cnt[i] += sc[i] < thr;
                        }
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
 * Persistent form: a grid sized to the resident CTA slots pulls (job, tile,
 * chunk) items from a device counter until the list is exhausted, so jobs of
 * any size and count share one launch.  The loop ends because every pull
 * advances the counter; there is no waiting on other CTAs.
 */
__device__ __forceinline__ bool next_item ( const WorkItem * items, uint32_t nitems, uint32_t * counter, WorkItem & w )
{
    __shared__ uint32_t s_item;
    __syncthreads ();
    if ( threadIdx.x == 0 ) s_item = atomicAdd ( counter, 1u );
    __syncthreads ();
    const uint32_t it = s_item;
    if ( it >= nitems ) return false;
    w = items[it];
    return true;
}

/*
 * Edit distance with NL factors per 32-bit register (SWAR), l <= 15.
 * Lane i holds a factor in bits [i*S, i*S+l), S = max(l+1, 6), with guard
 * bits from i*S+l up to the next lane (S >= 6 lets every S-bit count field
 * hold the 32 hits of one text block).  The text bits are cleared at the
 * guards, so Eq has 1 there; Pv and
 * Mv keep 0 there (Mv through the NG mask, Pv because the Mh that is shifted
 * up is taken without the lanes' top bits).  With those invariants no carry
 * of (Eq&Pv)+Pv and no shifted Ph/Mh bit crosses into the next lane.  The
 * per-lane scores live in bit fields at i*S (each in [0, l]); the hit test
 * adds 2^h-(e+1) per field and reads bit h of each field (h = ceil(log2 l)
 * for NL = 2, 3, whose count fields sit at bit h of each lane, so the hit
 * bits are added where they are; h = l-1 for NL = 4, whose count shifts
 * them to the lane base).  Hits are counted in per-lane fields and moved to
 * shared memory every 32 positions.
 * The step is bound by the ALU pipe (logic ops, shifts, adds); its adds and
 * left shifts are written as multiply-adds by runtime constants so that they
 * issue on the otherwise idle FMA pipe.
 */

/*
 * Shared memory of the SWAR body: hit counters [field][thread] (count in the
 * current text, texts seen, occurrences) and the per-thread match table
 * Eq[code][register][thread]: the Myers Eq vector of each of the thread's W
 * registers against each symbol code, so a step reads Eq with shared-memory
 * loads (LSU pipe) instead of forming it from the bit planes.  B <= 3: one
 * row per code; B = 4, 5: the low-three-bit and high-bit tables below.
 */
__host__ __device__ constexpr bool swar_table ( int B ) { return B <= 3; }
// B = 4, 5: Eq is a conjunction over the planes, so it splits into a table of
// the low three code bits and one of the high bits: Eq = lo[c & 7] & hi[c >> 3]
__host__ __device__ constexpr size_t swar_table_words ( int B )
{
    return swar_table ( B ) ? ( size_t ) ( 1 << B ) : ( size_t ) ( 8 + ( 1 << ( B - 3 ) ) );
}
__host__ __device__ constexpr size_t swar_smem_bytes ( int B, int NL, int W )
{
    return ( ( size_t ) 3 * W * NL + swar_table_words ( B ) * W ) * kDPThreads * sizeof ( uint32_t );
}

template <int B, int NL, int W, int UR>
__device__ __forceinline__ void dp_swar_body ( const DPArgs & a, const SwarConst & C, uint32_t tile, uint32_t chunk )
{
    extern __shared__ uint32_t smem[];
    constexpr int NF = W * NL;                      // factors per thread
    // [field][thread]: count in the current text, texts seen, occurrences
    uint32_t * s_cnt = smem;
    uint32_t * s_u = smem + NF * kDPThreads;
    uint32_t * s_v = smem + 2 * NF * kDPThreads;
    const int tid = threadIdx.x;
    for ( int f = 0; f < NF; ++f ) s_cnt[f * kDPThreads + tid] = s_u[f * kDPThreads + tid] = s_v[f * kDPThreads + tid] = 0;

    const uint32_t gbase = tile * ( kDPThreads * W ) + tid;              // first factor group of this thread
    const uint32_t l = a.l, sh = l - 1;
    uint32_t wp[W][B];
#pragma unroll
    for ( int i = 0; i < W; ++i )
    {
#pragma unroll
        for ( int b = 0; b < B; ++b ) wp[i][b] = 0;
        const uint32_t g = gbase + i * kDPThreads;
#pragma unroll
        for ( int j = 0; j < NL; ++j )
        {
            const uint32_t w = g * NL + j;
            if ( w < a.U )
#pragma unroll
                for ( int b = 0; b < B; ++b ) wp[i][b] |= __ldg ( a.wplanes32 + ( size_t ) b * a.U + w ) << ( j * C.S );
        }
    }
    uint32_t Pv[W], Mv[W], sc[W], cnt[W];
    // sc holds score + K per field (K added once): the hit test is then one AND
    const uint32_t sc0k = C.SC0 + C.K;
#pragma unroll
    for ( int i = 0; i < W; ++i ) { Pv[i] = C.NG; Mv[i] = 0; sc[i] = sc0k; cnt[i] = 0; }
    constexpr bool TAB = swar_table ( B );
    uint32_t * s_eq = smem + 3 * NF * kDPThreads;            // [code][register][thread]
    uint32_t * s_hi = s_eq + 8 * W * kDPThreads;             // B = 4, 5: [high bits][register][thread]
    if constexpr ( ! TAB )
    {
        for ( int c = 0; c < 8; ++c )
#pragma unroll
            for ( int i = 0; i < W; ++i )
            {
                uint32_t x = 0;
#pragma unroll
                for ( int b = 0; b < 3; ++b ) x |= wp[i][b] ^ ( ( ( c >> b ) & 1 ) ? C.NG : 0u );
                s_eq[( c * W + i ) * kDPThreads + tid] = ~x;
            }
        for ( int c = 0; c < ( 1 << ( B - 3 ) ); ++c )
#pragma unroll
            for ( int i = 0; i < W; ++i )
            {
                uint32_t x = 0;
#pragma unroll
                for ( int b = 3; b < B; ++b ) x |= wp[i][b] ^ ( ( ( c >> ( b - 3 ) ) & 1 ) ? C.NG : 0u );
                s_hi[( c * W + i ) * kDPThreads + tid] = ~x;
            }
    }
    if constexpr ( TAB )
    {
        // text bits are cleared at the guards, so Eq is 1 there (lanes stay apart)
        for ( int c = 0; c < ( 1 << B ); ++c )
#pragma unroll
            for ( int i = 0; i < W; ++i )
            {
                uint32_t x = 0;
#pragma unroll
                for ( int b = 0; b < B; ++b ) x |= wp[i][b] ^ ( ( ( c >> b ) & 1 ) ? C.NG : 0u );
                s_eq[( c * W + i ) * kDPThreads + tid] = ~x;
            }
    }

    const ChunkInfo ch = a.chunks[chunk];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;

    auto step_eq = [&] ( int i, const uint32_t Eq ) {
        // additions and left shifts as multiply-adds by runtime constants:
        // they run on the FMA pipe, which the logic ops leave idle
        const uint32_t Xv = Eq | Mv[i];
        const uint32_t s = ( Eq & Pv[i] ) * C.ONE + Pv[i];
        const uint32_t Xh = ( s ^ Pv[i] ) | Eq;
        const uint32_t Ph = Mv[i] | ~( Xh | Pv[i] );
        const uint32_t Mhs = Pv[i] & Xh & C.NGm1;
        const uint32_t mh = Pv[i] & Xh & C.HB;
        const uint32_t ph = Ph & C.HB;
        if constexpr ( NL != 3 )
        {
            // ph and mh are disjoint and their top bit is at most 30 (NL = 2:
            // 2l <= 30; NL = 4: 3(l+1) + l-1 <= 30), so ph - mh is exact as a
            // signed word and one arithmetic shift gives every field its
            // +1 / 0 / -1 (a field's borrow cancels against the next field)
            const int32_t d = ( int32_t ) ( mh * C.NEG1 + ph );
            sc[i] = ( uint32_t ) ( d >> sh ) * C.ONE + sc[i];
        }
        else
        {
            // NL = 3 with l = 10 has its top lane's bit l-1 at bit 31
            sc[i] = ( ph >> sh ) * C.ONE + sc[i];
            sc[i] = ( mh >> sh ) * C.NEG1 + sc[i];
        }
        const uint32_t Ph2 = Ph * C.TWO, Mh2 = Mhs * C.TWO;
        Pv[i] = Mh2 | ~( Xv | Ph2 );
        Mv[i] = Ph2 & Xv & C.NG;
    };
    // Eq-table rows of the text positions of a block: every thread walks the
    // same positions, so each warp computes the rows (code * W * kDPThreads;
    // for B = 4, 5 those of the low three code bits and of the high bits) once
    // per block, lane r taking position r, into its own shared buffer,
    // double-buffered so that one warp barrier per block suffices, instead of
    // every thread deriving every row from the bit planes
    __shared__ uint32_t s_rl[kDPThreads / 32][2][32], s_rh[kDPThreads / 32][2][32];
    const uint32_t lane = tid & 31, wid = tid >> 5;
    const uint32_t * my_eq = s_eq + tid;
    const uint32_t * my_hi = s_hi + tid;
    // NL = 2, 3: hit bits added where they are (count fields at C.Q of each
    // lane); NL = 4: shifted to the lane base
    constexpr bool HIT_IN_PLACE = NL != 4;
    auto count = [&] ( int i ) {
        if constexpr ( HIT_IN_PLACE ) cnt[i] = ( ~sc[i] & C.HQ ) * C.ONE + cnt[i];
        else cnt[i] = ( ( ~sc[i] & C.HQ ) >> sh ) * C.ONE + cnt[i];
    };
    auto drain = [&] () {                           // register fields -> shared counters
#pragma unroll
        for ( int i = 0; i < W; ++i )
        {
#pragma unroll
            for ( int j = 0; j < NL; ++j ) s_cnt[( i * NL + j ) * kDPThreads + tid] += ( cnt[i] >> ( j * C.S + C.Q ) ) & C.FM;
            cnt[i] = 0;
        }
    };
    auto end_sequence = [&] () {
        for ( int f = 0; f < NF; ++f )
        {
            const uint32_t c = s_cnt[f * kDPThreads + tid];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[f * kDPThreads + tid] += 1;
            else
            {
                const uint32_t w = ( gbase + ( f / NL ) * kDPThreads ) * NL + ( f % NL );
                if ( w < a.U ) a.split_flags[( size_t ) cur_split * a.U + w] = 1;
            }
            s_v[f * kDPThreads + tid] += c;
            s_cnt[f * kDPThreads + tid] = 0;
        }
    };

    for ( uint32_t k = ch.warm; k < ch.end; ++k )
    {
        uint32_t * rl = s_rl[wid][( k - ch.warm ) & 1];
        uint32_t * rh = s_rh[wid][( k - ch.warm ) & 1];
        {
            uint32_t c = 0;
#pragma unroll
            for ( int b = 0; b < B; ++b ) c |= ( ( __ldg ( planes + ( size_t ) b * stride + k + 1 ) >> lane ) & 1u ) << b;
            rl[lane] = ( TAB ? c : ( c & 7u ) ) * ( W * kDPThreads );
            if constexpr ( ! TAB ) rh[lane] = ( c >> 3 ) * ( W * kDPThreads );     // the high-bit table
        }
        __syncwarp ();
        const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
        const bool counting = k >= ch.begin;
        if ( counting && vm == 0xffffffffu && em == 0u )
        {
            // B >= 4 (protein-like: chance hits are rare): a group of UR
            // positions only ORs the factors' hit bits, and a group that saw one
            // is replayed from its starting state with exact per-position counts
            // (the steps are deterministic).  With 2-3 planes (DNA) hits are
            // frequent enough that the replays cost what the deferral saves, so
            // every step counts.
            constexpr bool DEFER = B >= 4;
#pragma unroll 1
            for ( int g = 0; g < 32; g += UR )
            {
                if constexpr ( ! DEFER )
                {
#pragma unroll
                    for ( int rr = 0; rr < UR; ++rr )
                    {
                        const uint32_t * row = my_eq + rl[g + rr];
#pragma unroll
                        for ( int i = 0; i < W; ++i )
                        {
                            step_eq ( i, row[i * kDPThreads] );
                            count ( i );
                        }
                    }
                }
                else
                {
                uint32_t P0[W], M0[W], S0[W];
#pragma unroll
                for ( int i = 0; i < W; ++i ) { P0[i] = Pv[i]; M0[i] = Mv[i]; S0[i] = sc[i]; }
                uint32_t hacc = 0;
#pragma unroll
                for ( int rr = 0; rr < UR; ++rr )
                {
                    const uint32_t * lo = my_eq + rl[g + rr];
                    const uint32_t * hi = my_hi + rh[g + rr];
#pragma unroll
                    for ( int i = 0; i < W; ++i )
                    {
                        step_eq ( i, TAB ? lo[i * kDPThreads] : ( lo[i * kDPThreads] & hi[i * kDPThreads] ) );
                        hacc |= ~sc[i] & C.HQ;
                    }
                }
                if ( hacc )
                {
#pragma unroll
                    for ( int i = 0; i < W; ++i ) { Pv[i] = P0[i]; Mv[i] = M0[i]; sc[i] = S0[i]; }
#pragma unroll 1
                    for ( int rr = 0; rr < UR; ++rr )
                    {
                        const uint32_t * lo = my_eq + rl[g + rr];
                        const uint32_t * hi = my_hi + rh[g + rr];
#pragma unroll
                        for ( int i = 0; i < W; ++i )
                        {
                            step_eq ( i, TAB ? lo[i * kDPThreads] : ( lo[i * kDPThreads] & hi[i * kDPThreads] ) );
                            count ( i );
                        }
                    }
                }
                }
            }
        }
        else
        {
            for ( int r = 0; r < 32; ++r )
            {
                const bool count_here = counting && ( ( vm >> r ) & 1u );
                if constexpr ( TAB )
                {
                    const uint32_t * row = my_eq + rl[r];
#pragma unroll
                    for ( int i = 0; i < W; ++i )
                    {
                        step_eq ( i, row[i * kDPThreads] );
                        if ( count_here ) count ( i );
                    }
                }
                else
                {
                    const uint32_t * lo = my_eq + rl[r];
                    const uint32_t * hi = my_hi + rh[r];
#pragma unroll
                    for ( int i = 0; i < W; ++i )
                    {
                        step_eq ( i, lo[i * kDPThreads] & hi[i * kDPThreads] );
                        if ( count_here ) count ( i );
                    }
                }
                if ( ( em >> r ) & 1u )
                {
                    if ( counting )
                    {
                        drain ();
                        end_sequence ();
                        cur_split = -1;
                    }
#pragma unroll
                    for ( int i = 0; i < W; ++i ) { Pv[i] = C.NG; Mv[i] = 0; sc[i] = sc0k; }
                }
            }
        }
        drain ();
    }
    // chunk end
    for ( int f = 0; f < NF; ++f )
    {
        const uint32_t w = ( gbase + ( f / NL ) * kDPThreads ) * NL + ( f % NL );
        if ( w >= a.U ) continue;
        const uint32_t c = s_cnt[f * kDPThreads + tid];
        uint32_t u = s_u[f * kDPThreads + tid];
        if ( c )
        {
            if ( ch.last_split >= 0 ) a.split_flags[( size_t ) ch.last_split * a.U + w] = 1;
            else u += 1;
        }
        const uint32_t v = s_v[f * kDPThreads + tid] + c;
        if ( u ) atomicAdd ( a.u_acc + w, u );
        if ( v ) atomicAdd ( a.v_acc + w, v );
    }
}

/*
 * Hamming, NL factors of l bits per register (lane j at bits [j*l, j*l+l),
 * symbol q of the factor at bit j*l+q; no guard bits, XOR and OR do not
 * carry).  Per text position the l-symbol window of each plane is shifted
 * down to bit 0 and replicated into every lane by one multiply with
 * REP = sum 2^(j*l) (the lanes do not overlap, so the product does not
 * carry); then each register costs B XOR/ORs for its NL factors, and each
 * lane a masked popc.  Hit counts live in l-bit register fields (l >= 6
 * holds a 32-position block), drained to shared memory per block like the
 * edit-distance SWAR body.
 *
 * E >= 0 (e = E <= 3): the popc-free form.  Lanes of l bits with a guard
 * bit above each (lane j at bits [j*S, j*S+l), S = l+1, guard bit j*S+l),
 * the guards set in the mismatch word x by plane 0 of the factor register.
 * E times, x = (x & (x - L)) | G clears the lowest set bit of every lane
 * (L: the lanes' bit 0; a lane already zero borrows from its own guard,
 * which the OR sets again, so no borrow crosses a lane).  Then the lane has
 * at most E mismatches exactly when it is zero, and x - L clears its guard
 * bit exactly then: the hits are ~(x - L) & G, added where they are into
 * 6-bit count fields at the guard bits.  Per register: B-1 logic ops for x,
 * one per clear and one for the hits on the ALU pipe; the subtractions and
 * the count add are multiply-adds (FMA pipe); no popc.  C holds S = l+1,
 * HB = the guard bits G, K = -L, REP = sum 2^(j*S), Q = l (count field
 * offset in a lane) and FM = 63.
 *
 * NL = 3 (6 <= l <= 10): the top lane, at 2S, has no guard (for l = 10 it
 * ends at bit 31).  Its clears need none: a borrow out of it leaves the
 * register or lands in bits that x and the AND keep zero.  It is zero
 * exactly when x < LIM = 2^(2S), and that hit is counted by one compare and
 * add into a count field at bit 0 (below lane 0's count field at bit l).
 */
template <int B, int NL, int W, int UR, int E = -1>
__device__ __forceinline__ void dp_hswar_body ( const DPArgs & a, const SwarConst & C, uint32_t tile, uint32_t chunk )
{
    extern __shared__ uint32_t smem[];
    constexpr int NF = W * NL;
    uint32_t * s_cnt = smem;
    uint32_t * s_u = smem + NF * kDPThreads;
    uint32_t * s_v = smem + 2 * NF * kDPThreads;
    const int tid = threadIdx.x;
    for ( int f = 0; f < NF; ++f ) s_cnt[f * kDPThreads + tid] = s_u[f * kDPThreads + tid] = s_v[f * kDPThreads + tid] = 0;

    const uint32_t gbase = tile * ( kDPThreads * W ) + tid;
    const uint32_t l = a.l, down = 32 - l, e = a.e;
    uint32_t fp[W][B];
#pragma unroll
    for ( int i = 0; i < W; ++i )
    {
#pragma unroll
        for ( int b = 0; b < B; ++b ) fp[i][b] = 0;
        const uint32_t g = gbase + i * kDPThreads;
#pragma unroll
        for ( int j = 0; j < NL; ++j )
        {
            const uint32_t w = g * NL + j;
            if ( w < a.U )
#pragma unroll
                for ( int b = 0; b < B; ++b ) fp[i][b] |= ( __ldg ( a.wplanes32 + ( size_t ) b * a.U + w ) >> down ) << ( j * C.S );
        }
        if constexpr ( E >= 0 ) fp[i][0] |= C.HB;                // guard bits: x has them set
    }
    uint32_t cnt[W];
#pragma unroll
    for ( int i = 0; i < W; ++i ) cnt[i] = 0;

    const ChunkInfo ch = a.chunks[chunk];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;

    auto count = [&] ( int i, const uint32_t ( &Y )[B] ) {
        uint32_t x = fp[i][0] ^ Y[0];
#pragma unroll
        for ( int b = 1; b < B; ++b ) x |= fp[i][b] ^ Y[b];
        if constexpr ( E >= 0 )
        {
#pragma unroll
            for ( int c = 0; c < E; ++c ) x = ( x & ( x * C.ONE + C.K ) ) | C.HB;
            cnt[i] = ( ~( x * C.ONE + C.K ) & C.HB ) * C.ONE + cnt[i];
            if constexpr ( NL == 3 )
                if ( x < C.LIM ) cnt[i] += 1u;
        }
        else
        {
#pragma unroll
            for ( int j = 0; j < NL; ++j )
                if ( __popc ( x & ( C.FM << ( j * C.S ) ) ) <= e ) cnt[i] += 1u << ( j * C.S );
        }
    };
    // the replicated windows of a block (32 positions x B planes) are the same
    // for every thread: built once per CTA into shared memory, double-buffered
    // so that one barrier per block suffices
    __shared__ uint32_t s_win[2][32 * B];
    const uint32_t * win = s_win[0];
    auto window = [&] ( int r, uint32_t ( &Y )[B] ) {
#pragma unroll
        for ( int b = 0; b < B; ++b ) Y[b] = win[b * 32 + r];
    };
    auto drain = [&] () {
#pragma unroll
        for ( int i = 0; i < W; ++i )
        {
#pragma unroll
            for ( int j = 0; j < NL; ++j ) s_cnt[( i * NL + j ) * kDPThreads + tid] += ( cnt[i] >> ( E < 0 ? j * C.S : ( NL == 3 && j == 2 ? 0u : j * C.S + C.Q ) ) ) & C.FM;
            cnt[i] = 0;
        }
    };
    auto end_sequence = [&] () {
        for ( int f = 0; f < NF; ++f )
        {
            const uint32_t c = s_cnt[f * kDPThreads + tid];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[f * kDPThreads + tid] += 1;
            else
            {
                const uint32_t w = ( gbase + ( f / NL ) * kDPThreads ) * NL + ( f % NL );
                if ( w < a.U ) a.split_flags[( size_t ) cur_split * a.U + w] = 1;
            }
            s_v[f * kDPThreads + tid] += c;
            s_cnt[f * kDPThreads + tid] = 0;
        }
    };

    for ( uint32_t k = ch.begin; k < ch.end; ++k )
    {
        {
            uint32_t * w = s_win[( k - ch.begin ) & 1];
            for ( uint32_t i = threadIdx.x; i < 32u * B; i += kDPThreads )
            {
                const uint32_t * pl = planes + ( size_t ) ( i >> 5 ) * stride;
                w[i] = ( __funnelshift_rc ( __ldg ( pl + k ), __ldg ( pl + k + 1 ), ( i & 31u ) + 1 ) >> down ) * C.REP;
            }
            win = w;
            __syncthreads ();
        }
        const uint32_t vm = __ldg ( a.text.vmask + k ), em = __ldg ( a.text.emask + k );
        if ( vm == 0xffffffffu && em == 0u )
        {
#pragma unroll 1
            for ( int g = 0; g < 32; g += UR )
            {
#pragma unroll
                for ( int rr = 0; rr < UR; ++rr )
                {
                    uint32_t Y[B];
                    window ( g + rr, Y );
#pragma unroll
                    for ( int i = 0; i < W; ++i ) count ( i, Y );
                }
            }
        }
        else
        {
            for ( int r = 0; r < 32; ++r )
            {
                if ( ( vm >> r ) & 1u )
                {
                    uint32_t Y[B];
                    window ( r, Y );
#pragma unroll
                    for ( int i = 0; i < W; ++i ) count ( i, Y );
                }
                if ( ( em >> r ) & 1u )
                {
                    drain ();
                    end_sequence ();
                    cur_split = -1;
                }
            }
        }
        drain ();
    }
    for ( int f = 0; f < NF; ++f )
    {
        const uint32_t w = ( gbase + ( f / NL ) * kDPThreads ) * NL + ( f % NL );
        if ( w >= a.U ) continue;
        const uint32_t c = s_cnt[f * kDPThreads + tid];
        uint32_t u = s_u[f * kDPThreads + tid];
        if ( c )
        {
            if ( ch.last_split >= 0 ) a.split_flags[( size_t ) ch.last_split * a.U + w] = 1;
            else u += 1;
        }
        const uint32_t v = s_v[f * kDPThreads + tid] + c;
        if ( u ) atomicAdd ( a.u_acc + w, u );
        if ( v ) atomicAdd ( a.v_acc + w, v );
    }
}

__host__ __device__ constexpr size_t hswar_smem_bytes ( int NL, int W )
{
    return ( size_t ) 3 * W * NL * kDPThreads * sizeof ( uint32_t );
}

} // namespace mtx
