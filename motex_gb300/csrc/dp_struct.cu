// Structured-motif search (two boxes, one gap) of the GB300 engine.
//
// Reference semantics (functions.cc:564-705 Hamming, 773-915 edit distance):
// for pattern position jx (end of box 0 in sequence x) and gap choice k of
// x, and every text position it (end of box 0 in text t) and gap choice l
// of t, the pair counts when box 0 matches at (it, jx) with <= e errors and
// box 1 -- x[jx+S_k+1 .. jx+S_k+b1] -- matches the text box ending at
// p = it+S_l+b1 with <= e1 errors, p inside t.  v[k, jx] counts the (it, l)
// combinations over all texts, u[k, jx] the texts with at least one.
//
// A warp owns 32 consecutive pattern positions P0..P0+31 (box-0 rows, one per
// lane) and the 32+G-1 box-1 rows P0+gmin+b1 .. P0+31+gmax+b1 they need
// (G = gmax-gmin+1 gap choices; lane r runs rows r and r+32).  All lanes walk
// the same text positions.  Box-1 hits are exchanged by two ballots; each
// lane keeps a shift register of its box-0 hits (bit d = hit at p-d), so a
// box-1 hit of row P0+lane+gmin+b1+k at p adds popc(history & bits
// [gmin+b1, gmax+b1]) to v[k, P0+lane] -- all text gap choices at once.
#include "kernels.cuh"

#include <algorithm>
#include <cstdlib>

namespace mtx
{

namespace
{

// Edit-distance column step (Myers/Hyyro, l <= 32); returns the new score.
template <int B>
__device__ __forceinline__ uint32_t ed_step ( const uint32_t ( &w )[B], const uint32_t ( &T )[B], uint32_t & Pv,
                                              uint32_t & Mv, uint32_t sc, uint32_t sh )
{
    uint32_t x = w[0] ^ T[0];
#pragma unroll
    for ( int b = 1; b < B; ++b ) x |= w[b] ^ T[b];
    const uint32_t Eq = ~x;
    const uint32_t Xv = Eq | Mv;
    const uint32_t Xh = ( ( ( Eq & Pv ) + Pv ) ^ Pv ) | Eq;
    uint32_t Ph = Mv | ~( Xh | Pv );
    uint32_t Mh = Pv & Xh;
    sc += ( ( Ph >> sh ) & 1u ) - ( ( Mh >> sh ) & 1u );
    Ph <<= 1;
    Mh <<= 1;
    Pv = Mh | ~( Xv | Ph );
    Mv = Ph & Xv;
    return sc;
}

template <int B>
__device__ __forceinline__ bool hd_hit ( const uint32_t ( &w )[B], const uint32_t ( &Y )[B], uint32_t mask, uint32_t e )
{
    uint32_t x = ( w[0] ^ Y[0] );
#pragma unroll
    for ( int b = 1; b < B; ++b ) x |= w[b] ^ Y[b];
    return __popc ( x & mask ) <= e;
}

// 1 when popc(x & mask) <= e, with ne = -(e+1): the sign bit of a multiply-add
template <int B>
__device__ __forceinline__ uint32_t hd_hitbit ( const uint32_t ( &w )[B], const uint32_t ( &Y )[B], uint32_t mask,
                                                uint32_t one, uint32_t ne )
{
    uint32_t x = ( w[0] ^ Y[0] );
#pragma unroll
    for ( int b = 1; b < B; ++b ) x |= w[b] ^ Y[b];
    return ( __popc ( x & mask ) * one + ne ) >> 31;
}

} // namespace

template <int B, bool ED>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_struct1 ( const StructArgs a )
{
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t G = a.G;
    // per (thread, k): hit count in the current text, texts seen, occurrences
    uint32_t * s_cnt = smem + ( size_t ) threadIdx.x * G * 3;
    uint32_t * s_u = s_cnt + G;
    uint32_t * s_v = s_u + G;
    for ( uint32_t k = 0; k < G; ++k ) s_cnt[k] = s_u[k] = s_v[k] = 0;

    const uint32_t P0 = ( blockIdx.x * ( kDPThreads / 32 ) + warp ) * 32;
    const uint32_t jx = P0 + lane;
    const uint32_t r0 = P0 + a.gmin + a.b1 + lane;               // box-1 rows of this lane
    const uint32_t r1 = r0 + 32;
    const bool has_r1 = lane + 1 < ( int ) G;

    uint32_t w0[B], w1a[B], w1b[B];
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        w0[b] = jx < a.total ? a.wpl0[( size_t ) b * a.total + jx] : 0u;
        w1a[b] = r0 < a.total ? a.wpl1[( size_t ) b * a.total + r0] : 0u;
        w1b[b] = ( has_r1 && r1 < a.total ) ? a.wpl1[( size_t ) b * a.total + r1] : 0u;
    }
    // gap choices k of x whose box 1 stays inside x's sequence
    uint32_t kvalid = 0;
    if ( jx < a.total && a.row_ok[jx] )
    {
        const uint32_t xend = a.row_end[jx];
        for ( uint32_t k = 0; k < G; ++k )
            if ( jx + a.gmin + k + a.b1 < xend ) kvalid |= 1u << k;
    }
    const uint32_t Gmask = G >= 32 ? 0xffffffffu : ( ( 1u << G ) - 1u );
    const uint32_t win = ( ( a.gmax + a.b1 >= 31 ) ? 0xffffffffu : ( ( 2u << ( a.gmax + a.b1 ) ) - 1u ) ) &
                         ~( ( 1u << ( a.gmin + a.b1 ) ) - 1u );

    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;
    const uint32_t l0 = a.l0, l1 = a.l1;
    const uint32_t top0 = l0 >= 32 ? 0xffffffffu : ~( ( 1u << ( 32 - l0 ) ) - 1u );
    const uint32_t top1 = l1 >= 32 ? 0xffffffffu : ~( ( 1u << ( 32 - l1 ) ) - 1u );
    uint32_t hist = 0;
    uint32_t Pv0 = ~0u, Mv0 = 0, sc0 = l0, Pva = ~0u, Mva = 0, sca = l1, Pvb = ~0u, Mvb = 0, scb = l1;

    auto flush = [&] () {
        for ( uint32_t k = 0; k < G; ++k )
        {
            const uint32_t c = s_cnt[k];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[k] += 1;
            else if ( jx < a.total ) a.split_flags[( ( size_t ) cur_split * a.total + jx ) * G + k] = 1;
            s_v[k] += c;
            s_cnt[k] = 0;
        }
    };

    uint32_t prev[B];
#pragma unroll
    for ( int b = 0; b < B; ++b ) prev[b] = __ldg ( planes + ( size_t ) b * stride + ch.warm );
    for ( uint32_t kb = ch.warm; kb < ch.end; ++kb )
    {
        uint32_t cur[B];
#pragma unroll
        for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( planes + ( size_t ) b * stride + kb + 1 );
        const uint32_t vm = __ldg ( a.text.vmask + kb ), em = __ldg ( a.text.emask + kb );
        const bool counting = kb >= ch.begin;
        for ( int r = 0; r < 32; ++r )
        {
            bool h0, ha, hb = false;
            if constexpr ( ED )
            {
                uint32_t T[B];
#pragma unroll
                for ( int b = 0; b < B; ++b ) T[b] = 0u - ( ( cur[b] >> r ) & 1u );
                sc0 = ed_step<B> ( w0, T, Pv0, Mv0, sc0, l0 - 1 );
                sca = ed_step<B> ( w1a, T, Pva, Mva, sca, l1 - 1 );
                if ( has_r1 ) scb = ed_step<B> ( w1b, T, Pvb, Mvb, scb, l1 - 1 );
                h0 = sc0 <= a.e0;
                ha = sca <= a.e1;
                hb = has_r1 && scb <= a.e1;
            }
            else
            {
                uint32_t Y[B];
#pragma unroll
                for ( int b = 0; b < B; ++b ) Y[b] = __funnelshift_rc ( prev[b], cur[b], r + 1 );
                h0 = hd_hit<B> ( w0, Y, top0, a.e0 );
                ha = hd_hit<B> ( w1a, Y, top1, a.e1 );
                hb = has_r1 && hd_hit<B> ( w1b, Y, top1, a.e1 );
            }
            h0 = h0 && ( ( vm >> r ) & 1u );           // box 0 must end a valid match
            hist = ( hist << 1 ) | ( uint32_t ) h0;
            const uint32_t Ha = __ballot_sync ( 0xffffffffu, ha ), Hb = __ballot_sync ( 0xffffffffu, hb );
            if ( counting && ( Ha | Hb ) )
            {
                const uint64_t H = ( ( uint64_t ) Hb << 32 ) | Ha;
                const uint32_t g = ( uint32_t ) ( H >> lane ) & Gmask & kvalid;
                if ( g )
                {
                    const uint32_t c = __popc ( hist & win );
                    if ( c )
                        for ( uint32_t k = 0; k < G; ++k )
                            if ( ( g >> k ) & 1u ) s_cnt[k] += c;
                }
            }
            if ( ( em >> r ) & 1u )
            {
                if ( counting )
                {
                    flush ();
                    cur_split = -1;
                }
                hist = 0;
                Pv0 = Pva = Pvb = ~0u;
                Mv0 = Mva = Mvb = 0;
                sc0 = l0;
                sca = scb = l1;
            }
        }
#pragma unroll
        for ( int b = 0; b < B; ++b ) prev[b] = cur[b];
    }
    // chunk end: the text cut by the boundary records presence in its split row
    for ( uint32_t k = 0; k < G; ++k )
    {
        const uint32_t c = s_cnt[k];
        if ( c )
        {
            if ( ch.last_split >= 0 && jx < a.total )
                a.split_flags[( ( size_t ) ch.last_split * a.total + jx ) * G + k] = 1;
            else
                s_u[k] += 1;
            s_v[k] += c;
        }
        if ( jx < a.total && ( s_u[k] | s_v[k] ) )
        {
            atomicAdd ( a.u_acc + ( size_t ) jx * G + k, s_u[k] );
            atomicAdd ( a.v_acc + ( size_t ) jx * G + k, s_v[k] );
        }
    }
}

/*
 * Hamming, one gap, block by block.  Same ownership as k_dp_struct1 (a warp
 * owns 32 box-0 rows and the 32+G-1 box-1 rows they need), but per block of
 * 32 text positions each lane first forms three hit masks -- its box-0 row
 * (valid ends only) and its two box-1 rows -- with no exchange, and box-0
 * hits join a 64-bit history word (bits 0-31 the previous block, 32-63 this
 * one).  Then one warp-uniform pass visits, in position order, only the
 * positions where some lane's box-1 row hits (OR-reduced over the warp) or
 * a sequence ends: the ballots, the gap window of box-0 ends behind the hit
 * (popc of the history word at gmin+b1 .. gmax+b1 behind it) and the
 * per-structure counts are those of k_dp_struct1; a sequence end flushes
 * and clears the history up to it.
 */
template <int B, bool PK, int GE = -1>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_struct1_hd ( const StructArgs a )
{
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t G = a.G;
    uint32_t * s_cnt = smem + ( size_t ) threadIdx.x * G * 3;
    uint32_t * s_u = s_cnt + G;
    uint32_t * s_v = s_u + G;
    for ( uint32_t k = 0; k < G; ++k ) s_cnt[k] = s_u[k] = s_v[k] = 0;

    const uint32_t P0 = ( blockIdx.x * ( kDPThreads / 32 ) + warp ) * 32;
    const uint32_t jx = P0 + lane;
    const uint32_t r0 = P0 + a.gmin + a.b1 + lane;
    const uint32_t r1 = r0 + 32;
    const bool has_r1 = lane + 1 < ( int ) G;

    uint32_t w0[B], w1a[B], w1b[B];
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        w0[b] = jx < a.total ? a.wpl0[( size_t ) b * a.total + jx] : 0u;
        w1a[b] = r0 < a.total ? a.wpl1[( size_t ) b * a.total + r0] : 0u;
        w1b[b] = ( has_r1 && r1 < a.total ) ? a.wpl1[( size_t ) b * a.total + r1] : 0u;
    }
    uint32_t kvalid = 0;
    if ( jx < a.total && a.row_ok[jx] )
    {
        const uint32_t xend = a.row_end[jx];
        for ( uint32_t k = 0; k < G; ++k )
            if ( jx + a.gmin + k + a.b1 < xend ) kvalid |= 1u << k;
    }
    const uint32_t Gmask = G >= 32 ? 0xffffffffu : ( ( 1u << G ) - 1u );
    const uint32_t lo = a.gmin + a.b1, hi = a.gmax + a.b1;            // hi <= 31 (launch check)
    const uint32_t wmask = hi - lo + 1 >= 32 ? 0xffffffffu : ( ( 1u << ( hi - lo + 1 ) ) - 1u );

    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;
    const uint32_t l0 = a.l0, l1 = a.l1;
    const uint32_t top0 = l0 >= 32 ? 0xffffffffu : ~( ( 1u << ( 32 - l0 ) ) - 1u );
    const uint32_t top1 = l1 >= 32 ? 0xffffffffu : ~( ( 1u << ( 32 - l1 ) ) - 1u );
    const uint32_t full = 0xffffffffu;
    const uint32_t one = a.one, two = a.one << 1, ne0 = a.ne0, ne1 = a.ne1;
    // PK: the three rows as lanes of L = max(l0, l1) <= 10 bits of one register
    // (box 0, row r0, row r1), each factor in the top of its lane; the window's
    // newest L symbols are replicated into the lanes by a multiply
    const uint32_t L = l0 > l1 ? l0 : l1;
    const uint32_t rep3 = 1u | ( 1u << L ) | ( 1u << ( 2 * L ) );
    const uint32_t mA = ( ( 1u << l0 ) - 1u ) << ( L - l0 );
    const uint32_t mB = ( ( 1u << l1 ) - 1u ) << ( 2 * L - l1 );
    const uint32_t mC = ( ( 1u << l1 ) - 1u ) << ( 3 * L - l1 );
    // GE >= 0 (e0 = e1 = GE, l0 + 2 l1 + 3 <= 32): the popc-free form.  The
    // three rows as lanes of l0, l1, l1 bits at o0, o1, o2 with a guard bit
    // above each, the top guard at bit 31; the guards set in the mismatch
    // word by plane 0 of fp; GE times x = (x & (x - L)) | G clears each
    // lane's lowest set bit, and bit g_j of t = x - L is clear exactly when
    // lane j has at most GE mismatches.  The masks take that bit by a funnel
    // shift per position (the multiply by 2^(31-g) moves it to bit 31 on the
    // FMA pipe) and are complemented with the bit reversal after the block.
    const uint32_t go0 = 32 - ( l0 + 2 * l1 + 3 ), go1 = go0 + l0 + 1, go2 = go1 + l1 + 1;
    const uint32_t gG = ( 1u << ( go0 + l0 ) ) | ( 1u << ( go1 + l1 ) ) | ( 1u << ( go2 + l1 ) );
    const uint32_t gnL = 0u - ( ( 1u << go0 ) | ( 1u << go1 ) | ( 1u << go2 ) );
    const uint32_t gsh0 = one << ( 31 - ( go0 + l0 ) ), gsh1 = one << ( 31 - ( go1 + l1 ) );
    uint32_t fp[B];
    if constexpr ( GE >= 0 )
    {
#pragma unroll
        for ( int b = 0; b < B; ++b )
            fp[b] = ( ( w0[b] >> ( 32 - l0 ) ) << go0 ) | ( ( w1a[b] >> ( 32 - l1 ) ) << go1 ) |
                    ( ( w1b[b] >> ( 32 - l1 ) ) << go2 );
        fp[0] |= gG;
    }
    else if constexpr ( PK )
    {
#pragma unroll
        for ( int b = 0; b < B; ++b )
            fp[b] = ( ( w0[b] >> ( 32 - l0 ) ) << ( L - l0 ) ) | ( ( w1a[b] >> ( 32 - l1 ) ) << ( 2 * L - l1 ) ) |
                    ( ( w1b[b] >> ( 32 - l1 ) ) << ( 3 * L - l1 ) );
    }

    auto flush = [&] () {
        for ( uint32_t k = 0; k < G; ++k )
        {
            const uint32_t c = s_cnt[k];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[k] += 1;
            else if ( jx < a.total ) a.split_flags[( ( size_t ) cur_split * a.total + jx ) * G + k] = 1;
            s_v[k] += c;
            s_cnt[k] = 0;
        }
    };

    uint64_t X = 0;
    uint32_t prev[B];
#pragma unroll
    for ( int b = 0; b < B; ++b ) prev[b] = __ldg ( planes + ( size_t ) b * stride + ch.warm );
    // packed form: every thread of the CTA walks the same text positions, so
    // the replicated windows of a block are built once into shared memory
    // (double-buffered: one barrier per block) instead of by every thread
    __shared__ uint32_t s_win[2][32 * B];
    for ( uint32_t kb = ch.warm; kb < ch.end; ++kb )
    {
        uint32_t cur[B];
        const uint32_t * win = s_win[( kb - ch.warm ) & 1];
        if constexpr ( PK || GE >= 0 )
        {
            uint32_t * w = s_win[( kb - ch.warm ) & 1];
            for ( uint32_t i = threadIdx.x; i < 32u * B; i += kDPThreads )
            {
                const uint32_t b = i >> 5, r = i & 31u;
                const uint32_t pw = __ldg ( planes + ( size_t ) b * stride + kb ), cw = __ldg ( planes + ( size_t ) b * stride + kb + 1 );
                const uint32_t W = __funnelshift_rc ( pw, cw, r + 1 );          // newest symbol at bit 31
                if constexpr ( GE >= 0 )
                    w[i] = ( ( W >> ( 32 - l0 ) ) << go0 ) | ( ( W >> ( 32 - l1 ) ) << go1 ) | ( ( W >> ( 32 - l1 ) ) << go2 );
                else
                    w[i] = ( W >> ( 32 - L ) ) * rep3;
            }
            __syncthreads ();
        }
        else
        {
#pragma unroll
            for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( planes + ( size_t ) b * stride + kb + 1 );
        }
        const uint32_t vm = __ldg ( a.text.vmask + kb ), em = __ldg ( a.text.emask + kb );
        const bool counting = kb >= ch.begin;
        // hit masks built in reverse bit order (position r at bit 31-r): the
        // hit is the sign bit of a multiply-add and enters the mask by one
        // funnel shift (m << 1 | bit 31 of the word); one bit reversal per block
        uint32_t m0 = 0, ma = 0, mb = 0;
#pragma unroll 8
        for ( int r = 0; r < 32; ++r )
        {
            uint32_t Y[B];
            if constexpr ( GE >= 0 )
            {
                uint32_t x = 0;
#pragma unroll
                for ( int b = 0; b < B; ++b ) x |= fp[b] ^ win[b * 32 + r];
#pragma unroll
                for ( int c = 0; c < GE; ++c ) x = ( x & ( x * one + gnL ) ) | gG;
                const uint32_t t = x * one + gnL;
                m0 = __funnelshift_l ( t * gsh0, m0, 1 );
                ma = __funnelshift_l ( t * gsh1, ma, 1 );
                mb = __funnelshift_l ( t, mb, 1 );                // lane 2's guard is bit 31
            }
            else if constexpr ( PK )
            {
                uint32_t x = 0;
#pragma unroll
                for ( int b = 0; b < B; ++b ) x |= fp[b] ^ win[b * 32 + r];
                m0 = __funnelshift_l ( __popc ( x & mA ) * one + ne0, m0, 1 );
                ma = __funnelshift_l ( __popc ( x & mB ) * one + ne1, ma, 1 );
                mb = __funnelshift_l ( __popc ( x & mC ) * one + ne1, mb, 1 );
            }
            else
            {
#pragma unroll
                for ( int b = 0; b < B; ++b ) Y[b] = __funnelshift_rc ( prev[b], cur[b], r + 1 );
                m0 = m0 * two + hd_hitbit<B> ( w0, Y, top0, one, ne0 );
                ma = ma * two + hd_hitbit<B> ( w1a, Y, top1, one, ne1 );
                mb = mb * two + hd_hitbit<B> ( w1b, Y, top1, one, ne1 );
            }
        }
        if constexpr ( GE >= 0 )
        {
            m0 = ~m0;                                   // a set guard bit is a miss
            ma = ~ma;
            mb = ~mb;
        }
        m0 = __brev ( m0 );
        ma = __brev ( ma );
        mb = __brev ( mb );
        if ( ! has_r1 ) mb = 0;
        X = ( ( uint64_t ) ( m0 & vm ) << 32 ) | ( X >> 32 );
        // positions where some lane's box-1 row hits: OR over the warp by a
        // shuffle butterfly (the redux form failed the parity tests here)
        uint32_t R = ma | mb;
#pragma unroll
        for ( int o = 16; o; o >>= 1 ) R |= __shfl_xor_sync ( full, R, o );
        if ( ! counting ) R = 0;
        uint32_t E = em;
        while ( R | E )
        {
            const int r = __ffs ( R | E ) - 1;
            const uint32_t bit = 1u << r;
            if ( R & bit )
            {
                const uint32_t Ha = __ballot_sync ( full, ( ma >> r ) & 1u ), Hb = __ballot_sync ( full, ( mb >> r ) & 1u );
                const uint64_t H = ( ( uint64_t ) Hb << 32 ) | Ha;
                const uint32_t g = ( uint32_t ) ( H >> lane ) & Gmask & kvalid;
                if ( g )
                {
                    const uint32_t c = __popc ( ( uint32_t ) ( X >> ( 32 + r - hi ) ) & wmask );
                    if ( c )
                        for ( uint32_t k = 0; k < G; ++k )
                            if ( ( g >> k ) & 1u ) s_cnt[k] += c;
                }
            }
            if ( E & bit )
            {
                if ( counting )
                {
                    flush ();
                    cur_split = -1;
                }
                X &= ~( ( 2ull << ( 32 + r ) ) - 1ull );          // box-0 ends of the finished sequence
            }
            R &= ~bit;
            E &= ~bit;
        }
        if constexpr ( ! PK )
#pragma unroll
            for ( int b = 0; b < B; ++b ) prev[b] = cur[b];
    }
    for ( uint32_t k = 0; k < G; ++k )
    {
        const uint32_t c = s_cnt[k];
        if ( c )
        {
            if ( ch.last_split >= 0 && jx < a.total )
                a.split_flags[( ( size_t ) ch.last_split * a.total + jx ) * G + k] = 1;
            else
                s_u[k] += 1;
            s_v[k] += c;
        }
        if ( jx < a.total && ( s_u[k] | s_v[k] ) )
        {
            atomicAdd ( a.u_acc + ( size_t ) jx * G + k, s_u[k] );
            atomicAdd ( a.v_acc + ( size_t ) jx * G + k, s_v[k] );
        }
    }
}

/*
 * Edit distance with the lane's three rows -- box 0 (length l0) and its two
 * box-1 rows (length b1) -- packed in one 32-bit register: SWAR lanes of
 * different lengths at offsets 0, oB = l0+1, oC = oB+b1+1, a guard bit above
 * each.  The guard invariants of the single-motif SWAR kernel keep the lanes
 * apart; the score of each lane sits in a bit field shifted down by the
 * common s = min(l0, b1) - 1 from the lane's top bit, and the hit test reads
 * each lane's top bit after adding 2^s - (e+1) per field, which needs
 * e + 1 <= 2^s and l - e - 1 < 2^s per lane.
 */
struct HSwarConst
{
    uint32_t HB, NG, NGm1, K, SC0, s;
    uint32_t bitA, bitB, bitC;      // top bit of box 0, row r0, row r1
    uint32_t oB, oC;
    // multipliers (runtime values: multiply-adds issue on the FMA pipe):
    // 1, 2, -1, and -2^(31-p) for the top bit p of each lane, so that
    // (sc * nm + nm) >> 31 = bit p of ~sc
    uint32_t one, two, neg1, nmA, nmB, nmC;
    uint32_t sd;                    // 1: the top lane ends below bit 31 (score update by one shift)
};

bool hswar_shape ( const StructArgs & a, HSwarConst * C )
{
    const uint32_t Ls[3] = { a.l0, a.b1, a.b1 }, es[3] = { a.e0, a.e1, a.e1 };
    const uint32_t oB = a.l0 + 1, oC = oB + a.b1 + 1;
    if ( oC + a.b1 > 32 ) return false;
    const uint32_t s = std::min ( a.l0, a.b1 ) - 1;
    if ( s < 1 || s > 30 ) return false;
    const uint32_t offs[3] = { 0, oB, oC };
    C->HB = C->K = C->SC0 = 0;
    uint32_t guards = 0;
    for ( int i = 0; i < 3; ++i )
    {
        if ( es[i] + 1 > ( 1u << s ) || Ls[i] - es[i] - 1 >= ( 1u << s ) ) return false;
        const uint32_t hb = offs[i] + Ls[i] - 1, f = hb - s;
        C->HB |= 1u << hb;
        if ( offs[i] + Ls[i] < 32 ) guards |= 1u << ( offs[i] + Ls[i] );
        C->K += ( ( 1u << s ) - ( es[i] + 1 ) ) << f;
        C->SC0 += Ls[i] << f;
    }
    C->NG = ~guards;
    C->NGm1 = C->NG & ~C->HB;
    C->s = s;
    C->bitA = 1u << ( a.l0 - 1 );
    C->bitB = 1u << ( oB + a.b1 - 1 );
    C->bitC = 1u << ( oC + a.b1 - 1 );
    C->oB = oB;
    C->oC = oC;
    C->one = 1u;
    C->two = 2u;
    C->neg1 = ~0u;
    C->nmA = 0u - ( 1u << ( 31 - ( a.l0 - 1 ) ) );
    C->nmB = 0u - ( 1u << ( 31 - ( oB + a.b1 - 1 ) ) );
    C->nmC = 0u - ( 1u << ( 31 - ( oC + a.b1 - 1 ) ) );
    C->sd = oC + a.b1 - 1 <= 30;
    return true;
}

template <int B>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_struct1_swar ( const StructArgs a, const HSwarConst C )
{
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t G = a.G;
    uint32_t * s_cnt = smem + ( size_t ) threadIdx.x * G * 3;
    uint32_t * s_u = s_cnt + G;
    uint32_t * s_v = s_u + G;
    for ( uint32_t k = 0; k < G; ++k ) s_cnt[k] = s_u[k] = s_v[k] = 0;

    const uint32_t P0 = ( blockIdx.x * ( kDPThreads / 32 ) + warp ) * 32;
    const uint32_t jx = P0 + lane;
    const uint32_t r0 = P0 + a.gmin + a.b1 + lane;
    const uint32_t r1 = r0 + 32;
    const bool has_r1 = lane + 1 < ( int ) G;
    uint32_t w[B];
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        const uint32_t x0 = jx < a.total ? a.wpl0[( size_t ) b * a.total + jx] : 0u;
        const uint32_t x1 = r0 < a.total ? a.wpl1[( size_t ) b * a.total + r0] : 0u;
        const uint32_t x2 = ( has_r1 && r1 < a.total ) ? a.wpl1[( size_t ) b * a.total + r1] : 0u;
        w[b] = x0 | ( x1 << C.oB ) | ( x2 << C.oC );
    }
    uint32_t kvalid = 0;
    if ( jx < a.total && a.row_ok[jx] )
    {
        const uint32_t xend = a.row_end[jx];
        for ( uint32_t k = 0; k < G; ++k )
            if ( jx + a.gmin + k + a.b1 < xend ) kvalid |= 1u << k;
    }
    const uint32_t Gmask = G >= 32 ? 0xffffffffu : ( ( 1u << G ) - 1u );
    const uint32_t win = ( ( a.gmax + a.b1 >= 31 ) ? 0xffffffffu : ( ( 2u << ( a.gmax + a.b1 ) ) - 1u ) ) &
                         ~( ( 1u << ( a.gmin + a.b1 ) ) - 1u );
    const uint32_t bitC = has_r1 ? C.bitC : 0u;
    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;
    const uint32_t sh = C.s;
    uint32_t hist = 0, Pv = C.NG, Mv = 0, sc = C.SC0;

    auto flush = [&] () {
        for ( uint32_t k = 0; k < G; ++k )
        {
            const uint32_t c = s_cnt[k];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[k] += 1;
            else if ( jx < a.total ) a.split_flags[( ( size_t ) cur_split * a.total + jx ) * G + k] = 1;
            s_v[k] += c;
            s_cnt[k] = 0;
        }
    };

    for ( uint32_t kb = ch.warm; kb < ch.end; ++kb )
    {
        uint32_t cur[B];
#pragma unroll
        for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( planes + ( size_t ) b * stride + kb + 1 );
        const uint32_t vm = __ldg ( a.text.vmask + kb ), em = __ldg ( a.text.emask + kb );
        const bool counting = kb >= ch.begin;
#pragma unroll 4
        for ( int r = 0; r < 32; ++r )
        {
            uint32_t x = 0;
#pragma unroll
            for ( int b = 0; b < B; ++b ) x |= w[b] ^ ( ( 0u - ( ( cur[b] >> r ) & 1u ) ) & C.NG );
            const uint32_t Xv = ~x | Mv;
            const uint32_t s1 = ( ~x & Pv ) + Pv;
            const uint32_t Xh = ( s1 ^ Pv ) | ~x;
            const uint32_t Ph = Mv | ~( Xh | Pv );
            const uint32_t Mhs = Pv & Xh & C.NGm1;
            const uint32_t mh = Pv & Xh & C.HB;
            const uint32_t ph = Ph & C.HB;
            sc = sc + ( ph >> sh ) - ( mh >> sh );
            const uint32_t Ph2 = Ph << 1, Mh2 = Mhs << 1;
            Pv = Mh2 | ~( Xv | Ph2 );
            Mv = Ph2 & Xv & C.NG;
            const uint32_t hits = ~( sc + C.K ) & C.HB;
            const bool h0 = ( hits & C.bitA ) && ( ( vm >> r ) & 1u );
            hist = ( hist << 1 ) | ( uint32_t ) h0;
            const uint32_t Ha = __ballot_sync ( 0xffffffffu, hits & C.bitB );
            const uint32_t Hb = __ballot_sync ( 0xffffffffu, hits & bitC );
            if ( counting && ( Ha | Hb ) )
            {
                const uint64_t H = ( ( uint64_t ) Hb << 32 ) | Ha;
                const uint32_t g = ( uint32_t ) ( H >> lane ) & Gmask & kvalid;
                if ( g )
                {
                    const uint32_t c = __popc ( hist & win );
                    if ( c )
                        for ( uint32_t k = 0; k < G; ++k )
                            if ( ( g >> k ) & 1u ) s_cnt[k] += c;
                }
            }
            if ( ( em >> r ) & 1u )
            {
                if ( counting )
                {
                    flush ();
                    cur_split = -1;
                }
                hist = 0;
                Pv = C.NG;
                Mv = 0;
                sc = C.SC0;
            }
        }
    }
    for ( uint32_t k = 0; k < G; ++k )
    {
        const uint32_t c = s_cnt[k];
        if ( c )
        {
            if ( ch.last_split >= 0 && jx < a.total )
                a.split_flags[( ( size_t ) ch.last_split * a.total + jx ) * G + k] = 1;
            else
                s_u[k] += 1;
            s_v[k] += c;
        }
        if ( jx < a.total && ( s_u[k] | s_v[k] ) )
        {
            atomicAdd ( a.u_acc + ( size_t ) jx * G + k, s_u[k] );
            atomicAdd ( a.v_acc + ( size_t ) jx * G + k, s_v[k] );
        }
    }
}

/*
 * Packed edit distance (as k_dp_struct1_swar), block by block like
 * k_dp_struct1_hd: phase 1 runs the packed Myers step over the 32 positions
 * of a block, with Eq read from a per-thread table by symbol code (shared
 * memory after the counters), and appends each lane's hit bit to its mask (box 0, row r0,
 * row r1; the lanes' top bits are ordered, so one shift and one funnel shift
 * append each), with the Myers state reset at sequence ends; phase 2 visits
 * only the positions where a box-1 row hits or a sequence ends.
 */
template <int B, bool SD>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_struct1_swar_blk ( const StructArgs a, const HSwarConst C )
{
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t G = a.G;
    uint32_t * s_cnt = smem + ( size_t ) threadIdx.x * G * 3;
    uint32_t * s_u = s_cnt + G;
    uint32_t * s_v = s_u + G;
    for ( uint32_t k = 0; k < G; ++k ) s_cnt[k] = s_u[k] = s_v[k] = 0;

    const uint32_t P0 = ( blockIdx.x * ( kDPThreads / 32 ) + warp ) * 32;
    const uint32_t jx = P0 + lane;
    const uint32_t r0 = P0 + a.gmin + a.b1 + lane;
    const uint32_t r1 = r0 + 32;
    const bool has_r1 = lane + 1 < ( int ) G;
    uint32_t w[B];
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        const uint32_t x0 = jx < a.total ? a.wpl0[( size_t ) b * a.total + jx] : 0u;
        const uint32_t x1 = r0 < a.total ? a.wpl1[( size_t ) b * a.total + r0] : 0u;
        const uint32_t x2 = ( has_r1 && r1 < a.total ) ? a.wpl1[( size_t ) b * a.total + r1] : 0u;
        w[b] = x0 | ( x1 << C.oB ) | ( x2 << C.oC );
    }
    // Myers Eq of the packed register against every symbol code (text bits
    // cleared at the guards, so Eq is 1 there): one shared load per position
    uint32_t * s_eq = smem + ( size_t ) kDPThreads * G * 3;          // [code][thread]
    for ( int c = 0; c < ( 1 << B ); ++c )
    {
        uint32_t x = 0;
#pragma unroll
        for ( int b = 0; b < B; ++b ) x |= w[b] ^ ( ( ( c >> b ) & 1 ) ? C.NG : 0u );
        s_eq[c * kDPThreads + threadIdx.x] = ~x;
    }
    uint32_t kvalid = 0;
    if ( jx < a.total && a.row_ok[jx] )
    {
        const uint32_t xend = a.row_end[jx];
        for ( uint32_t k = 0; k < G; ++k )
            if ( jx + a.gmin + k + a.b1 < xend ) kvalid |= 1u << k;
    }
    const uint32_t Gmask = G >= 32 ? 0xffffffffu : ( ( 1u << G ) - 1u );
    const uint32_t lo = a.gmin + a.b1, hi = a.gmax + a.b1;            // hi <= 31 (launch check)
    const uint32_t wmask = hi - lo + 1 >= 32 ? 0xffffffffu : ( ( 1u << ( hi - lo + 1 ) ) - 1u );
    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;
    const uint32_t sh = C.s;
    const uint32_t full = 0xffffffffu;
    uint32_t Pv = C.NG, Mv = 0, sc = C.SC0 + C.K;          // score + K per field
    uint64_t X = 0;

    auto flush = [&] () {
        for ( uint32_t k = 0; k < G; ++k )
        {
            const uint32_t c = s_cnt[k];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[k] += 1;
            else if ( jx < a.total ) a.split_flags[( ( size_t ) cur_split * a.total + jx ) * G + k] = 1;
            s_v[k] += c;
            s_cnt[k] = 0;
        }
    };

    // every thread walks the same text positions: each warp computes the
    // Eq-table row offset of each position of a block once (lane r takes
    // position r) into its own shared buffer (double-buffered: one warp
    // barrier per block) instead of every thread computing all of them
    __shared__ uint32_t s_row[kDPThreads / 32][2][32];
    const uint32_t * my_eq = s_eq + threadIdx.x;
    for ( uint32_t kb = ch.warm; kb < ch.end; ++kb )
    {
        uint32_t * rows = s_row[warp][( kb - ch.warm ) & 1];
        {
            uint32_t c = 0;
#pragma unroll
            for ( int b = 0; b < B; ++b ) c |= ( ( __ldg ( planes + ( size_t ) b * stride + kb + 1 ) >> lane ) & 1u ) << b;
            rows[lane] = c * kDPThreads;
        }
        __syncwarp ();
        const uint32_t vm = __ldg ( a.text.vmask + kb ), em = __ldg ( a.text.emask + kb );
        const bool counting = kb >= ch.begin;
        // hit masks built in reverse bit order (position r at bit 31-r): adds
        // and left shifts are multiply-adds (FMA pipe), each row's hit bit the
        // sign of a multiply-add, appended by one funnel shift
        uint32_t m0 = 0, ma = 0, mb = 0;
        auto step = [&] ( int r ) {
            const uint32_t Eq = my_eq[rows[r]];
            const uint32_t Xv = Eq | Mv;
            const uint32_t s1 = ( Eq & Pv ) * C.one + Pv;
            const uint32_t Xh = ( s1 ^ Pv ) | Eq;
            const uint32_t Ph = Mv | ~( Xh | Pv );
            const uint32_t Mhs = Pv & Xh & C.NGm1;
            const uint32_t mh = Pv & Xh & C.HB;
            const uint32_t ph = Ph & C.HB;
            if constexpr ( SD )
            {
                // ph, mh disjoint with the top bit below 31: ph - mh is exact
                // as a signed word, one arithmetic shift moves every lane's
                // +1 / 0 / -1 to its score field
                const int32_t d = ( int32_t ) ( mh * C.neg1 + ph );
                sc = ( uint32_t ) ( d >> sh ) * C.one + sc;
            }
            else
            {
                sc = ( ph >> sh ) * C.one + sc;
                sc = ( mh >> sh ) * C.neg1 + sc;
            }
            const uint32_t Ph2 = Ph * C.two, Mh2 = Mhs * C.two;
            Pv = Mh2 | ~( Xv | Ph2 );
            Mv = Ph2 & Xv & C.NG;
            m0 = __funnelshift_l ( sc * C.nmA + C.nmA, m0, 1 );
            ma = __funnelshift_l ( sc * C.nmB + C.nmB, ma, 1 );
            mb = __funnelshift_l ( sc * C.nmC + C.nmC, mb, 1 );
        };
        if ( em == 0u )
        {
#pragma unroll 4
            for ( int r = 0; r < 32; ++r ) step ( r );
        }
        else
        {
#pragma unroll 4
            for ( int r = 0; r < 32; ++r )
            {
                step ( r );
                if ( ( em >> r ) & 1u )
                {
                    Pv = C.NG;
                    Mv = 0;
                    sc = C.SC0 + C.K;
                }
            }
        }
        m0 = __brev ( m0 );
        ma = __brev ( ma );
        mb = __brev ( mb );
        if ( ! has_r1 ) mb = 0;
        X = ( ( uint64_t ) ( m0 & vm ) << 32 ) | ( X >> 32 );
        uint32_t R = ma | mb;
#pragma unroll
        for ( int o = 16; o; o >>= 1 ) R |= __shfl_xor_sync ( full, R, o );
        if ( ! counting ) R = 0;
        uint32_t E = em;
        while ( R | E )
        {
            const int r = __ffs ( R | E ) - 1;
            const uint32_t bit = 1u << r;
            if ( R & bit )
            {
                const uint32_t Ha = __ballot_sync ( full, ( ma >> r ) & 1u ), Hb = __ballot_sync ( full, ( mb >> r ) & 1u );
                const uint64_t H = ( ( uint64_t ) Hb << 32 ) | Ha;
                const uint32_t g = ( uint32_t ) ( H >> lane ) & Gmask & kvalid;
                if ( g )
                {
                    const uint32_t c = __popc ( ( uint32_t ) ( X >> ( 32 + r - hi ) ) & wmask );
                    if ( c )
                        for ( uint32_t k = 0; k < G; ++k )
                            if ( ( g >> k ) & 1u ) s_cnt[k] += c;
                }
            }
            if ( E & bit )
            {
                if ( counting )
                {
                    flush ();
                    cur_split = -1;
                }
                X &= ~( ( 2ull << ( 32 + r ) ) - 1ull );
            }
            R &= ~bit;
            E &= ~bit;
        }
    }
    for ( uint32_t k = 0; k < G; ++k )
    {
        const uint32_t c = s_cnt[k];
        if ( c )
        {
            if ( ch.last_split >= 0 && jx < a.total )
                a.split_flags[( ( size_t ) ch.last_split * a.total + jx ) * G + k] = 1;
            else
                s_u[k] += 1;
            s_v[k] += c;
        }
        if ( jx < a.total && ( s_u[k] | s_v[k] ) )
        {
            atomicAdd ( a.u_acc + ( size_t ) jx * G + k, s_u[k] );
            atomicAdd ( a.v_acc + ( size_t ) jx * G + k, s_v[k] );
        }
    }
}

template <int B>
static void launch_struct_b ( const StructArgs & a, bool ed, dim3 grid, size_t smem, cudaStream_t st )
{
    HSwarConst C;
    const bool block = ! getenv ( "MOTEX_STRUCT_NO_BLOCK" );
    if ( ed && ! getenv ( "MOTEX_STRUCT_NO_SWAR" ) && hswar_shape ( a, &C ) )
    {
        if ( block )
        {
            // + the per-thread Eq table of the block kernel
            const size_t smem_t = smem + ( size_t ) ( 1 << B ) * kDPThreads * sizeof ( uint32_t );
            auto kern = C.sd ? k_dp_struct1_swar_blk<B, true> : k_dp_struct1_swar_blk<B, false>;
            cudaFuncSetAttribute ( kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem_t );
            kern<<<grid, kDPThreads, smem_t, st>>> ( a, C );
        }
        else k_dp_struct1_swar<B><<<grid, kDPThreads, smem, st>>> ( a, C );
    }
    else if ( ed )
        k_dp_struct1<B, true><<<grid, kDPThreads, smem, st>>> ( a );
    else if ( block && a.e0 == a.e1 && a.e0 <= 3 && a.l0 + 2 * a.l1 + 3 <= 32 && ! getenv ( "MOTEX_STRUCT_NO_PACK" ) &&
              ! getenv ( "MOTEX_STRUCT_NO_CLEAR" ) )
    {
        // popc-free guarded lanes (equal errors in both boxes)
        switch ( a.e0 )
        {
            case 0: k_dp_struct1_hd<B, true, 0><<<grid, kDPThreads, smem, st>>> ( a ); break;
            case 1: k_dp_struct1_hd<B, true, 1><<<grid, kDPThreads, smem, st>>> ( a ); break;
            case 2: k_dp_struct1_hd<B, true, 2><<<grid, kDPThreads, smem, st>>> ( a ); break;
            default: k_dp_struct1_hd<B, true, 3><<<grid, kDPThreads, smem, st>>> ( a ); break;
        }
    }
    else if ( block && 3 * std::max ( a.l0, a.l1 ) <= 32 && ! getenv ( "MOTEX_STRUCT_NO_PACK" ) )
        k_dp_struct1_hd<B, true><<<grid, kDPThreads, smem, st>>> ( a );
    else if ( block )
        k_dp_struct1_hd<B, false><<<grid, kDPThreads, smem, st>>> ( a );
    else
        k_dp_struct1<B, false><<<grid, kDPThreads, smem, st>>> ( a );
}

bool launch_dp_struct1 ( const StructArgs & a, int B, bool ed, dim3 grid, cudaStream_t st )
{
    if ( a.l0 < 1 || a.l0 > 32 || a.l1 < 1 || a.l1 > 32 || a.G < 1 || a.G > 32 ) return false;
    if ( a.gmax + a.b1 > 31 ) return false;
    const size_t smem = ( size_t ) kDPThreads * a.G * 3 * sizeof ( uint32_t );
    if ( smem > 48 * 1024 ) return false;
    switch ( B )
    {
        case 1:
        case 2: launch_struct_b<2> ( a, ed, grid, smem, st ); return true;
        case 3: launch_struct_b<3> ( a, ed, grid, smem, st ); return true;
        case 4: launch_struct_b<4> ( a, ed, grid, smem, st ); return true;
        case 5: launch_struct_b<5> ( a, ed, grid, smem, st ); return true;
        default: return false;
    }
}

// Bit planes of the factor of length l ending at every position (zero where
// it would start before position 0); top-aligned for Hamming.
__global__ void k_wplanes_all ( const uint8_t * __restrict__ codes, uint32_t total, uint32_t l, uint32_t B,
                                int top_aligned, uint32_t * __restrict__ out )
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if ( pos >= total ) return;
    uint32_t pl[kMaxPlanes] = { 0, 0, 0, 0, 0 };
    if ( pos + 1 >= l )
        for ( uint32_t q = 0; q < l; ++q )
        {
            const uint32_t c = codes[pos + 1 - l + q];
            const uint32_t bit = top_aligned ? ( 32 - l + q ) : q;
#pragma unroll
            for ( int b = 0; b < kMaxPlanes; ++b ) pl[b] |= ( ( c >> b ) & 1u ) << bit;
        }
    for ( uint32_t b = 0; b < B; ++b ) out[( size_t ) b * total + pos] = pl[b];
}

// Row bookkeeping of the pattern side: row_ok = box 0 may end here (sequence
// long enough, full box inside it), row_end = end offset of its sequence.
__global__ void k_struct_rows ( const uint32_t * __restrict__ offs, uint32_t nseq, uint64_t total, uint32_t l0,
                                uint32_t tml, uint32_t npat, uint8_t * row_ok, uint32_t * row_end )
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if ( pos >= total ) return;
    uint32_t lo = 0, hi = nseq;
    while ( hi - lo > 1 )
    {
        const uint32_t mid = ( lo + hi ) >> 1;
        if ( offs[mid] <= pos ) lo = mid; else hi = mid;
    }
    while ( offs[lo + 1] <= pos ) ++lo;
    const uint32_t start = offs[lo], end = offs[lo + 1];
    row_end[pos] = end;
    row_ok[pos] = ( end - start ) >= tml && pos - start + 1 >= l0 && ( npat == 0 || lo < npat );
}

/*
 * Per (position, gap choice): add split-row presence, apply the quorum
 * filter and mark passing entries (pattern side of whole-set runs), or copy
 * totals out (pair mode).
 */
__global__ void k_struct_finalize ( StructFinalizeArgs a )
{
    const uint64_t i = ( uint64_t ) blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= a.n ) return;
    uint32_t u = a.u_acc[i];
    for ( uint32_t s = 0; s < a.n_split; ++s ) u += a.split_flags[( size_t ) s * a.n + i];
    const uint32_t v = a.v_acc[i];
    if ( a.u_out ) { a.u_out[i] = u; a.v_out[i] = v; return; }
    a.mark[i] = ( u >= 1 && u <= a.nseq && a.qok[u] && v >= a.nmin && v <= a.nmax ) ? 1 : 0;
    a.rec_u[i] = u;
    a.rec_v[i] = v;
}

} // namespace mtx

// ===================================================================== N gaps
//
// Structured motifs with any number of gaps (functions.cc:647-690 merge loop).
// One thread per pattern position jx runs the box-0 DP over the text chunk.
// On a box-0 hit at text position it, it enumerates every pattern structure
// k and text structure l like the reference's merge: box g+1 of the pattern
// ends at jx + xoff[k][g], the text box at it + xoff[l][g] (cumulative gap +
// box lengths), and both must lie inside their sequences.  Later boxes are
// checked directly at that end position: Hamming compares one window of the
// text bit planes with the box factor's planes; edit distance reruns the
// Myers column over the last l_b + e_b text symbols (a restart that far back
// is exact for the <= e_b test) or from the sequence start.  Word is the
// row width: 32-bit rows for boxes of at most 32 symbols, 64-bit rows
// (wpl64) when a box is longer, up to 64.

namespace mtx
{

namespace
{

template <typename Word>
struct WordBits;
template <>
struct WordBits<uint32_t>
{
    static constexpr uint32_t value = 32;
    __device__ static uint32_t popc ( uint32_t x ) { return __popc ( x ); }
};
template <>
struct WordBits<unsigned long long>
{
    static constexpr uint32_t value = 64;
    __device__ static uint32_t popc ( unsigned long long x ) { return __popcll ( x ); }
};

// The window of text symbols ending at position p, p at the top bit, from
// the plane words of the blocks (word k + 1 of a plane holds block k).
template <int B, typename Word>
__device__ __forceinline__ void text_window ( const TextView & tv, uint32_t p, Word ( &Y )[B] )
{
    const uint32_t blk = p >> 5, r = p & 31u;
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        const uint32_t * pl = tv.planes + ( size_t ) b * tv.plane_stride;
        const uint32_t cur = __ldg ( pl + blk + 1 ), prev = __ldg ( pl + blk );
        if constexpr ( WordBits<Word>::value == 32 )
            Y[b] = __funnelshift_rc ( prev, cur, r + 1 );
        else
        {
            const unsigned long long pp = blk >= 1 ? __ldg ( pl + blk - 1 ) : 0u;
            const unsigned long long lo = ( ( unsigned long long ) prev << 32 ) | pp;
            Y[b] = ( lo >> ( r + 1 ) ) | ( ( unsigned long long ) cur << ( 63 - r ) );
        }
    }
}

template <typename Word>
__device__ __forceinline__ Word top_mask ( uint32_t l )
{
    constexpr uint32_t BITS = WordBits<Word>::value;
    return l >= BITS ? ~( Word ) 0 : ~( ( ( Word ) 1 << ( BITS - l ) ) - 1 );
}

// Box planes of the factor ending at pattern position q.
template <int B, typename Word>
__device__ __forceinline__ void box_planes ( const StructNArgs & a, int box, uint32_t q, Word ( &w )[B] )
{
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        if constexpr ( WordBits<Word>::value == 32 )
            w[b] = __ldg ( a.wpl + ( ( size_t ) box * B + b ) * a.total + q );
        else
            w[b] = __ldg ( a.wpl64 + ( ( size_t ) box * B + b ) * a.total + q );
    }
}

template <int B, bool ED, typename Word>
__device__ bool box_hit ( const StructNArgs & a, int box, uint32_t q, uint32_t p, uint32_t tstart )
{
    const uint32_t lb = a.blen[box], eb = a.berr[box];
    Word w[B];
    box_planes<B, Word> ( a, box, q, w );
    if constexpr ( ! ED )
    {
        Word Y[B];
        text_window<B, Word> ( a.text, p, Y );
        Word x = w[0] ^ Y[0];
#pragma unroll
        for ( int b = 1; b < B; ++b ) x |= w[b] ^ Y[b];
        return WordBits<Word>::popc ( x & top_mask<Word> ( lb ) ) <= eb;
    }
    else
    {
        const uint32_t back = lb + eb - 1;
        const uint32_t s0 = ( p >= tstart + back ) ? p - back : tstart;
        Word Pv = ~( Word ) 0, Mv = 0;
        uint32_t sc = lb;
        const uint32_t sh = lb - 1;
        for ( uint32_t r = s0; r <= p; ++r )
        {
            const uint32_t blk = ( r >> 5 ) + 1, bit = r & 31u;
            Word x = 0;
#pragma unroll
            for ( int b = 0; b < B; ++b )
            {
                const Word T = ( Word ) 0 - ( Word ) ( ( __ldg ( a.text.planes + ( size_t ) b * a.text.plane_stride + blk ) >> bit ) & 1u );
                x |= w[b] ^ T;
            }
            const Word Eq = ~x;
            const Word Xv = Eq | Mv;
            const Word Xh = ( ( ( Eq & Pv ) + Pv ) ^ Pv ) | Eq;
            Word Ph = Mv | ~( Xh | Pv );
            Word Mh = Pv & Xh;
            sc += ( uint32_t ) ( ( Ph >> sh ) & 1u ) - ( uint32_t ) ( ( Mh >> sh ) & 1u );
            Ph <<= 1;
            Mh <<= 1;
            Pv = Mh | ~( Xv | Ph );
            Mv = Ph & Xv;
        }
        return sc <= eb;
    }
}

} // namespace

template <int B, bool ED, typename Word>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_structN ( const StructNArgs a )
{
    extern __shared__ uint32_t smem[];
    const uint32_t NS = a.nstructs, NG = a.ngaps;
    uint32_t * s_off = smem;                                        // NS * NG cumulative offsets
    uint32_t * s_cnt = smem + NS * NG + threadIdx.x;                // [k * kDPThreads + tid]
    uint32_t * s_u = s_cnt + NS * kDPThreads;
    uint32_t * s_v = s_u + NS * kDPThreads;
    for ( uint32_t i = threadIdx.x; i < NS * NG; i += kDPThreads ) s_off[i] = a.xoff[i];
    for ( uint32_t k = 0; k < NS; ++k ) s_cnt[k * kDPThreads] = s_u[k * kDPThreads] = s_v[k * kDPThreads] = 0;
    __syncthreads ();

    const uint32_t jx = blockIdx.x * kDPThreads + threadIdx.x;
    const bool row = jx < a.total && a.row_ok[jx];
    const uint32_t xend = jx < a.total ? a.row_end[jx] : 0;
    Word w0[B];
    if ( jx < a.total ) box_planes<B, Word> ( a, 0, jx, w0 );
    else
#pragma unroll
        for ( int b = 0; b < B; ++b ) w0[b] = 0;
    const uint32_t l0 = a.l0;
    const Word top0 = top_mask<Word> ( l0 );
    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    Word Pv = ~( Word ) 0, Mv = 0;
    uint32_t sc = l0;
    uint32_t tstart = 0;                                            // start of the current text sequence
    bool tstart_known = false;
    // plane words of the two blocks before the current one (Hamming windows)
    uint32_t prev[B], pp[B];
#pragma unroll
    for ( int b = 0; b < B; ++b )
    {
        prev[b] = __ldg ( a.text.planes + ( size_t ) b * a.text.plane_stride + ch.warm );
        pp[b] = ch.warm >= 1 ? __ldg ( a.text.planes + ( size_t ) b * a.text.plane_stride + ch.warm - 1 ) : 0u;
    }

    auto flush = [&] () {
        for ( uint32_t k = 0; k < NS; ++k )
        {
            const uint32_t c = s_cnt[k * kDPThreads];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[k * kDPThreads] += 1;
            else if ( jx < a.total ) a.split_flags[( ( size_t ) cur_split * a.total + jx ) * NS + k] = 1;
            s_v[k * kDPThreads] += c;
            s_cnt[k * kDPThreads] = 0;
        }
    };

    for ( uint32_t kb = ch.warm; kb < ch.end; ++kb )
    {
        uint32_t cur[B];
#pragma unroll
        for ( int b = 0; b < B; ++b ) cur[b] = __ldg ( a.text.planes + ( size_t ) b * a.text.plane_stride + kb + 1 );
        const uint32_t vm = __ldg ( a.text.vmask + kb ), em = __ldg ( a.text.emask + kb );
        const bool counting = kb >= ch.begin;
        for ( int r = 0; r < 32; ++r )
        {
            const uint32_t it = kb * 32 + r;
            bool h0;
            if constexpr ( ED )
            {
                Word x = 0;
#pragma unroll
                for ( int b = 0; b < B; ++b ) x |= w0[b] ^ ( ( Word ) 0 - ( Word ) ( ( cur[b] >> r ) & 1u ) );
                const Word Eq = ~x;
                const Word Xv = Eq | Mv;
                const Word Xh = ( ( ( Eq & Pv ) + Pv ) ^ Pv ) | Eq;
                Word Ph = Mv | ~( Xh | Pv );
                Word Mh = Pv & Xh;
                sc += ( uint32_t ) ( ( Ph >> ( l0 - 1 ) ) & 1u ) - ( uint32_t ) ( ( Mh >> ( l0 - 1 ) ) & 1u );
                Ph <<= 1;
                Mh <<= 1;
                Pv = Mh | ~( Xv | Ph );
                Mv = Ph & Xv;
                h0 = sc <= a.e0;
            }
            else
            {
                Word x = 0;
#pragma unroll
                for ( int b = 0; b < B; ++b )
                {
                    Word Y;
                    if constexpr ( WordBits<Word>::value == 32 ) Y = __funnelshift_rc ( prev[b], cur[b], r + 1 );
                    else
                        Y = ( ( ( ( unsigned long long ) prev[b] << 32 ) | pp[b] ) >> ( r + 1 ) ) |
                            ( ( unsigned long long ) cur[b] << ( 63 - r ) );
                    x |= w0[b] ^ Y;
                }
                h0 = WordBits<Word>::popc ( x & top0 ) <= a.e0;
            }
            if ( row && counting && h0 && ( ( vm >> r ) & 1u ) )
            {
                if ( ! tstart_known )
                {
                    tstart = a.seq_start[it];                   // once per text sequence and chunk
                    tstart_known = true;
                }
                const uint32_t tend = a.row_end[it];
                for ( uint32_t k = 0; k < NS; ++k )
                {
                    if ( jx + s_off[k * NG + NG - 1] >= xend ) continue;      // x structure must fit
                    for ( uint32_t l = 0; l < NS; ++l )
                    {
                        bool ok = true;
                        for ( uint32_t g = 0; g < NG && ok; ++g )
                        {
                            const uint32_t q = jx + s_off[k * NG + g], p = it + s_off[l * NG + g];
                            ok = p < tend && box_hit<B, ED, Word> ( a, ( int ) g + 1, q, p, tstart );
                        }
                        if ( ok ) s_cnt[k * kDPThreads] += 1;
                    }
                }
            }
            if ( ( em >> r ) & 1u )
            {
                if ( counting )
                {
                    flush ();
                    cur_split = -1;
                }
                Pv = ~( Word ) 0;
                Mv = 0;
                sc = l0;
                tstart_known = false;
            }
        }
#pragma unroll
        for ( int b = 0; b < B; ++b )
        {
            pp[b] = prev[b];
            prev[b] = cur[b];
        }
    }
    for ( uint32_t k = 0; k < NS; ++k )
    {
        const uint32_t c = s_cnt[k * kDPThreads];
        uint32_t u = s_u[k * kDPThreads];
        if ( c )
        {
            if ( ch.last_split >= 0 && jx < a.total )
                a.split_flags[( ( size_t ) ch.last_split * a.total + jx ) * NS + k] = 1;
            else
                u += 1;
        }
        const uint32_t v = s_v[k * kDPThreads] + c;
        if ( jx < a.total && ( u | v ) )
        {
            atomicAdd ( a.u_acc + ( size_t ) jx * NS + k, u );
            atomicAdd ( a.v_acc + ( size_t ) jx * NS + k, v );
        }
    }
}

size_t structN_smem_bytes ( const StructNArgs & a )
{
    return ( ( size_t ) a.nstructs * a.ngaps + ( size_t ) 3 * a.nstructs * kDPThreads ) * sizeof ( uint32_t );
}

namespace
{

template <int B, bool ED, typename Word>
bool launch_structN_k ( const StructNArgs & a, dim3 grid, cudaStream_t st )
{
    const size_t smem = structN_smem_bytes ( a );
    if ( cudaFuncSetAttribute ( k_dp_structN<B, ED, Word>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem ) !=
         cudaSuccess )
        return false;
    k_dp_structN<B, ED, Word><<<grid, kDPThreads, smem, st>>> ( a );
    return true;
}

template <int B>
bool launch_structN_b ( const StructNArgs & a, bool ed, bool wide, dim3 grid, cudaStream_t st )
{
    if ( wide )
        return ed ? launch_structN_k<B, true, unsigned long long> ( a, grid, st )
                  : launch_structN_k<B, false, unsigned long long> ( a, grid, st );
    return ed ? launch_structN_k<B, true, uint32_t> ( a, grid, st ) : launch_structN_k<B, false, uint32_t> ( a, grid, st );
}

} // namespace

bool launch_dp_structN ( const StructNArgs & a, int B, bool ed, dim3 grid, cudaStream_t st )
{
    if ( a.nstructs < 1 || a.nstructs > kMaxStructsN || a.ngaps < 1 || a.ngaps > kMaxGapsN ) return false;
    if ( structN_smem_bytes ( a ) > kStructNMaxSmem ) return false;
    uint32_t maxlen = 0;
    for ( uint32_t g = 0; g <= a.ngaps; ++g )
    {
        if ( a.blen[g] < 1 || a.blen[g] > kStructMaxBox ) return false;
        maxlen = std::max ( maxlen, a.blen[g] );
    }
    const bool wide = maxlen > 32;
    if ( wide != a.wide ) return false;                             // planes built at the other width
    switch ( B )
    {
        case 1:
        case 2: return launch_structN_b<2> ( a, ed, wide, grid, st );
        case 3: return launch_structN_b<3> ( a, ed, wide, grid, st );
        case 4: return launch_structN_b<4> ( a, ed, wide, grid, st );
        case 5: return launch_structN_b<5> ( a, ed, wide, grid, st );
        default: return false;
    }
}

namespace
{

// Symbol t of entry (pos, k)'s key: box 0 first, then each later box.
__device__ __forceinline__ uint32_t skey_sym_pos ( const SKeyArgs & a, uint32_t pos, uint32_t k, uint32_t t )
{
    if ( t < a.l ) return pos + 1 - a.l + t;
    t -= a.l;
    for ( uint32_t g = 0; g < a.NG; ++g )
    {
        if ( t < a.blen[g] ) return pos + a.xoff[k * a.NG + g] + 1 - a.blen[g] + t;
        t -= a.blen[g];
    }
    return pos;                                                     // not reached: t < key length
}

__device__ __forceinline__ uint32_t skey_len ( const SKeyArgs & a )
{
    uint32_t n = a.l;
    for ( uint32_t g = 0; g < a.NG; ++g ) n += a.blen[g];
    return n;
}

} // namespace

// Insert every passing entry's key: the slot keeps a representative entry
// (compared symbol by symbol on a hash match) and the least entry index.
__global__ void k_skey_insert ( SKeyArgs a )
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= a.nrec ) return;
    const uint32_t idx = a.recs[3 * ( size_t ) i];
    const uint32_t pos = idx / a.G, k = idx % a.G;
    const uint32_t L = skey_len ( a );
    unsigned long long h = 0xcbf29ce484222325ull;                  // FNV-1a over the key's codes
    for ( uint32_t t = 0; t < L; ++t )
    {
        h ^= a.codes[skey_sym_pos ( a, pos, k, t )];
        h *= 0x100000001b3ull;
    }
    const uint32_t tsize = 1u << a.tbits;
    uint32_t slot = ( uint32_t ) ( ( h * 0x9E3779B97F4A7C15ull ) >> ( 64 - a.tbits ) );
    for ( uint32_t probe = 0; probe < tsize; ++probe )
    {
        const uint32_t r = atomicCAS ( a.rep + slot, 0xffffffffu, i );
        bool same = r == 0xffffffffu;
        if ( ! same )
        {
            const uint32_t ridx = a.recs[3 * ( size_t ) r];
            const uint32_t rpos = ridx / a.G, rk = ridx % a.G;
            same = true;
            for ( uint32_t t = 0; t < L && same; ++t )
                same = a.codes[skey_sym_pos ( a, pos, k, t )] == a.codes[skey_sym_pos ( a, rpos, rk, t )];
        }
        if ( same )
        {
            atomicMin ( a.first + slot, i );
            a.slot_of[i] = slot;
            return;
        }
        slot = ( slot + 1 ) & ( tsize - 1 );
    }
    atomicExch ( a.err, 1u );
    a.slot_of[i] = 0;
}

__global__ void k_skey_keep ( SKeyArgs a )
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if ( i >= a.nrec ) return;
    a.keep[i] = a.first[a.slot_of[i]] == i ? 1 : 0;
}

// 64-bit planes of the factor of length l ending at every position (zero
// where it would start before position 0); top-aligned for Hamming.
__global__ void k_wplanes_all64 ( const uint8_t * __restrict__ codes, uint32_t total, uint32_t l, uint32_t B,
                                  int top_aligned, unsigned long long * __restrict__ out )
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if ( pos >= total ) return;
    unsigned long long pl[kMaxPlanes] = { 0, 0, 0, 0, 0 };
    if ( pos + 1 >= l )
        for ( uint32_t q = 0; q < l; ++q )
        {
            const unsigned long long c = codes[pos + 1 - l + q];
            const uint32_t bit = top_aligned ? ( 64 - l + q ) : q;
#pragma unroll
            for ( int b = 0; b < kMaxPlanes; ++b ) pl[b] |= ( ( c >> b ) & 1ull ) << bit;
        }
    for ( uint32_t b = 0; b < B; ++b ) out[( size_t ) b * total + pos] = pl[b];
}

// Start offset of the sequence holding each position.
__global__ void k_seq_start ( const uint32_t * __restrict__ offs, uint32_t nseq, uint64_t total, uint32_t * out )
{
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if ( pos >= total ) return;
    uint32_t lo = 0, hi = nseq;
    while ( hi - lo > 1 )
    {
        const uint32_t mid = ( lo + hi ) >> 1;
        if ( offs[mid] <= pos ) lo = mid; else hi = mid;
    }
    while ( offs[lo + 1] <= pos ) ++lo;
    out[pos] = offs[lo];
}

} // namespace mtx
