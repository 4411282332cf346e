// All-factors x all-texts approximate-matching DP of the GB300 engine: static-
// grid kernels (one job per launch) and their launchers.  The kernel bodies
// and the design notes are in dp_body.cuh.
#include "dp_body.cuh"

#include <algorithm>

namespace mtx
{

template <int B, int W, bool ED, bool SCALED, int UR>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_fast ( const DPArgs a )
{
    dp_fast_body<B, W, ED, SCALED, UR> ( a, blockIdx.x, blockIdx.y );
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

template <int B, int NL, int W, int UR>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_swar_ed ( const DPArgs a, const SwarConst C )
{
    dp_swar_body<B, NL, W, UR> ( a, C, blockIdx.x, blockIdx.y );
}

template <int B, int NL, int W, int UR>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_hswar ( const DPArgs a, const SwarConst C )
{
    dp_hswar_body<B, NL, W, UR> ( a, C, blockIdx.x, blockIdx.y );
}

// ------------------------------------------------------------------ launchers

template <int B, int W, int UR>
static void launch_fast_bwu ( const DPArgs & a, bool ed, dim3 grid, cudaStream_t st )
{
    const size_t smem = fast_smem_bytes ( B, W, ed );
    if ( ! ed )
        k_dp_fast<B, W, false, false, UR><<<grid, kDPThreads, 0, st>>> ( a );
    else if ( a.l <= 28 )
        k_dp_fast<B, W, true, true, UR><<<grid, kDPThreads, smem, st>>> ( a );
    else
        k_dp_fast<B, W, true, false, UR><<<grid, kDPThreads, smem, st>>> ( a );
}

template <int B, int W>
static bool launch_fast_bw ( const DPArgs & a, int UR, bool ed, dim3 grid, cudaStream_t st )
{
    switch ( UR )
    {
        case 4: launch_fast_bwu<B, W, 4> ( a, ed, grid, st ); return true;
        case 8: launch_fast_bwu<B, W, 8> ( a, ed, grid, st ); return true;
        case 32: launch_fast_bwu<B, W, 32> ( a, ed, grid, st ); return true;
        default: return false;
    }
}

template <int B>
static bool launch_fast_b ( const DPArgs & a, int W, int UR, bool ed, dim3 grid, cudaStream_t st )
{
    switch ( W )
    {
        case 4: return launch_fast_bw<B, 4> ( a, UR, ed, grid, st );
        case 8: return launch_fast_bw<B, 8> ( a, UR, ed, grid, st );
        default: return false;
    }
}

bool launch_dp_fast ( const DPArgs & a, int B, int W, int UR, bool ed, dim3 grid, cudaStream_t st )
{
    if ( a.l < 1 || a.l > 32 ) return false;
    switch ( B )
    {
        case 1:                                     // runs on the 2-plane kernel (plane 1 is zero)
        case 2: return launch_fast_b<2> ( a, W, UR, ed, grid, st );
        case 3: return launch_fast_b<3> ( a, W, UR, ed, grid, st );
        case 4: return launch_fast_b<4> ( a, W, UR, ed, grid, st );
        case 5: return launch_fast_b<5> ( a, W, UR, ed, grid, st );
        default: return false;
    }
}

// Lane stride: l symbols, a guard bit, and for l = 4 a spare bit, so that
// every S-bit count field holds the 32 hits of one text block.
static uint32_t swar_stride ( uint32_t l ) { return std::max ( l + 1, 6u ); }

int swar_lanes ( uint32_t l )
{
    if ( l < 4 || l > 15 ) return 1;
    return std::min ( 4, ( int ) ( ( 32 - l ) / swar_stride ( l ) ) + 1 );
}

template <int B, int NL, int W>
static bool launch_swar_bnw ( const DPArgs & a, const SwarConst & C, int UR, dim3 grid, cudaStream_t st )
{
    const size_t smem = swar_smem_bytes ( B, NL, W );
    switch ( UR )
    {
        case 4:
            cudaFuncSetAttribute ( k_dp_swar_ed<B, NL, W, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem );
            k_dp_swar_ed<B, NL, W, 4><<<grid, kDPThreads, smem, st>>> ( a, C );
            return true;
        case 8:
            cudaFuncSetAttribute ( k_dp_swar_ed<B, NL, W, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem );
            k_dp_swar_ed<B, NL, W, 8><<<grid, kDPThreads, smem, st>>> ( a, C );
            return true;
        default: return false;
    }
}

template <int B, int NL>
static bool launch_swar_bn ( const DPArgs & a, const SwarConst & C, int W, int UR, dim3 grid, cudaStream_t st )
{
    switch ( W )
    {
        case 4: return launch_swar_bnw<B, NL, 4> ( a, C, UR, grid, st );
        case 8: return launch_swar_bnw<B, NL, 8> ( a, C, UR, grid, st );
        default: return false;
    }
}

template <int B>
static bool launch_swar_b ( const DPArgs & a, const SwarConst & C, int NL, int W, int UR, dim3 grid, cudaStream_t st )
{
    switch ( NL )
    {
        case 2: return launch_swar_bn<B, 2> ( a, C, W, UR, grid, st );
        case 3: return launch_swar_bn<B, 3> ( a, C, W, UR, grid, st );
        case 4: return launch_swar_bn<B, 4> ( a, C, W, UR, grid, st );
        default: return false;
    }
}

SwarConst swar_const ( uint32_t l, uint32_t e, int NL )
{
    SwarConst C {};
    C.S = swar_stride ( l );
    // hit bit h of the score fields: score + 2^h - (e+1) stays in [0, 2^(h+1))
    // for every score in [0, l] when 2^h >= l (e < l), so bit h alone tells
    // score <= e; NL = 2, 3 have room for 6-bit count fields at h
    uint32_t h = l - 1;
    if ( NL != 4 )
        for ( h = 0; ( 1u << h ) < l; ++h ) {}
    uint32_t guards = 0;
    for ( int j = 0; j < NL; ++j )
    {
        const uint32_t o = j * C.S;
        C.HB |= 1u << ( o + l - 1 );
        C.HQ |= 1u << ( o + h );
        for ( uint32_t g = o + l; g < o + C.S && g < 32; ++g ) guards |= 1u << g;
        C.K += ( ( 1u << h ) - ( e + 1 ) ) << o;
        C.SC0 += l << o;
    }
    C.NG = ~guards;
    C.NGm1 = C.NG & ~C.HB;
    C.Q = NL != 4 ? h : 0;
    C.FM = NL != 4 ? 63u : ( 1u << C.S ) - 1u;
    C.ONE = 1u;
    C.TWO = 2u;
    C.NEG1 = ~0u;
    return C;
}

bool launch_dp_swar_ed ( const DPArgs & a, int B, int NL, int W, int UR, dim3 grid, cudaStream_t st )
{
    if ( NL < 2 || NL != swar_lanes ( a.l ) ) return false;
    const SwarConst C = swar_const ( a.l, a.e, NL );
    switch ( B )
    {
        case 1:
        case 2: return launch_swar_b<2> ( a, C, NL, W, UR, grid, st );
        case 3: return launch_swar_b<3> ( a, C, NL, W, UR, grid, st );
        case 4: return launch_swar_b<4> ( a, C, NL, W, UR, grid, st );
        case 5: return launch_swar_b<5> ( a, C, NL, W, UR, grid, st );
        default: return false;
    }
}

int hswar_lanes ( uint32_t l ) { return ( l >= 6 && l <= 16 ) ? ( int ) ( 32 / l ) : 1; }

SwarConst hswar_const ( uint32_t l, int NL )
{
    SwarConst C {};
    C.S = l;
    C.FM = ( 1u << l ) - 1u;
    for ( int j = 0; j < NL; ++j ) C.REP |= 1u << ( j * l );
    return C;
}

template <int B, int NL, int W>
static bool launch_hswar_bnw ( const DPArgs & a, const SwarConst & C, dim3 grid, cudaStream_t st )
{
    const size_t smem = hswar_smem_bytes ( NL, W );
    cudaFuncSetAttribute ( k_dp_hswar<B, NL, W, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem );
    k_dp_hswar<B, NL, W, 4><<<grid, kDPThreads, smem, st>>> ( a, C );
    return true;
}

template <int B, int NL>
static bool launch_hswar_bn ( const DPArgs & a, const SwarConst & C, int W, dim3 grid, cudaStream_t st )
{
    if ( W == 8 ) return launch_hswar_bnw<B, NL, 8> ( a, C, grid, st );
    if ( W == 4 ) return launch_hswar_bnw<B, NL, 4> ( a, C, grid, st );
    return false;
}

template <int B>
static bool launch_hswar_b ( const DPArgs & a, const SwarConst & C, int NL, int W, dim3 grid, cudaStream_t st )
{
    switch ( NL )
    {
        case 2: return launch_hswar_bn<B, 2> ( a, C, W, grid, st );
        case 3: return launch_hswar_bn<B, 3> ( a, C, W, grid, st );
        case 4: return launch_hswar_bn<B, 4> ( a, C, W, grid, st );
        case 5: return launch_hswar_bn<B, 5> ( a, C, W, grid, st );
        default: return false;
    }
}

// Packed Hamming kernels (unroll 4, the Hamming optimum) for 3-5 bit planes.
bool launch_dp_hswar ( const DPArgs & a, int B, int NL, int W, int, dim3 grid, cudaStream_t st )
{
    if ( NL < 2 || NL != hswar_lanes ( a.l ) ) return false;
    const SwarConst C = hswar_const ( a.l, NL );
    switch ( B )
    {
        case 3: return launch_hswar_b<3> ( a, C, NL, W, grid, st );
        case 4: return launch_hswar_b<4> ( a, C, NL, W, grid, st );
        case 5: return launch_hswar_b<5> ( a, C, NL, W, grid, st );
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
