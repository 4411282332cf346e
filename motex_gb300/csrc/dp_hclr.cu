// Popc-free packed Hamming (dp_hswar_body with E = e): factors in guarded
// lanes of one register, the mismatch count tested by clearing the lowest set
// bit of every lane e times.  Its own translation unit: 64 instances
// (B 2..5 x NL 2, 3 x W 4, 8 x e 0..3) compile beside the others.
#include "dp_body.cuh"

namespace mtx
{

template <int B, int NL, int W, int E>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_hclr ( const DPArgs a, const SwarConst C )
{
    dp_hswar_body<B, NL, W, 4, E> ( a, C, blockIdx.x, blockIdx.y );
}

// Two lanes of l bits with a guard bit above each and 6-bit count fields at
// the guards: 2(l+1) + 5 <= 31, so l <= 12 (l >= 5 keeps a count field below
// the next lane's guard).  Three lanes, the top one unguarded: 3l + 2 <= 32,
// and the top lane's count field at bit 0 below lane 0's at bit l: 6 <= l <= 10.
bool hclr_fits ( uint32_t l, int NL )
{
    if ( NL == 2 ) return l >= 5 && l <= 12;
    if ( NL == 3 ) return l >= 6 && l <= 10;
    return false;
}

int hclr_lanes ( uint32_t l ) { return hclr_fits ( l, 3 ) ? 3 : ( hclr_fits ( l, 2 ) ? 2 : 1 ); }

SwarConst hclr_const ( uint32_t l, int NL )
{
    SwarConst C {};
    C.S = l + 1;
    for ( int j = 0; j < NL; ++j )
    {
        if ( NL == 2 || j < 2 ) C.HB |= 1u << ( j * C.S + l );   // guards G (not the top lane of three)
        C.REP |= 1u << ( j * C.S );                            // L, and the window copies
    }
    C.K = 0u - C.REP;                                          // x + K = x - L
    C.Q = l;
    C.FM = 63u;
    C.ONE = 1u;
    C.LIM = NL == 3 ? 1u << ( 2 * C.S ) : 0u;
    return C;
}

namespace
{

template <int B, int NL, int W>
bool launch_bw ( const DPArgs & a, const SwarConst & C, dim3 grid, cudaStream_t st )
{
    const size_t smem = hswar_smem_bytes ( NL, W );
    switch ( a.e )
    {
#define MTX_HCLR( E )                                                                                          \
    case E:                                                                                                    \
        cudaFuncSetAttribute ( k_dp_hclr<B, NL, W, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem ); \
        k_dp_hclr<B, NL, W, E><<<grid, kDPThreads, smem, st>>> ( a, C );                                          \
        return true;
        MTX_HCLR ( 0 )
        MTX_HCLR ( 1 )
        MTX_HCLR ( 2 )
        MTX_HCLR ( 3 )
#undef MTX_HCLR
        default: return false;
    }
}

template <int B, int NL>
bool launch_bn ( const DPArgs & a, const SwarConst & C, int W, dim3 grid, cudaStream_t st )
{
    if ( W == 8 ) return launch_bw<B, NL, 8> ( a, C, grid, st );
    if ( W == 4 ) return launch_bw<B, NL, 4> ( a, C, grid, st );
    return false;
}

template <int B>
bool launch_b ( const DPArgs & a, const SwarConst & C, int NL, int W, dim3 grid, cudaStream_t st )
{
    if ( NL == 3 ) return launch_bn<B, 3> ( a, C, W, grid, st );
    if ( NL == 2 ) return launch_bn<B, 2> ( a, C, W, grid, st );
    return false;
}

} // namespace

bool launch_dp_hclr ( const DPArgs & a, int B, int NL, int W, dim3 grid, cudaStream_t st )
{
    if ( ! hclr_fits ( a.l, NL ) || a.e > kHclrMaxE ) return false;
    const SwarConst C = hclr_const ( a.l, NL );
    switch ( B )
    {
        case 1:                                     // one plane: the 2-plane kernel (plane 1 is zero)
        case 2: return launch_b<2> ( a, C, NL, W, grid, st );
        case 3: return launch_b<3> ( a, C, NL, W, grid, st );
        case 4: return launch_b<4> ( a, C, NL, W, grid, st );
        case 5: return launch_b<5> ( a, C, NL, W, grid, st );
        default: return false;
    }
}

} // namespace mtx
