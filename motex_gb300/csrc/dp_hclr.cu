// Popc-free packed Hamming (dp_hswar_body with E = e): factors in guarded
// lanes of one register, the mismatch count tested by clearing the lowest set
// bit of every lane e times.  Its own translation unit: 32 instances
// (B 2..5 x W 4, 8 x e 0..3) compile beside the others.
#include "dp_body.cuh"

namespace mtx
{

template <int B, int W, int E>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_hclr ( const DPArgs a, const SwarConst C )
{
    dp_hswar_body<B, 2, W, 4, E> ( a, C, blockIdx.x, blockIdx.y );
}

// Two lanes of l bits with a guard bit above each, and 6-bit count fields at
// the guards: 2(l+1) + 5 <= 31, so 5 <= l <= 12 (l >= 5 keeps a count field
// below the next lane's guard).
int hclr_lanes ( uint32_t l ) { return ( l >= 5 && l <= 12 ) ? 2 : 1; }

SwarConst hclr_const ( uint32_t l )
{
    SwarConst C {};
    C.S = l + 1;
    for ( uint32_t j = 0; j < 2; ++j )
    {
        C.HB |= 1u << ( j * C.S + l );                         // guards G
        C.REP |= 1u << ( j * C.S );                            // L, and the window copies
    }
    C.K = 0u - C.REP;                                          // x + K = x - L
    C.Q = l;
    C.FM = 63u;
    C.ONE = 1u;
    return C;
}

namespace
{

template <int B, int W>
bool launch_bw ( const DPArgs & a, const SwarConst & C, dim3 grid, cudaStream_t st )
{
    const size_t smem = hswar_smem_bytes ( 2, W );
    switch ( a.e )
    {
#define MTX_HCLR( E )                                                                                          \
    case E:                                                                                                    \
        cudaFuncSetAttribute ( k_dp_hclr<B, W, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem ); \
        k_dp_hclr<B, W, E><<<grid, kDPThreads, smem, st>>> ( a, C );                                          \
        return true;
        MTX_HCLR ( 0 )
        MTX_HCLR ( 1 )
        MTX_HCLR ( 2 )
        MTX_HCLR ( 3 )
#undef MTX_HCLR
        default: return false;
    }
}

template <int B>
bool launch_b ( const DPArgs & a, const SwarConst & C, int W, dim3 grid, cudaStream_t st )
{
    if ( W == 8 ) return launch_bw<B, 8> ( a, C, grid, st );
    if ( W == 4 ) return launch_bw<B, 4> ( a, C, grid, st );
    return false;
}

} // namespace

bool launch_dp_hclr ( const DPArgs & a, int B, int NL, int W, dim3 grid, cudaStream_t st )
{
    if ( NL != 2 || hclr_lanes ( a.l ) != 2 || a.e > kHclrMaxE ) return false;
    const SwarConst C = hclr_const ( a.l );
    switch ( B )
    {
        case 1:                                     // one plane: the 2-plane kernel (plane 1 is zero)
        case 2: return launch_b<2> ( a, C, W, grid, st );
        case 3: return launch_b<3> ( a, C, W, grid, st );
        case 4: return launch_b<4> ( a, C, W, grid, st );
        case 5: return launch_b<5> ( a, C, W, grid, st );
        default: return false;
    }
}

} // namespace mtx
