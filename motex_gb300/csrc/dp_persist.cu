// Persistent, batched form of the factor-search DP: one launch per kernel
// class serves any number of jobs; CTAs pull (job, tile, chunk) items from a
// device counter (see next_item in dp_body.cuh).
#include "dp_body.cuh"

#include <type_traits>

namespace mtx
{

/*
 * Each CTA copies the DPArgs of the job of its current item into shared
 * memory; the bodies then read the job's pointers and sizes from there once
 * per text block instead of holding them in registers for the whole item.
 * The lane constants of the packed bodies (SwarConst) are the same for every
 * job of a launch (the class key includes l and e) and come in as a kernel
 * parameter, i.e. from the constant bank like in the one-job kernels.  With
 * both, the persistent kernels need about the registers of the one-job
 * kernels.
 */
__device__ __forceinline__ void load_job ( const JobDesc * jobs, uint32_t job, DPArgs & s_job )
{
    constexpr int kWords = sizeof ( DPArgs ) / sizeof ( uint32_t );
    static_assert ( sizeof ( DPArgs ) % sizeof ( uint32_t ) == 0, "DPArgs is copied word by word" );
    const uint32_t * src = reinterpret_cast<const uint32_t *> ( &jobs[job].a );
    uint32_t * dst = reinterpret_cast<uint32_t *> ( &s_job );
    for ( int i = threadIdx.x; i < kWords; i += blockDim.x ) dst[i] = src[i];
    __syncthreads ();
}

template <int B, int W, bool ED, bool SCALED, int UR>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_fast_persist ( const JobDesc * jobs, const WorkItem * items,
                                                                     uint32_t nitems, uint32_t * counter )
{
    __shared__ DPArgs s_job;
    WorkItem w;
    while ( next_item ( items, nitems, counter, w ) )
    {
        load_job ( jobs, w.job, s_job );
        dp_fast_body<B, W, ED, SCALED, UR> ( s_job, w.tile, w.chunk );
    }
}

template <int B, int NL, int W, int UR>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_hswar_persist ( const JobDesc * jobs, const WorkItem * items,
                                                                      uint32_t nitems, uint32_t * counter,
                                                                      const SwarConst C )
{
    __shared__ DPArgs s_job;
    WorkItem w;
    while ( next_item ( items, nitems, counter, w ) )
    {
        load_job ( jobs, w.job, s_job );
        dp_hswar_body<B, NL, W, UR> ( s_job, C, w.tile, w.chunk );
    }
}

// popc-free Hamming (guarded lanes, E = e lowest-bit clears), 8 register
// words per thread, unroll 4
template <int B, int NL, int E>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_hclr_persist ( const JobDesc * jobs, const WorkItem * items,
                                                                     uint32_t nitems, uint32_t * counter,
                                                                     const SwarConst C )
{
    __shared__ DPArgs s_job;
    WorkItem w;
    while ( next_item ( items, nitems, counter, w ) )
    {
        load_job ( jobs, w.job, s_job );
        dp_hswar_body<B, NL, 8, 4, E> ( s_job, C, w.tile, w.chunk );
    }
}

template <int B, int NL, int W, int UR>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_swar_persist ( const JobDesc * jobs, const WorkItem * items,
                                                                     uint32_t nitems, uint32_t * counter,
                                                                     const SwarConst C )
{
    __shared__ DPArgs s_job;
    WorkItem w;
    while ( next_item ( items, nitems, counter, w ) )
    {
        load_job ( jobs, w.job, s_job );
        dp_swar_body<B, NL, W, UR> ( s_job, C, w.tile, w.chunk );
    }
}

namespace
{

template <typename K>
int ctas_per_sm ( K kernel, size_t smem )
{
    int n = 0;
    cudaFuncSetAttribute ( kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem );
    if ( cudaOccupancyMaxActiveBlocksPerMultiprocessor ( &n, kernel, kDPThreads, smem ) != cudaSuccess ) n = 1;
    return n > 0 ? n : 1;
}

template <int B, int NL, int E>
bool launch_hclr ( const JobDesc * jobs, const WorkItem * items, uint32_t nitems, uint32_t * counter,
                   const SwarConst & C, unsigned grid, cudaStream_t st, int * occ )
{
    const size_t smem = hswar_smem_bytes ( NL, 8 );
    if ( occ ) { *occ = ctas_per_sm ( k_dp_hclr_persist<B, NL, E>, smem ); return true; }
    cudaFuncSetAttribute ( k_dp_hclr_persist<B, NL, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem );
    k_dp_hclr_persist<B, NL, E><<<grid, kDPThreads, smem, st>>> ( jobs, items, nitems, counter, C );
    return true;
}

template <int B, int NL>
bool launch_hclr_e ( const JobDesc * jobs, const WorkItem * items, uint32_t nitems, uint32_t * counter, int E,
                     const SwarConst & C, unsigned grid, cudaStream_t st, int * occ )
{
    switch ( E )
    {
        case 0: return launch_hclr<B, NL, 0> ( jobs, items, nitems, counter, C, grid, st, occ );
        case 1: return launch_hclr<B, NL, 1> ( jobs, items, nitems, counter, C, grid, st, occ );
        case 2: return launch_hclr<B, NL, 2> ( jobs, items, nitems, counter, C, grid, st, occ );
        case 3: return launch_hclr<B, NL, 3> ( jobs, items, nitems, counter, C, grid, st, occ );
        default: return false;
    }
}

template <int B>
bool launch_b ( const JobDesc * jobs, const WorkItem * items, uint32_t nitems, uint32_t * counter, bool ed, bool scaled,
                int NL, int W, int UR, int E, const SwarConst & C, unsigned grid, cudaStream_t st, int * occ )
{
    if ( E >= 0 )
    {
        if ( ed || W != 8 || UR != 4 ) return false;
        if ( NL == 2 ) return launch_hclr_e<B, 2> ( jobs, items, nitems, counter, E, C, grid, st, occ );
        if ( NL == 3 ) return launch_hclr_e<B, 3> ( jobs, items, nitems, counter, E, C, grid, st, occ );
        return false;
    }
    if ( NL <= 1 )
    {
        if ( ! ed )
        {
            if ( occ ) { *occ = ctas_per_sm ( k_dp_fast_persist<B, 8, false, false, 4>, 0 ); return true; }
            k_dp_fast_persist<B, 8, false, false, 4><<<grid, kDPThreads, 0, st>>> ( jobs, items, nitems, counter );
        }
        else if ( scaled )
        {
            const size_t smem = fast_smem_bytes ( B, 8, true );
            if ( occ ) { *occ = ctas_per_sm ( k_dp_fast_persist<B, 8, true, true, 8>, smem ); return true; }
            k_dp_fast_persist<B, 8, true, true, 8><<<grid, kDPThreads, smem, st>>> ( jobs, items, nitems, counter );
        }
        else
        {
            const size_t smem = fast_smem_bytes ( B, 8, true );
            if ( occ ) { *occ = ctas_per_sm ( k_dp_fast_persist<B, 8, true, false, 8>, smem ); return true; }
            k_dp_fast_persist<B, 8, true, false, 8><<<grid, kDPThreads, smem, st>>> ( jobs, items, nitems, counter );
        }
        return true;
    }
    if ( ! ed )
    {
        // packed Hamming (3-5 bit planes), 8 register words per thread
        if constexpr ( B >= 3 )
        {
#define MTX_HSWAR_P( NLV )                                                                                  \
    case NLV:                                                                                               \
    {                                                                                                       \
        const size_t smem = hswar_smem_bytes ( NLV, 8 );                                                    \
        if ( occ ) { *occ = ctas_per_sm ( k_dp_hswar_persist<B, NLV, 8, 4>, smem ); return true; }           \
        cudaFuncSetAttribute ( k_dp_hswar_persist<B, NLV, 8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                               ( int ) smem );                                                              \
        k_dp_hswar_persist<B, NLV, 8, 4><<<grid, kDPThreads, smem, st>>> ( jobs, items, nitems, counter, C ); \
        return true;                                                                                        \
    }
            switch ( NL )
            {
                MTX_HSWAR_P ( 2 )
                MTX_HSWAR_P ( 3 )
                MTX_HSWAR_P ( 4 )
                MTX_HSWAR_P ( 5 )
                default: return false;
            }
#undef MTX_HSWAR_P
        }
        return false;
    }
    // packed edit distance: every (W, UR) the autotuner may pick for the one-job kernel
    auto swar = [&] ( auto nl, auto w, auto ur ) -> bool {
        constexpr int NLV = decltype ( nl )::value, WV = decltype ( w )::value, URV = decltype ( ur )::value;
        const size_t smem = swar_smem_bytes ( B, NLV, WV );
        if ( occ ) { *occ = ctas_per_sm ( k_dp_swar_persist<B, NLV, WV, URV>, smem ); return true; }
        cudaFuncSetAttribute ( k_dp_swar_persist<B, NLV, WV, URV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               ( int ) smem );
        k_dp_swar_persist<B, NLV, WV, URV><<<grid, kDPThreads, smem, st>>> ( jobs, items, nitems, counter, C );
        return true;
    };
    auto swar_nl = [&] ( auto nl ) -> bool {
        using I4 = std::integral_constant<int, 4>;
        using I8 = std::integral_constant<int, 8>;
        if ( W == 4 && UR == 4 ) return swar ( nl, I4 {}, I4 {} );
        if ( W == 4 && UR == 8 ) return swar ( nl, I4 {}, I8 {} );
        if ( W == 8 && UR == 4 ) return swar ( nl, I8 {}, I4 {} );
        if ( W == 8 && UR == 8 ) return swar ( nl, I8 {}, I8 {} );
        return false;
    };
    switch ( NL )
    {
        case 2: return swar_nl ( std::integral_constant<int, 2> {} );
        case 3: return swar_nl ( std::integral_constant<int, 3> {} );
        case 4: return swar_nl ( std::integral_constant<int, 4> {} );
        default: return false;
    }
}

bool dispatch ( const JobDesc * jobs, const WorkItem * items, uint32_t nitems, uint32_t * counter, int B, bool ed,
                bool scaled, int NL, int W, int UR, int E, const SwarConst & C, unsigned grid, cudaStream_t st,
                int * occ )
{
    switch ( B )
    {
        case 1:
        case 2: return launch_b<2> ( jobs, items, nitems, counter, ed, scaled, NL, W, UR, E, C, grid, st, occ );
        case 3: return launch_b<3> ( jobs, items, nitems, counter, ed, scaled, NL, W, UR, E, C, grid, st, occ );
        case 4: return launch_b<4> ( jobs, items, nitems, counter, ed, scaled, NL, W, UR, E, C, grid, st, occ );
        case 5: return launch_b<5> ( jobs, items, nitems, counter, ed, scaled, NL, W, UR, E, C, grid, st, occ );
        default: return false;
    }
}

} // namespace

int persistent_ctas_per_sm ( int B, bool ed, bool scaled, int NL, int W, int UR, int E )
{
    int occ = 1;
    if ( ! dispatch ( nullptr, nullptr, 0, nullptr, B, ed, scaled, NL, W, UR, E, SwarConst {}, 0, nullptr, &occ ) )
        return 1;
    return occ;
}

bool persistent_shape ( int B, bool ed, int NL, int W, int UR, int E )
{
    if ( E >= 0 ) return ! ed && ( NL == 2 || NL == 3 ) && W == 8 && UR == 4 && E <= ( int ) kHclrMaxE;
    if ( NL <= 1 ) return W == 8 && UR == ( ed ? 8 : 4 );
    if ( ! ed ) return B >= 3 && W == 8 && UR == 4;
    return ( W == 4 || W == 8 ) && ( UR == 4 || UR == 8 );
}

bool launch_dp_persistent ( const JobDesc * jobs, const WorkItem * items, uint32_t nitems, uint32_t * counter, int B,
                            bool ed, bool scaled, int NL, int W, int UR, int E, const SwarConst & C, unsigned grid,
                            cudaStream_t st )
{
    return dispatch ( jobs, items, nitems, counter, B, ed, scaled, NL, W, UR, E, C, grid, st, nullptr );
}

} // namespace mtx
