// Integer-pipe throughput microkernels (motex_probe_int_peak).
//
// The factor-search DP runs on the integer ALU and popc pipes, for which no
// vendor peak is published per clock on this part; these kernels measure
// it.  Each thread runs kChains independent dependency chains of inline-PTX
// operations (asm volatile, so nothing is folded away), enough to cover
// pipe latency; the grid fills every SM several times.
#include "motex_gpu.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace
{

constexpr int kChains = 8;
constexpr int kIters = 2048;
constexpr int kThreads = 256;

template <int OP>
__global__ void __launch_bounds__ ( kThreads ) k_int_probe ( uint32_t seed, uint32_t * out )
{
    uint32_t a[kChains];
#pragma unroll
    for ( int i = 0; i < kChains; ++i ) a[i] = seed * ( threadIdx.x + 7 * i + 1 ) + blockIdx.x;
    const uint32_t k = seed ^ 0x5bd1e995u;
    for ( int it = 0; it < kIters; ++it )
    {
#pragma unroll
        for ( int i = 0; i < kChains; ++i )
        {
            const uint32_t b = a[( i + 1 ) % kChains];
            if constexpr ( OP == 0 )
                asm volatile ( "lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"( a[i] ) : "r"( b ), "r"( k ) );
            else if constexpr ( OP == 1 )
                asm volatile ( "add.u32 %0, %0, %1;" : "+r"( a[i] ) : "r"( b ) );
            else
                asm volatile ( "popc.b32 %0, %0;" : "+r"( a[i] ) );
        }
    }
    uint32_t s = 0;
#pragma unroll
    for ( int i = 0; i < kChains; ++i ) s += a[i];
    if ( s == 0x12345678u ) out[0] = s;   // keeps the chains live
}

template <int OP>
double time_probe ( int sms, uint32_t * out, cudaEvent_t e0, cudaEvent_t e1 )
{
    const int blocks = sms * 8;
    k_int_probe<OP><<<blocks, kThreads>>> ( 3u, out );               // warm-up
    cudaEventRecord ( e0 );
    k_int_probe<OP><<<blocks, kThreads>>> ( 5u, out );
    cudaEventRecord ( e1 );
    cudaEventSynchronize ( e1 );
    float ms = 0.f;
    cudaEventElapsedTime ( &ms, e0, e1 );
    const double ops = ( double ) blocks * kThreads * kIters * kChains;
    return ms > 0 ? ops / ( ms * 1e-3 ) / 1e12 : 0.0;
}

} // namespace

extern "C" int motex_probe_int_peak ( int device, double * lop3_tops, double * iadd_tops, double * popc_tops )
{
    if ( ! lop3_tops || ! iadd_tops || ! popc_tops ) return MOTEX_EINVAL;
    if ( cudaSetDevice ( device ) != cudaSuccess ) return MOTEX_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute ( &sms, cudaDevAttrMultiProcessorCount, device );
    uint32_t * out = nullptr;
    if ( cudaMalloc ( &out, 16 ) != cudaSuccess ) return MOTEX_ENOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate ( &e0 );
    cudaEventCreate ( &e1 );
    *lop3_tops = time_probe<0> ( sms, out, e0, e1 );
    *iadd_tops = time_probe<1> ( sms, out, e0, e1 );
    *popc_tops = time_probe<2> ( sms, out, e0, e1 );
    cudaError_t err = cudaGetLastError ();
    cudaEventDestroy ( e0 );
    cudaEventDestroy ( e1 );
    cudaFree ( out );
    return err == cudaSuccess ? MOTEX_OK : MOTEX_ECUDA;
}
