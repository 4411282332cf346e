// motex_gpu_extract_pair_static: the per-pair factor search with no memory
// allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc -- code running inside
// another framework's memory pool or allocator hooks, code that must not
// allocate between its own set-up and tear-down (for example to keep a
// fixed memory budget or to avoid allocator synchronisation on a hot loop),
// and plug-ins that are only handed device buffers.  They pass the pattern
// and text sequences and the u / v outputs as device pointers they already
// own; every intermediate buffer of the search lives in one file-scope
// device array of kStaticScratchBytes, which every GPU that loads this
// library keeps until the process exits.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address with cudaGetSymbolAddress and keeps it, keyed by the
// unique id of the CUDA context it was looked up in (cuCtxGetId; ids are never
// reused within a process).  A later call in the same context reuses it; a
// call in another context of the device -- e.g. the new primary context after
// a cudaDeviceReset, which reloads the module and may move the array -- looks
// it up again, so no call ever hands a kernel a stale address.  Make the first
// call on a device before any stream capture.  The call returns after
// `stream` has finished its work (it reads an error word back).  All calls
// share the one array and it keeps the previous call's contents, so each call
// clears what must start at zero; calls that overlap on the GPU (different
// streams or host threads without ordering) race on it and must be
// serialised by the caller.
#include "motex_gpu.h"
#include "kernels.cuh"

#include <cuda.h>

#include <algorithm>
#include <mutex>

using namespace mtx;

namespace
{

constexpr size_t   kStaticScratchBytes = 4u << 20;   // 4 MiB per device
constexpr uint32_t kMaxPattern = 32768;               // m
constexpr uint32_t kMaxText = 1u << 20;               // n
constexpr uint32_t kMaxChunks = 512;
constexpr int      kMaxDevices = 64;

static __device__ __align__ ( 256 ) uint8_t g_pair_scratch[kStaticScratchBytes];

struct ScratchAddr
{
    unsigned long long ctx_id = 0;   // 0: not looked up yet (context ids start at 1)
    uint8_t * addr = nullptr;
};

std::mutex g_mu;
ScratchAddr g_scratch[kMaxDevices];

struct AlphaMap
{
    uint8_t code[256];   // 0xff: byte not in the alphabet
};

struct Layout
{
    size_t planes, vmask, emask, wplanes, u_acc, v_acc, flags, chunks, err, total;
};

size_t up256 ( size_t x ) { return ( x + 255 ) & ~( size_t ) 255; }

Layout layout_for ( uint32_t B, uint32_t nblk, uint32_t U, uint32_t nchunks )
{
    Layout L;
    size_t at = 0;
    const size_t stride = ( nblk + 1 + 31 ) & ~31u;
    L.planes = at;  at = up256 ( at + ( size_t ) B * stride * 4 );
    L.vmask = at;   at = up256 ( at + ( size_t ) nblk * 4 );
    L.emask = at;   at = up256 ( at + ( size_t ) nblk * 4 );
    L.wplanes = at; at = up256 ( at + ( size_t ) B * U * 4 );
    L.u_acc = at;   at = up256 ( at + ( size_t ) U * 4 );
    L.v_acc = at;   at = up256 ( at + ( size_t ) U * 4 );
    L.flags = at;   at = up256 ( at + ( size_t ) U );
    L.chunks = at;  at = up256 ( at + ( size_t ) nchunks * sizeof ( ChunkInfo ) );
    L.err = at;     at = up256 ( at + 4 );
    L.total = at;
    return L;
}

// The two driver calls used below, taken through the runtime's driver entry
// point query so that the library does not link libcuda itself (hosts
// without a driver still load it).  Called with g_mu held.
typedef CUresult ( *PfnCtxGetCurrent ) ( CUcontext * );
typedef CUresult ( *PfnCtxGetId ) ( CUcontext, unsigned long long * );
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

bool driver_calls ()
{
    if ( g_ctx_get_current && g_ctx_get_id ) return true;
    void * a = nullptr;
    void * b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if ( cudaGetDriverEntryPointByVersion ( "cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa ) != cudaSuccess ||
         qa != cudaDriverEntryPointSuccess || ! a )
        return false;
    if ( cudaGetDriverEntryPointByVersion ( "cuCtxGetId", &b, 12000, cudaEnableDefault, &qb ) != cudaSuccess ||
         qb != cudaDriverEntryPointSuccess || ! b )
        return false;
    g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent> ( a );
    g_ctx_get_id = reinterpret_cast<PfnCtxGetId> ( b );
    return true;
}

// Unique id of the calling thread's current CUDA context; 0 if none is current.
unsigned long long current_ctx_id ()
{
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if ( g_ctx_get_current ( &c ) != CUDA_SUCCESS || ! c ) return 0;
    if ( g_ctx_get_id ( c, &id ) != CUDA_SUCCESS ) return 0;
    return id;
}

// Device address of the static scratch array for device `dev` (current) in
// the current context.  In host code g_pair_scratch names a host-side
// stand-in, never a device address, so kernels only ever receive this
// looked-up pointer.
cudaError_t scratch_address ( int dev, uint8_t ** out )
{
    std::lock_guard<std::mutex> lk ( g_mu );
    if ( ! driver_calls () ) return cudaErrorNotSupported;
    ScratchAddr & s = g_scratch[dev];
    const unsigned long long id = current_ctx_id ();
    if ( id == 0 || id != s.ctx_id )
    {
        void * p = nullptr;
        // binds the device's primary context to this thread if none is current
        const cudaError_t e = cudaGetSymbolAddress ( &p, g_pair_scratch );
        if ( e != cudaSuccess ) return e;
        const unsigned long long now = current_ctx_id ();
        if ( now == 0 ) return cudaErrorInvalidDevice;
        s.ctx_id = now;
        s.addr = static_cast<uint8_t *> ( p );
    }
    *out = s.addr;
    return cudaSuccess;
}

// Zero the accumulators and the error word; write the text chunk table.
__global__ void k_na_setup ( ChunkInfo * chunks, uint32_t nchunks, uint32_t nblk, uint32_t warmup, uint32_t * u_acc,
                             uint32_t * v_acc, uint8_t * flags, uint32_t U, uint32_t * err )
{
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    for ( uint32_t i = tid; i < U; i += nthr )
    {
        u_acc[i] = 0;
        v_acc[i] = 0;
        flags[i] = 0;
    }
    if ( tid == 0 ) *err = 0;
    for ( uint32_t c = tid; c < nchunks; c += nthr )
    {
        ChunkInfo ch;
        ch.begin = ( uint32_t ) ( ( uint64_t ) nblk * c / nchunks );
        ch.end = ( uint32_t ) ( ( uint64_t ) nblk * ( c + 1 ) / nchunks );
        const int64_t w = ( int64_t ) ch.begin * 32 - ( int64_t ) warmup;
        ch.warm = ( c == 0 ) ? ch.begin : ( w <= 0 ? 0u : ( uint32_t ) ( w / 32 ) );
        // one text sequence: every inner chunk boundary cuts it (split row 0)
        ch.first_split = c > 0 ? 0 : -1;
        ch.last_split = c + 1 < nchunks ? 0 : -1;
        chunks[c] = ch;
    }
}

// Text t (one sequence): bit planes, match-end and sequence-end masks.
__global__ void k_na_text ( const uint8_t * __restrict__ t, uint32_t n, AlphaMap am, int B, uint32_t vstart,
                            uint32_t * planes, uint32_t stride, uint32_t * vmask, uint32_t * emask, uint32_t nblk,
                            uint32_t * err )
{
    const int lane = threadIdx.x & 31;
    const uint32_t warps = ( gridDim.x * blockDim.x ) >> 5;
    if ( blockIdx.x == 0 && threadIdx.x < ( unsigned ) B ) planes[( size_t ) threadIdx.x * stride] = 0;
    for ( uint32_t k = ( blockIdx.x * blockDim.x + threadIdx.x ) >> 5; k < nblk; k += warps )
    {
        const uint32_t pos = k * 32 + lane;
        uint32_t code = 0;
        bool valid = false;
        if ( pos < n )
        {
            code = am.code[t[pos]];
            if ( code == 0xffu ) { atomicOr ( err, 1u ); code = 0; }
            valid = pos >= vstart;
        }
        for ( int b = 0; b < B; ++b )
        {
            const uint32_t pl = __ballot_sync ( 0xffffffffu, ( code >> b ) & 1u );
            if ( lane == 0 ) planes[( size_t ) b * stride + k + 1] = pl;
        }
        const uint32_t vm = __ballot_sync ( 0xffffffffu, valid );
        const uint32_t em = __ballot_sync ( 0xffffffffu, pos == n - 1 );
        if ( lane == 0 ) { vmask[k] = vm; emask[k] = em; }
    }
}

// Bit planes of every factor p[w..w+l-1] (top-aligned for Hamming).
__global__ void k_na_words ( const uint8_t * __restrict__ p, uint32_t l, AlphaMap am, int B, int top_aligned,
                             uint32_t * wpl, uint32_t U, uint32_t * err )
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if ( w >= U ) return;
    uint32_t pl[kMaxPlanes] = { 0, 0, 0, 0, 0 };
    for ( uint32_t q = 0; q < l; ++q )
    {
        uint32_t c = am.code[p[w + q]];
        if ( c == 0xffu ) { atomicOr ( err, 1u ); c = 0; }
        const uint32_t bit = top_aligned ? ( 32 - l + q ) : q;
#pragma unroll
        for ( int b = 0; b < kMaxPlanes; ++b ) pl[b] |= ( ( c >> b ) & 1u ) << bit;
    }
    for ( int b = 0; b < B; ++b ) wpl[( size_t ) b * U + w] = pl[b];
}

// u[l-1+w] += occurs(w), v[l-1+w] += occurrences(w) -- skipped on bad input.
__global__ void k_na_accumulate ( const uint32_t * u_acc, const uint32_t * v_acc, const uint8_t * flags, int split,
                                  uint32_t U, uint32_t l, const uint32_t * err, uint32_t * d_u, uint32_t * d_v )
{
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if ( w >= U || *err ) return;
    d_u[l - 1 + w] += u_acc[w] + ( split ? flags[w] : 0u );
    d_v[l - 1 + w] += v_acc[w];
}

} // namespace

extern "C" int motex_gpu_extract_pair_static ( const motex_params * prm, const char * alphabet, const char * d_p,
                                               uint32_t m, const char * d_t, uint32_t n, uint32_t * d_u,
                                               uint32_t * d_v, void * stream )
{
    if ( ! prm || ! alphabet || ! d_p || ! d_t || ! d_u || ! d_v ) return MOTEX_EINVAL;
    if ( prm->d > 1 || prm->l == 0 || prm->e >= prm->l ) return MOTEX_EINVAL;
    if ( prm->nb_gaps ) return MOTEX_EUNSUPPORTED;
    if ( prm->l > 32 ) return MOTEX_EUNSUPPORTED;                   // fast kernels only
    if ( m > kMaxPattern || n > kMaxText ) return MOTEX_EUNSUPPORTED;
    if ( m < prm->l || n == 0 ) return MOTEX_OK;                    // no factor: nothing to add
    AlphaMap am;
    for ( int i = 0; i < 256; ++i ) am.code[i] = 0xff;
    uint32_t sigma = 0;
    for ( const char * a = alphabet; *a; ++a )
    {
        if ( sigma >= ( 1u << kMaxPlanes ) ) return MOTEX_EUNSUPPORTED;
        am.code[( uint8_t ) *a] = ( uint8_t ) sigma++;
    }
    if ( sigma == 0 ) return MOTEX_EINVAL;
    int B = 2;                                    // the DP kernels start at two bit planes
    while ( ( 1u << B ) < sigma ) ++B;

    // an error some earlier work left pending is reported and left pending,
    // so that the launch checks below see only this call's launches
    if ( cudaPeekAtLastError () != cudaSuccess ) return MOTEX_ECUDA;
    int dev = 0;
    if ( cudaGetDevice ( &dev ) != cudaSuccess || dev < 0 || dev >= kMaxDevices ) return MOTEX_ECUDA;
    uint8_t * base = nullptr;
    if ( scratch_address ( dev, &base ) != cudaSuccess ) return MOTEX_ECUDA;
    int sms = 0;
    if ( cudaDeviceGetAttribute ( &sms, cudaDevAttrMultiProcessorCount, dev ) != cudaSuccess || sms <= 0 )
        return MOTEX_ECUDA;
    cudaStream_t st = static_cast<cudaStream_t> ( stream );

    const bool ed = prm->d == 1;
    const uint32_t l = prm->l;
    const uint32_t U = m - l + 1;
    const uint32_t nblk = ( n + 31 ) / 32;
    const int W = U >= ( uint32_t ) sms * kDPThreads * 8 ? 8 : 4;
    const uint32_t per_cta = ( uint32_t ) kDPThreads * W;
    const uint32_t ntiles = ( U + per_cta - 1 ) / per_cta;
    uint32_t nchunks = ( ( uint32_t ) sms * 24 + ntiles - 1 ) / ntiles;
    nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, nblk / ( ed ? 16 : 4 ) ) );
    nchunks = std::max<uint32_t> ( 1, std::min<uint32_t> ( nchunks, kMaxChunks ) );
    const Layout L = layout_for ( ( uint32_t ) B, nblk, U, nchunks );
    if ( L.total > kStaticScratchBytes ) return MOTEX_EUNSUPPORTED;
    const uint32_t stride = ( nblk + 1 + 31 ) & ~31u;

    uint32_t * planes = reinterpret_cast<uint32_t *> ( base + L.planes );
    uint32_t * vmask = reinterpret_cast<uint32_t *> ( base + L.vmask );
    uint32_t * emask = reinterpret_cast<uint32_t *> ( base + L.emask );
    uint32_t * wpl = reinterpret_cast<uint32_t *> ( base + L.wplanes );
    uint32_t * u_acc = reinterpret_cast<uint32_t *> ( base + L.u_acc );
    uint32_t * v_acc = reinterpret_cast<uint32_t *> ( base + L.v_acc );
    uint8_t * flags = base + L.flags;
    ChunkInfo * chunks = reinterpret_cast<ChunkInfo *> ( base + L.chunks );
    uint32_t * err = reinterpret_cast<uint32_t *> ( base + L.err );

    const uint32_t warmup = ed ? l + prm->e - 1 : 0;
    k_na_setup<<<std::max<uint32_t> ( 1, std::min<uint32_t> ( 4 * sms, ( U + 255 ) / 256 ) ), 256, 0, st>>> (
        chunks, nchunks, nblk, warmup, u_acc, v_acc, flags, U, err );
    k_na_text<<<std::max<uint32_t> ( 1, std::min<uint32_t> ( 16 * sms, ( nblk + 7 ) / 8 ) ), 256, 0, st>>> (
        reinterpret_cast<const uint8_t *> ( d_t ), n, am, B, ed ? 0 : l - 1, planes, stride, vmask, emask, nblk, err );
    k_na_words<<<( U + 255 ) / 256, 256, 0, st>>> ( reinterpret_cast<const uint8_t *> ( d_p ), l, am, B, ed ? 0 : 1,
                                                     wpl, U, err );
    DPArgs da;
    da.text.planes = planes;
    da.text.plane_stride = stride;
    da.text.vmask = vmask;
    da.text.emask = emask;
    da.text.nblk = nblk;
    da.wplanes32 = wpl;
    da.wplanes64 = nullptr;
    da.U = U;
    da.l = l;
    da.e = prm->e;
    da.one = 1u;
    da.two = 2u;
    da.neg1 = ~0u;
    da.chunks = chunks;
    da.u_acc = u_acc;
    da.v_acc = v_acc;
    da.split_flags = flags;
    if ( ! launch_dp_fast ( da, B, W, 8, ed, dim3 ( ntiles, nchunks ), st ) ) return MOTEX_EUNSUPPORTED;
    k_na_accumulate<<<( U + 255 ) / 256, 256, 0, st>>> ( u_acc, v_acc, flags, nchunks > 1, U, l, err, d_u, d_v );
    if ( cudaGetLastError () != cudaSuccess ) return MOTEX_ECUDA;
    // report symbols outside the alphabet (the outputs were left untouched)
    uint32_t h_err = 0;
    if ( cudaMemcpyAsync ( &h_err, err, 4, cudaMemcpyDeviceToHost, st ) != cudaSuccess ) return MOTEX_ECUDA;
    if ( cudaStreamSynchronize ( st ) != cudaSuccess ) return MOTEX_ECUDA;
    return h_err ? MOTEX_EINVAL : MOTEX_OK;
}
