// C-ABI entry points (include/motex_gpu.h) and the device pipeline behind them:
//   upload -> symbol presence -> pack (codes, bit planes, masks, factor ends)
//   -> stable LSD radix sort of factor keys -> dedup (first occurrence kept)
//   -> factor planes -> DP over (unique factors x text chunks)
//   -> quorum filter at first occurrences -> ordered compaction -> download.
#include "motex_gpu.h"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_set>
#include <vector>

using namespace mtx;

namespace
{

thread_local std::string g_last_error;

int fail ( int code, const char * fmt, ... )
{
    char buf[512];
    va_list ap;
    va_start ( ap, fmt );
    vsnprintf ( buf, sizeof buf, fmt, ap );
    va_end ( ap );
    g_last_error = buf;
    return code;
}

#define MTX_CUDA( call )                                                                            \
    do {                                                                                            \
        cudaError_t err_ = ( call );                                                                \
        if ( err_ != cudaSuccess )                                                                  \
            return fail ( MOTEX_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString ( err_ ), \
                          __FILE__, __LINE__ );                                                     \
    } while ( 0 )

#define MTX_TRY( call )                                                                             \
    do {                                                                                            \
        int rc_ = ( call );                                                                         \
        if ( rc_ != MOTEX_OK ) return rc_;                                                          \
    } while ( 0 )

struct DevBuf
{
    void * p = nullptr;
    size_t cap = 0;
};

enum Slot
{
    S_RAW, S_OFFS, S_WSTART, S_QOK, S_CMAP, S_PRESENT, S_CODES, S_PLANES, S_VMASK, S_EMASK,
    S_WPOS, S_KEY0, S_KEY1, S_IDX1, S_HIST, S_HEAD, S_PREF, S_UNIQ, S_WPL32, S_WPL64,
    S_CHUNKS, S_UACC, S_VACC, S_FLAGS, S_MARK, S_RECU, S_RECV, S_PREF2, S_RECS, S_TILES,
    S_SCALAR, S_UOUT, S_VOUT, S_WPL0, S_WPL1, S_ROWOK, S_ROWEND, S_COUNT
};

} // namespace

struct DPTune
{
    int W = 8;     // register words per thread
    int NL = 1;    // factors per register word
    int UR = 8;    // unroll of the 32-position block
};

struct motex_ctx
{
    int device = 0;
    int num_sms = 148;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evd0 = nullptr, evd1 = nullptr;
    uint64_t launches = 0;
    uint32_t job_launches = 0;
    DevBuf buf[S_COUNT];
    void * pinned = nullptr;
    size_t pinned_cap = 0;

    // loaded job
    bool loaded = false, executed = false;
    motex_params prm {};
    std::vector<uint32_t> gmin, gmax, blens, berrs;
    uint32_t nseq = 0;
    std::vector<uint32_t> offs;                // nseq + 1
    uint64_t total = 0;
    uint32_t tml = 0;
    uint32_t nwords = 0;
    bool pair_mode = false;
    uint64_t ref_cells = 0;
    uint32_t G = 1;                            // gap choices (1 for single motifs)
    std::vector<char> raw_host;                // structured runs: input copy for key dedup

    // executed job
    int B = 0;
    uint32_t U = 0, nblk = 0, n_split = 0, nrec = 0;
    uint64_t exec_cells = 0;
    float device_ms = 0.f, dp_ms = 0.f;
    DPTune tune;
};

namespace
{

template <typename T>
int ensure ( motex_ctx * c, Slot s, size_t count, T ** out )
{
    size_t bytes = std::max<size_t> ( 1, count * sizeof ( T ) );
    DevBuf & b = c->buf[s];
    if ( b.cap < bytes )
    {
        if ( b.p ) cudaFree ( b.p );
        b.p = nullptr;
        b.cap = 0;
        size_t want = bytes + bytes / 4;
        if ( cudaMalloc ( &b.p, want ) != cudaSuccess )
        {
            cudaGetLastError ();
            return fail ( MOTEX_ENOMEM, "device allocation of %zu bytes failed", want );
        }
        b.cap = want;
    }
    *out = static_cast<T *> ( b.p );
    return MOTEX_OK;
}

template <typename T>
T * dptr ( motex_ctx * c, Slot s ) { return static_cast<T *> ( c->buf[s].p ); }

int ensure_pinned ( motex_ctx * c, size_t bytes )
{
    if ( c->pinned_cap >= bytes ) return MOTEX_OK;
    if ( c->pinned ) cudaFreeHost ( c->pinned );
    c->pinned = nullptr;
    c->pinned_cap = 0;
    size_t want = bytes + bytes / 4 + 4096;
    if ( cudaHostAlloc ( &c->pinned, want, cudaHostAllocDefault ) != cudaSuccess )
    {
        cudaGetLastError ();
        return fail ( MOTEX_ENOMEM, "pinned host allocation of %zu bytes failed", want );
    }
    c->pinned_cap = want;
    return MOTEX_OK;
}

int check_launch ( motex_ctx * c, const char * what )
{
    c->launches++;
    c->job_launches++;
    cudaError_t e = cudaGetLastError ();
    if ( e != cudaSuccess ) return fail ( MOTEX_ECUDA, "launch of %s failed: %s", what, cudaGetErrorString ( e ) );
    return MOTEX_OK;
}

#define MTX_LAUNCH( name, grid, block, ... )                                                       \
    do {                                                                                            \
        name<<<( grid ), ( block ), 0, c->st>>> ( __VA_ARGS__ );                                    \
        MTX_TRY ( check_launch ( c, #name ) );                                                      \
    } while ( 0 )

unsigned blocks_for ( uint64_t n, unsigned threads ) { return ( unsigned ) std::max<uint64_t> ( 1, ( n + threads - 1 ) / threads ); }

int validate ( const motex_params * p )
{
    if ( ! p ) return fail ( MOTEX_EINVAL, "null parameters" );
    if ( p->d > 1 ) return fail ( MOTEX_EINVAL, "d must be 0 (Hamming) or 1 (edit distance)" );
    if ( p->l == 0 ) return fail ( MOTEX_EINVAL, "factor length must be positive" );
    if ( p->e >= p->l ) return fail ( MOTEX_EINVAL, "e must be less than the factor length" );
    if ( p->l > MOTEX_MAX_FACTOR ) return fail ( MOTEX_EUNSUPPORTED, "factor length %u > %d", p->l, MOTEX_MAX_FACTOR );
    if ( p->nb_gaps )
    {
        if ( ! p->gap_min || ! p->gap_max || ! p->blens || ! p->berrs ) return fail ( MOTEX_EINVAL, "null box arrays" );
        if ( p->nb_gaps > 1 )
            return fail ( MOTEX_EUNSUPPORTED, "structured motifs with %u gaps (one gap is implemented)", p->nb_gaps );
        const uint32_t gmin = p->gap_min[0], gmax = p->gap_max[0], b1 = p->blens[0];
        if ( gmax < gmin ) return fail ( MOTEX_EINVAL, "gap range [%u,%u] is empty", gmin, gmax );
        if ( b1 == 0 ) return fail ( MOTEX_EINVAL, "box length must be positive" );
        if ( p->l > 32 || b1 > 32 || gmax - gmin + 1 > 32 || gmax + b1 > 31 )
            return fail ( MOTEX_EUNSUPPORTED, "structured boxes need l, box length <= 32, gap max + box length <= 31 and at most 32 gap choices" );
        if ( p->berrs[0] >= p->l + gmin + b1 )
            return fail ( MOTEX_EUNSUPPORTED, "box error bound %u not below the minimum motif length", p->berrs[0] );
    }
    return MOTEX_OK;
}

// Exclusive scan of n byte flags; device total written to *d_total (may be null).
int scan_flags ( motex_ctx * c, const uint8_t * in, uint32_t n, uint32_t * out, uint32_t * d_total )
{
    const uint32_t tiles = ( uint32_t ) blocks_for ( n, kScanTile );
    uint32_t * tsum;
    MTX_TRY ( ensure ( c, S_TILES, tiles, &tsum ) );
    cudaError_t e = scan_exclusive_u8 ( in, n, out, d_total, tsum, c->st );
    c->launches += 3;
    c->job_launches += 3;
    if ( e != cudaSuccess ) return fail ( MOTEX_ECUDA, "scan launch failed: %s", cudaGetErrorString ( e ) );
    return MOTEX_OK;
}

// Stable sort of the factor ends in idx by their packed keys; result in *idx_out.
int sort_factors ( motex_ctx * c, uint32_t n, uint32_t ** idx_out )
{
    const uint32_t l = c->prm.l, B = ( uint32_t ) c->B;
    const uint32_t bits = l * B;
    const uint32_t nchunk = ( bits + 31 ) / 32;
    const uint32_t ntiles = ( uint32_t ) blocks_for ( n, kSortTile );
    uint32_t *key0, *key1, *idx1, *hist;
    MTX_TRY ( ensure ( c, S_KEY0, n, &key0 ) );
    MTX_TRY ( ensure ( c, S_KEY1, n, &key1 ) );
    MTX_TRY ( ensure ( c, S_IDX1, n, &idx1 ) );
    MTX_TRY ( ensure ( c, S_HIST, ( size_t ) 256 * ntiles, &hist ) );
    uint32_t * idx0 = dptr<uint32_t> ( c, S_WPOS );
    uint32_t *kin = key0, *kout = key1, *iin = idx0, *iout = idx1;
    for ( uint32_t ch = 0; ch < nchunk; ++ch )
    {
        MTX_LAUNCH ( k_gather_key, blocks_for ( n, 256 ), 256, iin, n, dptr<uint8_t> ( c, S_CODES ), l, B, 32 * ch, kin );
        const uint32_t cbits = std::min<uint32_t> ( 32, bits - 32 * ch );
        for ( uint32_t pass = 0; pass * 8 < cbits; ++pass )
        {
            MTX_LAUNCH ( k_radix_hist, ntiles, kSortThreads, kin, n, ( int ) ( 8 * pass ), hist, ntiles );
            MTX_LAUNCH ( k_scan_single, 1, kScanThreads, hist, 256 * ntiles, ( uint32_t * ) nullptr );
            MTX_LAUNCH ( k_radix_scatter, ntiles, kSortThreads, kin, iin, kout, iout, n, ( int ) ( 8 * pass ), hist, ntiles );
            std::swap ( kin, kout );
            std::swap ( iin, iout );
        }
    }
    *idx_out = iin;
    return MOTEX_OK;
}

/*
 * DP launch shape: factors per thread (W), factors per 32-bit register (NL,
 * edit distance with l <= 15 packs 2-4), and the inner unroll of the
 * 32-position text block (UR, bounded to keep the loop in the instruction
 * cache).  MOTEX_DP_W / MOTEX_DP_UR / MOTEX_DP_SWAR=0 override the choice.
 */
DPTune choose_tune ( motex_ctx * c, uint32_t U, bool ed, bool generic )
{
    DPTune t;
    if ( generic ) { t.W = 1; t.NL = 1; t.UR = 32; return t; }
    t.NL = ed ? swar_lanes ( c->prm.l ) : 1;
    const uint32_t groups = ( U + t.NL - 1 ) / t.NL;
    t.W = groups >= ( uint32_t ) c->num_sms * kDPThreads * 8 ? 8 : 4;
    t.UR = ed ? 8 : 4;             // measured on GB300: Hamming prefers the shorter body
    if ( const char * e = getenv ( "MOTEX_DP_SWAR" ) )
        if ( atoi ( e ) == 0 ) t.NL = 1;
    if ( const char * e = getenv ( "MOTEX_DP_W" ) )
        if ( atoi ( e ) == 4 || atoi ( e ) == 8 ) t.W = atoi ( e );
    if ( const char * e = getenv ( "MOTEX_DP_UR" ) )
    {
        const int v = atoi ( e );
        if ( v == 4 || v == 8 || ( v == 32 && t.NL == 1 ) ) t.UR = v;
    }
    return t;
}

/*
 * Text chunks for the DP grid: equal block ranges; sequences cut by a chunk
 * boundary get a split index (one flag row each).  warmup = positions a
 * chunk must process before its first counted one (edit distance: l+e-1,
 * generic Hamming: l-1, fast Hamming: 0).
 */
void build_chunks ( motex_ctx * c, uint32_t first_blk, uint32_t nchunks, uint32_t warmup, std::vector<ChunkInfo> & out )
{
    const uint32_t nblk = c->nblk;
    const uint32_t span = nblk - first_blk;
    nchunks = std::max<uint32_t> ( 1, std::min ( nchunks, span ) );
    std::map<uint32_t, int> split_of;
    auto seq_at = [&] ( uint64_t pos ) -> uint32_t {
        // largest s with offs[s] <= pos, skipping empty sequences
        uint32_t s = ( uint32_t ) ( std::upper_bound ( c->offs.begin (), c->offs.end (), ( uint32_t ) pos ) - c->offs.begin () ) - 1;
        return s;
    };
    auto split_idx = [&] ( uint32_t s ) {
        auto it = split_of.find ( s );
        if ( it != split_of.end () ) return it->second;
        int id = ( int ) split_of.size ();
        split_of[s] = id;
        return id;
    };
    out.clear ();
    for ( uint32_t i = 0; i < nchunks; ++i )
    {
        ChunkInfo ch;
        ch.begin = first_blk + ( uint32_t ) ( ( uint64_t ) span * i / nchunks );
        ch.end = first_blk + ( uint32_t ) ( ( uint64_t ) span * ( i + 1 ) / nchunks );
        const uint64_t P = ( uint64_t ) ch.begin * 32;
        const int64_t wpos = ( int64_t ) P - ( int64_t ) warmup;
        ch.warm = ( i == 0 || wpos <= 0 ) ? ( i == 0 ? ch.begin : 0 ) : ( uint32_t ) ( wpos / 32 );
        if ( ch.warm < first_blk ) ch.warm = first_blk;
        ch.first_split = -1;
        ch.last_split = -1;
        if ( i > 0 && P < c->total )
        {
            uint32_t s = seq_at ( P );
            if ( c->offs[s] < P ) ch.first_split = split_idx ( s );
        }
        const uint64_t E = ( uint64_t ) ch.end * 32;
        if ( i + 1 < nchunks && E < c->total )
        {
            uint32_t s = seq_at ( E );
            if ( c->offs[s] < E ) ch.last_split = split_idx ( s );
        }
        out.push_back ( ch );
    }
    c->n_split = ( uint32_t ) split_of.size ();
}

/*
 * Structured motifs (one gap): box planes for every pattern position, the
 * two-box DP over (pattern position x text chunk), then per (position, gap
 * choice) filter and ordered compaction.  Factors are not deduplicated here:
 * u and v are computed per pattern position like the reference, and the
 * key deduplication of the writer happens on the passing entries only.
 */
int run_structured ( motex_ctx * c, const uint8_t * codes, uint32_t * planes, uint32_t stride, uint32_t * vmask,
                     uint32_t * emask, uint32_t * scalar, uint32_t * h_scalar, bool & dp_timed )
{
    const motex_params & P = c->prm;
    const bool ed = P.d == 1;
    cudaStream_t st = c->st;
    const int B = c->B;
    const uint32_t T = ( uint32_t ) c->total, G = c->G;
    const uint32_t b1 = c->blens[0], e1 = c->berrs[0], gmin = c->gmin[0], gmax = c->gmax[0];
    uint32_t *wpl0, *wpl1, *row_end;
    uint8_t * row_ok;
    MTX_TRY ( ensure ( c, S_WPL0, ( size_t ) B * T, &wpl0 ) );
    MTX_TRY ( ensure ( c, S_WPL1, ( size_t ) B * T, &wpl1 ) );
    MTX_TRY ( ensure ( c, S_ROWOK, T, &row_ok ) );
    MTX_TRY ( ensure ( c, S_ROWEND, T, &row_end ) );
    MTX_LAUNCH ( k_wplanes_all, blocks_for ( T, 256 ), 256, codes, T, P.l, ( uint32_t ) B, ed ? 0 : 1, wpl0 );
    MTX_LAUNCH ( k_wplanes_all, blocks_for ( T, 256 ), 256, codes, T, b1, ( uint32_t ) B, ed ? 0 : 1, wpl1 );
    MTX_LAUNCH ( k_struct_rows, blocks_for ( T, 256 ), 256, dptr<uint32_t> ( c, S_OFFS ), c->nseq, c->total, P.l,
                 c->tml, ( int ) c->pair_mode, row_ok, row_end );

    const uint32_t ctas_x = ( T + kDPThreads - 1 ) / kDPThreads;
    const uint32_t first_blk = c->pair_mode ? ( c->offs[1] / 32 ) : 0;
    const uint32_t warmup = ( ed ? std::max ( P.l + P.e - 1, b1 + e1 - 1 ) : 0 ) + gmax + b1;
    uint32_t nchunks = std::max<uint32_t> ( 1, ( ( uint32_t ) c->num_sms * 24 + ctas_x - 1 ) / ctas_x );
    nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, ( c->nblk - first_blk ) / 16 ) );
    nchunks = std::min<uint32_t> ( nchunks, 2048 );
    std::vector<ChunkInfo> chunks;
    build_chunks ( c, first_blk, nchunks, warmup, chunks );
    ChunkInfo * h_chunks = reinterpret_cast<ChunkInfo *> ( static_cast<uint8_t *> ( c->pinned ) + 4096 );
    std::copy ( chunks.begin (), chunks.end (), h_chunks );
    ChunkInfo * d_chunks;
    MTX_TRY ( ensure ( c, S_CHUNKS, chunks.size (), &d_chunks ) );
    MTX_CUDA ( cudaMemcpyAsync ( d_chunks, h_chunks, chunks.size () * sizeof ( ChunkInfo ), cudaMemcpyHostToDevice, st ) );
    uint64_t scanned = 0;
    for ( auto & ch : chunks ) scanned += ( uint64_t ) ( ch.end - ch.warm ) * 32;
    c->exec_cells = ( uint64_t ) T * scanned * 2;

    const uint64_t n = ( uint64_t ) T * G;
    if ( n >= 0xffffff00ull ) return fail ( MOTEX_EUNSUPPORTED, "positions x gap choices exceeds 2^32" );
    uint32_t *u_acc, *v_acc;
    uint8_t * flags;
    MTX_TRY ( ensure ( c, S_UACC, n, &u_acc ) );
    MTX_TRY ( ensure ( c, S_VACC, n, &v_acc ) );
    MTX_TRY ( ensure ( c, S_FLAGS, std::max<uint64_t> ( 1, c->n_split ) * n, &flags ) );
    MTX_CUDA ( cudaMemsetAsync ( u_acc, 0, n * 4, st ) );
    MTX_CUDA ( cudaMemsetAsync ( v_acc, 0, n * 4, st ) );
    if ( c->n_split ) MTX_CUDA ( cudaMemsetAsync ( flags, 0, ( size_t ) c->n_split * n, st ) );

    StructArgs sa;
    sa.text.planes = planes;
    sa.text.plane_stride = stride;
    sa.text.vmask = vmask;
    sa.text.emask = emask;
    sa.text.nblk = c->nblk;
    sa.wpl0 = wpl0;
    sa.wpl1 = wpl1;
    sa.row_ok = row_ok;
    sa.row_end = row_end;
    sa.total = T;
    sa.l0 = P.l;
    sa.e0 = P.e;
    sa.l1 = b1;
    sa.e1 = e1;
    sa.b1 = b1;
    sa.gmin = gmin;
    sa.gmax = gmax;
    sa.G = G;
    sa.chunks = d_chunks;
    sa.u_acc = u_acc;
    sa.v_acc = v_acc;
    sa.split_flags = flags;
    MTX_CUDA ( cudaEventRecord ( c->evd0, st ) );
    if ( ! launch_dp_struct1 ( sa, B, ed, dim3 ( ctas_x, ( unsigned ) chunks.size () ), st ) )
        return fail ( MOTEX_EUNSUPPORTED, "no structured DP kernel for this box shape" );
    MTX_TRY ( check_launch ( c, "k_dp_struct1" ) );
    MTX_CUDA ( cudaEventRecord ( c->evd1, st ) );
    dp_timed = true;
    c->U = T;

    StructFinalizeArgs fa {};
    fa.n = n;
    fa.u_acc = u_acc;
    fa.v_acc = v_acc;
    fa.split_flags = flags;
    fa.n_split = c->n_split;
    fa.qok = dptr<uint8_t> ( c, S_QOK );
    fa.nseq = c->nseq;
    fa.nmin = P.n;
    fa.nmax = P.N;
    if ( c->pair_mode )
    {
        uint32_t *uo, *vo;
        MTX_TRY ( ensure ( c, S_UOUT, n, &uo ) );
        MTX_TRY ( ensure ( c, S_VOUT, n, &vo ) );
        fa.u_out = uo;
        fa.v_out = vo;
        MTX_LAUNCH ( k_struct_finalize, blocks_for ( n, 256 ), 256, fa );
        c->nrec = 0;
        return MOTEX_OK;
    }
    uint8_t * mark;
    uint32_t *recu, *recv, *pref2, *recs;
    MTX_TRY ( ensure ( c, S_MARK, n, &mark ) );
    MTX_TRY ( ensure ( c, S_RECU, n, &recu ) );
    MTX_TRY ( ensure ( c, S_RECV, n, &recv ) );
    MTX_TRY ( ensure ( c, S_PREF2, n, &pref2 ) );
    fa.mark = mark;
    fa.rec_u = recu;
    fa.rec_v = recv;
    MTX_LAUNCH ( k_struct_finalize, blocks_for ( n, 256 ), 256, fa );
    MTX_TRY ( scan_flags ( c, mark, ( uint32_t ) n, pref2, scalar ) );
    MTX_CUDA ( cudaMemcpyAsync ( h_scalar, scalar, 4, cudaMemcpyDeviceToHost, st ) );
    MTX_CUDA ( cudaStreamSynchronize ( st ) );
    c->nrec = h_scalar[0];
    MTX_TRY ( ensure ( c, S_RECS, ( size_t ) 3 * std::max<uint32_t> ( 1, c->nrec ), &recs ) );
    MTX_LAUNCH ( k_compact, blocks_for ( n, 256 ), 256, mark, pref2, ( uint32_t ) n, recu, recv, recs );
    return MOTEX_OK;
}

int run_pipeline ( motex_ctx * c )
{
    const motex_params & P = c->prm;
    const bool ed = P.d == 1;
    cudaStream_t st = c->st;
    MTX_CUDA ( cudaEventRecord ( c->ev0, st ) );

    // symbol alphabet actually present -> dense codes, B bit planes
    uint32_t * present;
    MTX_TRY ( ensure ( c, S_PRESENT, 256, &present ) );
    MTX_CUDA ( cudaMemsetAsync ( present, 0, 256 * sizeof ( uint32_t ), st ) );
    MTX_LAUNCH ( k_presence, std::min<unsigned> ( 4 * c->num_sms, blocks_for ( c->total, 256 * 16 ) ), 256,
                 dptr<uint8_t> ( c, S_RAW ), c->total, present );
    uint32_t * h_present = static_cast<uint32_t *> ( c->pinned );
    MTX_CUDA ( cudaMemcpyAsync ( h_present, present, 256 * sizeof ( uint32_t ), cudaMemcpyDeviceToHost, st ) );
    MTX_CUDA ( cudaStreamSynchronize ( st ) );
    uint8_t * h_cmap = static_cast<uint8_t *> ( c->pinned ) + 1024;
    uint32_t sigma = 0;
    for ( int i = 0; i < 256; ++i ) h_cmap[i] = h_present[i] ? ( uint8_t ) sigma++ : 0;
    int B = 2;                                   // one- and two-symbol inputs run on the 2-plane kernels
    while ( ( 1u << B ) < sigma ) ++B;
    if ( B > kMaxPlanes ) return fail ( MOTEX_EUNSUPPORTED, "%u distinct symbols need %d bit planes (max %d)", sigma, B, kMaxPlanes );
    c->B = B;
    uint8_t * cmap;
    MTX_TRY ( ensure ( c, S_CMAP, 256, &cmap ) );
    MTX_CUDA ( cudaMemcpyAsync ( cmap, h_cmap, 256, cudaMemcpyHostToDevice, st ) );

    // pack
    c->nblk = ( uint32_t ) ( ( c->total + 31 ) / 32 );
    const uint32_t stride = ( c->nblk + 1 + 31 ) & ~31u;
    uint8_t * codes;
    uint32_t *planes, *vmask, *emask, *wpos;
    MTX_TRY ( ensure ( c, S_CODES, c->total + 64, &codes ) );
    MTX_TRY ( ensure ( c, S_PLANES, ( size_t ) B * stride, &planes ) );
    MTX_TRY ( ensure ( c, S_VMASK, c->nblk, &vmask ) );
    MTX_TRY ( ensure ( c, S_EMASK, c->nblk, &emask ) );
    MTX_TRY ( ensure ( c, S_WPOS, c->nwords, &wpos ) );
    MTX_CUDA ( cudaMemsetAsync ( planes, 0, ( size_t ) B * stride * sizeof ( uint32_t ), st ) );
    const bool generic = P.l > 32;
    PackArgs pa;
    pa.raw = dptr<uint8_t> ( c, S_RAW );
    pa.total = c->total;
    pa.offs = dptr<uint32_t> ( c, S_OFFS );
    pa.nseq = c->nseq;
    pa.cmap = cmap;
    pa.B = B;
    pa.l = P.l;
    pa.tml = c->tml;
    pa.vstart = ed ? 0 : P.l - 1;
    pa.pair_mode = c->pair_mode;
    pa.wstart = dptr<uint32_t> ( c, S_WSTART );
    pa.codes = codes;
    pa.planes = planes;
    pa.plane_stride = stride;
    pa.vmask = vmask;
    pa.emask = emask;
    pa.wpos = wpos;
    pa.nblk = c->nblk;
    MTX_LAUNCH ( k_pack, std::min<unsigned> ( 16 * c->num_sms, blocks_for ( c->nblk, 8 ) ), 256, pa );

    uint32_t * scalar;
    MTX_TRY ( ensure ( c, S_SCALAR, 4, &scalar ) );
    uint32_t * h_scalar = reinterpret_cast<uint32_t *> ( static_cast<uint8_t *> ( c->pinned ) + 2048 );
    c->n_split = 0;
    c->exec_cells = 0;
    c->dp_ms = 0.f;
    if ( P.nb_gaps )
    {
        bool timed = false;
        MTX_TRY ( run_structured ( c, codes, planes, stride, vmask, emask, scalar, h_scalar, timed ) );
        MTX_CUDA ( cudaEventRecord ( c->ev1, st ) );
        MTX_CUDA ( cudaEventSynchronize ( c->ev1 ) );
        MTX_CUDA ( cudaEventElapsedTime ( &c->device_ms, c->ev0, c->ev1 ) );
        if ( timed ) MTX_CUDA ( cudaEventElapsedTime ( &c->dp_ms, c->evd0, c->evd1 ) );
        return MOTEX_OK;
    }

    // dedup (whole-set runs); the pair drop-in searches every factor as is
    uint32_t * uniq = wpos;
    c->U = c->nwords;
    if ( ! c->pair_mode && c->nwords > 0 )
    {
        uint32_t * idx;
        MTX_TRY ( sort_factors ( c, c->nwords, &idx ) );
        uint8_t * head;
        uint32_t * pref;
        MTX_TRY ( ensure ( c, S_HEAD, c->nwords, &head ) );
        MTX_TRY ( ensure ( c, S_PREF, c->nwords, &pref ) );
        MTX_LAUNCH ( k_heads, blocks_for ( c->nwords, 256 ), 256, idx, c->nwords, codes, P.l, head );
        MTX_TRY ( scan_flags ( c, head, c->nwords, pref, scalar ) );
        MTX_CUDA ( cudaMemcpyAsync ( h_scalar, scalar, 4, cudaMemcpyDeviceToHost, st ) );
        MTX_CUDA ( cudaStreamSynchronize ( st ) );
        c->U = h_scalar[0];
        MTX_TRY ( ensure ( c, S_UNIQ, c->U, &uniq ) );
        MTX_LAUNCH ( k_unique, blocks_for ( c->nwords, 256 ), 256, idx, head, pref, c->nwords, uniq );
    }
    const uint32_t U = c->U;

    uint32_t *u_acc, *v_acc;
    MTX_TRY ( ensure ( c, S_UACC, U, &u_acc ) );
    MTX_TRY ( ensure ( c, S_VACC, U, &v_acc ) );
    bool dp_timed = false;
    if ( U > 0 )
    {
        // factor planes + DP
        DPArgs da;
        da.text.planes = planes;
        da.text.plane_stride = stride;
        da.text.vmask = vmask;
        da.text.emask = emask;
        da.text.nblk = c->nblk;
        da.U = U;
        da.l = P.l;
        da.e = P.e;
        da.wplanes32 = nullptr;
        da.wplanes64 = nullptr;
        const DPTune tune = choose_tune ( c, U, ed, generic );
        const int W = tune.W;
        const uint32_t groups = ( U + tune.NL - 1 ) / tune.NL;        // factors per register: NL
        const uint32_t per_cta = ( uint32_t ) kDPThreads * W;
        const uint32_t ntiles = ( groups + per_cta - 1 ) / per_cta;
        uint32_t nw64 = ( P.l + 63 ) / 64;
        if ( ! generic )
        {
            uint32_t * wpl;
            MTX_TRY ( ensure ( c, S_WPL32, ( size_t ) B * U, &wpl ) );
            MTX_LAUNCH ( k_wplanes32, blocks_for ( U, 256 ), 256, uniq, U, codes, P.l, ( uint32_t ) B, ed ? 0 : 1, wpl );
            da.wplanes32 = wpl;
        }
        else
        {
            uint64_t * wpl;
            MTX_TRY ( ensure ( c, S_WPL64, ( size_t ) B * U * nw64, &wpl ) );
            MTX_LAUNCH ( k_wplanes64, blocks_for ( U, 128 ), 128, uniq, U, codes, P.l, ( uint32_t ) B, nw64, ed ? 0 : 1, wpl );
            da.wplanes64 = wpl;
        }
        const uint32_t first_blk = c->pair_mode ? ( c->offs[1] / 32 ) : 0;
        const uint32_t warmup = ed ? P.l + P.e - 1 : ( generic ? P.l - 1 : 0 );
        const uint32_t target = ( uint32_t ) c->num_sms * 24;
        uint32_t nchunks = std::max<uint32_t> ( 1, ( target + ntiles - 1 ) / ntiles );
        const uint32_t min_blocks = ed ? 16 : 4;
        nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, ( c->nblk - first_blk ) / min_blocks ) );
        nchunks = std::min<uint32_t> ( nchunks, 65535 );
        std::vector<ChunkInfo> chunks;
        build_chunks ( c, first_blk, nchunks, warmup, chunks );
        ChunkInfo * h_chunks = reinterpret_cast<ChunkInfo *> ( static_cast<uint8_t *> ( c->pinned ) + 4096 );
        if ( 4096 + chunks.size () * sizeof ( ChunkInfo ) > c->pinned_cap )
            return fail ( MOTEX_ENOMEM, "chunk table does not fit the staging buffer" );
        std::copy ( chunks.begin (), chunks.end (), h_chunks );
        ChunkInfo * d_chunks;
        MTX_TRY ( ensure ( c, S_CHUNKS, chunks.size (), &d_chunks ) );
        MTX_CUDA ( cudaMemcpyAsync ( d_chunks, h_chunks, chunks.size () * sizeof ( ChunkInfo ), cudaMemcpyHostToDevice, st ) );
        for ( auto & ch : chunks ) c->exec_cells += ( uint64_t ) U * ( ch.end - ch.warm ) * 32;
        uint8_t * flags;
        MTX_TRY ( ensure ( c, S_FLAGS, ( size_t ) std::max<uint32_t> ( 1, c->n_split ) * U, &flags ) );
        MTX_CUDA ( cudaMemsetAsync ( u_acc, 0, ( size_t ) U * 4, st ) );
        MTX_CUDA ( cudaMemsetAsync ( v_acc, 0, ( size_t ) U * 4, st ) );
        if ( c->n_split ) MTX_CUDA ( cudaMemsetAsync ( flags, 0, ( size_t ) c->n_split * U, st ) );
        da.chunks = d_chunks;
        da.u_acc = u_acc;
        da.v_acc = v_acc;
        da.split_flags = flags;
        dim3 grid ( generic ? ( U + kDPThreads - 1 ) / kDPThreads : ntiles, ( unsigned ) chunks.size () );
        MTX_CUDA ( cudaEventRecord ( c->evd0, st ) );
        bool ok = generic        ? launch_dp_generic ( da, B, nw64, ed, grid, st )
                  : tune.NL > 1  ? launch_dp_swar_ed ( da, B, tune.NL, W, tune.UR, grid, st )
                                 : launch_dp_fast ( da, B, W, tune.UR, ed, grid, st );
        c->tune = tune;
        if ( ! ok ) return fail ( MOTEX_EUNSUPPORTED, "no DP kernel for l=%u B=%d", P.l, B );
        MTX_TRY ( check_launch ( c, "k_dp" ) );
        MTX_CUDA ( cudaEventRecord ( c->evd1, st ) );
        dp_timed = true;
    }

    // filter + ordered compaction
    FinalizeArgs fa {};
    fa.U = U;
    fa.u_acc = u_acc;
    fa.v_acc = v_acc;
    fa.split_flags = dptr<uint8_t> ( c, S_FLAGS );
    fa.n_split = c->n_split;
    fa.qok = dptr<uint8_t> ( c, S_QOK );
    fa.nseq = c->nseq;
    fa.nmin = P.n;
    fa.nmax = P.N;
    fa.uniq_pos = uniq;
    if ( c->pair_mode )
    {
        uint32_t *uo, *vo;
        MTX_TRY ( ensure ( c, S_UOUT, std::max<uint32_t> ( 1, U ), &uo ) );
        MTX_TRY ( ensure ( c, S_VOUT, std::max<uint32_t> ( 1, U ), &vo ) );
        fa.u_out = uo;
        fa.v_out = vo;
        if ( U ) MTX_LAUNCH ( k_finalize, blocks_for ( U, 256 ), 256, fa );
        c->nrec = 0;
    }
    else
    {
        uint8_t * mark;
        uint32_t *recu, *recv, *pref2, *recs;
        const uint32_t T = ( uint32_t ) c->total;
        MTX_TRY ( ensure ( c, S_MARK, T, &mark ) );
        MTX_TRY ( ensure ( c, S_RECU, T, &recu ) );
        MTX_TRY ( ensure ( c, S_RECV, T, &recv ) );
        MTX_TRY ( ensure ( c, S_PREF2, T, &pref2 ) );
        MTX_CUDA ( cudaMemsetAsync ( mark, 0, T, st ) );
        fa.mark = mark;
        fa.rec_u = recu;
        fa.rec_v = recv;
        if ( U ) MTX_LAUNCH ( k_finalize, blocks_for ( U, 256 ), 256, fa );
        MTX_TRY ( scan_flags ( c, mark, T, pref2, scalar ) );
        MTX_CUDA ( cudaMemcpyAsync ( h_scalar, scalar, 4, cudaMemcpyDeviceToHost, st ) );
        MTX_CUDA ( cudaStreamSynchronize ( st ) );
        c->nrec = h_scalar[0];
        MTX_TRY ( ensure ( c, S_RECS, ( size_t ) 3 * std::max<uint32_t> ( 1, c->nrec ), &recs ) );
        MTX_LAUNCH ( k_compact, blocks_for ( T, 256 ), 256, mark, pref2, T, recu, recv, recs );
    }
    MTX_CUDA ( cudaEventRecord ( c->ev1, st ) );
    MTX_CUDA ( cudaEventSynchronize ( c->ev1 ) );
    MTX_CUDA ( cudaEventElapsedTime ( &c->device_ms, c->ev0, c->ev1 ) );
    if ( dp_timed ) MTX_CUDA ( cudaEventElapsedTime ( &c->dp_ms, c->evd0, c->evd1 ) );
    return MOTEX_OK;
}

int load_common ( motex_ctx * c, const motex_params * prm, const char * const * seqs, const uint32_t * lens,
                  uint32_t nseq, bool pair_mode )
{
    MTX_TRY ( validate ( prm ) );
    if ( ! seqs || ! lens ) return fail ( MOTEX_EINVAL, "null sequence arrays" );
    if ( nseq == 0 ) return fail ( MOTEX_EINVAL, "no sequences" );
    c->loaded = c->executed = false;
    c->prm = *prm;
    c->gmin.assign ( prm->gap_min, prm->gap_min + prm->nb_gaps );
    c->gmax.assign ( prm->gap_max, prm->gap_max + prm->nb_gaps );
    c->blens.assign ( prm->blens, prm->blens + prm->nb_gaps );
    c->berrs.assign ( prm->berrs, prm->berrs + prm->nb_gaps );
    c->prm.gap_min = c->gmin.data ();
    c->prm.gap_max = c->gmax.data ();
    c->prm.blens = c->blens.data ();
    c->prm.berrs = c->berrs.data ();
    c->G = prm->nb_gaps ? c->gmax[0] - c->gmin[0] + 1 : 1;
    c->nseq = nseq;
    c->pair_mode = pair_mode;
    c->offs.assign ( nseq + 1, 0 );
    uint64_t total = 0;
    for ( uint32_t i = 0; i < nseq; ++i )
    {
        if ( lens[i] && ! seqs[i] ) return fail ( MOTEX_EINVAL, "null sequence %u", i );
        c->offs[i] = ( uint32_t ) total;
        total += lens[i];
        if ( total >= 0xffffff00ull ) return fail ( MOTEX_EUNSUPPORTED, "total input length exceeds 4 G symbols" );
    }
    c->offs[nseq] = ( uint32_t ) total;
    c->total = total;
    if ( total == 0 ) return fail ( MOTEX_EINVAL, "empty input" );
    const uint32_t l = prm->l;
    // total_mot_length (motex.cc:312-360): l plus minimum gaps and boxes
    uint32_t tml_full = l;
    for ( uint32_t g = 0; g < prm->nb_gaps; ++g ) tml_full += c->gmin[g] + c->blens[g];
    c->tml = pair_mode ? 0 : tml_full;
    // factor ends per sequence and the reference's cell count
    std::vector<uint32_t> wstart ( nseq + 1, 0 );
    uint64_t nw = 0, searched = 0;
    for ( uint32_t i = 0; i < nseq; ++i )
    {
        wstart[i] = ( uint32_t ) nw;
        const bool has_words = lens[i] >= std::max ( l, c->tml ) && ( ! pair_mode || i == 0 );
        if ( has_words ) nw += lens[i] - l + 1;
        if ( lens[i] >= c->tml ) searched += lens[i];
    }
    wstart[nseq] = ( uint32_t ) nw;
    c->nwords = ( uint32_t ) nw;
    c->ref_cells = ( pair_mode ? ( uint64_t ) lens[0] * lens[1] : searched * searched ) * ( prm->nb_gaps + 1 );
    // qok[u]: the reference's double-precision quorum test (functions.cc:1105-1108)
    std::vector<uint8_t> qok ( nseq + 1 );
    for ( uint32_t u = 0; u <= nseq; ++u )
    {
        volatile double r = ( ( double ) u / nseq ) * 100;
        qok[u] = r >= prm->q && r <= prm->Q;
    }
    // staging: raw bytes | offs | wstart | qok
    const size_t raw_b = ( total + 15 ) & ~15ull;
    const size_t offs_b = ( ( size_t ) ( nseq + 1 ) * 4 + 15 ) & ~15ull;
    MTX_TRY ( ensure_pinned ( c, 65536 + raw_b + 2 * offs_b + nseq + 16 ) );
    uint8_t * stage = static_cast<uint8_t *> ( c->pinned ) + 65536;
    size_t at = 0;
    for ( uint32_t i = 0; i < nseq; ++i )
    {
        memcpy ( stage + at, seqs[i], lens[i] );
        at += lens[i];
    }
    if ( prm->nb_gaps && ! pair_mode ) c->raw_host.assign ( stage, stage + total );
    else c->raw_host.clear ();
    memcpy ( stage + raw_b, c->offs.data (), ( size_t ) ( nseq + 1 ) * 4 );
    memcpy ( stage + raw_b + offs_b, wstart.data (), ( size_t ) ( nseq + 1 ) * 4 );
    memcpy ( stage + raw_b + 2 * offs_b, qok.data (), nseq + 1 );
    uint8_t * raw;
    uint32_t *doffs, *dws;
    uint8_t * dq;
    MTX_TRY ( ensure ( c, S_RAW, raw_b + 16, &raw ) );
    MTX_TRY ( ensure ( c, S_OFFS, nseq + 1, &doffs ) );
    MTX_TRY ( ensure ( c, S_WSTART, nseq + 1, &dws ) );
    MTX_TRY ( ensure ( c, S_QOK, nseq + 1, &dq ) );
    MTX_CUDA ( cudaMemcpyAsync ( raw, stage, total, cudaMemcpyHostToDevice, c->st ) );
    MTX_CUDA ( cudaMemcpyAsync ( doffs, stage + raw_b, ( size_t ) ( nseq + 1 ) * 4, cudaMemcpyHostToDevice, c->st ) );
    MTX_CUDA ( cudaMemcpyAsync ( dws, stage + raw_b + offs_b, ( size_t ) ( nseq + 1 ) * 4, cudaMemcpyHostToDevice, c->st ) );
    MTX_CUDA ( cudaMemcpyAsync ( dq, stage + raw_b + 2 * offs_b, nseq + 1, cudaMemcpyHostToDevice, c->st ) );
    MTX_CUDA ( cudaStreamSynchronize ( c->st ) );
    c->loaded = true;
    return MOTEX_OK;
}

int fetch_records ( motex_ctx * c, motex_result * out )
{
    memset ( out, 0, sizeof *out );
    out->num_seqs = c->nseq;
    out->ref_cells = c->ref_cells;
    out->exec_cells = c->exec_cells;
    out->unique_words = c->U;
    out->launches = c->job_launches;
    out->device_ms = c->device_ms;
    out->dp_ms = c->dp_ms;
    if ( c->nrec == 0 ) return MOTEX_OK;
    const size_t bytes = ( size_t ) c->nrec * 12;
    MTX_TRY ( ensure_pinned ( c, bytes + 65536 ) );
    uint32_t * h = static_cast<uint32_t *> ( c->pinned );
    MTX_CUDA ( cudaMemcpyAsync ( h, dptr<uint32_t> ( c, S_RECS ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_CUDA ( cudaStreamSynchronize ( c->st ) );
    out->motifs = static_cast<motex_motif *> ( malloc ( ( size_t ) c->nrec * sizeof ( motex_motif ) ) );
    if ( ! out->motifs ) return fail ( MOTEX_ENOMEM, "host allocation of the result failed" );
    const uint32_t G = c->prm.nb_gaps ? c->G : 1;
    std::unordered_set<std::string> seen;
    std::string key;
    uint32_t s = 0, kept = 0;
    for ( uint32_t i = 0; i < c->nrec; ++i )
    {
        const uint32_t idx = h[3 * i];
        const uint32_t pos = idx / G, k = idx % G;
        while ( c->offs[s + 1] <= pos ) ++s;        // records are in (position, gap choice) order
        if ( c->prm.nb_gaps )
        {
            // the writer's key: box 0 and box 1 joined by '_', gap left out
            // (functions.cc:1191-1239); the first passing entry of a key wins
            const uint32_t l = c->prm.l, b1 = c->blens[0], gap = c->gmin[0] + k;
            key.assign ( c->raw_host.data () + pos + 1 - l, l );
            key.push_back ( '_' );
            key.append ( c->raw_host.data () + pos + 1 + gap, b1 );
            if ( ! seen.insert ( key ).second ) continue;
        }
        out->motifs[kept++] = motex_motif { s, pos - c->offs[s], k, h[3 * i + 1], h[3 * i + 2] };
    }
    out->count = kept;
    return MOTEX_OK;
}

} // namespace

// ====================================================================== C ABI

extern "C" {

int motex_ctx_create ( motex_ctx ** ctx, int device )
{
    if ( ! ctx ) return fail ( MOTEX_EINVAL, "null context pointer" );
    *ctx = nullptr;
    int ndev = 0;
    if ( cudaGetDeviceCount ( &ndev ) != cudaSuccess || ndev == 0 )
    {
        cudaGetLastError ();
        return fail ( MOTEX_ECUDA, "no CUDA device available" );
    }
    if ( device < 0 || device >= ndev ) return fail ( MOTEX_EINVAL, "device %d out of range (%d devices)", device, ndev );
    MTX_CUDA ( cudaSetDevice ( device ) );
    motex_ctx * c = new motex_ctx ();
    c->device = device;
    cudaDeviceGetAttribute ( &c->num_sms, cudaDevAttrMultiProcessorCount, device );
    if ( cudaStreamCreateWithFlags ( &c->st, cudaStreamNonBlocking ) != cudaSuccess ||
         cudaEventCreate ( &c->ev0 ) != cudaSuccess || cudaEventCreate ( &c->ev1 ) != cudaSuccess ||
         cudaEventCreate ( &c->evd0 ) != cudaSuccess || cudaEventCreate ( &c->evd1 ) != cudaSuccess )
    {
        cudaGetLastError ();
        motex_ctx_destroy ( c );
        return fail ( MOTEX_ECUDA, "stream/event creation failed" );
    }
    int rc = ensure_pinned ( c, 1 << 20 );
    if ( rc != MOTEX_OK )
    {
        motex_ctx_destroy ( c );
        return rc;
    }
    *ctx = c;
    return MOTEX_OK;
}

int motex_ctx_destroy ( motex_ctx * c )
{
    if ( ! c ) return MOTEX_OK;
    cudaSetDevice ( c->device );
    if ( c->st ) cudaStreamSynchronize ( c->st );
    for ( auto & b : c->buf )
        if ( b.p ) cudaFree ( b.p );
    if ( c->pinned ) cudaFreeHost ( c->pinned );
    if ( c->ev0 ) cudaEventDestroy ( c->ev0 );
    if ( c->ev1 ) cudaEventDestroy ( c->ev1 );
    if ( c->evd0 ) cudaEventDestroy ( c->evd0 );
    if ( c->evd1 ) cudaEventDestroy ( c->evd1 );
    if ( c->st ) cudaStreamDestroy ( c->st );
    delete c;
    return MOTEX_OK;
}

int motex_gpu_load ( motex_ctx * c, const motex_params * prm, const char * const * seqs, const uint32_t * lens,
                     uint32_t nseq )
{
    if ( ! c ) return fail ( MOTEX_EINVAL, "null context" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    return load_common ( c, prm, seqs, lens, nseq, false );
}

int motex_gpu_execute ( motex_ctx * c )
{
    if ( ! c ) return fail ( MOTEX_EINVAL, "null context" );
    if ( ! c->loaded || c->pair_mode ) return fail ( MOTEX_EINVAL, "no sequences loaded" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    c->job_launches = 0;
    MTX_TRY ( run_pipeline ( c ) );
    c->executed = true;
    return MOTEX_OK;
}

int motex_gpu_fetch ( motex_ctx * c, motex_result * out )
{
    if ( ! c || ! out ) return fail ( MOTEX_EINVAL, "null argument" );
    if ( ! c->executed ) return fail ( MOTEX_EINVAL, "nothing executed" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    return fetch_records ( c, out );
}

int motex_gpu_run ( motex_ctx * c, const motex_params * prm, const char * const * seqs, const uint32_t * lens,
                    uint32_t nseq, motex_result * out )
{
    if ( ! c || ! out ) return fail ( MOTEX_EINVAL, "null argument" );
    memset ( out, 0, sizeof *out );
    MTX_TRY ( motex_gpu_load ( c, prm, seqs, lens, nseq ) );
    MTX_TRY ( motex_gpu_execute ( c ) );
    return motex_gpu_fetch ( c, out );
}

void motex_result_free ( motex_result * res )
{
    if ( ! res ) return;
    free ( res->motifs );
    res->motifs = nullptr;
    res->count = 0;
}

int motex_gpu_extract_pair ( motex_ctx * c, const motex_params * prm, const char * p, uint32_t m, const char * t,
                             uint32_t n, uint32_t * u, uint32_t * v )
{
    if ( ! c || ! u || ! v || ! p || ! t ) return fail ( MOTEX_EINVAL, "null argument" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    if ( m < prm->l || n == 0 ) return MOTEX_OK;                  // no factor of p: nothing to add
    const char * seqs[2] = { p, t };
    const uint32_t lens[2] = { m, n };
    MTX_TRY ( load_common ( c, prm, seqs, lens, 2, true ) );
    c->job_launches = 0;
    MTX_TRY ( run_pipeline ( c ) );
    if ( prm->nb_gaps )
    {
        // per (position of p, gap choice k): u[k*m + j] (functions.cc:676-684)
        const uint32_t G = c->G;
        const size_t bytes = ( size_t ) m * G * 4;
        MTX_TRY ( ensure_pinned ( c, 2 * bytes + 65536 ) );
        uint32_t * hu = static_cast<uint32_t *> ( c->pinned );
        uint32_t * hv = hu + ( size_t ) m * G;
        MTX_CUDA ( cudaMemcpyAsync ( hu, dptr<uint32_t> ( c, S_UOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
        MTX_CUDA ( cudaMemcpyAsync ( hv, dptr<uint32_t> ( c, S_VOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
        MTX_CUDA ( cudaStreamSynchronize ( c->st ) );
        for ( uint32_t j = 0; j < m; ++j )
            for ( uint32_t k = 0; k < G; ++k )
            {
                u[( size_t ) k * m + j] += hu[( size_t ) j * G + k];
                v[( size_t ) k * m + j] += hv[( size_t ) j * G + k];
            }
        c->loaded = false;
        return MOTEX_OK;
    }
    const uint32_t U = c->U;
    const size_t bytes = ( size_t ) U * 4;
    MTX_TRY ( ensure_pinned ( c, 2 * bytes + 65536 ) );
    uint32_t * hu = static_cast<uint32_t *> ( c->pinned );
    uint32_t * hv = hu + U;
    MTX_CUDA ( cudaMemcpyAsync ( hu, dptr<uint32_t> ( c, S_UOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_CUDA ( cudaMemcpyAsync ( hv, dptr<uint32_t> ( c, S_VOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_CUDA ( cudaStreamSynchronize ( c->st ) );
    // factor w ends at position l-1+w of p
    for ( uint32_t w = 0; w < U; ++w )
    {
        u[prm->l - 1 + w] += hu[w];
        v[prm->l - 1 + w] += hv[w];
    }
    c->loaded = false;
    return MOTEX_OK;
}

const char * motex_gpu_strerror ( int code )
{
    switch ( code )
    {
        case MOTEX_OK: return "success";
        case MOTEX_EINVAL: return "invalid argument";
        case MOTEX_ENOMEM: return "out of memory";
        case MOTEX_ECUDA: return "CUDA error";
        case MOTEX_EUNSUPPORTED: return "unsupported size or mode";
        case MOTEX_ETIMEOUT: return "bounded device wait timed out";
        case MOTEX_EBUSY: return "busy";
        case MOTEX_ENOTFOUND: return "not found";
        default: return "unknown error";
    }
}

const char * motex_gpu_last_error ( void ) { return g_last_error.c_str (); }

uint64_t motex_ctx_launches ( const motex_ctx * c ) { return c ? c->launches : 0; }

} // extern "C"
