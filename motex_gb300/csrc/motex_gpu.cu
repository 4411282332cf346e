// C-ABI entry points (include/motex_gpu.h) and the device pipeline behind them.
//
// One extraction ("job") runs in stages, with a host synchronisation only
// where the host needs a device-computed size:
//   presence    symbol alphabet actually present                  -> sync (B)
//   pack        codes, bit planes, masks, factor ends; stable LSD radix
//               sort of the factor keys and first-occurrence heads -> sync (U)
//   plan        unique factors, factor planes, DP shape and text chunks
//   dp          factor-search DP over (factor tiles x text chunks)
//   finalize    quorum filter at first occurrences, flag scan      -> sync (count)
//   compact     ordered compaction of the passing factors
// A batch of jobs walks the stages together (a handful of syncs in total) and
// puts the DP work of all single-motif jobs of one kernel class into one
// persistent launch fed from a device work queue.  Executing the same
// resident job again replays the whole staged sequence as one CUDA graph.
#include "motex_gpu.h"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
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
    S_SCALAR, S_UOUT, S_VOUT, S_WPL0, S_WPL1, S_ROWOK, S_ROWEND, S_WPLN, S_SEQSTART, S_XOFF, S_HTILES,
    S_STAB, S_SSLOT, S_SKEEP, S_COUNT
};

// Pinned staging layout of a job (bytes).
constexpr size_t kPinPresent = 0;          // 256 x u32 symbol presence
constexpr size_t kPinCmap = 1024;          // 256 B symbol -> code
constexpr size_t kPinScalar = 2048;        // u32 unique count, u32 motif count, key-table error flag, staging error flag
constexpr size_t kPinXoff = 4096;          // structure offset table (<= kPinXoffWords u32)
constexpr size_t kPinXoffWords = 4096;
constexpr size_t kPinChunks = kPinXoff + 4 * kPinXoffWords;        // chunk table
constexpr size_t kPinStage = 65536;        // input upload / result download
constexpr uint32_t kMaxChunks = ( kPinStage - kPinChunks ) / sizeof ( ChunkInfo );

struct DPTune
{
    int W = 8;     // register words per thread
    int NL = 1;    // factors per register word
    int UR = 8;    // unroll of the 32-position block
    int F = 0;     // Hamming form: 1 = guarded lanes with lowest-bit clears (no popc)
};

} // namespace

struct Job
{
    motex_ctx * ctx = nullptr;
    DevBuf buf[S_COUNT];
    void * pinned = nullptr;
    size_t pinned_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evd0 = nullptr, evd1 = nullptr;

    // loaded
    bool loaded = false, executed = false;
    motex_params prm {};
    std::vector<uint32_t> gmin, gmax, blens, berrs;
    uint32_t nseq = 0;
    std::vector<uint32_t> offs;                // nseq + 1
    uint64_t total = 0;
    uint32_t tml = 0;
    uint32_t nwords = 0;
    uint32_t npat = 0;                         // leading pattern sequences (0: all-pairs)
    uint64_t ref_cells = 0;
    uint32_t G = 1;                            // gap choices (1 for single motifs)

    // executed
    int B = 0;
    uint32_t U = 0, nblk = 0, stride = 0, n_split = 0, nrec = 0;
    uint64_t exec_cells = 0;
    float device_ms = 0.f, dp_ms = 0.f;
    uint32_t launches = 0;
    DPTune tune;

    // plan of the DP launch
    bool structured = false, generic = false, dp_pending = false, dp_timed = false, replaying = false;
    bool batched = false;                      // a member of a batch (persistent DP launch)
    uint32_t nw64 = 1;
    DPArgs da {};
    StructArgs sa {};
    StructNArgs san {};
    StructNBlk snb {};
    bool structN = false;
    bool structN_blk = false;                  // block form of the any-gap kernel
    std::vector<ChunkInfo> chunks;
    uint32_t ntiles = 0;
    uint32_t * uniq = nullptr;

    // replay of the staged sequence
    cudaGraphExec_t graph = nullptr;
    int runs_since_load = 0;
    uint32_t graph_kernels = 0;

    ~Job ();
};

struct motex_ctx
{
    int device = 0;
    int num_sms = 148;
    cudaStream_t st = nullptr;
    uint64_t launches = 0;
    Job main;
    std::vector<std::unique_ptr<Job>> pool;    // batch jobs
    DevBuf bjobs, bitems, bcounter;
    void * bpinned = nullptr;
    size_t bpinned_cap = 0;
    DevBuf mjobs, mres, mpart;                 // small-job pipeline: descriptors, result words, shares
    void * mpinned = nullptr;
    size_t mpinned_cap = 0;
    cudaEvent_t evb0 = nullptr, evb1 = nullptr;
};

Job::~Job ()
{
    for ( auto & b : buf )
        if ( b.p ) cudaFree ( b.p );
    if ( pinned ) cudaFreeHost ( pinned );
    if ( ev0 ) cudaEventDestroy ( ev0 );
    if ( ev1 ) cudaEventDestroy ( ev1 );
    if ( evd0 ) cudaEventDestroy ( evd0 );
    if ( evd1 ) cudaEventDestroy ( evd1 );
    if ( graph ) cudaGraphExecDestroy ( graph );
}

namespace
{

int alloc_dev ( DevBuf & b, size_t bytes )
{
    bytes = std::max<size_t> ( 1, bytes );
    if ( b.cap >= bytes ) return MOTEX_OK;
    if ( b.p ) cudaFree ( b.p );
    b.p = nullptr;
    b.cap = 0;
    const size_t want = bytes + bytes / 4;
    if ( cudaMalloc ( &b.p, want ) != cudaSuccess )
    {
        cudaGetLastError ();
        return fail ( MOTEX_ENOMEM, "device allocation of %zu bytes failed", want );
    }
    b.cap = want;
    return MOTEX_OK;
}

template <typename T>
int ensure ( Job * j, Slot s, size_t count, T ** out )
{
    MTX_TRY ( alloc_dev ( j->buf[s], count * sizeof ( T ) ) );
    *out = static_cast<T *> ( j->buf[s].p );
    return MOTEX_OK;
}

template <typename T>
T * dptr ( Job * j, Slot s ) { return static_cast<T *> ( j->buf[s].p ); }

int alloc_pinned ( void ** p, size_t * cap, size_t bytes, cudaStream_t st )
{
    if ( *cap >= bytes ) return MOTEX_OK;
    if ( *p )
    {
        cudaStreamSynchronize ( st );                 // no copy may still read the old buffer
        cudaFreeHost ( *p );
    }
    *p = nullptr;
    *cap = 0;
    const size_t want = bytes + bytes / 4 + 4096;
    if ( cudaHostAlloc ( p, want, cudaHostAllocDefault ) != cudaSuccess )
    {
        cudaGetLastError ();
        return fail ( MOTEX_ENOMEM, "pinned host allocation of %zu bytes failed", want );
    }
    *cap = want;
    return MOTEX_OK;
}

void drop_graph ( Job * j );

// A job's pinned buffer only grows; moving it invalidates a captured graph.
int ensure_pinned ( Job * j, size_t bytes )
{
    if ( j->pinned_cap >= bytes ) return MOTEX_OK;
    drop_graph ( j );
    return alloc_pinned ( &j->pinned, &j->pinned_cap, bytes, j->ctx->st );
}

template <typename T>
T * pin ( Job * j, size_t off ) { return reinterpret_cast<T *> ( static_cast<uint8_t *> ( j->pinned ) + off ); }

int check_launch ( Job * j, const char * what )
{
    j->ctx->launches++;
    j->launches++;
    cudaError_t e = cudaGetLastError ();
    if ( e != cudaSuccess ) return fail ( MOTEX_ECUDA, "launch of %s failed: %s", what, cudaGetErrorString ( e ) );
    return MOTEX_OK;
}

#define MTX_LAUNCH( name, grid, block, ... )                                                       \
    do {                                                                                            \
        name<<<( grid ), ( block ), 0, j->ctx->st>>> ( __VA_ARGS__ );                               \
        MTX_TRY ( check_launch ( j, #name ) );                                                      \
    } while ( 0 )

unsigned blocks_for ( uint64_t n, unsigned threads ) { return ( unsigned ) std::max<uint64_t> ( 1, ( n + threads - 1 ) / threads ); }

// Timing event on the job's stream; while a graph is being captured it is
// recorded as an external node, so the replayed graph records it too.
int record ( Job * j, cudaEvent_t ev )
{
    if ( j->replaying ) MTX_CUDA ( cudaEventRecordWithFlags ( ev, j->ctx->st, cudaEventRecordExternal ) );
    else MTX_CUDA ( cudaEventRecord ( ev, j->ctx->st ) );
    return MOTEX_OK;
}

int init_job ( motex_ctx * c, Job * j )
{
    j->ctx = c;
    if ( cudaEventCreate ( &j->ev0 ) != cudaSuccess || cudaEventCreate ( &j->ev1 ) != cudaSuccess ||
         cudaEventCreate ( &j->evd0 ) != cudaSuccess || cudaEventCreate ( &j->evd1 ) != cudaSuccess )
    {
        cudaGetLastError ();
        return fail ( MOTEX_ECUDA, "event creation failed" );
    }
    return ensure_pinned ( j, 1 << 20 );
}

void drop_graph ( Job * j )
{
    if ( j->graph ) cudaGraphExecDestroy ( j->graph );
    j->graph = nullptr;
    j->runs_since_load = 0;
}

// One gap within the shared-history kernel's limits (k_dp_struct1).
bool struct1_shape ( const motex_params * p )
{
    if ( p->nb_gaps != 1 ) return false;
    const uint32_t gmin = p->gap_min[0], gmax = p->gap_max[0], b1 = p->blens[0];
    return p->l <= 32 && b1 <= 32 && gmax >= gmin && gmax - gmin + 1 <= 32 && gmax + b1 <= 31;
}

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
        if ( p->nb_gaps > kMaxGapsN )
            return fail ( MOTEX_EUNSUPPORTED, "structured motifs with %u gaps (at most %u)", p->nb_gaps, kMaxGapsN );
        if ( p->l > kStructMaxBox ) return fail ( MOTEX_EUNSUPPORTED, "structured motifs need l <= %u", kStructMaxBox );
        uint64_t structs = 1, tml = p->l;
        for ( uint32_t g = 0; g < p->nb_gaps; ++g )
        {
            if ( p->gap_max[g] < p->gap_min[g] ) return fail ( MOTEX_EINVAL, "gap range [%u,%u] is empty", p->gap_min[g], p->gap_max[g] );
            if ( p->blens[g] == 0 ) return fail ( MOTEX_EINVAL, "box length must be positive" );
            if ( p->blens[g] > kStructMaxBox )
                return fail ( MOTEX_EUNSUPPORTED, "structured boxes need box length <= %u", kStructMaxBox );
            structs *= p->gap_max[g] - p->gap_min[g] + 1;
            if ( structs > 1u << 20 ) break;
            tml += p->gap_min[g] + p->blens[g];
        }
        if ( ! struct1_shape ( p ) && ( structs > kMaxStructsN || structs * p->nb_gaps > kPinXoffWords ) )
            return fail ( MOTEX_EUNSUPPORTED, "%llu gap structures (at most %u with several gaps, long gaps or boxes "
                          "longer than 32)", ( unsigned long long ) structs, kMaxStructsN );
        for ( uint32_t g = 0; g < p->nb_gaps; ++g )
            if ( p->berrs[g] >= tml )
                return fail ( MOTEX_EUNSUPPORTED, "box error bound %u not below the minimum motif length", p->berrs[g] );
    }
    return MOTEX_OK;
}

// Exclusive scan of n byte flags; device total written to *d_total (may be null).
int scan_flags ( Job * j, const uint8_t * in, uint32_t n, uint32_t * out, uint32_t * d_total )
{
    const uint32_t tiles = ( uint32_t ) blocks_for ( n, kScanTile );
    uint32_t * tsum;
    MTX_TRY ( ensure ( j, S_TILES, tiles, &tsum ) );
    cudaError_t e = scan_exclusive_u8 ( in, n, out, d_total, tsum, j->ctx->st );
    j->ctx->launches += 3;
    j->launches += 3;
    if ( e != cudaSuccess ) return fail ( MOTEX_ECUDA, "scan launch failed: %s", cudaGetErrorString ( e ) );
    return MOTEX_OK;
}

// Stable sort of the factor ends by their packed keys; result in *idx_out,
// the most significant 32-bit key chunk of every sorted factor in *keys_out
// (the whole factor when l * B <= 32, *full_key).
int sort_factors ( Job * j, uint32_t n, uint32_t ** idx_out, const uint32_t ** keys_out, bool * full_key )
{
    const uint32_t l = j->prm.l, B = ( uint32_t ) j->B;
    const uint32_t bits = l * B;
    const uint32_t nchunk = ( bits + 31 ) / 32;
    const uint32_t ntiles = ( uint32_t ) blocks_for ( n, kSortTile );
    const uint32_t nhist = 256 * ntiles;
    uint32_t *key0, *key1, *idx1, *hist, *tsum;
    MTX_TRY ( ensure ( j, S_KEY0, n, &key0 ) );
    MTX_TRY ( ensure ( j, S_KEY1, n, &key1 ) );
    MTX_TRY ( ensure ( j, S_IDX1, n, &idx1 ) );
    MTX_TRY ( ensure ( j, S_HIST, nhist, &hist ) );
    MTX_TRY ( ensure ( j, S_HTILES, blocks_for ( nhist, kScanTile ), &tsum ) );
    uint32_t * idx0 = dptr<uint32_t> ( j, S_WPOS );
    uint32_t *kin = key0, *kout = key1, *iin = idx0, *iout = idx1;
    for ( uint32_t ch = 0; ch < nchunk; ++ch )
    {
        // chunk 0 (the last symbols) came with the packing, in factor order
        if ( ch > 0 )
            MTX_LAUNCH ( k_gather_key, blocks_for ( n, 256 ), 256, iin, n, dptr<uint8_t> ( j, S_CODES ), l, B, 32 * ch, kin );
        const uint32_t cbits = std::min<uint32_t> ( 32, bits - 32 * ch );
        for ( uint32_t pass = 0; pass * 8 < cbits; ++pass )
        {
            MTX_LAUNCH ( k_radix_hist, ntiles, kSortThreads, kin, n, ( int ) ( 8 * pass ), hist, ntiles );
            // digit-major histogram -> scatter offsets, by the multi-CTA scan (in place)
            cudaError_t e = scan_exclusive_u32 ( hist, nhist, hist, nullptr, tsum, j->ctx->st );
            j->ctx->launches += 3;
            j->launches += 3;
            if ( e != cudaSuccess ) return fail ( MOTEX_ECUDA, "histogram scan failed: %s", cudaGetErrorString ( e ) );
            MTX_LAUNCH ( k_radix_scatter, ntiles, kSortThreads, kin, iin, kout, iout, n, ( int ) ( 8 * pass ), hist, ntiles );
            std::swap ( kin, kout );
            std::swap ( iin, iout );
        }
    }
    *idx_out = iin;
    *keys_out = kin;
    *full_key = nchunk == 1;
    return MOTEX_OK;
}

/*
 * DP launch shape: factors per thread (W), factors per 32-bit register (NL,
 * edit distance with l <= 15 packs 2-4), and the inner unroll of the
 * 32-position text block (UR, bounded to keep the loop in the instruction
 * cache).  MOTEX_DP_W / MOTEX_DP_UR / MOTEX_DP_SWAR=0 override the choice.
 */
bool hclr_eligible ( uint32_t l, uint32_t e ) { return e <= kHclrMaxE && hclr_lanes ( l ) >= 2; }

DPTune choose_tune ( Job * j, uint32_t U, bool ed, bool generic )
{
    DPTune t;
    if ( generic ) { t.W = 1; t.NL = 1; t.UR = 32; return t; }
    t.NL = ed ? swar_lanes ( j->prm.l ) : ( j->B >= 3 ? hswar_lanes ( j->prm.l ) : 1 );
    // Hamming with e <= 3 and 5 <= l <= 12: the popc-free guarded-lane form,
    // three lanes where they fit (measured on GB300: config 1 DP 0.235 ->
    // 0.201 ms with two lanes; config 3 Hamming 268 -> 207 ms with three).
    // MOTEX_DP_CLEAR: 0 keeps the popc forms; 2 or 3 fixes the lane count
    // where that fits
    const char * clr = getenv ( "MOTEX_DP_CLEAR" );
    const int clr_v = clr ? atoi ( clr ) : -1;
    if ( ! ed && hclr_eligible ( j->prm.l, j->prm.e ) && clr_v != 0 )
    {
        t.NL = ( clr_v >= 2 && hclr_fits ( j->prm.l, clr_v ) ) ? clr_v : hclr_lanes ( j->prm.l );
        t.F = 1;
    }
    const uint32_t groups = ( U + t.NL - 1 ) / t.NL;
    t.W = groups >= ( uint32_t ) j->ctx->num_sms * kDPThreads * 8 ? 8 : 4;
    if ( t.NL > 1 ) t.W = std::min ( t.W, swar_default_w ( j->B ) );
    t.UR = ed ? 8 : 4;             // measured on GB300: Hamming prefers the shorter body
    if ( const char * e = getenv ( "MOTEX_DP_SWAR" ) )
        if ( atoi ( e ) == 0 )
        {
            t.NL = 1;
            t.F = 0;
        }
    if ( const char * e = getenv ( "MOTEX_DP_W" ) )
        if ( atoi ( e ) == 4 || atoi ( e ) == 8 ) t.W = atoi ( e );
    if ( const char * e = getenv ( "MOTEX_DP_UR" ) )
    {
        const int v = atoi ( e );
        if ( ( v == 4 || v == 8 || ( v == 32 && t.NL == 1 ) ) && ! ( t.F && v != 4 ) ) t.UR = v;
    }
    return t;
}

/*
 * Autotuner.  For a job with at least kTuneMinCells DP cells whose key
 * (bit planes B, factor length l, errors e, distance d) has no entry yet,
 * every candidate launch shape -- register words per thread W, factors per
 * register NL (SWAR or 1-lane for edit distance), block unroll UR -- runs the
 * DP on a probe grid: up to 8 tiles per SM times as many 512-block text
 * chunks as fill every SM's CTA slots several times, like the real grid, and
 * long enough that the per-CTA set-up weighs as little as in the real run;
 * time per cell from CUDA events picks the winner; accumulators are cleared
 * afterwards.  Batched jobs do not tune (their probes would stall the
 * batch); a key's entry also picks the shape of the persistent kernel its
 * class runs (where one implements it).  Entries are shared by every context of the
 * process and, with MOTEX_TUNE_CACHE=<file>, read from and appended to that
 * file.  MOTEX_AUTOTUNE=0 turns tuning off (the defaults of choose_tune
 * apply); explicit MOTEX_DP_* overrides win over both.
 */
constexpr uint64_t kTuneMinCells = 50000000000ull;
constexpr uint32_t kTuneBlocks = 512;        // probe chunk: 16384 text positions

struct TuneKey
{
    int B;
    uint32_t l, e, d;
    bool operator< ( const TuneKey & o ) const { return std::tie ( B, l, e, d ) < std::tie ( o.B, o.l, o.e, o.d ); }
};

std::mutex g_tune_mu;
std::map<TuneKey, DPTune> g_tune;
bool g_tune_loaded = false;

// A launch shape the single-motif DP kernels implement for this key: the
// key a tunable job can have (2-5 bit planes, l <= 32, e < l, d 0/1), W 4 or
// 8, NL 1 or the key's packed lane count, UR 4 or 8 (32 for 1-lane kernels;
// packed Hamming only with 4).
bool tune_entry_valid ( const TuneKey & k, const DPTune & t )
{
    if ( k.B < 2 || k.B > kMaxPlanes || k.l < 1 || k.l > 32 || k.e >= k.l || k.d > 1 ) return false;
    if ( t.W != 4 && t.W != 8 ) return false;
    if ( t.F != 0 )                                         // guarded-lane Hamming
        return t.F == 1 && k.d == 0 && k.e <= kHclrMaxE && hclr_fits ( k.l, t.NL ) && t.UR == 4;
    const int packed = k.d == 1 ? swar_lanes ( k.l ) : ( k.B >= 3 ? hswar_lanes ( k.l ) : 1 );
    if ( t.NL != 1 && ( t.NL != packed || packed < 2 ) ) return false;
    if ( t.UR != 4 && t.UR != 8 && ! ( t.UR == 32 && t.NL == 1 ) ) return false;
    if ( k.d == 0 && t.NL > 1 && t.UR != 4 ) return false;
    return true;
}

// Entries of the MOTEX_TUNE_CACHE file, one "B l e d W NL UR F" line each (F,
// the Hamming form, may be absent: 0); a line that does not parse or names a
// shape the kernels do not implement is skipped (a later valid line for the
// same key wins).
void tune_load_locked ()
{
    if ( g_tune_loaded ) return;
    g_tune_loaded = true;
    const char * path = getenv ( "MOTEX_TUNE_CACHE" );
    if ( ! path || ! *path ) return;
    FILE * f = fopen ( path, "r" );
    if ( ! f ) return;
    char line[256];
    while ( fgets ( line, sizeof line, f ) )
    {
        TuneKey k;
        DPTune t;
        char extra;
        const int n = sscanf ( line, "%d %u %u %u %d %d %d %d %c", &k.B, &k.l, &k.e, &k.d, &t.W, &t.NL, &t.UR, &t.F, &extra );
        if ( n == 7 ) t.F = 0;
        else if ( n != 8 ) continue;
        if ( tune_entry_valid ( k, t ) ) g_tune[k] = t;
    }
    fclose ( f );
}

void tune_store_locked ( const TuneKey & k, const DPTune & t )
{
    g_tune[k] = t;
    const char * path = getenv ( "MOTEX_TUNE_CACHE" );
    if ( ! path || ! *path ) return;
    if ( FILE * f = fopen ( path, "a" ) )
    {
        fprintf ( f, "%d %u %u %u %d %d %d %d\n", k.B, k.l, k.e, k.d, t.W, t.NL, t.UR, t.F );
        fclose ( f );
    }
}

bool tune_lookup ( const TuneKey & k, DPTune * t )
{
    std::lock_guard<std::mutex> lk ( g_tune_mu );
    tune_load_locked ();
    auto it = g_tune.find ( k );
    if ( it == g_tune.end () ) return false;
    *t = it->second;
    return true;
}

bool launch_shape ( Job * j, const DPArgs & da, const DPTune & t, dim3 grid )
{
    const bool ed = j->prm.d == 1;
    if ( t.F ) return launch_dp_hclr ( da, j->B, t.NL, t.W, grid, j->ctx->st );
    if ( t.NL > 1 )
        return ed ? launch_dp_swar_ed ( da, j->B, t.NL, t.W, t.UR, grid, j->ctx->st )
                  : launch_dp_hswar ( da, j->B, t.NL, t.W, t.UR, grid, j->ctx->st );
    return launch_dp_fast ( da, j->B, t.W, t.UR, ed, grid, j->ctx->st );
}

int autotune ( Job * j, DPTune * best )
{
    const bool ed = j->prm.d == 1;
    const TuneKey key { j->B, j->prm.l, j->prm.e, j->prm.d };
    std::vector<DPTune> cands;
    const int packed = ed ? swar_lanes ( j->prm.l ) : ( j->B >= 3 ? hswar_lanes ( j->prm.l ) : 1 );
    for ( int NL : { packed, 1 } )
    {
        for ( int W : { 4, 8 } )
            for ( int UR : { 4, 8 } )
                if ( ed || NL == 1 || UR == 4 )              // packed Hamming exists with unroll 4 only
                    cands.push_back ( DPTune { W, NL, UR, 0 } );
        if ( NL == 1 ) break;
    }
    if ( ! ed && hclr_eligible ( j->prm.l, j->prm.e ) )
        for ( int NL : { 3, 2 } )
            if ( hclr_fits ( j->prm.l, NL ) )
                for ( int W : { 4, 8 } ) cands.push_back ( DPTune { W, NL, 4, 1 } );
    // probe chunks: consecutive 512-block ranges from the start of the text, no
    // splits; up to 64, so that a job with few factor tiles (a few thousand
    // distinct factors) still fills every SM in the probe as in the real grid
    // (with 16, a 4-tile shape ran 64 CTAs on 152 SMs and lost to a shape with
    // more tiles that is slower at full occupancy)
    const uint32_t pblk = std::min<uint32_t> ( j->nblk, kTuneBlocks );
    const uint32_t maxc = std::max<uint32_t> ( 1, std::min<uint32_t> ( 64, j->nblk / pblk ) );
    ChunkInfo * d_probe;
    MTX_TRY ( ensure ( j, S_TILES, maxc * ( ( sizeof ( ChunkInfo ) + 3 ) / 4 ), reinterpret_cast<uint32_t **> ( &d_probe ) ) );
    ChunkInfo * h_probe = pin<ChunkInfo> ( j, kPinChunks );
    for ( uint32_t c = 0; c < maxc; ++c ) h_probe[c] = ChunkInfo { c * pblk, c * pblk, ( c + 1 ) * pblk, -1, -1 };
    MTX_CUDA ( cudaMemcpyAsync ( d_probe, h_probe, maxc * sizeof ( ChunkInfo ), cudaMemcpyHostToDevice, j->ctx->st ) );
    DPArgs da = j->da;
    da.chunks = d_probe;
    float best_ms = 1e30f;
    for ( const DPTune & t : cands )
    {
        const uint32_t groups = ( j->U + t.NL - 1 ) / t.NL;
        const uint32_t ntiles = ( groups + kDPThreads * t.W - 1 ) / ( kDPThreads * t.W );
        // enough CTAs to fill every SM's slots several times, like the real grid
        const uint32_t gx = std::min<uint32_t> ( ntiles, 8u * j->ctx->num_sms );
        const uint32_t gy = std::min<uint32_t> ( maxc, std::max<uint32_t> ( 1, ( 16u * j->ctx->num_sms + gx - 1 ) / gx ) );
        const dim3 grid ( gx, gy );
        for ( int rep = 0; rep < 2; ++rep )                     // first launch warms up
        {
            MTX_TRY ( record ( j, j->evd0 ) );
            if ( ! launch_shape ( j, da, t, grid ) ) return fail ( MOTEX_EUNSUPPORTED, "autotune candidate failed" );
            MTX_TRY ( check_launch ( j, "k_dp (autotune)" ) );
            MTX_TRY ( record ( j, j->evd1 ) );
        }
        MTX_CUDA ( cudaEventSynchronize ( j->evd1 ) );
        float ms = 0.f;
        MTX_CUDA ( cudaEventElapsedTime ( &ms, j->evd0, j->evd1 ) );
        // time per cell the probe covered
        const double per = ms / ( ( double ) std::min<uint64_t> ( ( uint64_t ) grid.x * kDPThreads * t.W * t.NL, j->U ) *
                                  grid.y * pblk * 32.0 );
        if ( per < best_ms ) { best_ms = ( float ) per; *best = t; }
    }
    std::lock_guard<std::mutex> lk ( g_tune_mu );
    tune_store_locked ( key, *best );
    return MOTEX_OK;
}

/*
 * Text chunks for the DP grid: equal block ranges; sequences cut by a chunk
 * boundary get a split index (one flag row each).  warmup = positions a
 * chunk must process before its first counted one (edit distance: l+e-1,
 * generic Hamming: l-1, fast Hamming: 0).
 */
void build_chunks ( Job * j, uint32_t first_blk, uint32_t nchunks, uint32_t warmup, std::vector<ChunkInfo> & out )
{
    const uint32_t nblk = j->nblk;
    const uint32_t span = nblk - first_blk;
    nchunks = std::max<uint32_t> ( 1, std::min ( { nchunks, span, kMaxChunks } ) );
    std::map<uint32_t, int> split_of;
    auto seq_at = [&] ( uint64_t pos ) -> uint32_t {
        return ( uint32_t ) ( std::upper_bound ( j->offs.begin (), j->offs.end (), ( uint32_t ) pos ) - j->offs.begin () ) - 1;
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
        if ( i > 0 && P < j->total )
        {
            uint32_t s = seq_at ( P );
            if ( j->offs[s] < P ) ch.first_split = split_idx ( s );
        }
        const uint64_t E = ( uint64_t ) ch.end * 32;
        if ( i + 1 < nchunks && E < j->total )
        {
            uint32_t s = seq_at ( E );
            if ( j->offs[s] < E ) ch.last_split = split_idx ( s );
        }
        out.push_back ( ch );
    }
    j->n_split = ( uint32_t ) split_of.size ();
}

int upload_chunks ( Job * j, ChunkInfo ** d_out )
{
    ChunkInfo * h = pin<ChunkInfo> ( j, kPinChunks );
    std::copy ( j->chunks.begin (), j->chunks.end (), h );
    MTX_TRY ( ensure ( j, S_CHUNKS, j->chunks.size (), d_out ) );
    MTX_CUDA ( cudaMemcpyAsync ( *d_out, h, j->chunks.size () * sizeof ( ChunkInfo ), cudaMemcpyHostToDevice, j->ctx->st ) );
    return MOTEX_OK;
}

// ---------------------------------------------------------------- stages


int stage_presence ( Job * j )
{
    cudaStream_t st = j->ctx->st;
    j->launches = 0;
    j->dp_pending = j->dp_timed = false;
    MTX_TRY ( record ( j, j->ev0 ) );
    uint32_t * present;
    MTX_TRY ( ensure ( j, S_PRESENT, 256, &present ) );
    MTX_CUDA ( cudaMemsetAsync ( present, 0, 256 * sizeof ( uint32_t ), st ) );
    MTX_LAUNCH ( k_presence, std::min<unsigned> ( 4 * j->ctx->num_sms, blocks_for ( j->total, 256 * 16 ) ), 256,
                 dptr<uint8_t> ( j, S_RAW ), j->total, present );
    MTX_CUDA ( cudaMemcpyAsync ( pin<uint32_t> ( j, kPinPresent ), present, 256 * sizeof ( uint32_t ),
                                 cudaMemcpyDeviceToHost, st ) );
    return MOTEX_OK;
}

// Returns through *need_sync whether the unique count must be read back.
int stage_pack ( Job * j, bool * need_sync )
{
    const motex_params & P = j->prm;
    const bool ed = P.d == 1;
    cudaStream_t st = j->ctx->st;
    *need_sync = false;
    uint8_t * h_cmap = pin<uint8_t> ( j, kPinCmap );
    if ( ! j->replaying )
    {
        const uint32_t * h_present = pin<uint32_t> ( j, kPinPresent );
        uint32_t sigma = 0;
        for ( int i = 0; i < 256; ++i ) h_cmap[i] = h_present[i] ? ( uint8_t ) sigma++ : 0;
        int B = 2;                                   // one- and two-symbol inputs run on the 2-plane kernels
        while ( ( 1u << B ) < sigma ) ++B;
        if ( B > kMaxPlanes )
            return fail ( MOTEX_EUNSUPPORTED, "%u distinct symbols need %d bit planes (max %d)", sigma, B, kMaxPlanes );
        j->B = B;
    }
    const int B = j->B;
    uint8_t * cmap;
    MTX_TRY ( ensure ( j, S_CMAP, 256, &cmap ) );
    MTX_CUDA ( cudaMemcpyAsync ( cmap, h_cmap, 256, cudaMemcpyHostToDevice, st ) );

    j->nblk = ( uint32_t ) ( ( j->total + 31 ) / 32 );
    j->stride = ( j->nblk + 1 + 31 ) & ~31u;
    uint8_t * codes;
    uint32_t *planes, *vmask, *emask, *wpos;
    MTX_TRY ( ensure ( j, S_CODES, j->total + 64, &codes ) );
    MTX_TRY ( ensure ( j, S_PLANES, ( size_t ) B * j->stride, &planes ) );
    MTX_TRY ( ensure ( j, S_VMASK, j->nblk, &vmask ) );
    MTX_TRY ( ensure ( j, S_EMASK, j->nblk, &emask ) );
    MTX_TRY ( ensure ( j, S_WPOS, j->nwords, &wpos ) );
    MTX_CUDA ( cudaMemsetAsync ( planes, 0, ( size_t ) B * j->stride * sizeof ( uint32_t ), st ) );
    PackArgs pa;
    pa.raw = dptr<uint8_t> ( j, S_RAW );
    pa.total = j->total;
    pa.offs = dptr<uint32_t> ( j, S_OFFS );
    pa.nseq = j->nseq;
    pa.cmap = cmap;
    pa.B = B;
    pa.l = P.l;
    pa.tml = j->tml;
    pa.vstart = ed ? 0 : P.l - 1;
    pa.npat = j->npat;
    pa.wstart = dptr<uint32_t> ( j, S_WSTART );
    pa.codes = codes;
    pa.planes = planes;
    pa.plane_stride = j->stride;
    pa.vmask = vmask;
    pa.emask = emask;
    pa.wpos = wpos;
    pa.nblk = j->nblk;
    uint32_t * scalar;
    MTX_TRY ( ensure ( j, S_SCALAR, 4, &scalar ) );
    pa.err = scalar + 3;
    // MOTEX_PACK_WAIT_POLLS bounds the staging waits (0: give up at once, which
    // exercises the failure path: the run returns MOTEX_ETIMEOUT)
    pa.wait_polls = kStageWaitPolls;
    if ( const char * w = getenv ( "MOTEX_PACK_WAIT_POLLS" ) ) pa.wait_polls = ( uint32_t ) strtoul ( w, nullptr, 10 );
    MTX_CUDA ( cudaMemsetAsync ( scalar + 3, 0, 4, st ) );
    // the factor sort's first key chunk is formed by the packer itself
    const bool sorting = P.nb_gaps == 0 && ! j->npat && j->nwords > 0;
    pa.key0 = nullptr;
    pa.kwin = 0;
    if ( sorting )
    {
        MTX_TRY ( ensure ( j, S_KEY0, j->nwords, &pa.key0 ) );
        pa.kwin = std::min<uint32_t> ( P.l, 31u / ( uint32_t ) B + 1u );
    }
    // persistent: kPackCtasPerSm CTAs per SM (the launch bounds give every
    // one its registers), each with two staged tiles in flight
    const uint64_t ntiles = ( j->total + kPackTile - 1 ) / kPackTile;
    const size_t key_smem = sorting ? sizeof ( uint32_t ) * kPackKeyWords * ( kPackThreads / 32 ) : 0;
    MTX_CUDA ( cudaFuncSetAttribute ( k_pack, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) key_smem ) );
    k_pack<<<( unsigned ) std::min<uint64_t> ( ntiles, ( uint64_t ) kPackCtasPerSm * j->ctx->num_sms ), kPackThreads,
             key_smem, j->ctx->st>>> ( pa );
    MTX_TRY ( check_launch ( j, "k_pack" ) );

    j->structured = P.nb_gaps > 0;
    j->generic = ! j->structured && P.l > 32;
    if ( sorting )
    {
        uint32_t * idx;
        const uint32_t * keys;
        bool full_key;
        MTX_TRY ( sort_factors ( j, j->nwords, &idx, &keys, &full_key ) );
        uint8_t * head;
        uint32_t * pref;
        MTX_TRY ( ensure ( j, S_HEAD, j->nwords, &head ) );
        MTX_TRY ( ensure ( j, S_PREF, j->nwords, &pref ) );
        MTX_LAUNCH ( k_heads, blocks_for ( ( j->nwords + 3 ) / 4, 256 ), 256, idx, keys, ( int ) full_key, j->nwords, codes, P.l, head );
        MTX_TRY ( scan_flags ( j, head, j->nwords, pref, scalar ) );
        MTX_CUDA ( cudaMemcpyAsync ( pin<uint32_t> ( j, kPinScalar ), scalar, 4, cudaMemcpyDeviceToHost, st ) );
        j->uniq = idx;                               // sorted factor ends; compacted in stage_plan
        *need_sync = true;
    }
    else
    {
        j->uniq = wpos;
        j->U = j->nwords;
    }
    return MOTEX_OK;
}

int plan_structured ( Job * j );

int stage_plan ( Job * j, bool sorted )
{
    const motex_params & P = j->prm;
    const bool ed = P.d == 1;
    cudaStream_t st = j->ctx->st;
    j->n_split = 0;
    j->exec_cells = 0;
    j->dp_ms = 0.f;
    if ( j->structured ) return plan_structured ( j );
    const int B = j->B;
    const uint8_t * codes = dptr<uint8_t> ( j, S_CODES );
    if ( sorted )
    {
        if ( ! j->replaying ) j->U = pin<uint32_t> ( j, kPinScalar )[0];
        uint32_t * uniq;
        MTX_TRY ( ensure ( j, S_UNIQ, j->U, &uniq ) );
        MTX_LAUNCH ( k_unique, std::min<unsigned> ( blocks_for ( ( j->nwords + 15 ) / 16, 256 ), 64 * j->ctx->num_sms ), 256, j->uniq,
                     dptr<uint8_t> ( j, S_HEAD ),
                     dptr<uint32_t> ( j, S_PREF ), j->nwords, uniq );
        j->uniq = uniq;
    }
    const uint32_t U = j->U;
    uint32_t *u_acc, *v_acc;
    MTX_TRY ( ensure ( j, S_UACC, U, &u_acc ) );
    MTX_TRY ( ensure ( j, S_VACC, U, &v_acc ) );
    if ( U == 0 ) return MOTEX_OK;

    DPArgs & da = j->da;
    da = DPArgs {};
    da.text.planes = dptr<uint32_t> ( j, S_PLANES );
    da.text.plane_stride = j->stride;
    da.text.vmask = dptr<uint32_t> ( j, S_VMASK );
    da.text.emask = dptr<uint32_t> ( j, S_EMASK );
    da.text.nblk = j->nblk;
    da.U = U;
    da.l = P.l;
    da.e = P.e;
    da.one = 1u;
    da.two = 2u;
    da.neg1 = ~0u;
    if ( ! j->replaying ) j->tune = choose_tune ( j, U, ed, j->generic );
    bool tune_now = false;
    // a batched job takes the key's entry when there is one but does not
    // tune: the probes would stall its batch-mates (a serving batch above
    // all); batch_dp picks the persistent kernel's shape from the entry
    if ( ! j->replaying && ! j->generic && ! getenv ( "MOTEX_DP_W" ) && ! getenv ( "MOTEX_DP_UR" ) &&
         ! getenv ( "MOTEX_DP_SWAR" ) )
    {
        const char * at = getenv ( "MOTEX_AUTOTUNE" );
        const bool enabled = ! ( at && atoi ( at ) == 0 );
        DPTune cached;
        if ( enabled && tune_lookup ( TuneKey { B, P.l, P.e, P.d }, &cached ) ) j->tune = cached;
        else tune_now = enabled && ! j->batched && ( uint64_t ) U * j->total >= kTuneMinCells;
    }
    const DPTune & tune = j->tune;
    const uint32_t groups = ( U + tune.NL - 1 ) / tune.NL;        // factors per register: NL
    const uint32_t per_cta = ( uint32_t ) kDPThreads * tune.W;
    j->ntiles = j->generic ? ( U + kDPThreads - 1 ) / kDPThreads : ( groups + per_cta - 1 ) / per_cta;
    j->nw64 = ( P.l + 63 ) / 64;
    if ( ! j->generic )
    {
        uint32_t * wpl;
        MTX_TRY ( ensure ( j, S_WPL32, ( size_t ) B * U, &wpl ) );
        MTX_LAUNCH ( k_wplanes32, blocks_for ( U, 256 ), 256, j->uniq, U, codes, P.l, ( uint32_t ) B, ed ? 0 : 1, wpl );
        da.wplanes32 = wpl;
    }
    else
    {
        uint64_t * wpl;
        MTX_TRY ( ensure ( j, S_WPL64, ( size_t ) B * U * j->nw64, &wpl ) );
        MTX_LAUNCH ( k_wplanes64, blocks_for ( U, 128 ), 128, j->uniq, U, codes, P.l, ( uint32_t ) B, j->nw64, ed ? 0 : 1,
                     wpl );
        da.wplanes64 = wpl;
    }
    const uint32_t first_blk = j->npat ? ( j->offs[j->npat] / 32 ) : 0;
    const uint32_t warmup = ed ? P.l + P.e - 1 : ( j->generic ? P.l - 1 : 0 );
    const uint32_t target = ( uint32_t ) j->ctx->num_sms * 24;
    uint32_t nchunks = std::max<uint32_t> ( 1, ( target + j->ntiles - 1 ) / j->ntiles );
    const uint32_t min_blocks = ed ? 16 : 4;
    nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, ( j->nblk - first_blk ) / min_blocks ) );
    if ( tune_now )
    {
        // the probe runs before the real chunk table and the accumulator clears
        da.u_acc = u_acc;
        da.v_acc = v_acc;
        uint8_t * fl;
        MTX_TRY ( ensure ( j, S_FLAGS, U, &fl ) );
        da.split_flags = fl;
        DPTune best = j->tune;
        MTX_TRY ( autotune ( j, &best ) );
        j->tune = best;
        const uint32_t g2 = ( U + best.NL - 1 ) / best.NL;
        j->ntiles = ( g2 + kDPThreads * best.W - 1 ) / ( kDPThreads * best.W );
        nchunks = std::max<uint32_t> ( 1, ( target + j->ntiles - 1 ) / j->ntiles );
        nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, ( j->nblk - first_blk ) / min_blocks ) );
    }
    build_chunks ( j, first_blk, nchunks, warmup, j->chunks );
    ChunkInfo * d_chunks;
    MTX_TRY ( upload_chunks ( j, &d_chunks ) );
    for ( auto & ch : j->chunks ) j->exec_cells += ( uint64_t ) U * ( ch.end - ch.warm ) * 32;
    uint8_t * flags;
    MTX_TRY ( ensure ( j, S_FLAGS, ( size_t ) std::max<uint32_t> ( 1, j->n_split ) * U, &flags ) );
    MTX_CUDA ( cudaMemsetAsync ( u_acc, 0, ( size_t ) U * 4, st ) );
    MTX_CUDA ( cudaMemsetAsync ( v_acc, 0, ( size_t ) U * 4, st ) );
    if ( j->n_split ) MTX_CUDA ( cudaMemsetAsync ( flags, 0, ( size_t ) j->n_split * U, st ) );
    da.chunks = d_chunks;
    da.u_acc = u_acc;
    da.v_acc = v_acc;
    da.split_flags = flags;
    j->dp_pending = true;
    return MOTEX_OK;
}

/*
 * Structured motifs (one gap): box planes for every pattern position, the
 * two-box DP over (pattern position x text chunk), then per (position, gap
 * choice) filter and ordered compaction.  Factors are not deduplicated here:
 * u and v are computed per pattern position like the reference, and the
 * key deduplication of the writer happens on the passing entries only.
 */
int plan_structured_n ( Job * j );

int plan_structured ( Job * j )
{
    const motex_params & P = j->prm;
    if ( ! struct1_shape ( &P ) ) return plan_structured_n ( j );
    j->structN = false;
    const bool ed = P.d == 1;
    cudaStream_t st = j->ctx->st;
    const int B = j->B;
    const uint32_t T = ( uint32_t ) j->total, G = j->G;
    const uint32_t b1 = j->blens[0], e1 = j->berrs[0], gmin = j->gmin[0], gmax = j->gmax[0];
    const uint8_t * codes = dptr<uint8_t> ( j, S_CODES );
    uint32_t *wpl0, *wpl1, *row_end;
    uint8_t * row_ok;
    MTX_TRY ( ensure ( j, S_WPL0, ( size_t ) B * T, &wpl0 ) );
    MTX_TRY ( ensure ( j, S_WPL1, ( size_t ) B * T, &wpl1 ) );
    MTX_TRY ( ensure ( j, S_ROWOK, T, &row_ok ) );
    MTX_TRY ( ensure ( j, S_ROWEND, T, &row_end ) );
    MTX_LAUNCH ( k_wplanes_all, blocks_for ( T, 256 ), 256, codes, T, P.l, ( uint32_t ) B, ed ? 0 : 1, wpl0 );
    MTX_LAUNCH ( k_wplanes_all, blocks_for ( T, 256 ), 256, codes, T, b1, ( uint32_t ) B, ed ? 0 : 1, wpl1 );
    MTX_LAUNCH ( k_struct_rows, blocks_for ( T, 256 ), 256, dptr<uint32_t> ( j, S_OFFS ), j->nseq, j->total, P.l,
                 j->tml, j->npat, row_ok, row_end );
    // end offset of box 1 for every gap choice k (the key deduplication reads it)
    {
        uint32_t * xoff;
        MTX_TRY ( ensure ( j, S_XOFF, G, &xoff ) );
        uint32_t * h_xoff = pin<uint32_t> ( j, kPinXoff );
        for ( uint32_t k = 0; k < G; ++k ) h_xoff[k] = gmin + k + b1;
        MTX_CUDA ( cudaMemcpyAsync ( xoff, h_xoff, ( size_t ) G * 4, cudaMemcpyHostToDevice, st ) );
    }

    const uint32_t ctas_x = ( T + kDPThreads - 1 ) / kDPThreads;
    j->ntiles = ctas_x;
    const uint32_t first_blk = j->npat ? ( j->offs[j->npat] / 32 ) : 0;
    const uint32_t warmup = ( ed ? std::max ( P.l + P.e - 1, b1 + e1 - 1 ) : 0 ) + gmax + b1;
    uint32_t nchunks = std::max<uint32_t> ( 1, ( ( uint32_t ) j->ctx->num_sms * 24 + ctas_x - 1 ) / ctas_x );
    nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, ( j->nblk - first_blk ) / 16 ) );
    build_chunks ( j, first_blk, nchunks, warmup, j->chunks );
    ChunkInfo * d_chunks;
    MTX_TRY ( upload_chunks ( j, &d_chunks ) );
    uint64_t scanned = 0;
    for ( auto & ch : j->chunks ) scanned += ( uint64_t ) ( ch.end - ch.warm ) * 32;
    j->exec_cells = ( uint64_t ) T * scanned * 2;

    const uint64_t n = ( uint64_t ) T * G;
    if ( n >= 0xffffff00ull ) return fail ( MOTEX_EUNSUPPORTED, "positions x gap choices exceeds 2^32" );
    uint32_t *u_acc, *v_acc;
    uint8_t * flags;
    MTX_TRY ( ensure ( j, S_UACC, n, &u_acc ) );
    MTX_TRY ( ensure ( j, S_VACC, n, &v_acc ) );
    MTX_TRY ( ensure ( j, S_FLAGS, std::max<uint64_t> ( 1, j->n_split ) * n, &flags ) );
    MTX_CUDA ( cudaMemsetAsync ( u_acc, 0, n * 4, st ) );
    MTX_CUDA ( cudaMemsetAsync ( v_acc, 0, n * 4, st ) );
    if ( j->n_split ) MTX_CUDA ( cudaMemsetAsync ( flags, 0, ( size_t ) j->n_split * n, st ) );

    StructArgs & sa = j->sa;
    sa.text.planes = dptr<uint32_t> ( j, S_PLANES );
    sa.text.plane_stride = j->stride;
    sa.text.vmask = dptr<uint32_t> ( j, S_VMASK );
    sa.text.emask = dptr<uint32_t> ( j, S_EMASK );
    sa.text.nblk = j->nblk;
    sa.wpl0 = wpl0;
    sa.wpl1 = wpl1;
    sa.row_ok = row_ok;
    sa.row_end = row_end;
    sa.total = T;
    sa.l0 = P.l;
    sa.e0 = P.e;
    sa.l1 = b1;
    sa.e1 = e1;
    sa.one = 1u;
    sa.ne0 = ~P.e;
    sa.ne1 = ~e1;
    sa.b1 = b1;
    sa.gmin = gmin;
    sa.gmax = gmax;
    sa.G = G;
    sa.chunks = d_chunks;
    sa.u_acc = u_acc;
    sa.v_acc = v_acc;
    sa.split_flags = flags;
    j->U = T;
    j->dp_pending = true;
    return MOTEX_OK;
}

/*
 * Structured motifs with several gaps (or one gap outside the shared-history
 * kernel's limits): the box-0 DP per pattern position with a direct check
 * of the later boxes at every box-0 hit (k_dp_structN).
 */
int plan_structured_n ( Job * j )
{
    const motex_params & P = j->prm;
    const bool ed = P.d == 1;
    cudaStream_t st = j->ctx->st;
    const int B = j->B;
    const uint32_t T = ( uint32_t ) j->total, NS = j->G, NG = P.nb_gaps;
    j->structN = true;
    const uint8_t * codes = dptr<uint8_t> ( j, S_CODES );
    uint32_t *wpl, *row_end, *seq_start, *xoff;
    uint8_t * row_ok;
    // rows of 64 bits when a box (or l) is longer than 32 symbols
    uint32_t maxlen = P.l;
    for ( uint32_t g = 0; g < NG; ++g ) maxlen = std::max ( maxlen, j->blens[g] );
    const bool wide = maxlen > 32;
    MTX_TRY ( ensure ( j, S_WPLN, ( size_t ) ( NG + 1 ) * B * T * ( wide ? 2 : 1 ), &wpl ) );
    MTX_TRY ( ensure ( j, S_ROWOK, T, &row_ok ) );
    MTX_TRY ( ensure ( j, S_ROWEND, T, &row_end ) );
    MTX_TRY ( ensure ( j, S_SEQSTART, T, &seq_start ) );
    MTX_TRY ( ensure ( j, S_XOFF, ( size_t ) NS * NG, &xoff ) );
    for ( uint32_t b = 0; b <= NG; ++b )
    {
        if ( wide )
            MTX_LAUNCH ( k_wplanes_all64, blocks_for ( T, 256 ), 256, codes, T, b ? j->blens[b - 1] : P.l, ( uint32_t ) B,
                         ed ? 0 : 1, reinterpret_cast<unsigned long long *> ( wpl ) + ( size_t ) b * B * T );
        else
            MTX_LAUNCH ( k_wplanes_all, blocks_for ( T, 256 ), 256, codes, T, b ? j->blens[b - 1] : P.l, ( uint32_t ) B,
                         ed ? 0 : 1, wpl + ( size_t ) b * B * T );
    }
    MTX_LAUNCH ( k_struct_rows, blocks_for ( T, 256 ), 256, dptr<uint32_t> ( j, S_OFFS ), j->nseq, j->total, P.l,
                 j->tml, j->npat, row_ok, row_end );
    MTX_LAUNCH ( k_seq_start, blocks_for ( T, 256 ), 256, dptr<uint32_t> ( j, S_OFFS ), j->nseq, j->total, seq_start );
    // cumulative end offsets of boxes 1..NG for every structure k (motex.cc:439-486 order)
    uint32_t * h_xoff = pin<uint32_t> ( j, kPinXoff );
    for ( uint32_t k = 0; k < NS; ++k )
    {
        uint32_t rem = k, off = 0;
        std::vector<uint32_t> S ( NG );
        for ( int g = ( int ) NG - 1; g >= 0; --g )
        {
            const uint32_t span = j->gmax[g] - j->gmin[g] + 1;
            S[g] = j->gmin[g] + rem % span;
            rem /= span;
        }
        for ( uint32_t g = 0; g < NG; ++g )
        {
            off += S[g] + j->blens[g];
            h_xoff[k * NG + g] = off;
        }
    }
    MTX_CUDA ( cudaMemcpyAsync ( xoff, h_xoff, ( size_t ) NS * NG * 4, cudaMemcpyHostToDevice, st ) );
    StructNArgs & sa = j->san;
    sa = StructNArgs {};
    sa.l0 = P.l;
    sa.e0 = P.e;
    sa.blen[0] = P.l;
    sa.berr[0] = P.e;
    for ( uint32_t g = 0; g < NG; ++g )
    {
        sa.blen[g + 1] = j->blens[g];
        sa.berr[g + 1] = j->berrs[g];
    }
    sa.ngaps = NG;
    sa.nstructs = NS;
    sa.wide = wide;
    if ( structN_smem_bytes ( sa ) > kStructNMaxSmem )
        return fail ( MOTEX_EUNSUPPORTED, "%u gap structures need more shared memory than a CTA has", NS );
    // block form where the shape allows: a warp owns Pw pattern positions
    j->structN_blk = structN_blk_shape ( sa, h_xoff, ed, &j->snb );
    const uint32_t per_cta = j->structN_blk ? ( kDPThreads / 32 ) * j->snb.Pw : kDPThreads;
    const uint32_t ctas_x = ( T + per_cta - 1 ) / per_cta;
    j->ntiles = ctas_x;
    const uint32_t first_blk = j->npat ? ( j->offs[j->npat] / 32 ) : 0;
    // edit distance restarts every box row's column this far before its
    // first counted position (exact for the <= e test of each box)
    uint32_t warmup = 0;
    if ( ed )
        for ( uint32_t b = 0; b <= NG; ++b ) warmup = std::max ( warmup, sa.blen[b] + sa.berr[b] - 1 );
    uint32_t nchunks = std::max<uint32_t> ( 1, ( ( uint32_t ) j->ctx->num_sms * 24 + ctas_x - 1 ) / ctas_x );
    nchunks = std::min<uint32_t> ( nchunks, std::max<uint32_t> ( 1, ( j->nblk - first_blk ) / 16 ) );
    build_chunks ( j, first_blk, nchunks, warmup, j->chunks );
    ChunkInfo * d_chunks;
    MTX_TRY ( upload_chunks ( j, &d_chunks ) );
    uint64_t scanned = 0;
    for ( auto & ch : j->chunks ) scanned += ( uint64_t ) ( ch.end - ch.warm ) * 32;
    // block form: every lane of a CTA runs ngaps + 1 rows
    j->exec_cells = ( j->structN_blk ? ( uint64_t ) ctas_x * kDPThreads : ( uint64_t ) T ) * scanned * ( NG + 1 );
    const uint64_t n = ( uint64_t ) T * NS;
    if ( n >= 0xffffff00ull ) return fail ( MOTEX_EUNSUPPORTED, "positions x gap structures exceeds 2^32" );
    uint32_t *u_acc, *v_acc;
    uint8_t * flags;
    MTX_TRY ( ensure ( j, S_UACC, n, &u_acc ) );
    MTX_TRY ( ensure ( j, S_VACC, n, &v_acc ) );
    MTX_TRY ( ensure ( j, S_FLAGS, std::max<uint64_t> ( 1, j->n_split ) * n, &flags ) );
    MTX_CUDA ( cudaMemsetAsync ( u_acc, 0, n * 4, st ) );
    MTX_CUDA ( cudaMemsetAsync ( v_acc, 0, n * 4, st ) );
    if ( j->n_split ) MTX_CUDA ( cudaMemsetAsync ( flags, 0, ( size_t ) j->n_split * n, st ) );
    sa.text.planes = dptr<uint32_t> ( j, S_PLANES );
    sa.text.plane_stride = j->stride;
    sa.text.vmask = dptr<uint32_t> ( j, S_VMASK );
    sa.text.emask = dptr<uint32_t> ( j, S_EMASK );
    sa.text.nblk = j->nblk;
    sa.wpl = wide ? nullptr : wpl;
    sa.wpl64 = wide ? reinterpret_cast<const unsigned long long *> ( wpl ) : nullptr;
    sa.row_ok = row_ok;
    sa.row_end = row_end;
    sa.seq_start = seq_start;
    sa.xoff = xoff;
    sa.total = T;
    sa.chunks = d_chunks;
    sa.u_acc = u_acc;
    sa.v_acc = v_acc;
    sa.split_flags = flags;
    j->U = T;
    j->dp_pending = true;
    return MOTEX_OK;
}

// DP of one job as its own (static-grid) launch.
int stage_dp ( Job * j )
{
    if ( ! j->dp_pending ) return MOTEX_OK;
    cudaStream_t st = j->ctx->st;
    const bool ed = j->prm.d == 1;
    MTX_TRY ( record ( j, j->evd0 ) );
    bool ok;
    if ( j->structured && j->structN && j->structN_blk )
        ok = launch_dp_structN_blk ( j->san, j->snb, j->B, ed, dim3 ( j->ntiles, ( unsigned ) j->chunks.size () ), st );
    else if ( j->structured && j->structN )
        ok = launch_dp_structN ( j->san, j->B, ed, dim3 ( j->ntiles, ( unsigned ) j->chunks.size () ), st );
    else if ( j->structured )
        ok = launch_dp_struct1 ( j->sa, j->B, ed, dim3 ( j->ntiles, ( unsigned ) j->chunks.size () ), st );
    else
    {
        const dim3 grid ( j->ntiles, ( unsigned ) j->chunks.size () );
        ok = j->generic        ? launch_dp_generic ( j->da, j->B, j->nw64, ed, grid, st )
             : j->tune.F       ? launch_dp_hclr ( j->da, j->B, j->tune.NL, j->tune.W, grid, st )
             : j->tune.NL > 1  ? ( ed ? launch_dp_swar_ed ( j->da, j->B, j->tune.NL, j->tune.W, j->tune.UR, grid, st )
                                        : launch_dp_hswar ( j->da, j->B, j->tune.NL, j->tune.W, j->tune.UR, grid, st ) )
                               : launch_dp_fast ( j->da, j->B, j->tune.W, j->tune.UR, ed, grid, st );
    }
    if ( ! ok ) return fail ( MOTEX_EUNSUPPORTED, "no DP kernel for l=%u B=%d", j->prm.l, j->B );
    MTX_TRY ( check_launch ( j, "k_dp" ) );
    MTX_TRY ( record ( j, j->evd1 ) );
    j->dp_pending = false;
    j->dp_timed = true;
    return MOTEX_OK;
}

// Returns through *need_sync whether the motif count must be read back.
int stage_finalize ( Job * j, bool * need_sync )
{
    const motex_params & P = j->prm;
    cudaStream_t st = j->ctx->st;
    *need_sync = false;
    uint32_t * scalar = dptr<uint32_t> ( j, S_SCALAR );
    if ( j->structured )
    {
        const uint64_t n = ( uint64_t ) j->total * j->G;
        StructFinalizeArgs fa {};
        fa.n = n;
        fa.u_acc = dptr<uint32_t> ( j, S_UACC );
        fa.v_acc = dptr<uint32_t> ( j, S_VACC );
        fa.split_flags = dptr<uint8_t> ( j, S_FLAGS );
        fa.n_split = j->n_split;
        fa.qok = dptr<uint8_t> ( j, S_QOK );
        fa.nseq = j->nseq;
        fa.nmin = P.n;
        fa.nmax = P.N;
        if ( j->npat )
        {
            uint32_t *uo, *vo;
            MTX_TRY ( ensure ( j, S_UOUT, n, &uo ) );
            MTX_TRY ( ensure ( j, S_VOUT, n, &vo ) );
            fa.u_out = uo;
            fa.v_out = vo;
            MTX_LAUNCH ( k_struct_finalize, blocks_for ( n, 256 ), 256, fa );
            j->nrec = 0;
            return MOTEX_OK;
        }
        uint8_t * mark;
        uint32_t *recu, *recv, *pref2;
        MTX_TRY ( ensure ( j, S_MARK, n, &mark ) );
        MTX_TRY ( ensure ( j, S_RECU, n, &recu ) );
        MTX_TRY ( ensure ( j, S_RECV, n, &recv ) );
        MTX_TRY ( ensure ( j, S_PREF2, n, &pref2 ) );
        fa.mark = mark;
        fa.rec_u = recu;
        fa.rec_v = recv;
        MTX_LAUNCH ( k_struct_finalize, blocks_for ( n, 256 ), 256, fa );
        MTX_TRY ( scan_flags ( j, mark, ( uint32_t ) n, pref2, scalar ) );
        MTX_CUDA ( cudaMemcpyAsync ( pin<uint32_t> ( j, kPinScalar ) + 1, scalar, 4, cudaMemcpyDeviceToHost, st ) );
        *need_sync = true;
        return MOTEX_OK;
    }
    const uint32_t U = j->U;
    FinalizeArgs fa {};
    fa.U = U;
    fa.u_acc = dptr<uint32_t> ( j, S_UACC );
    fa.v_acc = dptr<uint32_t> ( j, S_VACC );
    fa.split_flags = dptr<uint8_t> ( j, S_FLAGS );
    fa.n_split = j->n_split;
    fa.qok = dptr<uint8_t> ( j, S_QOK );
    fa.nseq = j->nseq;
    fa.nmin = P.n;
    fa.nmax = P.N;
    fa.uniq_pos = j->uniq;
    if ( j->npat )
    {
        uint32_t *uo, *vo;
        MTX_TRY ( ensure ( j, S_UOUT, std::max<uint32_t> ( 1, U ), &uo ) );
        MTX_TRY ( ensure ( j, S_VOUT, std::max<uint32_t> ( 1, U ), &vo ) );
        fa.u_out = uo;
        fa.v_out = vo;
        if ( U ) MTX_LAUNCH ( k_finalize, blocks_for ( U, 256 ), 256, fa );
        j->nrec = 0;
        return MOTEX_OK;
    }
    uint8_t * mark;
    uint32_t *recu, *recv, *pref2;
    const uint32_t T = ( uint32_t ) j->total;
    MTX_TRY ( ensure ( j, S_MARK, T, &mark ) );
    MTX_TRY ( ensure ( j, S_RECU, T, &recu ) );
    MTX_TRY ( ensure ( j, S_RECV, T, &recv ) );
    MTX_TRY ( ensure ( j, S_PREF2, T, &pref2 ) );
    MTX_CUDA ( cudaMemsetAsync ( mark, 0, T, st ) );
    fa.mark = mark;
    fa.rec_u = recu;
    fa.rec_v = recv;
    if ( U ) MTX_LAUNCH ( k_finalize, blocks_for ( U, 256 ), 256, fa );
    MTX_TRY ( scan_flags ( j, mark, T, pref2, scalar ) );
    MTX_CUDA ( cudaMemcpyAsync ( pin<uint32_t> ( j, kPinScalar ) + 1, scalar, 4, cudaMemcpyDeviceToHost, st ) );
    *need_sync = true;
    return MOTEX_OK;
}

int stage_compact ( Job * j )
{
    uint32_t * scalar = dptr<uint32_t> ( j, S_SCALAR );
    MTX_CUDA ( cudaMemsetAsync ( scalar + 2, 0, 4, j->ctx->st ) );
    if ( ! j->npat )
    {
        if ( ! j->replaying ) j->nrec = pin<uint32_t> ( j, kPinScalar )[1];
        const uint32_t n = ( uint32_t ) ( j->structured ? j->total * j->G : j->total );
        uint32_t * recs;
        MTX_TRY ( ensure ( j, S_RECS, ( size_t ) 3 * std::max<uint32_t> ( 1, j->nrec ), &recs ) );
        MTX_LAUNCH ( k_compact, std::min<unsigned> ( blocks_for ( ( n + 15 ) / 16, 256 ), 64 * j->ctx->num_sms ), 256,
                     dptr<uint8_t> ( j, S_MARK ), dptr<uint32_t> ( j, S_PREF2 ), n,
                     dptr<uint32_t> ( j, S_RECU ), dptr<uint32_t> ( j, S_RECV ), recs );
        if ( j->structured && j->nrec )
        {
            // the writer's key deduplication (functions.cc:1191-1239) on the
            // device: a hash table of the entries' box symbols keeps the
            // first entry of every key in print order
            SKeyArgs ka {};
            ka.recs = recs;
            ka.nrec = j->nrec;
            ka.G = j->G;
            ka.NG = j->prm.nb_gaps;
            ka.l = j->prm.l;
            for ( uint32_t g = 0; g < ka.NG; ++g ) ka.blen[g] = j->blens[g];
            ka.codes = dptr<uint8_t> ( j, S_CODES );
            ka.xoff = dptr<uint32_t> ( j, S_XOFF );
            ka.tbits = 5;
            while ( ( 1ull << ka.tbits ) < 2ull * j->nrec ) ++ka.tbits;
            uint32_t * tab;
            MTX_TRY ( ensure ( j, S_STAB, ( size_t ) 2 << ka.tbits, &tab ) );
            MTX_TRY ( ensure ( j, S_SSLOT, j->nrec, &ka.slot_of ) );
            MTX_TRY ( ensure ( j, S_SKEEP, j->nrec, &ka.keep ) );
            ka.rep = tab;
            ka.first = tab + ( ( size_t ) 1 << ka.tbits );
            ka.err = scalar + 2;
            MTX_CUDA ( cudaMemsetAsync ( tab, 0xff, ( size_t ) 8 << ka.tbits, j->ctx->st ) );
            MTX_LAUNCH ( k_skey_insert, blocks_for ( j->nrec, 256 ), 256, ka );
            MTX_LAUNCH ( k_skey_keep, blocks_for ( j->nrec, 256 ), 256, ka );
        }
    }
    // the key-table and packer staging-wait flags come back with the results
    MTX_CUDA ( cudaMemcpyAsync ( pin<uint32_t> ( j, kPinScalar ) + 2, scalar + 2, 8, cudaMemcpyDeviceToHost, j->ctx->st ) );
    MTX_TRY ( record ( j, j->ev1 ) );
    return MOTEX_OK;
}

int read_times ( Job * j )
{
    MTX_CUDA ( cudaEventSynchronize ( j->ev1 ) );
    if ( const uint32_t e = pin<uint32_t> ( j, kPinScalar )[3] )
        return fail ( MOTEX_ETIMEOUT, "packing: a TMA staging wait gave up (copy not completed)%s",
                      ( e & 2u ) ? "; so did the drain of the copies in flight" : "" );
    if ( pin<uint32_t> ( j, kPinScalar )[2] ) return fail ( MOTEX_ECUDA, "structured key table overflow" );
    MTX_CUDA ( cudaEventElapsedTime ( &j->device_ms, j->ev0, j->ev1 ) );
    if ( j->dp_timed ) MTX_CUDA ( cudaEventElapsedTime ( &j->dp_ms, j->evd0, j->evd1 ) );
    return MOTEX_OK;
}

int sync ( motex_ctx * c )
{
    MTX_CUDA ( cudaStreamSynchronize ( c->st ) );
    return MOTEX_OK;
}

// All stages of one job on its own.
int run_job ( Job * j )
{
    motex_ctx * c = j->ctx;
    bool need;
    MTX_TRY ( stage_presence ( j ) );
    if ( ! j->replaying ) MTX_TRY ( sync ( c ) );
    MTX_TRY ( stage_pack ( j, &need ) );
    if ( need && ! j->replaying ) MTX_TRY ( sync ( c ) );
    MTX_TRY ( stage_plan ( j, need ) );
    MTX_TRY ( stage_dp ( j ) );
    MTX_TRY ( stage_finalize ( j, &need ) );
    if ( need && ! j->replaying ) MTX_TRY ( sync ( c ) );
    MTX_TRY ( stage_compact ( j ) );
    return MOTEX_OK;
}

/*
 * Repeated execution of the same resident job: after a first run fixed every
 * size the host reads back, the second run records the staged sequence into
 * a CUDA graph (no host syncs inside) and every later run replays it as one
 * launch.  Buffers do not move between runs, so the graph stays valid until
 * the next load.
 */
int execute_job ( Job * j )
{
    motex_ctx * c = j->ctx;
    if ( j->graph )
    {
        MTX_CUDA ( cudaGraphLaunch ( j->graph, c->st ) );
        j->ctx->launches += j->graph_kernels;         // kernels executed by the replay
        j->launches = j->graph_kernels;
        MTX_TRY ( read_times ( j ) );
        j->runs_since_load++;
        return MOTEX_OK;
    }
    const bool capture = j->runs_since_load >= 1 && ! getenv ( "MOTEX_NO_GRAPH" );
    if ( ! capture )
    {
        j->replaying = false;
        MTX_TRY ( run_job ( j ) );
        MTX_TRY ( read_times ( j ) );
        j->runs_since_load++;
        return MOTEX_OK;
    }
    j->replaying = true;
    cudaGraph_t g = nullptr;
    MTX_CUDA ( cudaStreamBeginCapture ( c->st, cudaStreamCaptureModeRelaxed ) );
    int rc = run_job ( j );
    cudaError_t ce = cudaStreamEndCapture ( c->st, &g );
    j->replaying = false;
    if ( rc != MOTEX_OK )
    {
        if ( g ) cudaGraphDestroy ( g );
        return rc;
    }
    if ( ce != cudaSuccess ) return fail ( MOTEX_ECUDA, "graph capture failed: %s", cudaGetErrorString ( ce ) );
    ce = cudaGraphInstantiate ( &j->graph, g, 0 );
    cudaGraphDestroy ( g );
    if ( ce != cudaSuccess )
    {
        j->graph = nullptr;
        return fail ( MOTEX_ECUDA, "graph instantiation failed: %s", cudaGetErrorString ( ce ) );
    }
    j->graph_kernels = j->launches;
    MTX_CUDA ( cudaGraphLaunch ( j->graph, c->st ) );
    MTX_TRY ( read_times ( j ) );
    j->runs_since_load++;
    return MOTEX_OK;
}

/*
 * npat = 0: all-pairs (every sequence gives factors and is searched).
 * npat > 0: sequences [0, npat) give the factors and [npat, nseq) are the
 * texts.  skip_short applies the reference's short-sequence skip
 * (total_mot_length > n) to the searched sequences.
 */
int load_job ( Job * j, const motex_params * prm, const char * const * seqs, const uint32_t * lens, uint32_t nseq,
               uint32_t npat, bool skip_short )
{
    MTX_TRY ( validate ( prm ) );
    if ( ! seqs || ! lens ) return fail ( MOTEX_EINVAL, "null sequence arrays" );
    if ( nseq == 0 ) return fail ( MOTEX_EINVAL, "no sequences" );
    drop_graph ( j );
    j->loaded = j->executed = false;
    j->prm = *prm;
    j->gmin.assign ( prm->gap_min, prm->gap_min + prm->nb_gaps );
    j->gmax.assign ( prm->gap_max, prm->gap_max + prm->nb_gaps );
    j->blens.assign ( prm->blens, prm->blens + prm->nb_gaps );
    j->berrs.assign ( prm->berrs, prm->berrs + prm->nb_gaps );
    j->prm.gap_min = j->gmin.data ();
    j->prm.gap_max = j->gmax.data ();
    j->prm.blens = j->blens.data ();
    j->prm.berrs = j->berrs.data ();
    j->G = 1;                                      // gap structures (lexicographic, gap 0 slowest)
    for ( uint32_t g = 0; g < prm->nb_gaps; ++g ) j->G *= j->gmax[g] - j->gmin[g] + 1;
    j->nseq = nseq;
    j->npat = npat;
    j->offs.assign ( nseq + 1, 0 );
    uint64_t total = 0;
    for ( uint32_t i = 0; i < nseq; ++i )
    {
        if ( lens[i] && ! seqs[i] ) return fail ( MOTEX_EINVAL, "null sequence %u", i );
        j->offs[i] = ( uint32_t ) total;
        total += lens[i];
        if ( total >= 0xffffff00ull ) return fail ( MOTEX_EUNSUPPORTED, "total input length exceeds 4 G symbols" );
    }
    j->offs[nseq] = ( uint32_t ) total;
    j->total = total;
    if ( total == 0 ) return fail ( MOTEX_EINVAL, "empty input" );
    const uint32_t l = prm->l;
    // total_mot_length (motex.cc:312-360): l plus minimum gaps and boxes
    uint32_t tml_full = l;
    for ( uint32_t g = 0; g < prm->nb_gaps; ++g ) tml_full += j->gmin[g] + j->blens[g];
    j->tml = skip_short ? tml_full : 0;
    // factor ends per sequence and the reference's cell count
    std::vector<uint32_t> wstart ( nseq + 1, 0 );
    uint64_t nw = 0, searched = 0, pattern_len = 0;
    for ( uint32_t i = 0; i < nseq; ++i )
    {
        wstart[i] = ( uint32_t ) nw;
        const bool has_words = lens[i] >= std::max ( l, j->tml ) && ( npat == 0 || i < npat );
        if ( has_words ) nw += lens[i] - l + 1;
        if ( i < npat ) pattern_len += lens[i];
        else if ( lens[i] >= j->tml ) searched += lens[i];
    }
    wstart[nseq] = ( uint32_t ) nw;
    j->nwords = ( uint32_t ) nw;
    j->ref_cells = ( npat ? pattern_len * searched : searched * searched ) * ( prm->nb_gaps + 1 );
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
    MTX_TRY ( ensure_pinned ( j, kPinStage + raw_b + 2 * offs_b + nseq + 16 ) );
    uint8_t * stage = pin<uint8_t> ( j, kPinStage );
    size_t at = 0;
    for ( uint32_t i = 0; i < nseq; ++i )
    {
        memcpy ( stage + at, seqs[i], lens[i] );
        at += lens[i];
    }
    memcpy ( stage + raw_b, j->offs.data (), ( size_t ) ( nseq + 1 ) * 4 );
    memcpy ( stage + raw_b + offs_b, wstart.data (), ( size_t ) ( nseq + 1 ) * 4 );
    memcpy ( stage + raw_b + 2 * offs_b, qok.data (), nseq + 1 );
    uint8_t * raw;
    uint32_t *doffs, *dws;
    uint8_t * dq;
    MTX_TRY ( ensure ( j, S_RAW, raw_b + 16, &raw ) );
    MTX_TRY ( ensure ( j, S_OFFS, nseq + 1, &doffs ) );
    MTX_TRY ( ensure ( j, S_WSTART, nseq + 1, &dws ) );
    MTX_TRY ( ensure ( j, S_QOK, nseq + 1, &dq ) );
    cudaStream_t st = j->ctx->st;
    MTX_CUDA ( cudaMemcpyAsync ( raw, stage, total, cudaMemcpyHostToDevice, st ) );
    MTX_CUDA ( cudaMemcpyAsync ( doffs, stage + raw_b, ( size_t ) ( nseq + 1 ) * 4, cudaMemcpyHostToDevice, st ) );
    MTX_CUDA ( cudaMemcpyAsync ( dws, stage + raw_b + offs_b, ( size_t ) ( nseq + 1 ) * 4, cudaMemcpyHostToDevice, st ) );
    MTX_CUDA ( cudaMemcpyAsync ( dq, stage + raw_b + 2 * offs_b, nseq + 1, cudaMemcpyHostToDevice, st ) );
    j->loaded = true;
    return MOTEX_OK;
}

// Queue the copy of the job's records into its pinned stage.
int fetch_issue ( Job * j )
{
    if ( j->nrec == 0 ) return MOTEX_OK;
    const size_t bytes = ( size_t ) j->nrec * 12;
    const bool keyed = j->prm.nb_gaps && ! j->npat;              // structured: the device's keep flags too
    MTX_TRY ( ensure_pinned ( j, kPinStage + bytes + ( keyed ? j->nrec : 0 ) ) );
    MTX_CUDA ( cudaMemcpyAsync ( pin<uint32_t> ( j, kPinStage ), dptr<uint32_t> ( j, S_RECS ), bytes,
                                 cudaMemcpyDeviceToHost, j->ctx->st ) );
    if ( keyed )
        MTX_CUDA ( cudaMemcpyAsync ( pin<uint8_t> ( j, kPinStage + bytes ), dptr<uint8_t> ( j, S_SKEEP ), j->nrec,
                                     cudaMemcpyDeviceToHost, j->ctx->st ) );
    return MOTEX_OK;
}

// The result from the copied records (the copy has completed).
int fetch_build ( Job * j, motex_result * out );

int fetch_records ( Job * j, motex_result * out )
{
    if ( j->nrec )
    {
        MTX_TRY ( sync ( j->ctx ) );
        MTX_TRY ( fetch_issue ( j ) );
        MTX_TRY ( sync ( j->ctx ) );
    }
    return fetch_build ( j, out );
}

int fetch_build ( Job * j, motex_result * out )
{
    memset ( out, 0, sizeof *out );
    out->num_seqs = j->nseq;
    out->ref_cells = j->ref_cells;
    out->exec_cells = j->exec_cells;
    out->unique_words = j->U;
    out->launches = j->launches;
    out->device_ms = j->device_ms;
    out->dp_ms = j->dp_ms;
    if ( j->nrec == 0 ) return MOTEX_OK;
    const uint32_t * h = pin<uint32_t> ( j, kPinStage );
    out->motifs = static_cast<motex_motif *> ( malloc ( ( size_t ) j->nrec * sizeof ( motex_motif ) ) );
    if ( ! out->motifs ) return fail ( MOTEX_ENOMEM, "host allocation of the result failed" );
    const uint32_t G = j->prm.nb_gaps ? j->G : 1;
    // structured: the first entry of every key in print order, flagged on the device
    const uint8_t * keep = j->prm.nb_gaps && ! j->npat ? pin<uint8_t> ( j, kPinStage + ( size_t ) j->nrec * 12 ) : nullptr;
    uint32_t s = 0, kept = 0;
    for ( uint32_t i = 0; i < j->nrec; ++i )
    {
        const uint32_t idx = h[3 * i];
        const uint32_t pos = idx / G, k = idx % G;
        while ( j->offs[s + 1] <= pos ) ++s;        // records are in (position, gap choice) order
        if ( keep && ! keep[i] ) continue;
        out->motifs[kept++] = motex_motif { s, pos - j->offs[s], k, h[3 * i + 1], h[3 * i + 2] };
    }
    out->count = kept;
    return MOTEX_OK;
}

// ---------------------------------------------------------------- batches

/*
 * DP of many jobs: single-motif jobs with the 32-bit kernels are grouped by
 * kernel class (alphabet planes, distance, score form, lanes per register)
 * and each class runs as one persistent launch over the list of all its
 * (job, tile, chunk) items, largest items first; other jobs (structured,
 * factors longer than 32) run their own static-grid launch.
 */
int batch_dp ( motex_ctx * c, std::vector<Job *> & jobs, float * dp_ms )
{
    // packed classes also key on l and e: their lane constants are a kernel
    // parameter shared by every job of the launch
    struct Class
    {
        int B;
        bool ed, scaled;
        int NL;
        uint32_t l, e;
        int W, UR;
        int E;                                       // popc-free Hamming: e; otherwise -1
        bool operator< ( const Class & o ) const
        {
            return std::tie ( B, ed, scaled, NL, l, e, W, UR, E ) <
                   std::tie ( o.B, o.ed, o.scaled, o.NL, o.l, o.e, o.W, o.UR, o.E );
        }
    };
    std::map<Class, std::vector<Job *>> classes;
    MTX_CUDA ( cudaEventRecord ( c->evb0, c->st ) );
    for ( Job * j : jobs )
    {
        if ( ! j->dp_pending ) continue;
        if ( j->structured || j->generic )
        {
            MTX_TRY ( stage_dp ( j ) );
            continue;
        }
        const bool ed = j->prm.d == 1;
        const int Bc = j->B < 2 ? 2 : j->B;
        // launch shape: the autotuner's entry for the key (from this process
        // or the tune cache) where a persistent kernel implements it, else
        // the persistent defaults (packed edit distance: W by bit planes,
        // unroll 8; otherwise W = 8 with the kernel's unroll)
        DPTune t;
        const bool tuned = ! getenv ( "MOTEX_DP_W" ) && ! getenv ( "MOTEX_DP_UR" ) && ! getenv ( "MOTEX_DP_SWAR" ) &&
                           tune_lookup ( TuneKey { j->B, j->prm.l, j->prm.e, j->prm.d }, &t ) &&
                           persistent_shape ( Bc, ed, t.NL, t.W, t.UR, t.F ? ( int ) j->prm.e : -1 );
        if ( tuned ) j->tune = t;
        else
        {
            // defaults (choose_tune's form and lane count): W = 8 except packed
            // edit distance, the kernel's unroll
            j->tune.W = ( j->tune.NL > 1 && ed ) ? swar_default_w ( Bc ) : 8;
            j->tune.UR = ( j->tune.NL > 1 ? ( ed ? 8 : 4 ) : ( ed ? 8 : 4 ) );
        }
        const bool packed = j->tune.NL > 1;
        const int E = j->tune.F ? ( int ) j->prm.e : -1;
        Class k { Bc, ed, ed && j->prm.l <= 28 && j->tune.NL == 1, j->tune.NL,
                  packed ? j->prm.l : 0u, packed && ( ed || E >= 0 ) ? j->prm.e : 0u, j->tune.W, j->tune.UR, E };
        const uint32_t groups = ( j->U + j->tune.NL - 1 ) / j->tune.NL;
        j->ntiles = ( groups + kDPThreads * j->tune.W - 1 ) / ( kDPThreads * j->tune.W );
        classes[k].push_back ( j );
    }
    // a class of one job runs that job's static grid: one launch over its
    // (tile, chunk) items either way, and the one-job kernel holds the job's
    // constants in the constant bank (measured on the 2000-protein edit-
    // distance set: 294 ms static against 315-328 ms persistent)
    for ( auto it = classes.begin (); it != classes.end (); )
    {
        if ( it->second.size () == 1 )
        {
            MTX_TRY ( stage_dp ( it->second[0] ) );
            it = classes.erase ( it );
        }
        else ++it;
    }
    size_t njobs = 0, nitems = 0;
    for ( auto & kv : classes )
        for ( Job * j : kv.second )
        {
            njobs++;
            nitems += ( size_t ) j->ntiles * j->chunks.size ();
        }
    if ( njobs )
    {
        const size_t jb = njobs * sizeof ( JobDesc ), ib = nitems * sizeof ( WorkItem );
        MTX_TRY ( alloc_pinned ( &c->bpinned, &c->bpinned_cap, jb + ib + 64, c->st ) );
        MTX_TRY ( alloc_dev ( c->bjobs, jb ) );
        MTX_TRY ( alloc_dev ( c->bitems, ib ) );
        MTX_TRY ( alloc_dev ( c->bcounter, classes.size () * sizeof ( uint32_t ) ) );
        JobDesc * hj = static_cast<JobDesc *> ( c->bpinned );
        WorkItem * hi = reinterpret_cast<WorkItem *> ( static_cast<uint8_t *> ( c->bpinned ) + jb );
        JobDesc * dj = static_cast<JobDesc *> ( c->bjobs.p );
        WorkItem * di = static_cast<WorkItem *> ( c->bitems.p );
        uint32_t * dcount = static_cast<uint32_t *> ( c->bcounter.p );
        MTX_CUDA ( cudaMemsetAsync ( dcount, 0, classes.size () * sizeof ( uint32_t ), c->st ) );
        size_t jat = 0, iat = 0, ci = 0;
        for ( auto & kv : classes )
        {
            const size_t jfirst = jat, ifirst = iat;
            // items of the class, largest first
            std::vector<std::pair<uint64_t, WorkItem>> items;
            for ( Job * j : kv.second )
            {
                hj[jat].a = j->da;
                hj[jat].C = j->tune.NL <= 1 ? SwarConst {}
                            : j->tune.F     ? hclr_const ( j->prm.l, j->tune.NL )
                            : ( j->prm.d == 1 ? swar_const ( j->prm.l, j->prm.e, j->tune.NL )
                                              : hswar_const ( j->prm.l, j->tune.NL ) );
                const uint64_t words = ( uint64_t ) kDPThreads * j->tune.W * j->tune.NL;
                for ( uint32_t ch = 0; ch < j->chunks.size (); ++ch )
                {
                    const uint64_t cost = words * ( j->chunks[ch].end - j->chunks[ch].warm );
                    for ( uint32_t t = 0; t < j->ntiles; ++t )
                        items.push_back ( { cost, WorkItem { ( uint32_t ) ( jat - jfirst ), t, ch } } );
                }
                j->dp_pending = false;
                jat++;
            }
            std::stable_sort ( items.begin (), items.end (),
                               [] ( const auto & a, const auto & b ) { return a.first > b.first; } );
            for ( auto & it : items ) hi[iat++] = it.second;
            const size_t cn = iat - ifirst;
            MTX_CUDA ( cudaMemcpyAsync ( dj + jfirst, hj + jfirst, ( jat - jfirst ) * sizeof ( JobDesc ),
                                         cudaMemcpyHostToDevice, c->st ) );
            MTX_CUDA ( cudaMemcpyAsync ( di + ifirst, hi + ifirst, cn * sizeof ( WorkItem ), cudaMemcpyHostToDevice, c->st ) );
            const Class & k = kv.first;
            const int per_sm = persistent_ctas_per_sm ( k.B, k.ed, k.scaled, k.NL, k.W, k.UR, k.E );
            const unsigned grid = ( unsigned ) std::min<size_t> ( cn, ( size_t ) per_sm * c->num_sms );
            if ( ! launch_dp_persistent ( dj + jfirst, di + ifirst, ( uint32_t ) cn, dcount + ci, k.B, k.ed, k.scaled,
                                          k.NL, k.W, k.UR, k.E, hj[jfirst].C, grid, c->st ) )
                return fail ( MOTEX_EUNSUPPORTED, "no persistent DP kernel for this class" );
            c->launches++;
            cudaError_t e = cudaGetLastError ();
            if ( e != cudaSuccess ) return fail ( MOTEX_ECUDA, "persistent DP launch failed: %s", cudaGetErrorString ( e ) );
            for ( Job * j : kv.second ) j->launches++;
            ci++;
        }
    }
    MTX_CUDA ( cudaEventRecord ( c->evb1, c->st ) );
    MTX_CUDA ( cudaEventSynchronize ( c->evb1 ) );
    MTX_CUDA ( cudaEventElapsedTime ( dp_ms, c->evb0, c->evb1 ) );
    return MOTEX_OK;
}

// ------------------------------------------------------- small jobs

/*
 * Whether a loaded job takes the small-job pipeline (mini.cu): a whole-set
 * run of plain motifs of at most kMiniMaxSymbols symbols whose factors pack
 * into 63 bits.  Its alphabet (code map and bit planes B) is taken here from
 * the staged input, which also spares the presence kernel and its sync.
 * MOTEX_MINI=0 sends every job down the staged pipeline.
 */
bool mini_eligible ( Job * j )
{
    const motex_params & P = j->prm;
    if ( const char * e = getenv ( "MOTEX_MINI" ) )
        if ( atoi ( e ) == 0 ) return false;
    if ( j->npat || P.nb_gaps || P.l > 31 || j->total > kMiniMaxSymbols ) return false;
    const uint8_t * raw = pin<uint8_t> ( j, kPinStage );          // load_job staged the input here
    uint8_t seen[256] = {};
    for ( uint64_t i = 0; i < j->total; ++i ) seen[raw[i]] = 1;
    uint8_t * cmap = pin<uint8_t> ( j, kPinCmap );
    uint32_t sigma = 0;
    for ( int i = 0; i < 256; ++i ) cmap[i] = seen[i] ? ( uint8_t ) sigma++ : 0;
    int B = 2;                                      // one- and two-symbol inputs run on the 2-plane kernels
    while ( ( 1u << B ) < sigma ) ++B;
    if ( B > kMaxPlanes || P.l * ( uint32_t ) B > 63 ) return false;
    j->B = B;
    return true;
}

/*
 * The small-job pipeline for loaded, eligible jobs: clear, pack, uniq,
 * planes (grids of every job's CTAs) -> sync (distinct-factor counts) -> the
 * DP (the job's static launch when alone, the batch's persistent launches
 * otherwise) -> final, count, write -> sync (motif counts) -> record copies
 * queued -> sync.  The caller reads the times and builds the results.
 */
int run_mini ( motex_ctx * c, std::vector<Job *> & js, float * dp_ms )
{
    const uint32_t n = ( uint32_t ) js.size ();
    cudaStream_t st = c->st;
    *dp_ms = 0.f;
    // text chunks: enough (job, tile, chunk) items to fill the GPU, tiles
    // estimated from the factor counts (the distinct count is not known yet)
    uint64_t tiles_all = 0;
    for ( Job * j : js )
    {
        const DPTune t = choose_tune ( j, std::max<uint32_t> ( 1, j->nwords ), j->prm.d == 1, false );
        const uint32_t groups = ( j->nwords + t.NL - 1 ) / t.NL;
        tiles_all += std::max<uint32_t> ( 1, ( groups + kDPThreads * t.W - 1 ) / ( kDPThreads * t.W ) );
    }
    const uint64_t target = ( uint64_t ) c->num_sms * 24;
    const uint32_t want_chunks = ( uint32_t ) std::max<uint64_t> ( 1, ( target + tiles_all - 1 ) / tiles_all );
    const size_t descb = ( ( size_t ) n * sizeof ( MiniJob ) + 255 ) & ~( size_t ) 255, resb = ( size_t ) n * 16;
    MTX_TRY ( alloc_pinned ( &c->mpinned, &c->mpinned_cap, descb + resb, st ) );
    MTX_TRY ( alloc_dev ( c->mjobs, descb ) );
    MTX_TRY ( alloc_dev ( c->mres, resb ) );
    MTX_TRY ( alloc_dev ( c->mpart, ( size_t ) n * kMiniMaxCtas * sizeof ( uint32_t ) ) );
    uint32_t max_ctas = 1;
    MiniJob * hd = static_cast<MiniJob *> ( c->mpinned );
    uint32_t * hres = reinterpret_cast<uint32_t *> ( static_cast<uint8_t *> ( c->mpinned ) + descb );
    MiniJob * dd = static_cast<MiniJob *> ( c->mjobs.p );
    uint32_t * dres = static_cast<uint32_t *> ( c->mres.p );
    for ( uint32_t i = 0; i < n; ++i )
    {
        Job * j = js[i];
        const motex_params & P = j->prm;
        const bool ed = P.d == 1;
        j->replaying = false;
        j->structured = j->generic = j->structN = j->structN_blk = false;
        j->launches = 0;
        j->exec_cells = 0;
        j->dp_ms = 0.f;
        j->dp_timed = false;
        j->dp_pending = false;
        j->nblk = ( uint32_t ) ( ( j->total + 31 ) / 32 );
        j->stride = ( j->nblk + 1 + 31 ) & ~31u;
        const uint32_t nchunks = std::min<uint32_t> ( { want_chunks, 32u, std::max<uint32_t> ( 1, j->nblk / ( ed ? 16 : 4 ) ) } );
        build_chunks ( j, 0, nchunks, ed ? P.l + P.e - 1 : 0, j->chunks );
        ChunkInfo * d_chunks;
        MTX_TRY ( upload_chunks ( j, &d_chunks ) );
        uint32_t tbits = 5;
        while ( ( 1ull << tbits ) < 2ull * j->nwords ) ++tbits;
        const uint32_t nw = std::max<uint32_t> ( 1, j->nwords );
        MiniJob & m = hd[i];
        m = MiniJob {};
        m.raw = dptr<uint8_t> ( j, S_RAW );
        m.offs = dptr<uint32_t> ( j, S_OFFS );
        m.qok = dptr<uint8_t> ( j, S_QOK );
        m.nseq = j->nseq;
        m.total = ( uint32_t ) j->total;
        m.l = P.l;
        m.tml = j->tml;
        m.vstart = ed ? 0 : P.l - 1;
        m.B = ( uint32_t ) j->B;
        m.nmin = P.n;
        m.nmax = P.N;
        m.n_split = j->n_split;
        m.nblk = j->nblk;
        m.plane_stride = j->stride;
        m.tbits = tbits;
        m.top_aligned = ed ? 0 : 1;
        unsigned long long * tkey;
        MTX_TRY ( ensure ( j, S_CODES, j->total + 64, &m.codes ) );
        MTX_TRY ( ensure ( j, S_PLANES, ( size_t ) j->B * j->stride, &m.planes ) );
        MTX_TRY ( ensure ( j, S_VMASK, j->nblk, &m.vmask ) );
        MTX_TRY ( ensure ( j, S_EMASK, j->nblk, &m.emask ) );
        MTX_TRY ( ensure ( j, S_KEY0, ( size_t ) 2 << tbits, reinterpret_cast<uint32_t **> ( &tkey ) ) );
        m.tkey = tkey;
        MTX_TRY ( ensure ( j, S_IDX1, ( size_t ) 1 << tbits, &m.tpos ) );
        MTX_TRY ( ensure ( j, S_UNIQ, nw, &m.uniq ) );
        MTX_TRY ( ensure ( j, S_WPL32, ( size_t ) j->B * nw, &m.wpl ) );
        MTX_TRY ( ensure ( j, S_UACC, nw, &m.u_acc ) );
        MTX_TRY ( ensure ( j, S_VACC, nw, &m.v_acc ) );
        MTX_TRY ( ensure ( j, S_FLAGS, ( size_t ) std::max<uint32_t> ( 1, j->n_split ) * nw, &m.flags ) );
        MTX_TRY ( ensure ( j, S_MARK, j->total, &m.mark ) );
        MTX_TRY ( ensure ( j, S_RECU, j->total, &m.rec_u ) );
        MTX_TRY ( ensure ( j, S_RECV, j->total, &m.rec_v ) );
        MTX_TRY ( ensure ( j, S_RECS, ( size_t ) 3 * nw, &m.recs ) );
        m.result = dres + 4 * i;
        m.part = static_cast<uint32_t *> ( c->mpart.p ) + ( size_t ) i * kMiniMaxCtas;
        m.nwords = j->nwords;
        // the stages around the DP are latency-bound (a few dependent loads and
        // atomics per position or factor): one 1024-thread CTA per 1024 symbols
        m.ctas = ( uint32_t ) std::min<uint64_t> ( kMiniMaxCtas, std::max<uint64_t> ( 1, ( j->total + 1023 ) / 1024 ) );
        max_ctas = std::max ( max_ctas, m.ctas );
        memcpy ( m.cmap, pin<uint8_t> ( j, kPinCmap ), 256 );
        pin<uint32_t> ( j, kPinScalar )[2] = 0;                     // no key table and no staging wait
        pin<uint32_t> ( j, kPinScalar )[3] = 0;                     // in this pipeline
    }
    MTX_CUDA ( cudaMemcpyAsync ( dd, hd, ( size_t ) n * sizeof ( MiniJob ), cudaMemcpyHostToDevice, st ) );
    MTX_CUDA ( cudaMemsetAsync ( dres, 0, resb, st ) );
    for ( Job * j : js ) MTX_TRY ( record ( j, j->ev0 ) );
    const dim3 grid ( max_ctas, n );
    auto launch = [&] ( void ( *k ) ( const MiniJob * ), const char * name ) -> int {
        k<<<grid, kMiniThreads, 0, st>>> ( dd );
        c->launches++;
        for ( Job * j : js ) j->launches++;
        if ( cudaError_t e = cudaGetLastError () ) return fail ( MOTEX_ECUDA, "launch of %s failed: %s", name, cudaGetErrorString ( e ) );
        return MOTEX_OK;
    };
    MTX_TRY ( launch ( k_mini_clear, "k_mini_clear" ) );
    MTX_TRY ( launch ( k_mini_pack, "k_mini_pack" ) );
    MTX_TRY ( launch ( k_mini_uniq, "k_mini_uniq" ) );
    MTX_TRY ( launch ( k_mini_planes, "k_mini_planes" ) );
    MTX_CUDA ( cudaMemcpyAsync ( hres, dres, resb, cudaMemcpyDeviceToHost, st ) );
    MTX_TRY ( sync ( c ) );
    for ( uint32_t i = 0; i < n; ++i )
        if ( hres[4 * i] ) return fail ( MOTEX_ECUDA, "small-job pipeline: factor table overflow" );

    // the DP of every job with factors
    for ( uint32_t i = 0; i < n; ++i )
    {
        Job * j = js[i];
        const motex_params & P = j->prm;
        const bool ed = P.d == 1;
        const uint32_t U = hres[4 * i + 1];
        j->U = U;
        j->uniq = dptr<uint32_t> ( j, S_UNIQ );
        if ( U == 0 ) continue;
        j->tune = choose_tune ( j, U, ed, false );
        DPTune cached;
        if ( ! getenv ( "MOTEX_DP_W" ) && ! getenv ( "MOTEX_DP_UR" ) && ! getenv ( "MOTEX_DP_SWAR" ) &&
             tune_lookup ( TuneKey { j->B, P.l, P.e, P.d }, &cached ) )
            j->tune = cached;
        const uint32_t groups = ( U + j->tune.NL - 1 ) / j->tune.NL;
        j->ntiles = ( groups + kDPThreads * j->tune.W - 1 ) / ( kDPThreads * j->tune.W );
        DPArgs & da = j->da;
        da = DPArgs {};
        da.text.planes = dptr<uint32_t> ( j, S_PLANES );
        da.text.plane_stride = j->stride;
        da.text.vmask = dptr<uint32_t> ( j, S_VMASK );
        da.text.emask = dptr<uint32_t> ( j, S_EMASK );
        da.text.nblk = j->nblk;
        da.wplanes32 = dptr<uint32_t> ( j, S_WPL32 );
        da.U = U;
        da.l = P.l;
        da.e = P.e;
        da.one = 1u;
        da.two = 2u;
        da.neg1 = ~0u;
        da.chunks = dptr<ChunkInfo> ( j, S_CHUNKS );
        da.u_acc = dptr<uint32_t> ( j, S_UACC );
        da.v_acc = dptr<uint32_t> ( j, S_VACC );
        da.split_flags = dptr<uint8_t> ( j, S_FLAGS );
        for ( auto & ch : j->chunks ) j->exec_cells += ( uint64_t ) U * ( ch.end - ch.warm ) * 32;
        j->dp_pending = true;
    }
    if ( n == 1 ) MTX_TRY ( stage_dp ( js[0] ) );
    else MTX_TRY ( batch_dp ( c, js, dp_ms ) );

    MTX_TRY ( launch ( k_mini_final, "k_mini_final" ) );
    MTX_TRY ( launch ( k_mini_count, "k_mini_count" ) );
    MTX_TRY ( launch ( k_mini_write, "k_mini_write" ) );
    for ( Job * j : js ) MTX_TRY ( record ( j, j->ev1 ) );
    MTX_CUDA ( cudaMemcpyAsync ( hres, dres, resb, cudaMemcpyDeviceToHost, st ) );
    MTX_TRY ( sync ( c ) );
    for ( uint32_t i = 0; i < n; ++i ) js[i]->nrec = hres[4 * i + 2];
    for ( Job * j : js ) MTX_TRY ( fetch_issue ( j ) );
    MTX_TRY ( sync ( c ) );
    return MOTEX_OK;
}

int ensure_pool ( motex_ctx * c, uint32_t n )
{
    while ( c->pool.size () < n )
    {
        std::unique_ptr<Job> j ( new Job () );
        MTX_TRY ( init_job ( c, j.get () ) );
        c->pool.push_back ( std::move ( j ) );
    }
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
         cudaEventCreate ( &c->evb0 ) != cudaSuccess || cudaEventCreate ( &c->evb1 ) != cudaSuccess )
    {
        cudaGetLastError ();
        motex_ctx_destroy ( c );
        return fail ( MOTEX_ECUDA, "stream/event creation failed" );
    }
    int rc = init_job ( c, &c->main );
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
    for ( DevBuf * b : { &c->bjobs, &c->bitems, &c->bcounter, &c->mjobs, &c->mres, &c->mpart } )
        if ( b->p ) cudaFree ( b->p );
    if ( c->bpinned ) cudaFreeHost ( c->bpinned );
    if ( c->mpinned ) cudaFreeHost ( c->mpinned );
    if ( c->evb0 ) cudaEventDestroy ( c->evb0 );
    if ( c->evb1 ) cudaEventDestroy ( c->evb1 );
    cudaStream_t st = c->st;
    delete c;                                        // jobs free their buffers
    if ( st ) cudaStreamDestroy ( st );
    return MOTEX_OK;
}

int motex_gpu_load ( motex_ctx * c, const motex_params * prm, const char * const * seqs, const uint32_t * lens,
                     uint32_t nseq )
{
    if ( ! c ) return fail ( MOTEX_EINVAL, "null context" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    return load_job ( &c->main, prm, seqs, lens, nseq, 0, true );
}

int motex_gpu_execute ( motex_ctx * c )
{
    if ( ! c ) return fail ( MOTEX_EINVAL, "null context" );
    Job * j = &c->main;
    if ( ! j->loaded || j->npat ) return fail ( MOTEX_EINVAL, "no sequences loaded" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    MTX_TRY ( execute_job ( j ) );
    j->executed = true;
    return MOTEX_OK;
}

int motex_gpu_fetch ( motex_ctx * c, motex_result * out )
{
    if ( ! c || ! out ) return fail ( MOTEX_EINVAL, "null argument" );
    if ( ! c->main.executed ) return fail ( MOTEX_EINVAL, "nothing executed" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    return fetch_records ( &c->main, out );
}

int motex_gpu_run ( motex_ctx * c, const motex_params * prm, const char * const * seqs, const uint32_t * lens,
                    uint32_t nseq, motex_result * out )
{
    if ( ! c || ! out ) return fail ( MOTEX_EINVAL, "null argument" );
    memset ( out, 0, sizeof *out );
    MTX_TRY ( motex_gpu_load ( c, prm, seqs, lens, nseq ) );
    Job * j = &c->main;
    if ( mini_eligible ( j ) )
    {
        // small input: the two-kernel pipeline around the DP
        std::vector<Job *> one { j };
        float dp_ms;
        MTX_TRY ( run_mini ( c, one, &dp_ms ) );
        MTX_TRY ( read_times ( j ) );
        j->executed = true;
        drop_graph ( j );                              // a later execute replays the staged pipeline
        return fetch_build ( j, out );
    }
    MTX_TRY ( motex_gpu_execute ( c ) );
    return motex_gpu_fetch ( c, out );
}

int motex_gpu_run_batch ( motex_ctx * c, const motex_job * jobs, uint32_t njobs, motex_result * results )
{
    if ( ! c || ! jobs || ! results ) return fail ( MOTEX_EINVAL, "null argument" );
    for ( uint32_t i = 0; i < njobs; ++i ) memset ( &results[i], 0, sizeof results[i] );
    if ( njobs == 0 ) return MOTEX_OK;
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    MTX_TRY ( ensure_pool ( c, njobs ) );
    std::vector<Job *> all ( njobs ), js, mini;
    std::vector<uint32_t> js_idx, mini_idx;
    for ( uint32_t i = 0; i < njobs; ++i )
    {
        all[i] = c->pool[i].get ();
        all[i]->replaying = false;
        all[i]->batched = true;
        MTX_TRY ( load_job ( all[i], jobs[i].prm, jobs[i].seqs, jobs[i].lens, jobs[i].nseq, 0, true ) );
        if ( mini_eligible ( all[i] ) ) { mini.push_back ( all[i] ); mini_idx.push_back ( i ); }
        else { js.push_back ( all[i] ); js_idx.push_back ( i ); }
    }
    // small jobs: the two-kernel pipeline, one launch per stage for all of them
    if ( ! mini.empty () )
    {
        float mini_dp = 0.f;
        MTX_TRY ( run_mini ( c, mini, &mini_dp ) );
        for ( uint32_t k = 0; k < mini.size (); ++k )
        {
            Job * j = mini[k];
            MTX_TRY ( read_times ( j ) );
            if ( mini.size () > 1 ) j->dp_ms = mini_dp;     // the batch shares its DP launches
            j->executed = true;
            MTX_TRY ( fetch_build ( j, &results[mini_idx[k]] ) );
        }
    }
    if ( js.empty () ) return MOTEX_OK;
    njobs = ( uint32_t ) js.size ();
    for ( Job * j : js ) MTX_TRY ( stage_presence ( j ) );
    MTX_TRY ( sync ( c ) );
    std::vector<char> sorted ( njobs );
    bool any = false;
    for ( uint32_t i = 0; i < njobs; ++i )
    {
        bool need;
        MTX_TRY ( stage_pack ( js[i], &need ) );
        sorted[i] = need;
        any |= need;
    }
    if ( any ) MTX_TRY ( sync ( c ) );
    for ( uint32_t i = 0; i < njobs; ++i ) MTX_TRY ( stage_plan ( js[i], sorted[i] ) );
    float dp_ms = 0.f;
    MTX_TRY ( batch_dp ( c, js, &dp_ms ) );
    any = false;
    for ( Job * j : js )
    {
        bool need;
        MTX_TRY ( stage_finalize ( j, &need ) );
        any |= need;
    }
    if ( any ) MTX_TRY ( sync ( c ) );
    for ( Job * j : js ) MTX_TRY ( stage_compact ( j ) );
    for ( uint32_t i = 0; i < njobs; ++i )
    {
        MTX_TRY ( read_times ( js[i] ) );
        js[i]->dp_ms = dp_ms;                        // the batch shares its DP launches
        js[i]->executed = true;
        MTX_TRY ( fetch_records ( js[i], &results[js_idx[i]] ) );
    }
    return MOTEX_OK;
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
    if ( ! c || ! u || ! v || ! p || ! t || ! prm ) return fail ( MOTEX_EINVAL, "null argument" );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    if ( m < prm->l || n == 0 ) return MOTEX_OK;                  // no factor of p: nothing to add
    const char * seqs[2] = { p, t };
    const uint32_t lens[2] = { m, n };
    Job * j = &c->main;
    MTX_TRY ( load_job ( j, prm, seqs, lens, 2, 1, false ) );
    j->replaying = false;
    MTX_TRY ( run_job ( j ) );
    MTX_TRY ( read_times ( j ) );
    const bool st_mode = prm->nb_gaps > 0;
    const uint32_t G = st_mode ? j->G : 1;
    const size_t cnt = st_mode ? ( size_t ) m * G : j->U;
    const size_t bytes = cnt * 4;
    MTX_TRY ( ensure_pinned ( j, kPinStage + 2 * bytes ) );
    uint32_t * hu = pin<uint32_t> ( j, kPinStage );
    uint32_t * hv = hu + cnt;
    MTX_CUDA ( cudaMemcpyAsync ( hu, dptr<uint32_t> ( j, S_UOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_CUDA ( cudaMemcpyAsync ( hv, dptr<uint32_t> ( j, S_VOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_TRY ( sync ( c ) );
    if ( st_mode )
    {
        // per (position of p, gap choice k): u[k*m + j] (functions.cc:676-684)
        for ( uint32_t q = 0; q < m; ++q )
            for ( uint32_t k = 0; k < G; ++k )
            {
                u[( size_t ) k * m + q] += hu[( size_t ) q * G + k];
                v[( size_t ) k * m + q] += hv[( size_t ) q * G + k];
            }
    }
    else
        // factor w ends at position l-1+w of p
        for ( uint32_t w = 0; w < j->U; ++w )
        {
            u[prm->l - 1 + w] += hu[w];
            v[prm->l - 1 + w] += hv[w];
        }
    j->loaded = false;
    return MOTEX_OK;
}

int motex_gpu_search ( motex_ctx * c, const motex_params * prm, const char * const * words, const uint32_t * wlens,
                       uint32_t nwords, const char * const * seqs, const uint32_t * lens, uint32_t nseq,
                       uint32_t * u, uint32_t * v )
{
    if ( ! c || ! prm ) return fail ( MOTEX_EINVAL, "null argument" );
    if ( nwords && ( ! words || ! wlens || ! u || ! v ) ) return fail ( MOTEX_EINVAL, "null word arrays" );
    if ( nseq && ( ! seqs || ! lens ) ) return fail ( MOTEX_EINVAL, "null sequence arrays" );
    if ( prm->nb_gaps ) return fail ( MOTEX_EUNSUPPORTED, "the word search takes plain motifs only" );
    MTX_TRY ( validate ( prm ) );
    MTX_CUDA ( cudaSetDevice ( c->device ) );
    const uint32_t l = prm->l;
    for ( uint32_t i = 0; i < nwords; ++i ) u[i] = v[i] = 0;
    // patterns: the last l symbols of every word long enough, then the sequences
    std::vector<const char *> all;
    std::vector<uint32_t> alens, which;
    for ( uint32_t i = 0; i < nwords; ++i )
    {
        if ( wlens[i] < l ) continue;
        if ( ! words[i] ) return fail ( MOTEX_EINVAL, "null word %u", i );
        all.push_back ( words[i] + wlens[i] - l );
        alens.push_back ( l );
        which.push_back ( i );
    }
    const uint32_t npat = ( uint32_t ) which.size ();
    bool searched = false;
    for ( uint32_t s = 0; s < nseq; ++s )
    {
        all.push_back ( seqs[s] );
        alens.push_back ( lens[s] );
        searched |= lens[s] >= l;
    }
    if ( npat == 0 || ! searched ) return MOTEX_OK;
    Job * j = &c->main;
    MTX_TRY ( load_job ( j, prm, all.data (), alens.data (), ( uint32_t ) all.size (), npat, true ) );
    j->replaying = false;
    MTX_TRY ( run_job ( j ) );
    MTX_TRY ( read_times ( j ) );
    if ( j->U != npat ) return fail ( MOTEX_ECUDA, "word search planned %u factors for %u words", j->U, npat );
    const size_t bytes = ( size_t ) npat * 4;
    MTX_TRY ( ensure_pinned ( j, kPinStage + 2 * bytes ) );
    uint32_t * hu = pin<uint32_t> ( j, kPinStage );
    uint32_t * hv = hu + npat;
    MTX_CUDA ( cudaMemcpyAsync ( hu, dptr<uint32_t> ( j, S_UOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_CUDA ( cudaMemcpyAsync ( hv, dptr<uint32_t> ( j, S_VOUT ), bytes, cudaMemcpyDeviceToHost, c->st ) );
    MTX_TRY ( sync ( c ) );
    for ( uint32_t w = 0; w < npat; ++w )
    {
        u[which[w]] = hu[w];
        v[which[w]] = hv[w];
    }
    j->loaded = false;
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

int motex_tune_lookup ( int B, uint32_t l, uint32_t e, uint32_t d, int * W, int * NL, int * UR )
{
    if ( ! W || ! NL || ! UR ) return fail ( MOTEX_EINVAL, "null output pointer" );
    DPTune t;
    if ( ! tune_lookup ( TuneKey { B, l, e, d }, &t ) )
        return fail ( MOTEX_ENOTFOUND, "no launch shape tuned for B=%d l=%u e=%u d=%u", B, l, e, d );
    *W = t.W;
    *NL = t.F ? -t.NL : t.NL;                   // negative: guarded lanes, lowest-bit clears
    *UR = t.UR;
    return MOTEX_OK;
}

} // extern "C"
