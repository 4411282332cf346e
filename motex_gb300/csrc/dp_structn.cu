// Structured motifs with any number of gaps, block by block.
//
// Reference semantics (functions.cc:564-705 Hamming, 773-915 edit distance;
// the merge loop at functions.cc:647-690 / 858-899): pattern position jx
// (end of box 0 in sequence x) and pattern structure k count one occurrence
// for every text position it (end of box 0 in text t) and text structure l
// such that box 0 matches at (it, jx) with <= e errors and, for every gap g,
// box g+1 of x -- ending at jx + xoff[k][g] -- matches the text box ending
// at it + xoff[l][g] with <= berr[g] errors, every box inside its sequence.
// v[k, jx] counts the (it, l) combinations over all texts, u[k, jx] the
// texts with at least one.
//
// Ownership.  xoff[k][g] (cumulative gap + box lengths) takes the D[g]
// consecutive values lo[g] .. lo[g] + D[g] - 1 over the structures.  A warp
// owns Pw = 33 - max D consecutive pattern positions P0 .. P0+Pw-1; lane r
// runs the box-0 row P0 + r and, for every gap g, the box-(g+1) row
// P0 + lo[g] + r, so the Pw + D[g] - 1 rows box g+1 needs from this warp are
// all in its lanes.  The rows of a lane are packed in one register: SWAR
// lanes with guard bits for edit distance (the single-motif SWAR invariants),
// lanes of Lmax bits with the text window replicated by a multiply for
// Hamming.
//
// Per block of 32 text positions each lane forms the 32-bit hit mask of each
// of its rows (no exchange) and stores them in a per-warp ring in shared
// memory holding the last nslot blocks.  Block E = kb - (nslot - 1) is then
// complete: every box of a chain starting in E ends by block kb.  Only where
// some lane of the warp has a box-0 hit in E does the warp merge: for each
// pattern structure k the lane fits and each text structure l, the chain
// word = box-0 hits AND, per gap, the mask of row r + xoff[k][g] - lo[g]
// shifted by xoff[l][g] (a funnel shift of two ring words) AND the positions
// whose chain of structure l ends before the next sequence end; its popc is
// the number of occurrences.  Sequence ends split a block into segments so
// that u counts texts.
#include "kernels.cuh"

#include <algorithm>
#include <cstdlib>

namespace mtx
{

namespace
{

template <int B, bool ED, int NR, bool SD>
__global__ void __launch_bounds__ ( kDPThreads ) k_dp_structN_blk ( const StructNArgs a, const StructNBlk C )
{
    constexpr int NGAP = NR - 1;
    constexpr int NWARP = kDPThreads / 32;
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t full = 0xffffffffu;
    const uint32_t NS = a.nstructs;
    const uint32_t nslot = C.nslot;
    // dynamic shared memory: structure offsets, per-thread counters, the
    // per-warp mask rings, and (edit distance) the per-thread Eq table
    uint32_t * s_o = smem;                                      // [k * NGAP + g] = xoff[k][g] - lo[g]
    uint32_t * s_t = s_o + NS * NGAP;                           // [l * NGAP + g] = xoff[l][g]
    uint32_t * s_cnt = s_t + NS * NGAP + threadIdx.x;           // [k * kDPThreads]
    uint32_t * s_u = s_cnt + NS * kDPThreads;
    uint32_t * s_v = s_u + NS * kDPThreads;
    uint32_t * ring_all = smem + 2 * NS * NGAP + 3 * NS * kDPThreads;
    uint32_t * ring = ring_all + ( size_t ) warp * nslot * NR * 32;   // [slot][row][lane]
    uint32_t * s_eq = ring_all + ( size_t ) NWARP * nslot * NR * 32;  // [code][thread]
    __shared__ uint32_t s_row[NWARP][2][32];                    // edit distance: Eq-table offsets of a block
    __shared__ uint32_t s_win[NWARP][2][32 * B];                // Hamming: replicated windows of a block, per warp
    __shared__ uint32_t s_fit[NWARP][32];                       // chain-fit masks by last-box offset

    for ( uint32_t i = threadIdx.x; i < NS * NGAP; i += kDPThreads )
    {
        const uint32_t x = a.xoff[i];
        uint32_t lo = 0;
#pragma unroll
        for ( int g = 0; g < NGAP; ++g )
            if ( ( int ) ( i % NGAP ) == g ) lo = C.lo[g];
        s_o[i] = x - lo;
        s_t[i] = x;
    }
    for ( uint32_t k = 0; k < NS; ++k ) s_cnt[k * kDPThreads] = s_u[k * kDPThreads] = s_v[k * kDPThreads] = 0;

    // pattern side
    const uint32_t P0 = ( blockIdx.x * NWARP + warp ) * C.Pw;
    const uint32_t jx = P0 + lane;
    const bool row = lane < ( int ) C.Pw && jx < a.total && a.row_ok[jx];
    uint32_t kvalid = 0;
    if ( row )
    {
        const uint32_t xend = a.row_end[jx];
        for ( uint32_t k = 0; k < NS; ++k )
            if ( jx + a.xoff[k * NGAP + NGAP - 1] < xend ) kvalid |= 1u << k;
    }
    // the lane's rows: box 0 at jx, box g+1 at P0 + lo[g] + lane
    uint32_t w[B];                                              // edit distance: the packed register
    uint32_t fp[B];                                             // Hamming: packed factors
#pragma unroll
    for ( int pl = 0; pl < B; ++pl ) w[pl] = fp[pl] = 0;
#pragma unroll
    for ( int b = 0; b < NR; ++b )
    {
        const uint32_t q = b == 0 ? jx : P0 + C.lo[b > 0 ? b - 1 : 0] + lane;
        const uint32_t Lb = a.blen[b];
#pragma unroll
        for ( int pl = 0; pl < B; ++pl )
        {
            const uint32_t x = q < a.total ? a.wpl[( ( size_t ) b * B + pl ) * a.total + q] : 0u;
            if constexpr ( ED ) w[pl] |= x << C.off[b];
            else fp[pl] |= ( x >> ( 32 - Lb ) ) << ( ( b + 1 ) * C.Lmax - Lb );
        }
    }
    if constexpr ( ED )
    {
        // Myers Eq of the packed register against every symbol code (text
        // bits cleared at the guards, so Eq is 1 there)
        for ( int c = 0; c < ( 1 << B ); ++c )
        {
            uint32_t x = 0;
#pragma unroll
            for ( int pl = 0; pl < B; ++pl ) x |= w[pl] ^ ( ( ( c >> pl ) & 1 ) ? C.NG : 0u );
            s_eq[c * kDPThreads + threadIdx.x] = ~x;
        }
    }
    __syncthreads ();

    const ChunkInfo ch = a.chunks[blockIdx.y];
    int cur_split = ch.first_split;
    const uint32_t * __restrict__ planes = a.text.planes;
    const uint32_t stride = a.text.plane_stride;
    const uint32_t nblk = a.text.nblk;
    const uint32_t look = nslot - 1;
    const uint32_t kend = ch.end + look;                        // blocks past the text hold no hits
    const uint32_t * my_eq = s_eq + threadIdx.x;
    uint32_t Pv = C.NG, Mv = 0, sc = C.SC0 + C.K;                // score + K per field

    auto flush = [&] () {
        for ( uint32_t k = 0; k < NS; ++k )
        {
            const uint32_t c = s_cnt[k * kDPThreads];
            if ( ! c ) continue;
            if ( cur_split < 0 ) s_u[k * kDPThreads] += 1;
            else a.split_flags[( ( size_t ) cur_split * a.total + jx ) * NS + k] = 1;
            s_v[k * kDPThreads] += c;
            s_cnt[k * kDPThreads] = 0;
        }
    };

    // occurrences of the chains starting at the positions `h` of block E
    auto count = [&] ( uint32_t E, uint32_t h ) {
        // cheap exit: none of the box-1 rows this lane's structures reach
        // hits in the blocks where box 1 of a chain starting in E can end
        {
            uint32_t any1 = 0;
            const uint32_t qa = E + ( C.lo[0] >> 5 ), qb = E + ( ( C.lo[0] + C.D[0] + 30 ) >> 5 );
            for ( uint32_t q = qa; q <= qb; ++q )
                for ( uint32_t o = 0; o < C.D[0]; ++o ) any1 |= ring[( ( q % nslot ) * NR + 1 ) * 32 + lane + o];
            if ( ! any1 ) return;
        }
        const uint32_t * fit = s_fit[warp];
        for ( uint32_t kk = kvalid; kk; kk &= kk - 1 )
        {
            const uint32_t k = __ffs ( kk ) - 1;
            uint32_t c = 0;
            for ( uint32_t l = 0; l < NS; ++l )
            {
                uint32_t wv = h & fit[s_t[l * NGAP + NGAP - 1] - C.lo_last];
#pragma unroll
                for ( int g = 0; g < NGAP; ++g )
                {
                    if ( ! wv ) break;
                    const uint32_t t = s_t[l * NGAP + g];
                    const uint32_t rr = lane + s_o[k * NGAP + g];
                    const uint32_t q = E + ( t >> 5 ), sh = t & 31u;
                    uint32_t m = ring[( ( q % nslot ) * NR + g + 1 ) * 32 + rr];
                    if ( sh )
                        m = __funnelshift_r ( m, ring[( ( ( q + 1 ) % nslot ) * NR + g + 1 ) * 32 + rr], sh );
                    wv &= m;
                }
                c += __popc ( wv );
            }
            s_cnt[k * kDPThreads] += c;
        }
    };

    uint32_t par = 0;
    for ( uint32_t kb = ch.warm; kb < kend; ++kb, par ^= 1u )
    {
        uint32_t m[NR];
#pragma unroll
        for ( int b = 0; b < NR; ++b ) m[b] = 0;
        uint32_t vm = 0;
        if ( kb < nblk )                                        // uniform over the CTA
        {
            vm = __ldg ( a.text.vmask + kb );
            const uint32_t em = __ldg ( a.text.emask + kb );
            if constexpr ( ED )
            {
                // each warp computes the Eq-table offsets of the block's
                // positions once (lane r takes position r); double-buffered
                uint32_t * rows = s_row[warp][par];
                {
                    uint32_t c = 0;
#pragma unroll
                    for ( int pl = 0; pl < B; ++pl )
                        c |= ( ( __ldg ( planes + ( size_t ) pl * stride + kb + 1 ) >> lane ) & 1u ) << pl;
                    rows[lane] = c * kDPThreads;
                }
                __syncwarp ();
                // masks built in reverse bit order (position r at bit 31-r); adds
                // and left shifts are multiply-adds, each hit the sign bit of one,
                // appended by a funnel shift
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
                        // ph, mh disjoint with the top bit below 31: one
                        // arithmetic shift of ph - mh updates every field
                        const int32_t d = ( int32_t ) ( mh * C.neg1 + ph );
                        sc = ( uint32_t ) ( d >> C.s ) * C.one + sc;
                    }
                    else
                    {
                        sc = ( ph >> C.s ) * C.one + sc;
                        sc = ( mh >> C.s ) * C.neg1 + sc;
                    }
                    const uint32_t Ph2 = Ph * C.two, Mh2 = Mhs * C.two;
                    Pv = Mh2 | ~( Xv | Ph2 );
                    Mv = Ph2 & Xv & C.NG;
#pragma unroll
                    for ( int b = 0; b < NR; ++b ) m[b] = __funnelshift_l ( sc * C.nm[b] + C.nm[b], m[b], 1 );
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
            }
            else
            {
                // the replicated windows are the same for every thread: each
                // warp builds the block's once into its own double-buffered
                // rows (lane r takes position r) -- a warp barrier, where a
                // CTA-wide buffer made the CTA barrier the top stall
                uint32_t * wsm = s_win[warp][par];
#pragma unroll
                for ( int pl = 0; pl < B; ++pl )
                {
                    const uint32_t pw = __ldg ( planes + ( size_t ) pl * stride + kb );
                    const uint32_t cw = __ldg ( planes + ( size_t ) pl * stride + kb + 1 );
                    wsm[pl * 32 + lane] = ( __funnelshift_rc ( pw, cw, lane + 1 ) >> ( 32 - C.Lmax ) ) * C.rep;
                }
                __syncwarp ();
#pragma unroll 8
                for ( int r = 0; r < 32; ++r )
                {
                    uint32_t x = 0;
#pragma unroll
                    for ( int pl = 0; pl < B; ++pl ) x |= fp[pl] ^ wsm[pl * 32 + r];
#pragma unroll
                    for ( int b = 0; b < NR; ++b )
                        m[b] = __funnelshift_l ( __popc ( x & C.hmask[b] ) * C.one + C.ne[b], m[b], 1 );
                }
            }
#pragma unroll
            for ( int b = 0; b < NR; ++b ) m[b] = __brev ( m[b] );
        }
        m[0] = row ? ( m[0] & vm ) : 0u;                        // box 0 must end a valid match of this warp's row
        uint32_t * rs = ring + ( kb % nslot ) * NR * 32;
#pragma unroll
        for ( int b = 0; b < NR; ++b ) rs[b * 32 + lane] = m[b];
        __syncwarp ();

        // block E is complete: count the chains starting in it
        if ( kb >= look )
        {
            const uint32_t E = kb - look;
            if ( E >= ch.begin && E < ch.end )
            {
                const uint32_t H0 = ring[( E % nslot ) * NR * 32 + lane];
                uint32_t Ebits = __ldg ( a.text.emask + E );
                if ( __any_sync ( full, H0 != 0u ) )
                {
                    // chain-fit masks: a chain of last offset t starting at
                    // position i of E stays in i's sequence when no sequence
                    // ends in [i, i + t - 1]
                    if ( lane < ( int ) C.D[NGAP - 1] )
                    {
                        const uint32_t t = C.lo_last + lane;
                        uint32_t fit = full;
                        for ( uint32_t q = 0; q <= look && E + q < nblk; ++q )
                        {
                            for ( uint32_t eb = __ldg ( a.text.emask + E + q ); eb; eb &= eb - 1 )
                            {
                                const int e = ( int ) ( q * 32 ) + __ffs ( eb ) - 1;     // end, relative to E
                                const int lo_i = max ( 0, e - ( int ) t + 1 ), hi_i = min ( 31, e );
                                if ( lo_i <= hi_i )
                                {
                                    const uint32_t upto = hi_i == 31 ? full : ( ( 2u << hi_i ) - 1u );
                                    fit &= ~( upto & ~( ( 1u << lo_i ) - 1u ) );
                                }
                            }
                        }
                        s_fit[warp][lane] = fit;
                    }
                    __syncwarp ();
                }
                // segments of E between sequence ends
                uint32_t start = 0;
                while ( true )
                {
                    const uint32_t endbit = Ebits ? ( uint32_t ) ( __ffs ( Ebits ) - 1 ) : 31u;
                    const uint32_t seg = ( endbit == 31 ? full : ( ( 2u << endbit ) - 1u ) ) & ~( ( 1u << start ) - 1u );
                    const uint32_t h = H0 & seg;
                    if ( h ) count ( E, h );
                    if ( ! Ebits ) break;
                    flush ();
                    cur_split = -1;
                    Ebits &= Ebits - 1;
                    if ( endbit == 31 ) break;
                    start = endbit + 1;
                }
                __syncwarp ();                                  // s_fit is rewritten by a later block
            }
        }
    }
    // chunk end: the text cut by the boundary records presence in its split row
    for ( uint32_t k = 0; k < NS; ++k )
    {
        const uint32_t c = s_cnt[k * kDPThreads];
        uint32_t u = s_u[k * kDPThreads];
        if ( c )
        {
            if ( ch.last_split >= 0 )
                a.split_flags[( ( size_t ) ch.last_split * a.total + jx ) * NS + k] = 1;
            else
                u += 1;
        }
        const uint32_t v = s_v[k * kDPThreads] + c;
        if ( row && ( u | v ) )
        {
            atomicAdd ( a.u_acc + ( size_t ) jx * NS + k, u );
            atomicAdd ( a.v_acc + ( size_t ) jx * NS + k, v );
        }
    }
}

size_t blk_smem_bytes ( const StructNArgs & a, const StructNBlk & C, int B, bool ed, int NR )
{
    const size_t NS = a.nstructs, NGAP = NR - 1;
    size_t words = 2 * NS * NGAP + 3 * NS * kDPThreads + ( size_t ) ( kDPThreads / 32 ) * C.nslot * NR * 32;
    if ( ed ) words += ( size_t ) ( 1 << B ) * kDPThreads;
    return words * sizeof ( uint32_t );
}

template <int B, bool ED, int NR>
bool launch_blk ( const StructNArgs & a, const StructNBlk & C, dim3 grid, cudaStream_t st )
{
    const size_t smem = blk_smem_bytes ( a, C, B, ED, NR );
    if ( smem > 200 * 1024 ) return false;
    auto kern = ED && C.sd ? k_dp_structN_blk<B, ED, NR, true> : k_dp_structN_blk<B, ED, NR, false>;
    cudaFuncSetAttribute ( kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ( int ) smem );
    kern<<<grid, kDPThreads, smem, st>>> ( a, C );
    return true;
}

template <int B, bool ED>
bool launch_blk_r ( const StructNArgs & a, const StructNBlk & C, dim3 grid, cudaStream_t st )
{
    switch ( a.ngaps + 1 )
    {
        case 2: return launch_blk<B, ED, 2> ( a, C, grid, st );
        case 3: return launch_blk<B, ED, 3> ( a, C, grid, st );
        case 4: return launch_blk<B, ED, 4> ( a, C, grid, st );
        default: return false;
    }
}

} // namespace

bool structN_blk_shape ( const StructNArgs & a, const uint32_t * h_xoff, bool ed, StructNBlk * C )
{
    const uint32_t NG = a.ngaps, NS = a.nstructs, NR = NG + 1;
    if ( NG < 1 || NR > kStructNBlkMaxRows || NS < 1 || NS > 32 ) return false;
    if ( const char * e = getenv ( "MOTEX_STRUCTN_NO_BLOCK" ) )
        if ( atoi ( e ) != 0 ) return false;
    *C = StructNBlk {};
    uint32_t Dmax = 1, tmax = 0;
    for ( uint32_t g = 0; g < NG; ++g )
    {
        uint32_t lo = 0xffffffffu, hi = 0;
        for ( uint32_t k = 0; k < NS; ++k )
        {
            lo = std::min ( lo, h_xoff[k * NG + g] );
            hi = std::max ( hi, h_xoff[k * NG + g] );
        }
        C->lo[g] = lo;
        C->D[g] = hi - lo + 1;
        Dmax = std::max ( Dmax, C->D[g] );
        tmax = std::max ( tmax, hi );
    }
    if ( Dmax > 17 ) return false;                              // at least 16 pattern positions per warp
    C->Pw = 33 - Dmax;
    C->nslot = ( tmax >> 5 ) + 2;
    if ( C->nslot > kStructNBlkMaxSlots ) return false;
    C->lo_last = C->lo[NG - 1];
    C->one = 1u;
    C->two = 2u;
    C->neg1 = ~0u;
    uint32_t L[kStructNBlkMaxRows], E[kStructNBlkMaxRows];
    for ( uint32_t b = 0; b < NR; ++b )
    {
        L[b] = a.blen[b];
        E[b] = a.berr[b];
        if ( L[b] < 1 || L[b] > 32 || E[b] >= L[b] ) return false;
    }
    if ( ed )
    {
        uint32_t o = 0, s = 32;
        for ( uint32_t b = 0; b < NR; ++b )
        {
            C->off[b] = o;
            s = std::min ( s, L[b] - 1 );
            o += L[b] + 1;
        }
        if ( C->off[NR - 1] + L[NR - 1] > 32 || s < 1 || s > 30 ) return false;
        uint32_t guards = 0;
        for ( uint32_t b = 0; b < NR; ++b )
        {
            if ( E[b] + 1 > ( 1u << s ) || L[b] - E[b] - 1 >= ( 1u << s ) ) return false;
            const uint32_t hb = C->off[b] + L[b] - 1, f = hb - s;
            C->HB |= 1u << hb;
            if ( C->off[b] + L[b] < 32 ) guards |= 1u << ( C->off[b] + L[b] );
            C->K += ( ( 1u << s ) - ( E[b] + 1 ) ) << f;
            C->SC0 += L[b] << f;
            C->nm[b] = 0u - ( 1u << ( 31 - hb ) );
        }
        C->NG = ~guards;
        C->NGm1 = C->NG & ~C->HB;
        C->s = s;
        C->sd = C->off[NR - 1] + L[NR - 1] - 1 <= 30;
    }
    else
    {
        uint32_t Lmax = 0;
        for ( uint32_t b = 0; b < NR; ++b ) Lmax = std::max ( Lmax, L[b] );
        if ( NR * Lmax > 32 ) return false;
        C->Lmax = Lmax;
        for ( uint32_t b = 0; b < NR; ++b )
        {
            C->rep |= 1u << ( b * Lmax );
            C->hmask[b] = ( ( 1u << L[b] ) - 1u ) << ( ( b + 1 ) * Lmax - L[b] );
            C->ne[b] = ~E[b];
        }
    }
    return true;
}

bool launch_dp_structN_blk ( const StructNArgs & a, const StructNBlk & C, int B, bool ed, dim3 grid, cudaStream_t st )
{
    switch ( B )
    {
        case 1:
        case 2: return ed ? launch_blk_r<2, true> ( a, C, grid, st ) : launch_blk_r<2, false> ( a, C, grid, st );
        case 3: return ed ? launch_blk_r<3, true> ( a, C, grid, st ) : launch_blk_r<3, false> ( a, C, grid, st );
        case 4: return ed ? launch_blk_r<4, true> ( a, C, grid, st ) : launch_blk_r<4, false> ( a, C, grid, st );
        case 5: return ed ? launch_blk_r<5, true> ( a, C, grid, st ) : launch_blk_r<5, false> ( a, C, grid, st );
        default: return false;
    }
}

} // namespace mtx
