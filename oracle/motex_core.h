/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * CPU restatement of the two approximate-matching primitives MoTeX drives
 * through libFLASM (functions.cc:538 flasm_hd, functions.cc:746 flasm_ed).
 * libFLASM is shipped with the reference only as a prebuilt x86-64 object,
 * so its behaviour is restated from its observable contract, which the
 * differential harness flasm_difftest.cc checks against the shipped library:
 *
 *   hd_scan(t,n,x,m,l,k): every (i,j) with l-1 <= i < n, l-1 <= j < m and
 *       err = Hamming(t[i-l+1..i], x[j-l+1..j]) <= k.
 *   ed_scan(t,n,x,m,l,k): every (i,j) with 0 <= i < n, l-1 <= j < m and
 *       err = min_s EditDistance(x[j-l+1..j], t[s..i]) <= k
 *       (semi-global: free start s in t, end fixed at i, empty t-factor
 *       allowed).
 *
 * Each pair (i,j) is reported at most once through hit(i, j, err).
 *
 * Hamming: one pass per diagonal i-j with a rolling mismatch count, O(1)
 * per cell for any l.  Edit distance: Myers/Hyyro bit-vector column
 * recurrence for l <= 64 (one 64-bit word per factor), plain Sellers DP
 * column for longer factors.
 */
#ifndef MOTEX_ORACLE_CORE_H
#define MOTEX_ORACLE_CORE_H

#include <stdint.h>
#include <string.h>
#include <vector>
#include <algorithm>

namespace motex_oracle
{

template <class F>
static void hd_scan ( const unsigned char * t, unsigned n, const unsigned char * x, unsigned m,
                      unsigned l, unsigned k, F && hit )
{
    if ( l == 0 || n < l || m < l ) return;
    for ( long d = - ( long ) ( m - 1 ); d <= ( long ) ( n - 1 ); ++d )
    {
        unsigned j0 = d < 0 ? ( unsigned ) ( -d ) : 0u;
        unsigned i0 = ( unsigned ) ( ( long ) j0 + d );
        unsigned len = std::min ( n - i0, m - j0 );
        unsigned cnt = 0;
        for ( unsigned s = 0; s < len; ++s )
        {
            cnt += t[i0 + s] != x[j0 + s];
            if ( s >= l ) cnt -= t[i0 + s - l] != x[j0 + s - l];
            if ( s + 1 >= l && cnt <= k ) hit ( i0 + s, j0 + s, cnt );
        }
    }
}

/*
 * Myers/Hyyro column recurrence for one factor of length l <= 64.
 * peq[c] = bit p set iff factor[p] == c, indexed by the text symbol.
 * Calls hit(i, D[l][i]) for every end position i with D[l][i] <= k.
 */
template <class F>
static void myers_factor ( const uint64_t * peq, unsigned l, const unsigned char * t, unsigned n,
                           unsigned k, F && hit )
{
    const uint64_t hb = 1ull << ( l - 1 );
    uint64_t Pv = ( l == 64 ) ? ~0ull : ( ( 1ull << l ) - 1 );
    uint64_t Mv = 0;
    unsigned score = l;
    for ( unsigned i = 0; i < n; ++i )
    {
        const uint64_t Eq = peq[t[i]];
        const uint64_t Xv = Eq | Mv;
        const uint64_t Xh = ( ( ( Eq & Pv ) + Pv ) ^ Pv ) | Eq;
        uint64_t Ph = Mv | ~( Xh | Pv );
        uint64_t Mh = Pv & Xh;
        if ( Ph & hb ) score++;
        else if ( Mh & hb ) score--;
        Ph <<= 1;
        Mh <<= 1;
        Pv = Mh | ~( Xv | Ph );
        Mv = Ph & Xv;
        if ( score <= k ) hit ( i, score );
    }
}

/* Plain Sellers DP column for one factor of any length. */
template <class F>
static void sellers_factor ( const unsigned char * w, unsigned l, const unsigned char * t, unsigned n,
                             unsigned k, F && hit )
{
    std::vector<unsigned> col ( l + 1 ), nxt ( l + 1 );
    for ( unsigned p = 0; p <= l; ++p ) col[p] = p;
    for ( unsigned i = 0; i < n; ++i )
    {
        nxt[0] = 0;
        for ( unsigned p = 1; p <= l; ++p )
        {
            unsigned sub = col[p - 1] + ( w[p - 1] != t[i] );
            unsigned del = col[p] + 1;
            unsigned ins = nxt[p - 1] + 1;
            nxt[p] = std::min ( sub, std::min ( del, ins ) );
        }
        col.swap ( nxt );
        if ( col[l] <= k ) hit ( i, col[l] );
    }
}

/* Generic byte-alphabet edit-distance scan (all factors of x over t). */
template <class F>
static void ed_scan ( const unsigned char * t, unsigned n, const unsigned char * x, unsigned m,
                      unsigned l, unsigned k, F && hit )
{
    if ( l == 0 || m < l ) return;
    std::vector<uint64_t> peq ( 256, 0 );
    for ( unsigned j = l - 1; j < m; ++j )
    {
        const unsigned char * w = x + j - l + 1;
        auto on = [&] ( unsigned i, unsigned err ) { hit ( i, j, err ); };
        if ( l <= 64 )
        {
            for ( unsigned p = 0; p < l; ++p ) peq[w[p]] |= 1ull << p;
            myers_factor ( peq.data (), l, t, n, k, on );
            for ( unsigned p = 0; p < l; ++p ) peq[w[p]] = 0;
        }
        else
            sellers_factor ( w, l, t, n, k, on );
    }
}

} // namespace motex_oracle

#endif
