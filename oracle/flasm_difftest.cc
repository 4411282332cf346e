/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Differential harness: the restated flasm_hd / flasm_ed (flasm_port.cc,
 * compiled here under the namespace libflasm_port) against the libflasm.so
 * shipped in the reference's libFLASM.zip, on seeded random cases.  Every
 * returned (pos_t, pos_x, error) multiset must be identical.  Runs only on
 * x86-64, the one architecture the shipped .so is built for.
 *
 * usage: flasm_difftest <cases> <seed> [edge]
 * (edge: texts shorter than the factor, or error bound >= factor
 * length -- regimes MoTeX itself never produces for the plain search)
 * prints "OK cases=<n> hits=<total>" and exits 0, or prints the first
 * mismatching case and exits 1.
 */
#include "libflasm.h"

#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <vector>
#include <tuple>
#include <algorithm>

namespace libflasm_port
{
    using libflasm::ResultTuple;
    using libflasm::ResultTupleSet;
    ResultTupleSet flasm_hd ( unsigned char *, unsigned int, unsigned char *, unsigned int, unsigned int, unsigned int, bool );
    ResultTupleSet flasm_ed ( unsigned char *, unsigned int, unsigned char *, unsigned int, unsigned int, unsigned int, bool );
}

static uint64_t rng_state;
static uint64_t rnd ( void )
{
    /* splitmix64 */
    uint64_t z = ( rng_state += 0x9E3779B97F4A7C15ull );
    z = ( z ^ ( z >> 30 ) ) * 0xBF58476D1CE4E5B9ull;
    z = ( z ^ ( z >> 27 ) ) * 0x94D049BB133111EBull;
    return z ^ ( z >> 31 );
}
static unsigned rint_in ( unsigned lo, unsigned hi ) { return lo + ( unsigned ) ( rnd () % ( hi - lo + 1 ) ); }

typedef std::vector<std::tuple<unsigned, unsigned, unsigned>> Hits;
static Hits flatten ( const libflasm::ResultTupleSet & s )
{
    Hits h;
    for ( auto & r : s ) h.emplace_back ( r.pos_t, r.pos_x, r.error );
    std::sort ( h.begin (), h.end () );
    return h;
}

int main ( int argc, char ** argv )
{
    unsigned cases = argc > 1 ? ( unsigned ) atoi ( argv[1] ) : 2000;
    rng_state = argc > 2 ? ( uint64_t ) atoll ( argv[2] ) : 1;
    bool edge = argc > 3 && argv[3][0] == 'e';      /* edge regimes outside MoTeX's own calls */
    static const unsigned sigmas[] = { 2, 4, 5, 8, 20, 27 };
    unsigned long total = 0;
    for ( unsigned c = 0; c < cases; ++c )
    {
        unsigned sigma = sigmas[rnd () % 6];
        bool longf = ( c % 10 ) == 9;                 /* every tenth case: factor length > 64 */
        unsigned l = longf ? rint_in ( 65, 90 ) : rint_in ( 1, c % 3 == 0 ? 64 : 24 );
        unsigned n = rint_in ( l, l + ( longf ? 120 : 260 ) );
        unsigned m = rint_in ( l, l + ( longf ? 60 : 200 ) );
        unsigned k = rint_in ( 0, l - 1 );
        if ( ! longf && ( c % 4 ) == 0 ) k = std::min ( k, 3u );
        if ( edge && ( c % 2 ) == 0 ) n = rint_in ( 1, l );          /* text shorter than the factor */
        if ( edge && ( c % 2 ) == 1 ) k = rint_in ( l, l + 3 );      /* error bound >= factor length */
        std::vector<unsigned char> t ( n + 1 ), x ( m + 1 );
        for ( unsigned i = 0; i < n; ++i ) t[i] = ( unsigned char ) ( 'A' + rnd () % sigma );
        for ( unsigned j = 0; j < m; ++j ) x[j] = ( unsigned char ) ( 'A' + rnd () % sigma );
        /* plant mutated copies of factors of x into t so low-error hits occur */
        unsigned plants = rint_in ( 0, 3 );
        for ( unsigned p = 0; p < plants && n >= l && m >= l; ++p )
        {
            unsigned src = rint_in ( 0, m - l ), dst = rint_in ( 0, n - l );
            for ( unsigned q = 0; q < l; ++q ) t[dst + q] = x[src + q];
            unsigned muts = rint_in ( 0, std::min ( l, 4u ) );
            for ( unsigned q = 0; q < muts; ++q ) t[dst + rint_in ( 0, l - 1 )] = ( unsigned char ) ( 'A' + rnd () % sigma );
        }
        bool ed = rnd () & 1;
        Hits a, b;
        if ( ed )
        {
            a = flatten ( libflasm::flasm_ed ( t.data (), n, x.data (), m, l, k, true ) );
            b = flatten ( libflasm_port::flasm_ed ( t.data (), n, x.data (), m, l, k, true ) );
        }
        else
        {
            a = flatten ( libflasm::flasm_hd ( t.data (), n, x.data (), m, l, k, true ) );
            b = flatten ( libflasm_port::flasm_hd ( t.data (), n, x.data (), m, l, k, true ) );
        }
        total += a.size ();
        if ( a != b )
        {
            printf ( "MISMATCH case=%u %s sigma=%u n=%u m=%u l=%u k=%u shipped=%zu port=%zu\n",
                     c, ed ? "ed" : "hd", sigma, n, m, l, k, a.size (), b.size () );
            return 1;
        }
    }
    printf ( "OK cases=%u hits=%lu\n", cases, total );
    return 0;
}
