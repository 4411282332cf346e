/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * motex_port: CPU restatement of the reference MoTeX word-based extraction
 * path, self-contained so it builds and runs on any host (the reference's
 * own build needs an x86-64-only libflasm.so).  It is the checker for the
 * GPU path and the CPU baseline that is timed beside it.  It follows:
 *
 *   CLI / defaults          functions.cc:2835-3043 (decode_switches)
 *   argument validation     motex.cc:98-201
 *   FASTA reader + split    motex.cc:225-300, 409-437
 *   boxes file              motex.cc:302-363
 *   gap cartesian product   motex.cc:439-486, functions.cc:710-729 (recurse)
 *   all-pairs driver        motex.cc:494-583 (OpenMP over i, as motexOMP)
 *   plain extraction        functions.cc:526-559 (HD), 734-768 (ED)
 *   structured extraction   functions.cc:564-705 (HD), 773-915 (ED)
 *   header                  functions.cc:1010-1068
 *   writers                 functions.cc:1073-1142, 1147-1260
 *   SMILE-like file (-S)    functions.cc:1262-1345, 1368-1461, 1463-1591
 *
 * The DP primitives are motex_core.h (restated libFLASM semantics, pinned
 * against the shipped library by flasm_difftest.cc).  The background and
 * unmatched-motif modes follow the reference built without MPFR (binomial.cc
 * long double flavour), which is what oracle/build_ref.sh compiles:
 *   -b -u [-S -U]           functions.cc:1613-2238 (-o/-u), 2241-2748 (SMILE)
 *   -I                      motex.cc:883-1137, functions.cc:2750-2829
 *   binomial tail           binomial.cc:78-103
 *
 * Built twice: as the CLI binary (main) and, with -DMOTEX_PORT_LIB, as a
 * shared library exposing oracle_extract_pair() and oracle_word_uv() for
 * fine-grained tests.
 */
#include "motex_core.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#include <getopt.h>
#include <math.h>
#include <time.h>
#include <sys/time.h>
#include <stdint.h>
#include <string>
#include <vector>
#include <unordered_map>
#include <unordered_set>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace motex_oracle;

static const char * const ALPHA_DNA  = "ACGTN";
static const char * const ALPHA_PROT = "ARNDCQEGHILKMFPSTWYVOUBZJX*";
static const char * const ALPHA_USR  = "0123456789";

struct Params
{
    unsigned l, e, d;
    unsigned nb_gaps, nb_boxes, nb_structs;
    std::vector<unsigned> blens, berrs;
    std::vector<std::vector<unsigned>> S;      /* S[k][g] gap lengths of struct k */
};

/* ---------------------------------------------------------------- extraction */

/* Symbol -> dense code, so the edit-distance tables stay small. */
struct Coded
{
    std::vector<std::vector<unsigned char>> seq;
    unsigned sigma;
};

static Coded encode ( const std::vector<std::string> & seqs )
{
    Coded c;
    int map[256];
    for ( int i = 0; i < 256; ++i ) map[i] = -1;
    unsigned sigma = 0;
    c.seq.resize ( seqs.size () );
    for ( size_t i = 0; i < seqs.size (); ++i )
    {
        c.seq[i].resize ( seqs[i].size () );
        for ( size_t p = 0; p < seqs[i].size (); ++p )
        {
            unsigned char ch = ( unsigned char ) seqs[i][p];
            if ( map[ch] < 0 ) map[ch] = ( int ) sigma++;
            c.seq[i][p] = ( unsigned char ) map[ch];
        }
    }
    c.sigma = sigma ? sigma : 1;
    return c;
}

/* Per-pattern-sequence Myers tables: factor j (end position) -> peq[sigma]. */
static void build_peq ( const std::vector<unsigned char> & x, unsigned l, unsigned sigma,
                        std::vector<uint64_t> & peq )
{
    unsigned m = ( unsigned ) x.size ();
    peq.assign ( ( size_t ) m * sigma, 0 );
    if ( l > 64 || m < l ) return;
    for ( unsigned j = l - 1; j < m; ++j )
    {
        uint64_t * P = &peq[( size_t ) j * sigma];
        for ( unsigned p = 0; p < l; ++p ) P[x[j - l + 1 + p]] |= 1ull << p;
    }
}

/* Hits of all factors (length ell, error <= err) of x inside t, as
 * hit(pos_t, pos_x, error) -- the flasm_hd / flasm_ed contract. */
template <class F>
static void flasm_like ( unsigned d, const std::vector<unsigned char> & t, const std::vector<unsigned char> & x,
                         const std::vector<uint64_t> * peq, unsigned sigma,
                         unsigned ell, unsigned err, F && hit )
{
    unsigned n = ( unsigned ) t.size (), m = ( unsigned ) x.size ();
    if ( d == 0 ) { hd_scan ( t.data (), n, x.data (), m, ell, err, hit ); return; }
    if ( ell == 0 || m < ell ) return;
    if ( ell <= 64 && peq )
    {
        for ( unsigned j = ell - 1; j < m; ++j )
            myers_factor ( &( *peq )[( size_t ) j * sigma], ell, t.data (), n, err,
                           [&] ( unsigned i, unsigned e ) { hit ( i, j, e ); } );
    }
    else
        ed_scan ( t.data (), n, x.data (), m, ell, err, hit );
}

/* functions.cc:526-559 / 734-768: u[pos_x] += 1 once per pair, v[pos_x] += hits */
static void extract_plain ( const Params & P, const std::vector<unsigned char> & x, const std::vector<unsigned char> & t,
                            const std::vector<uint64_t> * peq, unsigned sigma,
                            unsigned * u, unsigned * v, std::vector<unsigned char> & occ )
{
    occ.assign ( x.size (), 0 );
    flasm_like ( P.d, t, x, peq, sigma, P.l, P.e, [&] ( unsigned, unsigned j, unsigned err ) {
        if ( err <= P.e )
        {
            if ( ! occ[j] ) { u[j]++; occ[j] = 1; }
            v[j]++;
        }
    } );
}

/* functions.cc:564-705 / 773-915: per-box error matrices B[b][pos_t+1][pos_x+1]
 * (initialised to m), merged over every (struct k of x, struct l of t). */
static void extract_structured ( const Params & P, const std::vector<unsigned char> & x, const std::vector<unsigned char> & t,
                                 const std::vector<std::vector<uint64_t>> * peqs, unsigned sigma,
                                 unsigned * u, unsigned * v,
                                 std::vector<std::vector<unsigned>> & B, std::vector<unsigned char> & occ )
{
    const unsigned m = ( unsigned ) x.size (), n = ( unsigned ) t.size ();
    const size_t W = ( size_t ) m + 1;
    B.resize ( P.nb_boxes );
    for ( unsigned b = 0; b < P.nb_boxes; ++b )
    {
        B[b].assign ( ( size_t ) ( n + 1 ) * W, m );
        unsigned ell = b ? P.blens[b - 1] : P.l;
        unsigned err = b ? P.berrs[b - 1] : P.e;
        flasm_like ( P.d, t, x, peqs ? &( *peqs )[b] : nullptr, sigma, ell, err,
                     [&] ( unsigned i, unsigned j, unsigned e ) { B[b][( size_t ) ( i + 1 ) * W + j + 1] = e; } );
    }
    occ.assign ( ( size_t ) P.nb_structs * W, 0 );
    for ( unsigned i = 0; i < n + 1; ++i )
        for ( unsigned j = 0; j < m + 1; ++j )
        {
            if ( B[0][( size_t ) i * W + j] > P.e ) continue;
            for ( unsigned k = 0; k < P.nb_structs; ++k )
                for ( unsigned l = 0; l < P.nb_structs; ++l )
                {
                    unsigned oj = j, oi = i, r = 1;
                    for ( unsigned g = 0; g < P.nb_gaps; ++g )
                    {
                        oj += P.S[k][g] + P.blens[g];
                        oi += P.S[l][g] + P.blens[g];
                        if ( oi < n + 1 && oj < m + 1 )
                        {
                            if ( B[g + 1][( size_t ) oi * W + oj] <= P.berrs[g] )
                            {
                                r++;
                                if ( r == P.nb_boxes )
                                {
                                    size_t idx = ( size_t ) k * m + j - 1;
                                    if ( ! occ[( size_t ) k * W + j - 1] ) { u[idx]++; occ[( size_t ) k * W + j - 1] = 1; }
                                    v[idx]++;
                                }
                            }
                            else
                                break;
                        }
                    }
                }
        }
}

/* motex.cc:494-583 */
static void all_pairs ( const Params & P, const Coded & C, unsigned total_mot_length,
                        std::vector<std::vector<unsigned>> & U, std::vector<std::vector<unsigned>> & V,
                        const char * input_filename )
{
    const unsigned num = ( unsigned ) C.seq.size ();
    U.assign ( num, {} );
    V.assign ( num, {} );
    #pragma omp parallel for schedule(dynamic, 1)
    for ( unsigned i = 0; i < num; ++i )
    {
        const std::vector<unsigned char> & x = C.seq[i];
        const unsigned m = ( unsigned ) x.size ();
        U[i].assign ( ( size_t ) m * P.nb_structs, 0 );
        V[i].assign ( ( size_t ) m * P.nb_structs, 0 );
        std::vector<std::vector<uint64_t>> peqs ( P.nb_boxes );
        if ( P.d == 1 )
            for ( unsigned b = 0; b < P.nb_boxes; ++b )
                build_peq ( x, b ? P.blens[b - 1] : P.l, C.sigma, peqs[b] );
        std::vector<std::vector<unsigned>> B;
        std::vector<unsigned char> occ;
        for ( unsigned j = 0; j < num; ++j )
        {
            const std::vector<unsigned char> & t = C.seq[j];
            const unsigned n = ( unsigned ) t.size ();
            if ( total_mot_length > n || total_mot_length > m )
            {
                fprintf ( stderr, " Omitting short sequence in file %s!\n", input_filename );
                continue;
            }
            if ( P.nb_gaps == 0 )
                extract_plain ( P, x, t, P.d == 1 ? &peqs[0] : nullptr, C.sigma, U[i].data (), V[i].data (), occ );
            else
                extract_structured ( P, x, t, P.d == 1 ? &peqs : nullptr, C.sigma, U[i].data (), V[i].data (), B, occ );
        }
    }
}

/* ---------------------------------------------------------------- library API */

extern "C" int oracle_extract_pair ( int d, unsigned l, unsigned e, const char * p, unsigned m,
                                     const char * t, unsigned n, unsigned * u, unsigned * v )
{
    std::vector<std::string> s { std::string ( p, m ), std::string ( t, n ) };
    Coded C = encode ( s );
    Params P;
    P.l = l; P.e = e; P.d = ( unsigned ) d;
    P.nb_gaps = 0; P.nb_boxes = 1; P.nb_structs = 1;
    std::vector<uint64_t> peq;
    if ( d == 1 ) build_peq ( C.seq[0], l, C.sigma, peq );
    std::vector<unsigned char> occ;
    extract_plain ( P, C.seq[0], C.seq[1], d == 1 ? &peq : nullptr, C.sigma, u, v, occ );
    return 1;
}

/* structured_motifs_extraction_hd/_ed for one pair (functions.cc:564-705,
 * 773-915): u, v hold m * nb_structs entries, [k * m + j], accumulated. */
extern "C" int oracle_extract_pair_struct ( int d, unsigned l, unsigned e, unsigned nb_gaps, const unsigned * gmin,
                                            const unsigned * gmax, const unsigned * blens, const unsigned * berrs,
                                            const char * p, unsigned m, const char * t, unsigned n,
                                            unsigned * u, unsigned * v )
{
    std::vector<std::string> s { std::string ( p, m ), std::string ( t, n ) };
    Coded C = encode ( s );
    Params P;
    P.l = l; P.e = e; P.d = ( unsigned ) d;
    P.nb_gaps = nb_gaps;
    P.nb_boxes = nb_gaps + 1;
    P.blens.assign ( blens, blens + nb_gaps );
    P.berrs.assign ( berrs, berrs + nb_gaps );
    P.nb_structs = 1;
    for ( unsigned g = 0; g < nb_gaps; ++g ) P.nb_structs *= gmax[g] - gmin[g] + 1;
    P.S.assign ( P.nb_structs, std::vector<unsigned> ( nb_gaps ) );
    for ( unsigned k = 0; k < P.nb_structs; ++k )
    {
        unsigned rem = k;
        for ( int g = ( int ) nb_gaps - 1; g >= 0; --g )
        {
            unsigned span = gmax[g] - gmin[g] + 1;
            P.S[k][g] = gmin[g] + rem % span;
            rem /= span;
        }
    }
    std::vector<std::vector<uint64_t>> peqs ( P.nb_boxes );
    if ( d == 1 )
        for ( unsigned b = 0; b < P.nb_boxes; ++b ) build_peq ( C.seq[0], b ? P.blens[b - 1] : l, C.sigma, peqs[b] );
    std::vector<std::vector<unsigned>> B;
    std::vector<unsigned char> occ;
    extract_structured ( P, C.seq[0], C.seq[1], d == 1 ? &peqs : nullptr, C.sigma, u, v, B, occ );
    return 1;
}

/* u, v of one word over all searched sequences (length >= tml) of a set:
 * the per-word totals the all-pairs driver accumulates (motex.cc:531-581). */
extern "C" int oracle_word_uv ( int d, unsigned l, unsigned e, const char * word, const char * text,
                                const unsigned * offs, unsigned nseq, unsigned tml, unsigned * u, unsigned * v )
{
    *u = *v = 0;
    for ( unsigned s = 0; s < nseq; ++s )
    {
        const unsigned n = offs[s + 1] - offs[s];
        if ( n < tml ) continue;
        const unsigned char * t = ( const unsigned char * ) text + offs[s];
        unsigned hits = 0;
        auto on = [&] ( unsigned, unsigned, unsigned ) { hits++; };
        if ( d == 0 ) hd_scan ( t, n, ( const unsigned char * ) word, l, l, e, on );
        else ed_scan ( t, n, ( const unsigned char * ) word, l, l, e, on );
        *u += hits > 0;
        *v += hits;
    }
    return 1;
}

#ifndef MOTEX_PORT_LIB

/* ---------------------------------------------------------------- CLI */

struct Switch
{
    char * alphabet = nullptr, * input_filename = nullptr, * output_filename = nullptr;
    char * background_in_filename = nullptr, * un_in_filename = nullptr, * un_out_filename = nullptr;
    char * boxes_in_filename = nullptr, * smile_out_filename = nullptr, * un_smile_out_filename = nullptr;
    unsigned q = 0, Q = 100, l = 0, d = 0, e = 0, n = 1, N = 10000, t = 4;
};

static struct option long_options[] =
{
    { "alphabet", required_argument, NULL, 'a' },
    { "background-in-file", required_argument, NULL, 'b' },
    { "input-file", required_argument, NULL, 'i' },
    { "output-file", required_argument, NULL, 'o' },
    { "quorum", required_argument, NULL, 'q' },
    { "max-quorum", required_argument, NULL, 'Q' },
    { "motifs-length", required_argument, NULL, 'k' },
    { "distance", required_argument, NULL, 'd' },
    { "errors", required_argument, NULL, 'e' },
    { "num-of-occ", required_argument, NULL, 'n' },
    { "max-num-of-occ", required_argument, NULL, 'N' },
    { "num-of-threads", required_argument, NULL, 't' },
    { "boxes-in-file", required_argument, NULL, 's' },
    { "unmatched-in-file", required_argument, NULL, 'I' },
    { "unmatched-out-file", required_argument, NULL, 'u' },
    { "SMILE-out-file", required_argument, NULL, 'S' },
    { "unmatched-SMILE-out-file", required_argument, NULL, 'U' },
    { "help", no_argument, NULL, 'h' },
    { NULL, 0, NULL, 0 }
};

static void usage ( void )
{
    fprintf ( stdout, " Usage: motex_port <options>  (oracle restatement of motexCPU/motexOMP)\n"
                      "  -a <DNA|PROT|USR> -i <fasta> -o <out> -d <0|1> -k <int> -e <int> -q <int>\n"
                      "  [-Q <int>] [-n <int>] [-N <int>] [-s <boxes>] [-t <threads>]\n" );
}

/* functions.cc:2862-3043: returns optind, or 0 on a bad numeric argument / -h */
static int decode_switches ( int argc, char ** argv, Switch * sw )
{
    int oi, opt, args = 0;
    double val;
    char * ep;
    while ( ( opt = getopt_long ( argc, argv, "a:b:i:o:q:Q:k:d:e:n:N:s:t:I:S:u:U:h", long_options, &oi ) ) != -1 )
    {
        switch ( opt )
        {
            case 'a': sw->alphabet = strdup ( optarg ); args++; break;
            case 'i': sw->input_filename = strdup ( optarg ); args++; break;
            case 'o': sw->output_filename = strdup ( optarg ); args++; break;
            case 'b': sw->background_in_filename = strdup ( optarg ); break;
            case 'I': sw->un_in_filename = strdup ( optarg ); break;
            case 'u': sw->un_out_filename = strdup ( optarg ); break;
            case 'S': sw->smile_out_filename = strdup ( optarg ); break;
            case 'U': sw->un_smile_out_filename = strdup ( optarg ); break;
            case 's': sw->boxes_in_filename = strdup ( optarg ); break;
            case 'q': val = strtol ( optarg, &ep, 10 ); if ( optarg == ep ) return 0; sw->q = ( unsigned ) val; args++; break;
            case 'Q': val = strtol ( optarg, &ep, 10 ); if ( optarg == ep ) return 0; sw->Q = ( unsigned ) val; break;
            case 'k': val = strtol ( optarg, &ep, 10 ); if ( optarg == ep ) return 0; sw->l = ( unsigned ) val; args++; break;
            case 'n': val = strtol ( optarg, &ep, 10 ); if ( optarg == ep ) return 0; sw->n = ( unsigned ) val; break;
            case 'N': val = strtol ( optarg, &ep, 10 ); if ( optarg == ep ) return 0; sw->N = ( unsigned ) val; break;
            case 'd': val = strtol ( optarg, &ep, 10 ); if ( ! ep || ep == optarg ) return 0; sw->d = ( unsigned ) val; args++; break;
            case 't': val = strtol ( optarg, &ep, 10 ); if ( ! ep || ep == optarg ) return 0; sw->t = ( unsigned ) val; break;
            case 'e': val = strtol ( optarg, &ep, 10 ); if ( optarg == ep ) return 0; sw->e = ( unsigned ) val; args++; break;
            case 'h': return 0;
        }
    }
    if ( args < 7 ) { usage (); exit ( 1 ); }
    return optind;
}

static double gettime ( void )
{
    struct timeval tv;
    gettimeofday ( &tv, 0 );
    return tv.tv_sec + tv.tv_usec * 0.000001;
}

/* functions.cc:1010-1068 */
static void write_header ( FILE * out, const Switch & sw, const Params & P, const std::vector<unsigned> & gmin,
                           const std::vector<unsigned> & gmax, unsigned num_seqs, double exectime, int procs )
{
    time_t tt;
    time ( &tt );
    fprintf ( out, "####################################\n" );
    fprintf ( out, "# Program: MoTeX\n" );
    fprintf ( out, "# Rundate: %s", ctime ( &tt ) );
    fprintf ( out, "# Input file: %s\n", sw.input_filename );
    fprintf ( out, "# Output file: %s\n", sw.output_filename );
    fprintf ( out, "# For %d input sequences\n", num_seqs );
    fprintf ( out, "#     d = %d\n", sw.d );
    fprintf ( out, "#     q = %d\n", sw.q );
    if ( sw.Q != 100 ) fprintf ( out, "#     Q = %d\n", sw.Q );
    if ( sw.n != 1 ) fprintf ( out, "#     n = %d\n", sw.n );
    if ( sw.N != 10000 ) fprintf ( out, "#     N = %d\n", sw.N );
    if ( P.nb_boxes == 1 )
    {
        fprintf ( out, "#     l = %d\n", sw.l );
        fprintf ( out, "#     e = %d\n", sw.e );
    }
    else
    {
        fprintf ( out, "# Number of boxes: %d\n", P.nb_boxes );
        fprintf ( out, "#     l0 = %d\n", sw.l );
        fprintf ( out, "#     e0 = %d\n", sw.e );
        for ( unsigned i = 0; i < P.nb_gaps; ++i )
        {
            fprintf ( out, "#     g%d = [%d,%d]\n", i + 1, gmin[i], gmax[i] );
            fprintf ( out, "#     l%d = %d\n", i + 1, P.blens[i] );
            fprintf ( out, "#     e%d = %d\n", i + 1, P.berrs[i] );
        }
        fprintf ( out, "# Boxes input file: %s\n", sw.boxes_in_filename );
    }
    fprintf ( out, "# Run on %d proc(s) in %lf secs\n", procs, exectime );
    fprintf ( out, "####################################\n\n" );
}

static bool passes ( const Switch & sw, unsigned u, unsigned v, unsigned num_seqs )
{
    /* functions.cc:1107-1108, the same double expression */
    double r = ( ( double ) u / num_seqs ) * 100;
    return r >= sw.q && v >= sw.n && r <= sw.Q && v <= sw.N;
}

struct Printed
{
    std::string key;
    unsigned u, v;
};

/* functions.cc:1262-1345: the SMILE-like header */
static void write_smile_header ( FILE * out, const Switch & sw, const Params & P, const std::vector<unsigned> & gmin,
                                 const std::vector<unsigned> & gmax, unsigned num_seqs, unsigned total_length,
                                 const char * alphabet )
{
    char head[1024];
    int at;
    int abs_q = ( int ) ceil ( ( double ) ( ( double ) sw.q * num_seqs ) / ( double ) 100 );
    if ( P.nb_boxes == 1 )
        at = snprintf ( head, sizeof head, "%%%%%% 1 %d/%d %d %d %d %d alphabet %s$", abs_q, num_seqs, total_length,
                        sw.l, sw.l, sw.e, alphabet );
    else
    {
        unsigned tot = sw.l, errs = sw.e;
        for ( unsigned b = 0; b < P.nb_gaps; ++b ) { tot += P.blens[b]; errs += P.berrs[b]; }
        at = snprintf ( head, sizeof head, "%%%%%% %d %d/%d %d %d %d %d %d %d %d ", P.nb_boxes, abs_q, num_seqs,
                        total_length, tot, tot, errs, sw.l, sw.l, sw.e );
        for ( unsigned b = 0; b < P.nb_gaps; ++b )
            at += snprintf ( head + at, sizeof head - at, "%d %d %d %d %d ", gmin[b], gmax[b], P.blens[b], P.blens[b], P.berrs[b] );
        at += snprintf ( head + at, sizeof head - at, "alphabet %s$", alphabet );
    }
    fprintf ( out, "%s", head );
    int width = 0, blank_lines = 0;
    if ( ! strcmp ( sw.alphabet, "DNA" ) ) { width = 79; blank_lines = 2; }
    if ( ! strcmp ( sw.alphabet, "PROT" ) ) { width = 159; blank_lines = 1; }
    if ( width )
    {
        for ( int i = at; i < width; ++i ) fputc ( ' ', out );
        fputc ( '\n', out );
        for ( int b = 0; b < blank_lines; ++b ) fprintf ( out, "%79s\n", "" );
    }
    for ( int i = 0; i < 79; ++i ) fputc ( '=', out );
    fputc ( '\n', out );
}

/* functions.cc:1368-1461, 1463-1591: "key id u<TAB>v", id = '0' + rank of
   each symbol in the alphabet string ('-' for a separator) */
static std::string smile_line ( const Params & P, const char * alphabet, const Printed & p )
{
    const unsigned na = ( unsigned ) strlen ( alphabet );
    std::string id;
    for ( char c : p.key )
    {
        unsigned r = 0;
        while ( r < na && alphabet[r] != c ) ++r;
        id.push_back ( r < na ? ( char ) ( '0' + r ) : ( P.nb_gaps ? '-' : ( char ) ( '0' + r ) ) );
    }
    char tail[64];
    snprintf ( tail, sizeof tail, " %d\t%d\n", p.u, p.v );
    return std::string ( p.key.c_str () ) + " " + id + tail;
}

static void write_smile_lines ( FILE * out, const Params & P, const char * alphabet, const std::vector<Printed> & printed )
{
    for ( const Printed & p : printed ) fputs ( smile_line ( P, alphabet, p ).c_str (), out );
}

/* binomial.cc:78-103, the long double flavour (built without MPFR):
   a[i] = i!, and P(X < x) for X ~ Bin(N, p), 0 when p >= 1 */
static std::vector<long double> fact_table ( int n )
{
    std::vector<long double> a ( ( size_t ) n + 1 );
    a[0] = 1;
    for ( int i = 1; i <= n; ++i ) a[i] = a[i - 1] * i;
    return a;
}

static long double binomial_cdf_below ( int x, int N, long double p, const long double * LUT )
{
    long double prob = 0., pr = 0.;
    if ( p >= 1.0 ) return 0.;
    for ( int i = 0; i < x; ++i )
    {
        pr = ( LUT[N] / LUT[i] ) / LUT[N - i] * powl ( p, ( long double ) i ) * powl ( 1. - p, ( long double ) ( N - i ) );
        prob += pr;
        if ( x > N ) break;
    }
    return prob;
}

/* The header lines the background reader takes (functions.cc:1683-1712):
   line 6 "# For N input sequences" and line 8 "#     q = Q"; then one motif
   per line up to the next blank line: key (its first klen symbols), u, n,
   r, v.  A repeated key keeps its last entry. */
struct BgEntry
{
    unsigned u, n, v;
    double r;
};

static bool read_background ( const char * path, unsigned klen, int * bsize, int * bquorum,
                              std::unordered_map<std::string, int> & index, std::vector<BgEntry> & entries )
{
    FILE * in = fopen ( path, "r" );
    if ( ! in ) return false;
    char line[512];
    unsigned line_num = 0;
    std::string size_s, quorum_s;
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' )
    {
        ++line_num;
        if ( line_num == 6 || line_num == 8 )
        {
            char * save = nullptr;
            char * tok = strtok_r ( line, " ", &save );
            tok = tok ? strtok_r ( nullptr, " ", &save ) : nullptr;
            tok = tok ? strtok_r ( nullptr, " ", &save ) : nullptr;
            if ( line_num == 8 ) tok = tok ? strtok_r ( nullptr, "\n", &save ) : nullptr;
            ( line_num == 6 ? size_s : quorum_s ) = tok ? tok : "";
        }
    }
    *bsize = atoi ( size_s.c_str () );
    *bquorum = atoi ( quorum_s.c_str () );
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' )
    {
        char * save = nullptr;
        char * tok = strtok_r ( line, " ", &save );
        const char * f[4] = { nullptr, nullptr, nullptr, nullptr };
        for ( int q = 0; q < 4 && tok; ++q ) f[q] = strtok_r ( nullptr, " ", &save );
        if ( ! tok ) continue;
        std::string key ( tok, strnlen ( tok, klen ) );
        BgEntry b { ( unsigned ) atoi ( f[0] ? f[0] : "0" ), ( unsigned ) atoi ( f[1] ? f[1] : "0" ),
                    ( unsigned ) atoi ( f[3] ? f[3] : "0" ), atof ( f[2] ? f[2] : "0" ) };
        index[key] = ( int ) entries.size ();
        entries.push_back ( b );
    }
    fclose ( in );
    return true;
}

/* functions.cc:1613-1895 (plain) and 1900-2238 (structured), long double
   flavour: every printed motif either matches an unused background entry
   (p-value from binomial_cdf_below(u, num_seqs, that entry's u)) or is
   unmatched (p = Q / N of the background header) and also goes to -u. */
static bool write_background ( const Switch & sw, const Params & P, const std::vector<unsigned> & gmin,
                               const std::vector<unsigned> & gmax, unsigned num_seqs,
                               const std::vector<Printed> & printed, double exectime, int procs )
{
    FILE * out = fopen ( sw.output_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file!\n" ); return true; }
    write_header ( out, sw, P, gmin, gmax, num_seqs, exectime, procs );
    FILE * un = fopen ( sw.un_out_filename, "w" );
    if ( ! un ) { fprintf ( stderr, " Error: cannot open file!\n" ); fclose ( out ); return true; }
    write_header ( un, sw, P, gmin, gmax, num_seqs, exectime, procs );
    unsigned klen = sw.l;
    for ( unsigned b = 0; b < P.nb_gaps; ++b ) klen += P.blens[b] + 1;
    int bsize = 0, bquorum = 0;
    std::unordered_map<std::string, int> index;
    std::vector<BgEntry> bg;
    if ( ! read_background ( sw.background_in_filename, klen, &bsize, &bquorum, index, bg ) )
    {
        fprintf ( stderr, " Error: cannot open file!\n" );
        fclose ( out );
        fclose ( un );
        return true;
    }
    if ( ! ( bsize > 0 && bquorum > 0 ) )
    {
        /* the reference asserts here (functions.cc:1714) and aborts */
        fprintf ( stderr, " Error: background file %s gives no sequence count or no quorum!\n", sw.background_in_filename );
        fclose ( out );
        fclose ( un );
        return false;
    }
    std::vector<long double> LUT = fact_table ( ( int ) num_seqs );
    unsigned pvalid = 0, uvalid = 0;
    for ( const Printed & p : printed )
    {
        const double r = ( double ) p.u / num_seqs;
        auto it = index.find ( p.key );
        if ( it == index.end () || it->second < 0 )
        {
            long double cdf = binomial_cdf_below ( ( int ) p.u, ( int ) num_seqs, ( long double ) bquorum / bsize, LUT.data () );
            fprintf ( out, "%s %d %d %lf %d %d %d %Le\n", p.key.c_str (), p.u, num_seqs, r, p.v, 0, 0, 1. - cdf );
            fprintf ( un, "%s %d %d %lf %d\n", p.key.c_str (), p.u, num_seqs, r, p.v );
            uvalid++;
        }
        else
        {
            const BgEntry & b = bg[it->second];
            long double cdf = binomial_cdf_below ( ( int ) p.u, ( int ) num_seqs, ( long double ) b.u, LUT.data () );
            fprintf ( out, "%s %d %d %lf %d %lf %d %Le\n", p.key.c_str (), p.u, num_seqs, r, p.v, b.r, b.v, 1. - cdf );
            pvalid++;
        }
        index[p.key] = -1;
    }
    fprintf ( out, "\n#A total of %d background motifs were read.\n", ( int ) bg.size () );
    fprintf ( out, "#A total of %d valid motifs were extracted:\n", pvalid + uvalid );
    fprintf ( out, "#  %d of them were matched with background motifs\n", pvalid );
    fprintf ( out, "#  %d of them were not matched with any background motif.\n\n", uvalid );
    fprintf ( un, "\n#A total of %d background motifs were read.\n", ( int ) bg.size () );
    fprintf ( un, "#A total of %d valid motifs were extracted:\n", pvalid + uvalid );
    fprintf ( un, "#  %d of them were not matched with any background motif.\n\n", uvalid );
    fclose ( out );
    fclose ( un );
    return true;
}

/* functions.cc:2241-2468 (plain) and 2469-2748 (structured): -S gets every
   printed motif, -U the unmatched ones, both in the SMILE-like format */
static void write_background_smile ( const Switch & sw, const Params & P, const std::vector<unsigned> & gmin,
                                     const std::vector<unsigned> & gmax, unsigned num_seqs, unsigned total_length,
                                     const char * alphabet, const std::vector<Printed> & printed, double exectime )
{
    FILE * un = fopen ( sw.un_smile_out_filename, "w" );
    if ( ! un ) { fprintf ( stderr, " Error: cannot open file %s!\n", sw.un_smile_out_filename ); return; }
    write_smile_header ( un, sw, P, gmin, gmax, num_seqs, total_length, alphabet );
    FILE * out = fopen ( sw.smile_out_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file %s!\n", sw.smile_out_filename ); fclose ( un ); return; }
    write_smile_header ( out, sw, P, gmin, gmax, num_seqs, total_length, alphabet );
    unsigned klen = sw.l;
    for ( unsigned b = 0; b < P.nb_gaps; ++b ) klen += P.blens[b] + 1;
    int bsize = 0, bquorum = 0;
    std::unordered_map<std::string, int> index;
    std::vector<BgEntry> bg;
    if ( ! read_background ( sw.background_in_filename, klen, &bsize, &bquorum, index, bg ) )
    {
        fprintf ( stderr, " Error: cannot open file %s!\n", sw.background_in_filename );
        fclose ( out );
        fclose ( un );
        return;
    }
    unsigned pvalid = 0, uvalid = 0;
    for ( const Printed & p : printed )
    {
        auto it = index.find ( p.key );
        const std::string line = smile_line ( P, alphabet, p );
        if ( it == index.end () || it->second < 0 )
        {
            fputs ( line.c_str (), un );
            uvalid++;
        }
        else
            pvalid++;
        fputs ( line.c_str (), out );
        index[p.key] = -1;
    }
    fprintf ( out, "Nb models: %d\n", pvalid + uvalid );
    fprintf ( out, "User time: %lf sec.\n", exectime );
    fprintf ( un, "Nb models: %d\n", uvalid );
    fprintf ( un, "User time: %lf sec.\n", exectime );
    fclose ( un );
    fclose ( out );
}

/* motex.cc:883-1137 (-I): the motif file's lines after its first blank
   line, up to the next one, are "motif u n r v"; each motif (all of its
   factors) is searched in every sequence at least total_mot_length long,
   and write_motifs_fore (functions.cc:2750-2829) prints the entry of its
   last factor with p-value 1 - P(X < u_file), X ~ Bin(n_file, u / N). */
static int foreground ( const Switch & sw, const Params & P, const std::vector<std::string> & seqs,
                        unsigned total_mot_length, int procs )
{
    FILE * in = fopen ( sw.un_in_filename, "r" );
    if ( ! in ) { fprintf ( stderr, " Error: Cannot open file %s!\n", sw.un_in_filename ); return 1; }
    char line[512];
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' );
    std::vector<std::string> fseqs;
    std::vector<BgEntry> fdata;
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' )
    {
        char * save = nullptr;
        char * tok = strtok_r ( line, " ", &save );
        const char * f[4] = { nullptr, nullptr, nullptr, nullptr };
        for ( int q = 0; q < 4 && tok; ++q ) f[q] = strtok_r ( nullptr, " ", &save );
        if ( ! tok || ! f[3] )
        {
            fprintf ( stderr, " Error: file %s is not in the correct format!\n", sw.un_in_filename );
            fclose ( in );
            return 1;
        }
        fseqs.push_back ( tok );
        fdata.push_back ( { ( unsigned ) atoi ( f[0] ), ( unsigned ) atoi ( f[1] ), ( unsigned ) atoi ( f[3] ), atof ( f[2] ) } );
    }
    fclose ( in );

    const unsigned num_seqs = ( unsigned ) seqs.size (), nf = ( unsigned ) fseqs.size ();
    std::vector<std::string> all ( fseqs );
    all.insert ( all.end (), seqs.begin (), seqs.end () );
    Coded C = encode ( all );
    std::vector<std::vector<unsigned>> U ( nf ), V ( nf );
    double start = gettime ();
    #pragma omp parallel for schedule(dynamic, 1)
    for ( unsigned i = 0; i < nf; ++i )
    {
        const std::vector<unsigned char> & x = C.seq[i];
        const unsigned m = ( unsigned ) x.size ();
        U[i].assign ( m, 0 );
        V[i].assign ( m, 0 );
        if ( m < P.l ) continue;                      /* no factor (the reference's flasm call is undefined) */
        std::vector<uint64_t> peq;
        if ( P.d == 1 ) build_peq ( x, P.l, C.sigma, peq );
        std::vector<unsigned char> occ;
        for ( unsigned j = 0; j < num_seqs; ++j )
        {
            const std::vector<unsigned char> & t = C.seq[nf + j];
            if ( total_mot_length > t.size () ) continue;
            extract_plain ( P, x, t, P.d == 1 ? &peq : nullptr, C.sigma, U[i].data (), V[i].data (), occ );
        }
    }
    double end = gettime ();

    FILE * out = fopen ( sw.output_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file!\n" ); return 0; }
    std::vector<unsigned> none;
    write_header ( out, sw, P, none, none, num_seqs, end - start, procs );
    unsigned maxn = num_seqs;
    for ( const BgEntry & f : fdata ) maxn = std::max ( maxn, f.n );
    std::vector<long double> LUT = fact_table ( ( int ) maxn );
    unsigned valid = 0;
    for ( unsigned i = 0; i < nf; ++i )
    {
        const unsigned m = ( unsigned ) fseqs[i].size ();
        if ( m == 0 ) continue;
        const unsigned u = U[i][m - 1], v = V[i][m - 1];
        if ( ! passes ( sw, u, v, num_seqs ) ) continue;
        long double cdf = binomial_cdf_below ( ( int ) fdata[i].u, ( int ) fdata[i].n, ( long double ) u / num_seqs, LUT.data () );
        fprintf ( out, "%s %d %d %lf %d %lf %d %Le\n", fseqs[i].c_str (), fdata[i].u, fdata[i].n, fdata[i].r, fdata[i].v,
                  ( double ) u / num_seqs, v, 1. - cdf );
        valid++;
    }
    fprintf ( out, "\n#A total of %d valid motifs were extracted.\n\n", valid );
    fclose ( out );
    return 0;
}

int main ( int argc, char ** argv )
{
    Switch sw;
    int i = decode_switches ( argc, argv, &sw );
    if ( i < 15 ) { usage (); return 1; }
    if ( sw.q > 100 ) { fprintf ( stderr, " Error: quorum argument q (%%) should be less or equal to 100!\n" ); return 1; }
    if ( sw.Q > 100 ) { fprintf ( stderr, " Error: max-quorum argument Q (%%) should be less or equal to 100!\n" ); return 1; }
    if ( sw.e >= sw.l ) { fprintf ( stderr, " Error: error threshold e must be less than the fixed-length of motifs k!\n" ); return 1; }
    if ( sw.d != 0 && sw.d != 1 )
    {
        fprintf ( stderr, " Error: distance argument d should be `0' for Hamming distance or `1' for edit distance!\n" );
        return 1;
    }
    const char * alphabet;
    if ( ! strcmp ( "DNA", sw.alphabet ) ) alphabet = ALPHA_DNA;
    else if ( ! strcmp ( "PROT", sw.alphabet ) ) alphabet = ALPHA_PROT;
    else if ( ! strcmp ( "USR", sw.alphabet ) ) alphabet = ALPHA_USR;
    else
    {
        fprintf ( stderr, " Error: alphabet argument a should be `DNA' for nucleotide sequences or `PROT' for protein sequences or `USR' for sequences over a user-defined alphabet!\n" );
        return 1;
    }
    /* motex.cc:147-201 */
    if ( ! sw.background_in_filename && sw.un_out_filename ) { fprintf ( stderr, " Error: `-u' option must be used with `-b' option!\n" ); return 1; }
    if ( ! sw.background_in_filename && sw.un_smile_out_filename ) { fprintf ( stderr, " Error: `-U' option must be used with `-b' option!\n" ); return 1; }
    if ( sw.background_in_filename && ! sw.un_out_filename ) { fprintf ( stderr, " Error: `-b' option must be used with `-u' option!\n" ); return 1; }
    if ( sw.background_in_filename && sw.un_smile_out_filename && ! sw.smile_out_filename ) { fprintf ( stderr, " Error: `-U' option must be used with `-S' option!\n" ); return 1; }
    if ( sw.background_in_filename && sw.un_in_filename ) { fprintf ( stderr, " Error: `-I' option cannot be used with `-b' option!\n" ); return 1; }
    if ( sw.boxes_in_filename && sw.un_in_filename ) { fprintf ( stderr, " Error: `-I' option cannot be used with `-s' option!\n" ); return 1; }

    /* motex.cc:225-300 FASTA reader */
    FILE * in = fopen ( sw.input_filename, "r" );
    if ( ! in ) { fprintf ( stderr, " Error: Cannot open file %s!\n", sw.input_filename ); return 1; }
    std::vector<std::string> seqs;
    std::string cur;
    int c = fgetc ( in );
    do
    {
        if ( c != '>' ) { fprintf ( stderr, " Error: input file %s is not in FASTA format!\n", sw.input_filename ); return 1; }
        while ( ( c = fgetc ( in ) ) != EOF && c != '\n' );
        cur.clear ();
        while ( ( c = fgetc ( in ) ) != EOF && c != '>' )
        {
            if ( cur.empty () && c == '\n' )
            {
                fprintf ( stderr, " Omitting empty sequence in file %s!\n", sw.input_filename );
                c = fgetc ( in );
                break;
            }
            if ( c == '\n' ) continue;
            c = toupper ( c );
            if ( strchr ( alphabet, c ) ) cur.push_back ( ( char ) c );
            else { fprintf ( stderr, " Error: input file %s contains an unexpected character!\n", sw.input_filename ); return 1; }
        }
        if ( ! cur.empty () ) seqs.push_back ( cur );
    } while ( c != EOF );
    fclose ( in );

    /* motex.cc:302-363 boxes */
    Params P;
    P.l = sw.l; P.e = sw.e; P.d = sw.d;
    P.nb_gaps = 0;
    std::vector<unsigned> gmin, gmax;
    unsigned total_mot_length = sw.l;
    if ( sw.boxes_in_filename )
    {
        FILE * bf = fopen ( sw.boxes_in_filename, "r" );
        if ( ! bf ) { fprintf ( stderr, " Error: Cannot open file %s!\n", sw.boxes_in_filename ); return 1; }
        if ( fscanf ( bf, "%u", &P.nb_gaps ) != 1 ) { fprintf ( stderr, " Error: file %s is not in the correct format!\n", sw.boxes_in_filename ); return 1; }
        gmin.resize ( P.nb_gaps ); gmax.resize ( P.nb_gaps ); P.blens.resize ( P.nb_gaps ); P.berrs.resize ( P.nb_gaps );
        for ( unsigned g = 0; g < P.nb_gaps; ++g )
        {
            if ( fscanf ( bf, "%u", &gmin[g] ) != 1 || fscanf ( bf, "%u", &gmax[g] ) != 1 ||
                 fscanf ( bf, "%u", &P.blens[g] ) != 1 || fscanf ( bf, "%u", &P.berrs[g] ) != 1 )
            {
                fprintf ( stderr, " Error: file %s is not in the correct format!\n", sw.boxes_in_filename );
                return 1;
            }
            total_mot_length += gmin[g] + P.blens[g];
        }
        fclose ( bf );
    }
    P.nb_boxes = P.nb_gaps + 1;
    /* motex.cc:439-486 + recurse (functions.cc:710-729): gap 0 varies slowest */
    P.nb_structs = 1;
    for ( unsigned g = 0; g < P.nb_gaps; ++g ) P.nb_structs *= gmax[g] - gmin[g] + 1;
    P.S.assign ( P.nb_structs, std::vector<unsigned> ( P.nb_gaps ) );
    for ( unsigned k = 0; k < P.nb_structs; ++k )
    {
        unsigned rem = k;
        for ( int g = ( int ) P.nb_gaps - 1; g >= 0; --g )
        {
            unsigned span = gmax[g] - gmin[g] + 1;
            P.S[k][g] = gmin[g] + rem % span;
            rem /= span;
        }
    }

    unsigned threads = sw.t;
#ifdef _OPENMP
    omp_set_num_threads ( ( int ) threads );
#else
    threads = 1;
#endif
    const unsigned num_seqs = ( unsigned ) seqs.size ();
    if ( sw.un_in_filename )
        return foreground ( sw, P, seqs, total_mot_length, ( int ) threads );
    Coded C = encode ( seqs );
    std::vector<std::vector<unsigned>> U, V;
    double start = gettime ();
    all_pairs ( P, C, total_mot_length, U, V, sw.input_filename );
    double end = gettime ();

    /* the motifs every writer visits: first passing occurrence of each key,
       (sequence, end position[, structure]) order */
    std::unordered_set<std::string> seen;
    std::vector<Printed> printed;
    if ( P.nb_gaps == 0 )
    {
        /* functions.cc:1073-1142 */
        for ( unsigned s = 0; s < num_seqs; ++s )
        {
            unsigned m = ( unsigned ) seqs[s].size ();
            for ( unsigned j = sw.l - 1; j < m; ++j )
            {
                if ( ! passes ( sw, U[s][j], V[s][j], num_seqs ) ) continue;
                std::string w = seqs[s].substr ( j - sw.l + 1, sw.l );
                if ( seen.insert ( w ).second ) printed.push_back ( { w, U[s][j], V[s][j] } );
            }
        }
    }
    else
    {
        /* functions.cc:1147-1260: key = boxes joined by '_', gaps excluded */
        for ( unsigned s = 0; s < num_seqs; ++s )
        {
            unsigned m = ( unsigned ) seqs[s].size ();
            for ( unsigned j = sw.l - 1; j < m; ++j )
                for ( unsigned k = 0; k < P.nb_structs; ++k )
                {
                    size_t idx = ( size_t ) k * m + j;
                    if ( ! passes ( sw, U[s][idx], V[s][idx], num_seqs ) ) continue;
                    unsigned jj = j - sw.l + 1, offset = 0, ell = sw.l;
                    std::string key = seqs[s].substr ( jj, sw.l );
                    for ( unsigned b = 1; b < P.nb_boxes; ++b )
                    {
                        offset += P.S[k][b - 1] + ell;
                        ell = P.blens[b - 1];
                        key.push_back ( '_' );
                        for ( unsigned q = 0; q < ell; ++q )
                        {
                            size_t at = ( size_t ) jj + offset + q;
                            key.push_back ( at < m ? seqs[s][at] : '\0' );
                        }
                    }
                    if ( seen.insert ( key ).second ) printed.push_back ( { key, U[s][idx], V[s][idx] } );
                }
        }
    }
    unsigned total_length = 0;
    for ( const std::string & q : seqs ) total_length += ( unsigned ) q.size ();

    if ( sw.background_in_filename )
    {
        /* motex.cc:844-849, 860-865: the -o/-u pair, then the SMILE pair only with -U */
        if ( ! write_background ( sw, P, gmin, gmax, num_seqs, printed, end - start, ( int ) threads ) ) return 1;
        if ( sw.un_smile_out_filename )
            write_background_smile ( sw, P, gmin, gmax, num_seqs, total_length, alphabet, printed, end - start );
        return 0;
    }

    FILE * out = fopen ( sw.output_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file!\n" ); return 1; }
    write_header ( out, sw, P, gmin, gmax, num_seqs, end - start, ( int ) threads );
    for ( const Printed & pr : printed )
        fprintf ( out, "%s %d %d %lf %d\n", pr.key.c_str (), pr.u, num_seqs, ( double ) pr.u / num_seqs, pr.v );
    if ( P.nb_gaps == 0 )
        fprintf ( out, "\n#A total of %d valid motifs were extracted.\n\n", ( int ) printed.size () );
    else
        fprintf ( out, "\n#A total of %d valid structured motifs were extracted.\n\n", ( int ) printed.size () );
    if ( fclose ( out ) ) { fprintf ( stderr, " Error: file close error!\n" ); return 1; }
    if ( sw.smile_out_filename )
    {
        FILE * so = fopen ( sw.smile_out_filename, "w" );
        if ( ! so ) { fprintf ( stderr, " Error: cannot open file!\n" ); return 0; }
        write_smile_header ( so, sw, P, gmin, gmax, num_seqs, total_length, alphabet );
        write_smile_lines ( so, P, alphabet, printed );
        fprintf ( so, "Nb models: %d\n", ( int ) printed.size () );
        fprintf ( so, "User time: %lf sec.\n", end - start );
        fclose ( so );
    }
    return 0;
}

#endif
