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
 *
 * The DP primitives are motex_core.h (restated libFLASM semantics, pinned
 * against the shipped library by flasm_difftest.cc).  The statistics /
 * SMILE / background modes (-b -u -U -I -S) are outside the hot path and are
 * rejected with an error.
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
#include <time.h>
#include <sys/time.h>
#include <stdint.h>
#include <string>
#include <vector>
#include <unordered_set>
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
    if ( sw.background_in_filename || sw.un_in_filename || sw.un_out_filename || sw.smile_out_filename || sw.un_smile_out_filename )
    {
        fprintf ( stderr, " Error: -b/-u/-U/-I/-S are not part of the extraction path restated here!\n" );
        return 1;
    }

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
    Coded C = encode ( seqs );
    std::vector<std::vector<unsigned>> U, V;
    double start = gettime ();
    all_pairs ( P, C, total_mot_length, U, V, sw.input_filename );
    double end = gettime ();

    FILE * out = fopen ( sw.output_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file!\n" ); return 1; }
    write_header ( out, sw, P, gmin, gmax, num_seqs, end - start, ( int ) threads );
    std::unordered_set<std::string> seen;
    unsigned valid = 0;
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
                if ( seen.insert ( w ).second )
                {
                    fprintf ( out, "%s %d %d %lf %d\n", w.c_str (), U[s][j], num_seqs, ( double ) U[s][j] / num_seqs, V[s][j] );
                    valid++;
                }
            }
        }
        fprintf ( out, "\n#A total of %d valid motifs were extracted.\n\n", valid );
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
                    if ( seen.insert ( key ).second )
                    {
                        fprintf ( out, "%s %d %d %lf %d\n", key.c_str (), U[s][idx], num_seqs, ( double ) U[s][idx] / num_seqs, V[s][idx] );
                        valid++;
                    }
                }
        }
        fprintf ( out, "\n#A total of %d valid structured motifs were extracted.\n\n", valid );
    }
    if ( fclose ( out ) ) { fprintf ( stderr, " Error: file close error!\n" ); return 1; }
    return 0;
}

#endif
