/*
 * motexGPU -- drop-in for motexCPU / motexOMP on one GB300.
 *
 * Same command line, validation messages, FASTA/boxes parsing and output
 * file as the reference CLI; the all-pairs extraction, quorum filter and
 * first-occurrence deduplication run on the GPU behind include/motex_gpu.h.
 *
 * Follows the reference for:
 *   switches and defaults   functions.cc:2835-3043 (decode_switches)
 *   validation              motex.cc:98-201
 *   FASTA reader            motex.cc:225-300 (toupper, alphabet check,
 *                           empty records omitted) and the split at 409-437
 *   boxes file              motex.cc:302-363
 *   header                  functions.cc:1010-1068
 *   motif lines and footer  functions.cc:1118-1129, 1238-1247
 *   SMILE-like file (-S)    functions.cc:1262-1461 (header, plain motifs)
 *                           and 1463-1591 (structured motifs)
 *   option combinations     motex.cc:147-201
 *   background (-b -u -U)   functions.cc:1613-2238 (-o and -u files),
 *                           2241-2748 (the -S/-U pair)
 *   word search (-I)        motex.cc:883-1137, functions.cc:2750-2829;
 *                           the counting runs on the GPU (motex_gpu_search)
 *   binomial tail           binomial.cc:78-103 (the long double flavour:
 *                           the reference built without MPFR)
 * Differences: -L <int> is accepted as a real switch (the reference compiles
 * it out and getopt reports it as invalid; the output is the same) and -t is
 * accepted and ignored.
 *
 * Set MOTEX_METRICS=<file> to append a JSON line with the run's cell counts,
 * device time and GCUPS.
 */
#include "motex_gpu.h"

#include <ctype.h>
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>

#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

static const char * const ALPHA_DNA = "ACGTN";
static const char * const ALPHA_PROT = "ARNDCQEGHILKMFPSTWYVOUBZJX*";
static const char * const ALPHA_USR = "0123456789";

struct Switches
{
    char * alphabet = nullptr, * input_filename = nullptr, * output_filename = nullptr;
    char * background_in_filename = nullptr, * un_in_filename = nullptr, * un_out_filename = nullptr;
    char * boxes_in_filename = nullptr, * smile_out_filename = nullptr, * un_smile_out_filename = nullptr;
    unsigned q = 0, Q = 100, l = 0, d = 0, e = 0, n = 1, N = 10000, t = 4, L = 0;
};

static struct option long_options[] = {
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
    { "long-sequences", required_argument, NULL, 'L' },
    { "boxes-in-file", required_argument, NULL, 's' },
    { "unmatched-in-file", required_argument, NULL, 'I' },
    { "unmatched-out-file", required_argument, NULL, 'u' },
    { "SMILE-out-file", required_argument, NULL, 'S' },
    { "unmatched-SMILE-out-file", required_argument, NULL, 'U' },
    { "help", no_argument, NULL, 'h' },
    { NULL, 0, NULL, 0 } };

static void usage ( void )
{
    fprintf ( stdout, "\nm    m       mmmmmmm        m    m\n" );
    fprintf ( stdout, "##  ##  mmm     #     mmm    #  #\n" );
    fprintf ( stdout, "# ## # #\" \"#    #    #\"  #    ##\n" );
    fprintf ( stdout, "# \"\" # #   #    #    #\"\"\"\"   m\"\"m\n" );
    fprintf ( stdout, "#    # \"#m#\"    #    \"#mm\"  m\"  \"m\n\n" );
    fprintf ( stdout, " Usage: motexGPU <options>\n" );
    fprintf ( stdout, " Standard (Mandatory):\n" );
    fprintf ( stdout, "  -a, --alphabet            <str>     `DNA' for nucleotide  sequences or `PROT'\n"
                      "                                      for protein  sequences. You may use `USR'\n"
                      "                                      for user-defined alphabet.\n" );
    fprintf ( stdout, "  -i, --input-file          <str>     (Multi)FASTA input filename.\n" );
    fprintf ( stdout, "  -o, --output-file         <str>     MoTeX output filename.\n" );
    fprintf ( stdout, "  -d, --distance            <int>     The  distance  used  for extracting  the\n"
                      "                                      motifs. It can be  either 0 (for Hamming\n"
                      "                                      distance) or 1 (for edit distance).\n" );
    fprintf ( stdout, "  -k, --motifs-length       <int>     The length for motifs.\n" );
    fprintf ( stdout, "  -e, --errors              <int>     Limit the  max number  of errors to this\n"
                      "                                      value.\n" );
    fprintf ( stdout, "  -q, --quorum              <int>     The quorum is the minimum percentage (%%)\n"
                      "                                      of sequences in which a motif must occur.\n\n" );
    fprintf ( stdout, " Optional:\n" );
    fprintf ( stdout, "  -Q, --max-quorum          <int>     The maximum percentage (%%) of sequences\n"
                      "                                      in which a motif can occur (default: 100).\n" );
    fprintf ( stdout, "  -n, --num-of-occ          <int>     The minimum  number of  occurrences of a\n"
                      "                                      reported  motif in any  of the sequences\n"
                      "                                      (default: 1).\n" );
    fprintf ( stdout, "  -N, --max-num-of-occ      <int>     The maximum  number of  occurrences of a\n"
                      "                                      reported  motif in any  of the sequences\n"
                      "                                      (default: 10000).\n" );
    fprintf ( stdout, "  -s, --structured-motifs   <str>     Input filename  for the structure of the\n"
                      "                                      boxes in the case of structured motifs.\n" );
    fprintf ( stdout, "  -S, --SMILE-out-file      <str>     SMILE-like output filename to be used by\n"
                      "                                      SMILE.\n" );
    fprintf ( stdout, "  -L, --long-sequences      <int>     Accepted for compatibility; the GPU tiles\n"
                      "                                      long sequences by itself.\n" );
    fprintf ( stdout, "  -t, --threads             <int>     Accepted for compatibility (ignored).\n" );
}

static int decode_switches ( int argc, char ** argv, Switches * sw )
{
    int oi, opt, args = 0;
    double val;
    char * ep;
    while ( ( opt = getopt_long ( argc, argv, "a:b:i:o:q:Q:k:d:e:n:N:s:t:I:S:u:U:L:h", long_options, &oi ) ) != -1 )
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
            case 'L': val = strtol ( optarg, &ep, 10 ); if ( ! ep || ep == optarg ) return 0; sw->L = ( unsigned ) val; break;
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

static void write_header ( FILE * out, const Switches & sw, const motex_params & P, unsigned num_seqs, double secs )
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
    if ( P.nb_gaps == 0 )
    {
        fprintf ( out, "#     l = %d\n", sw.l );
        fprintf ( out, "#     e = %d\n", sw.e );
    }
    else
    {
        fprintf ( out, "# Number of boxes: %d\n", P.nb_gaps + 1 );
        fprintf ( out, "#     l0 = %d\n", sw.l );
        fprintf ( out, "#     e0 = %d\n", sw.e );
        for ( unsigned i = 0; i < P.nb_gaps; ++i )
        {
            fprintf ( out, "#     g%d = [%d,%d]\n", i + 1, P.gap_min[i], P.gap_max[i] );
            fprintf ( out, "#     l%d = %d\n", i + 1, P.blens[i] );
            fprintf ( out, "#     e%d = %d\n", i + 1, P.berrs[i] );
        }
        fprintf ( out, "# Boxes input file: %s\n", sw.boxes_in_filename );
    }
    fprintf ( out, "# Run on %d proc(s) in %lf secs\n", 1, secs );
    fprintf ( out, "####################################\n\n" );
}

/*
 * SMILE-like output (functions.cc:1262-1345 header, 1368-1461 plain motifs,
 * 1463-1591 structured motifs).  The header line starts with "%%%", gives the
 * box count, the absolute quorum ceil(q * num_seqs / 100) over num_seqs, the
 * total input length and, per box, length range and error budget, then the
 * alphabet; DNA pads it to 79 columns and adds two blank 79-column lines,
 * PROT pads to 159 columns and adds one, USR adds nothing before the rule of
 * '='.  Each motif line is the word (boxes joined by '_'), its symbol-index
 * string ('0' + rank in the alphabet string, '-' for a separator), u, a tab
 * and v.  The motif set and order are those of the main output.
 */
static void write_smile_header ( FILE * out, const Switches & sw, const motex_params & P, unsigned num_seqs,
                                 unsigned total_length, const char * alphabet )
{
    char buf[128];
    const int quorum = ( int ) ceil ( ( double ) ( ( double ) sw.q * num_seqs ) / ( double ) 100 );
    std::string line;
    if ( P.nb_gaps == 0 )
    {
        snprintf ( buf, sizeof buf, "%%%%%% 1 %d/%d %d %d %d %d alphabet ", quorum, num_seqs, total_length, sw.l, sw.l, sw.e );
        line = buf;
    }
    else
    {
        unsigned len = sw.l, errs = sw.e;
        for ( unsigned g = 0; g < P.nb_gaps; ++g ) { len += P.blens[g]; errs += P.berrs[g]; }
        snprintf ( buf, sizeof buf, "%%%%%% %d %d/%d %d %d %d %d %d %d %d ", P.nb_gaps + 1, quorum, num_seqs, total_length,
                   len, len, errs, sw.l, sw.l, sw.e );
        line = buf;
        for ( unsigned g = 0; g < P.nb_gaps; ++g )
        {
            snprintf ( buf, sizeof buf, "%d %d %d %d %d ", P.gap_min[g], P.gap_max[g], P.blens[g], P.blens[g], P.berrs[g] );
            line += buf;
        }
        line += "alphabet ";
    }
    line += alphabet;
    line += '$';
    fputs ( line.c_str (), out );
    const std::string blank ( 79, ' ' );
    if ( ! strcmp ( sw.alphabet, "DNA" ) )
    {
        if ( line.size () < 79 ) fputs ( std::string ( 79 - line.size (), ' ' ).c_str (), out );
        fprintf ( out, "\n%s\n%s\n", blank.c_str (), blank.c_str () );
    }
    if ( ! strcmp ( sw.alphabet, "PROT" ) )
    {
        if ( line.size () < 159 ) fputs ( std::string ( 159 - line.size (), ' ' ).c_str (), out );
        fprintf ( out, "\n%s\n", blank.c_str () );
    }
    fprintf ( out, "%s\n", std::string ( 79, '=' ).c_str () );
}

static void write_smile_line ( FILE * out, const motex_params & P, const char * alphabet, const std::string & w,
                               uint32_t u, uint32_t v )
{
    const size_t na = strlen ( alphabet );
    std::string id ( w.size (), '-' );
    for ( size_t i = 0; i < w.size (); ++i )
    {
        const char * at = w[i] ? ( const char * ) memchr ( alphabet, w[i], na ) : nullptr;
        id[i] = at ? ( char ) ( '0' + ( at - alphabet ) ) : ( P.nb_gaps ? '-' : ( char ) ( '0' + na ) );
    }
    fprintf ( out, "%s %s %d\t%d\n", w.c_str (), id.c_str (), u, v );
}

/*
 * P(X < x) for X ~ Bin(N, p), 0 when p >= 1 (binomial.cc:78-103, the long
 * double flavour).  fact[i] = i!.  The terms are formed and summed in the
 * reference's order so that the rounding, and so the printed tail
 * 1 - P(X < x), is the same on a host with the same long double format.
 */
static std::vector<long double> factorials ( unsigned n )
{
    std::vector<long double> f ( ( size_t ) n + 1 );
    f[0] = 1;
    for ( unsigned i = 1; i <= n; ++i ) f[i] = f[i - 1] * i;
    return f;
}

static long double binomial_below ( int x, int N, long double p, const std::vector<long double> & fact )
{
    long double sum = 0.;
    if ( p >= 1.0 ) return 0.;
    for ( int i = 0; i < x; ++i )
    {
        const long double term = ( fact[N] / fact[i] ) / fact[N - i] * powl ( p, ( long double ) i ) *
                                 powl ( 1. - p, ( long double ) ( N - i ) );
        sum += term;
        if ( x > N ) break;
    }
    return sum;
}

/*
 * A MoTeX output file read as a background (functions.cc:1683-1757): header
 * line 6 ("# For N input sequences") gives N, line 8 ("#     q = Q") gives Q;
 * after the header's blank line, one motif per line up to the next blank
 * line: its key (the first klen symbols), u, n, r and v.  A repeated key
 * keeps its last row.
 */
struct Background
{
    struct Row
    {
        unsigned u = 0, n = 0, v = 0;
        double r = 0;
    };
    int size = 0, quorum = 0;
    std::unordered_map<std::string, int> index;       // key -> row; -1 once printed
    std::vector<Row> rows;
};

static bool read_background ( const char * path, size_t klen, Background & bg )
{
    FILE * in = fopen ( path, "r" );
    if ( ! in ) return false;
    char line[512];
    std::string size_field, quorum_field;
    for ( unsigned ln = 1; fgets ( line, sizeof line, in ) && line[0] != '\n'; ++ln )
    {
        if ( ln != 6 && ln != 8 ) continue;
        char * save = nullptr;
        char * f = strtok_r ( line, " ", &save );
        for ( int k = 0; k < 2 && f; ++k ) f = strtok_r ( nullptr, " ", &save );
        if ( ln == 8 && f ) f = strtok_r ( nullptr, "\n", &save );
        ( ln == 6 ? size_field : quorum_field ) = f ? f : "";
    }
    bg.size = atoi ( size_field.c_str () );
    bg.quorum = atoi ( quorum_field.c_str () );
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' )
    {
        char * save = nullptr;
        char * key = strtok_r ( line, " ", &save );
        if ( ! key ) continue;
        const char * f[4] = {};
        for ( int k = 0; k < 4; ++k ) f[k] = strtok_r ( nullptr, " ", &save );
        Background::Row row;
        row.u = ( unsigned ) atoi ( f[0] ? f[0] : "0" );
        row.n = ( unsigned ) atoi ( f[1] ? f[1] : "0" );
        row.r = atof ( f[2] ? f[2] : "0" );
        row.v = ( unsigned ) atoi ( f[3] ? f[3] : "0" );
        bg.index[std::string ( key, strnlen ( key, klen ) )] = ( int ) bg.rows.size ();
        bg.rows.push_back ( row );
    }
    fclose ( in );
    return true;
}

/*
 * -I (motex.cc:883-1137): the motif file is read from after its first blank
 * line up to the next one, one "motif u n r v" per line; the GPU counts
 * every motif's last factor in every sequence at least l long, and
 * write_motifs_fore (functions.cc:2750-2829) prints the passing ones with
 * the file's u n r v, the new u/N and v, and 1 - P(X < u_file) for
 * X ~ Bin(n_file, u/N).
 */
static int run_foreground ( const Switches & sw, const motex_params & P, const std::vector<std::string> & seqs )
{
    FILE * in = fopen ( sw.un_in_filename, "r" );
    if ( ! in ) { fprintf ( stderr, " Error: Cannot open file %s!\n", sw.un_in_filename ); return 1; }
    char line[512];
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' );
    std::vector<std::string> motifs;
    std::vector<Background::Row> given;
    while ( fgets ( line, sizeof line, in ) && line[0] != '\n' )
    {
        char * save = nullptr;
        char * word = strtok_r ( line, " ", &save );
        const char * f[4] = {};
        for ( int k = 0; k < 4 && word; ++k ) f[k] = strtok_r ( nullptr, " ", &save );
        if ( ! word || ! f[3] )
        {
            fprintf ( stderr, " Error: file %s is not in the correct format!\n", sw.un_in_filename );
            fclose ( in );
            return 1;
        }
        motifs.push_back ( word );
        Background::Row row;
        row.u = ( unsigned ) atoi ( f[0] );
        row.n = ( unsigned ) atoi ( f[1] );
        row.r = atof ( f[2] );
        row.v = ( unsigned ) atoi ( f[3] );
        given.push_back ( row );
    }
    if ( fclose ( in ) ) { fprintf ( stderr, " Error: file close error!\n" ); return 1; }

    const unsigned num_seqs = ( unsigned ) seqs.size (), nm = ( unsigned ) motifs.size ();
    std::vector<const char *> wptr ( nm ), sptr ( num_seqs );
    std::vector<uint32_t> wlen ( nm ), slen ( num_seqs ), u ( nm ), v ( nm );
    for ( unsigned i = 0; i < nm; ++i ) { wptr[i] = motifs[i].data (); wlen[i] = ( uint32_t ) motifs[i].size (); }
    for ( unsigned s = 0; s < num_seqs; ++s ) { sptr[s] = seqs[s].data (); slen[s] = ( uint32_t ) seqs[s].size (); }
    motex_ctx * ctx = nullptr;
    int rc = motex_ctx_create ( &ctx, 0 );
    if ( rc != MOTEX_OK ) { fprintf ( stderr, " Error: %s: %s\n", motex_gpu_strerror ( rc ), motex_gpu_last_error () ); return 1; }
    double start = gettime ();
    rc = motex_gpu_search ( ctx, &P, wptr.data (), wlen.data (), nm, sptr.data (), slen.data (), num_seqs, u.data (), v.data () );
    double end = gettime ();
    motex_ctx_destroy ( ctx );
    if ( rc != MOTEX_OK )
    {
        fprintf ( stderr, " Error: word search failed: %s: %s\n", motex_gpu_strerror ( rc ), motex_gpu_last_error () );
        return 1;
    }

    FILE * out = fopen ( sw.output_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file!\n" ); return 0; }
    write_header ( out, sw, P, num_seqs, end - start );
    unsigned top = num_seqs;
    for ( const Background::Row & g : given ) top = std::max ( top, g.n );
    const std::vector<long double> fact = factorials ( top );
    unsigned valid = 0;
    for ( unsigned i = 0; i < nm; ++i )
    {
        if ( motifs[i].empty () ) continue;
        const double ratio = ( double ) u[i] / num_seqs;
        const double pct = ratio * 100;
        if ( ! ( pct >= sw.q && v[i] >= sw.n && pct <= sw.Q && v[i] <= sw.N ) ) continue;
        const long double below = binomial_below ( ( int ) given[i].u, ( int ) given[i].n, ( long double ) u[i] / num_seqs, fact );
        fprintf ( out, "%s %d %d %lf %d %lf %d %Le\n", motifs[i].c_str (), given[i].u, given[i].n, given[i].r, given[i].v,
                  ratio, v[i], 1. - below );
        valid++;
    }
    fprintf ( out, "\n#A total of %d valid motifs were extracted.\n\n", valid );
    if ( fclose ( out ) ) fprintf ( stderr, " Error: file close error!\n" );
    return 0;
}

/*
 * -b (functions.cc:1613-2238): each printed motif either matches a row of
 * the background not yet matched -- printed with that row's r and v and
 * 1 - P(X < u), X ~ Bin(N, row u) -- or is unmatched: printed with "0 0"
 * and 1 - P(X < u), X ~ Bin(N, Q_bg / N_bg), and also written to the -u
 * file.  With -U the same split goes to the -S/-U SMILE-like pair
 * (functions.cc:2241-2748).  Returns false on the reference's assertion
 * of a background without a sequence count or quorum.
 */
static bool write_background ( const Switches & sw, const motex_params & P, unsigned num_seqs, unsigned total_length,
                               const char * alphabet, const std::vector<std::string> & words, const motex_result & res,
                               double secs )
{
    size_t klen = sw.l;
    for ( unsigned g = 0; g < P.nb_gaps; ++g ) klen += P.blens[g] + 1;
    FILE * out = fopen ( sw.output_filename, "w" );
    if ( ! out ) { fprintf ( stderr, " Error: cannot open file!\n" ); return true; }
    write_header ( out, sw, P, num_seqs, secs );
    FILE * un = fopen ( sw.un_out_filename, "w" );
    if ( ! un ) { fprintf ( stderr, " Error: cannot open file!\n" ); fclose ( out ); return true; }
    write_header ( un, sw, P, num_seqs, secs );
    Background bg;
    if ( ! read_background ( sw.background_in_filename, klen, bg ) )
    {
        fprintf ( stderr, " Error: cannot open file!\n" );
        fclose ( out );
        fclose ( un );
        return true;
    }
    if ( ! ( bg.size > 0 && bg.quorum > 0 ) )
    {
        fprintf ( stderr, " Error: background file %s gives no sequence count or no quorum!\n", sw.background_in_filename );
        fclose ( out );
        fclose ( un );
        return false;
    }
    const std::vector<long double> fact = factorials ( num_seqs );
    const long double p_bg = ( long double ) bg.quorum / bg.size;
    std::vector<char> matched ( res.count, 0 );
    unsigned pvalid = 0, uvalid = 0;
    for ( uint32_t r = 0; r < res.count; ++r )
    {
        const motex_motif & m = res.motifs[r];
        const double ratio = ( double ) m.u / num_seqs;
        auto it = bg.index.find ( words[r] );
        if ( it != bg.index.end () && it->second >= 0 )
        {
            const Background::Row & row = bg.rows[it->second];
            const long double below = binomial_below ( ( int ) m.u, ( int ) num_seqs, ( long double ) row.u, fact );
            fprintf ( out, "%s %d %d %lf %d %lf %d %Le\n", words[r].c_str (), m.u, num_seqs, ratio, m.v, row.r, row.v,
                      1. - below );
            matched[r] = 1;
            pvalid++;
        }
        else
        {
            const long double below = binomial_below ( ( int ) m.u, ( int ) num_seqs, p_bg, fact );
            fprintf ( out, "%s %d %d %lf %d %d %d %Le\n", words[r].c_str (), m.u, num_seqs, ratio, m.v, 0, 0, 1. - below );
            fprintf ( un, "%s %d %d %lf %d\n", words[r].c_str (), m.u, num_seqs, ratio, m.v );
            uvalid++;
        }
        bg.index[words[r]] = -1;
    }
    fprintf ( out, "\n#A total of %d background motifs were read.\n", ( int ) bg.rows.size () );
    fprintf ( out, "#A total of %d valid motifs were extracted:\n", pvalid + uvalid );
    fprintf ( out, "#  %d of them were matched with background motifs\n", pvalid );
    fprintf ( out, "#  %d of them were not matched with any background motif.\n\n", uvalid );
    fprintf ( un, "\n#A total of %d background motifs were read.\n", ( int ) bg.rows.size () );
    fprintf ( un, "#A total of %d valid motifs were extracted:\n", pvalid + uvalid );
    fprintf ( un, "#  %d of them were not matched with any background motif.\n\n", uvalid );
    if ( fclose ( out ) || fclose ( un ) ) fprintf ( stderr, " Error: file close error!\n" );
    if ( ! sw.un_smile_out_filename ) return true;

    FILE * usm = fopen ( sw.un_smile_out_filename, "w" );
    if ( ! usm ) { fprintf ( stderr, " Error: cannot open file %s!\n", sw.un_smile_out_filename ); return true; }
    write_smile_header ( usm, sw, P, num_seqs, total_length, alphabet );
    FILE * sm = fopen ( sw.smile_out_filename, "w" );
    if ( ! sm ) { fprintf ( stderr, " Error: cannot open file %s!\n", sw.smile_out_filename ); fclose ( usm ); return true; }
    write_smile_header ( sm, sw, P, num_seqs, total_length, alphabet );
    for ( uint32_t r = 0; r < res.count; ++r )
    {
        if ( ! matched[r] ) write_smile_line ( usm, P, alphabet, words[r], res.motifs[r].u, res.motifs[r].v );
        write_smile_line ( sm, P, alphabet, words[r], res.motifs[r].u, res.motifs[r].v );
    }
    fprintf ( sm, "Nb models: %d\n", pvalid + uvalid );
    fprintf ( sm, "User time: %lf sec.\n", secs );
    fprintf ( usm, "Nb models: %d\n", uvalid );
    fprintf ( usm, "User time: %lf sec.\n", secs );
    if ( fclose ( usm ) || fclose ( sm ) ) fprintf ( stderr, " Error: file close error!\n" );
    return true;
}

int main ( int argc, char ** argv )
{
    Switches sw;
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
    /* option combinations (motex.cc:147-201) */
    if ( ! sw.background_in_filename )
    {
        if ( sw.un_out_filename ) { fprintf ( stderr, " Error: `-u' option must be used with `-b' option!\n" ); return 1; }
        if ( sw.un_smile_out_filename ) { fprintf ( stderr, " Error: `-U' option must be used with `-b' option!\n" ); return 1; }
    }
    else
    {
        if ( ! sw.un_out_filename ) { fprintf ( stderr, " Error: `-b' option must be used with `-u' option!\n" ); return 1; }
        if ( sw.un_smile_out_filename && ! sw.smile_out_filename )
        {
            fprintf ( stderr, " Error: `-U' option must be used with `-S' option!\n" );
            return 1;
        }
        if ( sw.un_in_filename ) { fprintf ( stderr, " Error: `-I' option cannot be used with `-b' option!\n" ); return 1; }
    }
    if ( sw.boxes_in_filename && sw.un_in_filename )
    {
        fprintf ( stderr, " Error: `-I' option cannot be used with `-s' option!\n" );
        return 1;
    }

    /* FASTA reader (motex.cc:225-300) */
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
            if ( c != 0 && strchr ( alphabet, c ) ) cur.push_back ( ( char ) c );
            else { fprintf ( stderr, " Error: input file %s contains an unexpected character!\n", sw.input_filename ); return 1; }
        }
        if ( ! cur.empty () ) seqs.push_back ( cur );
    } while ( c != EOF );
    if ( fclose ( in ) ) { fprintf ( stderr, " Error: file close error!\n" ); return 1; }
    if ( seqs.empty () ) { fprintf ( stderr, " Error: input file %s holds no sequence!\n", sw.input_filename ); return 1; }

    /* boxes file (motex.cc:302-363) */
    motex_params P {};
    P.d = sw.d; P.l = sw.l; P.e = sw.e; P.q = sw.q; P.Q = sw.Q; P.n = sw.n; P.N = sw.N;
    std::vector<uint32_t> gmin, gmax, blens, berrs;
    if ( sw.boxes_in_filename )
    {
        FILE * bf = fopen ( sw.boxes_in_filename, "r" );
        if ( ! bf ) { fprintf ( stderr, " Error: Cannot open file %s!\n", sw.boxes_in_filename ); return 1; }
        unsigned ng;
        if ( fscanf ( bf, "%u", &ng ) != 1 ) { fprintf ( stderr, " Error: file %s is not in the correct format!\n", sw.boxes_in_filename ); return 1; }
        gmin.resize ( ng ); gmax.resize ( ng ); blens.resize ( ng ); berrs.resize ( ng );
        for ( unsigned g = 0; g < ng; ++g )
            if ( fscanf ( bf, "%u", &gmin[g] ) != 1 || fscanf ( bf, "%u", &gmax[g] ) != 1 ||
                 fscanf ( bf, "%u", &blens[g] ) != 1 || fscanf ( bf, "%u", &berrs[g] ) != 1 )
            {
                fprintf ( stderr, " Error: file %s is not in the correct format!\n", sw.boxes_in_filename );
                return 1;
            }
        if ( fclose ( bf ) ) { fprintf ( stderr, " Error: file close error!\n" ); return 1; }
        P.nb_gaps = ng;
        P.gap_min = gmin.data (); P.gap_max = gmax.data (); P.blens = blens.data (); P.berrs = berrs.data ();
    }

    if ( sw.un_in_filename ) return run_foreground ( sw, P, seqs );

    std::vector<const char *> ptrs ( seqs.size () );
    std::vector<uint32_t> lens ( seqs.size () );
    for ( size_t s = 0; s < seqs.size (); ++s ) { ptrs[s] = seqs[s].data (); lens[s] = ( uint32_t ) seqs[s].size (); }

    motex_ctx * ctx = nullptr;
    int rc = motex_ctx_create ( &ctx, 0 );
    if ( rc != MOTEX_OK ) { fprintf ( stderr, " Error: %s: %s\n", motex_gpu_strerror ( rc ), motex_gpu_last_error () ); return 1; }
    motex_result res;
    double start = gettime ();
    rc = motex_gpu_run ( ctx, &P, ptrs.data (), lens.data (), ( uint32_t ) seqs.size (), &res );
    double end = gettime ();
    if ( rc != MOTEX_OK )
    {
        fprintf ( stderr, " Error: extraction failed: %s: %s\n", motex_gpu_strerror ( rc ), motex_gpu_last_error () );
        motex_ctx_destroy ( ctx );
        return 1;
    }
    const unsigned num_seqs = ( unsigned ) seqs.size ();

    /* the printed words: box 0, then each further box after its gap, joined
       by '_' (functions.cc:1191-1239); symbols past a sequence end read as NUL */
    std::vector<std::string> words ( res.count );
    std::vector<unsigned> S ( P.nb_gaps );
    for ( uint32_t r = 0; r < res.count; ++r )
    {
        const motex_motif & m = res.motifs[r];
        const std::string & s = seqs[m.seq];
        const size_t jj = m.pos + 1 - sw.l;
        std::string & word = words[r];
        word.assign ( s, jj, sw.l );
        if ( P.nb_gaps )
        {
            unsigned rem = m.strct;
            for ( int g = ( int ) P.nb_gaps - 1; g >= 0; --g )
            {
                unsigned span = P.gap_max[g] - P.gap_min[g] + 1;
                S[g] = P.gap_min[g] + rem % span;
                rem /= span;
            }
            size_t offset = 0, ell = sw.l;
            for ( unsigned b = 1; b <= P.nb_gaps; ++b )
            {
                offset += S[b - 1] + ell;
                ell = P.blens[b - 1];
                word.push_back ( '_' );
                for ( size_t q = 0; q < ell; ++q )
                    word.push_back ( jj + offset + q < s.size () ? s[jj + offset + q] : '\0' );
            }
        }
    }

    unsigned total_length = 0;
    for ( const std::string & q : seqs ) total_length += ( unsigned ) q.size ();

    /* a file that cannot be opened is reported and skipped; the exit status
       stays 0, as the reference ignores its writers' status (motex.cc:836-866) */
    if ( sw.background_in_filename )
    {
        if ( ! write_background ( sw, P, num_seqs, total_length, alphabet, words, res, end - start ) )
        {
            motex_result_free ( &res );
            motex_ctx_destroy ( ctx );
            return 1;
        }
    }
    else
    {
        FILE * out = fopen ( sw.output_filename, "w" );
        if ( ! out ) fprintf ( stderr, " Error: cannot open file!\n" );
        else
        {
            write_header ( out, sw, P, num_seqs, end - start );
            for ( uint32_t r = 0; r < res.count; ++r )
            {
                const motex_motif & m = res.motifs[r];
                fprintf ( out, "%s %d %d %lf %d\n", words[r].c_str (), m.u, num_seqs, ( double ) m.u / num_seqs, m.v );
            }
            if ( P.nb_gaps )
                fprintf ( out, "\n#A total of %d valid structured motifs were extracted.\n\n", res.count );
            else
                fprintf ( out, "\n#A total of %d valid motifs were extracted.\n\n", res.count );
            if ( fclose ( out ) ) fprintf ( stderr, " Error: file close error!\n" );
        }
        if ( sw.smile_out_filename )
        {
            FILE * so = fopen ( sw.smile_out_filename, "w" );
            if ( ! so ) fprintf ( stderr, " Error: cannot open file!\n" );
            else
            {
                write_smile_header ( so, sw, P, num_seqs, total_length, alphabet );
                for ( uint32_t r = 0; r < res.count; ++r )
                    write_smile_line ( so, P, alphabet, words[r], res.motifs[r].u, res.motifs[r].v );
                fprintf ( so, "Nb models: %d\n", res.count );
                fprintf ( so, "User time: %lf sec.\n", end - start );
                if ( fclose ( so ) ) fprintf ( stderr, " Error: file close error!\n" );
            }
        }
    }

    const char * mpath = getenv ( "MOTEX_METRICS" );
    if ( mpath && *mpath )
    {
        FILE * mf = fopen ( mpath, "a" );
        if ( mf )
        {
            double secs = end - start;
            fprintf ( mf, "{\"tool\": \"motexGPU\", \"num_seqs\": %u, \"motifs\": %u, \"unique_words\": %u, "
                          "\"ref_cells\": %llu, \"exec_cells\": %llu, \"wall_s\": %.6f, \"device_ms\": %.3f, "
                          "\"gcups_ref_wall\": %.3f, \"launches\": %u}\n",
                      num_seqs, res.count, res.unique_words, ( unsigned long long ) res.ref_cells,
                      ( unsigned long long ) res.exec_cells, secs, res.device_ms,
                      secs > 0 ? res.ref_cells / secs / 1e9 : 0.0, res.launches );
            fclose ( mf );
        }
    }
    motex_result_free ( &res );
    motex_ctx_destroy ( ctx );
    return 0;
}
