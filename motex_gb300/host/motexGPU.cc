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
 * Differences: -L <int> is accepted as a real switch (the reference compiles
 * it out and getopt reports it as invalid; the output is the same), -t is
 * accepted and ignored, and the background / unmatched-motif modes
 * (-b -u -U -I) are rejected after the reference's own checks of their
 * combinations.
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

#include <string>
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
static void write_smile ( FILE * out, const Switches & sw, const motex_params & P, unsigned num_seqs,
                          unsigned total_length, const char * alphabet, const std::vector<std::string> & words,
                          const motex_result & res, double secs )
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

    const size_t na = strlen ( alphabet );
    std::string id;
    for ( uint32_t r = 0; r < res.count; ++r )
    {
        const std::string & w = words[r];
        id.resize ( w.size () );
        for ( size_t i = 0; i < w.size (); ++i )
        {
            const char * at = w[i] ? ( const char * ) memchr ( alphabet, w[i], na ) : nullptr;
            id[i] = at ? ( char ) ( '0' + ( at - alphabet ) ) : ( P.nb_gaps ? '-' : ( char ) ( '0' + na ) );
        }
        fprintf ( out, "%s %s %d\t%d\n", w.c_str (), id.c_str (), res.motifs[r].u, res.motifs[r].v );
    }
    fprintf ( out, "Nb models: %d\n", res.count );
    fprintf ( out, "User time: %lf sec.\n", secs );
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
    if ( sw.background_in_filename || sw.un_in_filename )
    {
        fprintf ( stderr, " Error: the background and unmatched-motif modes (-b -u -U -I) are not part of motexGPU!\n" );
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

    /* a file that cannot be opened is reported and skipped; the exit status
       stays 0, as the reference ignores its writers' status (motex.cc:836-866) */
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
            unsigned total_length = 0;
            for ( const std::string & q : seqs ) total_length += ( unsigned ) q.size ();
            write_smile ( so, sw, P, num_seqs, total_length, alphabet, words, res, end - start );
            if ( fclose ( so ) ) fprintf ( stderr, " Error: file close error!\n" );
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
