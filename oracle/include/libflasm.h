/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * Declares the libFLASM interface that MoTeX calls (functions.cc:538, 633,
 * 746, 843).  libFLASM ships with the reference only as a header plus a
 * prebuilt x86-64 shared object (libFLASM.zip), so this header restates the
 * interface in its own words with the identical type layout:
 *   - ResultTuple {pos_t, pos_x, error} doubles as its own comparator
 *     (error, pos_t, pos_x ascending), exactly as the shipped header defines
 *     it, so std::multiset<ResultTuple, ResultTuple> is ABI-compatible with
 *     the shipped libflasm.so and the reference sources compile unchanged.
 *   - The SeqAn include of the shipped header is not needed by the interface
 *     and is omitted.
 * It is used (a) to link the unmodified reference sources against the
 * shipped libflasm.so on x86-64 and (b) to link them against the restated
 * flasm in flasm_port.cc (every other host, e.g. the aarch64 GPU host).
 */
#ifndef MOTEX_ORACLE_LIBFLASM_H
#define MOTEX_ORACLE_LIBFLASM_H

#include <stdio.h>
#include <cstring>
#include <cstdlib>
#include <cmath>
#include <climits>
#include <set>

using namespace std;

namespace libflasm
{
    struct ResultTuple {
        bool operator() (const ResultTuple& a, const ResultTuple& b) const
        {
            if ( a.error != b.error ) return a.error < b.error;
            if ( a.pos_t != b.pos_t ) return a.pos_t < b.pos_t;
            return a.pos_x < b.pos_x;
        }
        unsigned int pos_t;
        unsigned int pos_x;
        unsigned int error;
    };

    typedef std::multiset<ResultTuple, ResultTuple> ResultTupleSet;
    typedef ResultTupleSet::iterator ResultTupleSetIterator;

    ResultTupleSet flasm_ed ( unsigned char * t, unsigned int n, unsigned char * x, unsigned int m,
                              unsigned int factor_length, unsigned int max_error, bool return_all );
    ResultTupleSet flasm_hd ( unsigned char * t, unsigned int n, unsigned char * x, unsigned int m,
                              unsigned int factor_length, unsigned int max_error, bool return_all );
}

#endif
