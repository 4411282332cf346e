/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * Restated libFLASM entry points (libflasm.h interface, called from
 * functions.cc:538, 633, 746, 843) on top of motex_core.h.  Linked with the
 * unmodified reference sources wherever the shipped x86-64 libflasm.so
 * cannot be used, and differentially tested against that .so by
 * flasm_difftest.cc.  MoTeX always passes return_all = true; the flag is
 * accepted and ignored.
 */
#include "libflasm.h"
#include "motex_core.h"

namespace libflasm
{

ResultTupleSet flasm_hd ( unsigned char * t, unsigned int n, unsigned char * x, unsigned int m,
                          unsigned int factor_length, unsigned int max_error, bool )
{
    ResultTupleSet out;
    motex_oracle::hd_scan ( t, n, x, m, factor_length, max_error,
        [&] ( unsigned i, unsigned j, unsigned err ) { out.insert ( ResultTuple { i, j, err } ); } );
    return out;
}

ResultTupleSet flasm_ed ( unsigned char * t, unsigned int n, unsigned char * x, unsigned int m,
                          unsigned int factor_length, unsigned int max_error, bool )
{
    ResultTupleSet out;
    motex_oracle::ed_scan ( t, n, x, m, factor_length, max_error,
        [&] ( unsigned i, unsigned j, unsigned err ) { out.insert ( ResultTuple { i, j, err } ); } );
    return out;
}

}
