/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * The reference uses libdatrie 0.2.8 (shipped as a source tarball) purely as
 * an exact-string set in its writers (functions.cc:1092-1134, 1166-1252):
 * trie_retrieve() asks "was this word printed already?", trie_store() records
 * it.  This header declares that subset of the libdatrie C API (same names,
 * argument meaning and return values) so the reference sources compile
 * without running libdatrie's autotools build; datrie_set.cc implements it on
 * a std::unordered_map.  Keys are NUL-terminated AlphaChar (UCS-4) strings.
 */
#ifndef MOTEX_ORACLE_DATRIE_TRIE_H
#define MOTEX_ORACLE_DATRIE_TRIE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int Bool;
#ifndef FALSE
#define FALSE 0
#endif
#ifndef TRUE
#define TRUE 1
#endif

typedef uint32_t AlphaChar;
typedef int32_t  TrieData;
#define TRIE_DATA_ERROR (-1)

typedef struct _AlphaMap AlphaMap;
typedef struct _Trie Trie;

AlphaMap * alpha_map_new ( void );
void       alpha_map_free ( AlphaMap * alpha_map );
int        alpha_map_add_range ( AlphaMap * alpha_map, AlphaChar begin, AlphaChar end );

Trie *     trie_new ( const AlphaMap * alpha_map );
void       trie_free ( Trie * trie );
Bool       trie_retrieve ( const Trie * trie, const AlphaChar * key, TrieData * o_data );
Bool       trie_store ( Trie * trie, const AlphaChar * key, TrieData data );

#ifdef __cplusplus
}
#endif

#endif
