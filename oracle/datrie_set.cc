/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * Exact-string set/map with the libdatrie calls the reference writers make
 * (functions.cc:1092-1134: alpha_map_new, alpha_map_add_range, trie_new,
 * trie_retrieve, trie_store, trie_free, alpha_map_free).  Only the
 * set-membership behaviour matters to MoTeX: retrieve returns TRUE iff the
 * exact key was stored before; store inserts or overwrites.
 */
#include "datrie/trie.h"

#include <string>
#include <unordered_map>

struct _AlphaMap { AlphaChar lo, hi; };
struct _Trie { std::unordered_map<std::u32string, TrieData> map; };

static std::u32string key_of ( const AlphaChar * key )
{
    std::u32string s;
    for ( ; *key; ++key ) s.push_back ( ( char32_t ) *key );
    return s;
}

extern "C" {

AlphaMap * alpha_map_new ( void ) { return new _AlphaMap { 0, 0 }; }
void alpha_map_free ( AlphaMap * a ) { delete a; }
int alpha_map_add_range ( AlphaMap * a, AlphaChar begin, AlphaChar end )
{
    if ( begin > end ) return -1;
    a->lo = begin; a->hi = end;
    return 0;
}

Trie * trie_new ( const AlphaMap * ) { return new _Trie (); }
void trie_free ( Trie * t ) { delete t; }

Bool trie_retrieve ( const Trie * t, const AlphaChar * key, TrieData * o_data )
{
    auto it = t->map.find ( key_of ( key ) );
    if ( it == t->map.end () ) return FALSE;
    if ( o_data ) *o_data = it->second;
    return TRUE;
}

Bool trie_store ( Trie * t, const AlphaChar * key, TrieData data )
{
    t->map[ key_of ( key ) ] = data;
    return TRUE;
}

}
