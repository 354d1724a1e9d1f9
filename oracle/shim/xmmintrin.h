/* Portable stand-in for the one SSE intrinsic tools/csr.c uses (a prefetch
 * hint); lets the reference compile on any architecture.  Oracle build only. */
#ifndef GADE_ORACLE_XMMINTRIN_H
#define GADE_ORACLE_XMMINTRIN_H
#define _MM_HINT_T0 3
static inline void _mm_prefetch(const char *p, int hint) { (void)hint; __builtin_prefetch(p); }
#endif
