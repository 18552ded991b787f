/* Stand-in for librandombytes' randombytes.h (same prototype): the reference
 * library's randomness is routed to oracle/ref_harness.c, which serves each
 * calling thread from its own source (a fixed key seed, the per-request seed
 * chain, or the known-answer stream). */
#ifndef randombytes_h
#define randombytes_h
#define randombytes mcref_randombytes
extern void randombytes(void *, long long);
#endif
