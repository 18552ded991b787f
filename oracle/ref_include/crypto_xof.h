/* Stand-in for libmceliece's generated crypto_xof.h, seen by the xof sources
 * themselves; crypto_xof is renamed per source on the command line. */
#ifndef crypto_xof_h
#define crypto_xof_h
extern void crypto_xof(unsigned char *, long long, const unsigned char *, long long);
#endif
