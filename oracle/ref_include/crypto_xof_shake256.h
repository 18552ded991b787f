/* Stand-in for libmceliece's generated crypto_xof_shake256.h. */
#ifndef crypto_xof_shake256_h
#define crypto_xof_shake256_h
#define crypto_xof_shake256 mcref_xof_shake256
extern void crypto_xof_shake256(unsigned char *, long long, const unsigned char *, long long);
#endif
