/* Stand-in for libmceliece's generated crypto_xof_bitwrite16.h. */
#ifndef crypto_xof_bitwrite16_h
#define crypto_xof_bitwrite16_h
#define crypto_xof_bitwrite16 mcref_xof_bitwrite16
extern void crypto_xof_bitwrite16(unsigned char *, long long, const unsigned char *, long long);
#endif
