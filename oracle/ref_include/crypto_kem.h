/* Stand-in for the crypto_kem.h that libmceliece's configure script writes
 * per parameter set: maps the KEM's public names into the set's namespace
 * (CRYPTO_NAMESPACE is defined on the compiler command line per set).
 * Used only to compile the reference library as the checker / CPU baseline. */
#ifndef crypto_kem_h
#define crypto_kem_h
#define crypto_kem_keypair CRYPTO_NAMESPACE(keypair)
#define crypto_kem_enc CRYPTO_NAMESPACE(enc)
#define crypto_kem_dec CRYPTO_NAMESPACE(dec)
extern void crypto_kem_keypair(unsigned char *, unsigned char *);
extern int crypto_kem_enc(unsigned char *, unsigned char *, const unsigned char *);
extern int crypto_kem_dec(unsigned char *, const unsigned char *, const unsigned char *);
#endif
