/*
 * ref_harness.h -- entry points of oracle/_ref/libmcref.so: the reference's
 * own CPU implementation (libmceliece-20250507, portable `vec` code) with
 * seeded randomness and threaded batches.  TEST INFRASTRUCTURE AND CPU
 * BASELINE ONLY; the engine never links it.  Set ids as in
 * mceliece_oracle.h (id = s + 5 v).
 */
#ifndef MCREF_HARNESS_H
#define MCREF_HARNESS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCREF_NVARIANTS 20

typedef void (*mcref_rng_fn)(void *ctx, uint8_t *out, long long len);

/* out[8] = m, n, t, mt, k, pk bytes, sk bytes, ct bytes */
int mcref_sizes(int id, long long *out);
const char *mcref_name(int id);
const char *mcref_implementation(void);
void mcref_shake256(uint8_t *out, long long outlen, const uint8_t *in, long long inlen);

int mcref_keypair_rng(int id, uint8_t *pk, uint8_t *sk, mcref_rng_fn rng, void *ctx);
/* keypair whose single 32-byte randombytes draw returns seed32 */
int mcref_keypair(int id, uint8_t *pk, uint8_t *sk, const uint8_t *seed32);
int mcref_enc_rng(int id, uint8_t *c, uint8_t *key, const uint8_t *pk, mcref_rng_fn rng, void *ctx);
/* enc with its randombytes draws taken from the seed chain started at seed32 */
int mcref_enc(int id, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seed32);
int mcref_dec(int id, uint8_t *key, const uint8_t *c, const uint8_t *sk);

int mcref_enc_batch(int id, long long count, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seeds,
                    int *rc, int threads);
int mcref_dec_batch(int id, long long count, uint8_t *key, const uint8_t *c, const uint8_t *sk, int *rc,
                    int threads);

/* libmceliece's known-answer replay (oracle/kat.c) run against the library itself */
int mcref_kat_checksum(int id, int loops, int index_first, char *hex_out);

#ifdef __cplusplus
}
#endif
#endif
