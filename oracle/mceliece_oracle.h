/*
 * mceliece_oracle.h -- the CPU checker for the GPU Classic McEliece engine.
 * Test infrastructure only (tests, smoke check, CPU-baseline leg of the
 * benchmark); the engine in tensormceliece_gb300/ never links it.
 *
 * Parameter-set ids: 0 = 348864, 1 = 460896, 2 = 6688128, 3 = 6960119,
 * 4 = 8192128.
 */
#ifndef GMO_MCELIECE_ORACLE_H
#define GMO_MCELIECE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GMO_NSETS 5
#define GMO_NVARIANTS 20 /* id s + GMO_NSETS v: set s, variant v = 0 plain, 1 pc, 2 f, 3 pcf */
#define GMO_MAX_N 8192
#define GMO_MAX_T 128
#define GMO_MAX_M 13
#define GMO_MAX_MT (GMO_MAX_M * GMO_MAX_T)

/* randombytes replacement: fills out[0..len) */
typedef void (*gmo_rng_fn)(void *ctx, uint8_t *out, long long len);

/* out[8] = m, n, t, mt, k, pk bytes, sk bytes, ct bytes */
int gmo_sizes(int set, long long *out);

void gmo_shake256(uint8_t *out, long long outlen, const uint8_t *in, long long inlen);

/* The per-request seed chain: SHAKE256({64}||state, len), state <- out[0:32]. */
void gmo_chain_randombytes(void *ctx, uint8_t *out, long long len);

int gmo_keypair_rng(int set, uint8_t *pk, uint8_t *sk, gmo_rng_fn rng, void *ctx);
/* keygen whose single 32-byte randombytes draw returns seed32 */
int gmo_keypair(int set, uint8_t *pk, uint8_t *sk, const uint8_t *seed32);

int gmo_gen_e_rng(int set, uint8_t *e, gmo_rng_fn rng, void *ctx, uint16_t *ind_out);
int gmo_gen_e(int set, uint8_t *e, const uint8_t *seed32);
int gmo_syndrome(int set, uint8_t *s, const uint8_t *pk, const uint8_t *e);

int gmo_enc_rng(int set, uint8_t *c, uint8_t *key, const uint8_t *pk, gmo_rng_fn rng, void *ctx);
int gmo_enc(int set, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seed32);
int gmo_dec(int set, uint8_t *key, const uint8_t *c, const uint8_t *sk);

/* stage outputs: s_priv[2t], locator[t+1], e[n/8]; returns 0 on decode success */
int gmo_decrypt_stages(int set, const uint8_t *sk, const uint8_t *c, uint16_t *s_priv, uint16_t *locator,
                       uint8_t *e);
/* support L[n] and 1/g(L_i)^2 [n] (w2 may be NULL) */
int gmo_support(int set, const uint8_t *sk, uint16_t *L_out, uint16_t *w2_out);
int gmo_gf_mul(int m, int a, int b);
/* Benes control bits of pi (2^w entries), the keygen recursion */
int gmo_controlbits(uint8_t *out, const int16_t *pi, int w);

/* threaded batches (CPU baseline and fixture generation) */
int gmo_enc_batch(int set, long long count, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seeds,
                  int *rc, int threads);
int gmo_dec_batch(int set, long long count, uint8_t *key, const uint8_t *c, const uint8_t *sk, int *rc,
                  int threads);

/* libmceliece known-answer replay (oracle/kat.c): writes the 64-hex checksum */
int gmo_kat_checksum(int set, int loops, int index_first, char *hex_out);

#ifdef __cplusplus
}
#endif
#endif
