/*
 * kat.c -- replays libmceliece's known-answer test for the KEM on top of the
 * oracle, so the oracle can be compared with the checksums that library
 * publishes (mc:command/mceliece-test.c: test_kem_348864_impl at :4599-4735,
 * checksum table at :4567; the other sets have the same procedure).
 * TEST INFRASTRUCTURE ONLY.
 *
 * Procedure being replayed, per loop: keypair -> checksum(pk), checksum(sk);
 * enc -> checksum(c), checksum(k); dec -> checksum(k'); then three times a
 * ciphertext byte is bumped at a pseudo-random position and the dec result
 * (or the ciphertext itself when dec reports an error) is checksummed.
 * The randomness is the library's "knownrandombytes" stream (ChaCha20 keyed
 * by a rolling 32-byte state, 736 bytes per refill), the test inputs come
 * from a Salsa20 stream keyed by "generate inputs for test vectors", and the
 * checksum is a Salsa20-core chaining over 16-byte blocks.  Primitives are
 * written from the Salsa20 and ChaCha specifications.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#ifdef KAT_FOR_REFERENCE
/* the same replay against libmceliece itself (oracle/build_ref.py compiles
 * this file a second time with KAT_FOR_REFERENCE into libmcref.so) */
#include "ref_harness.h"
#define gmo_sizes mcref_sizes
#define gmo_keypair_rng mcref_keypair_rng
#define gmo_enc_rng mcref_enc_rng
#define gmo_dec mcref_dec
#define gmo_kat_checksum mcref_kat_checksum
#else
#include "mceliece_oracle.h"
#endif

static uint32_t rotl32(uint32_t x, int c) { return (x << c) | (x >> (32 - c)); }
static uint32_t le32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static void put32(uint8_t *p, uint32_t v) { for (int i = 0; i < 4; i++) p[i] = (uint8_t)(v >> (8 * i)); }

static const uint8_t SIGMA[16] = {'e','x','p','a','n','d',' ','3','2','-','b','y','t','e',' ','k'};

/* Salsa20 core (Salsa20 specification, 10 double rounds), 32-byte key k,
 * 16-byte input in; out (64 bytes) may alias k. */
static void salsa_core(uint8_t *out, const uint8_t *in, const uint8_t *k) {
  uint32_t x[16], j[16];
  x[0] = le32(SIGMA); x[5] = le32(SIGMA + 4); x[10] = le32(SIGMA + 8); x[15] = le32(SIGMA + 12);
  for (int i = 0; i < 4; i++) {
    x[1 + i] = le32(k + 4 * i);
    x[11 + i] = le32(k + 16 + 4 * i);
    x[6 + i] = le32(in + 4 * i);
  }
  memcpy(j, x, sizeof x);
#define QR(a, b, c, d)                 \
  x[b] ^= rotl32(x[a] + x[d], 7);      \
  x[c] ^= rotl32(x[b] + x[a], 9);      \
  x[d] ^= rotl32(x[c] + x[b], 13);     \
  x[a] ^= rotl32(x[d] + x[c], 18);
  for (int r = 0; r < 10; r++) {
    QR(0, 4, 8, 12) QR(5, 9, 13, 1) QR(10, 14, 2, 6) QR(15, 3, 7, 11)
    QR(0, 1, 2, 3) QR(5, 6, 7, 4) QR(10, 11, 8, 9) QR(15, 12, 13, 14)
  }
#undef QR
  for (int i = 0; i < 16; i++) put32(out + 4 * i, x[i] + j[i]);
}

/* ChaCha20 block (original 64-bit nonce / 64-bit counter layout). */
static void chacha_core(uint8_t *out, const uint8_t *in16, const uint8_t *k) {
  uint32_t x[16], j[16];
  for (int i = 0; i < 4; i++) { x[i] = le32(SIGMA + 4 * i); x[12 + i] = le32(in16 + 4 * i); }
  for (int i = 0; i < 8; i++) x[4 + i] = le32(k + 4 * i);
  memcpy(j, x, sizeof x);
#define CQ(a, b, c, d)                      \
  x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16); \
  x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12); \
  x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);  \
  x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
  for (int r = 0; r < 10; r++) {
    CQ(0, 4, 8, 12) CQ(1, 5, 9, 13) CQ(2, 6, 10, 14) CQ(3, 7, 11, 15)
    CQ(0, 5, 10, 15) CQ(1, 6, 11, 12) CQ(2, 7, 8, 13) CQ(3, 4, 9, 14)
  }
#undef CQ
  for (int i = 0; i < 16; i++) put32(out + 4 * i, x[i] + j[i]);
}

/* stream: block counter little-endian in the counter half, nonce in the other */
static void stream(uint8_t *c, uint64_t len, const uint8_t *nonce8, const uint8_t *k, int chacha) {
  uint8_t z[16], blk[64];
  memset(z, 0, 16);
  uint8_t *ctr = chacha ? z : z + 8;
  memcpy(chacha ? z + 8 : z, nonce8, 8);
  while (len) {
    if (chacha) chacha_core(blk, z, k); else salsa_core(blk, z, k);
    uint64_t take = len < 64 ? len : 64;
    memcpy(c, blk, take);
    c += take; len -= take;
    for (int i = 0; i < 8; i++) if (++ctr[i]) break;
  }
}

typedef struct {
  uint8_t g[32];
  uint8_t r[736];
  int pos;
  uint8_t tv_nonce[8];
  uint8_t state[64];
} katctx;

/* knownrandombytes: refill r (736 bytes) and roll the key from one ChaCha20
 * stream of 768 bytes whenever r is used up. */
static void known_rng(void *vctx, uint8_t *out, long long len) {
  katctx *K = (katctx *)vctx;
  static const uint8_t zero_nonce[8] = {0};
  while (len > 0) {
    if (K->pos == 736) {
      uint8_t x[32 + 736];
      stream(x, sizeof x, zero_nonce, K->g, 1);
      memcpy(K->g, x, 32);
      memcpy(K->r, x + 32, 736);
      K->pos = 0;
    }
    *out++ = K->r[K->pos];
    K->r[K->pos++] = 0;
    len--;
  }
}

static uint64_t test_random(katctx *K) {
  static const uint8_t key[32] = {'g','e','n','e','r','a','t','e',' ','i','n','p','u','t','s',' ',
                                  'f','o','r',' ','t','e','s','t',' ','v','e','c','t','o','r','s'};
  uint8_t x[8];
  stream(x, 8, K->tv_nonce, key, 0);
  for (int i = 0; i < 8; i++) if (++K->tv_nonce[i]) break;
  uint64_t r = 0;
  for (int i = 7; i >= 0; i--) r = (r << 8) | x[i];
  return r;
}

static void checksum(katctx *K, const uint8_t *x, long long len) {
  uint8_t blk[16];
  while (len >= 16) { salsa_core(K->state, x, K->state); x += 16; len -= 16; }
  memset(blk, 0, 16);
  memcpy(blk, x, (size_t)len);
  blk[len] = 1;
  K->state[0] ^= 1;
  salsa_core(K->state, blk, K->state);
}

/* index_first selects the order in which the two pseudo-random draws of
 * "c[random % clen] += 1 + random % 255" are taken (C leaves it unspecified). */
int gmo_kat_checksum(int set, int loops, int index_first, char *hex_out) {
  long long sz[8];
  if (gmo_sizes(set, sz)) return -1;
  long long plen = sz[5], slen = sz[6], clen = sz[7];
  uint8_t *p = malloc((size_t)plen), *s = malloc((size_t)slen), *c = malloc((size_t)clen);
  uint8_t k[32], t[32];
  katctx K;
  memset(&K, 0, sizeof K);
  K.pos = 736;
  int bad = 0;
  for (int loop = 0; loop < loops; loop++) {
    if (gmo_keypair_rng(set, p, s, known_rng, &K)) { bad = -2; break; }
    checksum(&K, p, plen);
    checksum(&K, s, slen);
    if (gmo_enc_rng(set, c, k, p, known_rng, &K) != 0) { bad = -3; break; }
    checksum(&K, c, clen);
    checksum(&K, k, 32);
    if (gmo_dec(set, t, c, s) != 0 || memcmp(t, k, 32)) { bad = -4; break; }
    checksum(&K, t, 32);
    for (int j = 0; j < 3; j++) {
      uint64_t a, b;
      if (index_first) { a = test_random(&K); b = test_random(&K); }
      else { b = test_random(&K); a = test_random(&K); }
      c[a % (uint64_t)clen] = (uint8_t)(c[a % (uint64_t)clen] + 1 + (b % 255));
      if (gmo_dec(set, t, c, s) == 0) checksum(&K, t, 32);
      else checksum(&K, c, clen);
    }
  }
  for (int i = 0; i < 32; i++) sprintf(hex_out + 2 * i, "%02x", K.state[i]);
  free(p); free(s); free(c);
  return bad;
}
