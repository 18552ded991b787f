/*
 * shim.c -- libmceliece's public keypair / enc / dec entry points (the names
 * declared in oracle/ref_gpu/mceliece.h) over oracle/_ref/libmcref.so.
 *
 * TEST INFRASTRUCTURE ONLY (the reference's GPU benchmark harness links it;
 * the engine never does). libmceliece draws its randomness from the OS; here
 * every call takes a fresh 32-byte seed from a deterministic counter hashed
 * with SHAKE256, so a harness run is repeatable: keypair's single 32-byte
 * draw is that seed, and enc's draws follow libmcref's seed chain from it.
 */
#include <stdint.h>
#include <string.h>

#include "../ref_harness.h"
#include "mceliece.h"

static uint64_t g_calls;

static void next_seed(uint8_t seed[32]) {
  uint8_t in[24] = "gmc reference gpu run";
  memcpy(in + 16, &g_calls, 8);
  g_calls++;
  mcref_shake256(seed, 32, in, (long long)sizeof in);
}

#define GMC_REF_GPU_DEFINE(set, id)                                                          \
  void mceliece_kem_##set##_keypair(unsigned char *pk, unsigned char *sk) {                  \
    uint8_t s[32];                                                                           \
    next_seed(s);                                                                            \
    mcref_keypair(id, pk, sk, s);                                                            \
  }                                                                                          \
  int mceliece_kem_##set##_enc(unsigned char *c, unsigned char *k, const unsigned char *pk) { \
    uint8_t s[32];                                                                           \
    next_seed(s);                                                                            \
    return mcref_enc(id, c, k, pk, s);                                                       \
  }                                                                                          \
  int mceliece_kem_##set##_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk) { \
    return mcref_dec(id, k, c, sk);                                                          \
  }

/* set ids as in oracle/ref_harness.h: the base sets are 0..4 */
GMC_REF_GPU_DEFINE(348864, 0)
GMC_REF_GPU_DEFINE(460896, 1)
GMC_REF_GPU_DEFINE(6688128, 2)
GMC_REF_GPU_DEFINE(6960119, 3)
GMC_REF_GPU_DEFINE(8192128, 4)
