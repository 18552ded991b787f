/*
 * ref_harness.c -- drives the reference's own CPU implementation of the KEM,
 * libmceliece-20250507's portable `vec` code (crypto_kem/<set>/vec), compiled
 * from the reference's bundled tarball by oracle/build_ref.py into
 * oracle/_ref/libmcref.so.
 *
 * TEST INFRASTRUCTURE AND CPU BASELINE ONLY: loaded by tests/, by the
 * cpu_baseline / --impl reference legs of bench.py and by its parity check,
 * never by the engine.
 *
 * Randomness.  The library draws randomness through randombytes(), which
 * oracle/ref_include/randombytes.h routes to mcref_randombytes() below.  Each
 * thread serves it from its own source, so batches run threaded:
 *   keypair   -- the single 32-byte draw of kem_keypair.c:36 returns the seed;
 *   enc       -- every draw (one per gen_e attempt, encrypt.c:42) comes from
 *                the per-request seed chain out = SHAKE256({64} || state, len),
 *                state = out[0:32] (the same stream the GPU sampler uses);
 *   KAT       -- the known-answer stream of oracle/kat.c.
 *
 * Set ids follow the oracle: id = s + 5 v, s in 348864, 460896, 6688128,
 * 6960119, 8192128; v = 0 plain, 1 pc, 2 f, 3 pcf.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "ref_harness.h"

/* ------------------------------------------------ the library's entry points */

#define DECL(S)                                                                         \
  void mcref_##S##_keypair(unsigned char *, unsigned char *);                          \
  int mcref_##S##_enc(unsigned char *, unsigned char *, const unsigned char *);        \
  int mcref_##S##_dec(unsigned char *, const unsigned char *, const unsigned char *);
#define DECL4(S) DECL(S) DECL(S##pc) DECL(S##f) DECL(S##pcf)
DECL4(348864)
DECL4(460896)
DECL4(6688128)
DECL4(6960119)
DECL4(8192128)

void mcref_xof_shake256(unsigned char *, long long, const unsigned char *, long long);

typedef struct {
  const char *name;
  void (*keypair)(unsigned char *, unsigned char *);
  int (*enc)(unsigned char *, unsigned char *, const unsigned char *);
  int (*dec)(unsigned char *, const unsigned char *, const unsigned char *);
} kem;

#define ROW(S) {#S, mcref_##S##_keypair, mcref_##S##_enc, mcref_##S##_dec}
static const kem KEMS[MCREF_NVARIANTS] = {
    ROW(348864),   ROW(460896),   ROW(6688128),   ROW(6960119),   ROW(8192128),
    ROW(348864pc), ROW(460896pc), ROW(6688128pc), ROW(6960119pc), ROW(8192128pc),
    ROW(348864f),  ROW(460896f),  ROW(6688128f),  ROW(6960119f),  ROW(8192128f),
    ROW(348864pcf), ROW(460896pcf), ROW(6688128pcf), ROW(6960119pcf), ROW(8192128pcf),
};

/* m, n, t, mt, k, pk bytes, sk bytes, ct bytes of the plain sets (the library's api table) */
static const long long SIZES[5][8] = {
    {12, 3488, 64, 768, 2720, 261120, 6492, 96},
    {13, 4608, 96, 1248, 3360, 524160, 13608, 156},
    {13, 6688, 128, 1664, 5024, 1044992, 13932, 208},
    {13, 6960, 119, 1547, 5413, 1047319, 13948, 194},
    {13, 8192, 128, 1664, 6528, 1357824, 14120, 208},
};

int mcref_sizes(int id, long long *out) {
  if (id < 0 || id >= MCREF_NVARIANTS) return -1;
  memcpy(out, SIZES[id % 5], sizeof SIZES[0]);
  int v = id / 5;
  if (v == 1 || v == 3) out[7] += 32; /* plaintext confirmation appends C1 */
  return 0;
}

const char *mcref_name(int id) { return (id >= 0 && id < MCREF_NVARIANTS) ? KEMS[id].name : NULL; }

const char *mcref_implementation(void) {
  return "libmceliece-20250507 crypto_kem/<set>/vec (portable C; gcc -O2 -fwrapv)";
}

/* ------------------------------------------------------------ randomness */

static __thread mcref_rng_fn t_rng;
static __thread void *t_ctx;

void mcref_randombytes(void *out, long long len) {
  if (t_rng) {
    t_rng(t_ctx, (uint8_t *)out, len);
  } else {
    /* no source set: a library call outside the harness's entry points */
    fprintf(stderr, "mcref: randombytes called with no source\n");
    memset(out, 0, (size_t)len);
  }
}

void mcref_shake256(uint8_t *out, long long outlen, const uint8_t *in, long long inlen) {
  mcref_xof_shake256(out, outlen, in, inlen);
}

static void chain_rng(void *ctx, uint8_t *out, long long len) {
  uint8_t *state = (uint8_t *)ctx;
  uint8_t in[33], tmp[32];
  in[0] = 64;
  memcpy(in + 1, state, 32);
  if (len >= 32) {
    mcref_xof_shake256(out, len, in, 33);
    memcpy(state, out, 32);
  } else {
    mcref_xof_shake256(tmp, 32, in, 33);
    memcpy(out, tmp, (size_t)len);
    memcpy(state, tmp, 32);
  }
}

typedef struct {
  const uint8_t *seed;
  int used;
} seedctx;

static void seed_rng(void *ctx, uint8_t *out, long long len) {
  seedctx *s = (seedctx *)ctx;
  if (s->used || len != 32) {
    fprintf(stderr, "mcref: keypair drew %lld bytes beyond its 32-byte seed\n", len);
    memset(out, 0, (size_t)len);
    return;
  }
  memcpy(out, s->seed, 32);
  s->used = 1;
}

/* ------------------------------------------------------------ single calls */

int mcref_keypair_rng(int id, uint8_t *pk, uint8_t *sk, mcref_rng_fn rng, void *ctx) {
  if (id < 0 || id >= MCREF_NVARIANTS) return -1;
  mcref_rng_fn pr = t_rng;
  void *pc = t_ctx;
  t_rng = rng;
  t_ctx = ctx;
  KEMS[id].keypair(pk, sk);
  t_rng = pr;
  t_ctx = pc;
  return 0;
}

int mcref_keypair(int id, uint8_t *pk, uint8_t *sk, const uint8_t *seed32) {
  seedctx s = {seed32, 0};
  return mcref_keypair_rng(id, pk, sk, seed_rng, &s);
}

int mcref_enc_rng(int id, uint8_t *c, uint8_t *key, const uint8_t *pk, mcref_rng_fn rng, void *ctx) {
  if (id < 0 || id >= MCREF_NVARIANTS) return -100;
  mcref_rng_fn pr = t_rng;
  void *pc = t_ctx;
  t_rng = rng;
  t_ctx = ctx;
  int r = KEMS[id].enc(c, key, pk);
  t_rng = pr;
  t_ctx = pc;
  return r;
}

int mcref_enc(int id, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seed32) {
  uint8_t state[32];
  memcpy(state, seed32, 32);
  return mcref_enc_rng(id, c, key, pk, chain_rng, state);
}

int mcref_dec(int id, uint8_t *key, const uint8_t *c, const uint8_t *sk) {
  if (id < 0 || id >= MCREF_NVARIANTS) return -100;
  return KEMS[id].dec(key, c, sk);
}

/* ------------------------------------------------------------ threaded batches */

typedef struct {
  int id, op;
  long long lo, hi, ct_bytes;
  uint8_t *out_c, *out_k;
  const uint8_t *in_c, *key, *seeds;
  int *rc;
} job;

static void *worker(void *arg) {
  job *J = (job *)arg;
  for (long long i = J->lo; i < J->hi; i++) {
    int r;
    if (J->op == 0)
      r = mcref_enc(J->id, J->out_c + i * J->ct_bytes, J->out_k + 32 * i, J->key, J->seeds + 32 * i);
    else
      r = mcref_dec(J->id, J->out_k + 32 * i, J->in_c + i * J->ct_bytes, J->key);
    if (J->rc) J->rc[i] = r;
  }
  return NULL;
}

static int run_batch(const job *base, long long count, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 512) threads = 512;
  pthread_t th[512];
  job jobs[512];
  long long per = (count + threads - 1) / threads;
  int used = 0, err = 0;
  for (int i = 0; i < threads; i++) {
    jobs[i] = *base;
    jobs[i].lo = i * per;
    jobs[i].hi = (i + 1) * per < count ? (i + 1) * per : count;
    if (jobs[i].lo >= jobs[i].hi) break;
    if (pthread_create(&th[i], NULL, worker, &jobs[i])) {
      err = -1;
      break;
    }
    used++;
  }
  for (int i = 0; i < used; i++) pthread_join(th[i], NULL);
  return err;
}

int mcref_enc_batch(int id, long long count, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seeds,
                    int *rc, int threads) {
  long long sz[8];
  if (mcref_sizes(id, sz)) return -1;
  job J;
  memset(&J, 0, sizeof J);
  J.id = id; J.op = 0; J.ct_bytes = sz[7]; J.out_c = c; J.out_k = key; J.key = pk; J.seeds = seeds; J.rc = rc;
  return run_batch(&J, count, threads);
}

int mcref_dec_batch(int id, long long count, uint8_t *key, const uint8_t *c, const uint8_t *sk, int *rc,
                    int threads) {
  long long sz[8];
  if (mcref_sizes(id, sz)) return -1;
  job J;
  memset(&J, 0, sizeof J);
  J.id = id; J.op = 1; J.ct_bytes = sz[7]; J.out_k = key; J.in_c = c; J.key = sk; J.rc = rc;
  return run_batch(&J, count, threads);
}
