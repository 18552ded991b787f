/*
 * gmc.h -- C ABI of the GB300 batched Classic McEliece KEM engine
 * (libgmc.so). Plain pointers and sizes only; no framework types.
 *
 * Parameter-set ids: 0 = mceliece348864, 1 = mceliece460896,
 * 2 = mceliece6688128, 3 = mceliece6960119, 4 = mceliece8192128.
 *
 * Return codes: 0 on success, a negative GMC_E* value on failure. Per-request
 * decapsulation status (the 6960119 ciphertext-padding rule) goes to the
 * optional rc[] array, exactly as libmceliece's dec return value.
 *
 * Every entry point runs on the calling thread's current CUDA device. There is
 * no CPU fallback: without a usable GPU the calls return GMC_ECUDA.
 */
#ifndef GMC_H
#define GMC_H

#ifdef __cplusplus
extern "C" {
#endif

#define GMC_OK 0
#define GMC_EINVAL -1   /* bad argument (set id, null pointer, negative n) */
#define GMC_ECUDA -2    /* CUDA error (no device, launch failure, ...) */
#define GMC_ENOMEM -3   /* device allocation failed */
#define GMC_EKEY -4     /* key handle of the wrong kind or a malformed key */

typedef struct gmc_key gmc_key;

/* ---- parameter sets --------------------------------------------------
 * Set id = s + 5 v for parameter set s (0 = 348864, 1 = 460896, 2 = 6688128,
 * 3 = 6960119, 4 = 8192128; gmc_set_count() = 5) and variant v
 * (GMC_NVARIANTS = 20 ids), as libmceliece's crypto_kem/<set><variant>:
 *   v = 0  the set itself;
 *   v = 1  "pc", plaintext confirmation: the same keys; ciphertexts
 *          C0 || C1 with C1 = SHAKE256(2 || e, 32) (32 bytes longer), the
 *          session key hashed over C0 || C1, decapsulation also rejecting
 *          when C1 does not match the decoded e;
 *   v = 2  "f": semi-systematic key generation (different keys, the same
 *          encapsulation and decapsulation as the set);
 *   v = 3  "pcf": both.
 * Every entry point taking a set id or a key accepts all of them. */
#define GMC_NVARIANTS 20
int gmc_set_count(void);
const char *gmc_set_name(int set);
/* looks up "348864", "mceliece348864", "8192128pc", "6960119pcf", ...; returns the id or GMC_EINVAL */
int gmc_set_id(const char *name);
/* out[8] = m, n, t, mt, k, public-key bytes, secret-key bytes, ciphertext bytes */
int gmc_set_sizes(int set, long long *out);

/* ---- resident keys ---------------------------------------------------
 * Replaces, for a batch, the per-call key argument of
 * mceliece_kem_<set>_enc(c,k,pk) / _dec(k,c,sk)
 * (libmceliece api: mc:crypto_kem/348864/vec/wrap_enc.c:4, wrap_dec.c:4;
 * harness use: mceliece-gpu-params/main.cu:19-21, 191-202, 279-323).
 * The key bytes are copied; the caller's buffer may be reused at once. */
int gmc_pk_load(gmc_key **out, int set, const unsigned char *pk);
int gmc_sk_load(gmc_key **out, int set, const unsigned char *sk);
void gmc_key_free(gmc_key *key);
int gmc_key_set(const gmc_key *key);

/* Persistence of a resident key: gmc_key_export writes the key's device state
 * (the tables gmc_pk_load / gmc_sk_load build on the host) as one
 * self-checking byte string and returns its length (buf = NULL: only the
 * length); gmc_key_import re-creates the handle on the current device with
 * plain copies. The string carries the set id, key kind and dimensions and a
 * SHAKE256 checksum; import rejects (GMC_EKEY) anything else. A secret-key
 * string holds the secret key's material: store it as the secret key. */
long long gmc_key_export(const gmc_key *key, unsigned char *buf, long long len);
int gmc_key_import(gmc_key **out, const unsigned char *buf, long long len);

/* ---- batched encapsulation --------------------------------------------
 * n requests against one public key. seeds: n x 32 bytes; request i draws its
 * randomness from the seed chain state_0 = seeds[i], each randombytes call of
 * libmceliece's enc returning SHAKE256({64}||state, len) and advancing
 * state = out[0:32]. With libmceliece's randombytes interposed by that chain
 * the outputs are byte-identical to mceliece_kem_<set>_enc
 * (mc:crypto_kem/348864/vec/encrypt.c:41-90, kem_enc.c:18).
 * c: n x ct bytes, k: n x 32 bytes, rc (optional): n ints (enc return value,
 * -1 only for a 6960119 key with nonzero padding bits, as the library).
 * _dev: all pointers are device pointers, work is queued on `stream`
 * (a cudaStream_t, 0 = default stream) and the call returns without waiting.
 * Without _dev: host pointers; the call copies in, runs and copies out.
 * GMC_SAMPLE_PIPELINE=0 in the environment (read once) selects the
 * lane-per-request sampler instead of the pipelined one (same outputs). */
int gmc_enc_batch_dev(const gmc_key *pk, unsigned char *c, unsigned char *k, const unsigned char *seeds,
                      long long n, int *rc, void *stream);
int gmc_enc_batch(const gmc_key *pk, unsigned char *c, unsigned char *k, const unsigned char *seeds,
                  long long n, int *rc);

/* ---- batched decapsulation ---------------------------------------------
 * n ciphertexts against one secret key (mc:crypto_kem/348864/vec/kem_dec.c:19,
 * implicit rejection; 6960119 padding rule mc:crypto_kem/6960119/vec/kem_dec.c:21).
 * k: n x 32 bytes; rc (optional): per-request dec return value (0, or -1 with
 * k = 0xff..ff for a 6960119 ciphertext whose padding bits are set). */
int gmc_dec_batch_dev(const gmc_key *sk, unsigned char *k, const unsigned char *c, long long n, int *rc,
                      void *stream);
int gmc_dec_batch(const gmc_key *sk, unsigned char *k, const unsigned char *c, long long n, int *rc);

/* ---- key generation -----------------------------------------------------
 * Keys in libmceliece's format (mc:crypto_kem/348864/vec/kem_keypair.c:20):
 * the keypair whose single 32-byte randombytes draw returns seed32.
 * pk/sk buffers of the set's public/secret-key size. Runs on the GPU: the
 * batched key generation below with one key. */
int gmc_keypair_seed(int set, unsigned char *pk, unsigned char *sk, const unsigned char *seed32);

/* Batched key generation on the device: nkeys keypairs, key i from the
 * 32-byte seed seeds + 32 i (the single randombytes draw of libmceliece's
 * keypair, mc:crypto_kem/<set>/vec/kem_keypair.c:36), written to
 * pk + i * pk_bytes and sk + i * sk_bytes (host memory). Every key is
 * byte-identical to gmc_keypair_seed's for the same seed. Each key walks the
 * library's seed chain until an attempt gives an irreducible Goppa
 * polynomial, a repetition-free support and a systematic public key; the
 * attempts run on the GPU (seed expansion, minimal polynomial, support sort,
 * Gaussian elimination, Benes control bits). Environment (optional):
 * GMC_KG_CHUNK_KEYS caps the keys staged on the device per chunk (default:
 * 2 GB of pk + sk), GMC_KG_AHEAD_LINKS the seed-chain links expanded ahead per
 * key (default ln(nkeys)/0.34 + 8); GMC_KG_TRACE=1 prints one line per round. */
int gmc_keypair_batch(int set, unsigned char *pk, unsigned char *sk, const unsigned char *seeds, long long nkeys);

/* ---- grouped launches over many keys and parameter sets -------------------
 * A group is one key's batch: a public key with n seeds (encapsulation) or a
 * secret key with n ciphertexts (decapsulation), device buffers. A plan
 * buckets its groups by (parameter set, enc/dec) into pipelines of up to 16
 * keys, each running the kernels once for all of its keys (uneven counts per
 * key are fine), and captures all pipelines as parallel branches of one CUDA
 * graph; gmc_plan_launch replays it with one cudaGraphLaunch. Outputs land in
 * each group's buffers, identical to per-key gmc_{enc,dec}_batch_dev calls.
 * The plan owns its scratch; the groups' buffers must stay valid while it is
 * launched. (Replaces the per-key launch loop of the reference harness,
 * mceliece-gpu-params/main.cu:228-370.) */
typedef struct gmc_group {
  const gmc_key *key;       /* public key: encapsulation; secret key: decapsulation */
  long long n;              /* requests */
  const unsigned char *in;  /* enc: n x 32 seeds; dec: n x ct ciphertexts */
  unsigned char *ct;        /* enc: n x ct ciphertexts out; dec: unused */
  unsigned char *k;         /* n x 32 session keys out */
  int *rc;                  /* optional n return codes */
} gmc_group;
typedef struct gmc_plan gmc_plan;
int gmc_plan_create(gmc_plan **plan, const gmc_group *groups, int ngroups);
int gmc_plan_launch(gmc_plan *plan, void *stream);
int gmc_plan_info(const gmc_plan *plan, int *pipelines, long long *padded_rows);
void gmc_plan_free(gmc_plan *plan);

/* ---- serving loop (continuous batching) -----------------------------------
 * gmc_server_create: `slots` batches may be in flight at once (each with its
 * own stream, device arena and pinned staging); a batch holds at most
 * max_batch requests and only what fits its arena (arenas take at most
 * mem_fraction of the device memory free at creation: admission by free
 * memory). Keys must be registered (gmc_server_add_key) before requests use
 * them; their device state is completed at registration.
 * gmc_server_submit queues one request with host buffers (in: 32-byte seed for
 * a public key, ciphertext for a secret key; ct out for a public key; k out;
 * optional rc; ciphertexts of pc keys are 32 bytes longer) and returns at
 * once; *done (optional) becomes 1 when the
 * outputs are written (-1 on failure). A dispatcher thread forms each batch
 * from everything queued when a slot frees up, so requests that arrive while
 * others run join the next batch. Results equal the one-request calls.
 * gmc_server_stats out[8]: completed, batches, mean batch size, p50 ms,
 * p99 ms (arrival to completion), ops/s since the first arrival, errors,
 * slots. gmc_server_loadgen drives the server with Poisson arrivals at `rate`
 * requests/s for `seconds` over npairs (public, secret) key pairs, a fraction
 * enc_fraction of them encapsulations, and writes out[8]: submitted,
 * completed, achieved ops/s, p50 ms, p99 ms, mean batch, batches, offered
 * rate. gmc_server_latency_ms gives any quantile q (0 < q <= 1; 1 = the
 * slowest request) of the latencies recorded since the last reset (the
 * histogram's buckets are 2% wide). gmc_server_worst_batch writes out[10] for
 * the batch whose oldest request had the longest latency since the last
 * reset: that latency, then its parts in ms (waiting in the queue for a free
 * slot, moving the requests out of the queue, grouping them by key with the
 * admission check, copying the inputs into pinned staging, issuing copies and
 * kernels, device work with the copies and the completion callback, scattering
 * the results), then the number of batches and of batches over 5 ms. */
typedef struct gmc_server gmc_server;
int gmc_server_create(gmc_server **server, long long max_batch, int slots, double mem_fraction);
int gmc_server_add_key(gmc_server *server, const gmc_key *key);
int gmc_server_submit(gmc_server *server, const gmc_key *key, const unsigned char *in, unsigned char *ct,
                      unsigned char *k, int *rc, int *done);
int gmc_server_drain(gmc_server *server, double timeout_s);
int gmc_server_stats(gmc_server *server, double *out);
int gmc_server_reset_stats(gmc_server *server);
int gmc_server_latency_ms(gmc_server *server, double q, double *ms);
int gmc_server_worst_batch(gmc_server *server, double *out);
int gmc_server_loadgen(gmc_server *server, const gmc_key *const *pks, const gmc_key *const *sks, int npairs,
                       double rate, double seconds, double enc_fraction, unsigned long long seed, double *out);
void gmc_server_destroy(gmc_server *server);
/* message of the server's last failed batch ("" if none) */
const char *gmc_server_error(gmc_server *server);

/* ---- libmceliece calling convention (one request per call) --------------
 * Same signatures and results as mceliece_kem_<set>_enc / _dec
 * (mc:crypto_kem/<set>/vec/wrap_keypair.c:4, wrap_enc.c:4, wrap_dec.c:4). keypair
 * and enc draw one 32-byte seed each from the randombytes source; enc draws
 * seed from the randombytes source (default: the OS generator) and runs the
 * GPU seed chain. dec tolerates k == c and k == sk (outputs written last). */
void gmc_kem_348864_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_348864_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_348864_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_460896_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_460896_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_460896_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6688128_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6688128_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6688128_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6960119_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6960119_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6960119_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_8192128_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_8192128_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_8192128_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
/* plaintext-confirmation variants (mc:crypto_kem/<set>pc/vec/wrap_{keypair,enc,dec}.c) */
void gmc_kem_348864pc_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_348864pc_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_348864pc_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_460896pc_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_460896pc_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_460896pc_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6688128pc_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6688128pc_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6688128pc_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6960119pc_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6960119pc_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6960119pc_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_8192128pc_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_8192128pc_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_8192128pc_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
/* semi-systematic key generation (mc:crypto_kem/<set>f, <set>pcf) */
void gmc_kem_348864f_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_348864f_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_348864f_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_460896f_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_460896f_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_460896f_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6688128f_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6688128f_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6688128f_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6960119f_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6960119f_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6960119f_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_8192128f_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_8192128f_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_8192128f_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_348864pcf_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_348864pcf_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_348864pcf_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_460896pcf_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_460896pcf_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_460896pcf_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6688128pcf_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6688128pcf_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6688128pcf_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_6960119pcf_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_6960119pcf_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_6960119pcf_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);
void gmc_kem_8192128pcf_keypair(unsigned char *pk, unsigned char *sk);
int gmc_kem_8192128pcf_enc(unsigned char *c, unsigned char *k, const unsigned char *pk);
int gmc_kem_8192128pcf_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);

/* randombytes source of the one-request keypair and enc entry points
 * (librandombytes' randombytes(), rb:include/randombytes.h:10). NULL restores
 * the OS generator. */
typedef void (*gmc_randombytes_fn)(void *ctx, unsigned char *out, long long len);
void gmc_set_randombytes(gmc_randombytes_fn fn, void *ctx);

/* ---- engine selection and diagnostics ----------------------------------- */
#define GMC_GEMM_POPC 0   /* CUDA-core AND/XOR + popcount */
#define GMC_GEMM_B1MMA 1  /* legacy mma.sync m8n8k128 .b1 AND.POPC */
#define GMC_GEMM_TC 2     /* tcgen05 (5th-gen tensor cores), 0/1 operands in FP8, TMEM accumulators */
#define GMC_GEMM_SPARSE 3 /* encapsulation only: XOR of the public-key columns at e's t positions,
                             gathered by the sampler (no GEMM launch); the default there */
/* Forces one engine for every set (-1 restores the per-set choices);
 * GMC_GEMM_SPARSE applies to the encapsulation syndrome only (the
 * decapsulation front end keeps its per-set GEMM engine).
 * gmc_get_gemm_engine returns the override or -1. */
int gmc_set_gemm_engine(int engine);
int gmc_get_gemm_engine(void);

/* Constant-time decapsulation (no counterpart in the reference, whose device
 * code disclaims side channels; libmceliece's own CPU code is constant-time).
 * on = 1: Berlekamp-Massey runs inversion-free with no tables and slot
 * counts fixed by the iteration alone (the same locators, normalized by one
 * bit-sliced inversion), and the root finder's top-down pass multiplies by
 * table-free columns of its public constants; 0 restores the table forms.
 * Session keys are identical either way. Process-wide, read at each batch
 * launch; GMC_DEC_CT=1 in the environment sets it at load. The
 * no-allocation entry point keeps the table forms. */
int gmc_set_dec_constant_time(int on);
int gmc_get_dec_constant_time(void);

/* ---- autotuner --------------------------------------------------------------
 * Per parameter set: the engine of the encapsulation syndrome (sparse or a
 * GEMM engine) and the GEMM engine of the decapsulation front end, and the
 * sampler block size (32/64/128). Defaults: sparse, tcgen05, 128. gmc_autotune times every candidate on this GPU with a
 * batch of n requests (median of 5), keeps the fastest and, when cache_path is
 * given, writes the choices of all tuned sets to that JSON file;
 * gmc_autotune_load applies such a file (returns the number of sets loaded).
 * gmc_tune_get returns 1 when the set's configuration was tuned or loaded.
 * The launch shape is tuned with them: the tcgen05 GEMM's pipeline depth
 * (gemm_stages 2..4 A/X buffers per CTA, default 4) and the requests per block
 * of the decoding kernels (bm_warps: Berlekamp-Massey warps of 32 requests,
 * 1..14, default 14, the constant-time form using at most 8; root_warps:
 * root-finding warps of one request, 1..8, default 8) and the
 * pipelined sampler's resident warps per SM (sample_sm_warps, 0 = as many as
 * fit, the default); gmc_tune_set_launch / gmc_tune_get_launch set and read
 * them by hand. */
int gmc_autotune(int set, long long n, const char *cache_path);
int gmc_autotune_load(const char *cache_path);
int gmc_tune_set(int set, int enc_engine, int dec_engine, int sample_threads);
int gmc_tune_get(int set, int *enc_engine, int *dec_engine, int *sample_threads);
int gmc_tune_set_launch(int set, int gemm_stages, int bm_warps, int root_warps, int sample_sm_warps);
int gmc_tune_get_launch(int set, int *gemm_stages, int *bm_warps, int *root_warps, int *sample_sm_warps);
/* Reads and clears the tensor-core engine's error word on the current device:
 * 1 when a CTA gave up on a bounded wait (its outputs are then invalid). */
int gmc_tc_status(void);
/* Measured integer-pipe rates of this GPU (lane-ops per second): 3-input
 * logic ops (lop3) and 32-bit funnel shifts, the instruction kinds of a
 * Keccak-f[1600] permutation on 32-bit halves. For the Keccak ceiling. */
int gmc_int32_peak(double *lop3_per_s, double *shf_per_s);
/* Measured rate of the GF(2) GEMM engine's tensor-core instruction
 * (tcgen05.mma .kind::f8f6f4, E4M3, M = 128, N = 256, K = 32, FP32
 * accumulator in tensor memory) with its operands resident in shared memory:
 * multiply-accumulates per second on the current device (the denominator of
 * the engine's tensor-pipe fraction). */
int gmc_tc_f8_peak(double *mac_per_s);
/* Measured rate of the legacy 1-bit tensor instruction the GMC_GEMM_B1MMA
 * engine issues (mma.sync m8n8k128 .b1 AND.POPC, register operands): bit
 * multiply-accumulates per second on the current device. */
int gmc_b1mma_peak(double *mac_per_s);

/* Stage outputs of a decapsulation batch (device pointers): the 2t packed
 * syndromes (s_words per request), the error vectors (e_words per request)
 * and the decode flags. For the staged parity tests. */
int gmc_dec_stages_dev(const gmc_key *sk, const unsigned char *c, long long n, unsigned int *synd,
                       int synd_words, unsigned int *e, int e_words, int *ok, void *stream);
/* Stage outputs of an encapsulation batch: error vectors and raw syndromes
 * T*e[mt:n] (device pointers). */
int gmc_enc_stages_dev(const gmc_key *pk, const unsigned char *seeds, long long n, unsigned int *e,
                       int e_words, unsigned int *synd, int synd_words, void *stream);
/* Raw GF(2) product Out[i] = A * X[i] on the selected engine (device
 * pointers, layouts as documented in the engine: rows_pad % 128 == 0,
 * kw_pad % 8 == 0, n_pad % 256 == 0, lda/ldx >= kw_pad; X has n_pad rows). */
int gmc_gf2_gemm_dev(int engine, const unsigned int *A, int lda, int rows_pad, const unsigned int *X, int ldx,
                     long long n_pad, int kw_pad, unsigned int *out, int ldo, int out_words, long long n,
                     void *stream);

/* ---- batched decapsulation without device allocation --------------------
 * No counterpart in the reference. For callers that cannot call cudaMalloc:
 * a process whose device memory belongs to another allocator with a fixed
 * budget, or a latency-critical path where cudaMalloc/cudaFree would
 * synchronize the device. Same inputs, outputs and results as
 * gmc_dec_batch_dev (device pointers, caller stream), but all intermediates
 * live in a fixed file-scope device array of about 7.6 MiB (plus 330 KB of
 * field tables) that every GPU loading the library keeps until exit; the
 * front-end product runs on the CUDA-core engine. At most
 * GMC_NOALLOC_MAX_REQUESTS ciphertexts per call (larger n: GMC_EINVAL).
 * The first call on a device does a one-time set-up (symbol lookup and a
 * synchronous table copy): make it before any stream capture. The key must
 * have been loaded on the current device (GMC_EKEY otherwise). Calls share the
 * array: calls that overlap on the GPU race, so order them on one stream. */
#define GMC_NOALLOC_MAX_REQUESTS 4096
int gmc_dec_batch_noalloc(const gmc_key *sk, unsigned char *k, const unsigned char *c, long long n, int *rc,
                          void *stream);

/* Host-only views of the per-key / per-field tables the engine uploads (no
 * GPU needed): support L[n], L_i^(2^d) [n], front-end matrix F (returns its
 * word count; *ldf = its row stride), GF(2^m) exp[2q-1]/log[q] and the
 * additive-FFT constants (alpha_log[q], twist_log[2^(d+1)]). */
int gmc_host_sk_tables(int set, const unsigned char *sk, unsigned short *L, unsigned short *Lpow, unsigned int *F,
                       long long f_words, int *ldf);
int gmc_host_field_tables(int set, unsigned short *gexp, unsigned short *glog, unsigned short *alpha_log,
                          unsigned short *twist_log);

/* Per-kernel device timing of the batches launched while enabled (events
 * recorded on the launching stream around every kernel; not during stream
 * capture). gmc_prof_enable(1) clears previous records. gmc_prof_report
 * writes lines "<kernel> <launches> <total ms>" and returns the kernel count. */
int gmc_prof_enable(int on);
int gmc_prof_report(char *buf, int len);

const char *gmc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
