/*
 * mceliece_oracle.c -- CPU restatement of the Classic McEliece KEM for the five
 * parameter sets (348864, 460896, 6688128, 6960119, 8192128), with the exact
 * input/output semantics of libmceliece-20250507.
 *
 * THIS IS TEST INFRASTRUCTURE. It is the checker for the GPU engine: only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 * The GPU engine never calls into it.
 *
 * Parity pin: oracle/kat.c replays libmceliece's own known-answer procedure
 * (command/mceliece-test.c, test_kem_<set>_impl) on top of these functions and
 * compares against the checksums published there; tests/test_oracle_kat.py
 * runs it for all five sets.
 *
 * Citations use paths inside the bundled tarball
 * deps/libmceliece-20250507.tar.gz (prefix "mc:") and inside the reference
 * project (mceliece-gpu-params/..., the device port of the same library).
 *
 * Written from the published algorithm (Classic McEliece specification, the
 * Nassimi-Sahni/Bernstein control-bit algorithm) in a plain, non-bitsliced
 * style; it is not a transcription of the vec or avx implementations.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#include "mceliece_oracle.h"

typedef uint16_t gf;

/* ---------------------------------------------------------------- sets */

typedef struct { int pos; int times_z; } ext_tap;

typedef struct {
  const char *name;
  int m, n, t;
  int ntaps;          /* y^t = sum of taps (times z when times_z) */
  ext_tap taps[4];
} setdef;

/* Extension-field reduction polynomials: mc:crypto_kem/<set>/vec/gf_2mt_mul.c
 * (GF_mul).  348864: y^64 = y^3 + y + z;  460896: y^96 = y^10 + y^9 + y^6 + 1;
 * 6688128 and 8192128: y^128 = y^7 + y^2 + y + 1;  6960119: y^119 = y^8 + 1. */
static const setdef SETS[GMO_NSETS] = {
  {"348864", 12, 3488, 64, 3, {{3, 0}, {1, 0}, {0, 1}}},
  {"460896", 13, 4608, 96, 4, {{10, 0}, {9, 0}, {6, 0}, {0, 0}}},
  {"6688128", 13, 6688, 128, 4, {{7, 0}, {2, 0}, {1, 0}, {0, 0}}},
  {"6960119", 13, 6960, 119, 2, {{8, 0}, {0, 0}}},
  {"8192128", 13, 8192, 128, 4, {{7, 0}, {2, 0}, {1, 0}, {0, 0}}},
};

typedef struct {
  int m, n, t, mt, k, q; /* q = 2^m */
  int pk_row_bytes, synd_bytes, cond_bytes, irr_bytes, e_bytes;
  long pk_bytes, sk_bytes;
  int pc;       /* plaintext-confirmation variant: c = C0 || C1 */
  int f;        /* semi-systematic key generation ("f" variants) */
  int ct_bytes; /* synd_bytes, + 32 with plaintext confirmation */
} sizes;

/* Set id = s + GMO_NSETS * v for parameter set s and variant v: 0 the set
 * itself, 1 "pc" (mc:crypto_kem/<set>pc: the same keys, ciphertexts C0 || C1
 * with C1 = SHAKE256(2 || e, 32)), 2 "f" (mc:crypto_kem/<set>f: semi-systematic
 * key generation, the same enc/dec), 3 "pcf" (both). */
static int get_sizes(int set, sizes *P) {
  if (set < 0 || set >= GMO_NVARIANTS) return -1;
  const setdef *S = &SETS[set % GMO_NSETS];
  P->m = S->m; P->n = S->n; P->t = S->t;
  P->mt = S->m * S->t;
  P->k = S->n - P->mt;
  P->q = 1 << S->m;
  P->pk_row_bytes = (P->k + 7) / 8;
  P->synd_bytes = (P->mt + 7) / 8;
  P->cond_bytes = (1 << (S->m - 4)) * (2 * S->m - 1);
  P->irr_bytes = 2 * S->t;
  P->e_bytes = S->n / 8;
  P->pk_bytes = (long)P->mt * P->pk_row_bytes;
  P->sk_bytes = 40 + P->irr_bytes + P->cond_bytes + P->e_bytes;
  P->pc = (set / GMO_NSETS) & 1;
  P->f = (set / GMO_NSETS) >> 1;
  P->ct_bytes = P->synd_bytes + (P->pc ? 32 : 0);
  return 0;
}

int gmo_sizes(int set, long long *out /* [8] */) {
  sizes P;
  if (get_sizes(set, &P)) return -1;
  out[0] = P.m; out[1] = P.n; out[2] = P.t; out[3] = P.mt; out[4] = P.k;
  out[5] = P.pk_bytes; out[6] = P.sk_bytes; out[7] = P.ct_bytes;
  return 0;
}

/* ---------------------------------------------------------------- GF(2^m) */

/* Field polynomials: m=12 x^12+x^3+1, m=13 x^13+x^4+x^3+x+1
 * (mc:crypto_kem/348864/vec/gf_2m_mul.c, mc:crypto_kem/8192128/vec/gf_2m_mul.c).
 * Multiplication by log/antilog tables over a generator found at start-up. */
typedef struct {
  int m; int q; gf mask;
  uint32_t poly;
  gf *exp; /* 2q entries */
  int *log;
} field;

static field FIELD[2];
static pthread_once_t init_once = PTHREAD_ONCE_INIT;

static gf clmul_mod(gf a, gf b, int m, uint32_t poly) {
  uint32_t acc = 0;
  for (int i = 0; i < m; i++)
    if ((b >> i) & 1) acc ^= (uint32_t)a << i;
  for (int i = 2 * m - 2; i >= m; i--)
    if ((acc >> i) & 1) acc ^= poly << (i - m);
  return (gf)acc;
}

static void field_init(field *F, int m, uint32_t poly) {
  F->m = m; F->q = 1 << m; F->mask = (gf)(F->q - 1); F->poly = poly;
  F->exp = (gf *)malloc(sizeof(gf) * 2 * F->q);
  F->log = (int *)malloc(sizeof(int) * F->q);
  for (gf g = 2;; g++) {
    gf x = 1; int order = 0;
    do { x = clmul_mod(x, g, m, poly); order++; } while (x != 1 && order < F->q);
    if (order == F->q - 1) {
      x = 1;
      for (int i = 0; i < F->q - 1; i++) { F->exp[i] = x; F->log[x] = i; x = clmul_mod(x, g, m, poly); }
      for (int i = F->q - 1; i < 2 * F->q; i++) F->exp[i] = F->exp[i - (F->q - 1)];
      F->log[0] = -1;
      break;
    }
  }
}

static inline gf fmul(const field *F, gf a, gf b) {
  if (!a || !b) return 0;
  return F->exp[F->log[a] + F->log[b]];
}
static inline gf finv(const field *F, gf a) { /* 0 -> 0, as a^(2^m-2) */
  if (!a) return 0;
  return F->exp[(F->q - 1 - F->log[a]) % (F->q - 1)];
}

/* ---------------------------------------------------------------- Keccak */

static uint64_t KRC[24];
static int KRHO[25];

static void keccak_consts(void) {
  uint8_t r = 1; /* LFSR x^8+x^6+x^5+x^4+1, FIPS 202 algorithm 5 */
  for (int ir = 0; ir < 24; ir++) {
    uint64_t c = 0;
    for (int j = 0; j < 7; j++) {
      if (r & 1) c |= 1ULL << ((1 << j) - 1);
      r = (uint8_t)((r << 1) ^ ((r & 0x80) ? 0x71 : 0));
    }
    KRC[ir] = c;
  }
  int x = 1, y = 0;
  KRHO[0] = 0;
  for (int t = 0; t < 24; t++) {
    KRHO[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
    int nx = y, ny = (2 * x + 3 * y) % 5;
    x = nx; y = ny;
  }
}

static inline uint64_t rol64(uint64_t v, int r) { return r ? (v << r) | (v >> (64 - r)) : v; }

static void keccak_f1600(uint64_t s[25]) {
  uint64_t C[5], D[5], B[25];
  for (int round = 0; round < 24; round++) {
    for (int x = 0; x < 5; x++) C[x] = s[x] ^ s[x + 5] ^ s[x + 10] ^ s[x + 15] ^ s[x + 20];
    for (int x = 0; x < 5; x++) D[x] = C[(x + 4) % 5] ^ rol64(C[(x + 1) % 5], 1);
    for (int i = 0; i < 25; i++) s[i] ^= D[i % 5];
    for (int x = 0; x < 5; x++)
      for (int y = 0; y < 5; y++)
        B[y + 5 * ((2 * x + 3 * y) % 5)] = rol64(s[x + 5 * y], KRHO[x + 5 * y]);
    for (int y = 0; y < 5; y++)
      for (int x = 0; x < 5; x++)
        s[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
    s[0] ^= KRC[round];
  }
}

static void global_init(void) {
  keccak_consts();
  field_init(&FIELD[0], 12, 0x1009);
  field_init(&FIELD[1], 13, 0x201B);
}
static void ensure_init(void) { pthread_once(&init_once, global_init); }

/* SHAKE256 (rate 136 bytes, domain byte 0x1F): the crypto_xof_shake256 and
 * crypto_hash_32b primitive of mc:crypto_kem/348864/vec/hash.h. */
void gmo_shake256(uint8_t *out, long long outlen, const uint8_t *in, long long inlen) {
  ensure_init();
  uint64_t s[25];
  uint8_t block[136];
  memset(s, 0, sizeof s);
  while (inlen >= 136) {
    for (int i = 0; i < 17; i++) {
      uint64_t w = 0;
      for (int b = 0; b < 8; b++) w |= (uint64_t)in[8 * i + b] << (8 * b);
      s[i] ^= w;
    }
    keccak_f1600(s);
    in += 136; inlen -= 136;
  }
  memset(block, 0, sizeof block);
  memcpy(block, in, (size_t)inlen);
  block[inlen] ^= 0x1F;
  block[135] ^= 0x80;
  for (int i = 0; i < 17; i++) {
    uint64_t w = 0;
    for (int b = 0; b < 8; b++) w |= (uint64_t)block[8 * i + b] << (8 * b);
    s[i] ^= w;
  }
  for (;;) {
    keccak_f1600(s);
    long long take = outlen < 136 ? outlen : 136;
    for (long long j = 0; j < take; j++) out[j] = (uint8_t)(s[j / 8] >> (8 * (j % 8)));
    out += take; outlen -= take;
    if (!outlen) break;
  }
}

/* ---------------------------------------------------------------- randomness */

/* The seed chain every GPU encapsulation uses, and that libmceliece reproduces
 * when its randombytes is interposed: each call returns
 * SHAKE256({64} || state, len) and the state becomes the first 32 output
 * bytes (mceliece-gpu-params/ref/348864.cuh:3434-3487, gen_e). */
void gmo_chain_randombytes(void *ctx, uint8_t *out, long long len) {
  uint8_t *state = (uint8_t *)ctx; /* 32 bytes */
  uint8_t in[33];
  in[0] = 64;
  memcpy(in + 1, state, 32);
  if (len >= 32) {
    gmo_shake256(out, len, in, 33);
    memcpy(state, out, 32);
  } else {
    uint8_t tmp[32];
    gmo_shake256(tmp, 32, in, 33);
    memcpy(out, tmp, (size_t)len);
    memcpy(state, tmp, 32);
  }
}

/* ---------------------------------------------------------------- helpers */

static inline gf load_gf(const uint8_t *p, gf mask) { return (gf)((p[0] | (p[1] << 8)) & mask); }
static inline uint32_t load4(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline gf bitrev_m(gf a, int m) {
  gf r = 0;
  for (int i = 0; i < m; i++) r |= (gf)(((a >> i) & 1) << (m - 1 - i));
  return r;
}

static gf poly_eval(const field *F, const gf *f, int deg, gf a) {
  gf r = f[deg];
  for (int i = deg - 1; i >= 0; i--) r = (gf)(fmul(F, r, a) ^ f[i]);
  return r;
}

static void sort_u16(uint16_t *x, int n) { /* insertion sort; n <= 128 */
  for (int i = 1; i < n; i++) {
    uint16_t v = x[i]; int j = i - 1;
    while (j >= 0 && x[j] > v) { x[j + 1] = x[j]; j--; }
    x[j + 1] = v;
  }
}

static void radix_sort_u32(uint32_t *a, uint32_t *tmp, long n) {
  if (n < 64) {
    for (long i = 1; i < n; i++) {
      uint32_t v = a[i]; long j = i - 1;
      while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; j--; }
      a[j + 1] = v;
    }
    return;
  }
  for (int shift = 0; shift < 32; shift += 8) {
    long cnt[257];
    memset(cnt, 0, sizeof cnt);
    for (long i = 0; i < n; i++) cnt[((a[i] >> shift) & 0xFF) + 1]++;
    for (int i = 0; i < 256; i++) cnt[i + 1] += cnt[i];
    for (long i = 0; i < n; i++) tmp[cnt[(a[i] >> shift) & 0xFF]++] = a[i];
    memcpy(a, tmp, sizeof(uint32_t) * (size_t)n);
  }
}

static int cmp_u64(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : x > y;
}

/* ---------------------------------------------------------------- keygen */

/* Multiplication in GF((2^m)^t) (mc:crypto_kem/<set>/vec/gf_2mt_mul.c). */
static void ext_mul(const setdef *S, const field *F, gf *out, const gf *a, const gf *b) {
  int t = S->t;
  gf prod[2 * GMO_MAX_T];
  memset(prod, 0, sizeof prod);
  for (int i = 0; i < t; i++)
    for (int j = 0; j < t; j++) prod[i + j] ^= fmul(F, a[i], b[j]);
  for (int i = 2 * t - 2; i >= t; i--)
    for (int k = 0; k < S->ntaps; k++) {
      gf v = S->taps[k].times_z ? fmul(F, prod[i], 2) : prod[i];
      prod[i - t + S->taps[k].pos] ^= v;
    }
  memcpy(out, prod, sizeof(gf) * (size_t)t);
}

/* Minimal polynomial of f in GF((2^m)^t): solve sum_c g_c f^c = f^t.
 * Follows genpoly_gen, mc:crypto_kem/348864/vec/sk_gen.c:29. Returns -1 when
 * f^0..f^(t-1) are dependent. */
static int genpoly(const setdef *S, const field *F, gf *g, const gf *f) {
  int t = S->t;
  gf (*mat)[GMO_MAX_T] = malloc(sizeof(gf) * GMO_MAX_T * (GMO_MAX_T + 1));
  memset(mat, 0, sizeof(gf) * GMO_MAX_T * (GMO_MAX_T + 1));
  mat[0][0] = 1;
  memcpy(mat[1], f, sizeof(gf) * (size_t)t);
  for (int j = 2; j <= t; j++) ext_mul(S, F, mat[j], mat[j - 1], f);
  /* mat[c][r]: column c = f^c, row r = coefficient r */
  for (int j = 0; j < t; j++) {
    if (!mat[j][j]) {
      int k;
      for (k = j + 1; k < t; k++) if (mat[j][k]) break;
      if (k == t) { free(mat); return -1; }
      for (int c = j; c <= t; c++) mat[c][j] ^= mat[c][k];
    }
    gf inv = finv(F, mat[j][j]);
    for (int c = j; c <= t; c++) mat[c][j] = fmul(F, mat[c][j], inv);
    for (int k = 0; k < t; k++) {
      if (k == j) continue;
      gf coef = mat[j][k];
      if (!coef) continue;
      for (int c = j; c <= t; c++) mat[c][k] ^= fmul(F, mat[c][j], coef);
    }
  }
  for (int i = 0; i < t; i++) g[i] = mat[t][i];
  free(mat);
  return 0;
}

static int mat_bit(const uint64_t *row, int c) { return (int)((row[c / 64] >> (c % 64)) & 1); }
static void mat_swap_cols(uint64_t *row, int a, int b) {
  if (mat_bit(row, a) != mat_bit(row, b)) {
    row[a / 64] ^= 1ULL << (a % 64);
    row[b / 64] ^= 1ULL << (b % 64);
  }
}

/* Semi-systematic step of the "f" variants (mc:crypto_kem/348864f/vec/pk_gen.c,
 * mov_columns; 6960119f at an unaligned row): with the first R = mt - 32
 * columns reduced, the last 32 rows' 32 x 64 block at columns R .. R+63
 * gives pivot columns c_0 < ... < c_31 (leftmost, by elimination on that
 * block; fail when its rank is below 32); pivots = sum 2^c_j; for j = 0..31
 * in turn, columns R+j and R+c_j of every row and pi[R+j], pi[R+c_j] are
 * swapped. */
static int mov_columns(const sizes *P, uint64_t *mat, int rw, int16_t *pi, uint64_t *pivots) {
  const int R = P->mt - 32;
  uint64_t buf[32];
  int ctz[32];
  for (int i = 0; i < 32; i++) {
    buf[i] = 0;
    for (int c = 0; c < 64; c++)
      if (R + c < P->n && mat_bit(&mat[(size_t)(R + i) * rw], R + c)) buf[i] |= 1ULL << c;
  }
  *pivots = 0;
  for (int i = 0; i < 32; i++) {
    uint64_t t = 0;
    for (int j = i; j < 32; j++) t |= buf[j];
    if (!t) return -1;
    int s = __builtin_ctzll(t);
    ctz[i] = s;
    *pivots |= 1ULL << s;
    for (int j = i + 1; j < 32; j++)
      if (!((buf[i] >> s) & 1)) buf[i] ^= buf[j];
    for (int j = i + 1; j < 32; j++)
      if ((buf[j] >> s) & 1) buf[j] ^= buf[i];
  }
  for (int j = 0; j < 32; j++) {
    if (ctz[j] == j) continue;
    int16_t tmp = pi[R + j]; pi[R + j] = pi[R + ctz[j]]; pi[R + ctz[j]] = tmp;
    for (int r = 0; r < P->mt; r++) mat_swap_cols(&mat[(size_t)r * rw], R + j, R + ctz[j]);
  }
  return 0;
}

/* Public key: systematic form [I_mt | T] of the parity-check matrix with rows
 * (i*m+b) = bit b of L_j^i / g(L_j); pk stores T row-major, PK_ROW_BYTES per
 * row, little-endian bit order.  Same output as pk_gen,
 * mc:crypto_kem/348864/vec/pk_gen.c:82 (the RREF is unique). The f variants
 * insert mov_columns before the last 32 rows (pivots != 0 then). */
static int pk_gen(const sizes *P, const field *F, uint8_t *pk, const gf *g, const uint32_t *perm, int16_t *pi,
                  uint64_t *pivots) {
  int m = P->m, n = P->n, t = P->t, mt = P->mt, q = P->q;
  int rw = (n + 63) / 64;
  uint64_t *buf = malloc(sizeof(uint64_t) * (size_t)q);
  for (int i = 0; i < q; i++) buf[i] = ((uint64_t)perm[i] << 31) | (uint64_t)i;
  qsort(buf, (size_t)q, sizeof(uint64_t), cmp_u64);
  for (int i = 1; i < q; i++)
    if ((buf[i - 1] >> 31) == (buf[i] >> 31)) { free(buf); return -1; }
  for (int i = 0; i < q; i++) pi[i] = (int16_t)(buf[i] & (uint64_t)(q - 1));
  free(buf);

  gf *L = malloc(sizeof(gf) * (size_t)n), *inv = malloc(sizeof(gf) * (size_t)n);
  for (int i = 0; i < n; i++) L[i] = bitrev_m((gf)pi[i], m);
  for (int i = 0; i < n; i++) {
    gf gl = poly_eval(F, g, t, L[i]); /* g monic: g[t] = 1 */
    inv[i] = finv(F, gl);
  }
  uint64_t *mat = calloc((size_t)mt * (size_t)rw, sizeof(uint64_t));
  for (int i = 0; i < t; i++) {
    for (int j = 0; j < n; j++)
      for (int b = 0; b < m; b++)
        if ((inv[j] >> b) & 1) mat[(size_t)(i * m + b) * rw + j / 64] |= 1ULL << (j % 64);
    for (int j = 0; j < n; j++) inv[j] = fmul(F, inv[j], L[j]);
  }
  free(L); free(inv);

  for (int row = 0; row < mt; row++) {
    if (P->f && row == mt - 32 && mov_columns(P, mat, rw, pi, pivots)) { free(mat); return -1; }
    int w = row / 64; uint64_t bit = 1ULL << (row % 64);
    int piv = -1;
    for (int r = row; r < mt; r++) if (mat[(size_t)r * rw + w] & bit) { piv = r; break; }
    if (piv < 0) { free(mat); return -1; }
    if (piv != row)
      for (int c = 0; c < rw; c++) mat[(size_t)row * rw + c] ^= mat[(size_t)piv * rw + c];
    const uint64_t *src = &mat[(size_t)row * rw];
    for (int r = 0; r < mt; r++) {
      if (r == row || !(mat[(size_t)r * rw + w] & bit)) continue;
      uint64_t *dst = &mat[(size_t)r * rw];
      for (int c = w; c < rw; c++) dst[c] ^= src[c];
    }
  }
  for (int r = 0; r < mt; r++) {
    uint8_t *out = pk + (size_t)r * P->pk_row_bytes;
    memset(out, 0, (size_t)P->pk_row_bytes);
    for (int j = 0; j < P->k; j++) {
      int col = mt + j;
      if ((mat[(size_t)r * rw + col / 64] >> (col % 64)) & 1) out[j / 8] |= (uint8_t)(1 << (j % 8));
    }
  }
  free(mat);
  return 0;
}

/* Control bits of a Benes network for the permutation pi of {0..2^w-1}.
 * Restates the Nassimi-Sahni / Bernstein "controlbits" recursion
 * (mc:crypto_kem/348864/vec/controlbits.c:29, cbrecursion).  Control bits
 * are not unique for a permutation, so the same sequence of sort steps is
 * kept to land on the same bits.  All packed values stay below 2^31, so the
 * signed int32 sort of the library equals this unsigned sort. */
static void cb_rec(uint8_t *out, long long pos, long long step, const int16_t *pi, int w, long n, uint32_t *tmp) {
  uint32_t *A = tmp, *B = tmp + n, *S = tmp + 2 * n; /* S: sort scratch (n) */
  int16_t *qq = (int16_t *)(tmp + 3 * n);              /* n int16 */
  if (w == 1) { out[pos >> 3] ^= (uint8_t)(pi[0] << (pos & 7)); return; }

  for (long x = 0; x < n; x++) A[x] = ((uint32_t)(pi[x] ^ 1) << 16) | (uint32_t)pi[x ^ 1];
  radix_sort_u32(A, S, n);
  for (long x = 0; x < n; x++) {
    uint32_t px = A[x] & 0xffff;
    uint32_t cx = px < (uint32_t)x ? px : (uint32_t)x;
    B[x] = (px << 16) | cx;
  }
  for (long x = 0; x < n; x++) A[x] = (A[x] << 16) | (uint32_t)x;
  radix_sort_u32(A, S, n);
  for (long x = 0; x < n; x++) A[x] = (A[x] << 16) + (B[x] >> 16);
  radix_sort_u32(A, S, n);

  if (w <= 10) {
    for (long x = 0; x < n; x++) B[x] = ((A[x] & 0xffff) << 10) | (B[x] & 0x3ff);
    for (int i = 1; i < w - 1; i++) {
      for (long x = 0; x < n; x++) A[x] = ((B[x] & ~0x3ffu) << 6) | (uint32_t)x;
      radix_sort_u32(A, S, n);
      for (long x = 0; x < n; x++) A[x] = (A[x] << 20) | B[x];
      radix_sort_u32(A, S, n);
      for (long x = 0; x < n; x++) {
        uint32_t ppcp = A[x] & 0xfffff;
        uint32_t ppc = (A[x] & 0xffc00) | (B[x] & 0x3ff);
        B[x] = ppc < ppcp ? ppc : ppcp;
      }
    }
    for (long x = 0; x < n; x++) B[x] &= 0x3ff;
  } else {
    for (long x = 0; x < n; x++) B[x] = (A[x] << 16) | (B[x] & 0xffff);
    for (int i = 1; i < w - 1; i++) {
      for (long x = 0; x < n; x++) A[x] = (B[x] & ~0xffffu) | (uint32_t)x;
      radix_sort_u32(A, S, n);
      for (long x = 0; x < n; x++) A[x] = (A[x] << 16) | (B[x] & 0xffff);
      if (i < w - 2) {
        for (long x = 0; x < n; x++) B[x] = (A[x] & ~0xffffu) | (B[x] >> 16);
        radix_sort_u32(B, S, n);
        for (long x = 0; x < n; x++) B[x] = (B[x] << 16) | (A[x] & 0xffff);
      }
      radix_sort_u32(A, S, n);
      for (long x = 0; x < n; x++) {
        uint32_t cp = (B[x] & ~0xffffu) | (A[x] & 0xffff);
        B[x] = B[x] < cp ? B[x] : cp;
      }
    }
    for (long x = 0; x < n; x++) B[x] &= 0xffff;
  }

  for (long x = 0; x < n; x++) A[x] = ((uint32_t)pi[x] << 16) + (uint32_t)x;
  radix_sort_u32(A, S, n);

  for (long j = 0; j < n / 2; j++) {
    long z = 2 * j;
    uint32_t fj = B[z] & 1;
    uint32_t Fz = (uint32_t)z + fj, Fz1 = Fz ^ 1;
    out[pos >> 3] ^= (uint8_t)(fj << (pos & 7));
    pos += step;
    B[z] = (A[z] << 16) | Fz;
    B[z + 1] = (A[z + 1] << 16) | Fz1;
  }
  radix_sort_u32(B, S, n);
  pos += (2 * w - 3) * step * (n / 2);
  for (long k = 0; k < n / 2; k++) {
    long y = 2 * k;
    uint32_t lk = B[y] & 1;
    uint32_t Ly = (uint32_t)y + lk, Ly1 = Ly ^ 1;
    out[pos >> 3] ^= (uint8_t)(lk << (pos & 7));
    pos += step;
    A[y] = (Ly << 16) | (B[y] & 0xffff);
    A[y + 1] = (Ly1 << 16) | (B[y + 1] & 0xffff);
  }
  radix_sort_u32(A, S, n);
  pos -= (2 * w - 2) * step * (n / 2);
  for (long j = 0; j < n / 2; j++) {
    qq[j] = (int16_t)((A[2 * j] & 0xffff) >> 1);
    qq[j + n / 2] = (int16_t)((A[2 * j + 1] & 0xffff) >> 1);
  }
  /* the sub-permutations must survive the recursive calls, which reuse tmp */
  int16_t *sub = malloc(sizeof(int16_t) * (size_t)n);
  memcpy(sub, qq, sizeof(int16_t) * (size_t)n);
  cb_rec(out, pos, step * 2, sub, w - 1, n / 2, tmp);
  cb_rec(out, pos + step, step * 2, sub + n / 2, w - 1, n / 2, tmp);
  free(sub);
}

/* One Benes layer: conditional swaps at stride 2^s, control bits read in
 * order (mc:crypto_kem/348864/vec/controlbits.c:162, layer). */
static void benes_layer(int16_t *p, const uint8_t *cb, int s, int n) {
  int stride = 1 << s, idx = 0;
  for (int i = 0; i < n; i += 2 * stride)
    for (int j = 0; j < stride; j++, idx++)
      if ((cb[idx >> 3] >> (idx & 7)) & 1) {
        int16_t d = p[i + j]; p[i + j] = p[i + j + stride]; p[i + j + stride] = d;
      }
}

/* Applies all 2w-1 layers to the identity: the permutation the bits encode. */
static void perm_from_controlbits(int16_t *p, const uint8_t *cb, int w) {
  int n = 1 << w;
  for (int i = 0; i < n; i++) p[i] = (int16_t)i;
  for (int i = 0; i < w; i++) { benes_layer(p, cb, i, n); cb += n >> 4; }
  for (int i = w - 2; i >= 0; i--) { benes_layer(p, cb, i, n); cb += n >> 4; }
}

static int controlbits(uint8_t *out, const int16_t *pi, int w) {
  long n = 1L << w;
  size_t nbytes = (size_t)(((2 * w - 1) * n / 2 + 7) / 8);
  uint32_t *tmp = malloc(sizeof(uint32_t) * (size_t)(4 * n));
  memset(out, 0, nbytes);
  cb_rec(out, 0, 1, pi, w, n, tmp);
  free(tmp);
  int16_t *chk = malloc(sizeof(int16_t) * (size_t)n);
  perm_from_controlbits(chk, out, w);
  int bad = 0;
  for (long i = 0; i < n; i++) bad |= chk[i] != pi[i];
  free(chk);
  return bad ? -1 : 0;
}

/* Control bits of a permutation of 2^w entries (the recursion above, as keygen
 * runs it); 0, or -1 when the bits do not re-encode pi. */
int gmo_controlbits(uint8_t *out, const int16_t *pi, int w) {
  if (w < 1 || w > 13) return -1;
  return controlbits(out, pi, w);
}

/* Key generation (mc:crypto_kem/348864/vec/kem_keypair.c:20, identical for
 * all five sets): one 32-byte randombytes draw, then the seed-expansion loop. */
int gmo_keypair_rng(int set, uint8_t *pk, uint8_t *sk, gmo_rng_fn rng, void *ctx) {
  sizes P;
  if (get_sizes(set, &P)) return -1;
  ensure_init();
  const setdef *S = &SETS[set % GMO_NSETS];
  const field *F = &FIELD[P.m - 12];
  uint8_t seed[33];
  seed[0] = 64;
  rng(ctx, seed + 1, 32);
  long rlen = P.e_bytes + 4L * P.q + 2L * P.t + 32;
  uint8_t *r = malloc((size_t)rlen);
  uint32_t *perm = malloc(sizeof(uint32_t) * (size_t)P.q);
  int16_t *pi = malloc(sizeof(int16_t) * (size_t)P.q);
  gf f[GMO_MAX_T], irr[GMO_MAX_T];
  for (;;) {
    gmo_shake256(r, rlen, seed, 33);
    memcpy(sk, seed + 1, 32);
    memcpy(seed + 1, r + rlen - 32, 32);
    const uint8_t *rp = r + rlen - 32 - 2 * P.t;
    for (int i = 0; i < P.t; i++) f[i] = load_gf(rp + 2 * i, (gf)(P.q - 1));
    if (genpoly(S, F, irr, f)) continue;
    uint8_t *skp = sk + 40;
    for (int i = 0; i < P.t; i++) { skp[2 * i] = (uint8_t)irr[i]; skp[2 * i + 1] = (uint8_t)(irr[i] >> 8); }
    skp += P.irr_bytes;
    rp -= 4L * P.q;
    for (int i = 0; i < P.q; i++) perm[i] = load4(rp + 4 * i);
    gf g[GMO_MAX_T + 1];
    memcpy(g, irr, sizeof(gf) * (size_t)P.t);
    g[P.t] = 1;
    uint64_t pivots = 0xFFFFFFFFULL;
    if (pk_gen(&P, F, pk, g, perm, pi, &pivots)) continue;
    if (controlbits(skp, pi, P.m)) { free(r); free(perm); free(pi); return -2; }
    skp += P.cond_bytes;
    memcpy(skp, r, (size_t)P.e_bytes);
    /* pivot word: store8(sk + 32, pivots), 0xFFFFFFFF without the semi-systematic step */
    for (int i = 0; i < 8; i++) sk[32 + i] = (uint8_t)(pivots >> (8 * i));
    break;
  }
  free(r); free(perm); free(pi);
  return 0;
}

static void fixed_rng(void *ctx, uint8_t *out, long long len) {
  memcpy(out, ctx, (size_t)len); /* exactly one 32-byte draw in keygen */
}

int gmo_keypair(int set, uint8_t *pk, uint8_t *sk, const uint8_t *seed32) {
  uint8_t s[32];
  memcpy(s, seed32, 32);
  return gmo_keypair_rng(set, pk, sk, fixed_rng, s);
}

/* ---------------------------------------------------------------- encaps */

/* Fixed-weight error vector (mc:crypto_kem/348864/vec/encrypt.c:41 gen_e;
 * n = 2^m variant mc:crypto_kem/8192128/vec/encrypt.c:31).  One randombytes
 * call per attempt: 4t bytes (2t candidates kept if < n) or, when n = 2^m,
 * 2t bytes.  Returns the number of attempts. */
int gmo_gen_e_rng(int set, uint8_t *e, gmo_rng_fn rng, void *ctx, uint16_t *ind_out) {
  sizes P;
  if (get_sizes(set, &P)) return -1;
  ensure_init();
  int t = P.t, n = P.n;
  gf mask = (gf)(P.q - 1);
  int full = (n == P.q);
  uint8_t buf[4 * GMO_MAX_T];
  uint16_t ind[GMO_MAX_T];
  int attempts = 0;
  for (;;) {
    attempts++;
    int nb = full ? 2 * t : 4 * t;
    rng(ctx, buf, nb);
    int count = 0;
    if (full) {
      for (int i = 0; i < t; i++) ind[i] = load_gf(buf + 2 * i, mask);
      count = t;
    } else {
      for (int i = 0; i < 2 * t && count < t; i++) {
        gf v = load_gf(buf + 2 * i, mask);
        if (v < n) ind[count++] = v;
      }
      if (count < t) continue;
    }
    sort_u16(ind, t);
    int dup = 0;
    for (int i = 1; i < t; i++) dup |= ind[i - 1] == ind[i];
    if (!dup) break;
  }
  memset(e, 0, (size_t)P.e_bytes);
  for (int j = 0; j < t; j++) e[ind[j] >> 3] |= (uint8_t)(1 << (ind[j] & 7));
  if (ind_out) memcpy(ind_out, ind, sizeof(uint16_t) * (size_t)t);
  return attempts;
}

int gmo_gen_e(int set, uint8_t *e, const uint8_t *seed32) {
  uint8_t st[32];
  memcpy(st, seed32, 32);
  return gmo_gen_e_rng(set, e, gmo_chain_randombytes, st, NULL);
}

/* c[0:mt] = e[0:mt] xor T * e[mt:n] over GF(2)
 * (mc:crypto_kem/348864/vec/encrypt.c:94; unaligned mt for 6960119:
 * mc:crypto_kem/6960119/vec/encrypt.c, syndrome). */
int gmo_syndrome(int set, uint8_t *s, const uint8_t *pk, const uint8_t *e) {
  sizes P;
  if (get_sizes(set, &P)) return -1;
  int kw = (P.k + 63) / 64;
  uint64_t ens[128];
  memset(ens, 0, sizeof ens);
  for (int j = 0; j < P.k; j++) {
    int b = P.mt + j;
    if ((e[b >> 3] >> (b & 7)) & 1) ens[j / 64] |= 1ULL << (j % 64);
  }
  memcpy(s, e, (size_t)P.synd_bytes);
  if (P.mt % 8) s[P.synd_bytes - 1] &= (uint8_t)((1 << (P.mt % 8)) - 1);
  for (int i = 0; i < P.mt; i++) {
    const uint8_t *row = pk + (size_t)i * P.pk_row_bytes;
    uint64_t acc = 0;
    for (int w = 0; w < kw; w++) {
      uint64_t v = 0;
      for (int b = 0; b < 8; b++) {
        int idx = 8 * w + b;
        if (idx < P.pk_row_bytes) v |= (uint64_t)row[idx] << (8 * b);
      }
      acc ^= v & ens[w];
    }
    s[i >> 3] ^= (uint8_t)(__builtin_parityll(acc) << (i & 7));
  }
  return 0;
}

static int pk_padding_bad(const sizes *P, const uint8_t *pk) {
  if (P->k % 8 == 0) return 0;
  uint8_t b = 0;
  for (int i = 0; i < P->mt; i++) b |= pk[(size_t)i * P->pk_row_bytes + P->pk_row_bytes - 1];
  return (b >> (P->k % 8)) != 0;
}

static int c_padding_bad(const sizes *P, const uint8_t *c) {
  if (P->mt % 8 == 0) return 0;
  return (c[P->synd_bytes - 1] >> (P->mt % 8)) != 0;
}

/* KEM encapsulation (mc:crypto_kem/348864/vec/kem_enc.c:18; pk padding rule
 * of 6960119 at mc:crypto_kem/6960119/vec/kem_enc.c:21-66):
 * K = SHAKE256(1 || e || c, 32). Plaintext confirmation
 * (mc:crypto_kem/348864pc/vec/kem_enc.c:24-35): c = C0 || SHAKE256(2 || e, 32). */
int gmo_enc_rng(int set, uint8_t *c, uint8_t *key, const uint8_t *pk, gmo_rng_fn rng, void *ctx) {
  sizes P;
  if (get_sizes(set, &P)) return -1;
  uint8_t e[GMO_MAX_N / 8];
  uint8_t pre[1 + GMO_MAX_N / 8 + GMO_MAX_MT / 8 + 32];
  int bad = pk_padding_bad(&P, pk);
  gmo_gen_e_rng(set, e, rng, ctx, NULL);
  gmo_syndrome(set, c, pk, e);
  if (P.pc) {
    pre[0] = 2;
    memcpy(pre + 1, e, (size_t)P.e_bytes);
    gmo_shake256(c + P.synd_bytes, 32, pre, 1 + P.e_bytes);
  }
  pre[0] = 1;
  memcpy(pre + 1, e, (size_t)P.e_bytes);
  memcpy(pre + 1 + P.e_bytes, c, (size_t)P.ct_bytes);
  gmo_shake256(key, 32, pre, 1 + P.e_bytes + P.ct_bytes);
  if (bad) {
    memset(c, 0, (size_t)P.ct_bytes);
    memset(key, 0, 32);
    return -1;
  }
  return 0;
}

int gmo_enc(int set, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seed32) {
  uint8_t st[32];
  memcpy(st, seed32, 32);
  return gmo_enc_rng(set, c, key, pk, gmo_chain_randombytes, st);
}

/* ---------------------------------------------------------------- decaps */

typedef struct {
  sizes P;
  const field *F;
  gf g[GMO_MAX_T + 1];
  gf *L;     /* n support elements */
  gf *w2;    /* 1 / g(L_i)^2 */
  const uint8_t *s; /* sk random string */
} keyctx;

static int key_prepare(int set, const uint8_t *sk, keyctx *K) {
  if (get_sizes(set, &K->P)) return -1;
  ensure_init();
  K->F = &FIELD[K->P.m - 12];
  const uint8_t *gp = sk + 40;
  for (int i = 0; i < K->P.t; i++) K->g[i] = load_gf(gp + 2 * i, (gf)(K->P.q - 1));
  K->g[K->P.t] = 1;
  int16_t *pi = malloc(sizeof(int16_t) * (size_t)K->P.q);
  perm_from_controlbits(pi, sk + 40 + K->P.irr_bytes, K->P.m);
  K->L = malloc(sizeof(gf) * (size_t)K->P.n);
  K->w2 = malloc(sizeof(gf) * (size_t)K->P.n);
  for (int i = 0; i < K->P.n; i++) {
    K->L[i] = bitrev_m((gf)pi[i], K->P.m);
    gf v = poly_eval(K->F, K->g, K->P.t, K->L[i]);
    K->w2[i] = finv(K->F, fmul(K->F, v, v));
  }
  free(pi);
  K->s = sk + 40 + K->P.irr_bytes + K->P.cond_bytes;
  return 0;
}

static void key_release(keyctx *K) { free(K->L); free(K->w2); }

/* 2t syndromes of a received word r (n bits): sum over r_i=1 of L_i^j/g(L_i)^2. */
static void synd2t(const keyctx *K, gf *out, const uint8_t *r, int nbits) {
  int t2 = 2 * K->P.t;
  memset(out, 0, sizeof(gf) * (size_t)t2);
  for (int i = 0; i < nbits; i++) {
    if (!((r[i >> 3] >> (i & 7)) & 1)) continue;
    gf v = K->w2[i];
    for (int j = 0; j < t2; j++) { out[j] ^= v; v = fmul(K->F, v, K->L[i]); }
  }
}

/* Berlekamp-Massey over GF(2^m) with the update rule of the libmceliece
 * decoder (mc:crypto_kem/348864/vec/bm.c:156; device port
 * mceliece-gpu-params/ref/348864.cuh:2797-2880).  out[i] = C[t-i], so the
 * roots of out are the error positions' support elements. */
static void bm(const field *F, int t, gf *out, const gf *s) {
  gf T[GMO_MAX_T + 1], C[GMO_MAX_T + 1], B[GMO_MAX_T + 1];
  gf b = 1;
  int L = 0;
  memset(C, 0, sizeof C); memset(B, 0, sizeof B);
  C[0] = 1; B[1] = 1;
  for (int N = 0; N < 2 * t; N++) {
    gf d = 0;
    int lim = N < t ? N : t;
    for (int i = 0; i <= lim; i++) d ^= fmul(F, C[i], s[N - i]);
    int nz = d != 0;
    int upd = nz && (N >= 2 * L);
    memcpy(T, C, sizeof(gf) * (size_t)(t + 1));
    if (nz) {
      gf f = fmul(F, finv(F, b), d);
      for (int i = 0; i <= t; i++) C[i] ^= fmul(F, f, B[i]);
    }
    if (upd) { L = N + 1 - L; memcpy(B, T, sizeof(gf) * (size_t)(t + 1)); b = d; }
    for (int i = t; i >= 1; i--) B[i] = B[i - 1];
    B[0] = 0;
  }
  for (int i = 0; i <= t; i++) out[i] = C[t - i];
}

/* Niederreiter decryption: returns 0 when a weight-t error with the
 * received syndrome was found (mc:crypto_kem/348864/vec/decrypt.c:135).
 * Optional stage outputs for the staged GPU parity tests. */
static int decrypt_ctx(const keyctx *K, uint8_t *e, const uint8_t *c, gf *s_out, gf *loc_out) {
  const sizes *P = &K->P;
  int t = P->t, n = P->n;
  uint8_t r[GMO_MAX_N / 8];
  gf s[2 * GMO_MAX_T], s2[2 * GMO_MAX_T], loc[GMO_MAX_T + 1];
  memset(r, 0, sizeof r);
  memcpy(r, c, (size_t)P->synd_bytes);
  synd2t(K, s, r, n);
  bm(K->F, t, loc, s);
  memset(e, 0, (size_t)P->e_bytes);
  int w = 0;
  for (int i = 0; i < n; i++) {
    if (poly_eval(K->F, loc, t, K->L[i]) == 0) { e[i >> 3] |= (uint8_t)(1 << (i & 7)); w++; }
  }
  synd2t(K, s2, e, n);
  int ok = (w == t);
  for (int i = 0; i < 2 * t; i++) ok &= s[i] == s2[i];
  if (s_out) memcpy(s_out, s, sizeof(gf) * (size_t)(2 * t));
  if (loc_out) memcpy(loc_out, loc, sizeof(gf) * (size_t)(t + 1));
  return ok ? 0 : 1;
}

/* KEM decapsulation with implicit rejection (mc:crypto_kem/348864/vec/kem_dec.c:19;
 * c padding rule of 6960119 at mc:crypto_kem/6960119/vec/kem_dec.c:21-78). */
static int dec_ctx(const keyctx *K, uint8_t *key, const uint8_t *c) {
  const sizes *P = &K->P;
  uint8_t cc[GMO_MAX_MT / 8 + 32];
  memcpy(cc, c, (size_t)P->ct_bytes); /* key may alias c */
  uint8_t e[GMO_MAX_N / 8];
  uint8_t pre[1 + GMO_MAX_N / 8 + GMO_MAX_MT / 8 + 32];
  int fail = decrypt_ctx(K, e, cc, NULL, NULL);
  if (P->pc) {
    /* plaintext confirmation (mc:crypto_kem/348864pc/vec/kem_dec.c:43-48):
     * reject unless SHAKE256(2 || e, 32) equals C1 */
    uint8_t conf[32];
    pre[0] = 2;
    memcpy(pre + 1, e, (size_t)P->e_bytes);
    gmo_shake256(conf, 32, pre, 1 + P->e_bytes);
    fail |= memcmp(conf, cc + P->synd_bytes, 32) != 0;
  }
  pre[0] = fail ? 0 : 1;
  memcpy(pre + 1, fail ? K->s : e, (size_t)P->e_bytes);
  memcpy(pre + 1 + P->e_bytes, cc, (size_t)P->ct_bytes);
  gmo_shake256(key, 32, pre, 1 + P->e_bytes + P->ct_bytes);
  if (c_padding_bad(P, cc)) { memset(key, 0xFF, 32); return -1; }
  return 0;
}

int gmo_dec(int set, uint8_t *key, const uint8_t *c, const uint8_t *sk) {
  keyctx K;
  /* sk may alias key: the key context copies what it needs first */
  uint8_t *skc = malloc(40 + 2 * GMO_MAX_T + 12800 + 1024);
  sizes P;
  if (get_sizes(set, &P)) { free(skc); return -1; }
  memcpy(skc, sk, (size_t)P.sk_bytes);
  if (key_prepare(set, skc, &K)) { free(skc); return -1; }
  int rc = dec_ctx(&K, key, c);
  key_release(&K);
  free(skc);
  return rc;
}

int gmo_decrypt_stages(int set, const uint8_t *sk, const uint8_t *c, uint16_t *s_priv, uint16_t *locator,
                       uint8_t *e) {
  keyctx K;
  if (key_prepare(set, sk, &K)) return -1;
  int rc = decrypt_ctx(&K, e, c, s_priv, locator);
  key_release(&K);
  return rc;
}

int gmo_support(int set, const uint8_t *sk, uint16_t *L_out, uint16_t *w2_out) {
  keyctx K;
  if (key_prepare(set, sk, &K)) return -1;
  memcpy(L_out, K.L, sizeof(gf) * (size_t)K.P.n);
  if (w2_out) memcpy(w2_out, K.w2, sizeof(gf) * (size_t)K.P.n);
  key_release(&K);
  return 0;
}

int gmo_gf_mul(int m, int a, int b) {
  ensure_init();
  return fmul(&FIELD[m - 12], (gf)a, (gf)b);
}

/* ---------------------------------------------------------------- batches */

typedef struct {
  int set, op;
  long long lo, hi;
  uint8_t *out_c, *out_k;
  const uint8_t *in_c, *pk, *seeds;
  const keyctx *K;
  int *rc;
} job;

static void *worker(void *arg) {
  job *J = (job *)arg;
  sizes P;
  get_sizes(J->set, &P);
  for (long long i = J->lo; i < J->hi; i++) {
    int r;
    if (J->op == 0)
      r = gmo_enc(J->set, J->out_c + i * P.ct_bytes, J->out_k + 32 * i, J->pk, J->seeds + 32 * i);
    else
      r = dec_ctx(J->K, J->out_k + 32 * i, J->in_c + i * P.ct_bytes);
    if (J->rc) J->rc[i] = r;
  }
  return NULL;
}

static int run_batch(job *base, long long count, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t th[256];
  job jobs[256];
  long long per = (count + threads - 1) / threads;
  int used = 0;
  for (int i = 0; i < threads; i++) {
    jobs[i] = *base;
    jobs[i].lo = i * per;
    jobs[i].hi = (i + 1) * per < count ? (i + 1) * per : count;
    if (jobs[i].lo >= jobs[i].hi) break;
    if (pthread_create(&th[i], NULL, worker, &jobs[i])) return -1;
    used++;
  }
  for (int i = 0; i < used; i++) pthread_join(th[i], NULL);
  return 0;
}

int gmo_enc_batch(int set, long long count, uint8_t *c, uint8_t *key, const uint8_t *pk, const uint8_t *seeds,
                  int *rc, int threads) {
  ensure_init();
  job J;
  memset(&J, 0, sizeof J);
  J.set = set; J.op = 0; J.out_c = c; J.out_k = key; J.pk = pk; J.seeds = seeds; J.rc = rc;
  return run_batch(&J, count, threads);
}

int gmo_dec_batch(int set, long long count, uint8_t *key, const uint8_t *c, const uint8_t *sk, int *rc,
                  int threads) {
  keyctx K;
  if (key_prepare(set, sk, &K)) return -1;
  job J;
  memset(&J, 0, sizeof J);
  J.set = set; J.op = 1; J.out_k = key; J.in_c = c; J.K = &K; J.rc = rc;
  int r = run_batch(&J, count, threads);
  key_release(&K);
  return r;
}
