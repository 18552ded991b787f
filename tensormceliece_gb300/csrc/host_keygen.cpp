// Key generation with libmceliece's output format and seed expansion
// (mc:crypto_kem/348864/vec/kem_keypair.c:20-100, identical for the five
// sets): one 32-byte randombytes draw delta; loop { r = SHAKE256({64}||delta,
// n/8 + 4*2^m + 2t + 32); next delta = last 32 bytes of r; irreducible g from
// the minimal polynomial of a random element of GF((2^m)^t) (sk_gen.c:29);
// support permutation from sorting 2^m random 32-bit values (pk_gen.c:82,
// reject on a tie); systematic public key [I | T] (reject if the first mt
// columns are singular); Benes control bits of the permutation
// (controlbits.c:29); s = r[0:n/8] }.
//
// Key generation is not on the batched enc/dec path; this is the host
// implementation behind gmc_keypair / gmc_kem_<set>_keypair.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "host_keys.h"

namespace gmc {

// ---------------------------------------------------------------- SHAKE256
namespace {
struct Keccak {
  uint64_t rc[24];
  int rho[25];
  Keccak() {
    unsigned r = 1;
    for (int ir = 0; ir < 24; ir++) {
      uint64_t c = 0;
      for (int j = 0; j < 7; j++) {
        if (r & 1) c |= 1ull << ((1 << j) - 1);
        r = ((r << 1) ^ ((r & 0x80) ? 0x71 : 0)) & 0xFF;
      }
      rc[ir] = c;
    }
    int x = 1, y = 0;
    rho[0] = 0;
    for (int t = 0; t < 24; t++) {
      rho[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
      int nx = y, ny = (2 * x + 3 * y) % 5;
      x = nx;
      y = ny;
    }
  }
  static uint64_t rot(uint64_t v, int n) { return n ? (v << n) | (v >> (64 - n)) : v; }
  void f(uint64_t *s) const {
    uint64_t C[5], D[5], B[25];
    for (int round = 0; round < 24; round++) {
      for (int x = 0; x < 5; x++) C[x] = s[x] ^ s[x + 5] ^ s[x + 10] ^ s[x + 15] ^ s[x + 20];
      for (int x = 0; x < 5; x++) D[x] = C[(x + 4) % 5] ^ rot(C[(x + 1) % 5], 1);
      for (int x = 0; x < 5; x++)
        for (int y = 0; y < 5; y++) B[y + 5 * ((2 * x + 3 * y) % 5)] = rot(s[x + 5 * y] ^ D[x], rho[x + 5 * y]);
      for (int y = 0; y < 5; y++)
        for (int x = 0; x < 5; x++)
          s[x + 5 * y] = B[x + 5 * y] ^ (~B[(x + 1) % 5 + 5 * y] & B[(x + 2) % 5 + 5 * y]);
      s[0] ^= rc[round];
    }
  }
};
const Keccak &keccak() {
  static Keccak k;
  return k;
}
}  // namespace

void host_shake256(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen) {
  const Keccak &K = keccak();
  uint64_t s[25] = {0};
  uint8_t blk[136];
  while (inlen >= 136) {
    for (int i = 0; i < 17; i++) {
      uint64_t w = 0;
      for (int b = 0; b < 8; b++) w |= (uint64_t)in[8 * i + b] << (8 * b);
      s[i] ^= w;
    }
    K.f(s);
    in += 136;
    inlen -= 136;
  }
  memset(blk, 0, sizeof blk);
  memcpy(blk, in, inlen);
  blk[inlen] ^= 0x1F;
  blk[135] ^= 0x80;
  for (int i = 0; i < 17; i++) {
    uint64_t w = 0;
    for (int b = 0; b < 8; b++) w |= (uint64_t)blk[8 * i + b] << (8 * b);
    s[i] ^= w;
  }
  for (;;) {
    K.f(s);
    size_t take = std::min<size_t>(outlen, 136);
    for (size_t j = 0; j < take; j++) out[j] = (uint8_t)(s[j / 8] >> (8 * (j % 8)));
    out += take;
    outlen -= take;
    if (!outlen) break;
  }
}

// ---------------------------------------------------------------- genpoly
// GF((2^m)^t) reduction taps y^t = sum taps (one tap is multiplied by z = 2
// for 348864): mc:crypto_kem/<set>/vec/gf_2mt_mul.c.
struct ExtTaps {
  int n;
  int pos[4];
  int times_z[4];
};
static const ExtTaps kTaps[GMC_NSETS] = {
    {3, {3, 1, 0, 0}, {0, 0, 1, 0}},
    {4, {10, 9, 6, 0}, {0, 0, 0, 0}},
    {4, {7, 2, 1, 0}, {0, 0, 0, 0}},
    {2, {8, 0, 0, 0}, {0, 0, 0, 0}},
    {4, {7, 2, 1, 0}, {0, 0, 0, 0}},
};

static void ext_mul(int set, const HostField &F, int t, uint16_t *out, const uint16_t *a, const uint16_t *b) {
  std::vector<uint16_t> prod(2 * t, 0);
  for (int i = 0; i < t; i++)
    if (a[i])
      for (int j = 0; j < t; j++) prod[i + j] ^= F.mul(a[i], b[j]);
  const ExtTaps &T = kTaps[set];
  for (int i = 2 * t - 2; i >= t; i--)
    for (int k = 0; k < T.n; k++) prod[i - t + T.pos[k]] ^= T.times_z[k] ? F.mul(prod[i], 2) : prod[i];
  memcpy(out, prod.data(), 2 * t);
}

// minimal polynomial of f: solve sum_{c<t} g_c f^c = f^t (Gauss-Jordan)
static bool min_poly(int set, const HostField &F, int t, const uint16_t *f, uint16_t *g) {
  std::vector<std::vector<uint16_t>> col(t + 1, std::vector<uint16_t>(t, 0));  // col[c] = f^c
  col[0][0] = 1;
  memcpy(col[1].data(), f, 2 * t);
  for (int c = 2; c <= t; c++) ext_mul(set, F, t, col[c].data(), col[c - 1].data(), f);
  for (int j = 0; j < t; j++) {
    if (!col[j][j]) {
      int k = j + 1;
      while (k < t && !col[j][k]) k++;
      if (k == t) return false;
      for (int c = j; c <= t; c++) col[c][j] ^= col[c][k];
    }
    const uint16_t inv = F.inv(col[j][j]);
    for (int c = j; c <= t; c++) col[c][j] = F.mul(col[c][j], inv);
    for (int r = 0; r < t; r++) {
      if (r == j || !col[j][r]) continue;
      const uint16_t coef = col[j][r];
      for (int c = j; c <= t; c++) col[c][r] ^= F.mul(col[c][j], coef);
    }
  }
  for (int i = 0; i < t; i++) g[i] = col[t][i];
  return true;
}

// ---------------------------------------------------------------- public key
static uint16_t bitrev_m(uint16_t a, int m) {
  uint16_t r = 0;
  for (int i = 0; i < m; i++) r |= (uint16_t)(((a >> i) & 1) << (m - 1 - i));
  return r;
}

// Semi-systematic step of the "f" variants (mc:crypto_kem/348864f/vec/pk_gen.c,
// mov_columns): with the first R = mt - 32 columns reduced, the last 32 rows'
// 32 x 64 block at columns R .. R+63 gives leftmost pivot columns c_0 < ... <
// c_31 (rejection below rank 32); pivots = sum 2^c_j, and for j = 0..31 in
// turn columns R+j, R+c_j of every row and pi[R+j], pi[R+c_j] trade places.
static bool move_pivot_columns(const gmc_setinfo &S, std::vector<uint64_t> &mat, int rw, std::vector<int16_t> &pi,
                               uint64_t *pivots) {
  const int R = S.mt - 32;
  auto bit = [&](int r, int c) { return (int)((mat[(size_t)r * rw + c / 64] >> (c % 64)) & 1); };
  uint64_t buf[32];
  int c_of[32];
  for (int i = 0; i < 32; i++) {
    buf[i] = 0;
    for (int c = 0; c < 64; c++)
      if (bit(R + i, R + c)) buf[i] |= 1ull << c;
  }
  *pivots = 0;
  for (int i = 0; i < 32; i++) {
    uint64_t t = 0;
    for (int j = i; j < 32; j++) t |= buf[j];
    if (!t) return false;
    const int s = __builtin_ctzll(t);
    c_of[i] = s;
    *pivots |= 1ull << s;
    int piv = i;
    while (!((buf[piv] >> s) & 1)) piv++;
    std::swap(buf[i], buf[piv]);
    for (int j = i + 1; j < 32; j++)
      if ((buf[j] >> s) & 1) buf[j] ^= buf[i];
  }
  for (int j = 0; j < 32; j++) {
    const int a = R + j, b = R + c_of[j];
    if (a == b) continue;
    std::swap(pi[a], pi[b]);
    for (int r = 0; r < S.mt; r++)
      if (bit(r, a) != bit(r, b)) {
        mat[(size_t)r * rw + a / 64] ^= 1ull << (a % 64);
        mat[(size_t)r * rw + b / 64] ^= 1ull << (b % 64);
      }
  }
  return true;
}

static bool public_key(const gmc_setinfo &S, const HostField &F, const uint16_t *g, const uint32_t *perm,
                       std::vector<int16_t> &pi, uint8_t *pk, bool semi, uint64_t *pivots) {
  const int m = S.m, n = S.n, t = S.t, mt = S.mt, q = S.q;
  std::vector<uint64_t> buf(q);
  for (int i = 0; i < q; i++) buf[i] = ((uint64_t)perm[i] << 31) | (uint64_t)i;
  std::sort(buf.begin(), buf.end());
  for (int i = 1; i < q; i++)
    if ((buf[i - 1] >> 31) == (buf[i] >> 31)) return false;
  pi.resize(q);
  for (int i = 0; i < q; i++) pi[i] = (int16_t)(buf[i] & (uint64_t)(q - 1));
  std::vector<uint16_t> L(n), inv(n);
  for (int i = 0; i < n; i++) {
    L[i] = bitrev_m((uint16_t)pi[i], m);
    uint16_t v = g[t];
    for (int j = t - 1; j >= 0; j--) v = (uint16_t)(F.mul(v, L[i]) ^ g[j]);
    inv[i] = F.inv(v);
  }
  const int rw = (n + 63) / 64;
  std::vector<uint64_t> mat((size_t)mt * rw, 0);
  for (int i = 0; i < t; i++) {
    for (int j = 0; j < n; j++)
      for (int b = 0; b < m; b++)
        if ((inv[j] >> b) & 1) mat[(size_t)(i * m + b) * rw + j / 64] |= 1ull << (j % 64);
    for (int j = 0; j < n; j++) inv[j] = F.mul(inv[j], L[j]);
  }
  for (int row = 0; row < mt; row++) {
    if (semi && row == mt - 32 && !move_pivot_columns(S, mat, rw, pi, pivots)) return false;
    const int w = row / 64;
    const uint64_t bit = 1ull << (row % 64);
    int piv = -1;
    for (int r = row; r < mt; r++)
      if (mat[(size_t)r * rw + w] & bit) { piv = r; break; }
    if (piv < 0) return false;  // not systematic
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
    uint8_t *out = pk + (size_t)r * S.pk_row_bytes;
    memset(out, 0, S.pk_row_bytes);
    for (int j = 0; j < S.k; j++) {
      const int col = mt + j;
      if ((mat[(size_t)r * rw + col / 64] >> (col % 64)) & 1) out[j / 8] |= (uint8_t)(1 << (j % 8));
    }
  }
  return true;
}

// ---------------------------------------------------------------- control bits
// Nassimi-Sahni / Bernstein recursion; the sort steps are kept identical to the
// library's (control bits are not unique for a permutation). Packed values
// stay below 2^31, so sorting them unsigned equals the library's int32 sort.
static void cb_recursion(uint8_t *out, long long pos, long long step, const int16_t *pi, int w, long n,
                         std::vector<uint32_t> &A, std::vector<uint32_t> &B) {
  if (w == 1) {
    out[pos >> 3] ^= (uint8_t)(pi[0] << (pos & 7));
    return;
  }
  auto srt = [&](std::vector<uint32_t> &v) { std::sort(v.begin(), v.begin() + n); };
  for (long x = 0; x < n; x++) A[x] = ((uint32_t)(pi[x] ^ 1) << 16) | (uint32_t)pi[x ^ 1];
  srt(A);
  for (long x = 0; x < n; x++) {
    uint32_t px = A[x] & 0xffff, cx = std::min<uint32_t>(px, (uint32_t)x);
    B[x] = (px << 16) | cx;
  }
  for (long x = 0; x < n; x++) A[x] = (A[x] << 16) | (uint32_t)x;
  srt(A);
  for (long x = 0; x < n; x++) A[x] = (A[x] << 16) + (B[x] >> 16);
  srt(A);
  if (w <= 10) {
    for (long x = 0; x < n; x++) B[x] = ((A[x] & 0xffff) << 10) | (B[x] & 0x3ff);
    for (int i = 1; i < w - 1; i++) {
      for (long x = 0; x < n; x++) A[x] = ((B[x] & ~0x3ffu) << 6) | (uint32_t)x;
      srt(A);
      for (long x = 0; x < n; x++) A[x] = (A[x] << 20) | B[x];
      srt(A);
      for (long x = 0; x < n; x++) {
        uint32_t ppcp = A[x] & 0xfffff, ppc = (A[x] & 0xffc00) | (B[x] & 0x3ff);
        B[x] = std::min(ppc, ppcp);
      }
    }
    for (long x = 0; x < n; x++) B[x] &= 0x3ff;
  } else {
    for (long x = 0; x < n; x++) B[x] = (A[x] << 16) | (B[x] & 0xffff);
    for (int i = 1; i < w - 1; i++) {
      for (long x = 0; x < n; x++) A[x] = (B[x] & ~0xffffu) | (uint32_t)x;
      srt(A);
      for (long x = 0; x < n; x++) A[x] = (A[x] << 16) | (B[x] & 0xffff);
      if (i < w - 2) {
        for (long x = 0; x < n; x++) B[x] = (A[x] & ~0xffffu) | (B[x] >> 16);
        srt(B);
        for (long x = 0; x < n; x++) B[x] = (B[x] << 16) | (A[x] & 0xffff);
      }
      srt(A);
      for (long x = 0; x < n; x++) {
        uint32_t cp = (B[x] & ~0xffffu) | (A[x] & 0xffff);
        B[x] = std::min(B[x], cp);
      }
    }
    for (long x = 0; x < n; x++) B[x] &= 0xffff;
  }
  for (long x = 0; x < n; x++) A[x] = ((uint32_t)pi[x] << 16) + (uint32_t)x;
  srt(A);
  for (long j = 0; j < n / 2; j++) {
    const long z = 2 * j;
    const uint32_t fj = B[z] & 1, Fz = (uint32_t)z + fj, Fz1 = Fz ^ 1;
    out[pos >> 3] ^= (uint8_t)(fj << (pos & 7));
    pos += step;
    B[z] = (A[z] << 16) | Fz;
    B[z + 1] = (A[z + 1] << 16) | Fz1;
  }
  srt(B);
  pos += (2 * w - 3) * step * (n / 2);
  for (long k = 0; k < n / 2; k++) {
    const long y = 2 * k;
    const uint32_t lk = B[y] & 1, Ly = (uint32_t)y + lk, Ly1 = Ly ^ 1;
    out[pos >> 3] ^= (uint8_t)(lk << (pos & 7));
    pos += step;
    A[y] = (Ly << 16) | (B[y] & 0xffff);
    A[y + 1] = (Ly1 << 16) | (B[y + 1] & 0xffff);
  }
  srt(A);
  pos -= (2 * w - 2) * step * (n / 2);
  std::vector<int16_t> sub(n);
  for (long j = 0; j < n / 2; j++) {
    sub[j] = (int16_t)((A[2 * j] & 0xffff) >> 1);
    sub[j + n / 2] = (int16_t)((A[2 * j + 1] & 0xffff) >> 1);
  }
  cb_recursion(out, pos, step * 2, sub.data(), w - 1, n / 2, A, B);
  cb_recursion(out, pos + step, step * 2, sub.data() + n / 2, w - 1, n / 2, A, B);
}

static bool control_bits(uint8_t *out, const std::vector<int16_t> &pi, int w) {
  const long n = 1L << w;
  memset(out, 0, (size_t)(((2 * w - 1) * n / 2 + 7) / 8));
  std::vector<uint32_t> A(n), B(n);
  cb_recursion(out, 0, 1, pi.data(), w, n, A, B);
  // the encoded permutation must be pi: apply the layers to the identity
  std::vector<int16_t> p(n);
  for (long i = 0; i < n; i++) p[i] = (int16_t)i;
  const uint8_t *cb = out;
  auto layer = [&](int s) {
    const int stride = 1 << s;
    int idx = 0;
    for (long i = 0; i < n; i += 2 * stride)
      for (int j = 0; j < stride; j++, idx++)
        if ((cb[idx >> 3] >> (idx & 7)) & 1) std::swap(p[i + j], p[i + j + stride]);
    cb += n >> 4;
  };
  for (int s = 0; s < w; s++) layer(s);
  for (int s = w - 2; s >= 0; s--) layer(s);
  for (long i = 0; i < n; i++)
    if (p[i] != pi[i]) return false;
  return true;
}

int host_keypair(int set, uint8_t *pk, uint8_t *sk, const uint8_t delta32[32], bool semi) {
  const gmc_setinfo &S = set_info(set);
  const HostField &F = host_field(S.m);
  uint8_t seed[33];
  seed[0] = 64;
  memcpy(seed + 1, delta32, 32);
  const size_t rlen = (size_t)S.e_bytes + 4 * (size_t)S.q + 2 * (size_t)S.t + 32;
  std::vector<uint8_t> r(rlen);
  std::vector<uint16_t> f(S.t), g(S.t + 1);
  std::vector<uint32_t> perm(S.q);
  std::vector<int16_t> pi;
  for (int attempt = 0; attempt < 100000; attempt++) {
    host_shake256(r.data(), rlen, seed, 33);
    memcpy(sk, seed + 1, 32);
    memcpy(seed + 1, r.data() + rlen - 32, 32);
    const uint8_t *rp = r.data() + rlen - 32 - 2 * S.t;
    for (int i = 0; i < S.t; i++) f[i] = (uint16_t)((rp[2 * i] | (rp[2 * i + 1] << 8)) & (S.q - 1));
    if (!min_poly(set, F, S.t, f.data(), g.data())) continue;
    g[S.t] = 1;
    uint8_t *skp = sk + 40;
    for (int i = 0; i < S.t; i++) {
      skp[2 * i] = (uint8_t)g[i];
      skp[2 * i + 1] = (uint8_t)(g[i] >> 8);
    }
    skp += S.irr_bytes;
    rp -= 4 * (size_t)S.q;
    for (int i = 0; i < S.q; i++)
      perm[i] = (uint32_t)rp[4 * i] | ((uint32_t)rp[4 * i + 1] << 8) | ((uint32_t)rp[4 * i + 2] << 16) |
                ((uint32_t)rp[4 * i + 3] << 24);
    uint64_t pivots = 0xFFFFFFFFull;
    if (!public_key(S, F, g.data(), perm.data(), pi, pk, semi, &pivots)) continue;
    if (!control_bits(skp, pi, S.m)) return -1;
    skp += S.cond_bytes;
    memcpy(skp, r.data(), S.e_bytes);
    for (int i = 0; i < 8; i++) sk[32 + i] = (uint8_t)(pivots >> (8 * i));  // 0xFFFFFFFF unless semi-systematic
    return 0;
  }
  return -1;
}

}  // namespace gmc
