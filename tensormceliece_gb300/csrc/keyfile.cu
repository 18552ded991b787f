// Persistence of resident keys: gmc_key_export writes a loaded key's device
// state (the tables gmc_pk_load / gmc_sk_load build on the host, once per key;
// ~2.8 MB for an 8192128 secret key) into a self-checking byte string;
// gmc_key_import re-creates the handle from it with plain copies after
// verifying the checksum, without rebuilding the tables.
//
// Format (little-endian): header, then the sections in order
//   public key: T (rows_pad x lda u32), TT ((k+1) x ldtt u32)
//   secret key: F (frows_pad x ldf u32), support tables (3n + 2^m u16),
//               s (n/8 bytes zero-padded to 16), HT (n x ldh u32),
//               the sk's Benes control bits (for constant-time decapsulation)
// The header's checksum is SHAKE256 of the whole string with the checksum
// field zeroed; import rejects any string whose magic, version, set, sizes or
// checksum do not match.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/gmc.h"
#include "engine_internal.h"
#include "host_keys.h"

namespace gmc {
// SHAKE256 on the host, for the key string's checksum (FIPS 202: Keccak-f[1600],
// rate 136 bytes, domain byte 0x1F)
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

}  // namespace gmc

namespace {
using namespace gmc;

constexpr char kMagic[8] = {'G', 'M', 'C', 'K', 'E', 'Y', '0', '1'};
constexpr uint32_t kVersion = 2;  // 2: secret keys carry their Benes control bits

struct KeyHeader {
  char magic[8];
  uint32_t version;
  int32_t set, variant, kind;
  int32_t lda, rows_pad, kw_pad, pad_bad, ldtt;  // public key
  int32_t ldf, frows_pad, cw_pad, ldh;           // secret key
  uint64_t section[5];                           // bytes of each section
  uint8_t checksum[32];
};
static_assert(sizeof(KeyHeader) % 8 == 0, "header keeps the sections 8-byte aligned");

int kf_fail(int code, const std::string &msg) {
  set_last_error(msg.c_str());
  return code;
}

size_t s_alloc_bytes(const gmc_setinfo &S) { return ((size_t)S.e_bytes + 15) / 16 * 16; }

// Section sizes implied by a header's dimensions. The dimensions must be
// exactly the ones gmc_pk_load / gmc_sk_load give a key of this set (the
// kernels assume that layout: a smaller padded width would make the GEMM skip
// words of the key or ciphertext and return wrong session keys with rc = 0),
// and the public key's padding flag must be 0 or 1.
bool section_sizes(const KeyHeader &h, uint64_t out[5]) {
  const gmc_setinfo &S = set_info(h.set);
  memset(out, 0, 5 * sizeof(uint64_t));
  if (h.kind == 0) {
    const int kw_pad = round_up((S.k + 31) / 32, kGemmKTile);
    const int ldtt = round_up((S.mt + 31) / 32, 32) < 64 ? 64 : round_up((S.mt + 31) / 32, 32);
    if (h.kw_pad != kw_pad || h.lda != kw_pad || h.rows_pad != round_up(S.mt, kGemmRowTile) || h.ldtt != ldtt ||
        (h.pad_bad != 0 && h.pad_bad != 1))
      return false;
    out[0] = (uint64_t)h.rows_pad * h.lda * 4;
    out[1] = (uint64_t)(S.k + 1) * h.ldtt * 4;
  } else {
    const int cw_pad = round_up((S.synd_bytes + 3) / 4, kGemmKTile);
    if (h.cw_pad != cw_pad || h.ldf != cw_pad || h.frows_pad != round_up(2 * S.t * S.m, kGemmRowTile) ||
        h.ldh != round_up((S.t * S.m + 31) / 32, 32))
      return false;
    out[0] = (uint64_t)h.frows_pad * h.ldf * 4;
    out[1] = (3ull * S.n + S.q) * 2;
    out[2] = s_alloc_bytes(S);
    out[3] = (uint64_t)S.n * h.ldh * 4;
    out[4] = (uint64_t)S.cond_bytes;
  }
  return true;
}

void checksum(const uint8_t *buf, long long len, uint8_t out[32]) {
  std::vector<uint8_t> copy(buf, buf + len);
  memset(copy.data() + offsetof(KeyHeader, checksum), 0, 32);
  host_shake256(out, 32, copy.data(), (size_t)len);
}
}  // namespace

extern "C" long long gmc_key_export(const gmc_key *key, unsigned char *buf, long long len) {
  if (!key) return kf_fail(GMC_EINVAL, "gmc_key_export: null key");
  KeyHeader h{};
  memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.set = key->set;
  h.variant = key->variant;
  h.kind = key->kind;
  h.lda = key->lda; h.rows_pad = key->rows_pad; h.kw_pad = key->kw_pad; h.pad_bad = key->pad_bad; h.ldtt = key->ldtt;
  h.ldf = key->ldf; h.frows_pad = key->frows_pad; h.cw_pad = key->cw_pad; h.ldh = key->dk.ldh;
  if (!section_sizes(h, h.section)) return kf_fail(GMC_EKEY, "gmc_key_export: key dimensions out of range");
  const long long total = (long long)sizeof(KeyHeader) +
                          (long long)(h.section[0] + h.section[1] + h.section[2] + h.section[3] + h.section[4]);
  if (!buf) return total;
  if (len < total) return kf_fail(GMC_EINVAL, "gmc_key_export: buffer too small");
  if (key->kind == 1 && !key->cond) return kf_fail(GMC_EKEY, "gmc_key_export: key without control bits");
  const void *src[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  if (key->kind == 0) {
    src[0] = key->T;
    src[1] = key->TT;
  } else {
    src[0] = key->F;
    src[1] = key->tabs;
    src[2] = key->s;
    src[3] = key->HT;
    src[4] = key->cond;
  }
  unsigned char *p = buf + sizeof(KeyHeader);
  for (int i = 0; i < 5; i++) {
    if (!h.section[i]) continue;
    cudaError_t e = cudaMemcpy(p, src[i], h.section[i], cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return kf_fail(GMC_ECUDA, std::string("gmc_key_export: ") + cudaGetErrorString(e));
    p += h.section[i];
  }
  memcpy(buf, &h, sizeof h);
  uint8_t sum[32];
  checksum(buf, total, sum);
  memcpy(buf + offsetof(KeyHeader, checksum), sum, 32);
  return total;
}

extern "C" int gmc_key_import(gmc_key **out, const unsigned char *buf, long long len) {
  if (!out || !buf || len < (long long)sizeof(KeyHeader)) return kf_fail(GMC_EINVAL, "gmc_key_import: bad argument");
  *out = nullptr;
  KeyHeader h;
  memcpy(&h, buf, sizeof h);
  if (memcmp(h.magic, kMagic, 8) || h.version != kVersion) return kf_fail(GMC_EKEY, "gmc_key_import: not a key string");
  if (h.set < 0 || h.set >= GMC_NSETS || h.variant < 0 || h.variant > 3 || (h.kind != 0 && h.kind != 1))
    return kf_fail(GMC_EKEY, "gmc_key_import: bad set, variant or kind");
  uint64_t sz[5];
  if (!section_sizes(h, sz) || memcmp(sz, h.section, sizeof sz))
    return kf_fail(GMC_EKEY, "gmc_key_import: section sizes do not match the key's dimensions");
  const long long total = (long long)sizeof(KeyHeader) + (long long)(sz[0] + sz[1] + sz[2] + sz[3] + sz[4]);
  if (len != total) return kf_fail(GMC_EKEY, "gmc_key_import: wrong length");
  uint8_t sum[32];
  checksum(buf, total, sum);
  if (memcmp(sum, h.checksum, 32)) return kf_fail(GMC_EKEY, "gmc_key_import: checksum mismatch");
  const gmc_setinfo &S = set_info(h.set);
  gmc_key *k = new gmc_key();
  k->a8_mu = new std::mutex();
  k->set = h.set;
  k->variant = h.variant;
  k->pc = h.variant & 1;
  k->kind = h.kind;
  cudaGetDevice(&k->device);
  void **dst[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  if (h.kind == 0) {
    k->lda = h.lda; k->rows_pad = h.rows_pad; k->kw_pad = h.kw_pad; k->pad_bad = h.pad_bad; k->ldtt = h.ldtt;
    dst[0] = (void **)&k->T;
    dst[1] = (void **)&k->TT;
  } else {
    k->ldf = h.ldf; k->frows_pad = h.frows_pad; k->cw_pad = h.cw_pad;
    dst[0] = (void **)&k->F;
    dst[1] = (void **)&k->tabs;
    dst[2] = (void **)&k->s;
    dst[3] = (void **)&k->HT;
    dst[4] = (void **)&k->cond;
  }
  const unsigned char *p = buf + sizeof(KeyHeader);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 5 && e == cudaSuccess; i++) {
    if (!sz[i]) continue;
    e = cudaMalloc(dst[i], sz[i]);
    if (e == cudaSuccess) e = cudaMemcpy(*dst[i], p, sz[i], cudaMemcpyHostToDevice);
    p += sz[i];
  }
  if (e != cudaSuccess) {
    for (int i = 0; i < 5; i++)
      if (dst[i] && *dst[i]) cudaFree(*dst[i]);
    delete k->a8_mu;
    delete k;
    return kf_fail(GMC_ECUDA, std::string("gmc_key_import: ") + cudaGetErrorString(e));
  }
  if (h.kind == 1) {
    const size_t n = S.n;
    k->dk.L = k->tabs;
    k->dk.LL = k->tabs + n;
    k->dk.LW2 = k->tabs + 2 * n;
    k->dk.invL = k->tabs + 3 * n;
    k->dk.s = k->s;
    k->dk.HT = k->HT;
    k->dk.ldh = h.ldh;
    k->dk.cond = k->cond;
  }
  *out = k;
  return GMC_OK;
}
