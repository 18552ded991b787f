// Device primitives shared by the encapsulation and decapsulation kernels:
// Keccak-f[1600] / SHAKE256 (thread-per-request), GF(2^m) log/antilog helpers.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "params.h"

namespace gmc {

// ---------------------------------------------------------------- Keccak
// FIPS 202 round constants, produced at compile time by the degree-8 LFSR
// x^8 + x^6 + x^5 + x^4 + 1 (FIPS 202, algorithm 5).
struct KeccakRC {
  uint64_t v[24];
  constexpr KeccakRC() : v() {
    unsigned r = 1;
    for (int ir = 0; ir < 24; ir++) {
      uint64_t c = 0;
      for (int j = 0; j < 7; j++) {
        if (r & 1) c |= 1ull << ((1 << j) - 1);
        r = ((r << 1) ^ ((r & 0x80) ? 0x71 : 0)) & 0xFF;
      }
      v[ir] = c;
    }
  }
};
static constexpr KeccakRC kKeccakRC{};
static __constant__ uint64_t c_keccak_rc[24] = {
    kKeccakRC.v[0],  kKeccakRC.v[1],  kKeccakRC.v[2],  kKeccakRC.v[3],  kKeccakRC.v[4],  kKeccakRC.v[5],
    kKeccakRC.v[6],  kKeccakRC.v[7],  kKeccakRC.v[8],  kKeccakRC.v[9],  kKeccakRC.v[10], kKeccakRC.v[11],
    kKeccakRC.v[12], kKeccakRC.v[13], kKeccakRC.v[14], kKeccakRC.v[15], kKeccakRC.v[16], kKeccakRC.v[17],
    kKeccakRC.v[18], kKeccakRC.v[19], kKeccakRC.v[20], kKeccakRC.v[21], kKeccakRC.v[22], kKeccakRC.v[23]};

__device__ __forceinline__ uint64_t rotl64(uint64_t x, int n) {
  return (x << n) | (x >> (64 - n));
}

// One Keccak-f[1600] permutation on 25 lanes held in registers. The
// rotation offsets follow rho's (x,y) walk; pi maps lane (x,y) to (y,2x+3y).
__device__ __forceinline__ void keccak_f1600(uint64_t A[25]) {
#pragma unroll 1
  for (int round = 0; round < 24; ++round) {
    uint64_t C0 = A[0] ^ A[5] ^ A[10] ^ A[15] ^ A[20];
    uint64_t C1 = A[1] ^ A[6] ^ A[11] ^ A[16] ^ A[21];
    uint64_t C2 = A[2] ^ A[7] ^ A[12] ^ A[17] ^ A[22];
    uint64_t C3 = A[3] ^ A[8] ^ A[13] ^ A[18] ^ A[23];
    uint64_t C4 = A[4] ^ A[9] ^ A[14] ^ A[19] ^ A[24];
    uint64_t D0 = C4 ^ rotl64(C1, 1);
    uint64_t D1 = C0 ^ rotl64(C2, 1);
    uint64_t D2 = C1 ^ rotl64(C3, 1);
    uint64_t D3 = C2 ^ rotl64(C4, 1);
    uint64_t D4 = C3 ^ rotl64(C0, 1);
    // theta + rho + pi: B[y + 5*((2x+3y)%5)] = rot(A[x+5y] ^ D[x], r(x,y))
    uint64_t B0 = A[0] ^ D0;
    uint64_t B10 = rotl64(A[1] ^ D1, 1);
    uint64_t B20 = rotl64(A[2] ^ D2, 62);
    uint64_t B5 = rotl64(A[3] ^ D3, 28);
    uint64_t B15 = rotl64(A[4] ^ D4, 27);
    uint64_t B16 = rotl64(A[5] ^ D0, 36);
    uint64_t B1 = rotl64(A[6] ^ D1, 44);
    uint64_t B11 = rotl64(A[7] ^ D2, 6);
    uint64_t B21 = rotl64(A[8] ^ D3, 55);
    uint64_t B6 = rotl64(A[9] ^ D4, 20);
    uint64_t B7 = rotl64(A[10] ^ D0, 3);
    uint64_t B17 = rotl64(A[11] ^ D1, 10);
    uint64_t B2 = rotl64(A[12] ^ D2, 43);
    uint64_t B12 = rotl64(A[13] ^ D3, 25);
    uint64_t B22 = rotl64(A[14] ^ D4, 39);
    uint64_t B23 = rotl64(A[15] ^ D0, 41);
    uint64_t B8 = rotl64(A[16] ^ D1, 45);
    uint64_t B18 = rotl64(A[17] ^ D2, 15);
    uint64_t B3 = rotl64(A[18] ^ D3, 21);
    uint64_t B13 = rotl64(A[19] ^ D4, 8);
    uint64_t B14 = rotl64(A[20] ^ D0, 18);
    uint64_t B24 = rotl64(A[21] ^ D1, 2);
    uint64_t B9 = rotl64(A[22] ^ D2, 61);
    uint64_t B19 = rotl64(A[23] ^ D3, 56);
    uint64_t B4 = rotl64(A[24] ^ D4, 14);
    // chi + iota
    A[0] = B0 ^ (~B1 & B2);  A[1] = B1 ^ (~B2 & B3);  A[2] = B2 ^ (~B3 & B4);
    A[3] = B3 ^ (~B4 & B0);  A[4] = B4 ^ (~B0 & B1);
    A[5] = B5 ^ (~B6 & B7);  A[6] = B6 ^ (~B7 & B8);  A[7] = B7 ^ (~B8 & B9);
    A[8] = B8 ^ (~B9 & B5);  A[9] = B9 ^ (~B5 & B6);
    A[10] = B10 ^ (~B11 & B12); A[11] = B11 ^ (~B12 & B13); A[12] = B12 ^ (~B13 & B14);
    A[13] = B13 ^ (~B14 & B10); A[14] = B14 ^ (~B10 & B11);
    A[15] = B15 ^ (~B16 & B17); A[16] = B16 ^ (~B17 & B18); A[17] = B17 ^ (~B18 & B19);
    A[18] = B18 ^ (~B19 & B15); A[19] = B19 ^ (~B15 & B16);
    A[20] = B20 ^ (~B21 & B22); A[21] = B21 ^ (~B22 & B23); A[22] = B22 ^ (~B23 & B24);
    A[23] = B23 ^ (~B24 & B20); A[24] = B24 ^ (~B20 & B21);
    A[0] ^= c_keccak_rc[round];
  }
}

// SHAKE256 of a message of compile-time length LEN bytes whose 8-byte
// little-endian lanes are produced by lane(i) (bytes past LEN must read as 0).
// Rate 17 lanes, domain byte 0x1F, final bit 0x80. Writes the first 32
// output bytes as 4 lanes.
template <int LEN, typename LaneFn>
__device__ __forceinline__ void shake256_32(uint64_t out[4], LaneFn lane) {
  constexpr int nfull = LEN / 136;           // full blocks
  constexpr int rem = LEN - nfull * 136;     // bytes in the final block
  uint64_t s[25];
#pragma unroll
  for (int i = 0; i < 25; i++) s[i] = 0;
#pragma unroll 1
  for (int b = 0; b < nfull; b++) {
#pragma unroll
    for (int i = 0; i < 17; i++) s[i] ^= lane(b * 17 + i);
    keccak_f1600(s);
  }
#pragma unroll
  for (int i = 0; i < 17; i++) {
    if (8 * i < rem) s[i] ^= lane(nfull * 17 + i);
    if (i == rem / 8) s[i] ^= 0x1Full << (8 * (rem % 8));
  }
  s[16] ^= 0x8000000000000000ull;
  keccak_f1600(s);
#pragma unroll
  for (int i = 0; i < 4; i++) out[i] = s[i];
}

// ---------------------------------------------------------------- KEM hash preimage
// 8 bytes of a little-endian word stream from byte offset off >= 0.
template <typename WordFn>
__device__ __forceinline__ uint64_t stream_u64(WordFn word, int off) {
  const int w = off >> 2, sh = 8 * (off & 3);
  uint64_t v = (uint64_t)word(w) | ((uint64_t)word(w + 1) << 32);
  if (sh) v = (v >> sh) | ((uint64_t)word(w + 2) << (64 - sh));
  return v;
}

// Lane i (bytes 8i .. 8i+7) of the session-key preimage b || e || c, where e
// has EB bytes given as 32-bit words by eword and c is given as 32-bit words
// by cword (zero past its length). Lanes inside e or inside c are funnels of
// three words; only the lane holding the e/c boundary is assembled bytewise.
template <int EB, typename EWord, typename CWord>
__device__ __forceinline__ uint64_t kem_preimage_lane(int i, uint32_t b, EWord eword, CWord cword) {
  const int o = 8 * i;
  if (o == 0) return (uint64_t)b | (stream_u64(eword, 0) << 8);
  if (o + 7 <= EB) return stream_u64(eword, o - 1);
  if (o >= 1 + EB) return stream_u64(cword, o - 1 - EB);
  uint64_t v = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int x = o + k - 1;  // byte of e || c
    const uint32_t byte = x < EB ? (eword(x >> 2) >> (8 * (x & 3))) : (cword((x - EB) >> 2) >> (8 * ((x - EB) & 3)));
    v |= (uint64_t)(byte & 0xFFu) << (8 * k);
  }
  return v;
}

// SHAKE256 (first 32 output bytes) of the KEM preimage b || e || c of PRE
// bytes, e of EB bytes, for the 32 requests of a warp (one per lane; every
// lane of the warp must call). erow is this lane's e as 32-bit words (zero
// past EB up to the next word); cword gives c as words (zero past c).
// The e words of each 136-byte absorb block are loaded for the whole warp as
// 35 independent loads per lane (word j of every request, and words 32..34 of
// the lane's own request), issued before the previous block is permuted so
// they land under the permutation, and handed over through shared memory
// (stage: 32 x 35 words, odd stride: no bank conflicts; rows: 32 pointers).
// Lanes outside e (the first, the e/c boundary, c) use kem_preimage_lane.
constexpr int kStageStride = 35;
template <int EB, int PRE, typename CWord>
__device__ __forceinline__ void kem_hash_staged(uint64_t out[4], uint32_t b, const uint32_t *erow, CWord cword,
                                                uint32_t *stage, const uint32_t **rows) {
  constexpr int EW = (EB + 3) / 4;
  constexpr int NB = PRE / 136 + 1;  // full blocks and the final (padded) one
  const int lane = threadIdx.x & 31;
  auto eword = [&](int w) -> uint32_t { return erow[w]; };
  rows[lane] = erow;
  __syncwarp();
  auto w_lo_of = [](int blk) { return blk > 0 ? (136 * blk - 1) >> 2 : 0; };
  uint32_t pf[32], pf2[3];
  auto prefetch = [&](int blk) {
    const int w_lo = w_lo_of(blk);
#pragma unroll
    for (int r = 0; r < 32; r++) {
      const int w = w_lo + lane;
      pf[r] = w < EW ? rows[r][w] : 0u;
    }
#pragma unroll
    for (int e = 0; e < 3; e++) {
      const int w = w_lo + 32 + e;
      pf2[e] = w < EW ? erow[w] : 0u;
    }
  };
  prefetch(0);
  uint64_t s[25];
#pragma unroll
  for (int i = 0; i < 25; i++) s[i] = 0;
#pragma unroll 1
  for (int blk = 0; blk < NB; blk++) {
    const int x0 = 136 * blk;
    const int w_lo = w_lo_of(blk);
    const bool in_e = x0 - 1 < EB;
    if (in_e) {
#pragma unroll
      for (int r = 0; r < 32; r++) stage[r * kStageStride + lane] = pf[r];
#pragma unroll
      for (int e = 0; e < 3; e++) stage[lane * kStageStride + 32 + e] = pf2[e];
      __syncwarp();
      if (blk + 1 < NB && 136 * (blk + 1) - 1 < EB) prefetch(blk + 1);
    }
    const int rem = (blk == NB - 1) ? PRE % 136 : 136;  // preimage bytes in this block
    const uint32_t *mine = stage + lane * kStageStride;
#pragma unroll
    for (int i = 0; i < 17; i++) {
      const int L = 17 * blk + i, o = 8 * L;
      uint64_t v = 0;
      if (8 * i < rem) {
        if (o > 0 && o + 7 <= EB) {
          const int rel = (o - 1) - 4 * w_lo, q = rel >> 2, sh = 8 * (rel & 3);
          v = (uint64_t)mine[q] | ((uint64_t)mine[q + 1] << 32);
          if (sh) v = (v >> sh) | ((uint64_t)mine[q + 2] << (64 - sh));
        } else {
          v = kem_preimage_lane<EB>(L, b, eword, cword);
        }
      }
      if (blk == NB - 1 && i == rem / 8) v ^= 0x1Full << (8 * (rem % 8));
      s[i] ^= v;
    }
    if (blk == NB - 1) s[16] ^= 0x8000000000000000ull;
    keccak_f1600(s);
    __syncwarp();  // every lane has read the staged words before they are replaced
  }
#pragma unroll
  for (int i = 0; i < 4; i++) out[i] = s[i];
}

// ---------------------------------------------------------------- GF(2^m)
// Log/antilog representation: log[0] = 2q-2 (sentinel), exp has 2q-1 entries
// with exp[2q-2] = 0, so a*b = exp[min(log a + log b, 2q-2)] without branches.
template <int M>
struct GFLog {
  static constexpr int q = 1 << M;
  static constexpr int zero_log = 2 * q - 2;
  static constexpr int exp_size = 2 * q - 1;
};

template <int M>
__device__ __forceinline__ uint16_t gf_mul_log(const uint16_t *__restrict__ ex, int la, int lb) {
  int s = la + lb;
  s = s < GFLog<M>::zero_log ? s : GFLog<M>::zero_log;
  return ex[s];
}

template <int M>
__device__ __forceinline__ uint16_t gf_mul(const uint16_t *__restrict__ ex, const uint16_t *__restrict__ lg,
                                           uint16_t a, uint16_t b) {
  return gf_mul_log<M>(ex, lg[a], lg[b]);
}

// x mod (2^M - 1) for x < 2^(2M+?) small: two folds leave a value <= 2^M,
// and exp[] is periodic with period 2^M - 1 over its first 2q-2 entries.
template <int M>
__device__ __forceinline__ int fold_mod(int x) {
  constexpr int mask = (1 << M) - 1;
  x = (x & mask) + (x >> M);
  x = (x & mask) + (x >> M);
  return x;
}

}  // namespace gmc
