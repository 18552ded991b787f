// Encapsulation kernels: fixed-weight sampling (thread per request) and the
// finalize step (ciphertext assembly + session-key hash).
//
// Reference behaviour: gen_e / syndrome / operation_enc of libmceliece
// (mceliece-gpu-params/ref/348864.cuh:3434-3565, 8192128.cuh:5967-6006;
// mc:crypto_kem/348864/vec/encrypt.c:41-132, kem_enc.c:18).
#include "kernels.h"
#include "device_common.cuh"

namespace gmc {

// ---------------------------------------------------------------- sampling
// One thread per request. Randomness is the per-request seed chain:
// attempt j draws SHAKE256({64} || state, cand_bytes) and the next state is
// the first 32 bytes of that draw. Candidates are little-endian 16-bit words
// masked to m bits; for n < 2^m the first t values below n are kept, else all
// t. A repeated position rejects the attempt. Duplicate detection uses a
// per-thread n-bit bitmap in shared memory (equivalent to the library's
// sort-and-compare: only the set of positions matters). The bitmap is the
// error vector e itself and is written out with the block's coalesced store.
template <int SET>
__global__ void __launch_bounds__(kSampleThreadsMax) sample_kernel(const uint8_t *__restrict__ seeds, const Segs segs,
                                                                uint32_t *__restrict__ E, int lde,
                                                                uint32_t *__restrict__ Ens, int ldx) {
  using p = P<SET>;
  constexpr int EWS = p::ew | 1;  // odd stride: bitmaps of neighbouring threads start in different banks
  extern __shared__ uint32_t sm[];
  uint32_t *bm = sm + threadIdx.x * EWS;
  const long long N = seg_rows(segs);
  const long long op0 = (long long)blockIdx.x * blockDim.x;
  const long long op = op0 + threadIdx.x;
  int seg;
  const bool live = seg_live(segs, op, &seg);

  for (int w = 0; w < p::ew; w++) bm[w] = 0;

  if (live) {
    uint64_t st[4];
    const uint8_t *sd = seeds + 32 * op;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      uint64_t v = 0;
#pragma unroll
      for (int b = 0; b < 8; b++) v |= (uint64_t)sd[8 * i + b] << (8 * b);
      st[i] = v;
    }
    constexpr int ncand = p::cand_bytes / 2;     // 16-bit candidates per attempt
    constexpr int nlanes = (ncand + 3) / 4;      // output lanes holding them
    constexpr uint32_t mask = p::q - 1;
#pragma unroll 1
    for (int attempt = 0; attempt < 1000000; attempt++) {
      uint64_t s[25];
#pragma unroll
      for (int i = 0; i < 25; i++) s[i] = 0;
      s[0] = 64ull | (st[0] << 8);
      s[1] = (st[0] >> 56) | (st[1] << 8);
      s[2] = (st[1] >> 56) | (st[2] << 8);
      s[3] = (st[2] >> 56) | (st[3] << 8);
      s[4] = (st[3] >> 56) | (0x1Full << 8);
      s[16] = 0x8000000000000000ull;
      keccak_f1600(s);
      uint64_t nst[4] = {s[0], s[1], s[2], s[3]};
      int count = 0;
      bool bad = false;
#pragma unroll 1
      for (int base = 0; base < nlanes && count < p::t && !bad; base += 17) {
        if (base) keccak_f1600(s);
#pragma unroll
        for (int i = 0; i < 17; i++) {
          if (base + i < nlanes) {
            uint64_t l = s[i];
#pragma unroll
            for (int h = 0; h < 4; h++) {
              uint32_t v = (uint32_t)(l >> (16 * h)) & mask;
              bool take = (4 * (base + i) + h < ncand) && (count < p::t) && !bad &&
                          (p::full || v < (uint32_t)p::n);
              if (take) {
                uint32_t word = bm[v >> 5], bit = 1u << (v & 31);
                if (word & bit) bad = true;
                else { bm[v >> 5] = word | bit; count++; }
              }
            }
          }
        }
      }
      if (!bad && count == p::t) break;
      for (int w = 0; w < p::ew; w++) bm[w] = 0;
      st[0] = nst[0]; st[1] = nst[1]; st[2] = nst[2]; st[3] = nst[3];
    }
  }
  __shared__ unsigned char live_rows[kSampleThreadsMax];
  live_rows[threadIdx.x] = live;
  __syncthreads();
  // coalesced copy-out of the block's error vectors, and of e[mt:n] shifted
  // to bit 0 (the GEMM operand); rows past a segment's live requests are skipped
  const int nthreads = blockDim.x;
  const long long nops = (N - op0) < nthreads ? (N - op0) : nthreads;
  for (long long idx = threadIdx.x; idx < nops * p::ew; idx += nthreads) {
    int r = (int)(idx / p::ew), w = (int)(idx % p::ew);
    if (live_rows[r]) E[(op0 + r) * lde + w] = sm[r * EWS + w];
  }
  constexpr int sh = p::mt % 32, w0 = p::mt / 32;
  for (long long idx = threadIdx.x; idx < nops * p::kw; idx += nthreads) {
    int r = (int)(idx / p::kw), w = (int)(idx % p::kw);
    if (!live_rows[r]) continue;
    uint32_t lo = sm[r * EWS + w0 + w];
    uint32_t hi = (w0 + w + 1 < p::ew) ? sm[r * EWS + w0 + w + 1] : 0u;
    Ens[(op0 + r) * ldx + w] = sh ? ((lo >> sh) | (hi << (32 - sh))) : lo;
  }
}

// ---------------------------------------------------------------- finalize
// c = e[0:mt] xor (T e[mt:n]); K = SHAKE256(1 || e || c). When the public
// key's padding bits are set (6960119 only), c and K are zeroed
// (mc:crypto_kem/6960119/vec/kem_enc.c:21-66).
template <int SET>
__global__ void __launch_bounds__(kTailThreads) finalize_kernel(const uint32_t *__restrict__ E, int lde,
                                                                const uint32_t *__restrict__ S, int lds,
                                                                uint8_t *__restrict__ C, uint8_t *__restrict__ K,
                                                                const Segs segs, uint32_t pk_bad_mask) {
  using p = P<SET>;
  const long long op = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int seg;
  if (!seg_live(segs, op, &seg)) return;
  const bool pk_bad = (pk_bad_mask >> seg) & 1u;
  const uint32_t *e = E + op * lde;
  const uint32_t *sy = S + op * lds;
  // c words (mt bits, tail bits cleared)
  uint32_t cw[p::cw];
#pragma unroll
  for (int w = 0; w < p::cw; w++) {
    uint32_t v = (w < p::mw) ? (e[w] ^ sy[w]) : 0u;
    if (w == p::mt / 32 && (p::mt % 32)) v &= (1u << (p::mt % 32)) - 1u;
    if (w > (p::mt - 1) / 32) v = 0;
    cw[w] = v;
  }
  // preimage byte x (x < pre_bytes): 1 | e bytes | c bytes
  auto ebyte = [&](int x) -> uint32_t { return (e[x >> 2] >> (8 * (x & 3))) & 0xFFu; };
  auto cbyte = [&](int x) -> uint32_t {
    uint32_t r = 0;
#pragma unroll
    for (int w = 0; w < p::cw; w++)
      if (w == (x >> 2)) r = (cw[w] >> (8 * (x & 3))) & 0xFFu;
    return r;
  };
  auto lane = [&](int i) -> uint64_t {
    const int o = 8 * i;
    if (o >= 8 && o + 7 <= p::e_bytes) {
      // bytes o..o+7 are e[o-1 .. o+6]: funnel of three 32-bit words
      int x = o - 1;  // x % 4 == 3
      uint32_t w0 = e[x >> 2], w1 = e[(x >> 2) + 1], w2 = e[(x >> 2) + 2];
      uint64_t lo = (uint64_t)(w0 >> 24) | ((uint64_t)w1 << 8) | ((uint64_t)(w2 & 0xFFFFFFu) << 40);
      return lo;
    }
    uint64_t v = 0;
    for (int b = 0; b < 8; b++) {
      int x = o + b;
      uint32_t byte;
      if (x == 0) byte = 1;
      else if (x <= p::e_bytes) byte = ebyte(x - 1);
      else if (x < p::pre_bytes) byte = cbyte(x - 1 - p::e_bytes);
      else byte = 0;
      v |= (uint64_t)byte << (8 * b);
    }
    return v;
  };
  uint64_t h[4];
  shake256_32<p::pre_bytes>(h, lane);
  uint8_t *c = C + op * p::synd_bytes;
  uint8_t *k = K + op * 32;
  for (int x = 0; x < p::synd_bytes; x++) c[x] = pk_bad ? 0 : (uint8_t)cbyte(x);
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int b = 0; b < 8; b++) k[8 * i + b] = pk_bad ? 0 : (uint8_t)(h[i] >> (8 * b));
}

// ---------------------------------------------------------------- launchers
template <int SET>
static int sample_smem_bytes(int threads) { return threads * (P<SET>::ew | 1) * 4; }

template <int SET>
cudaError_t launch_sample(const uint8_t *seeds, const Segs &segs, uint32_t *E, int lde, uint32_t *Ens, int ldx,
                          int threads, cudaStream_t st) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  if (threads != 32 && threads != 64 && threads != 128) return cudaErrorInvalidValue;
  const int smem = sample_smem_bytes<SET>(threads);
  cudaError_t err = cudaFuncSetAttribute(sample_kernel<SET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sample_smem_bytes<SET>(kSampleThreadsMax));
  if (err != cudaSuccess) return err;
  long long blocks = (N + threads - 1) / threads;
  sample_kernel<SET><<<(unsigned)blocks, threads, smem, st>>>(seeds, segs, E, lde, Ens, ldx);
  return cudaGetLastError();
}

template <int SET>
cudaError_t launch_finalize(const uint32_t *E, int lde, const uint32_t *S, int lds, uint8_t *C, uint8_t *K,
                            const Segs &segs, uint32_t pk_bad_mask, cudaStream_t st) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  long long blocks = (N + kTailThreads - 1) / kTailThreads;
  finalize_kernel<SET><<<(unsigned)blocks, kTailThreads, 0, st>>>(E, lde, S, lds, C, K, segs, pk_bad_mask);
  return cudaGetLastError();
}

#define GMC_INST_ENC(SET)                                                                                        \
  template cudaError_t launch_sample<SET>(const uint8_t *, const Segs &, uint32_t *, int, uint32_t *, int, int,  \
                                          cudaStream_t);                                                         \
  template cudaError_t launch_finalize<SET>(const uint32_t *, int, const uint32_t *, int, uint8_t *, uint8_t *, \
                                            const Segs &, uint32_t, cudaStream_t);
GMC_INST_ENC(0)
GMC_INST_ENC(1)
GMC_INST_ENC(2)
GMC_INST_ENC(3)
GMC_INST_ENC(4)

}  // namespace gmc
