// Encapsulation kernels: fixed-weight sampling (lane per request) and the
// finalize step (ciphertext assembly + session-key hash).
//
// Reference behaviour: gen_e / syndrome / operation_enc of libmceliece
// (mceliece-gpu-params/ref/348864.cuh:3434-3565, 8192128.cuh:5967-6006;
// mc:crypto_kem/348864/vec/encrypt.c:41-132, kem_enc.c:18).
#include <stdlib.h>

#include "kernels.h"
#include "device_common.cuh"

namespace gmc {

// ---------------------------------------------------------------- sampling
// Randomness is the per-request seed chain: attempt j draws
// SHAKE256({64} || state, cand_bytes) and the next state is the first 32
// bytes of that draw. Candidates are little-endian 16-bit words masked to m
// bits; for n < 2^m the first t values below n are kept, else all t. A
// repeated position rejects the attempt (only the set of positions matters,
// as in the library's sort-and-compare).
// Two forms: sample_pipe_kernel (below, the default) and this lane-per-request
// sample_kernel (GMC_SAMPLE_PIPELINE=0), which share the check and gather steps.
// Work split: each lane owns one request and runs its Keccak chain; lanes
// take requests from a launch-wide counter whenever their previous request
// is done, so a request that needs many attempts does not hold the warp's
// other lanes idle. Small batches leave lanes idle instead (only the first
// `lanes` of each warp take requests): more warps share the batch, so the
// Keccak latency is hidden across warps and the warp-serial repeat check and
// syndrome gather below run over fewer requests per warp. After every
// attempt the warp checks, one lane's
// candidates at a time, for repeats with a single n-bit bitmap per warp
// (atomicOr returns the previous word); on success that bitmap is the error
// vector e, written out by the whole warp (coalesced) together with e[mt:n]
// shifted to bit 0 (the syndrome GEMM operand). Only the touched bitmap
// words are cleared.
// S row = T e[mt:n]: XOR of the columns of TT (row j = column j of T, row k
// zero) at the request's t positions; positions < mt read the zero row.
// Each half-warp reads whole rows, lane c of a half the 16-byte chunk c, so a
// load instruction covers two rows contiguously (positions 2i and 2i + 1);
// the halves are added by one shuffle and lane c stores words 4c .. 4c + 3.
// The loop is unrolled 32 times: a warp gathers one request's columns at a
// time, so the loads in flight per lane set how many L2 round trips a
// request costs (2 for t = 128; unrolled 8 times it took 8, and 0.45 against
// 0.42-0.43 ms for 65536 requests).
template <int SET, typename PosFn>
__device__ __forceinline__ void sparse_syndrome_row(PosFn pos_of, const uint32_t *__restrict__ TT, int ldtt,
                                                    uint32_t *__restrict__ srow, int lane) {
  using p = P<SET>;
  constexpr int MW4 = (p::mw + 3) / 4;
  static_assert(MW4 <= 16, "a syndrome row fits half a warp of 16-byte chunks");
  const int c = lane & 15;
  uint4 acc = make_uint4(0, 0, 0, 0);
  if (c < MW4) {
#pragma unroll 32
    for (int i = lane >> 4; i < p::t; i += 2) {
      const int pos = pos_of(i);
      const uint4 v =
          reinterpret_cast<const uint4 *>(TT + (size_t)(pos >= p::mt ? pos - p::mt : p::k) * ldtt)[c];
      acc.x ^= v.x;
      acc.y ^= v.y;
      acc.z ^= v.z;
      acc.w ^= v.w;
    }
  }
  acc.x ^= __shfl_xor_sync(0xffffffffu, acc.x, 16);
  acc.y ^= __shfl_xor_sync(0xffffffffu, acc.y, 16);
  acc.z ^= __shfl_xor_sync(0xffffffffu, acc.z, 16);
  acc.w ^= __shfl_xor_sync(0xffffffffu, acc.w, 16);
  if (lane < MW4) {
    const uint32_t q4[4] = {acc.x, acc.y, acc.z, acc.w};
#pragma unroll
    for (int e2 = 0; e2 < 4; e2++)
      if (4 * lane + e2 < p::mw) srow[4 * lane + e2] = q4[e2];
  }
}

template <int SET>
struct SampleLayout {
  using p = P<SET>;
  static constexpr int bm_words = (p::ew + 1) & ~1;
  static constexpr int cand_u16 = 32 * p::t;  // candidate c of lane l at c*32 + (l ^ 2(c%16))
  static constexpr int warp_bytes = bm_words * 4 + cand_u16 * 2;
};

__device__ __forceinline__ int cand_slot(int c, int l) { return c * 32 + (l ^ ((c & 15) << 1)); }

template <int SET, bool SPARSE>
__global__ void __launch_bounds__(kSampleThreadsMax) sample_kernel(const uint8_t *__restrict__ seeds, const Segs segs,
                                                                uint32_t *__restrict__ E, int lde,
                                                                uint32_t *__restrict__ Ens, int ldx,
                                                                const GemmKeys keys, uint32_t *__restrict__ S,
                                                                int lds, unsigned int *__restrict__ counter,
                                                                int lanes) {
  using p = P<SET>;
  using LY = SampleLayout<SET>;
  constexpr int NCW = (p::t + 31) / 32;
  extern __shared__ __align__(16) uint32_t sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *bm = sm + warp * (LY::warp_bytes / 4);
  uint16_t *cand = reinterpret_cast<uint16_t *>(bm + LY::bm_words);
  for (int w = lane; w < LY::bm_words; w += 32) bm[w] = 0;
  __syncwarp();
  const long long N = seg_rows(segs);
  bool has = false, exhausted = lane >= lanes;  // idle lanes never take a request
  long long op = 0;
  int myseg = 0;
  uint64_t st[4] = {0, 0, 0, 0};
  constexpr int ncand = p::cand_bytes / 2;  // 16-bit candidates per attempt
  constexpr int nlanes = (ncand + 3) / 4;   // output lanes holding them
  constexpr uint32_t mask = p::q - 1;
  constexpr int sh = p::mt % 32, w0 = p::mt / 32;
#pragma unroll 1
  while (true) {
    // lanes without a request take the next ones (rows that are segment gaps are skipped)
    const uint32_t need = __ballot_sync(0xffffffffu, !has && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned int base = 0;
      if (lane == leader) base = atomicAdd(counter, (unsigned int)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if ((need >> lane) & 1) {
        const long long idx = (long long)base + __popc(need & ((1u << lane) - 1));
        if (idx >= N) {
          exhausted = true;
        } else {
          op = idx;
          has = seg_live(segs, idx, &myseg);
          if (has) {
            const uint8_t *sd = seeds + 32 * idx;
#pragma unroll
            for (int i = 0; i < 4; i++) {
              uint64_t v = 0;
#pragma unroll
              for (int b = 0; b < 8; b++) v |= (uint64_t)sd[8 * i + b] << (8 * b);
              st[i] = v;
            }
          }
        }
      }
    }
    if (!__any_sync(0xffffffffu, has)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    // one attempt per lane that holds a request
    int count = 0;
    uint64_t nst[4] = {0, 0, 0, 0};
    if (has) {
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
      nst[0] = s[0];
      nst[1] = s[1];
      nst[2] = s[2];
      nst[3] = s[3];
#pragma unroll 1
      for (int base = 0; base < nlanes && count < p::t; base += 17) {
        if (base) keccak_f1600(s);
#pragma unroll
        for (int i = 0; i < 17; i++) {
          if (base + i < nlanes) {
            const uint64_t l = s[i];
#pragma unroll
            for (int h = 0; h < 4; h++) {
              const uint32_t v = (uint32_t)(l >> (16 * h)) & mask;
              const bool take = (4 * (base + i) + h < ncand) && (count < p::t) && (p::full || v < (uint32_t)p::n);
              if (take) {
                cand[cand_slot(count, lane)] = (uint16_t)v;
                count++;
              }
            }
          }
        }
      }
    }
    __syncwarp();
    // repeats, one lane's candidate set at a time
    uint32_t pend = __ballot_sync(0xffffffffu, has && count == p::t);
    uint32_t okmask = 0;
#pragma unroll 1
    while (pend) {
      const int r = __ffs(pend) - 1;
      pend &= pend - 1;
      uint32_t vv[NCW];
      bool dup = false;
#pragma unroll
      for (int i = 0; i < NCW; i++) {
        const int c = lane + 32 * i;
        vv[i] = 0xFFFFFFFFu;
        if (c < p::t) {
          const uint32_t v = cand[cand_slot(c, r)];
          vv[i] = v;
          const uint32_t bit = 1u << (v & 31);
          dup |= (atomicOr(&bm[v >> 5], bit) & bit) != 0;
        }
      }
      const bool anydup = __any_sync(0xffffffffu, dup);
      const long long opr = __shfl_sync(0xffffffffu, op, r);
      if (!anydup) {
        okmask |= 1u << r;
        uint32_t *erow = E + opr * lde;
        for (int w = lane; w < p::ew; w += 32) erow[w] = bm[w];
        if (SPARSE) {
          sparse_syndrome_row<SET>([&](int c) { return (int)cand[cand_slot(c, r)]; },
                                   keys.TT[__shfl_sync(0xffffffffu, myseg, r)], keys.ldtt, S + opr * lds, lane);
        } else {
          uint32_t *xrow = Ens + opr * ldx;
          for (int w = lane; w < p::kw; w += 32) {
            const uint32_t lo = bm[w0 + w];
            const uint32_t hi = (w0 + w + 1 < p::ew) ? bm[w0 + w + 1] : 0u;
            xrow[w] = sh ? ((lo >> sh) | (hi << (32 - sh))) : lo;
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < NCW; i++)
        if (vv[i] != 0xFFFFFFFFu) bm[vv[i] >> 5] = 0;
      __syncwarp();
    }
    if (has) {
      if ((okmask >> lane) & 1) {
        has = false;
      } else {
        st[0] = nst[0];
        st[1] = nst[1];
        st[2] = nst[2];
        st[3] = nst[3];
      }
    }
  }
}

// ---------------------------------------------------------------- pipelined sampling
// The seed chain's next state is the first 32 bytes of an attempt's first
// Keccak-f block, so only that block is on the chain's critical path; the
// attempt's further squeeze blocks (P - 1 of them: P = 2 for 348864 and
// 8192128, 3 for 460896, 4 for 6688128 and 6960119) are not. A request is
// held by a group of G >= P lanes: at every step lane 0 of the group starts
// the next attempt (absorb 64 || state, permute) while lane r < P permutes the
// state lane r - 1 left in shared memory a step earlier (block r of an older
// attempt; the state is not held in registers through the check below); all
// lanes permute in lockstep, so a step costs one permutation and an attempt
// completes every step once the pipeline is full. Each block's 17 output
// words go to the attempt's slot of a per-group ring in shared memory; when
// block P - 1 lands, the warp checks the attempt (candidate filter, first t
// kept, repeats) exactly as the lane-per-request form does, and a success
// drops the group's younger attempts. Groups take further requests from the
// launch-wide counter like the lanes of sample_kernel. Per request this costs
// P - 1 speculative first blocks and P - 1 steps of pipeline fill, but the
// chain's critical path is one permutation per attempt instead of P, which
// matters most for the slowest chains of a batch (about 24 attempts for the
// slowest of 65536 requests).
template <int SET>
struct PipeLayout {
  using p = P<SET>;
  static constexpr int perms = (p::cand_bytes + 135) / 136;  // Keccak-f blocks per attempt
  static constexpr int G = perms <= 2 ? 2 : 4;                // lanes per group
  static constexpr int NG = 32 / G;                          // groups per warp at most
  static constexpr int raw_words = (p::cand_bytes + 7) / 8;  // u64 words of one attempt's draw
  static constexpr int bm_words = (p::ew + 1) & ~1;
  static constexpr int group_words = perms * raw_words + 1;  // odd u64 stride: groups on distinct banks
  static constexpr int cand_off = bm_words * 4;
  static constexpr int state_off = cand_off + (p::t * 2 + 7) / 8 * 8;  // [25][32] u64 block states
  static constexpr int ring_off = state_off + 25 * 32 * 8;
  static constexpr int warp_bytes = ring_off + NG * group_words * 8;
  static_assert(perms <= G && raw_words <= 17 * perms, "pipeline geometry");
};

template <int SET, bool SPARSE>
__global__ void __launch_bounds__(kSampleThreadsMax)
    sample_pipe_kernel(const uint8_t *__restrict__ seeds, const Segs segs, uint32_t *__restrict__ E, int lde,
                       uint32_t *__restrict__ Ens, int ldx, const GemmKeys keys, uint32_t *__restrict__ S, int lds,
                       unsigned int *__restrict__ counter, int groups) {
  using p = P<SET>;
  using LY = PipeLayout<SET>;
  constexpr int PP = LY::perms, G = LY::G, RW = LY::raw_words, NCW = (p::t + 31) / 32;
  constexpr int ncand = p::cand_bytes / 2;
  constexpr uint32_t mask = p::q - 1;
  constexpr int sh = p::mt % 32, w0 = p::mt / 32;
  extern __shared__ __align__(16) uint32_t sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint8_t *wb = reinterpret_cast<uint8_t *>(sm) + (size_t)warp * LY::warp_bytes;
  uint32_t *bm = reinterpret_cast<uint32_t *>(wb);
  uint16_t *cand = reinterpret_cast<uint16_t *>(wb + LY::cand_off);
  uint64_t *sts = reinterpret_cast<uint64_t *>(wb + LY::state_off);
  uint64_t *ring = reinterpret_cast<uint64_t *>(wb + LY::ring_off);
  for (int w = lane; w < LY::bm_words; w += 32) bm[w] = 0;
  __syncwarp();
  const int g = lane / G, r = lane % G;
  const bool chain = r == 0 && g < groups;  // the lane that owns the group's request and seed chain
  const long long N = seg_rows(segs);
  bool has = false, exhausted = !chain;
  long long op = 0;
  int myseg = 0, attempt = 0;
  uint64_t st[4] = {0, 0, 0, 0};
  bool valid = false;  // this lane holds block r of attempt att of the group's request
  int att = 0;
#pragma unroll 1
  while (true) {
    // chain lanes without a request take the next ones (segment gaps are skipped)
    const uint32_t need = __ballot_sync(0xffffffffu, !has && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned int base = 0;
      if (lane == leader) base = atomicAdd(counter, (unsigned int)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if ((need >> lane) & 1) {
        const long long idx = (long long)base + __popc(need & ((1u << lane) - 1));
        if (idx >= N) {
          exhausted = true;
        } else {
          op = idx;
          has = seg_live(segs, idx, &myseg);
          attempt = 0;
          if (has) {
            const uint8_t *sd = seeds + 32 * idx;
#pragma unroll
            for (int i = 0; i < 4; i++) {
              uint64_t v = 0;
#pragma unroll
              for (int b = 0; b < 8; b++) v |= (uint64_t)sd[8 * i + b] << (8 * b);
              st[i] = v;
            }
          }
        }
      }
    }
    if (!__any_sync(0xffffffffu, has || valid)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    // lane 0 of a group starts its request's next attempt (SHAKE256 absorb of
    // {64} || state); lane r > 0 continues the block state lane r - 1 left in
    // shared memory a step earlier
    if (r == 0) {
      valid = has;
      att = attempt;
    }
    uint64_t s[25];
    if (r == 0) {
#pragma unroll
      for (int i = 0; i < 25; i++) s[i] = 0;
      s[0] = 64ull | (st[0] << 8);
      s[1] = (st[0] >> 56) | (st[1] << 8);
      s[2] = (st[1] >> 56) | (st[2] << 8);
      s[3] = (st[2] >> 56) | (st[3] << 8);
      s[4] = (st[3] >> 56) | (0x1Full << 8);
      s[16] = 0x8000000000000000ull;
    } else {
#pragma unroll
      for (int i = 0; i < 25; i++) s[i] = sts[i * 32 + lane - 1];
    }
    __syncwarp();  // every predecessor state read before this step's states overwrite them
    keccak_f1600(s);
#pragma unroll
    for (int i = 0; i < 25; i++) sts[i * 32 + lane] = s[i];
    if (valid) {
      uint64_t *dst = ring + (size_t)g * LY::group_words + (size_t)(att % PP) * RW;
#pragma unroll
      for (int i = 0; i < 17; i++) {
        const int w = 17 * r + i;
        if (w < RW) dst[w] = s[i];
      }
      if (r == 0) {
        st[0] = s[0];
        st[1] = s[1];
        st[2] = s[2];
        st[3] = s[3];
        attempt++;
      }
    }
    __syncwarp();
    // attempts whose last block landed: filter, first t kept, repeats; one group at a time
    uint32_t pend = __ballot_sync(0xffffffffu, valid && r == PP - 1);
    uint32_t succ = 0;  // bit per group
#pragma unroll 1
    while (pend) {
      const int L = __ffs(pend) - 1;
      pend &= pend - 1;
      const int gg = L / G, owner = gg * G;
      const int a = __shfl_sync(0xffffffffu, att, L);
      const uint16_t *raw = reinterpret_cast<const uint16_t *>(ring + (size_t)gg * LY::group_words + (size_t)(a % PP) * RW);
      int total = 0;
#pragma unroll
      for (int base = 0; base < ncand; base += 32) {
        const int i = base + lane;
        uint32_t v = 0;
        bool keep = false;
        if (i < ncand) {
          v = raw[i] & mask;
          keep = p::full || v < (uint32_t)p::n;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, keep);
        const int idx = total + __popc(bal & ((1u << lane) - 1));
        if (keep && idx < p::t) cand[idx] = (uint16_t)v;
        total += __popc(bal);
      }
      __syncwarp();
      if (total < p::t) continue;  // too few candidates below n: the attempt fails (warp-uniform)
      uint32_t vv[NCW];
      bool dup = false;
#pragma unroll
      for (int i = 0; i < NCW; i++) {
        const int c = lane + 32 * i;
        vv[i] = 0xFFFFFFFFu;
        if (c < p::t) {
          const uint32_t v = cand[c];
          vv[i] = v;
          const uint32_t bit = 1u << (v & 31);
          dup |= (atomicOr(&bm[v >> 5], bit) & bit) != 0;
        }
      }
      const bool anydup = __any_sync(0xffffffffu, dup);
      if (!anydup) {
        succ |= 1u << gg;
        const long long opr = __shfl_sync(0xffffffffu, op, owner);
        uint32_t *erow = E + opr * lde;
        for (int w = lane; w < p::ew; w += 32) erow[w] = bm[w];
        if (SPARSE) {
          sparse_syndrome_row<SET>([&](int c) { return (int)cand[c]; },
                                   keys.TT[__shfl_sync(0xffffffffu, myseg, owner)], keys.ldtt, S + opr * lds, lane);
        } else {
          uint32_t *xrow = Ens + opr * ldx;
          for (int w = lane; w < p::kw; w += 32) {
            const uint32_t lo = bm[w0 + w];
            const uint32_t hi = (w0 + w + 1 < p::ew) ? bm[w0 + w + 1] : 0u;
            xrow[w] = sh ? ((lo >> sh) | (hi << (32 - sh))) : lo;
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < NCW; i++)
        if (vv[i] != 0xFFFFFFFFu) bm[vv[i] >> 5] = 0;
      __syncwarp();
    }
    // a success ends the request: its younger attempts in flight are dropped
    if ((succ >> g) & 1) {
      valid = false;
      if (r == 0) has = false;
    }
    // block r of an attempt moves one lane along the group (its state is in shared memory)
    const bool vin = __shfl_up_sync(0xffffffffu, valid ? 1 : 0, 1, G) != 0;
    const int ain = __shfl_up_sync(0xffffffffu, att, 1, G);
    if (r > 0) {
      valid = vin && r < PP;
      att = ain;
    }
  }
}

// ---------------------------------------------------------------- finalize
// c = e[0:mt] xor (T e[mt:n]); K = SHAKE256(1 || e || c). When the public
// key's padding bits are set (6960119 only), c and K are zeroed
// (mc:crypto_kem/6960119/vec/kem_enc.c:21-66).
template <int SET, bool PC>
__global__ void __launch_bounds__(kTailThreads) finalize_kernel(const uint32_t *__restrict__ E, int lde,
                                                                const uint32_t *__restrict__ S, int lds,
                                                                uint8_t *__restrict__ C, uint8_t *__restrict__ K,
                                                                const Segs segs, uint32_t pk_bad_mask) {
  using p = P<SET>;
  constexpr int SB = p::synd_bytes, CB = SB + (PC ? 32 : 0);  // C0 bytes, ciphertext bytes
  __shared__ uint32_t stage[kTailThreads / 32][32 * kStageStride];
  __shared__ const uint32_t *rows[kTailThreads / 32][32];
  const long long N = seg_rows(segs);
  const long long op = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long opc = op < N ? op : N - 1;  // every lane of a warp takes part in the staged hash
  int seg;
  const bool live = seg_live(segs, op, &seg);
  const uint32_t *e = E + opc * lde;
  const uint32_t *sy = S + opc * lds;
  // C0 word w: e[0:mt] xor the syndrome, bits from mt on cleared (zero past C0)
  auto c0word = [&](int w) -> uint32_t {
    if (w >= p::mw) return 0u;
    uint32_t v = e[w] ^ sy[w];
    if (w == p::mt / 32 && (p::mt % 32)) v &= (1u << (p::mt % 32)) - 1u;
    return v;
  };
  // plaintext confirmation: C1 = SHAKE256(2 || e, 32) (mc:crypto_kem/348864pc/vec/kem_enc.c:32)
  uint64_t h2[4] = {0, 0, 0, 0};
  if constexpr (PC) {
    auto none = [](int) -> uint32_t { return 0u; };
    kem_hash_staged<p::e_bytes, 1 + p::e_bytes>(h2, 2u, e, none, stage[threadIdx.x >> 5], rows[threadIdx.x >> 5]);
  }
  auto c1byte = [&](int j) -> uint32_t {
    const uint64_t v = j < 8 ? h2[0] : j < 16 ? h2[1] : j < 24 ? h2[2] : h2[3];
    return (uint32_t)(v >> (8 * (j & 7))) & 0xFFu;
  };
  auto cbyte = [&](int x) -> uint32_t {
    if (x < SB) return (c0word(x >> 2) >> (8 * (x & 3))) & 0xFFu;
    return x < CB ? c1byte(x - SB) : 0u;
  };
  // word w of the ciphertext C0 || C1 (zero past it)
  auto cword = [&](int w) -> uint32_t {
    if (!PC || 4 * w + 4 <= SB) return c0word(w);
    if (4 * w >= CB) return 0u;
    if (SB % 4 == 0) {
      const int j4 = w - SB / 4;
      const uint64_t v = j4 < 2 ? h2[0] : j4 < 4 ? h2[1] : j4 < 6 ? h2[2] : h2[3];
      return (uint32_t)(v >> (32 * (j4 & 1)));
    }
    return cbyte(4 * w) | (cbyte(4 * w + 1) << 8) | (cbyte(4 * w + 2) << 16) | (cbyte(4 * w + 3) << 24);
  };
  uint64_t h[4];
  kem_hash_staged<p::e_bytes, p::pre_bytes + (PC ? 32 : 0)>(h, 1u, e, cword, stage[threadIdx.x >> 5],
                                                             rows[threadIdx.x >> 5]);
  if (!live) return;
  const bool pk_bad = (pk_bad_mask >> seg) & 1u;
  uint8_t *c = C + op * CB;
  uint8_t *k = K + op * 32;
  for (int x = 0; x < CB; x++) c[x] = pk_bad ? 0 : (uint8_t)cbyte(x);
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int b = 0; b < 8; b++) k[8 * i + b] = pk_bad ? 0 : (uint8_t)(h[i] >> (8 * b));
}

// ---------------------------------------------------------------- column image of T
// One warp per (32 rows, 32 columns) block: lane b holds row 32w + b's word of
// the block, ballot j gives column 32jw + j's bits of those rows.
__global__ void transpose_pk_kernel(const uint32_t *__restrict__ T, int lda, int mt, int k, uint32_t *__restrict__ TT,
                                    int ldtt) {
  const int lane = threadIdx.x & 31;
  const long long task = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int mw = (mt + 31) / 32, kw = (k + 31) / 32;
  if (task >= (long long)mw * kw) return;  // warp-uniform
  const int w = (int)(task % mw), jw = (int)(task / mw);
  const int row = 32 * w + lane;
  const uint32_t x = row < mt ? T[(size_t)row * lda + jw] : 0u;
  uint32_t mine = 0;
#pragma unroll
  for (int j = 0; j < 32; j++) {
    const uint32_t v = __ballot_sync(0xffffffffu, (x >> j) & 1u);
    mine = (lane == j) ? v : mine;
  }
  const int col = 32 * jw + lane;
  if (col < k) TT[(size_t)col * ldtt + w] = mine;
}

cudaError_t launch_transpose_pk(const uint32_t *T, int lda, int mt, int k, uint32_t *TT, int ldtt, cudaStream_t st) {
  const long long warps = (long long)((mt + 31) / 32) * ((k + 31) / 32);
  transpose_pk_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(T, lda, mt, k, TT, ldtt);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- launchers
// GMC_SAMPLE_PIPELINE=0 in the environment (read once per process) puts
// every batch on the lane-per-request sampler instead of the pipelined one.
static bool sample_pipelined() {
  static const bool on = [] {
    const char *v = getenv("GMC_SAMPLE_PIPELINE");
    return !(v && v[0] == '0');
  }();
  return on;
}
template <int SET, bool SPARSE>
static cudaError_t launch_sample_mode(const uint8_t *seeds, const Segs &segs, uint32_t *E, int lde, uint32_t *Ens,
                                     int ldx, const GemmKeys &keys, uint32_t *S, int lds, int threads,
                                     unsigned int *counter, cudaStream_t st, int sample_sm_warps,
                                     void (*mark)(const char *, cudaStream_t)) {
  const long long N = seg_rows(segs);
  const int smem = (threads / 32) * SampleLayout<SET>::warp_bytes;
  cudaError_t err = cudaFuncSetAttribute(sample_kernel<SET, SPARSE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (kSampleThreadsMax / 32) * SampleLayout<SET>::warp_bytes);
  if (err != cudaSuccess) return err;
  if ((err = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st)) != cudaSuccess) return err;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sample_kernel<SET, SPARSE>, threads, smem);
  if (per_sm < 1) per_sm = 1;
  // fewer lanes than requests: a lane that finishes early takes further
  // requests, so the last slow chains hold few warps (kSampleWarpsPerSM)
  const int warps = threads / 32;
  int per_sm_target = (kSampleWarpsPerSM + warps - 1) / warps;
  // pipelined form (every set and batch size measured faster than the
  // lane-per-request form: 348864 / 460896 / 6688128 / 6960119 / 8192128 at
  // 65536 requests 0.31 / 0.63 / 0.89 / 0.77 / 0.57 ms against 0.37 / 0.80 /
  // 1.00 / 0.82 / 0.70 ms, and up to 2.3x at 16384); groups take further
  // requests when the batch outnumbers them
  if (sample_pipelined()) {
    using PL = PipeLayout<SET>;
    auto kern = sample_pipe_kernel<SET, SPARSE>;
    const int psmem = warps * PL::warp_bytes;
    err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (kSampleThreadsMax / 32) * PL::warp_bytes);
    if (err != cudaSuccess) return err;
    int pper = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pper, kern, threads, psmem);
    if (pper < 1) pper = 1;
    // the pipelined form fills the SMs (no tail cap: each warp's tail is one chain's)
    const int ptarget = sample_sm_warps > 0 && (sample_sm_warps + warps - 1) / warps < pper
                            ? (sample_sm_warps + warps - 1) / warps
                            : pper;
    const long long pslots = (long long)sms * ptarget * warps;
    // active groups per warp: the smallest power of two with which the
    // resident warps hold the whole batch at once, at most 32 / G
    int groups = 1;
    while (groups < PL::NG && (long long)groups * pslots < N) groups <<= 1;
    const long long per_block = (long long)warps * groups;
    const long long need = (N + per_block - 1) / per_block;
    const long long resident = (long long)sms * ptarget;
    const long long blocks = need < resident ? need : resident;
    kern<<<(unsigned)blocks, threads, psmem, st>>>(seeds, segs, E, lde, Ens, ldx, keys, S, lds, counter, groups);
    err = cudaGetLastError();
    if (mark) mark(SPARSE ? "enc_sample_syndrome" : "enc_sample", st);
    return err;
  }
  if (per_sm_target > per_sm) per_sm_target = per_sm;
  // active lanes per warp: the smallest power of two (<= 32) with which the
  // resident warps hold the whole batch at once
  const long long warp_slots = (long long)sms * per_sm_target * warps;
  int lanes = 1;
  while (lanes < 32 && (long long)lanes * warp_slots < N) lanes <<= 1;
  const long long per_block = (long long)warps * lanes;
  const long long need = (N + per_block - 1) / per_block;
  const long long resident = (long long)sms * per_sm_target;
  const long long blocks = need < resident ? need : resident;
  sample_kernel<SET, SPARSE><<<(unsigned)blocks, threads, smem, st>>>(seeds, segs, E, lde, Ens, ldx, keys, S, lds,
                                                                      counter, lanes);
  err = cudaGetLastError();
  if (mark) mark(SPARSE ? "enc_sample_syndrome" : "enc_sample", st);
  return err;
}

template <int SET>
cudaError_t launch_sample(const uint8_t *seeds, const Segs &segs, uint32_t *E, int lde, uint32_t *Ens, int ldx,
                          const GemmKeys *sparse, uint32_t *S, int lds, int threads, unsigned int *counter,
                          cudaStream_t st, int sm_warps, void (*mark)(const char *, cudaStream_t)) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  if ((threads != 32 && threads != 64 && threads != 128) || !counter || sm_warps < 0) return cudaErrorInvalidValue;
  if (sparse) {
    if (!S || lds < P<SET>::mw || sparse->ldtt < 64) return cudaErrorInvalidValue;
    for (int i = 0; i < segs.nseg; i++)
      if (!sparse->TT[i]) return cudaErrorInvalidValue;
    return launch_sample_mode<SET, true>(seeds, segs, E, lde, Ens, ldx, *sparse, S, lds, threads, counter, st,
                                         sm_warps, mark);
  }
  return launch_sample_mode<SET, false>(seeds, segs, E, lde, Ens, ldx, GemmKeys{}, S, lds, threads, counter, st,
                                        sm_warps, mark);
}

template <int SET>
cudaError_t launch_finalize(const uint32_t *E, int lde, const uint32_t *S, int lds, uint8_t *C, uint8_t *K,
                            const Segs &segs, uint32_t pk_bad_mask, bool pc, cudaStream_t st) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  long long blocks = (N + kTailThreads - 1) / kTailThreads;
  if (pc)
    finalize_kernel<SET, true><<<(unsigned)blocks, kTailThreads, 0, st>>>(E, lde, S, lds, C, K, segs, pk_bad_mask);
  else
    finalize_kernel<SET, false><<<(unsigned)blocks, kTailThreads, 0, st>>>(E, lde, S, lds, C, K, segs, pk_bad_mask);
  return cudaGetLastError();
}

#define GMC_INST_ENC(SET)                                                                                        \
  template cudaError_t launch_sample<SET>(const uint8_t *, const Segs &, uint32_t *, int, uint32_t *, int,       \
                                          const GemmKeys *, uint32_t *, int, int, unsigned int *, cudaStream_t,  \
                                          int, void (*)(const char *, cudaStream_t));                            \
  template cudaError_t launch_finalize<SET>(const uint32_t *, int, const uint32_t *, int, uint8_t *, uint8_t *, \
                                            const Segs &, uint32_t, bool, cudaStream_t);
GMC_INST_ENC(0)
GMC_INST_ENC(1)
GMC_INST_ENC(2)
GMC_INST_ENC(3)
GMC_INST_ENC(4)

}  // namespace gmc
