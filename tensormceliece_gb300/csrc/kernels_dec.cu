// Decapsulation kernels.
//
//  pack_ct     ciphertext bytes -> 32-bit words (the front-end GEMM operand)
//  decode      one warp per request: 2t syndromes (from the front-end GEMM)
//              -> Berlekamp-Massey -> additive FFT over all 2^m field
//              elements -> error positions at the key's support -> weight
//              and re-encryption (syndrome) check
//  dec_tail    K = SHAKE256(b || (e or s) || c), implicit rejection, and the
//              6960119 ciphertext-padding rule
//
// Reference behaviour: decrypt / operation_dec of libmceliece
// (mceliece-gpu-params/ref/348864.cuh:3251-3406, 3615-3650;
// mc:crypto_kem/348864/vec/decrypt.c:135, kem_dec.c:19;
// mc:crypto_kem/6960119/vec/kem_dec.c:21-78). Only the outcome is defined
// there: a weight-t error with the received syndrome is unique, so any exact
// decoder yields the same session key. The BM update rule follows the
// library's (mc:crypto_kem/348864/vec/bm.c:156), so locators agree with the
// oracle's stage output as well.
#include "kernels.h"
#include "device_common.cuh"

namespace gmc {

__device__ __forceinline__ uint32_t warp_xor(uint32_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v ^= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- pack_ct
template <int SET, bool PC>
__global__ void pack_ct_kernel(const uint8_t *__restrict__ C, const Segs segs, uint32_t *__restrict__ X, int ldx) {
  using p = P<SET>;
  constexpr int CB = p::synd_bytes + (PC ? 32 : 0);  // ciphertext row bytes
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long op = idx / ldx;
  const int w = (int)(idx % ldx);
  if (op >= seg_rows(segs)) return;
  int seg;
  uint32_t v = 0;  // rows past a segment's live requests stay zero
  if (seg_live(segs, op, &seg)) {
    const uint8_t *c = C + op * CB;
#pragma unroll
    for (int b = 0; b < 4; b++) {
      int x = 4 * w + b;
      if (x < p::synd_bytes) v |= (uint32_t)c[x] << (8 * b);
    }
  }
  X[op * ldx + w] = v;
}

// ---------------------------------------------------------------- BM
// One warp per group of 32 requests, bit-sliced: bit q of every word belongs
// to request 32g + q, and a GF(2^m) value of all 32 requests is m words
// (planes). Coefficient i of C (connection polynomial) lives in lane i%32,
// slot i/32, as m plane registers; B and the syndromes sit in per-warp shared
// memory as planes. Per iteration n:
//   d = sum_i C_i s_{n-i}: carry-less plane products accumulated unreduced,
//       one reduction, then one XOR reduction instruction per plane;
//   f = d/b per request: lane q extracts its request's d, divides with the
//       log tables (L and log b are per-request scalars in lane q) and the
//       32 quotients are sliced back by ballot;
//   C_i += f B_i (bit-sliced product), and B <- x (upd ? C_old : B) with the
//       per-request update mask from a ballot.
// This is the library's update rule (mc:crypto_kem/348864/vec/bm.c:156) on
// fixed arrays of t+1 coefficients, per request; the slot loops stop at the
// largest degree bound of the group: before iteration n, deg C <= L and
// deg B <= n+1-L, so the discrepancy needs i <= min(L, t) and the update
// i <= min(max(L, n+1-L), t). Rows that are not live run with zero
// syndromes (d = 0) and write nothing.
// Shared memory per warp is what fourteen warps per SM can hold (one round
// for 2048 groups on 152 SMs): iteration n reads s_{n-t} .. s_n only, so the
// syndromes sit in a ring of t+1 entries, filled one syndrome per iteration
// (its global load issued an iteration ahead); B keeps coefficients 0..t
// (reads above t are zero); the exponent table keeps the q-1 entries the
// division indexes. Lanes above deg C in an active discrepancy slot read
// ring entries of other iterations: C_i = 0 there (coefficients above t are
// never updated), so they add nothing.
template <int SET>
struct BMLayout {
  using p = P<SET>;
  static constexpr int Q = p::q, T = p::t, M = p::m;
  static constexpr int NS = (T + 1 + 31) / 32;
  static constexpr int R = T + 1;                              // syndrome ring entries
  static constexpr int exp_off = 0, log_off = Q;               // u16 tables (exp: indexes 0..q-2)
  static constexpr int zero_off = Q, zero_len = 16;            // u32: M zero planes (s_j, j < 0)
  static constexpr int shared_u32 = zero_off + zero_len;
  static constexpr int s_words = R * M;                        // syndrome planes [j mod R][b]
  static constexpr int b_words = (T + 1) * M;                  // B planes [i][b], i <= t
  static constexpr int warp_u32 = s_words + b_words;
  static constexpr int bytes(int warps) { return shared_u32 * 4 + warps * warp_u32 * 4; }
  static_assert(32 * NS * M <= warp_u32, "C planes are staged in the warp's area");
  static_assert(2 * T <= 2 * R, "ring index j - R for j < 2t");
};

// acc (2M-1 planes, unreduced) -> r (M planes) mod the field polynomial
template <int M>
__device__ __forceinline__ void bs_reduce(uint32_t (&r)[M], uint32_t (&acc)[2 * M - 1]) {
#pragma unroll
  for (int k = 2 * M - 2; k >= M; k--) {
    if (M == 13) {
      acc[k - 13] ^= acc[k];
      acc[k - 12] ^= acc[k];
      acc[k - 10] ^= acc[k];
      acc[k - 9] ^= acc[k];
    } else {
      acc[k - 12] ^= acc[k];
      acc[k - 9] ^= acc[k];
    }
  }
#pragma unroll
  for (int k = 0; k < M; k++) r[k] = acc[k];
}

template <int SET>
__global__ void __launch_bounds__(kBMWarps * 32, 1) dec_bm_kernel(const uint32_t *__restrict__ S2, int lds2,
                                                                  FieldDev fd, const Segs segs,
                                                                  uint16_t *__restrict__ Sig) {
  using p = P<SET>;
  using LY = BMLayout<SET>;
  constexpr int M = p::m, Q = p::q, T = p::t, D = p::fft_d;
  constexpr int NS = LY::NS, R = LY::R;
  constexpr int SIG = 1 << D;
  static_assert(M == 12 || M == 13, "field polynomial");
  extern __shared__ __align__(16) uint32_t bsm[];
  uint16_t *gexp = reinterpret_cast<uint16_t *>(bsm) + LY::exp_off;
  uint16_t *glog = reinterpret_cast<uint16_t *>(bsm) + LY::log_off;
  for (int i = threadIdx.x; i < Q - 1; i += blockDim.x) gexp[i] = fd.gexp[i];
  for (int i = threadIdx.x; i < Q; i += blockDim.x) glog[i] = fd.glog[i];
  for (int i = threadIdx.x; i < LY::zero_len; i += blockDim.x) bsm[LY::zero_off + i] = 0u;
  __syncthreads();
  const uint32_t *ZP = bsm + LY::zero_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *SP = bsm + LY::shared_u32 + warp * LY::warp_u32;
  uint32_t *BP = SP + LY::s_words;
  const long long N = seg_rows(segs);
  const long long ngroups = (N + 31) / 32;
  // each block (one per SM) takes an equal contiguous share of the groups and
  // its warps stride over it: with a grid-wide stride, 2048 groups over 152 x 8
  // warps left 48 SMs with half the work of the others
  const int nwb = blockDim.x >> 5;  // warps per block (a launch parameter up to kBMWarps)
  const long long g_lo = ngroups * blockIdx.x / gridDim.x, g_hi = ngroups * (blockIdx.x + 1) / gridDim.x;
  for (long long g = g_lo + warp; g < g_hi; g += nwb) {
    const long long op = g * 32 + lane;
    int seg;
    const bool live = op < N && seg_live(segs, op, &seg);
    const uint32_t *srow = S2 + op * lds2;
    // this lane's request's s_j (low M bits; 0 past the live rows)
    auto synd = [&](int j) -> uint32_t {
      uint32_t v = 0;
      if (live) {
        const int bb = j * M, w = bb >> 5, sh = bb & 31;
        v = srow[w] >> sh;
        if (sh + M > 32) v |= srow[w + 1] << (32 - sh);
      }
      return v;
    };
    // one syndrome of all 32 requests -> M planes in ring entry e (lane b < M stores plane b)
    auto to_ring = [&](uint32_t v, int e) {
      uint32_t pl[M];
#pragma unroll
      for (int b = 0; b < M; b++) pl[b] = __ballot_sync(0xffffffffu, (v >> b) & 1u);
      if (lane == 0) {  // the planes are warp-uniform: one lane stores them (no per-lane selects)
#pragma unroll
        for (int b = 0; b < M; b++) SP[e * M + b] = pl[b];
      }
    };
    to_ring(synd(0), 0);
    // C = 1, B = x
    uint32_t C[NS][M];
#pragma unroll
    for (int k = 0; k < NS; k++)
#pragma unroll
      for (int b = 0; b < M; b++) C[k][b] = (k == 0 && lane == 0 && b == 0) ? 0xFFFFFFFFu : 0u;
    for (int w = lane; w < LY::b_words; w += 32) BP[w] = (w == M) ? 0xFFFFFFFFu : 0u;
    __syncwarp();
    int L = 0, lb = 0;  // this lane's request: LFSR length, log b
#pragma unroll 1
    for (int n = 0; n < 2 * T; n++) {
      const uint32_t s_next = n + 1 < 2 * T ? synd(n + 1) : 0u;  // consumed at the end of the iteration
      const int Lc = L < T ? L : T;
      int Lu = (L > n + 1 - L) ? L : n + 1 - L;
      Lu = Lu < T ? Lu : T;
      const int bd = (int)__reduce_max_sync(0xffffffffu, live ? (unsigned)Lc : 0u);
      const int bu = (int)__reduce_max_sync(0xffffffffu, live ? (unsigned)Lu : 0u);
      // discrepancy planes
      uint32_t d[M];
      {
        uint32_t acc[2 * M - 1];
#pragma unroll
        for (int k = 0; k < 2 * M - 1; k++) acc[k] = 0;
#pragma unroll
        for (int k = 0; k < NS; k++) {
          if (32 * k <= bd) {
            const int j = n - lane - 32 * k;  // s_j (ring entry j mod R), j < 0 reads the zero planes
            const uint32_t *sp = j >= 0 ? SP + (j >= R ? j - R : j) * M : ZP;
#pragma unroll
            for (int b2 = 0; b2 < M; b2++) {
              const uint32_t sv = sp[b2];
#pragma unroll
              for (int b1 = 0; b1 < M; b1++) acc[b1 + b2] ^= C[k][b1] & sv;
            }
          }
        }
        bs_reduce<M>(d, acc);
#pragma unroll
        for (int b = 0; b < M; b++) d[b] = __reduce_xor_sync(0xffffffffu, d[b]);
      }
      // this lane's request: f = d / b, the update decision
      uint32_t dq = 0;
#pragma unroll
      for (int b = 0; b < M; b++) dq += ((d[b] >> lane) & 1u) << b;  // disjoint bits: the add may fuse
      const bool upd = dq != 0 && 2 * L <= n;
      uint32_t fq = 0;
      int ld = 0;
      if (dq) {
        ld = glog[dq];
        int lf = ld - lb;
        if (lf < 0) lf += Q - 1;
        fq = gexp[lf];
      }
      uint32_t f[M];
#pragma unroll
      for (int b = 0; b < M; b++) f[b] = __ballot_sync(0xffffffffu, (fq >> b) & 1u);
      const uint32_t U = __ballot_sync(0xffffffffu, upd);
      const bool anyf = __any_sync(0xffffffffu, dq != 0);
      if (upd) {
        L = n + 1 - L;
        lb = ld;
      }
      // C_i += f B_i; B_{i+1} <- (U ? C_i(old) : B_i); slots in descending
      // order so slot k's write of B_{32(k+1)} follows slot k+1's read of it
#pragma unroll
      for (int k = NS - 1; k >= 0; k--) {
        if (32 * k <= bu) {
          const int i = lane + 32 * k;
          const uint32_t *bp = BP + i * M;
          uint32_t bi[M];
#pragma unroll
          for (int b = 0; b < M; b++) bi[b] = i <= T ? bp[b] : 0u;
          __syncwarp();  // every lane holds its B_i before B_{i+1} is replaced
          const bool in = i <= T;  // coefficients above t stay zero
          uint32_t r[M];
          if (anyf) {
            // r = f * B_i, Horner over the planes of f
#pragma unroll
            for (int b = 0; b < M; b++) r[b] = bi[b] & f[M - 1];
#pragma unroll
            for (int jj = M - 2; jj >= 0; jj--) {
              const uint32_t top = r[M - 1];
#pragma unroll
              for (int b = M - 1; b > 0; b--) r[b] = r[b - 1];
              r[0] = top;
              if (M == 13) {
                r[1] ^= top;
                r[3] ^= top;
                r[4] ^= top;
              } else {
                r[3] ^= top;
              }
#pragma unroll
              for (int b = 0; b < M; b++) r[b] ^= bi[b] & f[jj];
            }
          } else {
#pragma unroll
            for (int b = 0; b < M; b++) r[b] = 0;
          }
          uint32_t *bq = BP + (i + 1) * M;
#pragma unroll
          for (int b = 0; b < M; b++) {
            const uint32_t cold = C[k][b];
            if (in) C[k][b] = cold ^ r[b];
            if (i + 1 <= T) bq[b] = (U & cold) | (~U & bi[b]);
          }
          // no barrier before the next (lower) slot: its reads, B_{32(k-1)} ..
          // B_{32k-1}, miss this slot's writes, B_{32k+1} .. B_{32k+32}, and
          // its writes follow its own barrier above, after this slot's reads
        }
      }
      if (lane < M) BP[lane] = 0;  // B_0 of x * (...) is zero (slot 0 read it before its barrier)
      // s_{n+1} replaces s_{n-t}, the oldest entry (read above, before the update's warp barriers)
      if (n + 1 < 2 * T) to_ring(s_next, n + 1 >= R ? n + 1 - R : n + 1);
      __syncwarp();
    }
    // sigma(x) = sum_deg C[t-deg] x^deg -> FFT coefficient slots (deg < 2^d);
    // coefficients are < 2^m <= 2^13, so bit 15 of the constant coefficient
    // is free for the flag of a final length L > t
#pragma unroll
    for (int k = 0; k < NS; k++)
#pragma unroll
      for (int b = 0; b < M; b++) SP[(lane + 32 * k) * M + b] = C[k][b];
    __syncwarp();
    if (live) {
      uint16_t *sig = Sig + op * SIG;
#pragma unroll 1
      for (int deg = 0; deg < SIG; deg++) {
        const int i = T - deg;
        uint32_t v = 0;
        if (i >= 0) {
#pragma unroll
          for (int b = 0; b < M; b++) v |= ((SP[i * M + b] >> lane) & 1u) << b;
        }
        if (deg == 0 && L > T) v |= 0x8000u;
        sig[deg] = (uint16_t)v;
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- BM, constant-time form
// Bit-sliced products with both operands in registers (the multiplier a is
// warp-uniform in the callers below): Horner over the planes of a, as bs_mul.
template <int M>
__device__ __forceinline__ void bs_mul_reg(uint32_t (&r)[M], const uint32_t (&a)[M], const uint32_t (&b)[M]) {
#pragma unroll
  for (int i = 0; i < M; i++) r[i] = b[i] & a[M - 1];
#pragma unroll
  for (int j = M - 2; j >= 0; j--) {
    const uint32_t top = r[M - 1];
#pragma unroll
    for (int i = M - 1; i > 0; i--) r[i] = r[i - 1];
    r[0] = top;
    if (M == 13) {
      r[1] ^= top;
      r[3] ^= top;
      r[4] ^= top;
    } else {
      r[3] ^= top;
    }
#pragma unroll
    for (int i = 0; i < M; i++) r[i] ^= b[i] & a[j];
  }
}

// r = a^2: the planes spread to the even positions, then the reduction
template <int M>
__device__ __forceinline__ void bs_sqr(uint32_t (&r)[M], const uint32_t (&a)[M]) {
  uint32_t acc[2 * M - 1];
#pragma unroll
  for (int k = 0; k < 2 * M - 1; k++) acc[k] = (k & 1) ? 0u : a[k >> 1];
  bs_reduce<M>(r, acc);
}

template <int M>
__device__ __forceinline__ void bs_sqr_n(uint32_t (&r)[M], const uint32_t (&a)[M], int n) {
#pragma unroll
  for (int i = 0; i < M; i++) r[i] = a[i];
#pragma unroll 1
  for (int k = 0; k < n; k++) {
    uint32_t t[M];
    bs_sqr<M>(t, r);
#pragma unroll
    for (int i = 0; i < M; i++) r[i] = t[i];
  }
}

// r = a^(2^M - 2) = a^-1 (0 for a = 0), by the chain of a^(2^k - 1):
// M = 13: k = 1, 2, 3, 6, 12, then one squaring; M = 12: k = 1, 2, 3, 5, 6, 11.
template <int M>
__device__ __forceinline__ void bs_inv(uint32_t (&r)[M], const uint32_t (&a)[M]) {
  uint32_t t[M], a2[M], a3[M];
  bs_sqr<M>(t, a);
  bs_mul_reg<M>(a2, t, a);  // a^(2^2 - 1)
  bs_sqr<M>(t, a2);
  bs_mul_reg<M>(a3, t, a);  // a^(2^3 - 1)
  if (M == 13) {
    uint32_t a6[M], a12[M];
    bs_sqr_n<M>(t, a3, 3);
    bs_mul_reg<M>(a6, t, a3);  // a^(2^6 - 1)
    bs_sqr_n<M>(t, a6, 6);
    bs_mul_reg<M>(a12, t, a6);  // a^(2^12 - 1)
    bs_sqr<M>(r, a12);
  } else {
    uint32_t a5[M], a6[M], a11[M];
    bs_sqr_n<M>(t, a3, 2);
    bs_mul_reg<M>(a5, t, a2);  // a^(2^5 - 1)
    bs_sqr_n<M>(t, a3, 3);
    bs_mul_reg<M>(a6, t, a3);  // a^(2^6 - 1)
    bs_sqr_n<M>(t, a6, 5);
    bs_mul_reg<M>(a11, t, a5);  // a^(2^11 - 1)
    bs_sqr<M>(r, a11);
  }
}

// The bit-sliced layout of dec_bm_kernel with nothing that depends on the
// syndromes in an address, a branch or a trip count:
//  - inversion-free update, no division d / b and no log tables: with b the
//    discrepancy of the last length change, C <- b C + d B (B carrying its x
//    shift as in dec_bm_kernel). By induction C = lambda C_lib for a nonzero
//    scalar lambda per request (a product of b's), with the same length L and
//    the same update decisions as the library's rule (d != 0 exactly when the
//    library's d is), also under the truncation to t + 1 coefficients;
//  - slot bounds from n alone: deg C <= L <= n and deg B <= n + 1;
//  - at the end every coefficient is multiplied by lambda^-1 (C_0 = lambda;
//    one bit-sliced inversion per group), which gives the library's locator
//    (C_0 = 1) exactly.
// The update decisions stay per-request masks (ballots), L is selected, never
// branched on.
// Shared memory: M zero planes, then per warp all 2t syndromes as planes and
// B over the 32 NS + 1 coefficient positions the slot loops address (the
// form needs about twice the registers of the table form, so it runs at
// kBMCtWarps warps per SM, where this layout fits).
template <int SET>
struct BMCtLayout {
  using p = P<SET>;
  static constexpr int T = p::t, M = p::m;
  static constexpr int NS = (T + 1 + 31) / 32;
  static constexpr int zero_len = 16;                 // u32: zero planes first, then the warps' areas
  static constexpr int s_words = 2 * T * M;           // syndrome planes [j][b]
  static constexpr int b_words = (32 * NS + 1) * M;   // B planes [i][b]
  static constexpr int warp_u32 = s_words + b_words;
  static constexpr int bytes(int warps) { return zero_len * 4 + warps * warp_u32 * 4; }
  static_assert(32 * NS * M <= s_words, "C planes are staged in the syndrome area");
};

template <int SET>
__global__ void __launch_bounds__(kBMCtWarps * 32, 1) dec_bm_ct_kernel(const uint32_t *__restrict__ S2, int lds2,
                                                                       const Segs segs, uint16_t *__restrict__ Sig) {
  using p = P<SET>;
  using LY = BMCtLayout<SET>;
  constexpr int M = p::m, T = p::t, D = p::fft_d;
  constexpr int NS = LY::NS;
  constexpr int SIG = 1 << D;
  static_assert(M == 12 || M == 13, "field polynomial");
  extern __shared__ __align__(16) uint32_t csm[];
  for (int i = threadIdx.x; i < LY::zero_len; i += blockDim.x) csm[i] = 0u;
  __syncthreads();
  const uint32_t *ZP = csm;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *SP = csm + LY::zero_len + warp * LY::warp_u32;
  uint32_t *BP = SP + LY::s_words;
  const long long N = seg_rows(segs);
  const long long ngroups = (N + 31) / 32;
  const int nwb = blockDim.x >> 5;
  const long long g_lo = ngroups * blockIdx.x / gridDim.x, g_hi = ngroups * (blockIdx.x + 1) / gridDim.x;
  for (long long g = g_lo + warp; g < g_hi; g += nwb) {
    const long long op = g * 32 + lane;
    int seg;
    const bool live = op < N && seg_live(segs, op, &seg);
    const uint32_t *srow = S2 + op * lds2;
#pragma unroll 1
    for (int j = 0; j < 2 * T; j++) {
      uint32_t v = 0;
      if (live) {
        const int bb = j * M, w = bb >> 5, sh = bb & 31;
        v = srow[w] >> sh;
        if (sh + M > 32) v |= srow[w + 1] << (32 - sh);
      }
      uint32_t mine = 0;
#pragma unroll
      for (int b = 0; b < M; b++) {
        const uint32_t pl = __ballot_sync(0xffffffffu, (v >> b) & 1u);
        mine = (lane == b) ? pl : mine;
      }
      if (lane < M) SP[j * M + lane] = mine;
    }
    uint32_t C[NS][M];
#pragma unroll
    for (int k = 0; k < NS; k++)
#pragma unroll
      for (int b = 0; b < M; b++) C[k][b] = (k == 0 && lane == 0 && b == 0) ? 0xFFFFFFFFu : 0u;
    for (int w = lane; w < LY::b_words; w += 32) BP[w] = (w == M) ? 0xFFFFFFFFu : 0u;
    uint32_t bq[M];  // b of every request (warp-uniform planes); b = 1
#pragma unroll
    for (int b = 0; b < M; b++) bq[b] = b == 0 ? 0xFFFFFFFFu : 0u;
    __syncwarp();
    int L = 0;  // this lane's request
#pragma unroll 1
    for (int n = 0; n < 2 * T; n++) {
      const int bd = n < T ? n : T;          // deg C <= L <= n
      const int bu = n + 1 < T ? n + 1 : T;  // deg B <= n + 1
      uint32_t d[M];
      {
        uint32_t acc[2 * M - 1];
#pragma unroll
        for (int k = 0; k < 2 * M - 1; k++) acc[k] = 0;
#pragma unroll
        for (int k = 0; k < NS; k++) {
          if (32 * k <= bd) {
            const int j = n - lane - 32 * k;  // s_j, j < 0 reads the zero planes
            const uint32_t *sp = j >= 0 ? SP + j * M : ZP;
#pragma unroll
            for (int b2 = 0; b2 < M; b2++) {
              const uint32_t sv = sp[b2];
#pragma unroll
              for (int b1 = 0; b1 < M; b1++) acc[b1 + b2] ^= C[k][b1] & sv;
            }
          }
        }
        bs_reduce<M>(d, acc);
#pragma unroll
        for (int b = 0; b < M; b++) d[b] = __reduce_xor_sync(0xffffffffu, d[b]);
      }
      uint32_t nz = 0;
#pragma unroll
      for (int b = 0; b < M; b++) nz |= d[b];
      const uint32_t U = nz & __ballot_sync(0xffffffffu, 2 * L <= n);
      L = ((U >> lane) & 1u) ? n + 1 - L : L;
      // C_i <- b C_i + d B_i; B_{i+1} <- (U ? C_i(old) : B_i); slots in
      // descending order (slot k's write of B_{32(k+1)} follows slot k+1's read)
#pragma unroll
      for (int k = NS - 1; k >= 0; k--) {
        if (32 * k <= bu) {
          const int i = lane + 32 * k;
          const uint32_t *bp = BP + i * M;
          uint32_t bi[M];
#pragma unroll
          for (int b = 0; b < M; b++) bi[b] = bp[b];
          __syncwarp();
          const bool in = (k < NS - 1) || (i <= T);
          uint32_t r[M];
#pragma unroll
          for (int b = 0; b < M; b++) r[b] = (C[k][b] & bq[M - 1]) ^ (bi[b] & d[M - 1]);
#pragma unroll
          for (int jj = M - 2; jj >= 0; jj--) {
            const uint32_t top = r[M - 1];
#pragma unroll
            for (int b = M - 1; b > 0; b--) r[b] = r[b - 1];
            r[0] = top;
            if (M == 13) {
              r[1] ^= top;
              r[3] ^= top;
              r[4] ^= top;
            } else {
              r[3] ^= top;
            }
#pragma unroll
            for (int b = 0; b < M; b++) r[b] ^= (C[k][b] & bq[jj]) ^ (bi[b] & d[jj]);
          }
          uint32_t *bn = BP + (i + 1) * M;
#pragma unroll
          for (int b = 0; b < M; b++) {
            const uint32_t cold = C[k][b];
            if (in) C[k][b] = r[b];
            if (i + 1 <= T) bn[b] = (U & cold) | (~U & bi[b]);
          }
          __syncwarp();
        }
      }
#pragma unroll
      for (int b = 0; b < M; b++) bq[b] = (U & d[b]) | (~U & bq[b]);
      if (lane < M) BP[lane] = 0;
      __syncwarp();
    }
    // C <- C / C_0 (C_0 = lambda != 0)
    {
      uint32_t c0[M], inv[M];
#pragma unroll
      for (int b = 0; b < M; b++) c0[b] = __shfl_sync(0xffffffffu, C[0][b], 0);
      bs_inv<M>(inv, c0);
#pragma unroll
      for (int k = 0; k < NS; k++) {
        uint32_t r[M];
        bs_mul_reg<M>(r, inv, C[k]);
#pragma unroll
        for (int b = 0; b < M; b++) C[k][b] = r[b];
      }
    }
#pragma unroll
    for (int k = 0; k < NS; k++)
#pragma unroll
      for (int b = 0; b < M; b++) SP[(lane + 32 * k) * M + b] = C[k][b];
    __syncwarp();
    if (live) {
      uint16_t *sig = Sig + op * SIG;
#pragma unroll 1
      for (int deg = 0; deg < SIG; deg++) {
        const int i = T - deg;
        uint32_t v = 0;
        if (i >= 0) {
#pragma unroll
          for (int b = 0; b < M; b++) v |= ((SP[i * M + b] >> lane) & 1u) << b;
        }
        v |= (deg == 0 && L > T) ? 0x8000u : 0u;
        sig[deg] = (uint16_t)v;
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- BM, latency form
// Used for small batches (fewer requests than the bit-sliced form needs to
// fill the GPU): per-request latency is one warp walking 2t iterations of
// ~100 instructions instead of a group of 32 walking ~1500.
// One warp per request (persistent grid). Coefficient i of C (connection
// polynomial) lives in lane i%32, slot i/32, as its log only: the update
// C_i += f B_i is done in the log domain with Zech logarithms,
// log(a + b) = log a + zech(log b - log a), one table lookup instead of an
// antilog and a log. Any log at or above the zero sentinel 2q-2 means 0.
// B = x^s B' is kept unshifted: B' (the connection polynomial before the last
// length change, as logs) sits in a per-warp shared array behind a guard of
// 2t zero logs, so B_i is the entry at i - s and the per-iteration shift is
// s += 1. The syndrome logs sit behind a 32-entry zero guard, so the
// discrepancy reads s_{n-i} for every lane of an active slot without a
// per-lane test (C_i = 0 above deg C). Coefficients above t are never
// updated, as in the library's fixed-size arrays.
// Degree bounds used to skip empty slots (exact, also for undecodable input):
// before iteration n, deg C <= L and deg B <= n+1-L, so the discrepancy needs
// coefficients i <= min(L, t) and the update i <= min(max(L, n+1-L), t).
template <int SET>
struct BMLatLayout {
  using p = P<SET>;
  static constexpr int Q = p::q, T = p::t;
  static constexpr int NS = (T + 1 + 31) / 32;
  static constexpr int exp_off = 0, log_off = 2 * Q, zech_off = 3 * Q;
  static constexpr int shared_u16 = 4 * Q;
  static constexpr int sguard = 32, bguard = 2 * T;
  static constexpr int s_off = 0, s_len = sguard + 2 * T;          // per warp, u16
  static constexpr int b_off = s_len, b_len = bguard + 32 * NS;
  static constexpr int warp_u16 = (s_len + b_len + 1) & ~1;
  static constexpr int bytes(int warps) { return shared_u16 * 2 + warps * warp_u16 * 2; }
};

template <int SET>
__global__ void __launch_bounds__(kBMLatWarps * 32, 2) dec_bm_lat_kernel(const uint32_t *__restrict__ S2, int lds2,
                                                                  FieldDev fd, const Segs segs,
                                                                  uint16_t *__restrict__ Sig) {
  using p = P<SET>;
  using LY = BMLatLayout<SET>;
  constexpr int M = p::m, Q = p::q, T = p::t, D = p::fft_d;
  constexpr int ZL = GFLog<M>::zero_log;
  constexpr int NS = LY::NS;
  constexpr int NSY = (2 * T + 31) / 32;
  constexpr int SIG = 1 << D;
  extern __shared__ __align__(16) uint16_t lsm[];
  uint16_t *gexp = lsm + LY::exp_off;
  uint16_t *glog = lsm + LY::log_off;
  uint16_t *zech = lsm + LY::zech_off;
  for (int i = threadIdx.x; i < 2 * Q - 1; i += blockDim.x) gexp[i] = fd.gexp[i];
  for (int i = threadIdx.x; i < Q; i += blockDim.x) {
    glog[i] = fd.glog[i];
    zech[i] = fd.zech[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint16_t *wsm = lsm + LY::shared_u16 + warp * LY::warp_u16;
  uint16_t *slog = wsm + LY::s_off + LY::sguard;  // slog[-32 .. -1] = zero logs
  uint16_t *blog = wsm + LY::b_off + LY::bguard;  // blog[-2t .. -1] = zero logs
  for (int i = lane; i < LY::sguard; i += 32) wsm[LY::s_off + i] = (uint16_t)ZL;
  for (int i = lane; i < LY::bguard; i += 32) wsm[LY::b_off + i] = (uint16_t)ZL;
  __syncthreads();
  const long long N = seg_rows(segs);
  const int nwb = blockDim.x >> 5;  // warps per block (a launch parameter up to kBMLatWarps)
  const long long nwarps = (long long)gridDim.x * nwb;
  for (long long op = (long long)blockIdx.x * nwb + warp; op < N; op += nwarps) {
    int seg;
    if (!seg_live(segs, op, &seg)) continue;  // warp-uniform
    const uint32_t *srow = S2 + op * lds2;
#pragma unroll
    for (int k = 0; k < NSY; k++) {
      const int j = lane + 32 * k;
      if (j < 2 * T) {
        const int b = j * M, w = b >> 5, sh = b & 31;
        uint32_t v = srow[w] >> sh;
        if (sh + M > 32) v |= srow[w + 1] << (32 - sh);
        slog[j] = glog[v & (Q - 1)];
      }
    }
    // B' = 1, s = 1 (B = x)
#pragma unroll
    for (int k = 0; k < NS; k++) blog[lane + 32 * k] = (lane + 32 * k == 0) ? 0 : (uint16_t)ZL;
    __syncwarp();
    uint32_t lC[NS];
#pragma unroll
    for (int k = 0; k < NS; k++) lC[k] = (lane + 32 * k == 0) ? 0 : ZL;
    int L = 0, sft = 1;
    uint32_t lb = 0;  // log b, b = 1
#pragma unroll 1
    for (int n = 0; n < 2 * T; n++) {
      const int bd = L < T ? L : T;                       // discrepancy: i <= min(L, t) (L <= n)
      int bu = (L > n + 1 - L) ? L : n + 1 - L;           // update: i <= min(max(L, n+1-L), t)
      bu = bu < T ? bu : T;
      uint32_t dp = 0;
      const uint16_t *sn = slog + n - lane;
#pragma unroll
      for (int k = 0; k < NS; k++)
        if (32 * k <= bd) dp ^= gf_mul_log<M>(gexp, lC[k], sn[-32 * k]);
      const uint32_t d = __reduce_xor_sync(0xffffffffu, dp);
      if (d) {
        const bool upd = (n >= 2 * L);
        const int ld = glog[d];
        int lf = ld - (int)lb;
        if (lf < 0) lf += Q - 1;
        const uint16_t *bs = blog + lane - sft;
        uint32_t lco[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) {
          lco[k] = lC[k];
          if (32 * k <= bu) {
            // log(C_i + f B_i): p = log(f B_i); zero B_i keeps C_i, zero C_i takes p
            constexpr uint32_t Q1 = Q - 1;
            const uint32_t lbi = bs[32 * k], lc = lC[k];
            uint32_t pl = (uint32_t)lf + lbi;
            pl = min(pl, pl - Q1);                      // < q-1 when B_i != 0
            uint32_t kk = pl - lc;                      // log(f B_i / C_i) mod q-1
            kk = min(kk + Q1, kk);
            const uint32_t z = zech[min(kk, Q1 - 1)];   // index clamped for the zero cases
            uint32_t nl = lc + z;
            nl = min(nl, nl - Q1);                      // >= 2q-2 when the sum is 0
            nl = (lc >= (uint32_t)ZL) ? pl : nl;
            nl = (lbi >= (uint32_t)ZL) ? lc : nl;
            const bool in = (k < NS - 1) || (lane + 32 * k <= T);  // coefficients above t stay zero
            if (in) lC[k] = nl;
          }
        }
        if (upd) {
          __syncwarp();  // every lane has read B' before it is replaced
#pragma unroll
          for (int k = 0; k < NS; k++)
            if (32 * k <= bu) blog[lane + 32 * k] = (uint16_t)lco[k];
          __syncwarp();
          L = n + 1 - L;
          lb = ld;
          sft = 0;
        }
      }
      sft++;
    }
    // sigma(x) = sum_deg C[t-deg] x^deg -> FFT coefficient slots (deg < 2^d);
    // coefficients are < 2^m <= 2^13, so bit 15 is free for the length flag
    uint16_t *sig = Sig + op * SIG;
    for (int x = lane; x < SIG; x += 32)
      if (x > T) sig[x] = 0;
#pragma unroll
    for (int k = 0; k < NS; k++) {
      const int i = lane + 32 * k;
      const int deg = T - i;
      // bit 15 of the constant coefficient flags a final length L > t
      const uint32_t c = gexp[min(lC[k], (uint32_t)ZL)];
      if (i <= T && deg < SIG) sig[deg] = (uint16_t)(c | ((deg == 0 && L > T) ? 0x8000u : 0u));
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- root finding
// One warp per request: additive FFT of sigma over all 2^m field elements
// (Gao-Mateer, basis beta_i = 2^i so point c is the element c), the error
// positions, the weight and the re-encryption check.
// The top-down part (twist + radix conversion) turns the 2^d coefficients
// into 2^d leaf constants. Every bottom-up butterfly level has stride < 2^d,
// so the 2^m evaluations split into 2^(m-d) independent chunks of 2^d
// consecutive elements that all start from the same leaves.
// The bottom-up pass is bit-sliced over the chunks: a 32-bit word carries one
// bit plane of the same element slot of 32 chunks, so a butterfly of 32
// chunks is one bit-sliced GF(2^m) product (m^2 AND-XOR steps and the
// reduction) instead of 64 table lookups. Lane and register slot together
// address the 2^d slots; a level whose pair bit is a lane bit first swaps
// that lane bit with the register bit of the oldest finished level (one
// shuffle per plane of half the slots), so every butterfly is in-register.
// A root (sigma(a) = 0, with a^(2^d) added for the separate leading term via
// Frobenius tables, since (hi + lo)^(2^d) = hi^(2^d) + lo^(2^d)) is mapped to
// its code position through the key's inverse support table; only roots touch
// that table.
template <int SET, bool CT>
struct RootLayout {
  using p = P<SET>;
  static constexpr int Q = p::q, D = p::fft_d, SIG = 1 << D, NC = Q >> D, NH = NC / 32, M = p::m;
  // u16 region: the table form's log/antilog tables and twist logs, or (constant-time form) the
  // multiplication columns c x^i of every twist constant c; then the Frobenius table
  static constexpr int exp_off = 0, exp_len = CT ? 0 : 2 * Q;
  static constexpr int log_off = exp_off + exp_len, log_len = CT ? 0 : Q;
  static constexpr int twist_off = log_off + log_len, twist_len = CT ? (2 << D) * M : 2 << D;
  static constexpr int frlo_off = twist_off + twist_len, frlo_len = SIG;
  static constexpr int shared_u16 = (frlo_off + frlo_len + 1) & ~1;
  // u32 region: bit-sliced alpha, bit-sliced frob_hi
  // bit-sliced butterfly constants, one row of NH * M planes per (level, block): rows padded to an odd
  // stride so that 32 lanes reading 32 different rows hit 32 different banks
  static constexpr int abs_row = NH * M, abs_stride = abs_row | 1;
  static constexpr int abs_off = shared_u16 / 2, abs_len = (SIG - 1) * abs_stride;
  static constexpr int fhbs_off = abs_off + abs_len, fhbs_len = NH * M;
  static constexpr int shared_u32 = fhbs_off + fhbs_len;
  static constexpr int ewp = (p::ew + 1) & ~1;
  // per warp (u32): e words | roots [t] (element, then pos << 16 | element)
  static constexpr int roots_off = ewp;
  static constexpr int warp_u32 = (roots_off + p::t + 1) & ~1;
  static constexpr int bytes(int warps) { return shared_u32 * 4 + warps * warp_u32 * 4; }
};

// Chunk-slot index held by (lane, register slot j = j0 + 2 j1) while level l
// of the bottom-up pass is processed (l = -1: after the last level).
// Register bit 0 pairs at every level but one: a level whose pair bit is a
// lane bit first swaps that lane bit with register bit 0, whose slot bit
// (the level before) is finished. D = 7 (4 slots per lane) starts with
// slot bits 6, 5 in register bits 0, 1 and lane bits 0..4 = slot bits 0..4;
// level 5 pairs on register bit 1. D = 6 (2 slots) starts with slot bit 5 in
// register bit 0.
template <int D>
__device__ __forceinline__ int chunk_slot(int l, int lane, int j) {
  const int j0 = j & 1, j1 = j >> 1;
  if (D == 7) {
    if (l >= 5) return lane | (j1 << 5) | (j0 << 6);
    if (l < 0) return j0 | ((lane & 15) << 1) | (j1 << 5) | ((lane >> 4) << 6);
    return (lane & ((1 << l) - 1)) | (j0 << l) | (((lane >> l) & ((1 << (4 - l)) - 1)) << (l + 1)) | (j1 << 5) |
           ((lane >> 4) << 6);
  } else {
    if (l >= 5) return lane | (j0 << 5);
    if (l < 0) return j0 | (lane << 1);
    return (lane & ((1 << l) - 1)) | (j0 << l) | ((lane >> l) << (l + 1));
  }
}

// r = a * b in GF(2^M), bit-sliced (plane i = bit i of 32 elements), Horner
// over the planes of a (read from shared memory one plane per step):
// r <- r x + a_j b, where r x reduces by x^M = x^4 + x^3 + x + 1 (M = 13) or
// x^3 + 1 (M = 12), the field polynomials of the log/antilog tables.
// M^2 AND-XOR steps plus 3 (1) XORs per step; only r and b stay live.
template <int M>
__device__ __forceinline__ void bs_mul(uint32_t (&r)[M], const uint32_t *__restrict__ a, const uint32_t (&b)[M]) {
  {
    const uint32_t aj = a[M - 1];
#pragma unroll
    for (int i = 0; i < M; i++) r[i] = b[i] & aj;
  }
#pragma unroll
  for (int j = M - 2; j >= 0; j--) {
    const uint32_t top = r[M - 1];
#pragma unroll
    for (int i = M - 1; i > 0; i--) r[i] = r[i - 1];
    r[0] = top;
    if (M == 13) {
      r[1] ^= top;
      r[3] ^= top;
      r[4] ^= top;
    } else {
      r[3] ^= top;
    }
    const uint32_t aj = a[j];
#pragma unroll
    for (int i = 0; i < M; i++) r[i] ^= b[i] & aj;
  }
}

// One radix-conversion step of the top-down pass on the coefficient slots
// x = lane + 32 j held in registers: with tau = 2^pb (a bit of x), pass 1
// adds slot x + tau into every slot x whose bits (pb+1, pb) are (1, 0), then
// pass 2 adds slot x + tau into every slot whose bits are (0, 1) (whose
// partner is a pass-1 target). Bits 0..4 of x are lane bits, bits 5.. the
// register index: a pair inside a lane is an XOR, a pair across lanes one
// shuffle per register.
template <int VPL>
__device__ __forceinline__ void radix_step(uint32_t (&v)[VPL], int pb, int lane) {
  if (pb >= 5) {  // bits 6, 5 = register bits 1, 0 (VPL == 4)
    if constexpr (VPL == 4) {
      v[2] ^= v[3];
      v[1] ^= v[2];
    }
  } else if (pb == 4) {  // bit 5 = register bit 0, bit 4 = lane bit 4
    const bool hi = (lane & 16) != 0;
#pragma unroll
    for (int j = 1; j < VPL; j += 2) {  // (1, 0) <- (1, 1): register bit 0 set, partner lane ^ 16
      const uint32_t got = __shfl_xor_sync(0xffffffffu, v[j], 16);
      if (!hi) v[j] ^= got;
    }
#pragma unroll
    for (int j = 0; j < VPL; j += 2) {  // (0, 1) <- (1, 0): register j + 1 of lane ^ 16
      const uint32_t got = __shfl_xor_sync(0xffffffffu, v[j + 1], 16);
      if (hi) v[j] ^= got;
    }
  } else {  // both lane bits
    const int b = (lane >> pb) & 3;
#pragma unroll
    for (int j = 0; j < VPL; j++) {
      const uint32_t got = __shfl_xor_sync(0xffffffffu, v[j], 1 << pb);
      if (b == 2) v[j] ^= got;
    }
#pragma unroll
    for (int j = 0; j < VPL; j++) {
      const uint32_t got = __shfl_xor_sync(0xffffffffu, v[j], 3 << pb);
      if (b == 1) v[j] ^= got;
    }
  }
}

// the even bits of x, compacted into the low 16 bits
__device__ __forceinline__ uint32_t comp_even16(uint32_t x) {
  x &= 0x55555555u;
  x = (x | (x >> 1)) & 0x33333333u;
  x = (x | (x >> 2)) & 0x0F0F0F0Fu;
  x = (x | (x >> 4)) & 0x00FF00FFu;
  x = (x | (x >> 8)) & 0x0000FFFFu;
  return x;
}
// exchanges the bits at p and p + d for every p in mask
__device__ __forceinline__ uint32_t delta_swap(uint32_t x, int d, uint32_t mask) {
  const uint32_t t = ((x >> d) ^ x) & mask;
  return x ^ t ^ (t << d);
}
// bit i -> bit bitrev_5(i): index bits 0 <-> 4 and 1 <-> 3 exchanged
__device__ __forceinline__ uint32_t rev5_bits(uint32_t x) {
  x = delta_swap(x, 15, 0x0000AAAAu);
  return delta_swap(x, 6, 0x00CC00CCu);
}

// v * c for a public constant c given by its columns c x^i (i < M): no
// address or branch depends on v
template <int M>
__device__ __forceinline__ uint32_t gf_mul_cols(uint32_t v, const uint16_t *cols) {
  uint32_t r = 0;
#pragma unroll
  for (int i = 0; i < M; i++) r ^= (uint32_t)cols[i] & (0u - ((v >> i) & 1u));
  return r;
}

// CT: the constant-time form (the twist multiplies by table-free columns; the
// tables indexed by coefficient values are not loaded)
template <int SET, bool CT>
__global__ void __launch_bounds__(kRootWarps * 32, 2) dec_root_kernel(const uint16_t *__restrict__ Sig,
                                                                   const uint32_t *__restrict__ S2, int lds2,
                                                                   const DecKeys keys, FieldDev fd, const Segs segs,
                                                                   uint32_t *__restrict__ E, int lde,
                                                                   int *__restrict__ okout) {
  using p = P<SET>;
  using LY = RootLayout<SET, CT>;
  constexpr int M = p::m, Q = p::q, T = p::t, D = p::fft_d, SIG = LY::SIG, NH = LY::NH;
  constexpr int NW = (p::n + 31) / 32;
  constexpr int VPL = SIG / 32;  // chunk slots per lane
  constexpr int LOGV = (VPL == 4) ? 2 : 1;
  static_assert(VPL == (1 << LOGV) && NH == 2, "chunk geometry: 64 chunks, two halves of 32");
  static_assert(M == 12 || M == 13, "field polynomial");
  extern __shared__ __align__(16) uint32_t rsm[];
  uint16_t *sh16 = reinterpret_cast<uint16_t *>(rsm);
  uint16_t *gexp = sh16 + LY::exp_off;
  uint16_t *glog = sh16 + LY::log_off;
  uint16_t *tlog = sh16 + LY::twist_off;
  uint16_t *frlo = sh16 + LY::frlo_off;
  uint32_t *abs_ = rsm + LY::abs_off;
  uint32_t *fhbs = rsm + LY::fhbs_off;
  if constexpr (CT) {
    for (int i = threadIdx.x; i < LY::twist_len; i += blockDim.x) tlog[i] = fd.fft_twist_cols[i];
  } else {
    for (int i = threadIdx.x; i < 2 * Q - 1; i += blockDim.x) gexp[i] = fd.gexp[i];
    for (int i = threadIdx.x; i < Q; i += blockDim.x) glog[i] = fd.glog[i];
    for (int i = threadIdx.x; i < (2 << D); i += blockDim.x) tlog[i] = fd.fft_twist_log[i];
  }
  for (int i = threadIdx.x; i < SIG; i += blockDim.x) frlo[i] = fd.frob_lo[i];
  for (int i = threadIdx.x; i < (SIG - 1) * LY::abs_row; i += blockDim.x)
    abs_[(i / LY::abs_row) * LY::abs_stride + i % LY::abs_row] = fd.fft_alpha_bs[i];
  for (int i = threadIdx.x; i < LY::fhbs_len; i += blockDim.x) fhbs[i] = fd.frob_hi_bs[i];
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *wbase = rsm + LY::shared_u32 + warp * LY::warp_u32;
  uint32_t *esm = wbase;
  uint32_t *roots = wbase + LY::roots_off;

  const long long N = seg_rows(segs);
  const int nwb = blockDim.x >> 5;  // warps per block (a launch parameter up to kRootWarps)
  const long long nwarps = (long long)gridDim.x * nwb;
  for (long long op = (long long)blockIdx.x * nwb + warp; op < N; op += nwarps) {
    int seg;
    if (!seg_live(segs, op, &seg)) continue;  // warp-uniform
    const DecKeyDev &key = keys.k[seg];
    const uint16_t *sig = Sig + op * SIG;
    for (int w = lane; w < NW; w += 32) esm[w] = 0;
    // top-down, in registers: lane holds the coefficient slots x = lane + 32 j
    // (j < VPL): twist by the level's first basis element, then radix-convert
    // g(x) = g0(x^2+x) + x g1(x^2+x) on the 2^l interleaved sub-polynomials
    uint32_t vv[VPL];
#pragma unroll
    for (int j = 0; j < VPL; j++) vv[j] = sig[lane + 32 * j];
    const bool long_lfsr = (__shfl_sync(0xffffffffu, vv[0], 0) >> 15) != 0;  // BM ended with L > t
    vv[0] &= 0x7FFFu;
#pragma unroll 1
    for (int l = 0; l < D; l++) {
      if (l) {
        const int tw0 = (2 << D) - (2 << (D - l));
        if constexpr (CT) {
#pragma unroll
          for (int j = 0; j < VPL; j++) vv[j] = gf_mul_cols<M>(vv[j], tlog + (tw0 + ((lane + 32 * j) >> l)) * M);
        } else {
#pragma unroll
          for (int j = 0; j < VPL; j++) vv[j] = gf_mul_log<M>(gexp, glog[vv[j]], tlog[tw0 + ((lane + 32 * j) >> l)]);
        }
      }
#pragma unroll 1
      for (int pb = D - 2; pb >= l; pb--) radix_step<VPL>(vv, pb, lane);
    }
    __syncwarp();  // esm cleared before the root stores below
    // leaves in the bottom-up pass's slot order (chunk_slot at level D - 1)
    uint32_t leaf[VPL];
    if constexpr (VPL == 4) {  // slot = lane | j1 << 5 | j0 << 6
      leaf[0] = vv[0];
      leaf[1] = vv[2];
      leaf[2] = vv[1];
      leaf[3] = vv[3];
    } else {  // slot = lane | j << 5
#pragma unroll
      for (int j = 0; j < VPL; j++) leaf[j] = vv[j];
    }

    uint32_t zm0[VPL], zm1[VPL];  // constant-time form: the zero masks of both chunk halves
    // table form: the roots, listed per half as found. sigma is monic of
    // degree t, so it has at most t zeros; each lane writes its own at an
    // offset from a warp prefix sum of the counts (shared memory only)
    int nfound = 0;
#pragma unroll 1
    for (int h = 0; h < NH; h++) {
      uint32_t v[VPL][M];
#pragma unroll
      for (int j = 0; j < VPL; j++)
#pragma unroll
        for (int b = 0; b < M; b++) v[j][b] = 0u - ((leaf[j] >> b) & 1u);
      // one loop body for every level (a runtime loop keeps the unrolled
      // bit-sliced products small enough for the instruction cache)
#pragma unroll 1
      for (int l = D - 1; l >= 0; l--) {
        if (VPL == 4 && l == D - 2) {
          // pairs on register bit 1 (slot bit 5)
#pragma unroll
          for (int j = 0; j < 2; j++) {
            const int xh = chunk_slot<D>(l, lane, j) >> (l + 1);
            const uint32_t *ap = abs_ + ((SIG - (SIG >> l)) + xh) * LY::abs_stride + h * M;
            uint32_t pr[M];
            bs_mul<M>(pr, ap, v[j + 2]);
#pragma unroll
            for (int b = 0; b < M; b++) {
              v[j][b] ^= pr[b];
              v[j + 2][b] ^= v[j][b];
            }
          }
          continue;
        }
        if (l < D - LOGV) {
          // lane bit l <-> register bit 0: the lane with lane bit 0 keeps its
          // slots with register bit 0 and trades the others with its partner
          const bool lo = ((lane >> l) & 1) == 0;
#pragma unroll
          for (int j = 0; j < VPL; j += 2) {
#pragma unroll
            for (int b = 0; b < M; b++) {
              const uint32_t send = lo ? v[j + 1][b] : v[j][b];
              const uint32_t got = __shfl_xor_sync(0xffffffffu, send, 1 << l);
              if (lo) v[j + 1][b] = got;
              else v[j][b] = got;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < VPL; j += 2) {
          const int xh = chunk_slot<D>(l, lane, j) >> (l + 1);
          const uint32_t *ap = abs_ + ((SIG - (SIG >> l)) + xh) * LY::abs_stride + h * M;
          uint32_t pr[M];
          bs_mul<M>(pr, ap, v[j + 1]);
#pragma unroll
          for (int b = 0; b < M; b++) {
            v[j][b] ^= pr[b];
            v[j + 1][b] ^= v[j][b];
          }
        }
      }
      // zero planes -> roots; slot VPL * lane + j of chunk 32 h + k
      uint32_t zero[VPL];
#pragma unroll
      for (int j = 0; j < VPL; j++) {
        // read here, not hoisted out of the chunk loop (the root stores below
        // may alias), so the per-plane masks are not held across it
        const uint32_t frl = p::lead ? frlo[chunk_slot<D>(-1, lane, j)] : 0u;
        uint32_t nz = 0;
#pragma unroll
        for (int b = 0; b < M; b++) {
          uint32_t w = v[j][b];
          if (p::lead) w ^= fhbs[h * M + b] ^ (0u - ((frl >> b) & 1u));
          nz |= w;
        }
        zero[j] = ~nz;
      }
      if constexpr (CT) {
#pragma unroll
        for (int j = 0; j < VPL; j++) {
          if (h == 0) zm0[j] = zero[j];
          else zm1[j] = zero[j];
        }
        continue;
      }
      int mine = 0;
#pragma unroll
      for (int j = 0; j < VPL; j++) mine += __popc(zero[j]);
      int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
      }
      int off = nfound + incl - mine;
      nfound += __shfl_sync(0xffffffffu, incl, 31);
#pragma unroll
      for (int j = 0; j < VPL; j++) {
        uint32_t z = zero[j];
        while (z) {
          const int k = __ffs(z) - 1;
          z &= z - 1;
          if (off < T) roots[off] = (uint32_t)(((32 * h + k) << D) | chunk_slot<D>(-1, lane, j));
          off++;
        }
      }
    }
    if constexpr (CT) {
      // the error vector in field-element order with bit-reversed index, the input order of the key's Benes
      // network: word w holds y[32 w + i] = zero(alpha) for alpha = bitrev_m(32 w + i), i.e. the slot
      // bitrev_d(w >> 1) of the chunks 2 bitrev_5(i) + (w & 1). Lane and register j hold that slot's zero
      // masks over all 64 chunks: every other bit, compacted, with its 5-bit index reversed.
      static_assert(M - D == 6, "64 chunks of 2^d slots");
      uint32_t *erow = E + op * lde;
#pragma unroll
      for (int j = 0; j < VPL; j++) {
        const int sl = chunk_slot<D>(-1, lane, j);
        const int wb = (int)(__brev((unsigned)sl) >> (32 - D)) << 1;
#pragma unroll
        for (int b0 = 0; b0 < 2; b0++) {
          const uint32_t e32 = comp_even16(zm0[j] >> b0) | (comp_even16(zm1[j] >> b0) << 16);
          erow[wb | b0] = rev5_bits(e32);
        }
      }
      if (lane == 0) okout[op] = long_lfsr ? 0 : 1;  // weight and syndromes are checked after the Benes network
      __syncwarp();
      continue;
    }
    // code positions of the listed roots: independent loads, lane r taking
    // entries r, r + 32, ...
    constexpr int NSC = (T + 31) / 32;
    const int nroots = nfound < T ? nfound : T;
    __syncwarp();
    int weight = 0;
    {
      uint32_t pos[NSC];
#pragma unroll
      for (int k = 0; k < NSC; k++) {
        const int r = lane + 32 * k;
        pos[k] = r < nroots ? key.invL[roots[r]] : 0xFFFFu;
      }
#pragma unroll
      for (int k = 0; k < NSC; k++) {
        const int r = lane + 32 * k;
        if (r < nroots && pos[k] < (uint32_t)p::n) {
          weight++;
          atomicOr(&esm[pos[k] >> 5], 1u << (pos[k] & 31));
          roots[r] |= pos[k] << 16;
        }
      }
    }
    weight = __reduce_add_sync(0xffffffffu, weight);
    __syncwarp();

    // Accept when the t roots lie in the support, BM's length is <= t and the
    // first t syndromes of the found error equal the received ones. That is
    // the library's full 2t-syndrome check: with L <= t, the connection
    // polynomial C (sigma reversed) annihilates the received sequence from
    // index t on, and also the found error's sequence sum_i w2_i L_i^j (sigma
    // vanishes at every L_i), so the two sequences agree iff their first t
    // terms do. With L > t no error of weight <= t has these syndromes (its
    // locator would be a shorter LFSR), so the library's check fails as well.
    bool ok = (weight == T) && !long_lfsr;
    if (ok) {
      // first t syndromes of the found error: XOR of the key's columns at the
      // t positions (then every root is in the support and in the list). Each
      // half-warp reads whole rows, lane c of a half the 16-byte chunk c, so a
      // load instruction covers two rows contiguously; the halves are added by
      // one shuffle and compared with the received words.
      constexpr int TW = (T * M + 31) / 32;
      constexpr int TW4 = (TW + 3) / 4;
      static_assert(TW4 <= 16, "a row of the first t syndromes fits half a warp of 16-byte chunks");
      const int c = lane & 15;
      uint4 acc = make_uint4(0, 0, 0, 0);
      if (c < TW4) {
#pragma unroll 16
        for (int r = lane >> 4; r < T; r += 2) {
          const uint4 v = reinterpret_cast<const uint4 *>(key.HT + (size_t)(roots[r] >> 16) * key.ldh)[c];
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
      uint32_t mism = 0;
      if (lane < TW4) {
        const uint32_t *srow = S2 + op * lds2;
        const uint32_t q4[4] = {acc.x, acc.y, acc.z, acc.w};
#pragma unroll
        for (int e2 = 0; e2 < 4; e2++) {
          const int word = 4 * lane + e2;
          if (word < TW) {
            const uint32_t msk = (word == TW - 1 && (T * M) % 32) ? ((1u << ((T * M) % 32)) - 1u) : 0xFFFFFFFFu;
            mism |= (q4[e2] ^ srow[word]) & msk;
          }
        }
      }
      ok = !__any_sync(0xffffffffu, mism != 0);
    }
    uint32_t *erow = E + op * lde;
    for (int it = lane; it < NW; it += 32) erow[it] = esm[it];
    if (lane == 0) okout[op] = ok ? 1 : 0;
    __syncwarp();
  }
}

// ---------------------------------------------------------------- tail
template <int SET, bool PC>
__global__ void __launch_bounds__(kTailThreads) dec_tail_kernel(const uint32_t *__restrict__ E, int lde,
                                                                const int *__restrict__ okin,
                                                                const uint8_t *__restrict__ Cin, const DecKeys keys,
                                                                uint8_t *__restrict__ K, int *__restrict__ rc,
                                                                const Segs segs) {
  using p = P<SET>;
  constexpr int SB = p::synd_bytes, CB = SB + (PC ? 32 : 0);  // C0 bytes, ciphertext bytes
  __shared__ uint32_t stage[kTailThreads / 32][32 * kStageStride];
  __shared__ const uint32_t *rows[kTailThreads / 32][32];
  const long long N = seg_rows(segs);
  const long long op = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long opc = op < N ? op : N - 1;  // every lane of a warp takes part in the staged hash
  int seg;
  const bool live = seg_live(segs, op, &seg);
  const DecKeyDev &key = keys.k[seg_find(segs, opc)];
  bool ok = okin[opc] != 0;
  const uint8_t *c = Cin + opc * CB;
  if constexpr (PC) {
    // plaintext confirmation (mc:crypto_kem/348864pc/vec/kem_dec.c:43-48): SHAKE256(2 || e, 32) of the
    // decoded e must equal C1 (its value when decoding failed does not change the outcome)
    auto none = [](int) -> uint32_t { return 0u; };
    uint64_t cf[4];
    kem_hash_staged<p::e_bytes, 1 + p::e_bytes>(cf, 2u, E + opc * lde, none, stage[threadIdx.x >> 5],
                                                rows[threadIdx.x >> 5]);
    uint32_t diff = 0;
#pragma unroll
    for (int j = 0; j < 32; j++) diff |= (uint32_t)c[SB + j] ^ ((uint32_t)(cf[j >> 3] >> (8 * (j & 7))) & 0xFFu);
    ok = ok && diff == 0;
  }
  // b || (e or s) || c, s the key's n/8 bytes (stored zero-padded to whole words). The choice is a
  // mask, not an address (mc:crypto_kem/348864/vec/kem_dec.c:51-55): the warp rewrites each of its
  // 32 rows as (e & mask) | (s & ~mask), reading both e and s with the same coalesced loads whatever
  // the outcome, and every lane hashes its own (blended) row.
  {
    const unsigned okmask = __ballot_sync(0xffffffffu, ok);
    const long long g0 = opc - (threadIdx.x & 31);  // the warp's first row (clamped rows repeat N-1)
    for (int r = 0; r < 32; r++) {
      const long long row = g0 + r < N ? g0 + r : N - 1;
      const uint32_t m = ((okmask >> r) & 1u) ? 0xFFFFFFFFu : 0u;
      const uint32_t *sr = reinterpret_cast<const uint32_t *>(keys.k[seg_find(segs, row)].s);
      uint32_t *er = const_cast<uint32_t *>(E) + row * lde;
      for (int w = threadIdx.x & 31; w < p::ew; w += 32) er[w] = (er[w] & m) | (sr[w] & ~m);
    }
    __syncwarp();
  }
  const uint32_t *erow = E + opc * lde;
  // word loads when every ciphertext row is 4-byte aligned (the buffer and the row length), else bytes
  const bool c_words = (CB % 4 == 0) && ((reinterpret_cast<uintptr_t>(Cin) & 3) == 0);
  auto cword = [&](int w) -> uint32_t {
    if (c_words) return 4 * w < CB ? reinterpret_cast<const uint32_t *>(c)[w] : 0u;
    uint32_t v = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (4 * w + k < CB) v |= (uint32_t)c[4 * w + k] << (8 * k);
    return v;
  };
  uint64_t h[4];
  kem_hash_staged<p::e_bytes, p::pre_bytes + (PC ? 32 : 0)>(h, ok ? 1u : 0u, erow, cword, stage[threadIdx.x >> 5],
                                                             rows[threadIdx.x >> 5]);
  if (!live) return;
  bool pad_bad = false;
  if (p::mt % 8) pad_bad = (c[SB - 1] >> (p::mt % 8)) != 0;
  uint8_t *k = K + op * 32;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int bb = 0; bb < 8; bb++) k[8 * i + bb] = pad_bad ? 0xFF : (uint8_t)(h[i] >> (8 * bb));
  if (rc) rc[op] = pad_bad ? -1 : 0;
}

// ---------------------------------------------------------------- launchers
template <int SET>
cudaError_t launch_pack_ct(const uint8_t *C, const Segs &segs, uint32_t *X, int ldx, bool pc, cudaStream_t st) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  const long long total = N * ldx;
  if (pc)
    pack_ct_kernel<SET, true><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(C, segs, X, ldx);
  else
    pack_ct_kernel<SET, false><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(C, segs, X, ldx);
  return cudaGetLastError();
}

template <typename K>
static int persistent_blocks(K kernel, int threads, int smem, long long work_items, int items_per_block) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (per_sm < 1) per_sm = 1;
  long long need = (work_items + items_per_block - 1) / items_per_block;
  long long blocks = (long long)sms * per_sm;
  return (int)(blocks < need ? blocks : need);
}

// Warps per block of the bit-sliced forms: at most `warps`, and no more than
// the groups of 32 requests need to spread over every SM (1024 groups take 7
// warps on 147 SMs, not 14 on 74).
static int bm_block_warps(long long N, int warps) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) return warps;
  const long long per_sm = ((N + 31) / 32 + sms - 1) / sms;
  return per_sm < warps ? (int)(per_sm > 0 ? per_sm : 1) : warps;
}

template <int SET>
cudaError_t launch_dec_bm(const uint32_t *S2, int lds2, FieldDev fd, const Segs &segs, uint16_t *Sig,
                          cudaStream_t st, int warps, bool ct) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  if (warps < 0 || warps > kBMWarps) return cudaErrorInvalidValue;
  if (warps == 0) warps = kBMWarps;
  if (ct) {  // constant-time form, every batch size
    warps = bm_block_warps(N, warps < kBMCtWarps ? warps : kBMCtWarps);
    const int smem_ct = BMCtLayout<SET>::bytes(warps);
    cudaError_t err = cudaFuncSetAttribute(dec_bm_ct_kernel<SET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           BMCtLayout<SET>::bytes(kBMCtWarps));
    if (err != cudaSuccess) return err;
    const int gb = persistent_blocks(dec_bm_ct_kernel<SET>, warps * 32, smem_ct, (N + 31) / 32, warps);
    dec_bm_ct_kernel<SET><<<gb, warps * 32, smem_ct, st>>>(S2, lds2, segs, Sig);
    return cudaGetLastError();
  }
  if (N < kBMBitslicedMinRows) {  // small batch: warp per request (lower latency per request)
    // warps per block: the requests in one round over two blocks per SM when
    // they fit (8192 requests: 27 warps on 304 blocks, where fixed 24-warp
    // blocks left 896 requests for a second round), else kBMLatWarps
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long per_block = sms > 0 ? (N + 2LL * sms - 1) / (2LL * sms) : kBMLatWarps;
    const int lw = per_block < kBMLatWarps ? (per_block > 0 ? (int)per_block : 1) : kBMLatWarps;
    const int smem_l = BMLatLayout<SET>::bytes(lw);
    cudaError_t err = cudaFuncSetAttribute(dec_bm_lat_kernel<SET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           BMLatLayout<SET>::bytes(kBMLatWarps));
    if (err != cudaSuccess) return err;
    const int gl = persistent_blocks(dec_bm_lat_kernel<SET>, lw * 32, smem_l, N, lw);
    dec_bm_lat_kernel<SET><<<gl, lw * 32, smem_l, st>>>(S2, lds2, fd, segs, Sig);
    return cudaGetLastError();
  }
  warps = bm_block_warps(N, warps);
  const int smem_bm = BMLayout<SET>::bytes(warps);
  cudaError_t err = cudaFuncSetAttribute(dec_bm_kernel<SET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         BMLayout<SET>::bytes(kBMWarps));
  if (err != cudaSuccess) return err;
  const int gb = persistent_blocks(dec_bm_kernel<SET>, warps * 32, smem_bm, (N + 31) / 32, warps);
  dec_bm_kernel<SET><<<gb, warps * 32, smem_bm, st>>>(S2, lds2, fd, segs, Sig);
  return cudaGetLastError();
}

template <int SET, bool CT>
static cudaError_t launch_dec_root_form(const uint16_t *Sig, const uint32_t *S2, int lds2, const DecKeys &keys,
                                        FieldDev fd, const Segs &segs, uint32_t *E, int lde, int *ok,
                                        cudaStream_t st, int warps) {
  const long long N = seg_rows(segs);
  const int smem_rt = RootLayout<SET, CT>::bytes(warps);
  cudaError_t err = cudaFuncSetAttribute(dec_root_kernel<SET, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         RootLayout<SET, CT>::bytes(kRootWarps));
  if (err != cudaSuccess) return err;
  const int gr = persistent_blocks(dec_root_kernel<SET, CT>, warps * 32, smem_rt, N, warps);
  dec_root_kernel<SET, CT><<<gr, warps * 32, smem_rt, st>>>(Sig, S2, lds2, keys, fd, segs, E, lde, ok);
  return cudaGetLastError();
}

template <int SET>
cudaError_t launch_dec_root(const uint16_t *Sig, const uint32_t *S2, int lds2, const DecKeys &keys, FieldDev fd,
                            const Segs &segs, uint32_t *E, int lde, int *ok, cudaStream_t st, int warps, bool ct) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  if (warps < 0 || warps > kRootWarps) return cudaErrorInvalidValue;
  if (warps == 0) warps = kRootWarps;
  if (ct) {
    if (!fd.fft_twist_cols) return cudaErrorInvalidValue;
    return launch_dec_root_form<SET, true>(Sig, S2, lds2, keys, fd, segs, E, lde, ok, st, warps);
  }
  return launch_dec_root_form<SET, false>(Sig, S2, lds2, keys, fd, segs, E, lde, ok, st, warps);
}

// ---------------------------------------------------------------- constant-time positions and check
// The key's Benes network (its sk control bits, 2m - 1 layers of conditional
// swaps with strides 2^0 .. 2^(m-1) .. 2^0) applied to the field-order error
// vector y (y[v] = e at field element bitrev_m(v)) gives x[i] = y[pi(i)] with
// L_i = bitrev_m(pi(i)), i.e. the error at code position i: the same network
// and bit order that define the support (support_gen in the library). Warp per
// request, the q-bit vector in registers (word w = lane + 32 r); every layer
// touches every word with the control words as masks, so nothing depends on the
// error's positions. Then: bits >= n cleared, weight == t folded into ok.
// a layer whose pairs are registers r and r + DR of one lane (stride 2^s, s >= 10)
template <int WPL, int DR>
__device__ __forceinline__ void benes_reg_layer(uint32_t (&x)[WPL], const uint32_t *cw, int lane, int s) {
#pragma unroll
  for (int r = 0; r < WPL; r++) {
    if ((r & DR) || r + DR >= WPL) continue;
    const int wlo = lane + 32 * r;
    const uint32_t c = __ldg(cw + (((wlo >> (s - 4)) << (s - 5)) | (wlo & (32 * DR - 1))));
    const uint32_t t = (x[r] ^ x[r + DR]) & c;
    x[r] ^= t;
    x[r + DR] ^= t;
  }
}

template <int SET>
__global__ void __launch_bounds__(256) benes_ct_kernel(uint32_t *__restrict__ E, int lde, int *__restrict__ okio,
                                                       const DecKeys keys, const Segs segs) {
  using p = P<SET>;
  constexpr int M = p::m, Q = p::q, T = p::t, N = p::n;
  constexpr int WPL = Q / 32 / 32;  // words per lane
  constexpr int LW = Q / 64;         // control words per layer
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long NR = seg_rows(segs);
  for (long long op = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); op < NR; op += nwarps) {
    int seg;
    if (!seg_live(segs, op, &seg)) continue;  // warp-uniform
    const uint32_t *cond = keys.k[seg].cond;
    uint32_t *row = E + op * lde;
    uint32_t x[WPL];
#pragma unroll
    for (int r = 0; r < WPL; r++) x[r] = row[lane + 32 * r];
#pragma unroll 1
    for (int li = 0; li < 2 * M - 1; li++) {
      const int s = li < M ? li : 2 * M - 2 - li;
      const uint32_t *cw = cond + li * LW;
      if (s < 5) {
        const int d = 1 << s;
#pragma unroll
        for (int r = 0; r < WPL; r++) {
          const int w = lane + 32 * r;
          uint32_t c = (__ldg(cw + (w >> 1)) >> (16 * (w & 1))) & 0xFFFFu;
          // deposit the 16 control bits at the pairs' lower positions (bit s of the position clear)
#pragma unroll
          for (int pb = 3; pb >= 0; pb--) {
            if (pb >= s) {
              const uint32_t mp = pb == 3 ? 0xFF00FF00u : pb == 2 ? 0xF0F0F0F0u : pb == 1 ? 0xCCCCCCCCu : 0xAAAAAAAAu;
              c = (c & ~mp) | ((c & mp) << (1 << pb));
            }
          }
          const uint32_t t = ((x[r] >> d) ^ x[r]) & c;
          x[r] ^= t ^ (t << d);
        }
      } else if (s < 10) {  // partner word in lane ^ 2^(s-5)
        const int dl = 1 << (s - 5);
#pragma unroll
        for (int r = 0; r < WPL; r++) {
          const int wlo = (lane & ~dl) + 32 * r;
          const uint32_t c = __ldg(cw + (((wlo >> (s - 4)) << (s - 5)) | (wlo & (dl - 1))));
          const uint32_t xp = __shfl_xor_sync(0xffffffffu, x[r], dl);
          x[r] ^= (x[r] ^ xp) & c;
        }
      } else if (s == 10) {  // partner word in register r ^ 2^(s-10)
        benes_reg_layer<WPL, 1>(x, cw, lane, 10);
      } else if (s == 11) {
        benes_reg_layer<WPL, 2>(x, cw, lane, 11);
      } else {
        benes_reg_layer<WPL, 4>(x, cw, lane, 12);
      }
    }
    int weight = 0;
#pragma unroll
    for (int r = 0; r < WPL; r++) {
      const int w = lane + 32 * r;
      const uint32_t keep = 32 * w + 32 <= N ? 0xFFFFFFFFu : 32 * w >= N ? 0u : (1u << (N % 32)) - 1u;
      x[r] &= keep;
      weight += __popc(x[r]);
      if (w < lde) row[w] = x[r];
    }
    weight = __reduce_add_sync(0xffffffffu, weight);
    if (lane == 0) okio[op] = okio[op] & (weight == T ? 1 : 0);
  }
}

// ok &= (first t syndromes of the decoded error == the received ones): S3 from
// the dense product with the key's first-t syndrome matrix, S2 the received 2t
// syndromes (same packing, m bits each). Thread per request, every word.
template <int SET>
__global__ void ct_check_kernel(const uint32_t *__restrict__ S3, int lds3, const uint32_t *__restrict__ S2, int lds2,
                                int *__restrict__ okio, const Segs segs) {
  using p = P<SET>;
  constexpr int TM = p::t * p::m, TW = (TM + 31) / 32;
  const long long op = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int seg;
  if (op >= seg_rows(segs) || !seg_live(segs, op, &seg)) return;
  uint32_t mism = 0;
#pragma unroll 4
  for (int w = 0; w < TW; w++) {
    const uint32_t msk = (w == TW - 1 && (TM % 32)) ? ((1u << (TM % 32)) - 1u) : 0xFFFFFFFFu;
    mism |= (S3[op * lds3 + w] ^ S2[op * lds2 + w]) & msk;
  }
  okio[op] = okio[op] & (mism == 0 ? 1 : 0);
}

template <int SET>
cudaError_t launch_dec_ct_finish(const DecKeys &keys, const GemmKeys &htt, int engine, const Segs &segs, uint32_t *E,
                                 int lde, const uint32_t *S2, int lds2, uint32_t *S3, int lds3, int *ok, int *err,
                                 cudaStream_t st) {
  using p = P<SET>;
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  if (lde < p::q / 32 || lde < ct_htt_words(p::n)) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (N + 7) / 8;
  const int blocks = (int)(want < 8LL * sms ? want : 8LL * sms);
  benes_ct_kernel<SET><<<blocks, 256, 0, st>>>(E, lde, ok, keys, segs);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_gf2_gemm_seg(engine, htt, segs, ct_htt_words(p::n), (p::t * p::m + kGemmRowTile - 1) / kGemmRowTile *
                          kGemmRowTile, E, lde, ct_htt_words(p::n), S3, lds3, (p::t * p::m + 31) / 32, err, st);
  if (e != cudaSuccess) return e;
  ct_check_kernel<SET><<<(unsigned)((N + 127) / 128), 128, 0, st>>>(S3, lds3, S2, lds2, ok, segs);
  return cudaGetLastError();
}

// HTT[r][w] bit b = bit r of HT[32 w + b] (r < t m, 32 w + b < n): the first t syndromes of every code position
// as a (t m) x n GF(2) matrix, rows_pad x kwn words
__global__ void ct_htt_kernel(const uint32_t *__restrict__ HT, int ldh, int n, int tm, int rows_pad, int kwn,
                              uint32_t *__restrict__ HTT) {
  const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= (long long)rows_pad * kwn) return;
  const int r = (int)(item / kwn), w = (int)(item % kwn);
  uint32_t v = 0;
  if (r < tm)
    for (int b = 0; b < 32; b++) {
      const int i = 32 * w + b;
      if (i < n) v |= ((HT[(size_t)i * ldh + (r >> 5)] >> (r & 31)) & 1u) << b;
    }
  HTT[item] = v;
}

cudaError_t launch_ct_htt(const uint32_t *HT, int ldh, int n, int tm, uint32_t *HTT, cudaStream_t st) {
  const int rows_pad = (tm + kGemmRowTile - 1) / kGemmRowTile * kGemmRowTile, kwn = ct_htt_words(n);
  const long long total = (long long)rows_pad * kwn;
  ct_htt_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(HT, ldh, n, tm, rows_pad, kwn, HTT);
  return cudaGetLastError();
}

template <int SET>
cudaError_t launch_dec_tail(const uint32_t *E, int lde, const int *ok, const uint8_t *C, const DecKeys &keys,
                            uint8_t *K, int *rc, const Segs &segs, bool pc, cudaStream_t st) {
  const long long N = seg_rows(segs);
  if (N <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((N + kTailThreads - 1) / kTailThreads);
  if (pc)
    dec_tail_kernel<SET, true><<<blocks, kTailThreads, 0, st>>>(E, lde, ok, C, keys, K, rc, segs);
  else
    dec_tail_kernel<SET, false><<<blocks, kTailThreads, 0, st>>>(E, lde, ok, C, keys, K, rc, segs);
  return cudaGetLastError();
}

#define GMC_INST_DEC(SET)                                                                                       \
  template cudaError_t launch_pack_ct<SET>(const uint8_t *, const Segs &, uint32_t *, int, bool, cudaStream_t);       \
  template cudaError_t launch_dec_bm<SET>(const uint32_t *, int, FieldDev, const Segs &, uint16_t *,             \
                                         cudaStream_t, int, bool);                                               \
  template cudaError_t launch_dec_root<SET>(const uint16_t *, const uint32_t *, int, const DecKeys &, FieldDev,  \
                                            const Segs &, uint32_t *, int, int *, cudaStream_t, int, bool);      \
  template cudaError_t launch_dec_tail<SET>(const uint32_t *, int, const int *, const uint8_t *, const DecKeys &, \
                                            uint8_t *, int *, const Segs &, bool, cudaStream_t);                 \
  template cudaError_t launch_dec_ct_finish<SET>(const DecKeys &, const GemmKeys &, int, const Segs &, uint32_t *, \
                                                 int, const uint32_t *, int, uint32_t *, int, int *, int *,      \
                                                 cudaStream_t);
GMC_INST_DEC(0)
GMC_INST_DEC(1)
GMC_INST_DEC(2)
GMC_INST_DEC(3)
GMC_INST_DEC(4)

}  // namespace gmc
