// Batched key generation on the device, byte-identical to libmceliece's
// keypair (mc:crypto_kem/<set>/vec/kem_keypair.c:20-100) for the same 32-byte
// randombytes draw of each key.
//
// Per key the library walks a seed chain: attempt a expands its seed with
// r = SHAKE256({64} || seed, n/8 + 4q + 2t + 32), the next seed is r's last
// 32 bytes, and the attempt succeeds when
//   (1) f = r[-32-2t:-32] has a minimal polynomial g of degree t (sk_gen.c:29),
//   (2) the 2^m 32-bit values r[n/8 : n/8+4q] are distinct (pk_gen.c:82), and
//   (3) the left mt x mt block A_L of the parity-check matrix
//       [A_L | A_R] built from g and the support is invertible (pk_gen.c:150).
// The key is then pk = T = A_L^-1 A_R (the unique reduced form), the Benes
// control bits of the support permutation, and sk = seed | pivots | g |
// control bits | r[0:n/8].
//
// Seed chains (stream 0): kg_expand, one thread per key and chain link,
// expands 16 links of every key ahead of the rounds into an expansion store
// (more for the rare key that needs them); a chain link costs 251 sequential
// Keccak-f permutations for 8192128, so expanding ahead keeps the chain
// latency off the rounds.
// Device pipeline of one round (each pending key gets k <= 8 attempts, k
// filling 4 x SMs attempts; stream 1):
//   kg_minpoly   one CTA per attempt  powers of f in GF((2^m)^t), Gauss-Jordan
//   kg_support   one CTA per attempt  bitonic sort of (value, index) pairs
//   kg_build     CTAs per attempt     columns of A_L (the rank test's matrix)
//   kg_elim      one CTA per attempt  blocked forward elimination of A_L (rank test)
// and for the first successful attempt of each key (the winner; stream 2,
// overlapping the next round, whose attempt buffers are the other half of a
// double buffer):
//   kg_build + kg_elim on the full mt x n matrix (row order of [I | T])
//   kg_cbits     one CTA per winner   control bits, checked by re-applying them
//   kg_assemble  pk and sk bytes
// Only the rank test runs on the ~70% of attempts whose A_L is singular; the
// full elimination (4-5x the rank test's work for 8192128) runs once per key.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/gmc.h"
#include "device_common.cuh"
#include "engine_internal.h"
#include "host_keys.h"

namespace gmc {

// ---------------------------------------------------------------- constants
// GF((2^m)^t) reduction y^t = sum_k c_k y^pos_k, c_k in {1, z} (z = the field
// element 2): mc:crypto_kem/<set>/vec/gf_2mt_mul.c.
template <int SET> struct ExtPoly;
#define GMC_EXT_POLY(SET, N, MAXPOS, P0, P1, P2, P3, Z0, Z1, Z2, Z3)                                   \
  template <> struct ExtPoly<SET> {                                                                 \
    static constexpr int n = N, maxpos = MAXPOS;                                                    \
    __device__ static constexpr int pos(int i) { return i == 0 ? P0 : i == 1 ? P1 : i == 2 ? P2 : P3; } \
    __device__ static constexpr int z(int i) { return i == 0 ? Z0 : i == 1 ? Z1 : i == 2 ? Z2 : Z3; }   \
  };
GMC_EXT_POLY(0, 3, 3, 3, 1, 0, 0, 0, 0, 1, 0)
GMC_EXT_POLY(1, 4, 10, 10, 9, 6, 0, 0, 0, 0, 0)
GMC_EXT_POLY(2, 4, 7, 7, 2, 1, 0, 0, 0, 0, 0)
GMC_EXT_POLY(3, 2, 8, 8, 0, 0, 0, 0, 0, 0, 0)
GMC_EXT_POLY(4, 4, 7, 7, 2, 1, 0, 0, 0, 0, 0)
#undef GMC_EXT_POLY

template <int SET> struct KG {
  using Q = P<SET>;
  static constexpr int m = Q::m, n = Q::n, t = Q::t, mt = Q::mt, k = Q::k, q = Q::q;
  static constexpr int rlen = Q::e_bytes + 4 * q + 2 * t + 32;    // SHAKE output bytes per attempt
  static constexpr int rblocks = (rlen + 135) / 136;
  static constexpr int dofs = rblocks * 136;                      // the attempt's seed follows its r blocks
  static constexpr int rstride = dofs + 32;                       // per-attempt bytes: r (whole blocks), seed
  static constexpr int rw = (((n + 31) / 32) + 31) / 32 * 32;     // u32 words per full row
  static constexpr int rwl = (((mt + 31) / 32) + 31) / 32 * 32;   // u32 words per A_L row
  static constexpr int gstride = (t + 2) & ~1;                    // u16 per g (t+1 coefficients)
  static constexpr int cond_bytes = (q / 16) * (2 * m - 1);
  static constexpr int pk_row_bytes = (k + 7) / 8;
  static constexpr long long pk_bytes = (long long)mt * pk_row_bytes;
  static constexpr long long sk_bytes = 40 + 2 * t + cond_bytes + n / 8;
  static constexpr int zl = 2 * q - 2;                            // log of 0
  static constexpr int exp_n = 2 * q - 1;
};

// barrier over every thread of the CTA's cluster; release/acquire order the
// global writes before it against the reads after it
__device__ __forceinline__ void kg_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// status bits per attempt
constexpr uint8_t kKgMinpoly = 1, kKgDistinct = 2, kKgRank = 4, kKgAll = 7;

// ---------------------------------------------------------------- expansion
// One link of every listed key's seed chain: thread i takes key = keys[i]
// (or i), expands r = SHAKE256({64} || seed) into slot (a, i) of a block of
// nb keys, stores the seed after r's blocks, and advances the key's chain
// to seed' = r[rlen-32 : rlen].
template <int SET>
__global__ void __launch_bounds__(32) kg_expand_kernel(uint8_t *__restrict__ seedc, const int *__restrict__ keys,
                                                       int nb, int a, uint8_t *__restrict__ out) {
  using C = KG<SET>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int key = keys ? keys[i] : i;
  uint8_t *r = out + ((long long)a * nb + i) * C::rstride;
  uint8_t in[40];
  in[0] = 64;
#pragma unroll
  for (int j = 0; j < 32; j++) in[1 + j] = seedc[32 * key + j];
  in[33] = 0x1F;
#pragma unroll
  for (int j = 34; j < 40; j++) in[j] = 0;
  uint64_t s[25];
#pragma unroll
  for (int j = 0; j < 25; j++) s[j] = 0;
  // absorb {64} || seed || 0x1F, final bit of the 136-byte block
#pragma unroll
  for (int l = 0; l < 5; l++) {
    uint64_t w = 0;
#pragma unroll
    for (int b = 0; b < 8; b++) w |= (uint64_t)in[8 * l + b] << (8 * b);
    s[l] = w;
  }
  s[16] ^= 0x8000000000000000ull;
  uint64_t *o = reinterpret_cast<uint64_t *>(r);
#pragma unroll 1
  for (int b = 0; b < C::rblocks; b++) {
    keccak_f1600(s);
#pragma unroll
    for (int j = 0; j < 17; j++) o[17 * b + j] = s[j];
  }
#pragma unroll
  for (int j = 0; j < 32; j++) {
    r[C::dofs + j] = in[1 + j];
    seedc[32 * key + j] = r[C::rlen - 32 + j];
  }
}

// ---------------------------------------------------------------- minimal polynomial
// CTA per attempt. Columns col[c] = f^c (c <= t) in GF((2^m)^t); solve
// sum_{c<t} g_c f^c = f^t by Gauss-Jordan (the solution is unique when it
// exists, so the pivot order does not change g). mc:crypto_kem/<set>/vec/sk_gen.c:29-75.
constexpr int kMinpolyThreads = 256;
template <int SET> struct MinpolySmem {
  using C = KG<SET>;
  static constexpr int ex = 0;                                   // exp_n u16
  static constexpr int lg = ex + ((C::exp_n + 1) & ~1);          // q u16
  static constexpr int col = lg + C::q;                          // (t+1) * t u16
  static constexpr int la = col + (C::t + 1) * C::t;             // t
  static constexpr int lf = la + C::t;                           // t
  static constexpr int prod = lf + C::t;                         // 2t
  static constexpr int r1 = prod + 2 * C::t;                     // t + 16
  static constexpr int lrow = r1 + C::t + 16;                    // t + 1
  static constexpr int lcoef = lrow + C::t + 2;                  // t
  static constexpr int total_u16 = (lcoef + C::t + 2 + 7) & ~7;  // flags (int) follow, aligned
  static constexpr int bytes = total_u16 * 2 + 16;
};

template <int SET>
__global__ void __launch_bounds__(kMinpolyThreads) kg_minpoly_kernel(const uint8_t *const *__restrict__ rptr, int natt,
                                                                     const uint16_t *__restrict__ gexp,
                                                                     const uint16_t *__restrict__ glog,
                                                                     uint16_t *__restrict__ gout,
                                                                     uint8_t *__restrict__ status) {
  using C = KG<SET>;
  using L = MinpolySmem<SET>;
  using X = ExtPoly<SET>;
  constexpr int T = C::t, q = C::q, ZL = C::zl;
  extern __shared__ __align__(16) uint16_t kgsm_mp[];
  uint16_t *ex = kgsm_mp + L::ex, *lg = kgsm_mp + L::lg, *col = kgsm_mp + L::col, *la = kgsm_mp + L::la,
           *lf = kgsm_mp + L::lf, *prod = kgsm_mp + L::prod, *r1 = kgsm_mp + L::r1, *lrow = kgsm_mp + L::lrow,
           *lcoef = kgsm_mp + L::lcoef;
  int *flags = reinterpret_cast<int *>(kgsm_mp + L::total_u16);
  const int att = blockIdx.x;
  if (att >= natt) return;
  const int tid = threadIdx.x;
  for (int i = tid; i < C::exp_n; i += kMinpolyThreads) ex[i] = gexp[i];
  for (int i = tid; i < q; i += kMinpolyThreads) lg[i] = glog[i];
  const uint8_t *rp = rptr[att] + C::rlen - 32 - 2 * T;
  if (tid < T) {
    const uint16_t f = (uint16_t)((rp[2 * tid] | (rp[2 * tid + 1] << 8)) & (q - 1));
    col[0 * T + tid] = tid == 0 ? 1 : 0;
    col[1 * T + tid] = f;
  }
  if (tid == 0) flags[0] = 0;
  __syncthreads();
  if (tid < T) lf[tid] = lg[col[T + tid]];
  const int log2 = lg[2];
  auto mulz = [&](uint16_t x) -> uint16_t { return ex[min((int)lg[x] + log2, ZL)]; };
  // powers f^c = f^(c-1) * f
  for (int c = 2; c <= T; c++) {
    const uint16_t *prev = col + (c - 1) * T;
    if (tid < T) la[tid] = lg[prev[tid]];
    __syncthreads();
    if (tid < 2 * T - 1) {
      const int lo = max(0, tid - T + 1), hi = min(tid, T - 1);
      uint16_t acc = 0;
      for (int i = lo; i <= hi; i++) acc ^= ex[min((int)la[i] + (int)lf[tid - i], ZL)];
      prod[tid] = acc;
    }
    __syncthreads();
    // fold the high half H (degrees t .. 2t-2) once: R1 = low + sum_k c_k H y^pos_k
    if (tid < T - 1 + X::maxpos) {
      uint16_t v = tid < T ? prod[tid] : 0;
#pragma unroll
      for (int kk = 0; kk < X::n; kk++) {
        const int h = tid - X::pos(kk);
        if (h >= 0 && h <= T - 2) {
          const uint16_t x = prod[T + h];
          v ^= X::z(kk) ? mulz(x) : x;
        }
      }
      r1[tid] = v;
    }
    __syncthreads();
    // fold R1's degrees t .. t+maxpos-2 once more (they land below degree 2 maxpos)
    if (tid < T) {
      uint16_t v = r1[tid];
#pragma unroll
      for (int kk = 0; kk < X::n; kk++) {
        const int h = tid - X::pos(kk);
        if (h >= 0 && h <= X::maxpos - 2) {
          const uint16_t x = r1[T + h];
          v ^= X::z(kk) ? mulz(x) : x;
        }
      }
      col[c * T + tid] = v;
    }
    __syncthreads();
  }
  // Gauss-Jordan on rows r < t of the columns c <= t
  for (int j = 0; j < T; j++) {
    if (tid == 0) {
      int kk = -1;
      if (col[j * T + j] == 0) {
        for (int r = j + 1; r < T; r++)
          if (col[j * T + r]) { kk = r; break; }
        if (kk < 0) flags[0] = 1;
      }
      flags[1] = kk;
    }
    __syncthreads();
    if (flags[0]) break;
    const int kk = flags[1];
    if (kk >= 0)
      for (int c = j + tid; c <= T; c += kMinpolyThreads) col[c * T + j] ^= col[c * T + kk];
    __syncthreads();
    const int lp = lg[col[j * T + j]];
    const int linv = (q - 1 - lp) % (q - 1);
    for (int c = j + tid; c <= T; c += kMinpolyThreads) {
      const uint16_t v = ex[min((int)lg[col[c * T + j]] + linv, ZL)];
      col[c * T + j] = v;
      lrow[c] = lg[v];
    }
    if (tid < T) lcoef[tid] = tid == j ? ZL : lg[col[j * T + tid]];
    __syncthreads();
    const int width = T + 1 - j;
    for (int idx = tid; idx < width * T; idx += kMinpolyThreads) {
      const int c = j + idx / T, r = idx - (idx / T) * T;
      col[c * T + r] ^= ex[min((int)lrow[c] + (int)lcoef[r], ZL)];
    }
    __syncthreads();
  }
  if (flags[0]) return;
  uint16_t *g = gout + (long long)att * C::gstride;
  if (tid < T) g[tid] = col[T * T + tid];
  if (tid == 0) {
    g[T] = 1;
    status[att] |= kKgMinpoly;
  }
}

// ---------------------------------------------------------------- support
// CTA per attempt: sort the 2^m pairs (value_i << 31 | i) (pk_gen.c:82-96),
// reject a repeated value, keep pi_i = the index part of the i-th smallest.
constexpr int kSupportThreads = 1024;
template <int SET>
__global__ void __launch_bounds__(kSupportThreads) kg_support_kernel(const uint8_t *const *__restrict__ rptr, int natt,
                                                                     uint16_t *__restrict__ pi_out,
                                                                     uint8_t *__restrict__ status) {
  using C = KG<SET>;
  constexpr int q = C::q;
  extern __shared__ __align__(16) uint64_t kgsm_sup[];
  const int att = blockIdx.x;
  if (att >= natt || !(status[att] & kKgMinpoly)) return;
  const int tid = threadIdx.x;
  const uint8_t *pv = rptr[att] + C::n / 8;
  for (int i = tid; i < q; i += kSupportThreads) {
    const uint32_t v = (uint32_t)pv[4 * i] | ((uint32_t)pv[4 * i + 1] << 8) | ((uint32_t)pv[4 * i + 2] << 16) |
                       ((uint32_t)pv[4 * i + 3] << 24);
    kgsm_sup[i] = ((uint64_t)v << 31) | (uint64_t)i;
  }
  __syncthreads();
  for (int size = 2; size <= q; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int p = tid; p < q / 2; p += kSupportThreads) {
        const int i = 2 * p - (p & (stride - 1)), j = i + stride;
        const bool up = (i & size) == 0;
        const uint64_t a = kgsm_sup[i], b = kgsm_sup[j];
        if ((a > b) == up) {
          kgsm_sup[i] = b;
          kgsm_sup[j] = a;
        }
      }
      __syncthreads();
    }
  int tie = 0;
  for (int i = tid + 1; i < q; i += kSupportThreads)
    if ((kgsm_sup[i - 1] >> 31) == (kgsm_sup[i] >> 31)) tie = 1;
  tie = __syncthreads_or(tie);
  if (tie) return;
  uint16_t *pi = pi_out + (long long)att * q;
  for (int i = tid; i < q; i += kSupportThreads) pi[i] = (uint16_t)(kgsm_sup[i] & (q - 1));
  if (tid == 0) status[att] |= kKgDistinct;
}

// ---------------------------------------------------------------- matrix
// Block (b, slot): columns 256 b .. 256 b + 255 (one warp per 32-column word)
// of the attempt's parity-check matrix, rows i*m + bit for i < t:
// bit of L_j^i / g(L_j), L_j = bitrev_m(pi_j) (pk_gen.c:98-140). Columns at
// or past n are zero. Words [0, nwords) of each row of stride ld are written.
constexpr int kBuildThreads = 256;
template <int SET> struct BuildSmem {
  using C = KG<SET>;
  static constexpr int ex = 0, lg = ex + ((C::exp_n + 1) & ~1), g = lg + C::q, tile_u16 = g + C::gstride;
  static constexpr int bytes = tile_u16 * 2 + C::mt * 8 * 4;
};
template <int SET>
__global__ void __launch_bounds__(kBuildThreads) kg_build_kernel(const uint16_t *__restrict__ gall,
                                                                 const uint16_t *__restrict__ piall,
                                                                 const int *__restrict__ att_of, const uint8_t *__restrict__ status,
                                                                 uint32_t *__restrict__ mat, int ld, int nwords,
                                                                 const uint16_t *__restrict__ gexp,
                                                                 const uint16_t *__restrict__ glog) {
  using C = KG<SET>;
  using L = BuildSmem<SET>;
  constexpr int q = C::q, T = C::t, M = C::m, ZL = C::zl;
  extern __shared__ __align__(16) uint16_t kgsm_bd[];
  uint16_t *ex = kgsm_bd + L::ex, *lg = kgsm_bd + L::lg, *gs = kgsm_bd + L::g;
  uint32_t *tile = reinterpret_cast<uint32_t *>(kgsm_bd + L::tile_u16);
  const int slot = blockIdx.y;
  const int att = att_of ? att_of[slot] : slot;
  if ((status[att] & (kKgMinpoly | kKgDistinct)) != (kKgMinpoly | kKgDistinct)) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < C::exp_n; i += kBuildThreads) ex[i] = gexp[i];
  for (int i = tid; i < q; i += kBuildThreads) lg[i] = glog[i];
  for (int i = tid; i <= T; i += kBuildThreads) gs[i] = gall[(long long)att * C::gstride + i];
  __syncthreads();
  const int col = (blockIdx.x * 8 + warp) * 32 + lane;
  uint16_t inv = 0;
  int lL = ZL;
  if (col < C::n) {
    const uint16_t p = piall[(long long)att * q + col];
    const uint16_t Lj = (uint16_t)(__brev((uint32_t)p) >> (32 - M));
    lL = lg[Lj];
    uint16_t v = gs[T];
    for (int i = T - 1; i >= 0; i--) v = ex[min((int)lg[v] + lL, ZL)] ^ gs[i];
    const int lv = lg[v];
    inv = lv < q - 1 ? ex[q - 1 - lv] : 0;
  }
  for (int i = 0; i < T; i++) {
#pragma unroll
    for (int b = 0; b < M; b++) {
      const uint32_t bal = __ballot_sync(0xffffffffu, (inv >> b) & 1);
      if (lane == 0) tile[(i * M + b) * 8 + warp] = bal;
    }
    inv = ex[min((int)lg[inv] + lL, ZL)];
  }
  __syncthreads();
  uint32_t *dst = mat + (long long)slot * C::mt * ld;
  for (int idx = tid; idx < C::mt * 8; idx += kBuildThreads) {
    const int row = idx >> 3, w = blockIdx.x * 8 + (idx & 7);
    if (w < nwords) dst[(long long)row * ld + w] = tile[idx];
  }
}

// ---------------------------------------------------------------- elimination
// CTA per matrix (mt rows of ld words; words [0, nwords) take part). Blocked
// Gauss-Jordan with 32-column panels: per panel the CTA finds pivot rows for
// the panel's columns (forward elimination on the panel word only), inverts
// their 32 x 32 panel block B, replaces the pivot rows P by P' = B^-1 P and
// clears the panel from every other row r with r ^= c_r P', c_r = r's panel
// word. The last update is a Four-Russians product: per 32-word group four
// 256-entry tables of XOR combinations of P' rows (8 rows each) in shared
// memory, four lookups per row word. Singular A_L: no pivot for some column,
// the attempt fails (pk_gen.c:150-156 rejects the same matrices).
// Table width: TB = 8 (four 256-entry tables per 32-word group, 128 KB,
// 1024 threads, one CTA per SM) or TB = 4 (eight 16-entry tables, 16 KB,
// 512 threads, three CTAs per SM, so one CTA's serial panel steps overlap the
// others' updates).
template <int TB> struct ElimCfg {
  static constexpr int nt = TB == 8 ? 1024 : 512, ntab = 32 / TB, nent = 1 << TB, minb = TB == 8 ? 1 : 3;
};
constexpr int kElimRows = 4;      // rows in flight per warp in the panel update
constexpr int kElimCluster = 4;   // CTAs per matrix in the full elimination
// measured: 4-bit tables (more resident CTAs) pay off only for 348864, whose
// A_L rows are one 24-word group; the larger sets are instruction-bound
template <int SET> constexpr int kg_table_bits() { return SET == 0 ? 4 : 8; }
template <int SET, int TB> struct ElimSmem {
  using C = KG<SET>;
  static constexpr int tab = 0;                                        // ntab * nent * 32 u32
  static constexpr int pw = tab + ElimCfg<TB>::ntab * ElimCfg<TB>::nent * 32;  // 32 * 32 u32
  static constexpr int colw = pw + 32 * 32;           // mt u32
  static constexpr int wk = colw + C::mt;             // mt u32
  static constexpr int binv = wk + C::mt;             // 32 u32
  static constexpr int misc = binv + 32;              // 4 ints: candidate, failure, search mode; 32: pivot columns
  static constexpr int rowid_u32 = misc + 36;         // mt u16
  static constexpr int bytes = rowid_u32 * 4 + C::mt * 2 + 16;
};
template <int SET, int TB>
__global__ void __launch_bounds__(ElimCfg<TB>::nt, ElimCfg<TB>::minb) kg_elim_kernel(uint32_t *__restrict__ mat, int ld, int nwords,
                                                                  const int *__restrict__ att_of,
                                                                  uint8_t *__restrict__ status, int need, int set_bit,
                                                                  int forward, int cl, uint16_t *__restrict__ rowid_out,
                                                                  int semi, uint8_t *__restrict__ clist_out,
                                                                  uint16_t *__restrict__ pi_all) {
  using C = KG<SET>;
  using L = ElimSmem<SET, TB>;
  constexpr int MT = C::mt, NT = ElimCfg<TB>::nt;
  extern __shared__ __align__(16) uint32_t kgsm_el[];
  uint32_t *tab = kgsm_el + L::tab, *Pw = kgsm_el + L::pw, *colw = kgsm_el + L::colw, *wk = kgsm_el + L::wk,
           *binv = kgsm_el + L::binv;
  int *misc = reinterpret_cast<int *>(kgsm_el + L::misc);
  uint16_t *rowid = reinterpret_cast<uint16_t *>(kgsm_el + L::rowid_u32);
  // cl CTAs (a cluster) per matrix: each repeats the panel factorization
  // (same inputs, same decisions) and updates the 32-word groups g = crank mod cl
  const int slot = blockIdx.x / cl, crank = blockIdx.x - slot * cl;
  const int att = att_of ? att_of[slot] : slot;
  if ((status[att] & need) != need) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint32_t *A = mat + (long long)slot * MT * ld;
  for (int i = tid; i < MT; i += NT) rowid[i] = (uint16_t)i;
  const int ngroups = nwords / 32;
  // Panels of up to 32 columns from column (= pivot row position) base. The
  // semi-systematic form ("f" variants) ends the regular panels at R = mt - 32
  // and takes the last 32 pivots as the leftmost independent columns of the
  // 64-column window from R (mc:crypto_kem/348864f/vec/pk_gen.c, mov_columns).
  const int R = semi ? MT - 32 : MT;
  int *clist = misc + 4;  // the window's pivot columns (offsets from R)
  for (int base = 0; base < MT;) {
    const bool fpanel = semi && base == R;
    const int np = fpanel ? 32 : min(32, (base < R ? R : MT) - base);
    const uint32_t npmask = np == 32 ? 0xffffffffu : ((1u << np) - 1);
    const int pw0 = base >> 5, psh = base & 31;
    // 32 bits of a row from column base + 32 h (a funnel of two words when base is unaligned)
    auto bits32 = [&](const uint32_t *row, int h) -> uint32_t {
      uint32_t v = row[pw0 + h] >> psh;
      if (psh) v |= row[pw0 + h + 1] << (32 - psh);
      return v;
    };
    if (fpanel) {
      // the 32 remaining rows' window (warp 0, lane = row): leftmost pivot columns
      if (warp == 0) {
        const uint32_t *row = A + (long long)rowid[base + lane] * ld;
        uint64_t w = (uint64_t)bits32(row, 0) | ((uint64_t)bits32(row, 1) << 32);
        int mode = 0;
        for (int i = 0; i < 32; i++) {
          const uint64_t live = lane >= i ? w : 0;
          const uint32_t lo = __reduce_or_sync(0xffffffffu, (uint32_t)live);
          const uint32_t hi = __reduce_or_sync(0xffffffffu, (uint32_t)(live >> 32));
          if (!lo && !hi) {
            mode = 2;  // rank below 32: the library rejects the attempt
            break;
          }
          const int sidx = lo ? __ffs(lo) - 1 : 32 + __ffs(hi) - 1;
          if (lane == 0) clist[i] = sidx;
          const uint32_t bal = __ballot_sync(0xffffffffu, lane >= i && ((w >> sidx) & 1));
          const int pl = __ffs(bal) - 1;
          const uint64_t wp = __shfl_sync(0xffffffffu, w, pl), wi = __shfl_sync(0xffffffffu, w, i);
          if (lane == i) w = wp;
          else if (lane == pl) w = wi;
          if (lane > i && ((w >> sidx) & 1)) w ^= wp;
        }
        if (lane == 0) misc[2] = mode;
      }
      __syncthreads();
      if (misc[2] == 2) return;
      // every row's coefficients: its bits at the 32 pivot columns
      for (int pos = tid; pos < MT; pos += NT) {
        const uint32_t *row = A + (long long)rowid[pos] * ld;
        const uint64_t w = (uint64_t)bits32(row, 0) | ((uint64_t)bits32(row, 1) << 32);
        uint32_t v = 0;
#pragma unroll 8
        for (int j = 0; j < 32; j++) v |= (uint32_t)((w >> clist[j]) & 1) << j;
        colw[pos] = v;
      }
      __syncthreads();
    } else {
    for (int pos = tid; pos < MT; pos += NT) colw[pos] = bits32(A + (long long)rowid[pos] * ld, 0);
    __syncthreads();
    // Pivot search, first in the window of positions base .. base+63 (warp 0,
    // slots in registers: forward elimination on the panel word, slot tags
    // follow the swaps). A window without a pivot for some column either
    // covers every remaining row (A_L is singular) or falls back to the
    // CTA-wide search below.
    if (warp == 0) {
      const bool in0 = base + lane < MT, in1 = base + 32 + lane < MT;
      uint32_t w0 = in0 ? colw[base + lane] : 0, w1 = in1 ? colw[base + 32 + lane] : 0;
      int t0 = lane, t1 = 32 + lane;
      int mode = 0;
      for (int j = 0; j < np; j++) {
        const uint32_t bit = 1u << j;
        const uint32_t b0 = __ballot_sync(0xffffffffu, lane >= j && (w0 & bit));
        const uint32_t b1 = __ballot_sync(0xffffffffu, (w1 & bit) != 0);
        if (!b0 && !b1) {
          mode = base + 64 >= MT ? 2 : 1;
          break;
        }
        const bool lo = b0 != 0;
        const int pl = __ffs(lo ? b0 : b1) - 1;
        const uint32_t wj = __shfl_sync(0xffffffffu, w0, j), tj = __shfl_sync(0xffffffffu, t0, j);
        const uint32_t wp = __shfl_sync(0xffffffffu, lo ? w0 : w1, pl);
        const int tp = __shfl_sync(0xffffffffu, lo ? t0 : t1, pl);
        if (lane == pl) {
          if (lo) { w0 = wj; t0 = tj; }
          else { w1 = wj; t1 = tj; }
        }
        if (lane == j) { w0 = wp; t0 = tp; }
        if (lane > j && (w0 & bit)) w0 ^= wp;
        if (w1 & bit) w1 ^= wp;
      }
      if (mode == 0) {
        // commit the window's permutation: position base + slot <- base + tag
        const uint16_t r0 = in0 ? rowid[base + t0] : 0, r1 = in1 ? rowid[base + t1] : 0;
        const uint32_t c0 = in0 ? colw[base + t0] : 0, c1 = in1 ? colw[base + t1] : 0;
        __syncwarp();
        if (in0) { rowid[base + lane] = r0; colw[base + lane] = c0; }
        if (in1) { rowid[base + 32 + lane] = r1; colw[base + 32 + lane] = c1; }
      }
      if (lane == 0) {
        misc[0] = INT_MAX;
        misc[1] = 0;
        misc[2] = mode;
      }
    }
    __syncthreads();
    if (misc[2] == 2) return;  // no pivot: A_L is singular
    if (misc[2] == 1) {
      // CTA-wide search: forward elimination of the panel word over all rows
      {
        int cand = INT_MAX;
        for (int pos = base + tid; pos < MT; pos += NT) {
          const uint32_t v = colw[pos];
          wk[pos] = v;
          if (v & 1) cand = min(cand, pos);
        }
        cand = (int)__reduce_min_sync(0xffffffffu, (unsigned)cand);
        if (lane == 0 && cand != INT_MAX) atomicMin(&misc[0], cand);
      }
      __syncthreads();
      for (int j = 0; j < np; j++) {
        if (tid == 0) {
          const int piv = misc[0];
          misc[0] = INT_MAX;
          if (piv == INT_MAX) {
            misc[1] = 1;
          } else if (piv != base + j) {
            const int at = base + j;
            uint32_t x0 = wk[piv]; wk[piv] = wk[at]; wk[at] = x0;
            x0 = colw[piv]; colw[piv] = colw[at]; colw[at] = x0;
            const uint16_t r0 = rowid[piv]; rowid[piv] = rowid[at]; rowid[at] = r0;
          }
        }
        __syncthreads();
        if (misc[1]) return;  // no pivot: A_L is singular
        const uint32_t pwd = wk[base + j], bit = 1u << j;
        int cand = INT_MAX;
        for (int pos = base + j + 1 + tid; pos < MT; pos += NT) {
          uint32_t x = wk[pos];
          if (x & bit) {
            x ^= pwd;
            wk[pos] = x;
          }
          if (j + 1 < np && ((x >> (j + 1)) & 1)) cand = min(cand, pos);
        }
        cand = (int)__reduce_min_sync(0xffffffffu, (unsigned)cand);
        if (lane == 0 && cand != INT_MAX) atomicMin(&misc[0], cand);
        __syncthreads();
      }
    }
    }  // regular panel
    // B^-1 for the pivot rows' original panel words (warp 0, lane = row)
    if (warp == 0) {
      uint32_t b = lane < np ? (colw[base + lane] & npmask) : 0;
      uint32_t e = lane < np ? (1u << lane) : 0;
      for (int i = 0; i < np; i++) {
        const uint32_t bal = __ballot_sync(0xffffffffu, lane >= i && lane < np && ((b >> i) & 1));
        const int pl = __ffs(bal) - 1;  // exists: the pivot rows are independent on the panel
        const uint32_t bp = __shfl_sync(0xffffffffu, b, pl), ep = __shfl_sync(0xffffffffu, e, pl);
        const uint32_t bi = __shfl_sync(0xffffffffu, b, i), ei = __shfl_sync(0xffffffffu, e, i);
        if (lane == i) { b = bp; e = ep; }
        else if (lane == pl) { b = bi; e = ei; }
        if (lane != i && ((b >> i) & 1)) {
          b ^= bp;
          e ^= ep;
        }
      }
      binv[lane] = e;
    }
    // every CTA of the cluster has read the panel words before any updates them
    if (cl > 1) kg_cluster_sync();
    else __syncthreads();
    for (int g = (pw0 >> 5) + ((crank - (pw0 >> 5)) % cl + cl) % cl; g < ngroups; g += cl) {
      const int w0 = 32 * g;
      for (int i = tid; i < 1024; i += NT) {
        const int b = i >> 5;
        Pw[i] = b < np ? A[(long long)rowid[base + b] * ld + w0 + lane] : 0;
      }
      __syncthreads();
      uint32_t v[1024 / NT];
#pragma unroll
      for (int u = 0; u < 1024 / NT; u++) {
        uint32_t e = binv[(tid + u * NT) >> 5], acc = 0;
        while (e) {
          const int b = __ffs(e) - 1;
          e &= e - 1;
          acc ^= Pw[b * 32 + lane];
        }
        v[u] = acc;
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < 1024 / NT; u++) {
        const int j = (tid + u * NT) >> 5;
        Pw[tid + u * NT] = v[u];
        if (j < np) A[(long long)rowid[base + j] * ld + w0 + lane] = v[u];
      }
      __syncthreads();
      if constexpr (TB == 8) {
        // four 256-entry tables: thread (kq, vhi, lane) writes entries vhi*32 .. vhi*32+31 of table kq
        const int kq = tid >> 8, vhi = (tid >> 5) & 7;
        const uint32_t *pr = Pw + 8 * kq * 32 + lane;
        uint32_t h = 0;
        if (vhi & 1) h ^= pr[5 * 32];
        if (vhi & 2) h ^= pr[6 * 32];
        if (vhi & 4) h ^= pr[7 * 32];
        const uint32_t p0 = pr[0], p1 = pr[32], p2 = pr[64], p3 = pr[96], p4 = pr[128];
        uint32_t *tp = tab + ((kq * 256 + vhi * 32) * 32) + lane;
        uint32_t r[32];
        r[0] = h;
#pragma unroll
        for (int vl = 1; vl < 32; vl++) {
          const int low = __ffs(vl) - 1;
          const uint32_t pb = low == 0 ? p0 : low == 1 ? p1 : low == 2 ? p2 : low == 3 ? p3 : p4;
          r[vl] = r[vl & (vl - 1)] ^ pb;
        }
#pragma unroll
        for (int vl = 0; vl < 32; vl++) tp[vl * 32] = r[vl];
      } else {
        // eight 16-entry tables: thread (kq, half, lane) writes entries half*8 .. half*8+7 of table kq
        const int kq = tid >> 6, half = (tid >> 5) & 1;
        const uint32_t *pr = Pw + 4 * kq * 32 + lane;
        const uint32_t p0 = pr[0], p1 = pr[32], p2 = pr[64], h = half ? pr[96] : 0;
        uint32_t *tp = tab + ((kq * 16 + half * 8) * 32) + lane;
        tp[0] = h;
        tp[32] = h ^ p0;
        tp[64] = h ^ p1;
        tp[96] = h ^ p1 ^ p0;
        tp[128] = h ^ p2;
        tp[160] = h ^ p2 ^ p0;
        tp[192] = h ^ p2 ^ p1;
        tp[224] = h ^ p2 ^ p1 ^ p0;
      }
      __syncthreads();
      constexpr int NW = NT / 32;
      for (int pos0 = (forward ? base + np : 0) + warp; pos0 < MT; pos0 += kElimRows * NW) {
        uint32_t x[kElimRows], c[kElimRows];
        uint32_t *ad[kElimRows];
#pragma unroll
        for (int u = 0; u < kElimRows; u++) {
          const int pos = pos0 + NW * u;
          const bool live = pos < MT && (unsigned)(pos - base) >= (unsigned)np;
          c[u] = live ? (colw[pos] & npmask) : 0;
          ad[u] = A + (long long)rowid[live ? pos : 0] * ld + w0 + lane;
          x[u] = c[u] ? *ad[u] : 0;
        }
#pragma unroll
        for (int u = 0; u < kElimRows; u++) {
          if (!c[u]) continue;
          const uint32_t cc = c[u];
          if constexpr (TB == 8) {
            x[u] ^= tab[((cc & 255) << 5) + lane] ^ tab[((256 + ((cc >> 8) & 255)) << 5) + lane] ^
                    tab[((512 + ((cc >> 16) & 255)) << 5) + lane] ^ tab[((768 + (cc >> 24)) << 5) + lane];
          } else {
#pragma unroll
            for (int kq = 0; kq < 8; kq++) x[u] ^= tab[((kq * 16 + ((cc >> (4 * kq)) & 15)) << 5) + lane];
          }
          *ad[u] = x[u];
        }
      }
      __syncthreads();
    }
    if (cl > 1) kg_cluster_sync();  // the next panel word is final in every row
    base += np;
  }
  if (crank) return;
  if (rowid_out)
    for (int i = tid; i < MT; i += NT) rowid_out[(long long)slot * MT + i] = rowid[i];
  if (semi && tid == 0) {
    if (clist_out)
      for (int j = 0; j < 32; j++) clist_out[(long long)slot * 32 + j] = (uint8_t)clist[j];
    // the support follows the library's column swaps: pi[R + j] <-> pi[R + c_j], j = 0..31 in turn
    if (pi_all) {
      uint16_t *pi = pi_all + (long long)att * C::q;
      for (int j = 0; j < 32; j++) {
        const uint16_t x = pi[R + j];
        pi[R + j] = pi[R + clist[j]];
        pi[R + clist[j]] = x;
      }
    }
  }
  if (tid == 0) status[att] |= (uint8_t)set_bit;
}

// ---------------------------------------------------------------- control bits
// CTA per winner. The library's recursion (controlbits.c:29-150) processes a
// permutation of 2^w entries and recurses into
// two halves with doubled bit stride; here every depth d runs all 2^d
// sub-permutations at once, each a segment of 2^(w-d) entries. Segment s at
// depth d writes layer d and layer 2w-2-d at bits offset_s + 2^d j,
// offset_s = bitrev_d(s).
// Every sort of the recursion orders packed words whose key field (bits 16+,
// or 20+ in one step) is a permutation of the segment's local indices: the
// sort's output at index i is the word whose key is i, so each sort is the
// scatter out[key] = word (one pass, no comparisons). The bits are checked by
// applying the 2w-1 layers to the identity.
constexpr int kCbitsThreads = 1024;
template <int SET> struct CbitsSmem {
  using C = KG<SET>;
  static constexpr int a = 0, b = a + C::q, t = b + C::q, cb = t + C::q, pi_u32 = cb + C::cond_bytes / 4;
  static constexpr int bytes = pi_u32 * 4 + C::q * 2 + 16;
};

template <int SET>
__global__ void __launch_bounds__(kCbitsThreads) kg_cbits_kernel(const uint16_t *__restrict__ piall,
                                                                 const int *__restrict__ att_of,
                                                                 const int *__restrict__ out_of, int nwin,
                                                                 uint8_t *__restrict__ cond_out,
                                                                 uint8_t *__restrict__ cb_ok) {
  using C = KG<SET>;
  using L = CbitsSmem<SET>;
  constexpr int q = C::q, W = C::m, H = q / 2;
  extern __shared__ __align__(16) uint32_t kgsm_cb[];
  uint32_t *A = kgsm_cb + L::a, *B = kgsm_cb + L::b, *T = kgsm_cb + L::t, *CB = kgsm_cb + L::cb;
  uint16_t *PI = reinterpret_cast<uint16_t *>(kgsm_cb + L::pi_u32);
  const int w = blockIdx.x;
  if (w >= nwin) return;
  const int tid = threadIdx.x;
  const uint16_t *pi0 = piall + (long long)att_of[w] * q;
  for (int i = tid; i < q; i += kCbitsThreads) PI[i] = pi0[i];
  for (int i = tid; i < C::cond_bytes / 4; i += kCbitsThreads) CB[i] = 0;
  __syncthreads();
  auto setbit = [&](int bit) { atomicOr(&CB[bit >> 5], 1u << (bit & 31)); };
  for (int d = 0; d < W; d++) {
    const int ww = W - d, nn = 1 << ww;
    auto offs = [&](int s) { return d == 0 ? 0 : (int)(__brev((uint32_t)s) >> (32 - d)); };
    // sort of arr by its key field (a permutation of each segment's indices)
    auto scatter = [&](uint32_t *&arr, int shift) {
      __syncthreads();
      for (int X = tid; X < q; X += kCbitsThreads) {
        const uint32_t v = arr[X];
        T[(X & ~(nn - 1)) + ((v >> shift) & (nn - 1))] = v;
      }
      __syncthreads();
      uint32_t *t = arr;
      arr = T;
      T = t;
    };
    if (ww == 1) {
      for (int s = tid; s < H; s += kCbitsThreads)
        if (PI[2 * s] & 1) setbit((W - 1) * H + offs(s));
      break;
    }
    for (int X = tid; X < q; X += kCbitsThreads) A[X] = ((uint32_t)(PI[X] ^ 1) << 16) | (uint32_t)PI[X ^ 1];
    scatter(A, 16);
    for (int X = tid; X < q; X += kCbitsThreads) {
      const uint32_t x = (uint32_t)(X & (nn - 1)), a = A[X], px = a & 0xffff;
      B[X] = (px << 16) | min(px, x);
      A[X] = (a << 16) | x;
    }
    scatter(A, 16);
    for (int X = tid; X < q; X += kCbitsThreads) A[X] = (A[X] << 16) + (B[X] >> 16);
    scatter(A, 16);
    if (ww <= 10) {
      for (int X = tid; X < q; X += kCbitsThreads) B[X] = ((A[X] & 0xffff) << 10) | (B[X] & 0x3ff);
      for (int i = 1; i < ww - 1; i++) {
        for (int X = tid; X < q; X += kCbitsThreads) A[X] = ((B[X] & ~0x3ffu) << 6) | (uint32_t)(X & (nn - 1));
        scatter(A, 16);
        for (int X = tid; X < q; X += kCbitsThreads) A[X] = (A[X] << 20) | B[X];
        scatter(A, 20);
        for (int X = tid; X < q; X += kCbitsThreads) {
          const uint32_t ppcp = A[X] & 0xfffff, ppc = (A[X] & 0xffc00) | (B[X] & 0x3ff);
          B[X] = min(ppc, ppcp);
        }
      }
      for (int X = tid; X < q; X += kCbitsThreads) B[X] &= 0x3ff;
    } else {
      for (int X = tid; X < q; X += kCbitsThreads) B[X] = (A[X] << 16) | (B[X] & 0xffff);
      for (int i = 1; i < ww - 1; i++) {
        for (int X = tid; X < q; X += kCbitsThreads) A[X] = (B[X] & ~0xffffu) | (uint32_t)(X & (nn - 1));
        scatter(A, 16);
        for (int X = tid; X < q; X += kCbitsThreads) A[X] = (A[X] << 16) | (B[X] & 0xffff);
        if (i < ww - 2) {
          for (int X = tid; X < q; X += kCbitsThreads) B[X] = (A[X] & ~0xffffu) | (B[X] >> 16);
          scatter(B, 16);
          for (int X = tid; X < q; X += kCbitsThreads) B[X] = (B[X] << 16) | (A[X] & 0xffff);
        }
        scatter(A, 16);
        for (int X = tid; X < q; X += kCbitsThreads) {
          const uint32_t cp = (B[X] & ~0xffffu) | (A[X] & 0xffff);
          B[X] = min(B[X], cp);
        }
      }
      for (int X = tid; X < q; X += kCbitsThreads) B[X] &= 0xffff;
    }
    for (int X = tid; X < q; X += kCbitsThreads) A[X] = ((uint32_t)PI[X] << 16) + (uint32_t)(X & (nn - 1));
    scatter(A, 16);
    for (int pr = tid; pr < H; pr += kCbitsThreads) {
      const int X = 2 * pr, z = X & (nn - 1), s = X >> ww;
      const uint32_t fj = B[X] & 1, Fz = (uint32_t)z + fj, Fz1 = Fz ^ 1;
      if (fj) setbit(d * H + offs(s) + ((z >> 1) << d));
      B[X] = (A[X] << 16) | Fz;
      B[X + 1] = (A[X + 1] << 16) | Fz1;
    }
    scatter(B, 16);
    for (int pr = tid; pr < H; pr += kCbitsThreads) {
      const int X = 2 * pr, y = X & (nn - 1), s = X >> ww;
      const uint32_t lk = B[X] & 1, Ly = (uint32_t)y + lk, Ly1 = Ly ^ 1;
      if (lk) setbit((2 * W - 2 - d) * H + offs(s) + ((y >> 1) << d));
      A[X] = (Ly << 16) | (B[X] & 0xffff);
      A[X + 1] = (Ly1 << 16) | (B[X + 1] & 0xffff);
    }
    scatter(A, 16);
    for (int pr = tid; pr < H; pr += kCbitsThreads) {
      const int X = 2 * pr, base = X & ~(nn - 1), j = (X & (nn - 1)) >> 1;
      PI[base + j] = (uint16_t)((A[X] & 0xffff) >> 1);
      PI[base + nn / 2 + j] = (uint16_t)((A[X + 1] & 0xffff) >> 1);
    }
    __syncthreads();
  }
  __syncthreads();
  // check: the layers applied to the identity give pi
  for (int i = tid; i < q; i += kCbitsThreads) A[i] = (uint32_t)i;
  __syncthreads();
  for (int l = 0; l < 2 * W - 1; l++) {
    const int s = l < W ? l : 2 * W - 2 - l, stride = 1 << s;
    for (int idx = tid; idx < H; idx += kCbitsThreads) {
      const int bit = l * H + idx;
      if ((CB[bit >> 5] >> (bit & 31)) & 1) {
        const int i0 = (idx >> s) * 2 * stride + (idx & (stride - 1)), i1 = i0 + stride;
        const uint32_t t0 = A[i0];
        A[i0] = A[i1];
        A[i1] = t0;
      }
    }
    __syncthreads();
  }
  int bad = 0;
  for (int i = tid; i < q; i += kCbitsThreads) bad |= A[i] != (uint32_t)pi0[i];
  bad = __syncthreads_or(bad);
  uint32_t *co = reinterpret_cast<uint32_t *>(cond_out + (long long)w * C::cond_bytes);
  for (int i = tid; i < C::cond_bytes / 4; i += kCbitsThreads) co[i] = CB[i];
  if (tid == 0) cb_ok[out_of[w]] = bad ? 0 : 1;
}

// ---------------------------------------------------------------- assembly
// pk row i = bits [mt, n) of the reduced row at position i; sk = seed |
// ff ff ff ff 00 00 00 00 | g_0..g_{t-1} (LE u16) | control bits | r[0:n/8].
template <int SET>
__global__ void kg_assemble_kernel(const int *__restrict__ att_of, const int *__restrict__ out_of, int nwin,
                                   const uint8_t *const *__restrict__ rptr, const uint16_t *__restrict__ gall,
                                   const uint8_t *__restrict__ cond, const uint32_t *__restrict__ matF,
                                   const uint16_t *__restrict__ rowid, const uint8_t *__restrict__ clist,
                                   uint8_t *__restrict__ pk_out, uint8_t *__restrict__ sk_out) {
  using C = KG<SET>;
  constexpr int R = C::mt - 32;
  __shared__ uint8_t src_of[64];  // semi-systematic form: original column offset (from R) at each window position
  __shared__ uint64_t pivots;
  const int w = blockIdx.y;
  if (w >= nwin) return;
  const int att = att_of[w];
  if (threadIdx.x == 0) {
    pivots = 0xFFFFFFFFull;
    if (clist) {
      // the library's swaps, positions R+j and R+c_j for j = 0..31 in turn
      for (int j = 0; j < 64; j++) src_of[j] = (uint8_t)j;
      pivots = 0;
      for (int j = 0; j < 32; j++) {
        const int c = clist[(long long)w * 32 + j];
        const uint8_t x = src_of[j];
        src_of[j] = src_of[c];
        src_of[c] = x;
        pivots |= 1ull << c;
      }
    }
  }
  __syncthreads();
  const long long pkb = C::pk_bytes, skb = C::sk_bytes;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < pkb + skb; i += stride) {
    if (i < pkb) {
      const int row = (int)(i / C::pk_row_bytes), byte = (int)(i - (long long)row * C::pk_row_bytes);
      const uint32_t *src = matF + ((long long)w * C::mt + rowid[(long long)w * C::mt + row]) * C::rw;
      const int bp = C::mt + 8 * byte, wd = bp >> 5, sh = bp & 31;
      uint32_t v;
      if (clist && bp < R + 64) {
        v = 0;
        for (int u = 0; u < 8; u++) {
          const int q = bp + u;
          const int col = q < R + 64 ? R + src_of[q - R] : q;
          if (q < C::n) v |= ((src[col >> 5] >> (col & 31)) & 1u) << u;
        }
      } else {
        v = src[wd] >> sh;
        if (sh > 24) v |= src[wd + 1] << (32 - sh);
      }
      pk_out[(long long)out_of[w] * pkb + i] = (uint8_t)v;
    } else {
      const int o = (int)(i - pkb);
      uint8_t v;
      if (o < 32) v = rptr[att][C::dofs + o];
      else if (o < 40) v = (uint8_t)(pivots >> (8 * (o - 32)));
      else if (o < 40 + 2 * C::t) {
        const uint16_t gv = gall[(long long)att * C::gstride + ((o - 40) >> 1)];
        v = (uint8_t)(((o - 40) & 1) ? gv >> 8 : gv);
      } else if (o < 40 + 2 * C::t + C::cond_bytes) v = cond[(long long)w * C::cond_bytes + (o - 40 - 2 * C::t)];
      else v = rptr[att][o - 40 - 2 * C::t - C::cond_bytes];
      sk_out[(long long)out_of[w] * skb + o] = v;
    }
  }
}

// ---------------------------------------------------------------- host side
namespace {
int kg_fail(int code, const std::string &msg) {
  set_last_error(msg.c_str());
  return code;
}
#define KG_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess) {                                                             \
      rc = kg_fail(GMC_ECUDA, std::string(#call) + ": " + cudaGetErrorString(_e));       \
      goto done;                                                                         \
    }                                                                                    \
  } while (0)

template <typename F>
cudaError_t smem_attr(F *fn, int bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int SET>
cudaError_t kg_attrs() {
  static cudaError_t once = [] {
    cudaError_t e = smem_attr(kg_minpoly_kernel<SET>, MinpolySmem<SET>::bytes);
    if (e == cudaSuccess) e = smem_attr(kg_support_kernel<SET>, KG<SET>::q * 8);
    if (e == cudaSuccess) e = smem_attr(kg_build_kernel<SET>, BuildSmem<SET>::bytes);
    if (e == cudaSuccess) e = smem_attr(kg_elim_kernel<SET, kg_table_bits<SET>()>, ElimSmem<SET, kg_table_bits<SET>()>::bytes);
    if (e == cudaSuccess) e = smem_attr(kg_elim_kernel<SET, kg_table_bits<SET>()>, ElimSmem<SET, kg_table_bits<SET>()>::bytes);
    if (e == cudaSuccess) e = smem_attr(kg_cbits_kernel<SET>, CbitsSmem<SET>::bytes);
    return e;
  }();
  return once;
}

template <typename T>
cudaError_t dalloc(T **p, size_t count, cudaStream_t st) {
  return cudaMallocAsync(reinterpret_cast<void **>(p), std::max<size_t>(count, 1) * sizeof(T), st);
}

constexpr long long kMaxAttemptsPerKey = 100000;
constexpr int kMaxSpeculation = 8;        // attempts per key and round
constexpr int kExpandBlock = 16;          // twice the minimum chain links per key of an extension block
constexpr long long kChunkBytes = 2ll << 30;  // device-side pk + sk staging per chunk of keys

// Round state, double-buffered: the winners of round r (stream 2) read round
// r's buffers while round r+1 (stream 1) fills the others.
struct KgRound {
  uint8_t *status = nullptr;
  uint16_t *g = nullptr, *pi = nullptr;
  uint32_t *matL = nullptr;
  const uint8_t **rptr = nullptr;                       // per attempt: its r in the expansion store
  int *win = nullptr;                                   // [2][wcap]: attempt, output slot
  const uint8_t **h_rptr = nullptr;                     // pinned
  uint8_t *h_status = nullptr;
  int *h_win = nullptr;
  cudaEvent_t ranked = nullptr, done = nullptr;
};

// Expansion store block: kExpandBlock chained attempts for each of nb keys,
// expanded on stream 0 ahead of the rounds; attempt a of the block's i-th key
// at base + (a * nb + i) * rstride.
struct KgBlock {
  uint8_t *base = nullptr;
  int *keys = nullptr;    // device list (null: keys 0..nb-1)
  int *h_keys = nullptr;  // pinned source of the list
  int nb = 0;
  int seq0 = 0;         // launch sequence number of the block's first link
  int a0 = 0, nlinks = 0;  // attempts a0 .. a0 + nlinks - 1 of each of its keys
  std::vector<int> slot;  // key -> index in the block, -1 if absent
};

template <int SET>
int keypair_batch(uint8_t *pk, uint8_t *sk, const uint8_t *seeds, long long nkeys, bool semi, cudaStream_t s0,
                  cudaStream_t s1, cudaStream_t s2) {
  using C = KG<SET>;
  int rc = GMC_OK;
  FieldDev fd{};
  int dev = 0, sms = 0, cap = 0, wcap = 0;
  long long kc = 0;
  KgRound R[2];
  std::vector<KgBlock> blocks;
  std::vector<cudaEvent_t> links;  // one per expansion launch, in stream-0 order
  std::vector<std::vector<int>> kblocks;  // per key: its store blocks, in chain order
  uint8_t *d_seedc = nullptr;
  uint32_t *d_matF = nullptr;
  uint16_t *d_rowid = nullptr;
  uint8_t *d_cond = nullptr, *d_cbok = nullptr, *d_pk = nullptr, *d_sk = nullptr, *d_clist = nullptr;
  std::vector<long long> pending, next;
  std::vector<int> na;
  std::vector<uint8_t> h_cbok;
  // GMC_KG_TRACE=1: one stderr line per round (host clock, ms since the call)
  static const bool trace = getenv("GMC_KG_TRACE") && getenv("GMC_KG_TRACE")[0] == '1';
  const auto t_start = std::chrono::steady_clock::now();
  auto ms_now = [&] { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count(); };
  if (field_tables(SET, &fd) != GMC_OK) return GMC_ECUDA;
  KG_CUDA(cudaGetDevice(&dev));
  KG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  KG_CUDA(kg_attrs<SET>());
  cap = 4 * sms;
  kc = std::max<long long>(1, std::min<long long>(nkeys, kChunkBytes / (C::pk_bytes + C::sk_bytes)));
  // GMC_KG_CHUNK_KEYS: keys per device-side staging chunk (lower than the default only)
  if (const char *v = getenv("GMC_KG_CHUNK_KEYS")) kc = std::max(1ll, std::min(kc, atoll(v)));
  wcap = (int)std::min<long long>(kc, cap);
  for (KgRound &b : R) {
    KG_CUDA(dalloc(&b.status, (size_t)cap, s1));
    KG_CUDA(dalloc(&b.g, (size_t)cap * C::gstride, s1));
    KG_CUDA(dalloc(&b.pi, (size_t)cap * C::q, s1));
    KG_CUDA(dalloc(&b.matL, (size_t)cap * C::mt * C::rwl, s1));
    KG_CUDA(dalloc(&b.rptr, (size_t)cap, s1));
    KG_CUDA(dalloc(&b.win, (size_t)2 * wcap, s1));
    KG_CUDA(cudaMallocHost(&b.h_rptr, (size_t)cap * sizeof(void *)));
    KG_CUDA(cudaMallocHost(&b.h_status, (size_t)cap));
    KG_CUDA(cudaMallocHost(&b.h_win, (size_t)2 * wcap * sizeof(int)));
    KG_CUDA(cudaEventCreateWithFlags(&b.ranked, cudaEventDisableTiming));
    KG_CUDA(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming));
  }
  KG_CUDA(dalloc(&d_seedc, (size_t)kc * 32, s1));
  KG_CUDA(dalloc(&d_matF, (size_t)wcap * C::mt * C::rw, s1));
  KG_CUDA(dalloc(&d_rowid, (size_t)wcap * C::mt, s1));
  KG_CUDA(dalloc(&d_cond, (size_t)wcap * C::cond_bytes, s1));
  KG_CUDA(dalloc(&d_clist, (size_t)wcap * 32, s1));
  KG_CUDA(dalloc(&d_cbok, (size_t)kc, s1));
  KG_CUDA(dalloc(&d_pk, (size_t)kc * C::pk_bytes, s1));
  KG_CUDA(dalloc(&d_sk, (size_t)kc * C::sk_bytes, s1));
  KG_CUDA(cudaStreamSynchronize(s1));
  for (long long k0 = 0; k0 < nkeys; k0 += kc) {
    const long long nk = std::min(kc, nkeys - k0);
    // chain heads, then the first store block for every key (stream 0 runs ahead of the rounds)
    KG_CUDA(cudaMemcpyAsync(d_seedc, seeds + 32 * k0, (size_t)nk * 32, cudaMemcpyHostToDevice, s0));
    kblocks.assign(nk, {});
    na.assign(nk, 0);
    pending.clear();
    for (long long i = 0; i < nk; i++) pending.push_back(i);
    auto add_block = [&](const std::vector<long long> *keys, int a0, int nlinks) -> cudaError_t {
      blocks.emplace_back();  // owned by the list from here on (freed with it on any exit)
      const int bid = (int)blocks.size() - 1;
      KgBlock &blk = blocks.back();
      blk.nb = keys ? (int)keys->size() : (int)nk;
      blk.a0 = a0;
      blk.nlinks = nlinks;
      blk.slot.assign(nk, -1);
      cudaError_t e = dalloc(&blk.base, (size_t)blk.nb * nlinks * C::rstride, s0);
      if (e != cudaSuccess) return e;
      if (keys) {
        if ((e = cudaMallocHost(&blk.h_keys, (size_t)blk.nb * sizeof(int))) != cudaSuccess) return e;
        for (int i = 0; i < blk.nb; i++) blk.h_keys[i] = (int)(*keys)[i];
        if ((e = dalloc(&blk.keys, (size_t)blk.nb, s0)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(blk.keys, blk.h_keys, (size_t)blk.nb * sizeof(int), cudaMemcpyHostToDevice,
                                 s0)) != cudaSuccess)
          return e;
      }
      for (int i = 0; i < blk.nb; i++) {
        const int key = keys ? (int)(*keys)[i] : i;
        blk.slot[key] = i;
        kblocks[key].push_back(bid);
      }
      blk.seq0 = (int)links.size();
      for (int a = 0; a < nlinks; a++) {
        kg_expand_kernel<SET><<<(blk.nb + 31) / 32, 32, 0, s0>>>(d_seedc, blk.keys, blk.nb, a, blk.base);
        cudaEvent_t ev;
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
        links.push_back(ev);
        if ((e = cudaEventRecord(ev, s0)) != cudaSuccess) return e;
      }
      return cudaGetLastError();
    };
    // links ahead: a key needs more than L attempts with probability ~0.71^L
    // (29% of attempts succeed for every set), so ln(nk)/0.34 + 8 links cover
    // the whole chunk but in ~6% of calls
    int ahead = std::min(64, std::max(12, (int)std::ceil(std::log((double)nk) / 0.3425) + 8));
    // GMC_KG_AHEAD_LINKS: links expanded ahead (1..64); fewer make the extension blocks carry the chains
    if (const char *v = getenv("GMC_KG_AHEAD_LINKS")) ahead = std::max(1, std::min(64, atoi(v)));
    KG_CUDA(add_block(nullptr, 0, ahead));
    KG_CUDA(cudaMemsetAsync(d_cbok, 0, (size_t)nk, s2));
    for (int round = 0; !pending.empty(); round++) {
      KgRound &b = R[round & 1];
      if (round >= 2) KG_CUDA(cudaEventSynchronize(b.done));  // round-2's winners released these buffers
      const int nr = (int)std::min<long long>((long long)pending.size(), cap);
      const int k = std::max(1, std::min(kMaxSpeculation, cap / nr));
      const int natt = nr * k;
      // chains that run past their store: one more block for every pending key
      // (every pending key has been in every block so far: the same attempts)
      {
        const KgBlock &last = blocks[kblocks[pending[0]].back()];
        const int end = last.a0 + last.nlinks;
        int need = end;
        for (int j = 0; j < nr; j++) need = std::max(need, na[pending[j]] + k);
        // as many links as this round needs, at least one extension block's worth
        if (need > end) KG_CUDA(add_block(&pending, end, std::max(need - end, kExpandBlock / 2)));
      }
      int wait_seq = 0;
      for (int j = 0; j < nr; j++) {
        const long long key = pending[j];
        for (int a = 0; a < k; a++) {
          const int A = na[key] + a;
          int bi = 0;
          while (A >= blocks[kblocks[key][bi]].a0 + blocks[kblocks[key][bi]].nlinks) bi++;
          const KgBlock &blk = blocks[kblocks[key][bi]];
          const int al = A - blk.a0;
          b.h_rptr[j * k + a] = blk.base + ((long long)al * blk.nb + blk.slot[key]) * C::rstride;
          wait_seq = std::max(wait_seq, blk.seq0 + al);
        }
      }
      KG_CUDA(cudaStreamWaitEvent(s1, links[wait_seq], 0));
      KG_CUDA(cudaMemcpyAsync(b.rptr, b.h_rptr, (size_t)natt * sizeof(void *), cudaMemcpyHostToDevice, s1));
      KG_CUDA(cudaMemsetAsync(b.status, 0, (size_t)natt, s1));
      kg_minpoly_kernel<SET><<<natt, kMinpolyThreads, MinpolySmem<SET>::bytes, s1>>>(b.rptr, natt, fd.gexp,
                                                                                   fd.glog, b.g, b.status);
      kg_support_kernel<SET><<<natt, kSupportThreads, C::q * 8, s1>>>(b.rptr, natt, b.pi, b.status);
      kg_build_kernel<SET><<<dim3(C::rwl / 8, natt), kBuildThreads, BuildSmem<SET>::bytes, s1>>>(
          b.g, b.pi, nullptr, b.status, b.matL, C::rwl, C::rwl, fd.gexp, fd.glog);
      kg_elim_kernel<SET, kg_table_bits<SET>()><<<natt, ElimCfg<kg_table_bits<SET>()>::nt, ElimSmem<SET, kg_table_bits<SET>()>::bytes, s1>>>(
          b.matL, C::rwl, C::rwl, nullptr, b.status, kKgMinpoly | kKgDistinct, kKgRank, 1, 1, nullptr, semi ? 1 : 0,
          nullptr, nullptr);
      KG_CUDA(cudaGetLastError());
      KG_CUDA(cudaMemcpyAsync(b.h_status, b.status, natt, cudaMemcpyDeviceToHost, s1));
      KG_CUDA(cudaEventRecord(b.ranked, s1));
      KG_CUDA(cudaStreamSynchronize(s1));
      int nw = 0;
      next.clear();
      for (int j = 0; j < nr; j++) {
        const long long key = pending[j];
        int a = 0;
        while (a < k && b.h_status[(size_t)j * k + a] != kKgAll) a++;
        if (a < k) {
          b.h_win[nw] = j * k + a;
          b.h_win[wcap + nw] = (int)key;
          nw++;
        } else {
          na[key] += k;
          if (na[key] >= kMaxAttemptsPerKey) {
            rc = kg_fail(GMC_EKEY, "gmc_keypair_batch: no systematic key within the attempt limit");
            goto done;
          }
          next.push_back(key);
        }
      }
      for (size_t j = nr; j < pending.size(); j++) next.push_back(pending[j]);
      if (nw) {
        int *watt = b.win, *wout = b.win + wcap;
        KG_CUDA(cudaStreamWaitEvent(s2, b.ranked, 0));
        KG_CUDA(cudaMemcpyAsync(b.win, b.h_win, (size_t)2 * wcap * sizeof(int), cudaMemcpyHostToDevice, s2));
        kg_build_kernel<SET><<<dim3(C::rw / 8, nw), kBuildThreads, BuildSmem<SET>::bytes, s2>>>(
            b.g, b.pi, watt, b.status, d_matF, C::rw, C::rw, fd.gexp, fd.glog);
        {
          // the winners' status has every bit: the full elimination re-derives the same pivots
          cudaLaunchConfig_t lc = {};
          cudaLaunchAttribute at[1];
          at[0].id = cudaLaunchAttributeClusterDimension;
          at[0].val.clusterDim.x = kElimCluster;
          at[0].val.clusterDim.y = 1;
          at[0].val.clusterDim.z = 1;
          lc.gridDim = dim3(nw * kElimCluster);
          lc.blockDim = dim3(ElimCfg<kg_table_bits<SET>()>::nt);
          lc.dynamicSmemBytes = ElimSmem<SET, kg_table_bits<SET>()>::bytes;
          lc.stream = s2;
          lc.attrs = at;
          lc.numAttrs = 1;
          KG_CUDA(cudaLaunchKernelEx(&lc, kg_elim_kernel<SET, kg_table_bits<SET>()>, d_matF, (int)C::rw, (int)C::rw, (const int *)watt,
                                     b.status, (int)kKgAll, (int)kKgAll, 0, kElimCluster, d_rowid, semi ? 1 : 0,
                                     semi ? d_clist : (uint8_t *)nullptr, semi ? b.pi : (uint16_t *)nullptr));
        }
        kg_cbits_kernel<SET><<<nw, kCbitsThreads, CbitsSmem<SET>::bytes, s2>>>(b.pi, watt, wout, nw, d_cond, d_cbok);
        kg_assemble_kernel<SET><<<dim3(256, nw), 256, 0, s2>>>(watt, wout, nw, (const uint8_t *const *)b.rptr, b.g,
                                                                d_cond, d_matF, d_rowid, semi ? d_clist : nullptr,
                                                                d_pk, d_sk);
        KG_CUDA(cudaGetLastError());
      }
      KG_CUDA(cudaEventRecord(b.done, s2));
      if (trace)
        fprintf(stderr, "[keygen] set %d round %d: %d keys x %d attempts (link <= %d, %zu blocks), %d winners, "
                        "ranked at %.2f ms\n", SET, round, nr, k, wait_seq, blocks.size(), nw, ms_now());
      pending.swap(next);
    }
    KG_CUDA(cudaStreamSynchronize(s2));
    if (trace) fprintf(stderr, "[keygen] winners done at %.2f ms\n", ms_now());
    KG_CUDA(cudaStreamSynchronize(s0));
    if (trace) fprintf(stderr, "[keygen] expansion done at %.2f ms\n", ms_now());
    h_cbok.resize(nk);
    KG_CUDA(cudaMemcpy(h_cbok.data(), d_cbok, (size_t)nk, cudaMemcpyDeviceToHost));
    for (long long i = 0; i < nk; i++)
      if (!h_cbok[i]) {
        rc = kg_fail(GMC_EKEY, "gmc_keypair_batch: control bits do not encode the support permutation");
        goto done;
      }
    KG_CUDA(cudaMemcpy(pk + k0 * C::pk_bytes, d_pk, (size_t)nk * C::pk_bytes, cudaMemcpyDeviceToHost));
    KG_CUDA(cudaMemcpy(sk + k0 * C::sk_bytes, d_sk, (size_t)nk * C::sk_bytes, cudaMemcpyDeviceToHost));
    for (KgBlock &blk : blocks) {
      cudaFreeAsync(blk.base, s1);
      if (blk.keys) cudaFreeAsync(blk.keys, s1);
      if (blk.h_keys) cudaFreeHost(blk.h_keys);
    }
    blocks.clear();
    for (cudaEvent_t ev : links) cudaEventDestroy(ev);
    links.clear();
  }
done:
  cudaStreamSynchronize(s0);
  cudaStreamSynchronize(s1);
  cudaStreamSynchronize(s2);
  for (KgBlock &blk : blocks) {
    if (blk.base) cudaFreeAsync(blk.base, s1);
    if (blk.keys) cudaFreeAsync(blk.keys, s1);
    if (blk.h_keys) cudaFreeHost(blk.h_keys);
  }
  for (cudaEvent_t ev : links) cudaEventDestroy(ev);
  for (KgRound &b : R) {
    for (void *p : {(void *)b.status, (void *)b.g, (void *)b.pi, (void *)b.matL, (void *)b.rptr, (void *)b.win})
      if (p) cudaFreeAsync(p, s1);
    if (b.h_rptr) cudaFreeHost(b.h_rptr);
    if (b.h_status) cudaFreeHost(b.h_status);
    if (b.h_win) cudaFreeHost(b.h_win);
    if (b.ranked) cudaEventDestroy(b.ranked);
    if (b.done) cudaEventDestroy(b.done);
  }
  for (void *p : {(void *)d_seedc, (void *)d_matF, (void *)d_rowid, (void *)d_cond, (void *)d_cbok, (void *)d_pk,
                  (void *)d_sk, (void *)d_clist})
    if (p) cudaFreeAsync(p, s1);
  {
    cudaError_t e = cudaStreamSynchronize(s1);
    if (rc == GMC_OK && e != cudaSuccess) rc = kg_fail(GMC_ECUDA, std::string("gmc_keypair_batch: ") + cudaGetErrorString(e));
  }
  return rc;
}
#undef KG_CUDA
}  // namespace

}  // namespace gmc

// Batched key generation (host buffers): key i from seeds[32 i .. 32 i + 31],
// the single randombytes draw of libmceliece's keypair; identical bytes to
// gmc_keypair_seed for every key.
extern "C" int gmc_keypair_batch(int set, unsigned char *pk, unsigned char *sk, const unsigned char *seeds,
                                 long long nkeys) {
  using namespace gmc;
  if (set < 0 || set >= GMC_NVARIANTS || nkeys < 0 || (nkeys > 0 && (!pk || !sk || !seeds)))
    return kg_fail(GMC_EINVAL, "gmc_keypair_batch: bad argument");
  // plaintext-confirmation variants have the keys of their set; f variants the semi-systematic form
  const bool semi = ((set / GMC_NSETS) & 2) != 0;
  set %= GMC_NSETS;
  if (nkeys == 0) return GMC_OK;
  // chain links and rounds are on the critical path (the host waits for each
  // round's ranks); the winners' work only has to finish by the end
  cudaStream_t s0 = nullptr, s1 = nullptr, s2 = nullptr;
  int prio_low = 0, prio_high = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s0, cudaStreamNonBlocking, prio_high);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s1, cudaStreamNonBlocking, prio_high);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s2, cudaStreamNonBlocking, prio_low);
  int rc = GMC_EINVAL;
  if (e != cudaSuccess) {
    rc = kg_fail(GMC_ECUDA, std::string("gmc_keypair_batch: ") + cudaGetErrorString(e));
  } else {
    switch (set) {
      case 0: rc = keypair_batch<0>(pk, sk, seeds, nkeys, semi, s0, s1, s2); break;
      case 1: rc = keypair_batch<1>(pk, sk, seeds, nkeys, semi, s0, s1, s2); break;
      case 2: rc = keypair_batch<2>(pk, sk, seeds, nkeys, semi, s0, s1, s2); break;
      case 3: rc = keypair_batch<3>(pk, sk, seeds, nkeys, semi, s0, s1, s2); break;
      case 4: rc = keypair_batch<4>(pk, sk, seeds, nkeys, semi, s0, s1, s2); break;
    }
  }
  if (s0) cudaStreamDestroy(s0);
  if (s1) cudaStreamDestroy(s1);
  if (s2) cudaStreamDestroy(s2);
  return rc;
}
