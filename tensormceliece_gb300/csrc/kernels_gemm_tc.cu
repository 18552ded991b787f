// Tensor-core engines for the batched GF(2) products Out[op] = A * X[op].
//
// GEMM_TC: 5th-generation tensor cores (tcgen05). 0/1 operands carried as FP8
// e4m3 (key bits 0x00 / 0x38 = 1.0, request bits 0x00 / 0x01 = 2^-9) through
// tcgen05.mma .kind::f8f6f4 with FP32 accumulators in tensor memory. Sums of
// products are integer counts <= K (at most 6656 here) times 2^-9, exact in
// FP32, so parity = the last mantissa bit of acc * 2^9 + 2^23 (K < 2^23).
// (.kind::i8 is not available on sm_103a.)
//   A (key matrix, fixed per key) is pre-expanded once into FP8 tiles laid
//   out exactly as the shared-memory image of one pipeline stage, so a stage
//   is one cp.async.bulk (TMA engine) completing on an mbarrier.
//   X (request bits) is expanded to FP8 by the CUDA cores into the same
//   canonical layout (no-swizzle K-major: 8-row x 16-byte core matrices,
//   K-adjacent core matrices 128 B apart, row groups 1024 B apart).
//   Warp roles: expander warps write the X stages, one warp's lane 0
//   issues the A copies, another's lane 0 issues 4 MMAs (K = 32 each) per
//   128-bit K stage. Stages hand over through mbarriers only: A full (copy
//   bytes landed), X full (one arrival per expander thread), empty (the MMA
//   commit that releases both buffers), so expansion, copies and MMAs of
//   different stages overlap. Epilogue warps read the accumulators with
//   tcgen05.ld and pack 32 parities per ballot.
//   Every wait is bounded (about 2 s of globaltimer); on expiry the CTA sets
//   the error word, stops issuing, waits (bounded) for its own copies and
//   MMAs, frees its tensor memory and returns.
//
// GEMM_B1MMA: the legacy 1-bit path, mma.sync m8n8k128 .b1 AND.POPC (the
// reference's engine family, mceliece-gpu-params/tc_kernels.cuh:97-123).
#include "kernels.h"

namespace gmc {

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
constexpr uint64_t kWaitLimitNs = 2000000000ull;
// bounded wait on an mbarrier phase; false when the limit expired
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Shared-memory matrix descriptor (tcgen05): start, leading- and stride-
// dimension byte offsets (16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, .kind::f8f6f4: D = F32 (bits 4-5 = 1), A = B = E4M3
// (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_f8f6f4_e4m3(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

#define GMC_TMEM_LD32(taddr, r)                                                                                 \
  asm volatile(                                                                                                 \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"  \
      "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                                        \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),         \
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),   \
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), \
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])  \
      : "r"(taddr))
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 4 bits -> 4 FP8 bytes (bit i -> byte i = 0x38 = 1.0 or 0): the key matrix
__device__ __forceinline__ uint32_t expand4(uint32_t v) {
  return ((v * 0x00204081u) & 0x01010101u) * 0x38u;
}
// 4 bits -> 4 FP8 bytes (bit i -> byte i = 0x01 or 0): the request bits, as
// the E4M3 subnormal 2^-9, one multiply fewer per nibble than 1.0. Products
// with the key's 1.0 are 2^-9, a K-sum is count * 2^-9 with count <= K
// (exact in FP32), and the epilogue scales it back by 2^9 before the parity.
__device__ __forceinline__ uint32_t expand4_x(uint32_t v) { return (v * 0x00204081u) & 0x01010101u; }
constexpr float kTcXScale = 512.0f;

// ---------------------------------------------------------------- tcgen05 engine
// Persistent: one CTA per SM walks the (request tile, key tile) list. The MMA
// is D[request][key row] = sum_k X[request][k] Key[row][k]: M = 128 requests
// (the A operand, staged in FP8 by the CUDA cores) by N = 256 key rows (the B
// operand: two 128-row slices of the key's FP8 image per stage, by bulk copy),
// so one 16 KB request stage feeds 4 MMAs of 128 x 256 x 32. The request
// staging is the CUDA-core work around the MMAs; with the requests as the
// N = 256 side it took twice as much per MMA. The stage ring runs on across
// tiles, and the FP32 accumulator is double-buffered in tensor memory (2 x 256
// columns), so the epilogue of one tile overlaps the MMAs of the next.
// Accumulator lane = request, column = key row: an epilogue thread reads 32
// columns of its request and packs their parities into one output word.
// Warp roles: the first TC_EXP_WARPS stage requests, the next issues the key
// copies, the next issues the MMAs, the last four drain accumulators (warp w
// reads TMEM lanes 32 (w % 4) .. +31).
constexpr int TC_REQ = 128;   // requests per tile (MMA M)
constexpr int TC_KEYN = 256;  // key rows per tile (MMA N): two kTcM-row slices of the key's FP8 image
constexpr int TC_EXP_WARPS = 8;
constexpr int TC_THREADS = (TC_EXP_WARPS + 2 + 4) * 32;  // expanders, producer, MMA, 4 epilogue warps
constexpr int TC_EXP_THREADS = TC_EXP_WARPS * 32;
constexpr int TC_A_BYTES = kTcM * kTcKB;    // 16 KB: one 128-row slice of the key image per stage
constexpr int TC_K_BYTES = 2 * TC_A_BYTES;  // 32 KB: the key stage (N = 256 rows)
constexpr int TC_X_BYTES = TC_REQ * kTcKB;  // 16 KB: the request stage (M = 128 rows)
constexpr int tc_smem(int stages) { return stages * (TC_K_BYTES + TC_X_BYTES) + 512; }
constexpr uint32_t TC_TMEM_COLS = 2 * TC_KEYN;  // two FP32 accumulators of 128 lanes x 256 columns
static_assert(TC_EXP_THREADS % TC_REQ == 0 && 4 % (TC_EXP_THREADS / TC_REQ) == 0,
              "expander threads split each request row into equal word ranges");
static_assert(TC_KEYN == 2 * kTcM, "a key tile is two slices of the FP8 image");

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1) gf2_gemm_tc(const GemmKeys keys, const Segs segs, int kstages,
                                                              int mtiles, long long rtiles,
                                                              const uint32_t *__restrict__ X, int ldx,
                                                              uint32_t *__restrict__ Out, int ldo, int out_words,
                                                              int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t tsm[];
  uint8_t *Ks = tsm;                        // key stages [STAGES][TC_K_BYTES]
  uint8_t *Xs = tsm + STAGES * TC_K_BYTES;  // request stages [STAGES][TC_X_BYTES]
  uint64_t *full_a = reinterpret_cast<uint64_t *>(Xs + STAGES * TC_X_BYTES);
  uint64_t *full_x = full_a + STAGES;
  uint64_t *empty = full_x + STAGES;
  uint64_t *acc_full = empty + STAGES;  // [2]
  uint64_t *acc_empty = acc_full + 2;      // [2]
  uint64_t *done = acc_empty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  int *last_copy = reinterpret_cast<int *>(tmem_slot + 2);  // [STAGES]: last stage copied per buffer

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ktiles = (mtiles + 1) >> 1;  // key tiles of 256 rows (the last one half when mtiles is odd)
  const long long ntile_all = (long long)ktiles * rtiles;
  if (tid == 0) {
    for (int i = 0; i < STAGES; i++) {
      mbar_init(&full_a[i], 1);
      mbar_init(&full_x[i], TC_EXP_THREADS);
      mbar_init(&empty[i], 1);
      last_copy[i] = -1;
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 4 * 32);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, TC_TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t idesc = idesc_f8f6f4_e4m3(TC_REQ, TC_KEYN);

  if (warp < TC_EXP_WARPS) {
    // request stagers: SPLIT threads share each 128-bit stage row; thread tid
    // takes row r = tid % TC_REQ, request words WPT * part .. + WPT - 1 of the
    // stage and their 16-bit chunks KCT * part .. + KCT - 1
    constexpr int SPLIT = TC_EXP_THREADS / TC_REQ;
    constexpr int WPT = 4 / SPLIT;
    constexpr int KCT = 8 / SPLIT;
    const int r = tid % TC_REQ, part = tid / TC_REQ;
    long long g = 0;  // global stage counter of this CTA
    for (long long tile = blockIdx.x; tile < ntile_all && !*abort_flag; tile += gridDim.x) {
      const long long op0 = (tile / ktiles) * TC_REQ;
      const uint32_t *xrow = X + (size_t)(op0 + r) * ldx + WPT * part;
      uint32_t xnext[WPT];
#pragma unroll
      for (int w = 0; w < WPT; w++) xnext[w] = xrow[w];
      for (int s = 0; s < kstages; s++, g++) {
        const int buf = (int)(g % STAGES);
        if (g >= STAGES && !mbar_wait(&empty[buf], (uint32_t)(g / STAGES - 1) & 1)) *abort_flag = 1;
        if (*abort_flag) break;
        uint32_t wv[WPT];
#pragma unroll
        for (int w = 0; w < WPT; w++) wv[w] = xnext[w];
        if (s + 1 < kstages) {
#pragma unroll
          for (int w = 0; w < WPT; w++) xnext[w] = xrow[4 * (s + 1) + w];
        }
        // request bits -> FP8 core matrices (row r, 16-bit chunk kc at
        // ((r/8)*8 + kc)*128 + (r%8)*16)
        uint8_t *rb = Xs + buf * TC_X_BYTES + (r >> 3) * 1024 + (r & 7) * 16;
#pragma unroll
        for (int c = 0; c < KCT; c++) {
          const int kc = KCT * part + c;
          const uint32_t bits = (c & 1) ? (wv[c >> 1] >> 16) : (wv[c >> 1] & 0xFFFFu);
          uint4 v;
          v.x = expand4_x(bits & 0xFu);
          v.y = expand4_x((bits >> 4) & 0xFu);
          v.z = expand4_x((bits >> 8) & 0xFu);
          v.w = expand4_x((bits >> 12) & 0xFu);
          *reinterpret_cast<uint4 *>(rb + kc * 128) = v;
        }
        fence_proxy_async();  // generic-proxy writes visible to the tensor core
        mbar_arrive(&full_x[buf]);
      }
    }
  } else if (warp == TC_EXP_WARPS) {
    if (lane == 0) {  // key producer: the tile's one or two 128-row slices per stage into a free buffer
      long long g = 0;
      for (long long tile = blockIdx.x; tile < ntile_all && !*abort_flag; tile += gridDim.x) {
        const int m0 = 2 * (int)(tile % ktiles);
        const bool two = m0 + 1 < mtiles;
        const int seg = seg_find(segs, (tile / ktiles) * TC_REQ);  // a tile never straddles segments
        const uint8_t *A0 = keys.A8[seg] + (size_t)m0 * kstages * TC_A_BYTES;
        for (int s = 0; s < kstages; s++, g++) {
          const int buf = (int)(g % STAGES);
          if (g >= STAGES && !mbar_wait(&empty[buf], (uint32_t)(g / STAGES - 1) & 1)) *abort_flag = 1;
          if (*abort_flag) break;
          mbar_expect_tx(&full_a[buf], two ? 2 * TC_A_BYTES : TC_A_BYTES);
          bulk_g2s(Ks + buf * TC_K_BYTES, A0 + (size_t)s * TC_A_BYTES, TC_A_BYTES, &full_a[buf]);
          if (two)
            bulk_g2s(Ks + buf * TC_K_BYTES + TC_A_BYTES, A0 + (size_t)(kstages + s) * TC_A_BYTES, TC_A_BYTES,
                     &full_a[buf]);
          last_copy[buf] = (int)g;
        }
      }
    }
  } else if (warp == TC_EXP_WARPS + 1) {
    if (lane == 0) {  // MMA issuer
      long long g = 0;
      int i = 0;  // local tile index
      for (long long tile = blockIdx.x; tile < ntile_all && !*abort_flag; tile += gridDim.x, i++) {
        const int ab = i & 1;
        // the epilogue has drained this accumulator's previous tile
        if (i >= 2 && !mbar_wait(&acc_empty[ab], (uint32_t)((i >> 1) - 1) & 1)) *abort_flag = 1;
        if (*abort_flag) break;
        tc_fence_after();
        const uint32_t dacc = tmem + (uint32_t)(ab * TC_KEYN);
        for (int s = 0; s < kstages; s++, g++) {
          const int buf = (int)(g % STAGES);
          const uint32_t par = (uint32_t)(g / STAGES) & 1;
          if (!mbar_wait(&full_a[buf], par) || !mbar_wait(&full_x[buf], par)) *abort_flag = 1;
          if (*abort_flag) break;
          tc_fence_after();
          const uint32_t x0 = smem_u32(Xs + buf * TC_X_BYTES), k0 = smem_u32(Ks + buf * TC_K_BYTES);
#pragma unroll
          for (int kk = 0; kk < kTcKB / 32; kk++) {
            const uint64_t ad = smem_desc(x0 + kk * 256, 128, 1024);  // A: 128 requests
            const uint64_t bd = smem_desc(k0 + kk * 256, 128, 1024);  // B: 256 key rows
            mma_f8(dacc, ad, bd, idesc, (s > 0 || kk > 0) ? 1u : 0u);
          }
          mma_commit(&empty[buf]);
        }
        if (*abort_flag) break;
        mma_commit(&acc_full[ab]);  // arrives when this tile's MMAs have completed
      }
      mma_commit(done);  // arrives once every MMA issued above has completed
    }
  } else {
    // epilogue: accumulator lanes 32 (warp % 4) .. +31 = this warp's requests;
    // lane l packs the parities of its request's 256 key rows into 8 words
    const int quad = warp & 3;
    const bool vec = (ldo & 3) == 0 && (reinterpret_cast<uintptr_t>(Out) & 15) == 0;
    int i = 0;
    for (long long tile = blockIdx.x; tile < ntile_all && !*abort_flag; tile += gridDim.x, i++) {
      const int ab = i & 1;
      if (!mbar_wait(&acc_full[ab], (uint32_t)(i >> 1) & 1)) *abort_flag = 1;
      if (*abort_flag) break;
      tc_fence_after();
      const int kt = (int)(tile % ktiles);
      const long long op0 = (tile / ktiles) * TC_REQ;
      const int seg = seg_find(segs, op0);
      const long long live_end = segs.row0[seg] + segs.nreq[seg];
      const long long op = op0 + 32 * quad + lane;
      const int wd0 = kt * (TC_KEYN / 32);
      uint32_t *orow = Out + op * ldo + wd0;
      const bool live = op < live_end, vec_ok = vec && wd0 + TC_KEYN / 32 <= out_words;
      // two halves of 4 x 32 columns (bounded register use), each stored at once
#pragma unroll 1
      for (int h = 0; h < 2; h++) {
        uint32_t w4[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
          uint32_t rr[32];
          GMC_TMEM_LD32(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(ab * TC_KEYN + 32 * (4 * h + c)), rr);
          tmem_ld_wait();
          uint32_t w = 0;
#pragma unroll
          for (int j = 0; j < 32; j++) {
            // acc * 2^9 + 2^23 = count + 2^23 exactly (count <= 6656 < 2^23): the
            // float's last mantissa bit is the count's parity, no conversion needed
            w |= (__float_as_uint(__fmaf_rn(__uint_as_float(rr[j]), kTcXScale, 8388608.0f)) & 1u) << j;
          }
          w4[c] = w;
        }
        if (live) {
          if (vec_ok) {
            reinterpret_cast<uint4 *>(orow)[h] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
          } else {
#pragma unroll
            for (int c = 0; c < 4; c++)
              if (wd0 + 4 * h + c < out_words) orow[4 * h + c] = w4[c];
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[ab]);
    }
  }
  __syncthreads();
  // drain: the MMAs (done barrier) and any key copy still landing
  bool ok = mbar_wait(done, 0);
  if (warp == TC_EXP_WARPS && lane == 0) {
    for (int b = 0; b < STAGES; b++)
      if (last_copy[b] >= 0 && !mbar_wait(&full_a[b], (uint32_t)(last_copy[b] / STAGES) & 1)) ok = false;
  }
  const int good = __syncthreads_and(ok && !*abort_flag);
  if (!good && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, TC_TMEM_COLS);
}

// A (packed bits, rows_pad x lda words) -> FP8 stage images:
// [m-tile][stage][row group g][16-byte chunk kc][row r&7][16 bytes]
__global__ void expand_a_kernel(const uint32_t *__restrict__ A, int lda, int rows_pad, int kstages,
                                uint8_t *__restrict__ A8) {
  const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // (row, 16-bit chunk)
  const long long total = (long long)rows_pad * kstages * 8;
  if (item >= total) return;
  const int row = (int)(item / (kstages * 8));
  const int rest = (int)(item % (kstages * 8));
  const int s = rest >> 3, kc = rest & 7;
  const uint32_t w = A[(size_t)row * lda + 4 * s + (kc >> 1)];
  const uint32_t bits = (kc & 1) ? (w >> 16) : (w & 0xFFFFu);
  uint4 v;
  v.x = expand4(bits & 0xFu);
  v.y = expand4((bits >> 4) & 0xFu);
  v.z = expand4((bits >> 8) & 0xFu);
  v.w = expand4((bits >> 12) & 0xFu);
  const int mt = row / kTcM, rr = row % kTcM;
  const size_t off = ((size_t)mt * kstages + s) * TC_A_BYTES + ((rr >> 3) * 8 + kc) * 128 + (rr & 7) * 16;
  *reinterpret_cast<uint4 *>(A8 + off) = v;
}

size_t tc_a8_bytes(int rows_pad, int kw_pad) { return (size_t)rows_pad * kw_pad * 32; }

cudaError_t launch_expand_a(const uint32_t *A, int lda, int rows_pad, int kw_pad, uint8_t *A8, cudaStream_t st) {
  if (rows_pad % kTcM || kw_pad % (kTcKB / 32)) return cudaErrorInvalidValue;
  const int kstages = kw_pad / (kTcKB / 32);
  const long long total = (long long)rows_pad * kstages * 8;
  expand_a_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(A, lda, rows_pad, kstages, A8);
  return cudaGetLastError();
}

cudaError_t launch_gf2_gemm_tc(const GemmKeys &keys, const Segs &segs, int rows_pad, const uint32_t *X, int ldx,
                               int kw_pad, uint32_t *Out, int ldo, int out_words, int *err, cudaStream_t st) {
  const long long rows = seg_rows(segs);
  if (rows <= 0) return cudaSuccess;
  if (!err || rows_pad % kTcM || kw_pad % (kTcKB / 32) || rows % TC_REQ || ldx < kw_pad) return cudaErrorInvalidValue;
  for (int i = 0; i < segs.nseg; i++)
    if (!keys.A8[i]) return cudaErrorInvalidValue;
  // pipeline depth: the set's tuned stage count (2, 3 or 4 buffers of A and X per CTA)
  const int stages = keys.tc_stages == 2 || keys.tc_stages == 3 ? keys.tc_stages : kTcStages;
  auto kern = stages == 2 ? gf2_gemm_tc<2> : stages == 3 ? gf2_gemm_tc<3> : gf2_gemm_tc<kTcStages>;
  const int smem = tc_smem(stages);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int mtiles = rows_pad / kTcM;
  const long long rtiles = rows / TC_REQ, tiles = rtiles * ((mtiles + 1) / 2);
  const int grid = (int)(tiles < sms ? tiles : sms);  // persistent: one CTA per SM (smem and TMEM bound)
  kern<<<grid, TC_THREADS, smem, st>>>(keys, segs, kw_pad / (kTcKB / 32), mtiles, rtiles, X, ldx, Out, ldo,
                                       out_words, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- tcgen05 FP8 peak
// The MMA rate of this GPU for the engine's instruction: tcgen05.mma
// .kind::f8f6f4, E4M3 operands, M = 128, N = 256, K = 32, FP32 accumulator in
// tensor memory, operands resident in shared memory (no copies, no
// expansion). One CTA per SM; lane 0 of warp 1 issues `iters` MMAs into one
// accumulator, cycling over the 4 K-slices of a 128-bit stage, then one
// commit; every thread waits (bounded) for it. The denominator of the GEMM's
// tensor-pipe fraction.
constexpr int TCP_THREADS = 128;
constexpr int TCP_A_BYTES = kTcM * kTcKB;  // 16 KB: A, 128 rows of one 128-bit K stage
constexpr int TCP_B_BYTES = kTcN * kTcKB;  // 32 KB: B, 256 rows

__global__ void __launch_bounds__(TCP_THREADS, 1) tc_f8_peak_kernel(int iters, int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t psm[];
  uint8_t *As = psm;
  uint8_t *Xs = psm + TCP_A_BYTES;
  uint64_t *done = reinterpret_cast<uint64_t *>(Xs + TCP_B_BYTES);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < (TCP_A_BYTES + TCP_B_BYTES) / 16; i += TCP_THREADS)
    reinterpret_cast<uint4 *>(psm)[i] = make_uint4(0x38383838u, 0, 0x38383838u, 0);
  if (tid == 0) {
    mbar_init(done, 1);
    fence_mbar_init();
  }
  fence_proxy_async();  // operand writes visible to the tensor core
  if (warp == 0) {
    tmem_alloc(tmem_slot, kTcN);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = idesc_f8f6f4_e4m3(kTcM, kTcN);
    const uint32_t a0 = smem_u32(As), x0 = smem_u32(Xs);
#pragma unroll 1
    for (int i = 0; i < iters; i++) {
      const int kk = i & (kTcKB / 32 - 1);
      mma_f8(tmem, smem_desc(a0 + kk * 256, 128, 1024), smem_desc(x0 + kk * 256, 128, 1024), idesc, i ? 1u : 0u);
    }
    mma_commit(done);
  }
  const bool ok = mbar_wait(done, 0);
  if (!__syncthreads_and(ok) && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTcN);
}

cudaError_t time_tc_f8_peak(double *mac_per_s, int *err_dev, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int smem = TCP_A_BYTES + TCP_B_BYTES + 64;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(tc_f8_peak_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int iters = 1 << 16;  // ~4.7 ms per launch at the nominal dense rate
  float best = 0;
  for (int rep = 0; rep < 5 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0, st);
    tc_f8_peak_kernel<<<sms, TCP_THREADS, smem, st>>>(iters, err_dev);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    if (rep >= 1 && (best == 0 || t < best)) best = t;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  *mac_per_s = (double)sms * iters * kTcM * kTcN * 32.0 / (best * 1e-3);
  return cudaSuccess;
}

// ---------------------------------------------------------------- legacy b1 MMA engine
// Warp tile 32 rows x 32 requests (4 x 4 m8n8k128 MMAs per 128-bit K step),
// 4 warps per block covering 128 rows. Fragments come straight from global
// memory (L1/L2): A row (lane/4) bits 32*(lane%4).., B column (lane/4) the same.
__global__ void __launch_bounds__(128) gf2_gemm_b1(const GemmKeys keys, const Segs segs, int lda,
                                                    const uint32_t *__restrict__ X, int ldx, int kw_pad,
                                                    uint32_t *__restrict__ Out, int ldo, int out_words) {
  __shared__ uint32_t words[4][32];  // per warp: output word (32 rows) per request
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.y * 128 + warp * 32;
  const long long op0 = (long long)blockIdx.x * 32;
  const int seg = seg_find(segs, op0);
  const uint32_t *__restrict__ A = keys.A[seg];
  const long long live_end = segs.row0[seg] + segs.nreq[seg];
  int acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j][0] = acc[i][j][1] = 0;
  const int fr = lane >> 2, fk = lane & 3;
  for (int k = 0; k < kw_pad; k += 4) {
    uint32_t a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = A[(size_t)(row0 + 8 * i + fr) * lda + k + fk];
#pragma unroll
    for (int j = 0; j < 4; j++) b[j] = X[(size_t)(op0 + 8 * j + fr) * ldx + k + fk];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++)
        asm volatile(
            "mma.sync.aligned.m8n8k128.row.col.s32.b1.b1.s32.and.popc {%0,%1}, {%2}, {%3}, {%0,%1};"
            : "+r"(acc[i][j][0]), "+r"(acc[i][j][1])
            : "r"(a[i]), "r"(b[j]));
  }
  // D fragment: row (lane/4) + 8i, request 2(lane%4) + e + 8j
  words[warp][lane] = 0;
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int e = 0; e < 2; e++)
        if (acc[i][j][e] & 1) atomicOr(&words[warp][8 * j + 2 * fk + e], 1u << (8 * i + fr));
  __syncwarp();
  const long long op = op0 + lane;
  const int wd = row0 / 32;
  if (op < live_end && wd < out_words) Out[op * ldo + wd] = words[warp][lane];
}

// The rate of the legacy 1-bit MMA on this GPU: every warp runs 8 independent
// accumulator chains of mma.sync m8n8k128 .b1 AND.POPC on register operands
// (no memory traffic), 8 blocks of 256 threads per SM. The denominator of the
// b1 engine's fraction.
constexpr int kB1Chains = 8;
__global__ void __launch_bounds__(256) b1_peak_kernel(int iters, uint32_t salt, int *__restrict__ out) {
  int acc[kB1Chains][2];
#pragma unroll
  for (int c = 0; c < kB1Chains; c++) acc[c][0] = acc[c][1] = 0;
  const uint32_t a = (threadIdx.x * 2654435761u) ^ salt, b = (blockIdx.x * 40503u) ^ (salt >> 3);
#pragma unroll 1
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kB1Chains; c++)
      asm volatile("mma.sync.aligned.m8n8k128.row.col.s32.b1.b1.s32.and.popc {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+r"(acc[c][0]), "+r"(acc[c][1])
                   : "r"(a ^ (uint32_t)c), "r"(b));
  }
  int x = 0;
#pragma unroll
  for (int c = 0; c < kB1Chains; c++) x ^= acc[c][0] ^ acc[c][1];
  if (x == 0x7fffffff) out[0] = x;  // keeps the chains live; practically never stored
}

cudaError_t time_b1_peak(double *mac_per_s, int *out_dev, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int blocks = 8 * sms, iters = 2048;
  float best = 0;
  for (int rep = 0; rep < 5 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0, st);
    b1_peak_kernel<<<blocks, 256, 0, st>>>(iters, 0x9e3779b9u + rep, out_dev);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    if (rep >= 1 && (best == 0 || t < best)) best = t;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  *mac_per_s = (double)blocks * 8 /* warps */ * iters * kB1Chains * 8.0 * 8.0 * 128.0 / (best * 1e-3);
  return cudaSuccess;
}

cudaError_t launch_gf2_gemm_b1(const GemmKeys &keys, const Segs &segs, int lda, int rows_pad, const uint32_t *X,
                               int ldx, int kw_pad, uint32_t *Out, int ldo, int out_words, cudaStream_t st) {
  const long long rows = seg_rows(segs);
  if (rows <= 0) return cudaSuccess;
  if (rows_pad % 128 || kw_pad % 4 || rows % 32) return cudaErrorInvalidValue;
  dim3 grid((unsigned)(rows / 32), rows_pad / 128);
  gf2_gemm_b1<<<grid, 128, 0, st>>>(keys, segs, lda, X, ldx, kw_pad, Out, ldo, out_words);
  return cudaGetLastError();
}

}  // namespace gmc
