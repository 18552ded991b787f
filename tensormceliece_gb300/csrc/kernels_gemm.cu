// Batched GF(2) matrix products Out[op] = A * X[op] over GF(2):
//   bit r of Out[op] = parity(popcount(A[r] & X[op]))  (K words of 32 bits).
// Used for the encryption syndrome T*e[mt:n] (A = T, mt x k bits) and for the
// decapsulation front end F*c (A = F, 2tm x mt bits, built per secret key).
//
// Reference: syndrome (mceliece-gpu-params/ref/348864.cuh:3489-3527) and the
// 1-bit tensor-core syndrome kernels (mceliece-gpu-params/tc_kernels.cuh:97-123,
// mceliece-gpu-bmma/bmma_enc.h:74-134).
#include "kernels.h"

namespace gmc {

// ---------------------------------------------------------------- CUDA cores
// The parity of a sum of ANDs equals the parity of the XOR of the ANDs, so
// each 32-bit word of the K dimension costs one LOP3 (acc ^= a & x) and the
// popcount is taken once per output bit. Block tile 128 rows x 64 requests,
// 4 warps; warp w owns requests 16w..16w+15 of the tile and all 128 rows
// (rows lane + 32g, g < 4), so the 32 parities of a row group for a request
// come out of one __ballot_sync as the packed output word.
constexpr int POPC_THREADS = 128;
constexpr int POPC_OPS_PER_WARP = 16;

__global__ void __launch_bounds__(POPC_THREADS) gf2_gemm_popc(const GemmKeys keys, const Segs segs, int lda,
                                                               const uint32_t *__restrict__ X, int ldx, int kw_pad,
                                                               uint32_t *__restrict__ Out, int ldo, int out_words) {
  __shared__ uint32_t As[2][kGemmKTile][kGemmRowTile];
  __shared__ __align__(16) uint32_t Xs[2][kGemmOpTile][kGemmKTile];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long op0 = (long long)blockIdx.x * kGemmOpTile;
  const int row0 = blockIdx.y * kGemmRowTile;
  const int seg = seg_find(segs, op0);  // a tile never straddles segments
  const uint32_t *__restrict__ A = keys.A[seg];
  const long long live_end = segs.row0[seg] + segs.nreq[seg];
  const uint32_t *Arow = A + (size_t)(row0 + tid) * lda;          // this thread stages row tid
  const uint32_t *Xrow = X + (size_t)(op0 + (tid >> 1)) * ldx + 4 * (tid & 1);

  uint32_t acc[4][POPC_OPS_PER_WARP];
#pragma unroll
  for (int g = 0; g < 4; g++)
#pragma unroll
    for (int j = 0; j < POPC_OPS_PER_WARP; j++) acc[g][j] = 0;

  const int nchunks = kw_pad / kGemmKTile;
  uint4 ra0 = *reinterpret_cast<const uint4 *>(Arow);
  uint4 ra1 = *reinterpret_cast<const uint4 *>(Arow + 4);
  uint4 rx = *reinterpret_cast<const uint4 *>(Xrow);
  for (int c = 0; c < nchunks; c++) {
    const int buf = c & 1;
    As[buf][0][tid] = ra0.x; As[buf][1][tid] = ra0.y; As[buf][2][tid] = ra0.z; As[buf][3][tid] = ra0.w;
    As[buf][4][tid] = ra1.x; As[buf][5][tid] = ra1.y; As[buf][6][tid] = ra1.z; As[buf][7][tid] = ra1.w;
    *reinterpret_cast<uint4 *>(&Xs[buf][tid >> 1][4 * (tid & 1)]) = rx;
    __syncthreads();
    if (c + 1 < nchunks) {  // prefetch the next chunk while this one is consumed
      const int o = (c + 1) * kGemmKTile;
      ra0 = *reinterpret_cast<const uint4 *>(Arow + o);
      ra1 = *reinterpret_cast<const uint4 *>(Arow + o + 4);
      rx = *reinterpret_cast<const uint4 *>(Xrow + o);
    }
#pragma unroll
    for (int kk = 0; kk < kGemmKTile; kk += 4) {
      uint32_t a[4][4];
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int g = 0; g < 4; g++) a[q][g] = As[buf][kk + q][lane + 32 * g];
#pragma unroll
      for (int j = 0; j < POPC_OPS_PER_WARP; j++) {
        const uint4 x = *reinterpret_cast<const uint4 *>(&Xs[buf][warp * POPC_OPS_PER_WARP + j][kk]);
#pragma unroll
        for (int g = 0; g < 4; g++) acc[g][j] ^= (a[0][g] & x.x) ^ (a[1][g] & x.y) ^ (a[2][g] & x.z) ^ (a[3][g] & x.w);
      }
    }
  }
  // epilogue: one ballot per (row group, request)
  uint32_t mine[4] = {0, 0, 0, 0};
#pragma unroll
  for (int g = 0; g < 4; g++)
#pragma unroll
    for (int j = 0; j < POPC_OPS_PER_WARP; j++) {
      uint32_t w = __ballot_sync(0xffffffffu, __popc(acc[g][j]) & 1);
      if (lane == j) mine[g] = w;
    }
  if (lane < POPC_OPS_PER_WARP) {
    const long long op = op0 + warp * POPC_OPS_PER_WARP + lane;
    if (op < live_end) {
#pragma unroll
      for (int g = 0; g < 4; g++) {
        const int word = row0 / 32 + g;
        if (word < out_words) Out[op * ldo + word] = mine[g];
      }
    }
  }
}

Segs one_segment(long long n) {
  Segs s{};
  s.nseg = 1;
  s.row0[0] = 0;
  s.row0[1] = (n + kGemmOpPad - 1) / kGemmOpPad * kGemmOpPad;
  s.nreq[0] = n;
  return s;
}

cudaError_t launch_gf2_gemm_seg(int engine, const GemmKeys &keys, const Segs &segs, int lda, int rows_pad,
                                const uint32_t *X, int ldx, int kw_pad, uint32_t *Out, int ldo, int out_words,
                                int *err, cudaStream_t st) {
  const long long rows = seg_rows(segs);
  if (rows <= 0) return cudaSuccess;
  if (segs.nseg < 1 || segs.nseg > kMaxSegs || rows_pad % kGemmRowTile || kw_pad % kGemmKTile || lda % 4 ||
      ldx % 4 || lda < kw_pad || ldx < kw_pad)
    return cudaErrorInvalidValue;
  for (int i = 0; i <= segs.nseg; i++)
    if (segs.row0[i] % kGemmOpPad) return cudaErrorInvalidValue;
  switch (engine) {
    case GEMM_TC:
      return launch_gf2_gemm_tc(keys, segs, rows_pad, X, ldx, kw_pad, Out, ldo, out_words, err, st);
    case GEMM_B1MMA:
      return launch_gf2_gemm_b1(keys, segs, lda, rows_pad, X, ldx, kw_pad, Out, ldo, out_words, st);
    case GEMM_POPC:
    default: {
      dim3 grid((unsigned)(rows / kGemmOpTile), rows_pad / kGemmRowTile);
      gf2_gemm_popc<<<grid, POPC_THREADS, 0, st>>>(keys, segs, lda, X, ldx, kw_pad, Out, ldo, out_words);
      return cudaGetLastError();
    }
  }
}

cudaError_t launch_gf2_gemm(int engine, const uint32_t *A, const uint8_t *A8, int lda, int rows_pad,
                            const uint32_t *X, int ldx, long long n_pad, int kw_pad, uint32_t *Out, int ldo,
                            int out_words, long long N, int *err, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  if (n_pad < N || n_pad % kGemmOpPad) return cudaErrorInvalidValue;
  GemmKeys keys{};
  keys.A[0] = A;
  keys.A8[0] = A8;
  Segs segs = one_segment(N);
  segs.row0[1] = n_pad;
  return launch_gf2_gemm_seg(engine, keys, segs, lda, rows_pad, X, ldx, kw_pad, Out, ldo, out_words, err, st);
}

}  // namespace gmc
