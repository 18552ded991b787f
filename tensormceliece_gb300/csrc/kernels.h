// Kernel launchers of the engine (host-callable, templated per parameter set).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "params.h"

namespace gmc {

constexpr int kSampleWarpsPerSM = 8;     // sampler: resident warps per SM (lanes fetch requests)
constexpr int kSampleThreadsMax = 128;  // sampler block size is a launch parameter (32, 64 or 128)
// hash kernels (thread per request, one wave): 64-thread blocks spread a
// 65536-request launch as 6-7 blocks per SM (128-thread blocks: 3-4, so a
// third of the SMs carried a block more than the rest)
constexpr int kTailThreads = 64;
constexpr int kBMWarps = 14;    // Berlekamp-Massey kernel: default and largest warps per block (32 requests per warp)
constexpr int kBMCtWarps = 8;   // its constant-time form: largest warps per block
constexpr int kBMLatWarps = 28;  // Berlekamp-Massey latency form: largest warps per block (one request per warp)
constexpr long long kBMBitslicedMinRows = 24576;  // smaller batches take the latency form
constexpr int kRootWarps = 8;  // root-finding kernel: default and largest warps per block

// ---------------------------------------------------------------- segments
// A launch covers up to kMaxSegs segments (one key each) laid out back to back
// in "padded row" space: segment s owns rows [row0[s], row0[s+1]), its live
// requests are the first nreq[s] of them, row0[] are multiples of kGemmOpPad
// (so no GEMM tile straddles two keys). Rows past a segment's live count are
// never read from or written to caller buffers. A single-key batch of n
// requests is the one-segment case {row0 = {0, round_up(n, kGemmOpPad)}}.
constexpr int kMaxSegs = 16;
struct Segs {
  int nseg;
  long long row0[kMaxSegs + 1];
  long long nreq[kMaxSegs];
};
#ifdef __CUDACC__
__host__ __device__ inline long long seg_rows(const Segs &S) { return S.row0[S.nseg]; }
__device__ inline int seg_find(const Segs &S, long long row) {
  int s = 0;
#pragma unroll 1
  for (int i = 1; i < S.nseg; i++)
    if (row >= S.row0[i]) s = i;
  return s;
}
// segment of a row and whether it is a live request
__device__ inline bool seg_live(const Segs &S, long long row, int *seg) {
  const int s = seg_find(S, row);
  *seg = s;
  return row < S.row0[S.nseg] && row - S.row0[s] < S.nreq[s];
}
#endif

// GF(2) GEMM engines for Out[op] = parity(A[row] & X[op]) over KW words.
// GEMM_SPARSE is the encapsulation-only alternative: e has weight t, so
// T e[mt:n] is the XOR of the <= t columns of T at e's positions, gathered by
// the sampler from a column-major image of T (no GEMM launch).
enum GemmEngine { GEMM_POPC = 0, GEMM_B1MMA = 1, GEMM_TC = 2, GEMM_SPARSE = 3 };

// Tiling of every engine: A padded to a multiple of kGemmRowTile rows and X
// to a multiple of kGemmOpTile requests, K to a multiple of kGemmKTile words.
constexpr int kGemmRowTile = 128;
constexpr int kGemmOpTile = 64;
constexpr int kGemmKTile = 8;

// Request-operand buffers (X) are padded to a multiple of kGemmOpPad rows.
constexpr int kGemmOpPad = 256;

// tcgen05 engine tiling: the key's FP8 image is kept in slices of kTcM rows;
// a CTA tile is 128 requests x 2 kTcM key rows, kTcKB bits of K per pipeline
// stage (4 MMAs of K = 32), up to kTcStages stage buffers. kTcN is the N of
// the FP8 peak measurement (128 x 256 x 32, the engine's MMA shape).
constexpr int kTcM = 128;
constexpr int kTcN = 256;
constexpr int kTcKB = 128;
constexpr int kTcStages = 4;

// Key matrices of the segments of a GEMM launch (same shape for all: one set).
// A8: the key matrix pre-expanded to FP8 stage images (GEMM_TC only).
// TT: public keys only, the columns of T as rows of ldtt words (column k is
// zero, the target of positions below mt), for GEMM_SPARSE.
struct GemmKeys {
  const uint32_t *A[kMaxSegs];
  const uint8_t *A8[kMaxSegs];
  const uint32_t *TT[kMaxSegs];
  int ldtt;
  int tc_stages;  // tcgen05 engine pipeline depth (2, 3 or 4; 0 = default 4)
};
// Out rows follow X rows (padded row space). err: device word set to 1 when a
// tensor-core CTA gave up on a bounded wait.
cudaError_t launch_gf2_gemm_seg(int engine, const GemmKeys &keys, const Segs &segs, int lda, int rows_pad,
                                const uint32_t *X, int ldx, int kw_pad, uint32_t *Out, int ldo, int out_words,
                                int *err, cudaStream_t st);
// single-key form: X has n_pad rows (multiple of kGemmOpPad), N live requests
cudaError_t launch_gf2_gemm(int engine, const uint32_t *A, const uint8_t *A8, int lda, int rows_pad,
                            const uint32_t *X, int ldx, long long n_pad, int kw_pad, uint32_t *Out, int ldo,
                            int out_words, long long N, int *err, cudaStream_t st);
size_t tc_a8_bytes(int rows_pad, int kw_pad);
// measured MMA rate of the engine's tcgen05 instruction (FP8 E4M3, M = 128, N = 256, K = 32), MACs per second;
// err_dev: a device word set to 1 if a bounded wait expired
cudaError_t time_tc_f8_peak(double *mac_per_s, int *err_dev, cudaStream_t st);
// measured rate of the legacy mma.sync m8n8k128 .b1 AND.POPC (register operands), bit-MACs per second
cudaError_t time_b1_peak(double *mac_per_s, int *out_dev, cudaStream_t st);
cudaError_t launch_expand_a(const uint32_t *A, int lda, int rows_pad, int kw_pad, uint8_t *A8, cudaStream_t st);
cudaError_t launch_gf2_gemm_tc(const GemmKeys &keys, const Segs &segs, int rows_pad, const uint32_t *X, int ldx,
                               int kw_pad, uint32_t *Out, int ldo, int out_words, int *err, cudaStream_t st);
cudaError_t launch_gf2_gemm_b1(const GemmKeys &keys, const Segs &segs, int lda, int rows_pad, const uint32_t *X,
                               int ldx, int kw_pad, uint32_t *Out, int ldo, int out_words, cudaStream_t st);
Segs one_segment(long long n);

// Encapsulation: seeds / C / K rows in padded row space; E, Ens, S have
// seg_rows(segs) rows. pk_bad_mask bit s: segment s's public key has
// nonzero padding bits (6960119), its c and K are zeroed.
// TT (k + 1 rows of ldtt words, zeroed by the caller): row j = column j of T
// (mt bits); row k stays zero.
cudaError_t launch_transpose_pk(const uint32_t *T, int lda, int mt, int k, uint32_t *TT, int ldtt, cudaStream_t st);

// Dense mode (sparse == nullptr): writes E and Ens (e[mt:n] at bit 0, the
// GEMM operand). Sparse mode: writes E and S = T e[mt:n] (lds words per row)
// from sparse->TT, and not Ens.
// counter: 4 bytes of device scratch (zeroed here, on st) that nothing else
// touches until the sampler ends; the pipelines lend the first word of the
// buffer the sampler does not write (S in dense mode, Ens in sparse mode).
// sm_warps: resident warps per SM of the pipelined sampler (0 = as many as fit).
// mark (optional): called after each kernel with its stage name (profiling).
template <int SET>
cudaError_t launch_sample(const uint8_t *seeds, const Segs &segs, uint32_t *E, int lde, uint32_t *Ens, int ldx,
                          const GemmKeys *sparse, uint32_t *S, int lds, int threads, unsigned int *counter,
                          cudaStream_t st, int sm_warps = 0, void (*mark)(const char *, cudaStream_t) = nullptr);
// C rows: synd_bytes, or synd_bytes + 32 with plaintext confirmation (pc):
// C0 || SHAKE256(2 || e, 32), K = SHAKE256(1 || e || C0 || C1).
template <int SET>
cudaError_t launch_finalize(const uint32_t *E, int lde, const uint32_t *S, int lds, uint8_t *C, uint8_t *K,
                            const Segs &segs, uint32_t pk_bad_mask, bool pc, cudaStream_t st);

// Per-key decapsulation state on the device (built once per secret key).
struct DecKeyDev {
  const uint16_t *L;     // support element of each code position [n]
  const uint16_t *LL;    // log L_i (zero sentinel when L_i = 0) [n]
  const uint16_t *LW2;   // log of 1/g(L_i)^2 [n]
  const uint16_t *invL;  // code position of each field element, 0xFFFF off the support [2^m]
  const uint8_t *s;      // implicit-rejection string [n/8]
  const uint32_t *HT;    // first t syndromes of each unit error [n][ldh] (m bits per syndrome)
  int ldh;
  const uint32_t *cond;  // the sk's Benes control bits ((2m - 1) 2^(m-1) bits, as 32-bit words)
};

// Per-field / per-set device tables (shared by all keys of a set).
struct FieldDev {
  const uint16_t *gexp;   // [2q-1]
  const uint16_t *glog;   // [q]
  const uint16_t *fft_twist_log;  // concatenated per level l = 0..d-1: [2^(d-l)]
  const uint16_t *frob_lo;        // x^(2^d) for x < 2^d
  // bit-sliced over 32 chunks per word (bit k: chunk 32 h + k), plane b = bit b
  const uint32_t *fft_alpha_bs;   // [(2^d - 2^(d-l) + xh) * H + h][m]: alpha_{l, (c << (d-1-l)) + xh}
  const uint32_t *frob_hi_bs;     // [h][m]: (c 2^d)^(2^d)
  const uint16_t *zech;           // [q]: log(1 + g^k), zech[0] = 3q (zero)
  // [2^(d+1)][m]: for the twist constant c of each fft_twist_log entry, c x^i (i < m), so a product
  // with c needs no table indexed by the other factor (constant-time form); null where not built
  const uint16_t *fft_twist_cols = nullptr;
};

// Per-key decapsulation tables of the segments of a launch.
struct DecKeys {
  DecKeyDev k[kMaxSegs];
};

// Decapsulation: C / K / rc rows in padded row space; X, S2, Sig, E, ok have
// seg_rows(segs) rows.
// C rows of synd_bytes (+ 32 with pc); only C0 is packed.
template <int SET>
cudaError_t launch_pack_ct(const uint8_t *C, const Segs &segs, uint32_t *X, int ldx, bool pc, cudaStream_t st);
// Berlekamp-Massey: S2 (2t packed syndromes) -> Sig [N][2^fft_d] u16, the
// error locator's coefficients by degree (the leading x^t term is implicit
// when t = 2^fft_d).
// warps: warps per block of the bit-sliced form (1..kBMWarps; 0 = kBMWarps;
// the constant-time form takes at most kBMCtWarps).
// ct: the constant-time form (inversion-free, no tables, slot bounds from the
// iteration alone; the same locators).
template <int SET>
cudaError_t launch_dec_bm(const uint32_t *S2, int lds2, FieldDev fd, const Segs &segs, uint16_t *Sig,
                          cudaStream_t st, int warps = 0, bool ct = false);
// Root finding + weight + re-encryption check: Sig -> E (error vectors), ok.
// warps: warps per block (1..kRootWarps; 0 = kRootWarps), one request per warp.
// ct: the twist multiplies by table-free columns (needs fd.fft_twist_cols).
template <int SET>
cudaError_t launch_dec_root(const uint16_t *Sig, const uint32_t *S2, int lds2, const DecKeys &keys, FieldDev fd,
                            const Segs &segs, uint32_t *E, int lde, int *ok, cudaStream_t st, int warps = 0,
                            bool ct = false);
// Constant-time decapsulation, after launch_dec_root(ct = true) left the field-order error vectors in E and the
// BM-length flag in ok: the key's Benes network to code order (E in place, weight == t into ok), the dense product
// of the first-t syndrome matrices (htt: per segment A / A8, rows t m padded to kGemmRowTile, ct_htt_words(n)
// words) with E into S3, and ok &= (S3 == the first t m bits of S2). E rows: lde >= max(q/32, ct_htt_words(n)).
// S3 rows: lds3 >= ceil(t m / 32) words (the packed-ciphertext buffer is large enough).
constexpr int ct_htt_words(int n) { return ((n + 31) / 32 + kGemmKTile - 1) / kGemmKTile * kGemmKTile; }
template <int SET>
cudaError_t launch_dec_ct_finish(const DecKeys &keys, const GemmKeys &htt, int engine, const Segs &segs, uint32_t *E,
                                 int lde, const uint32_t *S2, int lds2, uint32_t *S3, int lds3, int *ok, int *err,
                                 cudaStream_t st);
// HT (n rows of ldh words) -> HTT ((t m padded to kGemmRowTile) rows x ct_htt_words(n) words), once per key
cudaError_t launch_ct_htt(const uint32_t *HT, int ldh, int n, int tm, uint32_t *HTT, cudaStream_t st);
// With pc the decoded e must also give SHAKE256(2 || e, 32) = C1 (else implicit
// rejection), and the session-key preimage covers C0 || C1.
template <int SET>
cudaError_t launch_dec_tail(const uint32_t *E, int lde, const int *ok, const uint8_t *C, const DecKeys &keys,
                            uint8_t *K, int *rc, const Segs &segs, bool pc, cudaStream_t st);

}  // namespace gmc
