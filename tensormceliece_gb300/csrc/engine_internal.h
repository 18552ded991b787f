// Internal layout of a resident key handle, shared by the engine's
// translation units (not part of the C ABI).
#pragma once
#include <stdint.h>

#include <mutex>

#include "kernels.h"

struct gmc_key {
  int set = 0;     // parameter set 0..4
  int pc = 0;      // plaintext-confirmation variant: ciphertexts C0 || SHAKE256(2 || e, 32)
  int variant = 0; // public id = set + GMC_NSETS * variant (0 plain, 1 pc, 2 f, 3 pcf)
  int kind = 0;  // 0 public, 1 secret
  int device = 0;
  // public key
  uint32_t *T = nullptr;
  uint32_t *TT = nullptr;  // columns of T (sparse syndrome)
  int lda = 0, rows_pad = 0, kw_pad = 0, pad_bad = 0, ldtt = 0;
  // secret key
  uint32_t *F = nullptr;
  int ldf = 0, frows_pad = 0, cw_pad = 0;
  uint16_t *tabs = nullptr;  // L | LL | LW2 (n each) | invL (2^m)
  uint8_t *a8 = nullptr;     // FP8 stage images of T (public) or F (secret) for the tensor-core engine
  std::mutex *a8_mu = nullptr;
  uint8_t *s = nullptr;
  uint32_t *HT = nullptr;  // first t syndromes per code position (re-encryption check)
  uint32_t *cond = nullptr;  // the sk's Benes control bits (constant-time decapsulation)
  // constant-time decapsulation, built on first use: the first-t syndrome matrix (t m rows x n bits) and its
  // FP8 stage image for the tensor-core engine (under a8_mu)
  uint32_t *htt = nullptr;
  uint8_t *htt8 = nullptr;
  gmc::DecKeyDev dk{};
};


namespace gmc {
// sets the calling thread's message returned by gmc_last_error()
void set_last_error(const char *msg);
// the constant-time decapsulation switch (gmc_set_dec_constant_time)
bool dec_constant_time();

// per-parameter-set launch configuration chosen by the autotuner
struct SetTune {
  int enc_engine = GEMM_SPARSE;  // engine of the encapsulation syndrome
  int dec_engine = GEMM_TC;   // GF(2) GEMM engine of the decapsulation front end
  int sample_threads = 128;   // sampler block size (32, 64 or 128)
  int gemm_stages = 4;        // tcgen05 GEMM pipeline depth (2, 3 or 4 A/X buffers per CTA)
  int bm_warps = kBMWarps;    // Berlekamp-Massey (bit-sliced form) warps per block: 32 requests each
  int root_warps = 8;         // root-finding warps per block: one request each
  int sample_sm_warps = 0;    // pipelined sampler: resident warps per SM (0 = as many as fit)
  int tuned = 0;              // 1 when measured on this device
  double enc_ms = 0, dec_ms = 0;
  long long n = 0;
};
SetTune tune_get(int set);
void tune_put(int set, const SetTune &t);

// device word of the tensor-core engine's bounded waits (allocated on first use)
int *tc_err_word_ptr();
// per-set field / FFT tables of the current device (built on first use)
int field_tables(int set, FieldDev *out);
// builds everything a key needs resident on the device for any engine choice
// (FP8 image of its matrix, per-set tables), so later launches allocate nothing for it
int key_prepare_resident(const gmc_key *key);
// GEMM operands of the constant-time check (the keys' first-t syndrome matrices), built on first use
cudaError_t ct_gemm_keys(const gmc_key *const *keys, int nkeys, int engine, cudaStream_t st, GemmKeys *gk);
// decapsulation rows of the error-vector buffer: the table form needs ceil(n/32) words, the constant-time form
// the field-order vector (q/32 words) and the check product's K (ct_htt_words(n))
int dec_e_words(int set, bool ct);
}  // namespace gmc
