// Host-side per-key and per-field setup for the GPU engine: everything here
// runs once per loaded key (or once per field), never per request.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <vector>
#include "params.h"

namespace gmc {

const gmc_setinfo &set_info(int set);

// GF(2^m) with log/antilog tables in the device layout: exp has 2q-1 entries
// (exp[2q-2] = 0), log[0] = 2q-2 (sentinel), so a*b = exp[min(la+lb, 2q-2)].
struct HostField {
  int m = 0, q = 0;
  uint32_t poly = 0;
  std::vector<uint16_t> exp, log;
  void init(int m_);
  uint16_t mul(uint16_t a, uint16_t b) const;
  uint16_t inv(uint16_t a) const;
  uint16_t sq(uint16_t a) const { return mul(a, a); }
  int zero_log() const { return 2 * q - 2; }
};
const HostField &host_field(int m);

// Additive-FFT constants for (m, d): per level l the log of the first basis
// element's powers (twist) and of the butterfly constants alpha_{l,c'}.
struct FftTables {
  std::vector<uint16_t> twist_log;  // levels concatenated, 2^(d-l) each (2^(d+1) total)
  std::vector<uint16_t> twist_cols; // [2^(d+1)][m]: c x^i for the constant c of each twist_log entry
  std::vector<uint16_t> alpha_log;  // levels concatenated, 2^(m-l-1) each (padded to 2^m)
  std::vector<uint16_t> frob_lo;    // x^(2^d), x < 2^d
  std::vector<uint16_t> frob_hi;    // (c 2^d)^(2^d), c < 2^(m-d)
  // Bit-sliced copies for the chunked bottom-up pass, where bit k of a 32-bit
  // word belongs to chunk c = 32 h + k (h < 2^(m-d) / 32) and plane b holds
  // bit b of the field element. Stored as u32 words split into (low, high)
  // u16 halves so they travel in the u16 table buffers.
  //   alpha_bs[((2^d - 2^(d-l) + xh) * H + h) * m + b]: alpha_{l, (c << (d-1-l)) + xh}, xh < 2^(d-1-l)
  //   frob_hi_bs[h * m + b]: frob_hi[c]
  std::vector<uint16_t> alpha_bs;
  std::vector<uint16_t> frob_hi_bs;
  // Zech logarithms: zech[k] = log(1 + g^k) for 0 < k < q-1; zech[0] (1 + 1 = 0)
  // is 3q, a log at or above the zero sentinel 2q-2 that stays below 2^16
  // after adding any log < q-1 and reducing once by q-1.
  std::vector<uint16_t> zech;
};
FftTables build_fft_tables(int m, int d);

// Public key -> row-major T words for the syndrome GEMM.
struct PkHost {
  std::vector<uint32_t> T;   // rows_pad x lda
  int lda = 0, rows_pad = 0, kw_pad = 0;
  int ldtt = 0;              // row stride of the column image TT (built on the device)
  int pad_bad = 0;          // 6960119: nonzero pk padding bits
};
void build_pk(int set, const uint8_t *pk, PkHost &out);

// Secret key -> support, logs, front-end matrix F.
struct SkHost {
  std::vector<uint16_t> L, LL, LW2, Lpow;   // [n]
  std::vector<uint16_t> invL;               // [2^m]: position of each field element, 0xFFFF if none
  std::vector<uint8_t> s;                   // [n/8]
  std::vector<uint32_t> F;                  // frows_pad x ldf
  int ldf = 0, frows_pad = 0, cw_pad = 0;
  // per code position i: the first t syndromes of the unit error at i,
  // w2_i L_i^j (j < t), packed m bits each like the received syndromes
  std::vector<uint32_t> HT;                 // n x ldh
  int ldh = 0;
};
int build_sk(int set, const uint8_t *sk, SkHost &out);

// SHAKE256 on the host (the checksum of exported key strings, keyfile.cu)
void host_shake256(uint8_t *out, size_t outlen, const uint8_t *in, size_t inlen);

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace gmc
