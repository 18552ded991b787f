// Parameter sets of Classic McEliece as used by libmceliece-20250507
// (reference: mceliece-gpu-params/ref/<set>.cuh:5-18, params.h/gf_params.h of
// each crypto_kem/<set>/vec directory in deps/libmceliece-20250507.tar.gz).
#pragma once
#include <stdint.h>

#define GMC_NSETS 5
#define GMC_MAX_N 8192
#define GMC_MAX_T 128
#define GMC_MAX_M 13

// Host/device-visible description of one set; everything else is derived.
struct gmc_setinfo {
  int id;
  const char *name;
  int m, n, t;
  int mt, k, q;             // q = 2^m
  int pk_row_bytes;          // ceil(k/8)
  int synd_bytes;            // ct bytes = ceil(mt/8)
  int cond_bytes;            // Benes control bits
  int irr_bytes;             // 2t
  int e_bytes;               // n/8
  long long pk_bytes, sk_bytes;
  int fft_d;                 // FFT coefficient slots 2^fft_d
  int lead_term;             // 1 when the locator's x^t term is added separately (t = 2^fft_d)
};

#ifdef __CUDACC__
#define GMC_HD __host__ __device__
#else
#define GMC_HD
#endif

// Compile-time parameters for templated kernels.
template <int SET> struct Set;
template <> struct Set<0> { static constexpr int m = 12, n = 3488, t = 64; };
template <> struct Set<1> { static constexpr int m = 13, n = 4608, t = 96; };
template <> struct Set<2> { static constexpr int m = 13, n = 6688, t = 128; };
template <> struct Set<3> { static constexpr int m = 13, n = 6960, t = 119; };
template <> struct Set<4> { static constexpr int m = 13, n = 8192, t = 128; };

template <int SET> struct P {
  static constexpr int m = Set<SET>::m, n = Set<SET>::n, t = Set<SET>::t;
  static constexpr int mt = m * t;
  static constexpr int k = n - mt;
  static constexpr int q = 1 << m;
  static constexpr int synd_bytes = (mt + 7) / 8;
  static constexpr int pk_row_bytes = (k + 7) / 8;
  static constexpr int e_bytes = n / 8;
  static constexpr int ew = (n + 31) / 32;        // u32 words of e
  static constexpr int kw = (k + 31) / 32;        // u32 words of e[mt:n]
  static constexpr int mw = (mt + 31) / 32;       // u32 words of a syndrome
  static constexpr int cw = (synd_bytes + 3) / 4; // u32 words of a ciphertext
  static constexpr int s2w = (2 * t * m + 31) / 32; // u32 words of 2t packed syndromes
  static constexpr bool full = (n == q);          // n = 2^m: no range filter in sampling
  static constexpr int cand_bytes = full ? 2 * t : 4 * t;
  static constexpr int fft_d = (t <= 64) ? 6 : 7;
  static constexpr bool lead = (t == (1 << fft_d));
  static constexpr int pre_bytes = 1 + e_bytes + synd_bytes; // hash preimage
};
