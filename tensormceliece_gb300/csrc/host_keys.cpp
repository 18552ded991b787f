// Host-side per-key setup (run once per loaded key).
//
// Secret-key layout (mc:crypto_kem/348864/vec/kem_keypair.c:20-100, all five
// sets): delta(32) | pivots(8) | g_0..g_{t-1} (2 bytes LE each) |
// Benes control bits ((2m-1) 2^(m-1) bits) | s (n/8 bytes).
// The support element of code position i is bitrev_m(pi(i)) where pi is the
// permutation the control bits encode (support_gen in the reference library;
// device port mceliece-gpu-params/ref/348864.cuh:2553-2649, benes).
#include "host_keys.h"
#include "kernels.h"

#include <algorithm>
#include <cstring>
#include <atomic>
#include <functional>
#include <mutex>
#include <thread>

namespace gmc {

static const gmc_setinfo kSets[GMC_NSETS] = {
    {0, "348864", 12, 3488, 64, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {1, "460896", 13, 4608, 96, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {2, "6688128", 13, 6688, 128, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {3, "6960119", 13, 6960, 119, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {4, "8192128", 13, 8192, 128, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
};

const gmc_setinfo &set_info(int set) {
  static gmc_setinfo filled[GMC_NSETS];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int i = 0; i < GMC_NSETS; i++) {
      gmc_setinfo s = kSets[i];
      s.mt = s.m * s.t;
      s.k = s.n - s.mt;
      s.q = 1 << s.m;
      s.pk_row_bytes = (s.k + 7) / 8;
      s.synd_bytes = (s.mt + 7) / 8;
      s.cond_bytes = (1 << (s.m - 4)) * (2 * s.m - 1);
      s.irr_bytes = 2 * s.t;
      s.e_bytes = s.n / 8;
      s.pk_bytes = (long long)s.mt * s.pk_row_bytes;
      s.sk_bytes = 40 + s.irr_bytes + s.cond_bytes + s.e_bytes;
      s.fft_d = s.t <= 64 ? 6 : 7;
      s.lead_term = (s.t == (1 << s.fft_d));
      filled[i] = s;
    }
  });
  return filled[set];
}

// ---------------------------------------------------------------- field
static uint16_t clmul_mod(uint32_t a, uint32_t b, int m, uint32_t poly) {
  uint32_t acc = 0;
  for (int i = 0; i < m; i++)
    if ((b >> i) & 1) acc ^= a << i;
  for (int i = 2 * m - 2; i >= m; i--)
    if ((acc >> i) & 1) acc ^= poly << (i - m);
  return (uint16_t)acc;
}

void HostField::init(int m_) {
  m = m_;
  q = 1 << m;
  // field polynomials of the Classic McEliece sets: x^12+x^3+1, x^13+x^4+x^3+x+1
  poly = (m == 12) ? 0x1009u : 0x201Bu;
  exp.assign(2 * q - 1, 0);
  log.assign(q, 0);
  for (uint32_t g = 2; g < (uint32_t)q; g++) {
    uint32_t x = 1;
    int order = 0;
    do {
      x = clmul_mod(x, g, m, poly);
      order++;
    } while (x != 1 && order < q);
    if (order != q - 1) continue;
    x = 1;
    for (int i = 0; i < q - 1; i++) {
      exp[i] = (uint16_t)x;
      log[x] = (uint16_t)i;
      x = clmul_mod(x, g, m, poly);
    }
    for (int i = q - 1; i < 2 * q - 2; i++) exp[i] = exp[i - (q - 1)];
    exp[2 * q - 2] = 0;
    log[0] = (uint16_t)(2 * q - 2);
    return;
  }
}

uint16_t HostField::mul(uint16_t a, uint16_t b) const {
  int s = log[a] + log[b];
  if (s > 2 * q - 2) s = 2 * q - 2;
  return exp[s];
}

uint16_t HostField::inv(uint16_t a) const {
  if (!a) return 0;
  return exp[(q - 1 - log[a]) % (q - 1)];
}

const HostField &host_field(int m) {
  static HostField f12, f13;
  static std::once_flag once;
  std::call_once(once, [] {
    f12.init(12);
    f13.init(13);
  });
  return m == 12 ? f12 : f13;
}

// ---------------------------------------------------------------- FFT tables
// Gao-Mateer additive FFT over span(beta) with beta_i = 2^i (so the point
// with index c is the field element c). Level l: twist g(x) = f(b0 x), radix
// conversion at x^2+x; the next basis is delta_i^2 + delta_i with
// delta_i = beta_i / b0 (i >= 1). The butterfly constant for the pair with
// upper index c' is alpha = sum_{i>=1} bit_{i-1}(c') delta_i.
FftTables build_fft_tables(int m, int d) {
  const HostField &F = host_field(m);
  FftTables t;
  t.twist_log.assign(2 << d, 0);
  t.alpha_log.assign(1 << m, (uint16_t)F.zero_log());
  std::vector<uint16_t> beta(m);
  for (int i = 0; i < m; i++) beta[i] = (uint16_t)(1u << i);
  int toff = 0, aoff = 0;
  for (int l = 0; l < d; l++) {
    const int dim = m - l;  // basis size at this level
    const uint16_t b0 = beta[0];
    const int np = 1 << (d - l);
    uint16_t pw = 1;
    for (int i = 0; i < np; i++) {
      t.twist_log[toff + i] = F.log[pw];
      pw = F.mul(pw, b0);
    }
    toff += np;
    const uint16_t b0inv = F.inv(b0);
    std::vector<uint16_t> delta(dim);
    for (int i = 1; i < dim; i++) delta[i] = F.mul(beta[i], b0inv);
    const int na = 1 << (dim - 1);
    for (int c = 0; c < na; c++) {
      uint16_t a = 0;
      for (int i = 1; i < dim; i++)
        if ((c >> (i - 1)) & 1) a ^= delta[i];
      t.alpha_log[aoff + c] = F.log[a];
    }
    aoff += na;
    std::vector<uint16_t> nb(dim - 1);
    for (int i = 1; i < dim; i++) nb[i - 1] = (uint16_t)(F.sq(delta[i]) ^ delta[i]);
    beta = nb;
  }
  t.twist_cols.assign((size_t)(2 << d) * m, 0);
  for (int e = 0; e < (2 << d); e++)
    if (t.twist_log[e] < F.zero_log())
      for (int i = 0; i < m; i++) t.twist_cols[(size_t)e * m + i] = F.mul(F.exp[t.twist_log[e]], (uint16_t)(1u << i));
  auto frob = [&](uint16_t a) {
    for (int r = 0; r < d; r++) a = F.sq(a);
    return a;
  };
  t.frob_lo.resize(1 << d);
  for (int x = 0; x < (1 << d); x++) t.frob_lo[x] = frob((uint16_t)x);
  t.frob_hi.resize(1 << (m - d));
  for (int c = 0; c < (1 << (m - d)); c++) t.frob_hi[c] = frob((uint16_t)(c << d));

  t.zech.assign(1 << m, 0);
  t.zech[0] = (uint16_t)(3 << m);
  for (int k = 1; k < (1 << m) - 1; k++) t.zech[k] = F.log[1 ^ F.exp[k]];

  // bit-sliced forms: 32 chunks per word
  const int H = (1 << (m - d)) / 32;
  auto put_word = [](std::vector<uint16_t> &v, size_t w, uint32_t x) {
    v[2 * w] = (uint16_t)(x & 0xFFFFu);
    v[2 * w + 1] = (uint16_t)(x >> 16);
  };
  t.alpha_bs.assign((size_t)2 * ((1 << d) - 1) * H * m, 0);
  for (int l = 0, aoff = 0; l < d; aoff += 1 << (m - l - 1), l++)
    for (int xh = 0; xh < (1 << (d - 1 - l)); xh++)
      for (int h = 0; h < H; h++)
        for (int b = 0; b < m; b++) {
          uint32_t w = 0;
          for (int k = 0; k < 32; k++) {
            const int c = 32 * h + k;
            const uint16_t a = F.exp[t.alpha_log[aoff + (c << (d - 1 - l)) + xh]];
            w |= (uint32_t)((a >> b) & 1) << k;
          }
          put_word(t.alpha_bs, ((size_t)((1 << d) - (1 << (d - l)) + xh) * H + h) * m + b, w);
        }
  t.frob_hi_bs.assign((size_t)2 * H * m, 0);
  for (int h = 0; h < H; h++)
    for (int b = 0; b < m; b++) {
      uint32_t w = 0;
      for (int k = 0; k < 32; k++) w |= (uint32_t)((t.frob_hi[32 * h + k] >> b) & 1) << k;
      put_word(t.frob_hi_bs, (size_t)h * m + b, w);
    }
  return t;
}

// ---------------------------------------------------------------- public key
void build_pk(int set, const uint8_t *pk, PkHost &out) {
  const gmc_setinfo &S = set_info(set);
  const int kw = (S.k + 31) / 32;
  out.kw_pad = round_up(kw, kGemmKTile);
  out.lda = out.kw_pad;
  out.rows_pad = round_up(S.mt, kGemmRowTile);
  out.T.assign((size_t)out.rows_pad * out.lda, 0u);
  for (int r = 0; r < S.mt; r++) {
    const uint8_t *row = pk + (size_t)r * S.pk_row_bytes;
    uint32_t *dst = &out.T[(size_t)r * out.lda];
    for (int b = 0; b < S.pk_row_bytes; b++) dst[b >> 2] |= (uint32_t)row[b] << (8 * (b & 3));
  }
  out.ldtt = round_up((S.mt + 31) / 32, 32) < 64 ? 64 : round_up((S.mt + 31) / 32, 32);
  out.pad_bad = 0;
  if (S.k % 8) {
    uint8_t acc = 0;
    for (int r = 0; r < S.mt; r++) acc |= pk[(size_t)r * S.pk_row_bytes + S.pk_row_bytes - 1];
    out.pad_bad = (acc >> (S.k % 8)) != 0;
  }
}

// ---------------------------------------------------------------- secret key
static uint16_t bitrev(uint16_t a, int m) {
  uint16_t r = 0;
  for (int i = 0; i < m; i++) r |= (uint16_t)(((a >> i) & 1) << (m - 1 - i));
  return r;
}

int build_sk(int set, const uint8_t *sk, SkHost &out) {
  const gmc_setinfo &S = set_info(set);
  const HostField &F = host_field(S.m);
  const int q = S.q, m = S.m, t = S.t, n = S.n;
  std::vector<uint16_t> g(t + 1);
  for (int i = 0; i < t; i++) g[i] = (uint16_t)((sk[40 + 2 * i] | (sk[41 + 2 * i] << 8)) & (q - 1));
  g[t] = 1;
  // permutation encoded by the Benes control bits: layers of stride 2^0..2^(m-1)
  // then 2^(m-2)..2^0, conditional swaps in order, applied to the identity
  const uint8_t *cb = sk + 40 + S.irr_bytes;
  std::vector<int> pi(q);
  for (int i = 0; i < q; i++) pi[i] = i;
  auto layer = [&](int s, const uint8_t *bits) {
    const int stride = 1 << s;
    int idx = 0;
    for (int i = 0; i < q; i += 2 * stride)
      for (int j = 0; j < stride; j++, idx++)
        if ((bits[idx >> 3] >> (idx & 7)) & 1) std::swap(pi[i + j], pi[i + j + stride]);
  };
  for (int s = 0; s < m; s++) { layer(s, cb); cb += q >> 4; }
  for (int s = m - 2; s >= 0; s--) { layer(s, cb); cb += q >> 4; }

  out.L.resize(n); out.LL.resize(n); out.LW2.resize(n); out.Lpow.resize(n);
  out.invL.assign(q, 0xFFFF);
  std::vector<uint16_t> w2(n);
  const int d = S.fft_d;
  // per-position work split over host threads (positions, or 32-position word blocks where
  // threads would otherwise share a word)
  const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  auto parallel = [&](int count, const std::function<void(int, int)> &fn) {
    std::vector<std::thread> th;
    const int per = (count + nthreads - 1) / nthreads;
    for (int lo = 0; lo < count; lo += per) th.emplace_back(fn, lo, std::min(count, lo + per));
    for (auto &x : th) x.join();
  };
  std::atomic<int> bad{0};
  parallel(n, [&](int lo, int hi) {
    for (int i = lo; i < hi; i++) {
      const uint16_t a = bitrev((uint16_t)pi[i], m);
      uint16_t v = g[t];
      for (int j = t - 1; j >= 0; j--) v = (uint16_t)(F.mul(v, a) ^ g[j]);
      if (!v) bad = 1;  // g has a root on the support: not a valid key
      w2[i] = v ? F.inv(F.mul(v, v)) : 0;
      out.L[i] = a;
      out.LL[i] = F.log[a];
      out.LW2[i] = F.log[w2[i]];
      uint16_t pw = a;
      for (int r = 0; r < d; r++) pw = F.sq(pw);
      out.Lpow[i] = S.lead_term ? pw : 0;
    }
  });
  if (bad) return -1;
  for (int i = 0; i < n; i++) out.invL[out.L[i]] = (uint16_t)i;
  out.s.assign(sk + 40 + S.irr_bytes + S.cond_bytes, sk + 40 + S.irr_bytes + S.cond_bytes + S.e_bytes);

  // front-end matrix: row j*m+b, column i = bit b of w2_i * L_i^j, for every
  // ciphertext bit i (the 6960119 padding bits sit at code positions
  // mt..8*ct_bytes-1 and enter the syndrome as received bits, as in the
  // library's decrypt, mc:crypto_kem/6960119/vec/decrypt.c, preprocess)
  const int cw = (S.synd_bytes + 3) / 4;
  out.cw_pad = round_up(cw, kGemmKTile);
  out.ldf = out.cw_pad;
  out.frows_pad = round_up(2 * t * m, kGemmRowTile);
  out.F.assign((size_t)out.frows_pad * out.ldf, 0u);
  out.ldh = round_up((t * m + 31) / 32, 32);
  out.HT.assign((size_t)n * out.ldh, 0u);
  // HT row i: the m-bit values w2_i L_i^j, j < t, packed m bits apart
  parallel(n, [&](int lo, int hi) {
    for (int i = lo; i < hi; i++) {
      uint16_t v = w2[i];
      uint32_t *row = &out.HT[(size_t)i * out.ldh];
      for (int j = 0; j < t; j++) {
        const int pos = j * m, w = pos >> 5, sh = pos & 31;
        row[w] |= (uint32_t)v << sh;
        if (sh + m > 32) row[w + 1] |= (uint32_t)v >> (32 - sh);
        v = F.mul(v, out.L[i]);
      }
    }
  });
  const int ncols = std::min(n, 8 * S.synd_bytes);
  parallel((ncols + 31) / 32, [&](int lo, int hi) {
    for (int word = lo; word < hi; word++)
      for (int i = 32 * word; i < std::min(ncols, 32 * word + 32); i++) {
        uint16_t v = w2[i];
        const uint32_t bit = 1u << (i & 31);
        for (int j = 0; j < 2 * t; j++) {
          for (int b = 0; b < m; b++)
            if ((v >> b) & 1) out.F[(size_t)(j * m + b) * out.ldf + word] |= bit;
          v = F.mul(v, out.L[i]);
        }
      }
  });
  return 0;
}

}  // namespace gmc
