// Autotuner: per parameter set, times the candidate launch configurations on
// this GPU with a resident key pair and a batch of the requested size, keeps
// the fastest, and persists the choices in a JSON cache that later processes
// load with gmc_autotune_load.
//
// Candidates, tuned greedily in this order: the engine of the encapsulation
// syndrome (sparse column gather in the sampler, or the tcgen05 GEMM) crossed
// with the sampler's block size (32, 64, 128); the pipelined sampler's resident
// warps per SM (as many as fit, 16 or 8); the GEMM engine of the
// decapsulation front end (CUDA-core popcount or tcgen05); the tcgen05 GEMM's
// pipeline depth (2, 3 or 4 A/X stages per CTA, when either op uses that
// engine); and the requests per block of the two decoding kernels
// (Berlekamp-Massey: at most 14, 8 or 4 warps of 32 requests per block, fewer
// when the groups spread over every SM with fewer, timed only when the batch
// takes its bit-sliced form; root finding: 8, 4 or 2 warps of one request).
// The GEMM tile is fixed at 128 x 256 (one tcgen05 M=128 instruction shape
// and a TMEM accumulator pair) and K is never split: every CTA owns whole
// output tiles, so there is no split-K reduction to tune. A later candidate
// replaces the current choice only when it is more than 1% faster. Timing:
// CUDA events around whole batched calls (median of 5 after 2 warm-ups).
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gmc.h"
#include "engine_internal.h"
#include "host_keys.h"
#include "kernels.h"

using namespace gmc;

namespace {

const char *engine_name(int e) {
  return e == GEMM_SPARSE ? "sparse" : e == GEMM_TC ? "tc" : e == GEMM_B1MMA ? "b1mma" : "popc";
}
int engine_id(const std::string &s) {
  return s == "sparse" ? GEMM_SPARSE : s == "tc" ? GEMM_TC : s == "b1mma" ? GEMM_B1MMA : GEMM_POPC;
}

int tune_error(int code, const std::string &msg) {
  set_last_error(msg.c_str());
  return code;
}

__global__ void fill_bytes_kernel(uint8_t *p, long long n, uint32_t salt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    uint32_t x = (uint32_t)i * 2654435761u ^ salt;
    x ^= x >> 15;
    x *= 2246822519u;
    x ^= x >> 13;
    p[i] = (uint8_t)x;
  }
}

template <typename F>
float time_median(F fn, cudaStream_t st, cudaEvent_t a, cudaEvent_t b, int *rc) {
  for (int i = 0; i < 2; i++) *rc |= fn();
  std::vector<float> t;
  for (int i = 0; i < 5; i++) {
    cudaEventRecord(a, st);
    *rc |= fn();
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    t.push_back(ms);
  }
  std::sort(t.begin(), t.end());
  return t[t.size() / 2];
}

std::string read_file(const char *path) {
  std::ifstream f(path);
  if (!f) return "";
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

// value of "key": in the object text (string or number), "" if absent
std::string field(const std::string &obj, const char *key) {
  const std::string k = std::string("\"") + key + "\"";
  size_t p = obj.find(k);
  if (p == std::string::npos) return "";
  p = obj.find(':', p + k.size());
  if (p == std::string::npos) return "";
  p++;
  while (p < obj.size() && (obj[p] == ' ' || obj[p] == '"')) p++;
  size_t q = p;
  while (q < obj.size() && obj[q] != '"' && obj[q] != ',' && obj[q] != '}') q++;
  return obj.substr(p, q - p);
}

// the {...} object that follows "name": in text
std::string object_of(const std::string &text, const std::string &name) {
  size_t p = text.find("\"" + name + "\"");
  if (p == std::string::npos) return "";
  p = text.find('{', p);
  size_t q = text.find('}', p);
  if (p == std::string::npos || q == std::string::npos) return "";
  return text.substr(p, q - p + 1);
}

std::string set_entry(int set, const SetTune &t) {
  char buf[400];
  snprintf(buf, sizeof buf,
           "    \"%s\": {\"enc_engine\": \"%s\", \"dec_engine\": \"%s\", \"sample_threads\": %d, "
           "\"sample_sm_warps\": %d, \"gemm_stages\": %d, \"bm_warps\": %d, \"root_warps\": %d, \"n\": %lld, "
           "\"enc_ms\": %.4f, \"dec_ms\": %.4f}",
           set_info(set).name, engine_name(t.enc_engine), engine_name(t.dec_engine), t.sample_threads,
           t.sample_sm_warps, t.gemm_stages, t.bm_warps, t.root_warps, t.n, t.enc_ms, t.dec_ms);
  return buf;
}

int write_cache(const char *path) {
  cudaDeviceProp prop{};
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&prop, dev);
  // keep entries of sets tuned by an earlier run that this process did not tune
  const std::string old = read_file(path);
  std::string out = std::string("{\n  \"gpu\": \"") + prop.name + "\",\n  \"sets\": {\n";
  bool first = true;
  for (int s = 0; s < GMC_NSETS; s++) {
    SetTune t = tune_get(s);
    std::string entry;
    if (t.tuned) {
      entry = set_entry(s, t);
    } else {
      const std::string o = object_of(old, set_info(s).name);
      if (o.empty()) continue;
      entry = "    \"" + std::string(set_info(s).name) + "\": " + o;
    }
    out += (first ? "" : ",\n") + entry;
    first = false;
  }
  out += "\n  }\n}\n";
  std::ofstream f(path);
  if (!f) return tune_error(GMC_EINVAL, std::string("gmc_autotune: cannot write ") + path);
  f << out;
  return GMC_OK;
}

}  // namespace

extern "C" int gmc_tune_set(int set, int enc_engine, int dec_engine, int sample_threads) {
  if (set < 0 || set >= GMC_NSETS || enc_engine < 0 || enc_engine > GEMM_SPARSE || dec_engine < 0 ||
      dec_engine > GEMM_TC || (sample_threads != 32 && sample_threads != 64 && sample_threads != 128))
    return tune_error(GMC_EINVAL, "gmc_tune_set: bad argument");
  SetTune t = tune_get(set);
  t.enc_engine = enc_engine;
  t.dec_engine = dec_engine;
  t.sample_threads = sample_threads;
  tune_put(set, t);
  return GMC_OK;
}

extern "C" int gmc_tune_set_launch(int set, int gemm_stages, int bm_warps, int root_warps, int sample_sm_warps) {
  if (set < 0 || set >= GMC_NSETS || gemm_stages < 2 || gemm_stages > kTcStages || bm_warps < 1 ||
      bm_warps > kBMWarps || root_warps < 1 || root_warps > kRootWarps || sample_sm_warps < 0 ||
      sample_sm_warps > 64)
    return tune_error(GMC_EINVAL, "gmc_tune_set_launch: bad argument");
  SetTune t = tune_get(set);
  t.gemm_stages = gemm_stages;
  t.bm_warps = bm_warps;
  t.root_warps = root_warps;
  t.sample_sm_warps = sample_sm_warps;
  tune_put(set, t);
  return GMC_OK;
}

extern "C" int gmc_tune_get_launch(int set, int *gemm_stages, int *bm_warps, int *root_warps, int *sample_sm_warps) {
  if (set < 0 || set >= GMC_NSETS) return tune_error(GMC_EINVAL, "gmc_tune_get_launch: bad set");
  SetTune t = tune_get(set);
  if (gemm_stages) *gemm_stages = t.gemm_stages;
  if (bm_warps) *bm_warps = t.bm_warps;
  if (root_warps) *root_warps = t.root_warps;
  if (sample_sm_warps) *sample_sm_warps = t.sample_sm_warps;
  return t.tuned;
}

extern "C" int gmc_tune_get(int set, int *enc_engine, int *dec_engine, int *sample_threads) {
  if (set < 0 || set >= GMC_NSETS) return tune_error(GMC_EINVAL, "gmc_tune_get: bad set");
  SetTune t = tune_get(set);
  if (enc_engine) *enc_engine = t.enc_engine;
  if (dec_engine) *dec_engine = t.dec_engine;
  if (sample_threads) *sample_threads = t.sample_threads;
  return t.tuned;
}

extern "C" int gmc_autotune(int set, long long n, const char *cache_path) {
  if (set < 0 || set >= GMC_NSETS || n <= 0) return tune_error(GMC_EINVAL, "gmc_autotune: bad argument");
  const gmc_setinfo &S = set_info(set);
  std::vector<uint8_t> pk(S.pk_bytes), sk(S.sk_bytes);
  uint8_t seed[32];
  for (int i = 0; i < 32; i++) seed[i] = (uint8_t)(0xA5 ^ i);
  int r = gmc_keypair_seed(set, pk.data(), sk.data(), seed);
  if (r) return r;
  gmc_key *P = nullptr, *K = nullptr;
  if ((r = gmc_pk_load(&P, set, pk.data())) || (r = gmc_sk_load(&K, set, sk.data()))) {
    gmc_key_free(P);
    return r;
  }
  const int override_engine = gmc_get_gemm_engine();
  gmc_set_gemm_engine(-1);  // measure the per-set choices, not a global override
  uint8_t *seeds = nullptr, *ct = nullptr, *key = nullptr, *key2 = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaMalloc(&seeds, n * 32);
  if (e == cudaSuccess) e = cudaMalloc(&ct, n * S.synd_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&key, n * 32);
  if (e == cudaSuccess) e = cudaMalloc(&key2, n * 32);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  int rc = 0;
  SetTune best = tune_get(set);
  if (e == cudaSuccess) {
    fill_bytes_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(seeds, n * 32, 0x1234u + set);
    float best_enc = 1e30f, best_dec = 1e30f;
    const int enc_engines[2] = {GEMM_SPARSE, GEMM_TC};
    const int engines[2] = {GEMM_POPC, GEMM_TC};
    const int threads[3] = {32, 64, 128};
    for (int ei = 0; ei < 2; ei++)
      for (int ti = 0; ti < 3; ti++) {
        SetTune t = best;
        t.enc_engine = enc_engines[ei];
        t.sample_threads = threads[ti];
        tune_put(set, t);
        const float ms =
            time_median([&] { return gmc_enc_batch_dev(P, ct, key, seeds, n, nullptr, st); }, st, a, b, &rc);
        if (ms < best_enc) {
          best_enc = ms;
          best.enc_engine = enc_engines[ei];
          best.sample_threads = threads[ti];
        }
      }
    // resident warps per SM of the pipelined sampler (0: as many as fit)
    const int smw[3] = {0, 16, 8};
    for (int wi = 1; wi < 3; wi++) {
      SetTune t = best;
      t.sample_sm_warps = smw[wi];
      tune_put(set, t);
      const float ms =
          time_median([&] { return gmc_enc_batch_dev(P, ct, key, seeds, n, nullptr, st); }, st, a, b, &rc);
      if (ms < 0.99f * best_enc) {
        best_enc = ms;
        best.sample_sm_warps = smw[wi];
      }
    }
    tune_put(set, best);
    rc |= gmc_enc_batch_dev(P, ct, key, seeds, n, nullptr, st);  // valid ciphertexts for the dec timing
    for (int ei = 0; ei < 2; ei++) {
      SetTune t = best;
      t.dec_engine = engines[ei];
      tune_put(set, t);
      const float ms = time_median([&] { return gmc_dec_batch_dev(K, key2, ct, n, nullptr, st); }, st, a, b, &rc);
      if (ms < best_dec) {
        best_dec = ms;
        best.dec_engine = engines[ei];
      }
    }
    auto time_dec = [&](const SetTune &t) {
      tune_put(set, t);
      return time_median([&] { return gmc_dec_batch_dev(K, key2, ct, n, nullptr, st); }, st, a, b, &rc);
    };
    // pipeline depth of the tcgen05 GEMM (both ops share it)
    if (best.enc_engine == GEMM_TC || best.dec_engine == GEMM_TC) {
      const int stage_cand[3] = {4, 3, 2};
      float best_sum = 1e30f;
      for (int si = 0; si < 3; si++) {
        SetTune t = best;
        t.gemm_stages = stage_cand[si];
        tune_put(set, t);
        const float me =
            best.enc_engine == GEMM_TC
                ? time_median([&] { return gmc_enc_batch_dev(P, ct, key, seeds, n, nullptr, st); }, st, a, b, &rc)
                : best_enc;
        const float md = best.dec_engine == GEMM_TC ? time_dec(t) : best_dec;
        if (si == 0 || me + md < 0.99f * best_sum) {
          best_sum = me + md;
          best.gemm_stages = stage_cand[si];
          best_enc = me;
          best_dec = md;
        }
      }
      tune_put(set, best);
      rc |= gmc_enc_batch_dev(P, ct, key, seeds, n, nullptr, st);  // the ciphertexts the dec timings read
    }
    // requests per block of the decoding kernels
    const int bm_cand[3] = {kBMWarps, 8, 4};
    const int warp_cand[3] = {kRootWarps, 4, 2};
    if (n >= kBMBitslicedMinRows)
      for (int wi = 1; wi < 3; wi++) {
        SetTune t = best;
        t.bm_warps = bm_cand[wi];
        const float ms = time_dec(t);
        if (ms < 0.99f * best_dec) {
          best_dec = ms;
          best.bm_warps = bm_cand[wi];
        }
      }
    for (int wi = 1; wi < 3; wi++) {
      SetTune t = best;
      t.root_warps = warp_cand[wi];
      const float ms = time_dec(t);
      if (ms < 0.99f * best_dec) {
        best_dec = ms;
        best.root_warps = warp_cand[wi];
      }
    }
    best.tuned = 1;
    best.enc_ms = best_enc;
    best.dec_ms = best_dec;
    best.n = n;
    tune_put(set, best);
    e = cudaStreamSynchronize(st);
  }
  cudaFree(seeds);
  cudaFree(ct);
  cudaFree(key);
  cudaFree(key2);
  if (st) cudaStreamDestroy(st);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  gmc_key_free(P);
  gmc_key_free(K);
  gmc_set_gemm_engine(override_engine);
  if (e != cudaSuccess) return tune_error(GMC_ECUDA, std::string("gmc_autotune: ") + cudaGetErrorString(e));
  if (rc) return tune_error(GMC_ECUDA, "gmc_autotune: a timed batch failed");
  if (gmc_tc_status() == 1) return tune_error(GMC_ECUDA, "gmc_autotune: tensor-core engine error word set");
  if (cache_path && *cache_path) return write_cache(cache_path);
  return GMC_OK;
}

extern "C" int gmc_autotune_load(const char *cache_path) {
  if (!cache_path) return tune_error(GMC_EINVAL, "gmc_autotune_load: null path");
  const std::string text = read_file(cache_path);
  if (text.empty()) return tune_error(GMC_EINVAL, std::string("gmc_autotune_load: cannot read ") + cache_path);
  int loaded = 0;
  for (int s = 0; s < GMC_NSETS; s++) {
    const std::string o = object_of(text, set_info(s).name);
    if (o.empty()) continue;
    SetTune t = tune_get(s);
    t.enc_engine = engine_id(field(o, "enc_engine"));
    t.dec_engine = engine_id(field(o, "dec_engine"));
    if (t.dec_engine == GEMM_SPARSE) t.dec_engine = GEMM_TC;  // no sparse form for the front end
    const int th = atoi(field(o, "sample_threads").c_str());
    t.sample_threads = (th == 32 || th == 64 || th == 128) ? th : 128;
    const int gs = atoi(field(o, "gemm_stages").c_str());
    t.gemm_stages = (gs >= 2 && gs <= kTcStages) ? gs : kTcStages;
    const int bw = atoi(field(o, "bm_warps").c_str()), rw = atoi(field(o, "root_warps").c_str());
    t.bm_warps = (bw >= 1 && bw <= kBMWarps) ? bw : kBMWarps;
    t.root_warps = (rw >= 1 && rw <= kRootWarps) ? rw : kRootWarps;
    const int sw = atoi(field(o, "sample_sm_warps").c_str());
    t.sample_sm_warps = (sw >= 0 && sw <= 64) ? sw : 0;
    t.n = atoll(field(o, "n").c_str());
    t.enc_ms = atof(field(o, "enc_ms").c_str());
    t.dec_ms = atof(field(o, "dec_ms").c_str());
    t.tuned = 1;
    tune_put(s, t);
    loaded++;
  }
  return loaded;
}
