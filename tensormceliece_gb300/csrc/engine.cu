// Engine: resident keys, per-batch launch sequences, and the C ABI of gmc.h.
//
// Encapsulation of n requests (one public key):
//   sample (n threads)            seeds -> e (n bits), e[mt:n] (GEMM operand)
//   gf2_gemm (T x e[mt:n])        -> raw syndromes
//   finalize (n threads)          c = e[0:mt] ^ syndrome, K = H(1,e,c)
// Decapsulation of n ciphertexts (one secret key):
//   pack_ct                       ct bytes -> words
//   gf2_gemm (F x c)              -> 2t syndromes of the Goppa code
//   decode (one warp per request) BM, additive FFT, error, re-encryption check
//   dec_tail (n threads)          K = H(b, e or s, c)
// Reference flow: mceliece-gpu-params/main.cu:228-239 (encaps), 352-370 (decaps).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/random.h>

#include <atomic>
#include <list>
#include <map>
#include <memory>
#include <set>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gmc.h"
#include "engine_internal.h"
#include "host_keys.h"
#include "kernels.h"

using namespace gmc;

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;
static int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
static int cuda_fail(cudaError_t e, const char *where) {
  return fail(GMC_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define GMC_CUDA(call)                                   \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);  \
  } while (0)

extern "C" const char *gmc_last_error(void) { return g_last_error.c_str(); }
void gmc::set_last_error(const char *msg) { g_last_error = msg; }

// ---------------------------------------------------------------- keys
// (struct gmc_key: engine_internal.h)

// Per-set launch configuration (autotuned, see gmc_autotune) and an optional
// global GEMM-engine override (gmc_set_gemm_engine).
static SetTune g_tune[GMC_NSETS];
static int g_engine_override = -1;
// constant-time decapsulation kernels (gmc_set_dec_constant_time; GMC_DEC_CT=1)
static std::atomic<int> g_dec_ct{[] {
  const char *v = getenv("GMC_DEC_CT");
  return (v && v[0] == '1') ? 1 : 0;
}()};
bool gmc::dec_constant_time() { return g_dec_ct.load(std::memory_order_relaxed) != 0; }
static std::mutex g_tune_mu;
// op 0: encapsulation syndrome, 1: decapsulation front end (no sparse form:
// c is dense), where a GEMM_SPARSE override leaves the per-set engine.
static int engine_for(int set, int op) {
  if (g_engine_override >= 0 && !(op && g_engine_override == GEMM_SPARSE)) return g_engine_override;
  return op ? g_tune[set].dec_engine : g_tune[set].enc_engine;
}
SetTune gmc::tune_get(int set) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return g_tune[set];
}
void gmc::tune_put(int set, const SetTune &t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[set] = t;
}

// ---------------------------------------------------------------- profiler
// Optional per-kernel timing: when enabled, an event is recorded on the
// launching stream before the first and after every kernel of a batch, and
// gmc_prof_report() turns consecutive pairs into per-kernel device times.
struct ProfMark {
  const char *name;  // kernel that ended at this event (nullptr: batch start)
  cudaEvent_t ev;
};
static std::mutex g_prof_mu;
static bool g_prof = false;
static std::vector<ProfMark> g_marks;

static void prof_mark(const char *name, cudaStream_t st) {
  if (!g_prof) return;
  cudaStreamCaptureStatus cs;
  if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) return;
  cudaEvent_t ev;
  if (cudaEventCreate(&ev) != cudaSuccess) return;
  cudaEventRecord(ev, st);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_marks.push_back({name, ev});
}

extern "C" int gmc_prof_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto &mk : g_marks) cudaEventDestroy(mk.ev);
  g_marks.clear();
  g_prof = on != 0;
  return GMC_OK;
}

extern "C" int gmc_prof_report(char *buf, int len) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  std::map<std::string, std::pair<int, double>> agg;
  std::vector<std::string> order;
  for (size_t i = 1; i < g_marks.size(); i++) {
    if (!g_marks[i].name) continue;
    if (cudaEventSynchronize(g_marks[i].ev) != cudaSuccess) return fail(GMC_ECUDA, "gmc_prof_report: sync");
    float ms = 0;
    if (cudaEventElapsedTime(&ms, g_marks[i - 1].ev, g_marks[i].ev) != cudaSuccess) continue;
    std::string nm = g_marks[i].name;
    if (!agg.count(nm)) order.push_back(nm);
    agg[nm].first += 1;
    agg[nm].second += ms;
  }
  std::string out;
  for (auto &nm : order) {
    char line[160];
    snprintf(line, sizeof line, "%s %d %.6f\n", nm.c_str(), agg[nm].first, agg[nm].second);
    out += line;
  }
  if (buf && len > 0) {
    strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)order.size();
}

// per (device, set) field and FFT tables
struct FieldEntry {
  uint16_t *buf = nullptr;
  FieldDev fd{};
};
static std::mutex g_field_mu;
static std::map<std::pair<int, int>, FieldEntry> g_fields;

static int get_field(int set, FieldDev *out) {
  int dev = 0;
  GMC_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_field_mu);
  auto key = std::make_pair(dev, set);
  auto it = g_fields.find(key);
  if (it != g_fields.end()) {
    *out = it->second.fd;
    return GMC_OK;
  }
  const gmc_setinfo &S = set_info(set);
  const HostField &F = host_field(S.m);
  FftTables ft = build_fft_tables(S.m, S.fft_d);
  std::vector<uint16_t> all;
  // u16 tables, then the bit-sliced u32 tables at even (4-byte aligned) offsets
  auto put = [&](const std::vector<uint16_t> &v) {
    if (all.size() & 1) all.push_back(0);
    const size_t at = all.size();
    all.insert(all.end(), v.begin(), v.end());
    return at;
  };
  const size_t o_exp = put(F.exp), o_log = put(F.log), o_twist = put(ft.twist_log), o_frlo = put(ft.frob_lo),
               o_abs = put(ft.alpha_bs), o_fhbs = put(ft.frob_hi_bs), o_zech = put(ft.zech),
               o_tcols = put(ft.twist_cols);
  FieldEntry e;
  GMC_CUDA(cudaMalloc(&e.buf, all.size() * 2));
  GMC_CUDA(cudaMemcpy(e.buf, all.data(), all.size() * 2, cudaMemcpyHostToDevice));
  e.fd.gexp = e.buf + o_exp;
  e.fd.glog = e.buf + o_log;
  e.fd.fft_twist_log = e.buf + o_twist;
  e.fd.frob_lo = e.buf + o_frlo;
  e.fd.fft_alpha_bs = reinterpret_cast<const uint32_t *>(e.buf + o_abs);
  e.fd.frob_hi_bs = reinterpret_cast<const uint32_t *>(e.buf + o_fhbs);
  e.fd.zech = e.buf + o_zech;
  e.fd.fft_twist_cols = e.buf + o_tcols;
  g_fields[key] = e;
  *out = e.fd;
  return GMC_OK;
}

static bool valid_set(int set) { return set >= 0 && set < GMC_NSETS; }
// public set ids: s + GMC_NSETS v for parameter set s and variant v = 0 (the set), 1 pc
// (plaintext confirmation), 2 f (semi-systematic keys), 3 pcf
static bool valid_id(int id) { return id >= 0 && id < GMC_NVARIANTS; }
static int base_of(int id) { return id % GMC_NSETS; }
static int variant_of(int id) { return id / GMC_NSETS; }
static bool pc_of(int id) { return (variant_of(id) & 1) != 0; }
static bool semi_of(int id) { return (variant_of(id) & 2) != 0; }
static long long ct_bytes_of(int set, bool pc) { return set_info(set).synd_bytes + (pc ? 32 : 0); }
static long long ct_bytes_of(const gmc_key *k) { return ct_bytes_of(k->set, k->pc != 0); }

// Per-device error word of the tensor-core engine (a CTA that gave up on a
// bounded wait sets it to 1); gmc_tc_status() reads and clears it.
static std::mutex g_err_mu;
static std::map<int, int *> g_err_words;
static int *tc_err_word() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_err_mu);
  auto it = g_err_words.find(dev);
  if (it != g_err_words.end()) return it->second;
  int *w = nullptr;
  if (cudaMalloc(&w, sizeof(int)) != cudaSuccess) return nullptr;
  cudaMemset(w, 0, sizeof(int));
  g_err_words[dev] = w;
  return w;
}

extern "C" int gmc_tc_status(void) {
  int *w = tc_err_word();
  if (!w) return fail(GMC_ECUDA, "gmc_tc_status: no device");
  int v = 0;
  GMC_CUDA(cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost));
  GMC_CUDA(cudaMemset(w, 0, sizeof(int)));
  return v;
}

// FP8 stage images of the key matrix, built on first use by the tensor-core engine.
static cudaError_t key_a8(const gmc_key *kc, cudaStream_t st, const uint8_t **out) {
  gmc_key *k = const_cast<gmc_key *>(kc);
  std::lock_guard<std::mutex> lk(*k->a8_mu);
  if (!k->a8) {
    const uint32_t *A = k->kind == 0 ? k->T : k->F;
    const int lda = k->kind == 0 ? k->lda : k->ldf, rows = k->kind == 0 ? k->rows_pad : k->frows_pad;
    const int kw = k->kind == 0 ? k->kw_pad : k->cw_pad;
    uint8_t *p = nullptr;
    cudaError_t e = cudaMalloc(&p, tc_a8_bytes(rows, kw));
    if (e != cudaSuccess) return e;
    e = launch_expand_a(A, lda, rows, kw, p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaFree(p);
      return e;
    }
    k->a8 = p;
  }
  *out = k->a8;
  return cudaSuccess;
}


extern "C" int gmc_set_count(void) { return GMC_NSETS; }
static const char *const kVariantNames[GMC_NVARIANTS] = {
    "348864",    "460896",    "6688128",    "6960119",    "8192128",    "348864pc",  "460896pc",
    "6688128pc", "6960119pc", "8192128pc",  "348864f",    "460896f",    "6688128f",  "6960119f",
    "8192128f",  "348864pcf", "460896pcf",  "6688128pcf", "6960119pcf", "8192128pcf"};
extern "C" const char *gmc_set_name(int set) { return valid_id(set) ? kVariantNames[set] : nullptr; }
extern "C" int gmc_set_id(const char *name) {
  if (!name) return GMC_EINVAL;
  if (!strncmp(name, "mceliece", 8)) name += 8;
  for (int i = 0; i < GMC_NVARIANTS; i++)
    if (!strcmp(name, gmc_set_name(i))) return i;
  return GMC_EINVAL;
}
extern "C" int gmc_set_sizes(int set, long long *out) {
  if (!valid_id(set) || !out) return fail(GMC_EINVAL, "gmc_set_sizes: bad argument");
  const gmc_setinfo &S = set_info(base_of(set));
  out[0] = S.m; out[1] = S.n; out[2] = S.t; out[3] = S.mt; out[4] = S.k;
  out[5] = S.pk_bytes; out[6] = S.sk_bytes; out[7] = ct_bytes_of(base_of(set), pc_of(set));
  return GMC_OK;
}

extern "C" int gmc_pk_load(gmc_key **out, int id, const unsigned char *pk) {
  if (!out || !pk || !valid_id(id)) return fail(GMC_EINVAL, "gmc_pk_load: bad argument");
  const int set = base_of(id);
  *out = nullptr;
  PkHost h;
  build_pk(set, pk, h);
  gmc_key *k = new gmc_key();
  k->a8_mu = new std::mutex();
  k->set = set;
  k->pc = pc_of(id);
  k->variant = variant_of(id);
  k->kind = 0;
  cudaGetDevice(&k->device);
  k->lda = h.lda; k->rows_pad = h.rows_pad; k->kw_pad = h.kw_pad; k->pad_bad = h.pad_bad; k->ldtt = h.ldtt;
  const gmc_setinfo &S = set_info(set);
  const size_t tt_bytes = (size_t)(S.k + 1) * h.ldtt * 4;
  cudaError_t e = cudaMalloc(&k->T, h.T.size() * 4);
  if (e == cudaSuccess) e = cudaMalloc(&k->TT, tt_bytes);
  if (e == cudaSuccess) e = cudaMemcpy(k->T, h.T.data(), h.T.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(k->TT, 0, tt_bytes);
  if (e == cudaSuccess) e = launch_transpose_pk(k->T, k->lda, S.mt, S.k, k->TT, k->ldtt, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    cudaFree(k->T); cudaFree(k->TT);
    delete k->a8_mu;
    delete k;
    return cuda_fail(e, "gmc_pk_load");
  }
  *out = k;
  return GMC_OK;
}

extern "C" int gmc_sk_load(gmc_key **out, int id, const unsigned char *sk) {
  if (!out || !sk || !valid_id(id)) return fail(GMC_EINVAL, "gmc_sk_load: bad argument");
  const int set = base_of(id);
  *out = nullptr;
  SkHost h;
  if (build_sk(set, sk, h)) return fail(GMC_EKEY, "gmc_sk_load: Goppa polynomial vanishes on the support");
  const gmc_setinfo &S = set_info(set);
  gmc_key *k = new gmc_key();
  k->a8_mu = new std::mutex();
  k->set = set;
  k->pc = pc_of(id);
  k->variant = variant_of(id);
  k->kind = 1;
  cudaGetDevice(&k->device);
  k->ldf = h.ldf; k->frows_pad = h.frows_pad; k->cw_pad = h.cw_pad;
  const size_t n = S.n;
  cudaError_t e = cudaMalloc(&k->F, h.F.size() * 4);
  const size_t q = (size_t)S.q;
  if (e == cudaSuccess) e = cudaMalloc(&k->tabs, (3 * n + q) * 2);
  // s zero-padded to whole 16-byte units: the hash kernels read it as 32-bit words
  const size_t s_alloc = ((size_t)S.e_bytes + 15) / 16 * 16;
  if (e == cudaSuccess) e = cudaMalloc(&k->s, s_alloc);
  if (e == cudaSuccess) e = cudaMemset(k->s, 0, s_alloc);
  if (e == cudaSuccess) e = cudaMemcpy(k->F, h.F.data(), h.F.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(k->tabs, h.L.data(), n * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(k->tabs + n, h.LL.data(), n * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(k->tabs + 2 * n, h.LW2.data(), n * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(k->tabs + 3 * n, h.invL.data(), q * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(k->s, h.s.data(), S.e_bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&k->HT, h.HT.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(k->HT, h.HT.data(), h.HT.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&k->cond, S.cond_bytes);
  if (e == cudaSuccess) e = cudaMemcpy(k->cond, sk + 40 + S.irr_bytes, S.cond_bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(k->F); cudaFree(k->tabs); cudaFree(k->s); cudaFree(k->HT); cudaFree(k->cond);
    delete k->a8_mu;
    delete k;
    return cuda_fail(e, "gmc_sk_load");
  }
  k->dk.L = k->tabs;
  k->dk.LL = k->tabs + n;
  k->dk.LW2 = k->tabs + 2 * n;
  k->dk.invL = k->tabs + 3 * n;
  k->dk.s = k->s;
  k->dk.HT = k->HT;
  k->dk.ldh = h.ldh;
  k->dk.cond = k->cond;
  *out = k;
  return GMC_OK;
}

extern "C" void gmc_key_free(gmc_key *key) {
  if (!key) return;
  cudaFree(key->a8);
  delete key->a8_mu;
  cudaFree(key->T);
  cudaFree(key->TT);
  cudaFree(key->F);
  cudaFree(key->tabs);
  cudaFree(key->s);
  cudaFree(key->HT);
  cudaFree(key->cond);
  cudaFree(key->htt);
  cudaFree(key->htt8);
  delete key;
}

extern "C" int gmc_key_set(const gmc_key *key) { return key ? key->set + GMC_NSETS * key->variant : GMC_EINVAL; }

extern "C" int gmc_set_gemm_engine(int engine) {
  if (engine < -1 || engine > GEMM_SPARSE) return fail(GMC_EINVAL, "gmc_set_gemm_engine: unknown engine");
  g_engine_override = engine;
  return GMC_OK;
}
extern "C" int gmc_get_gemm_engine(void) { return g_engine_override; }

extern "C" int gmc_set_dec_constant_time(int on) {
  if (on != 0 && on != 1) return fail(GMC_EINVAL, "gmc_set_dec_constant_time: 0 or 1");
  g_dec_ct.store(on, std::memory_order_relaxed);
  return GMC_OK;
}
extern "C" int gmc_get_dec_constant_time(void) { return g_dec_ct.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------- workspace
// The default memory pool of the current device keeps freed blocks for reuse
// (release threshold raised once per device, for this process): without it
// the pool unmaps the batch scratch at every synchronization and the next
// batch maps it again.
static void keep_pool_warm() {
  static std::mutex mu;
  static std::set<int> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(mu);
  if (done.count(dev)) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done.insert(dev);
}

// Stream of the host-pointer batch calls: one per calling thread and device,
// created on first use (stream creation and destruction on every call cost
// tens of microseconds per call).
static cudaStream_t host_call_stream() {
  struct Holder {
    std::map<int, cudaStream_t> by_dev;
    ~Holder() {
      for (auto &kv : by_dev) cudaStreamDestroy(kv.second);
    }
  };
  thread_local Holder h;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  auto it = h.by_dev.find(dev);
  if (it != h.by_dev.end()) return it->second;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  h.by_dev[dev] = st;
  return st;
}

// Stream-ordered scratch: allocated from the device's default memory pool on
// the caller's stream and released on it after the last kernel.
struct Scratch {
  cudaStream_t st;
  std::vector<void *> ptrs;
  explicit Scratch(cudaStream_t s) : st(s) { keep_pool_warm(); }
  cudaError_t get(void **p, size_t bytes) {
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, st);
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
  ~Scratch() {
    for (void *p : ptrs) cudaFreeAsync(p, st);
  }
};

struct EncDims {
  int lde, ldx, lds;
  long long n_pad;
};
static EncDims enc_dims(int set, int kw_pad, long long rows) {
  const gmc_setinfo &S = set_info(set);
  EncDims d;
  d.lde = round_up((S.n + 31) / 32, 4);
  d.ldx = kw_pad;
  d.lds = round_up((S.mt + 31) / 32, 4);
  d.n_pad = (rows + kGemmOpPad - 1) / kGemmOpPad * kGemmOpPad;
  return d;
}
static EncDims enc_dims(const gmc_key *pk, long long n) { return enc_dims(pk->set, pk->kw_pad, n); }

// Key matrices of a segment list (FP8 images built first when the engine needs them).
static cudaError_t gemm_keys(const gmc_key *const *keys, int nkeys, int engine, cudaStream_t st, GemmKeys *gk,
                             int **err) {
  *gk = GemmKeys{};
  *err = nullptr;
  if (nkeys > 0) gk->tc_stages = tune_get(keys[0]->set).gemm_stages;
  for (int i = 0; i < nkeys; i++) {
    gk->A[i] = keys[i]->kind == 0 ? keys[i]->T : keys[i]->F;
    gk->TT[i] = keys[i]->TT;
    gk->ldtt = keys[i]->ldtt;
    if (engine == GEMM_TC) {
      cudaError_t e = key_a8(keys[i], st, &gk->A8[i]);
      if (e != cudaSuccess) return e;
    }
  }
  if (engine == GEMM_TC && !(*err = tc_err_word())) return cudaErrorMemoryAllocation;
  return cudaSuccess;
}

int gmc::dec_e_words(int set, bool ct) {
  const gmc_setinfo &S = set_info(set);
  const int tab = round_up((S.n + 31) / 32, 4);
  return ct ? std::max(S.q / 32, ct_htt_words(S.n)) : tab;
}

// the first-t syndrome matrix of a secret key (and its FP8 image for the tensor-core engine), built on first use
static cudaError_t key_ct(const gmc_key *kc, int engine, cudaStream_t st) {
  gmc_key *k = const_cast<gmc_key *>(kc);
  std::lock_guard<std::mutex> lk(*k->a8_mu);
  if (!k->cond) return cudaErrorInvalidValue;  // a key without control bits (see gmc_key_import)
  const gmc_setinfo &S = set_info(k->set);
  const int tm = S.t * S.m, rows_pad = round_up(tm, kGemmRowTile), kwn = ct_htt_words(S.n);
  cudaError_t e = cudaSuccess;
  if (!k->htt) {
    uint32_t *p = nullptr;
    e = cudaMalloc(&p, (size_t)rows_pad * kwn * 4);
    if (e == cudaSuccess) e = launch_ct_htt(k->HT, k->dk.ldh, S.n, tm, p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaFree(p);
      return e;
    }
    k->htt = p;
  }
  if (engine == GEMM_TC && !k->htt8) {
    uint8_t *p = nullptr;
    e = cudaMalloc(&p, tc_a8_bytes(rows_pad, kwn));
    if (e == cudaSuccess) e = launch_expand_a(k->htt, kwn, rows_pad, kwn, p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaFree(p);
      return e;
    }
    k->htt8 = p;
  }
  return cudaSuccess;
}

cudaError_t gmc::ct_gemm_keys(const gmc_key *const *keys, int nkeys, int engine, cudaStream_t st, GemmKeys *gk) {
  *gk = GemmKeys{};
  if (nkeys > 0) gk->tc_stages = tune_get(keys[0]->set).gemm_stages;
  for (int i = 0; i < nkeys; i++) {
    cudaError_t e = key_ct(keys[i], engine, st);
    if (e != cudaSuccess) return e;
    gk->A[i] = keys[i]->htt;
    gk->A8[i] = keys[i]->htt8;
  }
  return cudaSuccess;
}

// encapsulation kernels for the segments of one set: seeds / c / k rows in padded row space
template <int SET>
static cudaError_t enc_sample_gemm_seg(const Segs &segs, const gmc_key *ref, const GemmKeys &gk, int engine, int *err,
                                       const uint8_t *seeds, uint32_t *E, uint32_t *Ens, uint32_t *S,
                                       const EncDims &d, cudaStream_t st) {
  using p = P<SET>;
  prof_mark(nullptr, st);
  const SetTune tune = tune_get(SET);
  if (engine == GEMM_SPARSE)  // the sampler writes S itself; Ens lends its first word as the work counter
    return launch_sample<SET>(seeds, segs, E, d.lde, Ens, d.ldx, &gk, S, d.lds, tune.sample_threads,
                              reinterpret_cast<unsigned int *>(Ens), st, tune.sample_sm_warps, prof_mark);
  cudaError_t e = launch_sample<SET>(seeds, segs, E, d.lde, Ens, d.ldx, nullptr, S, d.lds, tune.sample_threads,
                                     reinterpret_cast<unsigned int *>(S), st, tune.sample_sm_warps, prof_mark);
  if (e != cudaSuccess) return e;
  e = launch_gf2_gemm_seg(engine, gk, segs, ref->lda, ref->rows_pad, Ens, d.ldx, ref->kw_pad, S, d.lds, p::mw, err,
                          st);
  prof_mark("enc_syndrome_gemm", st);
  return e;
}

template <int SET>
static cudaError_t enc_sample_gemm(const gmc_key *pk, const uint8_t *seeds, long long n, uint32_t *E, uint32_t *Ens,
                                   uint32_t *S, const EncDims &d, cudaStream_t st) {
  GemmKeys gk;
  int *err;
  const int engine = engine_for(pk->set, 0);
  cudaError_t e = gemm_keys(&pk, 1, engine, st, &gk, &err);
  if (e != cudaSuccess) return e;
  return enc_sample_gemm_seg<SET>(one_segment(n), pk, gk, engine, err, seeds, E, Ens, S, d, st);
}

template <int SET>
static cudaError_t enc_run(const gmc_key *pk, uint8_t *c, uint8_t *k, const uint8_t *seeds, long long n,
                           cudaStream_t st, Scratch &scr) {
  EncDims d = enc_dims(pk, n);
  uint32_t *E, *Ens, *S;
  cudaError_t e;
  if ((e = scr.get((void **)&E, (size_t)d.n_pad * d.lde * 4)) != cudaSuccess) return e;
  if ((e = scr.get((void **)&Ens, (size_t)d.n_pad * d.ldx * 4)) != cudaSuccess) return e;
  if ((e = scr.get((void **)&S, (size_t)d.n_pad * d.lds * 4)) != cudaSuccess) return e;
  if ((e = enc_sample_gemm<SET>(pk, seeds, n, E, Ens, S, d, st)) != cudaSuccess) return e;
  e = launch_finalize<SET>(E, d.lde, S, d.lds, c, k, one_segment(n), pk->pad_bad ? 1u : 0u, pk->pc != 0, st);
  prof_mark("enc_finalize_hash", st);
  return e;
}

struct DecDims {
  int ldx, lds2, lde;
  long long n_pad;
  bool ct;  // constant-time kernels (the switch as read once for this batch)
};
static DecDims dec_dims(int set, int cw_pad, long long rows) {
  const gmc_setinfo &S = set_info(set);
  DecDims d;
  d.ct = dec_constant_time();
  d.ldx = cw_pad;
  d.lds2 = round_up((2 * S.t * S.m + 31) / 32, 4);
  d.lde = dec_e_words(set, d.ct);
  d.n_pad = (rows + kGemmOpPad - 1) / kGemmOpPad * kGemmOpPad;
  return d;
}
static DecDims dec_dims(const gmc_key *sk, long long n) { return dec_dims(sk->set, sk->cw_pad, n); }

// decapsulation kernels up to the decode flags for the segments of one set
template <int SET>
static cudaError_t dec_front_decode_seg(const Segs &segs, const gmc_key *ref, const GemmKeys &gk, const DecKeys &dk,
                                        int engine, int *err, const uint8_t *c, uint32_t *X, uint32_t *S2,
                                        uint16_t *Sig, uint32_t *E, int *ok, const DecDims &d, cudaStream_t st,
                                        bool pc = false, const GemmKeys *ctk = nullptr) {
  using p = P<SET>;
  FieldDev fd;
  if (get_field(SET, &fd) != GMC_OK) return cudaErrorUnknown;
  prof_mark(nullptr, st);
  cudaError_t e = launch_pack_ct<SET>(c, segs, X, d.ldx, pc, st);
  if (e != cudaSuccess) return e;
  prof_mark("dec_pack_ct", st);
  e = launch_gf2_gemm_seg(engine, gk, segs, ref->ldf, ref->frows_pad, X, d.ldx, ref->cw_pad, S2, d.lds2, p::s2w, err,
                          st);
  if (e != cudaSuccess) return e;
  prof_mark("dec_front_gemm", st);
  const SetTune tune = tune_get(SET);
  e = launch_dec_bm<SET>(S2, d.lds2, fd, segs, Sig, st, tune.bm_warps, d.ct);
  if (e != cudaSuccess) return e;
  prof_mark("dec_bm", st);
  e = launch_dec_root<SET>(Sig, S2, d.lds2, dk, fd, segs, E, d.lde, ok, st, tune.root_warps, d.ct);
  prof_mark("dec_fft_roots_reenc", st);
  if (e != cudaSuccess || !d.ct) return e;
  // constant time: the Benes network to code positions, then the dense first-t syndrome check
  // (the packed ciphertexts in X are no longer needed: X takes the check's syndromes)
  if (!ctk) return cudaErrorInvalidValue;
  e = launch_dec_ct_finish<SET>(dk, *ctk, engine, segs, E, d.lde, S2, d.lds2, X, d.ldx, ok, err, st);
  prof_mark("dec_ct_positions_check", st);
  return e;
}

template <int SET>
static cudaError_t dec_front_decode(const gmc_key *sk, const uint8_t *c, long long n, uint32_t *X, uint32_t *S2,
                                    uint16_t *Sig, uint32_t *E, int *ok, const DecDims &d, cudaStream_t st) {
  GemmKeys gk;
  int *err;
  const int engine = engine_for(sk->set, 1);
  cudaError_t e = gemm_keys(&sk, 1, engine, st, &gk, &err);
  if (e != cudaSuccess) return e;
  DecKeys dk{};
  dk.k[0] = sk->dk;
  GemmKeys ctk;
  if (d.ct && (e = ct_gemm_keys(&sk, 1, engine, st, &ctk)) != cudaSuccess) return e;
  return dec_front_decode_seg<SET>(one_segment(n), sk, gk, dk, engine, err, c, X, S2, Sig, E, ok, d, st,
                                   sk->pc != 0, d.ct ? &ctk : nullptr);
}

template <int SET>
static cudaError_t dec_run(const gmc_key *sk, uint8_t *k, const uint8_t *c, long long n, int *rc, cudaStream_t st,
                           Scratch &scr) {
  DecDims d = dec_dims(sk, n);
  uint32_t *X, *S2, *E;
  uint16_t *Sig;
  int *ok;
  cudaError_t e;
  if ((e = scr.get((void **)&X, (size_t)d.n_pad * d.ldx * 4)) != cudaSuccess) return e;
  if ((e = scr.get((void **)&S2, (size_t)d.n_pad * d.lds2 * 4)) != cudaSuccess) return e;
  if ((e = scr.get((void **)&Sig, (size_t)d.n_pad * (2u << P<SET>::fft_d))) != cudaSuccess) return e;
  if ((e = scr.get((void **)&E, (size_t)d.n_pad * d.lde * 4)) != cudaSuccess) return e;
  if ((e = scr.get((void **)&ok, (size_t)d.n_pad * 4)) != cudaSuccess) return e;
  if ((e = dec_front_decode<SET>(sk, c, n, X, S2, Sig, E, ok, d, st)) != cudaSuccess) return e;
  DecKeys dk{};
  dk.k[0] = sk->dk;
  e = launch_dec_tail<SET>(E, d.lde, ok, c, dk, k, rc, one_segment(n), sk->pc != 0, st);
  prof_mark("dec_tail_hash", st);
  return e;
}

#define GMC_DISPATCH(set, call) \
  switch (set) {                \
    case 0: { constexpr int S_ = 0; call; } break; \
    case 1: { constexpr int S_ = 1; call; } break; \
    case 2: { constexpr int S_ = 2; call; } break; \
    case 3: { constexpr int S_ = 3; call; } break; \
    default: { constexpr int S_ = 4; call; } break; \
  }

static int check_key(const gmc_key *key, int kind, const char *fn) {
  if (!key) return fail(GMC_EINVAL, std::string(fn) + ": null key");
  if (key->kind != kind) return fail(GMC_EKEY, std::string(fn) + ": wrong key kind");
  return GMC_OK;
}

__global__ void fill_int_kernel(int *p, long long n, int v) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

extern "C" int gmc_enc_batch_dev(const gmc_key *pk, unsigned char *c, unsigned char *k, const unsigned char *seeds,
                                 long long n, int *rc, void *stream) {
  int r = check_key(pk, 0, "gmc_enc_batch_dev");
  if (r) return r;
  if (n < 0 || (n && (!c || !k || !seeds))) return fail(GMC_EINVAL, "gmc_enc_batch_dev: bad argument");
  if (!n) return GMC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  {
    Scratch scr(st);
    GMC_DISPATCH(pk->set, e = enc_run<S_>(pk, c, k, seeds, n, st, scr));
  }
  if (e != cudaSuccess) return cuda_fail(e, "gmc_enc_batch_dev");
  if (rc) {
    fill_int_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rc, n, pk->pad_bad ? -1 : 0);
    GMC_CUDA(cudaGetLastError());
  }
  return GMC_OK;
}

extern "C" int gmc_dec_batch_dev(const gmc_key *sk, unsigned char *k, const unsigned char *c, long long n, int *rc,
                                 void *stream) {
  int r = check_key(sk, 1, "gmc_dec_batch_dev");
  if (r) return r;
  if (n < 0 || (n && (!c || !k))) return fail(GMC_EINVAL, "gmc_dec_batch_dev: bad argument");
  if (!n) return GMC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  {
    Scratch scr(st);
    GMC_DISPATCH(sk->set, e = dec_run<S_>(sk, k, c, n, rc, st, scr));
  }
  if (e != cudaSuccess) return cuda_fail(e, "gmc_dec_batch_dev");
  return GMC_OK;
}

// host-pointer variants: own stream, copies in, run, copies out
extern "C" int gmc_enc_batch(const gmc_key *pk, unsigned char *c, unsigned char *k, const unsigned char *seeds,
                             long long n, int *rc) {
  int r = check_key(pk, 0, "gmc_enc_batch");
  if (r) return r;
  if (n < 0 || (n && (!c || !k || !seeds))) return fail(GMC_EINVAL, "gmc_enc_batch: bad argument");
  if (!n) return GMC_OK;
  const size_t cb = (size_t)ct_bytes_of(pk);
  keep_pool_warm();
  cudaStream_t st = host_call_stream();
  if (!st) return fail(GMC_ECUDA, "gmc_enc_batch: stream");
  uint8_t *d_seeds = nullptr, *d_c = nullptr, *d_k = nullptr;
  int *d_rc = nullptr;
  cudaError_t e = cudaMallocAsync(&d_seeds, (size_t)n * 32, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_c, (size_t)n * cb, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_k, (size_t)n * 32, st);
  if (e == cudaSuccess && rc) e = cudaMallocAsync(&d_rc, (size_t)n * 4, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_seeds, seeds, (size_t)n * 32, cudaMemcpyHostToDevice, st);
  int res = GMC_OK;
  if (e == cudaSuccess) {
    res = gmc_enc_batch_dev(pk, d_c, d_k, d_seeds, n, d_rc, st);
    if (res == GMC_OK) {
      e = cudaMemcpyAsync(c, d_c, (size_t)n * cb, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(k, d_k, (size_t)n * 32, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess && rc) e = cudaMemcpyAsync(rc, d_rc, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    }
  }
  cudaFreeAsync(d_seeds, st); cudaFreeAsync(d_c, st); cudaFreeAsync(d_k, st);
  if (d_rc) cudaFreeAsync(d_rc, st);
  cudaError_t e2 = cudaStreamSynchronize(st);
  if (res != GMC_OK) return res;
  if (e != cudaSuccess) return cuda_fail(e, "gmc_enc_batch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "gmc_enc_batch: sync");
  return GMC_OK;
}

extern "C" int gmc_dec_batch(const gmc_key *sk, unsigned char *k, const unsigned char *c, long long n, int *rc) {
  int r = check_key(sk, 1, "gmc_dec_batch");
  if (r) return r;
  if (n < 0 || (n && (!c || !k))) return fail(GMC_EINVAL, "gmc_dec_batch: bad argument");
  if (!n) return GMC_OK;
  const size_t cb = (size_t)ct_bytes_of(sk);
  keep_pool_warm();
  cudaStream_t st = host_call_stream();
  if (!st) return fail(GMC_ECUDA, "gmc_dec_batch: stream");
  uint8_t *d_c = nullptr, *d_k = nullptr;
  int *d_rc = nullptr;
  cudaError_t e = cudaMallocAsync(&d_c, (size_t)n * cb, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_k, (size_t)n * 32, st);
  if (e == cudaSuccess && rc) e = cudaMallocAsync(&d_rc, (size_t)n * 4, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_c, c, (size_t)n * cb, cudaMemcpyHostToDevice, st);
  int res = GMC_OK;
  if (e == cudaSuccess) {
    res = gmc_dec_batch_dev(sk, d_k, d_c, n, d_rc, st);
    if (res == GMC_OK) {
      e = cudaMemcpyAsync(k, d_k, (size_t)n * 32, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess && rc) e = cudaMemcpyAsync(rc, d_rc, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
    }
  }
  cudaFreeAsync(d_c, st); cudaFreeAsync(d_k, st);
  if (d_rc) cudaFreeAsync(d_rc, st);
  cudaError_t e2 = cudaStreamSynchronize(st);
  if (res != GMC_OK) return res;
  if (e != cudaSuccess) return cuda_fail(e, "gmc_dec_batch");
  if (e2 != cudaSuccess) return cuda_fail(e2, "gmc_dec_batch: sync");
  return GMC_OK;
}

// ---------------------------------------------------------------- stages
extern "C" int gmc_dec_stages_dev(const gmc_key *sk, const unsigned char *c, long long n, unsigned int *synd,
                                  int synd_words, unsigned int *ev, int e_words, int *ok, void *stream) {
  int r = check_key(sk, 1, "gmc_dec_stages_dev");
  if (r) return r;
  if (n <= 0 || !c || !synd || !ev || !ok) return fail(GMC_EINVAL, "gmc_dec_stages_dev: bad argument");
  DecDims d = dec_dims(sk, n);
  if (synd_words != d.lds2 || e_words != d.lde) return fail(GMC_EINVAL, "gmc_dec_stages_dev: row strides");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  {
    Scratch scr(st);
    uint32_t *X;
    uint16_t *Sig = nullptr;
    e = scr.get((void **)&X, (size_t)d.n_pad * d.ldx * 4);
    if (e == cudaSuccess) e = scr.get((void **)&Sig, (size_t)d.n_pad * 256);
    if (e == cudaSuccess) GMC_DISPATCH(sk->set, e = dec_front_decode<S_>(sk, c, n, X, synd, Sig, ev, ok, d, st));
    // (dec_front_decode packs C0 at the key's ciphertext stride: pc keys take C0 || C1 rows)
  }
  if (e != cudaSuccess) return cuda_fail(e, "gmc_dec_stages_dev");
  return GMC_OK;
}

extern "C" int gmc_enc_stages_dev(const gmc_key *pk, const unsigned char *seeds, long long n, unsigned int *ev,
                                  int e_words, unsigned int *synd, int synd_words, void *stream) {
  int r = check_key(pk, 0, "gmc_enc_stages_dev");
  if (r) return r;
  if (n <= 0 || !seeds || !ev || !synd) return fail(GMC_EINVAL, "gmc_enc_stages_dev: bad argument");
  EncDims d = enc_dims(pk, n);
  if (e_words != d.lde || synd_words != d.lds) return fail(GMC_EINVAL, "gmc_enc_stages_dev: row strides");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  {
    Scratch scr(st);
    uint32_t *Ens;
    e = scr.get((void **)&Ens, (size_t)d.n_pad * d.ldx * 4);
    if (e == cudaSuccess) GMC_DISPATCH(pk->set, e = enc_sample_gemm<S_>(pk, seeds, n, ev, Ens, synd, d, st));
  }
  if (e != cudaSuccess) return cuda_fail(e, "gmc_enc_stages_dev");
  return GMC_OK;
}

extern "C" int gmc_gf2_gemm_dev(int engine, const unsigned int *A, int lda, int rows_pad, const unsigned int *X,
                                int ldx, long long n_pad, int kw_pad, unsigned int *out, int ldo, int out_words,
                                long long n, void *stream) {
  if (!A || !X || !out || n < 0 || lda < kw_pad || ldx < kw_pad || ldo < out_words || engine < GEMM_POPC ||
      engine > GEMM_TC)
    return fail(GMC_EINVAL, "gmc_gf2_gemm_dev: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t *a8 = nullptr;
  int *err = nullptr;
  cudaError_t e = cudaSuccess;
  if (engine == GEMM_TC) {  // one-off FP8 image of A for this call
    if (!(err = tc_err_word())) return fail(GMC_ECUDA, "gmc_gf2_gemm_dev: error word");
    e = cudaMallocAsync(&a8, tc_a8_bytes(rows_pad, kw_pad), st);
    if (e == cudaSuccess) e = launch_expand_a(A, lda, rows_pad, kw_pad, a8, st);
  }
  if (e == cudaSuccess)
    e = launch_gf2_gemm(engine, A, a8, lda, rows_pad, X, ldx, n_pad, kw_pad, out, ldo, out_words, n, err, st);
  if (a8) cudaFreeAsync(a8, st);
  if (e != cudaSuccess) return cuda_fail(e, "gmc_gf2_gemm_dev");
  return GMC_OK;
}

// ---------------------------------------------------------------- one-request API
static std::mutex g_rng_mu;
static gmc_randombytes_fn g_rng = nullptr;
static void *g_rng_ctx = nullptr;

extern "C" void gmc_set_randombytes(gmc_randombytes_fn fn, void *ctx) {
  std::lock_guard<std::mutex> lk(g_rng_mu);
  g_rng = fn;
  g_rng_ctx = ctx;
}

static int draw_seed(uint8_t seed[32]) {
  gmc_randombytes_fn fn;
  void *ctx;
  {
    std::lock_guard<std::mutex> lk(g_rng_mu);
    fn = g_rng;
    ctx = g_rng_ctx;
  }
  if (fn) {
    fn(ctx, seed, 32);
    return GMC_OK;
  }
  size_t got = 0;
  while (got < 32) {
    ssize_t r = getrandom(seed + got, 32 - got, 0);
    if (r <= 0) return fail(GMC_ECUDA, "randombytes: getrandom failed");
    got += (size_t)r;
  }
  return GMC_OK;
}

// Resident keys of the one-request entry points, most recently used first: a
// caller of the libmceliece convention passes the key bytes with every
// request, so loading them each time (host tables, device copies) would cost
// milliseconds per call. An entry matches on set id, kind, device and the
// whole key (byte comparison); entries are shared, so an eviction never frees
// a handle that another thread is still using.
struct CachedKey {
  int id, kind, device;
  std::vector<uint8_t> bytes;
  std::shared_ptr<gmc_key> h;
};
static std::mutex g_kc_mu;
static std::list<CachedKey> g_kc;
constexpr size_t kKeyCacheEntries = 8;

static int cached_key(int id, int kind, const unsigned char *bytes, std::shared_ptr<gmc_key> *out) {
  if (!valid_id(id)) return fail(GMC_EINVAL, "bad set id");
  const gmc_setinfo &S = set_info(base_of(id));
  const size_t len = (size_t)(kind == 0 ? S.pk_bytes : S.sk_bytes);
  int dev = 0;
  GMC_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(g_kc_mu);
    for (auto it = g_kc.begin(); it != g_kc.end(); ++it)
      if (it->id == id && it->kind == kind && it->device == dev && !memcmp(it->bytes.data(), bytes, len)) {
        g_kc.splice(g_kc.begin(), g_kc, it);
        *out = g_kc.front().h;
        return GMC_OK;
      }
  }
  std::vector<uint8_t> copy(bytes, bytes + len);  // the caller's buffer may alias an output
  gmc_key *h = nullptr;
  const int r = kind == 0 ? gmc_pk_load(&h, id, copy.data()) : gmc_sk_load(&h, id, copy.data());
  if (r != GMC_OK) return r;
  std::shared_ptr<gmc_key> sp(h, gmc_key_free);
  std::lock_guard<std::mutex> lk(g_kc_mu);
  g_kc.push_front(CachedKey{id, kind, dev, std::move(copy), sp});
  while (g_kc.size() > kKeyCacheEntries) g_kc.pop_back();
  *out = sp;
  return GMC_OK;
}

static int one_enc(int set, unsigned char *c, unsigned char *k, const unsigned char *pk) {
  uint8_t seed[32];
  int r = draw_seed(seed);
  if (r) return r;
  std::shared_ptr<gmc_key> h;
  if ((r = cached_key(set, 0, pk, &h)) != GMC_OK) return r;
  int rc = 0;
  r = gmc_enc_batch(h.get(), c, k, seed, 1, &rc);
  return r ? r : rc;
}

static int one_dec(int set, unsigned char *k, const unsigned char *c, const unsigned char *sk) {
  std::vector<uint8_t> cc(c, c + ct_bytes_of(base_of(set), pc_of(set)));  // k may alias c or sk
  std::shared_ptr<gmc_key> h;
  int r = cached_key(set, 1, sk, &h);
  if (r) return r;
  uint8_t kk[32];
  int rc = 0;
  r = gmc_dec_batch(h.get(), kk, cc.data(), 1, &rc);
  if (r) return r;
  memcpy(k, kk, 32);
  return rc;
}

// One key pair: the GPU key generation with a batch of one (there is no host
// key generation; a plaintext-confirmation variant has the keys of its
// parameter set, an f variant the semi-systematic form).
extern "C" int gmc_keypair_seed(int set, unsigned char *pk, unsigned char *sk, const unsigned char *seed32) {
  if (!valid_id(set) || !pk || !sk || !seed32) return fail(GMC_EINVAL, "gmc_keypair_seed: bad argument");
  return gmc_keypair_batch(set, pk, sk, seed32, 1);
}

static int one_keypair(int set, unsigned char *pk, unsigned char *sk) {
  uint8_t seed[32];
  int r = draw_seed(seed);
  if (r) return r;
  return gmc_keypair_seed(set, pk, sk, seed);
}

#define GMC_ONE(NAME, SET)                                                                               \
  extern "C" void gmc_kem_##NAME##_keypair(unsigned char *pk, unsigned char *sk) {                      \
    one_keypair(SET, pk, sk);                                                                           \
  }                                                                                                     \
  extern "C" int gmc_kem_##NAME##_enc(unsigned char *c, unsigned char *k, const unsigned char *pk) {    \
    return one_enc(SET, c, k, pk);                                                                      \
  }                                                                                                     \
  extern "C" int gmc_kem_##NAME##_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk) { \
    return one_dec(SET, k, c, sk);                                                                      \
  }
GMC_ONE(348864, 0)
GMC_ONE(460896, 1)
GMC_ONE(6688128, 2)
GMC_ONE(6960119, 3)
GMC_ONE(8192128, 4)
GMC_ONE(348864pc, 5)
GMC_ONE(460896pc, 6)
GMC_ONE(6688128pc, 7)
GMC_ONE(6960119pc, 8)
GMC_ONE(8192128pc, 9)
GMC_ONE(348864f, 10)
GMC_ONE(460896f, 11)
GMC_ONE(6688128f, 12)
GMC_ONE(6960119f, 13)
GMC_ONE(8192128f, 14)
GMC_ONE(348864pcf, 15)
GMC_ONE(460896pcf, 16)
GMC_ONE(6688128pcf, 17)
GMC_ONE(6960119pcf, 18)
GMC_ONE(8192128pcf, 19)

// ---------------------------------------------------------------- host-only views
// Per-key tables exactly as uploaded, for host-side checks (no GPU needed).
extern "C" int gmc_host_sk_tables(int set, const unsigned char *sk, unsigned short *L, unsigned short *Lpow,
                                  unsigned int *F, long long f_words, int *ldf) {
  if (!valid_set(set) || !sk) return fail(GMC_EINVAL, "gmc_host_sk_tables: bad argument");
  SkHost h;
  if (build_sk(set, sk, h)) return fail(GMC_EKEY, "gmc_host_sk_tables: bad key");
  const gmc_setinfo &S = set_info(set);
  if (L) memcpy(L, h.L.data(), (size_t)S.n * 2);
  if (Lpow) memcpy(Lpow, h.Lpow.data(), (size_t)S.n * 2);
  if (ldf) *ldf = h.ldf;
  if (F) {
    if (f_words < (long long)h.F.size()) return fail(GMC_EINVAL, "gmc_host_sk_tables: F too small");
    memcpy(F, h.F.data(), h.F.size() * 4);
  }
  return (int)h.F.size();
}

extern "C" int gmc_host_field_tables(int set, unsigned short *gexp, unsigned short *glog, unsigned short *alpha_log,
                                     unsigned short *twist_log) {
  if (!valid_set(set)) return fail(GMC_EINVAL, "gmc_host_field_tables: bad set");
  const gmc_setinfo &S = set_info(set);
  const HostField &F = host_field(S.m);
  FftTables ft = build_fft_tables(S.m, S.fft_d);
  if (gexp) memcpy(gexp, F.exp.data(), F.exp.size() * 2);
  if (glog) memcpy(glog, F.log.data(), F.log.size() * 2);
  if (alpha_log) memcpy(alpha_log, ft.alpha_log.data(), ft.alpha_log.size() * 2);
  if (twist_log) memcpy(twist_log, ft.twist_log.data(), ft.twist_log.size() * 2);
  return GMC_OK;
}

int *gmc::tc_err_word_ptr() { return tc_err_word(); }
int gmc::field_tables(int set, FieldDev *out) { return get_field(set, out); }
int gmc::key_prepare_resident(const gmc_key *key) {
  if (!key) return fail(GMC_EINVAL, "key_prepare_resident: null key");
  cudaStream_t st;
  GMC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const uint8_t *a8;
  cudaError_t e = key_a8(key, st, &a8);
  cudaStreamDestroy(st);
  if (e != cudaSuccess) return cuda_fail(e, "key_prepare_resident");
  FieldDev fd;
  return get_field(key->set, &fd);
}

// ---------------------------------------------------------------- grouped plans
// A plan is a fixed set of request groups (key, op, n, device buffers). Groups
// are bucketed by (parameter set, enc/dec) into pipelines of at most kMaxSegs
// keys; each pipeline gathers its groups' inputs into one padded buffer
// (segment starts at multiples of kGemmOpPad), runs the segment-aware kernels
// once for all its keys, and scatters the outputs back. All pipelines are
// captured as parallel branches of one CUDA graph; gmc_plan_launch replays it
// with a single cudaGraphLaunch.
struct PlanPipe {
  int set = 0, kind = 0;  // kind 0 enc, 1 dec
  int pc = 0;             // plaintext-confirmation keys (ciphertexts C0 || C1)
  int engine = GEMM_TC;
  bool const_time = false;  // constant-time decapsulation kernels (the switch at plan creation)
  std::vector<int> groups;
  Segs segs{};
  uint32_t pk_bad_mask = 0;
  uint8_t *in = nullptr, *ct = nullptr, *k = nullptr;
  int *rc = nullptr;
  uint32_t *w0 = nullptr, *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;  // intermediates
  uint16_t *sig = nullptr;
  int *ok = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
};

struct gmc_plan {
  int device = 0;
  std::vector<gmc_group> groups;
  std::vector<PlanPipe> pipes;
  std::vector<void *> allocs;
  cudaStream_t cap = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static void plan_release(gmc_plan *p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (auto &pp : p->pipes) {
    if (pp.st) cudaStreamDestroy(pp.st);
    if (pp.done) cudaEventDestroy(pp.done);
  }
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->cap) cudaStreamDestroy(p->cap);
  for (void *a : p->allocs) cudaFree(a);
  delete p;
}

extern "C" void gmc_plan_free(gmc_plan *plan) { plan_release(plan); }

template <int SET>
static cudaError_t plan_pipe_kernels(gmc_plan *p, PlanPipe &pp) {
  const gmc_key *keys[kMaxSegs];
  for (size_t i = 0; i < pp.groups.size(); i++) keys[i] = p->groups[pp.groups[i]].key;
  const gmc_key *ref = keys[0];
  GemmKeys gk;
  int *err;
  cudaError_t e = gemm_keys(keys, (int)pp.groups.size(), pp.engine, pp.st, &gk, &err);
  if (e != cudaSuccess) return e;
  const long long rows = seg_rows(pp.segs);
  if (pp.kind == 0) {
    EncDims d = enc_dims(SET, ref->kw_pad, rows);
    e = enc_sample_gemm_seg<SET>(pp.segs, ref, gk, pp.engine, err, pp.in, pp.w0, pp.w1, pp.w2, d, pp.st);
    if (e == cudaSuccess)
      e = launch_finalize<SET>(pp.w0, d.lde, pp.w2, d.lds, pp.ct, pp.k, pp.segs, pp.pk_bad_mask, pp.pc != 0, pp.st);
  } else {
    DecDims d = dec_dims(SET, ref->cw_pad, rows);
    d.ct = pp.const_time;  // the buffers were laid out for the form chosen at creation
    d.lde = dec_e_words(SET, pp.const_time);
    DecKeys dk{};
    for (size_t i = 0; i < pp.groups.size(); i++) dk.k[i] = keys[i]->dk;
    GemmKeys ctk;
    if (d.ct) e = ct_gemm_keys(keys, (int)pp.groups.size(), pp.engine, pp.st, &ctk);
    if (e == cudaSuccess)
      e = dec_front_decode_seg<SET>(pp.segs, ref, gk, dk, pp.engine, err, pp.in, pp.w0, pp.w1, pp.sig, pp.w2, pp.ok,
                                    d, pp.st, pp.pc != 0, d.ct ? &ctk : nullptr);
    if (e == cudaSuccess)
      e = launch_dec_tail<SET>(pp.w2, d.lde, pp.ok, pp.in, dk, pp.k, pp.rc, pp.segs, pp.pc != 0, pp.st);
  }
  return e;
}

static cudaError_t plan_alloc(gmc_plan *p, void **ptr, size_t bytes) {
  cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
  if (e == cudaSuccess) p->allocs.push_back(*ptr);
  return e;
}

extern "C" int gmc_plan_create(gmc_plan **out, const gmc_group *groups, int ngroups) {
  if (!out || !groups || ngroups <= 0) return fail(GMC_EINVAL, "gmc_plan_create: bad argument");
  *out = nullptr;
  for (int i = 0; i < ngroups; i++) {
    const gmc_group &g = groups[i];
    if (!g.key || g.n < 0 || (g.n && (!g.in || !g.k || (g.key->kind == 0 && !g.ct))))
      return fail(GMC_EINVAL, "gmc_plan_create: bad group");
  }
  gmc_plan *p = new gmc_plan();
  cudaGetDevice(&p->device);
  p->groups.assign(groups, groups + ngroups);
  // bucket by (set, pc, kind), at most kMaxSegs groups per pipeline
  for (int i = 0; i < ngroups; i++) {
    const gmc_group &g = groups[i];
    if (!g.n) continue;
    PlanPipe *dst = nullptr;
    for (auto &pp : p->pipes)
      if (pp.set == g.key->set && pp.pc == g.key->pc && pp.kind == g.key->kind &&
          pp.groups.size() < (size_t)kMaxSegs)
        dst = &pp;
    if (!dst) {
      p->pipes.emplace_back();
      dst = &p->pipes.back();
      dst->set = g.key->set;
      dst->pc = g.key->pc;
      dst->kind = g.key->kind;
      dst->engine = engine_for(dst->set, dst->kind);
    }
    dst->groups.push_back(i);
  }
  cudaError_t e = cudaSuccess;
  for (auto &pp : p->pipes) {
    const gmc_setinfo &S = set_info(pp.set);
    pp.segs = Segs{};
    pp.segs.nseg = (int)pp.groups.size();
    long long row = 0;
    for (size_t j = 0; j < pp.groups.size(); j++) {
      const gmc_group &g = p->groups[pp.groups[j]];
      pp.segs.row0[j] = row;
      pp.segs.nreq[j] = g.n;
      row += (g.n + kGemmOpPad - 1) / kGemmOpPad * kGemmOpPad;
      if (pp.kind == 0 && g.key->pad_bad) pp.pk_bad_mask |= 1u << j;
    }
    pp.segs.row0[pp.groups.size()] = row;
    const gmc_key *ref = p->groups[pp.groups[0]].key;
    const size_t cb = (size_t)ct_bytes_of(pp.set, pp.pc != 0);
    const size_t in_b = pp.kind == 0 ? 32 : cb;
    if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.in, row * in_b);
    if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.k, row * 32);
    if (pp.kind == 0) {
      EncDims d = enc_dims(pp.set, ref->kw_pad, row);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.ct, row * cb);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.w0, row * d.lde * 4);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.w1, row * d.ldx * 4);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.w2, row * d.lds * 4);
    } else {
      DecDims d = dec_dims(pp.set, ref->cw_pad, row);
      pp.const_time = d.ct;
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.rc, row * 4);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.w0, row * d.ldx * 4);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.w1, row * d.lds2 * 4);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.sig, row * (2u << S.fft_d));
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.w2, row * d.lde * 4);
      if (e == cudaSuccess) e = plan_alloc(p, (void **)&pp.ok, row * 4);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&pp.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pp.done, cudaEventDisableTiming);
    // per-set tables and FP8 key images exist before capture
    FieldDev fd;
    if (e == cudaSuccess && pp.kind == 1 && get_field(pp.set, &fd) != GMC_OK) e = cudaErrorUnknown;
    if (e == cudaSuccess && pp.engine == GEMM_TC)
      for (int gi : pp.groups) {
        const uint8_t *a8;
        if ((e = key_a8(p->groups[gi].key, pp.st, &a8)) != cudaSuccess) break;
      }
    if (e == cudaSuccess && pp.engine == GEMM_TC && !tc_err_word()) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess && pp.kind == 1 && pp.const_time) {  // the constant-time check's matrices, before capture
      const gmc_key *ks[kMaxSegs];
      for (size_t j = 0; j < pp.groups.size(); j++) ks[j] = p->groups[pp.groups[j]].key;
      GemmKeys ctk;
      e = ct_gemm_keys(ks, (int)pp.groups.size(), pp.engine, pp.st, &ctk);
    }
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    plan_release(p);
    return cuda_fail(e, "gmc_plan_create: setup");
  }
  // capture: fork to one stream per pipeline, gather, kernels, scatter, join
  e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) e = cudaEventRecord(p->fork, p->cap);
  for (auto &pp : p->pipes) {
    if (e != cudaSuccess) break;
    const size_t cb = (size_t)ct_bytes_of(pp.set, pp.pc != 0);
    const size_t in_b = pp.kind == 0 ? 32 : cb;
    e = cudaStreamWaitEvent(pp.st, p->fork, 0);
    for (size_t j = 0; j < pp.groups.size() && e == cudaSuccess; j++) {
      const gmc_group &g = p->groups[pp.groups[j]];
      e = cudaMemcpyAsync(pp.in + pp.segs.row0[j] * in_b, g.in, g.n * in_b, cudaMemcpyDeviceToDevice, pp.st);
    }
    if (e == cudaSuccess) GMC_DISPATCH(pp.set, e = plan_pipe_kernels<S_>(p, pp));
    for (size_t j = 0; j < pp.groups.size() && e == cudaSuccess; j++) {
      const gmc_group &g = p->groups[pp.groups[j]];
      const long long r0 = pp.segs.row0[j];
      e = cudaMemcpyAsync(g.k, pp.k + r0 * 32, g.n * 32, cudaMemcpyDeviceToDevice, pp.st);
      if (e == cudaSuccess && pp.kind == 0)
        e = cudaMemcpyAsync(g.ct, pp.ct + r0 * cb, g.n * cb, cudaMemcpyDeviceToDevice, pp.st);
      if (e == cudaSuccess && g.rc) {
        if (pp.kind == 0)
          e = cudaMemsetAsync(g.rc, g.key->pad_bad ? 0xFF : 0, g.n * 4, pp.st);  // -1 or 0
        else
          e = cudaMemcpyAsync(g.rc, pp.rc + r0, g.n * 4, cudaMemcpyDeviceToDevice, pp.st);
      }
    }
    if (e == cudaSuccess) e = cudaEventRecord(pp.done, pp.st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->cap, pp.done, 0);
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(p->cap, &graph);
  if (e == cudaSuccess) e = e2;
  p->graph = graph;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  if (e != cudaSuccess) {
    plan_release(p);
    return cuda_fail(e, "gmc_plan_create: capture");
  }
  *out = p;
  return GMC_OK;
}

extern "C" int gmc_plan_launch(gmc_plan *plan, void *stream) {
  if (!plan || !plan->exec) return fail(GMC_EINVAL, "gmc_plan_launch: bad plan");
  GMC_CUDA(cudaGraphLaunch(plan->exec, (cudaStream_t)stream));
  return GMC_OK;
}

extern "C" int gmc_plan_info(const gmc_plan *plan, int *pipelines, long long *padded_rows) {
  if (!plan) return fail(GMC_EINVAL, "gmc_plan_info: bad plan");
  if (pipelines) *pipelines = (int)plan->pipes.size();
  if (padded_rows) {
    long long r = 0;
    for (auto &pp : plan->pipes) r += seg_rows(pp.segs);
    *padded_rows = r;
  }
  return GMC_OK;
}
