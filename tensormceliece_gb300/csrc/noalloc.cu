// Batched decapsulation that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host process whose device memory is
// owned by another allocator with a fixed budget (for example a serving
// framework that reserved the GPU's memory up front), or a latency-critical
// path where cudaMalloc/cudaFree would synchronize the device and stall other
// streams. For them gmc_dec_batch_noalloc runs the same decapsulation kernels
// as gmc_dec_batch_dev, but every intermediate buffer (ciphertext words, the
// 2t syndromes, the error locators, the error vectors, the decode flags) is
// carved from one file-scope device array of fixed size, and the per-set
// field and FFT tables come from a second one. Nothing here calls cudaMalloc,
// cudaMallocAsync, cudaFree or an allocating library routine; the front-end
// GF(2) product uses the CUDA-core engine, which needs no extra buffers.
//
// Set-up: the first call on a device (with that device current) looks up the
// device addresses of the two arrays with cudaGetSymbolAddress and copies the
// field tables into the second one (cudaMemcpy, synchronous). Make that first
// call before any stream capture. Later calls do no set-up. The key must have
// been loaded on the current device (the call refuses it otherwise).
//
// All calls share the arrays and the arrays keep the last call's contents.
// Every intermediate is written in full before it is read, so nothing has to
// start at zero. Calls whose work overlaps on the GPU (different streams or
// threads without ordering between them) race on the shared scratch: order
// them (one stream, or events) or use gmc_dec_batch_dev instead.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gmc.h"
#include "engine_internal.h"
#include "host_keys.h"
#include "kernels.h"

using namespace gmc;

namespace {

constexpr long long kMaxRequests = GMC_NOALLOC_MAX_REQUESTS;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// scratch of one decapsulation batch of n requests for a set
template <int SET>
struct DecScratch {
  using p = P<SET>;
  static constexpr int ldx = (p::cw + kGemmKTile - 1) / kGemmKTile * kGemmKTile;
  static constexpr int lds2 = (p::s2w + 3) / 4 * 4;
  static constexpr int lde = (p::ew + 3) / 4 * 4;
  static constexpr size_t x_bytes(long long n) {
    return align256((size_t)((n + kGemmOpPad - 1) / kGemmOpPad * kGemmOpPad) * ldx * 4);
  }
  static constexpr size_t s2_bytes(long long n) { return align256((size_t)n * lds2 * 4); }
  static constexpr size_t sig_bytes(long long n) { return align256((size_t)n * (2u << p::fft_d)); }
  static constexpr size_t e_bytes(long long n) { return align256((size_t)n * lde * 4); }
  static constexpr size_t ok_bytes(long long n) { return align256((size_t)n * 4); }
  static constexpr size_t total(long long n) {
    return x_bytes(n) + s2_bytes(n) + sig_bytes(n) + e_bytes(n) + ok_bytes(n);
  }
};

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kScratchBytes =
    cmax(cmax(cmax(DecScratch<0>::total(kMaxRequests), DecScratch<1>::total(kMaxRequests)),
              cmax(DecScratch<2>::total(kMaxRequests), DecScratch<3>::total(kMaxRequests))),
         DecScratch<4>::total(kMaxRequests));

// per-set field/FFT tables (u16 entries): exp (2q-1) | log (q) | twist (2^(d+1)) | frob_lo (2^d) |
// bit-sliced alpha (2 (2^d - 1) 2 m) | bit-sliced frob_hi (2 * 2 m) | zech (q), u32 tables at even offsets
constexpr int kFieldSlot = 2 * 8192 + 8192 + 256 + 128 + 2 * 127 * 2 * 13 + 2 * 2 * 13 + 8192 + 16;
static_assert(kFieldSlot % 2 == 0, "per-set slots must keep the u32 tables 4-byte aligned");

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];
static __device__ __align__(256) uint16_t g_noalloc_fields[GMC_NSETS][kFieldSlot];

namespace {

struct DeviceSetup {
  unsigned char *scratch = nullptr;
  uint16_t *fields = nullptr;
  FieldDev fd[GMC_NSETS];
};

// One set-up record per device ordinal, in a fixed array so that a record's
// address never changes: a call keeps using its record after the mutex is
// released while another thread sets up a different device. A record is
// written once, under the mutex, before its ready flag is published.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSetup g_setups[kMaxDevices];
std::atomic<bool> g_ready[kMaxDevices];

int set_error(int code, const char *msg) {
  gmc::set_last_error(msg);
  return code;
}

// once per device: symbol addresses, field tables copied into the static array
int device_setup(int dev, const DeviceSetup **out) {
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(GMC_EINVAL, "gmc_dec_batch_noalloc: device ordinal too large");
  if (g_ready[dev].load(std::memory_order_acquire)) {
    *out = &g_setups[dev];
    return GMC_OK;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (g_ready[dev].load(std::memory_order_acquire)) {
    *out = &g_setups[dev];
    return GMC_OK;
  }
  DeviceSetup &su = g_setups[dev];
  if (cudaGetSymbolAddress((void **)&su.scratch, g_noalloc_scratch) != cudaSuccess ||
      cudaGetSymbolAddress((void **)&su.fields, g_noalloc_fields) != cudaSuccess)
    return set_error(GMC_ECUDA, "gmc_dec_batch_noalloc: cudaGetSymbolAddress failed");
  for (int set = 0; set < GMC_NSETS; set++) {
    const gmc_setinfo &S = set_info(set);
    const HostField &F = host_field(S.m);
    FftTables ft = build_fft_tables(S.m, S.fft_d);
    std::vector<uint16_t> all(kFieldSlot, 0);
    size_t o = 0;
    bool fits = true;
    auto put = [&](const std::vector<uint16_t> &v) {
      o += o & 1;  // u32 tables start 4-byte aligned
      const size_t at = o;
      if (o + v.size() > all.size()) {
        fits = false;
        return at;
      }
      memcpy(all.data() + o, v.data(), v.size() * 2);
      o += v.size();
      return at;
    };
    const size_t o_exp = put(F.exp), o_log = put(F.log), o_twist = put(ft.twist_log), o_flo = put(ft.frob_lo),
                 o_abs = put(ft.alpha_bs), o_fhbs = put(ft.frob_hi_bs), o_zech = put(ft.zech);
    if (!fits) return set_error(GMC_ECUDA, "gmc_dec_batch_noalloc: field table slot too small");
    uint16_t *base = su.fields + (size_t)set * kFieldSlot;
    if (cudaMemcpy(base, all.data(), all.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess)
      return set_error(GMC_ECUDA, "gmc_dec_batch_noalloc: field table copy failed");
    su.fd[set].gexp = base + o_exp;
    su.fd[set].glog = base + o_log;
    su.fd[set].fft_twist_log = base + o_twist;
    su.fd[set].frob_lo = base + o_flo;
    su.fd[set].fft_alpha_bs = reinterpret_cast<const uint32_t *>(base + o_abs);
    su.fd[set].frob_hi_bs = reinterpret_cast<const uint32_t *>(base + o_fhbs);
    su.fd[set].zech = base + o_zech;
  }
  g_ready[dev].store(true, std::memory_order_release);
  *out = &su;
  return GMC_OK;
}

template <int SET>
cudaError_t run(const DeviceSetup &su, const gmc_key *sk, uint8_t *k, const uint8_t *c, long long n, int *rc,
                cudaStream_t st) {
  using D = DecScratch<SET>;
  unsigned char *q = su.scratch;
  uint32_t *X = reinterpret_cast<uint32_t *>(q);
  q += D::x_bytes(n);
  uint32_t *S2 = reinterpret_cast<uint32_t *>(q);
  q += D::s2_bytes(n);
  uint16_t *Sig = reinterpret_cast<uint16_t *>(q);
  q += D::sig_bytes(n);
  uint32_t *E = reinterpret_cast<uint32_t *>(q);
  q += D::e_bytes(n);
  int *ok = reinterpret_cast<int *>(q);
  const Segs segs = one_segment(n);  // only the first n rows are live and written
  GemmKeys gk{};
  gk.A[0] = sk->F;
  DecKeys dk{};
  dk.k[0] = sk->dk;
  cudaError_t e = launch_pack_ct<SET>(c, segs, X, D::ldx, sk->pc != 0, st);
  if (e == cudaSuccess)
    e = launch_gf2_gemm_seg(GEMM_POPC, gk, segs, sk->ldf, sk->frows_pad, X, D::ldx, sk->cw_pad, S2, D::lds2,
                            P<SET>::s2w, nullptr, st);
  const SetTune tune = tune_get(SET);
  if (e == cudaSuccess) e = launch_dec_bm<SET>(S2, D::lds2, su.fd[SET], segs, Sig, st, tune.bm_warps);
  if (e == cudaSuccess)
    e = launch_dec_root<SET>(Sig, S2, D::lds2, dk, su.fd[SET], segs, E, D::lde, ok, st, tune.root_warps);
  if (e == cudaSuccess) e = launch_dec_tail<SET>(E, D::lde, ok, c, dk, k, rc, segs, sk->pc != 0, st);
  return e;
}

}  // namespace

extern "C" int gmc_dec_batch_noalloc(const gmc_key *sk, unsigned char *k, const unsigned char *c, long long n,
                                     int *rc, void *stream) {
  if (!sk || sk->kind != 1) return set_error(GMC_EKEY, "gmc_dec_batch_noalloc: needs a secret-key handle");
  if (n < 0 || (n && (!k || !c))) return set_error(GMC_EINVAL, "gmc_dec_batch_noalloc: bad argument");
  if (n > kMaxRequests)
    return set_error(GMC_EINVAL, "gmc_dec_batch_noalloc: more than GMC_NOALLOC_MAX_REQUESTS requests; split the "
                                 "batch or use gmc_dec_batch_dev");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_error(GMC_ECUDA, "gmc_dec_batch_noalloc: no device");
  if (sk->device != dev)
    return set_error(GMC_EKEY, "gmc_dec_batch_noalloc: the key was loaded on another device; make that device "
                               "current");
  const DeviceSetup *su = nullptr;
  int r = device_setup(dev, &su);
  if (r) return r;
  if (!n) return GMC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  switch (sk->set) {
    case 0: e = run<0>(*su, sk, k, c, n, rc, st); break;
    case 1: e = run<1>(*su, sk, k, c, n, rc, st); break;
    case 2: e = run<2>(*su, sk, k, c, n, rc, st); break;
    case 3: e = run<3>(*su, sk, k, c, n, rc, st); break;
    default: e = run<4>(*su, sk, k, c, n, rc, st); break;
  }
  if (e != cudaSuccess) {
    gmc::set_last_error((std::string("gmc_dec_batch_noalloc: ") + cudaGetErrorString(e)).c_str());
    return GMC_ECUDA;
  }
  return GMC_OK;
}
