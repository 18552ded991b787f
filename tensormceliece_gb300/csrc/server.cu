// Serving loop: continuous batching of encapsulation / decapsulation requests
// against device-resident keys.
//
// Requests (key handle + host buffers) are queued by gmc_server_submit. A
// dispatcher thread forms a batch from everything queued (FIFO, up to the
// batch limit) whenever one of the server's slots is free, so requests that
// arrive while earlier batches run on the GPU join the next batch. Each slot
// owns a stream, a device arena and pinned staging buffers; a batch is
// admitted only up to what its slot's arena holds (the arenas are carved from
// the free device memory measured at start-up: admission by free HBM).
// A batch runs as: gather inputs into pinned staging -> one host-to-device
// copy -> per (parameter set, enc/dec, plaintext confirmation or not) the
// segment-aware kernels over all its keys, each pipeline on its own stream (forked from and joined back to the
// slot's stream, so they overlap) -> one device-to-host copy -> a host
// callback that hands the slot to the completion thread, which scatters the
// results (on persistent host workers), marks the requests done and records
// their latency (arrival to completion) in a log-bucket histogram (p50 / p99). Several slots keep several batches in
// flight, so their work overlaps on the device.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <random>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gmc.h"
#include "engine_internal.h"
#include "host_keys.h"
#include "kernels.h"

using namespace gmc;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// latency histogram: bucket b covers [1us * 1.02^b, 1us * 1.02^(b+1))
constexpr int kBuckets = 1400;
int bucket_of(double ms) {
  if (ms <= 0.001) return 0;
  int b = (int)(log(ms / 0.001) / log(1.02));
  return b < 0 ? 0 : (b >= kBuckets ? kBuckets - 1 : b);
}
double bucket_ms(int b) { return 0.001 * pow(1.02, b + 0.5); }

struct Req {
  const gmc_key *key;
  const uint8_t *in;
  uint8_t *ct, *k;
  int *rc;
  double t_arrive;
  std::atomic<int> *done;  // optional completion flag of the submitter
};

struct Piece {  // one request inside a batch
  const Req *r;                  // in the slot's incoming requests, which live as long as the batch
  size_t out_k, out_ct, out_rc;  // offsets in the slot's output staging
};

struct Pipe {
  int set, kind, pc;  // pc: plaintext-confirmation keys (ciphertext C0 || C1)
  std::vector<const gmc_key *> keys;
  std::vector<const std::vector<int> *> members;  // piece indices per key (the slot's member lists)
  Segs segs;
  size_t in_off, k_off, ct_off, rc_off, work_off;
};

constexpr int kPipes = 4 * GMC_NSETS;  // at most one pipeline per (set, op, pc) in a batch

struct Slot {
  cudaStream_t st = nullptr;
  cudaStream_t pst[kPipes] = {};     // one stream per pipeline: the pipelines of a batch overlap
  cudaEvent_t fork = nullptr, join[kPipes] = {};
  uint8_t *dev = nullptr;
  size_t dev_bytes = 0;
  uint8_t *h_in = nullptr, *h_out = nullptr;
  size_t h_in_bytes = 0, h_out_bytes = 0;
  std::vector<Piece> pieces;
  std::vector<Pipe> pipes;
  std::deque<Req> incoming;  // the requests of the batch being formed or in flight (moved out of the queue)
  // per-key member lists of a batch, kept from batch to batch so their storage is reused (a deque: the
  // lists keep their addresses while more are added)
  std::deque<std::vector<int>> member_pool;
  size_t in_used = 0, out_used = 0;
  bool busy = false;
  struct gmc_server *srv = nullptr;
  // stage times of the batch in flight (seconds, now_s clock): the oldest request's arrival, requests taken
  // from the queue, batch formed (inputs gathered), launches issued, device work and copies done (callback)
  double t_oldest = 0, t_take = 0, t_taken = 0, t_bucketed = 0, t_formed = 0, t_issued = 0, t_done = 0;
};

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// ciphertext bytes of a set's keys: C0, plus the 32-byte C1 with plaintext confirmation
size_t ct_len(int set, int pc) { return (size_t)set_info(set).synd_bytes + (pc ? 32 : 0); }

// Persistent host workers for the per-request gather and scatter of a batch
// (threads are started once, not per batch: thread creation on every batch
// showed up as latency jitter under load). Jobs from the dispatcher and from
// the completion thread may run at the same time; each waits only for its own
// pieces.
constexpr int kHostThreads = 8;
class HostPool {
 public:
  static HostPool &get() {
    static HostPool *pool = new HostPool();  // never destroyed: workers idle in wait at exit
    return *pool;
  }
  // runs `tasks` on the workers and `own` on the calling thread; returns when all are done
  template <typename Own>
  void run(std::vector<std::function<void()>> &tasks, Own own) {
    int left = (int)tasks.size();  // under dmu: a worker's last touch of this frame is under the lock
    std::mutex dmu;
    std::condition_variable dcv;
    {
      std::lock_guard<std::mutex> lk(mu_);
      for (auto &t : tasks)
        q_.push_back([&, fn = &t] {
          (*fn)();
          std::lock_guard<std::mutex> g(dmu);
          if (--left == 0) dcv.notify_all();
        });
    }
    cv_.notify_all();
    own();
    std::unique_lock<std::mutex> g(dmu);
    dcv.wait(g, [&] { return left == 0; });
  }

 private:
  HostPool() {
    for (int i = 0; i < 2 * (kHostThreads - 1); i++) std::thread([this] { work(); }).detach();
  }
  void work() {
    while (true) {
      std::function<void()> fn;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !q_.empty(); });
        fn = std::move(q_.front());
        q_.pop_front();
      }
      fn();
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> q_;
};

// Runs fn(begin, end) over [0, n) in up to kHostThreads pieces (the calling
// thread takes the first, the pool the others).
template <typename F>
void parallel_for(size_t n, F fn) {
  const size_t per = 4096;  // below this a piece is not worth a hand-off
  const int parts = (int)std::min<size_t>(kHostThreads, (n + per - 1) / per);
  if (parts <= 1) {
    fn((size_t)0, n);
    return;
  }
  const size_t chunk = (n + parts - 1) / parts;
  std::vector<std::function<void()>> tasks;
  tasks.reserve(parts - 1);
  for (int i = 1; i < parts; i++) {
    const size_t b = (size_t)i * chunk, e = std::min(n, b + chunk);
    tasks.emplace_back([=, &fn] { fn(b, e); });
  }
  HostPool::get().run(tasks, [&] { fn((size_t)0, std::min(n, chunk)); });
}

// device bytes of one pipeline's work buffers for `rows` padded rows
size_t work_bytes(int set, int kind, long long rows) {
  const gmc_setinfo &S = set_info(set);
  const size_t ew = (size_t)round_up((S.n + 31) / 32, 4), kw = (size_t)round_up((S.k + 31) / 32, kGemmKTile),
               mw = (size_t)round_up((S.mt + 31) / 32, 4), cw = (size_t)round_up((S.synd_bytes + 3) / 4, kGemmKTile),
               s2 = (size_t)round_up((2 * S.t * S.m + 31) / 32, 4);
  if (kind == 0) return align256(rows * ew * 4) + align256(rows * kw * 4) + align256(rows * mw * 4);
  // decapsulation rows are laid out for either form, so the constant-time switch can change between batches
  const size_t ewd = (size_t)dec_e_words(set, true);
  return align256(rows * cw * 4) + align256(rows * s2 * 4) + align256(rows * (2u << S.fft_d)) +
         align256(rows * ewd * 4) + align256(rows * 4);
}

}  // namespace

struct gmc_server {
  int device = 0;
  long long max_batch = 0;
  std::vector<Slot> slots;
  std::set<const gmc_key *> keys;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Req> queue;
  std::thread dispatcher;
  bool stop = false;
  // finished batches, handed from the CUDA host callback to the completion thread
  std::mutex done_mu;
  std::condition_variable done_cv;
  std::deque<Slot *> done_q;
  bool done_stop = false;
  std::thread completer;
  // statistics (under mu)
  std::vector<long long> hist = std::vector<long long>(kBuckets, 0);
  long long completed = 0, batches = 0, batched_requests = 0, errors = 0;
  double t_first = 0, t_last = 0;
  // the batch whose oldest request waited longest (arrival to results), by stage, and batches over 5 ms
  double worst[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long slow_batches = 0;
  std::string last_error;
};

namespace {

template <int SET>
cudaError_t run_pipe(Slot &sl, Pipe &pp, cudaStream_t pst) {
  const long long rows = seg_rows(pp.segs);
  uint8_t *in = sl.dev + pp.in_off, *kout = sl.dev + pp.k_off;
  uint8_t *work = sl.dev + pp.work_off;
  const gmc_key *ref = pp.keys[0];
  const SetTune tune = tune_get(SET);
  const int ov = gmc_get_gemm_engine();
  // a sparse override applies to encapsulation only (c is dense)
  const int engine = (ov >= 0 && !(pp.kind && ov == GEMM_SPARSE)) ? ov : (pp.kind ? tune.dec_engine : tune.enc_engine);
  GemmKeys gk{};
  for (size_t i = 0; i < pp.keys.size(); i++) {
    gk.A[i] = pp.kind == 0 ? pp.keys[i]->T : pp.keys[i]->F;
    gk.A8[i] = pp.keys[i]->a8;
    gk.TT[i] = pp.keys[i]->TT;
    gk.ldtt = pp.keys[i]->ldtt;
    gk.tc_stages = tune.gemm_stages;
    if (engine == GEMM_TC && !gk.A8[i]) return cudaErrorInvalidValue;  // registered keys carry their images
  }
  const gmc_setinfo &S = set_info(SET);
  using p = P<SET>;
  const int ew = round_up((S.n + 31) / 32, 4);
  if (pp.kind == 0) {
    const int kw = ref->kw_pad, mw = round_up((S.mt + 31) / 32, 4);
    uint32_t *E = (uint32_t *)work, *Ens = (uint32_t *)(work + align256(rows * ew * 4)),
             *Sy = (uint32_t *)(work + align256(rows * ew * 4) + align256(rows * kw * 4));
    uint32_t bad = 0;
    for (size_t i = 0; i < pp.keys.size(); i++)
      if (pp.keys[i]->pad_bad) bad |= 1u << i;
    cudaError_t e;
    if (engine == GEMM_SPARSE) {
      e = launch_sample<SET>(in, pp.segs, E, ew, Ens, kw, &gk, Sy, mw, tune.sample_threads,
                             reinterpret_cast<unsigned int *>(Ens), pst, tune.sample_sm_warps);
    } else {
      e = launch_sample<SET>(in, pp.segs, E, ew, Ens, kw, nullptr, Sy, mw, tune.sample_threads,
                             reinterpret_cast<unsigned int *>(Sy), pst, tune.sample_sm_warps);
      if (e == cudaSuccess)
        e = launch_gf2_gemm_seg(engine, gk, pp.segs, ref->lda, ref->rows_pad, Ens, kw, ref->kw_pad, Sy, mw, p::mw,
                                tc_err_word_ptr(), pst);
    }
    if (e == cudaSuccess)
      e = launch_finalize<SET>(E, ew, Sy, mw, sl.dev + pp.ct_off, kout, pp.segs, bad, pp.pc != 0, pst);
    return e;
  }
  const int cw = ref->cw_pad, s2 = round_up((2 * S.t * S.m + 31) / 32, 4);
  const bool ct = dec_constant_time();
  const int ewd = dec_e_words(SET, ct);
  uint8_t *q = work;
  uint32_t *X = (uint32_t *)q;
  q += align256(rows * cw * 4);
  uint32_t *S2 = (uint32_t *)q;
  q += align256(rows * s2 * 4);
  uint16_t *Sig = (uint16_t *)q;
  q += align256(rows * (2u << S.fft_d));
  uint32_t *E = (uint32_t *)q;
  q += align256(rows * (size_t)dec_e_words(SET, true) * 4);
  int *ok = (int *)q;
  FieldDev fd;
  if (field_tables(SET, &fd) != GMC_OK) return cudaErrorUnknown;
  DecKeys dk{};
  for (size_t i = 0; i < pp.keys.size(); i++) dk.k[i] = pp.keys[i]->dk;
  cudaError_t e = launch_pack_ct<SET>(in, pp.segs, X, cw, pp.pc != 0, pst);
  if (e == cudaSuccess)
    e = launch_gf2_gemm_seg(engine, gk, pp.segs, ref->ldf, ref->frows_pad, X, cw, ref->cw_pad, S2, s2, p::s2w,
                            tc_err_word_ptr(), pst);
  if (e == cudaSuccess) e = launch_dec_bm<SET>(S2, s2, fd, pp.segs, Sig, pst, tune.bm_warps, ct);
  if (e == cudaSuccess) e = launch_dec_root<SET>(Sig, S2, s2, dk, fd, pp.segs, E, ewd, ok, pst, tune.root_warps, ct);
  if (e == cudaSuccess && ct) {
    // the keys' first-t syndrome matrices are built on a key's first constant-time batch
    GemmKeys ctk;
    e = ct_gemm_keys(pp.keys.data(), (int)pp.keys.size(), engine, pst, &ctk);
    if (e == cudaSuccess)
      e = launch_dec_ct_finish<SET>(dk, ctk, engine, pp.segs, E, ewd, S2, s2, X, cw, ok, tc_err_word_ptr(), pst);
  }
  if (e == cudaSuccess)
    e = launch_dec_tail<SET>(E, ewd, ok, in, dk, kout, (int *)(sl.dev + pp.rc_off), pp.segs, pp.pc != 0, pst);
  return e;
}

// CUDA host callback at the end of a batch's stream work: only hands the slot
// to the completion thread (host functions run on the driver's callback
// thread, which the other slots' completions share).
void CUDART_CB on_batch_done(void *arg) {
  Slot *sl = (Slot *)arg;
  gmc_server *srv = sl->srv;
  sl->t_done = now_s();
  {
    std::lock_guard<std::mutex> lk(srv->done_mu);
    srv->done_q.push_back(sl);
  }
  srv->done_cv.notify_one();
}

// Scatters a finished batch's results, marks its requests done, records their
// latency (arrival to the results being in the caller's buffers) and frees
// the slot.
void complete_batch(Slot *sl) {
  gmc_server *srv = sl->srv;
  // scatter results, then bucket latencies (outside the lock), in parallel pieces
  const int parts = kHostThreads;
  std::vector<std::vector<long long>> local(parts, std::vector<long long>(kBuckets, 0));
  std::atomic<int> next_part{0};
  parallel_for(sl->pieces.size(), [&](size_t b, size_t e) {
    std::vector<long long> &h = local[next_part.fetch_add(1) % parts];
    for (size_t i = b; i < e; i++) {
      Piece &pc = sl->pieces[i];
      const Req &r = *pc.r;
      memcpy(r.k, sl->h_out + pc.out_k, 32);
      if (r.key->kind == 0) {
        memcpy(r.ct, sl->h_out + pc.out_ct, ct_len(r.key->set, r.key->pc));
        if (r.rc) *r.rc = r.key->pad_bad ? -1 : 0;
      } else if (r.rc) {
        memcpy(r.rc, sl->h_out + pc.out_rc, 4);
      }
    }
    const double t = now_s();  // this piece's results are in place
    double last_t = -1.0;
    int last_b = 0;
    for (size_t i = b; i < e; i++) {
      Piece &pc = sl->pieces[i];
      if (pc.r->t_arrive != last_t) {  // requests of a batch often share their bucket
        last_t = pc.r->t_arrive;
        last_b = bucket_of((t - last_t) * 1e3);
      }
      h[last_b]++;
      if (pc.r->done) pc.r->done->store(1, std::memory_order_release);
    }
  });
  const double t = now_s();
  std::lock_guard<std::mutex> lk(srv->mu);
  for (auto &h : local)
    for (int b = 0; b < kBuckets; b++) srv->hist[b] += h[b];
  srv->completed += (long long)sl->pieces.size();
  srv->t_last = t;
  const double lat = (t - sl->t_oldest) * 1e3;
  if (lat > 5.0) srv->slow_batches++;
  if (lat > srv->worst[0]) {
    srv->worst[0] = lat;
    srv->worst[1] = (sl->t_take - sl->t_oldest) * 1e3;      // waiting in the queue (no free slot yet)
    srv->worst[2] = (sl->t_taken - sl->t_take) * 1e3;       // moving the requests out of the queue
    srv->worst[3] = (sl->t_bucketed - sl->t_taken) * 1e3;   // grouping them by key, admission, layout
    srv->worst[4] = (sl->t_formed - sl->t_bucketed) * 1e3;  // copying the inputs into pinned staging
    srv->worst[5] = (sl->t_issued - sl->t_formed) * 1e3;    // issuing copies and kernels
    srv->worst[6] = (sl->t_done - sl->t_issued) * 1e3;      // device work, copies and the callback
    srv->worst[7] = (t - sl->t_done) * 1e3;                 // scattering the results
  }
  sl->busy = false;
  srv->cv.notify_all();
}

void completer_main(gmc_server *srv) {
  while (true) {
    Slot *sl = nullptr;
    {
      std::unique_lock<std::mutex> lk(srv->done_mu);
      srv->done_cv.wait(lk, [&] { return !srv->done_q.empty() || srv->done_stop; });
      if (srv->done_q.empty()) break;  // stopping, nothing left
      sl = srv->done_q.front();
      srv->done_q.pop_front();
    }
    complete_batch(sl);
  }
}

// device bytes of one pipeline (inputs, outputs, work) for `rows` padded rows
size_t pipe_bytes(int set, int kind, int pc, long long rows) {
  if (rows <= 0) return 0;
  const size_t inb = kind == 0 ? 32 : ct_len(set, pc);
  return align256(rows * inb) + align256(rows * 32) + align256(rows * ct_len(set, pc)) + align256(rows * 4) +
         work_bytes(set, kind, rows);
}

// staging bytes of one pipeline (padded rows, same layout as on the device)
size_t in_bytes(int set, int kind, int pc, long long rows) {
  if (rows <= 0) return 0;
  return align256(rows * (kind == 0 ? 32 : ct_len(set, pc)));
}
size_t out_bytes(int set, int kind, int pc, long long rows) {
  if (rows <= 0) return 0;
  return align256(rows * 32) + (kind == 0 ? align256(rows * ct_len(set, pc)) : align256(rows * 4));
}

// the largest padding a batch can carry: kPipes pipelines of kMaxSegs keys
constexpr long long kPadRows = (long long)kPipes * kMaxSegs * kGemmOpPad;

// Lays out the next batch in a free slot from sl.incoming (moved out of the
// queue by the dispatcher). Requests are taken in order while they fit the
// slot's arena and staging (admission by device memory); the rest go back to
// the queue front. Per request the work is O(1): sizes change only when a
// key's row count crosses a multiple of kGemmOpPad or a key joins a pipeline.
// Returns false when nothing was taken.
bool form_batch(gmc_server *srv, Slot &sl) {
  sl.pieces.clear();
  sl.pipes.clear();
  struct KeyAcc {
    const gmc_key *key;
    std::vector<int> *members;  // from the slot's pool
  };
  size_t pool_used = 0;
  auto member_list = [&]() {
    if (pool_used == sl.member_pool.size()) sl.member_pool.emplace_back();
    std::vector<int> *v = &sl.member_pool[pool_used++];
    v->clear();
    return v;
  };
  struct Acc {
    std::vector<KeyAcc> keys;
    int last = -1;
    long long rows = 0;
  };
  Acc by[GMC_NSETS][2][2];  // [set][op][pc]
  size_t in_b = 0, out_b = 0, dev_need = 0;
  size_t taken = 0;
  for (auto it = sl.incoming.cbegin(); it != sl.incoming.cend(); ++it, taken++) {
    const Req &r = *it;
    const int kind = r.key->kind, set = r.key->set, pc = r.key->pc ? 1 : 0;
    Acc &acc = by[set][kind][pc];
    int ki = acc.last;
    if (ki < 0 || acc.keys[ki].key != r.key) {
      ki = -1;
      for (size_t i = 0; i < acc.keys.size(); i++)
        if (acc.keys[i].key == r.key) {
          ki = (int)i;
          break;
        }
    }
    const size_t cnt = ki < 0 ? 0 : acc.keys[ki].members->size();
    if (cnt % kGemmOpPad == 0) {  // a new padded block of rows (or a new key): re-check the admission
      if (ki < 0 && acc.keys.size() >= (size_t)kMaxSegs) break;  // one pipeline per (set, op)
      const long long rows_new = acc.rows + kGemmOpPad;
      const size_t dev_new = dev_need - pipe_bytes(set, kind, pc, acc.rows) + pipe_bytes(set, kind, pc, rows_new);
      const size_t in_new = in_b - in_bytes(set, kind, pc, acc.rows) + in_bytes(set, kind, pc, rows_new);
      const size_t out_new = out_b - out_bytes(set, kind, pc, acc.rows) + out_bytes(set, kind, pc, rows_new);
      if (in_new > sl.h_in_bytes || out_new > sl.h_out_bytes || dev_new > sl.dev_bytes) break;
      acc.rows = rows_new;
      dev_need = dev_new;
      in_b = in_new;
      out_b = out_new;
      if (ki < 0) {
        acc.keys.push_back({r.key, member_list()});
        ki = (int)acc.keys.size() - 1;
      }
    }
    acc.last = ki;
    acc.keys[ki].members->push_back((int)sl.pieces.size());
    sl.pieces.push_back({&r, 0, 0, 0});
  }
  if (taken < sl.incoming.size()) {  // what did not fit waits for the next batch, in order
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      for (size_t i = sl.incoming.size(); i-- > taken;) srv->queue.push_front(sl.incoming[i]);
    }
    sl.incoming.resize(taken);  // the pieces point at the requests kept (the front of the deque)
  }
  if (sl.pieces.empty()) return false;
  // device layout: [inputs of all pipes][outputs of all pipes][work of each pipe]
  size_t off = 0;
  for (int set = 0; set < GMC_NSETS; set++)
    for (int kind = 0; kind < 2; kind++)
      for (int pc = 0; pc < 2; pc++) {
        Acc &acc = by[set][kind][pc];
        if (acc.keys.empty()) continue;
        Pipe pp{};
        pp.set = set;
        pp.kind = kind;
        pp.pc = pc;
        pp.segs = Segs{};
        long long row = 0;
        for (auto &kk : acc.keys) {
          pp.segs.row0[pp.keys.size()] = row;
          pp.segs.nreq[pp.keys.size()] = (long long)kk.members->size();
          row += (long long)((kk.members->size() + kGemmOpPad - 1) / kGemmOpPad) * kGemmOpPad;
          pp.keys.push_back(kk.key);
          pp.members.push_back(kk.members);
        }
        pp.segs.nseg = (int)pp.keys.size();
        pp.segs.row0[pp.keys.size()] = row;
        pp.in_off = off;
        off += align256(row * (pp.kind == 0 ? 32 : ct_len(pp.set, pp.pc)));
        sl.pipes.push_back(std::move(pp));
      }
  sl.in_used = off;
  for (auto &pp : sl.pipes) {
    const long long row = seg_rows(pp.segs);
    pp.k_off = off;
    off += align256(row * 32);
    pp.ct_off = off;
    if (pp.kind == 0) off += align256(row * ct_len(pp.set, pp.pc));
    pp.rc_off = off;
    if (pp.kind == 1) off += align256(row * 4);
  }
  sl.out_used = off - sl.in_used;
  for (auto &pp : sl.pipes) {
    pp.work_off = off;
    off += work_bytes(pp.set, pp.kind, seg_rows(pp.segs));
  }
  if (sl.in_used > sl.h_in_bytes || sl.out_used > sl.h_out_bytes || off > sl.dev_bytes) {
    // cannot happen when the admission above holds; never write past the buffers
    std::lock_guard<std::mutex> lk(srv->mu);
    for (size_t i = sl.pieces.size(); i-- > 0;) srv->queue.push_front(*sl.pieces[i].r);
    sl.pieces.clear();
    return false;
  }
  sl.t_bucketed = now_s();
  // gather inputs into pinned staging, mirroring the device input layout: one
  // parallel pass over the batch's (pipeline, key) segments laid end to end
  // (a pass per segment left the many small segments of a mixed batch on the
  // dispatcher thread alone)
  struct SegRef {
    Pipe *pp;
    int sg;
    size_t first;  // index of the segment's first member in the flat order
  };
  std::vector<SegRef> segs;
  size_t total = 0;
  for (auto &pp : sl.pipes)
    for (size_t sg = 0; sg < pp.keys.size(); sg++) {
      segs.push_back({&pp, (int)sg, total});
      total += pp.members[sg]->size();
    }
  parallel_for(total, [&](size_t b, size_t e) {
    // the segment holding flat index b, then walk forward
    size_t si = (size_t)(std::upper_bound(segs.begin(), segs.end(), b,
                                          [](size_t x, const SegRef &r) { return x < r.first; }) -
                         segs.begin()) - 1;
    for (size_t f = b; f < e; f++) {
      while (si + 1 < segs.size() && segs[si + 1].first <= f) si++;
      const SegRef &sr = segs[si];
      const Pipe &pp = *sr.pp;
      const size_t ctb = ct_len(pp.set, pp.pc);
      const size_t inb = pp.kind == 0 ? 32 : ctb;
      const size_t j = f - sr.first;
      Piece &pc = sl.pieces[(*pp.members[sr.sg])[j]];
      const long long row = pp.segs.row0[sr.sg] + (long long)j;
      memcpy(sl.h_in + pp.in_off + row * inb, pc.r->in, inb);
      pc.out_k = pp.k_off - sl.in_used + row * 32;
      pc.out_ct = pp.ct_off - sl.in_used + row * ctb;
      pc.out_rc = pp.rc_off - sl.in_used + row * 4;
    }
  });
  return true;
}

void dispatcher_main(gmc_server *srv) {
  cudaSetDevice(srv->device);
  std::unique_lock<std::mutex> lk(srv->mu);
  while (true) {
    Slot *free_slot = nullptr;
    srv->cv.wait(lk, [&] {
      if (srv->stop) return true;
      if (srv->queue.empty()) return false;
      for (auto &s : srv->slots)
        if (!s.busy) {
          free_slot = &s;
          return true;
        }
      return false;
    });
    if (srv->stop) break;
    Slot &sl = *free_slot;
    sl.busy = true;  // reserved while its batch is formed outside the lock
    const size_t take = std::min(srv->queue.size(), (size_t)srv->max_batch);
    sl.t_take = now_s();
    sl.t_oldest = srv->queue.front().t_arrive;  // first in, first out: the batch's oldest request
    sl.incoming.clear();  // the slot's previous batch is complete
    if (take == srv->queue.size()) {
      sl.incoming.swap(srv->queue);  // the whole queue: no copy under the lock
    } else {
      sl.incoming.assign(srv->queue.begin(), srv->queue.begin() + (long)take);
      srv->queue.erase(srv->queue.begin(), srv->queue.begin() + (long)take);
    }
    sl.t_taken = now_s();
    lk.unlock();
    const bool formed = form_batch(srv, sl);
    sl.t_formed = now_s();
    lk.lock();
    if (!formed) {  // the head request does not fit an empty slot: reject it
      sl.busy = false;
      if (!srv->queue.empty()) {
        srv->errors++;
        srv->last_error = "request does not fit a slot";
        Req r = srv->queue.front();
        srv->queue.pop_front();
        if (r.done) r.done->store(-1);
      }
      continue;
    }
    srv->batches++;
    srv->batched_requests += (long long)sl.pieces.size();
    lk.unlock();
    const char *step = "input copy";
    cudaError_t e = cudaMemcpyAsync(sl.dev, sl.h_in, sl.in_used, cudaMemcpyHostToDevice, sl.st);
    if (e == cudaSuccess) e = cudaEventRecord(sl.fork, sl.st);
    for (size_t i = 0; i < sl.pipes.size() && e == cudaSuccess; i++) {
      Pipe &pp = sl.pipes[i];
      step = pp.kind == 0 ? "encapsulation kernels" : "decapsulation kernels";
      e = cudaStreamWaitEvent(sl.pst[i], sl.fork, 0);
      if (e != cudaSuccess) break;
      switch (pp.set) {
        case 0: e = run_pipe<0>(sl, pp, sl.pst[i]); break;
        case 1: e = run_pipe<1>(sl, pp, sl.pst[i]); break;
        case 2: e = run_pipe<2>(sl, pp, sl.pst[i]); break;
        case 3: e = run_pipe<3>(sl, pp, sl.pst[i]); break;
        default: e = run_pipe<4>(sl, pp, sl.pst[i]); break;
      }
      if (e == cudaSuccess) e = cudaEventRecord(sl.join[i], sl.pst[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(sl.st, sl.join[i], 0);
    }
    if (e == cudaSuccess) {
      step = "output copy";
      e = cudaMemcpyAsync(sl.h_out, sl.dev + sl.in_used, sl.out_used, cudaMemcpyDeviceToHost, sl.st);
    }
    sl.t_issued = now_s();
    if (e == cudaSuccess) {
      step = "completion callback";
      e = cudaLaunchHostFunc(sl.st, on_batch_done, &sl);
    }
    lk.lock();
    if (e != cudaSuccess) {
      srv->errors += (long long)sl.pieces.size();
      srv->last_error = std::string(step) + ": " + cudaGetErrorString(e);
      for (auto &pc : sl.pieces)
        if (pc.r->done) pc.r->done->store(-1);
      sl.busy = false;
    }
  }
}

void server_release(gmc_server *s) {
  if (!s) return;
  if (s->dispatcher.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv.notify_all();
    s->dispatcher.join();
  }
  // every batch's device work and host callback ends before the completion
  // thread is stopped (it finishes what the callbacks handed it) and before
  // the slots' buffers go
  for (auto &sl : s->slots) {
    for (int i = 0; i < kPipes; i++)
      if (sl.pst[i]) cudaStreamSynchronize(sl.pst[i]);
    if (sl.st) cudaStreamSynchronize(sl.st);
  }
  if (s->completer.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->done_mu);
      s->done_stop = true;
    }
    s->done_cv.notify_all();
    s->completer.join();
  }
  for (auto &sl : s->slots) {
    if (sl.st) cudaStreamDestroy(sl.st);
    for (int i = 0; i < kPipes; i++) {
      if (sl.pst[i]) cudaStreamDestroy(sl.pst[i]);
      if (sl.join[i]) cudaEventDestroy(sl.join[i]);
    }
    if (sl.fork) cudaEventDestroy(sl.fork);
    cudaFree(sl.dev);
    cudaFreeHost(sl.h_in);
    cudaFreeHost(sl.h_out);
  }
  delete s;
}

int srv_fail(int code, const char *msg) {
  set_last_error(msg);
  return code;
}

}  // namespace

extern "C" int gmc_server_create(gmc_server **out, long long max_batch, int slots, double mem_fraction) {
  if (!out || max_batch <= 0 || slots <= 0 || slots > 16 || mem_fraction <= 0 || mem_fraction > 0.9)
    return srv_fail(GMC_EINVAL, "gmc_server_create: bad argument");
  *out = nullptr;
  gmc_server *s = new gmc_server();
  cudaGetDevice(&s->device);
  s->max_batch = max_batch;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    delete s;
    return srv_fail(GMC_ECUDA, "gmc_server_create: cudaMemGetInfo failed");
  }
  // per-slot arena: the worst case of a full batch of the largest set, capped by the memory budget
  const size_t per_req = 2 * 1024 + 1536;
  size_t arena = align256((size_t)max_batch * per_req + (size_t)kMaxSegs * 4 * kGemmOpPad * per_req);
  const size_t budget = (size_t)(mem_fraction * (double)free_b) / (size_t)slots;
  if (arena > budget) arena = budget;
  s->slots.resize(slots);
  cudaError_t e = cudaSuccess;
  for (auto &sl : s->slots) {
    sl.srv = s;
    sl.dev_bytes = arena;
    sl.h_in_bytes = (size_t)(max_batch + kPadRows) * 240 + kPipes * 256;
    sl.h_out_bytes = (size_t)(max_batch + kPadRows) * (240 + 32 + 4) + 3 * kPipes * 256;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
    for (int i = 0; i < kPipes && e == cudaSuccess; i++) {
      e = cudaStreamCreateWithFlags(&sl.pst[i], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&sl.dev, sl.dev_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_in, sl.h_in_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_out, sl.h_out_bytes);
  }
  if (e != cudaSuccess) {
    server_release(s);
    return srv_fail(GMC_ENOMEM, "gmc_server_create: slot allocation failed");
  }
  s->completer = std::thread(completer_main, s);
  s->dispatcher = std::thread(dispatcher_main, s);
  *out = s;
  return GMC_OK;
}

extern "C" int gmc_server_add_key(gmc_server *s, const gmc_key *key) {
  if (!s || !key) return srv_fail(GMC_EINVAL, "gmc_server_add_key: bad argument");
  // resident state needed by every engine choice is built now, outside the request path
  int r = key_prepare_resident(key);
  if (r) return r;
  if (!tc_err_word_ptr()) return srv_fail(GMC_ECUDA, "gmc_server_add_key: error word");
  std::lock_guard<std::mutex> lk(s->mu);
  s->keys.insert(key);
  return GMC_OK;
}

extern "C" int gmc_server_submit(gmc_server *s, const gmc_key *key, const unsigned char *in, unsigned char *ct,
                                 unsigned char *k, int *rc, int *done) {
  if (!s || !key || !in || !k || (key->kind == 0 && !ct)) return srv_fail(GMC_EINVAL, "gmc_server_submit: bad argument");
  Req r{key, in, ct, k, rc, now_s(), reinterpret_cast<std::atomic<int> *>(done)};
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->keys.count(key)) return srv_fail(GMC_EKEY, "gmc_server_submit: key not registered");
    if (!s->t_first) s->t_first = r.t_arrive;
    s->queue.push_back(r);
  }
  s->cv.notify_all();
  return GMC_OK;
}

extern "C" int gmc_server_drain(gmc_server *s, double timeout_s) {
  if (!s) return srv_fail(GMC_EINVAL, "gmc_server_drain: bad argument");
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    if (!s->queue.empty()) return false;
    for (auto &sl : s->slots)
      if (sl.busy) return false;
    return true;
  });
  return ok ? GMC_OK : srv_fail(GMC_ECUDA, "gmc_server_drain: timed out");
}

extern "C" int gmc_server_stats(gmc_server *s, double *out /* [8] */) {
  if (!s || !out) return srv_fail(GMC_EINVAL, "gmc_server_stats: bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  long long tot = 0;
  for (long long c : s->hist) tot += c;
  auto pct = [&](double q) {
    if (!tot) return 0.0;
    long long acc = 0, target = (long long)ceil(q * tot);
    for (int b = 0; b < kBuckets; b++) {
      acc += s->hist[b];
      if (acc >= target) return bucket_ms(b);
    }
    return bucket_ms(kBuckets - 1);
  };
  out[0] = (double)s->completed;
  out[1] = (double)s->batches;
  out[2] = s->batches ? (double)s->batched_requests / (double)s->batches : 0.0;
  out[3] = pct(0.50);
  out[4] = pct(0.99);
  out[5] = (s->t_last > s->t_first) ? (double)s->completed / (s->t_last - s->t_first) : 0.0;
  out[6] = (double)s->errors;
  out[7] = (double)s->slots.size();
  return GMC_OK;
}

extern "C" int gmc_server_latency_ms(gmc_server *s, double q, double *ms) {
  if (!s || !ms || !(q > 0.0 && q <= 1.0)) return srv_fail(GMC_EINVAL, "gmc_server_latency_ms: bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  long long tot = 0;
  for (long long c : s->hist) tot += c;
  *ms = 0.0;
  if (!tot) return GMC_OK;
  const long long target = (long long)ceil(q * (double)tot);
  long long acc = 0;
  for (int b = 0; b < kBuckets; b++) {
    acc += s->hist[b];
    if (acc >= target) {
      *ms = bucket_ms(b);
      return GMC_OK;
    }
  }
  *ms = bucket_ms(kBuckets - 1);
  return GMC_OK;
}

extern "C" int gmc_server_worst_batch(gmc_server *s, double *out /* [10] */) {
  if (!s || !out) return srv_fail(GMC_EINVAL, "gmc_server_worst_batch: bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  for (int i = 0; i < 8; i++) out[i] = s->worst[i];
  out[8] = (double)s->batches;
  out[9] = (double)s->slow_batches;
  return GMC_OK;
}

extern "C" int gmc_server_reset_stats(gmc_server *s) {
  if (!s) return srv_fail(GMC_EINVAL, "gmc_server_reset_stats: bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::fill(s->hist.begin(), s->hist.end(), 0);
  s->completed = s->batches = s->batched_requests = s->errors = 0;
  std::fill(s->worst, s->worst + 8, 0.0);
  s->slow_batches = 0;
  s->t_first = s->t_last = 0;
  return GMC_OK;
}

extern "C" void gmc_server_destroy(gmc_server *s) { server_release(s); }

extern "C" const char *gmc_server_error(gmc_server *s) {
  if (!s) return "";
  std::lock_guard<std::mutex> lk(s->mu);
  thread_local std::string copy;
  copy = s->last_error;
  return copy.c_str();
}

// Open-loop load generator: Poisson arrivals at `rate` requests/s for `seconds`
// over the given (public key, secret key) pairs, encapsulation with probability
// enc_fraction, a uniformly chosen pair per request. Decapsulation requests
// draw from pool_n valid ciphertexts per pair made at start. Latency is
// measured from each request's scheduled arrival time.
extern "C" int gmc_server_loadgen(gmc_server *s, const gmc_key *const *pks, const gmc_key *const *sks, int npairs,
                                  double rate, double seconds, double enc_fraction, unsigned long long seed,
                                  double *out /* [8] */) {
  if (!s || !pks || !sks || npairs <= 0 || rate <= 0 || seconds <= 0 || !out)
    return srv_fail(GMC_EINVAL, "gmc_server_loadgen: bad argument");
  for (int i = 0; i < npairs; i++)  // each pair's ciphertext pool is sized by its public key
    if (!pks[i] || !sks[i] || pks[i]->kind != 0 || sks[i]->kind != 1 || pks[i]->set != sks[i]->set ||
        pks[i]->pc != sks[i]->pc)
      return srv_fail(GMC_EINVAL, "gmc_server_loadgen: pair i must be a public and a secret key of one set and form");
  constexpr int pool_n = 256;
  std::vector<std::vector<uint8_t>> cts(npairs);
  std::vector<uint8_t> seeds((size_t)pool_n * 32);
  std::mt19937_64 rng(seed);
  for (auto &b : seeds) b = (uint8_t)rng();
  for (int i = 0; i < npairs; i++) {
    cts[i].resize((size_t)pool_n * ct_len(pks[i]->set, pks[i]->pc));
    std::vector<uint8_t> kk((size_t)pool_n * 32);
    int r = gmc_enc_batch(pks[i], cts[i].data(), kk.data(), seeds.data(), pool_n, nullptr);
    if (r) return r;
  }
  // output sinks (results are overwritten; correctness is checked by the tests on small runs)
  const size_t ring = 1 << 16;
  constexpr size_t kSinkCt = 256;  // the longest ciphertext (8192128 with plaintext confirmation: 240 bytes)
  std::vector<uint8_t> sink_ct(ring * kSinkCt), sink_k(ring * 32);
  std::vector<int> sink_rc(ring);
  gmc_server_reset_stats(s);
  // Arrivals come from kGenThreads generator threads, each a Poisson process at
  // rate / kGenThreads (their superposition is Poisson at `rate`): one thread's
  // per-request work (draws, logarithm, queue push) capped the offered rate
  // near the server's peak, and a request's latency counts from its scheduled
  // arrival, so a lagging generator showed up as queueing delay.
  constexpr int kGenThreads = 4;
  const size_t per_ring = ring / kGenThreads;
  const size_t queue_cap = (size_t)4 * (size_t)s->max_batch * s->slots.size();  // bounds host memory under overload
  const double t0 = now_s();
  std::atomic<long long> submitted{0};
  auto generate = [&](int gi) {
    // splitmix64 draws
    uint64_t sm = (seed + 0x632BE59BD9B4E019ull * (uint64_t)(gi + 1)) ^ 0x9E3779B97F4A7C15ull;
    auto next64 = [&]() {
      uint64_t z = (sm += 0x9E3779B97F4A7C15ull);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      return z ^ (z >> 31);
    };
    auto unit = [&]() { return (double)(next64() >> 11) * (1.0 / 9007199254740992.0); };  // [0, 1)
    const double grate = rate / kGenThreads;
    double t_next = t0 - log1p(-unit()) / grate;
    size_t idx = 0;
    long long mine = 0;
    std::vector<Req> due;
    while (true) {
      const double t = now_s();
      if (t - t0 > seconds) break;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->queue.size() > queue_cap) {
          t_next = std::max(t_next, t);  // arrivals while the queue is over its cap are not offered
        }
      }
      due.clear();
      while (t_next <= t && due.size() < (1u << 18)) {
        const uint64_t x = next64();
        const int pair = (int)(((x & 0xFFFFFFFFull) * (uint64_t)npairs) >> 32);
        const bool enc = (double)(x >> 40) * (1.0 / 16777216.0) < enc_fraction;
        const size_t slot = gi * per_ring + idx++ % per_ring;
        const int pi = (int)((x >> 32) & 0xFF) % pool_n;
        Req r{};
        r.key = enc ? pks[pair] : sks[pair];
        r.in = enc ? seeds.data() + (size_t)pi * 32
                   : cts[pair].data() + (size_t)pi * ct_len(sks[pair]->set, sks[pair]->pc);
        r.ct = sink_ct.data() + slot * kSinkCt;
        r.k = sink_k.data() + slot * 32;
        r.rc = &sink_rc[slot];
        r.t_arrive = t_next;
        r.done = nullptr;
        due.push_back(r);
        t_next += -log1p(-unit()) / grate;  // exponential inter-arrival gap
      }
      if (!due.empty()) {
        {
          std::lock_guard<std::mutex> lk(s->mu);
          if (!s->t_first) s->t_first = t0;
          s->queue.insert(s->queue.end(), due.begin(), due.end());
        }
        s->cv.notify_all();
        mine += (long long)due.size();
      } else {
        std::this_thread::yield();
      }
    }
    submitted += mine;
  };
  std::vector<std::thread> gens;
  for (int gi = 1; gi < kGenThreads; gi++) gens.emplace_back(generate, gi);
  generate(0);
  for (auto &g : gens) g.join();
  int r = gmc_server_drain(s, 60.0);
  double st[8];
  gmc_server_stats(s, st);
  out[0] = (double)submitted.load();
  out[1] = st[0];                       // completed
  out[2] = st[0] / (now_s() - t0);      // achieved ops/s over the run (incl. drain)
  out[3] = st[3];                       // p50 ms
  out[4] = st[4];                       // p99 ms
  out[5] = st[2];                       // mean batch size
  out[6] = st[1];                       // batches
  out[7] = (double)submitted.load() / seconds; // offered rate
  return r;
}
