// Internal layout of a resident key handle, shared by the engine's
// translation units (not part of the C ABI).
#pragma once
#include <stdint.h>

#include <mutex>

#include "kernels.h"

struct gmc_key {
  int set = 0;
  int kind = 0;  // 0 public, 1 secret
  int device = 0;
  // public key
  uint32_t *T = nullptr;
  int lda = 0, rows_pad = 0, kw_pad = 0, pad_bad = 0;
  // secret key
  uint32_t *F = nullptr;
  int ldf = 0, frows_pad = 0, cw_pad = 0;
  uint16_t *tabs = nullptr;  // L | LL | LW2 (n each) | invL (2^m)
  uint8_t *a8 = nullptr;     // FP8 stage images of T (public) or F (secret) for the tensor-core engine
  std::mutex *a8_mu = nullptr;
  uint8_t *s = nullptr;
  gmc::DecKeyDev dk{};
};


namespace gmc {
// sets the calling thread's message returned by gmc_last_error()
void set_last_error(const char *msg);
}  // namespace gmc
