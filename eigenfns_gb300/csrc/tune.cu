// Runtime schedule overrides chosen by the autotuner (eigenfns_gb300/tune.py).
//
// The Gram kernel choice (tensor cores or CUDA cores) and the tensor-core Gram's
// work units per SM (the split of K into chunks: more units balance the SMs better,
// fewer units cut the fp64 partial traffic and the reduction) are looked up per
// (ma, mb) shape at every call; shapes without an entry use the built-in defaults.
#include <mutex>

#include "common.cuh"
#include "status.h"

namespace ef {

namespace {
struct GramTune {
  int ma, mb, kernel, units;
};
constexpr int kMaxGramTunes = 256;
GramTune g_gram[kMaxGramTunes];
int g_gram_n = 0;
std::mutex g_gram_mu;
}  // namespace

bool gram_tune_get(int ma, int mb, int* kernel, int* units) {
  std::lock_guard<std::mutex> lock(g_gram_mu);
  for (int i = 0; i < g_gram_n; ++i) {
    if (g_gram[i].ma == ma && g_gram[i].mb == mb) {
      if (kernel) *kernel = g_gram[i].kernel;
      if (units) *units = g_gram[i].units;
      return true;
    }
  }
  return false;
}

}  // namespace ef

extern "C" {

int ef_tune_gram(int ma, int mb, int kernel, int units_per_sm) {
  if (ma <= 0 || mb <= 0) return ef_fail(EF_ERR_INVALID, "tune_gram: shape must be positive");
  if (kernel < 0 || kernel > 2) return ef_fail(EF_ERR_INVALID, "tune_gram: kernel is 0 (default), 1 (tensor cores) or 2 (CUDA cores)");
  if (units_per_sm < 0 || units_per_sm > 16) return ef_fail(EF_ERR_INVALID, "tune_gram: units per SM in 0..16");
  std::lock_guard<std::mutex> lock(ef::g_gram_mu);
  for (int i = 0; i < ef::g_gram_n; ++i) {
    if (ef::g_gram[i].ma == ma && ef::g_gram[i].mb == mb) {
      ef::g_gram[i].kernel = kernel;
      ef::g_gram[i].units = units_per_sm;
      return EF_OK;
    }
  }
  if (ef::g_gram_n >= ef::kMaxGramTunes) return ef_fail(EF_ERR_TOO_LARGE, "tune_gram: override table full");
  ef::g_gram[ef::g_gram_n++] = {ma, mb, kernel, units_per_sm};
  return EF_OK;
}

int ef_tune_reset(void) {
  std::lock_guard<std::mutex> lock(ef::g_gram_mu);
  ef::g_gram_n = 0;
  return EF_OK;
}

}  // extern "C"
