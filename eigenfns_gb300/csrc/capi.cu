// Library metadata and status reporting of the C ABI.
#include <cstdio>
#include <string>

#include "../../include/eigenfns_gb300.h"
#include "status.h"

#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace {
thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};
}

void ef_count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

namespace ef {
int sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int n = cached[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
    cached[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}
}  // namespace ef

namespace {
struct SmemEntry {
  const void* kernel;
  int device;
  size_t bytes;
};
std::mutex g_smem_mu;
std::vector<SmemEntry> g_smem;
}  // namespace

void ef::set_smem_limit(const void* kernel, size_t smem) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_smem_mu);
  for (SmemEntry& e : g_smem) {
    if (e.kernel == kernel && e.device == dev) {
      if (e.bytes >= smem) return;
      if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess)
        e.bytes = smem;
      return;
    }
  }
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess)
    g_smem.push_back({kernel, dev, smem});
}

int ef_fail(int code, const char* msg) {
  g_last_error = msg ? msg : "";
  return code;
}

int ef_check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ef_fail(EF_ERR_CUDA, cudaGetErrorString(e));
  return EF_OK;
}

extern "C" {

const char* ef_version(void) { return "eigenfns_gb300 0.1.0 (sm_103a)"; }

const char* ef_status_string(int status) {
  switch (status) {
    case EF_OK: return "ok";
    case EF_ERR_INVALID: return "invalid argument";
    case EF_ERR_UNSUPPORTED: return "unsupported grid size";
    case EF_ERR_CUDA: return "CUDA error";
    case EF_ERR_WORKSPACE: return "workspace too small";
    case EF_ERR_NONFINITE: return "non-finite or non-positive input";
    case EF_ERR_TOO_LARGE: return "size beyond the fixed maximum";
    default: return "unknown status";
  }
}

const char* ef_last_error(void) { return g_last_error.c_str(); }

unsigned long long ef_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
