// api.cu -- library plumbing: thread-local error text, version, device info.
#include <stdarg.h>
#include <atomic>
#include "common.cuh"

namespace fmc {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  if (dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

static const uint64_t* g_epoch = nullptr;
const uint64_t* rng_epoch() { return g_epoch; }

__global__ void k_epoch_advance(uint64_t* w) { *w += 1; }

static std::atomic<uint64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

}  // namespace fmc

extern "C" int fmc_launch_count(uint64_t* out) {
  FMC_CHECK_ARG(out != nullptr, "out is NULL");
  *out = fmc::g_launches.load(std::memory_order_relaxed);
  return FMC_OK;
}

extern "C" const char* fmc_last_error(void) { return fmc::g_err; }

extern "C" int fmc_version(void) { return FMC_ABI_VERSION; }

extern "C" int fmc_device_sm_count(int32_t* out) {
  FMC_CHECK_ARG(out != nullptr, "out is NULL");
  int dev = 0;
  FMC_CUDA_TRY(cudaGetDevice(&dev));
  int n = 0;
  FMC_CUDA_TRY(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  *out = n;
  return FMC_OK;
}

extern "C" int fmc_rng_epoch_attach(uint64_t* word) {
  fmc::g_epoch = word;
  return FMC_OK;
}

extern "C" int fmc_rng_epoch_advance(uint64_t* word, void* stream) {
  FMC_CHECK_ARG(word != nullptr, "word is NULL");
  fmc::k_epoch_advance<<<1, 1, 0, (cudaStream_t)stream>>>(word);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}
