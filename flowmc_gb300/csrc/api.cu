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

// ---- kernel timing: a fixed pool of event pairs, created when timing is
// enabled (on the device current then), slots taken in launch order
namespace {
constexpr int kTimerSlots = 16384;
struct TimerSlot {
  cudaEvent_t e0, e1;
  int kid;
  double flops, bytes;
};
std::atomic<int> g_timing_on{0};
std::atomic<int> g_timer_next{0};
TimerSlot* g_slots = nullptr;
struct KernelTotals {
  int64_t launches;
  double ms, flops, bytes;
};
KernelTotals g_totals[FMC_KT_COUNT];
std::atomic<int> g_grid[FMC_KT_COUNT][2];
}  // namespace

void note_grid(int kid, int ctas, int cluster) {
  if (kid < 0 || kid >= FMC_KT_COUNT) return;
  g_grid[kid][0].store(ctas, std::memory_order_relaxed);
  g_grid[kid][1].store(cluster, std::memory_order_relaxed);
}

// On a capturing stream the events become event-record nodes of the graph
// (cudaEventRecordExternal): a replay of the graph then records them with the
// kernels running back to back, which is how launches should be timed (an
// eager launch sequence can leave the GPU waiting for the host between an
// event and its kernel).
static cudaError_t record_event(cudaEvent_t e, cudaStream_t stream, bool capturing) {
  return capturing ? cudaEventRecordWithFlags(e, stream, cudaEventRecordExternal) : cudaEventRecord(e, stream);
}

KernelTimer::KernelTimer(int kid, cudaStream_t stream, double flops, double bytes) {
  if (!g_timing_on.load(std::memory_order_relaxed) || kid < 0 || kid >= FMC_KT_COUNT) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return;
  }
  const int i = g_timer_next.fetch_add(1, std::memory_order_relaxed);
  if (i >= kTimerSlots) return;
  TimerSlot& t = g_slots[i];
  t.kid = kid;
  t.flops = flops;
  t.bytes = bytes;
  capturing = cs == cudaStreamCaptureStatusActive;
  if (record_event(t.e0, stream, capturing) != cudaSuccess) {
    (void)cudaGetLastError();
    t.kid = -1;
    return;
  }
  slot = i;
  st = stream;
}

KernelTimer::~KernelTimer() {
  if (slot < 0) return;
  if (record_event(g_slots[slot].e1, st, capturing) != cudaSuccess) {
    (void)cudaGetLastError();
    g_slots[slot].kid = -1;
  }
}

}  // namespace fmc

extern "C" int fmc_kernel_timing_enable(int32_t on) {
  using namespace fmc;
  if (on && g_slots == nullptr) {
    TimerSlot* s = new TimerSlot[kTimerSlots];
    for (int i = 0; i < kTimerSlots; ++i) {
      FMC_CUDA_TRY(cudaEventCreate(&s[i].e0));
      FMC_CUDA_TRY(cudaEventCreate(&s[i].e1));
      s[i].kid = -1;
    }
    g_slots = s;
  }
  g_timing_on.store(on ? 1 : 0);
  return FMC_OK;
}

// fold the recorded launches into the per-kernel totals (synchronises on
// their stop events) and free the slots
static int fold_timers() {
  using namespace fmc;
  int n = g_timer_next.load();
  if (n > kTimerSlots) n = kTimerSlots;
  for (int i = 0; i < n; ++i) {
    TimerSlot& t = g_slots[i];
    if (t.kid < 0) continue;
    FMC_CUDA_TRY(cudaEventSynchronize(t.e1));
    float ms = 0.f;
    FMC_CUDA_TRY(cudaEventElapsedTime(&ms, t.e0, t.e1));
    KernelTotals& k = g_totals[t.kid];
    k.launches += 1;
    k.ms += ms;
    k.flops += t.flops;
    k.bytes += t.bytes;
    t.kid = -1;
  }
  g_timer_next.store(0);
  return FMC_OK;
}

extern "C" int fmc_kernel_timing_read(int32_t kid, int64_t* launches, double* ms, double* flops, double* bytes) {
  using namespace fmc;
  FMC_CHECK_ARG(kid >= 0 && kid < FMC_KT_COUNT, "kernel id %d out of range", kid);
  FMC_CHECK_ARG(launches && ms && flops && bytes, "NULL pointer");
  if (g_slots != nullptr) {
    int rc = fold_timers();
    if (rc) return rc;
  }
  *launches = g_totals[kid].launches;
  *ms = g_totals[kid].ms;
  *flops = g_totals[kid].flops;
  *bytes = g_totals[kid].bytes;
  return FMC_OK;
}

extern "C" int fmc_kernel_grid(int32_t kid, int32_t* ctas, int32_t* cluster) {
  using namespace fmc;
  FMC_CHECK_ARG(kid >= 0 && kid < FMC_KT_COUNT, "kernel id %d out of range", kid);
  FMC_CHECK_ARG(ctas && cluster, "NULL pointer");
  *ctas = g_grid[kid][0].load(std::memory_order_relaxed);
  *cluster = g_grid[kid][1].load(std::memory_order_relaxed);
  return FMC_OK;
}

extern "C" int fmc_kernel_timing_reset(void) {
  using namespace fmc;
  if (g_slots != nullptr) {
    int rc = fold_timers();
    if (rc) return rc;
  }
  for (auto& k : g_totals) k = KernelTotals{0, 0.0, 0.0, 0.0};
  return FMC_OK;
}

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
