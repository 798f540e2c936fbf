// memory.cu -- device and pinned-host memory of the solves.
//
// Solves that run side by side (threads of the batch and serving runtimes,
// or callers' own threads) must not serialise each other.  cudaMalloc /
// cudaFree and cudaFreeHost synchronise the whole device, so the solve path
// takes its device memory from a stream-ordered pool owned by the library
// (one per device; freed blocks stay cached for the next solve) and its
// mapped termination flags from a pinned slab allocated once.
#include <mutex>
#include <vector>

#include "common.cuh"

namespace pdlp {

namespace {

constexpr int kMaxDevices = 64;
cudaMemPool_t g_pool[kMaxDevices] = {};
std::mutex g_pool_mu;

cudaMemPool_t device_pool() {
  int dev = 0;
  PDLP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    throw CudaError(cudaErrorInvalidDevice, "device index out of range");
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p;
    PDLP_CUDA(cudaMemPoolCreate(&p, &props));
    // keep freed blocks for reuse instead of unmapping them at each sync
    unsigned long long keep = ~0ull;
    PDLP_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pool[dev] = p;
  }
  return g_pool[dev];
}

// Pinned, device-mapped termination flags: one slab, handed out by slot.
constexpr int kFlagSlots = 4096;
HostFlag *g_flags = nullptr;
std::vector<int> g_free_flags;
std::mutex g_flag_mu;

}  // namespace

void *dev_alloc(size_t bytes, cudaStream_t st) {
  void *p = nullptr;
  if (bytes == 0) bytes = 256;
  PDLP_CUDA(cudaMallocFromPoolAsync(&p, bytes, device_pool(), st));
  return p;
}

void dev_free(void *p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

HostFlag *hostflag_acquire() {
  std::lock_guard<std::mutex> lk(g_flag_mu);
  if (!g_flags) {
    void *p = nullptr;
    PDLP_CUDA(cudaHostAlloc(&p, sizeof(HostFlag) * kFlagSlots, cudaHostAllocMapped));
    g_flags = (HostFlag *)p;
    g_free_flags.reserve(kFlagSlots);
    for (int i = kFlagSlots - 1; i >= 0; --i) g_free_flags.push_back(i);
  }
  if (g_free_flags.empty()) {
    // more concurrent solves than slots: a flag of its own
    void *p = nullptr;
    PDLP_CUDA(cudaHostAlloc(&p, sizeof(HostFlag), cudaHostAllocMapped));
    return (HostFlag *)p;
  }
  int i = g_free_flags.back();
  g_free_flags.pop_back();
  return g_flags + i;
}

void hostflag_release(HostFlag *f) {
  if (!f) return;
  std::lock_guard<std::mutex> lk(g_flag_mu);
  if (g_flags && f >= g_flags && f < g_flags + kFlagSlots) {
    g_free_flags.push_back((int)(f - g_flags));
  } else {
    cudaFreeHost(f);
  }
}

void release_pooled_memory() {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  for (auto &p : g_pool)
    if (p) cudaMemPoolTrimTo(p, 0);
}

}  // namespace pdlp
