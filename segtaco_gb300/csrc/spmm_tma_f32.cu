// spmm_tma_f32.cu -- TMA SpMM launcher for fp32 B, and the device status word.
#include <mutex>

#include "spmm_tma_launch.cuh"

namespace segtaco {
namespace {
static __device__ int g_status;  // SEGTACO_ETIMEOUT after a timed-out wait
constexpr int kMaxDevices = 64;
std::mutex g_status_mu;
int *g_status_ptr[kMaxDevices] = {};
}  // namespace

int tma_status_ptr(int **out) {
  int dev = -1;
  SEGTACO_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= kMaxDevices) return set_error(SEGTACO_EUNSUPPORTED, "device %d", dev);
  std::lock_guard<std::mutex> lock(g_status_mu);
  if (!g_status_ptr[dev]) {
    void *p = nullptr;
    SEGTACO_TRY(check_cuda(cudaGetSymbolAddress(&p, g_status), "cudaGetSymbolAddress(status)"));
    g_status_ptr[dev] = static_cast<int *>(p);
  }
  *out = g_status_ptr[dev];
  return SEGTACO_OK;
}

int launch_spmm_tma_f32(const SpmmLaunch &L, bool rows, cudaStream_t s) {
  return launch_tma<float>(L, rows, s);
}

}  // namespace segtaco

extern "C" int segtaco_device_status(int clear) {
  using namespace segtaco;
  int v = 0;
  SEGTACO_TRY(check_cuda(cudaMemcpyFromSymbol(&v, g_status, sizeof(int)), "read status"));
  if (clear) {
    const int z = 0;
    SEGTACO_TRY(check_cuda(cudaMemcpyToSymbol(g_status, &z, sizeof(int)), "clear status"));
  }
  return v;
}
