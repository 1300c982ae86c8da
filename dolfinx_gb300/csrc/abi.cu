// Error state, device queries and small shared services of libdfxgpu.
#include "common.cuh"
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <vector>

namespace
{
thread_local char g_last_error[512] = "";
std::mutex g_mutex;
std::vector<int> g_sms;
std::vector<int*> g_status;
} // namespace

namespace dfx
{
int fail(int code, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line)
{
  // A failed allocation is not sticky: consume it, so that the next launch
  // check of this thread does not report it again as its own failure.
  if (e == cudaErrorMemoryAllocation)
  {
    (void)cudaGetLastError();
    return fail(DFX_ERR_NO_MEMORY, "CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e),
                cudaGetErrorString(e), what, file, line);
  }
  return fail(DFX_ERR_CUDA, "CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e),
              cudaGetErrorString(e), what, file, line);
}

int no_memory(const char* what)
{
  (void)cudaGetLastError(); // the failed allocation, not sticky: consume it
  return fail(DFX_ERR_NO_MEMORY, "%s: out of device memory", what);
}

void clear_error() { g_last_error[0] = 0; }

int num_sms()
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return 152;
  std::lock_guard<std::mutex> lk(g_mutex);
  if ((int)g_sms.size() <= dev)
    g_sms.resize(dev + 1, 0);
  if (g_sms[dev] == 0)
  {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    g_sms[dev] = n;
  }
  return g_sms[dev];
}

int* device_status_page()
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return nullptr;
  std::lock_guard<std::mutex> lk(g_mutex);
  if ((int)g_status.size() <= dev)
    g_status.resize(dev + 1, nullptr);
  if (!g_status[dev])
  {
    int* p = nullptr;
    if (cudaMalloc(&p, 256) != cudaSuccess)
      return nullptr;
    cudaMemset(p, 0, 256);
    g_status[dev] = p;
  }
  return g_status[dev];
}
} // namespace dfx

extern "C" const char* dfx_last_error(void) { return g_last_error; }
extern "C" int dfx_abi_version(void) { return 1; }
