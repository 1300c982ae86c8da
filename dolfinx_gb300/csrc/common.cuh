// Shared helpers of libdfxgpu: error reporting, launch geometry, warp and
// block reductions. Host + device.
#pragma once

#include "dfx_gpu.h"
#include <cstdint>
#include <cuda_runtime.h>

namespace dfx
{

// Record `msg` as the thread's last error and return `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void clear_error();

// Streaming-multiprocessor count of the current device (cached per device).
int num_sms();

// A small per-device status page owned by the library (allocated once per
// device on first use): device kernels record error codes there.
// DFX_ERR_NO_MEMORY after a failed allocation (the error is consumed).
int no_memory(const char* what);
int* device_status_page();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch parameters picked by the autotuner, per device and workload key
// (a process-wide table; 0 = no entry). what: kTuneAssembly (cells per
// block of the matrix assembly kernel) or kTuneSpmv (lanes per CSR row).
constexpr int kTuneAssembly = 1;
constexpr int kTuneSpmv = 2;
int tuned_get(int what, int64_t k0, int64_t k1, int64_t k2);
void tuned_set(int what, int64_t k0, int64_t k1, int64_t k2, int value); // 0 removes

} // namespace dfx

#define DFX_CUDA(call)                                                         \
  do                                                                           \
  {                                                                            \
    cudaError_t dfx_e_ = (call);                                               \
    if (dfx_e_ != cudaSuccess)                                                 \
      return dfx::cuda_fail(dfx_e_, #call, __FILE__, __LINE__);                \
  } while (0)

#define DFX_CHECK_LAUNCH() DFX_CUDA(cudaGetLastError())

#define DFX_REQUIRE(cond, ...)                                                 \
  do                                                                           \
  {                                                                            \
    if (!(cond))                                                               \
      return dfx::fail(DFX_ERR_INVALID, __VA_ARGS__);                          \
  } while (0)

#ifdef __CUDACC__
namespace dfx
{
// Sum over the lanes of a warp; every lane gets the total.
template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum (fixed tree order). `sh` holds >= 32 values.
// All threads of the block must call it; thread 0 receives the result.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh)
{
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0)
    sh[w] = v;
  __syncthreads();
  T t = T(0);
  if (w == 0)
  {
    t = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : T(0);
    t = warp_sum(t);
  }
  __syncthreads();
  return t;
}

// Read-only, streamed-once loads (bypass L1 allocation).
template <typename T>
__device__ __forceinline__ T ld_stream(const T* p)
{
  return __ldcs(p);
}
} // namespace dfx
#endif
