// SELL-32-sigma operator: builders (device, host fallback), value refill
// and SpMV.
#include "la_kernels.cuh"
#include "scan.cuh"
#include "sell.cuh"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <thread>
#include <vector>

namespace
{

template <typename F>
void parallel_for(int64_t n, F&& f)
{
  unsigned hc = std::thread::hardware_concurrency();
  const int nt = (int)std::min<int64_t>(hc ? std::min(hc, 64u) : 1, std::max<int64_t>(1, n / 2048));
  if (nt <= 1)
  {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&f, n, t, nt] { f(n * t / nt, n * (t + 1) / nt); });
  for (auto& t : th)
    t.join();
}

template <typename V>
__global__ void k_fill(const int32_t* __restrict__ map, const double* __restrict__ csr,
                       V* __restrict__ out, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t m = __ldcs(map + i);
    __stcs(out + i, m >= 0 ? (V)__ldg(csr + m) : V(0));
  }
}

// Values of a 3x3-block operator, one output value o of the 9 nslots per
// thread: slot row g = o / 288 (32 slots x 9 values), value e = o % 288 / 32
// of lane o % 32's block, slot 32 g + o % 32. Block CSR values are
// row-major 3x3 blocks, so e indexes them directly. Split operators store
// (hi, lo) of each value as one float2.
template <bool SPLIT>
__global__ void k_fill_b3(const int32_t* __restrict__ map, const double* __restrict__ csr,
                          void* __restrict__ out, int64_t nvals)
{
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nvals;
       o += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t g = o / 288;
    const int q = (int)(o - 288 * g);
    const int32_t m = __ldg(map + 32 * g + (q & 31));
    const double v = m >= 0 ? __ldg(csr + 9 * (int64_t)m + (q >> 5)) : 0.0;
    if constexpr (SPLIT)
    {
      float hi, lo;
      dfx::split_f64(v, hi, lo);
      __stcs(reinterpret_cast<float2*>(out) + o, make_float2(hi, lo));
    }
    else
      __stcs(reinterpret_cast<double*>(out) + o, v);
  }
}

// y = A x, 3x3-block operator (lane = block row), FP64 or split values,
// SL block slots per round.
template <bool SPLIT, int SL>
__global__ void __launch_bounds__(128, dfx::kBsellMinBlocks<SL>)
    k_bsell_spmv3(const dfx_operator_s op, const void* __restrict__ x, double* __restrict__ y)
{
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    double acc[3];
    if constexpr (SPLIT)
      dfx::bsell_row3_split<SL>(op, (const float2*)op.vals, (const float2*)x, s, lane, acc);
    else
      dfx::bsell_row3<SL>(op, (const double*)op.vals, (const double*)x, s, lane, acc);
    const int32_t row = 3 * (32 * s + lane);
    if (row < op.n)
    {
#pragma unroll
      for (int r = 0; r < 3; ++r)
        y[row + r] = acc[r];
    }
  }
}

// Split values (DFX_F32X2): hi = fl32(v) at i, lo = fl32(v - hi) at n + i.
__global__ void k_fill_split(const int32_t* __restrict__ map, const double* __restrict__ csr,
                             float* __restrict__ out, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t m = __ldcs(map + i);
    float hi = 0.f, lo = 0.f;
    if (m >= 0)
      dfx::split_f64(__ldg(csr + m), hi, lo);
    __stcs(out + i, hi);
    __stcs(out + n + i, lo);
  }
}

// (hi, lo) FP32 words of an FP64 vector, side by side: hi at 2i, lo at 2i+1.
__global__ void k_split(const double* __restrict__ x, float* __restrict__ out, int32_t n)
{
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    dfx::split_f64(x[i], out[2 * (int64_t)i], out[2 * (int64_t)i + 1]);
}

template <bool COMP>
__global__ void __launch_bounds__(128, 12)
    k_sell_spmv_split(const dfx_operator_s op, const float* __restrict__ x, double* __restrict__ y)
{
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  const float* vh = (const float*)op.vals;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const double acc = dfx::sell_row_split<COMP>(op, vh, vh + op.nslots,
                                                 reinterpret_cast<const float2*>(x), s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
      y[row] = acc;
  }
}

template <typename V, typename X, typename ACC, bool COMP, int CH = 4>
__global__ void __launch_bounds__(128)
    k_sell_spmv(const dfx_operator_s op, const V* __restrict__ vals, const X* __restrict__ x,
                X* __restrict__ y)
{
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const ACC acc = dfx::sell_row<V, X, ACC, COMP, CH>(op, vals, x, s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
      y[row] = (X)acc;
  }
}

template <typename T>
__global__ void k_permute(const T* __restrict__ in, T* __restrict__ out,
                          const int32_t* __restrict__ idx, int32_t n, int scatter)
{
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  if (scatter)
    out[idx[i]] = in[i];
  else
    out[i] = in[idx[i]];
}

// A stream-ordered memory pool per device for the values of operator
// shares (one set per request in a server): shares are made and dropped at
// the request rate, and a cudaFree waits for the whole device. The pool
// keeps freed memory for reuse (release threshold: no limit) until
// dfx_operator_pool_trim.
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[64] = {};

int share_pool(int dev, cudaMemPool_t* out)
{
  DFX_REQUIRE(dev >= 0 && dev < 64, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_pool_mutex);
  if (!g_pools[dev])
  {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    DFX_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = UINT64_MAX;
    DFX_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pools[dev] = pool;
  }
  *out = g_pools[dev];
  return DFX_OK;
}

void free_op(dfx_operator_s* op)
{
  if (!op)
    return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(op->device);
  if (op->pooled)
  {
    // No stream is known here: wait for the device, then return the values
    // to the pool (the synchronous cudaFree semantics).
    cudaDeviceSynchronize();
    for (void* p : {op->vals, op->tmp})
      if (p)
        cudaFreeAsync(p, 0);
    cudaStreamSynchronize(0);
    op->vals = op->tmp = nullptr;
  }
  if (op->owns_structure)
  {
    for (void* p : {(void*)op->perm, (void*)op->iperm, (void*)op->slice_ptr, (void*)op->cols,
                    (void*)op->delta, (void*)op->first, (void*)op->map})
      if (p)
        cudaFree(p);
  }
  else if (op->source)
  {
    op->source->shares -= 1;
  }
  for (void* p : {op->vals, op->tmp})
    if (p)
      cudaFree(p);
  cudaSetDevice(cur);
  delete op;
}

template <typename T>
int upload(T** dst, const std::vector<T>& src, cudaStream_t s)
{
  DFX_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(src.size(), 1)));
  if (!src.empty())
    DFX_CUDA(cudaMemcpyAsync(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, s));
  return DFX_OK;
}

// ---------------------------------------------------------------- device build
// The device builder computes the same arrays as the host builder below:
// the same stable length order per window, slice lengths, renumbered and
// sorted columns, padding and 16-bit deltas. Rows longer than kDevMaxRow
// entries, or windows wider than kDevMaxSigma rows, go to the host builder.
constexpr int kDevMaxRow = 256;
constexpr int kDevMaxSigma = 4096;
constexpr int kGapStatus = 100; // internal: a column gap above 65535
constexpr int kUseHost = -1;    // internal: the device build does not take this matrix

// Stable length-descending order inside each window of sigma rows (the
// host builder's std::stable_sort): the rank of row i is the number of rows
// of its window that are longer, or as long and earlier.
__global__ void k_window_perm(const int64_t* __restrict__ rp, int32_t n, int32_t sigma,
                              int32_t* __restrict__ perm, int* __restrict__ status)
{
  extern __shared__ int32_t slen[];
  const int64_t w0 = (int64_t)blockIdx.x * sigma;
  const int cnt = (int)min((int64_t)sigma, (int64_t)n - w0);
  for (int i = threadIdx.x; i < cnt; i += blockDim.x)
  {
    const int64_t len = rp[w0 + i + 1] - rp[w0 + i];
    if (len > kDevMaxRow)
      atomicExch(status, (int)DFX_ERR_UNSUPPORTED);
    slen[i] = (int32_t)min(len, (int64_t)INT32_MAX);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += blockDim.x)
  {
    const int32_t li = slen[i];
    int rank = 0;
    for (int j = 0; j < cnt; ++j)
    {
      const int32_t lj = slen[j];
      rank += (lj > li) || (lj == li && j < i);
    }
    perm[w0 + rank] = (int32_t)(w0 + i);
  }
}

__global__ void k_invert(const int32_t* __restrict__ perm, int32_t* __restrict__ iperm, int32_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    iperm[perm[i]] = (int32_t)i;
}

// 32 x (longest row of the slice), rounded up to even for k-pairs.
__global__ void k_slice_len(const int64_t* __restrict__ rp, const int32_t* __restrict__ perm,
                            int32_t n, int32_t ns, int pairs, int64_t* __restrict__ out)
{
  const int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sl >= ns)
    return;
  int64_t len = 0;
  for (int l = 0; l < 32; ++l)
  {
    const int64_t i = 32 * sl + l;
    if (i < n)
    {
      const int32_t r = perm[i];
      len = max(len, rp[r + 1] - rp[r]);
    }
  }
  if (pairs)
    len += len & 1;
  out[sl] = 32 * len;
}

// One thread per (renumbered) row of the padded slices: the row's columns
// renumbered by iperm and sorted (insertion sort, rows of at most
// kDevMaxRow entries), then its slots: CSR entry or -1, column or delta.
template <bool COMP, bool PAIRS>
__global__ void __launch_bounds__(128)
    k_sell_fill(const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
                const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm,
                const int64_t* __restrict__ sp, int32_t n, int32_t ns, int32_t* __restrict__ map,
                int32_t* __restrict__ scols, uint16_t* __restrict__ sdelta,
                int32_t* __restrict__ sfirst, int* __restrict__ status)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 32 * (int64_t)ns)
    return;
  const int64_t sl = i >> 5;
  const int l = (int)(i & 31);
  const int64_t base = sp[sl];
  const int64_t len = (sp[sl + 1] - base) >> 5;
  int32_t key[kDevMaxRow], val[kDevMaxRow];
  int cnt = 0;
  if (i < n)
  {
    const int32_t r = perm[i];
    const int64_t b = rp[r];
    const int64_t e = rp[r + 1];
    if (e - b > kDevMaxRow)
      return; // reported by k_window_perm
    cnt = (int)(e - b);
    for (int k = 0; k < cnt; ++k)
    {
      const int32_t c = iperm[cols[b + k]];
      int p = k;
      while (p > 0 && key[p - 1] > c)
      {
        key[p] = key[p - 1];
        val[p] = val[p - 1];
        --p;
      }
      key[p] = c;
      val[p] = (int32_t)(b + k);
    }
  }
  int32_t prev = cnt == 0 ? (int32_t)min(i, (int64_t)n - 1) : key[0];
  if (COMP)
    sfirst[32 * sl + l] = prev;
  for (int64_t k = 0; k < len; ++k)
  {
    const int64_t slot = PAIRS ? base + 64 * (k >> 1) + 2 * l + (k & 1) : base + 32 * k + l;
    const bool real = k < cnt;
    const int32_t c = real ? key[k] : prev;
    map[slot] = real ? val[k] : -1;
    if (COMP)
    {
      const int64_t d = k ? (int64_t)c - prev : 0;
      if (d < 0 || d > 65535)
        atomicExch(status, kGapStatus);
      sdelta[slot] = (uint16_t)max((int64_t)0, min(d, (int64_t)65535));
    }
    else
      scols[slot] = c;
    prev = c;
  }
}

int read_status(int* status, cudaStream_t s)
{
  int h = 0;
  DFX_CUDA(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return h;
}

// Structure of op built on the device; kUseHost: use the host builder.
int build_structure_device(const dfx_csr* A, dfx_operator_s* op, bool pairs, bool compress,
                           cudaStream_t s)
{
  const int32_t n = op->n, ns = op->nslices, sigma = op->sigma;
  if (sigma > kDevMaxSigma)
    return kUseHost;
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  DFX_CUDA(cudaMalloc(&op->perm, sizeof(int32_t) * std::max(n, 1)));
  DFX_CUDA(cudaMalloc(&op->iperm, sizeof(int32_t) * std::max(n, 1)));
  DFX_CUDA(cudaMalloc(&op->slice_ptr, sizeof(int64_t) * ((size_t)ns + 1)));
  int64_t* lens = nullptr;
  int64_t* scratch = nullptr;
  DFX_CUDA(cudaMalloc(&lens, sizeof(int64_t) * std::max(ns, 1)));
  const cudaError_t e = cudaMalloc(&scratch, sizeof(int64_t) * dfx::scan_scratch_count(ns));
  if (e != cudaSuccess)
  {
    cudaFree(lens);
    return dfx::cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
  }
  int st = DFX_OK;
  int64_t nslots = 0;
  if (n > 0)
  {
    const int nwin = (n + sigma - 1) / sigma;
    k_window_perm<<<nwin, 256, sizeof(int32_t) * sigma, s>>>(A->row_ptr, n, sigma, op->perm,
                                                             status);
    k_invert<<<(n + 255) / 256, 256, 0, s>>>(op->perm, op->iperm, n);
    k_slice_len<<<(ns + 127) / 128, 128, 0, s>>>(A->row_ptr, op->perm, n, ns, pairs ? 1 : 0,
                                                  lens);
    st = dfx::exclusive_scan(lens, op->slice_ptr, ns, scratch, s);
    if (!st && cudaGetLastError() != cudaSuccess)
      st = dfx::fail(DFX_ERR_CUDA, "operator structure kernels failed to launch");
    if (!st && cudaMemcpyAsync(&nslots, op->slice_ptr + ns, sizeof(int64_t),
                               cudaMemcpyDeviceToHost, s) != cudaSuccess)
      st = dfx::fail(DFX_ERR_CUDA, "slice pointer read-back failed");
    if (!st)
      st = read_status(status, s);
  }
  else if (cudaMemsetAsync(op->slice_ptr, 0, sizeof(int64_t), s) != cudaSuccess)
    st = dfx::fail(DFX_ERR_CUDA, "slice pointer reset failed");
  cudaStreamSynchronize(s);
  cudaFree(lens);
  cudaFree(scratch);
  if (st == DFX_ERR_UNSUPPORTED)
    return kUseHost; // a row is too long for the device build
  if (st)
    return st;
  DFX_REQUIRE(nslots < INT32_MAX, "operator too large");
  op->nslots = nslots;
  const size_t ms = (size_t)std::max<int64_t>(nslots, 1);
  DFX_CUDA(cudaMalloc(&op->map, sizeof(int32_t) * ms));
  if (compress)
  {
    DFX_CUDA(cudaMalloc(&op->delta, sizeof(uint16_t) * ms));
    DFX_CUDA(cudaMalloc(&op->first, sizeof(int32_t) * std::max<size_t>(32 * (size_t)ns, 1)));
  }
  else
    DFX_CUDA(cudaMalloc(&op->cols, sizeof(int32_t) * ms));
  if (ns > 0)
  {
    const unsigned grid = (unsigned)((32 * (int64_t)ns + 127) / 128);
    if (compress)
      k_sell_fill<true, true><<<grid, 128, 0, s>>>(A->row_ptr, A->cols, op->perm, op->iperm,
                                                   op->slice_ptr, n, ns, op->map, nullptr,
                                                   op->delta, op->first, status);
    else if (pairs)
      k_sell_fill<false, true><<<grid, 128, 0, s>>>(A->row_ptr, A->cols, op->perm, op->iperm,
                                                    op->slice_ptr, n, ns, op->map, op->cols,
                                                    nullptr, nullptr, status);
    else
      k_sell_fill<false, false><<<grid, 128, 0, s>>>(A->row_ptr, A->cols, op->perm, op->iperm,
                                                     op->slice_ptr, n, ns, op->map, op->cols,
                                                     nullptr, nullptr, status);
    DFX_CHECK_LAUNCH();
    const int h = read_status(status, s);
    if (h == kGapStatus)
      return dfx::fail(DFX_ERR_UNSUPPORTED,
                       "a row has a column gap above 65535: use 32-bit columns");
    if (h)
      return dfx::fail(h, "operator structure build failed");
  }
  return DFX_OK;
}
} // namespace

namespace
{
// Values and scratch of a built structure; on success *out = op and the
// values are filled from A's FP64 values when it has them.
int finish_create(dfx_operator_s* op, const dfx_csr* A, dfx_operator* out, void* stream)
{
  int st = DFX_OK;
  if (cudaMalloc(&op->vals, dfx::value_bytes(*op)) != cudaSuccess)
    st = dfx::no_memory("operator values");
  if (!st && cudaMalloc(&op->tmp, dfx::scratch_bytes(*op)) != cudaSuccess)
    st = dfx::no_memory("operator scratch");
  if (st)
  {
    free_op(op);
    return st;
  }
  *out = op;
  if (A->vals && A->dtype == DFX_F64)
    return dfx_operator_update_values(op, A, stream);
  return DFX_OK;
}

// The 3x3-block operator of a bs 3 block CSR (host build): block rows sorted
// by length, stable, within windows of sigma block rows; slices of 32 block
// rows; one 32-bit column per block. The scalar permutation is the block
// one expanded (row 3 i + c -> 3 perm[i] + c).
int create_b3(const dfx_csr* A, int32_t sigma, int32_t dtype, dfx_operator* out, void* stream)
{
  cudaStream_t s = dfx::as_stream(stream);
  const int32_t nb = A->nrows;
  DFX_REQUIRE((int64_t)3 * nb < INT32_MAX, "matrix too large for a 3x3-block operator");
  std::vector<int64_t> rp(nb + 1);
  std::vector<int32_t> cols(A->nnz);
  DFX_CUDA(cudaMemcpyAsync(rp.data(), A->row_ptr, sizeof(int64_t) * (nb + 1),
                           cudaMemcpyDeviceToHost, s));
  if (A->nnz)
    DFX_CUDA(cudaMemcpyAsync(cols.data(), A->cols, sizeof(int32_t) * A->nnz,
                             cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  std::vector<int32_t> bperm(nb), biperm(nb);
  std::iota(bperm.begin(), bperm.end(), 0);
  parallel_for((nb + sigma - 1) / sigma,
               [&](int64_t w0, int64_t w1)
               {
                 for (int64_t w = w0; w < w1; ++w)
                 {
                   auto b = bperm.begin() + w * sigma;
                   auto e = bperm.begin() + std::min<int64_t>((w + 1) * (int64_t)sigma, nb);
                   std::stable_sort(b, e, [&](int32_t a, int32_t c)
                                    { return rp[a + 1] - rp[a] > rp[c + 1] - rp[c]; });
                 }
               });
  for (int32_t i = 0; i < nb; ++i)
    biperm[bperm[i]] = i;
  const int32_t ns = (nb + 31) / 32;
  std::vector<int64_t> sp(ns + 1, 0);
  for (int32_t sl = 0; sl < ns; ++sl)
  {
    int64_t len = 0;
    for (int l = 0; l < 32; ++l)
    {
      const int64_t i = 32 * (int64_t)sl + l;
      if (i < nb)
        len = std::max(len, rp[bperm[i] + 1] - rp[bperm[i]]);
    }
    sp[sl + 1] = sp[sl] + 32 * len;
  }
  const int64_t nslots = sp[ns];
  DFX_REQUIRE(nslots < INT32_MAX, "operator too large");
  std::vector<int32_t> scols(nslots), smap(nslots);
  parallel_for(ns,
               [&](int64_t s0, int64_t s1)
               {
                 std::vector<std::pair<int32_t, int32_t>> row;
                 for (int64_t sl = s0; sl < s1; ++sl)
                 {
                   const int64_t len = (sp[sl + 1] - sp[sl]) / 32;
                   for (int l = 0; l < 32; ++l)
                   {
                     const int64_t i = 32 * sl + l;
                     row.clear();
                     if (i < nb)
                     {
                       const int32_t r = bperm[i];
                       for (int64_t j = rp[r]; j < rp[r + 1]; ++j)
                         row.push_back({biperm[cols[j]], (int32_t)j});
                       std::sort(row.begin(), row.end());
                     }
                     int32_t prev =
                         row.empty() ? (int32_t)std::min<int64_t>(i, nb - 1) : row[0].first;
                     for (int64_t k = 0; k < len; ++k)
                     {
                       const int64_t slot = sp[sl] + 32 * k + l;
                       const bool real = k < (int64_t)row.size();
                       const int32_t c = real ? row[k].first : prev;
                       smap[slot] = real ? row[k].second : -1;
                       scols[slot] = c;
                       prev = c;
                     }
                   }
                 }
               });
  std::vector<int32_t> perm(3 * (size_t)nb), iperm(3 * (size_t)nb);
  for (int32_t i = 0; i < nb; ++i)
    for (int c = 0; c < 3; ++c)
    {
      perm[3 * (size_t)i + c] = 3 * bperm[i] + c;
      iperm[3 * (size_t)i + c] = 3 * biperm[i] + c;
    }

  auto* op = new dfx_operator_s();
  op->serial = dfx::next_operator_serial();
  cudaGetDevice(&op->device);
  op->n = 3 * nb;
  op->bs = 3;
  // Four block slots per round (chunk 8): on the vector P2 elasticity
  // operator of a 96x24x24x6 tetrahedral mesh (13.0M blocks) the split SpMV
  // took 0.174 ms against 0.182 (two slots) and 0.202 (one).
  op->chunk = 8;
  op->nslices = ns;
  op->sigma = sigma;
  op->dtype = dtype;
  op->compressed = 0;
  op->nslots = nslots;
  op->csr_nnz = A->nnz;
  int st = DFX_OK;
  if (!st)
    st = upload(&op->perm, perm, s);
  if (!st)
    st = upload(&op->iperm, iperm, s);
  if (!st)
    st = upload(&op->slice_ptr, sp, s);
  if (!st)
    st = upload(&op->map, smap, s);
  if (!st)
    st = upload(&op->cols, scols, s);
  if (!st)
  {
    cudaError_t e = cudaStreamSynchronize(s); // host vectors die at return
    if (e != cudaSuccess)
      st = dfx::cuda_fail(e, "upload", __FILE__, __LINE__);
  }
  if (st)
  {
    free_op(op);
    return st;
  }
  return finish_create(op, A, out, stream);
}
} // namespace

namespace dfx
{
// One slice per warp in blocks of four warps: the block scheduler balances
// slices of different lengths (a static multi-slice split per warp left
// warps idle at the end of each block).
int sell_grid(int32_t nslices) { return std::max(1, (nslices + 3) / 4); }

int max_grid_blocks() { return 64 * num_sms(); }

uint64_t next_operator_serial()
{
  static std::atomic<uint64_t> counter{0};
  return ++counter;
}

size_t value_bytes(const dfx_operator_s& op)
{
  const size_t per = op.dtype == DFX_F32 ? 4 : 8; // F64, or two FP32 words
  return per * (size_t)op.bs * op.bs * (size_t)std::max<int64_t>(op.nslots, 1);
}

// dfx_operator_apply's permuted x and y (and, split operators, x's words).
size_t scratch_bytes(const dfx_operator_s& op)
{
  const size_t n = (size_t)std::max<int32_t>(op.n, 1);
  if (op.dtype == DFX_F32)
    return 4 * 2 * n;
  return 8 * (op.dtype == DFX_F32X2 ? 3 : 2) * n;
}

int sell_spmv(const dfx_operator_s& op, const void* x, void* y, cudaStream_t s)
{
  const unsigned grid = (unsigned)sell_grid(op.nslices);
  if (op.nslices == 0)
    return DFX_OK;
  if (op.bs == 3)
  {
    auto launch = [&](auto split, auto sl)
    {
      k_bsell_spmv3<decltype(split)::value, decltype(sl)::value>
          <<<grid, 128, 0, s>>>(op, x, (double*)y);
    };
    auto by_chunk = [&](auto split)
    {
      if (op.chunk == 2)
        launch(split, std::integral_constant<int, 1>{});
      else if (op.chunk == 8)
        launch(split, std::integral_constant<int, 4>{});
      else
        launch(split, std::integral_constant<int, 2>{});
    };
    if (op.dtype == DFX_F32X2)
      by_chunk(std::true_type{});
    else
      by_chunk(std::false_type{});
  }
  else if (op.dtype == DFX_F64)
    k_sell_spmv<double, double, double, false><<<grid, 128, 0, s>>>(
        op, (const double*)op.vals, (const double*)x, (double*)y);
  else if (op.dtype == DFX_F32X2)
  {
    if (op.compressed)
      k_sell_spmv_split<true><<<grid, 128, 0, s>>>(op, (const float*)x, (double*)y);
    else
      k_sell_spmv_split<false><<<grid, 128, 0, s>>>(op, (const float*)x, (double*)y);
  }
  else
  {
    auto launch = [&](auto comp, auto ch)
    {
      k_sell_spmv<float, float, float, decltype(comp)::value, decltype(ch)::value>
          <<<grid, 128, 0, s>>>(op, (const float*)op.vals, (const float*)x, (float*)y);
    };
    auto by_chunk = [&](auto comp)
    {
      if (op.chunk == 2)
        launch(comp, std::integral_constant<int, 2>{});
      else if (op.chunk == 8)
        launch(comp, std::integral_constant<int, 8>{});
      else
        launch(comp, std::integral_constant<int, 4>{});
    };
    if (op.compressed)
      by_chunk(std::true_type{});
    else
      by_chunk(std::false_type{});
  }
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}
} // namespace dfx

extern "C" int dfx_operator_create(const dfx_csr* A, int32_t sigma, int32_t dtype,
                                   int32_t compress_cols, dfx_operator* out, void* stream)
{
  return dfx_operator_create_ex(A, sigma, dtype, compress_cols, DFX_BUILD_AUTO, out, stream);
}

extern "C" int dfx_operator_create_ex(const dfx_csr* A, int32_t sigma, int32_t dtype,
                                      int32_t compress_cols, int32_t build, dfx_operator* out,
                                      void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(out, "output handle is NULL");
  *out = nullptr;
  DFX_REQUIRE(A->bs == 1 || A->bs == 3,
              "the sliced-ELL operator takes scalar (bs 1) or 3x3-block matrices");
  DFX_REQUIRE(A->nrows == A->ncols, "matrix must be square");
  DFX_REQUIRE(dtype == DFX_F64 || dtype == DFX_F32 || dtype == DFX_F32X2,
              "unknown value type %d", dtype);
  DFX_REQUIRE(!compress_cols || dtype != DFX_F64,
              "16-bit columns are for operators with FP32 words");
  DFX_REQUIRE(sigma >= 32 && sigma % 32 == 0, "sigma must be a positive multiple of 32");
  DFX_REQUIRE(A->nnz < INT32_MAX, "matrix too large for the operator slot map");
  DFX_REQUIRE(build == DFX_BUILD_AUTO || build == DFX_BUILD_DEVICE || build == DFX_BUILD_HOST,
              "unknown build place %d", build);
  if (A->bs == 3)
  {
    DFX_REQUIRE(dtype != DFX_F32, "3x3-block operators hold FP64 or split (DFX_F32X2) values");
    DFX_REQUIRE(!compress_cols, "3x3-block operators keep 32-bit block columns");
    DFX_REQUIRE(build != DFX_BUILD_DEVICE, "3x3-block operators are built on the host");
    return create_b3(A, sigma, dtype, out, stream);
  }
  cudaStream_t s = dfx::as_stream(stream);
  const int32_t n = A->nrows;
  if (build != DFX_BUILD_HOST)
  {
    auto* op = new dfx_operator_s();
    op->serial = dfx::next_operator_serial();
    cudaGetDevice(&op->device);
    op->n = n;
    op->nslices = (n + 31) / 32;
    op->sigma = sigma;
    op->dtype = dtype;
    op->compressed = compress_cols ? 1 : 0;
    op->csr_nnz = A->nnz;
    const int st = build_structure_device(A, op, dtype != DFX_F64, compress_cols != 0, s);
    if (st == DFX_OK)
      return finish_create(op, A, out, stream);
    free_op(op);
    if (st != kUseHost)
      return st;
    if (build == DFX_BUILD_DEVICE)
      return dfx::fail(DFX_ERR_UNSUPPORTED,
                       "the device build takes rows of at most %d entries and sigma <= %d",
                       kDevMaxRow, kDevMaxSigma);
  }
  std::vector<int64_t> rp(n + 1);
  std::vector<int32_t> cols(A->nnz);
  DFX_CUDA(cudaMemcpyAsync(rp.data(), A->row_ptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost,
                           s));
  if (A->nnz)
    DFX_CUDA(cudaMemcpyAsync(cols.data(), A->cols, sizeof(int32_t) * A->nnz,
                             cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));

  // Row permutation: length-descending, stable, within windows of sigma.
  std::vector<int32_t> perm(n), iperm(n);
  std::iota(perm.begin(), perm.end(), 0);
  parallel_for((n + sigma - 1) / sigma,
               [&](int64_t w0, int64_t w1)
               {
                 for (int64_t w = w0; w < w1; ++w)
                 {
                   auto b = perm.begin() + w * sigma;
                   auto e = perm.begin() + std::min<int64_t>((w + 1) * (int64_t)sigma, n);
                   std::stable_sort(b, e, [&](int32_t a, int32_t c)
                                    { return rp[a + 1] - rp[a] > rp[c + 1] - rp[c]; });
                 }
               });
  for (int32_t i = 0; i < n; ++i)
    iperm[perm[i]] = i;
  const int32_t ns = (n + 31) / 32;
  // FP32 operators store entries in k-pairs per lane (8-byte loads), so
  // their slices have an even length.
  const bool pairs = dtype != DFX_F64;
  std::vector<int64_t> sp(ns + 1, 0);
  for (int32_t sl = 0; sl < ns; ++sl)
  {
    int64_t len = 0;
    for (int l = 0; l < 32; ++l)
    {
      const int64_t i = 32 * (int64_t)sl + l;
      if (i < n)
        len = std::max(len, rp[perm[i] + 1] - rp[perm[i]]);
    }
    if (pairs)
      len += len & 1;
    sp[sl + 1] = sp[sl] + 32 * len;
  }
  auto slot_of = [&](int64_t sl, int64_t k, int l) -> int64_t
  { return pairs ? sp[sl] + 64 * (k >> 1) + 2 * l + (k & 1) : sp[sl] + 32 * k + l; };
  const int64_t nslots = sp[ns];
  DFX_REQUIRE(nslots < INT32_MAX, "operator too large");
  std::vector<int32_t> scols(compress_cols ? 0 : nslots), smap(nslots);
  std::vector<uint16_t> sdelta(compress_cols ? nslots : 0);
  std::vector<int32_t> sfirst(compress_cols ? 32 * (int64_t)ns : 0, 0);
  std::vector<int> bad(64, 0);
  parallel_for(ns,
               [&](int64_t s0, int64_t s1)
               {
                 std::vector<std::pair<int32_t, int32_t>> row;
                 for (int64_t sl = s0; sl < s1; ++sl)
                 {
                   const int64_t len = (sp[sl + 1] - sp[sl]) / 32;
                   for (int l = 0; l < 32; ++l)
                   {
                     const int64_t i = 32 * sl + l;
                     row.clear();
                     if (i < n)
                     {
                       const int32_t r = perm[i];
                       for (int64_t j = rp[r]; j < rp[r + 1]; ++j)
                         row.push_back({iperm[cols[j]], (int32_t)j});
                       std::sort(row.begin(), row.end());
                     }
                     int32_t prev = row.empty() ? (int32_t)std::min<int64_t>(i, n - 1) : row[0].first;
                     if (compress_cols)
                       sfirst[32 * sl + l] = prev;
                     for (int64_t k = 0; k < len; ++k)
                     {
                       const int64_t slot = slot_of(sl, k, l);
                       const bool real = k < (int64_t)row.size();
                       const int32_t c = real ? row[k].first : prev;
                       smap[slot] = real ? row[k].second : -1;
                       if (compress_cols)
                       {
                         const int64_t d = k ? (int64_t)c - prev : 0;
                         if (d < 0 || d > 65535)
                           bad[0] = 1;
                         sdelta[slot] = (uint16_t)std::max<int64_t>(0, std::min<int64_t>(d, 65535));
                       }
                       else
                         scols[slot] = c;
                       prev = c;
                     }
                   }
                 }
               });
  if (bad[0])
    return dfx::fail(DFX_ERR_UNSUPPORTED,
                     "a row has a column gap above 65535: use 32-bit columns");

  auto* op = new dfx_operator_s();
  op->serial = dfx::next_operator_serial();
  cudaGetDevice(&op->device);
  op->n = n;
  op->nslices = ns;
  op->sigma = sigma;
  op->dtype = dtype;
  op->compressed = compress_cols ? 1 : 0;
  op->nslots = nslots;
  op->csr_nnz = A->nnz;
  int st = DFX_OK;
  if (!st)
    st = upload(&op->perm, perm, s);
  if (!st)
    st = upload(&op->iperm, iperm, s);
  if (!st)
    st = upload(&op->slice_ptr, sp, s);
  if (!st)
    st = upload(&op->map, smap, s);
  if (!st && compress_cols)
    st = upload(&op->delta, sdelta, s);
  if (!st && compress_cols)
    st = upload(&op->first, sfirst, s);
  if (!st && !compress_cols)
    st = upload(&op->cols, scols, s);
  if (!st)
  {
    cudaError_t e = cudaStreamSynchronize(s); // host vectors die at return
    if (e != cudaSuccess)
      st = dfx::cuda_fail(e, "upload", __FILE__, __LINE__);
  }
  if (st)
  {
    free_op(op);
    return st;
  }
  return finish_create(op, A, out, stream);
}

extern "C" int dfx_operator_update_values(dfx_operator op, const dfx_csr* A, void* stream)
{
  DFX_REQUIRE(op && A && A->vals, "operator and matrix must be non-NULL");
  DFX_REQUIRE(op->vals, "operator values were released (dfx_operator_release_values): use a share");
  DFX_REQUIRE(A->dtype == DFX_F64, "values are refilled from FP64 CSR values");
  DFX_REQUIRE(A->nnz == op->csr_nnz && A->bs == op->bs && A->nrows * A->bs == op->n,
              "matrix does not match the operator");
  if (op->nslots == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  if (op->bs == 3)
  {
    const int64_t nv = 9 * op->nslots;
    const unsigned g3 = (unsigned)std::min<int64_t>((nv + 255) / 256, 16 * dfx::num_sms());
    if (op->dtype == DFX_F32X2)
      k_fill_b3<true><<<g3, 256, 0, s>>>(op->map, (const double*)A->vals, op->vals, nv);
    else
      k_fill_b3<false><<<g3, 256, 0, s>>>(op->map, (const double*)A->vals, op->vals, nv);
    DFX_CHECK_LAUNCH();
    return DFX_OK;
  }
  const unsigned grid = (unsigned)std::min<int64_t>((op->nslots + 255) / 256, 16 * dfx::num_sms());
  if (op->dtype == DFX_F64)
    k_fill<double><<<grid, 256, 0, s>>>(op->map, (const double*)A->vals, (double*)op->vals,
                                        op->nslots);
  else if (op->dtype == DFX_F32X2)
    k_fill_split<<<grid, 256, 0, s>>>(op->map, (const double*)A->vals, (float*)op->vals,
                                      op->nslots);
  else
    k_fill<float><<<grid, 256, 0, s>>>(op->map, (const double*)A->vals, (float*)op->vals,
                                       op->nslots);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_operator_destroy(dfx_operator op)
{
  if (op && op->shares > 0)
    return dfx::fail(DFX_ERR_INVALID, "operator structure is still shared by %d operators",
                     op->shares);
  free_op(op);
  return DFX_OK;
}

extern "C" int dfx_operator_share(dfx_operator src, dfx_operator* out)
{
  DFX_REQUIRE(src && out, "arguments must be non-NULL");
  DFX_REQUIRE(src->owns_structure, "share the source operator, not a share");
  *out = nullptr;
  auto* op = new dfx_operator_s(*src);
  op->serial = dfx::next_operator_serial();
  op->owns_structure = 0;
  op->shares = 0;
  op->source = src;
  op->vals = nullptr;
  op->tmp = nullptr;
  if (cudaMalloc(&op->vals, dfx::value_bytes(*op)) != cudaSuccess
      || cudaMalloc(&op->tmp, dfx::scratch_bytes(*op)) != cudaSuccess)
  {
    if (op->vals)
      cudaFree(op->vals);
    delete op;
    return dfx::no_memory("operator values");
  }
  src->shares += 1;
  *out = op;
  return DFX_OK;
}

extern "C" int dfx_operator_share_async(dfx_operator src, void* stream, dfx_operator* out)
{
  DFX_REQUIRE(src && out, "arguments must be non-NULL");
  DFX_REQUIRE(src->owns_structure, "share the source operator, not a share");
  *out = nullptr;
  cudaMemPool_t pool = nullptr;
  if (int st = share_pool(src->device, &pool))
    return st;
  cudaStream_t s = dfx::as_stream(stream);
  auto* op = new dfx_operator_s(*src);
  op->serial = dfx::next_operator_serial();
  op->owns_structure = 0;
  op->shares = 0;
  op->source = src;
  op->pooled = 1;
  op->vals = nullptr;
  op->tmp = nullptr;
  if (cudaMallocFromPoolAsync(&op->vals, dfx::value_bytes(*op), pool, s) != cudaSuccess
      || cudaMallocFromPoolAsync(&op->tmp, dfx::scratch_bytes(*op), pool, s) != cudaSuccess)
  {
    if (op->vals)
      cudaFreeAsync(op->vals, s);
    delete op;
    return dfx::no_memory("operator values");
  }
  src->shares += 1;
  *out = op;
  return DFX_OK;
}

extern "C" int dfx_operator_destroy_async(dfx_operator op, void* stream)
{
  if (!op)
    return DFX_OK;
  if (op->shares > 0)
    return dfx::fail(DFX_ERR_INVALID, "operator structure is still shared by %d operators",
                     op->shares);
  if (!op->pooled)
  {
    free_op(op);
    return DFX_OK;
  }
  cudaStream_t s = dfx::as_stream(stream);
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(op->device);
  for (void* p : {op->vals, op->tmp})
    if (p)
      cudaFreeAsync(p, s);
  cudaSetDevice(cur);
  if (op->source)
    op->source->shares -= 1;
  delete op;
  return DFX_OK;
}

extern "C" int dfx_operator_pool_trim(void)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess)
  {
    (void)cudaGetLastError();
    return DFX_OK; // no device: no pool
  }
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_pool_mutex);
    if (dev < 0 || dev >= 64 || !g_pools[dev])
      return DFX_OK;
    pool = g_pools[dev];
  }
  DFX_CUDA(cudaDeviceSynchronize());
  DFX_CUDA(cudaMemPoolTrimTo(pool, 0));
  return DFX_OK;
}

extern "C" int dfx_operator_set_chunk(dfx_operator op, int32_t chunk)
{
  DFX_REQUIRE(op, "operator is NULL");
  DFX_REQUIRE(chunk == 2 || chunk == 4 || chunk == 8, "chunk must be 2, 4 or 8 (got %d)", chunk);
  if (op->chunk != chunk)
  {
    op->chunk = chunk;
    op->serial = dfx::next_operator_serial(); // cached solver graphs bake the launch
  }
  return DFX_OK;
}

extern "C" int dfx_operator_info(dfx_operator op, int64_t* nslots, int32_t* nslices,
                                 const int32_t** d_perm)
{
  DFX_REQUIRE(op, "operator is NULL");
  if (nslots)
    *nslots = op->nslots;
  if (nslices)
    *nslices = op->nslices;
  if (d_perm)
    *d_perm = op->perm;
  return DFX_OK;
}

extern "C" int dfx_operator_release_values(dfx_operator op)
{
  DFX_REQUIRE(op, "operator is NULL");
  DFX_REQUIRE(op->owns_structure, "only a structure's own operator releases its values");
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(op->device);
  for (void* p : {op->vals, op->tmp})
    if (p)
      cudaFree(p);
  cudaSetDevice(cur);
  op->vals = nullptr;
  op->tmp = nullptr;
  op->serial = dfx::next_operator_serial();
  return DFX_OK;
}

extern "C" int dfx_operator_device_bytes(dfx_operator op, size_t* bytes)
{
  DFX_REQUIRE(op && bytes, "arguments must be non-NULL");
  // The allocations of the build (structure, owners only) and of
  // finish_create / dfx_operator_share (values and scratch, every operator).
  size_t b = op->vals ? dfx::value_bytes(*op) + dfx::scratch_bytes(*op) : 0;
  if (op->owns_structure)
  {
    const size_t n = (size_t)std::max<int32_t>(op->n, 1);
    const size_t ms = (size_t)std::max<int64_t>(op->nslots, 1);
    b += 2 * sizeof(int32_t) * n + sizeof(int64_t) * ((size_t)op->nslices + 1);
    b += sizeof(int32_t) * ms; // map
    if (op->delta)
      b += sizeof(uint16_t) * ms + sizeof(int32_t) * std::max<size_t>(32 * (size_t)op->nslices, 1);
    if (op->cols)
      b += sizeof(int32_t) * ms;
  }
  *bytes = b;
  return DFX_OK;
}

extern "C" int dfx_operator_apply(dfx_operator op, const void* d_x, void* d_y, void* stream)
{
  DFX_REQUIRE(op, "operator is NULL");
  DFX_REQUIRE(op->vals, "operator values were released (dfx_operator_release_values): use a share");
  const int32_t n = op->n;
  if (n == 0)
    return DFX_OK; // empty vectors may have NULL data
  DFX_REQUIRE(d_x && d_y, "arguments must be non-NULL");
  cudaStream_t s = dfx::as_stream(stream);
  const unsigned g = (unsigned)((n + 255) / 256);
  if (op->dtype == DFX_F64)
  {
    double* xp = (double*)op->tmp;
    double* yp = xp + n;
    k_permute<double><<<g, 256, 0, s>>>((const double*)d_x, xp, op->perm, n, 0);
    if (int st = dfx::sell_spmv(*op, xp, yp, s))
      return st;
    k_permute<double><<<g, 256, 0, s>>>(yp, (double*)d_y, op->perm, n, 1);
  }
  else if (op->dtype == DFX_F32X2)
  {
    double* xp = (double*)op->tmp;
    double* yp = xp + n;
    float* xs = (float*)(yp + n);
    k_permute<double><<<g, 256, 0, s>>>((const double*)d_x, xp, op->perm, n, 0);
    k_split<<<g, 256, 0, s>>>(xp, xs, n);
    if (int st = dfx::sell_spmv(*op, xs, yp, s))
      return st;
    k_permute<double><<<g, 256, 0, s>>>(yp, (double*)d_y, op->perm, n, 1);
  }
  else
  {
    float* xp = (float*)op->tmp;
    float* yp = xp + n;
    k_permute<float><<<g, 256, 0, s>>>((const float*)d_x, xp, op->perm, n, 0);
    if (int st = dfx::sell_spmv(*op, xp, yp, s))
      return st;
    k_permute<float><<<g, 256, 0, s>>>(yp, (float*)d_y, op->perm, n, 1);
  }
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_operator_apply_renumbered(dfx_operator op, const void* d_x, void* d_y,
                                             void* stream)
{
  DFX_REQUIRE(op, "operator is NULL");
  DFX_REQUIRE(op->vals, "operator values were released (dfx_operator_release_values): use a share");
  if (op->n == 0)
    return DFX_OK; // empty vectors may have NULL data
  DFX_REQUIRE(d_x && d_y, "arguments must be non-NULL");
  cudaStream_t s = dfx::as_stream(stream);
  if (op->dtype == DFX_F32X2)
  {
    // FP64 vectors: x's FP32 words go to the operator's scratch first.
    float* xs = (float*)((double*)op->tmp + 2 * (int64_t)op->n);
    k_split<<<(unsigned)((op->n + 255) / 256), 256, 0, s>>>((const double*)d_x, xs, op->n);
    DFX_CHECK_LAUNCH();
    return dfx::sell_spmv(*op, xs, d_y, s);
  }
  return dfx::sell_spmv(*op, d_x, d_y, s);
}
