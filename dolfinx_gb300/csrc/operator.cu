// SELL-32-sigma operator: host-side builder, value refill and SpMV.
#include "la_kernels.cuh"
#include "sell.cuh"

#include <algorithm>
#include <numeric>
#include <thread>
#include <vector>

namespace
{
constexpr int kThreads = 256;

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

template <typename V, typename X, typename ACC, bool COMP>
__global__ void __launch_bounds__(128)
    k_sell_spmv(const dfx_operator_s op, const V* __restrict__ vals, const X* __restrict__ x,
                X* __restrict__ y)
{
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const ACC acc = dfx::sell_row<V, X, ACC, COMP>(op, vals, x, s, lane);
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

void free_op(dfx_operator_s* op)
{
  if (!op)
    return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(op->device);
  if (op->owns_structure)
    for (void* p : {(void*)op->perm, (void*)op->iperm, (void*)op->slice_ptr, (void*)op->cols,
                    (void*)op->delta, (void*)op->first, (void*)op->map})
      if (p)
        cudaFree(p);
  else if (op->source)
    op->source->shares -= 1;
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
} // namespace

namespace dfx
{
// One slice per warp in blocks of four warps: the block scheduler balances
// slices of different lengths (a static multi-slice split per warp left
// warps idle at the end of each block).
int sell_grid(int32_t nslices) { return std::max(1, (nslices + 3) / 4); }

int max_grid_blocks() { return 64 * num_sms(); }

int sell_spmv(const dfx_operator_s& op, const void* x, void* y, cudaStream_t s)
{
  const unsigned grid = (unsigned)sell_grid(op.nslices);
  if (op.nslices == 0)
    return DFX_OK;
  if (op.dtype == DFX_F64)
    k_sell_spmv<double, double, double, false><<<grid, 128, 0, s>>>(
        op, (const double*)op.vals, (const double*)x, (double*)y);
  else if (op.compressed)
    k_sell_spmv<float, float, float, true><<<grid, 128, 0, s>>>(
        op, (const float*)op.vals, (const float*)x, (float*)y);
  else
    k_sell_spmv<float, float, float, false><<<grid, 128, 0, s>>>(
        op, (const float*)op.vals, (const float*)x, (float*)y);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}
} // namespace dfx

extern "C" int dfx_operator_create(const dfx_csr* A, int32_t sigma, int32_t dtype,
                                   int32_t compress_cols, dfx_operator* out, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(out, "output handle is NULL");
  *out = nullptr;
  DFX_REQUIRE(A->bs == 1, "the sliced-ELL operator takes scalar (bs 1) matrices");
  DFX_REQUIRE(A->nrows == A->ncols, "matrix must be square");
  DFX_REQUIRE(dtype == DFX_F64 || dtype == DFX_F32, "unknown value type %d", dtype);
  DFX_REQUIRE(!compress_cols || dtype == DFX_F32, "16-bit columns are for FP32 operators");
  DFX_REQUIRE(sigma >= 32 && sigma % 32 == 0, "sigma must be a positive multiple of 32");
  DFX_REQUIRE(A->nnz < INT32_MAX, "matrix too large for the operator slot map");
  cudaStream_t s = dfx::as_stream(stream);
  const int32_t n = A->nrows;
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
  const bool pairs = dtype == DFX_F32;
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
  const size_t vb = dtype == DFX_F64 ? 8 : 4;
  if (!st && cudaMalloc(&op->vals, vb * std::max<int64_t>(nslots, 1)) != cudaSuccess)
    st = dfx::fail(DFX_ERR_NO_MEMORY, "operator values: out of device memory");
  if (!st && cudaMalloc(&op->tmp, vb * 2 * std::max<int64_t>(n, 1)) != cudaSuccess)
    st = dfx::fail(DFX_ERR_NO_MEMORY, "operator scratch: out of device memory");
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
  *out = op;
  if (A->vals && A->dtype == DFX_F64)
    return dfx_operator_update_values(op, A, stream);
  return DFX_OK;
}

extern "C" int dfx_operator_update_values(dfx_operator op, const dfx_csr* A, void* stream)
{
  DFX_REQUIRE(op && A && A->vals, "operator and matrix must be non-NULL");
  DFX_REQUIRE(A->dtype == DFX_F64, "values are refilled from FP64 CSR values");
  DFX_REQUIRE(A->nnz == op->csr_nnz && A->nrows == op->n, "matrix does not match the operator");
  cudaStream_t s = dfx::as_stream(stream);
  const unsigned grid = (unsigned)std::min<int64_t>((op->nslots + 255) / 256, 16 * dfx::num_sms());
  if (op->dtype == DFX_F64)
    k_fill<double><<<grid, 256, 0, s>>>(op->map, (const double*)A->vals, (double*)op->vals,
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
  op->owns_structure = 0;
  op->shares = 0;
  op->source = src;
  op->vals = nullptr;
  op->tmp = nullptr;
  const size_t vb = op->dtype == DFX_F64 ? 8 : 4;
  if (cudaMalloc(&op->vals, vb * std::max<int64_t>(op->nslots, 1)) != cudaSuccess
      || cudaMalloc(&op->tmp, vb * 2 * std::max<int64_t>(op->n, 1)) != cudaSuccess)
  {
    if (op->vals)
      cudaFree(op->vals);
    delete op;
    return dfx::fail(DFX_ERR_NO_MEMORY, "operator values: out of device memory");
  }
  src->shares += 1;
  *out = op;
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

extern "C" int dfx_operator_apply(dfx_operator op, const void* d_x, void* d_y, void* stream)
{
  DFX_REQUIRE(op && d_x && d_y, "arguments must be non-NULL");
  cudaStream_t s = dfx::as_stream(stream);
  const int32_t n = op->n;
  if (n == 0)
    return DFX_OK;
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
  DFX_REQUIRE(op && d_x && d_y, "arguments must be non-NULL");
  return dfx::sell_spmv(*op, d_x, d_y, dfx::as_stream(stream));
}
