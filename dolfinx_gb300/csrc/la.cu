// Linear algebra on la::MatrixCSR / la::Vector storage: CSR SpMV (FP64,
// FP32 values, 3x3 blocks), the float cast of the values, the Jacobi
// diagonal and a deterministic inner product.
#include "la_kernels.cuh"

namespace
{
__global__ void k_to_f32(const double* __restrict__ v, float* __restrict__ o, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    o[i] = (float)v[i];
}

__global__ void k_jacobi(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                         const double* __restrict__ vals, int bs, int32_t nrows,
                         double* __restrict__ dinv)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nrows * bs)
    return;
  const int32_t r = (int32_t)(t / bs), k = (int32_t)(t % bs);
  int64_t b = row_ptr[r], e = row_ptr[r + 1];
  while (b < e)
  {
    const int64_t m = (b + e) >> 1;
    if (cols[m] < r)
      b = m + 1;
    else
      e = m;
  }
  const double d = (b < row_ptr[r + 1] && cols[b] == r) ? vals[b * bs * bs + k * bs + k] : 0.0;
  dinv[t] = d != 0.0 ? 1.0 / d : 0.0;
}

__global__ void k_dot_partial(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                              double* __restrict__ partial)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += a[i] * b[i];
  s = dfx::block_sum(s, sh);
  if (threadIdx.x == 0)
    partial[blockIdx.x] = s;
}

__global__ void k_sum_partials(const double* __restrict__ partial, int n, double* __restrict__ out)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    s += partial[i];
  s = dfx::block_sum(s, sh);
  if (threadIdx.x == 0)
    *out = s;
}
} // namespace

namespace dfx
{
int spmv_lanes(const dfx_csr* A)
{
  const int t = tuned_get(kTuneSpmv, A->nrows, A->nnz, 4 * A->bs + A->dtype);
  return t ? t : spmv_lanes_heuristic(A);
}

int launch_spmv(const dfx_csr* A, const void* x, void* y, double beta, cudaStream_t s, int lanes)
{
  const bool acc = beta != 0.0;
  if (A->nrows == 0)
    return DFX_OK;
  if (A->bs == 1)
  {
    if (lanes == 0)
      lanes = spmv_lanes(A);
    const int rows_per_block = kSpmvThreads / lanes;
    const unsigned grid = (unsigned)((A->nrows + rows_per_block - 1) / rows_per_block);
    if (A->dtype == DFX_F64)
    {
#define DFX_SPMV_CASE(L)                                                                           \
  case L:                                                                                          \
    if (acc)                                                                                       \
      k_spmv_csr<L, double, double, double, true><<<grid, kSpmvThreads, 0, s>>>(                   \
          A->nrows, A->row_ptr, A->cols, (const double*)A->vals, (const double*)x, (double*)y);    \
    else                                                                                           \
      k_spmv_csr<L, double, double, double, false><<<grid, kSpmvThreads, 0, s>>>(                  \
          A->nrows, A->row_ptr, A->cols, (const double*)A->vals, (const double*)x, (double*)y);    \
    break;
      switch (lanes)
      {
        DFX_SPMV_CASE(4)
        DFX_SPMV_CASE(8)
        DFX_SPMV_CASE(16)
        DFX_SPMV_CASE(32)
      }
#undef DFX_SPMV_CASE
    }
    else
    {
#define DFX_SPMV_CASE(L)                                                                           \
  case L:                                                                                          \
    if (acc)                                                                                       \
      k_spmv_csr<L, float, float, float, true><<<grid, kSpmvThreads, 0, s>>>(                      \
          A->nrows, A->row_ptr, A->cols, (const float*)A->vals, (const float*)x, (float*)y);       \
    else                                                                                           \
      k_spmv_csr<L, float, float, float, false><<<grid, kSpmvThreads, 0, s>>>(                     \
          A->nrows, A->row_ptr, A->cols, (const float*)A->vals, (const float*)x, (float*)y);       \
    break;
      switch (lanes)
      {
        DFX_SPMV_CASE(4)
        DFX_SPMV_CASE(8)
        DFX_SPMV_CASE(16)
        DFX_SPMV_CASE(32)
      }
#undef DFX_SPMV_CASE
    }
  }
  else if (A->bs == 3)
  {
    const int rows_per_block = kSpmvThreads / 8;
    const unsigned grid = (unsigned)((A->nrows + rows_per_block - 1) / rows_per_block);
    if (A->dtype == DFX_F64)
    {
      if (acc)
        k_spmv_bsr3<double, double, double, true><<<grid, kSpmvThreads, 0, s>>>(
            A->nrows, A->row_ptr, A->cols, (const double*)A->vals, (const double*)x, (double*)y);
      else
        k_spmv_bsr3<double, double, double, false><<<grid, kSpmvThreads, 0, s>>>(
            A->nrows, A->row_ptr, A->cols, (const double*)A->vals, (const double*)x, (double*)y);
    }
    else
    {
      if (acc)
        k_spmv_bsr3<float, float, float, true><<<grid, kSpmvThreads, 0, s>>>(
            A->nrows, A->row_ptr, A->cols, (const float*)A->vals, (const float*)x, (float*)y);
      else
        k_spmv_bsr3<float, float, float, false><<<grid, kSpmvThreads, 0, s>>>(
            A->nrows, A->row_ptr, A->cols, (const float*)A->vals, (const float*)x, (float*)y);
    }
  }
  else
    return fail(DFX_ERR_UNSUPPORTED, "block size %d not supported", A->bs);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

int check_csr(const dfx_csr* A)
{
  DFX_REQUIRE(A, "matrix is NULL");
  DFX_REQUIRE(A->nrows >= 0 && A->ncols >= 0 && A->nnz >= 0, "negative matrix sizes");
  DFX_REQUIRE(A->bs == 1 || A->bs == 3, "block size %d not supported", A->bs);
  DFX_REQUIRE(A->dtype == DFX_F64 || A->dtype == DFX_F32, "unknown dtype %d", A->dtype);
  if (A->nrows > 0)
    DFX_REQUIRE(A->row_ptr && A->cols && A->vals, "matrix arrays must be non-NULL");
  return DFX_OK;
}
} // namespace dfx

extern "C" int dfx_spmv(const dfx_csr* A, const void* d_x, void* d_y, double beta, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(beta == 0.0 || beta == 1.0, "beta must be 0 or 1");
  DFX_REQUIRE(d_x && d_y, "x and y must be non-NULL");
  return dfx::launch_spmv(A, d_x, d_y, beta, dfx::as_stream(stream));
}

extern "C" int dfx_tune_spmv(const dfx_csr* A, const void* d_x, void* d_y, int32_t* best_lanes,
                             float* ms, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->bs == 1, "the row split applies to scalar CSR matrices");
  DFX_REQUIRE(d_x && d_y && best_lanes, "x, y and best_lanes must be non-NULL");
  cudaStream_t s = dfx::as_stream(stream);
  constexpr int kCand[4] = {4, 8, 16, 32};
  constexpr int kReps = 5;
  cudaEvent_t e0, e1;
  DFX_CUDA(cudaEventCreate(&e0));
  DFX_CUDA(cudaEventCreate(&e1));
  int best = 0;
  float best_ms = 0.0f;
  int st = DFX_OK;
  for (int c = 0; c < 4 && !st; ++c)
  {
    st = dfx::launch_spmv(A, d_x, d_y, 0.0, s, kCand[c]); // warm-up
    if (!st && cudaEventRecord(e0, s) != cudaSuccess)
      st = dfx::fail(DFX_ERR_CUDA, "event record failed");
    for (int r = 0; r < kReps && !st; ++r)
      st = dfx::launch_spmv(A, d_x, d_y, 0.0, s, kCand[c]);
    float t = 0.0f;
    if (!st && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess
                || cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
      st = dfx::fail(DFX_ERR_CUDA, "SpMV timing failed");
    t /= kReps;
    if (ms)
      ms[c] = t;
    if (!st && (best == 0 || t < best_ms))
    {
      best = kCand[c];
      best_ms = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st)
    return st;
  dfx::tuned_set(dfx::kTuneSpmv, A->nrows, A->nnz, 4 * A->bs + A->dtype, best);
  *best_lanes = best;
  return DFX_OK;
}

extern "C" int dfx_set_spmv_lanes(const dfx_csr* A, int32_t lanes)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->bs == 1, "the row split applies to scalar CSR matrices");
  DFX_REQUIRE(lanes == 0 || lanes == 4 || lanes == 8 || lanes == 16 || lanes == 32,
              "lanes per row must be 4, 8, 16 or 32 (0: default)");
  dfx::tuned_set(dfx::kTuneSpmv, A->nrows, A->nnz, 4 * A->bs + A->dtype, lanes);
  return DFX_OK;
}

extern "C" int dfx_get_spmv_lanes(const dfx_csr* A, int32_t* lanes)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(lanes, "lanes must be non-NULL");
  *lanes = A->bs == 1 ? dfx::spmv_lanes(A) : 8;
  return DFX_OK;
}

extern "C" int dfx_csr_values_to_f32(const dfx_csr* A, float* d_vals32, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->dtype == DFX_F64, "source values must be FP64");
  const int64_t n = A->nnz * A->bs * A->bs;
  if (n == 0)
    return DFX_OK;
  const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 16 * dfx::num_sms());
  k_to_f32<<<grid, 256, 0, dfx::as_stream(stream)>>>((const double*)A->vals, d_vals32, n);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_jacobi_inverse_diagonal(const dfx_csr* A, double* d_dinv, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->dtype == DFX_F64, "values must be FP64");
  const int64_t n = (int64_t)A->nrows * A->bs;
  if (n == 0)
    return DFX_OK;
  k_jacobi<<<(unsigned)((n + 255) / 256), 256, 0, dfx::as_stream(stream)>>>(
      A->row_ptr, A->cols, (const double*)A->vals, A->bs, A->nrows, d_dinv);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" size_t dfx_inner_product_workspace_bytes(int64_t n)
{
  (void)n;
  return sizeof(double) * (size_t)(8 * 152 + 8);
}

extern "C" int dfx_inner_product(const double* d_a, const double* d_b, int64_t n, void* d_work,
                                 size_t work_bytes, double* result, void* stream)
{
  DFX_REQUIRE(result, "result must be non-NULL");
  DFX_REQUIRE(n >= 0, "negative size");
  if (n == 0)
  {
    *result = 0.0;
    return DFX_OK;
  }
  DFX_REQUIRE(d_a && d_b && d_work, "arrays must be non-NULL");
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4 * dfx::num_sms());
  DFX_REQUIRE(work_bytes >= sizeof(double) * (size_t)(blocks + 1), "workspace too small");
  cudaStream_t s = dfx::as_stream(stream);
  double* partial = (double*)d_work;
  k_dot_partial<<<blocks, 256, 0, s>>>(d_a, d_b, n, partial);
  k_sum_partials<<<1, 256, 0, s>>>(partial, blocks, partial + blocks);
  DFX_CHECK_LAUNCH();
  DFX_CUDA(cudaMemcpyAsync(result, partial + blocks, sizeof(double), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}

namespace
{
// Scalar row 3 I + k0 of a 3x3-block CSR: row_ptr = 9 rp[I] + 3 k0 len(I).
__global__ void k_expand_rowptr(const int64_t* __restrict__ rp, int32_t nrows, int bs,
                                int64_t* __restrict__ out)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nr = (int64_t)nrows * bs;
  if (t > nr)
    return;
  if (t == nr)
  {
    out[t] = (int64_t)bs * bs * rp[nrows];
    return;
  }
  const int64_t I = t / bs, k0 = t % bs;
  const int64_t len = rp[I + 1] - rp[I];
  out[t] = (int64_t)bs * bs * rp[I] + (int64_t)bs * k0 * len;
}

// One thread per scalar entry of the expanded matrix, in block order.
__global__ void k_expand_entries(const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                 const double* __restrict__ vals, int32_t nrows, int bs,
                                 const int64_t* __restrict__ orp, int32_t* __restrict__ ocols,
                                 double* __restrict__ ovals, int64_t nnz)
{
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz * bs * bs)
    return;
  const int64_t j = e / (bs * bs);
  const int r = (int)(e % (bs * bs)), k0 = r / bs, k1 = r % bs;
  // block row of entry j: binary search in rp
  int32_t lo = 0, hi = nrows;
  while (hi - lo > 1)
  {
    const int32_t m = (lo + hi) >> 1;
    if (rp[m] <= j)
      lo = m;
    else
      hi = m;
  }
  const int64_t I = lo;
  const int64_t pos = orp[bs * I + k0] + (int64_t)bs * (j - rp[I]) + k1;
  if (ocols)
    ocols[pos] = bs * cols[j] + k1;
  ovals[pos] = vals[e];
}
} // namespace

extern "C" int dfx_csr_expand_blocks(const dfx_csr* A, int64_t* d_row_ptr, int32_t* d_cols,
                                     double* d_vals, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->dtype == DFX_F64, "values must be FP64");
  DFX_REQUIRE(d_row_ptr && d_vals, "row_ptr and vals must be non-NULL");
  const int bs = A->bs;
  const int64_t nr = (int64_t)A->nrows * bs;
  DFX_REQUIRE(nr < INT32_MAX && (int64_t)A->ncols * bs < INT32_MAX, "matrix too large");
  cudaStream_t s = dfx::as_stream(stream);
  k_expand_rowptr<<<(unsigned)((nr + 256) / 256), 256, 0, s>>>(A->row_ptr, A->nrows, bs, d_row_ptr);
  const int64_t ne = A->nnz * bs * bs;
  if (ne > 0)
    k_expand_entries<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(
        A->row_ptr, A->cols, (const double*)A->vals, A->nrows, bs, d_row_ptr, d_cols,
        (double*)d_vals, A->nnz);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}
