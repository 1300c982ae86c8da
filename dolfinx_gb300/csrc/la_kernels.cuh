// CSR SpMV device building blocks shared by la.cu and the CG kernels.
//
// Scalar CSR: a group of L lanes per row walks the row's entries with a
// stride of L (coalesced 4/8-byte streams of values and column indices),
// gathers x through the read-only path (x stays L2-resident), and reduces
// with shuffles. 3x3 blocks: the row's values are streamed as one flat
// array (9 per block) so loads stay coalesced; each lane keeps three
// partial row sums.
#pragma once

#include "common.cuh"
#include <algorithm>

namespace dfx
{
constexpr int kSpmvThreads = 256;

// y (+)= A x with `lanes` lanes per row (scalar CSR; 0: spmv_lanes(A)).
int launch_spmv(const dfx_csr* A, const void* x, void* y, double beta, cudaStream_t s,
                int lanes = 0);
int check_csr(const dfx_csr* A);

// Lanes per row of a scalar CSR matrix: the autotuner's choice for this
// matrix shape (dfx_tune_spmv / dfx_set_spmv_lanes) if there is one, else
// spmv_lanes_heuristic.
int spmv_lanes(const dfx_csr* A);

// Lanes per row for a scalar CSR matrix from its mean row length.
inline int spmv_lanes_heuristic(const dfx_csr* A)
{
  const double avg = A->nrows ? (double)A->nnz / A->nrows : 0.0;
  if (avg <= 6)
    return 4;
  if (avg <= 14)
    return 8;
  if (avg <= 40)
    return 16;
  return 32;
}

#ifdef __CUDACC__
// Partial row sum of lane `lane` (0..L-1) of the group owning `row`.
template <int L, typename V, typename X, typename ACC>
__device__ __forceinline__ ACC csr_row_partial(const int64_t* __restrict__ rp,
                                               const int32_t* __restrict__ cols,
                                               const V* __restrict__ vals,
                                               const X* __restrict__ x, int32_t row, int lane)
{
  ACC s = ACC(0);
  const int64_t b = __ldg(rp + row), e = __ldg(rp + row + 1);
  for (int64_t j = b + lane; j < e; j += L)
    s += (ACC)ld_stream(vals + j) * (ACC)__ldg(x + ld_stream(cols + j));
  return s;
}

template <int L, typename T>
__device__ __forceinline__ T group_sum(T s)
{
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
    s += __shfl_down_sync(0xffffffffu, s, o, L);
  return s;
}

template <int L, typename V, typename X, typename ACC, bool BETA>
__global__ void __launch_bounds__(kSpmvThreads)
    k_spmv_csr(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
               const V* __restrict__ vals, const X* __restrict__ x, X* __restrict__ y)
{
  const int32_t row = blockIdx.x * (kSpmvThreads / L) + threadIdx.x / L;
  const int lane = threadIdx.x % L;
  ACC s = ACC(0);
  if (row < nrows)
    s = csr_row_partial<L, V, X, ACC>(rp, cols, vals, x, row, lane);
  s = group_sum<L>(s);
  if (row < nrows && lane == 0)
    y[row] = BETA ? (X)((ACC)y[row] + s) : (X)s;
}

// Three partial row sums of a 3x3-block row for lane `lane` of 8.
template <typename V, typename X, typename ACC>
__device__ __forceinline__ void bsr3_row_partial(const int64_t* __restrict__ rp,
                                                 const int32_t* __restrict__ cols,
                                                 const V* __restrict__ vals,
                                                 const X* __restrict__ x, int32_t row, int lane,
                                                 ACC& s0, ACC& s1, ACC& s2)
{
  const int64_t b = __ldg(rp + row), e = __ldg(rp + row + 1);
  const int64_t n = 9 * (e - b);
  const V* v = vals + 9 * b;
  for (int64_t t = lane; t < n; t += 8)
  {
    const int64_t blk = t / 9;
    const int r = (int)(t - 9 * blk);
    const int k0 = r / 3, k1 = r - 3 * k0;
    const ACC p = (ACC)ld_stream(v + t) * (ACC)__ldg(x + 3 * (int64_t)__ldg(cols + b + blk) + k1);
    if (k0 == 0)
      s0 += p;
    else if (k0 == 1)
      s1 += p;
    else
      s2 += p;
  }
}

template <typename V, typename X, typename ACC, bool BETA>
__global__ void __launch_bounds__(kSpmvThreads)
    k_spmv_bsr3(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
                const V* __restrict__ vals, const X* __restrict__ x, X* __restrict__ y)
{
  const int32_t row = blockIdx.x * (kSpmvThreads / 8) + threadIdx.x / 8;
  const int lane = threadIdx.x % 8;
  ACC s0 = 0, s1 = 0, s2 = 0;
  if (row < nrows)
    bsr3_row_partial<V, X, ACC>(rp, cols, vals, x, row, lane, s0, s1, s2);
  s0 = group_sum<8>(s0);
  s1 = group_sum<8>(s1);
  s2 = group_sum<8>(s2);
  if (row < nrows && lane == 0)
  {
    X* yr = y + 3 * (int64_t)row;
    yr[0] = BETA ? (X)((ACC)yr[0] + s0) : (X)s0;
    yr[1] = BETA ? (X)((ACC)yr[1] + s1) : (X)s1;
    yr[2] = BETA ? (X)((ACC)yr[2] + s2) : (X)s2;
  }
}
#endif
} // namespace dfx
