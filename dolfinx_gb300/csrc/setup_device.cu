// Device-side structure set-up: the cell sparsity pattern of a dofmap
// (fem::create_sparsity_pattern + SparsityPattern::finalize,
// fem/utils.h:197-314, la/SparsityPattern.cpp:264-491) built on the GPU.
//
// The pattern is defined as a set: row r holds, sorted and without
// repeats, every dof that shares a cell with dof r. The host builder
// (setup.cpp) and this one compute that same set, so their row pointers
// and columns are identical bit for bit whatever order the device visits
// the cells in.
//
//   1. dof -> cell transpose: counts (integer atomics), exclusive scan,
//      fill (the order inside a dof's list is arbitrary);
//   2. one warp per row gathers the dofs of the row's cells into shared
//      memory (at most kRowCap candidates), sorts them with a bitonic
//      network and keeps the first of each run of equal values;
//   3. pass A counts the row lengths, a scan gives the row pointers, and
//      pass B repeats 1-2 and writes the columns.
#include "scan.cuh"

#include <algorithm>

namespace
{
constexpr int kRowWarps = 4;
constexpr int kRowCap = 1024; // candidate columns of one row (cells x nd)

__global__ void k_scan_blocks(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                              int64_t* __restrict__ sums)
{
  __shared__ int64_t warp_tot[dfx::kScanBlock / 32];
  const int64_t i = (int64_t)blockIdx.x * dfx::kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t v = i < n ? in[i] : 0;
  int64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o)
      incl += t;
  }
  if (lane == 31)
    warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0)
  {
    int64_t t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    int64_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const int64_t u = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o)
        ti += u;
    }
    warp_tot[lane] = ti - t; // exclusive offset of each warp
    if (lane == 31)
      sums[blockIdx.x] = ti;
  }
  __syncthreads();
  if (i < n)
    out[i] = warp_tot[warp] + incl - v;
}

// One block: exclusive scan of the block totals in place, total -> *total.
__global__ void k_scan_sums(int64_t* __restrict__ sums, int64_t nb, int64_t* __restrict__ total)
{
  __shared__ int64_t warp_tot[dfx::kScanBlock / 32];
  __shared__ int64_t carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0)
    carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nb; b0 += dfx::kScanBlock)
  {
    const int64_t i = b0 + threadIdx.x;
    const int64_t v = i < nb ? sums[i] : 0;
    int64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o)
        incl += t;
    }
    if (lane == 31)
      warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
      const int64_t t = warp_tot[lane];
      int64_t ti = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
      {
        const int64_t u = __shfl_up_sync(0xffffffffu, ti, o);
        if (lane >= o)
          ti += u;
      }
      warp_tot[lane] = ti - t;
    }
    __syncthreads();
    const int64_t c = carry;
    if (i < nb)
      sums[i] = c + warp_tot[warp] + incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1)
      carry = c + warp_tot[warp] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0)
    *total = carry;
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ sums)
{
  const int64_t i = (int64_t)blockIdx.x * dfx::kScanBlock + threadIdx.x;
  if (i < n)
    out[i] += sums[blockIdx.x];
}

// Cells per dof. Out-of-range dofmap entries are reported and skipped.
__global__ void k_dof_count(const int32_t* __restrict__ dofmap, int64_t m, int32_t nrows,
                            unsigned long long* __restrict__ cnt, int* __restrict__ status)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t d = __ldg(dofmap + t);
    if (d < 0 || d >= nrows)
    {
      atomicExch(status, (int)DFX_ERR_INVALID);
      continue;
    }
    atomicAdd(cnt + d, 1ull);
  }
}

__global__ void k_dof_fill(const int32_t* __restrict__ dofmap, int64_t m, int32_t nd,
                           int32_t nrows, const int64_t* __restrict__ ptr,
                           unsigned long long* __restrict__ pos, int32_t* __restrict__ adj)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t d = __ldg(dofmap + t);
    if (d < 0 || d >= nrows)
      continue;
    const unsigned long long p = atomicAdd(pos + d, 1ull);
    adj[ptr[d] + (int64_t)p] = (int32_t)(t / nd);
  }
}

// Sorted unique columns of each row (see the file comment). FILL = false:
// row lengths into len; FILL = true: columns at row_ptr.
template <bool FILL>
__global__ void __launch_bounds__(32 * kRowWarps)
    k_sparsity_rows(int32_t nrows, int32_t nd, const int32_t* __restrict__ dofmap,
                    const int64_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj,
                    int64_t* __restrict__ len, const int64_t* __restrict__ row_ptr,
                    int32_t* __restrict__ cols, int* __restrict__ status)
{
  __shared__ int32_t sbuf[kRowWarps][kRowCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* buf = sbuf[warp];
  for (int64_t r = (int64_t)blockIdx.x * kRowWarps + warp; r < nrows;
       r += (int64_t)gridDim.x * kRowWarps)
  {
    const int64_t a0 = adj_ptr[r], a1 = adj_ptr[r + 1];
    const int64_t cand = (a1 - a0) * nd;
    if (cand > kRowCap)
    {
      if (lane == 0)
      {
        atomicExch(status, (int)DFX_ERR_UNSUPPORTED);
        if (!FILL)
          len[r] = 0;
      }
      continue;
    }
    int P = 32;
    while (P < cand)
      P <<= 1;
    for (int i = lane; i < P; i += 32)
    {
      int32_t v = INT32_MAX;
      if (i < cand)
      {
        const int k = i / nd, li = i - k * nd;
        v = __ldg(dofmap + (int64_t)adj[a0 + k] * nd + li);
      }
      buf[i] = v;
    }
    __syncwarp();
    // Bitonic sort, ascending: each compare-exchange pair (i, i^j) with
    // i < i^j belongs to one lane.
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1)
      {
        for (int i = lane; i < P; i += 32)
        {
          const int l = i ^ j;
          if (l > i)
          {
            const int32_t x = buf[i], y = buf[l];
            if ((x > y) == ((i & k) == 0))
            {
              buf[i] = y;
              buf[l] = x;
            }
          }
        }
        __syncwarp();
      }
    int64_t base = 0;
    for (int i0 = 0; i0 < P; i0 += 32)
    {
      const int i = i0 + lane;
      const int32_t v = buf[i];
      const bool first = v != INT32_MAX && (i == 0 || buf[i - 1] != v);
      const unsigned b = __ballot_sync(0xffffffffu, first);
      if (FILL && first)
        cols[row_ptr[r] + base + __popc(b & ((1u << lane) - 1u))] = v;
      base += __popc(b);
    }
    if (!FILL && lane == 0)
      len[r] = base;
    __syncwarp();
  }
}

struct SparsityWork
{
  int64_t* ptr;        // nrows + 1: dof -> cell offsets
  int64_t* cnt;        // nrows: counts, then fill positions; pass A: row lengths
  int32_t* adj;        // num_cells * nd
  int64_t* scratch;    // scan scratch
  size_t bytes;
};

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

SparsityWork carve(void* base, int32_t nrows, int32_t num_cells, int32_t nd)
{
  SparsityWork w{};
  char* p = (char*)base;
  size_t off = 0;
  auto take = [&](size_t b) -> char*
  {
    char* r = p ? p + off : nullptr;
    off += a256(b);
    return r;
  };
  w.ptr = (int64_t*)take(sizeof(int64_t) * ((size_t)nrows + 1));
  w.cnt = (int64_t*)take(sizeof(int64_t) * std::max<size_t>(1, (size_t)nrows + 1));
  w.adj = (int32_t*)take(sizeof(int32_t) * std::max<size_t>(1, (size_t)num_cells * nd));
  w.scratch = (int64_t*)take(sizeof(int64_t) * dfx::scan_scratch_count((int64_t)nrows + 1));
  w.bytes = off;
  return w;
}

int grid_for(int64_t m, int threads)
{
  const int64_t need = (m + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)dfx::num_sms() * 16));
}

int read_status(int* status, cudaStream_t s)
{
  int h = 0;
  DFX_CUDA(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return h;
}

// Steps 1 of the file comment: the dof -> cell transpose in w.
int transpose(const int32_t* dofmap, int32_t nrows, int32_t num_cells, int32_t nd,
              const SparsityWork& w, int* status, cudaStream_t s)
{
  const int64_t m = (int64_t)num_cells * nd;
  DFX_CUDA(cudaMemsetAsync(w.cnt, 0, sizeof(int64_t) * ((size_t)nrows + 1), s));
  k_dof_count<<<grid_for(m, 256), 256, 0, s>>>(dofmap, m, nrows, (unsigned long long*)w.cnt,
                                               status);
  DFX_CHECK_LAUNCH();
  if (int st = dfx::exclusive_scan(w.cnt, w.ptr, nrows, w.scratch, s))
    return st;
  DFX_CUDA(cudaMemsetAsync(w.cnt, 0, sizeof(int64_t) * ((size_t)nrows + 1), s));
  k_dof_fill<<<grid_for(m, 256), 256, 0, s>>>(dofmap, m, nd, nrows, w.ptr,
                                              (unsigned long long*)w.cnt, w.adj);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}
} // namespace

namespace dfx
{
int exclusive_scan(const int64_t* in, int64_t* out, int64_t n, int64_t* scratch, cudaStream_t s)
{
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb > 0)
  {
    k_scan_blocks<<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, n, scratch);
    DFX_CHECK_LAUNCH();
  }
  k_scan_sums<<<1, kScanBlock, 0, s>>>(scratch, nb, out + n);
  DFX_CHECK_LAUNCH();
  if (nb > 0)
  {
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(out, n, scratch);
    DFX_CHECK_LAUNCH();
  }
  return DFX_OK;
}
} // namespace dfx

extern "C" size_t dfx_sparsity_device_workspace_bytes(int32_t nrows, int32_t num_cells, int32_t nd)
{
  if (nrows < 0 || num_cells < 0 || nd <= 0)
    return 0;
  return carve(nullptr, nrows, num_cells, nd).bytes;
}

extern "C" int dfx_sparsity_create_device(int32_t nrows, int32_t num_cells, int32_t nd,
                                          const int32_t* d_dofmap, int64_t* d_row_ptr,
                                          int32_t* d_cols, int64_t* nnz, void* d_work,
                                          size_t work_bytes, void* stream)
{
  DFX_REQUIRE(nrows >= 0 && num_cells >= 0 && nd > 0, "invalid sparsity arguments");
  DFX_REQUIRE(d_row_ptr && nnz, "row_ptr and nnz must be non-NULL");
  DFX_REQUIRE(num_cells == 0 || d_dofmap, "dofmap must be non-NULL");
  DFX_REQUIRE((int64_t)num_cells * nd < INT32_MAX, "dofmap too large");
  const SparsityWork need = carve(nullptr, nrows, num_cells, nd);
  DFX_REQUIRE(d_work && work_bytes >= need.bytes, "workspace too small (%zu < %zu bytes)",
              work_bytes, need.bytes);
  DFX_REQUIRE(((uintptr_t)d_work & 255) == 0, "workspace must be 256-byte aligned");
  cudaStream_t s = dfx::as_stream(stream);
  const SparsityWork w = carve(d_work, nrows, num_cells, nd);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  if (int st = transpose(d_dofmap, nrows, num_cells, nd, w, status, s))
    return st;
  const int rows_grid =
      (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)nrows + kRowWarps - 1) / kRowWarps,
                                                  (int64_t)dfx::num_sms() * 32));
  if (!d_cols)
  {
    // Pass A: lengths into w.cnt, then row pointers.
    k_sparsity_rows<false><<<rows_grid, 32 * kRowWarps, 0, s>>>(
        nrows, nd, d_dofmap, w.ptr, w.adj, w.cnt, nullptr, nullptr, status);
    DFX_CHECK_LAUNCH();
    if (int st = dfx::exclusive_scan(w.cnt, d_row_ptr, nrows, w.scratch, s))
      return st;
    DFX_CUDA(cudaMemcpyAsync(nnz, d_row_ptr + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  }
  else
  {
    // Pass B: columns at the row pointers of pass A.
    k_sparsity_rows<true><<<rows_grid, 32 * kRowWarps, 0, s>>>(
        nrows, nd, d_dofmap, w.ptr, w.adj, nullptr, d_row_ptr, d_cols, status);
    DFX_CHECK_LAUNCH();
    DFX_CUDA(cudaMemcpyAsync(nnz, d_row_ptr + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  }
  const int h = read_status(status, s);
  if (h == DFX_ERR_INVALID)
    return dfx::fail(DFX_ERR_INVALID, "dofmap entry out of range [0, %d)", nrows);
  if (h == DFX_ERR_UNSUPPORTED)
    return dfx::fail(DFX_ERR_UNSUPPORTED,
                     "a row has more than %d candidate columns (cells x dofs per cell): use "
                     "the host builder",
                     kRowCap);
  return h;
}
