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

// ---------------------------------------------------------------------------
// Lagrange P1/P2 dofmap of a tetrahedral mesh on the device: the numbering
// of fem::create_dofmap (fem/dofmapbuilder.cpp:440-474, no reordering
// function), i.e. dofs numbered by their first appearance in the cell loop
// where cell c lists its dofs as (4 vertices, 6 edges in Basix order). The
// host builder (setup.cpp) and this one use the same definition, so their
// dofmaps are identical bit for bit:
//   1. every entity's first position p = c nd + i, by atomic minimum
//      (vertices by index; edges in an open-addressing table keyed by the
//      sorted vertex pair);
//   2. a mark at each first position, an exclusive scan of the marks;
//   3. every position takes the scan value at its entity's first position.
namespace
{
__constant__ int kDevEdges[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
constexpr uint64_t kEdgeEmpty = ~uint64_t(0);
constexpr int kEdgeProbes = 1 << 12; // bounded probing; a full table reports UNSUPPORTED

struct DofmapWork
{
  unsigned long long* vfirst; // num_vertices
  unsigned long long* ekey;   // cap
  unsigned long long* efirst; // cap
  int64_t* mark;              // np + 1
  int64_t* scratch;
  int64_t cap;
  size_t bytes;
};

int64_t edge_capacity(int64_t nc)
{
  // A Kuhn-split box has ~7/6 edges per cell, any tetrahedral mesh far
  // fewer than 6: a power of two at least 2.5 edges per cell keeps the
  // load of box meshes below one half.
  int64_t cap = 1024;
  while (cap < 5 * nc / 2 + 16)
    cap <<= 1;
  return cap;
}

DofmapWork carve_dofmap(void* base, int64_t nc, int64_t nv, int degree)
{
  DofmapWork w{};
  char* p = (char*)base;
  size_t off = 0;
  auto take = [&](size_t b) -> char*
  {
    char* r = p ? p + off : nullptr;
    off += a256(b);
    return r;
  };
  const int nd = degree == 1 ? 4 : 10;
  const int64_t np = nd * nc;
  w.cap = degree == 2 ? edge_capacity(nc) : 1;
  w.vfirst = (unsigned long long*)take(8 * (size_t)std::max<int64_t>(nv, 1));
  w.ekey = (unsigned long long*)take(8 * (size_t)w.cap);
  w.efirst = (unsigned long long*)take(8 * (size_t)w.cap);
  w.mark = (int64_t*)take(8 * (size_t)(np + 1));
  w.scratch = (int64_t*)take(8 * (size_t)dfx::scan_scratch_count(np + 1));
  w.bytes = off;
  return w;
}

__device__ __forceinline__ uint64_t mix64(uint64_t k)
{
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

__global__ void k_dofmap_init(DofmapWork w, int64_t nv)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride)
    w.vfirst[i] = ~0ULL;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < w.cap; i += stride)
  {
    w.ekey[i] = kEdgeEmpty;
    w.efirst[i] = ~0ULL;
  }
}

// Step 1; edge dofs keep their table slot in the dofmap until step 3.
template <int DEG>
__global__ void k_dofmap_first(const int32_t* __restrict__ cells, int64_t nc, int64_t nv,
                               DofmapWork w, int32_t* __restrict__ dofmap, int* status)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc)
    return;
  const int4 v4 = __ldg(reinterpret_cast<const int4*>(cells) + c);
  const int32_t v[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
  for (int i = 0; i < 4; ++i)
  {
    if (v[i] < 0 || v[i] >= nv)
    {
      atomicExch(status, (int)DFX_ERR_INVALID);
      return;
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
    atomicMin(w.vfirst + v[i], (unsigned long long)(ND * c + i));
  if constexpr (DEG == 2)
  {
#pragma unroll
    for (int e = 0; e < 6; ++e)
    {
      uint64_t a = (uint32_t)v[kDevEdges[e][0]], b = (uint32_t)v[kDevEdges[e][1]];
      if (a > b)
      {
        const uint64_t t = a;
        a = b;
        b = t;
      }
      const uint64_t key = (a << 32) | b;
      uint64_t slot = mix64(key) & (uint64_t)(w.cap - 1);
      bool placed = false;
      for (int probe = 0; probe < kEdgeProbes; ++probe)
      {
        const unsigned long long prev = atomicCAS(w.ekey + slot, kEdgeEmpty, key);
        if (prev == kEdgeEmpty || prev == key)
        {
          placed = true;
          break;
        }
        slot = (slot + 1) & (uint64_t)(w.cap - 1);
      }
      if (!placed)
      {
        atomicExch(status, (int)DFX_ERR_UNSUPPORTED);
        return;
      }
      atomicMin(w.efirst + slot, (unsigned long long)(ND * c + 4 + e));
      dofmap[ND * c + 4 + e] = (int32_t)slot;
    }
  }
}

// Step 2: marks at the first positions (the mark array was zeroed).
__global__ void k_dofmap_mark(DofmapWork w, int64_t nv)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride)
    if (w.vfirst[i] != ~0ULL)
      w.mark[w.vfirst[i]] = 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < w.cap; i += stride)
    if (w.ekey[i] != kEdgeEmpty)
      w.mark[w.efirst[i]] = 1;
}

// Step 3 (mark now holds the exclusive scan).
template <int DEG>
__global__ void k_dofmap_number(const int32_t* __restrict__ cells, int64_t nc, DofmapWork w,
                                int32_t* __restrict__ dofmap)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc)
    return;
  const int4 v4 = __ldg(reinterpret_cast<const int4*>(cells) + c);
  const int32_t v[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
  for (int i = 0; i < 4; ++i)
    dofmap[ND * c + i] = (int32_t)w.mark[w.vfirst[v[i]]];
  if constexpr (DEG == 2)
#pragma unroll
    for (int e = 0; e < 6; ++e)
    {
      const int32_t slot = dofmap[ND * c + 4 + e];
      dofmap[ND * c + 4 + e] = (int32_t)w.mark[w.efirst[slot]];
    }
}
} // namespace

extern "C" size_t dfx_dofmap_device_workspace_bytes(int32_t num_cells, int32_t num_vertices,
                                                    int32_t degree)
{
  if (num_cells < 0 || num_vertices < 0 || (degree != 1 && degree != 2))
    return 0;
  return carve_dofmap(nullptr, num_cells, num_vertices, degree).bytes;
}

extern "C" int dfx_dofmap_create_tet_device(int32_t num_cells, const int32_t* d_cells,
                                            int32_t num_vertices, int32_t degree,
                                            int32_t* d_dofmap, int32_t* num_nodes, void* d_work,
                                            size_t work_bytes, void* stream)
{
  DFX_REQUIRE(degree == 1 || degree == 2, "Lagrange degree %d not supported", degree);
  DFX_REQUIRE(num_cells >= 0 && num_vertices >= 0 && num_nodes, "invalid dofmap arguments");
  DFX_REQUIRE(num_cells == 0 || (d_cells && d_dofmap), "cells and dofmap must be non-NULL");
  DFX_REQUIRE((int64_t)num_cells * (degree == 1 ? 4 : 10) < INT32_MAX, "dofmap too large");
  DFX_REQUIRE(((uintptr_t)d_cells & 15) == 0, "cells must be 16-byte aligned");
  const DofmapWork need = carve_dofmap(nullptr, num_cells, num_vertices, degree);
  DFX_REQUIRE(d_work && work_bytes >= need.bytes, "workspace too small (%zu < %zu bytes)",
              work_bytes, need.bytes);
  DFX_REQUIRE(((uintptr_t)d_work & 255) == 0, "workspace must be 256-byte aligned");
  *num_nodes = 0;
  if (num_cells == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  const DofmapWork w = carve_dofmap(d_work, num_cells, num_vertices, degree);
  const int nd = degree == 1 ? 4 : 10;
  const int64_t np = (int64_t)nd * num_cells;
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  const unsigned sg = (unsigned)(8 * dfx::num_sms());
  const unsigned cg = (unsigned)((num_cells + 255) / 256);
  k_dofmap_init<<<sg, 256, 0, s>>>(w, num_vertices);
  if (degree == 1)
    k_dofmap_first<1><<<cg, 256, 0, s>>>(d_cells, num_cells, num_vertices, w, d_dofmap, status);
  else
    k_dofmap_first<2><<<cg, 256, 0, s>>>(d_cells, num_cells, num_vertices, w, d_dofmap, status);
  DFX_CHECK_LAUNCH();
  if (int h = read_status(status, s))
  {
    if (h == DFX_ERR_INVALID)
      return dfx::fail(DFX_ERR_INVALID, "cell vertex index out of range [0, %d)", num_vertices);
    return dfx::fail(DFX_ERR_UNSUPPORTED, "edge table full: use the host builder");
  }
  DFX_CUDA(cudaMemsetAsync(w.mark, 0, sizeof(int64_t) * (size_t)(np + 1), s));
  k_dofmap_mark<<<sg, 256, 0, s>>>(w, num_vertices);
  DFX_CHECK_LAUNCH();
  if (int st = dfx::exclusive_scan(w.mark, w.mark, np, w.scratch, s))
    return st;
  if (degree == 1)
    k_dofmap_number<1><<<cg, 256, 0, s>>>(d_cells, num_cells, w, d_dofmap);
  else
    k_dofmap_number<2><<<cg, 256, 0, s>>>(d_cells, num_cells, w, d_dofmap);
  DFX_CHECK_LAUNCH();
  int64_t total = 0;
  DFX_CUDA(cudaMemcpyAsync(&total, w.mark + np, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  *num_nodes = (int32_t)total;
  return DFX_OK;
}
