// Jacobi-preconditioned conjugate gradients on the device.
//
// The iteration of the reference demo (cpp/demo/poisson_matrix_free/
// main.cpp:84-132) as three fused kernels per iteration:
//   1. y = A p and p.y           (SpMV with a fused dot product)
//   2. x += a p, r -= a y, z = D^{-1} r, r.r and r.z, convergence test
//   3. p = z + b p
// Every reduction is two-stage and deterministic: per-block partial sums,
// then the last block to finish (atomic ticket) sums the partials in index
// order and updates the scalar state in device memory. Scalars never leave
// the device; kernels return immediately once the state says "done", so a
// CUDA graph of K iterations is replayed until the host sees done.
#include "la_kernels.cuh"

#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

namespace
{
constexpr int kThreads = 256;

struct CgState
{
  double rz;    // r.z
  double rr0;   // |r0|^2
  double rr;    // |r|^2
  double pAp;   // p.Ap
  double alpha;
  double beta;
  double rtol2;
  int32_t iter;
  int32_t max_iter;
  int32_t done;
  int32_t status;
  unsigned int ticket[4];
};

struct Work
{
  CgState* st;
  double* part0;
  double* part1;
  double* r;
  double* p;
  double* y;
  int blocks;
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int grid_blocks() { return 4 * dfx::num_sms(); }

size_t work_bytes(int64_t n, int blocks)
{
  return align256(sizeof(CgState)) + 2 * align256(sizeof(double) * blocks)
         + 3 * align256(sizeof(double) * (size_t)n);
}

Work carve(void* w, int64_t n, int blocks)
{
  char* p = (char*)w;
  Work k;
  k.st = (CgState*)p;
  p += align256(sizeof(CgState));
  k.part0 = (double*)p;
  p += align256(sizeof(double) * blocks);
  k.part1 = (double*)p;
  p += align256(sizeof(double) * blocks);
  k.r = (double*)p;
  p += align256(sizeof(double) * n);
  k.p = (double*)p;
  p += align256(sizeof(double) * n);
  k.y = (double*)p;
  k.blocks = blocks;
  return k;
}

// Publish this block's partial sums; returns true in the last block.
__device__ __forceinline__ bool publish(double v0, double v1, double* p0, double* p1,
                                        unsigned int* ticket, bool two)
{
  __shared__ double sh[32];
  __shared__ bool last;
  v0 = dfx::block_sum(v0, sh);
  if (two)
    v1 = dfx::block_sum(v1, sh);
  if (threadIdx.x == 0)
  {
    p0[blockIdx.x] = v0;
    if (two)
      p1[blockIdx.x] = v1;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  return last;
}

// Deterministic sum of gridDim.x partials (called by the last block).
__device__ __forceinline__ double final_sum(const double* p)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
    s += __ldcg(p + i);
  return dfx::block_sum(s, sh);
}

__device__ __forceinline__ bool is_done(const CgState* st)
{
  return __ldcg(&st->done) != 0;
}

template <bool PRE>
__global__ void __launch_bounds__(kThreads)
    k_cg_init(const double* __restrict__ b, const double* __restrict__ dinv, int64_t n,
              Work w, double rtol2, int max_iter)
{
  double rr = 0.0, rz = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const double r = b[i] - w.y[i];
    const double z = PRE ? dinv[i] * r : r;
    w.r[i] = r;
    w.p[i] = z;
    rr += r * r;
    rz += r * z;
  }
  if (publish(rr, rz, w.part0, w.part1, &w.st->ticket[0], true))
  {
    const double srr = final_sum(w.part0);
    const double srz = final_sum(w.part1);
    if (threadIdx.x == 0)
    {
      CgState* st = w.st;
      st->rr0 = srr;
      st->rr = srr;
      st->rz = srz;
      st->rtol2 = rtol2;
      st->iter = 0;
      st->max_iter = max_iter;
      st->done = (srr == 0.0) ? 1 : 0;
      st->status = DFX_OK;
      st->ticket[0] = 0;
      __threadfence();
    }
  }
}

// y = A p and p.y; alpha = rz / p.y.
template <int L, int BS>
__global__ void __launch_bounds__(kThreads)
    k_cg_spmv_dot(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
                  const double* __restrict__ vals, Work w)
{
  if (is_done(w.st))
    return;
  constexpr int G = BS == 1 ? L : 8; // lanes per row
  const int lane = threadIdx.x % G;
  const int groups = gridDim.x * (kThreads / G);
  double dot = 0.0;
  // The loop bound is uniform per block, so all lanes of a warp take part
  // in every shuffle below.
  for (int32_t base = blockIdx.x * (kThreads / G); base < nrows; base += groups)
  {
    const int32_t row = base + threadIdx.x / G;
    const bool active = row < nrows;
    if constexpr (BS == 1)
    {
      double s = active ? dfx::csr_row_partial<L, double, double, double>(rp, cols, vals, w.p,
                                                                          row, lane)
                        : 0.0;
      s = dfx::group_sum<L>(s);
      if (active && lane == 0)
      {
        w.y[row] = s;
        dot += s * w.p[row];
      }
    }
    else
    {
      double s0 = 0, s1 = 0, s2 = 0;
      if (active)
        dfx::bsr3_row_partial<double, double, double>(rp, cols, vals, w.p, row, lane, s0, s1, s2);
      s0 = dfx::group_sum<8>(s0);
      s1 = dfx::group_sum<8>(s1);
      s2 = dfx::group_sum<8>(s2);
      if (active && lane == 0)
      {
        double* yr = w.y + 3 * (int64_t)row;
        const double* pr = w.p + 3 * (int64_t)row;
        yr[0] = s0;
        yr[1] = s1;
        yr[2] = s2;
        dot += s0 * pr[0] + s1 * pr[1] + s2 * pr[2];
      }
    }
  }
  if (publish(dot, 0.0, w.part0, nullptr, &w.st->ticket[1], false))
  {
    const double pAp = final_sum(w.part0);
    if (threadIdx.x == 0)
    {
      CgState* st = w.st;
      st->pAp = pAp;
      if (!(pAp > 0.0) || !isfinite(pAp))
      {
        st->status = DFX_ERR_BREAKDOWN;
        st->done = 1;
      }
      else
        st->alpha = st->rz / pAp;
      st->ticket[1] = 0;
      __threadfence();
    }
  }
}

template <bool PRE>
__global__ void __launch_bounds__(kThreads)
    k_cg_update(double* __restrict__ x, const double* __restrict__ dinv, int64_t n, Work w)
{
  if (is_done(w.st))
    return;
  const double alpha = __ldcg(&w.st->alpha);
  double rr = 0.0, rz = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    x[i] += alpha * w.p[i];
    const double r = w.r[i] - alpha * w.y[i];
    w.r[i] = r;
    const double z = PRE ? dinv[i] * r : r;
    rr += r * r;
    rz += r * z;
  }
  if (publish(rr, rz, w.part0, w.part1, &w.st->ticket[2], true))
  {
    const double srr = final_sum(w.part0);
    const double srz = final_sum(w.part1);
    if (threadIdx.x == 0)
    {
      CgState* st = w.st;
      st->rr = srr;
      st->iter += 1;
      st->beta = srz / st->rz;
      st->rz = srz;
      if (srr / st->rr0 < st->rtol2)
        st->done = 1;
      else if (!isfinite(srr))
      {
        st->status = DFX_ERR_BREAKDOWN;
        st->done = 1;
      }
      else if (st->iter >= st->max_iter)
      {
        st->status = DFX_ERR_NOT_CONVERGED;
        st->done = 1;
      }
      st->ticket[2] = 0;
      __threadfence();
    }
  }
}

template <bool PRE>
__global__ void __launch_bounds__(kThreads)
    k_cg_pupdate(const double* __restrict__ dinv, int64_t n, Work w)
{
  if (is_done(w.st))
    return;
  const double beta = __ldcg(&w.st->beta);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const double z = PRE ? dinv[i] * w.r[i] : w.r[i];
    w.p[i] = z + beta * w.p[i];
  }
}

// Enqueue one CG iteration.
void enqueue_iteration(const dfx_csr* A, double* x, const double* dinv, int64_t n, const Work& w,
                       cudaStream_t s)
{
  const int blocks = w.blocks;
  const double* vals = (const double*)A->vals;
  if (A->bs == 1)
  {
    switch (dfx::spmv_lanes(A))
    {
    case 4:
      k_cg_spmv_dot<4, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
      break;
    case 8:
      k_cg_spmv_dot<8, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
      break;
    case 16:
      k_cg_spmv_dot<16, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
      break;
    default:
      k_cg_spmv_dot<32, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
    }
  }
  else
    k_cg_spmv_dot<8, 3><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
  if (dinv)
  {
    k_cg_update<true><<<blocks, kThreads, 0, s>>>(x, dinv, n, w);
    k_cg_pupdate<true><<<blocks, kThreads, 0, s>>>(dinv, n, w);
  }
  else
  {
    k_cg_update<false><<<blocks, kThreads, 0, s>>>(x, dinv, n, w);
    k_cg_pupdate<false><<<blocks, kThreads, 0, s>>>(dinv, n, w);
  }
}

// Graphs of K iterations, cached by the pointers and sizes they bake in.
using GraphKey = std::tuple<const void*, const void*, const void*, const void*, int64_t, int64_t,
                            int, const void*, const void*, const void*, int, int, int>;
std::mutex g_graph_mutex;
std::map<GraphKey, cudaGraphExec_t> g_graphs;

struct PinnedState
{
  CgState* h = nullptr;
  ~PinnedState()
  {
    if (h)
      cudaFreeHost(h);
  }
};
thread_local PinnedState t_pinned;

} // namespace

extern "C" size_t dfx_cg_workspace_bytes(int64_t n) { return work_bytes(n, grid_blocks()); }

extern "C" int dfx_cg_solve(const dfx_csr* A, const double* d_b, double* d_x,
                            const double* d_dinv, double rtol, int32_t max_iters,
                            int32_t graph_iters, void* d_work, size_t wbytes, dfx_cg_info* info,
                            void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->dtype == DFX_F64, "dfx_cg_solve runs in FP64");
  DFX_REQUIRE(A->nrows == A->ncols, "matrix must be square");
  DFX_REQUIRE(d_b && d_x && d_work, "b, x and workspace must be non-NULL");
  DFX_REQUIRE(rtol > 0.0 && max_iters > 0, "rtol and max_iters must be positive");
  const int64_t n = (int64_t)A->nrows * A->bs;
  const int blocks = grid_blocks();
  DFX_REQUIRE(wbytes >= work_bytes(n, blocks), "workspace too small (%zu < %zu)", wbytes,
              work_bytes(n, blocks));
  DFX_REQUIRE(((uintptr_t)d_work & 255) == 0, "workspace must be 256-byte aligned");
  cudaStream_t s = dfx::as_stream(stream);
  const int K = graph_iters > 0 ? graph_iters : 20;
  Work w = carve(d_work, n, blocks);
  DFX_CUDA(cudaMemsetAsync(w.st, 0, sizeof(CgState), s));

  // r0 = b - A x0, z0 = D^{-1} r0, p0 = z0.
  dfx_csr Ay = *A;
  if (int st = dfx::launch_spmv(&Ay, d_x, w.y, 0.0, s))
    return st;
  if (d_dinv)
    k_cg_init<true><<<blocks, kThreads, 0, s>>>(d_b, d_dinv, n, w, rtol * rtol, max_iters);
  else
    k_cg_init<false><<<blocks, kThreads, 0, s>>>(d_b, d_dinv, n, w, rtol * rtol, max_iters);
  DFX_CHECK_LAUNCH();

  cudaGraphExec_t exec = nullptr;
  {
    GraphKey key{A->row_ptr, A->cols, A->vals, d_b, n, A->nnz, A->bs, d_x, d_dinv, d_work, K,
                 blocks, A->dtype};
    std::lock_guard<std::mutex> lk(g_graph_mutex);
    auto it = g_graphs.find(key);
    if (it != g_graphs.end())
      exec = it->second;
    else
    {
      cudaStream_t cs;
      DFX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t graph;
      DFX_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < K; ++k)
        enqueue_iteration(A, d_x, d_dinv, n, w, cs);
      cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      cudaStreamDestroy(cs);
      DFX_CUDA(ce);
      ce = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      DFX_CUDA(ce);
      if (g_graphs.size() >= 16)
      {
        cudaGraphExecDestroy(g_graphs.begin()->second);
        g_graphs.erase(g_graphs.begin());
      }
      g_graphs[key] = exec;
    }
  }
  if (!t_pinned.h)
    DFX_CUDA(cudaMallocHost(&t_pinned.h, sizeof(CgState)));
  CgState* h = t_pinned.h;
  // Every graph replay advances K iterations until the state is done, and
  // the state is done at max_iters at the latest; the bound below only
  // guards against a corrupted state.
  const int64_t max_launches = (int64_t)max_iters / K + 2;
  for (int64_t launch = 0;; ++launch)
  {
    DFX_CUDA(cudaMemcpyAsync(h, w.st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    DFX_CUDA(cudaStreamSynchronize(s));
    if (h->done)
      break;
    if (launch > max_launches)
      return dfx::fail(DFX_ERR_TIMEOUT, "CG state never reported completion");
    DFX_CUDA(cudaGraphLaunch(exec, s));
  }
  if (info)
  {
    info->iterations = h->iter;
    info->status = h->status;
    info->rnorm0_sq = h->rr0;
    info->rnorm_sq = h->rr;
  }
  if (h->status == DFX_ERR_NOT_CONVERGED)
    return dfx::fail(DFX_ERR_NOT_CONVERGED,
                     "Solver exceeded max iterations (%d). Relative residual=%g.", h->iter,
                     h->rr0 > 0 ? h->rr / h->rr0 : 0.0);
  if (h->status == DFX_ERR_BREAKDOWN)
    return dfx::fail(DFX_ERR_BREAKDOWN, "CG breakdown at iteration %d (p.Ap=%g)", h->iter,
                     h->pAp);
  return DFX_OK;
}
