// Batched persistent CG for serving: one launch advances many small,
// independent systems, one CTA per system.
//
// A serving loop holds many small assemble-and-solve requests at once. Each
// alone cannot fill the GPU, and the whole-GPU solver pays three launches
// and a reduction hand-off per iteration. Here one CTA of 1024 threads runs
// the whole Jacobi-PCG of its system inside one launch: SpMV over the
// system's sliced-ELL operator (the matrix of a small system stays in L2),
// vector updates and block reductions, with only __syncthreads between the
// phases -- no grid synchronisation and no spin-waits. A launch runs at most
// `iterations` iterations per system and stores the state, so the host can
// retire converged systems and admit new ones between launches
// (iteration-level continuous batching). The launch is a CUDA graph of the
// active-list upload and the kernel; the grid is fixed at the context's
// capacity and CTAs beyond the active count return at once, so the graph
// never changes.
//
// Modes: 0 = FP64 PCG (FP64 operator and vectors); 1 = mixed precision:
// FP32 operator and vectors with FP64 reliable updates (the residual
// b - A x, its norm and x += d in FP64 with the FP64 operator), the same
// scheme as dfx_ir_solve's DFX_IR_RELIABLE. Each CTA's arithmetic depends
// only on its own system, so results do not depend on the batch mix.
#include "sell.cuh"

#include <vector>

namespace
{
constexpr int kBT = 1024;
constexpr int kWarps = kBT / 32;

struct BatchState
{
  double rz, rr0, rr, rmax2, pAp, beta;
  int32_t iter, done, status, updates, phase, pad;
};

struct BatchDesc
{
  dfx_operator_s op32;
  dfx_operator_s op64;
  const double* b;
  double* x;
  float* r32;
  float* p32;
  float* y32;
  float* d32;
  float* dinv32;
  double* r64;
  double* p64;
  double* y64;
  const double* dinv64;
  double rtol2;
  double delta2;
  int32_t max_iters;
  int32_t mode;
  int32_t n;
  int32_t pad;
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Deterministic block sum of (a, c); every thread gets the totals.
__device__ __forceinline__ void block_sum2(double& a, double& c, double* sh)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  a = dfx::warp_sum(a);
  c = dfx::warp_sum(c);
  if (lane == 0)
  {
    sh[w] = a;
    sh[32 + w] = c;
  }
  __syncthreads();
  if (w == 0)
  {
    double s0 = sh[lane], s1 = sh[32 + lane];
    s0 = dfx::warp_sum(s0);
    s1 = dfx::warp_sum(s1);
    if (lane == 0)
    {
      sh[64] = s0;
      sh[65] = s1;
    }
  }
  __syncthreads();
  a = sh[64];
  c = sh[65];
  __syncthreads();
}

// FP32 partials: warp sums in FP32, the 32 warp sums added in FP64.
__device__ __forceinline__ void block_sum2f(float a, float c, double& oa, double& oc, double* sh)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  a = dfx::warp_sum(a);
  c = dfx::warp_sum(c);
  if (lane == 0)
  {
    sh[w] = (double)a;
    sh[32 + w] = (double)c;
  }
  __syncthreads();
  if (w == 0)
  {
    double s0 = sh[lane], s1 = sh[32 + lane];
    s0 = dfx::warp_sum(s0);
    s1 = dfx::warp_sum(s1);
    if (lane == 0)
    {
      sh[64] = s0;
      sh[65] = s1;
    }
  }
  __syncthreads();
  oa = sh[64];
  oc = sh[65];
  __syncthreads();
}

// Mixed mode: r = b - A64 x in FP64, stored as FP32; returns |r|^2 and r.z
// (z = D^{-1} r) in FP64.
__device__ void rel_residual(const BatchDesc& d, double& rr, double& rz, double* sh)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double a = 0.0, c = 0.0;
  for (int32_t s = w; s < d.op64.nslices; s += kWarps)
  {
    const double ax = dfx::sell_row<double, double, double, false>(d.op64, (const double*)d.op64.vals,
                                                                   d.x, s, lane);
    const int32_t row = 32 * s + lane;
    if (row < d.n)
    {
      const double r = d.b[row] - ax;
      const float r32 = (float)r;
      d.r32[row] = r32;
      a += r * r;
      const double z = d.dinv32 ? (double)(d.dinv32[row] * r32) : (double)r32;
      c += (double)r32 * z;
    }
  }
  block_sum2(a, c, sh);
  rr = a;
  rz = c;
}

__global__ void __launch_bounds__(kBT)
    k_batch_cg(const BatchDesc* __restrict__ descs, BatchState* __restrict__ states,
               const int32_t* __restrict__ active, int32_t iterations)
{
  __shared__ double sh[72];
  const int32_t count = active[0];
  if ((int32_t)blockIdx.x >= count)
    return;
  const int32_t slot = active[1 + blockIdx.x];
  const BatchDesc& d = descs[slot];
  BatchState st = states[slot];
  if (st.done)
    return;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int32_t n = d.n;

  if (d.mode == 1)
  {
    float* r = d.r32;
    float* p = d.p32;
    float* y = d.y32;
    float* x = d.d32;
    const float* dinv = d.dinv32;
    if (st.phase == 0)
    {
      for (int32_t i = tid; i < n; i += kBT)
      {
        x[i] = 0.0f;
        p[i] = 0.0f;
      }
      __syncthreads();
      double rr, rz;
      rel_residual(d, rr, rz, sh);
      st.rr0 = rr;
      st.rr = rr;
      st.rmax2 = rr;
      st.rz = rz;
      st.beta = 0.0;
      st.phase = 1;
      if (rr == 0.0)
      {
        st.done = 1;
        st.status = DFX_OK;
      }
      else
      {
        for (int32_t i = tid; i < n; i += kBT)
          p[i] = dinv ? dinv[i] * r[i] : r[i];
        __syncthreads();
      }
    }
    for (int32_t it = 0; it < iterations && !st.done; ++it)
    {
      // y = A p, p.y
      float dot = 0.0f;
      for (int32_t s = w; s < d.op32.nslices; s += kWarps)
      {
        const float acc = d.op32.compressed
                              ? dfx::sell_row<float, float, float, true>(d.op32,
                                                                         (const float*)d.op32.vals,
                                                                         p, s, lane)
                              : dfx::sell_row<float, float, float, false>(
                                    d.op32, (const float*)d.op32.vals, p, s, lane);
        const int32_t row = 32 * s + lane;
        if (row < n)
        {
          y[row] = acc;
          dot += acc * p[row];
        }
      }
      double pAp, unused;
      block_sum2f(dot, 0.0f, pAp, unused, sh);
      if (!(pAp > 0.0) || !isfinite(pAp))
      {
        st.pAp = pAp;
        st.status = DFX_ERR_BREAKDOWN;
        st.done = 1;
        break;
      }
      const float alpha = (float)(st.rz / pAp);
      float rrp = 0.0f, rzp = 0.0f;
      for (int32_t i = tid; i < n; i += kBT)
      {
        x[i] += alpha * p[i];
        const float rn = r[i] - alpha * y[i];
        r[i] = rn;
        rrp += rn * rn;
        rzp += rn * (dinv ? dinv[i] * rn : rn);
      }
      double rr, rz;
      block_sum2f(rrp, rzp, rr, rz, sh);
      st.iter += 1;
      const bool conv = rr / st.rr0 < d.rtol2;
      if (conv || rr < d.delta2 * st.rmax2 || st.iter >= d.max_iters || !isfinite(rr))
      {
        // Reliable update: fold the correction into x in FP64 and replace
        // the residual by the FP64 one.
        for (int32_t i = tid; i < n; i += kBT)
        {
          d.x[i] += (double)x[i];
          x[i] = 0.0f;
        }
        __syncthreads();
        double rrt, rzt;
        rel_residual(d, rrt, rzt, sh);
        st.updates += 1;
        st.rr = rrt;
        st.rmax2 = rrt;
        if (rrt == 0.0 || rrt / st.rr0 < d.rtol2)
        {
          st.done = 1;
          st.status = DFX_OK;
          break;
        }
        if (!isfinite(rrt))
        {
          st.done = 1;
          st.status = DFX_ERR_BREAKDOWN;
          break;
        }
        if (st.iter >= d.max_iters)
        {
          st.done = 1;
          st.status = DFX_ERR_NOT_CONVERGED;
          break;
        }
        st.beta = rzt / st.rz;
        st.rz = rzt;
      }
      else
      {
        st.rr = rr;
        st.rmax2 = fmax(st.rmax2, rr);
        st.beta = rz / st.rz;
        st.rz = rz;
      }
      const float beta = (float)st.beta;
      for (int32_t i = tid; i < n; i += kBT)
        p[i] = (dinv ? dinv[i] * r[i] : r[i]) + beta * p[i];
      __syncthreads();
    }
  }
  else
  {
    double* r = d.r64;
    double* p = d.p64;
    double* y = d.y64;
    const double* dinv = d.dinv64;
    if (st.phase == 0)
    {
      double a = 0.0, c = 0.0;
      for (int32_t s = w; s < d.op64.nslices; s += kWarps)
      {
        const double ax = dfx::sell_row<double, double, double, false>(
            d.op64, (const double*)d.op64.vals, d.x, s, lane);
        const int32_t row = 32 * s + lane;
        if (row < n)
        {
          const double rv = d.b[row] - ax;
          r[row] = rv;
          const double z = dinv ? dinv[row] * rv : rv;
          p[row] = z;
          a += rv * rv;
          c += rv * z;
        }
      }
      block_sum2(a, c, sh);
      st.rr0 = a;
      st.rr = a;
      st.rz = c;
      st.phase = 1;
      if (a == 0.0)
      {
        st.done = 1;
        st.status = DFX_OK;
      }
    }
    for (int32_t it = 0; it < iterations && !st.done; ++it)
    {
      double dot = 0.0;
      for (int32_t s = w; s < d.op64.nslices; s += kWarps)
      {
        const double acc = dfx::sell_row<double, double, double, false>(
            d.op64, (const double*)d.op64.vals, p, s, lane);
        const int32_t row = 32 * s + lane;
        if (row < n)
        {
          y[row] = acc;
          dot += acc * p[row];
        }
      }
      double unused = 0.0;
      block_sum2(dot, unused, sh);
      if (!(dot > 0.0) || !isfinite(dot))
      {
        st.pAp = dot;
        st.status = DFX_ERR_BREAKDOWN;
        st.done = 1;
        break;
      }
      const double alpha = st.rz / dot;
      double rr = 0.0, rz = 0.0;
      for (int32_t i = tid; i < n; i += kBT)
      {
        d.x[i] += alpha * p[i];
        const double rn = r[i] - alpha * y[i];
        r[i] = rn;
        rr += rn * rn;
        rz += rn * (dinv ? dinv[i] * rn : rn);
      }
      block_sum2(rr, rz, sh);
      st.iter += 1;
      st.rr = rr;
      if (rr / st.rr0 < d.rtol2)
      {
        st.done = 1;
        st.status = DFX_OK;
        break;
      }
      if (!isfinite(rr) || st.iter >= d.max_iters)
      {
        st.done = 1;
        st.status = isfinite(rr) ? DFX_ERR_NOT_CONVERGED : DFX_ERR_BREAKDOWN;
        break;
      }
      const double beta = rz / st.rz;
      st.rz = rz;
      for (int32_t i = tid; i < n; i += kBT)
        p[i] = (dinv ? dinv[i] * r[i] : r[i]) + beta * p[i];
      __syncthreads();
    }
  }
  if (tid == 0)
    states[slot] = st;
}

__global__ void k_to_f32_vec(const double* __restrict__ in, float* __restrict__ out, int32_t n)
{
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = (float)in[i];
}
} // namespace

struct dfx_batch_s
{
  int32_t capacity = 0;
  BatchDesc* d_descs = nullptr;
  BatchState* d_states = nullptr;
  int32_t* d_active = nullptr;
  int32_t* h_active = nullptr;   // pinned
  BatchState* h_states = nullptr; // pinned
  std::vector<char> used;
  cudaGraphExec_t exec = nullptr;
  int32_t graph_iters = -1;
  int device = 0;
};

namespace
{
int capture_step(dfx_batch_s* b, int32_t iterations)
{
  if (b->exec && b->graph_iters == iterations)
    return DFX_OK;
  if (b->exec)
  {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  cudaStream_t cs;
  DFX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t graph;
  cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (ce == cudaSuccess)
  {
    cudaMemcpyAsync(b->d_active, b->h_active, sizeof(int32_t) * (b->capacity + 1),
                    cudaMemcpyHostToDevice, cs);
    k_batch_cg<<<b->capacity, kBT, 0, cs>>>(b->d_descs, b->d_states, b->d_active, iterations);
    ce = cudaStreamEndCapture(cs, &graph);
  }
  cudaStreamDestroy(cs);
  DFX_CUDA(ce);
  ce = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  DFX_CUDA(ce);
  b->graph_iters = iterations;
  return DFX_OK;
}
} // namespace

extern "C" size_t dfx_batch_workspace_bytes(int64_t n, int32_t mode)
{
  if (mode == 1)
    return 5 * align256(sizeof(float) * (size_t)n);
  return 3 * align256(sizeof(double) * (size_t)n);
}

extern "C" int dfx_batch_create(int32_t capacity, dfx_batch* out)
{
  DFX_REQUIRE(out && capacity > 0 && capacity <= 65535, "capacity must be in [1, 65535]");
  auto* b = new dfx_batch_s();
  b->capacity = capacity;
  b->used.assign(capacity, 0);
  cudaGetDevice(&b->device);
  int st = DFX_OK;
  if (cudaMalloc(&b->d_descs, sizeof(BatchDesc) * capacity) != cudaSuccess
      || cudaMalloc(&b->d_states, sizeof(BatchState) * capacity) != cudaSuccess
      || cudaMalloc(&b->d_active, sizeof(int32_t) * (capacity + 1)) != cudaSuccess
      || cudaMallocHost(&b->h_active, sizeof(int32_t) * (capacity + 1)) != cudaSuccess
      || cudaMallocHost(&b->h_states, sizeof(BatchState) * capacity) != cudaSuccess)
    st = dfx::no_memory("batch context");
  if (!st)
  {
    cudaMemset(b->d_states, 0, sizeof(BatchState) * capacity);
    b->h_active[0] = 0;
    *out = b;
    return DFX_OK;
  }
  dfx_batch_destroy(b);
  return st;
}

extern "C" int dfx_batch_destroy(dfx_batch b)
{
  if (!b)
    return DFX_OK;
  if (b->exec)
    cudaGraphExecDestroy(b->exec);
  cudaFree(b->d_descs);
  cudaFree(b->d_states);
  cudaFree(b->d_active);
  cudaFreeHost(b->h_active);
  cudaFreeHost(b->h_states);
  delete b;
  return DFX_OK;
}

extern "C" int dfx_batch_set(dfx_batch b, int32_t slot, const dfx_batch_system* sys, void* stream)
{
  DFX_REQUIRE(b && sys, "arguments must be non-NULL");
  DFX_REQUIRE(slot >= 0 && slot < b->capacity, "slot %d out of range", slot);
  DFX_REQUIRE(sys->mode == 0 || sys->mode == 1, "mode must be 0 (FP64) or 1 (mixed)");
  DFX_REQUIRE(sys->op64 && sys->op64->dtype == DFX_F64, "an FP64 operator is required");
  DFX_REQUIRE(sys->mode == 0 || (sys->op32 && sys->op32->dtype == DFX_F32),
              "mixed mode needs an FP32 operator");
  DFX_REQUIRE(sys->mode == 0 || (sys->op32->n == sys->op64->n
                                 && sys->op32->nslices == sys->op64->nslices
                                 && sys->op32->sigma == sys->op64->sigma),
              "FP32 and FP64 operators must share one structure");
  DFX_REQUIRE(sys->op64->vals && (sys->mode == 0 || sys->op32->vals),
              "operator values were released (dfx_operator_release_values): use a share");
  DFX_REQUIRE(sys->b && sys->x && sys->work, "b, x and work must be non-NULL");
  DFX_REQUIRE(((uintptr_t)sys->work & 255) == 0, "workspace must be 256-byte aligned");
  DFX_REQUIRE(sys->rtol > 0.0 && sys->max_iters > 0, "rtol and max_iters must be positive");
  const int32_t n = sys->op64->n;
  cudaStream_t s = dfx::as_stream(stream);
  BatchDesc d{};
  d.op64 = *sys->op64;
  if (sys->op32)
    d.op32 = *sys->op32;
  d.b = sys->b;
  d.x = sys->x;
  d.n = n;
  d.mode = sys->mode;
  d.rtol2 = sys->rtol * sys->rtol;
  d.delta2 = sys->delta > 0.0 ? sys->delta * sys->delta : 1e-4;
  d.max_iters = sys->max_iters;
  char* w = (char*)sys->work;
  if (sys->mode == 1)
  {
    const size_t vb = align256(sizeof(float) * (size_t)n);
    d.r32 = (float*)w;
    d.p32 = (float*)(w + vb);
    d.y32 = (float*)(w + 2 * vb);
    d.d32 = (float*)(w + 3 * vb);
    d.dinv32 = sys->dinv ? (float*)(w + 4 * vb) : nullptr;
    if (sys->dinv && n > 0)
      k_to_f32_vec<<<(n + 255) / 256, 256, 0, s>>>(sys->dinv, d.dinv32, n);
  }
  else
  {
    const size_t vb = align256(sizeof(double) * (size_t)n);
    d.r64 = (double*)w;
    d.p64 = (double*)(w + vb);
    d.y64 = (double*)(w + 2 * vb);
    d.dinv64 = sys->dinv;
  }
  DFX_CHECK_LAUNCH();
  DFX_CUDA(cudaMemcpyAsync(b->d_descs + slot, &d, sizeof(BatchDesc), cudaMemcpyHostToDevice, s));
  DFX_CUDA(cudaMemsetAsync(b->d_states + slot, 0, sizeof(BatchState), s));
  // The descriptor lives on this stack frame until the copy has run.
  DFX_CUDA(cudaStreamSynchronize(s));
  b->h_states[slot] = BatchState{};
  b->used[slot] = 1;
  return DFX_OK;
}

extern "C" int dfx_batch_clear(dfx_batch b, int32_t slot)
{
  DFX_REQUIRE(b && slot >= 0 && slot < b->capacity, "slot out of range");
  b->used[slot] = 0;
  return DFX_OK;
}

extern "C" int dfx_batch_step(dfx_batch b, int32_t iterations, int32_t* num_active, void* stream)
{
  DFX_REQUIRE(b && iterations > 0, "iterations must be positive");
  cudaStream_t s = dfx::as_stream(stream);
  // The active list is read by the graph from pinned memory: wait until the
  // previous step has consumed it.
  DFX_CUDA(cudaStreamSynchronize(s));
  int32_t cnt = 0;
  for (int32_t i = 0; i < b->capacity; ++i)
    if (b->used[i] && !b->h_states[i].done)
      b->h_active[1 + cnt++] = i;
  b->h_active[0] = cnt;
  if (num_active)
    *num_active = cnt;
  if (cnt == 0)
    return DFX_OK;
  if (int st = capture_step(b, iterations))
    return st;
  DFX_CUDA(cudaGraphLaunch(b->exec, s));
  DFX_CUDA(cudaMemcpyAsync(b->h_states, b->d_states, sizeof(BatchState) * b->capacity,
                           cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}

extern "C" int dfx_batch_info(dfx_batch b, int32_t slot, dfx_cg_info* info, int32_t* done,
                              int32_t* replacements)
{
  DFX_REQUIRE(b && slot >= 0 && slot < b->capacity, "slot out of range");
  const BatchState& st = b->h_states[slot];
  if (done)
    *done = st.done;
  if (replacements)
    *replacements = st.updates;
  if (info)
  {
    info->iterations = st.iter;
    info->status = st.status;
    info->rnorm0_sq = st.rr0;
    info->rnorm_sq = st.rr;
    info->kernel_launches = 0;
  }
  return DFX_OK;
}

namespace
{
__global__ void k_perm(const double* __restrict__ in, double* __restrict__ out,
                       const int32_t* __restrict__ perm, int32_t n, int to_operator)
{
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  if (to_operator)
    out[i] = in[perm[i]];
  else
    out[perm[i]] = in[i];
}
} // namespace

extern "C" int dfx_operator_permute(dfx_operator op, const double* d_in, double* d_out,
                                    int32_t to_operator, void* stream)
{
  DFX_REQUIRE(op && d_in && d_out, "arguments must be non-NULL");
  DFX_REQUIRE(d_in != d_out, "in-place permutation is not supported");
  const int32_t n = op->n;
  if (n == 0)
    return DFX_OK;
  k_perm<<<(n + 255) / 256, 256, 0, dfx::as_stream(stream)>>>(d_in, d_out, op->perm, n,
                                                               to_operator ? 1 : 0);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}
