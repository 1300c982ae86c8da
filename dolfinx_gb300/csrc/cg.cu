// Conjugate gradients on the device: FP64 Jacobi-PCG (CSR or sliced-ELL
// operator) and FP32-inner / FP64-outer iterative refinement.
//
// One PCG iteration (the demo's loop, cpp/demo/poisson_matrix_free/
// main.cpp:84-132, with z = D^{-1} r) is three kernels:
//   1. y = A p and p.y          (SpMV with a fused dot product)
//   2. x += a p, r -= a y, r.r and r.z with z = D^{-1} r; convergence test
//   3. p = z + b p
// Reductions are two-stage and deterministic: per-block partial sums in
// FP64, then the last block to finish (atomic ticket) sums the partials in
// index order and updates the scalar state in device memory. The FP32
// sliced-ELL SpMV is the exception: its blocks are short (one slice per
// warp), and the ticket at the end of each one held the block's slot for
// the length of a device-wide atomic (86 us against 74 us without it at P2
// 64^3); its warps store their p.y partials in fixed slots. By default one
// cooperative kernel then does the rest of the iteration (k_update_fused:
// the p.y sum, the x/r update and the p update, with grid-wide barriers),
// so the FP32 iteration is two kernels; otherwise a small fourth kernel
// reduces the partials. The FP64 SpMV, twice as long, keeps the fused
// ticket: a fourth launch cost it more. Scalars never
// leave the device; every kernel returns at once when the state says done,
// so a CUDA graph of K iterations is replayed until the host reads done.
//
// Mixed precision: the refinement loop keeps the residual r = b - A x, its
// norm and the update x += d in FP64 with the FP64 operator; the inner
// solve A d = r runs the same PCG with FP32 values, FP32 vectors and the
// 16-bit-column operator. Its dot products sum FP32 products per warp
// (a lane owns ~16 entries) and reduce the warp sums in FP64.
#include "la_kernels.cuh"
#include "q4.cuh"
#include "sell.cuh"

#include <atomic>
#include <map>
#include <type_traits>
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
  double rmax2;  // reliable updates: largest |r|^2 since the last update
  double delta2; // reliable updates: update when |r|^2 < delta2 * rmax2
  int32_t iter;
  int32_t max_iter;
  int32_t done;
  int32_t status;
  int32_t updates; // reliable updates performed
  int32_t since;   // iterations since the last reliable update
  int32_t forced;  // reliable updates: replace at least every `forced` iterations (0: never)
  unsigned int ticket[4];
  // Grid-wide barrier of the fused FP32 update (arrivals, generation).
  unsigned int bar_count;
  unsigned int bar_gen;
};

// Reliable updates with an assembled FP64 operator: a residual replacement
// at least this often, so that a stalled FP32 recurrence is caught by the
// stagnation test. A matrix-free FP64 action costs far more than an FP32
// iteration, so the Q4 solve replaces less often.
constexpr int32_t kForcedUpdate = 200;
constexpr int32_t kForcedUpdateQ4 = 1000;

// Internal pause codes of the reliable-update solve (never returned).
constexpr int32_t kPauseUpdate = 100;    // residual dropped by delta: replace it
constexpr int32_t kPauseConverged = 101; // iterated residual converged: verify in FP64

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Sliced-ELL kernels: 128 threads, one slice (32 rows) per warp; the
// hardware block scheduler balances slices of different lengths.
constexpr int kSellThreads = 128;
int sell_blocks(int64_t n) { return (int)std::max<int64_t>(1, (((n + 31) / 32) + 3) / 4); }

// Grid of the grid-stride kernels without SpMV (init, correction, CSR).
int stride_grid() { return 8 * dfx::num_sms(); }

// Elementwise kernels: 256 threads x 4 entries per block and round, all
// loads of a round issued before any use.
constexpr int kElemThreads = 256;
constexpr int kElemPerThread = 4;
int elem_grid(int64_t n)
{
  const int64_t per = (int64_t)kElemThreads * kElemPerThread;
  return (int)std::max<int64_t>(1, (n + per - 1) / per);
}

// Largest grid of any CG kernel for n unknowns (each block publishes one
// partial sum).
int max_blocks(int64_t n) { return std::max({sell_blocks(n), elem_grid(n), stride_grid()}); }

// Warps per reduction group of the two-level reduction.
constexpr int kGroup = 64;
int groups_of(int units) { return (units + kGroup - 1) / kGroup; }

// Carves typed arrays out of a workspace (p == nullptr: only counts).
struct Carver
{
  char* p;
  size_t used = 0;
  template <typename T>
  T* take(size_t count)
  {
    T* r = p ? (T*)(p + used) : nullptr;
    used += align256(sizeof(T) * count);
    return r;
  }
};

// Buffers of the deterministic two-level reduction: per-block partial sums,
// per-group sums, per-group tickets.
struct Red
{
  double* part0;
  double* part1;
  double* gpart0;
  double* gpart1;
  unsigned int* gticket;
};

Red carve_red(Carver& c, int blocks)
{
  Red r;
  r.part0 = c.take<double>(blocks);
  r.part1 = c.take<double>(blocks);
  r.gpart0 = c.take<double>(groups_of(blocks));
  r.gpart1 = c.take<double>(groups_of(blocks));
  r.gticket = c.take<unsigned int>(groups_of(blocks));
  return r;
}

template <typename T>
struct Work
{
  CgState* st;
  Red red;
  T* r;
  T* p;
  T* y;
  int blocks;
  // FP64 solves on a split operator (DFX_F32X2): p's FP32 words, (hi, lo)
  // side by side per row, written wherever p is, read by the SpMV.
  float* ph = nullptr;
  // Per-warp p.y partials of the sliced-ELL SpMV (one slot per warp of its
  // grid), summed by k_pap_reduce.
  double* wpart = nullptr;
  // Per-block partial sums of the fused FP32 update: p.y, r.r, r.z (three
  // rows of `blocks`).
  double* bpart = nullptr;
};

// p[i] and, when the solve keeps them, its FP32 words.
template <typename T>
__device__ __forceinline__ void store_p(const Work<T>& w, int64_t n, int64_t i, T v)
{
  w.p[i] = v;
  if constexpr (sizeof(T) == 8)
    if (w.ph)
    {
      float2 hl;
      dfx::split_f64(v, hl.x, hl.y);
      reinterpret_cast<float2*>(w.ph)[i] = hl;
    }
}

template <typename T>
Work<T> carve_work(Carver& c, int64_t n)
{
  Work<T> w;
  w.blocks = max_blocks(n);
  w.st = c.take<CgState>(1);
  w.red = carve_red(c, w.blocks);
  w.r = c.take<T>(n);
  w.p = c.take<T>(n);
  w.y = c.take<T>(n);
  w.wpart = c.take<double>((size_t)sell_blocks(n) * (kSellThreads / 32));
  w.bpart = c.take<double>(3 * (size_t)w.blocks);
  return w;
}

// Zero the state and the group tickets of a work area.
int reset_work(CgState* st, const Red& red, int blocks, cudaStream_t s)
{
  DFX_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), s));
  DFX_CUDA(cudaMemsetAsync(red.gticket, 0, sizeof(unsigned int) * groups_of(blocks), s));
  return DFX_OK;
}

// Deterministic reduction without block barriers. Each warp reduces its
// lanes and drops the result in shared memory; the last warp of the block
// to arrive (shared-memory ticket) sums the block's warps in index order and
// publishes one partial per block, in slot blockIdx.x. The last block of
// each group of kGroup blocks sums the group in index order; the last group
// to finish sums the group totals in index order and returns true in all
// lanes of that one warp. Kernels call block_reduce_init() once at entry.
struct WarpFinal
{
  bool last;
  double s0, s1; // valid in the last warp (all lanes)
};

// Per-block staging of partial sums: one value per lane (FP64 kernels) or
// per warp (FP32 kernels), for up to 8 warps.
struct BlockScratch
{
  double p0[256];
  double p1[256];
  unsigned int count;
};

__device__ __forceinline__ BlockScratch& block_scratch()
{
  __shared__ BlockScratch b;
  return b;
}

__device__ __forceinline__ void block_reduce_init()
{
  if (threadIdx.x == 0)
    block_scratch().count = 0;
  __syncthreads();
}

// T = float: each warp sums its lanes in FP32 (its lanes hold FP32 partials
// of at most a few entries each) and lane 0 stages the warp sum; the last
// warp adds the block's warp sums in FP64 in one lane. T = double: every lane
// stages its FP64 partial; the last warp adds them in lane-then-warp order.
// Both keep FP64 instructions -- 1/58 of the FP32 rate here -- off the
// per-warp path.
template <typename T>
__device__ __forceinline__ WarpFinal publish(T v0, T v1, const Red& red, unsigned int* ticket,
                                             bool two)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned nw = blockDim.x >> 5;
  BlockScratch& bs = block_scratch();
  WarpFinal out{false, 0.0, 0.0};
  if constexpr (sizeof(T) == 4)
  {
    v0 = dfx::warp_sum(v0);
    if (two)
      v1 = dfx::warp_sum(v1);
    if (lane == 0)
    {
      bs.p0[warp] = (double)v0;
      if (two)
        bs.p1[warp] = (double)v1;
    }
  }
  else
  {
    bs.p0[threadIdx.x] = (double)v0;
    if (two)
      bs.p1[threadIdx.x] = (double)v1;
  }
  __syncwarp();
  int flag = 0;
  if (lane == 0)
  {
    __threadfence_block();
    flag = atomicAdd(&bs.count, 1u) == nw - 1;
  }
  if (!__shfl_sync(0xffffffffu, flag, 0))
    return out;
  // Last warp of the block: the block partial, in a fixed order.
  __threadfence_block();
  volatile double* q0 = bs.p0;
  volatile double* q1 = bs.p1;
  double b0 = 0.0, b1 = 0.0;
  if constexpr (sizeof(T) == 4)
  {
    if (lane == 0)
      for (unsigned w = 0; w < nw; ++w)
      {
        b0 += q0[w];
        if (two)
          b1 += q1[w];
      }
  }
  else
  {
    for (unsigned w = 0; w < nw; ++w)
    {
      b0 += q0[32 * w + lane];
      if (two)
        b1 += q1[32 * w + lane];
    }
    b0 = dfx::warp_sum(b0);
    if (two)
      b1 = dfx::warp_sum(b1);
  }
  const unsigned unit = blockIdx.x, nunits = gridDim.x;
  const unsigned g = unit / kGroup;
  const unsigned ng = (nunits + kGroup - 1) / kGroup;
  const unsigned gsize = min((unsigned)kGroup, nunits - g * kGroup);
  if (lane == 0)
  {
    red.part0[unit] = b0;
    if (two)
      red.part1[unit] = b1;
    __threadfence();
    flag = atomicAdd(&red.gticket[g], 1u) == gsize - 1;
  }
  if (!__shfl_sync(0xffffffffu, flag, 0))
    return out;
  double s0 = 0.0, s1 = 0.0;
  for (unsigned i = lane; i < gsize; i += 32)
  {
    s0 += __ldcg(red.part0 + g * kGroup + i);
    if (two)
      s1 += __ldcg(red.part1 + g * kGroup + i);
  }
  s0 = dfx::warp_sum(s0);
  if (two)
    s1 = dfx::warp_sum(s1);
  if (lane == 0)
  {
    red.gpart0[g] = s0;
    if (two)
      red.gpart1[g] = s1;
    red.gticket[g] = 0;
    __threadfence();
    flag = atomicAdd(ticket, 1u) == ng - 1;
  }
  if (!__shfl_sync(0xffffffffu, flag, 0))
    return out;
  s0 = 0.0;
  s1 = 0.0;
  for (unsigned i = lane; i < ng; i += 32)
  {
    s0 += __ldcg(red.gpart0 + i);
    if (two)
      s1 += __ldcg(red.gpart1 + i);
  }
  out.last = true;
  out.s0 = dfx::warp_sum(s0);
  out.s1 = two ? dfx::warp_sum(s1) : 0.0;
  return out;
}


// Scalars of the state are produced by earlier kernels of the stream and
// only read by this one (the one warp that updates them does so after its
// last read), so they go through the read-only path: one L2 fetch per SM
// instead of one request per warp to a single L2 line.
__device__ __forceinline__ bool is_done(const CgState* st) { return __ldg(&st->done) != 0; }

// r = rhs - Ax (Ax == nullptr: x0 = 0 and x is zeroed), z = D^{-1} r,
// p = z; state initialised. rhs may alias w.r.
template <typename T, bool PRE>
__global__ void __launch_bounds__(kThreads)
    k_init(const T* rhs, const T* __restrict__ Ax, T* __restrict__ x, const T* __restrict__ dinv,
           int64_t n, Work<T> w, double rtol2, int max_iter)
{
  block_reduce_init();

  T rr = 0, rz = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const T r = Ax ? rhs[i] - Ax[i] : rhs[i];
    const T z = PRE ? dinv[i] * r : r;
    if (!Ax)
      x[i] = T(0);
    w.r[i] = r;
    store_p<T>(w, n, i, z);
    rr += r * r;
    rz += r * z;
  }
  const WarpFinal f = publish<T>(rr, rz, w.red, &w.st->ticket[0], true);
  if (f.last)
  {
    const double srr = f.s0, srz = f.s1;
    if ((threadIdx.x & 31) == 0)
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

// Last warp of an SpMV-dot kernel: alpha = rz / p.Ap.
__device__ __forceinline__ void finish_pap(const WarpFinal& f, CgState* st)
{
  if (!f.last)
    return;
  const double pAp = f.s0;
  if ((threadIdx.x & 31) == 0)
  {
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

// y = A p, p.y -- CSR operator (L lanes per row, or 8 lanes per 3x3 block row).
template <int L, int BS>
__global__ void __launch_bounds__(kThreads)
    k_spmv_dot_csr(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ cols,
                   const double* __restrict__ vals, Work<double> w)
{
  block_reduce_init();

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
  finish_pap(publish<double>(dot, 0.0, w.red, &w.st->ticket[1], false), w.st);
}

// The warp's p.y partial into its fixed slot (FP32 kernels: the lanes'
// FP32 partials summed in FP32, as one FP64 value).
template <typename T>
__device__ __forceinline__ void store_warp_partial(T dot, const Work<T>& w)
{
  const T sum = dfx::warp_sum(dot);
  if ((threadIdx.x & 31) == 0)
    w.wpart[(blockIdx.x * blockDim.x + threadIdx.x) >> 5] = (double)sum;
}

// y = A p, p.y -- sliced-ELL operator, one row per lane, warp per slice.
// The SpMV is bound by the latency of its loads, so its register budget
// (resident warps) is set by measurement at P2 64^3: the FP64 kernel at 12
// blocks per SM (40 registers; 64 when left to ptxas, 295 -> 246 ms per
// plain FP64 step), the FP32 kernel at 10 (48 registers: 150.0 -> 147.1 ms
// per mixed step against 12 blocks). Chunks of 8 keep 8 blocks so that they
// do not spill.
template <typename T, int CH>
constexpr int kSellMinBlocks = CH >= 8 ? 8 : (sizeof(T) == 4 ? 10 : 12);

template <typename V, typename T, bool COMP, int CH = 4>
__global__ void __launch_bounds__(kSellThreads, kSellMinBlocks<T, CH>)
    k_spmv_dot_sell(const dfx_operator_s op, Work<T> w)
{
  constexpr bool kSplitReduce = sizeof(T) == 4; // p.y summed by k_pap_reduce
  if constexpr (!kSplitReduce)
    block_reduce_init();

  if (is_done(w.st))
    return;
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  T dot = 0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const T acc = dfx::sell_row<V, T, T, COMP, CH>(op, (const V*)op.vals, w.p, s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
    {
      w.y[row] = acc;
      dot += acc * w.p[row];
    }
  }
  if constexpr (kSplitReduce)
    store_warp_partial<T>(dot, w);
  else
    finish_pap(publish<T>(dot, T(0), w.red, &w.st->ticket[1], false), w.st);
}

// p.Ap from the sliced-ELL SpMV's per-warp partials, in one short latency
// chain: each thread adds a fixed set of kPapPer slots (loads issued
// together, added in slot order), warps and then the block reduce by
// shuffles in a fixed pattern, and the last block to arrive (ticket) adds
// the block partials in block order and sets alpha (finish_pap). At most
// 32 blocks, so that one warp finishes.
constexpr int kPapThreads = 256;
constexpr int kPapPer = 16;
constexpr int kPapMaxBlocks = 32;
int pap_blocks(int64_t n)
{
  const int64_t parts = (int64_t)sell_blocks(n) * (kSellThreads / 32);
  const int64_t per_block = (int64_t)kPapThreads * kPapPer;
  return (int)std::max<int64_t>(1, (parts + per_block - 1) / per_block);
}

template <typename T>
__global__ void __launch_bounds__(kPapThreads) k_pap_reduce(Work<T> w, int nparts, int per_thread)
{
  __shared__ double wsum[kPapThreads / 32];
  __shared__ int last;
  if (is_done(w.st))
    return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // slots blockIdx.x * (per_thread * kPapThreads) + k * kPapThreads + threadIdx.x
  const int64_t base = (int64_t)blockIdx.x * per_thread * kPapThreads + threadIdx.x;
  double part[kPapPer];
#pragma unroll
  for (int k = 0; k < kPapPer; ++k)
  {
    const int64_t i = base + (int64_t)k * kPapThreads;
    part[k] = (k < per_thread && i < nparts) ? __ldcg(w.wpart + i) : 0.0;
  }
  double v = 0.0;
#pragma unroll
  for (int k = 0; k < kPapPer; ++k)
    v += part[k];
  for (int k = kPapPer; k < per_thread; ++k)
  {
    const int64_t i = base + (int64_t)k * kPapThreads;
    if (i < nparts)
      v += __ldcg(w.wpart + i);
  }
  v = dfx::warp_sum(v);
  if (lane == 0)
    wsum[warp] = v;
  __syncthreads();
  if (warp != 0)
    return;
  v = lane < kPapThreads / 32 ? wsum[lane] : 0.0;
  v = dfx::warp_sum(v);
  if (lane == 0)
  {
    w.red.part0[blockIdx.x] = v;
    __threadfence();
    last = atomicAdd(&w.st->ticket[1], 1u) == gridDim.x - 1;
  }
  __syncwarp();
  if (!last)
    return;
  __threadfence();
  double s = lane < (int)gridDim.x ? __ldcg(w.red.part0 + lane) : 0.0;
  s = dfx::warp_sum(s);
  finish_pap(WarpFinal{true, s, 0.0}, w.st);
}

// y = A p, p.y -- split operator (DFX_F32X2): FP32-pipe products of the
// FP32 words of the values and of p, FP64 y and dot.
template <bool COMP>
__global__ void __launch_bounds__(kSellThreads, 12)
    k_spmv_dot_sell_split(const dfx_operator_s op, Work<double> w)
{
  block_reduce_init();

  if (is_done(w.st))
    return;
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  const float* vh = (const float*)op.vals;
  double dot = 0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const double acc = dfx::sell_row_split<COMP>(op, vh, vh + op.nslots,
                                                 reinterpret_cast<const float2*>(w.ph), s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
    {
      w.y[row] = acc;
      dot += acc * w.p[row];
    }
  }
  finish_pap(publish<double>(dot, 0.0, w.red, &w.st->ticket[1], false), w.st);
}

// y = A p, p.y -- 3x3-block operator (bs 3, lane = block row): FP64
// values, or split values on the FP32 words of p; SL block slots per round.
template <bool SPLIT, int SL>
__global__ void __launch_bounds__(kSellThreads, dfx::kBsellMinBlocks<SL>)
    k_spmv_dot_bsell3(const dfx_operator_s op, Work<double> w)
{
  block_reduce_init();

  if (is_done(w.st))
    return;
  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  double dot = 0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    double acc[3];
    if constexpr (SPLIT)
      dfx::bsell_row3_split<SL>(op, (const float2*)op.vals,
                                reinterpret_cast<const float2*>(w.ph), s, lane, acc);
    else
      dfx::bsell_row3<SL>(op, (const double*)op.vals, w.p, s, lane, acc);
    const int32_t row = 3 * (32 * s + lane);
    if (row < op.n)
    {
#pragma unroll
      for (int r = 0; r < 3; ++r)
      {
        w.y[row + r] = acc[r];
        dot += acc[r] * w.p[row + r];
      }
    }
  }
  finish_pap(publish<double>(dot, 0.0, w.red, &w.st->ticket[1], false), w.st);
}

// 16-byte vectors of the elementwise kernels.
template <typename T>
struct Vec16;
template <>
struct Vec16<float>
{
  using type = float4;
  static constexpr int N = 4;
};
template <>
struct Vec16<double>
{
  using type = double2;
  static constexpr int N = 2;
};

// State update of the last warp of k_update: convergence test, beta, and
// (reliable updates) the decision to pause for a residual replacement.
template <bool RELIABLE>
__device__ __forceinline__ void update_finish(const WarpFinal& f, CgState* st)
{
  if (!f.last || (threadIdx.x & 31) != 0)
    return;
  const double srr = f.s0, srz = f.s1;
  st->rr = srr;
  st->iter += 1;
  bool pause = false;
  if (srr / st->rr0 < st->rtol2)
  {
    st->done = 1;
    if (RELIABLE)
    {
      st->status = kPauseConverged;
      pause = true;
    }
  }
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
  else if (RELIABLE
           && (srr < st->delta2 * st->rmax2 || (st->forced > 0 && st->since + 1 >= st->forced)))
  {
    st->status = kPauseUpdate;
    st->done = 1;
    pause = true;
  }
  if (RELIABLE)
    st->since = pause ? 0 : st->since + 1;
  // A pause keeps rz = r_old.z_old: beta is formed after the residual
  // has been replaced.
  if (!pause)
  {
    st->beta = srz / st->rz;
    st->rz = srz;
    if (RELIABLE)
      st->rmax2 = fmax(st->rmax2, srr);
  }
  st->ticket[2] = 0;
  __threadfence();
}

// x += alpha p, r -= alpha y, r.r and r.z (z = D^{-1} r). vec: every array
// is 16-byte aligned, and a thread moves 16 bytes per array and round over
// a grid of one resident wave; otherwise 4 scalar entries per thread and
// round.
template <typename T, bool PRE, bool RELIABLE>
__global__ void __launch_bounds__(kElemThreads)
    k_update(T* __restrict__ x, const T* __restrict__ dinv, int64_t n, Work<T> w, bool vec)
{
  block_reduce_init();

  if (is_done(w.st))
    return;
  const T alpha = (T)__ldg(&w.st->alpha);
  T rr = 0, rz = 0;
  if (vec)
  {
    using V = typename Vec16<T>::type;
    constexpr int L = Vec16<T>::N;
    const int64_t nvec = n / L;
    const int64_t stride = (int64_t)gridDim.x * kElemThreads;
    for (int64_t v = (int64_t)blockIdx.x * kElemThreads + threadIdx.x; v < nvec; v += stride)
    {
      V pv = reinterpret_cast<const V*>(w.p)[v];
      V yv = reinterpret_cast<const V*>(w.y)[v];
      V rv = reinterpret_cast<const V*>(w.r)[v];
      V xv = reinterpret_cast<const V*>(x)[v];
      V dv = pv;
      if (PRE)
        dv = reinterpret_cast<const V*>(dinv)[v];
      const T* pe = reinterpret_cast<const T*>(&pv);
      const T* ye = reinterpret_cast<const T*>(&yv);
      const T* de = reinterpret_cast<const T*>(&dv);
      T* re = reinterpret_cast<T*>(&rv);
      T* xe = reinterpret_cast<T*>(&xv);
#pragma unroll
      for (int e = 0; e < L; ++e)
      {
        xe[e] = xe[e] + alpha * pe[e];
        const T rn = re[e] - alpha * ye[e];
        re[e] = rn;
        rr += rn * rn;
        rz += rn * (PRE ? de[e] * rn : rn);
      }
      reinterpret_cast<V*>(x)[v] = xv;
      reinterpret_cast<V*>(w.r)[v] = rv;
    }
    if (blockIdx.x == 0)
      for (int64_t i = nvec * L + threadIdx.x; i < n; i += kElemThreads)
      {
        x[i] = x[i] + alpha * w.p[i];
        const T rn = w.r[i] - alpha * w.y[i];
        w.r[i] = rn;
        rr += rn * rn;
        rz += rn * (PRE ? dinv[i] * rn : rn);
      }
  }
  else
  {
    constexpr int E = kElemPerThread;
    const int64_t stride = (int64_t)gridDim.x * kElemThreads * E;
    for (int64_t base = (int64_t)blockIdx.x * kElemThreads * E + threadIdx.x; base < n;
         base += stride)
    {
      T p[E], y[E], r[E], xv[E], d[E];
#pragma unroll
      for (int e = 0; e < E; ++e)
      {
        const int64_t i = base + (int64_t)e * kElemThreads;
        const bool ok = i < n;
        p[e] = ok ? w.p[i] : T(0);
        y[e] = ok ? w.y[i] : T(0);
        r[e] = ok ? w.r[i] : T(0);
        xv[e] = ok ? x[i] : T(0);
        d[e] = (ok && PRE) ? dinv[i] : T(1);
      }
#pragma unroll
      for (int e = 0; e < E; ++e)
      {
        const int64_t i = base + (int64_t)e * kElemThreads;
        if (i >= n)
          continue;
        x[i] = xv[e] + alpha * p[e];
        const T rn = r[e] - alpha * y[e];
        w.r[i] = rn;
        rr += rn * rn;
        rz += rn * (PRE ? d[e] * rn : rn);
      }
    }
  }
  update_finish<RELIABLE>(publish<T>(rr, rz, w.red, &w.st->ticket[2], true), w.st);
}

// p = z + beta p with z = D^{-1} r (vec: as in k_update).
template <typename T, bool PRE>
__global__ void __launch_bounds__(kElemThreads)
    k_pupdate(const T* __restrict__ dinv, int64_t n, Work<T> w, bool vec)
{
  if (is_done(w.st))
    return;
  const T beta = (T)__ldg(&w.st->beta);
  if (vec)
  {
    using V = typename Vec16<T>::type;
    constexpr int L = Vec16<T>::N;
    const int64_t nvec = n / L;
    const int64_t stride = (int64_t)gridDim.x * kElemThreads;
    for (int64_t v = (int64_t)blockIdx.x * kElemThreads + threadIdx.x; v < nvec; v += stride)
    {
      V pv = reinterpret_cast<const V*>(w.p)[v];
      V rv = reinterpret_cast<const V*>(w.r)[v];
      V dv = rv;
      if (PRE)
        dv = reinterpret_cast<const V*>(dinv)[v];
      T* pe = reinterpret_cast<T*>(&pv);
      const T* re = reinterpret_cast<const T*>(&rv);
      const T* de = reinterpret_cast<const T*>(&dv);
#pragma unroll
      for (int e = 0; e < L; ++e)
        pe[e] = (PRE ? de[e] * re[e] : re[e]) + beta * pe[e];
      reinterpret_cast<V*>(w.p)[v] = pv;
      if constexpr (sizeof(T) == 8)
        if (w.ph)
        {
          // rows 2v and 2v+1: (hi, lo, hi, lo) in one 16-byte store
          float4 hl;
          dfx::split_f64(pe[0], hl.x, hl.y);
          dfx::split_f64(pe[1], hl.z, hl.w);
          reinterpret_cast<float4*>(w.ph)[v] = hl;
        }
    }
    if (blockIdx.x == 0)
      for (int64_t i = nvec * L + threadIdx.x; i < n; i += kElemThreads)
        store_p<T>(w, n, i, (PRE ? dinv[i] * w.r[i] : w.r[i]) + beta * w.p[i]);
    return;
  }
  constexpr int E = kElemPerThread;
  const int64_t stride = (int64_t)gridDim.x * kElemThreads * E;
  for (int64_t base = (int64_t)blockIdx.x * kElemThreads * E + threadIdx.x; base < n;
       base += stride)
  {
    T p[E], r[E], d[E];
#pragma unroll
    for (int e = 0; e < E; ++e)
    {
      const int64_t i = base + (int64_t)e * kElemThreads;
      const bool ok = i < n;
      p[e] = ok ? w.p[i] : T(0);
      r[e] = ok ? w.r[i] : T(0);
      d[e] = (ok && PRE) ? dinv[i] : T(1);
    }
#pragma unroll
    for (int e = 0; e < E; ++e)
    {
      const int64_t i = base + (int64_t)e * kElemThreads;
      if (i < n)
        store_p<T>(w, n, i, (PRE ? d[e] * r[e] : r[e]) + beta * p[e]);
    }
  }
}


// ---------------------------------------------------------------- fused update
// The FP32 sliced-ELL inner iteration in two kernels: the SpMV (per-warp
// p.y partials) and one cooperative launch that does what k_pap_reduce,
// k_update and k_pupdate do, with two grid-wide barriers in place of two
// kernel boundaries:
//   A. p.y: block b adds a fixed range of the SpMV's warp partials;
//      barrier; every block adds the block partials in index order (the
//      same order in every block, so all blocks hold the same alpha);
//   B. x += alpha p, r -= alpha y, z = D^{-1} r; r.r and r.z per block;
//      barrier; every block adds them in index order and takes the same
//      convergence / replacement decision as update_finish;
//   C. p = z + beta p from the values phase B kept in registers (entries
//      past EV float4 per thread are read again).
// Block 0 alone writes the state, after the last barrier. The launch is
// cooperative (all blocks resident), so the barrier waits end; each wait
// is bounded all the same and gives up with DFX_ERR_TIMEOUT.
constexpr int kBarrierPolls = 1 << 22;    // polls of one barrier wait (x 64 ns sleeps)

// Grid-wide barrier; false in every thread of the block when its wait gave
// up. All threads of every block call it.
__device__ __forceinline__ bool grid_barrier(CgState* st, unsigned int arrivals)
{
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    ok = 1;
    volatile unsigned int* gen = &st->bar_gen;
    const unsigned int g = *gen;
    // Arrival: an acquire-release add publishes this block's partials and,
    // for the last block, acquires everyone's (release sequence of the count).
    unsigned int old;
    asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], 1;"
                 : "=r"(old)
                 : "l"(&st->bar_count)
                 : "memory");
    if (old == arrivals - 1)
    {
      st->bar_count = 0;
      __threadfence();
      *gen = g + 1;
    }
    else
    {
      int i = 0;
      while (*gen == g)
      {
        if (++i > kBarrierPolls)
        {
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// Self-test of the barrier's bounded wait: the blocks wait for one arrival
// more than the grid has, so every wait runs out; each block records that
// it gave up (st->updates counts them) and the status DFX_ERR_TIMEOUT.
__global__ void k_barrier_selftest(CgState* st)
{
  if (!grid_barrier(st, gridDim.x + 1) && threadIdx.x == 0)
  {
    atomicAdd(&st->updates, 1);
    st->status = DFX_ERR_TIMEOUT;
  }
}

// Block sum in a fixed order (lane, then warp); thread 0 holds the result.
__device__ __forceinline__ double fused_block_sum(double v, double* sh)
{
  v = dfx::warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0)
  {
    t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    t = dfx::warp_sum(t);
  }
  __syncthreads();
  return t;
}

// Block sum of FP32 partials: each warp adds its lanes in FP32, the warp
// sums are added in FP64 in warp order; thread 0 holds the result.
__device__ __forceinline__ double fused_block_sum_f32(float v, double* sh)
{
  v = dfx::warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    sh[warp] = (double)v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0)
  {
    t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    t = dfx::warp_sum(t);
  }
  __syncthreads();
  return t;
}

// Sums of two rows of block partials (gridDim.x values each) in index
// order, the same in every block; every thread receives both. Blocks of at
// most 512 threads (16 warps: sh holds 32 values).
__device__ __forceinline__ void fused_grid_total2(const double* p0, const double* p1,
                                                  double* sh, double* bc, double& t0,
                                                  double& t1)
{
  double v0 = 0.0, v1 = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
  {
    v0 += __ldcg(p0 + i);
    v1 += __ldcg(p1 + i);
  }
  v0 = dfx::warp_sum(v0);
  v1 = dfx::warp_sum(v1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
  {
    sh[warp] = v0;
    sh[16 + warp] = v1;
  }
  __syncthreads();
  if (warp == 0)
  {
    const int nw = (int)(blockDim.x >> 5);
    double a = lane < nw ? sh[lane] : 0.0, b = lane < nw ? sh[16 + lane] : 0.0;
    a = dfx::warp_sum(a);
    b = dfx::warp_sum(b);
    if (lane == 0)
    {
      bc[0] = a;
      bc[1] = b;
    }
  }
  __syncthreads();
  t0 = bc[0];
  t1 = bc[1];
  __syncthreads();
}

// Sum of row k of the block partials (gridDim.x values) in index order,
// the same in every block; every thread receives it.
__device__ __forceinline__ double fused_grid_total(const double* part, double* sh, double* bc)
{
  double v = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
    v += __ldcg(part + i);
  v = fused_block_sum(v, sh);
  if (threadIdx.x == 0)
    *bc = v;
  __syncthreads();
  const double t = *bc;
  __syncthreads();
  return t;
}

template <bool PRE, bool RELIABLE, int kFusedThreads, int kFusedEV>
__global__ void __launch_bounds__(kFusedThreads, 1)
    k_update_fused(float* __restrict__ x, const float* __restrict__ dinv, int64_t n,
                   Work<float> w, int nparts)
{
  __shared__ double sh[32];
  __shared__ double bc;
  __shared__ double bc2[2];
  CgState* st = w.st;
  if (is_done(st))
    return;
  // State read before the first barrier: block 0 writes it only after the
  // last one.
  const double rz_old = __ldg(&st->rz), rr0 = __ldg(&st->rr0), rtol2 = __ldg(&st->rtol2);
  const double delta2 = __ldg(&st->delta2), rmax2 = __ldg(&st->rmax2);
  const int iter = __ldg(&st->iter), max_iter = __ldg(&st->max_iter);
  const int forced = __ldg(&st->forced), since = __ldg(&st->since);
  const unsigned G = gridDim.x;

  // The entries this thread keeps: p, y, r and D^{-1} are loaded before
  // phase A, so that their loads are in flight across the p.y reduction
  // and the first barrier.
  const int64_t nvec = n / 4;
  const int64_t T = (int64_t)G * kFusedThreads;
  const int64_t t0 = (int64_t)blockIdx.x * kFusedThreads + threadIdx.x;
  const float4* P4 = reinterpret_cast<const float4*>(w.p);
  const float4* Y4 = reinterpret_cast<const float4*>(w.y);
  float4* R4 = reinterpret_cast<float4*>(w.r);
  float4* X4 = reinterpret_cast<float4*>(x);
  const float4* D4 = reinterpret_cast<const float4*>(dinv);
  float4 kp[kFusedEV], ky[kFusedEV], kr[kFusedEV], kd[kFusedEV];
#pragma unroll
  for (int k = 0; k < kFusedEV; ++k)
  {
    const int64_t v = t0 + k * T;
    if (v < nvec)
    {
      kp[k] = P4[v];
      ky[k] = Y4[v];
      kr[k] = R4[v];
      kd[k] = PRE ? D4[v] : kp[k];
    }
  }

  // A. p.y
  {
    const int64_t per = ((int64_t)nparts + G - 1) / G;
    const int64_t b0 = (int64_t)blockIdx.x * per;
    const int64_t b1 = b0 + per < nparts ? b0 + per : nparts;
    double a = 0.0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kFusedThreads)
      a += __ldcg(w.wpart + i);
    a = fused_block_sum(a, sh);
    if (threadIdx.x == 0)
      w.bpart[blockIdx.x] = a;
  }
  if (!grid_barrier(st, gridDim.x))
  {
    if (threadIdx.x == 0)
    {
      st->status = DFX_ERR_TIMEOUT;
      st->done = 1;
    }
    return;
  }
  const double pAp = fused_grid_total(w.bpart, sh, &bc);
  if (!(pAp > 0.0) || !isfinite(pAp))
  {
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
      st->pAp = pAp;
      st->status = DFX_ERR_BREAKDOWN;
      st->done = 1;
    }
    return;
  }
  const float alpha = (float)(rz_old / pAp);

  // B. x, r; z = D^{-1} r
  float rr = 0.f, rz = 0.f;
  auto step = [&](float4& pv, float4 yv, float4& rv, float4& xv, float4 dv, float4& zv)
  {
    xv.x += alpha * pv.x;
    xv.y += alpha * pv.y;
    xv.z += alpha * pv.z;
    xv.w += alpha * pv.w;
    rv.x -= alpha * yv.x;
    rv.y -= alpha * yv.y;
    rv.z -= alpha * yv.z;
    rv.w -= alpha * yv.w;
    zv = PRE ? make_float4(dv.x * rv.x, dv.y * rv.y, dv.z * rv.z, dv.w * rv.w) : rv;
    rr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
    rz += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
  };
  {
    float4 kx[kFusedEV];
#pragma unroll
    for (int k = 0; k < kFusedEV; ++k)
    {
      const int64_t v = t0 + k * T;
      if (v < nvec)
        kx[k] = X4[v];
    }
#pragma unroll
    for (int k = 0; k < kFusedEV; ++k)
    {
      const int64_t v = t0 + k * T;
      if (v < nvec)
      {
        float4 z;
        step(kp[k], ky[k], kr[k], kx[k], kd[k], z);
        X4[v] = kx[k];
        R4[v] = kr[k];
      }
    }
  }
  // Entries past the kept ones, kRem float4 per round with every load of
  // the round issued first.
  constexpr int kRem = 2;
  for (int64_t v0 = t0 + kFusedEV * T; v0 < nvec; v0 += kRem * T)
  {
    float4 pv[kRem], yv[kRem], rv[kRem], xv[kRem], dv[kRem];
#pragma unroll
    for (int k = 0; k < kRem; ++k)
    {
      const int64_t v = v0 + k * T;
      if (v < nvec)
      {
        pv[k] = P4[v];
        yv[k] = Y4[v];
        rv[k] = R4[v];
        xv[k] = X4[v];
        dv[k] = PRE ? D4[v] : pv[k];
      }
    }
#pragma unroll
    for (int k = 0; k < kRem; ++k)
    {
      const int64_t v = v0 + k * T;
      if (v < nvec)
      {
        float4 z;
        step(pv[k], yv[k], rv[k], xv[k], dv[k], z);
        X4[v] = xv[k];
        R4[v] = rv[k];
      }
    }
  }
  if (blockIdx.x == 0)
    for (int64_t i = nvec * 4 + threadIdx.x; i < n; i += kFusedThreads)
    {
      x[i] += alpha * w.p[i];
      const float rn = w.r[i] - alpha * w.y[i];
      w.r[i] = rn;
      rr += rn * rn;
      rz += rn * (PRE ? dinv[i] * rn : rn);
    }
  {
    const double brr = fused_block_sum_f32(rr, sh);
    const double brz = fused_block_sum_f32(rz, sh);
    if (threadIdx.x == 0)
    {
      w.bpart[G + blockIdx.x] = brr;
      w.bpart[2 * G + blockIdx.x] = brz;
    }
  }
  if (!grid_barrier(st, gridDim.x))
  {
    if (threadIdx.x == 0)
    {
      st->status = DFX_ERR_TIMEOUT;
      st->done = 1;
    }
    return;
  }
  double srr, srz;
  fused_grid_total2(w.bpart + G, w.bpart + 2 * G, sh, bc2, srr, srz);

  // The decision of update_finish, taken alike in every block.
  bool done = false, pause = false;
  int status = DFX_OK;
  if (srr / rr0 < rtol2)
  {
    done = true;
    if (RELIABLE)
    {
      status = kPauseConverged;
      pause = true;
    }
  }
  else if (!isfinite(srr))
  {
    status = DFX_ERR_BREAKDOWN;
    done = true;
  }
  else if (iter + 1 >= max_iter)
  {
    status = DFX_ERR_NOT_CONVERGED;
    done = true;
  }
  else if (RELIABLE && (srr < delta2 * rmax2 || (forced > 0 && since + 1 >= forced)))
  {
    status = kPauseUpdate;
    done = true;
    pause = true;
  }
  const double beta = srz / rz_old;
  if (blockIdx.x == 0 && threadIdx.x == 0)
  {
    st->pAp = pAp;
    st->alpha = rz_old / pAp;
    st->rr = srr;
    st->iter = iter + 1;
    if (done)
    {
      st->status = status;
      st->done = 1;
    }
    if (RELIABLE)
      st->since = pause ? 0 : since + 1;
    if (!pause)
    {
      st->beta = beta;
      st->rz = srz;
      if (RELIABLE)
        st->rmax2 = fmax(rmax2, srr);
    }
  }
  if (done)
    return;

  // C. p = z + beta p
  const float fb = (float)beta;
  float4* PW = reinterpret_cast<float4*>(w.p);
#pragma unroll
  for (int k = 0; k < kFusedEV; ++k)
  {
    const int64_t v = t0 + k * T;
    if (v < nvec)
    {
      const float4 r = kr[k], d = kd[k], q = kp[k];
      const float4 z = PRE ? make_float4(d.x * r.x, d.y * r.y, d.z * r.z, d.w * r.w) : r;
      PW[v] = make_float4(z.x + fb * q.x, z.y + fb * q.y, z.z + fb * q.z, z.w + fb * q.w);
    }
  }
  for (int64_t v0 = t0 + kFusedEV * T; v0 < nvec; v0 += kRem * T)
  {
    float4 q[kRem], r[kRem], d[kRem];
#pragma unroll
    for (int k = 0; k < kRem; ++k)
    {
      const int64_t v = v0 + k * T;
      if (v < nvec)
      {
        q[k] = P4[v];
        r[k] = R4[v];
        d[k] = PRE ? D4[v] : r[k];
      }
    }
#pragma unroll
    for (int k = 0; k < kRem; ++k)
    {
      const int64_t v = v0 + k * T;
      if (v < nvec)
      {
        const float4 z = PRE ? make_float4(d[k].x * r[k].x, d[k].y * r[k].y, d[k].z * r[k].z,
                                           d[k].w * r[k].w)
                             : r[k];
        PW[v] = make_float4(z.x + fb * q[k].x, z.y + fb * q[k].y, z.z + fb * q[k].z,
                            z.w + fb * q[k].w);
      }
    }
  }
  if (blockIdx.x == 0)
    for (int64_t i = nvec * 4 + threadIdx.x; i < n; i += kFusedThreads)
      w.p[i] = (PRE ? dinv[i] * w.r[i] : w.r[i]) + fb * w.p[i];
}

// Outer residual of the refinement: r = b - A x in FP64 with the FP64
// operator, |r|^2 in FP64, r handed to the inner solve in FP32. The outer
// state counts residual evaluations; the first one sets |r0|^2.
__global__ void __launch_bounds__(kSellThreads)
    k_ir_residual(const dfx_operator_s op, const double* __restrict__ b,
                  const double* __restrict__ x, float* __restrict__ r32, CgState* st,
                  Red red, double rtol2, int max_outer)
{
  block_reduce_init();

  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  double rr = 0.0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const double ax = dfx::sell_row<double, double, double, false>(op, (const double*)op.vals, x,
                                                                   s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
    {
      const double r = b[row] - ax;
      r32[row] = (float)r;
      rr += r * r;
    }
  }
  const WarpFinal f = publish<double>(rr, 0.0, red, &st->ticket[3], false);
  if (f.last)
  {
    const double srr = f.s0;
    if ((threadIdx.x & 31) == 0)
    {
      if (st->iter == 0)
      {
        st->rr0 = srr;
        st->status = DFX_OK;
      }
      st->rr = srr;
      st->iter += 1;
      if (srr == 0.0 || srr / st->rr0 < rtol2)
        st->done = 1;
      else if (!isfinite(srr))
      {
        st->status = DFX_ERR_BREAKDOWN;
        st->done = 1;
      }
      else if (st->iter > max_outer)
      {
        st->status = DFX_ERR_NOT_CONVERGED;
        st->done = 1;
      }
      st->ticket[3] = 0;
      __threadfence();
    }
  }
}

// x += d in FP64; d is reset to zero for the next correction.
__global__ void k_ir_correct(double* __restrict__ x, float* __restrict__ d, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    x[i] += (double)d[i];
    d[i] = 0.0f;
  }
}

// ---- Flexible CG outer loop (DFX_IR_FLEXIBLE). The outer iteration is
// FP64 CG in which the preconditioned residual z is the inner FP32 PCG's
// correction d ~ A^{-1} r; since that correction depends nonlinearly on r,
// each new direction is A-orthogonalised against the previous one
// explicitly (truncated flexible CG, one stored direction):
//   p = z - (z.q_old / p_old.q_old) p_old,  q = A p,
//   alpha = p.r / p.q,  x += alpha p,  r -= alpha q.
// All outer vectors, products and scalars are FP64; the outer stopping test
// is the FP64 recursive residual, confirmed by the true residual b - A x.

// r = b - A x in FP64 (kept in r64 and handed to the inner solve in FP32),
// |r|^2; `first` sets |r0|^2. done = 1 when |r|^2 / |r0|^2 < rtol^2.
__global__ void __launch_bounds__(kSellThreads)
    k_fcg_residual(const dfx_operator_s op, const double* __restrict__ b,
                   const double* __restrict__ x, double* __restrict__ r64,
                   float* __restrict__ r32, CgState* st, Red red, int first)
{
  block_reduce_init();

  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  double rr = 0.0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const double ax = dfx::sell_row<double, double, double, false>(op, (const double*)op.vals, x,
                                                                   s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
    {
      const double r = b[row] - ax;
      r64[row] = r;
      r32[row] = (float)r;
      rr += r * r;
    }
  }
  const WarpFinal f = publish<double>(rr, 0.0, red, &st->ticket[3], false);
  if (f.last && lane == 0)
  {
    const double srr = f.s0;
    if (first)
      st->rr0 = srr;
    st->rr = srr;
    st->status = DFX_OK;
    st->done = 0;
    if (srr == 0.0 || srr / st->rr0 < st->rtol2)
      st->done = 1;
    else if (!isfinite(srr))
    {
      st->status = DFX_ERR_BREAKDOWN;
      st->done = 1;
    }
    st->ticket[3] = 0;
    __threadfence();
  }
}

// gamma = z.q_old with z = d; beta = gamma / (p_old.q_old).
__global__ void __launch_bounds__(kElemThreads)
    k_fcg_gamma(const float* __restrict__ d, const double* __restrict__ q, int64_t n, CgState* st,
                Red red)
{
  block_reduce_init();

  double g = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    g += (double)d[i] * q[i];
  const WarpFinal f = publish<double>(g, 0.0, red, &st->ticket[0], false);
  if (f.last && (threadIdx.x & 31) == 0)
  {
    st->beta = f.s0 / st->pAp;
    st->ticket[0] = 0;
    __threadfence();
  }
}

// p = d - beta p_old (first direction: p = d).
__global__ void k_fcg_direction(const float* __restrict__ d, double* __restrict__ p, int64_t n,
                                const CgState* st, int first)
{
  const double beta = first ? 0.0 : __ldg(&st->beta);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = first ? (double)d[i] : (double)d[i] - beta * p[i];
}

// q = A p with the FP64 operator, p.q and p.r; alpha = p.r / p.q.
__global__ void __launch_bounds__(kSellThreads)
    k_fcg_spmv(const dfx_operator_s op, const double* __restrict__ p, double* __restrict__ q,
               const double* __restrict__ r, CgState* st, Red red)
{
  block_reduce_init();

  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  double pq = 0.0, pr = 0.0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const double ap = dfx::sell_row<double, double, double, false>(op, (const double*)op.vals, p,
                                                                   s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
    {
      q[row] = ap;
      const double pv = p[row];
      pq += pv * ap;
      pr += pv * r[row];
    }
  }
  const WarpFinal f = publish<double>(pq, pr, red, &st->ticket[1], true);
  if (f.last && lane == 0)
  {
    st->pAp = f.s0;
    if (!(f.s0 > 0.0) || !isfinite(f.s0) || !isfinite(f.s1))
    {
      st->alpha = 0.0;
      st->status = DFX_ERR_BREAKDOWN;
      st->done = 1;
    }
    else
      st->alpha = f.s1 / f.s0;
    st->ticket[1] = 0;
    __threadfence();
  }
}

// x += alpha p, r -= alpha q, |r|^2, r handed to the inner solve in FP32;
// convergence test on the recursive FP64 residual.
__global__ void __launch_bounds__(kElemThreads)
    k_fcg_update(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                 const double* __restrict__ q, float* __restrict__ r32, int64_t n, CgState* st,
                 Red red)
{
  block_reduce_init();

  if (is_done(st))
    return;
  const double alpha = __ldg(&st->alpha);
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    x[i] += alpha * p[i];
    const double rn = r[i] - alpha * q[i];
    r[i] = rn;
    r32[i] = (float)rn;
    rr += rn * rn;
  }
  const WarpFinal f = publish<double>(rr, 0.0, red, &st->ticket[2], false);
  if (f.last && (threadIdx.x & 31) == 0)
  {
    const double srr = f.s0;
    st->rr = srr;
    st->iter += 1;
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

// Last warp of a residual replacement: the replaced |r|^2 and r.z decide
// whether the solve has converged, and give beta.
__device__ __forceinline__ void rel_finish(const WarpFinal& f, CgState* st)
{
  if (f.last)
  {
    const double srr = f.s0, srz = f.s1;
    if ((threadIdx.x & 31) == 0)
    {
      const bool first = st->iter == 0 && st->updates == 0;
      if (first)
        st->rr0 = srr;
      st->rr = srr;
      st->rmax2 = srr;
      st->updates += first ? 0 : 1;
      if (srr == 0.0 || srr / st->rr0 < st->rtol2)
      {
        st->status = DFX_OK;
        st->done = 1;
      }
      else if (!isfinite(srr))
      {
        st->status = DFX_ERR_BREAKDOWN;
        st->done = 1;
      }
      else
      {
        st->beta = first ? 0.0 : srz / st->rz;
        st->rz = srz;
        st->status = DFX_OK;
        st->done = 0;
      }
      st->ticket[3] = 0;
      __threadfence();
    }
  }
}

// Reliable update (residual replacement): r = b - A x in FP64 with the FP64
// operator; the FP32 iterated residual is replaced by it, |r|^2 and r.z are
// formed in FP64, and beta = (r.z)_new / (r.z)_old keeps the search
// direction. The first call (iter == 0) initialises |r0|^2 and sets beta = 0
// (p is zero then, so the following p = z + beta p gives p = z).
template <bool PRE>
__global__ void __launch_bounds__(kSellThreads)
    k_rel_residual(const dfx_operator_s op, const double* __restrict__ b,
                   const double* __restrict__ x, const float* __restrict__ dinv32, Work<float> w)
{
  block_reduce_init();

  const int lane = threadIdx.x & 31;
  const dfx::SliceRange sr = dfx::block_slices(op.nslices);
  double rr = 0.0, rz = 0.0;
  for (int32_t s = sr.begin; s < sr.end; s += sr.step)
  {
    const double ax = dfx::sell_row<double, double, double, false>(op, (const double*)op.vals, x,
                                                                   s, lane);
    const int32_t row = 32 * s + lane;
    if (row < op.n)
    {
      const double r = b[row] - ax;
      const float r32 = (float)r;
      w.r[row] = r32;
      rr += r * r;
      const double z = PRE ? (double)(dinv32[row] * r32) : (double)r32;
      rz += (double)r32 * z;
    }
  }
  rel_finish(publish<double>(rr, rz, w.red, &w.st->ticket[3], true), w.st);
}

// Residual replacement of the matrix-free solve: r = b - ax with ax = A x
// from the FP64 action, otherwise as k_rel_residual.
template <bool PRE>
__global__ void __launch_bounds__(kElemThreads)
    k_rel_residual_vec(const double* __restrict__ b, const double* __restrict__ ax,
                       const float* __restrict__ dinv32, int64_t n, Work<float> w)
{
  block_reduce_init();

  double rr = 0.0, rz = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const double r = b[i] - ax[i];
    const float r32 = (float)r;
    w.r[i] = r32;
    rr += r * r;
    const double z = PRE ? (double)(dinv32[i] * r32) : (double)r32;
    rz += (double)r32 * z;
  }
  rel_finish(publish<double>(rr, rz, w.red, &w.st->ticket[3], true), w.st);
}

// p.y and alpha, for an operator applied by a separate kernel (matrix-free).
template <typename T>
__global__ void __launch_bounds__(kElemThreads) k_dot_pap(int64_t n, Work<T> w)
{
  block_reduce_init();

  if (is_done(w.st))
    return;
  constexpr int E = kElemPerThread;
  const int64_t stride = (int64_t)gridDim.x * kElemThreads * E;
  T dot = 0;
  for (int64_t base = (int64_t)blockIdx.x * kElemThreads * E + threadIdx.x; base < n;
       base += stride)
  {
    T p[E], y[E];
#pragma unroll
    for (int e = 0; e < E; ++e)
    {
      const int64_t i = base + (int64_t)e * kElemThreads;
      p[e] = i < n ? w.p[i] : T(0);
      y[e] = i < n ? w.y[i] : T(0);
    }
#pragma unroll
    for (int e = 0; e < E; ++e)
      dot += p[e] * y[e];
  }
  finish_pap(publish<T>(dot, T(0), w.red, &w.st->ticket[1], false), w.st);
}

template <typename TI, typename TO>
__global__ void k_gather(const TI* __restrict__ in, TO* __restrict__ out,
                         const int32_t* __restrict__ perm, int32_t n)
{
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[i] = (TO)in[perm[i]];
}

__global__ void k_split_words(const double* __restrict__ x, float* __restrict__ out, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    dfx::split_f64(x[i], out[2 * i], out[2 * i + 1]);
}

__global__ void k_scatter(const double* __restrict__ in, double* __restrict__ out,
                          const int32_t* __restrict__ perm, int32_t n)
{
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    out[perm[i]] = in[i];
}

// ------------------------------------------------------------ enqueueing
enum OpKind
{
  kCsr = 0,
  kSell = 1,
  kQ4 = 2
};

struct OpRef
{
  OpKind kind;
  const dfx_csr* A;          // kCsr
  const dfx_operator_s* op;  // kSell
  const dfx_q4_mesh* q4;     // kQ4 (matrix-free action)
  int q4_tc = 0;             // kQ4, FP32: the tensor-core action
};

template <typename T>
void enqueue_spmv_dot(const OpRef& o, const Work<T>& w, cudaStream_t s);

template <typename T>
void enqueue_pap_reduce(int64_t n, const Work<T>& w, cudaStream_t s)
{
  const int nparts = sell_blocks(n) * (kSellThreads / 32);
  int blocks = pap_blocks(n);
  int per_thread = kPapPer;
  if (blocks > kPapMaxBlocks)
  {
    // very large systems: more slots per thread, at most 32 blocks
    blocks = kPapMaxBlocks;
    per_thread = (int)((nparts + (int64_t)blocks * kPapThreads - 1) / ((int64_t)blocks * kPapThreads));
  }
  k_pap_reduce<T><<<blocks, kPapThreads, 0, s>>>(w, nparts, per_thread);
}

// Kernels of one PCG iteration: the FP32 sliced-ELL operator adds the p.Ap
// reduction kernel to the three.
constexpr int kFusedIterKernels = 3;
constexpr int kF32SellIterKernels = 4;

template <>
void enqueue_spmv_dot<double>(const OpRef& o, const Work<double>& w, cudaStream_t s)
{
  const int blocks = stride_grid();
  if (o.kind == kSell)
  {
    if (o.op->bs == 3)
    {
      const unsigned g = (unsigned)dfx::sell_grid(o.op->nslices);
      auto launch = [&](auto split, auto sl)
      {
        k_spmv_dot_bsell3<decltype(split)::value, decltype(sl)::value>
            <<<g, kSellThreads, 0, s>>>(*o.op, w);
      };
      auto by_chunk = [&](auto split)
      {
        if (o.op->chunk == 2)
          launch(split, std::integral_constant<int, 1>{});
        else if (o.op->chunk == 8)
          launch(split, std::integral_constant<int, 4>{});
        else
          launch(split, std::integral_constant<int, 2>{});
      };
      if (o.op->dtype == DFX_F32X2)
        by_chunk(std::true_type{});
      else
        by_chunk(std::false_type{});
    }
    else if (o.op->dtype == DFX_F32X2)
    {
      if (o.op->compressed)
        k_spmv_dot_sell_split<true><<<sell_blocks(o.op->n), kSellThreads, 0, s>>>(*o.op, w);
      else
        k_spmv_dot_sell_split<false><<<sell_blocks(o.op->n), kSellThreads, 0, s>>>(*o.op, w);
    }
    else
      k_spmv_dot_sell<double, double, false><<<sell_blocks(o.op->n), kSellThreads, 0, s>>>(
          *o.op, w);
    return;
  }
  const dfx_csr* A = o.A;
  const double* vals = (const double*)A->vals;
  if (A->bs == 3)
  {
    k_spmv_dot_csr<8, 3><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
    return;
  }
  switch (dfx::spmv_lanes(A))
  {
  case 4:
    k_spmv_dot_csr<4, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
    break;
  case 8:
    k_spmv_dot_csr<8, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
    break;
  case 16:
    k_spmv_dot_csr<16, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
    break;
  default:
    k_spmv_dot_csr<32, 1><<<blocks, kThreads, 0, s>>>(A->nrows, A->row_ptr, A->cols, vals, w);
  }
}

// The FP32 sliced-ELL SpMV with per-warp p.y partials (no reduction).
void enqueue_spmv_f32(const OpRef& o, const Work<float>& w, cudaStream_t s);

template <>
void enqueue_spmv_dot<float>(const OpRef& o, const Work<float>& w, cudaStream_t s)
{
  enqueue_spmv_f32(o, w, s);
  enqueue_pap_reduce<float>(o.op->n, w, s);
}

void enqueue_spmv_f32(const OpRef& o, const Work<float>& w, cudaStream_t s)
{
  const unsigned g = (unsigned)sell_blocks(o.op->n);
  auto launch = [&](auto comp, auto ch)
  {
    k_spmv_dot_sell<float, float, decltype(comp)::value, decltype(ch)::value>
        <<<g, kSellThreads, 0, s>>>(*o.op, w);
  };
  using T_ = std::true_type;
  using F_ = std::false_type;
  const int ch = o.op->chunk;
  if (o.op->compressed)
  {
    if (ch == 2)
      launch(T_{}, std::integral_constant<int, 2>{});
    else if (ch == 8)
      launch(T_{}, std::integral_constant<int, 8>{});
    else
      launch(T_{}, std::integral_constant<int, 4>{});
  }
  else
  {
    if (ch == 2)
      launch(F_{}, std::integral_constant<int, 2>{});
    else if (ch == 8)
      launch(F_{}, std::integral_constant<int, 8>{});
    else
      launch(F_{}, std::integral_constant<int, 4>{});
  }
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

// Vectorised elementwise launch: 16-byte loads when every array allows it,
// over one wave of resident blocks (at most 8 per SM with 256 threads, so
// within max_blocks); the scalar path otherwise.
template <typename T, typename Kern>
int elementwise_grid(Kern kernel, int64_t n, bool vec)
{
  if (!vec)
    return elem_grid(n);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kElemThreads, 0)
          != cudaSuccess
      || per_sm < 1)
    per_sm = 1;
  const int64_t need = std::max<int64_t>(
      1, (n / Vec16<T>::N + kElemThreads - 1) / kElemThreads);
  return (int)std::min<int64_t>(need, (int64_t)std::min(per_sm, 8) * dfx::num_sms());
}

template <typename T>
bool vector_ok(const T* x, const T* dinv, const Work<T>& w)
{
  return aligned16(x) && (!dinv || aligned16(dinv)) && aligned16(w.p) && aligned16(w.r)
         && aligned16(w.y);
}

template <typename T>
void enqueue_pupdate(const T* dinv, int64_t n, const Work<T>& w, cudaStream_t s)
{
  const bool vec = vector_ok<T>(w.p, dinv, w);
  if (dinv)
    k_pupdate<T, true><<<elementwise_grid<T>(k_pupdate<T, true>, n, vec), kElemThreads, 0, s>>>(
        dinv, n, w, vec);
  else
    k_pupdate<T, false><<<elementwise_grid<T>(k_pupdate<T, false>, n, vec), kElemThreads, 0,
                          s>>>(dinv, n, w, vec);
}

template <typename T, bool PRE, bool RELIABLE>
void launch_update(T* x, const T* dinv, int64_t n, const Work<T>& w, bool vec, cudaStream_t s)
{
  const int g = elementwise_grid<T>(k_update<T, PRE, RELIABLE>, n, vec);
  k_update<T, PRE, RELIABLE><<<g, kElemThreads, 0, s>>>(x, dinv, n, w, vec);
}

// The fused FP32 update (k_update_fused) in place of k_pap_reduce, k_update
// and k_pupdate: on unless the calling host thread switched it off, and off
// for good in this process if a graph with its cooperative launch could not
// be built. Per host thread, because the cooperative kernel holds the
// registers of every SM while it runs: whole-GPU solves that run
// concurrently from several threads and streams (the serving workers) would
// take turns on the GPU. Measured on the serving sample: 33.1 solves/s
// fused against 38.3 unfused.
thread_local int t_fused_update = 1;
std::atomic<int> g_fused_broken{0};

bool fused_update_on() { return t_fused_update != 0 && g_fused_broken.load() == 0; }

template <bool PRE, bool RELIABLE, int kFusedThreads, int kFusedEV>
void launch_fused_as(float* x, const float* dinv, int64_t n, const Work<float>& w, cudaStream_t s)
{
  auto kern = k_update_fused<PRE, RELIABLE, kFusedThreads, kFusedEV>;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFusedThreads, 0)
          != cudaSuccess
      || per_sm < 1)
    per_sm = 1;
  const int64_t nvec = n / 4;
  const int64_t need = std::max<int64_t>(
      1, (nvec + (int64_t)kFusedEV * kFusedThreads - 1) / ((int64_t)kFusedEV * kFusedThreads));
  const int64_t cap = std::min<int64_t>((int64_t)dfx::num_sms(), w.blocks);
  const unsigned g = (unsigned)std::min(need, cap);
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(g);
  cfg.blockDim = dim3(kFusedThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, x, dinv, n, w, sell_blocks(n) * (kSellThreads / 32));
}

// One 512-thread block per SM, four float4 per thread kept in registers
// between phases B and C. Measured at P2 64^3 (mixed step): 143.6 ms
// against 147.2 ms for the four-kernel iteration; 256 threads at two or
// three blocks per SM measured 146.2 and 151.4 ms (more arrivals at each
// barrier), 1024 threads with two float4 per thread 154.8 ms.
template <bool PRE, bool RELIABLE>
void launch_fused(float* x, const float* dinv, int64_t n, const Work<float>& w, cudaStream_t s)
{
  launch_fused_as<PRE, RELIABLE, 512, 4>(x, dinv, n, w, s);
}

// Kernels of one FP32 sliced-ELL iteration.
int f32_sell_iter_kernels() { return fused_update_on() ? 2 : kF32SellIterKernels; }

template <typename T>
void enqueue_iteration(const OpRef& o, T* x, const T* dinv, int64_t n, const Work<T>& w,
                       bool reliable, cudaStream_t s)
{
  if constexpr (sizeof(T) == 4)
    if (o.kind == kSell && fused_update_on() && vector_ok<T>(x, dinv, w))
    {
      enqueue_spmv_f32(o, w, s);
      if (dinv)
      {
        if (reliable)
          launch_fused<true, true>(x, dinv, n, w, s);
        else
          launch_fused<true, false>(x, dinv, n, w, s);
      }
      else
      {
        if (reliable)
          launch_fused<false, true>(x, dinv, n, w, s);
        else
          launch_fused<false, false>(x, dinv, n, w, s);
      }
      return;
    }
  if (o.kind == kQ4)
  {
    // The colour kernels return at once when the state is done.
    if constexpr (sizeof(T) == 4)
    {
      if (o.q4_tc)
        dfx::q4_apply_tc(*o.q4, w.p, w.y, s, &w.st->done);
      else
        dfx::q4_apply<T>(*o.q4, w.p, w.y, s, &w.st->done);
    }
    else
      dfx::q4_apply<T>(*o.q4, w.p, w.y, s, &w.st->done);
    k_dot_pap<T><<<elem_grid(n), kElemThreads, 0, s>>>(n, w);
  }
  else
    enqueue_spmv_dot<T>(o, w, s);
  const bool vec = vector_ok<T>(x, dinv, w);
  if (dinv)
  {
    if (reliable)
      launch_update<T, true, true>(x, dinv, n, w, vec, s);
    else
      launch_update<T, true, false>(x, dinv, n, w, vec, s);
  }
  else
  {
    if (reliable)
      launch_update<T, false, true>(x, dinv, n, w, vec, s);
    else
      launch_update<T, false, false>(x, dinv, n, w, vec, s);
  }
  enqueue_pupdate<T>(dinv, n, w, s);
}

template <typename T>
void enqueue_init(const T* rhs, const T* Ax, T* x, const T* dinv, int64_t n, const Work<T>& w,
                  double rtol, int max_iters, cudaStream_t s)
{
  if (dinv)
    k_init<T, true><<<stride_grid(), kThreads, 0, s>>>(rhs, Ax, x, dinv, n, w, rtol * rtol,
                                                       max_iters);
  else
    k_init<T, false><<<stride_grid(), kThreads, 0, s>>>(rhs, Ax, x, dinv, n, w, rtol * rtol,
                                                        max_iters);
}

// Graphs of K iterations, cached by everything they bake in.
using GraphKey = std::tuple<int, const void*, const void*, const void*, const void*, const void*,
                            const void*, int64_t, int, int, int, int64_t, double>;
// Per host thread: a solve returns only after its graph launches have
// finished, so a thread can evict its own graphs safely; a process-wide
// cache let one thread destroy a graph another thread was launching.
struct GraphCache
{
  std::map<GraphKey, cudaGraphExec_t> graphs;
  ~GraphCache()
  {
    for (auto& kv : graphs)
      cudaGraphExecDestroy(kv.second);
  }
};
thread_local GraphCache t_graphs;

template <typename T>
int iteration_graph(const OpRef& o, T* x, const T* dinv, int64_t n, const Work<T>& w, int K,
                    bool reliable, cudaGraphExec_t* out)
{
  const bool q4 = o.kind == kQ4;
  const bool fused = sizeof(T) == 4 && o.kind == kSell && fused_update_on();
  GraphKey key{(fused ? 64 : 0) + (int)o.kind * 8 + (o.q4_tc ? 4 : 0) + (sizeof(T) == 4) * 2
                   + (reliable ? 1 : 0),
               q4 ? (const void*)o.q4->verts
                  : (o.kind == kSell ? (const void*)o.op : (const void*)o.A->row_ptr),
               q4 ? (const void*)o.q4->edges32
                  : (o.kind == kSell ? (const void*)o.op->vals : (const void*)o.A->vals),
               o.kind == kCsr ? (const void*)o.A->cols : nullptr,
               (const void*)x,
               (const void*)dinv,
               (const void*)w.st,
               n,
               K,
               w.blocks,
               o.kind == kCsr ? o.A->bs : 1,
               q4 ? (int64_t)o.q4->nx | ((int64_t)o.q4->ny << 21) | ((int64_t)o.q4->nz << 42)
                  : (o.kind == kSell ? (int64_t)o.op->serial : 0),
               q4 ? o.q4->kappa : 0.0};
  auto& g_graphs = t_graphs.graphs;
  auto it = g_graphs.find(key);
  if (it != g_graphs.end())
  {
    *out = it->second;
    return DFX_OK;
  }
  cudaStream_t cs;
  DFX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t graph;
  cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (ce == cudaSuccess)
  {
    for (int k = 0; k < K; ++k)
      enqueue_iteration<T>(o, x, dinv, n, w, reliable, cs);
    // A launch error inside capture invalidates the capture; EndCapture
    // reports it.
    ce = cudaStreamEndCapture(cs, &graph);
  }
  cudaStreamDestroy(cs);
  cudaGraphExec_t exec;
  if (ce == cudaSuccess)
  {
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
  }
  if (ce != cudaSuccess && fused)
  {
    // No graph with the cooperative launch here: the unfused iteration.
    (void)cudaGetLastError();
    g_fused_broken.store(1);
    return iteration_graph<T>(o, x, dinv, n, w, K, reliable, out);
  }
  DFX_CUDA(ce);
  if (g_graphs.size() >= 32)
  {
    cudaGraphExecDestroy(g_graphs.begin()->second);
    g_graphs.erase(g_graphs.begin());
  }
  g_graphs[key] = exec;
  *out = exec;
  return DFX_OK;
}

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

int read_state(const CgState* d, CgState** h, cudaStream_t s)
{
  if (!t_pinned.h)
    DFX_CUDA(cudaMallocHost(&t_pinned.h, 2 * sizeof(CgState)));
  *h = t_pinned.h;
  DFX_CUDA(cudaMemcpyAsync(*h, d, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}

// Replay the iteration graph until the state is done. Each replay runs K
// iterations and the state is done at max_iter at the latest, so the loop
// bound only guards against a corrupted state.
int run_to_done(cudaGraphExec_t exec, const CgState* dst, int max_iters, int K, CgState** h,
                cudaStream_t s, int64_t* kernels, int per_iter)
{
  const int64_t max_launches = (int64_t)max_iters / K + 2;
  for (int64_t launch = 0;; ++launch)
  {
    if (int st = read_state(dst, h, s))
      return st;
    if ((*h)->done)
      return DFX_OK;
    if (launch > max_launches)
      return dfx::fail(DFX_ERR_TIMEOUT, "CG state never reported completion");
    DFX_CUDA(cudaGraphLaunch(exec, s));
    *kernels += per_iter * (int64_t)K;
  }
}

int report(const CgState* h, dfx_cg_info* info, int64_t kernels)
{
  if (info)
  {
    info->iterations = h->iter;
    info->status = h->status;
    info->rnorm0_sq = h->rr0;
    info->rnorm_sq = h->rr;
    info->kernel_launches = kernels;
  }
  if (h->status == DFX_ERR_NOT_CONVERGED)
    return dfx::fail(DFX_ERR_NOT_CONVERGED,
                     "Solver exceeded max iterations (%d). Relative residual=%g.", h->iter,
                     h->rr0 > 0 ? h->rr / h->rr0 : 0.0);
  if (h->status == DFX_ERR_BREAKDOWN)
    return dfx::fail(DFX_ERR_BREAKDOWN, "CG breakdown at iteration %d (p.Ap=%g)", h->iter, h->pAp);
  return DFX_OK;
}

size_t csr_work_bytes(int64_t n)
{
  Carver c{nullptr};
  carve_work<double>(c, n);
  return c.used;
}

size_t op_work_bytes(int64_t n)
{
  Carver c{nullptr};
  carve_work<double>(c, n);
  c.take<double>(n); // x
  c.take<double>(n); // b
  c.take<double>(n); // dinv
  c.take<float>(2 * n); // p's FP32 words (split operators)
  return c.used;
}

size_t ir_work_bytes(int64_t n)
{
  Carver c{nullptr};
  carve_work<float>(c, n);
  c.take<CgState>(1);           // outer state
  carve_red(c, max_blocks(n));  // outer reduction
  c.take<double>(n); // x
  c.take<double>(n); // b
  c.take<double>(n); // dinv (unused FP64 copy kept for symmetry with op solve)
  c.take<float>(n);  // d
  c.take<float>(n);  // dinv32
  c.take<double>(n); // flexible outer loop: r
  c.take<double>(n); // p
  c.take<double>(n); // q = A p
  return c.used;
}

int check_solve_args(const double* b, const double* x, const void* work, double rtol,
                     int max_iters)
{
  DFX_REQUIRE(b && x && work, "b, x and workspace must be non-NULL");
  DFX_REQUIRE(rtol > 0.0 && max_iters > 0, "rtol and max_iters must be positive");
  DFX_REQUIRE(((uintptr_t)work & 255) == 0, "workspace must be 256-byte aligned");
  return DFX_OK;
}

} // namespace

extern "C" size_t dfx_cg_workspace_bytes(int64_t n) { return csr_work_bytes(n); }

extern "C" int dfx_cg_solve(const dfx_csr* A, const double* d_b, double* d_x,
                            const double* d_dinv, double rtol, int32_t max_iters,
                            int32_t graph_iters, void* d_work, size_t wbytes, dfx_cg_info* info,
                            void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->dtype == DFX_F64, "dfx_cg_solve runs in FP64");
  DFX_REQUIRE(A->nrows == A->ncols, "matrix must be square");
  if (int st = check_solve_args(d_b, d_x, d_work, rtol, max_iters))
    return st;
  const int64_t n = (int64_t)A->nrows * A->bs;
  DFX_REQUIRE(wbytes >= csr_work_bytes(n), "workspace too small (%zu < %zu)", wbytes,
              csr_work_bytes(n));
  cudaStream_t s = dfx::as_stream(stream);
  const int K = graph_iters > 0 ? graph_iters : 20;
  Carver c{(char*)d_work};
  Work<double> w = carve_work<double>(c, n);
  if (int st = reset_work(w.st, w.red, w.blocks, s))
    return st;
  if (int st = dfx::launch_spmv(A, d_x, w.y, 0.0, s))
    return st;
  enqueue_init<double>(d_b, w.y, d_x, d_dinv, n, w, rtol, max_iters, s);
  DFX_CHECK_LAUNCH();
  OpRef o{kCsr, A, nullptr};
  cudaGraphExec_t exec;
  if (int st = iteration_graph<double>(o, d_x, d_dinv, n, w, K, false, &exec))
    return st;
  CgState* h;
  int64_t kernels = 2;
  if (int st = run_to_done(exec, w.st, max_iters, K, &h, s, &kernels, kFusedIterKernels))
    return st;
  return report(h, info, kernels);
}

extern "C" size_t dfx_cg_op_workspace_bytes(int64_t n) { return op_work_bytes(n); }

extern "C" int dfx_cg_solve_op(dfx_operator op, const double* d_b, double* d_x,
                               const double* d_dinv, double rtol, int32_t max_iters,
                               int32_t graph_iters, void* d_work, size_t wbytes, dfx_cg_info* info,
                               void* stream)
{
  DFX_REQUIRE(op, "operator is NULL");
  DFX_REQUIRE(op->dtype == DFX_F64 || op->dtype == DFX_F32X2,
              "dfx_cg_solve_op needs an FP64 or split (DFX_F32X2) operator");
  DFX_REQUIRE(op->vals, "operator values were released (dfx_operator_release_values): use a share");
  if (int st = check_solve_args(d_b, d_x, d_work, rtol, max_iters))
    return st;
  const int64_t n = op->n;
  DFX_REQUIRE(wbytes >= op_work_bytes(n), "workspace too small (%zu < %zu)", wbytes,
              op_work_bytes(n));
  if (n == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  const int K = graph_iters > 0 ? graph_iters : 20;
  Carver c{(char*)d_work};
  Work<double> w = carve_work<double>(c, n);
  double* xp = c.take<double>(n);
  double* bp = c.take<double>(n);
  double* dp = d_dinv ? c.take<double>(n) : nullptr;
  if (op->dtype == DFX_F32X2)
    w.ph = c.take<float>(2 * n);
  const unsigned g = (unsigned)((n + 255) / 256);
  if (int st = reset_work(w.st, w.red, w.blocks, s))
    return st;
  k_gather<double, double><<<g, 256, 0, s>>>(d_x, xp, op->perm, (int32_t)n);
  k_gather<double, double><<<g, 256, 0, s>>>(d_b, bp, op->perm, (int32_t)n);
  if (dp)
    k_gather<double, double><<<g, 256, 0, s>>>(d_dinv, dp, op->perm, (int32_t)n);
  if (w.ph)
  {
    // A x0 from x0's FP32 words (the buffer of p's words is free until
    // k_init writes p).
    k_split_words<<<g, 256, 0, s>>>(xp, w.ph, n);
    if (int st = dfx::sell_spmv(*op, w.ph, w.y, s))
      return st;
  }
  else if (int st = dfx::sell_spmv(*op, xp, w.y, s))
    return st;
  enqueue_init<double>(bp, w.y, xp, dp, n, w, rtol, max_iters, s);
  DFX_CHECK_LAUNCH();
  OpRef o{kSell, nullptr, op};
  cudaGraphExec_t exec;
  if (int st = iteration_graph<double>(o, xp, dp, n, w, K, false, &exec))
    return st;
  CgState* h;
  int64_t kernels = 5 + (dp ? 1 : 0) + (w.ph ? 1 : 0);
  int st = run_to_done(exec, w.st, max_iters, K, &h, s, &kernels, kFusedIterKernels);
  CgState hs = *h;
  k_scatter<<<g, 256, 0, s>>>(xp, d_x, op->perm, (int32_t)n);
  DFX_CHECK_LAUNCH();
  if (st)
    return st;
  return report(&hs, info, kernels);
}

extern "C" size_t dfx_ir_workspace_bytes(int64_t n) { return ir_work_bytes(n); }

__global__ void k_state_init(CgState* st, double rtol2, double delta2, int max_iter, int forced)
{
  *st = CgState{};
  st->rtol2 = rtol2;
  st->delta2 = delta2;
  st->max_iter = max_iter;
  st->forced = forced;
}

extern "C" int dfx_ir_solve(dfx_operator op64, dfx_operator op32, const double* d_b, double* d_x,
                            const double* d_dinv, double rtol, double inner_rtol,
                            int32_t max_outer, int32_t max_inner, int32_t graph_iters,
                            int32_t variant, void* d_work, size_t wbytes, dfx_ir_info* info,
                            void* stream)
{
  DFX_REQUIRE(op64 && op32, "operators must be non-NULL");
  DFX_REQUIRE(op64->bs == 1 && op32->bs == 1, "refinement takes scalar (bs 1) operators");
  DFX_REQUIRE(op64->dtype == DFX_F64 && op32->dtype == DFX_F32,
              "refinement needs an FP64 outer and an FP32 inner operator");
  DFX_REQUIRE(op64->n == op32->n && op64->sigma == op32->sigma && op64->nslices == op32->nslices
                  && op64->csr_nnz == op32->csr_nnz,
              "inner and outer operators must come from the same matrix and sigma");
  DFX_REQUIRE(op64->vals && op32->vals, "operator values were released (dfx_operator_release_values): use a share");
  if (int st = check_solve_args(d_b, d_x, d_work, rtol, max_outer))
    return st;
  DFX_REQUIRE(inner_rtol > 0.0 && inner_rtol < 1.0 && max_inner > 0,
              "inner_rtol must be in (0, 1) and max_inner positive");
  DFX_REQUIRE(variant == DFX_IR_RESTART || variant == DFX_IR_RELIABLE
                  || variant == DFX_IR_FLEXIBLE,
              "unknown variant %d", variant);
  const int64_t n = op64->n;
  DFX_REQUIRE(wbytes >= ir_work_bytes(n), "workspace too small (%zu < %zu)", wbytes,
              ir_work_bytes(n));
  if (info)
    *info = dfx_ir_info{};
  if (n == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  const int K = graph_iters > 0 ? graph_iters : 20;
  Carver c{(char*)d_work};
  Work<float> w = carve_work<float>(c, n);
  CgState* outer = c.take<CgState>(1);
  Red ored = carve_red(c, max_blocks(n));
  double* xp = c.take<double>(n);
  double* bp = c.take<double>(n);
  c.take<double>(n);
  float* d32 = c.take<float>(n);
  float* dinv32 = d_dinv ? c.take<float>(n) : nullptr;
  double* r64 = c.take<double>(n);
  double* p64 = c.take<double>(n);
  double* q64 = c.take<double>(n);
  const unsigned g = (unsigned)((n + 255) / 256);
  k_gather<double, double><<<g, 256, 0, s>>>(d_x, xp, op64->perm, (int32_t)n);
  k_gather<double, double><<<g, 256, 0, s>>>(d_b, bp, op64->perm, (int32_t)n);
  if (dinv32)
    k_gather<double, float><<<g, 256, 0, s>>>(d_dinv, dinv32, op64->perm, (int32_t)n);
  DFX_CHECK_LAUNCH();
  const bool reliable = variant == DFX_IR_RELIABLE;
  const bool flexible = variant == DFX_IR_FLEXIBLE;
  OpRef o{kSell, nullptr, op32};
  cudaGraphExec_t exec;
  if (int st = iteration_graph<float>(o, d32, dinv32, n, w, K, reliable, &exec))
    return st;
  const int blocks = stride_grid();
  int inner_total = 0, outer_count = 0, st = DFX_OK;
  int64_t kernels = 2 + (dinv32 ? 1 : 0);
  CgState* h = nullptr;
  CgState ho{};
  if (flexible)
  {
    // Flexible CG: each outer iteration takes the inner FP32 PCG solve of
    // A d = r (to inner_rtol, at most max_inner iterations) as its
    // preconditioned residual. A converged recursive residual is confirmed
    // by the true residual; if that disagrees, the outer loop restarts from
    // it.
    if (int e = reset_work(outer, ored, w.blocks, s))
      return e;
    if (int e = reset_work(w.st, w.red, w.blocks, s))
      return e;
    k_state_init<<<1, 1, 0, s>>>(outer, rtol * rtol, 0.0, max_outer, 0);
    const int eg = elem_grid(n);
    auto true_residual = [&](int first) -> int
    {
      k_fcg_residual<<<sell_blocks(n), kSellThreads, 0, s>>>(*op64, bp, xp, r64, w.r, outer,
                                                             ored, first);
      DFX_CHECK_LAUNCH();
      kernels += 1;
      return read_state(outer, &h, s);
    };
    kernels += 1;
    bool restart = true;
    if (!(st = true_residual(1)) && !h->done)
    {
      for (;;)
      {
        enqueue_init<float>(w.r, nullptr, d32, dinv32, n, w, inner_rtol, max_inner, s);
        DFX_CHECK_LAUNCH();
        kernels += 1;
        if ((st = run_to_done(exec, w.st, max_inner, K, &h, s, &kernels, f32_sell_iter_kernels())))
          break;
        inner_total += h->iter;
        if (!restart)
        {
          k_fcg_gamma<<<eg, kElemThreads, 0, s>>>(d32, q64, n, outer, ored);
          kernels += 1;
        }
        k_fcg_direction<<<blocks, kThreads, 0, s>>>(d32, p64, n, outer, restart ? 1 : 0);
        k_fcg_spmv<<<sell_blocks(n), kSellThreads, 0, s>>>(*op64, p64, q64, r64, outer, ored);
        k_fcg_update<<<eg, kElemThreads, 0, s>>>(xp, r64, p64, q64, w.r, n, outer, ored);
        DFX_CHECK_LAUNCH();
        kernels += 3;
        if ((st = read_state(outer, &h, s)))
          break;
        restart = false;
        if (h->done)
        {
          if (h->status != DFX_OK)
            break;
          if ((st = true_residual(0)) || h->done)
            break;
          restart = true; // the recursive residual drifted: restart from b - A x
        }
      }
    }
    if (h)
    {
      ho = *h;
      outer_count = ho.iter;
    }
  }
  else if (!reliable)
  {
    // Restarted refinement: each correction is a fresh FP32 PCG solve.
    if (int e = reset_work(outer, ored, w.blocks, s))
      return e;
    if (int e = reset_work(w.st, w.red, w.blocks, s))
      return e;
    for (;;)
    {
      k_ir_residual<<<sell_blocks(n), kSellThreads, 0, s>>>(*op64, bp, xp, w.r, outer, ored,
                                                            rtol * rtol, max_outer);
      DFX_CHECK_LAUNCH();
      kernels += 1;
      if ((st = read_state(outer, &h, s)))
        break;
      ho = *h;
      if (ho.done)
        break;
      enqueue_init<float>(w.r, nullptr, d32, dinv32, n, w, inner_rtol, max_inner, s);
      DFX_CHECK_LAUNCH();
      if ((st = run_to_done(exec, w.st, max_inner, K, &h, s, &kernels, f32_sell_iter_kernels())))
        break;
      inner_total += h->iter;
      // A stalled or broken-down inner solve still yields a usable correction.
      k_ir_correct<<<blocks, kThreads, 0, s>>>(xp, d32, n);
      DFX_CHECK_LAUNCH();
      kernels += 2;
    }
    outer_count = ho.iter - 1;
  }
  else
  {
    // One FP32 PCG whose residual is replaced by the FP64 residual each time
    // it has dropped by inner_rtol (reliable updates); the FP32 correction
    // is folded into x in FP64 at every replacement.
    if (int e = reset_work(w.st, w.red, w.blocks, s))
      return e;
    k_state_init<<<1, 1, 0, s>>>(w.st, rtol * rtol, inner_rtol * inner_rtol, max_inner,
                                 kForcedUpdate);
    DFX_CUDA(cudaMemsetAsync(d32, 0, sizeof(float) * n, s));
    DFX_CUDA(cudaMemsetAsync(w.p, 0, sizeof(float) * n, s));
    auto replace = [&]() -> int
    {
      if (dinv32)
        k_rel_residual<true><<<sell_blocks(n), kSellThreads, 0, s>>>(*op64, bp, xp, dinv32, w);
      else
        k_rel_residual<false><<<sell_blocks(n), kSellThreads, 0, s>>>(*op64, bp, xp, dinv32, w);
      DFX_CHECK_LAUNCH();
      kernels += 1;
      return read_state(w.st, &h, s);
    };
    kernels += 1;
    // Stagnation: when the FP32 operator's rounding (about 6e-8 |A| per
    // entry) exceeds the smallest eigenvalue, replacements stop reducing the
    // FP64 residual; stop after kStall replacements without a 2x gain.
    constexpr int kStall = 4;
    double best = 0.0;
    int stall = 0;
    if (!(st = replace()) && !h->done)
    {
      best = h->rr;
      for (;;)
      {
        enqueue_pupdate<float>(dinv32, n, w, s);
        DFX_CHECK_LAUNCH();
        kernels += 1;
        if ((st = run_to_done(exec, w.st, max_inner, K, &h, s, &kernels, f32_sell_iter_kernels())))
          break;
        const int32_t why = h->status;
        k_ir_correct<<<blocks, kThreads, 0, s>>>(xp, d32, n);
        DFX_CHECK_LAUNCH();
        kernels += 1;
        if (why != kPauseUpdate && why != kPauseConverged)
          break; // not converged within max_inner, or breakdown
        if ((st = replace()) || h->done)
          break;
        if (h->rr < 0.25 * best)
        {
          best = h->rr;
          stall = 0;
        }
        else if (++stall >= kStall)
        {
          h->status = DFX_ERR_NOT_CONVERGED;
          break;
        }
        if (h->updates > max_outer)
        {
          st = dfx::fail(DFX_ERR_NOT_CONVERGED,
                         "Refinement exceeded max residual replacements (%d).", max_outer);
          break;
        }
      }
    }
    if (h)
    {
      ho = *h;
      inner_total = ho.iter;
      outer_count = ho.updates;
    }
  }
  k_scatter<<<g, 256, 0, s>>>(xp, d_x, op64->perm, (int32_t)n);
  DFX_CHECK_LAUNCH();
  if (st)
    return st;
  DFX_CUDA(cudaStreamSynchronize(s));
  if (info)
  {
    info->outer_iterations = outer_count;
    info->inner_iterations = inner_total;
    info->status = ho.status;
    info->rnorm0_sq = ho.rr0;
    info->rnorm_sq = ho.rr;
    info->kernel_launches = kernels + 1;
  }
  if (ho.status == DFX_ERR_NOT_CONVERGED)
    return dfx::fail(DFX_ERR_NOT_CONVERGED,
                     "Refinement did not converge. Relative residual=%g.",
                     ho.rr0 > 0 ? ho.rr / ho.rr0 : 0.0);
  if (ho.status == DFX_ERR_BREAKDOWN)
    return dfx::fail(DFX_ERR_BREAKDOWN, "refinement breakdown (non-finite residual or p.Ap <= 0)");
  return DFX_OK;
}

// ---------------------------------------------------------------------------
// CG on the matrix-free Q4 action.
namespace
{
// Kernels of one matrix-free iteration: 8 colour kernels, p.Ap, update,
// p update (the y memset is a graph memset node, not a kernel).
constexpr int kQ4IterKernels = 11;

size_t q4_work_bytes(int64_t n, int mode)
{
  Carver c{nullptr};
  if (mode == 0)
    carve_work<double>(c, n);
  else
  {
    carve_work<float>(c, n);
    c.take<double>(n); // A x in FP64
    c.take<float>(n);  // FP32 correction d
  }
  return c.used;
}
} // namespace

extern "C" size_t dfx_q4_cg_workspace_bytes(int64_t n, int32_t mode)
{
  return (mode >= 0 && mode <= 2) ? q4_work_bytes(n, mode) : 0;
}

extern "C" int dfx_q4_cg_solve(const dfx_q4_mesh* mesh, const double* d_b, double* d_x,
                               double rtol, int32_t max_iters, int32_t mode, double delta,
                               int32_t graph_iters, void* d_work, size_t wbytes, dfx_cg_info* info,
                               void* stream)
{
  DFX_REQUIRE(mesh && mesh->nx > 0 && mesh->ny > 0 && mesh->nz > 0 && mesh->verts,
              "invalid Q4 mesh");
  if (int st = check_solve_args(d_b, d_x, d_work, rtol, max_iters))
    return st;
  DFX_REQUIRE(mode >= 0 && mode <= 2,
              "mode must be 0 (FP64), 1 (mixed) or 2 (mixed, tensor cores), got %d", mode);
  DFX_REQUIRE(mode == 0 || (delta > 0.0 && delta < 1.0), "delta must be in (0, 1)");
  const int64_t n = dfx::q4_ndofs(*mesh);
  DFX_REQUIRE(wbytes >= q4_work_bytes(n, mode), "workspace too small (%zu < %zu)", wbytes,
              q4_work_bytes(n, mode));
  if (info)
    *info = dfx_cg_info{};
  if (int st = dfx::q4_prepare())
    return st;
  cudaStream_t s = dfx::as_stream(stream);
  const int K = graph_iters > 0 ? graph_iters : 20;
  const OpRef o{kQ4, nullptr, nullptr, mesh, mode == 2 ? 1 : 0};
  Carver c{(char*)d_work};
  CgState* h = nullptr;
  int64_t kernels = 0;
  if (mode == 0)
  {
    Work<double> w = carve_work<double>(c, n);
    if (int st = reset_work(w.st, w.red, w.blocks, s))
      return st;
    if (int st = dfx::q4_apply<double>(*mesh, d_x, w.y, s))
      return st;
    enqueue_init<double>(d_b, w.y, d_x, nullptr, n, w, rtol, max_iters, s);
    DFX_CHECK_LAUNCH();
    cudaGraphExec_t exec;
    if (int st = iteration_graph<double>(o, d_x, nullptr, n, w, K, false, &exec))
      return st;
    kernels = 9;
    if (int st = run_to_done(exec, w.st, max_iters, K, &h, s, &kernels, kQ4IterKernels))
      return st;
    return report(h, info, kernels);
  }
  // Mixed: FP32 CG on the FP32 action, its residual replaced by b - A x from
  // the FP64 action whenever |r| has dropped by delta (reliable updates); the
  // FP32 correction is folded into x in FP64 at each replacement.
  Work<float> w = carve_work<float>(c, n);
  double* ax = c.take<double>(n);
  float* d32 = c.take<float>(n);
  if (int st = reset_work(w.st, w.red, w.blocks, s))
    return st;
  k_state_init<<<1, 1, 0, s>>>(w.st, rtol * rtol, delta * delta, max_iters, kForcedUpdateQ4);
  DFX_CUDA(cudaMemsetAsync(d32, 0, sizeof(float) * n, s));
  DFX_CUDA(cudaMemsetAsync(w.p, 0, sizeof(float) * n, s));
  DFX_CHECK_LAUNCH();
  cudaGraphExec_t exec;
  if (int st = iteration_graph<float>(o, d32, nullptr, n, w, K, true, &exec))
    return st;
  kernels = 1;
  auto replace = [&]() -> int
  {
    if (int st = dfx::q4_apply<double>(*mesh, d_x, ax, s))
      return st;
    k_rel_residual_vec<false><<<elem_grid(n), kElemThreads, 0, s>>>(d_b, ax, nullptr, n, w);
    DFX_CHECK_LAUNCH();
    kernels += 9;
    return read_state(w.st, &h, s);
  };
  constexpr int kStall = 4;
  const int max_updates = max_iters / 10 + 100;
  int st = replace();
  if (!st && !h->done)
  {
    double best = h->rr;
    int stall = 0;
    for (;;)
    {
      enqueue_pupdate<float>(nullptr, n, w, s);
      DFX_CHECK_LAUNCH();
      kernels += 1;
      if ((st = run_to_done(exec, w.st, max_iters, K, &h, s, &kernels, kQ4IterKernels)))
        break;
      const int32_t why = h->status;
      k_ir_correct<<<stride_grid(), kThreads, 0, s>>>(d_x, d32, n);
      DFX_CHECK_LAUNCH();
      kernels += 1;
      if (why != kPauseUpdate && why != kPauseConverged)
        break; // iteration cap or breakdown
      if ((st = replace()) || h->done)
        break;
      if (h->rr < 0.25 * best)
      {
        best = h->rr;
        stall = 0;
      }
      else if (++stall >= kStall)
      {
        h->status = DFX_ERR_NOT_CONVERGED;
        break;
      }
      if (h->updates > max_updates)
      {
        h->status = DFX_ERR_NOT_CONVERGED;
        break;
      }
    }
  }
  if (st)
    return st;
  if (mode == 2)
    if (int e = dfx::q4_tc_check())
      return e;
  return report(h, info, kernels);
}

// ---------------------------------------------------------------------------
// CG without any allocation.
//
// For callers that may not allocate device or pinned host memory themselves
// or have the library do it: code running between a host application's own
// memory-pool set-up and its capture of a CUDA graph, plugins whose host
// owns every allocation, and real-time loops that forbid allocation after
// start-up. The solve uses a fixed scratch array that lives in the library's
// device image (loaded on every GPU that loads the library and kept until
// the process exits), launches its kernels directly (no graph is built) and
// reads the solver state back into pageable host memory.
namespace
{
// Largest problem of the no-allocation solve, in scalar unknowns.
constexpr int64_t kNoAllocMaxN = 524288;
// State, reduction buffers and the three CG vectors r, p, y for
// kNoAllocMaxN unknowns (13 MiB).
constexpr size_t kNoAllocBytes = (size_t)13 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array in the current context, looked up on
// every call: it allocates nothing, and a context that was reset and made
// again (cudaDeviceReset) may place the array elsewhere.
int noalloc_scratch(void** out)
{
  void* p = nullptr;
  DFX_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  *out = p;
  return DFX_OK;
}
} // namespace

extern "C" int dfx_cg_solve_noalloc(const dfx_csr* A, const double* d_b, double* d_x,
                                    const double* d_dinv, double rtol, int32_t max_iters,
                                    int32_t check_every, dfx_cg_info* info, void* stream)
{
  if (int st = dfx::check_csr(A))
    return st;
  DFX_REQUIRE(A->dtype == DFX_F64, "dfx_cg_solve_noalloc runs in FP64");
  DFX_REQUIRE(A->nrows == A->ncols, "matrix must be square");
  DFX_REQUIRE(d_b && d_x, "b and x must be non-NULL");
  DFX_REQUIRE(rtol > 0.0 && max_iters > 0, "rtol and max_iters must be positive");
  const int64_t n = (int64_t)A->nrows * A->bs;
  DFX_REQUIRE(n <= kNoAllocMaxN,
              "dfx_cg_solve_noalloc takes at most %lld unknowns (got %lld); use dfx_cg_solve",
              (long long)kNoAllocMaxN, (long long)n);
  DFX_REQUIRE(csr_work_bytes(n) <= kNoAllocBytes,
              "scratch of %zu bytes exceeds the fixed %zu bytes; use dfx_cg_solve",
              csr_work_bytes(n), kNoAllocBytes);
  void* scratch = nullptr;
  if (int st = noalloc_scratch(&scratch))
    return st;
  cudaStream_t s = dfx::as_stream(stream);
  const int K = check_every > 0 ? check_every : 20;
  Carver c{(char*)scratch};
  Work<double> w = carve_work<double>(c, n);
  // The array keeps the previous call's contents: the state and the group
  // tickets must start from zero.
  if (int st = reset_work(w.st, w.red, w.blocks, s))
    return st;
  if (int st = dfx::launch_spmv(A, d_x, w.y, 0.0, s))
    return st;
  enqueue_init<double>(d_b, w.y, d_x, d_dinv, n, w, rtol, max_iters, s);
  DFX_CHECK_LAUNCH();
  OpRef o{kCsr, A, nullptr};
  CgState h{};
  int64_t kernels = 2;
  const int64_t max_rounds = (int64_t)max_iters / K + 2;
  for (int64_t round = 0;; ++round)
  {
    DFX_CUDA(cudaMemcpyAsync(&h, w.st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    DFX_CUDA(cudaStreamSynchronize(s));
    if (h.done)
      break;
    if (round > max_rounds)
      return dfx::fail(DFX_ERR_TIMEOUT, "CG state never reported completion");
    for (int k = 0; k < K; ++k)
      enqueue_iteration<double>(o, d_x, d_dinv, n, w, false, s);
    DFX_CHECK_LAUNCH();
    kernels += 3 * (int64_t)K;
  }
  return report(&h, info, kernels);
}

extern "C" int dfx_set_cg_fused_update(int32_t on)
{
  t_fused_update = on ? 1 : 0;
  return DFX_OK;
}

extern "C" int dfx_get_cg_fused_update(int32_t* on)
{
  DFX_REQUIRE(on, "on is NULL");
  *on = fused_update_on() ? 1 : 0;
  return DFX_OK;
}

// Runs the grid barrier of the fused update with one arrival missing (two
// cooperative blocks waiting for three), so that its bounded waits run out;
// *gave_up = the number of blocks that reported the timeout (2 when the
// wait limit works). The device stays usable. Uses its own small state
// allocation.
extern "C" int dfx_selftest_grid_barrier(int32_t* gave_up)
{
  DFX_REQUIRE(gave_up, "gave_up is NULL");
  *gave_up = 0;
  CgState* st = nullptr;
  if (cudaMalloc(&st, sizeof(CgState)) != cudaSuccess)
    return dfx::no_memory("barrier self-test state");
  cudaError_t e = cudaMemset(st, 0, sizeof(CgState));
  if (e == cudaSuccess)
  {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(2);
    cfg.blockDim = dim3(64);
    cfg.stream = 0;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_barrier_selftest, st);
  }
  CgState h{};
  if (e == cudaSuccess)
    e = cudaMemcpy(&h, st, sizeof(CgState), cudaMemcpyDeviceToHost);
  cudaFree(st);
  DFX_CUDA(e);
  *gave_up = h.status == DFX_ERR_TIMEOUT ? h.updates : 0;
  return DFX_OK;
}
