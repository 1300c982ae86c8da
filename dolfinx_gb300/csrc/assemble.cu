// Cell assembly kernels: fem::assemble_matrix / assemble_vector /
// apply_lifting / DirichletBC::set / set_diagonal on sm_103a.
//
// Design (per block of CPB cells, RCM cell order keeps neighbouring
// cells' rows close together in L2):
//   stage 0  dofs, row starts and BC markers of the cells -> shared memory
//   stage 1  element tensor in FP64 (geometry + exact reference tensors,
//            minimal FP64 operation count) -> shared memory (upper
//            triangle, the tensors are symmetric)
//   stage 2  one thread per element entry: BC zeroing, CSR slot from the
//            cell->slot map, scatter. Consecutive threads write
//            consecutive columns of one row, so atomics and map reads
//            coalesce by sector.
// Modes: FP64 atomics (one launch), or colour classes with plain
// read-modify-write (deterministic summation order).
#include "common.cuh"
#include "element_tables.h"

#include <vector>

namespace
{
constexpr int kThreads = 128;

__device__ __forceinline__ void load_cell_coords(const dfx_form& a, int64_t c, double* xc)
{
  const int4 xd = __ldg(reinterpret_cast<const int4*>(a.x_dofmap) + c);
  const int nodes[4] = {xd.x, xd.y, xd.z, xd.w};
#pragma unroll
  for (int v = 0; v < 4; ++v)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      xc[3 * v + k] = __ldg(a.x + 3 * (int64_t)nodes[v] + k);
}

// adj(J) (= det J * J^{-1}) and det J of the affine map of a tetrahedron,
// J_ij = dx_i/dX_j with columns x1-x0, x2-x0, x3-x0.
__device__ __forceinline__ double tet_adjugate(const double* xc, double adj[3][3])
{
  double J[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      J[i][j] = xc[3 * (j + 1) + i] - xc[i];
  adj[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  adj[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  adj[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  adj[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  adj[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  adj[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  adj[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  adj[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  return J[0][0] * adj[0][0] + J[0][1] * adj[1][0] + J[0][2] * adj[2][0];
}

// G_ab = kappa |det J| (K K^T)_ab = kappa (adj adj^T)_ab / |det J|, in the
// order 00, 11, 22, 01, 02, 12. Returns |det J|.
__device__ __forceinline__ double tet_metric(const double* xc, double kappa, double* G)
{
  double adj[3][3];
  const double adet = fabs(tet_adjugate(xc, adj));
  const double s = kappa / adet;
  auto dot = [&](int a, int b)
  { return adj[a][0] * adj[b][0] + adj[a][1] * adj[b][1] + adj[a][2] * adj[b][2]; };
  G[0] = s * dot(0, 0);
  G[1] = s * dot(1, 1);
  G[2] = s * dot(2, 2);
  G[3] = s * dot(0, 1);
  G[4] = s * dot(0, 2);
  G[5] = s * dot(1, 2);
  return adet;
}

__device__ __forceinline__ double tet_absdet(const double* xc)
{
  double J[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      J[i][j] = xc[3 * (j + 1) + i] - xc[i];
  return fabs(J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1])
              - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0])
              + J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]));
}

__host__ __device__ constexpr int packed(int i, int j, int n)
{
  return i * n - i * (i - 1) / 2 + (j - i);
}

// Position of `col` in the sorted row [b, e) of cols, or -1.
__device__ __forceinline__ int64_t row_search(const int32_t* __restrict__ cols, int64_t b,
                                              int64_t e, int32_t col)
{
  while (b < e)
  {
    const int64_t m = (b + e) >> 1;
    const int32_t v = __ldg(cols + m);
    if (v < col)
      b = m + 1;
    else
      e = m;
  }
  return (e < 0) ? -1 : e;
}

// Bulk asynchronous copy global -> shared memory (the 1D form of TMA),
// completing on a CTA-local mbarrier. Both addresses 16-byte aligned, size
// a multiple of 16.
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], "
               "%2, [%3];" ::"r"(smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Wait for phase `parity` of the mbarrier, at most max_tries polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int max_tries)
{
  for (int i = 0; i < max_tries; ++i)
  {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    if (done)
      return true;
  }
  return false;
}

template <bool COLOURED>
__device__ __forceinline__ void scatter_add(double* p, double v)
{
  if constexpr (COLOURED)
    *p += v;
  else
    atomicAdd(p, v);
}

// Form traits: scalar P1/P2 Poisson(+mass) or vector P2 elasticity.
template <int DEG, bool ELAST>
struct Traits
{
  static constexpr int ND = DEG == 1 ? 4 : 10; // nodes per cell
  static constexpr int BS = ELAST ? 3 : 1;
  static constexpr int N = ND * BS; // element tensor dimension
  static constexpr int NU = N * (N + 1) / 2;
  static constexpr int CPB = ELAST ? 4 : 32; // cells per block
};

// Stage-1 element tensors for the CPB cells of a block into sA.
template <int DEG, bool ELAST, bool MASS>
__device__ __forceinline__ void element_tensors(const dfx_form& a, const int32_t* sCell,
                                                const int8_t* sActive, int nloc, double* sA,
                                                double* sScratch)
{
  using T = Traits<DEG, ELAST>;
  if constexpr (!ELAST)
  {
    const int cl = threadIdx.x;
    if (cl < nloc && sActive[cl])
    {
      const int64_t c = sCell[cl];
      double xc[12];
      load_cell_coords(a, c, xc);
      const double kap = a.kappa ? __ldg(a.kappa + c) : a.kappa_const;
      double G[6];
      const double adet = tet_metric(xc, kap, G);
      double A[T::NU];
      if constexpr (DEG == 1)
        tet_p1_poisson_upper<MASS>(G, a.k2 * adet, A);
      else
        tet_p2_poisson_upper<MASS>(G, a.k2 * adet, A);
#pragma unroll
      for (int k = 0; k < T::NU; ++k)
        sA[cl * T::NU + k] = A[k];
    }
    __syncthreads();
  }
  else
  {
    // sScratch layout per cell: K (9), w*|det| (1), mu (1), lambda (1),
    // then physical gradients g[q][i][3] (120).
    constexpr int SS = 132;
    const int cl = threadIdx.x;
    if (cl < nloc && sActive[cl])
    {
      const int64_t c = sCell[cl];
      double xc[12], adj[3][3];
      load_cell_coords(a, c, xc);
      const double det = tet_adjugate(xc, adj);
      const double inv = 1.0 / det;
      double* s = sScratch + cl * SS;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          s[3 * i + j] = adj[i][j] * inv; // K = J^{-1}
      const double E = a.kappa ? __ldg(a.kappa + c) : a.kappa_const;
      const double nu = a.nu;
      s[9] = fabs(det) * (1.0 / 24.0);
      s[10] = E / (2.0 * (1.0 + nu));
      s[11] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    }
    __syncthreads();
    // g_i(q) = K^T dphi_i(q): thread per (cell, q, i).
    for (int t = threadIdx.x; t < nloc * 40; t += blockDim.x)
    {
      const int c = t / 40, qi = t % 40, q = qi / 10, i = qi % 10;
      if (!sActive[c])
        continue;
      double* s = sScratch + c * SS;
      const double d0 = kP2GradQ4[q][i][0], d1 = kP2GradQ4[q][i][1], d2 = kP2GradQ4[q][i][2];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        s[12 + 3 * qi + k] = s[k] * d0 + s[3 + k] * d1 + s[6 + k] * d2;
    }
    __syncthreads();
    // 3x3 block (i <= j): thread per (cell, block pair).
    for (int t = threadIdx.x; t < nloc * 55; t += blockDim.x)
    {
      const int c = t / 55;
      if (!sActive[c])
        continue;
      int p = t % 55, i = 0;
      while (p >= 10 - i)
      {
        p -= 10 - i;
        ++i;
      }
      const int j = i + p;
      const double* s = sScratch + c * SS;
      const double w = s[9], mu = s[10], lm = s[11];
      double B[3][3] = {};
#pragma unroll
      for (int q = 0; q < 4; ++q)
      {
        const double* gi = s + 12 + 3 * (10 * q + i);
        const double* gj = s + 12 + 3 * (10 * q + j);
        const double gg = gi[0] * gj[0] + gi[1] * gj[1] + gi[2] * gj[2];
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int l = 0; l < 3; ++l)
            B[k][l] += w * (mu * ((k == l ? gg : 0.0) + gi[l] * gj[k]) + lm * gi[k] * gj[l]);
      }
      double* A = sA + c * T::NU;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l)
          if (i < j || k <= l)
            A[packed(3 * i + k, 3 * j + l, 30)] = B[k][l];
    }
    __syncthreads();
  }
}

// Lifting rows of the nloc element tensors in sA
// (fem/assemble_vector_impl.h:377-402): thread per element row,
// b[r] -= alpha * sum_c Ae[r,c] (g[c] - x0[c]) over constrained columns c.
template <int DEG, bool ELAST, bool COLOURED>
__device__ __forceinline__ void lift_rows(const double* sA, const int32_t* sDof, const int8_t* sBc,
                                          const int8_t* sActive, int nloc,
                                          const double* __restrict__ g,
                                          const double* __restrict__ x0, double alpha,
                                          double* __restrict__ b)
{
  using T = Traits<DEG, ELAST>;
  constexpr int ND = T::ND, BS = T::BS, N = T::N, NU = T::NU;
  for (int e = threadIdx.x; e < nloc * N; e += blockDim.x)
  {
    const int cl = e / N, I = e % N;
    if (!sActive[cl])
      continue;
    double acc = 0.0;
    for (int J = 0; J < N; ++J)
    {
      if (!sBc[cl * N + J])
        continue;
      const int64_t jj = (int64_t)BS * sDof[cl * ND + J / BS] + J % BS;
      const double gv = g[jj] - (x0 ? x0[jj] : 0.0);
      acc += sA[cl * NU + (I <= J ? packed(I, J, N) : packed(J, I, N))] * gv;
    }
    if (acc != 0.0)
      scatter_add<COLOURED>(b + (int64_t)BS * sDof[cl * ND + I / BS] + I % BS, -alpha * acc);
  }
}

// Matrix assembly over a list of cells (list == nullptr: cells [0, count)),
// CPB cells per block (the autotuner's choice, at most kThreads).
template <int DEG, bool ELAST, bool MASS, bool COLOURED, int CPB>
__global__ void __launch_bounds__(kThreads)
    k_cells_matrix(const dfx_form a, const int64_t* __restrict__ row_ptr,
                   const int32_t* __restrict__ cols, double* __restrict__ vals,
                   const uint8_t* __restrict__ map, const int8_t* __restrict__ bc,
                   const int32_t* __restrict__ list, int32_t count, int* __restrict__ status)
{
  static_assert(CPB <= kThreads, "stage 1 runs one thread per cell");
  using T = Traits<DEG, ELAST>;
  constexpr int ND = T::ND, BS = T::BS, N = T::N, NU = T::NU;
  __shared__ double sA[CPB * NU];
  __shared__ double sScratch[ELAST ? CPB * 132 : 1];
  __shared__ int32_t sCell[CPB];
  __shared__ __align__(16) int32_t sDof[CPB * ND];
  __shared__ int64_t sRow[CPB * ND];
  __shared__ int8_t sBc[CPB * N];
  __shared__ int8_t sActive[CPB];
  __shared__ uint64_t sBar;

  const int64_t base = (int64_t)blockIdx.x * CPB;
  const int nloc = (int)(((int64_t)count - base) < CPB ? ((int64_t)count - base) : CPB);
  if (nloc <= 0)
    return;
  // Stage 0. A full block of consecutive cells reads its dofmap rows as one
  // contiguous span: one bulk copy into shared memory (CPB*ND*4 bytes, a
  // multiple of 16 for every CPB candidate), when the dofmap is 16-byte
  // aligned. Other blocks load the rows entry by entry.
  constexpr uint32_t kRowBytes = (uint32_t)(CPB * ND * sizeof(int32_t));
  static_assert(kRowBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
  const bool bulk = !list && nloc == CPB && (((uintptr_t)a.dofmap & 15) == 0);
  if (bulk && threadIdx.x == 0)
  {
    mbar_init(&sBar, 1);
    mbar_expect_tx(&sBar, kRowBytes);
    bulk_g2s(sDof, a.dofmap + base * ND, kRowBytes, &sBar);
  }
  if (threadIdx.x < nloc)
  {
    sCell[threadIdx.x] = list ? __ldg(list + base + threadIdx.x) : (int32_t)(base + threadIdx.x);
    sActive[threadIdx.x] = 1;
  }
  __syncthreads();
  bool staged = bulk;
  if (bulk && !__syncthreads_and(mbar_wait(&sBar, 0, 1 << 20)))
  {
    // The copy did not land in time: report it and let it finish
    // (bounded), then load the rows directly (the copy writes the same
    // values). If it still has not landed, the block writes nothing: the
    // late copy could overwrite shared memory after the block exits. The
    // status marks the assembled values void either way.
    if (threadIdx.x == 0)
      atomicExch(status, (int)DFX_ERR_TIMEOUT);
    if (!__syncthreads_and(mbar_wait(&sBar, 0, 1 << 24)))
      return;
    staged = false;
  }
  for (int t = threadIdx.x; t < nloc * ND; t += blockDim.x)
  {
    const int cl = t / ND, i = t % ND;
    const int32_t d = staged ? sDof[t] : __ldg(a.dofmap + (int64_t)sCell[cl] * ND + i);
    if (!staged)
      sDof[t] = d;
    sRow[t] = __ldg(row_ptr + d);
#pragma unroll
    for (int k = 0; k < BS; ++k)
      sBc[cl * N + BS * i + k] = bc ? __ldg(bc + (int64_t)BS * d + k) : 0;
  }
  __syncthreads();
  element_tensors<DEG, ELAST, MASS>(a, sCell, sActive, nloc, sA, sScratch);

  // Stage 2: scatter Ae into the CSR values, BC rows/columns zeroed
  // (fem/assemble_matrix_impl.h:161-196).
  constexpr int NN = ND * ND;
  for (int e = threadIdx.x; e < nloc * N * N; e += blockDim.x)
  {
    const int cl = e / (N * N), IJ = e % (N * N), I = IJ / N, J = IJ % N;
    if (sBc[cl * N + I] | sBc[cl * N + J])
      continue;
    const int i = I / BS, j = J / BS, k = I % BS, l = J % BS;
    const double v = sA[cl * NU + (I <= J ? packed(I, J, N) : packed(J, I, N))];
    int64_t pos;
    if (map)
      pos = sRow[cl * ND + i] + map[(int64_t)sCell[cl] * NN + i * ND + j];
    else
    {
      const int32_t di = sDof[cl * ND + i];
      const int64_t rb = sRow[cl * ND + i], re = __ldg(row_ptr + di + 1);
      pos = row_search(cols, rb, re, sDof[cl * ND + j]);
      if (pos >= re || __ldg(cols + pos) != sDof[cl * ND + j])
      {
        atomicExch(status, (int)DFX_ERR_NOT_IN_SPARSITY);
        continue;
      }
    }
    scatter_add<COLOURED>(vals + pos * (BS * BS) + k * BS + l, v);
  }
}

// Lifting with the constrained cells compacted inside the block. Only cells
// with a constrained dof contribute (fem/assemble_vector_impl.h:377-384 skips
// the others), and RCM order spreads them over the whole cell range, so a
// launch with one element-kernel thread per cell would run the FP64 element
// code in nearly every warp. Each block scans kLiftRange cells of the range
// (or of `list`), appends the constrained ones to a shared queue in scan
// order, and runs the element kernel on full batches of CPB queued cells.
constexpr int kLiftRange = 2048;

template <int DEG, bool ELAST, bool MASS, bool COLOURED>
__global__ void __launch_bounds__(kThreads)
    k_cells_lift(const dfx_form a, const int8_t* __restrict__ bc, const double* __restrict__ g,
                 const double* __restrict__ x0, double alpha, double* __restrict__ b,
                 const int32_t* __restrict__ list, int32_t count)
{
  using T = Traits<DEG, ELAST>;
  constexpr int ND = T::ND, BS = T::BS, N = T::N, NU = T::NU, CPB = T::CPB;
  constexpr int kWarps = kThreads / 32;
  __shared__ double sA[CPB * NU];
  __shared__ double sScratch[ELAST ? CPB * 132 : 1];
  __shared__ int32_t sCell[CPB];
  __shared__ int32_t sDof[CPB * ND];
  __shared__ int8_t sBc[CPB * N];
  __shared__ int8_t sActive[CPB];
  __shared__ int32_t sQueue[kThreads + CPB];
  __shared__ int32_t sWarpCount[kWarps];

  const int64_t begin = (int64_t)blockIdx.x * kLiftRange;
  const int64_t end = min((int64_t)count, begin + kLiftRange);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int queued = 0; // block-uniform
  for (int64_t c0 = begin; c0 < end; c0 += kThreads)
  {
    const int64_t idx = c0 + threadIdx.x;
    int32_t cell = 0;
    bool constrained = false;
    if (idx < end)
    {
      cell = list ? __ldg(list + idx) : (int32_t)idx;
      const int32_t* dofs = a.dofmap + (int64_t)cell * ND;
#pragma unroll
      for (int i = 0; i < ND; ++i)
      {
        const int64_t d = __ldg(dofs + i);
#pragma unroll
        for (int k = 0; k < BS; ++k)
          constrained |= __ldg(bc + BS * d + k) != 0;
      }
    }
    // Append in scan order: warp ballots, then warp offsets.
    const unsigned ballot = __ballot_sync(0xffffffffu, constrained);
    if (lane == 0)
      sWarpCount[warp] = __popc(ballot);
    __syncthreads();
    int off = queued;
    for (int w = 0; w < warp; ++w)
      off += sWarpCount[w];
    int added = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w)
      added += sWarpCount[w];
    if (constrained)
      sQueue[off + __popc(ballot & ((1u << lane) - 1u))] = cell;
    queued += added;
    __syncthreads();
    const bool last = c0 + kThreads >= end;
    while (queued >= CPB || (last && queued > 0))
    {
      const int nloc = queued < CPB ? queued : CPB;
      queued -= nloc;
      if (threadIdx.x < nloc)
      {
        sCell[threadIdx.x] = sQueue[queued + threadIdx.x];
        sActive[threadIdx.x] = 1;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < nloc * ND; t += blockDim.x)
      {
        const int cl = t / ND, i = t % ND;
        const int32_t d = __ldg(a.dofmap + (int64_t)sCell[cl] * ND + i);
        sDof[t] = d;
#pragma unroll
        for (int k = 0; k < BS; ++k)
          sBc[cl * N + BS * i + k] = __ldg(bc + (int64_t)BS * d + k);
      }
      __syncthreads();
      element_tensors<DEG, ELAST, MASS>(a, sCell, sActive, nloc, sA, sScratch);
      lift_rows<DEG, ELAST, COLOURED>(sA, sDof, sBc, sActive, nloc, g, x0, alpha, b);
      __syncthreads();
    }
  }
}

// Vector assembly: source (scalar, P1 coefficient f) or body force.
template <int DEG, bool BODY, bool COLOURED>
__global__ void __launch_bounds__(kThreads)
    k_cells_vector(const dfx_form a, double* __restrict__ b, const int32_t* __restrict__ list,
                   int32_t count)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count)
    return;
  const int64_t c = list ? __ldg(list + t) : t;
  double xc[12];
  load_cell_coords(a, c, xc);
  const double adet = tet_absdet(xc);
  const int32_t* dofs = a.dofmap + c * ND;
  if constexpr (!BODY)
  {
    double f[4];
    const int4 xd = __ldg(reinterpret_cast<const int4*>(a.x_dofmap) + c);
    if (a.f)
    {
      f[0] = __ldg(a.f + xd.x);
      f[1] = __ldg(a.f + xd.y);
      f[2] = __ldg(a.f + xd.z);
      f[3] = __ldg(a.f + xd.w);
    }
    else
      f[0] = f[1] = f[2] = f[3] = a.f_const[0];
    double be[ND];
    if constexpr (DEG == 1)
      tet_p1_source(f, adet, be);
    else
      tet_p2_source(f, adet, be);
#pragma unroll
    for (int i = 0; i < ND; ++i)
      scatter_add<COLOURED>(b + __ldg(dofs + i), be[i]);
  }
  else
  {
#pragma unroll
    for (int i = 0; i < ND; ++i)
    {
      const int64_t d = __ldg(dofs + i);
      const double w = adet * kTetP2Integral[i];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        scatter_add<COLOURED>(b + 3 * d + k, w * a.f_const[k]);
    }
  }
}

// Cell -> CSR slot map (byte offset of each entry within its row).
template <int ND>
__global__ void k_slot_map(const int32_t* __restrict__ dofmap, int32_t num_cells,
                           const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                           uint8_t* __restrict__ map, int* __restrict__ status)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)num_cells * ND * ND)
    return;
  const int64_t c = t / (ND * ND);
  const int ij = (int)(t % (ND * ND)), i = ij / ND, j = ij % ND;
  const int32_t di = __ldg(dofmap + c * ND + i), dj = __ldg(dofmap + c * ND + j);
  const int64_t rb = __ldg(row_ptr + di), re = __ldg(row_ptr + di + 1);
  const int64_t p = row_search(cols, rb, re, dj);
  if (p >= re || __ldg(cols + p) != dj)
  {
    atomicExch(status, (int)DFX_ERR_NOT_IN_SPARSITY);
    map[t] = 0;
    return;
  }
  if (p - rb > 255)
  {
    atomicExch(status, (int)DFX_ERR_UNSUPPORTED);
    map[t] = 0;
    return;
  }
  map[t] = (uint8_t)(p - rb);
}

__global__ void k_set_bc(double* __restrict__ x, int64_t n, const int32_t* __restrict__ dofs,
                         int32_t ndofs, const double* __restrict__ g, double g_const,
                         const double* __restrict__ x0, double alpha)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ndofs)
    return;
  const int32_t d = dofs[i];
  if (d < 0 || d >= n)
    return;
  if (alpha == 0.0)
  {
    x[d] = 0.0;
    return;
  }
  const double gv = g ? g[d] : g_const;
  x[d] = alpha * (gv - (x0 ? x0[d] : 0.0));
}

__global__ void k_set_diagonal(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                               double* __restrict__ vals, int bs, int32_t nrows,
                               const int32_t* __restrict__ dofs, int32_t ndofs, double diag,
                               int* __restrict__ status)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ndofs)
    return;
  const int32_t d = dofs[i], r = d / bs, k = d % bs;
  if (r < 0 || r >= nrows)
    return;
  const int64_t rb = row_ptr[r], re = row_ptr[r + 1];
  const int64_t p = row_search(cols, rb, re, r);
  if (p >= re || cols[p] != r)
  {
    atomicExch(status, (int)DFX_ERR_NOT_IN_SPARSITY);
    return;
  }
  vals[p * bs * bs + k * bs + k] = diag;
}

int check_form(const dfx_form* a, bool bilinear)
{
  DFX_REQUIRE(a, "form is NULL");
  DFX_REQUIRE(a->num_cells >= 0, "negative cell count");
  if (a->num_cells == 0)
    return DFX_OK;
  DFX_REQUIRE(a->x_dofmap && a->x && a->dofmap, "form arrays must be non-NULL");
  DFX_REQUIRE(((uintptr_t)a->x_dofmap & 15) == 0, "x_dofmap must be 16-byte aligned");
  if (bilinear)
  {
    DFX_REQUIRE(a->kind == DFX_FORM_POISSON || a->kind == DFX_FORM_ELASTICITY,
                "form kind %d is not a bilinear form", a->kind);
  }
  else
  {
    DFX_REQUIRE(a->kind == DFX_FORM_SOURCE || a->kind == DFX_FORM_BODYFORCE,
                "form kind %d is not a linear form", a->kind);
  }
  DFX_REQUIRE(a->degree == 1 || a->degree == 2, "degree %d not supported", a->degree);
  DFX_REQUIRE(!((a->kind == DFX_FORM_ELASTICITY || a->kind == DFX_FORM_BODYFORCE)
                && a->degree != 2),
              "vector forms are P2 only");
  return DFX_OK;
}

int form_nd(const dfx_form* a) { return a->degree == 1 ? 4 : 10; }
int form_bs(const dfx_form* a)
{
  return (a->kind == DFX_FORM_ELASTICITY || a->kind == DFX_FORM_BODYFORCE) ? 3 : 1;
}

int read_status(int* status, cudaStream_t s)
{
  int h = 0;
  DFX_CUDA(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  if (h == DFX_ERR_NOT_IN_SPARSITY)
    return dfx::fail(DFX_ERR_NOT_IN_SPARSITY, "Entry not in sparsity");
  if (h == DFX_ERR_UNSUPPORTED)
    return dfx::fail(DFX_ERR_UNSUPPORTED, "CSR row longer than 255 entries");
  return h;
}

// Cells per block: candidates of the autotuner and the default, per form.
// Scalar forms: 16, 32 (default) or 64 cells; elasticity (30 x 30 element
// tensors): 2, 4 (default) or 8.
constexpr int kCpbScalar[3] = {16, 32, 64};
constexpr int kCpbElast[3] = {2, 4, 8};

const int* cpb_candidates(const dfx_form& a)
{
  return a.kind == DFX_FORM_ELASTICITY ? kCpbElast : kCpbScalar;
}

int default_cpb(const dfx_form& a) { return cpb_candidates(a)[1]; }

bool valid_cpb(const dfx_form& a, int c)
{
  const int* k = cpb_candidates(a);
  return c == k[0] || c == k[1] || c == k[2];
}

// Autotuner key of a matrix assembly: form kind, degree, mass term, mode.
int64_t assembly_key(const dfx_form& a, int32_t mode)
{
  const int mass = a.kind == DFX_FORM_POISSON && a.k2 != 0.0;
  return (((int64_t)a.kind * 4 + a.degree) * 2 + mass) * 2 + mode;
}

int cells_per_block(const dfx_form& a, int32_t mode)
{
  const int t = dfx::tuned_get(dfx::kTuneAssembly, a.num_cells, assembly_key(a, mode), 0);
  return t ? t : default_cpb(a);
}

template <int DEG, bool ELAST, bool MASS, bool COLOURED, int CPB>
void launch_cells_cpb(const dfx_form& a, const dfx_csr* A, const uint8_t* map, const int8_t* bc,
                      const int32_t* list, int32_t count, int* status, cudaStream_t s)
{
  const unsigned grid = (unsigned)((count + CPB - 1) / CPB);
  k_cells_matrix<DEG, ELAST, MASS, COLOURED, CPB><<<grid, kThreads, 0, s>>>(
      a, A->row_ptr, A->cols, (double*)A->vals, map, bc, list, count, status);
}

// Launch the matrix kernel for one cell list with cpb cells per block.
template <int DEG, bool ELAST, bool MASS, bool COLOURED>
void launch_cells(const dfx_form& a, const dfx_csr* A, const uint8_t* map, const int8_t* bc,
                  const int32_t* list, int32_t count, int* status, int cpb, cudaStream_t s)
{
  if (count <= 0)
    return;
  if constexpr (ELAST)
  {
    if (cpb == 2)
      launch_cells_cpb<DEG, ELAST, MASS, COLOURED, 2>(a, A, map, bc, list, count, status, s);
    else if (cpb == 8)
      launch_cells_cpb<DEG, ELAST, MASS, COLOURED, 8>(a, A, map, bc, list, count, status, s);
    else
      launch_cells_cpb<DEG, ELAST, MASS, COLOURED, 4>(a, A, map, bc, list, count, status, s);
  }
  else
  {
    if (cpb == 16)
      launch_cells_cpb<DEG, ELAST, MASS, COLOURED, 16>(a, A, map, bc, list, count, status, s);
    else if (cpb == 64)
      launch_cells_cpb<DEG, ELAST, MASS, COLOURED, 64>(a, A, map, bc, list, count, status, s);
    else
      launch_cells_cpb<DEG, ELAST, MASS, COLOURED, 32>(a, A, map, bc, list, count, status, s);
  }
}

template <bool COLOURED>
void dispatch_cells(const dfx_form& a, const dfx_csr* A, const uint8_t* map, const int8_t* bc,
                    const int32_t* list, int32_t count, int* status, int cpb, cudaStream_t s)
{
  const bool mass = a.kind == DFX_FORM_POISSON && a.k2 != 0.0;
  if (a.kind == DFX_FORM_ELASTICITY)
    launch_cells<2, true, false, COLOURED>(a, A, map, bc, list, count, status, cpb, s);
  else if (a.degree == 1)
  {
    if (mass)
      launch_cells<1, false, true, COLOURED>(a, A, map, bc, list, count, status, cpb, s);
    else
      launch_cells<1, false, false, COLOURED>(a, A, map, bc, list, count, status, cpb, s);
  }
  else
  {
    if (mass)
      launch_cells<2, false, true, COLOURED>(a, A, map, bc, list, count, status, cpb, s);
    else
      launch_cells<2, false, false, COLOURED>(a, A, map, bc, list, count, status, cpb, s);
  }
}

template <int DEG, bool ELAST, bool MASS, bool COLOURED>
void launch_lift(const dfx_form& a, const int8_t* bc, const double* g, const double* x0,
                 double alpha, double* b, const int32_t* list, int32_t count, cudaStream_t s)
{
  if (count <= 0)
    return;
  const unsigned grid = (unsigned)((count + kLiftRange - 1) / kLiftRange);
  k_cells_lift<DEG, ELAST, MASS, COLOURED><<<grid, kThreads, 0, s>>>(a, bc, g, x0, alpha, b, list,
                                                                    count);
}

template <bool COLOURED>
void dispatch_lift(const dfx_form& a, const int8_t* bc, const double* g, const double* x0,
                   double alpha, double* b, const int32_t* list, int32_t count, cudaStream_t s)
{
  const bool mass = a.kind == DFX_FORM_POISSON && a.k2 != 0.0;
  if (a.kind == DFX_FORM_ELASTICITY)
    launch_lift<2, true, false, COLOURED>(a, bc, g, x0, alpha, b, list, count, s);
  else if (a.degree == 1)
  {
    if (mass)
      launch_lift<1, false, true, COLOURED>(a, bc, g, x0, alpha, b, list, count, s);
    else
      launch_lift<1, false, false, COLOURED>(a, bc, g, x0, alpha, b, list, count, s);
  }
  else
  {
    if (mass)
      launch_lift<2, false, true, COLOURED>(a, bc, g, x0, alpha, b, list, count, s);
    else
      launch_lift<2, false, false, COLOURED>(a, bc, g, x0, alpha, b, list, count, s);
  }
}

} // namespace

extern "C" size_t dfx_slot_map_bytes(const dfx_form* a)
{
  if (!a)
    return 0;
  const int nd = form_nd(a);
  return (size_t)a->num_cells * nd * nd;
}

extern "C" int dfx_slot_map_create(const dfx_form* a, const dfx_csr* A, uint8_t* d_map,
                                   void* stream)
{
  if (int st = check_form(a, true))
    return st;
  DFX_REQUIRE(A && A->row_ptr && A->cols && d_map, "matrix/map must be non-NULL");
  if (a->num_cells == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  const int nd = form_nd(a);
  const int64_t n = (int64_t)a->num_cells * nd * nd;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (nd == 4)
    k_slot_map<4><<<grid, 256, 0, s>>>(a->dofmap, a->num_cells, A->row_ptr, A->cols, d_map, status);
  else
    k_slot_map<10><<<grid, 256, 0, s>>>(a->dofmap, a->num_cells, A->row_ptr, A->cols, d_map,
                                        status);
  DFX_CHECK_LAUNCH();
  return read_status(status, s);
}

namespace
{
// dfx_assemble_matrix with cpb cells per block (arguments checked).
int assemble_matrix_cpb(const dfx_form* a, const dfx_csr* A, const uint8_t* d_map,
                        const int8_t* d_bc, int32_t mode, const int32_t* d_order,
                        const int32_t* colour_offsets, int32_t num_colours, int cpb,
                        cudaStream_t s)
{
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  if (!d_map)
    DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  if (mode == DFX_MODE_ATOMIC)
    dispatch_cells<false>(*a, A, d_map, d_bc, nullptr, a->num_cells, status, cpb, s);
  else if (mode == DFX_MODE_COLOURED)
  {
    DFX_REQUIRE(d_order && colour_offsets && num_colours > 0, "coloured mode needs a colouring");
    for (int k = 0; k < num_colours; ++k)
      dispatch_cells<true>(*a, A, d_map, d_bc, d_order + colour_offsets[k],
                           colour_offsets[k + 1] - colour_offsets[k], status, cpb, s);
  }
  else
    return dfx::fail(DFX_ERR_INVALID, "unknown assembly mode %d", mode);
  DFX_CHECK_LAUNCH();
  if (!d_map)
    return read_status(status, s);
  return DFX_OK;
}

int check_matrix_args(const dfx_form* a, const dfx_csr* A)
{
  if (int st = check_form(a, true))
    return st;
  DFX_REQUIRE(A && A->row_ptr && A->cols && A->vals, "matrix must be non-NULL");
  DFX_REQUIRE(A->dtype == DFX_F64, "assembly writes FP64 values");
  DFX_REQUIRE(A->bs == form_bs(a), "matrix block size %d does not match the form (%d)", A->bs,
              form_bs(a));
  return DFX_OK;
}
} // namespace

extern "C" int dfx_assemble_matrix(const dfx_form* a, const dfx_csr* A, const uint8_t* d_map,
                                   const int8_t* d_bc, int32_t mode, const int32_t* d_order,
                                   const int32_t* colour_offsets, int32_t num_colours,
                                   void* stream)
{
  if (int st = check_matrix_args(a, A))
    return st;
  if (a->num_cells == 0)
    return DFX_OK;
  return assemble_matrix_cpb(a, A, d_map, d_bc, mode, d_order, colour_offsets, num_colours,
                             cells_per_block(*a, mode), dfx::as_stream(stream));
}

extern "C" int dfx_tune_assembly(const dfx_form* a, const dfx_csr* A, const uint8_t* d_map,
                                 const int8_t* d_bc, int32_t mode, const int32_t* d_order,
                                 const int32_t* colour_offsets, int32_t num_colours,
                                 double* d_scratch_vals, int32_t* best, float* ms, void* stream)
{
  if (int st = check_matrix_args(a, A))
    return st;
  DFX_REQUIRE(d_scratch_vals && best, "scratch values and best must be non-NULL");
  DFX_REQUIRE(mode == DFX_MODE_ATOMIC || mode == DFX_MODE_COLOURED, "unknown assembly mode %d",
              mode);
  cudaStream_t s = dfx::as_stream(stream);
  dfx_csr scratch = *A;
  scratch.vals = d_scratch_vals; // the candidates accumulate here, not into A
  const int* cand = cpb_candidates(*a);
  constexpr int kReps = 3;
  cudaEvent_t e0, e1;
  DFX_CUDA(cudaEventCreate(&e0));
  DFX_CUDA(cudaEventCreate(&e1));
  int pick = 0;
  float pick_ms = 0.0f;
  int st = DFX_OK;
  for (int c = 0; c < 3 && !st; ++c)
  {
    st = assemble_matrix_cpb(a, &scratch, d_map, d_bc, mode, d_order, colour_offsets,
                             num_colours, cand[c], s); // warm-up
    if (!st && cudaEventRecord(e0, s) != cudaSuccess)
      st = dfx::fail(DFX_ERR_CUDA, "event record failed");
    for (int r = 0; r < kReps && !st; ++r)
      st = assemble_matrix_cpb(a, &scratch, d_map, d_bc, mode, d_order, colour_offsets,
                               num_colours, cand[c], s);
    float t = 0.0f;
    if (!st && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess
                || cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
      st = dfx::fail(DFX_ERR_CUDA, "assembly timing failed");
    t /= kReps;
    if (ms)
      ms[c] = t;
    if (!st && (pick == 0 || t < pick_ms))
    {
      pick = cand[c];
      pick_ms = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st)
    return st;
  dfx::tuned_set(dfx::kTuneAssembly, a->num_cells, assembly_key(*a, mode), 0, pick);
  *best = pick;
  return DFX_OK;
}

extern "C" int dfx_set_cells_per_block(const dfx_form* a, int32_t mode, int32_t cpb)
{
  if (int st = check_form(a, true))
    return st;
  DFX_REQUIRE(cpb == 0 || valid_cpb(*a, cpb),
              "cells per block %d is not a candidate for this form", cpb);
  dfx::tuned_set(dfx::kTuneAssembly, a->num_cells, assembly_key(*a, mode), 0, cpb);
  return DFX_OK;
}

extern "C" int dfx_get_cells_per_block(const dfx_form* a, int32_t mode, int32_t* cpb)
{
  if (int st = check_form(a, true))
    return st;
  DFX_REQUIRE(cpb, "cpb must be non-NULL");
  *cpb = cells_per_block(*a, mode);
  return DFX_OK;
}

extern "C" int dfx_apply_lifting(const dfx_form* a, double* d_b, const int8_t* d_bc,
                                 const double* d_g, const double* d_x0, double alpha, int32_t mode,
                                 const int32_t* d_order, const int32_t* colour_offsets,
                                 int32_t num_colours, void* stream)
{
  if (int st = check_form(a, true))
    return st;
  DFX_REQUIRE(d_b && d_bc && d_g, "b, bc markers and g must be non-NULL");
  if (a->num_cells == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  if (mode == DFX_MODE_ATOMIC)
    dispatch_lift<false>(*a, d_bc, d_g, d_x0, alpha, d_b, nullptr, a->num_cells, s);
  else if (mode == DFX_MODE_COLOURED)
  {
    DFX_REQUIRE(d_order && colour_offsets && num_colours > 0, "coloured mode needs a colouring");
    for (int k = 0; k < num_colours; ++k)
      dispatch_lift<true>(*a, d_bc, d_g, d_x0, alpha, d_b, d_order + colour_offsets[k],
                          colour_offsets[k + 1] - colour_offsets[k], s);
  }
  else
    return dfx::fail(DFX_ERR_INVALID, "unknown assembly mode %d", mode);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_assemble_vector(const dfx_form* L, double* d_b, int32_t mode,
                                   const int32_t* d_order, const int32_t* colour_offsets,
                                   int32_t num_colours, void* stream)
{
  if (int st = check_form(L, false))
    return st;
  DFX_REQUIRE(d_b, "b must be non-NULL");
  if (L->num_cells == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  auto launch = [&](auto coloured, const int32_t* list, int32_t count)
  {
    constexpr bool C = decltype(coloured)::value;
    if (count <= 0)
      return;
    const unsigned grid = (unsigned)((count + kThreads - 1) / kThreads);
    if (L->kind == DFX_FORM_BODYFORCE)
      k_cells_vector<2, true, C><<<grid, kThreads, 0, s>>>(*L, d_b, list, count);
    else if (L->degree == 1)
      k_cells_vector<1, false, C><<<grid, kThreads, 0, s>>>(*L, d_b, list, count);
    else
      k_cells_vector<2, false, C><<<grid, kThreads, 0, s>>>(*L, d_b, list, count);
  };
  if (mode == DFX_MODE_ATOMIC)
    launch(std::false_type{}, nullptr, L->num_cells);
  else if (mode == DFX_MODE_COLOURED)
  {
    DFX_REQUIRE(d_order && colour_offsets && num_colours > 0, "coloured mode needs a colouring");
    for (int k = 0; k < num_colours; ++k)
      launch(std::true_type{}, d_order + colour_offsets[k],
             colour_offsets[k + 1] - colour_offsets[k]);
  }
  else
    return dfx::fail(DFX_ERR_INVALID, "unknown assembly mode %d", mode);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_set_bc(double* d_x, int64_t n, const int32_t* d_dofs, int32_t ndofs,
                          const double* d_g, double g_const, const double* d_x0, double alpha,
                          void* stream)
{
  DFX_REQUIRE(ndofs >= 0, "negative dof count");
  if (ndofs == 0)
    return DFX_OK;
  DFX_REQUIRE(d_x && d_dofs, "x and dofs must be non-NULL");
  k_set_bc<<<(ndofs + 255) / 256, 256, 0, dfx::as_stream(stream)>>>(d_x, n, d_dofs, ndofs, d_g,
                                                                    g_const, d_x0, alpha);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_set_diagonal(const dfx_csr* A, const int32_t* d_dofs, int32_t ndofs,
                                double diagonal, void* stream)
{
  DFX_REQUIRE(A && A->row_ptr && A->cols && A->vals, "matrix must be non-NULL");
  DFX_REQUIRE(A->dtype == DFX_F64, "set_diagonal writes FP64 values");
  if (ndofs == 0)
    return DFX_OK;
  DFX_REQUIRE(d_dofs && ndofs > 0, "dofs must be non-NULL");
  cudaStream_t s = dfx::as_stream(stream);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  k_set_diagonal<<<(ndofs + 255) / 256, 256, 0, s>>>(A->row_ptr, A->cols, (double*)A->vals, A->bs,
                                                     A->nrows, d_dofs, ndofs, diagonal, status);
  DFX_CHECK_LAUNCH();
  return read_status(status, s);
}

// ------------------------------------------------------------------------
// Exterior facet integrals and functionals.
//
// An exterior-facet domain is a list of (cell, local facet) pairs, facet f
// of a tetrahedron being the triangle opposite its vertex f (Basix
// numbering; fem/utils.h:155-162). The integrals use the exact P1/P2
// triangle integrals of area A (products of barycentrics,
// \int l0^a l1^b l2^c = 2A a! b! c! / (a+b+c+2)!), one thread per facet and
// FP64 atomics into the caller's vector or CSR values.
// ------------------------------------------------------------------------
namespace
{
// Local vertices of facet f, and the local P2 edge opposite each of them
// inside the facet (the edge joining the other two; edges in Basix order).
__constant__ int kFacetVerts[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
__constant__ int kFacetEdges[4][3] = {{0, 1, 2}, {0, 3, 4}, {1, 3, 5}, {2, 4, 5}};

// Facet vertices' coordinates (3 x 3) and area.
__device__ __forceinline__ double facet_geometry(const dfx_form& a, int32_t c, int f, int* lv,
                                                 int32_t* gnode)
{
  const int4 xd = __ldg(reinterpret_cast<const int4*>(a.x_dofmap) + c);
  const int32_t nodes[4] = {xd.x, xd.y, xd.z, xd.w};
  double p[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    lv[k] = kFacetVerts[f][k];
    gnode[k] = nodes[lv[k]];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      p[k][d] = __ldg(a.x + 3 * (int64_t)gnode[k] + d);
  }
  const double u[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
  const double v[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
  const double n0 = u[1] * v[2] - u[2] * v[1];
  const double n1 = u[2] * v[0] - u[0] * v[2];
  const double n2 = u[0] * v[1] - u[1] * v[0];
  return 0.5 * sqrt(n0 * n0 + n1 * n1 + n2 * n2);
}

// b += \int_F g v ds, g a P1 coefficient (per geometry node, or g_const):
// P1: A/12 (g_i + S); P2 vertex: A/60 (3 g_i - S); P2 edge opposite
// vertex i: A/15 (2 S - g_i), S = g_0 + g_1 + g_2.
template <int DEG>
__global__ void k_facets_vector(const dfx_form a, const int32_t* __restrict__ facets,
                                int32_t nf, double* __restrict__ b)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf)
    return;
  const int2 cf = __ldg(reinterpret_cast<const int2*>(facets) + t);
  int lv[3];
  int32_t gn[3];
  const double A = facet_geometry(a, cf.x, cf.y, lv, gn);
  double g[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    g[k] = a.f ? __ldg(a.f + gn[k]) : a.f_const[0];
  const double S = g[0] + g[1] + g[2];
  const int32_t* dofs = a.dofmap + (int64_t)ND * cf.x;
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    const double vk = DEG == 1 ? A / 12.0 * (g[k] + S) : A / 60.0 * (3.0 * g[k] - S);
    atomicAdd(b + __ldg(dofs + lv[k]), vk);
    if (DEG == 2)
      atomicAdd(b + __ldg(dofs + 4 + kFacetEdges[cf.y][k]), A / 15.0 * (2.0 * S - g[k]));
  }
}

// A += \int_F alpha u v ds (alpha per cell or constant) through the cell
// slot map; constrained rows and columns are skipped
// (fem/assemble_matrix_impl.h:265-379). Facet mass in units of A: P1
// (1 + delta_ij)/12; P2 (vertices, then the edge opposite each vertex)
// 1/180 x {6 diagonal, -1 vertex-vertex, -4 vertex-opposite edge, 0
// vertex-adjacent edge, 32 edge diagonal, 16 edge-edge}.
template <int DEG>
__global__ void k_facets_matrix(const dfx_form a, const int32_t* __restrict__ facets,
                                int32_t nf, const int64_t* __restrict__ row_ptr,
                                const int32_t* __restrict__ cols, double* __restrict__ vals,
                                const uint8_t* __restrict__ map, const int8_t* __restrict__ bc,
                                int* __restrict__ status)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  constexpr int NF = DEG == 1 ? 3 : 6; // facet dofs
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf)
    return;
  const int2 cf = __ldg(reinterpret_cast<const int2*>(facets) + t);
  int lv[3];
  int32_t gn[3];
  const double A = facet_geometry(a, cf.x, cf.y, lv, gn);
  const double s = (a.kappa ? __ldg(a.kappa + cf.x) : a.kappa_const) * A;
  int loc[NF];
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    loc[k] = lv[k];
    if (DEG == 2)
      loc[3 + k] = 4 + kFacetEdges[cf.y][k];
  }
  const int32_t* dofs = a.dofmap + (int64_t)ND * cf.x;
  for (int i = 0; i < NF; ++i)
  {
    const int32_t di = __ldg(dofs + loc[i]);
    if (bc && __ldg(bc + di))
      continue;
    const int64_t rb = __ldg(row_ptr + di);
    for (int j = 0; j < NF; ++j)
    {
      const int32_t dj = __ldg(dofs + loc[j]);
      if (bc && __ldg(bc + dj))
        continue;
      double m;
      if (DEG == 1)
        m = (i == j ? 2.0 : 1.0) / 12.0;
      else
      {
        const bool vi = i < 3, vj = j < 3;
        const int ii = i % 3, jj = j % 3;
        if (vi && vj)
          m = i == j ? 6.0 : -1.0;
        else if (!vi && !vj)
          m = i == j ? 32.0 : 16.0;
        else
          m = ii == jj ? -4.0 : 0.0;
        m /= 180.0;
      }
      int64_t pos;
      if (map)
        pos = rb + map[((int64_t)cf.x * ND + loc[i]) * ND + loc[j]];
      else
      {
        const int64_t re = __ldg(row_ptr + di + 1);
        pos = row_search(cols, rb, re, dj);
        if (pos >= re || __ldg(cols + pos) != dj)
        {
          atomicExch(status, (int)DFX_ERR_NOT_IN_SPARSITY);
          continue;
        }
      }
      atomicAdd(vals + pos, s * m);
    }
  }
}

// ------------------------------------------------------------------------
// Interior facet integrals (fem/assemble_vector_impl.h:252-360,
// fem/assemble_matrix_impl.h:443-667). The domain is a list of
// (cell0, local facet0, cell1, local facet1) quads; the element tensor of a
// facet lives on the macro element of both cells, dofs of cell0 then dofs
// of cell1, and is scattered with FP64 atomics.
//   vector: L(v) = \int_F avg(g) avg(v) dS, g a P1 coefficient -- each side
//           adds half of the exterior-facet formula on its own local facet;
//   matrix: a(u,v) = \int_F gamma |F| [grad u . n][grad v . n] dS, the
//           continuous interior penalty (gradient-jump) term, gamma the
//           average of the two cells' coefficients. The jumps are linear on
//           F (P2) and their product is integrated exactly by the
//           edge-midpoint rule; P1 gradients are constant.
// ------------------------------------------------------------------------

// Vertex coordinates (4 x 3) of cell c, its global geometry nodes, and the
// gradients of its barycentric coordinates (rows of J^{-1}; lambda_0 =
// 1 - lambda_1 - lambda_2 - lambda_3).
__device__ __forceinline__ void cell_barycentric_gradients(const dfx_form& a, int32_t c,
                                                           int32_t* node, double (*p)[3],
                                                           double (*g)[3])
{
  const int4 xd = __ldg(reinterpret_cast<const int4*>(a.x_dofmap) + c);
  node[0] = xd.x;
  node[1] = xd.y;
  node[2] = xd.z;
  node[3] = xd.w;
#pragma unroll
  for (int v = 0; v < 4; ++v)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      p[v][d] = __ldg(a.x + 3 * (int64_t)node[v] + d);
  double J[3][3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      J[d][k] = p[k + 1][d] - p[0][d];
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double id = 1.0 / det;
  // K = J^{-1}: row k is grad lambda_{k+1}.
  g[1][0] = c00 * id;
  g[1][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  g[1][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  g[2][0] = c01 * id;
  g[2][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  g[2][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  g[3][0] = c02 * id;
  g[3][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  g[3][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    g[0][d] = -(g[1][d] + g[2][d] + g[3][d]);
}

// Basix P2 edge k of the tetrahedron joins local vertices kEdgeV[k].
__constant__ int kEdgeV[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};

// The CIP macro-element tensor of one interior facet: jumps j[q][i] of the
// normal derivative of macro basis function i (cell0's nd, then cell1's)
// at the facet's quadrature points, and the weight w of each point.
template <int DEG>
struct CipFacet
{
  static constexpr int ND = DEG == 1 ? 4 : 10;
  static constexpr int NQ = DEG == 1 ? 1 : 3;
  double j[NQ][2 * ND];
  double w; // gamma |F| times the rule's weight |F| / NQ
  int32_t c[2];
};

template <int DEG>
__device__ void cip_facet(const dfx_form& a, int4 q, CipFacet<DEG>& out)
{
  constexpr int ND = CipFacet<DEG>::ND;
  const int32_t cell[2] = {q.x, q.z};
  const int lf[2] = {q.y, q.w};
  int32_t node[2][4];
  double p[2][4][3], g[2][4][3];
#pragma unroll
  for (int s = 0; s < 2; ++s)
    cell_barycentric_gradients(a, cell[s], node[s], p[s], g[s]);
  // Facet vertices (cell0's numbering), area and unit normal out of cell0.
  int fv[3];
  {
    int k = 0;
#pragma unroll
    for (int v = 0; v < 4; ++v)
      if (v != lf[0])
        fv[k++] = v;
  }
  const double* A0 = p[0][fv[0]];
  const double* B0 = p[0][fv[1]];
  const double* C0 = p[0][fv[2]];
  const double u[3] = {B0[0] - A0[0], B0[1] - A0[1], B0[2] - A0[2]};
  const double v[3] = {C0[0] - A0[0], C0[1] - A0[1], C0[2] - A0[2]};
  double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                 u[0] * v[1] - u[1] * v[0]};
  const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const double area = 0.5 * nn;
  const double* opp = p[0][lf[0]];
  const double side = n[0] * (opp[0] - A0[0]) + n[1] * (opp[1] - A0[1]) + n[2] * (opp[2] - A0[2]);
  const double sgn = (side > 0 ? -1.0 : 1.0) / nn;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    n[d] *= sgn;
  const double k0 = a.kappa ? __ldg(a.kappa + cell[0]) : a.kappa_const;
  const double k1 = a.kappa ? __ldg(a.kappa + cell[1]) : a.kappa_const;
  out.w = 0.5 * (k0 + k1) * area * area / CipFacet<DEG>::NQ;
  out.c[0] = cell[0];
  out.c[1] = cell[1];
  // grad lambda . n per cell and vertex; the jump takes cell1 with a minus.
  double gn[2][4];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int vv = 0; vv < 4; ++vv)
      gn[s][vv] = (s == 0 ? 1.0 : -1.0)
                  * (g[s][vv][0] * n[0] + g[s][vv][1] * n[1] + g[s][vv][2] * n[2]);
  if constexpr (DEG == 1)
  {
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int vv = 0; vv < 4; ++vv)
        out.j[0][s * ND + vv] = gn[s][vv];
    return;
  }
  else
  {
    // Quadrature point m: midpoint of the facet edge opposite facet vertex
    // m (global nodes a_m, b_m); barycentrics 1/2 at those two vertices.
#pragma unroll
    for (int m = 0; m < 3; ++m)
    {
      const int32_t na = node[0][fv[(m + 1) % 3]], nb = node[0][fv[(m + 2) % 3]];
#pragma unroll
      for (int s = 0; s < 2; ++s)
      {
        double lam[4];
#pragma unroll
        for (int vv = 0; vv < 4; ++vv)
          lam[vv] = (node[s][vv] == na || node[s][vv] == nb) ? 0.5 : 0.0;
        // vertex functions lambda (2 lambda - 1): gradient (4 lambda - 1) grad lambda
#pragma unroll
        for (int vv = 0; vv < 4; ++vv)
          out.j[m][s * ND + vv] = (4.0 * lam[vv] - 1.0) * gn[s][vv];
        // edge functions 4 lambda_a lambda_b
#pragma unroll
        for (int e = 0; e < 6; ++e)
        {
          const int ea = kEdgeV[e][0], eb = kEdgeV[e][1];
          out.j[m][s * ND + 4 + e] = 4.0 * (lam[ea] * gn[s][eb] + lam[eb] * gn[s][ea]);
        }
      }
    }
  }
}

template <int DEG>
__global__ void k_interior_facets_vector(const dfx_form a, const int4* __restrict__ quads,
                                         int32_t nf, double* __restrict__ b)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf)
    return;
  const int4 q = __ldg(quads + t);
  const int32_t cs[2] = {q.x, q.z};
  const int fs[2] = {q.y, q.w};
#pragma unroll
  for (int s = 0; s < 2; ++s)
  {
    int lv[3];
    int32_t gn[3];
    const double A = 0.5 * facet_geometry(a, cs[s], fs[s], lv, gn); // avg(v): half per side
    double g[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      g[k] = a.f ? __ldg(a.f + gn[k]) : a.f_const[0];
    const double S = g[0] + g[1] + g[2];
    const int32_t* dofs = a.dofmap + (int64_t)ND * cs[s];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
      const double vk = DEG == 1 ? A / 12.0 * (g[k] + S) : A / 60.0 * (3.0 * g[k] - S);
      atomicAdd(b + __ldg(dofs + lv[k]), vk);
      if (DEG == 2)
        atomicAdd(b + __ldg(dofs + 4 + kFacetEdges[fs[s]][k]), A / 15.0 * (2.0 * S - g[k]));
    }
  }
}

// A += the CIP macro tensor; rows and columns of constrained dofs skipped
// (as the cell loop zeroes them); insertion by binary search in the rows
// (the pattern must hold the facet couplings).
template <int DEG>
__global__ void k_interior_facets_matrix(const dfx_form a, const int4* __restrict__ quads,
                                         int32_t nf, const int64_t* __restrict__ row_ptr,
                                         const int32_t* __restrict__ cols,
                                         double* __restrict__ vals,
                                         const int8_t* __restrict__ bc, int* __restrict__ status)
{
  constexpr int ND = CipFacet<DEG>::ND, NQ = CipFacet<DEG>::NQ;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf)
    return;
  CipFacet<DEG> F;
  cip_facet<DEG>(a, __ldg(quads + t), F);
  for (int i = 0; i < 2 * ND; ++i)
  {
    const int32_t di = __ldg(a.dofmap + (int64_t)ND * F.c[i / ND] + i % ND);
    if (bc && __ldg(bc + di))
      continue;
    const int64_t rb = __ldg(row_ptr + di), re = __ldg(row_ptr + di + 1);
    for (int k = 0; k < 2 * ND; ++k)
    {
      const int32_t dk = __ldg(a.dofmap + (int64_t)ND * F.c[k / ND] + k % ND);
      if (bc && __ldg(bc + dk))
        continue;
      double v = 0.0;
#pragma unroll
      for (int m = 0; m < NQ; ++m)
        v += F.j[m][i] * F.j[m][k];
      const int64_t pos = row_search(cols, rb, re, dk);
      if (pos >= re || __ldg(cols + pos) != dk)
      {
        atomicExch(status, (int)DFX_ERR_NOT_IN_SPARSITY);
        continue;
      }
      atomicAdd(vals + pos, F.w * v);
    }
  }
}

// Lifting of facet integrals (lift_bc over facets, fem/assemble_vector_impl.h:
// 363-414, through assemble_matrix<true> on the facet domains): b[r] -=
// alpha sum_c A_F[r, c] (g_c - x0_c) over the constrained columns c of
// each facet's (macro) element tensor. Exterior facets: the facet mass of
// DFX_FORM_FACET_MASS; interior facets: the CIP term.
template <int DEG>
__global__ void k_lift_exterior_facets(const dfx_form a, const int2* __restrict__ pairs,
                                       int32_t nf, const int8_t* __restrict__ bc,
                                       const double* __restrict__ g,
                                       const double* __restrict__ x0, double alpha,
                                       double* __restrict__ b)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  constexpr int NF = DEG == 1 ? 3 : 6;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf)
    return;
  const int2 cf = __ldg(pairs + t);
  int lv[3];
  int32_t gnode[3];
  const double A = facet_geometry(a, cf.x, cf.y, lv, gnode);
  const double sc = (a.kappa ? __ldg(a.kappa + cf.x) : a.kappa_const) * A;
  int loc[NF];
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    loc[k] = lv[k];
    if (DEG == 2)
      loc[3 + k] = 4 + kFacetEdges[cf.y][k];
  }
  const int32_t* dofs = a.dofmap + (int64_t)ND * cf.x;
  for (int j = 0; j < NF; ++j)
  {
    const int32_t dj = __ldg(dofs + loc[j]);
    if (!__ldg(bc + dj))
      continue;
    const double gj = alpha * (__ldg(g + dj) - (x0 ? __ldg(x0 + dj) : 0.0));
    for (int i = 0; i < NF; ++i)
    {
      double m;
      if (DEG == 1)
        m = (i == j ? 2.0 : 1.0) / 12.0;
      else
      {
        const bool vi = i < 3, vj = j < 3;
        if (vi && vj)
          m = i == j ? 6.0 : -1.0;
        else if (!vi && !vj)
          m = i == j ? 32.0 : 16.0;
        else
          m = i % 3 == j % 3 ? -4.0 : 0.0;
        m /= 180.0;
      }
      atomicAdd(b + __ldg(dofs + loc[i]), -sc * m * gj);
    }
  }
}

template <int DEG>
__global__ void k_lift_interior_facets(const dfx_form a, const int4* __restrict__ quads,
                                       int32_t nf, const int8_t* __restrict__ bc,
                                       const double* __restrict__ g,
                                       const double* __restrict__ x0, double alpha,
                                       double* __restrict__ b)
{
  constexpr int ND = CipFacet<DEG>::ND, NQ = CipFacet<DEG>::NQ;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf)
    return;
  const int4 q = __ldg(quads + t);
  // Only facets with a constrained macro dof do work.
  bool any = false;
  for (int k = 0; k < 2 * ND && !any; ++k)
    any = __ldg(bc + __ldg(a.dofmap + (int64_t)ND * (k < ND ? q.x : q.z) + k % ND)) != 0;
  if (!any)
    return;
  CipFacet<DEG> F;
  cip_facet<DEG>(a, q, F);
  for (int k = 0; k < 2 * ND; ++k)
  {
    const int32_t dk = __ldg(a.dofmap + (int64_t)ND * F.c[k / ND] + k % ND);
    if (!__ldg(bc + dk))
      continue;
    const double gk = alpha * (__ldg(g + dk) - (x0 ? __ldg(x0 + dk) : 0.0));
    for (int i = 0; i < 2 * ND; ++i)
    {
      double v = 0.0;
#pragma unroll
      for (int m = 0; m < NQ; ++m)
        v += F.j[m][i] * F.j[m][k];
      atomicAdd(b + __ldg(a.dofmap + (int64_t)ND * F.c[i / ND] + i % ND), -F.w * v * gk);
    }
  }
}

// Functional cell loop (fem/assemble_scalar_impl.h:32-61): per cell
// a(u_e, u_e) with the Poisson/Helmholtz element tensor, or L(u_e) with the
// P1-source element vector; block partial sums in FP64, each block's
// warps summed in a fixed order.
template <int DEG, bool SOURCE, bool MASS>
__global__ void __launch_bounds__(kThreads)
    k_cells_scalar(const dfx_form a, const double* __restrict__ u, double* __restrict__ part)
{
  constexpr int ND = DEG == 1 ? 4 : 10;
  constexpr int NU = ND * (ND + 1) / 2;
  __shared__ double sh[kThreads / 32];
  double v = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * kThreads + threadIdx.x; c < a.num_cells;
       c += (int64_t)gridDim.x * kThreads)
  {
    double xc[12];
    load_cell_coords(a, c, xc);
    double ue[ND];
#pragma unroll
    for (int i = 0; i < ND; ++i)
      ue[i] = __ldg(u + __ldg(a.dofmap + c * ND + i));
    if constexpr (SOURCE)
    {
      double f[4];
      const int4 xd = __ldg(reinterpret_cast<const int4*>(a.x_dofmap) + c);
      if (a.f)
      {
        f[0] = __ldg(a.f + xd.x);
        f[1] = __ldg(a.f + xd.y);
        f[2] = __ldg(a.f + xd.z);
        f[3] = __ldg(a.f + xd.w);
      }
      else
        f[0] = f[1] = f[2] = f[3] = a.f_const[0];
      double be[ND];
      const double adet = tet_absdet(xc);
      if constexpr (DEG == 1)
        tet_p1_source(f, adet, be);
      else
        tet_p2_source(f, adet, be);
#pragma unroll
      for (int i = 0; i < ND; ++i)
        v += be[i] * ue[i];
    }
    else
    {
      const double kap = a.kappa ? __ldg(a.kappa + c) : a.kappa_const;
      double G[6];
      const double adet = tet_metric(xc, kap, G);
      double Ae[NU];
      if constexpr (DEG == 1)
        tet_p1_poisson_upper<MASS>(G, a.k2 * adet, Ae);
      else
        tet_p2_poisson_upper<MASS>(G, a.k2 * adet, Ae);
#pragma unroll
      for (int i = 0; i < ND; ++i)
      {
        double r = 0.0;
#pragma unroll
        for (int j = i + 1; j < ND; ++j)
          r += Ae[packed(i, j, ND)] * ue[j];
        v += ue[i] * (Ae[packed(i, i, ND)] * ue[i] + 2.0 * r);
      }
    }
  }
  v = dfx::warp_sum(v);
  if ((threadIdx.x & 31) == 0)
    sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; ++w)
      s += sh[w];
    part[blockIdx.x] = s;
  }
}

// Sum of the block partials in index order (one thread: a few thousand
// values at most).
__global__ void k_sum_partials(const double* __restrict__ part, int n, double* __restrict__ out)
{
  if (threadIdx.x == 0 && blockIdx.x == 0)
  {
    double s = 0.0;
    for (int i = 0; i < n; ++i)
      s += part[i];
    *out = s;
  }
}

int scalar_blocks(int32_t num_cells)
{
  const int need = (num_cells + kThreads - 1) / kThreads;
  return std::max(1, std::min(need, 8 * dfx::num_sms()));
}

int check_facet_form(const dfx_form* a, int32_t kind, const int32_t* d_facets, int32_t nf)
{
  DFX_REQUIRE(a, "form is NULL");
  DFX_REQUIRE(a->kind == kind, "form kind %d is not %d", a->kind, kind);
  DFX_REQUIRE(a->degree == 1 || a->degree == 2, "degree %d not supported", a->degree);
  DFX_REQUIRE(nf >= 0, "negative facet count");
  DFX_REQUIRE(nf == 0 || (d_facets && a->x_dofmap && a->x && a->dofmap),
              "facets and form arrays must be non-NULL");
  DFX_REQUIRE(((uintptr_t)d_facets & 7) == 0, "facets must be 8-byte aligned");
  DFX_REQUIRE(((uintptr_t)a->x_dofmap & 15) == 0, "x_dofmap must be 16-byte aligned");
  return DFX_OK;
}
} // namespace

extern "C" int dfx_assemble_vector_facets(const dfx_form* L, const int32_t* d_facets,
                                          int32_t num_facets, double* d_b, void* stream)
{
  if (int st = check_facet_form(L, DFX_FORM_SOURCE, d_facets, num_facets))
    return st;
  DFX_REQUIRE(d_b, "b must be non-NULL");
  if (num_facets == 0)
    return DFX_OK;
  const unsigned grid = (unsigned)((num_facets + kThreads - 1) / kThreads);
  cudaStream_t s = dfx::as_stream(stream);
  if (L->degree == 1)
    k_facets_vector<1><<<grid, kThreads, 0, s>>>(*L, d_facets, num_facets, d_b);
  else
    k_facets_vector<2><<<grid, kThreads, 0, s>>>(*L, d_facets, num_facets, d_b);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_assemble_matrix_facets(const dfx_form* a, const int32_t* d_facets,
                                          int32_t num_facets, const dfx_csr* A,
                                          const uint8_t* d_map, const int8_t* d_bc, void* stream)
{
  if (int st = check_facet_form(a, DFX_FORM_FACET_MASS, d_facets, num_facets))
    return st;
  DFX_REQUIRE(A && A->row_ptr && A->cols && A->vals, "matrix must be non-NULL");
  DFX_REQUIRE(A->dtype == DFX_F64 && A->bs == 1, "facet mass assembles scalar FP64 matrices");
  if (num_facets == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  const unsigned grid = (unsigned)((num_facets + kThreads - 1) / kThreads);
  if (a->degree == 1)
    k_facets_matrix<1><<<grid, kThreads, 0, s>>>(*a, d_facets, num_facets, A->row_ptr, A->cols,
                                                 (double*)A->vals, d_map, d_bc, status);
  else
    k_facets_matrix<2><<<grid, kThreads, 0, s>>>(*a, d_facets, num_facets, A->row_ptr, A->cols,
                                                 (double*)A->vals, d_map, d_bc, status);
  DFX_CHECK_LAUNCH();
  if (!d_map)
    return read_status(status, s);
  return DFX_OK;
}

namespace
{
int check_interior(const dfx_form* a, int32_t kind, const int32_t* d_facets, int32_t nf)
{
  DFX_REQUIRE(a, "form is NULL");
  DFX_REQUIRE(a->kind == kind, "form kind %d where %d is required", a->kind, kind);
  DFX_REQUIRE(a->degree == 1 || a->degree == 2, "degree must be 1 or 2");
  DFX_REQUIRE(nf >= 0, "negative facet count");
  DFX_REQUIRE(nf == 0 || (d_facets && a->x_dofmap && a->x && a->dofmap),
              "facets and form arrays must be non-NULL");
  DFX_REQUIRE(((uintptr_t)d_facets & 15) == 0, "interior facets must be 16-byte aligned");
  return DFX_OK;
}
} // namespace

extern "C" int dfx_assemble_vector_interior_facets(const dfx_form* L, const int32_t* d_facets,
                                                   int32_t num_facets, double* d_b, void* stream)
{
  if (int st = check_interior(L, DFX_FORM_SOURCE, d_facets, num_facets))
    return st;
  DFX_REQUIRE(d_b || num_facets == 0, "b must be non-NULL");
  if (num_facets == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  const unsigned grid = (unsigned)((num_facets + kThreads - 1) / kThreads);
  const int4* q = reinterpret_cast<const int4*>(d_facets);
  if (L->degree == 1)
    k_interior_facets_vector<1><<<grid, kThreads, 0, s>>>(*L, q, num_facets, d_b);
  else
    k_interior_facets_vector<2><<<grid, kThreads, 0, s>>>(*L, q, num_facets, d_b);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_assemble_matrix_interior_facets(const dfx_form* a, const int32_t* d_facets,
                                                   int32_t num_facets, const dfx_csr* A,
                                                   const int8_t* d_bc, void* stream)
{
  if (int st = check_interior(a, DFX_FORM_FACET_JUMP, d_facets, num_facets))
    return st;
  DFX_REQUIRE(A && A->row_ptr && A->cols && A->vals, "matrix must be non-NULL");
  DFX_REQUIRE(A->dtype == DFX_F64 && A->bs == 1, "the facet penalty assembles scalar FP64 matrices");
  if (num_facets == 0)
    return DFX_OK;
  cudaStream_t s = dfx::as_stream(stream);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  const unsigned grid = (unsigned)((num_facets + 127) / 128);
  const int4* q = reinterpret_cast<const int4*>(d_facets);
  if (a->degree == 1)
    k_interior_facets_matrix<1><<<grid, 128, 0, s>>>(*a, q, num_facets, A->row_ptr, A->cols,
                                                     (double*)A->vals, d_bc, status);
  else
    k_interior_facets_matrix<2><<<grid, 128, 0, s>>>(*a, q, num_facets, A->row_ptr, A->cols,
                                                     (double*)A->vals, d_bc, status);
  DFX_CHECK_LAUNCH();
  return read_status(status, s);
}

extern "C" int dfx_apply_lifting_facets(const dfx_form* a, const int32_t* d_facets,
                                        int32_t num_facets, int32_t interior, double* d_b,
                                        const int8_t* d_bc, const double* d_g,
                                        const double* d_x0, double alpha, void* stream)
{
  DFX_REQUIRE(a, "form is NULL");
  if (interior)
  {
    if (int st = check_interior(a, DFX_FORM_FACET_JUMP, d_facets, num_facets))
      return st;
  }
  else if (int st = check_facet_form(a, DFX_FORM_FACET_MASS, d_facets, num_facets))
    return st;
  if (num_facets == 0)
    return DFX_OK;
  DFX_REQUIRE(d_b && d_bc && d_g, "b, bc markers and g must be non-NULL");
  cudaStream_t s = dfx::as_stream(stream);
  if (interior)
  {
    const unsigned grid = (unsigned)((num_facets + 127) / 128);
    const int4* q = reinterpret_cast<const int4*>(d_facets);
    if (a->degree == 1)
      k_lift_interior_facets<1><<<grid, 128, 0, s>>>(*a, q, num_facets, d_bc, d_g, d_x0, alpha,
                                                     d_b);
    else
      k_lift_interior_facets<2><<<grid, 128, 0, s>>>(*a, q, num_facets, d_bc, d_g, d_x0, alpha,
                                                     d_b);
  }
  else
  {
    const unsigned grid = (unsigned)((num_facets + kThreads - 1) / kThreads);
    const int2* pr = reinterpret_cast<const int2*>(d_facets);
    if (a->degree == 1)
      k_lift_exterior_facets<1><<<grid, kThreads, 0, s>>>(*a, pr, num_facets, d_bc, d_g, d_x0,
                                                          alpha, d_b);
    else
      k_lift_exterior_facets<2><<<grid, kThreads, 0, s>>>(*a, pr, num_facets, d_bc, d_g, d_x0,
                                                          alpha, d_b);
  }
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" size_t dfx_assemble_scalar_workspace_bytes(int32_t num_cells)
{
  if (num_cells < 0)
    return 0;
  return sizeof(double) * ((size_t)scalar_blocks(num_cells) + 1);
}

extern "C" int dfx_assemble_scalar(const dfx_form* M, const double* d_u, double* value,
                                   void* d_work, size_t work_bytes, void* stream)
{
  DFX_REQUIRE(M && value, "form and value must be non-NULL");
  DFX_REQUIRE(M->kind == DFX_FORM_POISSON || M->kind == DFX_FORM_SOURCE,
              "functionals: a(u, u) of a Poisson/Helmholtz form or L(u) of a source form");
  if (int st = check_form(M, M->kind == DFX_FORM_POISSON))
    return st;
  *value = 0.0;
  if (M->num_cells == 0)
    return DFX_OK;
  DFX_REQUIRE(d_u, "u must be non-NULL");
  const int nb = scalar_blocks(M->num_cells);
  DFX_REQUIRE(d_work && work_bytes >= sizeof(double) * ((size_t)nb + 1),
              "workspace too small");
  double* part = (double*)d_work;
  cudaStream_t s = dfx::as_stream(stream);
  const bool mass = M->kind == DFX_FORM_POISSON && M->k2 != 0.0;
  if (M->kind == DFX_FORM_SOURCE)
  {
    if (M->degree == 1)
      k_cells_scalar<1, true, false><<<nb, kThreads, 0, s>>>(*M, d_u, part);
    else
      k_cells_scalar<2, true, false><<<nb, kThreads, 0, s>>>(*M, d_u, part);
  }
  else if (M->degree == 1)
  {
    if (mass)
      k_cells_scalar<1, false, true><<<nb, kThreads, 0, s>>>(*M, d_u, part);
    else
      k_cells_scalar<1, false, false><<<nb, kThreads, 0, s>>>(*M, d_u, part);
  }
  else
  {
    if (mass)
      k_cells_scalar<2, false, true><<<nb, kThreads, 0, s>>>(*M, d_u, part);
    else
      k_cells_scalar<2, false, false><<<nb, kThreads, 0, s>>>(*M, d_u, part);
  }
  DFX_CHECK_LAUNCH();
  k_sum_partials<<<1, 32, 0, s>>>(part, nb, part + nb);
  DFX_CHECK_LAUNCH();
  DFX_CUDA(cudaMemcpyAsync(value, part + nb, sizeof(double), cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}
