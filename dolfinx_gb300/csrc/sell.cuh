// Sliced-ELL (SELL-32-sigma) operator: the solver-side layout of a
// la::MatrixCSR.
//
// GB300 executes FP64 at ~1/58 of its FP32 rate, so an FP64 SpMV is bound
// by FP64 warp instructions as much as by HBM: a CSR kernel with several
// lanes per row spends more FP64 instructions on shuffle reductions and
// idle lanes than on products. SELL-32 gives every lane one row and no
// reduction: each FP64 instruction does 32 useful FMAs.
//   - rows are sorted by length (descending, stable) inside windows of
//     sigma rows, which keeps the RCM locality and cuts padding to a few
//     percent; the system is renumbered symmetrically with that
//     permutation, so vectors stay coalesced;
//   - slices of 32 consecutive (renumbered) rows are stored column-major:
//     entry k of row 32*s + lane sits at slice_ptr[s] + 32*k + lane;
//   - columns are int32, or (FP32 operator) a per-row first column plus
//     16-bit deltas between the row's sorted columns (2 bytes per entry);
//   - FP32 operators keep each lane's entries in consecutive pairs, so a
//     lane moves 8 bytes of values per load like the FP64 operator does;
//   - padding entries have value 0 and repeat a valid column.
// Values are refilled from the CSR values after every assembly through a
// precomputed slot map (SELL entry -> CSR entry, -1 for padding).
#pragma once

#include "common.cuh"

struct dfx_operator_s
{
  int32_t n = 0;        // scalar rows
  // 1, or 3: a 3x3-block operator. Its slices hold 32 block rows (lane =
  // block row), one column index per block, and the 9 values of slot j at
  // 9 (j - j % 32) + 32 e + j % 32, e = 3 r + c row-major within the block;
  // split operators keep (hi, lo) of a value together there as one float2.
  // perm / iperm are the block permutation expanded to the scalar rows.
  int32_t bs = 1;
  int32_t nslices = 0;
  int32_t sigma = 0;
  int32_t dtype = DFX_F64;
  int32_t compressed = 0;
  int64_t nslots = 0;   // SELL entries incl. padding (multiple of 32)
  int64_t csr_nnz = 0;
  int32_t* perm = nullptr;      // new -> old row (n)
  int32_t* iperm = nullptr;     // old -> new row (n)
  int64_t* slice_ptr = nullptr; // (nslices + 1), in entries
  int32_t* cols = nullptr;      // (nslots), uncompressed operators
  uint16_t* delta = nullptr;    // (nslots), compressed operators
  int32_t* first = nullptr;     // (32 * nslices), compressed operators
  int32_t* map = nullptr;       // (nslots) CSR entry or -1
  void* vals = nullptr;         // (nslots) f64 or f32; DFX_F32X2: hi (nslots) then lo (nslots)
  void* tmp = nullptr;          // 2 n scratch values for dfx_operator_apply
  int device = 0;
  // Structure sharing (dfx_operator_share): a share points at its source's
  // structure arrays and owns only its values; the source counts its shares
  // and may not be destroyed while any is alive.
  // Process-wide creation number: cached CUDA graphs bake the operator's
  // arrays into their launches, so they are keyed by this number and not
  // by addresses, which a later operator may reuse.
  uint64_t serial = 0;
  // FP32 operators: value pairs per load chunk of a lane (2, 4 or 8): the
  // loads of one chunk are in flight together (autotuned; 4 by default).
  // 3x3-block operators: 2, 4 or 8 for 1, 2 or 4 block slots per round
  // (8 by default).
  int32_t chunk = 4;
  int32_t owns_structure = 1;
  // Values and scratch come from the library's stream-ordered pool
  // (dfx_operator_share_async) and go back to it in stream order.
  int32_t pooled = 0;
  int32_t shares = 0;
  dfx_operator_s* source = nullptr;
};

namespace dfx
{
// A new operator serial (never 0).
uint64_t next_operator_serial();

#ifdef __CUDACC__
// Row sum of lane `lane` of slice `s` (row 32 s + lane, padded slices).
// FP64 operators: entry k of the lane at slice_ptr[s] + 32 k + lane.
// FP32 operators: entries in k-pairs, pair j of the lane at
// slice_ptr[s] + 64 j + 2 lane (+0, +1), read as one 8-byte load of values
// and one 4- or 8-byte load of column data.
template <typename V, typename X, typename ACC, bool COMP, int CH = 4>
__device__ __forceinline__ ACC sell_row(const dfx_operator_s& op, const V* __restrict__ vals,
                                        const X* __restrict__ x, int32_t s, int lane)
{
  const int64_t b = __ldg(op.slice_ptr + s);
  const int len = (int)((__ldg(op.slice_ptr + s + 1) - b) >> 5);
  ACC acc = ACC(0);
  if constexpr (sizeof(V) == 4)
  {
    // Chunks of kChunk pairs: the chunk's value/column loads are issued
    // together (and the next chunk's before this chunk's gathers), then
    // all its x gathers, then the FMAs in entry order. Measured on the P2
    // Poisson operator of a 64^3 x 6 tetrahedral mesh: 79 us against 104 us
    // for the same loop with loads, gathers and FMAs interleaved.
    constexpr int kChunk = CH; // pairs per chunk: the operator's `chunk` (autotuned)
    const float2* v = reinterpret_cast<const float2*>(vals + b) + lane;
    const int np = len >> 1;
    float2 vv[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u)
      vv[u] = u < np ? __ldcs(v + 32 * u) : make_float2(0.f, 0.f);
    if constexpr (COMP)
    {
      const ushort2* d = reinterpret_cast<const ushort2*>(op.delta + b) + lane;
      int32_t col = __ldg(op.first + 32 * (int64_t)s + lane);
      ushort2 dd[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
        dd[u] = u < np ? __ldcs(d + 32 * u) : make_ushort2(0, 0);
      for (int j0 = 0; j0 < np; j0 += kChunk)
      {
        float2 nv[kChunk];
        ushort2 nd[kChunk];
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          const bool ok = j0 + kChunk + u < np;
          nv[u] = ok ? __ldcs(v + 32 * (j0 + kChunk + u)) : make_float2(0.f, 0.f);
          nd[u] = ok ? __ldcs(d + 32 * (j0 + kChunk + u)) : make_ushort2(0, 0);
        }
        // Padding pairs past np have zero deltas: their gathers repeat a
        // valid column and their values are zero.
        int32_t c0[kChunk], c1[kChunk];
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          col += dd[u].x; // delta of entry 0 is stored as 0
          c0[u] = col;
          col += dd[u].y;
          c1[u] = col;
        }
        X x0[kChunk], x1[kChunk];
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          x0[u] = __ldg(x + c0[u]);
          x1[u] = __ldg(x + c1[u]);
        }
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          if (j0 + u < np)
          {
            acc = fma((ACC)vv[u].x, (ACC)x0[u], acc);
            acc = fma((ACC)vv[u].y, (ACC)x1[u], acc);
          }
          vv[u] = nv[u];
          dd[u] = nd[u];
        }
      }
    }
    else
    {
      const int2* c = reinterpret_cast<const int2*>(op.cols + b) + lane;
      int2 cc[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
        cc[u] = u < np ? __ldcs(c + 32 * u) : make_int2(0, 0);
      for (int j0 = 0; j0 < np; j0 += kChunk)
      {
        float2 nv[kChunk];
        int2 nc[kChunk];
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          const bool ok = j0 + kChunk + u < np;
          nv[u] = ok ? __ldcs(v + 32 * (j0 + kChunk + u)) : make_float2(0.f, 0.f);
          nc[u] = ok ? __ldcs(c + 32 * (j0 + kChunk + u)) : make_int2(0, 0);
        }
        X x0[kChunk], x1[kChunk];
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          x0[u] = __ldg(x + cc[u].x);
          x1[u] = __ldg(x + cc[u].y);
        }
#pragma unroll
        for (int u = 0; u < kChunk; ++u)
        {
          if (j0 + u < np)
          {
            acc = fma((ACC)vv[u].x, (ACC)x0[u], acc);
            acc = fma((ACC)vv[u].y, (ACC)x1[u], acc);
          }
          vv[u] = nv[u];
          cc[u] = nc[u];
        }
      }
    }
  }
  else
  {
    const V* v = vals + b + lane;
    const int32_t* c = op.cols + b + lane;
#pragma unroll 4
    for (int k = 0; k < len; ++k)
      acc = fma((ACC)__ldcs(v + 32 * k), (ACC)__ldg(x + __ldcs(c + 32 * k)), acc);
  }
  return acc;
}
#endif

#ifdef __CUDACC__
// Row sum of a split operator (DFX_F32X2): each FP64 value is carried as
// two FP32 words, hi = fl32(v) and lo = fl32(v - hi), stored in two arrays
// of the FP32 pair layout (vals and vals + nslots); x's words sit side by
// side, (hi, lo) per row, so an entry gathers them in one 8-byte load.
// Products and the running sum use the FP32 pipe with error-free
// transformations: hi*hi exactly as a sum of two floats (fma), the cross
// terms hi*lo + lo*hi into a low-order accumulator, and the high-order
// accumulator updated by a two-sum whose rounding error also goes to the
// low-order one. The result carries ~2^-44 relative error, far below what
// CG needs -- FP64-equivalent arithmetic without the FP64 pipe, which runs
// at 1/58 of the FP32 rate on this part.
template <bool COMP>
__device__ __forceinline__ double sell_row_split(const dfx_operator_s& op,
                                                 const float* __restrict__ vh,
                                                 const float* __restrict__ vl,
                                                 const float2* __restrict__ xw, int32_t s,
                                                 int lane)
{
  const int64_t b = __ldg(op.slice_ptr + s);
  const int len = (int)((__ldg(op.slice_ptr + s + 1) - b) >> 5);
  const int np = len >> 1;
  const float2* ph = reinterpret_cast<const float2*>(vh + b) + lane;
  const float2* pl = reinterpret_cast<const float2*>(vl + b) + lane;
  float S = 0.f, L = 0.f;
  // The _rn intrinsics keep the compiler from contracting the product
  // into the sums, which would break the exactness of the two-sum.
  auto add = [&](float ah, float al, float x0, float x1)
  {
    const float p = __fmul_rn(ah, x0);
    const float e = fmaf(ah, x0, -p);
    const float t = fmaf(ah, x1, fmaf(al, x0, e));
    const float u = __fadd_rn(S, p);
    const float bp = __fsub_rn(u, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(u, bp)), __fsub_rn(p, bp));
    S = u;
    L += err + t;
  };
  if constexpr (COMP)
  {
    const ushort2* d = reinterpret_cast<const ushort2*>(op.delta + b) + lane;
    int32_t col = __ldg(op.first + 32 * (int64_t)s + lane);
    constexpr int kChunk = 2;
    for (int j0 = 0; j0 < np; j0 += kChunk)
    {
      float2 hv[kChunk], lv[kChunk];
      ushort2 dd[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
      {
        const bool ok = j0 + u < np;
        hv[u] = ok ? __ldcs(ph + 32 * (j0 + u)) : make_float2(0.f, 0.f);
        lv[u] = ok ? __ldcs(pl + 32 * (j0 + u)) : make_float2(0.f, 0.f);
        dd[u] = ok ? __ldcs(d + 32 * (j0 + u)) : make_ushort2(0, 0);
      }
      int32_t c0[kChunk], c1[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
      {
        col += dd[u].x;
        c0[u] = col;
        col += dd[u].y;
        c1[u] = col;
      }
      // x's (hi, lo) words sit together: one 8-byte gather per entry.
      float2 x0[kChunk], x1[kChunk];
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
      {
        x0[u] = __ldg(xw + c0[u]);
        x1[u] = __ldg(xw + c1[u]);
      }
#pragma unroll
      for (int u = 0; u < kChunk; ++u)
      {
        add(hv[u].x, lv[u].x, x0[u].x, x0[u].y);
        add(hv[u].y, lv[u].y, x1[u].x, x1[u].y);
      }
    }
  }
  else
  {
    const int2* c = reinterpret_cast<const int2*>(op.cols + b) + lane;
    for (int j = 0; j < np; ++j)
    {
      const float2 hv = __ldcs(ph + 32 * j), lv = __ldcs(pl + 32 * j);
      const int2 cc = __ldcs(c + 32 * j);
      const float2 x0 = __ldg(xw + cc.x), x1 = __ldg(xw + cc.y);
      add(hv.x, lv.x, x0.x, x0.y);
      add(hv.y, lv.y, x1.x, x1.y);
    }
  }
  return (double)S + (double)L;
}

// Block row sums of a 3x3-block operator (bs 3): lane's block row
// 32 s + lane, acc[r] = row 3 (32 s + lane) + r. The entries of a scalar
// row are added in ascending column order, as in the scalar operator.
// FP64 values: 76 bytes per block (one column, nine values) against 108
// for the same nine entries in the scalar layout. SL block slots are read
// per round, their loads issued together (the operator's chunk / 2).
template <int SL>
__device__ __forceinline__ void bsell_row3(const dfx_operator_s& op, const double* __restrict__ vals,
                                           const double* __restrict__ x, int32_t s, int lane,
                                           double acc[3])
{
  const int64_t b = __ldg(op.slice_ptr + s);
  const int len = (int)((__ldg(op.slice_ptr + s + 1) - b) >> 5);
  const double* v = vals + 9 * b + lane;
  const int32_t* c = op.cols + b + lane;
  acc[0] = acc[1] = acc[2] = 0.0;
  for (int k0 = 0; k0 < len; k0 += SL)
  {
    int32_t cb[SL];
    double a[SL][9];
#pragma unroll
    for (int u = 0; u < SL; ++u)
    {
      const bool ok = SL == 1 || k0 + u < len;
      cb[u] = ok ? __ldcs(c + 32 * (k0 + u)) : 0;
#pragma unroll
      for (int e = 0; e < 9; ++e)
        a[u][e] = ok ? __ldcs(v + 288 * (int64_t)(k0 + u) + 32 * e) : 0.0;
    }
    double xv[SL][3];
#pragma unroll
    for (int u = 0; u < SL; ++u)
    {
      const double* xp = x + 3 * (int64_t)cb[u];
#pragma unroll
      for (int q = 0; q < 3; ++q)
        xv[u][q] = __ldg(xp + q);
    }
#pragma unroll
    for (int u = 0; u < SL; ++u)
      if (SL == 1 || k0 + u < len)
      {
#pragma unroll
        for (int r = 0; r < 3; ++r)
          acc[r] = fma(a[u][3 * r + 2], xv[u][2],
                       fma(a[u][3 * r + 1], xv[u][1], fma(a[u][3 * r], xv[u][0], acc[r])));
      }
  }
}

// The same for a split 3x3-block operator (DFX_F32X2, bs 3): each value's
// (hi, lo) words in one float2, x's words (hi, lo) per scalar row, and the
// error-free FP32 products and sums of sell_row_split per scalar row.
template <int SL>
__device__ __forceinline__ void bsell_row3_split(const dfx_operator_s& op,
                                                 const float2* __restrict__ vw,
                                                 const float2* __restrict__ xw, int32_t s,
                                                 int lane, double out[3])
{
  const int64_t b = __ldg(op.slice_ptr + s);
  const int len = (int)((__ldg(op.slice_ptr + s + 1) - b) >> 5);
  const float2* v = vw + 9 * b + lane;
  const int32_t* c = op.cols + b + lane;
  float S[3] = {0.f, 0.f, 0.f}, L[3] = {0.f, 0.f, 0.f};
  auto add = [&](int r, float ah, float al, float x0, float x1)
  {
    const float p = __fmul_rn(ah, x0);
    const float e = fmaf(ah, x0, -p);
    const float t = fmaf(ah, x1, fmaf(al, x0, e));
    const float u = __fadd_rn(S[r], p);
    const float bp = __fsub_rn(u, S[r]);
    const float err = __fadd_rn(__fsub_rn(S[r], __fsub_rn(u, bp)), __fsub_rn(p, bp));
    S[r] = u;
    L[r] += err + t;
  };
  for (int k0 = 0; k0 < len; k0 += SL)
  {
    int32_t cb[SL];
    float2 a[SL][9];
#pragma unroll
    for (int u = 0; u < SL; ++u)
    {
      const bool ok = SL == 1 || k0 + u < len;
      cb[u] = ok ? __ldcs(c + 32 * (k0 + u)) : 0;
#pragma unroll
      for (int e = 0; e < 9; ++e)
        a[u][e] = ok ? __ldcs(v + 288 * (int64_t)(k0 + u) + 32 * e) : make_float2(0.f, 0.f);
    }
    float2 xv[SL][3];
#pragma unroll
    for (int u = 0; u < SL; ++u)
    {
      const float2* xp = xw + 3 * (int64_t)cb[u];
#pragma unroll
      for (int q = 0; q < 3; ++q)
        xv[u][q] = __ldg(xp + q);
    }
#pragma unroll
    for (int u = 0; u < SL; ++u)
      if (SL == 1 || k0 + u < len)
      {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int q = 0; q < 3; ++q)
            add(r, a[u][3 * r + q].x, a[u][3 * r + q].y, xv[u][q].x, xv[u][q].y);
      }
  }
#pragma unroll
  for (int r = 0; r < 3; ++r)
    out[r] = (double)S[r] + (double)L[r];
}

// Blocks per SM of the 3x3-block SpMV kernels by slots per round: the
// registers of SL slots of values (64, 80 and 128 registers).
template <int SL>
constexpr int kBsellMinBlocks = SL == 1 ? 8 : (SL == 2 ? 6 : 4);

// Splits an FP64 vector into the (hi, lo) FP32 words a split operator reads.
__device__ __forceinline__ void split_f64(double v, float& hi, float& lo)
{
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - (double)hi);
}
#endif

#ifdef __CUDACC__
// Slices of this block: a contiguous run, so that the rows one SM works on
// are neighbours and their x gathers hit the same L1 lines. Warps of the
// block interleave inside the run.
struct SliceRange
{
  int32_t begin, end, step;
};
__device__ __forceinline__ SliceRange block_slices(int32_t nslices)
{
  const int32_t per = (nslices + (int32_t)gridDim.x - 1) / (int32_t)gridDim.x;
  const int32_t b = (int32_t)blockIdx.x * per;
  SliceRange r;
  r.begin = b + (int32_t)(threadIdx.x >> 5);
  r.end = min(nslices, b + per);
  r.step = (int32_t)(blockDim.x >> 5);
  return r;
}
#endif

// Grid of the sliced-ELL kernels (blocks of 256 threads), and the largest
// grid any kernel with per-block partial sums uses.
int sell_grid(int32_t nslices);
int max_grid_blocks();

// Launch y = A x on renumbered vectors (both of length op.n). A split
// operator (DFX_F32X2) takes x as its FP32 words, (hi, lo) per row, and
// writes y in FP64.
int sell_spmv(const dfx_operator_s& op, const void* x, void* y, cudaStream_t s);

// Bytes of an operator's value array and of its scratch vectors.
size_t value_bytes(const dfx_operator_s& op);
size_t scratch_bytes(const dfx_operator_s& op);
} // namespace dfx
