// Q4 hexahedral Laplacian action by sum factorisation.
//
// The gradient at the 125 quadrature points of a cell costs 8
// one-dimensional contractions of 5 terms per point instead of the
// 125 x 125 x 3 products of the full element matrix; the transpose costs 8
// more. The Jacobian of the trilinear map is formed at each quadrature
// point in the kernel's precision from the cell's edge vectors (vertex
// differences taken in FP64). Cells are processed in 8 colours (parity of
// i, j, k): cells of one colour share no node, so the scatter is a plain
// read-modify-write, deterministic and free of atomics.
#include "q4.cuh"

#include <algorithm>
#include <cstring>
#include <cmath>
#include <mutex>
#include <vector>

namespace
{
__constant__ double cB64[25], cD64[25], cW64[5], cG64[5];
__constant__ float cB32[25], cD32[25], cW32[5], cG32[5];

template <typename T>
struct Tab;
template <>
struct Tab<double>
{
  __device__ static double B(int q, int a) { return cB64[5 * q + a]; }
  __device__ static double D(int q, int a) { return cD64[5 * q + a]; }
  __device__ static double W(int q) { return cW64[q]; }
  __device__ static double G(int q) { return cG64[q]; }
};
template <>
struct Tab<float>
{
  __device__ static float B(int q, int a) { return cB32[5 * q + a]; }
  __device__ static float D(int q, int a) { return cD32[5 * q + a]; }
  __device__ static float W(int q) { return cW32[q]; }
  __device__ static float G(int q) { return cG32[q]; }
};

// Tables of the tensor-core variant (see k_q4_cells_tc below).
//
// Operand layout (both operands K-major, no swizzle): K is grouped by the
// 5 line positions of the contracted direction; position `pos` owns C_p
// core-matrix columns of 4 K slots, and input type tau (the tables' inputs
// at that position: u; or A, Ad; or C0, Cy, Cx; ...) its split words in
// slots 3 tau + s, s = 0, 1, 2 (unused slots hold 0). A's rows are 16 bytes
// apart through all 128 rows (SBO 128 B) and its core-matrix columns
// kTcLboA bytes apart, so the byte offset of (row, pos, slot) is linear in
// row and pos: a thread's writes into the rows of another phase's lines
// are constant offsets from one base, as 16-byte vector stores.
constexpr int kTcPhases = 6;
constexpr int kTcTypes[kTcPhases] = {1, 2, 3, 3, 3, 2};
constexpr int kTcLboA = 128 * 16 + 16;  // +16 B keeps the 5 positions off one bank group
constexpr int kTcLboB = 16 * 16;
constexpr int kTcACols = 16;             // core-matrix columns of the largest A (K = 64)
constexpr int kTcAFloats = kTcACols * kTcLboA / 4;
constexpr int kTcWaitPolls = 1 << 20;
// Core-matrix columns per position, and of K (a multiple of 2: K % 8 == 0).
__host__ __device__ constexpr int tc_cpp(int p) { return p == 0 ? 1 : (p == 1 || p == 5 ? 2 : 3); }
__host__ __device__ constexpr int tc_kcols(int p) { return ((5 * tc_cpp(p) + 1) / 2) * 2; }
// Table p's float offset: 16 rows x tc_kcols(p) columns of 4 floats each.
__host__ __device__ constexpr int tc_tab_off(int p)
{
  int o = 0;
  for (int q = 0; q < p; ++q)
    o += 64 * tc_kcols(q);
  return o;
}
constexpr int kTcTabFloats = tc_tab_off(kTcPhases);
constexpr int kTcSmemBytes = 4 * (kTcAFloats + kTcTabFloats); // dynamic shared memory

__device__ float g_q4tc_tab[kTcTabFloats];
__device__ int32_t g_q4tc_error; // set when an MMA completion wait gave up

// The B operands of the six phases: table p, row n (output), position pos,
// input type tau: C_p[n][5 tau + pos] as (hi, hi, lo) in slots 3 tau + s
// (the A data carries (hi, lo, hi)).
void build_tc_tables(const double B[25], const double D[25], float* out)
{
  auto b = [&](int q, int a) { return B[5 * q + a]; };
  auto d = [&](int q, int a) { return D[5 * q + a]; };
  // Logical coefficient of output n from input j = 5 tau + pos in phase p.
  auto coef = [&](int p, int n, int j) -> double
  {
    switch (p)
    {
    case 0: // x: A(qx) = sum_x B u, Ad(qx) = sum_x D u
      return n < 5 ? b(n, j) : (n < 10 ? d(n - 5, j) : 0.0);
    case 1: // y: inputs V0(y) j < 5, V1(y) 5 <= j < 10
      if (n < 5)
        return j < 5 ? b(n, j) : 0.0;
      if (n < 10)
        return j < 5 ? d(n - 5, j) : 0.0;
      if (n < 15)
        return j >= 5 ? b(n - 10, j - 5) : 0.0;
      return 0.0;
    case 2: // z: inputs C0(z), Cy(z), Cx(z) -> uz, uy, ux (qz)
      if (n < 5)
        return j < 5 ? d(n, j) : 0.0;
      if (n < 10)
        return (j >= 5 && j < 10) ? b(n - 5, j - 5) : 0.0;
      if (n < 15)
        return j >= 10 ? b(n - 10, j - 10) : 0.0;
      return 0.0;
    case 3: // z^T: inputs vx, vy, vz (qz) -> ex, ey, ez (z)
      if (n < 5)
        return j < 5 ? b(j, n) : 0.0;
      if (n < 10)
        return (j >= 5 && j < 10) ? b(j - 5, n - 5) : 0.0;
      if (n < 15)
        return j >= 10 ? d(j - 10, n - 10) : 0.0;
      return 0.0;
    case 4: // y^T: inputs ex, ey, ez (qy) -> x1 = B^T ex, x2 = D^T ey + B^T ez (y)
      if (n < 5)
        return j < 5 ? b(j, n) : 0.0;
      if (n < 10)
        return (j >= 5 && j < 10) ? d(j - 5, n - 5) : (j >= 10 ? b(j - 10, n - 5) : 0.0);
      return 0.0;
    default: // x^T: inputs x1, x2 (qx) -> y_e = D^T x1 + B^T x2 (x)
      if (n < 5)
        return j < 5 ? d(j, n) : b(j - 5, n);
      return 0.0;
    }
  };
  auto tf32 = [](double v) -> float
  {
    // nearest with 10 mantissa bits, ties away from zero (cvt.rna.tf32.f32)
    float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x1000u) & 0xffffe000u;
    std::memcpy(&f, &u, 4);
    return f;
  };
  std::fill(out, out + kTcTabFloats, 0.0f);
  for (int p = 0; p < kTcPhases; ++p)
  {
    float* T = out + tc_tab_off(p);
    for (int n = 0; n < 16; ++n)
      for (int pos = 0; pos < 5; ++pos)
        for (int tau = 0; tau < kTcTypes[p]; ++tau)
        {
          const double c = coef(p, n, 5 * tau + pos);
          const float hi = tf32(c);
          const float words[3] = {hi, hi, tf32(c - (double)hi)};
          for (int sp = 0; sp < 3; ++sp)
          {
            const int slot = 3 * tau + sp;
            const int col = pos * tc_cpp(p) + slot / 4;
            T[(n * 16 + col * kTcLboB + (slot % 4) * 4) / 4] = words[sp];
          }
        }
  }
}

std::mutex g_tab_mutex;
bool g_tab_ready[64] = {};

// GLL nodes of degree 4 on [0,1]; Gauss-Legendre points and weights on [0,1].
int upload_tables()
{
  int dev = 0;
  DFX_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tab_mutex);
  if (dev < 64 && g_tab_ready[dev])
    return DFX_OK;
  const double s = std::sqrt(3.0 / 7.0);
  const double xn[5] = {0.0, 0.5 * (1.0 - s), 0.5, 0.5 * (1.0 + s), 1.0};
  // 5-point Gauss-Legendre on [-1,1]
  const double r = 2.0 * std::sqrt(10.0 / 7.0);
  const double g1 = std::sqrt(5.0 - r) / 3.0, g2 = std::sqrt(5.0 + r) / 3.0;
  const double w0 = 128.0 / 225.0, w1 = (322.0 + 13.0 * std::sqrt(70.0)) / 900.0,
               w2 = (322.0 - 13.0 * std::sqrt(70.0)) / 900.0;
  const double gp[5] = {-g2, -g1, 0.0, g1, g2};
  const double gw[5] = {w2, w1, w0, w1, w2};
  double B[25], D[25], W[5], G[5];
  for (int q = 0; q < 5; ++q)
  {
    const double t = 0.5 * (gp[q] + 1.0);
    G[q] = t;
    W[q] = 0.5 * gw[q];
    for (int a = 0; a < 5; ++a)
    {
      double l = 1.0;
      for (int m = 0; m < 5; ++m)
        if (m != a)
          l *= (t - xn[m]) / (xn[a] - xn[m]);
      double dl = 0.0;
      for (int k = 0; k < 5; ++k)
      {
        if (k == a)
          continue;
        double p = 1.0 / (xn[a] - xn[k]);
        for (int m = 0; m < 5; ++m)
          if (m != a && m != k)
            p *= (t - xn[m]) / (xn[a] - xn[m]);
        dl += p;
      }
      B[5 * q + a] = l;
      D[5 * q + a] = dl;
    }
  }
  float Bf[25], Df[25], Wf[5], Gf[5];
  for (int i = 0; i < 25; ++i)
  {
    Bf[i] = (float)B[i];
    Df[i] = (float)D[i];
  }
  for (int i = 0; i < 5; ++i)
  {
    Wf[i] = (float)W[i];
    Gf[i] = (float)G[i];
  }
  DFX_CUDA(cudaMemcpyToSymbol(cB64, B, sizeof(B)));
  DFX_CUDA(cudaMemcpyToSymbol(cD64, D, sizeof(D)));
  DFX_CUDA(cudaMemcpyToSymbol(cW64, W, sizeof(W)));
  DFX_CUDA(cudaMemcpyToSymbol(cG64, G, sizeof(G)));
  DFX_CUDA(cudaMemcpyToSymbol(cB32, Bf, sizeof(Bf)));
  DFX_CUDA(cudaMemcpyToSymbol(cD32, Df, sizeof(Df)));
  DFX_CUDA(cudaMemcpyToSymbol(cW32, Wf, sizeof(Wf)));
  DFX_CUDA(cudaMemcpyToSymbol(cG32, Gf, sizeof(Gf)));
  std::vector<float> tc(kTcTabFloats);
  build_tc_tables(B, D, tc.data());
  DFX_CUDA(cudaMemcpyToSymbol(g_q4tc_tab, tc.data(), sizeof(float) * kTcTabFloats));
  const int32_t zero = 0;
  DFX_CUDA(cudaMemcpyToSymbol(g_q4tc_error, &zero, sizeof(zero)));
  if (dev < 64)
    g_tab_ready[dev] = true;
  return DFX_OK;
}

// Cells per CTA batch: 5 cells x 25 lines of 5 nodes = 125 threads.
constexpr int kBatch = 5;
constexpr int kLattice = 125;

// Shared-memory layouts of a cell's 5^3 values (x, y, z). Values written in
// one phase and read in the next go through layout A (phases 1->2, 4->5:
// lanes span (y, z), then (x, z)) or B (2->3, 3->4: lanes span (x, z), then
// (x, y)); in FP32 the strides make every access of the 4 warps free of bank
// conflicts (a 125-stride lattice gives 2-way conflicts). FP64 keeps the
// compact lattice: that kernel is bound by the FP64 pipe.
template <typename T>
struct Lay
{
  static constexpr int ay = 33, az = 5, by = 5, bz = 37, cell = 185;
};
template <>
struct Lay<double>
{
  static constexpr int ay = 5, az = 25, by = 5, bz = 25, cell = 125;
};
template <typename T>
__device__ __forceinline__ int lay_a(int x, int y, int z)
{
  return x + Lay<T>::ay * y + Lay<T>::az * z;
}
template <typename T>
__device__ __forceinline__ int lay_b(int x, int y, int z)
{
  return x + Lay<T>::by * y + Lay<T>::bz * z;
}

// The 12 edge components of one coordinate, read with 16-byte loads.
__device__ __forceinline__ void load_edges(const float* p, float (&e)[12])
{
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < 3; ++i)
  {
    const float4 v = q[i];
    e[4 * i] = v.x;
    e[4 * i + 1] = v.y;
    e[4 * i + 2] = v.z;
    e[4 * i + 3] = v.w;
  }
}
__device__ __forceinline__ void load_edges(const double* p, double (&e)[12])
{
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 6; ++i)
  {
    const double2 v = q[i];
    e[2 * i] = v.x;
    e[2 * i + 1] = v.y;
  }
}

// Edge e of a hexahedron (vertex v = bx + 2 by + 4 bz): e / 4 is its
// direction, e % 4 its position; returns the lower vertex (the upper is
// lower + 1, + 2 or + 4).
__device__ __forceinline__ int edge_lo(int e)
{
  const int d = e >> 2, m = e & 3;
  return d == 0 ? 2 * m : (d == 1 ? (m & 1) + 4 * (m >> 1) : m);
}

// A CTA takes batches of 5 cells of one colour. Thread t < 125 owns cell
// t / 25 of the batch and line l = t % 25 of its 5^3 lattice; in each
// phase the line runs along the direction being contracted, so a thread
// holds 5 values and produces 5, every table entry is a compile-time index
// (an immediate constant-bank operand of the FMA) and the 125 values of a
// cell pass between phases through shared memory:
//   1. x: u on the line (registers, from global)   -> A, Ad   (B, D in x)
//   2. y: A, Ad                                      -> C, Cy, Cx
//   3. z: C, Cy, Cx -> grad at 5 points -> G grad -> transpose in z
//   4. y transpose;  5. x transpose -> y += on the line (global).
// Lines of phases 1/5 are (y, z) node rows, of 2/4 (x, z), of 3 (x, y).
// One colour of cells (parity ci, cj, ck): hx x hy x hz cells, ordinal
// b = x + hx (y + hy z). A thread's cell advances by kBatch x gridDim.x
// ordinals per batch, given as mixed-radix digits (dx, dy, dz) so that the
// kernel needs no integer division after its first cell.
struct Colour
{
  int ci, cj, ck;
  int hx, hy, hz;
  int dx, dy, dz;
};

// x / y / z of a colour ordinal, advanced by the digits (dx, dy, dz).
struct CellIter
{
  int x, y, z;
  __device__ void advance(const Colour& col)
  {
    x += col.dx;
    const int cx = x >= col.hx;
    x -= cx ? col.hx : 0;
    y += col.dy + cx;
    const int cy = y >= col.hy;
    y -= cy ? col.hy : 0;
    z += col.dz + cy;
  }
};

// x / |d| in the kernel's precision: the fast reciprocal path in FP32 (a
// few ulp, far below the FP32 operator's own rounding), IEEE in FP64.
__device__ __forceinline__ float div_abs(float x, float d) { return __fdividef(x, fabsf(d)); }
__device__ __forceinline__ double div_abs(double x, double d) { return x / fabs(d); }

// GQ: read the cached geometric factors (dfx_q4_geometry) in phase 3 in
// place of the Jacobian, adjugate and determinant; the edge vectors are
// then not staged.
template <typename T, bool GQ>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 4 : 2)
    k_q4_cells(const dfx_q4_mesh_s m, const T* __restrict__ u, T* __restrict__ y,
               const Colour col, const int32_t* __restrict__ skip)
{
  if (skip && __ldg(skip))
    return;
  using Tb = Tab<T>;
  __shared__ T S[6][kBatch * Lay<T>::cell];
  __shared__ __align__(16) T se[kBatch][3][12]; // edge vectors by cell and component
  __shared__ double sv[kBatch][24];
  const int t = threadIdx.x;
  const bool act = t < kBatch * kLattice / 5;
  const int c = act ? t / 25 : 0, l = t % 25;
  const int la = l % 5, lb = l / 5;
  T* const S0 = S[0] + c * Lay<T>::cell;
  T* const S1 = S[1] + c * Lay<T>::cell;
  T* const S2 = S[2] + c * Lay<T>::cell;
  T* const S3 = S[3] + c * Lay<T>::cell;
  T* const S4 = S[4] + c * Lay<T>::cell;
  T* const S5 = S[5] + c * Lay<T>::cell;

  const int cells = col.hx * col.hy * col.hz; // < 2^31, checked on the host
  const int batches = (cells + kBatch - 1) / kBatch;
  const int NX = 4 * m.nx + 1, NY = 4 * m.ny + 1, NZ = 4 * m.nz + 1;
  // This thread's cell (c of the batch) and its phase-1/5 line: nodes
  // (4i + 0..4, 4j + la, 4k + lb).
  struct Line
  {
    int64_t base;
    bool row_bnd; // the whole line lies on a y or z boundary face
    bool x_lo, x_hi;
    bool valid;
    int i, j, k;
  };
  auto line_of = [&](const CellIter& it) -> Line
  {
    Line L{0, false, false, false, false, 0, 0, 0};
    if (!act || it.z >= col.hz)
      return L;
    L.i = col.ci + 2 * it.x;
    L.j = col.cj + 2 * it.y;
    L.k = col.ck + 2 * it.z;
    const int J = 4 * L.j + la, K = 4 * L.k + lb;
    L.base = ((int64_t)K * NY + J) * NX + 4 * (int64_t)L.i;
    L.row_bnd = J == 0 || K == 0 || J == NY - 1 || K == NZ - 1;
    L.x_lo = L.i == 0;
    L.x_hi = L.i == m.nx - 1;
    L.valid = true;
    return L;
  };
  // Coordinate l (< 24) of the cell's 8 vertices, loaded by its thread l.
  auto vert_of = [&](const Line& L) -> double
  {
    if (!L.valid || l >= 24)
      return 0.0;
    const int v = l / 3, comp = l % 3;
    const int64_t vi = L.i + (v & 1), vj = L.j + ((v >> 1) & 1), vk = L.k + ((v >> 2) & 1);
    return m.verts[3 * ((vk * (m.ny + 1) + vj) * (m.nx + 1) + vi) + comp];
  };
  // FP32 kernel with precomputed edges: 16 bytes l (< 9) of the cell's 36.
  const bool pre = sizeof(T) == 4 && m.edges32 != nullptr;
  auto edges_of = [&](const Line& L) -> float4
  {
    if (!L.valid || l >= 9)
      return make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t cell = L.i + (int64_t)m.nx * (L.j + (int64_t)m.ny * L.k);
    return __ldg(reinterpret_cast<const float4*>(m.edges32) + 9 * cell + l);
  };

  const T* geo = nullptr;
  if constexpr (sizeof(T) == 4)
    geo = m.geom32;
  else
    geo = m.geom64;
  constexpr bool gq = GQ;

  // Per-thread quadrature data of the phase-3 line (x = la, y = lb).
  const T X = Tb::G(la), Y = Tb::G(lb);
  const T qwl = Tb::W(la) * Tb::W(lb) * (T)m.kappa;

  CellIter it;
  {
    const int b = kBatch * blockIdx.x + c;
    it.x = b % col.hx;
    it.y = (b / col.hx) % col.hy;
    it.z = b / (col.hx * col.hy);
  }
  Line L = line_of(it);
  T un[5];
  double vn = 0.0;
  float4 en = make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (!GQ)
  {
    if (pre)
      en = edges_of(L);
    else
      vn = vert_of(L);
  }
#pragma unroll
  for (int a = 0; a < 5; ++a)
    un[a] = L.valid ? u[L.base + a] : T(0);
  for (int bt = blockIdx.x; bt < batches; bt += gridDim.x)
  {
    T ucur[5], yold[5];
    bool bnd[5];
#pragma unroll
    for (int a = 0; a < 5; ++a)
    {
      ucur[a] = un[a];
      bnd[a] = L.row_bnd || (a == 0 && L.x_lo) || (a == 4 && L.x_hi);
      // No other CTA of this colour touches this cell's nodes.
      yold[a] = (L.valid && !bnd[a]) ? y[L.base + a] : T(0);
    }
    if constexpr (sizeof(T) == 4)
    {
      if (!gq && pre && act && l < 9)
        reinterpret_cast<float4*>(&se[c][0][0])[l] = en;
    }
    if (!gq && !pre && act && l < 24)
      sv[c][l] = vn;
    // Inputs of the next batch, in flight while this one is processed.
    const Line Lc = L;
    it.advance(col);
    L = line_of(it);
    if (bt + (int)gridDim.x < batches)
    {
#pragma unroll
      for (int a = 0; a < 5; ++a)
        un[a] = L.valid ? u[L.base + a] : T(0);
      if constexpr (!GQ)
      {
        if (pre)
          en = edges_of(L);
        else
          vn = vert_of(L);
      }
    }
    __syncthreads();
    // Edge vectors: differences of the FP64 vertices, rounded once to T.
    for (int e = (pre || gq) ? kBatch * 36 : t; e < kBatch * 36; e += blockDim.x)
    {
      const int cc = e / 36, r = e % 36, comp = r / 12, ed = r % 12;
      const int lo = edge_lo(ed), hi = lo + (1 << (ed >> 2));
      se[cc][comp][ed] = (T)(sv[cc][3 * hi + comp] - sv[cc][3 * lo + comp]);
    }
    // Phase 1: contract x on the (y, z) = (la, lb) line.
    if (Lc.valid)
    {
      T v[5];
#pragma unroll
      for (int a = 0; a < 5; ++a)
        v[a] = bnd[a] ? T(0) : ucur[a];
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        T a0 = 0, a1 = 0;
#pragma unroll
        for (int a = 0; a < 5; ++a)
        {
          a0 += Tb::B(q, a) * v[a];
          a1 += Tb::D(q, a) * v[a];
        }
        S0[lay_a<T>(q, la, lb)] = a0;
        S1[lay_a<T>(q, la, lb)] = a1;
      }
    }
    __syncthreads();
    const bool cv = Lc.valid;
    // The cached geometric factors of this thread's phase-3 line (points
    // la + 5 lb + 25 q of the cell), loaded here so that phase 2 covers
    // their latency.
    T gm[GQ ? 6 : 1][5];
    if constexpr (GQ)
      if (cv)
      {
        const T* gp = geo + 750 * (Lc.i + (int64_t)m.nx * (Lc.j + (int64_t)m.ny * Lc.k)) + l;
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
          for (int q = 0; q < 5; ++q)
            gm[k][q] = __ldg(gp + 125 * k + 25 * q);
      }
    // Phase 2: contract y on the (x, z) = (la, lb) line.
    if (cv)
    {
      T va[5], vd[5];
#pragma unroll
      for (int b = 0; b < 5; ++b)
      {
        va[b] = S0[lay_a<T>(la, b, lb)];
        vd[b] = S1[lay_a<T>(la, b, lb)];
      }
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        T c0 = 0, cy = 0, cx = 0;
#pragma unroll
        for (int b = 0; b < 5; ++b)
        {
          c0 += Tb::B(q, b) * va[b];
          cy += Tb::D(q, b) * va[b];
          cx += Tb::B(q, b) * vd[b];
        }
        S2[lay_b<T>(la, q, lb)] = c0;
        S3[lay_b<T>(la, q, lb)] = cy;
        S4[lay_b<T>(la, q, lb)] = cx;
      }
    }
    __syncthreads();
    // Phase 3: contract z on the (x, y) = (la, lb) line, apply the
    // geometry at its 5 quadrature points, transpose z.
    if (cv)
    {
      T c0[5], cy[5], cx[5];
#pragma unroll
      for (int r = 0; r < 5; ++r)
      {
        c0[r] = S2[lay_b<T>(la, lb, r)];
        cy[r] = S3[lay_b<T>(la, lb, r)];
        cx[r] = S4[lay_b<T>(la, lb, r)];
      }
      T vx[5], vy[5], vz[5];
      if constexpr (GQ)
      {
#pragma unroll
        for (int q = 0; q < 5; ++q)
        {
          T ux = 0, uy = 0, uz = 0;
#pragma unroll
          for (int r = 0; r < 5; ++r)
          {
            ux += Tb::B(q, r) * cx[r];
            uy += Tb::B(q, r) * cy[r];
            uz += Tb::D(q, r) * c0[r];
          }
          vx[q] = gm[0][q] * ux + gm[1][q] * uy + gm[2][q] * uz;
          vy[q] = gm[1][q] * ux + gm[3][q] * uy + gm[4][q] * uz;
          vz[q] = gm[2][q] * ux + gm[4][q] * uy + gm[5][q] * uz;
        }
      }
      else
      {
        // Jacobian columns along the line: d/dX and d/dY are linear in Z,
        // d/dZ does not depend on Z.
        T P0[3], dP[3], Q0[3], dQ[3], R[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp)
        {
          T e[12];
          load_edges(se[c][comp], e);
          const T p0 = (1 - Y) * e[0] + Y * e[1], p1 = (1 - Y) * e[2] + Y * e[3];
          const T q0 = (1 - X) * e[4] + X * e[5], q1 = (1 - X) * e[6] + X * e[7];
          P0[comp] = p0;
          dP[comp] = p1 - p0;
          Q0[comp] = q0;
          dQ[comp] = q1 - q0;
          R[comp] = (1 - X) * (1 - Y) * e[8] + X * (1 - Y) * e[9] + (1 - X) * Y * e[10]
                    + X * Y * e[11];
        }
#pragma unroll
        for (int q = 0; q < 5; ++q)
        {
          T ux = 0, uy = 0, uz = 0;
#pragma unroll
          for (int r = 0; r < 5; ++r)
          {
            ux += Tb::B(q, r) * cx[r];
            uy += Tb::B(q, r) * cy[r];
            uz += Tb::D(q, r) * c0[r];
          }
          const T Z = Tb::G(q);
          T J[3][3];
#pragma unroll
          for (int comp = 0; comp < 3; ++comp)
          {
            J[comp][0] = P0[comp] + Z * dP[comp];
            J[comp][1] = Q0[comp] + Z * dQ[comp];
            J[comp][2] = R[comp];
          }
          T adj[3][3];
          adj[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
          adj[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
          adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
          adj[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
          adj[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
          adj[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
          adj[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
          adj[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
          adj[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
          const T det = J[0][0] * adj[0][0] + J[0][1] * adj[1][0] + J[0][2] * adj[2][0];
          // G grad = w kappa |det| K K^T grad = sc adj (adj^T grad), K = J^{-1} =
          // adj / det, sc = w kappa / |det|.
          const T sc = div_abs(qwl * Tb::W(q), det);
          const T w0 = sc * (adj[0][0] * ux + adj[1][0] * uy + adj[2][0] * uz);
          const T w1 = sc * (adj[0][1] * ux + adj[1][1] * uy + adj[2][1] * uz);
          const T w2 = sc * (adj[0][2] * ux + adj[1][2] * uy + adj[2][2] * uz);
          vx[q] = adj[0][0] * w0 + adj[0][1] * w1 + adj[0][2] * w2;
          vy[q] = adj[1][0] * w0 + adj[1][1] * w1 + adj[1][2] * w2;
          vz[q] = adj[2][0] * w0 + adj[2][1] * w1 + adj[2][2] * w2;
        }
      }
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        T ex = 0, ey = 0, ez = 0;
#pragma unroll
        for (int q = 0; q < 5; ++q)
        {
          ex += Tb::B(q, a) * vx[q];
          ey += Tb::B(q, a) * vy[q];
          ez += Tb::D(q, a) * vz[q];
        }
        S0[lay_b<T>(la, lb, a)] = ex;
        S1[lay_b<T>(la, lb, a)] = ey;
        S5[lay_b<T>(la, lb, a)] = ez;
      }
    }
    __syncthreads();
    // Phase 4: transpose y on the (x, z) = (la, lb) line.
    if (cv)
    {
      T ex[5], ey[5], ez[5];
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        ex[q] = S0[lay_b<T>(la, q, lb)];
        ey[q] = S1[lay_b<T>(la, q, lb)];
        ez[q] = S5[lay_b<T>(la, q, lb)];
      }
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        T x1 = 0, x2 = 0;
#pragma unroll
        for (int q = 0; q < 5; ++q)
        {
          x1 += Tb::B(q, a) * ex[q];
          x2 += Tb::D(q, a) * ey[q] + Tb::B(q, a) * ez[q];
        }
        S2[lay_a<T>(la, a, lb)] = x1;
        S3[lay_a<T>(la, a, lb)] = x2;
      }
    }
    __syncthreads();
    // Phase 5: transpose x on the (y, z) = (la, lb) line; scatter.
    if (Lc.valid)
    {
      T x1[5], x2[5];
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        x1[q] = S2[lay_a<T>(q, la, lb)];
        x2[q] = S3[lay_a<T>(q, la, lb)];
      }
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        T ye = 0;
#pragma unroll
        for (int q = 0; q < 5; ++q)
          ye += Tb::D(q, a) * x1[q] + Tb::B(q, a) * x2[q];
        y[Lc.base + a] = bnd[a] ? ucur[a] : yold[a] + ye;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Tensor-core variant of the FP32 action (k_q4_cells_tc). The same
// sum-factorised phases, but every 1D basis contraction of a batch of 5
// cells is one tcgen05.mma (a few K steps): the 125 lines of the batch are
// the 128 rows of M, the split words of a line's inputs are K, and the
// outputs (5 quadrature points or nodes per table, up to 3 tables) are
// N = 16. TF32 keeps 10 mantissa bits, so each operand is split,
// v = hi + lo with hi = tf32(v), and the products hi*hi + lo*hi + hi*lo are
// summed by the tensor core within the same MMA: A carries (hi, lo, hi) of
// each input, B the matching (hi, hi, lo) of the table, split in FP64 on the
// host. The error is ~2^-21 relative, the FP32 kernel's order.
//   P1  x: lines (y, z) of u            -> A(qx), Ad(qx)
//   P2  y: lines (qx, z)                -> C0, Cy, Cx (qy)
//   P3  z: lines (qx, qy)               -> uz, uy, ux (qz); geometry at the
//                                          5 points of the line (CUDA cores)
//   P3T z^T: same lines                 -> ex, ey, ez (z)
//   P4T y^T: lines (qx, z)              -> x1, x2 (y)
//   P5T x^T: lines (y, z)               -> y_e (x), scattered
// Thread t owns TMEM lane / row t in every phase; between phases a thread
// writes its row's outputs into the rows of the next phase's lines in
// shared memory (the transposes of the CUDA-core kernel), 16 bytes at a time.
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: no swizzle, K-major.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16)
         | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// kind::tf32, D FP32, A and B TF32 K-major, M = 128, N = 16.
constexpr uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17)
                              | ((128u >> 4) << 24);

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\t"
               "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}\n"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}

// Bounded wait for the MMA completion of phase `parity`.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
  for (int i = 0; i < kTcWaitPolls; ++i)
    if (mbar_try(bar, parity))
      return true;
  return false;
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
               "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                 "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i)
    v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_rna(float v)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

// Split words (hi, lo, hi) of the inputs of one position, packed into
// 4-float core-matrix rows: 1 input -> 1 row, 2 -> 2, 3 -> 3 (unused 0).
template <int T>
__device__ __forceinline__ void tc_store(char* at, const float (&in)[T])
{
  float w[4 * ((3 * T + 3) / 4)];
#pragma unroll
  for (int i = 0; i < (int)(sizeof(w) / sizeof(float)); ++i)
    w[i] = 0.f;
#pragma unroll
  for (int tau = 0; tau < T; ++tau)
  {
    const float hi = tf32_rna(in[tau]);
    w[3 * tau] = hi;
    w[3 * tau + 1] = in[tau] - hi;
    w[3 * tau + 2] = hi;
  }
#pragma unroll
  for (int c = 0; c < (3 * T + 3) / 4; ++c)
    *reinterpret_cast<float4*>(at + c * kTcLboA) =
        make_float4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
}

__device__ __forceinline__ void tc_zero(char* at)
{
  *reinterpret_cast<float4*>(at) = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void __launch_bounds__(128, 4)
    k_q4_cells_tc(const dfx_q4_mesh_s m, const float* __restrict__ u, float* __restrict__ y,
                  const Colour col, const int32_t* __restrict__ skip)
{
  if (skip && __ldg(skip))
    return;
  extern __shared__ __align__(1024) float tc_smem[]; // kTcSmemBytes: A operand, then tables
  float* const sA = tc_smem;
  float* const sT = tc_smem + kTcAFloats;
  __shared__ __align__(16) float se[kBatch][3][12];
  __shared__ double sv[kBatch][24];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  const int t = threadIdx.x;
  const bool act = t < kBatch * 25;
  const int c = act ? t / 25 : 0, l = t % 25;
  const int la = l % 5, lb = l / 5;

  for (int i = t; i < kTcTabFloats; i += blockDim.x)
    sT[i] = g_q4tc_tab[i];
  for (int i = t; i < kTcAFloats; i += blockDim.x)
    sA[i] = 0.f;
  const uint32_t bar = smem_addr(&mbar);
  if (t == 0)
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  if (t < 32)
  {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(
                     smem_addr(&tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t trow = tmem + ((uint32_t)(t & ~31) << 16); // this warp's 32 lanes
  const uint32_t sa = smem_addr(sA), st = smem_addr(sT);
  char* const A = reinterpret_cast<char*>(sA);
  // Write bases: own row t; rows (c, q, lb) at position la (P2 and P5T
  // operands: 2 columns per position); rows (c, la, q) at position lb (P3,
  // P4T operands: 3 columns per position). Row q of a set is +16 q or +80 q.
  char* const own = A + 16 * t;
  char* const to_p2 = A + 16 * (25 * c + 5 * lb) + 2 * la * kTcLboA;
  char* const to_p3 = A + 16 * (25 * c + la) + 3 * lb * kTcLboA;
  uint32_t parity = 0;
  bool timed_out = false;
  int issued = 0; // 1 while an MMA commit has not been observed complete

  // One phase: operands written by every thread -> MMA by thread 0 -> the
  // thread's TMEM row in v. Returns false (in every thread) once any
  // thread's wait has given up.
  auto run_phase = [&](int p, float (&v)[16]) -> bool
  {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if (__syncthreads_or(timed_out))
      return false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t dcol = tmem + (uint32_t)((p & 1) * 16);
    if (t == 0)
    {
      const uint32_t tb = st + 4u * tc_tab_off(p);
      for (int ks = 0; ks < tc_kcols(p) / 2; ++ks)
      {
        const uint64_t da = tc_desc(sa + 2u * ks * kTcLboA, kTcLboA, 128);
        const uint64_t db = tc_desc(tb + 2u * ks * kTcLboB, kTcLboB, 128);
        asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n\t}\n" ::"r"(dcol),
                     "l"(da), "l"(db), "r"(kTcIdesc), "r"(ks)
                     : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::
                       "r"(bar)
                   : "memory");
    }
    issued = 1;
    // Warp-uniform outcome: the TMEM load below is a warp-collective.
    if (!__all_sync(0xffffffffu, mbar_wait(bar, parity)))
    {
      timed_out = true;
      return true; // the vote at the next phase (or before the scatter) stops every thread
    }
    issued = 0;
    parity ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tc_ld16(trow + (uint32_t)((p & 1) * 16), v);
    return true;
  };

  const int cells = col.hx * col.hy * col.hz;
  const int batches = (cells + kBatch - 1) / kBatch;
  const int NX = 4 * m.nx + 1, NY = 4 * m.ny + 1, NZ = 4 * m.nz + 1;
  struct Line
  {
    int64_t base;
    bool row_bnd, x_lo, x_hi, valid;
    int i, j, k;
  };
  auto line_of = [&](const CellIter& it) -> Line
  {
    Line L{0, false, false, false, false, 0, 0, 0};
    if (!act || it.z >= col.hz)
      return L;
    L.i = col.ci + 2 * it.x;
    L.j = col.cj + 2 * it.y;
    L.k = col.ck + 2 * it.z;
    const int J = 4 * L.j + la, K = 4 * L.k + lb;
    L.base = ((int64_t)K * NY + J) * NX + 4 * (int64_t)L.i;
    L.row_bnd = J == 0 || K == 0 || J == NY - 1 || K == NZ - 1;
    L.x_lo = L.i == 0;
    L.x_hi = L.i == m.nx - 1;
    L.valid = true;
    return L;
  };
  auto vert_of = [&](const Line& L) -> double
  {
    if (!L.valid || l >= 24)
      return 0.0;
    const int vtx = l / 3, comp = l % 3;
    const int64_t vi = L.i + (vtx & 1), vj = L.j + ((vtx >> 1) & 1), vk = L.k + ((vtx >> 2) & 1);
    return m.verts[3 * ((vk * (m.ny + 1) + vj) * (m.nx + 1) + vi) + comp];
  };
  const bool pre = m.edges32 != nullptr;
  auto edges_of = [&](const Line& L) -> float4
  {
    if (!L.valid || l >= 9)
      return make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t cell = L.i + (int64_t)m.nx * (L.j + (int64_t)m.ny * L.k);
    return __ldg(reinterpret_cast<const float4*>(m.edges32) + 9 * cell + l);
  };
  const float X = Tab<float>::G(la), Y = Tab<float>::G(lb);
  const float qwl = Tab<float>::W(la) * Tab<float>::W(lb) * (float)m.kappa;

  CellIter it;
  {
    const int b0 = kBatch * blockIdx.x + c;
    it.x = b0 % col.hx;
    it.y = (b0 / col.hx) % col.hy;
    it.z = b0 / (col.hx * col.hy);
  }
  Line L = line_of(it);
  float un[5];
  double vn = 0.0;
  float4 en = make_float4(0.f, 0.f, 0.f, 0.f);
  if (pre)
    en = edges_of(L);
  else
    vn = vert_of(L);
#pragma unroll
  for (int a = 0; a < 5; ++a)
    un[a] = L.valid ? u[L.base + a] : 0.f;

  for (int bt = blockIdx.x; bt < batches; bt += gridDim.x)
  {
    float ucur[5];
    uint32_t bndm = 0; // bit a: node a of the line is a boundary node
#pragma unroll
    for (int a = 0; a < 5; ++a)
    {
      ucur[a] = un[a];
      if (L.row_bnd || (a == 0 && L.x_lo) || (a == 4 && L.x_hi))
        bndm |= 1u << a;
    }
    if (pre && act && l < 9)
      reinterpret_cast<float4*>(&se[c][0][0])[l] = en;
    if (!pre && act && l < 24)
      sv[c][l] = vn;
    const Line Lc = L;
    it.advance(col);
    L = line_of(it);
    if (bt + (int)gridDim.x < batches)
    {
#pragma unroll
      for (int a = 0; a < 5; ++a)
        un[a] = L.valid ? u[L.base + a] : 0.f;
      if (pre)
        en = edges_of(L);
      else
        vn = vert_of(L);
    }
    // P1 operand: this thread's line of u (boundary entries read as 0).
    if (act)
    {
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        const float in[1] = {(Lc.valid && !((bndm >> a) & 1)) ? ucur[a] : 0.f};
        tc_store<1>(own + a * kTcLboA, in);
      }
      tc_zero(own + 5 * kTcLboA);
    }
    __syncthreads(); // se / sv of this batch are complete
    if (!pre)
      for (int e = t; e < kBatch * 36; e += blockDim.x)
      {
        const int cc = e / 36, r = e % 36, comp = r / 12, ed = r % 12;
        const int lo = edge_lo(ed), hi = lo + (1 << (ed >> 2));
        se[cc][comp][ed] = (float)(sv[cc][3 * hi + comp] - sv[cc][3 * lo + comp]);
      }
    float v[16];
    if (!run_phase(0, v))
      break;
    // P1 -> P2: row (c, qx, z) gets A(qx), Ad(qx) at position y.
    if (act)
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        const float in[2] = {v[q], v[5 + q]};
        tc_store<2>(to_p2 + 16 * q, in);
      }
    if (!run_phase(1, v))
      break;
    // P2 -> P3: row (c, qx, qy) gets C0, Cy, Cx (qy) at position z.
    if (act)
    {
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        const float in[3] = {v[q], v[5 + q], v[10 + q]};
        tc_store<3>(to_p3 + 80 * q, in);
      }
      tc_zero(own + 15 * kTcLboA);
    }
    if (!run_phase(2, v))
      break;
    // P3: gradient at the 5 points of line (qx, qy) -> geometry -> own row.
    if (act)
    {
      float P0[3], dP[3], Q0[3], dQ[3], R[3];
#pragma unroll
      for (int comp = 0; comp < 3; ++comp)
      {
        float e[12];
        load_edges(se[c][comp], e);
        const float p0 = (1 - Y) * e[0] + Y * e[1], p1 = (1 - Y) * e[2] + Y * e[3];
        const float q0 = (1 - X) * e[4] + X * e[5], q1 = (1 - X) * e[6] + X * e[7];
        P0[comp] = p0;
        dP[comp] = p1 - p0;
        Q0[comp] = q0;
        dQ[comp] = q1 - q0;
        R[comp] = (1 - X) * (1 - Y) * e[8] + X * (1 - Y) * e[9] + (1 - X) * Y * e[10]
                  + X * Y * e[11];
      }
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        const float uz = v[q], uy = v[5 + q], ux = v[10 + q];
        const float Z = Tab<float>::G(q);
        float J[3][3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp)
        {
          J[comp][0] = P0[comp] + Z * dP[comp];
          J[comp][1] = Q0[comp] + Z * dQ[comp];
          J[comp][2] = R[comp];
        }
        float adj[3][3];
        adj[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        adj[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
        adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
        adj[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        adj[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
        adj[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
        adj[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        adj[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
        adj[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const float det = J[0][0] * adj[0][0] + J[0][1] * adj[1][0] + J[0][2] * adj[2][0];
        const float sc = div_abs(qwl * Tab<float>::W(q), det);
        const float w0 = sc * (adj[0][0] * ux + adj[1][0] * uy + adj[2][0] * uz);
        const float w1 = sc * (adj[0][1] * ux + adj[1][1] * uy + adj[2][1] * uz);
        const float w2 = sc * (adj[0][2] * ux + adj[1][2] * uy + adj[2][2] * uz);
        const float in[3] = {adj[0][0] * w0 + adj[0][1] * w1 + adj[0][2] * w2,
                             adj[1][0] * w0 + adj[1][1] * w1 + adj[1][2] * w2,
                             adj[2][0] * w0 + adj[2][1] * w1 + adj[2][2] * w2};
        tc_store<3>(own + 3 * q * kTcLboA, in);
      }
    }
    if (!run_phase(3, v))
      break;
    // P3T -> P4T: row (c, qx, z) gets ex, ey, ez (z) at position qy.
    if (act)
#pragma unroll
      for (int z = 0; z < 5; ++z)
      {
        const float in[3] = {v[z], v[5 + z], v[10 + z]};
        tc_store<3>(to_p3 + 80 * z, in);
      }
    if (!run_phase(4, v))
      break;
    // P4T -> P5T: row (c, y, z) gets x1, x2 (y) at position qx.
    if (act)
#pragma unroll
      for (int yy = 0; yy < 5; ++yy)
      {
        const float in[2] = {v[yy], v[5 + yy]};
        tc_store<2>(to_p2 + 16 * yy, in);
      }
    if (!run_phase(5, v))
      break;
    if (__syncthreads_or(timed_out))
      break;
    if (Lc.valid)
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        const bool bn = (bndm >> a) & 1;
        const float yo = bn ? 0.f : y[Lc.base + a]; // no other CTA of this colour writes it
        y[Lc.base + a] = bn ? ucur[a] : yo + v[a];
      }
  }
  if (timed_out && t == 0)
    atomicExch(&g_q4tc_error, 1);
  // An MMA whose completion was not observed may still be writing TMEM:
  // wait for it (bounded) before the columns are released.
  if (issued)
    mbar_wait(bar, parity);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (t < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
}

// Edge vectors of every cell in FP32, [cell][component][edge], cells
// lexicographic: the differences of the FP64 vertices rounded once, exactly
// what the colour kernel forms on the fly.
__global__ void k_q4_edges(const dfx_q4_mesh_s m, float* __restrict__ edges, int64_t cells)
{
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= cells * 36)
    return;
  const int64_t cell = g / 36;
  const int r = (int)(g % 36), comp = r / 12, ed = r % 12;
  const int64_t i = cell % m.nx, j = (cell / m.nx) % m.ny, k = cell / ((int64_t)m.nx * m.ny);
  const int lo = edge_lo(ed), hi = lo + (1 << (ed >> 2));
  auto coord = [&](int v)
  {
    const int64_t vi = i + (v & 1), vj = j + ((v >> 1) & 1), vk = k + ((v >> 2) & 1);
    return m.verts[3 * ((vk * (m.ny + 1) + vj) * (m.nx + 1) + vi) + comp];
  };
  edges[g] = (float)(coord(hi) - coord(lo));
}

// Geometric factors of every quadrature point, [cell][6][125]: the
// Jacobian at the point from the cell's edge vectors (rounded once to T
// from the FP64 vertices), G = w kappa adj adj^T / |det| in T, stored as
// 00, 01, 02, 11, 12, 22. One thread per (cell, point); the formulas are
// those of the colour kernel's phase 3.
template <typename T>
__global__ void k_q4_geom(const dfx_q4_mesh_s m, T* __restrict__ geom, int64_t cells)
{
  using Tb = Tab<T>;
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= cells * 125)
    return;
  const int64_t cell = g / 125;
  const int p = (int)(g % 125), la = p % 5, lb = (p / 5) % 5, q = p / 25;
  const int64_t i = cell % m.nx, j = (cell / m.nx) % m.ny, k = cell / ((int64_t)m.nx * m.ny);
  auto coord = [&](int v, int comp)
  {
    const int64_t vi = i + (v & 1), vj = j + ((v >> 1) & 1), vk = k + ((v >> 2) & 1);
    return m.verts[3 * ((vk * (m.ny + 1) + vj) * (m.nx + 1) + vi) + comp];
  };
  const T X = Tb::G(la), Y = Tb::G(lb), Z = Tb::G(q);
  T J[3][3];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp)
  {
    T e[12];
#pragma unroll
    for (int ed = 0; ed < 12; ++ed)
    {
      const int lo = edge_lo(ed), hi = lo + (1 << (ed >> 2));
      e[ed] = (T)(coord(hi, comp) - coord(lo, comp));
    }
    const T p0 = (1 - Y) * e[0] + Y * e[1], p1 = (1 - Y) * e[2] + Y * e[3];
    const T q0 = (1 - X) * e[4] + X * e[5], q1 = (1 - X) * e[6] + X * e[7];
    J[comp][0] = p0 + Z * (p1 - p0);
    J[comp][1] = q0 + Z * (q1 - q0);
    J[comp][2] = (1 - X) * (1 - Y) * e[8] + X * (1 - Y) * e[9] + (1 - X) * Y * e[10]
                 + X * Y * e[11];
  }
  T adj[3][3];
  adj[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  adj[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  adj[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  adj[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  adj[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  adj[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  adj[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  adj[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const T det = J[0][0] * adj[0][0] + J[0][1] * adj[1][0] + J[0][2] * adj[2][0];
  const T qwl = Tb::W(la) * Tb::W(lb) * (T)m.kappa;
  const T sc = div_abs(qwl * Tb::W(q), det);
  auto dot3 = [&](int a, int b)
  { return sc * (adj[a][0] * adj[b][0] + adj[a][1] * adj[b][1] + adj[a][2] * adj[b][2]); };
  T* o = geom + 750 * cell + p;
  o[0] = dot3(0, 0);
  o[125] = dot3(0, 1);
  o[250] = dot3(0, 2);
  o[375] = dot3(1, 1);
  o[500] = dot3(1, 2);
  o[625] = dot3(2, 2);
}

// Grid of the tensor-core colour kernel: 4 resident CTAs per SM, the
// register bound of its launch bounds; 4 x (52 KB dynamic + 2 KB static +
// 1 KB reserved) shared memory fits the SM's 228 KB. (The occupancy query
// reported 1 CTA per SM for this kernel, which left 3/4 of each SM idle.)
int q4_tc_grid_limit()
{
  static int ok = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    ok = cudaFuncSetAttribute(k_q4_cells_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kTcSmemBytes)
         == cudaSuccess;
  });
  static_assert(4 * (kTcSmemBytes + 2048 + 1024) <= 228 * 1024, "4 CTAs per SM must fit");
  return (ok ? 4 : 1) * dfx::num_sms();
}

// Resident CTAs per SM of the colour kernel (queried once per type and
// geometry source).
template <typename T, bool GQ>
int q4_grid_limit()
{
  static int per_sm = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_q4_cells<T, GQ>, 128, 0)
        != cudaSuccess)
      per_sm = 1;
  });
  return std::max(1, per_sm) * dfx::num_sms();
}
} // namespace

namespace dfx
{
int q4_prepare()
{
  // Also settles the grid sizes, so that nothing below queries the device
  // during a stream capture.
  q4_grid_limit<float, false>();
  q4_grid_limit<double, false>();
  q4_grid_limit<float, true>();
  q4_grid_limit<double, true>();
  q4_tc_grid_limit();
  return upload_tables();
}

// The colours of the structured mesh: parity (ci, cj, ck) of the cell
// indices, with the mixed-radix digits of one grid-stride step.
template <typename F>
void for_each_colour(const dfx_q4_mesh_s& m, int64_t grid_cap, F&& launch)
{
  for (int c = 0; c < 8; ++c)
  {
    Colour col;
    col.ci = c & 1;
    col.cj = (c >> 1) & 1;
    col.ck = (c >> 2) & 1;
    col.hx = (m.nx - col.ci + 1) / 2;
    col.hy = (m.ny - col.cj + 1) / 2;
    col.hz = (m.nz - col.ck + 1) / 2;
    const int64_t cells = (int64_t)col.hx * col.hy * col.hz;
    if (cells == 0)
      continue;
    const int64_t grid = std::min<int64_t>((cells + kBatch - 1) / kBatch, grid_cap);
    const int64_t step = kBatch * grid;
    col.dx = (int)(step % col.hx);
    col.dy = (int)((step / col.hx) % col.hy);
    col.dz = (int)(step / ((int64_t)col.hx * col.hy));
    launch(col, (unsigned)grid);
  }
}

int q4_apply_tc(const dfx_q4_mesh_s& m, const float* u, float* y, cudaStream_t s,
                const int32_t* skip)
{
  if (int st = q4_prepare())
    return st;
  DFX_REQUIRE((int64_t)m.nx * m.ny * m.nz < ((int64_t)1 << 31) && 4 * (int64_t)m.nx + 1 < (1 << 30)
                  && 4 * (int64_t)m.ny + 1 < (1 << 30),
              "Q4 mesh too large (%d x %d x %d cells)", m.nx, m.ny, m.nz);
  DFX_CUDA(cudaMemsetAsync(y, 0, sizeof(float) * q4_ndofs(m), s));
  for_each_colour(m, q4_tc_grid_limit(), [&](const Colour& col, unsigned grid)
                  { k_q4_cells_tc<<<grid, 128, kTcSmemBytes, s>>>(m, u, y, col, skip); });
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

int q4_tc_check()
{
  int32_t flag = 0, zero = 0;
  DFX_CUDA(cudaMemcpyFromSymbol(&flag, g_q4tc_error, sizeof(flag)));
  if (flag)
  {
    DFX_CUDA(cudaMemcpyToSymbol(g_q4tc_error, &zero, sizeof(zero)));
    return dfx::fail(DFX_ERR_TIMEOUT, "a tensor-core Q4 kernel gave up waiting for its MMA");
  }
  return DFX_OK;
}

template <typename T>
int q4_apply(const dfx_q4_mesh_s& m, const T* u, T* y, cudaStream_t s, const int32_t* skip)
{
  if (int st = q4_prepare())
    return st;
  DFX_REQUIRE((int64_t)m.nx * m.ny * m.nz < ((int64_t)1 << 31) && 4 * (int64_t)m.nx + 1 < (1 << 30)
                  && 4 * (int64_t)m.ny + 1 < (1 << 30),
              "Q4 mesh too large (%d x %d x %d cells)", m.nx, m.ny, m.nz);
  const int64_t n = q4_ndofs(m);
  DFX_CUDA(cudaMemsetAsync(y, 0, sizeof(T) * n, s));
  for (int c = 0; c < 8; ++c)
  {
    Colour col;
    col.ci = c & 1;
    col.cj = (c >> 1) & 1;
    col.ck = (c >> 2) & 1;
    col.hx = (m.nx - col.ci + 1) / 2;
    col.hy = (m.ny - col.cj + 1) / 2;
    col.hz = (m.nz - col.ck + 1) / 2;
    const int64_t cells = (int64_t)col.hx * col.hy * col.hz;
    if (cells == 0)
      continue;
    const bool gq = sizeof(T) == 4 ? m.geom32 != nullptr : m.geom64 != nullptr;
    const int64_t grid = std::min<int64_t>((cells + kBatch - 1) / kBatch,
                                           gq ? q4_grid_limit<T, true>()
                                              : q4_grid_limit<T, false>());
    const int64_t step = kBatch * grid;
    col.dx = (int)(step % col.hx);
    col.dy = (int)((step / col.hx) % col.hy);
    col.dz = (int)(step / ((int64_t)col.hx * col.hy));
    if (gq)
      k_q4_cells<T, true><<<(unsigned)grid, 128, 0, s>>>(m, u, y, col, skip);
    else
      k_q4_cells<T, false><<<(unsigned)grid, 128, 0, s>>>(m, u, y, col, skip);
  }
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

template int q4_apply<float>(const dfx_q4_mesh_s&, const float*, float*, cudaStream_t,
                             const int32_t*);
template int q4_apply<double>(const dfx_q4_mesh_s&, const double*, double*, cudaStream_t,
                              const int32_t*);
} // namespace dfx

extern "C" int64_t dfx_q4_num_dofs(const dfx_q4_mesh* m) { return m ? dfx::q4_ndofs(*m) : 0; }

extern "C" int dfx_q4_edges(const dfx_q4_mesh* mesh, float* d_edges, void* stream)
{
  DFX_REQUIRE(mesh && d_edges, "arguments must be non-NULL");
  DFX_REQUIRE(mesh->nx > 0 && mesh->ny > 0 && mesh->nz > 0 && mesh->verts, "invalid Q4 mesh");
  DFX_REQUIRE(((uintptr_t)d_edges & 15) == 0, "edges must be 16-byte aligned");
  const int64_t cells = (int64_t)mesh->nx * mesh->ny * mesh->nz;
  const int64_t total = 36 * cells;
  k_q4_edges<<<(unsigned)((total + 255) / 256), 256, 0, dfx::as_stream(stream)>>>(*mesh, d_edges,
                                                                                   cells);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_q4_geometry(const dfx_q4_mesh* mesh, int32_t dtype, void* d_geom,
                               void* stream)
{
  DFX_REQUIRE(mesh && d_geom, "arguments must be non-NULL");
  DFX_REQUIRE(mesh->nx > 0 && mesh->ny > 0 && mesh->nz > 0 && mesh->verts, "invalid Q4 mesh");
  const int64_t cells = (int64_t)mesh->nx * mesh->ny * mesh->nz;
  DFX_REQUIRE(cells < ((int64_t)1 << 31), "Q4 mesh too large (%lld cells)", (long long)cells);
  // The quadrature tables live in constant memory, uploaded on first use.
  if (int st = dfx::q4_prepare())
    return st;
  const unsigned grid = (unsigned)((125 * cells + 255) / 256);
  cudaStream_t s = dfx::as_stream(stream);
  if (dtype == DFX_F64)
    k_q4_geom<double><<<grid, 256, 0, s>>>(*mesh, (double*)d_geom, cells);
  else if (dtype == DFX_F32)
    k_q4_geom<float><<<grid, 256, 0, s>>>(*mesh, (float*)d_geom, cells);
  else
    return dfx::fail(DFX_ERR_INVALID, "unknown dtype %d", dtype);
  DFX_CHECK_LAUNCH();
  return DFX_OK;
}

extern "C" int dfx_q4_action_tc(const dfx_q4_mesh* mesh, const float* d_u, float* d_y,
                                void* stream)
{
  DFX_REQUIRE(mesh && d_u && d_y, "arguments must be non-NULL");
  const dfx_q4_mesh_s& m = *mesh;
  DFX_REQUIRE(m.nx > 0 && m.ny > 0 && m.nz > 0 && m.verts, "invalid Q4 mesh");
  DFX_REQUIRE((const void*)d_u != (const void*)d_y, "u and y must differ");
  DFX_REQUIRE(((uintptr_t)m.edges32 & 15) == 0, "edges32 must be 16-byte aligned");
  return dfx::q4_apply_tc(m, d_u, d_y, dfx::as_stream(stream));
}

extern "C" int dfx_q4_tc_check(void* stream)
{
  DFX_CUDA(cudaStreamSynchronize(dfx::as_stream(stream)));
  return dfx::q4_tc_check();
}

extern "C" int dfx_q4_action(const dfx_q4_mesh* mesh, int32_t dtype, const void* d_u, void* d_y,
                             void* stream)
{
  DFX_REQUIRE(mesh && d_u && d_y, "arguments must be non-NULL");
  const dfx_q4_mesh_s& m = *mesh;
  DFX_REQUIRE(m.nx > 0 && m.ny > 0 && m.nz > 0 && m.verts, "invalid Q4 mesh");
  DFX_REQUIRE(d_u != d_y, "u and y must differ");
  DFX_REQUIRE(((uintptr_t)m.edges32 & 15) == 0, "edges32 must be 16-byte aligned");
  cudaStream_t s = dfx::as_stream(stream);
  if (dtype == DFX_F64)
    return dfx::q4_apply<double>(m, (const double*)d_u, (double*)d_y, s);
  if (dtype == DFX_F32)
    return dfx::q4_apply<float>(m, (const float*)d_u, (float*)d_y, s);
  return dfx::fail(DFX_ERR_INVALID, "unknown dtype %d", dtype);
}
