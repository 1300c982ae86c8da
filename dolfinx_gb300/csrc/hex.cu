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

template <typename T>
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
  if (pre)
    en = edges_of(L);
  else
    vn = vert_of(L);
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
      if (pre && act && l < 9)
        reinterpret_cast<float4*>(&se[c][0][0])[l] = en;
    }
    if (!pre && act && l < 24)
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
      if (pre)
        en = edges_of(L);
      else
        vn = vert_of(L);
    }
    __syncthreads();
    // Edge vectors: differences of the FP64 vertices, rounded once to T.
    for (int e = pre ? kBatch * 36 : t; e < kBatch * 36; e += blockDim.x)
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
      T vx[5], vy[5], vz[5];
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

// Resident CTAs per SM of the colour kernel (queried once per type).
template <typename T>
int q4_grid_limit()
{
  static int per_sm = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_q4_cells<T>, 128, 0)
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
  q4_grid_limit<float>();
  q4_grid_limit<double>();
  return upload_tables();
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
    const int64_t grid = std::min<int64_t>((cells + kBatch - 1) / kBatch, q4_grid_limit<T>());
    const int64_t step = kBatch * grid;
    col.dx = (int)(step % col.hx);
    col.dy = (int)((step / col.hx) % col.hy);
    col.dz = (int)(step / ((int64_t)col.hx * col.hy));
    k_q4_cells<T><<<(unsigned)grid, 128, 0, s>>>(m, u, y, col, skip);
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
