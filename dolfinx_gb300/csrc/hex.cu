// Q4 hexahedral Laplacian action by sum factorisation.
//
// One CTA per cell, one thread per quadrature point / node of the 5x5x5
// tensor lattice. The gradient at the 125 quadrature points costs 8
// one-dimensional contractions (5 FMAs each per thread) instead of the
// 125 x 125 x 3 products of the full element matrix; the transpose costs 8
// more. The Jacobian of the trilinear map is formed at each quadrature
// point in the kernel's precision from the cell's 8 vertices (differences
// taken in FP64). Cells are processed in 8 colours (parity of i, j, k):
// cells of one colour share no node, so the scatter is a plain
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

// Per-thread rows of the 1D tables. The forward phases need B(q, a) and
// D(q, a) for the thread's quadrature index q in each direction; the
// transpose phases need B(q, a) and D(q, a) for the thread's node index a.
// FP32: held in registers for the whole kernel (each CTA processes many
// cells). FP64: read from shared memory (the FP64 pipe bounds that kernel).
template <typename T, bool REG>
struct Rows;

template <typename T>
struct Rows<T, true>
{
  T f[3][2][5]; // f[d][0][a] = B(t_d, a), f[d][1][a] = D(t_d, a)
  T c[3][2][5]; // c[d][0][q] = B(q, t_d), c[d][1][q] = D(q, t_d)
  __device__ void init(const T* sB, const T* sD, const int (&td)[3])
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        f[d][0][a] = sB[5 * td[d] + a];
        f[d][1][a] = sD[5 * td[d] + a];
        c[d][0][a] = sB[5 * a + td[d]];
        c[d][1][a] = sD[5 * a + td[d]];
      }
  }
  __device__ T fB(int d, int a) const { return f[d][0][a]; }
  __device__ T fD(int d, int a) const { return f[d][1][a]; }
  __device__ T cB(int d, int q) const { return c[d][0][q]; }
  __device__ T cD(int d, int q) const { return c[d][1][q]; }
};

template <typename T>
struct Rows<T, false>
{
  const T* B;
  const T* D;
  int td[3];
  __device__ void init(const T* sB, const T* sD, const int (&t)[3])
  {
    B = sB;
    D = sD;
    td[0] = t[0];
    td[1] = t[1];
    td[2] = t[2];
  }
  __device__ T fB(int d, int a) const { return B[5 * td[d] + a]; }
  __device__ T fD(int d, int a) const { return D[5 * td[d] + a]; }
  __device__ T cB(int d, int q) const { return B[5 * q + td[d]]; }
  __device__ T cD(int d, int q) const { return D[5 * q + td[d]]; }
};

// Edge e of a hexahedron (vertex v = bx + 2 by + 4 bz): e / 4 is its
// direction, e % 4 its position; returns the lower vertex (the upper is
// lower + 1, + 2 or + 4).
__device__ __forceinline__ int edge_lo(int e)
{
  const int d = e >> 2, m = e & 3;
  return d == 0 ? 2 * m : (d == 1 ? (m & 1) + 4 * (m >> 1) : m);
}

// The 12 edge components of one coordinate, read with 16-byte loads (the
// same address in every lane: one broadcast per load).
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

// One CTA processes the cells of one colour in turn; thread t < 125 owns
// quadrature point / node (t1, t2, t3) of the 5^3 lattice.
template <typename T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 3 : 2)
    k_q4_cells(const dfx_q4_mesh_s m, const T* __restrict__ u, T* __restrict__ y, int ci, int cj,
               int ck, const int32_t* __restrict__ skip)
{
  if (skip && __ldg(skip))
    return;
  constexpr bool REG = sizeof(T) == 4;
  __shared__ T su[128], sA[128], sAd[128], sC[128], sCx[128], sCy[128];
  __shared__ T sB[25], sD[25];
  __shared__ __align__(16) T se[3][12]; // edge vectors of the cell, by component
  __shared__ double sv[8][3];
  const int t = threadIdx.x;
  const bool act = t < 125;
  const int tt = act ? t : 0;
  const int td[3] = {tt % 5, (tt / 5) % 5, tt / 25};
  const int t1 = td[0], t2 = td[1], t3 = td[2];
  if (t < 25)
  {
    sB[t] = Tab<T>::B(t / 5, t % 5);
    sD[t] = Tab<T>::D(t / 5, t % 5);
  }
  // Trilinear-map weights of the Jacobian columns at this quadrature point.
  T wx[4], wy[4], wz[4];
  {
    const T X = Tab<T>::G(t1), Y = Tab<T>::G(t2), Z = Tab<T>::G(t3);
    wx[0] = (1 - Y) * (1 - Z), wx[1] = Y * (1 - Z), wx[2] = (1 - Y) * Z, wx[3] = Y * Z;
    wy[0] = (1 - X) * (1 - Z), wy[1] = X * (1 - Z), wy[2] = (1 - X) * Z, wy[3] = X * Z;
    wz[0] = (1 - X) * (1 - Y), wz[1] = X * (1 - Y), wz[2] = (1 - X) * Y, wz[3] = X * Y;
  }
  const T qw = Tab<T>::W(t1) * Tab<T>::W(t2) * Tab<T>::W(t3) * (T)m.kappa;
  __syncthreads();
  Rows<T, REG> R;
  R.init(sB, sD, td);

  const int hx = (m.nx - ci + 1) / 2, hy = (m.ny - cj + 1) / 2, hz = (m.nz - ck + 1) / 2;
  const int64_t cells = (int64_t)hx * hy * hz;
  const int64_t NX = 4 * (int64_t)m.nx + 1, NY = 4 * (int64_t)m.ny + 1, NZ = 4 * (int64_t)m.nz + 1;
  // This thread's node of cell b, and whether it lies on the boundary.
  auto node = [&](int64_t b, int64_t& gid, bool& bnd)
  {
    const int64_t i = ci + 2 * (b % hx), j = cj + 2 * ((b / hx) % hy);
    const int64_t k = ck + 2 * (b / ((int64_t)hx * hy));
    const int64_t I = 4 * i + t1, J = 4 * j + t2, K = 4 * k + t3;
    gid = (K * NY + J) * NX + I;
    bnd = I == 0 || J == 0 || K == 0 || I == NX - 1 || J == NY - 1 || K == NZ - 1;
  };
  // Loads of cell b's inputs (node value; one vertex coordinate for t < 24),
  // issued one cell ahead so that their latency overlaps a cell's work.
  auto fetch = [&](int64_t b, T& un, double& vn)
  {
    if (b >= cells)
      return;
    if (act)
    {
      int64_t g;
      bool bd;
      node(b, g, bd);
      un = u[g];
    }
    if (t < 24)
    {
      const int64_t i = ci + 2 * (b % hx), j = cj + 2 * ((b / hx) % hy);
      const int64_t k = ck + 2 * (b / ((int64_t)hx * hy));
      const int v = t / 3, c = t % 3;
      const int64_t vi = i + (v & 1), vj = j + ((v >> 1) & 1), vk = k + ((v >> 2) & 1);
      vn = m.verts[3 * ((vk * (m.ny + 1) + vj) * (m.nx + 1) + vi) + c];
    }
  };
  T un = 0;
  double vn = 0.0;
  fetch(blockIdx.x, un, vn);
  for (int64_t b = blockIdx.x; b < cells; b += gridDim.x)
  {
    int64_t gid = 0;
    bool bnd = false;
    const T ucur = un;
    T yold = 0;
    if (t < 24)
      sv[t / 3][t % 3] = vn;
    if (act)
    {
      node(b, gid, bnd);
      su[t] = bnd ? T(0) : ucur;
      // No other CTA of this colour touches this cell's nodes.
      if (!bnd)
        yold = y[gid];
    }
    fetch(b + gridDim.x, un, vn);
    __syncthreads();
    // Edge vectors: differences of the FP64 vertices, rounded once to T.
    if (t < 36)
    {
      const int c = t / 12, e = t % 12;
      const int lo = edge_lo(e), hi = lo + (1 << (e >> 2));
      se[c][e] = (T)(sv[hi][c] - sv[lo][c]);
    }
    // Gradient in reference coordinates: contract x, then y, then z.
    if (act)
    {
      T a0 = 0, a1 = 0;
#pragma unroll
      for (int a = 0; a < 5; ++a)
      {
        const T v = su[25 * t3 + 5 * t2 + a];
        a0 += R.fB(0, a) * v;
        a1 += R.fD(0, a) * v;
      }
      sA[t] = a0;
      sAd[t] = a1;
    }
    __syncthreads();
    if (act)
    {
      T c0 = 0, cy = 0, cx = 0;
#pragma unroll
      for (int bb = 0; bb < 5; ++bb)
      {
        const T va = sA[25 * t3 + 5 * bb + t1], vd = sAd[25 * t3 + 5 * bb + t1];
        c0 += R.fB(1, bb) * va;
        cy += R.fD(1, bb) * va;
        cx += R.fB(1, bb) * vd;
      }
      sC[t] = c0;
      sCy[t] = cy;
      sCx[t] = cx;
    }
    __syncthreads();
    if (act)
    {
      T ux = 0, uy = 0, uz = 0;
#pragma unroll
      for (int c = 0; c < 5; ++c)
      {
        const int o = 25 * c + 5 * t2 + t1;
        ux += R.fB(2, c) * sCx[o];
        uy += R.fB(2, c) * sCy[o];
        uz += R.fD(2, c) * sC[o];
      }
      T J[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
      {
        T e[12];
        load_edges(se[c], e);
        J[c][0] = wx[0] * e[0] + wx[1] * e[1] + wx[2] * e[2] + wx[3] * e[3];
        J[c][1] = wy[0] * e[4] + wy[1] * e[5] + wy[2] * e[6] + wy[3] * e[7];
        J[c][2] = wz[0] * e[8] + wz[1] * e[9] + wz[2] * e[10] + wz[3] * e[11];
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
      // G = w kappa |det| K K^T = w kappa adj adj^T / |det|, K = J^{-1}
      const T sc = qw / fabs(det);
      T G[3][3];
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = p; q < 3; ++q)
          G[p][q] = sc * (adj[p][0] * adj[q][0] + adj[p][1] * adj[q][1] + adj[p][2] * adj[q][2]);
      // su, sA, sAd were last read before the previous barrier.
      sA[t] = G[0][0] * ux + G[0][1] * uy + G[0][2] * uz;
      sAd[t] = G[0][1] * ux + G[1][1] * uy + G[1][2] * uz;
      su[t] = G[0][2] * ux + G[1][2] * uy + G[2][2] * uz;
    }
    __syncthreads();
    // Transpose: contract z, then y, then x.
    if (act)
    {
      T ex = 0, ey = 0, ez = 0;
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        const int o = 25 * q + 5 * t2 + t1;
        ex += R.cB(2, q) * sA[o];
        ey += R.cB(2, q) * sAd[o];
        ez += R.cD(2, q) * su[o];
      }
      sCx[t] = ex;
      sCy[t] = ey;
      sC[t] = ez;
    }
    __syncthreads();
    if (act)
    {
      T x1 = 0, x2 = 0;
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        const int o = 25 * t3 + 5 * q + t1;
        x1 += R.cB(1, q) * sCx[o];
        x2 += R.cD(1, q) * sCy[o] + R.cB(1, q) * sC[o];
      }
      sA[t] = x1;
      sAd[t] = x2;
    }
    __syncthreads();
    if (act)
    {
      T ye = 0;
#pragma unroll
      for (int q = 0; q < 5; ++q)
      {
        const int o = 25 * t3 + 5 * t2 + q;
        ye += R.cD(0, q) * sA[o] + R.cB(0, q) * sAd[o];
      }
      y[gid] = bnd ? ucur : yold + ye;
    }
  }
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
  const int64_t n = q4_ndofs(m);
  DFX_CUDA(cudaMemsetAsync(y, 0, sizeof(T) * n, s));
  for (int c = 0; c < 8; ++c)
  {
    const int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
    const int64_t hx = (m.nx - ci + 1) / 2, hy = (m.ny - cj + 1) / 2, hz = (m.nz - ck + 1) / 2;
    const int64_t cells = hx * hy * hz;
    if (cells == 0)
      continue;
    const int64_t grid = std::min<int64_t>(cells, q4_grid_limit<T>());
    k_q4_cells<T><<<(unsigned)grid, 128, 0, s>>>(m, u, y, ci, cj, ck, skip);
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

extern "C" int dfx_q4_action(const dfx_q4_mesh* mesh, int32_t dtype, const void* d_u, void* d_y,
                             void* stream)
{
  DFX_REQUIRE(mesh && d_u && d_y, "arguments must be non-NULL");
  const dfx_q4_mesh_s& m = *mesh;
  DFX_REQUIRE(m.nx > 0 && m.ny > 0 && m.nz > 0 && m.verts, "invalid Q4 mesh");
  DFX_REQUIRE(d_u != d_y, "u and y must differ");
  cudaStream_t s = dfx::as_stream(stream);
  if (dtype == DFX_F64)
    return dfx::q4_apply<double>(m, (const double*)d_u, (double*)d_y, s);
  if (dtype == DFX_F32)
    return dfx::q4_apply<float>(m, (const float*)d_u, (float*)d_y, s);
  return dfx::fail(DFX_ERR_INVALID, "unknown dtype %d", dtype);
}
