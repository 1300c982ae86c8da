// CPU oracle for the DOLFINx assembly + CG hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU path:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// load it. The product library (libdfxgpu.so) never links or calls it.
//
// It is a plain, sequential restatement of the reference algorithms,
// each function citing the reference file:line it follows (paths are
// relative to the DOLFINx source tree). Element kernels, which DOLFINx
// takes from FFCx-generated code that is not part of the reference tree,
// are restated from the finite-element mathematics: Lagrange P1/P2 on the
// Basix reference tetrahedron, integrated with a collapsed (Duffy) Gauss
// product rule that is exact for every integrand used here.
//
// Pinned against: the reference's own graph/ordering.cpp (RCM),
// common/sort.h (facet sort), la/matrix_csr_impl.h (insert_csr, spmv),
// compiled from the reference sources into oracle/_ref/ and frozen as
// golden vectors under tests/golden/.

#include <algorithm>
#include <chrono>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <unordered_map>
#include <vector>

namespace
{

enum
{
  ORC_OK = 0,
  ORC_ERR_INVALID = 1,
  ORC_ERR_NOT_IN_SPARSITY = 3,
  ORC_ERR_NOT_CONVERGED = 4,
};

// Basix reference tetrahedron sub-entities (vertex indices).
// Edges: basix cell topology of tetrahedron, dim 1; facets: dim 2.
const int kTetEdges[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
const int kTetFacets[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

//---------------------------------------------------------------------------
// Quadrature
//---------------------------------------------------------------------------

// Gauss-Legendre rule with m points on [0, 1] (Newton on P_m).
void gauss_legendre01(int m, std::vector<double>& x, std::vector<double>& w)
{
  x.resize(m);
  w.resize(m);
  for (int i = 0; i < m; ++i)
  {
    double z = std::cos(M_PI * (i + 0.75) / (m + 0.5));
    for (int it = 0; it < 100; ++it)
    {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= m; ++k)
      {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double dp = m * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::abs(dz) < 1e-16)
        break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= m; ++k)
    {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    double dp = m * (z * p1 - p0) / (z * z - 1.0);
    x[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Collapsed product rule on the reference tetrahedron
// {X,Y,Z >= 0, X+Y+Z <= 1}: X = u, Y = v(1-u), Z = w(1-u)(1-v).
// With m points per direction it integrates polynomials of total
// degree <= 2m-3 exactly.
struct TetQuad
{
  std::vector<double> X; // (nq, 3)
  std::vector<double> w;
};

TetQuad tet_quadrature(int m)
{
  std::vector<double> g, gw;
  gauss_legendre01(m, g, gw);
  TetQuad q;
  for (int a = 0; a < m; ++a)
    for (int b = 0; b < m; ++b)
      for (int c = 0; c < m; ++c)
      {
        double u = g[a], v = g[b], s = g[c];
        q.X.push_back(u);
        q.X.push_back(v * (1.0 - u));
        q.X.push_back(s * (1.0 - u) * (1.0 - v));
        q.w.push_back(gw[a] * gw[b] * gw[c] * (1.0 - u) * (1.0 - u) * (1.0 - v));
      }
  return q;
}

//---------------------------------------------------------------------------
// Lagrange basis on the reference tetrahedron (Basix dof ordering:
// vertices 0..3, then one dof per edge in kTetEdges order).
//---------------------------------------------------------------------------
void tabulate_tet(int degree, const double* X, double* phi, double (*dphi)[3])
{
  const double l[4] = {1.0 - X[0] - X[1] - X[2], X[0], X[1], X[2]};
  const double dl[4][3]
      = {{-1.0, -1.0, -1.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  if (degree == 1)
  {
    for (int i = 0; i < 4; ++i)
    {
      phi[i] = l[i];
      for (int k = 0; k < 3; ++k)
        dphi[i][k] = dl[i][k];
    }
    return;
  }
  for (int i = 0; i < 4; ++i)
  {
    phi[i] = l[i] * (2.0 * l[i] - 1.0);
    for (int k = 0; k < 3; ++k)
      dphi[i][k] = (4.0 * l[i] - 1.0) * dl[i][k];
  }
  for (int e = 0; e < 6; ++e)
  {
    const int a = kTetEdges[e][0], b = kTetEdges[e][1];
    phi[4 + e] = 4.0 * l[a] * l[b];
    for (int k = 0; k < 3; ++k)
      dphi[4 + e][k] = 4.0 * (l[a] * dl[b][k] + l[b] * dl[a][k]);
  }
}

int tet_ndofs(int degree) { return degree == 1 ? 4 : 10; }

// Affine P1 coordinate map: J_ij = dx_i/dX_j, K = J^{-1}.
double tet_geometry(const double* c, double J[3][3], double K[3][3])
{
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      J[i][j] = c[3 * (j + 1) + i] - c[i];
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1])
                     - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0])
                     + J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  K[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  K[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  K[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  K[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  K[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  K[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  K[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  K[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  K[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  return det;
}

const TetQuad& quad_for_tets()
{
  static const TetQuad q = tet_quadrature(4); // exact to degree 5
  return q;
}

// Symmetric 4-point rule, exact to degree 2 (barycentric (a,b,b,b) and
// permutations, a = (5+3 sqrt 5)/20, b = (5-sqrt 5)/20, weights 1/24):
// the rule a degree-2 integrand (stiffness, elasticity, P2 load) gets.
const TetQuad& quad_degree2()
{
  static const TetQuad q = []
  {
    TetQuad r;
    const double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, b = (5.0 - std::sqrt(5.0)) / 20.0;
    for (int p = 0; p < 4; ++p)
    {
      double l[4] = {b, b, b, b};
      l[p] = a;
      r.X.insert(r.X.end(), {l[1], l[2], l[3]});
      r.w.push_back(1.0 / 24.0);
    }
    return r;
  }();
  return q;
}

// Physical gradients g_i = K^T dphi_i.
void push_forward(int nd, const double K[3][3], const double (*dphi)[3],
                  double (*g)[3])
{
  for (int i = 0; i < nd; ++i)
    for (int k = 0; k < 3; ++k)
      g[i][k] = K[0][k] * dphi[i][0] + K[1][k] * dphi[i][1] + K[2][k] * dphi[i][2];
}

//---------------------------------------------------------------------------
// Element kernels (stand-ins for the FFCx tabulate_tensor ABI of
// cpp/dolfinx/fem/kernel.h:18-27: Ae row-major, coords 3 per node).
//---------------------------------------------------------------------------

// a(u, v) = \int kappa grad u . grad v + k2 u v dx on a P1/P2 tetrahedron.
void kernel_poisson(int degree, double* Ae, double kappa, double k2,
                    const double* coords)
{
  const int nd = tet_ndofs(degree);
  double J[3][3], K[3][3];
  const double adet = std::abs(tet_geometry(coords, J, K));
  // Stiffness alone has degree 2(p-1) <= 2; the mass term needs degree 2p.
  const TetQuad& q = k2 == 0.0 ? quad_degree2() : quad_for_tets();
  double phi[10], dphi[10][3], g[10][3];
  for (std::size_t p = 0; p < q.w.size(); ++p)
  {
    tabulate_tet(degree, &q.X[3 * p], phi, dphi);
    push_forward(nd, K, dphi, g);
    const double wq = q.w[p] * adet;
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j)
        Ae[i * nd + j] += wq
                          * (kappa * (g[i][0] * g[j][0] + g[i][1] * g[j][1]
                                      + g[i][2] * g[j][2])
                             + k2 * phi[i] * phi[j]);
  }
}

// L(v) = \int f v dx, f a P1 coefficient given by its 4 vertex values.
void kernel_source(int degree, double* be, const double* f,
                   const double* coords)
{
  const int nd = tet_ndofs(degree);
  double J[3][3], K[3][3];
  const double adet = std::abs(tet_geometry(coords, J, K));
  // integrand degree p + 1 <= 3: collapsed rule with 3 points per direction
  static const TetQuad q3 = tet_quadrature(3);
  const TetQuad& q = q3;
  double phi[10], dphi[10][3], l[4], dl[4][3];
  for (std::size_t p = 0; p < q.w.size(); ++p)
  {
    tabulate_tet(degree, &q.X[3 * p], phi, dphi);
    tabulate_tet(1, &q.X[3 * p], l, dl);
    const double fq = f[0] * l[0] + f[1] * l[1] + f[2] * l[2] + f[3] * l[3];
    for (int i = 0; i < nd; ++i)
      be[i] += q.w[p] * adet * fq * phi[i];
  }
}

// Linear elasticity, vector P2 (bs = 3, interleaved dofs 3*i + k):
// a(u, v) = \int 2 mu eps(u):eps(v) + lambda div u div v dx.
void kernel_elasticity(double* Ae, double E, double nu, const double* coords)
{
  const double mu = E / (2.0 * (1.0 + nu));
  const double lmbda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  double J[3][3], K[3][3];
  const double adet = std::abs(tet_geometry(coords, J, K));
  const TetQuad& q = quad_degree2();
  double phi[10], dphi[10][3], g[10][3];
  const int n = 30;
  for (std::size_t p = 0; p < q.w.size(); ++p)
  {
    tabulate_tet(2, &q.X[3 * p], phi, dphi);
    push_forward(10, K, dphi, g);
    const double wq = q.w[p] * adet;
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j)
      {
        const double gg = g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2];
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l)
            Ae[(3 * i + k) * n + 3 * j + l]
                += wq * (mu * ((k == l ? gg : 0.0) + g[i][l] * g[j][k])
                         + lmbda * g[i][k] * g[j][l]);
      }
  }
}

// L(v) = \int f . v dx with a constant vector f, vector P2.
void kernel_bodyforce(double* be, const double* f, const double* coords)
{
  double J[3][3], K[3][3];
  const double adet = std::abs(tet_geometry(coords, J, K));
  const TetQuad& q = quad_degree2();
  double phi[10], dphi[10][3];
  for (std::size_t p = 0; p < q.w.size(); ++p)
  {
    tabulate_tet(2, &q.X[3 * p], phi, dphi);
    for (int i = 0; i < 10; ++i)
      for (int k = 0; k < 3; ++k)
        be[3 * i + k] += q.w[p] * adet * f[k] * phi[i];
  }
}

//---------------------------------------------------------------------------
// Mesh ordering helpers
//---------------------------------------------------------------------------

// Level structure rooted at s (cpp/dolfinx/graph/ordering.cpp:23-60).
void level_structure(const int32_t* off, const int32_t* adj, int n, int s,
                     std::vector<int>& ls, std::vector<int>& loff)
{
  std::vector<char> seen(n, 0);
  seen[s] = 1;
  ls.assign(1, s);
  loff.assign(1, 0);
  int l = 0;
  while ((int)ls.size() > loff.back())
  {
    loff.push_back(ls.size());
    for (int i = loff[l]; i < loff[l + 1]; ++i)
    {
      const int node = ls[i];
      for (int k = off[node]; k < off[node + 1]; ++k)
      {
        const int w = adj[k];
        if (!seen[w])
        {
          ls.push_back(w);
          seen[w] = 1;
        }
      }
    }
    ++l;
  }
}

} // namespace

extern "C"
{

//---------------------------------------------------------------------------
// Mesh: box of tetrahedra (cpp/dolfinx/mesh/generation.h:332-426)
//---------------------------------------------------------------------------

// Original (unordered) cells and vertex coordinates of the Kuhn split:
// create_geom (generation.h:332-377) and build_tet (generation.h:380-426).
int orc_box_tet_raw(int nx, int ny, int nz, const double* p0, const double* p1,
                    int64_t* cells, double* x)
{
  if (nx < 1 || ny < 1 || nz < 1)
    return ORC_ERR_INVALID;
  const double ext[3] = {(p1[0] - p0[0]) / nx, (p1[1] - p0[1]) / ny,
                         (p1[2] - p0[2]) / nz};
  const int64_t sqxy = (int64_t)(nx + 1) * (ny + 1);
  const int64_t npts = sqxy * (nz + 1);
  for (int64_t v = 0; v < npts; ++v)
  {
    const int64_t p = v % sqxy;
    const int64_t idx[3] = {p % (nx + 1), p / (nx + 1), v / sqxy};
    for (int i = 0; i < 3; ++i)
      x[3 * v + i] = p0[i] + (double)idx[i] * ext[i];
  }
  const int64_t nhex = (int64_t)nx * ny * nz;
  for (int64_t i = 0; i < nhex; ++i)
  {
    const int64_t iz = i / ((int64_t)nx * ny);
    const int64_t j = i % ((int64_t)nx * ny);
    const int64_t iy = j / nx, ix = j % nx;
    const int64_t v0 = iz * sqxy + iy * (nx + 1) + ix;
    const int64_t v1 = v0 + 1, v2 = v0 + (nx + 1), v3 = v1 + (nx + 1);
    const int64_t v4 = v0 + sqxy, v5 = v1 + sqxy, v6 = v2 + sqxy, v7 = v3 + sqxy;
    const int64_t t[24] = {v0, v1, v3, v7, v0, v1, v7, v5, v0, v5, v7, v4,
                           v0, v3, v2, v7, v0, v6, v4, v7, v0, v2, v6, v7};
    std::memcpy(cells + 24 * i, t, sizeof(t));
  }
  return ORC_OK;
}

// Facet-connected dual graph of a tetrahedral mesh, serial path of
// build_local_dual_graph (cpp/dolfinx/mesh/graphbuild.cpp:566-905):
// facets as sorted vertex triples, a stable lexicographic sort, one
// edge per matched pair, both directions filled in edge order.
// offsets has nc+1 entries; adj must hold 4*nc entries.
int orc_dual_graph_tet(int nc, const int64_t* cells, int32_t* offsets,
                       int32_t* adj)
{
  const int64_t nf = 4 * (int64_t)nc;
  std::vector<int64_t> key(3 * nf);
  for (int c = 0; c < nc; ++c)
    for (int f = 0; f < 4; ++f)
    {
      int64_t v[3];
      for (int k = 0; k < 3; ++k)
        v[k] = cells[4 * (int64_t)c + kTetFacets[f][k]];
      std::sort(v, v + 3);
      for (int k = 0; k < 3; ++k)
        key[3 * (4 * (int64_t)c + f) + k] = v[k];
    }
  std::vector<int32_t> perm(nf);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(),
                   [&](int32_t a, int32_t b)
                   {
                     for (int k = 0; k < 3; ++k)
                       if (key[3 * a + k] != key[3 * b + k])
                         return key[3 * a + k] < key[3 * b + k];
                     return false;
                   });
  std::vector<std::pair<int32_t, int32_t>> edges;
  for (int64_t i = 0; i < nf;)
  {
    int64_t j = i + 1;
    while (j < nf && key[3 * perm[j]] == key[3 * perm[i]]
           && key[3 * perm[j] + 1] == key[3 * perm[i] + 1]
           && key[3 * perm[j] + 2] == key[3 * perm[i] + 2])
      ++j;
    for (int64_t a = i; a < j; ++a)
      for (int64_t b = a + 1; b < j; ++b)
        edges.push_back({perm[a] / 4, perm[b] / 4});
    i = j;
  }
  std::vector<int32_t> cnt(nc, 0);
  for (auto& e : edges)
  {
    ++cnt[e.first];
    ++cnt[e.second];
  }
  offsets[0] = 0;
  for (int c = 0; c < nc; ++c)
    offsets[c + 1] = offsets[c] + cnt[c];
  std::vector<int32_t> pos(offsets, offsets + nc);
  for (auto& e : edges)
  {
    adj[pos[e.first]++] = e.second;
    adj[pos[e.second]++] = e.first;
  }
  return ORC_OK;
}

// Reverse Cuthill-McKee (cpp/dolfinx/graph/ordering.cpp:66-170).
// r[old] = new position.
int orc_reorder_rcm(int n, const int32_t* off, const int32_t* adj, int32_t* r)
{
  std::fill(r, r + n, -1);
  auto deg = [&](int a) { return off[a + 1] - off[a]; };
  auto cmp = [&](int a, int b) { return deg(a) < deg(b); };
  int count = 0;
  std::vector<int> ls, loff, ls2, loff2;
  while (count < n)
  {
    int v = 0, dmin = INT32_MAX;
    for (int i = 0; i < n; ++i)
      if (r[i] == -1 && deg(i) < dmin)
      {
        v = i;
        dmin = deg(i);
      }
    level_structure(off, adj, n, v, ls, loff);
    for (;;)
    {
      const int nl = (int)loff.size() - 1;
      auto b = ls.begin() + loff[nl - 1], e = ls.begin() + loff[nl];
      const int s = *std::ranges::min_element(std::ranges::subrange(b, e), cmp);
      level_structure(off, adj, n, s, ls2, loff2);
      if (loff2.size() > loff.size())
      {
        v = s;
        ls.swap(ls2);
        loff.swap(loff2);
      }
      else
        break;
    }
    std::vector<char> lab(n, 0);
    std::vector<int> rv{v};
    lab[v] = 1;
    std::vector<int> nbr;
    for (std::size_t cur = 0; cur < rv.size(); ++cur)
    {
      nbr.clear();
      for (int k = off[rv[cur]]; k < off[rv[cur] + 1]; ++k)
        if (!lab[adj[k]])
        {
          nbr.push_back(adj[k]);
          lab[adj[k]] = 1;
        }
      std::ranges::sort(nbr, cmp);
      rv.insert(rv.end(), nbr.begin(), nbr.end());
    }
    std::reverse(rv.begin(), rv.end());
    for (int q : rv)
      r[q] = count++;
  }
  return ORC_OK;
}

// Full mesh pipeline for create_box(tetrahedron) on one rank:
// build_tet -> dual graph -> reorder_rcm -> cells permuted
// (cpp/dolfinx/mesh/utils.h:280-308; reorder_list utils.h:57-71) ->
// geometry nodes numbered by first appearance in the cell loop
// (cpp/dolfinx/fem/dofmapbuilder.cpp:440-474 with no graph reordering,
// create_geometry mesh/Geometry.h:235-311).
// Outputs: cells (nc, 4) geometry node indices, x (nv, 3).
int orc_create_box_tet(int nx, int ny, int nz, const double* p0,
                       const double* p1, int reorder, int32_t* cells_out,
                       double* x_out)
{
  const int64_t nc = 6 * (int64_t)nx * ny * nz;
  const int64_t nv = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
  std::vector<int64_t> cells(4 * nc);
  std::vector<double> x(3 * nv);
  int st = orc_box_tet_raw(nx, ny, nz, p0, p1, cells.data(), x.data());
  if (st)
    return st;
  std::vector<int64_t> cells_new(cells);
  if (reorder)
  {
    std::vector<int32_t> off(nc + 1), adj(4 * nc), r(nc);
    orc_dual_graph_tet((int)nc, cells.data(), off.data(), adj.data());
    orc_reorder_rcm((int)nc, off.data(), adj.data(), r.data());
    for (int64_t c = 0; c < nc; ++c)
      for (int k = 0; k < 4; ++k)
        cells_new[4 * (int64_t)r[c] + k] = cells[4 * c + k];
  }
  std::vector<int32_t> node(nv, -1);
  int32_t cnt = 0;
  for (int64_t i = 0; i < 4 * nc; ++i)
  {
    int64_t v = cells_new[i];
    if (node[v] < 0)
      node[v] = cnt++;
    cells_out[i] = node[v];
  }
  for (int64_t v = 0; v < nv; ++v)
    for (int k = 0; k < 3; ++k)
      x_out[3 * (int64_t)node[v] + k] = x[3 * v + k];
  return ORC_OK;
}

//---------------------------------------------------------------------------
// Dofmap: Lagrange P1/P2 on tetrahedra. Basic dofmap from the element
// dof layout (cpp/dolfinx/fem/dofmapbuilder.cpp:153-397), then owned
// dofs numbered by first appearance while iterating the cell dofmap
// (dofmapbuilder.cpp:440-474). create_functionspace passes no reorder
// function (cpp/dolfinx/fem/utils.h:925-950), so this is the final
// numbering. Returns the number of dof nodes (blocks).
//---------------------------------------------------------------------------
int orc_dofmap_tet(int nc, const int32_t* cells, int degree, int32_t* dofmap)
{
  if (degree == 1)
  {
    std::unordered_map<int32_t, int32_t> id;
    int32_t cnt = 0;
    for (int64_t i = 0; i < 4 * (int64_t)nc; ++i)
    {
      auto [it, ins] = id.try_emplace(cells[i], cnt);
      if (ins)
        ++cnt;
      dofmap[i] = it->second;
    }
    return cnt;
  }
  if (degree != 2)
    return -1;
  std::unordered_map<int64_t, int32_t> id;
  int32_t cnt = 0;
  for (int64_t c = 0; c < nc; ++c)
  {
    const int32_t* v = cells + 4 * c;
    for (int i = 0; i < 10; ++i)
    {
      int64_t k;
      if (i < 4)
        k = v[i];
      else
      {
        int64_t a = v[kTetEdges[i - 4][0]], b = v[kTetEdges[i - 4][1]];
        if (a > b)
          std::swap(a, b);
        k = ((a + 1) << 32) | b; // distinct from vertex keys
      }
      auto [it, ins] = id.try_emplace(k, cnt);
      if (ins)
        ++cnt;
      dofmap[10 * c + i] = it->second;
    }
  }
  return cnt;
}

//---------------------------------------------------------------------------
// Sparsity pattern: cell outer products (cpp/dolfinx/fem/sparsitybuild.cpp
// :16-54), rows deduplicated and sorted (cpp/dolfinx/la/SparsityPattern.cpp
// :264-491); one rank, so all columns are owned and in ascending order.
// Call with cols == nullptr to get nnz; then again to fill.
//---------------------------------------------------------------------------
int64_t orc_sparsity(int nrows, int nc, int nd, const int32_t* dofmap,
                     int64_t* row_ptr, int32_t* cols)
{
  std::vector<std::vector<int32_t>> rows(nrows);
  for (int64_t c = 0; c < nc; ++c)
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j)
        rows[dofmap[nd * c + i]].push_back(dofmap[nd * c + j]);
  int64_t nnz = 0;
  if (row_ptr)
    row_ptr[0] = 0;
  for (int r = 0; r < nrows; ++r)
  {
    auto& v = rows[r];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    if (cols)
      std::copy(v.begin(), v.end(), cols + nnz);
    nnz += v.size();
    if (row_ptr)
      row_ptr[r + 1] = nnz;
  }
  return nnz;
}

//---------------------------------------------------------------------------
// Element kernels, exposed for tests.
//---------------------------------------------------------------------------
void orc_kernel_poisson(int degree, double* Ae, double kappa, double k2,
                        const double* coords)
{
  kernel_poisson(degree, Ae, kappa, k2, coords);
}
void orc_kernel_source(int degree, double* be, const double* f,
                       const double* coords)
{
  kernel_source(degree, be, f, coords);
}
void orc_kernel_elasticity(double* Ae, double E, double nu, const double* coords)
{
  kernel_elasticity(Ae, E, nu, coords);
}

//---------------------------------------------------------------------------
// Forms used on the hot path. kind: 0 = Poisson/Helmholtz (scalar P1/P2),
// 1 = linear elasticity (vector P2, bs 3).
//---------------------------------------------------------------------------
struct orc_form
{
  int kind;
  int degree;
  const double* kappa; // per-cell coefficient (kappa or E); null -> 1
  double k2;           // mass coefficient (Helmholtz), scalar forms
  double nu;           // Poisson ratio, elasticity
};

// One cell of the matrix cell loop (cpp/dolfinx/fem/assemble_matrix_impl.h:
// 92-200): coordinates, element tensor, BC rows/columns zeroed, insertion
// by binary search (cpp/dolfinx/la/matrix_csr_impl.h:67-109). Ae holds
// (nd bs)^2 scratch values.
static int matrix_cell(const orc_form* form, int c, const int32_t* x_dofmap, const double* x,
                const int32_t* dofmap, const int8_t* bc, const int64_t* row_ptr,
                const int32_t* cols, double* vals, double* Ae)
{
  const int nd = tet_ndofs(form->degree);
  const int bs = form->kind == 1 ? 3 : 1;
  const int n = nd * bs;
  double coords[12];
  for (int v = 0; v < 4; ++v)
    for (int k = 0; k < 3; ++k)
      coords[3 * v + k] = x[3 * (int64_t)x_dofmap[4 * (int64_t)c + v] + k];
  std::fill_n(Ae, n * n, 0.0);
  const double kap = form->kappa ? form->kappa[c] : 1.0;
  if (form->kind == 0)
    kernel_poisson(form->degree, Ae, kap, form->k2, coords);
  else
    kernel_elasticity(Ae, kap, form->nu, coords);
  const int32_t* dofs = dofmap + (int64_t)nd * c;
  if (bc)
  {
    for (int i = 0; i < nd; ++i)
      for (int k = 0; k < bs; ++k)
        if (bc[bs * dofs[i] + k])
        {
          std::fill_n(Ae + n * (bs * i + k), n, 0.0);
          for (int r = 0; r < n; ++r)
            Ae[r * n + bs * i + k] = 0.0;
        }
  }
  for (int i = 0; i < nd; ++i)
  {
    const int32_t row = dofs[i];
    const int32_t* c0 = cols + row_ptr[row];
    const int32_t* c1 = cols + row_ptr[row + 1];
    for (int j = 0; j < nd; ++j)
    {
      const int32_t* it = std::lower_bound(c0, c1, dofs[j]);
      if (it == c1 || *it != dofs[j])
        return ORC_ERR_NOT_IN_SPARSITY;
      const int64_t d = (it - cols) * bs * bs;
      for (int a = 0; a < bs; ++a)
        for (int b = 0; b < bs; ++b)
          vals[d + a * bs + b] += Ae[(bs * i + a) * n + bs * j + b];
    }
  }
  return ORC_OK;
}

// Matrix cell loop (cpp/dolfinx/fem/assemble_matrix_impl.h:92-200) with
// insertion by binary search (cpp/dolfinx/la/matrix_csr_impl.h:67-109).
// dofmap holds node (block) indices; bc is indexed by bs*node + k.
int orc_assemble_matrix(const orc_form* form, int nc, const int32_t* x_dofmap,
                        const double* x, const int32_t* dofmap,
                        const int8_t* bc, const int64_t* row_ptr,
                        const int32_t* cols, double* vals)
{
  const int n = tet_ndofs(form->degree) * (form->kind == 1 ? 3 : 1);
  std::vector<double> Ae(n * n);
  for (int c = 0; c < nc; ++c)
    if (int st = matrix_cell(form, c, x_dofmap, x, dofmap, bc, row_ptr, cols, vals, Ae.data()))
      return st;
  return ORC_OK;
}

// Vector cell loop (cpp/dolfinx/fem/assemble_vector_impl.h:75-116).
// kind 0: L = \int f v, f a P1 coefficient (values per geometry node,
// f == nullptr -> f = 1). kind 1: L = \int fvec . v (vector P2).
int orc_assemble_vector(int kind, int degree, int nc, const int32_t* x_dofmap,
                        const double* x, const int32_t* dofmap, const double* f,
                        const double* fvec, double* b)
{
  const int nd = tet_ndofs(degree);
  const int bs = kind == 1 ? 3 : 1;
  double be[30], coords[12], fc[4];
  for (int c = 0; c < nc; ++c)
  {
    for (int v = 0; v < 4; ++v)
    {
      for (int k = 0; k < 3; ++k)
        coords[3 * v + k] = x[3 * (int64_t)x_dofmap[4 * c + v] + k];
      fc[v] = f ? f[x_dofmap[4 * c + v]] : 1.0;
    }
    std::fill_n(be, 30, 0.0);
    if (kind == 0)
      kernel_source(degree, be, fc, coords);
    else
      kernel_bodyforce(be, fvec, coords);
    const int32_t* dofs = dofmap + (int64_t)nd * c;
    for (int i = 0; i < nd; ++i)
      for (int k = 0; k < bs; ++k)
        b[bs * dofs[i] + k] += be[bs * i + k];
  }
  return ORC_OK;
}

// apply_lifting for one form (cpp/dolfinx/fem/assembler.h:341-421,
// lift_bc cpp/dolfinx/fem/assemble_vector_impl.h:361-414): cells with a
// constrained column only, b[r] -= Ae[r, c] * alpha * (g_c - x0_c).
int orc_apply_lifting(const orc_form* form, int nc, const int32_t* x_dofmap,
                      const double* x, const int32_t* dofmap,
                      const int8_t* bc, const double* g, const double* x0,
                      double alpha, double* b)
{
  const int nd = tet_ndofs(form->degree);
  const int bs = form->kind == 1 ? 3 : 1;
  const int n = nd * bs;
  std::vector<double> Ae(n * n);
  double coords[12];
  for (int c = 0; c < nc; ++c)
  {
    const int32_t* dofs = dofmap + (int64_t)nd * c;
    bool has = false;
    for (int i = 0; i < nd && !has; ++i)
      for (int k = 0; k < bs; ++k)
        has = has || bc[bs * dofs[i] + k];
    if (!has)
      continue;
    for (int v = 0; v < 4; ++v)
      for (int k = 0; k < 3; ++k)
        coords[3 * v + k] = x[3 * (int64_t)x_dofmap[4 * c + v] + k];
    std::fill(Ae.begin(), Ae.end(), 0.0);
    const double kap = form->kappa ? form->kappa[c] : 1.0;
    if (form->kind == 0)
      kernel_poisson(form->degree, Ae.data(), kap, form->k2, coords);
    else
      kernel_elasticity(Ae.data(), kap, form->nu, coords);
    for (int j = 0; j < nd; ++j)
      for (int k = 0; k < bs; ++k)
      {
        const int32_t jj = bs * dofs[j] + k;
        if (!bc[jj])
          continue;
        const double xb = g[jj], xz = x0 ? x0[jj] : 0.0;
        for (int i = 0; i < nd; ++i)
          for (int m = 0; m < bs; ++m)
            b[bs * dofs[i] + m] -= Ae[(bs * i + m) * n + bs * j + k] * alpha * (xb - xz);
      }
  }
  return ORC_OK;
}

// DirichletBC::set (cpp/dolfinx/fem/DirichletBC.h:495-578):
// x[dofs[i]] = alpha * (g[dofs[i]] - x0[dofs[i]]), skipping dofs >= n.
void orc_set_bc(int n, double* xv, int ndofs, const int32_t* dofs,
                const double* g, const double* x0, double alpha)
{
  for (int i = 0; i < ndofs; ++i)
    if (dofs[i] < n)
      xv[dofs[i]] = alpha == 0.0 ? 0.0 : alpha * (g[dofs[i]] - (x0 ? x0[dofs[i]] : 0.0));
}

// set_diagonal (cpp/dolfinx/fem/assembler.h:644-686) via MatrixCSR::set:
// A[d, d] = diag for each constrained scalar dof d (block row d / bs).
int orc_set_diagonal(int bs, const int64_t* row_ptr, const int32_t* cols,
                     double* vals, int ndofs, const int32_t* dofs, double diag)
{
  for (int i = 0; i < ndofs; ++i)
  {
    const int32_t r = dofs[i] / bs, k = dofs[i] % bs;
    const int32_t* c0 = cols + row_ptr[r];
    const int32_t* c1 = cols + row_ptr[r + 1];
    const int32_t* it = std::lower_bound(c0, c1, r);
    if (it == c1 || *it != r)
      return ORC_ERR_NOT_IN_SPARSITY;
    vals[(it - cols) * bs * bs + k * bs + k] = diag;
  }
  return ORC_OK;
}

// y += A x (cpp/dolfinx/la/matrix_csr_impl.h:259-286).
void orc_spmv(int nrows, int bs, const int64_t* row_ptr, const int32_t* cols,
              const double* vals, const double* xv, double* y)
{
  for (int k0 = 0; k0 < bs; ++k0)
    for (int i = 0; i < nrows; ++i)
    {
      double vi = 0.0;
      for (int64_t j = row_ptr[i]; j < row_ptr[i + 1]; ++j)
        for (int k1 = 0; k1 < bs; ++k1)
          vi += vals[j * bs * bs + k0 * bs + k1] * xv[cols[j] * bs + k1];
      y[i * bs + k0] += vi;
    }
}

// Same product, with float matrix values (MatrixCSR<float> obtained via
// the converting constructor cpp/dolfinx/la/MatrixCSR.h:223-237).
void orc_spmv_f32(int nrows, int bs, const int64_t* row_ptr,
                  const int32_t* cols, const float* vals, const float* xv,
                  float* y)
{
  for (int k0 = 0; k0 < bs; ++k0)
    for (int i = 0; i < nrows; ++i)
    {
      float vi = 0.0f;
      for (int64_t j = row_ptr[i]; j < row_ptr[i + 1]; ++j)
        for (int k1 = 0; k1 < bs; ++k1)
          vi += vals[j * bs * bs + k0 * bs + k1] * xv[cols[j] * bs + k1];
      y[i * bs + k0] += vi;
    }
}

// Conjugate gradients (cpp/demo/poisson_matrix_free/main.cpp:84-132),
// with optional Jacobi preconditioning (dinv != nullptr): z = D^{-1} r,
// rho = r.z drives alpha/beta; convergence is tested on the unpreconditioned
// residual, |r|^2 / |r0|^2 < rtol^2, as in the demo. x holds the initial
// guess. Returns iterations (negative on non-convergence).
int orc_cg(int nrows, int bs, const int64_t* row_ptr, const int32_t* cols,
           const double* vals, const double* b, double* xv, const double* dinv,
           double rtol, int kmax)
{
  const int64_t n = (int64_t)nrows * bs;
  std::vector<double> r(n), y(n, 0.0), p(n), z(n);
  orc_spmv(nrows, bs, row_ptr, cols, vals, xv, y.data());
  for (int64_t i = 0; i < n; ++i)
    r[i] = b[i] - y[i];
  for (int64_t i = 0; i < n; ++i)
    z[i] = dinv ? dinv[i] * r[i] : r[i];
  p = z;
  double rr0 = 0, rz = 0;
  for (int64_t i = 0; i < n; ++i)
  {
    rr0 += r[i] * r[i];
    rz += r[i] * z[i];
  }
  if (rr0 == 0.0)
    return 0;
  const double rtol2 = rtol * rtol;
  int k = 0;
  while (k < kmax)
  {
    ++k;
    std::fill(y.begin(), y.end(), 0.0);
    orc_spmv(nrows, bs, row_ptr, cols, vals, p.data(), y.data());
    double py = 0;
    for (int64_t i = 0; i < n; ++i)
      py += p[i] * y[i];
    const double alpha = rz / py;
    double rr = 0, rzn = 0;
    for (int64_t i = 0; i < n; ++i)
    {
      xv[i] += alpha * p[i];
      r[i] -= alpha * y[i];
      rr += r[i] * r[i];
      z[i] = dinv ? dinv[i] * r[i] : r[i];
      rzn += r[i] * z[i];
    }
    if (rr / rr0 < rtol2)
      return k;
    const double beta = rzn / rz;
    rz = rzn;
    for (int64_t i = 0; i < n; ++i)
      p[i] = z[i] + beta * p[i];
  }
  return -k;
}

} // extern "C"

//---------------------------------------------------------------------------
// Q4 hexahedral Laplacian action (matrix-free demo action,
// cpp/demo/poisson_matrix_free/main.cpp:201-222, on the Q4 configuration).
// Structured n_x x n_y x n_z mesh of the box with vertices `verts`
// ((nx+1)(ny+1)(nz+1) x 3, lexicographic, x fastest), trilinear geometry,
// Lagrange Q4 on Gauss-Lobatto-Legendre points (Basix's GLL variant, which
// on tensor-product cells is the GLL lattice), Gauss-Legendre 5^3
// quadrature. Global nodes: lexicographic on the (4n+1)^3 lattice.
// y = A u on interior nodes with boundary entries of u taken as 0, y = u on
// boundary nodes (homogeneous Dirichlet rows set to the identity). Plain
// quadrature loops with the full 125 x 125 element matrix (no sum
// factorisation): an independent check of the GPU kernels.
//---------------------------------------------------------------------------
namespace
{
void q4_tables(double B[5][5], double D[5][5], double* wq)
{
  const double s = std::sqrt(3.0 / 7.0);
  const double xn[5] = {0.0, 0.5 * (1.0 - s), 0.5, 0.5 * (1.0 + s), 1.0};
  std::vector<double> g, w;
  gauss_legendre01(5, g, w);
  for (int q = 0; q < 5; ++q)
  {
    wq[q] = w[q];
    for (int a = 0; a < 5; ++a)
    {
      double l = 1.0, dl = 0.0;
      for (int m = 0; m < 5; ++m)
      {
        if (m == a)
          continue;
        l *= (g[q] - xn[m]) / (xn[a] - xn[m]);
      }
      for (int k = 0; k < 5; ++k)
      {
        if (k == a)
          continue;
        double t = 1.0 / (xn[a] - xn[k]);
        for (int m = 0; m < 5; ++m)
          if (m != a && m != k)
            t *= (g[q] - xn[m]) / (xn[a] - xn[m]);
        dl += t;
      }
      B[q][a] = l;
      D[q][a] = dl;
    }
  }
}
} // namespace

extern "C" void orc_q4_tables(double* B, double* D, double* w)
{
  double b[5][5], d[5][5];
  q4_tables(b, d, w);
  std::memcpy(B, b, sizeof(b));
  std::memcpy(D, d, sizeof(d));
}

extern "C" int orc_q4_action(int nx, int ny, int nz, const double* verts, double kappa,
                             const double* u, double* y, int apply_bc)
{
  double B[5][5], D[5][5], w[5];
  q4_tables(B, D, w);
  std::vector<double> g, gw;
  gauss_legendre01(5, g, gw);
  const int64_t NX = 4 * (int64_t)nx + 1, NY = 4 * (int64_t)ny + 1, NZ = 4 * (int64_t)nz + 1;
  const int64_t ndofs = NX * NY * NZ;
  auto on_bnd = [&](int64_t I, int64_t J, int64_t K)
  {
    return apply_bc
           && (I == 0 || J == 0 || K == 0 || I == NX - 1 || J == NY - 1 || K == NZ - 1);
  };
  std::fill(y, y + ndofs, 0.0);
  std::vector<double> grad(125 * 125 * 3);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
      {
        double xv[8][3];
        for (int v = 0; v < 8; ++v)
        {
          const int64_t vi = i + (v & 1), vj = j + ((v >> 1) & 1), vk = k + ((v >> 2) & 1);
          const int64_t id = (vk * (ny + 1) + vj) * (nx + 1) + vi;
          for (int c = 0; c < 3; ++c)
            xv[v][c] = verts[3 * id + c];
        }
        int64_t dof[125];
        double ue[125];
        for (int c = 0; c < 5; ++c)
          for (int b = 0; b < 5; ++b)
            for (int a = 0; a < 5; ++a)
            {
              const int64_t I = 4 * i + a, J = 4 * j + b, K = 4 * k + c;
              const int e = a + 5 * b + 25 * c;
              dof[e] = (K * NY + J) * NX + I;
              ue[e] = on_bnd(I, J, K) ? 0.0 : u[dof[e]];
            }
        double ye[125] = {0.0};
        for (int q3 = 0; q3 < 5; ++q3)
          for (int q2 = 0; q2 < 5; ++q2)
            for (int q1 = 0; q1 < 5; ++q1)
            {
              const double px = g[q1], py = g[q2], pz = g[q3];
              double J[3][3];
              for (int c = 0; c < 3; ++c)
              {
                double dX = 0, dY = 0, dZ = 0;
                for (int v = 0; v < 8; ++v)
                {
                  const int bx = v & 1, by = (v >> 1) & 1, bz = (v >> 2) & 1;
                  const double Nx = bx ? px : 1 - px, Ny = by ? py : 1 - py, Nz = bz ? pz : 1 - pz;
                  const double sx = bx ? 1.0 : -1.0, sy = by ? 1.0 : -1.0, sz = bz ? 1.0 : -1.0;
                  dX += xv[v][c] * sx * Ny * Nz;
                  dY += xv[v][c] * Nx * sy * Nz;
                  dZ += xv[v][c] * Nx * Ny * sz;
                }
                J[c][0] = dX;
                J[c][1] = dY;
                J[c][2] = dZ;
              }
              double Jt[3][3], K[3][3];
              for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                  Jt[a][b] = J[a][b];
              const double det = Jt[0][0] * (Jt[1][1] * Jt[2][2] - Jt[1][2] * Jt[2][1])
                                 - Jt[0][1] * (Jt[1][0] * Jt[2][2] - Jt[1][2] * Jt[2][0])
                                 + Jt[0][2] * (Jt[1][0] * Jt[2][1] - Jt[1][1] * Jt[2][0]);
              K[0][0] = (Jt[1][1] * Jt[2][2] - Jt[1][2] * Jt[2][1]) / det;
              K[0][1] = (Jt[0][2] * Jt[2][1] - Jt[0][1] * Jt[2][2]) / det;
              K[0][2] = (Jt[0][1] * Jt[1][2] - Jt[0][2] * Jt[1][1]) / det;
              K[1][0] = (Jt[1][2] * Jt[2][0] - Jt[1][0] * Jt[2][2]) / det;
              K[1][1] = (Jt[0][0] * Jt[2][2] - Jt[0][2] * Jt[2][0]) / det;
              K[1][2] = (Jt[0][2] * Jt[1][0] - Jt[0][0] * Jt[1][2]) / det;
              K[2][0] = (Jt[1][0] * Jt[2][1] - Jt[1][1] * Jt[2][0]) / det;
              K[2][1] = (Jt[0][1] * Jt[2][0] - Jt[0][0] * Jt[2][1]) / det;
              K[2][2] = (Jt[0][0] * Jt[1][1] - Jt[0][1] * Jt[1][0]) / det;
              const double wq = w[q1] * w[q2] * w[q3] * std::abs(det) * kappa;
              // physical gradients of all 125 basis functions at this point
              double gr[125][3];
              for (int c = 0; c < 5; ++c)
                for (int b = 0; b < 5; ++b)
                  for (int a = 0; a < 5; ++a)
                  {
                    const double dref[3] = {D[q1][a] * B[q2][b] * B[q3][c],
                                            B[q1][a] * D[q2][b] * B[q3][c],
                                            B[q1][a] * B[q2][b] * D[q3][c]};
                    const int e = a + 5 * b + 25 * c;
                    for (int m = 0; m < 3; ++m)
                      gr[e][m] = K[0][m] * dref[0] + K[1][m] * dref[1] + K[2][m] * dref[2];
                  }
              double gu[3] = {0, 0, 0};
              for (int e = 0; e < 125; ++e)
                for (int m = 0; m < 3; ++m)
                  gu[m] += gr[e][m] * ue[e];
              for (int e = 0; e < 125; ++e)
                ye[e] += wq * (gr[e][0] * gu[0] + gr[e][1] * gu[1] + gr[e][2] * gu[2]);
            }
        for (int e = 0; e < 125; ++e)
          y[dof[e]] += ye[e];
      }
  for (int64_t K = 0; K < NZ; ++K)
    for (int64_t J = 0; J < NY; ++J)
      for (int64_t I = 0; I < NX; ++I)
        if (on_bnd(I, J, K))
        {
          const int64_t d = (K * NY + J) * NX + I;
          y[d] = u[d];
        }
  return 0;
}

//---------------------------------------------------------------------------
// Exterior facet integrals and functionals
//---------------------------------------------------------------------------
namespace
{
// Quadrature on facet f of the reference tetrahedron: points in tet
// reference coordinates and weights summing to 1/2 (the reference
// triangle's area), from a collapsed Gauss rule with 4 points per
// direction (exact to degree 6 on the triangle).
struct FacetQuad
{
  std::vector<double> X; // 3 per point
  std::vector<double> w;
};

const FacetQuad& facet_quadrature(int f)
{
  static const std::vector<FacetQuad> rules = []
  {
    std::vector<double> x, w;
    gauss_legendre01(4, x, w);
    const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    std::vector<FacetQuad> out(4);
    for (int fi = 0; fi < 4; ++fi)
    {
      const double* a = V[kTetFacets[fi][0]];
      const double* b = V[kTetFacets[fi][1]];
      const double* c = V[kTetFacets[fi][2]];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
        {
          const double s = x[i], t = x[j] * (1.0 - x[i]);
          for (int k = 0; k < 3; ++k)
            out[fi].X.push_back(a[k] + s * (b[k] - a[k]) + t * (c[k] - a[k]));
          out[fi].w.push_back(w[i] * w[j] * (1.0 - x[i]));
        }
    }
    return out;
  }();
  return rules[f];
}

// Physical area of facet f of a cell with vertex coordinates c (3 per
// vertex).
double facet_area(const double* c, int f)
{
  const double* a = c + 3 * kTetFacets[f][0];
  const double* b = c + 3 * kTetFacets[f][1];
  const double* d = c + 3 * kTetFacets[f][2];
  const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double v[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
  const double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                       u[0] * v[1] - u[1] * v[0]};
  return 0.5 * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
}

void cell_coords(const int32_t* x_dofmap, const double* x, int c, double* coords)
{
  for (int v = 0; v < 4; ++v)
    for (int k = 0; k < 3; ++k)
      coords[3 * v + k] = x[3 * (int64_t)x_dofmap[4 * c + v] + k];
}
} // namespace

extern "C"
{
// Exterior facets of a tetrahedral mesh as (cell, local facet) pairs, the
// integration domain of an exterior-facet integral on one rank:
// mesh::exterior_facet_indices (cpp/dolfinx/mesh/utils.cpp:61-89: facets
// with one attached cell) and compute_integration_domains
// (cpp/dolfinx/fem/utils.h:155-162: each facet as (cell, local index)).
// Pairs are written sorted by (cell, local facet). Returns the count.
int orc_exterior_facets_tet(int nc, const int32_t* cells, int32_t* pairs)
{
  std::vector<std::array<int32_t, 5>> keys; // sorted vertices, cell, local
  keys.reserve(4 * (size_t)nc);
  for (int c = 0; c < nc; ++c)
    for (int f = 0; f < 4; ++f)
    {
      std::array<int32_t, 3> v = {cells[4 * c + kTetFacets[f][0]],
                                  cells[4 * c + kTetFacets[f][1]],
                                  cells[4 * c + kTetFacets[f][2]]};
      std::sort(v.begin(), v.end());
      keys.push_back({v[0], v[1], v[2], c, f});
    }
  std::sort(keys.begin(), keys.end());
  std::vector<std::pair<int32_t, int32_t>> out;
  for (size_t i = 0; i < keys.size();)
  {
    size_t j = i + 1;
    while (j < keys.size() && keys[j][0] == keys[i][0] && keys[j][1] == keys[i][1]
           && keys[j][2] == keys[i][2])
      ++j;
    if (j - i == 1)
      out.push_back({keys[i][3], keys[i][4]});
    i = j;
  }
  std::sort(out.begin(), out.end());
  for (size_t i = 0; i < out.size(); ++i)
  {
    pairs[2 * i] = out[i].first;
    pairs[2 * i + 1] = out[i].second;
  }
  return (int)out.size();
}

// Interior facets of a tetrahedral mesh, the integration domain of an
// interior-facet integral on one rank (cpp/dolfinx/fem/utils.cpp:223-254:
// each facet with exactly two attached cells, written as (cell0, local
// facet0, cell1, local facet1)). Entries hold (cell0, facet0) <
// (cell1, facet1) and are sorted by (cell0, facet0). Returns the count.
int orc_interior_facets_tet(int nc, const int32_t* cells, int32_t* quads)
{
  // (sorted vertex triple) -> every (cell, local facet) with that triple
  std::map<std::array<int32_t, 3>, std::vector<std::pair<int32_t, int32_t>>> owners;
  for (int c = 0; c < nc; ++c)
    for (int f = 0; f < 4; ++f)
    {
      std::array<int32_t, 3> v = {cells[4 * c + kTetFacets[f][0]],
                                  cells[4 * c + kTetFacets[f][1]],
                                  cells[4 * c + kTetFacets[f][2]]};
      std::sort(v.begin(), v.end());
      owners[v].push_back({c, f});
    }
  std::vector<std::array<int32_t, 4>> out;
  for (auto& [v, cf] : owners)
    if (cf.size() == 2)
    {
      std::sort(cf.begin(), cf.end());
      out.push_back({cf[0].first, cf[0].second, cf[1].first, cf[1].second});
    }
  std::sort(out.begin(), out.end());
  for (size_t i = 0; i < out.size(); ++i)
    for (int k = 0; k < 4; ++k)
      quads[4 * i + k] = out[i][k];
  return (int)out.size();
}

// Exterior-facet vector loop (cpp/dolfinx/fem/assemble_vector_impl.h:
// 160-215, 571-600): L(v) = \int_F g v ds with g a P1 coefficient (values
// per geometry node; g == nullptr -> g_const), scalar P1/P2.
void orc_assemble_vector_facets(int degree, int nf, const int32_t* pairs,
                                const int32_t* x_dofmap, const double* x,
                                const int32_t* dofmap, const double* g, double g_const,
                                double* b)
{
  const int nd = tet_ndofs(degree);
  double coords[12], phi[10], dphi[10][3], l[4], dl[4][3];
  for (int e = 0; e < nf; ++e)
  {
    const int c = pairs[2 * e], f = pairs[2 * e + 1];
    cell_coords(x_dofmap, x, c, coords);
    const double two_area = 2.0 * facet_area(coords, f);
    const FacetQuad& q = facet_quadrature(f);
    double gc[4];
    for (int v = 0; v < 4; ++v)
      gc[v] = g ? g[x_dofmap[4 * c + v]] : g_const;
    for (size_t p = 0; p < q.w.size(); ++p)
    {
      tabulate_tet(degree, &q.X[3 * p], phi, dphi);
      tabulate_tet(1, &q.X[3 * p], l, dl);
      const double gq = gc[0] * l[0] + gc[1] * l[1] + gc[2] * l[2] + gc[3] * l[3];
      for (int i = 0; i < nd; ++i)
        b[dofmap[(int64_t)nd * c + i]] += q.w[p] * two_area * gq * phi[i];
    }
  }
}

// Exterior-facet matrix loop (cpp/dolfinx/fem/assemble_matrix_impl.h:
// 265-379): a(u, v) = \int_F alpha u v ds, alpha per cell of the facet
// (alpha == nullptr -> alpha_const); rows and columns of constrained dofs
// zeroed as in the cell loop; insertion by binary search.
int orc_assemble_matrix_facets(int degree, int nf, const int32_t* pairs,
                               const int32_t* x_dofmap, const double* x,
                               const int32_t* dofmap, const double* alpha,
                               double alpha_const, const int8_t* bc,
                               const int64_t* row_ptr, const int32_t* cols, double* vals)
{
  const int nd = tet_ndofs(degree);
  double coords[12], phi[10], dphi[10][3], Ae[100];
  for (int e = 0; e < nf; ++e)
  {
    const int c = pairs[2 * e], f = pairs[2 * e + 1];
    cell_coords(x_dofmap, x, c, coords);
    const double two_area = 2.0 * facet_area(coords, f);
    const double al = alpha ? alpha[c] : alpha_const;
    const FacetQuad& q = facet_quadrature(f);
    std::fill_n(Ae, 100, 0.0);
    for (size_t p = 0; p < q.w.size(); ++p)
    {
      tabulate_tet(degree, &q.X[3 * p], phi, dphi);
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j)
          Ae[i * nd + j] += q.w[p] * two_area * al * phi[i] * phi[j];
    }
    const int32_t* dofs = dofmap + (int64_t)nd * c;
    for (int i = 0; i < nd; ++i)
    {
      if (bc && bc[dofs[i]])
        continue;
      const int32_t* c0 = cols + row_ptr[dofs[i]];
      const int32_t* c1 = cols + row_ptr[dofs[i] + 1];
      for (int j = 0; j < nd; ++j)
      {
        if (bc && bc[dofs[j]])
          continue;
        const int32_t* it = std::lower_bound(c0, c1, dofs[j]);
        if (it == c1 || *it != dofs[j])
          return ORC_ERR_NOT_IN_SPARSITY;
        vals[it - cols] += Ae[i * nd + j];
      }
    }
  }
  return ORC_OK;
}

// Interior-facet matrix loop (cpp/dolfinx/fem/assemble_matrix_impl.h:
// 443-667) for the continuous interior penalty
// a(u, v) = \int_F gamma |F| [grad u . n][grad v . n] dS, gamma the mean of
// the two cells' coefficients (gamma == nullptr -> gamma_const). Macro
// element: cell0's dofs then cell1's. The facet quadrature is cell0's
// collapsed Gauss rule on its local facet, mapped to physical points and
// pulled back into cell1 through cell1's affine map; gradients are the
// reference gradients times J^{-T} of each cell; n is the unit normal out of
// cell0. Constrained rows and columns are skipped; insertion by binary
// search.
static void affine_map(const double* coords, double J[3][3], double K[3][3])
{
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < 3; ++k)
      J[d][k] = coords[3 * (k + 1) + d] - coords[d];
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1])
                     - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0])
                     + J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  K[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  K[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  K[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  K[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  K[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  K[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  K[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  K[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  K[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
}

int orc_assemble_matrix_interior_facets(int degree, int nf, const int32_t* quads,
                                        const int32_t* x_dofmap, const double* x,
                                        const int32_t* dofmap, const double* gamma,
                                        double gamma_const, const int8_t* bc,
                                        const int64_t* row_ptr, const int32_t* cols,
                                        double* vals)
{
  const int nd = tet_ndofs(degree);
  double c0[12], c1[12], J0[3][3], K0[3][3], J1[3][3], K1[3][3];
  double phi[10], dphi[10][3];
  std::vector<double> Ae(4 * nd * nd), jmp(2 * nd);
  for (int e = 0; e < nf; ++e)
  {
    const int cA = quads[4 * e], fA = quads[4 * e + 1], cB = quads[4 * e + 2];
    cell_coords(x_dofmap, x, cA, c0);
    cell_coords(x_dofmap, x, cB, c1);
    affine_map(c0, J0, K0);
    affine_map(c1, J1, K1);
    const double area = facet_area(c0, fA);
    const double* a = c0 + 3 * kTetFacets[fA][0];
    const double* b = c0 + 3 * kTetFacets[fA][1];
    const double* d = c0 + 3 * kTetFacets[fA][2];
    const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double v[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
    double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                   u[0] * v[1] - u[1] * v[0]};
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double* opp = c0 + 3 * fA;
    const double side = n[0] * (opp[0] - a[0]) + n[1] * (opp[1] - a[1]) + n[2] * (opp[2] - a[2]);
    for (int k = 0; k < 3; ++k)
      n[k] *= (side > 0 ? -1.0 : 1.0) / nn;
    const double g = 0.5 * ((gamma ? gamma[cA] : gamma_const) + (gamma ? gamma[cB] : gamma_const));
    std::fill(Ae.begin(), Ae.end(), 0.0);
    const FacetQuad& q = facet_quadrature(fA);
    for (size_t p = 0; p < q.w.size(); ++p)
    {
      const double* X0 = &q.X[3 * p];
      double xp[3], X1[3];
      for (int k = 0; k < 3; ++k)
        xp[k] = c0[k] + J0[k][0] * X0[0] + J0[k][1] * X0[1] + J0[k][2] * X0[2];
      for (int k = 0; k < 3; ++k)
        X1[k] = K1[k][0] * (xp[0] - c1[0]) + K1[k][1] * (xp[1] - c1[1])
                + K1[k][2] * (xp[2] - c1[2]);
      for (int side2 = 0; side2 < 2; ++side2)
      {
        tabulate_tet(degree, side2 == 0 ? X0 : X1, phi, dphi);
        const double(*K)[3] = side2 == 0 ? K0 : K1;
        for (int i = 0; i < nd; ++i)
        {
          // physical gradient = K^T dphi
          double gr[3];
          for (int k = 0; k < 3; ++k)
            gr[k] = K[0][k] * dphi[i][0] + K[1][k] * dphi[i][1] + K[2][k] * dphi[i][2];
          const double dn = gr[0] * n[0] + gr[1] * n[1] + gr[2] * n[2];
          jmp[side2 * nd + i] = side2 == 0 ? dn : -dn;
        }
      }
      const double wq = q.w[p] * 2.0 * area * g * area;
      for (int i = 0; i < 2 * nd; ++i)
        for (int k = 0; k < 2 * nd; ++k)
          Ae[i * 2 * nd + k] += wq * jmp[i] * jmp[k];
    }
    for (int i = 0; i < 2 * nd; ++i)
    {
      const int32_t di = dofmap[(int64_t)nd * quads[4 * e + 2 * (i / nd)] + i % nd];
      if (bc && bc[di])
        continue;
      const int32_t* r0 = cols + row_ptr[di];
      const int32_t* r1 = cols + row_ptr[di + 1];
      for (int k = 0; k < 2 * nd; ++k)
      {
        const int32_t dk = dofmap[(int64_t)nd * quads[4 * e + 2 * (k / nd)] + k % nd];
        if (bc && bc[dk])
          continue;
        const int32_t* it = std::lower_bound(r0, r1, dk);
        if (it == r1 || *it != dk)
          return ORC_ERR_NOT_IN_SPARSITY;
        vals[it - cols] += Ae[i * 2 * nd + k];
      }
    }
  }
  return ORC_OK;
}

// Functional cell loop (cpp/dolfinx/fem/assemble_scalar_impl.h:32-61),
// kind 0: M = a(u, u) = \int kappa |grad u|^2 + k2 u^2 dx; kind 1:
// M = L(u) = \int f u dx with f a P1 coefficient (f == nullptr -> 1).
double orc_assemble_scalar(int kind, int degree, int nc, const int32_t* x_dofmap,
                           const double* x, const int32_t* dofmap, const double* kappa,
                           double k2, const double* f, const double* u)
{
  const int nd = tet_ndofs(degree);
  double coords[12], Ae[100], be[10], fc[4], ue[10];
  double value = 0.0;
  for (int c = 0; c < nc; ++c)
  {
    cell_coords(x_dofmap, x, c, coords);
    for (int i = 0; i < nd; ++i)
      ue[i] = u[dofmap[(int64_t)nd * c + i]];
    if (kind == 0)
    {
      std::fill_n(Ae, 100, 0.0);
      kernel_poisson(degree, Ae, kappa ? kappa[c] : 1.0, k2, coords);
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j)
          value += ue[i] * Ae[i * nd + j] * ue[j];
    }
    else
    {
      for (int v = 0; v < 4; ++v)
        fc[v] = f ? f[x_dofmap[4 * c + v]] : 1.0;
      std::fill_n(be, 10, 0.0);
      kernel_source(degree, be, fc, coords);
      for (int i = 0; i < nd; ++i)
        value += be[i] * ue[i];
    }
  }
  return value;
}
} // extern "C"

//---------------------------------------------------------------------------
// One full step of the P2 Poisson benchmark workload on host threads: the
// CPU baseline timed beside the GPU. The reference assembles serially per
// MPI rank; here the same per-cell work (matrix_cell, the vector and
// lifting loops above) is shared by a thread team in colour classes --
// cells of one class share no dof, so no two threads add into the same
// entry -- and the solve is the demo's CG (cpp/demo/poisson_matrix_free/
// main.cpp:84-132) with Jacobi preconditioning, rows split across the
// threads and dot products summed per thread, then over the threads in
// index order (the result does not depend on thread timing).
//---------------------------------------------------------------------------
#include <barrier>
#include <thread>

namespace
{
// Element vector of the P1-coefficient source on cell c (the vector cell
// loop of orc_assemble_vector, one cell).
void vector_cell(int degree, int c, const int32_t* x_dofmap, const double* x,
                 const int32_t* dofmap, const double* f, double* b)
{
  const int nd = tet_ndofs(degree);
  double be[30], coords[12], fc[4];
  for (int v = 0; v < 4; ++v)
  {
    for (int k = 0; k < 3; ++k)
      coords[3 * v + k] = x[3 * (int64_t)x_dofmap[4 * (int64_t)c + v] + k];
    fc[v] = f ? f[x_dofmap[4 * (int64_t)c + v]] : 1.0;
  }
  std::fill_n(be, 30, 0.0);
  kernel_source(degree, be, fc, coords);
  const int32_t* dofs = dofmap + (int64_t)nd * c;
  for (int i = 0; i < nd; ++i)
    b[dofs[i]] += be[i];
}

// Lifting of one scalar cell with homogeneous-or-not BC values g (the
// loop body of orc_apply_lifting, x0 = 0, alpha = 1).
void lifting_cell(const orc_form* form, int c, const int32_t* x_dofmap, const double* x,
                  const int32_t* dofmap, const int8_t* bc, const double* g, double* b,
                  double* Ae)
{
  const int nd = tet_ndofs(form->degree);
  const int32_t* dofs = dofmap + (int64_t)nd * c;
  bool has = false;
  for (int i = 0; i < nd && !has; ++i)
    has = bc[dofs[i]] != 0;
  if (!has)
    return;
  double coords[12];
  for (int v = 0; v < 4; ++v)
    for (int k = 0; k < 3; ++k)
      coords[3 * v + k] = x[3 * (int64_t)x_dofmap[4 * (int64_t)c + v] + k];
  std::fill_n(Ae, nd * nd, 0.0);
  kernel_poisson(form->degree, Ae, form->kappa ? form->kappa[c] : 1.0, form->k2, coords);
  for (int j = 0; j < nd; ++j)
  {
    if (!bc[dofs[j]])
      continue;
    const double gj = g ? g[dofs[j]] : 0.0;
    for (int i = 0; i < nd; ++i)
      b[dofs[i]] -= Ae[i * nd + j] * gj;
  }
}

double now_s()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
} // namespace

extern "C"
{
// Greedy first-fit colouring of the cells in cell order: no two cells of a
// colour share a dof. order: (nc) cells grouped by colour; offsets:
// (max_colours + 1). Returns the number of colours, or -1 when more than
// min(max_colours, 256) are needed.
int orc_colour_cells(int nc, int nd, const int32_t* dofmap, int ndofs, int32_t* order,
                     int32_t* offsets, int max_colours)
{
  const int cap = std::min(max_colours, 256);
  std::vector<std::array<uint64_t, 4>> used(ndofs, {0, 0, 0, 0});
  std::vector<int32_t> colour(nc);
  int ncol = 0;
  for (int c = 0; c < nc; ++c)
  {
    std::array<uint64_t, 4> m{0, 0, 0, 0};
    for (int i = 0; i < nd; ++i)
      for (int w = 0; w < 4; ++w)
        m[w] |= used[dofmap[(int64_t)nd * c + i]][w];
    int col = -1;
    for (int w = 0; w < 4 && col < 0; ++w)
      if (~m[w])
        col = 64 * w + __builtin_ctzll(~m[w]);
    if (col < 0 || col >= cap)
      return -1;
    colour[c] = col;
    ncol = std::max(ncol, col + 1);
    for (int i = 0; i < nd; ++i)
      used[dofmap[(int64_t)nd * c + i]][col >> 6] |= uint64_t(1) << (col & 63);
  }
  std::fill_n(offsets, ncol + 1, 0);
  for (int c = 0; c < nc; ++c)
    ++offsets[colour[c] + 1];
  for (int k = 0; k < ncol; ++k)
    offsets[k + 1] += offsets[k];
  std::vector<int32_t> pos(offsets, offsets + ncol);
  for (int c = 0; c < nc; ++c)
    order[pos[colour[c]]++] = c;
  return ncol;
}

// One step of the scalar Poisson workload on `nthreads` threads: A = 0,
// matrix cell loop, A[d, d] = 1 on the constrained dofs, b = 0, vector cell
// loop (P1 coefficient f), lifting with BC values g, b[d] = g[d] on the
// constrained dofs, then Jacobi-PCG from u = 0 to |r|/|r0| < rtol. The
// colour classes (corder, coff, ncol) come from orc_colour_cells.
// seconds[0..2] receive the matrix, right-hand side and solve times.
// Returns the CG iteration count (negative: not converged in kmax), or
// -1000000 - status on an insertion error.
int orc_poisson_step_threaded(const orc_form* form, int nc, const int32_t* x_dofmap,
                              const double* x, const int32_t* dofmap, int ndofs,
                              const int8_t* bc, int nbc, const int32_t* bc_dofs,
                              const double* g, const double* f, const int64_t* row_ptr,
                              const int32_t* cols, double* vals, double* b, double* u,
                              const int32_t* corder, const int32_t* coff, int ncol, double rtol,
                              int kmax, int nthreads, double* seconds)
{
  if (ncol < 1 || coff[0] != 0 || coff[ncol] != nc)
    return -1000000 - ORC_ERR_INVALID; // the colour classes must cover the nc cells
  const int T = std::max(1, nthreads);
  const int64_t n = ndofs;
  const int64_t nnz = row_ptr[n];
  const int nd = tet_ndofs(form->degree);
  std::vector<double> r(n), p(n), y(n), dinv(n);
  // Row blocks with about nnz / T entries each.
  std::vector<int64_t> rb(T + 1, n);
  rb[0] = 0;
  {
    int t = 1;
    for (int64_t i = 0; i < n && t < T; ++i)
      if (row_ptr[i] >= nnz * t / T)
        rb[t++] = i;
  }
  struct alignas(64) Part
  {
    double v[3];
    int err;
  };
  std::vector<Part> part(T);
  std::barrier sync(T);
  double t0 = now_s(), t1 = 0, t2 = 0, t3 = 0;
  int result = 0;
  auto work = [&](int t)
  {
    std::vector<double> Ae(nd * nd);
    auto range = [&](int64_t lo, int64_t hi, int64_t& a, int64_t& e)
    {
      a = lo + (hi - lo) * t / T;
      e = lo + (hi - lo) * (t + 1) / T;
    };
    int64_t a, e;
    // ---- matrix
    range(0, nnz, a, e);
    std::fill(vals + a, vals + e, 0.0);
    part[t].err = 0;
    sync.arrive_and_wait();
    for (int k = 0; k < ncol; ++k)
    {
      range(coff[k], coff[k + 1], a, e);
      for (int64_t q = a; q < e; ++q)
        if (int st = matrix_cell(form, corder[q], x_dofmap, x, dofmap, bc, row_ptr, cols, vals,
                                 Ae.data()))
          part[t].err = st;
      sync.arrive_and_wait();
    }
    if (t == 0)
    {
      for (int i = 0; i < nbc; ++i)
      {
        const int32_t d = bc_dofs[i];
        const int32_t* c0 = cols + row_ptr[d];
        const int32_t* c1 = cols + row_ptr[d + 1];
        const int32_t* it = std::lower_bound(c0, c1, d);
        if (it == c1 || *it != d)
          part[0].err = ORC_ERR_NOT_IN_SPARSITY;
        else
          vals[it - cols] = 1.0;
      }
      t1 = now_s();
    }
    // ---- right-hand side
    range(0, n, a, e);
    std::fill(b + a, b + e, 0.0);
    sync.arrive_and_wait();
    for (int k = 0; k < ncol; ++k)
    {
      range(coff[k], coff[k + 1], a, e);
      for (int64_t q = a; q < e; ++q)
        vector_cell(form->degree, corder[q], x_dofmap, x, dofmap, f, b);
      sync.arrive_and_wait();
    }
    for (int k = 0; k < ncol; ++k)
    {
      range(coff[k], coff[k + 1], a, e);
      for (int64_t q = a; q < e; ++q)
        lifting_cell(form, corder[q], x_dofmap, x, dofmap, bc, g, b, Ae.data());
      sync.arrive_and_wait();
    }
    if (t == 0)
    {
      for (int i = 0; i < nbc; ++i)
        b[bc_dofs[i]] = g ? g[bc_dofs[i]] : 0.0;
      t2 = now_s();
    }
    sync.arrive_and_wait();
    // ---- Jacobi-PCG, u0 = 0: r = b, z = D^{-1} r, p = z
    const int64_t r0 = rb[t], r1 = rb[t + 1];
    double rr = 0, rz = 0;
    for (int64_t i = r0; i < r1; ++i)
    {
      double dg = 0.0;
      for (int64_t j = row_ptr[i]; j < row_ptr[i + 1]; ++j)
        if (cols[j] == i)
          dg = vals[j];
      dinv[i] = 1.0 / dg;
      u[i] = 0.0;
      r[i] = b[i];
      p[i] = dinv[i] * r[i];
      rr += r[i] * r[i];
      rz += r[i] * p[i];
    }
    part[t].v[0] = rr;
    part[t].v[1] = rz;
    sync.arrive_and_wait();
    auto total = [&](int which)
    {
      double s = 0.0;
      for (int q = 0; q < T; ++q)
        s += part[q].v[which];
      return s;
    };
    const double rr0 = total(0);
    double rzo = total(1);
    int k = 0;
    int out = 0;
    if (rr0 == 0.0)
      out = 0;
    else
      for (;;)
      {
        if (k >= kmax)
        {
          out = -k;
          break;
        }
        ++k;
        sync.arrive_and_wait(); // p complete, every thread has read the totals
        double py = 0;
        for (int64_t i = r0; i < r1; ++i)
        {
          double vi = 0.0;
          for (int64_t j = row_ptr[i]; j < row_ptr[i + 1]; ++j)
            vi += vals[j] * p[cols[j]];
          y[i] = vi;
          py += p[i] * vi;
        }
        part[t].v[2] = py;
        sync.arrive_and_wait();
        const double alpha = rzo / total(2);
        double rrn = 0, rzn = 0;
        for (int64_t i = r0; i < r1; ++i)
        {
          u[i] += alpha * p[i];
          r[i] -= alpha * y[i];
          rrn += r[i] * r[i];
          rzn += r[i] * dinv[i] * r[i];
        }
        part[t].v[0] = rrn;
        part[t].v[1] = rzn;
        sync.arrive_and_wait();
        const double rrt = total(0), rzt = total(1);
        if (rrt / rr0 < rtol * rtol)
        {
          out = k;
          break;
        }
        const double beta = rzt / rzo;
        rzo = rzt;
        for (int64_t i = r0; i < r1; ++i)
          p[i] = dinv[i] * r[i] + beta * p[i];
      }
    if (t == 0)
    {
      t3 = now_s();
      result = out;
    }
  };
  std::vector<std::thread> team;
  for (int t = 1; t < T; ++t)
    team.emplace_back(work, t);
  work(0);
  for (auto& th : team)
    th.join();
  for (int t = 0; t < T; ++t)
    if (part[t].err)
      return -1000000 - part[t].err;
  if (seconds)
  {
    seconds[0] = t1 - t0;
    seconds[1] = t2 - t1;
    seconds[2] = t3 - t2;
  }
  return result;
}
} // extern "C"
