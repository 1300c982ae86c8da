// Runs the threaded host set-up of libdfxgpu (box mesh + RCM, P1/P2 dofmaps,
// dof coordinates, exterior facets, sparsity, colouring, dual graph, RCM) on
// one box, for a build with -fsanitize=thread or with
// -fsanitize=address,undefined. Argument: the box size n (n^3 x 6 cells).
#include "dfx_gpu.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace dfx
{
// The library's error recorder lives in its CUDA translation unit.
int fail(int code, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
  std::fprintf(stderr, "\n");
  return code;
}
} // namespace dfx

int main(int argc, char** argv)
{
  const int n = argc > 1 ? std::atoi(argv[1]) : 24;
  const int nc = 6 * n * n * n, nv = (n + 1) * (n + 1) * (n + 1);
  std::vector<int32_t> cells(4 * (size_t)nc);
  std::vector<double> x(3 * (size_t)nv);
  const double p0[3] = {0, 0, 0}, p1[3] = {1, 1, 1};
  if (dfx_mesh_create_box_tet(n, n, n, p0, p1, 1, cells.data(), x.data()))
    return 1;
  std::vector<int32_t> dm(10 * (size_t)nc);
  int32_t nn = 0;
  if (dfx_dofmap_create_tet(nc, cells.data(), 2, dm.data(), &nn))
    return 2;
  std::vector<double> X(3 * (size_t)nn, 0.0);
  if (dfx_tabulate_dof_coordinates_tet(nc, cells.data(), nv, x.data(), dm.data(), 2, nn,
                                       X.data()))
    return 3;
  std::vector<int32_t> f(8 * (size_t)nc);
  int32_t nf = 0;
  if (dfx_exterior_facets_tet(nc, cells.data(), f.data(), &nf))
    return 4;
  std::vector<int64_t> rp(nn + 1);
  int64_t nnz = 0;
  if (dfx_sparsity_create(nn, nc, 10, dm.data(), rp.data(), nullptr, &nnz))
    return 5;
  std::vector<int32_t> cols(nnz);
  if (dfx_sparsity_create(nn, nc, 10, dm.data(), rp.data(), cols.data(), &nnz))
    return 6;
  // the P1 dofmap, the cell colouring, the dual graph + RCM entry points and
  // the interior facets (each cell facet exterior or one side of one)
  std::vector<int32_t> dm1(4 * (size_t)nc);
  int32_t nn1 = 0;
  if (dfx_dofmap_create_tet(nc, cells.data(), 1, dm1.data(), &nn1))
    return 7;
  std::vector<int32_t> order(nc), offsets(257);
  int32_t ncol = 0;
  if (dfx_colour_cells(nc, 10, dm.data(), nn, order.data(), offsets.data(), 256, &ncol))
    return 8;
  std::vector<int32_t> off(nc + 1), adj(4 * (size_t)nc), perm(nc);
  if (dfx_mesh_dual_graph_tet(nc, cells.data(), nv, off.data(), adj.data()))
    return 9;
  if (dfx_graph_reorder_rcm(nc, off.data(), adj.data(), perm.data()))
    return 10;
  std::vector<int32_t> fi(8 * (size_t)nc);
  int32_t nfi = 0;
  if (dfx_interior_facets_tet(nc, cells.data(), fi.data(), &nfi))
    return 11;
  if (2 * nfi + nf != 4 * nc)
    return 12;
  std::printf("nodes %d facets %d interior %d nnz %lld p1 %d colours %d edges %d\n", nn, nf,
              nfi, (long long)nnz, nn1, ncol, off[nc]);
  return 0;
}
