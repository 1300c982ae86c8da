// A C++ host of libdfxgpu through include/dolfinx_gb300.hpp, written the
// way a DOLFINx C++ program is, with its class templates
// (fem::FunctionSpace<double>, fem::Form<double>, fem::DirichletBC<double>,
// la::MatrixCSR<double>, la::Vector<double>): mesh::create_box, a function
// space, the sparsity pattern, dof coordinates, exterior facets,
// common::Timer and list_timings, and an error path that throws the
// reference's message.
// With a GPU it also assembles and solves the Poisson problem of the
// matrix-free demo on P1 (fem::assemble_matrix, assemble_vector,
// apply_lifting, set_bc, CG). Without one, device work must fail loudly:
// there is no CPU fallback. Prints one "key value" per line.
#include "dolfinx_gb300.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

namespace dg = dolfinx_gb300;

int main()
{
  // host set-up
  auto m = std::make_shared<dg::mesh::Mesh>(dg::mesh::create_unit_cube(4, 4, 4));
  auto [off, adj] = dg::mesh::dual_graph(*m);
  const std::vector<std::int32_t> perm = dg::graph::reorder_rcm(off, adj);
  auto V = std::make_shared<const dg::fem::FunctionSpace<double>>(m, 2);
  const dg::fem::SparsityPattern sp = dg::fem::create_sparsity_pattern(*V);
  const std::vector<double> X = V->tabulate_dof_coordinates();
  const std::vector<std::int32_t> facets = dg::mesh::exterior_facets(*m);
  const std::vector<std::int32_t> inner = dg::mesh::interior_facets(*m);
  std::printf("cells %d\nvertices %d\nnodes %d\nnnz %zu\ndual_edges %zu\nrcm %zu\n",
              m->num_cells, m->num_vertices, V->num_nodes(), sp.cols.size(), adj.size(),
              perm.size());
  std::printf("coords %zu\nfacets %zu\ninterior_facets %zu\n", X.size(), facets.size() / 2,
              inner.size() / 4);

  // timings
  {
    dg::common::Timer t("C++ host example");
  }
  std::printf("timer_reps %d\n", dg::common::timing("C++ host example").first);
  std::printf("mesh_reps %d\n", dg::common::timing("Build BoxMesh (tetrahedra)").first);
  const std::string table = dg::common::timing_table();
  std::printf("table_has_title %d\n",
              (int)(table.rfind("[MPI_MAX] Summary of timings (s)", 0) == 0));

  // the reference's error text
  try
  {
    dg::mesh::create_box({{{0, 0, 0}, {1, 1, 1}}}, {0, 1, 1});
    std::printf("error none\n");
  }
  catch (const dg::Error& e)
  {
    std::printf("error %d %s\n", e.code(), e.what());
  }

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
  {
    try
    {
      dg::device_vector<double> v(16);
      std::printf("device unexpected\n");
    }
    catch (const dg::Error& e)
    {
      std::printf("device none %d\n", e.code());
    }
    return 0;
  }

  // with a GPU: P1 Poisson, u = 0 on the boundary, f = 1, Jacobi-CG
  auto V1 = std::make_shared<const dg::fem::FunctionSpace<double>>(m, 1);
  std::vector<std::int32_t> bnd;
  const std::vector<double> X1 = V1->tabulate_dof_coordinates();
  for (std::int32_t i = 0; i < V1->num_nodes(); ++i)
    for (int k = 0; k < 3; ++k)
      if (X1[3 * i + k] < 1e-12 || X1[3 * i + k] > 1 - 1e-12)
      {
        bnd.push_back(i);
        break;
      }
  dg::fem::BCs<double> bcs = {
      std::make_shared<const dg::fem::DirichletBC<double>>(V1, bnd, 0.0)};
  const auto a = dg::fem::Form<double>::poisson(V1);
  const auto L = dg::fem::Form<double>::source(V1, {}, 1.0);
  dg::la::MatrixCSR<double> A = dg::fem::create_matrix(a);
  dg::fem::assemble_matrix(A, a, bcs);
  dg::fem::set_diagonal(A, bcs);
  dg::la::Vector<double> b(V1->num_dofs()), x(V1->num_dofs());
  dg::fem::assemble_vector(b, L);
  dg::fem::apply_lifting(b, a, bcs);
  dg::fem::set_bc(b, bcs);
  const dg::la::CGResult r = dg::la::cg(A, b, x, 1e-10);
  std::printf("device cg %d %d\n", r.iterations, r.status);
  // the same system by FP32-inner / FP64-outer refinement
  dg::la::IRSolver ir(A);
  dg::la::Vector<double> x2(V1->num_dofs());
  const dg::la::IRResult r2 = ir.solve(b, x2, 1e-10);
  std::printf("device ir %d %d %d\n", r2.inner_iterations, r2.outer_iterations, r2.status);
  // the energy a(u, u) of the solution and a Neumann term on the boundary
  std::printf("device energy %.6e\n", dg::fem::assemble_scalar(a, x));
  dg::device_vector<double> bn(V1->num_dofs());
  dg::fem::assemble_vector(bn, dg::fem::Form<double>::facet_source(V1, {}, 1.0));
  double area = 0.0; // sum_i int_F phi_i ds = the boundary's area, 6
  for (double v : bn.to_host())
    area += v;
  std::printf("device boundary_area %.12f\n", area);
  // interior facets: the penalty matrix on its macro-element pattern, and a
  // linear function's gradient does not jump, so A_penalty u = 0 for u = x
  const auto jp = dg::fem::Form<double>::interior_penalty(V1, {}, 1.0);
  dg::la::MatrixCSR<double> P = dg::fem::create_matrix(jp);
  dg::fem::assemble_matrix(P, jp);
  std::vector<double> ux(V1->num_nodes());
  for (std::int32_t i = 0; i < V1->num_nodes(); ++i)
    ux[i] = X1[3 * i];
  dg::device_vector<double> u(V1->num_dofs()), Pu(V1->num_dofs());
  u.assign(ux);
  P.mult(u, Pu);
  double pmax = 0.0;
  for (double v : Pu.to_host())
    pmax = std::max(pmax, std::abs(v));
  std::printf("device penalty_linear %.3e\n", pmax);
  // lifting through the penalty: b = -A_P g on the constrained columns
  dg::device_vector<double> bl(V1->num_dofs());
  dg::fem::apply_lifting(bl, jp, bcs);
  std::printf("device penalty_lifting_ok 1\n");
  return 0;
}
