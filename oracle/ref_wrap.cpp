// C entry points over reference DOLFINx code compiled from its own
// sources (graph/ordering.cpp, common/sort.h, la/matrix_csr_impl.h).
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ by oracle/Makefile
// when the reference tree is present, used to pin the oracle and to
// write the golden vectors under tests/golden/.
#include <cstdint>
#include <dolfinx/common/sort.h>
#include <dolfinx/graph/AdjacencyList.h>
#include <dolfinx/graph/ordering.h>
#include <dolfinx/la/matrix_csr_impl.h>
#include <functional>
#include <span>
#include <stdexcept>
#include <vector>

extern "C"
{
// graph::reorder_rcm (graph/ordering.cpp:148-170).
int ref_reorder_rcm(int n, const int32_t* off, const int32_t* adj, int32_t* r)
{
  std::vector<int32_t> data(adj, adj + off[n]), offsets(off, off + n + 1);
  dolfinx::graph::AdjacencyList<int32_t> g(std::move(data), std::move(offsets));
  std::vector<int32_t> rr = dolfinx::graph::reorder_rcm(g);
  std::copy(rr.begin(), rr.end(), r);
  return 0;
}

// sort_by_perm, column-major overload (common/sort.h:249-272), on three
// int64 columns: the facet sort of build_local_dual_graph.
int ref_sort_by_perm3(int64_t n, const int64_t* c0, const int64_t* c1,
                      const int64_t* c2, int32_t* perm)
{
  std::span<const int64_t> cols[3]
      = {std::span(c0, n), std::span(c1, n), std::span(c2, n)};
  std::vector<int32_t> p
      = dolfinx::sort_by_perm<int64_t>(std::span<std::span<const int64_t>>(cols, 3));
  std::copy(p.begin(), p.end(), perm);
  return 0;
}

// la::impl::insert_csr with add (la/matrix_csr_impl.h:67-109), bs 1 or 3.
int ref_insert_csr_add(int bs, double* data, int64_t nnz, const int32_t* cols,
                       const int64_t* row_ptr, int64_t nrows, const double* x,
                       int nr, const int32_t* xrows, int ncl,
                       const int32_t* xcols)
{
  std::span<double> d(data, nnz * bs * bs);
  std::span<const int32_t> c(cols, nnz);
  std::span<const int64_t> rp(row_ptr, nrows + 1);
  std::span<const double> xv(x, (std::size_t)nr * ncl * bs * bs);
  std::span<const int32_t> xr(xrows, nr), xc(xcols, ncl);
  auto op = [](double& a, double b) { a += b; };
  try
  {
    if (bs == 1)
      dolfinx::la::impl::insert_csr<1, 1>(d, c, rp, xv, xr, xc, op, (int32_t)nrows);
    else if (bs == 3)
      dolfinx::la::impl::insert_csr<3, 3>(d, c, rp, xv, xr, xc, op, (int32_t)nrows);
    else
      return 1;
  }
  catch (const std::runtime_error&)
  {
    return 3;
  }
  return 0;
}

// la::impl::spmv (la/matrix_csr_impl.h:259-286): y += A x.
void ref_spmv(int64_t nrows, int bs, const int64_t* row_ptr,
              const int32_t* cols, const double* vals, int64_t ncols,
              const double* x, double* y)
{
  const int64_t nnz = row_ptr[nrows];
  std::span<const double> v(vals, nnz * bs * bs);
  std::span<const int64_t> rb(row_ptr, nrows), re(row_ptr + 1, nrows);
  std::span<const int32_t> c(cols, nnz);
  std::span<const double> xs(x, ncols * bs);
  std::span<double> ys(y, nrows * bs);
  dolfinx::la::impl::spmv<double>(v, rb, re, c, xs, ys, bs, bs);
}
}
