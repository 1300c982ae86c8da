// dolfinx_gb300.hpp -- the C++ face of libdfxgpu: DOLFINx's C++ calls for
// the assembly + CG path (mesh::create_box, fem::assemble_matrix,
// assemble_vector, apply_lifting, DirichletBC::set, set_diagonal,
// la::MatrixCSR::mult, la::inner_product, common::Timer, list_timings, ...)
// as thin header-only wrappers over the C ABI of dfx_gpu.h. A failing call
// throws dolfinx_gb300::Error, a std::runtime_error carrying the library's
// message, which repeats the reference's text where it has one ("At least
// one cell is required.", "Entry not in sparsity", ...).
//
// Host set-up (meshes, dual graph, RCM, dofmaps, sparsity, dof coordinates,
// exterior facets, timings) runs on the CPU. Device data lives in
// device_vector, an owning container with .data() and .size() as DOLFINx's
// containers are used; there is no CPU fallback for device work.
//
// The classes keep DOLFINx's template shapes: la::MatrixCSR<Scalar,
// Container, ColContainer, RowPtrContainer>, la::Vector<T, Container>,
// fem::FunctionSpace<T>, fem::Form<T, U>, fem::DirichletBC<T, U>, with the
// containers defaulting to device_vector. The device kernels take FP64
// values and geometry, so each template admits double only (a
// static_assert says so).
//
// Paths cited below are relative to the DOLFINx source tree. C++20.
#pragma once

#include "dfx_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <string_view>
#include <type_traits>
#include <utility>
#include <vector>

namespace dolfinx_gb300
{
/// A failed library call: `code()` is the dfx_status, `what()` the message.
class Error : public std::runtime_error
{
public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int code() const noexcept { return code_; }

private:
  int code_;
};

/// Throws Error for a non-zero status with the library's message.
inline void check(int rc)
{
  if (rc != DFX_OK)
  {
    const char* m = dfx_last_error();
    throw Error(rc, (m && *m) ? m : "dfx error " + std::to_string(rc));
  }
}

inline void check_cuda(cudaError_t e, const char* what)
{
  if (e != cudaSuccess)
    throw Error(DFX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

/// Owning device array of T (cudaMalloc / cudaFree), move-only. Zeroed on
/// construction.
template <typename T>
class device_vector
{
public:
  using value_type = T;

  device_vector() = default;
  explicit device_vector(std::size_t n) { resize(n); }
  explicit device_vector(std::span<const T> host) { assign(host); }
  ~device_vector() { release(); }
  device_vector(const device_vector&) = delete;
  device_vector& operator=(const device_vector&) = delete;
  device_vector(device_vector&& o) noexcept : p_(o.p_), n_(o.n_)
  {
    o.p_ = nullptr;
    o.n_ = 0;
  }
  device_vector& operator=(device_vector&& o) noexcept
  {
    if (this != &o)
    {
      release();
      p_ = std::exchange(o.p_, nullptr);
      n_ = std::exchange(o.n_, 0);
    }
    return *this;
  }

  T* data() noexcept { return p_; }
  const T* data() const noexcept { return p_; }
  std::size_t size() const noexcept { return n_; }

  /// Reallocate to n zeroed entries.
  void resize(std::size_t n)
  {
    release();
    if (n > 0)
    {
      check_cuda(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)), "cudaMalloc");
      n_ = n;
      zero();
    }
  }
  /// Copy host values in (resizing to match).
  void assign(std::span<const T> host)
  {
    if (host.size() != n_)
      resize(host.size());
    if (n_ > 0)
      check_cuda(cudaMemcpy(p_, host.data(), n_ * sizeof(T), cudaMemcpyHostToDevice),
                 "cudaMemcpy");
  }
  std::vector<T> to_host() const
  {
    std::vector<T> h(n_);
    if (n_ > 0)
    {
      check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
      check_cuda(cudaMemcpy(h.data(), p_, n_ * sizeof(T), cudaMemcpyDeviceToHost),
                 "cudaMemcpy");
    }
    return h;
  }
  void zero()
  {
    if (n_ > 0)
      check_cuda(cudaMemset(p_, 0, n_ * sizeof(T)), "cudaMemset");
  }

private:
  void release() noexcept
  {
    if (p_)
      cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
  }
  T* p_ = nullptr;
  std::size_t n_ = 0;
};

// --------------------------------------------------------------- common
namespace common
{
/// common::Timer (common/Timer.h:38-141): started at construction;
/// stop/resume/elapsed; flush registers a stopped, named timer once; a
/// named timer still running at destruction registers its time then.
class Timer
{
  using clock = std::chrono::steady_clock;

public:
  explicit Timer(std::optional<std::string> task = std::nullopt)
      : task_(std::move(task)), start_(clock::now())
  {
  }
  ~Timer()
  {
    if (start_ && task_)
    {
      acc_ += clock::now() - *start_;
      dfx_timing_record(task_->c_str(), acc_.count());
    }
  }
  Timer(const Timer&) = delete;
  Timer& operator=(const Timer&) = delete;

  void start()
  {
    acc_ = std::chrono::duration<double>::zero();
    start_ = clock::now();
  }
  std::chrono::duration<double> elapsed() const
  {
    if (!start_)
      return acc_;
    return acc_ + std::chrono::duration<double>(clock::now() - *start_);
  }
  std::chrono::duration<double> stop()
  {
    if (start_)
    {
      acc_ += clock::now() - *start_;
      start_.reset();
    }
    return acc_;
  }
  void resume()
  {
    if (!start_)
      start_ = clock::now();
  }
  void flush()
  {
    if (start_)
      throw std::runtime_error("Timer must be stopped before flushing.");
    if (task_)
    {
      check(dfx_timing_record(task_->c_str(), acc_.count()));
      task_.reset();
    }
  }

private:
  std::optional<std::string> task_;
  std::chrono::duration<double> acc_ = std::chrono::duration<double>::zero();
  std::optional<clock::time_point> start_;
};

/// dolfinx::timing (common/timing.h:36-38): (repetitions, total seconds).
inline std::pair<int, std::chrono::duration<double>> timing(std::string_view task)
{
  const std::string t(task);
  int32_t n = 0;
  double s = 0.0;
  check(dfx_timing(t.c_str(), &n, &s));
  return {n, std::chrono::duration<double>(s)};
}

/// dolfinx::timings (common/timing.h:42-46), in byte-wise name order.
inline std::map<std::string, std::pair<int, std::chrono::duration<double>>> timings()
{
  std::map<std::string, std::pair<int, std::chrono::duration<double>>> out;
  int32_t num = 0;
  check(dfx_timing_num_tasks(&num));
  std::vector<char> name(256);
  for (int32_t i = 0; i < num; ++i)
  {
    int32_t len = 0, n = 0;
    double s = 0.0;
    check(dfx_timing_task(i, name.data(), (int32_t)name.size(), &len, &n, &s));
    if (len >= (int32_t)name.size())
    {
      name.resize(len + 1);
      check(dfx_timing_task(i, name.data(), (int32_t)name.size(), &len, &n, &s));
    }
    out.emplace(std::string(name.data(), len), std::make_pair(n, std::chrono::duration<double>(s)));
  }
  return out;
}

/// Table::Reduction (common/Table.h:33-38).
enum class Reduction : std::uint8_t
{
  average,
  max,
  min
};

/// The summary that list_timings prints for this process
/// (TimeLogger::timing_table + Table::reduce on one rank + Table::str,
/// common/TimeLogger.cpp:55-69, common/Table.cpp:71-262): title and task
/// names left-justified, reps/avg/tot right-justified, floats as "%f".
inline std::string timing_table(Reduction reduction = Reduction::max)
{
  static const char* prefix[] = {"[MPI_AVG] ", "[MPI_MAX] ", "[MPI_MIN] "};
  const std::string title = std::string(prefix[(int)reduction]) + "Summary of timings (s)";
  const auto t = timings();
  if (t.empty())
    return "";
  auto fmt = [](double v)
  {
    char b[64];
    std::snprintf(b, sizeof(b), "%f", v);
    return std::string(b);
  };
  std::vector<std::array<std::string, 4>> rows;
  std::array<std::size_t, 4> w = {title.size(), 4, 3, 3};
  for (const auto& [task, v] : t)
  {
    rows.push_back({task, std::to_string(v.first), fmt(v.second.count() / v.first),
                    fmt(v.second.count())});
    for (int j = 0; j < 4; ++j)
      w[j] = std::max(w[j], rows.back()[j].size());
  }
  auto cell = [](const std::string& s, std::size_t width, bool right)
  {
    const std::string pad(width - s.size(), ' ');
    return right ? pad + s : s + pad;
  };
  static const char* cols[] = {"reps", "avg", "tot"};
  std::string s = cell(title, w[0], false) + "  |";
  for (int j = 0; j < 3; ++j)
    s += "  " + cell(cols[j], w[j + 1], true);
  s += "\n" + std::string(2 * 4 + 1 + w[0] + w[1] + w[2] + w[3], '-');
  for (const auto& r : rows)
  {
    s += "\n" + cell(r[0], w[0], false) + "  |";
    for (int j = 1; j < 4; ++j)
      s += "  " + cell(r[j], w[j], true);
  }
  return s;
}

/// dolfinx::list_timings (common/timing.h:29) for this process.
inline void list_timings(Reduction reduction = Reduction::max)
{
  std::printf("\n%s\n", timing_table(reduction).c_str());
}
} // namespace common

// ----------------------------------------------------------------- mesh
namespace mesh
{
/// A tetrahedral mesh on the host: cells (num_cells, 4) geometry node
/// indices, x (num_vertices, 3).
struct Mesh
{
  std::int32_t num_cells = 0;
  std::int32_t num_vertices = 0;
  std::vector<std::int32_t> cells;
  std::vector<double> x;
};

/// mesh::create_box(comm, p, n, CellType::tetrahedron) on one rank, with
/// the default RCM cell order (mesh/generation.h:104-134, 380-426).
inline Mesh create_box(const std::array<std::array<double, 3>, 2>& p,
                       const std::array<std::int32_t, 3>& n, bool reorder = true)
{
  Mesh m;
  const std::int64_t nc = 6 * (std::int64_t)n[0] * n[1] * n[2];
  const std::int64_t nv = (std::int64_t)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
  if (n[0] >= 1 && n[1] >= 1 && n[2] >= 1)
  {
    m.cells.resize(4 * nc);
    m.x.resize(3 * nv);
  }
  check(dfx_mesh_create_box_tet(n[0], n[1], n[2], p[0].data(), p[1].data(), reorder ? 1 : 0,
                                m.cells.data(), m.x.data()));
  m.num_cells = (std::int32_t)nc;
  m.num_vertices = (std::int32_t)nv;
  return m;
}

/// The unit cube [0, 1]^3.
inline Mesh create_unit_cube(std::int32_t nx, std::int32_t ny, std::int32_t nz,
                             bool reorder = true)
{
  return create_box({{{0.0, 0.0, 0.0}, {1.0, 1.0, 1.0}}}, {nx, ny, nz}, reorder);
}

/// mesh::build_local_dual_graph (mesh/graphbuild.cpp:566-905): (offsets,
/// adjacency) of the cells that share a facet.
inline std::pair<std::vector<std::int32_t>, std::vector<std::int32_t>> dual_graph(const Mesh& m)
{
  std::vector<std::int32_t> off(m.num_cells + 1), adj(4 * (std::size_t)m.num_cells);
  check(dfx_mesh_dual_graph_tet(m.num_cells, m.cells.data(), m.num_vertices, off.data(),
                                adj.data()));
  adj.resize(off.back());
  return {std::move(off), std::move(adj)};
}

/// Exterior facets as (cell, local facet) pairs, sorted
/// (mesh::exterior_facet_indices + compute_integration_domains,
/// mesh/utils.cpp:61-89, fem/utils.h:155-162).
inline std::vector<std::int32_t> exterior_facets(const Mesh& m)
{
  std::vector<std::int32_t> f(8 * (std::size_t)m.num_cells);
  std::int32_t nf = 0;
  check(dfx_exterior_facets_tet(m.num_cells, m.cells.data(), f.data(), &nf));
  f.resize(2 * (std::size_t)nf);
  return f;
}

/// Interior facets as (cell0, local facet0, cell1, local facet1), sorted:
/// the interior-facet integration domain (compute_integration_domains,
/// fem/utils.cpp:223-254).
inline std::vector<std::int32_t> interior_facets(const Mesh& m)
{
  std::vector<std::int32_t> f(8 * (std::size_t)m.num_cells);
  std::int32_t nf = 0;
  check(dfx_interior_facets_tet(m.num_cells, m.cells.data(), f.data(), &nf));
  f.resize(4 * (std::size_t)nf);
  return f;
}
} // namespace mesh

// ---------------------------------------------------------------- graph
namespace graph
{
/// graph::reorder_rcm (graph/ordering.cpp:148-170): perm[old] = new.
inline std::vector<std::int32_t> reorder_rcm(std::span<const std::int32_t> offsets,
                                             std::span<const std::int32_t> adj)
{
  if (offsets.empty())
    throw Error(DFX_ERR_INVALID, "offsets must have n+1 entries");
  std::vector<std::int32_t> perm(offsets.size() - 1);
  check(dfx_graph_reorder_rcm((std::int32_t)perm.size(), offsets.data(), adj.data(),
                              perm.data()));
  return perm;
}
} // namespace graph

// ------------------------------------------------------- fem (host side)
namespace fem
{
/// Lagrange P1/P2 space (scalar, or vector with bs = 3) on a tetrahedral
/// mesh: the dofmap of fem::create_dofmap (fem/utils.cpp:32-76), numbered
/// as DOLFINx numbers it on one rank. Device copies of the mesh and dofmap
/// are made on first use.
template <typename T = double>
class FunctionSpace
{
  static_assert(std::is_same_v<T, double>, "the device kernels take FP64 geometry");

public:
  using geometry_type = T;
  FunctionSpace(std::shared_ptr<const mesh::Mesh> m, int degree, int bs = 1)
      : mesh_(std::move(m)), degree_(degree), bs_(bs)
  {
    if (bs != 1 && bs != 3)
      throw Error(DFX_ERR_UNSUPPORTED, "block size must be 1 or 3");
    dofmap_.resize((std::size_t)mesh_->num_cells * (degree == 1 ? 4 : 10));
    check(dfx_dofmap_create_tet(mesh_->num_cells, mesh_->cells.data(), degree, dofmap_.data(),
                                &num_nodes_));
  }
  const mesh::Mesh& mesh() const { return *mesh_; }
  int degree() const { return degree_; }
  int bs() const { return bs_; }
  int ndofs_cell() const { return degree_ == 1 ? 4 : 10; }
  std::int32_t num_nodes() const { return num_nodes_; }
  std::int64_t num_dofs() const { return (std::int64_t)num_nodes_ * bs_; }
  std::span<const std::int32_t> dofmap() const { return dofmap_; }

  /// FunctionSpace::tabulate_dof_coordinates (fem/FunctionSpace.h:218-330):
  /// (num_nodes, 3) row-major, vertices then edge midpoints.
  std::vector<double> tabulate_dof_coordinates() const
  {
    std::vector<double> X(3 * (std::size_t)num_nodes_, 0.0);
    check(dfx_tabulate_dof_coordinates_tet(mesh_->num_cells, mesh_->cells.data(),
                                           mesh_->num_vertices, mesh_->x.data(),
                                           dofmap_.data(), degree_, num_nodes_, X.data()));
    return X;
  }

  const std::int32_t* device_cells() const { return upload().cells.data(); }
  const double* device_x() const { return upload().x.data(); }
  const std::int32_t* device_dofmap() const { return upload().dofmap.data(); }

private:
  struct Device
  {
    device_vector<std::int32_t> cells, dofmap;
    device_vector<double> x;
  };
  const Device& upload() const
  {
    if (!dev_)
    {
      auto d = std::make_unique<Device>();
      d->cells.assign(mesh_->cells);
      d->x.assign(mesh_->x);
      d->dofmap.assign(dofmap_);
      dev_ = std::move(d);
    }
    return *dev_;
  }
  std::shared_ptr<const mesh::Mesh> mesh_;
  int degree_, bs_;
  std::int32_t num_nodes_ = 0;
  std::vector<std::int32_t> dofmap_;
  mutable std::unique_ptr<Device> dev_;
};

/// The cell sparsity pattern in CSR form (node blocks).
struct SparsityPattern
{
  std::vector<std::int64_t> row_ptr;
  std::vector<std::int32_t> cols;
};

/// fem::create_sparsity_pattern + SparsityPattern::finalize
/// (fem/utils.h:197-314, la/SparsityPattern.cpp:264-491), on the host.
template <typename U>
SparsityPattern create_sparsity_pattern(const FunctionSpace<U>& V)
{
  SparsityPattern sp;
  sp.row_ptr.resize(V.num_nodes() + 1);
  std::int64_t nnz = 0;
  const auto dm = V.dofmap();
  check(dfx_sparsity_create(V.num_nodes(), V.mesh().num_cells, V.ndofs_cell(), dm.data(),
                            sp.row_ptr.data(), nullptr, &nnz));
  sp.cols.resize(nnz);
  check(dfx_sparsity_create(V.num_nodes(), V.mesh().num_cells, V.ndofs_cell(), dm.data(),
                            sp.row_ptr.data(), sp.cols.data(), &nnz));
  return sp;
}
} // namespace fem

// ------------------------------------------------------------------- la
namespace la
{
/// la::Vector<T, Container> (la/Vector.h:35-120) on the device: the
/// entries of one rank (no ghosts), in block size bs.
template <typename T = double, typename Container = device_vector<T>>
class Vector
{
  static_assert(std::is_same_v<T, double>, "the device kernels take FP64 vectors");

public:
  using value_type = T;
  using container_type = Container;
  Vector(std::int64_t n, int bs = 1) : bs_(bs), x_((std::size_t)n * bs) {}
  int bs() const { return bs_; }
  std::size_t size() const { return x_.size(); }
  /// The entries (device memory).
  std::span<const T> array() const { return {x_.data(), x_.size()}; }
  std::span<T> mutable_array() { return {x_.data(), x_.size()}; }
  /// Set every entry to v.
  void set(T v)
  {
    if (v == T(0))
      x_.zero();
    else
      x_.assign(std::vector<T>(x_.size(), v));
  }
  Container& device() { return x_; }
  const Container& device() const { return x_; }

private:
  int bs_;
  Container x_;
};

/// la::MatrixCSR<Scalar, Container, ColContainer, RowPtrContainer>
/// (la/MatrixCSR.h:67-70) on the device: int64 row pointers, int32
/// columns, FP64 values of bs x bs row-major blocks.
template <typename Scalar = double, typename Container = device_vector<Scalar>,
          typename ColContainer = device_vector<std::int32_t>,
          typename RowPtrContainer = device_vector<std::int64_t>>
class MatrixCSR
{
  static_assert(std::is_same_v<Scalar, double>, "the device kernels take FP64 values");

public:
  using value_type = Scalar;
  MatrixCSR(const fem::SparsityPattern& sp, int bs = 1)
      : nrows_((std::int32_t)sp.row_ptr.size() - 1), bs_(bs), row_ptr_(sp.row_ptr),
        cols_(sp.cols), vals_(sp.cols.size() * bs * bs)
  {
  }
  std::int32_t num_rows() const { return nrows_; }
  int bs() const { return bs_; }
  /// MatrixCSR::block_size.
  std::array<int, 2> block_size() const { return {bs_, bs_}; }
  std::int64_t nnz() const { return (std::int64_t)cols_.size(); }
  Container& values() { return vals_; }
  const Container& values() const { return vals_; }
  const RowPtrContainer& row_ptr() const { return row_ptr_; }
  const ColContainer& cols() const { return cols_; }
  void set_zero() { vals_.zero(); }
  /// MatrixCSR::set: every stored value to x.
  void set(Scalar x)
  {
    if (x == Scalar(0))
      vals_.zero();
    else
      vals_.assign(std::vector<Scalar>(vals_.size(), x));
  }

  /// The dfx_csr view of this matrix for the C ABI.
  dfx_csr csr() const
  {
    return dfx_csr{nrows_,          nrows_,       bs_,
                   DFX_F64,         nnz(),        row_ptr_.data(),
                   cols_.data(),    const_cast<double*>(vals_.data())};
  }

  /// MatrixCSR::mult (la/MatrixCSR.h:877-946): y += A x.
  void mult(const device_vector<Scalar>& x, device_vector<Scalar>& y) const
  {
    const std::size_t n = (std::size_t)nrows_ * bs_;
    if (x.size() != n || y.size() != n)
      throw Error(DFX_ERR_INVALID, "x and y must have num_rows * bs entries");
    const dfx_csr A = csr();
    check(dfx_spmv(&A, x.data(), y.data(), 1.0, nullptr));
  }
  void mult(const Vector<Scalar>& x, Vector<Scalar>& y) const { mult(x.device(), y.device()); }

private:
  std::int32_t nrows_;
  int bs_;
  RowPtrContainer row_ptr_;
  ColContainer cols_;
  Container vals_;
};

/// la::inner_product (la/Vector.h:434-460), a deterministic reduction.
inline double inner_product(const device_vector<double>& a, const device_vector<double>& b)
{
  if (a.size() != b.size())
    throw Error(DFX_ERR_INVALID, "vectors must have the same size");
  const std::size_t wb = dfx_inner_product_workspace_bytes((std::int64_t)a.size());
  device_vector<double> work(wb / sizeof(double) + 1);
  double r = 0.0;
  check(dfx_inner_product(a.data(), b.data(), (std::int64_t)a.size(), work.data(), wb, &r,
                          nullptr));
  return r;
}

/// la::norm(x, Norm::l2) (la/Vector.h:489-514).
inline double norm(const device_vector<double>& x) { return std::sqrt(inner_product(x, x)); }

template <typename T>
T inner_product(const Vector<T>& a, const Vector<T>& b)
{
  return inner_product(a.device(), b.device());
}

/// la::Norm (la/utils.h): only the l2 norm is provided on the device.
enum class Norm
{
  l2
};

template <typename T>
T norm(const Vector<T>& x, Norm type = Norm::l2)
{
  (void)type;
  return norm(x.device());
}
} // namespace la

// ----------------------------------------------------- fem (device side)
namespace fem
{
/// A built-in form on a space (in place of a UFL form compiled by FFCx):
/// the element kernel is chosen by the kind, coefficients live on the
/// device. Per-cell coefficients have one value per cell, P1 sources one
/// value per geometry node; an empty span selects the constant.
template <typename T = double, typename U = T>
class Form
{
  static_assert(std::is_same_v<T, double> && std::is_same_v<U, double>,
                "the device kernels take FP64 values and geometry");
  using FunctionSpace = fem::FunctionSpace<U>;

public:
  using scalar_type = T;
  using geometry_type = U;
  static Form poisson(std::shared_ptr<const FunctionSpace> V, std::span<const double> kappa = {},
                      double kappa_const = 1.0, double k2 = 0.0)
  {
    Form a(DFX_FORM_POISSON, std::move(V));
    a.set_kappa(kappa, kappa_const);
    a.k2_ = k2;
    return a;
  }
  static Form elasticity(std::shared_ptr<const FunctionSpace> V, std::span<const double> E = {},
                         double E_const = 1.0, double nu = 0.3)
  {
    if (V->bs() != 3 || V->degree() != 2)
      throw Error(DFX_ERR_INVALID, "elasticity needs a vector P2 space (block size 3)");
    Form a(DFX_FORM_ELASTICITY, std::move(V));
    a.set_kappa(E, E_const);
    a.nu_ = nu;
    return a;
  }
  static Form source(std::shared_ptr<const FunctionSpace> V, std::span<const double> f = {},
                     double f_const = 1.0)
  {
    Form L(DFX_FORM_SOURCE, std::move(V));
    if (!f.empty())
    {
      if (f.size() != (std::size_t)L.V_->mesh().num_vertices)
        throw Error(DFX_ERR_INVALID, "f must have one value per geometry node");
      L.f_.assign(f);
    }
    L.f_const_ = {f_const, 0.0, 0.0};
    return L;
  }
  static Form body_force(std::shared_ptr<const FunctionSpace> V, std::array<double, 3> f)
  {
    if (V->bs() != 3 || V->degree() != 2)
      throw Error(DFX_ERR_INVALID, "a body force needs a vector P2 space (block size 3)");
    Form L(DFX_FORM_BODYFORCE, std::move(V));
    L.f_const_ = f;
    return L;
  }
  /// L(v) = int_F g v ds over exterior facets given as (cell, local facet)
  /// pairs (all boundary facets when empty); g per geometry node or g_const.
  static Form facet_source(std::shared_ptr<const FunctionSpace> V, std::span<const double> g = {},
                           double g_const = 1.0, std::span<const std::int32_t> facets = {})
  {
    Form L = source(std::move(V), g, g_const);
    L.set_facets(facets);
    return L;
  }
  /// a(u,v) = int_F alpha u v ds (a Robin term), alpha per cell or alpha_const.
  static Form facet_mass(std::shared_ptr<const FunctionSpace> V,
                         std::span<const double> alpha = {}, double alpha_const = 1.0,
                         std::span<const std::int32_t> facets = {})
  {
    if (V->bs() != 1)
      throw Error(DFX_ERR_INVALID, "facet forms need a scalar space");
    Form a(DFX_FORM_FACET_MASS, std::move(V));
    a.set_kappa(alpha, alpha_const);
    a.set_facets(facets);
    return a;
  }

  /// L(v) = int_F avg(g) avg(v) dS over interior facets given as (cell0,
  /// facet0, cell1, facet1) quads (all of them when empty).
  static Form interior_facet_source(std::shared_ptr<const FunctionSpace> V,
                                    std::span<const double> g = {}, double g_const = 1.0,
                                    std::span<const std::int32_t> facets = {})
  {
    Form L = source(std::move(V), g, g_const);
    L.set_interior_facets(facets);
    return L;
  }
  /// a(u,v) = int_F gamma |F| [grad u . n][grad v . n] dS (continuous
  /// interior penalty), gamma per cell (averaged over the facet's two
  /// cells) or gamma_const. Its matrix needs the facets' macro-element
  /// couplings: create_matrix adds them.
  static Form interior_penalty(std::shared_ptr<const FunctionSpace> V,
                               std::span<const double> gamma = {}, double gamma_const = 1.0,
                               std::span<const std::int32_t> facets = {})
  {
    if (V->bs() != 1)
      throw Error(DFX_ERR_INVALID, "facet forms need a scalar space");
    Form a(DFX_FORM_FACET_JUMP, std::move(V));
    a.set_kappa(gamma, gamma_const);
    a.set_interior_facets(facets);
    return a;
  }

  const FunctionSpace& function_space() const { return *V_; }
  bool bilinear() const
  {
    return kind_ == DFX_FORM_POISSON || kind_ == DFX_FORM_ELASTICITY ||
           kind_ == DFX_FORM_FACET_MASS || kind_ == DFX_FORM_FACET_JUMP;
  }
  /// A facet integral, exterior or interior (else a cell integral).
  bool on_facets() const { return num_facets_ >= 0; }
  /// An interior-facet integral (dS).
  bool interior() const { return interior_; }
  /// The interior facets as host quads (for the sparsity pattern).
  const std::vector<std::int32_t>& host_facets() const { return host_facets_; }
  const std::int32_t* device_facets() const { return facets_.data(); }
  std::int32_t num_facets() const { return num_facets_; }

  /// The dfx_form view for the C ABI (uploads the space on first use).
  dfx_form c() const
  {
    dfx_form f{};
    f.kind = kind_;
    f.degree = V_->degree();
    f.num_cells = V_->mesh().num_cells;
    f.num_nodes = V_->mesh().num_vertices;
    f.x_dofmap = V_->device_cells();
    f.x = V_->device_x();
    f.dofmap = V_->device_dofmap();
    f.kappa = kappa_.size() ? kappa_.data() : nullptr;
    f.kappa_const = kappa_const_;
    f.k2 = k2_;
    f.nu = nu_;
    f.f = f_.size() ? f_.data() : nullptr;
    for (int i = 0; i < 3; ++i)
      f.f_const[i] = f_const_[i];
    return f;
  }

private:
  Form(int kind, std::shared_ptr<const FunctionSpace> V) : kind_(kind), V_(std::move(V)) {}
  void set_kappa(std::span<const double> k, double c)
  {
    if (!k.empty())
    {
      if (k.size() != (std::size_t)V_->mesh().num_cells)
        throw Error(DFX_ERR_INVALID, "the coefficient must have one value per cell");
      kappa_.assign(k);
    }
    kappa_const_ = c;
  }
  void set_facets(std::span<const std::int32_t> facets)
  {
    if (V_->bs() != 1)
      throw Error(DFX_ERR_INVALID, "facet forms need a scalar space");
    std::vector<std::int32_t> f(facets.begin(), facets.end());
    if (f.empty())
      f = mesh::exterior_facets(V_->mesh());
    if (f.size() % 2)
      throw Error(DFX_ERR_INVALID, "facets must be (cell, local facet) pairs");
    for (std::size_t i = 0; i < f.size(); i += 2)
      if (f[i] < 0 || f[i] >= V_->mesh().num_cells || f[i + 1] < 0 || f[i + 1] > 3)
        throw Error(DFX_ERR_INVALID, "facets must be (cell, local facet < 4) pairs in the mesh");
    facets_.assign(f);
    num_facets_ = (std::int32_t)(f.size() / 2);
  }
  void set_interior_facets(std::span<const std::int32_t> facets)
  {
    if (V_->bs() != 1)
      throw Error(DFX_ERR_INVALID, "facet forms need a scalar space");
    std::vector<std::int32_t> f(facets.begin(), facets.end());
    if (f.empty())
      f = mesh::interior_facets(V_->mesh());
    if (f.size() % 4)
      throw Error(DFX_ERR_INVALID, "interior facets must be (cell, facet, cell, facet) quads");
    for (std::size_t i = 0; i < f.size(); i += 2)
      if (f[i] < 0 || f[i] >= V_->mesh().num_cells || f[i + 1] < 0 || f[i + 1] > 3)
        throw Error(DFX_ERR_INVALID, "interior facets must be quads of cells of the mesh");
    facets_.assign(f);
    num_facets_ = (std::int32_t)(f.size() / 4);
    interior_ = true;
    host_facets_ = std::move(f);
  }
  int kind_;
  bool interior_ = false;
  std::vector<std::int32_t> host_facets_;
  std::shared_ptr<const FunctionSpace> V_;
  device_vector<double> kappa_, f_;
  device_vector<std::int32_t> facets_;
  std::int32_t num_facets_ = -1;
  double kappa_const_ = 1.0, k2_ = 0.0, nu_ = 0.3;
  std::array<double, 3> f_const_ = {0.0, 0.0, 0.0};
};

/// DirichletBC (fem/DirichletBC.h): u = g on the given nodes (all bs
/// components), g a constant or a full vector of num_dofs values.
template <typename T = double, typename U = T>
class DirichletBC
{
  static_assert(std::is_same_v<T, double> && std::is_same_v<U, double>,
                "the device kernels take FP64 values and geometry");
  using FunctionSpace = fem::FunctionSpace<U>;

public:
  DirichletBC(std::shared_ptr<const FunctionSpace> V, std::span<const std::int32_t> nodes,
              double value)
      : V_(std::move(V)), g_const_(value)
  {
    set_dofs(nodes);
  }
  DirichletBC(std::shared_ptr<const FunctionSpace> V, std::span<const std::int32_t> nodes,
              std::span<const double> values)
      : V_(std::move(V))
  {
    if (values.size() != (std::size_t)V_->num_dofs())
      throw Error(DFX_ERR_INVALID, "BC value must be a constant or a full dof vector");
    set_dofs(nodes);
    g_.assign(values);
  }

  const FunctionSpace& function_space() const { return *V_; }
  /// The constrained scalar dofs (bs * node + component), sorted.
  std::span<const std::int32_t> dofs() const { return dofs_host_; }

  /// DirichletBC::set (fem/DirichletBC.h:495-578): x[d] = alpha (g - x0).
  void set(device_vector<double>& x, const device_vector<double>* x0 = nullptr,
           double alpha = 1.0) const
  {
    if (x.size() != (std::size_t)V_->num_dofs() || (x0 && x0->size() != x.size()))
      throw Error(DFX_ERR_INVALID, "x (and x0) must have num_dofs entries");
    check(dfx_set_bc(x.data(), (std::int64_t)x.size(), dofs_.data(),
                     (std::int32_t)dofs_host_.size(), g_.size() ? g_.data() : nullptr, g_const_,
                     x0 ? x0->data() : nullptr, alpha, nullptr));
  }
  void set(la::Vector<T>& x, const la::Vector<T>* x0 = nullptr, T alpha = 1.0) const
  {
    set(x.device(), x0 ? &x0->device() : nullptr, alpha);
  }
  const std::int32_t* device_dofs() const { return dofs_.data(); }

private:
  void set_dofs(std::span<const std::int32_t> nodes)
  {
    std::vector<std::int32_t> n(nodes.begin(), nodes.end());
    std::sort(n.begin(), n.end());
    n.erase(std::unique(n.begin(), n.end()), n.end());
    if (!n.empty() && (n.front() < 0 || n.back() >= V_->num_nodes()))
      throw Error(DFX_ERR_INVALID, "Dirichlet dofs must lie in the space");
    for (std::int32_t v : n)
      for (int k = 0; k < V_->bs(); ++k)
        dofs_host_.push_back(V_->bs() * v + k);
    dofs_.assign(dofs_host_);
  }
  std::shared_ptr<const FunctionSpace> V_;
  std::vector<std::int32_t> dofs_host_;
  device_vector<std::int32_t> dofs_;
  device_vector<double> g_;
  double g_const_ = 0.0;
};

/// The boundary conditions of an assembly call.
template <typename T = double, typename U = T>
using BCs = std::vector<std::shared_ptr<const DirichletBC<T, U>>>;

namespace detail
{
// Device markers (1 on constrained scalar dofs) and BC values of a space.
struct Lifting
{
  device_vector<std::int8_t> markers;
  device_vector<double> g;
};
template <typename T, typename U>
Lifting lifting_data(const FunctionSpace<U>& V, const BCs<T, U>& bcs)
{
  Lifting l;
  std::vector<std::int8_t> mk(V.num_dofs(), 0);
  for (const auto& bc : bcs)
    for (std::int32_t d : bc->dofs())
      mk[d] = 1;
  l.markers.assign(mk);
  l.g.resize(V.num_dofs());
  for (const auto& bc : bcs)
    bc->set(l.g);
  return l;
}
} // namespace detail

/// A zeroed matrix with the sparsity pattern of the form's space.
template <typename T, typename U>
la::MatrixCSR<T> create_matrix(const Form<T, U>& a)
{
  if (!a.interior())
    return la::MatrixCSR<T>(create_sparsity_pattern(a.function_space()),
                            a.function_space().bs());
  // sparsitybuild::cells + interior_facets: the cells, each listed twice so
  // that every element has 2 nd dofs (repeats are dropped), then every
  // facet's macro element (both cells' dofs).
  const FunctionSpace<U>& V = a.function_space();
  const int nd = V.degree() == 1 ? 4 : 10;
  const std::span<const std::int32_t> dm = V.dofmap();
  const std::vector<std::int32_t>& q = a.host_facets();
  const std::int64_t nc = V.mesh().num_cells, nf = (std::int64_t)q.size() / 4;
  std::vector<std::int32_t> macro((std::size_t)(nc + nf) * 2 * nd);
  for (std::int64_t c = 0; c < nc; ++c)
    for (int k = 0; k < 2 * nd; ++k)
      macro[(std::size_t)c * 2 * nd + k] = dm[(std::size_t)c * nd + k % nd];
  for (std::int64_t e = 0; e < nf; ++e)
    for (int k = 0; k < 2 * nd; ++k)
      macro[(std::size_t)(nc + e) * 2 * nd + k] =
          dm[(std::size_t)q[4 * e + 2 * (k / nd)] * nd + k % nd];
  SparsityPattern sp;
  sp.row_ptr.resize((std::size_t)V.num_nodes() + 1);
  std::int64_t nnz = 0;
  check(dfx_sparsity_create(V.num_nodes(), (std::int32_t)(nc + nf), 2 * nd, macro.data(),
                            sp.row_ptr.data(), nullptr, &nnz));
  sp.cols.resize((std::size_t)nnz);
  check(dfx_sparsity_create(V.num_nodes(), (std::int32_t)(nc + nf), 2 * nd, macro.data(),
                            sp.row_ptr.data(), sp.cols.data(), &nnz));
  return la::MatrixCSR<T>(sp, V.bs());
}

/// fem::assemble_matrix (fem/assembler.h:513-602): A += the cell
/// integrals, rows and columns of constrained dofs left out. A is not
/// zeroed (the reference's accumulate semantics).
template <typename T, typename U>
void assemble_matrix(la::MatrixCSR<T>& A, const Form<T, U>& a, const BCs<T, U>& bcs = {})
{
  if (!a.bilinear())
    throw Error(DFX_ERR_INVALID, "assemble_matrix needs a bilinear form");
  const FunctionSpace<U>& V = a.function_space();
  if (A.num_rows() != V.num_nodes() || A.bs() != V.bs())
    throw Error(DFX_ERR_INVALID, "A does not match the form's space");
  std::optional<detail::Lifting> l;
  if (!bcs.empty())
    l = detail::lifting_data(V, bcs);
  const dfx_form f = a.c();
  const dfx_csr csr = A.csr();
  const std::int8_t* bc = l ? l->markers.data() : nullptr;
  if (a.interior())
    check(dfx_assemble_matrix_interior_facets(&f, a.device_facets(), a.num_facets(), &csr, bc,
                                              nullptr));
  else if (a.on_facets())
    check(dfx_assemble_matrix_facets(&f, a.device_facets(), a.num_facets(), &csr, nullptr, bc,
                                     nullptr));
  else
    check(dfx_assemble_matrix(&f, &csr, nullptr, bc, DFX_MODE_ATOMIC, nullptr, nullptr, 0,
                              nullptr));
}

/// set_diagonal (fem/assembler.h:644-686): A[d, d] = diagonal on every
/// constrained dof.
template <typename T, typename U>
void set_diagonal(la::MatrixCSR<T>& A, const BCs<T, U>& bcs, T diagonal = 1.0)
{
  const dfx_csr csr = A.csr();
  for (const auto& bc : bcs)
    check(dfx_set_diagonal(&csr, bc->device_dofs(), (std::int32_t)bc->dofs().size(), diagonal,
                           nullptr));
}

/// fem::assemble_vector (fem/assembler.h:229-257): b += the cell integrals.
template <typename T, typename U>
void assemble_vector(device_vector<T>& b, const Form<T, U>& L)
{
  if (L.bilinear())
    throw Error(DFX_ERR_INVALID, "assemble_vector needs a linear form");
  if (b.size() != (std::size_t)L.function_space().num_dofs())
    throw Error(DFX_ERR_INVALID, "b must have num_dofs entries");
  const dfx_form f = L.c();
  if (L.interior())
    check(dfx_assemble_vector_interior_facets(&f, L.device_facets(), L.num_facets(), b.data(),
                                              nullptr));
  else if (L.on_facets())
    check(dfx_assemble_vector_facets(&f, L.device_facets(), L.num_facets(), b.data(), nullptr));
  else
    check(dfx_assemble_vector(&f, b.data(), DFX_MODE_ATOMIC, nullptr, nullptr, 0, nullptr));
}

/// fem::assemble_scalar over the cells (fem/assembler.h:173-215): a(u, u)
/// of a Poisson/Helmholtz form or L(u) of a source form, summed in a fixed
/// order.
template <typename T, typename U>
T assemble_scalar(const Form<T, U>& M, const device_vector<T>& u)
{
  if (M.on_facets())
    throw Error(DFX_ERR_UNSUPPORTED, "functionals are cell integrals");
  if (u.size() != (std::size_t)M.function_space().num_dofs())
    throw Error(DFX_ERR_INVALID, "u must have num_dofs entries");
  const dfx_form f = M.c();
  const std::size_t wb = dfx_assemble_scalar_workspace_bytes(f.num_cells);
  device_vector<double> work(wb / sizeof(double) + 1);
  double v = 0.0;
  check(dfx_assemble_scalar(&f, u.data(), &v, work.data(), wb, nullptr));
  return v;
}

/// fem::apply_lifting for one bilinear form (fem/assembler.h:336-421):
/// b -= alpha A (g - x0) over the constrained columns.
template <typename T, typename U>
void apply_lifting(device_vector<T>& b, const Form<T, U>& a, const BCs<T, U>& bcs,
                   const device_vector<T>* x0 = nullptr, T alpha = 1.0)
{
  if (bcs.empty())
    return;
  const FunctionSpace<U>& V = a.function_space();
  if (b.size() != (std::size_t)V.num_dofs() || (x0 && x0->size() != b.size()))
    throw Error(DFX_ERR_INVALID, "b (and x0) must have num_dofs entries");
  const detail::Lifting l = detail::lifting_data(V, bcs);
  const dfx_form f = a.c();
  if (a.on_facets())
  {
    // lift_bc over the facet domain (exterior mass or interior penalty)
    check(dfx_apply_lifting_facets(&f, a.device_facets(), a.num_facets(), a.interior() ? 1 : 0,
                                   b.data(), l.markers.data(), l.g.data(),
                                   x0 ? x0->data() : nullptr, alpha, nullptr));
    return;
  }
  check(dfx_apply_lifting(&f, b.data(), l.markers.data(), l.g.data(), x0 ? x0->data() : nullptr,
                          alpha, DFX_MODE_ATOMIC, nullptr, nullptr, 0, nullptr));
}

/// fem::set_bc: DirichletBC::set for each condition.
template <typename T, typename U>
void set_bc(device_vector<T>& b, const BCs<T, U>& bcs, const device_vector<T>* x0 = nullptr,
            T alpha = 1.0)
{
  for (const auto& bc : bcs)
    bc->set(b, x0, alpha);
}

// The same calls on la::Vector.
template <typename T, typename U>
void assemble_vector(la::Vector<T>& b, const Form<T, U>& L)
{
  assemble_vector(b.device(), L);
}
template <typename T, typename U>
T assemble_scalar(const Form<T, U>& M, const la::Vector<T>& u)
{
  return assemble_scalar(M, u.device());
}
template <typename T, typename U>
void apply_lifting(la::Vector<T>& b, const Form<T, U>& a, const BCs<T, U>& bcs,
                   const la::Vector<T>* x0 = nullptr, T alpha = 1.0)
{
  apply_lifting(b.device(), a, bcs, x0 ? &x0->device() : nullptr, alpha);
}
template <typename T, typename U>
void set_bc(la::Vector<T>& b, const BCs<T, U>& bcs, const la::Vector<T>* x0 = nullptr,
            T alpha = 1.0)
{
  set_bc(b.device(), bcs, x0 ? &x0->device() : nullptr, alpha);
}
} // namespace fem

namespace la
{
struct CGResult
{
  int iterations;
  int status;
  double rnorm0_sq, rnorm_sq;
};

/// Jacobi-preconditioned CG (the demo's CG, demo/poisson_matrix_free/
/// main.cpp:84-132, with z = D^-1 r), FP64, stopping at |r|/|r0| < rtol.
/// x holds the initial guess. Throws on non-convergence or breakdown.
template <typename T>
CGResult cg(const MatrixCSR<T>& A, const device_vector<T>& b, device_vector<T>& x,
            double rtol = 1e-10, int max_iters = 100000)
{
  const std::size_t n = (std::size_t)A.num_rows() * A.bs();
  if (b.size() != n || x.size() != n)
    throw Error(DFX_ERR_INVALID, "b and x must have num_rows * bs entries");
  const dfx_csr csr = A.csr();
  device_vector<double> dinv(n);
  check(dfx_jacobi_inverse_diagonal(&csr, dinv.data(), nullptr));
  const std::size_t wb = dfx_cg_workspace_bytes((std::int64_t)n);
  device_vector<double> work(wb / sizeof(double) + 1);
  dfx_cg_info info{};
  check(dfx_cg_solve(&csr, b.data(), x.data(), dinv.data(), rtol, max_iters, 0, work.data(), wb,
                     &info, nullptr));
  return {info.iterations, info.status, info.rnorm0_sq, info.rnorm_sq};
}

template <typename T>
CGResult cg(const MatrixCSR<T>& A, const Vector<T>& b, Vector<T>& x, double rtol = 1e-10,
            int max_iters = 100000)
{
  return cg(A, b.device(), x.device(), rtol, max_iters);
}

/// The solvers' sliced-ELL copy of a scalar MatrixCSR (rows sorted by
/// length in windows of sigma rows, 32-row column-major slices): FP64, or
/// FP32 with 16-bit column deltas. Owns the library's operator.
class SellOperator
{
public:
  SellOperator(const MatrixCSR<double>& A, bool fp32, int sigma = 256)
  {
    if (A.bs() != 1)
      throw Error(DFX_ERR_UNSUPPORTED, "the solver operator takes scalar (bs 1) matrices");
    const dfx_csr csr = A.csr();
    check(dfx_operator_create(&csr, sigma, fp32 ? DFX_F32 : DFX_F64, fp32 ? 1 : 0, &op_,
                              nullptr));
    n_ = A.num_rows();
  }
  ~SellOperator()
  {
    if (op_)
      dfx_operator_destroy(op_);
  }
  SellOperator(const SellOperator&) = delete;
  SellOperator& operator=(const SellOperator&) = delete;
  SellOperator(SellOperator&& o) noexcept : op_(std::exchange(o.op_, nullptr)), n_(o.n_) {}

  /// Refill the values from A (after re-assembly).
  void update_values(const MatrixCSR<double>& A)
  {
    const dfx_csr csr = A.csr();
    check(dfx_operator_update_values(op_, &csr, nullptr));
  }
  dfx_operator handle() const { return op_; }
  std::int32_t size() const { return n_; }

private:
  dfx_operator op_ = nullptr;
  std::int32_t n_ = 0;
};

struct IRResult
{
  int outer_iterations;
  int inner_iterations;
  int status;
  double rnorm0_sq, rnorm_sq;
};

/// Mixed precision: FP32 Jacobi-PCG on the FP32 operator with the residual
/// replaced by the FP64 residual b - A x each time it drops by inner_rtol
/// (reliable updates; x += d in FP64). Stops at the FP64 test |b - A x| <
/// rtol |b - A x0| of cg(). No reference counterpart; it wraps the demo's
/// CG (demo/poisson_matrix_free/main.cpp:84-132).
class IRSolver
{
public:
  explicit IRSolver(const MatrixCSR<double>& A, int sigma = 256, double inner_rtol = 0.03)
      : op64_(A, false, sigma), op32_(A, true, sigma), dinv_(A.num_rows()),
        inner_rtol_(inner_rtol)
  {
    wb_ = dfx_ir_workspace_bytes(A.num_rows());
    work_.resize(wb_ / sizeof(double) + 1);
    jacobi(A);
  }
  /// Re-read the values of A (after re-assembly).
  void refresh(const MatrixCSR<double>& A)
  {
    op64_.update_values(A);
    op32_.update_values(A);
    jacobi(A);
  }
  IRResult solve(const device_vector<double>& b, device_vector<double>& x, double rtol = 1e-10,
                 int max_outer = 200, int max_inner = 100000)
  {
    const std::size_t n = (std::size_t)op64_.size();
    if (b.size() != n || x.size() != n)
      throw Error(DFX_ERR_INVALID, "b and x must have num_rows entries");
    dfx_ir_info info{};
    check(dfx_ir_solve(op64_.handle(), op32_.handle(), b.data(), x.data(), dinv_.data(), rtol,
                       inner_rtol_, max_outer, max_inner, 0, DFX_IR_RELIABLE, work_.data(), wb_,
                       &info, nullptr));
    return {info.outer_iterations, info.inner_iterations, info.status, info.rnorm0_sq,
            info.rnorm_sq};
  }
  IRResult solve(const Vector<double>& b, Vector<double>& x, double rtol = 1e-10,
                 int max_outer = 200, int max_inner = 100000)
  {
    return solve(b.device(), x.device(), rtol, max_outer, max_inner);
  }

private:
  void jacobi(const MatrixCSR<double>& A)
  {
    const dfx_csr csr = A.csr();
    check(dfx_jacobi_inverse_diagonal(&csr, dinv_.data(), nullptr));
  }
  SellOperator op64_, op32_;
  device_vector<double> dinv_, work_;
  std::size_t wb_ = 0;
  double inner_rtol_;
};
} // namespace la
} // namespace dolfinx_gb300
