// C entry point over the reference's own sparsity-pattern code
// (la/SparsityPattern.cpp, common/IndexMap.cpp and what they include),
// compiled from its sources on one rank with the stand-in headers of
// oracle/ref_shim_la/. TEST INFRASTRUCTURE ONLY: built into oracle/_ref/
// by oracle/Makefile when the reference tree is present, used to write the
// golden sparsity patterns under tests/golden/ and to check the timing
// summary table against the reference's own TimeLogger and Table.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <dolfinx/common/IndexMap.h>
#include <dolfinx/common/Table.h>
#include <dolfinx/common/TimeLogger.h>
#include <dolfinx/la/SparsityPattern.h>
#include <memory>
#include <span>
#include <string>

extern "C"
{
// The cell sparsity pattern of a dofmap as fem::create_sparsity_pattern
// builds it on one rank: sparsitybuild::cells inserts each cell's dofs
// against themselves (fem/sparsitybuild.h:36-49), then
// SparsityPattern::finalize (la/SparsityPattern.cpp:264-491) and graph().
// Writes row_ptr (nrows+1) and, when cols != NULL, the columns; returns
// the entry count.
int64_t ref_sparsity(int32_t nrows, int32_t nc, int32_t nd, const int32_t* dofmap,
                     int64_t* row_ptr, int32_t* cols)
{
  auto map = std::make_shared<const dolfinx::common::IndexMap>(MPI_COMM_WORLD, nrows);
  dolfinx::la::SparsityPattern sp(MPI_COMM_WORLD, {map, map}, {1, 1});
  for (int32_t c = 0; c < nc; ++c)
  {
    std::span<const std::int32_t> d(dofmap + (int64_t)c * nd, nd);
    sp.insert(d, d);
  }
  sp.finalize();
  auto [edges, offsets] = sp.graph();
  for (int32_t r = 0; r <= nrows; ++r)
    row_ptr[r] = offsets[r];
  if (cols)
    for (std::size_t k = 0; k < edges.size(); ++k)
      cols[k] = edges[k];
  return (int64_t)edges.size();
}

// One more repetition of `seconds` for `task` in the reference's
// TimeLogger (common/TimeLogger.cpp:27-40).
void ref_timing_record(const char* task, double seconds)
{
  dolfinx::common::TimeLogger::instance().register_timing(
      task, std::chrono::duration<double>(seconds));
}

// The table list_timings prints (common/TimeLogger.cpp:42-53) on one rank,
// reduction 0/1/2 = average/max/min, without the surrounding newlines.
// Writes at most cap bytes including a NUL; returns the full length.
int64_t ref_timing_table(int reduction, char* buf, int64_t cap)
{
  const dolfinx::Table t = dolfinx::common::TimeLogger::instance().timing_table().reduce(
      MPI_COMM_WORLD, static_cast<dolfinx::Table::Reduction>(reduction));
  const std::string s = t.str();
  if (cap > 0)
  {
    const std::size_t n = std::min<std::size_t>(s.size(), cap - 1);
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return (int64_t)s.size();
}
}
