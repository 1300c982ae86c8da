// The autotuner's table: launch parameters chosen by timing the candidates
// (dfx_tune_assembly, dfx_tune_spmv) or pinned by the caller, per device
// and workload key. Kernels launched for a workload without an entry use
// their built-in defaults.
#include "common.cuh"

#include <map>
#include <mutex>
#include <tuple>

namespace
{
std::mutex g_mu;
std::map<std::tuple<int, int, int64_t, int64_t, int64_t>, int> g_table;

int current_device()
{
  int d = 0;
  cudaGetDevice(&d);
  return d;
}
} // namespace

namespace dfx
{
int tuned_get(int what, int64_t k0, int64_t k1, int64_t k2)
{
  const auto key = std::make_tuple(current_device(), what, k0, k1, k2);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(key);
  return it == g_table.end() ? 0 : it->second;
}

void tuned_set(int what, int64_t k0, int64_t k1, int64_t k2, int value)
{
  const auto key = std::make_tuple(current_device(), what, k0, k1, k2);
  std::lock_guard<std::mutex> lk(g_mu);
  if (value)
    g_table[key] = value;
  else
    g_table.erase(key);
}
} // namespace dfx

extern "C" int dfx_tune_clear(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  g_table.clear();
  return DFX_OK;
}
