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

extern "C" int dfx_tune_export(int64_t* rows, int64_t cap, int64_t* num)
{
  if (!num || cap < 0)
    return dfx::fail(DFX_ERR_INVALID, "invalid export arguments");
  std::lock_guard<std::mutex> lk(g_mu);
  const int64_t n = (int64_t)g_table.size();
  *num = n;
  if (!rows)
    return DFX_OK;
  if (cap < n)
    return dfx::fail(DFX_ERR_NO_MEMORY, "%lld rows needed, room for %lld", (long long)n,
                     (long long)cap);
  int64_t* r = rows;
  for (const auto& [key, value] : g_table)
  {
    r[0] = std::get<0>(key);
    r[1] = std::get<1>(key);
    r[2] = std::get<2>(key);
    r[3] = std::get<3>(key);
    r[4] = std::get<4>(key);
    r[5] = value;
    r += 6;
  }
  return DFX_OK;
}

namespace
{
// A value the kernels accept for this kind of choice. Assembly keys hold
// the form kind in k1 / 16 (16 kind + 4 degree + 2 mass + mode, as the
// assembly records them).
bool valid_choice(int64_t what, int64_t k1, int64_t value)
{
  if (what == dfx::kTuneAssembly)
  {
    if (k1 < 0)
      return false;
    if (k1 / 16 == DFX_FORM_ELASTICITY)
      return value == 2 || value == 4 || value == 8;
    return value == 16 || value == 32 || value == 64;
  }
  if (what == dfx::kTuneSpmv)
    return value == 4 || value == 8 || value == 16 || value == 32;
  return false;
}
} // namespace

extern "C" int dfx_tune_import(const int64_t* rows, int64_t num)
{
  if (num < 0 || (num > 0 && !rows))
    return dfx::fail(DFX_ERR_INVALID, "invalid import arguments");
  for (int64_t i = 0; i < num; ++i)
  {
    const int64_t* r = rows + 6 * i;
    if (r[0] < 0 || r[0] > INT32_MAX || !valid_choice(r[1], r[3], r[5]))
      return dfx::fail(DFX_ERR_INVALID,
                       "tuning row %lld (device %lld, what %lld, value %lld) is not a valid "
                       "choice",
                       (long long)i, (long long)r[0], (long long)r[1], (long long)r[5]);
  }
  std::lock_guard<std::mutex> lk(g_mu);
  for (int64_t i = 0; i < num; ++i)
  {
    const int64_t* r = rows + 6 * i;
    g_table[std::make_tuple((int)r[0], (int)r[1], r[2], r[3], r[4])] = (int)r[5];
  }
  return DFX_OK;
}
