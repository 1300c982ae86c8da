// The process-wide table of named timings (task -> repetitions, total
// seconds) behind dfx::ScopedTimer and the dfx_timing_* entry points. Tasks
// are kept in byte-wise name order, the order of the reference's
// dolfinx::timings() map (common/timing.h:42-46).
#include "dfx_gpu.h"
#include "timing.h"

#include <algorithm>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <string>
#include <string_view>
#include <utility>

namespace dfx
{
int fail(int code, const char* fmt, ...);
}

namespace
{
std::mutex g_mu;
std::map<std::string, std::pair<int32_t, double>, std::less<>> g_timings;
} // namespace

namespace dfx
{
void record_timing(const char* task, double seconds)
{
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_timings.find(std::string_view(task));
  if (it == g_timings.end())
    g_timings.emplace(task, std::make_pair(1, seconds));
  else
  {
    it->second.first += 1;
    it->second.second += seconds;
  }
}
} // namespace dfx

extern "C" int dfx_timing_record(const char* task, double seconds)
{
  if (!task)
    return dfx::fail(DFX_ERR_INVALID, "task name is NULL");
  dfx::record_timing(task, seconds);
  return DFX_OK;
}

extern "C" int dfx_timing(const char* task, int32_t* count, double* total_seconds)
{
  if (!task || !count || !total_seconds)
    return dfx::fail(DFX_ERR_INVALID, "invalid timing arguments");
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_timings.find(std::string_view(task));
  if (it == g_timings.end())
    return dfx::fail(DFX_ERR_INVALID, "No timings registered for task \"%s\".", task);
  *count = it->second.first;
  *total_seconds = it->second.second;
  return DFX_OK;
}

extern "C" int dfx_timing_num_tasks(int32_t* num)
{
  if (!num)
    return dfx::fail(DFX_ERR_INVALID, "num is NULL");
  std::lock_guard<std::mutex> lk(g_mu);
  *num = (int32_t)g_timings.size();
  return DFX_OK;
}

extern "C" int dfx_timing_task(int32_t i, char* name, int32_t name_cap, int32_t* name_len,
                               int32_t* count, double* total_seconds)
{
  if (!name_len || !count || !total_seconds || name_cap < 0 || (name_cap > 0 && !name))
    return dfx::fail(DFX_ERR_INVALID, "invalid timing arguments");
  std::lock_guard<std::mutex> lk(g_mu);
  if (i < 0 || i >= (int32_t)g_timings.size())
    return dfx::fail(DFX_ERR_INVALID, "task index %d out of range (%d tasks)", i,
                     (int)g_timings.size());
  auto it = g_timings.begin();
  std::advance(it, i);
  const std::string& s = it->first;
  *name_len = (int32_t)s.size();
  if (name_cap > 0)
  {
    const size_t n = std::min(s.size(), (size_t)name_cap - 1);
    std::memcpy(name, s.data(), n);
    name[n] = '\0';
  }
  *count = it->second.first;
  *total_seconds = it->second.second;
  return DFX_OK;
}

extern "C" int dfx_timing_clear(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  g_timings.clear();
  return DFX_OK;
}
