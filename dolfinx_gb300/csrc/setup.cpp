// Host-side one-time structure of the hot path: box mesh with RCM cell
// order, Lagrange dofmaps, CSR sparsity and cell colouring. These are the
// inputs the reference hands to its assemblers; the numbering reproduces
// DOLFINx on one rank bit for bit (checked against the oracle, whose
// mesh ordering is itself pinned to the reference's compiled
// graph/ordering.cpp and common/sort.h).
#include "dfx_gpu.h"
#include "timing.h"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <optional>
#include <thread>
#include <vector>

namespace dfx
{
int fail(int code, const char* fmt, ...);
}

namespace
{
// Basix reference tetrahedron sub-entities.
constexpr int kEdges[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
constexpr int kFacets[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

// Host threads of the set-up: DFX_NUM_THREADS when set (1-256), else the
// hardware concurrency (at most 64). Every result is independent of it.
int num_threads()
{
  if (const char* e = std::getenv("DFX_NUM_THREADS"))
  {
    const int v = std::atoi(e);
    if (v >= 1 && v <= 256)
      return v;
  }
  unsigned n = std::thread::hardware_concurrency();
  return n == 0 ? 1 : (int)std::min(n, 64u);
}

void atomic_min(int64_t& a, int64_t v)
{
  std::atomic_ref<int64_t> r(a);
  int64_t cur = r.load(std::memory_order_relaxed);
  while (v < cur && !r.compare_exchange_weak(cur, v, std::memory_order_relaxed))
  {
  }
}

template <typename F>
void parallel_for(int64_t n, F&& f)
{
  const int nt = (int)std::min<int64_t>(num_threads(), std::max<int64_t>(1, n / 4096));
  if (nt <= 1)
  {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
  {
    const int64_t a = n * t / nt, b = n * (t + 1) / nt;
    th.emplace_back([&f, a, b] { f(a, b); });
  }
  for (auto& t : th)
    t.join();
}

// Runs f(b) for every block b in [0, nb) on threads, consecutive blocks
// to a thread.
template <typename F>
void for_each_block(int64_t nb, F&& f)
{
  const int nt = (int)std::min<int64_t>(num_threads(), nb);
  if (nt <= 1)
  {
    for (int64_t b = 0; b < nb; ++b)
      f(b);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back(
        [&f, t, nt, nb]
        {
          for (int64_t b = nb * t / nt; b < nb * (t + 1) / nt; ++b)
            f(b);
        });
  for (auto& t : th)
    t.join();
}

// Stream compaction: emit(k, i) for the k-th index i in [0, n), in
// increasing order, that satisfies keep(i); returns the count. Fixed
// blocks are counted on threads, offset by a prefix sum and written on
// threads, so the output does not depend on the thread count.
template <typename Keep, typename Emit>
int64_t compact(int64_t n, const Keep& keep, const Emit& emit)
{
  constexpr int64_t kBlock = int64_t(1) << 16;
  const int64_t nb = (n + kBlock - 1) / kBlock;
  std::vector<int64_t> start(nb + 1, 0);
  for_each_block(nb,
                 [&](int64_t b)
                 {
                   int64_t c = 0;
                   for (int64_t i = b * kBlock, e = std::min(n, i + kBlock); i < e; ++i)
                     c += keep(i) ? 1 : 0;
                   start[b + 1] = c;
                 });
  for (int64_t b = 0; b < nb; ++b)
    start[b + 1] += start[b];
  for_each_block(nb,
                 [&](int64_t b)
                 {
                   int64_t k = start[b];
                   for (int64_t i = b * kBlock, e = std::min(n, i + kBlock); i < e; ++i)
                     if (keep(i))
                       emit(k++, i);
                 });
  return start[nb];
}

// Uninitialised array filled with `v` on threads.
template <typename T>
std::unique_ptr<T[]> filled(int64_t n, T v)
{
  std::unique_ptr<T[]> a(new T[std::max<int64_t>(n, 1)]);
  parallel_for(n, [&](int64_t i0, int64_t i1) { std::fill(a.get() + i0, a.get() + i1, v); });
  return a;
}

// Numbers ids 0..nid-1 by their first position in id[0..np): the first id
// seen gets 0, the next new one 1, and so on; ids that never appear get
// -1. Returns the count. On threads: first positions by atomic minimum,
// then a count of first positions before each one.
int64_t number_by_first_appearance(int64_t np, const int32_t* id, int64_t nid, int32_t* number)
{
  std::unique_ptr<int64_t[]> first = filled<int64_t>(nid, INT64_MAX);
  parallel_for(np, [&](int64_t a, int64_t b)
               {
                 for (int64_t p = a; p < b; ++p)
                   atomic_min(first[id[p]], p);
               });
  std::unique_ptr<int8_t[]> mark = filled<int8_t>(np, 0);
  parallel_for(nid, [&](int64_t a, int64_t b)
               {
                 for (int64_t v = a; v < b; ++v)
                 {
                   number[v] = -1;
                   if (first[v] != INT64_MAX)
                     mark[first[v]] = 1;
                 }
               });
  const int nt = (int)std::min<int64_t>(num_threads(), std::max<int64_t>(1, np / 4096));
  std::vector<int64_t> part(nt + 1, 0);
  auto chunks = [&](auto&& f)
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&f, t, np, nt] { f(t, np * t / nt, np * (t + 1) / nt); });
    for (auto& t : th)
      t.join();
  };
  chunks([&](int t, int64_t a, int64_t b)
         {
           int64_t c = 0;
           for (int64_t p = a; p < b; ++p)
             c += mark[p];
           part[t + 1] = c;
         });
  for (int t = 0; t < nt; ++t)
    part[t + 1] += part[t];
  chunks([&](int t, int64_t a, int64_t b)
         {
           int64_t c = part[t];
           for (int64_t p = a; p < b; ++p)
             if (mark[p])
               number[id[p]] = (int32_t)c++;
         });
  return part[nt];
}

// The facets of a tetrahedral mesh sorted by (key, facet index), the key
// being the sorted vertex triple (three 21-bit fields when every vertex
// index fits, else two words): equal facets are adjacent, in facet-index
// order. Built on threads: keys, then a bucket sort on the smallest vertex
// (buckets are increasing in the key, so sorting each bucket sorts all).
struct SortedFacets
{
  // (key hi, key lo | facet index), left uninitialised on allocation so
  // that the threads that fill it touch its pages first.
  struct Key
  {
    uint64_t first, second;
    bool operator<(const Key& o) const
    {
      return first < o.first || (first == o.first && second < o.second);
    }
  };
  std::unique_ptr<Key[]> key;
  int64_t n = 0;
  bool pack = true;
  bool same(int64_t a, int64_t b) const
  {
    if (pack)
      return key[a].first == key[b].first;
    return key[a].first == key[b].first && (key[a].second >> 32) == (key[b].second >> 32);
  }
  int64_t facet(int64_t p) const
  {
    return (int64_t)(pack ? key[p].second : (key[p].second & 0xffffffffu));
  }
};

// Facet index 4 c + f is stored in 32 bits of a sort key: callers reject
// meshes of 2^30 cells or more up front.
constexpr int64_t kMaxFacetCells = (int64_t)1 << 30;

template <typename I>
SortedFacets sort_facets(int64_t nc, const I* cells, int64_t nverts)
{
  using Key = SortedFacets::Key;
  const int64_t nf = 4 * nc;
  const bool pack = nverts <= (int64_t(1) << 21);
  std::unique_ptr<Key[]> keys(new Key[std::max<int64_t>(nf, 1)]);
  parallel_for(nc,
               [&](int64_t c0, int64_t c1)
               {
                 for (int64_t c = c0; c < c1; ++c)
                   for (int f = 0; f < 4; ++f)
                   {
                     uint64_t v[3];
                     for (int k = 0; k < 3; ++k)
                       v[k] = (uint64_t)cells[4 * c + kFacets[f][k]];
                     if (v[0] > v[1])
                       std::swap(v[0], v[1]);
                     if (v[1] > v[2])
                       std::swap(v[1], v[2]);
                     if (v[0] > v[1])
                       std::swap(v[0], v[1]);
                     const uint64_t idx = (uint64_t)(4 * c + f);
                     if (pack)
                       keys[4 * c + f] = {(v[0] << 42) | (v[1] << 21) | v[2], idx};
                     else
                       keys[4 * c + f] = {(v[0] << 32) | v[1], (v[2] << 32) | idx};
                   }
               });
  // (key, facet index) is a strict order, so any sort gives the stable-sort
  // permutation by key.
  const int shift = pack ? 42 : 32;
  const int64_t nv = std::max<int64_t>(nverts, 1);
  const int64_t nb = std::max<int64_t>(1, std::min<int64_t>(nf / 2048, nv));
  auto bucket = [&](const Key& k)
  { return (int64_t)((k.first >> shift) * (uint64_t)nb / (uint64_t)nv); };
  const int nt = (int)std::min<int64_t>(num_threads(), std::max<int64_t>(1, nf / 65536));
  std::vector<int64_t> cnt((size_t)nt * nb, 0), bstart(nb + 1, 0);
  auto team = [&](auto&& f)
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&f, t] { f(t); });
    for (auto& t : th)
      t.join();
  };
  team([&](int t)
       {
         int64_t* h = cnt.data() + (size_t)t * nb;
         for (int64_t i = nf * t / nt; i < nf * (t + 1) / nt; ++i)
           ++h[bucket(keys[i])];
       });
  // cnt[t][b] becomes thread t's first slot in bucket b.
  for (int64_t b = 0, s = 0; b < nb; ++b)
  {
    bstart[b] = s;
    for (int t = 0; t < nt; ++t)
    {
      const int64_t c = cnt[(size_t)t * nb + b];
      cnt[(size_t)t * nb + b] = s;
      s += c;
    }
  }
  bstart[nb] = nf;
  SortedFacets out;
  out.key.reset(new Key[std::max<int64_t>(nf, 1)]);
  out.n = nf;
  out.pack = pack;
  team([&](int t)
       {
         int64_t* h = cnt.data() + (size_t)t * nb;
         for (int64_t i = nf * t / nt; i < nf * (t + 1) / nt; ++i)
           out.key[h[bucket(keys[i])]++] = keys[i];
       });
  keys.reset();
  std::atomic<int64_t> next{0};
  team([&](int)
       {
         for (int64_t b; (b = next.fetch_add(64)) < nb;)
           for (int64_t e = std::min(b + 64, nb); b < e; ++b)
             std::sort(out.key.get() + bstart[b], out.key.get() + bstart[b + 1]);
       });
  return out;
}

// Facet-connected dual graph in the order of build_local_dual_graph
// (mesh/graphbuild.cpp:566-905, serial path). The reference sorts the facets
// by their sorted vertex triple (stably), turns each run of equal facets into
// the edges between its cells (pairs a < b in run order) and fills the
// adjacency in edge order. So a cell's neighbours are, for each of its facets
// in sorted order, the other cells of that facet's run in run order: each
// cell's list is filled from the runs on threads.
template <typename I>
void dual_graph(int64_t nc, const I* cells, int64_t nverts, std::vector<int32_t>& off,
                std::vector<int32_t>& adj)
{
  const int64_t nf = 4 * nc;
  std::optional<dfx::ScopedTimer> stage(std::in_place,
                                        "Compute local part of mesh dual graph: sort");
  const SortedFacets sf = sort_facets(nc, cells, nverts);
  stage.emplace("Compute local part of mesh dual graph: adjacency");
  auto cell_at = [&](int64_t p) { return (int32_t)(sf.facet(p) / 4); };
  // Sorted position of every facet; the run around a position.
  std::unique_ptr<int32_t[]> pos(new int32_t[std::max<int64_t>(nf, 1)]);
  parallel_for(nf,
               [&](int64_t a, int64_t b)
               {
                 for (int64_t p = a; p < b; ++p)
                   pos[sf.facet(p)] = (int32_t)p;
               });
  auto run = [&](int64_t p, int64_t& lo, int64_t& hi)
  {
    lo = p;
    while (lo > 0 && sf.same(lo - 1, p))
      --lo;
    hi = p + 1;
    while (hi < nf && sf.same(hi, p))
      ++hi;
  };
  off.assign(nc + 1, 0);
  parallel_for(nc,
               [&](int64_t a, int64_t b)
               {
                 for (int64_t c = a; c < b; ++c)
                 {
                   int64_t d = 0, lo, hi;
                   for (int f = 0; f < 4; ++f)
                   {
                     run(pos[4 * c + f], lo, hi);
                     d += hi - lo - 1;
                   }
                   off[c + 1] = (int32_t)d;
                 }
               });
  for (int64_t c = 0; c < nc; ++c)
    off[c + 1] += off[c];
  adj.resize(off[nc]);
  parallel_for(nc,
               [&](int64_t a, int64_t b)
               {
                 for (int64_t c = a; c < b; ++c)
                 {
                   int32_t q[4];
                   for (int f = 0; f < 4; ++f)
                     q[f] = pos[4 * c + f];
                   std::sort(q, q + 4);
                   int64_t w = off[c], lo, hi;
                   for (int f = 0; f < 4; ++f)
                   {
                     run(q[f], lo, hi);
                     for (int64_t p = lo; p < hi; ++p)
                       if (p != q[f])
                         adj[w++] = cell_at(p);
                   }
                 }
               });
}

// A reusable barrier for a team of host threads: arrivals count up, the
// last one starts the next generation; waiters spin briefly, then yield.
class SpinBarrier
{
public:
  explicit SpinBarrier(int n) : n_(n) {}
  void wait()
  {
    const int gen = gen_.load(std::memory_order_acquire);
    if (count_.fetch_add(1, std::memory_order_acq_rel) + 1 == n_)
    {
      count_.store(0, std::memory_order_relaxed);
      gen_.fetch_add(1, std::memory_order_release);
      return;
    }
    for (int spin = 0; gen_.load(std::memory_order_acquire) == gen; ++spin)
      if (spin > 256)
        std::this_thread::yield();
  }

private:
  const int n_;
  std::atomic<int> count_{0};
  std::atomic<int> gen_{0};
};

// Breadth-first search from s over the nodes whose mark is 0, in the order
// the serial queue gives: each level lists, for the nodes of the previous
// level in order, their unmarked neighbours in adjacency order, a node
// listed by the first that reaches it. With `sort_children`, each node's
// new neighbours are sorted by degree with std::ranges::sort before they
// are listed (the RCM queue of graph/ordering.cpp:148-170). `order`
// receives the nodes level by level, `lend` the end of each level (as the
// level structure of graph/ordering.cpp:22-57), and the nodes are marked.
//
// Large graphs run level by level on a team of threads, three barriers a
// level: a node's owner is the least (position in the level, position in
// the adjacency list) that reaches it (an atomic minimum); each thread
// collects its part of the level's children in order, sorted per parent;
// the parts are placed one after another. The owners and the inputs to
// each sort are those of the serial queue, so the order is the same.
int bfs(const std::vector<int32_t>& off, const std::vector<int32_t>& adj, int s,
        bool sort_children, std::vector<int8_t>& mark, std::vector<int64_t>& owner,
        std::vector<int>& order, std::vector<int>& lend)
{
  auto cmp = [&](int a, int b) { return off[a + 1] - off[a] < off[b + 1] - off[b]; };
  const int64_t n = (int64_t)off.size() - 1;
  const int nt = (int)std::min<int64_t>(num_threads(), std::max<int64_t>(1, n / 16384));
  lend.clear();
  if (nt <= 1)
  {
    order.clear();
    order.push_back(s);
    mark[s] = 1;
    size_t begin = 0;
    while (begin < order.size())
    {
      const size_t end = order.size();
      lend.push_back((int)end);
      for (size_t i = begin; i < end; ++i)
      {
        const size_t first = order.size();
        for (int k = off[order[i]]; k < off[order[i] + 1]; ++k)
          if (!mark[adj[k]])
          {
            mark[adj[k]] = 1;
            order.push_back(adj[k]);
          }
        if (sort_children)
          std::ranges::sort(order.begin() + first, order.end(), cmp);
      }
      begin = end;
    }
    return (int)lend.size();
  }
  order.resize(n);
  order[0] = s;
  mark[s] = 1;
  std::vector<int64_t> part(nt, 0);
  SpinBarrier sync(nt);
  auto key = [](int64_t i, int64_t j) { return (i << 32) | j; };
  int64_t end = 1;
  auto team = [&](int t)
  {
    std::vector<int> kids;
    for (int64_t fb = 0, fe = 1; fb < fe;)
    {
      const int64_t a = fb + (fe - fb) * t / nt, b = fb + (fe - fb) * (t + 1) / nt;
      // (1) claim: each unmarked neighbour keeps its least (i, j).
      for (int64_t i = a; i < b; ++i)
      {
        const int u = order[i];
        for (int j = off[u]; j < off[u + 1]; ++j)
          if (!mark[adj[j]])
            atomic_min(owner[adj[j]], key(i - fb, j - off[u]));
      }
      sync.wait();
      // (2) this thread's children, in order, sorted per parent.
      kids.clear();
      for (int64_t i = a; i < b; ++i)
      {
        const int u = order[i];
        const size_t first = kids.size();
        for (int j = off[u]; j < off[u + 1]; ++j)
          if (owner[adj[j]] == key(i - fb, j - off[u]))
            kids.push_back(adj[j]);
        if (sort_children)
          std::ranges::sort(kids.begin() + first, kids.end(), cmp);
      }
      part[t] = (int64_t)kids.size();
      sync.wait();
      // (3) place them after the level, mark them, clear their owners.
      int64_t w = fe, total = 0;
      for (int q = 0; q < nt; ++q)
      {
        w += q < t ? part[q] : 0;
        total += part[q];
      }
      for (int k : kids)
      {
        order[w++] = k;
        mark[k] = 1;
        owner[k] = INT64_MAX;
      }
      if (t == 0)
      {
        lend.push_back((int)fe);
        end = fe + total;
      }
      fb = fe;
      fe += total;
      sync.wait();
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t)
    th.emplace_back(team, t);
  team(0);
  for (auto& t : th)
    t.join();
  order.resize(end);
  return (int)lend.size();
}

// Reverse Cuthill-McKee with a George-Liu pseudo-peripheral root
// (graph/ordering.cpp:66-170). Ties in the degree sort follow
// std::ranges::sort exactly as the reference does. r[old] = new.
void rcm(const std::vector<int32_t>& off, const std::vector<int32_t>& adj,
         std::vector<int32_t>& r)
{
  const int n = (int)off.size() - 1;
  r.assign(n, -1);
  auto deg = [&](int a) { return off[a + 1] - off[a]; };
  auto cmp = [&](int a, int b) { return deg(a) < deg(b); };
  std::vector<int8_t> mark(n);
  std::vector<int64_t> owner(n, INT64_MAX);
  std::vector<int> ls, lend, ls2, lend2, rv, rvend;
  auto levels = [&](int s, std::vector<int>& order, std::vector<int>& ends)
  {
    dfx::ScopedTimer timer("Graph: create_level_structure");
    std::fill(mark.begin(), mark.end(), 0);
    return bfs(off, adj, s, false, mark, owner, order, ends);
  };
  int count = 0;
  while (count < n)
  {
    int v = 0, dmin = INT32_MAX;
    for (int i = 0; i < n; ++i)
      if (r[i] == -1 && deg(i) < dmin)
      {
        v = i;
        dmin = deg(i);
      }
    int nl = levels(v, ls, lend);
    for (;;)
    {
      const int b = nl > 1 ? lend[nl - 2] : 0;
      const int s = *std::ranges::min_element(
          std::ranges::subrange(ls.begin() + b, ls.begin() + lend[nl - 1]), cmp);
      const int nl2 = levels(s, ls2, lend2);
      if (nl2 > nl)
      {
        v = s;
        nl = nl2;
        ls.swap(ls2);
        lend.swap(lend2);
      }
      else
        break;
    }
    std::fill(mark.begin(), mark.end(), 0);
    bfs(off, adj, v, true, mark, owner, rv, rvend);
    for (auto it = rv.rbegin(); it != rv.rend(); ++it)
      r[*it] = count++;
  }
}

// Open-addressing map from 64-bit keys to int32 ids.
struct KeyMap
{
  std::vector<uint64_t> k;
  std::vector<int32_t> v;
  uint64_t mask;
  explicit KeyMap(int64_t n)
  {
    uint64_t cap = 16;
    while (cap < (uint64_t)(2 * n))
      cap <<= 1;
    k.assign(cap, ~uint64_t(0));
    v.assign(cap, -1);
    mask = cap - 1;
  }
  // Returns the id of `key`, inserting `next` if absent (flag set).
  int32_t get(uint64_t key, int32_t next, bool& inserted)
  {
    uint64_t h = (key * 0x9E3779B97F4A7C15ull) >> 17;
    for (;; ++h)
    {
      const uint64_t i = h & mask;
      if (k[i] == key)
      {
        inserted = false;
        return v[i];
      }
      if (k[i] == ~uint64_t(0))
      {
        k[i] = key;
        v[i] = next;
        inserted = true;
        return next;
      }
    }
  }
};

} // namespace

extern "C" int dfx_mesh_create_box_tet(int32_t nx, int32_t ny, int32_t nz, const double* p0,
                                       const double* p1, int32_t reorder, int32_t* cells_out,
                                       double* x_out)
{
  if (nx < 1 || ny < 1 || nz < 1)
    return dfx::fail(DFX_ERR_INVALID, "At least one cell is required.");
  for (int i = 0; i < 3; ++i)
    if (!(p0[i] < p1[i]))
      return dfx::fail(DFX_ERR_INVALID, "It must hold p[0] < p[1].");
  const int64_t sqxy = (int64_t)(nx + 1) * (ny + 1);
  const int64_t nv = sqxy * (nz + 1);
  const int64_t nhex = (int64_t)nx * ny * nz;
  const int64_t nc = 6 * nhex;
  if (nc > INT32_MAX / 4)
    return dfx::fail(DFX_ERR_INVALID, "mesh too large for int32 cell indices");
  dfx::ScopedTimer timer("Build BoxMesh (tetrahedra)");
  // Lexicographic vertices (generation.h:332-377) and the 6-tet split of
  // each hexahedron sharing the v0-v7 diagonal (generation.h:404-420).
  const double ext[3] = {(p1[0] - p0[0]) / nx, (p1[1] - p0[1]) / ny, (p1[2] - p0[2]) / nz};
  std::unique_ptr<int64_t[]> cells(new int64_t[4 * nc]);
  parallel_for(nhex, [&](int64_t i0, int64_t i1)
               {
                 for (int64_t i = i0; i < i1; ++i)
                 {
                   const int64_t iz = i / ((int64_t)nx * ny), j = i % ((int64_t)nx * ny);
                   const int64_t iy = j / nx, ix = j % nx;
                   const int64_t v0 = iz * sqxy + iy * (nx + 1) + ix, v1 = v0 + 1;
                   const int64_t v2 = v0 + (nx + 1), v3 = v1 + (nx + 1);
                   const int64_t v4 = v0 + sqxy, v5 = v1 + sqxy, v6 = v2 + sqxy,
                                 v7 = v3 + sqxy;
                   const int64_t t[24] = {v0, v1, v3, v7, v0, v1, v7, v5, v0, v5, v7, v4,
                                          v0, v3, v2, v7, v0, v6, v4, v7, v0, v2, v6, v7};
                   std::memcpy(&cells[24 * i], t, sizeof(t));
                 }
               });
  std::vector<int32_t> perm; // new -> old cell
  if (reorder)
  {
    std::vector<int32_t> off, adj, r;
    {
      dfx::ScopedTimer t("Compute local part of mesh dual graph");
      dual_graph(nc, cells.get(), nv, off, adj);
    }
    {
      dfx::ScopedTimer t("Reverse Cuthill-McKee ordering");
      rcm(off, adj, r);
    }
    perm.resize(nc);
    parallel_for(nc, [&](int64_t a, int64_t b)
                 {
                   for (int64_t c = a; c < b; ++c)
                     perm[r[c]] = (int32_t)c;
                 });
  }
  // Geometry nodes numbered by first appearance over the (reordered)
  // cells (fem/dofmapbuilder.cpp:440-474, no graph reordering): the
  // reordered cells' vertex ids go to cells_out, are numbered, and are
  // replaced by their numbers.
  parallel_for(nc, [&](int64_t a, int64_t b)
               {
                 for (int64_t c = a; c < b; ++c)
                 {
                   const int64_t co = reorder ? perm[c] : c;
                   for (int k = 0; k < 4; ++k)
                     cells_out[4 * c + k] = (int32_t)cells[4 * co + k];
                 }
               });
  cells.reset();
  std::unique_ptr<int32_t[]> node(new int32_t[nv]);
  number_by_first_appearance(4 * nc, cells_out, nv, node.get());
  parallel_for(4 * nc, [&](int64_t a, int64_t b)
               {
                 for (int64_t p = a; p < b; ++p)
                   cells_out[p] = node[cells_out[p]];
               });
  parallel_for(nv, [&](int64_t a, int64_t b)
               {
                 for (int64_t v = a; v < b; ++v)
                 {
                   const int64_t p = v % sqxy;
                   const int64_t idx[3] = {p % (nx + 1), p / (nx + 1), v / sqxy};
                   for (int i = 0; i < 3; ++i)
                     x_out[3 * (int64_t)node[v] + i] = p0[i] + (double)idx[i] * ext[i];
                 }
               });
  return DFX_OK;
}

extern "C" int dfx_mesh_dual_graph_tet(int32_t num_cells, const int32_t* cells,
                                       int32_t num_vertices, int32_t* offsets, int32_t* adj)
{
  if (num_cells < 0 || num_vertices < 0 || !offsets || (num_cells > 0 && (!cells || !adj)))
    return dfx::fail(DFX_ERR_INVALID, "invalid dual graph arguments");
  if ((int64_t)num_cells > INT32_MAX / 4)
    return dfx::fail(DFX_ERR_INVALID, "mesh too large for int32 facet indices");
  for (int64_t i = 0; i < 4 * (int64_t)num_cells; ++i)
    if (cells[i] < 0 || cells[i] >= num_vertices)
      return dfx::fail(DFX_ERR_INVALID, "cell %lld has a vertex index out of range",
                       (long long)(i / 4));
  dfx::ScopedTimer t("Compute local part of mesh dual graph");
  std::vector<int32_t> off, a;
  dual_graph(num_cells, cells, num_vertices, off, a);
  std::copy(off.begin(), off.end(), offsets);
  std::copy(a.begin(), a.end(), adj);
  return DFX_OK;
}

extern "C" int dfx_graph_reorder_rcm(int32_t n, const int32_t* offsets, const int32_t* adj,
                                     int32_t* perm)
{
  if (n < 0 || !offsets || (n > 0 && !perm) || offsets[0] != 0)
    return dfx::fail(DFX_ERR_INVALID, "invalid graph arguments");
  for (int32_t i = 0; i < n; ++i)
    if (offsets[i + 1] < offsets[i])
      return dfx::fail(DFX_ERR_INVALID, "offsets must not decrease (node %d)", i);
  if (offsets[n] > 0 && !adj)
    return dfx::fail(DFX_ERR_INVALID, "adjacency is NULL");
  for (int32_t k = 0; k < offsets[n]; ++k)
    if (adj[k] < 0 || adj[k] >= n)
      return dfx::fail(DFX_ERR_INVALID, "edge %d points outside the graph", k);
  dfx::ScopedTimer t("Reverse Cuthill-McKee ordering");
  std::vector<int32_t> off(offsets, offsets + n + 1), a(adj, adj + offsets[n]), r;
  rcm(off, a, r);
  std::copy(r.begin(), r.end(), perm);
  return DFX_OK;
}

namespace
{
// Concurrent open-addressing table from edge keys (sorted vertex pair) to
// the first position p = c*nd + local index at which the edge appears.
// Slots are claimed with compare-and-swap; the position is a running
// minimum, so the final table does not depend on the thread interleaving.
struct EdgeFirst
{
  static constexpr uint64_t kEmpty = ~uint64_t(0);
  struct Slot
  {
    uint64_t key;  // kEmpty when free
    int64_t first; // first position; later the edge's dof number
  };
  uint64_t cap, mask;
  std::unique_ptr<Slot[]> s; // key and position share a cache line
  explicit EdgeFirst(int64_t n)
  {
    cap = 16;
    while (cap < (uint64_t)(2 * n))
      cap <<= 1;
    mask = cap - 1;
    s = filled<Slot>((int64_t)cap, Slot{kEmpty, INT64_MAX});
  }
  uint64_t slot(uint64_t k)
  {
    for (uint64_t h = (k * 0x9E3779B97F4A7C15ull) >> 17;; ++h)
    {
      const uint64_t i = h & mask;
      std::atomic_ref<uint64_t> r(s[i].key);
      uint64_t cur = r.load(std::memory_order_acquire);
      if (cur == k)
        return i;
      if (cur == kEmpty)
      {
        if (r.compare_exchange_strong(cur, k, std::memory_order_acq_rel))
          return i;
        if (cur == k)
          return i;
      }
    }
  }
};
} // namespace

extern "C" int dfx_dofmap_create_tet(int32_t num_cells, const int32_t* cells, int32_t degree,
                                     int32_t* dofmap, int32_t* num_nodes)
{
  if (degree != 1 && degree != 2)
    return dfx::fail(DFX_ERR_UNSUPPORTED, "Lagrange degree %d not supported", degree);
  const int64_t nc = num_cells;
  const int nd = degree == 1 ? 4 : 10;
  int32_t vmax = -1;
  for (int64_t i = 0; i < 4 * nc; ++i)
  {
    if (cells[i] < 0)
      return dfx::fail(DFX_ERR_INVALID, "negative vertex index in cell %lld", (long long)(i / 4));
    vmax = std::max(vmax, cells[i]);
  }
  dfx::ScopedTimer timer("Dofmap builder: build dofmap data");
  std::optional<dfx::ScopedTimer> reorder(std::in_place,
                                          "Dofmap builder: compute dof reordering map");
  // Vertex dofs are keyed by vertex, edge dofs by their sorted vertex pair.
  // The reference numbers them by first appearance over the cell dofmap
  // (fem/dofmapbuilder.cpp:445-474). Here: (1) each entity's first position
  // p = c*nd + i (atomic minimum, order-independent), (2) those positions
  // marked, (3) the entity's number is the count of marks before its first
  // position, (4) every position takes its entity's number.
  const int64_t np = nd * nc;
  std::unique_ptr<int64_t[]> vfirst = filled<int64_t>(vmax + 1, INT64_MAX);
  EdgeFirst edges(degree == 2 ? 7 * nc / 5 + 16 : 1);
  auto edge_key = [&](int64_t c, int e)
  {
    uint64_t a = (uint32_t)cells[4 * c + kEdges[e][0]], b = (uint32_t)cells[4 * c + kEdges[e][1]];
    if (a > b)
      std::swap(a, b);
    return (a << 32) | b;
  };
  parallel_for(nc, [&](int64_t c0, int64_t c1)
               {
                 for (int64_t c = c0; c < c1; ++c)
                 {
                   for (int i = 0; i < 4; ++i)
                     atomic_min(vfirst[cells[4 * c + i]], nd * c + i);
                   if (degree == 2)
                     for (int e = 0; e < 6; ++e)
                     {
                       // the edge's slot waits in its dofmap entry until (4)
                       const uint64_t k = edges.slot(edge_key(c, e));
                       dofmap[nd * c + 4 + e] = (int32_t)k;
                       atomic_min(edges.s[k].first, nd * c + 4 + e);
                     }
                 }
               });
  // (2) marks at first positions, (3) exclusive prefix counts in place.
  std::unique_ptr<int32_t[]> number = filled<int32_t>(np, 0);
  parallel_for(vmax + 1, [&](int64_t a, int64_t b)
               {
                 for (int64_t v = a; v < b; ++v)
                   if (vfirst[v] != INT64_MAX)
                     number[vfirst[v]] = 1;
               });
  if (degree == 2)
    parallel_for((int64_t)edges.cap, [&](int64_t a, int64_t b)
                 {
                   for (int64_t i = a; i < b; ++i)
                     if (edges.s[i].key != EdgeFirst::kEmpty)
                       number[edges.s[i].first] = 1;
                 });
  const int nt = num_threads();
  std::vector<int64_t> part(nt + 1, 0);
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t]
                      {
                        int64_t s = 0;
                        for (int64_t p = np * t / nt; p < np * (t + 1) / nt; ++p)
                          s += number[p];
                        part[t + 1] = s;
                      });
    for (auto& t : th)
      t.join();
  }
  for (int t = 0; t < nt; ++t)
    part[t + 1] += part[t];
  if (part[nt] > INT32_MAX)
    return dfx::fail(DFX_ERR_UNSUPPORTED, "more than 2^31 dof nodes");
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t]
                      {
                        int64_t s = part[t];
                        for (int64_t p = np * t / nt; p < np * (t + 1) / nt; ++p)
                        {
                          const int32_t m = number[p];
                          number[p] = (int32_t)s;
                          s += m;
                        }
                      });
    for (auto& t : th)
      t.join();
  }
  reorder.reset();
  // (4) each entity takes the number of its first position, then every
  // position takes its entity's number.
  parallel_for(vmax + 1, [&](int64_t a, int64_t b)
               {
                 for (int64_t v = a; v < b; ++v)
                   if (vfirst[v] != INT64_MAX)
                     vfirst[v] = number[vfirst[v]];
               });
  if (degree == 2)
    parallel_for((int64_t)edges.cap, [&](int64_t a, int64_t b)
                 {
                   for (int64_t i = a; i < b; ++i)
                     if (edges.s[i].key != EdgeFirst::kEmpty)
                       edges.s[i].first = number[edges.s[i].first];
                 });
  number.reset();
  parallel_for(nc, [&](int64_t c0, int64_t c1)
               {
                 for (int64_t c = c0; c < c1; ++c)
                 {
                   for (int i = 0; i < 4; ++i)
                     dofmap[nd * c + i] = (int32_t)vfirst[cells[4 * c + i]];
                   if (degree == 2)
                     for (int e = 0; e < 6; ++e)
                       dofmap[nd * c + 4 + e] =
                           (int32_t)edges.s[(uint32_t)dofmap[nd * c + 4 + e]].first;
                 }
               });
  *num_nodes = (int32_t)part[nt];
  return DFX_OK;
}

extern "C" int dfx_sparsity_create(int32_t nrows, int32_t num_cells, int32_t nd,
                                   const int32_t* dofmap, int64_t* row_ptr, int32_t* cols,
                                   int64_t* nnz_out)
{
  if (nrows < 0 || num_cells < 0 || nd <= 0 || !row_ptr)
    return dfx::fail(DFX_ERR_INVALID, "invalid sparsity arguments");
  dfx::ScopedTimer timer("Build sparsity");
  // Transpose dofmap: node -> cells.
  std::vector<int32_t> coff(nrows + 1, 0);
  for (int64_t i = 0; i < (int64_t)num_cells * nd; ++i)
  {
    if (dofmap[i] < 0 || dofmap[i] >= nrows)
      return dfx::fail(DFX_ERR_INVALID, "dofmap entry %d out of range", dofmap[i]);
    ++coff[dofmap[i] + 1];
  }
  for (int r = 0; r < nrows; ++r)
    coff[r + 1] += coff[r];
  std::vector<int32_t> ccell(coff[nrows]);
  {
    std::vector<int32_t> pos(coff.begin(), coff.end() - 1);
    for (int64_t c = 0; c < num_cells; ++c)
      for (int i = 0; i < nd; ++i)
        ccell[pos[dofmap[c * nd + i]]++] = (int32_t)c;
  }
  auto row_cols = [&](int32_t r, std::vector<int32_t>& buf)
  {
    buf.clear();
    for (int k = coff[r]; k < coff[r + 1]; ++k)
    {
      const int32_t* d = dofmap + (int64_t)ccell[k] * nd;
      buf.insert(buf.end(), d, d + nd);
    }
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
  if (!cols)
  {
    std::vector<int64_t> len(nrows);
    parallel_for(nrows,
                 [&](int64_t a, int64_t b)
                 {
                   std::vector<int32_t> buf;
                   for (int64_t r = a; r < b; ++r)
                   {
                     row_cols((int32_t)r, buf);
                     len[r] = (int64_t)buf.size();
                   }
                 });
    row_ptr[0] = 0;
    for (int r = 0; r < nrows; ++r)
      row_ptr[r + 1] = row_ptr[r] + len[r];
    if (nnz_out)
      *nnz_out = row_ptr[nrows];
    return DFX_OK;
  }
  parallel_for(nrows,
               [&](int64_t a, int64_t b)
               {
                 std::vector<int32_t> buf;
                 for (int64_t r = a; r < b; ++r)
                 {
                   row_cols((int32_t)r, buf);
                   std::copy(buf.begin(), buf.end(), cols + row_ptr[r]);
                 }
               });
  if (nnz_out)
    *nnz_out = row_ptr[nrows];
  return DFX_OK;
}

extern "C" int dfx_tabulate_dof_coordinates_tet(int32_t num_cells, const int32_t* cells,
                                                int32_t num_vertices, const double* x,
                                                const int32_t* dofmap, int32_t degree,
                                                int32_t num_nodes, double* X)
{
  if (degree != 1 && degree != 2)
    return dfx::fail(DFX_ERR_UNSUPPORTED, "Lagrange degree %d not supported", degree);
  if (num_cells < 0 || num_vertices < 0 || num_nodes < 0 ||
      (num_cells > 0 && (!cells || !x || !dofmap || !X)))
    return dfx::fail(DFX_ERR_INVALID, "invalid dof coordinate arguments");
  const int nd = degree == 1 ? 4 : 10;
  const int64_t nc = num_cells;
  // Index checks first, so that nothing is written for a bad mesh.
  std::atomic<int64_t> bad{-1};
  parallel_for(nc, [&](int64_t a, int64_t b)
               {
                 for (int64_t c = a; c < b; ++c)
                 {
                   bool ok = true;
                   for (int i = 0; i < 4; ++i)
                     ok &= cells[4 * c + i] >= 0 && cells[4 * c + i] < num_vertices;
                   for (int i = 0; i < nd; ++i)
                     ok &= dofmap[nd * c + i] >= 0 && dofmap[nd * c + i] < num_nodes;
                   if (!ok)
                   {
                     int64_t e = -1;
                     bad.compare_exchange_strong(e, c);
                     return;
                   }
                 }
               });
  if (bad.load() >= 0)
    return dfx::fail(DFX_ERR_INVALID, "cell %lld has a vertex or dof index out of range",
                     (long long)bad.load());
  // Each cell writes its nodes: the vertices, then the edge midpoints in
  // Basix edge order (the P2 interpolation points pushed forward by the
  // affine map). A node shared by several cells gets the same value from
  // each, so the stores are relaxed atomics (no ordering is needed).
  parallel_for(nc, [&](int64_t a, int64_t b)
               {
                 for (int64_t c = a; c < b; ++c)
                 {
                   double v[4][3];
                   for (int i = 0; i < 4; ++i)
                     for (int k = 0; k < 3; ++k)
                       v[i][k] = x[3 * (int64_t)cells[4 * c + i] + k];
                   for (int i = 0; i < 4; ++i)
                     for (int k = 0; k < 3; ++k)
                       std::atomic_ref<double>(X[3 * (int64_t)dofmap[nd * c + i] + k])
                           .store(v[i][k], std::memory_order_relaxed);
                   if (degree == 2)
                     for (int e = 0; e < 6; ++e)
                       for (int k = 0; k < 3; ++k)
                       {
                         const double m = 0.5 * (v[kEdges[e][0]][k] + v[kEdges[e][1]][k]);
                         std::atomic_ref<double>(X[3 * (int64_t)dofmap[nd * c + 4 + e] + k])
                             .store(m, std::memory_order_relaxed);
                       }
                 }
               });
  return DFX_OK;
}

extern "C" int dfx_colour_cells(int32_t num_cells, int32_t nd, const int32_t* dofmap,
                                int32_t num_nodes, int32_t* order, int32_t* offsets,
                                int32_t max_colours, int32_t* num_colours)
{
  // Greedy first-fit in cell order; per-node bitmasks of used colours.
  constexpr int W = 4; // 256 colours max
  if (max_colours < 1)
    return dfx::fail(DFX_ERR_INVALID, "max_colours must be >= 1");
  std::vector<uint64_t> used((size_t)num_nodes * W, 0);
  std::vector<int32_t> colour(num_cells);
  int ncol = 0;
  for (int64_t c = 0; c < num_cells; ++c)
  {
    uint64_t m[W] = {0, 0, 0, 0};
    const int32_t* d = dofmap + c * nd;
    for (int i = 0; i < nd; ++i)
      for (int w = 0; w < W; ++w)
        m[w] |= used[(size_t)d[i] * W + w];
    int col = -1;
    for (int w = 0; w < W && col < 0; ++w)
      if (~m[w])
        col = 64 * w + __builtin_ctzll(~m[w]);
    if (col < 0 || col >= max_colours)
      return dfx::fail(DFX_ERR_UNSUPPORTED, "cell colouring needs more than %d colours",
                       std::min(max_colours, 64 * W));
    colour[c] = col;
    ncol = std::max(ncol, col + 1);
    for (int i = 0; i < nd; ++i)
      used[(size_t)d[i] * W + col / 64] |= uint64_t(1) << (col % 64);
  }
  std::fill(offsets, offsets + ncol + 1, 0);
  for (int64_t c = 0; c < num_cells; ++c)
    ++offsets[colour[c] + 1];
  for (int k = 0; k < ncol; ++k)
    offsets[k + 1] += offsets[k];
  std::vector<int32_t> pos(offsets, offsets + ncol);
  for (int64_t c = 0; c < num_cells; ++c)
    order[pos[colour[c]]++] = (int32_t)c;
  *num_colours = ncol;
  return DFX_OK;
}

namespace
{
// Largest vertex index of `nc` tetrahedra, or an error for a negative one.
int tet_vertex_max(int32_t nc, const int32_t* cells, int64_t* vmax)
{
  *vmax = 0;
  for (int64_t i = 0; i < 4 * (int64_t)nc; ++i)
  {
    if (cells[i] < 0)
      return dfx::fail(DFX_ERR_INVALID, "negative vertex index in cell %lld", (long long)(i / 4));
    *vmax = std::max<int64_t>(*vmax, cells[i]);
  }
  return DFX_OK;
}
} // namespace

extern "C" int dfx_exterior_facets_tet(int32_t num_cells, const int32_t* cells, int32_t* facets,
                                       int32_t* num_facets)
{
  if (num_cells < 0 || !num_facets || (num_cells > 0 && (!cells || !facets)))
    return dfx::fail(DFX_ERR_INVALID, "invalid exterior facet arguments");
  if (num_cells >= kMaxFacetCells)
    return dfx::fail(DFX_ERR_INVALID, "%d cells: facet indices need num_cells < 2^30", num_cells);
  const int64_t nf = 4 * (int64_t)num_cells;
  // Facets keyed by their sorted vertex triple (three 21-bit fields when
  // every vertex index fits, else two words); a facet seen once is
  // exterior (mesh/utils.cpp:61-89).
  int64_t vmax = 0;
  if (const int rc = tet_vertex_max(num_cells, cells, &vmax); rc != DFX_OK)
    return rc;
  const SortedFacets sf = sort_facets(num_cells, cells, vmax + 1);
  std::unique_ptr<uint8_t[]> exterior = filled<uint8_t>(nf, 0);
  parallel_for(nf, [&](int64_t a, int64_t b)
               {
                 for (int64_t p = a; p < b; ++p)
                   if (!(p > 0 && sf.same(p - 1, p)) && !(p + 1 < nf && sf.same(p, p + 1)))
                     exterior[sf.facet(p)] = 1;
               });
  const int64_t n = compact(
      nf, [&](int64_t i) { return exterior[i] != 0; },
      [&](int64_t k, int64_t i)
      {
        facets[2 * k] = (int32_t)(i / 4);
        facets[2 * k + 1] = (int32_t)(i % 4);
      });
  if (n > INT32_MAX)
    return dfx::fail(DFX_ERR_INVALID, "%lld exterior facets overflow the int32 count",
                     (long long)n);
  *num_facets = (int32_t)n;
  return DFX_OK;
}

extern "C" int dfx_interior_facets_tet(int32_t num_cells, const int32_t* cells, int32_t* facets,
                                       int32_t* num_facets)
{
  if (num_cells < 0 || !num_facets || (num_cells > 0 && (!cells || !facets)))
    return dfx::fail(DFX_ERR_INVALID, "invalid interior facet arguments");
  if (num_cells >= kMaxFacetCells)
    return dfx::fail(DFX_ERR_INVALID, "%d cells: facet indices need num_cells < 2^30", num_cells);
  const int64_t nf = 4 * (int64_t)num_cells;
  // A facet is interior when exactly two (cell, local facet) entries share
  // its vertex triple (fem/utils.cpp:223-254: facets with two attached
  // cells). The sort puts the two next to each other, the smaller
  // (cell, local facet) first; that one records its partner.
  int64_t vmax = 0;
  if (const int rc = tet_vertex_max(num_cells, cells, &vmax); rc != DFX_OK)
    return rc;
  const SortedFacets sf = sort_facets(num_cells, cells, vmax + 1);
  std::unique_ptr<int64_t[]> partner = filled<int64_t>(nf, -1);
  parallel_for(nf, [&](int64_t a, int64_t b)
               {
                 for (int64_t p = a; p < b; ++p)
                   if (p + 1 < nf && sf.same(p, p + 1) && !(p > 0 && sf.same(p - 1, p))
                       && !(p + 2 < nf && sf.same(p + 1, p + 2)))
                   {
                     const int64_t i = sf.facet(p), j = sf.facet(p + 1);
                     partner[std::min(i, j)] = std::max(i, j);
                   }
               });
  const int64_t n = compact(
      nf, [&](int64_t i) { return partner[i] >= 0; },
      [&](int64_t k, int64_t i)
      {
        const int64_t j = partner[i];
        int32_t* q = facets + 4 * k;
        q[0] = (int32_t)(i / 4);
        q[1] = (int32_t)(i % 4);
        q[2] = (int32_t)(j / 4);
        q[3] = (int32_t)(j % 4);
      });
  if (n > INT32_MAX)
    return dfx::fail(DFX_ERR_INVALID, "%lld interior facets overflow the int32 count",
                     (long long)n);
  *num_facets = (int32_t)n;
  return DFX_OK;
}
