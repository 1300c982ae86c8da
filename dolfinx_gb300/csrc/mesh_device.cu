// Device-side mesh set-up: the facet dual graph of a tetrahedral mesh
// (mesh::build_local_dual_graph, mesh/graphbuild.cpp:566-905), the reverse
// Cuthill-McKee ordering of a graph (graph::reorder_rcm,
// graph/ordering.cpp:22-170) and the RCM-ordered tetrahedral box
// (mesh::create_box, mesh/generation.h:332-426) built on the GPU. Each one
// computes the same definition as the host builder in setup.cpp, so the
// results are identical bit for bit:
//
//   dual graph: a cell's neighbours are, for each of its facets in the order
//     of the facets' sorted vertex triples, the cell across that facet. The
//     facets are grouped by their smallest vertex (count, scan, fill) and
//     each facet finds its twin in its group, so no global sort is needed.
//     A facet shared by more than two cells is reported as UNSUPPORTED.
//   RCM: level-synchronous breadth-first search. A node reached in a level
//     belongs to the least (position of the parent in the level, position in
//     the parent's adjacency) that reaches it (64-bit atomic minimum); each
//     parent lists its children in adjacency order, sorted by degree with a
//     stable insertion sort (libstdc++'s std::sort on at most 16 elements);
//     a scan of the child counts places them after the level. Roots and the
//     George-Liu pseudo-peripheral search are those of the host builder.
//     Graphs with a node of degree above 16 are reported as UNSUPPORTED.
//   box: the six-tetrahedron split of each hexahedron, RCM on its dual
//     graph, then geometry nodes numbered by first appearance over the
//     reordered cells and the coordinates p0 + i * (p1 - p0) / n evaluated
//     without contraction into a fused multiply-add.
#include "scan.cuh"

#include <algorithm>
#include <vector>

namespace
{
constexpr int kThreads = 256;
constexpr int kMaxChildren = 16;
__constant__ int kFacetVerts[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

struct Carver
{
  char* base;
  size_t off = 0;
  template <typename T>
  T* take(int64_t n)
  {
    T* r = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += a256(sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    return r;
  }
};

unsigned grid_for(int64_t m)
{
  const int64_t need = (m + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)dfx::num_sms() * 32));
}

int read_word(const void* d, void* h, size_t bytes, cudaStream_t s)
{
  DFX_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s));
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}

// ---------------------------------------------------------------------------
// Dual graph

struct DualWork
{
  int64_t* vptr;     // nv + 1: facets per smallest vertex, then offsets
  unsigned* vpos;    // nv: fill cursors
  int32_t* vlist;    // 4 nc: facet indices grouped by smallest vertex
  int32_t* twin;     // 4 nc: facet across, or -1
  int64_t* deg;      // nc + 1: neighbours per cell, then offsets
  int64_t* scratch;  // scan scratch
  size_t bytes;
};

DualWork carve_dual(void* base, int64_t nc, int64_t nv)
{
  Carver c{(char*)base};
  DualWork w{};
  w.vptr = c.take<int64_t>(nv + 1);
  w.vpos = c.take<unsigned>(nv);
  w.vlist = c.take<int32_t>(4 * nc);
  w.twin = c.take<int32_t>(4 * nc);
  w.deg = c.take<int64_t>(nc + 1);
  w.scratch = c.take<int64_t>(dfx::scan_scratch_count(std::max(nv, nc) + 1));
  w.bytes = c.off;
  return w;
}

__device__ __forceinline__ void facet_triple(const int32_t* __restrict__ cells, int64_t t,
                                             int32_t v[3])
{
  const int64_t c = t >> 2;
  const int f = (int)(t & 3);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    v[k] = __ldg(cells + 4 * c + kFacetVerts[f][k]);
  int32_t a;
  if (v[0] > v[1])
    a = v[0], v[0] = v[1], v[1] = a;
  if (v[1] > v[2])
    a = v[1], v[1] = v[2], v[2] = a;
  if (v[0] > v[1])
    a = v[0], v[0] = v[1], v[1] = a;
}

__device__ __forceinline__ bool triple_less(const int32_t* a, const int32_t* b)
{
  return a[0] < b[0] || (a[0] == b[0] && (a[1] < b[1] || (a[1] == b[1] && a[2] < b[2])));
}

__global__ void k_dual_count(const int32_t* __restrict__ cells, int64_t nf, int64_t nv,
                             DualWork w, int* status)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    int32_t v[3];
    facet_triple(cells, t, v);
    if (v[0] < 0 || v[2] >= nv)
    {
      atomicExch(status, (int)DFX_ERR_INVALID);
      continue;
    }
    atomicAdd(reinterpret_cast<unsigned long long*>(w.vptr) + v[0], 1ull);
  }
}

__global__ void k_dual_fill(const int32_t* __restrict__ cells, int64_t nf, DualWork w)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    int32_t v[3];
    facet_triple(cells, t, v);
    const unsigned p = atomicAdd(w.vpos + v[0], 1u);
    w.vlist[w.vptr[v[0]] + p] = (int32_t)t;
  }
}

// Twin of every facet; the neighbour count of every cell (4 facets of a
// cell are handled by one thread each, the counts added atomically).
__global__ void k_dual_twin(const int32_t* __restrict__ cells, int64_t nf, DualWork w,
                            int* status)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nf;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    int32_t v[3];
    facet_triple(cells, t, v);
    int32_t tw = -1;
    int m = 0;
    for (int64_t k = w.vptr[v[0]], e = w.vptr[v[0] + 1]; k < e; ++k)
    {
      const int32_t g = w.vlist[k];
      if (g == t)
        continue;
      int32_t u[3];
      facet_triple(cells, g, u);
      if (u[1] == v[1] && u[2] == v[2])
      {
        tw = g;
        ++m;
      }
    }
    if (m > 1)
      atomicExch(status, (int)DFX_ERR_UNSUPPORTED);
    w.twin[t] = tw;
    if (tw >= 0)
      atomicAdd(reinterpret_cast<unsigned long long*>(w.deg) + (t >> 2), 1ull);
  }
}

__global__ void k_dual_adj(const int32_t* __restrict__ cells, int64_t nc, DualWork w,
                           int32_t* __restrict__ offsets, int32_t* __restrict__ adj)
{
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x)
  {
    int32_t key[4][3];
    int ord[4] = {0, 1, 2, 3};
#pragma unroll
    for (int f = 0; f < 4; ++f)
      facet_triple(cells, 4 * c + f, key[f]);
    // Insertion sort of the four facets by vertex triple.
    for (int i = 1; i < 4; ++i)
    {
      const int x = ord[i];
      int j = i;
      while (j > 0 && triple_less(key[x], key[ord[j - 1]]))
      {
        ord[j] = ord[j - 1];
        --j;
      }
      ord[j] = x;
    }
    int64_t p = w.deg[c];
    offsets[c] = (int32_t)p;
    for (int i = 0; i < 4; ++i)
    {
      const int32_t tw = w.twin[4 * c + ord[i]];
      if (tw >= 0)
        adj[p++] = tw >> 2;
    }
    if (c == nc - 1)
      offsets[nc] = (int32_t)p;
  }
}

int dual_graph(int64_t nc, const int32_t* d_cells, int64_t nv, int32_t* d_off, int32_t* d_adj,
               const DualWork& w, int* status, cudaStream_t s)
{
  const int64_t nf = 4 * nc;
  DFX_CUDA(cudaMemsetAsync(w.vptr, 0, sizeof(int64_t) * (size_t)(nv + 1), s));
  DFX_CUDA(cudaMemsetAsync(w.vpos, 0, sizeof(unsigned) * (size_t)std::max<int64_t>(nv, 1), s));
  DFX_CUDA(cudaMemsetAsync(w.deg, 0, sizeof(int64_t) * (size_t)(nc + 1), s));
  k_dual_count<<<grid_for(nf), kThreads, 0, s>>>(d_cells, nf, nv, w, status);
  DFX_CHECK_LAUNCH();
  int h = 0;
  if (int st = read_word(status, &h, sizeof(int), s))
    return st;
  if (h)
    return dfx::fail(DFX_ERR_INVALID, "cell vertex index out of range [0, %lld)", (long long)nv);
  if (int st = dfx::exclusive_scan(w.vptr, w.vptr, nv, w.scratch, s))
    return st;
  k_dual_fill<<<grid_for(nf), kThreads, 0, s>>>(d_cells, nf, w);
  DFX_CHECK_LAUNCH();
  k_dual_twin<<<grid_for(nf), kThreads, 0, s>>>(d_cells, nf, w, status);
  DFX_CHECK_LAUNCH();
  if (int st = dfx::exclusive_scan(w.deg, w.deg, nc, w.scratch, s))
    return st;
  k_dual_adj<<<grid_for(nc), kThreads, 0, s>>>(d_cells, nc, w, d_off, d_adj);
  DFX_CHECK_LAUNCH();
  if (int st = read_word(status, &h, sizeof(int), s))
    return st;
  if (h)
    return dfx::fail(DFX_ERR_UNSUPPORTED,
                     "a facet is shared by more than two cells: use the host builder");
  return DFX_OK;
}

// ---------------------------------------------------------------------------
// Reverse Cuthill-McKee

struct RcmWork
{
  int32_t* order[2];          // n each: two level structures (George-Liu)
  int32_t* mark;              // n: stamp of the search that reached the node
  unsigned long long* owner;  // n: least (level position, adjacency position)
  int64_t* cnt;               // n + 1: children per parent, then offsets
  int64_t* scratch;           // scan scratch
  unsigned long long* red;    // reduction word
  size_t bytes;
};

RcmWork carve_rcm(void* base, int64_t n)
{
  Carver c{(char*)base};
  RcmWork w{};
  w.order[0] = c.take<int32_t>(n);
  w.order[1] = c.take<int32_t>(n);
  w.mark = c.take<int32_t>(n);
  w.owner = c.take<unsigned long long>(n);
  w.cnt = c.take<int64_t>(n + 1);
  w.scratch = c.take<int64_t>(dfx::scan_scratch_count(n + 1));
  w.red = c.take<unsigned long long>(1);
  w.bytes = c.off;
  return w;
}

constexpr unsigned long long kNoOwner = ~0ull;

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u < v ? u : v;
  }
  return v;
}

// Checks the graph (offsets non-decreasing from 0 to off[n], edges in
// range, degree at most kMaxChildren), resets the marks, owners and the
// permutation. Adjacency entries are read only below off[n], which the
// caller guarantees the adjacency holds.
__global__ void k_rcm_init(const int32_t* __restrict__ off, const int32_t* __restrict__ adj,
                           int64_t n, RcmWork w, int32_t* __restrict__ r, int* status)
{
  const int32_t total = off[n];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    w.mark[i] = 0;
    w.owner[i] = kNoOwner;
    r[i] = -1;
    const int32_t a = off[i], b = off[i + 1];
    if ((i == 0 && a != 0) || a < 0 || b < a || b > total)
    {
      atomicExch(status, (int)DFX_ERR_INVALID);
      continue;
    }
    if (b - a > kMaxChildren)
      atomicCAS(status, 0, (int)DFX_ERR_UNSUPPORTED);
    for (int32_t j = a; j < b; ++j)
      if (adj[j] < 0 || adj[j] >= n)
        atomicExch(status, (int)DFX_ERR_INVALID);
  }
}

// The first node of least degree among those not yet numbered.
__global__ void k_rcm_root(const int32_t* __restrict__ off, int64_t n,
                           const int32_t* __restrict__ r, unsigned long long* red)
{
  unsigned long long best = kNoOwner;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (r[i] == -1)
    {
      const unsigned long long k =
          ((unsigned long long)(off[i + 1] - off[i]) << 32) | (unsigned long long)i;
      best = k < best ? k : best;
    }
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0 && best != kNoOwner)
    atomicMin(red, best);
}

// The first node of least degree among order[0, m): (degree, position).
__global__ void k_rcm_level_min(const int32_t* __restrict__ off,
                                const int32_t* __restrict__ order, int64_t m,
                                unsigned long long* red)
{
  unsigned long long best = kNoOwner;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t u = order[i];
    const unsigned long long k =
        ((unsigned long long)(off[u + 1] - off[u]) << 32) | (unsigned long long)i;
    best = k < best ? k : best;
  }
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0 && best != kNoOwner)
    atomicMin(red, best);
}

__global__ void k_bfs_start(int32_t* order, int32_t* mark, int32_t s, int32_t stamp)
{
  order[0] = s;
  mark[s] = stamp;
}

__device__ __forceinline__ unsigned long long claim_key(int64_t i, int32_t j)
{
  return ((unsigned long long)i << 32) | (unsigned)j;
}

// (1) Every unvisited neighbour of the level keeps its least claim.
__global__ void k_bfs_claim(const int32_t* __restrict__ off, const int32_t* __restrict__ adj,
                            const int32_t* __restrict__ level, int64_t m,
                            const int32_t* __restrict__ mark, int32_t stamp,
                            unsigned long long* __restrict__ owner)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t u = level[i], a = off[u], b = off[u + 1];
    for (int32_t j = a; j < b; ++j)
    {
      const int32_t v = adj[j];
      if (mark[v] != stamp)
        atomicMin(owner + v, claim_key(i, j - a));
    }
  }
}

// (2) Children per parent.
__global__ void k_bfs_count(const int32_t* __restrict__ off, const int32_t* __restrict__ adj,
                            const int32_t* __restrict__ level, int64_t m,
                            const unsigned long long* __restrict__ owner,
                            int64_t* __restrict__ cnt)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t u = level[i], a = off[u], b = off[u + 1];
    int64_t k = 0;
    for (int32_t j = a; j < b; ++j)
      k += owner[adj[j]] == claim_key(i, j - a);
    cnt[i] = k;
  }
}

// (3) Each parent's children, in adjacency order (sorted stably by degree
// for the RCM queue), after the level at the scanned offsets; they are
// marked and their claims cleared.
template <bool SORT>
__global__ void k_bfs_place(const int32_t* __restrict__ off, const int32_t* __restrict__ adj,
                            const int32_t* __restrict__ level, int64_t m,
                            unsigned long long* __restrict__ owner,
                            const int64_t* __restrict__ pos, int32_t* __restrict__ next,
                            int32_t* __restrict__ mark, int32_t stamp)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t u = level[i], a = off[u], b = off[u + 1];
    int32_t kid[kMaxChildren], kdeg[kMaxChildren];
    int k = 0;
    for (int32_t j = a; j < b && k < kMaxChildren; ++j)
    {
      const int32_t v = adj[j];
      if (owner[v] == claim_key(i, j - a))
      {
        kid[k] = v;
        kdeg[k] = off[v + 1] - off[v];
        ++k;
      }
    }
    if (SORT)
      for (int x = 1; x < k; ++x)
      {
        const int32_t vk = kid[x], vd = kdeg[x];
        int y = x;
        while (y > 0 && vd < kdeg[y - 1])
        {
          kid[y] = kid[y - 1];
          kdeg[y] = kdeg[y - 1];
          --y;
        }
        kid[y] = vk;
        kdeg[y] = vd;
      }
    const int64_t p = pos[i];
    for (int x = 0; x < k; ++x)
    {
      next[p + x] = kid[x];
      mark[kid[x]] = stamp;
      owner[kid[x]] = kNoOwner;
    }
  }
}

__global__ void k_rcm_number(const int32_t* __restrict__ order, int64_t len, int64_t first,
                             int32_t* __restrict__ r)
{
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < len;
       k += (int64_t)gridDim.x * blockDim.x)
    r[order[k]] = (int32_t)(first + len - 1 - k);
}

class Rcm
{
public:
  Rcm(const int32_t* off, const int32_t* adj, int64_t n, const RcmWork& w, cudaStream_t s)
      : off_(off), adj_(adj), n_(n), w_(w), s_(s)
  {
  }

  // Breadth-first search from `root` into order[which]; the level ends in
  // `lend`. Returns DFX_OK or an error code.
  int bfs(int32_t root, bool sort, int which, std::vector<int64_t>& lend)
  {
    int32_t* ord = w_.order[which];
    ++stamp_;
    lend.clear();
    k_bfs_start<<<1, 1, 0, s_>>>(ord, w_.mark, root, stamp_);
    DFX_CHECK_LAUNCH();
    int64_t fb = 0, fe = 1;
    while (fb < fe)
    {
      lend.push_back(fe);
      const int64_t m = fe - fb;
      const unsigned g = grid_for(m);
      k_bfs_claim<<<g, kThreads, 0, s_>>>(off_, adj_, ord + fb, m, w_.mark, stamp_, w_.owner);
      k_bfs_count<<<g, kThreads, 0, s_>>>(off_, adj_, ord + fb, m, w_.owner, w_.cnt);
      DFX_CHECK_LAUNCH();
      if (int st = dfx::exclusive_scan(w_.cnt, w_.cnt, m, w_.scratch, s_))
        return st;
      if (sort)
        k_bfs_place<true><<<g, kThreads, 0, s_>>>(off_, adj_, ord + fb, m, w_.owner, w_.cnt,
                                                   ord + fe, w_.mark, stamp_);
      else
        k_bfs_place<false><<<g, kThreads, 0, s_>>>(off_, adj_, ord + fb, m, w_.owner, w_.cnt,
                                                    ord + fe, w_.mark, stamp_);
      DFX_CHECK_LAUNCH();
      int64_t total = 0;
      if (int st = read_word(w_.cnt + m, &total, sizeof(int64_t), s_))
        return st;
      if (total < 0 || fe + total > n_)
        return dfx::fail(DFX_ERR_INVALID, "breadth-first search overran the graph");
      fb = fe;
      fe += total;
    }
    return DFX_OK;
  }

  int min_word(unsigned long long* out)
  {
    return read_word(w_.red, out, sizeof(*out), s_);
  }

  int run(int32_t* r)
  {
    std::vector<int64_t> lend[2], rvend;
    int64_t count = 0;
    while (count < n_)
    {
      DFX_CUDA(cudaMemsetAsync(w_.red, 0xff, sizeof(unsigned long long), s_));
      k_rcm_root<<<grid_for(n_), kThreads, 0, s_>>>(off_, n_, r, w_.red);
      DFX_CHECK_LAUNCH();
      unsigned long long key = 0;
      if (int st = min_word(&key))
        return st;
      if (key == kNoOwner)
        return dfx::fail(DFX_ERR_INVALID, "no unnumbered node left");
      int32_t v = (int32_t)(key & 0xffffffffu);
      int cur = 0;
      if (int st = bfs(v, false, cur, lend[cur]))
        return st;
      for (;;)
      {
        const std::vector<int64_t>& le = lend[cur];
        const size_t nl = le.size();
        const int64_t b = nl > 1 ? le[nl - 2] : 0, e = le[nl - 1];
        DFX_CUDA(cudaMemsetAsync(w_.red, 0xff, sizeof(unsigned long long), s_));
        k_rcm_level_min<<<grid_for(e - b), kThreads, 0, s_>>>(off_, w_.order[cur] + b, e - b,
                                                              w_.red);
        DFX_CHECK_LAUNCH();
        if (int st = min_word(&key))
          return st;
        int32_t sn = 0;
        if (int st = read_word(w_.order[cur] + b + (int64_t)(key & 0xffffffffu), &sn,
                               sizeof(int32_t), s_))
          return st;
        const int alt = 1 - cur;
        if (int st = bfs(sn, false, alt, lend[alt]))
          return st;
        if (lend[alt].size() > nl)
        {
          v = sn;
          cur = alt;
        }
        else
          break;
      }
      // The final queue goes into the buffer not holding the chosen levels.
      const int q = 1 - cur;
      if (int st = bfs(v, true, q, rvend))
        return st;
      // The last level ends at the number of nodes reached.
      const int64_t len = rvend.back();
      k_rcm_number<<<grid_for(len), kThreads, 0, s_>>>(w_.order[q], len, count, r);
      DFX_CHECK_LAUNCH();
      count += len;
    }
    return DFX_OK;
  }

private:
  const int32_t* off_;
  const int32_t* adj_;
  int64_t n_;
  RcmWork w_;
  cudaStream_t s_;
  int32_t stamp_ = 0;
};

int rcm(const int32_t* d_off, const int32_t* d_adj, int64_t n, int32_t* d_r, const RcmWork& w,
        int* status, cudaStream_t s)
{
  if (n == 0)
    return DFX_OK;
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  k_rcm_init<<<grid_for(n), kThreads, 0, s>>>(d_off, d_adj, n, w, d_r, status);
  DFX_CHECK_LAUNCH();
  int h = 0;
  if (int st = read_word(status, &h, sizeof(int), s))
    return st;
  if (h == DFX_ERR_INVALID)
    return dfx::fail(DFX_ERR_INVALID,
                     "invalid graph: offsets must rise from 0 and edges lie in [0, %lld)",
                     (long long)n);
  if (h)
    return dfx::fail(DFX_ERR_UNSUPPORTED,
                     "a node has more than %d neighbours: use the host ordering", kMaxChildren);
  Rcm run(d_off, d_adj, n, w, s);
  return run.run(d_r);
}

// ---------------------------------------------------------------------------
// Box mesh

struct BoxWork
{
  int32_t* cells0;             // 4 nc: the box's cells, lexicographic vertices
  int32_t* cellsp;             // 4 nc: the reordered cells
  int32_t* off;                // nc + 1: dual graph
  int32_t* adj;                // 4 nc
  int32_t* r;                  // nc: r[old] = new
  unsigned long long* vfirst;  // nv: first position of each vertex
  int64_t* mark;               // 4 nc + 1: marks, then node numbers
  int64_t* scratch;
  DualWork dual;
  RcmWork rcm;
  size_t bytes;
};

BoxWork carve_box(void* base, int64_t nc, int64_t nv, bool reorder)
{
  Carver c{(char*)base};
  BoxWork w{};
  w.cells0 = c.take<int32_t>(4 * nc);
  w.cellsp = c.take<int32_t>(4 * nc);
  w.vfirst = c.take<unsigned long long>(nv);
  w.mark = c.take<int64_t>(4 * nc + 1);
  w.scratch = c.take<int64_t>(dfx::scan_scratch_count(4 * nc + 1));
  if (reorder)
  {
    w.off = c.take<int32_t>(nc + 1);
    w.adj = c.take<int32_t>(4 * nc);
    w.r = c.take<int32_t>(nc);
    // The dual graph's and the ordering's work areas are not live at once.
    const size_t at = c.off;
    const DualWork d = carve_dual(c.base ? c.base + at : nullptr, nc, nv);
    const RcmWork q = carve_rcm(c.base ? c.base + at : nullptr, nc);
    w.dual = d;
    w.rcm = q;
    c.off += std::max(d.bytes, q.bytes);
  }
  w.bytes = c.off;
  return w;
}

// Six tetrahedra per hexahedron, sharing its v0-v7 diagonal.
__global__ void k_box_cells(int32_t nx, int32_t ny, int64_t nhex, int32_t* __restrict__ cells)
{
  const int64_t sqxy = (int64_t)(nx + 1) * (ny + 1);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nhex;
       i += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t iz = i / ((int64_t)nx * ny), j = i % ((int64_t)nx * ny);
    const int64_t iy = j / nx, ix = j % nx;
    const int32_t v0 = (int32_t)(iz * sqxy + iy * (nx + 1) + ix), v1 = v0 + 1;
    const int32_t v2 = v0 + (nx + 1), v3 = v1 + (nx + 1);
    const int32_t v4 = v0 + (int32_t)sqxy, v5 = v1 + (int32_t)sqxy, v6 = v2 + (int32_t)sqxy,
                  v7 = v3 + (int32_t)sqxy;
    int4* out = reinterpret_cast<int4*>(cells) + 6 * i;
    out[0] = make_int4(v0, v1, v3, v7);
    out[1] = make_int4(v0, v1, v7, v5);
    out[2] = make_int4(v0, v5, v7, v4);
    out[3] = make_int4(v0, v3, v2, v7);
    out[4] = make_int4(v0, v6, v4, v7);
    out[5] = make_int4(v0, v2, v6, v7);
  }
}

__global__ void k_box_gather(const int32_t* __restrict__ r, int64_t nc,
                             const int32_t* __restrict__ cells0, int32_t* __restrict__ cellsp,
                             int* status)
{
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x)
  {
    const int32_t to = r[c];
    if (to < 0 || to >= nc)
    {
      atomicExch(status, (int)DFX_ERR_INVALID);
      continue;
    }
    reinterpret_cast<int4*>(cellsp)[to] = reinterpret_cast<const int4*>(cells0)[c];
  }
}

__global__ void k_box_first(const int32_t* __restrict__ cells, int64_t np,
                            unsigned long long* __restrict__ vfirst)
{
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x)
    atomicMin(vfirst + cells[p], (unsigned long long)p);
}

__global__ void k_box_mark(const unsigned long long* __restrict__ vfirst, int64_t nv,
                           int64_t* __restrict__ mark)
{
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x)
    if (vfirst[v] != ~0ull)
      mark[vfirst[v]] = 1;
}

__global__ void k_box_number(const int32_t* __restrict__ cellsp, int64_t np,
                             const unsigned long long* __restrict__ vfirst,
                             const int64_t* __restrict__ mark, int32_t* __restrict__ cells)
{
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x)
    cells[p] = (int32_t)mark[vfirst[cellsp[p]]];
}

struct BoxGeom
{
  double p0[3], ext[3];
};

__global__ void k_box_coords(int32_t nx, int64_t sqxy, int64_t nv, BoxGeom g,
                             const unsigned long long* __restrict__ vfirst,
                             const int64_t* __restrict__ mark, double* __restrict__ x)
{
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t p = v % sqxy;
    const int64_t idx[3] = {p % (nx + 1), p / (nx + 1), v / sqxy};
    if (vfirst[v] == ~0ull)
      continue;
    const int64_t node = mark[vfirst[v]];
#pragma unroll
    for (int i = 0; i < 3; ++i)
      x[3 * node + i] = __dadd_rn(g.p0[i], __dmul_rn((double)idx[i], g.ext[i]));
  }
}
} // namespace

extern "C" size_t dfx_mesh_dual_graph_tet_device_workspace_bytes(int32_t num_cells,
                                                                 int32_t num_vertices)
{
  if (num_cells < 0 || num_vertices < 0)
    return 0;
  return carve_dual(nullptr, num_cells, num_vertices).bytes;
}

extern "C" int dfx_mesh_dual_graph_tet_device(int32_t num_cells, const int32_t* d_cells,
                                              int32_t num_vertices, int32_t* d_offsets,
                                              int32_t* d_adj, void* d_work, size_t work_bytes,
                                              void* stream)
{
  DFX_REQUIRE(num_cells >= 0 && num_vertices >= 0 && d_offsets, "invalid dual graph arguments");
  DFX_REQUIRE(num_cells == 0 || (d_cells && d_adj), "cells and adjacency must be non-NULL");
  DFX_REQUIRE((int64_t)num_cells <= INT32_MAX / 4, "mesh too large for int32 facet indices");
  const DualWork need = carve_dual(nullptr, num_cells, num_vertices);
  DFX_REQUIRE(d_work && work_bytes >= need.bytes, "workspace too small (%zu < %zu bytes)",
              work_bytes, need.bytes);
  DFX_REQUIRE(((uintptr_t)d_work & 255) == 0, "workspace must be 256-byte aligned");
  cudaStream_t s = dfx::as_stream(stream);
  if (num_cells == 0)
  {
    DFX_CUDA(cudaMemsetAsync(d_offsets, 0, sizeof(int32_t), s));
    DFX_CUDA(cudaStreamSynchronize(s));
    return DFX_OK;
  }
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  const DualWork w = carve_dual(d_work, num_cells, num_vertices);
  return dual_graph(num_cells, d_cells, num_vertices, d_offsets, d_adj, w, status, s);
}

extern "C" size_t dfx_graph_reorder_rcm_device_workspace_bytes(int32_t n)
{
  if (n < 0)
    return 0;
  return carve_rcm(nullptr, n).bytes;
}

extern "C" int dfx_graph_reorder_rcm_device(int32_t n, const int32_t* d_offsets,
                                            const int32_t* d_adj, int32_t* d_perm, void* d_work,
                                            size_t work_bytes, void* stream)
{
  DFX_REQUIRE(n >= 0 && d_offsets && (n == 0 || d_perm), "invalid graph arguments");
  const RcmWork need = carve_rcm(nullptr, n);
  DFX_REQUIRE(d_work && work_bytes >= need.bytes, "workspace too small (%zu < %zu bytes)",
              work_bytes, need.bytes);
  DFX_REQUIRE(((uintptr_t)d_work & 255) == 0, "workspace must be 256-byte aligned");
  cudaStream_t s = dfx::as_stream(stream);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  const RcmWork w = carve_rcm(d_work, n);
  if (int st = rcm(d_offsets, d_adj, n, d_perm, w, status, s))
    return st;
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}

extern "C" size_t dfx_mesh_create_box_tet_device_workspace_bytes(int32_t nx, int32_t ny,
                                                                 int32_t nz, int32_t reorder)
{
  if (nx < 1 || ny < 1 || nz < 1)
    return 0;
  const int64_t nc = 6 * (int64_t)nx * ny * nz;
  const int64_t nv = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
  if (nc > INT32_MAX / 4)
    return 0;
  return carve_box(nullptr, nc, nv, reorder != 0).bytes;
}

extern "C" int dfx_mesh_create_box_tet_device(int32_t nx, int32_t ny, int32_t nz,
                                              const double* p0, const double* p1,
                                              int32_t reorder, int32_t* d_cells, double* d_x,
                                              void* d_work, size_t work_bytes, void* stream)
{
  DFX_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1, "At least one cell is required.");
  DFX_REQUIRE(p0 && p1 && d_cells && d_x, "points, cells and x must be non-NULL");
  for (int i = 0; i < 3; ++i)
    DFX_REQUIRE(p0[i] < p1[i], "It must hold p[0] < p[1].");
  const int64_t sqxy = (int64_t)(nx + 1) * (ny + 1);
  const int64_t nv = sqxy * (nz + 1);
  const int64_t nhex = (int64_t)nx * ny * nz;
  const int64_t nc = 6 * nhex;
  DFX_REQUIRE(nc <= INT32_MAX / 4, "mesh too large for int32 cell indices");
  DFX_REQUIRE(((uintptr_t)d_cells & 15) == 0, "cells must be 16-byte aligned");
  const BoxWork need = carve_box(nullptr, nc, nv, reorder != 0);
  DFX_REQUIRE(d_work && work_bytes >= need.bytes, "workspace too small (%zu < %zu bytes)",
              work_bytes, need.bytes);
  DFX_REQUIRE(((uintptr_t)d_work & 255) == 0, "workspace must be 256-byte aligned");
  cudaStream_t s = dfx::as_stream(stream);
  int* status = dfx::device_status_page();
  DFX_REQUIRE(status, "could not allocate the status page");
  DFX_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
  const BoxWork w = carve_box(d_work, nc, nv, reorder != 0);
  k_box_cells<<<grid_for(nhex), kThreads, 0, s>>>(nx, ny, nhex, w.cells0);
  DFX_CHECK_LAUNCH();
  const int32_t* cells = w.cells0;
  if (reorder)
  {
    if (int st = dual_graph(nc, w.cells0, nv, w.off, w.adj, w.dual, status, s))
      return st;
    if (int st = rcm(w.off, w.adj, nc, w.r, w.rcm, status, s))
      return st;
    k_box_gather<<<grid_for(nc), kThreads, 0, s>>>(w.r, nc, w.cells0, w.cellsp, status);
    DFX_CHECK_LAUNCH();
    int h = 0;
    if (int st = read_word(status, &h, sizeof(int), s))
      return st;
    if (h)
      return dfx::fail(DFX_ERR_INVALID, "cell ordering is not a permutation");
    cells = w.cellsp;
  }
  // Geometry nodes by first appearance over the (reordered) cells.
  const int64_t np = 4 * nc;
  DFX_CUDA(cudaMemsetAsync(w.vfirst, 0xff, sizeof(unsigned long long) * (size_t)nv, s));
  DFX_CUDA(cudaMemsetAsync(w.mark, 0, sizeof(int64_t) * (size_t)(np + 1), s));
  k_box_first<<<grid_for(np), kThreads, 0, s>>>(cells, np, w.vfirst);
  k_box_mark<<<grid_for(nv), kThreads, 0, s>>>(w.vfirst, nv, w.mark);
  DFX_CHECK_LAUNCH();
  if (int st = dfx::exclusive_scan(w.mark, w.mark, np, w.scratch, s))
    return st;
  k_box_number<<<grid_for(np), kThreads, 0, s>>>(cells, np, w.vfirst, w.mark, d_cells);
  BoxGeom g{};
  const int32_t n3[3] = {nx, ny, nz};
  for (int i = 0; i < 3; ++i)
  {
    g.p0[i] = p0[i];
    g.ext[i] = (p1[i] - p0[i]) / n3[i];
  }
  k_box_coords<<<grid_for(nv), kThreads, 0, s>>>(nx, sqxy, nv, g, w.vfirst, w.mark, d_x);
  DFX_CHECK_LAUNCH();
  DFX_CUDA(cudaStreamSynchronize(s));
  return DFX_OK;
}
