// Sparsity pattern, scatter map and tetrahedron colouring (host, once per mesh).
//
// The pattern is the set of (gi, gj) pairs over the six edges of every
// tetrahedron -- the triplets src/assemble_maxwell.cpp:191-204 hands to
// setFromTriplets -- plus every diagonal (Dirichlet rows are given a 1 there,
// :344-347) plus the dense port blocks of w w^H ports (:212-231), which the
// reference inserts with coeffRef.  Rows are edges, columns sorted.
//
// slot[36 t + 6 i + j] is the position in the value array of the entry
// (edge_i(t), edge_j(t)).  Tetrahedra are coloured greedily so that no two
// tetrahedra of one colour share an edge; the GPU assembly scatters one
// colour per launch with plain read-modify-writes and no atomics.
#include <algorithm>
#include <stdexcept>
#include <thread>

#include "pattern.hpp"

namespace edgefem {

namespace {

// Runs f(begin, end) over [0, n) split into contiguous ranges, one per host
// thread (at most 16; one for small n).  Each range writes disjoint outputs,
// so the result does not depend on the thread count.
template <class F>
void parallel_ranges(std::size_t n, F &&f) {
  std::size_t nt = std::min<std::size_t>(16, std::max(1u, std::thread::hardware_concurrency()));
  if (n < 65536) nt = 1;
  if (nt <= 1) {
    f(std::size_t{0}, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (std::size_t k = 0; k < nt; ++k) th.emplace_back([&, k] { f(n * k / nt, n * (k + 1) / nt); });
  for (auto &t : th) t.join();
}

}  // namespace

int Pattern::slot_of(int r, int c) const {
  const int *b = colidx.data() + rowptr[r];
  const int *e = colidx.data() + rowptr[r + 1];
  const int *p = std::lower_bound(b, e, c);
  if (p == e || *p != c) return -1;
  return static_cast<int>(p - colidx.data());
}

Pattern build_pattern(const Mesh &mesh, const std::vector<std::vector<int>> &dense_blocks) {
  Pattern P;
  const int n = static_cast<int>(mesh.edges.size());
  const std::size_t T = mesh.tets.size();
  P.n = n;
  // edge -> incident tets (CSR)
  std::vector<int> inc_ptr(n + 1, 0);
  for (const auto &t : mesh.tets)
    for (int e : t.edges) inc_ptr[e + 1]++;
  for (int i = 0; i < n; ++i) inc_ptr[i + 1] += inc_ptr[i];
  std::vector<int> inc(inc_ptr[n]);
  {
    std::vector<int> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (std::size_t t = 0; t < T; ++t)
      for (int e : mesh.tets[t].edges) inc[fill[e]++] = static_cast<int>(t);
  }
  // extra columns from dense blocks: row -> list of block ids
  std::vector<std::vector<int>> row_blocks;
  if (!dense_blocks.empty()) {
    row_blocks.resize(n);
    for (std::size_t b = 0; b < dense_blocks.size(); ++b)
      for (int e : dense_blocks[b]) {
        if (e < 0 || e >= n) throw std::runtime_error("build_pattern: port edge out of range");
        row_blocks[e].push_back(static_cast<int>(b));
      }
  }
  // Row r: its diagonal, the edges of its tets and its dense blocks, sorted
  // and unique.  Two parallel passes over the rows: lengths, then columns.
  auto row_cols = [&](int r, std::vector<int> &buf) {
    buf.clear();
    buf.push_back(r);
    for (int k = inc_ptr[r]; k < inc_ptr[r + 1]; ++k)
      for (int e : mesh.tets[inc[k]].edges) buf.push_back(e);
    if (!row_blocks.empty())
      for (int b : row_blocks[r])
        buf.insert(buf.end(), dense_blocks[b].begin(), dense_blocks[b].end());
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
  std::vector<long long> len(static_cast<std::size_t>(n) + 1, 0);
  parallel_ranges(static_cast<std::size_t>(n), [&](std::size_t r0, std::size_t r1) {
    std::vector<int> buf;
    for (std::size_t r = r0; r < r1; ++r) {
      row_cols(static_cast<int>(r), buf);
      len[r + 1] = static_cast<long long>(buf.size());
    }
  });
  for (int r = 0; r < n; ++r) len[r + 1] += len[r];
  if (len[n] > static_cast<long long>(0x7fffffff))
    throw std::runtime_error("build_pattern: more than 2^31-1 nonzeros");
  P.rowptr.assign(len.begin(), len.end());
  P.colidx.assign(static_cast<std::size_t>(len[n]), 0);
  P.diag.resize(n);
  parallel_ranges(static_cast<std::size_t>(n), [&](std::size_t r0, std::size_t r1) {
    std::vector<int> buf;
    for (std::size_t r = r0; r < r1; ++r) {
      row_cols(static_cast<int>(r), buf);
      std::copy(buf.begin(), buf.end(), P.colidx.begin() + P.rowptr[r]);
      P.diag[r] = P.slot_of(static_cast<int>(r), static_cast<int>(r));
    }
  });
  P.slots.resize(36 * T);
  parallel_ranges(T, [&](std::size_t t0, std::size_t t1) {
    for (std::size_t t = t0; t < t1; ++t) {
      const auto &ed = mesh.tets[t].edges;
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) P.slots[36 * t + 6 * i + j] = P.slot_of(ed[i], ed[j]);
    }
  });
  // Greedy colouring with bit masks of used colours per edge.
  const int W = 4;  // up to 256 colours
  std::vector<std::uint64_t> used(static_cast<std::size_t>(n) * W, 0);
  std::vector<int> color(T);
  int ncolors = 0;
  for (std::size_t t = 0; t < T; ++t) {
    std::uint64_t m[W] = {0, 0, 0, 0};
    for (int e : mesh.tets[t].edges)
      for (int w = 0; w < W; ++w) m[w] |= used[static_cast<std::size_t>(e) * W + w];
    int c = -1;
    for (int w = 0; w < W && c < 0; ++w)
      if (~m[w]) c = 64 * w + __builtin_ctzll(~m[w]);
    if (c < 0) throw std::runtime_error("build_pattern: more than 256 colours needed");
    color[t] = c;
    ncolors = std::max(ncolors, c + 1);
    for (int e : mesh.tets[t].edges) used[static_cast<std::size_t>(e) * W + c / 64] |= (1ull << (c % 64));
  }
  P.color_offsets.assign(ncolors + 1, 0);
  for (std::size_t t = 0; t < T; ++t) P.color_offsets[color[t] + 1]++;
  for (int c = 0; c < ncolors; ++c) P.color_offsets[c + 1] += P.color_offsets[c];
  P.color_tets.resize(T);
  {
    std::vector<int> fill(P.color_offsets.begin(), P.color_offsets.end() - 1);
    for (std::size_t t = 0; t < T; ++t) P.color_tets[fill[color[t]]++] = static_cast<int>(t);
  }
  return P;
}

}  // namespace edgefem
