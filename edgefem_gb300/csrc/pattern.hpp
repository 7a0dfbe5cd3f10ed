// Host-side CSR pattern, scatter map and colouring for one mesh.
#pragma once

#include <vector>

#include "edgefem.hpp"

namespace edgefem {

struct Pattern {
  int n = 0;
  std::vector<int> rowptr;         // n+1
  std::vector<int> colidx;         // nnz, sorted per row
  std::vector<int> diag;           // slot of (r, r)
  std::vector<int> slots;          // 36 per tet, row-major (i, j)
  std::vector<int> color_tets;     // tets grouped by colour
  std::vector<int> color_offsets;  // ncolors+1
  int nnz() const { return static_cast<int>(colidx.size()); }
  int slot_of(int r, int c) const;  // -1 if absent
};

Pattern build_pattern(const Mesh &mesh, const std::vector<std::vector<int>> &dense_blocks);

}  // namespace edgefem
