// Host-side sparsity pattern of a HEX8 mesh (node adjacency through shared cells).
// The per-node sorted neighbour lists reproduce the column order scipy gives the
// COO->CSR conversion of crystal_plasticity_OR_design/solver.py:279-282.
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cpfem_gb300.h"

namespace cpfem {
void set_error(const std::string& msg);
}

namespace {

int check_cells(int32_t num_cells, const int32_t* cells, int32_t num_nodes) {
  if (num_cells < 0 || num_nodes < 0 || (num_cells > 0 && cells == nullptr)) {
    cpfem::set_error("bad mesh arguments");
    return CPFEM_ERR_ARG;
  }
  for (int64_t i = 0; i < (int64_t)num_cells * 8; ++i)
    if (cells[i] < 0 || cells[i] >= num_nodes) {
      cpfem::set_error("cell node index out of range");
      return CPFEM_ERR_ARG;
    }
  return CPFEM_OK;
}

// node -> incident cells (CSR)
void incidence(int32_t num_cells, const int32_t* cells, int32_t num_nodes, std::vector<int64_t>& ptr,
               std::vector<int32_t>& inc) {
  ptr.assign((size_t)num_nodes + 1, 0);
  for (int64_t i = 0; i < (int64_t)num_cells * 8; ++i) ptr[cells[i] + 1]++;
  for (int32_t a = 0; a < num_nodes; ++a) ptr[a + 1] += ptr[a];
  inc.resize((size_t)num_cells * 8);
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  for (int32_t e = 0; e < num_cells; ++e)
    for (int k = 0; k < 8; ++k) inc[fill[cells[8 * (int64_t)e + k]]++] = e;
}

void neighbours(int32_t a, const int32_t* cells, const std::vector<int64_t>& ptr, const std::vector<int32_t>& inc,
                std::vector<int32_t>& out) {
  out.clear();
  for (int64_t t = ptr[a]; t < ptr[a + 1]; ++t) {
    const int32_t e = inc[t];
    for (int k = 0; k < 8; ++k) out.push_back(cells[8 * (int64_t)e + k]);
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}

}  // namespace

extern "C" {

int cpfem_pattern_count(int32_t num_cells, const int32_t* cells, int32_t num_nodes, int64_t* num_blocks) {
  int rc = check_cells(num_cells, cells, num_nodes);
  if (rc) return rc;
  if (!num_blocks) { cpfem::set_error("num_blocks is null"); return CPFEM_ERR_ARG; }
  std::vector<int64_t> ptr;
  std::vector<int32_t> inc, nb;
  incidence(num_cells, cells, num_nodes, ptr, inc);
  int64_t total = 0;
  for (int32_t a = 0; a < num_nodes; ++a) {
    neighbours(a, cells, ptr, inc, nb);
    total += (int64_t)nb.size();
  }
  if (9 * total > INT32_MAX) { cpfem::set_error("pattern too large for int32 CSR"); return CPFEM_ERR_SIZE; }
  *num_blocks = total;
  return CPFEM_OK;
}

int cpfem_pattern_build(int32_t num_cells, const int32_t* cells, int32_t num_nodes, int32_t* node_rowptr,
                        int32_t* node_cols, uint8_t* elem_pos, int32_t* node_tpos) {
  int rc = check_cells(num_cells, cells, num_nodes);
  if (rc) return rc;
  if (!node_rowptr || !node_cols) { cpfem::set_error("pattern outputs are null"); return CPFEM_ERR_ARG; }
  std::vector<int64_t> ptr;
  std::vector<int32_t> inc, nb;
  incidence(num_cells, cells, num_nodes, ptr, inc);
  node_rowptr[0] = 0;
  for (int32_t a = 0; a < num_nodes; ++a) {
    neighbours(a, cells, ptr, inc, nb);
    if (nb.size() > 255) { cpfem::set_error("node degree above 255"); return CPFEM_ERR_SIZE; }
    std::copy(nb.begin(), nb.end(), node_cols + node_rowptr[a]);
    node_rowptr[a + 1] = node_rowptr[a] + (int32_t)nb.size();
  }
  auto pos_of = [&](int32_t a, int32_t b) -> int32_t {
    const int32_t* beg = node_cols + node_rowptr[a];
    const int32_t* end = node_cols + node_rowptr[a + 1];
    return (int32_t)(std::lower_bound(beg, end, b) - beg);
  };
  if (elem_pos)
    for (int32_t e = 0; e < num_cells; ++e)
      for (int a = 0; a < 8; ++a)
        for (int b = 0; b < 8; ++b)
          elem_pos[64 * (int64_t)e + 8 * a + b] = (uint8_t)pos_of(cells[8 * (int64_t)e + a], cells[8 * (int64_t)e + b]);
  if (node_tpos)
    for (int32_t a = 0; a < num_nodes; ++a)
      for (int32_t j = node_rowptr[a]; j < node_rowptr[a + 1]; ++j) node_tpos[j] = pos_of(node_cols[j], a);
  return CPFEM_OK;
}

int cpfem_pattern_expand_csr(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                             int32_t* indptr, int32_t* indices) {
  if (num_nodes < 0 || !node_rowptr || !node_cols || !indptr || !indices) {
    cpfem::set_error("bad expand arguments");
    return CPFEM_ERR_ARG;
  }
  indptr[0] = 0;
  int64_t w = 0;
  for (int32_t a = 0; a < num_nodes; ++a) {
    const int32_t r0 = node_rowptr[a], r1 = node_rowptr[a + 1];
    for (int i = 0; i < 3; ++i) {
      for (int32_t j = r0; j < r1; ++j)
        for (int k = 0; k < 3; ++k) indices[w++] = 3 * node_cols[j] + k;
      indptr[3 * a + i + 1] = (int32_t)w;
    }
  }
  return CPFEM_OK;
}

}  // extern "C"

// ---- sliced-ELL layout of the same pattern ------------------------------------------
extern "C" {

int cpfem_sell_count(int32_t num_nodes, const int32_t* node_rowptr, int64_t* total_slots) {
  if (num_nodes < 0 || !node_rowptr || !total_slots) {
    cpfem::set_error("bad sell arguments");
    return CPFEM_ERR_ARG;
  }
  int64_t total = 0;
  for (int32_t g0 = 0; g0 < num_nodes; g0 += 32) {
    int32_t w = 0;
    for (int32_t a = g0; a < std::min(num_nodes, g0 + 32); ++a) w = std::max(w, node_rowptr[a + 1] - node_rowptr[a]);
    total += 32 * (int64_t)w;
  }
  if (9 * total > ((int64_t)1 << 40)) {
    cpfem::set_error("sell layout too large");
    return CPFEM_ERR_SIZE;
  }
  *total_slots = total;
  return CPFEM_OK;
}

int cpfem_sell_build(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                     const int32_t* node_tpos, int64_t* group_off, int32_t* group_width, int32_t* cols,
                     int32_t* tpos, int32_t* diag_slot) {
  if (num_nodes < 0 || !node_rowptr || !node_cols || !group_off || !group_width || !cols || !diag_slot) {
    cpfem::set_error("bad sell arguments");
    return CPFEM_ERR_ARG;
  }
  const int32_t ng = (num_nodes + 31) / 32;
  group_off[0] = 0;
  for (int32_t g = 0; g < ng; ++g) {
    const int32_t a0 = 32 * g, a1 = std::min(num_nodes, a0 + 32);
    int32_t w = 0;
    for (int32_t a = a0; a < a1; ++a) w = std::max(w, node_rowptr[a + 1] - node_rowptr[a]);
    group_width[g] = w;
    group_off[g + 1] = group_off[g] + 32 * (int64_t)w;
    for (int32_t lane = 0; lane < 32; ++lane) {
      const int32_t a = a0 + lane;
      for (int32_t j = 0; j < w; ++j) {
        const int64_t s = group_off[g] + 32 * (int64_t)j + lane;
        if (a < a1 && j < node_rowptr[a + 1] - node_rowptr[a]) {
          cols[s] = node_cols[node_rowptr[a] + j];
          if (tpos) tpos[s] = node_tpos ? node_tpos[node_rowptr[a] + j] : 0;
        } else {
          // padding: own node (or the group's first node past the end), zero values
          cols[s] = (a < a1) ? a : a0;
          if (tpos) tpos[s] = j;
        }
      }
      if (a < a1) {
        int32_t d = -1;
        for (int32_t j = node_rowptr[a]; j < node_rowptr[a + 1]; ++j)
          if (node_cols[j] == a) d = j - node_rowptr[a];
        if (d < 0) {
          cpfem::set_error("node missing from its own neighbour list");
          return CPFEM_ERR_ARG;
        }
        diag_slot[a] = d;
      }
    }
  }
  return CPFEM_OK;
}

int cpfem_sell_csr_map(int32_t num_nodes, const int32_t* node_rowptr, const int64_t* group_off, int64_t* map) {
  if (num_nodes < 0 || !node_rowptr || !group_off || !map) {
    cpfem::set_error("bad sell map arguments");
    return CPFEM_ERR_ARG;
  }
  int64_t w = 0;
  for (int32_t a = 0; a < num_nodes; ++a) {
    const int32_t g = a / 32, lane = a % 32;
    const int32_t deg = node_rowptr[a + 1] - node_rowptr[a];
    for (int i = 0; i < 3; ++i)
      for (int32_t j = 0; j < deg; ++j)
        for (int k = 0; k < 3; ++k) map[w++] = 9 * group_off[g] + 32 * (int64_t)(9 * j + 3 * i + k) + lane;
  }
  return CPFEM_OK;
}

}  // extern "C"

// ---- element colouring for a deterministic, atomic-free scatter -----------------------
extern "C" int cpfem_color_cells(int32_t num_cells, const int32_t* cells, int32_t num_nodes, int32_t* color,
                                 int32_t* num_colors) {
  int rc = check_cells(num_cells, cells, num_nodes);
  if (rc) return rc;
  if (!color || !num_colors) {
    cpfem::set_error("bad colouring arguments");
    return CPFEM_ERR_ARG;
  }
  // greedy in cell order: the smallest colour not held by a cell sharing a node
  std::vector<uint64_t> node_mask((size_t)num_nodes, 0);
  int32_t nc = 0;
  for (int32_t e = 0; e < num_cells; ++e) {
    uint64_t used = 0;
    for (int k = 0; k < 8; ++k) used |= node_mask[cells[8 * (int64_t)e + k]];
    int c = 0;
    while (c < 64 && (used >> c) & 1u) ++c;
    if (c >= 64) {
      cpfem::set_error("more than 64 colours needed");
      return CPFEM_ERR_SIZE;
    }
    color[e] = c;
    nc = std::max(nc, c + 1);
    for (int k = 0; k < 8; ++k) node_mask[cells[8 * (int64_t)e + k]] |= (uint64_t)1 << c;
  }
  *num_colors = nc;
  return CPFEM_OK;
}

// Slot of every neighbour offset of every node of a structured box (x fastest):
// out[27*i + (dz+1)*9 + (dy+1)*3 + (dx+1)] = position of that neighbour in row i of the
// node-block pattern (= its sliced-ELL slot), -1 where the neighbour does not exist.
extern "C" int cpfem_mg_slot_table(int32_t num_nodes, const int32_t* dims, const int32_t* node_rowptr,
                                   const int32_t* node_cols, int8_t* out) {
  if (num_nodes < 0 || !dims || !node_rowptr || !node_cols || !out) {
    cpfem::set_error("bad slot-table arguments");
    return CPFEM_ERR_ARG;
  }
  const int64_t nx = dims[0], ny = dims[1], nz = dims[2];
  if (nx < 1 || ny < 1 || nz < 1 || nx * ny * nz != num_nodes) {
    cpfem::set_error("dims do not match num_nodes");
    return CPFEM_ERR_ARG;
  }
  for (int64_t i = 0; i < num_nodes; ++i) {
    for (int c = 0; c < 27; ++c) out[27 * i + c] = -1;
    const int64_t ix = i % nx, iy = (i / nx) % ny, iz = i / (nx * ny);
    const int32_t r0 = node_rowptr[i], r1 = node_rowptr[i + 1];
    if (r1 - r0 > 127) {
      cpfem::set_error("row too long for a structured box");
      return CPFEM_ERR_ARG;
    }
    for (int32_t p = r0; p < r1; ++p) {
      const int64_t j = node_cols[p];
      if (j < 0 || j >= num_nodes) {
        cpfem::set_error("column out of range");
        return CPFEM_ERR_ARG;
      }
      const int64_t dx = j % nx - ix, dy = (j / nx) % ny - iy, dz = j / (nx * ny) - iz;
      if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) {
        cpfem::set_error("pattern is not a structured box of the given dims (neighbour beyond one node)");
        return CPFEM_ERR_ARG;
      }
      out[27 * i + (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)] = (int8_t)(p - r0);
    }
  }
  return CPFEM_OK;
}

extern "C" size_t cpfem_struct_size(int32_t which) {
  switch (which) {
    case 0: return sizeof(cpfem_material_t);
    case 1: return sizeof(cpfem_gp_args_t);
    case 2: return sizeof(cpfem_vjp_args_t);
    case 3: return sizeof(cpfem_sell_t);
    case 4: return sizeof(cpfem_mg_t);
    case 5: return sizeof(cpfem_krylov_opts_t);
    case 6: return sizeof(cpfem_solve_report_t);
    default: return 0;
  }
}
