// vibestran_gb300/csrc/dofmap.cpp — analysis DOF map and FORCE loads (host C++).
//
// The reference builds the map in three passes (src/core/dof_map.cpp:10-97,
// src/solver/analysis_support.cpp:176-214): six slots per node in ascending
// node-id order, constrain_batch of every slot no element activates, then
// constrain_batch of the SPC components; each batch shifts surviving indices
// down by the number of removed indices below them.  The net effect is that a
// surviving slot's equation equals the number of surviving slots before it in
// (node-id rank, dof) order — computed here in one sorted pass.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/vsgb.h"

namespace {

void put_err(char* err, size_t len, const std::string& m) {
  if (err && len > 0) std::snprintf(err, len, "%s", m.c_str());
}

}  // namespace

extern "C" int vsgb_write_node_csv(const char* path, int n_nodes, const int* node_ids,
                                   int n_subcases, const int* subcase_ids, const double* disp,
                                   char* err, size_t errlen) {
  if (!path || n_nodes < 0 || n_subcases < 0 || (n_nodes > 0 && (!node_ids || !disp)) ||
      (n_subcases > 0 && !subcase_ids)) {
    put_err(err, errlen, "vsgb_write_node_csv: invalid argument");
    return VSGB_ERR_INVALID;
  }
  std::FILE* f = std::fopen(path, "w");
  if (!f) {
    put_err(err, errlen, std::string("Cannot write CSV: ") + path);
    return VSGB_ERR_INVALID;
  }
  std::vector<int> order(static_cast<size_t>(n_nodes));
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [node_ids](int a, int b) { return node_ids[a] < node_ids[b]; });
  std::fputs("# node_id, subcase_id, T1, T2, T3, R1, R2, R3\n", f);
  char line[256];
  for (int s = 0; s < n_subcases; ++s) {
    const double* ds = disp + static_cast<size_t>(s) * n_nodes * 6;
    for (int i : order) {
      const double* d = ds + static_cast<size_t>(i) * 6;
      const int len =
          std::snprintf(line, sizeof(line), "%d, %d, %.8e, %.8e, %.8e, %.8e, %.8e, %.8e\n",
                        node_ids[i], subcase_ids[s], d[0], d[1], d[2], d[3], d[4], d[5]);
      std::fwrite(line, 1, static_cast<size_t>(len), f);
    }
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) {
    put_err(err, errlen, std::string("Cannot write CSV: ") + path);
    return VSGB_ERR_INVALID;
  }
  return VSGB_OK;
}

extern "C" int vsgb_build_dof_map(int n_nodes, const int* node_ids, int n_elem,
                                  const int* conn_ids, int n_spc, const int* spc_node_ids,
                                  const int* spc_masks, int* eq6_out, int* n_free, char* err,
                                  size_t errlen) {
  try {
    if (n_nodes < 0 || n_elem < 0 || n_spc < 0 || (n_nodes > 0 && (!node_ids || !eq6_out)) ||
        (n_elem > 0 && !conn_ids) || (n_spc > 0 && (!spc_node_ids || !spc_masks)) || !n_free) {
      put_err(err, errlen, "vsgb_build_dof_map: invalid argument");
      return VSGB_ERR_INVALID;
    }
    std::unordered_map<int, int> index;
    index.reserve(static_cast<size_t>(n_nodes) * 2);
    for (int i = 0; i < n_nodes; ++i) {
      if (!index.emplace(node_ids[i], i).second) {
        put_err(err, errlen, "duplicate node id " + std::to_string(node_ids[i]));
        return VSGB_ERR_INVALID;
      }
    }
    // Active mask: solids activate T1-T3 (analysis_support.cpp:39-57).
    std::vector<unsigned char> mask(static_cast<size_t>(n_nodes), 0);
    for (long long k = 0; k < 8LL * n_elem; ++k) {
      auto it = index.find(conn_ids[k]);
      if (it == index.end()) {
        put_err(err, errlen, "element " + std::to_string(k / 8) + " references unknown node " +
                                 std::to_string(conn_ids[k]));
        return VSGB_ERR_INVALID;
      }
      mask[static_cast<size_t>(it->second)] = 0b111;
    }
    // SPC components (bit d = DOF d+1) are removed from the active set.
    for (int s = 0; s < n_spc; ++s) {
      auto it = index.find(spc_node_ids[s]);
      if (it == index.end()) {
        put_err(err, errlen,
                "constrain_batch: node " + std::to_string(spc_node_ids[s]) + " not in DofMap");
        return VSGB_ERR_INVALID;
      }
      mask[static_cast<size_t>(it->second)] &= static_cast<unsigned char>(~spc_masks[s] & 0x3F);
    }
    std::vector<int> order(static_cast<size_t>(n_nodes));
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(),
              [&](int a, int b) { return node_ids[a] < node_ids[b]; });
    int next = 0;
    for (int i : order) {
      for (int d = 0; d < 6; ++d)
        eq6_out[6 * i + d] = (d < 3 && (mask[static_cast<size_t>(i)] >> d & 1)) ? next++ : -1;
    }
    *n_free = next;
    return VSGB_OK;
  } catch (const std::exception& e) {
    put_err(err, errlen, e.what());
    return VSGB_ERR_INVALID;
  }
}

// LinearStaticSolver::apply_point_loads (src/solver/linear_static.cpp:344-374)
// for FORCE cards in the basic frame (CID 0): F[eq] += scale * N_d for each
// free translational DOF of the loaded grid.
extern "C" int vsgb_apply_forces(int n_nodes, const int* node_ids, const int* eq6, int n_force,
                                 const int* force_node_ids, const double* scale,
                                 const double* dir, int n, double* F, char* err,
                                 size_t errlen) {
  try {
    std::unordered_map<int, int> index;
    index.reserve(static_cast<size_t>(n_nodes) * 2);
    for (int i = 0; i < n_nodes; ++i) index.emplace(node_ids[i], i);
    for (int f = 0; f < n_force; ++f) {
      auto it = index.find(force_node_ids[f]);
      if (it == index.end()) {
        put_err(err, errlen, "DofMap: node " + std::to_string(force_node_ids[f]) + " not found");
        return VSGB_ERR_INVALID;
      }
      for (int d = 0; d < 3; ++d) {
        const int eq = eq6[6 * it->second + d];
        if (eq < 0) continue;
        if (eq >= n) {
          put_err(err, errlen, "Force vector index out of range");
          return VSGB_ERR_INVALID;
        }
        F[eq] += scale[f] * dir[3 * f + d];
      }
    }
    return VSGB_OK;
  } catch (const std::exception& e) {
    put_err(err, errlen, e.what());
    return VSGB_ERR_INVALID;
  }
}
