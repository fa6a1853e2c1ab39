// Node layout inside each grain (pg_node_order): the permutation pg_create lays the device arrays
// out by. Grain node ranges do not change; only the order of the nodes inside a grain does.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/perigrain.h"

namespace pg {

struct NodeOrder {
  // perm[new] = original global index, at[original] = new index; both empty when the input is
  // already in the requested order (or PG_ORDER_INPUT)
  std::vector<uint32_t> perm, at;
  // the setup's boundary and clamped node lists with renumbered entries (list order kept: the
  // boundary list's order is the nl_bdry_only visit order); empty when perm is
  std::vector<uint32_t> bdry_nodes, clamped_nodes;
};

// Fills `o` for `order` (pg_node_order). Expects a setup that passed pg_create's host validation
// (boundary and clamped entries inside their grains). Returns PG_OK or PG_EINVAL (unknown order).
int make_node_order(const pg_setup_desc* s, int32_t order, NodeOrder* o, std::string* err);

}  // namespace pg
