// Node layout inside each grain: cell-sorted, cell-sorted then grouped by bond count (whole grain
// or 256-node windows), or a seeded shuffle; see pg_order.h.
#include "pg_order.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace pg {

namespace {

// the input's order is kept unless its mean bond index span exceeds this multiple of the cell
// order's (measured: generated row-major meshes 1.00, the same meshes shuffled 4-9)
constexpr double CELL_SPAN_RATIO = 1.5;
// window of PG_ORDER_CELL_BLOCK_DEGREE: sorting by degree inside 256 consecutive nodes lifts the
// bond slab's slot use (bonds / padded slots of 32-node chunks) from 0.80 to 0.95 on the 3D sphere
// and settling meshes while keeping nodes near their cell-order neighbours
constexpr uint32_t DEGREE_WINDOW = 256;

uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// Order of the nodes [n0, n1) of grain g as grain-local indices; returns false when it is the
// identity.
bool grain_order(const pg_setup_desc* s, uint32_t n0, uint32_t n1, int32_t order, uint32_t g,
                 std::vector<uint32_t>* loc) {
  const uint32_t n = n1 - n0, D = s->dim;
  loc->resize(n);
  std::iota(loc->begin(), loc->end(), 0u);
  if (order == PG_ORDER_SHUFFLE) {
    for (uint32_t i = n; i > 1; --i) {
      const uint32_t j = (uint32_t)(mix64(((uint64_t)g << 32) | i) % i);
      std::swap((*loc)[i - 1], (*loc)[j]);
    }
    return n > 1;
  }
  // strips one node spacing high, h = (mean node volume)^(1/dim): z then y (3D), y (2D); x within
  // a strip; the input index breaks ties
  double vsum = 0.0;
  for (uint32_t i = n0; i < n1; ++i) vsum += s->vol[i];
  const double h = std::pow(vsum / (double)n, 1.0 / (double)D);
  const bool fin = h > 0.0 && std::isfinite(h);
  double lo[3] = {INFINITY, INFINITY, INFINITY};
  for (uint32_t i = n0; i < n1; ++i)
    for (uint32_t c = 0; c < D; ++c) lo[c] = std::min(lo[c], s->pos[(size_t)i * D + c]);
  std::vector<int64_t> strip((size_t)n * 2, 0);
  for (uint32_t k = 0; k < n; ++k) {
    const double* x = s->pos + (size_t)(n0 + k) * D;
    strip[2 * k] = (D == 3 && fin) ? (int64_t)std::floor((x[2] - lo[2]) / h + 0.5) : 0;
    strip[2 * k + 1] = fin ? (int64_t)std::floor((x[1] - lo[1]) / h + 0.5) : 0;
  }
  auto before = [&](uint32_t a, uint32_t b) {
    if (strip[2 * a] != strip[2 * b]) return strip[2 * a] < strip[2 * b];
    if (strip[2 * a + 1] != strip[2 * b + 1]) return strip[2 * a + 1] < strip[2 * b + 1];
    const double xa = s->pos[(size_t)(n0 + a) * D], xb = s->pos[(size_t)(n0 + b) * D];
    if (xa != xb) return xa < xb;
    return a < b;
  };
  bool moved = false;
  for (uint32_t k = 1; k < n && !moved; ++k) moved = before(k, k - 1);
  if (moved) {
    std::sort(loc->begin(), loc->end(), before);
    // keep the input's order when it is about as local already: the bond rows stay in the
    // input's entry order, which suits the input's own node order (a mesh generator's row-major
    // order along another axis gathers better than the re-sorted one). Compared: the mean index
    // distance between bonded nodes over every fourth node of the grain, in both orders.
    std::vector<uint32_t> pos_of(n);
    for (uint32_t k = 0; k < n; ++k) pos_of[(*loc)[k]] = k;
    double span_in = 0.0, span_cell = 0.0;
    for (uint32_t a = 0; a < n; a += 4)
      for (uint64_t b = s->bond_offset[n0 + a]; b < s->bond_offset[n0 + a + 1]; ++b) {
        const uint32_t j = s->bond_local[b];
        span_in += std::fabs((double)j - (double)a);
        span_cell += std::fabs((double)pos_of[j] - (double)pos_of[a]);
      }
    if (span_in <= CELL_SPAN_RATIO * span_cell) {
      std::iota(loc->begin(), loc->end(), 0u);
      moved = false;
    }
  }
  auto deg_of = [&](uint32_t k) { return s->bond_offset[n0 + k + 1] - s->bond_offset[n0 + k]; };
  if (order == PG_ORDER_CELL_BLOCK_DEGREE) {
    // stable sort by bond count, most bonds first, inside each window of DEGREE_WINDOW nodes
    for (uint32_t w0 = 0; w0 < n; w0 += DEGREE_WINDOW) {
      const uint32_t w1 = std::min(n, w0 + DEGREE_WINDOW);
      std::stable_sort(loc->begin() + w0, loc->begin() + w1,
                       [&](uint32_t a, uint32_t b) { return deg_of(a) > deg_of(b); });
    }
    moved = false;
    for (uint32_t k = 0; k < n && !moved; ++k) moved = (*loc)[k] != k;
    return moved;
  }
  if (order == PG_ORDER_CELL_DEGREE) {
    // stable counting sort by bond count, most bonds first
    uint64_t dmax = 0;
    for (uint32_t k = 0; k < n; ++k) dmax = std::max<uint64_t>(dmax, s->bond_offset[n0 + k + 1] - s->bond_offset[n0 + k]);
    std::vector<uint32_t> cnt(dmax + 2, 0), out(n);
    auto deg = [&](uint32_t k) { return (uint32_t)(s->bond_offset[n0 + k + 1] - s->bond_offset[n0 + k]); };
    for (uint32_t k = 0; k < n; ++k) ++cnt[dmax - deg(k) + 1];
    for (size_t b = 1; b < cnt.size(); ++b) cnt[b] += cnt[b - 1];
    for (uint32_t k = 0; k < n; ++k) {
      const uint32_t v = (*loc)[k];
      out[cnt[dmax - deg(v)]++] = v;
    }
    for (uint32_t k = 0; k < n && !moved; ++k) moved = out[k] != k;
    *loc = std::move(out);
  }
  return moved;
}

}  // namespace

int make_node_order(const pg_setup_desc* s, int32_t order, NodeOrder* o, std::string* err) {
  o->perm.clear();
  o->at.clear();
  o->bdry_nodes.clear();
  o->clamped_nodes.clear();
  if (order == PG_ORDER_INPUT) return PG_OK;
  if (order != PG_ORDER_CELL && order != PG_ORDER_CELL_DEGREE && order != PG_ORDER_SHUFFLE &&
      order != PG_ORDER_CELL_BLOCK_DEGREE) {
    *err = "unknown node_order " + std::to_string(order);
    return PG_EINVAL;
  }
  const uint32_t N = s->n_nodes, G = s->n_grains;
  std::vector<uint32_t> perm(N), loc;
  bool any = false;
  for (uint32_t g = 0; g < G; ++g) {
    const uint32_t n0 = s->grain_node_offset[g], n1 = s->grain_node_offset[g + 1];
    any = grain_order(s, n0, n1, order, g, &loc) || any;
    for (uint32_t k = 0; k < n1 - n0; ++k) perm[n0 + k] = n0 + loc[k];
  }
  if (!any) return PG_OK;  // the input already is in this order
  o->perm = std::move(perm);
  o->at.resize(N);
  for (uint32_t i = 0; i < N; ++i) o->at[o->perm[i]] = i;
  auto lists = [&](const uint32_t* off, const uint32_t* nodes, std::vector<uint32_t>* dst) {
    dst->assign(nodes, nodes + off[G]);
    for (uint32_t g = 0; g < G; ++g) {
      const uint32_t n0 = s->grain_node_offset[g];
      for (uint32_t k = off[g]; k < off[g + 1]; ++k) (*dst)[k] = o->at[n0 + nodes[k]] - n0;
    }
  };
  lists(s->bdry_offset, s->bdry_nodes, &o->bdry_nodes);
  lists(s->clamped_offset, s->clamped_nodes, &o->clamped_nodes);
  return PG_OK;
}

}  // namespace pg
