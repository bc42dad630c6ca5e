// swe_layout.cu -- cell orders (Morton, reverse Cuthill-McKee), the edge and
// node orders that follow from them, and the gather cost model that picks one.
// Host code only.
#include "swe_layout.cuh"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>

namespace swe {

namespace {

// bits 0..31 of v to the even bits of the result
uint64_t spread2(uint64_t v) {
  v &= 0xffffffffull;
  v = (v | (v << 16)) & 0x0000ffff0000ffffull;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}

std::vector<int64_t> inverse(const std::vector<int64_t>& from) {
  std::vector<int64_t> to(from.size());
  for (size_t j = 0; j < from.size(); ++j) to[from[j]] = (int64_t)j;
  return to;
}

int64_t count_distinct(std::vector<int64_t>& v) {
  std::sort(v.begin(), v.end());
  return std::unique(v.begin(), v.end()) - v.begin();
}

}  // namespace

std::vector<int64_t> morton_cells(const HostInstance& h) {
  const int64_t C = h.C;
  std::vector<double> cx(C), cy(C);
  double x0 = std::numeric_limits<double>::infinity(), y0 = x0, x1 = -x0, y1 = -x0;
  for (int64_t i = 0; i < C; ++i) {
    const int64_t a = h.cn[3 * i], b = h.cn[3 * i + 1], c = h.cn[3 * i + 2];
    cx[i] = (h.geom[3 * a] + h.geom[3 * b] + h.geom[3 * c]) / 3.;
    cy[i] = (h.geom[3 * a + 1] + h.geom[3 * b + 1] + h.geom[3 * c + 1]) / 3.;
    x0 = std::min(x0, cx[i]);
    x1 = std::max(x1, cx[i]);
    y0 = std::min(y0, cy[i]);
    y1 = std::max(y1, cy[i]);
  }
  const double ext = std::max(x1 - x0, y1 - y0);
  const double scale = ext > 0. ? 2097151. / ext : 0.;  // 2^21 - 1 cells per side
  std::vector<uint64_t> key(C);
  for (int64_t i = 0; i < C; ++i) {
    const uint64_t qx = (uint64_t)std::min(2097151., std::max(0., (cx[i] - x0) * scale));
    const uint64_t qy = (uint64_t)std::min(2097151., std::max(0., (cy[i] - y0) * scale));
    key[i] = spread2(qx) | (spread2(qy) << 1);
  }
  std::vector<int64_t> order(C);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
  return order;
}

std::vector<int64_t> rcm_cells(const HostInstance& h) {
  const int64_t C = h.C;
  std::vector<int> deg(C, 0);
  for (int64_t i = 0; i < C; ++i)
    for (int k = 0; k < 3; ++k) deg[i] += h.ct[3 * i + k] >= 0;
  std::vector<int64_t> stamp(C, -1);
  int64_t pass = 0;
  std::vector<int64_t> level_now, level_next;
  // breadth-first levels from r; returns the number of levels and leaves the
  // last level in level_now
  auto levels = [&](int64_t r) {
    ++pass;
    level_now.assign(1, r);
    stamp[r] = pass;
    int n = 1;
    for (;;) {
      level_next.clear();
      for (int64_t v : level_now)
        for (int k = 0; k < 3; ++k) {
          const int64_t w = h.ct[3 * v + k];
          if (w >= 0 && stamp[w] != pass) {
            stamp[w] = pass;
            level_next.push_back(w);
          }
        }
      if (level_next.empty()) return n;
      level_now.swap(level_next);
      ++n;
    }
  };
  auto by_degree = [&](int64_t a, int64_t b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; };

  std::vector<char> placed(C, 0);
  std::vector<int64_t> order;
  order.reserve(C);
  std::vector<int64_t> nb;
  for (int64_t s = 0; s < C; ++s) {
    if (placed[s]) continue;
    // pseudo-peripheral start: walk to a lowest-degree cell of the last
    // level while the eccentricity grows
    int64_t r = s;
    int ecc = levels(r);
    for (int it = 0; it < 8; ++it) {
      const int64_t x = *std::min_element(level_now.begin(), level_now.end(), by_degree);
      const int e2 = levels(x);
      if (e2 <= ecc) break;
      ecc = e2;
      r = x;
    }
    // Cuthill-McKee from r: neighbours in increasing degree
    size_t head = order.size();
    order.push_back(r);
    placed[r] = 1;
    while (head < order.size()) {
      const int64_t v = order[head++];
      nb.clear();
      for (int k = 0; k < 3; ++k) {
        const int64_t w = h.ct[3 * v + k];
        if (w >= 0 && !placed[w]) {
          placed[w] = 1;
          nb.push_back(w);
        }
      }
      std::sort(nb.begin(), nb.end(), by_degree);
      order.insert(order.end(), nb.begin(), nb.end());
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

Layout layout_from_cells(const HostInstance& h, int strategy, std::vector<int64_t>&& cell_from) {
  Layout L;
  L.strategy = strategy;
  L.cell_from = std::move(cell_from);
  L.cell_to = inverse(L.cell_from);
  const int64_t C = h.C, E = h.E, N = h.N;
  std::vector<char> seen_e(E, 0), seen_n(N, 0);
  L.edge_from.reserve(E);
  L.node_from.reserve(N);
  for (int64_t j = 0; j < C; ++j) {
    const int64_t i = L.cell_from[j];
    for (int k = 0; k < 3; ++k) {
      const int64_t e = h.ce[3 * i + k];
      if (h.ec[2 * e] == i && !seen_e[e]) {
        seen_e[e] = 1;
        L.edge_from.push_back(e);
      }
      const int64_t n = h.cn[3 * i + k];
      if (!seen_n[n]) {
        seen_n[n] = 1;
        L.node_from.push_back(n);
      }
    }
  }
  for (int64_t e = 0; e < E; ++e)
    if (!seen_e[e]) L.edge_from.push_back(e);
  for (int64_t n = 0; n < N; ++n)
    if (!seen_n[n]) L.node_from.push_back(n);
  return L;
}

Layout make_layout(const HostInstance& h, int strategy) {
  if (strategy == kLayoutMorton) return layout_from_cells(h, strategy, morton_cells(h));
  if (strategy == kLayoutRcm) return layout_from_cells(h, strategy, rcm_cells(h));
  return Layout{};
}

HostInstance apply_layout(const HostInstance& h, const Layout& L) {
  if (L.identity()) return h;
  const int64_t C = h.C, E = h.E, N = h.N;
  const std::vector<int64_t> edge_to = inverse(L.edge_from), node_to = inverse(L.node_from);
  const std::vector<int64_t>& cell_to = L.cell_to;
  HostInstance o;
  o.C = C;
  o.E = E;
  o.N = N;
  o.cfl = h.cfl;
  o.cor = h.cor;
  o.geom.resize(3 * N);
  for (int64_t j = 0; j < N; ++j)
    for (int c = 0; c < 3; ++c) o.geom[3 * j + c] = h.geom[3 * L.node_from[j] + c];
  o.en.resize(2 * E);
  o.ec.resize(2 * E);
  for (int64_t j = 0; j < E; ++j) {
    const int64_t e = L.edge_from[j];
    for (int c = 0; c < 2; ++c) {
      o.en[2 * j + c] = node_to[h.en[2 * e + c]];
      const int64_t t = h.ec[2 * e + c];
      o.ec[2 * j + c] = t >= 0 ? cell_to[t] : t;
    }
  }
  o.cn.resize(3 * C);
  o.ce.resize(3 * C);
  o.ct.resize(3 * C);
  for (int64_t j = 0; j < C; ++j) {
    const int64_t i = L.cell_from[j];
    for (int k = 0; k < 3; ++k) {
      o.cn[3 * j + k] = node_to[h.cn[3 * i + k]];
      o.ce[3 * j + k] = edge_to[h.ce[3 * i + k]];
      const int64_t t = h.ct[3 * i + k];
      o.ct[3 * j + k] = t >= 0 ? cell_to[t] : t;
    }
  }
  return o;
}

double gather_sectors(const HostInstance& h) {
  const int64_t C = h.C, E = h.E;
  // above 2^18 cells every 4th warp is counted (and the sum scaled)
  const int64_t stride = C > (1 << 18) ? 4 * 32 : 32;
  const double scale = (double)(stride / 32);
  double cost = 0.;
  std::vector<int64_t> v;
  v.reserve(96);
  for (int64_t w0 = 0; w0 < C; w0 += stride) {
    const int64_t w1 = std::min(C, w0 + 32);
    v.clear();
    for (int64_t i = w0; i < w1; ++i)
      for (int k = 0; k < 3; ++k)
        if (h.ct[3 * i + k] >= 0) v.push_back(h.ct[3 * i + k] >> 2);
    cost += 4. * (double)count_distinct(v);
    v.clear();
    for (int64_t i = w0; i < w1; ++i)
      for (int k = 0; k < 3; ++k) v.push_back(h.cn[3 * i + k] >> 2);
    cost += 2. * (double)count_distinct(v);
    v.clear();
    for (int64_t i = w0; i < w1; ++i)
      for (int k = 0; k < 3; ++k) v.push_back(h.ce[3 * i + k] >> 2);
    cost += 3. * (double)count_distinct(v);
  }
  // slot (k, cell) of an edge at one of its cells lives at k * C + cell
  auto slot_sector = [&](int64_t e, int64_t cell) -> int64_t {
    int k = 0;
    while (k < 2 && h.ce[3 * cell + k] != e) ++k;
    return ((int64_t)k << 40) | (cell >> 2);
  };
  for (int64_t e0 = 0; e0 < E; e0 += stride) {
    const int64_t e1 = std::min(E, e0 + 32);
    v.clear();
    for (int64_t e = e0; e < e1; ++e) {
      v.push_back(slot_sector(e, h.ec[2 * e]));
      if (h.ec[2 * e + 1] >= 0) v.push_back(slot_sector(e, h.ec[2 * e + 1]));
    }
    cost += 3. * (double)count_distinct(v);
  }
  return cost * scale;
}

Layout choose_layout(const HostInstance& h, int strategy, double* cost3, HostInstance* applied) {
  if (strategy != kLayoutAuto) {
    Layout L = make_layout(h, strategy);
    if (applied) *applied = apply_layout(h, L);
    return L;
  }
  Layout cand[3] = {Layout{}, make_layout(h, kLayoutMorton), make_layout(h, kLayoutRcm)};
  HostInstance inst[3];
  double cost[3];
  cost[0] = gather_sectors(h);
  for (int q = 1; q < 3; ++q) {
    inst[q] = apply_layout(h, cand[q]);
    cost[q] = gather_sectors(inst[q]);
  }
  if (cost3)
    for (int q = 0; q < 3; ++q) cost3[q] = cost[q];
  int best = cost[1] <= cost[2] ? 1 : 2;
  if (!(cost[best] < 0.95 * cost[0])) best = 0;
  if (applied) *applied = best ? std::move(inst[best]) : h;
  return std::move(cand[best]);
}

}  // namespace swe
