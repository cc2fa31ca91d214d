// mesh_prep.cpp -- see mesh_prep.hpp.
#include "mesh_prep.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <queue>

namespace aero {
namespace {

constexpr int kPadLink = -0x7fffffff;
constexpr int kMaxFacesPerCell = 32;

// Interleave the low 16 bits of x and y (x in even bit positions).
uint32_t morton2(uint32_t x, uint32_t y) {
  auto spread = [](uint32_t v) {
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
  };
  return spread(x) | (spread(y) << 1);
}

std::vector<int> morton_order(const aero_mesh_desc& m) {
  const int n = m.num_cells;
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  for (int c = 0; c < n; ++c) {
    x0 = std::min(x0, m.cell_center[3 * c]);
    x1 = std::max(x1, m.cell_center[3 * c]);
    y0 = std::min(y0, m.cell_center[3 * c + 1]);
    y1 = std::max(y1, m.cell_center[3 * c + 1]);
  }
  const double sx = (x1 > x0) ? 65535.0 / (x1 - x0) : 0.0;
  const double sy = (y1 > y0) ? 65535.0 / (y1 - y0) : 0.0;
  std::vector<uint64_t> key(static_cast<size_t>(n));
  for (int c = 0; c < n; ++c) {
    const auto qx = static_cast<uint32_t>(std::lround((m.cell_center[3 * c] - x0) * sx));
    const auto qy = static_cast<uint32_t>(std::lround((m.cell_center[3 * c + 1] - y0) * sy));
    key[c] = (static_cast<uint64_t>(morton2(qx, qy)) << 32) | static_cast<uint32_t>(c);
  }
  std::sort(key.begin(), key.end());
  std::vector<int> perm(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) perm[i] = static_cast<int>(key[i] & 0xffffffffu);
  return perm;
}

// Reverse Cuthill-McKee on the cell adjacency graph; each connected component starts from
// a minimum-degree cell, neighbours are visited in increasing degree.
std::vector<int> rcm_order(const aero_mesh_desc& m) {
  const int n = m.num_cells;
  std::vector<int> deg(static_cast<size_t>(n), 0);
  for (int f = 0; f < m.num_faces; ++f) {
    if (m.face_neighbor[f] >= 0) {
      ++deg[m.face_owner[f]];
      ++deg[m.face_neighbor[f]];
    }
  }
  std::vector<int> start(static_cast<size_t>(n) + 1, 0);
  for (int c = 0; c < n; ++c) start[c + 1] = start[c] + deg[c];
  std::vector<int> adj(static_cast<size_t>(start[n]));
  std::vector<int> fill(start.begin(), start.end() - 1);
  for (int f = 0; f < m.num_faces; ++f) {
    const int o = m.face_owner[f], b = m.face_neighbor[f];
    if (b >= 0) {
      adj[fill[o]++] = b;
      adj[fill[b]++] = o;
    }
  }
  std::vector<int> order;
  order.reserve(static_cast<size_t>(n));
  std::vector<char> seen(static_cast<size_t>(n), 0);
  std::vector<int> by_degree(static_cast<size_t>(n));
  std::iota(by_degree.begin(), by_degree.end(), 0);
  std::stable_sort(by_degree.begin(), by_degree.end(), [&](int a, int b) { return deg[a] < deg[b]; });
  std::vector<int> nb;
  for (int seed : by_degree) {
    if (seen[seed]) continue;
    std::queue<int> q;
    q.push(seed);
    seen[seed] = 1;
    while (!q.empty()) {
      const int c = q.front();
      q.pop();
      order.push_back(c);
      nb.assign(adj.begin() + start[c], adj.begin() + start[c + 1]);
      std::stable_sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
      for (int x : nb) {
        if (!seen[x]) {
          seen[x] = 1;
          q.push(x);
        }
      }
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

}  // namespace

bool build_slots(const aero_mesh_desc& m, int ordering, HostSlots* out, std::string* err) {
  const int n = m.num_cells, nf = m.num_faces;
  if (n <= 0 || nf <= 0) {
    *err = "mesh must contain cells and faces";
    return false;
  }
  if (n >= (1 << 30) || nf >= (1 << 30)) {  // cell and face ids are packed with a side bit
    *err = "mesh too large: cell and face counts must be below 2^30";
    return false;
  }
  if (!m.face_owner || !m.face_neighbor || !m.face_bc || !m.face_normal || !m.face_center ||
      !m.face_area || !m.cell_volume || !m.cell_center || (m.num_wall_faces > 0 && !m.wall_faces) ||
      m.num_wall_faces < 0) {
    *err = "mesh descriptor has a null array";
    return false;
  }
  std::vector<int> count(static_cast<size_t>(n), 0);
  int nint = 0;
  for (int f = 0; f < nf; ++f) {
    const int o = m.face_owner[f], b = m.face_neighbor[f];
    if (o < 0 || o >= n || b >= n || b < -1 || b == o) {
      *err = "face " + std::to_string(f) + " has an invalid owner/neighbour";
      return false;
    }
    if (b >= 0) {
      ++nint;
      ++count[b];
    } else if (m.face_bc[f] != AERO_BC_FARFIELD && m.face_bc[f] != AERO_BC_WALL) {
      *err = "boundary face " + std::to_string(f) + " has no far-field/wall type";
      return false;
    }
    ++count[o];
    const double a = m.face_area[f];
    if (!std::isfinite(a) || !std::isfinite(m.face_normal[3 * f]) || !std::isfinite(m.face_normal[3 * f + 1])) {
      *err = "face " + std::to_string(f) + " has non-finite geometry";
      return false;
    }
  }
  int d = 0;
  for (int c = 0; c < n; ++c) {
    d = std::max(d, count[c]);
    if (!std::isfinite(m.cell_volume[c])) {
      *err = "cell " + std::to_string(c) + " has a non-finite volume";
      return false;
    }
  }
  if (d > kMaxFacesPerCell) {
    *err = "a cell has more than 32 faces";
    return false;
  }
  for (int i = 0; i < m.num_wall_faces; ++i) {
    const int f = m.wall_faces[i];
    if (f < 0 || f >= nf || m.face_neighbor[f] >= 0) {
      *err = "wall face list contains an interior or out-of-range face";
      return false;
    }
  }

  HostSlots& s = *out;
  s = HostSlots();
  s.n = n;
  s.d = d;
  s.nf = nf;
  s.interior_faces = nint;
  s.boundary_faces = nf - nint;
  if (ordering == AERO_ORDER_MORTON) {
    s.perm = morton_order(m);
  } else if (ordering == AERO_ORDER_RCM) {
    s.perm = rcm_order(m);
  } else {
    s.perm.resize(static_cast<size_t>(n));
    std::iota(s.perm.begin(), s.perm.end(), 0);
  }
  if (ordering == AERO_ORDER_MORTON || ordering == AERO_ORDER_RCM) {
    // cells that own wall faces first (each group keeps the chosen order), so that the wall
    // force sums and monitors of the last RK stage come from a few thread blocks
    std::vector<unsigned char> owns(static_cast<size_t>(n), 0);
    for (int f = 0; f < nf; ++f) {
      if (m.face_neighbor[f] < 0 && m.face_bc[f] == AERO_BC_WALL) owns[m.face_owner[f]] = 1;
    }
    for (int i = 0; i < m.num_wall_faces; ++i) owns[m.face_owner[m.wall_faces[i]]] = 1;
    std::stable_partition(s.perm.begin(), s.perm.end(), [&](int c) { return owns[c] != 0; });
  }
  s.iperm.assign(static_cast<size_t>(n), -1);
  for (int i = 0; i < n; ++i) s.iperm[s.perm[i]] = i;

  // per original cell, its faces in ascending face order (CSR)
  std::vector<int> cstart(static_cast<size_t>(n) + 1, 0);
  for (int c = 0; c < n; ++c) cstart[c + 1] = cstart[c] + count[c];
  std::vector<int> cface(static_cast<size_t>(cstart[n]));
  std::vector<int> fill(cstart.begin(), cstart.end() - 1);
  for (int f = 0; f < nf; ++f) {
    cface[fill[m.face_owner[f]]++] = f;
    if (m.face_neighbor[f] >= 0) cface[fill[m.face_neighbor[f]]++] = f;
  }

  const size_t total = static_cast<size_t>(d) * n;
  s.link.assign(total, kPadLink);
  s.nx.assign(total, 0.0);
  s.ny.assign(total, 0.0);
  s.area.assign(total, 0.0);
  s.fcx.assign(total, 0.0);
  s.fcy.assign(total, 0.0);
  s.slot_face.assign(total, -1);
  s.own_old.assign(total, 0);
  s.nbr_old.assign(total, 0);
  s.vol.resize(static_cast<size_t>(n));
  s.flags.assign(static_cast<size_t>(n), 0);
  s.ccx.resize(static_cast<size_t>(n));
  s.ccy.resize(static_cast<size_t>(n));
  for (int c = 0; c < n; ++c) {
    s.ccx[c] = m.cell_center[3 * c];
    s.ccy[c] = m.cell_center[3 * c + 1];
  }
  for (int cn = 0; cn < n; ++cn) {
    const int co = s.perm[cn];
    s.vol[cn] = m.cell_volume[co];
    int k = 0;
    for (int j = cstart[co]; j < cstart[co + 1]; ++j, ++k) {
      const int f = cface[j];
      const size_t slot = static_cast<size_t>(k) * n + cn;
      const int o = m.face_owner[f], b = m.face_neighbor[f];
      if (b >= 0) {
        const int other = (o == co) ? b : o;
        const int side = (o == co) ? 0 : 1;
        s.link[slot] = (s.iperm[other] << 1) | side;
      } else {
        s.link[slot] = (m.face_bc[f] == AERO_BC_WALL) ? -2 : -1;
        s.flags[cn] |= (m.face_bc[f] == AERO_BC_WALL) ? 1 : 2;
      }
      s.nx[slot] = m.face_normal[3 * f];
      s.ny[slot] = m.face_normal[3 * f + 1];
      s.area[slot] = m.face_area[f];
      s.fcx[slot] = m.face_center[3 * f];
      s.fcy[slot] = m.face_center[3 * f + 1];
      s.slot_face[slot] = f;
      s.own_old[slot] = o;
      s.nbr_old[slot] = b >= 0 ? b : o;
    }
  }
  // face table sorted by new owner, and each cell's faces as gather slots in ascending
  // original face order (the order the reference sums them in)
  {
    std::vector<int> order(static_cast<size_t>(nf));
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return s.iperm[m.face_owner[a]] < s.iperm[m.face_owner[b]]; });
    std::vector<int> face_new(static_cast<size_t>(nf));
    s.f_orig = order;
    s.f_own.resize(static_cast<size_t>(nf));
    s.f_nb.resize(static_cast<size_t>(nf));
    s.f_own_old.resize(static_cast<size_t>(nf));
    s.f_nb_old.resize(static_cast<size_t>(nf));
    s.f_nx.resize(static_cast<size_t>(nf));
    s.f_ny.resize(static_cast<size_t>(nf));
    s.f_area.resize(static_cast<size_t>(nf));
    s.f_cx.resize(static_cast<size_t>(nf));
    s.f_cy.resize(static_cast<size_t>(nf));
    for (int i = 0; i < nf; ++i) {
      const int f = order[i];
      face_new[f] = i;
      const int o = m.face_owner[f], b = m.face_neighbor[f];
      s.f_own[i] = s.iperm[o];
      s.f_nb[i] = b >= 0 ? s.iperm[b] : (m.face_bc[f] == AERO_BC_WALL ? -2 : -1);
      s.f_own_old[i] = o;
      s.f_nb_old[i] = b >= 0 ? b : o;
      s.f_nx[i] = m.face_normal[3 * f];
      s.f_ny[i] = m.face_normal[3 * f + 1];
      s.f_area[i] = m.face_area[f];
      s.f_cx[i] = m.face_center[3 * f];
      s.f_cy[i] = m.face_center[3 * f + 1];
    }
    s.gslot.assign(total, kPadLink);
    for (int cn = 0; cn < n; ++cn) {
      const int co = s.perm[cn];
      int k = 0;
      for (int j = cstart[co]; j < cstart[co + 1]; ++j, ++k) {
        const int f = cface[j];
        s.gslot[static_cast<size_t>(k) * n + cn] = (face_new[f] << 1) | (m.face_owner[f] == co ? 0 : 1);
      }
    }
  }

  // wall entries: (new owner, face, kind); a slip-wall face listed in the patch is merged
  // into its monitor entry once, further listings get entries of their own
  struct WallEntry {
    int cell, face;
    unsigned char kind;
  };
  std::vector<WallEntry> we;
  std::vector<int> slip_entry(static_cast<size_t>(nf), -1);
  for (int f = 0; f < nf; ++f) {
    if (m.face_neighbor[f] >= 0 || m.face_bc[f] != AERO_BC_WALL) continue;
    slip_entry[f] = static_cast<int>(we.size());
    we.push_back({s.iperm[m.face_owner[f]], f, 2});
    ++s.n_slip;
  }
  for (int i = 0; i < m.num_wall_faces; ++i) {
    const int f = m.wall_faces[i];
    if (slip_entry[f] >= 0 && !(we[slip_entry[f]].kind & 1)) {
      we[slip_entry[f]].kind |= 1;
    } else {
      we.push_back({s.iperm[m.face_owner[f]], f, 1});
    }
    ++s.n_patch;
  }
  std::stable_sort(we.begin(), we.end(), [](const WallEntry& a, const WallEntry& b) {
    return a.cell != b.cell ? a.cell < b.cell : a.face < b.face;
  });
  s.wall_first.assign(static_cast<size_t>(n), 0);
  std::vector<int> per_cell(static_cast<size_t>(n), 0);
  for (size_t j = 0; j < we.size(); ++j) {
    const WallEntry& e = we[j];
    if (per_cell[e.cell]++ == 0) s.wall_first[e.cell] = static_cast<int>(j);
    s.wkind.push_back(e.kind);
    s.w_face.push_back(e.face);
    s.wnx.push_back(m.face_normal[3 * e.face]);
    s.wny.push_back(m.face_normal[3 * e.face + 1]);
    s.warea.push_back(m.face_area[e.face]);
    s.wx.push_back(m.face_center[3 * e.face]);
    s.wy.push_back(m.face_center[3 * e.face + 1]);
  }
  for (int c = 0; c < n; ++c) {
    if (per_cell[c] > 63) {
      *err = "a cell owns more than 63 wall faces";
      return false;
    }
    s.flags[c] = static_cast<unsigned char>(s.flags[c] | (per_cell[c] << 2));
  }
  return true;
}

void map_geometry(const aero_mesh_desc& m, const HostSlots& s, HostSlots* geo) {
  HostSlots& g = *geo;
  const size_t total = s.slot_face.size();
  g.nx.assign(total, 0.0);
  g.ny.assign(total, 0.0);
  g.area.assign(total, 0.0);
  g.fcx.assign(total, 0.0);
  g.fcy.assign(total, 0.0);
  for (size_t k = 0; k < total; ++k) {
    const int f = s.slot_face[k];
    if (f < 0) continue;
    g.nx[k] = m.face_normal[3 * f];
    g.ny[k] = m.face_normal[3 * f + 1];
    g.area[k] = m.face_area[f];
    g.fcx[k] = m.face_center[3 * f];
    g.fcy[k] = m.face_center[3 * f + 1];
  }
  g.vol.resize(static_cast<size_t>(s.n));
  g.ccx.resize(static_cast<size_t>(s.n));
  g.ccy.resize(static_cast<size_t>(s.n));
  for (int cn = 0; cn < s.n; ++cn) g.vol[cn] = m.cell_volume[s.perm[cn]];
  for (int c = 0; c < s.n; ++c) {
    g.ccx[c] = m.cell_center[3 * c];
    g.ccy[c] = m.cell_center[3 * c + 1];
  }
  const size_t nf = s.f_orig.size();
  g.f_nx.resize(nf);
  g.f_ny.resize(nf);
  g.f_area.resize(nf);
  g.f_cx.resize(nf);
  g.f_cy.resize(nf);
  for (size_t i = 0; i < nf; ++i) {
    const int f = s.f_orig[i];
    g.f_nx[i] = m.face_normal[3 * f];
    g.f_ny[i] = m.face_normal[3 * f + 1];
    g.f_area[i] = m.face_area[f];
    g.f_cx[i] = m.face_center[3 * f];
    g.f_cy[i] = m.face_center[3 * f + 1];
  }
  const size_t nw = s.w_face.size();
  g.wnx.resize(nw);
  g.wny.resize(nw);
  g.warea.resize(nw);
  g.wx.resize(nw);
  g.wy.resize(nw);
  for (size_t j = 0; j < nw; ++j) {
    const int f = s.w_face[j];
    g.wnx[j] = m.face_normal[3 * f];
    g.wny[j] = m.face_normal[3 * f + 1];
    g.warea[j] = m.face_area[f];
    g.wx[j] = m.face_center[3 * f];
    g.wy[j] = m.face_center[3 * f + 1];
  }
}

}  // namespace aero
