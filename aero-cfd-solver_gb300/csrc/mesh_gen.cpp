// mesh_gen.cpp -- host mesh generators (include/aero_mesh.h).
#include "../../include/aero_mesh.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <exception>
#include <map>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

struct aero_mesh {
  int nc = 0, nf = 0, np = 0;
  std::vector<int> owner, neighbor, bc, face_vertices, conn, offsets, wall_faces, farfield_faces;
  std::vector<unsigned char> types;
  std::vector<double> normal, center, area, volume, cell_center, points;
};

namespace {

thread_local std::string g_mesh_error;

// ---------------------------------------------------------------------------------------
// Reference O-grid, float arithmetic (src/cfd_core/mesh/airfoil_mesh.cpp).
// ---------------------------------------------------------------------------------------
using P2 = std::array<float, 2>;
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kEpsF = 1.0e-7f;

float dist2(const P2& a, const P2& b) {
  const float dx = a[0] - b[0];
  const float dy = a[1] - b[1];
  return dx * dx + dy * dy;
}

// airfoil_mesh.cpp:42-56
float signed_area(const std::vector<P2>& p) {
  if (p.size() < 3) return 0.0f;
  double a2 = 0.0;
  for (size_t i = 0; i < p.size(); ++i) {
    const size_t j = (i + 1) % p.size();
    a2 += static_cast<double>(p[i][0]) * static_cast<double>(p[j][1]) -
          static_cast<double>(p[j][0]) * static_cast<double>(p[i][1]);
  }
  return static_cast<float>(0.5 * a2);
}

// airfoil_mesh.cpp:64-78
std::vector<P2> drop_duplicates(const std::vector<P2>& in) {
  std::vector<P2> out;
  out.reserve(in.size());
  for (const P2& p : in) {
    if (!out.empty() && dist2(out.back(), p) < 1.0e-12f) continue;
    out.push_back(p);
  }
  if (out.size() >= 2 && dist2(out.front(), out.back()) < 1.0e-12f) out.pop_back();
  return out;
}

// airfoil_mesh.cpp:80-120: uniform arc-length resampling of a closed curve
std::vector<P2> resample(const std::vector<P2>& in, int count) {
  if (count < 8) throw std::invalid_argument("Target curve resolution must be >= 8.");
  const std::vector<P2> p = drop_duplicates(in);
  if (p.size() < 8) throw std::invalid_argument("Airfoil contour has too few points.");
  const size_t n = p.size();
  std::vector<float> cum(n + 1, 0.0f);
  for (size_t i = 0; i < n; ++i) cum[i + 1] = cum[i] + std::sqrt(dist2(p[i], p[(i + 1) % n]));
  const float total = cum.back();
  if (total < kEpsF) throw std::invalid_argument("Airfoil contour has near-zero length.");
  std::vector<P2> out;
  out.reserve(static_cast<size_t>(count));
  size_t seg = 0;
  for (int k = 0; k < count; ++k) {
    const float target = total * static_cast<float>(k) / static_cast<float>(count);
    while (seg + 1 < cum.size() && cum[seg + 1] < target) ++seg;
    const size_t a = seg % n, b = (seg + 1) % n;
    const float t = (target - cum[seg]) / std::max(cum[seg + 1] - cum[seg], kEpsF);
    out.push_back({p[a][0] + t * (p[b][0] - p[a][0]), p[a][1] + t * (p[b][1] - p[a][1])});
  }
  return out;
}

// airfoil_mesh.cpp:395-457
std::vector<P2> naca4_contour(const std::string& code, int n_circ, float chord) {
  if (chord <= 0.0f) throw std::invalid_argument("Airfoil chord must be positive.");
  std::string dg;
  for (char ch : code) {
    if (ch >= '0' && ch <= '9') dg.push_back(ch);
  }
  if (dg.size() < 4) throw std::invalid_argument("NACA code must contain four digits.");
  const float m = static_cast<float>(dg[0] - '0') / 100.0f;
  const float pc = static_cast<float>(dg[1] - '0') / 10.0f;
  const float t = static_cast<float>(10 * (dg[2] - '0') + (dg[3] - '0')) / 100.0f;
  const int pps = std::max(16, n_circ / 2 + 1);
  std::vector<P2> up(static_cast<size_t>(pps)), lo(static_cast<size_t>(pps));
  for (int i = 0; i < pps; ++i) {
    const float beta = kPiF * static_cast<float>(i) / static_cast<float>(pps - 1);
    const float x = 0.5f * (1.0f - std::cos(beta));
    const float sx = std::sqrt(std::max(x, 0.0f));
    const float yt = 5.0f * t *
                     (0.2969f * sx - 0.1260f * x - 0.3516f * x * x + 0.2843f * x * x * x -
                      0.1036f * x * x * x * x);
    float yc = 0.0f, dyc = 0.0f;
    if (m > 0.0f && pc > 0.0f && pc < 1.0f) {
      if (x < pc) {
        yc = m / (pc * pc) * (2.0f * pc * x - x * x);
        dyc = 2.0f * m / (pc * pc) * (pc - x);
      } else {
        const float q = 1.0f - pc;
        yc = m / (q * q) * (1.0f - 2.0f * pc + 2.0f * pc * x - x * x);
        dyc = 2.0f * m / (q * q) * (pc - x);
      }
    }
    const float th = std::atan(dyc);
    up[i] = {(x - yt * std::sin(th)) * chord, (yc + yt * std::cos(th)) * chord};
    lo[i] = {(x + yt * std::sin(th)) * chord, (yc - yt * std::cos(th)) * chord};
  }
  std::vector<P2> contour;
  contour.reserve(static_cast<size_t>(2 * pps - 1));
  for (int i = pps - 1; i >= 0; --i) contour.push_back(up[i]);
  for (int i = 1; i < pps; ++i) contour.push_back(lo[i]);
  if (signed_area(contour) < 0.0f) std::reverse(contour.begin(), contour.end());
  return resample(contour, std::max(32, n_circ));
}

uint64_t edge_key(int a, int b) {
  const uint32_t lo = static_cast<uint32_t>(std::min(a, b)), hi = static_cast<uint32_t>(std::max(a, b));
  return (static_cast<uint64_t>(lo) << 32) | hi;
}

// airfoil_mesh.cpp:184-392 (triangles, float geometry) + mesh_geometry.cpp:49-80 (normals)
aero_mesh* reference_triangle_mesh(const std::vector<P2>& pts, std::vector<std::array<int, 3>> tris,
                                   const std::map<uint64_t, std::string>& edge_patch) {
  auto* m = new aero_mesh();
  m->nc = static_cast<int>(tris.size());
  m->np = static_cast<int>(pts.size());
  for (auto& tr : tris) {
    const P2 &a = pts[tr[0]], &b = pts[tr[1]], &c = pts[tr[2]];
    if ((b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]) < 0.0f) std::swap(tr[1], tr[2]);
  }
  m->volume.resize(m->nc);
  m->cell_center.assign(3 * static_cast<size_t>(m->nc), 0.0);
  for (int c = 0; c < m->nc; ++c) {
    const P2 &a = pts[tris[c][0]], &b = pts[tris[c][1]], &d = pts[tris[c][2]];
    const float a2 = (b[0] - a[0]) * (d[1] - a[1]) - (b[1] - a[1]) * (d[0] - a[0]);
    const float area = 0.5f * std::abs(a2);
    if (area < kEpsF) throw std::runtime_error("Degenerate triangle detected while building airfoil mesh.");
    m->volume[c] = area;
    m->cell_center[3 * c] = (a[0] + b[0] + d[0]) / 3.0f;
    m->cell_center[3 * c + 1] = (a[1] + b[1] + d[1]) / 3.0f;
  }
  struct Face {
    int owner, neighbor, v0, v1;
    float nx, ny, len;
  };
  std::vector<Face> faces;
  faces.reserve(static_cast<size_t>(m->nc) * 2);
  std::unordered_map<uint64_t, int> seen;
  seen.reserve(static_cast<size_t>(m->nc) * 3);
  for (int c = 0; c < m->nc; ++c) {
    const auto& t = tris[c];
    const int ev[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
    for (const auto& e : ev) {
      const uint64_t key = edge_key(e[0], e[1]);
      auto it = seen.find(key);
      if (it == seen.end()) {
        const float dx = pts[e[1]][0] - pts[e[0]][0];
        const float dy = pts[e[1]][1] - pts[e[0]][1];
        const float len = std::sqrt(dx * dx + dy * dy);
        if (len < kEpsF) throw std::runtime_error("Degenerate face detected while building airfoil mesh.");
        seen.emplace(key, static_cast<int>(faces.size()));
        faces.push_back({c, -1, e[0], e[1], dy / len, -dx / len, len});
      } else {
        faces[it->second].neighbor = c;
      }
    }
  }
  std::vector<int> order;
  std::map<std::string, std::vector<int>> bnd;
  for (int f = 0; f < static_cast<int>(faces.size()); ++f) {
    if (faces[f].neighbor >= 0) {
      order.push_back(f);
      continue;
    }
    auto it = edge_patch.find(edge_key(faces[f].v0, faces[f].v1));
    bnd[it == edge_patch.end() ? std::string("boundary") : it->second].push_back(f);
  }
  const char* first[4] = {"wall", "farfield", "wake", "cut"};
  std::vector<std::pair<std::string, std::vector<int>>> patches;
  for (const char* name : first) {
    auto it = bnd.find(name);
    if (it != bnd.end()) patches.emplace_back(it->first, it->second);
  }
  for (const auto& kv : bnd) {
    bool listed = false;
    for (const char* name : first) listed = listed || kv.first == name;
    if (!listed) patches.emplace_back(kv.first, kv.second);
  }
  for (const auto& pt : patches) {
    for (int f : pt.second) {
      if (pt.first == "wall") m->wall_faces.push_back(static_cast<int>(order.size()));
      else m->farfield_faces.push_back(static_cast<int>(order.size()));
      order.push_back(f);
    }
  }
  m->nf = static_cast<int>(order.size());
  m->owner.resize(m->nf);
  m->neighbor.resize(m->nf);
  m->bc.resize(m->nf);
  m->face_vertices.resize(2 * static_cast<size_t>(m->nf));
  m->normal.assign(3 * static_cast<size_t>(m->nf), 0.0);
  m->center.assign(3 * static_cast<size_t>(m->nf), 0.0);
  m->area.resize(m->nf);
  for (int nf = 0; nf < m->nf; ++nf) {
    const Face& s = faces[order[nf]];
    m->owner[nf] = s.owner;
    m->neighbor[nf] = s.neighbor;
    m->face_vertices[2 * nf] = s.v0;
    m->face_vertices[2 * nf + 1] = s.v1;
    // normalize_face_normals (mesh_geometry.cpp:49-80), tolerance 1e-5
    float nx = s.nx, ny = s.ny;
    const float norm = std::sqrt(nx * nx + ny * ny + 0.0f * 0.0f);
    if (!std::isfinite(norm) || norm < 1.0e-12f) {
      nx = 1.0f;
      ny = 0.0f;
    } else if (std::abs(norm - 1.0f) > 1.0e-5f) {
      const float inv = 1.0f / norm;
      nx *= inv;
      ny *= inv;
    }
    m->normal[3 * nf] = nx;
    m->normal[3 * nf + 1] = ny;
    m->area[nf] = s.len;
    m->center[3 * nf] = 0.5f * (pts[s.v0][0] + pts[s.v1][0]);
    m->center[3 * nf + 1] = 0.5f * (pts[s.v0][1] + pts[s.v1][1]);
  }
  for (int f : m->wall_faces) m->bc[f] = AERO_BC_WALL;
  for (int f : m->farfield_faces) m->bc[f] = AERO_BC_FARFIELD;
  m->points.assign(3 * static_cast<size_t>(m->np), 0.0);
  for (int i = 0; i < m->np; ++i) {
    m->points[3 * i] = pts[i][0];
    m->points[3 * i + 1] = pts[i][1];
  }
  int off = 0;
  for (const auto& t : tris) {
    m->conn.insert(m->conn.end(), t.begin(), t.end());
    off += 3;
    m->offsets.push_back(off);
    m->types.push_back(5);
  }
  return m;
}

// airfoil_mesh.cpp:459-544
aero_mesh* reference_ogrid(const std::string& code, int n_circ, int n_radial, float radius, float stretch_in,
                           float chord) {
  if (n_circ < 32) throw std::invalid_argument("num_circumferential must be >= 32.");
  if (n_radial < 4) throw std::invalid_argument("num_radial must be >= 4.");
  std::vector<P2> contour = naca4_contour(code, n_circ, chord);
  if (signed_area(contour) < 0.0f) std::reverse(contour.begin(), contour.end());
  P2 ctr{0.0f, 0.0f};
  for (const P2& p : contour) {
    ctr[0] += p[0];
    ctr[1] += p[1];
  }
  ctr[0] /= static_cast<float>(contour.size());
  ctr[1] /= static_cast<float>(contour.size());
  const float rff = std::max(radius, 2.5f) * chord;
  const float stretch = std::max(stretch_in, 1.0f);
  const int nt = n_circ, nr = n_radial;
  std::vector<P2> pts;
  pts.reserve(static_cast<size_t>((nr + 1) * nt));
  for (int j = 0; j <= nr; ++j) {
    const float eta = static_cast<float>(j) / static_cast<float>(nr);
    float sigma = eta;
    if (stretch > 1.0f + 1.0e-4f) sigma = (std::pow(stretch, eta) - 1.0f) / (stretch - 1.0f);
    for (int i = 0; i < nt; ++i) {
      const P2& in = contour[i];
      float dx = in[0] - ctr[0], dy = in[1] - ctr[1];
      float r = std::sqrt(dx * dx + dy * dy);
      if (r < kEpsF) {
        dx = 1.0f;
        dy = 0.0f;
        r = 1.0f;
      }
      const float inv = 1.0f / r;
      const float ox = ctr[0] + dx * inv * rff;
      const float oy = ctr[1] + dy * inv * rff;
      pts.push_back({in[0] + sigma * (ox - in[0]), in[1] + sigma * (oy - in[1])});
    }
  }
  std::vector<std::array<int, 3>> tris;
  tris.reserve(2 * static_cast<size_t>(nt) * nr);
  for (int j = 0; j < nr; ++j) {
    for (int i = 0; i < nt; ++i) {
      const int i1 = (i + 1) % nt;
      const int a = j * nt + i, b = j * nt + i1, c = (j + 1) * nt + i1, d = (j + 1) * nt + i;
      tris.push_back({a, b, c});
      tris.push_back({a, c, d});
    }
  }
  std::map<uint64_t, std::string> patch;
  for (int i = 0; i < nt; ++i) {
    const int i1 = (i + 1) % nt;
    patch.emplace(edge_key(i, i1), "wall");
    patch.emplace(edge_key(nr * nt + i, nr * nt + i1), "farfield");
  }
  return reference_triangle_mesh(pts, tris, patch);
}

// ---------------------------------------------------------------------------------------
// Synthetic benchmark O-grid, double arithmetic.
// ---------------------------------------------------------------------------------------
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
};

double naca00_half_thickness(double x, double t) {
  x = std::min(std::max(x, 0.0), 1.0);
  return 5.0 * t * (0.2969 * std::sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x - 0.1036 * x * x * x * x);
}

// Geometric ratio q with h0 * (q^n - 1) / (q - 1) = L (q > 1), by bisection.
double growth_ratio(double h0, double L, int n) {
  if (h0 * n >= L) return 1.0;
  double lo = 1.0 + 1e-12, hi = 4.0;
  auto total = [&](double q) { return h0 * (std::pow(q, n) - 1.0) / (q - 1.0); };
  while (total(hi) < L) hi *= 2.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (total(mid) < L) lo = mid;
    else hi = mid;
  }
  return 0.5 * (lo + hi);
}

aero_mesh* synthetic_ogrid(const aero_ogrid_spec& s) {
  const int nt = s.n_circ, nr = s.n_radial;
  if (nt < 8 || nr < 2) throw std::invalid_argument("synthetic O-grid needs n_circ >= 8 and n_radial >= 2");
  if (s.cell_type != 3 && s.cell_type != 4) throw std::invalid_argument("cell_type must be 3 or 4");
  const double c = s.chord > 0.0 ? s.chord : 1.0;
  const double R = s.farfield_radius * c;
  const double cx = 0.5 * c, cy = 0.0;
  const double pi = 3.14159265358979323846;
  SplitMix rng{s.seed * 0x2545F4914F6CDD1Dull + 1};
  std::vector<double> px(static_cast<size_t>(nt) * (nr + 1)), py(px.size());
  auto id = [nt](int i, int j) { return j * nt + ((i % nt) + nt) % nt; };
  for (int i = 0; i < nt; ++i) {
    const double th = 2.0 * pi * i / nt;
    const double x = 0.5 * (1.0 + std::cos(th));
    const double yt = naca00_half_thickness(x, s.thickness);
    const double wx = x * c, wy = (th < pi ? yt : (th > pi ? -yt : 0.0)) * c;
    const double qx = cx + R * std::cos(th), qy = cy + R * std::sin(th);
    const double L = std::hypot(qx - wx, qy - wy);
    const double q = growth_ratio(s.wall_spacing * c, L, nr);
    double dist = 0.0, h = s.wall_spacing * c;
    for (int j = 0; j <= nr; ++j) {
      const double f = (j == nr) ? 1.0 : dist / L;
      px[id(i, j)] = wx + f * (qx - wx);
      py[id(i, j)] = wy + f * (qy - wy);
      dist += h;
      h *= q;
    }
  }
  if (s.jitter > 0.0) {
    std::vector<double> jx(px.size(), 0.0), jy(px.size(), 0.0);
    for (int j = 1; j < nr; ++j) {
      for (int i = 0; i < nt; ++i) {
        const int k = id(i, j);
        double hmin = 1e300;
        const int nb[4] = {id(i + 1, j), id(i - 1, j), id(i, j + 1), id(i, j - 1)};
        for (int b : nb) hmin = std::min(hmin, std::hypot(px[b] - px[k], py[b] - py[k]));
        jx[k] = s.jitter * hmin * (2.0 * rng.uniform() - 1.0);
        jy[k] = s.jitter * hmin * (2.0 * rng.uniform() - 1.0);
      }
    }
    for (size_t k = 0; k < px.size(); ++k) {
      px[k] += jx[k];
      py[k] += jy[k];
    }
  }
  // cells, counter-clockwise
  std::vector<std::vector<int>> cells;
  cells.reserve(static_cast<size_t>(nt) * nr * (s.cell_type == 3 ? 2 : 1));
  auto ccw = [&](std::vector<int> v) {
    double a2 = 0.0;
    for (size_t k = 0; k < v.size(); ++k) {
      const int p = v[k], q = v[(k + 1) % v.size()];
      a2 += px[p] * py[q] - px[q] * py[p];
    }
    if (a2 < 0.0) std::reverse(v.begin(), v.end());
    return v;
  };
  for (int j = 0; j < nr; ++j) {
    for (int i = 0; i < nt; ++i) {
      const int a = id(i, j), b = id(i + 1, j), cc = id(i + 1, j + 1), d = id(i, j + 1);
      if (s.cell_type == 4) {
        cells.push_back(ccw({a, b, cc, d}));
      } else if (rng.next() & 1u) {
        cells.push_back(ccw({a, b, cc}));
        cells.push_back(ccw({a, cc, d}));
      } else {
        cells.push_back(ccw({a, b, d}));
        cells.push_back(ccw({b, cc, d}));
      }
    }
  }
  const int ncell = static_cast<int>(cells.size());
  std::vector<int> cperm(static_cast<size_t>(ncell));
  for (int k = 0; k < ncell; ++k) cperm[k] = k;
  if (s.permute) {
    for (int k = ncell - 1; k > 0; --k) std::swap(cperm[k], cperm[rng.next() % static_cast<uint64_t>(k + 1)]);
  }
  // cperm[new] = generation index
  std::vector<std::vector<int>> ordered(static_cast<size_t>(ncell));
  for (int k = 0; k < ncell; ++k) ordered[k] = cells[cperm[k]];
  auto* m = new aero_mesh();
  m->nc = ncell;
  m->np = static_cast<int>(px.size());
  m->volume.resize(ncell);
  m->cell_center.assign(3 * static_cast<size_t>(ncell), 0.0);
  for (int k = 0; k < ncell; ++k) {
    const auto& v = ordered[k];
    double a2 = 0.0, sx = 0.0, sy = 0.0;
    for (size_t e = 0; e < v.size(); ++e) {
      const int p = v[e], q = v[(e + 1) % v.size()];
      const double cr = px[p] * py[q] - px[q] * py[p];
      a2 += cr;
      sx += (px[p] + px[q]) * cr;
      sy += (py[p] + py[q]) * cr;
    }
    if (!(a2 > 0.0)) throw std::runtime_error("synthetic O-grid produced an inverted cell");
    m->volume[k] = 0.5 * a2;
    if (v.size() == 3) {
      m->cell_center[3 * k] = (px[v[0]] + px[v[1]] + px[v[2]]) / 3.0;
      m->cell_center[3 * k + 1] = (py[v[0]] + py[v[1]] + py[v[2]]) / 3.0;
    } else {
      m->cell_center[3 * k] = sx / (3.0 * a2);
      m->cell_center[3 * k + 1] = sy / (3.0 * a2);
    }
    m->conn.insert(m->conn.end(), v.begin(), v.end());
    m->offsets.push_back(static_cast<int>(m->conn.size()));
    m->types.push_back(v.size() == 3 ? 5 : 9);
  }
  struct Face {
    int owner, neighbor, v0, v1;
  };
  std::vector<Face> faces;
  std::unordered_map<uint64_t, int> seen;
  seen.reserve(static_cast<size_t>(ncell) * 4);
  for (int k = 0; k < ncell; ++k) {
    const auto& v = ordered[k];
    for (size_t e = 0; e < v.size(); ++e) {
      const int p = v[e], q = v[(e + 1) % v.size()];
      const uint64_t key = edge_key(p, q);
      auto it = seen.find(key);
      if (it == seen.end()) {
        seen.emplace(key, static_cast<int>(faces.size()));
        faces.push_back({k, -1, p, q});
      } else {
        faces[it->second].neighbor = k;
      }
    }
  }
  std::vector<int> interior, wall, farfield;
  for (int f = 0; f < static_cast<int>(faces.size()); ++f) {
    if (faces[f].neighbor >= 0) {
      interior.push_back(f);
    } else if (faces[f].v0 < nt && faces[f].v1 < nt) {
      wall.push_back(f);
    } else {
      farfield.push_back(f);
    }
  }
  if (s.permute) {
    for (auto* blk : {&interior, &wall, &farfield}) {
      for (int k = static_cast<int>(blk->size()) - 1; k > 0; --k)
        std::swap((*blk)[k], (*blk)[rng.next() % static_cast<uint64_t>(k + 1)]);
    }
  }
  std::vector<int> order;
  order.insert(order.end(), interior.begin(), interior.end());
  for (size_t k = 0; k < wall.size(); ++k) m->wall_faces.push_back(static_cast<int>(order.size() + k));
  order.insert(order.end(), wall.begin(), wall.end());
  for (size_t k = 0; k < farfield.size(); ++k) m->farfield_faces.push_back(static_cast<int>(order.size() + k));
  order.insert(order.end(), farfield.begin(), farfield.end());
  m->nf = static_cast<int>(order.size());
  m->owner.resize(m->nf);
  m->neighbor.resize(m->nf);
  m->bc.assign(m->nf, AERO_BC_INTERIOR);
  m->face_vertices.resize(2 * static_cast<size_t>(m->nf));
  m->normal.assign(3 * static_cast<size_t>(m->nf), 0.0);
  m->center.assign(3 * static_cast<size_t>(m->nf), 0.0);
  m->area.resize(m->nf);
  for (int nf = 0; nf < m->nf; ++nf) {
    const Face& fc = faces[order[nf]];
    m->owner[nf] = fc.owner;
    m->neighbor[nf] = fc.neighbor;
    m->face_vertices[2 * nf] = fc.v0;
    m->face_vertices[2 * nf + 1] = fc.v1;
    const double dx = px[fc.v1] - px[fc.v0], dy = py[fc.v1] - py[fc.v0];
    const double len = std::hypot(dx, dy);
    if (!(len > 0.0)) throw std::runtime_error("synthetic O-grid produced a degenerate face");
    m->normal[3 * nf] = dy / len;
    m->normal[3 * nf + 1] = -dx / len;
    m->area[nf] = len;
    m->center[3 * nf] = 0.5 * (px[fc.v0] + px[fc.v1]);
    m->center[3 * nf + 1] = 0.5 * (py[fc.v0] + py[fc.v1]);
  }
  for (int f : m->wall_faces) m->bc[f] = AERO_BC_WALL;
  for (int f : m->farfield_faces) m->bc[f] = AERO_BC_FARFIELD;
  m->points.assign(3 * px.size(), 0.0);
  for (size_t k = 0; k < px.size(); ++k) {
    m->points[3 * k] = px[k];
    m->points[3 * k + 1] = py[k];
  }
  return m;
}

// ---------------------------------------------------------------------------------------
// Geometry from node coordinates (the synthetic generator's double formulas) and its
// tangent along a node displacement, through one template on the scalar type.
// ---------------------------------------------------------------------------------------
struct Tan {  // value and one directional derivative
  double v, d;
};
inline Tan operator+(Tan a, Tan b) { return {a.v + b.v, a.d + b.d}; }
inline Tan operator-(Tan a, Tan b) { return {a.v - b.v, a.d - b.d}; }
inline Tan operator*(Tan a, Tan b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Tan operator*(double a, Tan b) { return {a * b.v, a * b.d}; }
inline Tan operator/(Tan a, Tan b) {
  const double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
inline Tan operator/(Tan a, double b) { return {a.v / b, a.d / b}; }
inline Tan operator-(Tan a) { return {-a.v, -a.d}; }
inline double val(double x) { return x; }
inline double val(Tan x) { return x.v; }
inline double hyp(double x, double y) { return std::hypot(x, y); }
inline Tan hyp(Tan x, Tan y) {
  const double h = std::hypot(x.v, y.v);
  return {h, h > 0.0 ? (x.v * x.d + y.v * y.d) / h : 0.0};
}

template <class S>
void node_geometry(const aero_mesh& m, const std::vector<S>& px, const std::vector<S>& py, std::vector<S>* normal,
                   std::vector<S>* center, std::vector<S>* area, std::vector<S>* volume,
                   std::vector<S>* cell_center) {
  volume->assign(static_cast<size_t>(m.nc), S{});
  cell_center->assign(3 * static_cast<size_t>(m.nc), S{});
  for (int k = 0; k < m.nc; ++k) {
    const int b = k == 0 ? 0 : m.offsets[k - 1], e = m.offsets[k], nv = e - b;
    S a2{}, sx{}, sy{};
    for (int j = 0; j < nv; ++j) {
      const int p = m.conn[b + j], q = m.conn[b + (j + 1) % nv];
      const S cr = px[p] * py[q] - px[q] * py[p];
      a2 = a2 + cr;
      sx = sx + (px[p] + px[q]) * cr;
      sy = sy + (py[p] + py[q]) * cr;
    }
    if (!(val(a2) > 0.0)) throw std::runtime_error("inverted or degenerate cell " + std::to_string(k));
    (*volume)[k] = 0.5 * a2;
    if (nv == 3) {
      const int v0 = m.conn[b], v1 = m.conn[b + 1], v2 = m.conn[b + 2];
      (*cell_center)[3 * k] = (px[v0] + px[v1] + px[v2]) / 3.0;
      (*cell_center)[3 * k + 1] = (py[v0] + py[v1] + py[v2]) / 3.0;
    } else {
      (*cell_center)[3 * k] = sx / (3.0 * a2);
      (*cell_center)[3 * k + 1] = sy / (3.0 * a2);
    }
  }
  normal->assign(3 * static_cast<size_t>(m.nf), S{});
  center->assign(3 * static_cast<size_t>(m.nf), S{});
  area->assign(static_cast<size_t>(m.nf), S{});
  for (int f = 0; f < m.nf; ++f) {
    const int v0 = m.face_vertices[2 * f], v1 = m.face_vertices[2 * f + 1];
    const S dx = px[v1] - px[v0], dy = py[v1] - py[v0];
    const S len = hyp(dx, dy);
    if (!(val(len) > 0.0)) throw std::runtime_error("degenerate face " + std::to_string(f));
    (*normal)[3 * f] = dy / len;
    (*normal)[3 * f + 1] = -dx / len;
    (*area)[f] = len;
    (*center)[3 * f] = 0.5 * (px[v0] + px[v1]);
    (*center)[3 * f + 1] = 0.5 * (py[v0] + py[v1]);
  }
}

// Transpose of node_geometry's derivative: from the derivatives of a scalar with respect to
// the face normals [3F], face centres [3F], face lengths [F], cell volumes [N] and cell centres
// [3N], its derivatives with respect to the node coordinates bp [3P] (z entries 0). Reverse
// mode of the same formulas, one pass over cells and faces.
void node_geometry_vjp(const aero_mesh& m, const double* bn, const double* bc, const double* ba, const double* bv,
                       const double* bcc, double* bp) {
  const std::vector<double>& P = m.points;
  std::fill(bp, bp + 3 * static_cast<size_t>(m.np), 0.0);
  for (int k = 0; k < m.nc; ++k) {
    const int b = k == 0 ? 0 : m.offsets[k - 1], e = m.offsets[k], nv = e - b;
    double a2 = 0.0, sx = 0.0, sy = 0.0;
    for (int j = 0; j < nv; ++j) {
      const int p = m.conn[b + j], q = m.conn[b + (j + 1) % nv];
      const double cr = P[3 * p] * P[3 * q + 1] - P[3 * q] * P[3 * p + 1];
      a2 += cr;
      sx += (P[3 * p] + P[3 * q]) * cr;
      sy += (P[3 * p + 1] + P[3 * q + 1]) * cr;
    }
    double ba2 = 0.5 * bv[k], bsx = 0.0, bsy = 0.0;  // volume = a2 / 2
    if (nv == 3) {  // centre = vertex mean
      for (int j = 0; j < 3; ++j) {
        const int v = m.conn[b + j];
        bp[3 * v] += bcc[3 * k] / 3.0;
        bp[3 * v + 1] += bcc[3 * k + 1] / 3.0;
      }
    } else {  // centre = (sx, sy) / (3 a2)
      bsx = bcc[3 * k] / (3.0 * a2);
      bsy = bcc[3 * k + 1] / (3.0 * a2);
      ba2 -= (bcc[3 * k] * sx + bcc[3 * k + 1] * sy) / (3.0 * a2 * a2);
    }
    for (int j = 0; j < nv; ++j) {
      const int p = m.conn[b + j], q = m.conn[b + (j + 1) % nv];
      const double xp = P[3 * p], yp = P[3 * p + 1], xq = P[3 * q], yq = P[3 * q + 1];
      const double cr = xp * yq - xq * yp;
      const double bcr = ba2 + bsx * (xp + xq) + bsy * (yp + yq);
      bp[3 * p] += bsx * cr + bcr * yq;
      bp[3 * q] += bsx * cr - bcr * yp;
      bp[3 * p + 1] += bsy * cr - bcr * xq;
      bp[3 * q + 1] += bsy * cr + bcr * xp;
    }
  }
  for (int f = 0; f < m.nf; ++f) {
    const int v0 = m.face_vertices[2 * f], v1 = m.face_vertices[2 * f + 1];
    const double dx = P[3 * v1] - P[3 * v0], dy = P[3 * v1 + 1] - P[3 * v0 + 1];
    const double len = std::hypot(dx, dy), l3 = len * len * len;
    // normal = (dy, -dx) / len, length = len, centre = (p0 + p1) / 2
    const double bnx = bn[3 * f], bny = bn[3 * f + 1];
    const double bdx = bnx * (-dy * dx / l3) + bny * (-dy * dy / l3) + ba[f] * dx / len;
    const double bdy = bnx * (dx * dx / l3) + bny * (dx * dy / l3) + ba[f] * dy / len;
    bp[3 * v1] += bdx + 0.5 * bc[3 * f];
    bp[3 * v0] += -bdx + 0.5 * bc[3 * f];
    bp[3 * v1 + 1] += bdy + 0.5 * bc[3 * f + 1];
    bp[3 * v0 + 1] += -bdy + 0.5 * bc[3 * f + 1];
  }
}

// Hicks-Henne bump on [0, 1]: sin(pi x^(ln 0.5 / ln peak))^width, 0 at both ends.
double hicks_henne(double x, double peak, double width) {
  if (!(x > 0.0) || !(x < 1.0)) return 0.0;
  const double e = std::log(0.5) / std::log(peak);
  const double s = std::sin(3.14159265358979323846 * std::pow(x, e));
  return std::pow(std::max(s, 0.0), width);
}

// Displacement modes of n bumps: the wall nodes move in y by the bump of their side of the
// airfoil (unit amplitude), the far-field nodes stay, every other node moves by the
// inverse-distance-weighted mean (weights |x - x_s|^-3) of those boundary displacements.
void hicks_henne_modes(const aero_mesh& m, int n, const double* peak, const int* upper, double width,
                       double* modes) {
  const int np = m.np;
  std::vector<char> kind(static_cast<size_t>(np), 0);  // 1 wall, 2 far field
  for (int f : m.wall_faces) {
    kind[m.face_vertices[2 * f]] = 1;
    kind[m.face_vertices[2 * f + 1]] = 1;
  }
  for (int f = 0; f < m.nf; ++f) {
    if (m.neighbor[f] < 0 && m.bc[f] == AERO_BC_FARFIELD) {
      for (int s = 0; s < 2; ++s) {
        if (kind[m.face_vertices[2 * f + s]] == 0) kind[m.face_vertices[2 * f + s]] = 2;
      }
    }
  }
  std::vector<int> wall, src;
  for (int p = 0; p < np; ++p) {
    if (kind[p] == 1) wall.push_back(p);
    if (kind[p] != 0) src.push_back(p);
  }
  if (wall.empty()) throw std::invalid_argument("mesh has no wall patch");
  double x0 = 1e300, x1 = -1e300;
  for (int p : wall) {
    x0 = std::min(x0, m.points[3 * p]);
    x1 = std::max(x1, m.points[3 * p]);
  }
  const double chord = x1 - x0;
  if (!(chord > 0.0)) throw std::invalid_argument("wall patch has no chord");
  // boundary displacements per source node and bump
  std::vector<double> sd(src.size() * static_cast<size_t>(n), 0.0);
  for (size_t s = 0; s < src.size(); ++s) {
    const int p = src[s];
    if (kind[p] != 1) continue;
    const double xi = (m.points[3 * p] - x0) / chord, y = m.points[3 * p + 1];
    for (int k = 0; k < n; ++k) {
      const bool on = upper[k] ? y > 0.0 : y < 0.0;
      if (on) sd[s * n + k] = hicks_henne(xi, peak[k], width);
    }
  }
  const size_t stride = 3 * static_cast<size_t>(np);
  std::fill(modes, modes + stride * n, 0.0);
  auto work = [&](int p_begin, int p_end) {
    std::vector<double> acc(static_cast<size_t>(n));
    for (int p = p_begin; p < p_end; ++p) {
      if (kind[p] == 1) {
        const size_t s = static_cast<size_t>(std::lower_bound(src.begin(), src.end(), p) - src.begin());
        for (int k = 0; k < n; ++k) modes[k * stride + 3 * p + 1] = sd[s * n + k];
        continue;
      }
      if (kind[p] == 2) continue;
      const double x = m.points[3 * p], y = m.points[3 * p + 1];
      double wsum = 0.0;
      std::fill(acc.begin(), acc.end(), 0.0);
      for (size_t s = 0; s < src.size(); ++s) {
        const int q = src[s];
        const double dx = x - m.points[3 * q], dy = y - m.points[3 * q + 1];
        const double d2 = dx * dx + dy * dy;
        const double w = 1.0 / (d2 * std::sqrt(d2));
        wsum += w;
        if (kind[q] == 1) {
          for (int k = 0; k < n; ++k) acc[k] += w * sd[s * n + k];
        }
      }
      for (int k = 0; k < n; ++k) modes[k * stride + 3 * p + 1] = acc[k] / wsum;
    }
  };
  const int threads = static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
  std::vector<std::thread> pool;
  const int chunk = (np + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int b = t * chunk, e = std::min(np, b + chunk);
    if (b < e) pool.emplace_back(work, b, e);
  }
  for (auto& th : pool) th.join();
}

template <class Fn>
int guarded(Fn&& fn) {
  try {
    fn();
    return AERO_OK;
  } catch (const std::bad_alloc&) {
    g_mesh_error = "host allocation failed";
    return AERO_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_mesh_error = e.what();
    return AERO_ERR_INVALID;
  }
}

}  // namespace

extern "C" {

int aero_mesh_ogrid_reference(const char* naca_code, int n_circ, int n_radial, double farfield_radius,
                              double radial_stretch, double chord, aero_mesh** out) {
  if (out == nullptr || naca_code == nullptr) {
    g_mesh_error = "null argument";
    return AERO_ERR_INVALID;
  }
  *out = nullptr;
  return guarded([&] {
    *out = reference_ogrid(naca_code, n_circ, n_radial, static_cast<float>(farfield_radius),
                           static_cast<float>(radial_stretch), static_cast<float>(chord));
  });
}

int aero_mesh_ogrid_synthetic(const aero_ogrid_spec* spec, aero_mesh** out) {
  if (out == nullptr || spec == nullptr) {
    g_mesh_error = "null argument";
    return AERO_ERR_INVALID;
  }
  *out = nullptr;
  return guarded([&] { *out = synthetic_ogrid(*spec); });
}

void aero_mesh_free(aero_mesh* m) { delete m; }

const char* aero_mesh_last_error(void) { return g_mesh_error.c_str(); }

int aero_mesh_get_sizes(const aero_mesh* m, aero_mesh_sizes* s) {
  if (m == nullptr || s == nullptr) return AERO_ERR_INVALID;
  s->num_cells = m->nc;
  s->num_faces = m->nf;
  s->num_points = m->np;
  s->num_wall_faces = static_cast<int>(m->wall_faces.size());
  s->num_farfield_faces = static_cast<int>(m->farfield_faces.size());
  s->conn_length = static_cast<int>(m->conn.size());
  return AERO_OK;
}

int aero_mesh_describe(const aero_mesh* m, aero_mesh_desc* d) {
  if (m == nullptr || d == nullptr) return AERO_ERR_INVALID;
  d->num_cells = m->nc;
  d->num_faces = m->nf;
  d->face_owner = m->owner.data();
  d->face_neighbor = m->neighbor.data();
  d->face_bc = m->bc.data();
  d->face_normal = m->normal.data();
  d->face_center = m->center.data();
  d->face_area = m->area.data();
  d->cell_volume = m->volume.data();
  d->cell_center = m->cell_center.data();
  d->num_wall_faces = static_cast<int>(m->wall_faces.size());
  d->wall_faces = m->wall_faces.data();
  return AERO_OK;
}

int aero_mesh_clone(const aero_mesh* m, aero_mesh** out) {
  if (m == nullptr || out == nullptr) {
    g_mesh_error = "null argument";
    return AERO_ERR_INVALID;
  }
  *out = nullptr;
  return guarded([&] { *out = new aero_mesh(*m); });
}

int aero_mesh_set_points(aero_mesh* m, const double* points) {
  if (m == nullptr || points == nullptr) {
    g_mesh_error = "null argument";
    return AERO_ERR_INVALID;
  }
  return guarded([&] {
    std::vector<double> px(static_cast<size_t>(m->np)), py(px.size());
    for (int p = 0; p < m->np; ++p) {
      px[p] = points[3 * p];
      py[p] = points[3 * p + 1];
    }
    std::vector<double> normal, center, area, volume, cc;
    node_geometry(*m, px, py, &normal, &center, &area, &volume, &cc);
    m->points.assign(points, points + 3 * static_cast<size_t>(m->np));
    m->normal.swap(normal);
    m->center.swap(center);
    m->area.swap(area);
    m->volume.swap(volume);
    m->cell_center.swap(cc);
  });
}

int aero_mesh_geometry_tangent(const aero_mesh* m, const double* dpoints, double* d_normal, double* d_center,
                               double* d_area, double* d_volume, double* d_cell_center) {
  if (m == nullptr || dpoints == nullptr || !d_normal || !d_center || !d_area || !d_volume || !d_cell_center) {
    g_mesh_error = "null argument";
    return AERO_ERR_INVALID;
  }
  return guarded([&] {
    std::vector<Tan> px(static_cast<size_t>(m->np)), py(px.size());
    for (int p = 0; p < m->np; ++p) {
      px[p] = Tan{m->points[3 * p], dpoints[3 * p]};
      py[p] = Tan{m->points[3 * p + 1], dpoints[3 * p + 1]};
    }
    std::vector<Tan> normal, center, area, volume, cc;
    node_geometry(*m, px, py, &normal, &center, &area, &volume, &cc);
    for (size_t i = 0; i < normal.size(); ++i) d_normal[i] = normal[i].d;
    for (size_t i = 0; i < center.size(); ++i) d_center[i] = center[i].d;
    for (size_t i = 0; i < area.size(); ++i) d_area[i] = area[i].d;
    for (size_t i = 0; i < volume.size(); ++i) d_volume[i] = volume[i].d;
    for (size_t i = 0; i < cc.size(); ++i) d_cell_center[i] = cc[i].d;
  });
}

int aero_mesh_geometry_vjp(const aero_mesh* m, const double* b_normal, const double* b_center, const double* b_area,
                           const double* b_volume, const double* b_cell_center, double* b_points) {
  if (m == nullptr || !b_normal || !b_center || !b_area || !b_volume || !b_cell_center || !b_points) {
    g_mesh_error = "null argument";
    return AERO_ERR_INVALID;
  }
  return guarded([&] { node_geometry_vjp(*m, b_normal, b_center, b_area, b_volume, b_cell_center, b_points); });
}

int aero_mesh_hicks_henne_modes(const aero_mesh* m, int n_bumps, const double* peak_x, const int* upper,
                                double width_exponent, double* modes) {
  if (m == nullptr || n_bumps <= 0 || peak_x == nullptr || upper == nullptr || modes == nullptr ||
      !(width_exponent > 0.0)) {
    g_mesh_error = "bad argument";
    return AERO_ERR_INVALID;
  }
  for (int k = 0; k < n_bumps; ++k) {
    if (!(peak_x[k] > 0.0 && peak_x[k] < 1.0)) {
      g_mesh_error = "bump peaks must lie in (0, 1)";
      return AERO_ERR_INVALID;
    }
  }
  return guarded([&] { hicks_henne_modes(*m, n_bumps, peak_x, upper, width_exponent, modes); });
}

int aero_mesh_get_aux(const aero_mesh* m, double* points, int* face_vertices, int* conn, int* offsets,
                      unsigned char* types, int* farfield_faces) {
  if (m == nullptr) return AERO_ERR_INVALID;
  if (points) std::copy(m->points.begin(), m->points.end(), points);
  if (face_vertices) std::copy(m->face_vertices.begin(), m->face_vertices.end(), face_vertices);
  if (conn) std::copy(m->conn.begin(), m->conn.end(), conn);
  if (offsets) std::copy(m->offsets.begin(), m->offsets.end(), offsets);
  if (types) std::copy(m->types.begin(), m->types.end(), types);
  if (farfield_faces) std::copy(m->farfield_faces.begin(), m->farfield_faces.end(), farfield_faces);
  return AERO_OK;
}

}  // extern "C"
