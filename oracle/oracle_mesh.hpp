// TEST INFRASTRUCTURE ONLY. Synthetic benchmark O-grid for the CPU arms of the benchmark,
// so that the oracle's timed runs build their workload mesh without the product library.
//
// The construction is the benchmark's (it has no counterpart in AeroCFD): closed-trailing-
// edge NACA 00xx contour sampled at n_circ angles (x = (1 + cos theta) / 2, i.e. cosine
// clustering at the leading and trailing edges), straight radial lines from each wall point
// to a far-field circle of radius R centred at mid-chord with a prescribed first spacing and
// per-line geometric growth, seeded jitter of interior nodes, quads or triangles with a
// seeded diagonal, then seeded permutations of the cells and of the faces within the
// interior / wall / far-field blocks. Random numbers come from SplitMix64 and are drawn in
// the same order as the product generator (aero_mesh_ogrid_synthetic) draws them, so both
// produce the same mesh; the CPU tests check that bit for bit. Face geometry follows the
// reference's convention (unit normal pointing out of the owner, mesh_geometry.cpp:49-80).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <unordered_map>
#include <vector>

namespace oracle_mesh {

struct Ogrid {
  int num_cells = 0, num_faces = 0;
  std::vector<int> owner, neighbor, bc, wall_faces;
  std::vector<double> normal, center, area, volume, cell_center;
};

class Rng64 {  // SplitMix64 (Steele, Lea, Flood 2014)
 public:
  explicit Rng64(uint64_t seed) : state_(seed) {}
  uint64_t bits() {
    state_ += 0x9e3779b97f4a7c15ull;
    uint64_t z = state_;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double unit() { return static_cast<double>(bits() >> 11) * 0x1.0p-53; }
  // Fisher-Yates from the back, swapping k with a draw in [0, k]
  template <class T>
  void shuffle(std::vector<T>& v) {
    for (size_t k = v.size(); k-- > 1;) std::swap(v[k], v[bits() % static_cast<uint64_t>(k + 1)]);
  }

 private:
  uint64_t state_;
};

// NACA 00xx with the closed trailing edge, each term evaluated left to right as written
inline double half_thickness(double x, double t) {
  const double s = std::min(std::max(x, 0.0), 1.0);
  return 5.0 * t * (0.2969 * std::sqrt(s) - 0.1260 * s - 0.3516 * s * s + 0.2843 * s * s * s -
                    0.1036 * s * s * s * s);
}

// q > 1 with h0 (q^n - 1) / (q - 1) = L by bisection (q = 1 when uniform spacing reaches L)
inline double stretch_ratio(double h0, double L, int n) {
  if (h0 * n >= L) return 1.0;
  const auto span = [&](double q) { return h0 * (std::pow(q, n) - 1.0) / (q - 1.0); };
  double a = 1.0 + 1e-12, b = 4.0;
  while (span(b) < L) b *= 2.0;
  for (int k = 0; k < 200; ++k) {
    const double m = 0.5 * (a + b);
    (span(m) < L ? a : b) = m;
  }
  return 0.5 * (a + b);
}

inline Ogrid ogrid_synthetic(int nt, int nr, int cell_type, bool permute, double chord, double thickness,
                             double wall_spacing, double farfield_radius, double jitter, uint64_t seed) {
  if (nt < 8 || nr < 2 || (cell_type != 3 && cell_type != 4)) throw std::invalid_argument("bad O-grid spec");
  const double c = chord > 0.0 ? chord : 1.0;
  const double R = farfield_radius * c, xc = 0.5 * c;
  const double pi = 3.14159265358979323846;
  Rng64 rng(seed * 0x2545F4914F6CDD1Dull + 1);
  const int npts = nt * (nr + 1);
  std::vector<double> X(npts), Y(npts);
  const auto node = [nt](int i, int j) { return j * nt + ((i % nt) + nt) % nt; };

  // radial lines: wall point -> far-field point, geometric spacing from the wall
  for (int i = 0; i < nt; ++i) {
    const double th = 2.0 * pi * i / nt;
    const double xw = 0.5 * (1.0 + std::cos(th));
    const double t = half_thickness(xw, thickness);
    const double ax = xw * c, ay = (th < pi ? t : (th > pi ? -t : 0.0)) * c;
    const double bx = xc + R * std::cos(th), by = R * std::sin(th);
    const double len = std::hypot(bx - ax, by - ay);
    const double q = stretch_ratio(wall_spacing * c, len, nr);
    double s = 0.0, h = wall_spacing * c;
    for (int j = 0; j <= nr; ++j) {
      const double f = j == nr ? 1.0 : s / len;
      X[node(i, j)] = ax + f * (bx - ax);
      Y[node(i, j)] = ay + f * (by - ay);
      s += h;
      h *= q;
    }
  }
  if (jitter > 0.0) {  // displacements drawn on the unjittered grid, then applied together
    std::vector<double> dx(npts, 0.0), dy(npts, 0.0);
    for (int j = 1; j < nr; ++j) {
      for (int i = 0; i < nt; ++i) {
        const int k = node(i, j);
        double hmin = 1e300;
        for (int b : {node(i + 1, j), node(i - 1, j), node(i, j + 1), node(i, j - 1)})
          hmin = std::min(hmin, std::hypot(X[b] - X[k], Y[b] - Y[k]));
        dx[k] = jitter * hmin * (2.0 * rng.unit() - 1.0);
        dy[k] = jitter * hmin * (2.0 * rng.unit() - 1.0);
      }
    }
    for (int k = 0; k < npts; ++k) {
      X[k] += dx[k];
      Y[k] += dy[k];
    }
  }

  // cells in generation order, vertices counter-clockwise
  std::vector<std::vector<int>> gen;
  const auto add = [&](std::vector<int> v) {
    double a2 = 0.0;
    for (size_t e = 0; e < v.size(); ++e) {
      const int p = v[e], q = v[(e + 1) % v.size()];
      a2 += X[p] * Y[q] - X[q] * Y[p];
    }
    if (a2 < 0.0) std::reverse(v.begin(), v.end());
    gen.push_back(std::move(v));
  };
  for (int j = 0; j < nr; ++j) {
    for (int i = 0; i < nt; ++i) {
      const int a = node(i, j), b = node(i + 1, j), d = node(i + 1, j + 1), e = node(i, j + 1);
      if (cell_type == 4) {
        add({a, b, d, e});
      } else if (rng.bits() & 1u) {
        add({a, b, d});
        add({a, d, e});
      } else {
        add({a, b, e});
        add({b, d, e});
      }
    }
  }
  const int N = static_cast<int>(gen.size());
  std::vector<int> perm(N);  // perm[new id] = generation index
  for (int k = 0; k < N; ++k) perm[k] = k;
  if (permute) rng.shuffle(perm);

  Ogrid g;
  g.num_cells = N;
  g.volume.resize(N);
  g.cell_center.assign(3 * static_cast<size_t>(N), 0.0);
  for (int k = 0; k < N; ++k) {
    const std::vector<int>& v = gen[perm[k]];
    double a2 = 0.0, mx = 0.0, my = 0.0;
    for (size_t e = 0; e < v.size(); ++e) {
      const int p = v[e], q = v[(e + 1) % v.size()];
      const double cr = X[p] * Y[q] - X[q] * Y[p];
      a2 += cr;
      mx += (X[p] + X[q]) * cr;
      my += (Y[p] + Y[q]) * cr;
    }
    if (!(a2 > 0.0)) throw std::runtime_error("inverted cell");
    g.volume[k] = 0.5 * a2;
    if (v.size() == 3) {  // vertex mean of a triangle
      g.cell_center[3 * k] = (X[v[0]] + X[v[1]] + X[v[2]]) / 3.0;
      g.cell_center[3 * k + 1] = (Y[v[0]] + Y[v[1]] + Y[v[2]]) / 3.0;
    } else {  // area centroid of a polygon
      g.cell_center[3 * k] = mx / (3.0 * a2);
      g.cell_center[3 * k + 1] = my / (3.0 * a2);
    }
  }

  // faces: first appearance of an edge makes the owner, the second the neighbour
  struct Edge {
    int owner, neighbor, v0, v1;
  };
  std::vector<Edge> edges;
  std::unordered_map<uint64_t, int> index;
  index.reserve(4 * static_cast<size_t>(N));
  for (int k = 0; k < N; ++k) {
    const std::vector<int>& v = gen[perm[k]];
    for (size_t e = 0; e < v.size(); ++e) {
      const int p = v[e], q = v[(e + 1) % v.size()];
      const uint64_t key = (static_cast<uint64_t>(static_cast<uint32_t>(std::min(p, q))) << 32) |
                           static_cast<uint32_t>(std::max(p, q));
      const auto [it, fresh] = index.try_emplace(key, static_cast<int>(edges.size()));
      if (fresh) edges.push_back({k, -1, p, q});
      else edges[it->second].neighbor = k;
    }
  }
  std::vector<int> blocks[3];  // interior, wall (both vertices on ring 0), far field
  for (int f = 0; f < static_cast<int>(edges.size()); ++f) {
    const Edge& e = edges[f];
    blocks[e.neighbor >= 0 ? 0 : ((e.v0 < nt && e.v1 < nt) ? 1 : 2)].push_back(f);
  }
  if (permute)
    for (auto& b : blocks) rng.shuffle(b);
  const int F = static_cast<int>(edges.size());
  g.num_faces = F;
  g.owner.resize(F);
  g.neighbor.resize(F);
  g.bc.assign(F, 0);
  g.normal.assign(3 * static_cast<size_t>(F), 0.0);
  g.center.assign(3 * static_cast<size_t>(F), 0.0);
  g.area.resize(F);
  const int bc_code[3] = {0, 2, 1};  // face_bc: 0 interior, 1 far field, 2 wall
  int out = 0;
  for (int b = 0; b < 3; ++b) {
    for (int f : blocks[b]) {
      const Edge& e = edges[f];
      g.owner[out] = e.owner;
      g.neighbor[out] = e.neighbor;
      g.bc[out] = bc_code[b];
      if (b == 1) g.wall_faces.push_back(out);
      const double ex = X[e.v1] - X[e.v0], ey = Y[e.v1] - Y[e.v0];
      const double len = std::hypot(ex, ey);
      if (!(len > 0.0)) throw std::runtime_error("degenerate face");
      g.normal[3 * out] = ey / len;
      g.normal[3 * out + 1] = -ex / len;
      g.area[out] = len;
      g.center[3 * out] = 0.5 * (X[e.v0] + X[e.v1]);
      g.center[3 * out + 1] = 0.5 * (Y[e.v0] + Y[e.v1]);
      ++out;
    }
  }
  return g;
}

}  // namespace oracle_mesh
