// oracle_capi.cpp -- TEST INFRASTRUCTURE ONLY.
//
// extern "C" entry points of the CPU oracle (liboracle.so), called by tests/ and by
// bench.py's CPU-baseline leg through ctypes. mode: 0 = float (the reference's
// arithmetic), 1 = double (FP64 oracle), 2 = float bulk with double accumulation.
#include "aero_oracle_driver.hpp"
#include "oracle_mesh.hpp"

#include <memory>
#include <new>

namespace {
struct Handle {
  int mode = 0;
  std::unique_ptr<aero_oracle::Solver<float, float>> f;
  std::unique_ptr<aero_oracle::Solver<double, double>> d;
  std::unique_ptr<aero_oracle::Solver<float, double>> m;
};

template <class Fn>
int dispatch(Handle* h, Fn&& fn) {
  if (h == nullptr) return AERO_ERR_INVALID;
  switch (h->mode) {
    case 0: return fn(*h->f);
    case 1: return fn(*h->d);
    default: return fn(*h->m);
  }
}

bool valid_mesh(const aero_mesh_desc* m) {
  return m != nullptr && m->num_cells > 0 && m->num_faces > 0 && m->face_owner && m->face_neighbor &&
         m->face_bc && m->face_normal && m->face_center && m->face_area && m->cell_volume &&
         m->cell_center && (m->num_wall_faces == 0 || m->wall_faces);
}
}  // namespace

extern "C" {

void* oracle_solver_create(int mode, const aero_mesh_desc* mesh, const aero_case_desc* cfg) {
  if (!valid_mesh(mesh) || cfg == nullptr || mode < 0 || mode > 2) return nullptr;
  Handle* h = new (std::nothrow) Handle();
  if (h == nullptr) return nullptr;
  h->mode = mode;
  if (mode == 0) h->f.reset(new aero_oracle::Solver<float, float>(*mesh, *cfg));
  if (mode == 1) h->d.reset(new aero_oracle::Solver<double, double>(*mesh, *cfg));
  if (mode == 2) h->m.reset(new aero_oracle::Solver<float, double>(*mesh, *cfg));
  return h;
}

void oracle_solver_destroy(void* h) { delete static_cast<Handle*>(h); }

int oracle_solver_set_state(void* h, const double* u) {
  return dispatch(static_cast<Handle*>(h), [&](auto& s) {
    s.set_state(u);
    return 0;
  });
}

int oracle_solver_get_state(void* h, double* u) {
  return dispatch(static_cast<Handle*>(h), [&](auto& s) {
    s.get_state(u);
    return 0;
  });
}

int oracle_solver_last_residual(void* h, double* r, double* sr) {
  return dispatch(static_cast<Handle*>(h), [&](auto& s) {
    s.last_residual(r, sr);
    return 0;
  });
}

int oracle_solver_reset_run(void* h) {
  return dispatch(static_cast<Handle*>(h), [&](auto& s) {
    s.reset_run();
    return 0;
  });
}

int oracle_solver_run(void* h, int n, aero_iter_record* recs, int* n_done) {
  return dispatch(static_cast<Handle*>(h), [&](auto& s) { return s.run(n, recs, n_done); });
}

// One residual evaluation (gradients + assembly) on the conserved state u [N][5].
// diag receives {first-order fallback faces, diffusive fallback faces, first failure face};
// fscale (may be null) receives per cell and component sum_faces |F_k A| (parity metric).
int oracle_solver_residual(void* h, const double* u, int second_order, double stab, int as_fix,
                           double as_fmin, double as_ramp, double* res, double* sr, double* grad,
                           int* diag, double* fscale) {
  return dispatch(static_cast<Handle*>(h), [&](auto& s) {
    s.residual(u, second_order, stab, as_fix, as_fmin, as_ramp, res, sr, grad, diag, fscale);
    return 0;
  });
}

// Synthetic benchmark O-grid (oracle_mesh.hpp). Returns a handle (null on a bad spec) whose
// sizes oracle_mesh_sizes gives as {cells, faces, wall faces} and whose arrays
// oracle_mesh_copy writes into caller buffers of those sizes.
void* oracle_mesh_ogrid(int n_circ, int n_radial, int cell_type, int permute, double chord, double thickness,
                        double wall_spacing, double farfield_radius, double jitter, unsigned long long seed) {
  try {
    return new oracle_mesh::Ogrid(oracle_mesh::ogrid_synthetic(n_circ, n_radial, cell_type, permute != 0, chord,
                                                               thickness, wall_spacing, farfield_radius, jitter,
                                                               seed));
  } catch (...) {
    return nullptr;
  }
}

void oracle_mesh_sizes(const void* h, int* sizes) {
  const auto* g = static_cast<const oracle_mesh::Ogrid*>(h);
  sizes[0] = g->num_cells;
  sizes[1] = g->num_faces;
  sizes[2] = static_cast<int>(g->wall_faces.size());
}

void oracle_mesh_copy(const void* h, int* owner, int* neighbor, int* bc, double* normal, double* center,
                      double* area, double* volume, double* cell_center, int* wall_faces) {
  const auto* g = static_cast<const oracle_mesh::Ogrid*>(h);
  std::copy(g->owner.begin(), g->owner.end(), owner);
  std::copy(g->neighbor.begin(), g->neighbor.end(), neighbor);
  std::copy(g->bc.begin(), g->bc.end(), bc);
  std::copy(g->normal.begin(), g->normal.end(), normal);
  std::copy(g->center.begin(), g->center.end(), center);
  std::copy(g->area.begin(), g->area.end(), area);
  std::copy(g->volume.begin(), g->volume.end(), volume);
  std::copy(g->cell_center.begin(), g->cell_center.end(), cell_center);
  std::copy(g->wall_faces.begin(), g->wall_faces.end(), wall_faces);
}

void oracle_mesh_free(void* h) { delete static_cast<oracle_mesh::Ogrid*>(h); }

}  // extern "C"
