// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// extern "C" adapter around the reference AeroCFD library compiled from its own
// sources (recipe: oracle/Makefile, output oracle/_ref/libaero_ref.so). It lets the
// golden-vector script and the oracle tests drive the reference's own functions:
//   - make_airfoil_ogrid_mesh (src/cfd_core/mesh/airfoil_mesh.cpp:459-544) and
//     make_demo_tri_mesh_2x2 (src/cfd_core/mesh/mesh.cpp:44) to export meshes;
//   - compute_green_gauss_gradients + assemble_euler_residual_cpu
//     (reconstruction.cpp:73, residual_assembly.cpp:73) on an injected mesh;
//   - run_euler_airfoil_case_cpu (euler_solver.cpp:1489) for whole-run histories.
// Nothing here is linked into the product library.
#include "cfd_core/mesh.hpp"
#include "cfd_core/mesh/airfoil_mesh.hpp"
#include "cfd_core/numerics/euler_flux.hpp"
#include "cfd_core/numerics/reconstruction.hpp"
#include "cfd_core/solvers/euler/mesh_geometry.hpp"
#include "cfd_core/solvers/euler/preconditioning.hpp"
#include "cfd_core/solvers/euler/residual_assembly.hpp"
#include "cfd_core/solvers/euler_solver.hpp"

#include "../include/aero_gb300.h"

#include <cmath>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

using namespace cfd::core;

namespace {
UnstructuredMesh g_mesh;
std::string g_error;

UnstructuredMesh from_desc(const aero_mesh_desc& d) {
  UnstructuredMesh m;
  m.dimension = 2;
  m.num_cells = d.num_cells;
  m.num_faces = d.num_faces;
  m.face_owner.assign(d.face_owner, d.face_owner + d.num_faces);
  m.face_neighbor.assign(d.face_neighbor, d.face_neighbor + d.num_faces);
  m.face_vertices.assign(2 * static_cast<size_t>(d.num_faces), 0);
  for (int i = 0; i < 3 * d.num_faces; ++i) {
    m.face_normal.push_back(static_cast<float>(d.face_normal[i]));
    m.face_center.push_back(static_cast<float>(d.face_center[i]));
  }
  for (int f = 0; f < d.num_faces; ++f) m.face_area.push_back(static_cast<float>(d.face_area[f]));
  for (int c = 0; c < d.num_cells; ++c) m.cell_volume.push_back(static_cast<float>(d.cell_volume[c]));
  for (int i = 0; i < 3 * d.num_cells; ++i)
    m.cell_center.push_back(static_cast<float>(d.cell_center[i]));
  return m;
}

void fill_config(const aero_case_desc& c, EulerAirfoilCaseConfig* e) {
  e->iterations = c.iterations;
  e->min_iterations = c.min_iterations;
  e->cfl_ramp_iters = c.cfl_ramp_iters;
  e->gamma = static_cast<float>(c.gamma);
  e->gas_constant = static_cast<float>(c.gas_constant);
  e->mach = static_cast<float>(c.mach);
  e->aoa_deg = static_cast<float>(c.aoa_deg);
  e->p_inf = static_cast<float>(c.p_inf);
  e->t_inf = static_cast<float>(c.t_inf);
  e->rho_inf = static_cast<float>(c.rho_inf);
  e->cfl_start = static_cast<float>(c.cfl_start);
  e->cfl_max = static_cast<float>(c.cfl_max);
  e->residual_reduction_target = static_cast<float>(c.residual_reduction_target);
  e->force_stability_tol = static_cast<float>(c.force_stability_tol);
  e->force_stability_window = c.force_stability_window;
  e->force_mean_drift_tol = static_cast<float>(c.force_mean_drift_tol);
  e->startup_first_order_iters = c.startup_first_order_iters;
  e->rk_stages = c.rk_stages;
  e->local_time_stepping = c.local_time_stepping != 0;
  e->precond_on = c.precond_on != 0;
  e->precond_mach_ref = static_cast<float>(c.precond_mach_ref);
  e->precond_mach_min = static_cast<float>(c.precond_mach_min);
  e->precond_beta_min = static_cast<float>(c.precond_beta_min);
  e->precond_beta_max = static_cast<float>(c.precond_beta_max);
  e->precond_farfield_bc = c.precond_farfield_bc != 0;
  e->stabilization_mach_floor_start = static_cast<float>(c.stab_floor_start);
  e->stabilization_mach_floor_target = static_cast<float>(c.stab_floor_target);
  e->stabilization_mach_floor_k_start = static_cast<float>(c.stab_floor_k_start);
  e->stabilization_mach_floor_k_target = static_cast<float>(c.stab_floor_k_target);
  e->stabilization_ramp_iters = c.stab_ramp_iters;
  e->x_ref = static_cast<float>(c.x_ref);
  e->y_ref = static_cast<float>(c.y_ref);
  e->flux_scheme = c.flux == AERO_FLUX_HLLC ? EulerFluxScheme::kHllc : EulerFluxScheme::kRusanov;
  e->limiter = c.limiter == AERO_LIMITER_VENKAT ? LimiterType::kVenkat : LimiterType::kMinmod;
  e->low_mach_fix = c.low_mach_fix != 0;
  e->mach_cutoff = static_cast<float>(c.mach_cutoff);
  e->all_speed_flux_fix = c.all_speed_flux_fix != 0;
  e->all_speed_mach_cutoff = static_cast<float>(c.all_speed_mach_cutoff);
  e->all_speed_f_min = static_cast<float>(c.all_speed_f_min);
  e->all_speed_ramp_start_iter = c.all_speed_ramp_start_iter;
  e->all_speed_ramp_iters = c.all_speed_ramp_iters;
  e->all_speed_staged_controller = c.all_speed_staged_controller != 0;
  e->all_speed_stage_a_min_iters = c.all_speed_stage_a_min_iters;
  e->all_speed_stage_a_max_iters = c.all_speed_stage_a_max_iters;
  e->all_speed_stage_f_min_high = static_cast<float>(c.all_speed_stage_f_min_high);
  e->all_speed_stage_f_min_mid = static_cast<float>(c.all_speed_stage_f_min_mid);
  e->all_speed_stage_f_min_low = static_cast<float>(c.all_speed_stage_f_min_low);
  e->all_speed_pjump_wall_target = static_cast<float>(c.all_speed_pjump_wall_target);
  e->all_speed_pjump_spike_factor = static_cast<float>(c.all_speed_pjump_spike_factor);
  e->all_speed_pjump_hold_iters = c.all_speed_pjump_hold_iters;
  e->all_speed_freeze_iters = c.all_speed_freeze_iters;
  e->all_speed_cfl_drop_factor = static_cast<float>(c.all_speed_cfl_drop_factor);
  e->all_speed_cfl_restore_factor = static_cast<float>(c.all_speed_cfl_restore_factor);
  e->all_speed_cfl_min_scale = static_cast<float>(c.all_speed_cfl_min_scale);
  e->aoa0_symmetry_enforce = c.aoa0_symmetry_enforce != 0;
  e->aoa0_symmetry_enforce_interval = c.aoa0_symmetry_enforce_interval;
}
}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

// Build the reference O-grid into the shim's current mesh; returns 0 on success.
int ref_ogrid_build(const char* naca, int n_circ, int n_radial, double farfield_radius,
                    double stretch, double chord) {
  try {
    AirfoilMeshConfig c;
    c.naca_code = naca;
    c.num_circumferential = n_circ;
    c.num_radial = n_radial;
    c.farfield_radius = static_cast<float>(farfield_radius);
    c.radial_stretch = static_cast<float>(stretch);
    c.chord = static_cast<float>(chord);
    g_mesh = make_airfoil_ogrid_mesh(c);
    normalize_face_normals(&g_mesh);
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

int ref_demo_mesh_build() {
  g_mesh = make_demo_tri_mesh_2x2();
  return 0;
}

// sizes[0..3] = cells, faces, points, patches
void ref_mesh_sizes(int* sizes) {
  sizes[0] = g_mesh.num_cells;
  sizes[1] = g_mesh.num_faces;
  sizes[2] = static_cast<int>(g_mesh.points.size() / 3);
  sizes[3] = static_cast<int>(g_mesh.boundary_patches.size());
}

// Copies the current mesh. bc receives the reference's boundary types
// (build_euler_boundary_types, mesh_geometry.cpp:82-104); patch_info receives
// (start, count, is_wall) per patch; conn receives 3 vertex ids per cell.
void ref_mesh_get(int* owner, int* neighbor, int* bc, int* face_vertices, float* normal,
                  float* center, float* area, float* volume, float* cell_center, float* points,
                  int* conn, int* patch_info) {
  const UnstructuredMesh& m = g_mesh;
  const std::vector<EulerBoundaryConditionType> bt = build_euler_boundary_types(m);
  for (int f = 0; f < m.num_faces; ++f) {
    owner[f] = m.face_owner[f];
    neighbor[f] = m.face_neighbor[f];
    bc[f] = static_cast<int>(bt[f]);
    face_vertices[2 * f] = m.face_vertices[2 * f];
    face_vertices[2 * f + 1] = m.face_vertices[2 * f + 1];
    area[f] = m.face_area[f];
  }
  std::memcpy(normal, m.face_normal.data(), sizeof(float) * m.face_normal.size());
  std::memcpy(center, m.face_center.data(), sizeof(float) * m.face_center.size());
  std::memcpy(volume, m.cell_volume.data(), sizeof(float) * m.cell_volume.size());
  std::memcpy(cell_center, m.cell_center.data(), sizeof(float) * m.cell_center.size());
  std::memcpy(points, m.points.data(), sizeof(float) * m.points.size());
  if (!m.cell_connectivity.empty())
    std::memcpy(conn, m.cell_connectivity.data(), sizeof(int) * m.cell_connectivity.size());
  for (size_t i = 0; i < m.boundary_patches.size(); ++i) {
    patch_info[3 * i] = m.boundary_patches[i].start_face;
    patch_info[3 * i + 1] = m.boundary_patches[i].face_count;
    patch_info[3 * i + 2] = m.boundary_patches[i].name == "wall" ? 1 : 0;
  }
}

// Residual of one stage on an injected mesh through the reference's own functions.
// The precondition parameters are used as given (they are the resolved values).
int ref_residual(const aero_mesh_desc* md, const aero_case_desc* c, const double* u,
                 int second_order, double stab, int as_fix, double as_fmin, double as_ramp,
                 double* res, double* sr, double* grad, int* diag) {
  try {
    const UnstructuredMesh m = from_desc(*md);
    const float gamma = static_cast<float>(c->gamma);
    std::vector<PrimitiveState> prim(static_cast<size_t>(m.num_cells));
    for (int i = 0; i < m.num_cells; ++i) {
      const ConservativeState s{static_cast<float>(u[5 * i]), static_cast<float>(u[5 * i + 1]),
                                static_cast<float>(u[5 * i + 2]), static_cast<float>(u[5 * i + 3]),
                                static_cast<float>(u[5 * i + 4])};
      prim[i] = conservative_to_primitive(s, gamma);
    }
    PrimitiveGradients g;
    if (second_order) {
      g = compute_green_gauss_gradients(m, prim);
    } else {
      g.num_components = 2;
      g.values.assign(static_cast<size_t>(m.num_cells) * 10, 0.0f);
    }
    std::vector<EulerBoundaryConditionType> bt(static_cast<size_t>(m.num_faces));
    for (int f = 0; f < m.num_faces; ++f) bt[f] = static_cast<EulerBoundaryConditionType>(md->face_bc[f]);

    float rho_inf = static_cast<float>(c->rho_inf);
    if (rho_inf <= 0.0f)
      rho_inf = static_cast<float>(c->p_inf) /
                (static_cast<float>(c->gas_constant) * static_cast<float>(c->t_inf));
    const float alpha = static_cast<float>(c->aoa_deg) * (3.14159265358979323846f / 180.0f);
    const float a_inf = std::sqrt(gamma * static_cast<float>(c->p_inf) / rho_inf);
    const float v_inf = std::max(static_cast<float>(c->mach), 0.0f) * a_inf;
    const PrimitiveState pinf{rho_inf, v_inf * std::cos(alpha), v_inf * std::sin(alpha), 0.0f,
                              static_cast<float>(c->p_inf)};

    LowMachPreconditionConfig pc;
    pc.enabled = c->precond_on != 0;
    pc.mach_ref = static_cast<float>(c->precond_mach_ref);
    pc.mach_min = static_cast<float>(c->precond_mach_min);
    pc.beta_min = static_cast<float>(c->precond_beta_min);
    pc.beta_max = static_cast<float>(c->precond_beta_max);

    EulerResidualAssemblyConfig a;
    a.mesh = &m;
    a.primitive = &prim;
    a.gradients = &g;
    a.boundary_type = &bt;
    a.farfield_state = primitive_to_conservative(pinf, gamma);
    a.gamma = gamma;
    a.flux_scheme = c->flux == AERO_FLUX_HLLC ? EulerFluxScheme::kHllc : EulerFluxScheme::kRusanov;
    a.limiter = c->limiter == AERO_LIMITER_VENKAT ? LimiterType::kVenkat : LimiterType::kMinmod;
    a.use_second_order = second_order != 0;
    a.low_mach_dissipation_fix = c->low_mach_fix != 0;
    a.low_mach_dissipation_cutoff = static_cast<float>(c->mach_cutoff);
    a.stabilization_mach_floor = static_cast<float>(stab);
    a.preconditioned_farfield_characteristic = c->precond_farfield_bc != 0;
    a.precondition = pc;
    a.all_speed_flux_fix = as_fix != 0;
    a.all_speed_mach_cutoff = static_cast<float>(c->all_speed_mach_cutoff);
    a.all_speed_f_min = static_cast<float>(as_fmin);
    a.all_speed_ramp_weight = static_cast<float>(as_ramp);
    std::vector<float> r(static_cast<size_t>(m.num_cells) * 5, 0.0f), s(static_cast<size_t>(m.num_cells), 0.0f);
    EulerResidualAssemblyDiagnostics dg;
    assemble_euler_residual_cpu(a, &r, &s, &dg);
    for (size_t i = 0; i < r.size(); ++i) res[i] = r[i];
    for (size_t i = 0; i < s.size(); ++i) sr[i] = s[i];
    if (grad)
      for (size_t i = 0; i < g.values.size(); ++i) grad[i] = g.values[i];
    if (diag) {
      diag[0] = dg.num_faces_first_order_fallback;
      diag[1] = dg.num_faces_diffusive_fallback;
      diag[2] = dg.first_failure_face;
    }
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

// Whole run through run_euler_airfoil_case_cpu on the reference's own O-grid.
// hist receives 7 values per executed iteration (iter, l1, l2, linf, cl, cd, cm);
// conserved/last_residual/last_sr receive the final arrays (sized from the mesh).
// The run's mesh becomes the shim's current mesh.
int ref_run_case(const aero_case_desc* c, const char* naca, int n_circ, int n_radial,
                 double farfield_radius, double stretch, const char* out_dir, double* hist,
                 int max_hist, int* n_done, double* conserved, double* last_res, double* last_sr,
                 double* max_wall_mass_flux) {
  try {
    EulerAirfoilCaseConfig e;
    fill_config(*c, &e);
    e.mesh.naca_code = naca;
    e.mesh.num_circumferential = n_circ;
    e.mesh.num_radial = n_radial;
    e.mesh.farfield_radius = static_cast<float>(farfield_radius);
    e.mesh.radial_stretch = static_cast<float>(stretch);
    e.mesh.chord = static_cast<float>(c->chord);
    e.output_dir = out_dir;
    const EulerRunResult r = run_euler_airfoil_case_cpu(e);
    const int n = static_cast<int>(r.history.size());
    *n_done = n;
    for (int i = 0; i < n && i < max_hist; ++i) {
      const EulerIterationRecord& h = r.history[i];
      const double row[7] = {static_cast<double>(h.iter), h.residual_l1, h.residual_l2,
                             h.residual_linf, h.cl, h.cd, h.cm};
      for (int k = 0; k < 7; ++k) hist[7 * i + k] = row[k];
    }
    for (size_t i = 0; i < r.conserved.size(); ++i) conserved[i] = r.conserved[i];
    for (size_t i = 0; i < r.last_residual.size(); ++i) last_res[i] = r.last_residual[i];
    for (size_t i = 0; i < r.last_spectral_radius.size(); ++i) last_sr[i] = r.last_spectral_radius[i];
    *max_wall_mass_flux = r.max_wall_mass_flux;
    g_mesh = r.mesh;
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

}  // extern "C"
