/* aero_driver.h -- case-level entry points of libaero_gb300.so (C ABI).
 *
 * These replace the "cuda" backend of AeroCFD's case dispatcher and Euler driver
 * (cfd::core::run_case, src/cfd_core/numerics/residual_stub.cpp:392-777, and
 * run_euler_airfoil_case, src/cfd_core/solvers/euler_solver.cpp:463-1487; paths relative to
 * the AeroCFD root). They read the same flat key=value case file (python/cfd/case.py:313-542
 * writes it), run the iterations on the device through aero_gb300.h, and write the same
 * outputs: residuals.csv, forces.csv, euler_diagnostics.csv, cp_wall.csv, wall_flux.csv,
 * dissipation_debug.csv, boundary_faces_debug.txt, effective_config_snapshot.txt,
 * field_0000.vtu and run.log. Added keys: precision=fp32|fp64 (default fp32), ordering,
 * precond_precision=auto|fp64|fp32|ff (aero_case_desc.precond_fp64 0|1|-1|2, default auto).
 */
#ifndef AERO_DRIVER_H
#define AERO_DRIVER_H

#include "aero_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The fields of the pybind run_case dict (src/cfd_core/bindings/pybind_module.cpp:19-38). */
typedef struct aero_run_summary {
  char status[16];
  char backend[16];
  char case_type[64];
  char run_log[1024];
  int iterations;
  double residual_l1, residual_l2, residual_linf;
  double cl, cd, cm;
} aero_run_summary;

/* O-grid settings of AirfoilMeshConfig (src/cfd_core/include/cfd_core/mesh/airfoil_mesh.hpp:10-19). */
typedef struct aero_airfoil_mesh_cfg {
  char naca_code[16];
  int num_circumferential;
  int num_radial;
  double farfield_radius;
  double radial_stretch;
  double chord;
} aero_airfoil_mesh_cfg;

/* Backend check of normalize_backend (residual_stub.cpp:308-327): returns AERO_OK for
 * "cuda" when a device is usable; AERO_ERR_INVALID for an unknown name or for "cpu"
 * (the CPU path is the reference library's, not this one); AERO_ERR_CUDA when "cuda"
 * is requested without a device. */
AERO_API int aero_normalize_backend(const char* backend, char* normalized, int len);

/* Parse a case file (parse_case_kv, residual_stub.cpp:160-190, and the key mapping of
 * :403-558) into a case descriptor and O-grid settings. case_type receives the case type. */
AERO_API int aero_parse_case(const char* case_path, aero_case_desc* cfg, aero_airfoil_mesh_cfg* mesh,
                             char* case_type, int case_type_len);

/* run_euler_airfoil_case(config, "cuda") on the reference O-grid built from `mesh`;
 * writes the reference's output files into out_dir. AERO_ENABLE_EXPERIMENTAL_PRECOND
 * gates preconditioning exactly as the reference does (euler_solver.cpp:483-489). */
AERO_API int aero_run_euler_airfoil_case(const aero_case_desc* cfg, const aero_airfoil_mesh_cfg* mesh,
                                         const char* out_dir, aero_run_summary* out);

/* run_case(case_path, out_dir, backend) for case_type=euler_airfoil_2d. */
AERO_API int aero_run_case(const char* case_path, const char* out_dir, const char* backend,
                           aero_run_summary* out);

/* Sweep of a base case over angles of attack, replacing the serial loop of the reference's
 * run_sweep (python/cfd/sweep.py:14-59, one run_case per angle, each into
 * <output root>/run_NNN). Reads the base case file, sets case k's aoa_deg = aoa_deg[k] (and
 * mach = mach[k] when mach is not NULL; no reference counterpart), runs all n_cases cases as
 * one batch on the base case's mesh, and writes each case's run_case outputs into
 * out_root/run_000, run_001, ... plus out_root/sweep_summary.csv (run, aoa_deg, mach,
 * iterations, residual_l2, cl, cd, cm, status). summaries[k] receives case k's run_case dict
 * values. Every case's results equal those of run_case on the modified case file. */
AERO_API int aero_run_sweep(const char* case_path, int n_cases, const double* aoa_deg, const double* mach,
                            const char* out_root, const char* backend, aero_run_summary* summaries);

/* State dump for continuation (no reference counterpart; the reference has no restart):
 * a 16-byte magic, int64 cell count, int64 component count (5), then the conserved state
 * [N][5] double in the reference's cell order and AoS layout, host byte order. Read checks
 * the magic and the cell count and returns AERO_ERR_INVALID on a mismatch or short file.
 * The driver's case file takes restart_in = <state file> (start from it instead of the free
 * stream; the iteration schedule starts again at 0) and restart_out = <file name in out_dir>
 * (dump the final state), and vtu_format = ascii (default, the reference's) | binary (raw
 * appended VTU arrays). */
AERO_API int aero_state_write(const char* path, int num_cells, const double* conserved);
AERO_API int aero_state_read(const char* path, int num_cells, double* conserved);

/* Message of the last failed driver call on this thread. */
AERO_API const char* aero_driver_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* AERO_DRIVER_H */
