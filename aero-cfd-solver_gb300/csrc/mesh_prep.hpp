// mesh_prep.hpp -- host preprocessing of a reference-layout mesh into the device layout:
// validation, cell renumbering (Morton / reverse Cuthill-McKee) and the cell-owned face
// slot table (ELL, slot (k, c) at k*N + c).
#pragma once

#include "../../include/aero_gb300.h"

#include <string>
#include <vector>

namespace aero {

struct HostSlots {
  int n = 0;      // cells
  int d = 0;      // slots per cell (max faces of any cell)
  int nf = 0;     // faces
  std::vector<int> perm;   // new -> original cell
  std::vector<int> iperm;  // original -> new cell
  std::vector<int> link;   // [d*n] (other_new << 1 | side), -1 far field, -2 wall, kPad
  std::vector<double> nx, ny, area;     // [d*n] canonical (owner-outward) face geometry
  std::vector<double> fcx, fcy;         // [d*n] face centre
  std::vector<int> own_old, nbr_old;    // [d*n] canonical owner / neighbour (original ids)
  std::vector<double> vol;              // [n] new order
  std::vector<double> ccx, ccy;         // [n] original order (cell centres)
  std::vector<unsigned char> wall_adj;  // [n] new order
  // wall patch in patch order
  std::vector<int> wall_cell;  // new owner index
  std::vector<double> wnx, wny, warea, wx, wy;
  // owners (new index) of the far-field faces in face order
  std::vector<int> far_cell;
  int interior_faces = 0, boundary_faces = 0;
};

// Validates the mesh and builds the slot table. Returns false with a message on bad input.
bool build_slots(const aero_mesh_desc& m, int ordering, HostSlots* out, std::string* err);

}  // namespace aero
