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
  std::vector<int> slot_face;           // [d*n] original face of the slot, -1 padding
  std::vector<int> own_old, nbr_old;    // [d*n] canonical owner / neighbour (original ids)
  // Face table: faces sorted by the new index of their owner, then by original index.
  std::vector<int> f_orig;                  // new face -> original face
  std::vector<int> f_own, f_nb;             // new owner; new neighbour, -1 far field, -2 wall
  std::vector<int> f_own_old, f_nb_old;     // original owner; original neighbour (owner if none)
  std::vector<double> f_nx, f_ny, f_area;   // unit normal out of the owner, length
  std::vector<double> f_cx, f_cy;           // face centre
  std::vector<int> gslot;                   // [d*n] (new face << 1) | (cell is the neighbour), kPad
  std::vector<double> vol;              // [n] new order
  std::vector<double> ccx, ccy;         // [n] original order (cell centres)
  // [n] new order: bit 0 owns slip-wall faces, bit 1 owns far-field faces, bits 2..7 number
  // of wall entries
  std::vector<unsigned char> flags;
  std::vector<int> wall_first;  // [n] first wall entry of the cell
  // Wall entries sorted by new owner index, then by face: the force patch faces (kind bit 0,
  // once per listing) and the slip-wall boundary faces (kind bit 1, the wall monitors); a
  // face in both sets shares one entry.
  std::vector<unsigned char> wkind;
  std::vector<double> wnx, wny, warea, wx, wy;
  std::vector<int> w_face;  // original face of each wall entry
  int n_patch = 0;  // force patch faces
  int n_slip = 0;   // slip-wall boundary faces
  int interior_faces = 0, boundary_faces = 0;
};

// Validates the mesh and builds the slot table. Returns false with a message on bad input.
bool build_slots(const aero_mesh_desc& m, int ordering, HostSlots* out, std::string* err);

// Refill the geometry arrays of *geo (slot, face-table and wall-entry normals, areas and
// centres, volumes and cell centres) from m, in the numbering and layout of `layout` (a
// build_slots result for a mesh of the same connectivity). Used for geometry tangents, whose
// arrays map through the same copies.
void map_geometry(const aero_mesh_desc& m, const HostSlots& layout, HostSlots* geo);

}  // namespace aero
