// solver_access.hpp — what the request server needs from a configured solver
// handle: its block layout (built exactly as eik_solve builds it, on the host or
// on the device) and the inputs its per-slot coefficients are computed from.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "setup.hpp"

struct eik_solver;

namespace eikgb {

struct Built3D;

struct MeshSnapshot {
  int dim = 3;
  int nv = 0, ne = 0;
  Layout layout;                // copy of the handle's layout (host part only when `built`)
  std::shared_ptr<Built3D> built;  // the layout's arrays built on the device (device_setup = 1)
  std::vector<float> xyz;       // 3 per vertex
  std::vector<int> elems;       // 3D: 4 per tet (0-based)
  std::vector<float> M6;        // 3D: 6 metric entries per tet
  std::vector<float> speed;     // 2D: speed per real face (1 where none was given)
  int max_iterations = 100;
  int fim_sweeps = -1;
  int threads = 0;
};

// Returns an EIK_* status; err receives the reason on failure.
int snapshot_for_server(eik_solver* h, MeshSnapshot& out, std::string& err);

}  // namespace eikgb
