// mesh_io.hpp — file formats around the solver (see mesh_io.cpp).
#pragma once

#include <string>
#include <vector>

namespace eikgb {

std::string read_ply(const std::string& path, std::vector<float>& xyz, std::vector<int>& faces);
std::string read_tetgen(const std::string& base, std::vector<float>& xyz, std::vector<int>& tets);
std::string write_vtk(const std::string& path, int dim, const std::vector<float>& xyz, const std::vector<int>& elems,
                      const float* values, int nv);

}  // namespace eikgb
