// mesh_io.cpp — mesh readers and the VTK writer of the solver's C ABI.
//
//   read_ply     ASCII / binary little-endian PLY triangle meshes (the 2D inputs the
//                reference reads with TriMesh::read, src/core2d/cuda/TriMesh_io.cu:154-262)
//   read_tetgen  TetGen .node/.ele pairs (tetgenio::load_tetmesh,
//                src/core3d/cuda/tetgen.cu:1993-...)
//   write_vtk    ASCII VTK unstructured grids with a "traveltime" point field
//                (meshFIM2d_eikonal.cu:74-109, meshFIM3dEikonal.cu:116-151)
#include <algorithm>
#include "mesh_io.hpp"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace eikgb {

namespace {
bool next_data_line(std::istream& in, std::string& line) {
  while (std::getline(in, line)) {
    const size_t p = line.find_first_not_of(" \t\r");
    if (p == std::string::npos || line[p] == '#') continue;
    return true;
  }
  return false;
}
}  // namespace

std::string read_ply(const std::string& path, std::vector<float>& xyz, std::vector<int>& faces) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return "cannot open " + path;
  std::string line;
  if (!std::getline(in, line) || line.compare(0, 3, "ply") != 0) return "not a PLY file: " + path;
  enum { ASCII, BLE, BBE } fmt = ASCII;
  long nvert = -1, nface = 0;
  std::vector<std::string> vprops, vtypes;
  std::string cur;
  std::string list_count_t = "uchar", list_index_t = "int";
  int face_extra = 0;  // scalar properties after the index list
  std::vector<std::string> face_extra_t;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string kw;
    ss >> kw;
    if (kw == "format") {
      std::string f;
      ss >> f;
      fmt = (f == "ascii") ? ASCII : (f == "binary_little_endian") ? BLE : BBE;
    } else if (kw == "element") {
      ss >> cur;
      long n = 0;
      ss >> n;
      if (cur == "vertex") nvert = n;
      else if (cur == "face") nface = n;
    } else if (kw == "property" || kw == "propert") {
      std::string t;
      ss >> t;
      if (cur == "vertex") {
        std::string name;
        ss >> name;
        vtypes.push_back(t);
        vprops.push_back(name);
      } else if (cur == "face") {
        if (t == "list") {
          ss >> list_count_t >> list_index_t;
        } else {
          ++face_extra;
          face_extra_t.push_back(t);
        }
      }
    } else if (kw == "end_header") {
      break;
    }
  }
  if (nvert <= 0) return "PLY file has no vertices: " + path;
  if (fmt == BBE) return "big-endian PLY is not supported: " + path;
  int ix = -1, iy = -1, iz = -1;
  for (size_t i = 0; i < vprops.size(); ++i) {
    if (vprops[i] == "x") ix = (int)i;
    if (vprops[i] == "y") iy = (int)i;
    if (vprops[i] == "z") iz = (int)i;
  }
  if (ix < 0 || iy < 0) return "PLY vertices need x and y: " + path;
  xyz.assign(3 * (size_t)nvert, 0.0f);
  faces.clear();
  auto type_size = [](const std::string& t) -> int {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "double" || t == "float64") return 8;
    return 4;
  };
  auto read_bin = [&](const std::string& t, double& v) -> bool {
    unsigned char buf[8];
    const int n = type_size(t);
    if (!in.read((char*)buf, n)) return false;
    if (t == "char" || t == "int8") v = (signed char)buf[0];
    else if (t == "uchar" || t == "uint8") v = buf[0];
    else if (t == "short" || t == "int16") { int16_t x; std::memcpy(&x, buf, 2); v = x; }
    else if (t == "ushort" || t == "uint16") { uint16_t x; std::memcpy(&x, buf, 2); v = x; }
    else if (t == "int" || t == "int32") { int32_t x; std::memcpy(&x, buf, 4); v = x; }
    else if (t == "uint" || t == "uint32") { uint32_t x; std::memcpy(&x, buf, 4); v = x; }
    else if (t == "float" || t == "float32") { float x; std::memcpy(&x, buf, 4); v = x; }
    else { double x; std::memcpy(&x, buf, 8); v = x; }
    return true;
  };
  for (long i = 0; i < nvert; ++i) {
    if (fmt == ASCII) {
      if (!next_data_line(in, line)) return "PLY vertex list truncated: " + path;
      std::istringstream ss(line);
      for (size_t p = 0; p < vprops.size(); ++p) {
        std::string tok;
        if (!(ss >> tok)) break;
        const float v = strtof(tok.c_str(), nullptr);
        if ((int)p == ix) xyz[3 * i] = v;
        if ((int)p == iy) xyz[3 * i + 1] = v;
        if ((int)p == iz) xyz[3 * i + 2] = v;
      }
    } else {
      for (size_t p = 0; p < vprops.size(); ++p) {
        double v;
        if (!read_bin(vtypes[p], v)) return "PLY vertex list truncated: " + path;
        if ((int)p == ix) xyz[3 * i] = (float)v;
        if ((int)p == iy) xyz[3 * i + 1] = (float)v;
        if ((int)p == iz) xyz[3 * i + 2] = (float)v;
      }
    }
  }
  std::vector<int> poly;
  for (long i = 0; i < nface; ++i) {
    poly.clear();
    if (fmt == ASCII) {
      if (!next_data_line(in, line)) return "PLY face list truncated: " + path;
      std::istringstream ss(line);
      int n = 0;
      ss >> n;
      for (int k = 0; k < n; ++k) {
        int v;
        if (!(ss >> v)) return "PLY face list truncated: " + path;
        poly.push_back(v);
      }
    } else {
      double dn;
      if (!read_bin(list_count_t, dn)) return "PLY face list truncated: " + path;
      for (int k = 0; k < (int)dn; ++k) {
        double v;
        if (!read_bin(list_index_t, v)) return "PLY face list truncated: " + path;
        poly.push_back((int)v);
      }
      for (const std::string& t : face_extra_t) {
        double v;
        if (!read_bin(t, v)) return "PLY face list truncated: " + path;
      }
    }
    for (size_t k = 1; k + 1 < poly.size(); ++k) {  // fan triangulation
      faces.push_back(poly[0]);
      faces.push_back(poly[k]);
      faces.push_back(poly[k + 1]);
    }
  }
  // Corner indices counted from 1 (min 1, max nvert, as in some test fixtures of
  // the reference) are read as 1-based, like the element indices of tet meshes.
  if (!faces.empty()) {
    const auto mm = std::minmax_element(faces.begin(), faces.end());
    if (*mm.first == 1 && *mm.second == nvert)
      for (int& v : faces) v -= 1;
  }
  for (int v : faces)
    if (v < 0 || v >= nvert) return "PLY face index out of range: " + path;
  return "";
}

std::string read_tetgen(const std::string& base, std::vector<float>& xyz, std::vector<int>& tets) {
  std::ifstream nin(base + ".node");
  if (!nin) return "cannot access " + base + ".node";
  std::string line;
  if (!next_data_line(nin, line)) return "empty node file";
  long np = 0;
  int dim = 3, nattr = 0, nmark = 0;
  {
    std::istringstream ss(line);
    ss >> np;
    if (!(ss >> dim)) dim = 3;
    if (!(ss >> nattr)) nattr = 0;
    if (!(ss >> nmark)) nmark = 0;
  }
  if (np <= 0 || dim != 3) return "node file must hold 3D points";
  xyz.assign(3 * (size_t)np, 0.0f);
  long first = 0;
  for (long i = 0; i < np; ++i) {
    if (!next_data_line(nin, line)) return "node file truncated";
    std::istringstream ss(line);
    long idx;
    double x, y, z;
    if (!(ss >> idx >> x >> y >> z)) return "bad node line";
    if (i == 0) first = idx;
    const long k = idx - first;
    if (k < 0 || k >= np) return "node index out of range";
    xyz[3 * k] = (float)x;
    xyz[3 * k + 1] = (float)y;
    xyz[3 * k + 2] = (float)z;
  }
  std::ifstream ein(base + ".ele");
  if (!ein) return "cannot access " + base + ".ele";
  if (!next_data_line(ein, line)) return "empty ele file";
  long nt = 0;
  int per = 4;
  {
    std::istringstream ss(line);
    ss >> nt;
    if (!(ss >> per)) per = 4;
  }
  if (nt <= 0 || per < 4) return "ele file must hold tetrahedra";
  tets.assign(4 * (size_t)nt, 0);
  for (long i = 0; i < nt; ++i) {
    if (!next_data_line(ein, line)) return "ele file truncated";
    std::istringstream ss(line);
    long idx;
    int v[4];
    if (!(ss >> idx >> v[0] >> v[1] >> v[2] >> v[3])) return "bad ele line";
    for (int k = 0; k < 4; ++k) tets[4 * (size_t)i + k] = v[k];
  }
  return "";
}

std::string write_vtk(const std::string& path, int dim, const std::vector<float>& xyz, const std::vector<int>& elems,
                      const float* values, int nv) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return "cannot write " + path;
  const int per = (dim == 3) ? 4 : 3;
  const size_t ne = elems.size() / per;
  std::fprintf(f, "# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %d float\n", nv);
  for (int i = 0; i < nv; ++i) std::fprintf(f, "%.12f %.12f %.12f\n", xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  std::fprintf(f, "CELLS %zu %zu\n", ne, ne * (per + 1));
  for (size_t i = 0; i < ne; ++i) {
    std::fprintf(f, "%d", per);
    for (int k = 0; k < per; ++k) std::fprintf(f, " %d", elems[per * i + k]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "CELL_TYPES %zu\n", ne);
  for (size_t i = 0; i < ne; ++i) std::fprintf(f, "%d\n", dim == 3 ? 10 : 5);
  std::fprintf(f, "POINT_DATA %d\nSCALARS traveltime float 1\nLOOKUP_TABLE default\n", nv);
  for (int i = 0; i < nv; ++i) std::fprintf(f, "%.12f\n", values[i]);
  const bool ok = std::fclose(f) == 0;
  return ok ? "" : "write failed: " + path;
}

}  // namespace eikgb
