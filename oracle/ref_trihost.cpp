// Host build of the reference's triangle-mesh preparation, for pinning the
// product's 2D host setup only (test infrastructure; nothing here is part of the
// product).  Compiled by build_oracle.py together with the reference's own
// trimesh sources where they lie (src/core2d/cuda/TriMesh_*.cu, filter.cc and the
// rest of that directory's host files) into _ref/libref_tri.so.
//
// ref_tri_setup runs the preparation the reference applies to a TriMesh before a
// 2D solve, in its order: meshFIM2dEikonal::SetMesh (src/core2d/include/
// meshFIM2d_eikonal.h:40-72: orient, normals, adjacent faces, across-edge map,
// triangle strips, speed type ONE, face edge lengths, InitializeAttributes, which
// builds the virtual faces of obtuse corners, TriMesh_stats.cu:46-70), on a mesh
// given as arrays (the reference also accepts a caller-filled triMesh_,
// src/Eikonal.cu:139-141).  It returns what the 2D solve then reads per face:
// the oriented corners, the three edge lengths, the inverse speed, and the list
// of virtual faces (corners, edge lengths, inverse speed).
#include <cstring>
#include <vector>

#include "TriMesh.h"
#include "TriMesh_algo.h"

extern "C" int ref_tri_setup(int nv, const float* xyz, int nf, const int* faces, const float* speeds, int nspeeds,
                             int* faces_out, float* edges_out, float* speed_inv_out, int* vf_count_out, int vf_cap,
                             int* vf_verts_out, float* vf_edges_out, float* vf_speed_inv_out) {
  TriMesh* m = new TriMesh();
  m->vertices.resize(nv);
  for (int v = 0; v < nv; ++v) m->vertices[v] = point(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
  m->faces.resize(nf);
  for (int f = 0; f < nf; ++f) m->faces[f] = TriMesh::Face(faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]);
  std::vector<float> face_speeds;
  if (speeds && nspeeds > 0) face_speeds.assign(speeds, speeds + nspeeds);
  // meshFIM2dEikonal::SetMesh with the Eikonal class's default speed type (ONE)
  m->speed_type_ = ONE;
  orient(m);
  if (!m->normals.empty()) m->normals.clear();
  m->need_normals();
  if (!m->adjacentfaces.empty()) m->adjacentfaces.clear();
  m->need_adjacentfaces();
  if (!m->across_edge.empty()) m->across_edge.clear();
  m->need_across_edge();
  if (!m->tstrips.empty()) m->tstrips.clear();
  m->need_tstrips();
  m->need_speed();
  m->need_faceedges();
  m->vertT.assign(nv, 0.0f);  // InitializeAttributes copies vertT into the faces
  m->InitializeAttributes(face_speeds);
  int total = 0;
  for (int f = 0; f < nf; ++f) {
    const TriMesh::Face& F = m->faces[f];
    for (int k = 0; k < 3; ++k) {
      faces_out[3 * f + k] = F[k];
      edges_out[3 * f + k] = F.edgeLens[k];
    }
    speed_inv_out[f] = F.speedInv;
    const std::vector<TriMesh::Face>& vf = m->faceVirtualFaces[f];
    vf_count_out[f] = (int)vf.size();
    for (const TriMesh::Face& G : vf) {
      if (total < vf_cap) {
        for (int k = 0; k < 3; ++k) {
          vf_verts_out[3 * total + k] = G[k];
          vf_edges_out[3 * total + k] = G.edgeLens[k];
        }
        vf_speed_inv_out[total] = G.speedInv;
      }
      ++total;
    }
  }
  delete m;
  return total;
}
