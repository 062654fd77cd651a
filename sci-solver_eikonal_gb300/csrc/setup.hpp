// setup.hpp — host-side mesh preparation, partitioning and block layout for the
// GB300 block-FIM solver.
//
// Everything here runs once per mesh (or once per speed change) on the host and
// produces flat, block-contiguous arrays that the CUDA kernels stream from HBM:
//
//   * triangle meshes: orientation, across-edge map, the obtuse-corner test and
//     the "virtual face" unfolding of obtuse corners, edge lengths, inverse speeds
//     (reference: src/core2d/include/meshFIM2d_eikonal.h:40-72 SetMesh,
//      src/core2d/cuda/TriMesh_connectivity.cu, src/core2d/include/TriMesh.h:191-313,
//      src/core2d/cuda/filter.cc:369-452)
//   * tet meshes: per-tet metric from speeds and the six metric edge products
//     (src/core3d/cuda/tetmesh.cu:9-80, src/core3d/cuda/meshFIM3dEikonal.cu:650-678)
//   * partitions: recursive coordinate bisection (a host replacement for the
//     reference's METIS k-way call) and the reference's structured-grid tiling
//     (meshFIM2d_eikonal.cu:206-252, meshFIM3dEikonal.cu:239-283)
//   * block layouts: per block the element slots (inside elements first, then the
//     elements shared with other blocks), local vertex ids, halo vertex lists and
//     the block-neighbour graph (meshFIM3dEikonal.cu:568-648, meshFIM2d_eikonal.cu:254-614)
//
// Host code is built with -ffp-contract=off so that every float expression rounds
// exactly like the reference's host compile.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace eikgb {

// ---- constants of the scheme (reference values) ----------------------------
constexpr float kLarge3D = 1000000000.0f;  // core3d/include/tetmesh.h:34-36
constexpr float kLarge2D = 10000000.0f;    // core2d/include/TriMesh.h:11-13
constexpr int kSlotCap2D = 6;              // core2d/include/CUDADefines.h:15-16
constexpr int kReduceCap2D = 32;           // core2d/cuda/CUDA_kernels.cu:8-30 with 32 threads
constexpr int kMaxSplitDepth = 64;         // guard for the recursive obtuse unfolding

// ---- triangle meshes ---------------------------------------------------------
struct TriPrep {
  int nv = 0, nf = 0;
  std::vector<int> faces;             // oriented, 3 per face
  std::vector<uint8_t> obtuse;        // bit k: corner k fails the non-obtuse test
  std::vector<int> vf_off;            // virtual faces of face i: [vf_off[i], vf_off[i+1])
  std::vector<int> vf_verts;          // 3 per virtual face
  std::vector<float> edges;           // 3 per face: |v1-v0|, |v2-v1|, |v0-v2|
  std::vector<float> vf_edges;        // 3 per virtual face
};
// Returns an empty string on success, else the reason.
std::string prepare_trimesh(int nv, const float* xyz, int nf, const int* faces, TriPrep& out);
// The reference's angle test at corner v of face f (TriMesh.h:191-212).
bool tri_corner_non_obtuse(const float* xyz, const int* f, int v);

// ---- tet meshes --------------------------------------------------------------
// Per-tet metric (6 entries M00 M01 M02 M11 M12 M22) from the reference's speed
// vector: 6*nt entries = full metric, nt entries = s*I, anything else = I.
void tet_metrics(int nt, const float* vals, size_t nvals, std::vector<float>& M);
// The six metric edge products of tet (A,B,C,D): AC.BC, BC.CD, AC.CD, AD.BD, AC.AD, BC.BD.
void tet_gram(const float* xyz, const int* tet, const float* M6, float out[6]);

// ---- partitions ----------------------------------------------------------------
// Block count rule of the reference's METIS wrappers: 2D floor(nv/k), 3D ceil(nv/k),
// at least 2 (meshFIM2d_eikonal.cu:119-121, meshFIM3dEikonal.cu:160-163).
int metis_rule_blocks(int nv, int max_verts_per_block, int dim);
// Recursive coordinate bisection into exactly `nparts` parts whose sizes differ by
// at most one vertex.  Deterministic (ties broken by vertex id).
void partition_rcb(int nv, const float* xyz, int nparts, std::vector<int>& labels);

// METIS k-way partition of the vertex graph (vertices adjacent when they share an
// element), the partitioner kind of the reference's GraphPartition_METIS2.  Parts
// METIS leaves empty are dropped: nb receives the number of non-empty blocks.
// Returns an error message when the build has no METIS.
std::string partition_metis(int nv, int ne, int nodes_per_elem, const int* elems, int nparts,
                            std::vector<int>& labels, int& nb);
bool metis_available();
// Structured tiling of a lexicographic grid (dims L x W [x D], tiles l x w [x d]).
std::string partition_square(int nv, int dim, int L, int W, int D, int bl, int bw, int bd,
                             std::vector<int>& labels, int& nblocks);

// ---- block layouts --------------------------------------------------------------
// Slots are padded per block to a multiple of 4 so every block's arrays start on a
// 16-byte boundary (bulk-copy friendly).
struct BlockDesc {
  int slot_begin;   // first slot of the block (multiple of 4)
  int nslots;       // real slots
  int nslots_pad;   // padded to a multiple of 4
  int vbase;        // first owned vertex (renumbered ids are block-contiguous)
  int nowned;
  int halo_begin;   // into halo_ids
  int nhalo;
  int ninside;      // slots whose vertices are all owned (lead the slot list)
};

struct Layout {
  int dim = 3;
  int nv = 0, ne = 0, nb = 0;
  std::vector<int> perm;          // original vertex id -> renumbered id
  std::vector<int> iperm;         // renumbered -> original
  std::vector<BlockDesc> blocks;
  int total_slots = 0;            // padded total
  int max_slots = 0, max_local = 0, max_owned = 0, max_halo = 0;
  // 3D: 6 floats per slot (SoA per block: 6 runs of nslots_pad)
  // 2D: 4 floats per slot (SoA per block: e01 e12 e20 speedInv)
  std::vector<float> coef;
  // corner local ids, 4 per slot (3D) or 4 per slot with the 4th unused (2D);
  // bit 15 marks a 2D corner whose copy is never refreshed by the reference
  std::vector<uint16_t> lv;
  std::vector<int> slot_elem;     // element (tet/face) id per slot, -1 for padding/virtual
  std::vector<int> halo_ids;      // renumbered ids of halo vertices, per block
  std::vector<int> nbr_off, nbr;  // block neighbour graph (sorted)
  double mean_slots_per_block = 0, mean_halo_per_block = 0;
  // independent solves packed together (a single mesh is one instance): blocks and
  // renumbered vertices of instance i are [inst_bbeg[i], inst_bbeg[i+1]) and
  // [inst_vbeg[i], inst_vbeg[i+1]); original vertex ids are per instance
  int ninst = 1;
  std::vector<int> blk_inst;      // instance of every block
  std::vector<int> inst_bbeg, inst_vbeg;
  // 3D precision mode: per slot the index of its tet's FP64 metric edge products
  // in coef64 (6 doubles each), -1 for tets that stay FP32; empty when off
  std::vector<int> slot_f64;
  std::vector<double> coef64;
  long long flagged_tets = 0;
};

// One layout holding several independent meshes (same dimension), instance by
// instance; the neighbour graph never crosses instances.
std::string concat_layouts(const std::vector<const Layout*>& parts, Layout& out);
// The host part of concat_layouts for layouts whose arrays live on the device:
// block descriptors (offset), renumbering, instance ranges and statistics; the
// per-slot arrays, halo lists and neighbour graph stay empty.  nhalo[i] is the
// halo list length of part i (its blocks' halo ranges are offset by the sum of
// the earlier ones).
std::string concat_layout_headers(const std::vector<const Layout*>& parts, const std::vector<int>& nhalo,
                                  Layout& out);

// 3D layout; gram terms computed from xyz and per-tet metrics.
std::string build_layout3d(int nv, const float* xyz, int nt, const int* tets, const float* M,
                           const int* labels, int nb, Layout& L);
// Recompute only the per-slot metric terms (speeds changed, mesh unchanged).
void refresh_gram3d(const float* xyz, const int* tets, const float* M, Layout& L);

// 2D layout on a prepared triangle mesh; speed_inv per real face.
std::string build_layout2d(int nv, const float* xyz, const TriPrep& P, const float* speed_inv,
                           const int* labels, int nb, Layout& L);
void refresh_speed2d(const TriPrep& P, const float* speed_inv, Layout& L);

// Precision mode (3D): flags tets whose metric edge Gram matrix G = E^T M E
// (E = the edges from the first corner) has ||G||_F ||G^-1||_F > kappa, and stores
// their six metric edge products computed in FP64 from the FP32 inputs.
// kappa <= 0 clears the precision data.
void build_precision3d(const float* xyz, const int* tets, const float* M, double kappa, Layout& L);
// Condition estimate used for the flagging (FP64; infinite for degenerate tets).
double tet_condition(const float* xyz, const int* tet, const float* M6);

// Normalise element indices to 0-based like TetMesh::init (tetmesh.cu:27-52):
// minimum index 0 or 1, anything else is an error.
std::string normalize_index_base(std::vector<int>& elems, int nv);

}  // namespace eikgb
