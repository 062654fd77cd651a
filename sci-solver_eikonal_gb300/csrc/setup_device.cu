// setup_device.cu — the 3D block layout built on the GPU.
//
// Same layout as build_layout3d (setup.cpp), from the same inputs (coordinates,
// tets, per-tet metric, partition labels), with sorts and scans instead of the
// host's per-block lists:
//   1. owned-vertex renumbering: stable sort of vertex ids by block label
//      (ascending original id inside a block, the reference's m_PartitionInVerts
//      order; meshFIM3dEikonal.cu:568-648);
//   2. element slots: every tet emits (block, inside|shared) keys — one for a tet
//      inside a block, one per distinct block for a shared tet — and a stable sort
//      puts each block's inside tets first, then its shared tets, both in
//      ascending tet id (m_PartitionTets / m_PartitionNbTets order);
//   3. halo lists: (block, renumbered id) keys of foreign corners, sorted and
//      made unique, so every block's halo is ascending in renumbered id;
//   4. corner local ids (owned: offset in the block; halo: position found by
//      binary search in the block's halo list) and the six metric edge products
//      per slot, in the host build's operation order (gettetmem / vMv);
//   5. the block-neighbour graph: sorted unique block pairs of shared tets.
// The result equals the host layout's arrays.  Device sorts, scans and
// selections come from CUB (part of the CUDA toolkit).
#include <cuda_runtime.h>

#include <cub/cub.cuh>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "device.hpp"

namespace eikgb {
namespace {

#define CKS(x)                                                                          \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) return std::string(#x ": ") + cudaGetErrorString(e_);       \
  } while (0)

constexpr int kThreads = 256;
inline int grid_for(long long n) {
  return (int)std::max(1LL, std::min(65535LL * 8, (n + kThreads - 1) / kThreads));
}

__global__ void k_iota(int* a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

__global__ void k_count_labels(const int* lab, int n, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(&cnt[lab[i]], 1);
}

// perm[iperm[n]] = n; vblock[n] = block of renumbered vertex n
__global__ void k_perm(const int* iperm, const int* lab_sorted, int nv, int* perm, int* vblock) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nv; n += gridDim.x * blockDim.x) {
    perm[iperm[n]] = n;
    vblock[n] = lab_sorted[n];
  }
}

// distinct sorted labels of a tet's corners
__device__ __forceinline__ int tet_labels(const int* tets, const int* lab, int t, int ls[4]) {
  int n = 0;
  for (int k = 0; k < 4; ++k) {
    const int l = lab[tets[4 * (size_t)t + k]];
    bool seen = false;
    for (int j = 0; j < n; ++j) seen |= (ls[j] == l);
    if (!seen) ls[n++] = l;
  }
  for (int x = 1; x < n; ++x)
    for (int y = x; y > 0 && ls[y - 1] > ls[y]; --y) {
      const int s = ls[y - 1];
      ls[y - 1] = ls[y];
      ls[y] = s;
    }
  return n;
}

// per tet: slot keys emitted (1 inside / n shared) and neighbour pairs n(n-1)
__global__ void k_tet_counts(const int* tets, const int* lab, int nt, int* nslot, int* npair) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    int ls[4];
    const int n = tet_labels(tets, lab, t, ls);
    nslot[t] = n;
    npair[t] = n * (n - 1);
  }
}

__global__ void k_tet_emit(const int* tets, const int* lab, int nt, const int* slot_off, const int* pair_off,
                           unsigned* key, int* val, unsigned long long* pairs) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    int ls[4];
    const int n = tet_labels(tets, lab, t, ls);
    int o = slot_off[t];
    if (n == 1) {
      key[o] = 2u * (unsigned)ls[0];
      val[o] = t;
    } else {
      for (int j = 0; j < n; ++j) {
        key[o + j] = 2u * (unsigned)ls[j] + 1u;
        val[o + j] = t;
      }
    }
    o = pair_off[t];
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b)
        if (a != b) pairs[o++] = ((unsigned long long)(unsigned)ls[a] << 32) | (unsigned)ls[b];
  }
}

__global__ void k_count_keys(const unsigned* key, int n, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(&cnt[key[i]], 1);
}

__global__ void k_pad_counts(const int* keycnt, int nb, int* padded) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
    padded[b] = (keycnt[2 * b] + keycnt[2 * b + 1] + 3) & ~3;
}

// BlockDesc of every block except the halo fields
__global__ void k_block_desc(const int* keycnt, const int* vbase, const int* slot_begin, int nb, BlockDesc* bd) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    BlockDesc d;
    d.ninside = keycnt[2 * b];
    d.nslots = keycnt[2 * b] + keycnt[2 * b + 1];
    d.nslots_pad = (d.nslots + 3) & ~3;
    d.slot_begin = slot_begin[b];
    d.vbase = vbase[b];
    d.nowned = vbase[b + 1] - vbase[b];
    d.halo_begin = 0;
    d.nhalo = 0;
    bd[b] = d;
  }
}

// sorted pair p -> slot: slot_elem, and the foreign-corner keys of the slot
__global__ void k_place(const unsigned* key, const int* val, int np, const int* keybeg, const BlockDesc* bd,
                        const int* tets, const int* lab, const int* perm, int* slot_elem, int* slot_of,
                        unsigned long long* hkeys) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const int b = (int)(key[p] >> 1);
    const int t = val[p];
    const int s = bd[b].slot_begin + (p - keybeg[2 * b]);
    slot_elem[s] = t;
    slot_of[p] = s;
    for (int k = 0; k < 4; ++k) {
      const int v = tets[4 * (size_t)t + k];
      hkeys[4 * (size_t)p + k] =
          (lab[v] != b) ? (((unsigned long long)(unsigned)b << 32) | (unsigned)perm[v]) : ~0ull;
    }
  }
}

__global__ void k_count_halo(const unsigned long long* uk, int n, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (uk[i] != ~0ull) atomicAdd(&cnt[(int)(uk[i] >> 32)], 1);
}

__global__ void k_halo_ids(const unsigned long long* uk, int n, int* halo) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (uk[i] != ~0ull) halo[i] = (int)(uk[i] & 0xffffffffu);
}

__global__ void k_halo_desc(const int* hcnt, const int* hbeg, int nb, BlockDesc* bd, int* too_many) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    bd[b].halo_begin = hbeg[b];
    bd[b].nhalo = hcnt[b];
    if (bd[b].nowned + hcnt[b] > 32767) atomicOr(too_many, 1);
  }
}

// the host build's tet_gram product u^T M w: float operations one at a time, in
// its order
__device__ __forceinline__ float uMw_host(const float* u, const float* m, const float* w) {
  const float x = __fadd_rn(__fadd_rn(__fmul_rn(u[0], m[0]), __fmul_rn(u[1], m[1])), __fmul_rn(u[2], m[2]));
  const float y = __fadd_rn(__fadd_rn(__fmul_rn(u[0], m[1]), __fmul_rn(u[1], m[3])), __fmul_rn(u[2], m[4]));
  const float z = __fadd_rn(__fadd_rn(__fmul_rn(u[0], m[2]), __fmul_rn(u[1], m[4])), __fmul_rn(u[2], m[5]));
  return __fadd_rn(__fadd_rn(__fmul_rn(x, w[0]), __fmul_rn(y, w[1])), __fmul_rn(z, w[2]));
}

// the six metric entries of tet t from mcomp stored per tet (a scalar s is s*I)
__device__ __forceinline__ void metric_entries(const float* M, int mcomp, int t, float* m) {
  if (mcomp == 6) {
    for (int q = 0; q < 6; ++q) m[q] = M[6 * (size_t)t + q];
  } else {
    const float s = M[t];
    m[0] = s; m[1] = 0.0f; m[2] = 0.0f; m[3] = s; m[4] = 0.0f; m[5] = s;
  }
}

// corner local ids and the six metric edge products of every slot
__global__ void k_slot_fill(const unsigned* key, const int* val, const int* slot_of, int np, const BlockDesc* bd,
                            const int* tets, const int* lab, const int* perm, const int* halo, const float* xyz,
                            const float* M, int mcomp, uint16_t* lv, float* coef) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const int b = (int)(key[p] >> 1);
    const int t = val[p];
    const int s = slot_of[p];
    const BlockDesc d = bd[b];
    const int* hl = halo + d.halo_begin;
    float P[4][3];
    for (int k = 0; k < 4; ++k) {
      const int v = tets[4 * (size_t)t + k];
      const int nvid = perm[v];
      int lid;
      if (lab[v] == b) {
        lid = nvid - d.vbase;
      } else {
        int lo = 0, hi = d.nhalo - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (hl[mid] < nvid) lo = mid + 1;
          else hi = mid;
        }
        lid = d.nowned + lo;
      }
      lv[4 * (size_t)s + k] = (uint16_t)lid;
      for (int c = 0; c < 3; ++c) P[k][c] = xyz[3 * (size_t)v + c];
    }
    float m[6];
    metric_entries(M, mcomp, t, m);
    float AC[3], AD[3], BC[3], CD[3], BD[3];
    for (int c = 0; c < 3; ++c) {
      AC[c] = __fsub_rn(P[2][c], P[0][c]);
      AD[c] = __fsub_rn(P[3][c], P[0][c]);
      BC[c] = __fsub_rn(P[2][c], P[1][c]);
      CD[c] = __fsub_rn(P[3][c], P[2][c]);
      BD[c] = __fsub_rn(P[3][c], P[1][c]);
    }
    const size_t np_ = (size_t)d.nslots_pad;
    float* base = coef + 6 * (size_t)d.slot_begin + (s - d.slot_begin);
    base[0 * np_] = uMw_host(AC, m, BC);
    base[1 * np_] = uMw_host(BC, m, CD);
    base[2 * np_] = uMw_host(AC, m, CD);
    base[3 * np_] = uMw_host(AD, m, BD);
    base[4 * np_] = uMw_host(AC, m, AD);
    base[5 * np_] = uMw_host(BC, m, BD);
  }
}

__global__ void k_count_nbr(const unsigned long long* uk, int n, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&cnt[(int)(uk[i] >> 32)], 1);
}

__global__ void k_nbr_ids(const unsigned long long* uk, int n, int* nbr) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    nbr[i] = (int)(uk[i] & 0xffffffffu);
}

// ---- 2D: the triangle layout of build_layout2d --------------------------------

// distinct sorted labels of a face's corners
__device__ __forceinline__ int face_labels(const int* faces, const int* lab, int f, int ls[3]) {
  int n = 0;
  for (int k = 0; k < 3; ++k) {
    const int l = lab[faces[3 * (size_t)f + k]];
    bool seen = false;
    for (int j = 0; j < n; ++j) seen |= (ls[j] == l);
    if (!seen) ls[n++] = l;
  }
  for (int x = 1; x < n; ++x)
    for (int y = x; y > 0 && ls[y - 1] > ls[y]; --y) {
      const int t = ls[y - 1];
      ls[y - 1] = ls[y];
      ls[y] = t;
    }
  return n;
}

// per face: slot keys (1 inside / n shared, plus its virtual faces once per obtuse
// corner, PartitionFaces meshFIM2d_eikonal.cu:254-347) and neighbour pairs n(n-1)
__global__ void k_face_counts(const int* faces, const int* lab, const unsigned char* obtuse, const int* vf_off,
                              int nf, int* nslot, int* npair) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
    int ls[3];
    const int n = face_labels(faces, lab, f, ls);
    nslot[f] = n + __popc((unsigned)obtuse[f]) * (vf_off[f + 1] - vf_off[f]);
    npair[f] = n * (n - 1);
  }
}

// keys 3b (inside), 3b+1 (shared), 3b+2 (virtual); values: face id, or -2 - the
// virtual face's index; emitted face by face so a stable sort keeps each block's
// faces in ascending id and its virtual faces in (face, corner, index) order
__global__ void k_face_emit(const int* faces, const int* lab, const unsigned char* obtuse, const int* vf_off, int nf,
                            const int* slot_off, const int* pair_off, unsigned* key, int* val,
                            unsigned long long* pairs) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
    int ls[3];
    const int n = face_labels(faces, lab, f, ls);
    int o = slot_off[f];
    if (n == 1) {
      key[o] = 3u * (unsigned)ls[0];
      val[o++] = f;
    } else {
      for (int j = 0; j < n; ++j) {
        key[o] = 3u * (unsigned)ls[j] + 1u;
        val[o++] = f;
      }
    }
    for (int k = 0; k < 3; ++k)
      if (obtuse[f] & (1u << k)) {
        const unsigned b = (unsigned)lab[faces[3 * (size_t)f + k]];
        for (int j = vf_off[f]; j < vf_off[f + 1]; ++j) {
          key[o] = 3u * b + 2u;
          val[o++] = -2 - j;
        }
      }
    o = pair_off[f];
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b)
        if (a != b) pairs[o++] = ((unsigned long long)(unsigned)ls[a] << 32) | (unsigned)ls[b];
  }
}

__global__ void k_pad_counts3(const int* keycnt, int nb, int* padded, int* nin, int* nrest) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    const int n = keycnt[3 * b] + keycnt[3 * b + 1] + keycnt[3 * b + 2];
    padded[b] = (n + 3) & ~3;
    nin[b] = keycnt[3 * b];
    nrest[b] = n - keycnt[3 * b];
  }
}

__global__ void k_block_desc2d(const int* keycnt, const int* vbase, const int* slot_begin, int nb, BlockDesc* bd) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    BlockDesc d;
    d.ninside = keycnt[3 * b];
    d.nslots = keycnt[3 * b] + keycnt[3 * b + 1] + keycnt[3 * b + 2];
    d.nslots_pad = (d.nslots + 3) & ~3;
    d.slot_begin = slot_begin[b];
    d.vbase = vbase[b];
    d.nowned = vbase[b + 1] - vbase[b];
    d.halo_begin = 0;
    d.nhalo = 0;
    bd[b] = d;
  }
}

__device__ __forceinline__ const int* slot_corners(const int* faces, const int* vf_verts, int e) {
  return (e >= 0) ? faces + 3 * (size_t)e : vf_verts + 3 * (size_t)(-2 - e);
}

// sorted pair p -> slot: slot_elem, halo keys of foreign corners, and the corner
// entries of blockVertMapping (meshFIM2d_eikonal.cu:404-614) in its order: every
// block's inside slots first (pass 1), then every block's other slots (pass 2)
__global__ void k_place2d(const unsigned* key, const int* val, int np, const int* keybeg, const BlockDesc* bd,
                          const int* inbase, const int* restbase, int ninside_total, const int* faces,
                          const int* vf_verts, const int* lab, const int* perm, int* slot_elem, int* slot_of,
                          unsigned long long* hkeys, int* ekey, unsigned long long* eval) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const int b = (int)(key[p] / 3u);
    const int e = val[p];
    const int j = p - keybeg[3 * b];
    const int s = bd[b].slot_begin + j;
    slot_elem[s] = e;
    slot_of[p] = s;
    const int* cv = slot_corners(faces, vf_verts, e);
    const int ni = bd[b].ninside;
    const long long ent = (j < ni) ? 3ll * (inbase[b] + j) : 3ll * ninside_total + 3ll * (restbase[b] + j - ni);
    for (int k = 0; k < 3; ++k) {
      const int v = cv[k];
      hkeys[3 * (size_t)p + k] = (lab[v] != b) ? (((unsigned long long)(unsigned)b << 32) | (unsigned)perm[v]) : ~0ull;
      ekey[ent + k] = v;
      eval[ent + k] = ((unsigned long long)(unsigned)b << 32) | (unsigned)(4 * s + k);
    }
  }
}

// corner local ids, edge lengths and inverse speeds of every slot (1 / speed as the
// host build computes it, TriMesh_stats.cu:64-68; 1 for virtual faces)
__global__ void k_slot_fill2d(const int* val, const int* slot_of, const unsigned* key, int np, const BlockDesc* bd,
                              const int* faces, const int* vf_verts, const float* edges, const float* vf_edges,
                              const float* speed, const int* lab, const int* perm, const int* halo, uint16_t* lv,
                              float* coef) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const int b = (int)(key[p] / 3u);
    const int e = val[p];
    const int s = slot_of[p];
    const BlockDesc d = bd[b];
    const int* hl = halo + d.halo_begin;
    const int* cv = slot_corners(faces, vf_verts, e);
    for (int k = 0; k < 3; ++k) {
      const int v = cv[k];
      const int nvid = perm[v];
      int lid;
      if (lab[v] == b) {
        lid = nvid - d.vbase;
      } else {
        int lo = 0, hi = d.nhalo - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (hl[mid] < nvid) lo = mid + 1;
          else hi = mid;
        }
        lid = d.nowned + lo;
      }
      lv[4 * (size_t)s + k] = (uint16_t)lid;
    }
    lv[4 * (size_t)s + 3] = 0;
    const float* ed = (e >= 0) ? edges + 3 * (size_t)e : vf_edges + 3 * (size_t)(-2 - e);
    const size_t np_ = (size_t)d.nslots_pad;
    float* base = coef + 4 * (size_t)d.slot_begin + (s - d.slot_begin);
    base[0] = ed[0];
    base[1 * np_] = ed[1];
    base[2 * np_] = ed[2];
    base[3 * np_] = (e >= 0) ? __fdiv_rn(1.0f, speed[e]) : 1.0f;
  }
}

__global__ void k_own_flags(const int* ekey, const unsigned long long* eval, const int* lab, int n, int* own) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    own[i] = ((int)(eval[i] >> 32) == lab[ekey[i]]) ? 1 : 0;
}

__global__ void k_seg_begin(const int* ekey, int n, int* vbeg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (i == 0 || ekey[i - 1] != ekey[i]) vbeg[ekey[i]] = i;
}

__global__ void k_first_own(const int* ekey, const int* own, const int* ownrank, const int* vbeg, int n,
                            int* first_own) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (own[i] && ownrank[i] == 0) first_own[ekey[i]] = i - vbeg[ekey[i]];
}

// The reference keeps a vertex's first kSlotCap2D own-block and first kSlotCap2D
// other-block copies live, in blockVertMapping order after moving the first
// own-block entry to the front (which shifts the other-block entries before it):
// the others are marked with bit 15 of their corner id.
__global__ void k_live2d(const int* ekey, const unsigned long long* eval, const int* own, const int* ownrank,
                         const int* vbeg, const int* first_own, int n, int cap, uint16_t* lv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = ekey[i];
    const int q = i - vbeg[v];
    bool live;
    if (own[i]) {
      live = ownrank[i] < cap;
    } else {
      const int f = first_own[v];
      int r = q - ownrank[i];
      if (f > 0) r = (q == 0) ? f - 1 : (q < f ? q - 1 : r);
      live = r < cap;
    }
    if (!live) {
      const unsigned c = (unsigned)(eval[i] & 0xffffffffu);
      lv[c] = (uint16_t)(lv[c] | 0x8000u);
    }
  }
}

// temporary device buffers of one build, freed on every exit
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  std::string get(T*& p, size_t n) {
    p = nullptr;
    CKS(cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T)));
    ptrs.push_back(p);
    return "";
  }
};

template <typename T>
std::string keep(T*& p, size_t n) {
  p = nullptr;
  CKS(cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T)));
  return "";
}

int bits_for(unsigned long long maxval) {
  int b = 1;
  while (b < 64 && (maxval >> b) != 0) ++b;
  return b;
}

std::string exclusive_scan(Scratch& S, const int* in, int* out, int n, cudaStream_t st) {
  size_t tb = 0;
  CKS(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, n, st));
  unsigned char* tmp;
  std::string e = S.get(tmp, tb);
  if (!e.empty()) return e;
  CKS(cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, n, st));
  return "";
}

template <typename K, typename V>
std::string sort_pairs(Scratch& S, const K* kin, K* kout, const V* vin, V* vout, int n, int end_bit,
                       cudaStream_t st) {
  size_t tb = 0;
  CKS(cub::DeviceRadixSort::SortPairs(nullptr, tb, kin, kout, vin, vout, n, 0, end_bit, st));
  unsigned char* tmp;
  std::string e = S.get(tmp, tb);
  if (!e.empty()) return e;
  CKS(cub::DeviceRadixSort::SortPairs(tmp, tb, kin, kout, vin, vout, n, 0, end_bit, st));
  return "";
}

// sorted unique 64-bit keys: out receives them, *count their number
std::string sort_unique(Scratch& S, const unsigned long long* in, unsigned long long* sorted,
                        unsigned long long* out, int n, int* d_count, int* count, cudaStream_t st) {
  size_t tb = 0;
  CKS(cub::DeviceRadixSort::SortKeys(nullptr, tb, in, sorted, n, 0, 64, st));
  unsigned char* tmp;
  std::string e = S.get(tmp, tb);
  if (!e.empty()) return e;
  CKS(cub::DeviceRadixSort::SortKeys(tmp, tb, in, sorted, n, 0, 64, st));
  size_t tb2 = 0;
  CKS(cub::DeviceSelect::Unique(nullptr, tb2, sorted, out, d_count, n, st));
  unsigned char* tmp2;
  if (!(e = S.get(tmp2, tb2)).empty()) return e;
  CKS(cub::DeviceSelect::Unique(tmp2, tb2, sorted, out, d_count, n, st));
  CKS(cudaMemcpyAsync(count, d_count, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  return "";
}

// Owned-vertex renumbering: a stable sort of vertex ids by block label (ascending
// original id inside a block, the reference's m_PartitionInVerts order); out.perm,
// out.vblock and the per-block first renumbered vertex d_vbase (nb + 1).
std::string renumber_device(Scratch& S, const int* d_lab, int nv, int nb, cudaStream_t st, Built3D& out,
                            int*& d_vbase) {
  std::string e;
  int *d_ids, *d_iperm, *d_lab_sorted, *d_cnt;
  if (!(e = S.get(d_ids, nv)).empty() || !(e = S.get(d_iperm, nv)).empty() ||
      !(e = S.get(d_lab_sorted, nv)).empty() || !(e = S.get(d_cnt, nb + 1)).empty() ||
      !(e = S.get(d_vbase, nb + 1)).empty() || !(e = keep(out.perm, nv)).empty() ||
      !(e = keep(out.vblock, nv)).empty())
    return e;
  k_iota<<<grid_for(nv), kThreads, 0, st>>>(d_ids, nv);
  if (!(e = sort_pairs(S, d_lab, d_lab_sorted, d_ids, d_iperm, nv, bits_for((unsigned long long)nb), st)).empty())
    return e;
  CKS(cudaMemsetAsync(d_cnt, 0, sizeof(int) * (nb + 1), st));
  k_count_labels<<<grid_for(nv), kThreads, 0, st>>>(d_lab, nv, d_cnt);
  if (!(e = exclusive_scan(S, d_cnt, d_vbase, nb + 1, st)).empty()) return e;
  k_perm<<<grid_for(nv), kThreads, 0, st>>>(d_iperm, d_lab_sorted, nv, out.perm, out.vblock);
  return "";
}

// Block-neighbour graph from the (block, block) pairs of shared elements: sorted
// unique pairs, then CSR.
std::string neighbour_graph(Scratch& S, unsigned long long* d_pairs, unsigned long long* d_pairs_s, int npairs,
                            int nb, int* d_cnt1, cudaStream_t st, Built3D& out, int* nn) {
  std::string e;
  *nn = 0;
  if (!(e = keep(out.nbr_off, nb + 1)).empty()) return e;
  if (npairs > 0) {
    unsigned long long* d_pu;
    if (!(e = S.get(d_pu, npairs)).empty()) return e;
    if (!(e = sort_unique(S, d_pairs, d_pairs_s, d_pu, npairs, d_cnt1, nn, st)).empty()) return e;
    int* d_ncnt;
    if (!(e = S.get(d_ncnt, nb + 1)).empty()) return e;
    CKS(cudaMemsetAsync(d_ncnt, 0, sizeof(int) * (nb + 1), st));
    k_count_nbr<<<grid_for(*nn), kThreads, 0, st>>>(d_pu, *nn, d_ncnt);
    if (!(e = exclusive_scan(S, d_ncnt, out.nbr_off, nb + 1, st)).empty()) return e;
    if (!(e = keep(out.nbr, *nn)).empty()) return e;
    k_nbr_ids<<<grid_for(*nn), kThreads, 0, st>>>(d_pu, *nn, out.nbr);
  } else {
    CKS(cudaMemsetAsync(out.nbr_off, 0, sizeof(int) * (nb + 1), st));
    if (!(e = keep(out.nbr, 1)).empty()) return e;
  }
  return "";
}

// The host part of a device-built layout: block descriptors, renumbering and
// statistics.
std::string host_part(int dim, int nv, int ne, int nb, int total_slots, const Built3D& out, const int* d_too,
                      cudaStream_t st, Layout& L) {
  int too = 0;
  L.dim = dim;
  L.nv = nv;
  L.ne = ne;
  L.nb = nb;
  L.total_slots = total_slots;
  L.blocks.resize(nb);
  L.perm.resize(nv);
  CKS(cudaMemcpyAsync(&too, d_too, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(L.blocks.data(), out.blocks, sizeof(BlockDesc) * nb, cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(L.perm.data(), out.perm, sizeof(int) * nv, cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  if (too) return "block has too many local vertices (limit 32767)";
  L.iperm.assign(nv, 0);
  for (int v = 0; v < nv; ++v) L.iperm[L.perm[v]] = v;
  double sl = 0, hl = 0;
  for (const BlockDesc& d : L.blocks) {
    L.max_slots = std::max(L.max_slots, d.nslots);
    L.max_owned = std::max(L.max_owned, d.nowned);
    L.max_halo = std::max(L.max_halo, d.nhalo);
    L.max_local = std::max(L.max_local, d.nowned + d.nhalo);
    sl += d.nslots;
    hl += d.nhalo;
  }
  L.mean_slots_per_block = sl / nb;
  L.mean_halo_per_block = hl / nb;
  L.ninst = 1;
  L.blk_inst.assign(nb, 0);
  L.inst_bbeg = {0, nb};
  L.inst_vbeg = {0, nv};
  return "";
}

}  // namespace

void Built3D::release() {
  void* ps[] = {blocks, coef, lv, halo, nbr_off, nbr, vblock, perm, slot_elem, xyz, tets, M6};
  for (void* p : ps)
    if (p) cudaFree(p);
  *this = Built3D();
}

std::string build_layout3d_device(int nv, const float* xyz, int nt, const int* tets, const float* M, int mcomp,
                                  const int* labels, int nb, cudaStream_t st, Built3D& out, Layout& L) {
  struct Range {
    Range() { nvtxRangePushA("eikonal: device setup"); }
    ~Range() { nvtxRangePop(); }
  } nvtx_range;
  out.release();
  L = Layout();
  if (nv <= 0 || nt <= 0 || nb <= 0) return "empty mesh";
  if (mcomp != 1 && mcomp != 6) return "metric entries per tet must be 1 or 6";
  for (int v = 0; v < nv; ++v)
    if (labels[v] < 0 || labels[v] >= nb) return "partition label out of range";
  Scratch S;
  std::string e;
  // inputs, kept: a speed change recomputes the metric terms from them
  if (!(e = keep(out.xyz, 3 * (size_t)nv)).empty() || !(e = keep(out.tets, 4 * (size_t)nt)).empty() ||
      !(e = keep(out.M6, (size_t)mcomp * nt)).empty())
    return e;
  out.mcomp = mcomp;
  int* d_lab;
  if (!(e = S.get(d_lab, nv)).empty()) return e;
  CKS(cudaMemcpyAsync(out.xyz, xyz, sizeof(float) * 3 * (size_t)nv, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(out.tets, tets, sizeof(int) * 4 * (size_t)nt, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(out.M6, M, sizeof(float) * mcomp * (size_t)nt, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(d_lab, labels, sizeof(int) * nv, cudaMemcpyHostToDevice, st));

  // 1. owned-vertex renumbering
  int* d_vbase;
  if (!(e = renumber_device(S, d_lab, nv, nb, st, out, d_vbase)).empty()) return e;

  // 2. element slots and neighbour pairs
  int *d_nslot, *d_npair, *d_slot_off, *d_pair_off;
  if (!(e = S.get(d_nslot, nt + 1)).empty() || !(e = S.get(d_npair, nt + 1)).empty() ||
      !(e = S.get(d_slot_off, nt + 1)).empty() || !(e = S.get(d_pair_off, nt + 1)).empty())
    return e;
  CKS(cudaMemsetAsync(d_nslot + nt, 0, sizeof(int), st));
  CKS(cudaMemsetAsync(d_npair + nt, 0, sizeof(int), st));
  k_tet_counts<<<grid_for(nt), kThreads, 0, st>>>(out.tets, d_lab, nt, d_nslot, d_npair);
  if (!(e = exclusive_scan(S, d_nslot, d_slot_off, nt + 1, st)).empty()) return e;
  if (!(e = exclusive_scan(S, d_npair, d_pair_off, nt + 1, st)).empty()) return e;
  int np = 0, npairs = 0;
  CKS(cudaMemcpyAsync(&np, d_slot_off + nt, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(&npairs, d_pair_off + nt, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  unsigned *d_key, *d_key_s;
  int *d_val, *d_val_s;
  unsigned long long *d_pairs, *d_pairs_s;
  if (!(e = S.get(d_key, np)).empty() || !(e = S.get(d_key_s, np)).empty() || !(e = S.get(d_val, np)).empty() ||
      !(e = S.get(d_val_s, np)).empty() || !(e = S.get(d_pairs, npairs)).empty() ||
      !(e = S.get(d_pairs_s, npairs)).empty())
    return e;
  k_tet_emit<<<grid_for(nt), kThreads, 0, st>>>(out.tets, d_lab, nt, d_slot_off, d_pair_off, d_key, d_val, d_pairs);
  if (!(e = sort_pairs(S, d_key, d_key_s, d_val, d_val_s, np, bits_for(2ull * (unsigned long long)nb), st)).empty())
    return e;
  int *d_keycnt, *d_keybeg, *d_pad, *d_slot_begin;
  if (!(e = S.get(d_keycnt, 2 * (size_t)nb + 1)).empty() || !(e = S.get(d_keybeg, 2 * (size_t)nb + 1)).empty() ||
      !(e = S.get(d_pad, nb + 1)).empty() || !(e = S.get(d_slot_begin, nb + 1)).empty())
    return e;
  CKS(cudaMemsetAsync(d_keycnt, 0, sizeof(int) * (2 * (size_t)nb + 1), st));
  k_count_keys<<<grid_for(np), kThreads, 0, st>>>(d_key_s, np, d_keycnt);
  if (!(e = exclusive_scan(S, d_keycnt, d_keybeg, 2 * nb + 1, st)).empty()) return e;
  CKS(cudaMemsetAsync(d_pad + nb, 0, sizeof(int), st));
  k_pad_counts<<<grid_for(nb), kThreads, 0, st>>>(d_keycnt, nb, d_pad);
  if (!(e = exclusive_scan(S, d_pad, d_slot_begin, nb + 1, st)).empty()) return e;
  int total_slots = 0;
  CKS(cudaMemcpyAsync(&total_slots, d_slot_begin + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (!(e = keep(out.blocks, nb)).empty()) return e;
  k_block_desc<<<grid_for(nb), kThreads, 0, st>>>(d_keycnt, d_vbase, d_slot_begin, nb, out.blocks);
  CKS(cudaStreamSynchronize(st));
  if (!(e = keep(out.slot_elem, total_slots)).empty() || !(e = keep(out.lv, 4 * (size_t)total_slots)).empty() ||
      !(e = keep(out.coef, 6 * (size_t)total_slots)).empty())
    return e;
  CKS(cudaMemsetAsync(out.slot_elem, 0xff, sizeof(int) * (size_t)total_slots, st));
  CKS(cudaMemsetAsync(out.lv, 0, sizeof(uint16_t) * 4 * (size_t)total_slots, st));
  CKS(cudaMemsetAsync(out.coef, 0, sizeof(float) * 6 * (size_t)total_slots, st));

  // 3. halo lists
  int *d_slot_of, *d_cnt1;
  unsigned long long *d_hk, *d_hk_s, *d_hk_u;
  if (!(e = S.get(d_slot_of, np)).empty() || !(e = S.get(d_hk, 4 * (size_t)np)).empty() ||
      !(e = S.get(d_hk_s, 4 * (size_t)np)).empty() || !(e = S.get(d_hk_u, 4 * (size_t)np)).empty() ||
      !(e = S.get(d_cnt1, 1)).empty())
    return e;
  k_place<<<grid_for(np), kThreads, 0, st>>>(d_key_s, d_val_s, np, d_keybeg, out.blocks, out.tets, d_lab, out.perm,
                                             out.slot_elem, d_slot_of, d_hk);
  int nu = 0;
  if (!(e = sort_unique(S, d_hk, d_hk_s, d_hk_u, 4 * np, d_cnt1, &nu, st)).empty()) return e;
  int *d_hcnt, *d_hbeg, *d_too;
  if (!(e = S.get(d_hcnt, nb + 1)).empty() || !(e = S.get(d_hbeg, nb + 1)).empty() || !(e = S.get(d_too, 1)).empty())
    return e;
  CKS(cudaMemsetAsync(d_hcnt, 0, sizeof(int) * (nb + 1), st));
  CKS(cudaMemsetAsync(d_too, 0, sizeof(int), st));
  k_count_halo<<<grid_for(nu), kThreads, 0, st>>>(d_hk_u, nu, d_hcnt);
  if (!(e = exclusive_scan(S, d_hcnt, d_hbeg, nb + 1, st)).empty()) return e;
  int nhalo_total = 0;
  CKS(cudaMemcpyAsync(&nhalo_total, d_hbeg + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  if (!(e = keep(out.halo, nhalo_total)).empty()) return e;
  k_halo_ids<<<grid_for(nu), kThreads, 0, st>>>(d_hk_u, nu, out.halo);  // the owned-corner key sorts last
  k_halo_desc<<<grid_for(nb), kThreads, 0, st>>>(d_hcnt, d_hbeg, nb, out.blocks, d_too);

  // 4. corner local ids and metric edge products
  k_slot_fill<<<grid_for(np), kThreads, 0, st>>>(d_key_s, d_val_s, d_slot_of, np, out.blocks, out.tets, d_lab,
                                                 out.perm, out.halo, out.xyz, out.M6, out.mcomp, out.lv,
                                                 out.coef);

  // 5. block-neighbour graph (sorted unique pairs -> CSR)
  int nn = 0;
  if (!(e = neighbour_graph(S, d_pairs, d_pairs_s, npairs, nb, d_cnt1, st, out, &nn)).empty()) return e;
  CKS(cudaGetLastError());
  if (!(e = host_part(3, nv, nt, nb, total_slots, out, d_too, st, L)).empty()) return e;
  out.total_slots = total_slots;
  out.nhalo = nhalo_total;
  out.nnbr = nn;
  return "";
}

}  // namespace eikgb

namespace eikgb {

std::string build_layout2d_device(int nv, const TriPrep& P, const float* speeds, const int* labels, int nb,
                                  cudaStream_t st, Built3D& out, Layout& L) {
  struct Range {
    Range() { nvtxRangePushA("eikonal: device setup 2D"); }
    ~Range() { nvtxRangePop(); }
  } nvtx_range;
  out.release();
  L = Layout();
  const int nf = P.nf;
  const int nvf = (int)(P.vf_verts.size() / 3);
  if (nv <= 0 || nf <= 0 || nb <= 0) return "empty mesh";
  for (int v = 0; v < nv; ++v)
    if (labels[v] < 0 || labels[v] >= nb) return "partition label out of range";
  Scratch S;
  std::string e;
  out.dim = 2;
  out.mcomp = 1;
  // kept: faces (tets) and face speeds (M6) for later speed changes
  if (!(e = keep(out.tets, 3 * (size_t)nf)).empty() || !(e = keep(out.M6, (size_t)nf)).empty()) return e;
  int *d_lab, *d_vf_off, *d_vf_verts;
  unsigned char* d_obt;
  float *d_edges, *d_vf_edges;
  if (!(e = S.get(d_lab, nv)).empty() || !(e = S.get(d_obt, nf)).empty() || !(e = S.get(d_vf_off, nf + 1)).empty() ||
      !(e = S.get(d_vf_verts, 3 * (size_t)std::max(nvf, 1))).empty() || !(e = S.get(d_edges, 3 * (size_t)nf)).empty() ||
      !(e = S.get(d_vf_edges, 3 * (size_t)std::max(nvf, 1))).empty())
    return e;
  std::vector<float> sp(nf, 1.0f);
  if (speeds) std::copy(speeds, speeds + nf, sp.begin());
  CKS(cudaMemcpyAsync(out.tets, P.faces.data(), sizeof(int) * 3 * (size_t)nf, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(out.M6, sp.data(), sizeof(float) * (size_t)nf, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(d_lab, labels, sizeof(int) * nv, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(d_obt, P.obtuse.data(), (size_t)nf, cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(d_vf_off, P.vf_off.data(), sizeof(int) * (nf + 1), cudaMemcpyHostToDevice, st));
  CKS(cudaMemcpyAsync(d_edges, P.edges.data(), sizeof(float) * 3 * (size_t)nf, cudaMemcpyHostToDevice, st));
  if (nvf > 0) {
    CKS(cudaMemcpyAsync(d_vf_verts, P.vf_verts.data(), sizeof(int) * 3 * (size_t)nvf, cudaMemcpyHostToDevice, st));
    CKS(cudaMemcpyAsync(d_vf_edges, P.vf_edges.data(), sizeof(float) * 3 * (size_t)nvf, cudaMemcpyHostToDevice, st));
  }

  // 1. owned-vertex renumbering
  int* d_vbase;
  if (!(e = renumber_device(S, d_lab, nv, nb, st, out, d_vbase)).empty()) return e;

  // 2. element slots (inside, shared, virtual per block) and neighbour pairs
  int *d_nslot, *d_npair, *d_slot_off, *d_pair_off;
  if (!(e = S.get(d_nslot, nf + 1)).empty() || !(e = S.get(d_npair, nf + 1)).empty() ||
      !(e = S.get(d_slot_off, nf + 1)).empty() || !(e = S.get(d_pair_off, nf + 1)).empty())
    return e;
  CKS(cudaMemsetAsync(d_nslot + nf, 0, sizeof(int), st));
  CKS(cudaMemsetAsync(d_npair + nf, 0, sizeof(int), st));
  k_face_counts<<<grid_for(nf), kThreads, 0, st>>>(out.tets, d_lab, d_obt, d_vf_off, nf, d_nslot, d_npair);
  if (!(e = exclusive_scan(S, d_nslot, d_slot_off, nf + 1, st)).empty()) return e;
  if (!(e = exclusive_scan(S, d_npair, d_pair_off, nf + 1, st)).empty()) return e;
  int np = 0, npairs = 0;
  CKS(cudaMemcpyAsync(&np, d_slot_off + nf, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(&npairs, d_pair_off + nf, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  unsigned *d_key, *d_key_s;
  int *d_val, *d_val_s;
  unsigned long long *d_pairs, *d_pairs_s;
  if (!(e = S.get(d_key, np)).empty() || !(e = S.get(d_key_s, np)).empty() || !(e = S.get(d_val, np)).empty() ||
      !(e = S.get(d_val_s, np)).empty() || !(e = S.get(d_pairs, npairs)).empty() ||
      !(e = S.get(d_pairs_s, npairs)).empty())
    return e;
  k_face_emit<<<grid_for(nf), kThreads, 0, st>>>(out.tets, d_lab, d_obt, d_vf_off, nf, d_slot_off, d_pair_off, d_key,
                                                 d_val, d_pairs);
  if (!(e = sort_pairs(S, d_key, d_key_s, d_val, d_val_s, np, bits_for(3ull * (unsigned long long)nb), st)).empty())
    return e;
  int *d_keycnt, *d_keybeg, *d_pad, *d_slot_begin, *d_nin, *d_nrest, *d_inbase, *d_restbase;
  if (!(e = S.get(d_keycnt, 3 * (size_t)nb + 1)).empty() || !(e = S.get(d_keybeg, 3 * (size_t)nb + 1)).empty() ||
      !(e = S.get(d_pad, nb + 1)).empty() || !(e = S.get(d_slot_begin, nb + 1)).empty() ||
      !(e = S.get(d_nin, nb + 1)).empty() || !(e = S.get(d_nrest, nb + 1)).empty() ||
      !(e = S.get(d_inbase, nb + 1)).empty() || !(e = S.get(d_restbase, nb + 1)).empty())
    return e;
  CKS(cudaMemsetAsync(d_keycnt, 0, sizeof(int) * (3 * (size_t)nb + 1), st));
  k_count_keys<<<grid_for(np), kThreads, 0, st>>>(d_key_s, np, d_keycnt);
  if (!(e = exclusive_scan(S, d_keycnt, d_keybeg, 3 * nb + 1, st)).empty()) return e;
  CKS(cudaMemsetAsync(d_pad + nb, 0, sizeof(int), st));
  CKS(cudaMemsetAsync(d_nin + nb, 0, sizeof(int), st));
  CKS(cudaMemsetAsync(d_nrest + nb, 0, sizeof(int), st));
  k_pad_counts3<<<grid_for(nb), kThreads, 0, st>>>(d_keycnt, nb, d_pad, d_nin, d_nrest);
  if (!(e = exclusive_scan(S, d_pad, d_slot_begin, nb + 1, st)).empty()) return e;
  if (!(e = exclusive_scan(S, d_nin, d_inbase, nb + 1, st)).empty()) return e;
  if (!(e = exclusive_scan(S, d_nrest, d_restbase, nb + 1, st)).empty()) return e;
  int total_slots = 0, ninside_total = 0;
  CKS(cudaMemcpyAsync(&total_slots, d_slot_begin + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(&ninside_total, d_inbase + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (!(e = keep(out.blocks, nb)).empty()) return e;
  k_block_desc2d<<<grid_for(nb), kThreads, 0, st>>>(d_keycnt, d_vbase, d_slot_begin, nb, out.blocks);
  CKS(cudaStreamSynchronize(st));
  if (!(e = keep(out.slot_elem, total_slots)).empty() || !(e = keep(out.lv, 4 * (size_t)total_slots)).empty() ||
      !(e = keep(out.coef, 4 * (size_t)total_slots)).empty())
    return e;
  CKS(cudaMemsetAsync(out.slot_elem, 0xff, sizeof(int) * (size_t)total_slots, st));
  CKS(cudaMemsetAsync(out.lv, 0, sizeof(uint16_t) * 4 * (size_t)total_slots, st));
  CKS(cudaMemsetAsync(out.coef, 0, sizeof(float) * 4 * (size_t)total_slots, st));

  // 3. slots, halo keys and the blockVertMapping entries
  int *d_slot_of, *d_cnt1, *d_ekey, *d_ekey_s;
  unsigned long long *d_hk, *d_hk_s, *d_hk_u, *d_eval, *d_eval_s;
  const size_t ne3 = 3 * (size_t)np;
  if (!(e = S.get(d_slot_of, np)).empty() || !(e = S.get(d_hk, ne3)).empty() || !(e = S.get(d_hk_s, ne3)).empty() ||
      !(e = S.get(d_hk_u, ne3)).empty() || !(e = S.get(d_cnt1, 1)).empty() || !(e = S.get(d_ekey, ne3)).empty() ||
      !(e = S.get(d_ekey_s, ne3)).empty() || !(e = S.get(d_eval, ne3)).empty() || !(e = S.get(d_eval_s, ne3)).empty())
    return e;
  k_place2d<<<grid_for(np), kThreads, 0, st>>>(d_key_s, d_val_s, np, d_keybeg, out.blocks, d_inbase, d_restbase,
                                               ninside_total, out.tets, d_vf_verts, d_lab, out.perm, out.slot_elem,
                                               d_slot_of, d_hk, d_ekey, d_eval);
  int nu = 0;
  if (!(e = sort_unique(S, d_hk, d_hk_s, d_hk_u, (int)ne3, d_cnt1, &nu, st)).empty()) return e;
  int *d_hcnt, *d_hbeg, *d_too;
  if (!(e = S.get(d_hcnt, nb + 1)).empty() || !(e = S.get(d_hbeg, nb + 1)).empty() || !(e = S.get(d_too, 1)).empty())
    return e;
  CKS(cudaMemsetAsync(d_hcnt, 0, sizeof(int) * (nb + 1), st));
  CKS(cudaMemsetAsync(d_too, 0, sizeof(int), st));
  k_count_halo<<<grid_for(nu), kThreads, 0, st>>>(d_hk_u, nu, d_hcnt);
  if (!(e = exclusive_scan(S, d_hcnt, d_hbeg, nb + 1, st)).empty()) return e;
  int nhalo_total = 0;
  CKS(cudaMemcpyAsync(&nhalo_total, d_hbeg + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  if (!(e = keep(out.halo, nhalo_total)).empty()) return e;
  k_halo_ids<<<grid_for(nu), kThreads, 0, st>>>(d_hk_u, nu, out.halo);
  k_halo_desc<<<grid_for(nb), kThreads, 0, st>>>(d_hcnt, d_hbeg, nb, out.blocks, d_too);

  // 4. corner local ids, edge lengths, inverse speeds
  k_slot_fill2d<<<grid_for(np), kThreads, 0, st>>>(d_val_s, d_slot_of, d_key_s, np, out.blocks, out.tets, d_vf_verts,
                                                   d_edges, d_vf_edges, out.M6, d_lab, out.perm, out.halo, out.lv,
                                                   out.coef);

  // 5. copies the reference never refreshes (bit 15): per vertex its entries in
  // blockVertMapping order (a stable sort of the entries, emitted in that order, by
  // vertex), own-block ranks by a segmented scan, then the cap rule
  if (!(e = sort_pairs(S, d_ekey, d_ekey_s, d_eval, d_eval_s, (int)ne3, bits_for((unsigned long long)nv), st)).empty())
    return e;
  int *d_own, *d_ownrank, *d_vbeg, *d_first;
  if (!(e = S.get(d_own, ne3)).empty() || !(e = S.get(d_ownrank, ne3)).empty() || !(e = S.get(d_vbeg, nv)).empty() ||
      !(e = S.get(d_first, nv)).empty())
    return e;
  k_own_flags<<<grid_for((long long)ne3), kThreads, 0, st>>>(d_ekey_s, d_eval_s, d_lab, (int)ne3, d_own);
  {
    size_t tb = 0;
    CKS(cub::DeviceScan::ExclusiveSumByKey(nullptr, tb, d_ekey_s, d_own, d_ownrank, (int)ne3, cuda::std::equal_to<int>(), st));
    unsigned char* tmp;
    if (!(e = S.get(tmp, tb)).empty()) return e;
    CKS(cub::DeviceScan::ExclusiveSumByKey(tmp, tb, d_ekey_s, d_own, d_ownrank, (int)ne3, cuda::std::equal_to<int>(), st));
  }
  CKS(cudaMemsetAsync(d_first, 0xff, sizeof(int) * nv, st));
  k_seg_begin<<<grid_for((long long)ne3), kThreads, 0, st>>>(d_ekey_s, (int)ne3, d_vbeg);
  k_first_own<<<grid_for((long long)ne3), kThreads, 0, st>>>(d_ekey_s, d_own, d_ownrank, d_vbeg, (int)ne3, d_first);
  k_live2d<<<grid_for((long long)ne3), kThreads, 0, st>>>(d_ekey_s, d_eval_s, d_own, d_ownrank, d_vbeg, d_first,
                                                          (int)ne3, kSlotCap2D, out.lv);

  // 6. block-neighbour graph from the shared faces
  int nn = 0;
  if (!(e = neighbour_graph(S, d_pairs, d_pairs_s, npairs, nb, d_cnt1, st, out, &nn)).empty()) return e;
  CKS(cudaGetLastError());
  if (!(e = host_part(2, nv, nf, nb, total_slots, out, d_too, st, L)).empty()) return e;
  out.total_slots = total_slots;
  out.nhalo = nhalo_total;
  out.nnbr = nn;
  return "";
}

}  // namespace eikgb
