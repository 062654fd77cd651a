// ref_gpu_driver.cpp — TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own CUDA kernels (compiled from the reference tree into
// _ref/ref3d.cubin and _ref/ref2d.cubin by build_oracle.py) under a restatement
// of the reference's host loop, on the padded layouts the CPU oracle builds.
// The GPU parity tests compare the product against these runs bit for bit.
//
//   3D loop: src/core3d/cuda/meshFIM3dEikonal.cu:285-566 (GenerateData)
//   2D loop: src/core2d/cuda/meshFIM2d_eikonal.cu:349-864 (GenerateData)
//
// Launch shapes are the reference's: one CUDA block per active mesh block with
// one thread per element slot (so a block may hold at most 1024 slots, the
// reference's own limit), host round trips every iteration.
#include <cuda_runtime.h>

#include <chrono>
#include <string>

#include "oracle_scheme.hpp"

using namespace oracle;

namespace {

std::string g_err;
double g_loop_ms = 0;  // wall time of the last solve's outer loop (3D or 2D)

#define RCK(x)                                                         \
  do {                                                                 \
    cudaError_t e_ = (x);                                              \
    if (e_ != cudaSuccess) {                                           \
      g_err = std::string(#x) + ": " + cudaGetErrorString(e_);         \
      return -2;                                                       \
    }                                                                  \
  } while (0)

struct Lib {
  cudaLibrary_t lib = nullptr;
  std::string path;
};
Lib g_lib3, g_lib2;

int load(Lib& L, const char* path) {
  if (L.lib && L.path == path) return 0;
  if (L.lib) cudaLibraryUnload(L.lib);
  L.lib = nullptr;
  RCK(cudaLibraryLoadFromFile(&L.lib, path, nullptr, nullptr, 0, nullptr, nullptr, 0));
  L.path = path;
  return 0;
}

int kernel(Lib& L, const char* name, cudaKernel_t* k) {
  RCK(cudaLibraryGetKernel(k, L.lib, name));
  return 0;
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  ~DBuf() { if (p) cudaFree(p); }
  int alloc(size_t n) {
    RCK(cudaMalloc((void**)&p, sizeof(T) * (n + 64)));  // slack: the reference reads one past some lists
    RCK(cudaMemset(p, 0, sizeof(T) * (n + 64)));
    return 0;
  }
  int put(const T* h, size_t n) { RCK(cudaMemcpy(p, h, sizeof(T) * n, cudaMemcpyHostToDevice)); return 0; }
  int get(T* h, size_t n) const { RCK(cudaMemcpy(h, p, sizeof(T) * n, cudaMemcpyDeviceToHost)); return 0; }
};

int launch(cudaKernel_t k, unsigned grid, unsigned block, size_t smem, void** args) {
  if (grid == 0) return 0;
  if (smem > 48 * 1024) RCK(cudaFuncSetAttribute((const void*)k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  RCK(cudaLaunchKernel((const void*)k, dim3(grid), dim3(block), args, smem, 0));
  RCK(cudaGetLastError());
  return 0;
}

#define TRY(x)            \
  do {                    \
    int r_ = (x);         \
    if (r_) return r_;    \
  } while (0)

}  // namespace

extern "C" {

const char* refgpu_last_error(void) { return g_err.c_str(); }

// Wall time (ms) of the outer loop of the last refgpu_solve3d: kernels and the
// reference's per-iteration host round trips, without the layout set-up.
double refgpu_last_loop_ms(void) { return g_loop_ms; }

// Element-wise reference local solver: out[i] = localSolverTet1(in[9i..9i+8]).
int refgpu_tet_local_solver(const char* cubin3d, const float* in, float* out, int n) {
  TRY(load(g_lib3, cubin3d));
  cudaKernel_t k;
  TRY(kernel(g_lib3, "ref3d_local_solver", &k));
  DBuf<float> din, dout;
  TRY(din.alloc(9 * (size_t)n));
  TRY(dout.alloc(n));
  TRY(din.put(in, 9 * (size_t)n));
  float* a0 = din.p;
  float* a1 = dout.p;
  void* args[] = {&a0, &a1, &n};
  TRY(launch(k, (n + 127) / 128, 128, 0, args));
  RCK(cudaDeviceSynchronize());
  TRY(dout.get(out, n));
  return 0;
}

// Whole 3D solve with the reference kernels.  Returns iterations, -1 for inputs
// the reference cannot launch (more than 1024 element slots or 1024 vertices in a
// block), -2 for CUDA errors (refgpu_last_error).
int refgpu_solve3d(const char* cubin3d, int nv, const float* xyz, int nt, const int* tets, const float* M,
                   const int* part, int nb, const int* seeds, int nseeds, int max_iters, float* out_final,
                   float* history, int hist_cap, long long* updates, int* max_tets) {
  Oracle3D<float> O;
  O.nv = nv; O.nt = nt; O.nb = nb; O.xyz = xyz; O.tets = tets; O.M = M; O.part = part;
  O.partition();
  O.layout();
  if (max_tets) *max_tets = O.maxTets;
  if (O.maxTets > 1024 || O.maxInVert > 1024) {
    g_err = "block exceeds the reference's 1024-thread launch";
    return -1;
  }
  TRY(load(g_lib3, cubin3d));
  cudaKernel_t kfim, kchk, kcopy, kred;
  TRY(kernel(g_lib3, "ref3d_fim", &kfim));
  TRY(kernel(g_lib3, "ref3d_check", &kchk));
  TRY(kernel(g_lib3, "ref3d_copyout", &kcopy));
  TRY(kernel(g_lib3, "ref3d_reduce", &kred));
  const int maxT = O.maxTets, maxIn = O.maxInVert, mapIn = std::max(O.maxMapIn, 1), mapOut = std::max(O.maxMapOut, 1);
  const size_t nslot = (size_t)nb * maxT;
  // GetTetMem / GetVertMem arrays (meshFIM3dEikonal.cu:680-923), padding as the reference writes it
  std::vector<float> m0(3 * nslot, 0.f), m1(3 * nslot, 0.f);
  for (size_t s = 0; s < nslot; ++s)
    for (int k = 0; k < 3; ++k) { m0[3 * s + k] = O.gram[6 * s + k]; m1[3 * s + k] = O.gram[6 * s + 3 + k]; }
  std::vector<int> vm((size_t)nb * maxIn * mapIn), vmo((size_t)nb * maxIn * mapOut);
  for (int b = 0; b < nb; ++b) {
    for (int k = 0; k < maxIn; ++k)
      for (int j = 0; j < mapIn; ++j) {
        const size_t i = ((size_t)b * maxIn + k) * mapIn + j;
        const int a = (O.maxMapIn > 0) ? O.vmIn[i] : -1;
        vm[i] = (a >= 0) ? a : -1 + b * maxT * 4;
      }
    for (int k = 0; k < maxIn; ++k)
      for (int j = 0; j < mapOut; ++j) {
        const size_t i = ((size_t)b * maxIn + k) * mapOut + j;
        vmo[i] = (O.maxMapOut > 0) ? O.vmOut[i] : -1;
      }
  }
  std::vector<float> tT(O.slotT.begin(), O.slotT.end());
  std::vector<char> blockCon(nb, 1);
  std::vector<int> label(nb, 0), bsz(O.blockSize);
  std::set<int> activeSet;
  for (int i = 0; i < nseeds; ++i) {
    const int s = seeds[i];
    activeSet.insert(part[s]);
    blockCon[part[s]] = 0;
    label[part[s]] = 1;
    for (int a : O.vmap[s]) tT[a] = 0.f;
  }
  DBuf<float> d_m0, d_m1, d_tT, d_vT, d_sp;
  DBuf<int> d_vm, d_vmo, d_bs, d_al;
  DBuf<char> d_con, d_bc;
  TRY(d_m0.alloc(3 * nslot)); TRY(d_m1.alloc(3 * nslot)); TRY(d_tT.alloc(4 * nslot));
  TRY(d_vT.alloc((size_t)nb * maxIn)); TRY(d_sp.alloc(nslot));
  TRY(d_vm.alloc(vm.size())); TRY(d_vmo.alloc(vmo.size())); TRY(d_bs.alloc(nb)); TRY(d_al.alloc(nb));
  TRY(d_con.alloc((size_t)nb * maxIn)); TRY(d_bc.alloc(nb));
  TRY(d_m0.put(m0.data(), m0.size())); TRY(d_m1.put(m1.data(), m1.size())); TRY(d_tT.put(tT.data(), tT.size()));
  TRY(d_vm.put(vm.data(), vm.size())); TRY(d_vmo.put(vmo.data(), vmo.size())); TRY(d_bs.put(bsz.data(), nb));
  TRY(d_bc.put(blockCon.data(), nb));
  std::vector<int> act(activeSet.begin(), activeSet.end()), alist(nb, 0), fresh;
  std::vector<float> hvT((size_t)nb * maxIn);
  int iters = 0;
  size_t total = 0;
  long long nupd = 0;
  float3* pm0 = (float3*)d_m0.p; float3* pm1 = (float3*)d_m1.p; float4* ptT = (float4*)d_tT.p;
  float* pvT = d_vT.p; float* psp = d_sp.p; int* pvm = d_vm.p; int* pvmo = d_vmo.p; int* pbs = d_bs.p;
  bool* pcon = (bool*)d_con.p; bool* pbc = (bool*)d_bc.p; int* pal = d_al.p;
  int nIter = 2;
  const size_t smem = 16 * (size_t)maxT + 4 * (size_t)maxIn * mapIn;
  const auto t_loop = std::chrono::steady_clock::now();
  while (!act.empty()) {
    if (++total > (size_t)max_iters) break;
    int na = (int)act.size();
    std::copy(act.begin(), act.end(), alist.begin());
    TRY(d_al.put(alist.data(), nb));
    void* a_fim[] = {&pm0, &pm1, &ptT, &pvT, &psp, &pvm, &pvmo, &pbs, &pcon, &pal,
                     (void*)&maxIn, (void*)&mapIn, (void*)&mapOut, &nIter};
    TRY(launch(kfim, na, maxT, smem, a_fim));
    int maxTv = maxT;
    void* a_cp[] = {&ptT, &pvT, &pvm, &pvmo, &pbs, &pal, (void*)&maxIn, &maxTv, (void*)&mapIn, (void*)&mapOut};
    TRY(launch(kcopy, na, maxIn, 0, a_cp));
    void* a_red[] = {&pcon, &pbc, &pal, &na, &pbs};
    TRY(launch(kred, na, maxIn, 0, a_red));
    TRY(d_bc.get(blockCon.data(), nb));
    for (int b : act) nupd += (long long)bsz[b] * nIter;
    for (int b : act) label[b] = blockCon[b] ? 0 : 1;
    fresh.clear();
    for (int b : act)
      if (blockCon[b])
        for (int nbk : O.blkNbrs[b])
          if (label[nbk] == 0) { label[nbk] = 1; fresh.push_back(nbk); }
    std::vector<int> next;
    for (int b : act) if (!blockCon[b]) next.push_back(b);
    if (!fresh.empty()) {
      int nf = (int)fresh.size();
      std::copy(fresh.begin(), fresh.end(), alist.begin());
      TRY(d_al.put(alist.data(), nf));
      void* a_chk[] = {&pm0, &pm1, &ptT, &psp, &pvm, &pvmo, &pbs, &pcon, &pal,
                       (void*)&maxIn, (void*)&mapIn, (void*)&mapOut};
      TRY(launch(kchk, nf, maxT, smem, a_chk));
      void* a_red2[] = {&pcon, &pbc, &pal, &nf, &pbs};
      TRY(launch(kred, nf, maxIn, 0, a_red2));
      TRY(d_bc.get(blockCon.data(), nb));
      for (int b : fresh) {
        nupd += bsz[b];
        if (!blockCon[b]) next.push_back(b); else label[b] = 0;
      }
    }
    TRY(d_vT.get(hvT.data(), hvT.size()));
    act.swap(next);
    ++iters;
    if (history && iters <= hist_cap)
      for (int b = 0; b < nb; ++b)
        for (size_t j = 0; j < O.inVerts[b].size(); ++j)
          history[(size_t)(iters - 1) * nv + O.inVerts[b][j]] = hvT[(size_t)b * maxIn + j];
  }
  TRY(d_vT.get(hvT.data(), hvT.size()));
  g_loop_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_loop).count();
  for (int b = 0; b < nb; ++b)
    for (size_t j = 0; j < O.inVerts[b].size(); ++j) out_final[O.inVerts[b][j]] = hvT[(size_t)b * maxIn + j];
  if (updates) *updates = nupd;
  return iters;
}

// Whole 2D solve with the reference kernels (same inputs as oracle2d_solve).
int refgpu_solve2d(const char* cubin2d, int nv, const float* xyz, int nf, const int* faces, const float* speed_inv,
                   const uint8_t* obtuse, const int* vf_off, const int* vf_verts, const float* vf_speed_inv,
                   const int* part, int nb, const int* seeds, int nseeds, const float* init_vals, int max_iters,
                   float* out_final, float* history, int hist_cap, long long* updates, int* max_faces) {
  Oracle2D<float> O;
  O.nv = nv; O.nf = nf; O.nb = nb; O.xyz = xyz; O.faces = faces; O.speedInv = speed_inv; O.obtuse = obtuse;
  O.vfOff = vf_off; O.vfVerts = vf_verts; O.vfSpeedInv = vf_speed_inv; O.part = part;
  O.partition();
  O.layout(seeds, nseeds);
  if (max_faces) *max_faces = O.maxFaces;
  if (O.maxFaces > 1024 || O.maxVert > 64) {
    g_err = "block exceeds the reference's launch or flag layout";
    return -1;
  }
  TRY(load(g_lib2, cubin2d));
  cudaKernel_t kfim, kchk, kred;
  TRY(kernel(g_lib2, "ref2d_fim", &kfim));
  TRY(kernel(g_lib2, "ref2d_check", &kchk));
  TRY(kernel(g_lib2, "ref2d_reduce", &kred));
  const int maxF = O.maxFaces, maxV = O.maxVert;
  const size_t nslot = (size_t)nb * maxF;
  std::vector<float> e0(nslot, 0.f), e1(nslot, 0.f), e2(nslot, 0.f), sp(nslot, 0.f);
  for (size_t s = 0; s < nslot; ++s) { e0[s] = O.edge[3 * s]; e1[s] = O.edge[3 * s + 1]; e2[s] = O.edge[3 * s + 2]; sp[s] = O.spd[s]; }
  std::vector<int> vm((size_t)nb * maxV * 6), vmo((size_t)nb * maxV * 6);
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < maxV; ++k)
      for (int j = 0; j < 6; ++j) {
        const size_t i = ((size_t)b * maxV + k) * 6 + j;
        vm[i] = (O.vmIn[i] >= 0) ? O.vmIn[i] : -1 + b * maxF * 3;
        vmo[i] = O.vmOut[i];
      }
  std::vector<int> blockCon(nb, 1), label(nb, 0), bsz(O.blockSize);
  std::set<int> activeSet;
  for (int i = 0; i < nseeds; ++i) { activeSet.insert(part[seeds[i]]); label[part[seeds[i]]] = 1; blockCon[part[seeds[i]]] = 0; }
  DBuf<float> d_tm, d_tmo, d_e0, d_e1, d_e2, d_sp;
  DBuf<int> d_vm, d_vmo, d_bs, d_con, d_bc, d_al;
  TRY(d_tm.alloc(3 * nslot)); TRY(d_tmo.alloc(3 * nslot)); TRY(d_e0.alloc(nslot)); TRY(d_e1.alloc(nslot));
  TRY(d_e2.alloc(nslot)); TRY(d_sp.alloc(nslot)); TRY(d_vm.alloc(vm.size())); TRY(d_vmo.alloc(vmo.size()));
  TRY(d_bs.alloc(nb)); TRY(d_con.alloc((size_t)nb * 64)); TRY(d_bc.alloc(nb)); TRY(d_al.alloc(nb));
  TRY(d_tm.put(O.triMem.data(), 3 * nslot)); TRY(d_tmo.put(O.triMem.data(), 3 * nslot));
  TRY(d_e0.put(e0.data(), nslot)); TRY(d_e1.put(e1.data(), nslot)); TRY(d_e2.put(e2.data(), nslot));
  TRY(d_sp.put(sp.data(), nslot)); TRY(d_vm.put(vm.data(), vm.size())); TRY(d_vmo.put(vmo.data(), vmo.size()));
  TRY(d_bs.put(bsz.data(), nb)); TRY(d_bc.put(blockCon.data(), nb));
  std::vector<int> act(activeSet.begin(), activeSet.end()), alist(nb, 0);
  std::vector<float> htm(3 * nslot), prev(init_vals, init_vals + nv);
  auto first = [&](int v) -> float { return O.vmap[v].empty() ? (float)kLarge2D : htm[O.vmap[v][0]]; };
  float* ptm = d_tm.p; float* ptmo = d_tmo.p; int* pvm = d_vm.p; int* pvmo = d_vmo.p; float* pe0 = d_e0.p;
  float* pe1 = d_e1.p; float* pe2 = d_e2.p; float* psp = d_sp.p; int* pbs = d_bs.p; int* pcon = d_con.p;
  int* pbc = d_bc.p; int* pal = d_al.p;
  float stopd = 50000.f;
  int stopi = 50000;
  const size_t smem = (size_t)maxF * 3 * 4 + (size_t)maxV * 6 * 2;
  int iters = 0, total = 0;
  long long nupd = 0;
  htm = O.triMem;
  const auto t_loop = std::chrono::steady_clock::now();
  while (!act.empty()) {
    if (++total > max_iters) break;
    int na = (int)act.size();
    std::copy(act.begin(), act.end(), alist.begin());
    TRY(d_al.put(alist.data(), nb));
    int mF = maxF, mV = maxV;
    void* a_fim[] = {&ptm, &ptmo, &pvm, &pvmo, &pe0, &pe1, &pe2, &psp, &pbs, &pcon, &pal, &na, &mF, &mV, &stopd};
    TRY(launch(kfim, na, maxF, smem, a_fim));
    void* a_red[] = {&pcon, &pbc, &pal, &na, &pbs};
    TRY(launch(kred, na, 32, 0, a_red));
    TRY(d_bc.get(blockCon.data(), nb));
    for (int b : act) nupd += (long long)bsz[b] * 7;
    std::vector<int> list = act;
    for (int b : act)
      if (blockCon[b])
        for (int nbk : O.blkNbrs[b])
          if (label[nbk] == 0) { label[nbk] = 1; list.push_back(nbk); }
    int nl = (int)list.size();
    std::copy(list.begin(), list.end(), alist.begin());
    TRY(d_al.put(alist.data(), nl));
    void* a_chk[] = {&ptmo, &ptm, &pvm, &pvmo, &pe0, &pe1, &pe2, &psp, &pbs, &pcon, &pal, &na, &mF, &mV, &nl, &stopi};
    TRY(launch(kchk, nl, maxF, smem, a_chk));
    void* a_red2[] = {&pcon, &pbc, &pal, &nl, &pbs};
    TRY(launch(kred, nl, 32, 0, a_red2));
    TRY(d_bc.get(blockCon.data(), nb));
    for (int b : list) nupd += bsz[b];
    std::vector<int> next;
    for (int b = 0; b < nb; ++b) {
      if (!blockCon[b]) { label[b] = 1; next.push_back(b); } else label[b] = 0;
    }
    TRY(d_tm.get(htm.data(), 3 * nslot));
    bool allConv = true;
    for (int v = 0; v < nv; ++v) {
      const float cur = first(v);
      const float diff = std::abs(prev[v] - cur);
      allConv = allConv && (diff <= 1e-5f) && ((double)cur < kLarge2D);
      prev[v] = cur;
    }
    ++iters;
    if (history && iters <= hist_cap)
      for (int v = 0; v < nv; ++v) history[(size_t)(iters - 1) * nv + v] = prev[v];
    act.swap(next);
    if (allConv) break;
  }
  g_loop_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_loop).count();
  for (int v = 0; v < nv; ++v) out_final[v] = first(v);
  if (updates) *updates = nupd;
  return iters;
}

// Each case is one triangle forming its own block (3 owned vertices, 1 element
// slot + 2 empty slots); one launch of the reference's 2D FIMCuda (7 sweeps, check
// = 0) or run_check_neighbor (1 sweep, check = 1).  in: T0 T1 T2 e01 e12 e20
// speedInv per case; out: the three vertex values the kernel writes back.
// Single-tet blocks through the reference's 3D FIMCuda with one sweep
// (CUDA_kernels.cu:383-489): block b holds one tet in slot 0 (three padding slots
// at LARGENUM) whose four corners are the block's vertices, so vertex k of block b
// ends at min(T_k, localSolverTet1 of apex k) as FIMCuda's four inlined updates
// compute it.  in: 10 floats per block (TA TB TC TD, then the six metric edge
// products ACBC BCCD ACCD ADBD ACAD BCBD); out: 4 floats per block.
int refgpu_tet_blocks(const char* cubin3d, const float* in, int n, float* out) {
  TRY(load(g_lib3, cubin3d));
  cudaKernel_t kfim;
  TRY(kernel(g_lib3, "ref3d_fim", &kfim));
  const int maxT = 4, maxIn = 4, mapIn = 1, mapOut = 1;
  const size_t nslot = (size_t)n * maxT;
  std::vector<float> m0(3 * nslot, 0.f), m1(3 * nslot, 0.f), tT(4 * nslot, (float)kLarge3D);
  std::vector<int> vm((size_t)n * maxIn), vmo((size_t)n * maxIn, -1), bs(n, 4), al(n);
  for (int b = 0; b < n; ++b) {
    const float* c = in + 10 * (size_t)b;
    const size_t s0 = (size_t)b * maxT;
    for (int k = 0; k < 4; ++k) tT[4 * s0 + k] = c[k];
    for (int k = 0; k < 3; ++k) {
      m0[3 * s0 + k] = c[4 + k];
      m1[3 * s0 + k] = c[7 + k];
    }
    for (int k = 0; k < 4; ++k) vm[(size_t)b * maxIn + k] = (int)(4 * s0) + k;
    al[b] = b;
  }
  DBuf<float> d_m0, d_m1, d_tT, d_vT, d_sp;
  DBuf<int> d_vm, d_vmo, d_bs, d_al;
  DBuf<char> d_con;
  TRY(d_m0.alloc(3 * nslot)); TRY(d_m1.alloc(3 * nslot)); TRY(d_tT.alloc(4 * nslot));
  TRY(d_vT.alloc((size_t)n * maxIn)); TRY(d_sp.alloc(nslot)); TRY(d_vm.alloc(vm.size()));
  TRY(d_vmo.alloc(vmo.size())); TRY(d_bs.alloc(n)); TRY(d_al.alloc(n)); TRY(d_con.alloc((size_t)n * maxIn));
  TRY(d_m0.put(m0.data(), m0.size())); TRY(d_m1.put(m1.data(), m1.size())); TRY(d_tT.put(tT.data(), tT.size()));
  TRY(d_vm.put(vm.data(), vm.size())); TRY(d_vmo.put(vmo.data(), vmo.size())); TRY(d_bs.put(bs.data(), n));
  TRY(d_al.put(al.data(), n));
  float3* pm0 = (float3*)d_m0.p; float3* pm1 = (float3*)d_m1.p; float4* ptT = (float4*)d_tT.p;
  float* pvT = d_vT.p; float* psp = d_sp.p; int* pvm = d_vm.p; int* pvmo = d_vmo.p; int* pbs = d_bs.p;
  bool* pcon = (bool*)d_con.p; int* pal = d_al.p;
  int mI = maxIn, mpI = mapIn, mpO = mapOut, nIter = 1;
  void* a_fim[] = {&pm0, &pm1, &ptT, &pvT, &psp, &pvm, &pvmo, &pbs, &pcon, &pal, &mI, &mpI, &mpO, &nIter};
  const size_t smem = 16 * (size_t)maxT + 4 * (size_t)maxIn * mapIn;
  TRY(launch(kfim, n, maxT, smem, a_fim));
  RCK(cudaDeviceSynchronize());
  TRY(d_vT.get(out, (size_t)n * maxIn));
  return 0;
}

int refgpu_tri_blocks(const char* cubin2d, const float* in, int n, int check, float* out) {
  TRY(load(g_lib2, cubin2d));
  cudaKernel_t kfim, kchk;
  TRY(kernel(g_lib2, "ref2d_fim", &kfim));
  TRY(kernel(g_lib2, "ref2d_check", &kchk));
  const int maxF = 3, maxV = 3;
  const size_t nslot = (size_t)n * maxF;
  std::vector<float> tm(3 * nslot, (float)kLarge2D), e0(nslot, 1.f), e1(nslot, 1.f), e2(nslot, 1.f), sp(nslot, 1.f);
  std::vector<int> vm((size_t)n * maxV * 6), vmo((size_t)n * maxV * 6, -1), bs(n, 3), al(n);
  for (int b = 0; b < n; ++b) {
    const float* c = in + 7 * (size_t)b;
    const int base = b * maxF * 3;
    for (int k = 0; k < 3; ++k) tm[base + k] = c[k];
    e0[(size_t)b * maxF] = c[3];
    e1[(size_t)b * maxF] = c[4];
    e2[(size_t)b * maxF] = c[5];
    sp[(size_t)b * maxF] = c[6];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 6; ++j) vm[((size_t)b * maxV + k) * 6 + j] = (j == 0) ? base + k : -1 + base;
    al[b] = b;
  }
  DBuf<float> d_tm, d_tmo, d_e0, d_e1, d_e2, d_sp;
  DBuf<int> d_vm, d_vmo, d_bs, d_con, d_al;
  TRY(d_tm.alloc(3 * nslot)); TRY(d_tmo.alloc(3 * nslot)); TRY(d_e0.alloc(nslot)); TRY(d_e1.alloc(nslot));
  TRY(d_e2.alloc(nslot)); TRY(d_sp.alloc(nslot)); TRY(d_vm.alloc(vm.size())); TRY(d_vmo.alloc(vmo.size()));
  TRY(d_bs.alloc(n)); TRY(d_con.alloc((size_t)n * 64)); TRY(d_al.alloc(n));
  TRY(d_tm.put(tm.data(), tm.size())); TRY(d_tmo.put(tm.data(), tm.size())); TRY(d_e0.put(e0.data(), nslot));
  TRY(d_e1.put(e1.data(), nslot)); TRY(d_e2.put(e2.data(), nslot)); TRY(d_sp.put(sp.data(), nslot));
  TRY(d_vm.put(vm.data(), vm.size())); TRY(d_vmo.put(vmo.data(), vmo.size())); TRY(d_bs.put(bs.data(), n));
  TRY(d_al.put(al.data(), n));
  float* ptm = d_tm.p; float* ptmo = d_tmo.p; int* pvm = d_vm.p; int* pvmo = d_vmo.p; float* pe0 = d_e0.p;
  float* pe1 = d_e1.p; float* pe2 = d_e2.p; float* psp = d_sp.p; int* pbs = d_bs.p; int* pcon = d_con.p;
  int* pal = d_al.p;
  int na = n, mF = maxF, mV = maxV, stopi = 50000;
  float stopd = 50000.f;
  const size_t smem = (size_t)maxF * 3 * 4 + (size_t)maxV * 6 * 2;
  if (!check) {
    void* a_fim[] = {&ptm, &ptmo, &pvm, &pvmo, &pe0, &pe1, &pe2, &psp, &pbs, &pcon, &pal, &na, &mF, &mV, &stopd};
    TRY(launch(kfim, n, maxF, smem, a_fim));
  } else {
    void* a_chk[] = {&ptm, &ptmo, &pvm, &pvmo, &pe0, &pe1, &pe2, &psp, &pbs, &pcon, &pal, &na, &mF, &mV, &na, &stopi};
    TRY(launch(kchk, n, maxF, smem, a_chk));
  }
  RCK(cudaDeviceSynchronize());
  TRY(d_tmo.get(tm.data(), tm.size()));
  for (int b = 0; b < n; ++b)
    for (int k = 0; k < 3; ++k) out[3 * (size_t)b + k] = tm[(size_t)b * maxF * 3 + k];
  return 0;
}

}  // extern "C"
