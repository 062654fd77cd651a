// device.hpp — the device-resident block-FIM solve (host side of the CUDA code).
//
// One DeviceSolve owns the device copy of a block layout (slots, metric terms,
// local vertex ids, halos, block graph) and the per-solve state (vertex travel
// times, block flags, active lists, control block).  A solve is one launch of a
// CUDA graph whose conditional while-node runs the reference's outer iteration
// (src/core3d/cuda/meshFIM3dEikonal.cu:411-542, src/core2d/cuda/meshFIM2d_eikonal.cu:683-816)
// entirely on the device: block visits, commit, neighbour activation and list
// compaction, with no host round trip per iteration.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "setup.hpp"

struct CUstream_st;
typedef struct CUstream_st* cudaStream_t;

namespace eikgb {

constexpr int kIterStatWords = 16;

struct SolveStats {
  int iterations = 0;
  long long vertex_updates = 0;  // owned vertices x sweeps over all block visits
  long long block_visits = 0;    // sweep visits + check visits
  long long fim_visits = 0;
  long long check_visits = 0;
  long long slot_visits = 0;     // element slots streamed over all visits
  long long halo_visits = 0;     // halo vertices gathered over all visits
  long long owned_visits = 0;    // owned vertices over all visits
  float solve_ms = 0.0f;         // device time of the last solve
  int error = 0;                 // device-side error flags (0 = none)
  long long fim_slots = 0, fim_halo = 0, fim_owned = 0;  // inputs of the sweep-kernel visits
  float fim_kernel_ms = 0.0f;    // summed launch spans of the sweep kernel (device timer)
  float check_kernel_ms = 0.0f;  // same for the neighbour-check kernel
  int fim_launches = 0, check_launches = 0;
  // per outer iteration, kIterStatWords values: sweep-kernel and check-kernel
  // launch spans (ns, device timer), then the sweep kernel's block visits, element
  // slots, halo vertices and owned vertices, then the same four for the check kernel,
  // then the two kernels' start times (ns after the first iteration's sweep start),
  // then visits, slots, halo and owned vertices of the sweep visits that followed a
  // check in the same visit (checks inside the sweep kernel)
  std::vector<long long> iter_stats;
  long long h2d_bytes = 0;       // host-to-device bytes the last solve copied (initial state)
  std::vector<int> inst_iters;   // outer iterations run by every instance
  // precision mode: FP64 residual check after the solve
  double residual_max_abs = 0, residual_max_rel = 0, residual_below_rel = 0;
  long long residual_vertices = 0;
  int polish_rounds = 0;         // rounds of FP64 re-visits after the solve
  long long polish_blocks = 0;   // blocks queued over those rounds
};

struct SolveOptions {
  int max_iterations = 100;  // reference default (src/Eikonal.cu:19)
  int fim_sweeps = -1;       // -1: reference value (3D: 2, 2D: 7)
  bool keep_history = false; // per-iteration snapshots (getResultAtIteration)
  int history_cap = 0;       // snapshots kept when keep_history
  int threads = 0;           // CTA size of the 3D visit kernels (0: from the largest block)
  bool direct_launch = false; // launch the loop body kernel by kernel (for profilers)
  bool telemetry = true;      // per-launch spans and visit counts on the device timer
  std::vector<int> inst_max_iterations;  // per instance; empty: max_iterations for all
};

// Coefficient inputs of one pool mesh for the serving path (original vertex and
// element order, host arrays; copied to the device by serve_setup).
struct ServeSource {
  int dim = 3;
  const float* xyz = nullptr;  // 3D: 3 per vertex
  int nv = 0;
  const int* tets = nullptr;   // 3D: 4 per tet (0-based)
  int nt = 0;
  const float* M6 = nullptr;   // 3D: 6 metric entries per tet (tet_metrics)
  const float* speed = nullptr;  // 2D: speed per real face
  int nf = 0;
};

// One request started on instance `inst`: 3D metric entries are multiplied by
// coef_scale, 2D face speeds by coef_scale; seeds are vertex ids of the instance.
struct Admission {
  int inst = 0;
  float coef_scale = 1.0f;
  int max_iterations = 100;
  std::vector<int> seeds;
};

// A 3D block layout built on the device (build_layout3d_device): the arrays a
// solve reads, plus the inputs kept for coefficient refreshes.  Owned until
// handed to DeviceSolve::upload_built or released.
struct Built3D {
  BlockDesc* blocks = nullptr;
  float* coef = nullptr;       // 6 per slot, SoA per block
  uint16_t* lv = nullptr;      // 4 corner local ids per slot
  int* halo = nullptr;
  int* nbr_off = nullptr;
  int* nbr = nullptr;
  int* vblock = nullptr;       // renumbered vertex -> block
  int* perm = nullptr;         // original -> renumbered
  int* slot_elem = nullptr;
  float* xyz = nullptr;
  int* tets = nullptr;
  float* M6 = nullptr;          // metric per tet: mcomp entries (6: full, 1: scalar times I)
  int mcomp = 6;
  int total_slots = 0, nhalo = 0, nnbr = 0;
  int dim = 3;                  // 2: tets holds the oriented faces (3 each), M6 the face speeds
  void release();
};

// Builds the 3D layout of build_layout3d on the device (same arrays).  L receives
// the host-side part: block descriptors, renumbering, statistics (no coefficient,
// corner-id, halo or neighbour arrays).
// M holds mcomp metric entries per tet: 6 (M00 M01 M02 M11 M12 M22) or 1 (a scalar
// s standing for s*I, which gives the same products as the 6 entries s 0 0 s 0 s).
std::string build_layout3d_device(int nv, const float* xyz, int nt, const int* tets, const float* M, int mcomp,
                                  const int* labels, int nb, cudaStream_t st, Built3D& out, Layout& L);

// The 2D layout of build_layout2d built on the device from a prepared triangle mesh
// (oriented faces, obtuse corners, virtual faces and edge lengths stay host work)
// and per-face speeds (null: all 1); same arrays, including the bit-15 marks of the
// copies the reference never refreshes.  out.dim = 2.
std::string build_layout2d_device(int nv, const TriPrep& P, const float* speeds, const int* labels, int nb,
                                  cudaStream_t st, Built3D& out, Layout& L);

// A non-blocking CUDA stream of the current device (null on failure), and its release.
cudaStream_t new_stream();
void free_stream(cudaStream_t st);

// Device bytes one instance of this layout occupies (layout arrays + state);
// b: the device-built arrays of a layout whose host part L holds none of them.
size_t device_footprint(const Layout& L, const Built3D* b = nullptr);

// Copies a device-built layout's arrays (coefficients, corner ids, element ids,
// halo lists, neighbour graph) into the host layout L that holds its host part,
// which then equals the host build's layout.
std::string download_built(const Built3D& b, Layout& L);

class DeviceSolve {
 public:
  DeviceSolve();
  ~DeviceSolve();
  DeviceSolve(const DeviceSolve&) = delete;
  DeviceSolve& operator=(const DeviceSolve&) = delete;

  // Upload (or re-upload) a layout.  Keeps the device arrays until the next call.
  std::string upload(const Layout& L);
  // Refresh only the per-slot coefficients (speed/metric change).
  std::string upload_coef(const Layout& L);
  // Take over a device-built 3D layout (L: its host part, kept by the caller).
  std::string upload_built(const Layout& L, Built3D& b);
  // Several instances of device-built layouts concatenated on the device (the
  // server's arena): parts[i] holds instance i's arrays (a part may repeat), L the
  // host part of the concatenation (concat_layout_headers).  The parts stay the
  // caller's.
  std::string upload_replicas(const Layout& L, const std::vector<const Built3D*>& parts);
  // Device-built layouts: recompute the per-slot coefficients on the device from
  // a new per-tet metric (6 entries per tet, host array).
  std::string refresh_coef_built(const float* M, int mcomp);
  // Device-built 2D layouts: new inverse speeds from per-face speeds (null: all 1).
  std::string refresh_speed_built(const float* speed);
  bool layout_built_on_device() const;
  // Copies of the uploaded layout's per-slot coefficients and (device-built 3D
  // layouts only) the element id of every slot, for checks against the reference.
  std::string layout_arrays(std::vector<float>* coef, std::vector<int>* slot_elem) const;
  // Seeds are original vertex ids.  init_vals (2D only, may be null) are the
  // vertex values the reference's all-vertex convergence test starts from.
  std::string set_seeds(const std::vector<int>& seeds_orig, const float* init_vals);
  // Several instances (a layout from concat_layouts): per instance its seeds
  // (vertex ids of that instance) and optional initial values.
  std::string set_seeds_multi(const std::vector<std::vector<int>>& seeds, const std::vector<const float*>& init_vals);
  // Runs the solve to completion on the solver's stream.
  std::string solve(const SolveOptions& opt);
  // Final travel times in original vertex order.
  std::string result(float* out_host) const;
  std::string result_device(float* out_dev) const;  // device pointer, original order
  std::string history(int i, float* out_host) const;
  // One visit of every block with the 2D kernel on the given vertex values
  // (renumbered order); sweep visit or neighbour check.  For self-tests.
  std::string visit_once(bool check, const float* T_host, float* out_host);
  // ---- serving: a resident arena of instances admitted one by one ----------
  // serve_setup makes every instance of the uploaded (concatenated) layout idle,
  // uploads the coefficient sources of the pool meshes and builds the serving
  // loop.  serve_admit starts instances (fresh state, request-scaled
  // coefficients, seeds); serve_run runs the device loop until some instance
  // finishes, the pending flag is raised or nothing runs; serve_poll reads which
  // instances are done; serve_fetch + serve_sync copy results to pinned memory.
  std::string serve_setup(const std::vector<ServeSource>& meshes, const std::vector<int>& inst_mesh, int sweeps,
                          int threads);
  std::string serve_admit(const std::vector<Admission>& adm);
  std::string serve_run();
  // stop running instances now (their list entries are skipped, then dropped)
  std::string serve_cancel(const std::vector<int>& insts);
  std::string serve_poll(std::vector<int>& done, std::vector<int>& iters);
  std::string serve_fetch(int inst);
  std::string serve_sync();
  const float* serve_host_result(int inst) const;  // valid after serve_sync
  volatile int* serve_pending() const;             // host side of the pending flag
  // Makes the device this object was created on current in the calling thread.
  void bind_thread() const;
  const SolveStats& stats() const { return stats_; }
  const Layout* layout() const { return L_; }
  void* stream() const { return stream_; }

 private:
  std::string finish_upload(const Layout& L, bool layout_on_device);
  struct Impl;
  Impl* p_;
  const Layout* L_ = nullptr;
  SolveStats stats_;
  void* stream_ = nullptr;
};

// Runs the device local updates element-wise: which = 0 tet (9 inputs per case),
// 1 triangle (7 inputs), 2 the two exact quotients (num, den -> small_quot,
// root_quot); 3 / 4: single-triangle blocks through the 2D sweep / check kernel
// (7 inputs -> 3 outputs).  Host arrays.
std::string selftest_device(int which, const float* in, float* out, int n);

// Runs a one-CTA kernel whose bounded barrier wait cannot complete: status gets
// the device error flag (nonzero when the wait gave up), waited_ms its duration.
std::string selftest_wait_timeout(int* status, double* waited_ms);

// Allocation-free 3D solve: the layout and every solver buffer live in a fixed
// 32 MiB array of the library's device image (no cudaMalloc / cudaFree).  Runs on
// `stream` (a cudaStream_t, may be null), one host round trip per outer
// iteration.  Fails with a message when the mesh needs more scratch than the array
// holds (bytes_needed reports the requirement); *failure says which kind of
// failure a non-empty message is.
enum class NoAllocFailure { kNone, kLimit, kDevice, kCuda };
std::string solve3d_noalloc(const Layout& L, const std::vector<int>& seeds, int max_iters, float* out_host,
                            cudaStream_t stream, int* iterations, size_t* bytes_needed, NoAllocFailure* failure);

}  // namespace eikgb
