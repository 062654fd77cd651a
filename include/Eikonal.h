// Eikonal.h — the reference's C++ `Eikonal` class (SCI-Solver_Eikonal
// src/Eikonal.h:14-61, src/Eikonal.cu) over the GB300 solver's C ABI
// (eikonal_gb300.h).  A program written against the reference compiles against
// this header unchanged when it uses the class's public methods and option
// members; link it with libeikonal_gb300.so instead of the reference library.
//
// Same as the reference:
//   * constructor arguments and defaults, every option member with its default
//     (maxBlocks_ 16, maxVertsPerBlock_ 64, stopDistance_ 50000, ...);
//   * filename_ is read on first use (".ply" for triangle meshes, TetGen
//     ".node"/".ele" base name for tet meshes);
//   * seeds: the vertices initializeVertices() set to 0, else vertex 0;
//   * iteration_values_ holds one vector per outer iteration; getFinalResult() is
//     the last one, numIterations() their count;
//   * maxBlocks_ is overwritten with the block count the partition produced.
// Different from the reference:
//   * errors throw std::runtime_error where the reference prints and calls exit();
//     compiled with EIKONAL_GB300_EXIT_ON_ERROR defined, the class prints the
//     message and exits with the reference's codes instead (1: unreadable mesh,
//     0: initial values of the wrong size, -1: any other failure), so programs and
//     tests that expect the process to end keep working;
//   * the reference's internal pointers (triMesh_, tetMesh_, FIMPtr2d_, FIMPtr3d_)
//     have no counterpart; setMesh() takes vertex / element arrays instead;
//   * keepHistory_ (default true) can be cleared to skip the per-iteration
//     snapshots: iteration_values_ then holds the final result only;
//   * precisionMode_ / precisionKappa_ select the mixed FP32/FP64 mode.
#ifndef EIKONAL_GB300_CPP_H
#define EIKONAL_GB300_CPP_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "eikonal_gb300.h"

class Eikonal {
 public:
  Eikonal(bool isTriMesh, std::string fname = "../src/test/test_data/sphere_74verts.ply", bool verbose = false)
      : verbose_(verbose), filename_(fname), isTriMesh_(isTriMesh) {
    eik_options o;
    eik_default_options(&o);
    maxBlocks_ = o.max_blocks;
    maxVertsPerBlock_ = o.max_verts_per_block;
    stopDistance_ = o.stop_distance;
    isStructured_ = o.is_structured != 0;
    speedType_ = o.speed_type;
    squareLength_ = o.square_length;
    squareWidth_ = o.square_width;
    squareDepth_ = o.square_depth;
    squareBlockLength_ = o.square_block_length;
    squareBlockWidth_ = o.square_block_width;
    squareBlockDepth_ = o.square_block_depth;
    maxIterations_ = o.max_iterations;
    keepHistory_ = o.keep_history != 0;
    precisionMode_ = o.precision;
    precisionKappa_ = o.precision_kappa;
    deviceSetup_ = o.device_setup;
    partitioner_ = o.partitioner;
    telemetry_ = o.telemetry;
    if (eik_create(isTriMesh ? 1 : 0, &h_) != EIK_OK) throw std::runtime_error("eik_create failed");
  }
  virtual ~Eikonal() { eik_destroy(h_); }
  Eikonal(const Eikonal&) = delete;
  Eikonal& operator=(const Eikonal&) = delete;

  // Reads filename_ once (src/Eikonal.cu:99-133).
  void initializeMesh() {
    if (meshLoaded_) return;
    check(eik_load_mesh(h_, filename_.c_str()));
    meshLoaded_ = true;
  }
  // Mesh from arrays: nv x 3 coordinates, 3 (triangles) or 4 (tets) indices per element.
  void setMesh(const std::vector<float>& xyz, const std::vector<int>& elems) {
    const int per = isTriMesh_ ? 3 : 4;
    check(eik_set_mesh(h_, xyz.data(), (int)(xyz.size() / 3), elems.data(), (int)(elems.size() / per)));
    meshLoaded_ = true;
  }
  // Vertices set to 0 become seeds (src/Eikonal.cu:69-97); the mesh must be loaded.
  void initializeVertices(std::vector<float> values) {
    if (!meshLoaded_) fatal(0, "You must initialize the mesh first!");
    if (eik_set_initial_values(h_, values.data(), (int)values.size()) != EIK_OK)
      fatal(0, std::string("eikonal: ") + eik_last_error(h_));
    userSetInitial_ = true;
  }
  // Per-face speeds (2D), or per-tet scalar / 6-entry metric (3D) (src/Eikonal.cu:62-67).
  void initSpeedMtxMultipliers(std::vector<float> values) { speedMtxMultipliers_ = values; }

  std::vector<float>& getFinalResult() { return iteration_values_.at(iteration_values_.size() - 1); }
  std::vector<float>& getResultAtIteration(size_t i) { return iteration_values_.at(i); }
  size_t numIterations() { return iteration_values_.size(); }
  // result<i>.vtk for the last (all = false) or every iteration (src/Eikonal.cu:50-60).
  void writeVTK(bool all) { check(eik_write_vtk(h_, "result", all ? 1 : 0)); }

  // Partition, layout, device solve (src/Eikonal.cu:135-238).
  void solveEikonal() {
    if (!meshLoaded_) initializeMesh();
    push_options();
    if (!speedsPushed_ || pushedSpeeds_ != speedMtxMultipliers_) {
      check(eik_set_speeds(h_, speedMtxMultipliers_.empty() ? nullptr : speedMtxMultipliers_.data(),
                           (long long)speedMtxMultipliers_.size()));
      pushedSpeeds_ = speedMtxMultipliers_;
      speedsPushed_ = true;
    }
    check(eik_solve(h_));
    eik_options o;
    check(eik_get_options(h_, &o));
    maxBlocks_ = o.max_blocks;
    const int nv = eik_num_vertices(h_);
    const int iters = eik_num_iterations(h_);
    iteration_values_.clear();
    if (keepHistory_) {
      for (int i = 0; i < iters; ++i) {
        iteration_values_.emplace_back(nv);
        check(eik_get_iteration(h_, i, iteration_values_.back().data(), nv));
      }
    }
    if (iteration_values_.empty()) {
      iteration_values_.emplace_back(nv);
      check(eik_get_result(h_, iteration_values_.back().data(), nv));
    }
  }

  // RMS error per iteration against `solution`, as a log-scale text graph
  // (src/Eikonal.cu:240-279).
  void printErrorGraph(std::vector<float> solution) {
    std::vector<float> rms(numIterations());
    for (size_t i = 0; i < numIterations(); ++i) {
      float sum = 0.f;
      const std::vector<float>& r = getResultAtIteration(i);
      for (size_t j = 0; j < solution.size(); ++j) {
        const float d = std::abs(solution[j] - r[j]);
        sum += d * d;
      }
      rms[i] = std::sqrt(sum / static_cast<float>(solution.size()));
    }
    int hi = -10, lo = 10;
    while (std::pow(10.f, (float)hi) < rms.front()) hi++;
    while (std::pow(10.f, (float)lo) > rms.back()) lo--;
    std::printf("\n\nlog(Err)|\n");
    bool tick = true;
    for (int e = hi; e >= lo; --e) {
      if (tick) std::printf("   10^%2d|", e);
      else std::printf("        |");
      for (size_t j = 0; j < rms.size(); ++j)
        std::printf("%s", (rms[j] > std::pow(10.f, (float)e) && rms[j] < std::pow(10.f, (float)(e + 1))) ? "*" : " ");
      std::printf("\n");
      tick = !tick;
    }
    std::printf("--------|------------------------------------------  Converged to: %.4f\n", rms.back());
    std::printf("        |1   5    10   15   20   25   30   35\n");
    std::printf("                   Iteration\n");
  }

  // solver statistics of the last solve (iterations, vertex updates, device time)
  eik_stats stats() const {
    eik_stats s{};
    eik_get_stats(h_, &s);
    return s;
  }
  eik_solver* handle() const { return h_; }

  // ---- option members (src/Eikonal.h:43-60) ----
  bool verbose_;
  std::string filename_;
  int maxBlocks_;
  int maxVertsPerBlock_;
  float stopDistance_;
  bool isStructured_;
  bool userSetInitial_ = false;
  int speedType_;
  int squareLength_, squareWidth_, squareDepth_;
  int squareBlockLength_, squareBlockWidth_, squareBlockDepth_;
  int maxIterations_;
  std::vector<std::vector<float> > iteration_values_;
  bool isTriMesh_;
  std::vector<float> speedMtxMultipliers_;
  bool keepHistory_;
  // precision mode (not in the reference): 1 = FP64 local updates on tets whose
  // metric edge Gram condition number exceeds precisionKappa_, FP64 residual check
  int precisionMode_;
  float precisionKappa_;
  // 1: 3D block layouts are built on the GPU; 0: on the host
  int deviceSetup_;
  // EIK_PARTITION_RCB (default) or EIK_PARTITION_METIS (the reference's partitioner
  // kind; METIS 5 here, METIS 4 in the reference)
  int partitioner_;
  // 1 (default): per-iteration launch spans and visit counts on the device timer;
  // 0: none (a slightly faster solve)
  int telemetry_;

 private:
  // the reference's exit codes for the failures it exits on (src/Eikonal.cu:71-88,
  // :103-118; cutil.h for CUDA errors)
  static int exit_code(int rc) { return (rc == EIK_ERR_MESH) ? 1 : -1; }
  [[noreturn]] static void fatal(int code, const std::string& msg) {
#ifdef EIKONAL_GB300_EXIT_ON_ERROR
    std::fprintf(stderr, "%s\n", msg.c_str());
    std::exit(code);
#else
    (void)code;
    throw std::runtime_error(msg);
#endif
  }
  void check(int rc) const {
    if (rc != EIK_OK) fatal(exit_code(rc), std::string("eikonal: ") + eik_last_error(h_));
  }
  void push_options() {
    eik_options o;
    check(eik_get_options(h_, &o));
    o.max_blocks = maxBlocks_;
    o.max_verts_per_block = maxVertsPerBlock_;
    o.stop_distance = stopDistance_;
    o.is_structured = isStructured_ ? 1 : 0;
    o.speed_type = speedType_;
    o.square_length = squareLength_;
    o.square_width = squareWidth_;
    o.square_depth = squareDepth_;
    o.square_block_length = squareBlockLength_;
    o.square_block_width = squareBlockWidth_;
    o.square_block_depth = squareBlockDepth_;
    o.max_iterations = maxIterations_;
    o.verbose = verbose_ ? 1 : 0;
    o.keep_history = keepHistory_ ? 1 : 0;
    o.precision = precisionMode_;
    o.precision_kappa = precisionKappa_;
    o.device_setup = deviceSetup_;
    o.partitioner = partitioner_;
    o.telemetry = telemetry_;
    check(eik_set_options(h_, &o));
  }
  eik_solver* h_ = nullptr;
  bool meshLoaded_ = false;
  bool speedsPushed_ = false;
  std::vector<float> pushedSpeeds_;
};

#endif
