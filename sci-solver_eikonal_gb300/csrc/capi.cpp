// capi.cpp — the C ABI (include/eikonal_gb300.h) over the host setup and the
// device-resident solve.  Mirrors the reference's Eikonal facade
// (src/Eikonal.cu:4-279): same defaults, same seed rules, same partition-size
// rules, status codes where the reference exits.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/eikonal_gb300.h"
#include "device.hpp"
#include "mesh_io.hpp"
#include "setup.hpp"
#include "solver_access.hpp"

using namespace eikgb;

// Solves build their block layout on the GPU unless eik_options.device_setup = 0
// (3D precision mode builds on the host)
#define DEVICE_SETUP_DEFAULT 1

struct eik_solver {
  int dim = 3;
  eik_options opt{};
  std::string err;
  // mesh as given (0-based after normalisation)
  std::vector<float> xyz;
  std::vector<int> elems;
  int nv = 0, ne = 0;
  unsigned mesh_ver = 0;
  // inputs
  std::vector<float> speeds;
  bool speeds_set = false;
  unsigned speed_ver = 0;
  std::vector<float> init_vals;
  bool user_initial = false;
  std::vector<int> seeds;
  bool user_seeds = false;
  std::vector<int> user_labels;
  int user_nb = 0;
  unsigned part_ver = 0;
  // derived
  TriPrep prep;
  unsigned prep_mesh = ~0u;
  std::vector<int> labels;
  int nb = 0;
  std::string labels_key;  // mesh version and partition inputs `labels` were made for
  unsigned lay_mesh = ~0u, lay_part = ~0u, lay_speed = ~0u;
  std::string lay_key;
  std::string prec_key;  // precision settings the layout's FP64 data was built for
  Layout layout;
  // 3D layout built on the device: its host part, and what it was built from
  Layout dlayout;
  unsigned dlay_mesh = ~0u, dlay_speed = ~0u;
  unsigned checked_speed = ~0u, checked_mesh = ~0u;  // speeds validated for these versions
  std::string dlay_key;
  std::unique_ptr<DeviceSolve> dev;
  bool uploaded = false;
  bool solved = false;
  eik_stats stats{};
};

namespace {

int fail(eik_solver* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

std::string partition_key(const eik_solver* h) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%u|%d|%d|%d|%d,%d,%d|%d,%d,%d|%d", h->part_ver, h->opt.is_structured,
                h->opt.max_verts_per_block, h->dim, h->opt.square_length, h->opt.square_width, h->opt.square_depth,
                h->opt.square_block_length, h->opt.square_block_width, h->opt.square_block_depth,
                h->opt.partitioner);
  return buf;
}

// Block labels as the reference chooses them (src/Eikonal.cu:162-174, 204-220).
int make_partition(eik_solver* h) {
  if (!h->user_labels.empty()) {
    h->labels = h->user_labels;
    h->nb = h->user_nb;
  } else if (h->opt.is_structured) {
    std::string e = partition_square(h->nv, h->dim, h->opt.square_length, h->opt.square_width, h->opt.square_depth,
                                     h->opt.square_block_length, h->opt.square_block_width,
                                     h->opt.square_block_depth, h->labels, h->nb);
    if (!e.empty()) return fail(h, EIK_ERR_ARG, e);
  } else if (h->opt.partitioner == EIK_PARTITION_METIS) {
    const int want = metis_rule_blocks(h->nv, h->opt.max_verts_per_block, h->dim);
    std::string e = partition_metis(h->nv, h->ne, h->dim == 3 ? 4 : 3, h->elems.data(), want, h->labels, h->nb);
    if (!e.empty()) return fail(h, EIK_ERR_ARG, e);
  } else {
    h->nb = metis_rule_blocks(h->nv, h->opt.max_verts_per_block, h->dim);
    partition_rcb(h->nv, h->xyz.data(), h->nb, h->labels);
  }
  h->opt.max_blocks = h->nb;  // the reference overwrites maxBlocks_ the same way
  h->labels_key = std::to_string(h->mesh_ver) + "/" + partition_key(h);
  return EIK_OK;
}

// make_partition unless `labels` already hold this mesh's partition for the
// current partition inputs.
int ensure_partition(eik_solver* h) {
  if (!h->labels.empty() && h->labels_key == std::to_string(h->mesh_ver) + "/" + partition_key(h)) return EIK_OK;
  return make_partition(h);
}

std::vector<float> speed_inverse(const eik_solver* h) {
  // TriMesh::InitializeAttributes (TriMesh_stats.cu:64-68): 1/speed per face when
  // the vector matches the face count, else 1
  std::vector<float> inv(h->ne, 1.0f);
  if (h->speeds_set && (int)h->speeds.size() == h->ne)
    for (int i = 0; i < h->ne; ++i) inv[i] = 1.f / h->speeds[i];
  return inv;
}

// Speeds / metrics the scheme can use: 2D speeds and 3D scalar metrics finite and
// positive, 3D 6-entry metrics finite.  6-entry metrics are not required to be
// positive definite: the reference's own anisotropic fixture (torus_matrices.txt)
// holds indefinite matrices for half of its tets and the reference solves it.
// The checks on one speed / metric vector of n values for ne elements: an empty
// message when the values are usable (vectors of other lengths mean the
// reference's defaults and are not checked).
std::string speed_values_problem(const float* v, size_t n, int ne, int dim) {
  if (!v || n == 0) return "";
  if (n == (size_t)ne) {
    for (size_t i = 0; i < n; ++i)
      if (!(std::isfinite(v[i]) && v[i] > 0.0f))
        return (dim == 2 ? "speed of face " : "metric of tet ") + std::to_string(i) +
               " is not a positive finite number";
  } else if (dim == 3 && n == 6 * (size_t)ne) {
    for (int t = 0; t < ne; ++t) {
      const float* m = v + 6 * (size_t)t;
      bool finite = true;
      for (int k = 0; k < 6; ++k) finite = finite && std::isfinite(m[k]);
      if (!finite) return "metric of tet " + std::to_string(t) + " is not finite";
    }
  }
  return "";
}

int check_speeds(eik_solver* h) {
  if (h->checked_speed == h->speed_ver && h->checked_mesh == h->mesh_ver) return EIK_OK;
  if (h->speeds_set) {
    const std::string msg = speed_values_problem(h->speeds.data(), h->speeds.size(), h->ne, h->dim);
    if (!msg.empty()) return fail(h, EIK_ERR_ARG, msg);
  }
  h->checked_speed = h->speed_ver;
  h->checked_mesh = h->mesh_ver;
  return EIK_OK;
}

// Partition + block layout on the host, cached while the mesh, the partition
// inputs and the speeds are unchanged; refreshes only the metric terms when just
// the speeds changed.
int host_prepare(eik_solver* h, bool* new_layout_out) {
  if (int rc = check_speeds(h)) return rc;
  bool new_layout = false;
  const std::string key = partition_key(h);
  if (h->lay_mesh != h->mesh_ver || h->lay_key != key) {
    int rc = make_partition(h);
    if (rc) return rc;
    std::string e;
    if (h->dim == 3) {
      std::vector<float> M;
      tet_metrics(h->ne, h->speeds_set ? h->speeds.data() : nullptr, h->speeds.size(), M);
      e = build_layout3d(h->nv, h->xyz.data(), h->ne, h->elems.data(), M.data(), h->labels.data(), h->nb,
                         h->layout);
    } else {
      const std::vector<float> inv = speed_inverse(h);
      e = build_layout2d(h->nv, h->xyz.data(), h->prep, inv.data(), h->labels.data(), h->nb, h->layout);
    }
    if (!e.empty()) return fail(h, EIK_ERR_MESH, e);
    h->lay_mesh = h->mesh_ver;
    h->lay_key = key;
    h->lay_speed = h->speed_ver;
    h->uploaded = false;  // device copy is stale until the next solve uploads it
    new_layout = true;
  } else if (h->lay_speed != h->speed_ver) {
    if (h->dim == 3) {
      std::vector<float> M;
      tet_metrics(h->ne, h->speeds_set ? h->speeds.data() : nullptr, h->speeds.size(), M);
      refresh_gram3d(h->xyz.data(), h->elems.data(), M.data(), h->layout);
    } else {
      const std::vector<float> inv = speed_inverse(h);
      refresh_speed2d(h->prep, inv.data(), h->layout);
    }
    h->lay_speed = h->speed_ver;
    h->prec_key.clear();  // FP64 products follow the metric
    if (h->uploaded) {
      std::string e = h->dev->upload_coef(h->layout);
      if (!e.empty()) return fail(h, EIK_ERR_CUDA, e);
    }
  }
  // precision mode data (3D): flagged tets and their FP64 metric edge products
  if (h->dim == 3) {
    const bool on = h->opt.precision == 1;
    const std::string pk = on ? ("1|" + std::to_string(h->opt.precision_kappa)) : "0";
    if (new_layout || pk != h->prec_key) {
      if (on) {
        std::vector<float> M;
        tet_metrics(h->ne, h->speeds_set ? h->speeds.data() : nullptr, h->speeds.size(), M);
        build_precision3d(h->xyz.data(), h->elems.data(), M.data(), (double)h->opt.precision_kappa, h->layout);
      } else {
        build_precision3d(nullptr, nullptr, nullptr, 0.0, h->layout);
      }
      if (!new_layout && pk != h->prec_key) h->uploaded = false;
      h->prec_key = pk;
    }
  }
  *new_layout_out = new_layout;
  return EIK_OK;
}

// Seeds and initial values as the reference derives them (src/Eikonal.cu:143-159,
// 186-202): vertices the user's initial values set to 0, else the explicit seed
// list, else vertex 0.  3D ignores initial values like the reference.
int resolve_seeds(eik_solver* h, std::vector<int>& seeds, const float** init) {
  seeds.clear();
  *init = nullptr;
  if (h->user_initial) {
    for (int v = 0; v < h->nv; ++v)
      if (h->init_vals[v] == 0.) seeds.push_back(v);
    if (h->dim == 2) *init = h->init_vals.data();
  } else if (h->user_seeds) {
    seeds = h->seeds;
  } else {
    seeds.push_back(0);
  }
  for (int s : seeds)
    if (s >= h->nv) return fail(h, EIK_ERR_ARG, "seed out of range");
  return EIK_OK;
}

SolveOptions solve_options(const eik_options& o) {
  SolveOptions so;
  so.max_iterations = o.max_iterations;
  so.fim_sweeps = o.fim_sweeps;
  so.keep_history = o.keep_history != 0;
  so.history_cap = o.max_iterations;
  so.direct_launch = o.direct_launch != 0;
  so.telemetry = o.telemetry != 0;
  if (o.threads_per_block > 0) so.threads = o.threads_per_block;
  return so;
}

void fill_stats(eik_stats& s, const SolveStats& st, const Layout& L, float setup_ms) {
  s.iterations = st.iterations;
  s.num_blocks = L.nb;
  s.vertex_updates = st.vertex_updates;
  s.fim_visits = st.fim_visits;
  s.check_visits = st.check_visits;
  s.slot_visits = st.slot_visits;
  s.halo_visits = st.halo_visits;
  s.owned_visits = st.owned_visits;
  s.solve_ms = st.solve_ms;
  s.setup_ms = setup_ms;
  s.max_slots_per_block = L.max_slots;
  s.max_local_vertices = L.max_local;
  s.total_slots = L.total_slots;
  s.mean_slots_per_block = L.mean_slots_per_block;
  s.mean_halo_per_block = L.mean_halo_per_block;
  s.device_error = st.error;
  s.fim_kernel_ms = st.fim_kernel_ms;
  s.check_kernel_ms = st.check_kernel_ms;
  s.fim_launches = st.fim_launches;
  s.check_launches = st.check_launches;
  s.fim_slots = st.fim_slots;
  s.fim_halo = st.fim_halo;
  s.fim_owned = st.fim_owned;
  s.h2d_bytes = st.h2d_bytes;
  s.flagged_tets = L.flagged_tets;
  s.residual_max_abs = st.residual_max_abs;
  s.residual_max_rel = st.residual_max_rel;
  s.residual_vertices = st.residual_vertices;
  s.residual_below_rel = st.residual_below_rel;
  s.polish_rounds = st.polish_rounds;
  s.polish_blocks = st.polish_blocks;
}

// The 3D layout built on the device (build_layout3d_device), cached while the mesh
// and partition inputs are unchanged; a speed change recomputes the metric terms
// on the device.  The partition itself stays on the host (make_partition).
// The tet metrics as the device build takes them (tet_metrics' rule without the
// expansion to 6 entries): the caller's 6 entries or scalars as given, else 1 per
// tet (identity); *mcomp receives the entries per tet.
const float* compact_metrics(const eik_solver* h, std::vector<float>& ones, int* mcomp) {
  if (h->speeds_set && h->speeds.size() == 6 * (size_t)h->ne) {
    *mcomp = 6;
    return h->speeds.data();
  }
  *mcomp = 1;
  if (h->speeds_set && h->speeds.size() == (size_t)h->ne) return h->speeds.data();
  ones.assign((size_t)h->ne, 1.0f);
  return ones.data();
}

// 2D face speeds as the layout takes them: the caller's per-face speeds, else none
// (inverse speed 1, TriMesh_stats.cu:64-68)
const float* face_speeds(const eik_solver* h) {
  return (h->speeds_set && (int)h->speeds.size() == h->ne) ? h->speeds.data() : nullptr;
}

int device_prepare(eik_solver* h) {
  if (int rc = check_speeds(h)) return rc;
  const std::string key = partition_key(h);
  if (!h->dev) h->dev.reset(new DeviceSolve);
  if (h->dlay_mesh != h->mesh_ver || h->dlay_key != key || !h->dev->layout_built_on_device()) {
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    int rc = make_partition(h);
    if (rc) return rc;
    const auto t1 = clk::now();
    std::vector<float> ones;
    int mcomp = 6;
    const float* M = (h->dim == 3) ? compact_metrics(h, ones, &mcomp) : nullptr;
    const auto t2 = clk::now();
    Built3D b;
    std::string e = (h->dim == 3)
                        ? build_layout3d_device(h->nv, h->xyz.data(), h->ne, h->elems.data(), M, mcomp,
                                                h->labels.data(), h->nb, (cudaStream_t)h->dev->stream(), b,
                                                h->dlayout)
                        : build_layout2d_device(h->nv, h->prep, face_speeds(h), h->labels.data(), h->nb,
                                                (cudaStream_t)h->dev->stream(), b, h->dlayout);
    if (h->opt.verbose) {
      const auto t3 = clk::now();
      auto ms = [](clk::time_point a, clk::time_point z) { return std::chrono::duration<double, std::milli>(z - a).count(); };
      std::printf("Eikonal GB300: device setup: partition %.2f ms, metrics %.2f ms, layout build %.2f ms\n",
                  ms(t0, t1), ms(t1, t2), ms(t2, t3));
    }
    if (!e.empty()) {
      b.release();
      h->dlay_mesh = ~0u;
      return fail(h, e.find("too many local") != std::string::npos ? EIK_ERR_LIMIT : EIK_ERR_CUDA, e);
    }
    h->uploaded = false;  // the device now holds this layout, not the host-built one
    e = h->dev->upload_built(h->dlayout, b);
    if (!e.empty()) {
      b.release();
      h->dlay_mesh = ~0u;
      return fail(h, e.find("shared memory") != std::string::npos ? EIK_ERR_LIMIT : EIK_ERR_CUDA, e);
    }
    h->dlay_mesh = h->mesh_ver;
    h->dlay_key = key;
    h->dlay_speed = h->speed_ver;
  } else if (h->dlay_speed != h->speed_ver) {
    std::vector<float> ones;
    int mcomp = 6;
    std::string e;
    if (h->dim == 3) {
      const float* M = compact_metrics(h, ones, &mcomp);
      e = h->dev->refresh_coef_built(M, mcomp);
    } else {
      e = h->dev->refresh_speed_built(face_speeds(h));
    }
    if (!e.empty()) return fail(h, EIK_ERR_CUDA, e);
    h->dlay_speed = h->speed_ver;
  }
  return EIK_OK;
}

bool use_device_setup(const eik_solver* h) {
  return h->opt.device_setup == 1 && (h->dim == 2 || h->opt.precision == 0);
}

}  // namespace

extern "C" {

void eik_default_options(eik_options* o) {
  if (!o) return;
  o->max_blocks = 16;
  o->max_verts_per_block = 64;
  o->stop_distance = 50000.f;
  o->is_structured = 0;
  o->speed_type = EIK_SPEED_ONE;
  o->square_length = o->square_width = o->square_depth = 16;
  o->square_block_length = o->square_block_width = o->square_block_depth = 1;
  o->max_iterations = 100;
  o->verbose = 0;
  o->keep_history = 1;
  o->fim_sweeps = -1;
  o->direct_launch = 0;
  o->threads_per_block = 0;
  o->precision = 0;
  o->precision_kappa = 1e4f;
  o->device_setup = DEVICE_SETUP_DEFAULT;
  o->partitioner = EIK_PARTITION_RCB;
  o->telemetry = 1;
}

int eik_create(int is_tri_mesh, eik_solver** out) {
  if (!out) return EIK_ERR_ARG;
  *out = nullptr;
  eik_solver* h = new eik_solver;
  h->dim = is_tri_mesh ? 2 : 3;
  eik_default_options(&h->opt);
  *out = h;
  return EIK_OK;
}

void eik_destroy(eik_solver* h) { delete h; }

int eik_set_options(eik_solver* h, const eik_options* o) {
  if (!h || !o) return fail(h, EIK_ERR_ARG, "null argument");
  if (o->max_verts_per_block <= 0) return fail(h, EIK_ERR_ARG, "max_verts_per_block must be positive");
  if (o->max_iterations < 0) return fail(h, EIK_ERR_ARG, "max_iterations must be >= 0");
  if (o->speed_type != EIK_SPEED_ONE) return fail(h, EIK_ERR_ARG, "only speed type ONE is supported");
  if (o->threads_per_block != 0 && o->threads_per_block != 128 && o->threads_per_block != 256 &&
      o->threads_per_block != 384 && o->threads_per_block != 512 && o->threads_per_block != 768 &&
      o->threads_per_block != 1024)
    return fail(h, EIK_ERR_ARG, "threads_per_block must be 0, 128, 256, 384, 512, 768 or 1024");
  if (o->precision != 0 && o->precision != 1) return fail(h, EIK_ERR_ARG, "precision must be 0 or 1");
  if (!(o->precision_kappa >= 1.0f)) return fail(h, EIK_ERR_ARG, "precision_kappa must be at least 1");
  if (o->device_setup != 0 && o->device_setup != 1) return fail(h, EIK_ERR_ARG, "device_setup must be 0 or 1");
  if (o->partitioner != EIK_PARTITION_RCB && o->partitioner != EIK_PARTITION_METIS)
    return fail(h, EIK_ERR_ARG, "partitioner must be EIK_PARTITION_RCB or EIK_PARTITION_METIS");
  if (o->telemetry != 0 && o->telemetry != 1) return fail(h, EIK_ERR_ARG, "telemetry must be 0 or 1");
  if (o->partitioner == EIK_PARTITION_METIS && !metis_available())
    return fail(h, EIK_ERR_ARG, "this build has no METIS (libmetis_static.a was not found at build time)");
  h->opt = *o;
  return EIK_OK;
}

int eik_get_options(const eik_solver* h, eik_options* o) {
  if (!h || !o) return EIK_ERR_ARG;
  *o = h->opt;
  return EIK_OK;
}

int eik_set_mesh(eik_solver* h, const float* xyz, int nv, const int* elems, int ne) {
  if (!h || !xyz || !elems || nv <= 0 || ne <= 0) return fail(h, EIK_ERR_ARG, "invalid mesh arrays");
  const int per = (h->dim == 3) ? 4 : 3;
  std::vector<int> e(elems, elems + (size_t)per * ne);
  std::string msg = normalize_index_base(e, nv);
  if (!msg.empty()) return fail(h, EIK_ERR_MESH, msg);
  h->xyz.assign(xyz, xyz + 3 * (size_t)nv);
  h->elems.swap(e);
  h->nv = nv;
  h->ne = ne;
  h->mesh_ver++;
  h->solved = false;
  if (h->dim == 2) {
    msg = prepare_trimesh(nv, h->xyz.data(), ne, h->elems.data(), h->prep);
    if (!msg.empty()) return fail(h, EIK_ERR_MESH, msg);
    h->prep_mesh = h->mesh_ver;
  }
  return EIK_OK;
}

int eik_load_mesh(eik_solver* h, const char* filename) {
  if (!h || !filename) return fail(h, EIK_ERR_ARG, "null argument");
  std::vector<float> xyz;
  std::vector<int> el;
  std::string msg = (h->dim == 2) ? read_ply(filename, xyz, el) : read_tetgen(filename, xyz, el);
  if (!msg.empty()) return fail(h, EIK_ERR_MESH, msg);
  const int per = (h->dim == 3) ? 4 : 3;
  return eik_set_mesh(h, xyz.data(), (int)(xyz.size() / 3), el.data(), (int)(el.size() / per));
}

int eik_set_speeds(eik_solver* h, const float* vals, long long n) {
  if (!h || (n > 0 && !vals) || n < 0) return fail(h, EIK_ERR_ARG, "invalid speed array");
  h->speeds.assign(vals, vals + n);
  h->speeds_set = n > 0;
  h->speed_ver++;
  return EIK_OK;
}

int eik_set_initial_values(eik_solver* h, const float* vals, int nv) {
  if (!h || !vals) return fail(h, EIK_ERR_ARG, "null argument");
  if (h->nv == 0) return fail(h, EIK_ERR_STATE, "You must initialize the mesh first!");
  if (nv != h->nv) return fail(h, EIK_ERR_ARG, "Initialize values size does not match number of vertices!");
  h->init_vals.assign(vals, vals + nv);
  h->user_initial = true;
  h->user_seeds = false;
  return EIK_OK;
}

int eik_set_seeds(eik_solver* h, const int* seeds, int n) {
  if (!h || (n > 0 && !seeds) || n < 0) return fail(h, EIK_ERR_ARG, "invalid seed array");
  for (int i = 0; i < n; ++i)
    if (seeds[i] < 0 || (h->nv > 0 && seeds[i] >= h->nv)) return fail(h, EIK_ERR_ARG, "seed out of range");
  h->seeds.assign(seeds, seeds + n);
  h->user_seeds = true;
  h->user_initial = false;
  return EIK_OK;
}

int eik_set_partition(eik_solver* h, const int* labels, int nv, int nblocks) {
  if (!h) return EIK_ERR_ARG;
  if (!labels) {
    h->user_labels.clear();
    h->user_nb = 0;
    h->part_ver++;
    return EIK_OK;
  }
  if (h->nv == 0) return fail(h, EIK_ERR_STATE, "set the mesh before the partition");
  if (nv != h->nv || nblocks <= 0) return fail(h, EIK_ERR_ARG, "partition size mismatch");
  for (int i = 0; i < nv; ++i)
    if (labels[i] < 0 || labels[i] >= nblocks) return fail(h, EIK_ERR_ARG, "partition label out of range");
  h->user_labels.assign(labels, labels + nv);
  h->user_nb = nblocks;
  h->part_ver++;
  return EIK_OK;
}

int eik_solve(eik_solver* h) {
  if (!h) return EIK_ERR_ARG;
  if (h->nv == 0) return fail(h, EIK_ERR_STATE, "no mesh: call eik_set_mesh or eik_load_mesh first");
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<int> seeds;
  const float* init = nullptr;
  int rc = resolve_seeds(h, seeds, &init);
  if (rc) return rc;
  const bool on_device = use_device_setup(h);
  if (on_device) {
    rc = device_prepare(h);
    if (rc) return rc;
  } else {
    bool new_layout = false;
    rc = host_prepare(h, &new_layout);
    if (rc) return rc;
    if (!h->dev) h->dev.reset(new DeviceSolve);
    if (new_layout || !h->uploaded || h->dev->layout_built_on_device()) {
      std::string e = h->dev->upload(h->layout);
      if (!e.empty()) {
        h->uploaded = false;
        return fail(h, e.find("shared memory") != std::string::npos ? EIK_ERR_LIMIT : EIK_ERR_CUDA, e);
      }
      h->uploaded = true;
    }
  }
  std::string e = h->dev->set_seeds(seeds, init);
  if (!e.empty()) return fail(h, EIK_ERR_ARG, e);
  const auto t1 = std::chrono::steady_clock::now();
  e = h->dev->solve(solve_options(h->opt));
  if (!e.empty()) {
    h->solved = false;
    return fail(h, h->dev->stats().error ? EIK_ERR_DEVICE : EIK_ERR_CUDA, e);
  }
  h->solved = true;
  const SolveStats& st = h->dev->stats();
  eik_stats& s = h->stats;
  fill_stats(s, st, on_device ? h->dlayout : h->layout, std::chrono::duration<float, std::milli>(t1 - t0).count());
  if (h->opt.verbose) {
    std::printf("Eikonal GB300: %d blocks, %d iterations, %.3f ms solve, %.3f ms setup\n", h->nb, st.iterations,
                st.solve_ms, s.setup_ms);
  }
  return EIK_OK;
}

int eik_prepare(eik_solver* h) {
  if (!h) return EIK_ERR_ARG;
  if (h->nv == 0) return fail(h, EIK_ERR_STATE, "no mesh: call eik_set_mesh or eik_load_mesh first");
  bool nl = false;
  const int rc = host_prepare(h, &nl);
  if (rc) return rc;
  // the layout the next (host-built) solve will use
  const Layout& L = h->layout;
  h->stats.num_blocks = L.nb;
  h->stats.max_slots_per_block = L.max_slots;
  h->stats.max_local_vertices = L.max_local;
  h->stats.total_slots = L.total_slots;
  h->stats.mean_slots_per_block = L.mean_slots_per_block;
  h->stats.mean_halo_per_block = L.mean_halo_per_block;
  h->stats.flagged_tets = L.flagged_tets;
  return EIK_OK;
}

int eik_num_vertices(const eik_solver* h) { return h ? h->nv : 0; }

int eik_num_elements(const eik_solver* h) { return h ? h->ne : 0; }

int eik_num_iterations(const eik_solver* h) { return (h && h->solved) ? h->stats.iterations : 0; }

int eik_get_result(const eik_solver* h, float* out, int nv) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h || !out) return fail(m, EIK_ERR_ARG, "null argument");
  if (!h->solved) return fail(m, EIK_ERR_STATE, "no solve has completed");
  if (nv != h->nv) return fail(m, EIK_ERR_ARG, "output size mismatch");
  std::string e = h->dev->result(out);
  return e.empty() ? EIK_OK : fail(m, EIK_ERR_CUDA, e);
}

int eik_get_result_device(const eik_solver* h, float* out_dev, int nv) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h || !out_dev) return fail(m, EIK_ERR_ARG, "null argument");
  if (!h->solved) return fail(m, EIK_ERR_STATE, "no solve has completed");
  if (nv != h->nv) return fail(m, EIK_ERR_ARG, "output size mismatch");
  std::string e = h->dev->result_device(out_dev);
  return e.empty() ? EIK_OK : fail(m, EIK_ERR_CUDA, e);
}

int eik_get_iteration(const eik_solver* h, int i, float* out, int nv) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h || !out) return fail(m, EIK_ERR_ARG, "null argument");
  if (!h->solved) return fail(m, EIK_ERR_STATE, "no solve has completed");
  if (nv != h->nv) return fail(m, EIK_ERR_ARG, "output size mismatch");
  if (i < 0 || i >= h->stats.iterations) return fail(m, EIK_ERR_ARG, "iteration index out of range");
  if (!h->opt.keep_history) return fail(m, EIK_ERR_STATE, "history was not kept (keep_history = 0)");
  std::string e = h->dev->history(i, out);
  return e.empty() ? EIK_OK : fail(m, EIK_ERR_CUDA, e);
}

int eik_get_partition(const eik_solver* h, int* labels, int nv, int* nblocks) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h) return EIK_ERR_ARG;
  if (h->labels.empty()) return fail(m, EIK_ERR_STATE, "no partition yet");
  if (nblocks) *nblocks = h->nb;
  if (labels) {
    if (nv != h->nv) return fail(m, EIK_ERR_ARG, "size mismatch");
    std::memcpy(labels, h->labels.data(), sizeof(int) * nv);
  }
  return EIK_OK;
}

int eik_get_stats(const eik_solver* h, eik_stats* s) {
  if (!h || !s) return EIK_ERR_ARG;
  *s = h->stats;
  return EIK_OK;
}

int eik_get_iteration_stats(const eik_solver* h, long long* out, int cap) {
  if (!h || cap < 0 || (cap > 0 && !out)) return -EIK_ERR_ARG;
  if (!h->solved || !h->dev) return -EIK_ERR_STATE;
  const std::vector<long long>& v = h->dev->stats().iter_stats;
  const int n = std::min(cap, (int)(v.size() / kIterStatWords));
  if (n > 0) std::memcpy(out, v.data(), sizeof(long long) * kIterStatWords * (size_t)n);
  return n;
}

int eik_write_vtk(const eik_solver* h, const char* prefix, int all) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h || !prefix) return fail(m, EIK_ERR_ARG, "null argument");
  if (!h->solved) return fail(m, EIK_ERR_STATE, "no solve has completed");
  std::vector<float> vals(h->nv);
  const std::vector<int>& el = (h->dim == 2) ? h->prep.faces : h->elems;
  const int nit = h->stats.iterations;
  std::vector<int> which;
  if (all && h->opt.keep_history) for (int i = 0; i < nit; ++i) which.push_back(i);
  else which.push_back(-1);
  int j = 0;
  for (int i : which) {
    int rc = (i < 0) ? eik_get_result(h, vals.data(), h->nv) : eik_get_iteration(h, i, vals.data(), h->nv);
    if (rc) return rc;
    const std::string path = std::string(prefix) + std::to_string(j++) + ".vtk";
    std::string e = write_vtk(path, h->dim, h->xyz, el, vals.data(), h->nv);
    if (!e.empty()) return fail(m, EIK_ERR_IO, e);
  }
  return EIK_OK;
}

int eik_tri_prep(const eik_solver* h, int* nf, int* nvirt, int* faces, unsigned char* obtuse, int* vf_off,
                 int* vf_verts) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h) return EIK_ERR_ARG;
  if (h->dim != 2 || h->prep_mesh != h->mesh_ver) return fail(m, EIK_ERR_STATE, "no triangle mesh set");
  const TriPrep& P = h->prep;
  if (nf) *nf = P.nf;
  if (nvirt) *nvirt = (int)(P.vf_verts.size() / 3);
  if (faces) std::memcpy(faces, P.faces.data(), sizeof(int) * P.faces.size());
  if (obtuse) std::memcpy(obtuse, P.obtuse.data(), P.obtuse.size());
  if (vf_off) std::memcpy(vf_off, P.vf_off.data(), sizeof(int) * P.vf_off.size());
  if (vf_verts && !P.vf_verts.empty()) std::memcpy(vf_verts, P.vf_verts.data(), sizeof(int) * P.vf_verts.size());
  return EIK_OK;
}

int eik_tet_gram(const eik_solver* h, int from_device, float* out, long long n) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h || !out) return EIK_ERR_ARG;
  if (h->dim != 3) return fail(m, EIK_ERR_STATE, "not a tet mesh");
  if (n != 6 * (long long)h->ne) return fail(m, EIK_ERR_ARG, "out must hold 6 floats per tet");
  const Layout* L = nullptr;
  std::vector<float> dcoef;
  std::vector<int> dse;
  const std::vector<float>* coef = nullptr;
  const std::vector<int>* se = nullptr;
  if (from_device) {
    if (!h->dev || !h->solved) return fail(m, EIK_ERR_STATE, "no solve has run");
    const bool built = h->dev->layout_built_on_device();
    L = built ? &h->dlayout : &h->layout;
    std::string e = h->dev->layout_arrays(&dcoef, built ? &dse : nullptr);
    if (!e.empty()) return fail(m, EIK_ERR_CUDA, e);
    coef = &dcoef;
    se = built ? &dse : &L->slot_elem;
  } else {
    if (h->lay_mesh != h->mesh_ver || h->layout.nb == 0) return fail(m, EIK_ERR_STATE, "no host layout: call eik_prepare");
    L = &h->layout;
    coef = &L->coef;
    se = &L->slot_elem;
  }
  std::vector<char> seen((size_t)h->ne, 0);
  for (const BlockDesc& d : L->blocks)
    for (int j = 0; j < d.nslots; ++j) {
      const int t = (*se)[(size_t)d.slot_begin + j];
      if (t < 0 || t >= h->ne) continue;
      for (int k = 0; k < 6; ++k) {
        const float v = (*coef)[6 * (size_t)d.slot_begin + (size_t)k * d.nslots_pad + j];
        float& o = out[6 * (size_t)t + k];
        if (!seen[t]) o = v;
        else if (std::memcmp(&o, &v, sizeof(float)) != 0)
          return fail(m, EIK_ERR_STATE, "copies of tet " + std::to_string(t) + " differ");
      }
      seen[t] = 1;
    }
  for (int t = 0; t < h->ne; ++t)
    if (!seen[t]) return fail(m, EIK_ERR_STATE, "tet " + std::to_string(t) + " has no slot");
  return EIK_OK;
}

int eik_tri_prep_values(const eik_solver* h, float* edges, float* speed_inv, float* vf_edges, float* vf_speed_inv) {
  eik_solver* m = const_cast<eik_solver*>(h);
  if (!h) return EIK_ERR_ARG;
  if (h->dim != 2 || h->prep_mesh != h->mesh_ver) return fail(m, EIK_ERR_STATE, "no triangle mesh set");
  const TriPrep& P = h->prep;
  const size_t nvf = P.vf_verts.size() / 3;
  if (edges) std::memcpy(edges, P.edges.data(), sizeof(float) * P.edges.size());
  if (speed_inv) {
    const std::vector<float> inv = speed_inverse(h);
    std::memcpy(speed_inv, inv.data(), sizeof(float) * inv.size());
  }
  if (vf_edges && nvf) std::memcpy(vf_edges, P.vf_edges.data(), sizeof(float) * P.vf_edges.size());
  // virtual faces take the inverse speed of the reference's default speed type
  // (ONE, TriMesh.h:240-257), whatever the faces' speeds
  if (vf_speed_inv)
    for (size_t i = 0; i < nvf; ++i) vf_speed_inv[i] = 1.0f;
  return EIK_OK;
}

int eik_selftest_wait_timeout(double* waited_ms) {
  int status = 0;
  double ms = 0;
  if (!selftest_wait_timeout(&status, &ms).empty()) return EIK_ERR_CUDA;
  if (waited_ms) *waited_ms = ms;
  return status ? EIK_ERR_DEVICE : EIK_OK;
}

int eik_selftest_local_update(int which, const float* in, float* out, int n) {
  if (which < 0 || which > 6 || n < 0 || (n > 0 && (!in || !out))) return EIK_ERR_ARG;
  return selftest_device(which, in, out, n).empty() ? EIK_OK : EIK_ERR_CUDA;
}

// Allocation-free 3D solve: see the header.  Builds the partition and the block
// layout on the host, then runs the solve with every device buffer inside the
// library's fixed scratch array.
int eik_solve3d_noalloc(const float* xyz, int nv, const int* tets, int nt, const float* speeds, long long nspeeds,
                        const int* seeds, int nseeds, int max_verts_per_block, int max_iterations, float* out_times,
                        void* stream, int* iterations, char* errbuf, int errlen) {
  auto report = [&](int code, const std::string& msg) {
    if (errbuf && errlen > 0) {
      std::snprintf(errbuf, (size_t)errlen, "%s", msg.c_str());
    }
    return code;
  };
  if (!xyz || !tets || !out_times || nv <= 0 || nt <= 0 || nseeds < 0 || (nseeds > 0 && !seeds) ||
      (nspeeds > 0 && !speeds) || max_verts_per_block <= 0 || max_iterations < 0)
    return report(EIK_ERR_ARG, "invalid argument");
  std::vector<int> el(tets, tets + 4 * (size_t)nt);
  std::string msg = normalize_index_base(el, nv);
  if (!msg.empty()) return report(EIK_ERR_MESH, msg);
  std::vector<int> sd = (nseeds > 0) ? std::vector<int>(seeds, seeds + nseeds) : std::vector<int>(1, 0);
  for (int v : sd)
    if (v < 0 || v >= nv) return report(EIK_ERR_ARG, "seed out of range");
  // the same speed / metric checks as eik_solve
  msg = speed_values_problem(nspeeds > 0 ? speeds : nullptr, (size_t)std::max(0ll, nspeeds), nt, 3);
  if (!msg.empty()) return report(EIK_ERR_ARG, msg);
  std::vector<float> M;
  tet_metrics(nt, nspeeds > 0 ? speeds : nullptr, (size_t)std::max(0ll, nspeeds), M);
  std::vector<int> labels;
  const int nb = metis_rule_blocks(nv, max_verts_per_block, 3);
  partition_rcb(nv, xyz, nb, labels);
  Layout L;
  msg = build_layout3d(nv, xyz, nt, el.data(), M.data(), labels.data(), nb, L);
  if (!msg.empty()) return report(EIK_ERR_MESH, msg);
  int it = 0;
  size_t need = 0;
  NoAllocFailure kind = NoAllocFailure::kNone;
  msg = solve3d_noalloc(L, sd, max_iterations, out_times, (cudaStream_t)stream, &it, &need, &kind);
  if (!msg.empty())
    return report(kind == NoAllocFailure::kLimit    ? EIK_ERR_LIMIT
                  : kind == NoAllocFailure::kDevice ? EIK_ERR_DEVICE
                                                    : EIK_ERR_CUDA,
                  msg);
  if (iterations) *iterations = it;
  return EIK_OK;
}

}  // extern "C"

// ---- request server support ---------------------------------------------------

int eikgb::snapshot_for_server(eik_solver* h, MeshSnapshot& out, std::string& err) {
  if (!h) return EIK_ERR_ARG;
  if (h->nv == 0) {
    err = "no mesh: call eik_set_mesh or eik_load_mesh first";
    return EIK_ERR_STATE;
  }
  out.built.reset();
  if (use_device_setup(h)) {
    // the layout built on the device, kept there until the server replicates it
    int rc = check_speeds(h);
    if (!rc) rc = ensure_partition(h);
    if (rc) {
      err = h->err;
      return rc;
    }
    cudaStream_t st = new_stream();
    if (!st) {
      err = "CUDA stream creation failed (no usable GPU?)";
      return EIK_ERR_CUDA;
    }
    std::shared_ptr<Built3D> b(new Built3D, [](Built3D* x) {
      x->release();
      delete x;
    });
    std::string e;
    if (h->dim == 3) {
      std::vector<float> ones;
      int mcomp = 6;
      const float* M = compact_metrics(h, ones, &mcomp);
      e = build_layout3d_device(h->nv, h->xyz.data(), h->ne, h->elems.data(), M, mcomp, h->labels.data(), h->nb, st,
                                *b, out.layout);
    } else {
      e = build_layout2d_device(h->nv, h->prep, face_speeds(h), h->labels.data(), h->nb, st, *b, out.layout);
    }
    free_stream(st);
    if (!e.empty()) {
      err = e;
      return e.find("too many local") != std::string::npos ? EIK_ERR_LIMIT : EIK_ERR_CUDA;
    }
    out.built = b;
  } else {
    bool nl = false;
    int rc = host_prepare(h, &nl);
    if (rc) {
      err = h->err;
      return rc;
    }
    out.layout = h->layout;
  }
  out.dim = h->dim;
  out.nv = h->nv;
  out.ne = h->ne;
  out.xyz = h->xyz;
  out.max_iterations = h->opt.max_iterations;
  out.fim_sweeps = h->opt.fim_sweeps;
  out.threads = h->opt.threads_per_block;
  if (h->dim == 3) {
    out.elems = h->elems;
    tet_metrics(h->ne, h->speeds_set ? h->speeds.data() : nullptr, h->speeds.size(), out.M6);
  } else {
    out.speed.assign(h->ne, 1.0f);
    if (h->speeds_set && (int)h->speeds.size() == h->ne) out.speed = h->speeds;
  }
  return EIK_OK;
}

extern "C" {

// ---- batches ----------------------------------------------------------------

struct eik_batch {
  std::vector<eik_solver*> solvers;
  std::vector<std::string> keys;  // per handle: layout identity at pack time
  Layout layout;
  std::unique_ptr<DeviceSolve> dev;
  bool packed = false, solved = false, have_host = false;
  std::vector<float> host_result;
  std::vector<int> iters;
  eik_stats stats{};
  std::string err;
};

namespace {

int bfail(eik_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

std::string layout_identity(const eik_solver* h) {
  return std::to_string(h->lay_mesh) + "/" + h->lay_key + "/" + std::to_string(h->lay_speed);
}

// A batch builds its layout on the device when every handle would build its own
// there (device_setup = 1; 3D precision mode builds on the host).
bool batch_on_device(const eik_batch* b) {
  for (const eik_solver* h : b->solvers)
    if (!use_device_setup(h)) return false;
  return true;
}

// The batch's layout built on the device in one pass: the instances' meshes as one
// disconnected mesh, vertex, element and block ids offset instance by instance.
// Its layout is the concatenation of the instances' own layouts (concat_layouts):
// the renumbering orders vertices by block, slots, halo lists and the 2D copy cap
// are decided block by block or vertex by vertex, and no element or block spans
// two instances.
std::string batch_device_pack(eik_batch* b) {
  const int n = (int)b->solvers.size();
  const int dim = b->solvers[0]->dim;
  Layout& L = b->layout;
  std::vector<int> labels, bbeg{0}, vbeg{0};
  int nb = 0, nv = 0, ne = 0;
  for (const eik_solver* h : b->solvers) {
    for (int l : h->labels) labels.push_back(l + nb);
    nb += h->nb;
    nv += h->nv;
    ne += h->ne;
    bbeg.push_back(nb);
    vbeg.push_back(nv);
  }
  if (!b->dev) b->dev.reset(new DeviceSolve);
  cudaStream_t st = (cudaStream_t)b->dev->stream();
  Built3D built;
  std::string e;
  if (dim == 2) {
    TriPrep U;
    U.nv = nv;
    U.vf_off.push_back(0);
    std::vector<float> speeds;
    speeds.reserve(ne);
    int voff = 0, vfoff = 0;
    for (const eik_solver* h : b->solvers) {
      const TriPrep& P = h->prep;
      for (int x : P.faces) U.faces.push_back(x + voff);
      U.obtuse.insert(U.obtuse.end(), P.obtuse.begin(), P.obtuse.end());
      U.edges.insert(U.edges.end(), P.edges.begin(), P.edges.end());
      U.vf_edges.insert(U.vf_edges.end(), P.vf_edges.begin(), P.vf_edges.end());
      for (int i = 1; i <= P.nf; ++i) U.vf_off.push_back(P.vf_off[i] + vfoff);
      for (int x : P.vf_verts) U.vf_verts.push_back(x + voff);
      const float* sp = face_speeds(h);
      if (sp) speeds.insert(speeds.end(), sp, sp + P.nf);
      else speeds.insert(speeds.end(), (size_t)P.nf, 1.0f);
      U.nf += P.nf;
      vfoff += P.vf_off[P.nf];
      voff += h->nv;
    }
    e = build_layout2d_device(nv, U, speeds.data(), labels.data(), nb, st, built, L);
  } else {
    // scalar metrics stay one float per tet unless some instance gives 6 entries,
    // then every instance's are expanded (s I: the same products)
    bool full = false;
    for (const eik_solver* h : b->solvers) full = full || (h->speeds_set && h->speeds.size() == 6 * (size_t)h->ne);
    std::vector<float> xyz, M;
    std::vector<int> tets;
    xyz.reserve(3 * (size_t)nv);
    tets.reserve(4 * (size_t)ne);
    int voff = 0;
    for (const eik_solver* h : b->solvers) {
      xyz.insert(xyz.end(), h->xyz.begin(), h->xyz.end());
      for (int x : h->elems) tets.push_back(x + voff);
      if (full) {
        std::vector<float> m6;
        tet_metrics(h->ne, h->speeds_set ? h->speeds.data() : nullptr, h->speeds.size(), m6);
        M.insert(M.end(), m6.begin(), m6.end());
      } else {
        std::vector<float> ones;
        int mc = 1;
        const float* m = compact_metrics(h, ones, &mc);
        M.insert(M.end(), m, m + h->ne);
      }
      voff += h->nv;
    }
    e = build_layout3d_device(nv, xyz.data(), ne, tets.data(), M.data(), full ? 6 : 1, labels.data(), nb, st, built,
                              L);
  }
  if (!e.empty()) {
    built.release();
    return e;
  }
  L.ninst = n;
  L.inst_bbeg = bbeg;
  L.inst_vbeg = vbeg;
  L.blk_inst.assign(nb, 0);
  for (int i = 0; i < n; ++i)
    for (int k = bbeg[i]; k < bbeg[i + 1]; ++k) L.blk_inst[k] = i;
  e = b->dev->upload_built(L, built);
  if (!e.empty()) built.release();
  return e;
}

}  // namespace

int eik_batch_create(eik_solver* const* solvers, int n, eik_batch** out) {
  if (!out || !solvers || n <= 0) return EIK_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!solvers[i]) return EIK_ERR_ARG;
    if (solvers[i]->dim != solvers[0]->dim) return fail(solvers[i], EIK_ERR_ARG, "batch mixes 2D and 3D handles");
  }
  eik_batch* b = new eik_batch;
  b->solvers.assign(solvers, solvers + n);
  *out = b;
  return EIK_OK;
}

void eik_batch_destroy(eik_batch* b) { delete b; }

int eik_batch_solve(eik_batch* b) {
  if (!b) return EIK_ERR_ARG;
  const auto t0 = std::chrono::steady_clock::now();
  const int n = (int)b->solvers.size();
  std::vector<std::vector<int>> seeds(n);
  std::vector<const float*> init(n, nullptr);
  bool repack = !b->packed || (int)b->keys.size() != n;
  b->keys.resize(n);
  const bool on_device = batch_on_device(b);
  for (int i = 0; i < n; ++i) {
    eik_solver* h = b->solvers[i];
    if (h->nv == 0) return bfail(b, EIK_ERR_STATE, "instance " + std::to_string(i) + ": no mesh");
    int rc = resolve_seeds(h, seeds[i], &init[i]);
    if (rc) return bfail(b, rc, "instance " + std::to_string(i) + ": " + h->err);
    std::string key;
    if (on_device) {
      rc = check_speeds(h);
      if (!rc) rc = ensure_partition(h);
      key = "device/" + std::to_string(h->mesh_ver) + "/" + partition_key(h) + "/" + std::to_string(h->speed_ver);
    } else {
      bool nl = false;
      rc = host_prepare(h, &nl);
      key = layout_identity(h);
    }
    if (rc) return bfail(b, rc, "instance " + std::to_string(i) + ": " + h->err);
    if (key != b->keys[i]) repack = true;
    b->keys[i] = key;
  }
  if (repack) {
    b->packed = false;
    std::string e;
    if (on_device) {
      e = batch_device_pack(b);
      if (!e.empty())
        return bfail(b, e.find("too many local") != std::string::npos || e.find("shared memory") != std::string::npos
                            ? EIK_ERR_LIMIT
                            : EIK_ERR_CUDA,
                     e);
    } else {
      std::vector<const Layout*> parts(n);
      for (int i = 0; i < n; ++i) parts[i] = &b->solvers[i]->layout;
      e = concat_layouts(parts, b->layout);
      if (!e.empty()) return bfail(b, EIK_ERR_ARG, e);
      if (!b->dev) b->dev.reset(new DeviceSolve);
      e = b->dev->upload(b->layout);
      if (!e.empty()) return bfail(b, e.find("shared memory") != std::string::npos ? EIK_ERR_LIMIT : EIK_ERR_CUDA, e);
    }
    b->packed = true;
  }
  std::string e = b->dev->set_seeds_multi(seeds, init);
  if (!e.empty()) return bfail(b, EIK_ERR_ARG, e);
  const auto t1 = std::chrono::steady_clock::now();
  SolveOptions so = solve_options(b->solvers[0]->opt);
  so.keep_history = false;
  so.inst_max_iterations.resize(n);
  for (int i = 0; i < n; ++i) so.inst_max_iterations[i] = b->solvers[i]->opt.max_iterations;
  b->solved = false;
  b->have_host = false;
  e = b->dev->solve(so);
  if (!e.empty()) return bfail(b, b->dev->stats().error ? EIK_ERR_DEVICE : EIK_ERR_CUDA, e);
  b->solved = true;
  b->iters = b->dev->stats().inst_iters;
  fill_stats(b->stats, b->dev->stats(), b->layout, std::chrono::duration<float, std::milli>(t1 - t0).count());
  return EIK_OK;
}

int eik_batch_num_instances(const eik_batch* b) { return b ? (int)b->solvers.size() : 0; }

int eik_batch_num_vertices(const eik_batch* b, int i) {
  if (!b || i < 0 || i >= (int)b->solvers.size()) return 0;
  return b->solvers[i]->nv;
}

int eik_batch_num_iterations(const eik_batch* b, int i) {
  if (!b || !b->solved || i < 0 || i >= (int)b->iters.size()) return 0;
  return b->iters[i];
}

int eik_batch_get_results(eik_batch* b, float* out, long long n) {
  if (!b || !out) return EIK_ERR_ARG;
  if (!b->solved) return bfail(b, EIK_ERR_STATE, "no batch solve yet");
  if (n != b->layout.nv) return bfail(b, EIK_ERR_ARG, "size mismatch");
  if (!b->have_host) {
    b->host_result.resize(b->layout.nv);
    std::string e = b->dev->result(b->host_result.data());
    if (!e.empty()) return bfail(b, EIK_ERR_CUDA, e);
    b->have_host = true;
  }
  std::memcpy(out, b->host_result.data(), sizeof(float) * (size_t)n);
  return EIK_OK;
}

int eik_batch_get_result(eik_batch* b, int i, float* out, int nv) {
  if (!b || !out || i < 0 || i >= (int)b->solvers.size()) return EIK_ERR_ARG;
  if (!b->solved) return bfail(b, EIK_ERR_STATE, "no batch solve yet");
  const int v0 = b->layout.inst_vbeg[i], cnt = b->layout.inst_vbeg[i + 1] - v0;
  if (nv != cnt) return bfail(b, EIK_ERR_ARG, "size mismatch");
  if (!b->have_host) {
    b->host_result.resize(b->layout.nv);
    std::string e = b->dev->result(b->host_result.data());
    if (!e.empty()) return bfail(b, EIK_ERR_CUDA, e);
    b->have_host = true;
  }
  std::memcpy(out, b->host_result.data() + v0, sizeof(float) * (size_t)cnt);
  return EIK_OK;
}

int eik_batch_get_results_device(eik_batch* b, float* out_dev, long long n) {
  if (!b || !out_dev) return EIK_ERR_ARG;
  if (!b->solved) return bfail(b, EIK_ERR_STATE, "no batch solve yet");
  if (n != b->layout.nv) return bfail(b, EIK_ERR_ARG, "size mismatch");
  std::string e = b->dev->result_device(out_dev);
  if (!e.empty()) return bfail(b, EIK_ERR_CUDA, e);
  return EIK_OK;
}

int eik_batch_get_stats(const eik_batch* b, eik_stats* s) {
  if (!b || !s) return EIK_ERR_ARG;
  *s = b->stats;
  return EIK_OK;
}

void* eik_batch_stream(const eik_batch* b) { return (b && b->dev) ? b->dev->stream() : nullptr; }

const char* eik_batch_last_error(const eik_batch* b) { return b ? b->err.c_str() : "null handle"; }

void* eik_stream(const eik_solver* h) { return (h && h->dev) ? h->dev->stream() : nullptr; }

const char* eik_last_error(const eik_solver* h) { return h ? h->err.c_str() : "null handle"; }

const char* eik_version(void) { return "eikonal-gb300 0.1 (sm_103a)"; }

}  // extern "C"
