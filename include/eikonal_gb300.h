/* eikonal_gb300.h — C ABI of the GB300 block-FIM Eikonal solver.
 *
 * This is the drop-in boundary for the reference's `Eikonal` class
 * (SCI-Solver_Eikonal src/Eikonal.h:14-61, src/Eikonal.cu): plain pointers and
 * sizes, status codes instead of exit(), no C++ or torch types.  A C++ class with
 * the reference's member names sits on top of it (Eikonal.h in this directory).
 *
 * Call order: create -> set_options (optional) -> set_mesh / load_mesh ->
 * set_speeds / set_initial_values / set_seeds / set_partition (optional, any
 * order) -> solve -> get_result / get_iteration.  A handle may be solved again
 * after changing speeds or seeds; unchanged mesh + partition data stay resident
 * on the GPU between solves.
 *
 * Every function returns EIK_OK (0) or an error code; eik_last_error() gives the
 * message of the last failure on that handle.  Handles are not thread-safe; use
 * one handle per host thread.
 */
#ifndef EIKONAL_GB300_H
#define EIKONAL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define EIK_OK 0
#define EIK_ERR_ARG 1    /* bad argument: null pointer, size mismatch, index out of range */
#define EIK_ERR_STATE 2  /* call order: e.g. solve() before a mesh is set */
#define EIK_ERR_MESH 3   /* unreadable or invalid mesh (the reference calls exit(1)) */
#define EIK_ERR_CUDA 4   /* CUDA runtime failure (the reference calls exit(-1)) */
#define EIK_ERR_LIMIT 5  /* a block does not fit in shared memory; use smaller blocks */
#define EIK_ERR_DEVICE 6 /* a device-side bounded wait expired */
#define EIK_ERR_IO 7     /* file output failed */
#define EIK_ERR_CANCELLED 8 /* a server request cancelled before it completed */

#define EIK_SPEED_ONE 1 /* the reference's speedType_ ONE (src/core2d/include/TriMesh.h:15-16) */

#define EIK_PARTITION_RCB 0   /* recursive coordinate bisection (default) */
#define EIK_PARTITION_METIS 1 /* METIS k-way on the vertex graph, as GraphPartition_METIS2
                                 (meshFIM3dEikonal.cu:153-237, meshFIM2d_eikonal.cu:111-204) */

typedef struct eik_solver eik_solver;

/* Public fields of the reference's Eikonal class (src/Eikonal.h:43-60) with its
 * constructor defaults (src/Eikonal.cu:4-24), plus two additions at the end. */
typedef struct eik_options {
  int max_blocks;          /* maxBlocks_ (16); overwritten by the partitioner like the reference */
  int max_verts_per_block; /* maxVertsPerBlock_ (64) */
  float stop_distance;     /* stopDistance_ (50000); stored, unused by the scheme as in the reference */
  int is_structured;       /* isStructured_ (0): lexicographic grid tiling instead of graph partition */
  int speed_type;          /* speedType_ (EIK_SPEED_ONE) */
  int square_length, square_width, square_depth;                 /* squareLength_/Width_/Depth_ (16) */
  int square_block_length, square_block_width, square_block_depth; /* squareBlock*_ (1) */
  int max_iterations;      /* maxIterations_ (100) */
  int verbose;             /* verbose_ (0) */
  int keep_history;        /* 1 (default): keep every iteration for eik_get_iteration */
  int fim_sweeps;          /* sweeps per active-block visit; -1 = reference (3D 2, 2D 7) */
  int direct_launch;       /* 0 (default): a solve is one CUDA-graph launch; 1: the same kernels
                              launched one by one with a host check per iteration, for profilers
                              that cannot see kernels inside conditional graphs */
  int threads_per_block;   /* CTA size of the 3D block-sweep kernels (128/256/384/512/768/1024).
                              0 (default): 384 for the apex-item kernels (three CTAs per SM);
                              for the slot kernels (precision mode, blocks too large for the
                              item kernels' shared memory) chosen per handle over its first
                              solves between one thread per slot of the largest block and 512,
                              by measured speed.  Results do not depend on it.  The slot check
                              kernel runs CTAs of half the size when this is 1024. */
  int precision;           /* 0 (default): the reference's FP32 arithmetic, bit for bit.  1 (3D):
                              tets whose metric edge Gram matrix has condition number above
                              precision_kappa (slivers, strong anisotropy) run their local
                              updates in FP64 from FP64 metric edge products; every other tet
                              stays FP32.  An FP64 residual check runs after the solve. */
  float precision_kappa;   /* flagging threshold on ||G||_F ||G^-1||_F (1e4) */
  int device_setup;        /* 1 (default): a solve builds its block layout (renumbering, element slots,
                              halo lists, metric edge products or inverse face speeds,
                              neighbour graph) on the GPU; 2D meshes keep their triangle
                              preparation (orientation, obtuse corners, virtual faces) on the
                              host.  0: on the host.  Same layout, same results.  A batch builds
                              on the device when all its handles do (one pass over all
                              instances); 3D precision mode and the server build on the host. */
  int partitioner;         /* EIK_PARTITION_RCB (default) or EIK_PARTITION_METIS: the reference's
                              partitioner kind, here METIS 5 from the CUDA toolkit where the
                              reference calls METIS 4 (so labels differ from the reference's);
                              EIK_ERR_ARG when the library was built without it.  Ignored when
                              is_structured is set or labels are given (eik_set_partition). */
  int telemetry;           /* 1 (default): every launch of the loop records its span on the device
                              timer and its visit counts (eik_get_iteration_stats, the *_kernel_ms
                              and *_launches fields of eik_stats); 0: none of that, and the solve
                              runs about 1.5% faster on a 1.6M-tet mesh.  Results do not depend
                              on it. */
} eik_options;

typedef struct eik_stats {
  int iterations;            /* outer iterations run (= numIterations()) */
  int num_blocks;
  long long vertex_updates;  /* owned vertices x sweeps summed over block visits */
  long long fim_visits;      /* active-block visits */
  long long check_visits;    /* neighbour-check visits */
  long long slot_visits;     /* element slots streamed */
  long long halo_visits;     /* halo vertices gathered */
  long long owned_visits;    /* owned vertices loaded/stored */
  float solve_ms;            /* device time of the last solve (CUDA events) */
  float setup_ms;            /* host setup of the last solve (partition, layout, upload) */
  int max_slots_per_block;
  int max_local_vertices;
  int total_slots;
  double mean_slots_per_block;
  double mean_halo_per_block;
  int device_error;          /* device error flags of the last solve */
  /* per-kernel figures of the last solve, from a device timer around every launch */
  float fim_kernel_ms;       /* summed launch spans of the block-sweep kernel */
  float check_kernel_ms;     /* summed launch spans of the neighbour-check kernel (0 where the
                                3D checks run inside the sweep kernel: the item kernels) */
  int fim_launches, check_launches;  /* launches that visited blocks (check: 0 as above) */
  long long fim_slots, fim_halo, fim_owned; /* inputs streamed by the block-sweep kernel */
  long long h2d_bytes;       /* host-to-device bytes copied by the last solve (initial state) */
  /* precision mode (precision = 1) */
  long long flagged_tets;    /* tets whose updates run in FP64 */
  /* FP64 check of the final times, c_v = min over incident tets of the FP64 update: */
  double residual_max_abs;   /* max (T_v - c_v) over vertices with c_v < T_v (more updates would lower T_v) */
  double residual_max_rel;   /* the same relative to T_v */
  long long residual_vertices; /* vertices with (T_v - c_v) > 1e-5 * T_v */
  /* precision mode's polish: after the solve, blocks owning a vertex that the FP64
   * update of its tets would lower by more than 1e-6 relative run the loop again
   * with every slot's update in FP64, round after round (at most 8) */
  int polish_rounds;          /* rounds run */
  long long polish_blocks;    /* blocks queued over those rounds */
  double residual_below_rel; /* max (c_v - T_v) / T_v over vertices below every FP64 update of their
                                tets: the local update is not monotone in its inputs, so a time can
                                end below the update of its final neighbour times (the FP64 run of
                                the scheme does too); no further update changes these */
} eik_stats;

/* Fills `o` with the reference's defaults (src/Eikonal.cu:4-24). */
void eik_default_options(eik_options* o);

/* Eikonal(isTriMesh, ...) — src/Eikonal.cu:4-24.  is_tri_mesh: 1 = 2D triangles, 0 = 3D tets. */
int eik_create(int is_tri_mesh, eik_solver** out);
/* ~Eikonal — src/Eikonal.cu:26-35.  Null is ignored. */
void eik_destroy(eik_solver* h);

int eik_set_options(eik_solver* h, const eik_options* o);
int eik_get_options(const eik_solver* h, eik_options* o);

/* initializeMesh from memory — src/Eikonal.cu:99-133 (TriMesh::read /
 * tetgenio::load_tetmesh + TetMesh::init).  xyz: 3*nv floats; elems: 3*ne (2D)
 * or 4*ne (3D) vertex ids starting at 0 or 1 (tetmesh.cu:27-52). */
int eik_set_mesh(eik_solver* h, const float* xyz, int nv, const int* elems, int ne);
/* initializeMesh from a file: 2D ASCII .ply, 3D TetGen basename (.node/.ele).
 * Returns EIK_ERR_MESH where the reference exits with status 1. */
int eik_load_mesh(eik_solver* h, const char* filename);

/* initSpeedMtxMultipliers — src/Eikonal.cu:62-67.  2D: ne speeds (inverse speed
 * 1/s per triangle, TriMesh_stats.cu:64-68); 3D: ne scalars (metric s*I) or 6*ne
 * metric entries M00 M01 M02 M11 M12 M22 (tetmesh.cu:54-79); any other count
 * means unit speed, as in the reference.  n = 0 clears. */
int eik_set_speeds(eik_solver* h, const float* vals, long long n);

/* initializeVertices — src/Eikonal.cu:69-97: vertices whose value is 0 are seeds. */
int eik_set_initial_values(eik_solver* h, const float* vals, int nv);

/* Explicit seed list (same effect as initial values with zeros at the seeds). */
int eik_set_seeds(eik_solver* h, const int* seeds, int n);

/* Use these block labels (0..nblocks-1 per vertex) instead of the built-in
 * partitioner (the reference calls METIS_PartGraphKway here,
 * meshFIM2d_eikonal.cu:111-204 / meshFIM3dEikonal.cu:153-237).  labels = NULL
 * returns to the built-in partitioner. */
int eik_set_partition(eik_solver* h, const int* labels, int nv, int nblocks);

/* solveEikonal — src/Eikonal.cu:135-231. */
int eik_solve(eik_solver* h);

/* The host half of solveEikonal alone (partition, block layout, metric terms),
 * without touching the GPU; afterwards eik_get_partition / eik_get_stats describe
 * the layout the next solve will use. */
int eik_prepare(eik_solver* h);

int eik_num_vertices(const eik_solver* h);
/* Triangles (2D) or tets (3D) of the mesh: triMesh_->faces.size() /
 * tetMesh_->tets.size() of the reference's public mesh members (src/Eikonal.h:54-55). */
int eik_num_elements(const eik_solver* h);
/* numIterations — src/Eikonal.cu:46-48. */
int eik_num_iterations(const eik_solver* h);
/* getFinalResult — src/Eikonal.cu:38-40 (nv floats, original vertex order). */
int eik_get_result(const eik_solver* h, float* out, int nv);
/* Same, into device memory (out_dev must hold nv floats on the current device). */
int eik_get_result_device(const eik_solver* h, float* out_dev, int nv);
/* getResultAtIteration — src/Eikonal.cu:42-44 (needs keep_history). */
int eik_get_iteration(const eik_solver* h, int i, float* out, int nv);
/* Block labels used by the last solve. */
int eik_get_partition(const eik_solver* h, int* labels, int nv, int* nblocks);
int eik_get_stats(const eik_solver* h, eik_stats* s);
/* Per-outer-iteration figures of the last solve (no counterpart in the reference,
 * whose GenerateData only prints totals under verbose, meshFIM3dEikonal.cu:544-548).
 * For iteration i, out[16*i .. 16*i+15] = sweep-kernel launch span (ns, device
 * timer), check-kernel launch span (ns), then the sweep kernel's block visits,
 * element slots, halo vertices and owned vertices, then the same four for the
 * neighbour checks of iteration i, then the sweep and check kernels' start times
 * (ns after the first iteration's sweep start; -1 where the kernel recorded none),
 * then the same four counts for the sweep visits of iteration i whose block was
 * staged by a check in the same visit.  Where the 3D checks run inside the sweep
 * kernel (the item kernels), the checks of iteration i run in the sweep launch of
 * iteration i+1 and there is no check launch (span 0, start -1).  Writes min(iterations, cap) rows and returns that count (>= 0), or
 * a negative status (-EIK_ERR_ARG, -EIK_ERR_STATE before the first solve). */
int eik_get_iteration_stats(const eik_solver* h, long long* out, int cap);
/* writeVTK — src/Eikonal.cu:50-60: <prefix><i>.vtk for the last (all=0) or every
 * (all=1) iteration; the reference's prefix is "result". */
int eik_write_vtk(const eik_solver* h, const char* prefix, int all);

/* 2D mesh preparation as the solver sees it after eik_set_mesh: oriented faces
 * and the virtual faces that unfold obtuse corners (meshFIM2d_eikonal.h:40-72).
 * Call with null arrays to get the sizes first. */
int eik_tri_prep(const eik_solver* h, int* nf, int* nvirt, int* faces, unsigned char* obtuse,
                 int* vf_off, int* vf_verts);
/* The six metric edge products of every tet (AC.BC, BC.CD, AC.CD, AD.BD, AC.AD,
 * BC.BD under the tet's metric) as the 3D block layout holds them, in tet order:
 * the values gettetmem computes for the reference's GetTetMem (meshFIM3dEikonal.cu:
 * 650-678).  from_device = 0: the host layout of the last eik_prepare / host-built
 * solve; 1: the layout on the device after a solve (built on the device or
 * uploaded).  Every slot copy of a tet must hold the same bits (EIK_ERR_STATE
 * otherwise).  out holds 6 * ne floats (n). */
int eik_tet_gram(const eik_solver* h, int from_device, float* out, long long n);
/* The values the 2D block layout takes from that preparation, in the same order:
 * per face the edge lengths |v1-v0|, |v2-v1|, |v0-v2| (TriMesh::need_faceedges,
 * TriMesh_connectivity.cu:54-75) and the inverse speed (InitializeAttributes,
 * TriMesh_stats.cu:64-68), per virtual face its edge lengths and inverse speed
 * (SplitFace, TriMesh.h:215-313).  Arrays of 3*nf, nf, 3*nvirt and nvirt floats
 * (sizes from eik_tri_prep); any may be null. */
int eik_tri_prep_values(const eik_solver* h, float* edges, float* speed_inv, float* vf_edges, float* vf_speed_inv);

/* Self-test of the device local updates on host arrays, element-wise:
 *   which = 0: tet update (localSolverTet1, core3d/cuda/CUDA_kernels.cu:69-225),
 *              9 inputs per case (TA TB TC ACAC ACBC ACCD BCBC BCCD CDCD), 1 output;
 *   which = 1: triangle update (core2d/cuda/CUDA_kernels.cu:143-204),
 *              7 inputs per case (TA TB TC LenAB LenBC LenAC speedInv), 1 output;
 *   which = 2: the FP32 forms of the reference's FP64 quotients, 2 inputs
 *              (num, h) -> 2 outputs (num/(h+1e-8), num/(2h));
 *   which = 3 / 4: each case is a triangle forming its own block (T0 T1 T2 LenAB
 *              (v0v1) LenBC (v1v2) LenCA (v2v0) speedInv), passed once through the
 *              2D block-sweep kernel (7 sweeps) / neighbour-check kernel (1 sweep);
 *              3 outputs per case;
 *   which = 5: the precision mode's FP64 tet update (no reference counterpart),
 *              inputs as for 0, the FP64 result rounded to FP32;
 *   which = 6: the four apex updates of one slot as the 3D visit kernels run them
 *              (FIMCuda's group, CUDA_kernels.cu:454-457, with its roundings), 10
 *              inputs per case (TA TB TC TD, then the stored products ACBC BCCD ACCD
 *              ADBD ACAD BCBD), 4 outputs min(T_k, update of apex k). */
int eik_selftest_local_update(int which, const float* in, float* out, int n);

/* Failure-path self-test (no counterpart in the reference, which has no bounded
 * waits): launches a kernel whose barrier waits for a copy that never comes.  The
 * wait gives up after about one second and reports it, as the solver kernels do
 * when a bulk copy does not land; the GPU context stays usable.  Returns
 * EIK_ERR_DEVICE when the wait gave up (the expected outcome), EIK_OK if it did not;
 * waited_ms (may be null) receives how long it waited. */
int eik_selftest_wait_timeout(double* waited_ms);

/* Allocation-free 3D solve.  No counterpart in the reference: an addition for
 * callers that cannot call cudaMalloc, such as code running while another
 * component captures the stream into a CUDA graph, real-time or embedded hosts
 * that reserve all device memory at start-up, and plugins whose host application
 * owns the device memory pool.
 *
 * Inputs and the output are host arrays, as in eik_set_mesh / eik_set_speeds /
 * eik_set_seeds / eik_get_result (nseeds = 0 means vertex 0; speeds follow
 * eik_set_speeds).  The partition is the built-in one with max_verts_per_block.
 * Every device buffer of the solve (block layout, travel times, flags, lists,
 * control block) lives in one fixed 32 MiB array in the library's device image,
 * which each GPU that loads the library holds until the process exits; the call
 * makes no cudaMalloc / cudaFree and uses no allocating library routine.
 *
 * The first call on a device looks up the array's device address (with that
 * device current) and caches it; make that first call before any stream capture.
 * All calls share the array and it keeps the previous call's contents (the call
 * clears what must start at zero), so calls that overlap on the GPU, on any
 * stream or thread, race: serialise them.  Work runs on `stream` (a cudaStream_t,
 * null = the default stream) with one host round trip per outer iteration (the
 * call synchronises `stream`); the call returns when the result is in out_times.
 * While another stream is being captured, pass a stream created with
 * cudaStreamNonBlocking (the legacy default stream would join the capture's
 * stream and break it) and call from a thread that is not itself capturing (with
 * cudaStreamCaptureModeGlobal or ThreadLocal the capturing thread may not
 * synchronise); `stream` itself must not be capturing.
 *
 * Speeds and metrics are checked as eik_solve checks them (EIK_ERR_ARG for a
 * non-positive or non-finite speed or scalar metric, or a non-finite metric
 * entry).  A device-side wait that gave up returns EIK_ERR_DEVICE, as eik_solve
 * does.  The visit kernels run 512-thread CTAs: eik_solve picks 512 or one
 * thread per slot from a handle's first solves, and this call, which keeps no
 * state between calls, takes 512, the size eik_solve keeps on isotropic meshes.
 *
 * Meshes whose layout and state exceed the array return EIK_ERR_LIMIT (about
 * 200k tets at 64 vertices per block); errbuf (may be null) receives the reason. */
int eik_solve3d_noalloc(const float* xyz, int nv, const int* tets, int nt, const float* speeds, long long nspeeds,
                        const int* seeds, int nseeds, int max_verts_per_block, int max_iterations, float* out_times,
                        void* stream, int* iterations, char* errbuf, int errlen);

/* ---- Batched solves --------------------------------------------------------
 * No counterpart in the reference, which solves one mesh per Eikonal object
 * (src/Eikonal.cu:139-279 solveEikonal).  A batch packs the solves of several
 * handles of the same dimension (each with its own mesh, speeds, seeds, initial
 * values, partition and max_iterations, set through the calls above) into one
 * device-resident layout and runs them in ONE device loop: every outer iteration
 * visits the active blocks of all unfinished instances from a single work list,
 * and each instance stops on its own rule (active list empty, its iteration cap,
 * 2D all-vertex test).  Every instance's result equals, bit for bit, the result
 * of eik_solve on its handle alone.  Launch shape (threads_per_block,
 * direct_launch, fim_sweeps) comes from the first handle's options.
 *
 * The packed layout is rebuilt when a handle's mesh, partition inputs or speeds
 * changed since the last eik_batch_solve; seeds and initial values are re-read on
 * every call.  The handles must outlive the batch. */
typedef struct eik_batch eik_batch;
int eik_batch_create(eik_solver* const* solvers, int n, eik_batch** out);
void eik_batch_destroy(eik_batch* b);
int eik_batch_solve(eik_batch* b);
int eik_batch_num_instances(const eik_batch* b);
/* vertices of instance i (= eik_num_vertices of its handle) */
int eik_batch_num_vertices(const eik_batch* b, int i);
/* outer iterations instance i ran in the last eik_batch_solve */
int eik_batch_num_iterations(const eik_batch* b, int i);
/* result of instance i in its handle's vertex order; nv must equal its vertex count */
int eik_batch_get_result(eik_batch* b, int i, float* out, int nv);
/* all instances' results, instance after instance (n = total vertices) */
int eik_batch_get_results(eik_batch* b, float* out, long long n);
/* the same into device memory (n floats, current device) */
int eik_batch_get_results_device(eik_batch* b, float* out_dev, long long n);
/* whole-batch statistics of the last eik_batch_solve (iterations = longest instance) */
int eik_batch_get_stats(const eik_batch* b, eik_stats* s);
void* eik_batch_stream(const eik_batch* b);
const char* eik_batch_last_error(const eik_batch* b);

/* ---- Request server -----------------------------------------------------------
 * No counterpart in the reference.  A server keeps a pool of meshes resident on
 * the device and solves requests (a pool mesh, seed vertices, a global speed
 * scale) as they arrive, with continuous batching: requests that arrive while
 * others run are admitted between outer iterations as instance slots free up, and
 * all admitted requests advance together in one device loop per dimension (one
 * worker thread and CUDA stream for the 2D pool meshes, one for the 3D ones).
 *
 * Memory: at eik_server_start the pool meshes are laid out as slots, each a
 * resident copy of one mesh's block layout and solver state (device_bytes per
 * slot, reported by eik_server_mesh_info).  A mesh added with slots = 0 gets
 * floor(share / device_bytes) slots (at least 1, at most 64), share being the
 * HBM budget divided evenly among such meshes; eik_server_start fails with
 * EIK_ERR_LIMIT when the slots need more bytes than a nonzero budget allows.  A request is admitted when a
 * slot of its mesh is free (and, with max_inflight > 0, fewer than max_inflight
 * requests run); it waits in arrival order otherwise.
 *
 * Speed scale s: 2D face speeds are multiplied by s; 3D metric entries by
 * fl32(1 / s^2).  Each request's result equals, bit for bit, eik_solve on its
 * mesh handle with those scaled speeds / metric and the request's seeds, and is
 * independent of what else runs.  max_inflight = 1 gives one-at-a-time solving. */
typedef struct eik_server eik_server;
typedef struct {
  long long id;       /* from eik_server_submit */
  int mesh;           /* pool mesh id */
  int iterations;     /* outer iterations the solve ran */
  int status;         /* EIK_OK, or the error that ended the server */
  double submit_s;    /* seconds since the server was created */
  double admit_s;
  double done_s;      /* results on the host */
} eik_completion;
typedef struct {
  long long submitted, completed, queued, running;
  long long device_bytes;  /* slots of both arenas (layouts + state) */
  int slots_2d, slots_3d;
  long long device_loops;  /* launches of the serving loop */
  double busy_s[2];        /* 2D, 3D arena: wall seconds inside device loops */
  long long vertex_updates[2]; /* 2D, 3D arena: vertex updates done */
} eik_server_stats;
int eik_server_create(long long hbm_budget_bytes, int max_inflight, int keep_results, eik_server** out);
/* Adds the handle's mesh, speeds, partition options and max_iterations to the pool
 * (the host layout is built now); slots = 0 sizes it from the budget. */
int eik_server_add_mesh(eik_server* s, eik_solver* h, int slots, int* mesh_id);
int eik_server_mesh_info(const eik_server* s, int mesh_id, int* nv, int* slots, long long* device_bytes);
int eik_server_start(eik_server* s);
int eik_server_submit(eik_server* s, int mesh_id, const int* seeds, int nseeds, float speed_scale, long long* id);
/* Completed requests since the last call (waits up to wait_ms for the first). */
int eik_server_poll(eik_server* s, eik_completion* out, int max, int wait_ms, int* n);
/* Travel times of a completed request (keep_results = 1); releases them. */
int eik_server_result(eik_server* s, long long id, float* out, int nv);
/* Cancels a queued or running request: it completes with status
 * EIK_ERR_CANCELLED (a running one at the end of its current outer iteration) and
 * frees its slot.  EIK_ERR_ARG if the id is unknown or already completed. */
int eik_server_cancel(eik_server* s, long long id);
/* Waits until nothing is queued or running (timeout_ms < 0: no limit). */
int eik_server_drain(eik_server* s, int timeout_ms);
int eik_server_get_stats(eik_server* s, eik_server_stats* out);
void eik_server_destroy(eik_server* s);
const char* eik_server_last_error(const eik_server* s);

/* The CUDA stream (cudaStream_t) the handle's solves and copies run on, or null
 * before the first solve.  Lets callers order their own work or time with events. */
void* eik_stream(const eik_solver* h);

const char* eik_last_error(const eik_solver* h);
/* Library build string (version, CUDA arch). */
const char* eik_version(void);

#ifdef __cplusplus
}
#endif
#endif /* EIKONAL_GB300_H */
