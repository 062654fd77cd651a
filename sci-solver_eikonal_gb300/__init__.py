"""Python binding of the GB300 block-FIM Eikonal solver.

The product is the C ABI in include/eikonal_gb300.h (libeikonal_gb300.so, built
by build.py next to this file).  This module loads that library with ctypes and
offers `Eikonal`, a class with the reference's member names and methods
(SCI-Solver_Eikonal src/Eikonal.h:14-61), so tests and scripts read like the
reference's own tests.  Importing never falls back to a CPU path: a missing or
unloadable library raises ImportError.

The directory name contains a hyphen, so import it with
``importlib.import_module("sci-solver_eikonal_gb300")``.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# EIKONAL_GB300_LIB names another build of the same library (for example one made
# with different compile-time options) to load instead of the in-tree one
LIB_PATH = os.environ.get("EIKONAL_GB300_LIB") or os.path.join(_HERE, "libeikonal_gb300.so")

EIK_OK = 0
PARTITION_RCB = 0    # recursive coordinate bisection (default)
PARTITION_METIS = 1  # METIS k-way on the vertex graph (the reference's partitioner kind)

ERRORS = {1: "EIK_ERR_ARG", 2: "EIK_ERR_STATE", 3: "EIK_ERR_MESH", 4: "EIK_ERR_CUDA",
          5: "EIK_ERR_LIMIT", 6: "EIK_ERR_DEVICE", 7: "EIK_ERR_IO", 8: "EIK_ERR_CANCELLED"}
ONE = 1  # speed type ONE


class EikOptions(ctypes.Structure):
    _fields_ = [
        ("max_blocks", ctypes.c_int), ("max_verts_per_block", ctypes.c_int),
        ("stop_distance", ctypes.c_float), ("is_structured", ctypes.c_int),
        ("speed_type", ctypes.c_int),
        ("square_length", ctypes.c_int), ("square_width", ctypes.c_int), ("square_depth", ctypes.c_int),
        ("square_block_length", ctypes.c_int), ("square_block_width", ctypes.c_int),
        ("square_block_depth", ctypes.c_int),
        ("max_iterations", ctypes.c_int), ("verbose", ctypes.c_int), ("keep_history", ctypes.c_int),
        ("fim_sweeps", ctypes.c_int), ("direct_launch", ctypes.c_int), ("threads_per_block", ctypes.c_int),
        ("precision", ctypes.c_int), ("precision_kappa", ctypes.c_float), ("device_setup", ctypes.c_int),
        ("partitioner", ctypes.c_int), ("telemetry", ctypes.c_int),
    ]


class EikStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int), ("num_blocks", ctypes.c_int),
        ("vertex_updates", ctypes.c_longlong), ("fim_visits", ctypes.c_longlong),
        ("check_visits", ctypes.c_longlong), ("slot_visits", ctypes.c_longlong),
        ("halo_visits", ctypes.c_longlong), ("owned_visits", ctypes.c_longlong),
        ("solve_ms", ctypes.c_float), ("setup_ms", ctypes.c_float),
        ("max_slots_per_block", ctypes.c_int), ("max_local_vertices", ctypes.c_int),
        ("total_slots", ctypes.c_int), ("mean_slots_per_block", ctypes.c_double),
        ("mean_halo_per_block", ctypes.c_double), ("device_error", ctypes.c_int),
        ("fim_kernel_ms", ctypes.c_float), ("check_kernel_ms", ctypes.c_float),
        ("fim_launches", ctypes.c_int), ("check_launches", ctypes.c_int),
        ("fim_slots", ctypes.c_longlong), ("fim_halo", ctypes.c_longlong), ("fim_owned", ctypes.c_longlong),
        ("h2d_bytes", ctypes.c_longlong),
        ("flagged_tets", ctypes.c_longlong), ("residual_max_abs", ctypes.c_double),
        ("residual_max_rel", ctypes.c_double), ("residual_vertices", ctypes.c_longlong),
        ("polish_rounds", ctypes.c_int), ("polish_blocks", ctypes.c_longlong),
        ("residual_below_rel", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = ctypes.c_void_p
_FP = ctypes.POINTER(ctypes.c_float)
_IP = ctypes.POINTER(ctypes.c_int)
_UP = ctypes.POINTER(ctypes.c_ubyte)

# name: (restype, argtypes) — every symbol declared in include/eikonal_gb300.h
class EikCompletion(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("mesh", ctypes.c_int), ("iterations", ctypes.c_int),
                ("status", ctypes.c_int), ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("done_s", ctypes.c_double)]


class EikServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong), ("queued", ctypes.c_longlong),
                ("running", ctypes.c_longlong), ("device_bytes", ctypes.c_longlong), ("slots_2d", ctypes.c_int),
                ("slots_3d", ctypes.c_int), ("device_loops", ctypes.c_longlong),
                ("busy_s", ctypes.c_double * 2), ("vertex_updates", ctypes.c_longlong * 2)]


SIGNATURES = {
    "eik_default_options": (None, [ctypes.POINTER(EikOptions)]),
    "eik_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "eik_destroy": (None, [_P]),
    "eik_set_options": (ctypes.c_int, [_P, ctypes.POINTER(EikOptions)]),
    "eik_get_options": (ctypes.c_int, [_P, ctypes.POINTER(EikOptions)]),
    "eik_set_mesh": (ctypes.c_int, [_P, _FP, ctypes.c_int, _IP, ctypes.c_int]),
    "eik_load_mesh": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "eik_set_speeds": (ctypes.c_int, [_P, _FP, ctypes.c_longlong]),
    "eik_set_initial_values": (ctypes.c_int, [_P, _FP, ctypes.c_int]),
    "eik_set_seeds": (ctypes.c_int, [_P, _IP, ctypes.c_int]),
    "eik_set_partition": (ctypes.c_int, [_P, _IP, ctypes.c_int, ctypes.c_int]),
    "eik_solve": (ctypes.c_int, [_P]),
    "eik_prepare": (ctypes.c_int, [_P]),
    "eik_num_vertices": (ctypes.c_int, [_P]),
    "eik_num_iterations": (ctypes.c_int, [_P]),
    "eik_get_result": (ctypes.c_int, [_P, _FP, ctypes.c_int]),
    "eik_get_result_device": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "eik_get_iteration": (ctypes.c_int, [_P, ctypes.c_int, _FP, ctypes.c_int]),
    "eik_get_partition": (ctypes.c_int, [_P, _IP, ctypes.c_int, _IP]),
    "eik_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(EikStats)]),
    "eik_get_iteration_stats": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "eik_write_vtk": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int]),
    "eik_tri_prep": (ctypes.c_int, [_P, _IP, _IP, _IP, _UP, _IP, _IP]),
    "eik_tri_prep_values": (ctypes.c_int, [_P, _FP, _FP, _FP, _FP]),
    "eik_tet_gram": (ctypes.c_int, [_P, ctypes.c_int, _FP, ctypes.c_longlong]),
    "eik_num_elements": (ctypes.c_int, [_P]),
    "eik_selftest_local_update": (ctypes.c_int, [ctypes.c_int, _FP, _FP, ctypes.c_int]),
    "eik_stream": (_P, [_P]),
    "eik_selftest_wait_timeout": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "eik_solve3d_noalloc": (ctypes.c_int, [_FP, ctypes.c_int, _IP, ctypes.c_int, _FP, ctypes.c_longlong, _IP,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, _FP, _P, _IP, ctypes.c_char_p,
                                           ctypes.c_int]),
    "eik_batch_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(_P)]),
    "eik_batch_destroy": (None, [_P]),
    "eik_batch_solve": (ctypes.c_int, [_P]),
    "eik_batch_num_instances": (ctypes.c_int, [_P]),
    "eik_batch_num_vertices": (ctypes.c_int, [_P, ctypes.c_int]),
    "eik_batch_num_iterations": (ctypes.c_int, [_P, ctypes.c_int]),
    "eik_batch_get_result": (ctypes.c_int, [_P, ctypes.c_int, _FP, ctypes.c_int]),
    "eik_batch_get_results": (ctypes.c_int, [_P, _FP, ctypes.c_longlong]),
    "eik_batch_get_results_device": (ctypes.c_int, [_P, _P, ctypes.c_longlong]),
    "eik_batch_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(EikStats)]),
    "eik_batch_stream": (_P, [_P]),
    "eik_batch_last_error": (ctypes.c_char_p, [_P]),
    "eik_server_create": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "eik_server_add_mesh": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "eik_server_mesh_info": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]),
    "eik_server_start": (ctypes.c_int, [_P]),
    "eik_server_submit": (ctypes.c_int, [_P, ctypes.c_int, _IP, ctypes.c_int, ctypes.c_float,
                                         ctypes.POINTER(ctypes.c_longlong)]),
    "eik_server_poll": (ctypes.c_int, [_P, ctypes.POINTER(EikCompletion), ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int)]),
    "eik_server_result": (ctypes.c_int, [_P, ctypes.c_longlong, _FP, ctypes.c_int]),
    "eik_server_drain": (ctypes.c_int, [_P, ctypes.c_int]),
    "eik_server_cancel": (ctypes.c_int, [_P, ctypes.c_longlong]),
    "eik_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(EikServerStats)]),
    "eik_server_destroy": (None, [_P]),
    "eik_server_last_error": (ctypes.c_char_p, [_P]),
    "eik_last_error": (ctypes.c_char_p, [_P]),
    "eik_version": (ctypes.c_char_p, []),
}


def load_library(path=LIB_PATH):
    """Loads the C ABI library and declares every entry point; raises ImportError."""
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with sci-solver_eikonal_gb300/build.py "
                          "(or __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = load_library()
    return _lib


class EikonalError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _fptr(a):
    return a.ctypes.data_as(_FP)


def _iptr(a):
    return a.ctypes.data_as(_IP)


class Eikonal:
    """The reference's Eikonal class over the C ABI.

    Attribute names follow src/Eikonal.h:43-60 (verbose_, filename_, maxBlocks_,
    maxVertsPerBlock_, ...).  Meshes come from a file (filename_) or from arrays
    (set_mesh); results are numpy float32 arrays.
    """

    _OPT_FIELDS = {
        "maxBlocks_": "max_blocks", "maxVertsPerBlock_": "max_verts_per_block",
        "stopDistance_": "stop_distance", "isStructured_": "is_structured", "speedType_": "speed_type",
        "squareLength_": "square_length", "squareWidth_": "square_width", "squareDepth_": "square_depth",
        "squareBlockLength_": "square_block_length", "squareBlockWidth_": "square_block_width",
        "squareBlockDepth_": "square_block_depth", "maxIterations_": "max_iterations",
        "verbose_": "verbose", "keepHistory_": "keep_history", "fimSweeps_": "fim_sweeps",
        "directLaunch_": "direct_launch", "threadsPerBlock_": "threads_per_block",
        "precisionMode_": "precision", "precisionKappa_": "precision_kappa", "deviceSetup_": "device_setup",
        "partitioner_": "partitioner", "telemetry_": "telemetry",
    }

    def __init__(self, isTriMesh, fname="../src/test/test_data/sphere_74verts.ply", verbose=False):
        self._lib = lib()
        h = _P()
        rc = self._lib.eik_create(1 if isTriMesh else 0, ctypes.byref(h))
        if rc:
            raise EikonalError(rc, "eik_create failed")
        self._h = h
        opts = EikOptions()
        self._lib.eik_default_options(ctypes.byref(opts))
        for py, c in self._OPT_FIELDS.items():
            object.__setattr__(self, py, getattr(opts, c))
        self.verbose_ = bool(verbose)
        self.isTriMesh_ = bool(isTriMesh)
        self.filename_ = fname
        self.userSetInitial_ = False
        self.speedMtxMultipliers_ = []
        self._mesh_loaded = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.eik_destroy(h)
            self._h = None

    # -- helpers ---------------------------------------------------------------
    def _check(self, rc):
        if rc:
            raise EikonalError(rc, self._lib.eik_last_error(self._h).decode())

    def _push_options(self):
        opts = EikOptions()
        for py, c in self._OPT_FIELDS.items():
            setattr(opts, c, type(getattr(opts, c))(getattr(self, py)))
        self._check(self._lib.eik_set_options(self._h, ctypes.byref(opts)))

    def _pull_options(self):
        opts = EikOptions()
        self._check(self._lib.eik_get_options(self._h, ctypes.byref(opts)))
        for py, c in self._OPT_FIELDS.items():
            object.__setattr__(self, py, getattr(opts, c))

    # -- reference API ------------------------------------------------------------
    def set_mesh(self, xyz, elems):
        """initializeMesh from arrays (nv x 3 floats, ne x 3 or ne x 4 ints)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        per = 3 if self.isTriMesh_ else 4
        elems = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1, per)
        self._check(self._lib.eik_set_mesh(self._h, _fptr(xyz), xyz.shape[0], _iptr(elems), elems.shape[0]))
        self._mesh_loaded = True

    def initializeMesh(self):
        """src/Eikonal.cu:99-133: loads filename_ (raises EikonalError EIK_ERR_MESH on failure)."""
        if not self._mesh_loaded:
            self._check(self._lib.eik_load_mesh(self._h, str(self.filename_).encode()))
            self._mesh_loaded = True

    def initializeVertices(self, values):
        v = np.ascontiguousarray(values, dtype=np.float32)
        self._check(self._lib.eik_set_initial_values(self._h, _fptr(v), v.size))
        self.userSetInitial_ = True

    def initSpeedMtxMultipliers(self, values):
        self.speedMtxMultipliers_ = np.ascontiguousarray(values, dtype=np.float32)
        v = self.speedMtxMultipliers_
        self._check(self._lib.eik_set_speeds(self._h, _fptr(v) if v.size else None, v.size))

    def setSeeds(self, seeds):
        s = np.ascontiguousarray(seeds, dtype=np.int32)
        self._check(self._lib.eik_set_seeds(self._h, _iptr(s), s.size))

    def setPartition(self, labels, nblocks=None):
        if labels is None:
            self._check(self._lib.eik_set_partition(self._h, None, 0, 0))
            return
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        nb = int(lab.max()) + 1 if nblocks is None else int(nblocks)
        self._check(self._lib.eik_set_partition(self._h, _iptr(lab), lab.size, nb))

    def solveEikonal(self):
        if not self._mesh_loaded:
            self.initializeMesh()
        self._push_options()
        self._check(self._lib.eik_solve(self._h))
        self._pull_options()

    def prepare(self):
        """Partition and block layout on the host only (no GPU needed)."""
        if not self._mesh_loaded:
            self.initializeMesh()
        self._push_options()
        self._check(self._lib.eik_prepare(self._h))
        self._pull_options()

    def numVertices(self):
        return self._lib.eik_num_vertices(self._h)

    def numIterations(self):
        return self._lib.eik_num_iterations(self._h)

    def getFinalResult(self, out=None):
        """Travel times in original vertex order; `out` (optional): a contiguous
        float32 array of numVertices() entries to fill, e.g. in pinned host memory
        (the copy then runs without staging)."""
        if out is None:
            out = np.empty(self.numVertices(), dtype=np.float32)
        elif out.dtype != np.float32 or out.size != self.numVertices() or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float32 array of numVertices() entries")
        self._check(self._lib.eik_get_result(self._h, _fptr(out), out.size))
        return out

    def getResultDevice(self, dev_ptr):
        self._check(self._lib.eik_get_result_device(self._h, ctypes.c_void_p(dev_ptr), self.numVertices()))

    def getResultAtIteration(self, i):
        out = np.empty(self.numVertices(), dtype=np.float32)
        self._check(self._lib.eik_get_iteration(self._h, int(i), _fptr(out), out.size))
        return out

    def getPartition(self):
        nb = ctypes.c_int()
        lab = np.empty(self.numVertices(), dtype=np.int32)
        self._check(self._lib.eik_get_partition(self._h, _iptr(lab), lab.size, ctypes.byref(nb)))
        return lab, nb.value

    def stream(self):
        """cudaStream_t (as an int) the solves run on, or 0 before the first solve."""
        return self._lib.eik_stream(self._h) or 0

    def stats(self):
        s = EikStats()
        self._check(self._lib.eik_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    ITERATION_STAT_COLUMNS = ("fim_ns", "check_ns", "fim_visits", "fim_slots", "fim_halo", "fim_owned",
                              "check_visits", "check_slots", "check_halo", "check_owned",
                              "fim_start_ns", "check_start_ns",
                              "fused_visits", "fused_slots", "fused_halo", "fused_owned")

    def iterationStats(self):
        """Per outer iteration of the last solve: launch spans of the sweep and check
        kernels (ns), the block visits, slots, halo and owned vertices of the sweeps
        and of the neighbour checks, the two kernels' start times (ns after the first
        sweep start) and the counts of the sweep visits that followed a check in the
        same visit, as an (iterations, 16) int64 array (ITERATION_STAT_COLUMNS)."""
        n = max(self.numIterations(), 0)
        out = np.zeros((n, len(self.ITERATION_STAT_COLUMNS)), dtype=np.int64)
        rc = self._lib.eik_get_iteration_stats(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), n)
        if rc < 0:
            self._check(-rc)
        return out[:rc]

    def writeVTK(self, all_iterations=False, prefix="result"):
        self._check(self._lib.eik_write_vtk(self._h, prefix.encode(), 1 if all_iterations else 0))

    def triPrep(self):
        """Oriented faces, obtuse-corner bits and virtual faces of a 2D mesh."""
        nf, nvf = ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.eik_tri_prep(self._h, ctypes.byref(nf), ctypes.byref(nvf), None, None, None, None))
        faces = np.empty((nf.value, 3), dtype=np.int32)
        obt = np.empty(nf.value, dtype=np.uint8)
        off = np.empty(nf.value + 1, dtype=np.int32)
        vfv = np.empty((max(nvf.value, 1), 3), dtype=np.int32)
        self._check(self._lib.eik_tri_prep(self._h, None, None, _iptr(faces), obt.ctypes.data_as(_UP),
                                           _iptr(off), _iptr(vfv)))
        return faces, obt, off, vfv[:nvf.value]

    def tetGram(self, from_device=False):
        """The six metric edge products per tet (ne, 6) as the block layout holds
        them: the host layout (after prepare) or the device's (after a solve)."""
        out = np.empty((self._lib.eik_num_elements(self._h), 6), dtype=np.float32)
        self._check(self._lib.eik_tet_gram(self._h, 1 if from_device else 0, _fptr(out), out.size))
        return out

    def triPrepValues(self):
        """Edge lengths and inverse speeds of the faces and virtual faces as the 2D
        block layout takes them: (edges (nf, 3), speed_inv (nf,), vf_edges
        (nvirt, 3), vf_speed_inv (nvirt,))."""
        faces, _, _, vfv = self.triPrep()
        nf, nvf = faces.shape[0], vfv.shape[0]
        ed = np.empty((nf, 3), dtype=np.float32)
        si = np.empty(nf, dtype=np.float32)
        ved = np.empty((max(nvf, 1), 3), dtype=np.float32)
        vsi = np.empty(max(nvf, 1), dtype=np.float32)
        self._check(self._lib.eik_tri_prep_values(self._h, _fptr(ed), _fptr(si), _fptr(ved), _fptr(vsi)))
        return ed, si, ved[:nvf], vsi[:nvf]

    def printErrorGraph(self, solution):
        """src/Eikonal.cu:233-279: ASCII plot of the RMS error per iteration."""
        sol = np.asarray(solution, dtype=np.float32)
        rms = [float(np.sqrt(np.mean((sol - self.getResultAtIteration(i)) ** 2)))
               for i in range(self.numIterations())]
        if not rms:
            return
        mx, mn = rms[0], rms[-1]
        hi, lo = -10, 10
        while 10.0 ** hi < mx:
            hi += 1
        while 10.0 ** lo > mn:
            lo -= 1
        print("\n\nlog(Err)|")
        tick = True
        for i in range(hi, lo - 1, -1):
            row = "".join("*" if 10.0 ** i < r < 10.0 ** (i + 1) else " " for r in rms)
            print((f"   10^{i:2d}|" if tick else "        |") + row)
            tick = not tick
        print("--------|------------------------------------------" + f"  Converged to: {rms[-1]:.4f}")
        print("        |1   5    10   15   20   25   30   35")
        print("                   Iteration")


class EikonalBatch:
    """Several Eikonal solves of one dimension in one device loop (eik_batch_*).

    Built from configured Eikonal objects (mesh, speeds, seeds, options); every
    solveEikonal() re-reads their seeds and initial values.  Each instance's result
    equals what solveEikonal() on its object alone gives.
    """

    def __init__(self, solvers):
        self._lib = lib()
        self._solvers = list(solvers)
        if not self._solvers:
            raise ValueError("empty batch")
        for e in self._solvers:
            if not e._mesh_loaded:
                e.initializeMesh()
        arr = (_P * len(self._solvers))(*[e._h for e in self._solvers])
        h = _P()
        rc = self._lib.eik_batch_create(arr, len(self._solvers), ctypes.byref(h))
        if rc:
            raise EikonalError(rc, "eik_batch_create failed: " + self._solvers[0]._lib.eik_last_error(
                self._solvers[0]._h).decode())
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.eik_batch_destroy(h)
            self._h = None

    def __len__(self):
        return len(self._solvers)

    def _check(self, rc):
        if rc:
            raise EikonalError(rc, self._lib.eik_batch_last_error(self._h).decode())

    def solveEikonal(self):
        for e in self._solvers:
            e._push_options()
        self._check(self._lib.eik_batch_solve(self._h))

    def numIterations(self, i):
        return self._lib.eik_batch_num_iterations(self._h, int(i))

    def getFinalResult(self, i):
        out = np.empty(self._lib.eik_batch_num_vertices(self._h, int(i)), dtype=np.float32)
        self._check(self._lib.eik_batch_get_result(self._h, int(i), _fptr(out), out.size))
        return out

    def getFinalResults(self, out=None):
        """All instances' results, split per instance; `out` (optional): a contiguous
        float32 array of the instances' total vertex count to fill (e.g. pinned host
        memory)."""
        sizes = [self._lib.eik_batch_num_vertices(self._h, i) for i in range(len(self))]
        total = int(sum(sizes))
        if out is None:
            out = np.empty(total, dtype=np.float32)
        elif out.dtype != np.float32 or out.size != total or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float32 array of the batch's total vertex count")
        self._check(self._lib.eik_batch_get_results(self._h, _fptr(out), out.size))
        return np.split(out, np.cumsum(sizes)[:-1])

    def getResultsDevice(self, dev_ptr, n):
        self._check(self._lib.eik_batch_get_results_device(self._h, ctypes.c_void_p(dev_ptr), int(n)))

    def stream(self):
        p = self._lib.eik_batch_stream(self._h)
        return p or 0

    def stats(self):
        s = EikStats()
        self._check(self._lib.eik_batch_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()


class EikonalServer:
    """Request server over resident pool meshes (eik_server_*).

    add_mesh() takes configured Eikonal objects (mesh, speeds, block options);
    start() lays the pool out in HBM and starts the device loops; submit() queues a
    request (mesh id, seeds, speed scale) and returns its id; poll() returns
    completions as dicts; result() the travel times of a completed request when
    keep_results is set.  max_inflight=1 solves one request at a time.
    """

    def __init__(self, hbm_budget_bytes=8 << 30, max_inflight=0, keep_results=False):
        self._lib = lib()
        h = _P()
        rc = self._lib.eik_server_create(int(hbm_budget_bytes), int(max_inflight), 1 if keep_results else 0,
                                         ctypes.byref(h))
        if rc:
            raise EikonalError(rc, "eik_server_create failed")
        self._h = h
        self._nv = []

    def __del__(self):
        self.close()

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.eik_server_destroy(h)
            self._h = None

    def _check(self, rc):
        if rc:
            raise EikonalError(rc, self._lib.eik_server_last_error(self._h).decode())

    def add_mesh(self, solver, slots=0):
        if not solver._mesh_loaded:
            solver.initializeMesh()
        solver._push_options()
        mid = ctypes.c_int()
        self._check(self._lib.eik_server_add_mesh(self._h, solver._h, int(slots), ctypes.byref(mid)))
        self._nv.append(solver.numVertices())
        return mid.value

    def mesh_info(self, mesh_id):
        nv, slots, nbytes = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        self._check(self._lib.eik_server_mesh_info(self._h, int(mesh_id), ctypes.byref(nv), ctypes.byref(slots),
                                                   ctypes.byref(nbytes)))
        return {"vertices": nv.value, "slots": slots.value, "device_bytes": nbytes.value}

    def start(self):
        self._check(self._lib.eik_server_start(self._h))

    def submit(self, mesh_id, seeds, speed_scale=1.0):
        sd = np.ascontiguousarray(seeds, dtype=np.int32).ravel()
        rid = ctypes.c_longlong()
        self._check(self._lib.eik_server_submit(self._h, int(mesh_id), _iptr(sd), sd.size, float(speed_scale),
                                                ctypes.byref(rid)))
        return rid.value

    def poll(self, max_items=1024, wait_ms=0):
        buf = (EikCompletion * max_items)()
        n = ctypes.c_int()
        rc = self._lib.eik_server_poll(self._h, buf, max_items, int(wait_ms), ctypes.byref(n))
        out = [{f: getattr(buf[i], f) for f, _ in EikCompletion._fields_} for i in range(n.value)]
        if rc and not out:
            self._check(rc)
        return out

    def result(self, request_id, mesh_id):
        out = np.empty(self._nv[mesh_id], dtype=np.float32)
        self._check(self._lib.eik_server_result(self._h, int(request_id), _fptr(out), out.size))
        return out

    def cancel(self, request_id):
        self._check(self._lib.eik_server_cancel(self._h, int(request_id)))

    def drain(self, timeout_ms=-1):
        self._check(self._lib.eik_server_drain(self._h, int(timeout_ms)))

    def stats(self):
        s = EikServerStats()
        self._check(self._lib.eik_server_get_stats(self._h, ctypes.byref(s)))
        out = {f: getattr(s, f) for f, _ in EikServerStats._fields_}
        out["busy_s"] = list(s.busy_s)
        out["vertex_updates"] = list(s.vertex_updates)
        return out


def selftest_local_update(which, inputs):
    """Evaluates the device local updates element-wise (see eik_selftest_local_update)."""
    nin, nout = {0: (9, 1), 1: (7, 1), 2: (2, 2), 3: (7, 3), 4: (7, 3), 5: (9, 1), 6: (10, 4)}[which]
    a = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, nin)
    out = np.empty((a.shape[0], nout), dtype=np.float32)
    rc = lib().eik_selftest_local_update(which, _fptr(a), _fptr(out), a.shape[0])
    if rc:
        raise EikonalError(rc, "self-test kernel failed")
    return out if nout > 1 else out[:, 0]


def selftest_wait_timeout():
    """Runs the bounded-wait failure self-test: returns (status code, waited ms);
    EIK_ERR_DEVICE (6) means the wait gave up as designed."""
    ms = ctypes.c_double()
    rc = lib().eik_selftest_wait_timeout(ctypes.byref(ms))
    return rc, ms.value


def solve3d_noalloc(xyz, tets, speeds=None, seeds=(0,), max_verts_per_block=64, max_iterations=100, stream=0):
    """The allocation-free 3D solve (eik_solve3d_noalloc): returns (times, iterations)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1, 4)
    sp = None if speeds is None else np.ascontiguousarray(speeds, dtype=np.float32).ravel()
    sd = np.ascontiguousarray(seeds, dtype=np.int32)
    out = np.empty(xyz.shape[0], dtype=np.float32)
    it = ctypes.c_int()
    err = ctypes.create_string_buffer(512)
    rc = lib().eik_solve3d_noalloc(_fptr(xyz), xyz.shape[0], _iptr(tets), tets.shape[0],
                                   _fptr(sp) if sp is not None else None, 0 if sp is None else sp.size,
                                   _iptr(sd), sd.size, int(max_verts_per_block), int(max_iterations), _fptr(out),
                                   ctypes.c_void_p(stream), ctypes.byref(it), err, len(err))
    if rc:
        raise EikonalError(rc, err.value.decode())
    return out, it.value


def version():
    return lib().eik_version().decode()
