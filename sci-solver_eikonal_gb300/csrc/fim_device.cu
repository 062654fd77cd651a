// fim_device.cu — GB300 (sm_103a) kernels and the device-resident outer loop of
// the block-partitioned Fast Iterative Method.
//
// Reference mapping (paths inside SCI-Solver_Eikonal):
//   k_sweep3d         FIMCuda           src/core3d/cuda/CUDA_kernels.cu:383-489   (2 sweeps, apex items)
//   k_check3d         run_check_neghbor CUDA_kernels.cu:493-602                    (1 sweep, flags only)
//   k_visit3d<false>  FIMCuda, slot per thread (blocks too large for the item kernels'
//                     shared memory, and precision mode)
//   k_visit3d<true>   run_check_neghbor, slot per thread (the same cases)
//   k_commit3d        CopyOutBack + host activation, meshFIM3dEikonal.cu:438-488, CUDA_kernels.cu:604-668
//   k_visit2d_slot / k_visit2d <false>  FIMCuda  src/core2d/cuda/CUDA_kernels.cu:36-409  (7 sweeps)
//   k_visit2d_slot / k_visit2d <true>   run_check_neighbor CUDA_kernels.cu:415-799    (1 sweep, writes values)
//   k_activate2d      host activation   src/core2d/cuda/meshFIM2d_eikonal.cu:734-756
//   k_vertex_test2d   all-vertex convergence test, meshFIM2d_eikonal.cu:801-815
//   k_close3d         end of the 3D host loop iteration, meshFIM3dEikonal.cu:411-417
//   run_reduction (both dims) is a __syncthreads_and inside the visit kernels.
//
// Design (GB300-first, not a translation):
//   * One CTA visits one block at a time: its own index first, then blocks from a
//     device counter; grids are sized by occupancy x 152 SMs and stay fixed so the
//     whole iteration is a CUDA-graph body.  A conditional while-node repeats the
//     body (four iterations a pass outside the server) until no block is active:
//     no host round trip per iteration.  Consecutive kernels of the body are joined
//     by programmatic dependencies.
//   * A block's metric terms, corner ids, memos and apex bounds are contiguous in
//     HBM (block-major slots, SoA runs, 16-byte aligned) and arrive in shared memory
//     by bulk copies completing on an mbarrier, while the threads gather owned and
//     halo travel times.
//   * Travel times live once per vertex in HBM (block-contiguous renumbering).
//     Owned vertices keep one shared-memory copy per visit; every slot corner that
//     belongs to another block keeps its own per-slot copy, as the reference's
//     per-slot storage does, and the per-vertex minimum is a shared-memory atomic.
//   * The tet update is explicitly rounded with the reference kernel's fused
//     roundings (local_update.cuh), so its bits do not depend on the kernel around
//     it; the item kernels then run only the apex updates that can change
//     something (all-far, unchanged-input, memo and plane-distance skips, each
//     exact) in 384-thread CTAs, three per SM.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device.hpp"
#include "local_update.cuh"

namespace eikgb {
namespace {

// ---------------------------------------------------------------------------
// device control block
// ---------------------------------------------------------------------------
struct Ctl {
  int iter;       // completed outer iterations
  int max_iters;
  int nact;       // active blocks this iteration
  int nnew;       // newly activated blocks this iteration
  int nnext;      // active list being built for the next iteration
  int work_a, work_c;  // claim counters of the sweep and check visits
  int done_d;     // 2D: CTAs of the all-vertex test finished (the last one closes)
  int error;
  int stop;       // set when the outer loop must end (read by the direct-launch loop)
  int f64_all;    // precision mode's polish: every slot's update in FP64
  int polish;     // precision mode's polish: blocks settle to a few ulps, not EPS
  // 3D checks inside the sweep kernel (DevArgs::fused): blocks a check activated
  // and appended behind the carried-over ones of this iteration's active list, and
  // per iteration parity the check candidates queued by that iteration's commit
  int nadd;
  int ncand[2];
  int idle_iters;  // trailing iterations that swept no block (their checks only)
  int last_idle;   // the last iteration swept no block
  unsigned long long updates, fim_visits, chk_visits, slot_visits, halo_visits, owned_visits;
  unsigned long long fim_slots, fim_halo, fim_owned;  // per-visit inputs of the sweep kernel only
};

enum : int { kErrWait = 1, kErrSmem = 2 };

struct DevArgs {
  const BlockDesc* blocks;
  const float* coef;
  const uint2* lv;
  const int* halo;
  const int* nbr_off;
  const int* nbr;
  const int* vblock;   // renumbered vertex -> block
  int nb, nv;
  float* Ta;           // 3D: committed times; 2D: main buffer
  float* Tb;           // 3D: visit outputs;   2D: out buffer
  const float* Tinit;  // 2D: value of never-refreshed copies
  float* prev;         // 2D: all-vertex test
  int* conv;
  int* stampA;         // 3D: block unconverged this iteration; 2D: block in active list
  int* stampC;         // block already queued for a check this iteration
  unsigned char* visited;
  int* list0;
  int* list1;
  int* list_new;
  Ctl* ctl;
  float* hist;
  int hist_cap;
  // per iteration, kKStride words: [~sweep start, sweep end, ~check start, check
  // end] (globaltimer ns; starts stored complemented so the zeroed buffer and
  // atomicMax give the earliest start), then the sweep kernel's visits, slots, halo and owned
  // vertices, then the same four for the check kernel, then the same four for the
  // sweep visits whose block arrived with a check in the same visit (checks inside
  // the sweep kernel)
  unsigned long long* ktime;
  int ktime_cap;
  int fim_sweeps;
  int max_slots_pad, max_local, max_owned;
  cudaGraphConditionalHandle cond;
  int use_cond;  // 1 inside the CUDA graph, 0 for direct launches
  // independent instances (a single solve is one): per block its instance, per
  // instance finished flag, iterations run, blocks queued for the next iteration,
  // and (2D) a vertex that failed the all-vertex test this iteration
  const int* blk_inst;
  int* inst_done;
  int* inst_iters;
  int* inst_nnext;
  const int* inst_maxit;  // iteration cap of every instance
  // precision mode (3D): per slot the FP64 product index of its tet (-1: FP32)
  const int* slot_f64;
  const double* coef64;
  int* inst_fail;
  int ninst;
  const int* inst_vbeg;  // renumbered vertex range of every instance (ninst + 1)
  const int2* chunks;    // (instance, first vertex) of every 2D vertex-test chunk
  int nchunks;
  // serving: the loop also ends after an iteration in which some instance
  // finished, or once the host raised *pending (requests waiting for admission)
  int serve;
  const volatile int* pending;
  // 3D check visits: per slot the four input times of an earlier check of this
  // solve that lowered no owned vertex by EPS (all ones: none recorded)
  uint4* chk_memo;
  // 3D sweep visits (k_sweep3d): per slot the four input times of the last sweep
  // of the block's latest visit in this solve (all ones: none recorded)
  uint4* fim_memo;
  // 3D: per slot four fp16 lower bounds, one per apex, on every candidate's
  // distance term (plane_skip); null: none
  const uint2* hsb;
  // precision mode: the same bounds for the FP64 updates of flagged tets, one uint2
  // per FP64 product set (k_plane_bounds64); null: none
  const uint2* hs64;
  // precision mode's polish: the bounds of the FP64 updates of slots without FP64
  // products, per slot (k_plane_bounds_u64); null: none
  const uint2* hsu64;
  int sweep_split;  // active blocks from which the large-grid sweep launch runs
  // 3D item path: the neighbour checks of iteration k run inside the sweep kernel
  // of iteration k+1 (they read the same committed times), a block that moves being
  // swept in the same visit.  cand: two lists of nb check candidates (by the parity
  // of the iteration whose commit queued them); per instance the blocks swept this
  // iteration and the candidates queued.  inst_done is then 0 running, 1 finished,
  // 2 at its iteration cap with checks still to run (checked, never swept).
  int fused;
  int* cand;
  int* inst_swept;
  int* inst_ncand;
};

constexpr float kEps3DLe = 0x1.4f8b58p-17f;  // largest float below the double 1e-5
// The change below which a vertex counts as settled: the reference's EPS, or in
// precision mode's polish (every update in FP64) a few units in the last place of
// the time, so that corrections smaller than EPS still reach the neighbour blocks
// Programmatic dependent launch between the kernels of the loop body: wait for the
// grid this one depends on to complete (a no-op without such a dependency, as in
// the kernel-by-kernel loop), then let the next grid begin launching, so its CTAs
// are scheduled while this one runs instead of after it.  Every kernel of the body
// starts with it, before touching global memory.
#ifndef EIK_PDL
#define EIK_PDL 1
#endif
__device__ __forceinline__ void pdl_begin() {
#if EIK_PDL
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

#ifndef EIK_POLISH_SETTLE
#define EIK_POLISH_SETTLE 0x1p-15f
#endif
__device__ __forceinline__ float settle_eps(float T, int polish) {
  return polish ? __fmul_rn(T, EIK_POLISH_SETTLE) : kEps3DLe;
}
constexpr float kEps2D = 1e-5f;
constexpr int kBodyCopies = 4;  // iterations per pass of the graph's loop body
typedef double PrecWide;  // precision mode's wide updates
// whether the driver accepted programmatic edges in a conditional loop body
bool g_pdl_ok = true;
constexpr int kKStride = 16;    // words of per-iteration telemetry (DevArgs::ktime)
#ifndef EIK_SWEEP_ITEMS
#define EIK_SWEEP_ITEMS 1
#endif
// active blocks below which the 3D sweep runs as 1024-thread CTAs (0: never)
#ifndef EIK_SWEEP_SPLIT
#define EIK_SWEEP_SPLIT 0
#endif
#ifndef EIK_SWEEP_MEMO
#define EIK_SWEEP_MEMO 1
#endif
// precision mode's polish: every slot's update in FP64 (1) or only the flagged
// tets' (0), and the relative gap to the FP64 update that re-queues a block
#ifndef EIK_POLISH_F64ALL
#define EIK_POLISH_F64ALL 1
#endif
#ifndef EIK_POLISH_TOL
#define EIK_POLISH_TOL 3e-5
#endif
// item kernels: warps take chunks of 32 items from a shared counter (1; warps that
// drew short updates take more, so fewer wait at the next barrier: sweep kernel 4%
// faster on the 65^3 workload, same bits) or a fixed stride of the CTA's threads (0)
#ifndef EIK_ITEM_STEAL
#define EIK_ITEM_STEAL 1
#endif
#ifndef EIK_CHECK_ITEMS
#define EIK_CHECK_ITEMS 1
#endif
// item kernels: CTA size when the caller gives none, and the register cap that
// lets three such CTAs share an SM's 64 K registers
#ifndef EIK_ITEM_THREADS
#define EIK_ITEM_THREADS 384
#endif
#ifndef EIK_ITEM_MAXNREG
#define EIK_ITEM_MAXNREG 56
#endif
// sweep visits: the block's sweep memos arrive with its bulk copies (1) or are read
// from memory while the first sweep's updates are listed (0)
#ifndef EIK_STAGE_SWEEP_MEMO
#define EIK_STAGE_SWEEP_MEMO 1
#endif
#ifndef EIK_SIZED_AUX
#define EIK_SIZED_AUX 1
#endif
#ifndef EIK_TELEMETRY
#define EIK_TELEMETRY 1
#endif

// 3D item kernels: the neighbour checks of an iteration run inside the next
// iteration's sweep launch (1) or as their own launch, k_check3d (0)
#ifndef EIK_FUSED_CHECK
#define EIK_FUSED_CHECK 1
#endif

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + 1D bulk copy (TMA engine)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (a few seconds at most); false means the copy never completed.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: gives up after about one second of device time (global timer;
// an iteration cap backs it up), so a copy that never lands becomes an error
// flag the host reads instead of a kernel that never ends.
constexpr unsigned long long kWaitLimitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  // the clock is read only once the wait has spun a while: most waits end at once,
  // and a timer read per visit cost the 65^3 solve 1.1%
  unsigned long long t0 = 0;
  for (int i = 0; i < (1 << 26); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i == 16) t0 = global_ns();
    if (i > 16) {
      __nanosleep(256);
      if ((i & 63) == 0 && global_ns() - t0 > kWaitLimitNs) return false;
    }
  }
  return false;
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// launch span of a visit kernel: earliest CTA start, latest CTA end
__device__ __forceinline__ void stamp_start(const DevArgs& a, int iter, int which) {
  if (EIK_TELEMETRY && threadIdx.x == 0 && a.ktime && iter < a.ktime_cap)
    atomicMax(&a.ktime[kKStride * iter + 2 * which], ~global_ns());
}
__device__ __forceinline__ void stamp_end(const DevArgs& a, int iter, int which) {
  if (EIK_TELEMETRY && threadIdx.x == 0 && a.ktime && iter < a.ktime_cap)
    atomicMax(&a.ktime[kKStride * iter + 2 * which + 1], global_ns());
}
// one visit's inputs into this iteration's telemetry (caller: one thread)
__device__ __forceinline__ void count_visit(const DevArgs& a, int iter, int which, int slots, int halo, int owned) {
  if (EIK_TELEMETRY && a.ktime && iter < a.ktime_cap) {
    unsigned long long* w = a.ktime + kKStride * iter + 4 + 4 * which;
    atomicAdd(w, 1ull);
    atomicAdd(w + 1, (unsigned long long)slots);
    atomicAdd(w + 2, (unsigned long long)halo);
    atomicAdd(w + 3, (unsigned long long)owned);
  }
}

// order-preserving float <-> int keys for shared-memory atomicMin
__device__ __forceinline__ int fkey(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float fval(int k) { return __int_as_float(k >= 0 ? k : (k ^ 0x7fffffff)); }

__device__ __forceinline__ int* act_list(const DevArgs& a, int iter) { return (iter & 1) ? a.list1 : a.list0; }
__device__ __forceinline__ int* next_list(const DevArgs& a, int iter) { return (iter & 1) ? a.list0 : a.list1; }

// shared-memory carve shared by the 2D and 3D visit kernels
struct Smem {
  float* coef;          // ncoef runs of max_slots_pad
  uint2* lv;            // max_slots_pad
  float* h0;            // 4 * max_slots_pad per-slot copies (current)
  float* h1;            // next
  unsigned char* m0;    // per-slot changed-corner masks (current)
  unsigned char* m1;
  float* vt;            // max_local: owned values then halo values
  int* vnew;            // max_owned keys
  unsigned char* vchg;  // max_owned
};

// `next` = false (single-sweep check visits): no second set of per-slot copies
// and masks (h1, m1 alias h0, m0 and are never written)
__device__ __forceinline__ Smem carve(unsigned char* sm, const DevArgs& a, int ncoef, bool next = true) {
  Smem s;
  const int np = a.max_slots_pad;
  s.coef = reinterpret_cast<float*>(sm);
  s.lv = reinterpret_cast<uint2*>(s.coef + (size_t)ncoef * np);
  s.h0 = reinterpret_cast<float*>(s.lv + np);
  s.h1 = next ? s.h0 + 4 * (size_t)np : s.h0;
  s.m0 = reinterpret_cast<unsigned char*>(s.h1 + 4 * (size_t)np);
  s.m1 = next ? s.m0 + np : s.m0;
  s.vt = reinterpret_cast<float*>(s.m1 + np);
  s.vnew = reinterpret_cast<int*>(s.vt + a.max_local);
  s.vchg = reinterpret_cast<unsigned char*>(s.vnew + a.max_owned);
  return s;
}

__host__ __device__ inline size_t smem_bytes(int ncoef, int max_slots_pad, int max_local, int max_owned,
                                             bool next = true) {
  const size_t sets = next ? 2 : 1;
  size_t n = (size_t)ncoef * max_slots_pad * 4 + (size_t)max_slots_pad * 8 + sets * 16 * (size_t)max_slots_pad +
             sets * (size_t)max_slots_pad + 4 * (size_t)max_local + 4 * (size_t)max_owned + (size_t)max_owned;
  return (n + 15) & ~(size_t)15;
}

// Issue the bulk copies of block `bd` (coefficients + corner ids; the memos of
// `gmemo`, the check memos by default, into smemo; the apex bounds into shs) and
// gather the owned / halo travel times from `Tsrc`.  Returns false on a copy timeout.
template <class S>
__device__ __forceinline__ bool load_block(const DevArgs& a, const BlockDesc& bd, int ncoef, const S& s,
                                           unsigned long long* bar, unsigned& parity, const float* Tsrc,
                                           uint4* smemo = nullptr, uint2* shs = nullptr,
                                           const uint4* gmemo = nullptr) {
  const int tid = threadIdx.x, NT = blockDim.x;
  if (tid == 0) {
    fence_proxy_async();
    const unsigned bc = 4u * ncoef * bd.nslots_pad, bl = 8u * bd.nslots_pad;
    const unsigned bm = smemo ? 16u * bd.nslots_pad : 0u;
    const unsigned bh = (shs && a.hsb) ? 8u * bd.nslots_pad : 0u;
    if (bc + bl + bm + bh > 0) {
      mbar_expect_tx(bar, bc + bl + bm + bh);
      bulk_g2s(s.coef, a.coef + (size_t)ncoef * bd.slot_begin, bc, bar);
      bulk_g2s(s.lv, a.lv + bd.slot_begin, bl, bar);
      if (bm) bulk_g2s(smemo, (gmemo ? gmemo : a.chk_memo) + bd.slot_begin, bm, bar);
      if (bh) bulk_g2s(shs, a.hsb + bd.slot_begin, bh, bar);
    } else {
      mbar_expect_tx(bar, 0);
    }
  }
  for (int k = tid; k < bd.nowned; k += NT) {
    const float v = Tsrc[bd.vbase + k];
    s.vt[k] = v;
    s.vnew[k] = fkey(v);
  }
  for (int k = tid; k < bd.nhalo; k += NT) s.vt[bd.nowned + k] = Tsrc[a.halo[bd.halo_begin + k]];
  const bool ok = mbar_wait(bar, parity);
  parity ^= 1u;
  return ok;
}

// Every candidate of a tet update is at least m (1 - 2^-22), m the smallest of the
// three input times: the point on the face is a convex combination of the inputs
// whose weights sum to at least 1 - 2^-24 after rounding, formed in at most four
// rounded nonnegative steps, and the candidate adds a square root (>= 0, or NaN,
// which the minimum ignores) to it; the edge candidates are an input plus a square
// root.  So an apex time T <= RN(m (1 - 2^-20)) < m (1 - 2^-21) keeps its value:
// min(T, update) = T, and the update can be skipped without changing any bit.
//
// The same with a lower bound hs on the distance term of every candidate: each
// candidate is a convex combination of the three other times (>= m (1 - 2^-22)) plus
// the rounded square root of a computed metric distance from the apex to a point of
// the opposite face's plane, which k_plane_bounds shows is >= hs^2; the rounded sum
// is then > RN(RN(m + hs) (1 - 2^-20)), and an apex at or below that keeps its time.
// hs = 0 gives the upwind bound above.
__device__ __forceinline__ bool plane_skip(float Tk, float m, float hs) {
  return Tk <= __fmul_rn(__fadd_rn(m, hs), 0x1.ffffep-1f);
}
// fp16 bit patterns (non-negative, normal or zero) to float, exactly
__device__ __forceinline__ float half_bits_value(unsigned h) {
  h &= 0xffffu;
  return (h >> 10) ? __uint_as_float((((h >> 10) + 112u) << 23) | ((h & 1023u) << 13)) : 0.0f;
}
// bound of apex k of slot j (the k-th fp16 of hsb[j])
__device__ __forceinline__ float slot_bound(const uint2* hs, int j, int k) {
  if (!hs) return 0.0f;
  const uint2 w = hs[j];
  return half_bits_value((k < 2 ? w.x : w.y) >> (16 * (k & 1)));
}
// Largest fp16 (non-negative, normal or zero) at or below x >= 0.
__device__ __forceinline__ unsigned half_bits_down(float x) {
  if (!(x > 0.0f)) return 0u;
  const unsigned b = __float_as_uint(x);
  const int e = (int)((b >> 23) & 255u) - 112;
  if (e <= 0) return 0u;
  if (e >= 31) return 0x7bffu;
  return ((unsigned)e << 10) | ((b >> 13) & 1023u);
}
// Lower bound on the metric distance terms of one apex update with inputs
// (XX, XY, XZ, YY, YZ, ZZ) as tet_update_x takes them (ACAC, ACBC, ACCD, BCBC, BCCD,
// CDCD).  Every distance the update computes is the quadratic form
// Q(l1, l2) = XX l1^2 + 2 XY l1 l2 + YY l2^2 + 2 XZ l1 + 2 YZ l2 + ZZ at a point of the
// face's plane (l1, l2 in [0, 1] or a corner), evaluated with at most ~36 u G of
// rounding error (u = 2^-24, G the largest input magnitude: at most three products
// and sums of terms <= 3 G feed each rounding); where the 2x2 block is positive
// definite, Q >= ZZ - (YY XZ^2 - 2 XY XZ YZ + XX YZ^2) / det everywhere on the plane.
// Evaluated in FP64 with directed rounding: the result is <= sqrt(min Q - 64 u G).
__device__ unsigned plane_bound_bits(float XXf, float XYf, float XZf, float YYf, float YZf, float ZZf) {
  const double XX = XXf, XY = XYf, XZ = XZf, YY = YYf, YZ = YZf, ZZ = ZZf;
  if (!(XX > 0.0)) return 0u;
  const double det = __dsub_rd(XX * YY, XY * XY);  // the products are exact
  if (!(det > 0.0)) return 0u;
  const double t = XY * XZ;  // exact
  const double num = __dadd_ru(__dadd_ru(__dmul_ru(YY, XZ * XZ), __dmul_ru(XX, YZ * YZ)), __dmul_ru(-2.0 * t, YZ));
  if (!(num >= 0.0)) return 0u;
  const double G = fmax(fmax(fmax(fabs(XX), fabs(XY)), fmax(fabs(XZ), fabs(YY))), fmax(fabs(YZ), fabs(ZZ)));
  const double h2 = __dsub_rd(__dsub_rd(ZZ, __ddiv_ru(num, det)), 0x1p-18 * G);
  if (!(h2 > 0.0)) return 0u;
  return half_bits_down(__fmul_rd(__double2float_rd(__dsqrt_rd(h2)), 0x1.ffep-1f));
}
// k_plane_bounds: the bounds of every slot of blocks [0, nb) from its stored metric
// products, with the remaining products formed as tet_gram9 forms them and the
// argument order of apex_update.
__global__ void k_plane_bounds(const BlockDesc* blocks, int nb, const float* coef, uint2* hsb) {
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const BlockDesc d = blocks[b];
    const size_t np = (size_t)d.nslots_pad;
    for (int j = threadIdx.x; j < d.nslots_pad; j += blockDim.x) {
      uint2 w = make_uint2(0u, 0u);
      if (j < d.nslots) {
        const float* c = coef + 6 * (size_t)d.slot_begin + j;
        const TetGram g = tet_gram9(c[0], c[np], c[2 * np], c[3 * np], c[4 * np], c[5 * np]);
        const unsigned hA = plane_bound_bits(g.BCBC, -g.BCCD, -g.ACBC, g.CDCD, g.ACCD, g.ACAC);
        const unsigned hB = plane_bound_bits(g.ACAC, -g.ACCD, -g.ACBC, g.CDCD, g.BCCD, g.BCBC);
        const unsigned hC = plane_bound_bits(g.ADAD, g.ADBD, -g.ADCD, g.BDBD, -g.CDBD, g.CDCD);
        const unsigned hD = plane_bound_bits(g.ACAC, g.ACBC, g.ACCD, g.BCBC, g.BCCD, g.CDCD);
        w = make_uint2(hA | (hB << 16), hC | (hD << 16));
      }
      hsb[(size_t)d.slot_begin + j] = w;
    }
  }
}

// (Re)computes the apex distance bounds of blocks [b0, b0 + nb) from their
// coefficients (3D layouts).
// The bound for one FP64 apex update (precision mode: FP64 products, FP64
// arithmetic, FP32 square roots of the distance terms).  h^2 is formed in FP64 with
// round-to-nearest where the 2x2 block is well conditioned (det > 2^-30 XX YY), which
// keeps its relative error below 2^-22 of the quotient, covered by a 2^-20 margin;
// the update's FP64 distance terms carry at most ~40 2^-53 G of rounding, covered by
// 2^-40 G; the FP32 square root costs at most 2^-23 relative, covered by 2^-20.
__device__ unsigned plane_bound_bits64(double XX, double XY, double XZ, double YY, double YZ, double ZZ) {
  if (!(XX > 0.0) || !(YY > 0.0)) return 0u;
  const double det = XX * YY - XY * XY;
  if (!(det > 0x1p-30 * XX * YY)) return 0u;
  const double num = YY * XZ * XZ - 2.0 * XY * XZ * YZ + XX * YZ * YZ;
  if (!(num >= 0.0)) return 0u;
  const double q = num / det;
  const double G = fmax(fmax(fmax(fabs(XX), fabs(XY)), fmax(fabs(XZ), fabs(YY))), fmax(fabs(YZ), fabs(ZZ)));
  const double h2 = ZZ - q - 0x1p-20 * q - 0x1p-40 * G;
  if (!(h2 > 0.0)) return 0u;
  return half_bits_down(__fmul_rd(__double2float_rd(__dsqrt_rd(h2)), 0x1.ffffep-1f));
}
// k_plane_bounds_u64: the bounds of the polish's FP64 updates of every slot of
// blocks [0, nb) from its FP32 products, formed in FP64 as the precision kernel
// forms them for slots without FP64 products.
__global__ void k_plane_bounds_u64(const BlockDesc* blocks, int nb, const float* coef, uint2* out) {
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const BlockDesc d = blocks[b];
    const size_t np = (size_t)d.nslots_pad;
    for (int j = threadIdx.x; j < d.nslots_pad; j += blockDim.x) {
      uint2 w = make_uint2(0u, 0u);
      if (j < d.nslots) {
        const float* c = coef + 6 * (size_t)d.slot_begin + j;
        const double dACBC = c[0], dBCCD = c[np], dACCD = c[2 * np], dADBD = c[3 * np], dACAD = c[4 * np],
                     dBCBD = c[5 * np];
        const double dADBC = dACBC + dBCCD, dACBD = dACBC + dACCD;
        const double dCDBD = dADBD - dACBD, dADCD = dADBD - dADBC;
        const double dCDCD = dADCD - dACCD, dADAD = dADCD + dACAD, dACAC = dACAD - dACCD;
        const double dBDBD = dBCBD + dCDBD, dBCBC = dBCBD - dBCCD;
        const unsigned hA = plane_bound_bits64(dBCBC, -dBCCD, -dACBC, dCDCD, dACCD, dACAC);
        const unsigned hB = plane_bound_bits64(dACAC, -dACCD, -dACBC, dCDCD, dBCCD, dBCBC);
        const unsigned hC = plane_bound_bits64(dADAD, dADBD, -dADCD, dBDBD, -dCDBD, dCDCD);
        const unsigned hD = plane_bound_bits64(dACAC, dACBC, dACCD, dBCBC, dBCCD, dCDCD);
        w = make_uint2(hA | (hB << 16), hC | (hD << 16));
      }
      out[(size_t)d.slot_begin + j] = w;
    }
  }
}

// k_plane_bounds64: the bounds of the FP64 updates of flagged tets [0, n), with the
// remaining products formed in FP64 as the precision kernel forms them.
__global__ void k_plane_bounds64(const double* coef64, int n, uint2* hs64) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
    const double* g = coef64 + 6 * (size_t)f;
    const double dACBC = g[0], dBCCD = g[1], dACCD = g[2], dADBD = g[3], dACAD = g[4], dBCBD = g[5];
    const double dADBC = dACBC + dBCCD, dACBD = dACBC + dACCD;
    const double dCDBD = dADBD - dACBD, dADCD = dADBD - dADBC;
    const double dCDCD = dADCD - dACCD, dADAD = dADCD + dACAD, dACAC = dACAD - dACCD;
    const double dBDBD = dBCBD + dCDBD, dBCBC = dBCBD - dBCCD;
    const unsigned hA = plane_bound_bits64(dBCBC, -dBCCD, -dACBC, dCDCD, dACCD, dACAC);
    const unsigned hB = plane_bound_bits64(dACAC, -dACCD, -dACBC, dCDCD, dBCCD, dBCBC);
    const unsigned hC = plane_bound_bits64(dADAD, dADBD, -dADCD, dBDBD, -dCDBD, dCDCD);
    const unsigned hD = plane_bound_bits64(dACAC, dACBC, dACCD, dBCBC, dBCCD, dCDCD);
    hs64[f] = make_uint2(hA | (hB << 16), hC | (hD << 16));
  }
}

std::string plane_bounds(const BlockDesc* blocks, int b0, int nb, const float* coef, uint2* hsb, cudaStream_t st) {
  if (!hsb || nb <= 0) return "";
  k_plane_bounds<<<std::max(1, std::min(nb, 4096)), 256, 0, st>>>(blocks + b0, nb, coef, hsb);
  const cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? std::string() : std::string("CUDA error: ") + cudaGetErrorString(err);
}

// ===========================================================================
// 3D visit: kCheck = false -> FIMCuda (fim_sweeps sweeps, writes visit outputs);
//           kCheck = true  -> run_check_neghbor (1 sweep, flags only)
// ===========================================================================
template <bool kCheck, bool kPrec = false>
__global__ void __launch_bounds__(1024) k_visit3d(DevArgs a) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_item;
  __shared__ volatile int s_moved;  // check visits: some owned vertex drops by >= EPS
  __shared__ int s_nlist;
  const Smem s0 = carve(sm, a, 6, !kCheck);
  // sweep visits: the slots the last sweep must recompute, packed into a list so
  // they fill few warps (the region behind the carve that check visits use for
  // memos; present whenever the check memo is).  Not in the precision kernel: there
  // the changed loop made the compiler fuse its FP32 path differently from the
  // FP32 kernel's, which it must equal bit for bit.
  int* const slist = (!kCheck && !kPrec && a.chk_memo)
                         ? reinterpret_cast<int*>(sm + smem_bytes(6, a.max_slots_pad, a.max_local, a.max_owned))
                         : nullptr;
  // check memos of the block's slots, staged behind the visit's carve
  uint4* const smemo = (kCheck && a.chk_memo)
                           ? reinterpret_cast<uint4*>(sm + smem_bytes(6, a.max_slots_pad, a.max_local, a.max_owned, false))
                           : nullptr;
  const int tid = threadIdx.x, NT = blockDim.x;
  const Ctl* ctl = a.ctl;
  const int iter = ctl->iter;
  const int stamp = iter + 1;
  const int count = kCheck ? ctl->nnew : ctl->nact;
  const int* list = kCheck ? a.list_new : act_list(a, iter);
  const int f64all = kPrec ? ctl->f64_all : 0;
  const int polish = kPrec ? ctl->polish : 0;
  int* nxt = next_list(a, iter);
  const int nsweeps = kCheck ? 1 : a.fim_sweeps;
  stamp_start(a, iter, kCheck ? 1 : 0);
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  unsigned parity = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(kCheck ? &a.ctl->work_c : &a.ctl->work_a, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= count) break;
    const int b = list[item];
    if (a.inst_done[a.blk_inst[b]]) {  // instance finished: leave its blocks alone
      __syncthreads();
      continue;
    }
    const BlockDesc bd = a.blocks[b];
    Smem s = s0;
    const bool ok = load_block(a, bd, 6, s, &bar, parity, a.Ta, smemo);
    if (!ok) {
      if (tid == 0) atomicOr(&a.ctl->error, kErrWait);
      (void)mbar_wait(&bar, parity ^ 1u);
      __syncthreads();
      continue;
    }
    __syncthreads();
    const int ns = bd.nslots, np = bd.nslots_pad, nown = bd.nowned;
    // per-slot copies of corners owned by other blocks start from the halo values
    for (int j = bd.ninside + tid; j < ns; j += NT) {
      const uint2 l = s.lv[j];
      const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
#pragma unroll
      for (int k = 0; k < 4; ++k) s.h0[4 * j + k] = (id[k] < nown) ? 0.0f : s.vt[id[k]];
      s.m0[j] = 0;
    }
    if (tid == 0) s_moved = 0;
    __syncthreads();
    int myconv = 1;
    for (int sw = 0; sw < nsweeps; ++sw) {
      const bool packed = (slist != nullptr) && sw > 0 && sw == nsweeps - 1;
      const int cnt = packed ? s_nlist : ns;
      for (int i = tid; i < cnt; i += NT) {
        const int j = packed ? slist[i] : i;
        // A check only decides whether the block stays converged; one candidate
        // that lowers an owned vertex by EPS or more decides it (the minimum can
        // only be lower), so the remaining slots are skipped.
        if (kCheck && s_moved) break;
        const uint2 l = s.lv[j];
        const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
        bool own[4];
        float T[4];
        unsigned ch = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          own[k] = id[k] < nown;
          T[k] = own[k] ? s.vt[id[k]] : s.h0[4 * j + k];
          const unsigned c = own[k] ? (unsigned)s.vchg[id[k]] : ((unsigned)s.m0[j] >> k) & 1u;
          ch |= c << k;
        }
        if (sw == 0) {
          ch = 0xfu;
        } else if (sw == nsweeps - 1) {
          // Last sweep: only the owned apexes count (copies of other blocks' corners
          // are dropped after the visit).  An owned apex whose three other corners
          // did not change repeats its previous candidate, which its time already
          // absorbed, so a slot with no such change for any owned apex is skipped.
          unsigned need = 0;
#pragma unroll
          for (int k = 0; k < 4; ++k) need |= (own[k] && (ch & ~(1u << k))) ? 1u : 0u;
          if (!need) ch = 0u;
        }
        // The check's outcome is a function of the slot's four input times (its
        // coefficients are fixed for the solve): inputs an earlier check found
        // lowering no owned vertex by EPS give that outcome again, so the slot is
        // skipped.
        bool memo = false;
        if (kCheck && smemo) {
          const uint4 R = smemo[j];
          memo = R.x == __float_as_uint(T[0]) && R.y == __float_as_uint(T[1]) && R.z == __float_as_uint(T[2]) &&
                 R.w == __float_as_uint(T[3]);
          if (memo) ch = 0u;
        }
        const TetGram gm = tet_gram9(s.coef[0 * np + j], s.coef[1 * np + j], s.coef[2 * np + j],
                                     s.coef[3 * np + j], s.coef[4 * np + j], s.coef[5 * np + j]);
        float nw[4] = {T[0], T[1], T[2], T[3]};
        // The four apex updates with the reference kernel's roundings (explicitly
        // rounded, so the code around them cannot change their bits).  A slot whose
        // four values did not change in the previous sweep would reproduce its
        // previous candidates exactly and is skipped.
        if (ch) {
          const float TA = T[0], TB = T[1], TC = T[2], TD = T[3];
          // flagged tets (and every slot in the polish) take FP64 updates instead
          const int f = kPrec ? a.slot_f64[bd.slot_begin + j] : -1;
          const bool fp64 = kPrec && (f >= 0 || f64all);
          if (!fp64) {
            // apexes at or below the plane-distance bound of their update keep their
            // time (plane_skip)
            const uint2* hs = a.hsb ? a.hsb + bd.slot_begin : nullptr;
            if (!plane_skip(TD, fminf(fminf(TA, TB), TC), slot_bound(hs, j, 3)))
              nw[3] = fminf(TD, apex_update<3>(T, gm));
            if (!plane_skip(TA, fminf(fminf(TB, TD), TC), slot_bound(hs, j, 0)))
              nw[0] = fminf(TA, apex_update<0>(T, gm));
            if (!plane_skip(TB, fminf(fminf(TA, TD), TC), slot_bound(hs, j, 1)))
              nw[1] = fminf(TB, apex_update<1>(T, gm));
            if (!plane_skip(TC, fminf(fminf(TA, TB), TD), slot_bound(hs, j, 2)))
              nw[2] = fminf(TC, apex_update<2>(T, gm));
          }
          if constexpr (kPrec) {
            // flagged tet: the four updates in FP64 from FP64 products
            // (polish: every slot, the unflagged ones from their FP32 products)
            if (fp64) {
              typedef PrecWide W;
              W g[6];
#pragma unroll
              for (int q = 0; q < 6; ++q)
                g[q] = (f >= 0) ? w_make(a.coef64[6 * (size_t)f + q], W{}) : w_make((double)s.coef[q * np + j], W{});
              const W dACBC = g[0], dBCCD = g[1], dACCD = g[2], dADBD = g[3], dACAD = g[4], dBCBD = g[5];
              const W dADBC = dACBC + dBCCD, dACBD = dACBC + dACCD;
              const W dCDBD = dADBD - dACBD, dADCD = dADBD - dADBC;
              const W dCDCD = dADCD - dACCD, dADAD = dADCD + dACAD, dACAC = dACAD - dACCD;
              const W dBDBD = dBCBD + dCDBD, dBCBC = dBCBD - dBCCD;
              const W A = w_make((double)TA, W{}), B = w_make((double)TB, W{}), C = w_make((double)TC, W{}),
                      D = w_make((double)TD, W{});
              // in a check and in a visit's last sweep only the owned apexes count
              // (the copies of other blocks' corners are dropped), so the FP64
              // updates of the others are left out there
              const bool all = !kCheck && sw != nsweeps - 1;
              // an apex at or below the plane-distance bound of its FP64 update (the
              // upwind bound where the tet has none: polish of unflagged tets) keeps
              // its time, which nw already holds
              const uint2* hs = (f >= 0) ? (a.hs64 ? a.hs64 + f : nullptr)
                                         : (a.hsu64 ? a.hsu64 + bd.slot_begin + j : nullptr);
              if ((all || own[3]) && !plane_skip(TD, fminf(fminf(TA, TB), TC), slot_bound(hs, 0, 3)))
                nw[3] = fminf(TD, w_float(tet_update_wide<W>(A, B, C, dACAC, dACBC, dACCD, dBCBC, dBCCD, dCDCD)));
              if ((all || own[0]) && !plane_skip(TA, fminf(fminf(TB, TD), TC), slot_bound(hs, 0, 0)))
                nw[0] = fminf(TA, w_float(tet_update_wide<W>(B, D, C, dBCBC, -dBCCD, -dACBC, dCDCD, dACCD, dACAC)));
              if ((all || own[1]) && !plane_skip(TB, fminf(fminf(TA, TD), TC), slot_bound(hs, 0, 1)))
                nw[1] = fminf(TB, w_float(tet_update_wide<W>(A, D, C, dACAC, -dACCD, -dACBC, dCDCD, dBCCD, dBCBC)));
              if ((all || own[2]) && !plane_skip(TC, fminf(fminf(TA, TB), TD), slot_bound(hs, 0, 2)))
                nw[2] = fminf(TC, w_float(tet_update_wide<W>(A, B, D, dADAD, dADBD, -dADCD, dBDBD, -dCDBD, dCDCD)));
            }
          }
        }
        if (kCheck) {
          bool moved = false;
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (own[k] && !((T[k] - nw[k]) <= settle_eps(T[k], polish))) moved = true;  // (double)(old - c) >= 1e-5
          if (moved)
            s_moved = 1;
          else if (smemo && !memo)
            a.chk_memo[bd.slot_begin + j] = make_uint4(__float_as_uint(T[0]), __float_as_uint(T[1]),
                                                       __float_as_uint(T[2]), __float_as_uint(T[3]));
        } else {
          unsigned m = 0;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (own[k]) {
              if (nw[k] < T[k]) atomicMin(&s.vnew[id[k]], fkey(nw[k]));
            } else {
              s.h1[4 * j + k] = nw[k];
              m |= (nw[k] != T[k] ? 1u : 0u) << k;
            }
          }
          s.m1[j] = (unsigned char)m;
        }
      }
      __syncthreads();
      if (kCheck) {
        myconv = s_moved ? 0 : 1;
        break;
      }
      const bool last = (sw == nsweeps - 1);
      for (int k = tid; k < nown; k += NT) {
        const float nv = fval(s.vnew[k]);
        const float ov = s.vt[k];
        if (last) {
          float res = ov - nv;
          if (!kCheck && res < 0.0f) res = -res;
          myconv &= (res <= settle_eps(ov, polish)) ? 1 : 0;
        }
        s.vchg[k] = (nv != ov) ? 1 : 0;
        s.vt[k] = nv;
      }
      float* th = s.h0; s.h0 = s.h1; s.h1 = th;
      unsigned char* tm = s.m0; s.m0 = s.m1; s.m1 = tm;
      __syncthreads();
      // list the slots with an owned apex whose other corners changed (the rest
      // repeat absorbed candidates in the last sweep, see the sweep loop)
      if (slist && sw + 1 == nsweeps - 1) {
        if (tid == 0) s_nlist = 0;
        __syncthreads();
        for (int j = tid; j < ns; j += NT) {
          const uint2 l = s.lv[j];
          const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
          unsigned ch = 0, om = 0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const bool o = id[q] < nown;
            const unsigned c = o ? (unsigned)s.vchg[id[q]] : ((unsigned)s.m0[j] >> q) & 1u;
            ch |= c << q;
            om |= (o ? 1u : 0u) << q;
          }
          unsigned need = 0;
#pragma unroll
          for (int q = 0; q < 4; ++q) need |= (((om >> q) & 1u) && (ch & ~(1u << q))) ? 1u : 0u;
          const unsigned am = __activemask();
          const unsigned bm = __ballot_sync(am, need != 0);
          const int lane = tid & 31, leader = __ffs(am) - 1;
          int base = 0;
          if (lane == leader && bm) base = atomicAdd(&s_nlist, __popc(bm));
          base = __shfl_sync(am, base, leader);
          if (need) slist[base + __popc(bm & ((1u << lane) - 1u))] = j;
        }
        __syncthreads();
      }
    }
    const int allc = __syncthreads_and(myconv);
    if (!kCheck)
      for (int k = tid; k < nown; k += NT) a.Tb[bd.vbase + k] = s.vt[k];
    if (tid == 0) {
      if (!kCheck) {
        a.conv[b] = allc;
        if (!allc) a.stampA[b] = stamp;
        atomicAdd(&a.ctl->fim_visits, 1ull);
      } else {
        if (!allc) {
          nxt[atomicAdd(&a.ctl->nnext, 1)] = b;
          atomicAdd(&a.inst_nnext[a.blk_inst[b]], 1);
        }
        atomicAdd(&a.ctl->chk_visits, 1ull);
      }
      atomicAdd(&a.ctl->updates, (unsigned long long)nown * nsweeps);
      count_visit(a, iter, kCheck ? 1 : 0, ns, bd.nhalo, nown);
      atomicAdd(&a.ctl->slot_visits, (unsigned long long)ns);
      atomicAdd(&a.ctl->halo_visits, (unsigned long long)bd.nhalo);
      atomicAdd(&a.ctl->owned_visits, (unsigned long long)nown);
      if (!kCheck) {
        atomicAdd(&a.ctl->fim_slots, (unsigned long long)ns);
        atomicAdd(&a.ctl->fim_halo, (unsigned long long)bd.nhalo);
        atomicAdd(&a.ctl->fim_owned, (unsigned long long)nown);
      }
    }
    __syncthreads();
  }
  stamp_end(a, iter, kCheck ? 1 : 0);
}


// ===========================================================================
// 3D sweep visit by apex items (FIMCuda, fim_sweeps sweeps).
//
// Each sweep first lists the apex updates that can change something, then runs
// them spread evenly over the CTA's threads:
//   * an apex whose three other corners are all at LARGENUM is skipped: its update
//     returns LARGENUM and min(T, LARGENUM) = T;
//   * after the first sweep, an apex none of whose three other corners changed in
//     the previous sweep is skipped: its update would repeat a candidate that the
//     previous sweep already folded into its value (the vertex minimum for an owned
//     apex, the slot's copy for a corner owned elsewhere);
//   * in the last sweep only owned apexes run (the per-slot copies of other
//     blocks' corners are dropped after the visit);
//   * an apex already at or below (1 - 2^-20) x (the smallest of its three other
//     corners + a lower bound of its distance terms) is skipped (plane_skip): no
//     candidate of its update can be lower.
// The four apex updates of a slot round differently (the reference's inlined
// copies), so the lists are kept per apex and warps run one apex kind at a time.
// Every update that runs is the reference's, bit for bit (apex_update); skipped
// updates are exactly those whose result cannot differ from the value kept, so the
// visit's outputs equal the reference's FIMCuda visit.
// ===========================================================================
struct SmemItems {
  float* coef;          // 6 runs of max_slots_pad
  uint2* lv;            // max_slots_pad
  float* h0;            // 4 per slot: copies of corners owned elsewhere (current)
  float* h1;            // the previous sweep's copies until this sweep's list is built
  float* vt;            // max_local: owned values then halo values
  int* vnew;            // max_owned keys
  unsigned char* vchg;  // max_owned
  unsigned short* items;  // 4 lists of max_slots_pad slot indices (one per apex)
  uint2* hs;              // max_slots_pad: the apexes' distance bounds (plane_skip)
};

__host__ __device__ inline size_t items_offsets(int np, int max_local, int max_owned, size_t off[9]) {
  size_t o = 0;
  auto take = [&](size_t bytes, size_t align) {
    o = (o + align - 1) & ~(align - 1);
    const size_t at = o;
    o += bytes;
    return at;
  };
  off[0] = take(24 * (size_t)np, 16);       // coef
  off[1] = take(8 * (size_t)np, 16);        // lv
  off[2] = take(16 * (size_t)np, 16);       // h0
  off[3] = take(16 * (size_t)np, 16);       // h1
  off[4] = take(4 * (size_t)max_local, 4);  // vt
  off[5] = take(4 * (size_t)max_owned, 4);  // vnew
  off[6] = take((size_t)max_owned, 1);      // vchg
  off[7] = take(8 * (size_t)np, 2);         // items
  off[8] = take(8 * (size_t)np, 16);        // hs
  return (o + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t smem_bytes_items(int np, int max_local, int max_owned) {
  size_t off[9];
  return items_offsets(np, max_local, max_owned, off);
}
__device__ __forceinline__ SmemItems carve_items(unsigned char* sm, const DevArgs& a) {
  size_t off[9];
  items_offsets(a.max_slots_pad, a.max_local, a.max_owned, off);
  SmemItems s;
  s.coef = reinterpret_cast<float*>(sm + off[0]);
  s.lv = reinterpret_cast<uint2*>(sm + off[1]);
  s.h0 = reinterpret_cast<float*>(sm + off[2]);
  s.h1 = reinterpret_cast<float*>(sm + off[3]);
  s.vt = reinterpret_cast<float*>(sm + off[4]);
  s.vnew = reinterpret_cast<int*>(sm + off[5]);
  s.vchg = sm + off[6];
  s.items = reinterpret_cast<unsigned short*>(sm + off[7]);
  s.hs = reinterpret_cast<uint2*>(sm + off[8]);
  return s;
}

// One check visit over a loaded block (run_check_neghbor, CUDA_kernels.cu:493-602):
// lists the owned apex updates that the check memo (smemo, staged with the block)
// and the plane bound (shs) do not settle, runs them until one lowers its vertex
// by more than EPS, and when none does records every slot's input times as
// settled.  Returns whether the block moved.  Called by all threads of the CTA.
template <class S>
__device__ __forceinline__ bool check_pass(const DevArgs& a, const BlockDesc& bd, const S& s, uint4* smemo,
                                           const uint2* shs, int* s_cnt, volatile int* s_moved) {
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31;
  const int np = a.max_slots_pad;
  if (tid == 0) *s_moved = 0;
  if (tid < 5) s_cnt[tid] = 0;
  __syncthreads();
  const int ns = bd.nslots, nown = bd.nowned, pitch = bd.nslots_pad;
  for (int j0 = 0; j0 < ns; j0 += NT) {
    const int j = j0 + tid;
    unsigned need = 0;
    if (j < ns) {
      const uint2 l = s.lv[j];
      const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
      float T[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) T[q] = s.vt[id[q]];
      bool memo = false;
      if (smemo) {
        const uint4 R = smemo[j];
        memo = R.x == __float_as_uint(T[0]) && R.y == __float_as_uint(T[1]) && R.z == __float_as_uint(T[2]) &&
               R.w == __float_as_uint(T[3]);
      }
      if (!memo) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float m = fminf(fminf(T[(k + 1) & 3], T[(k + 2) & 3]), T[(k + 3) & 3]);
          const bool run = id[k] < nown && m < kLarge3DDev && !plane_skip(T[k], m, slot_bound(shs, j, k));
          need |= (run ? 1u : 0u) << k;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const unsigned bal = __ballot_sync(0xffffffffu, (need >> k) & 1u);
      if (bal) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&s_cnt[k], __popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((need >> k) & 1u) s.items[k * np + base + __popc(bal & ((1u << lane) - 1u))] = (unsigned short)j;
      }
    }
  }
  __syncthreads();
  const int c0 = s_cnt[0], c01 = c0 + s_cnt[1], c012 = c01 + s_cnt[2], total = c012 + s_cnt[3];
#if EIK_ITEM_STEAL
  for (;;) {
    int i0 = 0;
    if (lane == 0) i0 = *s_moved ? total : atomicAdd(&s_cnt[4], 32);
    i0 = __shfl_sync(0xffffffffu, i0, 0);
    if (i0 >= total) break;
    const int i = i0 + lane;
    if (i >= total) continue;
#else
  for (int i = tid; i < total; i += NT) {
    if (*s_moved) break;
#endif
    const int k = (i < c0) ? 0 : (i < c01) ? 1 : (i < c012) ? 2 : 3;
    const int r = i - ((k == 0) ? 0 : (k == 1) ? c0 : (k == 2) ? c01 : c012);
    const int j = s.items[k * np + r];
    const uint2 l = s.lv[j];
    const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
    float T[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) T[q] = s.vt[id[q]];
    const TetGram gm = tet_gram9(s.coef[0 * pitch + j], s.coef[1 * pitch + j], s.coef[2 * pitch + j],
                                 s.coef[3 * pitch + j], s.coef[4 * pitch + j], s.coef[5 * pitch + j]);
    float u;
    switch (k) {
      case 0: u = apex_update<0>(T, gm); break;
      case 1: u = apex_update<1>(T, gm); break;
      case 2: u = apex_update<2>(T, gm); break;
      default: u = apex_update<3>(T, gm); break;
    }
    const float Tk = (k == 0) ? T[0] : (k == 1) ? T[1] : (k == 2) ? T[2] : T[3];
    // (double)(old - candidate) >= 1e-5 in the reference
    if (!((Tk - fminf(Tk, u)) <= kEps3DLe)) *s_moved = 1;
  }
  __syncthreads();
  const int allc = *s_moved ? 0 : 1;
  if (allc && smemo)
    for (int j = tid; j < ns; j += NT) {
      const uint2 l = s.lv[j];
      const uint4 R = smemo[j];
      const uint4 W = make_uint4(__float_as_uint(s.vt[l.x & 0xffffu]), __float_as_uint(s.vt[l.x >> 16]),
                                 __float_as_uint(s.vt[l.y & 0xffffu]), __float_as_uint(s.vt[l.y >> 16]));
      if (R.x != W.x || R.y != W.y || R.z != W.z || R.w != W.w) a.chk_memo[bd.slot_begin + j] = W;
    }
  return allc == 0;
}

// at most 56 registers: three CTAs of 384 threads fit one SM's register file
// role: 0 runs every iteration; where the loop body holds two sweep launches of
// different CTA sizes, 1 runs only iterations with at least a.sweep_split active
// blocks and 2 only the others (few blocks: a visit's latency, which more threads
// per block shorten, sets the launch's time).
// With a.fused, the CTAs also claim the check candidates queued by the previous
// iteration's commit (items nact.. of the claim range): a candidate's check runs
// on the staged block, and a block that moves is appended to this iteration's
// active list and swept in the same visit.
__global__ void __maxnreg__(EIK_ITEM_MAXNREG) k_sweep3d(DevArgs a, int role) {
  pdl_begin();
  if (role != 0 && ((a.ctl->nact >= a.sweep_split) != (role == 1))) return;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_item;
  __shared__ int s_cnt[5];  // items per apex kind, then the next unclaimed item
  __shared__ volatile int s_moved;
  const SmemItems s0 = carve_items(sm, a);
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31;
  const int np = a.max_slots_pad;
  Ctl* ctl = a.ctl;
  const int iter = ctl->iter;
  const int stamp = iter + 1;
  const int nact = ctl->nact;
  const int ncand = a.fused ? ctl->ncand[(iter + 1) & 1] : 0;
  const int* cand = a.fused ? a.cand + (size_t)((iter + 1) & 1) * a.nb : nullptr;
  const int count = nact + ncand;
  int* list = act_list(a, iter);
  const int nsweeps = a.fim_sweeps;
  stamp_start(a, iter, 0);
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  unsigned parity = 0;
  // the first block of a CTA is its own index; later ones come from the counter
  // (a CTA without a first block exits without touching it)
  int first_item = blockIdx.x;
  // a single instance's finished flag, read once (it changes only between launches):
  // spares every visit the instance lookup
  const int done1 = (a.ninst == 1) ? a.inst_done[0] : -1;
  for (;;) {
    int item = first_item;
    if (item < 0) {
      if (tid == 0) s_item = (int)gridDim.x + atomicAdd(&a.ctl->work_a, 1);
      __syncthreads();
      item = s_item;
    }
    first_item = -1;
    if (item >= count) break;
    const bool chk = item >= nact;  // a check candidate
    const int b = chk ? cand[item - nact] : list[item];
    const BlockDesc bd = a.blocks[b];
    // instance finished: leave its blocks alone; at its cap: its checks only
    const int ist = done1 >= 0 ? done1 : a.inst_done[a.blk_inst[b]];
    if (ist == 1 || (ist != 0 && !chk)) {
      __syncthreads();
      continue;
    }
    SmemItems s = s0;
    // a candidate's check memos, or an active block's sweep memos, arrive in the
    // per-slot copy buffer h0, which the first sweep neither reads nor writes
    uint4* const smemo = (chk ? a.chk_memo != nullptr : (EIK_STAGE_SWEEP_MEMO && a.fim_memo != nullptr))
                             ? reinterpret_cast<uint4*>(s.h0)
                             : nullptr;
    if (!load_block(a, bd, 6, s, &bar, parity, a.Ta, smemo, a.hsb ? s.hs : nullptr, chk ? nullptr : a.fim_memo)) {
      if (tid == 0) atomicOr(&a.ctl->error, kErrWait);
      (void)mbar_wait(&bar, parity ^ 1u);
      __syncthreads();
      continue;
    }
    __syncthreads();
    const int ns = bd.nslots, nown = bd.nowned, pitch = bd.nslots_pad;
    if (chk) {
      const bool moved = check_pass(a, bd, s, smemo, a.hsb ? s.hs : nullptr, s_cnt, &s_moved);
      if (tid == 0) {  // the previous iteration's check (run_check_neghbor)
        atomicAdd(&a.ctl->chk_visits, 1ull);
        atomicAdd(&a.ctl->updates, (unsigned long long)nown);
        count_visit(a, iter - 1, 1, ns, bd.nhalo, nown);
        atomicAdd(&a.ctl->slot_visits, (unsigned long long)ns);
        atomicAdd(&a.ctl->halo_visits, (unsigned long long)bd.nhalo);
        atomicAdd(&a.ctl->owned_visits, (unsigned long long)nown);
        if (moved && ist == 0) list[nact + atomicAdd(&ctl->nadd, 1)] = b;
      }
      if (!moved || ist != 0) {
        __syncthreads();
        continue;
      }
    }
    const bool fusedv = chk;  // the block arrived with this visit's check
    // per-slot copies of corners owned by other blocks start from the halo values,
    // which stay in vt for the whole visit: the first sweep reads them there, and
    // the second compares its copies with them
    int myconv = 1;
    for (int sw = 0; sw < nsweeps; ++sw) {
      const bool first = (sw == 0), last = (sw == nsweeps - 1);
      if (tid < 5) s_cnt[tid] = 0;
      __syncthreads();
      // ---- list the apex updates this sweep must run ----
      for (int j0 = 0; j0 < ns; j0 += NT) {
        const int j = j0 + tid;
        unsigned need = 0;
        if (j < ns) {
          const uint2 l = s.lv[j];
          const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
          unsigned big = 0, chg = 0, own = 0;
          float Tq[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const bool o = id[q] < nown;
            const float T = (o || first) ? s.vt[id[q]] : s.h0[4 * j + q];
            Tq[q] = T;
            big |= (T >= kLarge3DDev ? 1u : 0u) << q;
            // a copy changed in the previous sweep when it differs from that sweep's
            // input: the halo value after the first sweep, else still held in h1 (the
            // buffers swap after every sweep)
            chg |= (first ? 1u
                          : (o ? (unsigned)s.vchg[id[q]]
                               : (T != (sw == 1 ? s.vt[id[q]] : s.h1[4 * j + q]) ? 1u : 0u)))
                   << q;
            own |= (o ? 1u : 0u) << q;
            if (!o && !last) s.h1[4 * j + q] = T;  // kept unless its update below changes it
          }
          // sweep memo: an owned apex whose three other inputs equal (as bits) those
          // of the last sweep of the block's previous visit repeats an update whose
          // result its time has already absorbed (times only decrease)
          unsigned same = 0;
          if (first && a.fim_memo) {
            // staged with the block, or (a block its check activated) from memory
            const uint4 mm = (smemo && !chk) ? smemo[j] : a.fim_memo[bd.slot_begin + j];
            same = (__float_as_uint(Tq[0]) == mm.x ? 1u : 0u) | (__float_as_uint(Tq[1]) == mm.y ? 2u : 0u) |
                   (__float_as_uint(Tq[2]) == mm.z ? 4u : 0u) | (__float_as_uint(Tq[3]) == mm.w ? 8u : 0u);
          }
          if (last && a.fim_memo)
            a.fim_memo[bd.slot_begin + j] = make_uint4(__float_as_uint(Tq[0]), __float_as_uint(Tq[1]),
                                                       __float_as_uint(Tq[2]), __float_as_uint(Tq[3]));
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const unsigned others = 0xfu & ~(1u << k);
            const float m = fminf(fminf(Tq[(k + 1) & 3], Tq[(k + 2) & 3]), Tq[(k + 3) & 3]);
            const bool ownk = ((own >> k) & 1u) != 0;
            const bool run = ((big & others) != others) && (chg & others) && (!last || ownk) &&
                             !(ownk && (same & others) == others) &&
                             !plane_skip(Tq[k], m, slot_bound(a.hsb ? s.hs : nullptr, j, k));
            need |= (run ? 1u : 0u) << k;
          }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const unsigned bal = __ballot_sync(0xffffffffu, (need >> k) & 1u);
          if (bal) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&s_cnt[k], __popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if ((need >> k) & 1u) s.items[k * np + base + __popc(bal & ((1u << lane) - 1u))] = (unsigned short)j;
          }
        }
      }
      __syncthreads();
      // ---- run them ----
      const int c0 = s_cnt[0], c01 = c0 + s_cnt[1], c012 = c01 + s_cnt[2], total = c012 + s_cnt[3];
#if EIK_ITEM_STEAL
      for (;;) {
        int i0 = 0;
        if (lane == 0) i0 = atomicAdd(&s_cnt[4], 32);
        i0 = __shfl_sync(0xffffffffu, i0, 0);
        if (i0 >= total) break;
        const int i = i0 + lane;
        if (i >= total) continue;
#else
      for (int i = tid; i < total; i += NT) {
#endif
        const int k = (i < c0) ? 0 : (i < c01) ? 1 : (i < c012) ? 2 : 3;
        const int r = i - ((k == 0) ? 0 : (k == 1) ? c0 : (k == 2) ? c01 : c012);
        const int j = s.items[k * np + r];
        const uint2 l = s.lv[j];
        const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
        float T[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) T[q] = (id[q] < nown || sw == 0) ? s.vt[id[q]] : s.h0[4 * j + q];
        const TetGram gm = tet_gram9(s.coef[0 * pitch + j], s.coef[1 * pitch + j], s.coef[2 * pitch + j],
                                     s.coef[3 * pitch + j], s.coef[4 * pitch + j], s.coef[5 * pitch + j]);
        float u;
        switch (k) {
          case 0: u = apex_update<0>(T, gm); break;
          case 1: u = apex_update<1>(T, gm); break;
          case 2: u = apex_update<2>(T, gm); break;
          default: u = apex_update<3>(T, gm); break;
        }
        // T[k], id[k] by selects: a runtime index would put the arrays in local memory
        const float Tk = (k == 0) ? T[0] : (k == 1) ? T[1] : (k == 2) ? T[2] : T[3];
        const int idk = (k == 0) ? id[0] : (k == 1) ? id[1] : (k == 2) ? id[2] : id[3];
        const float nw = fminf(Tk, u);
        if (idk < nown) {
          if (nw < Tk) atomicMin(&s.vnew[idk], fkey(nw));
        } else if (!last) {
          s.h1[4 * j + k] = nw;
        }
      }
      __syncthreads();
      for (int k = tid; k < nown; k += NT) {
        const float nv = fval(s.vnew[k]);
        const float ov = s.vt[k];
        if (last) {
          float res = ov - nv;
          if (res < 0.0f) res = -res;
          myconv &= (res <= kEps3DLe) ? 1 : 0;
        }
        s.vchg[k] = (nv != ov) ? 1 : 0;
        s.vt[k] = nv;
      }
      float* th = s.h0; s.h0 = s.h1; s.h1 = th;
    }
    const int allc = __syncthreads_and(myconv);
    for (int k = tid; k < nown; k += NT) a.Tb[bd.vbase + k] = s.vt[k];
    if (tid == 0) {
      a.conv[b] = allc;
      if (!allc) a.stampA[b] = stamp;
      if (a.fused) atomicAdd(&a.inst_swept[a.blk_inst[b]], 1);
      atomicAdd(&a.ctl->fim_visits, 1ull);
      atomicAdd(&a.ctl->updates, (unsigned long long)nown * nsweeps);
      count_visit(a, iter, 0, ns, bd.nhalo, nown);
      if (fusedv) {  // streamed once, with the check
        count_visit(a, iter, 2, ns, bd.nhalo, nown);
      } else {
        atomicAdd(&a.ctl->slot_visits, (unsigned long long)ns);
        atomicAdd(&a.ctl->halo_visits, (unsigned long long)bd.nhalo);
        atomicAdd(&a.ctl->owned_visits, (unsigned long long)nown);
      }
      atomicAdd(&a.ctl->fim_slots, (unsigned long long)ns);
      atomicAdd(&a.ctl->fim_halo, (unsigned long long)bd.nhalo);
      atomicAdd(&a.ctl->fim_owned, (unsigned long long)nown);
    }
    __syncthreads();
  }
  stamp_end(a, iter, 0);
}

// ===========================================================================
// 3D neighbour check by apex items (run_check_neghbor, one sweep, flags only).
//
// Only owned apexes decide a check; an item runs the update of one owned apex of
// one slot, skipped where the sweep kernel skips it (three inputs at LARGENUM, or
// the apex already upwind of its corners) and for slots whose four input times an
// earlier check of this solve found settled (check memo).  The first candidate that
// lowers an owned vertex by EPS or more decides the block (later ones cannot change
// the flag) and stops the remaining items.  When the block stays converged, every
// slot that ran records its input times as settled.
// ===========================================================================
struct SmemCheck {
  float* coef;            // 6 runs of max_slots_pad
  uint2* lv;              // max_slots_pad
  uint4* memo;            // max_slots_pad check memos (staged with the block)
  float* vt;              // max_local
  int* vnew;              // max_owned (filled by load_block, unused here)
  unsigned short* items;  // 4 lists of max_slots_pad
  uint2* hs;              // max_slots_pad: the apexes' distance bounds (plane_skip)
};
__host__ __device__ inline size_t check_offsets(int np, int max_local, int max_owned, size_t off[7]) {
  size_t o = 0;
  auto take = [&](size_t bytes, size_t align) {
    o = (o + align - 1) & ~(align - 1);
    const size_t at = o;
    o += bytes;
    return at;
  };
  off[0] = take(24 * (size_t)np, 16);
  off[1] = take(8 * (size_t)np, 16);
  off[2] = take(16 * (size_t)np, 16);
  off[3] = take(4 * (size_t)max_local, 4);
  off[4] = take(4 * (size_t)max_owned, 4);
  off[5] = take(8 * (size_t)np, 2);
  off[6] = take(8 * (size_t)np, 16);
  return (o + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t smem_bytes_check(int np, int max_local, int max_owned) {
  size_t off[7];
  return check_offsets(np, max_local, max_owned, off);
}

__global__ void __maxnreg__(EIK_ITEM_MAXNREG) k_check3d(DevArgs a) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_item;
  __shared__ volatile int s_moved;
  __shared__ int s_cnt[5];  // items per apex kind, then the next unclaimed item
  size_t off[7];
  check_offsets(a.max_slots_pad, a.max_local, a.max_owned, off);
  SmemCheck s;
  s.coef = reinterpret_cast<float*>(sm + off[0]);
  s.lv = reinterpret_cast<uint2*>(sm + off[1]);
  s.memo = reinterpret_cast<uint4*>(sm + off[2]);
  s.vt = reinterpret_cast<float*>(sm + off[3]);
  s.vnew = reinterpret_cast<int*>(sm + off[4]);
  s.items = reinterpret_cast<unsigned short*>(sm + off[5]);
  s.hs = reinterpret_cast<uint2*>(sm + off[6]);
  uint4* const smemo = a.chk_memo ? s.memo : nullptr;
  const uint2* const shs = a.hsb ? s.hs : nullptr;
  const int tid = threadIdx.x;
  const Ctl* ctl = a.ctl;
  const int iter = ctl->iter;
  const int count = ctl->nnew;
  int* nxt = next_list(a, iter);
  stamp_start(a, iter, 1);
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  unsigned parity = 0;
  // the first block of a CTA is its own index; later ones come from the counter
  // (a CTA without a first block exits without touching it)
  int first_item = blockIdx.x;
  // a single instance's finished flag, read once (it changes only between launches):
  // spares every visit the instance lookup
  const int done1 = (a.ninst == 1) ? a.inst_done[0] : -1;
  for (;;) {
    int item = first_item;
    if (item < 0) {
      if (tid == 0) s_item = (int)gridDim.x + atomicAdd(&a.ctl->work_c, 1);
      __syncthreads();
      item = s_item;
    }
    first_item = -1;
    if (item >= count) break;
    const int b = a.list_new[item];
    const BlockDesc bd = a.blocks[b];
    if (done1 >= 0 ? done1 : a.inst_done[a.blk_inst[b]]) {
      __syncthreads();
      continue;
    }
    if (!load_block(a, bd, 6, s, &bar, parity, a.Ta, smemo, const_cast<uint2*>(shs))) {
      if (tid == 0) atomicOr(&a.ctl->error, kErrWait);
      (void)mbar_wait(&bar, parity ^ 1u);
      __syncthreads();
      continue;
    }
    const int ns = bd.nslots, nown = bd.nowned;
    const int allc = check_pass(a, bd, s, smemo, shs, s_cnt, &s_moved) ? 0 : 1;
    if (tid == 0) {
      if (!allc) {
        nxt[atomicAdd(&a.ctl->nnext, 1)] = b;
        atomicAdd(&a.inst_nnext[a.blk_inst[b]], 1);
      }
      atomicAdd(&a.ctl->chk_visits, 1ull);
      atomicAdd(&a.ctl->updates, (unsigned long long)nown);
      count_visit(a, iter, 1, ns, bd.nhalo, nown);
      atomicAdd(&a.ctl->slot_visits, (unsigned long long)ns);
      atomicAdd(&a.ctl->halo_visits, (unsigned long long)bd.nhalo);
      atomicAdd(&a.ctl->owned_visits, (unsigned long long)nown);
    }
    __syncthreads();
  }
  stamp_end(a, iter, 1);
}

// ===========================================================================
// 2D visit: kCheck = false -> FIMCuda (reads main, writes out, fim_sweeps sweeps)
//           kCheck = true  -> run_check_neighbor (reads out, writes main, 1 sweep)
// Corner ids carry bit 15 when the reference never refreshes that slot copy.
// ===========================================================================
template <bool kCheck>
__global__ void __launch_bounds__(256) k_visit2d(DevArgs a) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_item;
  const Smem s0 = carve(sm, a, 4);
  const int tid = threadIdx.x, NT = blockDim.x;
  const Ctl* ctl = a.ctl;
  const int iter = ctl->iter;
  const int stamp = iter + 1;
  const int nact = ctl->nact;
  const int count = kCheck ? nact + ctl->nnew : nact;
  const int* act = act_list(a, iter);
  int* nxt = next_list(a, iter);
  const int nsweeps = kCheck ? 1 : a.fim_sweeps;
  const float* Tsrc = kCheck ? a.Tb : a.Ta;
  float* Tdst = kCheck ? a.Ta : a.Tb;
  stamp_start(a, iter, kCheck ? 1 : 0);
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  unsigned parity = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(kCheck ? &a.ctl->work_c : &a.ctl->work_a, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= count) break;
    const int b = (item < nact) ? act[item] : a.list_new[item - nact];
    if (a.inst_done[a.blk_inst[b]]) {  // instance finished: leave its blocks alone
      __syncthreads();
      continue;
    }
    const BlockDesc bd = a.blocks[b];
    Smem s = s0;
    const bool ok = load_block(a, bd, 4, s, &bar, parity, Tsrc);
    if (!ok) {
      if (tid == 0) atomicOr(&a.ctl->error, kErrWait);
      (void)mbar_wait(&bar, parity ^ 1u);
      __syncthreads();
      continue;
    }
    __syncthreads();
    const int ns = bd.nslots, np = bd.nslots_pad, nown = bd.nowned;
    for (int j = tid; j < ns; j += NT) {
      const uint2 l = s.lv[j];
      const int raw[3] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu)};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int id = raw[k] & 0x7fff;
        float v = 0.0f;
        if (raw[k] & 0x8000) {
          const int g = (id < nown) ? bd.vbase + id : a.halo[bd.halo_begin + id - nown];
          v = a.Tinit[g];
        } else if (id >= nown) {
          v = s.vt[id];
        }
        s.h0[4 * j + k] = v;
      }
      s.m0[j] = 0;
    }
    __syncthreads();
    int myconv = 1;
    for (int sw = 0; sw < nsweeps; ++sw) {
      for (int j = tid; j < ns; j += NT) {
        const uint2 l = s.lv[j];
        const int raw[3] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu)};
        int id[3];
        bool live[3];
        float T[3];
        unsigned ch = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          id[k] = raw[k] & 0x7fff;
          live[k] = !(raw[k] & 0x8000) && id[k] < nown;  // owned copy refreshed by reconciliation
          T[k] = live[k] ? s.vt[id[k]] : s.h0[4 * j + k];
          const unsigned c = live[k] ? (unsigned)s.vchg[id[k]] : ((unsigned)s.m0[j] >> k) & 1u;
          ch |= c << k;
        }
        if (sw == 0) ch = 0x7u;
        float nw[3] = {T[0], T[1], T[2]};
        // all three corners together, as the reference's unrolled update does; a
        // slot with no changed value since the previous sweep is skipped
        if (!(T[0] >= kLarge2DDev && T[1] >= kLarge2DDev && T[2] >= kLarge2DDev) &&
            (ch || T[0] != T[0] || T[1] != T[1] || T[2] != T[2])) {
          const float e0 = s.coef[0 * np + j], e1 = s.coef[1 * np + j], e2 = s.coef[2 * np + j];
          const float F = s.coef[3 * np + j];
          // corner 0 from (v1, v2); corner 1 from (v2, v0); corner 2 from (v0, v1)
          nw[0] = tri_update<false>(T[1], T[2], T[0], e1, e2, e0, F, 0.f, 0.f);
          nw[1] = tri_update<false>(T[2], T[0], T[1], e2, e0, e1, F, 0.f, 0.f);
          nw[2] = tri_update<false>(T[0], T[1], T[2], e0, e1, e2, F, 0.f, 0.f);
        }
        unsigned m = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (live[k]) {
            if (nw[k] < T[k]) atomicMin(&s.vnew[id[k]], fkey(nw[k]));
          } else {
            s.h1[4 * j + k] = nw[k];
            m |= (nw[k] != T[k] ? 1u : 0u) << k;
          }
        }
        s.m1[j] = (unsigned char)m;
      }
      __syncthreads();
      const bool last = (sw == nsweeps - 1);
      for (int k = tid; k < nown; k += NT) {
        const float nv = fval(s.vnew[k]);
        const float ov = s.vt[k];
        if (last && k < kReduceCap2D) {
          if (kCheck) {
            myconv &= ((ov - nv) < kEps2D) ? 1 : 0;
          } else {
            float res = ov - nv;
            if (res < 0.0f) res = -res;
            myconv &= (res <= kEps2D) ? 1 : 0;
          }
        }
        s.vchg[k] = (nv != ov) ? 1 : 0;
        s.vt[k] = nv;
      }
      float* th = s.h0; s.h0 = s.h1; s.h1 = th;
      unsigned char* tm = s.m0; s.m0 = s.m1; s.m1 = tm;
      __syncthreads();
    }
    const int allc = __syncthreads_and(myconv);
    for (int k = tid; k < nown; k += NT) Tdst[bd.vbase + k] = s.vt[k];
    if (tid == 0) {
      if (!kCheck) {
        a.conv[b] = allc;
        atomicAdd(&a.ctl->fim_visits, 1ull);
      } else {
        if (!allc) {
          nxt[atomicAdd(&a.ctl->nnext, 1)] = b;
          atomicAdd(&a.inst_nnext[a.blk_inst[b]], 1);
          a.stampA[b] = stamp + 1;  // member of the next iteration's active list
        }
        atomicAdd(&a.ctl->chk_visits, 1ull);
      }
      atomicAdd(&a.ctl->updates, (unsigned long long)nown * nsweeps);
      count_visit(a, iter, kCheck ? 1 : 0, ns, bd.nhalo, nown);
      atomicAdd(&a.ctl->slot_visits, (unsigned long long)ns);
      atomicAdd(&a.ctl->halo_visits, (unsigned long long)bd.nhalo);
      atomicAdd(&a.ctl->owned_visits, (unsigned long long)nown);
      if (!kCheck) {
        atomicAdd(&a.ctl->fim_slots, (unsigned long long)ns);
        atomicAdd(&a.ctl->fim_halo, (unsigned long long)bd.nhalo);
        atomicAdd(&a.ctl->fim_owned, (unsigned long long)nown);
      }
    }
    __syncthreads();
  }
  stamp_end(a, iter, kCheck ? 1 : 0);
}

// ===========================================================================
// 2D visit, one thread per element slot (blocks of up to 1024 slots).  Each
// thread keeps its slot's edge lengths, inverse speed and the copies of corners
// that belong to other blocks in registers across the sweeps, and the sweep loop
// is unrolled at compile time, as in the reference's FIMCuda: the compiler then
// forms the same fused multiply-adds and the results match it bit for bit.
// kSweeps = 0 runs a runtime sweep count (fim_sweeps) instead.
// ===========================================================================
template <bool kCheck, int kSweeps>
__global__ void __launch_bounds__(1024) k_visit2d_slot(DevArgs a) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_item;
  const int np_max = a.max_slots_pad;
  float* s_coef = reinterpret_cast<float*>(sm);
  uint2* s_lv = reinterpret_cast<uint2*>(s_coef + 4 * (size_t)np_max);
  float* s_vt = reinterpret_cast<float*>(s_lv + np_max);
  int* s_vnew = reinterpret_cast<int*>(s_vt + a.max_local);
  unsigned char* s_vchg = reinterpret_cast<unsigned char*>(s_vnew + a.max_owned);
  Smem sv{};
  sv.coef = s_coef;
  sv.lv = s_lv;
  sv.vt = s_vt;
  sv.vnew = s_vnew;
  const int tid = threadIdx.x, NT = blockDim.x;
  const Ctl* ctl = a.ctl;
  const int iter = ctl->iter;
  const int stamp = iter + 1;
  const int nact = ctl->nact;
  const int count = kCheck ? nact + ctl->nnew : nact;
  const int* act = act_list(a, iter);
  int* nxt = next_list(a, iter);
  const int nsweeps = kSweeps > 0 ? kSweeps : (kCheck ? 1 : a.fim_sweeps);
  const float* Tsrc = kCheck ? a.Tb : a.Ta;
  float* Tdst = kCheck ? a.Ta : a.Tb;
  stamp_start(a, iter, kCheck ? 1 : 0);
  if (tid == 0) mbar_init(&bar, 1);
  __syncthreads();
  unsigned parity = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(kCheck ? &a.ctl->work_c : &a.ctl->work_a, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= count) break;
    const int b = (item < nact) ? act[item] : a.list_new[item - nact];
    if (a.inst_done[a.blk_inst[b]]) {  // instance finished: leave its blocks alone
      __syncthreads();
      continue;
    }
    const BlockDesc bd = a.blocks[b];
    const bool ok = load_block(a, bd, 4, sv, &bar, parity, Tsrc);
    if (!ok) {
      if (tid == 0) atomicOr(&a.ctl->error, kErrWait);
      (void)mbar_wait(&bar, parity ^ 1u);
      __syncthreads();
      continue;
    }
    __syncthreads();
    const int ns = bd.nslots, np = bd.nslots_pad, nown = bd.nowned;
    const int j = tid;
    const bool mine = j < ns;
    int id[3] = {0, 0, 0};
    bool live[3] = {true, true, true};
    float h[3] = {0.f, 0.f, 0.f};
    float e0 = 0.f, e1 = 0.f, e2 = 0.f, F = 0.f;
    if (mine) {
      const uint2 l = s_lv[j];
      const int raw[3] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu)};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        id[k] = raw[k] & 0x7fff;
        live[k] = !(raw[k] & 0x8000) && id[k] < nown;
        if (raw[k] & 0x8000) {
          const int g = (id[k] < nown) ? bd.vbase + id[k] : a.halo[bd.halo_begin + id[k] - nown];
          h[k] = a.Tinit[g];
        } else if (id[k] >= nown) {
          h[k] = s_vt[id[k]];
        }
      }
      e0 = s_coef[0 * np + j];
      e1 = s_coef[1 * np + j];
      e2 = s_coef[2 * np + j];
      F = s_coef[3 * np + j];
    }
    // edge-candidate products, rounded once per visit (see tri_update)
    const float eF0 = __fmul_rn(e0, F), eF1 = __fmul_rn(e1, F), eF2 = __fmul_rn(e2, F);
    unsigned hchg = 0;
    int myconv = 1;
#pragma unroll
    for (int sw = 0; sw < (kSweeps > 0 ? kSweeps : 1); ++sw) {
      for (int rs = 0; rs < (kSweeps > 0 ? 1 : nsweeps); ++rs) {
        const int swi = (kSweeps > 0) ? sw : rs;
        if (mine) {
          float T[3];
          unsigned ch = 0;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            T[k] = live[k] ? s_vt[id[k]] : h[k];
            const unsigned c = live[k] ? (unsigned)s_vchg[id[k]] : (hchg >> k) & 1u;
            ch |= c << k;
          }
          if (swi == 0) ch = 0x7u;
          float nw0 = T[0], nw1 = T[1], nw2 = T[2];
          if (!(T[0] >= kLarge2DDev && T[1] >= kLarge2DDev && T[2] >= kLarge2DDev) &&
              (ch || T[0] != T[0] || T[1] != T[1] || T[2] != T[2])) {
            // corner 0 from (v1, v2); corner 1 from (v2, v0); corner 2 from (v0, v1)
            nw0 = tri_update<!kCheck>(T[1], T[2], T[0], e1, e2, e0, F, eF0, eF2);
            nw1 = tri_update<!kCheck>(T[2], T[0], T[1], e2, e0, e1, F, eF1, eF0);
            nw2 = tri_update<!kCheck>(T[0], T[1], T[2], e0, e1, e2, F, eF2, eF1);
          }
          const float nw[3] = {nw0, nw1, nw2};
          hchg = 0;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            if (live[k]) {
              if (nw[k] < T[k]) atomicMin(&s_vnew[id[k]], fkey(nw[k]));
            } else {
              hchg |= (nw[k] != h[k] ? 1u : 0u) << k;
              h[k] = nw[k];
            }
          }
        }
        __syncthreads();
        const bool last = (swi == nsweeps - 1);
        for (int k = tid; k < nown; k += NT) {
          const float nv = fval(s_vnew[k]);
          const float ov = s_vt[k];
          if (last && k < kReduceCap2D) {
            if (kCheck) {
              myconv &= ((ov - nv) < kEps2D) ? 1 : 0;
            } else {
              float res = ov - nv;
              if (res < 0.0f) res = -res;
              myconv &= (res <= kEps2D) ? 1 : 0;
            }
          }
          s_vchg[k] = (nv != ov) ? 1 : 0;
          s_vt[k] = nv;
        }
        __syncthreads();
      }
    }
    const int allc = __syncthreads_and(myconv);
    for (int k = tid; k < nown; k += NT) Tdst[bd.vbase + k] = s_vt[k];
    if (tid == 0) {
      if (!kCheck) {
        a.conv[b] = allc;
        atomicAdd(&a.ctl->fim_visits, 1ull);
        atomicAdd(&a.ctl->fim_slots, (unsigned long long)ns);
        atomicAdd(&a.ctl->fim_halo, (unsigned long long)bd.nhalo);
        atomicAdd(&a.ctl->fim_owned, (unsigned long long)nown);
      } else {
        if (!allc) {
          nxt[atomicAdd(&a.ctl->nnext, 1)] = b;
          atomicAdd(&a.inst_nnext[a.blk_inst[b]], 1);
          a.stampA[b] = stamp + 1;
        }
        atomicAdd(&a.ctl->chk_visits, 1ull);
      }
      atomicAdd(&a.ctl->updates, (unsigned long long)nown * nsweeps);
      count_visit(a, iter, kCheck ? 1 : 0, ns, bd.nhalo, nown);
      atomicAdd(&a.ctl->slot_visits, (unsigned long long)ns);
      atomicAdd(&a.ctl->halo_visits, (unsigned long long)bd.nhalo);
      atomicAdd(&a.ctl->owned_visits, (unsigned long long)nown);
    }
    __syncthreads();
  }
  stamp_end(a, iter, kCheck ? 1 : 0);
}

size_t smem_bytes_slot2d(int max_slots_pad, int max_local, int max_owned) {
  size_t n = 16 * (size_t)max_slots_pad + 8 * (size_t)max_slots_pad + 4 * (size_t)max_local +
             4 * (size_t)max_owned + (size_t)max_owned;
  return (n + 15) & ~(size_t)15;
}

// ===========================================================================
// 3D: commit visit outputs (CopyOutBack), mark visited blocks, queue the
// neighbours of converged blocks for a check and carry unconverged blocks over.
// One warp per active block.
// ===========================================================================
__global__ void k_commit3d(DevArgs a) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  const int iter = a.ctl->iter, stamp = iter + 1;
  // with the checks inside the sweep kernel: the carried-over blocks and those its
  // checks activated; the candidates go to the list the next sweep launch reads
  const int count = a.ctl->nact + (a.fused ? a.ctl->nadd : 0);
  const int* act = act_list(a, iter);
  int* nxt = next_list(a, iter);
  int* const cl = a.fused ? a.cand + (size_t)(iter & 1) * a.nb : a.list_new;
  int* const cn = a.fused ? &a.ctl->ncand[iter & 1] : &a.ctl->nnew;
  // a single instance's state and the first list entries, read with the control block
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int done1 = (a.ninst == 1) ? a.inst_done[0] : -1;
  // the warp's first entry of either list (the iteration's parity picks one): a
  // dependent round trip less (65^3 solve 0.3% faster)
  const int spec0 = (gw < a.nb) ? a.list0[gw] : 0, spec1 = (gw < a.nb) ? a.list1[gw] : 0;
  if (done1 > 0) return;
  // one warp per list entry, assigned by warp index (no claim round trip).  The
  // launch is a chain of dependent loads, so every load that depends only on the
  // block is issued in one round before any branch on them.
  for (int item = gw; item < count; item += nwarps) {
    const int b = (item == gw) ? ((iter & 1) ? spec1 : spec0) : act[item];
    const BlockDesc bd = a.blocks[b];
    const int cv = a.conv[b];
    const int e0 = a.nbr_off[b], e1 = a.nbr_off[b + 1];
    const int inst = (done1 >= 0) ? 0 : a.blk_inst[b];
    const int dn = (done1 >= 0) ? 0 : a.inst_done[inst];
    const float t0 = (lane < bd.nowned) ? a.Tb[bd.vbase + lane] : 0.0f;
    const float t1 = (lane + 32 < bd.nowned) ? a.Tb[bd.vbase + lane + 32] : 0.0f;
    const int nb0 = (e0 + lane < e1) ? a.nbr[e0 + lane] : -1;
    if (dn) continue;
    if (lane < bd.nowned) a.Ta[bd.vbase + lane] = t0;
    if (lane + 32 < bd.nowned) a.Ta[bd.vbase + lane + 32] = t1;
    for (int k = lane + 64; k < bd.nowned; k += 32) a.Ta[bd.vbase + k] = a.Tb[bd.vbase + k];
    if (lane == 0) a.visited[b] = 1;
    if (cv) {
      // queue each neighbour not left unconverged this iteration, once: the stamp
      // test and the exchange go out together (an unconverged neighbour marked as
      // queued is never queued, which is what it needs)
      for (int base = e0; base < e1; base += 32) {
        const int nb = (base == e0) ? nb0 : ((base + lane < e1) ? a.nbr[base + lane] : -1);
        bool q = false;
        if (nb >= 0) {
          const int sa = a.stampA[nb];
          const int old = atomicExch(&a.stampC[nb], stamp);
          q = sa != stamp && old != stamp;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, q);
        if (bal) {
          int pos = 0;
          if (lane == 0) pos = atomicAdd(cn, __popc(bal));
          pos = __shfl_sync(0xffffffffu, pos, 0) + __popc(bal & ((1u << lane) - 1u));
          if (q) {
            cl[pos] = nb;
            if (a.fused) atomicAdd(&a.inst_ncand[inst], 1);
          }
        }
      }
    } else if (lane == 0) {
      nxt[atomicAdd(&a.ctl->nnext, 1)] = b;
      atomicAdd(&a.inst_nnext[inst], 1);
    }
  }
}

// 2D: queue the neighbours of converged active blocks that are not active.
__global__ void k_activate2d(DevArgs a) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  const int iter = a.ctl->iter, stamp = iter + 1;
  const int count = a.ctl->nact;
  const int* act = act_list(a, iter);
  // one warp per list entry, assigned by warp index (no claim round trip).  As in
  // k_commit3d, the launch is a chain of dependent loads: a single instance's state
  // and the warp's first entry of either list come with the control block, and
  // every load that depends only on the block goes out before any branch on them.
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int done1 = (a.ninst == 1) ? a.inst_done[0] : -1;
  const int spec0 = (gw < a.nb) ? a.list0[gw] : 0, spec1 = (gw < a.nb) ? a.list1[gw] : 0;
  if (done1 > 0) return;
  for (int item = gw; item < count; item += nwarps) {
    const int b = (item == gw) ? ((iter & 1) ? spec1 : spec0) : act[item];
    const int cv = a.conv[b];
    const int e0 = a.nbr_off[b], e1 = a.nbr_off[b + 1];
    const int dn = (done1 >= 0) ? 0 : a.inst_done[a.blk_inst[b]];
    const int nb0 = (e0 + lane < e1) ? a.nbr[e0 + lane] : -1;
    if (dn || !cv) continue;
    for (int base = e0; base < e1; base += 32) {
      const int nb = (base == e0) ? nb0 : ((base + lane < e1) ? a.nbr[base + lane] : -1);
      // the active-list test and the exchange go out together (a block already
      // in the list marked as queued is never queued, which is what it needs)
      bool q = false;
      if (nb >= 0) {
        const int sa = a.stampA[nb];
        const int old = atomicExch(&a.stampC[nb], stamp);
        q = sa != stamp && old != stamp;
      }
      const unsigned bal = __ballot_sync(0xffffffffu, q);
      if (bal) {
        int pos = 0;
        if (lane == 0) pos = atomicAdd(&a.ctl->nnew, __popc(bal));
        pos = __shfl_sync(0xffffffffu, pos, 0) + __popc(bal & ((1u << lane) - 1u));
        if (q) a.list_new[pos] = nb;
      }
    }
  }
}

// End of an outer iteration, run by all threads of one CTA: every running
// instance counts the iteration and stops when its next active list is empty, its
// iteration cap is reached, or (2D) every vertex passed the all-vertex test
// (the loop conditions of meshFIM3dEikonal.cu:411-417 / meshFIM2d_eikonal.cu:683-690,
// 813-815); the loop goes on while any instance runs.
__device__ void finish_iteration_cta(const DevArgs& a, bool vertex_test) {
  Ctl* c = a.ctl;
  // the control block's words and (below) each instance's, loaded in one round
  // before any decision: the close is a short chain of dependent loads
  const int it = c->iter + 1;
  const int nnext = c->nnext, err = c->error, idle0 = c->idle_iters;
  const int pending = (a.serve && threadIdx.x == 0) ? *a.pending : 0;
  int any = 0, fin = 0, swept = 0;
  for (int i = threadIdx.x; i < a.ninst; i += blockDim.x) {
    const int st = a.inst_done[i];
    const int nsw = a.fused ? a.inst_swept[i] : 1, ncd = a.fused ? a.inst_ncand[i] : 0;
    const int its = a.inst_iters[i], nn = a.inst_nnext[i], mx = a.inst_maxit[i];
    const int fl = vertex_test ? a.inst_fail[i] : 1;
    if (st == 0 && nsw == 0) {
      // its checks activated nothing: the reference's loop ended with the previous
      // iteration, which this one does not count
      a.inst_done[i] = 1;
      fin = 1;
    } else if (st == 0) {
      swept = 1;
      const int own = its + 1;  // iterations of this instance since it started
      a.inst_iters[i] = own;
      // blocks waiting: carried over, or (checks in the sweep kernel) to be checked
      const int pend = nn + ncd;
      const bool stop = pend == 0 || own >= mx || fl == 0;
      if (!stop) {
        any = 1;
      } else if (ncd > 0) {
        a.inst_done[i] = 2;  // at its cap: the checks of this iteration still run
        any = 1;
      } else {
        a.inst_done[i] = 1;
        fin = 1;
      }
    } else if (st == 2) {
      a.inst_done[i] = 1;
      fin = 1;
    }
    a.inst_nnext[i] = 0;
    a.inst_fail[i] = 0;
    if (a.fused) {
      a.inst_swept[i] = 0;
      a.inst_ncand[i] = 0;
    }
  }
  any = __syncthreads_or(any);
  fin = __syncthreads_or(fin);
  swept = __syncthreads_or(swept);
  if (threadIdx.x == 0) {
    c->iter = it;
    c->nact = nnext;
    c->nnext = 0;
    c->nnew = 0;
    c->nadd = 0;
    c->ncand[it & 1] = 0;  // consumed by this iteration's sweep launch
    const int idle = (a.fused && !swept) ? 1 : 0;
    c->last_idle = idle;
    c->idle_iters = idle0 + idle;
    c->work_a = c->work_c = 0;
    c->done_d = 0;
    bool go = any && err == 0;
    if (a.serve && (fin || pending != 0)) go = false;
    c->stop = go ? 0 : 1;
    if (a.use_cond) cudaGraphSetConditional(a.cond, go ? 1u : 0u);
  }
}

// last-CTA detection without any waiting: every CTA bumps the counter once
__device__ __forceinline__ bool last_cta(int* counter) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(counter, 1) == (int)gridDim.x - 1);
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

// 2D all-vertex convergence test (meshFIM2d_eikonal.cu:804-815) + iteration close
constexpr int kVertexChunk = 2048;  // vertices per chunk of the 2D all-vertex test

__global__ void k_vertex_test2d(DevArgs a, int copy) {
  pdl_begin();
  // a later copy of the iteration in the graph body, after the loop stopped
  if (copy > 0 && a.ctl->stop) return;
  // chunks of the running instances only (a server's idle slots and finished
  // batch members cost one flag read per chunk)
  for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x) {
    const int2 ch = a.chunks[c];
    if (a.inst_done[ch.x]) continue;  // uniform across the CTA
    const int v1 = min(ch.y + kVertexChunk, a.inst_vbeg[ch.x + 1]);
    int bad = 0;
    // eight vertices per thread per step, all loads issued before the stores
    constexpr int kU = 8;
    const float* __restrict__ Ta = a.Ta;
    float* __restrict__ prev = a.prev;
    for (int v0 = ch.y + threadIdx.x; v0 < v1; v0 += kU * blockDim.x) {
      float cur[kU], old[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int v = v0 + u * blockDim.x;
        cur[u] = (v < v1) ? Ta[v] : 0.0f;
        old[u] = (v < v1) ? prev[v] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int v = v0 + u * blockDim.x;
        if (v < v1) {
          float diff = old[u] - cur[u];
          if (diff < 0.0f) diff = -diff;
          if (!((diff <= kEps2D) && (cur[u] < kLarge2DDev))) bad = 1;
          prev[v] = cur[u];
        }
      }
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0 && bad && a.inst_fail[ch.x] == 0) atomicOr(&a.inst_fail[ch.x], 1);
  }
  if (last_cta(&a.ctl->done_d)) finish_iteration_cta(a, true);
}

// 3D close: a tiny single-CTA kernel after the check visits.  The graph body holds
// several copies of the iteration; the close of a later copy finds the loop already
// stopped when an earlier copy ended it, and leaves the state alone.  (A copy's close
// returns only after an earlier copy of the same pass set the loop's condition to 0.)
__global__ void k_close3d(DevArgs a, int copy) {
  pdl_begin();
  if (copy > 0 && a.ctl->stop) return;
  finish_iteration_cta(a, false);
}

// start of a solve: set the while-condition from the initial active list
// initial travel times: LARGENUM everywhere (prev too unless the caller's initial
// values were copied in) ...
__global__ void k_init_state(float* Ta, float* Tb, float* Tinit, float* prev, int nv, float large) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    Ta[v] = large;
    Tb[v] = large;
    Tinit[v] = large;
    if (prev) prev[v] = large;
  }
}

// ... then 0 at the seed vertices, and the starting blocks marked active (2D)
__global__ void k_seed_state(const int* ids, int n, float* Ta, float* Tb, float* Tinit, float* prev,
                             const int* act, int nact, int* stampA) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = ids[i];
    Ta[v] = 0.0f;
    Tb[v] = 0.0f;
    Tinit[v] = 0.0f;
    if (prev) prev[v] = 0.0f;
  }
  if (stampA)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nact; i += gridDim.x * blockDim.x) stampA[act[i]] = 1;
}

// work waiting: active blocks, or (checks inside the sweep kernel) check candidates
// queued by the last iteration's commit
__device__ __host__ inline bool has_work(const Ctl& c, int fused) {
  return (c.nact > 0 || (fused && c.ncand[(c.iter + 1) & 1] > 0)) && c.max_iters > 0;
}
__global__ void k_start(DevArgs a) {
  if (threadIdx.x == 0) cudaGraphSetConditional(a.cond, has_work(*a.ctl, a.fused) ? 1u : 0u);
}

// per-iteration snapshot in renumbered order (iteration index = iter - 1)
__global__ void k_snapshot(DevArgs a, int dim) {
  pdl_begin();
  const int slot = a.ctl->iter - 1;
  if (slot < 0 || slot >= a.hist_cap || a.ctl->last_idle) return;
  float* dst = a.hist + (size_t)slot * a.nv;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < a.nv; v += gridDim.x * blockDim.x)
    dst[v] = (dim == 3) ? (a.visited[a.vblock[v]] ? a.Ta[v] : 0.0f) : a.Ta[v];
}

// final values to original vertex order
__global__ void k_gather_result(const float* Ta, const unsigned char* visited, const int* vblock, const int* perm,
                                int nv, int dim, float* out) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    const int r = perm[v];
    out[v] = (dim == 3) ? (visited[vblock[r]] ? Ta[r] : 0.0f) : Ta[r];
  }
}
// FP64 residual check (precision mode): for every vertex the smallest FP64 tet
// update over its incident tets, from the final travel times.  Every tet incident
// to a vertex is a slot of the vertex's own block, and every copy of a tet holds the
// same products, so each block computes only its owned apexes.
// lower_only: only candidates that can lie below a vertex's time are needed (the
// polish's marking): apexes at or below the plane-distance bound of their FP64
// update are left out.
__global__ void k_residual3d(DevArgs a, unsigned long long* cand, int lower_only) {
  for (int b = blockIdx.x; b < a.nb; b += gridDim.x) {
    const BlockDesc bd = a.blocks[b];
    const size_t np = (size_t)bd.nslots_pad;
    for (int j = threadIdx.x; j < bd.nslots; j += blockDim.x) {
      const uint2 l = a.lv[bd.slot_begin + j];
      const int id[4] = {(int)(l.x & 0xffffu), (int)(l.x >> 16), (int)(l.y & 0xffffu), (int)(l.y >> 16)};
      int gid[4];
      double T[4];
      for (int k = 0; k < 4; ++k) {
        gid[k] = (id[k] < bd.nowned) ? bd.vbase + id[k] : a.halo[bd.halo_begin + id[k] - bd.nowned];
        T[k] = (double)a.Ta[gid[k]];
      }
      double g[6];
      const int f = a.slot_f64 ? a.slot_f64[bd.slot_begin + j] : -1;
      for (int k = 0; k < 6; ++k)
        g[k] = (f >= 0) ? a.coef64[6 * (size_t)f + k] : (double)a.coef[6 * (size_t)bd.slot_begin + k * np + j];
      const double ACBC = g[0], BCCD = g[1], ACCD = g[2], ADBD = g[3], ACAD = g[4], BCBD = g[5];
      const double ADBC = ACBC + BCCD, ACBD = ACBC + ACCD, CDBD = ADBD - ACBD, ADCD = ADBD - ADBC;
      const double CDCD = ADCD - ACCD, ADAD = ADCD + ACAD, ACAC = ACAD - ACCD, BDBD = BCBD + CDBD;
      const double BCBC = BCBD - BCCD;
      double u[4] = {-1.0, -1.0, -1.0, -1.0};
      bool run[4];
      {
        const uint2* hs = !lower_only ? nullptr
                          : (f >= 0) ? (a.hs64 ? a.hs64 + f : nullptr)
                                     : (a.hsu64 ? a.hsu64 + bd.slot_begin + j : nullptr);
        const float Tf[4] = {(float)T[0], (float)T[1], (float)T[2], (float)T[3]};
        for (int k = 0; k < 4; ++k) {
          const float m = fminf(fminf(Tf[(k + 1) & 3], Tf[(k + 2) & 3]), Tf[(k + 3) & 3]);
          run[k] = id[k] < bd.nowned && !(lower_only && plane_skip(Tf[k], m, slot_bound(hs, 0, k)));
        }
      }
      if (run[3]) u[3] = tet_update_f64(T[0], T[1], T[2], ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
      if (run[0]) u[0] = tet_update_f64(T[1], T[3], T[2], BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC);
      if (run[1]) u[1] = tet_update_f64(T[0], T[3], T[2], ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC);
      if (run[2]) u[2] = tet_update_f64(T[0], T[1], T[3], ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD);
      for (int k = 0; k < 4; ++k)
        if (u[k] >= 0.0) atomicMin(&cand[gid[k]], (unsigned long long)__double_as_longlong(u[k]));
    }
  }
}

// The residual split by sign (FP64 bits where not a count): out[0] = max (T - c) and
// out[1] = max (T - c) / T over vertices whose FP64 update c lies below T (more
// updates would lower T), out[2] = those above 1e-5 relative, out[3] = max (c - T) / T
// over vertices lying below every FP64 update of their tets (the local update is
// not monotone in its inputs, so a time can end below the update of its final
// neighbour times; the FP64 run of the scheme ends so too).  Seeds (T = 0) and
// unreached vertices are skipped.
__global__ void k_residual_reduce(DevArgs a, const unsigned long long* cand, unsigned long long* out) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < a.nv; v += gridDim.x * blockDim.x) {
    const double T = (double)a.Ta[v];
    const double c = __longlong_as_double((long long)cand[v]);
    if (!(T > 0.0) || T >= (double)kLarge3DDev || c >= 1e300) continue;
    if (c < T) {
      const double d = T - c, rel = d / T;
      atomicMax(&out[0], (unsigned long long)__double_as_longlong(d));
      atomicMax(&out[1], (unsigned long long)__double_as_longlong(rel));
      if (rel > 1e-5) atomicAdd(&out[2], 1ull);
    } else if (c > T) {
      atomicMax(&out[3], (unsigned long long)__double_as_longlong((c - T) / T));
    }
  }
}

// Precision mode's polish, start of a round: the loop continues from the current
// times with every slot's update in FP64; every instance runs again for at most
// `cap` iterations; the active list of the coming iteration is rebuilt by
// k_polish_mark.
__global__ void k_polish_begin(DevArgs a, int cap) {
  Ctl* c = a.ctl;
  for (int i = threadIdx.x; i < a.ninst; i += blockDim.x) {
    a.inst_done[i] = 0;
    a.inst_iters[i] = 0;
    a.inst_nnext[i] = 0;
    a.inst_fail[i] = 0;
    const_cast<int*>(a.inst_maxit)[i] = cap;
  }
  if (threadIdx.x == 0) {
    c->max_iters = c->iter + cap;
    c->nact = c->nnext = c->nnew = c->nadd = 0;
    c->ncand[0] = c->ncand[1] = 0;
    c->work_a = c->work_c = 0;
    c->done_d = 0;
    c->stop = 0;
    c->f64_all = EIK_POLISH_F64ALL;
    c->polish = 1;
  }
}

// Queues (once each, `mark` holding `tag`) the blocks owning a vertex whose FP64
// update `cand` lies below its time by more than tol relative.
__global__ void k_polish_mark(DevArgs a, const unsigned long long* cand, int* mark, int tag, double tol) {
  int* list = act_list(a, a.ctl->iter);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < a.nv; v += gridDim.x * blockDim.x) {
    const double T = (double)a.Ta[v];
    const double c = __longlong_as_double((long long)cand[v]);
    if (!(T > 0.0) || T >= (double)kLarge3DDev || !(c < T * (1.0 - tol))) continue;
    const int b = a.vblock[v];
    if (atomicExch(&mark[b], tag) != tag) list[atomicAdd(&a.ctl->nact, 1)] = b;
  }
}

__global__ void k_gather_hist(const float* h, const int* perm, int nv, float* out) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) out[v] = h[perm[v]];
}

// ---------------------------------------------------------------------------
// Serving: instances of a resident arena are admitted between device loops.
// ---------------------------------------------------------------------------

// Drops entries of finished instances from the active list of the coming
// iteration and (checks in the sweep kernel) from its pending check candidates
// (one CTA; list order does not affect results; list_new is scratch here).
__device__ void compact_list(const DevArgs& a, int* list, int* count) {
  __shared__ int s_n;
  const int n = *count;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int b = list[i];
    if (a.inst_done[a.blk_inst[b]] != 1) a.list_new[atomicAdd(&s_n, 1)] = b;
  }
  __syncthreads();
  const int m = s_n;
  for (int i = threadIdx.x; i < m; i += blockDim.x) list[i] = a.list_new[i];
  __syncthreads();
  if (threadIdx.x == 0) *count = m;
}
__global__ void k_compact_active(DevArgs a) {
  Ctl* c = a.ctl;
  compact_list(a, act_list(a, c->iter), &c->nact);
  if (a.fused) compact_list(a, a.cand + (size_t)((c->iter + 1) & 1) * a.nb, &c->ncand[(c->iter + 1) & 1]);
}

// Cancelled instances stop: marked finished, so visits skip their blocks.
__global__ void k_cancel(DevArgs a, const int* insts, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) a.inst_done[insts[i]] = 1;
}

// Fresh state for one instance: vertices [v0, v0+nv), blocks [b0, b0+nb).
__global__ void k_admit_state(DevArgs a, int v0, int nv, int b0, int nb, float large) {
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
    a.Ta[v0 + i] = large;
    a.Tb[v0 + i] = large;
    const_cast<float*>(a.Tinit)[v0 + i] = large;
    a.prev[v0 + i] = large;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += stride) {
    a.conv[b0 + i] = 0;
    a.stampA[b0 + i] = 0;
    a.stampC[b0 + i] = 0;
    a.visited[b0 + i] = 0;
  }
}

// Per-slot metric terms of one 3D instance from its mesh and the request's metric
// factor k (metric entries multiplied by k, then the six products u^T M w of
// tet_gram, every operation rounded separately in the host build's order).
__device__ __forceinline__ float uMw_rn(const float* u, const float* m, const float* w) {
  const float x = __fadd_rn(__fadd_rn(__fmul_rn(u[0], m[0]), __fmul_rn(u[1], m[1])), __fmul_rn(u[2], m[2]));
  const float y = __fadd_rn(__fadd_rn(__fmul_rn(u[0], m[1]), __fmul_rn(u[1], m[3])), __fmul_rn(u[2], m[4]));
  const float z = __fadd_rn(__fadd_rn(__fmul_rn(u[0], m[2]), __fmul_rn(u[1], m[4])), __fmul_rn(u[2], m[5]));
  return __fadd_rn(__fadd_rn(__fmul_rn(x, w[0]), __fmul_rn(y, w[1])), __fmul_rn(z, w[2]));
}

// `memo` (optional): check memos of the same slots, followed `memo_stride` entries
// later by their sweep memos, cleared with the new coefficients
__global__ void k_admit_coef3d(const BlockDesc* blocks, int nb, float* coef, const int* slot_elem, const float* xyz,
                               const int* tets, const float* M, int mcomp, float k, uint4* memo,
                               size_t memo_stride) {
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const BlockDesc d = blocks[b];
    for (int j = threadIdx.x; j < d.nslots; j += blockDim.x) {
      if (memo) {
        memo[d.slot_begin + j] = make_uint4(~0u, ~0u, ~0u, ~0u);
        memo[memo_stride + d.slot_begin + j] = make_uint4(~0u, ~0u, ~0u, ~0u);
      }
      const int t = slot_elem[d.slot_begin + j];
      float P[4][3], m[6];
      for (int q = 0; q < 4; ++q) {
        const int v = tets[4 * (size_t)t + q];
        for (int c = 0; c < 3; ++c) P[q][c] = xyz[3 * (size_t)v + c];
      }
      if (mcomp == 6) {
        for (int q = 0; q < 6; ++q) m[q] = __fmul_rn(M[6 * (size_t)t + q], k);
      } else {  // s*I: the entries s 0 0 s 0 s, each times k
        const float sk = __fmul_rn(M[t], k), zk = __fmul_rn(0.0f, k);
        m[0] = sk; m[1] = zk; m[2] = zk; m[3] = sk; m[4] = zk; m[5] = sk;
      }
      float AC[3], AD[3], BC[3], CD[3], BD[3];
      for (int c = 0; c < 3; ++c) {
        AC[c] = __fsub_rn(P[2][c], P[0][c]);
        AD[c] = __fsub_rn(P[3][c], P[0][c]);
        BC[c] = __fsub_rn(P[2][c], P[1][c]);
        CD[c] = __fsub_rn(P[3][c], P[2][c]);
        BD[c] = __fsub_rn(P[3][c], P[1][c]);
      }
      float* base = coef + 6 * (size_t)d.slot_begin + j;
      const size_t np = (size_t)d.nslots_pad;
      base[0 * np] = uMw_rn(AC, m, BC);
      base[1 * np] = uMw_rn(BC, m, CD);
      base[2 * np] = uMw_rn(AC, m, CD);
      base[3 * np] = uMw_rn(AD, m, BD);
      base[4 * np] = uMw_rn(AC, m, AD);
      base[5 * np] = uMw_rn(BC, m, BD);
    }
  }
}

// Inverse speed column of one 2D instance: 1 / (speed * s) per real face, 1 on
// the virtual faces of obtuse corners (as the host layout sets them).
__global__ void k_admit_coef2d(const BlockDesc* blocks, int nb, float* coef, const int* slot_elem, const float* speed,
                               float s) {
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const BlockDesc d = blocks[b];
    for (int j = threadIdx.x; j < d.nslots; j += blockDim.x) {
      const int e = slot_elem[d.slot_begin + j];
      const float F = (e >= 0) ? __fdiv_rn(1.0f, __fmul_rn(speed[e], s)) : 1.0f;
      coef[4 * (size_t)d.slot_begin + 3 * (size_t)d.nslots_pad + j] = F;
    }
  }
}

// Seeds of one admitted instance (renumbered ids) and its starting blocks appended
// to the active list of the coming iteration; the instance starts running.
__global__ void k_admit_seeds(DevArgs a, int inst, const int* seed_ids, int nseeds, const int* seed_blocks, int nsb,
                              int maxit, int dim) {
  __shared__ int s_base;
  Ctl* c = a.ctl;
  for (int i = threadIdx.x; i < nseeds; i += blockDim.x) {
    const int v = seed_ids[i];
    a.Ta[v] = 0.0f;
    a.Tb[v] = 0.0f;
    const_cast<float*>(a.Tinit)[v] = 0.0f;
    a.prev[v] = 0.0f;
  }
  if (threadIdx.x == 0) {
    s_base = c->nact;
    c->nact += nsb;
    a.inst_done[inst] = 0;
    a.inst_iters[inst] = 0;
    a.inst_nnext[inst] = 0;
    a.inst_fail[inst] = 0;
    if (a.fused) {
      a.inst_swept[inst] = 0;
      a.inst_ncand[inst] = 0;
    }
    const_cast<int*>(a.inst_maxit)[inst] = maxit;
  }
  __syncthreads();
  int* act = act_list(a, c->iter);
  for (int i = threadIdx.x; i < nsb; i += blockDim.x) {
    const int b = seed_blocks[i];
    act[s_base + i] = b;
    if (dim == 2) a.stampA[b] = c->iter + 1;
  }
}

// element-wise evaluation of the device local updates (self-test entry points)
// Failure-path self-test: a barrier that expects 16 bytes no copy ever brings;
// the bounded wait must give up and report it.
__global__ void k_selftest_wait(int* status, unsigned long long* waited_ns) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, 16);
    const unsigned long long t0 = global_ns();
    const bool ok = mbar_wait(&bar, 0);
    *waited_ns = global_ns() - t0;
    *status = ok ? 0 : kErrWait;
  }
}

__global__ void k_selftest_tet(const float* in, float* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float* a = in + 9 * (size_t)i;
    out[i] = tet_update(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
  }
}
// the four apex updates of a slot as the visit kernels run them: per case TA TB TC
// TD and the six stored metric edge products in, min(T_k, update of apex k) out
__global__ void k_selftest_tet_group(const float* in, float* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float* a = in + 10 * (size_t)i;
    const float T[4] = {a[0], a[1], a[2], a[3]};
    const TetGram g = tet_gram9(a[4], a[5], a[6], a[7], a[8], a[9]);
    float* o = out + 4 * (size_t)i;
    o[0] = fminf(T[0], apex_update<0>(T, g));
    o[1] = fminf(T[1], apex_update<1>(T, g));
    o[2] = fminf(T[2], apex_update<2>(T, g));
    o[3] = fminf(T[3], apex_update<3>(T, g));
  }
}
__global__ void k_selftest_tri(const float* in, float* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float* a = in + 7 * (size_t)i;
    out[i] = tri_update<false>(a[0], a[1], a[2], a[3], a[4], a[5], a[6], 0.f, 0.f);
  }
}
// precision mode's FP64 tet update from FP32 inputs (the Gram terms widened as the
// kernel widens its FP64 products)
__global__ void k_selftest_tet64(const float* in, float* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float* a = in + 9 * (size_t)i;
    out[i] = (float)tet_update_f64(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
  }
}
__global__ void k_selftest_quot(const float* in, float* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[2 * i] = small_quot(in[2 * i], in[2 * i + 1]);
    out[2 * i + 1] = root_quot(in[2 * i], in[2 * i + 1]);
  }
}

#define CK(x)                                                                           \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) return std::string(#x ": ") + cudaGetErrorString(e_);       \
  } while (0)

// Raises a kernel's dynamic shared-memory limit on the current device to at least
// `bytes`, never lowering it: handles, batches, servers and the allocation-free
// path share the kernels, and one that set a smaller limit after another had set a
// larger one would make the other's launches fail.  The read and the write are one
// step under a lock.
std::mutex g_smem_attr_mutex;
cudaError_t raise_smem_limit(const void* func, size_t bytes) {
  std::lock_guard<std::mutex> lock(g_smem_attr_mutex);
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, func);
  if (e != cudaSuccess) return e;
  if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// CTA size of the item sweep and check kernels when the caller gives none
constexpr int kItemThreads = EIK_ITEM_THREADS;

// Precision mode's polish: rounds, iterations per round, and the relative gap
// between a vertex's time and its FP64 update above which its block runs again.
constexpr int kPolishRounds = 8;
constexpr int kPolishIterations = 1000;
constexpr double kPolishTol = EIK_POLISH_TOL;

// CTA sizes of the 3D visit kernels when the caller gives none.  One thread per
// element slot of the largest block (up to 1024) runs every slot's updates side by
// side; 512 threads lets two CTAs (64 registers per thread) share an SM and overlap
// two block visits, threads of larger blocks taking several slots.  Which is faster
// depends on the updates' cost: on the isotropic 65^3 workload 512 measured 3.5%
// faster, on the anisotropic sliver workload 1024 was 10% faster (36% in precision
// mode, where flagged slots run FP64).  A handle's solves measure both (after one
// warm-up solve) and keep the faster by sweep-kernel time per slot visit; results
// do not depend on the CTA size.  The server uses 512.
int full_visit_threads(int max_slots_pad) {
  int t = 256;
  while (t < max_slots_pad && t < 1024) t *= 2;
  return t;
}
int auto_visit_threads(int max_slots_pad) { return std::min(full_visit_threads(max_slots_pad), 512); }

template <typename T>
std::string dev_alloc(T*& p, size_t n) {
  if (p) { cudaFree(p); p = nullptr; }
  if (n == 0) n = 1;
  CK(cudaMalloc((void**)&p, n * sizeof(T)));
  return "";
}

}  // namespace

// ===========================================================================
// host side
// ===========================================================================
// NVTX range for profilers (a no-op unless a tool injects itself)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

struct DeviceSolve::Impl {
  int dim = 3, nv = 0, nb = 0;
  BlockDesc* blocks = nullptr;
  float* coef = nullptr;
  uint2* lv = nullptr;
  int* halo = nullptr;
  int* nbr_off = nullptr;
  int* nbr = nullptr;
  int* vblock = nullptr;
  int* perm = nullptr;
  float* Ta = nullptr;
  float* Tb = nullptr;
  float* Tinit = nullptr;
  float* prev = nullptr;
  int* conv = nullptr;
  int* stampA = nullptr;
  int* stampC = nullptr;
  unsigned char* visited = nullptr;
  int* list0 = nullptr;
  int* list1 = nullptr;
  int* list_new = nullptr;
  Ctl* ctl = nullptr;
  float* hist = nullptr;
  int hist_cap = 0;
  unsigned long long* ktime = nullptr;
  int ktime_cap = 0;
  float* out_tmp = nullptr;
  int* blk_inst = nullptr;
  int* inst_vbeg = nullptr;
  int2* chunks = nullptr;
  int nchunks = 0;
  int* inst_done = nullptr;
  int* inst_iters = nullptr;
  int* inst_nnext = nullptr;
  int* inst_fail = nullptr;
  int* inst_maxit = nullptr;
  int* cand = nullptr;        // 2 x nb check candidates (checks inside the sweep kernel)
  int* inst_swept = nullptr;  // per instance: blocks swept this iteration
  int* inst_ncand = nullptr;  // per instance: check candidates queued this iteration
  int ninst = 1;
  size_t coef_n = 0;
  // online choice of the 3D visit CTA size (FP32 / precision kernels): candidates
  // measured so far and their sweep-kernel time per slot visit
  int tune_n[2] = {0, 0};
  float tune_cost[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  uint4* chk_memo = nullptr;
  uint2* hsb = nullptr;  // 3D: coef_n / 6 slots of apex distance bounds (k_plane_bounds)
  uint2* hs64 = nullptr;  // precision mode: bounds of the FP64 updates (k_plane_bounds64)
  uint2* hsu64 = nullptr;  // precision mode: per slot, bounds of the polish's FP64 updates  // 3D: check memos of the coef_n / 6 slots, then their sweep memos
  // host staging for the initial state
  std::vector<float> h_prev;  // caller's initial values (renumbered), empty when none
  std::vector<int> h_seed_ids, h_act, h_vblock, h_done, h_maxit;
  int* seed_ids = nullptr;
  size_t seed_cap = 0;
  // precision mode
  int* slot_f64 = nullptr;
  double* coef64 = nullptr;
  unsigned long long* res_cand = nullptr;  // nv + 4 words: per-vertex FP64 minimum, then the reduction
  bool prec = false;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  DevArgs args{};
  int g_sweeps = -1, g_threads = -1;
  bool g_hist = false;
  int g_histcap = -1;
  int g_serve = -1;
  bool g_tele = true;    // the graph's kernels record per-launch telemetry
  bool want_tele = true;  // what the next graph build records
  int device = 0;  // the device current when the object was created
  // serving: host flag (mapped pinned memory) that ends the device loop early
  int* pending_host = nullptr;
  const volatile int* pending_dev = nullptr;
  struct Source {
    float* xyz = nullptr;
    int* tets = nullptr;
    float* M6 = nullptr;  // mcomp metric entries per tet
    int mcomp = 6;
    float* speed = nullptr;
  };
  std::vector<Source> src;         // per pool mesh
  std::vector<int> inst_mesh;      // pool mesh of every instance
  int* slot_elem = nullptr;        // element id per slot (instance-local)
  float* host_res = nullptr;       // pinned: results of finished instances
  bool built = false;              // layout built on the device (src[0], slot_elem kept)
  void free_serve() {
    for (Source& x : src) {
      if (x.xyz) cudaFree(x.xyz);
      if (x.tets) cudaFree(x.tets);
      if (x.M6) cudaFree(x.M6);
      if (x.speed) cudaFree(x.speed);
    }
    src.clear();
    if (slot_elem) cudaFree(slot_elem);
    slot_elem = nullptr;
    built = false;
    if (host_res) cudaFreeHost(host_res);
    host_res = nullptr;
  }
  size_t smem = 0;
  int grid_visit = 0, grid_aux = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int max_slots_pad = 0, max_local = 0, max_owned = 0;
  struct Launch {
    void* func;
    int grid, block;
    size_t smem;
    int extra;  // second kernel argument (k_snapshot's dimension), unused otherwise
  };
  std::vector<Launch> body;  // one iteration of the loop body, in graph order

  void free_all() {
    void* ps[] = {blocks, coef, lv, halo, nbr_off, nbr, vblock, perm, Ta, Tb, Tinit, prev, conv,
                  stampA, stampC, visited, list0, list1, list_new, ctl, hist, ktime, out_tmp,
                  blk_inst, inst_done, inst_iters, inst_nnext, inst_fail, inst_maxit, seed_ids,
                  cand, inst_swept, inst_ncand, slot_f64, coef64, res_cand, inst_vbeg, chunks, chk_memo, hsb, hs64, hsu64};
    for (void* p : ps)
      if (p) cudaFree(p);
    hsb = nullptr;
    hs64 = nullptr;
    hsu64 = nullptr;
    slot_f64 = nullptr;
    coef64 = nullptr;
    res_cand = nullptr;
    inst_vbeg = nullptr;
    chunks = nullptr;
    chk_memo = nullptr;
    tune_n[0] = tune_n[1] = 0;
    nchunks = 0;
    prec = false;
    seed_ids = nullptr;
    seed_cap = 0;
    blocks = nullptr; coef = nullptr; lv = nullptr; halo = nullptr; nbr_off = nullptr; nbr = nullptr;
    vblock = nullptr; perm = nullptr; Ta = nullptr; Tb = nullptr; Tinit = nullptr; prev = nullptr;
    conv = nullptr; stampA = nullptr; stampC = nullptr; visited = nullptr; list0 = nullptr;
    list1 = nullptr; list_new = nullptr; ctl = nullptr; hist = nullptr; ktime = nullptr; out_tmp = nullptr;
    blk_inst = nullptr; inst_done = nullptr; inst_iters = nullptr; inst_nnext = nullptr; inst_fail = nullptr;
    inst_maxit = nullptr;
    cand = nullptr; inst_swept = nullptr; inst_ncand = nullptr;
    hist_cap = 0;
    ktime_cap = 0;
    drop_graph();
  }
  std::string build_graph(const Layout& L, int sweeps, int threads, int hcap, bool serve);
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    g_sweeps = g_threads = g_histcap = -1;
    g_serve = -1;
  }
};

std::string DeviceSolve::Impl::build_graph(const Layout& L, int sweeps, int threads, int hcap, bool serve) {
  Impl& P = *this;
  const bool want_hist = hcap > 0;
  {
    P.drop_graph();
    DevArgs& a = P.args;
    a = DevArgs{};
    a.blocks = P.blocks; a.coef = P.coef; a.lv = P.lv; a.halo = P.halo; a.nbr_off = P.nbr_off; a.nbr = P.nbr;
    a.vblock = P.vblock; a.nb = L.nb; a.nv = L.nv; a.Ta = P.Ta; a.Tb = P.Tb; a.Tinit = P.Tinit; a.prev = P.prev;
    a.conv = P.conv; a.stampA = P.stampA; a.stampC = P.stampC; a.visited = P.visited; a.list0 = P.list0;
    a.list1 = P.list1; a.list_new = P.list_new; a.ctl = P.ctl; a.hist = P.hist; a.hist_cap = hcap;
    a.ktime = P.want_tele ? P.ktime : nullptr;
    a.ktime_cap = P.want_tele ? P.ktime_cap : 0;
    a.fim_sweeps = sweeps; a.max_slots_pad = P.max_slots_pad; a.max_local = P.max_local;
    a.max_owned = P.max_owned;
    a.use_cond = 1;
    a.blk_inst = P.blk_inst; a.inst_done = P.inst_done; a.inst_iters = P.inst_iters;
    a.inst_nnext = P.inst_nnext; a.inst_fail = P.inst_fail; a.ninst = P.ninst; a.inst_maxit = P.inst_maxit;
    a.inst_vbeg = P.inst_vbeg;
    a.chunks = P.chunks;
    a.nchunks = P.nchunks;
    a.serve = serve ? 1 : 0;
    a.pending = P.pending_dev;
    a.slot_f64 = P.slot_f64;
    a.coef64 = P.coef64;
    // (serving clears an instance's memos when admission rewrites its coefficients)
    a.chk_memo = (L.dim == 3) ? P.chk_memo : nullptr;
    a.hsb = (L.dim == 3) ? P.hsb : nullptr;
    a.hs64 = P.hs64;
    a.hsu64 = P.hsu64;
    a.cand = P.cand;
    a.inst_swept = P.inst_swept;
    a.inst_ncand = P.inst_ncand;
    if (serve) { a.ktime = nullptr; a.ktime_cap = 0; }
    CK(cudaGraphCreate(&P.graph, 0));
    CK(cudaGraphConditionalHandleCreate(&a.cond, P.graph, 0, 0));
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    // 2D blocks of up to 1024 slots use the thread-per-slot kernel (bitwise equal
    // to the reference); larger 2D blocks fall back to the slot-loop kernel
    const bool slot2d = (L.dim == 2) && P.max_slots_pad <= 1024;
    int vthreads = threads;
    size_t vsmem = P.smem, vsmem_chk = P.smem;
    void* kv_fim;
    void* kv_chk;
    if (L.dim == 3) {
#if EIK_SWEEP_ITEMS
      kv_fim = P.prec ? (void*)k_visit3d<false, true> : (void*)k_sweep3d;
#else
      kv_fim = P.prec ? (void*)k_visit3d<false, true> : (void*)k_visit3d<false>;
#endif
#if EIK_CHECK_ITEMS
      kv_chk = P.prec ? (void*)k_visit3d<true, true> : (void*)k_check3d;
#else
      kv_chk = P.prec ? (void*)k_visit3d<true, true> : (void*)k_visit3d<true>;
#endif
      // check visits need one set of per-slot copies; they stage the block's check
      // memos (16 B per slot) behind it, and sweep visits their packed slot list
      // (4 B per slot) behind theirs
      const size_t np = (size_t)P.max_slots_pad;
      vsmem_chk = smem_bytes(6, P.max_slots_pad, P.max_local, P.max_owned, false);
      if (a.chk_memo) {
        int maxsm = 0;
        CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const size_t fim_list = P.smem + sizeof(int) * np, chk_memo = vsmem_chk + sizeof(uint4) * np;
        if (std::max(fim_list, chk_memo) + 64 <= (size_t)maxsm) {
          vsmem = fim_list;
          vsmem_chk = chk_memo;
        } else {
          a.chk_memo = nullptr;
        }
      }
      {
        // the item kernels keep more per-slot state in shared memory; blocks too
        // large for it run the slot kernels (same results)
        int maxsm = 0;
        CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const size_t si = smem_bytes_items(P.max_slots_pad, P.max_local, P.max_owned);
        const size_t sc = smem_bytes_check(P.max_slots_pad, P.max_local, P.max_owned);
#if EIK_SWEEP_ITEMS
        if (!P.prec && si + 64 <= (size_t)maxsm) vsmem = si;
        else if (!P.prec) kv_fim = (void*)k_visit3d<false>;
#endif
#if EIK_SWEEP_MEMO
        if (kv_fim == (void*)k_sweep3d && P.chk_memo) a.fim_memo = P.chk_memo + P.coef_n / 6;
#endif
#if EIK_CHECK_ITEMS
        if (!P.prec && sc + 64 <= (size_t)maxsm) vsmem_chk = sc;
        else if (!P.prec) kv_chk = (void*)k_visit3d<true>;
#endif
        (void)si;
        (void)sc;
      }
      a.fused = (EIK_FUSED_CHECK && kv_fim == (void*)k_sweep3d && kv_chk == (void*)k_check3d) ? 1 : 0;
    } else if (slot2d) {
      vthreads = std::max(32, (P.max_slots_pad + 31) & ~31);
      vsmem = vsmem_chk = smem_bytes_slot2d(P.max_slots_pad, P.max_local, P.max_owned);
      kv_fim = (sweeps == 7) ? (void*)k_visit2d_slot<false, 7> : (void*)k_visit2d_slot<false, 0>;
      kv_chk = (void*)k_visit2d_slot<true, 1>;
    } else {
      kv_fim = (void*)k_visit2d<false>;
      kv_chk = (void*)k_visit2d<true>;
      vthreads = std::min(vthreads, 256);  // the slot-loop kernel's launch bound
    }
    CK(raise_smem_limit(kv_fim, vsmem));
    CK(raise_smem_limit(kv_chk, vsmem_chk));
    int occ = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kv_fim, vthreads, vsmem));
    if (occ < 1) return "visit kernel cannot be resident (shared memory / registers)";
    P.grid_visit = std::min(occ * nsm, std::max(L.nb, 1));
    // 3D checks: most slots are settled by the check memo, so a visit is mostly
    // fixed latency (claim, copies, barriers); CTAs of half the size, two per SM,
    // overlap two visits (several slots per thread where a block is larger)
    int cthreads = vthreads, grid_chk = P.grid_visit;
    if (L.dim == 3 && vthreads >= 1024) {
      cthreads = vthreads / 2;
      int occc = 0;
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occc, kv_chk, cthreads, vsmem_chk));
      if (occc >= 2) grid_chk = std::min(occc * nsm, std::max(L.nb, 1));
      else cthreads = vthreads;
    }
    P.grid_aux = nsm * 4;
    // the per-block launches (one warp per list entry, eight a CTA) and the 2D vertex
    // test (a CTA per chunk) need no more CTAs than they have work for; every CTA of
    // the vertex test also takes part in its last-CTA close
#if EIK_SIZED_AUX
    const int grid_blocks = std::max(1, std::min(P.grid_aux, (L.nb + 7) / 8));
    const int grid_chunks = std::max(1, std::min(P.grid_aux, P.nchunks));
#else
    const int grid_blocks = P.grid_aux, grid_chunks = P.grid_aux;
#endif
    // the one-CTA close: a thread per instance, one warp at least (its barriers are
    // then a single warp's for a plain solve)
    const int close_threads = std::min(256, std::max(32, (P.ninst + 31) & ~31));
    // start node
    void* args_ptr[] = {&P.args};
    cudaGraphNode_t n_start, n_while;
    cudaKernelNodeParams kp{};
    kp.func = (void*)k_start; kp.gridDim = dim3(1); kp.blockDim = dim3(32); kp.kernelParams = args_ptr;
    CK(cudaGraphAddKernelNode(&n_start, P.graph, nullptr, 0, &kp));
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = a.cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    CK(cudaGraphAddNode(&n_while, P.graph, &n_start, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaGraphNode_t prevn = nullptr, n;
    P.body.clear();
    bool record = true;  // the direct-launch loop replays the body's first copy
    // consecutive kernels of the body are joined by programmatic edges (every body
    // kernel begins with pdl_begin); where the driver refuses them, ordinary edges
    const bool pdl = EIK_PDL && g_pdl_ok;
    auto add = [&](void* f, int grid, int block, size_t sm, void** params, int extra = -1) -> std::string {
      if (record)
        P.body.push_back(Impl::Launch{f, grid, block, sm, extra >= 0 ? extra : (f == (void*)k_snapshot) ? L.dim : 0});
      cudaKernelNodeParams q{};
      q.func = f; q.gridDim = dim3(grid); q.blockDim = dim3(block); q.sharedMemBytes = (unsigned)sm;
      q.kernelParams = params;
      if (prevn && pdl) {
        CK(cudaGraphAddKernelNode(&n, body, nullptr, 0, &q));
        cudaGraphEdgeData ed{};
        ed.from_port = cudaGraphKernelNodePortProgrammatic;
        ed.type = cudaGraphDependencyTypeProgrammatic;
        if (cudaGraphAddDependencies(body, &prevn, &n, &ed, 1) != cudaSuccess) {
          (void)cudaGetLastError();
          CK(cudaGraphAddDependencies(body, &prevn, &n, nullptr, 1));
        }
      } else {
        CK(cudaGraphAddKernelNode(&n, body, prevn ? &prevn : nullptr, prevn ? 1 : 0, &q));
      }
      prevn = n;
      return "";
    };
    static int dim3v = 3, dim2v = 2;
    void* snap_args[] = {&P.args, (L.dim == 3) ? (void*)&dim3v : (void*)&dim2v};
    std::string e;
    // Solves and batches: the body holds kBodyCopies iterations, so the loop's
    // condition node (which costs about as much as a kernel launch) runs once per
    // that many iterations.  Copies after the loop stopped find nothing to do: their
    // lists are empty or hold only finished instances' blocks, which every kernel
    // skips, and their close (3D) or vertex test (2D) returns at once.  The server
    // keeps one copy: it admits requests between passes.
    static int copy_idx[kBodyCopies] = {0, 1, 2, 3};  // read-only kernel arguments
    static_assert(kBodyCopies == 4, "copy_idx lists every copy");
    const int copies = serve ? 1 : kBodyCopies;
    // the item sweep at its usual CTA size for iterations with many active blocks
    // and at 1024 threads for the others (roles of k_sweep3d), each launch leaving
    // the other's iterations at once
    static int role_vals[3] = {0, 1, 2};  // read-only kernel arguments
    void* sweep_args[3][2] = {{&P.args, &role_vals[0]}, {&P.args, &role_vals[1]}, {&P.args, &role_vals[2]}};
    int grid_small = 0;
    if (kv_fim == (void*)k_sweep3d && EIK_SWEEP_SPLIT > 0 && vthreads == kItemThreads && !a.fused) {
      int occ2 = 0;
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, k_sweep3d, 1024, vsmem));
      if (occ2 >= 1) grid_small = std::min(occ2 * nsm, std::max(L.nb, 1));
    }
    a.sweep_split = grid_small ? EIK_SWEEP_SPLIT : 0;
    for (int u = 0; u < copies; ++u) {
      record = (u == 0);
      void* close_args[] = {&P.args, &copy_idx[u]};
      if (grid_small) {
        if (!(e = add(kv_fim, P.grid_visit, vthreads, vsmem, sweep_args[1], 1)).empty()) return e;
        if (!(e = add(kv_fim, grid_small, 1024, vsmem, sweep_args[2], 2)).empty()) return e;
      } else if (!(e = add(kv_fim, P.grid_visit, vthreads, vsmem, sweep_args[0], 0)).empty()) {
        return e;
      }
      if (L.dim == 3) {
        if (!(e = add((void*)k_commit3d, grid_blocks, 256, 0, args_ptr)).empty()) return e;
        if (!a.fused && !(e = add(kv_chk, grid_chk, cthreads, vsmem_chk, args_ptr)).empty()) return e;
        if (!(e = add((void*)k_close3d, 1, close_threads, 0, close_args)).empty()) return e;
      } else {
        if (!(e = add((void*)k_activate2d, grid_blocks, 256, 0, args_ptr)).empty()) return e;
        if (!(e = add(kv_chk, P.grid_visit, vthreads, vsmem, args_ptr)).empty()) return e;
        if (!(e = add((void*)k_vertex_test2d, grid_chunks, 256, 0, close_args)).empty()) return e;
      }
      if (want_hist)
        if (!(e = add((void*)k_snapshot, P.grid_aux, 256, 0, snap_args)).empty()) return e;
    }
    if (cudaGraphInstantiate(&P.exec, P.graph, 0) != cudaSuccess) {
      if (!pdl) CK(cudaGetLastError());
      // programmatic edges inside the loop body refused: build it again without
      (void)cudaGetLastError();
      g_pdl_ok = false;
      return build_graph(L, sweeps, threads, hcap, serve);
    }
    P.g_sweeps = sweeps;
    P.g_threads = threads;
    P.g_hist = want_hist;
    P.g_histcap = hcap;
    P.g_tele = P.want_tele;
    P.g_serve = serve ? 1 : 0;
  }
  return "";
}

DeviceSolve::DeviceSolve() : p_(new Impl) {
  cudaGetDevice(&p_->device);
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess) stream_ = s;
  cudaEventCreate(&p_->ev0);
  cudaEventCreate(&p_->ev1);
}

DeviceSolve::~DeviceSolve() {
  p_->free_all();
  p_->free_serve();
  if (p_->pending_host) cudaFreeHost(p_->pending_host);
  if (p_->ev0) cudaEventDestroy(p_->ev0);
  if (p_->ev1) cudaEventDestroy(p_->ev1);
  if (stream_) cudaStreamDestroy((cudaStream_t)stream_);
  delete p_;
}

std::string DeviceSolve::upload(const Layout& L) {
  NvtxRange nvtx("eikonal: upload layout");
  Impl& P = *p_;
  if (!stream_) return "CUDA stream creation failed (no usable GPU?)";
  P.free_all();
  P.free_serve();
  L_ = &L;
  P.dim = L.dim;
  P.nv = L.nv;
  P.nb = L.nb;
  const int ncoef = (L.dim == 3) ? 6 : 4;
  std::string e;
  if (!(e = dev_alloc(P.blocks, L.nb)).empty()) return e;
  if (!(e = dev_alloc(P.coef, L.coef.size())).empty()) return e;
  if (!(e = dev_alloc(P.lv, (size_t)L.total_slots)).empty()) return e;
  if (!(e = dev_alloc(P.halo, L.halo_ids.size())).empty()) return e;
  if (!(e = dev_alloc(P.nbr_off, L.nbr_off.size())).empty()) return e;
  if (!(e = dev_alloc(P.nbr, L.nbr.size())).empty()) return e;
  if (!(e = dev_alloc(P.vblock, (size_t)L.nv)).empty()) return e;
  if (!(e = dev_alloc(P.perm, (size_t)L.nv)).empty()) return e;
  cudaStream_t st = (cudaStream_t)stream_;
  CK(cudaMemcpyAsync(P.blocks, L.blocks.data(), sizeof(BlockDesc) * L.nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(P.coef, L.coef.data(), sizeof(float) * L.coef.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(P.lv, L.lv.data(), sizeof(uint16_t) * L.lv.size(), cudaMemcpyHostToDevice, st));
  if (!L.halo_ids.empty())
    CK(cudaMemcpyAsync(P.halo, L.halo_ids.data(), sizeof(int) * L.halo_ids.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(P.nbr_off, L.nbr_off.data(), sizeof(int) * L.nbr_off.size(), cudaMemcpyHostToDevice, st));
  if (!L.nbr.empty())
    CK(cudaMemcpyAsync(P.nbr, L.nbr.data(), sizeof(int) * L.nbr.size(), cudaMemcpyHostToDevice, st));
  P.coef_n = L.coef.size();
  (void)ncoef;
  return finish_upload(L, false);
}

std::string DeviceSolve::upload_built(const Layout& L, Built3D& b) {
  NvtxRange nvtx("eikonal: adopt device-built layout");
  Impl& P = *p_;
  if (!stream_) return "CUDA stream creation failed (no usable GPU?)";
  P.free_all();
  P.free_serve();
  L_ = &L;
  P.dim = b.dim;
  P.nv = L.nv;
  P.nb = L.nb;
  // the device arrays change owner here
  P.blocks = b.blocks;
  P.coef = b.coef;
  P.lv = reinterpret_cast<uint2*>(b.lv);
  P.halo = b.halo;
  P.nbr_off = b.nbr_off;
  P.nbr = b.nbr;
  P.vblock = b.vblock;
  P.perm = b.perm;
  P.slot_elem = b.slot_elem;
  P.src.assign(1, Impl::Source{});
  P.src[0].xyz = b.xyz;
  P.src[0].tets = b.tets;
  if (b.dim == 3) {
    P.src[0].M6 = b.M6;
    P.src[0].mcomp = b.mcomp;
  } else {
    P.src[0].speed = b.M6;  // 2D: the face speeds
  }
  P.coef_n = (b.dim == 3 ? 6 : 4) * (size_t)b.total_slots;
  P.built = true;
  b = Built3D();
  return finish_upload(L, true);
}

// dst[i] = src[i] + add
__global__ void k_offset_copy(int* dst, const int* src, int n, int add) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i] + add;
}

std::string DeviceSolve::upload_replicas(const Layout& L, const std::vector<const Built3D*>& parts) {
  NvtxRange nvtx("eikonal: replicate device-built layouts");
  Impl& P = *p_;
  if (!stream_) return "CUDA stream creation failed (no usable GPU?)";
  if ((int)parts.size() != L.ninst || (int)L.inst_bbeg.size() != L.ninst + 1) return "one part per instance expected";
  P.free_all();
  P.free_serve();
  L_ = &L;
  P.dim = L.dim;
  P.nv = L.nv;
  P.nb = L.nb;
  const int ncoef = (L.dim == 3) ? 6 : 4;
  long long nhalo = 0, nnbr = 0;
  for (const Built3D* b : parts) {
    if (!b || b->dim != L.dim) return "device-built part missing or of another dimension";
    nhalo += b->nhalo;
    nnbr += b->nnbr;
  }
  if (nhalo > 0x7fffffffll || nnbr > 0x7fffffffll) return "arena too large";
  std::string e;
  if (!(e = dev_alloc(P.blocks, L.nb)).empty()) return e;
  if (!(e = dev_alloc(P.coef, (size_t)ncoef * L.total_slots)).empty()) return e;
  if (!(e = dev_alloc(P.lv, (size_t)L.total_slots)).empty()) return e;
  if (!(e = dev_alloc(P.slot_elem, (size_t)std::max(L.total_slots, 1))).empty()) return e;
  if (!(e = dev_alloc(P.halo, (size_t)std::max(nhalo, 1ll))).empty()) return e;
  if (!(e = dev_alloc(P.nbr_off, (size_t)L.nb + 1)).empty()) return e;
  if (!(e = dev_alloc(P.nbr, (size_t)std::max(nnbr, 1ll))).empty()) return e;
  if (!(e = dev_alloc(P.vblock, (size_t)L.nv)).empty()) return e;
  if (!(e = dev_alloc(P.perm, (size_t)L.nv)).empty()) return e;
  cudaStream_t st = (cudaStream_t)stream_;
  CK(cudaMemcpyAsync(P.blocks, L.blocks.data(), sizeof(BlockDesc) * L.nb, cudaMemcpyHostToDevice, st));
  long long soff = 0, hoff = 0, noff = 0;
  auto grid = [](long long n) { return (int)std::max(1ll, std::min(4096ll, (n + 255) / 256)); };
  for (int i = 0; i < L.ninst; ++i) {
    const Built3D& b = *parts[i];
    const int boff = L.inst_bbeg[i], nbi = L.inst_bbeg[i + 1] - boff, voff = L.inst_vbeg[i];
    // per-block SoA runs are relative to the block's slot_begin, so a part's
    // arrays move as a whole
    CK(cudaMemcpyAsync(P.coef + (size_t)ncoef * soff, b.coef, sizeof(float) * ncoef * (size_t)b.total_slots,
                       cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(P.lv + soff, b.lv, sizeof(uint2) * (size_t)b.total_slots, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(P.slot_elem + soff, b.slot_elem, sizeof(int) * (size_t)b.total_slots, cudaMemcpyDeviceToDevice,
                       st));
    if (b.nhalo) k_offset_copy<<<grid(b.nhalo), 256, 0, st>>>(P.halo + hoff, b.halo, b.nhalo, voff);
    k_offset_copy<<<grid(nbi), 256, 0, st>>>(P.nbr_off + boff, b.nbr_off, nbi, (int)noff);
    if (b.nnbr) k_offset_copy<<<grid(b.nnbr), 256, 0, st>>>(P.nbr + noff, b.nbr, b.nnbr, boff);
    CK(cudaGetLastError());
    soff += b.total_slots;
    hoff += b.nhalo;
    noff += b.nnbr;
  }
  if (soff != L.total_slots) return "parts do not match the concatenated layout";
  const int last = (int)noff;
  CK(cudaMemcpyAsync(P.nbr_off + L.nb, &last, sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
  P.coef_n = (size_t)ncoef * L.total_slots;
  return finish_upload(L, false);
}

bool DeviceSolve::layout_built_on_device() const { return p_->built; }

std::string DeviceSolve::layout_arrays(std::vector<float>* coef, std::vector<int>* slot_elem) const {
  const Impl& P = *p_;
  if (!P.coef) return "no layout on the device";
  if (coef) {
    coef->resize(P.coef_n);
    CK(cudaMemcpy(coef->data(), P.coef, sizeof(float) * P.coef_n, cudaMemcpyDeviceToHost));
  }
  if (slot_elem) {
    if (!P.built || !P.slot_elem) return "element ids of the slots are kept on the host for this layout";
    slot_elem->resize(P.coef_n / (P.dim == 3 ? 6 : 4));
    CK(cudaMemcpy(slot_elem->data(), P.slot_elem, sizeof(int) * slot_elem->size(), cudaMemcpyDeviceToHost));
  }
  return "";
}

std::string DeviceSolve::refresh_speed_built(const float* speed) {
  Impl& P = *p_;
  if (!L_ || !P.built || P.src.empty() || P.dim != 2 || !P.src[0].speed) return "no device-built 2D layout";
  const Layout& L = *L_;
  cudaStream_t st = (cudaStream_t)stream_;
  std::vector<float> ones;
  if (!speed) {
    ones.assign((size_t)L.ne, 1.0f);
    speed = ones.data();
  }
  CK(cudaMemcpyAsync(P.src[0].speed, speed, sizeof(float) * (size_t)L.ne, cudaMemcpyHostToDevice, st));
  k_admit_coef2d<<<std::max(1, std::min(L.nb, 4096)), 256, 0, st>>>(P.blocks, L.nb, P.coef, P.slot_elem,
                                                                    P.src[0].speed, 1.0f);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return "";
}

std::string DeviceSolve::refresh_coef_built(const float* M, int mcomp) {
  Impl& P = *p_;
  if (!L_ || !P.built || P.src.empty()) return "no device-built layout";
  if (mcomp != 1 && mcomp != 6) return "metric entries per tet must be 1 or 6";
  const Layout& L = *L_;
  cudaStream_t st = (cudaStream_t)stream_;
  Impl::Source& src = P.src[0];
  if (src.mcomp != mcomp) {  // the kept metric changes shape
    CK(cudaStreamSynchronize(st));
    std::string e = dev_alloc(src.M6, (size_t)mcomp * L.ne);
    if (!e.empty()) return e;
    src.mcomp = mcomp;
  }
  CK(cudaMemcpyAsync(src.M6, M, sizeof(float) * mcomp * (size_t)L.ne, cudaMemcpyHostToDevice, st));
  k_admit_coef3d<<<std::max(1, std::min(L.nb, 4096)), 256, 0, st>>>(P.blocks, L.nb, P.coef, P.slot_elem, src.xyz,
                                                                    src.tets, src.M6, src.mcomp, 1.0f, nullptr, 0);
  CK(cudaGetLastError());
  {
    std::string e = plane_bounds(P.blocks, 0, L.nb, P.coef, P.hsb, st);
    if (!e.empty()) return e;
  }
  CK(cudaStreamSynchronize(st));
  return "";
}

std::string DeviceSolve::finish_upload(const Layout& L, bool layout_on_device) {
  Impl& P = *p_;
  std::string e;
  if (L.dim == 3) {
    if (!(e = dev_alloc(P.hsb, std::max<size_t>(P.coef_n / 6, 1))).empty()) return e;
    if (!(e = plane_bounds(P.blocks, 0, L.nb, P.coef, P.hsb, (cudaStream_t)stream_)).empty()) return e;
  }
  for (float** t : {&P.Ta, &P.Tb, &P.Tinit, &P.prev, &P.out_tmp})
    if (!(e = dev_alloc(*t, (size_t)L.nv)).empty()) return e;
  for (int** t : {&P.conv, &P.stampA, &P.stampC, &P.list0, &P.list1, &P.list_new})
    if (!(e = dev_alloc(*t, (size_t)L.nb)).empty()) return e;
  if (!(e = dev_alloc(P.visited, (size_t)L.nb)).empty()) return e;
  if (!(e = dev_alloc(P.ctl, 1)).empty()) return e;
  P.ninst = std::max(L.ninst, 1);
  if (!(e = dev_alloc(P.blk_inst, (size_t)L.nb)).empty()) return e;
  for (int** t : {&P.inst_done, &P.inst_iters, &P.inst_nnext, &P.inst_fail, &P.inst_maxit, &P.inst_swept,
                  &P.inst_ncand})
    if (!(e = dev_alloc(*t, (size_t)P.ninst)).empty()) return e;
  if (!(e = dev_alloc(P.cand, 2 * (size_t)L.nb)).empty()) return e;
  if (!(e = dev_alloc(P.inst_vbeg, (size_t)P.ninst + 1)).empty()) return e;
  cudaStream_t st = (cudaStream_t)stream_;
  std::vector<int>& vb = P.h_vblock;
  vb.assign(L.nv, 0);
  for (int b = 0; b < L.nb; ++b)
    for (int k = 0; k < L.blocks[b].nowned; ++k) vb[L.blocks[b].vbase + k] = b;
  if (!layout_on_device) {
    CK(cudaMemcpyAsync(P.vblock, vb.data(), sizeof(int) * L.nv, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(P.perm, L.perm.data(), sizeof(int) * L.nv, cudaMemcpyHostToDevice, st));
  }
  if (!L.slot_f64.empty()) {
    if (L.dim != 3 || L.slot_f64.size() != (size_t)L.total_slots) return "precision data does not match the layout";
    if (!(e = dev_alloc(P.slot_f64, L.slot_f64.size())).empty()) return e;
    if (!(e = dev_alloc(P.coef64, std::max<size_t>(L.coef64.size(), 6))).empty()) return e;
    if (!(e = dev_alloc(P.res_cand, (size_t)L.nv + 4)).empty()) return e;
    CK(cudaMemcpyAsync(P.slot_f64, L.slot_f64.data(), sizeof(int) * L.slot_f64.size(), cudaMemcpyHostToDevice, st));
    if (!L.coef64.empty())
      CK(cudaMemcpyAsync(P.coef64, L.coef64.data(), sizeof(double) * L.coef64.size(), cudaMemcpyHostToDevice, st));
    const int nf64 = (int)(L.coef64.size() / 6);
    if (!(e = dev_alloc(P.hs64, std::max<size_t>((size_t)nf64, 1))).empty()) return e;
    if (nf64 > 0) {
      k_plane_bounds64<<<std::max(1, std::min(4096, (nf64 + 255) / 256)), 256, 0, st>>>(P.coef64, nf64, P.hs64);
      CK(cudaGetLastError());
    }
    if (!(e = dev_alloc(P.hsu64, std::max<size_t>(P.coef_n / 6, 1))).empty()) return e;
    k_plane_bounds_u64<<<std::max(1, std::min(L.nb, 4096)), 256, 0, st>>>(P.blocks, L.nb, P.coef, P.hsu64);
    CK(cudaGetLastError());
    P.prec = true;
  }
  std::vector<int> bi(L.blk_inst);
  if ((int)bi.size() != L.nb) bi.assign(L.nb, 0);
  CK(cudaMemcpyAsync(P.blk_inst, bi.data(), sizeof(int) * L.nb, cudaMemcpyHostToDevice, st));
  std::vector<int> vb0(L.inst_vbeg);
  if ((int)vb0.size() != P.ninst + 1) vb0 = {0, L.nv};
  CK(cudaMemcpyAsync(P.inst_vbeg, vb0.data(), sizeof(int) * vb0.size(), cudaMemcpyHostToDevice, st));
  {
    std::vector<int2> ch;
    for (int i = 0; i < P.ninst; ++i)
      for (int v = vb0[i]; v < vb0[i + 1]; v += kVertexChunk) ch.push_back(make_int2(i, v));
    P.nchunks = (int)ch.size();
    if (!(e = dev_alloc(P.chunks, std::max<size_t>(ch.size(), 1))).empty()) return e;
    if (!ch.empty())
      CK(cudaMemcpyAsync(P.chunks, ch.data(), sizeof(int2) * ch.size(), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  CK(cudaStreamSynchronize(st));
  P.max_slots_pad = (L.max_slots + 3) & ~3;
  P.max_local = std::max(L.max_local, 1);
  P.max_owned = std::max(L.max_owned, 1);
  P.smem = smem_bytes((L.dim == 3) ? 6 : 4, P.max_slots_pad, P.max_local, P.max_owned);
  int dev = 0, maxsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (P.smem + 64 > (size_t)maxsm)
    return "block too large for shared memory (" + std::to_string(L.max_slots) +
           " element slots); use fewer vertices per block";
  return "";
}

std::string DeviceSolve::upload_coef(const Layout& L) {
  Impl& P = *p_;
  if (L.coef.size() != P.coef_n) return "coefficient size changed; upload the layout again";
  CK(cudaMemcpyAsync(P.coef, L.coef.data(), sizeof(float) * L.coef.size(), cudaMemcpyHostToDevice,
                     (cudaStream_t)stream_));
  if (L.dim == 3) {
    std::string e = plane_bounds(P.blocks, 0, L.nb, P.coef, P.hsb, (cudaStream_t)stream_);
    if (!e.empty()) return e;
  }
  CK(cudaStreamSynchronize((cudaStream_t)stream_));
  return "";
}

std::string DeviceSolve::set_seeds(const std::vector<int>& seeds, const float* init_vals) {
  return set_seeds_multi(std::vector<std::vector<int>>(1, seeds), std::vector<const float*>(1, init_vals));
}

std::string DeviceSolve::set_seeds_multi(const std::vector<std::vector<int>>& seeds,
                                         const std::vector<const float*>& init_vals) {
  Impl& P = *p_;
  if (!L_) return "no layout uploaded";
  const Layout& L = *L_;
  const int ninst = std::max(L.ninst, 1);
  if ((int)seeds.size() != ninst) return "one seed list per instance expected";
  const float large = (L.dim == 3) ? kLarge3D : kLarge2D;
  bool any_user = false;
  for (int i = 0; i < ninst && i < (int)init_vals.size(); ++i) any_user = any_user || init_vals[i] != nullptr;
  P.h_prev.clear();
  if (any_user) P.h_prev.assign(L.nv, large);
  P.h_seed_ids.clear();
  std::vector<char> act(L.nb, 0);
  P.h_done.assign(ninst, 1);
  for (int i = 0; i < ninst; ++i) {
    const int v0 = (L.ninst > 1) ? L.inst_vbeg[i] : 0;
    const int nvi = (L.ninst > 1) ? L.inst_vbeg[i + 1] - v0 : L.nv;
    for (int s : seeds[i]) {
      if (s < 0 || s >= nvi) return "seed vertex out of range";
      const int r = L.perm[v0 + s];
      P.h_seed_ids.push_back(r);
      act[P.h_vblock[r]] = 1;
      P.h_done[i] = 0;
    }
    // the reference's TriMesh::vertT: user values, or 0 at seeds and LARGENUM elsewhere
    const float* iv = (i < (int)init_vals.size()) ? init_vals[i] : nullptr;
    if (iv) {
      for (int v = 0; v < nvi; ++v) P.h_prev[L.perm[v0 + v]] = iv[v];
    } else if (any_user) {
      for (int s : seeds[i]) P.h_prev[L.perm[v0 + s]] = 0.0f;
    }
  }
  P.h_act.clear();
  for (int b = 0; b < L.nb; ++b)
    if (act[b]) P.h_act.push_back(b);
  return "";
}

std::string DeviceSolve::solve(const SolveOptions& opt) {
  NvtxRange nvtx("eikonal: solve");
  Impl& P = *p_;
  if (!L_) return "no layout uploaded";
  const Layout& L = *L_;
  cudaStream_t st = (cudaStream_t)stream_;
  const int sweeps = (opt.fim_sweeps > 0) ? opt.fim_sweeps : (L.dim == 3 ? 2 : 7);
  const bool given = opt.threads == 128 || opt.threads == 256 || opt.threads == 384 || opt.threads == 512 ||
                     opt.threads == 768 || opt.threads == 1024;
  int threads = given ? opt.threads : full_visit_threads(P.max_slots_pad);
  int tune_slot = -1;  // which candidate CTA size this solve measures
  const int tq = P.prec ? 1 : 0;
  bool items = false;  // the item sweep and check kernels run (their shared memory fits)
  if (L.dim == 3 && !P.prec && EIK_SWEEP_ITEMS) {
    int maxsm = 0, dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    items = smem_bytes_items(P.max_slots_pad, P.max_local, P.max_owned) + 64 <= (size_t)maxsm;
  }
  if (!given && items) {
    // item kernels: 384-thread CTAs, three per SM where their shared memory allows
    // (65^3 workload: solve 7.85 ms against 7.93 at 512 and 8.4 at one thread per slot)
    threads = kItemThreads;
  } else if (!given && L.dim == 3) {
    const int full = threads, half = auto_visit_threads(P.max_slots_pad);
    if (half < full) {
      if (P.tune_n[tq] < 3) {  // 0: warm-up, 1: measure 512, 2: measure the full size
        tune_slot = P.tune_n[tq];
        // the warm-up (often a handle's only solve) runs the size that usually wins:
        // the full size where FP64 updates make slots long (precision mode)
        threads = (tune_slot == 2 || (tune_slot == 0 && P.prec)) ? full : half;
      } else {
        threads = (P.tune_cost[tq][0] <= P.tune_cost[tq][1]) ? half : full;
      }
    }
  }
  // per-instance iteration caps (one cap for all when not given)
  std::vector<int> cap(P.ninst, opt.max_iterations);
  if ((int)opt.inst_max_iterations.size() == P.ninst) cap = opt.inst_max_iterations;
  int max_iters = 0;
  for (int m : cap) max_iters = std::max(max_iters, m);
  const int hcap = opt.keep_history ? std::max(0, opt.history_cap) : 0;
  if (hcap > 0 && hcap != P.hist_cap) {
    if (P.hist) cudaFree(P.hist);
    P.hist = nullptr;
    CK(cudaMalloc((void**)&P.hist, sizeof(float) * (size_t)hcap * L.nv));
    P.hist_cap = hcap;
    P.drop_graph();
  }
  if (max_iters + 1 > P.ktime_cap) {
    if (P.ktime) cudaFree(P.ktime);
    P.ktime = nullptr;
    P.ktime_cap = max_iters + 1;
    CK(cudaMalloc((void**)&P.ktime, sizeof(unsigned long long) * kKStride * (size_t)P.ktime_cap));
    P.drop_graph();
  }
  if (opt.telemetry || tune_slot >= 0)
    CK(cudaMemsetAsync(P.ktime, 0, sizeof(unsigned long long) * kKStride * (size_t)P.ktime_cap, st));
  // initial state
  // initial state built on the device: only the seed ids, the starting blocks and
  // (when given) the caller's initial values cross from the host
  if (P.h_seed_ids.size() > P.seed_cap) {
    if (P.seed_ids) cudaFree(P.seed_ids);
    P.seed_ids = nullptr;
    P.seed_cap = std::max<size_t>(P.h_seed_ids.size(), 64);
    CK(cudaMalloc((void**)&P.seed_ids, sizeof(int) * P.seed_cap));
  }
  const float large = (L.dim == 3) ? kLarge3D : kLarge2D;
  const bool user_prev = !P.h_prev.empty();
  const int nseed = (int)P.h_seed_ids.size();
  if (nseed > 0)
    CK(cudaMemcpyAsync(P.seed_ids, P.h_seed_ids.data(), sizeof(int) * nseed, cudaMemcpyHostToDevice, st));
  k_init_state<<<std::max(1, std::min(4096, (L.nv + 255) / 256)), 256, 0, st>>>(
      P.Ta, P.Tb, P.Tinit, user_prev ? nullptr : P.prev, L.nv, large);
  if (user_prev) CK(cudaMemcpyAsync(P.prev, P.h_prev.data(), sizeof(float) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(P.stampA, 0, sizeof(int) * L.nb, st));
  if (!P.h_act.empty())
    CK(cudaMemcpyAsync(P.list0, P.h_act.data(), sizeof(int) * P.h_act.size(), cudaMemcpyHostToDevice, st));
  {
    const int nact = (int)P.h_act.size();
    const int n = std::max(nseed, nact);
    if (n > 0)
      k_seed_state<<<std::max(1, std::min(1024, (n + 255) / 256)), 256, 0, st>>>(
          P.seed_ids, nseed, P.Ta, P.Tb, P.Tinit, user_prev ? nullptr : P.prev, P.list0, nact,
          (L.dim == 2) ? P.stampA : nullptr);
    CK(cudaGetLastError());
  }
  CK(cudaMemsetAsync(P.stampC, 0, sizeof(int) * L.nb, st));
  CK(cudaMemsetAsync(P.visited, 0, L.nb, st));
  CK(cudaMemsetAsync(P.conv, 0, sizeof(int) * L.nb, st));
  // 3D check memos (16 B per slot) hold only for this solve's coefficients and kernel
  if (L.dim == 3) {
    if (!P.chk_memo) {
      std::string e = dev_alloc(P.chk_memo, 2 * (P.coef_n / 6));
      if (!e.empty()) return e;
      P.drop_graph();
    }
    CK(cudaMemsetAsync(P.chk_memo, 0xff, sizeof(uint4) * 2 * (P.coef_n / 6), st));
  }
  {
    std::vector<int> done(P.h_done);
    for (int i = 0; i < P.ninst; ++i)
      if (cap[i] <= 0) done[i] = 1;
    P.h_maxit = cap;
    CK(cudaMemcpyAsync(P.inst_done, done.data(), sizeof(int) * P.ninst, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(P.inst_maxit, P.h_maxit.data(), sizeof(int) * P.ninst, cudaMemcpyHostToDevice, st));
    for (int* t : {P.inst_iters, P.inst_nnext, P.inst_fail, P.inst_swept, P.inst_ncand})
      CK(cudaMemsetAsync(t, 0, sizeof(int) * P.ninst, st));
  }
  stats_.h2d_bytes = (long long)sizeof(float) * P.h_prev.size() + (long long)sizeof(int) * nseed +
                     (long long)sizeof(int) * P.h_act.size() + 2ll * sizeof(int) * P.ninst + (long long)sizeof(Ctl);
  Ctl c{};
  c.max_iters = max_iters;
  c.nact = (int)P.h_act.size();
  CK(cudaMemcpyAsync(P.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st));

  // (re)build the graph when the launch shape changes; the CTA-size tuning of the
  // slot kernels measures with the telemetry whatever the option says
  const bool want_hist = hcap > 0;
  P.want_tele = opt.telemetry || tune_slot >= 0;
  if (!P.exec || P.g_sweeps != sweeps || P.g_threads != threads || P.g_hist != want_hist || P.g_histcap != hcap ||
      P.g_serve != 0 || P.g_tele != P.want_tele) {
    std::string e = P.build_graph(L, sweeps, threads, hcap, false);
    if (!e.empty()) return e;
  }
  // the device loop from the control block's current state
  auto run_loop = [&]() -> std::string {
    if (!opt.direct_launch) {
      CK(cudaGraphLaunch(P.exec, st));
      return "";
    }
    // the graph's kernels launched one by one, the host reading the control block
    // between iterations (profilers cannot see kernels inside conditional graphs)
    DevArgs d = P.args;
    d.use_cond = 0;
    for (bool first = true;; first = false) {
      Ctl h{};
      CK(cudaMemcpyAsync(&h, P.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      // the graph's start node's test, then its closes' decision
      if (h.error || (first ? !has_work(h, d.fused) : h.stop != 0)) break;
      for (const Impl::Launch& l : P.body) {
        void* args[2] = {&d, (void*)&l.extra};
        CK(cudaLaunchKernel(l.func, dim3(l.grid), dim3(l.block), args, l.smem, st));
      }
      CK(cudaGetLastError());
    }
    return "";
  };
  CK(cudaEventRecord(P.ev0, st));
  {
    std::string e = run_loop();
    if (!e.empty()) return e;
  }
  // Precision mode acts on its FP64 residual: the blocks owning a vertex that the
  // FP64 update of its tets would lower run the loop again, every slot in FP64,
  // until no such vertex is left (or kPolishRounds rounds).  With no tet flagged
  // the caller asked for FP32 throughout, and nothing is re-visited.
  stats_.polish_rounds = 0;
  stats_.polish_blocks = 0;
  if (P.prec && P.res_cand && L.flagged_tets > 0) {
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    for (int round = 0; round < kPolishRounds; ++round) {
      CK(cudaMemsetAsync(P.res_cand, 0x7f, sizeof(unsigned long long) * L.nv, st));
      k_residual3d<<<std::max(1, std::min(L.nb, 8 * nsm)), 256, 0, st>>>(P.args, P.res_cand, 1);
      k_polish_begin<<<1, 256, 0, st>>>(P.args, kPolishIterations);
      k_polish_mark<<<std::max(1, std::min(4 * nsm, (L.nv + 255) / 256)), 256, 0, st>>>(P.args, P.res_cand, P.stampC,
                                                                                      -(round + 1), kPolishTol);
      CK(cudaGetLastError());
      Ctl h{};
      CK(cudaMemcpyAsync(&h, P.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (h.error || h.nact == 0) break;
      if (P.chk_memo) CK(cudaMemsetAsync(P.chk_memo, 0xff, sizeof(uint4) * 2 * (P.coef_n / 6), st));
      std::string e = run_loop();
      if (!e.empty()) return e;
      stats_.polish_rounds = round + 1;
      stats_.polish_blocks += h.nact;
    }
  }
  CK(cudaEventRecord(P.ev1, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  Ctl out{};
  CK(cudaMemcpy(&out, P.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  cudaEventElapsedTime(&stats_.solve_ms, P.ev0, P.ev1);
  // a trailing iteration that swept nothing (its checks activated no block) is not
  // one of the reference's iterations
  stats_.iterations = out.iter - out.idle_iters;
  stats_.vertex_updates = (long long)out.updates;
  stats_.fim_visits = (long long)out.fim_visits;
  stats_.check_visits = (long long)out.chk_visits;
  stats_.block_visits = stats_.fim_visits + stats_.check_visits;
  stats_.slot_visits = (long long)out.slot_visits;
  stats_.halo_visits = (long long)out.halo_visits;
  stats_.owned_visits = (long long)out.owned_visits;
  stats_.error = out.error;
  stats_.inst_iters.assign(P.ninst, 0);
  CK(cudaMemcpy(stats_.inst_iters.data(), P.inst_iters, sizeof(int) * P.ninst, cudaMemcpyDeviceToHost));
  stats_.fim_slots = (long long)out.fim_slots;
  stats_.fim_halo = (long long)out.fim_halo;
  stats_.fim_owned = (long long)out.fim_owned;
  const bool measured = tune_slot >= 0 && stats_.error == 0 && stats_.fim_slots > 0;
  stats_.fim_kernel_ms = stats_.check_kernel_ms = 0.0f;
  stats_.fim_launches = stats_.check_launches = 0;
  stats_.iter_stats.clear();
  if (P.g_tele) {
    std::vector<unsigned long long> kt(kKStride * (size_t)P.ktime_cap);
    CK(cudaMemcpy(kt.data(), P.ktime, sizeof(unsigned long long) * kt.size(), cudaMemcpyDeviceToHost));
    double fim = 0, chk = 0;
    int nf = 0, nc = 0;
    // launch spans of every loop iteration; rows for the counted ones
    const int nloop = std::min(out.iter, P.ktime_cap);
    const int nit = std::min(stats_.iterations, nloop);
    stats_.iter_stats.assign(kIterStatWords * (size_t)nit, 0);
    const unsigned long long t00 = (nloop > 0 && kt[0]) ? ~kt[0] : 0;
    long long row[kIterStatWords];
    for (int i = 0; i < nloop; ++i) {
      const unsigned long long* k = &kt[kKStride * (size_t)i];
      long long* o = (i < nit) ? &stats_.iter_stats[kIterStatWords * (size_t)i] : row;
      const unsigned long long f0 = ~k[0], c0 = ~k[2];
      if (k[0] && k[1] > f0) { fim += (double)(k[1] - f0); ++nf; o[0] = (long long)(k[1] - f0); }
      if (k[2] && k[3] > c0) { chk += (double)(k[3] - c0); ++nc; o[1] = (long long)(k[3] - c0); }
      for (int w = 0; w < 8; ++w) o[2 + w] = (long long)k[4 + w];
      o[10] = (k[0] && t00) ? (long long)(f0 - t00) : -1;
      o[11] = (k[2] && t00) ? (long long)(c0 - t00) : -1;
      for (int w = 0; w < 4; ++w) o[12 + w] = (long long)k[12 + w];
    }
    stats_.fim_kernel_ms = (float)(fim * 1e-6);
    if (measured && fim > 0) {  // sweep-kernel time per slot visit of this CTA size
      if (tune_slot > 0) P.tune_cost[tq][tune_slot - 1] = (float)(fim / (double)stats_.fim_slots);
      P.tune_n[tq] = tune_slot + 1;
    }
    stats_.check_kernel_ms = (float)(chk * 1e-6);
    stats_.fim_launches = nf;
    stats_.check_launches = nc;
  }
  stats_.residual_max_abs = stats_.residual_max_rel = stats_.residual_below_rel = 0;
  stats_.residual_vertices = 0;
  if (P.prec && P.res_cand && !out.error) {
    // FP64 residual of the final travel times (after the timed region)
    CK(cudaMemsetAsync(P.res_cand, 0x7f, sizeof(unsigned long long) * L.nv, st));
    CK(cudaMemsetAsync(P.res_cand + L.nv, 0, sizeof(unsigned long long) * 4, st));
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    k_residual3d<<<std::max(1, std::min(L.nb, 8 * nsm)), 256, 0, st>>>(P.args, P.res_cand, 0);
    k_residual_reduce<<<std::max(1, std::min(4 * nsm, (L.nv + 255) / 256)), 256, 0, st>>>(P.args, P.res_cand,
                                                                                       P.res_cand + L.nv);
    CK(cudaGetLastError());
    unsigned long long r[4];
    CK(cudaMemcpyAsync(r, P.res_cand + L.nv, sizeof(r), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double d0, d1, d3;
    std::memcpy(&d0, &r[0], sizeof(double));
    std::memcpy(&d1, &r[1], sizeof(double));
    std::memcpy(&d3, &r[3], sizeof(double));
    stats_.residual_max_abs = d0;
    stats_.residual_max_rel = d1;
    stats_.residual_vertices = (long long)r[2];
    stats_.residual_below_rel = d3;
  }
  if (out.error) return "device reported error flags " + std::to_string(out.error);
  return "";
}

std::string DeviceSolve::result_device(float* out_dev) const {
  const Impl& P = *p_;
  if (!L_) return "no layout uploaded";
  k_gather_result<<<std::max(1, std::min(1024, (P.nv + 255) / 256)), 256, 0, (cudaStream_t)stream_>>>(
      P.Ta, P.visited, P.vblock, P.perm, P.nv, P.dim, out_dev);
  CK(cudaGetLastError());
  return "";
}

std::string DeviceSolve::result(float* out_host) const {
  const Impl& P = *p_;
  std::string e = result_device(P.out_tmp);
  if (!e.empty()) return e;
  CK(cudaMemcpyAsync(out_host, P.out_tmp, sizeof(float) * P.nv, cudaMemcpyDeviceToHost, (cudaStream_t)stream_));
  CK(cudaStreamSynchronize((cudaStream_t)stream_));
  return "";
}

std::string DeviceSolve::history(int i, float* out_host) const {
  const Impl& P = *p_;
  if (!P.hist || i < 0 || i >= P.hist_cap || i >= stats_.iterations) return "iteration not recorded";
  k_gather_hist<<<std::max(1, std::min(1024, (P.nv + 255) / 256)), 256, 0, (cudaStream_t)stream_>>>(
      P.hist + (size_t)i * P.nv, P.perm, P.nv, P.out_tmp);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out_host, P.out_tmp, sizeof(float) * P.nv, cudaMemcpyDeviceToHost, (cudaStream_t)stream_));
  CK(cudaStreamSynchronize((cudaStream_t)stream_));
  return "";
}

std::string DeviceSolve::visit_once(bool check, const float* T_host, float* out_host) {
  Impl& P = *p_;
  if (!L_) return "no layout uploaded";
  const Layout& L = *L_;
  cudaStream_t st = (cudaStream_t)stream_;
  std::vector<int> all(L.nb);
  for (int b = 0; b < L.nb; ++b) all[b] = b;
  CK(cudaMemcpyAsync(P.Ta, T_host, sizeof(float) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(P.Tb, T_host, sizeof(float) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(P.Tinit, T_host, sizeof(float) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(P.list0, all.data(), sizeof(int) * L.nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(P.stampA, 0, sizeof(int) * L.nb, st));
  Ctl c{};
  c.max_iters = 1;
  c.nact = L.nb;
  CK(cudaMemcpyAsync(P.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st));
  DevArgs a{};
  a.blocks = P.blocks; a.coef = P.coef; a.lv = P.lv; a.halo = P.halo; a.nbr_off = P.nbr_off; a.nbr = P.nbr;
  a.vblock = P.vblock; a.nb = L.nb; a.nv = L.nv; a.Ta = P.Ta; a.Tb = P.Tb; a.Tinit = P.Tinit; a.prev = P.prev;
  a.conv = P.conv; a.stampA = P.stampA; a.stampC = P.stampC; a.visited = P.visited; a.list0 = P.list0;
  a.list1 = P.list1; a.list_new = P.list_new; a.ctl = P.ctl; a.fim_sweeps = (L.dim == 3) ? 2 : 7;
  a.blk_inst = P.blk_inst; a.inst_done = P.inst_done; a.inst_iters = P.inst_iters;
  a.inst_nnext = P.inst_nnext; a.inst_fail = P.inst_fail; a.ninst = P.ninst;
  CK(cudaMemsetAsync(P.inst_done, 0, sizeof(int) * P.ninst, st));
  a.max_slots_pad = P.max_slots_pad; a.max_local = P.max_local; a.max_owned = P.max_owned;
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (L.dim != 2 || P.max_slots_pad > 1024) return "visit_once supports 2D blocks of up to 1024 slots";
  const int vthreads = std::max(32, (P.max_slots_pad + 31) & ~31);
  const size_t vsmem = smem_bytes_slot2d(P.max_slots_pad, P.max_local, P.max_owned);
  if (!check) {
    CK(raise_smem_limit((const void*)k_visit2d_slot<false, 7>, vsmem));
    k_visit2d_slot<false, 7><<<std::min(L.nb, nsm * 8), vthreads, vsmem, st>>>(a);
  } else {
    CK(raise_smem_limit((const void*)k_visit2d_slot<true, 1>, vsmem));
    k_visit2d_slot<true, 1><<<std::min(L.nb, nsm * 8), vthreads, vsmem, st>>>(a);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out_host, check ? P.Ta : P.Tb, sizeof(float) * L.nv, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return "";
}

// n independent triangles, each its own block owning its three corners; one
// visit with the product's 2D kernel.  in: 7 floats per case (T0 T1 T2 e01 e12
// e20 speedInv), out: 3 per case.
std::string selftest_tri_blocks(const float* in, int n, bool check, float* out) {
  Layout L;
  L.dim = 2;
  L.nv = 3 * n;
  L.ne = n;
  L.nb = n;
  L.perm.resize(L.nv);
  L.iperm.resize(L.nv);
  for (int v = 0; v < L.nv; ++v) L.perm[v] = L.iperm[v] = v;
  L.blocks.resize(n);
  L.total_slots = 4 * n;
  L.coef.assign(16 * (size_t)n, 0.f);
  L.lv.assign(16 * (size_t)n, 0);
  L.slot_elem.assign(4 * (size_t)n, -1);
  for (int b = 0; b < n; ++b) {
    BlockDesc& d = L.blocks[b];
    d.slot_begin = 4 * b; d.nslots = 1; d.nslots_pad = 4; d.vbase = 3 * b; d.nowned = 3;
    d.halo_begin = 0; d.nhalo = 0; d.ninside = 1;
    for (int k = 0; k < 4; ++k) L.coef[16 * (size_t)b + 4 * k] = in[7 * (size_t)b + 3 + k];
    L.lv[16 * (size_t)b + 0] = 0; L.lv[16 * (size_t)b + 1] = 1; L.lv[16 * (size_t)b + 2] = 2;
    L.slot_elem[4 * (size_t)b] = b;
  }
  L.nbr_off.assign(n + 1, 0);
  L.max_slots = 1; L.max_local = 3; L.max_owned = 3; L.max_halo = 0;
  std::vector<float> T(3 * (size_t)n);
  for (int b = 0; b < n; ++b)
    for (int k = 0; k < 3; ++k) T[3 * (size_t)b + k] = in[7 * (size_t)b + k];
  DeviceSolve ds;
  std::string e = ds.upload(L);
  if (!e.empty()) return e;
  return ds.visit_once(check, T.data(), out);
}

size_t device_footprint(const Layout& L, const Built3D* b) {
  const size_t nv = (size_t)L.nv, nb = (size_t)L.nb;
  const size_t ncoef = b ? (size_t)(L.dim == 3 ? 6 : 4) * L.total_slots : L.coef.size();
  const size_t nhalo = b ? (size_t)b->nhalo : L.halo_ids.size();
  const size_t ngraph = b ? nb + 1 + (size_t)b->nnbr : L.nbr_off.size() + L.nbr.size();
  return nb * sizeof(BlockDesc) + ncoef * sizeof(float) + (size_t)L.total_slots * (sizeof(uint2) + sizeof(int)) +
         (L.dim == 3 ? (size_t)L.total_slots * (2 * sizeof(uint4) + sizeof(uint2)) : 0) + nhalo * sizeof(int) +
         ngraph * sizeof(int) +
         nv * (2 * sizeof(int) + 5 * sizeof(float)) + nb * (9 * sizeof(int) + 1) + 7 * sizeof(int);
}

cudaStream_t new_stream() {
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  return st;
}

void free_stream(cudaStream_t st) {
  if (st) cudaStreamDestroy(st);
}

std::string download_built(const Built3D& b, Layout& L) {
  const int ncoef = (L.dim == 3) ? 6 : 4;
  L.coef.resize((size_t)ncoef * L.total_slots);
  L.lv.resize(4 * (size_t)L.total_slots);
  L.slot_elem.resize((size_t)L.total_slots);
  L.halo_ids.resize((size_t)b.nhalo);
  L.nbr_off.resize((size_t)L.nb + 1);
  L.nbr.resize((size_t)b.nnbr);
  CK(cudaMemcpy(L.coef.data(), b.coef, sizeof(float) * L.coef.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(L.lv.data(), b.lv, sizeof(uint16_t) * L.lv.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(L.slot_elem.data(), b.slot_elem, sizeof(int) * L.slot_elem.size(), cudaMemcpyDeviceToHost));
  if (b.nhalo) CK(cudaMemcpy(L.halo_ids.data(), b.halo, sizeof(int) * L.halo_ids.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(L.nbr_off.data(), b.nbr_off, sizeof(int) * L.nbr_off.size(), cudaMemcpyDeviceToHost));
  if (b.nnbr) CK(cudaMemcpy(L.nbr.data(), b.nbr, sizeof(int) * L.nbr.size(), cudaMemcpyDeviceToHost));
  if (L.iperm.size() != (size_t)L.nv) {
    L.iperm.assign(L.nv, 0);
    for (int v = 0; v < L.nv; ++v) L.iperm[L.perm[v]] = v;
  }
  return "";
}

std::string DeviceSolve::serve_setup(const std::vector<ServeSource>& meshes, const std::vector<int>& inst_mesh,
                                     int sweeps, int threads) {
  Impl& P = *p_;
  if (!L_) return "no layout uploaded";
  const Layout& L = *L_;
  if ((int)inst_mesh.size() != P.ninst) return "one pool mesh per instance expected";
  for (int m : inst_mesh)
    if (m < 0 || m >= (int)meshes.size()) return "pool mesh id out of range";
  cudaStream_t st = (cudaStream_t)stream_;
  // an arena replicated on the device (upload_replicas) brings its slots' element
  // ids; a host-built one has them in L
  int* replica_elems = (L.slot_elem.empty() && P.slot_elem) ? P.slot_elem : nullptr;
  if (replica_elems) P.slot_elem = nullptr;
  P.free_serve();
  P.slot_elem = replica_elems;
  P.src.resize(meshes.size());
  for (size_t m = 0; m < meshes.size(); ++m) {
    const ServeSource& x = meshes[m];
    Impl::Source& d = P.src[m];
    std::string e;
    if (x.dim != L.dim) return "pool mesh of another dimension";
    if (x.dim == 3) {
      if (!(e = dev_alloc(d.xyz, 3 * (size_t)x.nv)).empty()) return e;
      if (!(e = dev_alloc(d.tets, 4 * (size_t)x.nt)).empty()) return e;
      if (!(e = dev_alloc(d.M6, 6 * (size_t)x.nt)).empty()) return e;
      CK(cudaMemcpyAsync(d.xyz, x.xyz, sizeof(float) * 3 * x.nv, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.tets, x.tets, sizeof(int) * 4 * (size_t)x.nt, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.M6, x.M6, sizeof(float) * 6 * (size_t)x.nt, cudaMemcpyHostToDevice, st));
    } else {
      if (!(e = dev_alloc(d.speed, (size_t)std::max(x.nf, 1))).empty()) return e;
      CK(cudaMemcpyAsync(d.speed, x.speed, sizeof(float) * x.nf, cudaMemcpyHostToDevice, st));
    }
  }
  P.inst_mesh = inst_mesh;
  if (!replica_elems) {
    if (L.slot_elem.size() != (size_t)L.total_slots) return "element ids of the slots missing";
    std::string e;
    if (!(e = dev_alloc(P.slot_elem, (size_t)std::max(L.total_slots, 1))).empty()) return e;
    CK(cudaMemcpyAsync(P.slot_elem, L.slot_elem.data(), sizeof(int) * L.slot_elem.size(), cudaMemcpyHostToDevice,
                       st));
  }
  if (L.dim == 3) {
    std::string e;
    if (!P.chk_memo && !(e = dev_alloc(P.chk_memo, 2 * (P.coef_n / 6))).empty()) return e;
    CK(cudaMemsetAsync(P.chk_memo, 0xff, sizeof(uint4) * 2 * (P.coef_n / 6), st));
  }
  CK(cudaHostAlloc((void**)&P.host_res, sizeof(float) * std::max(L.nv, 1), cudaHostAllocDefault));
  if (!P.pending_host) {
    CK(cudaHostAlloc((void**)&P.pending_host, sizeof(int), cudaHostAllocMapped));
    void* d = nullptr;
    CK(cudaHostGetDevicePointer(&d, P.pending_host, 0));
    P.pending_dev = (const volatile int*)d;
  }
  *(volatile int*)P.pending_host = 0;
  // every instance idle, every vertex at LARGENUM
  std::vector<int> ones(P.ninst, 1);
  CK(cudaMemcpyAsync(P.inst_done, ones.data(), sizeof(int) * P.ninst, cudaMemcpyHostToDevice, st));
  for (int* t : {P.inst_iters, P.inst_nnext, P.inst_fail, P.inst_maxit, P.inst_swept, P.inst_ncand})
    CK(cudaMemsetAsync(t, 0, sizeof(int) * P.ninst, st));
  for (int* t : {P.conv, P.stampA, P.stampC}) CK(cudaMemsetAsync(t, 0, sizeof(int) * L.nb, st));
  CK(cudaMemsetAsync(P.visited, 0, L.nb, st));
  k_init_state<<<std::max(1, std::min(4096, (L.nv + 255) / 256)), 256, 0, st>>>(
      P.Ta, P.Tb, P.Tinit, P.prev, L.nv, (L.dim == 3) ? kLarge3D : kLarge2D);
  CK(cudaGetLastError());
  Ctl c{};
  c.max_iters = 1 << 30;
  CK(cudaMemcpyAsync(P.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st));
  const bool given = threads == 128 || threads == 256 || threads == 384 || threads == 512 || threads == 768 ||
                     threads == 1024;
  int th = given ? threads : auto_visit_threads(P.max_slots_pad);
  if (!given && L.dim == 3 && EIK_SWEEP_ITEMS) {
    // the item kernels run where their shared memory fits, at the CTA size a
    // plain solve uses
    int dev = 0, maxsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem_bytes_items(P.max_slots_pad, P.max_local, P.max_owned) + 64 <= (size_t)maxsm) th = kItemThreads;
  }
  const int sw = (sweeps > 0) ? sweeps : (L.dim == 3 ? 2 : 7);
  std::string e = P.build_graph(L, sw, th, 0, true);
  if (!e.empty()) return e;
  CK(cudaStreamSynchronize(st));
  return "";
}

std::string DeviceSolve::serve_admit(const std::vector<Admission>& adm) {
  NvtxRange nvtx("eikonal: admit requests");
  Impl& P = *p_;
  if (!L_ || P.g_serve != 1) return "serving not set up";
  const Layout& L = *L_;
  if (adm.empty()) return "";
  cudaStream_t st = (cudaStream_t)stream_;
  // stage every admission's seed ids (renumbered) and starting blocks in one copy
  std::vector<int> stage;
  std::vector<int> off(adm.size()), nsd(adm.size()), boff(adm.size()), nbk(adm.size());
  for (size_t q = 0; q < adm.size(); ++q) {
    const Admission& x = adm[q];
    if (x.inst < 0 || x.inst >= P.ninst) return "instance out of range";
    const int v0 = L.inst_vbeg[x.inst], nvi = L.inst_vbeg[x.inst + 1] - v0;
    off[q] = (int)stage.size();
    for (int sd : x.seeds) {
      if (sd < 0 || sd >= nvi) return "seed vertex out of range";
      stage.push_back(L.perm[v0 + sd]);
    }
    nsd[q] = (int)stage.size() - off[q];
    boff[q] = (int)stage.size();
    for (int i = off[q]; i < off[q] + nsd[q]; ++i) {
      const int b = P.h_vblock[stage[i]];
      bool seen = false;
      for (int j = boff[q]; j < (int)stage.size(); ++j) seen = seen || stage[j] == b;
      if (!seen) stage.push_back(b);
    }
    nbk[q] = (int)stage.size() - boff[q];
  }
  if (stage.size() > P.seed_cap) {
    if (P.seed_ids) cudaFree(P.seed_ids);
    P.seed_ids = nullptr;
    P.seed_cap = std::max<size_t>(stage.size(), 1024);
    CK(cudaMalloc((void**)&P.seed_ids, sizeof(int) * P.seed_cap));
  }
  CK(cudaMemcpyAsync(P.seed_ids, stage.data(), sizeof(int) * stage.size(), cudaMemcpyHostToDevice, st));
  // list entries of instances that finished since the last loop leave the list
  k_compact_active<<<1, 1024, 0, st>>>(P.args);
  const float large = (L.dim == 3) ? kLarge3D : kLarge2D;
  for (size_t q = 0; q < adm.size(); ++q) {
    const Admission& x = adm[q];
    const int i = x.inst;
    const int v0 = L.inst_vbeg[i], nvi = L.inst_vbeg[i + 1] - v0;
    const int b0 = L.inst_bbeg[i], nbi = L.inst_bbeg[i + 1] - b0;
    k_admit_state<<<std::max(1, std::min(2048, (std::max(nvi, nbi) + 255) / 256)), 256, 0, st>>>(
        P.args, v0, nvi, b0, nbi, large);
    const Impl::Source& src = P.src[P.inst_mesh[i]];
    const int g = std::max(1, std::min(nbi, 4096));
    if (L.dim == 3) {
      k_admit_coef3d<<<g, 256, 0, st>>>(P.blocks + b0, nbi, P.coef, P.slot_elem, src.xyz, src.tets, src.M6,
                                        src.mcomp, x.coef_scale, P.chk_memo, P.coef_n / 6);
      std::string e = plane_bounds(P.blocks, b0, nbi, P.coef, P.hsb, st);
      if (!e.empty()) return e;
    } else {
      k_admit_coef2d<<<g, 256, 0, st>>>(P.blocks + b0, nbi, P.coef, P.slot_elem, src.speed, x.coef_scale);
    }
    k_admit_seeds<<<1, 256, 0, st>>>(P.args, i, P.seed_ids + off[q], nsd[q], P.seed_ids + boff[q], nbk[q],
                                     x.max_iterations, L.dim);
  }
  CK(cudaGetLastError());
  return "";
}

std::string DeviceSolve::serve_cancel(const std::vector<int>& insts) {
  Impl& P = *p_;
  if (!L_ || P.g_serve != 1) return "serving not set up";
  if (insts.empty()) return "";
  cudaStream_t st = (cudaStream_t)stream_;
  if (insts.size() > P.seed_cap) {
    if (P.seed_ids) cudaFree(P.seed_ids);
    P.seed_ids = nullptr;
    P.seed_cap = std::max<size_t>(insts.size(), 1024);
    CK(cudaMalloc((void**)&P.seed_ids, sizeof(int) * P.seed_cap));
  }
  CK(cudaMemcpyAsync(P.seed_ids, insts.data(), sizeof(int) * insts.size(), cudaMemcpyHostToDevice, st));
  k_cancel<<<1, 256, 0, st>>>(P.args, P.seed_ids, (int)insts.size());
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return "";
}

std::string DeviceSolve::serve_run() {
  NvtxRange nvtx("eikonal: serving loop");
  Impl& P = *p_;
  if (!L_ || P.g_serve != 1) return "serving not set up";
  cudaStream_t st = (cudaStream_t)stream_;
  CK(cudaGraphLaunch(P.exec, st));
  CK(cudaStreamSynchronize(st));
  Ctl out{};
  CK(cudaMemcpy(&out, P.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  stats_.iterations = out.iter;
  stats_.error = out.error;
  stats_.vertex_updates = (long long)out.updates;  // cumulative since serve_setup
  if (out.error) return "device reported error flags " + std::to_string(out.error);
  return "";
}

std::string DeviceSolve::serve_poll(std::vector<int>& done, std::vector<int>& iters) {
  Impl& P = *p_;
  cudaStream_t st = (cudaStream_t)stream_;
  done.resize(P.ninst);
  iters.resize(P.ninst);
  CK(cudaMemcpyAsync(done.data(), P.inst_done, sizeof(int) * P.ninst, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(iters.data(), P.inst_iters, sizeof(int) * P.ninst, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  // an instance at its cap whose last checks have not run yet (2) is still running
  for (int& d : done) d = (d == 1) ? 1 : 0;
  return "";
}

std::string DeviceSolve::serve_fetch(int inst) {
  Impl& P = *p_;
  if (!L_ || inst < 0 || inst >= P.ninst || !P.host_res) return "instance out of range";
  const Layout& L = *L_;
  cudaStream_t st = (cudaStream_t)stream_;
  const int v0 = L.inst_vbeg[inst], nvi = L.inst_vbeg[inst + 1] - v0;
  k_gather_result<<<std::max(1, std::min(1024, (nvi + 255) / 256)), 256, 0, st>>>(
      P.Ta, P.visited, P.vblock, P.perm + v0, nvi, L.dim, P.out_tmp + v0);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(P.host_res + v0, P.out_tmp + v0, sizeof(float) * nvi, cudaMemcpyDeviceToHost, st));
  return "";
}

std::string DeviceSolve::serve_sync() {
  CK(cudaStreamSynchronize((cudaStream_t)stream_));
  return "";
}

const float* DeviceSolve::serve_host_result(int inst) const {
  const Impl& P = *p_;
  if (!L_ || !P.host_res || inst < 0 || inst >= P.ninst) return nullptr;
  return P.host_res + L_->inst_vbeg[inst];
}

volatile int* DeviceSolve::serve_pending() const { return (volatile int*)p_->pending_host; }

void DeviceSolve::bind_thread() const { cudaSetDevice(p_->device); }

std::string selftest_wait_timeout(int* status, double* waited_ms) {
  int* d_status = nullptr;
  unsigned long long* d_ns = nullptr;
  CK(cudaMalloc((void**)&d_status, sizeof(int)));
  CK(cudaMalloc((void**)&d_ns, sizeof(unsigned long long)));
  k_selftest_wait<<<1, 32>>>(d_status, d_ns);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long ns = 0;
  if (e == cudaSuccess) e = cudaMemcpy(status, d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&ns, d_ns, sizeof(ns), cudaMemcpyDeviceToHost);
  cudaFree(d_status);
  cudaFree(d_ns);
  if (e != cudaSuccess) return std::string("wait self-test: ") + cudaGetErrorString(e);
  *waited_ms = (double)ns * 1e-6;
  return "";
}

std::string selftest_device(int which, const float* in, float* out, int n) {
  if (which == 3 || which == 4) return selftest_tri_blocks(in, n, which == 4, out);
  const int nin = (which == 0 || which == 5) ? 9 : (which == 1) ? 7 : (which == 6) ? 10 : 2;
  const int nout = (which == 2) ? 2 : (which == 6) ? 4 : 1;
  float *din = nullptr, *dout = nullptr;
  CK(cudaMalloc((void**)&din, sizeof(float) * (size_t)nin * n + 16));
  CK(cudaMalloc((void**)&dout, sizeof(float) * (size_t)nout * n + 16));
  cudaMemcpy(din, in, sizeof(float) * (size_t)nin * n, cudaMemcpyHostToDevice);
  const int grid = (n + 127) / 128;
  if (n > 0) {
    if (which == 0) k_selftest_tet<<<grid, 128>>>(din, dout, n);
    else if (which == 5) k_selftest_tet64<<<grid, 128>>>(din, dout, n);
    else if (which == 1) k_selftest_tri<<<grid, 128>>>(din, dout, n);
    else if (which == 6) k_selftest_tet_group<<<grid, 128>>>(din, dout, n);
    else k_selftest_quot<<<grid, 128>>>(din, dout, n);
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(float) * (size_t)nout * n, cudaMemcpyDeviceToHost);
  cudaFree(din);
  cudaFree(dout);
  if (e != cudaSuccess) return std::string("self-test kernel: ") + cudaGetErrorString(e);
  return "";
}

}  // namespace eikgb

// ===========================================================================
// Allocation-free 3D solve (eik_solve3d_noalloc).
//
// Some callers cannot call cudaMalloc: code that runs while another component
// captures the stream into a CUDA graph, real-time or embedded hosts that reserve
// all device memory at start-up, and plugins whose host application owns the
// device memory pool.  This path keeps every device buffer of one solve (the
// block layout and the solver state) in one fixed array in the library's device
// image instead of allocating.  The array is kNoAllocScratchBytes (32 MiB) on
// every GPU that loads the library, for the life of the process.
// ===========================================================================
static __device__ __align__(256) unsigned char g_noalloc_scratch[32u << 20];

namespace eikgb {

constexpr size_t kNoAllocScratchBytes = sizeof(g_noalloc_scratch);

namespace {

// End of an outer iteration without a CUDA graph (the host reads the control
// block between iterations instead of a conditional node).
__global__ void k_close3d_noalloc(DevArgs a) {
  if (threadIdx.x != 0) return;
  Ctl* c = a.ctl;
  c->iter += 1;
  c->nact = c->nnext;
  c->nnext = 0;
  c->nnew = 0;
  c->work_a = c->work_c = 0;
  c->done_d = 0;
}

std::mutex g_noalloc_mutex;
void* g_noalloc_base[64] = {};

// Device address of the scratch array on the current device, looked up once per
// device with that device current.
std::string noalloc_base(void** out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return "device index out of range";
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_base[dev] = p;
  }
  *out = g_noalloc_base[dev];
  return "";
}

// carve `n` elements of T from the scratch cursor (256-byte aligned)
template <typename T>
T* carve_scratch(unsigned char* base, size_t& off, size_t n) {
  off = (off + 255) & ~(size_t)255;
  T* p = reinterpret_cast<T*>(base + off);
  off += sizeof(T) * (n ? n : 1);
  return p;
}

}  // namespace

// CTA size of the allocation-free path's visit kernels.  The regular path picks
// 512 or one thread per slot per handle from its first solves; this path keeps no
// state between calls, so it runs 512 (two CTAs per SM), the size the regular path
// keeps on isotropic meshes such as the jittered cubes.
constexpr int kNoAllocThreads = 512;

std::string solve3d_noalloc(const Layout& L, const std::vector<int>& seeds, int max_iters, float* out_host,
                            cudaStream_t st, int* iterations, size_t* bytes_needed, NoAllocFailure* failure) {
  NoAllocFailure dummy;
  NoAllocFailure& fk = failure ? *failure : dummy;
  fk = NoAllocFailure::kCuda;  // what a CK() return below means
  const int ncoef = 6;
  // byte budget of the layout and the state
  size_t need = 0;
  {
    unsigned char* z = nullptr;
    carve_scratch<BlockDesc>(z, need, L.nb);
    carve_scratch<float>(z, need, L.coef.size());
    carve_scratch<uint16_t>(z, need, L.lv.size());
    carve_scratch<int>(z, need, L.halo_ids.size());
    carve_scratch<int>(z, need, L.nbr_off.size());
    carve_scratch<int>(z, need, L.nbr.size());
    for (int k = 0; k < 2; ++k) carve_scratch<int>(z, need, L.nv);          // vblock, perm
    for (int k = 0; k < 3; ++k) carve_scratch<float>(z, need, L.nv);        // Ta, Tb, out
    for (int k = 0; k < 6; ++k) carve_scratch<int>(z, need, L.nb);          // conv, stamps, lists
    carve_scratch<unsigned char>(z, need, L.nb);                            // visited
    carve_scratch<Ctl>(z, need, 1);
    carve_scratch<int>(z, need, L.nb);                                      // block -> instance
    carve_scratch<int>(z, need, 4);                                         // instance control
  }
  if (bytes_needed) *bytes_needed = need;
  if (need > kNoAllocScratchBytes) {
    fk = NoAllocFailure::kLimit;
    return "mesh too large for the allocation-free path: needs " + std::to_string(need >> 20) +
           " MiB of scratch, the fixed array holds " + std::to_string(kNoAllocScratchBytes >> 20) + " MiB";
  }
  const int max_slots_pad = (L.max_slots + 3) & ~3;
  const int max_local = std::max(L.max_local, 1), max_owned = std::max(L.max_owned, 1);
  const size_t smem = smem_bytes(ncoef, max_slots_pad, max_local, max_owned);
  int dev = 0, maxsm = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (smem + 64 > (size_t)maxsm) {
    fk = NoAllocFailure::kLimit;
    return "block too large for shared memory; use fewer vertices per block";
  }
  void* basev = nullptr;
  std::string e = noalloc_base(&basev);
  if (!e.empty()) return e;
  unsigned char* base = static_cast<unsigned char*>(basev);
  size_t off = 0;
  DevArgs a{};
  BlockDesc* blocks = carve_scratch<BlockDesc>(base, off, L.nb);
  float* coef = carve_scratch<float>(base, off, L.coef.size());
  uint16_t* lv = carve_scratch<uint16_t>(base, off, L.lv.size());
  int* halo = carve_scratch<int>(base, off, L.halo_ids.size());
  int* nbr_off = carve_scratch<int>(base, off, L.nbr_off.size());
  int* nbr = carve_scratch<int>(base, off, L.nbr.size());
  int* vblock = carve_scratch<int>(base, off, L.nv);
  int* perm = carve_scratch<int>(base, off, L.nv);
  float* Ta = carve_scratch<float>(base, off, L.nv);
  float* Tb = carve_scratch<float>(base, off, L.nv);
  float* out = carve_scratch<float>(base, off, L.nv);
  int* conv = carve_scratch<int>(base, off, L.nb);
  int* stampA = carve_scratch<int>(base, off, L.nb);
  int* stampC = carve_scratch<int>(base, off, L.nb);
  int* list0 = carve_scratch<int>(base, off, L.nb);
  int* list1 = carve_scratch<int>(base, off, L.nb);
  int* list_new = carve_scratch<int>(base, off, L.nb);
  unsigned char* visited = carve_scratch<unsigned char>(base, off, L.nb);
  Ctl* ctl = carve_scratch<Ctl>(base, off, 1);
  int* blk_inst = carve_scratch<int>(base, off, L.nb);
  int* inst_ctl = carve_scratch<int>(base, off, 4);

  // inputs into the scratch array; everything that must start at zero is cleared
  // here because the array keeps the previous call's contents
  std::vector<int> vb(L.nv, 0);
  for (int b = 0; b < L.nb; ++b)
    for (int k = 0; k < L.blocks[b].nowned; ++k) vb[L.blocks[b].vbase + k] = b;
  std::vector<float> init(L.nv, kLarge3D);
  std::vector<char> act(L.nb, 0);
  for (int s : seeds) {
    init[L.perm[s]] = 0.0f;
    act[vb[L.perm[s]]] = 1;
  }
  std::vector<int> alist;
  for (int b = 0; b < L.nb; ++b)
    if (act[b]) alist.push_back(b);
  CK(cudaMemcpyAsync(blocks, L.blocks.data(), sizeof(BlockDesc) * L.nb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(coef, L.coef.data(), sizeof(float) * L.coef.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(lv, L.lv.data(), sizeof(uint16_t) * L.lv.size(), cudaMemcpyHostToDevice, st));
  if (!L.halo_ids.empty())
    CK(cudaMemcpyAsync(halo, L.halo_ids.data(), sizeof(int) * L.halo_ids.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(nbr_off, L.nbr_off.data(), sizeof(int) * L.nbr_off.size(), cudaMemcpyHostToDevice, st));
  if (!L.nbr.empty()) CK(cudaMemcpyAsync(nbr, L.nbr.data(), sizeof(int) * L.nbr.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(vblock, vb.data(), sizeof(int) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(perm, L.perm.data(), sizeof(int) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(Ta, init.data(), sizeof(float) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(Tb, init.data(), sizeof(float) * L.nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(conv, 0, sizeof(int) * L.nb, st));
  CK(cudaMemsetAsync(stampA, 0, sizeof(int) * L.nb, st));
  CK(cudaMemsetAsync(stampC, 0, sizeof(int) * L.nb, st));
  CK(cudaMemsetAsync(visited, 0, L.nb, st));
  CK(cudaMemsetAsync(blk_inst, 0, sizeof(int) * L.nb, st));
  CK(cudaMemsetAsync(inst_ctl, 0, sizeof(int) * 4, st));
  if (!alist.empty()) CK(cudaMemcpyAsync(list0, alist.data(), sizeof(int) * alist.size(), cudaMemcpyHostToDevice, st));
  Ctl c{};
  c.max_iters = max_iters;
  c.nact = (int)alist.size();
  CK(cudaMemcpyAsync(ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st));

  a.blocks = blocks; a.coef = coef; a.lv = reinterpret_cast<const uint2*>(lv); a.halo = halo; a.nbr_off = nbr_off;
  a.nbr = nbr; a.vblock = vblock; a.nb = L.nb; a.nv = L.nv; a.Ta = Ta; a.Tb = Tb; a.Tinit = Ta; a.prev = Tb;
  a.conv = conv; a.stampA = stampA; a.stampC = stampC; a.visited = visited; a.list0 = list0; a.list1 = list1;
  a.list_new = list_new; a.ctl = ctl; a.hist = nullptr; a.hist_cap = 0; a.ktime = nullptr; a.ktime_cap = 0;
  a.fim_sweeps = 2; a.max_slots_pad = max_slots_pad; a.max_local = max_local; a.max_owned = max_owned;
  a.blk_inst = blk_inst; a.inst_done = inst_ctl; a.inst_iters = inst_ctl + 1; a.inst_nnext = inst_ctl + 2;
  a.inst_fail = inst_ctl + 3; a.ninst = 1;
  CK(raise_smem_limit((const void*)k_visit3d<false>, smem));
  CK(raise_smem_limit((const void*)k_visit3d<true>, smem));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_visit3d<false>, kNoAllocThreads, smem));
  if (occ < 1) return "visit kernel cannot be resident";
  const int grid = std::min(occ * nsm, std::max(L.nb, 1));
  int iters = 0;
  for (;;) {
    Ctl h{};
    CK(cudaMemcpyAsync(&h, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    iters = h.iter;
    if (h.error) {
      fk = NoAllocFailure::kDevice;
      return "device reported error flags " + std::to_string(h.error);
    }
    if (h.nact == 0 || h.iter >= max_iters) break;
    k_visit3d<false><<<grid, kNoAllocThreads, smem, st>>>(a);
    k_commit3d<<<nsm * 4, 256, 0, st>>>(a);
    k_visit3d<true><<<grid, kNoAllocThreads, smem, st>>>(a);
    k_close3d_noalloc<<<1, 32, 0, st>>>(a);
    CK(cudaGetLastError());
  }
  k_gather_result<<<std::max(1, std::min(1024, (L.nv + 255) / 256)), 256, 0, st>>>(Ta, visited, vblock, perm, L.nv,
                                                                                   3, out);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out_host, out, sizeof(float) * L.nv, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (iterations) *iterations = iters;
  fk = NoAllocFailure::kNone;
  return "";
}

}  // namespace eikgb
