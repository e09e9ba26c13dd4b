// Batched, persistent adaptive Vern7: many independent small solves in one
// launch.  Each group of threads (a warp for states up to WARP_MAX_N entries, a
// CTA above that) owns a workspace slot and takes items -- a system solved from
// an initial state, or one Monte-Carlo trajectory -- from an atomic queue; every
// item runs the reference's integrator control flow with its own step size:
//   Explicit_RungeKutta.set_initial_value / _estimate_first_step / integrate /
//   _step_in_err / _compute_step / _prep_dense_out / _interpolate_step /
//   _recompute_safe_step   (qutip/solver/integrator/explicit_rk.pyx:204-467)
// and, for trajectories, MCIntegrator.integrate / _find_collapse_time /
// _do_collapse (qutip/solver/mcsolve.py:245-406) with numpy's PCG64 draws in the
// reference's order.
//
// Replicated control: every thread of a group keeps its own copy of the scalar
// integrator state (times, step sizes, status, dense-output factors, the PCG64
// stream) and takes every decision itself from group reductions that return the
// same bits to every thread (warp XOR butterflies are order-symmetric; the CTA
// reduction sums the per-warp results in one fixed order).  No thread publishes
// control state to the others, so all threads of a group follow one path by
// construction.  Vector data live in the slot's global workspace, ordered by
// group syncs.  The row-parallel work (matvec + fused stage combination, norms,
// expectation values) is spread over the group's threads.
//
// Every loop is bounded: steps per output interval (nsteps), iterations of the
// trajectory loop, bisection tries (norm_steps), jumps (max_jumps); an optional
// host-visible cancel flag is polled at each output time and inside long
// trajectory intervals.
#include <cooperative_groups.h>
#include <cstdio>
#include <mutex>

#include "capi_internal.h"
#include "common.cuh"

namespace qg {

// --------------------------------------------------------------- PCG64 ------
// Published PCG XSL-RR 128/64 generator: s <- s*M + inc (mod 2^128) before each
// output; output rotr64(hi(s) ^ lo(s), s >> 122); random() = (x >> 11) * 2^-53.
struct Pcg {
  unsigned long long hi, lo, ihi, ilo;
};
__device__ inline unsigned long long pcg_next(Pcg& r) {
  const unsigned long long MH = 0x2360ED051FC65DA4ULL, ML = 0x4385DF649FCCF645ULL;
  const unsigned long long lo = r.lo * ML;
  unsigned long long hi = __umul64hi(r.lo, ML) + r.lo * MH + r.hi * ML;
  const unsigned long long nlo = lo + r.ilo;
  hi += r.ihi + (nlo < lo ? 1ULL : 0ULL);
  r.lo = nlo;
  r.hi = hi;
  const unsigned long long x = hi ^ nlo;
  const unsigned rot = (unsigned)(hi >> 58);
  return (x >> rot) | (x << ((64u - rot) & 63u));
}
__device__ inline double pcg_random(Pcg& r) {
  return (double)(pcg_next(r) >> 11) * (1.0 / 9007199254740992.0);
}

// Host-visible flag read with system-scope acquire semantics.
__device__ __forceinline__ int read_flag(const volatile int32_t* p) {
  int v;
  asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Largest state handled by one warp per item; larger states use one CTA per item.
constexpr int WARP_MAX_N = 2048;
constexpr int WARP_BLOCK = 128;   // 4 warps (4 items) per CTA in warp mode
constexpr int CTA_BLOCK = 256;    // threads per item in CTA mode (per CTA in cluster mode)
constexpr int CLUSTER_CTAS = 8;   // CTAs per item in cluster mode (portable cluster size)
// Expectation-value sums an output record gathers behind one pair of group barriers.
constexpr int REC_SLOTS = 8;
// Stage inputs (ytmp, 2 x max_n entries per item) live in shared memory when all
// items of a CTA fit in this many bytes: the matvec gathers of x then hit shared
// memory instead of L1/L2.
constexpr int64_t STAGE_SMEM_CAP = 96 * 1024;
// Iterations of the trajectory loop within one output interval (each advances
// time by one accepted step) before the item stops with QG_TOO_MUCH_WORK.
constexpr int MC_MAX_ITER = 1 << 22;

// ------------------------------------------------------------ workspace -----
__host__ __device__ inline int64_t align256(int64_t b) { return (b + 255) & ~(int64_t)255; }

struct SlotLayout {
  int64_t y, ys, yl, k, ytmp, ctmp, total;
};
__host__ __device__ inline SlotLayout slot_layout(int64_t n, int dt) {
  const int64_t es = dt == QG_C128 ? 16 : 8;
  SlotLayout L;
  L.y = 0;                                  // 2 state buffers (complex128)
  L.ys = L.y + align256(2 * n * 16);        // 2 stage-dtype shadows (mixed form: hi parts)
  L.yl = L.ys + align256(2 * n * es);       // 2 low parts (mixed form only)
  L.k = L.yl + align256(dt == QG_C64 ? 2 * n * 8 : 0);  // 16 stage derivatives
  L.ytmp = L.k + align256(16 * n * es);     // 2 stage inputs
  L.ctmp = L.ytmp + align256(2 * n * es);   // 2 complex128 temporaries (MC)
  L.total = L.ctmp + align256(2 * n * 16);
  return L;
}

// Dynamic shared memory of a CTA holding `groups` items' stage inputs, or 0.
__host__ __device__ inline int64_t stage_smem_bytes(int64_t max_n, int dt, int groups) {
  const int64_t per = align256(2 * max_n * (dt == QG_C128 ? 16 : 8));
  const int64_t b = groups * per;
  return b <= STAGE_SMEM_CAP ? b : 0;
}

__host__ __device__ inline int64_t align16(int64_t b) { return (b + 15) & ~(int64_t)15; }

// Shared-memory bytes of a staged operator (row pointers, columns, values), or 0.
__host__ __device__ inline int64_t op_smem_bytes(const qg_batch& B) {
  if (B.stage_op_entries <= 0) return 0;
  const int64_t es = B.dtype == QG_C128 ? 16 : 8;
  return align16((int64_t)B.stage_op_rp * 4) + align16(B.stage_op_entries * 4) +
         align16(B.stage_op_entries * es);
}

// Copy the single system's generator into shared memory (called by every thread
// of the CTA, once, before the item loop): thread 0 issues three bulk async copies
// completing on one mbarrier; all threads wait at most WAIT_CYCLES and vote.  On
// success the Ctx reads the operator from shared memory; otherwise it keeps the
// global pointers, the fault word queue[2] is set, and `pending` tells the caller
// to drain the copies before the CTA exits.
template <int DT>
__device__ bool stage_operator(const qg_batch& B, unsigned char* smem_op, uint64_t* bar) {
  using ST = typename elem<DT>::T;
  const unsigned brp = (unsigned)align16((int64_t)B.stage_op_rp * 4);
  const unsigned bcol = (unsigned)align16(B.stage_op_entries * 4);
  const unsigned bval = (unsigned)align16(B.stage_op_entries * (int64_t)sizeof(ST));
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(bar, brp + bcol + bval);
    bulk_g2s(smem_op, B.op_rp, brp, bar);
    bulk_g2s(smem_op + brp, B.op_col, bcol, bar);
    bulk_g2s(smem_op + brp + bcol, B.op_val, bval, bar);
  }
  const bool ok = __syncthreads_and(mbar_poll(bar, 0) ? 1 : 0) != 0;
  if (!ok && threadIdx.x == 0) atomicOr(B.queue + 2, 1u);
  return ok;
}

// ----------------------------------------------------------------- groups ----
namespace cgrp = cooperative_groups;

struct WarpGroup {
  static constexpr int SIZE = 32;
  static constexpr bool DEFER = false;  // record sums: shuffles, no barrier to save
  int rank;
  int64_t slot;
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }
  // two sums in one pass: each component summed in the order of sum()
  __device__ __forceinline__ double2 sum2(double a, double b) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    return make_double2(a, b);
  }
  __device__ __forceinline__ int bcast(int v) const { return __shfl_sync(0xffffffffu, v, 0); }
};

template <int BB>
struct CtaGroup {
  static constexpr int SIZE = BB;
  static constexpr bool DEFER = true;  // record sums: put2 / sync / take2
  int rank;
  int64_t slot;
  double* red;  // shared [2 * BB/32]
  int* ibuf;    // shared [1]
  double* rec;  // shared [REC_SLOTS * 2 * BB/32]: warp partials of deferred sums
  // warp partial of deferred sum pair k; the totals are read by take2 after a sync()
  __device__ __forceinline__ void put2(int k, double a, double b) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((rank & 31) == 0) {
      rec[(2 * k) * (BB / 32) + (rank >> 5)] = a;
      rec[(2 * k + 1) * (BB / 32) + (rank >> 5)] = b;
    }
  }
  // sum pair k, each component in the order of sum()
  __device__ __forceinline__ double2 take2(int k) const {
    double ta = 0.0, tb = 0.0;
#pragma unroll
    for (int i = 0; i < BB / 32; ++i) {
      ta += rec[(2 * k) * (BB / 32) + i];
      tb += rec[(2 * k + 1) * (BB / 32) + i];
    }
    return make_double2(ta, tb);
  }
  __device__ __forceinline__ void put_flag(int v) const {
    if (rank == 0) *ibuf = v;
  }
  __device__ __forceinline__ int take_flag() const { return *ibuf; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();  // earlier readers of red are done
    if ((rank & 31) == 0) red[rank >> 5] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < BB / 32; ++i) t += red[i];
    return t;
  }
  // two sums behind one pair of barriers, each component in the order of sum()
  __device__ __forceinline__ double2 sum2(double a, double b) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __syncthreads();
    if ((rank & 31) == 0) {
      red[rank >> 5] = a;
      red[BB / 32 + (rank >> 5)] = b;
    }
    __syncthreads();
    double ta = 0.0, tb = 0.0;
#pragma unroll
    for (int i = 0; i < BB / 32; ++i) {
      ta += red[i];
      tb += red[BB / 32 + i];
    }
    return make_double2(ta, tb);
  }
  __device__ __forceinline__ int bcast(int v) const {
    __syncthreads();
    if (rank == 0) *ibuf = v;
    __syncthreads();
    return *ibuf;
  }
};

// A thread-block cluster of CS CTAs works on one item.  Reductions: each CTA's warp
// partials go to its own shared memory; after a cluster barrier (release/acquire at
// cluster scope, which also orders the slot's global-memory vectors) every thread
// reads all CS x BB/32 partials through distributed shared memory in one fixed
// order, so every thread of the cluster gets the same bits.
template <int BB, int CS>
struct ClusterGroup {
  static constexpr int SIZE = BB * CS;
  static constexpr bool DEFER = true;  // record sums: put2 / sync / take2
  int rank;
  int64_t slot;
  double* red;  // shared [2 * BB/32] of this CTA
  int* ibuf;    // shared [1] of this CTA
  double* rec;  // shared [REC_SLOTS * 2 * BB/32] of this CTA: warp partials
  __device__ __forceinline__ void put2(int k, double a, double b) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
      rec[(2 * k) * (BB / 32) + (threadIdx.x >> 5)] = a;
      rec[(2 * k + 1) * (BB / 32) + (threadIdx.x >> 5)] = b;
    }
  }
  // every CTA's partials through distributed shared memory, in the order of sum()
  __device__ __forceinline__ double2 take2(int k) const {
    cgrp::cluster_group cl = cgrp::this_cluster();
    double ta = 0.0, tb = 0.0;
    for (int c = 0; c < CS; ++c) {
      const double* rr = cl.map_shared_rank(rec, c);
#pragma unroll
      for (int i = 0; i < BB / 32; ++i) {
        ta += rr[(2 * k) * (BB / 32) + i];
        tb += rr[(2 * k + 1) * (BB / 32) + i];
      }
    }
    return make_double2(ta, tb);
  }
  __device__ __forceinline__ void put_flag(int v) const {
    if (rank == 0) *ibuf = v;
  }
  __device__ __forceinline__ int take_flag() const {
    return *cgrp::this_cluster().map_shared_rank(ibuf, 0);
  }
  __device__ __forceinline__ void sync() const { cgrp::this_cluster().sync(); }
  __device__ __forceinline__ double sum(double v) const {
    cgrp::cluster_group cl = cgrp::this_cluster();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    cl.sync();  // earlier readers of every CTA's red are done
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    cl.sync();
    double t = 0.0;
    for (int c = 0; c < CS; ++c) {
      const double* rr = cl.map_shared_rank(red, c);
#pragma unroll
      for (int i = 0; i < BB / 32; ++i) t += rr[i];
    }
    return t;
  }
  // two sums behind one pair of cluster barriers, each component in the order of sum()
  __device__ __forceinline__ double2 sum2(double a, double b) const {
    cgrp::cluster_group cl = cgrp::this_cluster();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    cl.sync();
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = a;
      red[BB / 32 + (threadIdx.x >> 5)] = b;
    }
    cl.sync();
    double ta = 0.0, tb = 0.0;
    for (int c = 0; c < CS; ++c) {
      const double* rr = cl.map_shared_rank(red, c);
#pragma unroll
      for (int i = 0; i < BB / 32; ++i) {
        ta += rr[i];
        tb += rr[BB / 32 + i];
      }
    }
    return make_double2(ta, tb);
  }
  __device__ __forceinline__ int bcast(int v) const {
    cgrp::cluster_group cl = cgrp::this_cluster();
    cl.sync();
    if (rank == 0) *ibuf = v;
    cl.sync();
    const int r = *cl.map_shared_rank(ibuf, 0);
    cl.sync();  // CTA 0's ibuf is read before anyone moves on
    return r;
  }
};

// ---------------------------------------------------------------- context ----
// Per-thread replicated control state of the item being integrated.
struct Ctl {
  double t, t_prev, t_front, dt_safe, dt_int;
  int status, cur, interp_ready, out_front, steps, rhs;
};

// Per-warp factor slice in shared memory (WF_FLOATS floats, 512 B): the stage factors
// (mixed: dt a_j, its low part, dt e_j, its low part as float[16] each; double:
// dt a_j, dt e_j as double[16]) and the combination / dense-output factors bf (double[16],
// dt-scaled) with their float pairs bfh, bfl (mixed form).  Lanes 0-15 of the warp write
// factor j = lane between two __syncwarp(); every lane reads them as broadcasts.  Held
// per thread, the arrays were indexed at run time and lived in local memory (1.6 KB of
// stack per thread, ~1.1e9 local-load sectors in one 4096-trajectory launch).
// The group coefficients at the current stage time follow (double2[8], float2[8]).
constexpr int WF_FLOATS = 128 + 4 * QG_MAX_GROUPS + 2 * QG_MAX_GROUPS;
__device__ __forceinline__ double* wf_bf(float* wf) { return reinterpret_cast<double*>(wf + 64); }
__device__ __forceinline__ float* wf_bfh(float* wf) { return wf + 96; }
__device__ __forceinline__ float* wf_bfl(float* wf) { return wf + 112; }
__device__ __forceinline__ double2* wf_coef(float* wf) {
  return reinterpret_cast<double2*>(wf + 128);
}
__device__ __forceinline__ float2* wf_coef_f(float* wf) {
  return reinterpret_cast<float2*>(wf + 128 + 4 * QG_MAX_GROUPS);
}

template <int DT>
struct Ctx {
  using ST = typename elem<DT>::T;
  const qg_batch* B;
  const qg_batch_system* S;
  int n, d, G;
  double2* y[2];
  ST* ys[2];
  ST* yl[2];  // mixed form: y = ys + yl to about 48 bits, the stage-input base
  ST* k;
  ST* ytmp;
  double2* ctmp[2];
  const ST* opval;        // generator entries: global pool, or the staged copy
  const int* op_col;
  const int* op_rp;
  float* wf;  // this warp's factor and coefficient slice (shared memory)
};

template <typename T>
__device__ __forceinline__ void st2(T* p, double re, double im);
template <>
__device__ __forceinline__ void st2<double2>(double2* p, double re, double im) {
  *p = make_double2(re, im);
}
template <>
__device__ __forceinline__ void st2<float2>(float2* p, double re, double im) {
  *p = make_float2((float)re, (float)im);
}

// Scalar FP64 work of the replicated control is spread over the lanes of each warp
// and shared with shuffles: lane i computes value i, every lane reads the same bits.
// (GB300 runs FP64 at 1/64 of the FP32 rate, so 256 threads each evaluating every
// coefficient program or dense-output polynomial kept the FP64 pipe busy.)
__device__ __forceinline__ int lane_id() { return (int)(threadIdx.x & 31); }
__device__ __forceinline__ double shfl_d(double v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// coefficients of the system's groups at time t: lane g evaluates group g
template <int DT>
__device__ __forceinline__ void load_coef(Ctx<DT>& X, double t) {
  cplx mine{1.0, 0.0};
  if (X.S->coef_off >= 0 && lane_id() < X.G) {
    const int st = __ldg(X.B->coef_start + X.S->coef_off + lane_id());
    mine = eval_coef(X.B->coef_code + st, X.B->coef_consts, t);
  }
  __syncwarp();  // the warp's earlier readers are done
  if (lane_id() < X.G) {
    wf_coef(X.wf)[lane_id()] = make_double2(mine.re, mine.im);
    wf_coef_f(X.wf)[lane_id()] = make_float2((float)mine.re, (float)mine.im);
  }
  __syncwarp();
}

// row r of A(t) x in the compute type
template <int DT, typename XT>
__device__ __forceinline__ void row_matvec(const Ctx<DT>& X, int r, const XT* x,
                                           typename elem<DT>::R& ar, typename elem<DT>::R& ai) {
  using CT = typename elem<DT>::R;
  ar = 0;
  ai = 0;
  const int* rp = X.op_rp + X.S->rp_off + (int64_t)r * X.G;
  for (int g = 0; g < X.G; ++g) {
    const int s = rp[g], e = rp[g + 1];
    CT gr = 0, gi = 0;
    for (int p = s; p < e; ++p) {
      const auto v = X.opval[p];
      const auto xv = x[X.op_col[p]];
      gr = fma((CT)v.x, (CT)xv.x, gr);
      gr = fma(-(CT)v.y, (CT)xv.y, gr);
      gi = fma((CT)v.x, (CT)xv.y, gi);
      gi = fma((CT)v.y, (CT)xv.x, gi);
    }
    CT cr, ci;
    if constexpr (DT == QG_C64) {
      const float2 k = wf_coef_f(X.wf)[g];
      cr = k.x;
      ci = k.y;
    } else {
      const double2 k = wf_coef(X.wf)[g];
      cr = k.x;
      ci = k.y;
    }
    ar += cr * gr - ci * gi;
    ai += cr * gi + ci * gr;
  }
}

// k_j = A(t) x for a stage-dtype input (first-step estimate)
template <int DT, class GT>
__device__ void matvec_to_k(const GT& g, Ctx<DT>& X, Ctl& c, double t,
                            const typename elem<DT>::T* x, int j) {
  using CT = typename elem<DT>::R;
  load_coef(X, t);
  for (int r = g.rank; r < X.n; r += GT::SIZE) {
    CT ar, ai;
    row_matvec(X, r, x, ar, ai);
    st2(X.k + (int64_t)j * X.n + r, (double)ar, (double)ai);
  }
  c.rhs += 1;
  g.sync();
}

// One fused stage: k_s = A(t_prev + c_s dt) x_s and the next stage input, or at
// s == 9 y_front and the WRMS error (returned).  In the mixed form the stage
// input x_{s+1} = y_prev + sum_j dt a_{s+1,j} k_j is accumulated in float-float
// from the complex128 y_prev and rounded once to complex64; the step increment
// is accumulated the same way and added to y_prev in FP64.
template <int DT, class GT>
__device__ __noinline__ double stage(const GT& g, Ctx<DT>& X, Ctl& c, int s, double dt) {
  using ST = typename elem<DT>::T;
  using CT = typename elem<DT>::R;
  constexpr bool MIXED = (DT == QG_C64);
  const bool last = (s == RK_STEP - 1);
  const bool forms_input = !last && s != RK_EXTRA_STEP - 1;
  const int nk = last ? RK_STEP : s + 1;  // k_j that enter the combination
  // factors: FP64 for the double form; float pairs from the hi/lo tableau for the
  // mixed form (no FP64 work per stage); lane j of each warp forms factor j
  const CT* fa;
  const CT* fe;
  const float* fl;
  const float* fel;
  {
    const int j = lane_id();
    __syncwarp();  // the warp's earlier readers of the slice are done
    if constexpr (MIXED) {
      float* w = X.wf;
      if (j < 16) {
        float dh, dl;
        split_f(dt, dh, dl);
        float ah = 0.f, al = 0.f, eh = 0.f, el = 0.f;
        if (j < nk) {
          if (last) {
            ah = VERN7_BH[j];
            al = VERN7_BL[j];
            eh = VERN7_EF[j];
            el = VERN7_EL[j];
          } else if (forms_input) {
            ah = VERN7_AH[s + 1][j];
            al = VERN7_AL[s + 1][j];
          }
        }
        ff_factor(dh, dl, ah, al, w[j], w[16 + j]);
        ff_factor(dh, dl, eh, el, w[32 + j], w[48 + j]);
      }
      fa = reinterpret_cast<const CT*>(w);
      fl = w + 16;
      fe = reinterpret_cast<const CT*>(w + 32);
      fel = w + 48;
    } else {
      double* w = reinterpret_cast<double*>(X.wf);
      if (j < 16) {
        double a = 0.0, e = 0.0;
        if (j < nk) {
          if (last) {
            a = dt * VERN7_B[j];
            e = dt * VERN7_E[j];
          } else if (forms_input) {
            a = dt * VERN7_A[s + 1][j];
          }
        }
        w[j] = a;
        w[16 + j] = e;
      }
      fa = reinterpret_cast<const CT*>(w);
      fe = reinterpret_cast<const CT*>(w + 16);
      fl = fel = nullptr;  // not used by the double form
    }
    __syncwarp();
  }
  load_coef(X, c.t_prev + VERN7_C[s] * dt);
  const int cur = c.cur;
  const ST* x;
  if (s == 0) {
    if constexpr (MIXED) x = X.ys[cur];
    else x = reinterpret_cast<const ST*>(X.y[cur]);
  } else {
    x = X.ytmp + (int64_t)(s & 1) * X.n;
  }
  ST* out = X.ytmp + (int64_t)((s + 1) & 1) * X.n;
  const int64_t n = X.n;
  double err_acc = 0.0;
  for (int r = g.rank; r < X.n; r += GT::SIZE) {
    CT ar, ai;
    row_matvec(X, r, x, ar, ai);
    st2(X.k + s * n + r, (double)ar, (double)ai);
    ST ks;  // the stored k_s entry, without reading it back
    ks.x = ar;
    ks.y = ai;
    if (forms_input) {
      if constexpr (MIXED) {
        float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
        for (int j = 0; j <= s; ++j) {
          if (fa[j] != 0.f || fl[j] != 0.f) {
            const ST kj = (j == s) ? ks : X.k[j * n + r];
            ff_acc(hr, lr, fa[j], fl[j], kj.x);
            ff_acc(hi, li, fa[j], fl[j], kj.y);
          }
        }
        const float2 bh = X.ys[cur][r], bl = X.yl[cur][r];
        out[r] = make_float2(ff_round4(bh.x, bl.x, hr, lr), ff_round4(bh.y, bl.y, hi, li));
      } else {
        CT vr = X.y[cur][r].x, vi = X.y[cur][r].y;
        for (int j = 0; j <= s; ++j) {
          const CT f = fa[j];
          if (f != (CT)0) {
            const ST kj = (j == s) ? ks : X.k[j * n + r];
            vr = fma(f, (CT)kj.x, vr);
            vi = fma(f, (CT)kj.y, vi);
          }
        }
        st2(out + r, (double)vr, (double)vi);
      }
    } else if (last) {
      if constexpr (MIXED) {
        float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
        float erh = 0.f, erl = 0.f, eih = 0.f, eil = 0.f;
        for (int j = 0; j < RK_STEP; ++j) {
          if (fa[j] == 0.f && fl[j] == 0.f && fe[j] == 0.f && fel[j] == 0.f) continue;
          const ST kj = (j == s) ? ks : X.k[j * n + r];
          ff_acc(hr, lr, fa[j], fl[j], kj.x);
          ff_acc(hi, li, fa[j], fl[j], kj.y);
          ff_acc(erh, erl, fe[j], fel[j], kj.x);   // error estimate in float-float
          ff_acc(eih, eil, fe[j], fel[j], kj.y);
        }
        // the once-per-step FP64 state update, then its float-pair shadow
        const double yr = X.y[cur][r].x + ((double)hr + (double)lr);
        const double yi = X.y[cur][r].y + ((double)hi + (double)li);
        X.y[cur ^ 1][r] = make_double2(yr, yi);
        float shr, slr, shi, sli;
        split_f(yr, shr, slr);
        split_f(yi, shi, sli);
        X.ys[cur ^ 1][r] = make_float2(shr, shi);
        X.yl[cur ^ 1][r] = make_float2(slr, sli);
        // WRMS error term in FP64 against the FP64 state (wrmn_error_dense,
        // qutip/core/data/ode.pyx:27-52), written as |e|^2 / (atol + rtol |y|)^2
        const double er = (double)erh + (double)erl, ei = (double)eih + (double)eil;
        err_acc += wrms_term(er * er + ei * ei, yr * yr + yi * yi, X.S->atol, X.S->rtol);
      } else {
        CT er = 0, ei = 0;
        double yr = X.y[cur][r].x, yi = X.y[cur][r].y;
        for (int j = 0; j < RK_STEP; ++j) {
          const double fb = (double)fa[j], fq = (double)fe[j];
          if (fb == 0.0 && fq == 0.0) continue;
          const ST kj = (j == s) ? ks : X.k[j * n + r];
          if (fb != 0.0) {
            yr = fma(fb, (double)kj.x, yr);
            yi = fma(fb, (double)kj.y, yi);
          }
          if (fq != 0.0) {
            er = fma((CT)fq, (CT)kj.x, er);
            ei = fma((CT)fq, (CT)kj.y, ei);
          }
        }
        X.y[cur ^ 1][r] = make_double2(yr, yi);
        // IEEE square roots and division: the complex128 form takes the reference's steps
        // (a 1e-13 change of the error norm moved one of 4096 BH trajectories' jumps)
        const double w = sqrt((double)er * er + (double)ei * ei) /
                         (X.S->atol + X.S->rtol * sqrt(yr * yr + yi * yi));
        err_acc += w * w;
      }
    }
  }
  c.rhs += 1;
  double err = 0.0;
  if (last) err = sqrt(g.sum(err_acc) / (double)X.n);
  g.sync();
  return err;
}

// Mixed form: out = fl32(y_prev + sum_{j<nk} dt a_{row,j} k_j) in float pairs from
// the (ys, yl) base -- the stage input of the first dense-output stage.
template <int DT, class GT>
__device__ void form_input_mixed(const GT& g, Ctx<DT>& X, const Ctl& c, typename elem<DT>::T* out,
                                 int row, int nk, double dt) {
  using ST = typename elem<DT>::T;
  float* fa = X.wf;
  float* fl = X.wf + 16;
  __syncwarp();
  if (lane_id() < 16) {
    const int j = lane_id();
    float dh, dl;
    split_f(dt, dh, dl);
    const float ah = j < nk ? VERN7_AH[row][j] : 0.f, al = j < nk ? VERN7_AL[row][j] : 0.f;
    ff_factor(dh, dl, ah, al, fa[j], fl[j]);
  }
  __syncwarp();
  const int cur = c.cur;
  const int64_t n = X.n;
  for (int r = g.rank; r < X.n; r += GT::SIZE) {
    float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
    for (int j = 0; j < nk; ++j) {
      if (fa[j] != 0.f || fl[j] != 0.f) {
        const ST kj = X.k[j * n + r];
        ff_acc(hr, lr, fa[j], fl[j], kj.x);
        ff_acc(hi, li, fa[j], fl[j], kj.y);
      }
    }
    const float2 bh = X.ys[cur][r], bl = X.yl[cur][r];
    out[r] = make_float2(ff_round4(bh.x, bl.x, hr, lr), ff_round4(bh.y, bl.y, hi, li));
  }
  g.sync();
}

// out = base + sum_{j<nk} bf[j] k_j (bf: the warp's factor slice)
template <int DT, class GT, typename OT, typename BT>
__device__ void combine(const GT& g, Ctx<DT>& X, const Ctl& c, OT* out, const BT* base, int nk) {
  const double* bf = wf_bf(X.wf);
  for (int r = g.rank; r < X.n; r += GT::SIZE) {
    double vr = (double)base[r].x, vi = (double)base[r].y;
    for (int j = 0; j < nk; ++j) {
      const double f = bf[j];
      if (f != 0.0) {
        vr = fma(f, (double)X.k[(int64_t)j * X.n + r].x, vr);
        vi = fma(f, (double)X.k[(int64_t)j * X.n + r].y, vi);
      }
    }
    st2(out + r, vr, vi);
  }
  g.sync();
}

// entry i of the current state: y_front, or y_prev + sum_j bf_j k_j (the mixed
// form sums the increment in float pairs and adds it to y_prev in FP64)
template <int DT>
__device__ __forceinline__ double2 state_at(const Ctx<DT>& X, const Ctl& c, int i) {
  if (c.out_front) return X.y[c.cur ^ 1][i];
  if constexpr (DT == QG_C64) {
    const float* bfh = wf_bfh(X.wf);
    const float* bfl = wf_bfl(X.wf);
    float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
    for (int j = 0; j < RK_EXTRA_STEP; ++j) {
      if (bfh[j] != 0.f || bfl[j] != 0.f) {
        const float2 kj = X.k[(int64_t)j * X.n + i];
        ff_acc(hr, lr, bfh[j], bfl[j], kj.x);
        ff_acc(hi, li, bfh[j], bfl[j], kj.y);
      }
    }
    return make_double2(X.y[c.cur][i].x + ((double)hr + (double)lr),
                        X.y[c.cur][i].y + ((double)hi + (double)li));
  } else {
    const double* bf = wf_bf(X.wf);
    double vr = X.y[c.cur][i].x, vi = X.y[c.cur][i].y;
    for (int j = 0; j < RK_EXTRA_STEP; ++j) {
      const double f = bf[j];
      if (f != 0.0) {
        vr = fma(f, (double)X.k[(int64_t)j * X.n + i].x, vr);
        vi = fma(f, (double)X.k[(int64_t)j * X.n + i].y, vi);
      }
    }
    return make_double2(vr, vi);
  }
}

template <int DT, class GT>
__device__ double state_norm2(const GT& g, const Ctx<DT>& X, const Ctl& c) {
  double acc = 0.0;
  for (int r = g.rank; r < X.n; r += GT::SIZE) {
    const double2 v = state_at(X, c, r);
    acc += v.x * v.x + v.y * v.y;
  }
  return g.sum(acc);
}

template <class GT, typename T>
__device__ double vec_norm2(const GT& g, const T* v, int n) {
  double acc = 0.0;
  for (int r = g.rank; r < n; r += GT::SIZE)
    acc += (double)v[r].x * (double)v[r].x + (double)v[r].y * (double)v[r].y;
  return g.sum(acc);
}

// ------------------------------------------------------ integrator (RK) ------
// set_initial_value (explicit_rk.pyx:204-230) with _estimate_first_step (:232-276)
template <int DT, class GT>
__device__ __noinline__ void set_initial(const GT& g, Ctx<DT>& X, Ctl& c, const double2* src, double t) {
  using ST = typename elem<DT>::T;
  constexpr bool MIXED = (DT == QG_C64);
  const int cur = c.cur;
  for (int r = g.rank; r < X.n; r += GT::SIZE) {
    const double2 v = src[r];
    X.y[cur][r] = v;
    X.y[cur ^ 1][r] = v;
    if constexpr (MIXED) {
      float hr, lr, hi, li;
      split_f(v.x, hr, lr);
      split_f(v.y, hi, li);
      X.ys[cur][r] = X.ys[cur ^ 1][r] = make_float2(hr, hi);
      X.yl[cur][r] = X.yl[cur ^ 1][r] = make_float2(lr, li);
    }
  }
  g.sync();
  c.t = c.t_prev = c.t_front = t;
  c.dt_int = 0.0;
  c.interp_ready = 0;
  c.out_front = 1;
  c.status = QG_NORMAL;
  const double atol = X.S->atol, rtol = X.S->rtol;
  double norm = sqrt(vec_norm2(g, X.y[cur], X.n));
  const double tol = atol + norm * rtol;
  const ST* x0;
  if constexpr (MIXED) x0 = X.ys[cur];
  else x0 = reinterpret_cast<const ST*>(X.y[cur]);
  matvec_to_k(g, X, c, t, x0, 0);
  if (norm <= atol) norm = 1.0;
  double tmp = sqrt(vec_norm2(g, X.k, X.n));
  double fact = 1.0;
  for (int i = 1; i <= RK_ORDER; ++i) fact *= i;
  double dt1;
  if (tmp >= atol * 1e-6)
    dt1 = pow(tol * fact * pow(norm, (double)RK_ORDER), 1.0 / (RK_ORDER + 1)) / tmp;
  else
    dt1 = pow(tol * fact, 1.0 / (RK_ORDER + 1)) * norm * 0.5;
  const double t1 = t + dt1 / 100;
  __syncwarp();
  if (lane_id() < 16) wf_bf(X.wf)[lane_id()] = lane_id() == 0 ? dt1 / 100 : 0.0;
  __syncwarp();
  ST* yt = X.ytmp + X.n;
  combine(g, X, c, yt, x0, 1);
  matvec_to_k(g, X, c, t1, yt, 1);
  tmp = sqrt(vec_norm2(g, X.k + X.n, X.n));
  double dt2;
  if (tmp >= atol * 1e-6)
    dt2 = pow(tol * fact * pow(norm, (double)RK_ORDER), 1.0 / (RK_ORDER + 1)) / tmp;
  else
    dt2 = dt1;
  c.dt_safe = fmax(1e-15, fmin(dt1, dt2));  // min_step defaults to 1e-15 (explicit_rk.pyx:133)
}

// _prep_dense_out (explicit_rk.pyx:399-410)
template <int DT, class GT>
__device__ __noinline__ void prep_dense_out(const GT& g, Ctx<DT>& X, Ctl& c) {
  using ST = typename elem<DT>::T;
  const double dt = c.dt_int;
  ST* x10 = X.ytmp + (int64_t)(RK_STEP & 1) * X.n;
  if constexpr (DT == QG_C64) {
    form_input_mixed(g, X, c, x10, RK_STEP, RK_STEP, dt);
  } else {
    __syncwarp();
    if (lane_id() < 16)
      wf_bf(X.wf)[lane_id()] = lane_id() < RK_STEP ? dt * VERN7_A[RK_STEP][lane_id()] : 0.0;
    __syncwarp();
    combine(g, X, c, x10, X.y[c.cur], RK_STEP);
  }
  for (int s = RK_STEP; s < RK_EXTRA_STEP; ++s) stage(g, X, c, s, dt);
  c.interp_ready = 1;
}

// dense-output factors at t (Horner in tau, explicit_rk.pyx:412-430); lane i
// evaluates factor i
template <int DT>
__device__ __forceinline__ void set_interp(const Ctx<DT>& X, Ctl& c, double t) {
  const double tau = (t - c.t_prev) / c.dt_int;
  double mine = 0.0;
  float mh = 0.f, ml = 0.f;
  if (lane_id() < RK_EXTRA_STEP) {
    double acc = 0.0;
    for (int j = DENSE_ORDER - 1; j >= 0; --j) {
      acc += VERN7_BI[lane_id()][j];
      acc *= tau;
    }
    mine = c.dt_int * acc;
    split_f(mine, mh, ml);
  }
  __syncwarp();
  if (lane_id() < RK_EXTRA_STEP) {
    wf_bf(X.wf)[lane_id()] = mine;
    wf_bfh(X.wf)[lane_id()] = mh;
    wf_bfl(X.wf)[lane_id()] = ml;
  }
  __syncwarp();
  c.out_front = 0;
  c.t = t;
}

// _step_in_err (explicit_rk.pyx:333-356) with interpolate=True time steps;
// returns the number of trial steps
template <int DT, class GT>
__device__ int step_in_err(const GT& g, Ctx<DT>& X, Ctl& c, int nsteps_left) {
  int nsteps = 0;
  while (true) {
    const double dt = c.dt_safe;
    double err = 0.0;
    for (int s = 0; s < RK_STEP; ++s) {
      const double e = stage(g, X, c, s, dt);
      if (s == RK_STEP - 1) err = e;
    }
    c.t_front = c.t_prev + dt;
    c.dt_int = dt;
    // _recompute_safe_step (explicit_rk.pyx:451-467) in FP64 for both forms.  Every
    // thread holds the same err; lane 0 of each warp takes the pow and shares it, so
    // the FP64 pipe sees one pow per warp, not one per thread.
    double factor;
    if (err == 0.0) {
      factor = 10.0;
    } else {
      double mine = 0.0;
      if (lane_id() == 0) mine = fmax(0.2, fmin(10.0, 0.9 * pow(err, -1.0 / (RK_ORDER + 1))));
      factor = shfl_d(mine, 0);
    }
    c.dt_safe = fmax(1e-15, dt * factor);
    c.interp_ready = 0;
    c.steps += 1;
    ++nsteps;
    if (dt == 1e-15 && err > 1.0) {
      c.status = QG_DT_UNDERFLOW;
      break;
    }
    if (nsteps > nsteps_left) {
      c.status = QG_TOO_MUCH_WORK;
      break;
    }
    if (err < 1.0) break;
  }
  return nsteps;
}

// integrate (explicit_rk.pyx:278-331); afterwards the state at c.t is y_front
// (out_front) or the dense output with factors bf.
template <int DT, class GT>
__device__ void integrate(const GT& g, Ctx<DT>& X, Ctl& c, double t, bool step) {
  if (t == c.t) return;
  if (t < c.t_prev) {
    c.status = QG_OUTSIDE_RANGE;
    return;
  }
  if (t < c.t_front) {
    if (!c.interp_ready) prep_dense_out(g, X, c);
    set_interp(X, c, t);
    return;
  }
  c.status = QG_NORMAL;
  if (step && c.t < c.t_front && t > c.t_front) t = c.t_front;
  int nsteps_left = X.S->nsteps;
  while (c.t_front < t && c.status >= 0) {
    c.cur ^= 1;  // y_prev <- y_front (buffer swap)
    c.t_prev = c.t_front;
    nsteps_left -= step_in_err(g, X, c, nsteps_left);
    if (step) break;
  }
  if (c.status < 0) return;
  if (c.t_front > t) {
    prep_dense_out(g, X, c);
    set_interp(X, c, t);
  } else {
    c.out_front = 1;
    c.t = c.t_front;
  }
}

// ------------------------------------------------------------- outputs ------
// expectation values of the current state into out[0..ne] (raw; host normalises).
// A ket is interpolated once into ctmp[0] and every e_op reads it there; a density
// matrix is read entry by entry (the e_ops touch a small part of it).
// CTA and cluster groups gather the warp partials of up to REC_SLOTS sums behind one
// pair of barriers (a barrier pair per sum made most of the cost of an output for
// large items in a cluster).  Returns the host cancel flag, read once per record by
// rank 0 and shared behind the same barriers (0 without a flag).
template <int DT, class GT>
__device__ __noinline__ int record(const GT& g, const Ctx<DT>& X, const Ctl& c, double2* out,
                                   bool ket, const volatile int32_t* cancel) {
  const int ne = X.S->n_eops;
  const int d = X.d;
  const double2* psi = X.ctmp[0];
  if (ket) {
    for (int r = g.rank; r < X.n; r += GT::SIZE) X.ctmp[0][r] = state_at(X, c, r);
    g.sync();
  }
  int flag = 0;
  for (int e0 = 0; e0 <= ne; e0 += REC_SLOTS) {
    const int e1 = min(ne + 1, e0 + REC_SLOTS);
    for (int e = e0; e < e1; ++e) {
      double ar = 0.0, ai = 0.0;
      if (e < ne) {
        const int* rp = X.B->eop_rp + X.S->eop_rp_off + (int64_t)e * (d + 1);
        for (int r = g.rank; r < d; r += GT::SIZE) {
          const int s = __ldg(rp + r), en = __ldg(rp + r + 1);
          double sr = 0.0, si = 0.0;
          for (int p = s; p < en; ++p) {
            const int col = __ldg(X.B->eop_col + p);
            const double vr = __ldg(X.B->eop_val + 2 * p), vi = __ldg(X.B->eop_val + 2 * p + 1);
            const double2 z = ket ? psi[col] : state_at(X, c, col + r * d);
            sr += vr * z.x - vi * z.y;
            si += vr * z.y + vi * z.x;
          }
          if (ket) {
            const double2 pr = psi[r];
            const double tr = pr.x * sr + pr.y * si, ti = pr.x * si - pr.y * sr;
            sr = tr;
            si = ti;
          }
          ar += sr;
          ai += si;
        }
      } else if (ket) {  // the norm
        for (int r = g.rank; r < X.n; r += GT::SIZE) {
          const double2 z = psi[r];
          ar += z.x * z.x + z.y * z.y;
        }
      } else {  // the trace
        for (int r = g.rank; r < d; r += GT::SIZE) {
          const double2 z = state_at(X, c, r + r * d);
          ar += z.x;
          ai += z.y;
        }
      }
      if constexpr (GT::DEFER) {
        g.put2(e - e0, ar, ai);
      } else {
        const double2 t = g.sum2(ar, ai);
        if (g.rank == 0) out[e] = t;
      }
    }
    if constexpr (GT::DEFER) {
      const bool final_chunk = e1 == ne + 1;
      if (final_chunk && cancel) g.put_flag(g.rank == 0 ? read_flag(cancel) : 0);
      g.sync();
      if (final_chunk && cancel) flag = g.take_flag();
      if (g.rank == 0)
        for (int e = e0; e < e1; ++e) out[e] = g.take2(e - e0);
      if (!final_chunk) g.sync();  // rank 0 has read the partials before they are reused
    }
  }
  if constexpr (!GT::DEFER) {
    if (cancel) flag = g.bcast(g.rank == 0 ? read_flag(cancel) : 0);
  }
  g.sync();
  return flag;
}

// ||c_i(t) psi||^2 for psi in ctmp[0]; optionally store c_i(t) psi in ctmp[1].
// c_i(t) = f_i(t) C_i for a time-dependent collapse operator (the product with f_i after
// the row sum, as the reference's QobjEvo matmul scales a term's product).
template <int DT, class GT>
__device__ double cop_apply(const GT& g, Ctx<DT>& X, int i, bool store, double t) {
  const int d = X.d;
  const int* rp = X.B->cop_rp + X.S->cop_rp_off + (int64_t)i * (d + 1);
  const bool scaled = X.S->cop_coef_off >= 0;
  cplx f{1.0, 0.0};
  if (scaled) {
    const int st = __ldg(X.B->coef_start + X.S->cop_coef_off + i);
    f = eval_coef(X.B->coef_code + st, X.B->coef_consts, t);
  }
  double acc = 0.0;
  for (int r = g.rank; r < d; r += GT::SIZE) {
    const int s = __ldg(rp + r), e = __ldg(rp + r + 1);
    double sr = 0.0, si = 0.0;
    for (int p = s; p < e; ++p) {
      const int col = __ldg(X.B->cop_col + p);
      const double vr = __ldg(X.B->cop_val + 2 * p), vi = __ldg(X.B->cop_val + 2 * p + 1);
      const double2 z = X.ctmp[0][col];
      sr += vr * z.x - vi * z.y;
      si += vr * z.y + vi * z.x;
    }
    if (scaled) {
      const double fr = f.re * sr - f.im * si;
      si = f.re * si + f.im * sr;
      sr = fr;
    }
    if (store) X.ctmp[1][r] = make_double2(sr, si);
    acc += sr * sr + si * si;
  }
  const double tot = g.sum(acc);
  g.sync();
  return tot;
}

// ------------------------------------------------------------------ item -----
template <int DT, class GT>
__device__ void run_item(const GT& g, const qg_batch& B, Ctx<DT>& X, int item) {
  const qg_batch_item I = B.items[item];
  // reject an item the workspace or the kernel's fixed-size arrays cannot hold
  // (the host builder never produces one; a raw C caller might)
  if (I.system < 0 || I.system >= B.n_systems || B.systems[I.system].n > B.max_n ||
      B.systems[I.system].n <= 0 || B.systems[I.system].n_groups > QG_MAX_GROUPS ||
      B.systems[I.system].n_groups <= 0) {
    if (g.rank == 0) {
      int32_t* st = B.status + 4 * (int64_t)item;
      st[0] = QG_BAD_ITEM;
      st[1] = st[2] = st[3] = 0;
    }
    g.sync();
    return;
  }
  const qg_batch_system* S = B.systems + I.system;
  X.S = S;
  X.n = S->n;
  X.d = S->d;
  X.G = S->n_groups;
  const bool ket = S->kind == 1;
  double2* out = reinterpret_cast<double2*>(B.out + 2 * I.out_off);
  const double* tl = B.tlist + S->tlist_off;
  const int ne1 = S->n_eops + 1;
  Ctl c;
  c.cur = 0;
  c.rhs = 0;
  c.steps = 0;
  Pcg rng{I.rng_state_hi, I.rng_state_lo, I.rng_inc_hi, I.rng_inc_lo};
  // MCIntegrator.set_state draws first, above the improved-sampling floor
  // (r * (1 - floor) + floor, rounded as the host computes it)
  const double floor_p = I.jump_prob_floor;
  double target = ket ? __dadd_rn(__dmul_rn(pcg_random(rng), 1.0 - floor_p), floor_p) : 0.0;
  int njumps = 0;
  set_initial(g, X, c, reinterpret_cast<const double2*>(B.y0) + I.y0_off, tl[0]);
  int cancelled = record(g, X, c, out, ket, B.cancel);
  for (int o = 1; o < S->n_out && c.status >= 0; ++o) {
    const double t = tl[o];
    if (B.progress && g.rank == 0)
      B.progress[g.slot] =
          ((int64_t)item << 32) | (int64_t)(unsigned)o;
    if (cancelled) {  // the flag as the last record read it
      c.status = QG_TIMEOUT;
      break;
    }
    if (!ket) {
      integrate(g, X, c, t, false);
    } else {
      // MCIntegrator.integrate (mcsolve.py:286-302)
      double t_old = c.t;
      double norm_old = state_norm2(g, X, c);
      int iters = 0;
      while (t_old < t && c.status >= 0) {
        if (++iters > MC_MAX_ITER) {
          c.status = QG_TOO_MUCH_WORK;
          break;
        }
        if (B.cancel && (iters & 63) == 0) {
          const int f = g.bcast(g.rank == 0 ? read_flag(B.cancel) : 0);
          if (f) {
            c.status = QG_TIMEOUT;
            break;
          }
        }
        if (B.debug && g.rank == 0) {  // ring of the last 8 loop states per slot
          double* dbg = B.debug + g.slot * 64 + (iters & 7) * 8;
          dbg[0] = (double)item;
          dbg[1] = (double)o;
          dbg[2] = c.t;
          dbg[3] = c.t_prev;
          dbg[4] = c.t_front;
          dbg[5] = c.dt_safe;
          dbg[6] = (double)iters;
          dbg[7] = target;
        }
        integrate(g, X, c, t, true);
        if (c.status < 0) break;
        const double t_step = c.t;
        const double nrm = state_norm2(g, X, c);
        if (nrm > target) {
          t_old = t_step;
          norm_old = nrm;
          continue;
        }
        // _find_collapse_time (mcsolve.py:321-369)
        double tp = t_old, tf = t_step, no = norm_old, nn = nrm, t_guess = tf;
        int tries = 0;
        while (tries < B.norm_steps) {
          ++tries;
          if ((tf - tp) < B.norm_t_tol) {
            t_guess = tf;
            break;
          }
          const double dtb = tf - tp;
          double ratio = log(no / target) / log(no / nn);
          if (ratio < B.norm_min_step) ratio = B.norm_min_step;
          if (ratio > 1.0 - B.norm_min_step) ratio = 1.0 - B.norm_min_step;
          t_guess = tp + dtb * ratio;
          if ((t_guess - tp) < B.norm_t_tol) t_guess = tp + B.norm_t_tol;
          integrate(g, X, c, t_guess, true);
          if (c.status < 0) break;
          const double n2 = state_norm2(g, X, c);
          if (fabs(target - n2) < B.norm_tol * target) break;
          if (n2 < target) {
            tf = t_guess;
            nn = n2;
          } else {
            tp = t_guess;
            no = n2;
          }
        }
        if (c.status < 0) break;
        if (tries >= B.norm_steps) {
          c.status = QG_NORM_SEARCH_FAILED;
          break;
        }
        // _do_collapse (mcsolve.py:371-406): psi = state at t_guess
        for (int r = g.rank; r < X.n; r += GT::SIZE) X.ctmp[0][r] = state_at(X, c, r);
        g.sync();
        int which = 0;
        const int nc = S->n_cops;
        if (nc > 1) {
          // sum of the jump probabilities, then the reference's walk over them;
          // each probability is recomputed (bit-identical, no per-operator array)
          double sum = 0.0;
          for (int i = 0; i < nc; ++i) sum += cop_apply(g, X, i, false, t_guess);
          double tgt = sum * pcg_random(rng) - cop_apply(g, X, 0, false, t_guess);
          while (tgt > 0 && which < nc - 1) {
            ++which;
            tgt -= cop_apply(g, X, which, false, t_guess);
          }
        }
        const double new_norm = sqrt(cop_apply(g, X, which, true, t_guess));
        if (new_norm < B.mc_corr_eps) {
          // the jump is numerical noise: renormalise the state, keep the target
          const double pn = sqrt(vec_norm2(g, X.ctmp[0], X.n));
          for (int r = g.rank; r < X.n; r += GT::SIZE)
            X.ctmp[1][r] = make_double2(X.ctmp[0][r].x / pn, X.ctmp[0][r].y / pn);
        } else {
          for (int r = g.rank; r < X.n; r += GT::SIZE)
            X.ctmp[1][r] = make_double2(X.ctmp[1][r].x / new_norm, X.ctmp[1][r].y / new_norm);
          if (njumps >= B.max_jumps) {
            c.status = QG_JUMP_OVERFLOW;
            break;
          }
          if (g.rank == 0) {
            B.jump_t[(int64_t)item * B.max_jumps + njumps] = t_guess;
            B.jump_which[(int64_t)item * B.max_jumps + njumps] = which;
          }
          ++njumps;
          target = pcg_random(rng);
        }
        g.sync();
        set_initial(g, X, c, X.ctmp[1], t_guess);
        t_old = c.t;
        norm_old = 1.0;
      }
    }
    if (c.status < 0) break;
    cancelled = record(g, X, c, out + (int64_t)o * ne1, ket, B.cancel);
  }
  if (g.rank == 0) {
    int32_t* st = B.status + 4 * (int64_t)item;
    st[0] = c.status < 0 ? c.status : 0;
    st[1] = c.steps;
    st[2] = c.rhs;
    st[3] = njumps;
  }
  g.sync();
}

template <int DT>
__device__ __forceinline__ void use_staged(Ctx<DT>& X, const qg_batch& B, unsigned char* smem_op) {
  using ST = typename elem<DT>::T;
  const int64_t brp = align16((int64_t)B.stage_op_rp * 4);
  const int64_t bcol = align16(B.stage_op_entries * 4);
  X.op_rp = reinterpret_cast<const int*>(smem_op);
  X.op_col = reinterpret_cast<const int*>(smem_op + brp);
  X.opval = reinterpret_cast<const ST*>(smem_op + brp + bcol);
}

template <int DT>
__device__ __forceinline__ void bind_slot(Ctx<DT>& X, const qg_batch& B, int64_t slot_index) {
  using ST = typename elem<DT>::T;
  const SlotLayout L = slot_layout(B.max_n, DT);
  char* slot = static_cast<char*>(B.work) + slot_index * L.total;
  X.B = &B;
  X.opval = static_cast<const ST*>(B.op_val);
  X.op_col = B.op_col;
  X.op_rp = B.op_rp;
  X.y[0] = reinterpret_cast<double2*>(slot + L.y);
  X.y[1] = X.y[0] + B.max_n;
  X.ys[0] = reinterpret_cast<ST*>(slot + L.ys);
  X.ys[1] = X.ys[0] + B.max_n;
  X.yl[0] = reinterpret_cast<ST*>(slot + L.yl);
  X.yl[1] = X.yl[0] + B.max_n;
  X.k = reinterpret_cast<ST*>(slot + L.k);
  X.ytmp = reinterpret_cast<ST*>(slot + L.ytmp);
  X.ctmp[0] = reinterpret_cast<double2*>(slot + L.ctmp);
  X.ctmp[1] = X.ctmp[0] + B.max_n;
}

// the group that finishes last resets the queue words for the next launch
__device__ __forceinline__ void finish_queue(const qg_batch& B, unsigned int n_groups) {
  __threadfence();
  if (atomicAdd(B.queue + 1, 1u) == n_groups - 1) {
    B.queue[0] = 0u;
    B.queue[1] = 0u;
  }
}

// One warp per item; slot = global warp index (n_slots warps own slots).
template <int DT>
__global__ void __launch_bounds__(WARP_BLOCK, 4) batch_warp_kernel(qg_batch B) {
  extern __shared__ __align__(256) unsigned char stage_smem[];
  __shared__ __align__(8) uint64_t op_bar;
  __shared__ __align__(16) float wf_s[WARP_BLOCK / 32][WF_FLOATS];
  const int64_t slot = (int64_t)blockIdx.x * (WARP_BLOCK / 32) + (threadIdx.x >> 5);
  WarpGroup g{(int)(threadIdx.x & 31), slot};
  const unsigned int n_groups = gridDim.x * (WARP_BLOCK / 32);
  const int64_t in_bytes = stage_smem_bytes(B.max_n, DT, WARP_BLOCK / 32);
  unsigned char* smem_op = stage_smem + in_bytes;
  bool staged = false, pending = false;
  if (B.stage_op_entries > 0) {
    staged = stage_operator<DT>(B, smem_op, &op_bar);
    pending = !staged;
  }
  if (slot < B.n_slots) {
    Ctx<DT> X;
    bind_slot(X, B, slot);
    X.wf = wf_s[threadIdx.x >> 5];
    if (staged) use_staged(X, B, smem_op);
    if (in_bytes > 0)
      X.ytmp = reinterpret_cast<typename elem<DT>::T*>(
          stage_smem + (threadIdx.x >> 5) * (stage_smem_bytes(B.max_n, DT, 1)));
    while (true) {
      int it = 0;
      if (g.rank == 0) {
        it = (int)atomicAdd(B.queue, 1u);
        if (B.cancel && read_flag(B.cancel)) it = B.n_items;  // stop taking work
      }
      it = g.bcast(it);
      if (it >= B.n_items) break;
      run_item(g, B, X, it);
    }
  }
  if (g.rank == 0) finish_queue(B, n_groups);
  if (pending && threadIdx.x == 0) (void)mbar_poll(&op_bar, 0);  // drain before exit
}

// One CTA of BB threads per item; slot = block index.
template <int DT, int BB>
__global__ void __launch_bounds__(BB, 65536 / (BB * 128)) batch_cta_kernel(qg_batch B) {
  __shared__ double red[2 * (BB / 32)];
  __shared__ int ibuf;
  __shared__ double rec[REC_SLOTS * 2 * (BB / 32)];
  extern __shared__ __align__(256) unsigned char stage_smem[];
  __shared__ __align__(8) uint64_t op_bar;
  __shared__ __align__(16) float wf_s[BB / 32][WF_FLOATS];
  CtaGroup<BB> g{(int)threadIdx.x, (int64_t)blockIdx.x, red, &ibuf, rec};
  Ctx<DT> X;
  bind_slot(X, B, blockIdx.x);
  X.wf = wf_s[threadIdx.x >> 5];
  const int64_t in_bytes = stage_smem_bytes(B.max_n, DT, 1);
  if (in_bytes > 0) X.ytmp = reinterpret_cast<typename elem<DT>::T*>(stage_smem);
  unsigned char* smem_op = stage_smem + in_bytes;
  bool pending = false;
  if (B.stage_op_entries > 0) {
    if (stage_operator<DT>(B, smem_op, &op_bar)) use_staged(X, B, smem_op);
    else pending = true;
  }
  while (true) {
    int it = 0;
    if (g.rank == 0) {
      it = (int)atomicAdd(B.queue, 1u);
      if (B.cancel && read_flag(B.cancel)) it = B.n_items;
    }
    it = g.bcast(it);
    if (it >= B.n_items) break;
    run_item(g, B, X, it);
  }
  if (g.rank == 0) finish_queue(B, gridDim.x);
  if (pending && threadIdx.x == 0) (void)mbar_poll(&op_bar, 0);  // drain before exit
}

// One cluster of CLUSTER_CTAS CTAs per item; slot = cluster index.
template <int DT>
__global__ void __launch_bounds__(CTA_BLOCK, 1) batch_cluster_kernel(qg_batch B) {
  __shared__ double red[2 * (CTA_BLOCK / 32)];
  __shared__ int ibuf;
  cgrp::cluster_group cl = cgrp::this_cluster();
  const int crank = (int)cl.block_rank();
  const int64_t slot = blockIdx.x / CLUSTER_CTAS;
  __shared__ __align__(16) float wf_s[CTA_BLOCK / 32][WF_FLOATS];
  __shared__ double rec[REC_SLOTS * 2 * (CTA_BLOCK / 32)];
  ClusterGroup<CTA_BLOCK, CLUSTER_CTAS> g{crank * CTA_BLOCK + (int)threadIdx.x, slot, red, &ibuf,
                                          rec};
  Ctx<DT> X;
  bind_slot(X, B, slot);
  X.wf = wf_s[threadIdx.x >> 5];
  while (true) {
    int it = 0;
    if (g.rank == 0) {
      it = (int)atomicAdd(B.queue, 1u);
      if (B.cancel && read_flag(B.cancel)) it = B.n_items;
    }
    it = g.bcast(it);
    if (it >= B.n_items) break;
    run_item(g, B, X, it);
  }
  if (g.rank == 0) finish_queue(B, gridDim.x / CLUSTER_CTAS);
  g.sync();  // no CTA leaves while another may still read its shared memory
}

static bool warp_mode(int64_t max_n, int group) {
  return group == QG_GROUP_WARP || (group == QG_GROUP_AUTO && max_n <= WARP_MAX_N);
}

// Opt a kernel into `bytes` of dynamic shared memory.  The 48 KB default limit counts the
// kernel's static shared memory too (the per-warp factor slices: up to 5.6 KB), so any
// dynamic size is opted in: 45.7 KB of staged vectors plus the slices had 0 blocks per SM.
template <typename K>
static bool allow_smem(K kernel, int64_t bytes) {
  if (bytes <= 0) return true;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
         cudaSuccess;
}

static bool valid_group(int group) {
  return group == QG_GROUP_AUTO || group == QG_GROUP_WARP || group == QG_GROUP_CTA ||
         group == QG_GROUP_CLUSTER || group == QG_GROUP_CTA128;
}

// Kernel, block size and items per CTA of a warp or CTA group shape.
using BatchKernel = void (*)(qg_batch);
struct Shape {
  BatchKernel kernel;
  int block, groups_per_cta;
};
static Shape shape_of(int64_t max_n, int dtype, int group) {
  const bool c64 = dtype == QG_C64;
  if (warp_mode(max_n, group))
    return {c64 ? batch_warp_kernel<QG_C64> : batch_warp_kernel<QG_C128>, WARP_BLOCK,
            WARP_BLOCK / 32};
  if (group == QG_GROUP_CTA128)
    return {c64 ? batch_cta_kernel<QG_C64, 128> : batch_cta_kernel<QG_C128, 128>, 128, 1};
  return {c64 ? batch_cta_kernel<QG_C64, CTA_BLOCK> : batch_cta_kernel<QG_C128, CTA_BLOCK>,
          CTA_BLOCK, 1};
}

static cudaLaunchConfig_t cluster_config(int n_clusters, cudaStream_t st, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)n_clusters * CLUSTER_CTAS, 1, 1);
  cfg.blockDim = dim3(CTA_BLOCK, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CLUSTER_CTAS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace qg

using namespace qg;

// ------------------------------------------------- allocation-free variant --
// Workspace and queue words of qg_batch_vern7_noalloc.  Loading the library
// reserves these on every GPU it is used on, until the process exits.
namespace qg {
constexpr size_t NOALLOC_WORK_BYTES = (size_t)QG_NOALLOC_WORK_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_work[NOALLOC_WORK_BYTES];
static __device__ __align__(256) unsigned int g_noalloc_queue[4];

// Device addresses of the arrays above, looked up once per device with that
// device current (the host-side names are stand-ins, not device addresses).
struct NoallocAddr {
  void* work = nullptr;
  unsigned int* queue = nullptr;
};
static NoallocAddr g_noalloc_addr[64];
static std::mutex g_noalloc_mu;

static int noalloc_setup(int dev, NoallocAddr& out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocAddr& a = g_noalloc_addr[dev];
  if (!a.work) {
    void* w = nullptr;
    void* q = nullptr;
    if (cudaGetSymbolAddress(&w, g_noalloc_work) != cudaSuccess || !w)
      return set_error(QG_ERR_CUDA, "cudaGetSymbolAddress failed for the static workspace");
    if (cudaGetSymbolAddress(&q, g_noalloc_queue) != cudaSuccess || !q)
      return set_error(QG_ERR_CUDA, "cudaGetSymbolAddress failed for the static queue words");
    a.work = w;
    a.queue = static_cast<unsigned int*>(q);
  }
  out = a;
  return QG_OK;
}
}  // namespace qg

extern "C" int qg_batch_vern7_noalloc(const qg_batch* B, void* stream) {
  if (!B || !B->systems || !B->items || !B->op_rp || !B->op_col || !B->op_val || !B->tlist ||
      !B->y0 || !B->out || !B->status)
    return set_error(QG_ERR_ARG, "null batch pointer");
  if (B->dtype != QG_C128 && B->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "batch dtype must be QG_C128 or QG_C64");
  if (B->n_items < 0 || B->max_n <= 0) return set_error(QG_ERR_ARG, "bad batch sizes");
  if (B->max_jumps > 0 && (!B->jump_t || !B->jump_which))
    return set_error(QG_ERR_ARG, "jump record buffers missing");
  const int64_t slot = slot_layout(B->max_n, B->dtype).total;
  if (slot > (int64_t)NOALLOC_WORK_BYTES)
    return set_error(QG_ERR_ARG,
                     "max_n too large: one workspace slot exceeds the static workspace "
                     "(QG_NOALLOC_WORK_BYTES); use qg_batch_vern7 with caller-owned memory");
  if (B->n_items == 0) return QG_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error(QG_ERR_CUDA, "no current CUDA device");
  NoallocAddr a;
  int rc = noalloc_setup(dev, a);
  if (rc) return rc;
  int occ = qg_batch_launch_slots(B);
  if (occ <= 0) return occ < 0 ? occ : set_error(QG_ERR_CUDA, "no resident CTA");
  int64_t slots = (int64_t)NOALLOC_WORK_BYTES / slot;
  if (slots > occ) slots = occ;
  if (slots > B->n_items) slots = B->n_items;
  qg_batch b = *B;
  b.work = a.work;
  b.queue = a.queue;
  b.n_slots = (int32_t)slots;
  cudaStream_t st = (cudaStream_t)stream;
  // the queue words must start at zero (a previous launch leaves them zero; clear anyway)
  if (cudaMemsetAsync(a.queue, 0, 4 * sizeof(unsigned int), st) != cudaSuccess)
    return set_error(QG_ERR_CUDA, "clearing the static queue words failed");
  return qg_batch_vern7(&b, stream);
}

extern "C" int qg_batch_noalloc_staging_fault(void* stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error(QG_ERR_CUDA, "no current CUDA device");
  NoallocAddr a;
  int rc = noalloc_setup(dev, a);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned int v = 0;
  if (cudaMemcpyFromSymbolAsync(&v, g_noalloc_queue, sizeof(v), 2 * sizeof(unsigned int),
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return set_error(QG_ERR_CUDA, "reading the static queue words failed");
  return v != 0 ? 1 : 0;
}

extern "C" int64_t qg_batch_slot_bytes(int64_t max_n, int dtype) {
  return slot_layout(max_n, dtype).total;
}

// Dynamic shared memory of a launch: stage inputs plus the staged operator.
static int64_t launch_smem(const qg_batch& B) {
  if (B.group == QG_GROUP_CLUSTER) return 0;
  const Shape sh = shape_of(B.max_n, B.dtype, B.group);
  return stage_smem_bytes(B.max_n, B.dtype, sh.groups_per_cta) + op_smem_bytes(B);
}

constexpr int64_t MAX_DYN_SMEM = 227 * 1024;

static int group_slots(int64_t max_n, int dtype, int group, int64_t smem) {
  if (!valid_group(group))
    return set_error(QG_ERR_ARG,
                     "group must be one of QG_GROUP_AUTO/WARP/CTA/CLUSTER/CTA128");
  int per_sm = 0;
  cudaError_t e;
  if (group == QG_GROUP_CLUSTER) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config(1, nullptr, attr);
    int clusters = 0;
    e = dtype == QG_C64
            ? cudaOccupancyMaxActiveClusters(&clusters, batch_cluster_kernel<QG_C64>, &cfg)
            : cudaOccupancyMaxActiveClusters(&clusters, batch_cluster_kernel<QG_C128>, &cfg);
    if (e != cudaSuccess || clusters <= 0) {
      char msg[160];
      snprintf(msg, sizeof(msg), "cluster occupancy query failed (%s, %d clusters)",
               e == cudaSuccess ? "no error" : cudaGetErrorString(e), clusters);
      return set_error(QG_ERR_CUDA, msg);
    }
    return clusters;
  }
  if (smem > MAX_DYN_SMEM) return set_error(QG_ERR_ARG, "staged data exceed shared memory");
  const Shape sh = shape_of(max_n, dtype, group);
  if (!allow_smem(sh.kernel, smem)) return set_error(QG_ERR_CUDA, "shared-memory opt-in failed");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sh.kernel, sh.block, smem);
  if (e != cudaSuccess || per_sm <= 0) {
    char msg[200];
    snprintf(msg, sizeof(msg),
             "occupancy query failed (%s; group %d, block %d, %lld bytes of shared memory)",
             e == cudaSuccess ? "0 blocks per SM" : cudaGetErrorString(e), group, sh.block,
             (long long)smem);
    return set_error(QG_ERR_CUDA, msg);
  }
  // slots are warps in warp mode, CTAs otherwise
  return sm_count() * per_sm * sh.groups_per_cta;
}

extern "C" int qg_batch_group_slots(int64_t max_n, int dtype, int group) {
  if (!valid_group(group)) return group_slots(max_n, dtype, group, 0);  // reports the error
  const int64_t smem =
      group == QG_GROUP_CLUSTER
          ? 0
          : stage_smem_bytes(max_n, dtype, shape_of(max_n, dtype, group).groups_per_cta);
  return group_slots(max_n, dtype, group, smem);
}

extern "C" int qg_batch_launch_slots(const qg_batch* B) {
  if (!B) return set_error(QG_ERR_ARG, "null batch pointer");
  return group_slots(B->max_n, B->dtype, B->group, launch_smem(*B));
}

extern "C" int64_t qg_batch_smem_bytes(const qg_batch* B) {
  if (!B) return set_error(QG_ERR_ARG, "null batch pointer");
  return launch_smem(*B);
}

extern "C" int qg_batch_max_slots(int64_t max_n, int dtype) {
  return qg_batch_group_slots(max_n, dtype, QG_GROUP_AUTO);
}

extern "C" int qg_batch_vern7(const qg_batch* B, void* stream) {
  if (!B || !B->systems || !B->items || !B->op_rp || !B->op_col || !B->op_val || !B->tlist ||
      !B->y0 || !B->out || !B->status || !B->work || !B->queue)
    return set_error(QG_ERR_ARG, "null batch pointer");
  if (B->dtype != QG_C128 && B->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "batch dtype must be QG_C128 or QG_C64");
  if (B->n_items < 0 || B->n_slots <= 0 || B->max_n <= 0)
    return set_error(QG_ERR_ARG, "bad batch sizes");
  if (B->max_jumps > 0 && (!B->jump_t || !B->jump_which))
    return set_error(QG_ERR_ARG, "jump record buffers missing");
  if (!valid_group(B->group))
    return set_error(QG_ERR_ARG,
                     "group must be one of QG_GROUP_AUTO/WARP/CTA/CLUSTER/CTA128");
  if (B->stage_op_entries > 0 &&
      (B->group == QG_GROUP_CLUSTER || B->n_systems != 1 || B->stage_op_rp <= 0))
    return set_error(QG_ERR_ARG,
                     "operator staging needs one system and a warp or CTA group");
  if (launch_smem(*B) > MAX_DYN_SMEM)
    return set_error(QG_ERR_ARG, "staged data exceed shared memory");
  if (B->n_items == 0) return QG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (B->group == QG_GROUP_CLUSTER) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config(B->n_slots, st, attr);
    const cudaError_t e = B->dtype == QG_C64
                              ? cudaLaunchKernelEx(&cfg, batch_cluster_kernel<QG_C64>, *B)
                              : cudaLaunchKernelEx(&cfg, batch_cluster_kernel<QG_C128>, *B);
    if (e != cudaSuccess) return set_error(QG_ERR_CUDA, "cluster launch failed");
    return check_launch("batch_cluster_kernel");
  }
  const Shape sh = shape_of(B->max_n, B->dtype, B->group);
  const int64_t smem = launch_smem(*B);
  if (!allow_smem(sh.kernel, smem)) return set_error(QG_ERR_CUDA, "shared-memory opt-in failed");
  const int grid = (B->n_slots + sh.groups_per_cta - 1) / sh.groups_per_cta;
  sh.kernel<<<grid, sh.block, smem, st>>>(*B);
  return check_launch("batch_vern7 (warp or CTA groups)");
}
