// The fused Vern7 stage epilogue shared by the stage kernels (sparse, matrix-free and
// dense): complex helpers, the AXPBY / Runge-Kutta epilogue arguments, the per-element
// epilogue (k_s store and the next stage input, or y_front and the WRMS error term), the
// deterministic grid reduction of the error, and the host-side stage preparation.
#pragma once
#include "capi_internal.h"
#include "common.cuh"

namespace qg {

enum Epi { EPI_AXPBY = 0, EPI_RK = 1 };

// ------------------------------------------------------- complex of type CT --
template <typename CT>
struct cx {
  CT re, im;
};
template <typename CT>
__device__ __forceinline__ cx<CT> ld_cx(const double2* p) {
  double2 v = *p;
  return cx<CT>{(CT)v.x, (CT)v.y};
}
template <typename CT>
__device__ __forceinline__ cx<CT> ld_cx(const float2* p) {
  float2 v = *p;
  return cx<CT>{(CT)v.x, (CT)v.y};
}
__device__ __forceinline__ void st_cx(double2* p, cx<double> v) { *p = make_double2(v.re, v.im); }
__device__ __forceinline__ void st_cx(double2* p, cx<float> v) {
  *p = make_double2((double)v.re, (double)v.im);
}
__device__ __forceinline__ void st_cx(float2* p, cx<float> v) { *p = make_float2(v.re, v.im); }
__device__ __forceinline__ void st_cx(float2* p, cx<double> v) {
  *p = make_float2((float)v.re, (float)v.im);
}
template <typename CT>
__device__ __forceinline__ cx<CT> cx_mul(cx<CT> a, cx<CT> b) {
  return cx<CT>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename CT>
__device__ __forceinline__ cx<CT> cx_add(cx<CT> a, cx<CT> b) {
  return cx<CT>{a.re + b.re, a.im + b.im};
}
// acc += f * k for real f
template <typename CT>
__device__ __forceinline__ void cx_axpy(cx<CT>& acc, CT f, cx<CT> k) {
  acc.re = fma(f, k.re, acc.re);
  acc.im = fma(f, k.im, acc.im);
}

struct AxpbyArgs {
  void* y;
  double alpha_re, alpha_im, beta_re, beta_im;
};

// Host-formed stage factors: fa = dt * a[s+1][0..s] (s < 9, 10 <= s < 15) or
// dt * b (s == 9); fe = dt * e (s == 9).  Zero factors are skipped, as the
// reference's iadd_data skips them (explicit_rk.pyx:34-44).
struct RkArgs {
  const void* y_prev;
  void* y_front;
  const void* y_prev_s;
  void* y_front_s;
  void* k;
  void* ytmp_out;
  int64_t n;
  int stage;
  double atol, rtol;
  double* scratch;
  unsigned int* counter;
  double* result;
  double fa_d[16], fe_d[16];
  float fa_f[16], fe_f[16];
  float fe_l[16];  // fe_d - fe_f: the error weights as float pairs (mixed form)
  // bit j set where fa_d[j] / fe_d[j] is nonzero: the factor loops test these integer
  // masks, not the factors (a floating-point compare per row would run on the FP64 pipe)
  unsigned int nz_a, nz_e;
};


template <typename CT>
__device__ __forceinline__ CT fa(const RkArgs& rk, int j);
template <>
__device__ __forceinline__ double fa<double>(const RkArgs& rk, int j) { return rk.fa_d[j]; }
template <>
__device__ __forceinline__ float fa<float>(const RkArgs& rk, int j) { return rk.fa_f[j]; }
template <typename CT>
__device__ __forceinline__ CT fe(const RkArgs& rk, int j);
template <>
__device__ __forceinline__ double fe<double>(const RkArgs& rk, int j) { return rk.fe_d[j]; }
template <>
__device__ __forceinline__ float fe<float>(const RkArgs& rk, int j) { return rk.fe_f[j]; }

// ---------------------------------------------------------------- epilogue --
// DT: stage dtype (operator, k, ytmp); YDT: state dtype.  CT = elem<DT>::R.
template <int DT, int YDT, int EPI>
__device__ __forceinline__ void epilogue(int row, cx<typename elem<DT>::R> acc,
                                         const AxpbyArgs& ax, const RkArgs& rk, double& err_acc) {
  using ST = typename elem<DT>::T;
  using YT = typename elem<YDT>::T;
  using CT = typename elem<DT>::R;
  if constexpr (EPI == EPI_AXPBY) {
    ST* y = static_cast<ST*>(ax.y);
    cx<CT> r = cx_mul(cx<CT>{(CT)ax.alpha_re, (CT)ax.alpha_im}, acc);
    if (ax.beta_re != 0.0 || ax.beta_im != 0.0)
      r = cx_add(r, cx_mul(cx<CT>{(CT)ax.beta_re, (CT)ax.beta_im}, ld_cx<CT>(y + row)));
    st_cx(y + row, r);
  } else {
    const int s = rk.stage;
    const size_t n64 = (size_t)rk.n;
    ST* k = static_cast<ST*>(rk.k);
    st_cx(k + (size_t)s * n64 + row, acc);
    const cx<CT> ks = ld_cx<CT>(k + (size_t)s * n64 + row);  // the stored (rounded) k_s
    constexpr bool MIXED = (DT != YDT);
    // The factor loops are unrolled over compile-time indices (the bound s is a runtime
    // value): indexed at run time, the factor arrays of the kernel parameters would be
    // copied to local memory by every thread.
    if (s != RK_STEP - 1 && s != RK_EXTRA_STEP - 1) {
      // next stage input: base + sum_{j<=s} fa_j k_j, in the reference's order
      cx<CT> v;
      if constexpr (MIXED)
        v = ld_cx<CT>(static_cast<const ST*>(rk.y_prev_s) + row);
      else
        v = ld_cx<CT>(static_cast<const YT*>(rk.y_prev) + row);
#pragma unroll
      for (int j = 0; j < RK_EXTRA_STEP - 1; ++j) {
        if (j > s) break;
        if ((rk.nz_a >> j) & 1u)
          cx_axpy(v, fa<CT>(rk, j), j == s ? ks : ld_cx<CT>(k + (size_t)j * n64 + row));
      }
      st_cx(static_cast<ST*>(rk.ytmp_out) + row, v);
    } else if (s == RK_STEP - 1) {
      cx<CT> e{0, 0};
      double ymag2 = 0.0;
      if constexpr (MIXED) {
        cx<CT> inc{0, 0};
        float erh = 0.f, erl = 0.f, eih = 0.f, eil = 0.f;
#pragma unroll
        for (int j = 0; j < RK_STEP; ++j) {
          const bool ub = (rk.nz_a >> j) & 1u, uq = (rk.nz_e >> j) & 1u;
          if (!ub && !uq) continue;
          const cx<CT> kj = (j == s) ? ks : ld_cx<CT>(k + (size_t)j * n64 + row);
          if (ub) cx_axpy(inc, fa<CT>(rk, j), kj);
          if (uq) {  // the error estimate in float-float
            ff_acc(erh, erl, fe<CT>(rk, j), rk.fe_l[j], (float)kj.re);
            ff_acc(eih, eil, fe<CT>(rk, j), rk.fe_l[j], (float)kj.im);
          }
        }
        // FP64 state update of the step; FP32 shadow for the next stages
        const double2 yp = static_cast<const double2*>(rk.y_prev)[row];
        const double2 yf = make_double2(yp.x + (double)inc.re, yp.y + (double)inc.im);
        static_cast<double2*>(rk.y_front)[row] = yf;
        static_cast<float2*>(rk.y_front_s)[row] = make_float2((float)yf.x, (float)yf.y);
        // WRMS error term in FP64 against the FP64 state (wrmn_error_dense,
        // qutip/core/data/ode.pyx:27-52), written as |e|^2 / (atol + rtol |y|)^2
        const double er = (double)erh + (double)erl, ei = (double)eih + (double)eil;
        err_acc += wrms_term(er * er + ei * ei, yf.x * yf.x + yf.y * yf.y, rk.atol, rk.rtol);
        return;
      } else {
        // reference order: y_front = y_prev, then += fb_j k_j term by term
        cx<CT> y = ld_cx<CT>(static_cast<const YT*>(rk.y_prev) + row);
#pragma unroll
        for (int j = 0; j < RK_STEP; ++j) {
          const bool ub = (rk.nz_a >> j) & 1u, uq = (rk.nz_e >> j) & 1u;
          if (!ub && !uq) continue;
          const cx<CT> kj = (j == s) ? ks : ld_cx<CT>(k + (size_t)j * n64 + row);
          if (ub) cx_axpy(y, fa<CT>(rk, j), kj);
          if (uq) cx_axpy(e, fe<CT>(rk, j), kj);
        }
        st_cx(static_cast<YT*>(rk.y_front) + row, y);
        const cx<CT> ys = ld_cx<CT>(static_cast<const YT*>(rk.y_front) + row);
        ymag2 = (double)ys.re * ys.re + (double)ys.im * ys.im;
      }
      // wrmn_error_dense (qutip/core/data/ode.pyx:27-52) as |e|^2 / (atol + rtol |y|)^2,
      // with IEEE square root and division: the complex128 form takes the reference's steps
      const double sc = rk.atol + rk.rtol * sqrt(ymag2);
      err_acc += ((double)e.re * e.re + (double)e.im * e.im) / (sc * sc);
    }
  }
}

// Deterministic grid reduction of the stage-9 error (FP64): per-block partials,
// the last block to finish sums them in index order.
template <int BLOCK>
__device__ __forceinline__ void finish_error(const RkArgs& rk, double err_acc, double* red) {
  double bs = block_sum<BLOCK>(err_acc, red);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    rk.scratch[blockIdx.x] = bs;
    __threadfence();
    unsigned int done = atomicAdd(rk.counter, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double v = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) v += __ldcg(rk.scratch + i);
    double tot = block_sum<BLOCK>(v, red);
    if (threadIdx.x == 0) {
      *rk.result = sqrt(tot / (double)rk.n);
      *rk.counter = 0u;
    }
  }
}

// Stage arguments of the fused Vern7 stage: the RK buffers, the factors dt * a_ij
// (dt * b_j and dt * e_j at the last stage) and the stage input x.
static inline int prepare_stage(const qg_rk_buffers* B, int op_dtype, int64_t n_rows, int stage,
                         double dt, double atol, double rtol, RkArgs& rk, const void*& x) {
  if (!B || !B->y_prev || !B->y_front || !B->k || !B->ytmp)
    return set_error(QG_ERR_ARG, "null Runge-Kutta buffer");
  if (stage < 0 || stage >= RK_EXTRA_STEP) return set_error(QG_ERR_ARG, "stage out of range");
  if (B->n != n_rows) return set_error(QG_ERR_ARG, "operator must be square with n rows");
  if (B->stage_dtype != op_dtype)
    return set_error(QG_ERR_UNSUPPORTED, "stage dtype must equal the operator dtype");
  const bool mixed = B->state_dtype != B->stage_dtype;
  if (mixed && (!B->y_prev_s || !B->y_front_s))
    return set_error(QG_ERR_ARG, "mixed form needs y_prev_s and y_front_s");
  if (stage == RK_STEP - 1 && (!B->scratch || !B->counter || !B->result))
    return set_error(QG_ERR_ARG, "error reduction buffers missing");
  if (!((B->state_dtype == QG_C128 && B->stage_dtype == QG_C128) ||
        (B->state_dtype == QG_C128 && B->stage_dtype == QG_C64) ||
        (B->state_dtype == QG_C64 && B->stage_dtype == QG_C64)))
    return set_error(QG_ERR_UNSUPPORTED, "unsupported state/stage dtype pair");
  const size_t n = (size_t)B->n;
  const size_t es = B->stage_dtype == QG_C128 ? 16 : 8;
  rk = RkArgs{};
  rk.y_prev = B->y_prev;
  rk.y_front = B->y_front;
  rk.y_prev_s = B->y_prev_s;
  rk.y_front_s = B->y_front_s;
  rk.k = B->k;
  rk.ytmp_out = (char*)B->ytmp + ((stage + 1) & 1) * n * es;
  rk.n = B->n;
  rk.stage = stage;
  rk.atol = atol;
  rk.rtol = rtol;
  rk.scratch = B->scratch;
  rk.counter = B->counter;
  rk.result = B->result;
  // factors dt * tableau, formed in double and rounded once for the FP32 paths
  for (int j = 0; j < 16; ++j) {
    double a = 0.0, e = 0.0;
    if (stage == RK_STEP - 1) {
      if (j < RK_STEP) {
        a = dt * VERN7_B_HOST[j];
        e = dt * VERN7_E_HOST[j];
      }
    } else if (stage + 1 < RK_EXTRA_STEP && j <= stage) {
      a = dt * VERN7_A_HOST[stage + 1][j];
    }
    rk.fa_d[j] = a;
    rk.fe_d[j] = e;
    rk.fa_f[j] = (float)a;
    rk.fe_f[j] = (float)e;
    rk.fe_l[j] = (float)(e - (double)rk.fe_f[j]);
    if (a != 0.0) rk.nz_a |= 1u << j;
    if (e != 0.0) rk.nz_e |= 1u << j;
  }
  x = stage == 0 ? (mixed ? B->y_prev_s : B->y_prev) : (const char*)B->ytmp + (stage & 1) * n * es;
  return QG_OK;
}

}  // namespace qg
