// Complex CSR matvec over coefficient groups, with two epilogues:
//   * AXPBY: y = alpha * A(t) x + beta * y           (qg_spmv_csr)
//   * RK:    Vern7 stage k_s = A(t_s) x_s fused with the next stage's input
//            combination, or with y_front and the WRMS error at the last stage
//            (qg_vern7_stage).
//
// Row partitioning: a sub-warp of LANES threads owns one row; consecutive
// sub-warps own consecutive rows, so operator values and column indices are
// read fully coalesced (each lane reads one 16 B / 8 B value and one 4 B index
// per iteration with streaming cache hints) and the partial dot products are
// combined with warp shuffles.  The gathered vector x stays L2-resident (it is
// at most 1/20 of the operator's bytes at the sizes this targets).  The grid is
// a whole number of waves over the SMs and strides over row blocks.
#include "capi_internal.h"
#include "common.cuh"

namespace qg {

constexpr int SPMV_BLOCK = 256;

enum Epi { EPI_AXPBY = 0, EPI_RK = 1 };

struct AxpbyArgs {
  void* y;
  cplx alpha, beta;
};

struct RkArgs {
  const void* y_prev;
  void* y_front;
  void* k;
  void* ytmp_out;
  int64_t n;
  int stage;
  double dt, atol, rtol;
  double* scratch;
  unsigned int* counter;
  double* result;
};

// Complex multiply-accumulate in the accumulation precision.
__device__ __forceinline__ void cmac_f(float& ar, float& ai, float2 v, float2 x) {
  ar = fmaf(v.x, x.x, ar);
  ar = fmaf(-v.y, x.y, ar);
  ai = fmaf(v.x, x.y, ai);
  ai = fmaf(v.y, x.x, ai);
}
__device__ __forceinline__ void cmac_d(double& ar, double& ai, double2 v, double2 x) {
  ar = fma(v.x, x.x, ar);
  ar = fma(-v.y, x.y, ar);
  ai = fma(v.x, x.y, ai);
  ai = fma(v.y, x.x, ai);
}
__device__ __forceinline__ void cmac_any(double& ar, double& ai, double2 v, double2 x) {
  cmac_d(ar, ai, v, x);
}
__device__ __forceinline__ void cmac_any(float& ar, float& ai, float2 v, float2 x) {
  cmac_f(ar, ai, v, x);
}

// Row dot product of one group for the LANES lanes of a sub-warp; every lane
// returns the full sum.
template <typename VT, typename R, int LANES>
__device__ __forceinline__ cplx row_dot(const int* __restrict__ col, const VT* __restrict__ val,
                                        const VT* __restrict__ x, int s, int e, int lane) {
  R ar = 0, ai = 0;
  int p = s + lane;
  // two independent loads in flight per lane
  for (; p + LANES < e; p += 2 * LANES) {
    VT v0 = ld_stream(val + p), v1 = ld_stream(val + p + LANES);
    int c0 = ld_stream(col + p), c1 = ld_stream(col + p + LANES);
    VT x0 = ld_gather(x + c0), x1 = ld_gather(x + c1);
    cmac_any(ar, ai, v0, x0);
    cmac_any(ar, ai, v1, x1);
  }
  if (p < e) {
    VT v0 = ld_stream(val + p);
    int c0 = ld_stream(col + p);
    cmac_any(ar, ai, v0, ld_gather(x + c0));
  }
#pragma unroll
  for (int o = LANES / 2; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    ai += __shfl_xor_sync(0xffffffffu, ai, o);
  }
  return cplx{(double)ar, (double)ai};
}

// DT: operator / stage / gathered-vector storage type, YDT: state storage type.
template <int DT, int YDT, int LANES, int EPI>
__global__ void __launch_bounds__(SPMV_BLOCK)
    spmv_groups_kernel(qg_csr_groups A, double t, const typename elem<DT>::T* __restrict__ x,
                       AxpbyArgs ax, RkArgs rk) {
  using ST = typename elem<DT>::T;
  using R = typename elem<DT>::R;
  using YT = typename elem<YDT>::T;
  __shared__ cplx coef[QG_MAX_GROUPS];
  __shared__ double red[SPMV_BLOCK / 32];
  const int G = A.n_groups;
  if (threadIdx.x < G) coef[threadIdx.x] = group_coef(A, threadIdx.x, t);
  __syncthreads();

  const int n = (int)A.n_rows;
  const int sub = threadIdx.x / LANES, lane = threadIdx.x % LANES;
  constexpr int RPB = SPMV_BLOCK / LANES;
  const ST* __restrict__ val = static_cast<const ST*>(A.val);
  double err_acc = 0.0;

  for (int base = blockIdx.x * RPB; base < n; base += gridDim.x * RPB) {
    const int row = base + sub;
    const bool valid = row < n;
    cplx acc{0.0, 0.0};
    for (int g = 0; g < G; ++g) {
      const int* rp = A.row_ptr + (size_t)g * (n + 1);
      int s = 0, e = 0;
      if (valid) {
        s = __ldg(rp + row);
        e = __ldg(rp + row + 1);
      }
      cplx d = row_dot<ST, R, LANES>(A.col, val, x, s, e, lane);
      acc = cadd(acc, cmul(coef[g], d));
    }
    if (!valid || lane != 0) continue;

    if constexpr (EPI == EPI_AXPBY) {
      ST* y = static_cast<ST*>(ax.y);
      cplx r = cmul(ax.alpha, acc);
      if (ax.beta.re != 0.0 || ax.beta.im != 0.0) r = cadd(r, cmul(ax.beta, to_c(y[row])));
      y[row] = from_c<ST>(r);
    } else {
      const int s = rk.stage;
      const size_t n64 = (size_t)rk.n;
      ST* k = static_cast<ST*>(rk.k);
      const ST ks_store = from_c<ST>(acc);
      k[(size_t)s * n64 + row] = ks_store;
      const cplx ks = to_c(ks_store);
      const YT* yp = static_cast<const YT*>(rk.y_prev);
      if (s != RK_STEP - 1 && s != RK_EXTRA_STEP - 1) {
        const int nx = s + 1;
        cplx v = to_c(yp[row]);
        for (int j = 0; j <= s; ++j) {
          const double f = rk.dt * VERN7_A[nx][j];
          if (f != 0.0) v = cadd(v, cscale(j == s ? ks : to_c(k[(size_t)j * n64 + row]), f));
        }
        static_cast<ST*>(rk.ytmp_out)[row] = from_c<ST>(v);
      } else if (s == RK_STEP - 1) {
        cplx y = to_c(yp[row]);
        cplx e{0.0, 0.0};
        for (int j = 0; j < RK_STEP; ++j) {
          const cplx kj = (j == s) ? ks : to_c(k[(size_t)j * n64 + row]);
          const double fb = rk.dt * VERN7_B[j];
          if (fb != 0.0) y = cadd(y, cscale(kj, fb));
          const double fe = rk.dt * VERN7_E[j];
          if (fe != 0.0) e = cadd(e, cscale(kj, fe));
        }
        const YT ys = from_c<YT>(y);
        static_cast<YT*>(rk.y_front)[row] = ys;
        const double w = sqrt(cabs2(e)) / (rk.atol + rk.rtol * sqrt(cabs2(to_c(ys))));
        err_acc += w * w;
      }
    }
  }

  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) {
      // deterministic two-level reduction: per-block partials, last block sums
      double bs = block_sum<SPMV_BLOCK>(err_acc, red);
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
        for (int i = threadIdx.x; i < (int)gridDim.x; i += SPMV_BLOCK)
          v += __ldcg(rk.scratch + i);
        // per-thread strided partials summed in a fixed order
        double tot = block_sum<SPMV_BLOCK>(v, red);
        if (threadIdx.x == 0) {
          *rk.result = sqrt(tot / (double)rk.n);
          *rk.counter = 0u;
        }
      }
    }
  }
}

template <int DT, int YDT, int EPI>
static int launch_lanes(int lanes, int grid, cudaStream_t st, const qg_csr_groups& A, double t,
                        const void* x, const AxpbyArgs& ax, const RkArgs& rk) {
  using ST = typename elem<DT>::T;
#define QG_CASE(L)                                                                      \
  case L:                                                                               \
    spmv_groups_kernel<DT, YDT, L, EPI><<<grid, SPMV_BLOCK, 0, st>>>(A, t, (const ST*)x, ax, \
                                                                     rk);               \
    break;
  switch (lanes) {
    QG_CASE(2)
    QG_CASE(4)
    QG_CASE(8)
    QG_CASE(16)
    QG_CASE(32)
    default:
      return set_error(QG_ERR_ARG, "lanes must be one of 2, 4, 8, 16, 32");
  }
#undef QG_CASE
  return check_launch("spmv_groups_kernel");
}

static int grid_for_rows(int64_t n_rows, int lanes) {
  const int rpb = SPMV_BLOCK / lanes;
  int64_t blocks = (n_rows + rpb - 1) / rpb;
  int64_t cap = (int64_t)sm_count() * 8;  // 8 resident 256-thread blocks per SM
  if (cap > qg_scratch_doubles()) cap = qg_scratch_doubles();
  return (int)(blocks < cap ? (blocks < 1 ? 1 : blocks) : cap);
}

static int check_groups(const qg_csr_groups* A) {
  if (!A || !A->row_ptr || !A->col || !A->val) return set_error(QG_ERR_ARG, "null operator");
  if (A->n_groups < 1 || A->n_groups > QG_MAX_GROUPS)
    return set_error(QG_ERR_ARG, "n_groups out of range");
  if (A->n_rows < 0 || A->n_rows >= (int64_t)INT32_MAX || A->n_cols < 0)
    return set_error(QG_ERR_ARG, "bad operator shape");
  if (A->dtype != QG_C128 && A->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "operator dtype must be QG_C128 or QG_C64");
  if (A->coef_code && (!A->coef_start || !A->coef_consts))
    return set_error(QG_ERR_ARG, "coefficient program tables incomplete");
  return QG_OK;
}

}  // namespace qg

using namespace qg;

extern "C" int qg_spmv_csr(const qg_csr_groups* A, double t, const void* x, void* y,
                           double alpha_re, double alpha_im, double beta_re, double beta_im,
                           int lanes, void* stream) {
  int rc = check_groups(A);
  if (rc) return rc;
  if (!x || !y) return set_error(QG_ERR_ARG, "null vector");
  if (A->n_rows == 0) return QG_OK;
  AxpbyArgs ax{y, cplx{alpha_re, alpha_im}, cplx{beta_re, beta_im}};
  RkArgs rk{};
  const int grid = grid_for_rows(A->n_rows, lanes);
  cudaStream_t st = (cudaStream_t)stream;
  if (A->dtype == QG_C128)
    return launch_lanes<QG_C128, QG_C128, EPI_AXPBY>(lanes, grid, st, *A, t, x, ax, rk);
  return launch_lanes<QG_C64, QG_C64, EPI_AXPBY>(lanes, grid, st, *A, t, x, ax, rk);
}

extern "C" int qg_vern7_stage(const qg_csr_groups* A, const qg_rk_buffers* B, int stage,
                              double t_prev, double dt, double atol, double rtol, int lanes,
                              void* stream) {
  int rc = check_groups(A);
  if (rc) return rc;
  if (!B || !B->y_prev || !B->y_front || !B->k || !B->ytmp)
    return set_error(QG_ERR_ARG, "null Runge-Kutta buffer");
  if (stage < 0 || stage >= RK_EXTRA_STEP) return set_error(QG_ERR_ARG, "stage out of range");
  if (B->n != A->n_rows || A->n_rows != A->n_cols)
    return set_error(QG_ERR_ARG, "operator must be square with n rows");
  if (B->stage_dtype != A->dtype)
    return set_error(QG_ERR_UNSUPPORTED, "stage dtype must equal the operator dtype");
  if (stage == RK_STEP - 1 && (!B->scratch || !B->counter || !B->result))
    return set_error(QG_ERR_ARG, "error reduction buffers missing");
  if (B->n == 0) return QG_OK;
  const size_t n = (size_t)B->n;
  const size_t es = B->stage_dtype == QG_C128 ? 16 : 8;
  RkArgs rk{B->y_prev, B->y_front, B->k,
            (char*)B->ytmp + ((stage + 1) & 1) * n * es, B->n, stage, dt, atol, rtol,
            B->scratch, B->counter, B->result};
  AxpbyArgs ax{};
  const int grid = grid_for_rows(A->n_rows, lanes);
  cudaStream_t st = (cudaStream_t)stream;
  const double t = t_prev + VERN7_C_HOST[stage] * dt;
  // Stage 0 gathers y_prev itself when state and stages share a dtype; in the
  // mixed form it gathers ytmp[0], which the caller fills with the rounded
  // y_prev (qg_rk_combine with n_k = 0).
  const bool mixed = B->state_dtype != B->stage_dtype;
  const void* x = (stage == 0 && !mixed) ? B->y_prev
                                         : (const char*)B->ytmp + (stage & 1) * n * es;
  if (B->state_dtype == QG_C128 && B->stage_dtype == QG_C128)
    return launch_lanes<QG_C128, QG_C128, EPI_RK>(lanes, grid, st, *A, t, x, ax, rk);
  if (B->state_dtype == QG_C128 && B->stage_dtype == QG_C64)
    return launch_lanes<QG_C64, QG_C128, EPI_RK>(lanes, grid, st, *A, t, x, ax, rk);
  if (B->state_dtype == QG_C64 && B->stage_dtype == QG_C64)
    return launch_lanes<QG_C64, QG_C64, EPI_RK>(lanes, grid, st, *A, t, x, ax, rk);
  return set_error(QG_ERR_UNSUPPORTED, "unsupported state/stage dtype pair");
}
