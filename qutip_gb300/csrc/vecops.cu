// Vector kernels around the matvec: Runge-Kutta combinations, FP64 norms,
// expectation values of e_ops on (lazily interpolated) states, the Dia matvec
// and the multi-vector CSR product.
#include "capi_internal.h"
#include "common.cuh"

namespace qg {

constexpr int VEC_BLOCK = 256;

template <int DT>
__device__ __forceinline__ cplx ld_c(const void* p, size_t i) {
  return to_c(static_cast<const typename elem<DT>::T*>(p)[i]);
}

// Entry i of base + sum_j f_j k_j.
template <int BDT, int KDT>
__device__ __forceinline__ cplx view_at(const qg_state_view& v, size_t i) {
  cplx r = ld_c<BDT>(v.base, i);
  const size_t n = (size_t)v.n;
  for (int j = 0; j < v.n_k; ++j) {
    const double f = v.f[j];
    if (f != 0.0) r = cadd(r, cscale(ld_c<KDT>(v.k, (size_t)j * n + i), f));
  }
  return r;
}

// out = base + sum_j f_j k_j.  Complex128 stages: FP64, term by term in the
// reference's order.  Complex64 stages: the increment is summed in FP32 (GB300's
// FP64 rate is a small fraction of FP32) and added to a complex128 base in FP64.
template <int BDT, int KDT, int ODT>
__global__ void __launch_bounds__(VEC_BLOCK) combine_kernel(qg_state_view v, void* out) {
  using OT = typename elem<ODT>::T;
  __shared__ float ff[16];
  if (threadIdx.x < 16) ff[threadIdx.x] = (float)v.f[threadIdx.x];
  __syncthreads();
  OT* o = static_cast<OT*>(out);
  const size_t n = (size_t)v.n;
  for (size_t i = (size_t)blockIdx.x * VEC_BLOCK + threadIdx.x; i < n;
       i += (size_t)gridDim.x * VEC_BLOCK) {
    if constexpr (KDT == QG_C128) {
      o[i] = from_c<OT>(view_at<BDT, KDT>(v, i));
    } else {
      const float2* k = static_cast<const float2*>(v.k);
      float ir = 0.f, ii = 0.f;
      if constexpr (BDT == QG_C64) {
        const float2 b = static_cast<const float2*>(v.base)[i];
        ir = b.x;
        ii = b.y;
      }
      for (int j = 0; j < v.n_k; ++j) {
        const float f = ff[j];
        if (f != 0.f) {
          const float2 kj = k[(size_t)j * n + i];
          ir = fmaf(f, kj.x, ir);
          ii = fmaf(f, kj.y, ii);
        }
      }
      if constexpr (BDT == QG_C64) {
        o[i] = from_c<OT>(cplx{(double)ir, (double)ii});
      } else {
        const double2 b = static_cast<const double2*>(v.base)[i];
        o[i] = from_c<OT>(cplx{b.x + (double)ir, b.y + (double)ii});
      }
    }
  }
}

template <int DT>
__global__ void __launch_bounds__(VEC_BLOCK)
    norm2_kernel(const void* x, int64_t n, double* scratch, unsigned int* counter,
                 double* result) {
  __shared__ double red[VEC_BLOCK / 32];
  __shared__ bool last;
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * VEC_BLOCK + threadIdx.x; i < (size_t)n;
       i += (size_t)gridDim.x * VEC_BLOCK)
    acc += cabs2(ld_c<DT>(x, i));
  double bs = block_sum<VEC_BLOCK>(acc, red);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = bs;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double v = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += VEC_BLOCK) v += __ldcg(scratch + i);
    double tot = block_sum<VEC_BLOCK>(v, red);
    if (threadIdx.x == 0) {
      *result = tot;
      *counter = 0u;
    }
  }
}

// One block per operator (blockIdx.x < G) plus one block for the trace/norm.
template <int BDT, int KDT, int ODT, bool KET>
__global__ void __launch_bounds__(VEC_BLOCK)
    expect_kernel(qg_csr_groups ops, int64_t d, qg_state_view v, double* out) {
  using OT = typename elem<ODT>::T;
  __shared__ double red[VEC_BLOCK / 32];
  const int g = blockIdx.x;
  const int G = ops.n_groups;
  double ar = 0.0, ai = 0.0;
  if (g < G) {
    const int n = (int)ops.n_rows;
    const OT* val = static_cast<const OT*>(ops.val);
    for (int r = threadIdx.x; r < n; r += VEC_BLOCK) {
      const int i = rp_index(ops, g, r);
      const int s = ops.row_ptr[i], e = ops.row_ptr[i + 1];
      if (s == e) continue;
      cplx acc{0.0, 0.0};
      for (int p = s; p < e; ++p) {
        const int c = ops.col[p];
        // dm: tr(op rho) = sum_r sum_c op[r,c] rho[c,r], rho[c,r] at c + r*d (F order)
        // ket: sum_r conj(psi_r) sum_c op[r,c] psi_c
        const size_t idx = KET ? (size_t)c : (size_t)c + (size_t)r * (size_t)d;
        acc = cadd(acc, cmul(to_c(val[p]), view_at<BDT, KDT>(v, idx)));
      }
      if (KET) {
        cplx pr = view_at<BDT, KDT>(v, (size_t)r);
        acc = cmul(cplx{pr.re, -pr.im}, acc);
      }
      ar += acc.re;
      ai += acc.im;
    }
  } else {
    const int64_t m = KET ? v.n : d;
    for (int64_t r = threadIdx.x; r < m; r += VEC_BLOCK) {
      if (KET) {
        ar += cabs2(view_at<BDT, KDT>(v, (size_t)r));
      } else {
        cplx z = view_at<BDT, KDT>(v, (size_t)r + (size_t)r * (size_t)d);
        ar += z.re;
        ai += z.im;
      }
    }
  }
  double sr = block_sum<VEC_BLOCK>(ar, red);
  double si = block_sum<VEC_BLOCK>(ai, red);
  if (threadIdx.x == 0) {
    out[2 * g] = sr;
    out[2 * g + 1] = si;
  }
}

template <int DT>
__global__ void __launch_bounds__(VEC_BLOCK)
    dia_kernel(qg_dia A, const void* x, void* y, cplx alpha, cplx beta) {
  using T = typename elem<DT>::T;
  const T* data = static_cast<const T*>(A.data);
  const T* xv = static_cast<const T*>(x);
  T* yv = static_cast<T*>(y);
  for (int64_t r = (int64_t)blockIdx.x * VEC_BLOCK + threadIdx.x; r < A.n_rows;
       r += (int64_t)gridDim.x * VEC_BLOCK) {
    cplx acc{0.0, 0.0};
    for (int dg = 0; dg < A.n_diags; ++dg) {
      const int64_t c = r + __ldg(A.offsets + dg);
      if (c < 0 || c >= A.n_cols) continue;
      acc = cadd(acc, cmul(to_c(__ldg(data + (size_t)dg * A.n_cols + c)), to_c(__ldg(xv + c))));
    }
    cplx o = cmul(alpha, acc);
    if (beta.re != 0.0 || beta.im != 0.0) o = cadd(o, cmul(beta, to_c(yv[r])));
    yv[r] = from_c<T>(o);
  }
}

// Multi-vector product: 8 lanes per row, up to 4 columns per pass.
constexpr int MM_LANES = 8, MM_COLS = 4;
template <int DT>
__global__ void __launch_bounds__(VEC_BLOCK)
    spmm_kernel(qg_csr_groups A, double t, const void* X, void* Y, int64_t n_vec, int64_t ld,
                cplx alpha, cplx beta) {
  using T = typename elem<DT>::T;
  __shared__ cplx coef[QG_MAX_GROUPS];
  if (threadIdx.x < A.n_groups) coef[threadIdx.x] = group_coef(A, threadIdx.x, t);
  __syncthreads();
  const T* val = static_cast<const T*>(A.val);
  const T* xv = static_cast<const T*>(X);
  T* yv = static_cast<T*>(Y);
  const int n = (int)A.n_rows;
  const int sub = threadIdx.x / MM_LANES, lane = threadIdx.x % MM_LANES;
  constexpr int RPB = VEC_BLOCK / MM_LANES;
  for (int base = blockIdx.x * RPB; base < n; base += gridDim.x * RPB) {
    const int row = base + sub;
    const bool valid = row < n;
    for (int64_t v0 = 0; v0 < n_vec; v0 += MM_COLS) {
      cplx acc[MM_COLS];
#pragma unroll
      for (int q = 0; q < MM_COLS; ++q) acc[q] = cplx{0.0, 0.0};
      for (int g = 0; g < A.n_groups; ++g) {
        const int i = valid ? rp_index(A, g, row) : 0;
        const int s = valid ? A.row_ptr[i] : 0, e = valid ? A.row_ptr[i + 1] : 0;
        cplx part[MM_COLS];
#pragma unroll
        for (int q = 0; q < MM_COLS; ++q) part[q] = cplx{0.0, 0.0};
        for (int p = s + lane; p < e; p += MM_LANES) {
          const cplx a = to_c(ld_stream(val + p));
          const int c = ld_stream(A.col + p);
#pragma unroll
          for (int q = 0; q < MM_COLS; ++q)
            if (v0 + q < n_vec) part[q] = cadd(part[q], cmul(a, to_c(xv[(size_t)(v0 + q) * ld + c])));
        }
#pragma unroll
        for (int q = 0; q < MM_COLS; ++q) {
#pragma unroll
          for (int o = MM_LANES / 2; o > 0; o >>= 1) {
            part[q].re += __shfl_xor_sync(0xffffffffu, part[q].re, o);
            part[q].im += __shfl_xor_sync(0xffffffffu, part[q].im, o);
          }
          acc[q] = cadd(acc[q], cmul(coef[g], part[q]));
        }
      }
      if (valid && lane == 0) {
#pragma unroll
        for (int q = 0; q < MM_COLS; ++q) {
          if (v0 + q >= n_vec) break;
          T* yp = yv + (size_t)(v0 + q) * ld + row;
          cplx o = cmul(alpha, acc[q]);
          if (beta.re != 0.0 || beta.im != 0.0) o = cadd(o, cmul(beta, to_c(*yp)));
          *yp = from_c<T>(o);
        }
      }
    }
  }
}

static int vec_grid(int64_t n) {
  int64_t blocks = (n + VEC_BLOCK - 1) / VEC_BLOCK;
  int64_t cap = (int64_t)sm_count() * 8;
  if (cap > qg_scratch_doubles()) cap = qg_scratch_doubles();
  return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

static bool dt_ok(int d) { return d == QG_C128 || d == QG_C64; }

}  // namespace qg

using namespace qg;

extern "C" int qg_rk_combine(const qg_state_view* v, void* out, int out_dtype, void* stream) {
  if (!v || !v->base || !out || (v->n_k > 0 && !v->k)) return set_error(QG_ERR_ARG, "null pointer");
  if (v->n_k < 0 || v->n_k > 16) return set_error(QG_ERR_ARG, "n_k out of range");
  if (!dt_ok(v->base_dtype) || !dt_ok(v->k_dtype) || !dt_ok(out_dtype))
    return set_error(QG_ERR_UNSUPPORTED, "dtype");
  if (v->n == 0) return QG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = vec_grid(v->n);
  const int code = v->base_dtype * 4 + v->k_dtype * 2 + out_dtype;
  switch (code) {
#define QG_C(B, K, O)                                                      \
  case B * 4 + K * 2 + O:                                                  \
    combine_kernel<B, K, O><<<grid, VEC_BLOCK, 0, st>>>(*v, out);          \
    break;
    QG_C(0, 0, 0) QG_C(0, 0, 1) QG_C(0, 1, 0) QG_C(0, 1, 1)
    QG_C(1, 0, 0) QG_C(1, 0, 1) QG_C(1, 1, 0) QG_C(1, 1, 1)
#undef QG_C
  }
  return check_launch("combine_kernel");
}

extern "C" int qg_norm2(const void* x, int dtype, int64_t n, double* scratch,
                        unsigned int* counter, double* result, void* stream) {
  if (!x || !scratch || !counter || !result) return set_error(QG_ERR_ARG, "null pointer");
  if (!dt_ok(dtype)) return set_error(QG_ERR_UNSUPPORTED, "dtype");
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = vec_grid(n);
  if (dtype == QG_C128)
    norm2_kernel<QG_C128><<<grid, VEC_BLOCK, 0, st>>>(x, n, scratch, counter, result);
  else
    norm2_kernel<QG_C64><<<grid, VEC_BLOCK, 0, st>>>(x, n, scratch, counter, result);
  return check_launch("norm2_kernel");
}

template <bool KET>
static int expect_launch(const qg_csr_groups* ops, int64_t d, const qg_state_view* v,
                         double* out, void* stream) {
  if (!ops || !v || !out || !v->base) return set_error(QG_ERR_ARG, "null pointer");
  if (ops->n_groups < 1 || ops->n_groups > QG_MAX_EOPS)
    return set_error(QG_ERR_ARG, "number of operators out of range");
  if (ops->layout != QG_LAYOUT_GROUP_MAJOR && ops->layout != QG_LAYOUT_ROW_MAJOR)
    return set_error(QG_ERR_UNSUPPORTED, "expect needs a CSR (group- or row-major) layout");
  if (!dt_ok(v->base_dtype) || !dt_ok(v->k_dtype) || !dt_ok(ops->dtype))
    return set_error(QG_ERR_UNSUPPORTED, "dtype");
  if (KET ? (ops->n_rows != v->n || ops->n_cols != v->n)
          : (ops->n_rows != d || ops->n_cols != d || d * d != v->n))
    return set_error(QG_ERR_ARG, "incompatible operator and state shapes");
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = ops->n_groups + 1;
  const int code = v->base_dtype * 4 + v->k_dtype * 2 + ops->dtype;
  switch (code) {
#define QG_C(B, K, O)                                                             \
  case B * 4 + K * 2 + O:                                                         \
    expect_kernel<B, K, O, KET><<<grid, VEC_BLOCK, 0, st>>>(*ops, d, *v, out);    \
    break;
    QG_C(0, 0, 0) QG_C(0, 0, 1) QG_C(0, 1, 0) QG_C(0, 1, 1)
    QG_C(1, 0, 0) QG_C(1, 0, 1) QG_C(1, 1, 0) QG_C(1, 1, 1)
#undef QG_C
  }
  return check_launch("expect_kernel");
}

extern "C" int qg_expect_dm(const qg_csr_groups* ops, int64_t d, const qg_state_view* rho,
                            double* out, void* stream) {
  return expect_launch<false>(ops, d, rho, out, stream);
}

extern "C" int qg_expect_ket(const qg_csr_groups* ops, const qg_state_view* psi, double* out,
                             void* stream) {
  return expect_launch<true>(ops, psi ? psi->n : 0, psi, out, stream);
}

extern "C" int qg_spmv_dia(const qg_dia* A, const void* x, void* y, double alpha_re,
                           double alpha_im, double beta_re, double beta_im, void* stream) {
  if (!A || !A->offsets || !A->data || !x || !y) return set_error(QG_ERR_ARG, "null pointer");
  if (!dt_ok(A->dtype)) return set_error(QG_ERR_UNSUPPORTED, "dtype");
  if (A->n_rows <= 0) return QG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = vec_grid(A->n_rows);
  cplx al{alpha_re, alpha_im}, be{beta_re, beta_im};
  if (A->dtype == QG_C128)
    dia_kernel<QG_C128><<<grid, VEC_BLOCK, 0, st>>>(*A, x, y, al, be);
  else
    dia_kernel<QG_C64><<<grid, VEC_BLOCK, 0, st>>>(*A, x, y, al, be);
  return check_launch("dia_kernel");
}

extern "C" int qg_spmm_csr(const qg_csr_groups* A, double t, const void* X, void* Y,
                           int64_t n_vec, int64_t ld, double alpha_re, double alpha_im,
                           double beta_re, double beta_im, void* stream) {
  if (!A || !A->row_ptr || !A->col || !A->val || !X || !Y)
    return set_error(QG_ERR_ARG, "null pointer");
  if (A->n_groups < 1 || A->n_groups > QG_MAX_GROUPS) return set_error(QG_ERR_ARG, "n_groups");
  if (!dt_ok(A->dtype)) return set_error(QG_ERR_UNSUPPORTED, "dtype");
  if (A->layout != QG_LAYOUT_GROUP_MAJOR && A->layout != QG_LAYOUT_ROW_MAJOR)
    return set_error(QG_ERR_UNSUPPORTED, "spmm needs a CSR (group- or row-major) layout");
  if (n_vec < 0 || ld < A->n_rows || ld < A->n_cols) return set_error(QG_ERR_ARG, "bad n_vec/ld");
  if (A->n_rows == 0 || n_vec == 0) return QG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t blocks = (A->n_rows + (VEC_BLOCK / MM_LANES) - 1) / (VEC_BLOCK / MM_LANES);
  int64_t cap = (int64_t)sm_count() * 8;
  const int grid = (int)(blocks < cap ? blocks : cap);
  cplx al{alpha_re, alpha_im}, be{beta_re, beta_im};
  if (A->dtype == QG_C128)
    spmm_kernel<QG_C128><<<grid, VEC_BLOCK, 0, st>>>(*A, t, X, Y, n_vec, ld, al, be);
  else
    spmm_kernel<QG_C64><<<grid, VEC_BLOCK, 0, st>>>(*A, t, X, Y, n_vec, ld, al, be);
  return check_launch("spmm_kernel");
}
