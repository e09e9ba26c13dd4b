// Dense small-dimension bucket: the Lindblad generator of a system of Hilbert dimension
// d <= 128 with dense operators, applied to rho (d x d) as GEMMs on the fifth-generation
// tensor cores (tcgen05, TF32 inputs split hi + lo for FP32 accuracy, FP32 accumulators
// in tensor memory):
//
//   L(t)[X] = A X + X A^dag + sum_i w_i C_i X C_i^dag,   A = sum_g a_g(t) A_g = -i H_nh,
//   w_i = |f_i(t)|^2,
//
// the reference's LindbladMatrixForm (qutip/core/cy/lindblad_matrix_form.pyx:105-204,
// full non-Hermitian branch) with dense operators.  Per collapse operator two products:
// T = X C^dag, then C T.  Each product runs into fresh TMEM accumulators: D (columns
// 0..255: real, imaginary) takes the hi*hi terms and E (256..511) the small hi*lo + lo*hi
// corrections, so no rounding of a correction happens at the magnitude of the product;
// D + E is then flushed by the CUDA cores, in FP32 with round-to-nearest, into the
// caller's workspace (the generator's accumulator, or T).  The accumulated generator
// goes through the same fused Vern7 epilogue as the sparse kernels (stage.cuh).  The
// stage vectors are complex64: this is the mixed form's generator.
//
// One CTA of 256 threads per application.  Operands are staged through shared memory in
// K chunks of 32: for each chunk every thread writes its share of the A- and B-operand
// planes (real / imaginary x hi / lo), then one thread issues the MMAs (12 per 8-wide K
// step: four real products of the complex product, three TF32 terms each) and commits
// them to an mbarrier that every thread waits on, with a bounded wait.
#include <mutex>

#include "capi_internal.h"
#include "common.cuh"
#include "stage.cuh"
#include "tc.cuh"

namespace qg {

constexpr int DN_THREADS = 256;
constexpr int DN_KC = 32;                          // K chunk
constexpr uint32_t DN_PLANE_A = 128u * DN_KC * 4u;  // one A-operand plane (M = 128 rows)
constexpr int DN_TMEM_COLS = 512;

__device__ unsigned int g_dense_fault = 0u;

// Where the rows of an operand chunk come from.
enum Src { SRC_OPA = 0, SRC_OPC = 1, SRC_XB = 2, SRC_XA = 3, SRC_TB = 4 };

struct DenseCtx {
  const qg_dense_lindblad* L;
  const float2* x;     // the argument, vec(X): X[r][c] at c*d + r
  int d, np;           // dimension, N (rows of the B operand) = d rounded up to 16
  int cop;             // collapse operator of SRC_OPC
  const float2* ca;    // a_g(t) in shared memory
  const float2* t;     // T = X C^dag, row-major: T[r][c] at r*d + c
};

// element (r, k) of a source: the operator sum A(t), C_cop, X read as (n, k) -> X[k][n]
// (B operand of A X and C X ...), or X read as (m, k) -> X[m][k] (A operand of X B^dag)
__device__ __forceinline__ float2 src_at(const DenseCtx& c, int src, int r, int k,
                                         const qg_dense_lindblad& L) {
  const int d = c.d;
  if (r >= d || k >= d) return make_float2(0.f, 0.f);
  if (src == SRC_XB) return c.x[(size_t)r * d + k];
  if (src == SRC_XA) return c.x[(size_t)k * d + r];
  if (src == SRC_TB) return c.t[(size_t)k * d + r];   // (n, k) -> T[k][n]
  const float2* base = static_cast<const float2*>(src == SRC_OPA ? L.a : L.c);
  if (src == SRC_OPC) return __ldg(base + ((size_t)c.cop * d + r) * d + k);
  float re = 0.f, im = 0.f;
  for (int g = 0; g < L.n_groups; ++g) {
    const float2 v = __ldg(base + ((size_t)g * d + r) * d + k);
    const float2 a = c.ca[g];
    re = fmaf(a.x, v.x, fmaf(-a.y, v.y, re));
    im = fmaf(a.x, v.y, fmaf(a.y, v.x, im));
  }
  return make_float2(re, im);
}

// Write rows [0, rows) x K chunk kc of a source into four planes (re hi, re lo, im hi,
// im lo), each rows x 32 values in the core-matrix layout.  Element e of the chunk maps to
// (r, kk) with the low 3 bits of e the row within an 8-row band and the next 2 bits the
// column within a 4-column core: a warp's 32 stores fall in 32 different banks.
__device__ __forceinline__ void stage_planes(const DenseCtx& c, int src, int rows, int kc,
                                             unsigned char* planes, uint32_t plane_bytes) {
  const qg_dense_lindblad& L = *c.L;
  for (int e = threadIdx.x; e < rows * DN_KC; e += DN_THREADS) {
    const int r = (e >> 8) * 8 + (e & 7);
    const int kk = ((e >> 5) & 7) * 4 + ((e >> 3) & 3);
    const float2 v = src_at(c, src, r, kc * DN_KC + kk, L);
    float rh, rl, ih, il;
    tc::tf32_split(v.x, rh, rl);
    tc::tf32_split(v.y, ih, il);
    const uint32_t off = tc::core_off(r, kk, DN_KC);
    *reinterpret_cast<float*>(planes + off) = rh;
    *reinterpret_cast<float*>(planes + plane_bytes + off) = rl;
    *reinterpret_cast<float*>(planes + 2 * plane_bytes + off) = ih;
    *reinterpret_cast<float*>(planes + 3 * plane_bytes + off) = il;
  }
}

// One K chunk of Aop Bop^T for complex operands (Bop conjugated when conj_b):
// re = Ar Br -/+ Ai Bi, im = +/- Ar Bi + Ai Br, each real product in three TF32 terms,
// hi*hi into D (TMEM columns 0 / 128 for re / im) and hi*lo, lo*hi into E (256 / 384).
// Issued by one thread; init: the chunk starts the product (first MMA of each region
// overwrites).
__device__ __forceinline__ void issue_chunk(uint32_t taddr, uint32_t a_base, uint32_t b_base,
                                            uint32_t b_plane, int np, int ksteps, bool conj_b,
                                            bool init) {
  const uint32_t sbo = tc::band_bytes(DN_KC);
  const uint32_t id_pos = tc::idesc_tf32(128, np, false), id_neg = tc::idesc_tf32(128, np, true);
  // (A plane pair, B plane pair, destination: 0 re / 1 im, negated)
  const int ap[4] = {0, 2, 0, 2}, bp[4] = {0, 2, 2, 0}, dst[4] = {0, 0, 1, 1};
  const bool neg[4] = {false, !conj_b, conj_b, false};
  bool first[4] = {init, init, init, init};  // D re, D im, E re, E im
  for (int ks = 0; ks < ksteps; ++ks) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      // hi*hi -> D; hi*lo, lo*hi -> E
      const int at[3] = {0, 0, 1}, bt[3] = {0, 1, 0};
#pragma unroll
      for (int tt = 0; tt < 3; ++tt) {
        const int region = dst[q] + (tt ? 2 : 0);
        const uint32_t a = a_base + (uint32_t)(ap[q] + at[tt]) * DN_PLANE_A + ks * 2 * tc::LBO;
        const uint32_t b = b_base + (uint32_t)(bp[q] + bt[tt]) * b_plane + ks * 2 * tc::LBO;
        tc::mma_tf32(taddr + 128u * region, tc::smem_desc(a, tc::LBO, sbo),
                     tc::smem_desc(b, tc::LBO, sbo), neg[q] ? id_neg : id_pos, !first[region]);
        first[region] = false;
      }
    }
  }
}

// Wait for the MMAs committed to bar (phase `parity`); false when the bounded wait gave up
__device__ __forceinline__ bool wait_mma(uint64_t* bar, unsigned& parity) {
  const bool ok = __syncthreads_and(mbar_poll(bar, parity) ? 1 : 0) != 0;
  parity ^= 1u;
  tc::fence_after();
  return ok;
}

template <int YDT, int EPI>
__global__ void __launch_bounds__(DN_THREADS, 1)
    dense_lindblad_kernel(qg_dense_lindblad L, double t, const float2* __restrict__ x,
                          AxpbyArgs ax, RkArgs rk) {
  extern __shared__ __align__(128) unsigned char dn_smem[];
  __shared__ float2 ca[QG_MAX_GROUPS];
  __shared__ float wc[QG_MAX_COPS];
  __shared__ uint32_t taddr_s;
  __shared__ __align__(8) uint64_t bar;
  __shared__ double red[DN_THREADS / 32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int d = L.d;
  const int np = (d + 15) & ~15;
  const uint32_t b_plane = (uint32_t)np * DN_KC * 4u;
  unsigned char* a_planes = dn_smem;
  unsigned char* b_planes = dn_smem + 4 * DN_PLANE_A;
  if (tid < L.n_groups) {
    cplx a{1.0, 0.0};
    if (L.a_coef_code) a = eval_coef(L.a_coef_code + L.a_coef_start[tid], L.a_coef_consts, t);
    ca[tid] = make_float2((float)a.re, (float)a.im);
  }
  if (tid < L.n_cops) {
    cplx f{1.0, 0.0};
    if (L.c_coef_code) f = eval_coef(L.c_coef_code + L.c_coef_start[tid], L.c_coef_consts, t);
    wc[tid] = (float)(f.re * f.re + f.im * f.im);
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&taddr_s, DN_TMEM_COLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = taddr_s;
  const uint32_t a_base = smem_u32(a_planes), b_base = smem_u32(b_planes);
  float2* acc = static_cast<float2*>(L.work);          // vec order, (m, n) at n*d + m
  float2* tmat = acc + (size_t)d * d;                    // T row-major, (m, n) at m*d + n
  DenseCtx c{&L, x, d, np, 0, ca, tmat};
  const int nchunks = (d + DN_KC - 1) / DN_KC;
  unsigned parity = 0u;
  bool ok = true;

  // one product op(srcA) op(srcB)^T over every K chunk, into fresh D and E
  auto gemm = [&](int src_a, int src_b, bool conj_b) {
    for (int kc = 0; kc < nchunks && ok; ++kc) {
      stage_planes(c, src_a, 128, kc, a_planes, DN_PLANE_A);
      stage_planes(c, src_b, np, kc, b_planes, b_plane);
      tc::fence_smem_to_async();
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      if (tid == 0) {
        const int ksteps = min(4, (d - kc * DN_KC + 7) >> 3);
        issue_chunk(taddr, a_base, b_base, b_plane, np, ksteps, conj_b, kc == 0);
        tc::mma_commit(&bar);
      }
      ok = wait_mma(&bar, parity);
    }
  };
  // D + E of the last product, times w, into the accumulator (add) or into T; row m of
  // the product lives in TMEM lane m, warps w and w + 4 share lanes 32 (w % 4) ...
  const int m = 32 * (warp & 3) + lane;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
  auto flush = [&](bool to_t, bool add, float w) {
    if (!ok) return;
    for (int cb = (warp >> 2) * 16; cb < np; cb += 32) {
      float dr[16], di[16], er[16], ei[16];
      tc::tmem_ld16(taddr + lane_base + (uint32_t)cb, dr);
      tc::tmem_ld16(taddr + lane_base + 128u + (uint32_t)cb, di);
      tc::tmem_ld16(taddr + lane_base + 256u + (uint32_t)cb, er);
      tc::tmem_ld16(taddr + lane_base + 384u + (uint32_t)cb, ei);
      if (m < d) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = cb + j;
          if (n >= d) continue;
          const float2 v = make_float2(w * (dr[j] + er[j]), w * (di[j] + ei[j]));
          if (to_t) {
            tmat[(size_t)m * d + n] = v;
          } else {
            float2* p = acc + (size_t)n * d + m;
            *p = add ? make_float2(p->x + v.x, p->y + v.y) : v;
          }
        }
      }
    }
    tc::fence_before();
    __syncthreads();  // the flushed values are visible to the block; TMEM may be rewritten
    tc::fence_after();
  };

  gemm(SRC_OPA, SRC_XB, false);  // A X
  flush(false, false, 1.f);
  gemm(SRC_XA, SRC_OPA, true);   // X A^dag
  flush(false, true, 1.f);
  for (int i = 0; i < L.n_cops && ok; ++i) {
    c.cop = i;
    gemm(SRC_XA, SRC_OPC, true);  // T = X C^dag
    flush(true, false, 1.f);
    gemm(SRC_OPC, SRC_TB, false);  // C T
    flush(false, true, wc[i]);
  }

  double err_acc = 0.0;
  if (ok) {
    for (int idx = tid; idx < d * d; idx += DN_THREADS) {
      const float2 v = acc[idx];
      epilogue<QG_C64, YDT, EPI>(idx, cx<float>{v.x, v.y}, ax, rk, err_acc);
    }
  } else if (tid == 0) {
    atomicOr(&g_dense_fault, 1u);
    (void)mbar_poll(&bar, parity ^ 1u);  // let an outstanding commit land before freeing TMEM
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_dealloc(taddr, DN_TMEM_COLS);
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<DN_THREADS>(rk, err_acc, red);
  }
}

static size_t dense_smem(int d) {
  const int np = (d + 15) & ~15;
  return 4 * (size_t)DN_PLANE_A + 4 * (size_t)np * DN_KC * 4;
}

template <int YDT, int EPI>
static int launch_dense(cudaStream_t st, const qg_dense_lindblad& L, double t, const void* x,
                        const AxpbyArgs& ax, const RkArgs& rk) {
  auto kern = dense_lindblad_kernel<YDT, EPI>;
  const size_t smem = dense_smem(L.d);
  static std::mutex mu;
  static size_t set_bytes[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error(QG_ERR_CUDA, "no current CUDA device");
  {
    std::lock_guard<std::mutex> lock(mu);
    if (set_bytes[dev] < smem) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
        return set_error(QG_ERR_CUDA, "dense Lindblad kernel: shared memory opt-in failed");
      set_bytes[dev] = smem;
    }
  }
  kern<<<1, DN_THREADS, smem, st>>>(L, t, static_cast<const float2*>(x), ax, rk);
  return check_launch("dense_lindblad_kernel");
}

static int check_dense(const qg_dense_lindblad* L) {
  if (!L) return set_error(QG_ERR_ARG, "null generator");
  if (L->d < 1 || L->d > QG_DENSE_MAX_D)
    return set_error(QG_ERR_ARG, "dense bucket: need 1 <= d <= QG_DENSE_MAX_D (128)");
  if (L->n_groups < 1 || L->n_groups > QG_MAX_GROUPS)
    return set_error(QG_ERR_ARG, "n_groups out of range");
  if (L->n_cops < 0 || L->n_cops > QG_MAX_COPS)
    return set_error(QG_ERR_ARG, "collapse operator count out of range");
  if (!L->a || (L->n_cops > 0 && !L->c)) return set_error(QG_ERR_ARG, "null operator storage");
  if (!L->work) return set_error(QG_ERR_ARG, "null workspace (2*d*d complex64 values)");
  if ((L->a_coef_code && (!L->a_coef_start || !L->a_coef_consts)) ||
      (L->c_coef_code && (!L->c_coef_start || !L->c_coef_consts)))
    return set_error(QG_ERR_ARG, "coefficient program tables incomplete");
  return QG_OK;
}

}  // namespace qg

using namespace qg;

int dense_fault_take() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_dense_fault, sizeof(v)) != cudaSuccess) return 0;
  if (v) cudaMemcpyToSymbol(g_dense_fault, &zero, sizeof(zero));
  return (int)v;
}

extern "C" int qg_dense_lindblad_apply(const qg_dense_lindblad* L, double t, const void* x,
                                       void* y, double alpha_re, double alpha_im,
                                       double beta_re, double beta_im, void* stream) {
  int rc = check_dense(L);
  if (rc) return rc;
  if (!x || !y) return set_error(QG_ERR_ARG, "null vector");
  AxpbyArgs ax{y, alpha_re, alpha_im, beta_re, beta_im};
  RkArgs rk{};
  return launch_dense<QG_C64, EPI_AXPBY>((cudaStream_t)stream, *L, t, x, ax, rk);
}

extern "C" int qg_dense_lindblad_stage(const qg_dense_lindblad* L, const qg_rk_buffers* B,
                                       int stage, double t_prev, double dt, double atol,
                                       double rtol, void* stream) {
  int rc = check_dense(L);
  if (rc) return rc;
  RkArgs rk;
  const void* x = nullptr;
  rc = prepare_stage(B, QG_C64, (int64_t)L->d * L->d, stage, dt, atol, rtol, rk, x);
  if (rc) return rc;
  AxpbyArgs ax{};
  const double t = t_prev + VERN7_C_HOST[stage] * dt;
  cudaStream_t st = (cudaStream_t)stream;
  if (B->state_dtype == QG_C128) return launch_dense<QG_C128, EPI_RK>(st, *L, t, x, ax, rk);
  return launch_dense<QG_C64, EPI_RK>(st, *L, t, x, ax, rk);
}
