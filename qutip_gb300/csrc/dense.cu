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
// T = X C^dag, then C T.
//
// Work split: CTA j owns the 16 output columns [16 j, 16 j + 16) of every product; column n
// of A X, X A^dag, T = X C^dag and C T needs only column n of X, of A^dag, of C^dag and of
// T, so the CTAs never exchange data and T's block stays in the CTA's shared memory.
// One CTA of 512 threads computes Y = Aop Bop^T (M = 128 rows, N = 16 columns) in K chunks
// of 32: every thread writes its share of the chunk's operand planes (real / imaginary x
// TF32 hi / lo) into one of two shared-memory buffers, one thread issues the 6 MMAs per
// 8-wide K step (real and imaginary output columns side by side, N = 32), and while they run the block loads the next chunk's operands into
// registers and reads the previous chunk's result out of tensor memory.  Each chunk runs into fresh accumulators: D takes the hi*hi terms and E
// the small hi*lo + lo*hi corrections, and the CUDA cores add D + E of every chunk into
// FP32 registers with round-to-nearest.  The tensor core's own accumulation (which does
// not round to nearest) is thereby limited to one chunk: that keeps the result at FP32
// level (a chain over all of K loses up to 5x more, growing with d).  The accumulated
// generator goes through the same fused Vern7 epilogue as the sparse kernels (stage.cuh).
// The stage vectors are complex64: this is the mixed form's generator.
#include <mutex>

#include "capi_internal.h"
#include "common.cuh"
#include "stage.cuh"
#include "tc.cuh"

namespace qg {

constexpr int DN_THREADS = 512;
constexpr int DN_KC = 32;                          // K chunk
constexpr int DN_NB = 16;                          // output columns per CTA (MMA N)
constexpr int DN_CW = 8;                           // columns of one part per thread
constexpr uint32_t DN_PLANE_A = 128u * DN_KC * 4u;  // one A-operand plane (M = 128 rows)
constexpr uint32_t DN_PLANE_B = 2 * DN_NB * DN_KC * 4u;  // one B-operand plane (N = 32 rows)
constexpr uint32_t DN_BUF_A = 4u * DN_PLANE_A, DN_BUF_B = 4u * DN_PLANE_B;
constexpr int DN_TS = 129;                         // row stride (float2) of the T block
constexpr int DN_TMEM_COLS = 128;                  // 2 buffers x (D re, D im, E re, E im) x 16
constexpr size_t DN_SMEM = 2 * (size_t)DN_BUF_A + 2 * (size_t)DN_BUF_B +
                           (size_t)DN_NB * DN_TS * sizeof(float2);

__device__ unsigned int g_dense_fault = 0u;

// Where the rows of an operand chunk come from.
enum Src { SRC_OPA = 0, SRC_OPC = 1, SRC_XB = 2, SRC_XA = 3, SRC_TB = 4 };

struct DenseCtx {
  const qg_dense_lindblad* L;
  const float2* x;     // the argument, vec(X): X[r][c] at c*d + r
  int d, n0;           // dimension, first output column of this CTA
  int cop;             // collapse operator of SRC_OPC
  const float2* ca;    // a_g(t) in shared memory
  const float2* t;     // this CTA's columns of T = X C^dag: T[k][n0 + j] at j*DN_TS + k
};

// Operand chunks.  Element e of a rows x 32 chunk maps to (r, kk) with the low 3 bits of
// e the row within an 8-row band and the next 2 bits the column within a 4-column core: a
// warp's 32 shared-memory stores fall in 32 different banks.  Thread t holds elements
// t, t + 256, ...: all of them are loaded first (the loads in flight together), then
// split and stored, so a chunk costs one memory latency, hidden behind the previous
// chunk's MMAs.
template <int ROWS>
struct Chunk {
  static constexpr int PER = ROWS * DN_KC / DN_THREADS;
  float2 v[PER];
};

__device__ __forceinline__ int chunk_row(int e) { return (e >> 8) * 8 + (e & 7); }
__device__ __forceinline__ int chunk_col(int e) { return ((e >> 5) & 7) * 4 + ((e >> 3) & 3); }

// Rows [row0, row0 + ROWS) x K chunk kc of a source: the operator sum A(t), C_cop, X read
// as (n, k) -> X[k][n] (B operand of A X), X read as (m, k) -> X[m][k] (A operand of
// X B^dag), or T read as (n, k) -> T[k][n] (B operand of C T); zero outside d x d.
template <int ROWS>
__device__ __forceinline__ void load_chunk(const DenseCtx& c, int src, int row0, int kc,
                                           Chunk<ROWS>& ch) {
  constexpr int PER = Chunk<ROWS>::PER;
  const qg_dense_lindblad& L = *c.L;
  const int d = c.d;
  int off[PER];
  bool in[PER];
  int sr = d, sk = 1;  // element (r, k) at base + r * sr + k * sk
  const float2* base;
  if (src == SRC_XB) {
    base = c.x;
  } else if (src == SRC_XA) {
    base = c.x;
    sr = 1;
    sk = d;
  } else if (src == SRC_TB) {
    base = c.t - (size_t)c.n0 * DN_TS;
    sr = DN_TS;
  } else if (src == SRC_OPC) {
    base = static_cast<const float2*>(L.c) + (size_t)c.cop * d * d;
  } else {
    base = static_cast<const float2*>(L.a);
  }
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = threadIdx.x + i * DN_THREADS;
    const int r = row0 + chunk_row(e), k = kc * DN_KC + chunk_col(e);
    in[i] = r < d && k < d;
    off[i] = in[i] ? r * sr + k * sk : 0;
    ch.v[i] = make_float2(0.f, 0.f);
  }
  if (src != SRC_OPA) {
#pragma unroll
    for (int i = 0; i < PER; ++i)
      if (in[i]) ch.v[i] = base[off[i]];
    return;
  }
  for (int g = 0; g < L.n_groups; ++g) {  // A(t) = sum_g a_g(t) A_g
    const float2 a = c.ca[g];
    const float2* bg = base + (size_t)g * d * d;
    float2 w[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) w[i] = in[i] ? __ldg(bg + off[i]) : make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      ch.v[i].x = fmaf(a.x, w[i].x, fmaf(-a.y, w[i].y, ch.v[i].x));
      ch.v[i].y = fmaf(a.x, w[i].y, fmaf(a.y, w[i].x, ch.v[i].y));
    }
  }
}

// The chunk as four planes (re hi, re lo, im hi, im lo) in the core-matrix layout.
template <int ROWS>
__device__ __forceinline__ void store_chunk(const Chunk<ROWS>& ch, unsigned char* planes,
                                            uint32_t plane_bytes) {
#pragma unroll
  for (int i = 0; i < Chunk<ROWS>::PER; ++i) {
    const int e = threadIdx.x + i * DN_THREADS;
    float rh, rl, ih, il;
    tc::tf32_split(ch.v[i].x, rh, rl);
    tc::tf32_split(ch.v[i].y, ih, il);
    const uint32_t off = tc::core_off(chunk_row(e), chunk_col(e), DN_KC);
    *reinterpret_cast<float*>(planes + off) = rh;
    *reinterpret_cast<float*>(planes + plane_bytes + off) = rl;
    *reinterpret_cast<float*>(planes + 2 * plane_bytes + off) = ih;
    *reinterpret_cast<float*>(planes + 3 * plane_bytes + off) = il;
  }
}

// The B operand (this CTA's 16 rows of Bop, conjugated when conj) stacked for complex
// products with N = 32: B1 = [Br ; s Bi] and B2 = [-s Bi ; Br] (s = -1 when conjugated), so
// that Ar B1^T + Ai B2^T = [re | im] of Aop Bop^T in 32 accumulator columns.  Planes:
// B1 hi, B1 lo, B2 hi, B2 lo.
__device__ __forceinline__ void store_chunk_b(const Chunk<DN_NB>& ch, unsigned char* planes,
                                              bool conj) {
#pragma unroll
  for (int i = 0; i < Chunk<DN_NB>::PER; ++i) {
    const int e = threadIdx.x + i * DN_THREADS;
    const int r = chunk_row(e), kk = chunk_col(e);
    const float re = ch.v[i].x, im = conj ? -ch.v[i].y : ch.v[i].y;
    float rh, rl, ih, il;
    tc::tf32_split(re, rh, rl);
    tc::tf32_split(im, ih, il);
    const uint32_t top = tc::core_off(r, kk, DN_KC), bot = tc::core_off(r + DN_NB, kk, DN_KC);
    float* p = reinterpret_cast<float*>(planes);
    constexpr uint32_t P = DN_PLANE_B / 4;
    p[(top >> 2)] = rh;            // B1 = [Br ; s Bi]
    p[(bot >> 2)] = ih;
    p[P + (top >> 2)] = rl;
    p[P + (bot >> 2)] = il;
    p[2 * P + (top >> 2)] = -ih;   // B2 = [-s Bi ; Br]
    p[2 * P + (bot >> 2)] = rh;
    p[3 * P + (top >> 2)] = -il;
    p[3 * P + (bot >> 2)] = rl;
  }
}

// One K chunk of Aop Bop^T (M = 128, N = 32: real and imaginary columns), each real
// product in three TF32 terms: hi*hi into D (TMEM columns +0..31), hi*lo and lo*hi into E
// (+32..63), 6 MMAs per 8-wide K step.  Issued by one thread; the chunk's first MMA into
// D and into E overwrites.  Descriptors advance by integer adds (16-byte units; shared
// memory addresses stay below 2^18 bytes, inside the 14-bit field).
__device__ __forceinline__ void issue_chunk(uint32_t tcols, uint32_t a_base, uint32_t b_base,
                                            int ksteps) {
  const uint32_t sbo = tc::band_bytes(DN_KC);
  const uint64_t da = tc::smem_desc(a_base, tc::LBO, sbo), db = tc::smem_desc(b_base, tc::LBO, sbo);
  constexpr uint64_t PA = DN_PLANE_A >> 4, PB = DN_PLANE_B >> 4;
  constexpr uint32_t id = tc::idesc_tf32(128, 2 * DN_NB, false);
  const uint32_t td = tcols, te = tcols + 2 * DN_NB;
  for (int ks = 0; ks < ksteps; ++ks) {
    const uint64_t k = (uint64_t)ks * (2 * tc::LBO >> 4);
    const bool acc = ks > 0;
    tc::mma_tf32(td, da + k, db + k, id, acc);                    // Ar hi . B1 hi
    tc::mma_tf32(td, da + 2 * PA + k, db + 2 * PB + k, id, true);  // Ai hi . B2 hi
    tc::mma_tf32(te, da + k, db + PB + k, id, acc);               // Ar hi . B1 lo
    tc::mma_tf32(te, da + PA + k, db + k, id, true);              // Ar lo . B1 hi
    tc::mma_tf32(te, da + 2 * PA + k, db + 3 * PB + k, id, true);  // Ai hi . B2 lo
    tc::mma_tf32(te, da + 3 * PA + k, db + 2 * PB + k, id, true);  // Ai lo . B2 hi
  }
}

template <int YDT, int EPI>
__global__ void __launch_bounds__(DN_THREADS, 1)
    dense_lindblad_kernel(qg_dense_lindblad L, double t, const float2* __restrict__ x,
                          AxpbyArgs ax, RkArgs rk) {
  extern __shared__ __align__(128) unsigned char dn_smem[];
  __shared__ float2 ca[QG_MAX_GROUPS];
  __shared__ float wc[QG_MAX_COPS];
  __shared__ uint32_t taddr_s;
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ double red[DN_THREADS / 32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int d = L.d;
  const int n0 = blockIdx.x * DN_NB;
  unsigned char* a_planes = dn_smem;                      // 2 buffers
  unsigned char* b_planes = dn_smem + 2 * DN_BUF_A;       // 2 buffers
  float2* t_blk = reinterpret_cast<float2*>(dn_smem + 2 * DN_BUF_A + 2 * DN_BUF_B);
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
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&taddr_s, DN_TMEM_COLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t taddr = taddr_s;
  DenseCtx c{&L, x, d, n0, 0, ca, t_blk};
  const int nchunks = (d + DN_KC - 1) / DN_KC;
  // Thread roles when reading tensor memory: warp w reads TMEM lanes 32 (w % 4) ... (its
  // rows m), the real (part 0) or imaginary (part 1) columns of bit 2 of w, and of those the
  // 8 columns cw0 ... cw0 + 7 chosen by bit 3.
  const int part = (warp >> 2) & 1;
  const int cw0 = DN_CW * (warp >> 3);
  const int m = 32 * (warp & 3) + lane;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
  unsigned par[2] = {0u, 0u};
  bool pend[2] = {false, false};  // a commit to bar[b] not yet waited for
  bool ok = true;
  int buf = 0;
  float prod[DN_CW], gen[DN_CW];
#pragma unroll
  for (int j = 0; j < DN_CW; ++j) gen[j] = 0.f;

  auto wait_buf = [&](int b) {
    const bool r = __syncthreads_and(mbar_poll(&bar[b], par[b]) ? 1 : 0) != 0;
    if (r) {
      par[b] ^= 1u;
      pend[b] = false;
    }
    tc::fence_after();
    return r;
  };
  // add D + E of buffer b (this thread's part, row m, 8 columns) into prod
  auto take = [&](int b, bool first) {
    float dv[DN_CW], ev[DN_CW];
    const uint32_t cols = taddr + lane_base + (uint32_t)(4 * DN_NB * b + DN_NB * part + cw0);
    tc::tmem_ld8(cols, dv);
    tc::tmem_ld8(cols + 2 * DN_NB, ev);
#pragma unroll
    for (int j = 0; j < DN_CW; ++j) {
      const float v = dv[j] + ev[j];
      prod[j] = first ? v : prod[j] + v;
    }
  };
  // one product op(srcA) op(srcB)^T of this CTA's columns into prod
  Chunk<128> cha;
  Chunk<DN_NB> chb;
  auto gemm = [&](int src_a, int src_b, bool conj_b) {
    load_chunk(c, src_a, 0, 0, cha);
    load_chunk(c, src_b, n0, 0, chb);
    for (int kc = 0; kc < nchunks && ok; ++kc) {
      const int b = buf;
      store_chunk(cha, a_planes + b * DN_BUF_A, DN_PLANE_A);
      store_chunk_b(chb, b_planes + b * DN_BUF_B, conj_b);
      tc::fence_smem_to_async();
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      if (tid == 0) {
        const int ksteps = min(4, (d - kc * DN_KC + 7) >> 3);
        issue_chunk(taddr + (uint32_t)(4 * DN_NB * b), smem_u32(a_planes + b * DN_BUF_A),
                    smem_u32(b_planes + b * DN_BUF_B), ksteps);
        tc::mma_commit(&bar[b]);
      }
      pend[b] = true;
      if (kc + 1 < nchunks) {  // the next chunk's loads, in flight during the MMAs
        load_chunk(c, src_a, 0, kc + 1, cha);
        load_chunk(c, src_b, n0, kc + 1, chb);
      }
      if (kc > 0) {  // the previous chunk, while this one runs
        ok = wait_buf(b ^ 1);
        if (ok) take(b ^ 1, kc == 1);
      }
      buf ^= 1;
    }
    if (ok) {
      ok = wait_buf(buf ^ 1);
      if (ok) take(buf ^ 1, nchunks == 1);
    }
    tc::fence_before();
    __syncthreads();  // every read of TMEM and of the planes is done
    tc::fence_after();
  };
  auto accumulate = [&](float w) {
#pragma unroll
    for (int j = 0; j < DN_CW; ++j) gen[j] = fmaf(w, prod[j], gen[j]);
  };

  gemm(SRC_OPA, SRC_XB, false);  // A X
#pragma unroll
  for (int j = 0; j < DN_CW; ++j) gen[j] = prod[j];
  gemm(SRC_XA, SRC_OPA, true);   // X A^dag
  accumulate(1.f);
  for (int i = 0; i < L.n_cops && ok; ++i) {
    c.cop = i;
    gemm(SRC_XA, SRC_OPC, true);  // T = X C^dag, this CTA's columns
    float* tp = reinterpret_cast<float*>(t_blk) + part;
#pragma unroll
    for (int j = 0; j < DN_CW; ++j) tp[2 * ((cw0 + j) * DN_TS + m)] = prod[j];
    __syncthreads();
    gemm(SRC_OPC, SRC_TB, false);  // C T
    accumulate(wc[i]);
  }

  double err_acc = 0.0;
  if (ok) {
    // real and imaginary parts meet in shared memory (the A planes are free now)
    float* ex = reinterpret_cast<float*>(a_planes) + part;
#pragma unroll
    for (int j = 0; j < DN_CW; ++j) ex[2 * ((cw0 + j) * 128 + m)] = gen[j];
    __syncthreads();
    const float2* exv = reinterpret_cast<const float2*>(a_planes);
    const int ncols = min(DN_NB, d - n0);
    for (int e = tid; e < ncols * d; e += DN_THREADS) {
      const int jl = e / d, mm = e - jl * d;
      const float2 v = exv[jl * 128 + mm];
      epilogue<QG_C64, YDT, EPI>((n0 + jl) * d + mm, cx<float>{v.x, v.y}, ax, rk,
                                 err_acc);
    }
  } else if (tid == 0) {
    atomicOr(&g_dense_fault, 1u);
    // let outstanding commits land before the tensor memory is freed
    for (int b = 0; b < 2; ++b)
      if (pend[b]) (void)mbar_poll(&bar[b], par[b]);
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_dealloc(taddr, DN_TMEM_COLS);
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<DN_THREADS>(rk, err_acc, red);
  }
}

static size_t dense_smem(int) { return DN_SMEM; }

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
  const int grid = (L.d + DN_NB - 1) / DN_NB;
  kern<<<grid, DN_THREADS, smem, st>>>(L, t, static_cast<const float2*>(x), ax, rk);
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
