// Complex CSR matvec over coefficient groups, with two epilogues:
//   * AXPBY: y = alpha * A(t) x + beta * y           (qg_spmv_csr)
//   * RK:    Vern7 stage k_s = A(t_s) x_s fused with the next stage's input
//            combination, or with y_front and the WRMS error at the last stage
//            (qg_vern7_stage).
//
// Two kernels share the row computation and the epilogues:
//   * direct: a sub-warp of LANES threads owns one row and reads values and
//     column indices straight from HBM (coalesced within the row);
//   * staged: persistent CTAs walk row tiles; one elected thread moves each
//     tile's values, column indices and row pointers into shared memory with
//     bulk async copies (cp.async.bulk, completion on an mbarrier), double
//     buffered so the next tile streams in while the current one is reduced.
// In both, the gathered vector x is read through the read-only path and stays
// L2-resident, and the grid is a whole number of waves over the SMs.
//
// Arithmetic: GB300 runs FP64 at a small fraction of its FP32 rate, so every
// complex64 path computes in FP32 (compute type CT = float): the row dots, the
// coefficient products and the stage combinations, whose factors dt * a_ij are
// formed once on the host.  FP64 remains where it carries the result: the
// complex128 path throughout, and in the mixed form the once-per-step state
// update y_front = y_prev + increment and the WRMS error reduction.
#include <mutex>

#include "capi_internal.h"
#include "common.cuh"
#include "stage.cuh"

namespace qg {

constexpr int SPMV_BLOCK = 256;
// Resident blocks per SM the sliced kernel is compiled for (40 registers).
constexpr int SLICED_MIN_BLOCKS = 6;

__device__ unsigned int g_fault = 0u;

// Complex multiply-accumulate in the accumulation precision.
__device__ __forceinline__ void cmac_any(double& ar, double& ai, double2 v, double2 x) {
  ar = fma(v.x, x.x, ar);
  ar = fma(-v.y, x.y, ar);
  ai = fma(v.x, x.y, ai);
  ai = fma(v.y, x.x, ai);
}
__device__ __forceinline__ void cmac_any(float& ar, float& ai, float2 v, float2 x) {
  ar = fmaf(v.x, x.x, ar);
  ar = fmaf(-v.y, x.y, ar);
  ai = fmaf(v.x, x.y, ai);
  ai = fmaf(v.y, x.x, ai);
}

template <int LANES, typename R>
__device__ __forceinline__ cx<R> sub_reduce(R ar, R ai) {
#pragma unroll
  for (int o = LANES / 2; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    ai += __shfl_xor_sync(0xffffffffu, ai, o);
  }
  return cx<R>{ar, ai};
}

// Partial row dot product over entries [s, e) for one lane of a LANES-wide
// sub-warp.  GLOBAL: val/col are global arrays; otherwise shared-memory
// pointers pre-offset so that entry p is val[p].
template <typename VT, typename R, int LANES, bool GLOBAL>
__device__ __forceinline__ void lane_dot(const int* __restrict__ col, const VT* __restrict__ val,
                                         const VT* __restrict__ x, int s, int e, int lane,
                                         R& ar, R& ai) {
  int p = s + lane;
  for (; p + LANES < e; p += 2 * LANES) {
    VT v0, v1;
    int c0, c1;
    if (GLOBAL) {
      v0 = ld_stream(val + p);
      v1 = ld_stream(val + p + LANES);
      c0 = ld_stream(col + p);
      c1 = ld_stream(col + p + LANES);
    } else {
      v0 = val[p];
      v1 = val[p + LANES];
      c0 = col[p];
      c1 = col[p + LANES];
    }
    VT x0 = ld_gather(x + c0), x1 = ld_gather(x + c1);
    cmac_any(ar, ai, v0, x0);
    cmac_any(ar, ai, v1, x1);
  }
  if (p < e) {
    VT v0 = GLOBAL ? ld_stream(val + p) : val[p];
    int c0 = GLOBAL ? ld_stream(col + p) : col[p];
    cmac_any(ar, ai, v0, ld_gather(x + c0));
  }
}

template <typename CT>
__device__ __forceinline__ void load_coefs(const qg_csr_groups& A, double t, cx<CT>* coef) {
  if (threadIdx.x < A.n_groups) {
    cplx c = group_coef(A, threadIdx.x, t);
    coef[threadIdx.x] = cx<CT>{(CT)c.re, (CT)c.im};
  }
}

// Class of each group's coefficient, decided once per block: 0 = exactly one (the
// group's sum goes straight into the row's), 1 = real, 2 = complex.
template <typename CT>
__device__ __forceinline__ void coef_classes(const qg_csr_groups& A, const cx<CT>* coef, int* cls) {
  if (threadIdx.x < A.n_groups) {
    const cx<CT> c = coef[threadIdx.x];
    cls[threadIdx.x] = (c.re == (CT)1 && c.im == (CT)0) ? 0 : (c.im == (CT)0 ? 1 : 2);
  }
}

// ------------------------------------------------------------ direct kernel --
template <int DT, int YDT, int LANES, int EPI>
__global__ void __launch_bounds__(SPMV_BLOCK)
    spmv_direct_kernel(qg_csr_groups A, double t, const typename elem<DT>::T* __restrict__ x,
                       AxpbyArgs ax, RkArgs rk) {
  using ST = typename elem<DT>::T;
  using R = typename elem<DT>::R;
  __shared__ cx<R> coef[QG_MAX_GROUPS];
  __shared__ double red[SPMV_BLOCK / 32];
  load_coefs(A, t, coef);
  __syncthreads();

  const int G = A.n_groups;
  const int n = (int)A.n_rows;
  const int sub = threadIdx.x / LANES, lane = threadIdx.x % LANES;
  constexpr int RPB = SPMV_BLOCK / LANES;
  const ST* __restrict__ val = static_cast<const ST*>(A.val);
  double err_acc = 0.0;

  for (int base = blockIdx.x * RPB; base < n; base += gridDim.x * RPB) {
    const int row = base + sub;
    const bool valid = row < n;
    cx<R> acc{0, 0};
    for (int g = 0; g < G; ++g) {
      int s = 0, e = 0;
      if (valid) {
        const int i = rp_index(A, g, row);
        s = __ldg(A.row_ptr + i);
        e = __ldg(A.row_ptr + i + 1);
      }
      R ar = 0, ai = 0;
      lane_dot<ST, R, LANES, true>(A.col, val, x, s, e, lane, ar, ai);
      acc = cx_add(acc, cx_mul(coef[g], sub_reduce<LANES>(ar, ai)));
    }
    if (valid && lane == 0) epilogue<DT, YDT, EPI>(row, acc, ax, rk, err_acc);
  }
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<SPMV_BLOCK>(rk, err_acc, red);
  }
}

// ------------------------------------------------------------ staged kernel --
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  const bool ok = mbar_poll(bar, parity);
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

struct TileGeom {
  int r0, r1;  // rows
  int pa, np;  // entries: aligned start and count (multiple of 4)
  int ra, nr;  // row-pointer words: aligned start and count (multiple of 4)
};

__device__ __forceinline__ TileGeom tile_geom(const qg_csr_groups& A, int tile) {
  TileGeom g;
  const int G = A.n_groups;
  g.r0 = __ldg(A.tile_row + tile);
  g.r1 = __ldg(A.tile_row + tile + 1);
  const int p0 = __ldg(A.row_ptr + g.r0 * G), p1 = __ldg(A.row_ptr + g.r1 * G);
  g.pa = p0 & ~3;
  g.np = (p1 - g.pa + 3) & ~3;
  g.ra = (g.r0 * G) & ~3;
  g.nr = (g.r1 * G + 1 - g.ra + 3) & ~3;
  return g;
}

template <int DT, int YDT, int LANES, int EPI, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    spmv_staged_kernel(qg_csr_groups A, double t, const typename elem<DT>::T* __restrict__ x,
                       AxpbyArgs ax, RkArgs rk, int rpt) {
  using ST = typename elem<DT>::T;
  using R = typename elem<DT>::R;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ cx<R> coef[QG_MAX_GROUPS];
  __shared__ double red[BLOCK / 32];
  __shared__ __align__(8) uint64_t bar[2];

  const int G = A.n_groups;
  const int nzt = A.tile_nnz;
  const size_t sb = (size_t)nzt * (sizeof(ST) + 4) + (size_t)rpt * 4;
  load_coefs(A, t, coef);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const int sub = threadIdx.x / LANES, lane = threadIdx.x % LANES;
  constexpr int NSUB = BLOCK / LANES;
  double err_acc = 0.0;

  auto issue = [&](int tile, int stage) {
    TileGeom g = tile_geom(A, tile);
    unsigned char* base = smem + stage * sb;
    const unsigned bv = (unsigned)(g.np * sizeof(ST)), bc = (unsigned)(g.np * 4),
                   br = (unsigned)(g.nr * 4);
    mbar_expect_tx(&bar[stage], bv + bc + br);
    bulk_g2s(base, static_cast<const ST*>(A.val) + g.pa, bv, &bar[stage]);
    bulk_g2s(base + (size_t)nzt * sizeof(ST), A.col + g.pa, bc, &bar[stage]);
    bulk_g2s(base + (size_t)nzt * (sizeof(ST) + 4), A.row_ptr + g.ra, br, &bar[stage]);
  };

  int tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < A.n_tiles) issue(tile, 0);
  unsigned phase[2] = {0u, 0u};
  bool fault = false;
  for (int it = 0; tile < A.n_tiles; ++it, tile += gridDim.x) {
    const int stage = it & 1;
    const int next = tile + gridDim.x;
    if (threadIdx.x == 0 && next < A.n_tiles) {
      // the other buffer was released by the __syncthreads ending the previous tile
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(next, stage ^ 1);
    }
    if (!mbar_wait_bounded(&bar[stage], phase[stage])) {
      fault = true;
      break;
    }
    phase[stage] ^= 1u;

    const TileGeom g = tile_geom(A, tile);
    unsigned char* base = smem + stage * sb;
    const ST* sval = reinterpret_cast<const ST*>(base) - g.pa;
    const int* scol = reinterpret_cast<const int*>(base + (size_t)nzt * sizeof(ST)) - g.pa;
    const int* srp = reinterpret_cast<const int*>(base + (size_t)nzt * (sizeof(ST) + 4)) - g.ra;
    const int nrows = g.r1 - g.r0;
    for (int b = 0; b < nrows; b += NSUB) {
      const int rr = b + sub;
      const bool valid = rr < nrows;
      const int row = g.r0 + rr;
      cx<R> acc{0, 0};
      for (int gg = 0; gg < G; ++gg) {
        int s = 0, e = 0;
        if (valid) {
          s = srp[row * G + gg];
          e = srp[row * G + gg + 1];
        }
        R ar = 0, ai = 0;
        lane_dot<ST, R, LANES, false>(scol, sval, x, s, e, lane, ar, ai);
        acc = cx_add(acc, cx_mul(coef[gg], sub_reduce<LANES>(ar, ai)));
      }
      if (valid && lane == 0) epilogue<DT, YDT, EPI>(row, acc, ax, rk, err_acc);
    }
    __syncthreads();
  }
  if (fault) {
    // drain the copies this block may still have in flight, then report
    if (threadIdx.x == 0) {
      atomicOr(&g_fault, 1u);
      for (int s = 0; s < 2; ++s) (void)mbar_poll(&bar[s], phase[s]);
    }
    __syncthreads();
    return;
  }
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<BLOCK>(rk, err_acc, red);
  }
}

// ------------------------------------------------------------ sliced kernel --
// Sliced ELLPACK: a warp owns a 32-row slice, one thread per row.  Entry j of
// every row in the slice is adjacent in memory, so each load instruction reads
// 32 consecutive values / column indices (256 B / 128 B), and with entries
// ordered by (col XOR row) the gathered x entries of a warp fall in the same few
// lines.  UNR entries per thread are in flight: chunks of UNR loads, the last
// chunk of a group predicated on the (warp-uniform) slice width.
// Resident blocks per SM: complex64 (HBM-bound) at 40 registers; complex128
// (FP64-bound, twice the live values) at 64.
template <int DT, int UNR>
struct SlicedBounds {
  static constexpr int MIN_BLOCKS = DT == QG_C64 ? SLICED_MIN_BLOCKS : 4;
};

template <int DT, int YDT, int EPI, int UNR>
__global__ void __launch_bounds__(SPMV_BLOCK, SlicedBounds<DT, UNR>::MIN_BLOCKS)
    spmv_sliced_kernel(qg_csr_groups A, double t, const typename elem<DT>::T* __restrict__ x,
                       AxpbyArgs ax, RkArgs rk) {
  using ST = typename elem<DT>::T;
  using R = typename elem<DT>::R;
  __shared__ cx<R> coef[QG_MAX_GROUPS];
  __shared__ double red[SPMV_BLOCK / 32];
  load_coefs(A, t, coef);
  __syncthreads();
  const int G = A.n_groups;
  const int n = (int)A.n_rows;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * SPMV_BLOCK + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * SPMV_BLOCK) >> 5;
  const ST* __restrict__ val = static_cast<const ST*>(A.val);
  const int* __restrict__ col = A.col;
  double err_acc = 0.0;
  for (int sl = warp; sl < A.n_tiles; sl += nwarps) {
    int goff = __ldg(A.row_ptr + sl) + lane;  // this lane's first entry of the group
    const int row = sl * 32 + lane;
    cx<R> acc{0, 0};
    for (int g = 0; g < G; ++g) {
      const int w = __ldg(A.tile_row + sl * G + g);
      R ar = 0, ai = 0;
      int j = 0;
      for (; j + UNR <= w; j += UNR) {
        ST v[UNR], xv[UNR];
        int c[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
          v[u] = ld_stream(val + goff + 32 * (j + u));
          c[u] = ld_stream(col + goff + 32 * (j + u));
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) xv[u] = ld_gather(x + c[u]);
#pragma unroll
        for (int u = 0; u < UNR; ++u) cmac_any(ar, ai, v[u], xv[u]);
      }
      if (j < w) {  // tail chunk: up to UNR - 1 entries, still all in flight
        ST v[UNR], xv[UNR];
        int c[UNR];
#pragma unroll
        for (int u = 0; u < UNR - 1; ++u) {
          if (j + u < w) {
            v[u] = ld_stream(val + goff + 32 * (j + u));
            c[u] = ld_stream(col + goff + 32 * (j + u));
          }
        }
#pragma unroll
        for (int u = 0; u < UNR - 1; ++u)
          if (j + u < w) xv[u] = ld_gather(x + c[u]);
#pragma unroll
        for (int u = 0; u < UNR - 1; ++u)
          if (j + u < w) cmac_any(ar, ai, v[u], xv[u]);
      }
      goff += 32 * w;
      acc = cx_add(acc, cx_mul(coef[g], cx<R>{ar, ai}));
    }
    if (row < n) epilogue<DT, YDT, EPI>(row, acc, ax, rk, err_acc);
  }
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<SPMV_BLOCK>(rk, err_acc, red);
  }
}

// ------------------------------------------------ dictionary-coded sliced --
// The sliced kernel with every stored entry replaced by a 1- or 2-byte code into its
// group's table of (column - row, value) pairs, staged in shared memory per block.  A
// Kronecker-structured Liouvillian repeats a few such pairs (the Ising L = 10 one: 20
// in the driven group, about 700 in the constant one), so the operator stream shrinks
// from 12 bytes per entry (complex64 value, int32 column) to 1-2 bytes, and a stage is
// bound by the shared-memory lookups and the L2 gathers of x instead of by HBM.
template <int CB>
struct Codes4;
template <>
struct Codes4<1> {
  using T = unsigned int;
  __device__ static int at(T c, int u) { return (int)((c >> (8 * u)) & 0xffu); }
};
template <>
struct Codes4<2> {
  using T = uint2;
  __device__ static int at(T c, int u) {
    const unsigned w = u < 2 ? c.x : c.y;
    return (int)((w >> (16 * (u & 1))) & 0xffffu);
  }
};

// One stored code: the table pair k applied to x[row + offset].  Whole complex values
// (QG_LAYOUT_SLICED_DICT) cost four multiply-adds.  With the real/imaginary split
// (QG_LAYOUT_SLICED_DICT_RI, complex128) a table entry is one real factor: toff holds
// (offset << 1) | imag and tval the pair (c1, c2) = (a, a) for a real part or (-a, a) for
// an imaginary part, applied as (c1 p, c2 q) with (p, q) = x, or x's parts exchanged for
// an imaginary part -- two FP64 multiply-adds, GB300's scarce FP64 rate being the bound.
template <bool RI, typename ST, typename R>
__device__ __forceinline__ void dict_mac(const ST* __restrict__ tval, const int* __restrict__ toff,
                                         const ST* __restrict__ x, int k, int row, int last_col,
                                         R& ar, R& ai) {
  if constexpr (RI) {
    const int oc = toff[k];
    const int col = min(max(row + (oc >> 1), 0), last_col);
    const ST v = tval[k];
    const ST xv = ld_gather(x + col);
    const bool sw = (oc & 1) != 0;
    ar = fma(v.x, sw ? xv.y : xv.x, ar);
    ai = fma(v.y, sw ? xv.x : xv.y, ai);
  } else {
    const int col = min(max(row + toff[k], 0), last_col);
    cmac_any(ar, ai, tval[k], ld_gather(x + col));
  }
}

// acc += c * (ar, ai).  In FP64 a real coefficient (every group of a Liouvillian with a
// real time dependence, and the constant group) takes two multiply-adds, not four; the
// branch is uniform (one coefficient per group).  FP32 keeps the plain product.
template <typename R>
__device__ __forceinline__ void coef_mac(cx<R>& acc, cx<R> c, R ar, R ai) {
  if constexpr (sizeof(R) == 8) {
    if (c.im == (R)0) {
      acc.re = fma(c.re, ar, acc.re);
      acc.im = fma(c.re, ai, acc.im);
      return;
    }
  }
  acc = cx_add(acc, cx_mul(c, cx<R>{ar, ai}));
}

template <int DT, int YDT, int EPI, int CB, bool RI>
__global__ void __launch_bounds__(SPMV_BLOCK, SlicedBounds<DT, 4>::MIN_BLOCKS)
    spmv_dict_kernel(qg_csr_groups A, double t, const typename elem<DT>::T* __restrict__ x,
                     AxpbyArgs ax, RkArgs rk) {
  using ST = typename elem<DT>::T;
  using R = typename elem<DT>::R;
  using C4 = typename Codes4<CB>::T;
  extern __shared__ __align__(16) unsigned char dict_smem[];
  __shared__ cx<R> coef[QG_MAX_GROUPS];
  __shared__ int ccls[QG_MAX_GROUPS];
  __shared__ int tstart[QG_MAX_GROUPS + 1];
  __shared__ double red[SPMV_BLOCK / 32];
  const int D = A.lanes;
  ST* tval = reinterpret_cast<ST*>(dict_smem);
  int* toff = reinterpret_cast<int*>(dict_smem + (size_t)D * sizeof(ST));
  load_coefs(A, t, coef);
  coef_classes(A, coef, ccls);
  for (int i = threadIdx.x; i < D; i += SPMV_BLOCK) {
    tval[i] = __ldg(static_cast<const ST*>(A.val) + i);
    toff[i] = __ldg(A.dict_off + i);
  }
  if (threadIdx.x <= (unsigned)A.n_groups) tstart[threadIdx.x] = __ldg(A.dict_start + threadIdx.x);
  __syncthreads();
  const int G = A.n_groups;
  const int n = (int)A.n_rows;
  const int S = A.n_tiles;
  const int last_col = (int)A.n_cols - 1;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * SPMV_BLOCK + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * SPMV_BLOCK) >> 5;
  const unsigned char* __restrict__ codes = reinterpret_cast<const unsigned char*>(A.col);
  double err_acc = 0.0;
  for (int sl = warp; sl < S; sl += nwarps) {
    const int row = sl * 32 + lane;
    cx<R> acc{0, 0};
    for (int g = 0; g < G; ++g) {
      // exact width (uniform over the warp): whole chunks of four codes, then a tail
      const int w = __ldg(A.tile_row + sl * G + g);
      const int wq = w >> 2, wr = w & 3;
      const int t0 = tstart[g], tn = tstart[g + 1] - t0;
      const C4* __restrict__ cp =
          reinterpret_cast<const C4*>(codes + (size_t)CB * __ldg(A.row_ptr + g * (S + 1) + sl)) +
          lane;
      // FP64: a group whose coefficient is one accumulates into the row's sum directly
      const bool direct = sizeof(R) == 8 && ccls[g] == 0;
      R ar = direct ? acc.re : (R)0, ai = direct ? acc.im : (R)0;
#pragma unroll 2
      for (int q = 0; q < wq; ++q) {
        const C4 c4 = ld_stream(cp + 32 * q);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          int k = Codes4<CB>::at(c4, u);
          if constexpr (RI) {  // FP64-bound: skip a position that is padding in every row
            if (!__any_sync(0xffffffffu, k != 0)) continue;
          }
          k = t0 + (k < tn ? k : 0);  // a table index of this group whatever the code
          dict_mac<RI>(tval, toff, x, k, row, last_col, ar, ai);
        }
      }
      if (wr) {
        const C4 c4 = ld_stream(cp + 32 * wq);
#pragma unroll
        for (int u = 0; u < 3; ++u) {
          if (u < wr) {
            int k = Codes4<CB>::at(c4, u);
            if constexpr (RI) {
              if (!__any_sync(0xffffffffu, k != 0)) continue;
            }
            k = t0 + (k < tn ? k : 0);
            dict_mac<RI>(tval, toff, x, k, row, last_col, ar, ai);
          }
        }
      }
      if (direct)
        acc = cx<R>{ar, ai};
      else
        coef_mac(acc, coef[g], ar, ai);
    }
    if (row < n) epilogue<DT, YDT, EPI>(row, acc, ax, rk, err_acc);
  }
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<SPMV_BLOCK>(rk, err_acc, red);
  }
}

// ---------------------------------------------------- matrix-free Lindblad --
// out(r, c) = D(r, c) x[r + c d]
//           + sum_g a_g sum_j A_g[r,j] x[j + c d] + conj(a_g) sum_k conj(A_g[c,k]) x[r + k d]
//           + sum_{i general} w_i sum_{j, k} C_i[r,j] conj(C_i[c,k]) x[j + k d],
// D(r, c) = sum_g a_g A_g[r,r] + conj(a_g A_g[c,c]) + sum_{i diagonal} w_i C_i[r,r] conj(C_i[c,c]),
// the Lindblad generator on vec(rho) = x (column-major, rho[r, c] at r + c d) without its
// d^2 x d^2 superoperator: A = -i H_nh and w_i = |f_i(t)|^2.  One thread per element; a
// warp covers 32 consecutive r of one column c.  Row-r operator entries are read from
// ELL blocks laid out so that the warp's loads are one contiguous run, row-c entries
// are warp-uniform (broadcast), and every gather is a contiguous run of one column of
// rho.  The d x d operators stay in L1/L2 and the state (d^2 entries) in L2: the HBM
// traffic of a stage is its vectors only.  Diagonal parts (the diagonal of A and the
// all-diagonal collapse operators, e.g. dephasing) fold into one factor on x[r + c d].
// With L.hermitian (rho Hermitian, the reference's A + A^dag branch) only the elements
// r >= c are evaluated; each also goes through the epilogue at its mirror c + r d as its
// conjugate, and the diagonal is taken real.
constexpr int LB_BLOCK = 256;

// acc += conj(v) * x
__device__ __forceinline__ void cmac_conj(double& ar, double& ai, double2 v, double2 x) {
  ar = fma(v.x, x.x, ar);
  ar = fma(v.y, x.y, ar);
  ai = fma(v.x, x.y, ai);
  ai = fma(-v.y, x.x, ai);
}
__device__ __forceinline__ void cmac_conj(float& ar, float& ai, float2 v, float2 x) {
  ar = fmaf(v.x, x.x, ar);
  ar = fmaf(v.y, x.y, ar);
  ai = fmaf(v.x, x.y, ai);
  ai = fmaf(-v.y, x.x, ai);
}

__device__ __forceinline__ cplx prog_coef(const int* code, const int* start, const double* consts,
                                          int g, double t) {
  if (code == nullptr) return cplx{1.0, 0.0};
  return eval_coef(code + start[g], consts, t);
}

template <int DT, int YDT, int EPI, bool HERM>
__global__ void __launch_bounds__(LB_BLOCK)
    lindblad_kernel(qg_lindblad L, double t, const typename elem<DT>::T* __restrict__ x,
                    AxpbyArgs ax, RkArgs rk) {
  using ST = typename elem<DT>::T;
  using R = typename elem<DT>::R;
  __shared__ cx<R> ca[QG_MAX_GROUPS];
  __shared__ R wc[QG_MAX_COPS];
  __shared__ double red[LB_BLOCK / 32];
  const int G = L.n_groups, ND = L.n_diag_cops, NE = L.n_cops - L.n_diag_cops;
  if (threadIdx.x < G) {
    const cplx k = prog_coef(L.a_coef_code, L.a_coef_start, L.a_coef_consts, threadIdx.x, t);
    ca[threadIdx.x] = cx<R>{(R)k.re, (R)k.im};
  }
  if (threadIdx.x < L.n_cops) {
    const cplx f = prog_coef(L.c_coef_code, L.c_coef_start, L.c_coef_consts, threadIdx.x, t);
    wc[threadIdx.x] = (R)(f.re * f.re + f.im * f.im);
  }
  __syncthreads();
  const int d = (int)L.d;
  const int n = d * d;
  const ST* __restrict__ dconst = static_cast<const ST*>(L.d_const);
  const ST* __restrict__ adiag = static_cast<const ST*>(L.a_diag);
  const int* __restrict__ acol = L.a_col;
  const ST* __restrict__ aval = static_cast<const ST*>(L.a_val);
  const ST* __restrict__ cdiag = static_cast<const ST*>(L.c_diag);
  const int* __restrict__ ccol = L.c_col;
  const ST* __restrict__ cval = static_cast<const ST*>(L.c_val);
  const int dmask = L.a_diag_const;
  const int nd0 = L.n_const_diag;
  int nw1 = 0;  // leading general collapse operators of width 1
  while (nw1 < NE && L.c_width[nw1] == 1) ++nw1;
  double err_acc = 0.0;
  // L[x] at (r, c)
  auto element = [&](int r, int c) -> cx<R> {
    const int cd = c * d;
    // diagonal factor D(r, c): the precomputed constant part plus the time-dependent rest
    R dr = 0, di = 0;
    if (dconst) {
      const ST p = __ldg(dconst + (r + cd));
      dr = p.x;
      di = p.y;
    }
    for (int g = 0; g < G; ++g) {
      if ((dmask >> g) & 1) continue;
      const cx<R> k = ca[g];
      const ST p = __ldg(adiag + g * d + r), q = __ldg(adiag + g * d + c);
      dr += k.re * (p.x + q.x) - k.im * (p.y - q.y);  // k p + conj(k q)
      di += k.re * (p.y - q.y) + k.im * (p.x + q.x);
    }
    for (int i = nd0; i < ND; ++i) {
      const R w = wc[i];
      const ST p = __ldg(cdiag + i * d + r), q = __ldg(cdiag + i * d + c);
      dr += w * (p.x * q.x + p.y * q.y);  // w p conj(q)
      di += w * (p.y * q.x - p.x * q.y);
    }
    const ST xe = ld_gather(x + (r + cd));
    cx<R> acc{dr * xe.x - di * xe.y, dr * xe.y + di * xe.x};
    // off-diagonal A: A rho (row r against column c) and rho A^dag (row c against row r)
    int base = 0;
    for (int g = 0; g < G; ++g) {
      const int W = L.a_width[g];
      if (W == 0) continue;
      R lr = 0, li = 0, qr = 0, qi = 0;
  #pragma unroll 4
      for (int j = 0; j < W; ++j) {
        const int e = base + j * d;
        const int cr = __ldg(acol + e + r), cc = __ldg(acol + e + c);
        const ST vr = __ldg(aval + e + r), vc = __ldg(aval + e + c);
        cmac_any(lr, li, vr, ld_gather(x + (cr + cd)));
        cmac_conj(qr, qi, vc, ld_gather(x + (r + cc * d)));
      }
      const cx<R> k = ca[g];
      acc.re += k.re * lr - k.im * li + k.re * qr + k.im * qi;
      acc.im += k.re * li + k.im * lr + k.re * qi - k.im * qr;
      base += W * d;
    }
    // general collapse operators: C rho C^dag.  The leading width-1 operators (s-, a, ...)
    // run branch-free in complex64 (a padding entry has value 0 and a valid column), so
    // the gathers of several operators are in flight at once: 56 -> 48 us per stage at
    // L = 10.  The FP64-bound complex128 form skips padding instead.
    base = 0;
    int i = 0;
  #pragma unroll 4
    for (; i < nw1; ++i) {
      const R w = wc[ND + i];
      const int er = base + r, ec = base + c;
      const ST b = __ldg(cval + ec), v = __ldg(cval + er);
      if constexpr (DT == QG_C128) {  // FP64-bound: skip padding rather than multiply by 0
        if ((b.x == (R)0 && b.y == (R)0) || (v.x == (R)0 && v.y == (R)0)) {
          base += d;
          continue;
        }
      }
      const ST xv = ld_gather(x + (__ldg(ccol + er) + __ldg(ccol + ec) * d));
      const R pr = w * (v.x * b.x + v.y * b.y), pi = w * (v.y * b.x - v.x * b.y);  // w v conj(b)
      acc.re += pr * xv.x - pi * xv.y;
      acc.im += pr * xv.y + pi * xv.x;
      base += d;
    }
    for (; i < NE; ++i) {
      const int W = L.c_width[i];
      const R w = wc[ND + i];
      if (W > 0) {
        R sr2 = 0, si2 = 0;
        for (int q = 0; q < W; ++q) {
          const int eq = base + q * d + c;
          const ST b = __ldg(cval + eq);
          if (b.x == (R)0 && b.y == (R)0) continue;  // warp-uniform: padding of row c
          const int kd = __ldg(ccol + eq) * d;
          R ir = 0, ii = 0;
          for (int p = 0; p < W; ++p) {
            const int ep = base + p * d + r;
            const ST v = __ldg(cval + ep);
            if (v.x != (R)0 || v.y != (R)0) cmac_any(ir, ii, v, ld_gather(x + (__ldg(ccol + ep) + kd)));
          }
          sr2 += b.x * ir + b.y * ii;  // conj(b) * inner
          si2 += b.x * ii - b.y * ir;
        }
        acc.re += w * sr2;
        acc.im += w * si2;
      }
      base += W * d;
    }
    return acc;
  };
  if constexpr (!HERM) {
    // (r, c) of idx, advanced by the grid stride without a division per element
    const int stride = gridDim.x * LB_BLOCK;
    const int sc = stride / d, sr = stride - (stride / d) * d;
    int idx = blockIdx.x * LB_BLOCK + threadIdx.x;
    int c = idx / d;
    int r = idx - c * d;
    for (; idx < n; idx += stride) {
      epilogue<DT, YDT, EPI>(idx, element(r, c), ax, rk, err_acc);
      c += sc;
      r += sr;
      if (r >= d) {
        r -= d;
        ++c;
      }
    }
  } else {
    // Hermitian rho: 32 x 32 tiles on or below the diagonal; warp w evaluates 32
    // consecutive r of the columns w, w + 8, w + 16, w + 24 (elements r >= c), then the
    // block writes the conjugates to the mirrors (c, r) through shared memory, a warp
    // covering 32 consecutive c of one row r.
    __shared__ cx<R> tile[32][33];  // [c - c0][r - r0]
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // only the n_t (n_t + 1) / 2 tiles on or below the diagonal are enumerated, column
    // block j holding row blocks j .. n_t - 1, so the blocks share the work evenly
    const int n_t = (d + 31) / 32;
    const int n_tiles = n_t * (n_t + 1) / 2;
    int tj = 0, tbase = 0;  // column block of tau and the index of its first tile
    for (int tau = blockIdx.x; tau < n_tiles; tau += gridDim.x) {
      while (tau >= tbase + (n_t - tj)) {
        tbase += n_t - tj;
        ++tj;
      }
      const int r0 = (tj + (tau - tbase)) * 32, c0 = tj * 32;
#pragma unroll 1
      for (int q = 0; q < 4; ++q) {
        const int cl = w + 8 * q, r = r0 + lane, c = c0 + cl;
        cx<R> acc{0, 0};
        if (r < d && c < d && r >= c) {
          acc = element(r, c);
          if (r == c) acc.im = 0;  // A + A^dag: real diagonal
          epilogue<DT, YDT, EPI>(r + c * d, acc, ax, rk, err_acc);
        }
        tile[cl][lane] = acc;
      }
      __syncthreads();
#pragma unroll 1
      for (int q = 0; q < 4; ++q) {
        const int rl = w + 8 * q;
        const int mr = r0 + rl, mc = c0 + lane;  // the mirror of (mr, mc)
        if (mr < d && mc < d && mr > mc) {
          const cx<R> v = tile[lane][rl];
          epilogue<DT, YDT, EPI>(mc + mr * d, cx<R>{v.re, -v.im}, ax, rk, err_acc);
        }
      }
      __syncthreads();
    }
  }
  if constexpr (EPI == EPI_RK) {
    if (rk.stage == RK_STEP - 1) finish_error<LB_BLOCK>(rk, err_acc, red);
  }
}

// ------------------------------------------------------------------ launch --
// Opt `kernel` into `smem` bytes of dynamic shared memory and return its
// resident blocks per SM.  The caller keeps one cache per kernel instantiation; it
// holds one entry per device (the attribute is set with that device current) and is
// shared by host threads under its mutex.
constexpr int OCC_MAX_DEVICES = 64;
struct OccCache {
  std::mutex mu;
  int occ[OCC_MAX_DEVICES] = {};
  size_t smem[OCC_MAX_DEVICES] = {};
};
template <typename K>
static int staged_occupancy(K kernel, int block, size_t smem, OccCache& c) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= OCC_MAX_DEVICES) return -1;
  std::lock_guard<std::mutex> lock(c.mu);
  if (c.occ[dev] > 0 && c.smem[dev] == smem) return c.occ[dev];
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess)
    return -1;
  c.smem[dev] = smem;
  c.occ[dev] = per_sm;
  return per_sm;
}

template <int DT, int YDT, int EPI, int LANES>
static int launch_staged(cudaStream_t st, const qg_csr_groups& A, double t, const void* x,
                         const AxpbyArgs& ax, const RkArgs& rk) {
  using ST = typename elem<DT>::T;
  constexpr int BLOCK = 256;
  const int rpt = ((QG_TILE_ROWS * A.n_groups + 8) + 3) & ~3;
  const size_t sb = (size_t)A.tile_nnz * (sizeof(ST) + 4) + (size_t)rpt * 4;
  const size_t smem = 2 * sb;
  auto kern = spmv_staged_kernel<DT, YDT, LANES, EPI, BLOCK>;
  static OccCache cache;  // one per instantiation of this function (and so of kern)
  const int per_sm = staged_occupancy(kern, BLOCK, smem, cache);
  if (per_sm <= 0) return set_error(QG_ERR_ARG, "staged tile does not fit in shared memory");
  int64_t grid = (int64_t)sm_count() * per_sm;
  if (grid > A.n_tiles) grid = A.n_tiles;
  if (grid > qg_scratch_doubles()) grid = qg_scratch_doubles();
  kern<<<(int)grid, BLOCK, smem, st>>>(A, t, (const ST*)x, ax, rk, rpt);
  return check_launch("spmv_staged_kernel");
}

template <int DT, int YDT, int EPI, int CB, bool RI>
static int launch_dict(cudaStream_t st, const qg_csr_groups& A, double t, const void* x,
                       const AxpbyArgs& ax, const RkArgs& rk) {
  using ST = typename elem<DT>::T;
  auto kern = spmv_dict_kernel<DT, YDT, EPI, CB, RI>;
  const size_t smem = ((size_t)A.lanes * (sizeof(ST) + sizeof(int)) + 15) & ~(size_t)15;
  static OccCache cache;  // one per instantiation
  const int per_sm = staged_occupancy(kern, SPMV_BLOCK, smem, cache);
  if (per_sm <= 0) return set_error(QG_ERR_ARG, "dictionary does not fit in shared memory");
  const int64_t blocks = ((int64_t)A.n_tiles * 32 + SPMV_BLOCK - 1) / SPMV_BLOCK;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (cap > qg_scratch_doubles()) cap = qg_scratch_doubles();
  const int grid = (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
  kern<<<grid, SPMV_BLOCK, smem, st>>>(A, t, (const ST*)x, ax, rk);
  return check_launch("spmv_dict_kernel");
}

template <int DT, int YDT, int EPI>
static int launch_any(cudaStream_t st, const qg_csr_groups& A, double t, const void* x,
                      const AxpbyArgs& ax, const RkArgs& rk) {
  using ST = typename elem<DT>::T;
  const int lanes = A.lanes > 0 ? A.lanes : 4;
  if (A.layout == QG_LAYOUT_SLICED_DICT)
    return A.tile_nnz == 1 ? launch_dict<DT, YDT, EPI, 1, false>(st, A, t, x, ax, rk)
                           : launch_dict<DT, YDT, EPI, 2, false>(st, A, t, x, ax, rk);
  if (A.layout == QG_LAYOUT_SLICED_DICT_RI) {
    if constexpr (DT == QG_C128)
      return A.tile_nnz == 1 ? launch_dict<DT, YDT, EPI, 1, true>(st, A, t, x, ax, rk)
                             : launch_dict<DT, YDT, EPI, 2, true>(st, A, t, x, ax, rk);
    return set_error(QG_ERR_UNSUPPORTED, "the real/imaginary split dictionary is complex128 only");
  }
  if (A.layout == QG_LAYOUT_SLICED) {
    // one wave: every block resident at once, warps striding over the slices.  (8
    // entries in flight at 64 registers measured slower than 4 at 40: 73 vs 68 us
    // per fused stage on the L=10 Liouvillian, so only the 4-entry variant is built.)
    auto kern = spmv_sliced_kernel<DT, YDT, EPI, 4>;
    static OccCache cache;  // one per instantiation
    const int per_sm = staged_occupancy(kern, SPMV_BLOCK, 0, cache);
    if (per_sm <= 0) return set_error(QG_ERR_CUDA, "occupancy query failed");
    int64_t warps_needed = A.n_tiles;
    int64_t blocks = (warps_needed * 32 + SPMV_BLOCK - 1) / SPMV_BLOCK;
    int64_t cap = (int64_t)sm_count() * per_sm;
    if (cap > qg_scratch_doubles()) cap = qg_scratch_doubles();
    const int grid = (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
    kern<<<grid, SPMV_BLOCK, 0, st>>>(A, t, (const ST*)x, ax, rk);
    return check_launch("spmv_sliced_kernel");
  }
  if (A.n_tiles > 0) {
    switch (lanes) {
      case 1: return launch_staged<DT, YDT, EPI, 1>(st, A, t, x, ax, rk);
      case 2: return launch_staged<DT, YDT, EPI, 2>(st, A, t, x, ax, rk);
      case 4: return launch_staged<DT, YDT, EPI, 4>(st, A, t, x, ax, rk);
      case 8: return launch_staged<DT, YDT, EPI, 8>(st, A, t, x, ax, rk);
      case 16: return launch_staged<DT, YDT, EPI, 16>(st, A, t, x, ax, rk);
      default: return set_error(QG_ERR_ARG, "staged kernel: lanes must be 1..16");
    }
  }
  const int rpb = SPMV_BLOCK / lanes;
  int64_t blocks = (A.n_rows + rpb - 1) / rpb;
  int64_t cap = (int64_t)sm_count() * (2048 / SPMV_BLOCK);
  if (cap > qg_scratch_doubles()) cap = qg_scratch_doubles();
  const int grid = (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
#define QG_CASE(L)                                                                          \
  case L:                                                                                   \
    spmv_direct_kernel<DT, YDT, L, EPI><<<grid, SPMV_BLOCK, 0, st>>>(A, t, (const ST*)x, ax, \
                                                                     rk);                   \
    break;
  switch (lanes) {
    QG_CASE(1)
    QG_CASE(2)
    QG_CASE(4)
    QG_CASE(8)
    QG_CASE(16)
    QG_CASE(32)
    default:
      return set_error(QG_ERR_ARG, "lanes must be a power of two in 1..32");
  }
#undef QG_CASE
  return check_launch("spmv_direct_kernel");
}

// The full form and the Hermitian branch are separate instantiations: sharing one kernel
// body, the full form's code generation degraded (dense d = 128 operators: 3x slower).
template <int DT, int YDT, int EPI, bool HERM>
static int launch_lindblad_form(cudaStream_t st, const qg_lindblad& L, double t, const void* x,
                                const AxpbyArgs& ax, const RkArgs& rk) {
  using ST = typename elem<DT>::T;
  auto kern = lindblad_kernel<DT, YDT, EPI, HERM>;
  static OccCache cache;  // one per instantiation
  const int per_sm = staged_occupancy(kern, LB_BLOCK, 0, cache);
  if (per_sm <= 0) return set_error(QG_ERR_CUDA, "occupancy query failed");
  const int64_t n = L.d * L.d;
  const int64_t n_t = (L.d + 31) / 32;
  const int64_t blocks = HERM ? n_t * (n_t + 1) / 2 : (n + LB_BLOCK - 1) / LB_BLOCK;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (cap > qg_scratch_doubles()) cap = qg_scratch_doubles();
  const int grid = (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
  kern<<<grid, LB_BLOCK, 0, st>>>(L, t, (const ST*)x, ax, rk);
  return check_launch("lindblad_kernel");
}

template <int DT, int YDT, int EPI>
static int launch_lindblad(cudaStream_t st, const qg_lindblad& L, double t, const void* x,
                           const AxpbyArgs& ax, const RkArgs& rk) {
  return L.hermitian ? launch_lindblad_form<DT, YDT, EPI, true>(st, L, t, x, ax, rk)
                     : launch_lindblad_form<DT, YDT, EPI, false>(st, L, t, x, ax, rk);
}

static int check_groups(const qg_csr_groups* A) {
  if (!A || !A->row_ptr || !A->col || !A->val) return set_error(QG_ERR_ARG, "null operator");
  if (A->n_groups < 1 || A->n_groups > QG_MAX_GROUPS)
    return set_error(QG_ERR_ARG, "n_groups out of range");
  if (A->n_rows < 0 || A->n_rows >= (int64_t)INT32_MAX / QG_MAX_GROUPS || A->n_cols < 0)
    return set_error(QG_ERR_ARG, "bad operator shape");
  if (A->dtype != QG_C128 && A->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "operator dtype must be QG_C128 or QG_C64");
  if (A->layout != QG_LAYOUT_GROUP_MAJOR && A->layout != QG_LAYOUT_ROW_MAJOR &&
      A->layout != QG_LAYOUT_SLICED && A->layout != QG_LAYOUT_SLICED_DICT &&
      A->layout != QG_LAYOUT_SLICED_DICT_RI)
    return set_error(QG_ERR_ARG, "unknown row-pointer layout");
  if (A->layout == QG_LAYOUT_SLICED_DICT_RI && A->dtype != QG_C128)
    return set_error(QG_ERR_UNSUPPORTED, "the real/imaginary split dictionary is complex128 only");
  if (A->layout == QG_LAYOUT_SLICED_DICT || A->layout == QG_LAYOUT_SLICED_DICT_RI) {
    if (!A->tile_row || !A->dict_off || !A->dict_start || A->n_tiles != (A->n_rows + 31) / 32)
      return set_error(QG_ERR_ARG,
                       "dictionary layout needs n_tiles = ceil(n_rows/32), widths and tables");
    if (A->tile_nnz != 1 && A->tile_nnz != 2)
      return set_error(QG_ERR_ARG, "dictionary codes must be 1 or 2 bytes");
    if (A->lanes < A->n_groups || A->lanes > QG_DICT_MAX)
      return set_error(QG_ERR_ARG, "dictionary size out of range");
    if ((int64_t)A->n_groups * (A->n_tiles + 1) >= (int64_t)INT32_MAX)
      return set_error(QG_ERR_ARG, "too many slices");
  } else if (A->layout == QG_LAYOUT_SLICED) {
    if (!A->tile_row || A->n_tiles != (A->n_rows + 31) / 32)
      return set_error(QG_ERR_ARG, "sliced layout needs n_tiles = ceil(n_rows/32) and widths");
  } else if (A->n_tiles > 0) {
    if (A->layout != QG_LAYOUT_ROW_MAJOR || !A->tile_row)
      return set_error(QG_ERR_ARG, "tiles need the row-major layout and tile_row");
    if (A->tile_nnz != 2048 && A->tile_nnz != 4096)
      return set_error(QG_ERR_ARG, "tile_nnz must be 2048 or 4096");
  }
  if (A->coef_code && (!A->coef_start || !A->coef_consts))
    return set_error(QG_ERR_ARG, "coefficient program tables incomplete");
  return QG_OK;
}

static int check_lindblad(const qg_lindblad* L) {
  if (!L) return set_error(QG_ERR_ARG, "null generator");
  const int64_t d = L->d;
  if (d < 1 || d * d >= (int64_t)INT32_MAX)
    return set_error(QG_ERR_ARG, "dimension out of range (need 1 <= d, d*d < 2^31)");
  if (L->dtype != QG_C128 && L->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "dtype must be QG_C128 or QG_C64");
  if (L->n_groups < 1 || L->n_groups > QG_MAX_GROUPS)
    return set_error(QG_ERR_ARG, "n_groups out of range");
  if (L->n_cops < 0 || L->n_cops > QG_MAX_COPS || L->n_diag_cops < 0 ||
      L->n_diag_cops > L->n_cops)
    return set_error(QG_ERR_ARG, "collapse operator counts out of range");
  if (!L->a_diag) return set_error(QG_ERR_ARG, "null A storage");
  if ((L->hermitian != 0 && L->hermitian != 1) || L->reserved != 0)
    return set_error(QG_ERR_ARG, "hermitian must be 0 or 1 and reserved 0");
  if (!L->d_const && (L->a_diag_const != 0 || L->n_const_diag != 0))
    return set_error(QG_ERR_ARG, "constant diagonal parts need d_const");
  if (L->n_const_diag < 0 || L->n_const_diag > L->n_diag_cops)
    return set_error(QG_ERR_ARG, "n_const_diag out of range");
  if (L->n_diag_cops > 0 && !L->c_diag) return set_error(QG_ERR_ARG, "null diagonal collapse storage");
  int64_t ta = 0, tc = 0;
  for (int g = 0; g < L->n_groups; ++g) {
    if (L->a_width[g] < 0) return set_error(QG_ERR_ARG, "negative ELL width");
    ta += L->a_width[g];
  }
  for (int i = 0; i < L->n_cops - L->n_diag_cops; ++i) {
    if (L->c_width[i] < 0) return set_error(QG_ERR_ARG, "negative ELL width");
    tc += L->c_width[i];
  }
  if (ta * d >= (int64_t)INT32_MAX || tc * d >= (int64_t)INT32_MAX)
    return set_error(QG_ERR_ARG, "ELL storage beyond 2^31 entries");
  if ((ta > 0 && (!L->a_col || !L->a_val)) || (tc > 0 && (!L->c_col || !L->c_val)))
    return set_error(QG_ERR_ARG, "null ELL storage");
  if (L->a_coef_code && (!L->a_coef_start || !L->a_coef_consts))
    return set_error(QG_ERR_ARG, "coefficient program tables incomplete");
  if (L->c_coef_code && (!L->c_coef_start || !L->c_coef_consts))
    return set_error(QG_ERR_ARG, "coefficient program tables incomplete");
  return QG_OK;
}

}  // namespace qg

using namespace qg;

extern "C" int qg_device_fault(void) {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_fault, sizeof(v)) != cudaSuccess)
    return set_error(QG_ERR_CUDA, "cannot read the device fault flag");
  if (v) cudaMemcpyToSymbol(g_fault, &zero, sizeof(zero));
  return (int)(v | (unsigned)dense_fault_take());
}

extern "C" int qg_spmv_csr(const qg_csr_groups* A, double t, const void* x, void* y,
                           double alpha_re, double alpha_im, double beta_re, double beta_im,
                           void* stream) {
  int rc = check_groups(A);
  if (rc) return rc;
  if (!x || !y) return set_error(QG_ERR_ARG, "null vector");
  if (A->n_rows == 0) return QG_OK;
  AxpbyArgs ax{y, alpha_re, alpha_im, beta_re, beta_im};
  RkArgs rk{};
  cudaStream_t st = (cudaStream_t)stream;
  if (A->dtype == QG_C128) return launch_any<QG_C128, QG_C128, EPI_AXPBY>(st, *A, t, x, ax, rk);
  return launch_any<QG_C64, QG_C64, EPI_AXPBY>(st, *A, t, x, ax, rk);
}

extern "C" int qg_vern7_stage(const qg_csr_groups* A, const qg_rk_buffers* B, int stage,
                              double t_prev, double dt, double atol, double rtol, void* stream) {
  int rc = check_groups(A);
  if (rc) return rc;
  if (A->n_rows != A->n_cols) return set_error(QG_ERR_ARG, "operator must be square with n rows");
  RkArgs rk;
  const void* x = nullptr;
  rc = prepare_stage(B, A->dtype, A->n_rows, stage, dt, atol, rtol, rk, x);
  if (rc) return rc;
  if (B->n == 0) return QG_OK;
  AxpbyArgs ax{};
  cudaStream_t st = (cudaStream_t)stream;
  const double t = t_prev + VERN7_C_HOST[stage] * dt;
  if (B->state_dtype == QG_C128 && B->stage_dtype == QG_C128)
    return launch_any<QG_C128, QG_C128, EPI_RK>(st, *A, t, x, ax, rk);
  if (B->state_dtype == QG_C128)
    return launch_any<QG_C64, QG_C128, EPI_RK>(st, *A, t, x, ax, rk);
  return launch_any<QG_C64, QG_C64, EPI_RK>(st, *A, t, x, ax, rk);
}

extern "C" int qg_lindblad_apply(const qg_lindblad* L, double t, const void* x, void* y,
                                 double alpha_re, double alpha_im, double beta_re, double beta_im,
                                 void* stream) {
  int rc = check_lindblad(L);
  if (rc) return rc;
  if (!x || !y) return set_error(QG_ERR_ARG, "null vector");
  AxpbyArgs ax{y, alpha_re, alpha_im, beta_re, beta_im};
  RkArgs rk{};
  cudaStream_t st = (cudaStream_t)stream;
  if (L->dtype == QG_C128) return launch_lindblad<QG_C128, QG_C128, EPI_AXPBY>(st, *L, t, x, ax, rk);
  return launch_lindblad<QG_C64, QG_C64, EPI_AXPBY>(st, *L, t, x, ax, rk);
}

extern "C" int qg_lindblad_stage(const qg_lindblad* L, const qg_rk_buffers* B, int stage,
                                 double t_prev, double dt, double atol, double rtol, void* stream) {
  int rc = check_lindblad(L);
  if (rc) return rc;
  RkArgs rk;
  const void* x = nullptr;
  rc = prepare_stage(B, L->dtype, L->d * L->d, stage, dt, atol, rtol, rk, x);
  if (rc) return rc;
  AxpbyArgs ax{};
  cudaStream_t st = (cudaStream_t)stream;
  const double t = t_prev + VERN7_C_HOST[stage] * dt;
  if (B->state_dtype == QG_C128 && B->stage_dtype == QG_C128)
    return launch_lindblad<QG_C128, QG_C128, EPI_RK>(st, *L, t, x, ax, rk);
  if (B->state_dtype == QG_C128)
    return launch_lindblad<QG_C64, QG_C128, EPI_RK>(st, *L, t, x, ax, rk);
  return launch_lindblad<QG_C64, QG_C64, EPI_RK>(st, *L, t, x, ax, rk);
}
